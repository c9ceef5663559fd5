"""C ABI checks that need no GPU: libpog.so builds and loads, exports every entry point that
include/pog.h declares, the ctypes mirrors have the C struct layouts, and the host-only
parameter validation reports errors the documented way."""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

from pour_over_coffee_lbm_gb300 import _lib
from pour_over_coffee_lbm_gb300.params import LatticeConfig, PogParams, PogParticleParams

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "pog.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pog_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "pog_step" in names and "pog_adjoint_step" in names and "pog_particles_couple" in names
    assert len(names) >= 15


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    # the ctypes signature table covers every declared entry point
    bound = {n for n, _, _ in _lib.SIGNATURES}
    assert set(declared_functions()) <= bound


def test_version_and_errors():
    lib = _lib.load()
    assert lib.pog_version() == 2
    p = LatticeConfig(nx=2).to_c()
    rc = lib.pog_validate_params(ctypes.byref(p))
    assert rc == -1
    assert b">= 4" in lib.pog_last_error()
    p = LatticeConfig(tau=0.5).to_c()
    assert lib.pog_validate_params(ctypes.byref(p)) == -1
    p = LatticeConfig(nx=1024, ny=1024, nz=1024).to_c()
    assert lib.pog_validate_params(ctypes.byref(p)) == -5  # POG_E_RANGE: 19*ncell >= 2^32
    p = LatticeConfig(storage=7).to_c()
    assert lib.pog_validate_params(ctypes.byref(p)) == -1
    p = LatticeConfig().to_c()
    assert lib.pog_validate_params(ctypes.byref(p)) == 0
    with pytest.raises(_lib.PogError):
        _lib.check(-1)


def _c_layout(struct, fields):
    prog = ["#include <stdio.h>", "#include <stddef.h>", '#include "%s"' % HEADER, "int main(void){",
            'printf("%%zu\\n", sizeof(%s));' % struct]
    for f in fields:
        prog.append('printf("%%zu\\n", offsetof(%s, %s));' % (struct, f))
    prog.append("return 0;}")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "l.c")
        exe = os.path.join(d, "l")
        open(c, "w").write("\n".join(prog))
        subprocess.run(["gcc", "-o", exe, c], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    return [int(x) for x in out]


@pytest.mark.parametrize("struct,cls", [("pog_params", PogParams), ("pog_particle_params", PogParticleParams)])
def test_struct_layout_matches_ctypes(struct, cls):
    names = [f[0] for f in cls._fields_]
    got = _c_layout(struct, names)
    assert got[0] == ctypes.sizeof(cls)
    for name, off in zip(names, got[1:]):
        assert getattr(cls, name).offset == off, name
