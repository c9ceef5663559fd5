"""pog_particles_bin_noalloc: particle binning and cell sort for callers that may not allocate
device memory while running (the library keeps its sort scratch in a fixed device array).

Checked through the C ABI against pog_particles_bin (caller scratch) on two calls in a row with
different particle sets: keys and the stable order are integers, so they must be identical.
This file runs last so that a failure here leaves every other test already run; it also passes
on its own in a fresh process (the first call resolves the array's device address).  The limit
np = POG_NOALLOC_MAX_PARTICLES is exercised (the sort scratch comes closest to the fixed array
there), np = 0 (the set-up call that reserves the array), and the set-up sequence itself in a
fresh process.
"""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest
import torch

from pour_over_coffee_lbm_gb300 import _lib
from pour_over_coffee_lbm_gb300.params import LatticeConfig

pytestmark = pytest.mark.gpu


def _inputs(n, grid, seed):
    rng = np.random.default_rng(seed)
    pos = np.stack([rng.uniform(-2, grid + 2, n) for _ in range(3)]).astype(np.float32)
    act = (rng.uniform(size=n) > 0.05).astype(np.int32)
    return pos, act


def _run(lib, p, pos, act, noalloc):
    n = act.shape[0]
    pos_t = torch.as_tensor(pos).cuda().contiguous()
    act_t = torch.as_tensor(act).cuda().contiguous()
    keys = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    perm = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    s = _lib.stream_handle()
    if noalloc:
        rc = lib.pog_particles_bin_noalloc(ctypes.byref(p), _lib.ptr(pos_t), _lib.ptr(act_t), n,
                                           _lib.ptr(keys), _lib.ptr(perm), s)
    else:
        scratch = torch.empty(int(lib.pog_particles_bin_scratch_bytes(n)), dtype=torch.uint8, device="cuda")
        rc = lib.pog_particles_bin(ctypes.byref(p), _lib.ptr(pos_t), _lib.ptr(act_t), n,
                                   _lib.ptr(keys), _lib.ptr(perm), _lib.ptr(scratch), s)
    _lib.check(rc)
    torch.cuda.synchronize()
    return keys.cpu().numpy(), perm.cpu().numpy()


def test_noalloc_bin_matches_scratch_version_twice(cuda):
    lib = _lib.load()
    cfg = LatticeConfig(nx=96, ny=96, nz=96)
    p = cfg.to_c()
    # two calls in a row, different sizes: the second reuses the array the first left behind
    for n, seed in ((150000, 1), (20000, 2)):
        pos, act = _inputs(n, 96, seed)
        k_ref, p_ref = _run(lib, p, pos, act, noalloc=False)
        k_na, p_na = _run(lib, p, pos, act, noalloc=True)
        assert np.array_equal(k_na, k_ref)
        assert np.array_equal(p_na, p_ref)
        assert np.array_equal(p_na, np.argsort(k_ref, kind="stable"))


def test_noalloc_rejects_oversize(cuda):
    lib = _lib.load()
    p = LatticeConfig(nx=16, ny=16, nz=16).to_c()
    rc = lib.pog_particles_bin_noalloc(ctypes.byref(p), None, None, (1 << 20) + 1, None, None,
                                       _lib.stream_handle())
    assert rc == -5
    assert b"at most" in lib.pog_last_error()


def test_noalloc_at_the_limit_and_empty(cuda):
    lib = _lib.load()
    cfg = LatticeConfig(nx=128, ny=128, nz=128)
    p = cfg.to_c()
    n = 1 << 20  # POG_NOALLOC_MAX_PARTICLES
    pos, act = _inputs(n, 128, 3)
    k_ref, p_ref = _run(lib, p, pos, act, noalloc=False)
    k_na, p_na = _run(lib, p, pos, act, noalloc=True)
    assert np.array_equal(k_na, k_ref) and np.array_equal(p_na, p_ref)
    assert np.array_equal(p_na, np.argsort(k_ref, kind="stable"))
    rc = lib.pog_particles_bin_noalloc(ctypes.byref(p), None, None, 0, None, None, _lib.stream_handle())
    assert rc == 0


def test_noalloc_setup_call_in_a_fresh_process():
    """A process that makes the np = 0 set-up call first, then bins twice without allocating."""
    code = r"""
import ctypes, sys
import numpy as np, torch
sys.path.insert(0, %r)
from pour_over_coffee_lbm_gb300 import _lib
from pour_over_coffee_lbm_gb300.params import LatticeConfig
L = _lib.load()
p = LatticeConfig(nx=64, ny=64, nz=64).to_c()
s = _lib.stream_handle()
assert L.pog_particles_bin_noalloc(ctypes.byref(p), None, None, 0, None, None, s) == 0
for n, seed in ((50000, 5), (7000, 6)):
    rng = np.random.default_rng(seed)
    pos = torch.as_tensor(np.stack([rng.uniform(0, 64, n) for _ in range(3)]).astype(np.float32)).cuda()
    act = torch.ones(n, dtype=torch.int32, device="cuda")
    k = torch.empty(n, dtype=torch.int32, device="cuda")
    q = torch.empty(n, dtype=torch.int32, device="cuda")
    _lib.check(L.pog_particles_bin_noalloc(ctypes.byref(p), _lib.ptr(pos), _lib.ptr(act), n, _lib.ptr(k), _lib.ptr(q), s))
    torch.cuda.synchronize()
    kk = k.cpu().numpy()
    assert np.array_equal(q.cpu().numpy(), np.argsort(kk, kind="stable"))
print("ok")
""" % os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and "ok" in out.stdout, out.stdout + out.stderr
