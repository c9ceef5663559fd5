"""Build libpog.so in-tree with nvcc for sm_103a (GB300).

Each .cu file compiles in parallel to an object, then one shared-library link.  geometry.cu and
particles.cu are compiled with -fmad=false (bit-exact integer geometry and particle
arithmetic); the lattice kernels keep FMA contraction.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpog.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# FP32 reciprocal/sqrt/denormal flags apply to single precision only (FP64 paths unaffected)
FAST_F32 = ["-prec-div=false", "-prec-sqrt=false", "-ftz=true"]
SOURCES = {
    "api.cu": [],
    "geometry.cu": ["-fmad=false"],
    "lbm_aa.cu": FAST_F32,
    "lbm_tma.cu": FAST_F32,
    "lbm_pair.cu": FAST_F32,
    "lbm_ref.cu": FAST_F32,
    "lbm_push.cu": [],
    "particles.cu": ["-fmad=false"],
    "particles_noalloc.cu": [],
    "adjoint.cu": FAST_F32,
    "pour.cu": [],
    "diag.cu": [],
    "filter.cu": ["-fmad=false"],
    "drive.cu": ["-fmad=false"],
    "multiphase.cu": ["-fmad=false"],
}
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpog.so")


def _deps():
    out = [os.path.join(HERE, "..", "include", "pog.h")]
    for f in os.listdir(CSRC):
        out.append(os.path.join(CSRC, f))
    return out


def build(force: bool = False, verbose: bool = False, extra=None) -> str:
    deps = _deps()
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in deps):
            return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    extra = list(extra or [])

    def compile_one(item):
        src, flags = item
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [cc] + ARCH + COMMON + flags + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, flush=True)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES.items()))
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    args = sys.argv[1:]
    extra = []
    if "--ptxas-v" in args:
        extra = ["-Xptxas", "-v"]
    print(build(force="--force" in args or bool(extra), verbose=True, extra=extra))
