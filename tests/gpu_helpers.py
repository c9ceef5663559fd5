"""Thin C-ABI drivers used by the GPU parity tests: every call goes through libpog.so's
extern "C" entry points (ctypes), on torch-owned device buffers."""
import ctypes

import numpy as np
import torch

from pour_over_coffee_lbm_gb300 import _lib
from pour_over_coffee_lbm_gb300.params import (LES_STENCIL, RED_COUNT, STEP_CELLS, STORE_BF16S, STORE_F16S,
                                               STORE_F32, STORE_F64)

DT = {STORE_F32: torch.float32, STORE_F16S: torch.float16, STORE_BF16S: torch.bfloat16,
      STORE_F64: torch.float64}


def lib():
    return _lib.load()


def S():
    return _lib.stream_handle()


def P(t):
    return _lib.ptr(t)


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (d if d > 0 else 1.0))


def gpu_flags(cfg):
    p = cfg.to_c()
    fl = torch.empty((cfg.nz, cfg.ny, cfg.nx), dtype=torch.int32, device="cuda")
    _lib.check(lib().pog_build_flags(ctypes.byref(p), P(fl), S()))
    return fl


def wall_list(p, flags):
    """The row-tiled step's bounce-back cell list (pog_wall_list: count, allocate, fill)."""
    count = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.check(lib().pog_wall_list(ctypes.byref(p), P(flags), None, 0, P(count), S()))
    n = int(count.item())
    cells = torch.empty(n, dtype=torch.int32, device="cuda")
    _lib.check(lib().pog_wall_list(ctypes.byref(p), P(flags), P(cells) if n else None, n, P(count), S()))
    assert int(count.item()) == n
    return cells


class AARun:
    """AA-pattern state driven through pog_step."""

    def __init__(self, cfg, flags=None, eps=None, force=None, pdrag=None, rows=False, cells=False,
                 ref_density=False):
        self.cfg = cfg
        self.p = cfg.to_c()
        if cells:
            self.p.step_kernel = STEP_CELLS  # the per-cell kernel even where the two-cell one applies
        self.dref = None
        if ref_density:  # FP16S relative to per-cell reference densities (set by the init below)
            self.dref = torch.zeros(cfg.ncell, dtype=torch.float16, device="cuda")
            self.p.density_ref = self.dref.data_ptr()
        shape = (cfg.nz, cfg.ny, cfg.nx)
        self.flags = gpu_flags(cfg) if flags is None else torch.as_tensor(np.asarray(flags).astype(np.int32)).cuda()
        self.walls = None
        if rows:
            self.walls = wall_list(self.p, self.flags)
            self.p.wall_cells = P(self.walls)
            self.p.n_wall_cells = int(self.walls.numel()) if self.walls.numel() > 0 else 0
        self.f = torch.empty((19,) + shape, dtype=DT[cfg.storage], device="cuda")
        self.rho = torch.zeros(shape, dtype=torch.float32, device="cuda")
        self.u = torch.zeros((3,) + shape, dtype=torch.float32, device="cuda")
        self.ul = [torch.zeros((3,) + shape, dtype=torch.float32, device="cuda") for _ in range(2)]
        self.eps = None if eps is None else torch.as_tensor(np.asarray(eps, np.float32)).cuda()
        self.force = None if force is None else torch.as_tensor(np.asarray(force, np.float32)).cuda()
        self.pdrag = None if pdrag is None else torch.as_tensor(np.asarray(pdrag, np.float32)).cuda()
        self.red = torch.zeros(RED_COUNT, dtype=torch.float64, device="cuda")
        self.t = 0
        _lib.check(lib().pog_init_equilibrium(ctypes.byref(self.p), P(self.f), P(self.flags),
                                              float(cfg.rho0), 0.0, 0.0, 0.0, S()))

    def step(self, n, reduce=False, macro=True):
        stencil = self.cfg.les_mode == LES_STENCIL
        _lib.check(lib().pog_step(ctypes.byref(self.p), P(self.f), P(self.flags), self.t, n,
                                  P(self.force), P(self.pdrag), P(self.eps),
                                  P(self.ul[0]) if stencil else None, P(self.ul[1]) if stencil else None,
                                  P(self.rho) if macro else None, P(self.u) if macro else None,
                                  P(self.red) if reduce else None, S()))
        if stencil and n % 2 == 1:
            self.ul.reverse()
        self.t += n

    def natural(self, dtype=np.float64):
        out_store = STORE_F64 if dtype == np.float64 else STORE_F32
        shape = (19, self.cfg.nz, self.cfg.ny, self.cfg.nx)
        nat = torch.empty(shape, dtype=torch.float64 if dtype == np.float64 else torch.float32, device="cuda")
        _lib.check(lib().pog_export_natural(ctypes.byref(self.p), P(self.f), P(self.flags), self.t,
                                            P(nat), out_store, S()))
        return nat.cpu().numpy()


def run_aa(cfg, steps, eps=None, force=None, reduce=True, pdrag=None, rows=False, cells=False):
    r = AARun(cfg, eps=eps, force=force, pdrag=pdrag, rows=rows, cells=cells)
    if steps > 1:
        r.step(steps - 1, reduce=reduce, macro=False)
    r.step(1, reduce=reduce, macro=True)
    torch.cuda.synchronize()
    assert lib().pog_device_status(1) == 0, lib().pog_last_error()
    return r


def run_push(cfg, steps, flags=None, eps=None, reduce=True):
    """Natural-layout two-buffer run through pog_step_push."""
    p = cfg.to_c()
    shape = (cfg.nz, cfg.ny, cfg.nx)
    fl = gpu_flags(cfg) if flags is None else flags
    a = torch.empty((19,) + shape, dtype=DT[cfg.storage], device="cuda")
    b = torch.zeros_like(a)
    _lib.check(lib().pog_init_equilibrium(ctypes.byref(p), P(a), P(fl), float(cfg.rho0), 0.0, 0.0, 0.0, S()))
    rho = torch.zeros(shape, dtype=torch.float32, device="cuda")
    u = torch.zeros((3,) + shape, dtype=torch.float32, device="cuda")
    up = torch.zeros_like(u)
    red = torch.zeros(RED_COUNT, dtype=torch.float64, device="cuda")
    e = None if eps is None else torch.as_tensor(np.asarray(eps, np.float32)).cuda()
    for i in range(steps):
        _lib.check(lib().pog_step_push(ctypes.byref(p), P(a), P(b), P(fl), None, None, P(e),
                                       P(up) if cfg.les_mode == LES_STENCIL else None,
                                       P(rho), P(u), P(red) if reduce else None, S()))
        up.copy_(u)
        a, b = b, a
    torch.cuda.synchronize()
    return a, rho, u, red, fl
