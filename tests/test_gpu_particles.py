"""GPU parity of the particle path through the C ABI.

Bit-exact: cell keys, the stable cell order (== numpy argsort(kind="stable")), and in
deterministic mode every per-particle output plus the fixed-point drag deposit (Kp, Kv).  The
float-atomic (warp-aggregated) deposit agrees with the fixed-point one to FP32 summation error.
"""
import ctypes
import os

import numpy as np
import pytest
import torch

from gpu_helpers import P, S, lib
from pour_over_coffee_lbm_gb300 import _lib
from pour_over_coffee_lbm_gb300.params import LatticeConfig, ParticleConfig, seed_particles

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "oracle_small.npz")


def gpu_bin(cfg, pos, active):
    n = active.shape[0]
    p = cfg.to_c()
    pos_t = torch.as_tensor(np.ascontiguousarray(pos, np.float32)).cuda()
    act_t = torch.as_tensor(np.ascontiguousarray(active, np.int32)).cuda()
    keys = torch.zeros(n, dtype=torch.int32, device="cuda")
    perm = torch.zeros(n, dtype=torch.int32, device="cuda")
    scratch = torch.empty(int(lib().pog_particles_bin_scratch_bytes(n)), dtype=torch.uint8, device="cuda")
    _lib.check(lib().pog_particles_bin(ctypes.byref(p), P(pos_t), P(act_t), n, P(keys), P(perm), P(scratch), S()))
    return keys.cpu().numpy(), perm.cpu().numpy()


def gpu_couple(cfg, pc, pos, vel, d, drag, act, u, order=None, deterministic=True):
    n = d.shape[0]
    p = cfg.to_c()
    pp = pc.to_c()
    pp.deterministic = int(deterministic)
    T = lambda a, dt=np.float32: torch.as_tensor(np.ascontiguousarray(a, dt)).cuda()  # noqa: E731
    pos_t, vel_t, d_t, drag_t, act_t, u_t = T(pos), T(vel), T(d), T(drag), T(act, np.int32), T(u)
    ord_t = None if order is None else T(order, np.int32)
    fix = torch.zeros(4 * cfg.ncell, dtype=torch.int64, device="cuda")
    force = torch.zeros(4 * cfg.ncell, dtype=torch.float32, device="cuda")
    uat = torch.zeros((3, n), dtype=torch.float32, device="cuda")
    _lib.check(lib().pog_particles_couple(ctypes.byref(p), ctypes.byref(pp), P(pos_t), P(vel_t), P(d_t),
                                          P(drag_t), P(act_t), n, P(ord_t), P(u_t),
                                          None if deterministic else P(force), P(fix) if deterministic else None,
                                          P(uat), S()))
    torch.cuda.synchronize()
    c = lambda t: t.cpu().numpy()  # noqa: E731
    return c(pos_t), c(vel_t), c(drag_t), c(act_t), c(fix), c(force), c(uat)


def test_bin_sort_fixture(cuda):
    g = np.load(GOLD)
    cfg = LatticeConfig(nx=16, ny=16, nz=16, cone_apex_z=3.0)
    keys, perm = gpu_bin(cfg, g["particles/pos"], g["particles/active"])
    assert np.array_equal(keys, g["particles/keys"])
    assert np.array_equal(perm, g["particles/perm"])


@pytest.mark.parametrize("n,grid", [(1, 16), (511, 24), (513, 24), (20000, 128), (200000, 96), (1000, 300)])
def test_bin_sort_random_vs_oracle(cuda, orc, n, grid):
    """Random positions including out-of-range, negative and NaN coordinates and inactive
    particles; many particles per cell for the small grids (ties keep id order)."""
    rng = np.random.default_rng(n + grid)
    cfg = LatticeConfig(nx=grid, ny=grid, nz=max(16, grid // 2))
    pos = np.stack([rng.uniform(-3, cfg.nx + 3, n), rng.uniform(-3, cfg.ny + 3, n),
                    rng.uniform(-3, cfg.nz + 3, n)]).astype(np.float32)
    if n > 10:
        pos[0, :: max(1, n // 7)] = np.nan
        pos[:, 1::13] = np.floor(pos[:, 1::13])  # exact integers (cell faces)
    act = (rng.uniform(size=n) > 0.1).astype(np.int32)
    keys, perm = gpu_bin(cfg, pos, act)
    ok, op = orc.particles_bin(cfg, pos, act)
    assert np.array_equal(keys, ok)
    assert np.array_equal(perm, op)
    assert np.array_equal(perm, np.argsort(ok, kind="stable"))


def test_bin_empty(cuda):
    cfg = LatticeConfig(nx=16, ny=16, nz=16)
    p = cfg.to_c()
    assert lib().pog_particles_bin(ctypes.byref(p), None, None, 0, None, None, None, S()) == 0
    assert lib().pog_particles_couple(ctypes.byref(p), ctypes.byref(ParticleConfig().to_c()), None, None,
                                      None, None, None, 0, None, None, None, None, None, S()) == 0


def test_couple_fixture_bit_exact(cuda):
    g = np.load(GOLD)
    cfg = LatticeConfig(nx=16, ny=16, nz=16, cone_apex_z=3.0)
    pc = ParticleConfig(count=600, deterministic=True)
    pos, vel, drag, act, fix, _, uat = gpu_couple(cfg, pc, g["particles/pos"], g["particles/vel"], g["particles/d"],
                                                  np.zeros_like(g["particles/pos"]), g["particles/active"],
                                                  g["particles/u"], order=g["particles/perm"])
    assert np.array_equal(pos, g["particles/pos_out"])
    assert np.array_equal(vel, g["particles/vel_out"])
    assert np.array_equal(drag, g["particles/drag_out"])
    assert np.array_equal(act, g["particles/active_out"])
    assert np.array_equal(uat, g["particles/u_at"])
    assert np.array_equal(fix, g["particles/force_fix"])


def _flow(cfg, rng):
    z, y, x = np.meshgrid(np.arange(cfg.nz), np.arange(cfg.ny), np.arange(cfg.nx), indexing="ij")
    return np.stack([0.02 * np.sin(0.11 * y + 0.3), 0.015 * np.cos(0.07 * x), -0.01 + 0.004 * np.sin(0.05 * z)]).astype(np.float32)


@pytest.mark.parametrize("drag_model", [0, 1])
def test_couple_random_vs_oracle(cuda, orc, drag_model):
    """20,000 particles on 128^3 (the coupled case's count): deterministic mode bit-exact
    (Stokes) / within 1e-6 (Schiller-Naumann uses powf); fast warp-aggregated atomics within
    FP32 summation error of the fixed-point grid."""
    rng = np.random.default_rng(11)
    cfg = LatticeConfig(nx=128, ny=128, nz=128, band_thickness=3.0)
    pc = ParticleConfig(count=20000, drag_model=drag_model)
    pos, vel, d, act = seed_particles(cfg, pc)
    vel = (rng.normal(size=vel.shape) * 0.01).astype(np.float32)
    drag = (rng.normal(size=vel.shape) * 1e-3).astype(np.float32)
    act[::101] = 0
    u = _flow(cfg, rng)
    _, order = orc.particles_bin(cfg, pos, act)
    o = orc.particles_couple(cfg, pc, pos, vel, d, drag, act, u)
    gd = gpu_couple(cfg, pc, pos, vel, d, drag, act, u, order=order, deterministic=True)
    if drag_model == 0:
        for a, b in zip(gd[:4], o[:4]):
            assert np.array_equal(a, b)
        assert np.array_equal(gd[4], o[4])
    else:
        for a, b in zip(gd[:3], o[:3]):
            assert np.allclose(a, b, rtol=1e-6, atol=1e-9)
    # fast mode, unsorted and sorted processing order: same per-particle results
    for order_used in (None, order):
        gf = gpu_couple(cfg, pc, pos, vel, d, drag, act, u, order=order_used, deterministic=False)
        assert np.array_equal(gf[0], gd[0]) and np.array_equal(gf[1], gd[1])
        ref = gd[4].astype(np.float64) / 2.0 ** 32
        got = gf[5].astype(np.float64)
        assert np.abs(got - ref).max() <= 1e-6 * max(1e-12, np.abs(ref).max()) + 1e-9


def test_couple_nonfinite_deactivates(cuda, orc):
    cfg = LatticeConfig(nx=32, ny=32, nz=32)
    pc = ParticleConfig(count=64)
    pos, vel, d, act = seed_particles(cfg, pc)
    vel[:, 5] = np.inf
    u = np.zeros((3, 32, 32, 32), np.float32)
    g = gpu_couple(cfg, pc, pos, vel, d, np.zeros_like(pos), act, u)
    o = orc.particles_couple(cfg, pc, pos, vel, d, np.zeros_like(pos), act, u)
    assert g[3][5] == 0 and o[3][5] == 0
    assert np.array_equal(g[3], o[3])


@pytest.mark.parametrize("sorted_order", [False, True])
def test_drag_from_fixed_cells_equals_full_conversion(cuda, orc, sorted_order):
    """pog_drag_from_fixed_cells converts the deterministic deposit at the particles' cells only:
    added to a field that already holds values, it gives exactly that field plus
    pog_drag_from_fixed's conversion, and it leaves the fixed-point field all zeros (20,000
    particles on 128^3, many sharing cells)."""
    rng = np.random.default_rng(5)
    cfg = LatticeConfig(nx=128, ny=128, nz=128, band_thickness=3.0)
    pc = ParticleConfig(count=20000)
    pos, vel, d, act = seed_particles(cfg, pc)
    act[::97] = 0
    u = torch.as_tensor(_flow(cfg, rng)).cuda()
    n = d.shape[0]
    p = cfg.to_c()
    pp = pc.to_c()
    pp.deterministic = 1
    dep = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    pp.deposit_cells = dep.data_ptr()
    T = lambda a, dt=np.float32: torch.as_tensor(np.ascontiguousarray(a, dt)).cuda()  # noqa: E731
    pos_t, vel_t, d_t, act_t = T(pos), T(vel), T(d), T(act, np.int32)
    drag_t = torch.zeros_like(vel_t)
    order = None
    if sorted_order:
        _, o = orc.particles_bin(cfg, pos, act)
        order = T(o, np.int32)
    fix = torch.zeros(4 * cfg.ncell, dtype=torch.int64, device="cuda")
    _lib.check(lib().pog_particles_couple(ctypes.byref(p), ctypes.byref(pp), P(pos_t), P(vel_t), P(d_t), P(drag_t),
                                          P(act_t), n, P(order), P(u), None, P(fix), None, S()))
    base = torch.randn(4 * cfg.ncell, device="cuda")  # values already in the field
    full = torch.empty_like(base)
    _lib.check(lib().pog_drag_from_fixed(ctypes.byref(p), P(fix), P(full), S()))
    cells = base.clone()
    _lib.check(lib().pog_drag_from_fixed_cells(ctypes.byref(p), P(fix), P(dep), n, P(order), P(cells), S()))
    torch.cuda.synchronize()
    assert int((dep >= 0).sum()) > 0 and int((dep == -7).sum()) == 0
    assert int(torch.count_nonzero(full)) > 0
    assert torch.equal(cells, base + full)
    assert int(torch.count_nonzero(fix)) == 0
