"""Filter-paper dynamics on the GPU against the oracle: the particle bounce and deposit
(pog_filter_particles, bit for bit), the blockage update (pog_filter_update), the FP64 step with
a blockage field, and the FilterPaperSystem surface on a coupled run."""
import ctypes

import numpy as np
import pytest
import torch

from gpu_helpers import AARun, P, S, lib, rel_l2
from pour_over_coffee_lbm_gb300 import _lib
from pour_over_coffee_lbm_gb300.params import CELL_POROUS, STORE_F64, LatticeConfig, ParticleConfig

pytestmark = pytest.mark.gpu


def _T(a, dt=np.float32):
    return torch.as_tensor(np.ascontiguousarray(a, dt)).cuda()


def test_filter_particles_bit_exact(cuda, orc):
    cfg = LatticeConfig(nx=40, ny=40, nz=40, band_thickness=3.0)
    flags = orc.build_flags(cfg)
    rng = np.random.default_rng(21)
    por = np.argwhere(flags & CELL_POROUS)
    npart = 20000
    pick = por[rng.integers(0, len(por), npart)]
    pos = (np.stack([pick[:, 2], pick[:, 1], pick[:, 0]]) + rng.uniform(0, 1, (3, npart))).astype(np.float32)
    pos[2] += rng.integers(-2, 3, npart)
    pos[:, :500] = rng.uniform(-3, 43, (3, 500))  # some outside the grid
    vel = rng.normal(0, 0.02, (3, npart)).astype(np.float32)
    active = (rng.uniform(size=npart) > 0.05).astype(np.int32)
    accum = rng.uniform(0, 0.3, flags.size).astype(np.float32)
    v, a = vel.copy(), accum.copy()
    p = cfg.to_c()
    fl_t, pos_t, vel_t, act_t, acc_t = _T(flags, np.int32), _T(pos), _T(vel), _T(active, np.int32), _T(accum)
    for step in range(3):
        orc.filter_particles(cfg, flags, pos, v, active, a, 99, step)
        _lib.check(lib().pog_filter_particles(ctypes.byref(p), P(fl_t), P(pos_t), P(vel_t), P(act_t), npart,
                                              P(acc_t), 99, step, S()))
    torch.cuda.synchronize()
    assert np.array_equal(vel_t.cpu().numpy(), v)
    assert np.array_equal(acc_t.cpu().numpy(), a)  # equal 0.01 addends: any order gives the same sum
    assert (v[2] != vel[2]).sum() > 1000


def test_filter_update_matches_oracle(cuda, orc):
    cfg = LatticeConfig(nx=48, ny=40, nz=44, band_thickness=3.0)
    flags = orc.build_flags(cfg)
    rng = np.random.default_rng(8)
    accum = rng.uniform(0, 40, flags.size).astype(np.float32)
    b = rng.uniform(0, 0.6, flags.size).astype(np.float32)
    p = cfg.to_c()
    fl_t, acc_t, b_t = _T(flags, np.int32), _T(accum), _T(b)
    for _ in range(25):
        orc.filter_update(cfg, flags, accum, b)
        _lib.check(lib().pog_filter_update(ctypes.byref(p), P(fl_t), P(acc_t), P(b_t), S()))
    torch.cuda.synchronize()
    assert np.array_equal(acc_t.cpu().numpy(), accum)
    # device expf and the host's may differ in the last bit
    assert np.allclose(b_t.cpu().numpy(), b, rtol=2e-6, atol=1e-7)


def test_blockage_step_fp64_matches_oracle(cuda, orc):
    cfg = LatticeConfig(nx=32, ny=32, nz=32, storage=STORE_F64, band_thickness=3.0, u_inlet=-0.03)
    steps = 15
    r = AARun(cfg)
    flags = r.flags.cpu().numpy().astype(np.uint32)
    rng = np.random.default_rng(4)
    blk = np.where(flags.reshape(-1) & CELL_POROUS, rng.uniform(0, 0.9, flags.size), 0).astype(np.float32)
    blk_t = _T(blk)
    r.p.filter_blockage = blk_t.data_ptr()
    r.step(steps)
    f = orc.init_equilibrium(cfg, flags, np.float64)
    for _ in range(steps):
        f, rho, u = orc.step(cfg, flags, f, blockage=blk)
    torch.cuda.synchronize()
    fluid = (flags & 1) == 0
    assert rel_l2(r.u.cpu().numpy()[:, fluid], u[:, fluid]) < 1e-6
    assert rel_l2(r.natural()[:, fluid], f[:, fluid]) < 1e-9


def test_adjoint_rejects_blockage(cuda):
    cfg = LatticeConfig(nx=16, ny=16, nz=16, band_thickness=2.0)
    p = cfg.to_c()
    b = torch.zeros(cfg.ncell, dtype=torch.float32, device="cuda")
    p.filter_blockage = b.data_ptr()
    f = torch.zeros((19, cfg.ncell), dtype=torch.float32, device="cuda")
    lam = torch.zeros_like(f)
    fl = torch.zeros(cfg.ncell, dtype=torch.int32, device="cuda")
    rc = lib().pog_adjoint_step(ctypes.byref(p), P(f), P(lam), P(torch.zeros_like(f)), P(fl), None, None, None, None,
                                None, None, None, None, S())
    assert rc != 0


def test_filter_paper_system_coupled(cuda, tmp_path):
    from pour_over_coffee_lbm_gb300.diagnostics import load_checkpoint, save_checkpoint
    from pour_over_coffee_lbm_gb300.filter import FilterPaperSystem
    from pour_over_coffee_lbm_gb300.particles import CoffeeParticleSystem
    from pour_over_coffee_lbm_gb300.solver import GB300LBMSolver
    cfg = LatticeConfig(nx=40, ny=40, nz=48, band_thickness=3.0, u_inlet=-0.03)
    pc = ParticleConfig(count=3000, deterministic=True)

    def make():
        s = GB300LBMSolver(cfg)
        ps = CoffeeParticleSystem(pc.count, lattice=cfg, config=pc)
        ps.seed()
        return s, ps, FilterPaperSystem(s, seed=3)

    def advance(s, ps, fs, n):
        for _ in range(n):
            s.step_with_two_way_coupling(ps)
            fs.step(ps)

    s, ps, fs = make()
    assert s.boundary_manager.filter_system is fs
    st0 = fs.get_filter_statistics()
    assert st0["total_filter_nodes"] == int(((s._flags & CELL_POROUS) != 0).sum().item())
    assert st0["average_blockage"] == 0.0
    advance(s, ps, fs, 30)
    st = fs.get_filter_statistics()
    assert st["max_blockage"] > 0.0 and fs.accumulated_particles.max().item() > 0.0
    assert st["average_resistance"] >= st0["average_resistance"]
    assert np.isfinite(st["average_flow_rate"]) and s.get_diagnostics()["stable"]
    bd = fs.get_coffee_bed_boundary()
    assert bd["get_radius_at_height"](bd["top_z"]) == bd["top_radius_lu"] > 0
    # checkpoint / resume carries the filter state bit for bit
    path = str(tmp_path / "ck.npz")
    save_checkpoint(path, s, ps, filter_system=fs)
    advance(s, ps, fs, 8)
    s2, ps2, fs2 = make()
    load_checkpoint(path, s2, ps2, filter_system=fs2)
    advance(s2, ps2, fs2, 8)
    assert np.array_equal(s2.f.to_numpy(), s.f.to_numpy())
    assert torch.equal(fs2.filter_blockage, fs.filter_blockage)
    assert torch.equal(ps2._vel, ps._vel)
