"""The pour nozzle on the GPU against the oracle: the device-side nozzle motion
(pog_pour_advance), the stream's force inside the fused step (FP64, a spiral pour advanced every
step), the particle impact in the coupling pass, and the PrecisePouringSystem surface on a
coupled run."""
import ctypes

import numpy as np
import pytest
import torch

from gpu_helpers import AARun, P, S, lib, rel_l2
from pour_over_coffee_lbm_gb300 import _lib
from pour_over_coffee_lbm_gb300.params import STORE_F64, LatticeConfig, ParticleConfig, seed_particles
from pour_over_coffee_lbm_gb300.pouring import (POUR_IMPACT, POUR_IMPACT_MAX, POUR_IMPACT_ZMIN, POUR_TIME, POUR_X,
                                                POUR_Y, PrecisePouringSystem)
from test_pour_oracle import _block

pytestmark = pytest.mark.gpu


def test_nozzle_motion_matches_oracle(cuda, orc):
    cfg = LatticeConfig(nx=40, ny=36, nz=24)
    hb = _block(20.0, 18.0, pattern=1, dt=0.9, diameter=3.0)
    db = torch.as_tensor(hb.copy()).cuda()
    p = cfg.to_c()
    p.pour_control = db.data_ptr()
    for _ in range(60):
        _lib.check(lib().pog_pour_advance(ctypes.byref(p), S()))
        orc.pour_advance(cfg, hb)
    got = db.cpu().numpy()
    assert abs(got[POUR_TIME] - hb[POUR_TIME]) < 1e-5
    assert abs(got[POUR_X] - hb[POUR_X]) < 1e-4 and abs(got[POUR_Y] - hb[POUR_Y]) < 1e-4


def test_pour_step_fp64_matches_oracle(cuda, orc):
    cfg = LatticeConfig(nx=32, ny=32, nz=32, storage=STORE_F64, band_thickness=3.0)
    steps = 21
    hb = _block(15.0, 16.0, pattern=1, dt=0.5, ztop=26.0, diameter=5.0)
    db = torch.as_tensor(hb.copy()).cuda()
    r = AARun(cfg)
    r.p.pour_control = db.data_ptr()
    flags = r.flags.cpu().numpy().astype(np.uint32)
    f = orc.init_equilibrium(cfg, flags, np.float64)
    for _ in range(steps):
        _lib.check(lib().pog_pour_advance(ctypes.byref(r.p), S()))
        r.step(1)
        orc.pour_advance(cfg, hb)
        f, rho, u = orc.step(cfg, flags, f, pour=hb)
    torch.cuda.synchronize()
    fluid = (flags & 1) == 0
    nat = r.natural()
    assert rel_l2(r.u.cpu().numpy()[:, fluid], u[:, fluid]) < 1e-6
    assert rel_l2(nat[:, fluid], f[:, fluid]) < 1e-9
    # the stream drives the fluid down: without the pour the same run is much slower there
    ref = AARun(cfg)
    ref.step(steps)
    torch.cuda.synchronize()
    # the stream's planes (k = 22..26, below the inlet plane k = 30)
    assert r.u[2, 22:27].min().item() < ref.u[2, 22:27].min().item() - 5e-3


def test_particle_impact_matches_oracle(cuda, orc):
    cfg = LatticeConfig(nx=48, ny=48, nz=48, band_thickness=0.0)
    pc = ParticleConfig(count=4000, deterministic=True)
    pos, vel, d, act = seed_particles(cfg, pc)
    hb = _block(24.0, 24.0, ztop=30.0, diameter=6.0)
    hb[POUR_IMPACT], hb[POUR_IMPACT_MAX], hb[POUR_IMPACT_ZMIN] = 13.0, 0.02, 6.0
    db = torch.as_tensor(hb.copy()).cuda()
    u = np.zeros((3, 48, 48, 48), np.float32)
    o = orc.particles_couple(cfg, pc, pos, vel, d, np.zeros_like(pos), act, u, pour=hb)
    n = orc.particles_couple(cfg, pc, pos, vel, d, np.zeros_like(pos), act, u)
    p = cfg.to_c()
    p.pour_control = db.data_ptr()
    pp = pc.to_c()
    T = lambda a, dt=np.float32: torch.as_tensor(np.ascontiguousarray(a, dt)).cuda()  # noqa: E731
    pos_t, vel_t, d_t, drag_t, act_t, u_t = T(pos), T(vel), T(d), T(np.zeros_like(pos)), T(act, np.int32), T(u)
    fix = torch.zeros(4 * cfg.ncell, dtype=torch.int64, device="cuda")
    _lib.check(lib().pog_particles_couple(ctypes.byref(p), ctypes.byref(pp), P(pos_t), P(vel_t), P(d_t), P(drag_t),
                                          P(act_t), pc.count, None, P(u_t), None, P(fix), None, S()))
    torch.cuda.synchronize()
    hit = np.abs(o[1] - n[1]).max(axis=0) > 0
    assert hit.sum() > 10  # some particles sit under the stream
    assert np.allclose(vel_t.cpu().numpy(), o[1], rtol=1e-5, atol=1e-7)
    assert np.allclose(pos_t.cpu().numpy(), o[0], rtol=1e-6, atol=1e-5)


def test_precise_pouring_system_surface(cuda):
    from pour_over_coffee_lbm_gb300.particles import CoffeeParticleSystem
    from pour_over_coffee_lbm_gb300.solver import GB300LBMSolver
    cfg = LatticeConfig(nx=48, ny=48, nz=48, band_thickness=3.0)
    solver = GB300LBMSolver(cfg)
    ps = CoffeeParticleSystem(2000, lattice=cfg, config=ParticleConfig(count=2000))
    ps.seed()
    pour = PrecisePouringSystem(cfg, diameter=4.0)
    assert pour.get_pouring_info()["active"] is False
    pour.start_pouring(pattern="spiral")
    pour.create_water_impact_force(ps, max_force=0.05)
    for _ in range(20):
        pour.apply_pouring_force(solver, dt=1.0)
        solver.step_with_two_way_coupling(ps)
    info = pour.get_pouring_info()
    assert info["active"] and info["pattern"] == 1 and abs(info["pour_time"] - 20.0) < 1e-4
    assert info["position"] != (24.0, 24.0)
    assert pour.get_current_flow_rate() > 0
    assert pour.get_pouring_diagnostics()["conditions_check"]["affected_cells"] > 0
    d = solver.get_diagnostics()
    assert d["stable"] and np.isfinite(d["mass"])
    pour.stop_pouring()
    t0 = pour.get_pouring_info()
    assert t0["active"] is False
