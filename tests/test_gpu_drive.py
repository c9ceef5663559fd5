"""The pressure-gradient drive on the GPU against the oracle: pog_pressure_force and
pog_density_drive bit for bit, and the PressureGradientDrive surface on a solver (force, mixed
and density modes, statistics)."""
import ctypes

import numpy as np
import pytest
import torch

from gpu_helpers import P, S, lib
from pour_over_coffee_lbm_gb300 import _lib
from pour_over_coffee_lbm_gb300.params import CELL_SOLID, LatticeConfig

pytestmark = pytest.mark.gpu


def _T(a, dt=np.float32):
    return torch.as_tensor(np.ascontiguousarray(a, dt)).cuda()


def test_pressure_force_bit_exact(cuda, orc):
    cfg = LatticeConfig(nx=40, ny=36, nz=44, band_thickness=3.0)
    flags = orc.build_flags(cfg)
    rng = np.random.default_rng(6)
    rho = (1.0 + 0.05 * rng.normal(size=flags.shape)).astype(np.float32)
    rho[10:12, 5:9, 7:9] = 0.0
    rho[20, 18, 18] = 5.0
    base = rng.normal(0, 1e-3, (3,) + flags.shape).astype(np.float32)
    p = cfg.to_c()
    fl_t, rho_t, F_t = _T(flags, np.int32), _T(rho), _T(base)
    F = base.copy()
    for scale in (1.0, 0.5):
        orc.pressure_force(cfg, flags, rho, F, scale, 0.12)
        _lib.check(lib().pog_pressure_force(ctypes.byref(p), P(fl_t), P(rho_t), P(F_t), scale, 0.12, S()))
    torch.cuda.synchronize()
    assert np.array_equal(F_t.cpu().numpy(), F)
    assert not np.array_equal(F, base)


def test_density_drive_bit_exact(cuda, orc):
    cfg = LatticeConfig(nx=36, ny=40, nz=32, band_thickness=3.0)
    flags = orc.build_flags(cfg)
    rng = np.random.default_rng(9)
    rho = (1.0 + 0.4 * rng.normal(size=flags.shape)).astype(np.float32)
    target = rng.uniform(0.4, 1.8, cfg.nz).astype(np.float32)
    p = cfg.to_c()
    fl_t, rho_t, tg_t = _T(flags, np.int32), _T(rho), _T(target)
    for _ in range(4):
        orc.density_drive(cfg, flags, rho, target, 0.025, 0.001, 0.5, 2.0)
        _lib.check(lib().pog_density_drive(ctypes.byref(p), P(fl_t), P(rho_t), P(tg_t), 0.025, 0.001, 0.5, 2.0, S()))
    torch.cuda.synchronize()
    assert np.array_equal(rho_t.cpu().numpy(), rho)


def test_pressure_gradient_drive_surface(cuda, orc):
    from pour_over_coffee_lbm_gb300.drive import PressureGradientDrive
    from pour_over_coffee_lbm_gb300.solver import GB300LBMSolver
    cfg = LatticeConfig(nx=32, ny=32, nz=40, band_thickness=3.0, u_inlet=-0.03)
    s = GB300LBMSolver(cfg)
    d = PressureGradientDrive(s)
    t = d.target_profile
    assert t[0] == np.float32(0.4) and abs(t[-1] - (1.0 + (39 / 40 - 0.8) / 0.2 * 0.8)) < 1e-5
    assert (t[int(0.3 * 40):int(0.75 * 40)] == 1.0).all()
    s.run(20, want_macro=True)
    flags = s._flags.cpu().numpy().astype(np.uint32)

    # force drive: body force += capped -cs^2 grad(rho)/rho
    d.activate_force_drive(True)
    assert d.get_status() == {"density_drive": False, "force_drive": True, "mixed_drive": False}
    s.clear_body_force()
    rho_np = s.rho.tensor.cpu().numpy()
    d.apply(0)
    F = np.zeros((3,) + flags.shape, np.float32)
    orc.pressure_force(cfg, flags, rho_np, F, 1.0, d.MAX_PRESSURE_FORCE)
    assert np.array_equal(s._force.cpu().numpy(), F) and np.abs(F).max() > 0
    # mixed drive: half of it
    d.activate_mixed_drive(True)
    s.clear_body_force()
    d.apply(1)
    assert np.array_equal(s._force.cpu().numpy(), np.float32(0.5) * F)
    s.run(1, want_macro=True)

    # density drive: rho moves toward the target by at most 0.001, the next step recomputes it
    d.activate_density_drive(True)
    before = s.rho.tensor.clone()
    d.apply(2)
    after = s.rho.tensor.clone()
    fluid = (s._flags & CELL_SOLID) == 0
    delta = (after - before)[fluid]
    assert delta.abs().max().item() <= 0.001 + 1e-7 and delta.abs().max().item() > 0
    st = d.get_statistics()
    assert st["max_pressure"] > st["min_pressure"] > 0 and st["pressure_ratio"] > 1
    assert d.check_enhanced_stability() in (0, 1, 2)
    diag = d.get_enhanced_diagnostics()
    assert diag["invalid_count"] == 0 and diag["max_force"] == d.MAX_PRESSURE_FORCE
    s.run(1, want_macro=True)
    assert not torch.equal(s.rho.tensor, after)

    # a force-driven run stays finite
    d.activate_force_drive(True)
    for k in range(30):
        s.clear_body_force()
        d.apply(k)
        s.run(1, want_macro=True)
    assert s.check_stability() and s.get_diagnostics()["stable"]
