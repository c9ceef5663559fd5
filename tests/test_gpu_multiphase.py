"""The multiphase phase field on the GPU against the oracle: the phase kernels bit for bit, the
pour stream's phase change, the FP64 lattice step reading a phase indicator, and
MultiphaseFlow3D in the reference's step order (pour phase change, surface tension before the
collision, lattice step, phase-field step) checked step by step against the oracle."""
import ctypes

import numpy as np
import pytest
import torch

from gpu_helpers import AARun, P, S, lib, rel_l2
from pour_over_coffee_lbm_gb300 import _lib
from pour_over_coffee_lbm_gb300.params import CELL_SOLID, LES_LOCAL, STORE_F64, LatticeConfig
from test_multiphase_oracle import _droplet
from test_pour_oracle import _block

pytestmark = pytest.mark.gpu

f32 = np.float32


def _T(a, dt=np.float32):
    return torch.as_tensor(np.ascontiguousarray(a, dt)).cuda()


def _case(orc, n=40):
    cfg = LatticeConfig(nx=n, ny=n - 4, nz=n + 4, band_thickness=3.0)
    flags = orc.build_flags(cfg)
    phi = _droplet(flags.shape, (n / 2, (n - 4) / 2, (n + 4) / 2), 7.0)
    return cfg, flags, phi


def test_phase_kernels_bit_exact(cuda, orc):
    cfg, flags, phi = _case(orc)
    shape = flags.shape
    rng = np.random.default_rng(3)
    p = cfg.to_c()
    fl_t, phi_t = _T(flags, np.int32), _T(phi)
    # chemical potential
    mu = np.zeros(shape, f32)
    orc.phase_chemical_potential(cfg, phi, 0.0027, mu)
    mu_t = torch.zeros(shape, dtype=torch.float32, device="cuda")
    _lib.check(lib().pog_phase_chemical_potential(ctypes.byref(p), P(phi_t), 0.0027, P(mu_t), S()))
    # normals
    normal, gmag = np.zeros((3,) + shape, f32), np.zeros(shape, f32)
    orc.phase_normals(cfg, phi, normal, gmag)
    n_t = torch.zeros((3,) + shape, dtype=torch.float32, device="cuda")
    g_t = torch.zeros(shape, dtype=torch.float32, device="cuda")
    _lib.check(lib().pog_phase_normals(ctypes.byref(p), P(phi_t), P(n_t), P(g_t), S()))
    # surface tension into a body force
    rho = (0.002 + rng.uniform(size=shape)).astype(f32)
    force = rng.normal(0, 1e-5, (3,) + shape).astype(f32)
    kap, F, bf = np.zeros(shape, f32), np.zeros((3,) + shape, f32), force.copy()
    orc.phase_surface_tension(cfg, flags, phi, normal, gmag, rho, 0.0036, bf, kap, F)
    rho_t, bf_t = _T(rho), _T(force)
    k_t = torch.zeros(shape, dtype=torch.float32, device="cuda")
    F_t = torch.zeros((3,) + shape, dtype=torch.float32, device="cuda")
    _lib.check(lib().pog_phase_surface_tension(ctypes.byref(p), P(fl_t), P(phi_t), P(n_t), P(g_t), P(rho_t), 0.0036,
                                               P(bf_t), P(k_t), P(F_t), S()))
    # phase update with and without mu, then the properties
    u = rng.normal(0, 0.05, (3,) + shape).astype(f32)
    u_t = _T(u)
    outs = []
    for m, m_t in ((None, None), (mu, mu_t)):
        pn, r, ph = np.zeros(shape, f32), np.zeros(shape, f32), np.zeros(shape, f32)
        orc.phase_update(cfg, flags, phi, pn, u, m, 0.001, 1.0, 0.0012472806, 1.0, r, ph)
        pn_t, r_t, ph_t = (torch.zeros(shape, dtype=torch.float32, device="cuda") for _ in range(3))
        _lib.check(lib().pog_phase_update(ctypes.byref(p), P(fl_t), P(phi_t), P(pn_t), P(u_t), P(m_t), 0.001, 1.0,
                                          0.0012472806, 1.0, P(r_t), P(ph_t), S()))
        outs.append(((pn, r, ph), (pn_t, r_t, ph_t)))
    r2, p2 = np.zeros(shape, f32), np.zeros(shape, f32)
    orc.phase_properties(cfg, phi, 0.0012472806, 1.0, r2, p2)
    r2_t, p2_t = torch.zeros_like(phi_t), torch.zeros_like(phi_t)
    _lib.check(lib().pog_phase_properties(ctypes.byref(p), P(phi_t), 0.0012472806, 1.0, P(r2_t), P(p2_t), S()))
    torch.cuda.synchronize()
    assert np.array_equal(mu_t.cpu().numpy(), mu)
    assert np.array_equal(n_t.cpu().numpy(), normal) and np.array_equal(g_t.cpu().numpy(), gmag)
    assert np.array_equal(k_t.cpu().numpy(), kap) and np.array_equal(F_t.cpu().numpy(), F)
    assert np.array_equal(bf_t.cpu().numpy(), bf) and not np.array_equal(bf, force)
    for ref, got in outs:
        for a, b in zip(ref, got):
            assert np.array_equal(b.cpu().numpy(), a)
    assert np.array_equal(r2_t.cpu().numpy(), r2) and np.array_equal(p2_t.cpu().numpy(), p2)


def test_pour_phase_matches_oracle(cuda, orc):
    cfg = LatticeConfig(nx=40, ny=40, nz=40, band_thickness=3.0)
    flags = orc.build_flags(cfg)
    phi = np.full(flags.shape, -1.0, f32)
    hb = _block(19.4, 20.7, ztop=30.0, diameter=6.0)
    p = cfg.to_c()
    hb_t = _T(hb)
    p.pour_control = hb_t.data_ptr()
    fl_t, phi_t = _T(flags, np.int32), _T(phi)
    for _ in range(5):
        orc.pour_phase(cfg, flags, phi, 0.4, hb)
        _lib.check(lib().pog_pour_phase(ctypes.byref(p), P(fl_t), P(phi_t), 0.4, S()))
    torch.cuda.synchronize()
    assert (phi > -0.5).sum() > 30
    assert np.allclose(phi_t.cpu().numpy(), phi, rtol=0, atol=1e-5)


@pytest.mark.parametrize("les", [0, LES_LOCAL])
def test_phase_step_fp64_matches_oracle(cuda, orc, les):
    cfg = LatticeConfig(nx=32, ny=32, nz=36, storage=STORE_F64, band_thickness=3.0, u_inlet=-0.03, les_mode=les,
                        tau_air=0.9, gravity=(0.0, 0.0, -5e-5))
    r = AARun(cfg)
    flags = r.flags.cpu().numpy().astype(np.uint32)
    # water in the lower half, an interface band, air above; some cells in (0.001, 0.5)
    z = np.arange(cfg.nz, dtype=np.float64)[:, None, None]
    phase = np.broadcast_to(np.clip(0.5 - (z - 18) / 6.0, 0.0, 1.0), flags.shape).astype(f32)
    ph_t = _T(phase)
    r.p.phase = ph_t.data_ptr()
    r.p.tau_air = 0.9
    steps = 13
    r.step(steps)
    f = orc.init_equilibrium(cfg, flags, np.float64)
    for _ in range(steps):
        f, rho, u = orc.step(cfg, flags, f, phase=phase)
    torch.cuda.synchronize()
    fluid = (flags & 1) == 0
    assert rel_l2(r.u.cpu().numpy()[:, fluid], u[:, fluid]) < 1e-6
    assert rel_l2(r.natural()[:, fluid], f[:, fluid]) < 1e-9


def test_multiphase_flow_matches_oracle_step_by_step(cuda, orc):
    from pour_over_coffee_lbm_gb300.multiphase import MultiphaseFlow3D
    from pour_over_coffee_lbm_gb300.pouring import PrecisePouringSystem
    from pour_over_coffee_lbm_gb300.solver import GB300LBMSolver
    cfg = LatticeConfig(nx=40, ny=40, nz=44, band_thickness=3.0, u_inlet=-0.02)
    s = GB300LBMSolver(cfg)
    mp = MultiphaseFlow3D(s)
    mp.standardize_initial_state(force_dry_state=True)
    st0 = mp.validate_initial_phase_consistency()
    assert st0["dry"] and st0["out_of_range"] == 0 and st0["density_inconsistent"] == 0
    pour = PrecisePouringSystem(cfg, diameter=6.0)
    pour.start_pouring()
    flags = s._flags.cpu().numpy().astype(np.uint32)
    mu0 = mp.mu.cpu().numpy()
    for step in range(14):
        s.clear_body_force()
        pour.apply_pouring_force(s)
        pour.apply_gradual_phase_change(mp, dt=1.0)
        phi0 = mp.phi.cpu().numpy()
        rho0 = s._rho.cpu().numpy()
        if step > 10:
            mp.accumulate_surface_tension_pre_collision()
            force = s._force.cpu().numpy()
            # oracle: the same surface tension from the same phi and rho
            n_, g_ = np.zeros((3,) + phi0.shape, f32), np.zeros(phi0.shape, f32)
            orc.phase_normals(cfg, phi0, n_, g_)
            bf = np.zeros((3,) + phi0.shape, f32)
            orc.phase_surface_tension(cfg, flags, phi0, n_, g_, rho0, mp.SURFACE_TENSION_COEFF, bf)
            assert np.array_equal(force, bf)
        s.run(1, want_macro=True)
        u = s._u.cpu().numpy()
        mp.step(step, precollision_applied=True)
        pn, rr, pp = (np.zeros(phi0.shape, f32) for _ in range(3))
        orc.phase_update(cfg, flags, phi0, pn, u, mu0, mp.MOBILITY, mp.DT, mp.RHO_AIR, mp.RHO_WATER, rr, pp)
        assert np.array_equal(mp.phi.cpu().numpy(), pn), step
        assert np.array_equal(s._rho.cpu().numpy(), rr) and np.array_equal(s._phase.cpu().numpy(), pp)
    st = mp.get_interface_statistics()
    assert st["water_fraction"] > 0 and np.isfinite(st["interface_thickness"])
    assert st["surface_tension_magnitude"] > 0
    assert s.check_stability()
    # the phase density stays the density field until the next step, whatever refreshes u
    s.clear_body_force()
    assert torch.equal(s.rho.tensor, torch.as_tensor(rr).cuda())
    assert ((mp.phi > -1) & ((s._flags & CELL_SOLID) == 0)).any()


def test_multiphase_checkpoint_resume(cuda, tmp_path):
    from pour_over_coffee_lbm_gb300.diagnostics import load_checkpoint, save_checkpoint
    from pour_over_coffee_lbm_gb300.multiphase import MultiphaseFlow3D
    from pour_over_coffee_lbm_gb300.pouring import PrecisePouringSystem
    from pour_over_coffee_lbm_gb300.solver import GB300LBMSolver
    cfg = LatticeConfig(nx=32, ny=32, nz=40, band_thickness=3.0)

    def make():
        s = GB300LBMSolver(cfg)
        mp = MultiphaseFlow3D(s)
        mp.standardize_initial_state()
        pour = PrecisePouringSystem(cfg, diameter=5.0)
        pour.start_pouring(pattern="spiral")
        return s, mp, pour

    def advance(s, mp, pour, n):
        for _ in range(n):
            k = s.step_count
            s.clear_body_force()
            pour.apply_pouring_force(s)
            pour.apply_gradual_phase_change(mp)
            if k > 10:
                mp.accumulate_surface_tension_pre_collision()
            s.run(1, want_macro=True)
            mp.step(k, precollision_applied=True)

    s, mp, pour = make()
    advance(s, mp, pour, 14)
    path = str(tmp_path / "mp.npz")
    save_checkpoint(path, s, pour=pour, multiphase=mp)
    advance(s, mp, pour, 5)
    s2, mp2, pour2 = make()
    load_checkpoint(path, s2, pour=pour2, multiphase=mp2)
    advance(s2, mp2, pour2, 5)
    assert np.array_equal(s2.f.to_numpy(), s.f.to_numpy())
    assert torch.equal(mp2.phi, mp.phi) and torch.equal(s2._rho, s._rho)
