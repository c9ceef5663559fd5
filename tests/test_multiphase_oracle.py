"""The oracle's multiphase phase field against the reference's formulas restated in numpy
(src/core/multiphase_3d.py: compute_chemical_potential :80-109, compute_gradients :111-132,
compute_curvature :134-149, update_phase_field_cahn_hilliard :151-197, compute_surface_tension_force
:313-331, apply_phase_separation :334-352, apply_surface_tension :354-363,
update_density_from_phase :365-381; precise_pouring.py apply_gradual_phase_change :166-193), and
the lattice step's phase indicator (legacy/lbm_solver.py:558-592)."""
import numpy as np

import oracle as orc
from pour_over_coffee_lbm_gb300.params import CELL_SOLID, LES_LOCAL, STORE_F64, LatticeConfig
from pour_over_coffee_lbm_gb300.pouring import (POUR_ACTIVE, POUR_FLOW, POUR_HEIGHT, POUR_NFIELDS, POUR_RADIUS,
                                                POUR_X, POUR_Y, POUR_ZTOP)

f32 = np.float32


def _droplet(shape, centre, radius, width=2.0):
    """A smooth drop of water (phi = +1 inside) in air."""
    nz, ny, nx = shape
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    r = np.sqrt((x - centre[0]) ** 2 + (y - centre[1]) ** 2 + (z - centre[2]) ** 2)
    return np.tanh((radius - r) / width).astype(f32)


def _sh(a, axis, d):
    """a shifted so that out[c] = a[c + d e_axis] (interior cells only are used)."""
    return np.roll(a, -d, axis=axis)


def _lap(a):
    # reference order: x+, x-, y+, y-, z+, z-, then - 6 a
    return (_sh(a, 2, 1) + _sh(a, 2, -1) + _sh(a, 1, 1) + _sh(a, 1, -1) + _sh(a, 0, 1) + _sh(a, 0, -1)
            - f32(6.0) * a)


def _interior(shape):
    m = np.zeros(shape, bool)
    m[1:-1, 1:-1, 1:-1] = True
    return m


def _reference_normals(phi):
    g = [(_sh(phi, ax, 1) - _sh(phi, ax, -1)) * f32(0.5) for ax in (2, 1, 0)]
    m = np.sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2])
    inner = _interior(phi.shape)
    ok = (m > f32(1e-10)) & inner
    with np.errstate(invalid="ignore", divide="ignore"):
        n = np.stack([np.where(ok, gg / m, f32(0)) for gg in g]).astype(f32)
    return n, np.where(inner, m, f32(0)).astype(f32)


def _reference_tension(phi, n, m, rho, flags, sigma, force):
    inner = _interior(phi.shape)
    kap = ((_sh(n[0], 2, 1) - _sh(n[0], 2, -1)) * f32(0.5) + (_sh(n[1], 1, 1) - _sh(n[1], 1, -1)) * f32(0.5)
           + (_sh(n[2], 0, 1) - _sh(n[2], 0, -1)) * f32(0.5))
    kap = np.where(inner & (m > f32(1e-10)), kap, f32(0)).astype(f32)
    on = inner & (np.abs(phi) < f32(0.9)) & (m > f32(1e-10))
    fm = f32(sigma) * kap * m
    F = np.stack([np.where(on, fm * n[a], f32(0)) for a in range(3)]).astype(f32)
    acc = inner & ((flags & CELL_SOLID) == 0) & (rho > f32(1e-10))
    out = force.copy()
    with np.errstate(invalid="ignore", divide="ignore"):
        for a in range(3):
            out[a] = np.where(acc, force[a] + F[a] / rho, force[a])
    return kap, F, out


def _case(n=20):
    cfg = LatticeConfig(nx=n, ny=n + 2, nz=n + 4, band_thickness=2.0)
    flags = orc.build_flags(cfg)
    phi = _droplet(flags.shape, (n / 2, (n + 2) / 2, (n + 4) / 2), 5.0)
    return cfg, flags, phi


def test_normals_and_surface_tension_match_reference():
    cfg, flags, phi = _case()
    shape = flags.shape
    n_ref, m_ref = _reference_normals(phi)
    normal = np.zeros((3,) + shape, f32)
    gmag = np.zeros(shape, f32)
    orc.phase_normals(cfg, phi, normal, gmag)
    assert np.array_equal(normal, n_ref) and np.array_equal(gmag, m_ref)
    rng = np.random.default_rng(1)
    rho = (0.5 + rng.uniform(size=shape)).astype(f32)
    force = rng.normal(0, 1e-4, (3,) + shape).astype(f32)
    kap_ref, F_ref, force_ref = _reference_tension(phi, n_ref, m_ref, rho, flags, 0.0036, force)
    kap = np.zeros(shape, f32)
    F = np.zeros((3,) + shape, f32)
    bf = force.copy()
    orc.phase_surface_tension(cfg, flags, phi, normal, gmag, rho, 0.0036, bf, kap, F)
    assert np.array_equal(kap, kap_ref) and np.array_equal(F, F_ref) and np.array_equal(bf, force_ref)
    # a drop of radius 5: curvature near the interface ~ -2/r (n points into the water)
    band = (np.abs(phi) < 0.5) & _interior(shape)
    assert abs(float(np.median(kap[band])) + 2 / 5) < 0.15
    assert np.abs(F).max() > 0


def test_chemical_potential_matches_reference():
    cfg, flags, phi = _case(16)
    kappa = 3.0 * 0.0036 * 2.0 / 8.0
    mu = np.zeros(phi.shape, f32)
    orc.phase_chemical_potential(cfg, phi, kappa, mu)
    ref = np.where(_interior(phi.shape), (phi * phi * phi - phi) + (-f32(kappa) * _lap(phi)), f32(0)).astype(f32)
    assert np.array_equal(mu, ref)


def _reference_update(phi, u, mu, flags, mobility, dt, rho_air, rho_water):
    inner = _interior(phi.shape)
    fluid = (flags & CELL_SOLID) == 0
    ux, uy, uz = (np.where(fluid, u[a], f32(0)) for a in range(3))
    dx = np.where(ux > 0, phi - _sh(phi, 2, -1), _sh(phi, 2, 1) - phi)
    dy = np.where(uy > 0, phi - _sh(phi, 1, -1), _sh(phi, 1, 1) - phi)
    dz = np.where(uz > 0, phi - _sh(phi, 0, -1), _sh(phi, 0, 1) - phi)
    conv = -(ux * dx + uy * dy + uz * dz)
    diff = f32(mobility) * _lap(mu) if mu is not None else np.zeros_like(phi)
    pn = phi + f32(dt) * (conv + diff)
    pn = np.maximum(f32(-1), np.minimum(f32(1), pn))
    chem = phi * (phi * phi - f32(1.0)) - f32(0.01) * _lap(phi)
    pn = np.where(np.abs(phi) < f32(0.99), pn + -f32(0.001) * chem * f32(dt), pn)
    pn = np.where(inner, pn, phi).astype(f32)
    pc = np.maximum(f32(-1), np.minimum(f32(1), pn))
    drho = f32(np.float64(rho_water) - np.float64(f32(rho_air)))
    rho = (f32(rho_air) + drho * (pc + f32(1.0)) / f32(2.0)).astype(f32)
    phase = ((pc + f32(1.0)) / f32(2.0)).astype(f32)
    return pn, rho, phase


def test_phase_update_matches_reference():
    cfg, flags, phi = _case()
    rng = np.random.default_rng(2)
    u = rng.normal(0, 0.05, (3,) + phi.shape).astype(f32)
    mu = (0.01 * rng.normal(size=phi.shape)).astype(f32)
    for m in (None, mu):
        ref = _reference_update(phi, u, m, flags, 0.001, 1.0, 0.0012472806, 1.0)
        pn = np.zeros_like(phi)
        rho = np.zeros_like(phi)
        phase = np.zeros_like(phi)
        orc.phase_update(cfg, flags, phi, pn, u, m, 0.001, 1.0, 0.0012472806, 1.0, rho, phase)
        assert np.array_equal(pn, ref[0]) and np.array_equal(rho, ref[1]) and np.array_equal(phase, ref[2])
    r2, p2 = np.zeros_like(phi), np.zeros_like(phi)
    orc.phase_properties(cfg, pn, 0.0012472806, 1.0, r2, p2)
    assert np.array_equal(r2, rho) and np.array_equal(p2, phase)
    assert r2.max() > 0.98 and abs(r2.min() - 0.0012472806) < 1e-4


def test_pour_phase_matches_reference():
    cfg = LatticeConfig(nx=24, ny=24, nz=24, band_thickness=0.0)
    flags = orc.build_flags(cfg)
    phi = np.full(flags.shape, -1.0, f32)
    b = np.zeros(POUR_NFIELDS, f32)
    b[POUR_ACTIVE], b[POUR_X], b[POUR_Y], b[POUR_RADIUS] = 1, 11.6, 12.3, 3.0
    b[POUR_ZTOP], b[POUR_HEIGHT], b[POUR_FLOW] = 18.0, 4.0, 1.3
    ref = phi.copy()
    B = [float(v) for v in b]
    for k in range(cfg.nz):
        for j in range(cfg.ny):
            for i in range(cfg.nx):
                if flags[k, j, i] & CELL_SOLID:
                    continue
                d = np.hypot(i - B[POUR_X], j - B[POUR_Y])
                if d <= B[POUR_RADIUS] and B[POUR_ZTOP] - B[POUR_HEIGHT] <= k <= B[POUR_ZTOP]:
                    inten = np.exp(-0.5 * (d / B[POUR_RADIUS]) ** 2) * np.exp(-(B[POUR_ZTOP] - k) / 2.0)
                    rate = min(max((1.0 - ref[k, j, i]) / 0.05, -2.0), 2.0)
                    ref[k, j, i] = min(max(ref[k, j, i] + rate * inten * 0.5 * B[POUR_FLOW], -1.0), 1.0)
    orc.pour_phase(cfg, flags, phi, 0.5, b)
    assert (phi > -1).sum() > 20
    assert np.allclose(phi, ref, rtol=0, atol=2e-6)


def test_step_phase_indicator():
    """phase = 1 is the single-phase step; phase = 0 drops gravity and relaxes with tau_air;
    phase p in (0.001, 1) scales gravity by p."""
    base = dict(nx=20, ny=20, nz=24, storage=STORE_F64, band_thickness=0.0, u_inlet=-0.03, gravity=(0.0, 0.0, -1e-4))
    cfg = LatticeConfig(les_mode=LES_LOCAL, **base)
    flags = orc.build_flags(cfg)
    f = orc.init_equilibrium(cfg, flags, np.float64)
    one = np.ones(flags.shape, f32)
    fa, fb = f, f
    for _ in range(6):
        fa, _, ua = orc.step(cfg, flags, fa)
        fb, _, ub = orc.step(cfg, flags, fb, phase=one)
    assert np.array_equal(fa, fb) and np.array_equal(ua, ub)
    # air everywhere == no gravity and tau_air
    air = LatticeConfig(tau_air=0.95, **base)
    ref = LatticeConfig(tau=0.95, tau_air=0.95, **{**base, "gravity": (0.0, 0.0, 0.0)})
    fa, fb = f, f
    for _ in range(6):
        fa, _, ua = orc.step(air, flags, fa, phase=np.zeros(flags.shape, f32))
        fb, _, ub = orc.step(ref, flags, fb)
    assert np.array_equal(ua, ub)
    # a water fraction of 0.7 scales gravity (the quiescent column's u_z = g_z phase / 2)
    still = LatticeConfig(**{**base, "u_inlet": 0.0})
    _, _, u7 = orc.step(still, flags, f, phase=np.full(flags.shape, 0.7, f32))
    fl = (flags & 0x7) == 0
    assert np.allclose(u7[2][fl], 0.5 * 0.7 * -1e-4, rtol=1e-9)


# ---- against the reference's own kernels (tests/golden/multiphase_reference.npz, made by
# tests/golden/make_multiphase_golden.py, which runs multiphase_3d.py's kernel source in float32) ----
def test_phase_kernels_match_reference_kernels():
    import os
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "multiphase_reference.npz"))
    nx, ny, nz = z["phi"].shape
    cfg = LatticeConfig(nx=nx, ny=ny, nz=nz)

    def zyx(a):
        return np.ascontiguousarray(a.transpose(2, 1, 0) if a.ndim == 3 else a.transpose(3, 2, 1, 0))
    inner = np.zeros((nz, ny, nx), bool)
    inner[1:-1, 1:-1, 1:-1] = True
    phi = zyx(z["phi"])
    sigma, width = float(z["sigma"]), float(z["width"])
    mu = np.zeros_like(phi)
    orc.phase_chemical_potential(cfg, phi, 3.0 * sigma * width / 8.0, mu)
    assert np.allclose(mu[inner], zyx(z["mu"])[inner], rtol=0, atol=2e-6)
    normal = np.zeros((3, nz, ny, nx), f32)
    gmag = np.zeros_like(phi)
    orc.phase_normals(cfg, phi, normal, gmag)
    ref_n = zyx(z["normal"])
    assert np.allclose(normal[:, inner], ref_n[:, inner], rtol=0, atol=1e-6)
    assert np.allclose(gmag[inner], np.sqrt((zyx(z["grad_phi"]).astype(np.float64) ** 2).sum(0))[inner], atol=1e-6)
    flags = zyx(z["solid"]).astype(np.uint32) * np.uint32(CELL_SOLID)
    body = zyx(z["base"])
    curv = np.zeros_like(phi)
    sf = np.zeros_like(normal)
    orc.phase_surface_tension(cfg, flags, phi, normal, gmag, zyx(z["rho"]), sigma, body, curv, sf)
    assert np.allclose(curv[inner], zyx(z["curvature"])[inner], rtol=0, atol=2e-6)
    assert np.allclose(sf, zyx(z["surface_force"]), rtol=0, atol=1e-8)
    assert np.allclose(body, zyx(z["body_force"]), rtol=1e-6, atol=1e-9)
    assert np.abs(zyx(z["surface_force"])).max() > 1e-5
    # Cahn-Hilliard step with the phase separation, then the density and phase indicator
    phi_new = np.zeros_like(phi)
    rho = np.zeros_like(phi)
    phase = np.zeros_like(phi)
    orc.phase_update(cfg, np.zeros_like(flags), phi, phi_new, zyx(z["u"]), mu, float(z["mobility"]), 1.0,
                     float(z["rho_air"]), float(z["rho_water"]), rho, phase)
    assert np.allclose(phi_new, zyx(z["phi_new"]), rtol=0, atol=2e-6)
    assert np.allclose(rho, zyx(z["rho_out"]), rtol=0, atol=2e-6)
    assert np.allclose(phase, zyx(z["phase_out"]), rtol=0, atol=2e-6)
