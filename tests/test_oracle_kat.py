"""Pins the CPU oracle to the reference's own known-answer tests (CPU only).

Each test restates a check of the reference's test suite (file:line in
latteine1217/pour-over-coffee-lbm) against the oracle's restated function, then the oracle's
small-case outputs are checked against the committed fixtures (tests/golden/).
"""
import math
import os

import numpy as np
import pytest

from pour_over_coffee_lbm_gb300.params import (CELL_POROUS, CELL_SOLID, DRAG_EXPLICIT_CAP,
                                               DRAG_SEMI_IMPLICIT, LES_STENCIL, LatticeConfig,
                                               ParticleConfig, plain_64, seed_particles)

GOLD = os.path.join(os.path.dirname(__file__), "golden", "oracle_small.npz")


# ---- tests/test_lbm_algorithms.py ----------------------------------------------------------
def test_weights_sum_to_one(orc):  # test_lbm_algorithms.py:39-52
    *_, w = orc.tables()
    assert abs(w.sum() - 1.0) < 1e-12


def test_velocity_set_symmetry_and_lengths(orc):  # test_lbm_algorithms.py:54-90
    cx, cy, cz, opp, _ = orc.tables()
    e = np.stack([cx, cy, cz], 1)
    assert np.all(e[0] == 0)
    for q in range(1, 19):
        assert np.all(e[q] + e[opp[q]] == 0)
        assert abs(np.linalg.norm(e[q]) - 1.0) < 1e-10 or abs(np.linalg.norm(e[q]) - math.sqrt(2)) < 1e-10
    # the computed opposite table of legacy/lbm_solver.py:431-439 for config/core.py ordering
    assert opp.tolist() == [0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15]


def test_equilibrium_conservation(orc):  # test_lbm_algorithms.py:99-130
    cx, cy, cz, _, _ = orc.tables()
    rho, u = 1.0, (0.1, 0.05, 0.02)
    feq = orc.equilibrium(rho, u)
    assert abs(feq.sum() - rho) < 1e-12
    mom = np.array([feq @ cx, feq @ cy, feq @ cz])
    assert np.linalg.norm(mom - rho * np.array(u)) < 1e-12


@pytest.mark.parametrize("rho,u", [(0.1, (0, 0, 0)), (10.0, (0, 0, 0)), (1.0, (0.3, 0, 0)),
                                   (1.0, (0.1, 0.1, 0.1)), (1e-6, (0, 0, 0))])
def test_equilibrium_stability(orc, rho, u):  # test_lbm_algorithms.py:132-170
    f = orc.equilibrium(rho, u)
    assert np.all(np.isfinite(f)) and np.all(np.abs(f) < 1e10)


def test_macroscopic_recovery(orc):  # test_lbm_algorithms.py:247-285
    rho, u = 1.2, (0.05, 0.1, 0.15)
    r, uu = orc.moments(orc.equilibrium(rho, u))
    assert abs(r - rho) < 1e-12
    assert np.linalg.norm(uu - np.array(u)) < 1e-12


def test_round_trip_block(orc):  # test_lbm_algorithms.py:302-348
    worst = 0.0
    for i in range(10, 20):
        for j in range(15, 25):
            for k in range(20, 30):
                rho0 = 1.0 + 0.1 * math.sin(i * 0.1)
                u0 = (0.05 * math.cos(j * 0.1), 0.03 * math.sin(k * 0.1), 0.02 * math.cos((i + j + k) * 0.1))
                f0 = orc.equilibrium(rho0, u0)
                r1, u1 = orc.moments(f0)
                f1 = orc.equilibrium(r1, tuple(u1))
                worst = max(worst, float(np.abs(f1 - f0).max()))
    assert worst < 1e-12


# ---- tests/test_trilinear_interpolation.py ---------------------------------------------------
TRILINEAR_POSITIONS = [  # test_trilinear_interpolation.py:145-155
    [5.0, 5.0, 5.0], [5.5, 5.5, 5.5], [5.25, 6.75, 7.1], [0.1, 0.1, 0.1], [14.9, 14.9, 14.9],
    [2.3, 8.7, 11.2], [7.8, 3.4, 9.6], [12.1, 13.5, 4.8], [1.7, 5.9, 14.3], [8.4, 11.2, 6.7]]


def test_trilinear_linear_field_exact(orc):
    """v = (x, y, z) on 16^3 is reproduced at the 10 reference positions.  The reference script
    prints < 1e-10 for FP32 fields; in FP32 arithmetic the attainable bound is a few ulp of the
    coordinate (the interpolation itself is exact for a linear field), so 2e-6 is used."""
    n = 16
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    u = np.stack([x, y, z]).astype(np.float32)
    pos = np.array(TRILINEAR_POSITIONS, np.float32)
    out = orc.trilinear(u, pos)
    assert np.abs(out - pos).max() < 2e-6


def test_trilinear_matches_reference_gather(orc):
    """The reference's own interpolate_fluid_velocity_from_field run on a seeded field at 300
    seeded positions, some outside the grid (tests/golden/trilinear_reference.npz, made by
    tests/golden/make_trilinear_golden.py): same clamping, weights and sum order."""
    import os
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "trilinear_reference.npz"))
    u = np.ascontiguousarray(z["u"].transpose(3, 2, 1, 0))  # (NX,NY,NZ,3) -> (3,NZ,NY,NX)
    out = orc.trilinear(u, z["pos"])
    assert np.array_equal(out, z["out"])  # bit for bit


# ---- tests/test_under_relaxation.py ----------------------------------------------------------
def test_under_relaxation_formula(orc):  # test_under_relaxation.py:108-134
    rng = np.random.default_rng(3)
    fnew = rng.normal(size=30).astype(np.float32)
    fold = rng.normal(size=30).astype(np.float32)
    out, fold2 = orc.under_relax(0.8, fnew, fold)
    a = np.float32(0.8)
    exp = (a * fnew + (np.float32(1.0) - a) * fold).astype(np.float32)
    assert np.array_equal(out, exp)
    assert np.array_equal(fold2, out)  # history updated (coffee_particles.py:1210-1211)


# ---- tests/test_les_turbulence.py -------------------------------------------------------------
def _vortex_u(n):
    # test_les_turbulence.py:40-57
    k, j, i = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    x, y, z = (i - 32) / 32.0, (j - 32) / 32.0, (k - 32) / 32.0
    return np.stack([0.1 * np.sin(2 * 3.14159 * y), 0.1 * np.cos(2 * 3.14159 * x),
                     0.05 * np.sin(3.14159 * z)]).astype(np.float32)


def test_les_zero_velocity_gives_zero(orc):  # test_les_turbulence.py:135-152
    cfg = LatticeConfig(nx=32, ny=32, nz=32, les_mode=LES_STENCIL, cs_smag=0.18)
    fl = orc.build_flags(cfg)
    nu = orc.les_nu(cfg, fl, np.zeros((3, 32, 32, 32), np.float32))
    assert np.allclose(nu, 0.0, atol=1e-10)


def test_les_finite_nonnegative_and_mask(orc):  # test_les_turbulence.py:69-130
    cfg = LatticeConfig(nx=64, ny=64, nz=64, les_mode=LES_STENCIL, cs_smag=0.18, band_thickness=3.0)
    fl = orc.build_flags(cfg)
    nu = orc.les_nu(cfg, fl, _vortex_u(64))
    assert np.all(np.isfinite(nu)) and np.all(nu >= 0) and nu.max() < 1.0
    assert nu.max() > 0.0
    assert np.all(nu[(fl & CELL_POROUS) != 0] == 0.0)  # filter zone masked (filter_paper.py:199)
    # domain shell zero (les_turbulence.py:376-380)
    assert np.all(nu[0] == 0) and np.all(nu[-1] == 0) and np.all(nu[:, 0] == 0) and np.all(nu[:, :, -1] == 0)


# ---- tests/test_forchheimer.py ------------------------------------------------------------------
@pytest.mark.parametrize("mode", [DRAG_SEMI_IMPLICIT, DRAG_EXPLICIT_CAP])
def test_forchheimer_in_band_only(orc, mode):  # test_forchheimer.py:31-74
    cfg = LatticeConfig(nx=48, ny=48, nz=48, band_thickness=3.0, drag_mode=mode)
    fl = orc.build_flags(cfg)
    n = (48, 48, 48)
    rho = np.ones(n, np.float32)
    u = np.zeros((3,) + n, np.float32)
    u[0] = 0.02
    u[2] = -0.015
    F = orc.porous_force(cfg, fl, rho, u)
    mag = np.sqrt((F.astype(np.float64) ** 2).sum(0))
    band = (fl & CELL_POROUS) != 0
    assert band.sum() > 0
    assert mag[band].mean() > 0.0
    assert mag[~band].mean() <= mag[band].mean() + 1e-6
    # drag opposes the velocity
    assert np.all((F[0][band] * u[0][band]) <= 0)


# ---- tests/test_filter_paper.py -----------------------------------------------------------------
def test_filter_band_fraction(orc):  # test_filter_paper.py:44-59
    cfg = plain_64().replace(band_thickness=3.0)
    fl = orc.build_flags(cfg)
    frac = ((fl & CELL_POROUS) != 0).mean()
    assert 0.0 < frac < 0.5
    assert np.all(fl[0] & CELL_SOLID) and np.all(fl[-1] & CELL_SOLID)


# ---- physics sanity of the restated step (tests/test_boundary_conditions.py:71-122) --------------
def test_step_positive_density_no_nan(orc):
    cfg = LatticeConfig(nx=32, ny=32, nz=32, band_thickness=3.0)
    red = np.zeros(6)
    flags, f, rho, u = orc.run(cfg, 30, np.float64, reductions=red)
    fluid = (flags & CELL_SOLID) == 0
    assert np.all(rho[fluid] > 0) and np.all(np.isfinite(u))
    assert red[5] == 0


def test_push_step_conserves_mass_without_inlet_outlet(orc):
    """A closed cone (no inlet/outlet disks) conserves mass to round-off: bounce-back walls and
    Guo forcing do not create mass."""
    cfg = LatticeConfig(nx=24, ny=24, nz=24, inlet_radius=-1.0, hole_radius=-1.0, band_thickness=2.0)
    fl = orc.build_flags(cfg)
    f = orc.init_equilibrium(cfg, fl, np.float64)
    fluid = (fl & CELL_SOLID) == 0
    m0 = f[:, fluid].sum()
    for _ in range(20):
        f, _, _ = orc.step(cfg, fl, f)
    assert abs(f[:, fluid].sum() - m0) / m0 < 1e-12


# ---- committed fixtures ---------------------------------------------------------------------------
def test_oracle_matches_committed_fixtures(orc):
    import sys
    sys.path.insert(0, os.path.dirname(GOLD))
    import make_golden as mg
    g = np.load(GOLD)
    for name, cfg in mg.cases().items():
        red = np.zeros(6)
        flags, f, rho, u = orc.run(cfg, mg.STEPS, np.float64, reductions=red)
        assert np.array_equal(flags, g[name + "/flags"]), name
        assert np.allclose(rho, g[name + "/rho"], rtol=0, atol=1e-13), name
        assert np.allclose(u, g[name + "/u"], rtol=0, atol=1e-13), name
    pc = ParticleConfig(count=600, deterministic=True)
    keys, perm = orc.particles_bin(LatticeConfig(nx=mg.N, ny=mg.N, nz=mg.N, cone_apex_z=3.0),
                                   g["particles/pos"], g["particles/active"])
    assert np.array_equal(keys, g["particles/keys"]) and np.array_equal(perm, g["particles/perm"])
    # the stable order is numpy's stable argsort of the keys
    assert np.array_equal(perm, np.argsort(keys, kind="stable"))


def test_seeded_inputs_are_deterministic():
    lc = LatticeConfig(nx=64, ny=64, nz=64)
    pc = ParticleConfig(count=2000, seed=1234)
    a = seed_particles(lc, pc)
    b = seed_particles(lc, pc)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    pos, vel, d, act = a
    assert np.all(np.isfinite(pos)) and d.min() > 0
    # inside the cone
    cx, cy = lc.axis
    r = np.hypot(pos[0] - cx, pos[1] - cy)
    rc = (pos[2] - lc.cone_apex_z) * lc.tan_half_angle
    assert np.all(r <= 0.8 * rc + 1e-4)
    # log-normal median close to 0.6
    assert abs(np.median(d) - 0.6) < 0.03
