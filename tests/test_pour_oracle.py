"""The oracle's pour nozzle against the reference's formulas restated in numpy
(src/physics/precise_pouring.py: _get_current_pour_position :81-98, _is_in_pouring_region
:100-130, apply_pouring_force :132-160, create_water_impact_force :190-226)."""
import math

import numpy as np

import oracle as orc
from pour_over_coffee_lbm_gb300.params import STORE_F64, LatticeConfig, ParticleConfig
from pour_over_coffee_lbm_gb300.pouring import (POUR_ACCEL_CAP, POUR_ACTIVE, POUR_CX, POUR_CY, POUR_DIAMETER,
                                                POUR_DT, POUR_FLOW, POUR_HEIGHT, POUR_IMPACT, POUR_IMPACT_MAX,
                                                POUR_IMPACT_ZMIN, POUR_NFIELDS, POUR_PATTERN, POUR_RADIUS,
                                                POUR_SPIRAL_R, POUR_SPIRAL_SPEED, POUR_TIME, POUR_VELOCITY,
                                                POUR_X, POUR_Y, POUR_ZTOP)


def _block(cx, cy, pattern=0, flow=1.3, dt=0.5, velocity=0.02, ztop=18.0, diameter=5.0):
    b = np.zeros(POUR_NFIELDS, np.float32)
    b[POUR_ACTIVE] = 1
    b[POUR_X], b[POUR_Y], b[POUR_CX], b[POUR_CY] = cx, cy, cx, cy
    b[POUR_RADIUS] = diameter / 2
    b[POUR_ZTOP], b[POUR_HEIGHT] = ztop, 4.0
    b[POUR_VELOCITY], b[POUR_FLOW], b[POUR_DT], b[POUR_ACCEL_CAP] = velocity, flow, dt, 10.0
    b[POUR_PATTERN] = pattern
    b[POUR_SPIRAL_R], b[POUR_SPIRAL_SPEED] = 5.0, 0.7
    b[POUR_DIAMETER] = diameter
    return b


def test_pour_force_matches_reference_formula():
    cfg = LatticeConfig(nx=24, ny=24, nz=24, storage=STORE_F64, band_thickness=0.0, u_inlet=0.0)
    flags = orc.build_flags(cfg)
    f = orc.init_equilibrium(cfg, flags, np.float64)
    b = _block(11.3, 12.6)
    _, rho, u = orc.step(cfg, flags, f, pour=b)
    # at rest u = (F/2)/rho, F_z = rho g_z - a: a = rho g_z - 2 rho u_z
    a = rho * cfg.gravity[2] - 2.0 * rho * u[2]
    ref = np.zeros_like(a)
    B = [float(v) for v in b]  # the block's float32 values, evaluated in float64 like the FP64 step
    R, ztop = B[POUR_RADIUS], B[POUR_ZTOP]
    for k in range(cfg.nz):
        for j in range(cfg.ny):
            for i in range(cfg.nx):
                if flags[k, j, i] & 1:
                    continue
                d = math.hypot(i - B[POUR_X], j - B[POUR_Y])
                if d <= R and ztop - B[POUR_HEIGHT] <= k <= ztop:
                    inten = math.exp(-0.5 * (d / R) ** 2) * math.exp(-(ztop - k) / 2.0)
                    ref[k, j, i] = min(B[POUR_VELOCITY] * inten * B[POUR_FLOW] / B[POUR_DT], 10.0)
    fluid = (flags & 0x7) == 0  # not solid, inlet or outlet (their velocity is imposed)
    assert np.count_nonzero(ref[fluid]) > 10
    assert np.allclose(a[fluid], ref[fluid], rtol=1e-9, atol=1e-12)


def test_spiral_trajectory_matches_reference():
    cfg = LatticeConfig(nx=40, ny=36, nz=24)
    b = _block(20.0, 18.0, pattern=1, dt=0.9, diameter=3.0)
    for step in range(1, 60):
        orc.pour_advance(cfg, b)
        t = step * 0.9 * 0.7  # pour_time (advanced before use) * spiral_speed
        r = 5.0 * (1.0 + 0.1 * t)
        x = min(max(20.0 + r * math.cos(t), 3.0), 40 - 3.0)
        y = min(max(18.0 + r * math.sin(t), 3.0), 36 - 3.0)
        assert abs(b[POUR_TIME] - step * 0.9) < 1e-4
        assert abs(b[POUR_X] - x) < 1e-3 and abs(b[POUR_Y] - y) < 1e-3, step


def test_particle_impact_matches_reference():
    cfg = LatticeConfig(nx=24, ny=24, nz=24, band_thickness=0.0)
    pc = ParticleConfig(count=3, deterministic=True)
    b = _block(12.0, 12.0)
    b[POUR_IMPACT], b[POUR_IMPACT_MAX], b[POUR_IMPACT_ZMIN] = 10.0 * b[POUR_FLOW], 0.05, 7.2
    # rows x, y, z: near the axis; 2 cells off it; on the axis but below IMPACT_ZMIN
    pos = np.array([[12.7, 14.0, 12.0], [12.4, 12.0, 12.0], [16.0, 16.0, 5.0]], np.float32)
    vel = np.zeros((3, 3), np.float32)
    d = np.array([0.6, 0.7, 0.8], np.float32)
    act = np.ones(3, np.int32)
    u = np.zeros((3, 24, 24, 24), np.float32)
    a = orc.particles_couple(cfg, pc, pos, vel, d, np.zeros((3, 3), np.float32), act, u, pour=b)
    n = orc.particles_couple(cfg, pc, pos, vel, d, np.zeros((3, 3), np.float32), act, u)
    dv = (a[1] - n[1]).astype(np.float64)  # velocity change = F_impact / m_p * dt
    rho_p = pc.density_ratio * cfg.rho0
    b = [float(v) for v in b]
    for p in range(3):
        x, y, z = (float(v) for v in pos[:, p])
        dx, dy = x - b[POUR_X], y - b[POUR_Y]
        r = math.hypot(dx, dy)
        F = np.zeros(3)
        if r <= 2 * b[POUR_RADIUS] and z > b[POUR_IMPACT_ZMIN]:
            inten = math.exp(-0.5 * (r / b[POUR_RADIUS]) ** 2)
            F[2] = -b[POUR_IMPACT] * inten
            if r > 0.1:
                F[0] = b[POUR_IMPACT] * 0.3 * inten * dx / r
                F[1] = b[POUR_IMPACT] * 0.3 * inten * dy / r
            fm = np.linalg.norm(F)
            if fm > b[POUR_IMPACT_MAX]:
                F *= b[POUR_IMPACT_MAX] / fm
        m = rho_p * math.pi / 6 * float(d[p]) ** 3
        assert np.allclose(dv[:, p], F / m * pc.dt, rtol=1e-4, atol=1e-7), p
    assert np.abs(dv[:, 0]).max() > 0 and np.abs(dv[:, 1]).max() > 0 and np.abs(dv[:, 2]).max() == 0


# ---- against the reference's own kernels (tests/golden/pour_reference.npz, made by
# tests/golden/make_pour_golden.py, which runs precise_pouring.py's kernel source in float32) ----
def _ref():
    import os
    return np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pour_reference.npz"))


def _ref_block(z, x, y, flow, dt, pattern=0):
    return _block(float(x), float(y), pattern=pattern, flow=flow, dt=dt, velocity=float(z["velocity"]),
                  ztop=float(z["ztop"]), diameter=float(z["diameter"]))


def test_pour_force_matches_reference_kernel():
    z = _ref()
    cfg = LatticeConfig(nx=24, ny=24, nz=24, storage=STORE_F64, band_thickness=0.0, u_inlet=0.0)
    flags = orc.build_flags(cfg)
    f = orc.init_equilibrium(cfg, flags, np.float64)
    b = _ref_block(z, *z["force_pos"], flow=1.3, dt=0.5)
    _, rho, u = orc.step(cfg, flags, f, pour=b)
    a = rho * cfg.gravity[2] - 2.0 * rho * u[2]  # the pour acceleration at rest (see above)
    ref = -z["force"][..., 2].transpose(2, 1, 0).astype(np.float64)  # (NX,NY,NZ) -> (NZ,NY,NX)
    fluid = (flags & 0x7) == 0
    assert np.count_nonzero(ref[fluid]) > 50
    assert np.allclose(a[fluid], ref[fluid], rtol=2e-6, atol=1e-9)


def test_spiral_trajectory_matches_reference_kernel():
    z = _ref()
    cfg = LatticeConfig(nx=64, ny=64, nz=24)
    b = _ref_block(z, 32.0, 30.0, flow=1.0, dt=0.9, pattern=1)
    b[POUR_SPIRAL_SPEED] = 1.0  # start_pouring's spiral speed
    for step, (x, y) in enumerate(z["trajectory"]):
        orc.pour_advance(cfg, b)
        assert abs(b[POUR_X] - x) < 2e-4 and abs(b[POUR_Y] - y) < 2e-4, (step, b[POUR_X], b[POUR_Y], x, y)


def test_pour_phase_matches_reference_kernel():
    z = _ref()
    cfg = LatticeConfig(nx=24, ny=24, nz=24, band_thickness=0.0)
    flags = np.zeros((24, 24, 24), np.uint32)  # the reference case has no solid cells
    phi = np.ascontiguousarray(z["phase_in"].transpose(2, 1, 0))
    b = _ref_block(z, 12.0, 11.0, flow=1.3, dt=0.5)
    orc.pour_phase(cfg, flags, phi, 0.5, b)
    ref = z["phase_out"].transpose(2, 1, 0)
    assert np.count_nonzero(ref != z["phase_in"].transpose(2, 1, 0)) > 100
    assert np.allclose(phi, ref, rtol=0, atol=2e-6)


def test_particle_impact_matches_reference_kernel():
    z = _ref()
    cfg = LatticeConfig(nx=24, ny=24, nz=24, band_thickness=0.0)
    pc = ParticleConfig(count=3, deterministic=True)
    b = _ref_block(z, 12.0, 12.0, flow=1.3, dt=1.0)
    b[POUR_IMPACT], b[POUR_IMPACT_MAX], b[POUR_IMPACT_ZMIN] = 10.0 * b[POUR_FLOW], 0.05, 0.3 * 24
    pos = np.ascontiguousarray(z["impact_pos"].T)
    vel = np.zeros((3, 3), np.float32)
    d = np.array([0.6, 0.7, 0.8], np.float32)
    act = np.ones(3, np.int32)
    u = np.zeros((3, 24, 24, 24), np.float32)
    a = orc.particles_couple(cfg, pc, pos, vel, d, np.zeros((3, 3), np.float32), act, u, pour=b)
    n = orc.particles_couple(cfg, pc, pos, vel, d, np.zeros((3, 3), np.float32), act, u)
    dv = (a[1] - n[1]).astype(np.float64)
    m = pc.density_ratio * cfg.rho0 * math.pi / 6 * d.astype(np.float64) ** 3
    F = dv * m / pc.dt  # the impact force each particle received
    assert np.abs(z["impact_force"]).max() > 0
    assert np.allclose(F, z["impact_force"].T, rtol=1e-4, atol=1e-8)
