"""The oracle's pressure-gradient drive against the reference's formulas restated in numpy
(src/physics/pressure_gradient_drive.py: compute_pressure_gradient :124-177, the force
accumulation :188-193 / :274-279, apply_density_drive :95-122)."""
import numpy as np

import oracle as orc
from pour_over_coffee_lbm_gb300.params import CELL_SOLID, LatticeConfig

f32 = np.float32


def _reference_force(flags, rho, max_force):
    nz, ny, nx = rho.shape
    F = np.zeros((3, nz, ny, nx), f32)
    cs2 = f32(1.0 / 3.0)
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                if flags[k, j, i] & CELL_SOLID:
                    continue
                r = rho[k, j, i]
                g = []
                for (a, b, lo, hi) in (((k, j, i + 1), (k, j, i - 1), i == 0, i == nx - 1),
                                       ((k, j + 1, i), (k, j - 1, i), j == 0, j == ny - 1),
                                       ((k + 1, j, i), (k - 1, j, i), k == 0, k == nz - 1)):
                    if not lo and not hi:
                        g.append((rho[a] - rho[b]) * f32(0.5))
                    elif lo:
                        g.append(rho[a] - r)
                    else:
                        g.append(r - rho[b])
                if r > f32(1e-12):
                    fv = [-(gg * cs2) / r for gg in g]
                    m = np.sqrt(fv[0] * fv[0] + fv[1] * fv[1] + fv[2] * fv[2])
                    if m > f32(max_force):
                        s = f32(max_force) / m
                        fv = [v * s for v in fv]
                    F[:, k, j, i] = fv
    return F


def test_pressure_force_matches_reference():
    cfg = LatticeConfig(nx=12, ny=10, nz=14, band_thickness=2.0)
    flags = orc.build_flags(cfg)
    rng = np.random.default_rng(2)
    rho = (1.0 + 0.05 * rng.normal(size=flags.shape)).astype(f32)
    rho[3, 4, 5] = 0.0  # rho <= 1e-12: no force there
    rho[7, 5, 5] = 4.0  # a spike: the cap acts around it
    ref = _reference_force(flags, rho, 0.12)
    F = np.zeros((3,) + flags.shape, f32)
    orc.pressure_force(cfg, flags, rho, F, 1.0, 0.12)
    assert np.array_equal(F, ref)
    mag = np.sqrt((F.astype(np.float64) ** 2).sum(0))
    assert mag.max() <= 0.12 * (1 + 1e-6) and (mag > 0.119).any()
    # accumulation with the mixed drive's half weight on top of an existing force
    base = rng.normal(size=F.shape).astype(f32)
    G = base.copy()
    orc.pressure_force(cfg, flags, rho, G, 0.5, 0.12)
    assert np.array_equal(G, base + f32(0.5) * ref)


def test_pressure_force_one_sided_faces():
    # an all-fluid box (no shell): the domain faces use one-sided differences
    cfg = LatticeConfig(nx=6, ny=5, nz=7)
    flags = np.zeros((7, 5, 6), np.uint32)
    z = np.arange(7, dtype=f32)[:, None, None]
    rho = np.ascontiguousarray(np.broadcast_to(f32(1) + f32(0.01) * z * z, flags.shape), f32)
    F = np.zeros((3,) + flags.shape, f32)
    orc.pressure_force(cfg, flags, rho, F, 1.0, 1.0)
    assert np.array_equal(F, _reference_force(flags, rho, 1.0))
    assert F[2, 0, 2, 2] == -((rho[1, 2, 2] - rho[0, 2, 2]) * f32(1 / 3)) / rho[0, 2, 2]
    assert F[2, 6, 2, 2] == -((rho[6, 2, 2] - rho[5, 2, 2]) * f32(1 / 3)) / rho[6, 2, 2]


def test_density_drive_matches_reference():
    cfg = LatticeConfig(nx=10, ny=9, nz=16, band_thickness=2.0)
    flags = orc.build_flags(cfg)
    rng = np.random.default_rng(4)
    rho = (1.0 + 0.3 * rng.normal(size=flags.shape)).astype(f32)
    target = np.linspace(0.4, 1.8, cfg.nz).astype(f32)
    ref = rho.copy()
    for _ in range(3):
        a = (target[:, None, None] - ref) * f32(0.025)
        a = np.where(np.abs(a) > f32(0.001), np.where(a > 0, f32(0.001), f32(-0.001)), a).astype(f32)
        new = np.maximum(f32(0.5), np.minimum(f32(2.0), ref + a))
        ref = np.where(flags & CELL_SOLID, ref, new).astype(f32)
        orc.density_drive(cfg, flags, rho, target, 0.025, 0.001, 0.5, 2.0)
    assert np.array_equal(rho, ref)


# ---- against the reference's own kernels (tests/golden/drive_reference.npz, made by
# tests/golden/make_drive_golden.py, which runs pressure_gradient_drive.py's kernel source) ----
def _ref():
    import os
    return np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "drive_reference.npz"))


def _zyx(a):
    """(NX, NY, NZ[, 3]) of the reference -> (NZ, NY, NX) / (3, NZ, NY, NX)."""
    return np.ascontiguousarray(a.transpose(2, 1, 0) if a.ndim == 3 else a.transpose(3, 2, 1, 0))


def test_drive_matches_reference_kernels():
    z = _ref()
    nx, ny, nz = z["rho"].shape
    cfg = LatticeConfig(nx=nx, ny=ny, nz=nz)
    flags = _zyx(z["solid"]).astype(np.uint32) * np.uint32(CELL_SOLID)
    rho = _zyx(z["rho"])
    for case, scale, cap, base in (("force", 1.0, 0.12, None), ("capped", 1.0, 0.002, None),
                                   ("mixed", 0.5, 0.12, "base")):
        F = _zyx(z[base]) if base else np.zeros((3, nz, ny, nx), f32)
        orc.pressure_force(cfg, flags, rho, F, scale, cap)
        assert np.array_equal(F, _zyx(z[case + "_force"])), case
    # the density drive: a per-plane target (the reference's target field is uniform in x, y)
    t = z["target"]
    assert np.array_equal(t, np.broadcast_to(t[:1, :1, :], t.shape))
    r = rho.copy()
    for _ in range(3):
        orc.density_drive(cfg, flags, r, np.ascontiguousarray(t[0, 0, :]), 0.025, 0.001, 0.5, 2.0)
    assert np.array_equal(r, _zyx(z["density_rho"]))
    assert np.count_nonzero(r != rho) > 1000
