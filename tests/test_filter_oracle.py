"""The oracle's filter-paper dynamics against the reference's formulas restated in numpy
(src/physics/filter_paper.py: block_particles_at_filter :616-700, update_dynamic_resistance
:702-746, the blockage factor of apply_filter_effects :586-588)."""
import numpy as np

import oracle as orc
from pour_over_coffee_lbm_gb300.params import CELL_POROUS, STORE_F64, LatticeConfig


def _lowbias32(x):
    x = np.uint32(x)
    with np.errstate(over="ignore"):
        x ^= x >> np.uint32(16)
        x = np.uint32(x * np.uint32(0x7FEB352D))
        x ^= x >> np.uint32(15)
        x = np.uint32(x * np.uint32(0x846CA68B))
        x ^= x >> np.uint32(16)
    return x


def _uniform(seed, step, pid, lane):
    """The counter hash that stands in for ti.random(): 24 bits of lowbias32 chains."""
    with np.errstate(over="ignore"):
        h = _lowbias32(np.uint32(seed) ^ _lowbias32(np.uint32(step) ^ _lowbias32(np.uint32(pid * 2 + lane))))
    return np.float32(h >> np.uint32(8)) * np.float32(1.0 / 16777216.0)


def _reference_block(flags, pos, vel, active, accum, seed, step):
    nz, ny, nx = flags.shape
    vel, accum = vel.copy(), accum.copy().reshape(nz, ny, nx)
    for p in range(active.shape[0]):
        if not active[p]:
            continue
        x, y, z = (float(v) for v in pos[:, p])
        if x < 0 or y < 0 or z < 0:
            continue
        i, j, k = int(x), int(y), int(z)
        if not (i < nx and j < ny and k < nz):
            continue
        for o in range(-2, 3):
            kk = k + o
            if 0 <= kk < nz and flags[kk, j, i] & CELL_POROUS:
                if vel[2, p] < 0:
                    vel[2, p] = -vel[2, p] * np.float32(0.3)
                    vel[0, p] += (_uniform(seed, step, p, 0) - np.float32(0.5)) * np.float32(0.01)
                    vel[1, p] += (_uniform(seed, step, p, 1) - np.float32(0.5)) * np.float32(0.01)
                    accum[kk, j, i] += np.float32(0.01)
                break
    return vel, accum.reshape(-1)


def _band_case(n=24):
    cfg = LatticeConfig(nx=n, ny=n, nz=n, band_thickness=3.0)
    flags = orc.build_flags(cfg)
    return cfg, flags


def test_hash_is_uniform():
    u = np.array([_uniform(7, 3, p, lane) for p in range(2000) for lane in (0, 1)])
    assert 0.0 <= u.min() and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 0.02 and abs(u.std() - np.sqrt(1 / 12)) < 0.02


def test_block_particles_matches_reference():
    cfg, flags = _band_case()
    rng = np.random.default_rng(11)
    por = np.argwhere(flags & CELL_POROUS)
    npart = 600
    # particles near the paper (the bounce case), anywhere (most miss), and out of the grid
    pick = por[rng.integers(0, len(por), npart // 2)]
    near = np.stack([pick[:, 2], pick[:, 1], pick[:, 0]]).astype(np.float32) + rng.uniform(0, 1, (3, npart // 2))
    near[2] += rng.integers(-2, 3, npart // 2)
    anywhere = rng.uniform(-2, cfg.nx + 2, (3, npart // 2))
    pos = np.ascontiguousarray(np.concatenate([near, anywhere], 1).astype(np.float32))
    vel = np.ascontiguousarray(rng.normal(0, 0.02, (3, npart)).astype(np.float32))
    active = (rng.uniform(size=npart) > 0.1).astype(np.int32)
    accum = np.ascontiguousarray(rng.uniform(0, 0.5, flags.size).astype(np.float32))
    ref_v, ref_a = _reference_block(flags, pos, vel, active, accum, 1234, 77)
    v, a = vel.copy(), accum.copy()
    orc.filter_particles(cfg, flags, pos, v, active, a, 1234, 77)
    assert np.array_equal(v, ref_v) and np.array_equal(a, ref_a)
    bounced = (v[2] != vel[2])
    assert bounced.sum() > 50 and (v[2][bounced] > 0).all()
    assert np.array_equal(v[:, active == 0], vel[:, active == 0])


def test_blockage_update_matches_reference():
    cfg, flags = _band_case()
    rng = np.random.default_rng(5)
    accum = np.ascontiguousarray(rng.uniform(0, 30, flags.size).astype(np.float32))
    b = np.ascontiguousarray(rng.uniform(0, 0.5, flags.size).astype(np.float32))
    a_ref, b_ref = accum.copy(), b.copy()
    zone = (flags.reshape(-1) & CELL_POROUS) != 0
    for _ in range(40):
        nb = np.float32(0.9) * (np.float32(1) - np.exp(np.float32(-0.1) * a_ref[zone]))
        b_ref[zone] = np.float32(0.95) * b_ref[zone] + np.float32(0.05) * nb
        a_ref[zone] *= np.float32(0.999)
        orc.filter_update(cfg, flags, accum, b)
    assert np.allclose(b, b_ref, rtol=1e-6, atol=1e-7) and np.array_equal(accum, a_ref)
    assert np.array_equal(b[~zone], b_ref[~zone])  # outside the paper nothing changes


def test_uniform_blockage_equals_scaled_permeability():
    """(1 + b) on nu/K and C_F/sqrt(K) is the same step as K/(1+b) and C_F sqrt(1+b)."""
    b = 0.7
    cfg = LatticeConfig(nx=24, ny=24, nz=28, storage=STORE_F64, band_thickness=3.0, u_inlet=-0.03)
    flags = orc.build_flags(cfg)
    f = orc.init_equilibrium(cfg, flags, np.float64)
    scaled = LatticeConfig(nx=24, ny=24, nz=28, storage=STORE_F64, band_thickness=3.0, u_inlet=-0.03,
                           permeability=cfg.permeability / (1 + b), forchheimer=cfg.forchheimer * np.sqrt(1 + b))
    fa, fb = f, f
    blk = np.full(flags.size, b, np.float32)
    for _ in range(12):
        fa, _, ua = orc.step(cfg, flags, fa, blockage=blk)
        fb, _, ub = orc.step(scaled, flags, fb)
    fl = (flags & 1) == 0
    assert np.allclose(ua[:, fl], ub[:, fl], rtol=1e-5, atol=1e-10)
    # and the blockage slows the band
    f0 = f
    for _ in range(12):
        f0, _, u0 = orc.step(cfg, flags, f0)
    band = (flags & CELL_POROUS) != 0
    assert np.abs(ua[:, band]).sum() < np.abs(u0[:, band]).sum()


# ---- against the reference's own kernels (tests/golden/filter_reference.npz, made by
# tests/golden/make_filter_golden.py, which runs filter_paper.py's kernel source in float32) ----
def test_filter_kernels_match_reference_kernels():
    import os
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "filter_reference.npz"))
    nx, ny, nz = z["zone"].shape
    cfg = LatticeConfig(nx=nx, ny=ny, nz=nz)
    zyx = lambda a: np.ascontiguousarray(a.transpose(2, 1, 0))  # noqa: E731
    flags = zyx(z["zone"]).astype(np.uint32) * np.uint32(CELL_POROUS)
    pos = np.ascontiguousarray(z["pos"].T)
    vel = np.ascontiguousarray(z["vel"].T)
    accum = np.zeros(flags.shape, np.float32)
    orc.filter_particles(cfg, flags, pos, vel, z["active"].copy(), accum, 7, 3)
    ref_v = z["vel_after"].T
    bounced = ref_v[2] != z["vel"][:, 2]
    assert bounced.sum() >= 5
    # v_z and the deposit exactly; the horizontal kick is the one random part (zero in the fixture,
    # a counter hash within +-0.005 here)
    assert np.array_equal(vel[2], ref_v[2])
    assert np.array_equal(accum, zyx(z["accum_after"]))
    assert np.all(np.abs(vel[:2] - ref_v[:2]) <= 0.005 + 1e-7)
    assert np.array_equal(vel[:2, ~bounced], ref_v[:2, ~bounced])
    # three blockage updates
    a, b = zyx(z["accum0"]), zyx(z["block0"])
    for _ in range(3):
        orc.filter_update(cfg, flags, a, b)
    assert np.allclose(a, zyx(z["accum3"]), rtol=0, atol=1e-6)
    assert np.allclose(b, zyx(z["block3"]), rtol=0, atol=1e-6)
