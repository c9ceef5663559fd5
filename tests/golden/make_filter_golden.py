"""Write tests/golden/filter_reference.npz from the reference's own FilterPaperSystem kernels
(src/physics/filter_paper.py: block_particles_at_filter :616-700, update_dynamic_resistance
:702-746).  Their source runs in this container through taichi_standin.py, serially and in
float32.

    python tests/golden/make_filter_golden.py <path of the reference checkout>

The script runs only where the reference checkout exists (its path is the script's required first argument).  The fixture
travels with tests/test_filter_oracle.py.

The kernels read only the paper mask and the two dynamic fields, so the object is made without
its geometry set-up (object.__new__) and given a seeded 10 x 9 x 12 mask: planes 3-4, 80 % of the
cells.  block_particles_at_filter divides positions by config.SCALE_LENGTH, so it is given
lattice positions times SCALE_LENGTH.  The positions keep their fractional parts in
[0.1, 0.9], so the cell index survives that round trip.  ti.random() is 0.5 in the stand-in, which
makes the reference's horizontal kick zero.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SHAPE = (10, 9, 12)  # (NX, NY, NZ)
NP = 60


def main():
    sys.path.insert(0, HERE)
    import taichi_standin
    ti = taichi_standin.install()
    sys.path.insert(0, sys.argv[1])
    import config  # the reference's config package
    config.NX, config.NY, config.NZ = SHAPE
    from src.physics.filter_paper import FilterPaperSystem
    rng = np.random.default_rng(9)
    k = np.arange(SHAPE[2])[None, None, :]
    zone = (((k == 3) | (k == 4)) & (rng.uniform(size=SHAPE) < 0.8)).astype(np.int32)
    cells = np.stack([rng.integers(0, SHAPE[0], NP), rng.integers(0, SHAPE[1], NP), rng.integers(0, 8, NP)], 1)
    pos = (cells + rng.uniform(0.1, 0.9, size=(NP, 3))).astype(np.float32)
    vel = (0.02 * rng.normal(size=(NP, 3))).astype(np.float32)
    active = (rng.uniform(size=NP) < 0.9).astype(np.int32)

    fp = object.__new__(FilterPaperSystem)
    fp.filter_zone = ti.field(ti.i32, SHAPE)
    fp.filter_zone.from_numpy(zone)
    fp.accumulated_particles = ti.field(ti.f32, SHAPE)
    fp.filter_blockage = ti.field(ti.f32, SHAPE)
    P = ti.Vector.field(3, ti.f32, (NP,))
    P.from_numpy((pos * np.float32(config.SCALE_LENGTH)).astype(np.float32))
    V = ti.Vector.field(3, ti.f32, (NP,))
    V.from_numpy(vel)
    R = ti.field(ti.f32, (NP,))
    A = ti.field(ti.i32, (NP,))
    A.from_numpy(active)
    count = ti.field(ti.i32, ())
    count[None] = NP
    fp.block_particles_at_filter(P, V, R, A, count)
    out = {"zone": zone, "pos": pos, "vel": vel, "active": active, "vel_after": V.to_numpy(),
           "accum_after": fp.accumulated_particles.to_numpy()}
    # dynamic resistance, three updates from a seeded deposit and blockage
    a0 = (rng.uniform(0, 3, size=SHAPE)).astype(np.float32)
    b0 = (rng.uniform(0, 0.5, size=SHAPE)).astype(np.float32)
    fp.accumulated_particles.from_numpy(a0)
    fp.filter_blockage.from_numpy(b0)
    for _ in range(3):
        fp.update_dynamic_resistance()
    out.update(accum0=a0, block0=b0, accum3=fp.accumulated_particles.to_numpy(), block3=fp.filter_blockage.to_numpy())
    np.savez_compressed(os.path.join(HERE, "filter_reference.npz"), **out)
    print("wrote filter_reference.npz")


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: make_filter_golden.py <path of the reference checkout>")
    main()
