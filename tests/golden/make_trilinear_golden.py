"""Write tests/golden/trilinear_reference.npz: the reference's own particle gather
(src/physics/coffee_particles.py interpolate_fluid_velocity_from_field :1156-1198, the
interpolation compute_two_way_coupling_forces uses).  It runs on a seeded velocity field at
seeded positions, including positions outside the grid that the gather clamps.  The kernel source
runs in this container through taichi_standin.py, serially and in float32.

    python tests/golden/make_trilinear_golden.py <path of the reference checkout>

The script runs only where the reference checkout exists (its path is the script's required first argument).  The fixture
travels with tests/test_oracle_kat.py.  The method reads only the particles' positions, so the
object is made without its constructor (object.__new__).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SHAPE = (12, 10, 14)  # (NX, NY, NZ)
NP = 300


def main():
    sys.path.insert(0, HERE)
    import taichi_standin
    ti = taichi_standin.install()
    sys.path.insert(0, sys.argv[1])
    import config  # the reference's config package
    config.NX, config.NY, config.NZ = SHAPE
    from src.physics.coffee_particles import CoffeeParticleSystem
    rng = np.random.default_rng(21)
    u = rng.normal(size=SHAPE + (3,)).astype(np.float32)
    lo, hi = -1.5, np.array(SHAPE, np.float64) + 0.5  # a margin outside the grid on every side
    pos = (lo + rng.uniform(size=(NP, 3)) * (hi - lo)).astype(np.float32)
    cps = object.__new__(CoffeeParticleSystem)
    cps.position = ti.Vector.field(3, ti.f32, (NP,))
    cps.position.from_numpy(pos)
    uf = ti.Vector.field(3, ti.f32, SHAPE)
    uf.from_numpy(u)
    out = np.array([cps.interpolate_fluid_velocity_from_field(p, uf) for p in range(NP)], np.float32)
    np.savez_compressed(os.path.join(HERE, "trilinear_reference.npz"), u=u, pos=pos, out=out)
    print("wrote trilinear_reference.npz")


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: make_trilinear_golden.py <path of the reference checkout>")
    main()
