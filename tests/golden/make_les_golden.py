"""Write tests/golden/les_reference.npz from the reference's own LES model
(src/physics/les_turbulence.py: update_turbulent_viscosity -> _compute_sgs_from_vector :318-380,
the path LBMSolver.step takes).  Its kernel source runs in this container through
taichi_standin.py, serially and in float32.

    python tests/golden/make_les_golden.py <path of the reference checkout>

The script runs only where the reference checkout exists (its path is the script's required first argument).  The fixture
travels with tests/test_les_reference.py.

Grid: 10 x 9 x 12 (config.NX/NY/NZ set before construction).  u = 0.05 N(0, 1) with one
low-shear block at 1e-5 N(0, 1), so that the strain floor gates part of the grid.  The LES mask
(set_mask) is 0 on about 15 % of the cells, and the phase field is the default all-ones.  The
model's own C_s is 0.18.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SHAPE = (10, 9, 12)  # (NX, NY, NZ)


def main():
    sys.path.insert(0, HERE)
    import taichi_standin
    ti = taichi_standin.install()
    sys.path.insert(0, sys.argv[1])
    import config  # the reference's config package
    config.NX, config.NY, config.NZ = SHAPE
    from src.physics.les_turbulence import LESTurbulenceModel
    rng = np.random.default_rng(17)
    u = (0.05 * rng.normal(size=SHAPE + (3,))).astype(np.float32)
    u[2:6, 2:6, 3:8] = (1e-5 * rng.normal(size=(4, 4, 5, 3))).astype(np.float32)
    mask = (rng.uniform(size=SHAPE) >= 0.15).astype(np.int32)
    les = LESTurbulenceModel()
    m = ti.field(ti.i32, SHAPE)
    m.from_numpy(mask)
    les.set_mask(m)
    uf = ti.Vector.field(3, ti.f32, SHAPE)
    uf.from_numpy(u)
    les.update_turbulent_viscosity(uf)
    np.savez_compressed(os.path.join(HERE, "les_reference.npz"), u=u, mask=mask, nu=les.nu_sgs.to_numpy(),
                        cs=np.float64(les.cs))
    print("wrote les_reference.npz")


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: make_les_golden.py <path of the reference checkout>")
    main()
