"""Write tests/golden/drive_reference.npz from the reference's own PressureGradientDrive
(src/physics/pressure_gradient_drive.py).  Its kernel source runs in this container through
taichi_standin.py, serially and in float32.

    python tests/golden/make_drive_golden.py <path of the reference checkout>

The script runs only where the reference checkout exists (its path is the script's required first argument).  The fixture
travels with tests/test_drive_oracle.py.

Grid: 12 x 10 x 14 (config.NX/NY/NZ set before construction), about 10 % solid cells, seeded
density 1 + 0.05 N(0, 1) with one zero cell and one spike.  The fixture holds four cases, all
through apply():
- force: force drive, cap 0.12, into a zero body force;
- capped: force drive, MAX_PRESSURE_FORCE lowered to 0.002;
- mixed: mixed drive, half the pressure force onto a seeded body force;
- density: density drive, three calls, with the target field initialize_target_density built.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SHAPE = (12, 10, 14)  # (NX, NY, NZ)


def main():
    sys.path.insert(0, HERE)
    import taichi_standin
    ti = taichi_standin.install()
    sys.path.insert(0, sys.argv[1])
    import config  # the reference's config package
    config.NX, config.NY, config.NZ = SHAPE
    from src.physics.pressure_gradient_drive import PressureGradientDrive
    rng = np.random.default_rng(2)
    solid0 = (rng.uniform(size=SHAPE) < 0.1).astype(np.uint8)
    rho0 = (1.0 + 0.05 * rng.normal(size=SHAPE)).astype(np.float32)
    rho0[5, 4, 3] = 0.0  # rho <= 1e-12: no force there
    rho0[5, 5, 7] = 4.0  # a spike: the cap acts around it
    base = rng.normal(size=SHAPE + (3,)).astype(np.float32) * np.float32(1e-3)

    class Lattice:
        pass
    lbm = Lattice()
    lbm.solid = ti.field(ti.u8, SHAPE)
    lbm.solid.from_numpy(solid0)
    lbm.rho = ti.field(ti.f32, SHAPE)
    lbm.body_force = ti.Vector.field(3, ti.f32, SHAPE)
    lbm.u = ti.Vector.field(3, ti.f32, SHAPE)
    drive = PressureGradientDrive(lbm)
    out = {"solid": solid0, "rho": rho0, "base": base, "target": drive.target_density.to_numpy()}

    def run(case, force_on, mixed_on, density_on, body, calls=1):
        lbm.rho.from_numpy(rho0)
        lbm.body_force.from_numpy(body)
        drive.force_drive_active[None] = force_on
        drive.mixed_drive_active[None] = mixed_on
        drive.density_drive_active[None] = density_on
        for _ in range(calls):
            drive.apply(0)
        out[case + "_force"] = lbm.body_force.to_numpy()
        out[case + "_rho"] = lbm.rho.to_numpy()

    zero = np.zeros_like(base)
    run("force", 1, 0, 0, zero)
    drive.MAX_PRESSURE_FORCE = 0.002
    run("capped", 1, 0, 0, zero)
    drive.MAX_PRESSURE_FORCE = 0.12
    run("mixed", 0, 1, 0, base)
    run("density", 0, 0, 1, zero, calls=3)
    np.savez_compressed(os.path.join(HERE, "drive_reference.npz"), **out)
    print("wrote drive_reference.npz")


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: make_drive_golden.py <path of the reference checkout>")
    main()
