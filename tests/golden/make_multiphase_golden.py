"""Write tests/golden/multiphase_reference.npz from the reference's own MultiphaseFlow3D kernels
(src/core/multiphase_3d.py).  Their source runs in this container through taichi_standin.py,
serially and in float32.

    python tests/golden/make_multiphase_golden.py <path of the reference checkout>

The script runs only where the reference checkout exists (its path is the script's required first argument).  The fixture
travels with tests/test_multiphase_oracle.py.

Grid: 10 x 9 x 12 (config.NX/NY/NZ set before construction).  The phase field is a drop of water
in air, tanh((3 - r) / 1.5) around (5, 4.5, 6), plus 0.05 noise, with u = 0.02 N(0, 1).  The
surface tension goes into a seeded body force over a seeded density, with about 10 % solid
cells.  The kernels run in the order of the reference's step(), except that the chemical
potential is computed first:
compute_chemical_potential, compute_gradients, compute_curvature,
compute_surface_tension_force (the later of its two definitions, the one Python keeps),
apply_surface_tension, update_phase_field_cahn_hilliard, apply_phase_separation,
copy_phase_field and update_density_from_phase.  Each output is recorded.  phi_new starts
equal to phi, as standardize_initial_state leaves it.  The kernels never write the domain shell of
phi_new, so the shell carries phi over.
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
    from src.core.multiphase_3d import MultiphaseFlow3D
    rng = np.random.default_rng(13)
    x, y, z = np.meshgrid(*[np.arange(n) for n in SHAPE], indexing="ij")
    r = np.sqrt((x - 5.0) ** 2 + (y - 4.5) ** 2 + (z - 6.0) ** 2)
    phi0 = np.clip(np.tanh((3.0 - r) / 1.5) + 0.05 * rng.normal(size=SHAPE), -1, 1).astype(np.float32)
    u0 = (0.02 * rng.normal(size=SHAPE + (3,))).astype(np.float32)
    rho0 = (1.0 + 0.01 * rng.normal(size=SHAPE)).astype(np.float32)
    base = (1e-4 * rng.normal(size=SHAPE + (3,))).astype(np.float32)
    solid0 = (rng.uniform(size=SHAPE) < 0.1).astype(np.uint8)

    class Lattice:
        pass
    lbm = Lattice()
    lbm.u = ti.Vector.field(3, ti.f32, SHAPE)
    lbm.u.from_numpy(u0)
    lbm.rho = ti.field(ti.f32, SHAPE)
    lbm.rho.from_numpy(rho0)
    lbm.phase = ti.field(ti.f32, SHAPE)
    lbm.solid = ti.field(ti.u8, SHAPE)
    lbm.solid.from_numpy(solid0)
    lbm.body_force = ti.Vector.field(3, ti.f32, SHAPE)
    lbm.body_force.from_numpy(base)
    mp = MultiphaseFlow3D(lbm)
    mp.phi.from_numpy(phi0)
    mp.phi_new.from_numpy(phi0)  # as after standardize_initial_state: phi_new's shell holds phi's
    out = {"phi": phi0, "u": u0, "rho": rho0, "base": base, "solid": solid0,
           "sigma": np.float32(mp.SURFACE_TENSION_COEFF), "width": np.float32(mp.INTERFACE_WIDTH),
           "mobility": np.float32(mp.MOBILITY), "rho_air": config.RHO_AIR, "rho_water": config.RHO_WATER}
    mp.compute_chemical_potential()
    out["mu"] = mp.mu.to_numpy()
    mp.compute_gradients()
    out["grad_phi"], out["normal"] = mp.grad_phi.to_numpy(), mp.normal.to_numpy()
    mp.compute_curvature()
    out["curvature"] = mp.curvature.to_numpy()
    mp.compute_surface_tension_force()
    out["surface_force"] = mp.surface_force.to_numpy()
    mp.apply_surface_tension()
    out["body_force"] = lbm.body_force.to_numpy()
    mp.update_phase_field_cahn_hilliard()
    out["phi_ch"] = mp.phi_new.to_numpy()
    mp.apply_phase_separation()
    out["phi_new"] = mp.phi_new.to_numpy()
    mp.copy_phase_field()
    mp.update_density_from_phase()
    out["rho_out"], out["phase_out"] = lbm.rho.to_numpy(), lbm.phase.to_numpy()
    np.savez_compressed(os.path.join(HERE, "multiphase_reference.npz"), **out)
    print("wrote multiphase_reference.npz")


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: make_multiphase_golden.py <path of the reference checkout>")
    main()
