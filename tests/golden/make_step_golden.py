"""Write tests/golden/step_reference.npz from the reference's own lattice-step kernels:

  src/core/legacy/lbm_solver.py
    _compute_macroscopic_quantities   :488-535  (rho, Guo half-force velocity)
    _apply_collision_and_streaming    :537-579  (BGK with tau by phase and the tau clamp)
    _compute_forcing_term / _compute_stable_guo_forcing / _calculate_forcing_terms
                                      :594-607, 688-764 (the legacy Guo form and its clamps)
    _perform_streaming                :609-628  (push with half-way bounce-back)
    swap_fields                       :630-654
  src/physics/filter_paper.py
    compute_forchheimer_resistance    :471-536  (explicit Darcy-Forchheimer drag with its cap)

executed in this container through taichi_standin.py (serially, float32).

    python tests/golden/make_step_golden.py <path of the reference checkout>

Lattice constants are patched into the reference's `config` so that the kernels run in a sane
regime (tau_water 0.52 and tau_air 2.0, so that the tau clamp [0.55, 1.90] binds in both phases;
gravity 2e-4 lattice units), and the seeded inputs put cells into every clamp: forces above the
|F| <= 10 scaling, post-scaling |F_q| above 0.5, velocities above the |u| <= 0.2 scaling.  LES is
off here (its viscosity is pinned by make_les_golden.py).  Three cases:
  step     random near-equilibrium state with u in all three directions (the reference's
           collision then mixes two D3Q19 orderings: its f_eq comes from lbm_algorithms.py's
           table while it streams along config/core.py's);
  step_x   a state whose velocity and forces point along x only, where the two orderings give
           the same f_eq;
  forch    the Forchheimer kernel on a random velocity field, with the physical prefactors
           patched to lattice values and a cap that binds in part of the cells.
The fixture travels with tests/test_step_reference.py.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SHAPE = (12, 10, 14)  # (NX, NY, NZ)
GRAVITY = 2e-4
TAU_WATER, TAU_AIR = 0.52, 2.0
CX = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0])
CY = np.array([0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1])
CZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1])
W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)


def feq(rho, u):
    """f_eq [19, ...] (float64) in the config/core.py ordering."""
    eu = CX[:, None] * u[0][None] + CY[:, None] * u[1][None] + CZ[:, None] * u[2][None]
    usq = (u ** 2).sum(0)
    return W[:, None] * rho[None] * (1 + 3 * eu + 4.5 * eu * eu - 1.5 * usq[None])


def inputs(rng, along_x):
    nx, ny, nz = SHAPE
    n = nx * ny * nz
    solid = rng.uniform(size=SHAPE) < 0.1
    solid[0] = solid[-1] = True
    solid[:, 0] = solid[:, -1] = True
    solid[:, :, 0] = solid[:, :, -1] = True
    phase = np.where(rng.uniform(size=SHAPE) < 0.2, 0.2, 1.0).astype(np.float32)
    rho = 1.0 + 0.05 * rng.uniform(-1, 1, n)
    u = 0.05 * rng.uniform(-1, 1, (3, n))
    force = 1e-4 * rng.normal(size=(3, n))
    if along_x:
        u[1:] = 0.0
        force[1:] = 0.0
        phase[:] = 1.0  # gravity points along z: this case runs without it
    f = feq(rho, u)
    if not along_x:
        f = f + 0.002 * rng.normal(size=f.shape) * W[:, None]
    else:
        # noise symmetric in +-y and +-z keeps the y and z momenta exactly zero
        pairs_y = [(3, 4), (7, 9), (8, 10), (15, 16), (17, 18)]
        pairs_z = [(5, 6), (11, 13), (12, 14), (15, 17), (16, 18)]
        noise = 0.002 * rng.normal(size=(19, n)) * W[:, None]
        for a, b in pairs_y + pairs_z:
            noise[b] = noise[a]
        f = f + noise
    flat = solid.reshape(-1, order="C")
    idx = np.flatnonzero(~flat)
    if not along_x:
        # clamp regimes: strong forces (|F| > 10 scaling; |F_q| > 0.5 in air cells), fast cells
        # (|u| > 0.2 scaling)
        strong = rng.choice(idx, 12, replace=False)
        force[:, strong] = rng.normal(size=(3, 12)) * 20.0
        fast = rng.choice(np.setdiff1d(idx, strong), 8, replace=False)
        uf = 0.35 * rng.uniform(-1, 1, (3, 8))
        f[:, fast] = feq(rho[fast], uf)
    # (NX, NY, NZ, ...) Taichi layouts
    f4 = f.reshape((19,) + SHAPE).astype(np.float32)
    bf = np.moveaxis(force.reshape((3,) + SHAPE), 0, -1).astype(np.float32)
    return solid, phase, f4, bf


def run_step(LBMSolver, ti, solid, phase, f4, bf, gravity):
    import config
    config.GRAVITY_LU = gravity
    s = LBMSolver()
    s.solid.from_numpy(solid.astype(np.uint8))
    s.phase.from_numpy(phase)
    s.body_force.from_numpy(bf)
    s.f.from_numpy(f4)
    s.f_new.from_numpy(np.zeros_like(f4))
    s._compute_macroscopic_quantities()
    rho = s.rho.to_numpy()
    u = s.u.to_numpy()
    s._apply_collision_and_streaming()
    s.swap_fields()
    return rho, u, s.f.to_numpy()


def main():
    sys.path.insert(0, HERE)
    import taichi_standin
    ti = taichi_standin.install()
    sys.path.insert(0, sys.argv[1])
    import config  # the reference's config package
    config.NX, config.NY, config.NZ = SHAPE
    config.ENABLE_LES = False
    config.TAU_WATER, config.TAU_AIR = TAU_WATER, TAU_AIR
    from src.core.legacy.lbm_solver import LBMSolver
    rng = np.random.default_rng(2024)
    out = {"gravity": np.float64(GRAVITY), "tau_water": np.float64(TAU_WATER), "tau_air": np.float64(TAU_AIR)}
    for name, along_x in (("step", False), ("step_x", True)):
        solid, phase, f4, bf = inputs(rng, along_x)
        g = 0.0 if along_x else GRAVITY
        rho, u, fo = run_step(LBMSolver, ti, solid, phase, f4, bf, g)
        out.update({name + "/solid": solid.astype(np.uint8), name + "/phase": phase, name + "/f_in": f4,
                    name + "/body_force": bf, name + "/rho": rho, name + "/u": u, name + "/f_out": fo,
                    name + "/gravity": np.float64(g)})
    # Forchheimer drag: lattice prefactors (viscosity 0.1, density 1, unit scales), cap 0.01 * 0.02
    config.WATER_VISCOSITY_90C, config.WATER_DENSITY_90C = 0.1, 1.0
    config.SCALE_TIME, config.SCALE_LENGTH, config.SCALE_VELOCITY, config.DT = 1.0, 1.0, 0.02, 1.0
    from src.physics.filter_paper import FilterPaperSystem
    lbm = LBMSolver()
    fps = FilterPaperSystem(lbm)
    zone = (rng.uniform(size=SHAPE) < 0.4).astype(np.int32)
    solid = np.zeros(SHAPE, np.uint8)
    solid[rng.uniform(size=SHAPE) < 0.1] = 1
    K, beta = 5e-3, 0.8
    fps.filter_zone.from_numpy(zone)
    lbm.solid.from_numpy(solid)
    fps.permeability.from_numpy(np.where(zone == 1, K, 0.0).astype(np.float32))
    fps.forchheimer_coeff.from_numpy(np.where(zone == 1, beta, 0.0).astype(np.float32))
    # |u| log-uniform over 1e-7 .. 1e-2: the drag is below the cap for the slow cells, capped above
    dirs = rng.normal(size=SHAPE + (3,))
    dirs /= np.linalg.norm(dirs, axis=-1, keepdims=True)
    uu = (dirs * 10.0 ** rng.uniform(-7, -2, size=SHAPE + (1,))).astype(np.float32)
    uu[rng.uniform(size=SHAPE) < 0.05] = 0.0  # the |u| <= 1e-8 gate
    lbm.u.from_numpy(uu)
    bf0 = (1e-5 * rng.normal(size=SHAPE + (3,))).astype(np.float32)
    lbm.body_force.from_numpy(bf0)
    fps.compute_forchheimer_resistance()
    out.update({"forch/zone": zone, "forch/solid": solid, "forch/u": uu, "forch/body_force_in": bf0,
                "forch/body_force_out": lbm.body_force.to_numpy(), "forch/K": np.float64(K),
                "forch/beta": np.float64(beta), "forch/viscosity": np.float64(0.1),
                "forch/cap": np.float64(0.01 * 0.02 / 1.0)})
    np.savez_compressed(os.path.join(HERE, "step_reference.npz"), **out)
    print("wrote step_reference.npz")


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: make_step_golden.py <path of the reference checkout>")
    main()
