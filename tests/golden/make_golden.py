"""Generate the golden fixtures of tests/golden/ from the CPU oracle.

    python tests/golden/make_golden.py

The reference (Python + Taichi) cannot run in this environment, so trajectory-level goldens
come from the oracle (oracle/pog_oracle*.cpp), whose function-level behaviour is pinned by the
reference's own known-answer tests (tests/test_oracle_kat.py).  The fixtures freeze the oracle's
outputs on small seeded cases so the GPU tests can compare against them without the oracle, and
the CPU tests can detect any drift of the oracle itself.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from pour_over_coffee_lbm_gb300.params import (DRAG_EXPLICIT_CAP, FORCING_REFERENCE, LES_LOCAL,  # noqa: E402
                                               LES_STENCIL, LatticeConfig, ParticleConfig,
                                               porosity_field, seed_particles)

N = 16
STEPS = 40


def cases():
    base = LatticeConfig(nx=N, ny=N, nz=N, cone_apex_z=3.0, inlet_radius=5.0)
    band = base.replace(band_thickness=3.0)
    # a faster jet and a larger Smagorinsky constant so the LES relaxation visibly matters
    les = band.replace(u_inlet=-0.06, cs_smag=0.4, les_strain_floor=1e-4)
    return {
        "plain": base,
        "les_off_fast": les,
        "les_local": les.replace(les_mode=LES_LOCAL),
        "les_stencil": les.replace(les_mode=LES_STENCIL),
        "porous_explicit": band.replace(drag_mode=DRAG_EXPLICIT_CAP, drag_cap=1e-4),
        "reference_forcing": base.replace(forcing_mode=FORCING_REFERENCE, clamp_tau=True),
        "profile": base.replace(inlet_coef=(0.1, -0.2, 0.05) + (0.0,) * 13),
    }


def adjoint_case():
    return LatticeConfig(nx=12, ny=12, nz=12, cone_apex_z=2.0, inlet_radius=4.0, hole_radius=2.0,
                         band_thickness=2.0, les_mode=LES_LOCAL, les_strain_floor=0.0, cs_smag=0.3,
                         u_inlet=-0.05, inlet_coef=(0.05,) + (0.0,) * 15)


def main():
    out = {}
    for name, cfg in cases().items():
        red = np.zeros(6)
        flags, f, rho, u = O.run(cfg, STEPS, np.float64, reductions=red)
        out[name + "/flags"] = flags
        out[name + "/rho"] = rho.astype(np.float64)
        out[name + "/u"] = u.astype(np.float64)
        out[name + "/red"] = red
    # per-cell porosity (band) case
    cfg = cases()["les_local"]
    flags = O.build_flags(cfg)
    eps = porosity_field(cfg, flags, seed=1234)
    red = np.zeros(6)
    _, f, rho, u = O.run(cfg, STEPS, np.float64, flags=flags, eps=eps, reductions=red)
    out["eps_field/eps"] = eps
    out["eps_field/rho"] = rho
    out["eps_field/u"] = u
    out["eps_field/red"] = red
    # particles: 600 seeded particles on a 20^3 lattice with a smooth velocity field
    pc = ParticleConfig(count=600, deterministic=True)
    lc = LatticeConfig(nx=N, ny=N, nz=N, cone_apex_z=3.0)
    pos, vel, d, act = seed_particles(lc, pc)
    act[::37] = 0
    z, y, x = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    u = np.stack([0.01 * np.sin(0.3 * y), 0.01 * np.cos(0.2 * x), -0.005 * np.sin(0.25 * z)]).astype(np.float32)
    keys, perm = O.particles_bin(lc, pos, act)
    p2, v2, dr2, a2, fix, uat = O.particles_couple(lc, pc, pos, vel, d, np.zeros_like(pos), act, u)
    out.update({"particles/pos": pos, "particles/vel": vel, "particles/d": d, "particles/active": act,
                "particles/u": u, "particles/keys": keys, "particles/perm": perm,
                "particles/pos_out": p2, "particles/vel_out": v2, "particles/drag_out": dr2,
                "particles/active_out": a2, "particles/force_fix": fix, "particles/u_at": uat})
    # adjoint: 12^3, 12 steps, LES local, band with per-cell porosity
    acfg = adjoint_case()
    aflags = O.build_flags(acfg)
    aeps = porosity_field(acfg, aflags, seed=7)
    ge, gi = O.outflow_gradient(acfg, 12, flags=aflags, eps=aeps)
    out["adjoint/eps"] = aeps
    out["adjoint/grad_eps"] = ge
    out["adjoint/grad_inlet"] = gi
    out["adjoint/loss"] = np.array([O.outflow_loss(acfg, 12, flags=aflags, eps=aeps)])
    path = os.path.join(HERE, "oracle_small.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
