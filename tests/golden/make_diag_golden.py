"""Generate tests/golden/diag_reference.{npz,json}: the reference's own LBMDiagnostics
(src/visualization/lbm_diagnostics.py, plain numpy, importable without Taichi) run on seeded
synthetic fields.

    python tests/golden/make_diag_golden.py <path of the reference checkout>

The script imports the reference from its checkout (its path is the script's required first argument), so it runs only
where that checkout exists; the fixtures it writes travel with the tests.  The reference reads its
grid size, gravity and scales from its `config` package.  Its NX/NY/NZ (the region split of
detailed_flow_analysis and the particles' radial centre) are set to the fixture's grid, and
GRAVITY_LU to the lattice gravity 1e-5 of LatticeConfig's default, so that the same fields fed to
pour_over_coffee_lbm_gb300's LBMDiagnostics give comparable reports.  DT, SCALE_LENGTH and
SCALE_VELOCITY keep the reference's values (1.0, 0.000625, 0.01).

Two checks are recorded: state A at step 0 (first call: no previous fields), then state B at step
100, both with force_update=True, with a phase field, particles and a constant pour flow rate.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SHAPE = (16, 12, 20)  # (NX, NY, NZ), the reference's field indexing
NP = 300
FLOW = 0.05


class _Field:
    def __init__(self, a):
        self.a = a

    def to_numpy(self):
        return self.a.copy()


class _Lattice:
    pass


class _Holder:
    pass


class _Pour:
    def get_current_flow_rate(self):
        return FLOW


def states(seed=11):
    rng = np.random.default_rng(seed)
    nx, ny, nz = SHAPE
    z = np.arange(nz)[None, None, :]
    out = []
    for k in range(2):
        # a wet lower region (plane-mean density > 1.1) that rises between the two checks
        wet = (z < 6 + 3 * k).astype(np.float32)
        rho = (1.0 + 0.01 * rng.normal(size=SHAPE) + 0.2 * wet).astype(np.float32)
        u = (0.03 * rng.normal(size=SHAPE + (3,))).astype(np.float32)
        u[:, :, 10:12] = 0.0  # cells at rest (|u| <= 1e-10)
        u[0, 0, 0] = (0.1, 0.05, -0.02)  # one cell above Mach 0.1
        phi = np.clip(rng.uniform(-0.2, 1.2, size=SHAPE), 0.0, 1.0).astype(np.float32)
        out.append((rho, u, phi))
    pos = np.stack([rng.uniform(0, nx, NP), rng.uniform(0, ny, NP), rng.uniform(0, nz / 2, NP)], 1).astype(np.float32)
    active = (rng.uniform(size=NP) < 0.8).astype(np.int32)
    return out, pos, active


def clean(d):
    """The report without its wall-clock entries, as JSON-ready Python values."""
    d = {k: v for k, v in d.items() if k not in ("timestamp", "diagnostics_performance")}

    def conv(v):
        if isinstance(v, dict):
            return {k: conv(x) for k, x in v.items()}
        if isinstance(v, (list, tuple)):
            return [conv(x) for x in v]
        if isinstance(v, np.generic):
            return v.item()
        return v
    return conv(d)


def main():
    ref = sys.argv[1]
    sys.path.insert(0, ref)
    import config  # the reference's config package
    config.NX, config.NY, config.NZ = SHAPE
    config.GRAVITY_LU = 1e-5
    from src.visualization.lbm_diagnostics import LBMDiagnostics
    (a, b), pos, active = states()
    lbm, mp, ps = _Lattice(), _Holder(), _Holder()
    ps.position, ps.active = _Field(pos), _Field(active)
    diag = LBMDiagnostics(lbm, multiphase=mp, particles=ps, pouring=_Pour())
    reports = []
    for step, (rho, u, phi) in ((0, a), (100, b)):
        lbm.rho, lbm.u, mp.phi = _Field(rho), _Field(u), _Field(phi)
        reports.append(clean(diag.update_diagnostics(step, float(step), force_update=True)))
    np.savez_compressed(os.path.join(HERE, "diag_reference.npz"), rho_a=a[0], u_a=a[1], phi_a=a[2],
                        rho_b=b[0], u_b=b[1], phi_b=b[2], position=pos, active=active)
    with open(os.path.join(HERE, "diag_reference.json"), "w") as f:
        json.dump({"shape": list(SHAPE), "flow_rate": FLOW, "dt": config.DT,
                   "scale_length": config.SCALE_LENGTH, "scale_velocity": config.SCALE_VELOCITY,
                   "gravity_lu": config.GRAVITY_LU, "reports": reports}, f, indent=1, sort_keys=True)
    print("wrote diag_reference.npz / .json")


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: make_diag_golden.py <path of the reference checkout>")
    main()
