"""The reference's own LBMDiagnostics outputs (tests/golden/diag_reference.*): the fixture is
self-consistent, and the particle-bed statistics, which pour_over_coffee_lbm_gb300 computes with
the reference's numpy arithmetic on host copies, match it bit for bit on the CPU."""
import numpy as np

from diag_golden import Field, Holder, load
from pour_over_coffee_lbm_gb300.diagnostics import LBMDiagnostics


def test_fixture_is_the_documented_case():
    z, meta = load()
    nx, ny, nz = meta["shape"]
    assert z["rho_a"].shape == (nx, ny, nz) and z["u_b"].shape == (nx, ny, nz, 3)
    r0, r1 = meta["reports"]
    assert r0["temporal_stability"] == {"status": "first_step"}
    # numpy on the stored fields reproduces the stored reference values
    um = np.sqrt((z["u_b"] ** 2).sum(-1))
    assert r1["flow_analysis"]["max_velocity"] == float(np.max(um))
    assert r1["lbm_quality"]["max_density_deviation"] == float(np.max(np.abs(z["rho_b"] - 1.0)))
    assert r1["multiphase"]["interface_thickness"] == int(((z["phi_b"] > 0.1) & (z["phi_b"] < 0.9)).sum())


def test_bed_dynamics_bit_exact():
    z, meta = load()
    nx, ny, nz = meta["shape"]
    lbm = Holder()
    lbm.NX, lbm.NY, lbm.NZ = nx, ny, nz
    ps = Holder()
    ps.position, ps.active = Field(z["position"]), Field(z["active"])
    d = LBMDiagnostics(lbm, particles=ps)
    d.scale_length = meta["scale_length"]
    assert d._analyze_coffee_bed_dynamics() == meta["reports"][1]["v60_physics"]["particle_dynamics"]
