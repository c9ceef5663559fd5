"""Constants mirrored from the reference's config package, checked against its own values
(tests/golden/reference_config.json, written by tests/golden/make_config_golden.py from the
reference's `config`): the reference-config mapping of the lattice parameters, the multiphase
defaults and the physical scales of the diagnostics and the analysis export."""
import json
import math
import os
import types

from pour_over_coffee_lbm_gb300 import diagnostics, multiphase
from pour_over_coffee_lbm_gb300.params import LatticeConfig, from_reference_config

REF = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_config.json")))


def test_from_reference_config_maps_the_lattice_parameters():
    lc = from_reference_config(types.SimpleNamespace(**REF))
    assert (lc.nx, lc.ny, lc.nz) == (REF["NX"], REF["NY"], REF["NZ"])
    assert lc.tau == REF["TAU_WATER"] and lc.cs_smag == REF["SMAGORINSKY_CONSTANT"] and lc.rho0 == REF["RHO_0"]
    assert from_reference_config(types.SimpleNamespace(**REF), nx=32).nx == 32


def test_multiphase_defaults():
    assert LatticeConfig().tau_air == REF["TAU_AIR"]
    assert multiphase.RHO_WATER == REF["RHO_WATER"] and multiphase.RHO_AIR == REF["RHO_AIR"]
    assert multiphase.SURFACE_TENSION_LU == REF["SURFACE_TENSION_LU"]
    assert multiphase.SCALE_LENGTH == REF["SCALE_LENGTH"]


def test_export_scales():
    sc = diagnostics.EXPORT_SCALES
    assert math.isclose(sc["scale_length"], REF["SCALE_LENGTH"], rel_tol=1e-15)
    assert sc["scale_velocity"] == REF["SCALE_VELOCITY"]
    assert sc["time_factor"] == REF["TIME_SCALE_OPTIMIZATION_FACTOR"]
    assert math.isclose(sc["scale_length"] / sc["scale_velocity"] * sc["time_factor"], REF["SCALE_TIME"], rel_tol=1e-12)
    assert (sc["l_char"], sc["u_char"], sc["nu_char"]) == (REF["L_CHAR"], REF["U_CHAR"], REF["NU_CHAR"])
