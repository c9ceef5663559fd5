"""Write tests/golden/reference_config.json: the reference's config constants that
pour_over_coffee_lbm_gb300 mirrors (lattice and multiphase parameters, the physical scales of the
diagnostics and the analysis export), read by importing the reference's own `config` package.

    python tests/golden/make_config_golden.py <path of the reference checkout>

Runs only where the reference checkout exists (its path is the script's required first argument); the JSON travels with
the tests (tests/test_reference_config.py).
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
NAMES = ["NX", "NY", "NZ", "TAU_WATER", "TAU_AIR", "SMAGORINSKY_CONSTANT", "RHO_0", "RHO_WATER", "RHO_AIR",
         "CS2", "DT", "SCALE_LENGTH", "SCALE_VELOCITY", "SCALE_TIME", "TIME_SCALE_OPTIMIZATION_FACTOR",
         "L_CHAR", "U_CHAR", "NU_CHAR", "SURFACE_TENSION_LU", "PHYSICAL_DOMAIN_SIZE", "Q_3D"]


def main():
    sys.path.insert(0, sys.argv[1])
    import config  # the reference's config package
    out = {k: getattr(config, k) for k in NAMES}
    with open(os.path.join(HERE, "reference_config.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("wrote reference_config.json")


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: make_config_golden.py <path of the reference checkout>")
    main()
