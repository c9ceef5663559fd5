"""The oracle's Smagorinsky viscosity (the step's LES stencil mode) against the reference's own
LES kernel run on the same velocity field (tests/golden/les_reference.npz, made by
tests/golden/make_les_golden.py from src/physics/les_turbulence.py:318-380): the strain-rate
floor, the mask gate, the boundary zeros and nu = C_s^2 |S|."""
import os

import numpy as np

import oracle as orc
from pour_over_coffee_lbm_gb300.params import CELL_POROUS, LES_STENCIL, LatticeConfig


def test_les_viscosity_matches_reference_kernel():
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "les_reference.npz"))
    nx, ny, nz = z["mask"].shape
    cfg = LatticeConfig(nx=nx, ny=ny, nz=nz, les_mode=LES_STENCIL, cs_smag=float(z["cs"]),
                        les_strain_floor=1e-3, les_nu_max=0.1)
    # the reference's LES mask 0 is the porous band of the flag words
    flags = np.ascontiguousarray(np.where(z["mask"] == 0, CELL_POROUS, 0).transpose(2, 1, 0)).astype(np.uint32)
    u = np.ascontiguousarray(z["u"].transpose(3, 2, 1, 0))
    nu = orc.les_nu(cfg, flags, u)
    ref = z["nu"].transpose(2, 1, 0)
    assert np.array_equal(nu == 0, ref == 0)  # the same gates fire in the same cells
    assert (ref > 0).sum() > 300 and (ref == 0).sum() > 300
    assert np.allclose(nu, ref, rtol=1e-6, atol=0)
