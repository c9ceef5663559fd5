"""z-slab decomposition on one GPU: SlabLattice (each slab its own buffer through pog_step,
device-local halo copies around every odd step) against the undivided lattice.  Every cell is
computed by the same kernel from the same inputs, so the states and macroscopic fields must be
bit-identical; the FP64 sums differ only in summation order."""
import numpy as np
import pytest
import torch

from gpu_helpers import run_aa
from pour_over_coffee_lbm_gb300.params import LES_LOCAL, LES_STENCIL, STORE_F16S, STORE_F32, LatticeConfig
from pour_over_coffee_lbm_gb300.slabs import SlabLattice

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("storage,nslabs", [(STORE_F32, 2), (STORE_F32, 3), (STORE_F16S, 2)])
def test_slab_lattice_bit_identical(cuda, storage, nslabs):
    cfg = LatticeConfig(nx=40, ny=36, nz=44, storage=storage, band_thickness=3.0, les_mode=LES_LOCAL,
                        u_inlet=-0.05)
    steps = 21  # ends on the odd parity: the export reads the ghost slots
    ref = run_aa(cfg, steps)
    sl = SlabLattice(cfg, nslabs, flags=ref.flags.cpu().numpy())
    red = sl.run(steps, reduce=True, want_macro=True)
    torch.cuda.synchronize()
    assert np.array_equal(sl.natural(torch.float64).cpu().numpy(), ref.natural(np.float64))
    rho, u = sl.macroscopic()
    assert torch.equal(rho, ref.rho) and torch.equal(u, ref.u)
    assert np.allclose(red.cpu().numpy(), ref.red.cpu().numpy(), rtol=1e-12, atol=1e-12)
    # three more steps, an even count, from the decomposed state
    sl.run(3)
    ref.step(3)
    torch.cuda.synchronize()
    assert np.array_equal(sl.natural(torch.float64).cpu().numpy(), ref.natural(np.float64))


def test_slab_lattice_rejects_stencil_les(cuda):
    with pytest.raises(ValueError):
        SlabLattice(LatticeConfig(nx=16, ny=16, nz=16, les_mode=LES_STENCIL), 2)
