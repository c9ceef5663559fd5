"""GPU parity of the row-tiled step kernel (csrc/lbm_tma.cu) against the register-staged step
kernel (csrc/lbm_aa.cu, selected with POG_STEP_CELLS), both through pog_step.

Both kernels run the same per-cell collision code on the same incoming populations, so the bar is
bit equality: the whole distribution state, and the rho / u outputs, after even and odd step
counts, in every storage the row-tiled kernel serves and with every optional input of the step.
The FP64 sums are accumulated by atomics in a block order that differs between the kernels, so
they agree to 1e-12 relative.  The register-staged kernel itself is pinned to the oracle by
test_gpu_lbm.py."""
import ctypes

import numpy as np
import pytest
import torch

from gpu_helpers import AARun, P, S, gpu_flags, lib, wall_list
from pour_over_coffee_lbm_gb300 import _lib
from pour_over_coffee_lbm_gb300.params import (CELL_POROUS, CELL_SOLID, DRAG_EXPLICIT_CAP, LES_LOCAL,
                                               LES_STENCIL, STORE_BF16S, STORE_F16S, STORE_F32, LatticeConfig,
                                               porosity_field)

pytestmark = pytest.mark.gpu


def _pair(cfg, steps, eps=None, force=None, pdrag=None, reduce=True):
    """Run the same case with both kernels; return the two AARun objects."""
    out = []
    for rows in (False, True):
        r = AARun(cfg, eps=eps, force=force, pdrag=pdrag, rows=rows, cells=not rows)
        if steps > 1:
            r.step(steps - 1, reduce=reduce, macro=False)
        r.step(1, reduce=reduce, macro=True)
        out.append(r)
    torch.cuda.synchronize()
    assert lib().pog_device_status(1) == 0, lib().pog_last_error()
    return out


def _assert_same(a, b):
    assert np.array_equal(a.natural(), b.natural())
    assert torch.equal(a.rho, b.rho)
    assert torch.equal(a.u, b.u)
    ra, rb = a.red.cpu().numpy(), b.red.cpu().numpy()
    assert np.allclose(ra[:5], rb[:5], rtol=1e-12, atol=1e-12), (ra, rb)
    assert ra[5] == rb[5] == 0


def test_wall_list_is_the_fluid_cells_with_a_solid_neighbour(cuda):
    cfg = LatticeConfig(nx=64, ny=48, nz=56, band_thickness=3.0)
    p = cfg.to_c()
    fl = gpu_flags(cfg)
    cells = np.sort(wall_list(p, fl).cpu().numpy())
    f = fl.cpu().numpy().reshape(-1).astype(np.int64)
    c = np.arange(f.size)
    i, k = c % cfg.nx, c // (cfg.nx * cfg.ny)
    want = c[((f & CELL_SOLID) == 0) & (((f >> 8) & 0x7FFFE) != 0) & (k >= 1) & (k < cfg.nz - 1) & (i >= 1)
             & (i < cfg.nx - 1)]
    assert np.array_equal(cells, want)
    # a short capacity writes a prefix but still reports the full count
    count = torch.zeros(1, dtype=torch.int32, device="cuda")
    buf = torch.full((10,), -7, dtype=torch.int32, device="cuda")
    _lib.check(lib().pog_wall_list(ctypes.byref(p), P(fl), P(buf), 5, P(count), S()))
    assert int(count.item()) == want.size
    b = buf.cpu().numpy()
    assert np.all(b[5:] == -7) and np.all(np.isin(b[:5], want))


CASES = {
    "fp32_plain": LatticeConfig(nx=64, ny=64, nz=64),
    "fp32_les_band": LatticeConfig(nx=64, ny=64, nz=64, les_mode=LES_LOCAL, band_thickness=3.0, u_inlet=-0.05,
                                   cs_smag=0.3),
    "fp16s_les_band": LatticeConfig(nx=64, ny=64, nz=64, les_mode=LES_LOCAL, band_thickness=3.0, storage=STORE_F16S,
                                    u_inlet=-0.05, cs_smag=0.3),
    "bf16s_les_band": LatticeConfig(nx=64, ny=64, nz=64, les_mode=LES_LOCAL, band_thickness=3.0, storage=STORE_BF16S),
    "fp32_explicit_drag_96": LatticeConfig(nx=96, ny=88, nz=72, band_thickness=3.0, drag_mode=DRAG_EXPLICIT_CAP),
    "fp16s_les_stencil": LatticeConfig(nx=48, ny=40, nz=52, les_mode=LES_STENCIL, band_thickness=2.0,
                                       storage=STORE_F16S, u_inlet=-0.05, cs_smag=0.3),
    "fp16s_row_320": LatticeConfig(nx=320, ny=28, nz=24, storage=STORE_F16S, les_mode=LES_LOCAL,
                                   band_thickness=2.0, inlet_radius=5.0),
}


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("steps", [37, 40])
def test_rows_kernel_equals_register_kernel(cuda, name, steps):
    a, b = _pair(CASES[name], steps)
    assert b.walls.numel() > 0
    _assert_same(a, b)


def test_rows_kernel_with_every_step_input(cuda, orc):
    """Per-cell porosity, an explicit force field, and a particle drag deposit (dense and masked)."""
    cfg = LatticeConfig(nx=64, ny=56, nz=60, band_thickness=3.0, les_mode=LES_LOCAL, u_inlet=-0.04)
    fl = orc.build_flags(cfg)
    eps = porosity_field(cfg, fl, seed=7).reshape(cfg.nz, cfg.ny, cfg.nx)
    rng = np.random.default_rng(3)
    shape = (cfg.nz, cfg.ny, cfg.nx)
    force = (1e-6 * rng.standard_normal((3,) + shape)).astype(np.float32)
    pdrag = np.zeros((4,) + shape, np.float32)
    dep = rng.uniform(size=shape) < 0.02
    pdrag[0][dep] = rng.uniform(0.0, 0.05, int(dep.sum()))
    for a in range(1, 4):
        pdrag[a][dep] = 1e-3 * rng.standard_normal(int(dep.sum()))
    a, b = _pair(cfg, 25, eps=eps, force=force, pdrag=pdrag)
    _assert_same(a, b)
    # the same deposit read through the deposit mask (bits only at the deposit cells)
    n = cfg.ncell
    words = np.zeros((n + 31) // 32, np.uint32)
    idx = np.flatnonzero(dep.reshape(-1))
    np.bitwise_or.at(words, idx >> 5, (np.uint32(1) << (idx & 31).astype(np.uint32)))
    mask = torch.as_tensor(words.view(np.int32)).cuda()
    runs = []
    for rows in (False, True):
        r = AARun(cfg, eps=eps, force=force, pdrag=pdrag, rows=rows, cells=not rows)
        r.p.deposit_mask = P(mask)
        r.step(24, reduce=True, macro=False)
        r.step(1, reduce=True, macro=True)
        runs.append(r)
    torch.cuda.synchronize()
    _assert_same(*runs)
    # the masked read is the dense read wherever the deposit is zero outside the mask
    assert np.array_equal(runs[1].natural(), b.natural())


def test_kernels_mix_step_by_step(cuda):
    """Between steps both kernels leave the same state: alternating them changes nothing."""
    cfg = LatticeConfig(nx=64, ny=64, nz=64, les_mode=LES_LOCAL, band_thickness=3.0, storage=STORE_F16S)
    ref = AARun(cfg, cells=True)
    mix = AARun(cfg, rows=True, cells=True)
    walls = mix.p.wall_cells
    for t in range(30):
        ref.step(1, macro=False)
        mix.p.wall_cells = walls if (t % 3) else None  # registers every third step
        mix.step(1, macro=False)
    torch.cuda.synchronize()
    assert np.array_equal(ref.natural(), mix.natural())


def test_rows_kernel_falls_back_where_it_does_not_apply(cuda):
    """72-byte FP16 rows (nx = 36) cannot be bulk-copied: pog_step takes the register kernel."""
    cfg = LatticeConfig(nx=36, ny=32, nz=40, storage=STORE_F16S, band_thickness=2.0)
    a, b = _pair(cfg, 9)
    _assert_same(a, b)


def test_solver_uses_the_rows_kernel(cuda):
    from pour_over_coffee_lbm_gb300.solver import GB300LBMSolver
    cfg = LatticeConfig(nx=64, ny=64, nz=64, les_mode=LES_LOCAL, band_thickness=3.0)
    s1 = GB300LBMSolver(cfg)
    s2 = GB300LBMSolver(cfg, step_kernel="rows")
    assert s2._p.wall_cells and s2._p.n_wall_cells > 0 and not s1._p.wall_cells
    s1.run(21, want_macro=True)
    s2.run(21, want_macro=True)
    torch.cuda.synchronize()
    # solid slots differ (the row-tiled kernel keeps its bounce-back mailboxes there): compare the
    # natural-layout state, which holds the fluid cells' populations
    assert np.array_equal(s1.f.to_numpy(), s2.f.to_numpy())
    assert torch.equal(s1._u, s2._u) and torch.equal(s1._rho, s2._rho)
    # porous cells exist in this case
    assert int(((s2.flags & CELL_POROUS) != 0).sum()) > 0
