"""The two-cell even-step kernel of the 16-bit storages (aa_pair_even_kernel, lbm_pair.cu) against
the per-cell kernel (aa_step_kernel) and the oracle's emulation of the same storage rounding.

The two kernels compute the same update; the two-cell kernel chooses its own FMA contraction in
the collision, so from the same state one step stores values that agree to one unit in the last
place of the 16-bit format (FP16: 2^-10 relative, BF16: 2^-7), or to FP32 rounding of the
collision's terms where they cancel, and the same macroscopic outputs.  Over many steps they are held to the storage's parity bar against the oracle
(5e-3 relative L2 on u after 100 steps, as the per-cell kernel), and to each other.  Where the
two-cell kernel does not apply (odd nx, the LES stencil mode, the reference forcing form) pog_step
runs the per-cell kernel: bit for bit the same state.
"""
import ctypes

import numpy as np
import pytest
import torch

from gpu_helpers import AARun, P, lib, rel_l2, run_aa
from pour_over_coffee_lbm_gb300.params import (CELL_SOLID, FORCING_REFERENCE, LES_LOCAL, LES_STENCIL,
                                               STEP_CELLS, STORE_BF16S, STORE_F16S, LatticeConfig)

pytestmark = pytest.mark.gpu

STORAGES = [STORE_F16S, STORE_BF16S]


def _cfg(storage, **kw):
    base = dict(nx=48, ny=48, nz=48, band_thickness=3.0, les_mode=LES_LOCAL, storage=storage)
    base.update(kw)
    return LatticeConfig(**base)


def _ordered(t):
    """16-bit floats as integers in value order (adjacent representable values differ by 1)."""
    b = t.contiguous().view(torch.int16).cpu().numpy().astype(np.int32)
    mag = b & 0x7FFF
    return np.where(b < 0, -mag, mag)


def _agree(fa, fb):
    """Stored 16-bit values within one unit in the last place, or -- where the collision's terms
    cancel to a value far below their size -- within FP32 rounding of the terms (2^-20 of the
    largest stored value of the direction).  Returns (fraction identical, largest ulp distance)."""
    ka, kb = _ordered(fa), _ordered(fb)
    d = np.abs(ka - kb)
    a = fa.float().cpu().numpy()
    b = fb.float().cpu().numpy()
    atol = 2.0 ** -20 * np.abs(a).reshape(19, -1).max(1).reshape(19, 1, 1, 1)
    ok = (d <= 1) | (np.abs(a - b) <= atol)
    bad = np.argwhere(~ok)
    assert ok.all(), (bad[:5], a[tuple(bad[:5].T)], b[tuple(bad[:5].T)])
    return (d == 0).mean(), d.max()


def _twin(cfg, steps, force=None, pdrag=None, dmask=None):
    """A flowing state after `steps` per-cell steps, and a second run holding a copy of it; the
    first runs the per-cell kernel from here on, the second the default (two-cell) kernel."""
    a = AARun(cfg, force=force, pdrag=pdrag, cells=True)
    if dmask is not None:
        a.dmask = dmask
        a.p.deposit_mask = P(dmask)
    a.step(steps, macro=False)
    b = AARun(cfg, flags=a.flags.cpu().numpy(), force=force, pdrag=pdrag)
    if dmask is not None:
        b.dmask = dmask
        b.p.deposit_mask = P(dmask)
    b.f.copy_(a.f)
    b.t = a.t
    assert a.p.step_kernel == STEP_CELLS and b.p.step_kernel == 0
    return a, b


@pytest.mark.parametrize("storage", STORAGES)
def test_odd_step_is_the_per_cell_kernel(cuda, storage):
    """The two-cell kernel takes the even steps only: an odd step leaves the same bits."""
    a, b = _twin(_cfg(storage), 41)
    a.step(1, macro=True)
    b.step(1, macro=True)
    assert torch.equal(a.f.view(torch.int16), b.f.view(torch.int16))
    assert torch.equal(a.u, b.u) and torch.equal(a.rho, b.rho)


@pytest.mark.parametrize("storage", STORAGES)
def test_even_step_matches_per_cell_kernel(cuda, storage):
    parity = 0
    cfg = _cfg(storage)
    a, b = _twin(cfg, 40 + parity)
    for r in (a, b):
        r.red.zero_()
        r.step(1, reduce=True, macro=True)
    torch.cuda.synchronize()
    assert lib().pog_device_status(1) == 0
    same, dmax = _agree(a.f, b.f)
    print("storage %d parity %d: %.4f of the slots identical, largest difference %d ulp" % (storage, parity, same, dmax))
    # the two-cell kernel ran: its own rounding shows somewhere
    assert same < 1.0
    fluid = ((a.flags & CELL_SOLID) == 0).cpu().numpy()
    ua, ub = a.u.cpu().numpy()[:, fluid], b.u.cpu().numpy()[:, fluid]
    assert rel_l2(ub, ua) < 1e-5
    assert np.abs(b.rho.cpu().numpy()[fluid] - a.rho.cpu().numpy()[fluid]).max() < 1e-6
    ra, rb = a.red.cpu().numpy(), b.red.cpu().numpy()
    assert abs(rb[0] - ra[0]) < 1e-9 * abs(ra[0])  # mass: the same moment sums, summed the same way
    assert np.allclose(rb[1:4], ra[1:4], rtol=1e-4, atol=1e-9 * abs(ra[0]))


@pytest.mark.parametrize("storage", STORAGES)
def test_one_step_with_force_and_deposit(cuda, storage):
    """External force field, particle deposit at a few cells (their pairs take the per-cell
    path inside the two-cell kernel, the rest stays paired)."""
    cfg = _cfg(storage)
    rng = np.random.default_rng(3)
    shape = (cfg.nz, cfg.ny, cfg.nx)
    force = (1e-6 * rng.standard_normal((3,) + shape)).astype(np.float32)
    pdrag = np.zeros((4,) + shape, np.float32)
    cells = rng.choice(cfg.ncell, 300, replace=False)
    flat = pdrag.reshape(4, -1)
    flat[0, cells] = 1e-3
    flat[1:, cells] = 1e-6 * rng.standard_normal((3, cells.size))
    words = np.zeros((cfg.ncell + 31) // 32, np.uint32)
    np.bitwise_or.at(words, cells // 32, (1 << (cells % 32)).astype(np.uint32))
    dmask = torch.as_tensor(words.view(np.int32)).cuda()
    for parity in (0, 1):
        a, b = _twin(cfg, 30 + parity, force=force, pdrag=pdrag, dmask=dmask)
        a.step(1, macro=True)
        b.step(1, macro=True)
        torch.cuda.synchronize()
        _agree(a.f, b.f)
        fluid = ((a.flags & CELL_SOLID) == 0).cpu().numpy()
        assert rel_l2(b.u.cpu().numpy()[:, fluid], a.u.cpu().numpy()[:, fluid]) < 1e-5
        # the deposit cells' own velocities: the per-cell path inside the two-cell kernel
        ua, ub = a.u.cpu().numpy().reshape(3, -1)[:, cells], b.u.cpu().numpy().reshape(3, -1)[:, cells]
        live = fluid.reshape(-1)[cells]
        assert np.array_equal(ua[:, live], ub[:, live])


@pytest.mark.parametrize("storage", STORAGES)
@pytest.mark.parametrize("cells", [False, True])
def test_100_steps_vs_oracle_emulation(cuda, orc, storage, cells):
    cfg = _cfg(storage)
    r = run_aa(cfg, 100, cells=cells)
    flags, f, rho, u = orc.run(cfg, 100, np.float32)
    fluid = (flags & CELL_SOLID) == 0
    e = rel_l2(r.u.cpu().numpy()[:, fluid], u[:, fluid])
    print("storage %d %s kernel: u rel L2 vs oracle %.2e" % (storage, "per-cell" if cells else "two-cell", e))
    assert e < 5e-3
    assert rel_l2(r.rho.cpu().numpy()[fluid], rho[fluid]) < 1e-4


@pytest.mark.parametrize("storage", STORAGES)
def test_200_steps_two_kernels_stay_together(cuda, storage):
    cfg = _cfg(storage, nx=64, ny=64, nz=64)
    a = run_aa(cfg, 200, cells=True)
    b = run_aa(cfg, 200)
    fluid = ((a.flags & CELL_SOLID) == 0).cpu().numpy()
    e = rel_l2(b.u.cpu().numpy()[:, fluid], a.u.cpu().numpy()[:, fluid])
    print("storage %d: two-cell vs per-cell u rel L2 after 200 steps %.2e" % (storage, e))
    assert e < 5e-3
    ra, rb = a.red.cpu().numpy(), b.red.cpu().numpy()
    assert abs(rb[0] - ra[0]) < 1e-6 * abs(ra[0])


@pytest.mark.parametrize("kw", [dict(nx=37, ny=29, nz=41, center_x=17.25, center_y=13.0, inlet_radius=7.5,
                                     hole_radius=1.5, cone_apex_z=5.5, cone_half_angle_deg=35.0),
                                dict(les_mode=LES_STENCIL), dict(forcing_mode=FORCING_REFERENCE)])
def test_where_it_does_not_apply_the_per_cell_kernel_runs(cuda, kw):
    cfg = _cfg(STORE_F16S, **kw)
    a = run_aa(cfg, 21, cells=True)
    b = run_aa(cfg, 21)
    assert torch.equal(a.f.view(torch.int16), b.f.view(torch.int16))


def test_solver_default_is_the_two_cell_kernel(cuda):
    from pour_over_coffee_lbm_gb300 import GB300LBMSolver
    cfg = _cfg(STORE_F16S)
    s1 = GB300LBMSolver(cfg)
    s2 = GB300LBMSolver(cfg, step_kernel="registers")
    assert s1._p.step_kernel == 0 and s2._p.step_kernel == STEP_CELLS
    for s in (s1, s2):
        s.run(59)
        s.run(1, want_macro=True)
    assert s1.check_stability() and s2.check_stability()
    assert not torch.equal(s1._f.view(torch.int16), s2._f.view(torch.int16))
    fluid = ((s1.flags & CELL_SOLID) == 0)
    assert rel_l2(s1._u[:, fluid].cpu().numpy(), s2._u[:, fluid].cpu().numpy()) < 5e-3
    # enable_les_turbulence keeps the kernel choice
    s2.enable_les_turbulence(0.1)
    assert s2._p.step_kernel == STEP_CELLS


def test_unknown_step_kernel_is_rejected(cuda):
    p = _cfg(STORE_F16S).to_c()
    p.step_kernel = 7
    assert lib().pog_validate_params(ctypes.byref(p)) == -1
    assert b"step_kernel" in lib().pog_last_error()
