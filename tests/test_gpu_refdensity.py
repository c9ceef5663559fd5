"""FP16S with a per-cell reference density (pog_params.density_ref, lbm_ref.cu).

Each slot is stored relative to the reference density of the cell that owns it, refreshed by that
cell every even step; the odd step moves streamed populations between the neighbours' references
and its own.  The stored state therefore decodes to the same f, only the rounding point differs
from plain FP16S.  Checked through the C ABI:
- against a GPU FP64 run of the same case: the u error stays at FP16S's level or below it (5e-3
  relative L2 after 100 steps, the storage's parity bar, and no larger than plain FP16S's error
  times 1.5), ρ within 1e-4;
- the natural export decodes every slot with its owner's reference, at even and odd parity: import
  then export returns the state to FP16 rounding;
- pog_macroscopic gives the moments the next step computes;
- mass is conserved as in plain FP16S (FP64 sums);
- checkpoint and resume of a solver in this form continue bit for bit;
- invalid uses are rejected (another storage, the push step)."""
import ctypes

import numpy as np
import pytest
import torch

from gpu_helpers import AARun, P, S, lib, rel_l2
from pour_over_coffee_lbm_gb300 import _lib
from pour_over_coffee_lbm_gb300.params import CELL_SOLID, LES_LOCAL, STORE_F16S, STORE_F32, STORE_F64, LatticeConfig

pytestmark = pytest.mark.gpu


def _cfg(**kw):
    base = dict(nx=48, ny=48, nz=48, band_thickness=3.0, les_mode=LES_LOCAL, storage=STORE_F16S)
    base.update(kw)
    return LatticeConfig(**base)


def _ref_run(cfg):
    return AARun(cfg, ref_density=True)


def _advance(r, steps, reduce=False):
    if steps > 1:
        r.step(steps - 1, reduce=reduce, macro=False)
    r.step(1, reduce=reduce, macro=True)
    torch.cuda.synchronize()
    assert lib().pog_device_status(1) == 0


def test_error_vs_fp64_at_most_plain_fp16s(cuda):
    cfg = _cfg()
    steps = 100
    ref = _ref_run(cfg)
    _advance(ref, steps, reduce=True)
    plain = AARun(cfg)
    _advance(plain, steps, reduce=True)
    f64 = AARun(cfg.replace(storage=STORE_F64))
    _advance(f64, steps, reduce=True)
    fluid = ((f64.flags & CELL_SOLID) == 0).cpu().numpy()
    u64 = f64.u.cpu().numpy()[:, fluid]
    e_ref = rel_l2(ref.u.cpu().numpy()[:, fluid], u64)
    e_plain = rel_l2(plain.u.cpu().numpy()[:, fluid], u64)
    print("u rel L2 vs FP64 after %d steps: reference density %.2e, plain FP16S %.2e" % (steps, e_ref, e_plain))
    assert e_ref < 5e-3 and e_ref <= 1.5 * e_plain
    assert rel_l2(ref.rho.cpu().numpy()[fluid], f64.rho.cpu().numpy()[fluid]) < 1e-4
    # mass: the same FP64 sums as plain FP16S to storage rounding
    assert abs(ref.red[0].item() - plain.red[0].item()) < 1e-6 * abs(plain.red[0].item())
    # the reference holds this step's densities (FP16-rounded deviations) on fluid cells
    d = ref.dref.float().cpu().numpy().reshape(cfg.nz, cfg.ny, cfg.nx)
    assert np.abs(d[fluid]).max() > 0


@pytest.mark.parametrize("steps", [20, 21])
def test_export_import_round_trip(cuda, steps):
    cfg = _cfg(nx=24, ny=24, nz=24)
    r = _ref_run(cfg)
    _advance(r, steps)
    nat = r.natural(np.float64)
    assert np.isfinite(nat).all()
    # the export's decoding (each slot with its owner's reference) against the macroscopic pass's
    # (its own code path, which moves every streamed slot to the reading cell's reference)
    rho = torch.empty_like(r.rho)
    _lib.check(lib().pog_macroscopic(ctypes.byref(r.p), P(r.f), P(r.flags), r.t, None, None, P(rho), None, S()))
    torch.cuda.synchronize()
    fluid = ((r.flags & CELL_SOLID) == 0).cpu().numpy()
    inlet_outlet = ((r.flags & 0x06) != 0).cpu().numpy()  # their rho is imposed, not summed
    keep = fluid & ~inlet_outlet
    assert np.abs(nat.sum(0)[keep] - rho.cpu().numpy()[keep]).max() < 1e-6
    if steps % 2:
        return  # import writes an even-parity state
    f2 = torch.empty_like(r.f)
    _lib.check(lib().pog_import_natural(ctypes.byref(r.p), P(torch.as_tensor(nat).cuda()), STORE_F64, P(r.flags),
                                        P(f2), S()))
    r.f = f2
    nat2 = r.natural(np.float64)
    fluid = ((r.flags & CELL_SOLID) == 0).cpu().numpy()
    # one FP16 rounding of deviations of a few 1e-3 at scale 2^12
    assert np.abs(nat2[:, fluid] - nat[:, fluid]).max() < 1e-7


def test_macroscopic_matches_next_step_moments(cuda):
    cfg = _cfg(nx=32, ny=32, nz=32)
    r = _ref_run(cfg)
    _advance(r, 11)
    rho = torch.empty_like(r.rho)
    u = torch.empty_like(r.u)
    _lib.check(lib().pog_macroscopic(ctypes.byref(r.p), P(r.f), P(r.flags), r.t, None, None, P(rho), P(u), S()))
    r.step(1, macro=True)
    torch.cuda.synchronize()
    fluid = (r.flags & CELL_SOLID) == 0
    assert torch.allclose(rho[fluid], r.rho[fluid], rtol=1e-6, atol=0)
    assert torch.allclose(u[:, fluid], r.u[:, fluid], rtol=0, atol=1e-8)


def test_solver_checkpoint_resume(cuda, tmp_path):
    from pour_over_coffee_lbm_gb300 import GB300LBMSolver
    from pour_over_coffee_lbm_gb300.diagnostics import load_checkpoint, save_checkpoint
    cfg = _cfg(nx=32, ny=32, nz=32)
    s1 = GB300LBMSolver(cfg, density_reference=True)
    s1.run(15)
    path = str(tmp_path / "ck.npz")
    save_checkpoint(path, s1)
    s1.run(10, want_macro=True)
    s2 = GB300LBMSolver(cfg, density_reference=True)
    load_checkpoint(path, s2)
    s2.run(10, want_macro=True)
    torch.cuda.synchronize()
    assert torch.equal(s1._f.view(torch.int16), s2._f.view(torch.int16))
    assert torch.equal(s1._dref.view(torch.int16), s2._dref.view(torch.int16))
    assert torch.equal(s1._u, s2._u)
    s3 = GB300LBMSolver(cfg)
    with pytest.raises(ValueError):
        load_checkpoint(path, s3)


def test_rejected_uses(cuda):
    p = _cfg(storage=STORE_F32).to_c()
    d = torch.zeros(p.nx * p.ny * p.nz, dtype=torch.float16, device="cuda")
    p.density_ref = d.data_ptr()
    assert lib().pog_validate_params(ctypes.byref(p)) == -1
    assert b"density_ref" in lib().pog_last_error()
    cfg = _cfg(nx=16, ny=16, nz=16)
    p = cfg.to_c()
    d = torch.zeros(cfg.ncell, dtype=torch.float16, device="cuda")
    p.density_ref = d.data_ptr()
    f = torch.zeros((19, cfg.ncell), dtype=torch.float16, device="cuda")
    g = torch.zeros_like(f)
    fl = torch.zeros(cfg.ncell, dtype=torch.int32, device="cuda")
    rc = lib().pog_step_push(ctypes.byref(p), P(f), P(g), P(fl), None, None, None, None, None, None, None, S())
    assert rc == -1
    assert b"reference density" in lib().pog_last_error()
    with pytest.raises(ValueError):
        from pour_over_coffee_lbm_gb300 import GB300LBMSolver
        GB300LBMSolver(_cfg(storage=STORE_F32), density_reference=True)


def test_stencil_les_and_particles(cuda):
    """The per-cell reference form with the LES stencil mode (per-cell kernel on both steps) and
    with two-way coupled particles (their deposit cells take the per-cell path of the two-cell
    even step): both stay with plain FP16S to FP16 rounding."""
    from pour_over_coffee_lbm_gb300 import CoffeeParticleSystem, GB300LBMSolver, ParticleConfig
    from pour_over_coffee_lbm_gb300.params import LES_STENCIL
    cfg = _cfg(nx=40, ny=40, nz=40, les_mode=LES_STENCIL)
    out = []
    for ref in (False, True):
        s = GB300LBMSolver(cfg, density_reference=ref)
        s.run(59)
        s.run(1, want_macro=True)
        out.append(s)
    fluid = ((out[0].flags & CELL_SOLID) == 0)
    e = rel_l2(out[1]._u[:, fluid].cpu().numpy(), out[0]._u[:, fluid].cpu().numpy())
    print("LES stencil, reference vs plain FP16S after 60 steps: u rel L2 %.2e" % e)
    assert out[1].check_stability() and e < 5e-3
    cfg = _cfg(nx=48, ny=48, nz=48)
    pc = ParticleConfig(count=3000, deterministic=True)
    runs = []
    for ref in (False, True):
        s = GB300LBMSolver(cfg, density_reference=ref)
        ps = CoffeeParticleSystem(max_particles=pc.count, lattice=cfg, config=pc)
        ps.seed()
        for _ in range(40):
            s.step_with_two_way_coupling(ps)
        s.run(1, want_macro=True)
        runs.append((s, ps))
    fluid = ((runs[0][0].flags & CELL_SOLID) == 0)
    e = rel_l2(runs[1][0]._u[:, fluid].cpu().numpy(), runs[0][0]._u[:, fluid].cpu().numpy())
    dp = (runs[1][1]._pos[:, :pc.count] - runs[0][1]._pos[:, :pc.count]).abs().max().item()
    print("coupled, reference vs plain FP16S after 40 steps: u rel L2 %.2e, particle max |dx| %.1e" % (e, dp))
    assert runs[1][0].check_stability() and e < 5e-3 and dp < 1e-2


def test_odd_nx_per_cell_even_step(cuda):
    """An odd nx keeps the even step per cell (ref_even_cell) in the reference form too."""
    cfg = LatticeConfig(nx=37, ny=29, nz=41, band_thickness=2.5, cone_apex_z=5.5, center_x=17.25, center_y=13.0,
                        cone_half_angle_deg=35.0, inlet_radius=7.5, hole_radius=1.5, les_mode=LES_LOCAL,
                        storage=STORE_F16S)
    ref = _ref_run(cfg)
    _advance(ref, 40)
    plain = AARun(cfg)
    _advance(plain, 40)
    fluid = ((ref.flags & CELL_SOLID) == 0).cpu().numpy()
    assert rel_l2(ref.u.cpu().numpy()[:, fluid], plain.u.cpu().numpy()[:, fluid]) < 5e-3
