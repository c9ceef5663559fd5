"""Diagnostics and outputs on the GPU: pog_field_stats against numpy on the same fields, the
LBMDiagnostics reports against the reference's formulas evaluated with numpy on to_numpy()
copies (src/visualization/lbm_diagnostics.py:151-407), the asynchronous snapshot files, and a
checkpoint/resume that continues a coupled run bit for bit."""
import ctypes
import math

import numpy as np
import pytest
import torch

from gpu_helpers import P, S, lib
from pour_over_coffee_lbm_gb300 import _lib
from pour_over_coffee_lbm_gb300.diagnostics import (STAT_COUNT, LBMDiagnostics, SnapshotWriter, load_checkpoint,
                                                    save_checkpoint)
from pour_over_coffee_lbm_gb300.params import LatticeConfig, ParticleConfig

pytestmark = pytest.mark.gpu


# one cell per thread; runs of several steps whose plane boundaries fall inside a 32-cell step;
# planes of 20 cells (several boundaries per step); long runs (about 1,100 cells per warp)
@pytest.mark.parametrize("shape", [(40, 36, 44), (100, 60, 50), (5, 4, 3000), (256, 256, 64)])
def test_field_stats_match_numpy(cuda, shape):
    cfg = LatticeConfig(nx=shape[0], ny=shape[1], nz=shape[2])
    rng = np.random.default_rng(3)
    shape = (cfg.nz, cfg.ny, cfg.nx)
    rho = (1.0 + 0.01 * rng.normal(size=shape)).astype(np.float32)
    u = (0.05 * rng.normal(size=(3,) + shape)).astype(np.float32)
    u[:, 5:9] = 0.0  # some cells at rest (|u| <= 1e-10)
    rp = (rho + 1e-4 * rng.normal(size=shape)).astype(np.float32)
    upv = (u + 1e-3 * rng.normal(size=u.shape)).astype(np.float32)
    dev = [torch.as_tensor(a).cuda() for a in (rho, u, rp, upv)]  # kept alive across the call
    st = torch.empty(STAT_COUNT, dtype=torch.float64, device="cuda")
    zp = torch.empty(cfg.nz, dtype=torch.float64, device="cuda")
    p = cfg.to_c()
    _lib.check(lib().pog_field_stats(ctypes.byref(p), *[P(t) for t in dev], P(st), P(zp), S()))
    st, zp = st.cpu().numpy(), zp.cpu().numpy()
    r, ud = rho.astype(np.float64), u.astype(np.float64)
    um = np.sqrt((ud ** 2).sum(0))
    act = um > 1e-10
    nz = cfg.nz
    z30, z80 = int(0.3 * nz), int(0.8 * nz)
    ref = [r.sum(), (r * r).sum(), (r * ud[0]).sum(), (r * ud[1]).sum(), (r * ud[2]).sum(), um.max(),
           um[act].sum(), act.sum(), (um ** 2).sum(), um.sum(), (um > 0.1 / math.sqrt(3)).sum(),
           np.abs(r - cfg.rho0).max(), ((r - rp) ** 2).sum(), ((ud - upv) ** 2).sum(),
           ud[0].sum(), ud[1].sum(), ud[2].sum(), (ud[0] ** 2).sum(), (ud[1] ** 2).sum(), (ud[2] ** 2).sum(),
           um[:z30].sum(), um[z30:z80].sum(), um[z80:].sum()]
    assert np.allclose(st, ref, rtol=1e-9, atol=1e-9)
    assert np.allclose(zp, r.sum(axis=(1, 2)), rtol=1e-12)


def _reference_reports(rho_np, u_np, prev, n):
    """The reference's formulas on (NX, NY, NZ) host arrays (lbm_diagnostics.py:151-226,372-407)."""
    umag = np.sqrt((u_np.astype(np.float64) ** 2).sum(-1))
    cs = 1 / math.sqrt(3)
    out = {"max_mach": umag.max() / cs, "mean_density": rho_np.astype(np.float64).mean(),
           "density_variation_coeff": rho_np.astype(np.float64).std() / rho_np.astype(np.float64).mean(),
           "max_velocity": umag.max(), "velocity_std": umag.std()}
    act = umag[umag > 1e-10]
    out["mean_velocity"] = act.mean()
    out["flow_complexity"] = float(np.linalg.norm(np.std(u_np.astype(np.float64), axis=(0, 1, 2))))
    nz = rho_np.shape[2]
    out["top_region_flow"] = umag[:, :, int(nz * 0.8):].mean()
    out["bottom_region_flow"] = umag[:, :, :int(nz * 0.3)].mean()
    if prev is not None:
        out["relative_density_change"] = np.linalg.norm(rho_np - prev[0]) / np.linalg.norm(rho_np)
        out["relative_velocity_change"] = np.linalg.norm(u_np - prev[1]) / (np.linalg.norm(u_np) + 1e-10)
    return out


def test_diagnostics_reports_match_reference_formulas(cuda):
    from pour_over_coffee_lbm_gb300.solver import GB300LBMSolver
    cfg = LatticeConfig(nx=32, ny=32, nz=40, band_thickness=3.0)
    s = GB300LBMSolver(cfg)
    diag = LBMDiagnostics(s)
    s.run(20, want_macro=True)
    d0 = diag.update_diagnostics(0, 0.0, force_update=True)
    prev = (s.rho.to_numpy().astype(np.float64), s.u.to_numpy().astype(np.float64))
    s.run(10, want_macro=True)
    d1 = diag.update_diagnostics(100, 10.0, force_update=True)
    ref = _reference_reports(s.rho.to_numpy(), s.u.to_numpy(), prev, s.n)
    q, fa, ts = d1["lbm_quality"], d1["flow_analysis"], d1["temporal_stability"]
    for k in ("max_mach", "mean_density", "density_variation_coeff"):
        assert math.isclose(q[k], ref[k], rel_tol=1e-6), k
    for k in ("max_velocity", "mean_velocity", "velocity_std", "flow_complexity", "top_region_flow",
              "bottom_region_flow"):
        assert math.isclose(fa[k], ref[k], rel_tol=1e-5, abs_tol=1e-12), k
    assert math.isclose(ts["relative_density_change"], ref["relative_density_change"], rel_tol=1e-5)
    assert math.isclose(ts["relative_velocity_change"], ref["relative_velocity_change"], rel_tol=1e-5)
    assert d0["temporal_stability"] == {"status": "first_step"}
    c = d1["conservation"]
    assert math.isclose(c["total_mass"], float(s.rho.to_numpy().astype(np.float64).sum()), rel_tol=1e-9)
    assert "wetting_front_position" in d1["v60_physics"]


def test_reports_match_the_reference_diagnostics(cuda):
    """The reference's LBMDiagnostics run on the same fields (tests/golden/diag_reference.*,
    made by tests/golden/make_diag_golden.py from its own code): every report of both checks,
    to the reference's float32 precision, with a phase field, particles and a pour flow rate."""
    from diag_golden import Field, Holder, Pour, compare, load
    from pour_over_coffee_lbm_gb300.solver import GB300LBMSolver
    z, meta = load()
    nx, ny, nz = meta["shape"]
    s = GB300LBMSolver(LatticeConfig(nx=nx, ny=ny, nz=nz, gravity=(0.0, 0.0, -meta["gravity_lu"])))
    mp, ps = Holder(), Holder()
    ps.position, ps.active = Field(z["position"]), Field(z["active"])
    diag = LBMDiagnostics(s, multiphase=mp, particles=ps, pouring=Pour(meta["flow_rate"]))
    diag.dt, diag.scale_length, diag.scale_velocity = meta["dt"], meta["scale_length"], meta["scale_velocity"]
    ours = []
    for step, tag in ((0, "a"), (100, "b")):
        # the fields as the solver's moments, (NX, NY, NZ[, 3]) -> device (NZ, NY, NX) / (3, NZ, NY, NX)
        s._rho.copy_(torch.as_tensor(z["rho_" + tag].transpose(2, 1, 0).copy()))
        s._u.copy_(torch.as_tensor(z["u_" + tag].transpose(3, 2, 1, 0).copy()))
        s._macro_dirty = s._u_stale = False
        mp.phi = torch.as_tensor(z["phi_" + tag].transpose(2, 1, 0).copy()).cuda()
        ours.append(diag.update_diagnostics(step, float(step), force_update=True))
    for o, r in zip(ours, meta["reports"]):
        compare(o, r, loose=("mass_conservation_error", "total_mass", "initial_mass"))


def test_snapshot_files(cuda, tmp_path):
    from pour_over_coffee_lbm_gb300.solver import GB300LBMSolver
    s = GB300LBMSolver(LatticeConfig(nx=24, ny=28, nz=32))
    s.run(5, want_macro=True)
    w = SnapshotWriter(s)
    base = str(tmp_path / "coffee_sim_3d_000005")
    w.save(base)
    w.wait()
    rho = np.load(base + "_density_data.npy")
    umag = np.load(base + "_velocity_data.npy")
    assert rho.shape == (24, 28, 32) and np.array_equal(rho, s.rho.to_numpy())
    ref = np.sqrt((s.u.to_numpy().astype(np.float32) ** 2).sum(-1))
    assert np.allclose(umag, ref, rtol=1e-6, atol=1e-9)


def test_export_data_for_analysis(cuda, tmp_path):
    from pour_over_coffee_lbm_gb300.diagnostics import export_data_for_analysis
    from pour_over_coffee_lbm_gb300.solver import GB300LBMSolver
    s = GB300LBMSolver(LatticeConfig(nx=12, ny=10, nz=14))
    s.run(5, want_macro=True)
    out = export_data_for_analysis(s, 5.0, 5, out_dir=str(tmp_path))
    assert len(out) == 2
    z = np.load(out[1])
    assert np.array_equal(z["density_field"], s.rho.to_numpy().astype(np.float64))


def test_checkpoint_resume_is_bit_identical(cuda, tmp_path):
    from pour_over_coffee_lbm_gb300.particles import CoffeeParticleSystem
    from pour_over_coffee_lbm_gb300.pouring import PrecisePouringSystem
    from pour_over_coffee_lbm_gb300.solver import GB300LBMSolver
    cfg = LatticeConfig(nx=32, ny=32, nz=40, band_thickness=3.0)
    pc = ParticleConfig(count=800, deterministic=True)

    def make():
        s = GB300LBMSolver(cfg)
        ps = CoffeeParticleSystem(pc.count, lattice=cfg, config=pc)
        ps.seed()
        pour = PrecisePouringSystem(cfg, diameter=4.0)
        pour.start_pouring(pattern="spiral")
        return s, ps, pour

    def advance(s, ps, pour, n):
        for _ in range(n):
            pour.apply_pouring_force(s)
            s.step_with_two_way_coupling(ps)

    s, ps, pour = make()
    advance(s, ps, pour, 7)
    path = str(tmp_path / "ck.npz")
    save_checkpoint(path, s, ps, pour)
    advance(s, ps, pour, 6)
    f_a, pos_a = s.f.to_numpy(), ps.position.to_numpy()
    s2, ps2, pour2 = make()
    load_checkpoint(path, s2, ps2, pour2)
    advance(s2, ps2, pour2, 6)
    assert s2.t == s.t
    assert np.array_equal(s2.f.to_numpy(), f_a)
    assert np.array_equal(ps2.position.to_numpy(), pos_a)
