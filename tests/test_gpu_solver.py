"""The reference-facing solver object on the GPU: protocol conformance, accessors, the
coupled step against the oracle's coupled sequence, geometry replacement, VTK export."""
import os

import numpy as np
import pytest
import torch

from pour_over_coffee_lbm_gb300 import (CoffeeParticleSystem, GB300LBMSolver, LatticeConfig,
                                        ParticleConfig, create_unified_solver, validate_lbm_solver)
from pour_over_coffee_lbm_gb300.params import CELL_SOLID, LES_LOCAL, LES_STENCIL, seed_particles
from pour_over_coffee_lbm_gb300.protocol import ParticleCoupledLBMProtocol, get_solver_capabilities

pytestmark = pytest.mark.gpu


def test_protocol_and_accessors(cuda):
    s = GB300LBMSolver(LatticeConfig(nx=32, ny=32, nz=32, band_thickness=3.0))
    assert validate_lbm_solver(s)
    assert isinstance(s, ParticleCoupledLBMProtocol)
    caps = get_solver_capabilities(s)
    assert caps["basic_lbm"] and caps["les_turbulence"] and caps["vtk_export"]
    assert s.rho.shape == (32, 32, 32) and s.u.shape == (32, 32, 32, 3)
    assert s.f.shape == (32, 32, 32, 19)
    s.init_fields()
    for _ in range(5):
        s.step()
    d = s.get_diagnostics()
    assert d["stable"] and d["step"] == 5
    assert s.get_mass_conservation_error() < 1e-2
    assert s.get_kinetic_energy() >= 0
    rho = s.rho.to_numpy()
    assert rho.shape == (32, 32, 32) and np.isfinite(rho).all()
    assert s.opposite_dir.tolist() == [0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15]
    mem = s.get_memory_usage()
    assert mem["f"] == 19 * 32 ** 3 * 4
    u = create_unified_solver("auto", config=LatticeConfig(nx=16, ny=16, nz=16))
    assert validate_lbm_solver(u)


def test_body_force_and_geometry(cuda, tmp_path):
    s = GB300LBMSolver(LatticeConfig(nx=24, ny=24, nz=24))
    F = np.zeros((24, 24, 24, 3), np.float32)
    F[..., 0] = 1e-5
    s.add_force_term(F)
    s.step()
    assert s.body_force.to_numpy()[..., 0].max() == pytest.approx(1e-5)
    s.clear_body_force()
    mask = s.solid.to_numpy().astype(bool)
    mask[10:13, 10:13, 10:13] = True
    s.set_geometry(mask)
    assert np.array_equal(s.solid.to_numpy().astype(bool), mask)
    s.step()
    assert s.check_stability()
    shell_open = mask.copy()
    shell_open[0, 5, 5] = False
    with pytest.raises(ValueError):
        s.set_geometry(shell_open)
    path = str(tmp_path / "out")
    s.export_vtk(path)
    assert os.path.getsize(path + ".vtk") > 24 ** 3 * 4 * 5


def test_les_stencil_solver_matches_oracle(cuda, orc):
    cfg = LatticeConfig(nx=32, ny=32, nz=32, band_thickness=3.0, les_mode=LES_STENCIL, u_inlet=-0.05, cs_smag=0.3)
    s = GB300LBMSolver(cfg)
    s.run(29)
    _ = s.u.to_numpy()  # reading the accessor must not disturb the LES velocity history
    s.run(1, want_macro=True)
    flags, f, rho, u = orc.run(cfg, 30, np.float32)
    _, _, _, u64 = orc.run(cfg.replace(storage=3), 30, np.float64)
    fluid = (flags & CELL_SOLID) == 0
    gu = s._u.cpu().numpy()
    # FP32 bar: within 2x the FP32 oracle's own error against the FP64 oracle
    e_orc = np.linalg.norm(u[:, fluid] - u64[:, fluid]) / np.linalg.norm(u64[:, fluid])
    assert np.linalg.norm(gu[:, fluid] - u64[:, fluid]) / np.linalg.norm(u64[:, fluid]) <= 2 * e_orc + 1e-7
    assert np.linalg.norm(gu[:, fluid] - u[:, fluid]) / np.linalg.norm(u[:, fluid]) <= 2 * e_orc + 1e-7


def test_two_way_coupled_steps_vs_oracle(cuda, orc):
    """Coupled step = coupling pass on u of the current state, then one LBM step with the spread
    force (legacy/lbm_solver.py:1485-1509), repeated; oracle runs the same sequence."""
    cfg = LatticeConfig(nx=40, ny=40, nz=40, band_thickness=3.0, les_mode=LES_LOCAL)
    pc = ParticleConfig(count=3000, deterministic=True, sort_interval=5)
    s = GB300LBMSolver(cfg)
    ps = CoffeeParticleSystem(max_particles=3000, lattice=cfg, config=pc)
    ps.seed()
    steps = 12
    for _ in range(steps):
        s.step_with_two_way_coupling(ps, dt=1.0, relaxation_factor=0.8)
    torch.cuda.synchronize()
    # oracle: same sequence, FP32
    flags = orc.build_flags(cfg)
    f = orc.init_equilibrium(cfg, flags, np.float32)
    pos, vel, d, act = seed_particles(cfg, pc)
    drag = np.zeros_like(pos)
    fluid = (flags & CELL_SOLID) == 0
    # moments of the initial state (the step's rho/u outputs are those of its incoming state)
    _, _, u = orc.step(cfg, flags, f)
    for _ in range(steps):
        pos, vel, drag, act, fix, _ = orc.particles_couple(cfg, pc, pos, vel, d, drag, act, u)
        pdrag = (fix.astype(np.float64) / 2.0 ** 32).astype(np.float32).reshape(4, cfg.nz, cfg.ny, cfg.nx)
        f, rho, u = orc.step(cfg, flags, f, pdrag=pdrag)
    gpos = ps._pos[:, : pc.count].cpu().numpy()
    assert np.abs(gpos - pos).max() < 1e-4
    gu = s._u.cpu().numpy()
    assert np.linalg.norm(gu[:, fluid] - u[:, fluid]) / np.linalg.norm(u[:, fluid]) < 1e-4
    diag = ps.get_coupling_diagnostics()
    assert diag["active_particles"] > 0 and diag["max_reaction_force"] > 0
