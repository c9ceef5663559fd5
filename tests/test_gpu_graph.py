"""CUDA-graph replay of the solver's steps (GB300LBMSolver.capture / StepGraph) against the same
steps launched one by one: plain steps and two-way coupled steps (deterministic deposit, so the
particle order cannot change a bit) give identical states."""
import pytest
import torch

from pour_over_coffee_lbm_gb300.params import LES_LOCAL, LatticeConfig, ParticleConfig

pytestmark = pytest.mark.gpu


def _cfg():
    return LatticeConfig(nx=40, ny=40, nz=44, band_thickness=3.0, les_mode=LES_LOCAL)


def test_plain_graph_matches_eager(cuda):
    from pour_over_coffee_lbm_gb300.solver import GB300LBMSolver
    a, b = GB300LBMSolver(_cfg()), GB300LBMSolver(_cfg())
    a.run(20)
    g = b.capture(10)
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    assert a.t == b.t == 20
    assert torch.equal(a._f, b._f)
    assert torch.equal(a.rho.tensor, b.rho.tensor) and torch.equal(a.u.tensor, b.u.tensor)


def test_coupled_graph_matches_eager(cuda):
    from pour_over_coffee_lbm_gb300.particles import CoffeeParticleSystem
    from pour_over_coffee_lbm_gb300.solver import GB300LBMSolver
    pc = ParticleConfig(count=2000, deterministic=True, sort_interval=5)

    def make():
        s = GB300LBMSolver(_cfg())
        ps = CoffeeParticleSystem(pc.count, lattice=_cfg(), config=pc)
        ps.seed()
        for _ in range(4):
            s.step_with_two_way_coupling(ps)
        return s, ps

    (a, pa), (b, pb) = make(), make()
    for _ in range(20):
        a.step_with_two_way_coupling(pa)
    g = b.capture(10, pb)
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    assert a.t == b.t
    assert torch.equal(a._f, b._f)
    assert torch.equal(pa._pos, pb._pos) and torch.equal(pa._vel, pb._vel)
    assert torch.equal(a._pdrag, b._pdrag) and torch.equal(a._dmask, b._dmask)
    # and the next eager step continues both alike
    a.step_with_two_way_coupling(pa)
    b.step_with_two_way_coupling(pb)
    torch.cuda.synchronize()
    assert torch.equal(a._f, b._f)
