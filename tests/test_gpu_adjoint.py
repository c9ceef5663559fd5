"""GPU adjoint checks.

1. The hand-written CUDA adjoint (FP64 storage) equals the oracle's forward-mode dual-number
   differentiation of the restated step (committed fixture, 12^3, 12 steps) to 1e-7 relative
   (the loss is an outlet momentum sum that cancels to ~1e-4 of its terms, so FP64 runs with
   different FMA contraction agree to ~1e-9 on it).
2. Checkpointed recomputation (every K steps) gives the same gradients as K = T.
3. Gradients agree with central finite differences (h = 1e-3) of the FP64 forward to 1e-4
   relative, on the inlet-profile coefficients and on porous cells with non-negligible
   gradients.
4. The torch.autograd.Function returns those gradients; the FP32 adjoint is within 1e-3 of FP64.
"""
import os
import sys

import numpy as np
import pytest
import torch

from pour_over_coffee_lbm_gb300.adjoint import OutflowAdjoint, outflow_loss
from pour_over_coffee_lbm_gb300.params import CELL_POROUS, STORE_F32, STORE_F64, porosity_field

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "oracle_small.npz")
sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))


def _case():
    import make_golden as mg
    return mg.adjoint_case()


def test_adjoint_matches_dual_number_oracle(cuda):
    g = np.load(GOLD)
    cfg = _case().replace(storage=STORE_F64)
    run = OutflowAdjoint(cfg, steps=12, checkpoint_every=4)
    eps = torch.as_tensor(g["adjoint/eps"]).reshape(cfg.nz, cfg.ny, cfg.nx)
    J = run.forward(eps, cfg.inlet_coef)
    res = run.backward()
    assert abs(J - g["adjoint/loss"][0]) <= 1e-8 * abs(g["adjoint/loss"][0])
    gi = res.grad_inlet.cpu().numpy()
    ref_i = g["adjoint/grad_inlet"]
    assert np.abs(gi - ref_i).max() <= 1e-7 * np.abs(ref_i).max()
    ge = res.grad_porosity.cpu().numpy()
    ref = g["adjoint/grad_eps"]
    assert np.abs(ge - ref).max() <= 1e-7 * np.abs(ref).max()


def test_checkpointing_is_exact(cuda):
    cfg = _case().replace(storage=STORE_F64, nx=16, ny=16, nz=16)
    from gpu_helpers import gpu_flags
    fl = gpu_flags(cfg).cpu().numpy()
    eps = torch.as_tensor(porosity_field(cfg, fl, seed=3)).reshape(cfg.nz, cfg.ny, cfg.nx)
    a = OutflowAdjoint(cfg, steps=20, checkpoint_every=20)
    a.forward(eps, cfg.inlet_coef)
    ra = a.backward()
    b = OutflowAdjoint(cfg, steps=20, checkpoint_every=3)
    b.forward(eps, cfg.inlet_coef)
    rb = b.backward()
    assert torch.equal(ra.grad_inlet, rb.grad_inlet)
    assert torch.equal(ra.grad_porosity, rb.grad_porosity)


def test_finite_differences(cuda):
    cfg = _case().replace(storage=STORE_F64, nx=20, ny=20, nz=20, cone_apex_z=3.0, inlet_radius=5.0)
    T = 40
    from gpu_helpers import gpu_flags
    fl = gpu_flags(cfg).cpu().numpy()
    eps = torch.as_tensor(porosity_field(cfg, fl, seed=5)).reshape(cfg.nz, cfg.ny, cfg.nx)
    run = OutflowAdjoint(cfg, steps=T, checkpoint_every=10)
    run.forward(eps, cfg.inlet_coef)
    res = run.backward()
    h = 1e-3
    coef = np.array(cfg.inlet_coef, np.float64)
    for k in (0, 1, 5, 15):
        cp = coef.copy(); cp[k] += h
        cm = coef.copy(); cm[k] -= h
        fd = (run.loss(eps, cp) - run.loss(eps, cm)) / (2 * h)
        ad = res.grad_inlet[k].item()
        assert abs(ad - fd) <= 1e-4 * abs(fd) + 1e-14, (k, ad, fd)
    ge = res.grad_porosity.cpu().numpy().reshape(-1)
    band = np.flatnonzero((fl.reshape(-1) & CELL_POROUS) != 0)
    big = band[np.argsort(-np.abs(ge[band]))[:8]]
    flat = eps.reshape(-1)
    for c in big:
        ep = flat.clone(); ep[c] += h
        em = flat.clone(); em[c] -= h
        # eps is float32: use the representable perturbation actually applied
        hh = (ep[c].double() - em[c].double()).item() / 2
        fd = (run.loss(ep.reshape(eps.shape), coef) - run.loss(em.reshape(eps.shape), coef)) / (2 * hh)
        assert abs(ge[c] - fd) <= 1e-4 * abs(fd), (c, ge[c], fd)


def test_autograd_function_and_fp32(cuda):
    cfg = _case().replace(storage=STORE_F64, nx=16, ny=16, nz=16)
    from gpu_helpers import gpu_flags
    fl = gpu_flags(cfg).cpu().numpy()
    eps = torch.as_tensor(porosity_field(cfg, fl, seed=9)).reshape(cfg.nz, cfg.ny, cfg.nx).cuda().requires_grad_(True)
    coef = torch.tensor(cfg.inlet_coef, dtype=torch.float64, device="cuda", requires_grad=True)
    run = OutflowAdjoint(cfg, steps=16, checkpoint_every=4)
    J = outflow_loss(eps, coef, run)
    ge, gc = torch.autograd.grad(J, (eps, coef))
    ref = OutflowAdjoint(cfg, steps=16, checkpoint_every=16)
    ref.forward(eps.detach(), cfg.inlet_coef)
    rr = ref.backward()
    assert torch.allclose(gc, rr.grad_inlet, rtol=1e-12, atol=0)
    assert torch.allclose(ge.double(), rr.grad_porosity.float().double(), rtol=1e-6, atol=0)
    r32 = OutflowAdjoint(cfg.replace(storage=STORE_F32), steps=16, checkpoint_every=4)
    r32.forward(eps.detach(), cfg.inlet_coef)
    g32 = r32.backward()
    assert torch.allclose(g32.grad_inlet, rr.grad_inlet, rtol=1e-3, atol=1e-3 * rr.grad_inlet.abs().max().item())


def test_adjoint_rejects_unsupported_modes(cuda):
    from pour_over_coffee_lbm_gb300 import _lib
    from pour_over_coffee_lbm_gb300.params import DRAG_EXPLICIT_CAP
    cfg = _case().replace(storage=STORE_F64, drag_mode=DRAG_EXPLICIT_CAP)
    run = OutflowAdjoint(cfg, steps=2, checkpoint_every=1)
    with pytest.raises(_lib.PogError):
        run.forward(None, cfg.inlet_coef)
        run.backward()


def _stencil_case():
    from pour_over_coffee_lbm_gb300.params import LES_STENCIL
    # the reference-faithful LES: nu_sgs from central differences of the previous step's u
    return _case().replace(storage=STORE_F64, les_mode=LES_STENCIL, cs_smag=0.4)


def test_stencil_adjoint_matches_dual_number_oracle(cuda, orc):
    """LES stencil mode (les_turbulence.py:318-380): dJ/du crosses steps through the stencil; the
    GPU adjoint equals the oracle's dual-number adjoint, which seeds the six neighbours'
    velocities as directions and carries the same velocity adjoint back."""
    cfg = _stencil_case()
    from gpu_helpers import gpu_flags
    fl = gpu_flags(cfg).cpu().numpy()
    eps_np = porosity_field(cfg, fl, seed=5)
    eps = torch.as_tensor(eps_np).reshape(cfg.nz, cfg.ny, cfg.nx)
    T = 14
    run = OutflowAdjoint(cfg, steps=T, checkpoint_every=4)
    run.forward(eps, cfg.inlet_coef)
    res = run.backward()
    ge, gi = orc.outflow_gradient(cfg, T, flags=fl, eps=eps_np.reshape(cfg.nz, cfg.ny, cfg.nx))
    gin = res.grad_inlet.cpu().numpy()
    assert np.abs(gin - gi).max() <= 1e-7 * np.abs(gi).max()
    g_gpu = res.grad_porosity.cpu().numpy()
    assert np.abs(g_gpu - ge).max() <= 1e-7 * np.abs(ge).max()
    # checkpoint spacing does not change the result
    one = OutflowAdjoint(cfg, steps=T, checkpoint_every=T)
    one.forward(eps, cfg.inlet_coef)
    r1 = one.backward()
    assert torch.equal(r1.grad_inlet, res.grad_inlet) and torch.equal(r1.grad_porosity, res.grad_porosity)


def test_stencil_adjoint_finite_differences(cuda):
    cfg = _stencil_case().replace(nx=20, ny=20, nz=20, cone_apex_z=3.0, inlet_radius=5.0)
    from gpu_helpers import gpu_flags
    fl = gpu_flags(cfg).cpu().numpy()
    eps = torch.as_tensor(porosity_field(cfg, fl, seed=25)).reshape(cfg.nz, cfg.ny, cfg.nx)
    run = OutflowAdjoint(cfg, steps=40, checkpoint_every=10)
    run.forward(eps, cfg.inlet_coef)
    res = run.backward()
    h = 1e-3
    coef = np.array(cfg.inlet_coef, np.float64)
    for k in (0, 1, 5, 15):
        cp = coef.copy(); cp[k] += h
        cm = coef.copy(); cm[k] -= h
        fd = (run.loss(eps, cp) - run.loss(eps, cm)) / (2 * h)
        ad = res.grad_inlet[k].item()
        assert abs(ad - fd) <= 1e-4 * abs(fd) + 1e-14, (k, ad, fd)
    ge = res.grad_porosity.cpu().numpy().reshape(-1)
    band = np.flatnonzero((fl.reshape(-1) & CELL_POROUS) != 0)
    flat = eps.reshape(-1)
    for c in band[np.argsort(-np.abs(ge[band]))[:6]]:
        ep = flat.clone(); ep[c] += h
        em = flat.clone(); em[c] -= h
        hh = (ep[c].double() - em[c].double()).item() / 2
        fd = (run.loss(ep.reshape(eps.shape), coef) - run.loss(em.reshape(eps.shape), coef)) / (2 * hh)
        assert abs(ge[c] - fd) <= 1e-4 * abs(fd), (c, ge[c], fd)


def test_forward_from_a_given_state(cuda):
    """J over steps 6..13 from the exported state at t = 6 equals J(14) - J(6) from rest."""
    from pour_over_coffee_lbm_gb300 import _lib
    from pour_over_coffee_lbm_gb300.solver import GB300LBMSolver
    cfg = _case().replace(storage=STORE_F64, nx=16, ny=16, nz=16)
    j14 = OutflowAdjoint(cfg, steps=14, checkpoint_every=7).forward(None, cfg.inlet_coef)
    j6 = OutflowAdjoint(cfg, steps=6, checkpoint_every=3).forward(None, cfg.inlet_coef)
    s = GB300LBMSolver(cfg)
    s.run(6)
    nat = torch.empty((19, cfg.nz, cfg.ny, cfg.nx), dtype=torch.float64, device="cuda")
    _lib.check(s.lib.pog_export_natural(s._p, _lib.ptr(s._f), _lib.ptr(s._flags), s.t, _lib.ptr(nat), STORE_F64,
                                        _lib.stream_handle()))
    run = OutflowAdjoint(cfg, steps=8, checkpoint_every=4)
    j8 = run.forward(None, cfg.inlet_coef, initial=nat)
    assert abs(j8 - (j14 - j6)) <= 1e-9 * abs(j14)
    # the band next to the outlet is within reach of 8 steps (the inlet, 13 planes up, is not)
    eps = torch.full((cfg.nz, cfg.ny, cfg.nx), cfg.porosity, dtype=torch.float32, device="cuda")
    run.forward(eps, cfg.inlet_coef, initial=nat)
    r = run.backward()
    assert torch.isfinite(r.grad_porosity).all() and r.grad_porosity.abs().max() > 0


def _coupled_case():
    from pour_over_coffee_lbm_gb300.params import ParticleConfig
    cfg = _case().replace(storage=STORE_F64, nx=20, ny=20, nz=24, cone_apex_z=3.0, inlet_radius=5.0)
    # heavy enough particles for their drag to matter in a short run
    pc = ParticleConfig(count=400, density_ratio=1.5, median_diameter=0.9, seed=77)
    return cfg, pc


def test_coupled_adjoint_matches_dual_number_oracle(cuda, orc):
    """With particles: the GPU adjoint (deposits recorded per step, held fixed) equals the oracle's
    dual-number adjoint through the same deposits and its own FP64 forward states."""
    cfg, pc = _coupled_case()
    from gpu_helpers import gpu_flags
    fl = gpu_flags(cfg).cpu().numpy()
    eps_np = porosity_field(cfg, fl, seed=21)
    eps = torch.as_tensor(eps_np).reshape(cfg.nz, cfg.ny, cfg.nx)
    T = 12
    run = OutflowAdjoint(cfg, steps=T, checkpoint_every=5, particles=pc)
    J = run.forward(eps, cfg.inlet_coef, record_deposits=True)
    res = run.backward()
    deps = [d.cpu().numpy() for d in run._dep_hist]
    assert max(float(np.abs(d[0]).max()) for d in deps) > 0  # the particles deposited drag
    assert run.loss_frozen(eps, cfg.inlet_coef) == J  # the recorded forcing reproduces J bit for bit
    # oracle: forward states under the recorded deposits, then the dual-number adjoint back
    f = orc.init_equilibrium(cfg, fl, np.float64)
    states = []
    for t in range(T):
        states.append(f)
        f, _, _ = orc.step(cfg, fl, f, eps=eps_np.reshape(cfg.nz, cfg.ny, cfg.nx), pdrag=deps[t])
    lam = np.zeros_like(f)
    ge = np.zeros(cfg.ncell)
    gi = np.zeros(16)
    for t in reversed(range(T)):
        lam = orc.adjoint_step(cfg, fl, states[t], lam, eps=eps_np, grad_eps=ge, grad_inlet=gi, pdrag=deps[t])
    g_gpu = res.grad_porosity.cpu().numpy().reshape(-1)
    assert np.abs(g_gpu - ge).max() <= 1e-7 * np.abs(ge).max()
    gin = res.grad_inlet.cpu().numpy()
    assert np.abs(gin - gi).max() <= 1e-7 * np.abs(gi).max()
    # and the particles change the gradient (the deposit term is live)
    bare = OutflowAdjoint(cfg, steps=T, checkpoint_every=5)
    bare.forward(eps, cfg.inlet_coef)
    rb = bare.backward()
    assert np.abs(rb.grad_porosity.cpu().numpy().reshape(-1) - g_gpu).max() > 1e-6 * np.abs(g_gpu).max()


def test_coupled_adjoint_finite_differences(cuda):
    """Central differences (h = 1e-3) of J under the recorded particle forcing."""
    cfg, pc = _coupled_case()
    from gpu_helpers import gpu_flags
    fl = gpu_flags(cfg).cpu().numpy()
    eps = torch.as_tensor(porosity_field(cfg, fl, seed=23)).reshape(cfg.nz, cfg.ny, cfg.nx)
    run = OutflowAdjoint(cfg, steps=40, checkpoint_every=10, particles=pc)
    run.forward(eps, cfg.inlet_coef, record_deposits=True)
    res = run.backward()
    h = 1e-3
    coef = np.array(cfg.inlet_coef, np.float64)
    for k in (0, 2, 7):
        cp = coef.copy(); cp[k] += h
        cm = coef.copy(); cm[k] -= h
        fd = (run.loss_frozen(eps, cp) - run.loss_frozen(eps, cm)) / (2 * h)
        ad = res.grad_inlet[k].item()
        assert abs(ad - fd) <= 1e-4 * abs(fd) + 1e-14, (k, ad, fd)
    ge = res.grad_porosity.cpu().numpy().reshape(-1)
    band = np.flatnonzero((fl.reshape(-1) & CELL_POROUS) != 0)
    flat = eps.reshape(-1)
    for c in band[np.argsort(-np.abs(ge[band]))[:6]]:
        ep = flat.clone(); ep[c] += h
        em = flat.clone(); em[c] -= h
        hh = (ep[c].double() - em[c].double()).item() / 2
        fd = (run.loss_frozen(ep.reshape(eps.shape), coef) - run.loss_frozen(em.reshape(eps.shape), coef)) / (2 * hh)
        assert abs(ge[c] - fd) <= 1e-4 * abs(fd), (c, ge[c], fd)


def test_loss_repeats_bit_for_bit(cuda):
    """J is an order-independent fixed-point sum: repeated forward runs give the same bits."""
    cfg = _case().replace(storage=STORE_F64, nx=24, ny=24, nz=24)
    run = OutflowAdjoint(cfg, steps=30, checkpoint_every=10)
    js = {run.forward(None, cfg.inlet_coef) for _ in range(3)}
    assert len(js) == 1 and next(iter(js)) != 0.0


@pytest.mark.parametrize("mode", ["plain_f32", "stencil", "coupled"])
def test_graph_replayed_segments_equal_eager(cuda, mode):
    """backward() replays full checkpoint segments as captured CUDA graphs (one capture per
    ping-pong parity, after one eager segment); the same launches on the same buffers give the
    eager pass's gradients bit for bit.  K = 5 (odd) makes the adjoint buffers alternate between
    segments, so two graphs are captured; the stencil case carries the velocity adjoint too."""
    pc = None
    if mode == "coupled":
        cfg, pc = _coupled_case()
    elif mode == "stencil":
        cfg = _stencil_case()
    else:
        cfg = _case().replace(storage=STORE_F32, nx=20, ny=20, nz=24, cone_apex_z=3.0, inlet_radius=5.0)
    from gpu_helpers import gpu_flags
    fl = gpu_flags(cfg).cpu().numpy()
    eps = torch.as_tensor(porosity_field(cfg, fl, seed=9)).reshape(cfg.nz, cfg.ny, cfg.nx)
    run = OutflowAdjoint(cfg, steps=22, checkpoint_every=5, particles=pc)
    run.forward(eps, cfg.inlet_coef)
    ra = run.backward(graphs=False)
    rb = run.backward(graphs=True)
    assert torch.equal(ra.grad_inlet, rb.grad_inlet) and torch.equal(ra.grad_porosity, rb.grad_porosity)
    assert rb.grad_porosity.abs().max() > 0


def test_inlet_gradient_with_and_without_scratch(cuda):
    """pog_adjoint_step sums the inlet plane's dJ/da_k by many blocks when given scratch (per-block
    sums added in block order) and by one block without it: the same lam_t bit for bit, the same
    gradients to FP64 rounding, and each form repeats itself bit for bit."""
    from pour_over_coffee_lbm_gb300 import _lib
    cfg = _case().replace(storage=STORE_F64, nx=40, ny=40, nz=24, cone_apex_z=3.0, inlet_radius=14.0)
    run = OutflowAdjoint(cfg, steps=4, checkpoint_every=4)
    run.forward(None, cfg.inlet_coef)
    torch.manual_seed(3)
    lam = torch.randn((19,) + run.shape, dtype=torch.float64, device="cuda")
    outs = []
    for scratch in (run._scratch, None, run._scratch, None):
        lt = torch.empty_like(lam)
        gi = torch.zeros(16, dtype=torch.float64, device="cuda")
        _lib.check(run.lib.pog_adjoint_step(run._p, _lib.ptr(run._states[2]), _lib.ptr(lam), _lib.ptr(lt),
                                            _lib.ptr(run.flags), None, None, None, None, None, _lib.ptr(scratch),
                                            None, _lib.ptr(gi), _lib.stream_handle()))
        outs.append((lt, gi))
    torch.cuda.synchronize()
    (la, ga), (lb, gb), (lc, gc), (ld, gd) = outs
    assert torch.equal(la, lb) and torch.equal(la, lc) and torch.equal(la, ld)
    assert torch.equal(ga, gc) and torch.equal(gb, gd)
    assert ga.abs().max() > 0
    assert torch.allclose(ga, gb, rtol=1e-12, atol=1e-15 * gb.abs().max().item())
