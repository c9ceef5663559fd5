"""The oracle's adjoint (forward-mode dual numbers through its restated step) against central finite
differences of its own FP64 forward, on the CPU.  The GPU adjoint is checked against this oracle in
tests/test_gpu_adjoint.py, so this closes the chain adjoint -> oracle -> finite differences.

Case: LES stencil mode (les_turbulence.py:318-380), where step t's viscosity reads the velocity
step t-1 output, so the adjoint carries dJ/du across steps; h = 1e-4 on the inlet coefficients
(bar 1e-5 relative) and h = 1e-3 on float32 porosities (bar 1e-4 relative).  The cross-step term
is live: dropping it moves the gradient by far more than the bar."""
import os
import sys

import numpy as np

from pour_over_coffee_lbm_gb300.params import CELL_POROUS, LES_STENCIL, STORE_F64, porosity_field

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))


def test_stencil_adjoint_oracle_vs_finite_differences(orc):
    import make_golden as mg
    cfg = mg.adjoint_case().replace(storage=STORE_F64, les_mode=LES_STENCIL, cs_smag=0.4)
    fl = orc.build_flags(cfg)
    eps = porosity_field(cfg, fl, seed=5).reshape(cfg.nz, cfg.ny, cfg.nx)
    T = 14
    ge, gi = orc.outflow_gradient(cfg, T, flags=fl, eps=eps)
    h = 1e-4
    coef = np.array(cfg.inlet_coef)
    for k in (0, 1, 3):
        cp = coef.copy(); cp[k] += h
        cm = coef.copy(); cm[k] -= h
        fd = (orc.outflow_loss(cfg.replace(inlet_coef=tuple(cp)), T, flags=fl, eps=eps)
              - orc.outflow_loss(cfg.replace(inlet_coef=tuple(cm)), T, flags=fl, eps=eps)) / (2 * h)
        assert abs(gi[k] - fd) <= 1e-5 * abs(fd), (k, gi[k], fd)
    g = ge.reshape(-1)
    band = np.flatnonzero((fl.reshape(-1) & CELL_POROUS) != 0)
    for c in band[np.argsort(-np.abs(g[band]))[:3]]:
        ep = eps.reshape(-1).copy(); ep[c] += np.float32(1e-3)
        em = eps.reshape(-1).copy(); em[c] -= np.float32(1e-3)
        hh = (np.float64(ep[c]) - np.float64(em[c])) / 2
        fd = (orc.outflow_loss(cfg, T, flags=fl, eps=ep.reshape(eps.shape))
              - orc.outflow_loss(cfg, T, flags=fl, eps=em.reshape(eps.shape))) / (2 * hh)
        assert abs(g[c] - fd) <= 1e-4 * abs(fd), (c, g[c], fd)
    # without the velocity adjoint the gradient is off by far more than the bars
    f = orc.init_equilibrium(cfg, fl, np.float64)
    u = np.zeros((3, cfg.nz, cfg.ny, cfg.nx))
    states, ups = [], []
    for _ in range(T):
        states.append(f)
        ups.append(u)
        f, _, u = orc.step(cfg, fl, f, eps=eps, u_prev=u)
    lam = np.zeros_like(f)
    gi0 = np.zeros(16)
    for t in reversed(range(T)):
        lam = orc.adjoint_step(cfg, fl, states[t], lam, eps=eps, grad_inlet=gi0, u_prev=ups[t])
    assert np.abs(gi0 - gi).max() > 100 * 1e-5 * np.abs(gi).max()
