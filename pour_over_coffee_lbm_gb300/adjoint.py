"""Gradients of the time-integrated outflow mass flux with respect to the per-cell porosity of
the filter band and the 16 radial inlet-profile coefficients.

Forward: T natural-layout push steps (pog_step_push) from equilibrium, J = sum_t outflow_t
(FP64 device reduction), with the state checkpointed every K steps.  Backward: for each
segment, last first, the K states are recomputed from the checkpoint and the hand-written
adjoint kernel (pog_adjoint_step) runs back through them; parameter gradients accumulate in
FP64.  Memory: T/K checkpoints + K states.  `OutflowLoss` exposes this as a
torch.autograd.Function of (porosity, inlet_coef).

The reference has no differentiable path (no Taichi autodiff on it); this is new work.
"""
import dataclasses
from typing import Optional

import torch

from . import _lib
from .params import (INLET_NCOEF, RED_COUNT, RED_OUTFLOW, STORE_F32, STORE_F64,
                     LatticeConfig)

_DT = {STORE_F32: torch.float32, STORE_F64: torch.float64}


@dataclasses.dataclass
class AdjointResult:
    loss: float
    grad_porosity: Optional[torch.Tensor]  # float64 [NZ, NY, NX]
    grad_inlet: torch.Tensor  # float64 [16]


class OutflowAdjoint:
    def __init__(self, cfg: LatticeConfig, steps: int, checkpoint_every: int, device="cuda"):
        if cfg.storage not in _DT:
            raise ValueError("the adjoint runs on FP32 or FP64 storage")
        self.lib = _lib.load()
        self.cfg = cfg
        self.T = int(steps)
        self.K = int(checkpoint_every)
        if self.T <= 0 or self.K <= 0:
            raise ValueError("steps and checkpoint_every must be positive")
        self.device = torch.device(device)
        shape = (cfg.nz, cfg.ny, cfg.nx)
        self.shape = shape
        self.flags = torch.empty(shape, dtype=torch.int32, device=self.device)
        _lib.check(self.lib.pog_build_flags(cfg.to_c(), _lib.ptr(self.flags), _lib.stream_handle()))
        self.dtype = _DT[cfg.storage]
        self.nseg = (self.T + self.K - 1) // self.K
        self._ckpt = [torch.empty((19,) + shape, dtype=self.dtype, device=self.device)
                      for _ in range(self.nseg)]
        self._states = [torch.empty((19,) + shape, dtype=self.dtype, device=self.device)
                        for _ in range(self.K)]
        self._red = torch.zeros(RED_COUNT, dtype=torch.float64, device=self.device)
        self._p = None
        self._eps = None

    def _params(self, coef):
        c = self.cfg.replace(inlet_coef=tuple(float(x) for x in coef))
        return c.to_c()

    def _push(self, fin, fout, red=None):
        _lib.check(self.lib.pog_step_push(self._p, _lib.ptr(fin), _lib.ptr(fout), _lib.ptr(self.flags),
                                          None, None, _lib.ptr(self._eps), None, None, None,
                                          _lib.ptr(red), _lib.stream_handle()))

    def forward(self, porosity: Optional[torch.Tensor], inlet_coef, initial: Optional[torch.Tensor] = None) -> float:
        """Run the forward pass, keep checkpoints, return J.  initial: plain distributions f_q in
        natural layout [19, NZ, NY, NX], float32 or float64 on the device (pog_export_natural's
        output), the T steps start from (default: equilibrium at rest)."""
        self._p = self._params(inlet_coef)
        self._eps = None if porosity is None else porosity.to(self.device, torch.float32).contiguous().reshape(self.shape)
        s = _lib.stream_handle()
        cur = self._states[0]
        nxt = self._states[1] if self.K > 1 else torch.empty_like(cur)
        if initial is None:
            _lib.check(self.lib.pog_init_equilibrium(self._p, _lib.ptr(cur), _lib.ptr(self.flags),
                                                     float(self.cfg.rho0), 0.0, 0.0, 0.0, s))
        else:
            if initial.dtype not in (torch.float32, torch.float64) or initial.numel() != cur.numel():
                raise ValueError("initial must be float32/float64 [19, NZ, NY, NX]")
            src = initial.contiguous()
            in_store = STORE_F32 if src.dtype == torch.float32 else STORE_F64
            _lib.check(self.lib.pog_import_natural(self._p, _lib.ptr(src), in_store, _lib.ptr(self.flags),
                                                   _lib.ptr(cur), s))
        self._red.zero_()
        for t in range(self.T):
            if t % self.K == 0:
                self._ckpt[t // self.K].copy_(cur)
            self._push(cur, nxt, self._red)
            cur, nxt = nxt, cur
        return float(self._red[RED_OUTFLOW])

    def backward(self, want_porosity_grad: bool = True) -> AdjointResult:
        s = _lib.stream_handle()
        lam_next = torch.zeros((19,) + self.shape, dtype=self.dtype, device=self.device)
        lam_t = torch.zeros_like(lam_next)
        g_eps = torch.zeros(self.shape, dtype=torch.float64, device=self.device) \
            if (want_porosity_grad and self._eps is not None) else None
        g_in = torch.zeros(INLET_NCOEF, dtype=torch.float64, device=self.device)
        for seg in reversed(range(self.nseg)):
            t0 = seg * self.K
            t1 = min(self.T, t0 + self.K)
            self._states[0].copy_(self._ckpt[seg])
            for i in range(t1 - t0 - 1):
                self._push(self._states[i], self._states[i + 1])
            for t in reversed(range(t0, t1)):
                _lib.check(self.lib.pog_adjoint_step(
                    self._p, _lib.ptr(self._states[t - t0]), _lib.ptr(lam_next), _lib.ptr(lam_t),
                    _lib.ptr(self.flags), _lib.ptr(self._eps), _lib.ptr(g_eps), _lib.ptr(g_in), s))
                lam_next, lam_t = lam_t, lam_next
        return AdjointResult(float(self._red[RED_OUTFLOW]), g_eps, g_in)

    def loss(self, porosity: Optional[torch.Tensor], inlet_coef) -> float:
        """Forward only (for finite differences)."""
        return self.forward(porosity, inlet_coef)


class OutflowLoss(torch.autograd.Function):
    """J(porosity, inlet_coef) = time-integrated outflow flux, with the hand-written adjoint
    as backward.  porosity: float32 [NZ, NY, NX] (only porous cells matter); inlet_coef: [16]."""

    @staticmethod
    def forward(ctx, porosity, inlet_coef, runner: OutflowAdjoint):
        coef = [float(x) for x in inlet_coef.detach().cpu().tolist()]
        J = runner.forward(porosity.detach(), coef)
        res = runner.backward(want_porosity_grad=True)
        ctx.save_for_backward(res.grad_porosity.to(porosity.dtype), res.grad_inlet.to(inlet_coef.dtype))
        ctx.dev = (porosity.device, inlet_coef.device)
        return torch.tensor(J, dtype=torch.float64, device=porosity.device)

    @staticmethod
    def backward(ctx, gJ):
        ge, gi = ctx.saved_tensors
        g = gJ.to(torch.float64)
        return (ge.to(ctx.dev[0]) * g.to(ge.device).to(ge.dtype),
                gi.to(ctx.dev[1]) * g.to(gi.device).to(gi.dtype), None)


def outflow_loss(porosity, inlet_coef, runner: OutflowAdjoint):
    return OutflowLoss.apply(porosity, inlet_coef, runner)
