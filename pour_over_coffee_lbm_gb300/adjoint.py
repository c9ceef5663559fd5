"""Gradients of the time-integrated outflow mass flux with respect to the per-cell porosity of
the filter band and the 16 radial inlet-profile coefficients.

Forward: T natural-layout push steps (pog_step_push) from equilibrium, J = sum_t outflow_t
(pog_outflow_fixed: an order-independent fixed-point sum, so J repeats bit for bit), with the
state checkpointed every K steps.  Backward: for each
segment, last first, the K states are recomputed from the checkpoint and the hand-written
adjoint kernel (pog_adjoint_step) runs back through them; parameter gradients accumulate in
FP64.  Memory: T/K checkpoints + K states.  `OutflowLoss` exposes this as a
torch.autograd.Function of (porosity, inlet_coef).

The reference has no differentiable path (no Taichi autodiff on it); this is new work.
"""
import dataclasses
from typing import Optional

import numpy as np
import torch

from . import _lib
from .params import INLET_NCOEF, LES_STENCIL, STORE_F32, STORE_F64, LatticeConfig

_DT = {STORE_F32: torch.float32, STORE_F64: torch.float64}


@dataclasses.dataclass
class AdjointResult:
    loss: float
    grad_porosity: Optional[torch.Tensor]  # float64 [NZ, NY, NX]
    grad_inlet: torch.Tensor  # float64 [16]


class OutflowAdjoint:
    """J and its gradients for a lattice run of `steps` steps, checkpointed every
    `checkpoint_every` steps.

    particles (ParticleConfig, optional): the run is two-way coupled as
    GB300LBMSolver.step_with_two_way_coupling (legacy/lbm_solver.py:1485-1509): before step t a
    coupling pass moves the particles in the velocity the previous step computed (zero before the
    first step) and deposits their drag (Kp, Kv), which step t reads.  The deposit is recorded per
    step (deterministic fixed-point mode) and enters the adjoint as a fixed input of its step: the
    gradient is that of J with the particles' forcing held at its recorded history.  `loss_frozen`
    evaluates J under that same recorded forcing, which is what finite differences of these
    gradients compare against."""

    def __init__(self, cfg: LatticeConfig, steps: int, checkpoint_every: int, device="cuda", particles=None):
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
        # J in two-word fixed point (units of 2^-48 and 2^-96): the exact sum, the same bits on every run
        self._jfix = torch.zeros(2, dtype=torch.int64, device=self.device)
        self._p = None
        self._eps = None
        self.pc = particles
        self.stencil = cfg.les_mode == LES_STENCIL
        # the velocity each step outputs feeds the next step's LES stencil and the particles'
        # coupling pass: kept as a ping-pong (read / written), checkpointed with the state
        self._need_u = self.stencil or particles is not None
        if self._need_u:
            self._u = torch.zeros((3,) + shape, dtype=torch.float32, device=self.device)
            self._un = torch.zeros_like(self._u)
            self._uck = [torch.zeros_like(self._u) for _ in range(self.nseg)]
        if self.stencil:
            self._ups = [torch.zeros_like(self._u) for _ in range(self.K)]  # the segment's u_prev
        # the stencil mode's per-cell terms and the inlet plane's per-block gradient sums
        self._scratch = torch.empty(int(self.lib.pog_adjoint_scratch_bytes(cfg.to_c())), dtype=torch.uint8,
                                    device=self.device)
        if particles is not None:
            self._init_particles(particles)

    # ---- particles -----------------------------------------------------------------------------
    def _init_particles(self, pc):
        from .params import seed_particles
        if pc.count <= 0:
            raise ValueError("a coupled adjoint needs particles")
        pc = dataclasses.replace(pc, deterministic=True)  # the recomputed deposits repeat bit for bit
        self.pc = pc
        self._pp = pc.to_c()
        pos, vel, d, act = seed_particles(self.cfg, pc)
        dev = self.device
        self._p0 = [torch.as_tensor(a).to(dev) for a in (pos, vel, np.zeros_like(pos), act)]
        self._d = torch.as_tensor(d).to(dev)
        self._part = [a.clone() for a in self._p0]  # pos, vel, drag_old, active
        self._pck = [[a.clone() for a in self._p0] for _ in range(self.nseg)]
        n = self.cfg.ncell
        # the fixed-point deposit: all zeros between passes (each pass's conversion takes back
        # every entry it deposited); the base cell of each particle's deposit
        self._fix = torch.zeros(4 * n, dtype=torch.int64, device=dev)
        self._depc = torch.full((pc.count,), -1, dtype=torch.int32, device=dev)
        self._pp.deposit_cells = self._depc.data_ptr()
        self._deps = [torch.zeros((4,) + self.shape, dtype=torch.float32, device=dev) for _ in range(self.K)]
        self._dep_hist = None  # all T deposits of the last forward (for loss_frozen), on request

    def _couple(self, u, out):
        """One coupling pass on the current particle state in velocity u; deposit into out."""
        pos, vel, drag, act = self._part
        out.zero_()
        _lib.check(self.lib.pog_particles_couple(self._p, self._pp, _lib.ptr(pos), _lib.ptr(vel), _lib.ptr(self._d),
                                                 _lib.ptr(drag), _lib.ptr(act), int(self.pc.count), None,
                                                 _lib.ptr(u), None, _lib.ptr(self._fix), None, _lib.stream_handle()))
        _lib.check(self.lib.pog_drag_from_fixed_cells(self._p, _lib.ptr(self._fix), _lib.ptr(self._depc),
                                                      int(self.pc.count), None, _lib.ptr(out), _lib.stream_handle()))

    # ---- steps ---------------------------------------------------------------------------------
    def _params(self, coef):
        c = self.cfg.replace(inlet_coef=tuple(float(x) for x in coef))
        return c.to_c()

    def _push(self, fin, fout, pdrag=None):
        """One step fin -> fout; with a velocity history it reads self._u (LES stencil) and writes
        the step's velocity into self._un, then swaps the two."""
        _lib.check(self.lib.pog_step_push(self._p, _lib.ptr(fin), _lib.ptr(fout), _lib.ptr(self.flags),
                                          None, _lib.ptr(pdrag), _lib.ptr(self._eps),
                                          _lib.ptr(self._u) if self.stencil else None, None,
                                          _lib.ptr(self._un) if self._need_u else None,
                                          None, _lib.stream_handle()))
        if self._need_u:
            self._u, self._un = self._un, self._u

    def _start(self, porosity, inlet_coef, initial):
        self._p = self._params(inlet_coef)
        self._eps = None if porosity is None else porosity.to(self.device, torch.float32).contiguous().reshape(self.shape)
        s = _lib.stream_handle()
        cur = self._states[0]
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
        self._jfix.zero_()
        return cur

    def forward(self, porosity: Optional[torch.Tensor], inlet_coef, initial: Optional[torch.Tensor] = None,
                record_deposits: bool = False) -> float:
        """Run the forward pass, keep checkpoints, return J.  initial: plain distributions f_q in
        natural layout [19, NZ, NY, NX], float32 or float64 on the device (pog_export_natural's
        output), the T steps start from (default: equilibrium at rest).  With particles,
        record_deposits keeps all T deposits for loss_frozen."""
        cur = self._start(porosity, inlet_coef, initial)
        s = _lib.stream_handle()
        nxt = self._states[1] if self.K > 1 else torch.empty_like(cur)
        if self._need_u:
            self._u.zero_()  # the velocity before the first step (the solver starts at rest)
        if self.pc is not None:
            for a, b in zip(self._part, self._p0):
                a.copy_(b)
            if record_deposits:
                self._dep_hist = [torch.empty((4,) + self.shape, dtype=torch.float32, device=self.device)
                                  for _ in range(self.T)]
        dep = self._deps[0] if self.pc is not None else None
        for t in range(self.T):
            if t % self.K == 0:
                seg = t // self.K
                self._ckpt[seg].copy_(cur)
                if self._need_u:
                    self._uck[seg].copy_(self._u)
                if self.pc is not None:
                    for a, b in zip(self._pck[seg], self._part):
                        a.copy_(b)
            _lib.check(self.lib.pog_outflow_fixed(self._p, _lib.ptr(cur), _lib.ptr(self.flags), _lib.ptr(self._jfix), s))
            if self.pc is not None:
                self._couple(self._u, dep)
                if record_deposits:
                    self._dep_hist[t].copy_(dep)
            self._push(cur, nxt, dep)
            cur, nxt = nxt, cur
        return self._loss()

    def loss_frozen(self, porosity: Optional[torch.Tensor], inlet_coef) -> float:
        """J with the particles' deposits held at those recorded by the last
        forward(..., record_deposits=True): the function the coupled adjoint differentiates."""
        if self.pc is None or self._dep_hist is None:
            raise RuntimeError("loss_frozen needs a forward(..., record_deposits=True) with particles")
        cur = self._start(porosity, inlet_coef, None)
        s = _lib.stream_handle()
        nxt = self._states[1] if self.K > 1 else torch.empty_like(cur)
        self._u.zero_()
        for t in range(self.T):
            _lib.check(self.lib.pog_outflow_fixed(self._p, _lib.ptr(cur), _lib.ptr(self.flags), _lib.ptr(self._jfix), s))
            self._push(cur, nxt, self._dep_hist[t])
            cur, nxt = nxt, cur
        return self._loss()

    def _loss(self) -> float:
        hi, lo = (int(v) for v in self._jfix.tolist())
        return float(hi) * 2.0 ** -48 + float(lo) * 2.0 ** -96

    def _segment(self, n, lam_next, lam_t, mu, mu_prev, g_eps, g_in):
        """Recompute n states from self._states[0] (and the velocity / particles restored beside
        it), then run the adjoint back through them.  Returns the ping-pong buffers as they stand
        after the n adjoint steps."""
        s = _lib.stream_handle()
        for i in range(n):
            if self.stencil:
                self._ups[i].copy_(self._u)
            if self.pc is not None:
                self._couple(self._u, self._deps[i])
            if i + 1 < n:
                self._push(self._states[i], self._states[i + 1], self._deps[i] if self.pc is not None else None)
        for i in reversed(range(n)):
            dep = self._deps[i] if self.pc is not None else None
            _lib.check(self.lib.pog_adjoint_step(
                self._p, _lib.ptr(self._states[i]), _lib.ptr(lam_next), _lib.ptr(lam_t),
                _lib.ptr(self.flags), _lib.ptr(self._eps), _lib.ptr(dep),
                _lib.ptr(self._ups[i]) if self.stencil else None, _lib.ptr(mu), _lib.ptr(mu_prev),
                _lib.ptr(self._scratch), _lib.ptr(g_eps), _lib.ptr(g_in), s))
            lam_next, lam_t = lam_t, lam_next
            if self.stencil:
                mu, mu_prev = mu_prev, mu
        return lam_next, lam_t, mu, mu_prev

    def backward(self, want_porosity_grad: bool = True, graphs: bool = True) -> AdjointResult:
        """Segments last first.  With `graphs`, a full segment (K steps) is captured into a CUDA
        graph once per backward pass (after one segment has run eagerly) and replayed for the
        others: the same launches on the same buffers, so the gradients are bit-identical to the
        eager pass; the segment's restore copies stay outside the graph."""
        lam_next = torch.zeros((19,) + self.shape, dtype=self.dtype, device=self.device)
        lam_t = torch.zeros_like(lam_next)
        g_eps = torch.zeros(self.shape, dtype=torch.float64, device=self.device) \
            if (want_porosity_grad and self._eps is not None) else None
        g_in = torch.zeros(INLET_NCOEF, dtype=torch.float64, device=self.device)
        # dJ/du of the velocity a step outputs (LES stencil: read by the next step), ping-pong
        mu = mu_prev = None
        if self.stencil:
            mu = torch.zeros((3,) + self.shape, dtype=self.dtype, device=self.device)
            mu_prev = torch.zeros_like(mu)
        u_pair = (self._u, self._un) if self._need_u else None
        captured = {}  # (lam_next, mu) buffer identity at segment start -> (graph, buffers after it)
        warm = False
        for seg in reversed(range(self.nseg)):
            t0 = seg * self.K
            n = min(self.T, t0 + self.K) - t0
            if u_pair is not None:  # the same velocity buffers at every segment start
                self._u, self._un = u_pair
            self._states[0].copy_(self._ckpt[seg])
            # recompute the segment: the same states, velocities and deposits as the forward pass
            if self._need_u:
                self._u.copy_(self._uck[seg])
            if self.pc is not None:
                for a, b in zip(self._part, self._pck[seg]):
                    a.copy_(b)
            key = (lam_next.data_ptr(), mu.data_ptr() if mu is not None else 0)
            if graphs and warm and n == self.K and key not in captured:
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g):
                    out = self._segment(n, lam_next, lam_t, mu, mu_prev, g_eps, g_in)
                captured[key] = (g, out, (self._u, self._un) if self._need_u else None)
            if key in captured and n == self.K:
                g, out, u_end = captured[key]
                g.replay()
                lam_next, lam_t, mu, mu_prev = out
                if u_end is not None:
                    self._u, self._un = u_end
            else:
                lam_next, lam_t, mu, mu_prev = self._segment(n, lam_next, lam_t, mu, mu_prev, g_eps, g_in)
                warm = True
        if u_pair is not None:
            self._u, self._un = u_pair
        return AdjointResult(self._loss(), g_eps, g_in)

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
