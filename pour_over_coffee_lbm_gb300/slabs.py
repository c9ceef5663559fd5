"""z-slab decomposition of the AA-pattern lattice (the reference's only multi-GPU strategy splits
the domain along z the same way: src/core/cuda_dual_gpu_lbm.py:67-76).

Slab s owns planes [z0, z1) and holds them between two ghost planes, (z1 - z0 + 2) planes in all,
ghost-below | owned | ghost-above.  The step kernel never updates the ghost planes (they fall
outside its one-plane guard), so a slab runs pog_step unchanged on its own buffer.

Only the odd AA step crosses an interface, and across the interface between slab s (below) and
s+1 (above) it touches exactly the slots of the five directions with c_z = -1 (DOWN) on the lower
side and the five with c_z = +1 (UP) on the upper side, each read and then written by the same
cell.  So one odd step needs:

  before:  ghost_below(s+1)[DOWN] <- top_owned(s)[DOWN]
           ghost_above(s)[UP]     <- bottom_owned(s+1)[UP]
  after:   top_owned(s)[DOWN]     <- ghost_below(s+1)[DOWN]   where the slot's writer is fluid
           bottom_owned(s+1)[UP]  <- ghost_above(s)[UP]       where the slot's writer is fluid

The writer of slot (x, q), q in DOWN, is the cell x - e_q on the upper slab's first plane; when it
is solid, x itself may have bounced f into that slot on its own side, so the copy-back is masked
(`writer_masks`).  The even step is local.  An interface moves five population planes each way
before and again after every odd step (320 x 320 FP16: 1.0 MB per face and direction).

`SlabLattice` runs all slabs on one GPU with device-local copies (bit-identical to the undivided
lattice: the kernel computes every cell from the same inputs).  `RankHalo` is the same protocol
between processes over torch.distributed point-to-point messages (one slab per rank).
"""
from typing import List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _lib
from .params import CELL_SOLID, LES_STENCIL, LatticeConfig, RED_COUNT
from .solver import CX, CY, CZ, _STORAGE_DTYPE

UP = [q for q in range(19) if CZ[q] == 1]     # 5, 11, 12, 15, 16
DOWN = [q for q in range(19) if CZ[q] == -1]  # 6, 13, 14, 17, 18


def slab_bounds(nz: int, nslabs: int) -> List[Tuple[int, int]]:
    """Balanced [z0, z1) per slab."""
    if not 1 <= nslabs <= nz // 2:
        raise ValueError("nslabs must be in [1, nz/2]")
    cuts = [s * nz // nslabs for s in range(nslabs + 1)]
    return [(cuts[s], cuts[s + 1]) for s in range(nslabs)]


def slab_flags(flags: np.ndarray, z0: int, z1: int) -> np.ndarray:
    """Flag words of planes z0-1 .. z1 of a [nz, ny, nx] array, out-of-domain ghost planes solid."""
    nz = flags.shape[0]
    out = np.full((z1 - z0 + 2,) + flags.shape[1:], CELL_SOLID, dtype=flags.dtype)
    lo, hi = max(z0 - 1, 0), min(z1 + 1, nz)
    out[lo - (z0 - 1): hi - (z0 - 1)] = flags[lo:hi]
    return out


def writer_masks(writer_plane_flags: np.ndarray, slots: Sequence[int]) -> np.ndarray:
    """[len(slots), ny, nx] bool: slot (x, q) of the interface plane is written by the fluid cell
    x - e_q of the neighbouring plane, whose flag words are `writer_plane_flags` [ny, nx]."""
    fluid = (writer_plane_flags & CELL_SOLID) == 0
    ny, nx = fluid.shape
    out = np.zeros((len(slots), ny, nx), dtype=bool)
    for a, q in enumerate(slots):
        # mask[j, i] = fluid[j - cy, i - cx] (False outside the plane)
        sy, sx = int(CY[q]), int(CX[q])
        dst = out[a, max(sy, 0): ny + min(sy, 0), max(sx, 0): nx + min(sx, 0)]
        dst[...] = fluid[max(-sy, 0): ny + min(-sy, 0), max(-sx, 0): nx + min(-sx, 0)]
    return out


class SlabLattice:
    """One lattice split into z-slabs on one GPU, each slab a separate distribution buffer driven
    through pog_step, with device-local halo copies around every odd step."""

    def __init__(self, cfg: LatticeConfig, nslabs: int, flags: Optional[np.ndarray] = None,
                 device: str = "cuda"):
        if cfg.les_mode == LES_STENCIL:
            raise ValueError("slab decomposition supports les_mode OFF or LOCAL (no u halo)")
        self.lib = _lib.load()
        self.cfg = cfg
        self.device = torch.device(device)
        dev = self.device
        shape = (cfg.nz, cfg.ny, cfg.nx)
        if flags is None:
            p = cfg.to_c()
            g = torch.empty(shape, dtype=torch.int32, device=dev)
            _lib.check(self.lib.pog_build_flags(p, _lib.ptr(g), _lib.stream_handle()))
            flags = g.cpu().numpy()
        flags = np.asarray(flags).astype(np.int32).reshape(shape)
        self.global_flags = flags
        self.bounds = slab_bounds(cfg.nz, nslabs)
        self.slabs = []
        for z0, z1 in self.bounds:
            sc = cfg.replace(nz=z1 - z0 + 2)
            p = sc.to_c()
            _lib.check(self.lib.pog_validate_params(p))
            fl = torch.as_tensor(slab_flags(flags, z0, z1)).to(dev)
            f = torch.empty((19, z1 - z0 + 2, cfg.ny, cfg.nx), dtype=_STORAGE_DTYPE[cfg.storage], device=dev)
            self.slabs.append({"z0": z0, "z1": z1, "cfg": sc, "p": p, "flags": fl, "f": f,
                               "rho": torch.zeros((z1 - z0 + 2, cfg.ny, cfg.nx), dtype=torch.float32, device=dev),
                               "u": torch.zeros((3, z1 - z0 + 2, cfg.ny, cfg.nx), dtype=torch.float32, device=dev)})
        # copy-back masks per interface: DOWN slots of the lower slab's top plane are written by
        # the upper slab's first plane, UP slots of the upper slab's first plane by the lower top
        self.masks = []
        for s in range(nslabs - 1):
            lo, up = self.slabs[s], self.slabs[s + 1]
            m_down = writer_masks(flags[up["z0"]], DOWN)
            m_up = writer_masks(flags[lo["z1"] - 1], UP)
            self.masks.append((torch.as_tensor(m_down).to(dev), torch.as_tensor(m_up).to(dev)))
        self.down = torch.as_tensor(DOWN, device=dev)
        self.up = torch.as_tensor(UP, device=dev)
        self.red = torch.zeros(RED_COUNT, dtype=torch.float64, device=dev)
        self.t = 0
        self._in_done = False
        self.init_equilibrium(cfg.rho0)

    def _s(self):
        return _lib.stream_handle()

    def init_equilibrium(self, rho0: float, u0=(0.0, 0.0, 0.0)):
        for sl in self.slabs:
            _lib.check(self.lib.pog_init_equilibrium(sl["p"], _lib.ptr(sl["f"]), _lib.ptr(sl["flags"]),
                                                     float(rho0), float(u0[0]), float(u0[1]), float(u0[2]),
                                                     self._s()))
        self.t = 0
        self._in_done = False

    # ---- halo protocol ----------------------------------------------------------------------
    def exchange_in(self):
        """Before an odd step: fill the ghost slots the boundary cells will read."""
        for s in range(len(self.slabs) - 1):
            lo, up = self.slabs[s], self.slabs[s + 1]
            top = lo["z1"] - lo["z0"]  # local index of the lower slab's top owned plane
            up["f"][self.down, 0] = lo["f"][self.down, top]
            lo["f"][self.up, top + 1] = up["f"][self.up, 1]
        self._in_done = True

    def exchange_out(self):
        """After an odd step: return the ghost slots written by fluid boundary cells."""
        for s in range(len(self.slabs) - 1):
            lo, up = self.slabs[s], self.slabs[s + 1]
            top = lo["z1"] - lo["z0"]
            m_down, m_up = self.masks[s]
            lo["f"][self.down, top] = torch.where(m_down, up["f"][self.down, 0], lo["f"][self.down, top])
            up["f"][self.up, 1] = torch.where(m_up, lo["f"][self.up, top + 1], up["f"][self.up, 1])
        self._in_done = False

    # ---- stepping ------------------------------------------------------------------------
    def run(self, nsteps: int, reduce: bool = False, want_macro: bool = False):
        if reduce:
            self.red.zero_()
        for i in range(nsteps):
            odd = self.t & 1
            if odd and not self._in_done:
                self.exchange_in()
            last = i == nsteps - 1
            for sl in self.slabs:
                _lib.check(self.lib.pog_step(
                    sl["p"], _lib.ptr(sl["f"]), _lib.ptr(sl["flags"]), self.t, 1, None, None, None, None, None,
                    _lib.ptr(sl["rho"]) if (want_macro and last) else None,
                    _lib.ptr(sl["u"]) if (want_macro and last) else None,
                    _lib.ptr(self.red) if reduce else None, self._s()))
            if odd:
                self.exchange_out()
            self.t += 1
        return self.red if reduce else None

    def natural(self, dtype=torch.float64) -> torch.Tensor:
        """The assembled natural-layout state [19, nz, ny, nx] (exporting an odd-parity state reads
        the ghost slots, so they are filled first)."""
        if self.t & 1 and not self._in_done:
            self.exchange_in()
        out_store = 3 if dtype == torch.float64 else 0
        cfg = self.cfg
        out = torch.empty((19, cfg.nz, cfg.ny, cfg.nx), dtype=dtype, device=self.device)
        for sl in self.slabs:
            nat = torch.empty((19,) + tuple(sl["f"].shape[1:]), dtype=dtype, device=self.device)
            _lib.check(self.lib.pog_export_natural(sl["p"], _lib.ptr(sl["f"]), _lib.ptr(sl["flags"]), self.t,
                                                   _lib.ptr(nat), out_store, self._s()))
            out[:, sl["z0"]: sl["z1"]] = nat[:, 1:-1]
        return out

    def macroscopic(self) -> Tuple[torch.Tensor, torch.Tensor]:
        """rho [nz, ny, nx] and u [3, nz, ny, nx] written by the last want_macro step."""
        rho = torch.cat([sl["rho"][1:-1] for sl in self.slabs], dim=0)
        u = torch.cat([sl["u"][:, 1:-1] for sl in self.slabs], dim=1)
        return rho, u


class RankHalo:
    """The same halo protocol between processes: this rank holds slab `rank` of `world` as a
    [19, nz_s + 2, ny, nx] tensor f (its flags as [nz_s + 2, ny, nx]) and trades boundary slots
    with its neighbours by torch.distributed send/recv (gloo on CPU tensors, NCCL on CUDA)."""

    def __init__(self, flags_slab: np.ndarray, rank: int, world: int):
        import torch.distributed as dist
        self.dist = dist
        self.rank, self.world = rank, world
        fl = np.asarray(flags_slab)
        n = fl.shape[0]
        self.top = n - 2  # local index of the top owned plane
        # masks for the planes this rank receives back: its top plane's DOWN slots (written by
        # the upper neighbour's first plane = this rank's top ghost) and its first plane's UP
        # slots (written by the lower neighbour's top plane = this rank's bottom ghost)
        self.m_down = torch.as_tensor(writer_masks(fl[n - 1], DOWN))
        self.m_up = torch.as_tensor(writer_masks(fl[0], UP))

    def _trade(self, send_to, send_buf, recv_from, recv_buf):
        ops = []
        if send_to is not None:
            ops.append(self.dist.P2POp(self.dist.isend, send_buf.contiguous(), send_to))
        if recv_from is not None:
            ops.append(self.dist.P2POp(self.dist.irecv, recv_buf, recv_from))
        if ops:
            for r in self.dist.batch_isend_irecv(ops):
                r.wait()

    def reduce_sums(self, t: torch.Tensor) -> torch.Tensor:
        """Sum a per-rank tensor over all ranks, in place (all-reduce).  For the step's FP64 sums
        (POG_RED_*: each rank's pog_step sums only its owned planes, the ghost planes lying
        outside the step's guard range), the adjoint's inlet-coefficient gradients and, exactly,
        the integer words of the fixed-point outflow loss.  The per-cell porosity gradient is
        owned by slab and needs no reduction."""
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return t

    def exchange_in(self, f: torch.Tensor):
        below = self.rank - 1 if self.rank > 0 else None
        above = self.rank + 1 if self.rank < self.world - 1 else None
        # my top plane's DOWN slots go up into the upper neighbour's bottom ghost
        buf = torch.empty_like(f[DOWN, 0])
        self._trade(above, f[DOWN, self.top], below, buf)
        if below is not None:
            f[DOWN, 0] = buf
        # my first plane's UP slots go down into the lower neighbour's top ghost
        buf = torch.empty_like(f[UP, 0])
        self._trade(below, f[UP, 1], above, buf)
        if above is not None:
            f[UP, self.top + 1] = buf

    def exchange_out(self, f: torch.Tensor):
        below = self.rank - 1 if self.rank > 0 else None
        above = self.rank + 1 if self.rank < self.world - 1 else None
        # my bottom ghost's DOWN slots return to the lower neighbour's top plane
        buf = torch.empty_like(f[DOWN, 0])
        self._trade(below, f[DOWN, 0], above, buf)
        if above is not None:
            f[DOWN, self.top] = torch.where(self.m_down, buf, f[DOWN, self.top])
        # my top ghost's UP slots return to the upper neighbour's first plane
        buf = torch.empty_like(f[UP, 0])
        self._trade(above, f[UP, self.top + 1], below, buf)
        if below is not None:
            f[UP, 1] = torch.where(self.m_up, buf, f[UP, 1])


def owner_plane(z: torch.Tensor, nz: int) -> torch.Tensor:
    """The cell plane a particle at height z gathers from: int(clamp(z, 0, nz - 2))
    (coffee_particles.py:1162-1164), the plane that decides which slab owns it."""
    return torch.clamp(z, 0.0, float(nz - 2)).to(torch.int64)


class RankParticles:
    """Particles owned by z-slab, one slab per rank, coupled to a RankHalo lattice.

    A particle belongs to the rank whose planes [z0, z1) contain its cell plane
    k = int(clamp(z, 0, nz - 2)); its trilinear corners are planes k and k + 1, so the coupling
    pass of the rank reads planes z0 .. z1 and writes its deposit there.  Around each pass:

      exchange_u      before it: the velocity of the first owned plane goes down into the lower
                      neighbour's top ghost plane (particles in plane z1 - 1 gather from z1);
      reduce_deposit  after it: the deposit in the top ghost plane goes up and is added to the
                      upper neighbour's first owned plane (the spread's reduce-add);
      migrate         particles whose cell plane left [z0, z1) move to the neighbour that owns it
                      (one plane per step at most: the lattice velocity is far below one cell per
                      step).

    Slab tensors have the RankHalo layout [..., z1 - z0 + 2, ny, nx] (ghost below | owned | ghost
    above).  With the fixed-point (int64) deposit of deterministic mode the reduce-add is exact,
    so a decomposed coupled run repeats the undivided one bit for bit."""

    FIELDS = ("pos", "vel", "diam", "drag_old", "active", "ident")

    def __init__(self, rank: int, world: int, z0: int, z1: int, nz: int):
        import torch.distributed as dist
        self.dist = dist
        self.rank, self.world = rank, world
        self.z0, self.z1, self.nz = z0, z1, nz
        self.below = rank - 1 if rank > 0 else None
        self.above = rank + 1 if rank < world - 1 else None

    def _trade(self, send_to, send_buf, recv_from, recv_buf):
        ops = []
        if send_to is not None:
            ops.append(self.dist.P2POp(self.dist.isend, send_buf.contiguous(), send_to))
        if recv_from is not None:
            ops.append(self.dist.P2POp(self.dist.irecv, recv_buf, recv_from))
        if ops:
            for r in self.dist.batch_isend_irecv(ops):
                r.wait()

    def exchange_u(self, u: torch.Tensor) -> None:
        """u [3, nzs + 2, ny, nx]: fill the top ghost plane from the upper neighbour."""
        top = u.shape[1] - 1
        buf = torch.empty_like(u[:, 0])
        self._trade(self.below, u[:, 1], self.above, buf)
        if self.above is not None:
            u[:, top] = buf

    def reduce_deposit(self, dep: torch.Tensor) -> None:
        """dep [4, nzs + 2, ny, nx]: send the top ghost plane up, add the lower neighbour's into
        the first owned plane, and clear the ghost planes."""
        top = dep.shape[1] - 1
        buf = torch.empty_like(dep[:, 0])
        self._trade(self.above, dep[:, top], self.below, buf)
        if self.below is not None:
            dep[:, 1] += buf
        dep[:, 0] = 0
        dep[:, top] = 0

    def migrate(self, parts: dict) -> dict:
        """parts: the FIELDS as tensors over this rank's particles (pos/vel/drag_old [3, m], the
        rest [m]).  Returns the particles this rank owns after the move, its own first (in their
        order), then those received from below, then from above."""
        k = owner_plane(parts["pos"][2], self.nz)
        down = k < self.z0
        up = k >= self.z1
        keep = ~(down | up)
        if (down.any() and self.below is None) or (up.any() and self.above is None):
            raise RuntimeError("a particle left the domain's slabs")

        def pick(mask):
            return {f: (v[:, mask] if v.dim() == 2 else v[mask]) for f, v in parts.items()}

        dev = parts["pos"].device

        def exchange(to, mask, frm):
            # counts first, then one message per field
            n_out = torch.tensor([int(mask.sum())], dtype=torch.int64, device=dev)
            n_in = torch.zeros(1, dtype=torch.int64, device=dev)
            self._trade(to, n_out, frm, n_in)
            out = pick(mask)
            got = {}
            for f, v in parts.items():
                shape = (v.shape[0], int(n_in)) if v.dim() == 2 else (int(n_in),)
                buf = torch.empty(shape, dtype=v.dtype, device=dev)
                self._trade(to, out[f], frm, buf)
                got[f] = buf
            return got

        # downward moves first (every rank sends down / receives from above), then upward
        from_above = exchange(self.below, down, self.above)
        from_below = exchange(self.above, up, self.below)
        mine = pick(keep)
        res = {}
        for f in parts:
            parts_f = [mine[f]]
            if self.below is not None:
                parts_f.append(from_below[f])
            if self.above is not None:
                parts_f.append(from_above[f])
            res[f] = torch.cat(parts_f, dim=-1)
        return res
