"""CoffeeParticleSystem on libpog.so: Lagrangian coffee particles two-way coupled to the
GB300 lattice.

Same accessor names as src/physics/coffee_particles.py:30-64 (position, velocity, radius, mass,
active, force, drag_force, drag_force_old, drag_force_new, fluid_velocity_at_particle,
particle_reynolds, drag_coefficient, reaction_force_field, particle_count[None],
active_count[None]) and get_coupling_diagnostics() (:1214).  Units are lattice units
throughout (the reference mixes SI radius/density with lattice positions).  State is
structure-of-arrays on the device: pos[3][n], vel[3][n], diameter[n], drag_old[3][n],
active[n].
"""
import math
from typing import Optional

import numpy as np
import torch

from . import _lib
from .params import LatticeConfig, ParticleConfig, seed_particles


class _Scalar:
    """Supports the reference's `field[None]` scalar access."""

    def __init__(self, get):
        self._get = get

    def __getitem__(self, idx):
        return self._get()

    def __int__(self):
        return int(self._get())


class ParticleView:
    """(n, comps) view of an SoA [comps][n] particle tensor."""

    def __init__(self, t: torch.Tensor, n: int):
        self._t = t
        self._n = n

    @property
    def tensor(self):
        return self._t

    def to_numpy(self):
        t = self._t[..., : self._n]
        return (t.t() if t.dim() == 2 else t).contiguous().cpu().numpy()

    def from_numpy(self, arr):
        a = torch.as_tensor(np.asarray(arr)).to(self._t.device, self._t.dtype)
        if self._t.dim() == 2:
            self._t[:, : a.shape[0]].copy_(a.t())
        else:
            self._t[: a.shape[0]].copy_(a)

    def __getitem__(self, i):
        t = self._t
        v = t[:, i] if t.dim() == 2 else t[i]
        return v.cpu().numpy() if v.numel() > 1 else v.item()


class CoffeeParticleSystem:
    def __init__(self, max_particles: int = 15000, lattice: Optional[LatticeConfig] = None,
                 config: Optional[ParticleConfig] = None, device: str = "cuda"):
        if not torch.cuda.is_available():
            raise RuntimeError("CoffeeParticleSystem needs a CUDA device")
        self.lib = _lib.load()
        self.max_particles = int(max_particles)
        self.lattice = lattice if lattice is not None else LatticeConfig()
        self.pcfg = config if config is not None else ParticleConfig(count=self.max_particles)
        dev = torch.device(device)
        self.device = dev
        n = self.max_particles
        self._pos = torch.zeros((3, n), dtype=torch.float32, device=dev)
        self._vel = torch.zeros((3, n), dtype=torch.float32, device=dev)
        self._d = torch.zeros(n, dtype=torch.float32, device=dev)
        self._drag_old = torch.zeros((3, n), dtype=torch.float32, device=dev)
        self._active = torch.zeros(n, dtype=torch.int32, device=dev)
        self._u_at = torch.zeros((3, n), dtype=torch.float32, device=dev)
        self._keys = torch.zeros(n, dtype=torch.int32, device=dev)
        self._perm = torch.arange(n, dtype=torch.int32, device=dev)
        self._scratch = torch.empty(int(self.lib.pog_particles_bin_scratch_bytes(n)), dtype=torch.uint8, device=dev)
        self._fix = None
        # base cell of each particle's last drag deposit (-1: none), for the sparse clear
        self._dep = torch.full((n,), -1, dtype=torch.int32, device=dev)
        self._dep_n = 0
        self._dep_valid = False
        self._pp = None
        self._pp_key = None
        self.count = 0
        self._since_sort = None
        self._solver = None

    # ---- seeding ---------------------------------------------------------------------------
    def seed(self, lattice: Optional[LatticeConfig] = None, config: Optional[ParticleConfig] = None):
        """Seeded particles uniform in the lower cone, log-normal diameters."""
        lc = lattice or self.lattice
        pc = config or self.pcfg
        pos, vel, d, act = seed_particles(lc, pc)
        self.load_state(pos, vel, d, act)

    def load_state(self, pos, vel, diameter, active, drag_old=None):
        n = int(np.asarray(diameter).shape[0])
        if n > self.max_particles:
            raise ValueError("more particles than max_particles")
        self.count = n
        self._pos[:, :n].copy_(torch.as_tensor(np.asarray(pos, np.float32)))
        self._vel[:, :n].copy_(torch.as_tensor(np.asarray(vel, np.float32)))
        self._d[:n].copy_(torch.as_tensor(np.asarray(diameter, np.float32)))
        self._active.zero_()
        self._active[:n].copy_(torch.as_tensor(np.asarray(active, np.int32)))
        self._drag_old.zero_()
        self._dep_valid = False
        if drag_old is not None:
            self._drag_old[:, :n].copy_(torch.as_tensor(np.asarray(drag_old, np.float32)))
        self._since_sort = None

    # ---- kernels -----------------------------------------------------------------------------
    def _params(self, solver):
        return solver._p

    def bin(self, solver_or_params, sort: bool = True):
        """Cell keys of every particle and (sort=True) their stable cell order."""
        p = solver_or_params._p if hasattr(solver_or_params, "_p") else solver_or_params
        n = self.count
        s = _lib.stream_handle()
        _lib.check(self.lib.pog_particles_bin(p, _lib.ptr(self._pos), _lib.ptr(self._active), n,
                                              _lib.ptr(self._keys), _lib.ptr(self._perm) if sort else None,
                                              _lib.ptr(self._scratch) if sort else None, s))
        if sort:
            self._since_sort = 0
        return self._keys[:n], (self._perm[:n] if sort else None)

    def couple(self, solver, dt: float = 1.0, relaxation_factor: float = 0.8,
               pdrag: Optional[torch.Tensor] = None, deposit_mask: Optional[torch.Tensor] = None):
        """One coupling pass against solver's current velocity field: drag, under-relaxation,
        integration, and the drag deposit (Kp, Kv) added into `pdrag` ([4, NZ, NY, NX], not
        cleared here) for the fluid-side force Kv - Kp u of the next lattice step: the implicit
        drag by default, or with config.reaction = REACTION_EXPLICIT(_NEW) the reaction -F spread
        as an explicit body force (Kp = 0), as the reference's distribute_force_to_grid does.
        deposit_mask (int32 [ceil(ncell/32)]): the bits of the deposited cells are set."""
        n = self.count
        if n == 0:
            return
        pc = self.pcfg
        if self._since_sort is None or (pc.sort_interval > 0 and self._since_sort >= pc.sort_interval):
            self.bin(solver, sort=True)
        # the parameter block is rebuilt only when one of its inputs changes
        mptr = None if deposit_mask is None else deposit_mask.data_ptr()
        key = (pc.density_ratio, pc.drag_model, pc.deterministic, pc.wall_margin, pc.wall_pullback,
               pc.wall_damping, pc.z_floor, pc.reaction, dt, relaxation_factor, mptr)
        if self._pp_key != key:
            pp = pc.to_c()
            pp.dt = float(dt)
            pp.relaxation = float(relaxation_factor)
            pp.deposit_cells = self._dep.data_ptr()
            pp.deposit_mask = mptr
            self._pp, self._pp_key = pp, key
        pp = self._pp
        f_out = pdrag if pdrag is not None else solver._pdrag
        fix = None
        if pc.deterministic:
            # all zeros between passes: each pass's conversion takes back every entry it deposited
            if self._fix is None or self._fix.numel() != 4 * solver.n:
                self._fix = torch.zeros(4 * solver.n, dtype=torch.int64, device=self.device)
            fix = self._fix
        s = _lib.stream_handle()
        _lib.check(self.lib.pog_particles_couple(
            solver._p, pp, _lib.ptr(self._pos), _lib.ptr(self._vel), _lib.ptr(self._d),
            _lib.ptr(self._drag_old), _lib.ptr(self._active), n, _lib.ptr(self._perm),
            _lib.ptr(solver._u), None if pc.deterministic else _lib.ptr(f_out), _lib.ptr(fix),
            _lib.ptr(self._u_at), s))
        if pc.deterministic:
            _lib.check(self.lib.pog_drag_from_fixed_cells(solver._p, _lib.ptr(fix), _lib.ptr(self._dep), n,
                                                          _lib.ptr(self._perm), _lib.ptr(f_out), s))
        self._solver = solver
        self._since_sort = (self._since_sort or 0) + 1
        self._dep_n = n
        self._dep_valid = True

    def clear_deposit(self, solver, pdrag: Optional[torch.Tensor] = None,
                      deposit_mask: Optional[torch.Tensor] = None) -> None:
        """Zero the cells of the last couple() deposit in pdrag (default: the solver's) and clear
        their bits in deposit_mask (default: the solver's), so a deposit field that held only
        that deposit is all zeros again."""
        if not self._dep_valid or self._dep_n == 0:
            return
        f_out = pdrag if pdrag is not None else solver._pdrag
        mask = deposit_mask if deposit_mask is not None else getattr(solver, "_dmask", None)
        _lib.check(self.lib.pog_particles_clear_deposit(solver._p, _lib.ptr(self._dep), self._dep_n,
                                                        _lib.ptr(self._perm), _lib.ptr(f_out), _lib.ptr(mask),
                                                        _lib.stream_handle()))

    # ---- reference accessors -----------------------------------------------------------------
    @property
    def position(self):
        return ParticleView(self._pos, self.count)

    @property
    def velocity(self):
        return ParticleView(self._vel, self.count)

    @property
    def radius(self):
        return ParticleView(self._d * 0.5, self.count)

    @property
    def diameter(self):
        return ParticleView(self._d, self.count)

    @property
    def mass(self):
        rho_p = self.pcfg.density_ratio * self.lattice.rho0
        return ParticleView(rho_p * (math.pi / 6.0) * self._d ** 3, self.count)

    @property
    def active(self):
        return ParticleView(self._active, self.count)

    @property
    def drag_force(self):
        return ParticleView(self._drag_old, self.count)

    drag_force_old = drag_force
    force = drag_force

    @property
    def drag_force_new(self):
        return ParticleView(self._drag_old, self.count)

    @property
    def fluid_velocity_at_particle(self):
        return ParticleView(self._u_at, self.count)

    @property
    def reaction_force_field(self):
        """Force density on the fluid from the last coupling (coffee_particles.py:45)."""
        from .solver import FieldView
        if self._solver is None:
            raise AttributeError("no coupling step has run yet")
        return FieldView(self._solver.particle_reaction_force(), ncomp=3, readonly=True)

    @property
    def particle_count(self):
        return _Scalar(lambda: self.count)

    @property
    def active_count(self):
        return _Scalar(lambda: int(self._active[: self.count].sum()))

    def _reynolds(self):
        n = self.count
        lc = self.lattice
        mu = lc.rho0 * lc.nu0
        urel = self._u_at[:, :n] - self._vel[:, :n]
        return lc.rho0 * torch.sqrt((urel.double() ** 2).sum(0)) * self._d[:n].double() / mu

    @property
    def particle_reynolds(self):
        return ParticleView(self._reynolds().float(), self.count)

    @property
    def drag_coefficient(self):
        re = self._reynolds().clamp_min(0.01)
        return ParticleView((24.0 / re).float(), self.count)

    def get_coupling_diagnostics(self) -> dict:
        n = self.count
        if n == 0:
            return {"active_particles": 0, "avg_reynolds": 0.0, "avg_drag_coeff": 0.0,
                    "max_reaction_force": 0.0, "coupling_quality": "no_particles"}
        act = self._active[:n] != 0
        re = self._reynolds()[act]
        cd = (24.0 / re.clamp_min(0.01))
        mr = 0.0
        if self._solver is not None:
            rf = self._solver.particle_reaction_force()
            mr = float(torch.sqrt((rf.double() ** 2).sum(0)).max())
        return {"active_particles": int(act.sum()),
                "avg_reynolds": float(re.mean()) if re.numel() else 0.0,
                "max_reynolds": float(re.max()) if re.numel() else 0.0,
                "avg_drag_coeff": float(cd.mean()) if cd.numel() else 0.0,
                "max_reaction_force": mr,
                "coupling_quality": "active" if re.numel() else "inactive"}
