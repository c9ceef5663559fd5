"""GB300LBMSolver: the reference's solver object on top of libpog.so.

Drop-in for src/core/legacy/lbm_solver.py:LBMSolver (physics and attribute surface) and
src/core/lbm_unified.py:UnifiedLBMSolver (constructor/factory), satisfying
LBMSolverProtocol and ParticleCoupledLBMProtocol (src/core/lbm_protocol.py).  Device state
lives in torch CUDA tensors; every step is one fused libpog kernel launch.  There is no CPU
path: without a GPU and the library, construction raises.
"""
from typing import Any, Optional, Tuple

import numpy as np
import torch

from . import _lib
from .params import (CELL_INLET, CELL_NEAR_SOLID, CELL_OUTLET, CELL_POROUS, CELL_SOLID, STEP_AUTO, STEP_CELLS,
                     LES_LOCAL, LES_OFF, LES_STENCIL, RED_COUNT, STORE_BF16S, STORE_F16S, STORE_F32, STORE_F64,
                     LatticeConfig)

OPPOSITE = np.array([0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15], dtype=np.int32)
CX = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0], dtype=np.int32)
CY = np.array([0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1], dtype=np.int32)
CZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1], dtype=np.int32)
WEIGHTS = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12, dtype=np.float64)

_STORAGE_DTYPE = {STORE_F32: torch.float32, STORE_F16S: torch.float16,
                  STORE_BF16S: torch.bfloat16, STORE_F64: torch.float64}


class FieldView:
    """Taichi-field-like view of a device tensor stored x-fastest ([..., NZ, NY, NX]).

    Presents the reference's (NX, NY, NZ[, comps]) indexing: `to_numpy()`, `from_numpy()`,
    `fill()`, `shape`, `[i, j, k]`.  `refresh` (optional) is called before every read so
    lazily computed fields (rho, u) are current.
    """

    def __init__(self, tensor: torch.Tensor, ncomp: int = 0, refresh=None, on_write=None,
                 readonly: bool = False):
        self._t = tensor
        self._ncomp = ncomp
        self._refresh = refresh
        self._on_write = on_write
        self._readonly = readonly

    @property
    def tensor(self) -> torch.Tensor:
        if self._refresh:
            self._refresh()
        return self._t

    def _ref_view(self) -> torch.Tensor:
        t = self.tensor
        if self._ncomp:
            return t.permute(3, 2, 1, 0)  # [c, z, y, x] -> [x, y, z, c]
        return t.permute(2, 1, 0)

    @property
    def shape(self):
        nz, ny, nx = self._t.shape[-3:]
        return (nx, ny, nz, self._ncomp) if self._ncomp else (nx, ny, nz)

    @property
    def dtype(self):
        return self._t.dtype

    def to_numpy(self) -> np.ndarray:
        return self._ref_view().contiguous().cpu().numpy()

    def to_torch(self) -> torch.Tensor:
        return self._ref_view()

    def from_numpy(self, arr) -> None:
        if self._readonly:
            raise AttributeError("this field is derived; change the geometry with set_geometry()")
        a = torch.as_tensor(np.ascontiguousarray(arr)).to(self._t.device, self._t.dtype)
        if self._ncomp:
            self._t.copy_(a.permute(3, 2, 1, 0))
        else:
            self._t.copy_(a.permute(2, 1, 0))
        if self._on_write:
            self._on_write()

    def fill(self, value) -> None:
        if self._readonly:
            raise AttributeError("this field is derived")
        self._t.fill_(value)
        if self._on_write:
            self._on_write()

    def __getitem__(self, idx):
        v = self._ref_view()[idx]
        return v.item() if v.numel() == 1 else v.cpu().numpy()

    def __setitem__(self, idx, value):
        if self._readonly:
            raise AttributeError("this field is derived")
        self._ref_view()[idx] = torch.as_tensor(value, dtype=self._t.dtype)
        if self._on_write:
            self._on_write()

    def norm_max(self) -> float:
        t = self.tensor
        if self._ncomp:
            return float(torch.sqrt((t.double() ** 2).sum(0)).max())
        return float(t.abs().max())


class _FusedBoundaryManager:
    """Stand-in for BoundaryConditionManager (boundary_conditions.py:327-409): the inlet,
    outlet and bounce-back walls are applied inside the fused step, so this only keeps the
    reference's call surface."""

    def __init__(self):
        self.filter_system = None

    def set_filter_system(self, fs):
        self.filter_system = fs

    def apply_all_boundaries(self, solver):
        return None


class GB300LBMSolver:
    """D3Q19 BGK + Guo gravity + LES + porous filter band + half-way bounce-back on the V60
    mask, stepped by libpog.so on one GB300 (sm_103a)."""

    def __init__(self, config: Optional[LatticeConfig] = None, device: str = "cuda",
                 porosity: Optional[np.ndarray] = None, preferred_backend: Optional[str] = None,
                 step_kernel: str = "auto", density_reference: bool = False):
        if not torch.cuda.is_available():
            raise RuntimeError("GB300LBMSolver needs a CUDA device (no CPU path exists)")
        self.lib = _lib.load()
        self.cfg = config if config is not None else LatticeConfig()
        self.device = torch.device(device)
        self.preferred_backend = preferred_backend or "cuda"
        c = self.cfg
        self.NX, self.NY, self.NZ = c.nx, c.ny, c.nz
        self.n = c.ncell
        self._p = c.to_c()
        _lib.check(self.lib.pog_validate_params(self._p))
        shape = (c.nz, c.ny, c.nx)
        dev = self.device
        # one 32-bit word per cell: flag bits + bit (8+q) when neighbour q is solid
        self._flags = torch.empty(shape, dtype=torch.int32, device=dev)
        self._build_flags()
        # "auto" (default): the two-cell step kernel for FP16S/BF16S storage where it applies,
        # else the per-cell register-staged kernel; "registers": the per-cell kernel for every
        # storage; "rows": the row-tiled TMA-staged step (with its bounce-back cell list) where it
        # applies.  Same update in each.
        if step_kernel not in ("auto", "rows", "registers"):
            raise ValueError("step_kernel must be 'auto', 'rows' or 'registers'")
        self.step_kernel = step_kernel
        self._p.step_kernel = STEP_CELLS if step_kernel == "registers" else STEP_AUTO
        # FP16S with a per-cell reference density (pog_params.density_ref): each slot is stored
        # relative to its owner cell's density instead of rho0
        self._dref = None
        if density_reference:
            if c.storage != STORE_F16S:
                raise ValueError("density_reference needs FP16S storage")
            self._dref = torch.zeros(self.n, dtype=torch.float16, device=self.device)
            self._p.density_ref = self._dref.data_ptr()
        self._walls = None
        self._build_wall_list()
        self._f = torch.empty((19,) + shape, dtype=_STORAGE_DTYPE[c.storage], device=dev)
        self._rho = torch.ones(shape, dtype=torch.float32, device=dev)
        self._u = torch.zeros((3,) + shape, dtype=torch.float32, device=dev)
        # LES stencil mode: velocity ping-pong read/written by the step (separate from the
        # accessor buffer self._u so that reading solver.u never disturbs the LES input)
        self._ul = None
        if c.les_mode == LES_STENCIL:
            self._ul = [torch.zeros((3,) + shape, dtype=torch.float32, device=dev) for _ in range(2)]
        self._force = torch.zeros((3,) + shape, dtype=torch.float32, device=dev)
        self._force_active = False
        # particle drag deposit (Kp, Kv_x, Kv_y, Kv_z) written by the coupling pass
        self._pdrag = torch.zeros((4,) + shape, dtype=torch.float32, device=dev)
        self._pdrag_active = False
        self._pdrag_owner = None  # the particle system whose last deposit is all _pdrag holds
        # one bit per cell: set where _pdrag may be nonzero (the step reads the deposit there only)
        self._dmask = torch.zeros((self.n + 31) // 32, dtype=torch.int32, device=dev)
        self._p.deposit_mask = self._dmask.data_ptr()
        self._phase = torch.ones(shape, dtype=torch.float32, device=dev)
        self._red = torch.zeros(RED_COUNT, dtype=torch.float64, device=dev)
        self._porosity = None
        self._inlet_ctl = None
        self._pour_ctl = None
        self._blockage = None
        # rho written by a plugin (phase density, density drive) until the next step; a lazy
        # refresh of u then leaves it alone, as the reference's lbm.rho
        self._rho_external = False
        self._rho_scratch = None
        self._u_stale = False  # u must be recomputed (a force input changed), rho is current
        if porosity is not None:
            self.set_porosity(porosity)
        self.t = 0
        self._macro_dirty = True
        self._mass0 = None
        self.step_count = 0
        self.use_les = c.les_mode != LES_OFF
        self.boundary_manager = _FusedBoundaryManager()
        self.opposite_dir = OPPOSITE.copy()
        self._timing = {"steps": 0, "seconds": 0.0}
        self.initialize_fields(c.rho0, (0.0, 0.0, 0.0))

    # ---- plumbing -------------------------------------------------------------------------
    def _s(self):
        return _lib.stream_handle()

    def _build_flags(self):
        _lib.check(self.lib.pog_build_flags(self._p, _lib.ptr(self._flags), self._s()))

    def _build_wall_list(self):
        """The cells of the row-tiled step's bounce-back mailbox pass (pog_wall_list), kept on
        the device and referenced from the parameter block."""
        self._walls = None
        self._p.wall_cells = None
        self._p.n_wall_cells = 0
        if self.step_kernel != "rows":
            return
        count = torch.zeros(1, dtype=torch.int32, device=self.device)
        _lib.check(self.lib.pog_wall_list(self._p, _lib.ptr(self._flags), None, 0, _lib.ptr(count), self._s()))
        n = int(count.item())
        self._walls = torch.empty(max(n, 1), dtype=torch.int32, device=self.device)
        _lib.check(self.lib.pog_wall_list(self._p, _lib.ptr(self._flags), _lib.ptr(self._walls), n,
                                          _lib.ptr(count), self._s()))
        self._p.wall_cells = self._walls.data_ptr()
        self._p.n_wall_cells = n

    def _refresh_macro(self):
        """Recompute the moments the next read needs: rho and u when the state changed since they
        were taken (_macro_dirty), u alone when only a force input changed (_u_stale; rho does
        not depend on forces), never a density a plugin wrote (_rho_external)."""
        if not (self._macro_dirty or self._u_stale):
            return
        rho_out = self._rho
        if self._rho_external or not self._macro_dirty:
            if self._rho_scratch is None:
                self._rho_scratch = torch.empty_like(self._rho)
            rho_out = self._rho_scratch
        _lib.check(self.lib.pog_macroscopic(self._p, _lib.ptr(self._f), _lib.ptr(self._flags),
                                            self.t, _lib.ptr(self._force) if self._force_active else None,
                                            _lib.ptr(self._pdrag) if self._pdrag_active else None,
                                            _lib.ptr(rho_out), _lib.ptr(self._u), self._s()))
        self._macro_dirty = False
        self._u_stale = False

    def _current_rho(self) -> torch.Tensor:
        """The density field as the reference's lbm.rho holds it: a plugin-written density until
        the next step, else the moments of the current state."""
        if not self._rho_external:
            self._refresh_macro()
        return self._rho

    def _force_written(self):
        self._force_active = True
        self._u_stale = True

    # ---- fields (reference attribute surface) ---------------------------------------------
    @property
    def flags(self) -> torch.Tensor:
        return self._flags

    @property
    def f(self) -> FieldView:
        """Distributions in natural layout (f_q at each cell), a copy in FP32 [19, NZ, NY, NX]
        presented as (NX, NY, NZ, 19)."""
        nat = torch.empty((19, self.NZ, self.NY, self.NX), dtype=torch.float32, device=self.device)
        _lib.check(self.lib.pog_export_natural(self._p, _lib.ptr(self._f), _lib.ptr(self._flags),
                                               self.t, _lib.ptr(nat), STORE_F32, self._s()))
        return FieldView(nat, ncomp=19, readonly=True)

    @property
    def f_new(self) -> FieldView:
        """The AA pattern keeps one distribution buffer; f_new is the same state as f."""
        return self.f

    @property
    def rho(self) -> FieldView:
        return FieldView(self._rho, refresh=self._refresh_macro, readonly=True)

    @property
    def u(self) -> FieldView:
        return FieldView(self._u, ncomp=3, refresh=self._refresh_macro, readonly=True)

    @property
    def ux(self) -> FieldView:
        return FieldView(self._u[0], refresh=self._refresh_macro, readonly=True)

    @property
    def uy(self) -> FieldView:
        return FieldView(self._u[1], refresh=self._refresh_macro, readonly=True)

    @property
    def uz(self) -> FieldView:
        return FieldView(self._u[2], refresh=self._refresh_macro, readonly=True)

    @property
    def solid(self) -> FieldView:
        return FieldView((self._flags & CELL_SOLID), readonly=True)

    @property
    def phase(self) -> FieldView:
        """Phase indicator (0 air, 1 water).  1 everywhere for single-phase runs; the step reads
        it once a phase field is attached (set_phase_field, MultiphaseFlow3D)."""
        return FieldView(self._phase, on_write=self._phase_written)

    def _phase_written(self):
        self._u_stale = True

    @property
    def body_force(self) -> FieldView:
        # any access may write the tensor in place: the field then counts as live (an inactive
        # field is skipped by the step and by clear_body_force, which relies on it being zero)
        return FieldView(self._force, ncomp=3, refresh=self._force_written, on_write=self._force_written)

    @property
    def les_mask(self) -> FieldView:
        return FieldView(((self._flags & CELL_POROUS) == 0).to(torch.int32), readonly=True)

    @property
    def filter_zone(self) -> FieldView:
        return FieldView(((self._flags & CELL_POROUS) != 0).to(torch.int32), readonly=True)

    def get_velocity_vector_field(self) -> FieldView:
        return self.u

    def get_velocity_magnitude(self) -> np.ndarray:
        self._refresh_macro()
        return torch.sqrt((self._u.double() ** 2).sum(0)).permute(2, 1, 0).cpu().numpy()

    # ---- initialisation -------------------------------------------------------------------
    def initialize_fields(self, initial_density: float = 1.0,
                          initial_velocity: Tuple[float, float, float] = (0.0, 0.0, 0.0)) -> None:
        ux, uy, uz = (float(v) for v in initial_velocity)
        _lib.check(self.lib.pog_init_equilibrium(self._p, _lib.ptr(self._f), _lib.ptr(self._flags),
                                                 float(initial_density), ux, uy, uz, self._s()))
        self.t = 0
        self.step_count = 0
        fluid = (self._flags & CELL_SOLID) == 0
        self._rho.fill_(1.0)
        self._rho[fluid] = float(initial_density)
        self._u.zero_()
        for a, v in enumerate((ux, uy, uz)):
            self._u[a][fluid] = v
        if self._ul is not None:
            for b in self._ul:
                b.copy_(self._u)
        self._macro_dirty = False
        self._u_stale = False
        self._rho_external = False
        self._mass0 = float(self._rho[fluid].double().sum())

    def init_fields(self) -> None:
        """LBMSolver.init_fields (legacy/lbm_solver.py:1067): rho=1, u=0, f=w rho."""
        self.initialize_fields(self.cfg.rho0, (0.0, 0.0, 0.0))

    def set_geometry(self, geometry_function: Any) -> None:
        """Replace the solid mask.  `geometry_function` is an (NX, NY, NZ) boolean array or a
        callable f(i, j, k) -> bool array over index grids.  Inlet/outlet/porous bits of the
        V60 build are kept on cells that stay fluid; the outer one-cell shell must stay solid
        (the in-place AA step needs every fluid cell's 18 neighbours inside the grid)."""
        if callable(geometry_function):
            i, j, k = np.meshgrid(np.arange(self.NX), np.arange(self.NY), np.arange(self.NZ), indexing="ij")
            mask = np.asarray(geometry_function(i, j, k), dtype=bool)
        else:
            mask = np.asarray(geometry_function, dtype=bool)
        if mask.shape != (self.NX, self.NY, self.NZ):
            raise ValueError("geometry mask must have shape (NX, NY, NZ)")
        shell = np.ones_like(mask)
        shell[1:-1, 1:-1, 1:-1] = False
        if np.any(shell & ~mask):
            raise ValueError("the outer one-cell shell of the grid must be solid")
        solid = np.ascontiguousarray(mask.transpose(2, 1, 0))  # -> [z, y, x]
        old = self._flags.cpu().numpy().astype(np.uint32)
        fl = np.where(solid, CELL_SOLID, old & (CELL_INLET | CELL_OUTLET | CELL_POROUS)).astype(np.uint32)
        links = np.zeros(solid.shape, np.uint32)
        for q in range(1, 19):
            nb_solid = np.roll(solid, shift=(-CZ[q], -CY[q], -CX[q]), axis=(0, 1, 2))
            links |= nb_solid.astype(np.uint32) << np.uint32(8 + q)
        fl = np.where(~solid & (links != 0), fl | CELL_NEAR_SOLID | links, fl).astype(np.uint32)
        self._flags.copy_(torch.from_numpy(fl.astype(np.int32)))
        self._build_wall_list()
        self.initialize_fields(self.cfg.rho0)

    def set_porosity(self, eps) -> None:
        """Per-cell porosity for porous cells (x-fastest flat or (NX,NY,NZ) array)."""
        a = np.asarray(eps, dtype=np.float32)
        if a.shape == (self.NX, self.NY, self.NZ):
            a = a.transpose(2, 1, 0)
        self._porosity = torch.as_tensor(np.ascontiguousarray(a).reshape(self.NZ, self.NY, self.NX)).to(self.device)
        self._u_stale = True

    # ---- stepping -------------------------------------------------------------------------
    def run(self, nsteps: int, reduce: bool = False, want_macro: bool = False) -> Optional[torch.Tensor]:
        """Advance nsteps fused steps (one kernel launch each).  reduce=True accumulates the
        FP64 mass/momentum/outflow/non-finite sums of these steps into a returned tensor."""
        if nsteps <= 0:
            return None
        red = None
        st = self._s()
        if reduce:
            red = self._red.data_ptr()
            _lib.check(self.lib.pog_zero(red, self._red.numel() * 8, st))
        stencil = self.cfg.les_mode == LES_STENCIL
        up = _lib.ptr(self._ul[0]) if stencil else None
        un = _lib.ptr(self._ul[1]) if stencil else None
        _lib.check(self.lib.pog_step(
            self._p, _lib.ptr(self._f), _lib.ptr(self._flags), self.t, int(nsteps),
            _lib.ptr(self._force) if self._force_active else None,
            _lib.ptr(self._pdrag) if self._pdrag_active else None,
            _lib.ptr(self._porosity), up, un,
            _lib.ptr(self._rho) if want_macro else None,
            _lib.ptr(self._u) if want_macro else None,
            red, st))
        if stencil and nsteps % 2 == 1:
            self._ul.reverse()
        self.t += int(nsteps)
        self.step_count += int(nsteps)
        # with want_macro, rho/u hold the moments computed inside the last step (of the state
        # that step started from, as the reference's solver.rho/u after step()); otherwise they
        # are recomputed from the current state when read.
        self._macro_dirty = not want_macro
        self._u_stale = False
        self._rho_external = False
        return self._red if reduce else None

    def step(self) -> None:
        """One full LBM time step (LBMSolver.step, legacy/lbm_solver.py:817-867)."""
        self.run(1)

    def collision_step(self) -> None:
        """Collision and streaming are one fused in-place pass: this performs the whole step."""
        self.run(1)

    def streaming_step(self) -> None:
        """Streaming is fused into collision_step (AA pattern); nothing is left to do."""
        return None

    def compute_macroscopic_quantities(self) -> None:
        self._rho_external = False
        self._macro_dirty = True
        self._refresh_macro()

    def apply_boundary_conditions(self) -> None:
        """Inlet, outlet and bounce-back walls are applied inside the fused step."""
        return None

    def step_with_particles(self, particle_system: Optional[object]) -> None:
        """legacy/lbm_solver.py:869-900: one step, then particle_system.update(self) if it
        has one."""
        self.step()
        if particle_system is not None and hasattr(particle_system, "update"):
            particle_system.update(self)

    def clear_body_force(self) -> None:
        # an inactive force field is all zeros already (every writer marks it active)
        if self._force_active:
            self._force.zero_()
            self._force_active = False
            self._u_stale = True

    def add_force_term(self, force_field: Any) -> None:
        """body_force += force_field ((NX,NY,NZ,3) array/tensor or a FieldView)."""
        if isinstance(force_field, FieldView):
            t = force_field.tensor
            if t.shape != self._force.shape:
                raise ValueError("force field shape mismatch")
        else:
            t = torch.as_tensor(np.asarray(force_field), dtype=torch.float32).to(self.device).permute(3, 2, 1, 0)
        self._force.add_(t)
        self._force_written()

    def step_with_two_way_coupling(self, particle_system, dt: float = 1.0,
                                   relaxation_factor: float = 0.8, reduce: bool = False):
        """legacy/lbm_solver.py:1485-1509: clear body force, particle drag + relaxed reaction
        spread into body_force, one LBM step with that force, particle integration.  With
        reduce=True returns the step's FP64 sums (mass, momentum, outflow, non-finite)."""
        self._refresh_macro()  # the coupling reads u of the current state
        self.clear_body_force()  # legacy/lbm_solver.py:1489
        # the deposit field holds only this particle system's previous deposit: zero those
        # cells instead of the whole field
        if self._pdrag_owner is particle_system and particle_system._dep_valid:
            particle_system.clear_deposit(self, self._pdrag, self._dmask)
        else:
            self._pdrag.zero_()
            self._dmask.zero_()
        particle_system.couple(self, dt=dt, relaxation_factor=relaxation_factor, pdrag=self._pdrag,
                               deposit_mask=self._dmask)
        self._pdrag_owner = particle_system
        self._pdrag_active = True
        return self.run(1, want_macro=True, reduce=reduce)

    def particle_reaction_force(self) -> torch.Tensor:
        """Force density the particles exerted on the fluid in the last coupled step,
        Kv - Kp u ([3, NZ, NY, NX]); zero before any coupled step."""
        if not self._pdrag_active:
            return torch.zeros_like(self._force)
        self._refresh_macro()
        return self._pdrag[1:] - self._pdrag[0:1] * self._u

    def set_inlet_control(self, control: Optional[torch.Tensor]) -> None:
        """Feed the pour from a device tensor [u_inlet, a_0..a_15] (float32, 17 values) that the
        step reads on the device, so it may change between steps (or graph replays) without a
        new parameter block.  None returns to the configured u_inlet/inlet_coef."""
        if control is not None:
            if control.dtype != torch.float32 or control.numel() != 17 or not control.is_cuda:
                raise ValueError("inlet control must be a CUDA float32 tensor of 17 values")
            control = control.contiguous()
        self._inlet_ctl = control
        self._p.inlet_control = None if control is None else control.data_ptr()

    def save_checkpoint(self, path: str, particles=None, pour=None, filter_system=None, multiphase=None) -> None:
        """Raw state of the run (and of its particles / pour nozzle / filter paper / phase field)
        to an .npz file that load_checkpoint continues bit for bit."""
        from .diagnostics import save_checkpoint
        save_checkpoint(path, self, particles, pour, filter_system, multiphase)

    def load_checkpoint(self, path: str, particles=None, pour=None, filter_system=None, multiphase=None) -> None:
        from .diagnostics import load_checkpoint
        load_checkpoint(path, self, particles, pour, filter_system, multiphase)

    def set_pour_control(self, block: Optional[torch.Tensor]) -> None:
        """Attach a pour-nozzle block (PrecisePouringSystem.block: CUDA float32, POG_POUR_NFIELDS
        values) read by the step kernel and the particle coupling; None detaches it."""
        if block is not None:
            if block.dtype != torch.float32 or block.numel() != 20 or not block.is_cuda or not block.is_contiguous():
                raise ValueError("pour block must be a contiguous CUDA float32 tensor of 20 values")
        self._pour_ctl = block
        self._p.pour_control = None if block is None else block.data_ptr()
        self._u_stale = True

    def set_phase_field(self, phase: Optional[torch.Tensor], tau_air: Optional[float] = None) -> None:
        """Let the step read a phase indicator (CUDA float32, one value per cell, 0 air .. 1 water):
        gravity on the water fraction, tau = tau where phase > 0.5 else tau_air, no LES where
        |phase| < 0.9.  None returns to single-phase water."""
        if phase is not None:
            if (phase.dtype != torch.float32 or phase.numel() != self.n or not phase.is_cuda
                    or not phase.is_contiguous()):
                raise ValueError("phase must be a contiguous CUDA float32 tensor of ncell values")
        if tau_air is not None:
            self._p.tau_air = float(tau_air)
        self._phase_attached = phase
        self._p.phase = None if phase is None else phase.data_ptr()
        _lib.check(self.lib.pog_validate_params(self._p))
        self._u_stale = True

    def set_filter_blockage(self, blockage: Optional[torch.Tensor]) -> None:
        """Attach the filter-paper blockage field b (CUDA float32, one value per cell, written by
        FilterPaperSystem): porous cells scale their Darcy and Forchheimer coefficients by
        (1 + b).  None detaches it."""
        if blockage is not None:
            if (blockage.dtype != torch.float32 or blockage.numel() != self.n or not blockage.is_cuda
                    or not blockage.is_contiguous()):
                raise ValueError("filter blockage must be a contiguous CUDA float32 tensor of ncell values")
        self._blockage = blockage
        self._p.filter_blockage = None if blockage is None else blockage.data_ptr()
        self._u_stale = True

    def capture(self, nsteps: int, particle_system=None, dt: float = 1.0,
                relaxation_factor: float = 0.8) -> "StepGraph":
        """Capture `nsteps` (even) plain or two-way coupled steps into a CUDA graph; replaying
        it advances the solver by nsteps with one graph launch."""
        return StepGraph(self, nsteps, particle_system, dt, relaxation_factor)

    def update_particle_coupling(self, particle_system: Any) -> None:
        self.step_with_two_way_coupling(particle_system)

    def compute_drag_force(self) -> FieldView:
        """ParticleCoupledLBMProtocol: the particles' force on the fluid (lbm_protocol.py:235)."""
        return FieldView(self.particle_reaction_force(), ncomp=3, readonly=True)

    # ---- diagnostics ------------------------------------------------------------------------
    def conservation(self) -> dict:
        """FP64 device sums over fluid cells of the current state (mass, momentum)."""
        self._refresh_macro()
        fluid = (self._flags & CELL_SOLID) == 0
        rho = self._rho.double()
        m = float((rho * fluid).sum())
        mom = [float((rho * self._u[a].double() * fluid).sum()) for a in range(3)]
        return {"mass": m, "momentum": mom}

    def get_kinetic_energy(self) -> float:
        self._refresh_macro()
        fluid = (self._flags & CELL_SOLID) == 0
        e = 0.5 * self._rho.double() * (self._u.double() ** 2).sum(0)
        return float((e * fluid).sum())

    def get_mass_conservation_error(self) -> float:
        m = self.conservation()["mass"]
        return abs(m - self._mass0) / self._mass0 if self._mass0 else 0.0

    def check_stability(self) -> bool:
        self._refresh_macro()
        fluid = (self._flags & CELL_SOLID) == 0
        finite = bool(torch.isfinite(self._rho[fluid]).all() and torch.isfinite(self._u[:, fluid]).all())
        if not finite:
            return False
        umax = float(torch.sqrt((self._u.double() ** 2).sum(0)).max())
        return umax < 0.3

    def get_diagnostics(self) -> dict:
        cons = self.conservation()
        self._refresh_macro()
        umax = float(torch.sqrt((self._u.double() ** 2).sum(0)).max())
        return {"step": self.step_count, "t": self.t, "mass": cons["mass"],
                "momentum": cons["momentum"], "max_velocity": umax,
                "mass_conservation_error": self.get_mass_conservation_error(),
                "stable": self.check_stability(), "les_mode": self.cfg.les_mode,
                "storage": self.cfg.storage, "grid": (self.NX, self.NY, self.NZ)}

    def get_memory_usage(self) -> dict:
        out = {"f": self._f.numel() * self._f.element_size(),
               "flags": self._flags.numel(), "rho": self._rho.numel() * 4,
               "u": self._u.numel() * 4 * (3 if self._ul is not None else 1),
               "body_force": self._force.numel() * 4}
        if self._porosity is not None:
            out["porosity"] = self._porosity.numel() * 4
        out["total"] = sum(out.values())
        return out

    def optimize_memory_layout(self) -> None:
        """The layout is fixed: SoA planes, x fastest, one AA buffer."""
        return None

    def enable_les_turbulence(self, smagorinsky_constant: float = 0.1, mode: int = LES_LOCAL) -> None:
        if mode == LES_STENCIL and self._ul is None:
            self._ul = [self._u.clone(), self._u.clone()]
        self.cfg = self.cfg.replace(les_mode=mode, cs_smag=float(smagorinsky_constant))
        p = self.cfg.to_c()
        for name in ("inlet_control", "pour_control", "filter_blockage", "phase", "deposit_mask",
                     "wall_cells", "n_wall_cells", "step_kernel", "density_ref", "tau_air"):
            setattr(p, name, getattr(self._p, name))
        self._p = p
        self.use_les = True

    def export_vtk(self, filename: str) -> None:
        """Legacy binary VTK structured points with rho, u and the solid flag."""
        self._refresh_macro()
        rho = self._rho.cpu().numpy()
        u = self._u.cpu().numpy()
        solid = (self._flags & CELL_SOLID).cpu().numpy().astype(np.float32)
        name = filename if filename.endswith(".vtk") else filename + ".vtk"
        with open(name, "wb") as fh:
            hdr = ("# vtk DataFile Version 3.0\npour-over D3Q19\nBINARY\nDATASET STRUCTURED_POINTS\n"
                   "DIMENSIONS %d %d %d\nORIGIN 0 0 0\nSPACING 1 1 1\nPOINT_DATA %d\n"
                   % (self.NX, self.NY, self.NZ, self.n))
            fh.write(hdr.encode())
            fh.write(b"SCALARS rho float 1\nLOOKUP_TABLE default\n")
            fh.write(rho.astype(">f4").tobytes())
            fh.write(b"\nSCALARS solid float 1\nLOOKUP_TABLE default\n")
            fh.write(solid.astype(">f4").tobytes())
            fh.write(b"\nVECTORS u float\n")
            fh.write(np.stack([u[0], u[1], u[2]], axis=-1).astype(">f4").tobytes())
            fh.write(b"\n")


class StepGraph:
    """A CUDA graph of an even number of steps (the AA parity repeats every two steps).

    Capture runs the normal Python step path once on torch's capture stream; the host-side
    counters it advanced are restored, and every replay() advances them instead.  The first
    eager steps before capture must already have run (they initialise the launch shapes).
    """

    def __init__(self, solver: GB300LBMSolver, nsteps: int, particle_system=None, dt: float = 1.0,
                 relaxation_factor: float = 0.8):
        if nsteps <= 0 or nsteps % 2:
            raise ValueError("a step graph needs a positive even number of steps")
        self.solver = solver
        self.ps = particle_system
        self.nsteps = nsteps
        saved = (solver.t, solver.step_count)
        ps_saved = particle_system._since_sort if particle_system is not None else None
        if particle_system is not None and ps_saved is None:
            particle_system.bin(solver, sort=True)
            ps_saved = 0
        _lib.load().pog_launch_count(1)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            for _ in range(nsteps):
                if particle_system is None:
                    solver.run(1)
                else:
                    solver.step_with_two_way_coupling(particle_system, dt, relaxation_factor)
        self.kernels = int(_lib.load().pog_launch_count(1))
        solver.t, solver.step_count = saved
        self._ps_after = particle_system._since_sort if particle_system is not None else None
        if particle_system is not None:
            particle_system._since_sort = ps_saved

    def replay(self) -> None:
        s = self.solver
        if s.t % 2:
            raise RuntimeError("a step graph must be replayed at an even time index")
        self.graph.replay()
        s.t += self.nsteps
        s.step_count += self.nsteps
        s._macro_dirty = self.ps is None
        s._u_stale = False
        s._rho_external = False
        if self.ps is not None:
            self.ps._since_sort = self._ps_after


class UnifiedLBMSolver(GB300LBMSolver):
    """Constructor surface of src/core/lbm_unified.py:32-44 (preferred_backend accepted and
    recorded; there is one backend)."""

    def __init__(self, preferred_backend: Optional[str] = None, config: Optional[LatticeConfig] = None):
        super().__init__(config=config, preferred_backend=preferred_backend)


def create_unified_solver(preferred_backend: Optional[str] = None,
                          config: Optional[LatticeConfig] = None) -> UnifiedLBMSolver:
    """lbm_unified.py:316."""
    return UnifiedLBMSolver(preferred_backend, config=config)


LBMSolver = GB300LBMSolver
