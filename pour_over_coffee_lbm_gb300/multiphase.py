"""MultiphaseFlow3D on libpog.so: the Cahn-Hilliard phase field of src/core/multiphase_3d.py.

phi in [-1, 1] (-1 air, +1 water) is advected by the lattice velocity, relaxed by the
phase-separation term and turned into the solver's phase indicator (phi + 1)/2 and density
rho_air + (rho_water - rho_air)(phi + 1)/2 after every lattice step.  The lattice step reads the
phase indicator itself: gravity acts on the water fraction, tau switches between the water and
air values at phase 0.5 and the LES viscosity is off where |phase| < 0.9.  The surface tension
sigma kappa |grad phi| n (continuum surface force) enters the solver's body force before the
collision.

Kernels (csrc/multiphase.cu), one pass each over [NZ][NY][NX] float fields:
  pog_phase_normals          grad phi -> unit normal and |grad phi|
  pog_phase_surface_tension  curvature div n, the CSF force, body_force += F / rho
  pog_phase_update           advection + M lap(mu) + clamp + phase separation + rho/phase
phi lives in two buffers used in turn (the reference's phi / phi_new with the copy folded into
the swap).  The reference's step() recomputes the normals, curvature and surface force of phi every step
even when they feed nothing; here they are computed when the body force or the statistics need
them, and the curvature / surface_force fields are filled on demand.

The reference's chemical potential mu is computed once, at standardize_initial_state, and only
read afterwards (compute_chemical_potential is not part of its step); the same holds here.
"""
from typing import Any, Dict

import torch

from . import _lib
from .params import CELL_SOLID

# reference constants in lattice units (config/physics.py, config/core.py)
SURFACE_TENSION_LU = 0.0036
RHO_WATER = 1.0
RHO_AIR = 0.0012472806381435824
SCALE_LENGTH = 0.000625  # m per lattice unit (statistics only)


class MultiphaseFlow3D:
    def __init__(self, lbm_solver: Any, surface_tension: float = SURFACE_TENSION_LU, interface_width: float = 2.0,
                 mobility: float = 0.001, rho_water: float = RHO_WATER, rho_air: float = RHO_AIR, dt: float = 1.0,
                 scale_length: float = SCALE_LENGTH):
        if not torch.cuda.is_available():
            raise RuntimeError("MultiphaseFlow3D needs a CUDA device")
        self.lib = _lib.load()
        self.lbm = lbm_solver
        s = lbm_solver
        shape = (s.NZ, s.NY, s.NX)
        dev = s._flags.device
        self.INTERFACE_WIDTH = float(interface_width)
        self.MOBILITY = float(mobility)
        self.SURFACE_TENSION_COEFF = float(surface_tension)
        self.CAHN_NUMBER = 0.005
        self.BETA = 12.0 * self.SURFACE_TENSION_COEFF / self.INTERFACE_WIDTH
        self.KAPPA = 1.5 * self.SURFACE_TENSION_COEFF * self.INTERFACE_WIDTH
        self.RHO_WATER, self.RHO_AIR, self.DT = float(rho_water), float(rho_air), float(dt)
        self.SCALE_LENGTH = float(scale_length)
        # phi and phi_new (zero until an initial state is set, as the reference's fields)
        self._phi = [torch.zeros(shape, dtype=torch.float32, device=dev) for _ in range(2)]
        self._cur = 0
        self.mu = torch.zeros(shape, dtype=torch.float32, device=dev)
        self._mu_live = False  # mu is identically zero until compute_chemical_potential
        self.normal = torch.zeros((3,) + shape, dtype=torch.float32, device=dev)
        self.gmag = torch.zeros(shape, dtype=torch.float32, device=dev)
        self.curvature = torch.zeros(shape, dtype=torch.float32, device=dev)
        self.surface_force = torch.zeros((3,) + shape, dtype=torch.float32, device=dev)
        self._version = 0  # bumped whenever phi changes
        self._geo_version = -1  # phi version the normals belong to
        self._out_version = -1  # phi version the curvature / surface_force fields belong to
        s.set_phase_field(s._phase)

    # ---- fields --------------------------------------------------------------------------------
    @property
    def phi(self) -> torch.Tensor:
        return self._phi[self._cur]

    @property
    def phi_new(self) -> torch.Tensor:
        return self._phi[1 - self._cur]

    @property
    def grad_phi(self) -> torch.Tensor:
        """|grad phi| times the unit normal (the normal is zero where |grad phi| <= 1e-10)."""
        return self.normal * self.gmag

    def phi_changed(self) -> None:
        """Call after writing phi directly."""
        self._version += 1

    def _ctx(self):
        s = self.lbm
        return s._p, _lib.stream_handle()

    # ---- initial state -------------------------------------------------------------------------
    def init_phase_field(self) -> None:
        """Dry filter: air everywhere (init_phase_field :55-78)."""
        for b in self._phi:
            b.fill_(-1.0)
        self.phi_changed()

    def _set_dry_initial_state(self) -> None:
        fluid = (self.lbm._flags & CELL_SOLID) == 0
        for b in self._phi:
            b.masked_fill_(fluid, -1.0)
        self.phi_changed()

    def standardize_initial_state(self, force_dry_state: bool = True) -> None:
        """:542-571: air in every fluid cell, then rho/phase, mu and the gradients from it."""
        if force_dry_state:
            self._set_dry_initial_state()
        self.update_density_from_phase()
        self.compute_chemical_potential()
        self.compute_gradients()
        self.validate_initial_phase_consistency()

    # ---- device passes -------------------------------------------------------------------------
    def compute_chemical_potential(self) -> None:
        p, st = self._ctx()
        kappa = 3.0 * self.SURFACE_TENSION_COEFF * self.INTERFACE_WIDTH / 8.0
        _lib.check(self.lib.pog_phase_chemical_potential(p, _lib.ptr(self.phi), kappa, _lib.ptr(self.mu), st))
        self._mu_live = True

    def compute_gradients(self) -> None:
        p, st = self._ctx()
        _lib.check(self.lib.pog_phase_normals(p, _lib.ptr(self.phi), _lib.ptr(self.normal), _lib.ptr(self.gmag), st))
        self._geo_version = self._version

    def _tension(self, accumulate: bool, outputs: bool = True) -> None:
        s = self.lbm
        rho = s._current_rho()
        p, st = self._ctx()
        _lib.check(self.lib.pog_phase_surface_tension(
            p, _lib.ptr(s._flags), _lib.ptr(self.phi), _lib.ptr(self.normal), _lib.ptr(self.gmag), _lib.ptr(rho),
            self.SURFACE_TENSION_COEFF, _lib.ptr(s._force) if accumulate else None,
            _lib.ptr(self.curvature) if outputs else None, _lib.ptr(self.surface_force) if outputs else None, st))
        if accumulate:
            s._force_written()
        if outputs:
            self._out_version = self._version

    def compute_curvature(self) -> None:
        """Curvature and surface force of the current normals (one fused pass)."""
        self._tension(False)

    def compute_surface_tension_force(self) -> None:
        self._tension(False)

    def apply_surface_tension(self) -> None:
        """body_force += F / rho on the fluid cells, rho being the solver's current density field
        (the phase density the last step of this class wrote)."""
        self._tension(True, outputs=False)

    def _normals_current(self) -> None:
        if self._geo_version != self._version:
            self.compute_gradients()

    def accumulate_surface_tension_pre_collision(self) -> None:
        """:409-414: normals, curvature and force of the current phi into the body force (the
        curvature and force fields themselves are filled on demand, for the statistics)."""
        self._normals_current()
        self._tension(True, outputs=False)

    def update_phase_field_cahn_hilliard(self) -> None:
        """Advection, M lap(mu), clamp and phase separation into phi_new, then rho and the phase
        indicator from it (:151-197, :334-352, :365-381 in one pass); phi_new becomes phi."""
        s = self.lbm
        p, st = self._ctx()
        u = s.u.tensor
        _lib.check(self.lib.pog_phase_update(
            p, _lib.ptr(s._flags), _lib.ptr(self.phi), _lib.ptr(self.phi_new), _lib.ptr(u),
            _lib.ptr(self.mu) if self._mu_live else None, self.MOBILITY, self.DT, self.RHO_AIR, self.RHO_WATER,
            _lib.ptr(s._rho), _lib.ptr(s._phase), st))
        s._rho_external = True
        self._cur = 1 - self._cur
        self.phi_changed()

    def update_density_from_phase(self) -> None:
        s = self.lbm
        p, st = self._ctx()
        s._refresh_macro()  # u stays the moment of the current state
        _lib.check(self.lib.pog_phase_properties(p, _lib.ptr(self.phi), self.RHO_AIR, self.RHO_WATER, _lib.ptr(s._rho),
                                                 _lib.ptr(s._phase), st))
        s._rho_external = True

    def copy_phase_field(self) -> None:
        self.phi_new.copy_(self.phi)

    def step(self, step_count: int = 0, precollision_applied: bool = False) -> None:
        """One phase-field step after a lattice step (:389-407).  The reference also recomputes
        the normals, curvature and force here; they only feed the body force (when not applied
        before the collision) and the statistics, so they are computed when one of those needs
        them."""
        if (not precollision_applied) and step_count > 10:
            self._normals_current()
            self._tension(True, outputs=False)
        self.update_phase_field_cahn_hilliard()

    # ---- statistics and checks -----------------------------------------------------------------
    def get_interface_statistics(self) -> Dict[str, float]:
        """:290-311 on the device fields."""
        self._normals_current()
        if self._out_version != self._version:
            self._tension(False)
        phi = self.phi
        mask = phi.abs() < 0.9
        nmask = int(mask.sum().item())
        thick = (1.0 / (self.gmag.double() + 1e-10))[mask].mean().item() if nmask else float("nan")
        return {"interface_volume": nmask * self.SCALE_LENGTH ** 3,
                "water_fraction": float((phi > 0).sum().item()) / phi.numel(),
                "interface_thickness": thick * self.SCALE_LENGTH,
                "max_curvature": float(self.curvature.abs().max().item()),
                "surface_tension_magnitude": float(self.surface_force.double().norm(dim=0).max().item())}

    def _fluid(self):
        return (self.lbm._flags & CELL_SOLID) == 0

    def validate_initial_phase_consistency(self) -> Dict[str, Any]:
        """:420-540: phi range, density/phase consistency, solid count, air fraction."""
        phi = self.phi
        out_of_range = int(((phi < -1.1) | (phi > 1.1)).sum().item())
        if out_of_range:
            raise ValueError("%d phase-field values outside [-1, 1]" % out_of_range)
        fl = self._fluid()
        expected = (self.RHO_WATER * (1.0 + phi.double()) + self.RHO_AIR * (1.0 - phi.double())) * 0.5
        rel = ((self.lbm._rho.double() - expected).abs() / expected)[fl]
        nfluid = int(fl.sum().item())
        air = float((phi[fl] < -0.5).sum().item()) / max(nfluid, 1)
        return {"out_of_range": out_of_range, "density_inconsistent": int((rel > 0.05).sum().item()),
                "solid_nodes": int((~fl).sum().item()), "air_fraction": air, "dry": air >= 0.9}
