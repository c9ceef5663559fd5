"""The reference's solver protocols, restated without Taichi.

Same names, members and meaning as src/core/lbm_protocol.py:12-285 (LBMSolverProtocol,
MultiphaseLBMProtocol, ParticleCoupledLBMProtocol, validate_lbm_solver,
get_solver_capabilities); field annotations are `Any` because the fields are FieldView
objects over device tensors instead of ti.field.
"""
from typing import Any, Protocol, Tuple, runtime_checkable


@runtime_checkable
class LBMSolverProtocol(Protocol):
    f: Any
    f_new: Any
    rho: Any
    u: Any
    solid: Any
    phase: Any

    def step(self) -> None: ...
    def collision_step(self) -> None: ...
    def streaming_step(self) -> None: ...
    def compute_macroscopic_quantities(self) -> None: ...
    def apply_boundary_conditions(self) -> None: ...
    def initialize_fields(self, initial_density: float = 1.0,
                          initial_velocity: Tuple[float, float, float] = (0.0, 0.0, 0.0)) -> None: ...
    def set_geometry(self, geometry_function: Any) -> None: ...
    def get_diagnostics(self) -> dict: ...
    def check_stability(self) -> bool: ...
    def get_kinetic_energy(self) -> float: ...
    def get_mass_conservation_error(self) -> float: ...
    def get_memory_usage(self) -> dict: ...
    def optimize_memory_layout(self) -> None: ...
    def enable_les_turbulence(self, smagorinsky_constant: float = 0.1) -> None: ...
    def add_force_term(self, force_field: Any) -> None: ...
    def export_vtk(self, filename: str) -> None: ...


@runtime_checkable
class MultiphaseLBMProtocol(LBMSolverProtocol, Protocol):
    def compute_phase_field(self) -> None: ...
    def apply_surface_tension(self) -> None: ...
    def set_contact_angle(self, angle: float) -> None: ...


@runtime_checkable
class ParticleCoupledLBMProtocol(LBMSolverProtocol, Protocol):
    def update_particle_coupling(self, particle_system: Any) -> None: ...
    def compute_drag_force(self) -> Any: ...


def validate_lbm_solver(solver: Any) -> bool:
    """lbm_protocol.py:241: isinstance check against LBMSolverProtocol."""
    return isinstance(solver, LBMSolverProtocol)


def get_solver_capabilities(solver: Any) -> dict:
    """lbm_protocol.py:260: capability flags."""
    return {
        "basic_lbm": True,
        "multiphase": isinstance(solver, MultiphaseLBMProtocol),
        "particle_coupling": isinstance(solver, ParticleCoupledLBMProtocol),
        "les_turbulence": hasattr(solver, "enable_les_turbulence"),
        "vtk_export": hasattr(solver, "export_vtk"),
        "apple_silicon_optimized": hasattr(solver, "apple_config"),
        "jax_hybrid": hasattr(solver, "jax_enabled"),
    }


LBMSolver = LBMSolverProtocol
MultiphaseLBM = MultiphaseLBMProtocol
ParticleCoupledLBM = ParticleCoupledLBMProtocol
