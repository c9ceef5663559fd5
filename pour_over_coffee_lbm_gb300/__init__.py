"""pour_over_coffee_lbm_gb300 -- GB300-native (sm_103a) D3Q19 lattice-Boltzmann step and
coffee-particle coupling of the pour-over V60 simulator, behind the reference's solver
protocol.  Compute runs in libpog.so (hand-written CUDA, C ABI in include/pog.h); this package
binds it with ctypes and mirrors the reference's Python interface.

Importing the package needs neither a GPU nor the built library; constructing a solver needs
both (there is no CPU fallback).
"""
from .params import (CELL_INLET, CELL_NEAR_SOLID, CELL_OUTLET, CELL_POROUS, CELL_SOLID,
                     DRAG_EXPLICIT_CAP, DRAG_SEMI_IMPLICIT, FORCING_GUO, FORCING_REFERENCE,
                     INLET_NCOEF, LES_LOCAL, LES_OFF, LES_STENCIL, STORE_BF16S, STORE_F16S,
                     STORE_F32, STORE_F64, LatticeConfig, ParticleConfig, PogParams,
                     PogParticleParams, coupled_128, differentiation_96, from_reference_config,
                     plain_64, porosity_field, precision_256, scale_320x384, seed_particles)
from .protocol import (LBMSolverProtocol, MultiphaseLBMProtocol, ParticleCoupledLBMProtocol,
                       get_solver_capabilities, validate_lbm_solver)

__all__ = [
    "LatticeConfig", "ParticleConfig", "GB300LBMSolver", "UnifiedLBMSolver",
    "create_unified_solver", "CoffeeParticleSystem", "OutflowAdjoint", "outflow_loss",
    "LBMSolverProtocol", "ParticleCoupledLBMProtocol", "validate_lbm_solver",
    "PrecisePouringSystem", "SlabLattice", "LBMDiagnostics", "SnapshotWriter", "export_data_for_analysis",
    "FilterPaperSystem",
    "PressureGradientDrive", "MultiphaseFlow3D",
]


def __getattr__(name):
    # torch-dependent classes load lazily so `import pour_over_coffee_lbm_gb300` stays light
    if name in ("GB300LBMSolver", "UnifiedLBMSolver", "create_unified_solver", "LBMSolver",
                "FieldView"):
        from . import solver
        return getattr(solver, name)
    if name == "CoffeeParticleSystem":
        from .particles import CoffeeParticleSystem
        return CoffeeParticleSystem
    if name in ("OutflowAdjoint", "outflow_loss", "OutflowLoss"):
        from . import adjoint
        return getattr(adjoint, name)
    if name == "PrecisePouringSystem":
        from .pouring import PrecisePouringSystem
        return PrecisePouringSystem
    if name in ("LBMDiagnostics", "SnapshotWriter", "export_data_for_analysis"):
        from . import diagnostics
        return getattr(diagnostics, name)
    if name == "MultiphaseFlow3D":
        from .multiphase import MultiphaseFlow3D
        return MultiphaseFlow3D
    if name == "PressureGradientDrive":
        from .drive import PressureGradientDrive
        return PressureGradientDrive
    if name == "FilterPaperSystem":
        from .filter import FilterPaperSystem
        return FilterPaperSystem
    if name == "SlabLattice":
        from .slabs import SlabLattice
        return SlabLattice
    raise AttributeError(name)
