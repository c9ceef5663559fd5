"""PrecisePouringSystem on libpog.so: the pour nozzle of src/physics/precise_pouring.py:12-420.

Same methods as the reference class (start_pouring, stop_pouring, apply_pouring_force,
create_water_impact_force, get_pouring_info, get_pouring_diagnostics, get_current_flow_rate,
adjust_flow_rate, switch_to_spiral_pour, move_pour_center), in lattice units.  The nozzle state
lives in a small device block (layout POG_POUR_* of include/pog.h) that the lattice step and the
particle kernel read: the stream's downward force is applied inside the fused step to the cells
of the nozzle's planes only, instead of through a separate body-force field, and
pog_pour_advance moves the nozzle on the device (a captured CUDA graph replays a moving pour).
apply_gradual_phase_change turns the stream's cells toward water in a MultiphaseFlow3D phase
field (pog_pour_phase).
"""
import math
from typing import Optional

import torch

from . import _lib
from .params import LatticeConfig

POUR_ACTIVE, POUR_X, POUR_Y, POUR_RADIUS, POUR_ZTOP, POUR_HEIGHT = 0, 1, 2, 3, 4, 5
POUR_VELOCITY, POUR_FLOW, POUR_DT, POUR_ACCEL_CAP, POUR_PATTERN = 6, 7, 8, 9, 10
POUR_CX, POUR_CY, POUR_SPIRAL_R, POUR_SPIRAL_SPEED, POUR_TIME = 11, 12, 13, 14, 15
POUR_DIAMETER, POUR_IMPACT, POUR_IMPACT_MAX, POUR_IMPACT_ZMIN = 16, 17, 18, 19
POUR_NFIELDS = 20


class PrecisePouringSystem:
    """A vertical stream of `diameter` cells ending `stream_height` planes below plane `height`,
    driven at `velocity` lattice units per step (the reference: 0.5 cm stream, POUR_HEIGHT just
    above the cup rim capped at NZ - 6, POUR_VELOCITY = INLET_VELOCITY)."""

    def __init__(self, lattice: LatticeConfig, diameter: float = 2.0, height: Optional[float] = None,
                 velocity: Optional[float] = None, stream_height: float = 4.0, device: str = "cuda"):
        if not torch.cuda.is_available():
            raise RuntimeError("PrecisePouringSystem needs a CUDA device")
        self.lib = _lib.load()
        self.lattice = lattice
        self.POUR_DIAMETER_GRID = float(diameter)
        self.POUR_HEIGHT = float(height if height is not None else max(8, lattice.nz - 6))
        self.POUR_VELOCITY = float(velocity if velocity is not None else abs(lattice.u_inlet))
        self.POUR_STREAM_HEIGHT = float(stream_height)
        self.block = torch.zeros(POUR_NFIELDS, dtype=torch.float32, device=device)
        self._set(POUR_RADIUS, self.POUR_DIAMETER_GRID / 2.0)
        self._set(POUR_ZTOP, self.POUR_HEIGHT)
        self._set(POUR_HEIGHT, self.POUR_STREAM_HEIGHT)
        self._set(POUR_VELOCITY, self.POUR_VELOCITY)
        self._set(POUR_ACCEL_CAP, 10.0)  # apply_pouring_force's cap (:156)
        self._set(POUR_DIAMETER, self.POUR_DIAMETER_GRID)
        self._set(POUR_IMPACT_ZMIN, 0.3 * lattice.nz)
        self._solvers = []
        self._dt = None

    def _set(self, idx: int, value: float) -> None:
        self.block[idx] = float(value)

    def _get(self, idx: int) -> float:
        return float(self.block[idx].item())

    # ---- reference control surface ----------------------------------------------------------
    def start_pouring(self, center_x=None, center_y=None, flow_rate=1.0, pattern="center"):
        """precise_pouring.py:46-72."""
        cx = self.lattice.nx // 2 if center_x is None else center_x
        cy = self.lattice.ny // 2 if center_y is None else center_y
        for idx, v in ((POUR_CX, cx), (POUR_CY, cy), (POUR_X, cx), (POUR_Y, cy), (POUR_FLOW, flow_rate),
                       (POUR_TIME, 0.0), (POUR_ACTIVE, 1.0)):
            self._set(idx, v)
        if pattern == "spiral":
            self._set(POUR_PATTERN, 1.0)
            self._set(POUR_SPIRAL_R, 5.0)
            self._set(POUR_SPIRAL_SPEED, 1.0)
        else:
            self._set(POUR_PATTERN, 0.0)

    def stop_pouring(self):
        self._set(POUR_ACTIVE, 0.0)

    def apply_pouring_force(self, solver, dt: float = 1.0) -> None:
        """Advance the nozzle one step (pour_time += dt, new position) and make `solver`'s next
        lattice steps apply its force (apply_pouring_force, :132-160).  Call once per step."""
        if solver not in self._solvers:
            self._solvers.append(solver)
        if solver._pour_ctl is not self.block:
            solver.set_pour_control(self.block)
        if self._dt != dt:  # a host write only when the step size changes (graph-capturable)
            self._set(POUR_DT, dt)
            self._dt = dt
        _lib.check(self.lib.pog_pour_advance(solver._p, _lib.stream_handle()))

    def apply_gradual_phase_change(self, multiphase, solid=None, dt: float = 1.0) -> None:
        """Turn the stream's cells toward water in a phase field (apply_gradual_phase_change,
        :166-193): multiphase is a MultiphaseFlow3D (or its phi tensor, with the solver as
        `solid`); non-solid cells of the stream change by clamp((1 - phi)/0.05, +-2) * intensity
        * dt * flow_rate."""
        if hasattr(multiphase, "phi_changed"):
            phi, solver = multiphase.phi, multiphase.lbm
        else:
            phi, solver = multiphase, solid
        if solver is None or not hasattr(solver, "_flags"):
            raise ValueError("apply_gradual_phase_change needs the solver (for its solid cells)")
        p = self.lattice.to_c()
        p.pour_control = self.block.data_ptr()
        _lib.check(self.lib.pog_pour_phase(p, _lib.ptr(solver._flags), _lib.ptr(phi), float(dt),
                                           _lib.stream_handle()))
        if hasattr(multiphase, "phi_changed"):
            multiphase.phi_changed()

    def create_water_impact_force(self, particle_system=None, max_force: float = 1.0, dt: float = 1.0) -> None:
        """Let the stream push the particles near it in the next coupling passes
        (create_water_impact_force, :190-226): strength 10 * flow_rate, |F| <= max_force."""
        self._set(POUR_IMPACT, 10.0 * self._get(POUR_FLOW))
        self._set(POUR_IMPACT_MAX, max_force)

    def adjust_flow_rate(self, new_rate: float) -> None:
        self._set(POUR_FLOW, max(0.1, min(3.0, float(new_rate))))
        if self._get(POUR_IMPACT) > 0:
            self._set(POUR_IMPACT, 10.0 * self._get(POUR_FLOW))

    def switch_to_spiral_pour(self, radius: float = 10.0, speed: float = 1.0) -> None:
        if self._get(POUR_ACTIVE) != 0.0:
            self._set(POUR_PATTERN, 1.0)
            self._set(POUR_SPIRAL_R, radius)
            self._set(POUR_SPIRAL_SPEED, speed)

    def move_pour_center(self, new_x: float, new_y: float) -> None:
        self._set(POUR_CX, max(5, min(self.lattice.nx - 5, new_x)))
        self._set(POUR_CY, max(5, min(self.lattice.ny - 5, new_y)))

    def get_pouring_info(self) -> dict:
        b = self.block.cpu().tolist()
        if b[POUR_ACTIVE] == 0.0:
            return {"active": False, "position": (0, 0), "diameter_grid": 0, "velocity": 0, "flow_rate": 0,
                    "pour_time": 0, "pattern": 0}
        return {"active": True, "position": (b[POUR_X], b[POUR_Y]), "diameter_grid": self.POUR_DIAMETER_GRID,
                "velocity": self.POUR_VELOCITY, "flow_rate": b[POUR_FLOW], "pour_time": b[POUR_TIME],
                "pattern": int(b[POUR_PATTERN])}

    def get_current_flow_rate(self) -> float:
        """Volume flow of the stream in lattice units (lu^3/step)."""
        b = self.block.cpu().tolist()
        if b[POUR_ACTIVE] == 0.0:
            return 0.0
        area = math.pi * (self.POUR_DIAMETER_GRID / 2.0) ** 2
        return b[POUR_FLOW] * self.POUR_VELOCITY * area

    def get_pouring_diagnostics(self) -> dict:
        """Configuration, state and the number of cells inside the stream cylinder at the lattice
        centre (_check_pouring_conditions, :300-338)."""
        r = self.POUR_DIAMETER_GRID / 2.0
        cx, cy = self.lattice.nx // 2, self.lattice.ny // 2
        z0, z1 = self.POUR_HEIGHT - self.POUR_STREAM_HEIGHT, self.POUR_HEIGHT
        cells = 0
        for i in range(max(0, int(cx - r)), min(self.lattice.nx, int(cx + r + 1))):
            for j in range(max(0, int(cy - r)), min(self.lattice.ny, int(cy + r + 1))):
                if (i - cx) ** 2 + (j - cy) ** 2 <= r * r:
                    cells += sum(1 for k in range(max(0, int(z0)), min(self.lattice.nz, int(z1) + 1))
                                 if z0 <= k <= z1)
        return {"configuration": {"diameter_grid": self.POUR_DIAMETER_GRID, "height": self.POUR_HEIGHT,
                                  "velocity": self.POUR_VELOCITY},
                "current_state": self.get_pouring_info(),
                "conditions_check": {"affected_cells": cells, "z_range": [z0, z1]}}
