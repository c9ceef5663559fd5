"""FilterPaperSystem on libpog.so: the filter-paper dynamics of src/physics/filter_paper.py:616-840.

The paper is the solver's porous band (CELL_POROUS flags).  Its Darcy/Forchheimer resistance
is applied inside the fused lattice step (apply_filter_effects, :539-615, is therefore a no-op
here); this class owns the two fields the reference adds on top of it:

* accumulated_particles -- deposits of the particles that met the paper
  (block_particles_at_filter, :616-700: a particle moving down within two planes of a paper
  cell bounces with restitution 0.3, gets a horizontal roughness kick and leaves 0.01 there);
* filter_blockage -- b = 0.95 b + 0.05 * 0.9 (1 - exp(-0.1 a)), with a decaying by 0.999 a step
  (update_dynamic_resistance, :702-746).  The step kernel scales the band's Darcy and
  Forchheimer coefficients by (1 + b), the reference's blockage_factor (:586-588).

The reference draws the roughness kicks from ti.random(); here they come from a counter hash
of (seed, step, particle), so a run repeats bit for bit and a CUDA graph may replay it.
"""
import math
from typing import Any, Dict, Optional

import torch

from . import _lib
from .params import CELL_POROUS, CELL_SOLID


class FilterPaperSystem:
    def __init__(self, lbm_solver: Any, seed: int = 0x5EED):
        if not torch.cuda.is_available():
            raise RuntimeError("FilterPaperSystem needs a CUDA device")
        self.lib = _lib.load()
        self.lbm = lbm_solver
        self.seed = int(seed) & 0xFFFFFFFF
        self.step_count = 0
        n = lbm_solver.n
        dev = lbm_solver._flags.device
        self.accumulated_particles = torch.zeros(n, dtype=torch.float32, device=dev)
        self.filter_blockage = torch.zeros(n, dtype=torch.float32, device=dev)
        self.initialize_filter_geometry()

    # ---- reference surface -------------------------------------------------------------------
    def initialize_filter_geometry(self) -> None:
        """The paper cells are the solver's porous band; start unblocked and attach the blockage
        field to the solver's step (and to the boundary manager, as the reference does)."""
        self.accumulated_particles.zero_()
        self.filter_blockage.zero_()
        self.lbm.set_filter_blockage(self.filter_blockage)
        bm = getattr(self.lbm, "boundary_manager", None)
        if bm is not None and hasattr(bm, "set_filter_system"):
            bm.set_filter_system(self)

    def apply_filter_effects(self) -> None:
        """The band resistance (with the blockage factor) is part of every lattice step."""
        return None

    def block_particles_at_filter(self, particle_system) -> None:
        n = int(particle_system.count)
        if n == 0:
            return
        s = self.lbm
        _lib.check(self.lib.pog_filter_particles(
            s._p, _lib.ptr(s._flags), _lib.ptr(particle_system._pos), _lib.ptr(particle_system._vel),
            _lib.ptr(particle_system._active), n, _lib.ptr(self.accumulated_particles), self.seed, self.step_count,
            _lib.stream_handle()))

    def update_dynamic_resistance(self) -> None:
        s = self.lbm
        _lib.check(self.lib.pog_filter_update(s._p, _lib.ptr(s._flags), _lib.ptr(self.accumulated_particles),
                                              _lib.ptr(self.filter_blockage), _lib.stream_handle()))

    def step(self, particle_system: Optional[Any] = None) -> None:
        """filter_paper.py:748-790: resistance (in the lattice step), particle bounce, blockage."""
        self.apply_filter_effects()
        if particle_system is not None:
            self.block_particles_at_filter(particle_system)
        self.update_dynamic_resistance()
        self.step_count += 1

    def get_filter_statistics(self) -> Dict[str, Any]:
        """Same keys as the reference (:793-839).  average_resistance is the band's lattice Darcy
        coefficient nu/K times (1 + b), averaged over the paper cells (the reference reports its
        own precomputed mu L / K there); average_flow_rate is the mean |u| over them."""
        s = self.lbm
        fl = s._flags.reshape(-1)
        zone = ((fl & CELL_POROUS) != 0) & ((fl & CELL_SOLID) == 0)
        total = int(zone.sum().item())
        if total == 0:
            return {"total_filter_nodes": 0, "average_resistance": 0.0, "average_blockage": 0.0,
                    "average_flow_rate": 0.0, "max_blockage": 0.0}
        b = self.filter_blockage[zone].double()
        cfg = s.cfg
        nu = (cfg.tau - 0.5) / 3.0
        if s._porosity is not None:
            e = s._porosity.reshape(-1)[zone].double()
            g = e ** 3 / (1 - e) ** 2
            g0 = cfg.porosity ** 3 / (1 - cfg.porosity) ** 2
            K = cfg.permeability * g / g0
        else:
            K = torch.full_like(b, cfg.permeability)
        res = (nu / K) * (1.0 + b)
        u = s.u.tensor.reshape(3, -1)[:, zone].double()
        return {"total_filter_nodes": total, "average_resistance": float(res.mean().item()),
                "average_blockage": float(b.mean().item() * 100.0),
                "average_flow_rate": float(u.norm(dim=0).mean().item()),
                "max_blockage": float(self.filter_blockage.max().item() * 100.0)}

    def get_coffee_bed_boundary(self) -> Dict[str, Any]:
        """Cone geometry in lattice units (:856-895): the paper's inner radius grows linearly
        from 0 at the cone apex to the rim at the inlet plane nz - 2."""
        g = self.lbm.cfg
        tan_t = math.tan(math.radians(g.cone_half_angle_deg))
        bottom, top = float(g.cone_apex_z), float(g.nz - 2)

        def radius_at(z: float) -> float:
            return max(min(float(z), top) - bottom, 0.0) * tan_t

        return {"center_x": float(g.center_x) if g.center_x >= 0 else 0.5 * g.nx,
                "center_y": float(g.center_y) if g.center_y >= 0 else 0.5 * g.ny,
                "bottom_z": bottom, "top_z": top, "top_radius_lu": radius_at(top), "bottom_radius_lu": 0.0,
                "get_radius_at_height": radius_at}

    def get_filter_inner_radius_at_height(self, z: float) -> float:
        return self.get_coffee_bed_boundary()["get_radius_at_height"](z)

    def print_status(self) -> None:
        st = self.get_filter_statistics()
        print("filter paper: %d nodes, blockage avg %.3f%% max %.3f%%, resistance %.4g, |u| %.4g"
              % (st["total_filter_nodes"], st["average_blockage"], st["max_blockage"], st["average_resistance"],
                 st["average_flow_rate"]))

