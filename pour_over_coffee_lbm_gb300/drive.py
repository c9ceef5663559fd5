"""PressureGradientDrive on libpog.so: the pressure drive of src/physics/pressure_gradient_drive.py.

Same surface as the reference class (activate_density_drive / activate_force_drive /
activate_mixed_drive, apply(step), initialize_target_density, compute_pressure_gradient,
get_statistics, get_status, check_enhanced_stability, get_enhanced_diagnostics).

* force drive: F = -c_s^2 grad(rho) / rho, capped at MAX_PRESSURE_FORCE, is added to the solver's
  explicit force field, which the next step applies with Guo forcing (pog_pressure_force; the
  mixed drive adds 0.5 F).
* density drive: rho relaxes toward a per-plane target (high at the top, low at the bottom) by
  ADJUSTMENT_RATE, at most 0.001 a call (pog_density_drive).  As in the reference, this rewrites
  the macroscopic rho field only: the next step recomputes rho from the distributions, so it shows
  in the statistics, not in the flow.
"""
from typing import Any, Dict

import numpy as np
import torch

from . import _lib
from .params import CELL_SOLID

CS2 = 1.0 / 3.0


class PressureGradientDrive:
    def __init__(self, lbm_solver: Any):
        if not torch.cuda.is_available():
            raise RuntimeError("PressureGradientDrive needs a CUDA device")
        self.lib = _lib.load()
        self.lbm = lbm_solver
        self.HIGH_PRESSURE_RATIO = 1.8
        self.LOW_PRESSURE_RATIO = 0.4
        self.HIGH_PRESSURE_ZONE = 0.8
        self.LOW_PRESSURE_ZONE = 0.2
        self.ADJUSTMENT_RATE = 0.025
        self.MAX_PRESSURE_FORCE = 0.12
        self.GRADIENT_SMOOTHING = 0.1
        self.density_drive_active = 0
        self.force_drive_active = 0
        self.mixed_drive_active = 0
        self.pressure_force = torch.zeros_like(lbm_solver._force)
        self.pressure_stats = np.zeros(10, np.float32)
        self.target_density = None
        self.initialize_target_density()

    # ---- set-up ------------------------------------------------------------------------------
    def initialize_target_density(self) -> None:
        """Per-plane target (initialize_target_density :54-72) in float32; the constant
        sub-expressions of the parameters are formed in float64 first, as a traced kernel
        folds them."""
        nz = self.lbm.NZ
        f32 = np.float32
        HZ, LZ, HR, LR = self.HIGH_PRESSURE_ZONE, self.LOW_PRESSURE_ZONE, self.HIGH_PRESSURE_RATIO, self.LOW_PRESSURE_RATIO
        z = np.arange(nz, dtype=f32) / f32(nz)
        t = np.ones(nz, f32)
        hi = z >= f32(HZ)
        t[hi] = f32(1) + (z[hi] - f32(HZ)) / f32(1.0 - HZ) * f32(HR - 1.0)
        lo = (~hi) & (z <= f32(LZ))
        t[lo] = f32(LR) + z[lo] / f32(LZ) * f32(1.0 - LR)
        self.target_profile = t
        self._target = torch.as_tensor(t).to(self.lbm.device)
        self.target_density = self._target.view(nz, 1, 1).expand(nz, self.lbm.NY, self.lbm.NX)

    def activate_density_drive(self, enable: bool = True) -> None:
        self.density_drive_active, self.force_drive_active, self.mixed_drive_active = int(bool(enable)), 0, 0

    def activate_force_drive(self, enable: bool = True) -> None:
        self.density_drive_active, self.force_drive_active, self.mixed_drive_active = 0, int(bool(enable)), 0

    def activate_mixed_drive(self, enable: bool = True) -> None:
        self.density_drive_active, self.force_drive_active, self.mixed_drive_active = 0, 0, int(bool(enable))

    # ---- device passes -----------------------------------------------------------------------
    def apply_density_drive(self, rate_scale: float = 1.0, max_adjust: float = 0.001,
                            rho_min: float = 0.5, rho_max: float = 2.0) -> None:
        s = self.lbm
        rho = s._current_rho()
        _lib.check(self.lib.pog_density_drive(s._p, _lib.ptr(s._flags), _lib.ptr(rho), _lib.ptr(self._target),
                                              self.ADJUSTMENT_RATE * rate_scale, max_adjust, rho_min, rho_max,
                                              _lib.stream_handle()))
        s._rho_external = True

    def compute_pressure_gradient(self) -> None:
        """pressure_force := capped -c_s^2 grad(rho) / rho on the non-solid cells."""
        s = self.lbm
        self.pressure_force.zero_()
        _lib.check(self.lib.pog_pressure_force(s._p, _lib.ptr(s._flags), _lib.ptr(s._current_rho()),
                                               _lib.ptr(self.pressure_force), 1.0, self.MAX_PRESSURE_FORCE,
                                               _lib.stream_handle()))

    def _accumulate(self, scale: float) -> None:
        s = self.lbm
        _lib.check(self.lib.pog_pressure_force(s._p, _lib.ptr(s._flags), _lib.ptr(s._current_rho()),
                                               _lib.ptr(s._force), scale, self.MAX_PRESSURE_FORCE,
                                               _lib.stream_handle()))
        s._force_written()

    def apply_force_drive(self) -> None:
        if self.force_drive_active:
            self._accumulate(1.0)

    def apply_mixed_drive(self) -> None:
        if self.mixed_drive_active:
            self._accumulate(0.5)

    def apply(self, step: int = 0) -> None:
        """The drive of one step (apply :257-272): the density drive, then the force drive or
        the mixed drive's half force, added to the solver's body force."""
        if self.density_drive_active:
            self.apply_density_drive()
        if self.force_drive_active:
            self._accumulate(1.0)
            return
        if self.mixed_drive_active:
            self._accumulate(0.5)

    # ---- statistics --------------------------------------------------------------------------
    def _fluid(self):
        return (self.lbm._flags & CELL_SOLID) == 0

    def compute_statistics(self) -> None:
        rho = self.lbm.rho.tensor[self._fluid()].double()
        if rho.numel() == 0:
            self.pressure_stats[:4] = (0.0, 999.0, 0.0, -999.0)
            return
        p = rho * CS2
        mx, mn, av = p.max().item(), p.min().item(), p.mean().item()
        self.pressure_stats[:4] = (mx, mn, av, mx - mn)

    def get_statistics(self) -> Dict[str, float]:
        self.compute_statistics()
        st = self.pressure_stats
        return {"max_pressure": float(st[0]), "min_pressure": float(st[1]), "avg_pressure": float(st[2]),
                "pressure_drop": float(st[3]), "pressure_ratio": float(st[0] / st[1]) if st[1] > 0 else 0}

    def get_status(self) -> Dict[str, bool]:
        return {"density_drive": bool(self.density_drive_active), "force_drive": bool(self.force_drive_active),
                "mixed_drive": bool(self.mixed_drive_active)}

    def check_enhanced_stability(self) -> int:
        """0 stable, 1 velocity warning, 2 density warning, 3 unstable (:326-372)."""
        fl = self._fluid()
        rho = self.lbm.rho.tensor[fl].double()
        um = self.lbm.u.tensor.double().norm(dim=0)[fl]
        vmax = um.max().item() if um.numel() else 0.0
        dmin = rho.min().item() if rho.numel() else 999.0
        dmax = rho.max().item() if rho.numel() else 0.0
        bad = int(((rho <= 0) | (rho > 100) | (um > 1.0) | ~torch.isfinite(rho) | ~torch.isfinite(um)).sum().item())
        self.pressure_stats[4:8] = (vmax, dmin, dmax, bad)
        if bad > 0 or vmax > 0.12 or dmin < 0.0005 or dmax > 8.0:
            return 3
        if dmin < 0.001 or dmax > 6.0:
            return 2
        if vmax > 0.08:
            return 1
        return 0

    def get_enhanced_diagnostics(self) -> Dict[str, Any]:
        code = self.check_enhanced_stability()
        st = self.pressure_stats
        return {"stability_code": code,
                "stability_status": {0: "stable", 1: "velocity warning", 2: "density warning", 3: "unstable"}[code],
                "max_velocity": float(st[4]), "density_range": [float(st[5]), float(st[6])],
                "invalid_count": int(st[7]), "enhancement_level": "MEDIUM",
                "pressure_ratio_range": "%.1f - %.1f" % (self.LOW_PRESSURE_RATIO, self.HIGH_PRESSURE_RATIO),
                "max_force": self.MAX_PRESSURE_FORCE}
