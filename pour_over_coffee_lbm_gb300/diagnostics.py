"""LBMDiagnostics on libpog.so: the reference's diagnostics (src/visualization/lbm_diagnostics.py:
33-490) from one device reduction per check, plus asynchronous field snapshots
(main.py:1187-1205 `_save_basic_snapshot`: density and |u| as .npy) and a raw checkpoint/resume
of a run.

The reference computes every statistic with numpy on full `to_numpy()` copies of rho and u (two
field transfers per check, plus a host copy of both as `prev`).  Here pog_field_stats reduces
rho and u on the device to POG_STAT_COUNT doubles and the per-plane density profile; `prev` stays
on the device; only the small vectors come back.  Method names and dict keys follow the
reference so callers read the same reports.  Lengths, velocities and times are in lattice units
unless `scale_length`, `scale_velocity` and `dt` are set to the reference's config scales, which
reproduce its physical-unit reports.
"""
import math
import os
import threading
import time
from typing import Optional

import numpy as np
import torch

from . import _lib

STAT_MASS, STAT_RHO2, STAT_MOMX, STAT_UMAX, STAT_UACT_SUM, STAT_UACT_N = 0, 1, 2, 5, 6, 7
STAT_U2, STAT_UABS, STAT_MACH_N, STAT_DRHO_MAX, STAT_DRHO2, STAT_DU2 = 8, 9, 10, 11, 12, 13
STAT_USUM, STAT_USQ, STAT_UREG, STAT_COUNT = 14, 17, 20, 23


def field_stats(solver, prev=None) -> tuple:
    """(stats [STAT_COUNT] float64 numpy, z-profile [nz] of per-plane rho sums) of the solver's
    current rho/u; prev = (rho_prev, u_prev) device tensors or None."""
    solver._refresh_macro()
    dev = solver.device
    st = torch.empty(STAT_COUNT, dtype=torch.float64, device=dev)
    zp = torch.empty(solver.NZ, dtype=torch.float64, device=dev)
    rp, up = (None, None) if prev is None else prev
    _lib.check(solver.lib.pog_field_stats(solver._p, _lib.ptr(solver._rho), _lib.ptr(solver._u), _lib.ptr(rp),
                                          _lib.ptr(up), _lib.ptr(st), _lib.ptr(zp), _lib.stream_handle()))
    return st.cpu().numpy(), zp.cpu().numpy()


class LBMDiagnostics:
    def __init__(self, lbm_solver, multiphase=None, particles=None, pouring=None, filter_system=None):
        self.lbm = lbm_solver
        self.multiphase = multiphase
        self.particles = particles
        self.pouring = pouring
        self.filter = filter_system
        self.history = []
        self.light_monitoring_freq, self.medium_monitoring_freq, self.heavy_monitoring_freq = 5, 10, 100
        self.prev = None  # device (rho, u) of the previous check
        self.prev_momentum = np.zeros(3)
        self.initial_mass = 0.0
        self.accumulated_inflow = 0.0
        self.reference_density = 1.0
        # lattice units by default; the reference's config.DT, SCALE_LENGTH and SCALE_VELOCITY
        # (1.0, 0.000625 m, 0.01) reproduce its reports in physical units
        self.dt = 1.0
        self.scale_length = 1.0
        self.scale_velocity = 1.0
        self.prev_phi = None  # device copy of the phase field at the previous check
        self.calculation_times = {"light": [], "medium": [], "heavy": []}
        self._stats = None
        self._zp = None

    # ---- one reduction per check ------------------------------------------------------------
    def _fetch(self):
        self._stats, self._zp = field_stats(self.lbm, self.prev)
        return self._stats

    def adaptive_monitoring_frequency(self, step_num: int) -> None:
        if step_num < 100:
            self.light_monitoring_freq, self.medium_monitoring_freq = 2, 5
        elif step_num < 500:
            self.light_monitoring_freq, self.medium_monitoring_freq = 5, 10
        else:
            self.light_monitoring_freq, self.medium_monitoring_freq = 10, 20

    def update_diagnostics(self, step_num: int, simulation_time: float, force_update: bool = False) -> dict:
        """lbm_diagnostics.py:85-149."""
        self.adaptive_monitoring_frequency(step_num)
        d = {"step": step_num, "time": simulation_time, "timestamp": time.time()}
        light = step_num % self.light_monitoring_freq == 0 or force_update
        medium = step_num % self.medium_monitoring_freq == 0 or force_update
        heavy = step_num % self.heavy_monitoring_freq == 0 or force_update
        if light or medium or heavy:
            self._fetch()
        if light:
            t0 = time.time()
            d["temporal_stability"] = self.calculate_temporal_stability(refresh=False)
            d["lbm_quality"] = self.analyze_lbm_numerical_quality(refresh=False)
            self.calculation_times["light"].append(time.time() - t0)
        if medium:
            t0 = time.time()
            d["conservation"] = self.check_conservation_laws(refresh=False)
            d["multiphase"] = self.analyze_multiphase_quality()
            self.calculation_times["medium"].append(time.time() - t0)
        if heavy:
            t0 = time.time()
            d["v60_physics"] = self.track_v60_physics(refresh=False)
            d["flow_analysis"] = self.detailed_flow_analysis(refresh=False)
            d["diagnostics_performance"] = self.get_performance_stats()
            self.calculation_times["heavy"].append(time.time() - t0)
        self.history.append((simulation_time, d))
        self._update_previous_step_data()
        return d

    def _s(self, refresh: bool):
        return self._fetch() if (refresh or self._stats is None) else self._stats

    def calculate_temporal_stability(self, refresh: bool = True) -> dict:
        """lbm_diagnostics.py:151-186: norms of the change since the previous check."""
        st = self._s(refresh)
        if self.prev is None:
            return {"status": "first_step"}
        rho_norm = math.sqrt(st[STAT_RHO2])
        u_norm = math.sqrt(st[STAT_U2])
        rho_change, u_change = math.sqrt(st[STAT_DRHO2]), math.sqrt(st[STAT_DU2])
        out = {"density_change_rate": rho_change / self.dt, "relative_density_change": rho_change / rho_norm,
               "velocity_change_rate": u_change / self.dt, "relative_velocity_change": u_change / (u_norm + 1e-10)}
        if out["relative_density_change"] < 1e-6 and out["relative_velocity_change"] < 1e-4:
            out["stability_grade"] = "Excellent"
        elif out["relative_density_change"] < 1e-4 and out["relative_velocity_change"] < 1e-2:
            out["stability_grade"] = "Good"
        else:
            out["stability_grade"] = "Monitoring"
        return out

    def analyze_lbm_numerical_quality(self, refresh: bool = True) -> dict:
        """lbm_diagnostics.py:188-226: Mach numbers and density deviation."""
        st = self._s(refresh)
        n = self.lbm.n
        cs = 1.0 / math.sqrt(3.0)
        mean_rho = st[STAT_MASS] / n
        var = max(st[STAT_RHO2] / n - mean_rho * mean_rho, 0.0)
        q = {"max_mach": st[STAT_UMAX] / cs,
             "mean_mach": (st[STAT_UACT_SUM] / st[STAT_UACT_N]) / cs if st[STAT_UACT_N] > 0 else 0.0,
             "mach_violation_ratio": st[STAT_MACH_N] / n,
             "max_density_deviation": st[STAT_DRHO_MAX], "mean_density": mean_rho,
             "density_variation_coeff": math.sqrt(var) / mean_rho}
        if q["max_mach"] < 0.1 and q["max_density_deviation"] < 0.1:
            q["lbm_grade"] = "Excellent"
        elif q["max_mach"] < 0.2 and q["max_density_deviation"] < 0.2:
            q["lbm_grade"] = "Good"
        else:
            q["lbm_grade"] = "Caution"
        return q

    def check_conservation_laws(self, refresh: bool = True) -> dict:
        """lbm_diagnostics.py:228-291: open-system mass balance and the gravity momentum budget."""
        st = self._s(refresh)
        mass = st[STAT_MASS]
        if self.initial_mass == 0.0:
            self.initial_mass = mass
        if self.pouring is not None and hasattr(self.pouring, "get_current_flow_rate"):
            self.accumulated_inflow += self.pouring.get_current_flow_rate() * self.dt
        expected = self.initial_mass + self.accumulated_inflow
        err = abs(mass - expected)
        mom = np.array(st[STAT_MOMX:STAT_MOMX + 3])
        dmom = mom - self.prev_momentum
        g = abs(self.lbm.cfg.gravity[2])
        grav = g * mass * self.dt
        c = {"total_mass": mass, "initial_mass": self.initial_mass, "accumulated_inflow": self.accumulated_inflow,
             "mass_conservation_error": err, "relative_mass_error": err / self.initial_mass,
             "total_momentum": mom.tolist(), "momentum_z_change": float(dmom[2]),
             "expected_gravity_change": grav, "momentum_conservation_error": abs(dmom[2] - grav)}
        c["conservation_grade"] = ("Excellent" if c["relative_mass_error"] < 1e-6 else
                                   "Good" if c["relative_mass_error"] < 1e-4 else "Moderate")
        self.prev_momentum = mom
        return c

    def track_v60_physics(self, refresh: bool = True) -> dict:
        """lbm_diagnostics.py:328-370: wetting front from the plane-mean density, water volume,
        inlet/outlet flow."""
        st = self._s(refresh)
        plane_mean = self._zp / float(self.lbm.NX * self.lbm.NY)
        wet = np.where(plane_mean > self.reference_density + 0.1)[0]
        L = self.scale_length
        inlet = 0.0
        if self.pouring is not None and hasattr(self.pouring, "get_current_flow_rate"):
            inlet = float(self.pouring.get_current_flow_rate())
        phys = {"wetting_front_position": float(wet.max()) * L if wet.size else 0.0,
                "system_water_volume": max(0.0, (st[STAT_MASS] - self.reference_density * self.lbm.n) * L ** 3),
                "inlet_flow_rate": inlet, "outlet_flow_rate": self._estimate_outlet_flow()}
        if self.particles is not None:
            phys["particle_dynamics"] = self._analyze_coffee_bed_dynamics()
        return phys

    def _estimate_outlet_flow(self) -> float:
        """lbm_diagnostics.py:439-452: the downward z velocity summed over the five bottom planes,
        times scale_velocity * scale_length^2; reduced on the device."""
        uz = self.lbm._u[2, :5]
        down = torch.clamp(-uz, min=0.0).double().sum().item()
        return float(down * self.scale_velocity * self.scale_length ** 2)

    def _analyze_coffee_bed_dynamics(self) -> dict:
        """lbm_diagnostics.py:409-437: height and radial spread of the active particles (the
        reference's numpy arithmetic on host copies of the particle arrays)."""
        p = self.particles
        if not hasattr(p, "position") or not hasattr(p, "active"):
            return {"status": "no_particle_data"}
        pos = p.position.to_numpy()
        act = p.active.to_numpy()
        ap = pos[act == 1]
        if len(ap) == 0:
            return {"status": "no_active_particles"}
        L = self.scale_length
        z = ap[:, 2]
        d = {"active_particle_count": len(ap), "bed_height_mean": float(np.mean(z) * L),
             "bed_height_std": float(np.std(z) * L),
             "bed_height_range": [float(np.min(z) * L), float(np.max(z) * L)]}
        cx, cy = self.lbm.NX * 0.5, self.lbm.NY * 0.5
        r = np.sqrt((ap[:, 0] - cx) ** 2 + (ap[:, 1] - cy) ** 2)
        d["radial_distribution_mean"] = float(np.mean(r) * L)
        d["radial_distribution_std"] = float(np.std(r) * L)
        return d

    def _phi(self) -> Optional[torch.Tensor]:
        """The multiphase object's phase field as a device tensor (a tensor, a FieldView, or any
        field with to_numpy)."""
        phi = getattr(self.multiphase, "phi", None) if self.multiphase is not None else None
        if phi is None:
            return None
        if isinstance(phi, torch.Tensor):
            return phi
        t = getattr(phi, "tensor", None)
        if isinstance(t, torch.Tensor):
            return t
        return torch.as_tensor(np.asarray(phi.to_numpy()), device=self.lbm.device)

    def analyze_multiphase_quality(self) -> dict:
        """lbm_diagnostics.py:293-326: interface cells (0.1 < phi < 0.9), water fraction and the
        change of phi since the previous check, reduced on the device."""
        phi = self._phi()
        if phi is None:
            return {"status": "no_multiphase"}
        a = {"interface_thickness": int(((phi > 0.1) & (phi < 0.9)).sum().item()),
             "water_fraction": float(phi.double().mean().item())}
        if self.prev_phi is not None:
            change = torch.linalg.vector_norm((phi - self.prev_phi).double()).item()
            a["phase_change_rate"] = float(change / self.dt)
        else:
            a["phase_change_rate"] = 0.0
        r = a["phase_change_rate"]
        a["phase_stability_grade"] = "Excellent" if r < 1e-6 else ("Good" if r < 1e-4 else "Dynamic")
        return a

    def detailed_flow_analysis(self, refresh: bool = True) -> dict:
        """lbm_diagnostics.py:372-407: |u| statistics, per-component spread, region means."""
        st = self._s(refresh)
        n = self.lbm.n
        mean_abs = st[STAT_UABS] / n
        comp_std = [math.sqrt(max(st[STAT_USQ + a] / n - (st[STAT_USUM + a] / n) ** 2, 0.0)) for a in range(3)]
        nz, plane = self.lbm.NZ, self.lbm.NX * self.lbm.NY
        z30, z80 = int(nz * 0.3), int(nz * 0.8)
        counts = [z30 * plane, (z80 - z30) * plane, (nz - z80) * plane]
        return {"max_velocity": st[STAT_UMAX],
                "mean_velocity": st[STAT_UACT_SUM] / st[STAT_UACT_N] if st[STAT_UACT_N] > 0 else 0.0,
                "velocity_std": math.sqrt(max(st[STAT_U2] / n - mean_abs * mean_abs, 0.0)),
                "flow_complexity": float(np.linalg.norm(comp_std)),
                "top_region_flow": st[STAT_UREG + 2] / counts[2] if counts[2] else 0.0,
                "middle_region_flow": st[STAT_UREG + 1] / counts[1] if counts[1] else 0.0,
                "bottom_region_flow": st[STAT_UREG] / counts[0] if counts[0] else 0.0}

    def _update_previous_step_data(self) -> None:
        if self.prev is None:
            self.prev = (self.lbm._rho.clone(), self.lbm._u.clone())
        else:
            self.prev[0].copy_(self.lbm._rho)
            self.prev[1].copy_(self.lbm._u)
        phi = self._phi()
        if phi is not None:
            if self.prev_phi is None or self.prev_phi.shape != phi.shape:
                self.prev_phi = phi.clone()
            else:
                self.prev_phi.copy_(phi)

    def get_performance_stats(self) -> dict:
        out = {}
        for k, v in self.calculation_times.items():
            out[k + "_calc_count"] = len(v)
            out[k + "_avg_time"] = float(np.mean(v)) if v else 0.0
            out[k + "_total_time"] = float(np.sum(v)) if v else 0.0
        return out


class SnapshotWriter:
    """Field snapshots written without stalling the step loop (main.py:1187-1205 saves
    `<base>_density_data.npy` and `<base>_velocity_data.npy` = |u|): |u| is formed on the
    device, both fields are copied into pinned host buffers on a side stream, and a background
    thread writes the files once the copy has finished."""

    def __init__(self, solver):
        self.solver = solver
        shape = (solver.NX, solver.NY, solver.NZ)
        self._rho = torch.empty(shape, dtype=torch.float32).pin_memory()
        self._umag = torch.empty(shape, dtype=torch.float32).pin_memory()
        self._stream = torch.cuda.Stream()
        self._thread: Optional[threading.Thread] = None

    def save(self, filename_base: str) -> None:
        self.wait()
        s = self.solver
        s._refresh_macro()
        umag = torch.sqrt((s._u * s._u).sum(0))
        rho = s._rho
        self._stream.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(self._stream):
            # (NZ, NY, NX) device layout -> the reference's (NX, NY, NZ) arrays
            self._rho.copy_(rho.permute(2, 1, 0), non_blocking=True)
            self._umag.copy_(umag.permute(2, 1, 0), non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(self._stream)
        rho.record_stream(self._stream)
        umag.record_stream(self._stream)

        def write():
            ev.synchronize()
            np.save(filename_base + "_density_data.npy", self._rho.numpy())
            np.save(filename_base + "_velocity_data.npy", self._umag.numpy())

        self._thread = threading.Thread(target=write, daemon=True)
        self._thread.start()

    def wait(self) -> None:
        if self._thread is not None:
            self._thread.join()
            self._thread = None


# Physical scales of the reference's config, used only for the export's metadata
# (config/core.py:59-81: 14 cm over 224 planes, 0.01 lu/ts, time factor 1.2;
# config/physics.py:42,69,107-111: V60 height, 2 cm/s, water at 90 C).
EXPORT_SCALES = {"scale_length": 0.14 / 224, "scale_velocity": 0.01, "time_factor": 1.2,
                 "l_char": 0.085, "u_char": 0.02, "nu_char": 3.15e-7}


def export_data_for_analysis(lbm, simulation_time, step_num, particles=None, filter_system=None,
                             out_dir: str = ".", scales: Optional[dict] = None) -> list:
    """The reference's analysis export (src/visualization/enhanced_visualizer.py:1487-1560):
    `cfd_data_export_step_NNNN.json` with the velocity, density and pressure fields (ρ c_s^2),
    the active particles, the filter statistics and the run's metadata, and
    `cfd_data_export_step_NNNN.npz` with the entries that are arrays (density and pressure, float64,
    indexed (NX, NY, NZ)).  The Reynolds number of the metadata follows
    calculate_flow_characteristics (:450-471): mean physical |u| over |u| > 1e-6 m/s (u_char when
    none) times l_char over nu_char.  Returns the two paths, or [] after a failure, which is
    printed, as the reference does."""
    import json
    sc = dict(EXPORT_SCALES, **(scales or {}))
    try:
        export = {}
        if hasattr(lbm, "u") and hasattr(lbm, "rho"):
            u = lbm.u.to_numpy()
            rho = lbm.rho.to_numpy()
            export["velocity_field"] = {"u_x": u[..., 0].tolist(), "u_y": u[..., 1].tolist(),
                                        "u_z": u[..., 2].tolist(),
                                        "magnitude": np.sqrt(np.sum(u ** 2, axis=3)).tolist()}
            export["density_field"] = rho.tolist()
            export["pressure_field"] = (rho * (1.0 / 3.0)).tolist()
            umag = np.sqrt(u[..., 0] ** 2 + u[..., 1] ** 2 + u[..., 2] ** 2) * sc["scale_velocity"]
            act = umag[umag > 1e-6]
            uc = float(np.mean(act)) if act.size else sc["u_char"]
            reynolds = uc * sc["l_char"] / sc["nu_char"] if uc > 0 and sc["nu_char"] > 0 else 0.0
        else:
            reynolds = 0
        if particles is not None:
            pos = particles.position.to_numpy()
            vel = particles.velocity.to_numpy()
            active = particles.active.to_numpy()
            export["particles"] = {"positions": pos[active == 1].tolist(),
                                   "velocities": vel[active == 1].tolist(),
                                   "count": int(np.sum(active))}
        if filter_system is not None:
            export["filter"] = filter_system.get_filter_statistics()
        nx, ny, nz = (int(lbm.NX), int(lbm.NY), int(lbm.NZ))
        export["metadata"] = {"simulation_time": simulation_time, "step_number": step_num,
                              "grid_size": [nx, ny, nz],
                              "physical_parameters": {
                                  "scale_length": sc["scale_length"],
                                  "scale_time": sc["scale_length"] / sc["scale_velocity"] * sc["time_factor"],
                                  "reynolds_number": float(reynolds)}}
        base = os.path.join(out_dir, "cfd_data_export_step_%04d" % step_num)
        json_file, numpy_file = base + ".json", base + ".npz"
        with open(json_file, "w") as f:
            json.dump(export, f, indent=2)
        np.savez_compressed(numpy_file, **{k: np.array(v) for k, v in export.items()
                                           if isinstance(v, (list, np.ndarray))})
        return [json_file, numpy_file]
    except Exception as e:  # the reference reports and carries on
        print("data export failed: %s" % e)
        return []


def save_checkpoint(path: str, solver, particles=None, pour=None, filter_system=None, multiphase=None) -> None:
    """Everything a run needs to continue bit for bit: the raw distribution buffer in its
    storage format, time index, flags, porosity, explicit force, LES velocity buffers, the phase
    indicator, and the particle, pour-nozzle, filter-paper and phase-field state."""
    s = solver
    d = {"t": np.int64(s.t), "step_count": np.int64(s.step_count), "storage": np.int32(s.cfg.storage),
         "shape": np.array([s.NX, s.NY, s.NZ], np.int64),
         "f": s._f.view(torch.uint8).cpu().numpy(), "flags": s._flags.cpu().numpy(),
         "force": s._force.cpu().numpy(), "force_active": np.int8(s._force_active),
         # rho/u as the last step left them (the moments the next coupling pass reads) and the
         # particle drag deposit of the last coupled step
         "rho": s._rho.cpu().numpy(), "u": s._u.cpu().numpy(), "macro_dirty": np.int8(s._macro_dirty),
         "u_stale": np.int8(s._u_stale),
         "pdrag": s._pdrag.cpu().numpy(), "pdrag_active": np.int8(s._pdrag_active),
         "phase": s._phase.cpu().numpy(), "rho_external": np.int8(s._rho_external),
         "deposit_mask": s._dmask.cpu().numpy()}
    if s._porosity is not None:
        d["porosity"] = s._porosity.cpu().numpy()
    if s._dref is not None:
        d["density_ref"] = s._dref.view(torch.int16).cpu().numpy()
    if s._ul is not None:
        d["u_les0"], d["u_les1"] = s._ul[0].cpu().numpy(), s._ul[1].cpu().numpy()
    if particles is not None:
        p = particles
        d.update({"p_count": np.int64(p.count), "p_pos": p._pos.cpu().numpy(), "p_vel": p._vel.cpu().numpy(),
                  "p_d": p._d.cpu().numpy(), "p_drag_old": p._drag_old.cpu().numpy(),
                  "p_active": p._active.cpu().numpy(), "p_perm": p._perm.cpu().numpy(),
                  "p_keys": p._keys.cpu().numpy(),
                  "p_since_sort": np.int64(-1 if p._since_sort is None else p._since_sort)})
    if pour is not None:
        d["pour"] = pour.block.cpu().numpy()
        d["pour_attached"] = np.int8(s._pour_ctl is pour.block)
    if multiphase is not None:
        m = multiphase
        d.update({"mp_phi": m.phi.cpu().numpy(), "mp_phi_new": m.phi_new.cpu().numpy(), "mp_mu": m.mu.cpu().numpy(),
                  "mp_mu_live": np.int8(m._mu_live)})
    if filter_system is not None:
        d.update({"filter_accum": filter_system.accumulated_particles.cpu().numpy(),
                  "filter_blockage": filter_system.filter_blockage.cpu().numpy(),
                  "filter_step": np.int64(filter_system.step_count), "filter_seed": np.int64(filter_system.seed)})
    tmp = path + ".tmp.npz"
    np.savez(tmp, **d)
    os.replace(tmp, path)


def load_checkpoint(path: str, solver, particles=None, pour=None, filter_system=None, multiphase=None) -> None:
    """Restore a save_checkpoint file into objects built with the same configuration."""
    s = solver
    z = np.load(path)
    if tuple(z["shape"]) != (s.NX, s.NY, s.NZ) or int(z["storage"]) != s.cfg.storage:
        raise ValueError("checkpoint grid/storage does not match the solver")
    if ("density_ref" in z) != (s._dref is not None):
        raise ValueError("checkpoint and solver differ in the FP16S reference-density form")
    s._f.view(torch.uint8).copy_(torch.from_numpy(z["f"]))
    if s._dref is not None:
        s._dref.view(torch.int16).copy_(torch.from_numpy(z["density_ref"]))
    s._flags.copy_(torch.from_numpy(z["flags"]))
    s._force.copy_(torch.from_numpy(z["force"]))
    s._force_active = bool(z["force_active"])
    if "porosity" in z:
        s.set_porosity(z["porosity"].transpose(2, 1, 0))
    if "u_les0" in z and s._ul is not None:
        s._ul[0].copy_(torch.from_numpy(z["u_les0"]))
        s._ul[1].copy_(torch.from_numpy(z["u_les1"]))
    s._rho.copy_(torch.from_numpy(z["rho"]))
    s._u.copy_(torch.from_numpy(z["u"]))
    s._pdrag.copy_(torch.from_numpy(z["pdrag"]))
    s._pdrag_owner = None
    if "deposit_mask" in z:
        s._dmask.copy_(torch.from_numpy(z["deposit_mask"]))
    else:  # every cell may hold a deposit
        s._dmask.fill_(-1)
    s._pdrag_active = bool(z["pdrag_active"])
    if "phase" in z:
        s._phase.copy_(torch.from_numpy(z["phase"]))
        s._rho_external = bool(z["rho_external"])
    if pour is not None and "pour" in z:
        pour.block.copy_(torch.from_numpy(z["pour"]))
        if "pour_attached" in z and bool(z["pour_attached"]):
            s.set_pour_control(pour.block)  # before the moments' state is restored below
    s.t = int(z["t"])
    s.step_count = int(z["step_count"])
    s._macro_dirty = bool(z["macro_dirty"])
    s._u_stale = bool(z["u_stale"]) if "u_stale" in z else False
    if particles is not None and "p_count" in z:
        p = particles
        p.count = int(z["p_count"])
        for name in ("pos", "vel", "d", "drag_old", "active", "perm", "keys"):
            getattr(p, "_" + name).copy_(torch.from_numpy(z["p_" + name]))
        ss = int(z["p_since_sort"])
        p._since_sort = None if ss < 0 else ss
    if multiphase is not None and "mp_phi" in z:
        m = multiphase
        m.phi.copy_(torch.from_numpy(z["mp_phi"]))
        m.phi_new.copy_(torch.from_numpy(z["mp_phi_new"]))
        m.mu.copy_(torch.from_numpy(z["mp_mu"]))
        m._mu_live = bool(z["mp_mu_live"])
        m.phi_changed()
    if filter_system is not None and "filter_accum" in z:
        filter_system.accumulated_particles.copy_(torch.from_numpy(z["filter_accum"]))
        filter_system.filter_blockage.copy_(torch.from_numpy(z["filter_blockage"]))
        filter_system.step_count = int(z["filter_step"])
        filter_system.seed = int(z["filter_seed"])
