"""Throughput of the D3Q19 + coffee-particle hot path on GB300 (one JSON line on rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Headline workload (the metric's configuration): 256^3 D3Q19 in FP32 storage -- BGK, Smagorinsky
LES (Cs 0.1, local strain), Guo gravity, a 3-cell Darcy-Forchheimer filter band (eps 0.6, K 1e-3,
C_F 0.55), half-way bounce-back on the V60 cone, inlet disk and drain outlet.  MLUPS = cells x
steps / time (all cells, as the reference's benchmark_suite.py:129).  Inputs are seeded synthetic
(no dataset exists).

`value` is the median over 5 timed regions of exactly K steps (CUDA graphs of 20 steps, CUDA
events on the launching stream, all state resident in HBM; the 1.27 GB distribution buffer is far
larger than L2, so no flush is needed).  `e2e` drives the public solver API step by step with a
host-to-device copy of the pour control (17 floats) and a device-to-host copy of the step's FP64
sums every step.  `roofline` divides the step's algorithmic bytes by the same timing.
Extra lines: FP16S / BF16S storage at 256^3 (both step kernels, errors against an FP64 run), the
128^3 two-way coupled case with 20,000 particles, the plugin kernels, the 96^3 differentiation
case and the 320x320x384 / 1M-particle scale case.
The reference arm (--impl reference) times the CPU restatement of the same workload on the host
cores (the reference itself is Python + Taichi and cannot run here).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FALLBACK_HBM_GBS = 6800.0
GRAPH_STEPS = 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-extra", action="store_true", help="skip the 256^3 precision lines")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--error-steps", type=int, default=2000, help="steps of the FP64 error runs")
    ap.add_argument("--small", action="store_true", help="64^3 / 2,000 particles (profiling)")
    ap.add_argument("--scale-steps", type=int, default=5000,
                    help="coupled steps of the 320x320x384 / 1M-particle line (0 = skip)")
    ap.add_argument("--precision-only", choices=["fp32", "fp16s", "bf16s"], default=None,
                    help="time only the 256^3 precision case in this storage for --steps steps (profiling)")
    ap.add_argument("--precision-case", choices=["les_band", "plain"], default="les_band")
    ap.add_argument("--coupled-only", action="store_true",
                    help="print only the coupled 128^3 / 20,000-particle line (profiling)")
    ap.add_argument("--adjoint-only", type=int, default=0, metavar="N",
                    help="time the adjoint step kernel alone on an N^3 FP32 LES + band lattice")
    ap.add_argument("--scale-only", action="store_true",
                    help="run --steps coupled steps of the 320x320x384 / 1M-particle case (profiling)")
    ap.add_argument("--step-kernel", choices=["auto", "rows", "registers"], default="auto",
                    help="lattice step kernel: auto (two-cell kernel for 16-bit storage, else per-cell), "
                         "row-tiled TMA-staged, or per-cell register-staged")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.index)], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for name, v in zip(names[1:], r[5:9]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def workload(small=False):
    from pour_over_coffee_lbm_gb300.params import coupled_128
    cfg, pc = coupled_128()
    if small:
        cfg = cfg.replace(nx=64, ny=64, nz=64)
        pc.count = 2000
    return cfg, pc


def fluid_cells(flags):
    import torch
    from pour_over_coffee_lbm_gb300.params import CELL_SOLID
    return int(((flags & CELL_SOLID) == 0).sum().item())


def time_graph(graph, replays):
    import torch
    stream = torch.cuda.current_stream()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    start.record(stream)
    for _ in range(replays):
        graph.replay()
    end.record(stream)
    torch.cuda.synchronize()
    return start.elapsed_time(end) / 1e3


def kernel_roofline(cfg, pc, steps, peak, step_kernel="auto"):
    """Average duration of the fused LBM step kernel alone with the arguments it has inside the
    coupled step (the particle drag deposit and its cell mask of a real coupling pass, rho/u
    written), over `steps` graph-replayed launches."""
    import torch
    from pour_over_coffee_lbm_gb300.params import CELL_SOLID
    from pour_over_coffee_lbm_gb300.particles import CoffeeParticleSystem
    from pour_over_coffee_lbm_gb300.solver import GB300LBMSolver
    s = GB300LBMSolver(cfg, step_kernel=step_kernel)
    ps = CoffeeParticleSystem(pc.count, lattice=cfg, config=pc)
    ps.seed()
    for _ in range(6):
        s.step_with_two_way_coupling(ps)
    torch.cuda.synchronize()
    g = GraphOfSteps(s, GRAPH_STEPS)
    time_graph(g, 2)
    reps = max(1, steps // GRAPH_STEPS)
    dt = time_graph(g, reps)
    per_launch = dt / (reps * GRAPH_STEPS)
    fluid = (s._flags.reshape(-1) & CELL_SOLID) == 0
    nf = int(fluid.sum().item())
    bits = ((s._dmask.view(-1, 1) >> torch.arange(32, device=s._dmask.device, dtype=torch.int32)) & 1).reshape(-1)
    nd = int((bits[:s.n].bool() & fluid).sum().item())
    esize = s._f.element_size()
    # per fluid cell: 19 populations read + written, rho/u written; per deposit cell: the 16 B
    # deposit read; per cell: the 4 B flag word and one bit of the deposit mask
    bytes_per_launch = nf * (2 * 19 * esize + 4 + 12) + nd * 16 + s.n * 4 + s.n // 8
    achieved = bytes_per_launch / per_launch / 1e9
    out = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak[0], "unit": "GB/s",
           "frac": round(achieved / peak[0], 4), "peak_source": peak[1],
           "kernel": ("rows_step_kernel with its bounce-back mailbox passes" if step_kernel == "rows" else
                      "aa_step_kernel") + " (fused collide-stream, particle drag read at deposit cells, rho/u write): "
                                         "one lattice step",
           "kernel_us": round(per_launch * 1e6, 2), "algorithmic_bytes_per_launch": bytes_per_launch,
           "fluid_cells": nf, "deposit_cells": nd, "cells": s.n}
    del s, g, ps
    return out


class GraphOfSteps:
    """CUDA graph of n plain steps with the solver's current force/macro options."""

    def __init__(self, solver, n):
        import torch
        self.s = solver
        self.n = n
        t0 = solver.t
        self.g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.g):
            for _ in range(n):
                solver.run(1, want_macro=True)
        solver.t = t0

    def replay(self):
        self.g.replay()
        self.s.t += self.n


def _time_launches(fn, n):
    """Mean device time of fn() (a few kernel launches) over n graph-captured calls."""
    import torch
    fn()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        for _ in range(n):
            fn()

    class _G:
        def replay(self_inner):
            g.replay()
    time_graph(_G(), 1)
    return time_graph(_G(), 3) / (3 * n)


def plugin_rows(cfg, pc, steps, peak):
    """The reference's production step (main.py step_stable: pour stream and its phase change,
    pressure drive, surface tension before the collision, lattice step, filter paper, phase-field
    step) on the coupled workload, graph-replayed, and the HBM rooflines of the plugin kernels."""
    import torch
    from pour_over_coffee_lbm_gb300 import _lib
    from pour_over_coffee_lbm_gb300.drive import PressureGradientDrive
    from pour_over_coffee_lbm_gb300.filter import FilterPaperSystem
    from pour_over_coffee_lbm_gb300.multiphase import MultiphaseFlow3D
    from pour_over_coffee_lbm_gb300.params import CELL_SOLID
    from pour_over_coffee_lbm_gb300.particles import CoffeeParticleSystem
    from pour_over_coffee_lbm_gb300.pouring import PrecisePouringSystem
    from pour_over_coffee_lbm_gb300.solver import GB300LBMSolver
    lib = _lib.load()
    s = GB300LBMSolver(cfg)
    ps = CoffeeParticleSystem(pc.count, lattice=cfg, config=pc)
    ps.seed()
    # sigma and the drive's force cap are lowered from the reference's 0.0036 and 0.12: with
    # rho_air = 0.00125 those make F / rho at the interface O(0.1) and the run non-finite
    mp = MultiphaseFlow3D(s, surface_tension=1e-5)
    mp.standardize_initial_state()
    pour = PrecisePouringSystem(cfg, diameter=8.0)
    pour.start_pouring(pattern="spiral")
    drive = PressureGradientDrive(s)
    drive.MAX_PRESSURE_FORCE = 1e-5
    drive.activate_force_drive(True)
    fs = FilterPaperSystem(s)

    def production(k):
        s.clear_body_force()
        pour.apply_pouring_force(s)
        pour.apply_gradual_phase_change(mp)
        drive.apply(k)
        if k > 10:
            mp.accumulate_surface_tension_pre_collision()
        s.run(1, want_macro=True)
        fs.step(ps)
        mp.step(k, precollision_applied=True)

    for k in range(12 + (s.t % 2)):
        production(k)
    torch.cuda.synchronize()
    t0 = s.t
    lib.pog_launch_count(1)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        for _ in range(GRAPH_STEPS):
            production(100)
    kernels = int(lib.pog_launch_count(1)) // GRAPH_STEPS
    s.t = t0

    class _G:
        def replay(self_inner):
            g.replay()
            s.t += GRAPH_STEPS
    time_graph(_G(), 2)
    reps = max(1, steps // GRAPH_STEPS)
    per_step = time_graph(_G(), reps) / (reps * GRAPH_STEPS)
    stable = bool(s.check_stability())
    wf = mp.get_interface_statistics()["water_fraction"]
    del g

    n = s.n
    inner = (cfg.nx - 2) * (cfg.ny - 2) * (cfg.nz - 2)
    m = mp.gmag.reshape(-1)
    fl = s._flags.reshape(-1)
    n_on = int(((m > 1e-10) & (mp.phi.reshape(-1).abs() < 0.9) & ((fl & CELL_SOLID) == 0)).sum().item())
    n_grad = int((m > 1e-10).sum().item())
    n_por = int(((fl & 8) != 0).sum().item())
    rows = {}

    def row(name, fn, nbytes):
        us = _time_launches(fn, 20) * 1e6
        rows[name] = {"kernel_us": round(us, 2)}
        if nbytes:
            gbs = nbytes / (us * 1e-6) / 1e9
            rows[name].update({"algorithmic_bytes": int(nbytes), "achieved_gbs": round(gbs, 1),
                               "frac": round(gbs / peak[0], 4)})

    row("pog_phase_normals", mp.compute_gradients, inner * (4 + 16))
    row("pog_phase_surface_tension", lambda: mp._tension(True, outputs=False),
        inner * 4 + n_grad * 4 + n_on * (12 + 4 + 4 + 24))
    row("pog_phase_update", mp.update_phase_field_cahn_hilliard, n * (4 + 4 + 12 + 4 + 4 + 4) + inner * 4)
    row("pog_pressure_force", lambda: drive._accumulate(1.0), n * (4 + 4 + 24))
    row("pog_filter_update", fs.update_dynamic_resistance, n * 4 + n_por * 16)
    row("pog_filter_particles", lambda: fs.block_particles_at_filter(ps), pc.count * (4 + 12 + 12))
    row("pog_phase_properties", mp.update_density_from_phase, n * (4 + 4 + 4))
    row("pog_pour_phase", lambda: pour.apply_gradual_phase_change(mp), 0)
    # diagnostics: one pass over rho, u and the previous check's rho, u
    rho_prev, u_prev = s._rho.clone(), s._u.clone()
    st = torch.empty(24, dtype=torch.float64, device="cuda")
    zp = torch.empty(cfg.nz, dtype=torch.float64, device="cuda")

    def stats():
        _lib.check(lib.pog_field_stats(s._p, s._rho.data_ptr(), s._u.data_ptr(), rho_prev.data_ptr(),
                                       u_prev.data_ptr(), st.data_ptr(), zp.data_ptr(), _lib.stream_handle()))
    row("pog_field_stats", stats, n * 32)
    out = {"workload": "%dx%dx%d production step: pour stream + phase change, pressure drive (force, cap 1e-5), "
                       "surface tension (sigma 1e-5), FP32 lattice step reading the phase field, filter paper "
                       "(%d particles), phase-field step" % (cfg.nx, cfg.ny, cfg.nz, pc.count),
           "mlups": round(n / per_step / 1e6, 1), "ms_per_step": round(per_step * 1e3, 4),
           "kernels_per_step": kernels, "stable": stable, "water_fraction": round(wf, 5),
           "kernels": rows,
           "note": "algorithmic bytes: normals 4 B read + 16 B written per interior cell; surface tension "
                   "4 B per interior cell + 4 B per cell with a gradient + 44 B per interface cell; phase "
                   "update 28 B per cell + 4 B mu per interior cell; pressure force 32 B per cell; "
                   "filter update 4 B per cell + 16 B per paper cell; filter particles 28 B per particle; "
                   "phase properties 12 B per cell; field stats 32 B per cell; pour phase: the stream's "
                   "planes only (time alone)"}
    del s, ps, mp, pour, drive, fs
    torch.cuda.empty_cache()
    return out


def differentiation_rows(peak):
    """96^3 + band with per-cell porosity 0.6 +- 0.05, the 16-coefficient inlet profile and 5,000
    two-way coupled particles: 500 steps forward and the adjoint with checkpoints every 50, FP32
    and FP64, timed.  The particles' drag deposit is recorded per step and held fixed by the
    adjoint; FP64 central differences (h = 1e-3) of J under that recorded forcing on the 8 porous
    cells with the largest gradients and all 16 coefficients check it (bar 1e-4 of the largest
    component).  The differences of the fully coupled J (particles responding) are reported beside
    them: their gap to the adjoint is the particles' feedback, which the adjoint leaves out."""
    import numpy as np
    import torch
    from pour_over_coffee_lbm_gb300.adjoint import OutflowAdjoint
    from pour_over_coffee_lbm_gb300.params import (CELL_POROUS, STORE_F32, STORE_F64, differentiation_96,
                                                   porosity_field)
    cfg, pc = differentiation_96()
    T, K = 500, 50
    out = {"workload": "%dx%dx%d D3Q19 + LES(local) + band, porosity 0.6 +- 0.05, 16-coefficient inlet, %d particles "
                       "two-way coupled (deposit recorded per step); J = sum of outflow over %d steps, checkpoints "
                       "every %d" % (cfg.nx, cfg.ny, cfg.nz, pc.count, T, K)}
    res = {}
    for name, st in (("fp32", STORE_F32), ("fp64", STORE_F64)):
        c = cfg.replace(storage=st)
        run = OutflowAdjoint(c, T, K, particles=pc)
        fl = run.flags.cpu().numpy()
        eps = torch.as_tensor(porosity_field(c, fl, seed=1234)).reshape(c.nz, c.ny, c.nx).cuda()
        run.forward(eps, c.inlet_coef)  # warm-up
        run.backward()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        ev[0].record()
        J = run.forward(eps, c.inlet_coef, record_deposits=(st == STORE_F64))
        ev[1].record()
        r = run.backward()
        ev[2].record()
        torch.cuda.synchronize()
        fwd, bwd = ev[0].elapsed_time(ev[1]) / 1e3, ev[1].elapsed_time(ev[2]) / 1e3
        gbs = 458 * c.ncell * T / bwd / 1e9
        out[name] = {"forward_ms": round(fwd * 1e3, 2), "backward_ms": round(bwd * 1e3, 2),
                     "adjoint_mlups": round(c.ncell * T / bwd / 1e6, 1), "loss": J,
                     "adjoint_roofline": {"achieved_gbs": round(gbs, 1), "frac": round(gbs / peak[0], 4),
                                          "bytes": "458 B per cell update"}}
        res[name] = (run, eps, fl, r)
    g32, g64 = res["fp32"][3], res["fp64"][3]
    rel = {"inlet": float((g32.grad_inlet - g64.grad_inlet).norm() / g64.grad_inlet.norm()),
           "porosity": float((g32.grad_porosity - g64.grad_porosity).norm() / g64.grad_porosity.norm())}
    # bars: the FP32 run recomputes its forward states in FP32, whose u resolution limits the porosity
    # gradient (concentrated in the band) more than the inlet's
    out["fp32_vs_fp64_grad_rel"] = dict(rel, bars={"inlet": 1e-3, "porosity": 1e-2},
                                        ok=rel["inlet"] <= 1e-3 and rel["porosity"] <= 1e-2)
    run, eps, fl, r = res["fp64"]
    h = 1e-3
    coef = np.array(cfg.inlet_coef, np.float64)
    fds, fdc, ads = [], [], []
    for k in range(16):
        cp, cm = coef.copy(), coef.copy()
        cp[k] += h
        cm[k] -= h
        fds.append((run.loss_frozen(eps, cp) - run.loss_frozen(eps, cm)) / (2 * h))
        ads.append(r.grad_inlet[k].item())
    for k in range(16):
        cp, cm = coef.copy(), coef.copy()
        cp[k] += h
        cm[k] -= h
        fdc.append((run.loss(eps, cp) - run.loss(eps, cm)) / (2 * h))
    fds, fdc, ads = np.array(fds), np.array(fdc), np.array(ads)
    err_in = float(np.max(np.abs(ads - fds)) / np.max(np.abs(fds)))
    ge = r.grad_porosity.cpu().numpy().reshape(-1)
    band = np.flatnonzero((fl.reshape(-1) & CELL_POROUS) != 0)
    flat = eps.reshape(-1)
    err_eps = 0.0
    for c in band[np.argsort(-np.abs(ge[band]))[:8]]:
        ep, em = flat.clone(), flat.clone()
        ep[c] += h
        em[c] -= h
        hh = (ep[c].double() - em[c].double()).item() / 2
        fd = (run.loss_frozen(ep.reshape(eps.shape), coef) - run.loss_frozen(em.reshape(eps.shape), coef)) / (2 * hh)
        err_eps = max(err_eps, abs(ge[c] - fd) / max(abs(fd), 1e-30))
    err_eps = float(err_eps)
    out["fd_fp64_h1e-3"] = {"inlet_16_vs_largest": err_in, "porosity_8_max_rel": err_eps,
                            "bar": 1e-4, "ok": bool(err_in <= 1e-4 and err_eps <= 1e-4),
                            "inlet_fd_recorded_forcing": fds.tolist(), "inlet_adjoint": ads.tolist(),
                            "inlet_fd_particles_responding": fdc.tolist(),
                            "particle_feedback_vs_largest": float(np.max(np.abs(fdc - fds)) / np.max(np.abs(fds)))}
    del res, run
    torch.cuda.empty_cache()
    return out


def scale_row(steps, peak, adj_steps=200, ckpt=20, step_kernel="auto"):
    """320x320x384 FP16S + LES + band + 1,000,000 particles: exactly `steps` two-way coupled steps
    (4 eager, the rest graph-replayed), then the outflow adjoint over the last adj_steps of them
    (recomputed in FP32 from the FP16S state exported at step steps - adj_steps, checkpoints every
    ckpt).  Roofline fractions: the coupled step at 93 B per cell update (FP16S lattice 77 B, and the
    rho/u the coupling pass gathers from, 16 B, written by the step) plus 268 B
    per particle (gather, drag, integration, deposit), the adjoint at 458 B per cell update (one
    forward recomputation, the state and the adjoint state read and written)."""
    import torch
    from pour_over_coffee_lbm_gb300 import _lib
    from pour_over_coffee_lbm_gb300.adjoint import OutflowAdjoint
    from pour_over_coffee_lbm_gb300.params import STORE_F32, scale_320x384
    from pour_over_coffee_lbm_gb300.particles import CoffeeParticleSystem
    from pour_over_coffee_lbm_gb300.solver import GB300LBMSolver
    cfg, pc = scale_320x384()
    s = GB300LBMSolver(cfg, step_kernel=step_kernel)
    ps = CoffeeParticleSystem(pc.count, lattice=cfg, config=pc)
    ps.seed()
    for _ in range(4):
        s.step_with_two_way_coupling(ps)
    g = s.capture(GRAPH_STEPS, ps)
    torch.cuda.synchronize()
    split = steps - adj_steps  # the adjoint window starts here
    before = split - 4
    reps1, rem1 = divmod(before, GRAPH_STEPS)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    ev[0].record()
    for _ in range(reps1):
        g.replay()
    for _ in range(rem1):
        s.step_with_two_way_coupling(ps)
    ev[1].record()
    nat = torch.empty((19, cfg.nz, cfg.ny, cfg.nx), dtype=torch.float32, device="cuda")
    _lib.check(s.lib.pog_export_natural(s._p, _lib.ptr(s._f), _lib.ptr(s._flags), s.t, _lib.ptr(nat), STORE_F32,
                                        _lib.stream_handle()))
    ev[2].record()
    left = adj_steps
    if s.t % 2:  # graphs replay at even time indices
        s.step_with_two_way_coupling(ps)
        left -= 1
    reps2, rem2 = divmod(left, GRAPH_STEPS)
    for _ in range(reps2):
        g.replay()
    for _ in range(rem2):
        s.step_with_two_way_coupling(ps)
    ev[3].record()
    torch.cuda.synchronize()
    timed = before + adj_steps
    el = (ev[0].elapsed_time(ev[1]) + ev[2].elapsed_time(ev[3])) / 1e3
    stable = bool(s.check_stability())
    done = s.t
    per_step = el / timed
    fwd_bytes = (77 + 16) * cfg.ncell + 268 * pc.count
    fwd_gbs = fwd_bytes / per_step / 1e9
    del g
    particles = particle_pass(s, ps, peak)
    del s, ps
    torch.cuda.empty_cache()
    run = OutflowAdjoint(cfg.replace(storage=STORE_F32), adj_steps, ckpt)
    # gradients w.r.t. the band's per-cell porosity (the inlet is more than adj_steps planes
    # above the outlet, so its coefficients cannot reach J within the window)
    eps = torch.full((cfg.nz, cfg.ny, cfg.nx), cfg.porosity, dtype=torch.float32, device="cuda")
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    e[0].record()
    J = run.forward(eps, cfg.inlet_coef, initial=nat)
    e[1].record()
    r = run.backward(want_porosity_grad=True)
    e[2].record()
    torch.cuda.synchronize()
    fwd, bwd = e[0].elapsed_time(e[1]) / 1e3, e[1].elapsed_time(e[2]) / 1e3
    adj_gbs = 458 * cfg.ncell * adj_steps / bwd / 1e9
    out = {"workload": "%dx%dx%d FP16S + LES(local) + band + %d particles, two-way coupled; adjoint of the outflow "
                       "over the last %d steps (FP32 recompute, checkpoints every %d)"
                       % (cfg.nx, cfg.ny, cfg.nz, pc.count, adj_steps, ckpt),
           "coupled_steps": done, "timed_coupled_steps": timed, "coupled_mlups": round(cfg.ncell / per_step / 1e6, 1),
           "coupled_ms_per_step": round(per_step * 1e3, 4), "stable": stable,
           "coupled_roofline": {"algorithmic_bytes_per_step": fwd_bytes, "achieved_gbs": round(fwd_gbs, 1),
                                "frac": round(fwd_gbs / peak[0], 4), "peak": peak[0], "peak_source": peak[1],
                                "bytes": "77 B per cell update (FP16S) + 16 B rho/u write + 268 B per particle"},
           "particle_pass": particles,
           "adjoint": {"steps": adj_steps, "forward_ms": round(fwd * 1e3, 1), "backward_ms": round(bwd * 1e3, 1),
                       "adjoint_mlups": round(cfg.ncell * adj_steps / bwd / 1e6, 1), "loss": J,
                       "roofline": {"achieved_gbs": round(adj_gbs, 1), "frac": round(adj_gbs / peak[0], 4),
                                    "bytes": "458 B per cell update"},
                       "grad_porosity_finite": bool(torch.isfinite(r.grad_porosity).all()),
                       "grad_porosity_nonzero_cells": int((r.grad_porosity != 0).sum().item())},
           "max_memory_gb": round(torch.cuda.max_memory_allocated() / 1e9, 1)}
    del run, nat, eps, r
    torch.cuda.empty_cache()
    return out


def run_scale_only(args):
    """A few coupled steps of the 320x320x384 / 1M-particle case (profiling the coupling kernels)."""
    import torch
    from pour_over_coffee_lbm_gb300.params import scale_320x384
    from pour_over_coffee_lbm_gb300.particles import CoffeeParticleSystem
    from pour_over_coffee_lbm_gb300.solver import GB300LBMSolver
    torch.cuda.set_device(0)
    cfg, pc = scale_320x384()
    s = GB300LBMSolver(cfg, step_kernel=args.step_kernel)
    ps = CoffeeParticleSystem(pc.count, lattice=cfg, config=pc)
    ps.seed()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(4):
        s.step_with_two_way_coupling(ps)
    start.record()
    for _ in range(args.steps):
        s.step_with_two_way_coupling(ps)
    end.record()
    torch.cuda.synchronize()
    print(json.dumps({"scale_only_steps": args.steps, "ms_per_step": round(start.elapsed_time(end) / args.steps, 4),
                      "stable": bool(s.check_stability())}), flush=True)


PRECISION_CASES = {
    # the 256^3 target case: D3Q19 + LES (local strain) + 3-cell porous band
    "les_band": {},
    # the plain 256^3 physics of the 64^3 case (no LES, no porous band)
    "plain": {"les": False, "band": 0.0},
}


def precision_cfg(storage, case):
    from pour_over_coffee_lbm_gb300.params import LES_LOCAL, LES_OFF, precision_256
    kw = PRECISION_CASES[case]
    return precision_256(storage=storage, les_mode=LES_LOCAL if kw.get("les", True) else LES_OFF,
                         band=kw.get("band", 3.0))


def precision_line(storage, steps, peak, case="les_band", step_kernel="auto", density_reference=False):
    import torch
    from pour_over_coffee_lbm_gb300.solver import GB300LBMSolver
    cfg = precision_cfg(storage, case)
    s = GB300LBMSolver(cfg, step_kernel=step_kernel, density_reference=density_reference)
    for _ in range(4):
        s.run(1)
    torch.cuda.synchronize()
    t0 = s.t
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        for _ in range(GRAPH_STEPS):
            s.run(1)
    s.t = t0

    class _G:
        def replay(self_inner):
            g.replay()
            s.t += GRAPH_STEPS
    gg = _G()
    time_graph(gg, 2)
    reps = max(1, steps // GRAPH_STEPS)
    dt = time_graph(gg, reps)
    per = dt / (reps * GRAPH_STEPS)
    nf = fluid_cells(s.flags)
    esize = s._f.element_size()
    bpl = nf * 2 * 19 * esize + s.n * 4
    mlups = s.n / per / 1e6
    ach = bpl / per / 1e9
    out = {"mlups": round(mlups, 1), "kernel_us": round(per * 1e6, 2), "achieved_gbs": round(ach, 1),
           "frac": round(ach / peak[0], 4), "bytes_per_lup": round(bpl / s.n, 2)}
    del s, g
    torch.cuda.empty_cache()
    return out


def precision_errors(steps, case="les_band"):
    """u and rho relative L2 error (fluid cells) of FP32 / FP16S / BF16S storage against an FP64
    run of the same 256^3 case from the same initial state, after 500, 1000, ... `steps` steps."""
    import torch
    from pour_over_coffee_lbm_gb300.params import STORE_BF16S, STORE_F16S, STORE_F32, STORE_F64
    from pour_over_coffee_lbm_gb300.solver import GB300LBMSolver
    checks = sorted({c for c in (500, 1000, steps) if c <= steps})

    def trajectory(st, ref=False):
        s = GB300LBMSolver(precision_cfg(st, case), density_reference=ref)
        done, out = 0, {}
        for c in checks:
            s.run(c - done - 1)
            s.run(1, want_macro=True)
            done = c
            out[c] = (s._u.double().clone(), s._rho.double().clone())
        fluid = (s.flags & 1) == 0
        del s
        torch.cuda.empty_cache()
        return out, fluid

    ref, fluid = trajectory(STORE_F64)
    res = {"steps": checks}
    for name, st, ref_d in (("fp32", STORE_F32, False), ("fp16s", STORE_F16S, False),
                            ("fp16s_ref", STORE_F16S, True), ("bf16s", STORE_BF16S, False)):
        got, _ = trajectory(st, ref_d)
        res[name] = {"u_rel_l2": [], "rho_rel_l2": []}
        for c in checks:
            u, r = got[c]
            u64, r64 = ref[c]
            res[name]["u_rel_l2"].append(float(torch.linalg.norm((u - u64)[:, fluid]) / torch.linalg.norm(u64[:, fluid])))
            res[name]["rho_rel_l2"].append(float(torch.linalg.norm((r - r64)[fluid]) / torch.linalg.norm(r64[fluid])))
        del got
        torch.cuda.empty_cache()
    return res


def cpu_baseline_coupled(cfg, pc, seconds):
    """The CPU restatement (oracle, OpenMP on all host cores, particles serial) on the coupled
    workload, time-bounded: returns MLUPS and the sample it measured."""
    import numpy as np
    import oracle as O
    from pour_over_coffee_lbm_gb300.params import seed_particles
    flags = O.build_flags(cfg)
    f = O.init_equilibrium(cfg, flags, np.float32)
    pos, vel, d, act = seed_particles(cfg, pc)
    drag = np.zeros_like(pos)
    _, _, u = O.step(cfg, flags, f)
    steps = 0
    t0 = time.perf_counter()
    while True:
        pos, vel, drag, act, fix, _ = O.particles_couple(cfg, pc, pos, vel, d, drag, act, u)
        pdrag = (fix.astype(np.float64) / 2.0 ** 32).astype(np.float32).reshape(4, cfg.nz, cfg.ny, cfg.nx)
        f, rho, u = O.step(cfg, flags, f, pdrag=pdrag)
        steps += 1
        el = time.perf_counter() - t0
        if el >= seconds or steps >= 500:
            break
    return cfg.ncell * steps / el / 1e6, steps, el


def cpu_lattice_steps(cfg, seconds, max_steps):
    """The CPU restatement's FP32 lattice step (OpenMP on all host cores) on `cfg`, time-bounded:
    (MLUPS, steps, seconds).  One untimed step first (allocation, page faults)."""
    import numpy as np
    import oracle as O
    flags = O.build_flags(cfg)
    f = O.init_equilibrium(cfg, flags, np.float32)
    f, _, _ = O.step(cfg, flags, f)
    steps = 0
    t0 = time.perf_counter()
    while True:
        f, _, _ = O.step(cfg, flags, f)
        steps += 1
        el = time.perf_counter() - t0
        if el >= seconds or steps >= max_steps:
            break
    return cfg.ncell * steps / el / 1e6, steps, el


HEADLINE = ("256^3 D3Q19 FP32: BGK + Smagorinsky LES (Cs 0.1, local strain) + Guo gravity + 3-cell "
            "Darcy-Forchheimer filter band (eps 0.6, K 1e-3, C_F 0.55) + half-way bounce-back on the V60 "
            "cone, inlet disk and drain outlet; no particles")
REPEATS = 5


def headline_cfg():
    from pour_over_coffee_lbm_gb300.params import STORE_F32
    return precision_cfg(STORE_F32, "les_band")


def step_bytes(solver):
    """Algorithmic bytes of one plain lattice step: per fluid cell the 19 populations read and
    written, per cell the 4-byte flag word."""
    nf = fluid_cells(solver.flags)
    return nf * 2 * 19 * solver._f.element_size() + solver.n * 4


def headline(args, peak, world, local):
    """The metric's configuration on this GPU: `value` = median over REPEATS timed regions of
    exactly K steps (graph replays, CUDA events on the launching stream); `e2e` = the same steps
    through the public solver API with a host->device pour control and a device->host read of the
    step's FP64 sums every step; `roofline` from the same timing."""
    import torch
    from pour_over_coffee_lbm_gb300.solver import GB300LBMSolver
    cfg = headline_cfg()
    s = GB300LBMSolver(cfg, step_kernel=args.step_kernel)
    W = max(3, args.warmup)
    s.run(W + (W % 2))
    torch.cuda.synchronize()
    lib = s.lib
    graph = s.capture(GRAPH_STEPS)
    graph.replay()
    torch.cuda.synchronize()
    K = args.steps
    reps, rem = divmod(K, GRAPH_STEPS)
    stream = torch.cuda.current_stream()
    clocks = ClockSampler(local)
    clocks.start()
    times = []
    lib.pog_launch_count(1)
    for _ in range(REPEATS):
        if s.t % 2:
            s.run(1)  # graphs replay at even time indices
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        start.record(stream)
        for _ in range(reps):
            graph.replay()
        if rem:
            s.run(rem)
        end.record(stream)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        times.append(start.elapsed_time(end) / 1e3)
    clk = clocks.stop()
    eager = int(lib.pog_launch_count(1))
    if world > 1:
        t = torch.tensor(times, device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        times = t.tolist()
    elapsed = statistics.median(times)
    launches_per_region = graph.kernels // GRAPH_STEPS * GRAPH_STEPS * reps + eager // REPEATS
    stable = bool(s.check_stability())
    nbytes = step_bytes(s)
    per_step = elapsed / K
    achieved = nbytes / per_step / 1e9
    roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak[0], "unit": "GB/s",
            "frac": round(achieved / peak[0], 4), "peak_source": peak[1],
            "kernel": "rows_step_kernel (row-tiled TMA-staged fused collide-stream) with its bounce-back mailbox "
                      "passes: one lattice step" if args.step_kernel == "rows" else
                      "aa_step_kernel (register-staged fused collide-stream): one lattice step",
            "step_us": round(per_step * 1e6, 2), "algorithmic_bytes_per_step": nbytes,
            "bytes_per_lup": round(nbytes / s.n, 2), "fluid_cells": fluid_cells(s.flags), "cells": s.n}

    # end to end through the public API: per step an H2D pour control and a D2H of the FP64 sums
    ctl_h = torch.zeros((K, 17), dtype=torch.float32).pin_memory()
    for i in range(K):
        ctl_h[i, 0] = cfg.u_inlet * (1.0 + 0.1 * ((i % 50) / 50.0))  # a slowly varying pour
    ctl_d = torch.zeros(17, dtype=torch.float32, device="cuda")
    ctl_d.copy_(ctl_h[0])
    s.set_inlet_control(ctl_d)
    red_h = torch.zeros((K, 6), dtype=torch.float64).pin_memory()
    for _ in range(2):
        s.run(1, reduce=True)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for i in range(K):
        ctl_d.copy_(ctl_h[i], non_blocking=True)
        red = s.run(1, reduce=True)
        red_h[i].copy_(red, non_blocking=True)
    torch.cuda.synchronize()
    e2e_el = time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([e2e_el], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_el = float(t.item())
    e2e_ok = bool(torch.isfinite(red_h[:, :5]).all()) and float(red_h[:, 5].sum()) == 0.0
    s.set_inlet_control(None)
    e2e = {"value": round(world * cfg.ncell * K / e2e_el / 1e6, 1), "unit": "MLUPS",
           "h2d_bytes_per_step": 17 * 4, "d2h_bytes_per_step": 6 * 8,
           "api": "GB300LBMSolver.run(1, reduce=True) per step (pog_step through the C ABI)",
           "results_finite": e2e_ok}
    out = {"value": world * cfg.ncell * K / elapsed / 1e6, "elapsed": elapsed, "times": times, "K": K, "W": W,
           "roofline": roof, "e2e": e2e, "clocks": clk, "launches": launches_per_region, "stable": stable,
           "ncell": cfg.ncell}
    del graph, s
    torch.cuda.empty_cache()
    return out


def particle_pass(solver, ps, peak, reps=10):
    """The coupling pass alone (couple_kernel: trilinear gather, drag, relaxation, integration with
    the cone constraint, deposit), `reps` passes on the current state into a scratch deposit field,
    timed with CUDA events between two particle sorts: 268 B per active particle (8 x 12 B u
    gathers, 8 x 12 B deposit, position / velocity / drag state read and written, diameter),
    reported as its own particle GB/s beside the lattice's."""
    import torch
    scratch = torch.zeros_like(solver._pdrag)
    mask = torch.zeros_like(solver._dmask)
    for _ in range(3):
        ps.couple(solver, pdrag=scratch, deposit_mask=mask)
    ps._since_sort = 0  # no sort inside the timed passes (sort_interval > reps)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ev[0].record()
    for _ in range(reps):
        ps.couple(solver, pdrag=scratch, deposit_mask=mask)
    ev[1].record()
    torch.cuda.synchronize()
    us = ev[0].elapsed_time(ev[1]) * 1e3 / reps
    active = int((ps._active[:ps.count] != 0).sum().item())
    gbs = 268 * active / us / 1e3
    return {"kernel": "couple_kernel (one coupling pass)", "us_per_pass": round(us, 2), "active_particles": active,
            "bytes_per_particle": 268, "achieved_gbs": round(gbs, 1), "frac": round(gbs / peak[0], 4)}


def coupled_line(args, peak):
    """The 128^3 two-way coupled case (20,000 particles): graph-replayed steps, the public-API
    coupled step end to end, and the step kernel's roofline."""
    import torch
    from pour_over_coffee_lbm_gb300.particles import CoffeeParticleSystem
    from pour_over_coffee_lbm_gb300.solver import GB300LBMSolver
    cfg, pc = workload(args.small)
    solver = GB300LBMSolver(cfg, step_kernel=args.step_kernel)
    ps = CoffeeParticleSystem(pc.count, lattice=cfg, config=pc)
    ps.seed()
    for _ in range(max(3, args.warmup)):
        solver.step_with_two_way_coupling(ps)
    if solver.t % 2:
        solver.step_with_two_way_coupling(ps)
    torch.cuda.synchronize()
    graph = solver.capture(GRAPH_STEPS, ps)
    graph.replay()
    torch.cuda.synchronize()
    reps = max(1, 200 // GRAPH_STEPS)
    times = []
    for _ in range(REPEATS):
        times.append(time_graph(graph, reps) / (reps * GRAPH_STEPS))
    per = statistics.median(times)
    K = reps * GRAPH_STEPS
    ctl_h = torch.zeros((K, 17), dtype=torch.float32).pin_memory()
    for i in range(K):
        ctl_h[i, 0] = cfg.u_inlet * (1.0 + 0.1 * ((i % 50) / 50.0))
    ctl_d = torch.zeros(17, dtype=torch.float32, device="cuda")
    ctl_d.copy_(ctl_h[0])
    solver.set_inlet_control(ctl_d)
    red_h = torch.zeros((K, 6), dtype=torch.float64).pin_memory()
    for _ in range(2):
        solver.step_with_two_way_coupling(ps, reduce=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(K):
        ctl_d.copy_(ctl_h[i], non_blocking=True)
        red = solver.step_with_two_way_coupling(ps, reduce=True)
        red_h[i].copy_(red, non_blocking=True)
    torch.cuda.synchronize()
    e2e_el = time.perf_counter() - t0
    e2e_ok = bool(torch.isfinite(red_h[:, :5]).all()) and float(red_h[:, 5].sum()) == 0.0
    solver.set_inlet_control(None)
    diag = solver.get_diagnostics()
    particles = particle_pass(solver, ps, peak)
    out = {"workload": "coupled FP32: %dx%dx%d D3Q19, LES Cs 0.1 (local strain), porous band 3 cells (eps 0.6, "
                       "K 1e-3, C_F 0.55), %d log-normal particles two-way coupled; a step = coupling pass + "
                       "lattice step" % (cfg.nx, cfg.ny, cfg.nz, pc.count),
           "mlups": round(cfg.ncell / per / 1e6, 1), "ms_per_step": round(per * 1e3, 4),
           "repeats_ms_per_step": [round(t * 1e3, 4) for t in times],
           "kernels_per_step": graph.kernels // GRAPH_STEPS,
           "e2e": {"value": round(cfg.ncell * K / e2e_el / 1e6, 1), "unit": "MLUPS", "h2d_bytes_per_step": 68,
                   "d2h_bytes_per_step": 48, "results_finite": e2e_ok,
                   "api": "GB300LBMSolver.step_with_two_way_coupling(reduce=True) per step"},
           "stable": diag["stable"], "particle_pass": particles,
           "l2": "distributions %.0f MB > 129 MB L2 (no flush)" % (19 * 4 * cfg.ncell / 1e6)}
    del graph, solver, ps
    torch.cuda.empty_cache()
    out["roofline"] = kernel_roofline(cfg, pc, 200, peak, args.step_kernel)
    traffic_path = os.path.join(ROOT, "profiles", "aa_step_traffic.json")
    if os.path.exists(traffic_path):
        with open(traffic_path) as fh:
            tr = json.load(fh)
        key = "coupled %dx%dx%d" % (cfg.nx, cfg.ny, cfg.nz)
        if key in tr:
            out["roofline"]["traffic"] = tr[key]["bytes_per_launch"]
            out["roofline"]["traffic_source"] = tr[key].get("source")
    if not args.no_cpu:
        mlups, steps, el = cpu_baseline_coupled(cfg, pc, min(args.cpu_seconds, 10.0))
        out["cpu_baseline"] = {"value": round(mlups, 3), "unit": "MLUPS", "cores": os.cpu_count(), "kind": "port",
                               "sample": "%d coupled steps of this workload (%.1f s), CPU restatement (OpenMP "
                                         "lattice, serial particles)" % (steps, el)}
    return out


def run_ours(args):
    import torch
    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from pour_over_coffee_lbm_gb300 import _lib
    _lib.load()
    peak = peaks()
    h = headline(args, peak, world, local)
    traffic_path = os.path.join(ROOT, "profiles", "aa_step_traffic.json")
    h["roofline"]["traffic"] = None
    if os.path.exists(traffic_path):
        with open(traffic_path) as fh:
            tr = json.load(fh)
        # FP32 storage: "auto" runs the per-cell register-staged kernel
        key = "les_band 256x256x256 fp32 %s" % ("registers" if args.step_kernel == "auto" else args.step_kernel)
        if key in tr:
            h["roofline"]["traffic"] = tr[key]["bytes_per_step"]
            h["roofline"]["traffic_source"] = tr[key].get("source")

    extra = coupled = rows = diff = scale = adj = None
    if not args.no_extra and not args.small and rank == 0:
        from pour_over_coffee_lbm_gb300.params import STORE_BF16S, STORE_F16S, STORE_F32
        extra = {}
        for case, label in (("les_band", "256^3 D3Q19 + LES(local) + porous band, no particles"),
                            ("plain", "256^3 D3Q19, gravity + inlet/outlet + cone walls (no LES, no band)")):
            lines = {}
            for name, st in (("fp32", STORE_F32), ("fp16s", STORE_F16S), ("bf16s", STORE_BF16S)):
                kernels = ("rows", "registers") if st == STORE_F32 else ("rows", "registers", "auto")
                lines[name] = {k: precision_line(st, 200, peak, case, k) for k in kernels}
            # FP16S stored relative to per-cell reference densities (pog_params.density_ref)
            lines["fp16s_ref"] = {"auto": precision_line(STORE_F16S, 200, peak, case, "auto", True)}
            best = {n: max(v.values(), key=lambda d: d["mlups"]) for n, v in lines.items()}
            errs = precision_errors(args.error_steps, case) if args.error_steps > 0 else None
            extra[case] = {"workload": label, "lines": lines, "error_vs_fp64": errs,
                           "fp16s_vs_fp32_mlups": round(best["fp16s"]["mlups"] / best["fp32"]["mlups"], 3),
                           "fp16s_ref_vs_fp32_mlups": round(best["fp16s_ref"]["mlups"] / best["fp32"]["mlups"], 3),
                           "bf16s_vs_fp32_mlups": round(best["bf16s"]["mlups"] / best["fp32"]["mlups"], 3)}
        coupled = coupled_line(args, peak)
        rows = plugin_rows(*workload(False), 200, peak)
        diff = differentiation_rows(peak)
        adj = adjoint_line(256, 20, peak)
        if args.scale_steps > 0:
            scale = scale_row(args.scale_steps, peak, step_kernel=args.step_kernel)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        mlups, steps, el = cpu_lattice_steps(headline_cfg(), args.cpu_seconds, 200)
        cpu = {"value": round(mlups, 3), "unit": "MLUPS", "cores": os.cpu_count(), "kind": "port",
               "sample": "%d FP32 lattice steps of the same 256^3 LES + porous-band workload (%.1f s), the CPU "
                         "restatement of the reference path (OpenMP on all host cores)" % (steps, el)}

    if rank == 0:
        line = {
            "metric": "D3Q19 MLUPS & % HBM roofline; FP16-store vs FP32 MLUPS at <=1e-3 rel err",
            "value": round(h["value"], 1), "unit": "MLUPS", "n_gpus": world, "steps": h["K"], "warmup": h["W"],
            "ms_per_step": round(h["elapsed"] * 1e3 / h["K"], 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded V60 geometry)",
            "config": {"workload": HEADLINE, "cells": h["ncell"], "step_kernel": args.step_kernel,
                       "graph_steps": GRAPH_STEPS, "repeats": REPEATS,
                       "repeat_ms_per_step": [round(t * 1e3 / h["K"], 4) for t in h["times"]],
                       "l2": "distributions %.2f GB > 129 MB L2 (no flush needed)" % (19 * 4 * h["ncell"] / 1e9),
                       "parallelism": "replicas x%d (one independent lattice per GPU)" % world},
            "e2e": h["e2e"],
            "gpu_launches": int(h["launches"]),
            "roofline": h["roofline"],
            "cpu_baseline": cpu,
            "clocks": h["clocks"],
            "stable": h["stable"],
            "precision_256": extra,
            "coupled_128": coupled,
            "plugin_rows": rows,
            "differentiation_96": diff,
            "adjoint_256": adj,
            "scale_320x320x384": scale,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_reference(args):
    """The reference arm: the reference's path on the host cores.  The reference is Python +
    Taichi and cannot be installed here, so this times its CPU restatement (the oracle, OpenMP on
    all host cores) on the same 256^3 workload, each step a full lattice step, bounded so the run
    ends within about two minutes."""
    world, rank, local = dist_env()
    if rank != 0:
        return
    import numpy as np
    import oracle as O
    cfg = headline_cfg()
    flags = O.build_flags(cfg)
    f = O.init_equilibrium(cfg, flags, np.float32)
    W = max(3, args.warmup)
    t0 = time.perf_counter()
    f, _, _ = O.step(cfg, flags, f)
    per = time.perf_counter() - t0
    for _ in range(min(W, max(1, int(20.0 / per))) - 1):
        f, _, _ = O.step(cfg, flags, f)
    K = args.steps
    k_run = min(K, max(3, int(120.0 / per)))
    t0 = time.perf_counter()
    for _ in range(k_run):
        f, _, _ = O.step(cfg, flags, f)
    el = time.perf_counter() - t0
    mlups = cfg.ncell * k_run / el / 1e6
    line = {"impl": "reference",
            "metric": "D3Q19 MLUPS & % HBM roofline; FP16-store vs FP32 MLUPS at <=1e-3 rel err",
            "value": round(mlups, 3), "unit": "MLUPS", "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": round(el * 1e3 / k_run, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded V60 geometry)",
            "config": {"workload": HEADLINE, "cells": cfg.ncell},
            "cpu_baseline": {"value": round(mlups, 3), "unit": "MLUPS", "cores": os.cpu_count(), "kind": "port",
                             "sample": "%d of %d requested lattice steps timed (%.1f s); the reference is "
                                       "Python+Taichi (not installable here), this is its CPU restatement"
                                       % (k_run, K, el)},
            "e2e": {"value": round(mlups, 3), "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_precision_only(args):
    import torch
    from pour_over_coffee_lbm_gb300.params import STORE_BF16S, STORE_F16S, STORE_F32
    torch.cuda.set_device(0)
    st = {"fp32": STORE_F32, "fp16s": STORE_F16S, "bf16s": STORE_BF16S}[args.precision_only]
    out = precision_line(st, max(GRAPH_STEPS, args.steps), peaks(), args.precision_case, args.step_kernel)
    print(json.dumps({"precision_only": args.precision_only, "step_kernel": args.step_kernel, **out}), flush=True)


def run_coupled_only(args):
    import torch
    torch.cuda.set_device(0)
    args.no_cpu = True
    print(json.dumps({"coupled_only": coupled_line(args, peaks())}), flush=True)


def adjoint_line(N, calls, peak):
    """The adjoint step (pog_adjoint_step: adjoint_kernel + the inlet-plane pass) alone on an N^3
    FP32 LES(local) + porous-band lattice with a porosity field, on a recomputed forward state:
    `calls` calls timed with CUDA events after 3 warm-up calls.  Algorithmic bytes per call:
    232 B per non-solid cell (f_t, lam_{t+1} and lam_t, 19 x 4 B each, and the flag word), 80 B
    per solid cell (flag word, lam_t zeroed), and 20 B more per porous cell (porosity, the FP64
    porosity gradient read and written)."""
    import torch
    from pour_over_coffee_lbm_gb300 import _lib
    from pour_over_coffee_lbm_gb300.adjoint import OutflowAdjoint
    from pour_over_coffee_lbm_gb300.params import CELL_POROUS, CELL_SOLID, LES_LOCAL, STORE_F32, LatticeConfig, \
        porosity_field
    cfg = LatticeConfig(nx=N, ny=N, nz=N, band_thickness=3.0, les_mode=LES_LOCAL, storage=STORE_F32, u_inlet=-0.05)
    run = OutflowAdjoint(cfg, 8, 4)
    fl = run.flags.cpu().numpy()
    eps = torch.as_tensor(porosity_field(cfg, fl, seed=1234)).reshape(cfg.nz, cfg.ny, cfg.nx).cuda()
    run.forward(eps, cfg.inlet_coef)
    run.backward()
    gen = torch.Generator(device="cuda").manual_seed(7)
    lam = torch.randn((19,) + run.shape, device="cuda", generator=gen) * 1e-3
    lam_t = torch.zeros_like(lam)
    g_eps = torch.zeros(run.shape, dtype=torch.float64, device="cuda")
    g_in = torch.zeros(16, dtype=torch.float64, device="cuda")
    s = _lib.stream_handle()

    def call():
        _lib.check(run.lib.pog_adjoint_step(run._p, _lib.ptr(run._states[1]), _lib.ptr(lam), _lib.ptr(lam_t),
                                            _lib.ptr(run.flags), _lib.ptr(run._eps), None, None, None, None,
                                            _lib.ptr(run._scratch), _lib.ptr(g_eps), _lib.ptr(g_in), s))
    for _ in range(3):
        call()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ev[0].record()
    for _ in range(calls):
        call()
    ev[1].record()
    torch.cuda.synchronize()
    us = ev[0].elapsed_time(ev[1]) * 1e3 / calls
    solid = int(((run.flags & CELL_SOLID) != 0).sum().item())
    porous = int((((run.flags & CELL_POROUS) != 0) & ((run.flags & CELL_SOLID) == 0)).sum().item())
    nbytes = 232 * (cfg.ncell - solid) + 80 * solid + 20 * porous
    gbs = nbytes / us / 1e3
    out = {"workload": "adjoint step alone, %d^3 FP32 LES(local) + porous band with a porosity field" % N,
           "calls": calls, "us_per_call": round(us, 1), "mlups": round(cfg.ncell / us, 1),
           "algorithmic_bytes": nbytes, "achieved_gbs": round(gbs, 1), "frac": round(gbs / peak[0], 4),
           "peak_source": peak[1], "finite": bool(torch.isfinite(lam_t).all()),
           "bytes": "232 B per fluid cell, 80 per solid cell, +20 per porous cell"}
    del run, lam, lam_t, g_eps
    torch.cuda.empty_cache()
    return out


def run_adjoint_only(args):
    import torch
    torch.cuda.set_device(0)
    print(json.dumps({"adjoint_only": args.adjoint_only, **adjoint_line(args.adjoint_only, args.steps, peaks())}),
          flush=True)


def main():
    args = parse()
    if args.adjoint_only:
        run_adjoint_only(args)
    elif args.precision_only:
        run_precision_only(args)
    elif args.coupled_only:
        run_coupled_only(args)
    elif args.scale_only:
        run_scale_only(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
