"""CPU oracle of the hot path -- TEST INFRASTRUCTURE ONLY.

numpy/ctypes front of oracle/_build/liborc.so (built from pog_oracle.cpp and
pog_oracle_particles.cpp by oracle/build.py).  Imported only by tests/, by
__graft_entry__.smoke() and by bench.py's CPU-baseline leg; the product never imports it.
Arrays use the product's layout: x fastest, distributions [19, NZ, NY, NX], vectors
[3, NZ, NY, NX].
"""
import ctypes
import os
import threading

import numpy as np

from . import build as _build

_lock = threading.Lock()
_lib = None

_v = ctypes.c_void_p
_i = ctypes.c_int


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def load():
    global _lib
    with _lock:
        if _lib is None:
            path = _build.build()
            lib = ctypes.CDLL(path)
            for name in ("orc_build_flags", "orc_init_equilibrium_f32", "orc_step_f32",
                         "orc_step_f64", "orc_les_nu_f32", "orc_porous_force_f32",
                         "orc_particles_bin", "orc_particles_couple", "orc_trilinear_f32",
                         "orc_adjoint_step_f64", "orc_d3q19_tables", "orc_step_aa_f32", "orc_step_aa_f64"):
                getattr(lib, name).restype = _i
            lib.orc_init_equilibrium_f64.restype = _i
            lib.orc_init_equilibrium_f64.argtypes = [_v, _v, _v, ctypes.c_double, ctypes.c_double,
                                                     ctypes.c_double, ctypes.c_double]
            lib.orc_init_equilibrium_f32.argtypes = [_v, _v, _v, ctypes.c_float, ctypes.c_float,
                                                     ctypes.c_float, ctypes.c_float]
            lib.orc_equilibrium_f64.argtypes = [ctypes.c_double] * 4 + [_v]
            lib.orc_equilibrium_f32.argtypes = [ctypes.c_float] * 4 + [_v]
            lib.orc_moments_f64.argtypes = [_v, _v, _v]
            lib.orc_under_relax.argtypes = [ctypes.c_float, _v, _v, _v, _i]
            lib.orc_trilinear_f32.argtypes = [_i, _i, _i, _v, _v, _i, _v]
            lib.orc_round_storage.restype = ctypes.c_float
            lib.orc_round_storage.argtypes = [_i, ctypes.c_float, _i, ctypes.c_float]
            lib.orc_inlet_velocity_f64.argtypes = [_v, _v, _v, _i]
            lib.orc_pour_advance.restype = None
            lib.orc_filter_particles.restype = None
            lib.orc_filter_update.restype = None
            lib.orc_pressure_force.restype = None
            lib.orc_density_drive.restype = None
            for name in ("orc_phase_chemical_potential", "orc_phase_normals", "orc_phase_surface_tension",
                         "orc_phase_update", "orc_phase_properties", "orc_pour_phase"):
                getattr(lib, name).restype = None
            lib.orc_pour_advance.argtypes = [_v, _v]
            lib.orc_set_legacy_feq_order.restype = None
            lib.orc_set_legacy_feq_order.argtypes = [_i]
            _lib = lib
        return _lib


def _params(cfg, pour=None):
    """ctypes params of cfg; `pour` (float32 [POG_POUR_NFIELDS] host array) becomes the
    restatement's pour-nozzle block."""
    p = cfg.to_c()
    if pour is not None:
        p.pour_control = pour.ctypes.data_as(ctypes.c_void_p).value
    return p, ctypes.byref(p)


def filter_particles(cfg, flags, pos, vel, active, accum, seed, step):
    """Particle-filter bounce (in place on vel and accum).  flags uint32 [ncell], pos/vel float32
    [3][np], active int32 [np], accum float32 [ncell], all C-contiguous."""
    for a, dt in ((flags, np.uint32), (pos, np.float32), (vel, np.float32), (active, np.int32), (accum, np.float32)):
        assert a.dtype == dt and a.flags.c_contiguous
    lib = load()
    _, pp = _params(cfg)
    lib.orc_filter_particles(pp, _p(flags), _p(pos), _p(vel), _p(active), int(active.shape[0]), _p(accum),
                             ctypes.c_uint32(seed), ctypes.c_longlong(step))


def filter_update(cfg, flags, accum, blockage):
    """Blockage update of the porous cells (in place on accum and blockage, float32 [ncell])."""
    for a, dt in ((flags, np.uint32), (accum, np.float32), (blockage, np.float32)):
        assert a.dtype == dt and a.flags.c_contiguous
    lib = load()
    _, pp = _params(cfg)
    lib.orc_filter_update(pp, _p(flags), _p(accum), _p(blockage))


def pressure_force(cfg, flags, rho, force, scale, max_force):
    """Pressure-gradient force added in place to force (float32 [3][ncell])."""
    for a, dt in ((flags, np.uint32), (rho, np.float32), (force, np.float32)):
        assert a.dtype == dt and a.flags.c_contiguous
    lib = load()
    _, pp = _params(cfg)
    lib.orc_pressure_force(pp, _p(flags), _p(rho), _p(force), ctypes.c_float(scale), ctypes.c_float(max_force))


def density_drive(cfg, flags, rho, target, rate, max_adjust, lo, hi):
    """Density relaxation toward target [nz], in place on rho (float32 [ncell])."""
    for a, dt in ((flags, np.uint32), (rho, np.float32), (target, np.float32)):
        assert a.dtype == dt and a.flags.c_contiguous
    lib = load()
    _, pp = _params(cfg)
    lib.orc_density_drive(pp, _p(flags), _p(rho), _p(target), *(ctypes.c_float(v) for v in (rate, max_adjust, lo, hi)))


def _f32(*arrays):
    for a in arrays:
        if a is not None:
            assert a.dtype == np.float32 and a.flags.c_contiguous


def phase_chemical_potential(cfg, phi, kappa, mu):
    _f32(phi, mu)
    lib = load()
    _, pp = _params(cfg)
    lib.orc_phase_chemical_potential(pp, _p(phi), ctypes.c_float(kappa), _p(mu))


def phase_normals(cfg, phi, normal, gmag):
    _f32(phi, normal, gmag)
    lib = load()
    _, pp = _params(cfg)
    lib.orc_phase_normals(pp, _p(phi), _p(normal), _p(gmag))


def phase_surface_tension(cfg, flags, phi, normal, gmag, rho, sigma, body_force=None, curvature=None,
                          surface_force=None):
    _f32(phi, normal, gmag, rho, body_force, curvature, surface_force)
    assert flags.dtype == np.uint32
    lib = load()
    _, pp = _params(cfg)
    lib.orc_phase_surface_tension(pp, _p(flags), _p(phi), _p(normal), _p(gmag), _p(rho), ctypes.c_float(sigma),
                                  _p(body_force), _p(curvature), _p(surface_force))


def phase_update(cfg, flags, phi, phi_new, u, mu, mobility, dt, rho_air, rho_water, rho=None, phase=None):
    _f32(phi, phi_new, u, mu, rho, phase)
    assert flags.dtype == np.uint32
    lib = load()
    _, pp = _params(cfg)
    lib.orc_phase_update(pp, _p(flags), _p(phi), _p(phi_new), _p(u), _p(mu),
                         *(ctypes.c_float(v) for v in (mobility, dt, rho_air, rho_water)), _p(rho), _p(phase))


def phase_properties(cfg, phi, rho_air, rho_water, rho, phase):
    _f32(phi, rho, phase)
    lib = load()
    _, pp = _params(cfg)
    lib.orc_phase_properties(pp, _p(phi), ctypes.c_float(rho_air), ctypes.c_float(rho_water), _p(rho), _p(phase))


def pour_phase(cfg, flags, phi, dt, pour):
    _f32(phi, pour)
    assert flags.dtype == np.uint32
    lib = load()
    _, pp = _params(cfg, pour)
    lib.orc_pour_phase(pp, _p(flags), _p(phi), ctypes.c_float(dt))


def pour_advance(cfg, pour):
    """One nozzle step of a host pour block, in place."""
    lib = load()
    _, pp = _params(cfg)
    lib.orc_pour_advance(pp, _p(pour))


def tables():
    lib = load()
    cx = np.zeros(19, np.int32); cy = np.zeros(19, np.int32); cz = np.zeros(19, np.int32)
    opp = np.zeros(19, np.int32); w = np.zeros(19, np.float64)
    lib.orc_d3q19_tables(_p(cx), _p(cy), _p(cz), _p(opp), _p(w))
    return cx, cy, cz, opp, w


def build_flags(cfg) -> np.ndarray:
    lib = load()
    _, pp = _params(cfg)
    flags = np.zeros((cfg.nz, cfg.ny, cfg.nx), np.uint32)
    lib.orc_build_flags(pp, _p(flags))
    return flags


def init_equilibrium(cfg, flags, dtype=np.float64, rho0=None, u0=(0.0, 0.0, 0.0)):
    lib = load()
    _, pp = _params(cfg)
    f = np.zeros((19, cfg.nz, cfg.ny, cfg.nx), dtype)
    r = cfg.rho0 if rho0 is None else rho0
    if dtype == np.float64:
        lib.orc_init_equilibrium_f64(pp, _p(flags), _p(f), r, *u0)
    else:
        lib.orc_init_equilibrium_f32(pp, _p(flags), _p(f), r, *u0)
    return f


def step(cfg, flags, f, force=None, eps=None, u_prev=None, reductions=None, pdrag=None, pour=None,
         blockage=None, phase=None):
    """One push step.  force: [3][n] explicit force; pdrag: [4][n] particle drag deposit
    (Kp, Kv); pour: host pour-nozzle block; blockage: [n] filter blockage; phase: [n] phase
    indicator (0 air, 1 water).  Returns (f_next, rho, u)."""
    lib = load()
    _keep, pp = _params(cfg, pour)
    if blockage is not None:
        blockage = np.ascontiguousarray(blockage, np.float32)
        _keep.filter_blockage = blockage.ctypes.data_as(ctypes.c_void_p).value
    if phase is not None:
        phase = np.ascontiguousarray(phase, np.float32)
        _keep.phase = phase.ctypes.data_as(ctypes.c_void_p).value
    dt = f.dtype
    fo = f.copy()
    rho = np.zeros((cfg.nz, cfg.ny, cfg.nx), dt)
    u = np.zeros((3, cfg.nz, cfg.ny, cfg.nx), dt)
    if force is not None:
        force = np.ascontiguousarray(force, np.float32)
    if eps is not None:
        eps = np.ascontiguousarray(eps, np.float32)
    if pdrag is not None:
        pdrag = np.ascontiguousarray(pdrag, np.float32)
    if u_prev is not None:
        u_prev = np.ascontiguousarray(u_prev, dt)
    fn = lib.orc_step_f64 if dt == np.float64 else lib.orc_step_f32
    fn(pp, _p(flags), _p(f), _p(fo), _p(force), _p(pdrag), _p(eps), _p(u_prev), _p(rho), _p(u),
       _p(reductions))
    return fo, rho, u


def step_aa(cfg, flags, f, t, force=None, eps=None, pdrag=None, reductions=None, macro=False):
    """One AA-pattern step of f (AA layout, [19, NZ, NY, NX] float32 or float64, C-contiguous) in
    place at time t.  Returns (rho, u) of the step when macro, else None."""
    assert f.flags.c_contiguous and f.dtype in (np.float32, np.float64)
    lib = load()
    _keep, pp = _params(cfg)
    dt = f.dtype
    rho = np.zeros((cfg.nz, cfg.ny, cfg.nx), dt) if macro else None
    u = np.zeros((3, cfg.nz, cfg.ny, cfg.nx), dt) if macro else None
    force = None if force is None else np.ascontiguousarray(force, np.float32)
    eps = None if eps is None else np.ascontiguousarray(eps, np.float32)
    pdrag = None if pdrag is None else np.ascontiguousarray(pdrag, np.float32)
    fn = lib.orc_step_aa_f64 if dt == np.float64 else lib.orc_step_aa_f32
    rc = fn(pp, _p(np.ascontiguousarray(flags, np.uint32)), _p(f), ctypes.c_longlong(t), _p(force), _p(pdrag),
            _p(eps), _p(rho), _p(u), _p(reductions))
    if rc != 0:
        raise ValueError("the AA step restatement supports les_mode OFF or LOCAL")
    return (rho, u) if macro else None


def run(cfg, nsteps, dtype=np.float64, flags=None, force=None, eps=None, reductions=None):
    """nsteps from equilibrium.  Returns (flags, f, rho, u) of the last step (rho/u are the
    moments computed inside that step)."""
    if flags is None:
        flags = build_flags(cfg)
    f = init_equilibrium(cfg, flags, dtype)
    u = np.zeros((3, cfg.nz, cfg.ny, cfg.nx), dtype)
    rho = None
    for _ in range(nsteps):
        f, rho, u_new = step(cfg, flags, f, force=force, eps=eps,
                             u_prev=u if cfg.les_mode == 1 else None, reductions=reductions)
        u = u_new
    return flags, f, rho, u


def les_nu(cfg, flags, u):
    lib = load()
    _, pp = _params(cfg)
    u = np.ascontiguousarray(u, np.float32)
    nu = np.zeros((cfg.nz, cfg.ny, cfg.nx), np.float32)
    lib.orc_les_nu_f32(pp, _p(flags), _p(u), _p(nu))
    return nu


def porous_force(cfg, flags, rho, u):
    lib = load()
    _, pp = _params(cfg)
    F = np.zeros((3, cfg.nz, cfg.ny, cfg.nx), np.float32)
    lib.orc_porous_force_f32(pp, _p(flags), _p(np.ascontiguousarray(rho, np.float32)),
                             _p(np.ascontiguousarray(u, np.float32)), _p(F))
    return F


class legacy_feq_order:
    """Context manager: inside it the oracle's collision builds f_eq for directions 7-18 with the
    velocity table of the reference's lbm_algorithms.py (as its legacy collision does) while it
    streams with config/core.py's.  Test-only: it reproduces a reference defect so that the rest of
    the step can be pinned against the reference's own kernels."""

    def __enter__(self):
        load().orc_set_legacy_feq_order(1)
        return self

    def __exit__(self, *exc):
        load().orc_set_legacy_feq_order(0)
        return False


def equilibrium(rho, u, dtype=np.float64):
    lib = load()
    out = np.zeros(19, dtype)
    if dtype == np.float64:
        lib.orc_equilibrium_f64(rho, *u, _p(out))
    else:
        lib.orc_equilibrium_f32(rho, *u, _p(out))
    return out


def moments(f):
    lib = load()
    f = np.ascontiguousarray(f, np.float64)
    rho = np.zeros(1); u = np.zeros(3)
    lib.orc_moments_f64(_p(f), _p(rho), _p(u))
    return float(rho[0]), u


def trilinear(u, pos):
    """u: [3, NZ, NY, NX] float32; pos: (m, 3) float32 -> (m, 3)."""
    lib = load()
    u = np.ascontiguousarray(u, np.float32)
    pos = np.ascontiguousarray(pos, np.float32)
    out = np.zeros_like(pos)
    nz, ny, nx = u.shape[1:]
    lib.orc_trilinear_f32(nx, ny, nz, _p(u), _p(pos), pos.shape[0], _p(out))
    return out


def under_relax(alpha, fnew, fold):
    lib = load()
    fnew = np.ascontiguousarray(fnew, np.float32)
    fold = np.ascontiguousarray(fold, np.float32).copy()
    out = np.zeros_like(fnew)
    lib.orc_under_relax(alpha, _p(fnew), _p(fold), _p(out), fnew.size)
    return out, fold


def particles_bin(cfg, pos, active):
    lib = load()
    _, pp = _params(cfg)
    pos = np.ascontiguousarray(pos, np.float32)
    active = np.ascontiguousarray(active, np.int32)
    n = active.shape[0]
    keys = np.zeros(n, np.int32)
    perm = np.zeros(n, np.int32)
    lib.orc_particles_bin(pp, _p(pos), _p(active), n, _p(keys), _p(perm))
    return keys, perm


def particles_couple(cfg, pcfg, pos, vel, diam, drag_old, active, u, force_fix=None, pour=None):
    """One coupling pass (serial, id order) on copies of the state.  Returns the updated
    (pos, vel, drag_old, active, force_fix, u_at); force_fix is the [4][n] int64 drag deposit
    (Kp, Kv) scaled by 2^32.  pour: host pour-nozzle block (impact force)."""
    lib = load()
    _keep, pp = _params(cfg, pour)
    ppp = pcfg.to_c()
    pos = np.ascontiguousarray(pos, np.float32).copy()
    vel = np.ascontiguousarray(vel, np.float32).copy()
    diam = np.ascontiguousarray(diam, np.float32)
    drag_old = np.ascontiguousarray(drag_old, np.float32).copy()
    active = np.ascontiguousarray(active, np.int32).copy()
    u = np.ascontiguousarray(u, np.float32)
    n = diam.shape[0]
    if force_fix is None:
        force_fix = np.zeros(4 * cfg.ncell, np.int64)
    u_at = np.zeros((3, n), np.float32)
    lib.orc_particles_couple(pp, ctypes.byref(ppp), _p(pos), _p(vel), _p(diam), _p(drag_old),
                             _p(active), n, _p(u), _p(force_fix), _p(u_at))
    return pos, vel, drag_old, active, force_fix, u_at


def adjoint_step(cfg, flags, f_t, lam_next, eps=None, grad_eps=None, grad_inlet=None, pdrag=None,
                 u_prev=None, mu_in=None, mu_out=None):
    """Adjoint of one FP64 push step by forward-mode dual numbers; pdrag: the step's particle drag
    deposit [4][n] (float32), held fixed.  LES stencil mode: u_prev [3][n] the velocity the step's
    nu_sgs reads, mu_in dJ/du of the velocity the step outputs, mu_out (float64 [3][n], added to)
    receives dJ/du_prev."""
    lib = load()
    _, pp = _params(cfg)
    lam_t = np.zeros_like(lam_next)
    if eps is not None:
        eps = np.ascontiguousarray(eps, np.float32)
    if pdrag is not None:
        pdrag = np.ascontiguousarray(pdrag, np.float32)
    if u_prev is not None:
        u_prev = np.ascontiguousarray(u_prev, np.float64)
    if mu_in is not None:
        mu_in = np.ascontiguousarray(mu_in, np.float64)
    if mu_out is not None:
        assert mu_out.dtype == np.float64 and mu_out.flags.c_contiguous
    rc = lib.orc_adjoint_step_f64(pp, _p(flags), _p(np.ascontiguousarray(f_t, np.float64)),
                                  _p(np.ascontiguousarray(lam_next, np.float64)), _p(lam_t), _p(eps), _p(pdrag),
                                  _p(u_prev), _p(mu_in), _p(mu_out), _p(grad_eps), _p(grad_inlet))
    if rc != 0:
        raise ValueError("the stencil-mode adjoint needs u_prev")
    return lam_t


def outflow_loss(cfg, nsteps, flags=None, eps=None):
    """J = sum over steps of the outflow flux, FP64 forward."""
    red = np.zeros(6, np.float64)
    run(cfg, nsteps, np.float64, flags=flags, eps=eps, reductions=red)
    return float(red[4])


def outflow_gradient(cfg, nsteps, flags=None, eps=None):
    """Adjoint of outflow_loss by storing every state (small grids only)."""
    if flags is None:
        flags = build_flags(cfg)
    f = init_equilibrium(cfg, flags, np.float64)
    stencil = cfg.les_mode == 1
    u = np.zeros((3, cfg.nz, cfg.ny, cfg.nx), np.float64)
    states, uprevs = [], []
    for _ in range(nsteps):
        states.append(f)
        uprevs.append(u)
        f, _, u = step(cfg, flags, f, eps=eps, u_prev=u if stencil else None)
    lam = np.zeros_like(f)
    mu = np.zeros((3, cfg.nz, cfg.ny, cfg.nx), np.float64)
    ge = np.zeros((cfg.nz, cfg.ny, cfg.nx), np.float64) if eps is not None else None
    gi = np.zeros(16, np.float64)
    for t in reversed(range(nsteps)):
        mu_out = np.zeros_like(mu) if stencil else None
        lam = adjoint_step(cfg, flags, states[t], lam, eps=eps, grad_eps=ge, grad_inlet=gi,
                           u_prev=uprevs[t] if stencil else None, mu_in=mu if stencil else None, mu_out=mu_out)
        if stencil:
            mu = mu_out
    return ge, gi
