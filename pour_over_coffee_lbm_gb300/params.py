"""Parameter blocks of libpog.so (ctypes mirrors of include/pog.h) and the workload presets.

Field names follow the reference's config module where one exists (config/core.py:23-93:
NX, NY, NZ, TAU_WATER, SMAGORINSKY_CONSTANT ...); `from_reference_config` maps a reference
`config` module onto a parameter block for drop-in use.
"""
import ctypes
import dataclasses
import math

import numpy as np

STORE_F32, STORE_F16S, STORE_BF16S, STORE_F64 = 0, 1, 2, 3
STORAGE_NAMES = {"f32": STORE_F32, "f16s": STORE_F16S, "bf16s": STORE_BF16S, "f64": STORE_F64}
LES_OFF, LES_STENCIL, LES_LOCAL = 0, 1, 2
DRAG_SEMI_IMPLICIT, DRAG_EXPLICIT_CAP = 0, 1
REACTION_IMPLICIT, REACTION_EXPLICIT, REACTION_EXPLICIT_NEW = 0, 1, 2
FORCING_GUO, FORCING_REFERENCE = 0, 1
STEP_AUTO, STEP_CELLS = 0, 1
INLET_NCOEF = 16

CELL_SOLID, CELL_INLET, CELL_OUTLET, CELL_POROUS, CELL_NEAR_SOLID = 0x01, 0x02, 0x04, 0x08, 0x10

RED_MASS, RED_MOMX, RED_MOMY, RED_MOMZ, RED_OUTFLOW, RED_NONFINITE = range(6)
RED_COUNT = 6


class PogParams(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
        ("storage", ctypes.c_int32), ("les_mode", ctypes.c_int32), ("drag_mode", ctypes.c_int32),
        ("forcing_mode", ctypes.c_int32), ("clamp_tau", ctypes.c_int32),
        ("tau", ctypes.c_float), ("rho0", ctypes.c_float),
        ("gx", ctypes.c_float), ("gy", ctypes.c_float), ("gz", ctypes.c_float),
        ("cs_smag", ctypes.c_float), ("les_strain_floor", ctypes.c_float),
        ("les_nu_max", ctypes.c_float), ("tau_min", ctypes.c_float), ("tau_max", ctypes.c_float),
        ("cone_apex_z", ctypes.c_float), ("cone_half_angle_deg", ctypes.c_float),
        ("cone_wall", ctypes.c_float), ("hole_radius", ctypes.c_float),
        ("inlet_radius", ctypes.c_float), ("band_thickness", ctypes.c_float),
        ("center_x", ctypes.c_float), ("center_y", ctypes.c_float),
        ("porosity", ctypes.c_float), ("permeability", ctypes.c_float),
        ("forchheimer", ctypes.c_float), ("drag_cap", ctypes.c_float),
        ("u_inlet", ctypes.c_float), ("inlet_coef", ctypes.c_float * INLET_NCOEF),
        ("rho_outlet", ctypes.c_float),
        ("inlet_control", ctypes.c_void_p),
        ("pour_control", ctypes.c_void_p),
        ("filter_blockage", ctypes.c_void_p),
        ("phase", ctypes.c_void_p), ("tau_air", ctypes.c_float),
        ("deposit_mask", ctypes.c_void_p),
        ("wall_cells", ctypes.c_void_p), ("n_wall_cells", ctypes.c_int32),
        ("step_kernel", ctypes.c_int32),
        ("density_ref", ctypes.c_void_p),
    ]


class PogParticleParams(ctypes.Structure):
    _fields_ = [
        ("density_ratio", ctypes.c_float), ("relaxation", ctypes.c_float), ("dt", ctypes.c_float),
        ("drag_model", ctypes.c_int32), ("deterministic", ctypes.c_int32),
        ("wall_margin", ctypes.c_float), ("wall_pullback", ctypes.c_float),
        ("wall_damping", ctypes.c_float), ("z_floor", ctypes.c_float),
        ("deposit_cells", ctypes.c_void_p), ("deposit_mask", ctypes.c_void_p),
        ("reaction", ctypes.c_int32),
    ]


@dataclasses.dataclass
class LatticeConfig:
    """One lattice workload (lattice units).  Defaults = the 64^3 plain-method case."""
    nx: int = 64
    ny: int = 64
    nz: int = 64
    storage: int = STORE_F32
    les_mode: int = LES_OFF
    drag_mode: int = DRAG_SEMI_IMPLICIT
    forcing_mode: int = FORCING_GUO
    clamp_tau: bool = False
    tau: float = 0.8
    tau_air: float = 0.8
    rho0: float = 1.0
    gravity: tuple = (0.0, 0.0, -1e-5)
    cs_smag: float = 0.1
    les_strain_floor: float = 1e-3
    les_nu_max: float = 0.1
    tau_min: float = 0.55
    tau_max: float = 1.90
    cone_apex_z: float = 4.0
    cone_half_angle_deg: float = 30.0
    cone_wall: float = 2.0
    hole_radius: float = 2.0
    inlet_radius: float = 6.0
    band_thickness: float = 0.0
    center_x: float = -1.0
    center_y: float = -1.0
    porosity: float = 0.6
    permeability: float = 1e-3
    forchheimer: float = 0.55
    drag_cap: float = 1e-4
    u_inlet: float = -0.02
    inlet_coef: tuple = (0.0,) * INLET_NCOEF
    rho_outlet: float = 1.0

    @property
    def ncell(self) -> int:
        return self.nx * self.ny * self.nz

    def to_c(self) -> PogParams:
        p = PogParams()
        for f in ("nx", "ny", "nz", "storage", "les_mode", "drag_mode", "forcing_mode"):
            setattr(p, f, int(getattr(self, f)))
        p.clamp_tau = int(bool(self.clamp_tau))
        for f in ("tau", "tau_air", "rho0", "cs_smag", "les_strain_floor", "les_nu_max", "tau_min",
                  "tau_max", "cone_apex_z", "cone_half_angle_deg", "cone_wall", "hole_radius",
                  "inlet_radius", "band_thickness", "center_x", "center_y", "porosity",
                  "permeability", "forchheimer", "drag_cap", "u_inlet", "rho_outlet"):
            setattr(p, f, float(getattr(self, f)))
        p.gx, p.gy, p.gz = (float(v) for v in self.gravity)
        coef = list(self.inlet_coef) + [0.0] * INLET_NCOEF
        for k in range(INLET_NCOEF):
            p.inlet_coef[k] = float(coef[k])
        return p

    def replace(self, **kw) -> "LatticeConfig":
        return dataclasses.replace(self, **kw)

    @property
    def nu0(self) -> float:
        return (self.tau - 0.5) / 3.0

    @property
    def tan_half_angle(self) -> float:
        return math.tan(math.radians(self.cone_half_angle_deg))

    @property
    def axis(self):
        cx = 0.5 * self.nx if self.center_x < 0 else self.center_x
        cy = 0.5 * self.ny if self.center_y < 0 else self.center_y
        return cx, cy


@dataclasses.dataclass
class ParticleConfig:
    """Lagrangian coffee-particle model (coffee_particles.py), lattice units."""
    count: int = 0
    median_diameter: float = 0.6
    sigma_log: float = 0.35
    density_ratio: float = 1.2
    relaxation: float = 0.8
    dt: float = 1.0
    drag_model: int = 0
    deterministic: bool = False
    wall_margin: float = 0.9
    wall_pullback: float = 0.8
    wall_damping: float = 0.3
    z_floor: float = 3.0
    seed: int = 1234
    sort_interval: int = 20
    reaction: int = REACTION_IMPLICIT

    def to_c(self) -> PogParticleParams:
        pp = PogParticleParams()
        pp.density_ratio = self.density_ratio
        pp.relaxation = self.relaxation
        pp.dt = self.dt
        pp.drag_model = int(self.drag_model)
        pp.deterministic = int(bool(self.deterministic))
        pp.wall_margin = self.wall_margin
        pp.wall_pullback = self.wall_pullback
        pp.wall_damping = self.wall_damping
        pp.z_floor = self.z_floor
        pp.reaction = int(self.reaction)
        return pp


# ---- the five workloads (lattice units; sizes and physics as stated) ----------------------------
def plain_64() -> LatticeConfig:
    """D3Q19 BGK single phase 64^3 FP32, tau 0.8, Guo gravity, V60 cone, 200 steps."""
    return LatticeConfig()


def coupled_128(les_mode: int = LES_LOCAL):
    """128^3 + Smagorinsky Cs 0.1 + 3-cell porous band + 20,000 particles, 1,000 steps."""
    return (LatticeConfig(nx=128, ny=128, nz=128, les_mode=les_mode, band_thickness=3.0),
            ParticleConfig(count=20000))


def precision_256(storage: int = STORE_F32, les_mode: int = LES_LOCAL, band: float = 3.0) -> LatticeConfig:
    """256^3, distributions in FP32 / FP16S / BF16S / FP64, 2,000 steps."""
    return LatticeConfig(nx=256, ny=256, nz=256, storage=storage, les_mode=les_mode,
                         band_thickness=band)


def differentiation_96():
    """96^3 + band with per-cell porosity 0.6 +- 0.05, 16-coefficient inlet profile, 500 steps,
    checkpoints every 50."""
    return (LatticeConfig(nx=96, ny=96, nz=96, les_mode=LES_LOCAL, band_thickness=3.0),
            ParticleConfig(count=5000))


def scale_320x384():
    """320x320x384 FP16S + LES + band + 1,000,000 particles."""
    return (LatticeConfig(nx=320, ny=320, nz=384, storage=STORE_F16S, les_mode=LES_LOCAL,
                          band_thickness=3.0), ParticleConfig(count=1000000))


def from_reference_config(cfg, **overrides) -> LatticeConfig:
    """Map a reference `config` module (NX, NY, NZ, TAU_WATER, SMAGORINSKY_CONSTANT, ...)
    onto a LatticeConfig.  Physical constants the reference derives (GRAVITY_LU = 44.1 ...)
    are not taken over: they make the step unstable without the reference's clamps."""
    lc = LatticeConfig(nx=int(getattr(cfg, "NX", 64)), ny=int(getattr(cfg, "NY", 64)),
                       nz=int(getattr(cfg, "NZ", 64)))
    if hasattr(cfg, "TAU_WATER"):
        lc.tau = float(cfg.TAU_WATER)
    if hasattr(cfg, "SMAGORINSKY_CONSTANT"):
        lc.cs_smag = float(cfg.SMAGORINSKY_CONSTANT)
    if hasattr(cfg, "RHO_0"):
        lc.rho0 = float(cfg.RHO_0)
    return lc.replace(**overrides)


# ---- seeded synthetic inputs --------------------------------------------------------------------
def porosity_field(cfg: LatticeConfig, flags: np.ndarray, seed: int = 1234,
                   amplitude: float = 0.05) -> np.ndarray:
    """Per-cell porosity eps = porosity + amplitude*U(-1,1) on porous cells (porosity
    elsewhere), float32, x-fastest flat layout.  PCG64 seeded."""
    rng = np.random.Generator(np.random.PCG64(seed))
    eps = np.full(cfg.ncell, cfg.porosity, dtype=np.float32)
    band = (flags.reshape(-1) & CELL_POROUS) != 0
    eps[band] = (cfg.porosity + amplitude * rng.uniform(-1.0, 1.0, int(band.sum()))).astype(np.float32)
    return eps


def seed_particles(cfg: LatticeConfig, pc: ParticleConfig):
    """Particles uniform in the lower cone (rejection sampling inside 0.8 of the cone radius),
    log-normal diameters (median `median_diameter`, log-sigma `sigma_log`).  Returns SoA
    float32 arrays pos[3][n], vel[3][n] (zero), diameter[n] and int32 active[n] (ones)."""
    n = int(pc.count)
    rng = np.random.Generator(np.random.PCG64(pc.seed))
    cx, cy = cfg.axis
    t = cfg.tan_half_angle
    z_lo = cfg.cone_apex_z + pc.z_floor + 1.0
    z_hi = cfg.cone_apex_z + 0.4 * (cfg.nz - 3 - cfg.cone_apex_z)
    out = np.empty((3, n), dtype=np.float64)
    got = 0
    while got < n:
        m = max(1024, 2 * (n - got))
        z = rng.uniform(z_lo, z_hi, m)
        rmax = 0.8 * (z - cfg.cone_apex_z) * t
        # uniform in the box around the cone, keep points inside
        x = rng.uniform(-1.0, 1.0, m) * rmax.max()
        y = rng.uniform(-1.0, 1.0, m) * rmax.max()
        keep = (x * x + y * y) <= rmax * rmax
        x, y, z = x[keep], y[keep], z[keep]
        k = min(n - got, len(z))
        out[0, got:got + k] = cx + x[:k]
        out[1, got:got + k] = cy + y[:k]
        out[2, got:got + k] = z[:k]
        got += k
    d = np.exp(rng.normal(math.log(pc.median_diameter), pc.sigma_log, n))
    pos = out.astype(np.float32)
    vel = np.zeros((3, n), dtype=np.float32)
    return pos, vel, d.astype(np.float32), np.ones(n, dtype=np.int32)
