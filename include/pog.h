/*
 * pog.h -- C ABI of libpog.so, the GB300 (sm_103a) D3Q19 lattice-Boltzmann step and
 * Lagrangian coffee-particle coupling of the pour-over V60 simulator.
 *
 * The reference (latteine1217/pour-over-coffee-lbm) is Python + Taichi and has no FFI: its
 * "operator API" is the solver object (src/core/lbm_protocol.py:12-238, the legacy
 * LBMSolver in src/core/legacy/lbm_solver.py and CoffeeParticleSystem in
 * src/physics/coffee_particles.py).  Each entry point below replaces one Taichi kernel (or a
 * fused group of them) of that object; the replaced reference code is cited beside it.  The
 * Python package pour_over_coffee_lbm_gb300 binds these with ctypes and exposes the
 * reference's solver protocol and accessors on top.
 *
 * Conventions
 *   - Every pointer argument is caller-owned DEVICE memory (for example a torch CUDA
 *     tensor) unless the comment says "host".  The library allocates no device memory.
 *   - Fields are structure-of-arrays with x fastest: cell index c = (k*ny + j)*nx + i, a
 *     distribution array is f[q*ncell + c], a vector field is v[a*ncell + c] (a = x,y,z).
 *   - Calls are stream-ordered on the cudaStream_t passed as `stream` (0 = legacy default
 *     stream).  Nothing synchronises the host unless stated.
 *   - Return value: 0 (POG_OK) on success, a negative POG_E_* code on failure; the message
 *     is available from pog_last_error() (thread-local).  No exception crosses the ABI and
 *     the library never exits the process.
 *   - D3Q19 ordering is the reference's config/core.py:36-47 ordering; opposite(q) is
 *     {0,2,1,4,3,6,5,10,9,8,7,14,13,12,11,18,17,16,15} (legacy/lbm_solver.py:431-439).
 */
#ifndef POG_H
#define POG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define POG_VERSION 2

/* ---- error codes ---------------------------------------------------------------------- */
#define POG_OK 0
#define POG_E_ARG (-1)      /* invalid argument (null pointer, bad size, bad enum)         */
#define POG_E_CUDA (-2)     /* a CUDA runtime call failed                                    */
#define POG_E_NAN (-3)      /* a non-finite density or velocity was detected                 */
#define POG_E_INJECTED (-4) /* host-side fault injection (POG_FAULT_INJECT_STEP) fired       */
#define POG_E_RANGE (-5)    /* a size is beyond a documented limit                           */
#define POG_E_STATE (-6)    /* call sequence error (e.g. odd AA parity where even required)  */

/* ---- cell flag word (one uint32 per cell) --------------------------------------------------
 * Low byte: the cell's own flags below.  Bit POG_LINK_SHIFT + q (q = 1..18) is set when the
 * neighbour c + e_q is solid, so bounce-back needs no neighbour reads in the step kernels. */
#define POG_LINK_SHIFT 8
#define POG_CELL_SOLID 0x01u      /* half-way bounce-back wall (filter_paper.py:206-286)     */
#define POG_CELL_INLET 0x02u      /* fixed-velocity inlet disk (equilibrium at rho_local)    */
#define POG_CELL_OUTLET 0x04u     /* pressure outlet under the apex hole (equilibrium rho_out)*/
#define POG_CELL_POROUS 0x08u     /* filter-paper band: Darcy-Forchheimer drag, LES off      */
#define POG_CELL_NEAR_SOLID 0x10u /* at least one of the 18 neighbours is solid              */

/* ---- enums -------------------------------------------------------------------------------- */
enum pog_storage {     /* how the distributions are stored in HBM                           */
  POG_STORE_F32 = 0,   /* float (f_i - w_i*rho0); collision in FP32 on the deviations        */
  POG_STORE_F16S = 1,  /* IEEE half of (f_i - w_i*rho0)*2^12; collision in FP32              */
  POG_STORE_BF16S = 2, /* bfloat16 of (f_i - w_i*rho0); collision in FP32                    */
  POG_STORE_F64 = 3    /* double (f_i - w_i*rho0); collision in FP64 (reference runs)       */
};
/* The stored form is internal: pog_export_natural / pog_import_natural convert to and from
 * plain f_i in FP32 or FP64 for every storage. */
enum pog_les_mode {
  POG_LES_OFF = 0,
  POG_LES_STENCIL = 1, /* |S| by central differences of the previous step's u
                          (les_turbulence.py:318-380); needs the u ping-pong buffers         */
  POG_LES_LOCAL = 2    /* |S| from the local non-equilibrium stress (Hou et al. 1996)         */
};
enum pog_drag_mode {
  POG_DRAG_SEMI_IMPLICIT = 0, /* velocity solved with the drag (Guo & Zhao 2002)             */
  POG_DRAG_EXPLICIT_CAP = 1   /* reference form: drag from the force-free velocity, |F| capped
                                 (filter_paper.py:471-536)                                    */
};
enum pog_forcing_mode {
  POG_FORCING_GUO = 0,       /* standard Guo 2002 (docs/mathematical/mathematical_models.md)  */
  POG_FORCING_REFERENCE = 1  /* legacy form 3e.F + 9(e.u)(u.F) with its clamps
                                (legacy/lbm_solver.py:594-607,688-764)                        */
};

#define POG_INLET_NCOEF 16

/* Run-time parameters of one lattice (lattice units throughout).  Field names follow the
 * reference's config names where one exists (config/core.py, config/physics.py). */
typedef struct pog_params {
  int32_t nx, ny, nz;       /* NX, NY, NZ                                                     */
  int32_t storage;          /* enum pog_storage                                               */
  int32_t les_mode;         /* enum pog_les_mode                                              */
  int32_t drag_mode;        /* enum pog_drag_mode                                             */
  int32_t forcing_mode;     /* enum pog_forcing_mode                                          */
  int32_t clamp_tau;        /* 1: clamp tau_eff into [tau_min, tau_max] (lbm_solver.py:571)   */
  float tau;                /* molecular relaxation time (TAU_WATER)                          */
  float rho0;               /* reference density, also the storage shift                     */
  float gx, gy, gz;         /* gravity acceleration; force density is rho*g                   */
  float cs_smag;            /* Smagorinsky constant (SMAGORINSKY_CONSTANT)                    */
  float les_strain_floor;   /* |S| below which nu_sgs = 0 (reference 1e-3)                    */
  float les_nu_max;         /* upper clamp of nu_sgs (reference 0.1)                           */
  float tau_min, tau_max;   /* tau_eff clamp when clamp_tau (reference 0.55, 1.90)            */
  /* V60 geometry (filter_paper.py:206-364), lattice units */
  float cone_apex_z;        /* z of the cone apex                                             */
  float cone_half_angle_deg;/* half angle of the cone                                         */
  float cone_wall;          /* horizontal wall thickness                                      */
  float hole_radius;        /* radius of the drain hole through the apex                      */
  float inlet_radius;       /* radius of the inlet disk on plane k = nz-2                     */
  float band_thickness;     /* filter-paper band thickness inside the wall (0 = none)         */
  float center_x, center_y; /* cone axis; negative = nx*0.5, ny*0.5 (filter_paper.py:229)     */
  /* filter-paper porous band (filter_paper.py:423-536) */
  float porosity;           /* eps0 at which permeability/forchheimer are quoted              */
  float permeability;       /* Darcy permeability K0 (lattice units)                          */
  float forchheimer;        /* Forchheimer coefficient C_F0                                   */
  float drag_cap;           /* |F_drag| cap in POG_DRAG_EXPLICIT_CAP mode                      */
  /* inlet / outlet */
  float u_inlet;            /* base inlet velocity u_z (negative = downward)                   */
  float inlet_coef[POG_INLET_NCOEF]; /* radial profile: u_z(r) = u_inlet*(1 + sum a_k T_k(2r/R-1)) */
  float rho_outlet;         /* density imposed on outlet cells                                */
  /* Optional DEVICE pointer to a pour-control block [u_inlet, a_0 .. a_15] (17 floats) that
   * overrides u_inlet/inlet_coef when non-null, so a time-varying pour is fed by one small
   * host-to-device copy per step (and survives CUDA-graph replay).  NULL = use the fields. */
  const float* inlet_control;
  /* Optional DEVICE pointer to a pour-nozzle block (POG_POUR_* below) or NULL.  While its
   * ACTIVE field is non-zero, pog_step adds the nozzle's downward force to the fluid and
   * pog_particles_couple adds the stream's impact force to the particles near it. */
  const float* pour_control;
  /* Optional DEVICE pointer to the filter-paper blockage field b [ncell] (pog_filter_update) or
   * NULL: porous cells scale their Darcy and Forchheimer coefficients by (1 + b[c])
   * (apply_filter_effects' blockage_factor, filter_paper.py:584-587). */
  const float* filter_blockage;
  /* Optional DEVICE pointer to the phase indicator [ncell] (lbm.phase: 0 = air, 1 = water) or
   * NULL (water everywhere).  Per cell (legacy/lbm_solver.py:558-592, les_turbulence.py:362-366):
   * gravity rho*g*phase where phase > 0.001 and none elsewhere; tau = tau where phase > 0.5,
   * else tau_air; nu_sgs = 0 where |phase| < 0.9. */
  const float* phase;
  float tau_air;            /* molecular relaxation time of the air phase (TAU_AIR)           */
  /* Optional DEVICE bit mask [ceil(ncell/32)] or NULL: bit c set where the particle drag deposit
   * pdrag may be nonzero (pog_particles_couple sets the bits of the cells it deposits into,
   * pog_particles_clear_deposit clears them).  With a mask the step reads pdrag only at set bits
   * and takes zero elsewhere; the caller keeps pdrag zero wherever the bit is clear. */
  const uint32_t* deposit_mask;
  /* Optional DEVICE list of the cells pog_wall_list returns (fluid cells with a solid neighbour),
   * n_wall_cells entries, or NULL.  Non-null selects the row-tiled step kernel in pog_step: whole
   * grid rows staged through shared memory by bulk TMA copies, bounce-back through per-link
   * mailbox slots copied by a pass over these cells around each odd step.  It needs nx * element
   * size to be a multiple of 16 bytes, nx <= 320 and a 16-byte aligned distribution buffer, and
   * serves FP32/FP16S/BF16S storage; otherwise pog_step takes the register-staged kernel.  Both
   * compute the same update and leave the same state between steps. */
  const int32_t* wall_cells;
  int32_t n_wall_cells;
  /* enum pog_step_kernel: which register-staged step kernel pog_step runs when wall_cells is NULL.
   * POG_STEP_AUTO: FP16S/BF16S storage takes the two-cell kernel (two x-adjacent cells per
   * thread, paired 32-bit population accesses, packed FP32x2 collision) where it applies -- even
   * nx, Guo forcing, no phase field, LES off or local -- and every other case the per-cell
   * kernel.  POG_STEP_CELLS: the per-cell kernel always.  Both compute the same update; the
   * two-cell kernel's collision rounds differently in FP32, so 16-bit stored values can differ
   * by one unit in their last place. */
  int32_t step_kernel;
  /* Optional DEVICE array [ncell] of IEEE half values d_c, or NULL (FP16S storage only).  With it,
   * FP16S stores each slot relative to the reference density rho0 + d_c of the cell that owns
   * the slot instead of rho0: every even step a cell sets d_c to its density deviation (rounded
   * to FP16) and re-encodes its populations, every odd step moves the populations it streams
   * between its neighbours' references and its own.  The stored deviations then carry the
   * velocity information without the pressure waves' density swing, which FP16's 11-bit
   * significand otherwise rounds against (u error against FP64 at 256^3 LES + band after 2,000
   * steps: 8.2e-4 with references, 2.4e-3 without).  pog_init_equilibrium sets it; pog_export_natural /
   * pog_import_natural / pog_macroscopic read it; pog_step_push rejects it; the two-cell and
   * row-tiled kernels do not run with it.  Keep it with the distributions (checkpoints, halos):
   * the stored state means nothing without it.  No counterpart in the reference. */
  void* density_ref;
} pog_params;

enum pog_step_kernel { POG_STEP_AUTO = 0, POG_STEP_CELLS = 1 };

/* Pour-nozzle block, floats (PrecisePouringSystem, src/physics/precise_pouring.py:12-193):
 * a stream of radius R ending at plane ZTOP, HEIGHT planes tall, centred at (X, Y).  A fluid cell
 * at distance r <= R from the axis on plane ZTOP - HEIGHT <= k <= ZTOP receives the force
 * density -min(VELOCITY * I * FLOW / DT, ACCEL_CAP) e_z, I = exp(-(r/R)^2 / 2) exp(-(ZTOP - k)/2)
 * (apply_pouring_force :132-160, _is_in_pouring_region :100-130).  pog_pour_advance moves the
 * nozzle: TIME += DT, then (X, Y) = (CX, CY) (PATTERN 0) or the growing spiral (PATTERN 1)
 * t = TIME*SPIRAL_SPEED, r = SPIRAL_R (1 + 0.1 t), (CX + r cos t, CY + r sin t) clamped to
 * [DIAMETER, nx - DIAMETER] x [DIAMETER, ny - DIAMETER] (_get_current_pour_position :81-98).
 * A particle within 2R of the axis and above IMPACT_ZMIN feels -IMPACT I e_z plus a radial push
 * 0.3 IMPACT I along (dx, dy)/r (for r > 0.1), I = exp(-(r/R)^2 / 2), |F| <= IMPACT_MAX
 * (create_water_impact_force :190-226); IMPACT = 0 turns it off. */
#define POG_POUR_ACTIVE 0
#define POG_POUR_X 1
#define POG_POUR_Y 2
#define POG_POUR_RADIUS 3
#define POG_POUR_ZTOP 4
#define POG_POUR_HEIGHT 5
#define POG_POUR_VELOCITY 6
#define POG_POUR_FLOW 7
#define POG_POUR_DT 8
#define POG_POUR_ACCEL_CAP 9
#define POG_POUR_PATTERN 10
#define POG_POUR_CX 11
#define POG_POUR_CY 12
#define POG_POUR_SPIRAL_R 13
#define POG_POUR_SPIRAL_SPEED 14
#define POG_POUR_TIME 15
#define POG_POUR_DIAMETER 16
#define POG_POUR_IMPACT 17
#define POG_POUR_IMPACT_MAX 18
#define POG_POUR_IMPACT_ZMIN 19
#define POG_POUR_NFIELDS 20

/* Reduction slots written by pog_step when `reductions` is non-null (FP64, accumulated with
 * atomics: zero them before a call to get that call's sums).  Replaces the host-side np.sum
 * conservation checks of src/visualization/lbm_diagnostics.py:228-291. */
#define POG_RED_MASS 0      /* sum over fluid cells of rho                                   */
#define POG_RED_MOMX 1      /* sum of rho*u_x                                                */
#define POG_RED_MOMY 2
#define POG_RED_MOMZ 3
#define POG_RED_OUTFLOW 4   /* outflow mass flux: -sum over outlet cells of sum_i c_iz f_i   */
#define POG_RED_NONFINITE 5 /* number of cells whose rho or u is not finite                  */
#define POG_RED_COUNT 6

/* Particle-model parameters (coffee_particles.py:1048-1212, 641-831). */
typedef struct pog_particle_params {
  float density_ratio;  /* rho_p / rho0                                                       */
  float relaxation;     /* under-relaxation alpha of the drag force (lbm_solver.py:1485: 0.8)  */
  float dt;             /* particle time step (lattice units)                                 */
  int32_t drag_model;   /* 0 Stokes, 1 Schiller-Naumann correction (coffee_particles.py:1088)  */
  int32_t deterministic;/* 1: fixed-point integer accumulation of the drag deposit           */
  float wall_margin;    /* radial limit as a fraction of the cone radius (0.9)                 */
  float wall_pullback;  /* radius a violating particle is moved to, fraction (0.8)             */
  float wall_damping;   /* velocity factor on a wall hit (0.3)                                 */
  float z_floor;        /* particles are kept above cone_apex_z + z_floor                      */
  /* Optional DEVICE array [np] or NULL: pog_particles_couple writes the base cell (i, j, k
   * corner) of each particle's 8-cell drag deposit, -1 for a particle that deposited nothing, so
   * that pog_particles_clear_deposit can zero exactly those cells after the lattice step. */
  int32_t* deposit_cells;
  /* Optional DEVICE bit mask [ceil(ncell/32)] or NULL: the coupling pass sets bit c for every
   * cell it deposits into (see pog_params.deposit_mask). */
  uint32_t* deposit_mask;
  /* How the particles act on the fluid (enum pog_reaction). */
  int32_t reaction;
} pog_particle_params;

/* Particle-to-fluid exchange of pog_particles_couple.  The deposit pdrag = (Kp, Kv) enters the
 * step as the force Kv - Kp u with u implicit, so an explicit force is a deposit with Kp = 0. */
enum pog_reaction {
  POG_REACTION_IMPLICIT = 0,     /* Kp = w beta, Kv = w beta v_new: the drag beta (v_new - u)
                                    taken with the fluid's updated u (stable at any loading)     */
  POG_REACTION_EXPLICIT = 1,     /* Kp = 0, Kv = -w F: the reaction of the relaxed drag F that
                                    moves the particle, spread with the trilinear weights
                                    (distribute_force_to_grid, coffee_particles.py:1048-1086,
                                    added as a body force, legacy/lbm_solver.py:1478-1483)       */
  POG_REACTION_EXPLICIT_NEW = 2  /* Kp = 0, Kv = -w F_new: the reaction of the unrelaxed drag, as
                                    compute_two_way_coupling_forces spreads it
                                    (coffee_particles.py:1141-1149)                               */
};

/* ---- library ------------------------------------------------------------------------------- */
int pog_version(void);
const char* pog_last_error(void);
/* Number of kernel launches this thread issued through the library since the last reset. */
long long pog_launch_count(int reset);

/* Zero `bytes` bytes of device memory at p, asynchronously on `stream` (the FP64 reduction block
 * before a reducing step, without a framework's fill kernel). */
int pog_zero(void* p, size_t bytes, void* stream);

/* Check a parameter block (sizes, enum values, ranges).  Host only. */
int pog_validate_params(const pog_params* p);

/* Advance the pour nozzle of p->pour_control by one step on the device (TIME += DT and the new
 * (X, Y), see above), so a captured CUDA graph replays a moving nozzle.  No-op while ACTIVE is 0.
 * POG_E_ARG without a pour block. */
int pog_pour_advance(const pog_params* p, void* stream);

/* ---- filter-paper dynamics (FilterPaperSystem.step, filter_paper.py:616-790) ------------------ */
/* Particles meeting the paper: each active particle at cell (i, j, k) = int(pos) looks for a
 * porous cell at (i, j, k + o), o = -2..2 in that order; at the first one, a particle moving
 * down (v_z < 0) bounces with v_z := -0.3 v_z, gets a horizontal roughness kick of +-0.005 per
 * axis, and adds 0.01 to accum at that cell (block_particles_at_filter, :616-700).  The kicks
 * come from a counter-based hash of (seed, step, particle): lowbias32 (C. Wellons), so runs
 * are reproducible.  accum [ncell] is added to atomically. */
int pog_filter_particles(const pog_params* p, const uint32_t* flags, const float* pos, float* vel,
                         const int32_t* active, int np, float* accum, uint32_t seed, long long step,
                         void* stream);
/* Dynamic blockage of the porous cells (update_dynamic_resistance, :702-750):
 * b := 0.95 b + 0.05 * 0.9 (1 - exp(-0.1 accum)), accum := 0.999 accum. */
int pog_filter_update(const pog_params* p, const uint32_t* flags, float* accum, float* blockage,
                      void* stream);

/* ---- multiphase phase field (MultiphaseFlow3D, src/core/multiphase_3d.py) ------------------- */
/* phi [ncell] in [-1, 1] (-1 air, +1 water), natural order, DEVICE pointers.  The stencil passes
 * touch interior cells only (1 <= i < nx-1, ...); fields they write keep their outer shell. */
/* mu = phi^3 - phi - kappa lap(phi) (compute_chemical_potential :80-109). */
int pog_phase_chemical_potential(const pog_params* p, const float* phi, float kappa, float* mu,
                                 void* stream);
/* normal [3][ncell] = grad(phi)/|grad(phi)| (0 where |grad| <= 1e-10), gmag [ncell] = |grad|
 * (compute_gradients :111-132).  Allocate both zeroed: the shell is never written. */
int pog_phase_normals(const pog_params* p, const float* phi, float* normal, float* gmag,
                      void* stream);
/* Curvature kappa = div(normal) (:134-149) and the surface-tension force F = sigma kappa |grad|
 * normal where |phi| < 0.9 (:313-331).  body_force (nullable, needs rho): += F / rho on non-solid
 * cells with rho > 1e-10 (apply_surface_tension :354-363).  curvature [ncell] and surface_force
 * [3][ncell] are optional outputs. */
int pog_phase_surface_tension(const pog_params* p, const uint32_t* flags, const float* phi,
                              const float* normal, const float* gmag, const float* rho,
                              float sigma, float* body_force, float* curvature,
                              float* surface_force, void* stream);
/* One phase-field step into phi_new (phi_new != phi): upwind advection by u [3][ncell] (zero in
 * solid cells) + mobility lap(mu) (mu NULL = 0), clamp to [-1, 1], then the phase-separation
 * relaxation where |phi| < 0.99 (:151-197, :334-352); non-interior cells carry phi over.  With
 * rho and phase (both or neither): rho = rho_air + (rho_water - rho_air)(phi' + 1)/2 and
 * phase = (phi' + 1)/2 from the clamped new phi' (update_density_from_phase :365-381). */
int pog_phase_update(const pog_params* p, const uint32_t* flags, const float* phi, float* phi_new,
                     const float* u, const float* mu, float mobility, float dt, float rho_air,
                     float rho_water, float* rho, float* phase, void* stream);
/* rho and phase from phi alone (update_density_from_phase :365-381). */
int pog_phase_properties(const pog_params* p, const float* phi, float rho_air, float rho_water,
                         float* rho, float* phase, void* stream);
/* The pour stream's phase change (apply_gradual_phase_change, precise_pouring.py:166-193): in the
 * stream of p->pour_control, non-solid cells move toward water by
 * clamp((1 - phi)/0.05, +-2) * intensity * dt * flow, clamped to [-1, 1]. */
int pog_pour_phase(const pog_params* p, const uint32_t* flags, float* phi, float dt, void* stream);

/* ---- pressure-gradient drive (PressureGradientDrive, src/physics/pressure_gradient_drive.py) ---- */
/* force[a][c] += scale * F_a(c) for every non-solid cell, F = -c_s^2 grad(rho) / rho (central
 * differences, one-sided on the domain faces; 0 where rho <= 1e-12), capped at |F| <= max_force
 * (compute_pressure_gradient :124-177; scale 1 = force drive :188-193, 0.5 = mixed drive
 * :274-279).  rho [ncell], force [3][ncell], natural order, DEVICE pointers. */
int pog_pressure_force(const pog_params* p, const uint32_t* flags, const float* rho, float* force,
                       float scale, float max_force, void* stream);
/* rho[c] := clamp(rho[c] + clamp((target[k] - rho[c]) * rate, +-max_adjust), rho_min, rho_max)
 * for every non-solid cell, target [nz] per plane (apply_density_drive :95-122). */
int pog_density_drive(const pog_params* p, const uint32_t* flags, float* rho, const float* target,
                      float rate, float max_adjust, float rho_min, float rho_max, void* stream);

/* ---- diagnostics ----------------------------------------------------------------------------- */
/* Field statistics of rho [ncell] and u [3][ncell] (FP32, every cell of the grid, as the
 * reference's host-side LBMDiagnostics computes them from to_numpy() copies,
 * src/visualization/lbm_diagnostics.py:151-460), in one device pass.  stats receives
 * POG_STAT_COUNT doubles (zeroed by the call); rho_prev/u_prev (nullable) feed the temporal
 * change sums; zprofile (nullable) receives the nz per-plane sums of rho.  |u| thresholds are in
 * lattice units: 1e-10 (active cells) and 0.1 c_s (Mach 0.1).  Region sums split the planes at
 * int(0.3 nz) and int(0.8 nz) (detailed_flow_analysis :393-402). */
#define POG_STAT_MASS 0        /* sum rho                                                     */
#define POG_STAT_RHO2 1        /* sum rho^2                                                   */
#define POG_STAT_MOMX 2        /* sum rho u_x (3 slots: x, y, z)                               */
#define POG_STAT_UMAX 5        /* max |u|                                                     */
#define POG_STAT_UACT_SUM 6    /* sum |u| over |u| > 1e-10                                    */
#define POG_STAT_UACT_N 7      /* number of cells with |u| > 1e-10                            */
#define POG_STAT_U2 8          /* sum |u|^2                                                   */
#define POG_STAT_UABS 9        /* sum |u|                                                     */
#define POG_STAT_MACH_N 10     /* number of cells with |u| > 0.1 c_s                          */
#define POG_STAT_DRHO_MAX 11   /* max |rho - rho0|                                            */
#define POG_STAT_DRHO2 12      /* sum (rho - rho_prev)^2                                      */
#define POG_STAT_DU2 13        /* sum |u - u_prev|^2                                          */
#define POG_STAT_USUM 14       /* sum u_a (3 slots)                                           */
#define POG_STAT_USQ 17        /* sum u_a^2 (3 slots)                                         */
#define POG_STAT_UREG 20       /* sum |u| over planes [0,z30), [z30,z80), [z80,nz) (3 slots)  */
#define POG_STAT_COUNT 23
int pog_field_stats(const pog_params* p, const float* rho, const float* u, const float* rho_prev,
                    const float* u_prev, double* stats, double* zprofile, void* stream);

/* ---- geometry ------------------------------------------------------------------------------ */
/* Build the cell flag words (own flags + the 18 solid-neighbour link bits) of the V60 mask,
 * drain hole, inlet/outlet disks and porous band: flags[c], c = (k*ny + j)*nx + i.
 * Replaces FilterPaperSystem._setup_v60_geometry / _setup_filter_zones
 * (filter_paper.py:206-364) and the LES mask copy (filter_paper.py:199-204).  Computed in FP64
 * without contraction: the result is bit-exact with the CPU restatement. */
int pog_build_flags(const pog_params* p, uint32_t* flags, void* stream);

/* ---- distributions --------------------------------------------------------------------------- */
/* f := equilibrium(rho0, u0) on every non-solid cell, 0 on solid cells, in the storage format
 * of p->storage.  The state is left at AA parity 0 (natural layout).
 * Replaces LBMSolver.init_fields (legacy/lbm_solver.py:1067-1112). */
int pog_init_equilibrium(const pog_params* p, void* f, const uint32_t* flags, float rho0,
                         float ux, float uy, float uz, void* stream);

/* Advance `nsteps` time steps in place (AA pattern: one distribution buffer).  `t` is the time
 * index of the incoming state; its parity selects the AA read/write pattern.  Each step is
 * LBMSolver.step (legacy/lbm_solver.py:817-867): macroscopic moments (:488-535), Guo forcing
 * (:594-607,688-764), LES relaxation (les_turbulence.py:289-380), BGK collision and push
 * streaming with half-way bounce-back (:537-628), the filter-band Darcy-Forchheimer drag
 * (filter_paper.py:471-536), the particle reaction force (:1478-1483) and the inlet/outlet
 * boundary overwrite (boundary_conditions.py:384-409), fused into one pass per step.
 *   force      [3][ncell] explicit external force density (plugins, pouring) or NULL
 *   pdrag      [4][ncell] particle drag deposit of pog_particles_couple (Kp, Kv) or NULL; the
 *              particle force Kv - Kp u enters implicitly (add_particle_reaction_forces,
 *              legacy/lbm_solver.py:1478-1483)
 *   porosity   [ncell] per-cell eps for porous cells, or NULL (uniform p->porosity)
 *   u_prev/u_next [3][ncell] velocity ping-pong buffers: required for POG_LES_STENCIL (step s
 *              reads u_prev and writes u_next; the pointers are swapped every step inside
 *              the call; after an odd nsteps the newest u is in u_next, else in u_prev)
 *   rho_out, u_out  macroscopic output (rho and Guo-corrected u of the incoming state) of
 *              the LAST step, or NULL
 *   reductions POG_RED_COUNT doubles accumulated over all nsteps, or NULL
 * Kernel: the row-tiled TMA-staged step when p->wall_cells is set and applies (see pog_params),
 * else the register-staged step.  Both compute the same update. */
int pog_step(const pog_params* p, void* f, const uint32_t* flags, long long t, int nsteps,
             const float* force, const float* pdrag, const float* porosity, float* u_prev, float* u_next,
             float* rho_out, float* u_out, double* reductions, void* stream);

/* The cells the row-tiled step's bounce-back mailbox pass serves: fluid cells with at least one
 * solid neighbour on the planes 1 .. nz-2 with 1 <= i <= nx-2, derived from the flag words (the
 * link bits replace the solid-neighbour tests of legacy/lbm_solver.py:621-628).  `count` is a
 * DEVICE int32 that receives the number of such cells; up to `capacity` of them are written to
 * `cells` (DEVICE, nullable: count only).  The order of the list is unspecified (the mailbox
 * copies are independent of one another).  Call once with cells NULL, read the count, allocate,
 * call again. */
int pog_wall_list(const pog_params* p, const uint32_t* flags, int32_t* cells, int32_t capacity,
                  int32_t* count, void* stream);

/* Same step on the natural (two-buffer) layout: reads f_in at time t, writes f_out at t+1
 * with push streaming exactly as legacy/lbm_solver.py:609-628.  Both buffers hold slot (q, c) in
 * p->storage's stored form (the shifted deviation of enum pog_storage), which is also the AA
 * state at an even t: pog_import_natural fills f_in, pog_export_natural (t even) reads f_out.
 * Used for checkpointed recomputation under the adjoint and for FP64 reference runs. */
int pog_step_push(const pog_params* p, const void* f_in, void* f_out, const uint32_t* flags,
                  const float* force, const float* pdrag, const float* porosity, const float* u_prev,
                  float* rho_out, float* u_out, double* reductions, void* stream);

/* Copy the AA state at time t into natural layout (f_nat[q][c] = f_q at cell c), converting
 * the storage format to `out_storage` (POG_STORE_F32 or POG_STORE_F64). */
int pog_export_natural(const pog_params* p, const void* f, const uint32_t* flags, long long t,
                       void* f_nat, int out_storage, void* stream);
/* Inverse at an even t: natural FP32/FP64 -> AA state in p->storage. */
int pog_import_natural(const pog_params* p, const void* f_nat, int in_storage,
                       const uint32_t* flags, void* f, void* stream);

/* Density and Guo-corrected velocity of the AA state at time t, without advancing it.
 * Replaces LBMSolver._compute_macroscopic_quantities (legacy/lbm_solver.py:488-535). */
int pog_macroscopic(const pog_params* p, const void* f, const uint32_t* flags, long long t,
                    const float* force, const float* pdrag, float* rho_out, float* u_out, void* stream);

/* Synchronise the device and report whether a kernel raised the device error word (a bounded
 * mbarrier wait that gave up): POG_OK or POG_E_STATE; `reset` clears the word. */
int pog_device_status(int reset);

/* ---- particles ----------------------------------------------------------------------------- */
/* Cell key of every particle, key = i + nx*(j + ny*k) with (i,j,k) = int(clamp(pos, 0, n-2))
 * (coffee_particles.py:1162-1164); inactive particles get key = ncell.  `perm` receives the
 * stable ascending order of the keys (equal to numpy.argsort(keys, kind="stable")).
 * `scratch` must hold pog_particles_bin_scratch_bytes(np) bytes of device memory. */
size_t pog_particles_bin_scratch_bytes(int np);
int pog_particles_bin(const pog_params* p, const float* pos, const int32_t* active, int np,
                      int32_t* keys, int32_t* perm, void* scratch, void* stream);

/* Same binning and stable cell sort as pog_particles_bin, but it allocates nothing and takes
 * no scratch argument: for callers that may not allocate device memory once running (a host
 * application that gives the library a fixed device-memory budget, or a loop that must not block
 * on an allocator).  Its scratch is a fixed 20 MiB device array inside libpog.so.  CUDA loads the
 * library's device code lazily, so the array is reserved on a GPU by the first call on that GPU,
 * which also looks up its address (cudaGetSymbolAddress) with that device current, and stays
 * reserved until the process exits: make one call with np = 0 on each device at set-up time,
 * before the memory budget is fixed and before any stream capture.  Limit: np <=
 * POG_NOALLOC_MAX_PARTICLES (larger np returns POG_E_RANGE).  The current device must be the
 * stream's device; the cached address does not survive cudaDeviceReset.  All calls share the
 * array: calls that overlap on the GPU race and must be ordered by the caller.  No counterpart in
 * the reference (it has no sort and no scratch). */
#define POG_NOALLOC_MAX_PARTICLES (1 << 20)
int pog_particles_bin_noalloc(const pog_params* p, const float* pos, const int32_t* active, int np,
                              int32_t* keys, int32_t* perm, void* stream);

/* One two-way coupling pass (LBMSolver.step_with_two_way_coupling, legacy/lbm_solver.py:
 * 1485-1509, with CoffeeParticleSystem.compute_two_way_coupling_forces 1107-1154,
 * apply_under_relaxation 1200-1212 and update_particle_physics 641-720): for each active
 * particle, trilinear u at its position, drag, under-relaxation of the drag, spreading of the
 * velocity/position update with the cone constraint, then the particle's drag coefficient
 * beta = m_p/(tau_p + dt) and beta*v_new are deposited onto the 8 surrounding nodes with the
 * trilinear weights (Kp = sum w beta, Kv = sum w beta v).  pog_step applies the particle force
 * on the fluid, Kv - Kp u, implicitly in u, which stays stable where particles pile up (the
 * reference spreads the explicit reaction -F, distribute_force_to_grid 1048-1086, which
 * diverges once the particle mass in a cell exceeds the fluid's).  `order` (nullable) lists
 * the particles in processing order (the `perm` of pog_particles_bin) so neighbouring lanes
 * hit neighbouring cells.
 *   pdrag     [4][ncell] float accumulator (Kp, Kv_x, Kv_y, Kv_z; fast mode; caller zeroes), or
 *   pdrag_fix [4][ncell] int64 fixed-point accumulator, scale 2^32 (deterministic mode) */
int pog_particles_couple(const pog_params* p, const pog_particle_params* pp, float* pos,
                         float* vel, const float* diameter, float* drag_old, int32_t* active,
                         int np, const int32_t* order, const float* u, float* pdrag,
                         long long* pdrag_fix, float* u_at_particle, void* stream);
/* Zero the 4 x 8 deposit slots pdrag[a][corner + {0,1} + nx {0,1} + nx ny {0,1}] of every
 * particle whose deposit_cells entry (from pog_particles_couple) is >= 0: after the lattice step
 * has read the deposit, this returns pdrag to all zeros at the cost of the particles' cells
 * instead of a full-field fill.  order (nullable): the coupling pass's particle order, so that
 * neighbouring threads write neighbouring cells.  deposit_mask (nullable): cleared entirely in
 * the same kernel (no cell holds a deposit afterwards). */
int pog_particles_clear_deposit(const pog_params* p, const int32_t* deposit_cells, int np,
                                const int32_t* order, float* pdrag, uint32_t* deposit_mask, void* stream);
/* pdrag[a][c] = pdrag_fix[a][c] * 2^-32, a = 0..3 (deterministic-mode conversion). */
int pog_drag_from_fixed(const pog_params* p, const long long* pdrag_fix, float* pdrag,
                        void* stream);
/* The same conversion at the deposit cells of the np particles only (deposit_cells from the
 * pog_particles_couple pass that filled pdrag_fix; order nullable, as in
 * pog_particles_clear_deposit): pdrag[a][c] += pdrag_fix[a][c] * 2^-32 at each cell a particle
 * deposited on, and those pdrag_fix entries -- all its nonzero ones -- are zeroed, each entry
 * taken once however many particles share the cell.  pdrag_fix is therefore all zeros again for
 * the next pass, and pdrag equals pog_drag_from_fixed's field added to it, at the cost of the
 * particles' cells rather than of two full-field passes. */
int pog_drag_from_fixed_cells(const pog_params* p, long long* pdrag_fix, const int32_t* deposit_cells, int np,
                              const int32_t* order, float* pdrag, void* stream);

/* ---- adjoint --------------------------------------------------------------------------------- */
/* Reverse of one pog_step_push step (natural layout, storage F32 or F64).
 *   f_t       forward state at time t (natural), the input of the step being reversed
 *   lam_next  adjoint of the state at t+1;  lam_t  receives the adjoint at t
 *   pdrag     [4][ncell] the particle drag deposit (Kp, Kv) the forward step read, or NULL: a
 *             fixed input, its force Kv - Kp u differentiated through u (the coupled step of
 *             legacy/lbm_solver.py:1485-1509 with the particles' deposit recorded per step)
 *   LES stencil mode (les_turbulence.py:318-380: step t's nu_sgs reads the velocity u_{t-1} that
 *   step t-1 output, so dJ/du crosses steps):
 *   u_prev     [3][ncell] float, the velocity the forward step's stencil read (required)
 *   dJ_du      [3][ncell] (storage type) dJ/du_t of the velocity this step outputs, or NULL (0)
 *   dJ_du_prev [3][ncell] receives dJ/du_{t-1} (overwritten; required, != dJ_du)
 *   In the other LES modes these three are ignored (pass NULL).
 *   scratch   pog_adjoint_scratch_bytes(p) bytes of device memory, 16-byte aligned: required in
 *             LES stencil mode; otherwise optional -- with it the inlet plane's dJ/da_k is summed
 *             by many blocks (per-block sums added in block order), without it by one block;
 *             either way in a fixed order, so gradients repeat bit for bit.
 *   The loss is J = sum_t flux_t with flux_t = POG_RED_OUTFLOW of step t, so each outlet
 *   cell adds dJ/df_i = -c_iz.  Parameter gradients are accumulated in FP64:
 *   grad_porosity [ncell] (nullable; needs porosity), grad_inlet [POG_INLET_NCOEF] (nullable).
 *   Supported: les_mode OFF/LOCAL/STENCIL, drag SEMI_IMPLICIT, forcing GUO, clamp_tau 0, force NULL,
 *   pour_control, filter_blockage and phase NULL (POG_E_ARG otherwise). */
int pog_adjoint_step(const pog_params* p, const void* f_t, const void* lam_next, void* lam_t,
                     const uint32_t* flags, const float* porosity, const float* pdrag,
                     const float* u_prev, const void* dJ_du, void* dJ_du_prev, void* scratch,
                     double* grad_porosity, double* grad_inlet, void* stream);
/* Scratch of pog_adjoint_step: 10 values per cell in LES stencil mode (rounded up to 16 bytes), then
 * 16 doubles per 1,024 cells of an xy plane for the inlet plane's per-block sums. */
size_t pog_adjoint_scratch_bytes(const pog_params* p);

/* The outflow flux of a natural-layout state f_nat (F32 or F64 storage), flux = -sum over outlet
 * cells of sum_q c_qz f_q -- the POG_RED_OUTFLOW contribution of the step that starts from f_nat --
 * added to acc[0..1] (DEVICE int64 x 2) in two-word fixed point: acc[0] in units of 2^-48 (each
 * cell's flux rounded), acc[1] the cells' rounding remainders in units of 2^-96, so
 * acc[0] 2^-48 + acc[1] 2^-96 is the exact sum of the cells' FP64 fluxes.  Integer sums do not
 * depend on the order of accumulation, so a loss J = sum_t flux_t built from it is the same bits
 * on every run, and finite differences of J carry neither reduction-order nor quantisation noise. */
int pog_outflow_fixed(const pog_params* p, const void* f_nat, const uint32_t* flags, long long* acc,
                      void* stream);

#ifdef __cplusplus
}
#endif
#endif /* POG_H */
