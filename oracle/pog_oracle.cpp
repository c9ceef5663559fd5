// pog_oracle.cpp -- CPU restatement of the reference hot path.  TEST INFRASTRUCTURE ONLY.
//
// This file is the oracle the CUDA library (libpog.so) is checked against.  Only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg load it, and only as the checker
// or the timed CPU baseline; the product never calls it.
//
// The reference (latteine1217/pour-over-coffee-lbm) is Python + Taichi and cannot run here
// (no Taichi).  Each function below restates the reference code it cites, with the
// reference's own structure (separate macroscopic pass, collide, push streaming into a
// second buffer with half-way bounce-back), written as plain loops in FP32 or FP64.  Where the
// reference contradicts itself the build spec decides (D3Q19 ordering of config/core.py,
// standard Guo forcing, lattice-unit Stokes drag); those choices are the same ones the CUDA
// library makes, and they are listed in the project's design notes.
//
// Pinning: the equilibrium, moment, trilinear-interpolation, LES-gate, Forchheimer and
// under-relaxation functions are checked against the known-answer cases of the reference's
// own tests (tests/test_lbm_algorithms.py, test_trilinear_interpolation.py,
// test_les_turbulence.py, test_forchheimer.py, test_filter_paper.py,
// test_under_relaxation.py) in tests/test_oracle_kat.py.  No reference test pins a
// multi-step trajectory, so trajectory parity is pinned by this restatement only.
//
// Build: g++ -O2 -fopenmp -ffp-contract=off -shared -fPIC (see oracle/build.py).  No FP
// contraction, so particle arithmetic is bit-identical with the GPU kernels (which are also
// compiled without contraction).

#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "../include/pog.h"

namespace {

// D3Q19 in the reference's config/core.py:36-47 ordering.
const int CX[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
const int CY[19] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1};
const int CZ[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
const double WD[19] = {1.0 / 3.0,  1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0,
                       1.0 / 18.0, 1.0 / 18.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
                       1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
                       1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};

// opposite(q): the search of legacy/lbm_solver.py:431-439 over the table above.
int OPP[19];
struct OppInit {
  OppInit() {
    for (int q = 0; q < 19; ++q)
      for (int p = 0; p < 19; ++p)
        if (CX[q] == -CX[p] && CY[q] == -CY[p] && CZ[q] == -CZ[p]) OPP[q] = p;
  }
} opp_init;

template <typename T>
T wq(int q) {
  return (T)WD[q];
}

// Test-only switch reproducing the reference legacy collision's mixed D3Q19 orderings: its f_eq
// (equilibrium_d3q19_unified, lbm_algorithms.py:155-218) indexes the velocity table of
// lbm_algorithms.py:158-164, whose entries 8/10 (y), 12/14 and 16/18 (z) are mirrored against the
// config/core.py:36-38 table it streams with (legacy/lbm_solver.py:576 vs :617-619).  Off by
// default: the build spec uses one ordering.  It exists so that the rest of the step can be pinned
// against the reference's own kernels on states with flow in every direction.
int g_legacy_feq_order = 0;
const int ALG_CY[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1};
const int ALG_CZ[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1};

// Storage rounding of the shifted forms (f - w*rho0): FP16 is scaled by 2^12 so small
// deviations stay normal numbers; BF16 needs no scale.
const float F16_SCALE = 4096.0f;

float round_bf16(float x) {
  uint32_t u;
  memcpy(&u, &x, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return x;  // inf/nan unchanged
  uint32_t lsb = (u >> 16) & 1u;
  u += 0x7fffu + lsb;
  u &= 0xffff0000u;
  float y;
  memcpy(&y, &u, 4);
  return y;
}
float round_f16s(float x) {
  _Float16 h = (_Float16)(x * F16_SCALE);
  return (float)h / F16_SCALE;
}

template <typename T>
T store_round(int storage, T v, int q, T rho0) {
  if (storage == POG_STORE_F16S) {
    T w = wq<T>(q) * rho0;
    return w + (T)round_f16s((float)(v - w));
  }
  if (storage == POG_STORE_BF16S) {
    T w = wq<T>(q) * rho0;
    return w + (T)round_bf16((float)(v - w));
  }
  return v;
}

struct Geo {
  int nx, ny, nz;
  long long n;
  double cx, cy, tanth;
  long long idx(int i, int j, int k) const { return ((long long)k * ny + j) * nx + i; }
};

Geo make_geo(const pog_params* p) {
  Geo g;
  g.nx = p->nx;
  g.ny = p->ny;
  g.nz = p->nz;
  g.n = (long long)p->nx * p->ny * p->nz;
  g.cx = p->center_x < 0 ? 0.5 * p->nx : (double)p->center_x;
  g.cy = p->center_y < 0 ? 0.5 * p->ny : (double)p->center_y;
  g.tanth = tan((double)p->cone_half_angle_deg * M_PI / 180.0);
  return g;
}

// ---------------------------------------------------------------------------------------
// Equilibrium: lbm_algorithms.py:183-218, f_eq = w rho (1 + 3 e.u + 4.5 (e.u)^2 - 1.5 u.u)
template <typename T>
void equilibrium(T rho, T ux, T uy, T uz, T feq[19]) {
  T usq = ux * ux + uy * uy + uz * uz;
  for (int q = 0; q < 19; ++q) {
    T eu = (T)CX[q] * ux + (T)CY[q] * uy + (T)CZ[q] * uz;
    feq[q] = wq<T>(q) * rho * ((T)1 + (T)3 * eu + (T)4.5 * eu * eu - (T)1.5 * usq);
  }
}

// Radial inlet profile u_z(r) = u_inlet (1 + sum_k a_k T_k(2r/R - 1)), Chebyshev T_k.
// `coef` overrides p->inlet_coef (the adjoint oracle passes dual numbers there).
template <typename T>
T inlet_velocity(const pog_params* p, T r, const T* coef = nullptr) {
  T a[POG_INLET_NCOEF];
  for (int k = 0; k < POG_INLET_NCOEF; ++k) a[k] = coef ? coef[k] : (T)p->inlet_coef[k];
  T R = (T)p->inlet_radius;
  T s = R > (T)0 ? (T)2 * r / R - (T)1 : (T)0;
  T t0 = (T)1, t1 = s, acc = a[0];
  acc += a[1] * t1;
  for (int k = 2; k < POG_INLET_NCOEF; ++k) {
    T t2 = (T)2 * s * t1 - t0;
    acc += a[k] * t2;
    t0 = t1;
    t1 = t2;
  }
  return (T)p->u_inlet * ((T)1 + acc);
}

// Kozeny-Carman permeability and Ergun-type Forchheimer coefficient at porosity eps,
// normalised so that (permeability, forchheimer) are the values at p->porosity
// (filter_paper.py:423-469 uses K = d^2 eps^3/(180(1-eps)^2), beta = 1.75(1-eps)/eps^3).
template <typename T>
void porous_coeffs(const pog_params* p, T eps, T& K, T& CF) {
  T e0 = (T)p->porosity;
  T g0 = e0 * e0 * e0 / (((T)1 - e0) * ((T)1 - e0));
  T g = eps * eps * eps / (((T)1 - eps) * ((T)1 - eps));
  K = (T)p->permeability * (g / g0);
  T r = e0 / eps;
  CF = (T)p->forchheimer * (r * sqrt(r));
}

// LES nu_sgs from central differences of a stored velocity field
// (les_turbulence.py:318-380).  u is [3][n].  Returns 0 where the reference does.
// nu_sgs from the velocities of the six neighbours, un[m][a]: m = (i+1, i-1, j+1, j-1, k+1, k-1),
// a = (x, y, z) component.
template <typename T>
T les_nu_from_neighbours(const pog_params* p, const T un[6][3]) {
  T dudx = (un[0][0] - un[1][0]) * (T)0.5, dudy = (un[2][0] - un[3][0]) * (T)0.5,
    dudz = (un[4][0] - un[5][0]) * (T)0.5;
  T dvdx = (un[0][1] - un[1][1]) * (T)0.5, dvdy = (un[2][1] - un[3][1]) * (T)0.5,
    dvdz = (un[4][1] - un[5][1]) * (T)0.5;
  T dwdx = (un[0][2] - un[1][2]) * (T)0.5, dwdy = (un[2][2] - un[3][2]) * (T)0.5,
    dwdz = (un[4][2] - un[5][2]) * (T)0.5;
  T S11 = dudx, S22 = dvdy, S33 = dwdz;
  T S12 = (T)0.5 * (dudy + dvdx), S13 = (T)0.5 * (dudz + dwdx), S23 = (T)0.5 * (dvdz + dwdy);
  T smag = sqrt((T)2 * (S11 * S11 + S22 * S22 + S33 * S33 +
                        (T)2 * (S12 * S12 + S13 * S13 + S23 * S23)));
  if (smag < (T)p->les_strain_floor) return 0;
  T cs = (T)p->cs_smag;
  T nu = cs * cs * smag;
  return std::min(nu, (T)p->les_nu_max);
}

// Cell offsets of the six stencil neighbours, in les_nu_from_neighbours' order.
inline void stencil_neighbours(const Geo& g, int i, int j, int k, long long nb[6]) {
  nb[0] = g.idx(i + 1, j, k);
  nb[1] = g.idx(i - 1, j, k);
  nb[2] = g.idx(i, j + 1, k);
  nb[3] = g.idx(i, j - 1, k);
  nb[4] = g.idx(i, j, k + 1);
  nb[5] = g.idx(i, j, k - 1);
}

// Whether cell (i, j, k) takes a stencil nu at all (interior, outside the filter zone's LES mask).
inline bool les_stencil_cell(const Geo& g, const uint32_t* flags, int i, int j, int k) {
  if (i < 1 || j < 1 || k < 1 || i > g.nx - 2 || j > g.ny - 2 || k > g.nz - 2) return false;
  return !(flags[g.idx(i, j, k)] & POG_CELL_POROUS);  // filter zone: LES mask 0 (filter_paper.py:199)
}

// LES nu_sgs from central differences of a stored velocity field
// (les_turbulence.py:318-380).  u is [3][n].  Returns 0 where the reference does.
template <typename T>
T les_nu_stencil(const pog_params* p, const Geo& g, const uint32_t* flags, const T* u, int i,
                 int j, int k) {
  if (!les_stencil_cell(g, flags, i, j, k)) return 0;
  long long nb[6];
  stencil_neighbours(g, i, j, k, nb);
  T un[6][3];
  for (int m = 0; m < 6; ++m)
    for (int a = 0; a < 3; ++a) un[m][a] = u[a * g.n + nb[m]];
  return les_nu_from_neighbours<T>(p, un);
}

// Per-cell collision (legacy/lbm_solver.py:488-535 moments, :537-579 BGK, :594-607/688-764
// forcing, filter_paper.py:471-536 porous drag, boundary_conditions.py:384-409 inlet/outlet).
// Inputs: incoming populations f, flag, optional external force Fe and porosity.  Output:
// post-collision populations fs, rho, u, and reduction contributions.
// Pour nozzle (precise_pouring.py:100-160).  For the restatement `pour_control` is a HOST copy of
// the POG_POUR_* block: the stream cylinder's downward force density on cell (i, j, k).
template <typename T>
T pour_accel(const float* b, int nz, int i, int j, int k) {
  if (b[POG_POUR_ACTIVE] == 0.0f) return (T)0;
  const float ztop = b[POG_POUR_ZTOP];
  if (!((float)k <= ztop && (float)k >= ztop - b[POG_POUR_HEIGHT]) || k < 0 || k > nz - 1) return (T)0;
  const T dx = (T)i - (T)b[POG_POUR_X], dy = (T)j - (T)b[POG_POUR_Y];
  const T R = (T)b[POG_POUR_RADIUS];
  const T d = sqrt(dx * dx + dy * dy);
  if (!(d <= R)) return (T)0;
  const T dr = d / R;
  const T I = exp((T)-0.5 * dr * dr) * exp(-((T)ztop - (T)k) / (T)2);
  const T dt = (T)b[POG_POUR_DT];
  T a = dt > (T)1e-8 ? (T)b[POG_POUR_VELOCITY] * I * (T)b[POG_POUR_FLOW] / dt : (T)0;
  const T cap = (T)b[POG_POUR_ACCEL_CAP];
  return a < cap ? a : cap;
}

template <typename T>
void collide(const pog_params* p, const Geo& g, uint32_t flag, int i, int j, int k, const T f[19],
             const T* Fe, const T* Pd, bool has_eps, T eps, T nu_stencil, T fs[19], T& rho_o,
             T u_o[3], double* red, const T* coef = nullptr) {
  T rho = 0, mx = 0, my = 0, mz = 0;
  for (int q = 0; q < 19; ++q) {
    rho += f[q];
    mx += (T)CX[q] * f[q];
    my += (T)CY[q] * f[q];
    mz += (T)CZ[q] * f[q];
  }
  T ux, uy, uz;
  T feq[19];
  if (flag & POG_CELL_INLET) {
    T dx = (T)i - (T)g.cx, dy = (T)j - (T)g.cy;
    T r = sqrt(dx * dx + dy * dy);
    ux = 0;
    uy = 0;
    uz = inlet_velocity<T>(p, r, coef);
    equilibrium<T>(rho, ux, uy, uz, fs);
  } else if (flag & POG_CELL_OUTLET) {
    ux = mx / rho;
    uy = my / rho;
    uz = mz / rho;
    equilibrium<T>((T)p->rho_outlet, ux, uy, uz, fs);
    if (red) red[POG_RED_OUTFLOW] += -(double)mz;
  } else {
    // phase indicator (HOST array for the restatement): gravity on the water fraction,
    // tau by phase, LES gate |phase| < 0.9 (legacy/lbm_solver.py:558-592, les_turbulence.py:362-366)
    const T ph = p->phase ? (T)p->phase[g.idx(i, j, k)] : (T)1;
    const T rg = p->phase ? (ph > (T)0.001 ? rho * ph : (T)0) : rho;
    T Gx = rg * (T)p->gx, Gy = rg * (T)p->gy, Gz = rg * (T)p->gz;
    if (Fe) {
      Gx += Fe[0];
      Gy += Fe[1];
      Gz += Fe[2];
    }
    if (p->pour_control) Gz -= pour_accel<T>(p->pour_control, p->nz, i, j, k);
    // particle drag deposit Pd = (Kp, Kv): fluid force Kv - Kp u, implicit in u
    T Kp = 0, Kvx = 0, Kvy = 0, Kvz = 0;
    if (Pd) {
      Kp = Pd[0];
      Kvx = Pd[1];
      Kvy = Pd[2];
      Kvz = Pd[3];
    }
    T A = (T)1 + (T)0.5 * Kp / rho;
    T vx = (mx + (T)0.5 * (Gx + Kvx)) / rho, vy = (my + (T)0.5 * (Gy + Kvy)) / rho,
      vz = (mz + (T)0.5 * (Gz + Kvz)) / rho;
    T Fx = Gx, Fy = Gy, Fz = Gz;
    ux = vx;
    uy = vy;
    uz = vz;
    bool porous = (flag & POG_CELL_POROUS) != 0;
    T nu0 = ((T)p->tau - (T)0.5) / (T)3;
    if (porous) {
      T K, CF;
      if (has_eps) {
        porous_coeffs<T>(p, eps, K, CF);
      } else {
        K = (T)p->permeability;
        CF = (T)p->forchheimer;
      }
      T sK = sqrt(K);
      // Darcy and Forchheimer coefficients times the filter blockage factor 1 + b (for the
      // restatement `filter_blockage` is a HOST array)
      const T bf = p->filter_blockage ? (T)1 + (T)p->filter_blockage[g.idx(i, j, k)] : (T)1;
      const T dk = nu0 / K * bf, fk = CF / sK * bf;
      if (p->drag_mode == POG_DRAG_SEMI_IMPLICIT) {
        // u (A + nu/(2K) + C_F |u| / (2 sqrt K)) = v
        T c0 = (T)0.5 * (A + (T)0.5 * dk);
        T c1 = (T)0.5 * fk;
        T vm = sqrt(vx * vx + vy * vy + vz * vz);
        T s = (T)1 / (c0 + sqrt(c0 * c0 + c1 * vm));
        ux = vx * s;
        uy = vy * s;
        uz = vz * s;
        T um = sqrt(ux * ux + uy * uy + uz * uz);
        T coef = rho * (dk + fk * um);
        Fx = Gx + Kvx - (coef + Kp) * ux;
        Fy = Gy + Kvy - (coef + Kp) * uy;
        Fz = Gz + Kvz - (coef + Kp) * uz;
      } else {
        T wx = vx / A, wy = vy / A, wz = vz / A;  // velocity before the porous drag
        T vm = sqrt(wx * wx + wy * wy + wz * wz);
        T coef = rho * (dk + fk * vm);
        T dx = -coef * wx, dy = -coef * wy, dz = -coef * wz;
        T dm = sqrt(dx * dx + dy * dy + dz * dz);
        T cap = (T)p->drag_cap;
        if (dm > cap) {
          T sc = cap / dm;
          dx *= sc;
          dy *= sc;
          dz *= sc;
        }
        ux = (mx + (T)0.5 * (Gx + dx + Kvx)) / (rho * A);
        uy = (my + (T)0.5 * (Gy + dy + Kvy)) / (rho * A);
        uz = (mz + (T)0.5 * (Gz + dz + Kvz)) / (rho * A);
        Fx = Gx + dx + Kvx - Kp * ux;
        Fy = Gy + dy + Kvy - Kp * uy;
        Fz = Gz + dz + Kvz - Kp * uz;
      }
    } else if (Pd) {
      ux = vx / A;
      uy = vy / A;
      uz = vz / A;
      Fx = Gx + Kvx - Kp * ux;
      Fy = Gy + Kvy - Kp * uy;
      Fz = Gz + Kvz - Kp * uz;
    }
    equilibrium<T>(rho, ux, uy, uz, feq);
    if (g_legacy_feq_order) {
      const T usq15 = (T)1.5 * (ux * ux + uy * uy + uz * uz);
      for (int q = 7; q < 19; ++q) {
        T eu = (T)CX[q] * ux + (T)ALG_CY[q] * uy + (T)ALG_CZ[q] * uz;
        feq[q] = wq<T>(q) * rho * ((T)1 + (T)3 * eu + (T)4.5 * eu * eu - usq15);
      }
    }
    T tau0 = p->phase ? (ph > (T)0.5 ? (T)p->tau : (T)p->tau_air) : (T)p->tau;
    const bool les_on = !porous && !(p->phase && ph < (T)0.9 && ph > (T)-0.9);
    T nu = 0;
    if (les_on && p->les_mode == POG_LES_LOCAL) {
      T P[6] = {0, 0, 0, 0, 0, 0};  // xx yy zz xy xz yz
      for (int q = 0; q < 19; ++q) {
        T d = f[q] - feq[q];
        T ex = (T)CX[q], ey = (T)CY[q], ez = (T)CZ[q];
        P[0] += ex * ex * d;
        P[1] += ey * ey * d;
        P[2] += ez * ez * d;
        P[3] += ex * ey * d;
        P[4] += ex * ez * d;
        P[5] += ey * ez * d;
      }
      T PP = P[0] * P[0] + P[1] * P[1] + P[2] * P[2] + (T)2 * (P[3] * P[3] + P[4] * P[4] + P[5] * P[5]);
      T Q = sqrt((T)2 * PP);
      T cs = (T)p->cs_smag;
      T tl = (T)0.5 * (tau0 + sqrt(tau0 * tau0 + (T)18 * cs * cs * Q / rho));
      T smag = (T)3 * Q / ((T)2 * rho * tl);
      nu = (tl - tau0) / (T)3;
      if (smag < (T)p->les_strain_floor) nu = 0;
      nu = std::min(nu, (T)p->les_nu_max);
    } else if (les_on && p->les_mode == POG_LES_STENCIL) {
      nu = nu_stencil;
    }
    T tau = tau0 + (T)3 * nu;
    if (p->clamp_tau) tau = std::max((T)p->tau_min, std::min((T)p->tau_max, tau));
    T omega = (T)1 / tau;
    if (p->forcing_mode == POG_FORCING_GUO) {
      T pref = (T)1 - (T)0.5 * omega;
      for (int q = 0; q < 19; ++q) {
        T ex = (T)CX[q], ey = (T)CY[q], ez = (T)CZ[q];
        T eu = ex * ux + ey * uy + ez * uz;
        T eF = ex * Fx + ey * Fy + ez * Fz;
        T emuF = (ex - ux) * Fx + (ey - uy) * Fy + (ez - uz) * Fz;
        T S = pref * wq<T>(q) * ((T)3 * emuF + (T)9 * eu * eF);
        fs[q] = f[q] - omega * (f[q] - feq[q]) + S;
      }
    } else {
      // legacy/lbm_solver.py:594-607 and 688-764
      T taus = std::max((T)0.6, std::min((T)1.5, tau));
      T fn = sqrt(Fx * Fx + Fy * Fy + Fz * Fz);
      T sf = fn > (T)10 ? (T)10 / fn : (T)1;
      T fx = Fx * sf, fy = Fy * sf, fz = Fz * sf;
      T un = sqrt(ux * ux + uy * uy + uz * uz);
      T su = un <= (T)0.2 ? (T)1 : (T)0.2 / un;
      T sx = ux * su, sy = uy * su, sz = uz * su;
      T uf = sx * fx + sy * fy + sz * fz;
      for (int q = 0; q < 19; ++q) {
        T S = 0;
        if (fn > (T)1e-15) {
          T ex = (T)CX[q], ey = (T)CY[q], ez = (T)CZ[q];
          T eu = ex * sx + ey * sy + ez * sz;
          T ef = ex * fx + ey * fy + ez * fz;
          S = wq<T>(q) * ((T)1 - (T)0.5 / taus) * ((T)3 * ef + (T)9 * eu * uf);
          S = std::max((T)-0.5, std::min((T)0.5, S));
        }
        fs[q] = f[q] - omega * (f[q] - feq[q]) + S;
      }
    }
  }
  rho_o = rho;
  u_o[0] = ux;
  u_o[1] = uy;
  u_o[2] = uz;
  if (red) {
    red[POG_RED_MASS] += (double)rho;
    red[POG_RED_MOMX] += (double)rho * (double)ux;
    red[POG_RED_MOMY] += (double)rho * (double)uy;
    red[POG_RED_MOMZ] += (double)rho * (double)uz;
    if (!std::isfinite((double)rho) || !std::isfinite((double)ux) || !std::isfinite((double)uy) ||
        !std::isfinite((double)uz))
      red[POG_RED_NONFINITE] += 1.0;
  }
}

// One push step on natural layout (legacy/lbm_solver.py:460-486 + :609-628): every fluid
// cell collides and pushes f*_q to x+e_q, or into opp(q) at x when x+e_q is solid.
template <typename T>
int step_push(const pog_params* p, const uint32_t* flags, const T* f, T* fo, const float* Fe,
              const float* Pd, const float* eps, const T* u_prev, T* rho_out, T* u_out, double* red) {
  Geo g = make_geo(p);
  const long long n = g.n;
  double acc[POG_RED_COUNT] = {0, 0, 0, 0, 0, 0};
  const T rho0 = (T)p->rho0;
#pragma omp parallel
  {
    double loc[POG_RED_COUNT] = {0, 0, 0, 0, 0, 0};
#pragma omp for schedule(static)
    for (int k = 0; k < g.nz; ++k)
      for (int j = 0; j < g.ny; ++j)
        for (int i = 0; i < g.nx; ++i) {
          long long c = g.idx(i, j, k);
          uint32_t fl = flags[c];
          if (fl & POG_CELL_SOLID) continue;
          T fin[19], fs[19], rho, u[3];
          for (int q = 0; q < 19; ++q) fin[q] = f[q * n + c];
          T fe[3];
          const T* fep = nullptr;
          if (Fe) {
            fe[0] = (T)Fe[c];
            fe[1] = (T)Fe[n + c];
            fe[2] = (T)Fe[2 * n + c];
            fep = fe;
          }
          T pd[4];
          const T* pdp = nullptr;
          if (Pd) {
            for (int a = 0; a < 4; ++a) pd[a] = (T)Pd[a * n + c];
            pdp = pd;
          }
          T nus = 0;
          if (p->les_mode == POG_LES_STENCIL && u_prev)
            nus = les_nu_stencil<T>(p, g, flags, u_prev, i, j, k);
          collide<T>(p, g, fl, i, j, k, fin, fep, pdp, eps != nullptr, eps ? (T)eps[c] : (T)0, nus,
                     fs, rho, u, red ? loc : nullptr);
          if (rho_out) rho_out[c] = rho;
          if (u_out) {
            u_out[c] = u[0];
            u_out[n + c] = u[1];
            u_out[2 * n + c] = u[2];
          }
          for (int q = 0; q < 19; ++q) {
            long long nb = g.idx(i + CX[q], j + CY[q], k + CZ[q]);
            T v = store_round<T>(p->storage, fs[q], q, rho0);
            if (flags[nb] & POG_CELL_SOLID)
              fo[OPP[q] * n + c] = v;
            else
              fo[q * n + nb] = v;
          }
        }
#pragma omp critical
    for (int r = 0; r < POG_RED_COUNT; ++r) acc[r] += loc[r];
  }
  if (red)
    for (int r = 0; r < POG_RED_COUNT; ++r) red[r] += acc[r];
  return 0;
}

// One AA-pattern step in place (the CUDA step's stepping order, Bailey et al. 2009): at an even
// time t slot (c, q) holds f_q(c), the step reads it and writes f*_q to (c, opp q); at an odd t
// the step reads f_q from (c - e_q, opp q) -- or (c, q) when c - e_q is solid -- and writes f*_q
// to (c + e_q, q) -- or (c, opp q) when c + e_q is solid.  Each cell reads and writes the same 19
// slots, so the cells are independent.  Cells within one plane + row + 1 of either end of the
// grid are never updated (the CUDA kernels' guard).  The collision is `collide`, as in step_push.
template <typename T>
int step_aa(const pog_params* p, const uint32_t* flags, T* f, long long t, const float* Fe, const float* Pd,
            const float* eps, T* rho_out, T* u_out, double* red) {
  Geo g = make_geo(p);
  const long long n = g.n;
  const long long guard = (long long)g.nx * g.ny + g.nx + 1;
  const bool odd = (t & 1) != 0;
  double acc[POG_RED_COUNT] = {0, 0, 0, 0, 0, 0};
  const T rho0 = (T)p->rho0;
#pragma omp parallel
  {
    double loc[POG_RED_COUNT] = {0, 0, 0, 0, 0, 0};
#pragma omp for schedule(static)
    for (int k = 0; k < g.nz; ++k)
      for (int j = 0; j < g.ny; ++j)
        for (int i = 0; i < g.nx; ++i) {
          const long long c = g.idx(i, j, k);
          const uint32_t fl = flags[c];
          if ((fl & POG_CELL_SOLID) || c < guard || c > n - 1 - guard) continue;
          T fin[19], fs[19], rho, u[3];
          for (int q = 0; q < 19; ++q) {
            if (!odd) {
              fin[q] = f[q * n + c];
            } else {
              const long long src = g.idx(i - CX[q], j - CY[q], k - CZ[q]);
              fin[q] = (q != 0 && (flags[src] & POG_CELL_SOLID)) ? f[q * n + c] : f[OPP[q] * n + src];
            }
          }
          T fe[3];
          const T* fep = nullptr;
          if (Fe) {
            fe[0] = (T)Fe[c];
            fe[1] = (T)Fe[n + c];
            fe[2] = (T)Fe[2 * n + c];
            fep = fe;
          }
          T pd[4];
          const T* pdp = nullptr;
          if (Pd) {
            for (int a = 0; a < 4; ++a) pd[a] = (T)Pd[a * n + c];
            pdp = pd;
          }
          collide<T>(p, g, fl, i, j, k, fin, fep, pdp, eps != nullptr, eps ? (T)eps[c] : (T)0, (T)0, fs, rho, u,
                     red ? loc : nullptr);
          if (rho_out) rho_out[c] = rho;
          if (u_out) {
            u_out[c] = u[0];
            u_out[n + c] = u[1];
            u_out[2 * n + c] = u[2];
          }
          for (int q = 0; q < 19; ++q) {
            const T v = store_round<T>(p->storage, fs[q], q, rho0);
            if (!odd) {
              f[OPP[q] * n + c] = v;
            } else {
              const long long dst = g.idx(i + CX[q], j + CY[q], k + CZ[q]);
              if (q != 0 && (flags[dst] & POG_CELL_SOLID))
                f[OPP[q] * n + c] = v;
              else
                f[q * n + dst] = v;
            }
          }
        }
#pragma omp critical
    for (int r = 0; r < POG_RED_COUNT; ++r) acc[r] += loc[r];
  }
  if (red)
    for (int r = 0; r < POG_RED_COUNT; ++r) red[r] += acc[r];
  return 0;
}

template <typename T>
void init_eq(const pog_params* p, const uint32_t* flags, T* f, T rho0, T ux, T uy, T uz) {
  Geo g = make_geo(p);
  T feq[19];
  equilibrium<T>(rho0, ux, uy, uz, feq);
  for (int q = 0; q < 19; ++q) feq[q] = store_round<T>(p->storage, feq[q], q, (T)p->rho0);
  for (long long c = 0; c < g.n; ++c)
    for (int q = 0; q < 19; ++q) f[q * g.n + c] = (flags[c] & POG_CELL_SOLID) ? (T)0 : feq[q];
}

}  // namespace

// =========================================================================================
extern "C" {

int orc_d3q19_tables(int* cx, int* cy, int* cz, int* opp, double* w) {
  for (int q = 0; q < 19; ++q) {
    cx[q] = CX[q];
    cy[q] = CY[q];
    cz[q] = CZ[q];
    opp[q] = OPP[q];
    w[q] = WD[q];
  }
  return 0;
}

// V60 geometry + band + inlet/outlet (filter_paper.py:206-364).  FP64, no contraction.
// solid: the outer one-cell shell; below the apex everything outside the drain hole; above it
// the cone wall (rc, rc + wall] minus the hole bore.  Inlet disk on k = nz-2, outlet disk on
// k = 1.  Porous band: fluid cells at/above the apex inside the wall within band_thickness of
// it (this includes the hole bore, which the filter paper covers).
int orc_build_flags(const pog_params* p, uint32_t* flags) {
  if (p->inlet_control) return -1;  // device pointer: not readable by the CPU restatement
  Geo g = make_geo(p);
  const double apex = p->cone_apex_z, wall = p->cone_wall, hole = p->hole_radius;
  const double rin = p->inlet_radius, band = p->band_thickness;
  std::vector<uint8_t> solid(g.n);
  for (int k = 0; k < g.nz; ++k)
    for (int j = 0; j < g.ny; ++j)
      for (int i = 0; i < g.nx; ++i) {
        double x = i, y = j, z = k;
        double dx = x - g.cx, dy = y - g.cy;
        double r = sqrt(dx * dx + dy * dy);
        bool s = (i == 0 || j == 0 || k == 0 || i == g.nx - 1 || j == g.ny - 1 || k == g.nz - 1);
        double rc = (z - apex) * g.tanth;
        if (z < apex) {
          if (r > hole) s = true;
        } else if (r > rc && r <= rc + wall && r > hole) {
          s = true;
        }
        solid[g.idx(i, j, k)] = s ? 1 : 0;
      }
  for (int k = 0; k < g.nz; ++k)
    for (int j = 0; j < g.ny; ++j)
      for (int i = 0; i < g.nx; ++i) {
        long long c = g.idx(i, j, k);
        uint32_t fl = 0;
        if (solid[c]) {
          flags[c] = POG_CELL_SOLID;
          continue;
        }
        double x = i, y = j, z = k;
        double dx = x - g.cx, dy = y - g.cy;
        double r = sqrt(dx * dx + dy * dy);
        double rc = (z - apex) * g.tanth;
        if (k == g.nz - 2 && r <= rin) fl |= POG_CELL_INLET;
        if (k == 1 && r <= hole) fl |= POG_CELL_OUTLET;
        if (!(fl & (POG_CELL_INLET | POG_CELL_OUTLET)) && band > 0 && z >= apex && r > rc - band &&
            r <= rc + wall)
          fl |= POG_CELL_POROUS;
        for (int q = 1; q < 19; ++q)
          if (solid[g.idx(i + CX[q], j + CY[q], k + CZ[q])]) fl |= POG_CELL_NEAR_SOLID | (1u << (POG_LINK_SHIFT + q));
        flags[c] = fl;
      }
  return 0;
}

int orc_init_equilibrium_f32(const pog_params* p, const uint32_t* flags, float* f, float rho0,
                             float ux, float uy, float uz) {
  init_eq<float>(p, flags, f, rho0, ux, uy, uz);
  return 0;
}
int orc_init_equilibrium_f64(const pog_params* p, const uint32_t* flags, double* f, double rho0,
                             double ux, double uy, double uz) {
  init_eq<double>(p, flags, f, rho0, ux, uy, uz);
  return 0;
}

// One step, natural layout, f_out must be a different buffer.  u_prev: [3][n] velocity of the
// previous step (LES stencil mode) or null.  Fe: [3][n] float external force or null.
// Pd: [4][n] float particle drag deposit (Kp, Kv) or null.
int orc_step_f32(const pog_params* p, const uint32_t* flags, const float* f, float* fo,
                 const float* Fe, const float* Pd, const float* eps, const float* u_prev,
                 float* rho_out, float* u_out, double* red) {
  return step_push<float>(p, flags, f, fo, Fe, Pd, eps, u_prev, rho_out, u_out, red);
}
int orc_step_f64(const pog_params* p, const uint32_t* flags, const double* f, double* fo,
                 const float* Fe, const float* Pd, const float* eps, const double* u_prev,
                 double* rho_out, double* u_out, double* red) {
  return step_push<double>(p, flags, f, fo, Fe, Pd, eps, u_prev, rho_out, u_out, red);
}

// In-place AA-pattern step at time t (les_mode OFF or LOCAL: the stencil mode's u history is the
// push step's business).
int orc_step_aa_f32(const pog_params* p, const uint32_t* flags, float* f, long long t, const float* Fe,
                    const float* Pd, const float* eps, float* rho_out, float* u_out, double* red) {
  if (p->les_mode == POG_LES_STENCIL) return -1;
  return step_aa<float>(p, flags, f, t, Fe, Pd, eps, rho_out, u_out, red);
}
int orc_step_aa_f64(const pog_params* p, const uint32_t* flags, double* f, long long t, const float* Fe,
                    const float* Pd, const float* eps, double* rho_out, double* u_out, double* red) {
  if (p->les_mode == POG_LES_STENCIL) return -1;
  return step_aa<double>(p, flags, f, t, Fe, Pd, eps, rho_out, u_out, red);
}

// ---- function-level helpers for the known-answer tests ------------------------------------
void orc_set_legacy_feq_order(int on) { g_legacy_feq_order = on ? 1 : 0; }
void orc_equilibrium_f64(double rho, double ux, double uy, double uz, double* feq) {
  equilibrium<double>(rho, ux, uy, uz, feq);
}
void orc_equilibrium_f32(float rho, float ux, float uy, float uz, float* feq) {
  equilibrium<float>(rho, ux, uy, uz, feq);
}
// rho = sum f, u = sum f e / rho (lbm_algorithms.py macroscopic_density/velocity_unified).
void orc_moments_f64(const double* f, double* rho, double* u) {
  double r = 0, mx = 0, my = 0, mz = 0;
  for (int q = 0; q < 19; ++q) {
    r += f[q];
    mx += CX[q] * f[q];
    my += CY[q] * f[q];
    mz += CZ[q] * f[q];
  }
  *rho = r;
  u[0] = r > 1e-12 ? mx / r : 0;
  u[1] = r > 1e-12 ? my / r : 0;
  u[2] = r > 1e-12 ? mz / r : 0;
}
// LES nu_sgs field from a [3][n] velocity (les_turbulence.py:318-380).
int orc_les_nu_f32(const pog_params* p, const uint32_t* flags, const float* u, float* nu) {
  Geo g = make_geo(p);
  for (int k = 0; k < g.nz; ++k)
    for (int j = 0; j < g.ny; ++j)
      for (int i = 0; i < g.nx; ++i) nu[g.idx(i, j, k)] = les_nu_stencil<float>(p, g, flags, u, i, j, k);
  return 0;
}
// Darcy-Forchheimer force density at a given rho/u in porous cells, the drag_mode form
// (filter_paper.py:471-536).  F: [3][n]; zero outside the band.
int orc_porous_force_f32(const pog_params* p, const uint32_t* flags, const float* rho,
                         const float* u, float* F) {
  Geo g = make_geo(p);
  const long long n = g.n;
  float nu0 = (p->tau - 0.5f) / 3.0f;
  for (long long c = 0; c < n; ++c) {
    F[c] = F[n + c] = F[2 * n + c] = 0;
    if (!(flags[c] & POG_CELL_POROUS) || (flags[c] & POG_CELL_SOLID)) continue;
    float K = p->permeability, CF = p->forchheimer, sK = sqrtf(K);
    float ux = u[c], uy = u[n + c], uz = u[2 * n + c];
    float um = sqrtf(ux * ux + uy * uy + uz * uz);
    float coef = rho[c] * (nu0 / K + CF / sK * um);
    float dx = -coef * ux, dy = -coef * uy, dz = -coef * uz;
    if (p->drag_mode == POG_DRAG_EXPLICIT_CAP) {
      float dm = sqrtf(dx * dx + dy * dy + dz * dz);
      if (dm > p->drag_cap) {
        float s = p->drag_cap / dm;
        dx *= s;
        dy *= s;
        dz *= s;
      }
    }
    F[c] = dx;
    F[n + c] = dy;
    F[2 * n + c] = dz;
  }
  return 0;
}
void orc_inlet_velocity_f64(const pog_params* p, const double* r, double* uz, int m) {
  for (int i = 0; i < m; ++i) uz[i] = inlet_velocity<double>(p, r[i]);
}
// Filter-paper dynamics (filter_paper.py:616-750), the library's filter.cu restated: the
// particle bounce with the lowbias32 roughness kicks, and the blockage update.
static uint32_t lowbias32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}
static float hash_uniform(uint32_t seed, uint32_t step, uint32_t id, uint32_t lane) {
  const uint32_t h = lowbias32(seed ^ lowbias32(step ^ lowbias32(id * 2u + lane)));
  return (float)(h >> 8) * (1.0f / 16777216.0f);
}
void orc_filter_particles(const pog_params* p, const uint32_t* flags, const float* pos, float* vel,
                          const int32_t* active, int np, float* accum, uint32_t seed, long long step) {
  const uint32_t nx = p->nx, ny = p->ny, nz = p->nz;
  for (int q = 0; q < np; ++q) {
    if (!active[q]) continue;
    const float x = pos[q], y = pos[np + q], z = pos[2 * np + q];
    if (!(x >= 0.0f && y >= 0.0f && z >= 0.0f)) continue;
    const uint32_t i = (uint32_t)x, j = (uint32_t)y, k = (uint32_t)z;
    if (i >= nx || j >= ny || k >= nz) continue;
    for (int o = -2; o <= 2; ++o) {
      const int kk = (int)k + o;
      if (kk < 0 || kk >= (int)nz) continue;
      const uint32_t c = ((uint32_t)kk * ny + j) * nx + i;
      if (!(flags[c] & POG_CELL_POROUS)) continue;
      const float vz = vel[2 * np + q];
      if (vz < 0.0f) {
        vel[2 * np + q] = -vz * 0.3f;
        vel[q] = vel[q] + (hash_uniform(seed, (uint32_t)step, (uint32_t)q, 0u) - 0.5f) * 0.01f;
        vel[np + q] = vel[np + q] + (hash_uniform(seed, (uint32_t)step, (uint32_t)q, 1u) - 0.5f) * 0.01f;
        accum[c] = accum[c] + 0.01f;
      }
      break;
    }
  }
}
void orc_filter_update(const pog_params* p, const uint32_t* flags, float* accum, float* blockage) {
  const long long n = (long long)p->nx * p->ny * p->nz;
  for (long long c = 0; c < n; ++c) {
    if (!(flags[c] & POG_CELL_POROUS)) continue;
    const float a = accum[c];
    const float nb = 0.9f * (1.0f - expf(-0.1f * a));
    blockage[c] = 0.95f * blockage[c] + 0.05f * nb;
    accum[c] = a * 0.999f;
  }
}

// Pressure-gradient drive (pressure_gradient_drive.py:95-193), the library's drive.cu restated.
void orc_pressure_force(const pog_params* p, const uint32_t* flags, const float* rho, float* force, float scale,
                        float max_force) {
  const long long nx = p->nx, ny = p->ny, nz = p->nz, n = nx * ny * nz, pl = nx * ny;
  for (long long k = 0; k < nz; ++k)
    for (long long j = 0; j < ny; ++j)
      for (long long i = 0; i < nx; ++i) {
        const long long c = (k * ny + j) * nx + i;
        if (flags[c] & POG_CELL_SOLID) continue;
        const float r = rho[c];
        float gx, gy, gz;
        if (i > 0 && i < nx - 1) gx = (rho[c + 1] - rho[c - 1]) * 0.5f;
        else if (i == 0) gx = rho[c + 1] - r;
        else gx = r - rho[c - 1];
        if (j > 0 && j < ny - 1) gy = (rho[c + nx] - rho[c - nx]) * 0.5f;
        else if (j == 0) gy = rho[c + nx] - r;
        else gy = r - rho[c - nx];
        if (k > 0 && k < nz - 1) gz = (rho[c + pl] - rho[c - pl]) * 0.5f;
        else if (k == 0) gz = rho[c + pl] - r;
        else gz = r - rho[c - pl];
        float fx = 0.0f, fy = 0.0f, fz = 0.0f;
        if (r > 1e-12f) {
          const float cs2 = 1.0f / 3.0f;
          fx = -(gx * cs2) / r;
          fy = -(gy * cs2) / r;
          fz = -(gz * cs2) / r;
          const float m = sqrtf(fx * fx + fy * fy + fz * fz);
          if (m > max_force) {
            const float s = max_force / m;
            fx *= s;
            fy *= s;
            fz *= s;
          }
        }
        force[c] += scale * fx;
        force[n + c] += scale * fy;
        force[2 * n + c] += scale * fz;
      }
}
void orc_density_drive(const pog_params* p, const uint32_t* flags, float* rho, const float* target, float rate,
                       float max_adjust, float lo, float hi) {
  const long long pl = (long long)p->nx * p->ny, n = pl * p->nz;
  for (long long c = 0; c < n; ++c) {
    if (flags[c] & POG_CELL_SOLID) continue;
    const float r = rho[c];
    float a = (target[c / pl] - r) * rate;
    if (fabsf(a) > max_adjust) a = a > 0.0f ? max_adjust : -max_adjust;
    rho[c] = std::max(lo, std::min(hi, r + a));
  }
}

// Multiphase phase field (multiphase_3d.py:80-381) and the pour stream's phase change
// (precise_pouring.py:166-193), the library's multiphase.cu restated.
struct PG {
  long long nx, ny, nz, pl, n;
  bool interior(long long c) const {
    const long long i = c % nx, j = (c / nx) % ny, k = c / pl;
    return i >= 1 && i + 1 < nx && j >= 1 && j + 1 < ny && k >= 1 && k + 1 < nz;
  }
  float lap7(const float* a, long long c) const {
    return a[c + 1] + a[c - 1] + a[c + nx] + a[c - nx] + a[c + pl] + a[c - pl] - 6.0f * a[c];
  }
};
static PG pgrid(const pog_params* p) {
  PG g;
  g.nx = p->nx;
  g.ny = p->ny;
  g.nz = p->nz;
  g.pl = g.nx * g.ny;
  g.n = g.pl * g.nz;
  return g;
}
void orc_phase_chemical_potential(const pog_params* p, const float* phi, float kappa, float* mu) {
  const PG g = pgrid(p);
  for (long long c = 0; c < g.n; ++c) {
    if (!g.interior(c)) continue;
    const float ph = phi[c];
    const float lap = g.lap7(phi, c);
    mu[c] = (ph * ph * ph - ph) + (-kappa * lap);
  }
}
void orc_phase_normals(const pog_params* p, const float* phi, float* normal, float* gmag) {
  const PG g = pgrid(p);
  for (long long c = 0; c < g.n; ++c) {
    if (!g.interior(c)) continue;
    const float gx = (phi[c + 1] - phi[c - 1]) * 0.5f;
    const float gy = (phi[c + g.nx] - phi[c - g.nx]) * 0.5f;
    const float gz = (phi[c + g.pl] - phi[c - g.pl]) * 0.5f;
    const float m = sqrtf(gx * gx + gy * gy + gz * gz);
    float nx = 0.0f, ny = 0.0f, nz = 0.0f;
    if (m > 1e-10f) {
      nx = gx / m;
      ny = gy / m;
      nz = gz / m;
    }
    normal[c] = nx;
    normal[g.n + c] = ny;
    normal[2 * g.n + c] = nz;
    gmag[c] = m;
  }
}
void orc_phase_surface_tension(const pog_params* p, const uint32_t* flags, const float* phi, const float* normal,
                               const float* gmag, const float* rho, float sigma, float* body_force, float* curvature,
                               float* sforce) {
  const PG g = pgrid(p);
  for (long long c = 0; c < g.n; ++c) {
    if (!g.interior(c)) continue;
    const float m = gmag[c];
    float kap = 0.0f;
    if (m > 1e-10f)
      kap = (normal[c + 1] - normal[c - 1]) * 0.5f + (normal[g.n + c + g.nx] - normal[g.n + c - g.nx]) * 0.5f +
            (normal[2 * g.n + c + g.pl] - normal[2 * g.n + c - g.pl]) * 0.5f;
    float fx = 0.0f, fy = 0.0f, fz = 0.0f;
    if (fabsf(phi[c]) < 0.9f && m > 1e-10f) {
      const float fm = sigma * kap * m;
      fx = fm * normal[c];
      fy = fm * normal[g.n + c];
      fz = fm * normal[2 * g.n + c];
    }
    if (curvature) curvature[c] = kap;
    if (sforce) {
      sforce[c] = fx;
      sforce[g.n + c] = fy;
      sforce[2 * g.n + c] = fz;
    }
    if (body_force && !(flags[c] & POG_CELL_SOLID) && rho[c] > 1e-10f) {
      body_force[c] += fx / rho[c];
      body_force[g.n + c] += fy / rho[c];
      body_force[2 * g.n + c] += fz / rho[c];
    }
  }
}
void orc_phase_update(const pog_params* p, const uint32_t* flags, const float* phi, float* phi_new, const float* u,
                      const float* mu, float mobility, float dt, float rho_air, float rho_water, float* rho,
                      float* phase) {
  const PG g = pgrid(p);
  const float drho = (float)((double)rho_water - (double)rho_air);
  for (long long c = 0; c < g.n; ++c) {
    const float ph = phi[c];
    float pn = ph;
    if (g.interior(c)) {
      float ux = 0.0f, uy = 0.0f, uz = 0.0f;
      if (!(flags[c] & POG_CELL_SOLID)) {
        ux = u[c];
        uy = u[g.n + c];
        uz = u[2 * g.n + c];
      }
      const float dx = ux > 0.0f ? ph - phi[c - 1] : phi[c + 1] - ph;
      const float dy = uy > 0.0f ? ph - phi[c - g.nx] : phi[c + g.nx] - ph;
      const float dz = uz > 0.0f ? ph - phi[c - g.pl] : phi[c + g.pl] - ph;
      const float conv = -(ux * dx + uy * dy + uz * dz);
      float diff = 0.0f;
      if (mu) diff = mobility * g.lap7(mu, c);
      pn = ph + dt * (conv + diff);
      pn = std::max(-1.0f, std::min(1.0f, pn));
      if (fabsf(ph) < 0.99f) {
        const float lap = g.lap7(phi, c);
        const float chem = ph * (ph * ph - 1.0f) - 0.01f * lap;
        pn = pn + -0.001f * chem * dt;
      }
    }
    phi_new[c] = pn;
    if (rho) {
      const float pc = std::max(-1.0f, std::min(1.0f, pn));
      rho[c] = rho_air + drho * (pc + 1.0f) / 2.0f;
      phase[c] = (pc + 1.0f) / 2.0f;
    }
  }
}
void orc_phase_properties(const pog_params* p, const float* phi, float rho_air, float rho_water, float* rho,
                          float* phase) {
  const PG g = pgrid(p);
  const float drho = (float)((double)rho_water - (double)rho_air);
  for (long long c = 0; c < g.n; ++c) {
    const float pc = std::max(-1.0f, std::min(1.0f, phi[c]));
    rho[c] = rho_air + drho * (pc + 1.0f) / 2.0f;
    phase[c] = (pc + 1.0f) / 2.0f;
  }
}
void orc_pour_phase(const pog_params* p, const uint32_t* flags, float* phi, float dt) {
  const float* b = p->pour_control;  // HOST block for the restatement
  if (!b || b[POG_POUR_ACTIVE] == 0.0f) return;
  const PG g = pgrid(p);
  const float ztop = b[POG_POUR_ZTOP];
  const float klo = ceilf(ztop - b[POG_POUR_HEIGHT]), khi = floorf(ztop);
  if (!(khi >= 0.0f) || klo > (float)(g.nz - 1) || khi < klo) return;
  const long long k0 = (long long)std::max(klo, 0.0f), k1 = (long long)std::min(khi, (float)(g.nz - 1));
  const float R = b[POG_POUR_RADIUS], px = b[POG_POUR_X], py = b[POG_POUR_Y], flow = b[POG_POUR_FLOW];
  for (long long k = k0; k <= k1; ++k)
    for (long long j = 0; j < g.ny; ++j)
      for (long long i = 0; i < g.nx; ++i) {
        const long long c = k * g.pl + j * g.nx + i;
        if (flags[c] & POG_CELL_SOLID) continue;
        const float dx = (float)i - px, dy = (float)j - py;
        const float d = sqrtf(dx * dx + dy * dy);
        if (!(d <= R)) continue;
        const float dr = d / R;
        const float I = expf(-0.5f * dr * dr) * expf(-(ztop - (float)k) / 2.0f);
        if (!(I > 0.0f)) continue;
        const float cur = phi[c];
        float rate = (1.0f - cur) / 0.05f;
        rate = std::max(-2.0f, std::min(2.0f, rate));
        const float nw = cur + rate * I * dt * flow;
        phi[c] = std::max(-1.0f, std::min(1.0f, nw));
      }
}

// One nozzle step of a host pour block (pour_advance_kernel in the library).
void orc_pour_advance(const pog_params* p, float* b) {
  if (b[POG_POUR_ACTIVE] == 0.0f) return;
  const float time = b[POG_POUR_TIME] + b[POG_POUR_DT];
  b[POG_POUR_TIME] = time;
  float x = b[POG_POUR_CX], y = b[POG_POUR_CY];
  if (b[POG_POUR_PATTERN] == 1.0f) {
    const float t = time * b[POG_POUR_SPIRAL_SPEED];
    const float r = b[POG_POUR_SPIRAL_R] * (1.0f + 0.1f * t);
    const float d = b[POG_POUR_DIAMETER];
    x = std::fmax(d, std::fmin((float)p->nx - d, x + r * std::cos(t)));
    y = std::fmax(d, std::fmin((float)p->ny - d, y + r * std::sin(t)));
  }
  b[POG_POUR_X] = x;
  b[POG_POUR_Y] = y;
}
float orc_round_storage(int storage, float v, int q, float rho0) {
  return store_round<float>(storage, v, q, rho0);
}

}  // extern "C"

// =========================================================================================
// Adjoint oracle: forward-mode dual numbers pushed through the same collide<T> above.  For a
// fluid cell the 19 incoming populations, the cell porosity and the 16 inlet coefficients
// are seeded as independent directions, which gives the exact Jacobian of the restated
// collision; the adjoint of one push step is then lam_t(c) = J^T lam*(c) (+ dflux/df), with
// lam* pulled through the transpose of push streaming.  This is automatic differentiation of
// the restatement, independent of the hand-derived CUDA adjoint it checks.
namespace {
const int ND = 19 + 1 + POG_INLET_NCOEF + 18;  // f_q, eps, a_k, the stencil neighbours' u
struct Dual {
  double v;
  double d[ND];
  Dual() : v(0) { memset(d, 0, sizeof(d)); }
  Dual(double x) : v(x) { memset(d, 0, sizeof(d)); }  // NOLINT (implicit from constants)
  explicit operator double() const { return v; }
};
inline Dual operator+(const Dual& a, const Dual& b) {
  Dual r(a.v + b.v);
  for (int i = 0; i < ND; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
inline Dual operator-(const Dual& a, const Dual& b) {
  Dual r(a.v - b.v);
  for (int i = 0; i < ND; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
inline Dual operator-(const Dual& a) {
  Dual r(-a.v);
  for (int i = 0; i < ND; ++i) r.d[i] = -a.d[i];
  return r;
}
inline Dual operator*(const Dual& a, const Dual& b) {
  Dual r(a.v * b.v);
  for (int i = 0; i < ND; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
inline Dual operator/(const Dual& a, const Dual& b) {
  Dual r(a.v / b.v);
  for (int i = 0; i < ND; ++i) r.d[i] = (a.d[i] * b.v - a.v * b.d[i]) / (b.v * b.v);
  return r;
}
inline Dual& operator+=(Dual& a, const Dual& b) { return a = a + b; }
inline Dual& operator-=(Dual& a, const Dual& b) { return a = a - b; }
inline Dual& operator*=(Dual& a, const Dual& b) { return a = a * b; }
inline bool operator<(const Dual& a, const Dual& b) { return a.v < b.v; }
inline bool operator>(const Dual& a, const Dual& b) { return a.v > b.v; }
inline bool operator<=(const Dual& a, const Dual& b) { return a.v <= b.v; }
inline bool operator>=(const Dual& a, const Dual& b) { return a.v >= b.v; }
inline Dual exp(const Dual& a) {
  Dual r(::exp(a.v));
  for (int i = 0; i < ND; ++i) r.d[i] = a.d[i] * r.v;
  return r;
}
inline Dual sqrt(const Dual& a) {
  Dual r(::sqrt(a.v));
  double g = a.v > 0 ? 0.5 / r.v : 0.0;  // zero subgradient at 0, as the CUDA adjoint
  for (int i = 0; i < ND; ++i) r.d[i] = a.d[i] * g;
  return r;
}
}  // namespace

// Pd (nullable): the step's particle drag deposit [4][n] (Kp, Kv), a fixed input (constants in
// the dual numbers), as the CUDA adjoint takes it.
// LES stencil mode: u_prev [3][n] is the velocity the step's nu_sgs reads (the previous step's
// output), mu_in [3][n] (nullable) dJ/du of the velocity this step outputs (read by the next
// step's stencil), mu_out [3][n] receives (+=) dJ/du_prev; the six neighbours' velocities are
// seeded as dual directions 36..53.
extern "C" int orc_adjoint_step_f64(const pog_params* p, const uint32_t* flags, const double* ft,
                                    const double* lam_next, double* lam_t, const float* eps,
                                    const float* Pd, const double* u_prev, const double* mu_in,
                                    double* mu_out, double* grad_eps, double* grad_inlet) {
  const bool stencil = p->les_mode == POG_LES_STENCIL;
  if (stencil && !u_prev) return -1;
  Geo g = make_geo(p);
  const long long n = g.n;
  std::vector<double> gi_acc(POG_INLET_NCOEF, 0.0);
#pragma omp parallel
  {
    std::vector<double> gi(POG_INLET_NCOEF, 0.0);
#pragma omp for schedule(static)
    for (int k = 0; k < g.nz; ++k)
      for (int j = 0; j < g.ny; ++j)
        for (int i = 0; i < g.nx; ++i) {
          long long c = g.idx(i, j, k);
          uint32_t fl = flags[c];
          if (fl & POG_CELL_SOLID) {
            for (int q = 0; q < 19; ++q) lam_t[q * n + c] = 0;
            continue;
          }
          double ls[19];
          for (int q = 0; q < 19; ++q) {
            long long nb = g.idx(i + CX[q], j + CY[q], k + CZ[q]);
            ls[q] = (flags[nb] & POG_CELL_SOLID) ? lam_next[OPP[q] * n + c] : lam_next[q * n + nb];
          }
          Dual f[19], fs[19], rho, u[3];
          for (int q = 0; q < 19; ++q) {
            f[q] = Dual(ft[q * n + c]);
            f[q].d[q] = 1.0;
          }
          Dual e(eps ? (double)eps[c] : 0.0);
          e.d[19] = 1.0;
          Dual coef[POG_INLET_NCOEF];
          for (int kk = 0; kk < POG_INLET_NCOEF; ++kk) {
            coef[kk] = Dual((double)p->inlet_coef[kk]);
            coef[kk].d[20 + kk] = 1.0;
          }
          Dual pd[4];
          if (Pd)
            for (int a = 0; a < 4; ++a) pd[a] = Dual((double)Pd[a * n + c]);
          Dual nus(0.0);
          long long nb[6];
          const bool st_cell = stencil && les_stencil_cell(g, flags, i, j, k);
          if (st_cell) {
            stencil_neighbours(g, i, j, k, nb);
            Dual un[6][3];
            for (int m = 0; m < 6; ++m)
              for (int a = 0; a < 3; ++a) {
                un[m][a] = Dual(u_prev[a * n + nb[m]]);
                un[m][a].d[36 + 3 * m + a] = 1.0;
              }
            nus = les_nu_from_neighbours<Dual>(p, un);
          }
          collide<Dual>(p, g, fl, i, j, k, f, nullptr, Pd ? pd : nullptr, eps != nullptr, e, nus, fs,
                        rho, u, nullptr, coef);
          // dJ/du of this step's output velocity (stencil mode) joins through u's derivatives
          double mu[3] = {0, 0, 0};
          if (stencil && mu_in)
            for (int a = 0; a < 3; ++a) mu[a] = mu_in[a * n + c];
          auto pull = [&](int dir) {
            double acc = 0;
            for (int pq = 0; pq < 19; ++pq) acc += ls[pq] * fs[pq].d[dir];
            for (int a = 0; a < 3; ++a) acc += mu[a] * u[a].d[dir];
            return acc;
          };
          for (int q = 0; q < 19; ++q) {
            double acc = pull(q);
            if (fl & POG_CELL_OUTLET) acc += -(double)CZ[q];
            lam_t[q * n + c] = acc;
          }
          if (grad_eps && eps) grad_eps[c] += pull(19);
          for (int kk = 0; kk < POG_INLET_NCOEF; ++kk) gi[kk] += pull(20 + kk);
          if (st_cell && mu_out)
            for (int m = 0; m < 6; ++m)
              for (int a = 0; a < 3; ++a) {
                double acc = 0;
                for (int pq = 0; pq < 19; ++pq) acc += ls[pq] * fs[pq].d[36 + 3 * m + a];
                if (acc != 0.0) {
#pragma omp atomic
                  mu_out[a * n + nb[m]] += acc;
                }
              }
        }
#pragma omp critical
    for (int kk = 0; kk < POG_INLET_NCOEF; ++kk) gi_acc[kk] += gi[kk];
  }
  if (grad_inlet)
    for (int kk = 0; kk < POG_INLET_NCOEF; ++kk) grad_inlet[kk] += gi_acc[kk];
  return 0;
}
