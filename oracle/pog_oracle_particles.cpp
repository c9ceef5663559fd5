// pog_oracle_particles.cpp -- CPU restatement of the particle side.  TEST INFRASTRUCTURE ONLY.
//
// Restates CoffeeParticleSystem's two-way coupling (src/physics/coffee_particles.py:
// interpolate_fluid_velocity_from_field 1156-1198, distribute_force_to_grid 1048-1086,
// compute_drag_coefficient 1088-1099, compute_two_way_coupling_forces 1107-1154,
// apply_under_relaxation 1200-1212, update_particle_physics 641-720 with the cone constraint
// 734-831) and the coupled-step order of LBMSolver.step_with_two_way_coupling
// (legacy/lbm_solver.py:1485-1509), in lattice units, with the build-spec corrections:
// Stokes drag in lattice units (the reference's magnitude misses a |u_rel| factor), the
// relaxed force is integrated, the particles are integrated in the coupled step, and the
// fluid receives the drag implicitly: each particle deposits beta = m_p/(tau_p + dt) and
// beta*v_new (Kp, Kv) on the 8 gather nodes and the lattice step applies Kv - Kp u.  Every operation is a single IEEE float operation evaluated in the written
// order (compiled with -ffp-contract=off), so per-particle results are bit-identical with the
// CUDA kernels, and the fixed-point drag deposit is bit-identical too.
//
// Only tests/, smoke() and bench.py's CPU leg use this file.

#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "../include/pog.h"

namespace {
const float PI_F = 3.14159265358979f;
const double FIX_SCALE = 4294967296.0;  // 2^32

struct PGeo {
  int nx, ny, nz;
  long long n;
  float cx, cy, tanth;
};
PGeo pgeo(const pog_params* p) {
  PGeo g;
  g.nx = p->nx;
  g.ny = p->ny;
  g.nz = p->nz;
  g.n = (long long)p->nx * p->ny * p->nz;
  g.cx = (float)(p->center_x < 0 ? 0.5 * p->nx : (double)p->center_x);
  g.cy = (float)(p->center_y < 0 ? 0.5 * p->ny : (double)p->center_y);
  g.tanth = (float)tan((double)p->cone_half_angle_deg * M_PI / 180.0);
  return g;
}

// Cell of a position: int(max(0, min(n-2, x))) per axis (coffee_particles.py:1162-1164).
inline int cell_axis(float x, int n) {
  float a = fminf((float)(n - 2), x);
  a = fmaxf(0.0f, a);
  return (int)a;
}
}  // namespace

extern "C" {

int orc_particles_bin(const pog_params* p, const float* pos, const int32_t* active, int np,
                      int32_t* keys, int32_t* perm) {
  PGeo g = pgeo(p);
  for (int q = 0; q < np; ++q) {
    if (!active[q]) {
      keys[q] = (int32_t)g.n;
      continue;
    }
    int i = cell_axis(pos[q], g.nx);
    int j = cell_axis(pos[np + q], g.ny);
    int k = cell_axis(pos[2 * np + q], g.nz);
    keys[q] = (int32_t)(i + (long long)g.nx * (j + (long long)g.ny * k));
  }
  std::vector<int32_t> idx(np);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int32_t a, int32_t b) { return keys[a] < keys[b]; });
  for (int q = 0; q < np; ++q) perm[q] = idx[q];
  return 0;
}

// Trilinear interpolation of a [3][n] field at positions (coffee_particles.py:1156-1198),
// summed in the reference's order.  Used by the interpolation known-answer test.
int orc_trilinear_f32(int nx, int ny, int nz, const float* u, const float* pos, int m, float* out) {
  long long n = (long long)nx * ny * nz;
  for (int q = 0; q < m; ++q) {
    float x = pos[3 * q], y = pos[3 * q + 1], z = pos[3 * q + 2];
    int i = cell_axis(x, nx), j = cell_axis(y, ny), k = cell_axis(z, nz);
    float fx = fmaxf(0.0f, fminf(1.0f, x - (float)i));
    float fy = fmaxf(0.0f, fminf(1.0f, y - (float)j));
    float fz = fmaxf(0.0f, fminf(1.0f, z - (float)k));
    float w000 = (1 - fx) * (1 - fy) * (1 - fz), w001 = (1 - fx) * (1 - fy) * fz;
    float w010 = (1 - fx) * fy * (1 - fz), w011 = (1 - fx) * fy * fz;
    float w100 = fx * (1 - fy) * (1 - fz), w101 = fx * (1 - fy) * fz;
    float w110 = fx * fy * (1 - fz), w111 = fx * fy * fz;
    auto I = [&](int a, int b, int c) { return ((long long)c * ny + b) * nx + a; };
    for (int a = 0; a < 3; ++a) {
      const float* v = u + a * n;
      float s = w000 * v[I(i, j, k)];
      s = s + w001 * v[I(i, j, k + 1)];
      s = s + w010 * v[I(i, j + 1, k)];
      s = s + w011 * v[I(i, j + 1, k + 1)];
      s = s + w100 * v[I(i + 1, j, k)];
      s = s + w101 * v[I(i + 1, j, k + 1)];
      s = s + w110 * v[I(i + 1, j + 1, k)];
      s = s + w111 * v[I(i + 1, j + 1, k + 1)];
      out[3 * q + a] = s;
    }
  }
  return 0;
}

// Under-relaxation F = a F_new + (1-a) F_old (coffee_particles.py:1200-1212).
void orc_under_relax(float a, const float* fnew, float* fold, float* fout, int m) {
  for (int q = 0; q < m; ++q) {
    fout[q] = a * fnew[q] + (1.0f - a) * fold[q];
    fold[q] = fout[q];
  }
}

// One coupling pass over all particles (serial, in id order).  force_fix: [4][n] int64
// accumulator (scale 2^32) of the drag deposit (Kp, Kv_x, Kv_y, Kv_z), added to.  u: [3][n]
// fluid velocity.  u_at (nullable): [3][np].
int orc_particles_couple(const pog_params* p, const pog_particle_params* pp, float* pos,
                         float* vel, const float* diam, float* drag_old, int32_t* active, int np,
                         const float* u, long long* force_fix, float* u_at) {
  PGeo g = pgeo(p);
  const long long n = g.n;
  const float nu0 = (p->tau - 0.5f) / 3.0f;
  const float mu = p->rho0 * nu0;
  const float rho_p = pp->density_ratio * p->rho0;
  const float alpha = pp->relaxation, dt = pp->dt;
  const float zlo = p->cone_apex_z + pp->z_floor, zhi = (float)(g.nz - 3);
  auto I = [&](int a, int b, int c) { return ((long long)c * g.ny + b) * g.nx + a; };
  for (int q = 0; q < np; ++q) {
    if (!active[q]) continue;
    float x = pos[q], y = pos[np + q], z = pos[2 * np + q];
    int i = cell_axis(x, g.nx), j = cell_axis(y, g.ny), k = cell_axis(z, g.nz);
    float fx = fmaxf(0.0f, fminf(1.0f, x - (float)i));
    float fy = fmaxf(0.0f, fminf(1.0f, y - (float)j));
    float fz = fmaxf(0.0f, fminf(1.0f, z - (float)k));
    float w[8];
    w[0] = (1 - fx) * (1 - fy) * (1 - fz);  // 000
    w[1] = (1 - fx) * (1 - fy) * fz;        // 001
    w[2] = (1 - fx) * fy * (1 - fz);        // 010
    w[3] = (1 - fx) * fy * fz;              // 011
    w[4] = fx * (1 - fy) * (1 - fz);        // 100
    w[5] = fx * (1 - fy) * fz;              // 101
    w[6] = fx * fy * (1 - fz);              // 110
    w[7] = fx * fy * fz;                    // 111
    long long nodes[8] = {I(i, j, k),         I(i, j, k + 1),         I(i, j + 1, k),
                          I(i, j + 1, k + 1), I(i + 1, j, k),         I(i + 1, j, k + 1),
                          I(i + 1, j + 1, k), I(i + 1, j + 1, k + 1)};
    float uf[3];
    for (int a = 0; a < 3; ++a) {
      const float* v = u + a * n;
      float s = w[0] * v[nodes[0]];
      for (int c = 1; c < 8; ++c) s = s + w[c] * v[nodes[c]];
      uf[a] = s;
    }
    if (u_at) {
      u_at[q] = uf[0];
      u_at[np + q] = uf[1];
      u_at[2 * np + q] = uf[2];
    }
    float v0[3] = {vel[q], vel[np + q], vel[2 * np + q]};
    float ur[3] = {uf[0] - v0[0], uf[1] - v0[1], uf[2] - v0[2]};
    float d = diam[q];
    float vol = (PI_F / 6.0f) * (d * d * d);
    float mp = rho_p * vol;
    float mf = p->rho0 * vol;
    float taup = mp / (3.0f * PI_F * mu * d);
    if (pp->drag_model == 1) {
      float urm = sqrtf(ur[0] * ur[0] + ur[1] * ur[1] + ur[2] * ur[2]);
      float re = p->rho0 * urm * d / mu;
      float fac = 1.0f;
      if (re >= 1000.0f)
        fac = 0.44f * re / 24.0f;
      else if (re >= 0.1f)
        fac = 1.0f + 0.15f * powf(re, 0.687f);
      taup = taup / fac;
    }
    float gvec[3] = {p->gx, p->gy, p->gz};
    float beta = mp / (taup + dt);  // drag coefficient: F_new = beta (u_f - v)
    float F[3], Fn[3];
    for (int a = 0; a < 3; ++a) {
      float fnew = mp * ur[a] / (taup + dt);
      Fn[a] = fnew;
      F[a] = alpha * fnew + (1.0f - alpha) * drag_old[a * np + q];
      drag_old[a * np + q] = F[a];
    }
    float nv[3], np3[3] = {x, y, z};
    // impact of the pour stream (create_water_impact_force, precise_pouring.py:190-226)
    float Fi[3] = {0.0f, 0.0f, 0.0f};
    bool impact = false;
    const float* b = p->pour_control;  // host copy of the POG_POUR_* block
    if (b && b[POG_POUR_ACTIVE] != 0.0f && b[POG_POUR_IMPACT] > 0.0f) {
      const float dx = x - b[POG_POUR_X], dy = y - b[POG_POUR_Y];
      const float R = b[POG_POUR_RADIUS];
      const float r = sqrtf(dx * dx + dy * dy);
      if (r <= R * 2.0f && z > b[POG_POUR_IMPACT_ZMIN]) {
        impact = true;
        const float S = b[POG_POUR_IMPACT];
        const float rr = r / R;
        const float I = expf(-0.5f * (rr * rr));
        Fi[2] = -S * I;
        if (r > 0.1f) {
          const float rm = S * 0.3f * I;
          Fi[0] = rm * dx / r;
          Fi[1] = rm * dy / r;
        }
        const float fm = sqrtf(Fi[0] * Fi[0] + Fi[1] * Fi[1] + Fi[2] * Fi[2]);
        if (fm > b[POG_POUR_IMPACT_MAX]) {
          const float sc = b[POG_POUR_IMPACT_MAX] / fm;
          for (int a = 0; a < 3; ++a) Fi[a] = Fi[a] * sc;
        }
      }
    }
    for (int a = 0; a < 3; ++a) {
      float acc = impact ? (F[a] + (mp - mf) * gvec[a] + Fi[a]) / mp : (F[a] + (mp - mf) * gvec[a]) / mp;
      nv[a] = v0[a] + acc * dt;
      np3[a] = np3[a] + nv[a] * dt;
    }
    bool hit = false;
    if (np3[2] < zlo) {
      np3[2] = zlo;
      hit = true;
    }
    if (np3[2] > zhi) {
      np3[2] = zhi;
      hit = true;
    }
    float rc = (np3[2] - p->cone_apex_z) * g.tanth;
    float dx = np3[0] - g.cx, dy = np3[1] - g.cy;
    float r = sqrtf(dx * dx + dy * dy);
    if (r > pp->wall_margin * rc) {
      float s = r > 0.0f ? (pp->wall_pullback * rc) / r : 0.0f;
      np3[0] = g.cx + dx * s;
      np3[1] = g.cy + dy * s;
      hit = true;
    }
    if (hit)
      for (int a = 0; a < 3; ++a) nv[a] = nv[a] * pp->wall_damping;
    bool ok = true;
    for (int a = 0; a < 3; ++a)
      if (!std::isfinite(np3[a]) || !std::isfinite(nv[a])) ok = false;
    if (!ok) {
      active[q] = 0;
      continue;
    }
    for (int a = 0; a < 3; ++a) {
      pos[a * np + q] = np3[a];
      vel[a * np + q] = nv[a];
    }
    // deposit Kp += w beta, Kv += w beta v_new on the 8 nodes of the gather position; the lattice
    // step takes the particle force on the fluid, Kv - Kp u, implicitly.  The explicit reactions
    // deposit Kp = 0, Kv = -w F (relaxed drag) or -w F_new (unrelaxed; distribute_force_to_grid,
    // coffee_particles.py:1048-1086 called at :1145-1149), which the step adds as a body force.
    float dep[4] = {beta, beta * nv[0], beta * nv[1], beta * nv[2]};
    if (pp->reaction != POG_REACTION_IMPLICIT) {
      const float* R = pp->reaction == POG_REACTION_EXPLICIT ? F : Fn;
      dep[0] = 0.0f;
      for (int a = 0; a < 3; ++a) dep[1 + a] = -R[a];
    }
    for (int a = 0; a < 4; ++a)
      for (int c = 0; c < 8; ++c) {
        float contrib = w[c] * dep[a];
        force_fix[a * n + nodes[c]] += (long long)llrint((double)contrib * FIX_SCALE);
      }
  }
  return 0;
}

}  // extern "C"
