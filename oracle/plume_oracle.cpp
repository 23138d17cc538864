// plume_oracle.cpp -- TEST INFRASTRUCTURE ONLY (see plume_oracle.h).
//
// FP64, single-threaded restatement of the reference's full-rank smoke step.
// Every function follows the reference code block cited beside it, operation
// for operation and in the same order, so that with the same compiler
// settings (no FMA contraction) it reproduces the reference bit for bit.
// Paths below are relative to the reference project root.
#include "plume_oracle.h"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <utility>
#include <vector>

namespace {

typedef double Real;

struct Grid {
  int X, Y, Z, slab, N;
  Grid(const int32_t r[3]) : X(r[0]), Y(r[1]), Z(r[2]), slab(r[0] * r[1]), N(r[0] * r[1] * r[2]) {}
};

// ---------------------------------------------------------------- noise
// SplitMix64 finaliser; the same integer recipe runs in the CUDA source kernel.
inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

inline double source_value(uint64_t seed, int32_t step, int64_t cell, double noise) {
  uint64_t h = mix64(seed + 0x9E3779B97F4A7C15ull);
  h = mix64(h + (uint64_t)(uint32_t)step * 0xD1B54A32D192ED03ull);
  h = mix64(h + (uint64_t)cell);
  double u = (double)(h >> 11) * (1.0 / 9007199254740992.0);  // [0,1), 53 bits
  return 1.0 + noise * (2.0 * u - 1.0);
}

// ---------------------------------------------------------------- obstacles
// Wall slabs from the six flags, FLUID_3D_MIC.cpp:105-159 (front/back = z,
// bottom/top = y, left/right = x).
void build_obstacles(const Grid& g, const int32_t bc[6], std::vector<uint8_t>& obst) {
  obst.assign(g.N, 0);
  const int front = bc[0], back = bc[1], left = bc[2], right = bc[3], top = bc[4], bottom = bc[5];
  for (int y = 0; y < g.Y; y++)
    for (int x = 0; x < g.X; x++) {
      int index = x + y * g.X;
      if (front == 1) obst[index] = 1;
      index += g.N - g.slab;
      if (back == 1) obst[index] = 1;
    }
  for (int z = 0; z < g.Z; z++)
    for (int x = 0; x < g.X; x++) {
      int index = x + z * g.slab;
      if (bottom == 1) obst[index] = 1;
      index += g.slab - g.X;
      if (top == 1) obst[index] = 1;
    }
  for (int z = 0; z < g.Z; z++)
    for (int y = 0; y < g.Y; y++) {
      int index = y * g.X + z * g.slab;
      if (left == 1) obst[index] = 1;
      index += g.X - 1;
      if (right == 1) obst[index] = 1;
    }
}

// ---------------------------------------------------------------- border ops
// VECTOR3_FIELD_3D::setZeroBorder, VECTOR3_FIELD_3D.cpp:2828-2867 (all 3 comps)
void vec_set_zero_border(const Grid& g, Real* v) {
  for (int z = 0; z < g.Z; z++)
    for (int y = 0; y < g.Y; y++) {
      int index = y * g.X + z * g.slab;
      v[3 * index] = v[3 * index + 1] = v[3 * index + 2] = 0.0;
      index += g.X - 1;
      v[3 * index] = v[3 * index + 1] = v[3 * index + 2] = 0.0;
    }
  for (int z = 0; z < g.Z; z++)
    for (int x = 0; x < g.X; x++) {
      int index = x + z * g.slab;
      v[3 * index] = v[3 * index + 1] = v[3 * index + 2] = 0.0;
      index += g.slab - g.X;
      v[3 * index] = v[3 * index + 1] = v[3 * index + 2] = 0.0;
    }
  for (int y = 0; y < g.Y; y++)
    for (int x = 0; x < g.X; x++) {
      int index = x + y * g.X;
      v[3 * index] = v[3 * index + 1] = v[3 * index + 2] = 0.0;
      index += g.N - g.slab;
      v[3 * index] = v[3 * index + 1] = v[3 * index + 2] = 0.0;
    }
}

// FIELD_3D::setZeroBorder, FIELD_3D.cpp:6408-6444
void sca_set_zero_border(const Grid& g, Real* s) {
  for (int z = 0; z < g.Z; z++)
    for (int y = 0; y < g.Y; y++) {
      int index = y * g.X + z * g.slab;
      s[index] = 0.0;
      s[index + g.X - 1] = 0.0;
    }
  for (int z = 0; z < g.Z; z++)
    for (int x = 0; x < g.X; x++) {
      int index = x + z * g.slab;
      s[index] = 0.0;
      s[index + g.slab - g.X] = 0.0;
    }
  for (int y = 0; y < g.Y; y++)
    for (int x = 0; x < g.X; x++) {
      int index = x + y * g.X;
      s[index] = 0.0;
      s[index + g.N - g.slab] = 0.0;
    }
}

// Per-axis face ops on one component.  mode: 0 zero (setZeroX/Y/Z,
// VECTOR3_FIELD_3D.cpp:2872-2924), 1 copy from 1 cell in (copyBorderX/Y/Z,
// 3005-3053), 2 copy from 2 cells in (setNeumannX/Y/Z, 2929-3000).
void vec_face(const Grid& g, Real* v, int axis, int mode) {
  if (axis == 0) {
    for (int z = 0; z < g.Z; z++)
      for (int y = 0; y < g.Y; y++) {
        int index = y * g.X + z * g.slab;
        v[3 * index] = (mode == 0) ? 0.0 : v[3 * (index + mode)];
        index += g.X - 1;
        v[3 * index] = (mode == 0) ? 0.0 : v[3 * (index - mode)];
      }
  } else if (axis == 1) {
    for (int z = 0; z < g.Z; z++)
      for (int x = 0; x < g.X; x++) {
        int index = x + z * g.slab;
        v[3 * index + 1] = (mode == 0) ? 0.0 : v[3 * (index + mode * g.X) + 1];
        index += g.slab - g.X;
        v[3 * index + 1] = (mode == 0) ? 0.0 : v[3 * (index - mode * g.X) + 1];
      }
  } else {
    for (int y = 0; y < g.Y; y++)
      for (int x = 0; x < g.X; x++) {
        int index = x + y * g.X;
        v[3 * index + 2] = (mode == 0) ? 0.0 : v[3 * (index + mode * g.slab) + 2];
        index += g.N - g.slab;
        v[3 * index + 2] = (mode == 0) ? 0.0 : v[3 * (index - mode * g.slab) + 2];
      }
  }
}

// FIELD_3D::copyBorderAll, FIELD_3D.cpp:1382-1420 (z faces, then y, then x)
void sca_copy_border_all(const Grid& g, Real* s) {
  for (int y = 0; y < g.Y; y++)
    for (int x = 0; x < g.X; x++) {
      int index = x + y * g.X;
      s[index] = s[index + g.slab];
      index += g.N - g.slab;
      s[index] = s[index - g.slab];
    }
  for (int z = 0; z < g.Z; z++)
    for (int x = 0; x < g.X; x++) {
      int index = x + z * g.slab;
      s[index] = s[index + g.X];
      index += g.slab - g.X;
      s[index] = s[index - g.X];
    }
  for (int z = 0; z < g.Z; z++)
    for (int y = 0; y < g.Y; y++) {
      int index = y * g.X + z * g.slab;
      s[index] = s[index + 1];
      index += g.X - 1;
      s[index] = s[index - 1];
    }
}

// ---------------------------------------------------------------- advection
// VECTOR3_FIELD_3D::advect (scalar 2082-2158, vector 2001-2077): trilinear
// backtrace in index space, clamped to [1.5, res-2.5], over every cell.
inline void trace(const Grid& g, Real dt, const Real* vel, int x, int y, int z, int& i000,
                  int& i010, int& i100, int& i110, int& i001, int& i011, int& i101,
                  int& i111, Real& s0, Real& s1, Real& t0, Real& t1, Real& u0, Real& u1) {
  const int index = x + y * g.X + z * g.slab;
  Real xTrace = x - dt * vel[3 * index];
  Real yTrace = y - dt * vel[3 * index + 1];
  Real zTrace = z - dt * vel[3 * index + 2];
  xTrace = (xTrace < 1.5) ? 1.5 : xTrace;
  xTrace = (xTrace > g.X - 2.5) ? g.X - 2.5 : xTrace;
  yTrace = (yTrace < 1.5) ? 1.5 : yTrace;
  yTrace = (yTrace > g.Y - 2.5) ? g.Y - 2.5 : yTrace;
  zTrace = (zTrace < 1.5) ? 1.5 : zTrace;
  zTrace = (zTrace > g.Z - 2.5) ? g.Z - 2.5 : zTrace;
  const int x0 = (int)xTrace, x1 = x0 + 1;
  const int y0 = (int)yTrace, y1 = y0 + 1;
  const int z0 = (int)zTrace, z1 = z0 + 1;
  s1 = xTrace - x0; s0 = 1.0 - s1;
  t1 = yTrace - y0; t0 = 1.0 - t1;
  u1 = zTrace - z0; u0 = 1.0 - u1;
  i000 = x0 + y0 * g.X + z0 * g.slab;
  i010 = x0 + y1 * g.X + z0 * g.slab;
  i100 = x1 + y0 * g.X + z0 * g.slab;
  i110 = x1 + y1 * g.X + z0 * g.slab;
  i001 = x0 + y0 * g.X + z1 * g.slab;
  i011 = x0 + y1 * g.X + z1 * g.slab;
  i101 = x1 + y0 * g.X + z1 * g.slab;
  i111 = x1 + y1 * g.X + z1 * g.slab;
}

// stride/offset select a component of an AoS field (stride 3) or a scalar (1).
void advect(const Grid& g, Real dt, const Real* vel, const Real* old_f, Real* new_f,
            int stride, int comp) {
  for (int z = 0; z < g.Z; z++)
    for (int y = 0; y < g.Y; y++)
      for (int x = 0; x < g.X; x++) {
        int i000, i010, i100, i110, i001, i011, i101, i111;
        Real s0, s1, t0, t1, u0, u1;
        trace(g, dt, vel, x, y, z, i000, i010, i100, i110, i001, i011, i101, i111, s0, s1,
              t0, t1, u0, u1);
        const int index = x + y * g.X + z * g.slab;
#define F(i) old_f[stride * (i) + comp]
        new_f[stride * index + comp] =
            u0 * (s0 * (t0 * F(i000) + t1 * F(i010)) + s1 * (t0 * F(i100) + t1 * F(i110))) +
            u1 * (s0 * (t0 * F(i001) + t1 * F(i011)) + s1 * (t0 * F(i101) + t1 * F(i111)));
#undef F
      }
}

// ---------------------------------------------------------------- Poisson
struct Solver {
  std::vector<Real> Adiag, Api, Apj, Apk, precon, residual, direction, q, z;
  void alloc(int N) {
    Adiag.assign(N, 0.0); Api.assign(N, 0.0); Apj.assign(N, 0.0); Apk.assign(N, 0.0);
    precon.assign(N, 0.0); residual.assign(N, 0.0); direction.assign(N, 0.0);
    q.assign(N, 0.0); z.assign(N, 0.0);
  }
};

// FLUID_3D_MIC::buildA, FLUID_3D_MIC.cpp:772-801 (heat = false: Aoff = 1)
void build_a(const Grid& g, const uint8_t* skip, Solver& s) {
  const int xs = 1, ys = g.X, zs = g.slab;
  const Real Aoff = 1.0;
  int index = g.slab + g.X + 1;
  for (int z = 1; z < g.Z - 1; z++, index += 2 * g.X)
    for (int y = 1; y < g.Y - 1; y++, index += 2)
      for (int x = 1; x < g.X - 1; x++, index++) {
        if (skip[index]) continue;
        s.Adiag[index] = 0.0;
        if (!skip[index + xs]) s.Adiag[index] += Aoff;
        if (!skip[index - xs]) s.Adiag[index] += Aoff;
        if (!skip[index + ys]) s.Adiag[index] += Aoff;
        if (!skip[index - ys]) s.Adiag[index] += Aoff;
        if (!skip[index + zs]) s.Adiag[index] += Aoff;
        if (!skip[index - zs]) s.Adiag[index] += Aoff;
        s.Api[index - xs] = skip[index - xs] ? 0.0 : -Aoff;
        s.Api[index] = skip[index + xs] ? 0.0 : -Aoff;
        s.Apj[index - ys] = skip[index - ys] ? 0.0 : -Aoff;
        s.Apj[index] = skip[index + ys] ? 0.0 : -Aoff;
        s.Apk[index - zs] = skip[index - zs] ? 0.0 : -Aoff;
        s.Apk[index] = skip[index + zs] ? 0.0 : -Aoff;
      }
}

// FLUID_3D_MIC::buildMICPreconditioner, FLUID_3D_MIC.cpp:825-856
void build_mic(const Grid& g, Real tau, Real sig, Solver& s) {
  const int xs = 1, ys = g.X, zs = g.slab;
  Real* P = s.precon.data();
  const Real *Ai = s.Api.data(), *Aj = s.Apj.data(), *Ak = s.Apk.data(), *Ad = s.Adiag.data();
  int index = g.slab + g.X + 1;
  for (int z = 1; z < g.Z - 1; z++, index += 2 * g.X)
    for (int y = 1; y < g.Y - 1; y++, index += 2)
      for (int x = 1; x < g.X - 1; x++, index++) {
        Real pmini2 = P[index - xs] * P[index - xs];
        Real pminj2 = P[index - ys] * P[index - ys];
        Real pmink2 = P[index - zs] * P[index - zs];
        Real e0 = Ai[index - xs] * Ai[index - xs] * pmini2 +
                  Aj[index - ys] * Aj[index - ys] * pminj2 +
                  Ak[index - zs] * Ak[index - zs] * pmink2;
        Real e1 = tau * (Ai[index - xs] * (Aj[index - xs] + Ak[index - xs]) * pmini2 +
                         Aj[index - ys] * (Ai[index - ys] + Ak[index - ys]) * pminj2 +
                         Ak[index - zs] * (Ai[index - zs] + Aj[index - zs]) * pmink2);
        Real e = Ad[index] - e0 - e1;
        if (e < sig * Ad[index]) e = Ad[index];
        if (fabs(Ad[index]) < 0.000001)
          P[index] = 0;
        else
          P[index] = 1.0 / sqrt(e);
      }
}

// FLUID_3D_MIC::multA, FLUID_3D_MIC.cpp:803-823
void mult_a(const Grid& g, const Solver& s, const Real* xf, Real* bf) {
  const int xs = 1, ys = g.X, zs = g.slab;
  const Real *Ai = s.Api.data(), *Aj = s.Apj.data(), *Ak = s.Apk.data(), *Ad = s.Adiag.data();
  int index = g.slab + g.X + 1;
  for (int z = 1; z < g.Z - 1; z++, index += 2 * g.X)
    for (int y = 1; y < g.Y - 1; y++, index += 2)
      for (int x = 1; x < g.X - 1; x++, index++)
        bf[index] = Ad[index] * xf[index] + xf[index - xs] * Ai[index - xs] +
                    xf[index + xs] * Ai[index] + xf[index - ys] * Aj[index - ys] +
                    xf[index + ys] * Aj[index] + xf[index - zs] * Ak[index - zs] +
                    xf[index + zs] * Ak[index];
}

// FLUID_3D_MIC::applyMICPreconditioner, FLUID_3D_MIC.cpp:864-899
void apply_mic(const Grid& g, const Solver& s, Real* zf, const Real* r, Real* q) {
  const int xs = 1, ys = g.X, zs = g.slab;
  const Real *Ai = s.Api.data(), *Aj = s.Apj.data(), *Ak = s.Apk.data(), *P = s.precon.data();
  int index = g.slab + g.X + 1;
  for (int z = 1; z < g.Z - 1; z++, index += 2 * g.X)
    for (int y = 1; y < g.Y - 1; y++, index += 2)
      for (int x = 1; x < g.X - 1; x++, index++) {
        int xm = index - xs, ym = index - ys, zm = index - zs;
        Real t = r[index] - Ai[xm] * P[xm] * q[xm] - Aj[ym] * P[ym] * q[ym] -
                 Ak[zm] * P[zm] * q[zm];
        q[index] = t * P[index];
      }
  index = g.N - (g.slab + g.X + 2);
  for (int z = g.Z - 2; z > 0; z--, index -= 2 * g.X)
    for (int y = g.Y - 2; y > 0; y--, index -= 2)
      for (int x = g.X - 2; x > 0; x--, index--) {
        Real precon = P[index];
        Real t = q[index] - Ai[index] * precon * zf[index + xs] -
                 Aj[index] * precon * zf[index + ys] - Ak[index] * precon * zf[index + zs];
        zf[index] = t * precon;
      }
}

// FLUID_3D_MIC::zeroBoundary, FLUID_3D_MIC.cpp:901-909
void zero_boundary(const Grid& g, Real* x, const uint8_t* skip) {
  for (int i = 0; i < g.N; i++) x[i] = skip[i] ? 0.0 : x[i];
}

// FIELD_3D::dot, FIELD_3D.cpp:6591-6602 (serial, x fastest)
Real dot(const Grid& g, const Real* a, const Real* b) {
  Real f = 0;
  for (int i = 0; i < g.N; i++) f += b[i] * a[i];
  return f;
}

// FIELD_3D::max, FIELD_3D.cpp:1529-1538 (signed maximum)
Real fmax_signed(const Grid& g, const Real* a) {
  Real f = a[0];
  for (int i = 0; i < g.N; i++)
    if (a[i] > f) f = a[i];
  return f;
}

// FLUID_3D_MIC::solvePoisson, FLUID_3D_MIC.cpp:918-1015.  criterion REFERENCE
// is the reference's loop verbatim; REL2 is the same loop with the stop test
// ||r||_2 <= tol ||b||_2 (the reference has no such mode; restated here for
// the 1e-6 configurations).
int solve_poisson(const Grid& g, const plume_params& p, Real* x, const Real* b,
                  const uint8_t* skip, Solver& s, plume_step_stats* st) {
  build_a(g, skip, s);
  build_mic(g, p.mic_tau, p.mic_sigma, s);
  Real* r = s.residual.data();
  Real* d = s.direction.data();
  Real* z = s.z.data();
  Real* q = s.q.data();
  mult_a(g, s, x, r);
  int index = g.slab + g.X + 1;
  for (int zi = 1; zi < g.Z - 1; zi++, index += 2 * g.X)
    for (int yi = 1; yi < g.Y - 1; yi++, index += 2)
      for (int xi = 1; xi < g.X - 1; xi++, index++) r[index] = b[index] - r[index];
  zero_boundary(g, r, skip);
  apply_mic(g, s, z, r, q);
  for (int i = 0; i < g.N; i++) d[i] = z[i];
  Real deltaNew = dot(g, r, z);

  const bool rel2 = (p.criterion == PLUME_CRIT_REL2);
  const Real eps = rel2 ? 0.0 : p.tol;
  const Real bnorm = sqrt(dot(g, b, b));
  Real maxR = 2.0 * eps;
  Real rnorm = sqrt(dot(g, r, r));
  int i = 0;
  bool converged = false;
  if (rel2) converged = (rnorm <= p.tol * bnorm);
  while (i < p.max_iters && (rel2 ? !converged : (maxR > eps))) {
    mult_a(g, s, d, z);
    Real alpha = dot(g, d, z);
    if (fabs(alpha) > 0.0)
      alpha = deltaNew / alpha;
    else
      break;
    for (int k = 0; k < g.N; k++) x[k] += alpha * d[k];
    for (int k = 0; k < g.N; k++) r[k] += (-alpha) * z[k];
    apply_mic(g, s, z, r, q);
    zero_boundary(g, q, skip);
    Real oldMaxR = maxR;
    sca_set_zero_border(g, r);
    maxR = fmax_signed(g, r);
    Real deltaOld = deltaNew;
    deltaNew = dot(g, r, z);
    Real beta = deltaNew / deltaOld;
    for (int k = 0; k < g.N; k++) d[k] *= beta;
    for (int k = 0; k < g.N; k++) d[k] += z[k];
    zero_boundary(g, d, skip);
    i++;
    if (rel2) {
      rnorm = sqrt(dot(g, r, r));
      converged = (rnorm <= p.tol * bnorm);
    } else {
      Real relative = fabs((maxR - oldMaxR) / oldMaxR);
      if (relative < 1e-7) break;
    }
  }
  if (!rel2) {
    rnorm = sqrt(dot(g, r, r));
    converged = !(maxR > eps);
  }
  if (st) {
    st->iterations = i;
    st->converged = converged ? 1 : 0;
    st->max_residual = maxR;
    st->rhs_norm = bnorm;
    st->rel_residual = bnorm > 0 ? rnorm / bnorm : 0.0;
  }
  return i;
}

}  // namespace

// ======================================================================= state
struct orc_handle {
  plume_params p;
  Grid g;
  Real dx, dt, totalTime;
  int totalSteps;
  std::vector<Real> density, densityOld, heat, heatOld, pressure, divergence, cachedPressure,
      cachedDivergence;
  std::vector<Real> velocity, velocityOld, force, vorticity, preprojection, prediffusion,
      preadvection, cachedQuadratic, postadvection, prevorticity;
  // moving box: postIOP and the obstacle matrix N of the last moving step, as
  // the map of SPARSE_MATRIX (row, col) -> value; both empty before it
  std::vector<Real> postIOP;
  std::map<std::pair<int, int>, Real> neumannIOP;
  int iopRows = 0, iopCols = 0;
  std::vector<uint8_t> obst;
  Solver solver;
  explicit orc_handle(const plume_params& pp) : p(pp), g(pp.res) {}

  std::vector<Real>* field(int f, int& comps) {
    comps = 1;
    switch (f) {
      case PLUME_F_DENSITY: return &density;
      case PLUME_F_DENSITY_OLD: return &densityOld;
      case PLUME_F_HEAT: return &heat;
      case PLUME_F_HEAT_OLD: return &heatOld;
      case PLUME_F_PRESSURE: return &pressure;
      case PLUME_F_DIVERGENCE: return &divergence;
      case PLUME_F_CACHED_PRESSURE: return &cachedPressure;
      case PLUME_F_CACHED_DIVERGENCE: return &cachedDivergence;
      default: break;
    }
    comps = 3;
    switch (f) {
      case PLUME_F_VELOCITY: return &velocity;
      case PLUME_F_VELOCITY_OLD: return &velocityOld;
      case PLUME_F_FORCE: return &force;
      case PLUME_F_VORTICITY: return &vorticity;
      case PLUME_F_PREPROJECTION: return &preprojection;
      case PLUME_F_PREDIFFUSION: return &prediffusion;
      case PLUME_F_PREADVECTION: return &preadvection;
      case PLUME_F_CACHED_QUADRATIC: return &cachedQuadratic;
      case PLUME_F_POSTADVECTION: return &postadvection;
      case PLUME_F_PREVORTICITY: return &prevorticity;
      case PLUME_F_POST_IOP: return &postIOP;
      default: return nullptr;
    }
  }
};

namespace {

// FLUID_3D_MIC::addVorticity, FLUID_3D_MIC.cpp:524-590
void add_vorticity(orc_handle& h) {
  const Grid& g = h.g;
  if (h.p.vorticity_eps <= 0.) return;
  const uint8_t* ob = h.obst.data();
  Real* v = h.velocity.data();
  Real* w = h.vorticity.data();
  Real* f = h.force.data();
  const Real dxg = h.dx;
  const Real gridSize = 0.5 / dxg;
  int index = g.slab + g.X + 1;
  for (int z = 1; z < g.Z - 1; z++, index += 2 * g.X)
    for (int y = 1; y < g.Y - 1; y++, index += 2)
      for (int x = 1; x < g.X - 1; x++, index++) {
        int up = ob[index + g.X] || y == g.Y - 2 ? index : index + g.X;
        int down = ob[index - g.X] || y == 1 ? index : index - g.X;
        Real dy = (up == index || down == index) ? 1.0 / dxg : gridSize;
        int out = ob[index + g.slab] || z == g.Z - 2 ? index : index + g.slab;
        int in = ob[index - g.slab] || z == 1 ? index : index - g.slab;
        Real dz = (out == index || in == index) ? 1.0 / dxg : gridSize;
        int right = ob[index + 1] || x == g.X - 2 ? index : index + 1;
        int left = ob[index - 1] || x == 1 ? index : index - 1;
        Real dx = (left == index || right == index) ? 1.0 / dxg : gridSize;
        w[3 * index + 0] = (v[3 * up + 2] - v[3 * down + 2]) * dy + (-v[3 * out + 1] + v[3 * in + 1]) * dz;
        w[3 * index + 1] = (v[3 * out + 0] - v[3 * in + 0]) * dz + (-v[3 * right + 2] + v[3 * left + 2]) * dx;
        w[3 * index + 2] = (v[3 * right + 1] - v[3 * left + 1]) * dx + (-v[3 * up + 0] + v[3 * down + 0]) * dy;
      }
  // VECTOR3_FIELD_3D::magnitudeField, VECTOR3_FIELD_3D.cpp:353-361
  std::vector<Real> mag(g.N);
  for (int i = 0; i < g.N; i++)
    mag[i] = sqrt(w[3 * i] * w[3 * i] + w[3 * i + 1] * w[3 * i + 1] + w[3 * i + 2] * w[3 * i + 2]);
  const Real eps = h.p.vorticity_eps;
  index = g.slab + g.X + 1;
  for (int z = 1; z < g.Z - 1; z++, index += 2 * g.X)
    for (int y = 1; y < g.Y - 1; y++, index += 2)
      for (int x = 1; x < g.X - 1; x++, index++) {
        if (ob[index]) continue;
        Real N[3];
        int up = ob[index + g.X] || y == g.Y - 2 ? index : index + g.X;
        int down = ob[index - g.X] || y == 1 ? index : index - g.X;
        Real dy = (up == index || down == index) ? 1.0 / dxg : gridSize;
        int out = ob[index + g.slab] || z == g.Z - 2 ? index : index + g.slab;
        int in = ob[index - g.slab] || z == 1 ? index : index - g.slab;
        Real dz = (out == index || in == index) ? 1.0 / dxg : gridSize;
        int right = ob[index + 1] || x == g.X - 2 ? index : index + 1;
        int left = ob[index - 1] || x == 1 ? index : index - 1;
        Real dx = (right == index || left == index) ? 1.0 / dxg : gridSize;
        N[0] = (mag[right] - mag[left]) * dx;
        N[1] = (mag[up] - mag[down]) * dy;
        N[2] = (mag[out] - mag[in]) * dz;
        Real magnitude = sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
        if (magnitude > 0.0) {
          magnitude = 1.0 / magnitude;
          N[0] *= magnitude;
          N[1] *= magnitude;
          N[2] *= magnitude;
          f[3 * index + 0] += (N[1] * w[3 * index + 2] - N[2] * w[3 * index + 1]) * dxg * eps;
          f[3 * index + 1] -= (N[0] * w[3 * index + 2] - N[2] * w[3 * index + 0]) * dxg * eps;
          f[3 * index + 2] += (N[0] * w[3 * index + 1] - N[1] * w[3 * index + 0]) * dxg * eps;
        }
      }
}

// VECTOR3_FIELD_3D::axpy, VECTOR3_FIELD_3D.cpp:3113-3120 (v += f * alpha)
void vec_axpy(const Grid& g, Real alpha, Real* v, const Real* f) {
  for (int i = 0; i < 3 * g.N; i++) v[i] += f[i] * alpha;
}

// the per-axis boundary choice shared by advectStam (FLUID_3D_MIC.cpp:600-613,
// 633-646) and project (320-334): open faces copy (mode 1 or 2), walls zero.
void velocity_bcs(orc_handle& h, int copy_mode) {
  vec_face(h.g, h.velocity.data(), 0, h.p.bc[2] == 0 ? copy_mode : 0);
  vec_face(h.g, h.velocity.data(), 1, h.p.bc[4] == 0 ? copy_mode : 0);
  vec_face(h.g, h.velocity.data(), 2, h.p.bc[0] == 0 ? copy_mode : 0);
}

// FLUID_3D_MIC::advectStam, FLUID_3D_MIC.cpp:595-650
void advect_stam(orc_handle& h) {
  const Grid& g = h.g;
  velocity_bcs(h, 1);
  h.preadvection = h.velocity;
  h.velocity.swap(h.velocityOld);
  h.density.swap(h.densityOld);
  h.heat.swap(h.heatOld);
  const Real dt0 = h.dt / h.dx;
  advect(g, dt0, h.velocityOld.data(), h.densityOld.data(), h.density.data(), 1, 0);
  advect(g, dt0, h.velocityOld.data(), h.heatOld.data(), h.heat.data(), 1, 0);
  for (int c = 0; c < 3; c++)
    advect(g, dt0, h.velocityOld.data(), h.velocityOld.data(), h.velocity.data(), 3, c);
  for (int i = 0; i < 3 * g.N; i++) h.cachedQuadratic[i] = h.velocity[i] - h.velocityOld[i];
  h.postadvection = h.velocity;
  vec_set_zero_border(g, h.velocity.data());
  velocity_bcs(h, 1);
  sca_set_zero_border(g, h.density.data());
  sca_set_zero_border(g, h.heat.data());
}

// buildPeeledDampingMatrixFull (FLUID_3D_MIC.cpp:1251-1306) applied through the
// map-ordered sparse product (SPARSE_MATRIX.cpp:83-105): per row the terms are
// summed in increasing column order z-1, y-1, x-1, self, x+1, y+1, z+1, and
// neighbours outside the peeled grid are dropped.
void damping(orc_handle& h) {
  const Grid& g = h.g;
  const Real w = h.p.damping_w;
  const Real wMinus = 1.0 - w;
  const Real sixth = (1. / 6.) * w;
  const int xp = g.X - 2, yp = g.Y - 2, zp = g.Z - 2;
  std::vector<Real> out(3 * (size_t)xp * yp * zp);
  const Real* v = h.velocity.data();
  size_t o = 0;
  for (int z = 0; z < zp; z++)
    for (int y = 0; y < yp; y++)
      for (int x = 0; x < xp; x++) {
        const int c = (x + 1) + (y + 1) * g.X + (z + 1) * g.slab;
        for (int i = 0; i < 3; i++, o++) {
          Real acc = 0.0;
          if (z != 0) acc += v[3 * (c - g.slab) + i] * sixth;
          if (y != 0) acc += v[3 * (c - g.X) + i] * sixth;
          if (x != 0) acc += v[3 * (c - 1) + i] * sixth;
          acc += v[3 * c + i] * wMinus;
          if (x != xp - 1) acc += v[3 * (c + 1) + i] * sixth;
          if (y != yp - 1) acc += v[3 * (c + g.X) + i] * sixth;
          if (z != zp - 1) acc += v[3 * (c + g.slab) + i] * sixth;
          out[o] = acc;
        }
      }
  // VECTOR3_FIELD_3D::setWithPeeled, VECTOR3_FIELD_3D.cpp:3415-3429
  o = 0;
  for (int z = 1; z < g.Z - 1; z++)
    for (int y = 1; y < g.Y - 1; y++)
      for (int x = 1; x < g.X - 1; x++, o++) {
        const int c = x + y * g.X + z * g.slab;
        h.velocity[3 * c] = out[3 * o];
        h.velocity[3 * c + 1] = out[3 * o + 1];
        h.velocity[3 * c + 2] = out[3 * o + 2];
      }
}

// FLUID_3D_MIC::setObstacleBoundaries, FLUID_3D_MIC.cpp:404-485 (both passes)
void set_obstacle_boundaries(orc_handle& h) {
  const Grid& g = h.g;
  uint8_t* ob = h.obst.data();
  for (int z = 1, index = g.slab + g.X + 1; z < g.Z - 1; z++, index += 2 * g.X)
    for (int y = 1; y < g.Y - 1; y++, index += 2)
      for (int x = 1; x < g.X - 1; x++, index++)
        if (ob[index]) {
          int counter = 0;
          if (ob[index + g.X]) counter++;
          if (ob[index - g.X]) counter++;
          if (ob[index - 1]) counter++;
          if (ob[index + 1]) counter++;
          if (ob[index + g.slab]) counter++;
          if (ob[index - g.slab]) counter++;
          if (counter < 3) ob[index] = 0;
        }
  Real* p = h.pressure.data();
  Real* v = h.velocity.data();
  for (int z = 1, index = g.slab + g.X + 1; z < g.Z - 1; z++, index += 2 * g.X)
    for (int y = 1; y < g.Y - 1; y++, index += 2)
      for (int x = 1; x < g.X - 1; x++, index++) {
        if (!ob[index]) continue;
        const int top = ob[index + g.slab], bottom = ob[index - g.slab];
        const int up = ob[index + g.X], down = ob[index - g.X];
        const int left = ob[index - 1], right = ob[index + 1];
        v[3 * index] = v[3 * index + 1] = v[3 * index + 2] = 0.0;
        p[index] = 0.0;
        Real pcnt = 0.;
        if (left && !right) { p[index] += p[index + 1]; pcnt += 1.; }
        if (!left && right) { p[index] += p[index - 1]; pcnt += 1.; }
        if (up && !down) { p[index] += p[index - g.X]; pcnt += 1.; }
        if (!up && down) { p[index] += p[index + g.X]; pcnt += 1.; }
        if (top && !bottom) { p[index] += p[index - g.X]; pcnt += 1.; }
        if (!top && bottom) { p[index] += p[index + g.X]; pcnt += 1.; }
        p[index] /= pcnt;
      }
}

// FLUID_3D_MIC::project, FLUID_3D_MIC.cpp:314-399
void project(orc_handle& h, plume_step_stats* st) {
  const Grid& g = h.g;
  set_obstacle_boundaries(h);
  velocity_bcs(h, 2);
  const uint8_t* ob = h.obst.data();
  const Real* v = h.velocity.data();
  Real* div = h.divergence.data();
  Real* p = h.pressure.data();
  const bool keep_p = (h.p.warm_start == PLUME_WARM_PREVIOUS);
  int index = g.slab + g.X + 1;
  for (int z = 1; z < g.Z - 1; z++, index += 2 * g.X)
    for (int y = 1; y < g.Y - 1; y++, index += 2)
      for (int x = 1; x < g.X - 1; x++, index++) {
        Real xright = v[3 * (index + 1)];
        Real xleft = v[3 * (index - 1)];
        Real yup = v[3 * (index + g.X) + 1];
        Real ydown = v[3 * (index - g.X) + 1];
        Real ztop = v[3 * (index + g.slab) + 2];
        Real zbottom = v[3 * (index - g.slab) + 2];
        if (ob[index + 1]) xright = -v[3 * index];
        if (ob[index - 1]) xleft = -v[3 * index];
        if (ob[index + g.X]) yup = -v[3 * index + 1];
        if (ob[index - g.X]) ydown = -v[3 * index + 1];
        if (ob[index + g.slab]) ztop = -v[3 * index + 2];
        if (ob[index - g.slab]) zbottom = -v[3 * index + 2];
        div[index] = -h.dx * 0.5 * (xright - xleft + yup - ydown + ztop - zbottom);
        if (!keep_p) p[index] = 0.0;
      }
  sca_copy_border_all(g, p);
  h.cachedDivergence = h.divergence;
  solve_poisson(g, h.p, p, div, ob, h.solver, st);
  h.cachedPressure = h.pressure;
  Real* u = h.velocity.data();
  const Real invDx = 1.0 / h.dx;
  index = g.slab + g.X + 1;
  for (int z = 1; z < g.Z - 1; z++, index += 2 * g.X)
    for (int y = 1; y < g.Y - 1; y++, index += 2)
      for (int x = 1; x < g.X - 1; x++, index++) {
        if (x == 1)
          u[3 * index] -= (p[index + 1] - p[index]) * invDx;
        else if (x == g.X - 2)
          u[3 * index] -= (p[index] - p[index - 1]) * invDx;
        else
          u[3 * index] -= 0.5 * (p[index + 1] - p[index - 1]) * invDx;
        if (y == 1)
          u[3 * index + 1] -= (p[index + g.X] - p[index]) * invDx;
        else if (y == g.Y - 2)
          u[3 * index + 1] -= (p[index] - p[index - g.X]) * invDx;
        else
          u[3 * index + 1] -= 0.5 * (p[index + g.X] - p[index - g.X]) * invDx;
        if (z == 1)
          u[3 * index + 2] -= (p[index + g.slab] - p[index]) * invDx;
        else if (z == g.Z - 2)
          u[3 * index + 2] -= (p[index] - p[index - g.slab]) * invDx;
        else
          u[3 * index + 2] -= 0.5 * (p[index + g.slab] - p[index - g.slab]) * invDx;
      }
}

// FLUID_3D_MIC::addSmokeTestCase, FLUID_3D_MIC.cpp:674-700 (float sqrtf and
// float literals as in the reference).
void smoke_column(const Grid& g, Real* field) {
  int maxRes = g.X;
  if (g.Y > maxRes) maxRes = g.Y;
  if (g.Z > maxRes) maxRes = g.Z;
  Real dx = 1.0f / (Real)maxRes;
  Real xTotal = dx * g.X;
  Real zTotal = dx * g.Z;
  Real heighMin = 0.05, heighMax = 0.10;
  for (int z = 0; z < g.Z; z++)
    for (int y = (int)(heighMin * g.Y); y <= (int)(heighMax * g.Y); y++)
      for (int x = 0; x < g.X; x++) {
        Real xLength = x * dx - xTotal * 0.4f;
        Real zLength = z * dx - zTotal * 0.5f;
        Real radius = sqrtf(xLength * xLength + zLength * zLength);
        if (radius < 0.075f * xTotal) field[x + y * g.X + z * g.slab] = 1.0f;
      }
}

}  // namespace

// ======================================================================= C API
extern "C" {

orc_handle* orc_create(const plume_params* p) {
  if (!p || p->res[0] < 3 || p->res[1] < 3 || p->res[2] < 3) return nullptr;
  orc_handle* h = new orc_handle(*p);
  const Grid& g = h->g;
  int maxRes = g.X;
  if (g.Y > maxRes) maxRes = g.Y;
  if (g.Z > maxRes) maxRes = g.Z;
  h->dx = 1.0f / (Real)maxRes;  // FLUID_3D_MIC.cpp:46
  h->dt = p->dt;
  h->totalTime = 0.0;
  h->totalSteps = 0;
  std::vector<Real>* sc[] = {&h->density, &h->densityOld, &h->heat, &h->heatOld, &h->pressure,
                             &h->divergence, &h->cachedPressure, &h->cachedDivergence};
  for (auto* f : sc) f->assign(g.N, 0.0);
  std::vector<Real>* vc[] = {&h->velocity, &h->velocityOld, &h->force, &h->vorticity,
                             &h->preprojection, &h->prediffusion, &h->preadvection,
                             &h->cachedQuadratic, &h->postadvection, &h->prevorticity};
  for (auto* f : vc) f->assign(3 * (size_t)g.N, 0.0);
  build_obstacles(g, p->bc, h->obst);
  h->solver.alloc(g.N);
  return h;
}

void orc_destroy(orc_handle* h) { delete h; }

double orc_source_value(uint64_t seed, int32_t step_index, int64_t cell, double noise) {
  return source_value(seed, step_index, cell, noise);
}

void orc_add_source(orc_handle* h, int32_t step_index) {
  const Grid& g = h->g;
  if (h->p.source == PLUME_SRC_COLUMN) {
    smoke_column(g, h->density.data());
    smoke_column(g, h->heat.data());
  } else if (h->p.source == PLUME_SRC_BOX) {
    for (int z = h->p.box_lo[2]; z < h->p.box_hi[2]; z++)
      for (int y = h->p.box_lo[1]; y < h->p.box_hi[1]; y++)
        for (int x = h->p.box_lo[0]; x < h->p.box_hi[0]; x++) {
          const int64_t c = x + (int64_t)y * g.X + (int64_t)z * g.slab;
          const Real val = source_value(h->p.seed, step_index, c, h->p.source_noise);
          h->density[c] = val;
          h->heat[c] = val;
        }
  }
}

// FLUID_3D_MIC::step, FLUID_3D_MIC.cpp:179-223
void orc_step(orc_handle* h, plume_step_stats* st) {
  const Grid& g = h->g;
  h->dt = h->p.dt;
  std::fill(h->force.begin(), h->force.end(), 0.0);
  vec_set_zero_border(g, h->velocity.data());
  sca_set_zero_border(g, h->density.data());
  // addBuoyancy, FLUID_3D_MIC.cpp:491-502
  const Real beta = h->p.buoyancy;
  if (beta != 0.)
    for (int i = 0; i < g.N; i++) h->force[3 * i + 1] += beta * h->heat[i];
  vec_axpy(g, h->dt, h->velocity.data(), h->force.data());
  std::fill(h->force.begin(), h->force.end(), 0.0);
  h->prevorticity = h->velocity;
  add_vorticity(*h);
  vec_axpy(g, h->dt, h->velocity.data(), h->force.data());
  advect_stam(*h);
  h->prediffusion = h->velocity;
  damping(*h);
  h->preprojection = h->velocity;
  plume_step_stats local{};
  project(*h, st ? st : &local);
  h->totalTime += 0.1;
  h->totalSteps++;
}

// SUBSPACE_FLUID_3D_EIGEN::stepReorderedCubatureStam, lines 243-268, up to the
// projection of the velocity onto the reduced basis
void orc_reduced_prestep(orc_handle* h) {
  const Grid& g = h->g;
  h->dt = 0.1;  // _dt = goalTime (lines 246-250)
  std::fill(h->force.begin(), h->force.end(), 0.0);
  vec_set_zero_border(g, h->velocity.data());
  // addBuoyancy (FLUID_3D_MIC.cpp:491-502) and the axpy
  const Real beta = h->p.buoyancy;
  if (beta != 0.)
    for (int i = 0; i < g.N; i++) h->force[3 * i + 1] += beta * h->heat[i];
  vec_axpy(g, h->dt, h->velocity.data(), h->force.data());
  std::fill(h->force.begin(), h->force.end(), 0.0);
  add_vorticity(*h);
  vec_axpy(g, h->dt, h->velocity.data(), h->force.data());
  // advectHeatAndDensityStam (lines 573-601): the velocity's face conditions,
  // then density and heat advected by the current velocity
  velocity_bcs(*h, 1);
  h->density.swap(h->densityOld);
  h->heat.swap(h->heatOld);
  const Real dt0 = h->dt / h->dx;
  advect(g, dt0, h->velocity.data(), h->densityOld.data(), h->density.data(), 1, 0);
  advect(g, dt0, h->velocity.data(), h->heatOld.data(), h->heat.data(), 1, 0);
  sca_set_zero_border(g, h->density.data());
  sca_set_zero_border(g, h->heat.data());
  h->totalTime += 0.1;
  h->totalSteps++;
}

// ------------------------------------------------------------- moving box
// BOX (src/geometry/BOX.cpp) restated on the plume_box struct.
namespace {
const Real kPi = 3.14159265358979323846;
const Real kAxis[3] = {0.0, 0.0, 1.0};  // BOX.cpp:36

// MATRIX3::rotation (src/linearalgebra/MATRIX3.h:96-117)
void rotation(const Real axis_in[3], Real theta, Real R[9]) {
  Real a[3] = {axis_in[0], axis_in[1], axis_in[2]};
  const Real n = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  const Real inv = 1.0 / n;
  for (int k = 0; k < 3; k++) a[k] *= inv;
  const Real c = cos(theta), s = sin(theta), v = (1.0 - c);
  R[0] = a[0] * a[0] * v + c;
  R[1] = a[0] * a[1] * v - a[2] * s;
  R[2] = a[0] * a[2] * v + a[1] * s;
  R[3] = a[1] * a[0] * v + a[2] * s;
  R[4] = a[1] * a[1] * v + c;
  R[5] = a[1] * a[2] * v - a[0] * s;
  R[6] = a[2] * a[0] * v - a[1] * s;
  R[7] = a[2] * a[1] * v + a[0] * s;
  R[8] = a[2] * a[2] * v + c;
}

// FLUID_3D_MIC::cellCenter (FLUID_3D_MIC.cpp:1704-1733)
void cell_center(const Grid& g, int x, int y, int z, Real p[3]) {
  const Real dx = 1.0 / g.X, dy = 1.0 / g.Y, dz = 1.0 / g.Z;
  p[0] = 0.0;
  p[1] = 0.0;
  p[2] = 0.0;
  p[0] += x * dx;
  p[1] += y * dy;
  p[2] += z * dz;
  p[0] += dx * 0.5;
  p[1] += dy * 0.5;
  p[2] += dz * 0.5;
}

// BOX::inside (BOX.cpp:59-70)
bool box_inside(const plume_box& b, const Real p[3]) {
  Real t[3] = {p[0] - b.center[0], p[1] - b.center[1], p[2] - b.center[2]};
  Real q[3];
  for (int r = 0; r < 3; r++)
    q[r] = b.rotation[3 * r] * t[0] + b.rotation[3 * r + 1] * t[1] + b.rotation[3 * r + 2] * t[2];
  const Real half[3] = {b.lengths[0] * 0.5, b.lengths[1] * 0.5, b.lengths[2] * 0.5};
  return fabs(q[0]) <= half[0] && fabs(q[1]) <= half[1] && fabs(q[2]) <= half[2];
}

// BOX::update_r + update_linearVelocity (BOX.cpp:72-91, BOX.h:65-83, VEC3.h:154-155, 293-296)
void box_velocity(const plume_box& b, const Real p[3], Real v[3]) {
  const Real u[3] = {p[0] - b.center[0], p[1] - b.center[1], p[2] - b.center[2]};
  const Real dot = u[0] * kAxis[0] + u[1] * kAxis[1] + u[2] * kAxis[2];
  const Real n2 = kAxis[0] * kAxis[0] + kAxis[1] * kAxis[1] + kAxis[2] * kAxis[2];
  const Real sc = dot / n2;
  const Real r[3] = {u[0] - kAxis[0] * sc, u[1] - kAxis[1] * sc, u[2] - kAxis[2] * sc};
  const Real w[3] = {0.0, 0.0, 2 * kPi / b.period};
  const Real d[3] = {0.25 * 2 * kPi / b.translation_period * cos(b.phi), 0.0, 0.0};
  const Real c[3] = {w[1] * r[2] - r[1] * w[2], -w[0] * r[2] + r[0] * w[2], w[0] * r[1] - r[0] * w[1]};
  for (int k = 0; k < 3; k++) v[k] = c[k] + d[k];
}

// setPeeledSparseMovingIOP + setVelocityNeumann + N * [u; 1] + setWithPeeled
// (FLUID_3D_MIC.cpp:1645-1701, SPARSE_MATRIX.cpp:83-105, 429-440)
void moving_iop(orc_handle& h, const plume_box& b) {
  const Grid& g = h.g;
  const int peeled = 3 * (g.X - 2) * (g.Y - 2) * (g.Z - 2);
  h.iopRows = peeled;
  h.iopCols = peeled + 1;
  h.neumannIOP.clear();
  for (int k = 0; k < peeled; k++) h.neumannIOP[std::make_pair(k, k)] = 1.0;
  const int last = h.iopCols - 1;
  int index = 0;
  for (int z = 1; z < g.Z - 1; z++)
    for (int y = 1; y < g.Y - 1; y++)
      for (int x = 1; x < g.X - 1; x++)
        for (int i = 0; i < 3; i++, index++) {
          Real p[3];
          cell_center(g, x, y, z, p);
          if (box_inside(b, p)) {
            h.neumannIOP[std::make_pair(index, index)] = 0.0;
            Real v[3];
            box_velocity(b, p, v);
            h.neumannIOP[std::make_pair(index, last)] = v[i];
          }
        }
  std::vector<Real> un(peeled + 1);
  index = 0;
  for (int z = 1; z < g.Z - 1; z++)
    for (int y = 1; y < g.Y - 1; y++)
      for (int x = 1; x < g.X - 1; x++) {
        const int c = x + y * g.X + z * g.slab;
        for (int i = 0; i < 3; i++) un[index++] = h.velocity[3 * c + i];
      }
  un[peeled] = 1.0;
  std::vector<Real> y(peeled, 0.0);
  for (const auto& e : h.neumannIOP) y[e.first.first] += un[e.first.second] * e.second;
  index = 0;
  for (int z = 1; z < g.Z - 1; z++)
    for (int yy = 1; yy < g.Y - 1; yy++)
      for (int x = 1; x < g.X - 1; x++) {
        const int c = x + yy * g.X + z * g.slab;
        for (int i = 0; i < 3; i++) h.velocity[3 * c + i] = y[index++];
      }
}
}  // namespace

void orc_box_init(plume_box* b, const double center[3], const double lengths[3], double period,
                  double translation_period) {
  for (int k = 0; k < 3; k++) {
    b->center[k] = center[k];
    b->original_center[k] = center[k];
    b->lengths[k] = lengths[k];
  }
  for (int k = 0; k < 9; k++) b->rotation[k] = (k == 0 || k == 4 || k == 8) ? 1.0 : 0.0;
  b->theta = 0.0;
  b->phi = 0.0;
  b->period = period;
  b->translation_period = translation_period;
  b->dt = 0.0;
}

// BOX::spin (BOX.cpp:93-101)
void orc_box_spin(plume_box* b) {
  const Real dTheta = 2 * kPi * b->dt / b->period;
  b->theta += dTheta;
  if (b->theta >= 2 * kPi) b->theta = 0.0;
  rotation(kAxis, -1 * b->theta, b->rotation);
}

// BOX::translate_center (BOX.cpp:104-113)
void orc_box_translate(plume_box* b) {
  const Real dPhi = 2 * kPi * b->dt / b->translation_period;
  b->phi += dPhi;
  if (b->phi >= 2 * kPi) b->phi = 0.0;
  const Real disp = 0.25 * sin(b->phi);
  b->center[0] = b->original_center[0] + disp;
}

// FLUID_3D_MIC::stepWithMovingObstacle, FLUID_3D_MIC.cpp:236-310
void orc_step_moving_box(orc_handle* h, const plume_box* box, plume_step_stats* st) {
  const Grid& g = h->g;
  h->dt = h->p.dt;
  std::fill(h->force.begin(), h->force.end(), 0.0);
  vec_set_zero_border(g, h->velocity.data());
  sca_set_zero_border(g, h->density.data());
  vec_axpy(g, h->dt, h->velocity.data(), h->force.data());
  std::fill(h->force.begin(), h->force.end(), 0.0);
  h->prevorticity = h->velocity;
  add_vorticity(*h);
  vec_axpy(g, h->dt, h->velocity.data(), h->force.data());
  advect_stam(*h);
  h->prediffusion = h->velocity;
  damping(*h);
  h->preprojection = h->velocity;
  moving_iop(*h, *box);
  h->postIOP = h->velocity;
  plume_step_stats local{};
  project(*h, st ? st : &local);
  h->totalTime += 0.1;
  h->totalSteps++;
}

// FLUID_3D_MIC::setInitialVelocity(BOX*), FLUID_3D_MIC.cpp:744-764
void orc_set_initial_velocity_box(orc_handle* h, const plume_box* box) {
  const Grid& g = h->g;
  for (int z = 1; z < g.Z - 1; z++)
    for (int y = 1; y < g.Y - 1; y++)
      for (int x = 1; x < g.X - 1; x++) {
        Real p[3];
        cell_center(g, x, y, z, p);
        if (box_inside(*box, p)) {
          Real v[3];
          box_velocity(*box, p, v);
          const int c = x + y * g.X + z * g.slab;
          for (int k = 0; k < 3; k++) h->velocity[3 * c + k] = v[k];
        }
      }
}

int orc_box_inside(const plume_box* b, const double p[3]) { return box_inside(*b, p) ? 1 : 0; }
void orc_box_velocity(const plume_box* b, const double p[3], double v[3]) { box_velocity(*b, p, v); }

// The obstacle matrix as (row, col, value) triples in map order; returns the
// entry count (or -1 before the first moving step).  rows_cols may be NULL;
// the triples are written only when the buffers are given.
int64_t orc_iop_entries(orc_handle* h, int32_t rows_cols[2], int32_t* ij, double* val) {
  if (h->iopRows == 0) return -1;
  if (rows_cols) {
    rows_cols[0] = h->iopRows;
    rows_cols[1] = h->iopCols;
  }
  int64_t k = 0;
  for (const auto& e : h->neumannIOP) {
    if (ij) {
      ij[2 * k] = e.first.first;
      ij[2 * k + 1] = e.first.second;
    }
    if (val) val[k] = e.second;
    k++;
  }
  return k;
}

int orc_get(orc_handle* h, int32_t field, double* dst, size_t n) {
  int comps = 0;
  std::vector<Real>* f = h->field(field, comps);
  if (!f || n != f->size()) return 1;
  memcpy(dst, f->data(), n * sizeof(double));
  return 0;
}

int orc_set(orc_handle* h, int32_t field, const double* src, size_t n) {
  int comps = 0;
  std::vector<Real>* f = h->field(field, comps);
  if (!f || n != f->size()) return 1;
  memcpy(f->data(), src, n * sizeof(double));
  return 0;
}

int orc_get_obstacles(orc_handle* h, uint8_t* dst, size_t n) {
  if (n != h->obst.size()) return 1;
  memcpy(dst, h->obst.data(), n);
  return 0;
}

int32_t orc_total_steps(orc_handle* h) { return h->totalSteps; }

void orc_mic_precon(const int32_t res[3], const int32_t bc[6], double tau, double sigma,
                    double* precon) {
  Grid g(res);
  std::vector<uint8_t> ob;
  build_obstacles(g, bc, ob);
  Solver s;
  s.alloc(g.N);
  build_a(g, ob.data(), s);
  build_mic(g, tau, sigma, s);
  memcpy(precon, s.precon.data(), g.N * sizeof(double));
}

void orc_mic_apply(const int32_t res[3], const int32_t bc[6], const double* precon,
                   const double* r, double* z, double* q) {
  Grid g(res);
  std::vector<uint8_t> ob;
  build_obstacles(g, bc, ob);
  Solver s;
  s.alloc(g.N);
  build_a(g, ob.data(), s);
  memcpy(s.precon.data(), precon, g.N * sizeof(double));
  apply_mic(g, s, z, r, q);
}

void orc_mult_a(const int32_t res[3], const int32_t bc[6], const double* x, double* b) {
  Grid g(res);
  std::vector<uint8_t> ob;
  build_obstacles(g, bc, ob);
  Solver s;
  s.alloc(g.N);
  build_a(g, ob.data(), s);
  mult_a(g, s, x, b);
}

void orc_advect_scalar(const int32_t res[3], double dt0, const double* vel_aos,
                       const double* old_field, double* new_field) {
  Grid g(res);
  advect(g, dt0, vel_aos, old_field, new_field, 1, 0);
}

int32_t orc_solve_poisson(const plume_params* p, double* x, const double* b,
                          plume_step_stats* st) {
  Grid g(p->res);
  std::vector<uint8_t> ob;
  build_obstacles(g, p->bc, ob);
  Solver s;
  s.alloc(g.N);
  return solve_poisson(g, *p, x, b, ob.data(), s, st);
}

}  // extern "C"
