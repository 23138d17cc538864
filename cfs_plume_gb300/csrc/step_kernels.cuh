// step_kernels.cuh -- the non-solver stages of FLUID_3D_MIC::step as CUDA
// kernels, templated on the field type T (double: parity mode, compiled
// without multiply-add contraction so each cell reproduces the reference's
// rounding; float: performance mode).
//
// Storage is SoA: a vector field is three planes x[N], y[N], z[N]; scalars are
// one plane.  Interior obstacles are not supported (the plume path has none:
// obstacles are the wall slabs set from the six BC flags,
// FLUID_3D_MIC.cpp:105-159), so the obstacle tests of the reference reduce to
// index tests on the grid faces.
#pragma once
#include "common.cuh"

namespace plume {

template <typename T>
struct V3 {
  T* x;
  T* y;
  T* z;
};

// Per-step scalar constants, each evaluated in double exactly as the reference
// evaluates it and rounded once to T.
template <typename T>
struct StepConsts {
  T dt;          // _dt
  T beta;        // _buoyancy
  T eps;         // _vorticityEps
  T dx;          // _dx = 1/maxRes
  T gridSize;    // 0.5f/_dx   (FLUID_3D_MIC.cpp:529)
  T oneOverDx;   // 1.0f/_dx   (one-sided vorticity differences, and invDx of project)
  T dt0;         // _dt/_dx    (advectStam, FLUID_3D_MIC.cpp:622)
  T divc;        // -_dx*0.5f  (project, FLUID_3D_MIC.cpp:354)
  T wMinus;      // 1 - w      (damping, FLUID_3D_MIC.cpp:1262)
  T sixth;       // w/6
  T xHi, yHi, zHi;  // res - 2.5: upper advection clamps
  int has_vort;  // eps > 0
  int has_beta;  // beta != 0
};

// ---------------------------------------------------------------- sources
// Box source: density = heat = 1 + noise*(2u-1) on [lo, hi).
template <typename T>
__device__ __forceinline__ void source_box_body(Blk blk_, T* dens, T* heat, Grid g, int x0, int y0, int z0,
                                                int bx, int by, int bz, uint64_t seed, int step,
                                                double noise) {
  const int n = bx * by * bz;
  PL_BLK_STRIDE(i, n, blk_) {
    const int x = x0 + i % bx;
    const int t = i / bx;
    const int y = y0 + t % by;
    const int z = z0 + t / by;
    const int64_t c = x + (int64_t)y * g.X + (int64_t)z * g.slab;
    const T v = (T)source_value(seed, step, c, noise);
    dens[c] = v;
    heat[c] = v;
  }
}
template <typename T>
__global__ void k_source_box(T* dens, T* heat, Grid g, int x0, int y0, int z0, int bx, int by,
                             int bz, uint64_t seed, int step, double noise) {
  source_box_body<T>(hw_blk(), dens, heat, g, x0, y0, z0, bx, by, bz, seed, step, noise);
}

// Box source with host-supplied values (x fastest over the box).
template <typename T>
__global__ void k_source_box_values(T* dens, T* heat, Grid g, int x0, int y0, int z0, int bx,
                                    int by, int bz, const T* vals) {
  const int n = bx * by * bz;
  PL_GRID_STRIDE(i, n) {
    const int x = x0 + i % bx;
    const int t = i / bx;
    const int y = y0 + t % by;
    const int z = z0 + t / by;
    const int64_t c = x + (int64_t)y * g.X + (int64_t)z * g.slab;
    dens[c] = vals[i];
    heat[c] = vals[i];
  }
}

// Column source (FLUID_3D_MIC::addSmokeTestCase): the cell list is computed
// once on the host with the reference's float arithmetic.
template <typename T>
__global__ void k_source_list(T* dens, T* heat, const int* cells, int n) {
  PL_GRID_STRIDE(i, n) {
    const int c = cells[i];
    dens[c] = T(1);
    heat[c] = T(1);
  }
}

// ------------------------------------------------ step start: walls + buoyancy
// FLUID_3D_MIC::step lines 188-199: force.clear, velocity/density
// setZeroBorder, addBuoyancy (force.y = beta*heat), velocity += force*dt,
// prevorticity = velocity.
template <typename T>
__device__ __forceinline__ void forces_body(Blk blk_, Grid g, V3<T> vel, T* dens, const T* heat,
                                            V3<T> prevort, StepConsts<T> c, int cache) {
  PL_BLK_STRIDE(i, g.N, blk_) {
    const int x = i % g.X;
    const int t = i / g.X;
    const int y = t % g.Y;
    const int z = t / g.Y;
    T vx = vel.x[i], vy = vel.y[i], vz = vel.z[i];
    if (on_border(g, x, y, z)) {
      vx = vy = vz = T(0);
      if (dens) dens[i] = T(0);  // null: the reduced step leaves density alone
    }
    if (c.has_beta) {
      const T fy = c.beta * heat[i];
      vy = vy + fy * c.dt;
    }
    vel.x[i] = vx;
    vel.y[i] = vy;
    vel.z[i] = vz;
    if (cache) {
      prevort.x[i] = vx;
      prevort.y[i] = vy;
      prevort.z[i] = vz;
    }
  }
}
template <typename T>
__global__ void k_forces(Grid g, V3<T> vel, T* dens, const T* heat, V3<T> prevort,
                         StepConsts<T> c, int cache) {
  forces_body<T>(hw_blk(), g, vel, dens, heat, prevort, c, cache);
}

// ----------------------------------------------------------- face conditions
// One component per pair of faces: mode 0 zero (setZeroX/Y/Z), 1 copy from one
// cell in (copyBorderX/Y/Z), 2 copy from two cells in (setNeumannX/Y/Z)
// (VECTOR3_FIELD_3D.cpp:2872-3053).  Each face writes only its own axis's
// component and reads that component from a cell no face of the same axis
// writes, so all six faces run in one launch.  Threads enumerate the cells of
// the x faces, then the y faces, then the z faces.
template <typename T>
__device__ __forceinline__ void face_bc_body(Blk blk_, Grid g, V3<T> v, int mode_x, int mode_y, int mode_z) {
  const int nxf = 2 * g.Y * g.Z, nyf = 2 * g.X * g.Z, nzf = 2 * g.X * g.Y;
  PL_BLK_STRIDE(i, nxf + nyf + nzf, blk_) {
    if (i < nxf) {
      const int side = i & 1, r = i >> 1;
      const int y = r % g.Y, z = r / g.Y;
      const int x = side ? g.X - 1 : 0;
      const int c = x + y * g.X + z * g.slab;
      const int m = mode_x;
      v.x[c] = (m == 0) ? T(0) : v.x[side ? c - m : c + m];
    } else if (i < nxf + nyf) {
      const int j = i - nxf;
      const int side = j & 1, r = j >> 1;
      const int x = r % g.X, z = r / g.X;
      const int y = side ? g.Y - 1 : 0;
      const int c = x + y * g.X + z * g.slab;
      const int m = mode_y * g.X;
      v.y[c] = (mode_y == 0) ? T(0) : v.y[side ? c - m : c + m];
    } else {
      const int j = i - nxf - nyf;
      const int side = j & 1, r = j >> 1;
      const int x = r % g.X, y = r / g.X;
      const int z = side ? g.Z - 1 : 0;
      const int c = x + y * g.X + z * g.slab;
      const int m = mode_z * g.slab;
      v.z[c] = (mode_z == 0) ? T(0) : v.z[side ? c - m : c + m];
    }
  }
}
template <typename T>
__global__ void k_face_bc(Grid g, V3<T> v, int mode_x, int mode_y, int mode_z) {
  face_bc_body<T>(hw_blk(), g, v, mode_x, mode_y, mode_z);
}

// ---------------------------------------------------------------- advection
// First-order semi-Lagrangian lookup of VECTOR3_FIELD_3D::advect
// (VECTOR3_FIELD_3D.cpp:2001-2158): backtrace in index space by dt0*u, clamp
// to [1.5, res-2.5], trilinear weights, evaluated in the reference's order.
template <typename T>
struct Trilinear {
  int i000, i010, i100, i110, i001, i011, i101, i111;
  T s0, s1, t0, t1, u0, u1;
  __device__ inline T apply(const T* f) const {
    return u0 * (s0 * (t0 * f[i000] + t1 * f[i010]) + s1 * (t0 * f[i100] + t1 * f[i110])) +
           u1 * (s0 * (t0 * f[i001] + t1 * f[i011]) + s1 * (t0 * f[i101] + t1 * f[i111]));
  }
};

template <typename T>
__device__ inline Trilinear<T> backtrace(const Grid& g, const StepConsts<T>& c, V3<T> vo, int i,
                                         int x, int y, int z) {
  T xt = T(x) - c.dt0 * vo.x[i];
  T yt = T(y) - c.dt0 * vo.y[i];
  T zt = T(z) - c.dt0 * vo.z[i];
  xt = (xt < T(1.5)) ? T(1.5) : xt;
  xt = (xt > c.xHi) ? c.xHi : xt;
  yt = (yt < T(1.5)) ? T(1.5) : yt;
  yt = (yt > c.yHi) ? c.yHi : yt;
  zt = (zt < T(1.5)) ? T(1.5) : zt;
  zt = (zt > c.zHi) ? c.zHi : zt;
  const int x0 = (int)xt, y0 = (int)yt, z0 = (int)zt;
  const int x1 = x0 + 1, y1 = y0 + 1, z1 = z0 + 1;
  Trilinear<T> w;
  w.s1 = xt - T(x0);
  w.s0 = T(1) - w.s1;
  w.t1 = yt - T(y0);
  w.t0 = T(1) - w.t1;
  w.u1 = zt - T(z0);
  w.u0 = T(1) - w.u1;
  w.i000 = x0 + y0 * g.X + z0 * g.slab;
  w.i010 = x0 + y1 * g.X + z0 * g.slab;
  w.i100 = x1 + y0 * g.X + z0 * g.slab;
  w.i110 = x1 + y1 * g.X + z0 * g.slab;
  w.i001 = x0 + y0 * g.X + z1 * g.slab;
  w.i011 = x0 + y1 * g.X + z1 * g.slab;
  w.i101 = x1 + y0 * g.X + z1 * g.slab;
  w.i111 = x1 + y1 * g.X + z1 * g.slab;
  return w;
}

// advectStam after its first boundary pass (FLUID_3D_MIC.cpp:621-649): all
// three fields advected with one backtrace per cell, then the border fix-up
// (velocity.setZeroBorder, copyBorder on the open axes, density/heat
// setZeroBorder) folded in: a border cell's final value along an open axis is
// its interior neighbour's new value, which the border thread recomputes.
// postadvection (the pre-fix-up velocity) is written when `cache` is set.
template <typename T>
__device__ __forceinline__ void advect_body(Blk blk_, Grid g, StepConsts<T> c, V3<T> vo, const T* dens_o,
                                            const T* heat_o, V3<T> vn, T* dens_n, T* heat_n, V3<T> postadv,
                                            int cache, int open_x, int open_y, int open_z, int vel_out) {
  PL_BLK_STRIDE(i, g.N, blk_) {
    const int x = i % g.X;
    const int t = i / g.X;
    const int y = t % g.Y;
    const int z = t / g.Y;
    const Trilinear<T> w = backtrace(g, c, vo, i, x, y, z);
    if (!vel_out) {  // advectHeatAndDensityStam: the scalars alone
      const bool b = on_border(g, x, y, z);
      dens_n[i] = b ? T(0) : w.apply(dens_o);
      heat_n[i] = b ? T(0) : w.apply(heat_o);
      continue;
    }
    const T ux = w.apply(vo.x), uy = w.apply(vo.y), uz = w.apply(vo.z);
    if (cache) {
      postadv.x[i] = ux;
      postadv.y[i] = uy;
      postadv.z[i] = uz;
    }
    if (!on_border(g, x, y, z)) {
      dens_n[i] = w.apply(dens_o);
      heat_n[i] = w.apply(heat_o);
      vn.x[i] = ux;
      vn.y[i] = uy;
      vn.z[i] = uz;
    } else {
      dens_n[i] = T(0);
      heat_n[i] = T(0);
      const bool yin = (y >= 1 && y <= g.Y - 2), zin = (z >= 1 && z <= g.Z - 2),
                 xin = (x >= 1 && x <= g.X - 2);
      T bx = T(0), by = T(0), bz = T(0);
      if (open_x && (x == 0 || x == g.X - 1) && yin && zin) {
        const int nx = (x == 0) ? 1 : g.X - 2;
        const int n = nx + y * g.X + z * g.slab;
        bx = backtrace(g, c, vo, n, nx, y, z).apply(vo.x);
      }
      if (open_y && (y == 0 || y == g.Y - 1) && xin && zin) {
        const int ny = (y == 0) ? 1 : g.Y - 2;
        const int n = x + ny * g.X + z * g.slab;
        by = backtrace(g, c, vo, n, x, ny, z).apply(vo.y);
      }
      if (open_z && (z == 0 || z == g.Z - 1) && xin && yin) {
        const int nz = (z == 0) ? 1 : g.Z - 2;
        const int n = x + y * g.X + nz * g.slab;
        bz = backtrace(g, c, vo, n, x, y, nz).apply(vo.z);
      }
      vn.x[i] = bx;
      vn.y[i] = by;
      vn.z[i] = bz;
    }
  }
}
template <typename T>
__global__ void k_advect(Grid g, StepConsts<T> c, V3<T> vo, const T* dens_o, const T* heat_o,
                         V3<T> vn, T* dens_n, T* heat_n, V3<T> postadv, int cache,
                         int open_x, int open_y, int open_z, int vel_out = 1) {
  advect_body<T>(hw_blk(), g, c, vo, dens_o, heat_o, vn, dens_n, heat_n, postadv, cache, open_x, open_y, open_z, vel_out);
}

// --------------------------------------------------------------- projection
// FIELD_3D::copyBorderAll (FIELD_3D.cpp:1382-1420): z faces, then y faces, then
// x faces.  Composed, every border cell takes the value of the cell with each
// coordinate clamped into the interior.
template <typename T>
__device__ __forceinline__ void copy_border_all_body(Blk blk_, Grid g, T* p) {
  const int nxf = 2 * g.Y * g.Z, nyf = 2 * g.X * g.Z, nzf = 2 * g.X * g.Y;
  PL_BLK_STRIDE(i, nxf + nyf + nzf, blk_) {
    int x, y, z;
    if (i < nxf) {
      const int r = i >> 1;
      x = (i & 1) ? g.X - 1 : 0;
      y = r % g.Y;
      z = r / g.Y;
    } else if (i < nxf + nyf) {
      const int j = i - nxf, r = j >> 1;
      y = (j & 1) ? g.Y - 1 : 0;
      x = r % g.X;
      z = r / g.X;
    } else {
      const int j = i - nxf - nyf, r = j >> 1;
      z = (j & 1) ? g.Z - 1 : 0;
      x = r % g.X;
      y = r / g.X;
    }
    const int cx = x < 1 ? 1 : (x > g.X - 2 ? g.X - 2 : x);
    const int cy = y < 1 ? 1 : (y > g.Y - 2 ? g.Y - 2 : y);
    const int cz = z < 1 ? 1 : (z > g.Z - 2 ? g.Z - 2 : z);
    p[x + y * g.X + z * g.slab] = p[cx + cy * g.X + cz * g.slab];
  }
}
template <typename T>
__global__ void k_copy_border_all(Grid g, T* p) {
  copy_border_all_body<T>(hw_blk(), g, p);
}

// ------------------------------------------------------------ moving box
// The box of FLUID_3D_MIC::stepWithMovingObstacle as the stomp kernel sees
// it: every constant is computed once per step on the host (box.cpp).  Cells
// outside [lo, hi) are certainly outside the box (a bound with a margin of
// two cells around its circumscribed sphere), so only the cells near the box
// run the FP64 geometry.
struct BoxDev {
  double center[3], half[3], R[9], axis[3], omega[3], disp[3];
  double d[3];  // cell size per axis, 1 / res (FLUID_3D_MIC::cellCenter)
  int lo[3], hi[3];
  // FP32 copies for the pre-test that sends clearly-outside cells past the
  // FP64 geometry (FP64 issues at a small fraction of the FP32 rate here)
  float fc[3], fh[3], fR[9], fd[3], ftol;
};

// Inside test and rigid velocity of interior cell (x, y, z), in FP64 with
// every operation rounded separately in the reference's order (the explicit
// _rn intrinsics keep the compiler from contracting them into FMAs in the
// FP32 engine too):
//   cellCenter          FLUID_3D_MIC.cpp:1717-1730
//   BOX::inside         BOX.cpp:59-70        |R (p - c)| <= half, per axis
//   BOX::update_r       BOX.cpp:72-81        r = u - axis (u.axis / |axis|^2)
//   update_linearVelocity BOX.h:78-83, VEC3.h:154-155   v = w x r + disp
__device__ inline bool box_cell(const BoxDev& b, int x, int y, int z, double v[3]) {
  if (x < b.lo[0] || x >= b.hi[0] || y < b.lo[1] || y >= b.hi[1] || z < b.lo[2] ||
      z >= b.hi[2])
    return false;
  const int xyz[3] = {x, y, z};
  {
    // |q| in FP32 beyond half + tol means outside: tol bounds the FP32
    // rounding of the centre, offset and R q many times over
    float uf[3], amax = 0.f;
    for (int k = 0; k < 3; k++) {
      uf[k] = ((float)xyz[k] + 0.5f) * b.fd[k] - b.fc[k];
      amax += fabsf(uf[k]);
    }
    const float tol = b.ftol * (1.0f + amax);
    for (int k = 0; k < 3; k++) {
      const float q = b.fR[3 * k] * uf[0] + b.fR[3 * k + 1] * uf[1] + b.fR[3 * k + 2] * uf[2];
      if (fabsf(q) > b.fh[k] * 1.000001f + tol) return false;
    }
  }
  double u[3];
  for (int k = 0; k < 3; k++) {
    double p = __dadd_rn(0.0, __dmul_rn((double)xyz[k], b.d[k]));
    p = __dadd_rn(p, __dmul_rn(b.d[k], 0.5));
    u[k] = __dsub_rn(p, b.center[k]);
  }
  for (int k = 0; k < 3; k++) {
    const double q = __dadd_rn(__dadd_rn(__dmul_rn(b.R[3 * k], u[0]), __dmul_rn(b.R[3 * k + 1], u[1])),
                               __dmul_rn(b.R[3 * k + 2], u[2]));
    if (!(fabs(q) <= b.half[k])) return false;
  }
  const double* a = b.axis;
  const double s = __ddiv_rn(
      __dadd_rn(__dadd_rn(__dmul_rn(u[0], a[0]), __dmul_rn(u[1], a[1])), __dmul_rn(u[2], a[2])),
      __dadd_rn(__dadd_rn(__dmul_rn(a[0], a[0]), __dmul_rn(a[1], a[1])), __dmul_rn(a[2], a[2])));
  double r[3];
  for (int k = 0; k < 3; k++) r[k] = __dsub_rn(u[k], __dmul_rn(a[k], s));
  const double* w = b.omega;
  v[0] = __dadd_rn(__dsub_rn(__dmul_rn(w[1], r[2]), __dmul_rn(r[1], w[2])), b.disp[0]);
  v[1] = __dadd_rn(__dadd_rn(__dmul_rn(-w[0], r[2]), __dmul_rn(r[0], w[2])), b.disp[1]);
  v[2] = __dadd_rn(__dsub_rn(__dmul_rn(w[0], r[1]), __dmul_rn(r[0], w[1])), b.disp[2]);
  return true;
}

// -0 by its bit pattern (std::signbit would widen a float to double first,
// an FP64-pipe conversion per value)
__device__ inline bool is_neg_zero(float v) { return __float_as_uint(v) == 0x80000000u; }
__device__ inline bool is_neg_zero(double v) {
  return (unsigned long long)__double_as_longlong(v) == 0x8000000000000000ull;
}

// The obstacle stomp u <- N [u; 1] over the interior (setPeeledSparseMovingIOP,
// setVelocityNeumann and the sparse product, FLUID_3D_MIC.cpp:1645-1701 and
// SPARSE_MATRIX.cpp:83-105).  Row i of N holds (i, i) = 1 outside the box,
// 0 inside, and (i, last) = the box velocity inside; the product accumulates
// y_i = 0 + u_i N(i,i), then + 1 N(i,last), in that order, which these
// kernels repeat (so a -0 outside the box becomes +0 as in the reference).
// Two passes on one stream:
//   k_box_post   every cell, no FP64: outside-box value 0 + u*1 (u itself but
//                for -0 -> +0, exact in T, stored only when it changes),
//                postIOP = that field (border cells copied), inside[] = 0;
//   k_box_stomp  the box's bounding cells [lo, hi) only: the FP64 inside test
//                and, inside, u = (0 + u*0) + 1*v_box, postIOP, inside[] = 1
//                and the last-column values.
// Keeping the FP64 geometry in its own launch over the bounding cells stops
// it from running (hoisted by the compiler) for every cell of the grid.
template <typename T>
__global__ void k_box_post(Grid g, V3<T> vel, V3<T> post, int cache, uint8_t* inside) {
  PL_GRID_STRIDE(i, g.N) {
    const int x = i % g.X;
    const int t = i / g.X;
    const int y = t % g.Y;
    const int z = t / g.Y;
    T* comp[3] = {vel.x, vel.y, vel.z};
    T* pc[3] = {post.x, post.y, post.z};
    const bool border = on_border(g, x, y, z);
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const T u = comp[c][i];
      T o = u;
      if (!border) {
        o = T(0) + u * T(1);
        if (is_neg_zero(u)) comp[c][i] = o;
      }
      if (cache) pc[c][i] = o;
    }
    if (!border) inside[i] = 0;
  }
}

// mode 0: the stomp of the cells inside the box (after k_box_post);
// mode 1: setInitialVelocity(BOX*) (FLUID_3D_MIC.cpp:744-764): u = box
//         velocity inside, other cells untouched.
template <typename T>
__global__ void k_box_stomp(Grid g, BoxDev b, V3<T> vel, V3<T> post, int cache, uint8_t* inside,
                            double* vals, int mode) {
  const int nx = b.hi[0] - b.lo[0], ny = b.hi[1] - b.lo[1];
  const int n = nx * ny * (b.hi[2] - b.lo[2]);
  PL_GRID_STRIDE(k, n) {
    const int x = b.lo[0] + k % nx;
    const int t = k / nx;
    const int y = b.lo[1] + t % ny;
    const int z = b.lo[2] + t / ny;
    double bv[3];
    if (!box_cell(b, x, y, z, bv)) continue;
    const int i = x + y * g.X + z * g.slab;
    if (mode == 1) {
      vel.x[i] = (T)bv[0];
      vel.y[i] = (T)bv[1];
      vel.z[i] = (T)bv[2];
      continue;
    }
    T* comp[3] = {vel.x, vel.y, vel.z};
    T out[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const double y0 = __dadd_rn(0.0, __dmul_rn((double)comp[c][i], 0.0));
      out[c] = (T)__dadd_rn(y0, __dmul_rn(bv[c], 1.0));
    }
    vel.x[i] = out[0];
    vel.y[i] = out[1];
    vel.z[i] = out[2];
    if (cache) {
      post.x[i] = out[0];
      post.y[i] = out[1];
      post.z[i] = out[2];
    }
    inside[i] = 1;
    vals[3 * (size_t)i] = bv[0];
    vals[3 * (size_t)i + 1] = bv[1];
    vals[3 * (size_t)i + 2] = bv[2];
  }
}

}  // namespace plume
