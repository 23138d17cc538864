// tile_kernels.cuh -- the neighbour stencils of the step (vorticity
// confinement, damping, divergence, pressure gradient) as 2.5D tiled kernels.
//
// A block owns a tile of kTX x kTY cells of an xy plane (32 x 8: one warp per
// 128-byte row of FP32 values) and marches it through a chunk of z planes.
// Each thread owns one (x, y) column of the tile: it keeps the values of the
// planes below, at and above its cell in registers (the z neighbours), and
// publishes its current value into a shared-memory tile with a one-cell halo,
// from which it reads its x and y neighbours; only the halo is loaded from
// global memory a second time.  Every plane of every field is read from global
// memory once by its owning thread, in coalesced rows.
//
// Each cell evaluates the reference's expression in the reference's order
// (the FLUID_3D_MIC.cpp lines are cited per kernel), so the FP64 results are
// bit-identical to the reference's serial loops; only where the neighbour
// values come from differs.  Tiles are handed to a plume's blocks
// round-robin through a Blk (common.cuh), so the same bodies serve one plume
// and the batch.
#pragma once
#include "common.cuh"
#include "step_kernels.cuh"

namespace plume {

constexpr int kTX = 32, kTY = 8;
constexpr int kTileThreads = kTX * kTY;
constexpr int kTileZ = 4;  // planes per tile of a single plume's launch (4 beat 2, 8, 16 at 128x192x128)

// The tiles of a grid: ceil(X/32) x ceil(Y/8) x ceil(Z/zc).
struct TileGrid {
  int ntx, nty, nzc, zc;
  __host__ __device__ int count() const { return ntx * nty * nzc; }
};
__host__ __device__ inline TileGrid tile_grid(const Grid& g, int zc) {
  TileGrid t;
  t.zc = zc;
  t.ntx = (g.X + kTX - 1) / kTX;
  t.nty = (g.Y + kTY - 1) / kTY;
  t.nzc = (g.Z + zc - 1) / zc;
  return t;
}

// One field's plane tile with its one-cell halo: [ty + 1][tx + 1] is the
// thread's own cell.  `fill` publishes the centre value (from a register)
// and loads the halo cells (x-halo by the first and last thread of a row,
// y-halo by the first and last row); cells outside the grid are never read
// by a valid cell.
template <typename T>
struct HaloTile {
  T v[kTY + 2][kTX + 2];
};

template <typename T>
__device__ __forceinline__ void tile_fill(HaloTile<T>& t, const T* plane, const Grid& g, int x, int y, int tx,
                                          int ty, T centre, bool hx, bool hy) {
  t.v[ty + 1][tx + 1] = centre;
  if (hx) {
    if (tx == 0 && x > 0 && y < g.Y) t.v[ty + 1][0] = plane[(x - 1) + y * g.X];
    if (tx == kTX - 1 && x + 1 < g.X && y < g.Y) t.v[ty + 1][kTX + 1] = plane[(x + 1) + y * g.X];
  }
  if (hy) {
    if (ty == 0 && y > 0 && x < g.X) t.v[0][tx + 1] = plane[x + (y - 1) * g.X];
    if (ty == kTY - 1 && y + 1 < g.Y && x < g.X) t.v[kTY + 1][tx + 1] = plane[x + (y + 1) * g.X];
  }
}

// Column state of one field: the values at z-1, z and z+1 of the thread's
// (x, y) column (0 outside the grid).
template <typename T>
struct ZCol {
  T m, c, p;
  __device__ __forceinline__ void start(const T* f, const Grid& g, int col, bool in, int z) {
    m = (in && z > 0) ? f[col + (z - 1) * g.slab] : T(0);
    c = in ? f[col + z * g.slab] : T(0);
  }
  // load plane z + 1 (the cell at z is about to be computed)
  __device__ __forceinline__ void ahead(const T* f, const Grid& g, int col, bool in, int z) {
    p = (in && z + 1 < g.Z) ? f[col + (z + 1) * g.slab] : T(0);
  }
  __device__ __forceinline__ void shift() {
    m = c;
    c = p;
  }
};

#define PL_TILE_LOOP(blk_, g, zc)                                               \
  const TileGrid tg_ = tile_grid(g, zc);                                        \
  const int tx = (int)threadIdx.x % kTX, ty = (int)threadIdx.x / kTX;           \
  for (int tile_ = (blk_).id; tile_ < tg_.count(); tile_ += (blk_).n)

// Tile coordinates of tile_: the thread's column and the tile's z range.
#define PL_TILE_COORDS(g)                                                       \
  const int tix_ = tile_ % tg_.ntx, tiy_ = (tile_ / tg_.ntx) % tg_.nty,         \
            tiz_ = tile_ / (tg_.ntx * tg_.nty);                                 \
  const int x = tix_ * kTX + tx, y = tiy_ * kTY + ty;                           \
  const int z0 = tiz_ * tg_.zc, z1 = min(z0 + tg_.zc, (g).Z);                   \
  const bool in = x < (g).X && y < (g).Y;                                       \
  const int col = x + y * (g).X

// ---------------------------------------------------------------- vorticity
// Pass 1 of FLUID_3D_MIC::addVorticity: vorticity = curl(velocity) on the
// interior (lines 530-547) and |vorticity| on every cell
// (VECTOR3_FIELD_3D::magnitudeField, 353-361).  The neighbours are those of
// lines 533-545: one-sided at the first and last interior index of each axis
// (the obstacle test there is true exactly on those cells, since only the wall
// slabs are obstacles).
template <typename T>
__device__ __forceinline__ void vort1_tile_body(Blk blk_, Grid g, V3<T> v, V3<T> w, T* mag, StepConsts<T> c,
                                                int zc) {
  __shared__ HaloTile<T> sx, sy, sz;
  PL_TILE_LOOP(blk_, g, zc) {
    PL_TILE_COORDS(g);
    ZCol<T> vx, vy;
    vx.start(v.x, g, col, in, z0);
    vy.start(v.y, g, col, in, z0);
    for (int z = z0; z < z1; z++) {
      vx.ahead(v.x, g, col, in, z);
      vy.ahead(v.y, g, col, in, z);
      const int i = col + z * g.slab;
      const T vzc = in ? v.z[i] : T(0);
      __syncthreads();  // the previous plane's tiles have been read
      tile_fill(sx, v.x + z * g.slab, g, x, y, tx, ty, vx.c, false, true);
      tile_fill(sy, v.y + z * g.slab, g, x, y, tx, ty, vy.c, true, false);
      tile_fill(sz, v.z + z * g.slab, g, x, y, tx, ty, vzc, true, true);
      __syncthreads();
      if (in) {
        T wx, wy, wz;
        if (!on_border(g, x, y, z)) {
          const bool up_c = y == g.Y - 2, down_c = y == 1, out_c = z == g.Z - 2, in_c = z == 1;
          const bool right_c = x == g.X - 2, left_c = x == 1;
          const bool oy = up_c || down_c, oz = out_c || in_c, ox = right_c || left_c;
          const T dy = oy ? c.oneOverDx : c.gridSize;
          const T dz = oz ? c.oneOverDx : c.gridSize;
          const T dx = ox ? c.oneOverDx : c.gridSize;
          const T z_up = up_c ? vzc : sz.v[ty + 2][tx + 1], z_down = down_c ? vzc : sz.v[ty][tx + 1];
          const T z_right = right_c ? vzc : sz.v[ty + 1][tx + 2], z_left = left_c ? vzc : sz.v[ty + 1][tx];
          const T y_out = out_c ? vy.c : vy.p, y_in = in_c ? vy.c : vy.m;
          const T y_right = right_c ? vy.c : sy.v[ty + 1][tx + 2], y_left = left_c ? vy.c : sy.v[ty + 1][tx];
          const T x_out = out_c ? vx.c : vx.p, x_in = in_c ? vx.c : vx.m;
          const T x_up = up_c ? vx.c : sx.v[ty + 2][tx + 1], x_down = down_c ? vx.c : sx.v[ty][tx + 1];
          wx = (z_up - z_down) * dy + (-y_out + y_in) * dz;
          wy = (x_out - x_in) * dz + (-z_right + z_left) * dx;
          wz = (y_right - y_left) * dx + (-x_up + x_down) * dy;
          w.x[i] = wx;
          w.y[i] = wy;
          w.z[i] = wz;
        } else {
          wx = w.x[i];
          wy = w.y[i];
          wz = w.z[i];
        }
        mag[i] = sqrt_t(wx * wx + wy * wy + wz * wz);
      }
      vx.shift();
      vy.shift();
    }
  }
}

// Pass 2: N = grad|w| / |grad|w||, force = eps*dx*(N x w) on the interior
// (lines 552-589), then velocity += force*dt (line 202).
template <typename T>
__device__ __forceinline__ void vort2_tile_body(Blk blk_, Grid g, V3<T> vel, V3<T> w, const T* mag, V3<T> force,
                                                StepConsts<T> c, int cache, int zc) {
  __shared__ HaloTile<T> sm;
  PL_TILE_LOOP(blk_, g, zc) {
    PL_TILE_COORDS(g);
    ZCol<T> m;
    m.start(mag, g, col, in, z0);
    for (int z = z0; z < z1; z++) {
      m.ahead(mag, g, col, in, z);
      const int i = col + z * g.slab;
      // the cell's own w and velocity, loaded before the barriers so that
      // their latency overlaps the tile exchange
      T wx = T(0), wy = T(0), wz = T(0), ux = T(0), uy = T(0), uz = T(0);
      if (in) {
        wx = w.x[i];
        wy = w.y[i];
        wz = w.z[i];
        ux = vel.x[i];
        uy = vel.y[i];
        uz = vel.z[i];
      }
      __syncthreads();
      tile_fill(sm, mag + z * g.slab, g, x, y, tx, ty, m.c, true, true);
      __syncthreads();
      if (in) {
        T fx = T(0), fy = T(0), fz = T(0);
        bool has_f = false;
        if (!on_border(g, x, y, z)) {
          const bool up_c = y == g.Y - 2, down_c = y == 1, out_c = z == g.Z - 2, in_c = z == 1;
          const bool right_c = x == g.X - 2, left_c = x == 1;
          const T dy = (up_c || down_c) ? c.oneOverDx : c.gridSize;
          const T dz = (out_c || in_c) ? c.oneOverDx : c.gridSize;
          const T dx = (right_c || left_c) ? c.oneOverDx : c.gridSize;
          const T m_right = right_c ? m.c : sm.v[ty + 1][tx + 2], m_left = left_c ? m.c : sm.v[ty + 1][tx];
          const T m_up = up_c ? m.c : sm.v[ty + 2][tx + 1], m_down = down_c ? m.c : sm.v[ty][tx + 1];
          const T m_out = out_c ? m.c : m.p, m_in = in_c ? m.c : m.m;
          T N0 = (m_right - m_left) * dx;
          T N1 = (m_up - m_down) * dy;
          T N2 = (m_out - m_in) * dz;
          T mm = sqrt_t(N0 * N0 + N1 * N1 + N2 * N2);
          if (mm > T(0)) {
            mm = T(1) / mm;
            N0 *= mm;
            N1 *= mm;
            N2 *= mm;
            fx = (N1 * wz - N2 * wy) * c.dx * c.eps;
            fy = -((N0 * wz - N2 * wx) * c.dx * c.eps);
            fz = (N0 * wy - N1 * wx) * c.dx * c.eps;
            has_f = true;
          }
        }
        if (has_f) {
          vel.x[i] = ux + fx * c.dt;
          vel.y[i] = uy + fy * c.dt;
          vel.z[i] = uz + fz * c.dt;
        }
        if (cache) {
          force.x[i] = fx;
          force.y[i] = fy;
          force.z[i] = fz;
        }
      }
      m.shift();
    }
  }
}

// ------------------------------------------------------------------ damping
// The peeled damping product (buildPeeledDampingMatrixFull, FLUID_3D_MIC.cpp:
// 1251-1306, applied through SPARSE_MATRIX operator*, SPARSE_MATRIX.cpp:83-105):
// out = (1-w) v + (w/6) * (existing peeled neighbours), summed in the map's
// column order z-1, y-1, x-1, self, x+1, y+1, z+1.  Border cells pass through.
// Out of place; `preproj` receives a copy of the result when caching.
template <typename T>
__device__ __forceinline__ T damp1_tile(const Grid& g, int x, int y, int z, T zm, T ym, T xm, T ctr, T xp, T yp, T zp,
                                        T wm, T s6) {
  T acc = T(0);
  if (z != 1) acc += zm * s6;
  if (y != 1) acc += ym * s6;
  if (x != 1) acc += xm * s6;
  acc += ctr * wm;
  if (x != g.X - 2) acc += xp * s6;
  if (y != g.Y - 2) acc += yp * s6;
  if (z != g.Z - 2) acc += zp * s6;
  return acc;
}

template <typename T>
__device__ __forceinline__ void damping_tile_body(Blk blk_, Grid g, StepConsts<T> c, V3<T> vin, V3<T> vout,
                                                  V3<T> preproj, int cache, int zc) {
  __shared__ HaloTile<T> s3[3];
  PL_TILE_LOOP(blk_, g, zc) {
    PL_TILE_COORDS(g);
    ZCol<T> a[3];
    const T* f[3] = {vin.x, vin.y, vin.z};
    T* o[3] = {vout.x, vout.y, vout.z};
    T* pp[3] = {preproj.x, preproj.y, preproj.z};
#pragma unroll
    for (int k = 0; k < 3; k++) a[k].start(f[k], g, col, in, z0);
    for (int z = z0; z < z1; z++) {
#pragma unroll
      for (int k = 0; k < 3; k++) a[k].ahead(f[k], g, col, in, z);
      __syncthreads();
#pragma unroll
      for (int k = 0; k < 3; k++) tile_fill(s3[k], f[k] + z * g.slab, g, x, y, tx, ty, a[k].c, true, true);
      __syncthreads();
      if (in) {
        const int i = col + z * g.slab;
        const bool border = on_border(g, x, y, z);
#pragma unroll
        for (int k = 0; k < 3; k++) {
          const HaloTile<T>& t = s3[k];
          const T out = border ? a[k].c
                               : damp1_tile(g, x, y, z, a[k].m, t.v[ty][tx + 1], t.v[ty + 1][tx], a[k].c,
                                            t.v[ty + 1][tx + 2], t.v[ty + 2][tx + 1], a[k].p, c.wMinus, c.sixth);
          o[k][i] = out;
          if (cache) pp[k][i] = out;
        }
      }
#pragma unroll
      for (int k = 0; k < 3; k++) a[k].shift();
    }
  }
}

// --------------------------------------------------------------- projection
// Divergence of FLUID_3D_MIC::project (lines 337-361) with the reflection at
// wall neighbours, and p = 0 on the interior unless the previous pressure is
// kept as the initial guess.
template <typename T>
__device__ __forceinline__ void divergence_tile_body(Blk blk_, Grid g, StepConsts<T> c, V3<T> v, T* div, T* p,
                                                     int keep_p, int zc) {
  __shared__ HaloTile<T> sx, sy;
  PL_TILE_LOOP(blk_, g, zc) {
    PL_TILE_COORDS(g);
    ZCol<T> vz;
    vz.start(v.z, g, col, in, z0);
    for (int z = z0; z < z1; z++) {
      vz.ahead(v.z, g, col, in, z);
      const int i = col + z * g.slab;
      const T vxc = in ? v.x[i] : T(0), vyc = in ? v.y[i] : T(0);
      __syncthreads();
      tile_fill(sx, v.x + z * g.slab, g, x, y, tx, ty, vxc, true, false);
      tile_fill(sy, v.y + z * g.slab, g, x, y, tx, ty, vyc, false, true);
      __syncthreads();
      if (in && !on_border(g, x, y, z)) {
        T xright = sx.v[ty + 1][tx + 2], xleft = sx.v[ty + 1][tx];
        T yup = sy.v[ty + 2][tx + 1], ydown = sy.v[ty][tx + 1];
        T ztop = vz.p, zbottom = vz.m;
        if (wall_xp(g, x)) xright = -vxc;
        if (wall_xm(g, x)) xleft = -vxc;
        if (wall_yp(g, y)) yup = -vyc;
        if (wall_ym(g, y)) ydown = -vyc;
        if (wall_zp(g, z)) ztop = -vz.c;
        if (wall_zm(g, z)) zbottom = -vz.c;
        div[i] = c.divc * (xright - xleft + yup - ydown + ztop - zbottom);
        if (!keep_p) p[i] = T(0);
      }
      vz.shift();
    }
  }
}

// Pressure-gradient subtraction (lines 372-398): central differences,
// one-sided at the first and last interior index of each axis.
template <typename T>
__device__ __forceinline__ void gradient_tile_body(Blk blk_, Grid g, StepConsts<T> c, V3<T> v, const T* p, int zc) {
  __shared__ HaloTile<T> sp;
  PL_TILE_LOOP(blk_, g, zc) {
    PL_TILE_COORDS(g);
    ZCol<T> pc;
    pc.start(p, g, col, in, z0);
    for (int z = z0; z < z1; z++) {
      pc.ahead(p, g, col, in, z);
      const int i = col + z * g.slab;
      const bool inner = in && !on_border(g, x, y, z);
      // the velocity being corrected, loaded before the barriers
      T ux = T(0), uy = T(0), uz = T(0);
      if (inner) {
        ux = v.x[i];
        uy = v.y[i];
        uz = v.z[i];
      }
      __syncthreads();
      tile_fill(sp, p + z * g.slab, g, x, y, tx, ty, pc.c, true, true);
      __syncthreads();
      if (inner) {
        const T inv = c.oneOverDx;
        const T pxp = sp.v[ty + 1][tx + 2], pxm = sp.v[ty + 1][tx];
        const T pyp = sp.v[ty + 2][tx + 1], pym = sp.v[ty][tx + 1];
        T gx, gy, gz;
        if (x == 1)
          gx = (pxp - pc.c) * inv;
        else if (x == g.X - 2)
          gx = (pc.c - pxm) * inv;
        else
          gx = T(0.5) * (pxp - pxm) * inv;
        if (y == 1)
          gy = (pyp - pc.c) * inv;
        else if (y == g.Y - 2)
          gy = (pc.c - pym) * inv;
        else
          gy = T(0.5) * (pyp - pym) * inv;
        if (z == 1)
          gz = (pc.p - pc.c) * inv;
        else if (z == g.Z - 2)
          gz = (pc.c - pc.m) * inv;
        else
          gz = T(0.5) * (pc.p - pc.m) * inv;
        v.x[i] = ux - gx;
        v.y[i] = uy - gy;
        v.z[i] = uz - gz;
      }
      pc.shift();
    }
  }
}

#undef PL_TILE_COORDS
#undef PL_TILE_LOOP

// single-plume launches: one tile per block
template <typename T>
__global__ void __launch_bounds__(kTileThreads) k_vort1_t(Grid g, V3<T> v, V3<T> w, T* mag, StepConsts<T> c) {
  vort1_tile_body<T>(hw_blk(), g, v, w, mag, c, kTileZ);
}
template <typename T>
__global__ void __launch_bounds__(kTileThreads) k_vort2_t(Grid g, V3<T> vel, V3<T> w, const T* mag, V3<T> force,
                                                           StepConsts<T> c, int cache) {
  vort2_tile_body<T>(hw_blk(), g, vel, w, mag, force, c, cache, kTileZ);
}
template <typename T>
__global__ void __launch_bounds__(kTileThreads) k_damping_t(Grid g, StepConsts<T> c, V3<T> vin, V3<T> vout,
                                                             V3<T> preproj, int cache) {
  damping_tile_body<T>(hw_blk(), g, c, vin, vout, preproj, cache, kTileZ);
}
template <typename T>
__global__ void __launch_bounds__(kTileThreads) k_divergence_t(Grid g, StepConsts<T> c, V3<T> v, T* div, T* p,
                                                                int keep_p) {
  divergence_tile_body<T>(hw_blk(), g, c, v, div, p, keep_p, kTileZ);
}
template <typename T>
__global__ void __launch_bounds__(kTileThreads) k_gradient_t(Grid g, StepConsts<T> c, V3<T> v, const T* p) {
  gradient_tile_body<T>(hw_blk(), g, c, v, p, kTileZ);
}

inline int tile_blocks(const Grid& g) { return tile_grid(g, kTileZ).count(); }

}  // namespace plume
