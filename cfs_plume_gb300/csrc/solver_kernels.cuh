// solver_kernels.cuh -- MIC(0)-preconditioned CG of FLUID_3D_MIC::solvePoisson
// (FLUID_3D_MIC.cpp:918-1015) as device kernels.
//
// The Poisson matrix of the plume (heat = false, FLUID_3D_MIC.cpp:772-801) has
// off-diagonal entries -1 (fluid neighbour) or 0 (wall neighbour) and a
// diagonal equal to the number of non-wall neighbours, so the kernels derive
// every coefficient from the cell's position and the wall flags instead of
// reading the reference's four coefficient fields.
//
// CG scalars live in device memory (CgState) and are computed by the last
// block of each reduction kernel from per-block partials summed in a fixed
// order, so a solve is deterministic and needs no host round trip per
// iteration.  Every iteration kernel returns at entry once `done` is set.
#pragma once
#include "common.cuh"

namespace plume {

struct CgState {
  double deltaNew, deltaOld, alpha, beta;
  double maxR, oldMaxR;  // signed max of r (reference criterion)
  double rr, bb;         // r.r and b.b
  double dq;             // d.(A d)
  double tol;            // absolute (reference) or relative (rel2) tolerance
  double guess_scale, guess_scale2;  // Galerkin factors of the last learned guess
  double guess_mean, guess_mean2;    // interior means removed (closed boxes)
  int iter, max_iters, criterion, done;
  int converged, broke, wave_err, bodies;  // bodies: CG-graph loop bodies run this solve
  unsigned int ticket[4];
};

constexpr int kRedThreads = 256;
constexpr int kRedBlocks = 912;  // 6 x 152 SMs: every reduction kernel keeps 6 blocks of 8 warps resident

// Off-diagonal coefficient toward a neighbour: -1 unless the neighbour is a wall.
template <typename T>
__device__ inline T coef(bool wall) {
  return wall ? T(0) : T(-1);
}

// Diagonal: number of non-wall neighbours (buildA, FLUID_3D_MIC.cpp:784-791).
template <typename T>
__device__ inline T adiag(const Grid& g, int x, int y, int z) {
  T a = T(0);
  if (!wall_xp(g, x)) a += T(1);
  if (!wall_xm(g, x)) a += T(1);
  if (!wall_yp(g, y)) a += T(1);
  if (!wall_ym(g, y)) a += T(1);
  if (!wall_zp(g, z)) a += T(1);
  if (!wall_zm(g, z)) a += T(1);
  return a;
}

// multA (FLUID_3D_MIC.cpp:811-822) at one interior cell, in the reference order.
template <typename T>
__device__ inline T mult_a_cell(const Grid& g, const T* xf, int i, int x, int y, int z) {
  return adiag<T>(g, x, y, z) * xf[i] + xf[i - 1] * coef<T>(wall_xm(g, x)) +
         xf[i + 1] * coef<T>(wall_xp(g, x)) + xf[i - g.X] * coef<T>(wall_ym(g, y)) +
         xf[i + g.X] * coef<T>(wall_yp(g, y)) + xf[i - g.slab] * coef<T>(wall_zm(g, z)) +
         xf[i + g.slab] * coef<T>(wall_zp(g, z));
}

// ------------------------------------------------- last-block reductions
// True in the last of `nblk` blocks to arrive (the blocks sharing one
// plume's reduction: the whole grid for a single-plume launch).
__device__ inline bool arrive_last(unsigned int* ticket, int nblk) {
  __shared__ bool last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned int t = atomicAdd(ticket, 1u);
    last = (t == (unsigned)nblk - 1u);
  }
  __syncthreads();
  if (last) __threadfence();
  return last;
}
__device__ inline bool arrive_last(unsigned int* ticket) { return arrive_last(ticket, (int)gridDim.x); }

// Sum the first `nblk` partials in a fixed order (valid in thread 0).
__device__ inline double sum_partials(const double* part, double* sh, int nblk) {
  double s = 0.0;
  for (int k = threadIdx.x; k < nblk; k += blockDim.x) s += __ldcg(part + k);
  return block_sum(s, sh);
}
__device__ inline double sum_partials(const double* part, double* sh) {
  return sum_partials(part, sh, (int)gridDim.x);
}
__device__ inline double max_partials(const double* part, double* sh, int nblk) {
  double s = -1.0e308;
  for (int k = threadIdx.x; k < nblk; k += blockDim.x) {
    const double v = __ldcg(part + k);
    s = v > s ? v : s;
  }
  return block_max(s, sh, -1.0e308);
}
__device__ inline double max_partials(const double* part, double* sh) {
  return max_partials(part, sh, (int)gridDim.x);
}

// ------------------------------------------------- initial guess from two
// candidate vectors u (the previous step's pressure) and v (the network's
// guess): x0 = a (u - mu) + b (v - mv) with (a, b) the A-norm Galerkin
// projection of the solution onto their span, i.e. the 2x2 system
//   [u.Au u.Av; u.Av v.Av] [a; b] = [u.b; v.b]
// (a single-vector projection when the pair is degenerate, 0 when neither
// helps).  The result is never further from the solution than x = 0, u or v
// alone in the A-norm, the norm CG's error bound starts from.  With all six
// walls closed the constant vector is A's null space: the A-norm does not see
// it, but a large constant offset in an FP32 guess sets a rounding floor under
// the residual, so each candidate's interior mean (mu, mv) is removed first.
// u and v must be 0 on the border.  Grid: kRedBlocks blocks; part holds
// 8 * gridDim.x doubles; st->ticket[3] is left at 0.
template <typename T>
__global__ void k_guess_dots(Grid g, const T* u, const T* v, const T* b, CgState* st, double* part) {
  __shared__ double sh[32];
  double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // ub vb uAu vAv uAv su sv sb
  PL_GRID_STRIDE(k, g.nint) {
    int cx, cy, cz;
    const int i = interior_cell(g, k, cx, cy, cz);
    const double ui = (double)u[i], vi = (double)v[i], bi = (double)b[i];
    const double au = (double)mult_a_cell(g, u, i, cx, cy, cz);
    const double av = (double)mult_a_cell(g, v, i, cx, cy, cz);
    acc[0] += ui * bi;
    acc[1] += vi * bi;
    acc[2] += ui * au;
    acc[3] += vi * av;
    acc[4] += ui * av;
    acc[5] += ui;
    acc[6] += vi;
    acc[7] += bi;
  }
  for (int q = 0; q < 8; q++) {
    const double t = block_sum(acc[q], sh);
    if (threadIdx.x == 0) part[q * gridDim.x + blockIdx.x] = t;
  }
  if (arrive_last(&st->ticket[3])) {
    double tot[8];
    for (int q = 0; q < 8; q++) tot[q] = sum_partials(part + q * gridDim.x, sh);
    if (threadIdx.x == 0) {
      const bool closed = g.wall[0] && g.wall[1] && g.wall[2] && g.wall[3] && g.wall[4] && g.wall[5];
      const double n = (double)g.nint;
      const double mu = closed ? tot[5] / n : 0.0, mv = closed ? tot[6] / n : 0.0;
      // with the means removed: (u - mu).b = u.b - mu sum(b); A 1 = 0 leaves the A-products
      const double ub = tot[0] - mu * tot[7], vb = tot[1] - mv * tot[7];
      const double uu = tot[2], vv = tot[3], uv = tot[4];
      double a = 0.0, c = 0.0;
      const double det = uu * vv - uv * uv;
      if (uu > 0.0 && vv > 0.0 && det > 1e-10 * uu * vv) {
        a = (ub * vv - vb * uv) / det;
        c = (uu * vb - uv * ub) / det;
      } else {  // degenerate pair: the better single candidate (gain g^2 / a)
        const double gu = uu > 0.0 ? ub * ub / uu : 0.0, gv = vv > 0.0 ? vb * vb / vv : 0.0;
        if (gu >= gv && gu > 0.0) a = ub / uu;
        else if (gv > 0.0) c = vb / vv;
      }
      const bool ok = isfinite(a) && isfinite(c) && isfinite(mu) && isfinite(mv);
      st->guess_scale = ok ? a : 0.0;
      st->guess_scale2 = ok ? c : 0.0;
      st->guess_mean = ok ? mu : 0.0;
      st->guess_mean2 = ok ? mv : 0.0;
      st->ticket[3] = 0;
    }
  }
}

// x = base + a (u - mu) + b (v - mv) on the interior (base may be null; x may
// alias base or u); terms with a zero coefficient are dropped, so a
// non-finite candidate never survives
template <typename T>
__global__ void k_guess_apply(Grid g, const T* base, const T* u, const T* v, const CgState* st, T* x) {
  const double a = st->guess_scale, c = st->guess_scale2, mu = st->guess_mean, mv = st->guess_mean2;
  PL_GRID_STRIDE(k, g.nint) {
    int cx, cy, cz;
    const int i = interior_cell(g, k, cx, cy, cz);
    double r = base ? (double)base[i] : 0.0;
    if (a != 0.0) r += a * ((double)u[i] - mu);
    if (c != 0.0) r += c * ((double)v[i] - mv);
    x[i] = (T)r;
  }
}

// r = b - A x on interior cells (FP64 accumulation), 0 on the border
template <typename T>
__global__ void k_residual(Grid g, const T* b, const T* x, T* r) {
  PL_GRID_STRIDE(i, g.N) {
    const int cx = i % g.X, cy = (i / g.X) % g.Y, cz = i / g.slab;
    const bool in = cx > 0 && cy > 0 && cz > 0 && cx < g.X - 1 && cy < g.Y - 1 && cz < g.Z - 1;
    double v = 0.0;
    if (in) {
      const double ax = (double)adiag<T>(g, cx, cy, cz) * (double)x[i] +
                        (double)x[i - 1] * (double)coef<T>(wall_xm(g, cx)) +
                        (double)x[i + 1] * (double)coef<T>(wall_xp(g, cx)) +
                        (double)x[i - g.X] * (double)coef<T>(wall_ym(g, cy)) +
                        (double)x[i + g.X] * (double)coef<T>(wall_yp(g, cy)) +
                        (double)x[i - g.slab] * (double)coef<T>(wall_zm(g, cz)) +
                        (double)x[i + g.slab] * (double)coef<T>(wall_zp(g, cz));
      v = (double)b[i] - ax;
    }
    r[i] = (T)v;
  }
}

// zero the six border faces of a full-grid field (face cells only: the two
// z faces, the two y faces, the two x faces; edges are written more than once)
template <typename T>
__global__ void k_zero_border(Grid g, T* f) {
  const int nz = 2 * g.slab, ny = 2 * g.X * g.Z, nx = 2 * g.Y * g.Z;
  PL_GRID_STRIDE(k, nz + ny + nx) {
    int i;
    if (k < nz) {
      const int side = k / g.slab, j = k - side * g.slab;
      i = j + (side ? (g.Z - 1) * g.slab : 0);
    } else if (k < nz + ny) {
      const int m = k - nz, side = m / (g.X * g.Z), j = m - side * g.X * g.Z;
      const int x = j % g.X, z = j / g.X;
      i = x + (side ? g.Y - 1 : 0) * g.X + z * g.slab;
    } else {
      const int m = k - nz - ny, side = m / (g.Y * g.Z), j = m - side * g.Y * g.Z;
      const int y = j % g.Y, z = j / g.Y;
      i = (side ? g.X - 1 : 0) + y * g.X + z * g.slab;
    }
    f[i] = T(0);
  }
}

// Last node of the CG-graph loop body: keep looping while the solve is not
// done.  The body count also bounds the loop on the device: a body holds 16
// iterations and every iteration counts towards max_iters, so a loop that ran
// (max_iters + 64) / 16 bodies stops even if no kernel ever set `done`.
static __global__ void k_cg_continue(cudaGraphConditionalHandle h, CgState* st) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    st->bodies += 1;
    const bool more = !st->done && st->bodies * 16 <= st->max_iters + 64;
    cudaGraphSetConditional(h, more ? 1u : 0u);
  }
}

// ------------------------------------------------------------ MIC diagonal
// buildMICPreconditioner (FLUID_3D_MIC.cpp:825-856) for the cells of one
// hyperplane x+y+z = const (interior coordinates); the recurrence only reads
// the x-1, y-1, z-1 neighbours, which lie on the previous hyperplane.  FP64.
// `P64` is zero on the border, as the reference's _precon is.  Defined only in
// the FP64 translation unit (compiled without multiply-add contraction), so
// both engines use the same diagonal bits.
#ifdef PLUME_DEFINE_PRECON
__global__ void k_mic_precon_plane(Grid g, double* P64, int s, double tau, double sig) {
  PL_GRID_STRIDE(k, g.ny * g.nz) {
    const int j = k % g.ny, l = k / g.ny;
    const int ix = s - j - l;
    if (ix < 0 || ix >= g.nx) continue;
    const int x = ix + 1, y = j + 1, z = l + 1;
    const int i = x + y * g.X + z * g.slab;
    const int xm = i - 1, ym = i - g.X, zm = i - g.slab;
    // A+ at the minus neighbours (FLUID_3D_MIC.cpp:792-797 written by this
    // cell, or by the neighbour itself when it is an interior cell):
    const double ai_xm = coef<double>(wall_xm(g, x));
    const double aj_ym = coef<double>(wall_ym(g, y));
    const double ak_zm = coef<double>(wall_zm(g, z));
    // A+ of the neighbours toward their other plus-directions; only needed
    // when the neighbour is interior (its diagonal entry P is 0 otherwise).
    const double aj_xm = (x > 1) ? coef<double>(wall_yp(g, y)) : 0.0;
    const double ak_xm = (x > 1) ? coef<double>(wall_zp(g, z)) : 0.0;
    const double ai_ym = (y > 1) ? coef<double>(wall_xp(g, x)) : 0.0;
    const double ak_ym = (y > 1) ? coef<double>(wall_zp(g, z)) : 0.0;
    const double ai_zm = (z > 1) ? coef<double>(wall_xp(g, x)) : 0.0;
    const double aj_zm = (z > 1) ? coef<double>(wall_yp(g, y)) : 0.0;
    const double pmini2 = P64[xm] * P64[xm];
    const double pminj2 = P64[ym] * P64[ym];
    const double pmink2 = P64[zm] * P64[zm];
    const double e0 = ai_xm * ai_xm * pmini2 + aj_ym * aj_ym * pminj2 + ak_zm * ak_zm * pmink2;
    const double e1 = tau * (ai_xm * (aj_xm + ak_xm) * pmini2 + aj_ym * (ai_ym + ak_ym) * pminj2 +
                             ak_zm * (ai_zm + aj_zm) * pmink2);
    const double ad = adiag<double>(g, x, y, z);
    double e = ad - e0 - e1;
    if (e < sig * ad) e = ad;
    P64[i] = (fabs(ad) < 0.000001) ? 0.0 : 1.0 / sqrt(e);
  }
}
#endif
// Builds the FP64 MIC diagonal into P64 (hyperplane launches on `s`).
cudaError_t build_mic_diagonal(const Grid& g, double* P64, double tau, double sig, cudaStream_t s);

}  // namespace plume
