// products.cu -- the projected operators of the reduced model on the GPU
// (plume_reduced_build_products, include/plume_reduced.h).
//
// SUBSPACE_FLUID_3D_EIGEN::buildOutOfCoreMatrices (SUBSPACE_FLUID_3D_EIGEN.cpp:
// 1355-1490) with the four bases in HBM (FP64, column-major):
//   projected.A    = U_p^T  A^T U_p    A: buildFlatA (2162-2200)
//   projected.vtod = U_p^T  V   U_pp   V: computeVelocityToDivergence (1989-2107)
//   damping.peeled = U_pp^T D^T U_pd   D: buildPeeledDampingMatrixFlat (2112-2157)
//   projected.ptof = U_f^T      U_pp      EIGEN::transposeProduct
//   projected.ptov = U_f^T  G   U_p    G: computePressureToVelocity (627-695)
//   inverseProduct = (ptov projected.A^-1) vtod
// (SPARSE_MATRIX_ARRAY::projectVerySparse is left^T M^T right, and
// SPARSE_MATRIX::project is left^T M right.)  The sparse operators are never
// stored: k_apply evaluates one operator's row stencil for every column of a
// basis (W = M U; A and D are symmetric, so M^T U = M U), k_atb forms L^T R
// split over the long dimension with a fixed-order reduction (k_sum_split),
// and the inverse is a Gauss-Jordan elimination with partial pivoting: in
// one block's shared memory up to rank 96 (k_gj_small), above that one pivot
// column per launch pair (k_gj_pivot, k_gj_update).
//
// The bases stay resident for the whole build (the reference reads and drops
// them one at a time to fit host memory); at 128x192x128 one basis of rank
// 300 is 21.7 GB, so the four fit HBM with room for the work matrix.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <memory>
#include <string>
#include <vector>

#include "../../include/plume.h"
#include "../../include/plume_reduced.h"
#include "engine.h"
#include "matrix_file.cuh"

namespace plume {
namespace products {

// The peeled grid and the wall flags (front, back, left, right, top,
// bottom): z low, z high, x low, x high, y high, y low.
struct Peeled {
  int nx, ny, nz;
  long long n;  // N_int
  int bc[6];
  double dx;
};

enum Op { OP_A = 0, OP_V = 1, OP_D = 2, OP_G = 3 };

// The entries of one operator row in fixed slots (an absent entry is
// column `self` with value 0, which adds exactly nothing), so that the
// slots stay in registers.
struct Row {
  long long col[7];
  double val[7];
};

template <int OP>
struct Slots {
  static constexpr int n = OP == OP_V ? 6 : (OP == OP_G ? 2 : 7);
};

__device__ inline void cell_of(const Peeled& g, long long i, int& x, int& y, int& z) {
  x = (int)(i % g.nx);
  const long long t = i / g.nx;
  y = (int)(t % g.ny);
  z = (int)(t / g.ny);
}

__device__ inline void put(Row& r, int k, bool present, long long col, long long self, double v) {
  r.col[k] = present ? col : self;
  r.val[k] = present ? v : 0.0;
}

// buildFlatA, row i: the wall slabs are the only obstacles
// (FLUID_3D_MIC.cpp:121-158, a slab is an obstacle when its flag is 1), so a
// face neighbour is skipped exactly when it is a wall; off-diagonal -1 only
// towards interior neighbours.
__device__ inline void row_a(const Peeled& g, long long i, Row& r) {
  int x, y, z;
  cell_of(g, i, x, y, z);
  const long long sx = (long long)g.nx * g.ny;
  double diag = 6.0;
  diag -= (x == 0 && g.bc[2] == 1) + (x == g.nx - 1 && g.bc[3] == 1);
  diag -= (y == 0 && g.bc[5] == 1) + (y == g.ny - 1 && g.bc[4] == 1);
  diag -= (z == 0 && g.bc[0] == 1) + (z == g.nz - 1 && g.bc[1] == 1);
  put(r, 0, true, i, i, diag);
  put(r, 1, x != 0, i - 1, i, -1.0);
  put(r, 2, x != g.nx - 1, i + 1, i, -1.0);
  put(r, 3, y != 0, i - g.nx, i, -1.0);
  put(r, 4, y != g.ny - 1, i + g.nx, i, -1.0);
  put(r, 5, z != 0, i - sx, i, -1.0);
  put(r, 6, z != g.nz - 1, i + sx, i, -1.0);
}

// computeVelocityToDivergence, row i (columns are interleaved velocity
// components, 3 j + c): per axis a high-side and a low-side term, replaced at
// the last / first interior index by the wall's own-cell term (flag != 0) or
// the mirrored neighbour (flag 0).  The reference accumulates with +=, so two
// terms on one column are one entry (coeff - coeff = 0 on a mirrored face).
__device__ inline void row_v(const Peeled& g, long long i, Row& r) {
  int p[3];
  cell_of(g, i, p[0], p[1], p[2]);
  const int len[3] = {g.nx, g.ny, g.nz};
  const long long step[3] = {1, g.nx, (long long)g.nx * g.ny};
  const int hi_bc[3] = {g.bc[3], g.bc[4], g.bc[1]};  // right, top, back
  const int lo_bc[3] = {g.bc[2], g.bc[5], g.bc[0]};  // left, bottom, front
  const double coeff = -g.dx * 0.5;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const long long s = step[c];
    long long ch, cl;
    double vh, vl;
    if (p[c] != len[c] - 1) {
      ch = 3 * (i + s) + c;
      vh = coeff;
    } else if (hi_bc[c] != 0) {
      ch = 3 * i + c;
      vh = -coeff;
    } else {
      ch = 3 * (i - s) + c;
      vh = coeff;
    }
    if (p[c] != 0) {
      cl = 3 * (i - s) + c;
      vl = -coeff;
    } else if (lo_bc[c] != 0) {
      cl = 3 * i + c;
      vl = coeff;
    } else {
      cl = 3 * (i + s) + c;
      vl = -coeff;
    }
    if (ch == cl) {
      r.col[2 * c] = ch;
      r.val[2 * c] = vh + vl;
      r.col[2 * c + 1] = ch;
      r.val[2 * c + 1] = 0.0;
    } else {
      r.col[2 * c] = ch;
      r.val[2 * c] = vh;
      r.col[2 * c + 1] = cl;
      r.val[2 * c + 1] = vl;
    }
  }
}

// buildPeeledDampingMatrixFlat, row 3 i + c: (1 - w) on the diagonal, w / 6
// to the same component of each interior neighbour, w = 0.9.
__device__ inline void row_d(const Peeled& g, long long row, Row& r) {
  const double w = 0.9;
  const double sixth = (1. / 6.) * w;
  const long long i = row / 3;
  const int c = (int)(row % 3);
  int x, y, z;
  cell_of(g, i, x, y, z);
  const long long sx = (long long)g.nx * g.ny;
  put(r, 0, true, row, row, 1.0 - w);
  put(r, 1, x != g.nx - 1, 3 * (i + 1) + c, row, sixth);
  put(r, 2, x != 0, 3 * (i - 1) + c, row, sixth);
  put(r, 3, y != g.ny - 1, 3 * (i + g.nx) + c, row, sixth);
  put(r, 4, y != 0, 3 * (i - g.nx) + c, row, sixth);
  put(r, 5, z != g.nz - 1, 3 * (i + sx) + c, row, sixth);
  put(r, 6, z != 0, 3 * (i - sx) + c, row, sixth);
}

// computePressureToVelocity, row 3 i + c: one-sided difference at the first
// (then the last) interior index, central otherwise.
__device__ inline void row_g(const Peeled& g, long long row, Row& r) {
  const double inv = 1.0 / g.dx, half = 0.5 / g.dx;
  const long long i = row / 3;
  const int c = (int)(row % 3);
  int x, y, z;
  cell_of(g, i, x, y, z);
  const int pc = c == 0 ? x : (c == 1 ? y : z);
  const int len = c == 0 ? g.nx : (c == 1 ? g.ny : g.nz);
  const long long s = c == 0 ? 1 : (c == 1 ? (long long)g.nx : (long long)g.nx * g.ny);
  if (pc == 0) {
    r.col[0] = i + s;
    r.val[0] = -inv;
    r.col[1] = i;
    r.val[1] = inv;
  } else if (pc == len - 1) {
    r.col[0] = i;
    r.val[0] = -inv;
    r.col[1] = i - s;
    r.val[1] = inv;
  } else {
    r.col[0] = i + s;
    r.val[0] = -half;
    r.col[1] = i - s;
    r.val[1] = half;
  }
}

// W(:, j) = M U(:, j) for every column j: one thread per row of M, the row's
// entries in registers, the columns in a loop (each column read coalesced).
template <int OP>
__global__ void k_apply(Peeled g, long long rows, const double* __restrict__ U, long long ldu, int cols,
                        double* __restrict__ W) {
  const long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= rows) return;
  Row r;
  if (OP == OP_A) row_a(g, row, r);
  if (OP == OP_V) row_v(g, row, r);
  if (OP == OP_D) row_d(g, row, r);
  if (OP == OP_G) row_g(g, row, r);
#pragma unroll 4
  for (int j = 0; j < cols; j++) {
    const double* u = U + (size_t)j * ldu;
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < Slots<OP>::n; k++) s = fma(r.val[k], __ldg(u + r.col[k]), s);
    W[(size_t)j * rows + row] = s;
  }
}

constexpr int kTile = 32;
constexpr int kAtbThreads = 256;

// partial[s] = L^T R over the s-th chunk of the K rows, L(k, i) at
// L[k lsk + i lsi], R(k, j) at R[k rsk + j rsj], output column-major (a x b).
// A 32 x 32 output tile per block, 2 x 2 outputs per thread, the K rows
// staged through shared memory 32 at a time.
__global__ void __launch_bounds__(kAtbThreads) k_atb(const double* __restrict__ L, long long lsk, long long lsi,
                                                      const double* __restrict__ R, long long rsk, long long rsj,
                                                      long long K, int a, int b, long long chunk,
                                                      double* __restrict__ partial) {
  __shared__ double sL[kTile][kTile + 1], sR[kTile][kTile + 1];
  const int i0 = blockIdx.x * kTile, j0 = blockIdx.y * kTile;
  const long long kbeg = (long long)blockIdx.z * chunk;
  const long long kend = K < kbeg + chunk ? K : kbeg + chunk;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
  for (long long k0 = kbeg; k0 < kend; k0 += kTile) {
    for (int e = threadIdx.x; e < kTile * kTile; e += kAtbThreads) {
      const int kk = e % kTile, c = e / kTile;
      const long long k = k0 + kk;
      const bool kin = k < kend;
      sL[kk][c] = (kin && i0 + c < a) ? L[k * lsk + (long long)(i0 + c) * lsi] : 0.0;
      sR[kk][c] = (kin && j0 + c < b) ? R[k * rsk + (long long)(j0 + c) * rsj] : 0.0;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < kTile; kk++) {
      const double l0 = sL[kk][tx], l1 = sL[kk][tx + 16];
      const double r0 = sR[kk][ty], r1 = sR[kk][ty + 16];
      acc[0][0] = fma(l0, r0, acc[0][0]);
      acc[1][0] = fma(l1, r0, acc[1][0]);
      acc[0][1] = fma(l0, r1, acc[0][1]);
      acc[1][1] = fma(l1, r1, acc[1][1]);
    }
    __syncthreads();
  }
  double* out = partial + (size_t)blockIdx.z * a * b;
  for (int u = 0; u < 2; u++)
    for (int v = 0; v < 2; v++) {
      const int i = i0 + tx + 16 * u, j = j0 + ty + 16 * v;
      if (i < a && j < b) out[(size_t)j * a + i] = acc[u][v];
    }
}

// C = sum over the splits: a block per 32 consecutive outputs, its 8 warps
// taking every 8th split (reads coalesced along the outputs), then the 8
// partial sums added in warp order, so the result is the same on every run.
constexpr int kSumWarps = 8;
__global__ void __launch_bounds__(32 * kSumWarps) k_sum_split(const double* __restrict__ partial, int nsplit,
                                                              long long count, double* __restrict__ C) {
  __shared__ double part[kSumWarps][33];
  const int lane = threadIdx.x % 32, w = threadIdx.x / 32;
  const long long e = (long long)blockIdx.x * 32 + lane;
  double s = 0.0;
  if (e < count)
    for (int p = w; p < nsplit; p += kSumWarps) s += partial[(size_t)p * count + e];
  part[w][lane] = s;
  __syncthreads();
  if (w == 0 && e < count) {
    double t = part[0][lane];
    for (int k = 1; k < kSumWarps; k++) t += part[k][lane];
    C[e] = t;
  }
}

// M = [A | I] (r x 2r, column-major) from the column-major A.
__global__ void k_gj_init(const double* __restrict__ A, int r, double* __restrict__ M) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= 2LL * r * r) return;
  const int i = (int)(e % r), j = (int)(e / r);
  M[e] = j < r ? A[e] : (j - r == i ? 1.0 : 0.0);
}

// Pivot step k: the row p >= k with the largest |M(p, k)| (the first one on
// ties); row p divided by the pivot (the new row k), row k and column k
// copied for the update, so that the update reads nothing it writes.  status[0] = 1 + k when column k has no
// nonzero pivot (the matrix is singular); later steps then do nothing.
__global__ void k_gj_pivot(const double* __restrict__ M, int r, int k, double* __restrict__ prow,
                           double* __restrict__ krow, double* __restrict__ kcol, int* __restrict__ status) {
  __shared__ double sv[256];
  __shared__ int si[256];
  if (status[0] != 0) return;
  double best = -1.0;
  int bi = r;
  for (int i = k + threadIdx.x; i < r; i += blockDim.x) {
    const double v = fabs(M[(size_t)k * r + i]);
    if (v > best) {
      best = v;
      bi = i;
    }
  }
  sv[threadIdx.x] = best;
  si[threadIdx.x] = bi;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      const double v = sv[threadIdx.x + o];
      const int vi = si[threadIdx.x + o];
      if (v > sv[threadIdx.x] || (v == sv[threadIdx.x] && vi < si[threadIdx.x])) {
        sv[threadIdx.x] = v;
        si[threadIdx.x] = vi;
      }
    }
    __syncthreads();
  }
  const int p = si[0];
  if (!(sv[0] > 0.0)) {  // zero or NaN pivot
    if (threadIdx.x == 0) status[0] = 1 + k;
    return;
  }
  const double pivot = M[(size_t)k * r + p];
  for (int j = threadIdx.x; j < 2 * r; j += blockDim.x) {
    prow[j] = M[(size_t)j * r + p] / pivot;  // the new row k, one division per column
    krow[j] = M[(size_t)j * r + k];
  }
  for (int i = threadIdx.x; i < r; i += blockDim.x) kcol[i] = M[(size_t)k * r + i];
  if (threadIdx.x == 0) status[1] = p;
}

// Update step k: row k <- the new row k; row p (when p != k) <- old row k
// minus its multiple of the new row k; every other row i <- row i -
// M(i, k) x new row k.
__global__ void k_gj_update(double* __restrict__ M, int r, int k, const double* __restrict__ prow,
                            const double* __restrict__ krow, const double* __restrict__ kcol,
                            const int* __restrict__ status) {
  if (status[0] != 0) return;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= 2LL * r * r) return;
  const int i = (int)(e % r), j = (int)(e / r);
  const int p = status[1];
  const double pr = prow[j];
  if (i == k) {
    M[e] = pr;
  } else if (i == p) {
    M[e] = krow[j] - krow[k] * pr;
  } else {
    M[e] = M[e] - kcol[i] * pr;
  }
}

// The whole elimination in one block with [A | I] in shared memory, for
// ranks whose 2 r^2 doubles fit: one launch in place of r launch pairs.  The
// same pivot choice (first largest |M(i, k)|, i >= k) and the same update
// arithmetic as k_gj_pivot + k_gj_update.
constexpr int kGjSmallMax = 96;  // (2 r^2 + 5 r) doubles = 151 KB at r = 96
constexpr int kGjThreads = 512;
__global__ void __launch_bounds__(kGjThreads) k_gj_small(const double* __restrict__ A, int r, double* __restrict__ M,
                                                         int* __restrict__ status) {
  extern __shared__ double gj[];
  double* S = gj;                // r x 2r, column-major
  double* prow = S + 2 * r * r;  // pivot row, 2r
  double* krow = prow + 2 * r;   // row k, 2r
  double* kcol = krow + 2 * r;   // column k, r
  __shared__ double wv[kGjThreads / 32];
  __shared__ int wi[kGjThreads / 32];
  __shared__ int piv;
  const int lane = threadIdx.x % 32, warp = threadIdx.x / 32;
  const int n2 = 2 * r * r;
  for (int e = threadIdx.x; e < n2; e += blockDim.x) {
    const int i = e % r, j = e / r;
    S[e] = j < r ? A[e] : (j - r == i ? 1.0 : 0.0);
  }
  __syncthreads();
  for (int k = 0; k < r; k++) {
    double best = -1.0;
    int bi = r;
    for (int i = k + threadIdx.x; i < r; i += blockDim.x) {
      const double v = fabs(S[k * r + i]);
      if (v > best) {
        best = v;
        bi = i;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_down_sync(0xffffffffu, best, o);
      const int oi = __shfl_down_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi < bi)) {
        best = ov;
        bi = oi;
      }
    }
    if (lane == 0) {
      wv[warp] = best;
      wi[warp] = bi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double b = wv[0];
      int ii = wi[0];
      for (int w = 1; w < kGjThreads / 32; w++)
        if (wv[w] > b || (wv[w] == b && wi[w] < ii)) {
          b = wv[w];
          ii = wi[w];
        }
      piv = b > 0.0 ? ii : -1;  // zero or NaN pivot: singular
    }
    __syncthreads();
    const int p = piv;
    if (p < 0) {  // every thread sees the same p and leaves together
      if (threadIdx.x == 0) status[0] = 1 + k;
      return;
    }
    const double pivot = S[k * r + p];
    for (int j = threadIdx.x; j < 2 * r; j += blockDim.x) {
      prow[j] = S[j * r + p] / pivot;  // the new row k, one division per column
      krow[j] = S[j * r + k];
    }
    for (int i = threadIdx.x; i < r; i += blockDim.x) kcol[i] = S[k * r + i];
    __syncthreads();
    for (int e = threadIdx.x; e < n2; e += blockDim.x) {
      const int i = e % r, j = e / r;
      const double pr = prow[j];
      if (i == k)
        S[e] = pr;
      else if (i == p)
        S[e] = krow[j] - krow[k] * pr;
      else
        S[e] = S[e] - kcol[i] * pr;
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < n2; e += blockDim.x) M[e] = S[e];
}

}  // namespace products
}  // namespace plume

using namespace plume::products;
using namespace plume::matrix_file;

namespace {

int fail(int code, const std::string& msg) {
  plume::global_error() = msg;
  return code;
}

struct DevBuf {
  double* p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  cudaError_t alloc(size_t count) { return cudaMalloc(&p, std::max<size_t>(1, count) * sizeof(double)); }
};

// How many splits of the K rows give four blocks to every SM (chunks of at
// least 256 rows).  With one output tile, as for rank-32 bases, that is
// exactly 4 x SMs equal chunks: a whole number of blocks per SM, so no SM
// waits on a partial last wave (352 splits of a 361,336-row basis left 2 or
// 3 blocks per SM and 70 % of the SMs' throughput).
int split_count(long long K, int a, int b, int sms) {
  const long long tiles = (long long)((a + kTile - 1) / kTile) * ((b + kTile - 1) / kTile);
  const long long want = (4LL * sms + tiles - 1) / tiles;
  const long long most = std::max(1LL, K / 256);
  return (int)std::max(1LL, std::min(std::min(want, most), 65535LL));
}

// The dense projections of one build, launched on one stream.
struct Projector {
  cudaStream_t s;
  int sms;
  double* partial;
  double flops = 0;
  // C (a x b, column-major) = L^T R
  void atb(const double* L, long long lsk, long long lsi, const double* R, long long rsk, long long rsj, long long K,
           int a, int b, double* C) {
    if (a == 0 || b == 0) return;
    const int nsplit = split_count(K, a, b, sms);
    // equal chunks (not rounded to whole 32-row tiles, which would leave the
    // last splits empty and the SMs unevenly loaded again)
    const long long chunk = (K + nsplit - 1) / nsplit;
    const dim3 grid((unsigned)((a + kTile - 1) / kTile), (unsigned)((b + kTile - 1) / kTile), (unsigned)nsplit);
    if (nsplit == 1) {
      k_atb<<<grid, kAtbThreads, 0, s>>>(L, lsk, lsi, R, rsk, rsj, K, a, b, chunk, C);
    } else {
      k_atb<<<grid, kAtbThreads, 0, s>>>(L, lsk, lsi, R, rsk, rsj, K, a, b, chunk, partial);
      const long long count = (long long)a * b;
      k_sum_split<<<(unsigned)((count + 31) / 32), 32 * kSumWarps, 0, s>>>(partial, nsplit, count, C);
    }
    flops += 2.0 * K * a * b;
  }
  static size_t partial_size(long long K, int a, int b, int sms) {
    const int nsplit = split_count(K, a, b, sms);
    return nsplit == 1 ? 0 : (size_t)nsplit * a * b;
  }
};

template <int OP>
void apply(const Peeled& g, long long rows, const double* U, long long ldu, int cols, double* W, cudaStream_t s) {
  if (rows == 0 || cols == 0) return;
  k_apply<OP><<<(unsigned)((rows + 255) / 256), 256, 0, s>>>(g, rows, U, ldu, cols, W);
}

}  // namespace

extern "C" int plume_reduced_build_products(plume_handle* h, const char* reduced_path, plume_products_info* info) {
  if (!h || !reduced_path) return fail(PLUME_ERR_INVALID, "bad argument");
  const auto t0 = std::chrono::steady_clock::now();
  plume::Engine* e = plume::engine_of(h);
  const plume_params& p = e->params();
  if (cudaSetDevice(p.device) != cudaSuccess) return fail(PLUME_ERR_CUDA, "cudaSetDevice failed");
  Peeled g;
  g.nx = p.res[0] - 2;
  g.ny = p.res[1] - 2;
  g.nz = p.res[2] - 2;
  if (g.nx < 2 || g.ny < 2 || g.nz < 2) return fail(PLUME_ERR_INVALID, "grid too small for the reduced operators");
  g.n = (long long)g.nx * g.ny * g.nz;
  for (int k = 0; k < 6; k++) g.bc[k] = p.bc[k];
  g.dx = e->dx();
  const long long n = g.n, m = 3 * g.n;
  const std::string dir = reduced_path;
  std::string err;
  // the bases, in the order buildOutOfCoreMatrices reads them
  DevBuf Up, Upp, Upd, Uf;
  int rp = 0, rpp = 0, rpd = 0, rf = 0;
  int rc = upload_basis(dir + "U.pressure.matrix", (size_t)n, Up.p, rp, err);
  if (rc == PLUME_OK) rc = upload_basis(dir + "U.preproject.matrix", (size_t)m, Upp.p, rpp, err);
  if (rc == PLUME_OK) rc = upload_basis(dir + "U.prediffuse.matrix", (size_t)m, Upd.p, rpd, err);
  if (rc == PLUME_OK) rc = upload_basis(dir + "U.final.matrix", (size_t)m, Uf.p, rf, err);
  if (rc != PLUME_OK) return fail(rc, "cannot build the projected operators: " + err);
  if (rp == 0) return fail(PLUME_ERR_INVALID, "U.pressure.matrix has no columns");
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p.device);
  sms = std::max(sms, 1);
  const long long wsize = std::max(std::max(n * rp, n * rpp), std::max(m * rpd, m * rp));
  size_t psize = 0;
  psize = std::max(psize, Projector::partial_size(n, rp, rp, sms));
  psize = std::max(psize, Projector::partial_size(n, rp, rpp, sms));
  psize = std::max(psize, Projector::partial_size(m, rpp, rpd, sms));
  psize = std::max(psize, Projector::partial_size(m, rf, rpp, sms));
  psize = std::max(psize, Projector::partial_size(m, rf, rp, sms));
  psize = std::max(psize, Projector::partial_size(rp, rf, rp, sms));
  psize = std::max(psize, Projector::partial_size(rp, rf, rpp, sms));
  DevBuf W, part, Ar, vtod, damp, ptof, ptov, M, T, G, prow, krow, kcol;
  int* status = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  auto release = [&]() {
    if (status) cudaFree(status);
    for (auto x : ev)
      if (x) cudaEventDestroy(x);
  };
  if (W.alloc((size_t)wsize) != cudaSuccess || part.alloc(psize) != cudaSuccess ||
      Ar.alloc((size_t)rp * rp) != cudaSuccess || vtod.alloc((size_t)rp * rpp) != cudaSuccess ||
      damp.alloc((size_t)rpp * rpd) != cudaSuccess || ptof.alloc((size_t)rf * rpp) != cudaSuccess ||
      ptov.alloc((size_t)rf * rp) != cudaSuccess || M.alloc(2 * (size_t)rp * rp) != cudaSuccess ||
      T.alloc((size_t)rf * rp) != cudaSuccess || G.alloc((size_t)rf * rpp) != cudaSuccess ||
      prow.alloc(2 * (size_t)rp) != cudaSuccess || krow.alloc(2 * (size_t)rp) != cudaSuccess ||
      kcol.alloc((size_t)rp) != cudaSuccess || cudaMalloc(&status, 2 * sizeof(int)) != cudaSuccess ||
      cudaEventCreate(&ev[0]) != cudaSuccess || cudaEventCreate(&ev[1]) != cudaSuccess) {
    release();
    return fail(PLUME_ERR_OOM, "the projected-operator build does not fit on the device");
  }
  cudaStream_t s = (cudaStream_t)e->stream_handle();
  Projector pj{s, sms, part.p};
  cudaMemsetAsync(status, 0, 2 * sizeof(int), s);
  cudaEventRecord(ev[0], s);
  // projected.A = U_p^T A U_p
  apply<OP_A>(g, n, Up.p, n, rp, W.p, s);
  pj.atb(Up.p, 1, n, W.p, 1, n, n, rp, rp, Ar.p);
  // projected.vtod = U_p^T V U_pp
  apply<OP_V>(g, n, Upp.p, m, rpp, W.p, s);
  pj.atb(Up.p, 1, n, W.p, 1, n, n, rp, rpp, vtod.p);
  // damping.peeled = U_pp^T D U_pd
  apply<OP_D>(g, m, Upd.p, m, rpd, W.p, s);
  pj.atb(Upp.p, 1, m, W.p, 1, m, m, rpp, rpd, damp.p);
  // projected.ptof = U_f^T U_pp
  pj.atb(Uf.p, 1, m, Upp.p, 1, m, m, rf, rpp, ptof.p);
  // projected.ptov = U_f^T G U_p
  apply<OP_G>(g, m, Up.p, n, rp, W.p, s);
  pj.atb(Uf.p, 1, m, W.p, 1, m, m, rf, rp, ptov.p);
  // projected.A^-1: Gauss-Jordan on [A | I]
  const long long mcount = 2LL * rp * rp;
  if (rp <= kGjSmallMax) {
    const size_t smem = (2 * (size_t)rp * rp + 5 * (size_t)rp) * sizeof(double);
    const cudaError_t attr = cudaFuncSetAttribute(
        k_gj_small, cudaFuncAttributeMaxDynamicSharedMemorySize,
        (int)((2 * kGjSmallMax * kGjSmallMax + 5 * kGjSmallMax) * sizeof(double)));
    if (attr != cudaSuccess) {
      release();
      return fail(PLUME_ERR_CUDA, "cannot reserve shared memory for the elimination");
    }
    k_gj_small<<<1, kGjThreads, smem, s>>>(Ar.p, rp, M.p, status);
  } else {
    k_gj_init<<<(unsigned)((mcount + 255) / 256), 256, 0, s>>>(Ar.p, rp, M.p);
    for (int k = 0; k < rp; k++) {
      k_gj_pivot<<<1, 256, 0, s>>>(M.p, rp, k, prow.p, krow.p, kcol.p, status);
      k_gj_update<<<(unsigned)((mcount + 255) / 256), 256, 0, s>>>(M.p, rp, k, prow.p, krow.p, kcol.p, status);
    }
  }
  const double gj_flops = 4.0 * rp * (double)rp * rp;
  // inverseProduct = (ptov A^-1) vtod
  pj.atb(ptov.p, rf, 1, M.p + (size_t)rp * rp, 1, rp, rp, rf, rp, T.p);
  pj.atb(T.p, rf, 1, vtod.p, 1, rp, rp, rf, rpp, G.p);
  cudaEventRecord(ev[1], s);
  int hstatus[2] = {0, 0};
  cudaError_t ce = cudaGetLastError();
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(hstatus, status, sizeof(hstatus), cudaMemcpyDeviceToHost, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  float ms = 0.f;
  if (ce == cudaSuccess) cudaEventElapsedTime(&ms, ev[0], ev[1]);
  release();
  if (ce != cudaSuccess) return fail(PLUME_ERR_CUDA, std::string("projected-operator build: ") + cudaGetErrorString(ce));
  if (hstatus[0] != 0)
    return fail(PLUME_ERR_INVALID, "projected.A is singular (no pivot in column " + std::to_string(hstatus[0] - 1) + ")");
  // the six files, in the reference's order
  struct Out {
    const char* name;
    int rows, cols;
    const double* d;
  } outs[6] = {{"projected.A.matrix", rp, rp, Ar.p},       {"projected.vtod.matrix", rp, rpp, vtod.p},
               {"damping.peeled.matrix", rpp, rpd, damp.p}, {"projected.ptof.matrix", rf, rpp, ptof.p},
               {"projected.ptov.matrix", rf, rp, ptov.p},   {"inverseProduct.matrix", rf, rpp, G.p}};
  std::vector<double> hbuf;
  for (const Out& o : outs) {
    hbuf.resize((size_t)o.rows * o.cols);
    if (!hbuf.empty() && cudaMemcpy(hbuf.data(), o.d, hbuf.size() * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
      return fail(PLUME_ERR_CUDA, "projected-operator download failed");
    if (!write_matrix_colmajor(dir + o.name, o.rows, o.cols, hbuf.data()))
      return fail(PLUME_ERR_IO, "could not write " + dir + o.name);
  }
  if (info) {
    info->ranks[0] = rp;
    info->ranks[1] = rpp;
    info->ranks[2] = rpd;
    info->ranks[3] = rf;
    info->ms_device = ms;
    info->ms_total =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    info->gflop = (pj.flops + gj_flops) * 1e-9;
  }
  return PLUME_OK;
}
