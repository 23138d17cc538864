// svd.cu -- the snapshot SVD of svdOutOfCoreMultiple on the GPU
// (include/plume_svd.h).
//
// A (n x m, FP64, column j = snapshot j, contiguous) lives whole in HBM.
//   1. Modified Gram-Schmidt, BIG_MATRIX::outOfCoreQR (BIG_MATRIX.cpp:100-259):
//      column i is normalised, then removed from every later column; R(i, j) =
//      q_i . a_j.  One pass per column reads and writes the later columns once:
//      it scales a_i into q_i, updates a_j -= R(i, j) q_i and, with the updated
//      values still in registers, accumulates a_{i+1} . a_j for the next pass
//      (so R(i+1, j) = (a_{i+1} . a_j) / |a_{i+1}|, the same product up to
//      rounding order).  Dot products reduce in a fixed order (deterministic).
//   2. R = U_R S V^T by a one-sided (Hestenes) Jacobi SVD: columns of W = R are
//      rotated pairwise, in round-robin order, until every pair is orthogonal
//      to working precision; S = column norms, U_R = normalised columns.  One
//      cooperative launch, a grid barrier between rounds.
//   3. U = Q U_R[:, :kept] by a tiled FP64 GEMM writing the row-major layout of
//      writeFinalU (BIG_MATRIX.cpp:613-647) directly.
// FP64 issues at 1/64 of the FP32 rate on this part, so steps 1 and 3 are
// FP64-FMA-bound at full size; their traffic is streamed once per pass.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/plume.h"
#include "../../include/plume_svd.h"
#include "engine.h"

namespace cg = cooperative_groups;

namespace plume {
namespace svd {

constexpr int kThreads = 256;
constexpr int kRowsPerThread = 8;                       // q and a_{i+1} kept in registers
constexpr int kRowsPerBlock = kThreads * kRowsPerThread;  // 2048 rows per block
constexpr int kWarps = kThreads / 32;

__device__ inline double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Column j of A starts at A + j n.
__device__ inline double* col(double* A, size_t n, int j) { return A + (size_t)j * n; }

// Pass -1: dots of column 0 with columns 0..m-1 (partials per block).
__global__ void k_dots0(double* A, size_t n, int m, double* partial, int nblk) {
  extern __shared__ double sm[];  // [m][kWarps]
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const size_t base = (size_t)blockIdx.x * kRowsPerBlock + threadIdx.x;
  double a0[kRowsPerThread];
#pragma unroll
  for (int k = 0; k < kRowsPerThread; k++) {
    const size_t r = base + (size_t)k * kThreads;
    a0[k] = r < n ? A[r] : 0.0;
  }
  for (int j = 0; j < m; j++) {
    const double* aj = col(A, n, j);
    double p = 0.0;
#pragma unroll
    for (int k = 0; k < kRowsPerThread; k++) {
      const size_t r = base + (size_t)k * kThreads;
      if (r < n) p = fma(a0[k], aj[r], p);
    }
    p = warp_sum(p);
    if (lane == 0) sm[j * kWarps + warp] = p;
  }
  __syncthreads();
  for (int j = threadIdx.x; j < m; j += kThreads) {
    double s = 0.0;
    for (int w = 0; w < kWarps; w++) s += sm[j * kWarps + w];
    partial[(size_t)j * nblk + blockIdx.x] = s;
  }
}

// Pass i (0 <= i < m): q_i = a_i / |a_i| (inv from the finaliser), then for
// j > i: a_j -= R(i, j) q_i, accumulating a_{i+1}.a_{i+1} and a_{i+1}.a_j.
__global__ void k_mgs_pass(double* A, size_t n, int m, int i, const double* R, const double* inv_ptr,
                           double* partial, int nblk) {
  extern __shared__ double sm[];  // [m - i - 1][kWarps] then R row [m - i - 1]
  const int cnt = m - i - 1;
  double* rrow = sm + (size_t)cnt * kWarps;
  for (int jj = threadIdx.x; jj < cnt; jj += kThreads) rrow[jj] = R[(size_t)(i + 1 + jj) * m + i];
  __syncthreads();
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const size_t base = (size_t)blockIdx.x * kRowsPerBlock + threadIdx.x;
  const double inv = *inv_ptr;
  double* ai = col(A, n, i);
  double q[kRowsPerThread], nx[kRowsPerThread];
#pragma unroll
  for (int k = 0; k < kRowsPerThread; k++) {
    const size_t r = base + (size_t)k * kThreads;
    q[k] = 0.0;
    nx[k] = 0.0;
    if (r < n) {
      q[k] = ai[r] * inv;  // VECTOR::operator*= (BIG_MATRIX.cpp:231-232)
      ai[r] = q[k];
    }
  }
  for (int jj = 0; jj < cnt; jj++) {
    double* aj = col(A, n, i + 1 + jj);
    const double rij = rrow[jj];
    double p = 0.0;
#pragma unroll
    for (int k = 0; k < kRowsPerThread; k++) {
      const size_t r = base + (size_t)k * kThreads;
      if (r < n) {
        const double v = fma(-rij, q[k], aj[r]);  // axpy(-dot, column) (BIG_MATRIX.cpp:240)
        aj[r] = v;
        if (jj == 0) nx[k] = v;
        p = fma(nx[k], v, p);
      }
    }
    p = warp_sum(p);
    if (lane == 0) sm[jj * kWarps + warp] = p;
  }
  __syncthreads();
  for (int jj = threadIdx.x; jj < cnt; jj += kThreads) {
    double s = 0.0;
    for (int w = 0; w < kWarps; w++) s += sm[jj * kWarps + w];
    partial[(size_t)jj * nblk + blockIdx.x] = s;
  }
}

// dot[first + jj] = sum over blocks of partial[jj][.], one warp per jj, in a
// fixed order.
__global__ void k_reduce(const double* partial, int nblk, int cnt, double* dot, int first) {
  const int jj = blockIdx.x * kWarps + threadIdx.x / 32, lane = threadIdx.x % 32;
  if (jj >= cnt) return;
  double s = 0.0;
  for (int b = lane; b < nblk; b += 32) s += partial[(size_t)jj * nblk + b];
  s = warp_sum(s);
  if (lane == 0) dot[first + jj] = s;
}

// Column i's norm and R row i (BIG_MATRIX.cpp:222-243): R(i, i) = |a_i|,
// R(i, j) = (a_i . a_j) / |a_i|; inv = 1 / |a_i|.
__global__ void k_finalize(const double* dot, int m, int i, double* R, double* inv_out) {
  const double norm = sqrt(dot[i]);
  const double inv = 1.0 / norm;
  if (threadIdx.x == 0) {
    R[(size_t)i * m + i] = norm;
    *inv_out = inv;
  }
  for (int j = i + 1 + threadIdx.x; j < m; j += blockDim.x) R[(size_t)j * m + i] = dot[j] * inv;
}

// ---- one-sided Jacobi SVD of W (m x m, column-major) ----------------------
struct JacobiCtl {
  unsigned long long rotations[2];  // per sweep parity
  int sweeps;
};

// Round-robin pairing (circle method) over M = m rounded up to even players:
// round k pairs players (k + t) mod (M-1) and (k - t) mod (M-1) for
// t = 1..M/2-1, and k with the fixed player M-1.
__device__ inline void pair_of(int k, int t, int M, int& p, int& q) {
  if (t == 0) {
    p = k;
    q = M - 1;
  } else {
    p = (k + t) % (M - 1);
    q = (k - t + (M - 1)) % (M - 1);
  }
}

// V is not formed: the reference keeps only U and S of R's SVD.
__global__ void k_jacobi(double* W, int m, JacobiCtl* ctl, int max_sweeps, double tol) {
  cg::grid_group grid = cg::this_grid();
  const int M = m + (m & 1);
  const int warps_total = gridDim.x * kWarps;
  const int gw = blockIdx.x * kWarps + threadIdx.x / 32, lane = threadIdx.x % 32;
  int sweep = 0;
  for (; sweep < max_sweeps; sweep++) {
    const int par = sweep & 1;
    if (gw == 0 && lane == 0) ctl->rotations[par ^ 1] = 0;  // the next sweep's counter
    unsigned long long mine = 0;
    for (int k = 0; k < M - 1; k++) {
      for (int t = gw; t < M / 2; t += warps_total) {
        int p, q;
        pair_of(k, t, M, p, q);
        if (p >= m || q >= m) continue;  // the padding column
        if (p > q) {
          const int s = p;
          p = q;
          q = s;
        }
        double* wp = W + (size_t)p * m;
        double* wq = W + (size_t)q * m;
        double al = 0.0, be = 0.0, ga = 0.0;
        for (int r = lane; r < m; r += 32) {
          const double x = wp[r], y = wq[r];
          al = fma(x, x, al);
          be = fma(y, y, be);
          ga = fma(x, y, ga);
        }
        al = __shfl_sync(0xffffffffu, warp_sum(al), 0);
        be = __shfl_sync(0xffffffffu, warp_sum(be), 0);
        ga = __shfl_sync(0xffffffffu, warp_sum(ga), 0);
        if (!(fabs(ga) > tol * sqrt(al * be))) continue;
        // the rotation that zeroes the pair's inner product
        const double zeta = (be - al) / (2.0 * ga);
        const double t_ = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
        const double c = 1.0 / sqrt(1.0 + t_ * t_), s = c * t_;
        for (int r = lane; r < m; r += 32) {
          const double x = wp[r], y = wq[r];
          wp[r] = c * x - s * y;
          wq[r] = s * x + c * y;
        }
        mine++;
      }
      grid.sync();
    }
    if (lane == 0 && mine) atomicAdd(&ctl->rotations[par], mine);
    grid.sync();
    const unsigned long long total = *((volatile unsigned long long*)&ctl->rotations[par]);
    grid.sync();
    if (total == 0) break;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->sweeps = sweep + (sweep < max_sweeps ? 1 : 0);
}

// sigma_k = |w_k|, one warp per column
__global__ void k_col_norms(const double* W, int m, double* sigma) {
  const int k = blockIdx.x * kWarps + threadIdx.x / 32, lane = threadIdx.x % 32;
  if (k >= m) return;
  double s = 0.0;
  for (int r = lane; r < m; r += 32) s = fma(W[(size_t)k * m + r], W[(size_t)k * m + r], s);
  s = warp_sum(s);
  if (lane == 0) sigma[k] = sqrt(s);
}

// Decreasing order (ties by index): rank of each sigma, then U_R column
// rank = w_k / sigma_k and sorted sigma.
__global__ void k_sort_normalize(const double* W, const double* sigma, int m, double* UR,
                                 double* sigma_sorted) {
  for (int k = blockIdx.x; k < m; k += gridDim.x) {
    __shared__ int rank_s;
    if (threadIdx.x == 0) rank_s = 0;
    __syncthreads();
    const double sk = sigma[k];
    int cnt = 0;
    for (int j = threadIdx.x; j < m; j += blockDim.x) {
      const double sj = sigma[j];
      cnt += (sj > sk || (sj == sk && j < k)) ? 1 : 0;
    }
    atomicAdd(&rank_s, cnt);
    __syncthreads();
    const int rk = rank_s;
    const double inv = sk > 0.0 ? 1.0 / sk : 0.0;
    for (int r = threadIdx.x; r < m; r += blockDim.x) UR[(size_t)rk * m + r] = W[(size_t)k * m + r] * inv;
    if (threadIdx.x == 0) sigma_sorted[rk] = sk;
    __syncthreads();
  }
}

// ---- U = Q U_R[:, :kept] -------------------------------------------------
// 64 x 64 output tile per block, 16 x 16 threads with 4 x 4 outputs each;
// row_major: out[r * kept + c], else out[c * n + r].
constexpr int kTile = 64, kK = 16;
__global__ void __launch_bounds__(256) k_gemm_u(const double* Q, size_t n, int m, const double* UR,
                                                int kept, double* out, int row_major) {
  __shared__ double qs[kK][kTile + 1];
  __shared__ double us[kK][kTile + 1];
  const size_t r0 = (size_t)blockIdx.x * kTile;
  const int c0 = blockIdx.y * kTile;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc[4][4] = {};
  for (int q0 = 0; q0 < m; q0 += kK) {
    for (int e = threadIdx.x; e < kK * kTile; e += 256) {
      const int kk = e / kTile, rr = e % kTile;
      const size_t r = r0 + rr;
      qs[kk][rr] = (q0 + kk < m && r < n) ? Q[(size_t)(q0 + kk) * n + r] : 0.0;
      const int c = c0 + rr;
      us[kk][rr] = (q0 + kk < m && c < kept) ? UR[(size_t)c * m + q0 + kk] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kK; kk++) {
      double a[4], b[4];
#pragma unroll
      for (int x = 0; x < 4; x++) a[x] = qs[kk][ty * 4 + x];
#pragma unroll
      for (int y = 0; y < 4; y++) b[y] = us[kk][tx * 4 + y];
#pragma unroll
      for (int x = 0; x < 4; x++)
#pragma unroll
        for (int y = 0; y < 4; y++) acc[x][y] = fma(a[x], b[y], acc[x][y]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int x = 0; x < 4; x++) {
    const size_t r = r0 + ty * 4 + x;
    if (r >= n) continue;
#pragma unroll
    for (int y = 0; y < 4; y++) {
      const int c = c0 + tx * 4 + y;
      if (c >= kept) continue;
      if (row_major)
        out[r * kept + c] = acc[x][y];
      else
        out[(size_t)c * n + r] = acc[x][y];
    }
  }
}

// ---- y = U^T c and |c - U y| for a row-major U (n x k), diagnostics --------
__global__ void k_utc(const double* U, size_t n, int k, const double* c, double* partial, int nblk) {
  // block b covers rows [b * 2048, ...); warp w of the block takes columns w, w + 8, ...
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const size_t r0 = (size_t)blockIdx.x * kRowsPerBlock;
  for (int kk = warp; kk < k; kk += kWarps) {
    double s = 0.0;
    for (int t = lane; t < kRowsPerBlock; t += 32) {
      const size_t r = r0 + t;
      if (r < n) s = fma(U[r * k + kk], c[r], s);
    }
    s = warp_sum(s);
    if (lane == 0) partial[(size_t)kk * nblk + blockIdx.x] = s;
  }
}

__global__ void k_resid(const double* U, size_t n, int k, const double* c, const double* y,
                        double* partial) {
  __shared__ double sh[kWarps];
  const size_t r = (size_t)blockIdx.x * kThreads + threadIdx.x;
  double d = 0.0;
  if (r < n) {
    double v = 0.0;
    for (int kk = 0; kk < k; kk++) v = fma(U[r * k + kk], y[kk], v);
    d = c[r] - v;
    d = d * d;
  }
  d = warp_sum(d);
  if (threadIdx.x % 32 == 0) sh[threadIdx.x / 32] = d;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kWarps; w++) s += sh[w];
    partial[blockIdx.x] = s;
  }
}

// ------------------------------------------------------------------ host side
#define SVD_TRY(expr)                                                                    \
  do {                                                                                   \
    cudaError_t e_ = (expr);                                                             \
    if (e_ != cudaSuccess) {                                                             \
      err = std::string(cudaGetErrorString(e_)) + ": " #expr;                            \
      return e_ == cudaErrorMemoryAllocation ? (int)PLUME_ERR_OOM : (int)PLUME_ERR_CUDA; \
    }                                                                                    \
  } while (0)

inline int nblocks_rows(size_t n) { return (int)((n + kRowsPerBlock - 1) / kRowsPerBlock); }

// The device state of one factorisation.
struct Runner {
  size_t n = 0;
  int m = 0;
  cudaStream_t s = nullptr;
  double *A = nullptr, *R = nullptr, *partial = nullptr, *dot = nullptr, *inv = nullptr;
  double *W = nullptr, *sigma = nullptr, *sigma_sorted = nullptr, *UR = nullptr, *U = nullptr;
  JacobiCtl* ctl = nullptr;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  int sweeps = 0;
  bool owns_a = true;  // false: A belongs to a plume_snapshots object
  std::string err;

  ~Runner() {
    if (s) cudaStreamSynchronize(s);
    if (!owns_a) A = nullptr;
    double* bufs[] = {A, R, partial, dot, inv, W, sigma, sigma_sorted, UR, U};
    for (double* b : bufs)
      if (b) cudaFree(b);
    if (ctl) cudaFree(ctl);
    for (auto e : ev)
      if (e) cudaEventDestroy(e);
    if (s) cudaStreamDestroy(s);
  }

  int init(int device, size_t n_, int m_, double* external_a = nullptr) {
    n = n_;
    m = m_;
    if (n < 1 || m < 1) {
      err = "empty snapshot matrix";
      return PLUME_ERR_INVALID;
    }
    if (m > 2048) {  // shared memory of one Gram-Schmidt pass: 72 bytes per later column
      err = "more than 2048 snapshots in one stream";
      return PLUME_ERR_UNSUPPORTED;
    }
    SVD_TRY(cudaSetDevice(device));
    SVD_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    for (auto& e : ev) SVD_TRY(cudaEventCreate(&e));
    const size_t mm = (size_t)m * m;
    if (external_a) {
      A = external_a;
      owns_a = false;
    } else {
      SVD_TRY(cudaMalloc(&A, n * m * sizeof(double)));
    }
    SVD_TRY(cudaMalloc(&R, mm * sizeof(double)));
    SVD_TRY(cudaMalloc(&W, mm * sizeof(double)));
    SVD_TRY(cudaMalloc(&UR, mm * sizeof(double)));
    SVD_TRY(cudaMalloc(&partial, (size_t)m * nblocks_rows(n) * sizeof(double)));
    SVD_TRY(cudaMalloc(&dot, m * sizeof(double)));
    SVD_TRY(cudaMalloc(&inv, sizeof(double)));
    SVD_TRY(cudaMalloc(&sigma, m * sizeof(double)));
    SVD_TRY(cudaMalloc(&sigma_sorted, m * sizeof(double)));
    SVD_TRY(cudaMalloc(&ctl, sizeof(JacobiCtl)));
    SVD_TRY(cudaMemsetAsync(R, 0, mm * sizeof(double), s));
    return PLUME_OK;
  }

  // BIG_MATRIX::outOfCoreQR: A -> Q in place, R upper triangular.
  int qr() {
    const int nblk = nblocks_rows(n);
    const size_t smem_max = ((size_t)m * kWarps + m) * sizeof(double);
    SVD_TRY(cudaFuncSetAttribute(k_dots0, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max));
    SVD_TRY(cudaFuncSetAttribute(k_mgs_pass, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max));
    SVD_TRY(cudaEventRecord(ev[0], s));
    k_dots0<<<nblk, kThreads, (size_t)m * kWarps * sizeof(double), s>>>(A, n, m, partial, nblk);
    SVD_TRY(cudaGetLastError());
    k_reduce<<<(m + kWarps - 1) / kWarps, kThreads, 0, s>>>(partial, nblk, m, dot, 0);
    SVD_TRY(cudaGetLastError());
    k_finalize<<<1, kThreads, 0, s>>>(dot, m, 0, R, inv);
    SVD_TRY(cudaGetLastError());
    for (int i = 0; i < m; i++) {
      const int cnt = m - i - 1;
      const size_t smem = ((size_t)cnt * kWarps + cnt) * sizeof(double);
      k_mgs_pass<<<nblk, kThreads, smem, s>>>(A, n, m, i, R, inv, partial, nblk);
      SVD_TRY(cudaGetLastError());
      if (cnt == 0) break;
      k_reduce<<<(cnt + kWarps - 1) / kWarps, kThreads, 0, s>>>(partial, nblk, cnt, dot, i + 1);
      SVD_TRY(cudaGetLastError());
      k_finalize<<<1, kThreads, 0, s>>>(dot, m, i + 1, R, inv);
      SVD_TRY(cudaGetLastError());
    }
    SVD_TRY(cudaEventRecord(ev[1], s));
    return PLUME_OK;
  }

  // SVD of R: sorted singular values and U_R (column-major m x m).
  int svd_r() {
    const size_t mm = (size_t)m * m;
    SVD_TRY(cudaMemcpyAsync(W, R, mm * sizeof(double), cudaMemcpyDeviceToDevice, s));
    SVD_TRY(cudaMemsetAsync(ctl, 0, sizeof(JacobiCtl), s));
    int dev = 0, sms = 0, per_sm = 0;
    SVD_TRY(cudaGetDevice(&dev));
    SVD_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    SVD_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_jacobi, kThreads, 0));
    const int pairs = (m + (m & 1)) / 2;
    int grid = (pairs + kWarps - 1) / kWarps;
    grid = std::max(1, std::min(grid, std::max(1, per_sm) * sms));
    int max_sweeps = 60;
    double tol = (double)m * 2.220446049250313e-16;  // m * DBL_EPSILON
    double* Wp = W;
    int mm_ = m;
    JacobiCtl* c = ctl;
    void* args[] = {&Wp, &mm_, &c, &max_sweeps, &tol};
    SVD_TRY(cudaLaunchCooperativeKernel((void*)k_jacobi, dim3(grid), dim3(kThreads), args, 0, s));
    k_col_norms<<<(m + kWarps - 1) / kWarps, kThreads, 0, s>>>(W, m, sigma);
    SVD_TRY(cudaGetLastError());
    k_sort_normalize<<<std::min(m, 1024), kThreads, 0, s>>>(W, sigma, m, UR, sigma_sorted);
    SVD_TRY(cudaGetLastError());
    SVD_TRY(cudaEventRecord(ev[2], s));
    JacobiCtl h{};
    SVD_TRY(cudaMemcpyAsync(&h, ctl, sizeof(h), cudaMemcpyDeviceToHost, s));
    SVD_TRY(cudaStreamSynchronize(s));
    sweeps = h.sweeps;
    return PLUME_OK;
  }

  // U = Q U_R[:, :kept]
  int form_u(int kept, bool row_major) {
    if (kept < 1) {
      SVD_TRY(cudaEventRecord(ev[3], s));
      return PLUME_OK;
    }
    SVD_TRY(cudaMalloc(&U, n * kept * sizeof(double)));
    const dim3 grid((unsigned)((n + kTile - 1) / kTile), (unsigned)((kept + kTile - 1) / kTile));
    k_gemm_u<<<grid, 256, 0, s>>>(A, n, m, UR, kept, U, row_major ? 1 : 0);
    SVD_TRY(cudaGetLastError());
    SVD_TRY(cudaEventRecord(ev[3], s));
    return PLUME_OK;
  }

  int pca(std::vector<double>& out) {
    out.resize(m);
    SVD_TRY(cudaMemcpyAsync(out.data(), sigma_sorted, m * sizeof(double), cudaMemcpyDeviceToHost, s));
    SVD_TRY(cudaStreamSynchronize(s));
    for (double& v : out) v = v * v;  // "give back PCA values" (BIG_MATRIX.cpp:316-317)
    return PLUME_OK;
  }

  double ms(int a, int b) {
    float f = 0.f;
    if (cudaEventElapsedTime(&f, ev[a], ev[b]) != cudaSuccess) return 0.0;
    return f;
  }
};

// BIG_MATRIX.cpp:320-326: keep columns until the first PCA ratio below the
// threshold
int kept_columns(const std::vector<double>& pca, double threshold) {
  int keep = 0;
  for (size_t x = 0; x < pca.size(); x++) {
    if (pca[x] / pca[0] < threshold) break;
    keep++;
  }
  return keep;
}

int fail(int code, const std::string& msg) {
  global_error() = msg;
  return code;
}

bool read_dims(const std::string& path, int& rows, int& cols) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) return false;
  const bool ok = fread(&rows, sizeof(int), 1, f) == 1 && fread(&cols, sizeof(int), 1, f) == 1;
  fclose(f);
  return ok;
}

// Streams the first `count` snapshots (n doubles each) of `path` into dst on
// the device through two pinned staging buffers.
int upload_stream(const std::string& path, size_t n, int count, double* dst, cudaStream_t s,
                  std::string& err) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) {
    err = "could not open " + path;
    return PLUME_ERR_IO;
  }
  const size_t total = n * (size_t)count, chunk = (size_t)8 << 20;  // 64 MB of doubles
  double* stage[2] = {nullptr, nullptr};
  cudaEvent_t done[2] = {nullptr, nullptr};
  int rc = PLUME_OK;
  for (int b = 0; b < 2 && rc == PLUME_OK; b++) {
    if (cudaMallocHost(&stage[b], chunk * sizeof(double)) != cudaSuccess ||
        cudaEventCreateWithFlags(&done[b], cudaEventDisableTiming) != cudaSuccess)
      rc = PLUME_ERR_OOM;
  }
  for (size_t off = 0, k = 0; rc == PLUME_OK && off < total; off += chunk, k++) {
    const int b = (int)(k & 1);
    const size_t len = std::min(chunk, total - off);
    if (cudaEventSynchronize(done[b]) != cudaSuccess) rc = PLUME_ERR_CUDA;
    if (rc == PLUME_OK && fread(stage[b], sizeof(double), len, f) != len) {
      err = "stream shorter than its dims file: " + path;
      rc = PLUME_ERR_IO;
    }
    if (rc == PLUME_OK &&
        (cudaMemcpyAsync(dst + off, stage[b], len * sizeof(double), cudaMemcpyHostToDevice, s) != cudaSuccess ||
         cudaEventRecord(done[b], s) != cudaSuccess))
      rc = PLUME_ERR_CUDA;
  }
  cudaStreamSynchronize(s);
  for (int b = 0; b < 2; b++) {
    if (stage[b]) cudaFreeHost(stage[b]);
    if (done[b]) cudaEventDestroy(done[b]);
  }
  fclose(f);
  if (rc == PLUME_ERR_CUDA) err = "copy of " + path + " to the device failed";
  if (rc == PLUME_ERR_OOM) err = "pinned staging buffers";
  return rc;
}

// VECTOR::write (VECTOR.cpp:118-143): int32 size, then the doubles
bool write_vector(const std::string& path, const std::vector<double>& v) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) return false;
  const int size = (int)v.size();
  bool ok = fwrite(&size, sizeof(int), 1, f) == 1 && fwrite(v.data(), sizeof(double), v.size(), f) == v.size();
  return fclose(f) == 0 && ok;
}

// writeFinalU: int32 rows, cols, then the row-major U, from the device in
// pieces through pinned memory
int write_u(const std::string& path, const double* U, size_t n, int kept, cudaStream_t s, std::string& err) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) {
    err = "could not open " + path;
    return PLUME_ERR_IO;
  }
  const int rows = (int)n, cols = kept;
  bool ok = fwrite(&rows, sizeof(int), 1, f) == 1 && fwrite(&cols, sizeof(int), 1, f) == 1;
  const size_t total = n * (size_t)kept, chunk = (size_t)8 << 20;
  double* stage = nullptr;
  int rc = PLUME_OK;
  if (total && cudaMallocHost(&stage, std::min(chunk, total) * sizeof(double)) != cudaSuccess) rc = PLUME_ERR_OOM;
  for (size_t off = 0; rc == PLUME_OK && ok && off < total; off += chunk) {
    const size_t len = std::min(chunk, total - off);
    if (cudaMemcpyAsync(stage, U + off, len * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
      rc = PLUME_ERR_CUDA;
      break;
    }
    ok = fwrite(stage, sizeof(double), len, f) == len;
  }
  if (stage) cudaFreeHost(stage);
  const bool closed = fclose(f) == 0;
  if (rc != PLUME_OK) {
    err = "copy of U from the device failed";
    return rc;
  }
  if (!ok || !closed) {
    err = "write failed: " + path;
    return PLUME_ERR_IO;
  }
  return PLUME_OK;
}

// ---- peeled copies of a handle's field into a snapshot column ---------------
// appendStreams' peelBoundary().flattened() (VECTOR3_FIELD_3D.cpp:3139-3151,
// 3222-3232; FIELD_3D.cpp:6679-6689, 6722-6733): interior cells, x fastest,
// vector components interleaved; FP32 fields widen exactly to FP64.
template <typename T>
__global__ void k_peel(int X, int Y, int Z, const T* a, const T* b, const T* c, int comps, double* out) {
  const long long nx = X - 2, ny = Y - 2, nint = nx * ny * (Z - 2);
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nint;
       k += (long long)gridDim.x * blockDim.x) {
    const long long x = k % nx, t = k / nx, y = t % ny, z = t / ny;
    const size_t cell = (size_t)(x + 1) + (size_t)(y + 1) * X + (size_t)(z + 1) * X * Y;
    if (comps == 1) {
      out[k] = (double)a[cell];
    } else {
      out[3 * k] = (double)a[cell];
      out[3 * k + 1] = (double)b[cell];
      out[3 * k + 2] = (double)c[cell];
    }
  }
}

__global__ void k_sumsq(const double* v, size_t n, double* partial) {
  __shared__ double sh[kWarps];
  double s = 0.0;
  for (size_t r = blockIdx.x * (size_t)blockDim.x + threadIdx.x; r < n; r += (size_t)gridDim.x * blockDim.x)
    s = fma(v[r], v[r], s);
  s = warp_sum(s);
  if (threadIdx.x % 32 == 0) sh[threadIdx.x / 32] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kWarps; w++) t += sh[w];
    partial[blockIdx.x] = t;
  }
}

constexpr int kNormBlocks = 1024;

}  // namespace svd
}  // namespace plume

using namespace plume::svd;

struct plume_snapshots {
  plume_handle* h = nullptr;
  int stream = 0;
  int capacity = 0;
  int count = 0;
  int device = 0;
  size_t n = 0;
  double* A = nullptr;
  double* partial = nullptr;
  double* total = nullptr;
};

namespace {

// The fields of one appendStreams call for a stream (FLUID_3D_MIC.cpp:1402-1461)
int stream_fields(int stream, int fields[2]) {
  switch (stream) {
    case PLUME_STREAM_FINAL: fields[0] = PLUME_F_VELOCITY; return 1;
    case PLUME_STREAM_PREPROJECT: fields[0] = PLUME_F_PREPROJECTION; return 1;
    case PLUME_STREAM_PREDIFFUSE: fields[0] = PLUME_F_PREDIFFUSION; return 1;
    case PLUME_STREAM_PREADVECT: fields[0] = PLUME_F_PREADVECTION; return 1;
    case PLUME_STREAM_IOP: fields[0] = PLUME_F_POST_IOP; return 1;
    case PLUME_STREAM_PRESSURE:
      fields[0] = PLUME_F_PRESSURE;
      fields[1] = PLUME_F_DIVERGENCE;
      return 2;
    default: return 0;
  }
}

}  // namespace

extern "C" {

int plume_snapshots_create(plume_handle* h, int32_t stream, int32_t capacity, plume_snapshots** out) {
  if (!h || !out || capacity < 1 || capacity > 2048) return fail(PLUME_ERR_INVALID, "bad argument");
  int f[2];
  if (!stream_fields(stream, f)) return fail(PLUME_ERR_INVALID, "unknown stream");
  *out = nullptr;
  plume::Engine* e = plume::engine_of(h);
  const plume_params& p = e->params();
  const size_t nint = (size_t)(p.res[0] - 2) * (p.res[1] - 2) * (p.res[2] - 2);
  std::unique_ptr<plume_snapshots> s(new plume_snapshots());
  s->h = h;
  s->stream = stream;
  s->capacity = capacity;
  s->device = p.device;
  s->n = stream == PLUME_STREAM_PRESSURE ? nint : 3 * nint;
  if (cudaSetDevice(p.device) != cudaSuccess ||
      cudaMalloc(&s->A, s->n * (size_t)capacity * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&s->partial, kNormBlocks * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&s->total, sizeof(double)) != cudaSuccess) {
    plume_snapshots_destroy(s.release());
    (void)cudaGetLastError();
    return fail(PLUME_ERR_OOM, "snapshot matrix does not fit on the device");
  }
  *out = s.release();
  return PLUME_OK;
}

void plume_snapshots_destroy(plume_snapshots* s) {
  if (!s) return;
  cudaSetDevice(s->device);
  for (double* b : {s->A, s->partial, s->total})
    if (b) cudaFree(b);
  delete s;
}

int plume_snapshots_append(plume_snapshots* s, int32_t* appended) {
  if (!s) return fail(PLUME_ERR_INVALID, "null snapshots");
  if (appended) *appended = 0;
  plume::Engine* e = plume::engine_of(s->h);
  const plume_params& p = e->params();
  cudaStream_t st = (cudaStream_t)e->stream_handle();
  int f[2];
  const int nf = stream_fields(s->stream, f);
  const bool fp32 = p.precision == PLUME_PREC_FP32;
  for (int k = 0; k < nf; k++) {
    if (s->count >= s->capacity) return fail(PLUME_ERR_STATE, "snapshot capacity reached");
    const void* planes[3] = {nullptr, nullptr, nullptr};
    int comps = 3;
    if (s->stream == PLUME_STREAM_PRESSURE) {
      planes[0] = e->device_field(f[k]);
      comps = 1;
    } else if (!e->device_vector(f[k], planes)) {
      return fail(PLUME_ERR_STATE, "the stream's field is not kept (cache_fields = 0, or no moving step for postIOP)");
    }
    if (!planes[0]) return fail(PLUME_ERR_STATE, "the stream's field is not kept");
    double* colp = s->A + (size_t)s->count * s->n;
    const int grid = (int)std::min<size_t>((s->n / comps + kThreads - 1) / kThreads, 152 * 16);
    if (fp32)
      k_peel<float><<<grid, kThreads, 0, st>>>(p.res[0], p.res[1], p.res[2], (const float*)planes[0],
                                               (const float*)planes[1], (const float*)planes[2], comps, colp);
    else
      k_peel<double><<<grid, kThreads, 0, st>>>(p.res[0], p.res[1], p.res[2], (const double*)planes[0],
                                                (const double*)planes[1], (const double*)planes[2], comps, colp);
    k_sumsq<<<kNormBlocks, kThreads, 0, st>>>(colp, s->n, s->partial);
    k_reduce<<<1, kThreads, 0, st>>>(s->partial, kNormBlocks, 1, s->total, 0);
    double t = 0.0;
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(&t, s->total, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return fail(PLUME_ERR_CUDA, "snapshot copy on the device failed");
    if (std::sqrt(t) > 1e-7) {  // `if (velocity.norm2() > 1e-7)` (FLUID_3D_MIC.cpp:1404)
      s->count++;
      if (appended) ++*appended;
    }
  }
  return PLUME_OK;
}

int plume_snapshots_dims(plume_snapshots* s, int32_t* rows, int32_t* cols) {
  if (!s) return fail(PLUME_ERR_INVALID, "null snapshots");
  if (rows) *rows = s->count;
  if (cols) *cols = (int32_t)s->n;
  return PLUME_OK;
}

int plume_snapshots_download(plume_snapshots* s, double* dst, size_t n) {
  if (!s || !dst || n != s->n * (size_t)s->count) return fail(PLUME_ERR_INVALID, "bad argument");
  if (n && cudaMemcpy(dst, s->A, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail(PLUME_ERR_CUDA, "download failed");
  return PLUME_OK;
}

int plume_snapshots_svd(plume_snapshots* s, double discard_threshold, const char* u_path, const char* pca_path,
                        double* pca_out, int32_t* kept_out, plume_svd_info* info) {
  if (!s) return fail(PLUME_ERR_INVALID, "null snapshots");
  if (s->count < 1) return fail(PLUME_ERR_STATE, "no snapshots held");
  cudaStreamSynchronize((cudaStream_t)plume::engine_of(s->h)->stream_handle());
  Runner r;
  int rc = r.init(s->device, s->n, s->count, s->A);
  if (rc == PLUME_OK) rc = r.qr();
  if (rc == PLUME_OK) rc = r.svd_r();
  std::vector<double> pca;
  if (rc == PLUME_OK) rc = r.pca(pca);
  int kept = 0;
  if (rc == PLUME_OK) {
    kept = kept_columns(pca, discard_threshold);
    rc = r.form_u(u_path ? kept : 0, true);
  }
  if (rc == PLUME_OK && cudaStreamSynchronize(r.s) != cudaSuccess) {
    r.err = "U = Q U_R failed";
    rc = PLUME_ERR_CUDA;
  }
  const int m = s->count;
  s->count = 0;  // the columns now hold Q
  if (rc != PLUME_OK) return fail(rc, r.err);
  const auto t0 = std::chrono::steady_clock::now();
  if (pca_path && !write_vector(pca_path, pca)) return fail(PLUME_ERR_IO, std::string("could not write ") + pca_path);
  if (u_path) {
    rc = write_u(u_path, r.U, s->n, kept, r.s, r.err);
    if (rc != PLUME_OK) return fail(rc, r.err);
  }
  if (pca_out) memcpy(pca_out, pca.data(), m * sizeof(double));
  if (kept_out) *kept_out = kept;
  if (info) {
    info->rows = (int32_t)s->n;
    info->cols = m;
    info->kept = kept;
    info->sweeps = r.sweeps;
    info->ms_qr = r.ms(0, 1);
    info->ms_svd = r.ms(1, 2);
    info->ms_u = r.ms(2, 3);
    info->ms_io = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  return PLUME_OK;
}

}  // extern "C"

extern "C" {

int plume_svd_stream(const char* prefix, const char* reduced_path, const char* scratch_path,
                     double discard_threshold, const char* u_path, const char* pca_path, int32_t device,
                     plume_svd_info* info) {
  if (!prefix || !reduced_path || !scratch_path || !u_path) return fail(PLUME_ERR_INVALID, "null path");
  const auto t0 = std::chrono::steady_clock::now();
  const std::string pre = prefix;
  int drows = 0, dcols = 0;
  if (!read_dims(pre + ".dims", drows, dcols)) return fail(PLUME_ERR_IO, "could not read " + pre + ".dims");
  // the stream holds one snapshot per row: A is (cols x rows) (BIG_MATRIX.cpp:139-141)
  const size_t n = (size_t)dcols;
  const int m = drows;
  Runner r;
  int rc = r.init(device, n, m);
  if (rc == PLUME_OK) rc = upload_stream(pre + ".transpose", n, m, r.A, r.s, r.err);
  const auto t1 = std::chrono::steady_clock::now();
  if (rc == PLUME_OK) rc = r.qr();
  if (rc == PLUME_OK) rc = r.svd_r();
  std::vector<double> pca;
  if (rc == PLUME_OK) rc = r.pca(pca);
  int kept = 0;
  if (rc == PLUME_OK) {
    kept = kept_columns(pca, discard_threshold);
    rc = r.form_u(kept, true);
  }
  if (rc == PLUME_OK && cudaStreamSynchronize(r.s) != cudaSuccess) {
    r.err = "U = Q U_R failed";
    rc = PLUME_ERR_CUDA;
  }
  const auto t2 = std::chrono::steady_clock::now();
  if (rc != PLUME_OK) return fail(rc, r.err);
  // the singular-value file under the scratch path, with the reference's name
  // rule (BIG_MATRIX.cpp:333-338)
  const std::string red = reduced_path, scr = scratch_path;
  std::string svname = pre.size() > red.size() + 1 ? pre.substr(1 + red.size()) : std::string();
  svname = scr + svname + ".singularValues.vector";
  if (!write_vector(svname, pca)) return fail(PLUME_ERR_IO, "could not write " + svname);
  if (pca_path && !write_vector(pca_path, pca)) return fail(PLUME_ERR_IO, std::string("could not write ") + pca_path);
  rc = write_u(u_path, r.U, n, kept, r.s, r.err);
  if (rc != PLUME_OK) return fail(rc, r.err);
  const auto t3 = std::chrono::steady_clock::now();
  if (info) {
    info->rows = (int32_t)n;
    info->cols = m;
    info->kept = kept;
    info->sweeps = r.sweeps;
    info->ms_qr = r.ms(0, 1);
    info->ms_svd = r.ms(1, 2);
    info->ms_u = r.ms(2, 3);
    info->ms_io = std::chrono::duration<double, std::milli>((t1 - t0) + (t3 - t2)).count();
  }
  return PLUME_OK;
}

int plume_svd_columns(const double* columns, int32_t n, int32_t m, double discard_threshold, int32_t device,
                      double* pca_out, double* u, int32_t* kept_out, plume_svd_info* info) {
  if (!columns || !pca_out || n < 1 || m < 1) return fail(PLUME_ERR_INVALID, "bad argument");
  Runner r;
  int rc = r.init(device, (size_t)n, m);
  if (rc == PLUME_OK && cudaMemcpyAsync(r.A, columns, (size_t)n * m * sizeof(double), cudaMemcpyHostToDevice,
                                        r.s) != cudaSuccess) {
    r.err = "copy of the snapshots to the device failed";
    rc = PLUME_ERR_CUDA;
  }
  if (rc == PLUME_OK) rc = r.qr();
  if (rc == PLUME_OK) rc = r.svd_r();
  std::vector<double> pca;
  if (rc == PLUME_OK) rc = r.pca(pca);
  int kept = 0;
  if (rc == PLUME_OK) {
    kept = kept_columns(pca, discard_threshold);
    rc = r.form_u(u ? kept : 0, false);
  }
  if (rc == PLUME_OK && u && kept > 0 &&
      (cudaMemcpyAsync(u, r.U, (size_t)n * kept * sizeof(double), cudaMemcpyDeviceToHost, r.s) != cudaSuccess ||
       cudaStreamSynchronize(r.s) != cudaSuccess)) {
    r.err = "copy of U from the device failed";
    rc = PLUME_ERR_CUDA;
  }
  if (rc != PLUME_OK) return fail(rc, r.err);
  memcpy(pca_out, pca.data(), m * sizeof(double));
  if (kept_out) *kept_out = kept;
  if (info) {
    info->rows = n;
    info->cols = m;
    info->kept = kept;
    info->sweeps = r.sweeps;
    info->ms_qr = r.ms(0, 1);
    info->ms_svd = r.ms(1, 2);
    info->ms_u = r.ms(2, 3);
    info->ms_io = 0;
  }
  return PLUME_OK;
}

int plume_svd_verify(const char* prefix, const char* u_path, int32_t count, int32_t device, double* diffs) {
  if (!prefix || !u_path || !diffs || count < 0) return fail(PLUME_ERR_INVALID, "bad argument");
  const std::string pre = prefix;
  int drows = 0, dcols = 0;
  if (!read_dims(pre + ".dims", drows, dcols)) return fail(PLUME_ERR_IO, "could not read " + pre + ".dims");
  FILE* f = fopen(u_path, "rb");
  if (!f) return fail(PLUME_ERR_IO, std::string("could not open ") + u_path);
  int urows = 0, ucols = 0;
  const bool hdr = fread(&urows, sizeof(int), 1, f) == 1 && fread(&ucols, sizeof(int), 1, f) == 1;
  if (!hdr || urows != dcols || ucols < 0) {
    fclose(f);
    return fail(PLUME_ERR_IO, "U file does not match the stream");
  }
  std::vector<double> hu((size_t)urows * ucols);
  const bool full = fread(hu.data(), sizeof(double), hu.size(), f) == hu.size();
  fclose(f);
  if (!full) return fail(PLUME_ERR_IO, "U file is short");
  const size_t n = (size_t)urows;
  const int k = ucols, cnt = std::min(count, drows);
  std::string err;
  cudaStream_t s = nullptr;
  double *dU = nullptr, *dC = nullptr, *part = nullptr, *y = nullptr;
  const int nblk = nblocks_rows(n), rblk = (int)((n + kThreads - 1) / kThreads);
  auto cleanup = [&] {
    if (s) cudaStreamSynchronize(s);
    for (double* b : {dU, dC, part, y})
      if (b) cudaFree(b);
    if (s) cudaStreamDestroy(s);
  };
  int rc = PLUME_OK;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&dU, std::max<size_t>(1, hu.size()) * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&dC, std::max<size_t>(1, n * cnt) * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&part, (size_t)std::max(k, 1) * std::max(nblk, rblk) * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&y, std::max(k, 1) * sizeof(double)) != cudaSuccess)
    rc = PLUME_ERR_OOM;
  if (rc == PLUME_OK && cudaMemcpyAsync(dU, hu.data(), hu.size() * sizeof(double), cudaMemcpyHostToDevice, s) != cudaSuccess)
    rc = PLUME_ERR_CUDA;
  if (rc == PLUME_OK && cnt > 0) rc = upload_stream(pre + ".transpose", n, cnt, dC, s, err);
  std::vector<double> hp((size_t)rblk);
  for (int x = 0; rc == PLUME_OK && x < cnt; x++) {
    const double* c = dC + (size_t)x * n;
    if (k > 0) {
      k_utc<<<nblk, kThreads, 0, s>>>(dU, n, k, c, part, nblk);
      k_reduce<<<(k + kWarps - 1) / kWarps, kThreads, 0, s>>>(part, nblk, k, y, 0);
    }
    k_resid<<<rblk, kThreads, 0, s>>>(dU, n, k, c, y, part);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(hp.data(), part, rblk * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
      rc = PLUME_ERR_CUDA;
      break;
    }
    double t = 0.0;
    for (double v : hp) t += v;
    diffs[x] = std::sqrt(t);
  }
  cleanup();
  if (rc != PLUME_OK) return fail(rc, err.empty() ? std::string("verification on the device failed") : err);
  return PLUME_OK;
}

}  // extern "C"
