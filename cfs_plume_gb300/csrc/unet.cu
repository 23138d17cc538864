// unet.cu -- the learned warm start: network runtime, pair store, trainer and
// their C ABI (include/plume_net.h).  Device code lives in unet_kernels.cuh.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "../../include/plume.h"
#include "../../include/plume_net.h"
#include "../../include/plume_solver.h"
#include "engine.h"
#include "unet.h"
#include "unet_kernels.cuh"
#include "unet_tc.cuh"

namespace plume {
namespace unet {

namespace {

constexpr int kThreads = 256;
constexpr int kMaxBlocks = 152 * 8;

inline int blocks_for(long long n) {
  long long b = (n + kThreads - 1) / kThreads;
  if (b < 1) b = 1;
  if (b > kMaxBlocks) b = kMaxBlocks;
  return (int)b;
}
inline size_t al(size_t n) { return (n + 255) & ~(size_t)255; }

std::string cuda_msg(cudaError_t e, const char* what) {
  std::string s = cudaGetErrorString(e);
  s += ": ";
  s += what;
  return s;
}

// A failed CUDA call: its text goes to `err` and to the calling thread's
// error detail (plume_last_error(NULL)), which the handle-less C entry points
// below report.
#define NT(x)                                     \
  do {                                            \
    cudaError_t e_ = (x);                         \
    if (e_ != cudaSuccess) {                      \
      err = cuda_msg(e_, #x);                     \
      plume::global_error() = err;                \
      (void)cudaGetLastError();                   \
      return e_ == cudaErrorMemoryAllocation ? PLUME_ERR_OOM : PLUME_ERR_CUDA; \
    }                                             \
  } while (0)
#define NT_LAUNCH() NT(cudaGetLastError())

// The ten 3x3x3 convolutions: input channels, output channels, pyramid level.
struct LayerSpec {
  int cin, cout, level;
};
enum { E1A, E1B, E2A, E2B, B3A, B3B, D2A, D2B, D1A, D1B, NCONV };
constexpr LayerSpec kLayers[NCONV] = {{16, 16, 0}, {16, 16, 0}, {16, 32, 1}, {32, 32, 1}, {32, 64, 2},
                                      {64, 64, 2}, {96, 32, 1}, {32, 32, 1}, {48, 16, 0}, {16, 16, 0}};

Dims make_dims(int X, int Y, int Z) {
  Dims d;
  d.X = X;
  d.Y = Y;
  d.Z = Z;
  d.cells = (long long)X * Y * Z;
  return d;
}

View view(bf16* p, int C, const Dims& d, int co = 0) {
  View v;
  v.p = p;
  v.cs = C;
  v.co = co;
  v.bs = d.cells * C;
  return v;
}
View none() {
  View v;
  v.p = nullptr;
  v.cs = 0;
  v.co = 0;
  v.bs = 0;
  return v;
}

// ---------------------------------------------------------- launch helpers
template <int CI, int CO, int MF>
cudaError_t conv_t(const Dims& d, int batch, View in, const uint2* wf, const float* bias, View out, View mask,
                   int relu, cudaStream_t s) {
  using C = ConvCfg<CI, CO, MF>;
  cudaError_t e =
      cudaFuncSetAttribute(k_conv3<CI, CO, MF>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
  if (e != cudaSuccess) return e;
  dim3 grid(conv_bricks<CI, CO, MF>(d), batch);
  k_conv3<CI, CO, MF><<<grid, 256, C::SMEM, s>>>(d, in, wf, bias, out, mask, relu);
  return cudaGetLastError();
}

// The tensor-core (tcgen05) convolution for a layer shape whose halo brick
// and weights fit in shared memory, launched as a one-CTA cluster (its
// mbarrier commit names the cluster window); false if the shape has none.
template <int CI, int CO>
cudaError_t conv_tc_t(const Dims& d, int batch, View in, const bf16* wpack, const float* bias, View out,
                      View mask, int relu, int* err, cudaStream_t s) {
  using C = TcCfg<CI, CO>;
  cudaError_t e = cudaFuncSetAttribute(k_conv3_tc<CI, CO>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
  if (e != cudaSuccess) return e;
  const long long items =
      (long long)((d.X + C::BX - 1) / C::BX) * ((d.Y + C::BY - 1) / C::BY) * ((d.Z + C::BZ - 1) / C::BZ) * batch;
  // persistent: as many CTAs as shared memory and TMEM (512 columns per SM)
  // keep resident at once
  int dev = 0, sms = 0, per_sm = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_conv3_tc<CI, CO>, 256, C::SMEM)) != cudaSuccess)
    return e;
  per_sm = std::max(1, std::min(per_sm, 512 / C::NCOLS));
  const long long grid = std::min<long long>(items, (long long)sms * per_sm);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)std::max<long long>(1, grid));
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = C::SMEM;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = 1;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_conv3_tc<CI, CO>, d, batch, in, wpack, bias, out, mask, relu, err);
}

// The shapes that run on tcgen05: measured at 128x192x128 (ncu, serialised),
// <32,64> 20.1 us against 29-32 us for the best mma.sync tile, <32,32> 66-68
// against 71-77, <16,32> 45 against 45.  With 16 output channels (N = 16)
// the tensor-core version loses (<16,16> 262 against 167 us, <48,16> 606
// against 424): each MMA re-reads a 4 KB A tile for 8 KFLOP-per-row of work,
// the tensor pipe sits at 7-9 % active and the per-item phases (stage, issue,
// wait, epilogue) of one resident CTA do not overlap, so those layers keep the
// mma.sync kernel.
inline bool conv_tc_supported(int ci, int co) {
  return (ci == 16 && co == 32) || (ci == 32 && co == 32) || (ci == 32 && co == 64);
}

cudaError_t conv_tc(int ci, int co, const Dims& d, int batch, View in, const bf16* wpack, const float* bias,
                    View out, View mask, int relu, int* err, cudaStream_t s) {
  if (ci == 16 && co == 32) return conv_tc_t<16, 32>(d, batch, in, wpack, bias, out, mask, relu, err, s);
  if (ci == 32 && co == 32) return conv_tc_t<32, 32>(d, batch, in, wpack, bias, out, mask, relu, err, s);
  if (ci == 32 && co == 64) return conv_tc_t<32, 64>(d, batch, in, wpack, bias, out, mask, relu, err, s);
  return cudaErrorInvalidValue;
}

// Tile shapes (rows per warp) a layer shape may use: accumulators MF*NF*4 <= 64
// registers and the halo brick within 227 KB of shared memory.
inline int conv_shapes(int ci, int co, int* mfs) {
  int n = 0;
  for (int mf = 1; mf <= 8; mf *= 2) {
    const int by = mf >= 4 ? 8 : 4, bz = 8 * mf / by;
    const long long smem = 18LL * (by + 2) * (bz + 2) * (ci + 8) * 2;
    if (mf * (co / 8) <= 16 && smem <= 227 * 1024) mfs[n++] = mf;
  }
  return n;
}

cudaError_t conv(int ci, int co, int mf, const Dims& d, int batch, View in, const uint2* wf, const float* bias,
                 View out, View mask, int relu, cudaStream_t s) {
#define PL_CONV(A, B, M) \
  if (ci == A && co == B && mf == M) return conv_t<A, B, M>(d, batch, in, wf, bias, out, mask, relu, s);
#define PL_CONV4(A, B) PL_CONV(A, B, 1) PL_CONV(A, B, 2) PL_CONV(A, B, 4) PL_CONV(A, B, 8)
#define PL_CONV3(A, B) PL_CONV(A, B, 1) PL_CONV(A, B, 2) PL_CONV(A, B, 4)
#define PL_CONV2(A, B) PL_CONV(A, B, 1) PL_CONV(A, B, 2)
  PL_CONV4(16, 16)
  PL_CONV3(16, 32)
  PL_CONV4(32, 16)
  PL_CONV3(32, 32)
  PL_CONV2(32, 64)
  PL_CONV3(64, 32)
  PL_CONV2(64, 64)
  PL_CONV3(96, 32)
  PL_CONV(32, 96, 1)
  PL_CONV4(48, 16)
  PL_CONV2(16, 48)
#undef PL_CONV4
#undef PL_CONV3
#undef PL_CONV2
#undef PL_CONV
  return cudaErrorInvalidValue;
}

// weight-gradient split count for a layer: about two CTAs per SM in total
template <int CI, int CO, int GO>
int wgrad_splits(const Dims& d, int batch) {
  using C = WgCfg<CI, CO, GO>;
  const long long items =
      (long long)((d.X + 15) / 16) * ((d.Y + C::BY - 1) / C::BY) * ((d.Z + C::BZ - 1) / C::BZ) * batch;
  long long n = 304 / C::NGROUPS;
  if (n < 1) n = 1;
  if (n > items) n = items;
  return (int)n;
}

template <int CI, int CO, int GO>
cudaError_t wgrad_t(const Dims& d, int batch, View x, View g, float* part, float* dw, cudaStream_t s) {
  using C = WgCfg<CI, CO, GO>;
  cudaError_t e =
      cudaFuncSetAttribute(k_conv3_wgrad<CI, CO, GO>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
  if (e != cudaSuccess) return e;
  const int ns = wgrad_splits<CI, CO, GO>(d, batch);
  k_conv3_wgrad<CI, CO, GO><<<dim3(ns, C::NGROUPS), 256, C::SMEM, s>>>(d, batch, x, g, part);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const long long n = 27LL * CI * CO;
  k_sum_parts<<<blocks_for(n), kThreads, 0, s>>>(part, ns, n, dw, 0);
  return cudaGetLastError();
}

cudaError_t wgrad(int ci, int co, const Dims& d, int batch, View x, View g, float* part, float* dw,
                  cudaStream_t s) {
#define PL_WG(A, B, G) \
  if (ci == A && co == B) return wgrad_t<A, B, G>(d, batch, x, g, part, dw, s);
  PL_WG(16, 16, 27)
  PL_WG(16, 32, 27)
  PL_WG(32, 32, 14)
  PL_WG(32, 64, 9)
  PL_WG(64, 64, 6)
  PL_WG(96, 32, 6)
  PL_WG(48, 16, 27)
#undef PL_WG
  return cudaErrorInvalidValue;
}

// largest partial-sum buffer any layer's weight gradient needs (floats)
size_t wgrad_part_floats() { return (size_t)304 * 27 * 96 * 64; }

}  // namespace

// --------------------------------------------------------------- workspace
struct Workspace {
  Dims d[3];
  int batch = 0;
  bool train = false;
  char* arena = nullptr;
  // activations
  bf16 *xin = nullptr, *e1a = nullptr, *cat1 = nullptr, *d1a = nullptr, *d1b = nullptr;
  bf16 *p1 = nullptr, *e2a = nullptr, *cat2 = nullptr, *d2a = nullptr, *d2b = nullptr;
  bf16 *p2 = nullptr, *b3a = nullptr, *b3b = nullptr;
  // gradients with respect to layer outputs / pre-activations
  bf16 *g_d1b = nullptr, *g_d1a = nullptr, *g_cat1 = nullptr, *g_e1b = nullptr, *g_e1a = nullptr;
  bf16 *g_p1 = nullptr, *g_d2b = nullptr, *g_d2a = nullptr, *g_cat2 = nullptr, *g_e2b = nullptr,
       *g_e2a = nullptr;
  bf16 *g_p2 = nullptr, *g_b3b = nullptr, *g_b3a = nullptr;
  float *y = nullptr, *t = nullptr, *gy = nullptr, *host_in = nullptr, *ebuf = nullptr;
  float* part = nullptr;  // weight-gradient partial sums
  float* misc = nullptr;  // bias / loss / output-layer partial sums
  double* dpart = nullptr;
  float* scale = nullptr;
  double* loss_acc = nullptr;
  int* idx = nullptr;

  ~Workspace() {
    if (arena) cudaFree(arena);
  }

  int alloc(const int res[3], int nb, bool with_grads, std::string& err) {
    for (int k = 0; k < 3; k++)
      if (res[k] < 4 || res[k] % 4 != 0) {
        err = "network grids need every dimension a multiple of 4 (two 2x pooling levels)";
        return PLUME_ERR_INVALID;
      }
    d[0] = make_dims(res[0], res[1], res[2]);
    d[1] = make_dims(res[0] / 2, res[1] / 2, res[2] / 2);
    d[2] = make_dims(res[0] / 4, res[1] / 4, res[2] / 4);
    batch = nb;
    train = with_grads;
    struct Req {
      void** p;
      size_t bytes;
    };
    std::vector<Req> req;
    auto act = [&](bf16** p, int C, int lvl) { req.push_back({(void**)p, al(d[lvl].cells * C * nb * 2)}); };
    act(&xin, 16, 0);
    act(&e1a, 16, 0);
    act(&cat1, 48, 0);
    act(&d1a, 16, 0);
    act(&d1b, 16, 0);
    act(&p1, 16, 1);
    act(&e2a, 32, 1);
    act(&cat2, 96, 1);
    act(&d2a, 32, 1);
    act(&d2b, 32, 1);
    act(&p2, 32, 2);
    act(&b3a, 64, 2);
    act(&b3b, 64, 2);
    const size_t n1 = (size_t)d[0].cells * nb;
    req.push_back({(void**)&y, al(n1 * 4)});
    req.push_back({(void**)&host_in, al(n1 * 4)});
    req.push_back({(void**)&dpart, al(kMaxBlocks * 8)});
    req.push_back({(void**)&scale, al(16)});
    req.push_back({(void**)&loss_acc, al(16)});
    if (with_grads) {
      act(&g_d1b, 16, 0);
      act(&g_d1a, 16, 0);
      act(&g_cat1, 48, 0);
      act(&g_e1b, 16, 0);
      act(&g_e1a, 16, 0);
      act(&g_p1, 16, 1);
      act(&g_d2b, 32, 1);
      act(&g_d2a, 32, 1);
      act(&g_cat2, 96, 1);
      act(&g_e2b, 32, 1);
      act(&g_e2a, 32, 1);
      act(&g_p2, 32, 2);
      act(&g_b3b, 64, 2);
      act(&g_b3a, 64, 2);
      req.push_back({(void**)&t, al(n1 * 4)});
      req.push_back({(void**)&gy, al(n1 * 4)});
      req.push_back({(void**)&ebuf, al(n1 * 4)});
      req.push_back({(void**)&part, al(wgrad_part_floats() * 4)});
      req.push_back({(void**)&misc, al((size_t)kMaxBlocks * 64 * 4)});
      req.push_back({(void**)&idx, al((size_t)nb * 4)});
    }
    size_t total = 0;
    for (auto& r : req) total += r.bytes;
    NT(cudaMalloc((void**)&arena, total));
    char* cur = arena;
    for (auto& r : req) {
      *r.p = cur;
      cur += r.bytes;
    }
    return PLUME_OK;
  }
};

// ---------------------------------------------------------------- network
class Net : public NetRuntime {
 public:
  ~Net() override {
    if (params_) cudaFree(params_);
    for (bf16* p : wtc_)
      if (p) cudaFree(p);
    if (tc_err_host_) cudaFreeHost(tc_err_host_);
    if (s_) cudaStreamDestroy(s_);
  }

  int init(uint64_t seed, int device, std::string& err) {
    device_ = device;
    NT(cudaSetDevice(device));
    NT(cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking));
    // parameter layout
    long long n = 0;
    for (int l = 0; l < NCONV; l++) {
      woff_[l] = n;
      n += 27LL * kLayers[l].cin * kLayers[l].cout;
      boff_[l] = n;
      n += kLayers[l].cout;
    }
    woff_[NCONV] = n;
    n += 16;
    boff_[NCONV] = n;
    n += 1;
    nparams_ = n;
    size_t frag = 0;
    for (int l = 0; l < NCONV; l++) frag += al(27LL * kLayers[l].cin * kLayers[l].cout * 2);
    const size_t pbytes = al(n * 4);
    NT(cudaMalloc((void**)&params_, 4 * pbytes + 2 * frag));
    w_ = (float*)params_;
    g_ = (float*)(params_ + pbytes);
    m_ = (float*)(params_ + 2 * pbytes);
    v_ = (float*)(params_ + 3 * pbytes);
    char* cur = params_ + 4 * pbytes;
    for (int l = 0; l < NCONV; l++) {
      const size_t fb = al(27LL * kLayers[l].cin * kLayers[l].cout * 2);
      wf_[l] = (uint2*)cur;
      cur += fb;
      wb_[l] = (uint2*)cur;
      cur += fb;
      if (conv_tc_supported(kLayers[l].cin, kLayers[l].cout))
        NT(cudaMalloc((void**)&wtc_[l], 27LL * kLayers[l].cin * kLayers[l].cout * sizeof(bf16)));
    }
    NT(cudaHostAlloc((void**)&tc_err_host_, sizeof(int), cudaHostAllocMapped));
    *tc_err_host_ = 0;
    NT(cudaHostGetDevicePointer((void**)&tc_err_, tc_err_host_, 0));
    // He-normal weights (fan-in 27*cin; the output layer 16), zero biases.
    // Input channels 1..15 of the first layer carry zeros and keep their
    // weights; only channel 0 (the right-hand side) is drawn.
    std::vector<float> h((size_t)n, 0.f);
    uint64_t st = seed * 0x9E3779B97F4A7C15ULL + 0x632BE59BD9B4E019ULL;
    auto next = [&]() {
      st += 0x9E3779B97F4A7C15ULL;
      uint64_t z = st;
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
      z ^= z >> 31;
      return ((z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    };
    auto normal = [&]() {  // Box-Muller
      const double u1 = next(), u2 = next();
      return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    };
    for (int l = 0; l < NCONV; l++) {
      const int cin = kLayers[l].cin, cout = kLayers[l].cout;
      const int fan = 27 * (l == E1A ? 1 : cin);
      const double sd = std::sqrt(2.0 / fan);
      for (int o = 0; o < 27; o++)
        for (int ci = 0; ci < cin; ci++)
          for (int co = 0; co < cout; co++) {
            const double v = normal() * sd;
            if (l != E1A || ci == 0) h[woff_[l] + ((size_t)o * cin + ci) * cout + co] = (float)v;
          }
    }
    for (int c = 0; c < 16; c++) h[woff_[NCONV] + c] = (float)(normal() * std::sqrt(1.0 / 16));
    NT(cudaMemcpyAsync(w_, h.data(), n * 4, cudaMemcpyHostToDevice, s_));
    NT(cudaMemsetAsync(m_, 0, n * 4, s_));
    NT(cudaMemsetAsync(v_, 0, n * 4, s_));
    NT(cudaStreamSynchronize(s_));
    return prep(s_, err);
  }

  // bf16 fragment copies of every layer's weights (after any change of w_)
  int prep(cudaStream_t s, std::string& err) {
    for (int l = 0; l < NCONV; l++) {
      const int cin = kLayers[l].cin, cout = kLayers[l].cout;
      const long long n = 27LL * cin * cout / 4;  // fragment lanes: 4 elements each
      k_prep_fwd<<<blocks_for(n), kThreads, 0, s>>>(w_ + woff_[l], cin, cout, wf_[l]);
      NT_LAUNCH();
      if (wtc_[l]) {
        k_prep_tc<<<blocks_for(27LL * cin * cout), kThreads, 0, s>>>(w_ + woff_[l], cin, cout, wtc_[l]);
        NT_LAUNCH();
      }
      if (l != E1A) {
        k_prep_bwd<<<blocks_for(n), kThreads, 0, s>>>(w_ + woff_[l], cin, cout, wb_[l]);
        NT_LAUNCH();
      }
    }
    return PLUME_OK;
  }

  // forward pass from ws.xin to ws.y
  int forward(Workspace& ws, int nb, cudaStream_t s, std::string& err) {
    const Dims* d = ws.d;
    const View no = none();
    auto cv = [&](int l, View in, View out) {
      if (wtc_[l] && !tc_off_)
        return conv_tc(kLayers[l].cin, kLayers[l].cout, d[kLayers[l].level], nb, in, wtc_[l], w_ + boff_[l], out,
                       no, 1, tc_err_, s);
      return conv_tuned(kLayers[l].cin, kLayers[l].cout, d[kLayers[l].level], nb, in, wf_[l], w_ + boff_[l], out,
                        no, 1, s);
    };
    NT(cv(E1A, view(ws.xin, 16, d[0]), view(ws.e1a, 16, d[0])));
    NT(cv(E1B, view(ws.e1a, 16, d[0]), view(ws.cat1, 48, d[0], 32)));
    k_pool<<<blocks_for(d[1].cells * 2 * nb), kThreads, 0, s>>>(d[0], d[1], nb, 16, view(ws.cat1, 48, d[0], 32),
                                                                view(ws.p1, 16, d[1]));
    NT_LAUNCH();
    NT(cv(E2A, view(ws.p1, 16, d[1]), view(ws.e2a, 32, d[1])));
    NT(cv(E2B, view(ws.e2a, 32, d[1]), view(ws.cat2, 96, d[1], 64)));
    k_pool<<<blocks_for(d[2].cells * 4 * nb), kThreads, 0, s>>>(d[1], d[2], nb, 32, view(ws.cat2, 96, d[1], 64),
                                                                view(ws.p2, 32, d[2]));
    NT_LAUNCH();
    NT(cv(B3A, view(ws.p2, 32, d[2]), view(ws.b3a, 64, d[2])));
    NT(cv(B3B, view(ws.b3a, 64, d[2]), view(ws.b3b, 64, d[2])));
    k_upsample<<<blocks_for(d[1].cells * 8 * nb), kThreads, 0, s>>>(d[1], d[2], nb, 64, view(ws.b3b, 64, d[2]),
                                                                    view(ws.cat2, 96, d[1], 0));
    NT_LAUNCH();
    NT(cv(D2A, view(ws.cat2, 96, d[1]), view(ws.d2a, 32, d[1])));
    NT(cv(D2B, view(ws.d2a, 32, d[1]), view(ws.d2b, 32, d[1])));
    k_upsample<<<blocks_for(d[0].cells * 4 * nb), kThreads, 0, s>>>(d[0], d[1], nb, 32, view(ws.d2b, 32, d[1]),
                                                                    view(ws.cat1, 48, d[0], 0));
    NT_LAUNCH();
    NT(cv(D1A, view(ws.cat1, 48, d[0]), view(ws.d1a, 16, d[0])));
    NT(cv(D1B, view(ws.d1a, 16, d[0]), view(ws.d1b, 16, d[0])));
    k_out_fwd<<<blocks_for(d[0].cells * nb), kThreads, 0, s>>>(d[0].cells, nb, view(ws.d1b, 16, d[0]),
                                                               w_ + woff_[NCONV], ws.y);
    NT_LAUNCH();
    return PLUME_OK;
  }

  // Loss of ws.y against ws.t over interior cells, its sum added to
  // ws.loss_acc and d(sum * inv_count)/dy in ws.gy.  kind 0: squared error;
  // kind 1: energy norm e^T A e of the error (+ 1e-4 e^T e, which pins the
  // constant mode the closed-box operator does not see).
  int loss(Workspace& ws, int nb, int kind, double inv_count, cudaStream_t s, std::string& err) {
    const Dims* d = ws.d;
    const long long n1 = d[0].cells * nb;
    const int lb = blocks_for(n1);
    if (kind == 1) {
      k_err<<<lb, kThreads, 0, s>>>(d[0], nb, ws.y, ws.t, ws.ebuf);
      NT_LAUNCH();
      k_loss_energy<<<lb, kThreads, 0, s>>>(d[0], nb, ws.ebuf, ws.gy, (float)inv_count, 1e-4f, ws.misc);
    } else {
      k_loss<<<lb, kThreads, 0, s>>>(d[0], nb, ws.y, ws.t, ws.gy, (float)inv_count, ws.misc);
    }
    NT_LAUNCH();
    k_sum_parts<<<1, 32, 0, s>>>(ws.misc, lb, 1, ws.misc + kMaxBlocks * 64 - 1, 0);
    NT_LAUNCH();
    k_add_to_double<<<1, 1, 0, s>>>(ws.misc + kMaxBlocks * 64 - 1, ws.loss_acc);
    NT_LAUNCH();
    return PLUME_OK;
  }

  // loss (see loss()) and the gradient of the mean loss in g_ (every
  // parameter written)
  int backward(Workspace& ws, int nb, int kind, double inv_count, cudaStream_t s, std::string& err) {
    const Dims* d = ws.d;
    const long long n1 = d[0].cells * nb;
    int lrc = loss(ws, nb, kind, inv_count, s, err);
    if (lrc != PLUME_OK) return lrc;
    const int ob = blocks_for(n1);
    k_out_bwd<<<ob, kThreads, 0, s>>>(d[0].cells, nb, view(ws.d1b, 16, d[0]), w_ + woff_[NCONV], ws.gy,
                                      view(ws.g_d1b, 16, d[0]), ws.misc);
    NT_LAUNCH();
    k_sum_parts<<<1, 32, 0, s>>>(ws.misc, ob, 17, g_ + woff_[NCONV], 0);
    NT_LAUNCH();

    auto wg = [&](int l, View x, View g) -> int {
      const Dims& dd = d[kLayers[l].level];
      NT(wgrad(kLayers[l].cin, kLayers[l].cout, dd, nb, x, g, ws.part, g_ + woff_[l], s));
      const int cb = blocks_for(dd.cells * nb / 8 + 1);
      k_chan_sum<<<cb, kThreads, 0, s>>>(g, kLayers[l].cout, dd.cells, nb, ws.misc);
      NT_LAUNCH();
      k_sum_parts<<<1, 64, 0, s>>>(ws.misc, cb, kLayers[l].cout, g_ + boff_[l], 0);
      NT_LAUNCH();
      return PLUME_OK;
    };
    // input gradient of layer l: conv with the mirrored weights
    auto dx = [&](int l, View g, View out, View mask) {
      return conv_tuned(kLayers[l].cout, kLayers[l].cin, d[kLayers[l].level], nb, g, wb_[l], nullptr, out, mask, 0,
                        s);
    };
    int rc;
    // level 1, decoder
    if ((rc = wg(D1B, view(ws.d1a, 16, d[0]), view(ws.g_d1b, 16, d[0]))) != PLUME_OK) return rc;
    NT(dx(D1B, view(ws.g_d1b, 16, d[0]), view(ws.g_d1a, 16, d[0]), view(ws.d1a, 16, d[0])));
    if ((rc = wg(D1A, view(ws.cat1, 48, d[0]), view(ws.g_d1a, 16, d[0]))) != PLUME_OK) return rc;
    NT(dx(D1A, view(ws.g_d1a, 16, d[0]), view(ws.g_cat1, 48, d[0]), none()));
    k_upsample_bwd<<<blocks_for(d[1].cells * 4 * nb), kThreads, 0, s>>>(
        d[0], d[1], nb, 32, view(ws.g_cat1, 48, d[0], 0), view(ws.d2b, 32, d[1]), view(ws.g_d2b, 32, d[1]));
    NT_LAUNCH();
    // level 2, decoder
    if ((rc = wg(D2B, view(ws.d2a, 32, d[1]), view(ws.g_d2b, 32, d[1]))) != PLUME_OK) return rc;
    NT(dx(D2B, view(ws.g_d2b, 32, d[1]), view(ws.g_d2a, 32, d[1]), view(ws.d2a, 32, d[1])));
    if ((rc = wg(D2A, view(ws.cat2, 96, d[1]), view(ws.g_d2a, 32, d[1]))) != PLUME_OK) return rc;
    NT(dx(D2A, view(ws.g_d2a, 32, d[1]), view(ws.g_cat2, 96, d[1]), none()));
    k_upsample_bwd<<<blocks_for(d[2].cells * 8 * nb), kThreads, 0, s>>>(
        d[1], d[2], nb, 64, view(ws.g_cat2, 96, d[1], 0), view(ws.b3b, 64, d[2]), view(ws.g_b3b, 64, d[2]));
    NT_LAUNCH();
    // level 3
    if ((rc = wg(B3B, view(ws.b3a, 64, d[2]), view(ws.g_b3b, 64, d[2]))) != PLUME_OK) return rc;
    NT(dx(B3B, view(ws.g_b3b, 64, d[2]), view(ws.g_b3a, 64, d[2]), view(ws.b3a, 64, d[2])));
    if ((rc = wg(B3A, view(ws.p2, 32, d[2]), view(ws.g_b3a, 64, d[2]))) != PLUME_OK) return rc;
    NT(dx(B3A, view(ws.g_b3a, 64, d[2]), view(ws.g_p2, 32, d[2]), none()));
    // level 2, encoder: skip gradient + pooled gradient, masked by e2b
    k_pool_bwd<<<blocks_for(d[1].cells * 4 * nb), kThreads, 0, s>>>(
        d[1], d[2], nb, 32, view(ws.g_p2, 32, d[2]), view(ws.g_cat2, 96, d[1], 64), view(ws.cat2, 96, d[1], 64),
        view(ws.g_e2b, 32, d[1]));
    NT_LAUNCH();
    if ((rc = wg(E2B, view(ws.e2a, 32, d[1]), view(ws.g_e2b, 32, d[1]))) != PLUME_OK) return rc;
    NT(dx(E2B, view(ws.g_e2b, 32, d[1]), view(ws.g_e2a, 32, d[1]), view(ws.e2a, 32, d[1])));
    if ((rc = wg(E2A, view(ws.p1, 16, d[1]), view(ws.g_e2a, 32, d[1]))) != PLUME_OK) return rc;
    NT(dx(E2A, view(ws.g_e2a, 32, d[1]), view(ws.g_p1, 16, d[1]), none()));
    // level 1, encoder
    k_pool_bwd<<<blocks_for(d[0].cells * 2 * nb), kThreads, 0, s>>>(
        d[0], d[1], nb, 16, view(ws.g_p1, 16, d[1]), view(ws.g_cat1, 48, d[0], 32), view(ws.cat1, 48, d[0], 32),
        view(ws.g_e1b, 16, d[0]));
    NT_LAUNCH();
    if ((rc = wg(E1B, view(ws.e1a, 16, d[0]), view(ws.g_e1b, 16, d[0]))) != PLUME_OK) return rc;
    NT(dx(E1B, view(ws.g_e1b, 16, d[0]), view(ws.g_e1a, 16, d[0]), view(ws.e1a, 16, d[0])));
    if ((rc = wg(E1A, view(ws.xin, 16, d[0]), view(ws.g_e1a, 16, d[0]))) != PLUME_OK) return rc;
    return PLUME_OK;
  }

  // Convolution with the tile shape the autotuner chose for this layer shape,
  // grid and batch.  On first use every valid shape runs three times between
  // CUDA events on `s` (after one untimed run) and the fastest is kept; all
  // shapes give the same bits, so the timing runs leave a valid output.
  cudaError_t conv_tuned(int ci, int co, const Dims& d, int nb, View in, const uint2* wf, const float* bias,
                         View out, View mask, int relu, cudaStream_t s) {
    const std::tuple<int, int, int, int, int, int> key(ci, co, d.X, d.Y, d.Z, nb);
    std::lock_guard<std::mutex> lock(tune_mu_);  // handles sharing this network may step concurrently
    auto it = tuned_.find(key);
    if (it != tuned_.end()) return conv(ci, co, it->second, d, nb, in, wf, bias, out, mask, relu, s);
    int mfs[4];
    const int n = conv_shapes(ci, co, mfs);
    int best = mfs[0];
    if (n > 1 && !tune_off_) {
      cudaEvent_t a = nullptr, b = nullptr;
      cudaError_t e = cudaEventCreate(&a);
      if (e == cudaSuccess) e = cudaEventCreate(&b);
      float best_ms = 1e30f;
      for (int k = 0; k < n && e == cudaSuccess; k++) {
        e = conv(ci, co, mfs[k], d, nb, in, wf, bias, out, mask, relu, s);
        if (e == cudaSuccess) e = cudaEventRecord(a, s);
        for (int r = 0; r < 3 && e == cudaSuccess; r++) e = conv(ci, co, mfs[k], d, nb, in, wf, bias, out, mask, relu, s);
        if (e == cudaSuccess) e = cudaEventRecord(b, s);
        if (e == cudaSuccess) e = cudaEventSynchronize(b);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
        if (e == cudaSuccess && ms < best_ms) {
          best_ms = ms;
          best = mfs[k];
        }
      }
      if (a) cudaEventDestroy(a);
      if (b) cudaEventDestroy(b);
      if (e != cudaSuccess) return e;
    }
    tuned_[key] = best;
    return conv(ci, co, best, d, nb, in, wf, bias, out, mask, relu, s);
  }

  int adam_step(int t, float lr, cudaStream_t s, std::string& err) {
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = 1.f - std::pow(b1, (float)t), bc2 = 1.f - std::pow(b2, (float)t);
    k_adam<<<blocks_for(nparams_), kThreads, 0, s>>>(nparams_, w_, g_, m_, v_, lr, b1, b2, 1e-8f, bc1, bc2);
    NT_LAUNCH();
    return prep(s, err);
  }

  // ---- NetRuntime
  void* new_workspace(const int res[3], std::string& err) override {
    if (cudaSetDevice(device_) != cudaSuccess) {
      err = "cudaSetDevice failed";
      return nullptr;
    }
    Workspace* ws = new (std::nothrow) Workspace();
    if (!ws) return nullptr;
    if (ws->alloc(res, 1, false, err) != PLUME_OK) {
      delete ws;
      return nullptr;
    }
    return ws;
  }
  void free_workspace(void* ws) override { delete (Workspace*)ws; }

  int predict(void* wsp, const void* b, void* x, int is_double, void* stream, std::string& err) override {
    Workspace& ws = *(Workspace*)wsp;
    cudaStream_t s = (cudaStream_t)stream;
    const Dims& d = ws.d[0];
    const int nb = blocks_for(d.cells);
    const double count = (double)(d.X - 2) * (d.Y - 2) * (d.Z - 2);
    if (is_double)
      k_sumsq_interior<double><<<nb, kThreads, 0, s>>>(d, (const double*)b, ws.dpart);
    else
      k_sumsq_interior<float><<<nb, kThreads, 0, s>>>(d, (const float*)b, ws.dpart);
    NT_LAUNCH();
    k_rms_scale<<<1, 256, 0, s>>>(ws.dpart, nb, count, ws.scale);
    NT_LAUNCH();
    if (is_double)
      k_input_from_rhs<double><<<nb, kThreads, 0, s>>>(d, (const double*)b, ws.scale, view(ws.xin, 16, d));
    else
      k_input_from_rhs<float><<<nb, kThreads, 0, s>>>(d, (const float*)b, ws.scale, view(ws.xin, 16, d));
    NT_LAUNCH();
    int rc = forward(ws, 1, s, err);
    if (rc != PLUME_OK) return rc;
    if (is_double)
      k_guess_from_output<double><<<nb, kThreads, 0, s>>>(d, ws.y, ws.scale, scale_c_, (double*)x);
    else
      k_guess_from_output<float><<<nb, kThreads, 0, s>>>(d, ws.y, ws.scale, scale_c_, (float*)x);
    NT_LAUNCH();
    return PLUME_OK;
  }

  // scale (2) + input (1) + forward (10 convolutions, 2 pools, 2 upsamplings,
  // output layer) + guess (1)
  int launches_per_predict() const override { return 19; }
  int kind() const override { return kind_; }

  // PLUME_ERR_TIMEOUT (and clears the flag) if a tensor-core convolution's
  // bounded wait expired since the last call; the caller has synchronised
  // the stream the convolutions ran on.
  int take_error(std::string& err) override {
    if (!tc_err_host_ || *(volatile int*)tc_err_host_ == 0) return PLUME_OK;
    *(volatile int*)tc_err_host_ = 0;
    err = "tensor-core convolution: a bounded wait for its MMAs expired (output invalid)";
    plume::global_error() = err;
    return PLUME_ERR_TIMEOUT;
  }

  int device_ = 0;
  cudaStream_t s_ = nullptr;
  char* params_ = nullptr;
  float *w_ = nullptr, *g_ = nullptr, *m_ = nullptr, *v_ = nullptr;
  uint2* wf_[NCONV] = {};
  uint2* wb_[NCONV] = {};
  bf16* wtc_[NCONV] = {};   // tcgen05 B-operand copies (supported shapes only)
  // set by a tensor-core convolution whose wait expired: host memory mapped
  // into the device, read after the stream is synchronised (take_error)
  int* tc_err_host_ = nullptr;
  int* tc_err_ = nullptr;
  bool tc_off_ = getenv("PLUME_CONV_TC") != nullptr && getenv("PLUME_CONV_TC")[0] == '0';
  long long woff_[NCONV + 1] = {}, boff_[NCONV + 1] = {};
  long long nparams_ = 0;
  float scale_c_ = 1.f;
  int kind_ = 0;  // what the network was trained to map (PLUME_PAIRS_*)
  std::map<std::tuple<int, int, int, int, int, int>, int> tuned_;  // tile shape per (cin, cout, grid, batch)
  std::mutex tune_mu_;
  bool tune_off_ = getenv("PLUME_CONV_TUNE_OFF") != nullptr;  // fixed first shape
  std::string err_;
};

// ------------------------------------------------------------- pair store
struct Dataset {
  Dims d{};
  int pairs = 0;
  bf16* in = nullptr;
  float* tgt = nullptr;
  double target_rms = 0;
  double seconds = 0;
  int device = 0;
  int kind = 0;  // PLUME_PAIRS_SOLVE or PLUME_PAIRS_CORRECTION
  ~Dataset() {
    if (in) cudaFree(in);
    if (tgt) cudaFree(tgt);
  }
};

}  // namespace unet
}  // namespace plume

struct plume_net {
  plume::unet::Net net;
};
struct plume_dataset {
  plume::unet::Dataset ds;
};

using plume::global_error;
using namespace plume::unet;

namespace {

int fail(int code, const std::string& msg) {
  global_error() = msg;
  return code;
}

uint64_t mix(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
double uniform(uint64_t seed, uint64_t k) { return (mix(mix(seed) + k) >> 11) * (1.0 / 9007199254740992.0); }

// Host-buffer helpers share one temporary workspace per call.
int host_forward(Net& n, const int32_t res[3], int32_t batch, const float* input, Workspace& ws, std::string& err) {
  const int r[3] = {res[0], res[1], res[2]};
  int rc = ws.alloc(r, batch, true, err);
  if (rc != PLUME_OK) return rc;
  const long long n1 = ws.d[0].cells * batch;
  NT(cudaMemcpyAsync(ws.host_in, input, n1 * 4, cudaMemcpyHostToDevice, n.s_));
  k_input16<<<blocks_for(n1), 256, 0, n.s_>>>(ws.d[0].cells, batch, ws.host_in, view(ws.xin, 16, ws.d[0]));
  NT_LAUNCH();
  return n.forward(ws, batch, n.s_, err);
}

}  // namespace

extern "C" {

int plume_net_create(uint64_t seed, int32_t device, plume_net** out) {
  if (!out) return fail(PLUME_ERR_INVALID, "null output pointer");
  plume_net* h = new (std::nothrow) plume_net();
  if (!h) return fail(PLUME_ERR_OOM, "out of host memory");
  std::string err;
  const int rc = h->net.init(seed, device, err);
  if (rc != PLUME_OK) {
    delete h;
    return fail(rc, err);
  }
  *out = h;
  return PLUME_OK;
}

void plume_net_destroy(plume_net* net) { delete net; }

int plume_net_num_params(plume_net* net, int64_t* n) {
  if (!net || !n) return fail(PLUME_ERR_INVALID, "null argument");
  *n = net->net.nparams_;
  return PLUME_OK;
}

int plume_net_get_params(plume_net* net, float* dst, int64_t n) {
  if (!net || !dst || n != net->net.nparams_) return fail(PLUME_ERR_INVALID, "bad parameter buffer");
  std::string err;
  Net& m = net->net;
  NT(cudaSetDevice(m.device_));
  NT(cudaMemcpyAsync(dst, m.w_, n * 4, cudaMemcpyDeviceToHost, m.s_));
  NT(cudaStreamSynchronize(m.s_));
  return PLUME_OK;
}

int plume_net_set_params(plume_net* net, const float* src, int64_t n) {
  if (!net || !src || n != net->net.nparams_) return fail(PLUME_ERR_INVALID, "bad parameter buffer");
  std::string err;
  Net& m = net->net;
  NT(cudaSetDevice(m.device_));
  NT(cudaMemcpyAsync(m.w_, src, n * 4, cudaMemcpyHostToDevice, m.s_));
  int rc = m.prep(m.s_, err);
  if (rc != PLUME_OK) return fail(rc, err);
  NT(cudaStreamSynchronize(m.s_));
  return PLUME_OK;
}

int plume_net_get_scale(plume_net* net, float* scale) {
  if (!net || !scale) return fail(PLUME_ERR_INVALID, "null argument");
  *scale = net->net.scale_c_;
  return PLUME_OK;
}

int plume_net_set_scale(plume_net* net, float scale) {
  if (!net || !(scale > 0.f)) return fail(PLUME_ERR_INVALID, "scale must be positive");
  net->net.scale_c_ = scale;
  return PLUME_OK;
}

// file: "PLUMENET", int32 version 1, int32 0, int64 n, float scale, float 0, n floats
int plume_net_save(plume_net* net, const char* path) {
  if (!net || !path) return fail(PLUME_ERR_INVALID, "null argument");
  const int64_t n = net->net.nparams_;
  std::vector<float> w((size_t)n);
  int rc = plume_net_get_params(net, w.data(), n);
  if (rc != PLUME_OK) return rc;
  FILE* f = fopen(path, "wb");
  if (!f) return fail(PLUME_ERR_IO, std::string("cannot write ") + path);
  const int32_t hdr[2] = {1, net->net.kind_};
  const float sc[2] = {net->net.scale_c_, 0.f};
  bool ok = fwrite("PLUMENET", 1, 8, f) == 8 && fwrite(hdr, 4, 2, f) == 2 && fwrite(&n, 8, 1, f) == 1 &&
            fwrite(sc, 4, 2, f) == 2 && fwrite(w.data(), 4, (size_t)n, f) == (size_t)n;
  ok = (fclose(f) == 0) && ok;
  return ok ? PLUME_OK : fail(PLUME_ERR_IO, std::string("short write to ") + path);
}

int plume_net_load(plume_net* net, const char* path) {
  if (!net || !path) return fail(PLUME_ERR_INVALID, "null argument");
  FILE* f = fopen(path, "rb");
  if (!f) return fail(PLUME_ERR_IO, std::string("cannot read ") + path);
  char magic[8];
  int32_t hdr[2];
  int64_t n = 0;
  float sc[2];
  bool ok = fread(magic, 1, 8, f) == 8 && memcmp(magic, "PLUMENET", 8) == 0 && fread(hdr, 4, 2, f) == 2 &&
            hdr[0] == 1 && fread(&n, 8, 1, f) == 1 && n == net->net.nparams_ && fread(sc, 4, 2, f) == 2;
  std::vector<float> w(ok ? (size_t)n : 0);
  ok = ok && fread(w.data(), 4, (size_t)n, f) == (size_t)n;
  fclose(f);
  if (!ok) return fail(PLUME_ERR_IO, std::string("not a network file of this layout: ") + path);
  int rc = plume_net_set_params(net, w.data(), n);
  if (rc != PLUME_OK) return rc;
  net->net.kind_ = (hdr[1] == 1) ? 1 : 0;
  return plume_net_set_scale(net, sc[0]);
}

int plume_net_forward(plume_net* net, const int32_t res[3], int32_t batch, const float* input, float* output) {
  if (!net || !res || !input || !output || batch < 1) return fail(PLUME_ERR_INVALID, "bad argument");
  std::string err;
  Net& m = net->net;
  NT(cudaSetDevice(m.device_));
  Workspace ws;
  int rc = host_forward(m, res, batch, input, ws, err);
  if (rc != PLUME_OK) return fail(rc, err);
  NT(cudaMemcpyAsync(output, ws.y, ws.d[0].cells * batch * 4, cudaMemcpyDeviceToHost, m.s_));
  NT(cudaStreamSynchronize(m.s_));
  return m.take_error(err);
}

int plume_net_loss_grad(plume_net* net, const int32_t res[3], int32_t batch, int32_t loss_kind,
                        const float* input, const float* target, double* loss, float* grad) {
  if (!net || !res || !input || !target || !loss || !grad || batch < 1 || loss_kind < 0 || loss_kind > 1)
    return fail(PLUME_ERR_INVALID, "bad argument");
  std::string err;
  Net& m = net->net;
  NT(cudaSetDevice(m.device_));
  Workspace ws;
  int rc = host_forward(m, res, batch, input, ws, err);
  if (rc != PLUME_OK) return fail(rc, err);
  const Dims& d = ws.d[0];
  NT(cudaMemcpyAsync(ws.t, target, d.cells * batch * 4, cudaMemcpyHostToDevice, m.s_));
  NT(cudaMemsetAsync(ws.loss_acc, 0, 8, m.s_));
  const double count = (double)batch * (d.X - 2) * (d.Y - 2) * (d.Z - 2);
  rc = m.backward(ws, batch, loss_kind, 1.0 / count, m.s_, err);
  if (rc != PLUME_OK) return fail(rc, err);
  double sum = 0;
  NT(cudaMemcpyAsync(&sum, ws.loss_acc, 8, cudaMemcpyDeviceToHost, m.s_));
  NT(cudaMemcpyAsync(grad, m.g_, m.nparams_ * 4, cudaMemcpyDeviceToHost, m.s_));
  NT(cudaStreamSynchronize(m.s_));
  *loss = sum / count;
  return m.take_error(err);
}

int plume_dataset_generate(const plume_dataset_spec* spec, plume_dataset** out) {
  if (!spec || !out) return fail(PLUME_ERR_INVALID, "null argument");
  const plume_dataset_spec& sp = *spec;
  if (sp.plumes < 1 || sp.steps < 1 || sp.skip < 0 || sp.skip >= sp.steps || sp.threads < 1 ||
      sp.kind < 0 || sp.kind > 2)
    return fail(PLUME_ERR_INVALID, "plumes, steps, skip, threads or kind out of range");
  for (int k = 0; k < 3; k++)
    if (sp.res[k] < 8 || sp.res[k] % 4 != 0) return fail(PLUME_ERR_INVALID, "grid dimensions must be multiples of 4");
  std::string err;
  NT(cudaSetDevice(sp.device));
  plume_dataset* h = new (std::nothrow) plume_dataset();
  if (!h) return fail(PLUME_ERR_OOM, "out of host memory");
  Dataset& ds = h->ds;
  ds.d = make_dims(sp.res[0], sp.res[1], sp.res[2]);
  ds.device = sp.device;
  ds.kind = sp.kind;
  const int per = sp.steps - sp.skip;
  ds.pairs = sp.plumes * per;
  const size_t cells = (size_t)ds.d.cells;
  if (cudaMalloc((void**)&ds.in, cells * ds.pairs * 2) != cudaSuccess ||
      cudaMalloc((void**)&ds.tgt, cells * ds.pairs * 4) != cudaSuccess) {
    (void)cudaGetLastError();
    delete h;
    return fail(PLUME_ERR_OOM, "pair store does not fit on the device");
  }
  const auto t0 = std::chrono::steady_clock::now();
  const int T = std::min(sp.threads, sp.plumes);
  std::vector<std::string> errs(T);
  std::vector<int> rcs(T, PLUME_OK);
  auto worker = [&](int t) {
    std::string& e = errs[t];
    if (cudaSetDevice(sp.device) != cudaSuccess) {
      rcs[t] = PLUME_ERR_CUDA;
      e = "cudaSetDevice";
      return;
    }
    double* dpart = nullptr;
    float* scale = nullptr;
    const size_t cells_al = al(cells * 4);
    if (cudaMalloc((void**)&dpart, kMaxBlocks * 8 + 256 + (sp.kind != 0 ? 2 * cells_al : 0)) != cudaSuccess) {
      rcs[t] = PLUME_ERR_OOM;
      e = "workspace";
      return;
    }
    scale = (float*)((char*)dpart + kMaxBlocks * 8);
    // correction pairs: the previous pressure and the residual it leaves;
    // iterate pairs: the k-th PCG iterate in its place
    float* p_prev = sp.kind != 0 ? (float*)((char*)dpart + kMaxBlocks * 8 + 256) : nullptr;
    float* r0 = sp.kind != 0 ? (float*)((char*)p_prev + cells_al) : nullptr;
    for (int i = t; i < sp.plumes && rcs[t] == PLUME_OK; i += T) {
      const uint64_t seed = sp.seed + (uint64_t)i;
      plume_params p;
      plume_default_params(&p);
      for (int k = 0; k < 3; k++) p.res[k] = sp.res[k];
      for (int k = 0; k < 6; k++) p.bc[k] = 1;
      p.precision = PLUME_PREC_FP32;
      p.criterion = PLUME_CRIT_REL2;
      p.tol = sp.tol;
      p.max_iters = 1000;
      p.cache_fields = 0;
      p.device = sp.device;
      p.source = PLUME_SRC_BOX;
      p.source_noise = 0.05;
      p.seed = seed;
      p.buoyancy = 0.5 + 1.5 * uniform(seed, 1);
      p.vorticity_eps = 4.0 * uniform(seed, 2);
      // box of the 48x64x48 source scaled to the grid, centre uniform in the
      // middle third of the floor
      const int X = sp.res[0], Y = sp.res[1], Z = sp.res[2];
      const int wx = (28 * X) / 48 - (20 * X) / 48, wz = (28 * Z) / 48 - (20 * Z) / 48;
      const double cx = X / 3.0 + (X / 3.0) * uniform(seed, 3), cz = Z / 3.0 + (Z / 3.0) * uniform(seed, 4);
      p.box_lo[0] = std::max(1, std::min(X - 1 - wx, (int)std::lround(cx - wx / 2.0)));
      p.box_lo[2] = std::max(1, std::min(Z - 1 - wz, (int)std::lround(cz - wz / 2.0)));
      p.box_hi[0] = p.box_lo[0] + wx;
      p.box_hi[2] = p.box_lo[2] + wz;
      p.box_lo[1] = (2 * Y) / 64;
      p.box_hi[1] = (6 * Y) / 64;
      plume_handle* ph = nullptr;
      int rc = plume_create(&p, &ph);
      if (rc != PLUME_OK) {
        rcs[t] = rc;
        e = plume_last_error(nullptr);
        break;
      }
      plume::Engine* eng = plume::engine_of(ph);
      cudaStream_t s = (cudaStream_t)eng->stream_handle();
      const float* b = (const float*)eng->device_field(PLUME_F_DIVERGENCE);
      const float* x = (const float*)eng->device_field(PLUME_F_PRESSURE);
      const int nb = blocks_for(ds.d.cells);
      const double count = (double)(X - 2) * (Y - 2) * (Z - 2);
      if (sp.kind == 1 && cudaMemsetAsync(p_prev, 0, cells * 4, s) != cudaSuccess) rc = PLUME_ERR_CUDA;
      for (int st = 0; st < sp.steps && rc == PLUME_OK; st++) {
        if (sp.kind == 1 && st > 0 &&
            cudaMemcpyAsync(p_prev, x, cells * 4, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
          rc = PLUME_ERR_CUDA;
          e = "copy of the previous pressure";
          break;
        }
        rc = plume_add_source(ph, st);
        plume_step_stats sst;
        if (rc == PLUME_OK) rc = plume_step(ph, sp.kind == 2 ? &sst : nullptr);
        if (rc != PLUME_OK) {
          e = plume_last_error(ph);
          break;
        }
        if (st < sp.skip) continue;
        const size_t slot = (size_t)i * per + (st - sp.skip);
        if (sp.kind == 2) {  // x_k: the same solve from 0, stopped after k iterations
          // k below half the solve's own count, so that x_k is not yet the
          // solution (whose residual the target p - x_k would not solve)
          const int kmax = std::max(1, std::min(32, sst.iterations / 2 - 1));
          const int kits = 1 + (int)(mix(seed * 0x9E3779B97F4A7C15ULL + (uint64_t)st) % (uint64_t)kmax);
          rc = eng->partial_solve(kits, p_prev);
          if (rc != PLUME_OK) {
            e = eng->last_error();
            break;
          }
        }
        if (sp.kind != 0) {  // (r, p - x) with r = b - A x, x = p_prev or x_k
          k_closed_box_residual<float><<<nb, kThreads, 0, s>>>(ds.d, b, p_prev, r0);
          k_sumsq_interior<float><<<nb, kThreads, 0, s>>>(ds.d, r0, dpart);
          k_rms_scale<<<1, 256, 0, s>>>(dpart, nb, count, scale);
          k_store_correction<float><<<nb, kThreads, 0, s>>>(ds.d, r0, x, p_prev, scale, ds.in + slot * cells,
                                                            ds.tgt + slot * cells);
        } else {
          k_sumsq_interior<float><<<nb, kThreads, 0, s>>>(ds.d, b, dpart);
          k_rms_scale<<<1, 256, 0, s>>>(dpart, nb, count, scale);
          k_store_pair<float><<<nb, kThreads, 0, s>>>(ds.d, b, x, scale, ds.in + slot * cells,
                                                      ds.tgt + slot * cells);
        }
        if (cudaGetLastError() != cudaSuccess) {
          rc = PLUME_ERR_CUDA;
          e = "pair store launch";
        }
      }
      if (rc == PLUME_OK && plume_sync(ph) != PLUME_OK) {
        rc = PLUME_ERR_CUDA;
        e = plume_last_error(ph);
      }
      plume_destroy(ph);
      rcs[t] = rc;
    }
    cudaFree(dpart);
  };
  std::vector<std::thread> pool;
  for (int t = 0; t < T; t++) pool.emplace_back(worker, t);
  for (auto& th : pool) th.join();
  for (int t = 0; t < T; t++)
    if (rcs[t] != PLUME_OK) {
      delete h;
      return fail(rcs[t], "pair generation: " + errs[t]);
    }
  // rms of all stored solutions
  {
    double* part = nullptr;
    NT(cudaMalloc((void**)&part, kMaxBlocks * 8));
    const long long n = (long long)cells * ds.pairs;
    const int nb = blocks_for(n);
    k_sumsq_f<<<nb, kThreads>>>(n, ds.tgt, part);
    std::vector<double> hp(nb);
    cudaError_t e1 = cudaMemcpy(hp.data(), part, nb * 8, cudaMemcpyDeviceToHost);
    cudaFree(part);
    if (e1 != cudaSuccess) {
      delete h;
      return fail(PLUME_ERR_CUDA, "pair store reduction");
    }
    double s = 0;
    for (double v : hp) s += v;
    const double interior = (double)(sp.res[0] - 2) * (sp.res[1] - 2) * (sp.res[2] - 2);
    ds.target_rms = std::sqrt(s / (interior * ds.pairs));
  }
  ds.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  *out = h;
  return PLUME_OK;
}

void plume_dataset_destroy(plume_dataset* ds) { delete ds; }

int plume_dataset_info(plume_dataset* ds, int32_t* pairs, double* target_rms, double* seconds) {
  if (!ds) return fail(PLUME_ERR_INVALID, "null dataset");
  if (pairs) *pairs = ds->ds.pairs;
  if (target_rms) *target_rms = ds->ds.target_rms;
  if (seconds) *seconds = ds->ds.seconds;
  return PLUME_OK;
}

int plume_dataset_get_pair(plume_dataset* ds, int32_t index, float* input, float* target) {
  if (!ds || !input || !target || index < 0 || index >= ds->ds.pairs)
    return fail(PLUME_ERR_INVALID, "bad pair index or buffer");
  std::string err;
  const Dataset& d = ds->ds;
  NT(cudaSetDevice(d.device));
  const size_t cells = (size_t)d.d.cells;
  std::vector<uint16_t> tmp(cells);
  NT(cudaMemcpy(tmp.data(), d.in + (size_t)index * cells, cells * 2, cudaMemcpyDeviceToHost));
  for (size_t i = 0; i < cells; i++) {
    const uint32_t u = (uint32_t)tmp[i] << 16;
    memcpy(&input[i], &u, 4);
  }
  NT(cudaMemcpy(target, d.tgt + (size_t)index * cells, cells * 4, cudaMemcpyDeviceToHost));
  return PLUME_OK;
}

int plume_net_train(plume_net* net, plume_dataset* dsh, const plume_train_spec* spec, float* train_loss,
                    float* val_loss, double* seconds) {
  if (!net || !dsh || !spec) return fail(PLUME_ERR_INVALID, "null argument");
  const plume_train_spec& sp = *spec;
  const Dataset& ds = dsh->ds;
  const int ntrain = ds.pairs - sp.val_pairs;
  if (sp.epochs < 1 || sp.batch < 1 || sp.val_pairs < 0 || ntrain < sp.batch || !(sp.lr > 0.f) ||
      sp.loss < 0 || sp.loss > 1)
    return fail(PLUME_ERR_INVALID, "epochs, batch, val_pairs, lr or loss out of range");
  std::string err;
  Net& m = net->net;
  NT(cudaSetDevice(m.device_));
  cudaStream_t s = m.s_;
  Workspace ws;
  const int r[3] = {ds.d.X, ds.d.Y, ds.d.Z};
  int rc = ws.alloc(r, sp.batch, true, err);
  if (rc != PLUME_OK) return fail(rc, err);
  m.scale_c_ = (float)ds.target_rms;
  m.kind_ = ds.kind;
  const float inv_scale = ds.target_rms > 0 ? (float)(1.0 / ds.target_rms) : 1.f;
  const double interior = (double)(r[0] - 2) * (r[1] - 2) * (r[2] - 2);
  int* hidx = nullptr;
  NT(cudaMallocHost((void**)&hidx, sizeof(int) * sp.batch));
  std::vector<int> order(ntrain);
  for (int i = 0; i < ntrain; i++) order[i] = i;
  const int steps_per_epoch = ntrain / sp.batch;
  const long long total_steps = (long long)steps_per_epoch * sp.epochs;
  long long t = 0;
  const auto t0 = std::chrono::steady_clock::now();
  uint64_t rng = mix(sp.seed);
  auto fail_free = [&](int code, const std::string& msg) {
    cudaStreamSynchronize(s);
    cudaFreeHost(hidx);
    return fail(code, msg);
  };
  for (int ep = 0; ep < sp.epochs; ep++) {
    for (int i = ntrain - 1; i > 0; i--) {  // Fisher-Yates with a SplitMix64 stream
      rng = mix(rng);
      const int j = (int)(rng % (uint64_t)(i + 1));
      std::swap(order[i], order[j]);
    }
    if (cudaMemsetAsync(ws.loss_acc, 0, 8, s) != cudaSuccess) return fail_free(PLUME_ERR_CUDA, "memset");
    for (int k = 0; k < steps_per_epoch; k++) {
      // the pinned index buffer is reused: wait for the previous copy
      if (cudaStreamSynchronize(s) != cudaSuccess) return fail_free(PLUME_ERR_CUDA, "training step");
      for (int q = 0; q < sp.batch; q++) hidx[q] = order[k * sp.batch + q];
      if (cudaMemcpyAsync(ws.idx, hidx, sizeof(int) * sp.batch, cudaMemcpyHostToDevice, s) != cudaSuccess)
        return fail_free(PLUME_ERR_CUDA, "index upload");
      k_gather_batch<<<blocks_for(ws.d[0].cells * sp.batch), kThreads, 0, s>>>(
          ws.d[0].cells, sp.batch, ds.in, ds.tgt, ws.idx, inv_scale, view(ws.xin, 16, ws.d[0]), ws.t);
      rc = m.forward(ws, sp.batch, s, err);
      if (rc == PLUME_OK) rc = m.backward(ws, sp.batch, sp.loss, 1.0 / (interior * sp.batch), s, err);
      t += 1;
      const double frac = total_steps > 1 ? (double)(t - 1) / (double)(total_steps - 1) : 1.0;
      const float lr = sp.lr_final + 0.5f * (sp.lr - sp.lr_final) * (float)(1.0 + std::cos(3.141592653589793 * frac));
      if (rc == PLUME_OK) rc = m.adam_step((int)t, lr, s, err);
      if (rc != PLUME_OK) return fail_free(rc, err);
    }
    double sum = 0;
    if (cudaMemcpyAsync(&sum, ws.loss_acc, 8, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return fail_free(PLUME_ERR_CUDA, "loss readback");
    if (train_loss) train_loss[ep] = (float)(sum / (interior * (double)steps_per_epoch * sp.batch));
    if (val_loss) {
      // held-out pairs: forward + loss only (the gradient pass is skipped)
      double vsum = 0;
      int vcount = 0;
      for (int k = 0; k + sp.batch <= sp.val_pairs; k += sp.batch) {
        if (cudaStreamSynchronize(s) != cudaSuccess) return fail_free(PLUME_ERR_CUDA, "validation");
        for (int q = 0; q < sp.batch; q++) hidx[q] = ntrain + k + q;
        cudaMemcpyAsync(ws.idx, hidx, sizeof(int) * sp.batch, cudaMemcpyHostToDevice, s);
        k_gather_batch<<<blocks_for(ws.d[0].cells * sp.batch), kThreads, 0, s>>>(
            ws.d[0].cells, sp.batch, ds.in, ds.tgt, ws.idx, inv_scale, view(ws.xin, 16, ws.d[0]), ws.t);
        rc = m.forward(ws, sp.batch, s, err);
        if (rc != PLUME_OK) return fail_free(rc, err);
        cudaMemsetAsync(ws.loss_acc, 0, 8, s);
        rc = m.loss(ws, sp.batch, sp.loss, 0.0, s, err);
        if (rc != PLUME_OK) return fail_free(rc, err);
        double v = 0;
        cudaMemcpyAsync(&v, ws.loss_acc, 8, cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) return fail_free(PLUME_ERR_CUDA, "validation loss");
        vsum += v;
        vcount += sp.batch;
      }
      val_loss[ep] = vcount ? (float)(vsum / (interior * vcount)) : 0.f;
    }
  }
  if (cudaStreamSynchronize(s) != cudaSuccess) return fail_free(PLUME_ERR_CUDA, "training");
  rc = m.take_error(err);
  if (rc != PLUME_OK) return fail_free(rc, err);
  cudaFreeHost(hidx);
  if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return PLUME_OK;
}

int plume_attach_net(plume_handle* h, plume_net* net) {
  if (!h || !net) return fail(PLUME_ERR_INVALID, "null argument");
  return plume::engine_of(h)->attach_net(&net->net);
}

}  // extern "C"
