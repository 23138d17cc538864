// batch.cpp -- many independent plumes on one GPU (include/plume_batch.h).
//
// Host C++ over the C ABI.  The fused engine (batched.cuh) advances every
// plume in lockstep, one launch per stage; the streams engine keeps each
// instance as a plume_handle with its own CUDA stream, stepped concurrently
// from a pool of host threads.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/plume.h"
#include "../../include/plume_batch.h"
#include "../../include/plume_solver.h"
#include "batched.h"
#include "engine.h"

struct plume_batch {
  int engine = PLUME_BATCH_STREAMS;
  std::vector<plume_handle*> h;         // streams engine
  plume::BatchEngine* fused = nullptr;  // fused engine
  int n = 0;
};

namespace {

uint64_t mix(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
double uniform(uint64_t seed, uint64_t k) { return (mix(mix(seed) + k) >> 11) * (1.0 / 9007199254740992.0); }

int fail(int code, const std::string& msg) {
  plume::global_error() = msg;
  return code;
}

}  // namespace

extern "C" {

int plume_batch_params(uint64_t seed, int32_t index, plume_params* p) {
  if (!p || index < 0) return fail(PLUME_ERR_INVALID, "bad argument");
  static const int kGrids[4][3] = {{32, 32, 32}, {48, 64, 48}, {64, 96, 64}, {96, 128, 96}};
  const uint64_t s = seed + (uint64_t)index;
  plume_default_params(p);
  const int* g = kGrids[(int)(uniform(s, 0) * 4.0) & 3];
  const int X = g[0], Y = g[1], Z = g[2];
  p->res[0] = X;
  p->res[1] = Y;
  p->res[2] = Z;
  for (int k = 0; k < 6; k++) p->bc[k] = 1;
  p->precision = PLUME_PREC_FP32;
  p->criterion = PLUME_CRIT_REL2;
  p->tol = 1e-6;
  p->max_iters = 1000;
  p->source = PLUME_SRC_BOX;
  p->source_noise = 0.05;
  p->seed = s;
  p->buoyancy = 0.5 + 1.5 * uniform(s, 1);
  p->vorticity_eps = 4.0 * uniform(s, 2);
  const int wx = (28 * X) / 48 - (20 * X) / 48, wz = (28 * Z) / 48 - (20 * Z) / 48;
  const double cx = X / 3.0 + (X / 3.0) * uniform(s, 3), cz = Z / 3.0 + (Z / 3.0) * uniform(s, 4);
  p->box_lo[0] = std::max(1, std::min(X - 1 - wx, (int)std::lround(cx - wx / 2.0)));
  p->box_lo[2] = std::max(1, std::min(Z - 1 - wz, (int)std::lround(cz - wz / 2.0)));
  p->box_hi[0] = p->box_lo[0] + wx;
  p->box_hi[2] = p->box_lo[2] + wz;
  p->box_lo[1] = (2 * Y) / 64;
  p->box_hi[1] = (6 * Y) / 64;
  return PLUME_OK;
}

void plume_batch_default_options(plume_batch_options* o) {
  if (!o) return;
  memset(o, 0, sizeof(*o));
  o->engine = PLUME_BATCH_FUSED;
  o->graph = 1;
  o->tune = 1;
  o->tune_cache = nullptr;
}

int plume_batch_create_ex(const plume_params* params, int32_t n, const plume_batch_options* opt,
                          plume_batch** out) {
  if (!params || !out || n < 1) return fail(PLUME_ERR_INVALID, "bad argument");
  plume_batch_options o;
  plume_batch_default_options(&o);
  if (opt) o = *opt;
  if (o.engine != PLUME_BATCH_FUSED && o.engine != PLUME_BATCH_STREAMS)
    return fail(PLUME_ERR_INVALID, "unknown batch engine");
  plume_batch* b = new (std::nothrow) plume_batch();
  if (!b) return fail(PLUME_ERR_OOM, "out of host memory");
  b->engine = o.engine;
  b->n = n;
  if (o.engine == PLUME_BATCH_FUSED) {
    const bool fp64 = params[0].precision == PLUME_PREC_FP64;
    if (!fp64 && params[0].precision != PLUME_PREC_FP32) {
      delete b;
      return fail(PLUME_ERR_INVALID, "unknown precision");
    }
    b->fused = fp64 ? plume::make_batch_engine_f64() : plume::make_batch_engine_f32();
    const int rc = b->fused ? b->fused->init(params, n, o) : (int)PLUME_ERR_OOM;
    if (rc != PLUME_OK) {
      const std::string why = b->fused ? b->fused->last_error() : std::string("out of host memory");
      plume_batch_destroy(b);
      return fail(rc, why);
    }
    *out = b;
    return PLUME_OK;
  }
  for (int i = 0; i < n; i++) {
    plume_handle* h = nullptr;
    const int rc = plume_create(&params[i], &h);
    if (rc != PLUME_OK) {
      const std::string why = "instance " + std::to_string(i) + ": " + plume_last_error(nullptr);
      plume_batch_destroy(b);
      return fail(rc, why);
    }
    // concurrent instances interleave better with host-driven CG loops than
    // with one conditional graph launch per solve (measured: 1.8e8 vs 1.1e8
    // cell-steps/s for the 64-plume batch)
    plume::engine_of(h)->use_cg_graph(false);
    b->h.push_back(h);
  }
  *out = b;
  return PLUME_OK;
}

int plume_batch_create(const plume_params* params, int32_t n, plume_batch** out) {
  return plume_batch_create_ex(params, n, nullptr, out);
}

void plume_batch_destroy(plume_batch* b) {
  if (!b) return;
  for (plume_handle* h : b->h) plume_destroy(h);
  delete b->fused;
  delete b;
}

int plume_batch_size(plume_batch* b, int32_t* n) {
  if (!b || !n) return fail(PLUME_ERR_INVALID, "bad argument");
  *n = (int32_t)b->n;
  return PLUME_OK;
}

int plume_batch_handle(plume_batch* b, int32_t i, plume_handle** h) {
  if (!b || !h) return fail(PLUME_ERR_INVALID, "bad argument");
  if (b->engine == PLUME_BATCH_FUSED)
    return fail(PLUME_ERR_STATE, "a fused batch has no per-plume handles (plume_batch_download)");
  if (i < 0 || i >= (int32_t)b->h.size()) return fail(PLUME_ERR_INVALID, "bad instance");
  *h = b->h[i];
  return PLUME_OK;
}

int plume_batch_download(plume_batch* b, int32_t i, int32_t field, double* dst, size_t n) {
  if (!b || i < 0 || i >= b->n) return fail(PLUME_ERR_INVALID, "bad instance");
  if (b->engine == PLUME_BATCH_FUSED) {
    const int rc = b->fused->download(i, field, dst, n);
    return rc == PLUME_OK ? rc : fail(rc, b->fused->last_error());
  }
  const int rc = plume_download(b->h[i], field, dst, n);
  return rc == PLUME_OK ? rc : fail(rc, plume_last_error(b->h[i]));
}

int plume_batch_tuning(plume_batch* b, char* json, size_t cap, size_t* len) {
  if (!b) return fail(PLUME_ERR_INVALID, "bad argument");
  const std::string s = b->engine == PLUME_BATCH_FUSED ? b->fused->tuning_json() : std::string("{}");
  if (len) *len = s.size();
  if (json && cap > 0) {
    const size_t k = std::min(cap - 1, s.size());
    memcpy(json, s.data(), k);
    json[k] = 0;
  }
  return PLUME_OK;
}

int plume_batch_run(plume_batch* b, int32_t first_step, int32_t steps, int32_t threads, double* seconds,
                    plume_step_stats* stats) {
  if (!b || steps < 0 || threads < 0) return fail(PLUME_ERR_INVALID, "bad argument");
  if (b->engine == PLUME_BATCH_FUSED) {
    const int rc = b->fused->run(first_step, steps, seconds, stats);
    return rc == PLUME_OK ? rc : fail(rc, b->fused->last_error());
  }
  const int n = (int)b->h.size();
  const int T = threads == 0 ? n : std::min(threads, n);
  std::vector<int> rcs(n, PLUME_OK);
  std::vector<std::string> errs(n);
  const auto t0 = std::chrono::steady_clock::now();
  // thread t owns instances t, t+T, ...; it advances them round-robin one step
  // at a time, so every instance makes progress while another one's solve waits
  auto worker = [&](int t) {
    for (int s = 0; s < steps; s++)
      for (int i = t; i < n; i += T) {
        if (rcs[i] != PLUME_OK) continue;
        int rc = plume_add_source(b->h[i], first_step + s);
        if (rc == PLUME_OK) rc = plume_step(b->h[i], stats ? &stats[(size_t)i * steps + s] : nullptr);
        if (rc != PLUME_OK) {
          rcs[i] = rc;
          errs[i] = plume_last_error(b->h[i]);
        }
      }
    for (int i = t; i < n; i += T)
      if (rcs[i] == PLUME_OK && plume_sync(b->h[i]) != PLUME_OK) {
        rcs[i] = PLUME_ERR_CUDA;
        errs[i] = plume_last_error(b->h[i]);
      }
  };
  std::vector<std::thread> pool;
  for (int t = 0; t < T; t++) pool.emplace_back(worker, t);
  for (auto& th : pool) th.join();
  if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  for (int i = 0; i < n; i++)
    if (rcs[i] != PLUME_OK) return fail(rcs[i], "instance " + std::to_string(i) + ": " + errs[i]);
  return PLUME_OK;
}

}  // extern "C"
