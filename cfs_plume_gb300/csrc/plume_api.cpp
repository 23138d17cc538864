// plume_api.cpp -- the C ABI of libplume (include/plume.h).
//
// Thin layer: argument checks, status codes, and the host-side file output.
// All field arithmetic happens in the CUDA engines; there is no CPU path.
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <string>
#include <vector>

#include <cuda_runtime_api.h>

#include "../../include/plume.h"
#include "../../include/plume_box.h"
#include "../../include/plume_solver.h"
#include "engine.h"
#include "state_read.h"
#include "snapshot.h"

// Background writer of one handle: snapshot jobs run in call order on one
// thread, at most two in flight (queued or running); the first error is
// kept until it is reported.  Field buffers are recycled between jobs.
class SnapshotWriter {
 public:
  using FieldSet = std::vector<std::vector<double>>;
  SnapshotWriter() : th_([this] { run(); }) {}
  ~SnapshotWriter() {
    {
      std::lock_guard<std::mutex> l(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    th_.join();  // pending jobs finish first
  }
  std::shared_ptr<FieldSet> field_set() {
    std::lock_guard<std::mutex> l(mu_);
    if (!spare_.empty()) {
      auto f = spare_.back();
      spare_.pop_back();
      return f;
    }
    return std::make_shared<FieldSet>(PLUME_F_COUNT);
  }
  void recycle(std::shared_ptr<FieldSet> f) {
    std::lock_guard<std::mutex> l(mu_);
    if (spare_.size() < 2) spare_.push_back(std::move(f));
  }
  void push(std::function<int(std::string&)> job) {
    std::unique_lock<std::mutex> l(mu_);
    cv_.wait(l, [&] { return inflight_ < 2; });
    ++inflight_;
    q_.push_back(std::move(job));
    cv_.notify_all();
  }
  int take_error(std::string& e, bool wait_all) {
    std::unique_lock<std::mutex> l(mu_);
    if (wait_all) cv_.wait(l, [&] { return inflight_ == 0; });
    const int r = rc_;
    e = err_;
    rc_ = PLUME_OK;
    err_.clear();
    return r;
  }

 private:
  void run() {
    for (;;) {
      std::function<int(std::string&)> job;
      {
        std::unique_lock<std::mutex> l(mu_);
        cv_.wait(l, [&] { return stop_ || !q_.empty(); });
        if (q_.empty()) return;
        job = std::move(q_.front());
        q_.pop_front();
      }
      std::string e;
      const int r = job(e);
      {
        std::lock_guard<std::mutex> l(mu_);
        if (r != PLUME_OK && rc_ == PLUME_OK) {
          rc_ = r;
          err_ = e;
        }
        --inflight_;
      }
      cv_.notify_all();
    }
  }
  std::mutex mu_;
  std::condition_variable cv_;
  std::deque<std::function<int(std::string&)>> q_;
  std::vector<std::shared_ptr<FieldSet>> spare_;
  int inflight_ = 0;
  bool stop_ = false;
  int rc_ = PLUME_OK;
  std::string err_;
  std::thread th_;  // last: started after every other member exists
};

struct plume_handle {
  plume::Engine* eng = nullptr;
  std::string err;
  std::unique_ptr<SnapshotWriter> writer;
};

namespace plume {
Engine* engine_of(plume_handle* h) { return h->eng; }
std::string& global_error() {
  static thread_local std::string e;
  return e;
}
}  // namespace plume

namespace {

int set_err(plume_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}
int from_engine(plume_handle* h, int code) {
  if (code != PLUME_OK) h->err = h->eng->last_error();
  return code;
}
// A handle's engine with the handle's device made current: every call on a
// handle runs on its own GPU, so one thread may drive handles on several
// GPUs (cudaSetDevice returns at once when the device is already current;
// if it fails, the engine's next CUDA call reports the error).
plume::Engine* eng(plume_handle* h) {
  if (cudaSetDevice(h->eng->params().device) != cudaSuccess) (void)cudaGetLastError();
  return h->eng;
}
}  // namespace

extern "C" {

void plume_default_params(plume_params* p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->abi_version = PLUME_ABI_VERSION;
  p->res[0] = 48;  // fluid3D.cpp:313-315
  p->res[1] = 64;
  p->res[2] = 48;
  const int bc[6] = {1, 1, 1, 1, 0, 0};  // fluid3D.cpp:321-327
  for (int k = 0; k < 6; k++) p->bc[k] = bc[k];
  p->dt = 0.1;
  p->buoyancy = (double)0.1f;
  p->vorticity_eps = 0.0;
  p->damping_w = 0.9;
  p->mic_tau = 0.97;
  p->mic_sigma = 0.25;
  p->source = PLUME_SRC_COLUMN;
  p->precision = PLUME_PREC_FP64;
  p->criterion = PLUME_CRIT_REFERENCE;
  p->tol = 1e-10;
  p->max_iters = 1000;
  p->warm_start = PLUME_WARM_ZERO;
  p->cache_fields = 1;
  p->device = 0;
}

int plume_create(const plume_params* p, plume_handle** out) {
  if (!out) return PLUME_ERR_INVALID;
  *out = nullptr;
  if (!p) {
    plume::global_error() = "null params";
    return PLUME_ERR_INVALID;
  }
  if (p->abi_version != PLUME_ABI_VERSION) {
    plume::global_error() = "abi_version mismatch";
    return PLUME_ERR_INVALID;
  }
  if (p->precision != PLUME_PREC_FP64 && p->precision != PLUME_PREC_FP32) {
    plume::global_error() = "unknown precision";
    return PLUME_ERR_INVALID;
  }
  plume_handle* h = new (std::nothrow) plume_handle();
  if (!h) return PLUME_ERR_OOM;
  h->eng = (p->precision == PLUME_PREC_FP64) ? plume::make_engine_f64() : plume::make_engine_f32();
  const int rc = h->eng->init(*p);
  if (rc != PLUME_OK) {
    plume::global_error() = h->eng->last_error();
    delete h->eng;
    delete h;
    return rc;
  }
  *out = h;
  return PLUME_OK;
}

void plume_destroy(plume_handle* h) {
  if (!h) return;
  h->writer.reset();  // waits for pending snapshots
  (void)eng(h);       // frees on the handle's device
  delete h->eng;
  delete h;
}

int plume_add_source(plume_handle* h, int32_t step_index) {
  if (!h) return PLUME_ERR_INVALID;
  return from_engine(h, eng(h)->add_source(step_index));
}

int plume_add_source_values(plume_handle* h, const double* values, size_t n) {
  if (!h) return PLUME_ERR_INVALID;
  return from_engine(h, eng(h)->add_source_values(values, n));
}

int plume_run_timed(plume_handle* h, int32_t first_step_index, int32_t n, double* ms_device,
                    plume_step_stats* stats) {
  if (!h || !ms_device) return PLUME_ERR_INVALID;
  if (n < 0) return set_err(h, PLUME_ERR_INVALID, "negative step count");
  return from_engine(h, eng(h)->run_timed(first_step_index, n, ms_device, stats));
}

int plume_step(plume_handle* h, plume_step_stats* stats) {
  if (!h) return PLUME_ERR_INVALID;
  return from_engine(h, eng(h)->step(stats));
}

int plume_run(plume_handle* h, int32_t first_step_index, int32_t n, plume_step_stats* stats) {
  if (!h) return PLUME_ERR_INVALID;
  if (n < 0) return set_err(h, PLUME_ERR_INVALID, "negative step count");
  return from_engine(h, eng(h)->run(first_step_index, n, stats));
}

int plume_download(plume_handle* h, int32_t field, double* dst, size_t n) {
  if (!h) return PLUME_ERR_INVALID;
  if (field < 0 || field >= PLUME_F_COUNT) return set_err(h, PLUME_ERR_INVALID, "unknown field");
  return from_engine(h, eng(h)->download(field, dst, n));
}

int plume_upload(plume_handle* h, int32_t field, const double* src, size_t n) {
  if (!h) return PLUME_ERR_INVALID;
  if (field < 0 || field >= PLUME_F_COUNT) return set_err(h, PLUME_ERR_INVALID, "unknown field");
  return from_engine(h, eng(h)->upload(field, src, n));
}

int plume_download_obstacles(plume_handle* h, uint8_t* dst, size_t n) {
  if (!h) return PLUME_ERR_INVALID;
  return from_engine(h, eng(h)->download_obstacles(dst, n));
}

int plume_read_state(plume_handle* h, const char* path) {
  if (!h) return PLUME_ERR_INVALID;
  if (!path) return set_err(h, PLUME_ERR_INVALID, "null path");
  int32_t ints[10];
  double consts[7];
  int rc = plume_state_read_header(path, ints, consts);
  if (rc != PLUME_OK) return set_err(h, rc, plume::global_error());
  const plume_params& p = eng(h)->params();
  if (ints[0] != p.res[0] || ints[1] != p.res[1] || ints[2] != p.res[2])
    return set_err(h, PLUME_ERR_INVALID,
                   std::string("the state file's grid ") + std::to_string(ints[0]) + "x" + std::to_string(ints[1]) +
                       "x" + std::to_string(ints[2]) + " is not the handle's");
  // header doubles: dx, totalTime, dt, buoyancy, vorticityEps (lines 1150-1160)
  if (consts[0] != eng(h)->dx() || consts[2] != p.dt || consts[3] != p.buoyancy || consts[4] != p.vorticity_eps)
    return set_err(h, PLUME_ERR_INVALID,
                   "the state file was written with another dx, dt, buoyancy or vorticityEps than the handle's");
  const size_t N = (size_t)p.res[0] * p.res[1] * p.res[2];
  const int scalars[5] = {PLUME_F_DENSITY, PLUME_F_DENSITY_OLD, PLUME_F_HEAT, PLUME_F_HEAT_OLD, PLUME_F_PRESSURE};
  const int vectors[2] = {PLUME_F_VELOCITY, PLUME_F_VELOCITY_OLD};
  std::vector<std::vector<double>> bufs(7);
  plume::StateRequest req;
  for (int k = 0; k < 5; k++) {
    bufs[k].resize(N);
    req.push_back({scalars[k], bufs[k].data(), N});
  }
  for (int k = 0; k < 2; k++) {
    bufs[5 + k].resize(3 * N);
    req.push_back({vectors[k], bufs[5 + k].data(), 3 * N});
  }
  rc = plume::read_state_fields(path, req, nullptr);
  if (rc != PLUME_OK) return set_err(h, rc, plume::global_error());
  for (const plume::StateField& w : req) {
    rc = from_engine(h, eng(h)->upload(w.field, w.dst, w.n));
    if (rc != PLUME_OK) return rc;
  }
  eng(h)->set_clock(ints[9], consts[1]);
  return PLUME_OK;
}

int plume_get_info(plume_handle* h, int32_t res[3], int32_t* total_steps, double* total_time,
                   double* dx) {
  if (!h) return PLUME_ERR_INVALID;
  const plume_params& p = eng(h)->params();
  if (res)
    for (int k = 0; k < 3; k++) res[k] = p.res[k];
  if (total_steps) *total_steps = eng(h)->total_steps();
  if (total_time) *total_time = eng(h)->total_time();
  if (dx) *dx = eng(h)->dx();
  return PLUME_OK;
}

// The obstacle matrix of the last moving step, empty before the first one.
static int fetch_iop(plume_handle* h, plume::IopRecord& iop) {
  iop.inside.clear();
  iop.values.clear();
  if (!eng(h)->has_iop()) return PLUME_OK;
  const plume_params& p = eng(h)->params();
  const size_t N = (size_t)p.res[0] * p.res[1] * p.res[2];
  iop.inside.resize(N);
  iop.values.resize(3 * N);
  return eng(h)->download_iop(iop.inside.data(), iop.values.data(), N);
}

static plume::FieldFetch make_fetch(plume_handle* h) {
  return [h](int field, std::vector<double>& buf) {
    const plume_params& p = eng(h)->params();
    const size_t N = (size_t)p.res[0] * p.res[1] * p.res[2];
    const bool vec = field == PLUME_F_VELOCITY || field == PLUME_F_VELOCITY_OLD ||
                     field == PLUME_F_FORCE || field == PLUME_F_VORTICITY ||
                     field == PLUME_F_PREPROJECTION || field == PLUME_F_PREDIFFUSION ||
                     field == PLUME_F_PREADVECTION || field == PLUME_F_CACHED_QUADRATIC ||
                     field == PLUME_F_POSTADVECTION || field == PLUME_F_PREVORTICITY ||
                     field == PLUME_F_POST_IOP;
    if (field == PLUME_F_POST_IOP && !eng(h)->has_iop()) {
      buf.clear();  // never assigned: written as an empty field
      return (int)PLUME_OK;
    }
    buf.resize(vec ? 3 * N : N);
    return eng(h)->download(field, buf.data(), buf.size());
  };
}

int plume_write_state(plume_handle* h, const char* path) {
  if (!h) return PLUME_ERR_INVALID;
  if (!path) return set_err(h, PLUME_ERR_INVALID, "null path");
  const plume_params& p = eng(h)->params();
  if (!p.cache_fields) return set_err(h, PLUME_ERR_STATE, "state file needs cache_fields = 1");
  plume::StateHeader hd;
  for (int k = 0; k < 3; k++) hd.res[k] = p.res[k];
  hd.total_steps = eng(h)->total_steps();
  hd.dx = eng(h)->dx();
  hd.total_time = eng(h)->total_time();
  hd.dt = p.dt;
  hd.buoyancy = p.buoyancy;
  hd.vorticity_eps = p.vorticity_eps;
  std::vector<uint8_t> ob((size_t)p.res[0] * p.res[1] * p.res[2]);
  int rc = eng(h)->download_obstacles(ob.data(), ob.size());
  if (rc != PLUME_OK) return from_engine(h, rc);
  plume::IopRecord iop;
  rc = fetch_iop(h, iop);
  if (rc != PLUME_OK) return from_engine(h, rc);
  return plume::write_state_gz(path, hd, make_fetch(h), ob, iop, h->err);
}

int plume_append_streams(plume_handle* h, const char* dir) {
  if (!h) return PLUME_ERR_INVALID;
  if (!dir) return set_err(h, PLUME_ERR_INVALID, "null directory");
  const plume_params& p = eng(h)->params();
  if (!p.cache_fields) return set_err(h, PLUME_ERR_STATE, "streams need cache_fields = 1");
  plume::IopRecord iop;
  const int rc = fetch_iop(h, iop);
  if (rc != PLUME_OK) return from_engine(h, rc);
  return plume::append_streams(dir, p.res, make_fetch(h), iop, h->err);
}

const char* plume_strerror(int status) {
  switch (status) {
    case PLUME_OK: return "ok";
    case PLUME_ERR_INVALID: return "invalid argument";
    case PLUME_ERR_CUDA: return "CUDA error";
    case PLUME_ERR_OOM: return "out of memory";
    case PLUME_ERR_TIMEOUT: return "device wait timed out";
    case PLUME_ERR_IO: return "file I/O error";
    case PLUME_ERR_NOT_CONVERGED: return "solver did not converge";
    case PLUME_ERR_UNSUPPORTED: return "unsupported";
    case PLUME_ERR_STATE: return "call not allowed in this state";
    default: return "unknown status";
  }
}

const char* plume_last_error(plume_handle* h) {
  if (!h) return plume::global_error().c_str();
  return h->err.c_str();
}

// ---- solver-level entry points (include/plume_solver.h) ----
int plume_solve_poisson(plume_handle* h, const double* b, double* x, plume_step_stats* stats) {
  if (!h) return PLUME_ERR_INVALID;
  return from_engine(h, eng(h)->solve(b, x, stats));
}

int plume_mic_apply(plume_handle* h, const double* r, double* z, double* q) {
  if (!h || !r || !z) return PLUME_ERR_INVALID;
  return from_engine(h, eng(h)->mic_apply(r, z, q));
}

int plume_mic_diagonal(plume_handle* h, double* precon) {
  if (!h || !precon) return PLUME_ERR_INVALID;
  return from_engine(h, eng(h)->mic_precon(precon));
}

int plume_sync(plume_handle* h) {
  if (!h) return PLUME_ERR_INVALID;
  const int rc = from_engine(h, eng(h)->sync());
  if (rc != PLUME_OK) return rc;
  return plume_wait_snapshots(h);
}

int plume_wait_snapshots(plume_handle* h) {
  if (!h) return PLUME_ERR_INVALID;
  if (!h->writer) return PLUME_OK;
  std::string e;
  const int rc = h->writer->take_error(e, true);
  return rc == PLUME_OK ? PLUME_OK : set_err(h, rc, e);
}

int plume_snapshot_async(plume_handle* h, const char* dir, int32_t step, int32_t what) {
  if (!h) return PLUME_ERR_INVALID;
  if (!dir || step < 0 || (what & 3) == 0 || (what & ~3) != 0)
    return set_err(h, PLUME_ERR_INVALID, "need a directory, step >= 0 and what in 1..3");
  const plume_params& p = eng(h)->params();
  if (!p.cache_fields) return set_err(h, PLUME_ERR_STATE, "snapshots need cache_fields = 1");
  if (!h->writer) h->writer.reset(new (std::nothrow) SnapshotWriter());
  if (!h->writer) return set_err(h, PLUME_ERR_OOM, "writer thread");
  {
    std::string e;
    const int rc = h->writer->take_error(e, false);  // an earlier snapshot's failure
    if (rc != PLUME_OK) return set_err(h, rc, e);
  }
  // copy every field the writers read while the step loop waits; the rest
  // happens on the writer thread
  const size_t N = (size_t)p.res[0] * p.res[1] * p.res[2];
  std::shared_ptr<SnapshotWriter::FieldSet> fs = h->writer->field_set();
  const plume::FieldFetch live = make_fetch(h);
  for (int f = 0; f < PLUME_F_COUNT; f++) {
    const int rc = live(f, (*fs)[f]);
    if (rc != PLUME_OK) return from_engine(h, rc);
  }
  auto ob = std::make_shared<std::vector<uint8_t>>(N);
  int rc = eng(h)->download_obstacles(ob->data(), ob->size());
  if (rc != PLUME_OK) return from_engine(h, rc);
  auto iop = std::make_shared<plume::IopRecord>();
  rc = fetch_iop(h, *iop);
  if (rc != PLUME_OK) return from_engine(h, rc);
  plume::StateHeader hd;
  for (int k = 0; k < 3; k++) hd.res[k] = p.res[k];
  hd.total_steps = eng(h)->total_steps();
  hd.dx = eng(h)->dx();
  hd.total_time = eng(h)->total_time();
  hd.dt = p.dt;
  hd.buoyancy = p.buoyancy;
  hd.vorticity_eps = p.vorticity_eps;
  char name[64];
  snprintf(name, sizeof(name), "fluid.%04i.fluid3d", step);
  const std::string d = dir, state_path = d + name;
  int res[3] = {p.res[0], p.res[1], p.res[2]};
  SnapshotWriter* w = h->writer.get();
  h->writer->push([=](std::string& e) {
    const plume::FieldFetch held = [fs](int f, std::vector<double>& buf) {
      buf = (*fs)[f];
      return PLUME_OK;
    };
    int r = PLUME_OK;
    if (what & 1) r = plume::write_state_gz(state_path, hd, held, *ob, *iop, e);
    if (r == PLUME_OK && (what & 2)) r = plume::append_streams(d, res, held, *iop, e);
    w->recycle(fs);
    return r;
  });
  return PLUME_OK;
}

// ---- moving box obstacle (include/plume_box.h) ----
int plume_step_moving_box(plume_handle* h, const plume_box* box, plume_step_stats* stats) {
  if (!h) return PLUME_ERR_INVALID;
  if (!box) return set_err(h, PLUME_ERR_INVALID, "null box");
  return from_engine(h, eng(h)->step_moving_box(*box, stats));
}

int plume_set_initial_velocity_box(plume_handle* h, const plume_box* box) {
  if (!h) return PLUME_ERR_INVALID;
  if (!box) return set_err(h, PLUME_ERR_INVALID, "null box");
  return from_engine(h, eng(h)->set_initial_velocity_box(*box));
}

int plume_run_moving_timed(plume_handle* h, plume_box* box, int32_t first_step_index, int32_t n,
                           double* ms_device, plume_step_stats* stats) {
  if (!h) return PLUME_ERR_INVALID;
  if (!box || !ms_device || n < 0) return set_err(h, PLUME_ERR_INVALID, "bad argument");
  return from_engine(h, eng(h)->run_moving_timed(*box, first_step_index, n, ms_device, stats));
}

int plume_box_stomp_times(plume_handle* h, double* ms_total, int64_t* launches) {
  if (!h || !ms_total || !launches) return PLUME_ERR_INVALID;
  return from_engine(h, eng(h)->stomp_times(ms_total, launches));
}

int plume_download_iop(plume_handle* h, uint8_t* inside, double* values, size_t n) {
  if (!h) return PLUME_ERR_INVALID;
  return from_engine(h, eng(h)->download_iop(inside, values, n));
}

int plume_profile_sweeps(plume_handle* h, int on) {
  if (!h) return PLUME_ERR_INVALID;
  return from_engine(h, eng(h)->profile_sweeps(on));
}

int plume_sweep_times(plume_handle* h, double* ms_total, int64_t* launches) {
  if (!h || !ms_total || !launches) return PLUME_ERR_INVALID;
  return from_engine(h, eng(h)->sweep_times(ms_total, launches));
}

int plume_set_wait_gate(plume_handle* h, int32_t closed, int64_t poll_limit) {
  if (!h) return PLUME_ERR_INVALID;
  return from_engine(h, eng(h)->set_wait_gate(closed, (long long)poll_limit));
}

}  // extern "C"
