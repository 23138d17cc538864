/*
 * plume.h -- C ABI of libplume, a GB300 (sm_103a) implementation of the
 * full-rank Stam-style smoke step of the Compressing-Fluid-Subspaces
 * pipeline (aadjones/CFS_PLUME, stage `fluid3D`).
 *
 * The reference has no FFI: its hot path is the C++ class FLUID_3D_MIC
 * (src/integrators/FLUID_3D_MIC.h:37-120) driven by projects/fluid3D/fluid3D.cpp.
 * Each entry point below names the reference member or code block it
 * replaces.  Everything is plain C: pointers, sizes and status codes.
 *
 * Conventions
 *  - Every function returns a plume_status (0 = PLUME_OK).  No function
 *    calls exit() or throws across the ABI; the reference exit(0)s on I/O
 *    failures (FLUID_3D_MIC.cpp:1030-1037).
 *  - The handle owns all device memory.  Host buffers belong to the caller.
 *  - One host thread per handle.  Work is ordered on the handle's own CUDA
 *    stream; functions that return host data synchronise that stream.
 *  - Grid layout is the reference's: index = x + y*xRes + z*xRes*yRes,
 *    vector fields are downloaded as interleaved (x,y,z) doubles per cell
 *    (VECTOR3_FIELD_3D, VEC3F = 3 doubles, src/geometry/VEC3.h:319-320).
 */
#ifndef PLUME_H
#define PLUME_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PLUME_ABI_VERSION 2

typedef enum plume_status {
  PLUME_OK = 0,
  PLUME_ERR_INVALID = 1,       /* bad argument or parameter combination      */
  PLUME_ERR_CUDA = 2,          /* a CUDA runtime call failed                 */
  PLUME_ERR_OOM = 3,           /* device or host allocation failed           */
  PLUME_ERR_TIMEOUT = 4,       /* a bounded device wait gave up              */
  PLUME_ERR_IO = 5,            /* snapshot / stream file could not be written*/
  PLUME_ERR_NOT_CONVERGED = 6, /* solver missed its target (stats say more)  */
  PLUME_ERR_UNSUPPORTED = 7,   /* valid request this build does not handle   */
  PLUME_ERR_STATE = 8          /* call not allowed in the handle's state     */
} plume_status;

typedef enum plume_precision {
  PLUME_PREC_FP64 = 0, /* every field and operation in FP64 (reference parity) */
  PLUME_PREC_FP32 = 1  /* FP32 fields/stencils, FP64 CG scalars & MIC diagonal */
} plume_precision;

typedef enum plume_criterion {
  /* the reference's own stop test: signed max(r) <= tol (absolute), bail on
     relative change of max(r) < 1e-7, alpha breakdown
     (FLUID_3D_MIC.cpp:943-1010) */
  PLUME_CRIT_REFERENCE = 0,
  /* ||r||_2 <= tol * ||b||_2 (used for the 1e-6 configurations) */
  PLUME_CRIT_REL2 = 1
} plume_criterion;

typedef enum plume_source {
  PLUME_SRC_COLUMN = 0, /* FLUID_3D_MIC::addSmokeColumn, FLUID_3D_MIC.cpp:655-700 */
  PLUME_SRC_BOX = 1,    /* axis-aligned box, density = heat = 1 + noise*(2u-1) */
  PLUME_SRC_NONE = 2
} plume_source;

typedef enum plume_warm_start {
  PLUME_WARM_ZERO = 0,     /* p = 0 before every solve (FLUID_3D_MIC.cpp:360)   */
  PLUME_WARM_PREVIOUS = 1, /* previous step's pressure                         */
  PLUME_WARM_LEARNED = 2   /* learned initial guess; plain MIC-PCG still judges */
} plume_warm_start;

typedef enum plume_preconditioner {
  /* MIC(0)-PCG, the reference's solve (FLUID_3D_MIC.cpp:918-1015) */
  PLUME_PRECOND_MIC = 0,
  /* flexible CG (Notay's FCG(1): each new direction A-orthogonal to the last,
     exact line search) with the attached network as the preconditioner
     stage, z = net(r); no counterpart in the reference.  Same stop test; a
     solve that misses it within its iteration cap reruns as MIC-PCG from
     p = 0, so plain MIC-PCG stays the fallback and the judge. */
  PLUME_PRECOND_NET = 1
} plume_preconditioner;

typedef enum plume_field {
  /* order = the state file order of FLUID_3D_MIC::writeGz (FLUID_3D_MIC.cpp:1057-1103) */
  PLUME_F_DENSITY = 0,
  PLUME_F_DENSITY_OLD,
  PLUME_F_HEAT,
  PLUME_F_HEAT_OLD,
  PLUME_F_PRESSURE,
  PLUME_F_DIVERGENCE,
  PLUME_F_VELOCITY,          /* vector */
  PLUME_F_VELOCITY_OLD,      /* vector */
  PLUME_F_FORCE,             /* vector */
  PLUME_F_VORTICITY,         /* vector */
  PLUME_F_PREPROJECTION,     /* vector */
  PLUME_F_PREDIFFUSION,      /* vector */
  PLUME_F_PREADVECTION,      /* vector */
  PLUME_F_CACHED_QUADRATIC,  /* vector */
  PLUME_F_POSTADVECTION,     /* vector */
  PLUME_F_CACHED_PRESSURE,
  PLUME_F_CACHED_DIVERGENCE,
  PLUME_F_PREVORTICITY,      /* vector */
  PLUME_F_POST_IOP,          /* vector: velocity after the obstacle stomp of the
                                last moving-box step (FLUID_3D_MIC.h:178), before
                                projection; PLUME_ERR_STATE before the first one */
  PLUME_F_COUNT
} plume_field;

typedef struct plume_params {
  int32_t abi_version;     /* PLUME_ABI_VERSION                                 */
  int32_t res[3];          /* xRes, yRes, zRes (cfg xres/yres/zres, fluid3D.cpp:313-315) */
  int32_t bc[6];           /* front, back, left, right, top, bottom; 1 = wall slab
                              (obstacle), 0 = open (fluid3D.cpp:321-327)        */
  double dt;               /* 0.1 (FLUID_3D_MIC.cpp:181-185)                    */
  double buoyancy;         /* (double)0.1f (FLUID_3D_MIC.cpp:36)                */
  double vorticity_eps;    /* cfg `vorticity`, default 0 (fluid3D.cpp:316,346)  */
  double damping_w;        /* 0.9 (FLUID_3D_MIC.cpp:1255)                       */
  double mic_tau;          /* 0.97 (FLUID_3D_MIC.cpp:829)                       */
  double mic_sigma;        /* 0.25 (FLUID_3D_MIC.cpp:830)                       */
  int32_t source;          /* plume_source                                      */
  int32_t box_lo[3];       /* PLUME_SRC_BOX: half-open cell box [lo, hi)        */
  int32_t box_hi[3];
  double source_noise;     /* PLUME_SRC_BOX: amplitude of the seeded noise       */
  uint64_t seed;           /* noise seed                                        */
  int32_t precision;       /* plume_precision                                   */
  int32_t criterion;       /* plume_criterion                                   */
  double tol;              /* 1e-10 (reference) / 1e-6 (rel2)                   */
  int32_t max_iters;       /* 1000 (FLUID_3D_MIC.cpp:33)                        */
  int32_t warm_start;      /* plume_warm_start                                  */
  int32_t cache_fields;    /* 1: keep every cached field the state file holds
                              (prevorticity, preadvection, ... , FLUID_3D_MIC.h:156-190);
                              0: keep only what the step itself needs          */
  int32_t device;          /* CUDA device ordinal                               */
  int32_t preconditioner;  /* plume_preconditioner (0: MIC(0), the reference's) */
  int32_t reserved[7];
} plume_params;

typedef struct plume_step_stats {
  int32_t iterations;       /* PCG iterations of this step's solve             */
  int32_t converged;        /* 1 if the stop test was met                      */
  int32_t fallback;         /* 1 if the learned start was rejected             */
  int32_t launches;         /* kernels this library launched for the step      */
  double max_residual;      /* signed max of r at exit (reference criterion)   */
  double rel_residual;      /* ||r||_2 / ||b||_2 at exit (recursive residual)  */
  double rhs_norm;          /* ||b||_2                                         */
  double ms_total;          /* device time of the step, CUDA events            */
  double ms_solve;          /* device time of the Poisson solve                */
  /* Device time of each stage of the step (CUDA events on the handle's
     stream): the reference's TIMER buckets (src/util/TIMER.cpp:33-149, one
     per FLUID_3D_MIC member) measured on the device.  The stages and
     ms_solve add up to ms_total. */
  double ms_forces;         /* walls, addBuoyancy (FLUID_3D_MIC.cpp:188-199)   */
  double ms_vorticity;      /* addVorticity and its axpy (524-590, 202)        */
  double ms_advection;      /* advectStam (595-650)                            */
  double ms_damping;        /* the damping product (209-212)                   */
  double ms_divergence;     /* project up to the solve: boundary conditions and
                               divergence (314-360), the moving box's stomp    */
  double ms_guess;          /* learned initial guess (residual, network,
                               Galerkin step); 0 for the other starts         */
  double ms_gradient;       /* project after the solve: gradient (372-398)     */
} plume_step_stats;

typedef struct plume_handle plume_handle;

/* Fill *p with the reference's defaults: 48x64x48, walls front/back/left/right,
   open top/bottom, column source, FP64, reference criterion at 1e-10
   (fluid3D.cpp:313-327, FLUID_3D_MIC.cpp:29-54). */
void plume_default_params(plume_params* p);

/* FLUID_3D_MIC::FLUID_3D_MIC(xRes, yRes, zRes, amplify, boundaries)
   (FLUID_3D_MIC.cpp:29-160) plus `fluid->vorticityEps() = vorticity`
   (fluid3D.cpp:346). Allocates all device state on p->device. */
int plume_create(const plume_params* p, plume_handle** out);

/* FLUID_3D_MIC::~FLUID_3D_MIC (FLUID_3D_MIC.cpp:162-167). NULL is allowed. */
void plume_destroy(plume_handle* h);

/* FLUID_3D_MIC::addSmokeColumn (FLUID_3D_MIC.cpp:655-700) or the box source,
   whichever p->source selects; `step_index` keys the box noise. */
int plume_add_source(plume_handle* h, int32_t step_index);

/* The same injection with caller-supplied values: density = heat = values[k]
   over the cells of the source box (PLUME_SRC_BOX; k runs x fastest over the
   box), copied from host memory.  The reference's addSmokeTestCase writes the
   source into its host arrays the same way (FLUID_3D_MIC.cpp:694-697).
   n must equal the number of box cells. */
int plume_add_source_values(plume_handle* h, const double* values, size_t n);

/* FLUID_3D_MIC::step (FLUID_3D_MIC.cpp:179-223).  Enqueues the whole step on
   the handle's stream; `stats` (may be NULL) is filled after the step ends,
   which synchronises. */
int plume_step(plume_handle* h, plume_step_stats* stats);

/* Run `n` x (add_source; step) back to back without host synchronisation
   between steps (fluid3D.cpp:357-398 without the file output).  `stats` may be
   NULL or point to n entries. */
int plume_run(plume_handle* h, int32_t first_step_index, int32_t n,
              plume_step_stats* stats);

/* plume_run bracketed by CUDA events recorded on the handle's stream;
   *ms_device receives the device time of all n steps; `stats` may be NULL
   or point to n entries. */
int plume_run_timed(plume_handle* h, int32_t first_step_index, int32_t n,
                    double* ms_device, plume_step_stats* stats);

/* Copy one field to host FP64, in the reference layout.  `n` is the number of
   doubles in `dst`: N for scalar fields, 3N for vector fields. */
int plume_download(plume_handle* h, int32_t field, double* dst, size_t n);

/* Overwrite one field from host FP64 (reference layout). */
int plume_upload(plume_handle* h, int32_t field, const double* src, size_t n);

/* Copy the obstacle flags (N bytes, FLUID_3D_MIC.h:153). */
int plume_download_obstacles(plume_handle* h, uint8_t* dst, size_t n);

/* Grid sizes and step counter. */
int plume_get_info(plume_handle* h, int32_t res[3], int32_t* total_steps,
                   double* total_time, double* dx);

/* FLUID_3D_MIC::writeGz (FLUID_3D_MIC.cpp:1020-1110): write the full state in
   the reference format (gzip level 1) to `path` ('.gz' appended when missing). */
int plume_write_state(plume_handle* h, const char* path);

/* FLUID_3D_MIC::readGz (FLUID_3D_MIC.cpp:1115-1246) for one field, on the
   host only (no handle, no device): opens `path` ('.gz' appended unless the
   name ends in "gz"), returns the file's grid in res (may be NULL) and, when
   dst is not NULL, copies the field in the reference layout (n = N or 3N
   doubles, as the file holds it).  The file holds every field id up to
   PLUME_F_CACHED_DIVERGENCE, PLUME_F_PREVORTICITY and PLUME_F_POST_IOP (empty
   unless a moving-box step wrote it).  PLUME_ERR_IO for a missing or
   truncated file, PLUME_ERR_INVALID when n does not match the field,
   PLUME_ERR_UNSUPPORTED in a build without zlib. */
int plume_state_read_field(const char* path, int32_t field, double* dst, size_t n, int32_t res[3]);

/* The header of a state file (FLUID_3D_MIC.cpp:1134-1160), host only:
   ints = xRes, yRes, zRes, maxRes, xs, ys, zs, totalCells, slabSize,
   totalSteps; consts = dx, totalTime, dt, buoyancy, vorticityEps,
   heatDiffusion, solverEps. */
int plume_state_read_header(const char* path, int32_t ints[10], double consts[7]);

/* FLUID_3D_MIC::readGz into a handle: the state file as a checkpoint.  The
   file's grid must be the handle's, and its dx, dt, buoyancy and vorticityEps
   must equal the handle's parameters (PLUME_ERR_INVALID otherwise; the file
   holds no wall flags, which stay the handle's).  Restores density, heat,
   velocity, their Old copies, pressure, and the step count and time; every
   other field is rebuilt by the next step, so stepping on continues the run
   that wrote the file (a learned warm start's iteration cap restarts). */
int plume_read_state(plume_handle* h, const char* path);

/* SUBSPACE_FLUID_3D_EIGEN::diffGroundTruth's norms
   (SUBSPACE_FLUID_3D_EIGEN.cpp:804-835) for full-grid fields in the reference
   layout: errors = { |peel(u) - peel(u_t)|, that / |peel(u)|,
   |peel(rho) - peel(rho_t)|, that / |peel(rho)| } over the interior cells.
   Host only. */
int plume_peeled_errors(const int32_t res[3], const double* velocity, const double* density,
                        const double* truth_velocity, const double* truth_density, double errors[4]);

/* FLUID_3D_MIC::appendStreams (FLUID_3D_MIC.cpp:1329-1477): append this step's
   peeled rows to <dir>velocity.{final,preproject,prediffuse,preadvect}.matrix.transpose
   and <dir>pressure.matrix.transpose, and rewrite the six .dims files. */
int plume_append_streams(plume_handle* h, const char* dir);

/* Asynchronous snapshot (no counterpart in the reference, whose writeGz and
   appendStreams block the step loop): the fields are copied to host memory
   before the call returns; deflating (in parallel, gzip level 1) and the file
   writes run on the handle's writer thread, in call order.  what: bit 0 = the
   state file "<dir>fluid.%04i.fluid3d.gz" of `step` (as plume_write_state),
   bit 1 = the stream rows under `dir` (as plume_append_streams).  At most two
   snapshots are in flight; a third call waits for the oldest.  A write error
   is returned by the next plume_snapshot_async, plume_wait_snapshots or
   plume_sync; plume_destroy waits for pending writes. */
int plume_snapshot_async(plume_handle* h, const char* dir, int32_t step, int32_t what);
/* Wait until every snapshot of the handle is on disk. */
int plume_wait_snapshots(plume_handle* h);

/* Human-readable text of a status code. */
const char* plume_strerror(int status);

/* Detail of the last error on this handle (or the last create failure if h is
   NULL); valid until the next call on the same handle. */
const char* plume_last_error(plume_handle* h);

#ifdef __cplusplus
}
#endif

#endif /* PLUME_H */
