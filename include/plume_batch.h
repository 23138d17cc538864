/*
 * plume_batch.h -- many independent plumes on one GPU.
 *
 * No counterpart in the reference (it runs one FLUID_3D_MIC per process).
 * Two engines:
 *
 *  - PLUME_BATCH_FUSED (the default): the plumes advance in lockstep, each
 *    stage of FLUID_3D_MIC::step (FLUID_3D_MIC.cpp:179-223) one kernel launch
 *    over every plume (a block finds its plume in a per-stage table), the MIC
 *    sweeps one launch per shape class (plumes with the same cells per lane
 *    and depth) with the classes running side by side, the CG iterations in
 *    lockstep (a plume that met its stop test skips its share of every later
 *    launch), and each whole step -- source, forces, vorticity, advection,
 *    damping, projection, the CG loop as a conditional-while node, gradient,
 *    per-plume statistics -- one CUDA graph launch.  Block counts per plume
 *    and the sweeps' slab heights are tile shapes chosen by an autotuner
 *    whose choices are cached in a JSON file.  Each plume evaluates the
 *    single-plume engine's per-cell expressions; its dot products are summed
 *    over its own block count, so its FP32 results are not bit-identical to
 *    the same plume stepped alone (FP64: the same within rounding).
 *  - PLUME_BATCH_STREAMS: every instance is a plume_handle of its own (own
 *    device state and CUDA stream) stepped from a pool of host threads; the
 *    GPU interleaves the instances' kernels.  Results are identical to
 *    stepping each handle alone.
 *
 * Instances never exchange data.
 */
#ifndef PLUME_BATCH_H
#define PLUME_BATCH_H

#include <stddef.h>
#include <stdint.h>

#include "plume.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct plume_batch plume_batch;

/* Parameters of instance `index` of the batched-plume configuration: grid
   drawn from {32^3, 48x64x48, 64x96x64, 96x128x96}, closed box, box source
   (the 48x64x48 source box scaled to the grid) with its centre uniform in the
   middle third of the floor, buoyancy U[0.5, 2], vorticity U[0, 4], +-0.05
   noise seeded by seed + index, FP32 fields, rel-L2 1e-6.  Deterministic in
   (seed, index). */
int plume_batch_params(uint64_t seed, int32_t index, plume_params* out);

typedef enum plume_batch_engine {
  PLUME_BATCH_FUSED = 0,  /* one launch per stage over all plumes, CUDA graph */
  PLUME_BATCH_STREAMS = 1 /* one handle + stream per plume, host threads      */
} plume_batch_engine;

typedef struct plume_batch_options {
  int32_t engine;         /* plume_batch_engine                                   */
  int32_t graph;          /* fused: 1 = each step one CUDA graph launch, 0 = the
                             same launches driven from the host                   */
  int32_t tune;           /* fused: 1 = tile shapes from the tuning cache, timed
                             on this GPU when the cache has none; 0 = defaults    */
  int32_t groups;         /* fused: CG groups advanced as parallel graph branches,
                             each its own lockstep loop (1 to 4; 0 = 4 for a batch
                             of 32 or more plumes, 2 for 8 or more, else 1)       */
  const char* tune_cache; /* fused: JSON file of tuned shapes; NULL = the file
                             named by $PLUME_TUNE_CACHE, else
                             $HOME/.cache/cfs_plume_gb300/tune.json               */
  int32_t persistent;     /* fused: 1 = every stage a persistent launch (grid =
                             resident blocks walking the stage's block table);
                             0 = one block per table entry (measured faster)     */
  int32_t reserved[7];
} plume_batch_options;

/* engine = FUSED, graph = 1, tune = 1, groups = 0, tune_cache = NULL. */
void plume_batch_default_options(plume_batch_options* o);

/* n instances, params[i] each.  The fused engine needs every instance on the
   same device and precision, a box (or no) source, warm start ZERO or
   PREVIOUS, the MIC preconditioner, interior x extent <= 256 and z extent
   <= 256 (PLUME_ERR_UNSUPPORTED otherwise); it keeps none of the cached
   fields whatever cache_fields says. */
int plume_batch_create_ex(const plume_params* params, int32_t n, const plume_batch_options* opt,
                          plume_batch** out);
/* plume_batch_create_ex with the default options. */
int plume_batch_create(const plume_params* params, int32_t n, plume_batch** out);
void plume_batch_destroy(plume_batch* b);
int plume_batch_size(plume_batch* b, int32_t* n);
/* Instance i's handle (owned by the batch) for downloads, state files, ...
   (streams engine; PLUME_ERR_STATE for a fused batch). */
int plume_batch_handle(plume_batch* b, int32_t i, plume_handle** h);

/* plume_download for instance i, either engine.  The fused engine keeps
   density, heat (and their _OLD buffers), pressure, divergence and velocity. */
int plume_batch_download(plume_batch* b, int32_t i, int32_t field, double* dst, size_t n);

/* The fused engine's tile shapes as a JSON object (NUL-terminated into json,
   at most cap bytes; *len = the full length).  "{}" for the streams engine. */
int plume_batch_tuning(plume_batch* b, char* json, size_t cap, size_t* len);

/* Every instance runs steps first_step .. first_step+steps-1 (source, then
   step).  Streams engine: instances spread over `threads` host threads (0:
   one per instance); fused engine: `threads` is ignored, and a step's
   ms_total in stats is the device time of the whole call / steps.
   seconds = wall time of the whole call; stats (may be NULL) receives
   n*steps entries, instance-major.  Returns the first failing status
   (plume_last_error(NULL) names the instance). */
int plume_batch_run(plume_batch* b, int32_t first_step, int32_t steps, int32_t threads, double* seconds,
                    plume_step_stats* stats);

#ifdef __cplusplus
}
#endif

#endif /* PLUME_BATCH_H */
