/*
 * plume_batch.h -- many independent plumes on one GPU.
 *
 * No counterpart in the reference (it runs one FLUID_3D_MIC per process).
 * Every instance is a plume_handle of its own (own device state and CUDA
 * stream); plume_batch_run advances all of them concurrently from a pool of
 * host threads, so the GPU interleaves the instances' kernels: the MIC
 * wavefront of one plume occupies one thread-block cluster (<= 16 SMs), and
 * up to ~9 plumes' sweeps run side by side on 152 SMs.  Instances never
 * exchange data; results are identical to stepping each handle alone.
 */
#ifndef PLUME_BATCH_H
#define PLUME_BATCH_H

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

/* n instances, params[i] each (plume_create semantics). */
int plume_batch_create(const plume_params* params, int32_t n, plume_batch** out);
void plume_batch_destroy(plume_batch* b);
int plume_batch_size(plume_batch* b, int32_t* n);
/* Instance i's handle (owned by the batch) for downloads, state files, ... */
int plume_batch_handle(plume_batch* b, int32_t i, plume_handle** h);

/* Every instance runs steps first_step .. first_step+steps-1 (source, then
   step), instances spread over `threads` host threads (0: one per
   instance).  seconds = wall time of the whole call; stats (may be NULL)
   receives n*steps entries, instance-major.  Returns the first failing
   status (plume_last_error(NULL) names the instance). */
int plume_batch_run(plume_batch* b, int32_t first_step, int32_t steps, int32_t threads, double* seconds,
                    plume_step_stats* stats);

#ifdef __cplusplus
}
#endif

#endif /* PLUME_BATCH_H */
