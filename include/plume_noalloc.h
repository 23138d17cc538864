/*
 * plume_noalloc.h -- an entry point that allocates no device memory.
 */
#ifndef PLUME_NOALLOC_H
#define PLUME_NOALLOC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Largest skewed work vector (interior cells plus row padding: for a grid
   X x Y x Z this is (Z-2) * (Y+29) * 32*ceil((X-2)/32)) and the largest
   number of interior planes the fixed scratch holds.  The scratch is one
   device array of about 8.4 MB that every GPU loading the library keeps until
   the process exits. */
#define PLUME_NOALLOC_MAX_ELEMS (1 << 18)
#define PLUME_NOALLOC_MAX_PLANES 1024

/* MIC(0) preconditioner apply, z = M^-1 r, in FP64, without allocating.
   No counterpart in the reference: it has no such entry point.  It is for
   callers that run their own solver on the GPU and cannot call cudaMalloc
   where they need the preconditioner -- inside a region being captured into
   a CUDA graph, or under a host framework that owns all device memory.

   res, bc     : grid size and the six wall flags, as in plume_params.
   precon, r   : device pointers, N = res[0]*res[1]*res[2] doubles each, full
                 grid in the reference layout (precon as from
                 plume_mic_diagonal; border entries of r are ignored).
   z           : device pointer, N doubles; the interior receives M^-1 r and
                 the border is set to 0.
   stream      : cudaStream_t to order the work on (NULL = legacy default);
                 it must belong to the current device, whose copy of the
                 scratch array the call uses.

   Work vectors live in one file-scope device array (sizes above); grids that
   do not fit are rejected with PLUME_ERR_INVALID, as are x resolutions above
   258.  The first call on each device looks up that array's device address
   with the device current and keeps it for the life of the process, so make
   the first call on a device before any stream capture, and make no call on
   a device after cudaDeviceReset on it (the kept address would be stale).
   Every call uses the same array and clears the parts that must start at
   zero; calls whose work overlaps on the GPU (different streams
   or threads, no ordering between them) race on the array and must not be
   issued.  Returns a plume_status for the checks and launches; the work is
   only queued, so the caller orders or synchronizes on `stream` before
   reading z.  If a sweep's inter-CTA wait expires on the GPU, z is set to NaN
   everywhere, and the next call starts afresh (it clears the state it
   needs).  Otherwise z equals plume_mic_apply on an FP64 handle of the same
   grid bit for bit.  Test hook: with PLUME_NOALLOC_WAIT_GATE=<polls> in the
   environment, each sweep first polls a device flag that nothing sets, at
   most <polls> times, before it issues any copy, so the wait expires and z
   comes back NaN. */
int plume_mic_apply_noalloc(const int32_t res[3], const int32_t bc[6],
                            const double* precon, const double* r, double* z,
                            void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PLUME_NOALLOC_H */
