/*
 * plume_solver.h -- solver-level entry points of libplume.
 *
 * The reference's Poisson solver is protected inside FLUID_3D_MIC
 * (FLUID_3D_MIC.h:263-276); these entry points expose the same operators on a
 * handle's grid and wall layout so callers (and the parity tests) can run them
 * on their own vectors.  Arrays are full grids, FP64, reference layout.
 */
#ifndef PLUME_SOLVER_H
#define PLUME_SOLVER_H

#include "plume.h"

#ifdef __cplusplus
extern "C" {
#endif

/* FLUID_3D_MIC::solvePoisson (FLUID_3D_MIC.cpp:918-1015) with the handle's
   criterion, tolerance and iteration cap: solves A x = b on the interior;
   x holds the initial guess on entry and the solution on return.  Uses the
   handle's pressure and divergence storage as workspace (the step's state in
   them is overwritten). */
int plume_solve_poisson(plume_handle* h, const double* b, double* x,
                        plume_step_stats* stats);

/* FLUID_3D_MIC::applyMICPreconditioner (FLUID_3D_MIC.cpp:864-899): z = M^-1 r;
   q (may be NULL) receives the forward-sweep intermediate. */
int plume_mic_apply(plume_handle* h, const double* r, double* z, double* q);

/* The MIC(0) diagonal of FLUID_3D_MIC::buildMICPreconditioner
   (FLUID_3D_MIC.cpp:825-856), FP64, N doubles. */
int plume_mic_diagonal(plume_handle* h, double* precon);

/* Wait for all work queued on the handle's stream. */
int plume_sync(plume_handle* h);

/* Per-launch device timing of the MIC sweep kernels (the reference's TIMER
   around applyMICPreconditioner, FLUID_3D_MIC.cpp:866, made per launch):
   on != 0 clears the totals and brackets every later forward and backward
   sweep launch with CUDA events on the handle's stream; 0 stops. */
int plume_profile_sweeps(plume_handle* h, int on);

/* Totals since profiling was switched on: summed device milliseconds of the
   timed sweep launches and their number.  Waits for the handle's stream. */
int plume_sweep_times(plume_handle* h, double* ms_total, int64_t* launches);

/* Test hook for the bounded device waits of the MIC sweeps (no counterpart in
   the reference, whose sweeps are serial loops).  With closed != 0, every
   later sweep of this handle first polls a device flag that nothing sets, at
   most poll_limit times (> 0), before it issues any copy; the wait then
   expires, the sweep records it and returns without touching the vectors, and
   the solve or step returns PLUME_ERR_TIMEOUT with the handle still usable.
   closed = 0 restores normal sweeps (poll_limit is ignored).  The sweeps'
   real waits keep their own, fixed limits. */
int plume_set_wait_gate(plume_handle* h, int32_t closed, int64_t poll_limit);

#ifdef __cplusplus
}
#endif

#endif /* PLUME_SOLVER_H */
