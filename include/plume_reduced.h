/*
 * plume_reduced.h -- the reduced (subspace) plume step on the GPU.
 *
 * Replaces, for a C / ctypes caller:
 *   src/integrators/SUBSPACE_FLUID_3D_EIGEN.cpp:243-304  stepReorderedCubatureStam
 *     (full-space buoyancy, vorticity and scalar advection, then the velocity in
 *      reduced coordinates: projection on U.preadvect, cubature advection,
 *      reduced damping, staged reduced pressure projection, unprojection on
 *      U.final)
 *   src/integrators/SUBSPACE_FLUID_3D_EIGEN.cpp:1206-1319  readAdvectionCubature
 *     (the cubature file and the advection cubature cache, built and written
 *      when missing)
 *   src/integrators/SUBSPACE_FLUID_3D_EIGEN.cpp:1911-1931  loadReducedRuntimeBases
 *   projects/reduced3D/reduced3D.cpp:344-375             the stage's step loop
 *
 * A reduced model is attached to a plume handle (its grid, walls, buoyancy,
 * vorticity and sources): plume_add_source + plume_reduced_step replace
 * addSmokeColumn + stepReorderedCubatureStam.  The model's files are the
 * reference's, under `reduced_path`: U.preadvect.matrix, U.final.matrix,
 * projected.ptof.matrix, inverseProduct.matrix, damping.peeled.matrix (the
 * projected operators that SUBSPACE_FLUID_3D_EIGEN's constructor builds),
 * cubature, and advection.cubature.cache (built from U.preadvect.matrix and
 * U.prediffuse.matrix and written when missing, as the reference does).
 * The bases and the reduced arithmetic are FP64 in both field precisions.
 */
#ifndef PLUME_REDUCED_H
#define PLUME_REDUCED_H

#include <stddef.h>
#include <stdint.h>

#include "plume.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct plume_reduced plume_reduced;

/* Loads the model for the handle's grid; PLUME_ERR_IO when a file is missing
   or does not match the grid, PLUME_ERR_INVALID on inconsistent ranks.  The
   handle must outlive the model. */
int plume_reduced_create(plume_handle* h, const char* reduced_path, plume_reduced** out);
void plume_reduced_destroy(plume_reduced* r);

/* One stepReorderedCubatureStam on the handle's state.  stats (may be NULL):
   launches and the step's device time. */
int plume_reduced_step(plume_reduced* r, plume_step_stats* stats);

/* The reduced coordinates after the last step (the reference's _qDot, in the
   U.final basis): *size values written to q when n >= *size. */
int plume_reduced_qdot(plume_reduced* r, double* q, int32_t n, int32_t* size);

/* Ranks: dims[0] = U.preadvect columns, [1] = advected (prediffuse) rank,
   [2] = damped (preproject) rank, [3] = U.final columns, [4] = cubature
   points. */
int plume_reduced_dims(plume_reduced* r, int32_t dims[5]);

#ifdef __cplusplus
}
#endif

#endif /* PLUME_REDUCED_H */
