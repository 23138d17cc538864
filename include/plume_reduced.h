/*
 * plume_reduced.h -- the reduced (subspace) plume step on the GPU.
 *
 * Replaces, for a C / ctypes caller:
 *   src/integrators/SUBSPACE_FLUID_3D_EIGEN.cpp:243-304  stepReorderedCubatureStam
 *     (with its closing diffGroundTruth, lines 804-835, when a full-rank path
 *      is set)
 *     (full-space buoyancy, vorticity and scalar advection, then the velocity in
 *      reduced coordinates: projection on U.preadvect, cubature advection,
 *      reduced damping, staged reduced pressure projection, unprojection on
 *      U.final)
 *   src/integrators/SUBSPACE_FLUID_3D_EIGEN.cpp:1206-1319  readAdvectionCubature
 *     (the cubature file and the advection cubature cache, built and written
 *      when missing)
 *   src/integrators/SUBSPACE_FLUID_3D_EIGEN.cpp:1911-1931  loadReducedRuntimeBases
 *   src/integrators/SUBSPACE_FLUID_3D_EIGEN.cpp:82-167     initOutOfCore (which
 *     files make a built model; stale operators are rebuilt)
 *   src/integrators/SUBSPACE_FLUID_3D_EIGEN.cpp:1355-1490  buildOutOfCoreMatrices
 *     (the projected operators, run by projects/buildProducts through the
 *      constructor): plume_reduced_build_products
 *   projects/reduced3D/reduced3D.cpp:344-375             the stage's step loop
 *
 * A reduced model is attached to a plume handle (its grid, walls, buoyancy,
 * vorticity and sources): plume_add_source + plume_reduced_step replace
 * addSmokeColumn + stepReorderedCubatureStam.  The model's files are the
 * reference's, under `reduced_path`: U.preadvect.matrix, U.final.matrix,
 * the projected operators (projected.A, projected.vtod, damping.peeled,
 * projected.ptof, projected.ptov, inverseProduct .matrix; built on the
 * device from U.pressure, U.preproject, U.prediffuse and U.final when one is
 * missing or projected.ptof no longer matches U.final, as the reference's
 * constructor does), cubature, and advection.cubature.cache (built from
 * U.preadvect.matrix and U.prediffuse.matrix and written when missing).
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

/* What plume_reduced_build_products did. */
typedef struct plume_products_info {
  int32_t ranks[4]; /* columns of U.pressure, U.preproject, U.prediffuse, U.final */
  double ms_device; /* device time: operator stencils, projections, inverse    */
  double ms_total;  /* wall time, file reads and writes included               */
  double gflop;     /* FP64 work of the projections, the inverse and products */
} plume_products_info;

/* buildOutOfCoreMatrices for the handle's grid and walls: reads U.pressure,
   U.preproject, U.prediffuse and U.final under reduced_path and writes
   projected.A  = U_p^T A U_p      (A: the peeled Poisson matrix, buildFlatA)
   projected.vtod = U_p^T V U_pp   (V: computeVelocityToDivergence)
   damping.peeled = U_pp^T D U_pd  (D: buildPeeledDampingMatrixFlat)
   projected.ptof = U_f^T U_pp
   projected.ptov = U_f^T G U_p    (G: computePressureToVelocity)
   inverseProduct = ptov projected.A^-1 vtod
   there (EIGEN::write layout).  PLUME_ERR_IO when a basis is missing or does
   not match the grid, PLUME_ERR_INVALID when projected.A is singular.
   info may be NULL. */
int plume_reduced_build_products(plume_handle* h, const char* reduced_path, plume_products_info* info);

/* Loads the model for the handle's grid; PLUME_ERR_IO when a file is missing
   or does not match the grid, PLUME_ERR_INVALID on inconsistent ranks.  The
   handle must outlive the model. */
int plume_reduced_create(plume_handle* h, const char* reduced_path, plume_reduced** out);
void plume_reduced_destroy(plume_reduced* r);

/* One stepReorderedCubatureStam on the handle's state.  stats (may be NULL):
   launches and the step's device time. */
int plume_reduced_step(plume_reduced* r, plume_step_stats* stats);

/* diffGroundTruth (SUBSPACE_FLUID_3D_EIGEN.cpp:804-835), which the reference
   runs at the end of every reduced step: with a full-rank path set (the
   `snapshot path` of the fluid3D run, with its trailing '/'), every
   plume_reduced_step then reads <path>fluid.%04i.fluid3d.gz of the frame it
   just stepped (the handle's step count - 1) and records the peeled velocity
   and density errors (plume_peeled_errors).  NULL or "" turns it off.  A
   missing or mismatched file fails that step's call with PLUME_ERR_IO /
   PLUME_ERR_INVALID after the step itself has run. */
int plume_reduced_set_ground_truth(plume_reduced* r, const char* full_rank_path);

/* The recorded errors, 4 per compared step (velocity abs, velocity relative,
   density abs, density relative: the reference's velocityErrorAbs,
   velocityErrorRelative, densityErrorAbs, densityErrorRelative): *count
   steps, the first min(n / 4, *count) of them copied to out. */
int plume_reduced_errors(plume_reduced* r, double* out, int32_t n, int32_t* count);

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
