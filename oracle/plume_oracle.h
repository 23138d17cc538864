/*
 * plume_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * A CPU, FP64, single-threaded restatement of the reference's full-rank smoke
 * step (aadjones/CFS_PLUME, src/integrators/FLUID_3D_MIC.cpp).  It exists to
 * check the CUDA implementation and to provide the CPU baseline in bench.py.
 * Nothing in the product (cfs_plume_gb300/, include/plume.h) links or calls
 * it.  Only tests/, __graft_entry__.smoke() and bench.py's cpu-baseline /
 * reference legs may load it.
 *
 * Parity of this restatement is pinned against the reference itself: the
 * recipe in oracle/Makefile compiles the reference's own FLUID_3D_MIC.cpp
 * into oracle/_ref/fluid3d_ref, and tests/golden/make_golden.py runs it and
 * stores its outputs as fixtures that tests compare bit for bit.
 */
#ifndef PLUME_ORACLE_H
#define PLUME_ORACLE_H

#include <stddef.h>
#include <stdint.h>
#include "../include/plume.h"
#include "../include/plume_box.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_handle orc_handle;

/* Same parameter struct as the product; `precision` is ignored (always FP64). */
orc_handle* orc_create(const plume_params* p);
void orc_destroy(orc_handle* h);
void orc_add_source(orc_handle* h, int32_t step_index);
void orc_step(orc_handle* h, plume_step_stats* stats);

/* The full-space part of SUBSPACE_FLUID_3D_EIGEN::stepReorderedCubatureStam
   (SUBSPACE_FLUID_3D_EIGEN.cpp:243-268): velocity border wiped, buoyancy,
   vorticity confinement, then advectHeatAndDensityStam (573-601).  The
   reduced part is oracle/reduced_oracle.py; the step counter advances here. */
void orc_reduced_prestep(orc_handle* h);
/* field = plume_field; n = N or 3N doubles. Returns 0 on success. */
int orc_get(orc_handle* h, int32_t field, double* dst, size_t n);
int orc_set(orc_handle* h, int32_t field, const double* src, size_t n);
int orc_get_obstacles(orc_handle* h, uint8_t* dst, size_t n);
int32_t orc_total_steps(orc_handle* h);

/* ---- single primitives on caller arrays (full grid, reference layout) ---- */
/* buildA + buildMICPreconditioner for the Poisson matrix of the wall layout
   `bc` (FLUID_3D_MIC.cpp:772-801, 825-856).  precon: N doubles out. */
void orc_mic_precon(const int32_t res[3], const int32_t bc[6], double tau,
                    double sigma, double* precon);
/* applyMICPreconditioner (FLUID_3D_MIC.cpp:864-899): z = M^-1 r, q = fwd sweep. */
void orc_mic_apply(const int32_t res[3], const int32_t bc[6], const double* precon,
                   const double* r, double* z, double* q);
/* multA (FLUID_3D_MIC.cpp:803-823): b = A x on the interior. */
void orc_mult_a(const int32_t res[3], const int32_t bc[6], const double* x, double* b);
/* VECTOR3_FIELD_3D::advect, scalar form (VECTOR3_FIELD_3D.cpp:2082-2158). */
void orc_advect_scalar(const int32_t res[3], double dt0, const double* vel_aos,
                       const double* old_field, double* new_field);
/* Stand-alone Poisson solve with the configured criterion (solvePoisson,
   FLUID_3D_MIC.cpp:918-1015): x in/out (N), b (N). Returns iterations. */
int32_t orc_solve_poisson(const plume_params* p, double* x, const double* b,
                          plume_step_stats* stats);
/* ---- moving box (plume_box, include/plume_box.h) ---- */
/* BOX constructor, spin, translate_center, inside, rigid velocity (BOX.cpp). */
void orc_box_init(plume_box* b, const double center[3], const double lengths[3], double period,
                  double translation_period);
void orc_box_spin(plume_box* b);
void orc_box_translate(plume_box* b);
int orc_box_inside(const plume_box* b, const double p[3]);
void orc_box_velocity(const plume_box* b, const double p[3], double v[3]);
/* FLUID_3D_MIC::stepWithMovingObstacle (FLUID_3D_MIC.cpp:236-310). */
void orc_step_moving_box(orc_handle* h, const plume_box* box, plume_step_stats* stats);
/* FLUID_3D_MIC::setInitialVelocity(BOX*) (FLUID_3D_MIC.cpp:744-764). */
void orc_set_initial_velocity_box(orc_handle* h, const plume_box* box);
/* The last moving step's obstacle matrix as map-ordered triples; returns the
   entry count, -1 before the first moving step. */
int64_t orc_iop_entries(orc_handle* h, int32_t rows_cols[2], int32_t* ij, double* val);

/* Seeded source value 1 + noise*(2u-1) for (seed, step, cell). */
double orc_source_value(uint64_t seed, int32_t step_index, int64_t cell, double noise);

#ifdef __cplusplus
}
#endif
#endif
