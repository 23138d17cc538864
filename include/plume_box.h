/*
 * plume_box.h -- the moving box obstacle of the full-rank step.
 *
 * Replaces, for a C / ctypes caller:
 *   src/geometry/BOX.h:29-121, BOX.cpp:26-130   the BOX class (state, spin,
 *                                                translate_center, inside,
 *                                                update_r, linear velocity)
 *   src/integrators/FLUID_3D_MIC.cpp:236-310     stepWithMovingObstacle
 *   src/integrators/FLUID_3D_MIC.cpp:1645-1692   setPeeledSparseMovingIOP
 *   src/integrators/FLUID_3D_MIC.cpp:1695-1701   setVelocityNeumann
 *   src/integrators/FLUID_3D_MIC.cpp:744-764     setInitialVelocity(BOX*)
 *   src/integrators/FLUID_3D_MIC.h:83,100        postIOP(), neumannIOPMatrix()
 *
 * Coordinates are those of FLUID_3D_MIC::cellCenter (FLUID_3D_MIC.cpp:1704-
 * 1733): cell (x, y, z) of an X x Y x Z grid has its centre at
 * ((x + 0.5) / X, (y + 0.5) / Y, (z + 0.5) / Z), each axis scaled to [0, 1].
 *
 * The box spins about +z through its centre (angular velocity 2 pi / period)
 * and sways along x, 0.25 sin(phi) about its original centre (phase speed
 * 2 pi / translation_period).  A moving step stomps the velocity of every
 * interior cell whose centre lies inside the box with the box's rigid velocity
 * there (the IOP product N [u; 1] of the reference), caches that field as
 * postIOP and projects.  The host advances the box between steps with
 * plume_box_spin / plume_box_translate, as the reference's BOX::spin and
 * BOX::translate_center.
 */
#ifndef PLUME_BOX_H
#define PLUME_BOX_H

#include <stddef.h>
#include <stdint.h>

#include "plume.h"

#ifdef __cplusplus
extern "C" {
#endif

/* The state of one BOX (BOX.h:99-121), minus the scratch velocity. */
typedef struct plume_box {
  double center[3];          /* current centre                                  */
  double original_center[3]; /* centre at construction; the sway is about it     */
  double lengths[3];         /* edge lengths; the inside test uses half of them  */
  double rotation[9];        /* row-major R = rotation(+z, -theta), the clockwise
                                matrix of BOX::update_rotationMatrix; identity
                                until the first spin                             */
  double theta;              /* spin angle; reset to 0 once it reaches 2 pi      */
  double phi;                /* sway phase; reset to 0 once it reaches 2 pi      */
  double period;             /* spin period                                      */
  double translation_period; /* sway period                                      */
  double dt;                 /* BOX::set_dt: the time step spin / translate use  */
} plume_box;

/* BOX::BOX(center, lengths, period, translationPeriod) (BOX.cpp:26-41):
   theta = phi = dt = 0, rotation = I, original_center = center. */
int plume_box_init(plume_box* box, const double center[3], const double lengths[3],
                   double period, double translation_period);

/* BOX::spin (BOX.cpp:93-101): theta += 2 pi dt / period (0 once >= 2 pi),
   then rotation = rotation(+z, -theta). */
int plume_box_spin(plume_box* box);

/* BOX::translate_center (BOX.cpp:104-113): phi += 2 pi dt / translation_period
   (0 once >= 2 pi); center.x = original_center.x + 0.25 sin(phi). */
int plume_box_translate(plume_box* box);

/* BOX::inside (BOX.cpp:59-70): |R (point - center)| <= lengths / 2 per axis.
   *inside = 1 or 0. */
int plume_box_inside(const plume_box* box, const double point[3], int32_t* inside);

/* The rigid velocity at `point`: BOX::update_r then update_linearVelocity
   (BOX.cpp:72-90, BOX.h:78-83), omega x r + (0.25 (2 pi / T) cos(phi), 0, 0)
   with r the offset of `point` from the spin axis. */
int plume_box_velocity(const plume_box* box, const double point[3], double velocity[3]);

/* FLUID_3D_MIC::stepWithMovingObstacle: the step of plume_step without the
   buoyancy force, and between damping and projection the obstacle stomp,
   u <- N [u; 1], on every interior cell.  Uses the box as given; it does not
   advance it.  stats as plume_step. */
int plume_step_moving_box(plume_handle* h, const plume_box* box, plume_step_stats* stats);

/* FLUID_3D_MIC::setInitialVelocity(BOX*): velocity = the box's rigid
   velocity on every interior cell inside the box; other cells unchanged. */
int plume_set_initial_velocity_box(plume_handle* h, const plume_box* box);

/* n moving steps timed on the device: for k = 0..n-1, plume_add_source(
   first_step_index + k), plume_step_moving_box(box), then plume_box_spin and
   plume_box_translate on *box.  ms_device: CUDA-event time on the library's
   stream around all n steps.  stats: NULL or n entries. */
int plume_run_moving_timed(plume_handle* h, plume_box* box, int32_t first_step_index, int32_t n,
                           double* ms_device, plume_step_stats* stats);

/* While sweep profiling is on (plume_profile_sweeps), every obstacle stomp
   launch is bracketed by CUDA events too: its summed device time and count
   since profiling was switched on. */
int plume_box_stomp_times(plume_handle* h, double* ms_total, int64_t* launches);

/* The obstacle matrix N of the last moving step (neumannIOPMatrix(),
   3 n_int x (3 n_int + 1), n_int = (X-2)(Y-2)(Z-2)), in full-grid layout:
   inside[c] = 1 where the interior cell c was inside the box (its diagonal
   entries are 0 and its last-column entries the box velocity), else 0;
   values[3c + i] = that last-column entry, 0 where inside[c] = 0.  n = N
   cells; either pointer may be NULL.  PLUME_ERR_STATE before the first
   moving step. */
int plume_download_iop(plume_handle* h, uint8_t* inside, double* values, size_t n);

#ifdef __cplusplus
}
#endif

#endif /* PLUME_BOX_H */
