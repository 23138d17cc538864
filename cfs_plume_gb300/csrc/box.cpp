// box.cpp -- host side of the moving box obstacle (include/plume_box.h).
//
// The box's motion is a handful of scalar updates per step, so it stays on
// the host; the per-cell inside test and stomp run on the GPU (k_box_stomp).
// Compiled with -ffp-contract=off: each expression rounds after every
// operation in C order, as the reference's x86-64 build does, so the box
// state is the same bits on every host.
#include <cmath>

#include "../../include/plume_box.h"
#include "engine.h"

namespace {

constexpr double kPi = 3.14159265358979323846;  // M_PI

int fail(const char* msg) {
  plume::global_error() = msg;
  return PLUME_ERR_INVALID;
}

// MATRIX3::rotation(axis, angle) (src/linearalgebra/MATRIX3.h:96-117): the
// Rodrigues formula R = cos I + sin [a]x + (1 - cos) a a^T for the unit axis a.
void rodrigues(const double axis_in[3], double angle, double R[9]) {
  const double len = std::sqrt(axis_in[0] * axis_in[0] + axis_in[1] * axis_in[1] +
                               axis_in[2] * axis_in[2]);
  const double inv = 1.0 / len;
  const double a0 = axis_in[0] * inv, a1 = axis_in[1] * inv, a2 = axis_in[2] * inv;
  const double c = std::cos(angle), s = std::sin(angle), v = 1.0 - c;
  R[0] = a0 * a0 * v + c;
  R[1] = a0 * a1 * v - a2 * s;
  R[2] = a0 * a2 * v + a1 * s;
  R[3] = a1 * a0 * v + a2 * s;
  R[4] = a1 * a1 * v + c;
  R[5] = a1 * a2 * v - a0 * s;
  R[6] = a2 * a0 * v - a1 * s;
  R[7] = a2 * a1 * v + a0 * s;
  R[8] = a2 * a2 * v + c;
}

const double kAxis[3] = {0.0, 0.0, 1.0};  // BOX.cpp:36, the spin axis

}  // namespace

namespace plume {

// Everything the device stomp needs of a box, as computed once per step on
// the host (BOX.h:65-83, BOX.cpp:84-91).
void box_constants(const plume_box& b, double half[3], double omega[3], double disp[3]) {
  for (int k = 0; k < 3; k++) half[k] = b.lengths[k] * 0.5;  // set_halfLengths: 0.5 * lengths
  omega[0] = 0.0;                                             // set_angularVelocity
  omega[1] = 0.0;
  omega[2] = 2 * kPi / b.period;
  disp[0] = 0.25 * 2 * kPi / b.translation_period * std::cos(b.phi);  // displacement velocity
  disp[1] = 0.0;
  disp[2] = 0.0;
}

bool box_finite(const plume_box& b) {
  for (int k = 0; k < 3; k++)
    if (!std::isfinite(b.center[k]) || !std::isfinite(b.lengths[k])) return false;
  for (int k = 0; k < 9; k++)
    if (!std::isfinite(b.rotation[k])) return false;
  return std::isfinite(b.phi) && std::isfinite(b.period) && std::isfinite(b.translation_period) &&
         b.period != 0.0 && b.translation_period != 0.0;
}

}  // namespace plume

extern "C" {

int plume_box_init(plume_box* b, const double center[3], const double lengths[3], double period,
                   double translation_period) {
  if (!b || !center || !lengths) return fail("bad argument");
  for (int k = 0; k < 3; k++) {
    b->center[k] = center[k];
    b->original_center[k] = center[k];
    b->lengths[k] = lengths[k];
  }
  for (int k = 0; k < 9; k++) b->rotation[k] = (k % 4 == 0) ? 1.0 : 0.0;
  b->theta = 0.0;
  b->phi = 0.0;
  b->period = period;
  b->translation_period = translation_period;
  b->dt = 0.0;
  return PLUME_OK;
}

int plume_box_spin(plume_box* b) {
  if (!b) return fail("bad argument");
  const double d_theta = 2 * kPi * b->dt / b->period;
  b->theta += d_theta;
  if (b->theta >= 2 * kPi) b->theta = 0.0;
  rodrigues(kAxis, -1 * b->theta, b->rotation);  // clockwise, BOX.cpp:52-56
  return PLUME_OK;
}

int plume_box_translate(plume_box* b) {
  if (!b) return fail("bad argument");
  const double d_phi = 2 * kPi * b->dt / b->translation_period;
  b->phi += d_phi;
  if (b->phi >= 2 * kPi) b->phi = 0.0;
  const double displacement = 0.25 * std::sin(b->phi);
  b->center[0] = b->original_center[0] + displacement;
  return PLUME_OK;
}

int plume_box_inside(const plume_box* b, const double p[3], int32_t* inside) {
  if (!b || !p || !inside) return fail("bad argument");
  const double u[3] = {p[0] - b->center[0], p[1] - b->center[1], p[2] - b->center[2]};
  const double* R = b->rotation;
  double q[3];
  for (int k = 0; k < 3; k++) q[k] = R[3 * k] * u[0] + R[3 * k + 1] * u[1] + R[3 * k + 2] * u[2];
  *inside = (std::fabs(q[0]) <= b->lengths[0] * 0.5 && std::fabs(q[1]) <= b->lengths[1] * 0.5 &&
             std::fabs(q[2]) <= b->lengths[2] * 0.5)
                ? 1
                : 0;
  return PLUME_OK;
}

int plume_box_velocity(const plume_box* b, const double p[3], double v[3]) {
  if (!b || !p || !v) return fail("bad argument");
  double half[3], w[3], d[3];
  plume::box_constants(*b, half, w, d);
  const double u[3] = {p[0] - b->center[0], p[1] - b->center[1], p[2] - b->center[2]};
  // project_onto(u, axis) = axis ((u . axis) / |axis|^2) (VEC3.h:293-296)
  const double s = (u[0] * kAxis[0] + u[1] * kAxis[1] + u[2] * kAxis[2]) /
                   (kAxis[0] * kAxis[0] + kAxis[1] * kAxis[1] + kAxis[2] * kAxis[2]);
  const double r[3] = {u[0] - kAxis[0] * s, u[1] - kAxis[1] * s, u[2] - kAxis[2] * s};
  // cross(w, r) (VEC3.h:154-155) plus the displacement velocity
  v[0] = (w[1] * r[2] - r[1] * w[2]) + d[0];
  v[1] = (-w[0] * r[2] + r[0] * w[2]) + d[1];
  v[2] = (w[0] * r[1] - r[0] * w[1]) + d[2];
  return PLUME_OK;
}

}  // extern "C"
