// ccd2d.hpp -- the yes/no and time-of-impact answers of the disc-disc continuous collision test
// (CollisionDetectionUtilities::ballBallCCDCollisionHappens, CollisionDetectionUtilities.cpp:3-126),
// on the coefficients c0 + c1 t + c2 t^2 of the squared gap over the step.  Host and device code
// (no CUDA types) so that a host test can compare the two answers on any inputs.
#pragma once

#include <cmath>

#ifdef __CUDACC__
#define SG_CCD_FN __host__ __device__ __forceinline__
#else
#define SG_CCD_FN inline
#endif

namespace sg {

SG_CCD_FN bool ccd_happens(double c0, double c1, double c2, double* t) {
  // Touching or overlapping at t = 0: the roots below give root1 >= 0 >= root0 for any c1, c2 (a
  // quadratic with c2 >= 0 and c0 <= 0), so the answer is yes without the square root and the
  // divisions; only the time of impact needs them.
  if (!t && c0 <= 0.0) return true;
  if (c2 != 0.0) {
    const double c1c1 = c1 * c1;
    const double fc2c0 = 4.0 * c2 * c0;
    if (c1c1 < fc2c0) return false;
    const double ds = std::sqrt(c1c1 - fc2c0);
    const double root1 = (c1 > 0.0) ? (2.0 * c0) / (-c1 - ds) : (-c1 + ds) / (2.0 * c2);
    if (root1 < 0.0) return false;
    const double root0 = (c1 >= 0.0) ? (-c1 - ds) / (2.0 * c2) : (2.0 * c0) / (-c1 + ds);
    if (root0 > 1.0) return false;
    if (t) *t = std::fmax(0.0, root0);
    return true;
  }
  if (c0 <= 0.0) {
    if (t) *t = 0.0;
    return true;
  }
  return false;
}

// ccd_happens's yes or no without the time of impact, taking the square root and the divisions only
// where signs do not decide.  With c0 > 0 and c2 > 0, both finite and within [2^-500, 2^500] where
// it matters, after the same discriminant test: for c1 > 0 the larger root (2 c0)/(-c1 - ds) is
// negative and does not underflow to -0, so no impact; for c1 < 0 the larger root is >= 0, and
// 2 c0 <= -c1 makes the smaller root (2 c0)/(-c1 + ds) <= 1 in the same rounding (the rounded
// denominator is >= -c1), so impact.  Everything else goes through ccd_happens.
SG_CCD_FN bool ccd_hits(double c0, double c1, double c2) {
  if (c0 <= 0.0) return true;
  if (c2 != 0.0 && c2 <= 0x1p500 && std::fabs(c1) <= 0x1p500 && c0 >= 0x1p-500 && c0 <= 0x1p500) {
    const double c1c1 = c1 * c1;
    const double fc2c0 = 4.0 * c2 * c0;
    if (c1c1 < fc2c0) return false;
    if (c1 > 0.0) return false;
    if (c1 < 0.0 && 2.0 * c0 <= -c1) return true;
  }
  return ccd_happens(c0, c1, c2, nullptr);
}

}  // namespace sg
