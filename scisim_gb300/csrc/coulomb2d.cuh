// coulomb2d.cuh -- the 2x2 block Coulomb law of the Gauss-Seidel solvers (Ball2D discs, RigidBody2D
// circles): the Fischer-Burmeister error in the mu-scaled self-dual cone (De Saxce change of variable,
// the residual of the solve) and the local solve of u = W r + b (take-off, stick, slide), restated from
// the published method (Daviet, Bertails-Descoubes & Boissieux 2011) that So-bogus implements.
#pragma once

namespace sg {

// Fischer-Burmeister Coulomb error (mu-scaled self-dual cone, De Saxce change of
// variable); normal component first.
__device__ __forceinline__ double fb_error_2d(double r0, double r1, double u0, double u1, double mu) {
  const double nut = sqrt(u1 * u1);
  if (mu == 0.0) {
    const double fn = r0 + u0 - sqrt(r0 * r0 + u0 * u0);
    double e2 = fn * fn;
    e2 += r1 * r1;
    return sqrt(e2);
  }
  const double x0 = mu * r0, x1 = r1;
  const double y0 = u0 + mu * nut, y1 = mu * u1;
  double z0 = 0.0;
  z0 += x0 * x0;
  z0 += x1 * x1;
  z0 += y0 * y0;
  z0 += y1 * y1;
  const double zb = 2.0 * (x0 * x1 + y0 * y1);
  double nzb2 = 0.0;
  nzb2 += zb * zb;
  const double nzb = sqrt(nzb2);
  double l1 = z0 - nzb;
  if (l1 < 0.0) l1 = 0.0;
  const double l2 = z0 + nzb;
  const double s1 = sqrt(l1), s2 = sqrt(l2);
  const double sq0 = 0.5 * (s1 + s2);
  const double half_diff = 0.5 * (s2 - s1);
  const double sq1 = (nzb > 0.0) ? half_diff * (zb / nzb) : half_diff;
  double e2 = 0.0;
  const double p0 = x0 + y0 - sq0;
  e2 += p0 * p0;
  const double p1 = x1 + y1 - sq1;
  e2 += p1 * p1;
  return sqrt(e2);
}

// Local 2x2 Coulomb problem u = W r + b: take-off, stick, slide (+/-), else the
// admissible candidate with the smallest FB error.
// The local solve for an isotropic block W = w I (a disc contact: no rotation, so the normal and
// tangent rows have the same inverse-mass weight and no coupling): take-off when b0 >= 0, else the
// stick impulse -b / w clamped onto the friction cone's edge on the side of its tangential part.
// It agrees with local_solve_2d on such blocks to rounding; the FP32 form's FP64 sweeps use it.
__device__ __forceinline__ void local_solve_2d_iso(double w, double b0, double b1, double mu, double& r0,
                                                   double& r1) {
  if (b0 >= 0.0) {
    r0 = 0.0;
    r1 = 0.0;
    return;
  }
  const double inv = 1.0 / w;
  const double rn = -b0 * inv, rt = -b1 * inv, lim = mu * rn;
  r0 = rn;
  r1 = fabs(rt) <= lim ? rt : copysign(lim, rt);
}

__device__ __forceinline__ void local_solve_2d(double w00, double w01, double w11, double b0, double b1, double mu,
                                               double& r0, double& r1) {
  if (b0 >= 0.0) {
    r0 = 0.0;
    r1 = 0.0;
    return;
  }
  const double det = w00 * w11 - w01 * w01;
  const double rs0 = (w01 * b1 - w11 * b0) / det;
  const double rs1 = (w01 * b0 - w00 * b1) / det;
  if (rs0 >= 0.0 && fabs(rs1) <= mu * rs0) {
    r0 = rs0;
    r1 = rs1;
    return;
  }
  double c0[2], c1[2];
  bool have[2] = {false, false};
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const double s = (k == 0) ? 1.0 : -1.0;
    const double den = w00 - s * mu * w01;
    if (!(den > 0.0)) continue;
    const double rn = -b0 / den;
    const double rt = -s * mu * rn;
    const double ut = w01 * rn + w11 * rt + b1;
    c0[k] = rn;
    c1[k] = rt;
    have[k] = true;
    if (s * ut >= 0.0) {
      r0 = rn;
      r1 = rt;
      return;
    }
  }
  double best = INFINITY, br0 = 0.0, br1 = 0.0;
  {
    const double e = fb_error_2d(0.0, 0.0, b0, b1, mu);
    if (e < best) {
      best = e;
      br0 = 0.0;
      br1 = 0.0;
    }
  }
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    if (!have[k]) continue;
    const double u0 = w00 * c0[k] + w01 * c1[k] + b0;
    const double u1 = w01 * c0[k] + w11 * c1[k] + b1;
    const double e = fb_error_2d(c0[k], c1[k], u0, u1, mu);
    if (e < best) {
      best = e;
      br0 = c0[k];
      br1 = c1[k];
    }
  }
  r0 = br0;
  r1 = br1;
}

}  // namespace sg
