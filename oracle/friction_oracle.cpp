// friction_oracle.cpp -- CPU oracle: block Gauss-Seidel Coulomb solve.
//
// TEST INFRASTRUCTURE ONLY (see oracle.h).
//
// Restates SCISim's So-bogus friction path:
//   Sobogus::solve                       scisim/ConstrainedMaps/Sobogus.cpp:880-1088
//   SobogusFrictionProblem::initialize2D scisim/ConstrainedMaps/Sobogus.cpp:40-108
//   SobogusFrictionProblem::solve2D      scisim/ConstrainedMaps/Sobogus.cpp:273-373
//   Balls2DSobogusInterface::fromPrimal  scisim/ConstrainedMaps/bogus/Ball2DSobogusInterface.cpp:31-94
//   Balls2DSobogusInterface::solve       scisim/ConstrainedMaps/bogus/Ball2DSobogusInterface.cpp:102-148
//   GaussSeidel best-iterate + iteration count: scripts_include/sobogus_patch.patch:60-70
//
// So-bogus itself (rev 99f279d, not vendored) holds the Delassus product, the
// GS sweep, the SOC Coulomb law and its residual.  They are restated from the
// published method (Daviet, Bertails-Descoubes & Boissieux, "A hybrid iterative
// solver for robustly capturing Coulomb friction in hair dynamics", 2011):
//  * dual problem u = W r + b with W = H M^-1 H^T, b = E^T w + H v0
//    (evaluated matrix-free through body velocities v = v0 + M^-1 H^T r),
//  * sequential block GS over contacts in active-set order (colouring is off in
//    SCISim: Ball2DSobogusInterface.cpp:127 passes max_threads = 0),
//  * per-contact analytic local solve (take-off / stick / slide),
//  * error = max over contacts of the Euclidean norm of the SOC
//    Fischer-Burmeister function of (r, u + mu |u_T| e_n) in the mu-scaled
//    self-dual cone (parity unpinned: So-bogus's exact scale is not available).
#include "oracle.h"

#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// Fischer-Burmeister function on the unit Lorentz cone K1 of dimension D.
// x, y in K1; phi = x + y - sqrt(x o x + y o y) (Jordan algebra).
template <int D>
double fb_norm_k1(const double* x, const double* y) {
  // z = x o x + y o y = (|x|^2 + |y|^2, 2 (x0 xbar + y0 ybar))
  double z0 = 0.0;
  for (int i = 0; i < D; ++i) z0 += x[i] * x[i];
  for (int i = 0; i < D; ++i) z0 += y[i] * y[i];
  double zb[D - 1];
  double nzb2 = 0.0;
  for (int i = 1; i < D; ++i) {
    zb[i - 1] = 2.0 * (x[0] * x[i] + y[0] * y[i]);
    nzb2 += zb[i - 1] * zb[i - 1];
  }
  const double nzb = std::sqrt(nzb2);
  double l1 = z0 - nzb;
  if (l1 < 0.0) l1 = 0.0;
  const double l2 = z0 + nzb;
  const double s1 = std::sqrt(l1), s2 = std::sqrt(l2);
  double sq[D];
  sq[0] = 0.5 * (s1 + s2);
  const double half_diff = 0.5 * (s2 - s1);
  for (int i = 1; i < D; ++i) sq[i] = (nzb > 0.0) ? half_diff * (zb[i - 1] / nzb) : (i == 1 ? half_diff : 0.0);
  double e2 = 0.0;
  for (int i = 0; i < D; ++i) {
    const double phi = x[i] + y[i] - sq[i];
    e2 += phi * phi;
  }
  return std::sqrt(e2);
}

// Coulomb error of local impulse r and local velocity u (both D, normal first).
template <int D>
double fb_error(const double* r, const double* u, double mu) {
  double ut2 = 0.0;
  for (int i = 1; i < D; ++i) ut2 += u[i] * u[i];
  const double nut = std::sqrt(ut2);
  if (mu == 0.0) {
    // Frictionless: scalar FB on (r_n, u_n); tangential impulse must vanish.
    const double fn = r[0] + u[0] - std::sqrt(r[0] * r[0] + u[0] * u[0]);
    double e2 = fn * fn;
    for (int i = 1; i < D; ++i) e2 += r[i] * r[i];
    return std::sqrt(e2);
  }
  // De Saxce change of variable: ut = u + mu |u_T| e_n, then map K_mu -> K1:
  // x = (mu r_n, r_T), y = (ut_n, mu u_T).
  double x[D], y[D];
  x[0] = mu * r[0];
  y[0] = u[0] + mu * nut;
  for (int i = 1; i < D; ++i) {
    x[i] = r[i];
    y[i] = mu * u[i];
  }
  return fb_norm_k1<D>(x, y);
}

// ---------------------------------------------------------------------------
// 2D local Coulomb solve, W = [w00 w01; w01 w11] SPD.
void local_solve_2d(const double* W, const double* b, double mu, double* r) {
  // Take-off: r = 0, u = b admissible iff b_n >= 0.
  if (b[0] >= 0.0) {
    r[0] = 0.0;
    r[1] = 0.0;
    return;
  }
  const double w00 = W[0], w01 = W[1], w11 = W[2];
  // Stick: u = 0, r = -W^-1 b.
  const double det = w00 * w11 - w01 * w01;
  const double rs0 = (w01 * b[1] - w11 * b[0]) / det;
  const double rs1 = (w01 * b[0] - w00 * b[1]) / det;
  if (rs0 >= 0.0 && std::fabs(rs1) <= mu * rs0) {
    r[0] = rs0;
    r[1] = rs1;
    return;
  }
  // Slide: u_n = 0, r_t = -s mu r_n, sign(u_t) = s.
  double cand[2][2];
  bool have[2] = {false, false};
  for (int k = 0; k < 2; ++k) {
    const double s = (k == 0) ? 1.0 : -1.0;
    const double den = w00 - s * mu * w01;
    if (!(den > 0.0)) continue;
    const double rn = -b[0] / den;
    const double rt = -s * mu * rn;
    const double ut = w01 * rn + w11 * rt + b[1];
    cand[k][0] = rn;
    cand[k][1] = rt;
    have[k] = true;
    if (s * ut >= 0.0) {
      r[0] = rn;
      r[1] = rt;
      return;
    }
  }
  // Degenerate: keep the admissible candidate with the smallest error.
  double best = std::numeric_limits<double>::infinity();
  double br[2] = {0.0, 0.0};
  auto consider = [&](double c0, double c1) {
    const double rc[2] = {c0, c1};
    const double u[2] = {w00 * c0 + w01 * c1 + b[0], w01 * c0 + w11 * c1 + b[1]};
    const double e = fb_error<2>(rc, u, mu);
    if (e < best) {
      best = e;
      br[0] = c0;
      br[1] = c1;
    }
  };
  consider(0.0, 0.0);
  for (int k = 0; k < 2; ++k)
    if (have[k]) consider(cand[k][0], cand[k][1]);
  r[0] = br[0];
  r[1] = br[1];
}

// 3D local Coulomb solve, W symmetric SPD stored as w00 w01 w02 w11 w12 w22.
void local_solve_3d(const double* W, const double* b, double mu, double* r) {
  if (b[0] >= 0.0) {
    r[0] = r[1] = r[2] = 0.0;
    return;
  }
  const double a00 = W[0], a01 = W[1], a02 = W[2], a11 = W[3], a12 = W[4], a22 = W[5];
  // Stick: solve W r = -b by the adjugate.
  const double c00 = a11 * a22 - a12 * a12;
  const double c01 = a02 * a12 - a01 * a22;
  const double c02 = a01 * a12 - a02 * a11;
  const double c11 = a00 * a22 - a02 * a02;
  const double c12 = a01 * a02 - a00 * a12;
  const double c22 = a00 * a11 - a01 * a01;
  const double det = a00 * c00 + a01 * c01 + a02 * c02;
  const double rs0 = -(c00 * b[0] + c01 * b[1] + c02 * b[2]) / det;
  const double rs1 = -(c01 * b[0] + c11 * b[1] + c12 * b[2]) / det;
  const double rs2 = -(c02 * b[0] + c12 * b[1] + c22 * b[2]) / det;
  if (rs0 >= 0.0 && std::sqrt(rs1 * rs1 + rs2 * rs2) <= mu * rs0) {
    r[0] = rs0;
    r[1] = rs1;
    r[2] = rs2;
    return;
  }
  // Slide: u_n = 0, r_T = -mu r_n d with |d| = 1, u_T = alpha d with alpha >= 0.  For a given
  // r_n, (alpha I + mu r_n W_TT) d = W_Tn r_n + b_T =: g, and |d(alpha)|^2 - 1 is convex and
  // decreasing in alpha, so Newton from alpha = 0 climbs monotonically to the root.  r_n
  // follows from the normal row, r_n (W_nn - mu W_nT . d) = -b_n; the two are iterated.
  double d0 = 1.0, d1 = 0.0;
  double rn = -b[0] / a00, rt0 = 0.0, rt1 = 0.0, ut0 = 0.0, ut1 = 0.0;
  bool slide_ok = false;
  if (mu == 0.0) {
    rt0 = 0.0;
    rt1 = 0.0;
    slide_ok = true;
  } else {
    for (int outer = 0; outer < 8; ++outer) {
      const double c = mu * rn;
      const double g0 = a01 * rn + b[1], g1 = a02 * rn + b[2];
      const double m00 = c * a11, m01 = c * a12, m11 = c * a22;
      // Start at alpha = |g| - lambda_max(c W_TT) (the root when W_TT is isotropic), which
      // is never right of the root.
      const double hs = 0.5 * (m00 + m11), hd = 0.5 * (m00 - m11);
      const double lmax = hs + std::sqrt(hd * hd + m01 * m01);
      double al = std::sqrt(g0 * g0 + g1 * g1) - lmax;
      if (!(al > 0.0)) al = 0.0;
      double e0 = 0.0, e1 = 0.0;
      for (int it = 0; it < 64; ++it) {
        const double p00 = al + m00, p11 = al + m11;
        const double inv = 1.0 / (p00 * p11 - m01 * m01);
        e0 = (p11 * g0 - m01 * g1) * inv;
        e1 = (p00 * g1 - m01 * g0) * inv;
        const double f = e0 * e0 + e1 * e1 - 1.0;
        const double q0 = (p11 * e0 - m01 * e1) * inv, q1 = (p00 * e1 - m01 * e0) * inv;
        const double fp = -2.0 * (e0 * q0 + e1 * q1);
        if (!(f > 0.0) || !(fp < 0.0)) break;
        const double step = -f / fp;
        al = al + step;
        if (!(step > 1.0e-15 * (1.0 + al))) {
          const double p00n = al + m00, p11n = al + m11;
          const double invn = 1.0 / (p00n * p11n - m01 * m01);
          e0 = (p11n * g0 - m01 * g1) * invn;
          e1 = (p00n * g1 - m01 * g0) * invn;
          break;
        }
      }
      const double ne = std::sqrt(e0 * e0 + e1 * e1);
      if (!(ne > 0.0)) break;
      d0 = e0 / ne;
      d1 = e1 / ne;
      const double den = a00 - mu * (a01 * d0 + a02 * d1);
      if (!(den > 0.0)) break;
      const double rn_new = -b[0] / den;
      const bool same = std::fabs(rn_new - rn) <= 1.0e-15 * std::fabs(rn_new);
      rn = rn_new;
      if (same) {
        slide_ok = true;
        break;
      }
    }
    rt0 = -mu * rn * d0;
    rt1 = -mu * rn * d1;
  }
  ut0 = a01 * rn + a11 * rt0 + a12 * rt1 + b[1];
  ut1 = a02 * rn + a12 * rt0 + a22 * rt1 + b[2];
  if (slide_ok && rn >= 0.0 && (mu == 0.0 || (ut0 * d0 + ut1 * d1) >= 0.0)) {
    r[0] = rn;
    r[1] = rt0;
    r[2] = rt1;
    return;
  }
  // Anisotropic fallback: root search on the sliding direction.  d(s) runs over
  // the unit circle through the rational chart d = +-((1-s^2), 2s)/(1+s^2),
  // s in [-1, 1] per half circle (no trigonometry); g(d) = u_T x d must vanish
  // with u_T . d >= 0 and r_n >= 0.  Sign changes on a 256-point grid per half are
  // refined by bisection; the root with the smallest Coulomb error is kept.
  {
    auto eval = [&](double s, double sign, double* out) -> bool {
      const double den_s = 1.0 + s * s;
      const double e0 = sign * (1.0 - s * s) / den_s, e1 = sign * (2.0 * s) / den_s;
      const double den = a00 - mu * (a01 * e0 + a02 * e1);
      if (!(den > 0.0)) return false;
      const double n_ = -b[0] / den;
      const double t0 = -mu * n_ * e0, t1 = -mu * n_ * e1;
      const double v0 = a01 * n_ + a11 * t0 + a12 * t1 + b[1];
      const double v1 = a02 * n_ + a12 * t0 + a22 * t1 + b[2];
      out[0] = v0 * e1 - v1 * e0;  // g
      out[1] = v0 * e0 + v1 * e1;  // h
      out[2] = n_;
      out[3] = t0;
      out[4] = t1;
      return true;
    };
    double best_e = std::numeric_limits<double>::infinity();
    double best_r[3] = {0.0, 0.0, 0.0};
    constexpr int kGrid = 256;
    for (int half = 0; half < 2; ++half) {
      const double sign = half == 0 ? 1.0 : -1.0;
      double s_prev = -1.0, f_prev[5];
      bool ok_prev = eval(s_prev, sign, f_prev);
      for (int k = 1; k <= kGrid; ++k) {
        const double s_cur = -1.0 + 2.0 * double(k) / double(kGrid);
        double f_cur[5];
        const bool ok_cur = eval(s_cur, sign, f_cur);
        if (ok_prev && ok_cur && ((f_prev[0] <= 0.0) != (f_cur[0] <= 0.0))) {
          double lo = s_prev, hi = s_cur, flo = f_prev[0];
          double fm[5] = {f_cur[0], f_cur[1], f_cur[2], f_cur[3], f_cur[4]};
          for (int it = 0; it < 80; ++it) {
            const double mid = 0.5 * (lo + hi);
            if (!eval(mid, sign, fm)) break;
            if ((fm[0] <= 0.0) == (flo <= 0.0)) {
              lo = mid;
              flo = fm[0];
            } else {
              hi = mid;
            }
          }
          if (fm[1] >= 0.0 && fm[2] >= 0.0) {
            const double rc[3] = {fm[2], fm[3], fm[4]};
            const double u[3] = {a00 * rc[0] + a01 * rc[1] + a02 * rc[2] + b[0],
                                 a01 * rc[0] + a11 * rc[1] + a12 * rc[2] + b[1],
                                 a02 * rc[0] + a12 * rc[1] + a22 * rc[2] + b[2]};
            const double e = fb_error<3>(rc, u, mu);
            if (e < best_e) {
              best_e = e;
              best_r[0] = rc[0];
              best_r[1] = rc[1];
              best_r[2] = rc[2];
            }
          }
        }
        s_prev = s_cur;
        ok_prev = ok_cur;
        for (int i = 0; i < 5; ++i) f_prev[i] = f_cur[i];
      }
    }
    if (best_e < std::numeric_limits<double>::infinity()) {
      r[0] = best_r[0];
      r[1] = best_r[1];
      r[2] = best_r[2];
      return;
    }
  }
  // Degenerate: smallest-error candidate.
  double best = std::numeric_limits<double>::infinity();
  double br[3] = {0.0, 0.0, 0.0};
  auto consider = [&](double x0, double x1, double x2) {
    const double rc[3] = {x0, x1, x2};
    const double u[3] = {a00 * x0 + a01 * x1 + a02 * x2 + b[0], a01 * x0 + a11 * x1 + a12 * x2 + b[1],
                         a02 * x0 + a12 * x1 + a22 * x2 + b[2]};
    const double e = fb_error<3>(rc, u, mu);
    if (e < best) {
      best = e;
      br[0] = x0;
      br[1] = x1;
      br[2] = x2;
    }
  };
  consider(0.0, 0.0, 0.0);
  if (rs0 >= 0.0) {
    const double nt = std::sqrt(rs1 * rs1 + rs2 * rs2);
    const double sc = (nt > mu * rs0 && nt > 0.0) ? (mu * rs0) / nt : 1.0;
    consider(rs0, rs1 * sc, rs2 * sc);
  }
  if (slide_ok && rn >= 0.0) consider(rn, rt0, rt1);
  r[0] = br[0];
  r[1] = br[1];
  r[2] = br[2];
}

}  // namespace

// ---------------------------------------------------------------------------
extern "C" double or_fb_error(int dim, const double* r, const double* u, double mu) {
  return dim == 2 ? fb_error<2>(r, u, mu) : fb_error<3>(r, u, mu);
}

extern "C" void or_local_solve(int dim, const double* W, const double* b, double mu, double* r) {
  if (dim == 2)
    local_solve_2d(W, b, mu, r);
  else
    local_solve_3d(W, b, mu, r);
}

// ---------------------------------------------------------------------------
// Ball2D Sobogus::solve.  eval_only: set up from (alpha, beta) and return the
// residual of that impulse without iterating.
static double solve2d_impl(int nb, const double* m, const double* v0, int nc, const int32_t* ia, const int32_t* ib,
                           const double* bases, const double* CoR, const double* mu, const or_gs_params* p,
                           double* alpha, double* beta, double* v2, double* f, or_gs_result* res, bool eval_only,
                           const double* nrel_in = nullptr, const double* drel_in = nullptr);

extern "C" void or_sobogus_solve_2d(int nb, const double* m, const double* v0, int nc, const int32_t* ia,
                                    const int32_t* ib, const double* bases, const double* CoR,
                                    const double* mu, const or_gs_params* p, double* alpha, double* beta,
                                    double* v2, double* f, or_gs_result* res) {
  solve2d_impl(nb, m, v0, nc, ia, ib, bases, CoR, mu, p, alpha, beta, v2, f, res, false);
}

// With the extra relative velocities of the map (FrictionSolver::solve's nrel_extra, drel_extra;
// SymplecticEulerImpactFrictionMap.cpp:293-321).
extern "C" void or_sobogus_solve_2d_ex(int nb, const double* m, const double* v0, int nc, const int32_t* ia,
                                       const int32_t* ib, const double* bases, const double* CoR, const double* mu,
                                       const double* nrel, const double* drel, const or_gs_params* p, double* alpha,
                                       double* beta, double* v2, double* f, or_gs_result* res) {
  solve2d_impl(nb, m, v0, nc, ia, ib, bases, CoR, mu, p, alpha, beta, v2, f, res, false, nrel, drel);
}

extern "C" double or_residual_2d(int nb, const double* m, const double* v0, int nc, const int32_t* ia,
                                 const int32_t* ib, const double* bases, const double* CoR, const double* mu,
                                 const double* alpha, const double* beta) {
  std::vector<double> a(alpha, alpha + nc), b(beta, beta + nc);
  return solve2d_impl(nb, m, v0, nc, ia, ib, bases, CoR, mu, nullptr, a.data(), b.data(), nullptr, nullptr, nullptr,
                      true);
}

// The residual with the map's extra relative velocities folded into the forcing terms.
extern "C" double or_residual_2d_ex(int nb, const double* m, const double* v0, int nc, const int32_t* ia,
                                    const int32_t* ib, const double* bases, const double* CoR, const double* mu,
                                    const double* nrel, const double* drel, const double* alpha,
                                    const double* beta) {
  std::vector<double> a(alpha, alpha + nc), b(beta, beta + nc);
  return solve2d_impl(nb, m, v0, nc, ia, ib, bases, CoR, mu, nullptr, a.data(), b.data(), nullptr, nullptr, nullptr,
                      true, nrel, drel);
}

static double solve2d_impl(int nb, const double* m, const double* v0, int nc, const int32_t* ia, const int32_t* ib,
                           const double* bases, const double* CoR, const double* mu, const or_gs_params* p,
                           double* alpha, double* beta, double* v2, double* f, or_gs_result* res, bool eval_only,
                           const double* nrel_in, const double* drel_in) {
  // Minv as the reference builds it: 1.0 / m (ball2d/Ball2DState.cpp:55-67).
  std::vector<double> minv(nb);
  for (int i = 0; i < nb; ++i) minv[i] = 1.0 / m[i];

  // Bodies touched by contacts (Sobogus.cpp:656-687): untouched bodies keep v0.
  std::vector<char> touched(nb, 0);
  for (int k = 0; k < nc; ++k) {
    touched[ia[k]] = 1;
    if (ib[k] >= 0) touched[ib[k]] = 1;
  }

  // Per-contact assembly (Sobogus.cpp:64-90, Constraint.cpp:18-34, 92-126).
  std::vector<double> N(2 * nc), T(2 * nc), C(2 * nc), Wd(3 * nc), R(2 * nc);
  for (int k = 0; k < nc; ++k) {
    const double* B = bases + 4 * k;  // column-major [n t]
    const double nx = B[0], ny = B[1], tx = B[2], ty = B[3];
    N[2 * k] = nx;
    N[2 * k + 1] = ny;
    T[2 * k] = tx;
    T[2 * k + 1] = ty;
    const int a = ia[k], bb = ib[k];
    // Relative velocity v_a - v_b (static plane velocity is zero).
    double vrx = v0[2 * a], vry = v0[2 * a + 1];
    if (bb >= 0) {
      vrx = vrx - v0[2 * bb];
      vry = vry - v0[2 * bb + 1];
    } else {
      vrx = vrx - 0.0;
      vry = vry - 0.0;
    }
    const double ndotv = nx * vrx + ny * vry;
    // Kinematic relative velocity is zero for balls and static planes:
    // nrel = -(0 . n), drel = -(0 . t)  (Constraint.cpp:110-123).
    // Kinematic relative velocities, plus the map's extra ones (Sobogus.cpp:890-904).
    double nrel = -(0.0 * nx + 0.0 * ny);
    double drel = -(0.0 * tx + 0.0 * ty);
    if (nrel_in) nrel = nrel + nrel_in[k];
    if (drel_in) drel = drel + drel_in[k];
    // Forcing term w = n (CoR ndotv + nrel) + t drel (Constraint.cpp:27-33).
    const double s = CoR[k] * ndotv + nrel;
    const double wx = (0.0 + nx * s) + tx * drel;
    const double wy = (0.0 + ny * s) + ty * drel;
    // Local forcing E^T w.
    C[2 * k] = nx * wx + ny * wy;
    C[2 * k + 1] = tx * wx + ty * wy;
    // Diagonal Delassus block: sum over bodies of B Minv B^T (H rows [n^T; t^T]).
    const double nn = nx * nx + ny * ny;
    const double nt = nx * tx + ny * ty;
    const double tt = tx * tx + ty * ty;
    double w00 = minv[a] * nn, w01 = minv[a] * nt, w11 = minv[a] * tt;
    if (bb >= 0) {
      w00 = w00 + minv[bb] * nn;
      w01 = w01 + minv[bb] * nt;
      w11 = w11 + minv[bb] * tt;
    }
    Wd[3 * k] = w00;
    Wd[3 * k + 1] = w01;
    Wd[3 * k + 2] = w11;
    // Warm start r = alpha n + beta t, then r_loc = E^T r (Sobogus.cpp:299-301,
    // Ball2DSobogusInterface.cpp:115).
    const double rwx = alpha[k] * nx + beta[k] * tx;
    const double rwy = alpha[k] * ny + beta[k] * ty;
    R[2 * k] = nx * rwx + ny * rwy;
    R[2 * k + 1] = tx * rwx + ty * rwy;
  }

  // Adjacency (bodies -> contacts in ascending contact order) for the
  // fixed-order gather of H^T r.
  std::vector<int> cnt(nb + 1, 0);
  for (int k = 0; k < nc; ++k) {
    cnt[ia[k] + 1]++;
    if (ib[k] >= 0) cnt[ib[k] + 1]++;
  }
  for (int i = 0; i < nb; ++i) cnt[i + 1] += cnt[i];
  std::vector<int> adj(cnt[nb]);
  {
    std::vector<int> cur(cnt.begin(), cnt.end() - 1);
    for (int k = 0; k < nc; ++k) {
      adj[cur[ia[k]]++] = k;
      if (ib[k] >= 0) adj[cur[ib[k]]++] = k;
    }
  }
  // H^T r gathered per body in ascending contact order.
  auto gather_htr = [&](int body, const std::vector<double>& Rv, double& hx, double& hy) {
    hx = 0.0;
    hy = 0.0;
    for (int e = cnt[body]; e < cnt[body + 1]; ++e) {
      const int k = adj[e];
      const double sgn = (ia[k] == body) ? 1.0 : -1.0;
      const double px = N[2 * k] * Rv[2 * k] + T[2 * k] * Rv[2 * k + 1];
      const double py = N[2 * k + 1] * Rv[2 * k] + T[2 * k + 1] * Rv[2 * k + 1];
      hx = hx + sgn * px;
      hy = hy + sgn * py;
    }
  };

  // Running body velocity v = v0 + Minv H^T r.
  std::vector<double> V(2 * nb);
  for (int i = 0; i < nb; ++i) {
    double hx, hy;
    gather_htr(i, R, hx, hy);
    V[2 * i] = v0[2 * i] + minv[i] * hx;
    V[2 * i + 1] = v0[2 * i + 1] + minv[i] * hy;
  }

  auto local_u = [&](int k, double& u0, double& u1) {
    const int a = ia[k], bb = ib[k];
    const double nx = N[2 * k], ny = N[2 * k + 1], tx = T[2 * k], ty = T[2 * k + 1];
    double hn = nx * V[2 * a] + ny * V[2 * a + 1];
    double ht = tx * V[2 * a] + ty * V[2 * a + 1];
    if (bb >= 0) {
      hn = hn - (nx * V[2 * bb] + ny * V[2 * bb + 1]);
      ht = ht - (tx * V[2 * bb] + ty * V[2 * bb + 1]);
    }
    u0 = hn + C[2 * k];
    u1 = ht + C[2 * k + 1];
  };

  auto residual = [&]() {
    double err = 0.0;
    for (int k = 0; k < nc; ++k) {
      double u[2];
      local_u(k, u[0], u[1]);
      const double e = fb_error<2>(&R[2 * k], u, mu[k]);
      if (e > err || e != e) err = e;  // a NaN error sticks as the maximum
    }
    return err;
  };

  if (eval_only) return nc == 0 ? 0.0 : residual();
  const uint32_t eval_every = p->eval_every == 0 ? 1 : p->eval_every;
  std::vector<double> Rbest(R);
  double err_best = std::numeric_limits<double>::infinity();
  uint32_t it = 0;
  bool converged = false;
  for (it = 1; it <= p->max_iters; ++it) {
    for (int s = 0; s < nc; ++s) {
      const int k = p->order ? p->order[s] : s;
      const int a = ia[k], bb = ib[k];
      double u[2];
      local_u(k, u[0], u[1]);
      const double r0 = R[2 * k], r1 = R[2 * k + 1];
      const double* W = &Wd[3 * k];
      const double bt[2] = {u[0] - (W[0] * r0 + W[1] * r1), u[1] - (W[1] * r0 + W[2] * r1)};
      double rn[2];
      local_solve_2d(W, bt, mu[k], rn);
      const double d0 = rn[0] - r0, d1 = rn[1] - r1;
      const double nx = N[2 * k], ny = N[2 * k + 1], tx = T[2 * k], ty = T[2 * k + 1];
      const double px = nx * d0 + tx * d1;
      const double py = ny * d0 + ty * d1;
      V[2 * a] = V[2 * a] + minv[a] * px;
      V[2 * a + 1] = V[2 * a + 1] + minv[a] * py;
      if (bb >= 0) {
        V[2 * bb] = V[2 * bb] - minv[bb] * px;
        V[2 * bb + 1] = V[2 * bb + 1] - minv[bb] * py;
      }
      R[2 * k] = rn[0];
      R[2 * k + 1] = rn[1];
    }
    if (it % eval_every == 0) {
      const double err = residual();
      if (err < err_best) {
        err_best = err;
        Rbest = R;
      }
      if (err < p->tol) {
        converged = true;
        break;
      }
    }
  }
  if (!converged) {
    // Best evaluated iterate (So-bogus GaussSeidel: x = x_best when GSIter > maxIters).
    if (err_best < std::numeric_limits<double>::infinity()) R = Rbest;
    it = p->max_iters;
  }
  if (nc == 0) err_best = 0.0;

  // Outgoing velocity v = Minv (H^T r - f), f = -M v0 (Ball2DSobogusInterface.cpp:142).
  for (int i = 0; i < nb; ++i) {
    if (!touched[i]) {
      v2[2 * i] = v0[2 * i];
      v2[2 * i + 1] = v0[2 * i + 1];
      continue;
    }
    double hx, hy;
    gather_htr(i, R, hx, hy);
    const double fx = -(m[i] * v0[2 * i]);
    const double fy = -(m[i] * v0[2 * i + 1]);
    v2[2 * i] = minv[i] * (hx - fx);
    v2[2 * i + 1] = minv[i] * (hy - fy);
  }

  // r back to world coordinates and impulse extraction (Sobogus.cpp:309-347).
  for (int i = 0; i < 2 * nb; ++i) f[i] = 0.0;
  for (int k = 0; k < nc; ++k) {
    const double nx = N[2 * k], ny = N[2 * k + 1], tx = T[2 * k], ty = T[2 * k + 1];
    const double rwx = nx * R[2 * k] + tx * R[2 * k + 1];
    const double rwy = ny * R[2 * k] + ty * R[2 * k + 1];
    alpha[k] = rwx * nx + rwy * ny;
    beta[k] = (mu[k] == 0.0) ? 0.0 : (rwx * tx + rwy * ty);
    const double f0x = beta[k] * tx, f0y = beta[k] * ty;
    f[2 * ia[k]] += f0x;
    f[2 * ia[k] + 1] += f0y;
    if (ib[k] >= 0) {
      f[2 * ib[k]] -= f0x;
      f[2 * ib[k] + 1] -= f0y;
    }
  }
  res->error = err_best;
  res->iterations = it;
  res->succeeded = err_best < p->tol ? 1 : 0;
  return err_best;
}
