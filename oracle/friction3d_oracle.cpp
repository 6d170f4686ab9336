// friction3d_oracle.cpp -- CPU oracle: block Gauss-Seidel Coulomb solve for 3D rigid bodies.
//
// TEST INFRASTRUCTURE ONLY (see oracle.h).
//
// Restates SCISim's So-bogus path for RigidBodies3D:
//   SobogusFrictionProblem::initialize3D   scisim/ConstrainedMaps/Sobogus.cpp:184-251
//   SobogusFrictionProblem::solve3D        scisim/ConstrainedMaps/Sobogus.cpp:486-594
//   RigidBodies3DSobogusInterface          scisim/ConstrainedMaps/bogus/RigidBody3DSobogusInterface.cpp:31-145
//   H rows (sphere-sphere, plane-sphere)   rigidbody3d/Constraints/SphereSphereConstraint.cpp:229-271,
//                                          rigidbody3d/Constraints/StaticPlaneSphereConstraint.cpp:197-221
// with the same matrix-free block GS as the 2D oracle (friction_oracle.cpp), 3x3 blocks:
// body b has 6 velocity dofs (v, omega), inverse mass minv and world inverse inertia Iinv
// (3x3, row-major).  Contact k: basis [n s t] (column-major 3x3), arms ra = p - x_a and
// rb = p - x_b (plane contacts: ra = -r n).  H_a = [n^T 0; s^T (ra x s)^T; t^T (ra x t)^T],
// H_b the same with rb, entering with a minus sign.
#include "oracle.h"

#include <cmath>
#include <limits>
#include <vector>

namespace {

inline void cross3(const double* a, const double* b, double* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
inline double dot3(const double* a, const double* b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
inline void matvec3(const double* M, const double* x, double* y) {
  for (int i = 0; i < 3; ++i) y[i] = (M[3 * i] * x[0] + M[3 * i + 1] * x[1]) + M[3 * i + 2] * x[2];
}

struct Contact3 {
  double B[3][3];   // rows n, s, t
  double Aa[3][3];  // angular rows for body a: 0, ra x s, ra x t
  double Ab[3][3];  // angular rows for body b
  double c[3];      // local forcing E^T w
  double W[6];      // w00 w01 w02 w11 w12 w22
};

}  // namespace

extern "C" void or_local_solve(int dim, const double* W, const double* b, double mu, double* r);
extern "C" double or_fb_error(int dim, const double* r, const double* u, double mu);

// ---------------------------------------------------------------------------
static double solve3d_impl(int nb, const double* m, const double* Iinv, const double* Iw, const double* v0, int nc,
                           const int32_t* ia, const int32_t* ib, const double* bases, const double* arm_a,
                           const double* arm_b, const double* CoR, const double* mu, const or_gs_params* p,
                           double* alpha, double* beta, double* v2, double* f, or_gs_result* res, bool eval_only,
                           const double* nrel_in = nullptr, const double* drel_in = nullptr) {
  std::vector<double> minv(nb);
  for (int i = 0; i < nb; ++i) minv[i] = 1.0 / m[i];
  std::vector<char> touched(nb, 0);
  for (int k = 0; k < nc; ++k) {
    touched[ia[k]] = 1;
    if (ib[k] >= 0) touched[ib[k]] = 1;
  }
  std::vector<Contact3> C(nc);
  std::vector<double> R(3 * nc);
  for (int k = 0; k < nc; ++k) {
    Contact3& ct = C[k];
    const double* E = bases + 9 * k;  // column-major: columns n, s, t
    for (int row = 0; row < 3; ++row)
      for (int j = 0; j < 3; ++j) ct.B[row][j] = E[3 * row + j];
    const double* n = ct.B[0];
    const double* s = ct.B[1];
    const double* t = ct.B[2];
    const double* ra = arm_a + 3 * k;
    const double* rb = arm_b + 3 * k;
    for (int j = 0; j < 3; ++j) ct.Aa[0][j] = 0.0;
    cross3(ra, s, ct.Aa[1]);
    cross3(ra, t, ct.Aa[2]);
    for (int j = 0; j < 3; ++j) ct.Ab[0][j] = 0.0;
    cross3(rb, s, ct.Ab[1]);
    cross3(rb, t, ct.Ab[2]);
    const int a = ia[k], b = ib[k];
    // ndotv = n . (v_a - v_b): linear velocities only (n is parallel to the arms).
    double vr[3];
    for (int j = 0; j < 3; ++j) vr[j] = v0[3 * a + j] - (b >= 0 ? v0[3 * b + j] : 0.0);
    const double ndotv = dot3(n, vr);
    // Kinematic relative velocity is zero (static planes have no motion).
    const double zero3[3] = {0.0, 0.0, 0.0};
    // Plus the map's extra relative velocities when it supplies them (Sobogus.cpp:890-904).
    double nrel = -dot3(zero3, n);
    double drel0 = -dot3(zero3, s), drel1 = -dot3(zero3, t);
    if (nrel_in) nrel = nrel + nrel_in[k];
    if (drel_in) {
      drel0 = drel0 + drel_in[2 * k];
      drel1 = drel1 + drel_in[2 * k + 1];
    }
    const double sc = CoR[k] * ndotv + nrel;
    double w[3];
    for (int j = 0; j < 3; ++j) w[j] = ((0.0 + n[j] * sc) + s[j] * drel0) + t[j] * drel1;
    ct.c[0] = dot3(n, w);
    ct.c[1] = dot3(s, w);
    ct.c[2] = dot3(t, w);
    // W = H_a Minv_a H_a^T + H_b Minv_b H_b^T.
    // The normal row has no angular part (n is parallel to the arms): its angular
    // terms are skipped rather than multiplied by zero.
    int q = 0;
    for (int i = 0; i < 3; ++i)
      for (int j = i; j < 3; ++j) {
        double wij = minv[a] * dot3(ct.B[i], ct.B[j]);
        if (i > 0) {
          double Ia[3];
          matvec3(&Iinv[9 * a], ct.Aa[j], Ia);
          wij = wij + dot3(ct.Aa[i], Ia);
        }
        if (b >= 0) {
          double wb = minv[b] * dot3(ct.B[i], ct.B[j]);
          if (i > 0) {
            double Ib[3];
            matvec3(&Iinv[9 * b], ct.Ab[j], Ib);
            wb = wb + dot3(ct.Ab[i], Ib);
          }
          wij = wij + wb;
        }
        ct.W[q++] = wij;
      }
    // Warm start r = alpha n + beta0 s + beta1 t, then r_loc = E^T r.
    double rw[3];
    for (int j = 0; j < 3; ++j) rw[j] = (alpha[k] * n[j] + beta[2 * k] * s[j]) + beta[2 * k + 1] * t[j];
    R[3 * k] = dot3(n, rw);
    R[3 * k + 1] = dot3(s, rw);
    R[3 * k + 2] = dot3(t, rw);
  }
  // Adjacency (ascending contact order per body).
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
  // H^T r per body: linear part B^T r, angular part A^T r, signed.
  auto gather = [&](int body, const std::vector<double>& Rv, double* hl, double* ha) {
    for (int j = 0; j < 3; ++j) hl[j] = ha[j] = 0.0;
    for (int e = cnt[body]; e < cnt[body + 1]; ++e) {
      const int k = adj[e];
      const bool is_a = ia[k] == body;
      const double sgn = is_a ? 1.0 : -1.0;
      const Contact3& ct = C[k];
      const double (*A)[3] = is_a ? ct.Aa : ct.Ab;
      const double* rk = &Rv[3 * k];
      for (int j = 0; j < 3; ++j) {
        const double pl = (ct.B[0][j] * rk[0] + ct.B[1][j] * rk[1]) + ct.B[2][j] * rk[2];
        const double pa = A[1][j] * rk[1] + A[2][j] * rk[2];
        hl[j] = hl[j] + sgn * pl;
        ha[j] = ha[j] + sgn * pa;
      }
    }
  };
  // Running velocities v = v0 + Minv H^T r (linear block then angular block).
  std::vector<double> V(6 * nb);
  for (int i = 0; i < nb; ++i) {
    double hl[3], ha[3], wa[3];
    gather(i, R, hl, ha);
    matvec3(&Iinv[9 * i], ha, wa);
    for (int j = 0; j < 3; ++j) {
      V[3 * i + j] = v0[3 * i + j] + minv[i] * hl[j];
      V[3 * nb + 3 * i + j] = v0[3 * nb + 3 * i + j] + wa[j];
    }
  }
  auto local_u = [&](int k, double* u) {
    const Contact3& ct = C[k];
    const int a = ia[k], b = ib[k];
    for (int i = 0; i < 3; ++i) {
      double h = dot3(ct.B[i], &V[3 * a]);
      if (i > 0) h = h + dot3(ct.Aa[i], &V[3 * nb + 3 * a]);
      if (b >= 0) {
        double hb = dot3(ct.B[i], &V[3 * b]);
        if (i > 0) hb = hb + dot3(ct.Ab[i], &V[3 * nb + 3 * b]);
        h = h - hb;
      }
      u[i] = h + ct.c[i];
    }
  };
  auto residual = [&]() {
    double err = 0.0;
    for (int k = 0; k < nc; ++k) {
      double u[3];
      local_u(k, u);
      const double e = or_fb_error(3, &R[3 * k], u, mu[k]);
      if (e > err || e != e) err = e;
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
    for (int sidx = 0; sidx < nc; ++sidx) {
      const int k = p->order ? p->order[sidx] : sidx;
      const Contact3& ct = C[k];
      const int a = ia[k], b = ib[k];
      double u[3];
      local_u(k, u);
      const double* W = ct.W;
      const double r0 = R[3 * k], r1 = R[3 * k + 1], r2 = R[3 * k + 2];
      const double bt[3] = {u[0] - ((W[0] * r0 + W[1] * r1) + W[2] * r2),
                            u[1] - ((W[1] * r0 + W[3] * r1) + W[4] * r2),
                            u[2] - ((W[2] * r0 + W[4] * r1) + W[5] * r2)};
      double rn[3];
      or_local_solve(3, W, bt, mu[k], rn);
      const double d[3] = {rn[0] - r0, rn[1] - r1, rn[2] - r2};
      double pl[3], pa[3], pb[3];
      for (int j = 0; j < 3; ++j) {
        pl[j] = (ct.B[0][j] * d[0] + ct.B[1][j] * d[1]) + ct.B[2][j] * d[2];
        pa[j] = ct.Aa[1][j] * d[1] + ct.Aa[2][j] * d[2];
        pb[j] = ct.Ab[1][j] * d[1] + ct.Ab[2][j] * d[2];
      }
      double wa[3];
      matvec3(&Iinv[9 * a], pa, wa);
      for (int j = 0; j < 3; ++j) {
        V[3 * a + j] = V[3 * a + j] + minv[a] * pl[j];
        V[3 * nb + 3 * a + j] = V[3 * nb + 3 * a + j] + wa[j];
      }
      if (b >= 0) {
        double wb[3];
        matvec3(&Iinv[9 * b], pb, wb);
        for (int j = 0; j < 3; ++j) {
          V[3 * b + j] = V[3 * b + j] - minv[b] * pl[j];
          V[3 * nb + 3 * b + j] = V[3 * nb + 3 * b + j] - wb[j];
        }
      }
      R[3 * k] = rn[0];
      R[3 * k + 1] = rn[1];
      R[3 * k + 2] = rn[2];
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
    if (err_best < std::numeric_limits<double>::infinity()) R = Rbest;
    it = p->max_iters;
  }
  if (nc == 0) err_best = 0.0;
  // v2 = Minv (H^T r - f), f = -M v0 (M: m I and the world inertia Iw).
  for (int i = 0; i < nb; ++i) {
    if (!touched[i]) {
      for (int j = 0; j < 3; ++j) {
        v2[3 * i + j] = v0[3 * i + j];
        v2[3 * nb + 3 * i + j] = v0[3 * nb + 3 * i + j];
      }
      continue;
    }
    double hl[3], ha[3], Lw[3], rhs[3], wa[3];
    gather(i, R, hl, ha);
    matvec3(&Iw[9 * i], &v0[3 * nb + 3 * i], Lw);
    for (int j = 0; j < 3; ++j) {
      const double fl = -(m[i] * v0[3 * i + j]);
      v2[3 * i + j] = minv[i] * (hl[j] - fl);
      rhs[j] = ha[j] - (-Lw[j]);
    }
    matvec3(&Iinv[9 * i], rhs, wa);
    for (int j = 0; j < 3; ++j) v2[3 * nb + 3 * i + j] = wa[j];
  }
  // Impulses and friction force (Sobogus.cpp:526-567).
  for (int i = 0; i < 6 * nb; ++i) f[i] = 0.0;
  for (int k = 0; k < nc; ++k) {
    const Contact3& ct = C[k];
    double rw[3];
    for (int j = 0; j < 3; ++j) rw[j] = (ct.B[0][j] * R[3 * k] + ct.B[1][j] * R[3 * k + 1]) + ct.B[2][j] * R[3 * k + 2];
    alpha[k] = dot3(rw, ct.B[0]);
    const double b0 = dot3(rw, ct.B[1]), b1 = dot3(rw, ct.B[2]);
    beta[2 * k] = b0;
    beta[2 * k + 1] = b1;
    const int a = ia[k], b = ib[k];
    for (int j = 0; j < 3; ++j) {
      const double f0 = b0 * ct.B[1][j] + b1 * ct.B[2][j];
      const double ta = b0 * ct.Aa[1][j] + b1 * ct.Aa[2][j];
      f[3 * a + j] += f0;
      f[3 * nb + 3 * a + j] += ta;
      if (b >= 0) {
        const double tb = b0 * ct.Ab[1][j] + b1 * ct.Ab[2][j];
        f[3 * b + j] -= f0;
        f[3 * nb + 3 * b + j] -= tb;
      }
    }
  }
  res->error = err_best;
  res->iterations = it;
  res->succeeded = err_best < p->tol ? 1 : 0;
  return err_best;
}

extern "C" void or_sobogus_solve_3d(int nb, const double* m, const double* Iinv, const double* Iw, const double* v0,
                                    int nc, const int32_t* ia, const int32_t* ib, const double* bases,
                                    const double* arm_a, const double* arm_b, const double* CoR, const double* mu,
                                    const or_gs_params* p, double* alpha, double* beta, double* v2, double* f,
                                    or_gs_result* res) {
  solve3d_impl(nb, m, Iinv, Iw, v0, nc, ia, ib, bases, arm_a, arm_b, CoR, mu, p, alpha, beta, v2, f, res, false);
}

// With the extra relative velocities of the map (nrel: 1, drel: 2 per contact;
// SymplecticEulerImpactFrictionMap.cpp:293-321).
extern "C" void or_sobogus_solve_3d_ex(int nb, const double* m, const double* Iinv, const double* Iw,
                                       const double* v0, int nc, const int32_t* ia, const int32_t* ib,
                                       const double* bases, const double* arm_a, const double* arm_b,
                                       const double* CoR, const double* mu, const double* nrel, const double* drel,
                                       const or_gs_params* p, double* alpha, double* beta, double* v2, double* f,
                                       or_gs_result* res) {
  solve3d_impl(nb, m, Iinv, Iw, v0, nc, ia, ib, bases, arm_a, arm_b, CoR, mu, p, alpha, beta, v2, f, res, false,
               nrel, drel);
}

extern "C" double or_residual_3d(int nb, const double* m, const double* Iinv, const double* Iw, const double* v0,
                                 int nc, const int32_t* ia, const int32_t* ib, const double* bases,
                                 const double* arm_a, const double* arm_b, const double* CoR, const double* mu,
                                 const double* alpha, const double* beta) {
  std::vector<double> a(alpha, alpha + nc), b(beta, beta + 2 * nc);
  return solve3d_impl(nb, m, Iinv, Iw, v0, nc, ia, ib, bases, arm_a, arm_b, CoR, mu, nullptr, a.data(), b.data(),
                      nullptr, nullptr, nullptr, true);
}

// The residual with the map's extra relative velocities folded into the forcing terms.
extern "C" double or_residual_3d_ex(int nb, const double* m, const double* Iinv, const double* Iw, const double* v0,
                                    int nc, const int32_t* ia, const int32_t* ib, const double* bases,
                                    const double* arm_a, const double* arm_b, const double* CoR, const double* mu,
                                    const double* nrel, const double* drel, const double* alpha,
                                    const double* beta) {
  std::vector<double> a(alpha, alpha + nc), b(beta, beta + 2 * nc);
  return solve3d_impl(nb, m, Iinv, Iw, v0, nc, ia, ib, bases, arm_a, arm_b, CoR, mu, nullptr, a.data(), b.data(),
                      nullptr, nullptr, nullptr, true, nrel, drel);
}
