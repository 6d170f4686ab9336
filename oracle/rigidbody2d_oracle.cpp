// rigidbody2d_oracle.cpp -- CPU oracle: RigidBody2D circles stepped by GeometricImpactFrictionMap
// with Sobogus(RigidBody2D).
//
// TEST INFRASTRUCTURE ONLY (see oracle.h).
//
// Restates the reference's circle path of rigidbody2d:
//   SymplecticEulerMap::flow / VerletMap::flow   rigidbody2d/SymplecticEulerMap.cpp:12-31,
//                                                rigidbody2d/VerletMap.cpp:23-37
//   NearEarthGravityForce::computeForce          rigidbody2d/NearEarthGravityForce.cpp:20-28
//   CircleGeometry::computeCollisionAABB         rigidbody2d/CircleGeometry.cpp:19-23
//   RigidBody2DSim::computeActiveSet             rigidbody2d/RigidBody2DSim.cpp:696-714 (body pairs
//                                                :1066-1100 + narrow phase :248-312, planes :638-694)
//   CircleCircleConstraint                       rigidbody2d/CircleCircleConstraint.cpp (n and the
//                                                contact point p fixed at q0; evalNdotV, evalH)
//   StaticPlaneCircleConstraint                  rigidbody2d/StaticPlaneCircleConstraint.cpp
//   Constraint::computeForcingTerm               scisim/Constraints/Constraint.cpp:18-34, 92-126
//   SobogusFrictionProblem::initializeRigidBody2D scisim/ConstrainedMaps/Sobogus.cpp:110-182
//   SobogusFrictionProblem::solveRigidBody2D     scisim/ConstrainedMaps/Sobogus.cpp:375-470
//   RigidBody2DSobogusInterface::fromPrimal      scisim/ConstrainedMaps/bogus/RigidBody2DSobogusInterface.cpp:31-89
//   GeometricImpactFrictionMap::flow             scisim/ConstrainedMaps/GeometricImpactFrictionMap.cpp:267-442
//   StabilizedImpactFrictionMap::flow            scisim/ConstrainedMaps/StabilizedImpactFrictionMap.cpp:48-167
//   ConstraintCache                              rigidbody2d/ConstraintCache.cpp (keys (i, j) for circle
//                                                pairs, (plane, body) for planes)
// A body has three degrees of freedom (x, y, theta) and the mass block diag(m, m, I).  The normal
// row of a circle contact has no angular part (the normal passes through both centres); the
// tangent row's angular entry is cross(arm, t) with the arm from the body's centre to the contact
// point.  So-bogus (not vendored) holds the Delassus product, the sweep, the local solve and the
// residual; they are restated as for Ball2D in friction_oracle.cpp, on 3-dof bodies, and the
// So-bogus side is unpinned in the same way.  Kinematic bodies, boxes and portals are not part of
// this restatement.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <limits>
#include <map>
#include <utility>
#include <vector>

#include "oracle.h"

struct or_rb2d {
  int nb = 0, np = 0;
  std::vector<double> q, v;           // 3 per body
  std::vector<double> r, m, I;        // per body
  std::vector<double> minv, Iinv;     // 1 / m, 1 / I (RigidBody2DState's Minv)
  std::vector<double> px, pn, pt;     // planes: point, unit normal, tangent (-n_y, n_x)
  or_rb2d_params p{};
  std::map<std::pair<unsigned, unsigned>, std::pair<double, double>> cache_cc, cache_pc;
  std::vector<int32_t> last_ia, last_ib;
  std::vector<double> last_n, last_ta, last_tb, last_alpha, last_beta;
  std::vector<int32_t> next_order;
};

namespace {

struct Contact {
  int32_t a, b;     // b >= 0 circle, b = -1 - plane for a static plane
  double nx, ny;    // normal (basis column 0)
  double tx, ty;    // tangent (-n_y, n_x) (basis column 1)
  double ca, cb;    // tangent-row angular entries: cross(arm_a, t), cross(arm_b, t) (0 for a plane)
};

// MathUtilities::cross (scisim/Math/MathUtilities.h:16-19)
inline double cross2(double ax, double ay, double bx, double by) { return ax * by - ay * bx; }

// SymplecticEulerMap / VerletMap of rigidbody2d with F = (m g, 0) per body (the force vector is
// zeroed, then gravity adds m g to the translational entries).
void umap_flow(const or_rb2d* s, const double* q0, const double* v0, double* q1, double* v1) {
  const double dt = s->p.dt;
  for (int i = 0; i < s->nb; ++i) {
    const double F[3] = {0.0 + s->m[i] * s->p.gravity[0], 0.0 + s->m[i] * s->p.gravity[1], 0.0};
    const double mi[3] = {s->minv[i], s->minv[i], s->Iinv[i]};
    if (s->p.integrator == OR_SYMPLECTIC_EULER) {
      // v1 = v0 + (dt Minv) F ; q1 = q0 + dt v1
      for (int d = 0; d < 3; ++d) {
        const double sc = dt * mi[d];
        v1[3 * i + d] = v0[3 * i + d] + sc * F[d];
        q1[3 * i + d] = q0[3 * i + d] + dt * v1[3 * i + d];
      }
    } else {
      // v = v0 + (0.5 dt Minv) F(q0) ; q1 = q0 + dt v ; v1 = v + (0.5 dt Minv) F(q1), F constant
      for (int d = 0; d < 3; ++d) {
        const double sc = (0.5 * dt) * mi[d];
        const double vh = v0[3 * i + d] + sc * F[d];
        q1[3 * i + d] = q0[3 * i + d] + dt * vh;
        v1[3 * i + d] = vh + sc * F[d];
      }
    }
  }
}

// RigidBody2DSim::computeActiveSet: circle pairs whose swept AABBs overlap, in (i < j) order,
// kept when the CCD test says they touch during the step, with n and p taken at q0; then every
// (plane, circle) with the circle's predictor centre within r of the plane, plane-major.
void active_set(const or_rb2d* s, const double* q0, const double* q1, std::vector<Contact>& out) {
  out.clear();
  const int nb = s->nb;
  std::vector<double> aabb(4 * static_cast<size_t>(nb));
  for (int i = 0; i < nb; ++i)
    for (int d = 0; d < 2; ++d) {
      aabb[4 * i + d] = std::min(q0[3 * i + d], q1[3 * i + d]) - s->r[i];
      aabb[4 * i + 2 + d] = std::max(q0[3 * i + d], q1[3 * i + d]) + s->r[i];
    }
  int64_t total = 0;
  std::vector<int32_t> pairs(2 * static_cast<size_t>(std::max(16, 8 * nb)));
  int64_t np = or_grid_overlaps_2d(nb, aabb.data(), int64_t(pairs.size() / 2), pairs.data(), &total);
  if (np < 0 || total > int64_t(pairs.size() / 2)) {
    pairs.resize(2 * static_cast<size_t>(total));
    np = or_grid_overlaps_2d(nb, aabb.data(), total, pairs.data(), &total);
  }
  for (int64_t k = 0; k < np; ++k) {
    const int a = pairs[2 * k], b = pairs[2 * k + 1];
    const double q0a[2] = {q0[3 * a], q0[3 * a + 1]}, q1a[2] = {q1[3 * a], q1[3 * a + 1]};
    const double q0b[2] = {q0[3 * b], q0[3 * b + 1]}, q1b[2] = {q1[3 * b], q1[3 * b + 1]};
    double c[3];
    or_ccd_coeffs_2d(q0a, q1a, s->r[a], q0b, q1b, s->r[b], c);
    if (!or_ccd_happens(c, nullptr)) continue;
    // n = (q0a - q0b).normalized(); p = q0a + (ra / (ra + rb)) (q0b - q0a)
    double nx = q0a[0] - q0b[0], ny = q0a[1] - q0b[1];
    const double z = nx * nx + ny * ny;
    if (z > 0.0) {
      const double sq = std::sqrt(z);
      nx = nx / sq;
      ny = ny / sq;
    }
    const double f = s->r[a] / (s->r[a] + s->r[b]);
    const double pxc = q0a[0] + f * (q0b[0] - q0a[0]);
    const double pyc = q0a[1] + f * (q0b[1] - q0a[1]);
    const double tx = -ny, ty = nx;
    // evalH at q0: ri = p - x_a, rj = p - x_b
    const double ca = cross2(pxc - q0a[0], pyc - q0a[1], tx, ty);
    const double cb = cross2(pxc - q0b[0], pyc - q0b[1], tx, ty);
    out.push_back(Contact{a, b, nx, ny, tx, ty, ca, cb});
  }
  for (int pl = 0; pl < s->np; ++pl) {
    const double nx = s->pn[2 * pl], ny = s->pn[2 * pl + 1];
    const double tx = s->pt[2 * pl], ty = s->pt[2 * pl + 1];
    for (int i = 0; i < nb; ++i) {
      const double d = nx * (q1[3 * i] - s->px[2 * pl]) + ny * (q1[3 * i + 1] - s->px[2 * pl + 1]);
      if (d <= s->r[i]) {
        // evalH: r_world = -r n, H0(1,2) = cross(r_world, t)
        const double ca = cross2(-s->r[i] * nx, -s->r[i] * ny, tx, ty);
        out.push_back(Contact{i, int32_t(-1 - pl), nx, ny, tx, ty, ca, 0.0});
      }
    }
  }
}

std::pair<unsigned, unsigned> cache_key(const Contact& c) {
  if (c.b >= 0) return {unsigned(c.a), unsigned(c.b)};
  return {unsigned(-1 - c.b), unsigned(c.a)};
}

// Sobogus::solve for RigidBody2D contacts (Sobogus.cpp:110-182 setup, :375-470 solve and impulse
// extraction): dual problem u = W r + b evaluated through body velocities v = v0 + Minv H^T r,
// sequential block Gauss-Seidel in active-set order (or the given order), residual every
// eval_every sweeps, best iterate at max_iters.  v0, v2: 3 per body.  alpha, beta: in = warm
// start, out = solution.
void solve_rb2d(const or_rb2d* s, const double* v0, const std::vector<Contact>& cs, const int32_t* order,
                double* alpha, double* beta, double* v2, or_gs_result* res) {
  const int nb = s->nb, nc = int(cs.size());
  const double CoR = s->p.CoR, mu = s->p.mu;
  std::vector<char> touched(nb, 0);
  for (const Contact& c : cs) {
    touched[c.a] = 1;
    if (c.b >= 0) touched[c.b] = 1;
  }
  // Per-contact forcing E^T w, diagonal Delassus block and warm start in local coordinates.
  std::vector<double> C(2 * nc), Wd(3 * nc), R(2 * nc);
  for (int k = 0; k < nc; ++k) {
    const Contact& c = cs[k];
    const int a = c.a, b = c.b;
    // evalNdotV at (q0, v0): n . (v_a - v_b) on the translational entries (a static plane moves
    // with velocity zero); nrel, drel: minus the kinematic relative velocity (zero here) on n, t.
    double vrx = v0[3 * a], vry = v0[3 * a + 1];
    if (b >= 0) {
      vrx = vrx - v0[3 * b];
      vry = vry - v0[3 * b + 1];
    } else {
      vrx = vrx - 0.0;
      vry = vry - 0.0;
    }
    const double ndotv = c.nx * vrx + c.ny * vry;
    const double nrel = -(0.0 * c.nx + 0.0 * c.ny);
    const double drel = -(0.0 * c.tx + 0.0 * c.ty);
    const double sv = CoR * ndotv + nrel;
    const double wx = (0.0 + c.nx * sv) + c.tx * drel;
    const double wy = (0.0 + c.ny * sv) + c.ty * drel;
    C[2 * k] = c.nx * wx + c.ny * wy;
    C[2 * k + 1] = c.tx * wx + c.ty * wy;
    // W = sum over the contact's bodies of H_i Minv_i H_i^T, H_i rows [n^T 0; t^T c_i].
    const double nn = c.nx * c.nx + c.ny * c.ny;
    const double nt = c.nx * c.tx + c.ny * c.ty;
    const double tt = c.tx * c.tx + c.ty * c.ty;
    double w00 = s->minv[a] * nn;
    double w01 = s->minv[a] * nt;
    double w11 = s->minv[a] * tt + s->Iinv[a] * (c.ca * c.ca);
    if (b >= 0) {
      w00 = w00 + s->minv[b] * nn;
      w01 = w01 + s->minv[b] * nt;
      w11 = w11 + (s->minv[b] * tt + s->Iinv[b] * (c.cb * c.cb));
    }
    Wd[3 * k] = w00;
    Wd[3 * k + 1] = w01;
    Wd[3 * k + 2] = w11;
    // r = alpha n + beta t (Sobogus.cpp:400-402), then r_loc = E^T r.
    const double rwx = alpha[k] * c.nx + beta[k] * c.tx;
    const double rwy = alpha[k] * c.ny + beta[k] * c.ty;
    R[2 * k] = c.nx * rwx + c.ny * rwy;
    R[2 * k + 1] = c.tx * rwx + c.ty * rwy;
  }
  // Body -> contacts in ascending contact order, for a fixed-order gather of H^T r.
  std::vector<int> cnt(nb + 1, 0);
  for (const Contact& c : cs) {
    cnt[c.a + 1]++;
    if (c.b >= 0) cnt[c.b + 1]++;
  }
  for (int i = 0; i < nb; ++i) cnt[i + 1] += cnt[i];
  std::vector<int> adj(cnt[nb]);
  {
    std::vector<int> cur(cnt.begin(), cnt.end() - 1);
    for (int k = 0; k < nc; ++k) {
      adj[cur[cs[k].a]++] = k;
      if (cs[k].b >= 0) adj[cur[cs[k].b]++] = k;
    }
  }
  auto gather = [&](int body, const std::vector<double>& Rv, double* h) {
    h[0] = h[1] = h[2] = 0.0;
    for (int e = cnt[body]; e < cnt[body + 1]; ++e) {
      const int k = adj[e];
      const Contact& c = cs[k];
      const bool is_a = c.a == body;
      const double sgn = is_a ? 1.0 : -1.0;
      const double r0 = Rv[2 * k], r1 = Rv[2 * k + 1];
      h[0] = h[0] + sgn * (c.nx * r0 + c.tx * r1);
      h[1] = h[1] + sgn * (c.ny * r0 + c.ty * r1);
      h[2] = h[2] + sgn * ((is_a ? c.ca : c.cb) * r1);
    }
  };
  std::vector<double> V(3 * static_cast<size_t>(nb));
  for (int i = 0; i < nb; ++i) {
    double h[3];
    gather(i, R, h);
    V[3 * i] = v0[3 * i] + s->minv[i] * h[0];
    V[3 * i + 1] = v0[3 * i + 1] + s->minv[i] * h[1];
    V[3 * i + 2] = v0[3 * i + 2] + s->Iinv[i] * h[2];
  }
  auto local_u = [&](int k, double* u) {
    const Contact& c = cs[k];
    const double* va = &V[3 * c.a];
    double hn = c.nx * va[0] + c.ny * va[1];
    double ht = (c.tx * va[0] + c.ty * va[1]) + c.ca * va[2];
    if (c.b >= 0) {
      const double* vb = &V[3 * c.b];
      hn = hn - (c.nx * vb[0] + c.ny * vb[1]);
      ht = ht - ((c.tx * vb[0] + c.ty * vb[1]) + c.cb * vb[2]);
    }
    u[0] = hn + C[2 * k];
    u[1] = ht + C[2 * k + 1];
  };
  auto residual = [&]() {
    double err = 0.0;
    for (int k = 0; k < nc; ++k) {
      double u[2];
      local_u(k, u);
      const double e = or_fb_error(2, &R[2 * k], u, mu);
      if (e > err || e != e) err = e;
    }
    return err;
  };
  const uint32_t eval_every = s->p.eval_every == 0 ? 1 : s->p.eval_every;
  std::vector<double> Rbest(R);
  double err_best = std::numeric_limits<double>::infinity();
  uint32_t it = 0;
  bool converged = false;
  for (it = 1; it <= s->p.max_iters; ++it) {
    for (int q = 0; q < nc; ++q) {
      const int k = order ? order[q] : q;
      const Contact& c = cs[k];
      double u[2];
      local_u(k, u);
      const double r0 = R[2 * k], r1 = R[2 * k + 1];
      const double* W = &Wd[3 * k];
      const double bt[2] = {u[0] - (W[0] * r0 + W[1] * r1), u[1] - (W[1] * r0 + W[2] * r1)};
      double rn[2];
      or_local_solve(2, W, bt, mu, rn);
      const double d0 = rn[0] - r0, d1 = rn[1] - r1;
      const double px = c.nx * d0 + c.tx * d1, py = c.ny * d0 + c.ty * d1;
      double* va = &V[3 * c.a];
      va[0] = va[0] + s->minv[c.a] * px;
      va[1] = va[1] + s->minv[c.a] * py;
      va[2] = va[2] + s->Iinv[c.a] * (c.ca * d1);
      if (c.b >= 0) {
        double* vb = &V[3 * c.b];
        vb[0] = vb[0] - s->minv[c.b] * px;
        vb[1] = vb[1] - s->minv[c.b] * py;
        vb[2] = vb[2] - s->Iinv[c.b] * (c.cb * d1);
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
      if (err < s->p.tol) {
        converged = true;
        break;
      }
    }
  }
  if (!converged) {
    if (err_best < std::numeric_limits<double>::infinity()) R = Rbest;
    it = s->p.max_iters;
  }
  if (nc == 0) err_best = 0.0;
  // v2 = Minv (H^T r - f) with f = -M v0 for the bodies in contacts; the others keep v0.
  for (int i = 0; i < nb; ++i) {
    if (!touched[i]) {
      for (int d = 0; d < 3; ++d) v2[3 * i + d] = v0[3 * i + d];
      continue;
    }
    double h[3];
    gather(i, R, h);
    v2[3 * i] = s->minv[i] * (h[0] - (-(s->m[i] * v0[3 * i])));
    v2[3 * i + 1] = s->minv[i] * (h[1] - (-(s->m[i] * v0[3 * i + 1])));
    v2[3 * i + 2] = s->Iinv[i] * (h[2] - (-(s->I[i] * v0[3 * i + 2])));
  }
  // Impulses alpha = r . n, beta = r . t (zero when mu is zero) (Sobogus.cpp:421-437).
  for (int k = 0; k < nc; ++k) {
    const Contact& c = cs[k];
    const double rwx = c.nx * R[2 * k] + c.tx * R[2 * k + 1];
    const double rwy = c.ny * R[2 * k] + c.ty * R[2 * k + 1];
    alpha[k] = rwx * c.nx + rwy * c.ny;
    beta[k] = (mu == 0.0) ? 0.0 : (rwx * c.tx + rwy * c.ty);
  }
  res->error = err_best;
  res->iterations = it;
  res->succeeded = err_best < s->p.tol ? 1 : 0;
}

}  // namespace

extern "C" or_rb2d* or_rb2d_create(int nb, const double* q, const double* v, const double* r, const double* m,
                                   const double* I, int np, const double* plane_x, const double* plane_n,
                                   const or_rb2d_params* p) {
  auto* s = new or_rb2d;
  s->nb = nb;
  s->np = np;
  s->q.assign(q, q + 3 * nb);
  s->v.assign(v, v + 3 * nb);
  s->r.assign(r, r + nb);
  s->m.assign(m, m + nb);
  s->I.assign(I, I + nb);
  s->minv.resize(nb);
  s->Iinv.resize(nb);
  for (int i = 0; i < nb; ++i) {
    s->minv[i] = 1.0 / m[i];
    s->Iinv[i] = 1.0 / I[i];
  }
  s->px.assign(plane_x, plane_x + 2 * np);
  s->pn.resize(2 * np);
  s->pt.resize(2 * np);
  for (int pl = 0; pl < np; ++pl) {
    // the scene parser stores n.normalized() (RigidBody2DSceneParser.cpp:271-277); t = (-n_y, n_x)
    double nx = plane_n[2 * pl], ny = plane_n[2 * pl + 1];
    const double z = nx * nx + ny * ny;
    if (z > 0.0) {
      const double sq = std::sqrt(z);
      nx = nx / sq;
      ny = ny / sq;
    }
    s->pn[2 * pl] = nx;
    s->pn[2 * pl + 1] = ny;
    s->pt[2 * pl] = -ny;
    s->pt[2 * pl + 1] = nx;
  }
  s->p = *p;
  return s;
}

extern "C" void or_rb2d_destroy(or_rb2d* s) { delete s; }

// GeometricImpactFrictionMap::flow (GeometricImpactFrictionMap.cpp:267-442) for RigidBody2DSim:
// unconstrained predictor, active set, impulses from the cache, the solve, impulses into the cache,
// and the final map from q0 with the post-impact velocity.
extern "C" int or_rb2d_step(or_rb2d* s, uint32_t iteration, or_step_stats* stats) {
  (void)iteration;
  const int nb = s->nb;
  // StabilizedImpactFrictionMap::flow (StabilizedImpactFrictionMap.cpp:48-167): the unconstrained
  // step first, a cold solve from its velocity v1, then q1 = q0 + dt v.
  const bool stab = s->p.staggering == OR_STAGGER_STABILIZED;
  std::vector<double> q1(3 * static_cast<size_t>(nb)), v1(3 * static_cast<size_t>(nb));
  umap_flow(s, s->q.data(), s->v.data(), q1.data(), v1.data());
  std::vector<Contact> cs;
  active_set(s, s->q.data(), q1.data(), cs);
  const int nc = int(cs.size());
  int64_t ncc = 0;
  for (const Contact& c : cs) ncc += (c.b >= 0);
  if (stats) {
    stats->n_contacts = nc;
    stats->n_ball_ball = ncc;
    stats->n_ball_plane = nc - ncc;
    stats->iterations = 0;
    stats->succeeded = 1;
    stats->error = 0.0;
  }
  s->last_ia.assign(nc, 0);
  s->last_ib.assign(nc, 0);
  s->last_n.assign(2 * static_cast<size_t>(nc), 0.0);
  s->last_ta.assign(nc, 0.0);
  s->last_tb.assign(nc, 0.0);
  s->last_alpha.assign(nc, 0.0);
  s->last_beta.assign(nc, 0.0);
  if (nc == 0) {
    // No contacts: keep the predictor and clear the cache.
    s->cache_cc.clear();
    s->cache_pc.clear();
    s->next_order.clear();
    s->q.swap(q1);
    s->v.swap(v1);
    return 0;
  }
  std::vector<double> alpha(nc, 0.0), beta(nc, 0.0);
  if (s->p.cache_mode != OR_CACHE_NONE) {
    for (int k = 0; k < nc; ++k) {
      const auto& cache = cs[k].b >= 0 ? s->cache_cc : s->cache_pc;
      const auto it = cache.find(cache_key(cs[k]));
      if (it != cache.end()) {
        alpha[k] = it->second.first;
        beta[k] = (s->p.cache_mode == OR_CACHE_NORMAL_AND_FRICTION) ? it->second.second : 0.0;
      }
    }
  }
  s->cache_cc.clear();
  s->cache_pc.clear();
  std::vector<double> v2(3 * static_cast<size_t>(nb));
  or_gs_result gr{};
  const int32_t* order = int64_t(s->next_order.size()) == int64_t(nc) ? s->next_order.data() : nullptr;
  solve_rb2d(s, stab ? v1.data() : s->v.data(), cs, order, alpha.data(), beta.data(), v2.data(), &gr);
  s->next_order.clear();
  if (s->p.cache_mode != OR_CACHE_NONE) {
    for (int k = 0; k < nc; ++k) {
      auto& cache = cs[k].b >= 0 ? s->cache_cc : s->cache_pc;
      cache[cache_key(cs[k])] = {alpha[k], s->p.cache_mode == OR_CACHE_NORMAL_AND_FRICTION ? beta[k] : 0.0};
    }
  }
  for (int k = 0; k < nc; ++k) {
    s->last_ia[k] = cs[k].a;
    s->last_ib[k] = cs[k].b;
    s->last_n[2 * k] = cs[k].nx;
    s->last_n[2 * k + 1] = cs[k].ny;
    s->last_ta[k] = cs[k].ca;
    s->last_tb[k] = cs[k].cb;
    s->last_alpha[k] = alpha[k];
    s->last_beta[k] = beta[k];
  }
  if (stats) {
    stats->iterations = gr.iterations;
    stats->succeeded = gr.succeeded;
    stats->error = gr.error;
  }
  if (stab) {
    for (int i = 0; i < 3 * nb; ++i) {
      v1[i] = v2[i];
      q1[i] = s->q[i] + s->p.dt * v1[i];
    }
  } else {
    // Final map with the post-impact velocity (GeometricImpactFrictionMap.cpp:441).
    umap_flow(s, s->q.data(), v2.data(), q1.data(), v1.data());
  }
  s->q.swap(q1);
  s->v.swap(v1);
  return gr.succeeded ? 0 : 1;
}

extern "C" int or_rb2d_run(or_rb2d* s, uint32_t first_iteration, uint32_t n_steps, or_step_stats* stats,
                           int64_t* total_contacts) {
  int bad = 0;
  int64_t tot = 0;
  or_step_stats st{};
  for (uint32_t k = 0; k < n_steps; ++k) {
    bad += or_rb2d_step(s, first_iteration + k, &st);
    tot += st.n_contacts;
  }
  if (stats) *stats = st;
  if (total_contacts) *total_contacts = tot;
  return bad;
}

extern "C" void or_rb2d_get_state(const or_rb2d* s, double* q, double* v) {
  std::copy(s->q.begin(), s->q.end(), q);
  std::copy(s->v.begin(), s->v.end(), v);
}

extern "C" void or_rb2d_set_state(or_rb2d* s, const double* q, const double* v) {
  s->q.assign(q, q + 3 * s->nb);
  s->v.assign(v, v + 3 * s->nb);
}

extern "C" void or_rb2d_set_solver(or_rb2d* s, double tol, uint32_t max_iters) {
  s->p.tol = tol;
  s->p.max_iters = max_iters;
}

extern "C" void or_rb2d_set_next_order(or_rb2d* s, int64_t nc, const int32_t* order) {
  s->next_order.assign(order, order + nc);
}

extern "C" int64_t or_rb2d_last_contacts(const or_rb2d* s, int64_t cap, int32_t* ia, int32_t* ib, double* n,
                                         double* ta, double* tb, double* alpha, double* beta) {
  const int64_t nc = int64_t(s->last_ia.size());
  if (nc > cap) return -nc - 1;
  for (int64_t k = 0; k < nc; ++k) {
    if (ia) ia[k] = s->last_ia[k];
    if (ib) ib[k] = s->last_ib[k];
    if (n) {
      n[2 * k] = s->last_n[2 * k];
      n[2 * k + 1] = s->last_n[2 * k + 1];
    }
    if (ta) ta[k] = s->last_ta[k];
    if (tb) tb[k] = s->last_tb[k];
    if (alpha) alpha[k] = s->last_alpha[k];
    if (beta) beta[k] = s->last_beta[k];
  }
  return nc;
}
