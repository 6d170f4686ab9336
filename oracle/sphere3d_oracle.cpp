// sphere3d_oracle.cpp -- CPU oracle: one RigidBody3D sphere step (TEST INFRASTRUCTURE ONLY, see oracle.h).
//
// Restates, for scenes of spheres and static planes:
//   RigidBodySphere::computeMassAndInertia       rigidbody3d/Geometry/RigidBodySphere.cpp:10-18
//   world mass matrices at construction          rigidbody3d/RigidBody3DState.cpp:140-230
//   RigidBody3DState::updateMandMinv             rigidbody3d/RigidBody3DState.cpp:428-462
//   NearEarthGravityForce::computeForce          rigidbody3d/Forces/NearEarthGravityForce.cpp:39-54
//   SplitHamMap::flow                            rigidbody3d/UnconstrainedMaps/SplitHamMap.cpp:17-182
//   active set (q1 AABBs, grid, sphere-sphere)   rigidbody3d/RigidBody3DSim.cpp:1057-1140, 793-819
//   plane-sphere active set (plane-major)        rigidbody3d/RigidBody3DSim.cpp:1414-1452
//   StaticPlane (normal normalised)              rigidbody3d/StaticGeometry/StaticPlane.cpp:10-15
//   contact bases                                rigidbody3d/Constraints/SphereSphereConstraint.cpp:273-300,
//                                                StaticPlaneSphereConstraint.cpp:255-283, FrictionUtilities.cpp:19-29
//   GeometricImpactFrictionMap::flow             scisim/ConstrainedMaps/GeometricImpactFrictionMap.cpp:267-442
//                                                (3D scenes force the impulse cache to NONE:
//                                                rigidbody3dutils/RigidBody3DSceneParser.cpp:1877-1880)
// Fixed-size Eigen products are evaluated as separately rounded sequential sums ((a0+a1)+a2), the
// order of the reference's SSE2 build; a scalar times a sparse matrix is folded into its coefficients.
#include "oracle.h"

#include <cmath>
#include <cstring>
#include <array>
#include <map>
#include <vector>

extern "C" void or_sobogus_solve_3d(int nb, const double* m, const double* Iinv, const double* Iw, const double* v0,
                                    int nc, const int32_t* ia, const int32_t* ib, const double* bases,
                                    const double* arm_a, const double* arm_b, const double* CoR, const double* mu,
                                    const or_gs_params* p, double* alpha, double* beta, double* v2, double* f,
                                    or_gs_result* res);

namespace {

inline double dot3(const double* a, const double* b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
inline void cross3(const double* a, const double* b, double* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
inline void normalize3(double* v) {
  const double z = dot3(v, v);
  if (z > 0.0) {
    const double s = std::sqrt(z);
    v[0] = v[0] / s;
    v[1] = v[1] / s;
    v[2] = v[2] / s;
  }
}
// C = A B (3x3 row-major).
inline void matmul3(const double* A, const double* B, double* C) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) C[3 * i + j] = (A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j]) + A[3 * i + 2] * B[6 + j];
}
inline void matvec3(const double* A, const double* x, double* y) {
  double t[3];
  for (int i = 0; i < 3; ++i) t[i] = (A[3 * i] * x[0] + A[3 * i + 1] * x[1]) + A[3 * i + 2] * x[2];
  y[0] = t[0];
  y[1] = t[1];
  y[2] = t[2];
}
// R diag(d) R^T (row-major), element (i,j) = sum_k (R_ik d_k) R_jk.
inline void rdrt(const double* R, const double* d, double* out) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      out[3 * i + j] = ((R[3 * i] * d[0]) * R[3 * j] + (R[3 * i + 1] * d[1]) * R[3 * j + 1]) +
                       (R[3 * i + 2] * d[2]) * R[3 * j + 2];
}
// Rotation by `angle` about the unit axis -e_axis (Rodrigues' formula).
inline void rot_neg_axis(int axis, double angle, double* R) {
  const double c = std::cos(angle), s = std::sin(angle);
  double a[3] = {0.0, 0.0, 0.0};
  a[axis] = -1.0;
  const double omc = 1.0 - c;
  R[0] = (omc * a[0]) * a[0] + c;
  R[4] = (omc * a[1]) * a[1] + c;
  R[8] = (omc * a[2]) * a[2] + c;
  R[1] = (omc * a[0]) * a[1] - s * a[2];
  R[3] = (omc * a[0]) * a[1] + s * a[2];
  R[2] = (omc * a[0]) * a[2] + s * a[1];
  R[6] = (omc * a[0]) * a[2] - s * a[1];
  R[5] = (omc * a[1]) * a[2] - s * a[0];
  R[7] = (omc * a[1]) * a[2] + s * a[0];
}

struct Contact3 {
  int32_t a, b;  // b = -1 - plane for plane contacts
  double n[3];
  double p[3];   // sphere-sphere contact point at q0
};

}  // namespace

struct or_sphere3d {
  int nb = 0;
  std::vector<double> q, v;      // q: [x (3nb) | R row-major (9nb)], v: [v (3nb) | omega (3nb)]
  std::vector<double> r, m, I0;  // radius, mass, body-frame principal inertia (3 per body)
  std::vector<double> Iw, Iinv;  // world inertia and inverse (row-major 3x3 per body)
  int np = 0;
  std::vector<double> px, pn;
  or_sphere3d_params prm{};
  std::vector<int32_t> next_order;
  // last step
  std::vector<Contact3> contacts;
  std::vector<double> bases, arm_a, arm_b, alpha, beta;
  // SymplecticEulerImpactFrictionMap's impulse cache (rigidbody3d/ConstraintCache.cpp): keys (i, j)
  // for sphere pairs, (plane, sphere) for planes; values [alpha, 0, ...] (normal) or
  // [n (3) | alpha n + beta0 s + beta1 t (3)] (normal and friction).
  std::map<std::pair<unsigned, unsigned>, std::array<double, 6>> cache_ss, cache_ps;
};

namespace {

void update_world_inertia(or_sphere3d* s, bool construction) {
  for (int b = 0; b < s->nb; ++b) {
    const double* R = &s->q[3 * s->nb + 9 * b];
    const double d[3] = {s->I0[3 * b], s->I0[3 * b + 1], s->I0[3 * b + 2]};
    const double di[3] = {1.0 / d[0], 1.0 / d[1], 1.0 / d[2]};
    double I[9], Ii[9];
    rdrt(R, d, I);
    rdrt(R, di, Ii);
    if (construction) {
      // The constructor inserts I(row, col) at sparse entry (col, row) (RigidBody3DState.cpp:175-182).
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          s->Iw[9 * b + 3 * i + j] = I[3 * j + i];
          s->Iinv[9 * b + 3 * i + j] = Ii[3 * j + i];
        }
    } else {
      std::memcpy(&s->Iw[9 * b], I, sizeof I);
      std::memcpy(&s->Iinv[9 * b], Ii, sizeof Ii);
    }
  }
}

// SplitHamMap::flow with the state's current world inertia (the sparse M of the reference).
void splitham(const or_sphere3d* s, const double* q0, const double* v0, double* q1, double* v1) {
  const int nb = s->nb;
  const double dt = s->prm.dt;
  const double h = 0.5 * dt;
  const double hdt = (0.5 * dt) * dt;
  std::memcpy(q1, q0, sizeof(double) * 12 * nb);
  for (int b = 0; b < nb; ++b) {
    const double m = s->m[b];
    const double minv = 1.0 / m;
    double p[3], L[3];
    for (int j = 0; j < 3; ++j) {
      const double F = m * s->prm.gravity[j];
      p[j] = m * v0[3 * b + j];
      p[j] = p[j] + h * F;
      q1[3 * b + j] = q0[3 * b + j] + (dt * v0[3 * b + j] + (hdt * minv) * F);
    }
    // Angular momentum M_w omega; torque-free half kick adds (0.5 dt) * 0.
    matvec3(&s->Iw[9 * b], &v0[3 * nb + 3 * b], L);
    for (int j = 0; j < 3; ++j) L[j] = L[j] + h * 0.0;
    const double* I = &s->I0[3 * b];
    const double* R0 = &q0[3 * nb + 9 * b];
    double* R1 = &q1[3 * nb + 9 * b];
    double pB[3];
    for (int i = 0; i < 3; ++i) pB[i] = (R0[i] * L[0] + R0[3 + i] * L[1]) + R0[6 + i] * L[2];
    double Rc[9], Rf[9], Ri[9], tmp[9];
    std::memcpy(Rc, R0, sizeof Rc);
    const int axes[5] = {2, 1, 0, 1, 2};
    for (int st = 0; st < 5; ++st) {
      const int ax = axes[st];
      const double ang = st == 2 ? (dt * pB[ax]) / I[ax] : (h * pB[ax]) / I[ax];
      rot_neg_axis(ax, -ang, Ri);
      matmul3(Rc, Ri, tmp);
      std::memcpy(Rc, tmp, sizeof Rc);
      rot_neg_axis(ax, ang, Rf);
      matvec3(Rf, pB, pB);
    }
    std::memcpy(R1, Rc, sizeof Rc);
    for (int j = 0; j < 3; ++j) {
      const double F = m * s->prm.gravity[j];
      p[j] = p[j] + h * F;
      L[j] = L[j] + h * 0.0;
      v1[3 * b + j] = p[j] / m;
    }
    const double di[3] = {1.0 / I[0], 1.0 / I[1], 1.0 / I[2]};
    double W[9];
    rdrt(R1, di, W);
    matvec3(W, L, &v1[3 * nb + 3 * b]);
  }
}

void orthogonal_vector(const double* n, double* o) {
  const double ax = std::fabs(n[0]), ay = std::fabs(n[1]), az = std::fabs(n[2]);
  o[0] = o[1] = o[2] = 0.0;
  if (ax <= ay && ax <= az)
    o[0] = 1.0;
  else if (ay <= az)
    o[1] = 1.0;
  else
    o[2] = 1.0;
  const double d = dot3(n, o);
  for (int j = 0; j < 3; ++j) o[j] = o[j] - d * n[j];
  normalize3(o);
}

// Tangent basis from the relative contact velocity s (SphereSphereConstraint.cpp:273-300).
void basis_from_relvel(const double* n, const double* sv, double* E) {
  double s[3] = {sv[0], sv[1], sv[2]};
  double c[3];
  cross3(n, s, c);
  if (dot3(c, c) < 1.0e-9) {
    orthogonal_vector(n, s);
  } else {
    const double d = dot3(s, n);
    for (int j = 0; j < 3; ++j) s[j] = s[j] - d * n[j];
    normalize3(s);
  }
  for (int j = 0; j < 3; ++j) s[j] = s[j] * -1.0;
  double t[3];
  cross3(n, s, t);
  normalize3(t);
  for (int j = 0; j < 3; ++j) {
    E[j] = n[j];
    E[3 + j] = s[j];
    E[6 + j] = t[j];
  }
}

void active_set(const or_sphere3d* s, const double* q0, const double* q1, std::vector<Contact3>& out,
                int64_t* n_ss) {
  const int nb = s->nb;
  out.clear();
  std::vector<double> aabb(6 * static_cast<size_t>(nb));
  for (int b = 0; b < nb; ++b)
    for (int j = 0; j < 3; ++j) {
      aabb[6 * b + j] = q1[3 * b + j] - s->r[b];
      aabb[6 * b + 3 + j] = q1[3 * b + j] + s->r[b];
    }
  int64_t total = 0;
  std::vector<int32_t> pairs(2 * 1024);
  int64_t got = or_grid_overlaps_3d(nb, aabb.data(), 1024, pairs.data(), &total);
  if (got < 0) {
    pairs.resize(2 * static_cast<size_t>(total));
    got = or_grid_overlaps_3d(nb, aabb.data(), total, pairs.data(), &total);
  }
  for (int64_t k = 0; k < got; ++k) {
    const int i = pairs[2 * k], j = pairs[2 * k + 1];
    double d[3];
    for (int c = 0; c < 3; ++c) d[c] = q1[3 * i + c] - q1[3 * j + c];
    const double rs = s->r[i] + s->r[j];
    if (!(dot3(d, d) <= rs * rs)) continue;
    Contact3 ct;
    ct.a = i;
    ct.b = j;
    for (int c = 0; c < 3; ++c) ct.n[c] = q0[3 * i + c] - q0[3 * j + c];
    normalize3(ct.n);
    const double frac = s->r[i] / (s->r[i] + s->r[j]);
    for (int c = 0; c < 3; ++c) ct.p[c] = q0[3 * i + c] + frac * (q0[3 * j + c] - q0[3 * i + c]);
    out.push_back(ct);
  }
  *n_ss = static_cast<int64_t>(out.size());
  for (int pl = 0; pl < s->np; ++pl) {
    const double* x = &s->px[3 * pl];
    const double* n = &s->pn[3 * pl];
    for (int b = 0; b < nb; ++b) {
      const double d[3] = {q1[3 * b] - x[0], q1[3 * b + 1] - x[1], q1[3 * b + 2] - x[2]};
      if (!(dot3(n, d) <= s->r[b])) continue;
      Contact3 ct;
      ct.a = b;
      ct.b = -1 - pl;
      for (int c = 0; c < 3; ++c) {
        ct.n[c] = n[c];
        ct.p[c] = 0.0;
      }
      out.push_back(ct);
    }
  }
}

}  // namespace

extern "C" void or_sphere_mass_inertia(double r, double density, double* M, double* I) {
  double m = 4.0 * M_PI * r * r * r / 3.0;
  double i = 2.0 * m * r * r / 5.0;
  m *= density;
  i *= density;
  *M = m;
  *I = i;
}

extern "C" or_sphere3d* or_sphere3d_create(int nb, const double* q, const double* v, const double* r,
                                           const double* m, const double* I0, int np, const double* plane_x,
                                           const double* plane_n, const or_sphere3d_params* p) {
  auto* s = new or_sphere3d;
  s->nb = nb;
  s->q.assign(q, q + 12 * static_cast<size_t>(nb));
  s->v.assign(v, v + 6 * static_cast<size_t>(nb));
  s->r.assign(r, r + nb);
  s->m.assign(m, m + nb);
  s->I0.assign(I0, I0 + 3 * static_cast<size_t>(nb));
  s->Iw.resize(9 * static_cast<size_t>(nb));
  s->Iinv.resize(9 * static_cast<size_t>(nb));
  s->np = np;
  s->px.assign(plane_x, plane_x + 3 * np);
  s->pn.assign(plane_n, plane_n + 3 * np);
  for (int pl = 0; pl < np; ++pl) normalize3(&s->pn[3 * pl]);  // StaticPlane.cpp:10-15
  s->prm = *p;
  update_world_inertia(s, true);
  return s;
}

extern "C" void or_sphere3d_destroy(or_sphere3d* s) { delete s; }

extern "C" void or_sphere3d_get_state(const or_sphere3d* s, double* q, double* v) {
  std::memcpy(q, s->q.data(), sizeof(double) * s->q.size());
  std::memcpy(v, s->v.data(), sizeof(double) * s->v.size());
}

extern "C" void or_sphere3d_set_state(or_sphere3d* s, const double* q, const double* v) {
  std::memcpy(s->q.data(), q, sizeof(double) * s->q.size());
  std::memcpy(s->v.data(), v, sizeof(double) * s->v.size());
  update_world_inertia(s, false);
}

extern "C" void or_sphere3d_world_inertia(const or_sphere3d* s, double* Iw, double* Iinv) {
  std::memcpy(Iw, s->Iw.data(), sizeof(double) * s->Iw.size());
  std::memcpy(Iinv, s->Iinv.data(), sizeof(double) * s->Iinv.size());
}

extern "C" void or_sphere3d_umap(const or_sphere3d* s, const double* q0, const double* v0, double* q1, double* v1) {
  splitham(s, q0, v0, q1, v1);
}

extern "C" void or_sphere3d_set_solver(or_sphere3d* s, double tol, uint32_t max_iters) {
  s->prm.tol = tol;
  s->prm.max_iters = max_iters;
}

extern "C" void or_sphere3d_set_next_order(or_sphere3d* s, int64_t nc, const int32_t* order) {
  s->next_order.assign(order, order + nc);
}

extern "C" int64_t or_sphere3d_active_set(const or_sphere3d* s, const double* q0, const double* q1, int64_t cap,
                                          int32_t* ia, int32_t* ib) {
  std::vector<Contact3> cs;
  int64_t nss = 0;
  active_set(s, q0, q1, cs, &nss);
  const int64_t n = static_cast<int64_t>(cs.size());
  for (int64_t k = 0; k < n && k < cap; ++k) {
    ia[k] = cs[k].a;
    ib[k] = cs[k].b;
  }
  return n;
}

extern "C" int64_t or_sphere3d_last_contacts(const or_sphere3d* s, int64_t cap, int32_t* ia, int32_t* ib,
                                             double* bases, double* arm_a, double* arm_b, double* alpha,
                                             double* beta) {
  const int64_t n = static_cast<int64_t>(s->contacts.size());
  for (int64_t k = 0; k < n && k < cap; ++k) {
    if (ia) ia[k] = s->contacts[k].a;
    if (ib) ib[k] = s->contacts[k].b;
    for (int j = 0; j < 9 && bases; ++j) bases[9 * k + j] = s->bases[9 * k + j];
    for (int j = 0; j < 3; ++j) {
      if (arm_a) arm_a[3 * k + j] = s->arm_a[3 * k + j];
      if (arm_b) arm_b[3 * k + j] = s->arm_b[3 * k + j];
    }
    if (alpha) alpha[k] = s->alpha[k];
    if (beta) {
      beta[2 * k] = s->beta[2 * k];
      beta[2 * k + 1] = s->beta[2 * k + 1];
    }
  }
  return n;
}

// Per contact of s->contacts: body indices, arms from the centres to the contact point at q0
// (-r n for a plane) and the velocity-dependent basis [n s t] from the relative velocity at v0
// (SphereSphereConstraint.cpp:273-300, StaticPlaneSphereConstraint.cpp:255-283).
// IntegrationTools::exponentialEuler (rigidbody3d/UnconstrainedMaps/IntegrationTools.cpp:3-47):
// x1 = x0 + dt v; R1 = rot(omega / |omega|, |omega| dt) R0, the rotation by the Rodrigues formula
// (Eigen's AngleAxis::toRotationMatrix).
static void exponential_euler(const or_sphere3d* s, const double* q0, const double* v, double* q1) {
  const int nb = s->nb;
  const double dt = s->prm.dt;
  for (int i = 0; i < nb; ++i)
    for (int j = 0; j < 3; ++j) q1[3 * i + j] = q0[3 * i + j] + dt * v[3 * i + j];
  for (int i = 0; i < nb; ++i) {
    double ax[3] = {v[3 * nb + 3 * i], v[3 * nb + 3 * i + 1], v[3 * nb + 3 * i + 2]};
    double theta = std::sqrt(dot3(ax, ax));
    if (theta != 0.0)
      for (int j = 0; j < 3; ++j) ax[j] = ax[j] / theta;
    theta = theta * dt;
    const double sn = std::sin(theta), c = std::cos(theta);
    const double sa[3] = {sn * ax[0], sn * ax[1], sn * ax[2]};
    const double c1[3] = {(1.0 - c) * ax[0], (1.0 - c) * ax[1], (1.0 - c) * ax[2]};
    double R[9];
    double t = c1[0] * ax[1];
    R[1] = t - sa[2];
    R[3] = t + sa[2];
    t = c1[0] * ax[2];
    R[2] = t + sa[1];
    R[6] = t - sa[1];
    t = c1[1] * ax[2];
    R[5] = t - sa[0];
    R[7] = t + sa[0];
    R[0] = c1[0] * ax[0] + c;
    R[4] = c1[1] * ax[1] + c;
    R[8] = c1[2] * ax[2] + c;
    matmul3(R, &q0[3 * nb + 9 * i], &q1[3 * nb + 9 * i]);
  }
}

// Quaternion (w, x, y, z) rotating direction a onto direction b (Eigen's
// Quaternion::setFromTwoVectors: half-angle form; nearly opposite directions turn by pi about an
// axis orthogonal to a).
static void quat_from_two_vectors(const double* a, const double* b, double* q) {
  double v0[3] = {a[0], a[1], a[2]}, v1[3] = {b[0], b[1], b[2]};
  normalize3(v0);
  normalize3(v1);
  const double c = dot3(v1, v0);
  if (c < -1.0 + 1e-12) {
    double axis[3];
    orthogonal_vector(v0, axis);
    normalize3(axis);
    const double w2 = (1.0 + std::max(c, -1.0)) * 0.5;
    const double sv = std::sqrt(1.0 - w2);
    q[0] = std::sqrt(w2);
    for (int j = 0; j < 3; ++j) q[1 + j] = axis[j] * sv;
    return;
  }
  double axis[3];
  cross3(v0, v1, axis);
  const double s2 = std::sqrt((1.0 + c) * 2.0);
  const double invs = 1.0 / s2;
  for (int j = 0; j < 3; ++j) q[1 + j] = axis[j] * invs;
  q[0] = s2 * 0.5;
}

// q v q* for a unit quaternion: uv = 2 (q_v x v); v + w uv + q_v x uv.
static void quat_rotate(const double* q, const double* v, double* out) {
  double uv[3], uuv[3];
  cross3(&q[1], v, uv);
  for (int j = 0; j < 3; ++j) uv[j] = uv[j] + uv[j];
  cross3(&q[1], uv, uuv);
  for (int j = 0; j < 3; ++j) out[j] = (v[j] + q[0] * uv[j]) + uuv[j];
}

static std::pair<unsigned, unsigned> cache_key3(const Contact3& c) {
  if (c.b >= 0) return {unsigned(c.a), unsigned(c.b)};
  return {unsigned(-1 - c.b), unsigned(c.a)};
}

static void contact_frames(or_sphere3d* s, const double* q0, const double* v0, std::vector<int32_t>& ia,
                           std::vector<int32_t>& ib) {
  const int nb = s->nb;
  const int nc = static_cast<int>(s->contacts.size());
  for (int k = 0; k < nc; ++k) {
    const Contact3& ct = s->contacts[k];
    const int a = ct.a;
    ia[k] = a;
    double* ra = &s->arm_a[3 * k];
    double* rb = &s->arm_b[3 * k];
    double sv[3];
    if (ct.b >= 0) {
      const int b = ct.b;
      ib[k] = b;
      for (int j = 0; j < 3; ++j) {
        ra[j] = ct.p[j] - q0[3 * a + j];
        rb[j] = ct.p[j] - q0[3 * b + j];
      }
      double ca[3], cb[3];
      cross3(&v0[3 * nb + 3 * a], ra, ca);
      cross3(&v0[3 * nb + 3 * b], rb, cb);
      for (int j = 0; j < 3; ++j) sv[j] = ((v0[3 * a + j] + ca[j]) - v0[3 * b + j]) - cb[j];
    } else {
      ib[k] = -1;
      for (int j = 0; j < 3; ++j) ra[j] = (-s->r[a]) * ct.n[j];
      double ca[3];
      cross3(&v0[3 * nb + 3 * a], ra, ca);
      for (int j = 0; j < 3; ++j) sv[j] = (v0[3 * a + j] + ca[j]) - 0.0;
    }
    basis_from_relvel(ct.n, sv, &s->bases[9 * k]);
  }
}

// SymplecticEulerImpactFrictionMap::flow for spheres (SymplecticEulerImpactFrictionMap.cpp:201-407):
// vdelta = dt (Minv F); predictor by exponential Euler from v0 + vdelta; the active set; impulses
// from the cache, cached forces turned from the cached normal to the new one (:48-131); the solve
// from v0 with nrel = N^T vdelta (+ min(0, gap) / dt when stabilising) and drel = D^T vdelta;
// v1 = v2 + vdelta, impulses into the cache (:133-199), configuration by exponential Euler from v1.
static int se_step(or_sphere3d* s, or_step_stats* stats) {
  const int nb = s->nb;
  const double dt = s->prm.dt;
  const double* q0 = s->q.data();
  const double* v0 = s->v.data();
  const size_t nv = 6 * static_cast<size_t>(nb);
  std::vector<double> vdelta(nv), vp(nv), q1(12 * static_cast<size_t>(nb)), v1(nv);
  for (int i = 0; i < nb; ++i) {
    const double minv = 1.0 / s->m[i];
    const double* Ii = &s->Iinv[9 * static_cast<size_t>(i)];
    for (int j = 0; j < 3; ++j) {
      const double F = 0.0 + s->m[i] * s->prm.gravity[j];  // NearEarthGravityForce: no torque
      vdelta[3 * i + j] = dt * (0.0 + minv * F);
      vdelta[3 * nb + 3 * i + j] = dt * (((0.0 + Ii[3 * j] * 0.0) + Ii[3 * j + 1] * 0.0) + Ii[3 * j + 2] * 0.0);
    }
  }
  for (size_t k = 0; k < nv; ++k) vp[k] = v0[k] + vdelta[k];
  exponential_euler(s, q0, vp.data(), q1.data());
  int64_t nss = 0;
  active_set(s, q0, q1.data(), s->contacts, &nss);
  const int nc = static_cast<int>(s->contacts.size());
  or_step_stats st{};
  st.n_contacts = nc;
  st.n_ball_ball = nss;
  st.n_ball_plane = nc - nss;
  st.succeeded = 1;
  s->bases.assign(9 * static_cast<size_t>(nc), 0.0);
  s->arm_a.assign(3 * static_cast<size_t>(nc), 0.0);
  s->arm_b.assign(3 * static_cast<size_t>(nc), 0.0);
  s->alpha.assign(nc, 0.0);
  s->beta.assign(2 * static_cast<size_t>(nc), 0.0);
  if (nc == 0) {
    for (size_t k = 0; k < nv; ++k) v1[k] = v0[k] + vdelta[k];
    exponential_euler(s, q0, v1.data(), q1.data());
    s->cache_ss.clear();
    s->cache_ps.clear();
  } else {
    std::vector<int32_t> ia(nc), ib(nc);
    contact_frames(s, q0, v0, ia, ib);
    // initializeImpulses (:48-131)
    const int cm = s->prm.cache_mode;
    for (int k = 0; k < nc && cm != OR_CACHE_NONE; ++k) {
      const Contact3& ct = s->contacts[k];
      const auto& cache = ct.b >= 0 ? s->cache_ss : s->cache_ps;
      const auto it = cache.find(cache_key3(ct));
      if (it == cache.end()) continue;  // a missing entry reads as zeros
      const std::array<double, 6>& c = it->second;
      if (cm == OR_CACHE_NORMAL) {
        s->alpha[k] = c[0];
        continue;
      }
      bool zero = true;
      for (double x : c) zero = zero && x == 0.0;
      if (zero) continue;
      const double* E = &s->bases[9 * static_cast<size_t>(k)];
      double qr[4], f[3];
      quat_from_two_vectors(&c[0], E, qr);
      quat_rotate(qr, &c[3], f);
      s->alpha[k] = dot3(f, E);
      s->beta[2 * k] = dot3(f, E + 3);
      s->beta[2 * k + 1] = dot3(f, E + 6);
    }
    s->cache_ss.clear();
    s->cache_ps.clear();
    // nrel = N^T vdelta, drel = D^T vdelta: each column's entries in row order (linear rows of a,
    // of b, then angular rows of a, of b), accumulated from zero; the normal has no angular rows,
    // a tangent's angular rows are arm x tangent.
    std::vector<double> nrel(nc), drel(2 * static_cast<size_t>(nc));
    for (int k = 0; k < nc; ++k) {
      const Contact3& ct = s->contacts[k];
      const double* E = &s->bases[9 * static_cast<size_t>(k)];
      const int a = ct.a, b = ct.b;
      const double* la = &vdelta[3 * a];
      const double* wa = &vdelta[3 * nb + 3 * a];
      double tn = 0.0;
      for (int j = 0; j < 3; ++j) tn = tn + E[j] * la[j];
      if (b >= 0)
        for (int j = 0; j < 3; ++j) tn = tn + (-E[j]) * vdelta[3 * b + j];
      nrel[k] = 0.0 + 1.0 * tn;
      for (int d = 0; d < 2; ++d) {
        const double* T = E + 3 * (d + 1);
        double xa[3];
        cross3(&s->arm_a[3 * k], T, xa);
        double tt = 0.0;
        for (int j = 0; j < 3; ++j) tt = tt + T[j] * la[j];
        if (b >= 0)
          for (int j = 0; j < 3; ++j) tt = tt + (-T[j]) * vdelta[3 * b + j];
        for (int j = 0; j < 3; ++j) tt = tt + xa[j] * wa[j];
        if (b >= 0) {
          double xb[3];
          cross3(&s->arm_b[3 * k], T, xb);
          for (int j = 0; j < 3; ++j) tt = tt + (-xb[j]) * vdelta[3 * nb + 3 * b + j];
        }
        drel[2 * k + d] = 0.0 + 1.0 * tt;
      }
      if (s->prm.stabilize) {
        double gap;
        if (b >= 0) {
          // SphereSphereConstraint::evaluateGapFunction (SphereSphereConstraint.cpp:28-31)
          const double d[3] = {q0[3 * a] - q0[3 * b], q0[3 * a + 1] - q0[3 * b + 1], q0[3 * a + 2] - q0[3 * b + 2]};
          gap = (std::sqrt(dot3(d, d)) - s->r[a]) - s->r[b];
        } else {
          // StaticPlaneSphereConstraint::evaluateGapFunction (StaticPlaneSphereConstraint.cpp:31-35)
          const int pl = -1 - b;
          const double d[3] = {q0[3 * a] - s->px[3 * pl], q0[3 * a + 1] - s->px[3 * pl + 1],
                               q0[3 * a + 2] - s->px[3 * pl + 2]};
          gap = dot3(&s->pn[3 * pl], d) - s->r[a];
        }
        double g0 = std::min(0.0, gap);
        if (std::fabs(g0) < s->prm.penetration_threshold) g0 = 0.0;
        nrel[k] = nrel[k] + g0 / dt;
      }
    }
    std::vector<double> CoR(nc, s->prm.CoR), mu(nc, s->prm.mu), v2(nv), f(nv);
    or_gs_params gp{s->prm.tol, s->prm.max_iters, s->prm.eval_every, nullptr};
    if (static_cast<int64_t>(s->next_order.size()) == nc) gp.order = s->next_order.data();
    or_gs_result res{};
    or_sobogus_solve_3d_ex(nb, s->m.data(), s->Iinv.data(), s->Iw.data(), v0, nc, ia.data(), ib.data(),
                           s->bases.data(), s->arm_a.data(), s->arm_b.data(), CoR.data(), mu.data(), nrel.data(),
                           drel.data(), &gp, s->alpha.data(), s->beta.data(), v2.data(), f.data(), &res);
    st.iterations = res.iterations;
    st.succeeded = res.succeeded;
    st.error = res.error;
    for (size_t k = 0; k < nv; ++k) v1[k] = v2[k] + vdelta[k];
    // cacheImpulses (:133-199)
    for (int k = 0; k < nc && cm != OR_CACHE_NONE; ++k) {
      const Contact3& ct = s->contacts[k];
      auto& cache = ct.b >= 0 ? s->cache_ss : s->cache_ps;
      std::array<double, 6> c{};
      if (cm == OR_CACHE_NORMAL) {
        c[0] = s->alpha[k];
      } else {
        const double* E = &s->bases[9 * static_cast<size_t>(k)];
        for (int j = 0; j < 3; ++j) {
          c[j] = E[j];
          c[3 + j] = (s->alpha[k] * E[j] + s->beta[2 * k] * E[3 + j]) + s->beta[2 * k + 1] * E[6 + j];
        }
      }
      cache[cache_key3(ct)] = c;
    }
    exponential_euler(s, q0, v1.data(), q1.data());
  }
  s->next_order.clear();
  s->q.swap(q1);
  s->v.swap(v1);
  update_world_inertia(s, false);
  if (stats) *stats = st;
  return st.succeeded ? 0 : 1;
}

extern "C" int or_sphere3d_step(or_sphere3d* s, uint32_t iteration, or_step_stats* stats) {
  (void)iteration;
  if (s->prm.staggering == OR_STAGGER_SYMPLECTIC_EULER) return se_step(s, stats);
  const int nb = s->nb;
  std::vector<double> q1(12 * static_cast<size_t>(nb)), v1(6 * static_cast<size_t>(nb));
  splitham(s, s->q.data(), s->v.data(), q1.data(), v1.data());
  int64_t nss = 0;
  active_set(s, s->q.data(), q1.data(), s->contacts, &nss);
  const int nc = static_cast<int>(s->contacts.size());
  or_step_stats st{};
  st.n_contacts = nc;
  st.n_ball_ball = nss;
  st.n_ball_plane = nc - nss;
  st.succeeded = 1;
  s->bases.assign(9 * static_cast<size_t>(nc), 0.0);
  s->arm_a.assign(3 * static_cast<size_t>(nc), 0.0);
  s->arm_b.assign(3 * static_cast<size_t>(nc), 0.0);
  s->alpha.assign(nc, 0.0);
  s->beta.assign(2 * static_cast<size_t>(nc), 0.0);
  if (nc > 0) {
    const double* q0 = s->q.data();
    const double* v0 = s->v.data();
    std::vector<int32_t> ia(nc), ib(nc);
    contact_frames(s, q0, v0, ia, ib);
    std::vector<double> CoR(nc, s->prm.CoR), mu(nc, s->prm.mu);
    or_gs_params gp{s->prm.tol, s->prm.max_iters, s->prm.eval_every, nullptr};
    if (static_cast<int64_t>(s->next_order.size()) == nc) gp.order = s->next_order.data();
    std::vector<double> v2(6 * static_cast<size_t>(nb)), f(6 * static_cast<size_t>(nb));
    or_gs_result res{};
    or_sobogus_solve_3d(nb, s->m.data(), s->Iinv.data(), s->Iw.data(), v0, nc, ia.data(), ib.data(),
                        s->bases.data(), s->arm_a.data(), s->arm_b.data(), CoR.data(), mu.data(), &gp,
                        s->alpha.data(), s->beta.data(), v2.data(), f.data(), &res);
    st.iterations = res.iterations;
    st.succeeded = res.succeeded;
    st.error = res.error;
    splitham(s, q0, v2.data(), q1.data(), v1.data());
  }
  s->next_order.clear();
  s->q.swap(q1);
  s->v.swap(v1);
  update_world_inertia(s, false);
  if (stats) *stats = st;
  return st.succeeded ? 0 : 1;
}

extern "C" int or_sphere3d_run(or_sphere3d* s, uint32_t first_iteration, uint32_t n_steps, or_step_stats* stats,
                               int64_t* total_contacts) {
  int failures = 0;
  int64_t tot = 0;
  or_step_stats st{};
  for (uint32_t k = 0; k < n_steps; ++k) {
    failures += or_sphere3d_step(s, first_iteration + k, &st);
    tot += st.n_contacts;
  }
  if (stats) *stats = st;
  if (total_contacts) *total_contacts = tot;
  return failures;
}
