// ball2d_oracle.cpp -- CPU oracle: Ball2D system and its geometric impact-friction step.
//
// TEST INFRASTRUCTURE ONLY (see oracle.h).  Restates, with the same FP64
// operation order:
//   SpatialGridDetector (2D)          ball2d/SpatialGridDetector.cpp:8-147
//   SpatialGridDetector (3D)          rigidbody3d/SpatialGridDetector.cpp:8-151
//   swept AABBs + CCD active set      ball2d/Ball2DSim.cpp:553-608
//   ball-plane active set             ball2d/Ball2DSim.cpp:747-762
//   CCD quadratic + root test         scisim/CollisionDetection/CollisionDetectionUtilities.cpp:3-126
//   BallBallConstraint                ball2d/Constraints/BallBallConstraint.cpp:26-37, 244-252
//   StaticPlaneConstraint / StaticPlane ball2d/Constraints/BallStaticPlaneConstraint.cpp:10-14,
//                                     ball2d/StaticGeometry/StaticPlane.cpp:10-19
//   SymplecticEulerMap / VerletMap    ball2d/SymplecticEulerMap.cpp:21-32, ball2d/VerletMap.cpp:15-41
//   gravity                           ball2d/Forces/Ball2DGravityForce.cpp:36-46
//   ConstraintCache                   ball2d/ConstraintCache.cpp:20-120
//   GeometricImpactFrictionMap::flow  scisim/ConstrainedMaps/GeometricImpactFrictionMap.cpp:174-442
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <set>
#include <utility>
#include <vector>

namespace {

using PairSet = std::set<std::pair<unsigned, unsigned>>;

int64_t emit_pairs(const PairSet& s, int64_t cap, int32_t* pairs, int64_t* total) {
  *total = int64_t(s.size());
  if (int64_t(s.size()) > cap) return -1;
  int64_t k = 0;
  for (const auto& pr : s) {
    pairs[2 * k] = int32_t(pr.first);
    pairs[2 * k + 1] = int32_t(pr.second);
    ++k;
  }
  return k;
}

// ---- uniform grid broad phase, dimension-generic restatement ----------------
template <int D>
struct Box {
  double mn[D], mx[D];
};

template <int D>
bool overlaps(const Box<D>& a, const Box<D>& b) {
  for (int i = 0; i < D; ++i)
    if (a.mx[i] < b.mn[i]) return false;
  for (int i = 0; i < D; ++i)
    if (b.mx[i] < a.mn[i]) return false;
  return true;
}

template <int D>
void grid_overlaps(const std::vector<Box<D>>& boxes, PairSet& out) {
  if (boxes.empty()) return;
  // initializeSpatialGrid (ball2d/SpatialGridDetector.cpp:77-104)
  double mn[D], mx[D];
  for (int i = 0; i < D; ++i) {
    mn[i] = INFINITY;
    mx[i] = -INFINITY;
  }
  for (const auto& b : boxes)
    for (int i = 0; i < D; ++i) {
      mn[i] = std::min(mn[i], b.mn[i]);
      mx[i] = std::max(mx[i], b.mx[i]);
    }
  for (int i = 0; i < D; ++i) {
    mn[i] -= 2.0e-6;
    mx[i] += 2.0e-6;
  }
  double delta[D];
  for (int i = 0; i < D; ++i) delta[i] = 0.0;
  for (const auto& b : boxes)
    for (int i = 0; i < D; ++i) delta[i] += b.mx[i] - b.mn[i];
  double dmax = delta[0];
  for (int i = 1; i < D; ++i) dmax = std::max(dmax, delta[i]);
  const double h = dmax / double(boxes.size());
  unsigned dims[D];
  for (int i = 0; i < D; ++i) dims[i] = unsigned(std::ceil((mx[i] - mn[i]) / h));
  // rasterizeAABBs (:43-73): each box, inflated by 1e-6, into every cell it touches.
  std::map<unsigned, std::vector<unsigned>> voxels;
  for (unsigned bi = 0; bi < boxes.size(); ++bi) {
    unsigned lo[D], hi[D];
    for (int i = 0; i < D; ++i) {
      lo[i] = unsigned(((boxes[bi].mn[i] - 1.0e-6) - mn[i]) / h);
      hi[i] = unsigned(((boxes[bi].mx[i] + 1.0e-6) - mn[i]) / h);
    }
    if (D == 2) {
      for (unsigned x = lo[0]; x <= hi[0]; ++x)
        for (unsigned y = lo[1]; y <= hi[1]; ++y) voxels[x + dims[0] * y].push_back(bi);
    } else {
      for (unsigned x = lo[0]; x <= hi[0]; ++x)
        for (unsigned y = lo[1]; y <= hi[1]; ++y)
          for (unsigned z = lo[D - 1]; z <= hi[D - 1]; ++z)
            voxels[x + dims[0] * y + dims[0] * dims[1] * z].push_back(bi);  // unsigned key (may wrap)
    }
  }
  // getPotentialOverlaps (:106-133): all pairs within a voxel, kept if they overlap.
  for (const auto& kv : voxels) {
    const auto& v = kv.second;
    for (size_t a = 0; a + 1 < v.size(); ++a)
      for (size_t b = a + 1; b < v.size(); ++b)
        if (overlaps<D>(boxes[v[a]], boxes[v[b]])) out.insert(std::make_pair(v[a], v[b]));
  }
}

template <int D>
void allpairs_overlaps(const std::vector<Box<D>>& boxes, PairSet& out) {
  for (unsigned a = 0; a < boxes.size(); ++a)
    for (unsigned b = a + 1; b < boxes.size(); ++b)
      if (overlaps<D>(boxes[a], boxes[b])) out.insert(std::make_pair(a, b));
}

template <int D>
std::vector<Box<D>> load_boxes(int n, const double* aabb) {
  std::vector<Box<D>> boxes(n);
  for (int k = 0; k < n; ++k)
    for (int i = 0; i < D; ++i) {
      boxes[k].mn[i] = aabb[2 * D * k + i];
      boxes[k].mx[i] = aabb[2 * D * k + D + i];
    }
  return boxes;
}

// ---- CCD ----------------------------------------------------------------------
void ccd_coeffs(const double* q0a, const double* q1a, double ra, const double* q0b, const double* q1b,
                double rb, double* c) {
  const double d0x = q0a[0] - q0b[0], d0y = q0a[1] - q0b[1];
  // q1a - q1b - q0delta, evaluated left to right
  const double ex = (q1a[0] - q1b[0]) - d0x, ey = (q1a[1] - q1b[1]) - d0y;
  const double rs = ra + rb;
  c[0] = (d0x * d0x + d0y * d0y) - rs * rs;
  c[1] = 2.0 * (d0x * ex + d0y * ey);
  c[2] = ex * ex + ey * ey;
}

bool ccd_happens(const double* c, double* t) {
  if (c[2] != 0.0) {
    const double c1c1 = c[1] * c[1];
    const double fc2c0 = 4.0 * c[2] * c[0];
    if (c1c1 < fc2c0) return false;
    const double ds = std::sqrt(c1c1 - fc2c0);
    // second (larger) root, numerically stable form
    const double root1 = (c[1] > 0.0) ? (2.0 * c[0]) / (-c[1] - ds) : (-c[1] + ds) / (2.0 * c[2]);
    if (root1 < 0.0) return false;
    const double root0 = (c[1] >= 0.0) ? (-c[1] - ds) / (2.0 * c[2]) : (2.0 * c[0]) / (-c[1] + ds);
    if (root0 > 1.0) return false;
    if (t) *t = std::max(0.0, root0);
    return true;
  }
  if (c[0] <= 0.0) {
    if (t) *t = 0.0;
    return true;
  }
  return false;
}

}  // namespace

// ============================================================================
extern "C" int64_t or_grid_overlaps_2d(int n, const double* aabb, int64_t cap, int32_t* pairs, int64_t* total) {
  PairSet s;
  grid_overlaps<2>(load_boxes<2>(n, aabb), s);
  return emit_pairs(s, cap, pairs, total);
}
extern "C" int64_t or_allpairs_overlaps_2d(int n, const double* aabb, int64_t cap, int32_t* pairs,
                                           int64_t* total) {
  PairSet s;
  allpairs_overlaps<2>(load_boxes<2>(n, aabb), s);
  return emit_pairs(s, cap, pairs, total);
}
extern "C" int64_t or_grid_overlaps_3d(int n, const double* aabb, int64_t cap, int32_t* pairs, int64_t* total) {
  PairSet s;
  grid_overlaps<3>(load_boxes<3>(n, aabb), s);
  return emit_pairs(s, cap, pairs, total);
}
extern "C" int64_t or_allpairs_overlaps_3d(int n, const double* aabb, int64_t cap, int32_t* pairs,
                                           int64_t* total) {
  PairSet s;
  allpairs_overlaps<3>(load_boxes<3>(n, aabb), s);
  return emit_pairs(s, cap, pairs, total);
}

extern "C" void or_ccd_coeffs_2d(const double* q0a, const double* q1a, double ra, const double* q0b,
                                 const double* q1b, double rb, double* c3) {
  ccd_coeffs(q0a, q1a, ra, q0b, q1b, rb, c3);
}
extern "C" int or_ccd_happens(const double* c3, double* t_out) { return ccd_happens(c3, t_out) ? 1 : 0; }

// ============================================================================
// Ball2D scene
struct or_ball2d {
  int nb = 0, np = 0;
  std::vector<double> q, v, r, m, minv;
  std::vector<double> px, pn, pt;  // planes: point, unit normal, tangent (-n_y, n_x)
  or_ball2d_params p{};
  // ConstraintCache: (i,j) for ball-ball, (plane, ball) for ball-plane.
  std::map<std::pair<unsigned, unsigned>, std::pair<double, double>> cache_bb, cache_pb;
  // last step's contacts
  std::vector<int32_t> last_ia, last_ib;
  std::vector<double> last_n, last_alpha, last_beta;
  // sweep order for the next step only (empty: sequential active-set order)
  std::vector<int32_t> next_order;
};

namespace {

struct Contact {
  int32_t a, b;    // b >= 0 ball, b = -1 - plane for a static plane
  double nx, ny;   // contact normal
  double tx, ty;   // tangent
};

// SymplecticEulerMap::flow / VerletMap::flow with gravity F = m g.
void umap_flow(const or_ball2d* s, const double* q0, const double* v0, double* q1, double* v1) {
  const double dt = s->p.dt;
  for (int i = 0; i < s->nb; ++i) {
    const double fx = s->m[i] * s->p.gravity[0];
    const double fy = s->m[i] * s->p.gravity[1];
    if (s->p.integrator == OR_SYMPLECTIC_EULER) {
      // v1 = v0 + (dt Minv) F ; q1 = q0 + dt v1
      const double sc = dt * s->minv[i];
      v1[2 * i] = v0[2 * i] + sc * fx;
      v1[2 * i + 1] = v0[2 * i + 1] + sc * fy;
      q1[2 * i] = q0[2 * i] + dt * v1[2 * i];
      q1[2 * i + 1] = q0[2 * i + 1] + dt * v1[2 * i + 1];
    } else {
      // v_half = v0 + (0.5 dt Minv) F(q0) ; q1 = q0 + dt v_half ; v1 = v_half + (0.5 dt Minv) F(q1)
      const double sc = (0.5 * dt) * s->minv[i];
      const double vhx = v0[2 * i] + sc * fx;
      const double vhy = v0[2 * i + 1] + sc * fy;
      q1[2 * i] = q0[2 * i] + dt * vhx;
      q1[2 * i + 1] = q0[2 * i + 1] + dt * vhy;
      v1[2 * i] = vhx + sc * fx;
      v1[2 * i + 1] = vhy + sc * fy;
    }
  }
}

// Ball2DSim::computeActiveSet: ball-ball (grid + CCD) then ball-plane.
void active_set(const or_ball2d* s, const double* q0, const double* q1, std::vector<Contact>& out) {
  out.clear();
  const int nb = s->nb;
  std::vector<Box<2>> boxes(nb);
  for (int i = 0; i < nb; ++i) {
    for (int d = 0; d < 2; ++d) {
      const double lo = std::min(q1[2 * i + d], q0[2 * i + d]);
      const double hi = std::max(q1[2 * i + d], q0[2 * i + d]);
      boxes[i].mn[d] = lo - s->r[i];
      boxes[i].mx[d] = hi + s->r[i];
    }
  }
  PairSet cand;
  grid_overlaps<2>(boxes, cand);
  for (const auto& pr : cand) {
    const unsigned a = pr.first, b = pr.second;
    double c[3];
    ccd_coeffs(&q0[2 * a], &q1[2 * a], s->r[a], &q0[2 * b], &q1[2 * b], s->r[b], c);
    if (!ccd_happens(c, nullptr)) continue;
    // BallBallConstraint: n = normalized(q0a - q0b)
    double dx = q0[2 * a] - q0[2 * b], dy = q0[2 * a + 1] - q0[2 * b + 1];
    const double z = dx * dx + dy * dy;
    if (z > 0.0) {
      const double sq = std::sqrt(z);
      dx = dx / sq;
      dy = dy / sq;
    }
    out.push_back(Contact{int32_t(a), int32_t(b), dx, dy, -dy, dx});
  }
  for (int pl = 0; pl < s->np; ++pl) {
    const double nx = s->pn[2 * pl], ny = s->pn[2 * pl + 1];
    for (int i = 0; i < nb; ++i) {
      const double d = nx * (q1[2 * i] - s->px[2 * pl]) + ny * (q1[2 * i + 1] - s->px[2 * pl + 1]);
      if (d <= s->r[i]) out.push_back(Contact{int32_t(i), int32_t(-1 - pl), nx, ny, s->pt[2 * pl], s->pt[2 * pl + 1]});
    }
  }
}

std::pair<unsigned, unsigned> cache_key(const Contact& c) {
  if (c.b >= 0) return {unsigned(c.a), unsigned(c.b)};
  return {unsigned(-1 - c.b), unsigned(c.a)};
}

}  // namespace

extern "C" or_ball2d* or_ball2d_create(int nb, const double* q, const double* v, const double* r,
                                       const double* m, int np, const double* plane_x, const double* plane_n,
                                       const or_ball2d_params* p) {
  auto* s = new or_ball2d;
  s->nb = nb;
  s->np = np;
  s->q.assign(q, q + 2 * nb);
  s->v.assign(v, v + 2 * nb);
  s->r.assign(r, r + nb);
  s->m.assign(m, m + nb);
  s->minv.resize(nb);
  for (int i = 0; i < nb; ++i) s->minv[i] = 1.0 / m[i];
  s->px.assign(plane_x, plane_x + 2 * np);
  s->pn.resize(2 * np);
  s->pt.resize(2 * np);
  for (int pl = 0; pl < np; ++pl) {
    // StaticPlane: n = normalized(n), t = (-n_y, n_x)
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

extern "C" void or_ball2d_destroy(or_ball2d* s) { delete s; }

extern "C" void or_ball2d_get_state(const or_ball2d* s, double* q, double* v) {
  std::memcpy(q, s->q.data(), sizeof(double) * 2 * s->nb);
  std::memcpy(v, s->v.data(), sizeof(double) * 2 * s->nb);
}

extern "C" void or_ball2d_set_state(or_ball2d* s, const double* q, const double* v) {
  std::memcpy(s->q.data(), q, sizeof(double) * 2 * s->nb);
  std::memcpy(s->v.data(), v, sizeof(double) * 2 * s->nb);
}

extern "C" void or_ball2d_umap(const or_ball2d* s, uint32_t, const double* q0, const double* v0, double* q1,
                               double* v1) {
  umap_flow(s, q0, v0, q1, v1);
}

extern "C" int64_t or_ball2d_active_set(const or_ball2d* s, const double* q0, const double* q1, int64_t cap,
                                        int32_t* ia, int32_t* ib) {
  std::vector<Contact> cs;
  active_set(s, q0, q1, cs);
  if (int64_t(cs.size()) > cap) return -int64_t(cs.size()) - 1;
  for (size_t k = 0; k < cs.size(); ++k) {
    ia[k] = cs[k].a;
    ib[k] = cs[k].b;
  }
  return int64_t(cs.size());
}

extern "C" int64_t or_ball2d_last_contacts(const or_ball2d* s, int64_t cap, int32_t* ia, int32_t* ib, double* n,
                                           double* alpha, double* beta) {
  const int64_t nc = int64_t(s->last_ia.size());
  if (nc > cap) return -nc - 1;
  for (int64_t k = 0; k < nc; ++k) {
    if (ia) ia[k] = s->last_ia[k];
    if (ib) ib[k] = s->last_ib[k];
    if (n) {
      n[2 * k] = s->last_n[2 * k];
      n[2 * k + 1] = s->last_n[2 * k + 1];
    }
    if (alpha) alpha[k] = s->last_alpha[k];
    if (beta) beta[k] = s->last_beta[k];
  }
  return nc;
}

// GeometricImpactFrictionMap::flow with Sobogus(Balls2D), or SymplecticEulerImpactFrictionMap::flow
// (SymplecticEulerImpactFrictionMap.cpp:201-400) when p.staggering says so.
extern "C" int or_ball2d_step(or_ball2d* s, uint32_t iteration, or_step_stats* stats) {
  (void)iteration;
  const int nb = s->nb;
  const bool se = s->p.staggering == OR_STAGGER_SYMPLECTIC_EULER;
  // StabilizedImpactFrictionMap::flow (StabilizedImpactFrictionMap.cpp:48-167): the unconstrained
  // step first, then a cold solve from its velocity v1, then q1 = q0 + dt v.
  const bool stab = s->p.staggering == OR_STAGGER_STABILIZED;
  const double dt = s->p.dt;
  std::vector<double> q1(2 * nb), v1(2 * nb), vdelta;
  if (se) {
    // F = 0 + m g (Ball2DSim::computeForce, Ball2DGravityForce.cpp:36-46); vdelta = dt (Minv F), the
    // sparse product accumulating from zero; predictor q1 = q0 + dt (v0 + vdelta) (:219-229).
    vdelta.resize(2 * nb);
    for (int i = 0; i < nb; ++i)
      for (int d = 0; d < 2; ++d) {
        const double F = 0.0 + s->m[i] * s->p.gravity[d];
        vdelta[2 * i + d] = dt * (0.0 + s->minv[i] * F);
        v1[2 * i + d] = s->v[2 * i + d] + vdelta[2 * i + d];
        q1[2 * i + d] = s->q[2 * i + d] + dt * v1[2 * i + d];
      }
  } else {
    // Unconstrained predictor (GeometricImpactFrictionMap.cpp:279).
    umap_flow(s, s->q.data(), s->v.data(), q1.data(), v1.data());
  }
  std::vector<Contact> cs;
  active_set(s, s->q.data(), q1.data(), cs);
  const int nc = int(cs.size());
  int64_t nbb = 0;
  for (const auto& c : cs) nbb += (c.b >= 0);
  s->last_ia.resize(nc);
  s->last_ib.resize(nc);
  s->last_n.resize(2 * nc);
  s->last_alpha.assign(nc, 0.0);
  s->last_beta.assign(nc, 0.0);
  if (stats) {
    stats->n_contacts = nc;
    stats->n_ball_ball = nbb;
    stats->n_ball_plane = nc - nbb;
    stats->iterations = 0;
    stats->succeeded = 1;
    stats->error = 0.0;
  }
  if (nc == 0) {
    // No contacts: keep the predictor, clear the cache (:286-298).
    s->cache_bb.clear();
    s->cache_pb.clear();
    s->q.swap(q1);
    s->v.swap(v1);
    return 0;
  }
  std::vector<int32_t> ia(nc), ib(nc);
  std::vector<double> bases(4 * nc), CoR(nc, s->p.CoR), mu(nc, s->p.mu), alpha(nc, 0.0), beta(nc, 0.0);
  for (int k = 0; k < nc; ++k) {
    ia[k] = cs[k].a;
    ib[k] = cs[k].b >= 0 ? cs[k].b : -1;
    bases[4 * k] = cs[k].nx;
    bases[4 * k + 1] = cs[k].ny;
    bases[4 * k + 2] = cs[k].tx;
    bases[4 * k + 3] = cs[k].ty;
  }
  // initializeImpulses (:174-220): decache, then clear the cache.
  if (s->p.cache_mode != OR_CACHE_NONE) {
    for (int k = 0; k < nc; ++k) {
      const auto key = cache_key(cs[k]);
      const auto& cache = cs[k].b >= 0 ? s->cache_bb : s->cache_pb;
      const auto it = cache.find(key);
      if (it != cache.end()) {
        alpha[k] = it->second.first;
        beta[k] = (s->p.cache_mode == OR_CACHE_NORMAL_AND_FRICTION) ? it->second.second : 0.0;
      }
    }
  }
  s->cache_bb.clear();
  s->cache_pb.clear();
  std::vector<double> v2(2 * nb), f(2 * nb);
  or_gs_params gp{s->p.tol, s->p.max_iters, s->p.eval_every,
                  int64_t(s->next_order.size()) == int64_t(nc) ? s->next_order.data() : nullptr};
  or_gs_result gr{};
  if (se) {
    // nrel = N^T vdelta, drel = D^T vdelta (:294-305): per contact the column's entries in row
    // order (body a's, then body b's, a < b), accumulated from zero as Eigen's sparse product does;
    // N holds n, -n and D holds t, -t.  Stabilisation: nrel += min(0, gap(q0)) / dt unless the gap
    // is smaller in magnitude than the penetration threshold (:307-321).
    std::vector<double> nrel(nc), drel(nc);
    for (int k = 0; k < nc; ++k) {
      const auto& c = cs[k];
      const double* da = &vdelta[2 * c.a];
      double tn = 0.0, tt = 0.0;
      tn = tn + c.nx * da[0];
      tn = tn + c.ny * da[1];
      tt = tt + c.tx * da[0];
      tt = tt + c.ty * da[1];
      if (c.b >= 0) {
        const double* db = &vdelta[2 * c.b];
        tn = tn + (-c.nx) * db[0];
        tn = tn + (-c.ny) * db[1];
        tt = tt + (-c.tx) * db[0];
        tt = tt + (-c.ty) * db[1];
      }
      nrel[k] = 0.0 + 1.0 * tn;
      drel[k] = 0.0 + 1.0 * tt;
      if (s->p.stabilize) {
        double gap;
        if (c.b >= 0) {
          // BallBallConstraint::evaluateGapFunction (:76-86)
          const double dx = s->q[2 * c.a] - s->q[2 * c.b], dy = s->q[2 * c.a + 1] - s->q[2 * c.b + 1];
          gap = std::sqrt(dx * dx + dy * dy) - (s->r[c.a] + s->r[c.b]);
        } else {
          // StaticPlaneConstraint::evaluateGapFunction (BallStaticPlaneConstraint.cpp:58-63)
          const int pl = -1 - c.b;
          const double dx = s->q[2 * c.a] - s->px[2 * pl], dy = s->q[2 * c.a + 1] - s->px[2 * pl + 1];
          gap = (s->pn[2 * pl] * dx + s->pn[2 * pl + 1] * dy) - s->r[c.a];
        }
        double g0 = std::min(0.0, gap);
        if (std::fabs(g0) < s->p.penetration_threshold) g0 = 0.0;
        nrel[k] = nrel[k] + g0 / dt;
      }
    }
    or_sobogus_solve_2d_ex(nb, s->m.data(), s->v.data(), nc, ia.data(), ib.data(), bases.data(), CoR.data(),
                           mu.data(), nrel.data(), drel.data(), &gp, alpha.data(), beta.data(), v2.data(), f.data(),
                           &gr);
  } else {
    or_sobogus_solve_2d(nb, s->m.data(), stab ? v1.data() : s->v.data(), nc, ia.data(), ib.data(), bases.data(),
                        CoR.data(), mu.data(), &gp, alpha.data(), beta.data(), v2.data(), f.data(), &gr);
  }
  s->next_order.clear();
  // cacheImpulses (:222-264)
  if (s->p.cache_mode != OR_CACHE_NONE) {
    for (int k = 0; k < nc; ++k) {
      auto& cache = cs[k].b >= 0 ? s->cache_bb : s->cache_pb;
      cache[cache_key(cs[k])] = {alpha[k], s->p.cache_mode == OR_CACHE_NORMAL_AND_FRICTION ? beta[k] : 0.0};
    }
  }
  for (int k = 0; k < nc; ++k) {
    s->last_ia[k] = cs[k].a;
    s->last_ib[k] = cs[k].b;
    s->last_n[2 * k] = cs[k].nx;
    s->last_n[2 * k + 1] = cs[k].ny;
    s->last_alpha[k] = alpha[k];
    s->last_beta[k] = beta[k];
  }
  if (stats) {
    stats->iterations = gr.iterations;
    stats->succeeded = gr.succeeded;
    stats->error = gr.error;
  }
  if (se) {
    // v1 = v2 + vdelta, q1 = q0 + dt v1 (:363, :406).
    for (int i = 0; i < 2 * nb; ++i) {
      v1[i] = v2[i] + vdelta[i];
      q1[i] = s->q[i] + dt * v1[i];
    }
  } else if (stab) {
    // v1 = v2, q1 = q0 + dt v1 (StabilizedImpactFrictionMap.cpp:136, :167).
    for (int i = 0; i < 2 * nb; ++i) {
      v1[i] = v2[i];
      q1[i] = s->q[i] + dt * v1[i];
    }
  } else {
    // Final map with the post-impact velocity (:441).
    umap_flow(s, s->q.data(), v2.data(), q1.data(), v1.data());
  }
  s->q.swap(q1);
  s->v.swap(v1);
  return gr.succeeded ? 0 : 1;
}

extern "C" int or_ball2d_run(or_ball2d* s, uint32_t first_iteration, uint32_t n_steps, or_step_stats* stats,
                             int64_t* total_contacts) {
  int bad = 0;
  int64_t tot = 0;
  or_step_stats st{};
  for (uint32_t k = 0; k < n_steps; ++k) {
    bad += or_ball2d_step(s, first_iteration + k, &st);
    tot += st.n_contacts;
  }
  if (stats) *stats = st;
  if (total_contacts) *total_contacts = tot;
  return bad;
}

extern "C" void or_ball2d_set_solver(or_ball2d* s, double tol, uint32_t max_iters) {
  s->p.tol = tol;
  s->p.max_iters = max_iters;
}

// Replaces the impulse cache (ConstraintCache, ball2d/ConstraintCache.cpp:20-120) with the given contacts'
// impulses: ia, ib as the step's contacts (ib = -1 - plane for a static plane), alpha, beta.  Used to
// start the oracle from another solver's state, impulse cache included.
extern "C" void or_ball2d_set_cache(or_ball2d* s, int64_t nc, const int32_t* ia, const int32_t* ib, const double* alpha,
                                    const double* beta) {
  s->cache_bb.clear();
  s->cache_pb.clear();
  for (int64_t k = 0; k < nc; ++k) {
    Contact c{};
    c.a = ia[k];
    c.b = ib[k];
    auto& cache = c.b >= 0 ? s->cache_bb : s->cache_pb;
    cache[cache_key(c)] = {alpha[k], beta[k]};
  }
}

extern "C" void or_ball2d_set_next_order(or_ball2d* s, int64_t nc, const int32_t* order) {
  s->next_order.assign(order, order + nc);
}
