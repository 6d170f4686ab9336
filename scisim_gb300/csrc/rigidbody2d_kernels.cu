// rigidbody2d_kernels.cu -- RigidBody2D circles: one GeometricImpactFrictionMap::flow (or
// StabilizedImpactFrictionMap::flow) step of a RigidBody2DSim whose bodies are circles, with
// Sobogus(RigidBody2D), on the GPU.
//
// A body has three degrees of freedom (x, y, theta), mass block diag(m, m, I) and velocity
// (vx, vy, omega).  Reference path:
//   SymplecticEulerMap / VerletMap          rigidbody2d/SymplecticEulerMap.cpp:12-31,
//                                           rigidbody2d/VerletMap.cpp:23-37 (gravity on x, y only,
//                                           rigidbody2d/NearEarthGravityForce.cpp:20-28)
//   RigidBody2DSim::computeActiveSet        rigidbody2d/RigidBody2DSim.cpp:696-714 (swept circle
//                                           AABBs, grid pairs, CCD :248-312; planes :638-694)
//   CircleCircleConstraint                  rigidbody2d/CircleCircleConstraint.cpp (n and the contact
//                                           point p fixed at q0; H rows [n^T 0; t^T cross(arm, t)])
//   StaticPlaneCircleConstraint             rigidbody2d/StaticPlaneCircleConstraint.cpp (arm -r n)
//   SobogusFrictionProblem::initializeRigidBody2D / solveRigidBody2D
//                                           scisim/ConstrainedMaps/Sobogus.cpp:110-182, :375-484
//   RigidBody2DSobogusInterface             scisim/ConstrainedMaps/bogus/RigidBody2DSobogusInterface.cpp
//   ConstraintCache                         rigidbody2d/ConstraintCache.cpp (keys (i, j), (plane, body))
// The broad phase, its CCD and the plane test are the Ball2D kernels on the centres the predictor
// copies out (pos0, pos1); the contact graph colouring is the shared one.  The Delassus block of a
// circle contact is diagonal in (n, t) up to rounding but not isotropic: w_tt adds arm^2 / I per
// side.  Sweeps run in FP64 in colour order; every operation follows the reference's order, so the
// oracle replaying the colour order reproduces every step bit for bit.
#include "coulomb2d.cuh"
#include "ctx.hpp"

#include <algorithm>
#include <utility>

namespace sg {
namespace {

constexpr int kBlock = 256;
constexpr int kGsRbBlock = 512;
inline int blocks_for(long n) { return (int)((n + kBlock - 1) / kBlock); }

// MathUtilities::cross (scisim/Math/MathUtilities.h:16-19)
__device__ __forceinline__ double cross2(double ax, double ay, double bx, double by) { return ax * by - ay * bx; }

// The unconstrained map of 3-dof bodies with F = (m g, 0): symplectic Euler v1 = v0 + (dt Minv) F,
// q1 = q0 + dt v1; Verlet with half kicks (the force does not depend on q).  With aabb non-null it
// also writes the body's centres at q0 and q1 and its swept AABB (the predictor of the step).
__global__ void k_rb2d_umap(int nb, int integrator, double dt, double gx, double gy, const double* __restrict__ q0,
                            const double* __restrict__ vin, const double* __restrict__ m,
                            const double* __restrict__ minv, const double* __restrict__ Iinv,
                            const double* __restrict__ rad, double* __restrict__ q1, double* __restrict__ v1,
                            double2* __restrict__ pos0, double2* __restrict__ pos1, double4_32a* __restrict__ aabb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const double F[3] = {0.0 + m[i] * gx, 0.0 + m[i] * gy, 0.0};
  const double mi[3] = {minv[i], minv[i], Iinv[i]};
  double a[3], b[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double x0 = q0[3 * (size_t)i + d], w0 = vin[3 * (size_t)i + d];
    if (integrator == SG_VERLET) {
      const double sc = (0.5 * dt) * mi[d];
      const double vh = w0 + sc * F[d];
      a[d] = x0 + dt * vh;
      b[d] = vh + sc * F[d];
    } else {
      const double sc = dt * mi[d];
      b[d] = w0 + sc * F[d];
      a[d] = x0 + dt * b[d];
    }
    q1[3 * (size_t)i + d] = a[d];
    v1[3 * (size_t)i + d] = b[d];
  }
  if (aabb) {
    const double x0 = q0[3 * (size_t)i], y0 = q0[3 * (size_t)i + 1], r = rad[i];
    pos0[i] = make_double2(x0, y0);
    pos1[i] = make_double2(a[0], a[1]);
    // CircleGeometry::computeCollisionAABB over the step: min / max of the two centres, -/+ r.
    const double lx = (a[0] < x0) ? a[0] : x0, ly = (a[1] < y0) ? a[1] : y0;
    const double hx = (x0 < a[0]) ? a[0] : x0, hy = (y0 < a[1]) ? a[1] : y0;
    aabb[i] = make_double4_32a(lx - r, ly - r, hx + r, hy + r);
  }
}

// StabilizedImpactFrictionMap's closing update: v1 = v2, q1 = q0 + dt v1.
__global__ void k_rb2d_final_stab(int nb, double dt, const double* __restrict__ q0, const double* __restrict__ v2,
                                  double* __restrict__ q1, double* __restrict__ v1) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= 3 * nb) return;
  v1[j] = v2[j];
  q1[j] = q0[j] + dt * v1[j];
}

__device__ __forceinline__ unsigned long long rb_contact_key(int a, int b) {
  if (b >= 0) return ((unsigned long long)(unsigned)a << 32) | (unsigned)b;
  const unsigned p = (unsigned)(-1 - b);
  return 0x8000000000000000ull | ((unsigned long long)p << 32) | (unsigned)a;
}

__device__ __forceinline__ long rb_find_key(const unsigned long long* keys, long n, unsigned long long k) {
  long lo = 0, hi = n;
  while (lo < hi) {
    const long mid = (lo + hi) >> 1;
    if (keys[mid] < k)
      lo = mid + 1;
    else
      hi = mid;
  }
  return (lo < n && keys[lo] == k) ? lo : -1;
}

struct RbAssemble {
  int nc;
  const int* ia;
  const int* ib;
  const double2* pos0;      // centres at q0
  const double* v0;         // 3 per body
  const double* rad;
  const double* minv;
  const double* Iinv;
  const double2* plane_n;
  const double2* plane_t;
  double mu, CoR;
  int cache_mode;
  const unsigned long long* prev_key;
  const double2* prev_ab;
  long prev_n;
  double2* n;
  double2* ct;              // cross(arm_a, t), cross(arm_b, t)
  double2* c;
  double* W;
  double* mu_out;
  double2* r;
  unsigned long long* key;
};

// Per contact: basis, angular tangent entries, forcing term, diagonal Delassus block and the warm
// start from the previous step's impulses (CircleCircleConstraint / StaticPlaneCircleConstraint,
// Constraint::computeForcingTerm, SobogusFrictionProblem::initializeRigidBody2D, initializeImpulses).
__global__ void k_rb2d_assemble(RbAssemble A) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= A.nc) return;
  const int a = A.ia[k], b = A.ib[k];
  double nx, ny, tx, ty, ca, cb = 0.0, vrx, vry;
  const double vax = A.v0[3 * (size_t)a], vay = A.v0[3 * (size_t)a + 1];
  if (b >= 0) {
    const double2 qa = A.pos0[a], qb = A.pos0[b];
    // n = (q0a - q0b).normalized(); p = q0a + (ra / (ra + rb)) (q0b - q0a)
    double dx = qa.x - qb.x, dy = qa.y - qb.y;
    const double z = dx * dx + dy * dy;
    if (z > 0.0) {
      const double sq = sqrt(z);
      dx = dx / sq;
      dy = dy / sq;
    }
    nx = dx;
    ny = dy;
    tx = -ny;
    ty = nx;
    const double f = A.rad[a] / (A.rad[a] + A.rad[b]);
    const double pxc = qa.x + f * (qb.x - qa.x);
    const double pyc = qa.y + f * (qb.y - qa.y);
    ca = cross2(pxc - qa.x, pyc - qa.y, tx, ty);
    cb = cross2(pxc - qb.x, pyc - qb.y, tx, ty);
    vrx = vax - A.v0[3 * (size_t)b];
    vry = vay - A.v0[3 * (size_t)b + 1];
  } else {
    const int p = -1 - b;
    const double2 pn = A.plane_n[p], pt = A.plane_t[p];
    nx = pn.x;
    ny = pn.y;
    tx = pt.x;
    ty = pt.y;
    // arm r_world = -r n
    ca = cross2(-A.rad[a] * nx, -A.rad[a] * ny, tx, ty);
    vrx = vax - 0.0;
    vry = vay - 0.0;
  }
  const double ndotv = nx * vrx + ny * vry;
  const double nrel = -(0.0 * nx + 0.0 * ny);
  const double drel = -(0.0 * tx + 0.0 * ty);
  const double sv = A.CoR * ndotv + nrel;
  const double wx = (0.0 + nx * sv) + tx * drel;
  const double wy = (0.0 + ny * sv) + ty * drel;
  A.n[k] = make_double2(nx, ny);
  A.ct[k] = make_double2(ca, cb);
  A.c[k] = make_double2(nx * wx + ny * wy, tx * wx + ty * wy);
  const double nn = nx * nx + ny * ny;
  const double nt = nx * tx + ny * ty;
  const double tt = tx * tx + ty * ty;
  const double ma = A.minv[a];
  double w00 = ma * nn;
  double w01 = ma * nt;
  double w11 = ma * tt + A.Iinv[a] * (ca * ca);
  if (b >= 0) {
    const double mb = A.minv[b];
    w00 = w00 + mb * nn;
    w01 = w01 + mb * nt;
    w11 = w11 + (mb * tt + A.Iinv[b] * (cb * cb));
  }
  A.W[3 * (size_t)k] = w00;
  A.W[3 * (size_t)k + 1] = w01;
  A.W[3 * (size_t)k + 2] = w11;
  A.mu_out[k] = A.mu;
  const unsigned long long key = rb_contact_key(a, b);
  A.key[k] = key;
  double alpha = 0.0, beta = 0.0;
  if (A.cache_mode != SG_CACHE_NONE && A.prev_n > 0) {
    const long idx = rb_find_key(A.prev_key, A.prev_n, key);
    if (idx >= 0) {
      const double2 ab = A.prev_ab[idx];
      alpha = ab.x;
      beta = (A.cache_mode == SG_CACHE_NORMAL_AND_FRICTION) ? ab.y : 0.0;
    }
  }
  // r = alpha n + beta t, local r = E^T r (Sobogus.cpp:400-402)
  const double rwx = alpha * nx + beta * tx;
  const double rwy = alpha * ny + beta * ty;
  A.r[k] = make_double2(nx * rwx + ny * rwy, tx * rwx + ty * rwy);
}

// H^T r of one body over its contacts in ascending contact order: (x, y, theta).
__device__ __forceinline__ void rb_gather(int body, const int* __restrict__ off, const int* __restrict__ adj,
                                          const int* __restrict__ ia, const double2* __restrict__ n,
                                          const double2* __restrict__ ct, const double2* r, double* h) {
  h[0] = h[1] = h[2] = 0.0;
  const int e = off[body + 1];
  for (int p = off[body]; p < e; ++p) {
    const int k = adj[p];
    const bool is_a = ia[k] == body;
    const double sgn = is_a ? 1.0 : -1.0;
    const double2 nk = n[k], rk = r[k], ck = ct[k];
    const double tx = -nk.y, ty = nk.x;
    h[0] = h[0] + sgn * (nk.x * rk.x + tx * rk.y);
    h[1] = h[1] + sgn * (nk.y * rk.x + ty * rk.y);
    h[2] = h[2] + sgn * ((is_a ? ck.x : ck.y) * rk.y);
  }
}

// Running velocities v = v0 + Minv H^T r.
__global__ void k_rb2d_vel_init(int nb, const int* __restrict__ off, const int* __restrict__ adj,
                                const int* __restrict__ ia, const double2* __restrict__ n,
                                const double2* __restrict__ ct, const double2* __restrict__ r,
                                const double* __restrict__ v0, const double* __restrict__ minv,
                                const double* __restrict__ Iinv, double4_32a* __restrict__ V) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  double h[3];
  rb_gather(i, off, adj, ia, n, ct, r, h);
  const double* w = v0 + 3 * (size_t)i;
  V[i] = make_double4_32a(w[0] + minv[i] * h[0], w[1] + minv[i] * h[1], w[2] + Iinv[i] * h[2], 0.0);
}

// v2 = Minv (H^T r - f), f = -M v0, for bodies in contacts; the others keep v0.
__global__ void k_rb2d_final_velocity(int nb, const int* __restrict__ off, const int* __restrict__ adj,
                                      const int* __restrict__ ia, const double2* __restrict__ n,
                                      const double2* __restrict__ ct, const double2* __restrict__ r,
                                      const double* __restrict__ v0, const double* __restrict__ m,
                                      const double* __restrict__ I, const double* __restrict__ minv,
                                      const double* __restrict__ Iinv, double* __restrict__ v2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const double* w = v0 + 3 * (size_t)i;
  double* o = v2 + 3 * (size_t)i;
  if (off[i + 1] == off[i]) {
    o[0] = w[0];
    o[1] = w[1];
    o[2] = w[2];
    return;
  }
  double h[3];
  rb_gather(i, off, adj, ia, n, ct, r, h);
  o[0] = minv[i] * (h[0] - (-(m[i] * w[0])));
  o[1] = minv[i] * (h[1] - (-(m[i] * w[1])));
  o[2] = Iinv[i] * (h[2] - (-(I[i] * w[2])));
}

// alpha = r . n, beta = r . t (zero when mu is zero) (Sobogus.cpp:421-437).
__global__ void k_rb2d_extract(int nc, const double2* __restrict__ n, const double2* __restrict__ r,
                               const double* __restrict__ mu, double2* __restrict__ ab) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nc) return;
  const double2 nk = n[k], rk = r[k];
  const double nx = nk.x, ny = nk.y, tx = -ny, ty = nx;
  const double rwx = nx * rk.x + tx * rk.y;
  const double rwy = ny * rk.x + ty * rk.y;
  ab[k] = make_double2(rwx * nx + rwy * ny, (mu[k] == 0.0) ? 0.0 : (rwx * tx + rwy * ty));
}

struct RbGsArgs {
  int nc;
  const int* ia;
  const int* ib;
  const double2* n;
  const double2* ct;
  const double2* c;
  const double* W;
  const double* mu;
  const double* minv;
  const double* Iinv;
  const int* perm;
  double2* r;
  double2* r_a;  // snapshot buffers for best-iterate tracking
  double2* r_b;
  double4_32a* v;
  SolveStats* st;
  GridBarrier* gb;
  unsigned long long spin;
  double tol;
  unsigned max_iters;
  unsigned eval_every;
};

// Running velocities are written by other SMs between grid barriers: read at L2.
__device__ __forceinline__ double4_32a ld_v(const double4_32a* p) {
  const double2* q = reinterpret_cast<const double2*>(p);
  const double2 a = __ldcg(q), b = __ldcg(q + 1);
  return make_double4_32a(a.x, a.y, b.x, b.y);
}

// u = H v + c of contact k at the running velocities.
__device__ __forceinline__ void rb_local_u(const RbGsArgs& A, int k, const double4_32a& va, bool has_b,
                                           const double4_32a& vb, double& u0, double& u1) {
  const double2 nk = A.n[k], ck = A.ct[k], cc = A.c[k];
  const double nx = nk.x, ny = nk.y, tx = -ny, ty = nx;
  double hn = nx * va.x + ny * va.y;
  double ht = (tx * va.x + ty * va.y) + ck.x * va.z;
  if (has_b) {
    hn = hn - (nx * vb.x + ny * vb.y);
    ht = ht - ((tx * vb.x + ty * vb.y) + ck.y * vb.z);
  }
  u0 = hn + cc.x;
  u1 = ht + cc.y;
}

__device__ __forceinline__ void rb_gs_update(const RbGsArgs& A, int k) {
  const int a = A.ia[k], b = A.ib[k];
  const bool has_b = b >= 0;
  const double4_32a va = ld_v(&A.v[a]);
  const double4_32a vb = has_b ? ld_v(&A.v[b]) : make_double4_32a(0.0, 0.0, 0.0, 0.0);
  double u0, u1;
  rb_local_u(A, k, va, has_b, vb, u0, u1);
  const double2 rk = __ldcg(&A.r[k]);
  const double r0 = rk.x, r1 = rk.y;
  const double w00 = A.W[3 * (size_t)k], w01 = A.W[3 * (size_t)k + 1], w11 = A.W[3 * (size_t)k + 2];
  const double bt0 = u0 - (w00 * r0 + w01 * r1);
  const double bt1 = u1 - (w01 * r0 + w11 * r1);
  double rn0, rn1;
  local_solve_2d(w00, w01, w11, bt0, bt1, A.mu[k], rn0, rn1);
  const double d0 = rn0 - r0, d1 = rn1 - r1;
  const double2 nk = A.n[k], ck = A.ct[k];
  const double nx = nk.x, ny = nk.y, tx = -ny, ty = nx;
  const double px = nx * d0 + tx * d1, py = ny * d0 + ty * d1;
  const double ma = A.minv[a];
  A.v[a] = make_double4_32a(va.x + ma * px, va.y + ma * py, va.z + A.Iinv[a] * (ck.x * d1), 0.0);
  if (has_b) {
    const double mb = A.minv[b];
    A.v[b] = make_double4_32a(vb.x - mb * px, vb.y - mb * py, vb.z - A.Iinv[b] * (ck.y * d1), 0.0);
  }
  A.r[k] = make_double2(rn0, rn1);
}

// Coloured block Gauss-Seidel over 3-dof bodies in FP64 (Sobogus's GaussSeidel with the 2D SOC
// law): colours separated by grid barriers, the FB residual every eval_every sweeps, the best
// iterate kept when max_iters is reached (sobogus_patch.patch:60-70).
__global__ void __launch_bounds__(kGsRbBlock, 1) k_gs_rb2d(RbGsArgs A) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nthr = gridDim.x * blockDim.x;
  if (*((volatile int*)&A.st->status) != 0) return;
  __shared__ int s_off[kMaxColors + 1];
  __shared__ int s_ncol;
  if (threadIdx.x == 0) s_ncol = A.st->n_colors;
  for (int c = threadIdx.x; c <= kMaxColors; c += blockDim.x) s_off[c] = A.st->color_off[c];
  __syncthreads();
  const int ncol = s_ncol;
  const unsigned eval_every = A.eval_every ? A.eval_every : 1u;
  double2* best = A.r_a;
  double2* cand = A.r_b;
  double err_best = INFINITY;
  bool converged = false;
  unsigned it = 0, n_eval = 0;
  for (it = 1; it <= A.max_iters; ++it) {
    for (int col = 0; col < ncol; ++col) {
      const int e = s_off[col + 1];
      for (int s = s_off[col] + tid; s < e; s += nthr) rb_gs_update(A, A.perm[s]);
      if (!grid_sync(A.gb, A.spin)) {
        if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
        return;
      }
    }
    if (it % eval_every == 0) {
      double emax = 0.0;
      for (int k = tid; k < A.nc; k += nthr) {
        const int a = A.ia[k], b = A.ib[k];
        const bool has_b = b >= 0;
        const double4_32a va = ld_v(&A.v[a]);
        const double4_32a vb = has_b ? ld_v(&A.v[b]) : make_double4_32a(0.0, 0.0, 0.0, 0.0);
        double u0, u1;
        rb_local_u(A, k, va, has_b, vb, u0, u1);
        const double2 rk = __ldcg(&A.r[k]);
        cand[k] = rk;
        emax = nanmax(emax, fb_error_2d(rk.x, rk.y, u0, u1, A.mu[k]));
      }
      emax = block_nanmax(emax);
      const int slot = n_eval % 3;
      if (threadIdx.x == 0) atomicMax(&A.st->err_slot[slot], f64_to_ordered(emax));
      if (tid == 0) A.st->err_slot[(n_eval + 1) % 3] = 0ull;
      if (!grid_sync(A.gb, A.spin)) {
        if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
        return;
      }
      const double err = ordered_to_f64(*((volatile unsigned long long*)&A.st->err_slot[slot]));
      ++n_eval;
      if (err < err_best) {
        err_best = err;
        double2* t = best;
        best = cand;
        cand = t;
      }
      if (err < A.tol) {
        converged = true;
        break;
      }
    }
  }
  if (!converged) {
    if (err_best < INFINITY)
      for (int k = tid; k < A.nc; k += nthr) A.r[k] = __ldcg(&best[k]);
    it = A.max_iters;
  }
  if (tid == 0) {
    A.st->iterations = it;
    A.st->converged = converged ? 1 : 0;
    A.st->error = err_best;
    A.st->sweeps64 = it;
    A.st->evals = n_eval;
  }
}

}  // namespace

// One step of a RigidBody2D circle scene: GeometricImpactFrictionMap::flow
// (scisim/ConstrainedMaps/GeometricImpactFrictionMap.cpp:267-442) or, with SG_STAGGER_STABILIZED,
// StabilizedImpactFrictionMap::flow (scisim/ConstrainedMaps/StabilizedImpactFrictionMap.cpp:48-167).
int rb2d_step(sg_ctx* ctx, sg_step_stats* out) {
  const int nb = ctx->nb;
  cudaStream_t s = ctx->stream;
  sg_step_stats st{};
  const bool stab = ctx->staggering == SG_STAGGER_STABILIZED;
  if (stab && ctx->cfg.cache_mode != SG_CACHE_NONE) {
    set_error("the stabilized staggering keeps no impulse cache");
    return SG_BAD_INPUT;
  }
  if (ctx->staggering == SG_STAGGER_SYMPLECTIC_EULER) {
    set_error("RigidBody2D scenes step with the geometric or the stabilized map");
    return SG_BAD_INPUT;
  }
  if (nb == 0) {
    if (out) *out = st;
    return SG_OK;
  }
  const double* g = ctx->cfg.gravity;
  const double* minv = ctx->minv.as<double>();
  const double* Iinv = ctx->rb_Iinv.as<double>();
  // Predictor, centres and swept AABBs.
  k_rb2d_umap<<<blocks_for(nb), kBlock, 0, s>>>(nb, ctx->cfg.integrator, ctx->cfg.dt, g[0], g[1], ctx->q.as<double>(),
                                                ctx->v.as<double>(), ctx->m.as<double>(), minv, Iinv,
                                                ctx->r.as<double>(), ctx->q1.as<double>(), ctx->v1.as<double>(),
                                                ctx->pos0.as<double2>(), ctx->pos1.as<double2>(),
                                                ctx->aabb.as<double4_32a>());
  SG_CUDA_TRY(cudaGetLastError());
  const double* aabb = ctx->aabb.as<double>();
  if (int r = broadphase_build_grid(ctx, aabb, nb)) return r;
  if (int r = broadphase_count_pairs(ctx, aabb, nb, true)) return r;
  if (int r = plane_flags(ctx)) return r;
  int totals[2] = {0, 0};
  SG_CUDA_TRY(cudaMemcpyAsync(&totals[0], ctx->pair_off.as<int>() + nb, sizeof(int), cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaMemcpyAsync(&totals[1], ctx->plane_off.as<int>() + (long)nb * ctx->np, sizeof(int),
                              cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaStreamSynchronize(s));
  const int npairs = totals[0], nplanes = totals[1];
  const int nc = npairs + nplanes;
  ctx->kernel_launches += 1 + 8 + 4 + (ctx->np > 0 ? 4 : 0);
  ctx->steps += 1;
  ctx->contacts_total += (uint64_t)nc;
  st.n_contacts = nc;
  st.n_ball_ball = npairs;
  st.n_ball_plane = nplanes;
  ctx->last_nc = nc;
  ctx->last_nbb = npairs;
  if (nc == 0) {
    // No active constraints: keep the predictor and clear the cache (:286-298).
    std::swap(ctx->q, ctx->q1);
    std::swap(ctx->v, ctx->v1);
    ctx->prev_n = 0;
    ctx->prev_rows = false;
    ctx->prev_color_valid = false;
    st.succeeded = 1;
    if (out) *out = st;
    return SG_OK;
  }
  if (int r = ensure_contact_capacity(ctx, nc)) return r;
  if (int r = grow(ctx->rb_ct, sizeof(double2) * (size_t)ctx->ccap)) return r;
  int* ia = ctx->ia.as<int>();
  int* ib = ctx->ib.as<int>();
  if (int r = broadphase_write_pairs(ctx, aabb, nb, true, ia, ib)) return r;
  if (int r = plane_write(ctx, npairs)) return r;
  // The stabilized map solves from the unconstrained step's velocity (StabilizedImpactFrictionMap.cpp:127).
  const double* v0 = stab ? ctx->v1.as<double>() : ctx->v.as<double>();
  RbAssemble A;
  A.nc = nc;
  A.ia = ia;
  A.ib = ib;
  A.pos0 = ctx->pos0.as<double2>();
  A.v0 = v0;
  A.rad = ctx->r.as<double>();
  A.minv = minv;
  A.Iinv = Iinv;
  A.plane_n = ctx->plane_n.as<double2>();
  A.plane_t = ctx->plane_t.as<double2>();
  A.mu = ctx->cfg.mu;
  A.CoR = ctx->cfg.CoR;
  A.cache_mode = ctx->cfg.cache_mode;
  A.prev_key = ctx->prev_key.as<unsigned long long>();
  A.prev_ab = ctx->prev_ab.as<double2>();
  A.prev_n = ctx->prev_n;
  A.n = ctx->n.as<double2>();
  A.ct = ctx->rb_ct.as<double2>();
  A.c = ctx->c.as<double2>();
  A.W = ctx->W.as<double>();
  A.mu_out = ctx->mu.as<double>();
  A.r = ctx->r_loc.as<double2>();
  A.key = ctx->key.as<unsigned long long>();
  k_rb2d_assemble<<<blocks_for(nc), kBlock, 0, s>>>(A);
  SG_CUDA_TRY(cudaGetLastError());

  // Solve.
  if (int r = ensure_solver_capacity(ctx, nb, nc)) return r;
  if (int r = grow(ctx->rb_vrun, sizeof(double4_32a) * (size_t)nb)) return r;
  if (int r = grow(ctx->v2, sizeof(double) * 3 * (size_t)nb)) return r;
  if (int r = prepare_contact_graph(ctx, nb, nc, ia, ib)) return r;
  const int* off = ctx->body_off.as<int>();
  const int* adj = ctx->body_adj.as<int>();
  double4_32a* V = ctx->rb_vrun.as<double4_32a>();
  k_rb2d_vel_init<<<blocks_for(nb), kBlock, 0, s>>>(nb, off, adj, ia, A.n, A.ct, A.r, v0, minv, Iinv, V);
  SG_CUDA_TRY(cudaGetLastError());
  SolveStats* sst = ctx->stats.as<SolveStats>();
  GridBarrier* gb = ctx->barrier.as<GridBarrier>();
  SG_CUDA_TRY(cudaMemsetAsync(gb, 0, sizeof(GridBarrier), s));
  RbGsArgs G;
  G.nc = nc;
  G.ia = ia;
  G.ib = ib;
  G.n = A.n;
  G.ct = A.ct;
  G.c = A.c;
  G.W = A.W;
  G.mu = A.mu_out;
  G.minv = minv;
  G.Iinv = Iinv;
  G.perm = ctx->perm.as<int>();
  G.r = A.r;
  G.r_a = ctx->r_cand.as<double2>();
  G.r_b = ctx->r_best.as<double2>();
  G.v = V;
  G.st = sst;
  G.gb = gb;
  G.spin = ctx->spin_limit;
  G.tol = ctx->cfg.tol;
  G.max_iters = ctx->cfg.max_iters;
  G.eval_every = ctx->cfg.eval_every;
  void* args[] = {&G};
  const int grid = coop_grid(ctx, k_gs_rb2d, nc, kGsRbBlock, 1);
  if (ctx->profile) SG_CUDA_TRY(cudaEventRecord(ctx->ev_gs0, s));
  SG_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_gs_rb2d, dim3(grid), dim3(kGsRbBlock), args, 0, s));
  if (ctx->profile) SG_CUDA_TRY(cudaEventRecord(ctx->ev_gs1, s));
  double* v2 = ctx->v2.as<double>();
  k_rb2d_final_velocity<<<blocks_for(nb), kBlock, 0, s>>>(nb, off, adj, ia, A.n, A.ct, A.r, v0, ctx->m.as<double>(),
                                                          ctx->rb_I.as<double>(), minv, Iinv, v2);
  k_rb2d_extract<<<blocks_for(nc), kBlock, 0, s>>>(nc, A.n, A.r, A.mu_out, ctx->ab.as<double2>());
  SG_CUDA_TRY(cudaGetLastError());
  SG_CUDA_TRY(cudaMemcpyAsync(&ctx->h_stats, sst, sizeof(SolveStats), cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaStreamSynchronize(s));
  // pair write, plane write, assemble, vel init, gs, final velocity, extract
  ctx->kernel_launches += 6 + (ctx->np > 0 ? 1 : 0);
  if (ctx->h_stats.status == SG_DEVICE_TIMEOUT) {
    set_error("a device-side wait exceeded its spin limit");
    return SG_DEVICE_TIMEOUT;
  }
  if (ctx->h_stats.status == SG_CAPACITY) {
    set_error("contact colouring exceeded 64 colours or its round limit");
    return SG_CAPACITY;
  }
  ctx->gs_launches += 1;
  ctx->contact_sweeps += (uint64_t)ctx->h_stats.sweeps64 * (uint64_t)nc;
  ctx->contact_evals += (uint64_t)ctx->h_stats.evals * (uint64_t)nc;
  if (ctx->profile) {
    float ms = 0.f;
    SG_CUDA_TRY(cudaEventElapsedTime(&ms, ctx->ev_gs0, ctx->ev_gs1));
    ctx->gs_ms += ms;
  }
  st.iterations = ctx->h_stats.iterations;
  st.succeeded = ctx->h_stats.converged;
  st.error = ctx->h_stats.error;
  st.n_colors = (uint32_t)ctx->h_stats.n_colors;
  // The impulses of this step become the cache of the next (cacheImpulses, :428).
  if (ctx->cfg.cache_mode != SG_CACHE_NONE) {
    std::swap(ctx->key, ctx->prev_key);
    std::swap(ctx->ab, ctx->prev_ab);
    ctx->prev_n = nc;
    ctx->prev_rows = false;
    ctx->prev_color_valid = false;
    const int64_t kcap =
        (int64_t)std::min(ctx->key.bytes / sizeof(unsigned long long), ctx->ab.bytes / (2 * sizeof(double)));
    ctx->ccap = std::min<int64_t>(ctx->ccap, kcap);
  } else {
    ctx->prev_n = 0;
    ctx->prev_rows = false;
    ctx->prev_color_valid = false;
  }
  // Final map: from q0 with the post-impact velocity (:441), or the stabilized map's update.
  if (stab)
    k_rb2d_final_stab<<<blocks_for(3L * nb), kBlock, 0, s>>>(nb, ctx->cfg.dt, ctx->q.as<double>(), v2,
                                                             ctx->q1.as<double>(), ctx->v1.as<double>());
  else
    k_rb2d_umap<<<blocks_for(nb), kBlock, 0, s>>>(nb, ctx->cfg.integrator, ctx->cfg.dt, g[0], g[1],
                                                  ctx->q.as<double>(), v2, ctx->m.as<double>(), minv, Iinv,
                                                  ctx->r.as<double>(), ctx->q1.as<double>(), ctx->v1.as<double>(),
                                                  nullptr, nullptr, nullptr);
  SG_CUDA_TRY(cudaGetLastError());
  ctx->kernel_launches += 1;
  std::swap(ctx->q, ctx->q1);
  std::swap(ctx->v, ctx->v1);
  if (out) *out = st;
  return st.succeeded ? SG_OK : SG_NOT_CONVERGED;
}

}  // namespace sg
