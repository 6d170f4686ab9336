// sphere3d_kernels.cu -- RigidBody3D spheres on sm_103a: split-Hamiltonian map, q1 grid
// broad phase, sphere/plane narrow phase, velocity-dependent contact bases, 3x3 Delassus
// blocks and the coloured block Gauss-Seidel Coulomb solve over 6-dof bodies.
//
// Reference path (breannansmith/scisim), one step of GeometricImpactFrictionMap::flow
// (scisim/ConstrainedMaps/GeometricImpactFrictionMap.cpp:267-442) driven by
// RigidBody3DSim::flow (rigidbody3d/RigidBody3DSim.cpp:557-630):
//   k_splitham        SplitHamMap::flow (rigidbody3d/UnconstrainedMaps/SplitHamMap.cpp:17-182),
//                     gravity NearEarthGravityForce (rigidbody3d/Forces/NearEarthGravityForce.cpp:39-54),
//                     q1 AABBs cm +- r (rigidbody3d/Geometry/RigidBodySphere.cpp:45-49)
//   k_inertia         RigidBody3DState::updateMandMinv (rigidbody3d/RigidBody3DState.cpp:428-462)
//   k_*3 grid         SpatialGridDetector::getPotentialOverlaps (rigidbody3d/SpatialGridDetector.cpp:110-137):
//                     the all-pairs AABB-overlap set, lexicographic (i < j), from a uniform
//                     grid whose cell exceeds every box, scanning 27 cells
//   k_pair_*3         sphereSphereNarrowPhaseCollision (RigidBody3DSim.cpp:793-819): active at q1
//   k_plane_*3        computeBodyPlaneActiveSetAllPairs (RigidBody3DSim.cpp:1414-1452), plane-major
//   k_assemble3       computeContactBasis (SphereSphereConstraint.cpp:273-300,
//                     StaticPlaneSphereConstraint.cpp:255-283, FrictionUtilities.cpp:19-29),
//                     forcing terms (scisim/Constraints/Constraint.cpp:18-34, 92-126),
//                     H rows (SphereSphereConstraint.cpp:229-271, StaticPlaneSphereConstraint.cpp:197-221),
//                     Sobogus initialize3D / solve3D warm start (scisim/ConstrainedMaps/Sobogus.cpp:184-251,
//                     486-518)
//   k_gs3             RigidBodies3DSobogusInterface::solve (scisim/ConstrainedMaps/bogus/
//                     RigidBody3DSobogusInterface.cpp:99-145) with So-bogus's GaussSeidel and
//                     SOCLaw<3>: matrix-free through body velocities (v, omega) = v0 + M^-1 H^T r
//   k_final_vel3      v2 = M^-1 (H^T r - f), f = -M v0
//   k_extract3        alpha, beta (Sobogus.cpp:526-542)
// Every FP64 expression keeps the operation order of the CPU restatement (products of
// fixed-size matrices as sequential sums, no contraction: the library is built with
// -fmad=false), so contact sets and solver iterates are bit-identical to it.  sin and cos
// come from CUDA's math library, so orientations and angular velocities agree with the
// host's to a few ulps rather than bit for bit.
//
// Layout in HBM: q = [x (3nb) | R row-major (9nb)], v = [v (3nb) | omega (3nb)] (SCISim's
// VectorXs layouts), per-body r, m, 1/m, I0 (3), world inertia and inverse (9 each, row
// major); contacts SoA: basis rows (9), angular rows (6 + 6), forcing (3), Delassus
// block (6), mu, impulse (3); running velocities as two double4_32a per body.
#include "ctx.hpp"

#include <algorithm>
#include <cmath>
#include <utility>

namespace sg {
namespace {

constexpr int kBlock = 256;
constexpr int kGs3Block = 256;
inline int blocks_for(long n) { return (int)((n + kBlock - 1) / kBlock); }

struct Grid3 {
  unsigned long long enc_min[3];
  unsigned long long enc_max[3];
  unsigned long long enc_ext[3];
  double origin[3];
  double h;
  int dims[3];
  int ncells;
};

// ---------------------------------------------------------------------------
// Small fixed-size algebra (sequential sums, as the host restatement).
__device__ __forceinline__ double dot3(const double* a, const double* b) {
  return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}
__device__ __forceinline__ void cross3(const double* a, const double* b, double* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
__device__ __forceinline__ void normalize3(double* v) {
  const double z = dot3(v, v);
  if (z > 0.0) {
    const double s = sqrt(z);
    v[0] = v[0] / s;
    v[1] = v[1] / s;
    v[2] = v[2] / s;
  }
}
// y = A x (A row-major); y may alias x.
__device__ __forceinline__ void matvec3(const double* A, const double* x, double* y) {
  const double t0 = (A[0] * x[0] + A[1] * x[1]) + A[2] * x[2];
  const double t1 = (A[3] * x[0] + A[4] * x[1]) + A[5] * x[2];
  const double t2 = (A[6] * x[0] + A[7] * x[1]) + A[8] * x[2];
  y[0] = t0;
  y[1] = t1;
  y[2] = t2;
}
__device__ __forceinline__ void matmul3(const double* A, const double* B, double* C) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) C[3 * i + j] = (A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j]) + A[3 * i + 2] * B[6 + j];
}
// R diag(d) R^T, element (i,j) = sum_k (R_ik d_k) R_jk.
__device__ __forceinline__ void rdrt(const double* R, const double* d, double* out) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      out[3 * i + j] = ((R[3 * i] * d[0]) * R[3 * j] + (R[3 * i + 1] * d[1]) * R[3 * j + 1]) +
                       (R[3 * i + 2] * d[2]) * R[3 * j + 2];
}
// Rotation by `angle` about the unit axis -e_axis (Rodrigues' formula); the axis
// components are 0 or -1, so every product below is exact except 1 - cos.
__device__ __forceinline__ void rot_neg_axis(int axis, double angle, double* R) {
  const double c = cos(angle), s = sin(angle);
  const double a0 = axis == 0 ? -1.0 : 0.0, a1 = axis == 1 ? -1.0 : 0.0, a2 = axis == 2 ? -1.0 : 0.0;
  const double omc = 1.0 - c;
  R[0] = (omc * a0) * a0 + c;
  R[4] = (omc * a1) * a1 + c;
  R[8] = (omc * a2) * a2 + c;
  R[1] = (omc * a0) * a1 - s * a2;
  R[3] = (omc * a0) * a1 + s * a2;
  R[2] = (omc * a0) * a2 + s * a1;
  R[6] = (omc * a0) * a2 - s * a1;
  R[5] = (omc * a1) * a2 - s * a0;
  R[7] = (omc * a1) * a2 + s * a0;
}

// ---------------------------------------------------------------------------
// SplitHamMap::flow for one sphere with the state's world inertia Iw (the reference's
// sparse M); gravity F = m g, no torque.  Optionally writes the q1 AABB.
__global__ void k_splitham(int nb, double dt, double gx, double gy, double gz, const double* __restrict__ q0,
                           const double* __restrict__ v0, const double* __restrict__ m,
                           const double* __restrict__ I0, const double* __restrict__ Iw,
                           const double* __restrict__ rad, double* __restrict__ q1, double* __restrict__ v1,
                           double* __restrict__ aabb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const double h = 0.5 * dt;
  const double hdt = (0.5 * dt) * dt;
  const double mi = m[i];
  const double minv = 1.0 / mi;
  const double g[3] = {gx, gy, gz};
  double p[3], x1[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const double F = mi * g[j];
    p[j] = mi * v0[3 * i + j];
    p[j] = p[j] + h * F;
    x1[j] = q0[3 * i + j] + (dt * v0[3 * i + j] + (hdt * minv) * F);
  }
  double Iwi[9], w0[3], L[3];
#pragma unroll
  for (int j = 0; j < 9; ++j) Iwi[j] = Iw[9 * (size_t)i + j];
#pragma unroll
  for (int j = 0; j < 3; ++j) w0[j] = v0[3 * (size_t)nb + 3 * i + j];
  matvec3(Iwi, w0, L);
#pragma unroll
  for (int j = 0; j < 3; ++j) L[j] = L[j] + h * 0.0;
  const double I[3] = {I0[3 * i], I0[3 * i + 1], I0[3 * i + 2]};
  double Rc[9];
#pragma unroll
  for (int j = 0; j < 9; ++j) Rc[j] = q0[3 * (size_t)nb + 9 * (size_t)i + j];
  double pB[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) pB[k] = (Rc[k] * L[0] + Rc[3 + k] * L[1]) + Rc[6 + k] * L[2];
  const int axes[5] = {2, 1, 0, 1, 2};
#pragma unroll
  for (int st = 0; st < 5; ++st) {
    const int ax = axes[st];
    const double ang = st == 2 ? (dt * pB[ax]) / I[ax] : (h * pB[ax]) / I[ax];
    double Ri[9], Rf[9], tmp[9];
    rot_neg_axis(ax, -ang, Ri);
    matmul3(Rc, Ri, tmp);
#pragma unroll
    for (int j = 0; j < 9; ++j) Rc[j] = tmp[j];
    rot_neg_axis(ax, ang, Rf);
    matvec3(Rf, pB, pB);
  }
#pragma unroll
  for (int j = 0; j < 9; ++j) q1[3 * (size_t)nb + 9 * (size_t)i + j] = Rc[j];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const double F = mi * g[j];
    p[j] = p[j] + h * F;
    L[j] = L[j] + h * 0.0;
    q1[3 * i + j] = x1[j];
    v1[3 * i + j] = p[j] / mi;
  }
  const double di[3] = {1.0 / I[0], 1.0 / I[1], 1.0 / I[2]};
  double Wm[9], w1[3];
  rdrt(Rc, di, Wm);
  matvec3(Wm, L, w1);
#pragma unroll
  for (int j = 0; j < 3; ++j) v1[3 * (size_t)nb + 3 * i + j] = w1[j];
  if (aabb) {
    const double r = rad[i];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      aabb[6 * (size_t)i + j] = x1[j] - r;
      aabb[6 * (size_t)i + 3 + j] = x1[j] + r;
    }
  }
}

// IntegrationTools::exponentialEuler (rigidbody3d/UnconstrainedMaps/IntegrationTools.cpp:3-47) for
// body i: x1 = x0 + dt v; R1 = rot(omega / |omega|, |omega| dt) R0, the rotation by the Rodrigues
// formula (Eigen's AngleAxis::toRotationMatrix).  sin and cos are CUDA's.
__device__ __forceinline__ void exp_euler_body(int nb, int i, double dt, const double* __restrict__ q0,
                                               const double* v, const double* w, double* __restrict__ q1) {
#pragma unroll
  for (int j = 0; j < 3; ++j) q1[3 * i + j] = q0[3 * i + j] + dt * v[j];
  double ax[3] = {w[0], w[1], w[2]};
  double theta = sqrt(dot3(ax, ax));
  if (theta != 0.0)
#pragma unroll
    for (int j = 0; j < 3; ++j) ax[j] = ax[j] / theta;
  theta = theta * dt;
  const double sn = sin(theta), c = cos(theta);
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
  double R0[9], R1[9];
#pragma unroll
  for (int j = 0; j < 9; ++j) R0[j] = q0[3 * (size_t)nb + 9 * (size_t)i + j];
  matmul3(R, R0, R1);
#pragma unroll
  for (int j = 0; j < 9; ++j) q1[3 * (size_t)nb + 9 * (size_t)i + j] = R1[j];
}

// SymplecticEulerImpactFrictionMap::flow, first half (SymplecticEulerImpactFrictionMap.cpp:201-260):
// vdelta = dt M^-1 F (gravity, no torque), the predictor by exponential Euler from v0 + vdelta and
// its AABBs (centre +- r).
__global__ void k_se3_predict(int nb, double dt, double gx, double gy, double gz, const double* __restrict__ q0,
                              const double* __restrict__ v0, const double* __restrict__ m,
                              const double* __restrict__ Iinv, const double* __restrict__ rad,
                              double* __restrict__ vdelta, double* __restrict__ q1, double* __restrict__ aabb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const double g[3] = {gx, gy, gz};
  const double mi = m[i];
  const double minv = 1.0 / mi;
  double vp[3], wp[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const double F = 0.0 + mi * g[j];
    const double* Ii = Iinv + 9 * (size_t)i + 3 * j;
    const double dl = dt * (0.0 + minv * F);
    const double da = dt * (((0.0 + Ii[0] * 0.0) + Ii[1] * 0.0) + Ii[2] * 0.0);
    vdelta[3 * (size_t)i + j] = dl;
    vdelta[3 * (size_t)nb + 3 * (size_t)i + j] = da;
    vp[j] = v0[3 * (size_t)i + j] + dl;
    wp[j] = v0[3 * (size_t)nb + 3 * (size_t)i + j] + da;
  }
  exp_euler_body(nb, i, dt, q0, vp, wp, q1);
  const double r = rad[i];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    aabb[6 * (size_t)i + j] = q1[3 * i + j] - r;
    aabb[6 * (size_t)i + 3 + j] = q1[3 * i + j] + r;
  }
}

// The map's end (:330-407): v1 = v2 + vdelta, the configuration by exponential Euler from v1 (with
// v2 = v0 where no constraint is active).
__global__ void k_se3_final(int nb, double dt, const double* __restrict__ q0, const double* __restrict__ v2,
                            const double* __restrict__ vdelta, double* __restrict__ q1, double* __restrict__ v1) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  double vl[3], wl[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    vl[j] = v2[3 * (size_t)i + j] + vdelta[3 * (size_t)i + j];
    wl[j] = v2[3 * (size_t)nb + 3 * (size_t)i + j] + vdelta[3 * (size_t)nb + 3 * (size_t)i + j];
    v1[3 * (size_t)i + j] = vl[j];
    v1[3 * (size_t)nb + 3 * (size_t)i + j] = wl[j];
  }
  exp_euler_body(nb, i, dt, q0, vl, wl, q1);
}

// World inertia and its inverse from R (updateMandMinv).  At construction the
// reference inserts I(row, col) at sparse entry (col, row) (RigidBody3DState.cpp:175-182).
__global__ void k_inertia(int nb, const double* __restrict__ q, const double* __restrict__ I0,
                          double* __restrict__ Iw, double* __restrict__ Iinv, int construction) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  double R[9];
#pragma unroll
  for (int j = 0; j < 9; ++j) R[j] = q[3 * (size_t)nb + 9 * (size_t)i + j];
  const double d[3] = {I0[3 * i], I0[3 * i + 1], I0[3 * i + 2]};
  const double di[3] = {1.0 / d[0], 1.0 / d[1], 1.0 / d[2]};
  double A[9], B[9];
  rdrt(R, d, A);
  rdrt(R, di, B);
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int src = construction ? 3 * c + r : 3 * r + c;
      Iw[9 * (size_t)i + 3 * r + c] = A[src];
      Iinv[9 * (size_t)i + 3 * r + c] = B[src];
    }
}

// ---------------------------------------------------------------------------
// Broad phase on a uniform 3D grid.
__global__ void k_bounds3_init(Grid3* g) {
  for (int a = 0; a < 3; ++a) {
    g->enc_min[a] = ~0ull;
    g->enc_max[a] = 0ull;
    g->enc_ext[a] = 0ull;
  }
}

__global__ void k_bounds3(int n, const double* __restrict__ aabb, Grid3* g) {
  double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY}, ex[3] = {0.0, 0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const double lo = aabb[6 * (size_t)i + a], hi = aabb[6 * (size_t)i + 3 + a];
      mn[a] = fmin(mn[a], lo);
      mx[a] = fmax(mx[a], hi);
      ex[a] = fmax(ex[a], hi - lo);
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a)
    for (int o = 16; o > 0; o >>= 1) {
      mn[a] = fmin(mn[a], __shfl_down_sync(0xffffffffu, mn[a], o));
      mx[a] = fmax(mx[a], __shfl_down_sync(0xffffffffu, mx[a], o));
      ex[a] = fmax(ex[a], __shfl_down_sync(0xffffffffu, ex[a], o));
    }
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      atomicMin(&g->enc_min[a], f64_to_ordered(mn[a]));
      atomicMax(&g->enc_max[a], f64_to_ordered(mx[a]));
      atomicMax(&g->enc_ext[a], f64_to_ordered(ex[a]));
    }
  }
}

// Cell width strictly above the largest box extent: two overlapping boxes have min
// corners in the same or adjacent cells, so 27 cells suffice.  The cell count is capped
// at `cap` (h grows; larger cells stay correct).
__global__ void k_grid3_setup(Grid3* g, long cap) {
  double mn[3], span[3];
  double e = 0.0;
  for (int a = 0; a < 3; ++a) {
    mn[a] = ordered_to_f64(g->enc_min[a]);
    span[a] = ordered_to_f64(g->enc_max[a]) - mn[a];
    if (!isfinite(span[a]) || span[a] < 0.0) span[a] = 0.0;
    e = fmax(e, ordered_to_f64(g->enc_ext[a]));
  }
  double h = e * (1.0 + 0x1p-20) + 1e-300;
  if (!(h > 0.0) || !isfinite(h)) h = 1.0;
  double d[3];
  for (int a = 0; a < 3; ++a) d[a] = floor(span[a] / h) + 1.0;
  while (d[0] * d[1] * d[2] > (double)cap) {
    h = h * fmax(1.01, cbrt(d[0] * d[1] * d[2] / (double)cap));
    for (int a = 0; a < 3; ++a) d[a] = floor(span[a] / h) + 1.0;
  }
  for (int a = 0; a < 3; ++a) {
    g->origin[a] = isfinite(mn[a]) ? mn[a] : 0.0;
    g->dims[a] = (int)d[a];
  }
  g->h = h;
  g->ncells = (int)(d[0] * d[1] * d[2]);
}

__device__ __forceinline__ int cell_coord3(double x, double o, double h, int dim) {
  const double f = (x - o) / h;
  const int c = (f > 0.0) ? (int)f : 0;  // NaN -> 0
  return c < dim ? c : dim - 1;
}

__global__ void k_cell_count3(int n, const double* __restrict__ aabb, const Grid3* __restrict__ g,
                              int* __restrict__ cell_of, int* __restrict__ cell_count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int cx = cell_coord3(aabb[6 * (size_t)i], g->origin[0], g->h, g->dims[0]);
  const int cy = cell_coord3(aabb[6 * (size_t)i + 1], g->origin[1], g->h, g->dims[1]);
  const int cz = cell_coord3(aabb[6 * (size_t)i + 2], g->origin[2], g->h, g->dims[2]);
  const int cell = cx + g->dims[0] * (cy + g->dims[1] * cz);
  cell_of[i] = cell;
  atomicAdd(&cell_count[cell], 1);
}

__global__ void k_cell_scatter3(int n, const int* __restrict__ cell_of, const int* __restrict__ cell_start,
                                int* __restrict__ cell_fill, int* __restrict__ sorted) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int cell = cell_of[i];
  sorted[cell_start[cell] + atomicAdd(&cell_fill[cell], 1)] = i;
}

struct Scan3 {
  const double* aabb;
  const Grid3* g;         // one grid, or one per scene (batches)
  const int* cell_start;
  const int* sorted;
  const double* x1;   // q1 positions (3 per body)
  const double* rad;
  const int* scene_of;    // batches: scene of each body (null for one scene)
  const int* cell_off;    // batches: first cell of each scene's grid
};

// AABB::overlaps (rigidbody3d/SpatialGridDetector.cpp:8-25) then SphereSphereConstraint::isActive
// at q1 (SphereSphereConstraint.cpp:9-12), for every j > i found in the 27 cells around the
// cell of box i's min corner.
template <typename F>
__device__ __forceinline__ void visit_pairs3(const Scan3& s, int i, F&& f) {
  double bi[6];
#pragma unroll
  for (int a = 0; a < 6; ++a) bi[a] = s.aabb[6 * (size_t)i + a];
  const int sc = s.scene_of ? s.scene_of[i] : 0;
  const Grid3& g = s.g[sc];
  const int coff = s.cell_off ? s.cell_off[sc] : 0;
  const int cx = cell_coord3(bi[0], g.origin[0], g.h, g.dims[0]);
  const int cy = cell_coord3(bi[1], g.origin[1], g.h, g.dims[1]);
  const int cz = cell_coord3(bi[2], g.origin[2], g.h, g.dims[2]);
  const double xi[3] = {s.x1[3 * (size_t)i], s.x1[3 * (size_t)i + 1], s.x1[3 * (size_t)i + 2]};
  const double ri = s.rad[i];
  for (int z = max(cz - 1, 0); z <= min(cz + 1, g.dims[2] - 1); ++z)
    for (int y = max(cy - 1, 0); y <= min(cy + 1, g.dims[1] - 1); ++y)
      for (int x = max(cx - 1, 0); x <= min(cx + 1, g.dims[0] - 1); ++x) {
        const int cell = coff + x + g.dims[0] * (y + g.dims[1] * z);
        const int e = s.cell_start[cell + 1];
        for (int p = s.cell_start[cell]; p < e; ++p) {
          const int j = s.sorted[p];
          if (j <= i) continue;
          const double* bj = s.aabb + 6 * (size_t)j;
          if (bi[3] < bj[0] || bi[4] < bj[1] || bi[5] < bj[2]) continue;
          if (bj[3] < bi[0] || bj[4] < bi[1] || bj[5] < bi[2]) continue;
          const double d[3] = {xi[0] - s.x1[3 * (size_t)j], xi[1] - s.x1[3 * (size_t)j + 1],
                               xi[2] - s.x1[3 * (size_t)j + 2]};
          const double rs = ri + s.rad[j];
          if (!(dot3(d, d) <= rs * rs)) continue;
          f(j);
        }
      }
}

__global__ void k_pair_count3(int n, Scan3 s, int* __restrict__ cnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c = 0;
  visit_pairs3(s, i, [&](int) { ++c; });
  cnt[i] = c;
}

__global__ void k_pair_write3(int n, Scan3 s, const int* __restrict__ off, int* __restrict__ out_a,
                              int* __restrict__ out_b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int base = off[i];
  int c = 0;
  visit_pairs3(s, i, [&](int j) {
    int p = base + c;
    while (p > base && out_b[p - 1] > j) {
      out_b[p] = out_b[p - 1];
      --p;
    }
    out_b[p] = j;
    ++c;
  });
  for (int k = 0; k < c; ++k) out_a[base + k] = i;
}

// StaticPlaneSphereConstraint::isActive at q1 (StaticPlaneSphereConstraint.cpp:13-17), plane-major.
__global__ void k_plane_flags3(int nb, int np, const double* __restrict__ x1, const double* __restrict__ rad,
                               const double* __restrict__ px, const double* __restrict__ pn, int* __restrict__ flag) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)nb * np) return;
  const int p = (int)(t / nb), i = (int)(t - (long)p * nb);
  const double d[3] = {x1[3 * (size_t)i] - px[3 * p], x1[3 * (size_t)i + 1] - px[3 * p + 1],
                       x1[3 * (size_t)i + 2] - px[3 * p + 2]};
  const double n[3] = {pn[3 * p], pn[3 * p + 1], pn[3 * p + 2]};
  flag[t] = (dot3(n, d) <= rad[i]) ? 1 : 0;
}

__global__ void k_plane_write3(int nb, int np, int npairs, const int* __restrict__ flag, const int* __restrict__ off,
                               int* __restrict__ ia, int* __restrict__ ib) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)nb * np) return;
  if (!flag[t]) return;
  const int p = (int)(t / nb), i = (int)(t - (long)p * nb);
  const int k = npairs + off[t];
  ia[k] = i;
  ib[k] = -1 - p;
}

// ---------------------------------------------------------------------------
// Batched sphere scenes: scene s owns bodies [sb_off[s], sb_off[s+1]), planes
// [sp_off[s], sp_off[s+1]) and plane flags [sf_off[s], sf_off[s+1]) (plane-major, n_s per
// plane); its contacts are [sc_off[s], sc_off[s+1]): its pairs in the order above, then its
// plane contacts plane-major, as the scene alone would order them.

__global__ void k_fill_int(int n, int v, int* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = v;
}

// One grid per scene (one block per scene), as k_bounds3 + k_grid3_setup do for one scene.
__global__ void k_scene_grid3(const int* __restrict__ sb_off, const double* __restrict__ aabb,
                              Grid3* __restrict__ grids, int* __restrict__ s_cells) {
  const int sc = blockIdx.x;
  const int b0 = sb_off[sc], b1 = sb_off[sc + 1];
  double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY}, e = 0.0;
  for (int i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const double lo = aabb[6 * (size_t)i + a], hi = aabb[6 * (size_t)i + 3 + a];
      mn[a] = fmin(mn[a], lo);
      mx[a] = fmax(mx[a], hi);
      e = fmax(e, hi - lo);
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a)
    for (int o = 16; o > 0; o >>= 1) {
      mn[a] = fmin(mn[a], __shfl_down_sync(0xffffffffu, mn[a], o));
      mx[a] = fmax(mx[a], __shfl_down_sync(0xffffffffu, mx[a], o));
    }
  for (int o = 16; o > 0; o >>= 1) e = fmax(e, __shfl_down_sync(0xffffffffu, e, o));
  __shared__ double red[7][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    for (int a = 0; a < 3; ++a) {
      red[a][wid] = mn[a];
      red[3 + a][wid] = mx[a];
    }
    red[6][wid] = e;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  const int nw = (blockDim.x + 31) >> 5;
  for (int w = 1; w < nw; ++w) {
    for (int a = 0; a < 3; ++a) {
      mn[a] = fmin(mn[a], red[a][w]);
      mx[a] = fmax(mx[a], red[3 + a][w]);
    }
    e = fmax(e, red[6][w]);
  }
  const long cap = 4L * (b1 - b0) + 64;
  double h = e * (1.0 + 0x1p-20) + 1e-300;
  if (!(h > 0.0) || !isfinite(h)) h = 1.0;
  double span[3], d[3];
  for (int a = 0; a < 3; ++a) {
    span[a] = mx[a] - mn[a];
    if (!isfinite(span[a]) || span[a] < 0.0) span[a] = 0.0;
    d[a] = floor(span[a] / h) + 1.0;
  }
  while (d[0] * d[1] * d[2] > (double)cap) {
    h = h * fmax(1.01, cbrt(d[0] * d[1] * d[2] / (double)cap));
    for (int a = 0; a < 3; ++a) d[a] = floor(span[a] / h) + 1.0;
  }
  Grid3& g = grids[sc];
  for (int a = 0; a < 3; ++a) {
    g.origin[a] = isfinite(mn[a]) ? mn[a] : 0.0;
    g.dims[a] = (int)d[a];
  }
  g.h = h;
  g.ncells = (int)(d[0] * d[1] * d[2]);
  s_cells[sc] = g.ncells;
}

__global__ void k_cell_count3_b(int n, const int* __restrict__ scene_of, const double* __restrict__ aabb,
                                const Grid3* __restrict__ grids, const int* __restrict__ cell_off,
                                int* __restrict__ cell_of, int* __restrict__ cell_count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int sc = scene_of[i];
  const Grid3& g = grids[sc];
  const int cx = cell_coord3(aabb[6 * (size_t)i], g.origin[0], g.h, g.dims[0]);
  const int cy = cell_coord3(aabb[6 * (size_t)i + 1], g.origin[1], g.h, g.dims[1]);
  const int cz = cell_coord3(aabb[6 * (size_t)i + 2], g.origin[2], g.h, g.dims[2]);
  const int cell = cell_off[sc] + cx + g.dims[0] * (cy + g.dims[1] * cz);
  cell_of[i] = cell;
  atomicAdd(&cell_count[cell], 1);
}

// Pairs of body i into its scene's contact slots (sorted by partner, as k_pair_write3).
__global__ void k_pair_write3_b(int n, Scan3 s, const int* __restrict__ sb_off, const int* __restrict__ off,
                                const int* __restrict__ sc_off, int* __restrict__ out_a, int* __restrict__ out_b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int sc = s.scene_of[i];
  const int base = sc_off[sc] + (off[i] - off[sb_off[sc]]);
  int c = 0;
  visit_pairs3(s, i, [&](int j) {
    int p = base + c;
    while (p > base && out_b[p - 1] > j) {
      out_b[p] = out_b[p - 1];
      --p;
    }
    out_b[p] = j;
    ++c;
  });
  for (int k = 0; k < c; ++k) out_a[base + k] = i;
}

// Plane tests of body i against its scene's planes (flag index sf_off[s] + p_local n_s + i_local).
__global__ void k_plane_flags3_b(int n, const int* __restrict__ scene_of, const int* __restrict__ sb_off,
                                 const int* __restrict__ sp_off, const int* __restrict__ sf_off,
                                 const double* __restrict__ x1, const double* __restrict__ rad,
                                 const double* __restrict__ px, const double* __restrict__ pn, int* __restrict__ flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int sc = scene_of[i], b0 = sb_off[sc], ns = sb_off[sc + 1] - b0;
  const double xi[3] = {x1[3 * (size_t)i], x1[3 * (size_t)i + 1], x1[3 * (size_t)i + 2]};
  for (int p = sp_off[sc]; p < sp_off[sc + 1]; ++p) {
    const double d[3] = {xi[0] - px[3 * p], xi[1] - px[3 * p + 1], xi[2] - px[3 * p + 2]};
    const double nn[3] = {pn[3 * p], pn[3 * p + 1], pn[3 * p + 2]};
    flag[sf_off[sc] + (long)(p - sp_off[sc]) * ns + (i - b0)] = (dot3(nn, d) <= rad[i]) ? 1 : 0;
  }
}

__global__ void k_plane_write3_b(int n, const int* __restrict__ scene_of, const int* __restrict__ sb_off,
                                 const int* __restrict__ sp_off, const int* __restrict__ sf_off,
                                 const int* __restrict__ flag, const int* __restrict__ off,
                                 const int* __restrict__ sc_off, const int* __restrict__ s_npairs,
                                 int* __restrict__ ia, int* __restrict__ ib) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int sc = scene_of[i], b0 = sb_off[sc], ns = sb_off[sc + 1] - b0;
  const int base = sc_off[sc] + s_npairs[sc] - off[sf_off[sc]];
  for (int p = sp_off[sc]; p < sp_off[sc + 1]; ++p) {
    const long t = sf_off[sc] + (long)(p - sp_off[sc]) * ns + (i - b0);
    if (!flag[t]) continue;
    const int k = base + off[t];
    ia[k] = i;
    ib[k] = -1 - p;
  }
}

// Contacts per scene: pairs of its bodies plus its plane contacts.
__global__ void k_scene_counts3(int S, const int* __restrict__ sb_off, const int* __restrict__ sf_off,
                                const int* __restrict__ pair_off, const int* __restrict__ plane_off,
                                int* __restrict__ s_nc, int* __restrict__ s_npairs) {
  const int sc = blockIdx.x * blockDim.x + threadIdx.x;
  if (sc >= S) return;
  const int np = pair_off[sb_off[sc + 1]] - pair_off[sb_off[sc]];
  s_npairs[sc] = np;
  s_nc[sc] = np + (plane_off[sf_off[sc + 1]] - plane_off[sf_off[sc]]);
}

// ---------------------------------------------------------------------------
// Contact assembly.
struct Assemble3 {
  int nb, nc;
  const int* ia;
  const int* ib;
  const double* q0;
  const double* v0;
  const double* rad;
  const double* minv;
  const double* Iinv;
  const double* plane_n;
  double mu, CoR;
  const int* scene_of;   // batches: scene of each body, and each scene's mu and CoR (null: mu, CoR)
  const double* s_mu;
  const double* s_CoR;
  double* E;    // 9 per contact: n, s, t
  double* Aa;   // 6: r_a x s, r_a x t
  double* Ab;   // 6: r_b x s, r_b x t
  double* c;    // 3
  double* W;    // 6: w00 w01 w02 w11 w12 w22
  double* mu_out;
  double* r;    // 3
  // SymplecticEulerImpactFrictionMap (vdelta non-null): the force's velocity change, the pose
  // stabilisation, and the impulse cache of the step before (keys ascending, 6 doubles each: the
  // cached normal and force); this step's keys go to key.
  const double* vdelta = nullptr;   // 6 nb [linear | angular]
  const double* plane_x = nullptr;
  double dt = 0.0;
  int stabilize = 0;
  double pen_thresh = 0.0;
  int cache_mode = 0;
  const unsigned long long* prev_key = nullptr;
  const double* prev_c6 = nullptr;
  int prev_n = 0;
  unsigned long long* key = nullptr;
};

// Impulse-cache key of a sphere contact: (a, b) for a pair, (plane, a) flagged by the top bit for a
// plane; contacts are written pairs first (a, then b ascending), then plane-major, so a step's keys
// ascend.
__device__ __forceinline__ unsigned long long contact_key3(int a, int b) {
  if (b >= 0) return ((unsigned long long)(unsigned)a << 32) | (unsigned)b;
  return (1ull << 63) | ((unsigned long long)(unsigned)(-1 - b) << 32) | (unsigned)a;
}

__device__ __forceinline__ int find_key3(const unsigned long long* keys, int n, unsigned long long k) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (keys[mid] < k)
      lo = mid + 1;
    else
      hi = mid;
  }
  return (lo < n && keys[lo] == k) ? lo : -1;
}

__device__ void orthogonal_vector(const double* n, double* o) {
  const double ax = fabs(n[0]), ay = fabs(n[1]), az = fabs(n[2]);
  o[0] = o[1] = o[2] = 0.0;
  if (ax <= ay && ax <= az)
    o[0] = 1.0;
  else if (ay <= az)
    o[1] = 1.0;
  else
    o[2] = 1.0;
  const double d = dot3(n, o);
#pragma unroll
  for (int j = 0; j < 3; ++j) o[j] = o[j] - d * n[j];
  normalize3(o);
}

// Quaternion (w, x, y, z) turning direction a onto direction b (Eigen's
// Quaternion::setFromTwoVectors, half-angle form; directions within 1e-12 of opposite turn by pi
// about an axis orthogonal to a).
__device__ void quat_from_two_vectors(const double* a, const double* b, double* q) {
  double v0[3] = {a[0], a[1], a[2]}, v1[3] = {b[0], b[1], b[2]};
  normalize3(v0);
  normalize3(v1);
  const double c = dot3(v1, v0);
  if (c < -1.0 + 1e-12) {
    double axis[3];
    orthogonal_vector(v0, axis);
    normalize3(axis);
    const double w2 = (1.0 + fmax(c, -1.0)) * 0.5;
    const double sv = sqrt(1.0 - w2);
    q[0] = sqrt(w2);
#pragma unroll
    for (int j = 0; j < 3; ++j) q[1 + j] = axis[j] * sv;
    return;
  }
  double axis[3];
  cross3(v0, v1, axis);
  const double s2 = sqrt((1.0 + c) * 2.0);
  const double invs = 1.0 / s2;
#pragma unroll
  for (int j = 0; j < 3; ++j) q[1 + j] = axis[j] * invs;
  q[0] = s2 * 0.5;
}

// q v q* for a unit quaternion: uv = 2 (q_v x v), v + w uv + q_v x uv.
__device__ __forceinline__ void quat_rotate(const double* q, const double* v, double* out) {
  double uv[3], uuv[3];
  cross3(q + 1, v, uv);
#pragma unroll
  for (int j = 0; j < 3; ++j) uv[j] = uv[j] + uv[j];
  cross3(q + 1, uv, uuv);
#pragma unroll
  for (int j = 0; j < 3; ++j) out[j] = (v[j] + q[0] * uv[j]) + uuv[j];
}

__global__ void k_assemble3(Assemble3 A) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= A.nc) return;
  const int nb = A.nb;
  const int a = A.ia[k], b = A.ib[k];
  const bool has_b = b >= 0;
  double n[3], ra[3], rb[3] = {0.0, 0.0, 0.0}, sv[3], vr[3];
  const double* xa = A.q0 + 3 * (size_t)a;
  const double* va = A.v0 + 3 * (size_t)a;
  const double* wa = A.v0 + 3 * (size_t)nb + 3 * (size_t)a;
  if (has_b) {
    const double* xb = A.q0 + 3 * (size_t)b;
    const double* vb = A.v0 + 3 * (size_t)b;
    const double* wb = A.v0 + 3 * (size_t)nb + 3 * (size_t)b;
#pragma unroll
    for (int j = 0; j < 3; ++j) n[j] = xa[j] - xb[j];
    normalize3(n);
    const double frac = A.rad[a] / (A.rad[a] + A.rad[b]);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const double p = xa[j] + frac * (xb[j] - xa[j]);
      ra[j] = p - xa[j];
      rb[j] = p - xb[j];
    }
    double ca[3], cb[3];
    const double wa_[3] = {wa[0], wa[1], wa[2]}, wb_[3] = {wb[0], wb[1], wb[2]};
    cross3(wa_, ra, ca);
    cross3(wb_, rb, cb);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      sv[j] = ((va[j] + ca[j]) - vb[j]) - cb[j];
      vr[j] = va[j] - vb[j];
    }
  } else {
    const int pl = -1 - b;
#pragma unroll
    for (int j = 0; j < 3; ++j) n[j] = A.plane_n[3 * pl + j];
    const double nr = -A.rad[a];
#pragma unroll
    for (int j = 0; j < 3; ++j) ra[j] = nr * n[j];
    double ca[3];
    const double wa_[3] = {wa[0], wa[1], wa[2]};
    cross3(wa_, ra, ca);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      sv[j] = (va[j] + ca[j]) - 0.0;
      vr[j] = va[j] - 0.0;
    }
  }
  // Basis [n s t]: s opposes the tangential relative velocity, t = n x s.
  double s[3] = {sv[0], sv[1], sv[2]}, t[3], tmp[3];
  cross3(n, s, tmp);
  if (dot3(tmp, tmp) < 1.0e-9) {
    orthogonal_vector(n, s);
  } else {
    const double d = dot3(s, n);
#pragma unroll
    for (int j = 0; j < 3; ++j) s[j] = s[j] - d * n[j];
    normalize3(s);
  }
#pragma unroll
  for (int j = 0; j < 3; ++j) s[j] = s[j] * -1.0;
  cross3(n, s, t);
  normalize3(t);
  double* E = A.E + 9 * (size_t)k;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    E[j] = n[j];
    E[3 + j] = s[j];
    E[6 + j] = t[j];
  }
  double as[3], at[3], bs[3] = {0.0, 0.0, 0.0}, bt[3] = {0.0, 0.0, 0.0};
  cross3(ra, s, as);
  cross3(ra, t, at);
  if (has_b) {
    cross3(rb, s, bs);
    cross3(rb, t, bt);
  }
  double* Aa = A.Aa + 6 * (size_t)k;
  double* Ab = A.Ab + 6 * (size_t)k;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    Aa[j] = as[j];
    Aa[3 + j] = at[j];
    Ab[j] = bs[j];
    Ab[3 + j] = bt[j];
  }
  // Forcing term w = n (CoR n.v + nrel) + s drel0 + t drel1 (kinematic velocities are zero).
  const double ndotv = dot3(n, vr);
  const double zero[3] = {0.0, 0.0, 0.0};
  double nrel = -dot3(zero, n);
  double drel0 = -dot3(zero, s), drel1 = -dot3(zero, t);
  if (A.vdelta) {
    // SymplecticEulerImpactFrictionMap.cpp:291-329: nrel += N^T vdelta (+ min(0, gap) / dt when
    // stabilising), drel += D^T vdelta, each column's entries in row order (linear rows of a, of b,
    // then angular rows of a, of b) accumulated from zero.
    const double* la = A.vdelta + 3 * (size_t)a;
    const double* wda = A.vdelta + 3 * (size_t)nb + 3 * (size_t)a;
    const double* lb = has_b ? A.vdelta + 3 * (size_t)b : nullptr;
    const double* wdb = has_b ? A.vdelta + 3 * (size_t)nb + 3 * (size_t)b : nullptr;
    double tn = 0.0;
#pragma unroll
    for (int j = 0; j < 3; ++j) tn = tn + n[j] * la[j];
    if (has_b)
#pragma unroll
      for (int j = 0; j < 3; ++j) tn = tn + (-n[j]) * lb[j];
    double xn = 0.0 + 1.0 * tn;
    double xd[2];
#pragma unroll
    for (int d = 0; d < 2; ++d) {
      const double* T = d == 0 ? s : t;
      double xt[3];
      cross3(ra, T, xt);
      double tt = 0.0;
#pragma unroll
      for (int j = 0; j < 3; ++j) tt = tt + T[j] * la[j];
      if (has_b)
#pragma unroll
        for (int j = 0; j < 3; ++j) tt = tt + (-T[j]) * lb[j];
#pragma unroll
      for (int j = 0; j < 3; ++j) tt = tt + xt[j] * wda[j];
      if (has_b) {
        double xb[3];
        cross3(rb, T, xb);
#pragma unroll
        for (int j = 0; j < 3; ++j) tt = tt + (-xb[j]) * wdb[j];
      }
      xd[d] = 0.0 + 1.0 * tt;
    }
    if (A.stabilize) {
      double gap;
      if (has_b) {
        // SphereSphereConstraint::evaluateGapFunction (SphereSphereConstraint.cpp:28-31)
        const double* xb = A.q0 + 3 * (size_t)b;
        const double dd[3] = {xa[0] - xb[0], xa[1] - xb[1], xa[2] - xb[2]};
        gap = (sqrt(dot3(dd, dd)) - A.rad[a]) - A.rad[b];
      } else {
        // StaticPlaneSphereConstraint::evaluateGapFunction (StaticPlaneSphereConstraint.cpp:31-35)
        const int pl = -1 - b;
        const double dd[3] = {xa[0] - A.plane_x[3 * pl], xa[1] - A.plane_x[3 * pl + 1], xa[2] - A.plane_x[3 * pl + 2]};
        gap = dot3(A.plane_n + 3 * pl, dd) - A.rad[a];
      }
      double g0 = fmin(0.0, gap);
      if (fabs(g0) < A.pen_thresh) g0 = 0.0;
      xn = xn + g0 / A.dt;
    }
    nrel = nrel + xn;
    drel0 = drel0 + xd[0];
    drel1 = drel1 + xd[1];
  }
  const int scene = A.scene_of ? A.scene_of[a] : -1;
  const double CoR = scene >= 0 ? A.s_CoR[scene] : A.CoR;
  const double sc = CoR * ndotv + nrel;
  double w[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) w[j] = ((0.0 + n[j] * sc) + s[j] * drel0) + t[j] * drel1;
  A.c[3 * (size_t)k] = dot3(n, w);
  A.c[3 * (size_t)k + 1] = dot3(s, w);
  A.c[3 * (size_t)k + 2] = dot3(t, w);
  // Delassus block W = H_a M_a^-1 H_a^T + H_b M_b^-1 H_b^T; the normal row has no angular part.
  const double* B[3] = {n, s, t};
  const double* AaR[3] = {nullptr, as, at};
  const double* AbR[3] = {nullptr, bs, bt};
  double Ia[9], Ib[9];
#pragma unroll
  for (int j = 0; j < 9; ++j) Ia[j] = A.Iinv[9 * (size_t)a + j];
  if (has_b) {
#pragma unroll
    for (int j = 0; j < 9; ++j) Ib[j] = A.Iinv[9 * (size_t)b + j];
  }
  const double ma = A.minv[a], mb = has_b ? A.minv[b] : 0.0;
  double* Wk = A.W + 6 * (size_t)k;
  int q = 0;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = i; j < 3; ++j) {
      double wij = ma * dot3(B[i], B[j]);
      if (i > 0) {
        double x[3];
        matvec3(Ia, AaR[j], x);
        wij = wij + dot3(AaR[i], x);
      }
      if (has_b) {
        double wb = mb * dot3(B[i], B[j]);
        if (i > 0) {
          double x[3];
          matvec3(Ib, AbR[j], x);
          wb = wb + dot3(AbR[i], x);
        }
        wij = wij + wb;
      }
      Wk[q++] = wij;
    }
  A.mu_out[k] = scene >= 0 ? A.s_mu[scene] : A.mu;
  // Warm start: r = alpha n + beta0 s + beta1 t, then local r = E^T r.  The geometric map starts
  // from zero (no 3D impulse cache); the symplectic-Euler map from its cache, the cached force
  // turned from the cached normal onto the new one (SymplecticEulerImpactFrictionMap.cpp:48-131;
  // a missing entry reads as zeros).
  double al = 0.0, b0 = 0.0, b1 = 0.0;
  if (A.vdelta) {
    const unsigned long long key = contact_key3(a, b);
    A.key[k] = key;
    const int p = (A.cache_mode != SG_CACHE_NONE && A.prev_n > 0) ? find_key3(A.prev_key, A.prev_n, key) : -1;
    if (p >= 0) {
      double c6[6];
#pragma unroll
      for (int j = 0; j < 6; ++j) c6[j] = A.prev_c6[6 * (size_t)p + j];
      if (A.cache_mode == SG_CACHE_NORMAL) {
        al = c6[0];
      } else if (c6[0] != 0.0 || c6[1] != 0.0 || c6[2] != 0.0 || c6[3] != 0.0 || c6[4] != 0.0 || c6[5] != 0.0) {
        double qr[4], f[3];
        quat_from_two_vectors(c6, n, qr);
        quat_rotate(qr, c6 + 3, f);
        al = dot3(f, n);
        b0 = dot3(f, s);
        b1 = dot3(f, t);
      }
    }
  }
  double rw[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) rw[j] = (al * n[j] + b0 * s[j]) + b1 * t[j];
  A.r[3 * (size_t)k] = dot3(n, rw);
  A.r[3 * (size_t)k + 1] = dot3(s, rw);
  A.r[3 * (size_t)k + 2] = dot3(t, rw);
}

// ---------------------------------------------------------------------------
// Coulomb law, 3D: Fischer-Burmeister error in the mu-scaled self-dual cone (De Saxce
// change of variable) and the local solve (take-off, stick, slide).
__device__ double fb_error_3d(const double* r, const double* u, double mu) {
  double ut2 = 0.0;
  ut2 += u[1] * u[1];
  ut2 += u[2] * u[2];
  const double nut = sqrt(ut2);
  if (mu == 0.0) {
    const double fn = r[0] + u[0] - sqrt(r[0] * r[0] + u[0] * u[0]);
    double e2 = fn * fn;
    e2 += r[1] * r[1];
    e2 += r[2] * r[2];
    return sqrt(e2);
  }
  const double x[3] = {mu * r[0], r[1], r[2]};
  const double y[3] = {u[0] + mu * nut, mu * u[1], mu * u[2]};
  double z0 = 0.0;
  z0 += x[0] * x[0];
  z0 += x[1] * x[1];
  z0 += x[2] * x[2];
  z0 += y[0] * y[0];
  z0 += y[1] * y[1];
  z0 += y[2] * y[2];
  const double zb0 = 2.0 * (x[0] * x[1] + y[0] * y[1]);
  const double zb1 = 2.0 * (x[0] * x[2] + y[0] * y[2]);
  double nzb2 = 0.0;
  nzb2 += zb0 * zb0;
  nzb2 += zb1 * zb1;
  const double nzb = sqrt(nzb2);
  double l1 = z0 - nzb;
  if (l1 < 0.0) l1 = 0.0;
  const double l2 = z0 + nzb;
  const double s1 = sqrt(l1), s2 = sqrt(l2);
  const double sq0 = 0.5 * (s1 + s2);
  const double half_diff = 0.5 * (s2 - s1);
  const double sq1 = (nzb > 0.0) ? half_diff * (zb0 / nzb) : half_diff;
  const double sq2 = (nzb > 0.0) ? half_diff * (zb1 / nzb) : 0.0;
  double e2 = 0.0;
  const double p0 = x[0] + y[0] - sq0;
  e2 += p0 * p0;
  const double p1 = x[1] + y[1] - sq1;
  e2 += p1 * p1;
  const double p2 = x[2] + y[2] - sq2;
  e2 += p2 * p2;
  return sqrt(e2);
}

__device__ __forceinline__ void apply_w(const double* a, const double* rc, const double* b, double* u) {
  u[0] = a[0] * rc[0] + a[1] * rc[1] + a[2] * rc[2] + b[0];
  u[1] = a[1] * rc[0] + a[3] * rc[1] + a[4] * rc[2] + b[1];
  u[2] = a[2] * rc[0] + a[4] * rc[1] + a[5] * rc[2] + b[2];
}

// Anisotropic sliding: root search on the sliding direction over the unit circle through
// the rational chart d = +-((1-s^2), 2s)/(1+s^2), s in [-1, 1] per half circle; sign
// changes of g = u_T x d on a 256-point grid per half are refined by bisection and the
// admissible root with the smallest Coulomb error is kept.  Rarely reached (the fixed
// point on the direction handles near-isotropic tangential blocks), so kept out of line.
__device__ __noinline__ bool slide_root_search(const double* a, const double* b, double mu, double* r) {
  const double a00 = a[0], a01 = a[1], a02 = a[2], a11 = a[3], a12 = a[4], a22 = a[5];
  auto eval = [&](double s, double sign, double* out) -> bool {
    const double den_s = 1.0 + s * s;
    const double e0 = sign * (1.0 - s * s) / den_s, e1 = sign * (2.0 * s) / den_s;
    const double den = a00 - mu * (a01 * e0 + a02 * e1);
    if (!(den > 0.0)) return false;
    const double n_ = -b[0] / den;
    const double t0 = -mu * n_ * e0, t1 = -mu * n_ * e1;
    const double v0 = a01 * n_ + a11 * t0 + a12 * t1 + b[1];
    const double v1 = a02 * n_ + a12 * t0 + a22 * t1 + b[2];
    out[0] = v0 * e1 - v1 * e0;
    out[1] = v0 * e0 + v1 * e1;
    out[2] = n_;
    out[3] = t0;
    out[4] = t1;
    return true;
  };
  double best_e = INFINITY;
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
          double u[3];
          apply_w(a, rc, b, u);
          const double e = fb_error_3d(rc, u, mu);
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
  if (best_e < INFINITY) {
    r[0] = best_r[0];
    r[1] = best_r[1];
    r[2] = best_r[2];
    return true;
  }
  return false;
}

__device__ __noinline__ void local_fallback_3d(const double* a, const double* b, double mu, double rs0, double rs1,
                                               double rs2, bool slide_ok, double rn, double rt0, double rt1,
                                               double* r) {
  if (slide_root_search(a, b, mu, r)) return;
  double best = INFINITY;
  double br[3] = {0.0, 0.0, 0.0};
  auto consider = [&](double x0, double x1, double x2) {
    const double rc[3] = {x0, x1, x2};
    double u[3];
    apply_w(a, rc, b, u);
    const double e = fb_error_3d(rc, u, mu);
    if (e < best) {
      best = e;
      br[0] = x0;
      br[1] = x1;
      br[2] = x2;
    }
  };
  consider(0.0, 0.0, 0.0);
  if (rs0 >= 0.0) {
    const double nt = sqrt(rs1 * rs1 + rs2 * rs2);
    const double sc = (nt > mu * rs0 && nt > 0.0) ? (mu * rs0) / nt : 1.0;
    consider(rs0, rs1 * sc, rs2 * sc);
  }
  if (slide_ok && rn >= 0.0) consider(rn, rt0, rt1);
  r[0] = br[0];
  r[1] = br[1];
  r[2] = br[2];
}

// Local Coulomb problem u = W r + b, W = (w00 w01 w02 w11 w12 w22) SPD.
__device__ __forceinline__ void local_solve_3d(const double* a, const double* b, double mu, double* r) {
  if (b[0] >= 0.0) {
    r[0] = r[1] = r[2] = 0.0;
    return;
  }
  const double a00 = a[0], a01 = a[1], a02 = a[2], a11 = a[3], a12 = a[4], a22 = a[5];
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
  if (rs0 >= 0.0 && sqrt(rs1 * rs1 + rs2 * rs2) <= mu * rs0) {
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
      const double lmax = hs + sqrt(hd * hd + m01 * m01);
      double al = sqrt(g0 * g0 + g1 * g1) - lmax;
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
      const double ne = sqrt(e0 * e0 + e1 * e1);
      if (!(ne > 0.0)) break;
      d0 = e0 / ne;
      d1 = e1 / ne;
      const double den = a00 - mu * (a01 * d0 + a02 * d1);
      if (!(den > 0.0)) break;
      const double rn_new = -b[0] / den;
      const bool same = fabs(rn_new - rn) <= 1.0e-15 * fabs(rn_new);
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
  local_fallback_3d(a, b, mu, rs0, rs1, rs2, slide_ok, rn, rt0, rt1, r);
}

// ---------------------------------------------------------------------------
// Solver.  Running velocities: V[2i] = (v, 0), V[2i+1] = (omega, 0).
struct Contacts3 {
  const int* ia;
  const int* ib;
  const double* E;
  const double* Aa;
  const double* Ab;
  const double* c;
  const double* W;
  const double* mu;
};

// Running velocities are written by other SMs between grid barriers: read at L2.
__device__ __forceinline__ double4_32a ld4cg(const double4_32a* p) {
  const double2* q = reinterpret_cast<const double2*>(p);
  const double2 a = __ldcg(q), b = __ldcg(q + 1);
  return make_double4_32a(a.x, a.y, b.x, b.y);
}

// u = H v + c at the current running velocities.
__device__ __forceinline__ void local_u3(const Contacts3& C, int k, const double4_32a* V, double* u, int a, int b,
                                        const double* E, const double* Aa, const double* Ab) {
  const double4_32a la = ld4cg(&V[2 * a]), wa = ld4cg(&V[2 * a + 1]);
  const double va[3] = {la.x, la.y, la.z}, oa[3] = {wa.x, wa.y, wa.z};
  double vb[3] = {0.0, 0.0, 0.0}, ob[3] = {0.0, 0.0, 0.0};
  const bool has_b = b >= 0;
  if (has_b) {
    const double4_32a lb = ld4cg(&V[2 * b]), wb = ld4cg(&V[2 * b + 1]);
    vb[0] = lb.x;
    vb[1] = lb.y;
    vb[2] = lb.z;
    ob[0] = wb.x;
    ob[1] = wb.y;
    ob[2] = wb.z;
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    double h = dot3(E + 3 * i, va);
    if (i > 0) h = h + dot3(Aa + 3 * (i - 1), oa);
    if (has_b) {
      double hb = dot3(E + 3 * i, vb);
      if (i > 0) hb = hb + dot3(Ab + 3 * (i - 1), ob);
      h = h - hb;
    }
    u[i] = h + C.c[3 * (size_t)k + i];
  }
}

__device__ __forceinline__ void load_contact(const Contacts3& C, int k, double* E, double* Aa, double* Ab) {
#pragma unroll
  for (int j = 0; j < 9; ++j) E[j] = C.E[9 * (size_t)k + j];
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    Aa[j] = C.Aa[6 * (size_t)k + j];
    Ab[j] = C.Ab[6 * (size_t)k + j];
  }
}

__device__ __forceinline__ void gather_htr3(int body, const int* __restrict__ off, const int* __restrict__ adj,
                                            const Contacts3& C, const double* r, double* hl, double* ha) {
  hl[0] = hl[1] = hl[2] = 0.0;
  ha[0] = ha[1] = ha[2] = 0.0;
  const int e = off[body + 1];
  for (int p = off[body]; p < e; ++p) {
    const int k = adj[p];
    const bool is_a = C.ia[k] == body;
    const double sgn = is_a ? 1.0 : -1.0;
    const double* E = C.E + 9 * (size_t)k;
    const double* A = (is_a ? C.Aa : C.Ab) + 6 * (size_t)k;
    const double r0 = r[3 * (size_t)k], r1 = r[3 * (size_t)k + 1], r2 = r[3 * (size_t)k + 2];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const double pl = (E[j] * r0 + E[3 + j] * r1) + E[6 + j] * r2;
      const double pa = A[j] * r1 + A[3 + j] * r2;
      hl[j] = hl[j] + sgn * pl;
      ha[j] = ha[j] + sgn * pa;
    }
  }
}

__global__ void k_vel_init3(int nb, const int* __restrict__ off, const int* __restrict__ adj, Contacts3 C,
                            const double* __restrict__ r, const double* __restrict__ v0,
                            const double* __restrict__ minv, const double* __restrict__ Iinv, double4_32a* __restrict__ V) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  double hl[3], ha[3], Ii[9], wa[3];
  gather_htr3(i, off, adj, C, r, hl, ha);
#pragma unroll
  for (int j = 0; j < 9; ++j) Ii[j] = Iinv[9 * (size_t)i + j];
  matvec3(Ii, ha, wa);
  const double mi = minv[i];
  const double* vl = v0 + 3 * (size_t)i;
  const double* va = v0 + 3 * (size_t)nb + 3 * (size_t)i;
  V[2 * i] = make_double4_32a(vl[0] + mi * hl[0], vl[1] + mi * hl[1], vl[2] + mi * hl[2], 0.0);
  V[2 * i + 1] = make_double4_32a(va[0] + wa[0], va[1] + wa[1], va[2] + wa[2], 0.0);
}

__global__ void k_final_vel3(int nb, const int* __restrict__ off, const int* __restrict__ adj, Contacts3 C,
                             const double* __restrict__ r, const double* __restrict__ v0, const double* __restrict__ m,
                             const double* __restrict__ minv, const double* __restrict__ Iw,
                             const double* __restrict__ Iinv, double* __restrict__ v2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const double* vl = v0 + 3 * (size_t)i;
  const double* va = v0 + 3 * (size_t)nb + 3 * (size_t)i;
  double* ol = v2 + 3 * (size_t)i;
  double* oa = v2 + 3 * (size_t)nb + 3 * (size_t)i;
  if (off[i + 1] == off[i]) {
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      ol[j] = vl[j];
      oa[j] = va[j];
    }
    return;
  }
  double hl[3], ha[3], Lw[3], rhs[3], wa[3], M[9];
  gather_htr3(i, off, adj, C, r, hl, ha);
#pragma unroll
  for (int j = 0; j < 9; ++j) M[j] = Iw[9 * (size_t)i + j];
  const double w0[3] = {va[0], va[1], va[2]};
  matvec3(M, w0, Lw);
  const double mi = m[i], ivm = minv[i];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const double fl = -(mi * vl[j]);
    ol[j] = ivm * (hl[j] - fl);
    rhs[j] = ha[j] - (-Lw[j]);
  }
#pragma unroll
  for (int j = 0; j < 9; ++j) M[j] = Iinv[9 * (size_t)i + j];
  matvec3(M, rhs, wa);
#pragma unroll
  for (int j = 0; j < 3; ++j) oa[j] = wa[j];
}

__global__ void k_extract3(int nc, const double* __restrict__ E3, const double* __restrict__ r, double* __restrict__ ab) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nc) return;
  const double* E = E3 + 9 * (size_t)k;
  const double r0 = r[3 * (size_t)k], r1 = r[3 * (size_t)k + 1], r2 = r[3 * (size_t)k + 2];
  double rw[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) rw[j] = (E[j] * r0 + E[3 + j] * r1) + E[6 + j] * r2;
  ab[3 * (size_t)k] = dot3(rw, E);
  ab[3 * (size_t)k + 1] = dot3(rw, E + 3);
  ab[3 * (size_t)k + 2] = dot3(rw, E + 6);
}

// SymplecticEulerImpactFrictionMap::cacheImpulses (SymplecticEulerImpactFrictionMap.cpp:133-199):
// per contact the normal and the force f = alpha n + beta0 s + beta1 t (or alpha alone when only
// normals are cached), from the step's (alpha, beta0, beta1).
__global__ void k_cache3(int nc, int cache_mode, const double* __restrict__ E3, const double* __restrict__ ab,
                         double* __restrict__ c6) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nc) return;
  double* c = c6 + 6 * (size_t)k;
  const double al = ab[3 * (size_t)k], b0 = ab[3 * (size_t)k + 1], b1 = ab[3 * (size_t)k + 2];
  if (cache_mode == SG_CACHE_NORMAL) {
    c[0] = al;
#pragma unroll
    for (int j = 1; j < 6; ++j) c[j] = 0.0;
    return;
  }
  const double* E = E3 + 9 * (size_t)k;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    c[j] = E[j];
    c[3 + j] = (al * E[j] + b0 * E[3 + j]) + b1 * E[6 + j];
  }
}

struct Gs3Args {
  int nc;
  Contacts3 C;
  const double* minv;
  const double* Iinv;
  const int* perm;
  double* r;
  double* r_a;
  double* r_b;
  double4_32a* V;
  SolveStats* st;
  GridBarrier* gb;
  unsigned long long spin;
  double tol;
  unsigned max_iters;
  unsigned eval_every;
};

__device__ __forceinline__ void gs_update3(const Gs3Args& A, int k) {
  const Contacts3& C = A.C;
  const int a = C.ia[k], b = C.ib[k];
  const bool has_b = b >= 0;
  double E[9], Aa[6], Ab[6];
  load_contact(C, k, E, Aa, Ab);
  double u[3];
  local_u3(C, k, A.V, u, a, b, E, Aa, Ab);
  const double r0 = __ldcg(&A.r[3 * (size_t)k]), r1 = __ldcg(&A.r[3 * (size_t)k + 1]),
               r2 = __ldcg(&A.r[3 * (size_t)k + 2]);
  double W[6];
#pragma unroll
  for (int j = 0; j < 6; ++j) W[j] = C.W[6 * (size_t)k + j];
  const double bt[3] = {u[0] - ((W[0] * r0 + W[1] * r1) + W[2] * r2), u[1] - ((W[1] * r0 + W[3] * r1) + W[4] * r2),
                        u[2] - ((W[2] * r0 + W[4] * r1) + W[5] * r2)};
  double rn[3];
  local_solve_3d(W, bt, C.mu[k], rn);
  const double d0 = rn[0] - r0, d1 = rn[1] - r1, d2 = rn[2] - r2;
  double pl[3], pa[3], pb[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    pl[j] = (E[j] * d0 + E[3 + j] * d1) + E[6 + j] * d2;
    pa[j] = Aa[j] * d1 + Aa[3 + j] * d2;
    pb[j] = Ab[j] * d1 + Ab[3 + j] * d2;
  }
  double Ii[9], wa[3];
#pragma unroll
  for (int j = 0; j < 9; ++j) Ii[j] = A.Iinv[9 * (size_t)a + j];
  matvec3(Ii, pa, wa);
  const double ma = A.minv[a];
  {
    const double4_32a la = ld4cg(&A.V[2 * a]), oa = ld4cg(&A.V[2 * a + 1]);
    A.V[2 * a] = make_double4_32a(la.x + ma * pl[0], la.y + ma * pl[1], la.z + ma * pl[2], 0.0);
    A.V[2 * a + 1] = make_double4_32a(oa.x + wa[0], oa.y + wa[1], oa.z + wa[2], 0.0);
  }
  if (has_b) {
    double wb[3];
#pragma unroll
    for (int j = 0; j < 9; ++j) Ii[j] = A.Iinv[9 * (size_t)b + j];
    matvec3(Ii, pb, wb);
    const double mb = A.minv[b];
    const double4_32a lb = ld4cg(&A.V[2 * b]), ob = ld4cg(&A.V[2 * b + 1]);
    A.V[2 * b] = make_double4_32a(lb.x - mb * pl[0], lb.y - mb * pl[1], lb.z - mb * pl[2], 0.0);
    A.V[2 * b + 1] = make_double4_32a(ob.x - wb[0], ob.y - wb[1], ob.z - wb[2], 0.0);
  }
  A.r[3 * (size_t)k] = rn[0];
  A.r[3 * (size_t)k + 1] = rn[1];
  A.r[3 * (size_t)k + 2] = rn[2];
}

__global__ void __launch_bounds__(kGs3Block, 1) k_gs3(Gs3Args A) {
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
  double* best = A.r_a;
  double* cand = A.r_b;
  double err_best = INFINITY;
  bool converged = false;
  unsigned it = 0;
  unsigned n_eval = 0;
  for (it = 1; it <= A.max_iters; ++it) {
    for (int col = 0; col < ncol; ++col) {
      // Consecutive contacts of a colour go to consecutive blocks (one per SM), so that a
      // small colour spreads its FP64 work over every SM instead of filling a few.
      const int e = s_off[col + 1];
      for (int s = s_off[col] + blockIdx.x + gridDim.x * threadIdx.x; s < e; s += nthr) gs_update3(A, A.perm[s]);
      if (!grid_sync(A.gb, A.spin)) {
        if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
        return;
      }
    }
    if (it % eval_every == 0) {
      double emax = 0.0;
      for (int k = tid; k < A.nc; k += nthr) {
        const int a = A.C.ia[k], b = A.C.ib[k];
        double E[9], Aa[6], Ab[6], u[3];
        load_contact(A.C, k, E, Aa, Ab);
        local_u3(A.C, k, A.V, u, a, b, E, Aa, Ab);
        const double rk[3] = {__ldcg(&A.r[3 * (size_t)k]), __ldcg(&A.r[3 * (size_t)k + 1]),
                              __ldcg(&A.r[3 * (size_t)k + 2])};
        cand[3 * (size_t)k] = rk[0];
        cand[3 * (size_t)k + 1] = rk[1];
        cand[3 * (size_t)k + 2] = rk[2];
        emax = nanmax(emax, fb_error_3d(rk, u, A.C.mu[k]));
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
        double* t = best;
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
      for (int k = tid; k < 3 * A.nc; k += nthr) A.r[k] = __ldcg(&best[k]);
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

// ---------------------------------------------------------------------------
// Batched sphere scenes: one coloured sweep over the contacts of all scenes (scenes share no
// body, so the global colouring colours every scene), with each scene's own residual, best
// iterate, convergence test and iteration count, as if every scene were solved alone
// (Sobogus::solve per RigidBody3DSim).  A converged scene's contacts stop updating; the kernel
// ends when every scene has converged or at max_iters.  FP64.
struct Gs3BatchArgs {
  Gs3Args g;                     // g.r_a / g.r_b: the two snapshot buffers
  const int* scene_of;           // body -> scene (a contact's scene is that of its first body)
  const int* sc_off;             // scene contact offsets (S + 1)
  int S;
  unsigned long long* err_slot;  // 3 S ordered residual maxima (rotating)
  double* best;                  // S
  int* bestbuf;                  // S
  int* done;                     // S
  unsigned* iters;               // S
  int* done_count;
  unsigned long long* unconverged;
  unsigned long long* work;      // [1] contact updates, [2] contact evaluations
};

__device__ __forceinline__ void run_max_atomic3(unsigned long long v, int key, unsigned long long* slots) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long w = __shfl_down_sync(0xffffffffu, v, o);
    const int kw = __shfl_down_sync(0xffffffffu, key, o);
    if (lane + o < 32 && kw == key && w > v) v = w;
  }
  const int kprev = __shfl_up_sync(0xffffffffu, key, 1);
  if (key >= 0 && (lane == 0 || kprev != key)) atomicMax(&slots[key], v);
}

__global__ void __launch_bounds__(kGs3Block, 1) k_gs3_batch(Gs3BatchArgs B) {
  const Gs3Args& A = B.g;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nthr = gridDim.x * blockDim.x;
  if (*((volatile int*)&A.st->status) != 0) return;
  __shared__ int s_off[kMaxColors + 1];
  __shared__ int s_ncol;
  if (threadIdx.x == 0) s_ncol = A.st->n_colors;
  for (int c = threadIdx.x; c <= kMaxColors; c += blockDim.x) s_off[c] = A.st->color_off[c];
  const int nc = A.nc, S = B.S;
  for (int sc = tid; sc < S; sc += nthr) {
    B.best[sc] = INFINITY;
    B.bestbuf[sc] = 0;
    B.iters[sc] = 0;
    const bool empty = B.sc_off[sc + 1] == B.sc_off[sc];
    B.done[sc] = empty ? 1 : 0;
    if (empty) atomicAdd(B.done_count, 1);
  }
  __syncthreads();
  const int ncol = s_ncol;
  const unsigned eval_every = A.eval_every ? A.eval_every : 1u;
  double* bufs[2] = {A.r_a, A.r_b};
  if (!grid_sync(A.gb, A.spin)) {
    if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
    return;
  }
  unsigned n_eval = 0, it = 0;
  unsigned long long nupd = 0, nevw = 0;
  if (*((volatile int*)B.done_count) < S) {
    for (it = 1; it <= A.max_iters; ++it) {
      for (int col = 0; col < ncol; ++col) {
        const int e = s_off[col + 1];
        for (int s = s_off[col] + blockIdx.x + gridDim.x * threadIdx.x; s < e; s += nthr) {
          const int k = A.perm[s];
          if (__ldcg(&B.done[B.scene_of[A.C.ia[k]]])) continue;
          gs_update3(A, k);
          ++nupd;
        }
        if (!grid_sync(A.gb, A.spin)) {
          if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
          return;
        }
      }
      if (it % eval_every != 0) continue;
      const int slot = n_eval % 3;
      unsigned long long* slots = B.err_slot + (size_t)slot * S;
      const int lane = threadIdx.x & 31;
      for (int k0 = tid - lane; k0 < nc; k0 += nthr) {
        const int k = k0 + lane;
        int key = -1;
        unsigned long long v = 0ull;
        if (k < nc) {
          const int a = A.C.ia[k], b = A.C.ib[k];
          const int sc = B.scene_of[a];
          if (!__ldcg(&B.done[sc])) {
            double E[9], Aa[6], Ab[6], u[3];
            load_contact(A.C, k, E, Aa, Ab);
            local_u3(A.C, k, A.V, u, a, b, E, Aa, Ab);
            const double rk[3] = {__ldcg(&A.r[3 * (size_t)k]), __ldcg(&A.r[3 * (size_t)k + 1]),
                                  __ldcg(&A.r[3 * (size_t)k + 2])};
            double* cand = bufs[1 - __ldcg(&B.bestbuf[sc])];
            cand[3 * (size_t)k] = rk[0];
            cand[3 * (size_t)k + 1] = rk[1];
            cand[3 * (size_t)k + 2] = rk[2];
            v = f64_to_ordered(fb_error_3d(rk, u, A.C.mu[k]));
            key = sc;
            ++nevw;
          }
        }
        run_max_atomic3(v, key, slots);
      }
      if (!grid_sync(A.gb, A.spin)) {
        if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
        return;
      }
      unsigned long long* next = B.err_slot + (size_t)((n_eval + 1) % 3) * S;
      for (int sc = tid; sc < S; sc += nthr) {
        next[sc] = 0ull;
        if (B.done[sc]) continue;
        const double err = ordered_to_f64(__ldcg(&slots[sc]));
        if (err < B.best[sc]) {
          B.best[sc] = err;
          B.bestbuf[sc] ^= 1;
        }
        if (err < A.tol) {
          B.done[sc] = 1;
          B.iters[sc] = it;
          atomicAdd(B.done_count, 1);
        }
      }
      ++n_eval;
      if (!grid_sync(A.gb, A.spin)) {
        if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
        return;
      }
      if (*((volatile int*)B.done_count) == S) break;
    }
  }
  // Scenes that did not converge return their best iterate (GaussSeidel: x = x_best).
  for (int k = tid; k < nc; k += nthr) {
    const int sc = B.scene_of[A.C.ia[k]];
    if (__ldcg(&B.done[sc]) || !(__ldcg(&B.best[sc]) < INFINITY)) continue;
    const double* src = bufs[__ldcg(&B.bestbuf[sc])];
    for (int j = 0; j < 3; ++j) A.r[3 * (size_t)k + j] = __ldcg(&src[3 * (size_t)k + j]);
  }
  for (int sc = tid; sc < S; sc += nthr)
    if (!__ldcg(&B.done[sc])) B.iters[sc] = A.max_iters;
  if (tid == 0) *B.unconverged += (unsigned long long)(S - *((volatile int*)B.done_count));
  atomicAdd(&B.work[1], nupd);
  atomicAdd(&B.work[2], nevw);
  if (tid == 0) {
    A.st->iterations = it > A.max_iters ? A.max_iters : it;
    A.st->sweeps64 = it > A.max_iters ? A.max_iters : it;
    A.st->evals = n_eval;
    A.st->converged = *((volatile int*)B.done_count) == S ? 1 : 0;
  }
}

// ---------------------------------------------------------------------------
// Mixed precision for spheres, as k_gs_mixed for discs: FP32 sweeps over colour-packed
// FP32 copies (contact s of the packed arrays is contact perm[s]), the FP64 image lifted and
// checked on a growing schedule, FP64 sweeps to finish once FP32 reached tol or its rounding
// floor.
constexpr int kGs3mBlock = 256;

struct Gs3m {
  const int2* ab;       // (a, b) per packed contact
  const float* E;       // 9 per packed contact
  const float* Aa;      // 6
  const float* Ab;      // 6
  const float* c;       // 3
  const float* W;       // 6
  const float* mu;
  float* r;             // 3
  float4* V;            // 2 per body: (v, 0), (omega, 0)
  const float* minv;
  const float* Iinv;    // 9 per body
  const double* v0;     // [v (3nb) | omega (3nb)]
  const int* body_off;
  const int* body_adj;
  int nb;
  unsigned eval32;
  unsigned long long* work;  // [0] FP32 updates, [1] FP64 updates, [2] evaluations, [3] lifts (contacts), [4] lifts (bodies)
};

__device__ __forceinline__ float dot3f(const float* a, const float* b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
__device__ __forceinline__ void matvec3f(const float* A, const float* x, float* y) {
  const float t0 = (A[0] * x[0] + A[1] * x[1]) + A[2] * x[2];
  const float t1 = (A[3] * x[0] + A[4] * x[1]) + A[5] * x[2];
  const float t2 = (A[6] * x[0] + A[7] * x[1]) + A[8] * x[2];
  y[0] = t0;
  y[1] = t1;
  y[2] = t2;
}

// The 3D local Coulomb solve in FP32: take-off, stick, and the slide by Newton on the slip
// speed; a degenerate problem takes the stick solution projected onto the cone.
__device__ void local_solve_3d_f(const float* a, const float* b, float mu, float* r) {
  if (b[0] >= 0.0f) {
    r[0] = r[1] = r[2] = 0.0f;
    return;
  }
  const float a00 = a[0], a01 = a[1], a02 = a[2], a11 = a[3], a12 = a[4], a22 = a[5];
  const float c00 = a11 * a22 - a12 * a12, c01 = a02 * a12 - a01 * a22, c02 = a01 * a12 - a02 * a11;
  const float c11 = a00 * a22 - a02 * a02, c12 = a01 * a02 - a00 * a12, c22 = a00 * a11 - a01 * a01;
  const float det = a00 * c00 + a01 * c01 + a02 * c02;
  const float rs0 = -(c00 * b[0] + c01 * b[1] + c02 * b[2]) / det;
  const float rs1 = -(c01 * b[0] + c11 * b[1] + c12 * b[2]) / det;
  const float rs2 = -(c02 * b[0] + c12 * b[1] + c22 * b[2]) / det;
  if (rs0 >= 0.0f && sqrtf(rs1 * rs1 + rs2 * rs2) <= mu * rs0) {
    r[0] = rs0;
    r[1] = rs1;
    r[2] = rs2;
    return;
  }
  float rn = -b[0] / a00, d0 = 1.0f, d1 = 0.0f;
  bool ok = false;
  if (mu == 0.0f) {
    r[0] = rn;
    r[1] = r[2] = 0.0f;
    return;
  }
  for (int outer = 0; outer < 4; ++outer) {
    const float cc = mu * rn;
    const float g0 = a01 * rn + b[1], g1 = a02 * rn + b[2];
    const float m00 = cc * a11, m01 = cc * a12, m11 = cc * a22;
    const float hs = 0.5f * (m00 + m11), hd = 0.5f * (m00 - m11);
    float al = sqrtf(g0 * g0 + g1 * g1) - (hs + sqrtf(hd * hd + m01 * m01));
    if (!(al > 0.0f)) al = 0.0f;
    float e0 = 0.0f, e1 = 0.0f;
    for (int it = 0; it < 24; ++it) {
      const float p00 = al + m00, p11 = al + m11;
      const float inv = 1.0f / (p00 * p11 - m01 * m01);
      e0 = (p11 * g0 - m01 * g1) * inv;
      e1 = (p00 * g1 - m01 * g0) * inv;
      const float f = e0 * e0 + e1 * e1 - 1.0f;
      const float q0 = (p11 * e0 - m01 * e1) * inv, q1 = (p00 * e1 - m01 * e0) * inv;
      const float fp = -2.0f * (e0 * q0 + e1 * q1);
      if (!(f > 0.0f) || !(fp < 0.0f)) break;
      const float step = -f / fp;
      al += step;
      if (!(step > 1e-7f * (1.0f + al))) break;
    }
    const float ne = sqrtf(e0 * e0 + e1 * e1);
    if (!(ne > 0.0f)) break;
    d0 = e0 / ne;
    d1 = e1 / ne;
    const float den = a00 - mu * (a01 * d0 + a02 * d1);
    if (!(den > 0.0f)) break;
    const float rn_new = -b[0] / den;
    const bool same = fabsf(rn_new - rn) <= 1e-7f * fabsf(rn_new);
    rn = rn_new;
    if (same) {
      ok = true;
      break;
    }
  }
  if (ok && rn >= 0.0f) {
    r[0] = rn;
    r[1] = -mu * rn * d0;
    r[2] = -mu * rn * d1;
    return;
  }
  const float rn2 = fmaxf(rs0, 0.0f);
  const float nt = sqrtf(rs1 * rs1 + rs2 * rs2);
  const float sc = (nt > mu * rn2 && nt > 0.0f) ? (mu * rn2) / nt : 1.0f;
  r[0] = rn2;
  r[1] = rs1 * sc;
  r[2] = rs2 * sc;
}

__device__ __forceinline__ void gs_update3_f(const Gs3m& B, int s) {
  const int2 ab = B.ab[s];
  const int a = ab.x, b = ab.y;
  const bool has_b = b >= 0;
  float E[9], Aa[6], Ab[6], W[6], c[3];
#pragma unroll
  for (int j = 0; j < 9; ++j) E[j] = B.E[9 * (size_t)s + j];
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    Aa[j] = B.Aa[6 * (size_t)s + j];
    Ab[j] = B.Ab[6 * (size_t)s + j];
    W[j] = B.W[6 * (size_t)s + j];
  }
#pragma unroll
  for (int j = 0; j < 3; ++j) c[j] = B.c[3 * (size_t)s + j];
  const float4 la = __ldcg(&B.V[2 * a]), wa = __ldcg(&B.V[2 * a + 1]);
  const float va[3] = {la.x, la.y, la.z}, oa[3] = {wa.x, wa.y, wa.z};
  float vb[3] = {0.0f, 0.0f, 0.0f}, ob[3] = {0.0f, 0.0f, 0.0f};
  float4 lb = make_float4(0.f, 0.f, 0.f, 0.f), wb = lb;
  if (has_b) {
    lb = __ldcg(&B.V[2 * b]);
    wb = __ldcg(&B.V[2 * b + 1]);
    vb[0] = lb.x;
    vb[1] = lb.y;
    vb[2] = lb.z;
    ob[0] = wb.x;
    ob[1] = wb.y;
    ob[2] = wb.z;
  }
  float u[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    float h = dot3f(E + 3 * i, va);
    if (i > 0) h += dot3f(Aa + 3 * (i - 1), oa);
    if (has_b) {
      float hb = dot3f(E + 3 * i, vb);
      if (i > 0) hb += dot3f(Ab + 3 * (i - 1), ob);
      h -= hb;
    }
    u[i] = h + c[i];
  }
  const float r0 = __ldcg(&B.r[3 * (size_t)s]), r1 = __ldcg(&B.r[3 * (size_t)s + 1]), r2 = __ldcg(&B.r[3 * (size_t)s + 2]);
  const float bt[3] = {u[0] - ((W[0] * r0 + W[1] * r1) + W[2] * r2), u[1] - ((W[1] * r0 + W[3] * r1) + W[4] * r2),
                       u[2] - ((W[2] * r0 + W[4] * r1) + W[5] * r2)};
  float rn[3];
  local_solve_3d_f(W, bt, B.mu[s], rn);
  const float d0 = rn[0] - r0, d1 = rn[1] - r1, d2 = rn[2] - r2;
  float pl[3], pa[3], pb[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    pl[j] = (E[j] * d0 + E[3 + j] * d1) + E[6 + j] * d2;
    pa[j] = Aa[j] * d1 + Aa[3 + j] * d2;
    pb[j] = Ab[j] * d1 + Ab[3 + j] * d2;
  }
  float Ii[9], w[3];
#pragma unroll
  for (int j = 0; j < 9; ++j) Ii[j] = B.Iinv[9 * (size_t)a + j];
  matvec3f(Ii, pa, w);
  const float ma = B.minv[a];
  B.V[2 * a] = make_float4(la.x + ma * pl[0], la.y + ma * pl[1], la.z + ma * pl[2], 0.0f);
  B.V[2 * a + 1] = make_float4(wa.x + w[0], wa.y + w[1], wa.z + w[2], 0.0f);
  if (has_b) {
#pragma unroll
    for (int j = 0; j < 9; ++j) Ii[j] = B.Iinv[9 * (size_t)b + j];
    matvec3f(Ii, pb, w);
    const float mb = B.minv[b];
    B.V[2 * b] = make_float4(lb.x - mb * pl[0], lb.y - mb * pl[1], lb.z - mb * pl[2], 0.0f);
    B.V[2 * b + 1] = make_float4(wb.x - w[0], wb.y - w[1], wb.z - w[2], 0.0f);
  }
  B.r[3 * (size_t)s] = rn[0];
  B.r[3 * (size_t)s + 1] = rn[1];
  B.r[3 * (size_t)s + 2] = rn[2];
}

__global__ void k_pack3(int nc, const int* __restrict__ perm, Contacts3 C, const double* __restrict__ r, Gs3m B,
                        float* __restrict__ r32) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nc) return;
  const int k = perm[s];
  const int b = C.ib[k];
  const_cast<int2*>(B.ab)[s] = make_int2(C.ia[k], b >= 0 ? b : -1);
  float* E = const_cast<float*>(B.E) + 9 * (size_t)s;
  float* Aa = const_cast<float*>(B.Aa) + 6 * (size_t)s;
  float* Ab = const_cast<float*>(B.Ab) + 6 * (size_t)s;
  float* W = const_cast<float*>(B.W) + 6 * (size_t)s;
  float* cc = const_cast<float*>(B.c) + 3 * (size_t)s;
  for (int j = 0; j < 9; ++j) E[j] = (float)C.E[9 * (size_t)k + j];
  for (int j = 0; j < 6; ++j) {
    Aa[j] = (float)C.Aa[6 * (size_t)k + j];
    Ab[j] = (float)C.Ab[6 * (size_t)k + j];
    W[j] = (float)C.W[6 * (size_t)k + j];
  }
  for (int j = 0; j < 3; ++j) {
    cc[j] = (float)C.c[3 * (size_t)k + j];
    r32[3 * (size_t)s + j] = (float)r[3 * (size_t)k + j];
  }
  const_cast<float*>(B.mu)[s] = (float)C.mu[k];
}

__global__ void k_body32(int nb, const double4_32a* __restrict__ V, const double* __restrict__ minv,
                         const double* __restrict__ Iinv, float4* __restrict__ V32, float* __restrict__ minv32,
                         float* __restrict__ Iinv32) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const double4_32a a = V[2 * i], w = V[2 * i + 1];
  V32[2 * i] = make_float4((float)a.x, (float)a.y, (float)a.z, 0.0f);
  V32[2 * i + 1] = make_float4((float)w.x, (float)w.y, (float)w.z, 0.0f);
  minv32[i] = (float)minv[i];
  for (int j = 0; j < 9; ++j) Iinv32[9 * (size_t)i + j] = (float)Iinv[9 * (size_t)i + j];
}

__global__ void __launch_bounds__(kGs3mBlock, 1) k_gs3_mixed(Gs3Args A, Gs3m B) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nthr = gridDim.x * blockDim.x;
  if (*((volatile int*)&A.st->status) != 0) return;
  __shared__ int s_off[kMaxColors + 1];
  __shared__ int s_ncol;
  if (threadIdx.x == 0) s_ncol = A.st->n_colors;
  for (int c = threadIdx.x; c <= kMaxColors; c += blockDim.x) s_off[c] = A.st->color_off[c];
  __syncthreads();
  const int ncol = s_ncol;
  const unsigned eval64 = A.eval_every ? A.eval_every : 1u;
  const unsigned eval32 = B.eval32 ? B.eval32 : 1u;
  double* best = A.r_a;
  double* cand = A.r_b;
  double err_best = INFINITY;
  bool converged = false, fp64 = false;
  unsigned it = 0, n_eval = 0, s32 = 0, s64 = 0, lifts = 0, since_best = 0;
  unsigned next_eval = 1, interval = eval32;
  for (it = 1; it <= A.max_iters; ++it) {
    bool do_eval;
    if (!fp64) {
      for (int col = 0; col < ncol; ++col) {
        const int e = s_off[col + 1];
        for (int s = s_off[col] + blockIdx.x + gridDim.x * threadIdx.x; s < e; s += nthr) gs_update3_f(B, s);
        if (!grid_sync(A.gb, A.spin)) {
          if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
          return;
        }
      }
      ++s32;
      do_eval = it == next_eval || it == A.max_iters;
      if (do_eval) {
        for (int s = tid; s < A.nc; s += nthr) {
          const int k = A.perm[s];
#pragma unroll
          for (int j = 0; j < 3; ++j) A.r[3 * (size_t)k + j] = (double)__ldcg(&B.r[3 * (size_t)s + j]);
        }
        if (!grid_sync(A.gb, A.spin)) {
          if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
          return;
        }
        for (int i = tid; i < B.nb; i += nthr) {
          double hl[3], ha[3], Ii[9], wa[3];
          gather_htr3(i, B.body_off, B.body_adj, A.C, A.r, hl, ha);
#pragma unroll
          for (int j = 0; j < 9; ++j) Ii[j] = A.Iinv[9 * (size_t)i + j];
          matvec3(Ii, ha, wa);
          const double mi = A.minv[i];
          const double* vl = B.v0 + 3 * (size_t)i;
          const double* va = B.v0 + 3 * (size_t)B.nb + 3 * (size_t)i;
          const double4_32a lv = make_double4_32a(vl[0] + mi * hl[0], vl[1] + mi * hl[1], vl[2] + mi * hl[2], 0.0);
          const double4_32a wv = make_double4_32a(va[0] + wa[0], va[1] + wa[1], va[2] + wa[2], 0.0);
          A.V[2 * i] = lv;
          A.V[2 * i + 1] = wv;
          B.V[2 * i] = make_float4((float)lv.x, (float)lv.y, (float)lv.z, 0.0f);
          B.V[2 * i + 1] = make_float4((float)wv.x, (float)wv.y, (float)wv.z, 0.0f);
        }
        ++lifts;
        if (!grid_sync(A.gb, A.spin)) {
          if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
          return;
        }
      }
    } else {
      for (int col = 0; col < ncol; ++col) {
        const int e = s_off[col + 1];
        for (int s = s_off[col] + blockIdx.x + gridDim.x * threadIdx.x; s < e; s += nthr) gs_update3(A, A.perm[s]);
        if (!grid_sync(A.gb, A.spin)) {
          if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
          return;
        }
      }
      ++s64;
      do_eval = (it % eval64 == 0) || it == A.max_iters;
    }
    if (!do_eval) continue;
    double emax = 0.0, excess = -INFINITY;
    for (int k = tid; k < A.nc; k += nthr) {
      const int a = A.C.ia[k], b = A.C.ib[k];
      double E[9], Aa[6], Ab[6], u[3];
      load_contact(A.C, k, E, Aa, Ab);
      local_u3(A.C, k, A.V, u, a, b, E, Aa, Ab);
      const double rk[3] = {__ldcg(&A.r[3 * (size_t)k]), __ldcg(&A.r[3 * (size_t)k + 1]),
                            __ldcg(&A.r[3 * (size_t)k + 2])};
      cand[3 * (size_t)k] = rk[0];
      cand[3 * (size_t)k + 1] = rk[1];
      cand[3 * (size_t)k + 2] = rk[2];
      const double ek = fb_error_3d(rk, u, A.C.mu[k]);
      emax = nanmax(emax, ek);
      const double4_32a la = ld4cg(&A.V[2 * a]), wa = ld4cg(&A.V[2 * a + 1]);
      double scale = fabs(la.x) + fabs(la.y) + fabs(la.z) + fabs(wa.x) + fabs(wa.y) + fabs(wa.z);
      if (b >= 0) {
        const double4_32a lb = ld4cg(&A.V[2 * b]), wb = ld4cg(&A.V[2 * b + 1]);
        scale += fabs(lb.x) + fabs(lb.y) + fabs(lb.z) + fabs(wb.x) + fabs(wb.y) + fabs(wb.z);
      }
      scale += fabs(A.C.c[3 * (size_t)k]) + fabs(A.C.c[3 * (size_t)k + 1]) + fabs(A.C.c[3 * (size_t)k + 2]) +
               fabs(rk[0]) + fabs(rk[1]) + fabs(rk[2]);
      excess = nanmax(excess, ek - 64.0 * 1.1920929e-7 * scale);
    }
    emax = block_nanmax(emax);
    const double mag = block_nanmax(excess);
    const int slot = n_eval % 3;
    if (threadIdx.x == 0) {
      atomicMax(&A.st->err_slot[slot], f64_to_ordered(emax));
      atomicMax(&A.st->mag_slot[slot], f64_to_ordered(mag));
    }
    if (tid == 0) {
      A.st->err_slot[(n_eval + 1) % 3] = 0ull;
      A.st->mag_slot[(n_eval + 1) % 3] = 0ull;
    }
    if (!grid_sync(A.gb, A.spin)) {
      if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
      return;
    }
    const double err = ordered_to_f64(*((volatile unsigned long long*)&A.st->err_slot[slot]));
    const double excess32 = ordered_to_f64(*((volatile unsigned long long*)&A.st->mag_slot[slot]));
    ++n_eval;
    if (err < err_best) {
      err_best = err;
      double* t = best;
      best = cand;
      cand = t;
      since_best = 0;
    } else {
      ++since_best;
    }
    if (!fp64) {
      if (it < eval32) {
        next_eval = 2 * it;
      } else {
        interval = (err > 1e3 * A.tol) ? min(2u * interval, 16u * eval32) : (err > 10.0 * A.tol ? interval : eval32);
        next_eval = it + interval;
      }
    }
    if (fp64) {
      if (err < A.tol) {
        converged = true;
        break;
      }
    } else if (err < A.tol || excess32 <= A.tol || (since_best >= 16 && excess32 <= 16.0 * A.tol)) {
      fp64 = true;
    }
  }
  if (it > A.max_iters) it = A.max_iters;
  if (!converged) {
    if (err_best < INFINITY)
      for (int k = tid; k < 3 * A.nc; k += nthr) A.r[k] = __ldcg(&best[k]);
  }
  if (tid == 0) {
    A.st->iterations = it;
    A.st->converged = converged ? 1 : 0;
    A.st->error = err_best;
    A.st->sweeps32 = s32;
    A.st->sweeps64 = s64;
    A.st->evals = n_eval;
    A.st->lifts = lifts;
  }
}

// Batched sphere scenes in the FP32 form: k_gs3_batch's per-scene control with k_gs3_mixed's
// per-scene modes (0: FP32 sweeps with FP64 checks on a growing schedule, 1: FP64 sweeps to finish,
// entered when the scene reaches tol or its FP32 rounding floor), as k_gs_mixed_batch does for discs.
struct Gs3MixedBatchArgs {
  Gs3BatchArgs X;
  int* mode;                        // S
  unsigned* since;                  // S: checks since the scene's best residual
  unsigned long long* exc_slot;     // 3 S ordered FP32-floor excess maxima (rotating)
  unsigned long long* gmax;         // 3: largest FP32-mode residual of a check (interval control)
  int* n64;                         // scenes in mode 1
};

__global__ void __launch_bounds__(kGs3mBlock, 1) k_gs3_mixed_batch(Gs3MixedBatchArgs M, Gs3m B) {
  Gs3BatchArgs& X = M.X;
  const Gs3Args& A = X.g;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nthr = gridDim.x * blockDim.x;
  if (*((volatile int*)&A.st->status) != 0) return;
  __shared__ int s_off[kMaxColors + 1];
  __shared__ int s_ncol;
  if (threadIdx.x == 0) s_ncol = A.st->n_colors;
  for (int c = threadIdx.x; c <= kMaxColors; c += blockDim.x) s_off[c] = A.st->color_off[c];
  const int nc = A.nc, S = X.S;
  for (int sc = tid; sc < S; sc += nthr) {
    X.best[sc] = INFINITY;
    X.bestbuf[sc] = 0;
    X.iters[sc] = 0;
    M.mode[sc] = 0;
    M.since[sc] = 0;
    const bool empty = X.sc_off[sc + 1] == X.sc_off[sc];
    X.done[sc] = empty ? 1 : 0;
    if (empty) atomicAdd(X.done_count, 1);
  }
  __syncthreads();
  const int ncol = s_ncol;
  const unsigned eval64 = A.eval_every ? A.eval_every : 1u;
  const unsigned eval32 = B.eval32 ? B.eval32 : 1u;
  double* bufs[2] = {A.r_a, A.r_b};
  if (!grid_sync(A.gb, A.spin)) {
    if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
    return;
  }
  unsigned long long n32 = 0, n64 = 0, nev = 0, nlc = 0, nlb = 0;
  unsigned it = 0, n_eval = 0, next_eval = 1, interval = eval32;
  if (*((volatile int*)X.done_count) < S) {
    for (it = 1; it <= A.max_iters; ++it) {
      for (int col = 0; col < ncol; ++col) {
        const int e = s_off[col + 1];
        for (int s = s_off[col] + blockIdx.x + gridDim.x * threadIdx.x; s < e; s += nthr) {
          const int sc = X.scene_of[B.ab[s].x];
          if (__ldcg(&X.done[sc])) continue;
          if (__ldcg(&M.mode[sc]) == 0) {
            gs_update3_f(B, s);
            ++n32;
          } else {
            gs_update3(A, A.perm[s]);
            ++n64;
          }
        }
        if (!grid_sync(A.gb, A.spin)) {
          if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
          return;
        }
      }
      const bool due32 = it == next_eval || it == A.max_iters;
      const bool due64 = *((volatile int*)M.n64) > 0 && ((it % eval64 == 0) || it == A.max_iters);
      if (!due32 && !due64) continue;
      if (due32) {
        // Lift the FP32 scenes' iterates to FP64 and resynchronise their FP32 body velocities.
        for (int s = tid; s < nc; s += nthr) {
          const int sc = X.scene_of[B.ab[s].x];
          if (__ldcg(&X.done[sc]) || __ldcg(&M.mode[sc]) != 0) continue;
          const int k = A.perm[s];
#pragma unroll
          for (int j = 0; j < 3; ++j) A.r[3 * (size_t)k + j] = (double)__ldcg(&B.r[3 * (size_t)s + j]);
          ++nlc;
        }
        if (!grid_sync(A.gb, A.spin)) {
          if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
          return;
        }
        for (int i = tid; i < B.nb; i += nthr) {
          const int sc = X.scene_of[i];
          if (__ldcg(&X.done[sc]) || __ldcg(&M.mode[sc]) != 0) continue;
          double hl[3], ha[3], Ii[9], wa[3];
          gather_htr3(i, B.body_off, B.body_adj, A.C, A.r, hl, ha);
#pragma unroll
          for (int j = 0; j < 9; ++j) Ii[j] = A.Iinv[9 * (size_t)i + j];
          matvec3(Ii, ha, wa);
          const double mi = A.minv[i];
          const double* vl = B.v0 + 3 * (size_t)i;
          const double* va = B.v0 + 3 * (size_t)B.nb + 3 * (size_t)i;
          const double4_32a lv = make_double4_32a(vl[0] + mi * hl[0], vl[1] + mi * hl[1], vl[2] + mi * hl[2], 0.0);
          const double4_32a wv = make_double4_32a(va[0] + wa[0], va[1] + wa[1], va[2] + wa[2], 0.0);
          A.V[2 * i] = lv;
          A.V[2 * i + 1] = wv;
          B.V[2 * i] = make_float4((float)lv.x, (float)lv.y, (float)lv.z, 0.0f);
          B.V[2 * i + 1] = make_float4((float)wv.x, (float)wv.y, (float)wv.z, 0.0f);
          ++nlb;
        }
        if (!grid_sync(A.gb, A.spin)) {
          if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
          return;
        }
      }
      // FP64 residual and FP32-floor excess of every due scene (contacts are scene-major).
      const int slot = n_eval % 3;
      unsigned long long* eslots = X.err_slot + (size_t)slot * S;
      unsigned long long* xslots = M.exc_slot + (size_t)slot * S;
      const int lane = threadIdx.x & 31;
      for (int k0 = tid - lane; k0 < nc; k0 += nthr) {
        const int k = k0 + lane;
        int key = -1;
        unsigned long long ve = 0ull, vx = 0ull;
        if (k < nc) {
          const int a = A.C.ia[k], b = A.C.ib[k];
          const int sc = X.scene_of[a];
          const int md = __ldcg(&M.mode[sc]);
          if (!__ldcg(&X.done[sc]) && ((md == 0 && due32) || (md == 1 && due64))) {
            double E[9], Aa[6], Ab[6], u[3];
            load_contact(A.C, k, E, Aa, Ab);
            local_u3(A.C, k, A.V, u, a, b, E, Aa, Ab);
            const double rk[3] = {__ldcg(&A.r[3 * (size_t)k]), __ldcg(&A.r[3 * (size_t)k + 1]),
                                  __ldcg(&A.r[3 * (size_t)k + 2])};
            double* cand = bufs[1 - __ldcg(&X.bestbuf[sc])];
            cand[3 * (size_t)k] = rk[0];
            cand[3 * (size_t)k + 1] = rk[1];
            cand[3 * (size_t)k + 2] = rk[2];
            const double ek = fb_error_3d(rk, u, A.C.mu[k]);
            const double4_32a la = ld4cg(&A.V[2 * a]), wa = ld4cg(&A.V[2 * a + 1]);
            double scale = fabs(la.x) + fabs(la.y) + fabs(la.z) + fabs(wa.x) + fabs(wa.y) + fabs(wa.z);
            if (b >= 0) {
              const double4_32a lb = ld4cg(&A.V[2 * b]), wb = ld4cg(&A.V[2 * b + 1]);
              scale += fabs(lb.x) + fabs(lb.y) + fabs(lb.z) + fabs(wb.x) + fabs(wb.y) + fabs(wb.z);
            }
            scale += fabs(A.C.c[3 * (size_t)k]) + fabs(A.C.c[3 * (size_t)k + 1]) + fabs(A.C.c[3 * (size_t)k + 2]) +
                     fabs(rk[0]) + fabs(rk[1]) + fabs(rk[2]);
            ve = f64_to_ordered(ek);
            vx = f64_to_ordered(ek - 64.0 * 1.1920929e-7 * scale);
            key = sc;
            ++nev;
          }
        }
        run_max_atomic3(ve, key, eslots);
        run_max_atomic3(vx, key, xslots);
      }
      if (!grid_sync(A.gb, A.spin)) {
        if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
        return;
      }
      unsigned long long* enext = X.err_slot + (size_t)((n_eval + 1) % 3) * S;
      unsigned long long* xnext = M.exc_slot + (size_t)((n_eval + 1) % 3) * S;
      double gm = 0.0;
      for (int sc = tid; sc < S; sc += nthr) {
        enext[sc] = 0ull;
        xnext[sc] = 0ull;
        if (X.done[sc]) continue;
        const int md = M.mode[sc];
        if (!((md == 0 && due32) || (md == 1 && due64))) continue;
        const double err = ordered_to_f64(__ldcg(&eslots[sc]));
        const double exc = ordered_to_f64(__ldcg(&xslots[sc]));
        if (err < X.best[sc]) {
          X.best[sc] = err;
          X.bestbuf[sc] ^= 1;
          M.since[sc] = 0;
        } else {
          M.since[sc] += 1;
        }
        if (md == 1) {
          if (err < A.tol) {
            X.done[sc] = 1;
            X.iters[sc] = it;
            atomicAdd(X.done_count, 1);
            atomicSub(M.n64, 1);
          }
        } else {
          gm = nanmax(gm, err);
          if (err < A.tol || exc <= A.tol || (M.since[sc] >= 16 && exc <= 16.0 * A.tol)) {
            M.mode[sc] = 1;
            atomicAdd(M.n64, 1);
          }
        }
      }
      gm = block_nanmax(gm);
      if (threadIdx.x == 0 && due32) atomicMax(&M.gmax[slot], f64_to_ordered(gm));
      if (tid == 0) M.gmax[(n_eval + 1) % 3] = 0ull;
      ++n_eval;
      if (!grid_sync(A.gb, A.spin)) {
        if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
        return;
      }
      if (due32) {
        const double g = ordered_to_f64(*((volatile unsigned long long*)&M.gmax[slot]));
        if (it < eval32) {
          next_eval = 2 * it;
        } else {
          interval = (g > 1e3 * A.tol) ? min(2u * interval, 16u * eval32) : (g > 10.0 * A.tol ? interval : eval32);
          next_eval = it + interval;
        }
      }
      if (*((volatile int*)X.done_count) == S) break;
    }
  }
  for (int k = tid; k < nc; k += nthr) {
    const int sc = X.scene_of[A.C.ia[k]];
    if (__ldcg(&X.done[sc]) || !(__ldcg(&X.best[sc]) < INFINITY)) continue;
    const double* src = bufs[__ldcg(&X.bestbuf[sc])];
    for (int j = 0; j < 3; ++j) A.r[3 * (size_t)k + j] = __ldcg(&src[3 * (size_t)k + j]);
  }
  for (int sc = tid; sc < S; sc += nthr)
    if (!__ldcg(&X.done[sc])) X.iters[sc] = A.max_iters;
  if (tid == 0) *X.unconverged += (unsigned long long)(S - *((volatile int*)X.done_count));
  atomicAdd(&X.work[0], n32);
  atomicAdd(&X.work[1], n64);
  atomicAdd(&X.work[2], nev);
  atomicAdd(&X.work[3], nlc);
  atomicAdd(&X.work[4], nlb);
  if (tid == 0) {
    A.st->iterations = it > A.max_iters ? A.max_iters : it;
    A.st->evals = n_eval;
    A.st->converged = *((volatile int*)X.done_count) == S ? 1 : 0;
  }
}


// Assembly of caller-given sphere contacts (the FrictionSolver entry, sg_sobogus_solve_3d): the basis
// [n s t] (column-major, stored as the rows E), the angular rows r x s and r x t from the caller's arms,
// the forcing term with the map's extra relative velocities, the Delassus block and the warm start,
// in the arithmetic of k_assemble3 (SobogusFrictionProblem::initialize3D, Sobogus.cpp:184-251;
// Constraint::computeForcingTerm, scisim/Constraints/Constraint.cpp:18-34).
struct FsAssemble3 {
  int nb, nc;
  const int* ia;
  const int* ib;
  const double* bases;   // 9 per contact
  const double* arm_a;   // 3 per contact
  const double* arm_b;   // 3 per contact
  const double* v0;      // 6nb
  const double* minv;
  const double* Iinv;
  const double* CoR;
  const double* mu;
  const double* nrel;    // nc or null
  const double* drel;    // 2nc or null
  const double* alpha;   // nc
  const double* beta;    // 2nc
  double* E;
  double* Aa;
  double* Ab;
  double* c;
  double* W;
  double* mu_out;
  double* r;
};

__global__ void k_fs_assemble3(FsAssemble3 A) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= A.nc) return;
  const int nb = A.nb;
  const int a = A.ia[k], b = A.ib[k];
  const bool has_b = b >= 0;
  double n[3], s[3], t[3], ra[3], rb[3];
  const double* Bk = A.bases + 9 * (size_t)k;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    n[j] = Bk[j];
    s[j] = Bk[3 + j];
    t[j] = Bk[6 + j];
    ra[j] = A.arm_a[3 * (size_t)k + j];
    rb[j] = has_b ? A.arm_b[3 * (size_t)k + j] : 0.0;
  }
  double* E = A.E + 9 * (size_t)k;
#pragma unroll
  for (int j = 0; j < 9; ++j) E[j] = Bk[j];
  double as[3], at[3], bs[3] = {0.0, 0.0, 0.0}, bt[3] = {0.0, 0.0, 0.0};
  cross3(ra, s, as);
  cross3(ra, t, at);
  if (has_b) {
    cross3(rb, s, bs);
    cross3(rb, t, bt);
  }
  double* Aa = A.Aa + 6 * (size_t)k;
  double* Ab = A.Ab + 6 * (size_t)k;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    Aa[j] = as[j];
    Aa[3 + j] = at[j];
    Ab[j] = bs[j];
    Ab[3 + j] = bt[j];
  }
  // n . (v_a - v_b) on the linear velocities (the normal row has no angular part).
  double vr[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) vr[j] = A.v0[3 * (size_t)a + j] - (has_b ? A.v0[3 * (size_t)b + j] : 0.0);
  const double ndotv = dot3(n, vr);
  const double zero[3] = {0.0, 0.0, 0.0};
  double nrel = -dot3(zero, n);
  double drel0 = -dot3(zero, s), drel1 = -dot3(zero, t);
  if (A.nrel) nrel = nrel + A.nrel[k];
  if (A.drel) {
    drel0 = drel0 + A.drel[2 * (size_t)k];
    drel1 = drel1 + A.drel[2 * (size_t)k + 1];
  }
  const double sc = A.CoR[k] * ndotv + nrel;
  double w[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) w[j] = ((0.0 + n[j] * sc) + s[j] * drel0) + t[j] * drel1;
  A.c[3 * (size_t)k] = dot3(n, w);
  A.c[3 * (size_t)k + 1] = dot3(s, w);
  A.c[3 * (size_t)k + 2] = dot3(t, w);
  const double* B[3] = {n, s, t};
  const double* AaR[3] = {nullptr, as, at};
  const double* AbR[3] = {nullptr, bs, bt};
  double Ia[9], Ib[9];
#pragma unroll
  for (int j = 0; j < 9; ++j) Ia[j] = A.Iinv[9 * (size_t)a + j];
  if (has_b) {
#pragma unroll
    for (int j = 0; j < 9; ++j) Ib[j] = A.Iinv[9 * (size_t)b + j];
  }
  const double ma = A.minv[a], mb = has_b ? A.minv[b] : 0.0;
  double* Wk = A.W + 6 * (size_t)k;
  int q = 0;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = i; j < 3; ++j) {
      double wij = ma * dot3(B[i], B[j]);
      if (i > 0) {
        double x[3];
        matvec3(Ia, AaR[j], x);
        wij = wij + dot3(AaR[i], x);
      }
      if (has_b) {
        double wb = mb * dot3(B[i], B[j]);
        if (i > 0) {
          double x[3];
          matvec3(Ib, AbR[j], x);
          wb = wb + dot3(AbR[i], x);
        }
        wij = wij + wb;
      }
      Wk[q++] = wij;
    }
  A.mu_out[k] = A.mu[k];
  // Warm start r = alpha n + beta0 s + beta1 t, then local r = E^T r (Sobogus.cpp:514-518).
  const double al = A.alpha[k], b0 = A.beta[2 * (size_t)k], b1 = A.beta[2 * (size_t)k + 1];
  double rw[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) rw[j] = (al * n[j] + b0 * s[j]) + b1 * t[j];
  A.r[3 * (size_t)k] = dot3(n, rw);
  A.r[3 * (size_t)k + 1] = dot3(s, rw);
  A.r[3 * (size_t)k + 2] = dot3(t, rw);
  (void)nb;
}

}  // namespace

// ===========================================================================
int sphere3d_update_inertia(sg_ctx* ctx, bool construction) {
  const int nb = ctx->nb;
  if (nb <= 0) return SG_OK;
  k_inertia<<<blocks_for(nb), kBlock, 0, ctx->stream>>>(nb, ctx->q.as<double>(), ctx->I0.as<double>(),
                                                        ctx->Iw.as<double>(), ctx->Iinv.as<double>(),
                                                        construction ? 1 : 0);
  SG_CUDA_TRY(cudaGetLastError());
  return SG_OK;
}

static int ensure_contacts3(sg_ctx* ctx, int64_t nc) {
  if (nc <= ctx->ccap3 && ctx->E3.p) return SG_OK;
  const int64_t cap = std::max<int64_t>(nc + nc / 4 + 64, 1024);
  const size_t c = (size_t)cap;
  if (int r = grow(ctx->ia, sizeof(int) * c)) return r;
  if (int r = grow(ctx->ib, sizeof(int) * c)) return r;
  if (int r = grow(ctx->mu, sizeof(double) * c)) return r;
  if (int r = grow(ctx->E3, sizeof(double) * 9 * c)) return r;
  if (int r = grow(ctx->Aa3, sizeof(double) * 6 * c)) return r;
  if (int r = grow(ctx->Ab3, sizeof(double) * 6 * c)) return r;
  if (int r = grow(ctx->c3, sizeof(double) * 3 * c)) return r;
  if (int r = grow(ctx->W3, sizeof(double) * 6 * c)) return r;
  if (int r = grow(ctx->r3, sizeof(double) * 3 * c)) return r;
  if (int r = grow(ctx->r3a, sizeof(double) * 3 * c)) return r;
  if (int r = grow(ctx->r3b, sizeof(double) * 3 * c)) return r;
  if (int r = grow(ctx->ab3, sizeof(double) * 3 * c)) return r;
  ctx->ccap3 = cap;
  return SG_OK;
}

static int splitham(sg_ctx* ctx, const double* v0, bool with_aabb) {
  const int nb = ctx->nb;
  const double* g = ctx->cfg.gravity;
  k_splitham<<<blocks_for(nb), kBlock, 0, ctx->stream>>>(
      nb, ctx->cfg.dt, g[0], g[1], g[2], ctx->q.as<double>(), v0, ctx->m.as<double>(), ctx->I0.as<double>(),
      ctx->Iw.as<double>(), ctx->r.as<double>(), ctx->q1.as<double>(), ctx->v1.as<double>(),
      with_aabb ? ctx->aabb.as<double>() : nullptr);
  SG_CUDA_TRY(cudaGetLastError());
  return SG_OK;
}

// The block Gauss-Seidel solve of nc assembled sphere contacts (C, impulses rimp in local
// coordinates, in = start, out = result) over nb bodies (v0 6nb [v | omega], masses, world inertia
// and its inverse): running velocities, the FP64 or FP32+FP64 sweeps, v2 = M^-1 (H^T r - f) with
// f = -M v0, and (alpha, beta0, beta1) per contact into ab.  Fills ctx->h_stats and the work counters.
static int solve3_contacts(sg_ctx* ctx, int nb, int nc, const int* ia, const int* ib, const Contacts3& C, double* rimp,
                           const double* v0, const double* m, const double* minv, const double* Iw,
                           const double* Iinv, double* v2, double* ab, double tol, unsigned max_iters,
                           unsigned eval_every) {
  cudaStream_t s = ctx->stream;
  if (int r = ensure_solver_capacity(ctx, nb, nc)) return r;
  if (int r = grow(ctx->vrun3, sizeof(double4_32a) * 2 * (size_t)nb)) return r;
  if (int r = prepare_contact_graph(ctx, nb, nc, ia, ib)) return r;
  const int* off = ctx->body_off.as<int>();
  const int* adj = ctx->body_adj.as<int>();
  double4_32a* V = ctx->vrun3.as<double4_32a>();
  k_vel_init3<<<blocks_for(nb), kBlock, 0, s>>>(nb, off, adj, C, rimp, v0, minv, Iinv, V);
  SG_CUDA_TRY(cudaGetLastError());
  SolveStats* sst = ctx->stats.as<SolveStats>();
  GridBarrier* gb = ctx->barrier.as<GridBarrier>();
  SG_CUDA_TRY(cudaMemsetAsync(gb, 0, sizeof(GridBarrier), s));
  Gs3Args G;
  G.nc = nc;
  G.C = C;
  G.minv = minv;
  G.Iinv = Iinv;
  G.perm = ctx->perm.as<int>();
  G.r = rimp;
  G.r_a = ctx->r3a.as<double>();
  G.r_b = ctx->r3b.as<double>();
  G.V = V;
  G.st = sst;
  G.gb = gb;
  G.spin = ctx->spin_limit;
  G.tol = tol;
  G.max_iters = max_iters;
  G.eval_every = eval_every;
  if (ctx->cfg.precision == SG_PRECISION_FP32_REFINE) {
    const size_t c = (size_t)std::max(nc, 1), b1 = (size_t)std::max(nb, 1);
    if (int r = grow(ctx->pk_ab, sizeof(int2) * c)) return r;
    if (int r = grow(ctx->pk3, sizeof(float) * 31 * c)) return r;   // E 9, Aa 6, Ab 6, c 3, W 6, mu 1
    if (int r = grow(ctx->pk_r, sizeof(float) * 3 * c)) return r;
    if (int r = grow(ctx->v32, sizeof(float4) * 2 * b1)) return r;
    if (int r = grow(ctx->minv32, sizeof(float) * b1)) return r;
    if (int r = grow(ctx->Iinv32, sizeof(float) * 9 * b1)) return r;
    float* f = ctx->pk3.as<float>();
    Gs3m B;
    B.ab = ctx->pk_ab.as<int2>();
    B.E = f;
    B.Aa = f + 9 * c;
    B.Ab = f + 15 * c;
    B.c = f + 21 * c;
    B.W = f + 24 * c;
    B.mu = f + 30 * c;
    B.r = ctx->pk_r.as<float>();
    B.V = ctx->v32.as<float4>();
    B.minv = ctx->minv32.as<float>();
    B.Iinv = ctx->Iinv32.as<float>();
    B.v0 = v0;
    B.body_off = off;
    B.body_adj = adj;
    B.nb = nb;
    B.eval32 = (unsigned)ctx->check_interval;
    B.work = nullptr;
    k_pack3<<<blocks_for(nc), kBlock, 0, s>>>(nc, ctx->perm.as<int>(), C, rimp, B, B.r);
    k_body32<<<blocks_for(nb), kBlock, 0, s>>>(nb, V, minv, Iinv, B.V,
                                              const_cast<float*>(B.minv), const_cast<float*>(B.Iinv));
    SG_CUDA_TRY(cudaGetLastError());
    void* args[] = {&G, &B};
    const int grid = coop_grid(ctx, k_gs3_mixed, (long)ctx->num_sms * kGs3mBlock, kGs3mBlock, 1);
    if (ctx->profile) SG_CUDA_TRY(cudaEventRecord(ctx->ev_gs0, s));
    SG_CUDA_TRY(launch_cooperative((const void*)k_gs3_mixed, grid, kGs3mBlock, args, s));
    if (ctx->profile) SG_CUDA_TRY(cudaEventRecord(ctx->ev_gs1, s));
    ctx->kernel_launches += 2;
  } else {
    void* args[] = {&G};
    const int grid = coop_grid(ctx, k_gs3, (long)ctx->num_sms * kGs3Block, kGs3Block, 1);
    if (ctx->profile) SG_CUDA_TRY(cudaEventRecord(ctx->ev_gs0, s));
    SG_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_gs3, dim3(grid), dim3(kGs3Block), args, 0, s));
    if (ctx->profile) SG_CUDA_TRY(cudaEventRecord(ctx->ev_gs1, s));
  }
  k_final_vel3<<<blocks_for(nb), kBlock, 0, s>>>(nb, off, adj, C, rimp, v0, m, minv, Iw, Iinv, v2);
  k_extract3<<<blocks_for(nc), kBlock, 0, s>>>(nc, C.E, rimp, ab);
  SG_CUDA_TRY(cudaGetLastError());
  SG_CUDA_TRY(cudaMemcpyAsync(&ctx->h_stats, sst, sizeof(SolveStats), cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaStreamSynchronize(s));
  // vel init, gs, final velocity, extract
  ctx->kernel_launches += 4;
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
  ctx->contact_sweeps32 += (uint64_t)ctx->h_stats.sweeps32 * (uint64_t)nc;
  ctx->contact_evals += (uint64_t)ctx->h_stats.evals * (uint64_t)nc;
  ctx->contact_lifts += (uint64_t)ctx->h_stats.lifts * (uint64_t)nc;
  ctx->body_lifts += (uint64_t)ctx->h_stats.lifts * (uint64_t)nb;
  if (ctx->profile) {
    float ms = 0.f;
    SG_CUDA_TRY(cudaEventElapsedTime(&ms, ctx->ev_gs0, ctx->ev_gs1));
    ctx->gs_ms += ms;
  }
  return SG_OK;
}


// ---------------------------------------------------------------------------
// FrictionSolver::solve for spheres on host buffers (sg_sobogus_solve_3d).
static inline void h_cross3(const double* a, const double* b, double* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

int sobogus_solve_3d(sg_ctx* ctx, int nb, const double* m, const double* Iw, const double* Iinv, const double* v0,
                     int nc, const int* ia, const int* ib, const double* bases, const double* arm_a,
                     const double* arm_b, const double* CoR, const double* mu, const double* nrel_extra,
                     const double* drel_extra, unsigned max_iters, double tol, unsigned eval_every, double* alpha,
                     double* beta, double* v2, double* f, double* error, unsigned* iterations) {
  if (!ctx || nb < 0 || nc < 0 || (nb > 0 && (!m || !Iw || !Iinv || !v0 || !v2 || !f)) ||
      (nc > 0 && (!ia || !ib || !bases || !arm_a || !arm_b || !CoR || !mu || !alpha || !beta))) {
    set_error("sg_sobogus_solve_3d: invalid arguments");
    return SG_BAD_INPUT;
  }
  // The reference's invariants (asserts in Sobogus.cpp:497-512 and SphereSphereConstraint::evalH):
  // valid body indices, right-handed orthonormal bases, arms parallel to the normal.
  for (int k = 0; k < nc; ++k) {
    if (ia[k] < 0 || ia[k] >= nb || ib[k] >= nb || ib[k] == ia[k] || ib[k] < -1) {
      set_error("sg_sobogus_solve_3d: contact body index out of range");
      return SG_BAD_INPUT;
    }
    const double* E = bases + 9 * (size_t)k;
    double dev = 0.0;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        const double d = E[3 * i] * E[3 * j] + E[3 * i + 1] * E[3 * j + 1] + E[3 * i + 2] * E[3 * j + 2];
        dev = std::max(dev, std::fabs(d - (i == j ? 1.0 : 0.0)));
      }
    double nxs[3];
    h_cross3(E, E + 3, nxs);
    const double det = nxs[0] * E[6] + nxs[1] * E[7] + nxs[2] * E[8];
    double xa[3], xb[3] = {0.0, 0.0, 0.0};
    h_cross3(arm_a + 3 * (size_t)k, E, xa);
    if (ib[k] >= 0) h_cross3(arm_b + 3 * (size_t)k, E, xb);
    double par = 0.0;
    for (int j = 0; j < 3; ++j) par = std::max(par, std::max(std::fabs(xa[j]), std::fabs(xb[j])));
    if (!(dev <= 1.0e-6) || !(std::fabs(det - 1.0) <= 1.0e-6) || !(par <= 1.0e-6)) {
      set_error("sg_sobogus_solve_3d: basis not right-handed orthonormal or arm not parallel to the normal");
      return SG_BAD_INPUT;
    }
  }
  if (nc == 0) {
    for (int i = 0; i < 6 * nb; ++i) {
      v2[i] = v0[i];
      f[i] = 0.0;
    }
    if (error) *error = 0.0;
    if (iterations) *iterations = 0;
    ctx->last_nc = 0;
    return SG_OK;
  }
  SG_CUDA_TRY(cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  std::vector<double> minv(nb);
  for (int i = 0; i < nb; ++i) minv[i] = 1.0 / m[i];
  const size_t nbs = (size_t)nb, ncs = (size_t)nc;
  // Body data: m, minv, Iw, Iinv, v0, v2; contact inputs packed after each other.
  if (int r = grow(ctx->fs_m, sizeof(double) * nbs)) return r;
  if (int r = grow(ctx->fs_minv, sizeof(double) * nbs)) return r;
  if (int r = grow(ctx->fs_v0, sizeof(double) * 6 * nbs)) return r;
  if (int r = grow(ctx->fs_v2, sizeof(double) * 6 * nbs)) return r;
  if (int r = grow(ctx->fs_I, sizeof(double) * 18 * nbs)) return r;
  const size_t in_doubles = ncs * (9 + 3 + 3 + 1 + 1 + 1 + 2 + 1 + 2);
  if (int r = grow(ctx->fs_in, sizeof(double) * in_doubles)) return r;
  if (int r = ensure_contacts3(ctx, nc)) return r;
  double* dI = ctx->fs_I.as<double>();
  double* din = ctx->fs_in.as<double>();
  double* d_bases = din;
  double* d_arm_a = d_bases + 9 * ncs;
  double* d_arm_b = d_arm_a + 3 * ncs;
  double* d_CoR = d_arm_b + 3 * ncs;
  double* d_mu = d_CoR + ncs;
  double* d_nrel = d_mu + ncs;
  double* d_drel = d_nrel + ncs;
  double* d_alpha = d_drel + 2 * ncs;
  double* d_beta = d_alpha + ncs;
  SG_CUDA_TRY(cudaMemcpyAsync(ctx->fs_m.p, m, sizeof(double) * nbs, cudaMemcpyHostToDevice, s));
  SG_CUDA_TRY(cudaMemcpyAsync(ctx->fs_minv.p, minv.data(), sizeof(double) * nbs, cudaMemcpyHostToDevice, s));
  SG_CUDA_TRY(cudaMemcpyAsync(ctx->fs_v0.p, v0, sizeof(double) * 6 * nbs, cudaMemcpyHostToDevice, s));
  SG_CUDA_TRY(cudaMemcpyAsync(dI, Iw, sizeof(double) * 9 * nbs, cudaMemcpyHostToDevice, s));
  SG_CUDA_TRY(cudaMemcpyAsync(dI + 9 * nbs, Iinv, sizeof(double) * 9 * nbs, cudaMemcpyHostToDevice, s));
  SG_CUDA_TRY(cudaMemcpyAsync(ctx->ia.p, ia, sizeof(int) * ncs, cudaMemcpyHostToDevice, s));
  SG_CUDA_TRY(cudaMemcpyAsync(ctx->ib.p, ib, sizeof(int) * ncs, cudaMemcpyHostToDevice, s));
  SG_CUDA_TRY(cudaMemcpyAsync(d_bases, bases, sizeof(double) * 9 * ncs, cudaMemcpyHostToDevice, s));
  SG_CUDA_TRY(cudaMemcpyAsync(d_arm_a, arm_a, sizeof(double) * 3 * ncs, cudaMemcpyHostToDevice, s));
  SG_CUDA_TRY(cudaMemcpyAsync(d_arm_b, arm_b, sizeof(double) * 3 * ncs, cudaMemcpyHostToDevice, s));
  SG_CUDA_TRY(cudaMemcpyAsync(d_CoR, CoR, sizeof(double) * ncs, cudaMemcpyHostToDevice, s));
  SG_CUDA_TRY(cudaMemcpyAsync(d_mu, mu, sizeof(double) * ncs, cudaMemcpyHostToDevice, s));
  if (nrel_extra) SG_CUDA_TRY(cudaMemcpyAsync(d_nrel, nrel_extra, sizeof(double) * ncs, cudaMemcpyHostToDevice, s));
  if (drel_extra)
    SG_CUDA_TRY(cudaMemcpyAsync(d_drel, drel_extra, sizeof(double) * 2 * ncs, cudaMemcpyHostToDevice, s));
  SG_CUDA_TRY(cudaMemcpyAsync(d_alpha, alpha, sizeof(double) * ncs, cudaMemcpyHostToDevice, s));
  SG_CUDA_TRY(cudaMemcpyAsync(d_beta, beta, sizeof(double) * 2 * ncs, cudaMemcpyHostToDevice, s));
  FsAssemble3 A;
  A.nb = nb;
  A.nc = nc;
  A.ia = ctx->ia.as<int>();
  A.ib = ctx->ib.as<int>();
  A.bases = d_bases;
  A.arm_a = d_arm_a;
  A.arm_b = d_arm_b;
  A.v0 = ctx->fs_v0.as<double>();
  A.minv = ctx->fs_minv.as<double>();
  A.Iinv = dI + 9 * nbs;
  A.CoR = d_CoR;
  A.mu = d_mu;
  A.nrel = nrel_extra ? d_nrel : nullptr;
  A.drel = drel_extra ? d_drel : nullptr;
  A.alpha = d_alpha;
  A.beta = d_beta;
  A.E = ctx->E3.as<double>();
  A.Aa = ctx->Aa3.as<double>();
  A.Ab = ctx->Ab3.as<double>();
  A.c = ctx->c3.as<double>();
  A.W = ctx->W3.as<double>();
  A.mu_out = ctx->mu.as<double>();
  A.r = ctx->r3.as<double>();
  k_fs_assemble3<<<blocks_for(nc), kBlock, 0, s>>>(A);
  SG_CUDA_TRY(cudaGetLastError());
  ctx->kernel_launches += 1;
  const Contacts3 C{A.ia, A.ib, A.E, A.Aa, A.Ab, A.c, A.W, A.mu_out};
  const int sr = solve3_contacts(ctx, nb, nc, A.ia, A.ib, C, A.r, A.v0, ctx->fs_m.as<double>(), A.minv, dI, A.Iinv,
                                 ctx->fs_v2.as<double>(), ctx->ab3.as<double>(), tol, max_iters,
                                 eval_every == 0 ? 1u : eval_every);
  if (sr != SG_OK) return sr;
  ctx->last_nc = nc;
  std::vector<double> ab(3 * ncs), E(9 * ncs);
  SG_CUDA_TRY(cudaMemcpyAsync(v2, ctx->fs_v2.p, sizeof(double) * 6 * nbs, cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaMemcpyAsync(ab.data(), ctx->ab3.p, sizeof(double) * 3 * ncs, cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaStreamSynchronize(s));
  // alpha, beta and the friction impulse with its torque, in contact order (Sobogus.cpp:533-567).
  for (size_t i = 0; i < 6 * nbs; ++i) f[i] = 0.0;
  for (int k = 0; k < nc; ++k) {
    const double* Bk = bases + 9 * (size_t)k;
    const double* sv = Bk + 3;
    const double* tv = Bk + 6;
    alpha[k] = ab[3 * (size_t)k];
    const double b0 = ab[3 * (size_t)k + 1], b1 = ab[3 * (size_t)k + 2];
    beta[2 * (size_t)k] = b0;
    beta[2 * (size_t)k + 1] = b1;
    double as[3], at[3];
    h_cross3(arm_a + 3 * (size_t)k, sv, as);
    h_cross3(arm_a + 3 * (size_t)k, tv, at);
    const int a = ia[k], b = ib[k];
    for (int j = 0; j < 3; ++j) {
      const double f0 = b0 * sv[j] + b1 * tv[j];
      const double ta = b0 * as[j] + b1 * at[j];
      f[3 * (size_t)a + j] += f0;
      f[3 * nbs + 3 * (size_t)a + j] += ta;
      if (b >= 0) {
        double bs[3], bt[3];
        h_cross3(arm_b + 3 * (size_t)k, sv, bs);
        h_cross3(arm_b + 3 * (size_t)k, tv, bt);
        const double tb = b0 * bs[j] + b1 * bt[j];
        f[3 * (size_t)b + j] -= f0;
        f[3 * nbs + 3 * (size_t)b + j] -= tb;
      }
    }
  }
  if (error) *error = ctx->h_stats.error;
  if (iterations) *iterations = ctx->h_stats.iterations;
  return ctx->h_stats.converged ? SG_OK : SG_NOT_CONVERGED;
}

// One GeometricImpactFrictionMap::flow step of a sphere scene (cache forced NONE in 3D:
// rigidbody3dutils/RigidBody3DSceneParser.cpp:1877-1880), then updateMandMinv.
int sphere3d_step(sg_ctx* ctx, sg_step_stats* out) {
  const int nb = ctx->nb, np = ctx->np;
  cudaStream_t s = ctx->stream;
  sg_step_stats st{};
  const bool se = ctx->staggering == SG_STAGGER_SYMPLECTIC_EULER;
  if (ctx->staggering == SG_STAGGER_STABILIZED) {
    set_error("sphere scenes step with the geometric or the symplectic Euler staggering");
    return SG_BAD_INPUT;
  }
  if (se && ctx->cfg.CoR != 0.0) {
    set_error("the symplectic Euler staggering needs CoR = 0");
    return SG_BAD_INPUT;
  }
  if (nb == 0) {
    if (out) *out = st;
    return SG_OK;
  }
  // Predictor and q1 AABBs: the unconstrained map (geometric staggering), or vdelta and the
  // exponential-Euler predictor (symplectic Euler).
  if (se) {
    if (int r = grow(ctx->vdelta, sizeof(double) * 6 * (size_t)nb)) return r;
    const double* g = ctx->cfg.gravity;
    k_se3_predict<<<blocks_for(nb), kBlock, 0, s>>>(nb, ctx->cfg.dt, g[0], g[1], g[2], ctx->q.as<double>(),
                                                    ctx->v.as<double>(), ctx->m.as<double>(), ctx->Iinv.as<double>(),
                                                    ctx->r.as<double>(), ctx->vdelta.as<double>(), ctx->q1.as<double>(),
                                                    ctx->aabb.as<double>());
    SG_CUDA_TRY(cudaGetLastError());
  } else if (int r = splitham(ctx, ctx->v.as<double>(), true)) {
    return r;
  }
  // Grid.
  const long cap = 4L * nb + 64;
  if (int r = grow(ctx->grid, sizeof(Grid3))) return r;
  if (int r = grow(ctx->cell_count, sizeof(int) * (size_t)(cap + 1))) return r;
  if (int r = grow(ctx->cell_start, sizeof(int) * (size_t)(cap + 1))) return r;
  if (int r = grow(ctx->cell_fill, sizeof(int) * (size_t)(cap + 1))) return r;
  if (int r = grow(ctx->cell_of, sizeof(int) * (size_t)nb)) return r;
  if (int r = grow(ctx->sorted, sizeof(int) * (size_t)nb)) return r;
  if (int r = grow(ctx->pair_cnt, sizeof(int) * (size_t)(nb + 1))) return r;
  if (int r = grow(ctx->pair_off, sizeof(int) * (size_t)(nb + 1))) return r;
  Grid3* g = ctx->grid.as<Grid3>();
  const double* aabb = ctx->aabb.as<double>();
  k_bounds3_init<<<1, 1, 0, s>>>(g);
  k_bounds3<<<std::max(1, std::min(blocks_for(nb), ctx->num_sms * 8)), kBlock, 0, s>>>(nb, aabb, g);
  k_grid3_setup<<<1, 1, 0, s>>>(g, cap);
  SG_CUDA_TRY(cudaMemsetAsync(ctx->cell_count.p, 0, sizeof(int) * (size_t)(cap + 1), s));
  SG_CUDA_TRY(cudaMemsetAsync(ctx->cell_fill.p, 0, sizeof(int) * (size_t)(cap + 1), s));
  k_cell_count3<<<blocks_for(nb), kBlock, 0, s>>>(nb, aabb, g, ctx->cell_of.as<int>(), ctx->cell_count.as<int>());
  SG_CUDA_TRY(cudaGetLastError());
  if (int r = scan_exclusive(ctx, ctx->cell_count.as<int>(), ctx->cell_start.as<int>(), (int)cap)) return r;
  k_cell_scatter3<<<blocks_for(nb), kBlock, 0, s>>>(nb, ctx->cell_of.as<int>(), ctx->cell_start.as<int>(),
                                                   ctx->cell_fill.as<int>(), ctx->sorted.as<int>());
  Scan3 sc{aabb, g, ctx->cell_start.as<int>(), ctx->sorted.as<int>(), ctx->q1.as<double>(), ctx->r.as<double>(),
           nullptr, nullptr};
  k_pair_count3<<<blocks_for(nb), kBlock, 0, s>>>(nb, sc, ctx->pair_cnt.as<int>());
  SG_CUDA_TRY(cudaGetLastError());
  if (int r = scan_exclusive(ctx, ctx->pair_cnt.as<int>(), ctx->pair_off.as<int>(), nb)) return r;
  // Planes.
  const long t = (long)nb * np;
  if (int r = grow(ctx->plane_flag, sizeof(int) * (size_t)(t + 1))) return r;
  if (int r = grow(ctx->plane_off, sizeof(int) * (size_t)(t + 1))) return r;
  if (t > 0) {
    k_plane_flags3<<<blocks_for(t), kBlock, 0, s>>>(nb, np, ctx->q1.as<double>(), ctx->r.as<double>(),
                                                    ctx->plane_x.as<double>(), ctx->plane_n.as<double>(),
                                                    ctx->plane_flag.as<int>());
    SG_CUDA_TRY(cudaGetLastError());
    if (int r = scan_exclusive(ctx, ctx->plane_flag.as<int>(), ctx->plane_off.as<int>(), (int)t)) return r;
  } else {
    SG_CUDA_TRY(cudaMemsetAsync(ctx->plane_off.p, 0, sizeof(int), s));
  }
  int totals[2] = {0, 0};
  SG_CUDA_TRY(cudaMemcpyAsync(&totals[0], ctx->pair_off.as<int>() + nb, sizeof(int), cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaMemcpyAsync(&totals[1], ctx->plane_off.as<int>() + t, sizeof(int), cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaStreamSynchronize(s));
  const int npairs = totals[0], nplanes = totals[1];
  const int nc = npairs + nplanes;
  // splitham 1, bounds 3, cell count 1, scan 3, scatter 1, pair count 1, scan 3, planes 1 + 3
  ctx->kernel_launches += 14 + (t > 0 ? 4 : 0);
  ctx->steps += 1;
  ctx->contacts_total += (uint64_t)nc;
  st.n_contacts = nc;
  st.n_ball_ball = npairs;
  st.n_ball_plane = nplanes;
  ctx->last_nc = nc;
  ctx->last_nbb = npairs;
  if (nc == 0) {
    if (se) {
      // No active constraint: v1 = v0 + vdelta, the configuration from v1; the cache empties.
      k_se3_final<<<blocks_for(nb), kBlock, 0, s>>>(nb, ctx->cfg.dt, ctx->q.as<double>(), ctx->v.as<double>(),
                                                    ctx->vdelta.as<double>(), ctx->q1.as<double>(),
                                                    ctx->v1.as<double>());
      SG_CUDA_TRY(cudaGetLastError());
      ctx->prev_n = 0;
      ctx->prev_rows = false;
      ctx->prev_color_valid = false;
      ctx->kernel_launches += 1;
    }
    std::swap(ctx->q, ctx->q1);
    std::swap(ctx->v, ctx->v1);
    if (int r = sphere3d_update_inertia(ctx, false)) return r;
    ctx->kernel_launches += 1;
    st.succeeded = 1;
    if (out) *out = st;
    return SG_OK;
  }
  if (int r = ensure_contacts3(ctx, nc)) return r;
  int* ia = ctx->ia.as<int>();
  int* ib = ctx->ib.as<int>();
  k_pair_write3<<<blocks_for(nb), kBlock, 0, s>>>(nb, sc, ctx->pair_off.as<int>(), ia, ib);
  if (t > 0)
    k_plane_write3<<<blocks_for(t), kBlock, 0, s>>>(nb, np, npairs, ctx->plane_flag.as<int>(),
                                                    ctx->plane_off.as<int>(), ia, ib);
  SG_CUDA_TRY(cudaGetLastError());
  Assemble3 A;
  A.nb = nb;
  A.nc = nc;
  A.ia = ia;
  A.ib = ib;
  A.q0 = ctx->q.as<double>();
  A.v0 = ctx->v.as<double>();
  A.rad = ctx->r.as<double>();
  A.minv = ctx->minv.as<double>();
  A.Iinv = ctx->Iinv.as<double>();
  A.plane_n = ctx->plane_n.as<double>();
  A.mu = ctx->cfg.mu;
  A.CoR = ctx->cfg.CoR;
  A.scene_of = nullptr;
  A.s_mu = A.s_CoR = nullptr;
  A.E = ctx->E3.as<double>();
  A.Aa = ctx->Aa3.as<double>();
  A.Ab = ctx->Ab3.as<double>();
  A.c = ctx->c3.as<double>();
  A.W = ctx->W3.as<double>();
  A.mu_out = ctx->mu.as<double>();
  A.r = ctx->r3.as<double>();
  if (se) {
    const size_t c = (size_t)nc;
    if (int r = grow(ctx->key, sizeof(unsigned long long) * c)) return r;
    if (int r = grow(ctx->c6, sizeof(double) * 6 * c)) return r;
    A.vdelta = ctx->vdelta.as<double>();
    A.plane_x = ctx->plane_x.as<double>();
    A.dt = ctx->cfg.dt;
    A.stabilize = ctx->stabilize;
    A.pen_thresh = ctx->pen_thresh;
    A.cache_mode = ctx->cfg.cache_mode;
    A.prev_key = ctx->prev_key.as<unsigned long long>();
    A.prev_c6 = ctx->prev_c6.as<double>();
    A.prev_n = (int)ctx->prev_n;
    A.key = ctx->key.as<unsigned long long>();
  }
  k_assemble3<<<blocks_for(nc), kBlock, 0, s>>>(A);
  SG_CUDA_TRY(cudaGetLastError());

  // Solve.
  if (int r = grow(ctx->v2, sizeof(double) * 6 * (size_t)nb)) return r;
  const Contacts3 C{ia, ib, A.E, A.Aa, A.Ab, A.c, A.W, A.mu_out};
  // pair write, plane write, assemble
  ctx->kernel_launches += 2 + (t > 0 ? 1 : 0);
  if (int r = solve3_contacts(ctx, nb, nc, ia, ib, C, A.r, ctx->v.as<double>(), ctx->m.as<double>(),
                              ctx->minv.as<double>(), ctx->Iw.as<double>(), ctx->Iinv.as<double>(),
                              ctx->v2.as<double>(), ctx->ab3.as<double>(), ctx->cfg.tol, ctx->cfg.max_iters,
                              ctx->cfg.eval_every))
    return r;
  st.iterations = ctx->h_stats.iterations;
  st.succeeded = ctx->h_stats.converged;
  st.error = ctx->h_stats.error;
  st.n_colors = (uint32_t)ctx->h_stats.n_colors;
  if (se) {
    // Impulses into the cache, v1 = v2 + vdelta and the configuration from v1.
    if (ctx->cfg.cache_mode != SG_CACHE_NONE) {
      k_cache3<<<blocks_for(nc), kBlock, 0, s>>>(nc, ctx->cfg.cache_mode, A.E, ctx->ab3.as<double>(),
                                                 ctx->c6.as<double>());
      SG_CUDA_TRY(cudaGetLastError());
      std::swap(ctx->key, ctx->prev_key);
      std::swap(ctx->c6, ctx->prev_c6);
      ctx->prev_n = nc;
      ctx->prev_rows = false;
      ctx->prev_color_valid = false;
      ctx->kernel_launches += 1;
    } else {
      ctx->prev_n = 0;
      ctx->prev_rows = false;
      ctx->prev_color_valid = false;
    }
    k_se3_final<<<blocks_for(nb), kBlock, 0, s>>>(nb, ctx->cfg.dt, ctx->q.as<double>(), ctx->v2.as<double>(),
                                                  ctx->vdelta.as<double>(), ctx->q1.as<double>(), ctx->v1.as<double>());
    SG_CUDA_TRY(cudaGetLastError());
  } else if (int r = splitham(ctx, ctx->v2.as<double>(), false)) {
    return r;
  }
  std::swap(ctx->q, ctx->q1);
  std::swap(ctx->v, ctx->v1);
  if (int r = sphere3d_update_inertia(ctx, false)) return r;
  ctx->kernel_launches += 2;
  if (out) *out = st;
  return st.succeeded ? SG_OK : SG_NOT_CONVERGED;
}

// ---------------------------------------------------------------------------
// Batched sphere scenes (sg_sphere3d_batch_upload): buffers, and one step of every scene.
int sphere3d_batch_setup(sg_ctx* ctx, long flags, long cells) {
  const int S = ctx->n_scenes, N = ctx->nb;
  const size_t s1 = sizeof(int) * (size_t)(S + 1), nbs = (size_t)std::max(N, 1);
  Buf* ints_s1[] = {&ctx->s_cells, &ctx->s_cell_off, &ctx->s_nc, &ctx->s_npairs, &ctx->sc_off, &ctx->prev_sc_off,
                    &ctx->s_bestbuf, &ctx->s_done, &ctx->s_iters};
  for (Buf* b : ints_s1)
    if (int e = grow(*b, s1)) return e;
  if (int e = grow(ctx->s_grid, sizeof(Grid3) * (size_t)S)) return e;
  if (int e = grow(ctx->s_best, sizeof(double) * (size_t)S)) return e;
  if (int e = grow(ctx->s_err, sizeof(unsigned long long) * 3 * (size_t)S)) return e;
  if (int e = grow(ctx->b_ctl, 4 * sizeof(int))) return e;
  if (int e = grow(ctx->b_sums, 4 * sizeof(unsigned long long))) return e;
  if (int e = grow(ctx->b_work, 5 * sizeof(unsigned long long))) return e;
  if (int e = grow(ctx->cell_count, sizeof(int) * (size_t)(cells + 1))) return e;
  if (int e = grow(ctx->cell_start, sizeof(int) * (size_t)(cells + 1))) return e;
  if (int e = grow(ctx->cell_fill, sizeof(int) * (size_t)(cells + 1))) return e;
  if (int e = grow(ctx->cell_of, sizeof(int) * nbs)) return e;
  if (int e = grow(ctx->sorted, sizeof(int) * nbs)) return e;
  if (int e = grow(ctx->pair_cnt, sizeof(int) * (nbs + 1))) return e;
  if (int e = grow(ctx->pair_off, sizeof(int) * (nbs + 1))) return e;
  if (int e = grow(ctx->plane_flag, sizeof(int) * (size_t)(flags + 1))) return e;
  if (int e = grow(ctx->plane_off, sizeof(int) * (size_t)(flags + 1))) return e;
  SG_CUDA_TRY(cudaMemsetAsync(ctx->sc_off.p, 0, s1, ctx->stream));
  SG_CUDA_TRY(cudaMemsetAsync(ctx->b_sums.p, 0, 4 * sizeof(unsigned long long), ctx->stream));
  return SG_OK;
}

int sphere3d_batch_step(sg_ctx* ctx, sg_step_stats* out) {
  const int N = ctx->nb, S = ctx->n_scenes;
  cudaStream_t s = ctx->stream;
  sg_step_stats st{};
  if (int r = splitham(ctx, ctx->v.as<double>(), true)) return r;
  const double* aabb = ctx->aabb.as<double>();
  const int* sb_off = ctx->sb_off.as<int>();
  const int* sp_off = ctx->sp_off.as<int>();
  const int* sf_off = ctx->sf_off.as<int>();
  const int* scene_of = ctx->scene_of.as<int>();
  Grid3* grids = ctx->s_grid.as<Grid3>();
  // Per-scene grids, cells, pairs and planes.
  k_scene_grid3<<<S, kBlock, 0, s>>>(sb_off, aabb, grids, ctx->s_cells.as<int>());
  SG_CUDA_TRY(cudaGetLastError());
  if (int r = scan_exclusive(ctx, ctx->s_cells.as<int>(), ctx->s_cell_off.as<int>(), S)) return r;
  SG_CUDA_TRY(cudaMemsetAsync(ctx->cell_count.p, 0, sizeof(int) * (size_t)(ctx->bcells + 1), s));
  SG_CUDA_TRY(cudaMemsetAsync(ctx->cell_fill.p, 0, sizeof(int) * (size_t)(ctx->bcells + 1), s));
  k_cell_count3_b<<<blocks_for(N), kBlock, 0, s>>>(N, scene_of, aabb, grids, ctx->s_cell_off.as<int>(),
                                                  ctx->cell_of.as<int>(), ctx->cell_count.as<int>());
  SG_CUDA_TRY(cudaGetLastError());
  if (int r = scan_exclusive(ctx, ctx->cell_count.as<int>(), ctx->cell_start.as<int>(), (int)ctx->bcells)) return r;
  k_cell_scatter3<<<blocks_for(N), kBlock, 0, s>>>(N, ctx->cell_of.as<int>(), ctx->cell_start.as<int>(),
                                                  ctx->cell_fill.as<int>(), ctx->sorted.as<int>());
  Scan3 sc{aabb, grids, ctx->cell_start.as<int>(), ctx->sorted.as<int>(), ctx->q1.as<double>(), ctx->r.as<double>(),
           scene_of, ctx->s_cell_off.as<int>()};
  k_pair_count3<<<blocks_for(N), kBlock, 0, s>>>(N, sc, ctx->pair_cnt.as<int>());
  SG_CUDA_TRY(cudaGetLastError());
  if (int r = scan_exclusive(ctx, ctx->pair_cnt.as<int>(), ctx->pair_off.as<int>(), N)) return r;
  if (ctx->bflags > 0) {
    k_plane_flags3_b<<<blocks_for(N), kBlock, 0, s>>>(N, scene_of, sb_off, sp_off, sf_off, ctx->q1.as<double>(),
                                                     ctx->r.as<double>(), ctx->plane_x.as<double>(),
                                                     ctx->plane_n.as<double>(), ctx->plane_flag.as<int>());
    SG_CUDA_TRY(cudaGetLastError());
    if (int r = scan_exclusive(ctx, ctx->plane_flag.as<int>(), ctx->plane_off.as<int>(), (int)ctx->bflags)) return r;
  } else {
    SG_CUDA_TRY(cudaMemsetAsync(ctx->plane_off.p, 0, sizeof(int), s));
  }
  k_scene_counts3<<<blocks_for(S), kBlock, 0, s>>>(S, sb_off, sf_off, ctx->pair_off.as<int>(),
                                                  ctx->plane_off.as<int>(), ctx->s_nc.as<int>(),
                                                  ctx->s_npairs.as<int>());
  SG_CUDA_TRY(cudaGetLastError());
  if (int r = scan_exclusive(ctx, ctx->s_nc.as<int>(), ctx->sc_off.as<int>(), S)) return r;
  int totals[2] = {0, 0};
  SG_CUDA_TRY(cudaMemcpyAsync(&totals[0], ctx->sc_off.as<int>() + S, sizeof(int), cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaMemcpyAsync(&totals[1], ctx->pair_off.as<int>() + N, sizeof(int), cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaStreamSynchronize(s));
  const int nc = totals[0], npairs = totals[1];
  // splitham 1, scene grid 1 + scan 3, cell count 1 + scan 3, scatter 1, pair count 1 + scan 3,
  // planes 1 + scan 3, scene counts 1 + scan 3
  ctx->kernel_launches += 19 + (ctx->bflags > 0 ? 4 : 0);
  ctx->steps += 1;
  ctx->contacts_total += (uint64_t)nc;
  st.n_contacts = nc;
  st.n_ball_ball = npairs;
  st.n_ball_plane = nc - npairs;
  ctx->last_nc = nc;
  ctx->last_nbb = npairs;
  if (nc == 0) {
    k_fill_int<<<blocks_for(S), kBlock, 0, s>>>(S, 1, ctx->s_done.as<int>());
    SG_CUDA_TRY(cudaMemsetAsync(ctx->s_iters.p, 0, sizeof(unsigned) * (size_t)S, s));
    std::swap(ctx->q, ctx->q1);
    std::swap(ctx->v, ctx->v1);
    if (int r = sphere3d_update_inertia(ctx, false)) return r;
    ctx->kernel_launches += 2;
    SG_CUDA_TRY(cudaStreamSynchronize(s));
    st.succeeded = 1;
    if (out) *out = st;
    return SG_OK;
  }
  if (int r = ensure_contacts3(ctx, nc)) return r;
  int* ia = ctx->ia.as<int>();
  int* ib = ctx->ib.as<int>();
  const int* sc_off = ctx->sc_off.as<int>();
  k_pair_write3_b<<<blocks_for(N), kBlock, 0, s>>>(N, sc, sb_off, ctx->pair_off.as<int>(), sc_off, ia, ib);
  if (ctx->bflags > 0)
    k_plane_write3_b<<<blocks_for(N), kBlock, 0, s>>>(N, scene_of, sb_off, sp_off, sf_off, ctx->plane_flag.as<int>(),
                                                     ctx->plane_off.as<int>(), sc_off, ctx->s_npairs.as<int>(), ia, ib);
  SG_CUDA_TRY(cudaGetLastError());
  Assemble3 A;
  A.nb = N;
  A.nc = nc;
  A.ia = ia;
  A.ib = ib;
  A.q0 = ctx->q.as<double>();
  A.v0 = ctx->v.as<double>();
  A.rad = ctx->r.as<double>();
  A.minv = ctx->minv.as<double>();
  A.Iinv = ctx->Iinv.as<double>();
  A.plane_n = ctx->plane_n.as<double>();
  A.mu = ctx->cfg.mu;
  A.CoR = ctx->cfg.CoR;
  A.scene_of = scene_of;
  A.s_mu = ctx->s_mu.as<double>();
  A.s_CoR = ctx->s_CoR.as<double>();
  A.E = ctx->E3.as<double>();
  A.Aa = ctx->Aa3.as<double>();
  A.Ab = ctx->Ab3.as<double>();
  A.c = ctx->c3.as<double>();
  A.W = ctx->W3.as<double>();
  A.mu_out = ctx->mu.as<double>();
  A.r = ctx->r3.as<double>();
  k_assemble3<<<blocks_for(nc), kBlock, 0, s>>>(A);
  SG_CUDA_TRY(cudaGetLastError());
  // Solve every scene to its own tolerance (FP64).
  if (int r = ensure_solver_capacity(ctx, N, nc)) return r;
  if (int r = grow(ctx->vrun3, sizeof(double4_32a) * 2 * (size_t)N)) return r;
  if (int r = grow(ctx->v2, sizeof(double) * 6 * (size_t)N)) return r;
  if (int r = prepare_contact_graph(ctx, N, nc, ia, ib)) return r;
  const int* off = ctx->body_off.as<int>();
  const int* adj = ctx->body_adj.as<int>();
  Contacts3 C{ia, ib, A.E, A.Aa, A.Ab, A.c, A.W, A.mu_out};
  double4_32a* V = ctx->vrun3.as<double4_32a>();
  k_vel_init3<<<blocks_for(N), kBlock, 0, s>>>(N, off, adj, C, A.r, ctx->v.as<double>(), ctx->minv.as<double>(),
                                               ctx->Iinv.as<double>(), V);
  SG_CUDA_TRY(cudaGetLastError());
  SolveStats* sst = ctx->stats.as<SolveStats>();
  GridBarrier* gb = ctx->barrier.as<GridBarrier>();
  SG_CUDA_TRY(cudaMemsetAsync(gb, 0, sizeof(GridBarrier), s));
  SG_CUDA_TRY(cudaMemsetAsync(ctx->s_err.p, 0, sizeof(unsigned long long) * 3 * (size_t)S, s));
  SG_CUDA_TRY(cudaMemsetAsync(ctx->b_ctl.p, 0, 4 * sizeof(int), s));
  SG_CUDA_TRY(cudaMemsetAsync(ctx->b_work.p, 0, 5 * sizeof(unsigned long long), s));
  Gs3BatchArgs B;
  B.g.nc = nc;
  B.g.C = C;
  B.g.minv = ctx->minv.as<double>();
  B.g.Iinv = ctx->Iinv.as<double>();
  B.g.perm = ctx->perm.as<int>();
  B.g.r = A.r;
  B.g.r_a = ctx->r3a.as<double>();
  B.g.r_b = ctx->r3b.as<double>();
  B.g.V = V;
  B.g.st = sst;
  B.g.gb = gb;
  B.g.spin = ctx->spin_limit;
  B.g.tol = ctx->cfg.tol;
  B.g.max_iters = ctx->cfg.max_iters;
  B.g.eval_every = ctx->cfg.eval_every;
  B.scene_of = scene_of;
  B.sc_off = sc_off;
  B.S = S;
  B.err_slot = ctx->s_err.as<unsigned long long>();
  B.best = ctx->s_best.as<double>();
  B.bestbuf = ctx->s_bestbuf.as<int>();
  B.done = ctx->s_done.as<int>();
  B.iters = ctx->s_iters.as<unsigned>();
  B.done_count = ctx->b_ctl.as<int>();
  B.unconverged = ctx->b_sums.as<unsigned long long>() + 1;
  B.work = ctx->b_work.as<unsigned long long>();
  if (ctx->cfg.precision == SG_PRECISION_FP32_REFINE) {
    // FP32 sweeps with FP64 refinement, scene by scene.
    const size_t c = (size_t)std::max(nc, 1), b1 = (size_t)std::max(N, 1);
    if (int r = grow(ctx->pk_ab, sizeof(int2) * c)) return r;
    if (int r = grow(ctx->pk3, sizeof(float) * 31 * c)) return r;   // E 9, Aa 6, Ab 6, c 3, W 6, mu 1
    if (int r = grow(ctx->pk_r, sizeof(float) * 3 * c)) return r;
    if (int r = grow(ctx->v32, sizeof(float4) * 2 * b1)) return r;
    if (int r = grow(ctx->minv32, sizeof(float) * b1)) return r;
    if (int r = grow(ctx->Iinv32, sizeof(float) * 9 * b1)) return r;
    if (int r = grow(ctx->s_mode, sizeof(int) * (size_t)S)) return r;
    if (int r = grow(ctx->s_since, sizeof(unsigned) * (size_t)S)) return r;
    if (int r = grow(ctx->s_exc, sizeof(unsigned long long) * 3 * (size_t)S)) return r;
    if (int r = grow(ctx->s_gmax, sizeof(unsigned long long) * 3)) return r;
    float* f = ctx->pk3.as<float>();
    Gs3m P;
    P.ab = ctx->pk_ab.as<int2>();
    P.E = f;
    P.Aa = f + 9 * c;
    P.Ab = f + 15 * c;
    P.c = f + 21 * c;
    P.W = f + 24 * c;
    P.mu = f + 30 * c;
    P.r = ctx->pk_r.as<float>();
    P.V = ctx->v32.as<float4>();
    P.minv = ctx->minv32.as<float>();
    P.Iinv = ctx->Iinv32.as<float>();
    P.v0 = ctx->v.as<double>();
    P.body_off = off;
    P.body_adj = adj;
    P.nb = N;
    P.eval32 = (unsigned)ctx->check_interval;
    P.work = nullptr;
    k_pack3<<<blocks_for(nc), kBlock, 0, s>>>(nc, ctx->perm.as<int>(), C, A.r, P, P.r);
    k_body32<<<blocks_for(N), kBlock, 0, s>>>(N, V, ctx->minv.as<double>(), ctx->Iinv.as<double>(), P.V,
                                             const_cast<float*>(P.minv), const_cast<float*>(P.Iinv));
    SG_CUDA_TRY(cudaGetLastError());
    SG_CUDA_TRY(cudaMemsetAsync(ctx->s_exc.p, 0, sizeof(unsigned long long) * 3 * (size_t)S, s));
    SG_CUDA_TRY(cudaMemsetAsync(ctx->s_gmax.p, 0, sizeof(unsigned long long) * 3, s));
    Gs3MixedBatchArgs M;
    M.X = B;
    M.mode = ctx->s_mode.as<int>();
    M.since = ctx->s_since.as<unsigned>();
    M.exc_slot = ctx->s_exc.as<unsigned long long>();
    M.gmax = ctx->s_gmax.as<unsigned long long>();
    M.n64 = ctx->b_ctl.as<int>() + 1;
    void* args[] = {&M, &P};
    const int grid = coop_grid(ctx, k_gs3_mixed_batch, (long)ctx->num_sms * kGs3mBlock, kGs3mBlock, 1);
    if (ctx->profile) SG_CUDA_TRY(cudaEventRecord(ctx->ev_gs0, s));
    SG_CUDA_TRY(launch_cooperative((const void*)k_gs3_mixed_batch, grid, kGs3mBlock, args, s));
    if (ctx->profile) SG_CUDA_TRY(cudaEventRecord(ctx->ev_gs1, s));
    ctx->kernel_launches += 2;
  } else {
    void* args[] = {&B};
    const int grid = coop_grid(ctx, k_gs3_batch, (long)ctx->num_sms * kGs3Block, kGs3Block, 1);
    if (ctx->profile) SG_CUDA_TRY(cudaEventRecord(ctx->ev_gs0, s));
    SG_CUDA_TRY(launch_cooperative((const void*)k_gs3_batch, grid, kGs3Block, args, s));
    if (ctx->profile) SG_CUDA_TRY(cudaEventRecord(ctx->ev_gs1, s));
  }
  k_final_vel3<<<blocks_for(N), kBlock, 0, s>>>(N, off, adj, C, A.r, ctx->v.as<double>(), ctx->m.as<double>(),
                                                ctx->minv.as<double>(), ctx->Iw.as<double>(), ctx->Iinv.as<double>(),
                                                ctx->v2.as<double>());
  k_extract3<<<blocks_for(nc), kBlock, 0, s>>>(nc, A.E, A.r, ctx->ab3.as<double>());
  SG_CUDA_TRY(cudaGetLastError());
  unsigned long long work[5];
  std::vector<double> best(S);
  std::vector<int> done(S);
  SG_CUDA_TRY(cudaMemcpyAsync(&ctx->h_stats, sst, sizeof(SolveStats), cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaMemcpyAsync(work, ctx->b_work.p, sizeof(work), cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaMemcpyAsync(best.data(), ctx->s_best.p, sizeof(double) * S, cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaMemcpyAsync(done.data(), ctx->s_done.p, sizeof(int) * S, cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaStreamSynchronize(s));
  // pair write, plane write, assemble, vel init, gs, final velocity, extract
  ctx->kernel_launches += 6 + (ctx->bflags > 0 ? 1 : 0);
  if (ctx->h_stats.status == SG_DEVICE_TIMEOUT) {
    set_error("a device-side wait exceeded its spin limit");
    return SG_DEVICE_TIMEOUT;
  }
  if (ctx->h_stats.status == SG_CAPACITY) {
    set_error("contact colouring exceeded 64 colours or its round limit");
    return SG_CAPACITY;
  }
  ctx->gs_launches += 1;
  ctx->contact_sweeps32 += work[0];
  ctx->contact_sweeps += work[1];
  ctx->contact_evals += work[2];
  ctx->contact_lifts += work[3];
  ctx->body_lifts += work[4];
  if (ctx->profile) {
    float ms = 0.f;
    SG_CUDA_TRY(cudaEventElapsedTime(&ms, ctx->ev_gs0, ctx->ev_gs1));
    ctx->gs_ms += ms;
  }
  int all_done = 1;
  double worst = 0.0;
  for (int k = 0; k < S; ++k) {
    all_done &= done[k] ? 1 : 0;
    if (best[k] < INFINITY && best[k] > worst) worst = best[k];
  }
  st.iterations = ctx->h_stats.iterations;
  st.succeeded = all_done;
  st.error = worst;
  st.n_colors = (uint32_t)ctx->h_stats.n_colors;
  if (int r = splitham(ctx, ctx->v2.as<double>(), false)) return r;
  std::swap(ctx->q, ctx->q1);
  std::swap(ctx->v, ctx->v1);
  if (int r = sphere3d_update_inertia(ctx, false)) return r;
  ctx->kernel_launches += 2;
  if (out) *out = st;
  return st.succeeded ? SG_OK : SG_NOT_CONVERGED;
}

}  // namespace sg
