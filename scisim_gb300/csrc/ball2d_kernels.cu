// ball2d_kernels.cu -- Ball2D unconstrained maps, broad phase, narrow phase and
// contact assembly for sm_103a.
//
// Every kernel here computes in FP64 with the operation order of the SCISim
// reference (the library is built with -fmad=false, so no multiply-add is
// contracted); contact sets and forcing terms are therefore bit-identical to the
// reference arithmetic.
//
// Layout in HBM: q, v interleaved [x0 y0 x1 y1 ...] (double2 per body, as SCISim's
// VectorXs), r, m, minv one double per body; contacts as SoA arrays (ia, ib int32,
// n double2, forcing c double2, W 3 doubles, mu, local impulse r double2, key u64).
#include "ccd2d.hpp"
#include "ctx.hpp"

#include <algorithm>
#include <cmath>
#include <utility>

namespace sg {
namespace {

constexpr int kBlock = 256;

inline int blocks_for(long n, int per = kBlock) { return (int)((n + per - 1) / per); }

// std::min(a, b) / std::max(a, b) semantics (Eigen cwise min/max on arrays).
__device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }

// ---------------------------------------------------------------------------
// Unconstrained map with gravity F = m g (SymplecticEulerMap.cpp:21-32,
// VerletMap.cpp:15-41, Ball2DGravityForce.cpp:36-46).
__device__ __forceinline__ void umap_body(int integrator, double dt, double gx, double gy, double m, double minv,
                                          double q0x, double q0y, double v0x, double v0y, double& q1x,
                                          double& q1y, double& v1x, double& v1y) {
  const double fx = m * gx;
  const double fy = m * gy;
  if (integrator == SG_SYMPLECTIC_EULER) {
    const double sc = dt * minv;
    v1x = v0x + sc * fx;
    v1y = v0y + sc * fy;
    q1x = q0x + dt * v1x;
    q1y = q0y + dt * v1y;
  } else {
    const double sc = (0.5 * dt) * minv;
    const double vhx = v0x + sc * fx;
    const double vhy = v0y + sc * fy;
    q1x = q0x + dt * vhx;
    q1y = q0y + dt * vhy;
    v1x = vhx + sc * fx;
    v1y = vhy + sc * fy;
  }
}

__global__ void k_predict_aabb(int nb, int integrator, double dt, double gx, double gy,
                               const double2* __restrict__ q, const double2* __restrict__ v,
                               const double* __restrict__ m, const double* __restrict__ minv,
                               const double* __restrict__ rad, double2* __restrict__ q1, double2* __restrict__ v1,
                               double4_32a* __restrict__ aabb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const double2 q0 = q[i], v0 = v[i];
  double2 qn, vn;
  umap_body(integrator, dt, gx, gy, m[i], minv[i], q0.x, q0.y, v0.x, v0.y, qn.x, qn.y, vn.x, vn.y);
  q1[i] = qn;
  v1[i] = vn;
  // Swept AABB [min(q0, q1) - r, max(q0, q1) + r] (Ball2DSim.cpp:566-572).
  const double r = rad[i];
  double4_32a b;
  b.x = smin(qn.x, q0.x) - r;
  b.y = smin(qn.y, q0.y) - r;
  b.z = smax(qn.x, q0.x) + r;
  b.w = smax(qn.y, q0.y) + r;
  aabb[i] = b;
}

// SymplecticEulerImpactFrictionMap predictor (SymplecticEulerImpactFrictionMap.cpp:219-229): the
// velocity change vdelta = dt (Minv F) with F = 0 + m g accumulated as the reference's force and
// sparse product do, q1 = q0 + dt (v0 + vdelta); swept AABBs as k_predict_aabb.
__global__ void k_predict_se(int nb, double dt, double gx, double gy, const double2* __restrict__ q,
                             const double2* __restrict__ v, const double* __restrict__ m,
                             const double* __restrict__ minv, const double* __restrict__ rad, double2* __restrict__ q1,
                             double2* __restrict__ v1, double2* __restrict__ vdelta, double4_32a* __restrict__ aabb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const double2 q0 = q[i], v0 = v[i];
  const double mi = m[i], wi = minv[i];
  const double2 vd = make_double2(dt * (0.0 + wi * (0.0 + mi * gx)), dt * (0.0 + wi * (0.0 + mi * gy)));
  const double2 vn = make_double2(v0.x + vd.x, v0.y + vd.y);
  const double2 qn = make_double2(q0.x + dt * vn.x, q0.y + dt * vn.y);
  vdelta[i] = vd;
  q1[i] = qn;
  v1[i] = vn;
  const double r = rad[i];
  double4_32a b;
  b.x = smin(qn.x, q0.x) - r;
  b.y = smin(qn.y, q0.y) - r;
  b.z = smax(qn.x, q0.x) + r;
  b.w = smax(qn.y, q0.y) + r;
  aabb[i] = b;
}

// Its final update: v1 = v2 + vdelta, q1 = q0 + dt v1 (:363, :406); without vdelta the
// StabilizedImpactFrictionMap's v1 = v2, q1 = q0 + dt v1 (StabilizedImpactFrictionMap.cpp:136, :167).
__global__ void k_final_se(int nb, double dt, const double2* __restrict__ q0, const double2* __restrict__ v2,
                           const double2* __restrict__ vdelta, double2* __restrict__ q1, double2* __restrict__ v1) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const double2 q = q0[i], w = v2[i];
  double2 vn = w;
  if (vdelta) {
    const double2 d = vdelta[i];
    vn = make_double2(w.x + d.x, w.y + d.y);
  }
  v1[i] = vn;
  q1[i] = make_double2(q.x + dt * vn.x, q.y + dt * vn.y);
}

// Bounds of all boxes and the largest extent per axis (exact: min/max are order free).
// With aabb32 non-null it also writes each box rounded outward to FP32 (min corners down, max
// corners up), the pair scans' prefilter: FP32 boxes apart imply FP64 boxes apart.
__global__ void k_bounds(int n, const double4_32a* __restrict__ aabb, GridParams* gp, float4* __restrict__ aabb32) {
  double mn0 = INFINITY, mn1 = INFINITY, mx0 = -INFINITY, mx1 = -INFINITY, e0 = 0.0, e1 = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double4_32a b = aabb[i];
    if (aabb32)
      aabb32[i] = make_float4(__double2float_rd(b.x), __double2float_rd(b.y), __double2float_ru(b.z),
                              __double2float_ru(b.w));
    mn0 = fmin(mn0, b.x);
    mn1 = fmin(mn1, b.y);
    mx0 = fmax(mx0, b.z);
    mx1 = fmax(mx1, b.w);
    e0 = fmax(e0, b.z - b.x);
    e1 = fmax(e1, b.w - b.y);
  }
  for (int o = 16; o > 0; o >>= 1) {
    mn0 = fmin(mn0, __shfl_down_sync(0xffffffffu, mn0, o));
    mn1 = fmin(mn1, __shfl_down_sync(0xffffffffu, mn1, o));
    mx0 = fmax(mx0, __shfl_down_sync(0xffffffffu, mx0, o));
    mx1 = fmax(mx1, __shfl_down_sync(0xffffffffu, mx1, o));
    e0 = fmax(e0, __shfl_down_sync(0xffffffffu, e0, o));
    e1 = fmax(e1, __shfl_down_sync(0xffffffffu, e1, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&gp->enc_min[0], f64_to_ordered(mn0));
    atomicMin(&gp->enc_min[1], f64_to_ordered(mn1));
    atomicMax(&gp->enc_max[0], f64_to_ordered(mx0));
    atomicMax(&gp->enc_max[1], f64_to_ordered(mx1));
    atomicMax(&gp->enc_ext[0], f64_to_ordered(e0));
    atomicMax(&gp->enc_ext[1], f64_to_ordered(e1));
  }
}

__global__ void k_bounds_init(GridParams* gp) {
  gp->enc_min[0] = gp->enc_min[1] = ~0ull;
  gp->enc_max[0] = gp->enc_max[1] = 0ull;
  gp->enc_ext[0] = gp->enc_ext[1] = 0ull;
}

// Cell width h strictly above the largest box extent, so two overlapping boxes
// have min corners in the same or adjacent cells (3x3 neighbourhood suffices).
// The cell count is capped at `cap`; h grows if needed (larger cells stay correct).
__global__ void k_grid_setup(GridParams* gp, long cap) {
  const double mn0 = ordered_to_f64(gp->enc_min[0]), mn1 = ordered_to_f64(gp->enc_min[1]);
  const double mx0 = ordered_to_f64(gp->enc_max[0]), mx1 = ordered_to_f64(gp->enc_max[1]);
  const double e = fmax(ordered_to_f64(gp->enc_ext[0]), ordered_to_f64(gp->enc_ext[1]));
  double h = e * (1.0 + 0x1p-20) + 1e-300;
  if (!(h > 0.0) || !isfinite(h)) h = 1.0;
  double span0 = mx0 - mn0, span1 = mx1 - mn1;
  if (!isfinite(span0) || span0 < 0.0) span0 = 0.0;
  if (!isfinite(span1) || span1 < 0.0) span1 = 0.0;
  double d0 = floor(span0 / h) + 1.0, d1 = floor(span1 / h) + 1.0;
  while (d0 * d1 > (double)cap) {
    h = h * fmax(1.01, sqrt(d0 * d1 / (double)cap));
    d0 = floor(span0 / h) + 1.0;
    d1 = floor(span1 / h) + 1.0;
  }
  gp->origin[0] = isfinite(mn0) ? mn0 : 0.0;
  gp->origin[1] = isfinite(mn1) ? mn1 : 0.0;
  gp->h = h;
  gp->dims[0] = (int)d0;
  gp->dims[1] = (int)d1;
  gp->ncells = (int)(d0 * d1);
}

__device__ __forceinline__ int cell_coord(double x, double o, double h, int dim) {
  double f = (x - o) / h;
  int c = (f > 0.0) ? (int)f : 0;  // NaN -> 0
  return c < dim ? c : dim - 1;
}

__global__ void k_cell_count(int n, const double4_32a* __restrict__ aabb, const GridParams* __restrict__ gp,
                             int* __restrict__ cell_of, int* __restrict__ cell_count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double4_32a b = aabb[i];
  const int cx = cell_coord(b.x, gp->origin[0], gp->h, gp->dims[0]);
  const int cy = cell_coord(b.y, gp->origin[1], gp->h, gp->dims[1]);
  const int cell = cx + gp->dims[0] * cy;
  cell_of[i] = cell;
  atomicAdd(&cell_count[cell], 1);
}

// With box32 non-null the FP32 boxes go along into cell order (box32_sorted), so that the pair
// scans read each cell's boxes as one contiguous run.
__global__ void k_cell_scatter(int n, const int* __restrict__ cell_of, const int* __restrict__ cell_start,
                               int* __restrict__ cell_fill, int* __restrict__ sorted,
                               const float4* __restrict__ box32 = nullptr, float4* __restrict__ box32_sorted = nullptr) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int cell = cell_of[i];
  const int pos = cell_start[cell] + atomicAdd(&cell_fill[cell], 1);
  sorted[pos] = i;
  if (box32) box32_sorted[pos] = box32[i];
}

// AABB::overlaps (ball2d/SpatialGridDetector.cpp:15-26): touching boxes overlap.
__device__ __forceinline__ bool aabb_overlap(const double4_32a& a, const double4_32a& b) {
  if (a.z < b.x || a.w < b.y) return false;
  if (b.z < a.x || b.w < a.y) return false;
  return true;
}

// CollisionDetectionUtilities::computeCCDQuadraticCoeffs (CollisionDetectionUtilities.cpp:3-126);
// the answers on these coefficients are in ccd2d.hpp.
__device__ __forceinline__ void ccd_coeffs(double2 q0a, double2 q1a, double ra, double2 q0b, double2 q1b,
                                           double rb, double& c0, double& c1, double& c2) {
  const double d0x = q0a.x - q0b.x, d0y = q0a.y - q0b.y;
  const double ex = (q1a.x - q1b.x) - d0x, ey = (q1a.y - q1b.y) - d0y;
  const double rs = ra + rb;
  c0 = (d0x * d0x + d0y * d0y) - rs * rs;
  c1 = 2.0 * (d0x * ex + d0y * ey);
  c2 = ex * ex + ey * ey;
}

struct PairScan {
  const double4_32a* aabb;
  const float4* aabb32;   // the boxes rounded outward to FP32 (prefilter), by body
  const float4* aabb32s;  // the same in cell order (position p holds body sorted[p])
  const GridParams* gp;
  const int* cell_start;
  const int* sorted;
  const int* cell_of;     // each box's cell (of its min corner), as k_cell_count placed it
  // narrow phase inputs (ccd mode)
  const double2* q0;
  const double2* q1;
  const double* rad;
};

// Visits every j > i whose box overlaps box i (and, in ccd mode, whose CCD test
// hits).  Scans the 3x3 cells around the cell of box i's min corner.
template <bool kCcd, typename F>
__device__ __forceinline__ void visit_pairs(const PairScan& s, int i, F&& f) {
  const double4_32a bi = s.aabb[i];
  const float4 fi = s.aabb32[i];
  const GridParams& g = *s.gp;
  const int cx = cell_coord(bi.x, g.origin[0], g.h, g.dims[0]);
  const int cy = cell_coord(bi.y, g.origin[1], g.h, g.dims[1]);
  double2 q0a, q1a;
  double ra = 0.0;
  if (kCcd) {
    q0a = s.q0[i];
    q1a = s.q1[i];
    ra = s.rad[i];
  }
  for (int y = max(cy - 1, 0); y <= min(cy + 1, g.dims[1] - 1); ++y) {
    for (int x = max(cx - 1, 0); x <= min(cx + 1, g.dims[0] - 1); ++x) {
      const int cell = x + g.dims[0] * y;
      const int e = s.cell_start[cell + 1];
      for (int p = s.cell_start[cell]; p < e; ++p) {
        const float4 fj = s.aabb32s[p];
        if (fi.z < fj.x || fi.w < fj.y || fj.z < fi.x || fj.w < fi.y) continue;
        const int j = s.sorted[p];
        if (j <= i) continue;
        if (!aabb_overlap(bi, s.aabb[j])) continue;
        if (kCcd) {
          double c0, c1, c2;
          ccd_coeffs(q0a, q1a, ra, s.q0[j], s.q1[j], s.rad[j], c0, c1, c2);
          if (!ccd_hits(c0, c1, c2)) continue;
        }
        f(j);
      }
    }
  }
}

// The counting pass keeps each box's first kPairSlots partners (in visiting order) so that the
// writing pass of a box with at most that many only sorts them; a box with more visits again.
constexpr int kPairSlots = 8;
// Partners a thread queues for its warp's FP64 tests.
constexpr int kPairQueue = 16;

// Pair counting in two phases per warp.  Each thread runs the FP32 box prefilter over its 3x3 cells
// and queues the partners j > i that pass; the warp then runs the FP64 box test and the CCD test
// over all its queued partners 32 at a time, so that the FP64 pipe (narrow on this GPU) issues them
// for full warps rather than for the few lanes of a warp whose cell loops hit at the same step.  The
// tests and their arithmetic are those of visit_pairs, so the pairs (and the slots, in visiting
// order) are the same; a thread whose queue overflows counts with visit_pairs after the warp phase.
template <bool kCcd>
__global__ void __launch_bounds__(kBlock) k_pair_count(int n, PairScan s, int* __restrict__ cnt,
                                                       int* __restrict__ slots) {
  __shared__ int queue[kBlock * kPairQueue];             // per thread: partner j, -1 once rejected
  __shared__ unsigned short order[kBlock * kPairQueue];  // per warp: its queue entries in lane order
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  int* mine_q = queue + threadIdx.x * kPairQueue;
  int i = -1, m = 0;
  if (t < n) {
    i = s.sorted[t];  // bodies in cell order: neighbouring threads scan the same cells
    const float4 fi = s.aabb32[i];
    const GridParams& g = *s.gp;
    const int cell = s.cell_of[i];
    const int cy = cell / g.dims[0], cx = cell - cy * g.dims[0];
    for (int y = max(cy - 1, 0); y <= min(cy + 1, g.dims[1] - 1); ++y) {
      for (int x = max(cx - 1, 0); x <= min(cx + 1, g.dims[0] - 1); ++x) {
        const int c = x + g.dims[0] * y;
        const int e = s.cell_start[c + 1];
        for (int p = s.cell_start[c]; p < e; ++p) {
          const float4 fj = s.aabb32s[p];
          if (fi.z < fj.x || fi.w < fj.y || fj.z < fi.x || fj.w < fi.y) continue;
          const int j = s.sorted[p];
          if (j <= i) continue;
          if (m < kPairQueue) mine_q[m] = j;
          ++m;
        }
      }
    }
  }
  const int q = m <= kPairQueue ? m : 0;
  int incl = q;
  for (int d = 1; d < 32; d <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += u;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  unsigned short* w_order = order + (threadIdx.x - lane) * kPairQueue;
  for (int k = 0; k < q; ++k) w_order[incl - q + k] = (unsigned short)(threadIdx.x * kPairQueue + k);
  __syncwarp();
  const int block0 = blockIdx.x * blockDim.x;
  for (int k = lane; k < total; k += 32) {
    const int e = w_order[k];
    const int io = s.sorted[block0 + e / kPairQueue];
    const int j = queue[e];
    bool hit = aabb_overlap(s.aabb[io], s.aabb[j]);
    if (kCcd && hit) {
      double c0, c1, c2;
      ccd_coeffs(s.q0[io], s.q1[io], s.rad[io], s.q0[j], s.q1[j], s.rad[j], c0, c1, c2);
      hit = ccd_hits(c0, c1, c2);
    }
    if (!hit) queue[e] = -1;
  }
  __syncwarp();
  if (t >= n) return;
  int c = 0;
  int* mine = slots + (size_t)i * kPairSlots;
  if (m <= kPairQueue) {
    for (int k = 0; k < m; ++k) {
      const int j = mine_q[k];
      if (j < 0) continue;
      if (c < kPairSlots) mine[c] = j;
      ++c;
    }
  } else {
    visit_pairs<kCcd>(s, i, [&](int j) {
      if (c < kPairSlots) mine[c] = j;
      ++c;
    });
  }
  cnt[i] = c;
}

template <bool kCcd>
__global__ void k_pair_write(int n, PairScan s, const int* __restrict__ off, const int* __restrict__ slots,
                             int* __restrict__ out_a, int* __restrict__ out_b) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = s.sorted[t];
  const int base = off[i];
  const int total = off[i + 1] - base;
  if (total <= kPairSlots) {
    const int* mine = slots + (size_t)i * kPairSlots;
    for (int c = 0; c < total; ++c) {
      const int j = mine[c];
      int p = base + c;
      while (p > base && out_b[p - 1] > j) {
        out_b[p] = out_b[p - 1];
        --p;
      }
      out_b[p] = j;
    }
    for (int k = 0; k < total; ++k) out_a[base + k] = i;
    return;
  }
  int c = 0;
  visit_pairs<kCcd>(s, i, [&](int j) {
    // insertion into the sorted segment [base, base + c)
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

// StaticPlaneConstraint::isActive at the predictor position (BallStaticPlaneConstraint.cpp:10-14),
// flattened plane-major like Ball2DSim::computeBallPlaneActiveSetAllPairs (Ball2DSim.cpp:747-762).
__global__ void k_plane_flags(int nb, int np, const double2* __restrict__ q1, const double* __restrict__ rad,
                              const double2* __restrict__ px, const double2* __restrict__ pn, int* __restrict__ flag) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)nb * np) return;
  const int p = (int)(t / nb), i = (int)(t - (long)p * nb);
  const double2 x = px[p], nn = pn[p], qi = q1[i];
  const double d = nn.x * (qi.x - x.x) + nn.y * (qi.y - x.y);
  flag[t] = (d <= rad[i]) ? 1 : 0;
}

__global__ void k_plane_write(int nb, int np, int npairs, const int* __restrict__ flag, const int* __restrict__ off,
                              int* __restrict__ ia, int* __restrict__ ib) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)nb * np) return;
  if (!flag[t]) return;
  const int p = (int)(t / nb), i = (int)(t - (long)p * nb);
  const int k = npairs + off[t];
  ia[k] = i;
  ib[k] = -1 - p;
}

// Contact keys: ball-ball (i, j) and plane-ball (p, i) in one sorted key space
// (ConstraintCache keys, ball2d/ConstraintCache.cpp:20-50).
__device__ __forceinline__ unsigned long long contact_key(int a, int b) {
  if (b >= 0) return ((unsigned long long)(unsigned)a << 32) | (unsigned)b;
  const unsigned p = (unsigned)(-1 - b);
  return 0x8000000000000000ull | ((unsigned long long)p << 32) | (unsigned)a;
}

__device__ __forceinline__ long find_key(const unsigned long long* keys, long n, unsigned long long k) {
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

struct AssembleArgs {
  int nc;
  const int* ia;
  const int* ib;
  const double2* q0;
  const double2* v0;
  const double* minv;
  const double2* plane_n;
  const double2* plane_t;
  double mu, CoR;
  int cache_mode;
  const unsigned long long* prev_key;
  const double2* prev_ab;
  long prev_n;
  double2* n;
  double2* c;
  double* W;
  double* mu_out;
  double2* r;
  unsigned long long* key;
  // SymplecticEulerImpactFrictionMap: the velocity change of the step (null for the geometric
  // map), and its pose stabilisation (positions, radii, plane points, dt, threshold).
  const double2* vdelta = nullptr;
  const double* rad = nullptr;
  const double2* plane_x = nullptr;
  double dt = 0.0;
  int stabilize = 0;
  double pen_thresh = 0.0;
  // The step before's rows (single-scene steps): its pair offsets per body, plane flags and their
  // scan, so that a contact's cache entry is found in O(1): a pair (a, b) among a's pairs of the
  // step before, a plane contact by its flag (null: binary search over all keys).
  const int* prev_pair_off = nullptr;
  const int* prev_plane_off = nullptr;
  const int* prev_plane_flag = nullptr;
  int prev_npairs = 0;
  int nb = 0;
  // Colours carried over: init_color[k] = the step before's colour of contact k (prev_color, by
  // cache index) or -1 for a new contact (null: none).
  const int* prev_color = nullptr;
  int* init_color = nullptr;
};

// Index of key among the cached contacts of the step before, through its rows: a pair (a, b) among
// a's pairs (sorted by b), a plane contact (plane p, body a) at prev_npairs + its flag's scan.
__device__ __forceinline__ long find_key_rows(const AssembleArgs& A, int a, int b, unsigned long long key) {
  long idx = -1;
  if (b >= 0) {
    long lo = A.prev_pair_off[a], hi = A.prev_pair_off[a + 1];
    while (lo < hi) {
      const long mid = (lo + hi) >> 1;
      if (A.prev_key[mid] < key)
        lo = mid + 1;
      else
        hi = mid;
    }
    if (lo < A.prev_pair_off[a + 1] && A.prev_key[lo] == key) idx = lo;
  } else {
    const long t = (long)(-1 - b) * A.nb + a;
    if (A.prev_plane_flag[t]) {
      const long j = (long)A.prev_npairs + A.prev_plane_off[t];
      if (j < A.prev_n && A.prev_key[j] == key) idx = j;
    }
  }
  return idx;
}

// Contact basis, forcing term, diagonal Delassus block and warm start per contact:
// BallBallConstraint ctor (:26-37) and computeContactBasis (:244-252),
// Constraint::computeForcingTerm (Constraint.cpp:18-34), evalKinematicRelVelGivenBases
// (Constraint.cpp:92-126), Balls2DSobogusInterface::fromPrimal (:31-94),
// initializeImpulses (GeometricImpactFrictionMap.cpp:174-220), solve2D warm start (Sobogus.cpp:299-301).
__device__ __forceinline__ void assemble_one(const AssembleArgs& A, int k, double mu, double CoR,
                                             const unsigned long long* prev_key, const double2* prev_ab,
                                             long prev_n) {
  const int a = A.ia[k], b = A.ib[k];
  double nx, ny, tx, ty;
  double vrx, vry;
  const double2 va = A.v0[a];
  if (b >= 0) {
    const double2 qa = A.q0[a], qb = A.q0[b];
    double dx = qa.x - qb.x, dy = qa.y - qb.y;
    const double z = dx * dx + dy * dy;
    if (z > 0.0) {
      const double sq = sqrt(z);
      dx = dx / sq;
      dy = dy / sq;
    }
    nx = dx;
    ny = dy;
    tx = -dy;
    ty = dx;
    const double2 vb = A.v0[b];
    vrx = va.x - vb.x;
    vry = va.y - vb.y;
  } else {
    const int p = -1 - b;
    const double2 pn = A.plane_n[p], pt = A.plane_t[p];
    nx = pn.x;
    ny = pn.y;
    tx = pt.x;
    ty = pt.y;
    vrx = va.x - 0.0;
    vry = va.y - 0.0;
  }
  const double ndotv = nx * vrx + ny * vry;
  double nrel = -(0.0 * nx + 0.0 * ny);
  double drel = -(0.0 * tx + 0.0 * ty);
  if (A.vdelta) {
    // nrel = N^T vdelta, drel = D^T vdelta (SymplecticEulerImpactFrictionMap.cpp:294-305): the
    // column's entries (n, -n / t, -t) in row order, accumulated from zero as the sparse product;
    // then the stabilisation nrel += min(0, gap(q0)) / dt beyond the threshold (:307-321).
    const double2 da = A.vdelta[a];
    double tn = 0.0, tt = 0.0;
    tn = tn + nx * da.x;
    tn = tn + ny * da.y;
    tt = tt + tx * da.x;
    tt = tt + ty * da.y;
    if (b >= 0) {
      const double2 db = A.vdelta[b];
      tn = tn + (-nx) * db.x;
      tn = tn + (-ny) * db.y;
      tt = tt + (-tx) * db.x;
      tt = tt + (-ty) * db.y;
    }
    double ext_n = 0.0 + 1.0 * tn;
    const double ext_d = 0.0 + 1.0 * tt;
    if (A.stabilize) {
      const double2 qa = A.q0[a];
      double gap;
      if (b >= 0) {
        const double2 qb = A.q0[b];
        const double gx = qa.x - qb.x, gy = qa.y - qb.y;
        gap = sqrt(gx * gx + gy * gy) - (A.rad[a] + A.rad[b]);
      } else {
        const double2 px = A.plane_x[-1 - b];
        gap = (nx * (qa.x - px.x) + ny * (qa.y - px.y)) - A.rad[a];
      }
      double g0 = (gap < 0.0) ? gap : 0.0;  // std::min(0.0, gap)
      if (fabs(g0) < A.pen_thresh) g0 = 0.0;
      ext_n = ext_n + g0 / A.dt;
    }
    // Sobogus::solve adds the map's extra relative velocities to the kinematic ones (Sobogus.cpp:890-904).
    nrel = nrel + ext_n;
    drel = drel + ext_d;
  }
  const double s = CoR * ndotv + nrel;
  const double wx = (0.0 + nx * s) + tx * drel;
  const double wy = (0.0 + ny * s) + ty * drel;
  A.n[k] = make_double2(nx, ny);
  A.c[k] = make_double2(nx * wx + ny * wy, tx * wx + ty * wy);
  const double nn = nx * nx + ny * ny;
  const double nt = nx * tx + ny * ty;
  const double tt = tx * tx + ty * ty;
  const double ma = A.minv[a];
  double w00 = ma * nn, w01 = ma * nt, w11 = ma * tt;
  if (b >= 0) {
    const double mb = A.minv[b];
    w00 = w00 + mb * nn;
    w01 = w01 + mb * nt;
    w11 = w11 + mb * tt;
  }
  A.W[3 * k] = w00;
  A.W[3 * k + 1] = w01;
  A.W[3 * k + 2] = w11;
  A.mu_out[k] = mu;
  const unsigned long long key = contact_key(a, b);
  A.key[k] = key;
  double alpha = 0.0, beta = 0.0;
  long idx = -1;
  if (A.cache_mode != SG_CACHE_NONE && prev_n > 0) {
    idx = A.prev_pair_off ? find_key_rows(A, a, b, key) : find_key(prev_key, prev_n, key);
    if (idx >= 0) {
      const double2 ab = prev_ab[idx];
      alpha = ab.x;
      beta = (A.cache_mode == SG_CACHE_NORMAL_AND_FRICTION) ? ab.y : 0.0;
    }
  }
  if (A.init_color) A.init_color[k] = idx >= 0 ? A.prev_color[idx] : -1;
  const double rwx = alpha * nx + beta * tx;
  const double rwy = alpha * ny + beta * ty;
  A.r[k] = make_double2(nx * rwx + ny * rwy, tx * rwx + ty * rwy);
}

__global__ void k_assemble(AssembleArgs A) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= A.nc) return;
  assemble_one(A, k, A.mu, A.CoR, A.prev_key, A.prev_ab, A.prev_n);
}

// alpha = r_world . n, beta = r_world . t (Sobogus.cpp:312-330); caches (alpha, beta)
// (cacheImpulses, GeometricImpactFrictionMap.cpp:222-264).
__global__ void k_extract(int nc, const int* __restrict__ nc_dev, const double2* __restrict__ n,
                          const double2* __restrict__ r, const double* __restrict__ mu, int cache_mode,
                          double2* __restrict__ ab) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (nc_dev) nc = *nc_dev;
  if (k >= nc) return;
  const double2 nk = n[k], rk = r[k];
  const double nx = nk.x, ny = nk.y, tx = -ny, ty = nx;
  const double rwx = nx * rk.x + tx * rk.y;
  const double rwy = ny * rk.x + ty * rk.y;
  const double alpha = rwx * nx + rwy * ny;
  const double beta = (mu[k] == 0.0) ? 0.0 : (rwx * tx + rwy * ty);
  (void)cache_mode;  // decaching applies the mode (k_assemble)
  ab[k] = make_double2(alpha, beta);
}

__global__ void k_final_map(int nb, int integrator, double dt, double gx, double gy, const double2* __restrict__ q0,
                            const double2* __restrict__ vin, const double* __restrict__ m,
                            const double* __restrict__ minv, double2* __restrict__ q1, double2* __restrict__ v1) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const double2 q = q0[i], v = vin[i];
  double2 qn, vn;
  umap_body(integrator, dt, gx, gy, m[i], minv[i], q.x, q.y, v.x, v.y, qn.x, qn.y, vn.x, vn.y);
  q1[i] = qn;
  v1[i] = vn;
}

// ---------------------------------------------------------------------------
// Batched scenes.  Scene s owns bodies [sb_off[s], sb_off[s+1]) and planes
// [sp_off[s], sp_off[s+1]); each scene has its own uniform grid (cells
// [s_cell_off[s], s_cell_off[s+1]) of one global cell array) and its contacts are
// [sc_off[s], sc_off[s+1]) of the step: its ball-ball pairs in (i, j) order, then its
// plane contacts plane-major (Ball2DSim::computeActiveSet per scene, Ball2DSim.cpp:151-173).
// Every launch is sized by static counts (bodies, scenes, cell and flag capacities,
// contact capacity); the contact count lives on the device, so a step enqueues with no
// host synchronisation and can be captured in a CUDA graph.
struct SceneGrid {
  double origin[2];
  double h;
  int dims[2];
  int ncells;
  int pad;
};

// One block per scene: bounds and largest extent of the scene's boxes, then the grid
// (cell strictly wider than any box, at most 4 n + 64 cells), as k_grid_setup.
__global__ void k_scene_grid(const int* __restrict__ sb_off, const double4_32a* __restrict__ aabb,
                             SceneGrid* __restrict__ grids, int* __restrict__ s_cells) {
  const int sc = blockIdx.x;
  const int b0 = sb_off[sc], b1 = sb_off[sc + 1];
  double mn0 = INFINITY, mn1 = INFINITY, mx0 = -INFINITY, mx1 = -INFINITY, e = 0.0;
  for (int i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
    const double4_32a b = aabb[i];
    mn0 = fmin(mn0, b.x);
    mn1 = fmin(mn1, b.y);
    mx0 = fmax(mx0, b.z);
    mx1 = fmax(mx1, b.w);
    e = fmax(e, fmax(b.z - b.x, b.w - b.y));
  }
  for (int o = 16; o > 0; o >>= 1) {
    mn0 = fmin(mn0, __shfl_down_sync(0xffffffffu, mn0, o));
    mn1 = fmin(mn1, __shfl_down_sync(0xffffffffu, mn1, o));
    mx0 = fmax(mx0, __shfl_down_sync(0xffffffffu, mx0, o));
    mx1 = fmax(mx1, __shfl_down_sync(0xffffffffu, mx1, o));
    e = fmax(e, __shfl_down_sync(0xffffffffu, e, o));
  }
  __shared__ double red[5][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    red[0][wid] = mn0;
    red[1][wid] = mn1;
    red[2][wid] = mx0;
    red[3][wid] = mx1;
    red[4][wid] = e;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  const int nw = (blockDim.x + 31) >> 5;
  for (int w = 1; w < nw; ++w) {
    mn0 = fmin(mn0, red[0][w]);
    mn1 = fmin(mn1, red[1][w]);
    mx0 = fmax(mx0, red[2][w]);
    mx1 = fmax(mx1, red[3][w]);
    e = fmax(e, red[4][w]);
  }
  const long cap = 4L * (b1 - b0) + 64;
  double h = e * (1.0 + 0x1p-20) + 1e-300;
  if (!(h > 0.0) || !isfinite(h)) h = 1.0;
  double span0 = mx0 - mn0, span1 = mx1 - mn1;
  if (!isfinite(span0) || span0 < 0.0) span0 = 0.0;
  if (!isfinite(span1) || span1 < 0.0) span1 = 0.0;
  double d0 = floor(span0 / h) + 1.0, d1 = floor(span1 / h) + 1.0;
  while (d0 * d1 > (double)cap) {
    h = h * fmax(1.01, sqrt(d0 * d1 / (double)cap));
    d0 = floor(span0 / h) + 1.0;
    d1 = floor(span1 / h) + 1.0;
  }
  SceneGrid g;
  g.origin[0] = isfinite(mn0) ? mn0 : 0.0;
  g.origin[1] = isfinite(mn1) ? mn1 : 0.0;
  g.h = h;
  g.dims[0] = (int)d0;
  g.dims[1] = (int)d1;
  g.ncells = (int)(d0 * d1);
  g.pad = 0;
  grids[sc] = g;
  s_cells[sc] = g.ncells;
}

__global__ void k_cell_count_b(int n, const int* __restrict__ scene_of, const double4_32a* __restrict__ aabb,
                               const SceneGrid* __restrict__ grids, const int* __restrict__ s_cell_off,
                               int* __restrict__ cell_of, int* __restrict__ cell_count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int sc = scene_of[i];
  const SceneGrid g = grids[sc];
  const double4_32a b = aabb[i];
  const int cx = cell_coord(b.x, g.origin[0], g.h, g.dims[0]);
  const int cy = cell_coord(b.y, g.origin[1], g.h, g.dims[1]);
  const int cell = s_cell_off[sc] + cx + g.dims[0] * cy;
  cell_of[i] = cell;
  atomicAdd(&cell_count[cell], 1);
}

struct BatchScan {
  const int* scene_of;
  const SceneGrid* grids;
  const int* s_cell_off;
  const double4_32a* aabb;
  const int* cell_start;
  const int* sorted;
  const double2* q0;
  const double2* q1;
  const double* rad;
};

// visit_pairs<true> within the scene grid of body i.
template <typename F>
__device__ __forceinline__ void visit_pairs_b(const BatchScan& s, int i, F&& f) {
  const int sc = s.scene_of[i];
  const SceneGrid g = s.grids[sc];
  const int base = s.s_cell_off[sc];
  const double4_32a bi = s.aabb[i];
  const int cx = cell_coord(bi.x, g.origin[0], g.h, g.dims[0]);
  const int cy = cell_coord(bi.y, g.origin[1], g.h, g.dims[1]);
  const double2 q0a = s.q0[i], q1a = s.q1[i];
  const double ra = s.rad[i];
  for (int y = max(cy - 1, 0); y <= min(cy + 1, g.dims[1] - 1); ++y) {
    for (int x = max(cx - 1, 0); x <= min(cx + 1, g.dims[0] - 1); ++x) {
      const int cell = base + x + g.dims[0] * y;
      const int e = s.cell_start[cell + 1];
      for (int p = s.cell_start[cell]; p < e; ++p) {
        const int j = s.sorted[p];
        if (j <= i) continue;
        if (!aabb_overlap(bi, s.aabb[j])) continue;
        double c0, c1, c2;
        ccd_coeffs(q0a, q1a, ra, s.q0[j], s.q1[j], s.rad[j], c0, c1, c2);
        if (!ccd_hits(c0, c1, c2)) continue;
        f(j);
      }
    }
  }
}

__global__ void k_pair_count_b(int n, BatchScan s, int* __restrict__ cnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c = 0;
  visit_pairs_b(s, i, [&](int) { ++c; });
  cnt[i] = c;
}

// StaticPlaneConstraint::isActive per (plane, body) of each scene, plane-major within
// the scene's flag range [sf_off[s], sf_off[s+1]).
__global__ void k_plane_flags_b(int n, const int* __restrict__ scene_of, const int* __restrict__ sb_off,
                                const int* __restrict__ sp_off, const int* __restrict__ sf_off,
                                const double2* __restrict__ q1, const double* __restrict__ rad,
                                const double2* __restrict__ px, const double2* __restrict__ pn,
                                int* __restrict__ flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int sc = scene_of[i];
  const int b0 = sb_off[sc], ns = sb_off[sc + 1] - b0;
  const int p0 = sp_off[sc], p1 = sp_off[sc + 1];
  const double2 qi = q1[i];
  const double ri = rad[i];
  for (int p = p0; p < p1; ++p) {
    const double2 x = px[p], nn = pn[p];
    const double d = nn.x * (qi.x - x.x) + nn.y * (qi.y - x.y);
    flag[sf_off[sc] + (long)(p - p0) * ns + (i - b0)] = (d <= ri) ? 1 : 0;
  }
}

// Per scene: ball-ball and plane contact counts.
__global__ void k_scene_counts(int S, const int* __restrict__ sb_off, const int* __restrict__ sf_off,
                               const int* __restrict__ pair_off, const int* __restrict__ plane_off,
                               int* __restrict__ s_nc, int* __restrict__ s_npairs) {
  const int sc = blockIdx.x * blockDim.x + threadIdx.x;
  if (sc >= S) return;
  const int np = pair_off[sb_off[sc + 1]] - pair_off[sb_off[sc]];
  const int nq = plane_off[sf_off[sc + 1]] - plane_off[sf_off[sc]];
  s_npairs[sc] = np;
  s_nc[sc] = np + nq;
}

// Total contacts against the capacity: on overflow the step keeps no contacts and the
// needed count is recorded for the host, which restores the chunk's starting state,
// grows the buffers and steps again.
__global__ void k_capacity(const int* __restrict__ total, int cap, int* __restrict__ nc_dev,
                           int* __restrict__ overflow, unsigned long long* __restrict__ contacts_sum) {
  const int nc = *total;
  if (nc > cap) {
    *nc_dev = 0;
    if (nc > *overflow) *overflow = nc;
  } else {
    *nc_dev = nc;
    *contacts_sum += (unsigned long long)nc;
  }
}

__global__ void k_pair_write_b(int n, BatchScan s, const int* __restrict__ sb_off, const int* __restrict__ pair_off,
                               const int* __restrict__ sc_off, const int* __restrict__ pair_cnt, int cap,
                               int* __restrict__ out_a, int* __restrict__ out_b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int sc = s.scene_of[i];
  const int base = sc_off[sc] + (pair_off[i] - pair_off[sb_off[sc]]);
  if (base + pair_cnt[i] > cap) return;
  int c = 0;
  visit_pairs_b(s, i, [&](int j) {
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

__global__ void k_plane_write_b(int n, const int* __restrict__ scene_of, const int* __restrict__ sb_off,
                                const int* __restrict__ sp_off, const int* __restrict__ sf_off,
                                const int* __restrict__ flag, const int* __restrict__ plane_off,
                                const int* __restrict__ sc_off, const int* __restrict__ s_npairs, int cap,
                                int* __restrict__ ia, int* __restrict__ ib) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int sc = scene_of[i];
  const int b0 = sb_off[sc], ns = sb_off[sc + 1] - b0;
  const int p0 = sp_off[sc], p1 = sp_off[sc + 1];
  const int fbase = sf_off[sc];
  const int cbase = sc_off[sc] + s_npairs[sc] - plane_off[fbase];
  for (int p = p0; p < p1; ++p) {
    const long t = fbase + (long)(p - p0) * ns + (i - b0);
    if (!flag[t]) continue;
    const int k = cbase + plane_off[t];
    if (k < cap) {
      ia[k] = i;
      ib[k] = -1 - p;
    }
  }
}

// Per-scene mu and CoR, warm start searched in the scene's own slice of the previous
// step's (sorted) keys.
__global__ void k_assemble_b(AssembleArgs A, const int* __restrict__ nc_dev, const int* __restrict__ scene_of,
                             const double* __restrict__ s_mu, const double* __restrict__ s_CoR,
                             const int* __restrict__ prev_sc_off, int* __restrict__ cscene) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= *nc_dev) return;
  const int sc = scene_of[A.ia[k]];
  cscene[k] = sc;
  const int p0 = prev_sc_off[sc], p1 = prev_sc_off[sc + 1];
  assemble_one(A, k, s_mu[sc], s_CoR[sc], A.prev_key + p0, A.prev_ab + p0, (long)(p1 - p0));
}

__global__ void k_ccd_batch(int n, const double2* q0a, const double2* q1a, const double* ra, const double2* q0b,
                            const double2* q1b, const double* rb, double* coeffs, int* hit, double* t) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double c0, c1, c2;
  ccd_coeffs(q0a[i], q1a[i], ra[i], q0b[i], q1b[i], rb[i], c0, c1, c2);
  coeffs[3 * i] = c0;
  coeffs[3 * i + 1] = c1;
  coeffs[3 * i + 2] = c2;
  double tt = 0.0;
  const bool h = ccd_happens(c0, c1, c2, &tt);
  hit[i] = h ? 1 : 0;
  t[i] = h ? tt : -1.0;
}

}  // namespace

// ===========================================================================
int ball2d_predict_and_bounds(sg_ctx* ctx) {
  const int nb = ctx->nb;
  if (nb <= 0) return SG_OK;
  if (ctx->staggering == SG_STAGGER_SYMPLECTIC_EULER && ctx->n_scenes == 0) {
    if (int r = grow(ctx->vdelta, sizeof(double) * 2 * (size_t)nb)) return r;
    k_predict_se<<<blocks_for(nb), kBlock, 0, ctx->stream>>>(
        nb, ctx->cfg.dt, ctx->cfg.gravity[0], ctx->cfg.gravity[1], ctx->q.as<double2>(), ctx->v.as<double2>(),
        ctx->m.as<double>(), ctx->minv.as<double>(), ctx->r.as<double>(), ctx->q1.as<double2>(),
        ctx->v1.as<double2>(), ctx->vdelta.as<double2>(), ctx->aabb.as<double4_32a>());
    SG_CUDA_TRY(cudaGetLastError());
    return SG_OK;
  }
  k_predict_aabb<<<blocks_for(nb), kBlock, 0, ctx->stream>>>(
      nb, ctx->cfg.integrator, ctx->cfg.dt, ctx->cfg.gravity[0], ctx->cfg.gravity[1], ctx->q.as<double2>(),
      ctx->v.as<double2>(), ctx->m.as<double>(), ctx->minv.as<double>(), ctx->r.as<double>(), ctx->q1.as<double2>(),
      ctx->v1.as<double2>(), ctx->aabb.as<double4_32a>());
  SG_CUDA_TRY(cudaGetLastError());
  return SG_OK;
}

static long grid_cap(int n) { return 4L * n + 64; }

int broadphase_build_grid(sg_ctx* ctx, const double* aabb, int n) {
  if (int r = grow(ctx->grid, sizeof(GridParams))) return r;
  const long cap = grid_cap(n);
  if (int r = grow(ctx->cell_count, sizeof(int) * (size_t)(cap + 1))) return r;
  if (int r = grow(ctx->cell_start, sizeof(int) * (size_t)(cap + 1))) return r;
  if (int r = grow(ctx->cell_fill, sizeof(int) * (size_t)(cap + 1))) return r;
  if (int r = grow(ctx->cell_of, sizeof(int) * (size_t)n)) return r;
  if (int r = grow(ctx->sorted, sizeof(int) * (size_t)n)) return r;
  GridParams* gp = ctx->grid.as<GridParams>();
  const double4_32a* bx = reinterpret_cast<const double4_32a*>(aabb);
  k_bounds_init<<<1, 1, 0, ctx->stream>>>(gp);
  const int nblk = std::min(blocks_for(n), ctx->num_sms * 8);
  if (int r = grow(ctx->aabb32, sizeof(float4) * (size_t)std::max(n, 1))) return r;
  k_bounds<<<std::max(nblk, 1), kBlock, 0, ctx->stream>>>(n, bx, gp, ctx->aabb32.as<float4>());
  k_grid_setup<<<1, 1, 0, ctx->stream>>>(gp, cap);
  SG_CUDA_TRY(cudaMemsetAsync(ctx->cell_count.p, 0, sizeof(int) * (size_t)(cap + 1), ctx->stream));
  SG_CUDA_TRY(cudaMemsetAsync(ctx->cell_fill.p, 0, sizeof(int) * (size_t)(cap + 1), ctx->stream));
  k_cell_count<<<blocks_for(n), kBlock, 0, ctx->stream>>>(n, bx, gp, ctx->cell_of.as<int>(), ctx->cell_count.as<int>());
  SG_CUDA_TRY(cudaGetLastError());
  if (int r = scan_exclusive(ctx, ctx->cell_count.as<int>(), ctx->cell_start.as<int>(), (int)cap)) return r;
  if (int r = grow(ctx->aabb32s, sizeof(float4) * (size_t)std::max(n, 1))) return r;
  k_cell_scatter<<<blocks_for(n), kBlock, 0, ctx->stream>>>(n, ctx->cell_of.as<int>(), ctx->cell_start.as<int>(),
                                                            ctx->cell_fill.as<int>(), ctx->sorted.as<int>(),
                                                            ctx->aabb32.as<float4>(), ctx->aabb32s.as<float4>());
  SG_CUDA_TRY(cudaGetLastError());
  return SG_OK;
}

static PairScan make_scan(sg_ctx* ctx, const double* aabb, bool ccd) {
  PairScan s;
  s.aabb = reinterpret_cast<const double4_32a*>(aabb);
  s.aabb32 = ctx->aabb32.as<float4>();
  s.aabb32s = ctx->aabb32s.as<float4>();
  s.gp = ctx->grid.as<GridParams>();
  s.cell_start = ctx->cell_start.as<int>();
  s.sorted = ctx->sorted.as<int>();
  s.cell_of = ctx->cell_of.as<int>();
  // RigidBody2D circles keep 3 entries per body: their CCD reads the centres the predictor copied out.
  s.q0 = ccd ? (ctx->rb2d ? ctx->pos0.as<double2>() : ctx->q.as<double2>()) : nullptr;
  s.q1 = ccd ? (ctx->rb2d ? ctx->pos1.as<double2>() : ctx->q1.as<double2>()) : nullptr;
  s.rad = ccd ? ctx->r.as<double>() : nullptr;
  return s;
}

int broadphase_count_pairs(sg_ctx* ctx, const double* aabb, int n, bool ccd) {
  if (int r = grow(ctx->pair_cnt, sizeof(int) * (size_t)(n + 1))) return r;
  if (int r = grow(ctx->pair_off, sizeof(int) * (size_t)(n + 1))) return r;
  if (int r = grow(ctx->pair_slots, sizeof(int) * kPairSlots * (size_t)std::max(n, 1))) return r;
  const PairScan s = make_scan(ctx, aabb, ccd);
  if (ccd)
    k_pair_count<true><<<blocks_for(n), kBlock, 0, ctx->stream>>>(n, s, ctx->pair_cnt.as<int>(),
                                                                 ctx->pair_slots.as<int>());
  else
    k_pair_count<false><<<blocks_for(n), kBlock, 0, ctx->stream>>>(n, s, ctx->pair_cnt.as<int>(),
                                                                  ctx->pair_slots.as<int>());
  SG_CUDA_TRY(cudaGetLastError());
  return scan_exclusive(ctx, ctx->pair_cnt.as<int>(), ctx->pair_off.as<int>(), n);
}

int broadphase_write_pairs(sg_ctx* ctx, const double* aabb, int n, bool ccd, int* out_a, int* out_b) {
  const PairScan s = make_scan(ctx, aabb, ccd);
  if (ccd)
    k_pair_write<true><<<blocks_for(n), kBlock, 0, ctx->stream>>>(n, s, ctx->pair_off.as<int>(),
                                                                 ctx->pair_slots.as<int>(), out_a, out_b);
  else
    k_pair_write<false><<<blocks_for(n), kBlock, 0, ctx->stream>>>(n, s, ctx->pair_off.as<int>(),
                                                                  ctx->pair_slots.as<int>(), out_a, out_b);
  SG_CUDA_TRY(cudaGetLastError());
  return SG_OK;
}

int plane_flags(sg_ctx* ctx) {
  const long t = (long)ctx->nb * ctx->np;
  if (int r = grow(ctx->plane_flag, sizeof(int) * (size_t)(t + 1))) return r;
  if (int r = grow(ctx->plane_off, sizeof(int) * (size_t)(t + 1))) return r;
  if (t == 0) {
    SG_CUDA_TRY(cudaMemsetAsync(ctx->plane_off.p, 0, sizeof(int), ctx->stream));
    return SG_OK;
  }
  const double2* q1 = ctx->rb2d ? ctx->pos1.as<double2>() : ctx->q1.as<double2>();
  k_plane_flags<<<blocks_for(t), kBlock, 0, ctx->stream>>>(ctx->nb, ctx->np, q1, ctx->r.as<double>(),
                                                           ctx->plane_x.as<double2>(), ctx->plane_n.as<double2>(),
                                                           ctx->plane_flag.as<int>());
  SG_CUDA_TRY(cudaGetLastError());
  return scan_exclusive(ctx, ctx->plane_flag.as<int>(), ctx->plane_off.as<int>(), (int)t);
}

int plane_write(sg_ctx* ctx, int npairs) {
  const long t = (long)ctx->nb * ctx->np;
  if (t == 0) return SG_OK;
  k_plane_write<<<blocks_for(t), kBlock, 0, ctx->stream>>>(ctx->nb, ctx->np, npairs, ctx->plane_flag.as<int>(),
                                                           ctx->plane_off.as<int>(), ctx->ia.as<int>(), ctx->ib.as<int>());
  SG_CUDA_TRY(cudaGetLastError());
  return SG_OK;
}

int assemble_contacts(sg_ctx* ctx, int nc) {
  if (nc <= 0) return SG_OK;
  AssembleArgs A;
  A.nc = nc;
  A.ia = ctx->ia.as<int>();
  A.ib = ctx->ib.as<int>();
  A.q0 = ctx->q.as<double2>();
  A.v0 = ctx->v.as<double2>();
  A.minv = ctx->minv.as<double>();
  A.plane_n = ctx->plane_n.as<double2>();
  A.plane_t = ctx->plane_t.as<double2>();
  A.mu = ctx->cfg.mu;
  A.CoR = ctx->cfg.CoR;
  A.cache_mode = ctx->cfg.cache_mode;
  A.prev_key = ctx->prev_key.as<unsigned long long>();
  A.prev_ab = ctx->prev_ab.as<double2>();
  A.prev_n = ctx->prev_n;
  if (ctx->prev_color_valid && ctx->prev_n > 0 && ctx->n_scenes == 0 && !ctx->rb2d &&
      ctx->cfg.cache_mode != SG_CACHE_NONE) {
    if (int r = grow(ctx->init_color, sizeof(int) * (size_t)nc)) return r;
    A.prev_color = ctx->prev_color.as<int>();
    A.init_color = ctx->init_color.as<int>();
  }
  if (ctx->prev_rows && ctx->n_scenes == 0 && !ctx->rb2d) {
    A.prev_pair_off = ctx->prev_pair_off.as<int>();
    A.prev_plane_off = ctx->prev_plane_off.as<int>();
    A.prev_plane_flag = ctx->prev_plane_flag.as<int>();
    A.prev_npairs = ctx->prev_npairs;
    A.nb = ctx->nb;
  }
  A.n = ctx->n.as<double2>();
  A.c = ctx->c.as<double2>();
  A.W = ctx->W.as<double>();
  A.mu_out = ctx->mu.as<double>();
  A.r = ctx->r_loc.as<double2>();
  A.key = ctx->key.as<unsigned long long>();
  if (ctx->staggering == SG_STAGGER_STABILIZED) A.v0 = ctx->v1.as<double2>();  // the unconstrained step's
  if (ctx->staggering == SG_STAGGER_SYMPLECTIC_EULER) {
    A.vdelta = ctx->vdelta.as<double2>();
    A.rad = ctx->r.as<double>();
    A.plane_x = ctx->plane_x.as<double2>();
    A.dt = ctx->cfg.dt;
    A.stabilize = ctx->stabilize;
    A.pen_thresh = ctx->pen_thresh;
  }
  k_assemble<<<blocks_for(nc), kBlock, 0, ctx->stream>>>(A);
  SG_CUDA_TRY(cudaGetLastError());
  return SG_OK;
}

int extract_and_cache(sg_ctx* ctx, int nc) {
  if (nc <= 0) return SG_OK;
  k_extract<<<blocks_for(nc), kBlock, 0, ctx->stream>>>(nc, nullptr, ctx->n.as<double2>(), ctx->r_loc.as<double2>(),
                                                        ctx->mu.as<double>(), ctx->cfg.cache_mode, ctx->ab.as<double2>());
  SG_CUDA_TRY(cudaGetLastError());
  return SG_OK;
}

int ball2d_final_map(sg_ctx* ctx, const double* vin) {
  const int nb = ctx->nb;
  if (nb <= 0) return SG_OK;
  if (ctx->staggering != SG_STAGGER_GEOMETRIC && ctx->n_scenes == 0) {
    const bool se = ctx->staggering == SG_STAGGER_SYMPLECTIC_EULER;
    k_final_se<<<blocks_for(nb), kBlock, 0, ctx->stream>>>(nb, ctx->cfg.dt, ctx->q.as<double2>(),
                                                          reinterpret_cast<const double2*>(vin),
                                                          se ? ctx->vdelta.as<double2>() : nullptr,
                                                          ctx->q1.as<double2>(), ctx->v1.as<double2>());
    SG_CUDA_TRY(cudaGetLastError());
    return SG_OK;
  }
  k_final_map<<<blocks_for(nb), kBlock, 0, ctx->stream>>>(nb, ctx->cfg.integrator, ctx->cfg.dt, ctx->cfg.gravity[0],
                                                          ctx->cfg.gravity[1], ctx->q.as<double2>(),
                                                          reinterpret_cast<const double2*>(vin), ctx->m.as<double>(),
                                                          ctx->minv.as<double>(), ctx->q1.as<double2>(),
                                                          ctx->v1.as<double2>());
  SG_CUDA_TRY(cudaGetLastError());
  return SG_OK;
}

// ===========================================================================
// Batched scenes: capacity and one step.
int batch2d_reserve(sg_ctx* ctx, int cap) {
  const size_t c = (size_t)std::max(cap, 1), nb = (size_t)std::max(ctx->nb, 1);
  if (int r = grow(ctx->ia, sizeof(int) * c)) return r;
  if (int r = grow(ctx->ib, sizeof(int) * c)) return r;
  if (int r = grow(ctx->n, sizeof(double) * 2 * c)) return r;
  if (int r = grow(ctx->c, sizeof(double) * 2 * c)) return r;
  if (int r = grow(ctx->W, sizeof(double) * 3 * c)) return r;
  if (int r = grow(ctx->mu, sizeof(double) * c)) return r;
  if (int r = grow(ctx->r_loc, sizeof(double) * 2 * c)) return r;
  if (int r = grow(ctx->cscene, sizeof(int) * c)) return r;
  // The impulse cache keeps its contents across a capacity change.
  for (Buf* b : {&ctx->key, &ctx->prev_key, &ctx->snap_key}) {
    if (b->bytes >= sizeof(unsigned long long) * c && b->p) continue;
    Buf nbuf;
    if (int r = grow(nbuf, sizeof(unsigned long long) * c)) return r;
    SG_CUDA_TRY(cudaMemsetAsync(nbuf.p, 0, nbuf.bytes, ctx->stream));
    if (b->p) SG_CUDA_TRY(cudaMemcpyAsync(nbuf.p, b->p, b->bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    SG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    release(*b);
    *b = nbuf;
  }
  for (Buf* b : {&ctx->ab, &ctx->prev_ab, &ctx->snap_ab}) {
    if (b->bytes >= sizeof(double) * 2 * c && b->p) continue;
    Buf nbuf;
    if (int r = grow(nbuf, sizeof(double) * 2 * c)) return r;
    SG_CUDA_TRY(cudaMemsetAsync(nbuf.p, 0, nbuf.bytes, ctx->stream));
    if (b->p) SG_CUDA_TRY(cudaMemcpyAsync(nbuf.p, b->p, b->bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    SG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    release(*b);
    *b = nbuf;
  }
  if (int r = ensure_solver_capacity(ctx, ctx->nb, (int)c)) return r;
  if (int r = grow(ctx->v2, sizeof(double) * 2 * nb)) return r;
  // FP32 sweep data (packed in colour order) and per-scene mode state.
  if (int r = grow(ctx->pk_ab, sizeof(int2) * c)) return r;
  if (int r = grow(ctx->pk_n, sizeof(float2) * c)) return r;
  if (int r = grow(ctx->pk_c, sizeof(float2) * c)) return r;
  if (int r = grow(ctx->pk_w, sizeof(float4) * c)) return r;
  if (int r = grow(ctx->pk_r, sizeof(float2) * c)) return r;
  if (int r = grow(ctx->pk_scene, sizeof(int) * c)) return r;
  if (int r = grow(ctx->v32, sizeof(float2) * nb)) return r;
  if (int r = grow(ctx->minv32, sizeof(float) * nb)) return r;
  const size_t S = (size_t)std::max(ctx->n_scenes, 1);
  if (int r = grow(ctx->s_mode, sizeof(int) * S)) return r;
  if (int r = grow(ctx->s_since, sizeof(unsigned) * S)) return r;
  if (int r = grow(ctx->s_exc, sizeof(unsigned long long) * 3 * S)) return r;
  if (int r = grow(ctx->s_gmax, sizeof(unsigned long long) * 3)) return r;
  if (int r = grow(ctx->b_work, sizeof(unsigned long long) * 5)) return r;
  // One block per scene: (scene, colour) keys and the contacts in their order.
  const size_t keys = S * kMaxColors + 1;
  if (ctx->s_smax > 0) {
    if (int r = grow(ctx->s_kcnt, sizeof(int) * keys)) return r;
    if (int r = grow(ctx->s_kstart, sizeof(int) * keys)) return r;
    if (int r = grow(ctx->s_kfill, sizeof(int) * keys)) return r;
    if (int r = grow(ctx->s_sperm, sizeof(int) * c)) return r;
    if (int r = grow(ctx->s_next, sizeof(int))) return r;
    if (int r = scene_blocks_prepare(ctx->s_smax)) return r;
  }
  // Scan scratch for the largest scan of a step, so that nothing allocates while capturing.
  const long big = std::max<long>({(long)ctx->nb + 1, ctx->bcells + 1, ctx->bflags + 1, (long)ctx->n_scenes + 1,
                                   (long)c, (long)keys});
  if (int r = grow(ctx->scan_tmp, sizeof(int) * (size_t)(scan_tile_count((int)big) + 2))) return r;
  ctx->bcap = (int)c;
  ctx->ccap = std::min<int64_t>(ctx->ccap, (int64_t)c);
  return SG_OK;
}

int batch2d_step_enqueue(sg_ctx* ctx) {
  const int N = ctx->nb, S = ctx->n_scenes, cap = ctx->bcap;
  cudaStream_t s = ctx->stream;
  if (int r = ball2d_predict_and_bounds(ctx)) return r;
  const double4_32a* aabb = ctx->aabb.as<double4_32a>();
  SceneGrid* grids = ctx->s_grid.as<SceneGrid>();
  k_scene_grid<<<S, kBlock, 0, s>>>(ctx->sb_off.as<int>(), aabb, grids, ctx->s_cells.as<int>());
  SG_CUDA_TRY(cudaGetLastError());
  if (int r = scan_exclusive(ctx, ctx->s_cells.as<int>(), ctx->s_cell_off.as<int>(), S)) return r;
  SG_CUDA_TRY(cudaMemsetAsync(ctx->cell_count.p, 0, sizeof(int) * (size_t)(ctx->bcells + 1), s));
  SG_CUDA_TRY(cudaMemsetAsync(ctx->cell_fill.p, 0, sizeof(int) * (size_t)(ctx->bcells + 1), s));
  k_cell_count_b<<<blocks_for(N), kBlock, 0, s>>>(N, ctx->scene_of.as<int>(), aabb, grids, ctx->s_cell_off.as<int>(),
                                                 ctx->cell_of.as<int>(), ctx->cell_count.as<int>());
  SG_CUDA_TRY(cudaGetLastError());
  if (int r = scan_exclusive(ctx, ctx->cell_count.as<int>(), ctx->cell_start.as<int>(), (int)ctx->bcells)) return r;
  k_cell_scatter<<<blocks_for(N), kBlock, 0, s>>>(N, ctx->cell_of.as<int>(), ctx->cell_start.as<int>(),
                                                 ctx->cell_fill.as<int>(), ctx->sorted.as<int>());
  BatchScan bs{ctx->scene_of.as<int>(), grids,          ctx->s_cell_off.as<int>(), aabb,
               ctx->cell_start.as<int>(), ctx->sorted.as<int>(), ctx->q.as<double2>(), ctx->q1.as<double2>(),
               ctx->r.as<double>()};
  k_pair_count_b<<<blocks_for(N), kBlock, 0, s>>>(N, bs, ctx->pair_cnt.as<int>());
  SG_CUDA_TRY(cudaGetLastError());
  if (int r = scan_exclusive(ctx, ctx->pair_cnt.as<int>(), ctx->pair_off.as<int>(), N)) return r;
  if (ctx->bflags > 0) {
    k_plane_flags_b<<<blocks_for(N), kBlock, 0, s>>>(N, ctx->scene_of.as<int>(), ctx->sb_off.as<int>(),
                                                     ctx->sp_off.as<int>(), ctx->sf_off.as<int>(), ctx->q1.as<double2>(),
                                                     ctx->r.as<double>(), ctx->plane_x.as<double2>(),
                                                     ctx->plane_n.as<double2>(), ctx->plane_flag.as<int>());
    SG_CUDA_TRY(cudaGetLastError());
    if (int r = scan_exclusive(ctx, ctx->plane_flag.as<int>(), ctx->plane_off.as<int>(), (int)ctx->bflags)) return r;
  } else {
    SG_CUDA_TRY(cudaMemsetAsync(ctx->plane_off.p, 0, sizeof(int), s));
  }
  k_scene_counts<<<blocks_for(S), kBlock, 0, s>>>(S, ctx->sb_off.as<int>(), ctx->sf_off.as<int>(),
                                                 ctx->pair_off.as<int>(), ctx->plane_off.as<int>(), ctx->s_nc.as<int>(),
                                                 ctx->s_npairs.as<int>());
  if (int r = scan_exclusive(ctx, ctx->s_nc.as<int>(), ctx->sc_off.as<int>(), S)) return r;
  int* ctl = ctx->b_ctl.as<int>();  // [0] contact count, [1] overflow (largest count seen)
  unsigned long long* sums = ctx->b_sums.as<unsigned long long>();  // [0] contacts, [1] unconverged scene solves
  k_capacity<<<1, 1, 0, s>>>(ctx->sc_off.as<int>() + S, cap, ctl, ctl + 1, sums);
  k_pair_write_b<<<blocks_for(N), kBlock, 0, s>>>(N, bs, ctx->sb_off.as<int>(), ctx->pair_off.as<int>(),
                                                 ctx->sc_off.as<int>(), ctx->pair_cnt.as<int>(), cap,
                                                 ctx->ia.as<int>(), ctx->ib.as<int>());
  if (ctx->bflags > 0)
    k_plane_write_b<<<blocks_for(N), kBlock, 0, s>>>(N, ctx->scene_of.as<int>(), ctx->sb_off.as<int>(),
                                                     ctx->sp_off.as<int>(), ctx->sf_off.as<int>(),
                                                     ctx->plane_flag.as<int>(), ctx->plane_off.as<int>(),
                                                     ctx->sc_off.as<int>(), ctx->s_npairs.as<int>(), cap,
                                                     ctx->ia.as<int>(), ctx->ib.as<int>());
  SG_CUDA_TRY(cudaGetLastError());
  AssembleArgs A;
  A.nc = cap;
  A.ia = ctx->ia.as<int>();
  A.ib = ctx->ib.as<int>();
  A.q0 = ctx->q.as<double2>();
  A.v0 = ctx->v.as<double2>();
  A.minv = ctx->minv.as<double>();
  A.plane_n = ctx->plane_n.as<double2>();
  A.plane_t = ctx->plane_t.as<double2>();
  A.mu = 0.0;
  A.CoR = 0.0;
  A.cache_mode = ctx->cfg.cache_mode;
  A.prev_key = ctx->prev_key.as<unsigned long long>();
  A.prev_ab = ctx->prev_ab.as<double2>();
  A.prev_n = 0;
  A.n = ctx->n.as<double2>();
  A.c = ctx->c.as<double2>();
  A.W = ctx->W.as<double>();
  A.mu_out = ctx->mu.as<double>();
  A.r = ctx->r_loc.as<double2>();
  A.key = ctx->key.as<unsigned long long>();
  k_assemble_b<<<blocks_for(cap), kBlock, 0, s>>>(A, ctl, ctx->scene_of.as<int>(), ctx->s_mu.as<double>(),
                                                 ctx->s_CoR.as<double>(), ctx->prev_sc_off.as<int>(),
                                                 ctx->cscene.as<int>());
  SG_CUDA_TRY(cudaGetLastError());
  ContactProblem P;
  P.nb = N;
  P.nc = cap;
  P.minv = ctx->minv.as<double>();
  P.m = ctx->m.as<double>();
  P.v0 = ctx->v.as<double>();
  P.ia = ctx->ia.as<int>();
  P.ib = ctx->ib.as<int>();
  P.n = ctx->n.as<double>();
  P.c = ctx->c.as<double>();
  P.W = ctx->W.as<double>();
  P.mu = ctx->mu.as<double>();
  P.r = ctx->r_loc.as<double>();
  P.v2 = ctx->v2.as<double>();
  BatchSolve X;
  X.S = S;
  X.nc_dev = ctl;
  X.cscene = ctx->cscene.as<int>();
  X.sc_off = ctx->sc_off.as<int>();
  X.err_slot = ctx->s_err.as<unsigned long long>();
  X.best = ctx->s_best.as<double>();
  X.bestbuf = ctx->s_bestbuf.as<int>();
  X.done = ctx->s_done.as<int>();
  X.iters = ctx->s_iters.as<unsigned>();
  X.done_count = ctl + 2;
  X.unconverged = sums + 1;
  X.pscene = ctx->pk_scene.as<int>();
  X.scene_of = ctx->scene_of.as<int>();
  X.mode = ctx->s_mode.as<int>();
  X.since = ctx->s_since.as<unsigned>();
  X.exc_slot = ctx->s_exc.as<unsigned long long>();
  X.gmax = ctx->s_gmax.as<unsigned long long>();
  X.work = ctx->b_work.as<unsigned long long>();
  X.n64 = ctl + 3;
  if (ctx->s_smax > 0) {
    X.scene_blocks = true;
    X.sb_off = ctx->sb_off.as<int>();
    X.key_cnt = ctx->s_kcnt.as<int>();
    X.key_start = ctx->s_kstart.as<int>();
    X.key_fill = ctx->s_kfill.as<int>();
    X.sperm = ctx->s_sperm.as<int>();
    X.order = ctx->s_order.as<int>();
    X.next = ctx->s_next.as<int>();
    X.smax = ctx->s_smax;
  }
  SolveParams sp{ctx->cfg.tol, ctx->cfg.max_iters, ctx->cfg.eval_every, ctx->cfg.precision};
  if (int r = solve_contacts_batch(ctx, P, sp, X)) return r;
  k_extract<<<blocks_for(cap), kBlock, 0, s>>>(cap, ctl, ctx->n.as<double2>(), ctx->r_loc.as<double2>(),
                                              ctx->mu.as<double>(), ctx->cfg.cache_mode, ctx->ab.as<double2>());
  SG_CUDA_TRY(cudaGetLastError());
  if (int r = ball2d_final_map(ctx, ctx->v2.as<double>())) return r;
  // predictor 1, scene grid 1 + scan 3, cell count 1 + scan 3, scatter 1, pair count 1 + scan 3,
  // plane flags 1 + scan 3, scene counts 1 + scan 3, capacity 1, pair write 1, plane write 1,
  // assemble 1, extract 1, final map 1 (+ the solver's own count)
  ctx->kernel_launches += 25 + (ctx->bflags > 0 ? 5 : 0);
  ctx->steps += 1;
  std::swap(ctx->q, ctx->q1);
  std::swap(ctx->v, ctx->v1);
  if (ctx->cfg.cache_mode != SG_CACHE_NONE) {
    std::swap(ctx->key, ctx->prev_key);
    std::swap(ctx->ab, ctx->prev_ab);
    std::swap(ctx->sc_off, ctx->prev_sc_off);
  }
  return SG_OK;
}

int ccd_batch(sg_ctx* ctx, int n, const double* q0a, const double* q1a, const double* ra, const double* q0b,
              const double* q1b, const double* rb, double* coeffs, int* hit, double* t) {
  if (n <= 0) return SG_OK;
  k_ccd_batch<<<blocks_for(n), kBlock, 0, ctx->stream>>>(
      n, reinterpret_cast<const double2*>(q0a), reinterpret_cast<const double2*>(q1a), ra,
      reinterpret_cast<const double2*>(q0b), reinterpret_cast<const double2*>(q1b), rb, coeffs, hit, t);
  SG_CUDA_TRY(cudaGetLastError());
  return SG_OK;
}

}  // namespace sg
