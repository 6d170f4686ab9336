// solver_kernels.cu -- graph-coloured block Gauss-Seidel Coulomb solve (FP64).
//
// The GPU form of Balls2DSobogusInterface::solve (scisim/ConstrainedMaps/bogus/
// Ball2DSobogusInterface.cpp:102-148) and So-bogus's GaussSeidel + SOCLaw<2,double,true>.
// The dual problem u = W r + b is evaluated matrix-free through body velocities
// v = v0 + M^-1 H^T r: a contact's update reads the velocities of its two bodies,
// solves the 2x2 local Coulomb problem with the diagonal block W_ii, and pushes
// the impulse change back into the velocities.  Contacts of one colour share no
// body, so a colour is one parallel phase; colours are separated by a bounded
// grid barrier inside one persistent cooperative kernel per solve.
//
// Stages (all on the context stream):
//   k_body_count/k_body_fill/k_body_sort  body -> contacts adjacency (ascending contact order)
//   k_vel_init                             v = v0 + Minv H^T r_warm
//   k_color_jp  (cooperative)              Jones-Plassmann colouring with hashed priorities,
//                                          then the colour-ordered processing permutation
//   k_gs        (cooperative)              sweeps, FB residual every eval_every sweeps,
//                                          best-iterate tracking, early exit at tol
//   k_final_velocity                       v2 = Minv (H^T r - f), f = -M v0
#include "ctx.hpp"
#include "coulomb2d.cuh"
#include "ffloat.hpp"
#include "na_cache.hpp"

#include <cuda.h>

#include <algorithm>
#include <cstring>

namespace sg {
namespace {

constexpr int kBlock = 256;
constexpr int kGsBlock = 512;    // FP64 sweep kernel: one fat block per SM (fewer barrier arrivals)
constexpr int kGs32Block = 768;  // FP32 sweep kernel: enough threads for the largest colours
constexpr int kPatchBlock = 384;  // two-level kernel
constexpr int kColorBlock = 1024;  // colouring kernel
// FP32 form: the one-level FP64 sweeps of the probe that starts every solve.  A solve that needs
// more goes on on the two-level partition, whose setup (~1 ms at 500k contacts) pays back after
// about six of its sweeps; steps of a settled pile mostly need 2-8.
constexpr unsigned kFp64Probe = 8;
// FP32 form, two_level 1: one-level FP64 sweeps after the probe before the two-level partition.
constexpr unsigned kOneLevel64 = 160;
inline int blocks_for(long n) { return (int)((n + kBlock - 1) / kBlock); }

// u = H v + c for contact k (body b < 0: static).
__device__ __forceinline__ void local_velocity(const double2 nk, const double2 ck, const double2 va, bool has_b,
                                               const double2 vb, double& u0, double& u1) {
  const double nx = nk.x, ny = nk.y, tx = -ny, ty = nx;
  double hn = nx * va.x + ny * va.y;
  double ht = tx * va.x + ty * va.y;
  if (has_b) {
    hn = hn - (nx * vb.x + ny * vb.y);
    ht = ht - (tx * vb.x + ty * vb.y);
  }
  u0 = hn + ck.x;
  u1 = ht + ck.y;
}

// ---------------------------------------------------------------------------
// nc_dev (optional): the contact count on the device, for launches sized to a capacity.
__global__ void k_body_count(int nc, const int* __restrict__ nc_dev, const int* __restrict__ ia,
                             const int* __restrict__ ib, int* __restrict__ cnt) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (nc_dev) nc = *nc_dev;
  if (k >= nc) return;
  atomicAdd(&cnt[ia[k]], 1);
  const int b = ib[k];
  if (b >= 0) atomicAdd(&cnt[b], 1);
}

__global__ void k_body_fill(int nc, const int* __restrict__ nc_dev, const int* __restrict__ ia,
                            const int* __restrict__ ib, const int* __restrict__ off, int* __restrict__ fill,
                            int* __restrict__ adj) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (nc_dev) nc = *nc_dev;
  if (k >= nc) return;
  const int a = ia[k];
  adj[off[a] + atomicAdd(&fill[a], 1)] = k;
  const int b = ib[k];
  if (b >= 0) adj[off[b] + atomicAdd(&fill[b], 1)] = k;
}

__global__ void k_body_sort(int nb, const int* __restrict__ off, int* __restrict__ adj) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const int s = off[i], e = off[i + 1];
  for (int p = s + 1; p < e; ++p) {
    const int x = adj[p];
    int q = p;
    while (q > s && adj[q - 1] > x) {
      adj[q] = adj[q - 1];
      --q;
    }
    adj[q] = x;
  }
}

// H^T r gathered per body in ascending contact order.
__device__ __forceinline__ void gather_htr(int body, const int* __restrict__ off, const int* __restrict__ adj,
                                           const int* __restrict__ ia, const double2* __restrict__ n,
                                           const double2* __restrict__ r, double& hx, double& hy) {
  hx = 0.0;
  hy = 0.0;
  const int e = off[body + 1];
  for (int p = off[body]; p < e; ++p) {
    const int k = adj[p];
    const double sgn = (ia[k] == body) ? 1.0 : -1.0;
    const double2 nk = n[k], rk = r[k];
    const double tx = -nk.y, ty = nk.x;
    const double px = nk.x * rk.x + tx * rk.y;
    const double py = nk.y * rk.x + ty * rk.y;
    hx = hx + sgn * px;
    hy = hy + sgn * py;
  }
}

__global__ void k_vel_init(int nb, const int* __restrict__ off, const int* __restrict__ adj, const int* __restrict__ ia,
                           const double2* __restrict__ n, const double2* __restrict__ r, const double2* __restrict__ v0,
                           const double* __restrict__ minv, double2* __restrict__ v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  double hx, hy;
  gather_htr(i, off, adj, ia, n, r, hx, hy);
  const double2 a = v0[i];
  const double mi = minv[i];
  v[i] = make_double2(a.x + mi * hx, a.y + mi * hy);
}

__global__ void k_final_velocity(int nb, const int* __restrict__ off, const int* __restrict__ adj,
                                 const int* __restrict__ ia, const double2* __restrict__ n, const double2* __restrict__ r,
                                 const double2* __restrict__ v0, const double* __restrict__ m,
                                 const double* __restrict__ minv, double2* __restrict__ v2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const double2 a = v0[i];
  if (off[i + 1] == off[i]) {
    v2[i] = a;
    return;
  }
  double hx, hy;
  gather_htr(i, off, adj, ia, n, r, hx, hy);
  const double fx = -(m[i] * a.x);
  const double fy = -(m[i] * a.y);
  const double mi = minv[i];
  v2[i] = make_double2(mi * (hx - fx), mi * (hy - fy));
}

// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned hash_prio(unsigned k) {
  k ^= k >> 16;
  k *= 0x7feb352du;
  k ^= k >> 15;
  k *= 0x846ca68bu;
  k ^= k >> 16;
  return k;
}
__device__ __forceinline__ bool prio_greater(unsigned pj, int j, unsigned pk, int k) {
  return pj > pk || (pj == pk && j > k);
}

struct ColorArgs {
  int nc;
  const int* nc_dev;  // optional device-side count (overrides nc)
  const int* ia;
  const int* ib;
  const int* body_off;
  const int* body_adj;
  int* color;  // packed (round << 8) | colour, -1 uncoloured
  int* perm;
  SolveStats* st;
  GridBarrier* gb;
  unsigned long long spin;
  int max_rounds;
  // Warm start: contacts with a colour >= 0 on entry keep it (colours of an earlier step, valid
  // among themselves) and the Jones-Plassmann rounds begin at 1, so those count as coloured before
  // them; then ig_passes recolouring passes.
  int first_round = 0;
  int ig_passes = 3;
};

__global__ void __launch_bounds__(kColorBlock, 1) k_color_jp(ColorArgs A) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nthr = gridDim.x * blockDim.x;
  if (A.nc_dev) A.nc = *A.nc_dev;
  volatile int* vcolor = A.color;
  for (int round = A.first_round;; ++round) {
    if (round >= A.max_rounds) {
      if (tid == 0) atomicExch(&A.st->status, (int)SG_CAPACITY);
      return;
    }
    int rem = 0;
    for (int k = tid; k < A.nc; k += nthr) {
      if (vcolor[k] >= 0) continue;
      const unsigned pk = hash_prio((unsigned)k);
      unsigned long long used = 0ull;
      bool is_max = true;
      const int bodies[2] = {A.ia[k], A.ib[k]};
      for (int bi = 0; bi < 2 && is_max; ++bi) {
        const int body = bodies[bi];
        if (body < 0) continue;
        const int e = A.body_off[body + 1];
        for (int p = A.body_off[body]; p < e; ++p) {
          const int j = A.body_adj[p];
          if (j == k) continue;
          const int cj = vcolor[j];
          if (cj >= 0 && (cj >> 8) < round) {
            used |= 1ull << (cj & 63);
          } else if (prio_greater(hash_prio((unsigned)j), j, pk, k)) {
            is_max = false;
            break;
          }
        }
      }
      if (is_max) {
        const unsigned long long freec = ~used;
        if (freec == 0ull) {
          atomicExch(&A.st->status, (int)SG_CAPACITY);
          vcolor[k] = (round << 8) | 63;
        } else {
          vcolor[k] = (round << 8) | (__ffsll((long long)freec) - 1);
        }
      } else {
        ++rem;
      }
    }
    rem = warp_sum(rem);
    if ((threadIdx.x & 31) == 0 && rem) atomicAdd(&A.st->remaining[round % 3], rem);
    if (tid == 0) A.st->remaining[(round + 1) % 3] = 0;
    if (!grid_sync(A.gb, A.spin)) {
      if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
      return;
    }
    const int left = *((volatile int*)&A.st->remaining[round % 3]);
    if (left == 0) break;
  }
  // Iterated greedy recolouring (Culberson): re-colour the classes one at a time in
  // reverse order, each vertex taking the smallest colour unused by the neighbours
  // already re-coloured in this pass.  A class is an independent set, so a class is
  // re-coloured in parallel; a pass never adds colours and usually removes some.
  // A.perm serves as the new-colour array until the permutation is built.
  {
    int cmax_local = 0;
    for (int k = tid; k < A.nc; k += nthr) {
      const int c = vcolor[k] & 63;
      vcolor[k] = c;
      cmax_local = max(cmax_local, c);
    }
    for (int o = 16; o > 0; o >>= 1) cmax_local = max(cmax_local, __shfl_down_sync(0xffffffffu, cmax_local, o));
    if ((threadIdx.x & 31) == 0) atomicMax(&A.st->n_colors, cmax_local);
    if (!grid_sync(A.gb, A.spin)) {
      if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
      return;
    }
    int cmax = *((volatile int*)&A.st->n_colors);
    volatile int* vnew = A.perm;
    for (int pass = 0; pass < A.ig_passes; ++pass) {
      for (int k = tid; k < A.nc; k += nthr) vnew[k] = -1;
      if (!grid_sync(A.gb, A.spin)) {
        if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
        return;
      }
      int newmax = 0;
      for (int c = cmax; c >= 0; --c) {
        for (int k = tid; k < A.nc; k += nthr) {
          if (vcolor[k] != c) continue;
          unsigned long long used = 0ull;
          const int bodies[2] = {A.ia[k], A.ib[k]};
          for (int bi = 0; bi < 2; ++bi) {
            const int body = bodies[bi];
            if (body < 0) continue;
            const int e = A.body_off[body + 1];
            for (int p = A.body_off[body]; p < e; ++p) {
              const int j = A.body_adj[p];
              const int cj = vnew[j];
              if (j != k && cj >= 0) used |= 1ull << cj;
            }
          }
          int nc_k = __ffsll((long long)~used) - 1;
          if (nc_k < 0) {
            atomicExch(&A.st->status, (int)SG_CAPACITY);
            nc_k = 63;
          }
          vnew[k] = nc_k;
          newmax = max(newmax, nc_k);
        }
        if (!grid_sync(A.gb, A.spin)) {
          if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
          return;
        }
      }
      for (int k = tid; k < A.nc; k += nthr) vcolor[k] = vnew[k];
      for (int o = 16; o > 0; o >>= 1) newmax = max(newmax, __shfl_down_sync(0xffffffffu, newmax, o));
      if ((threadIdx.x & 31) == 0) atomicMax(&A.st->ig_max[pass], newmax);
      if (!grid_sync(A.gb, A.spin)) {
        if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
        return;
      }
      cmax = *((volatile int*)&A.st->ig_max[pass]);
    }
  }
  // Colour histogram.
  __shared__ int hist[kMaxColors];
  for (int c = threadIdx.x; c < kMaxColors; c += blockDim.x) hist[c] = 0;
  __syncthreads();
  for (int k = tid; k < A.nc; k += nthr) atomicAdd(&hist[vcolor[k] & 63], 1);
  __syncthreads();
  for (int c = threadIdx.x; c < kMaxColors; c += blockDim.x)
    if (hist[c]) atomicAdd(&A.st->color_count[c], hist[c]);
  if (!grid_sync(A.gb, A.spin)) {
    if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
    return;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    int off = 0, ncol = 0;
    for (int c = 0; c < kMaxColors; ++c) {
      A.st->color_off[c] = off;
      const int cc = A.st->color_count[c];
      off += cc;
      if (cc) ncol = c + 1;
    }
    A.st->color_off[kMaxColors] = off;
    A.st->n_colors = ncol;
  }
  if (!grid_sync(A.gb, A.spin)) {
    if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
    return;
  }
  for (int k = tid; k < A.nc; k += nthr) {
    const int c = vcolor[k] & 63;
    A.perm[*((volatile int*)&A.st->color_off[c]) + atomicAdd(&A.st->color_fill[c], 1)] = k;
  }
}

// ---------------------------------------------------------------------------
struct GsArgs {
  int nc;
  const int* ia;
  const int* ib;
  const double2* n;
  const double2* c;
  const double* W;
  const double* mu;
  const double* minv;
  const int* perm;
  double2* r;
  double2* r_a;  // snapshot buffers for best-iterate tracking
  double2* r_b;
  double2* v;
  SolveStats* st;
  GridBarrier* gb;
  unsigned long long spin;
  double tol;
  unsigned max_iters;
  unsigned eval_every;
  int iso = 0;  // isotropic blocks take local_solve_2d_iso (the FP32 form's FP64 sweeps)
  unsigned first_eval = 1;  // k_gs: no residual check before this sweep (the FP32 form's probe: 2)
  unsigned eval_stride = 1; // k_gs: after sweep 4, checks every eval_stride sweeps (the probe: 2)
};

__device__ __forceinline__ void gs_update(const GsArgs& A, int k) {
  const int a = A.ia[k], b = A.ib[k];
  const double2 nk = A.n[k], ck = A.c[k];
  // Velocities and impulses are written by other SMs between grid barriers: read
  // them at L2 (ld.global.cg) so a stale L1 line is never used.
  const double2 va = __ldcg(&A.v[a]);
  const bool has_b = b >= 0;
  const double2 vb = has_b ? __ldcg(&A.v[b]) : make_double2(0.0, 0.0);
  double u0, u1;
  local_velocity(nk, ck, va, has_b, vb, u0, u1);
  const double2 rk = __ldcg(&A.r[k]);
  const double r0 = rk.x, r1 = rk.y;
  const double w00 = A.W[3 * k], w01 = A.W[3 * k + 1], w11 = A.W[3 * k + 2];
  const double bt0 = u0 - (w00 * r0 + w01 * r1);
  const double bt1 = u1 - (w01 * r0 + w11 * r1);
  double rn0, rn1;
  if (A.iso && w01 == 0.0 && w00 == w11)
    local_solve_2d_iso(w00, bt0, bt1, A.mu[k], rn0, rn1);
  else
    local_solve_2d(w00, w01, w11, bt0, bt1, A.mu[k], rn0, rn1);
  const double d0 = rn0 - r0, d1 = rn1 - r1;
  const double nx = nk.x, ny = nk.y, tx = -ny, ty = nx;
  const double px = nx * d0 + tx * d1;
  const double py = ny * d0 + ty * d1;
  const double ma = A.minv[a];
  A.v[a] = make_double2(va.x + ma * px, va.y + ma * py);
  if (has_b) {
    const double mb = A.minv[b];
    A.v[b] = make_double2(vb.x - mb * px, vb.y - mb * py);
  }
  A.r[k] = make_double2(rn0, rn1);
}

__global__ void __launch_bounds__(kGsBlock, 1) k_gs(GsArgs A) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nthr = gridDim.x * blockDim.x;
  // A colouring that gave up (timeout or capacity) leaves no valid permutation.
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
  unsigned it = 0;
  unsigned n_eval = 0;
  for (it = 1; it <= A.max_iters; ++it) {
    for (int col = 0; col < ncol; ++col) {
      const int e = s_off[col + 1];
      for (int s = s_off[col] + tid; s < e; s += nthr) gs_update(A, A.perm[s]);
      if (!grid_sync(A.gb, A.spin)) {
        if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
        return;
      }
    }
    if (it % eval_every == 0 && it >= A.first_eval && (it <= 4 || it % A.eval_stride == 0 || it == A.max_iters)) {
      double emax = 0.0;
      for (int k = tid; k < A.nc; k += nthr) {
        const int a = A.ia[k], b = A.ib[k];
        const bool has_b = b >= 0;
        const double2 va = __ldcg(&A.v[a]);
        const double2 vb = has_b ? __ldcg(&A.v[b]) : make_double2(0.0, 0.0);
        double u0, u1;
        local_velocity(A.n[k], A.c[k], va, has_b, vb, u0, u1);
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
    // Return the best iterate (GaussSeidel: x = x_best when GSIter > maxIters).
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

// ---------------------------------------------------------------------------
// Batched scenes: one coloured sweep over the contacts of all scenes (scenes share no
// body, so the global colouring is a colouring of every scene), with each scene's own
// residual, best iterate, convergence test and iteration count, as if every scene were
// solved alone (Sobogus::solve per Ball2DSim).  A converged scene's contacts stop
// updating; the kernel ends when every scene has converged or at max_iters.
struct GsBatchArgs {
  GsArgs g;              // g.nc unused; g.r_a / g.r_b are the two snapshot buffers
  const int* nc_dev;     // contact count on the device
  const int* cscene;     // contact -> scene
  const int* sc_off;     // scene contact offsets (S + 1)
  int S;
  unsigned long long* err_slot;  // 3 S ordered residual maxima (rotating)
  double* best;                  // S
  int* bestbuf;                  // S: which snapshot buffer holds the scene's best iterate
  int* done;                     // S: converged (or no contacts)
  unsigned* iters;               // S
  int* done_count;
  unsigned long long* unconverged;  // running count of scene solves that hit max_iters
  unsigned long long* work;         // [1] FP64 contact updates, [2] contact evaluations
};

// Max of v over the lanes of each run of equal keys (runs are contiguous lanes); the
// first lane of each run with key >= 0 adds it to slots[key].
__device__ __forceinline__ void run_max_atomic(unsigned long long v, int key, unsigned long long* slots) {
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

__global__ void __launch_bounds__(kGsBlock, 1) k_gs_batch(GsBatchArgs B) {
  const GsArgs& A = B.g;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nthr = gridDim.x * blockDim.x;
  if (*((volatile int*)&A.st->status) != 0) return;
  __shared__ int s_off[kMaxColors + 1];
  __shared__ int s_ncol;
  if (threadIdx.x == 0) s_ncol = A.st->n_colors;
  for (int c = threadIdx.x; c <= kMaxColors; c += blockDim.x) s_off[c] = A.st->color_off[c];
  const int nc = *B.nc_dev;
  const int S = B.S;
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
  double2* bufs[2] = {A.r_a, A.r_b};
  if (!grid_sync(A.gb, A.spin)) {
    if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
    return;
  }
  unsigned n_eval = 0;
  unsigned it = 0;
  unsigned long long n64w = 0, nevw = 0;
  if (*((volatile int*)B.done_count) < S) {
    for (it = 1; it <= A.max_iters; ++it) {
      for (int col = 0; col < ncol; ++col) {
        const int e = s_off[col + 1];
        for (int s = s_off[col] + tid; s < e; s += nthr) {
          const int k = A.perm[s];
          if (__ldcg(&B.done[B.cscene[k]])) continue;
          gs_update(A, k);
          ++n64w;
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
          const int sc = B.cscene[k];
          if (!__ldcg(&B.done[sc])) {
            const int a = A.ia[k], b = A.ib[k];
            const bool has_b = b >= 0;
            const double2 va = __ldcg(&A.v[a]);
            const double2 vb = has_b ? __ldcg(&A.v[b]) : make_double2(0.0, 0.0);
            double u0, u1;
            local_velocity(A.n[k], A.c[k], va, has_b, vb, u0, u1);
            const double2 rk = __ldcg(&A.r[k]);
            bufs[1 - __ldcg(&B.bestbuf[sc])][k] = rk;
            v = f64_to_ordered(fb_error_2d(rk.x, rk.y, u0, u1, A.mu[k]));
            key = sc;
            ++nevw;
          }
        }
        run_max_atomic(v, key, slots);
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
    const int sc = B.cscene[k];
    if (__ldcg(&B.done[sc])) continue;
    if (__ldcg(&B.best[sc]) < INFINITY) A.r[k] = __ldcg(&bufs[__ldcg(&B.bestbuf[sc])][k]);
  }
  for (int sc = tid; sc < S; sc += nthr)
    if (!__ldcg(&B.done[sc])) B.iters[sc] = A.max_iters;
  if (tid == 0) *B.unconverged += (unsigned long long)(S - *((volatile int*)B.done_count));
  atomicAdd(&B.work[1], n64w);
  atomicAdd(&B.work[2], nevw);
  if (tid == 0) {
    A.st->iterations = it > A.max_iters ? A.max_iters : it;
    A.st->sweeps64 = it > A.max_iters ? A.max_iters : it;
    A.st->evals = n_eval;
  }
}

// ---------------------------------------------------------------------------
// Mixed precision: FP32 sweeps over colour-packed FP32 copies of the contact data,
// FP64 residual on the FP64 image of the iterate every eval32 sweeps, and FP64
// sweeps to finish (a closing refinement sweep once FP32 reaches tol, or FP64
// sweeps from the point where FP32 stops making progress near tol).
__device__ __forceinline__ void local_solve_2d_f(float w00, float w01, float w11, float b0, float b1, float mu,
                                                 float& r0, float& r1) {
  if (b0 >= 0.0f) {
    r0 = 0.0f;
    r1 = 0.0f;
    return;
  }
  const float det = w00 * w11 - w01 * w01;
  const float rs0 = (w01 * b1 - w11 * b0) / det;
  const float rs1 = (w01 * b0 - w00 * b1) / det;
  if (rs0 >= 0.0f && fabsf(rs1) <= mu * rs0) {
    r0 = rs0;
    r1 = rs1;
    return;
  }
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const float s = (k == 0) ? 1.0f : -1.0f;
    const float den = w00 - s * mu * w01;
    if (!(den > 0.0f)) continue;
    const float rn = -b0 / den;
    const float rt = -s * mu * rn;
    const float ut = w01 * rn + w11 * rt + b1;
    if (s * ut >= 0.0f) {
      r0 = rn;
      r1 = rt;
      return;
    }
  }
  // Degenerate local problem in FP32: project the stick solution onto the cone.
  const float rn = fmaxf(rs0, 0.0f);
  r0 = rn;
  r1 = fminf(fmaxf(rs1, -mu * rn), mu * rn);
}

struct Gs32Args {
  const int2* ab;    // (ia, ib) in colour order
  const float2* n;   // normal
  const float2* c;   // local forcing
  const float4* w;   // w00, w01, w11, mu
  float2* r;         // local impulse
  float2* v;         // running body velocity
  const float* minv;
  const double* minv64;
  const double2* v0;
  const int* body_off;
  const int* body_adj;
  int nb;
  unsigned eval32;
  // FP64 sweeps take over once the FP64 residual is at or below fp64_below (and from the first
  // sweep with fp64_start: a start already that close to tol).
  double fp64_below = 0.0;
  int fp64_start = 0;
  int fp64_local = 1;  // k_gs_patch: FP64 sweeps on the two-level partition (0: one-level colours)
};

// The velocity-independent data of one packed contact (prefetched before the
// barrier that precedes its colour).
struct C32 {
  int2 ab;
  float2 n, c;
  float4 w;
  float2 r;
};

__device__ __forceinline__ C32 load32(const Gs32Args& B, int s) {
  C32 x;
  x.ab = B.ab[s];
  x.n = B.n[s];
  x.c = B.c[s];
  x.w = B.w[s];
  x.r = __ldcg(&B.r[s]);  // written only by this thread, in the previous sweep
  return x;
}

__device__ __forceinline__ void apply32(const Gs32Args& B, int s, const C32& x) {
  const int2 ab = x.ab;
  const float2 nk = x.n, ck = x.c;
  const float4 w = x.w;
  const float2 va = __ldcg(&B.v[ab.x]);
  const bool has_b = ab.y >= 0;
  const float2 vb = has_b ? __ldcg(&B.v[ab.y]) : make_float2(0.0f, 0.0f);
  const float nx = nk.x, ny = nk.y, tx = -ny, ty = nx;
  float hn = nx * va.x + ny * va.y;
  float ht = tx * va.x + ty * va.y;
  if (has_b) {
    hn -= nx * vb.x + ny * vb.y;
    ht -= tx * vb.x + ty * vb.y;
  }
  const float u0 = hn + ck.x, u1 = ht + ck.y;
  const float2 rk = x.r;
  const float bt0 = u0 - (w.x * rk.x + w.y * rk.y);
  const float bt1 = u1 - (w.y * rk.x + w.z * rk.y);
  float rn0, rn1;
  local_solve_2d_f(w.x, w.y, w.z, bt0, bt1, w.w, rn0, rn1);
  const float d0 = rn0 - rk.x, d1 = rn1 - rk.y;
  const float px = nx * d0 + tx * d1, py = ny * d0 + ty * d1;
  const float ma = B.minv[ab.x];
  B.v[ab.x] = make_float2(va.x + ma * px, va.y + ma * py);
  if (has_b) {
    const float mb = B.minv[ab.y];
    B.v[ab.y] = make_float2(vb.x - mb * px, vb.y - mb * py);
  }
  B.r[s] = make_float2(rn0, rn1);
}

__device__ __forceinline__ void gs_update32(const Gs32Args& B, int s) {
  const int2 ab = B.ab[s];
  const float2 nk = B.n[s], ck = B.c[s];
  const float4 w = B.w[s];
  const float2 va = __ldcg(&B.v[ab.x]);
  const bool has_b = ab.y >= 0;
  const float2 vb = has_b ? __ldcg(&B.v[ab.y]) : make_float2(0.0f, 0.0f);
  const float nx = nk.x, ny = nk.y, tx = -ny, ty = nx;
  float hn = nx * va.x + ny * va.y;
  float ht = tx * va.x + ty * va.y;
  if (has_b) {
    hn -= nx * vb.x + ny * vb.y;
    ht -= tx * vb.x + ty * vb.y;
  }
  const float u0 = hn + ck.x, u1 = ht + ck.y;
  const float2 rk = __ldcg(&B.r[s]);
  const float bt0 = u0 - (w.x * rk.x + w.y * rk.y);
  const float bt1 = u1 - (w.y * rk.x + w.z * rk.y);
  float rn0, rn1;
  local_solve_2d_f(w.x, w.y, w.z, bt0, bt1, w.w, rn0, rn1);
  const float d0 = rn0 - rk.x, d1 = rn1 - rk.y;
  const float px = nx * d0 + tx * d1, py = ny * d0 + ty * d1;
  const float ma = B.minv[ab.x];
  B.v[ab.x] = make_float2(va.x + ma * px, va.y + ma * py);
  if (has_b) {
    const float mb = B.minv[ab.y];
    B.v[ab.y] = make_float2(vb.x - mb * px, vb.y - mb * py);
  }
  B.r[s] = make_float2(rn0, rn1);
}

__global__ void k_pack32(int nc, const int* __restrict__ perm, const int* __restrict__ ia, const int* __restrict__ ib,
                         const double2* __restrict__ n, const double2* __restrict__ c, const double* __restrict__ W,
                         const double* __restrict__ mu, const double2* __restrict__ r, int2* __restrict__ ab,
                         float2* __restrict__ n32, float2* __restrict__ c32, float4* __restrict__ w32,
                         float2* __restrict__ r32) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nc) return;
  const int k = perm[s];
  const int b = ib[k];
  ab[s] = make_int2(ia[k], b >= 0 ? b : -1);
  const double2 nk = n[k], ck = c[k], rk = r[k];
  n32[s] = make_float2((float)nk.x, (float)nk.y);
  c32[s] = make_float2((float)ck.x, (float)ck.y);
  w32[s] = make_float4((float)W[3 * k], (float)W[3 * k + 1], (float)W[3 * k + 2], (float)mu[k]);
  r32[s] = make_float2((float)rk.x, (float)rk.y);
}

// Batched packing: device-side count; also the scene of every packed contact.
__global__ void k_pack32_b(const int* __restrict__ nc_dev, const int* __restrict__ perm, const int* __restrict__ ia,
                           const int* __restrict__ ib, const double2* __restrict__ n, const double2* __restrict__ c,
                           const double* __restrict__ W, const double* __restrict__ mu, const double2* __restrict__ r,
                           const int* __restrict__ cscene, int2* __restrict__ ab, float2* __restrict__ n32,
                           float2* __restrict__ c32, float4* __restrict__ w32, float2* __restrict__ r32,
                           int* __restrict__ pscene) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= *nc_dev) return;
  const int k = perm[s];
  const int b = ib[k];
  ab[s] = make_int2(ia[k], b >= 0 ? b : -1);
  const double2 nk = n[k], ck = c[k], rk = r[k];
  n32[s] = make_float2((float)nk.x, (float)nk.y);
  c32[s] = make_float2((float)ck.x, (float)ck.y);
  w32[s] = make_float4((float)W[3 * k], (float)W[3 * k + 1], (float)W[3 * k + 2], (float)mu[k]);
  r32[s] = make_float2((float)rk.x, (float)rk.y);
  pscene[s] = cscene[k];
}

__global__ void k_vel32(int nb, const double2* __restrict__ v, const double* __restrict__ minv, float2* __restrict__ v32,
                        float* __restrict__ minv32) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const double2 a = v[i];
  v32[i] = make_float2((float)a.x, (float)a.y);
  minv32[i] = (float)minv[i];
}

__global__ void __launch_bounds__(kGs32Block, 1) k_gs_mixed(GsArgs A, Gs32Args B) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nthr = gridDim.x * blockDim.x;
  if (*((volatile int*)&A.st->status) != 0) return;
  __shared__ int s_off[kMaxColors + 1];
  __shared__ int s_ncol;
  if (threadIdx.x == 0) s_ncol = A.st->n_colors;
  for (int c = threadIdx.x; c <= kMaxColors; c += blockDim.x) s_off[c] = A.st->color_off[c];
  __syncthreads();
  const int ncol = s_ncol;
  // Trailing colours with at most two contacts per thread of one block form the tail.
  int tail = ncol;
  while (tail > 0 && s_off[tail] - s_off[tail - 1] <= 2 * (int)blockDim.x) --tail;
  const unsigned eval64 = A.eval_every ? A.eval_every : 1u;
  const unsigned eval32 = B.eval32 ? B.eval32 : 1u;
  double2* best = A.r_a;
  double2* cand = A.r_b;
  double err_best = INFINITY;
  bool converged = false, fp64 = B.fp64_start != 0;
  unsigned it = 0, n_eval = 0, s32 = 0, s64 = 0, lifts = 0, since_best = 0;
  unsigned next_eval = 1, interval = eval32;
  // FP64 sweeps' checks as in k_gs_patch64: where the residual's rate over the last two checks
  // predicts tol, at most 16 eval64 apart, the gap doubling where the residual did not decrease.
  unsigned next64 = 0, interval64 = eval64, prev64_it = 0;
  double prev64_err = INFINITY;
  C32 pf;
  bool have_pf = false, have_pf_valid = false;
  for (it = 1; it <= A.max_iters; ++it) {
    bool do_eval;
    if (!fp64) {
      // Each thread's first contact of the next colour is loaded before the barrier
      // that precedes it; after the barrier only the two body velocities remain.
      if (!have_pf_valid) {
        const int s0 = s_off[0] + tid;
        have_pf = tail > 0 && s0 < s_off[1];
        if (have_pf) pf = load32(B, s0);
        have_pf_valid = true;
      }
      for (int col = 0; col < tail; ++col) {
        const int s0 = s_off[col] + tid, e = s_off[col + 1];
        const C32 cur = pf;
        const bool have = have_pf;
        const int nxt = (col + 1 < tail) ? col + 1 : 0;
        const int sn = s_off[nxt] + tid;
        have_pf = sn < s_off[nxt + 1];
        if (have_pf && nxt != 0) pf = load32(B, sn);
        if (have) apply32(B, s0, cur);
        for (int s = s0 + nthr; s < e; s += nthr) gs_update32(B, s);
        if (nxt == 0 && have_pf) pf = load32(B, sn);  // colour 0 of the next sweep, after our own writes
        if (!grid_sync(A.gb, A.spin)) {
          if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
          return;
        }
      }
      if (tail < ncol) {
        // The small trailing colours run in block 0 alone, separated by block
        // barriers, then one grid barrier (instead of one grid barrier each).
        if (blockIdx.x == 0) {
          for (int col = tail; col < ncol; ++col) {
            for (int s = s_off[col] + threadIdx.x; s < s_off[col + 1]; s += blockDim.x) gs_update32(B, s);
            __syncthreads();
          }
        }
        if (!grid_sync(A.gb, A.spin)) {
          if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
          return;
        }
      }
      ++s32;
      // FP64 checks after sweeps 1, 2, 4, ... eval32, then at an interval that grows
      // (up to 16 eval32) while the residual is far above tol: a check costs several
      // sweeps, and the final check at max_iters always happens.
      do_eval = it == next_eval || it == A.max_iters;
      if (do_eval) {
        // Lift the FP32 iterate to FP64: impulses, then body velocities v = v0 + Minv H^T r.
        for (int s = tid; s < A.nc; s += nthr) {
          const float2 r32 = __ldcg(&B.r[s]);
          A.r[A.perm[s]] = make_double2((double)r32.x, (double)r32.y);
        }
        if (!grid_sync(A.gb, A.spin)) {
          if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
          return;
        }
        for (int i = tid; i < B.nb; i += nthr) {
          double hx = 0.0, hy = 0.0;
          const int e = B.body_off[i + 1];
          for (int p = B.body_off[i]; p < e; ++p) {
            const int k = B.body_adj[p];
            const double sgn = (A.ia[k] == i) ? 1.0 : -1.0;
            const double2 nk = A.n[k], rk = __ldcg(&A.r[k]);
            const double px = nk.x * rk.x + (-nk.y) * rk.y;
            const double py = nk.y * rk.x + nk.x * rk.y;
            hx = hx + sgn * px;
            hy = hy + sgn * py;
          }
          const double2 a = B.v0[i];
          const double mi = B.minv64[i];
          const double2 vi = make_double2(a.x + mi * hx, a.y + mi * hy);
          A.v[i] = vi;
          // Resynchronise the FP32 running velocity with the impulses: removes the
          // rounding drift that incremental FP32 updates accumulate.
          B.v[i] = make_float2((float)vi.x, (float)vi.y);
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
        for (int s = s_off[col] + tid; s < e; s += nthr) gs_update(A, A.perm[s]);
        if (!grid_sync(A.gb, A.spin)) {
          if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
          return;
        }
      }
      ++s64;
      if (next64 == 0) next64 = it + eval64 - 1;  // the first FP64 sweep: a check eval64 sweeps on
      do_eval = it >= next64 || it == A.max_iters;
    }
    if (!do_eval) continue;
    // emax: the residual.  excess: the largest amount by which a contact's error exceeds
    // the FP32 rounding floor of that contact, 64 eps_fp32 times the magnitudes entering
    // u = H v + c (|v_a| + |v_b| + |c|) and r; when it is below tol, FP32 sweeps can no
    // longer make progress and FP64 sweeps take over.
    double emax = 0.0, excess = -INFINITY;
    for (int k = tid; k < A.nc; k += nthr) {
      const int a = A.ia[k], b = A.ib[k];
      const bool has_b = b >= 0;
      const double2 va = __ldcg(&A.v[a]);
      const double2 vb = has_b ? __ldcg(&A.v[b]) : make_double2(0.0, 0.0);
      const double2 ck = A.c[k];
      double u0, u1;
      local_velocity(A.n[k], ck, va, has_b, vb, u0, u1);
      const double2 rk = __ldcg(&A.r[k]);
      cand[k] = rk;
      const double ek = fb_error_2d(rk.x, rk.y, u0, u1, A.mu[k]);
      emax = nanmax(emax, ek);
      const double scale = fabs(va.x) + fabs(va.y) + fabs(vb.x) + fabs(vb.y) + fabs(ck.x) + fabs(ck.y) +
                           fabs(rk.x) + fabs(rk.y);
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
      double2* t = best;
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
      if (err < prev64_err && prev64_err < INFINITY && err > 0.0) {
        const double per_sweep = (log(err) - log(prev64_err)) / (double)(it - prev64_it);
        const double need = (log(A.tol) - log(err)) / per_sweep;
        interval64 = need >= (double)(16u * eval64) ? 16u * eval64 : max(eval64, (unsigned)need);
      } else {
        interval64 = prev64_err < INFINITY ? min(2u * interval64, 16u * eval64) : eval64;
      }
      prev64_err = err;
      prev64_it = it;
      next64 = it + interval64;
    } else if (err < A.tol || err <= B.fp64_below || excess32 <= A.tol ||
               (since_best >= 16 && excess32 <= 16.0 * A.tol)) {
      // FP64 refinement from the FP64 image: a closing sweep once FP32 reached tol, or
      // FP64 sweeps once every contact's remaining error is within FP32 rounding of
      // its floor (or FP32 stopped improving the best iterate close to it).
      fp64 = true;
      prev64_err = err;
      prev64_it = it;
    }
  }
  if (it > A.max_iters) it = A.max_iters;
  if (!converged) {
    if (err_best < INFINITY)
      for (int k = tid; k < A.nc; k += nthr) A.r[k] = __ldcg(&best[k]);
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

// ---------------------------------------------------------------------------
// Two-level sweeps: bodies are split into spatial patches (one per block, one block per SM).
// A contact whose two bodies lie in one patch (or whose second body is a static plane) is
// interior to that patch; the others are boundary contacts.  One FP32 sweep processes every
// patch's interior contacts colour by colour inside its block, on shared-memory copies of the
// patch's velocities with block barriers only, then the boundary contacts colour by colour
// over the grid.  Patches share no body through interior contacts, so the sweep equals the
// sequential Gauss-Seidel order "interior contacts patch by patch, each patch by colour, then
// boundary contacts by colour" -- a valid Gauss-Seidel order of the same kind as the colour
// order of k_gs_mixed, with about one grid barrier per boundary colour instead of one per colour.
constexpr int kPatchBodyCap = 16384;  // bodies of one patch in shared memory (12 B each)

// Patches: T0 x T1 tiles of broad-phase grid cells (one block each), and the same tiling shifted
// by half a tile, (T0 + 1) x (T1 + 1) tiles whose centres are the patch corners.
struct PatchSetup {
  int T0, T1, P, d0, d1, Pb;
};

// Contact groups (the "patch" of a contact's key): g < P, the interior of patch g; P <= g < P + Pb,
// a contact between patches whose bodies share shifted tile g - P; g = P + Pb, the rest.
struct PatchArgs {
  const PatchSetup* ps;
  const int* pstart;  // P + 1 body offsets
  const int* pbody;   // bodies in patch order, each patch's band bodies first
  const int* pband;   // band bodies (endpoints of contacts between patches) per patch
  const int* qstart;  // Pb + 1 offsets of the shifted tiles' band bodies
  const int* qbody;
  const int* goff;    // (P + Pb + 1) * kMaxColors + 1 contact offsets by (group, colour)
  const int* order;   // packed index -> contact
  int cap;            // shared-memory body slots for a patch
  int capq;           // and for a shifted tile
  int stage_p;        // contacts of a patch staged in shared memory (its first ones, by colour)
  int stage_q;        // and of a shifted tile
  const int* cbody;   // bodies of the remaining contacts (group P + Pb), and each body's slot
  const int* cslot;   //   among them (valid for those bodies only)
  int capc;           // their shared-memory slots (even), 0 if the remainder is not staged
  int ncbody;         // their number
  int stage_c;        // remaining contacts staged in block 0 (all of them, or 0)
  int rest64;         // k_gs_patch64: the remainder's bodies held in block 0's shared memory
                      //   (all of them, or 0: the remainder then sweeps on global velocities)
};

// Bodies of the remaining contacts (group P + Pb): flagged here, compacted by a scan.
__global__ void k_rest_mark(int nc, const int* __restrict__ ia, const int* __restrict__ ib,
                            const int* __restrict__ cpatch, const PatchSetup* __restrict__ ps, int* __restrict__ flag) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nc || cpatch[k] != ps->P + ps->Pb) return;
  flag[ia[k]] = 1;
  flag[ib[k]] = 1;
}

__global__ void k_rest_scatter(int nb, const int* __restrict__ flag, const int* __restrict__ pos,
                               int* __restrict__ cbody) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nb && flag[i]) cbody[pos[i]] = i;
}

// T0 x T1 with (T0 + 1)(T1 + 1) <= max_patches, the largest T0 T1 weighted towards square
// tiles (cells are square).
__global__ void k_patch_setup(const GridParams* __restrict__ gp, int max_patches, PatchSetup* ps) {
  const int d0 = gp->dims[0], d1 = gp->dims[1];
  int bT0 = 1, bT1 = 1;
  double best = -1.0;
  for (int T0 = 1; T0 <= d0 && 2 * (T0 + 1) <= max_patches; ++T0) {
    const int T1 = min(d1, max_patches / (T0 + 1) - 1);
    if (T1 < 1) break;
    const double a = ((double)d0 * T1) / ((double)d1 * T0);
    const double score = (double)T0 * T1 * sqrt(a < 1.0 ? a : 1.0 / a);
    if (score > best) {
      best = score;
      bT0 = T0;
      bT1 = T1;
    }
  }
  ps->T0 = bT0;
  ps->T1 = bT1;
  ps->P = bT0 * bT1;
  ps->Pb = (bT0 + 1) * (bT1 + 1);
  ps->d0 = d0;
  ps->d1 = d1;
}

// Contacts (by the cell of their first body) plus bodies per cell column and per cell row: the
// cuts between patches sit at quantiles of these, so that patches carry about equal work and
// no patch collects every body that is still in free flight.
__global__ void k_patch_hist(int nc, int nb, const int* __restrict__ ia, const int* __restrict__ cell_of,
                             const PatchSetup* __restrict__ ps, int* __restrict__ hx, int* __restrict__ hy) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nc + nb) return;
  const int d0 = ps->d0;
  const int cell = cell_of[k < nc ? ia[k] : k - nc];
  atomicAdd(&hx[cell % d0], 1);
  atomicAdd(&hy[cell / d0], 1);
}

// Cuts X[0..T0] (cell columns) and Y[0..T1] (rows), strictly increasing from 0 to d: cut t at
// the first cell where the exclusive prefix count reaches t/T of the total.  One block.
__device__ void cuts_1d(const int* __restrict__ pref, int d, int T, int* __restrict__ cut) {
  const long total = pref[d];
  for (int t = 1 + threadIdx.x; t < T; t += blockDim.x) {
    const long target = total * t / T;
    int lo = 0, hi = d;  // first c in [0, d] with pref[c] >= target
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (pref[mid] >= target)
        hi = mid;
      else
        lo = mid + 1;
    }
    cut[t] = lo;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    cut[0] = 0;
    cut[T] = d;
    for (int t = 1; t < T; ++t) cut[t] = max(cut[t], cut[t - 1] + 1);
    for (int t = T - 1; t >= 1; --t) cut[t] = min(cut[t], cut[t + 1] - 1);
  }
  __syncthreads();
}

__global__ void k_patch_cuts(const PatchSetup* __restrict__ ps, const int* __restrict__ px,
                             const int* __restrict__ py, int* __restrict__ cx, int* __restrict__ cy) {
  cuts_1d(px, ps->d0, ps->T0, cx);
  cuts_1d(py, ps->d1, ps->T1, cy);
}

// Cell column/row -> patch column/row and shifted-tile column/row.  The shifted tiles' cuts sit
// halfway between neighbouring patch cuts, so every patch corner is a shifted tile's centre.
__device__ __forceinline__ void tile_maps_1d(int c, const int* __restrict__ cut, int T, int* __restrict__ a,
                                             int* __restrict__ b) {
  int ta = 0, tb = 0;
  for (int t = 1; t < T; ++t) ta += cut[t] <= c;
  for (int t = 0; t < T; ++t) tb += (cut[t] + cut[t + 1] + 1) / 2 <= c;
  a[c] = ta;
  b[c] = tb;
}

__global__ void k_patch_maps(const PatchSetup* __restrict__ ps, const int* __restrict__ cx, const int* __restrict__ cy,
                             int* __restrict__ colA, int* __restrict__ colB, int* __restrict__ rowA,
                             int* __restrict__ rowB) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < ps->d0) tile_maps_1d(i, cx, ps->T0, colA, colB);
  if (i < ps->d1) tile_maps_1d(i, cy, ps->T1, rowA, rowB);
}

__global__ void k_patch_of_body(int nb, const int* __restrict__ cell_of, const PatchSetup* __restrict__ ps,
                                const int* __restrict__ colA, const int* __restrict__ colB,
                                const int* __restrict__ rowA, const int* __restrict__ rowB, int* __restrict__ patch,
                                int* __restrict__ qpatch, int* __restrict__ pcount) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const int d0 = ps->d0, T0 = ps->T0;
  const int cell = cell_of[i];
  const int cx = cell % d0, cy = cell / d0;
  const int p = colA[cx] + T0 * rowA[cy];
  const int q = colB[cx] + (T0 + 1) * rowB[cy];
  patch[i] = p;
  qpatch[i] = q;
  atomicAdd(&pcount[p], 1);
}

__global__ void k_band_count(int nb, const int* __restrict__ band, const int* __restrict__ patch,
                             const int* __restrict__ qpatch, int* __restrict__ bcount, int* __restrict__ qcount) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb || !band[i]) return;
  atomicAdd(&bcount[patch[i]], 1);
  atomicAdd(&qcount[qpatch[i]], 1);
}

// Bodies by patch, band bodies first; band bodies also by shifted tile.  Patch-local slots.
__global__ void k_patch_scatter(int nb, const int* __restrict__ patch, const int* __restrict__ qpatch,
                                const int* __restrict__ band, const int* __restrict__ pstart,
                                const int* __restrict__ bcount, int* __restrict__ bfill, int* __restrict__ nfill,
                                int* __restrict__ pbody, int* __restrict__ lidx, const int* __restrict__ qstart,
                                int* __restrict__ qfill, int* __restrict__ qbody, int* __restrict__ lidxq) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const int p = patch[i];
  const bool bd = band[i] != 0;
  const int j = bd ? atomicAdd(&bfill[p], 1) : bcount[p] + atomicAdd(&nfill[p], 1);
  pbody[pstart[p] + j] = i;
  lidx[i] = j;
  if (bd) {
    const int q = qpatch[i];
    const int jq = atomicAdd(&qfill[q], 1);
    qbody[qstart[q] + jq] = i;
    lidxq[i] = jq;
  }
}

__global__ void k_patch_max(int n, const int* __restrict__ pcount, int* __restrict__ out) {
  int m = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) m = max(m, pcount[i]);
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// Group of each contact (PatchArgs); the endpoints of contacts between patches are band bodies.
// Contacts of groups >= P get their own colouring below.
__global__ void k_contact_side(int nc, const int* __restrict__ ia, const int* __restrict__ ib,
                               const int* __restrict__ patch, const int* __restrict__ qpatch,
                               const PatchSetup* __restrict__ ps, int* __restrict__ cpatch, int* __restrict__ bcolor,
                               int* __restrict__ band) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nc) return;
  const int a = ia[k], b = ib[k];
  const int pa = patch[a];
  bcolor[k] = -1;
  if (b < 0 || patch[b] == pa) {
    cpatch[k] = pa;
    return;
  }
  band[a] = 1;
  band[b] = 1;
  const int qa = qpatch[a];
  cpatch[k] = qpatch[b] == qa ? ps->P + qa : ps->P + ps->Pb;
}

// Jones-Plassmann colouring of the contacts between patches, each group (shifted tile, or the
// remainder) on its own: contacts of other groups neither take nor block colours.  These
// subgraphs are short bands, so they need far fewer colours than the whole contact graph.
struct BColorArgs {
  int nc;
  const int* ia;
  const int* ib;
  const int* body_off;
  const int* body_adj;
  const int* cpatch;
  const PatchSetup* ps;
  int* bcolor;     // packed (round << 8) | colour, -1 uncoloured
  int* remaining;  // 3 rotating counters
  int* status;
  GridBarrier* gb;
  unsigned long long spin;
  int max_rounds;
};

__global__ void k_color_boundary(BColorArgs A) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nthr = gridDim.x * blockDim.x;
  const int P = A.ps->P;
  volatile int* vcolor = A.bcolor;
  for (int round = 0;; ++round) {
    if (round >= A.max_rounds) {
      if (tid == 0) atomicExch(A.status, (int)SG_CAPACITY);
      return;
    }
    int rem = 0;
    for (int k = tid; k < A.nc; k += nthr) {
      const int gk = A.cpatch[k];
      if (gk < P || vcolor[k] >= 0) continue;
      const unsigned pk = hash_prio((unsigned)k);
      unsigned long long used = 0ull;
      bool is_max = true;
      const int bodies[2] = {A.ia[k], A.ib[k]};
      for (int bi = 0; bi < 2 && is_max; ++bi) {
        const int body = bodies[bi];
        if (body < 0) continue;
        const int e = A.body_off[body + 1];
        for (int p = A.body_off[body]; p < e; ++p) {
          const int j = A.body_adj[p];
          if (j == k || A.cpatch[j] != gk) continue;
          const int cj = vcolor[j];
          if (cj >= 0 && (cj >> 8) < round) {
            used |= 1ull << (cj & 63);
          } else if (prio_greater(hash_prio((unsigned)j), j, pk, k)) {
            is_max = false;
            break;
          }
        }
      }
      if (is_max) {
        const unsigned long long freec = ~used;
        if (freec == 0ull) {
          atomicExch(A.status, (int)SG_CAPACITY);
          vcolor[k] = (round << 8) | 63;
        } else {
          vcolor[k] = (round << 8) | (__ffsll((long long)freec) - 1);
        }
      } else {
        ++rem;
      }
    }
    rem = warp_sum(rem);
    if ((threadIdx.x & 31) == 0 && rem) atomicAdd(&A.remaining[round % 3], rem);
    if (tid == 0) A.remaining[(round + 1) % 3] = 0;
    if (!grid_sync(A.gb, A.spin)) {
      if (tid == 0) atomicExch(A.status, (int)SG_DEVICE_TIMEOUT);
      return;
    }
    if (*((volatile int*)&A.remaining[round % 3]) == 0) break;
  }
}

// Colour of each contact within its group: the global colour inside a patch, the group's own
// colouring between patches (in place over the latter); the highest colour into *maxc.
__global__ void k_group_color_init(int nc, const int* __restrict__ color, const int* __restrict__ cpatch,
                                   const PatchSetup* __restrict__ ps, int* __restrict__ gcolor, int* __restrict__ maxc) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  int c = 0;
  if (k < nc) {
    c = (cpatch[k] >= ps->P ? gcolor[k] : color[k]) & (kMaxColors - 1);
    gcolor[k] = c;
  }
  for (int o = 16; o > 0; o >>= 1) c = max(c, __shfl_down_sync(0xffffffffu, c, o));
  if ((threadIdx.x & 31) == 0) atomicMax(maxc, c);
}

struct RecolorArgs {
  int nc;
  const int* ia;
  const int* ib;
  const int* body_off;
  const int* body_adj;
  const int* cpatch;
  int* gcolor;
  const int* maxc;
  int* status;
  GridBarrier* gb;
  unsigned long long spin;
};

// Each group's colouring compacted on its own (the group's contacts are swept by one block or
// one grid, so its colour count, not the global one, sets its barriers): colour classes from
// the highest down, every contact of the class moves to the lowest colour that its neighbours
// in the group leave free.  Two contacts of one class share no body, so a class moves at once
// and the colouring stays proper.
__global__ void k_recolor_groups(RecolorArgs A) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nthr = gridDim.x * blockDim.x;
  const int top = *((volatile const int*)A.maxc);
  for (int col = top; col >= 1; --col) {
    for (int k = tid; k < A.nc; k += nthr) {
      if (__ldcg(&A.gcolor[k]) != col) continue;
      const int g = A.cpatch[k];
      unsigned long long used = 0ull;
      const int bodies[2] = {A.ia[k], A.ib[k]};
      for (int bi = 0; bi < 2; ++bi) {
        const int body = bodies[bi];
        if (body < 0) continue;
        const int e = A.body_off[body + 1];
        for (int p = A.body_off[body]; p < e; ++p) {
          const int j = A.body_adj[p];
          if (j != k && A.cpatch[j] == g) used |= 1ull << (__ldcg(&A.gcolor[j]) & (kMaxColors - 1));
        }
      }
      const int lowest = __ffsll((long long)~used) - 1;
      if (lowest >= 0 && lowest < col) A.gcolor[k] = lowest;
    }
    if (!grid_sync(A.gb, A.spin)) {
      if (tid == 0) atomicExch(A.status, (int)SG_DEVICE_TIMEOUT);
      return;
    }
  }
}

__global__ void k_contact_key(int nc, const int* __restrict__ gcolor, const int* __restrict__ cpatch,
                              int* __restrict__ key, int* __restrict__ kcount) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nc) return;
  const int cp = cpatch[k];
  const int c = gcolor[k] & (kMaxColors - 1);
  const int kk = cp * kMaxColors + c;
  key[k] = kk;
  atomicAdd(&kcount[kk], 1);
}

// Largest contact count of a patch (out[0]) and of a shifted tile (out[1]); the remaining
// contacts (out[2]).
__global__ void k_group_max(const PatchSetup* __restrict__ ps, const int* __restrict__ kstart, int* __restrict__ out) {
  const int P = ps->P, Pb = ps->Pb;
  if (threadIdx.x == 0) out[2] = kstart[(P + Pb + 1) * kMaxColors] - kstart[(P + Pb) * kMaxColors];
  int mp = 0, mq = 0;
  for (int g = threadIdx.x; g < P + Pb; g += blockDim.x) {
    const int n = kstart[(g + 1) * kMaxColors] - kstart[g * kMaxColors];
    if (g < P)
      mp = max(mp, n);
    else
      mq = max(mq, n);
  }
  for (int o = 16; o > 0; o >>= 1) {
    mp = max(mp, __shfl_down_sync(0xffffffffu, mp, o));
    mq = max(mq, __shfl_down_sync(0xffffffffu, mq, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&out[0], mp);
    atomicMax(&out[1], mq);
  }
}

__global__ void k_contact_scatter(int nc, const int* __restrict__ key, const int* __restrict__ kstart,
                                  int* __restrict__ kfill, int* __restrict__ order) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nc) return;
  const int kk = key[k];
  order[kstart[kk] + atomicAdd(&kfill[kk], 1)] = k;
}

// Packs in (group, colour) order; contacts of a patch carry patch-local body slots, those of a
// shifted tile tile-local slots, the rest global body indices.
__global__ void k_pack32_patch(int nc, const int* __restrict__ order, const int* __restrict__ key,
                               const PatchSetup* __restrict__ ps, const int* __restrict__ ia,
                               const int* __restrict__ ib, const int* __restrict__ lidx, const int* __restrict__ lidxq,
                               const double2* __restrict__ n, const double2* __restrict__ c,
                               const double* __restrict__ W, const double* __restrict__ mu,
                               const double2* __restrict__ r, int2* __restrict__ ab, float2* __restrict__ n32,
                               float2* __restrict__ c32, float4* __restrict__ w32, float2* __restrict__ r32) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nc) return;
  const int k = order[s];
  const int a = ia[k], b = ib[k];
  const int g = key[k] / kMaxColors;
  if (g < ps->P)
    ab[s] = make_int2(lidx[a], b >= 0 ? lidx[b] : -1);
  else if (g < ps->P + ps->Pb)
    ab[s] = make_int2(lidxq[a], lidxq[b]);
  else
    ab[s] = make_int2(a, b >= 0 ? b : -1);
  const double2 nk = n[k], ck = c[k], rk = r[k];
  n32[s] = make_float2((float)nk.x, (float)nk.y);
  c32[s] = make_float2((float)ck.x, (float)ck.y);
  w32[s] = make_float4((float)W[3 * k], (float)W[3 * k + 1], (float)W[3 * k + 2], (float)mu[k]);
  r32[s] = make_float2((float)rk.x, (float)rk.y);
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// A contact staged in shared memory: both body slots in one word (16 bits each, 0xffff for a
// static plane), normal, forcing and friction coefficient; the impulse kept there too (written
// back to global memory before each FP64 check).  The Delassus block of a disc contact is
// (1/m_a + 1/m_b) I (n and t = (-n_y, n_x) are orthonormal, so n.t is exactly 0 and
// n.n = t.t = 1 to rounding), so it is formed from the slots' inverse masses.
struct Staged {
  unsigned* ab;
  float2* n;
  float2* c;
  float* mu;
  float2* r;
};

__device__ __forceinline__ void stage_contact(const Gs32Args& B, const Staged& S, int i, int s) {
  const int2 ab = B.ab[s];
  S.ab[i] = (unsigned)ab.x | ((ab.y >= 0 ? (unsigned)ab.y : 0xffffu) << 16);
  S.n[i] = B.n[s];
  S.c[i] = B.c[s];
  S.mu[i] = B.w[s].w;
  S.r[i] = B.r[s];
}

__device__ __forceinline__ void gs_update32_staged(const Staged& S, int i, float2* sv, const float* sm) {
  const unsigned ab = S.ab[i];
  const int a = (int)(ab & 0xffffu), b = (int)(ab >> 16);
  const bool has_b = b != 0xffff;
  const float2 nk = S.n[i], ck = S.c[i];
  const float2 va = sv[a];
  const float2 vb = has_b ? sv[b] : make_float2(0.0f, 0.0f);
  const float ma = sm[a], mb = has_b ? sm[b] : 0.0f;
  const float nx = nk.x, ny = nk.y, tx = -ny, ty = nx;
  float hn = nx * va.x + ny * va.y;
  float ht = tx * va.x + ty * va.y;
  if (has_b) {
    hn -= nx * vb.x + ny * vb.y;
    ht -= tx * vb.x + ty * vb.y;
  }
  const float u0 = hn + ck.x, u1 = ht + ck.y;
  const float2 rk = S.r[i];
  const float wd = ma + mb;
  const float bt0 = u0 - wd * rk.x;
  const float bt1 = u1 - wd * rk.y;
  // Coulomb local problem with W = wd I: open if bt0 >= 0; otherwise r = -bt / wd with its
  // tangential part clamped to the cone (for an isotropic W the sliding solution keeps the
  // stick solution's normal part, so stick and slide are this one expression).
  float rn0 = 0.0f, rn1 = 0.0f;
  if (bt0 < 0.0f) {
    const float inv = __frcp_rn(wd);
    const float mu = S.mu[i];
    rn0 = -bt0 * inv;
    rn1 = fminf(fmaxf(-bt1 * inv, -mu * rn0), mu * rn0);
  }
  const float d0 = rn0 - rk.x, d1 = rn1 - rk.y;
  const float px = nx * d0 + tx * d1, py = ny * d0 + ty * d1;
  sv[a] = make_float2(va.x + ma * px, va.y + ma * py);
  if (has_b) sv[b] = make_float2(vb.x - mb * px, vb.y - mb * py);
  S.r[i] = make_float2(rn0, rn1);
}

// A patch or tile contact that did not fit in shared memory: gs_update32_staged's arithmetic
// (the isotropic block from the slots' inverse masses, the closed-form local solve) on the
// contact's global record, so that a contact's update does not depend on whether it was
// staged.  Which contacts are staged depends on their order within a colour, and that order is
// not fixed from run to run; with one arithmetic for both, the sweep's result does not depend
// on it.
__device__ __forceinline__ void gs_update32_iso(const Gs32Args& B, int s, float2* sv, const float* sm) {
  const int2 ab = B.ab[s];
  const int a = ab.x, b = ab.y;
  const bool has_b = b >= 0;
  const float2 nk = B.n[s], ck = B.c[s];
  const float2 va = sv[a];
  const float2 vb = has_b ? sv[b] : make_float2(0.0f, 0.0f);
  const float ma = sm[a], mb = has_b ? sm[b] : 0.0f;
  const float nx = nk.x, ny = nk.y, tx = -ny, ty = nx;
  float hn = nx * va.x + ny * va.y;
  float ht = tx * va.x + ty * va.y;
  if (has_b) {
    hn -= nx * vb.x + ny * vb.y;
    ht -= tx * vb.x + ty * vb.y;
  }
  const float u0 = hn + ck.x, u1 = ht + ck.y;
  const float2 rk = B.r[s];
  const float wd = ma + mb;
  const float bt0 = u0 - wd * rk.x;
  const float bt1 = u1 - wd * rk.y;
  float rn0 = 0.0f, rn1 = 0.0f;
  if (bt0 < 0.0f) {
    const float inv = __frcp_rn(wd);
    const float mu = B.w[s].w;
    rn0 = -bt0 * inv;
    rn1 = fminf(fmaxf(-bt1 * inv, -mu * rn0), mu * rn0);
  }
  const float d0 = rn0 - rk.x, d1 = rn1 - rk.y;
  const float px = nx * d0 + tx * d1, py = ny * d0 + ty * d1;
  sv[a] = make_float2(va.x + ma * px, va.y + ma * py);
  if (has_b) sv[b] = make_float2(vb.x - mb * px, vb.y - mb * py);
  B.r[s] = make_float2(rn0, rn1);
}

// FP64 update of contact k (gs_update's arithmetic: the FP64 record, the general 2x2 local solve)
// on shared-memory FP64 velocities: la, lb are the bodies' slots (lb < 0 for a static plane).
__device__ __forceinline__ void gs_update64_local(const GsArgs& A, int k, int la, int lb, double2* sv,
                                                  const double* sm) {
  const double2 nk = A.n[k], ck = A.c[k];
  const double2 va = sv[la];
  const bool has_b = lb >= 0;
  const double2 vb = has_b ? sv[lb] : make_double2(0.0, 0.0);
  double u0, u1;
  local_velocity(nk, ck, va, has_b, vb, u0, u1);
  const double2 rk = A.r[k];
  const double r0 = rk.x, r1 = rk.y;
  const double w00 = A.W[3 * k], w01 = A.W[3 * k + 1], w11 = A.W[3 * k + 2];
  const double bt0 = u0 - (w00 * r0 + w01 * r1);
  const double bt1 = u1 - (w01 * r0 + w11 * r1);
  double rn0, rn1;
  if (w01 == 0.0 && w00 == w11)
    local_solve_2d_iso(w00, bt0, bt1, A.mu[k], rn0, rn1);
  else
    local_solve_2d(w00, w01, w11, bt0, bt1, A.mu[k], rn0, rn1);
  const double d0 = rn0 - r0, d1 = rn1 - r1;
  const double nx = nk.x, ny = nk.y, tx = -ny, ty = nx;
  const double px = nx * d0 + tx * d1;
  const double py = ny * d0 + ty * d1;
  const double ma = sm[la];
  sv[la] = make_double2(va.x + ma * px, va.y + ma * py);
  if (has_b) {
    const double mb = sm[lb];
    sv[lb] = make_double2(vb.x - mb * px, vb.y - mb * py);
  }
  A.r[k] = make_double2(rn0, rn1);
}

// Highest non-empty colour + 1 of a group's offsets.
__device__ __forceinline__ int group_colors(const int* off) {
  int n = kMaxColors;
  while (n > 0 && off[n] == off[n - 1]) --n;
  return n;
}

__global__ void __launch_bounds__(kPatchBlock, 1) k_gs_patch(GsArgs A, Gs32Args B, PatchArgs Q) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nthr = gridDim.x * blockDim.x;
  if (*((volatile int*)&A.st->status) != 0) return;
  __shared__ int s_off[kMaxColors + 1];
  __shared__ int s_ncol;
  if (threadIdx.x == 0) s_ncol = A.st->n_colors;
  for (int c = threadIdx.x; c <= kMaxColors; c += blockDim.x) s_off[c] = A.st->color_off[c];
  __syncthreads();
  const int ncol = s_ncol;
  // This block's patch (its bodies, band bodies first, and its interior contacts by colour)
  // and its shifted tile (band bodies, contacts by colour), both swept on shared-memory
  // velocities; the remaining contacts by colour over the grid, with a tail of small colours
  // as in k_gs_mixed.  Slots: patch velocities, patch 1/m, tile velocities, tile 1/m (cap and
  // capq even, so every float2 stays 8-byte aligned), then the staged contacts (Staged), the
  // patch's first stage_p in slots [0, stage_p), the tile's first stage_q after them.
  extern __shared__ __align__(16) float2 sv[];
  float* sm = reinterpret_cast<float*>(sv + Q.cap);
  float2* svq = reinterpret_cast<float2*>(sm + Q.cap);
  float* smq = reinterpret_cast<float*>(svq + Q.capq);
  const int cs = Q.stage_p + Q.stage_q;
  Staged S;
  S.n = reinterpret_cast<float2*>(smq + Q.capq);
  S.c = S.n + cs;
  S.r = S.c + cs;
  S.ab = reinterpret_cast<unsigned*>(S.r + cs);
  S.mu = reinterpret_cast<float*>(S.ab + cs);
  // Then the remainder's bodies (velocities, 1/m) and contacts, used by block 0 alone.
  float2* svc = reinterpret_cast<float2*>(S.mu + cs);
  float* smc = reinterpret_cast<float*>(svc + Q.capc);
  Staged SC;
  SC.n = reinterpret_cast<float2*>(smc + Q.capc);
  SC.c = SC.n + Q.stage_c;
  SC.r = SC.c + Q.stage_c;
  SC.ab = reinterpret_cast<unsigned*>(SC.r + Q.stage_c);
  SC.mu = reinterpret_cast<float*>(SC.ab + Q.stage_c);
  __shared__ int s_goff[kMaxColors + 1];
  __shared__ int s_hoff[kMaxColors + 1];
  __shared__ int s_boff[kMaxColors + 1];
  const int P = Q.ps->P, Pb = Q.ps->Pb;
  const bool has_p = blockIdx.x < P, has_q = blockIdx.x < Pb;
  const int pb0 = has_p ? Q.pstart[blockIdx.x] : 0;
  const int pb1 = has_p ? Q.pstart[blockIdx.x + 1] : 0;
  const int pbe = pb0 + (has_p ? Q.pband[blockIdx.x] : 0);  // band bodies: [pb0, pbe)
  const int qb0 = has_q ? Q.qstart[blockIdx.x] : 0;
  const int qb1 = has_q ? Q.qstart[blockIdx.x + 1] : 0;
  for (int c = threadIdx.x; c <= kMaxColors; c += blockDim.x) {
    s_goff[c] = has_p ? Q.goff[blockIdx.x * kMaxColors + c] : 0;
    s_hoff[c] = has_q ? Q.goff[(P + blockIdx.x) * kMaxColors + c] : 0;
    s_boff[c] = Q.goff[(P + Pb) * kMaxColors + c];
  }
  for (int j = pb0 + threadIdx.x; j < pb1; j += blockDim.x) sm[j - pb0] = B.minv[Q.pbody[j]];
  for (int j = qb0 + threadIdx.x; j < qb1; j += blockDim.x) smq[j - qb0] = B.minv[Q.qbody[j]];
  __syncthreads();
  // Colours of each group (a group's own colouring may use more colours than the whole graph's).
  const int ncol_p = group_colors(s_goff), ncol_q = group_colors(s_hoff);
  const int ncol_r = group_colors(s_boff);
  const int sp0 = s_goff[0], sq0 = s_hoff[0];
  const int sp_end = sp0 + min(s_goff[ncol_p] - sp0, Q.stage_p);  // staged: [sp0, sp_end)
  const int sq_end = sq0 + min(s_hoff[ncol_q] - sq0, Q.stage_q);
  for (int s = sp0 + threadIdx.x; s < sp_end; s += blockDim.x) stage_contact(B, S, s - sp0, s);
  for (int s = sq0 + threadIdx.x; s < sq_end; s += blockDim.x) stage_contact(B, S, Q.stage_p + s - sq0, s);
  int btail = ncol_r;
  while (btail > 0 && s_boff[btail] - s_boff[btail - 1] <= 2 * (int)blockDim.x) --btail;
  // The remainder swept by block 0 in shared memory when all its colours are small and it
  // was staged whole (bodies compacted on the host side: cslot maps a body to its slot).
  const int sc0 = s_boff[0], nrest = s_boff[ncol_r] - sc0;
  const bool rest_staged = btail == 0 && nrest > 0 && Q.stage_c == nrest;
  const int ncb = rest_staged ? Q.ncbody : 0;
  if (rest_staged && blockIdx.x == 0) {
    for (int s = sc0 + threadIdx.x; s < sc0 + nrest; s += blockDim.x) {
      const int2 ab = B.ab[s];
      const int i = s - sc0;
      SC.ab[i] = (unsigned)Q.cslot[ab.x] | ((unsigned)Q.cslot[ab.y] << 16);
      SC.n[i] = B.n[s];
      SC.c[i] = B.c[s];
      SC.mu[i] = B.w[s].w;
      SC.r[i] = B.r[s];
    }
    for (int j = threadIdx.x; j < ncb; j += blockDim.x) smc[j] = B.minv[Q.cbody[j]];
  }
  __syncthreads();
  const unsigned eval64 = A.eval_every ? A.eval_every : 1u;
  const unsigned eval32 = B.eval32 ? B.eval32 : 1u;
  double2* best = A.r_a;
  double2* cand = A.r_b;
  double err_best = INFINITY;
  bool converged = false, fp64 = B.fp64_start != 0;
  unsigned it = 0, n_eval = 0, s32 = 0, s64 = 0, lifts = 0, since_best = 0;
  unsigned next_eval = 1, interval = eval32;
  // FP64 sweeps' checks, at most 16 eval64 apart: the next one where the residual's rate of
  // decrease over the last two checks predicts tol, sooner than that never, and twice as far as the
  // last gap where it did not decrease (a check costs about a sweep; GB300's FP64 pipe makes the
  // Fischer-Burmeister error the dearest part of it).
  unsigned next64 = eval64, interval64 = eval64, prev64_it = 0;
  double prev64_err = INFINITY;
  // Phase timers of block 0 (shared memory, so that they take no registers from the sweeps):
  // interior, wait, boundary totals, then the current sweep's marks.
  __shared__ unsigned long long s_t[6];
  const bool timer = tid == 0;
  const bool btimer = threadIdx.x == 0;  // every block: its own patch-interior total in s_t[0]
  if (btimer) s_t[0] = s_t[1] = s_t[2] = 0ull;
  // The patch's shared-memory velocities persist between sweeps: only band bodies are
  // touched outside the patch, so only they are reloaded and written back, except after an
  // FP64 check, which resets every velocity from the impulses.
  bool reload_all = true;
  // Entering the FP64 sweeps: every velocity and inverse mass is loaded afresh.
  bool fresh64 = true;
  for (it = 1; it <= A.max_iters; ++it) {
    bool do_eval;
    if (!fp64) {
      if (btimer) s_t[3] = globaltimer_ns();
      // Interior contacts of this block's patch, colour by colour (block barriers only).
      const int lend = reload_all ? pb1 : pbe;
      reload_all = false;
      for (int j = pb0 + threadIdx.x; j < lend; j += blockDim.x) sv[j - pb0] = __ldcg(&B.v[Q.pbody[j]]);
      __syncthreads();
      for (int col = 0; col < ncol_p; ++col) {
        const int e = s_goff[col + 1];
        for (int s = s_goff[col] + threadIdx.x; s < e; s += blockDim.x) {
          if (s < sp_end)
            gs_update32_staged(S, s - sp0, sv, sm);
          else
            gs_update32_iso(B, s, sv, sm);
        }
        __syncthreads();
      }
      for (int j = pb0 + threadIdx.x; j < pbe; j += blockDim.x) B.v[Q.pbody[j]] = sv[j - pb0];
      if (btimer) {
        s_t[4] = globaltimer_ns();
        s_t[0] += s_t[4] - s_t[3];
      }
      if (!grid_sync(A.gb, A.spin)) {
        if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
        return;
      }
      if (timer) s_t[5] = globaltimer_ns();
      // Contacts between patches within this block's shifted tile, colour by colour on the
      // tile's shared-memory velocities (block barriers only).
      if (qb1 > qb0) {
        for (int j = qb0 + threadIdx.x; j < qb1; j += blockDim.x) svq[j - qb0] = __ldcg(&B.v[Q.qbody[j]]);
        __syncthreads();
        for (int col = 0; col < ncol_q; ++col) {
          const int e = s_hoff[col + 1];
          for (int s = s_hoff[col] + threadIdx.x; s < e; s += blockDim.x) {
            if (s < sq_end)
              gs_update32_staged(S, Q.stage_p + s - sq0, svq, smq);
            else
              gs_update32_iso(B, s, svq, smq);
          }
          __syncthreads();
        }
        for (int j = qb0 + threadIdx.x; j < qb1; j += blockDim.x) B.v[Q.qbody[j]] = svq[j - qb0];
      }
      if (!grid_sync(A.gb, A.spin)) {
        if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
        return;
      }
      // The remaining contacts (across patches and shifted tiles): staged, by block 0 on
      // shared-memory velocities; otherwise colour by colour over the grid, the small trailing
      // colours in block 0 alone.
      if (rest_staged) {
        if (blockIdx.x == 0) {
          for (int j = threadIdx.x; j < ncb; j += blockDim.x) svc[j] = __ldcg(&B.v[Q.cbody[j]]);
          __syncthreads();
          for (int col = 0; col < ncol_r; ++col) {
            for (int s = s_boff[col] + threadIdx.x; s < s_boff[col + 1]; s += blockDim.x)
              gs_update32_staged(SC, s - sc0, svc, smc);
            __syncthreads();
          }
          for (int j = threadIdx.x; j < ncb; j += blockDim.x) B.v[Q.cbody[j]] = svc[j];
        }
        if (!grid_sync(A.gb, A.spin)) {
          if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
          return;
        }
      } else {
        for (int col = 0; col < btail; ++col) {
          const int b0 = s_boff[col], e = s_boff[col + 1];
          if (b0 == e) continue;
          for (int s = b0 + tid; s < e; s += nthr) gs_update32(B, s);
          if (!grid_sync(A.gb, A.spin)) {
            if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
            return;
          }
        }
        if (btail < ncol_r && s_boff[btail] < s_boff[ncol_r]) {
          if (blockIdx.x == 0) {
            for (int col = btail; col < ncol_r; ++col) {
              for (int s = s_boff[col] + threadIdx.x; s < s_boff[col + 1]; s += blockDim.x) gs_update32(B, s);
              __syncthreads();
            }
          }
          if (!grid_sync(A.gb, A.spin)) {
            if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
            return;
          }
        }
      }
      if (timer) {
        const unsigned long long t3 = globaltimer_ns();
        s_t[1] += s_t[5] - s_t[4];
        s_t[2] += t3 - s_t[5];
      }
      ++s32;
      // FP64 checks after sweeps 1, 2, 4, ... eval32, then at an interval that grows
      // (up to 16 eval32) while the residual is far above tol: a check costs several
      // sweeps, and the final check at max_iters always happens.
      do_eval = it == next_eval || it == A.max_iters;
      if (do_eval) {
        // Staged impulses back to global memory first.
        for (int s = sp0 + threadIdx.x; s < sp_end; s += blockDim.x) B.r[s] = S.r[s - sp0];
        for (int s = sq0 + threadIdx.x; s < sq_end; s += blockDim.x) B.r[s] = S.r[Q.stage_p + s - sq0];
        if (rest_staged && blockIdx.x == 0)
          for (int s = sc0 + threadIdx.x; s < sc0 + nrest; s += blockDim.x) B.r[s] = SC.r[s - sc0];
        if (!grid_sync(A.gb, A.spin)) {
          if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
          return;
        }
        // Lift the FP32 iterate to FP64: impulses, then body velocities v = v0 + Minv H^T r.
        for (int s = tid; s < A.nc; s += nthr) {
          const float2 r32 = __ldcg(&B.r[s]);
          A.r[Q.order[s]] = make_double2((double)r32.x, (double)r32.y);
        }
        if (!grid_sync(A.gb, A.spin)) {
          if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
          return;
        }
        for (int i = tid; i < B.nb; i += nthr) {
          double hx = 0.0, hy = 0.0;
          const int e = B.body_off[i + 1];
          for (int p = B.body_off[i]; p < e; ++p) {
            const int k = B.body_adj[p];
            const double sgn = (A.ia[k] == i) ? 1.0 : -1.0;
            const double2 nk = A.n[k], rk = __ldcg(&A.r[k]);
            const double px = nk.x * rk.x + (-nk.y) * rk.y;
            const double py = nk.y * rk.x + nk.x * rk.y;
            hx = hx + sgn * px;
            hy = hy + sgn * py;
          }
          const double2 a = B.v0[i];
          const double mi = B.minv64[i];
          const double2 vi = make_double2(a.x + mi * hx, a.y + mi * hy);
          A.v[i] = vi;
          // Resynchronise the FP32 running velocity with the impulses: removes the
          // rounding drift that incremental FP32 updates accumulate.
          B.v[i] = make_float2((float)vi.x, (float)vi.y);
        }
        ++lifts;
        reload_all = true;
        if (!grid_sync(A.gb, A.spin)) {
          if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
          return;
        }
      }
    } else if (!B.fp64_local) {
      for (int col = 0; col < ncol; ++col) {
        const int e = s_off[col + 1];
        for (int q = s_off[col] + tid; q < e; q += nthr) gs_update(A, A.perm[q]);
        if (!grid_sync(A.gb, A.spin)) {
          if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
          return;
        }
      }
      ++s64;
      do_eval = it >= next64 || it == A.max_iters;
    } else {
      // FP64 sweeps on the same partition: the patch's FP64 velocities and inverse masses in
      // shared memory (the FP32 layout is dead once the solve is in FP64, which it never leaves),
      // the shifted tile's likewise, the remainder by block 0 on global velocities; three grid
      // barriers a sweep.  Before a residual evaluation every patch body goes back to global memory.
      do_eval = it >= next64 || it == A.max_iters;
      double2* sv64 = reinterpret_cast<double2*>(sv);
      double* sm64 = reinterpret_cast<double*>(sv64 + Q.cap);
      double2* svq64 = reinterpret_cast<double2*>(sm64 + Q.cap);
      double* smq64 = reinterpret_cast<double*>(svq64 + Q.capq);
      if (fresh64) {
        for (int j = pb0 + threadIdx.x; j < pb1; j += blockDim.x) sm64[j - pb0] = A.minv[Q.pbody[j]];
        for (int j = qb0 + threadIdx.x; j < qb1; j += blockDim.x) smq64[j - qb0] = A.minv[Q.qbody[j]];
      }
      const int lend = fresh64 ? pb1 : pbe;
      fresh64 = false;
      for (int j = pb0 + threadIdx.x; j < lend; j += blockDim.x) sv64[j - pb0] = __ldcg(&A.v[Q.pbody[j]]);
      __syncthreads();
      for (int col = 0; col < ncol_p; ++col) {
        const int e = s_goff[col + 1];
        for (int q = s_goff[col] + threadIdx.x; q < e; q += blockDim.x) {
          const int2 ab = B.ab[q];
          gs_update64_local(A, Q.order[q], ab.x, ab.y, sv64, sm64);
        }
        __syncthreads();
      }
      const int wend = do_eval ? pb1 : pbe;
      for (int j = pb0 + threadIdx.x; j < wend; j += blockDim.x) A.v[Q.pbody[j]] = sv64[j - pb0];
      if (!grid_sync(A.gb, A.spin)) {
        if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
        return;
      }
      if (qb1 > qb0) {
        for (int j = qb0 + threadIdx.x; j < qb1; j += blockDim.x) svq64[j - qb0] = __ldcg(&A.v[Q.qbody[j]]);
        __syncthreads();
        for (int col = 0; col < ncol_q; ++col) {
          const int e = s_hoff[col + 1];
          for (int q = s_hoff[col] + threadIdx.x; q < e; q += blockDim.x) {
            const int2 ab = B.ab[q];
            gs_update64_local(A, Q.order[q], ab.x, ab.y, svq64, smq64);
          }
          __syncthreads();
        }
        for (int j = qb0 + threadIdx.x; j < qb1; j += blockDim.x) A.v[Q.qbody[j]] = svq64[j - qb0];
      }
      if (!grid_sync(A.gb, A.spin)) {
        if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
        return;
      }
      if (blockIdx.x == 0 && nrest > 0) {
        for (int col = 0; col < ncol_r; ++col) {
          for (int q = s_boff[col] + threadIdx.x; q < s_boff[col + 1]; q += blockDim.x) gs_update(A, Q.order[q]);
          __syncthreads();
        }
      }
      if (!grid_sync(A.gb, A.spin)) {
        if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
        return;
      }
      ++s64;
    }
    if (!do_eval) continue;
    // emax: the residual.  excess: the largest amount by which a contact's error exceeds
    // the FP32 rounding floor of that contact, 64 eps_fp32 times the magnitudes entering
    // u = H v + c (|v_a| + |v_b| + |c|) and r; when it is below tol, FP32 sweeps can no
    // longer make progress and FP64 sweeps take over.
    double emax = 0.0, excess = -INFINITY;
    for (int k = tid; k < A.nc; k += nthr) {
      const int a = A.ia[k], b = A.ib[k];
      const bool has_b = b >= 0;
      const double2 va = __ldcg(&A.v[a]);
      const double2 vb = has_b ? __ldcg(&A.v[b]) : make_double2(0.0, 0.0);
      const double2 ck = A.c[k];
      double u0, u1;
      local_velocity(A.n[k], ck, va, has_b, vb, u0, u1);
      const double2 rk = __ldcg(&A.r[k]);
      cand[k] = rk;
      const double ek = fb_error_2d(rk.x, rk.y, u0, u1, A.mu[k]);
      emax = nanmax(emax, ek);
      if (!fp64) {
        const double scale = fabs(va.x) + fabs(va.y) + fabs(vb.x) + fabs(vb.y) + fabs(ck.x) + fabs(ck.y) +
                             fabs(rk.x) + fabs(rk.y);
        excess = nanmax(excess, ek - 64.0 * 1.1920929e-7 * scale);
      }
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
      double2* t = best;
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
      if (err < prev64_err && prev64_err < INFINITY && err > 0.0) {
        const double per_sweep = (log(err) - log(prev64_err)) / (double)(it - prev64_it);
        const double need = (log(A.tol) - log(err)) / per_sweep;  // sweeps to tol at that rate
        interval64 = need >= (double)(16u * eval64) ? 16u * eval64 : max(eval64, (unsigned)need);
      } else {
        interval64 = min(2u * interval64, 16u * eval64);
      }
      prev64_err = err;
      prev64_it = it;
      next64 = it + interval64;
    } else if (err < A.tol || err <= B.fp64_below || excess32 <= A.tol ||
               (since_best >= 16 && excess32 <= 16.0 * A.tol)) {
      // FP64 refinement from the FP64 image: a closing sweep once FP32 reached tol, or
      // FP64 sweeps once every contact's remaining error is within FP32 rounding of
      // its floor (or FP32 stopped improving the best iterate close to it).
      fp64 = true;
      next64 = it + eval64;
      prev64_err = INFINITY;
    }
  }
  if (it > A.max_iters) it = A.max_iters;
  if (!converged) {
    if (err_best < INFINITY)
      for (int k = tid; k < A.nc; k += nthr) A.r[k] = __ldcg(&best[k]);
  }
  if (btimer) atomicMax(&A.st->interior_max, (s_t[0] << 8) | (unsigned long long)blockIdx.x);
  if (tid == 0) {
    A.st->iterations = it;
    A.st->converged = converged ? 1 : 0;
    A.st->error = err_best;
    A.st->sweeps32 = s32;
    A.st->sweeps64 = s64;
    A.st->evals = n_eval;
    A.st->lifts = lifts;
    A.st->phase_ns[0] = s_t[0];
    A.st->phase_ns[1] = s_t[1];
    A.st->phase_ns[2] = s_t[2];
    A.st->boundary_contacts = Q.goff[(P + Pb + 1) * kMaxColors] - Q.goff[P * kMaxColors];
    int nbc = 0;
    for (int c = 0; c < ncol_r; ++c) nbc += s_boff[c + 1] > s_boff[c];
    A.st->boundary_colors = nbc;
  }
}

// ---------------------------------------------------------------------------
// FP64 sweeps on the two-level partition, for solves that stay in FP64 (the FP32 form's FP64
// probe left them within fp64_factor tol): k_gs_patch's FP64 phase in a kernel of its own, so
// that each thread can hold its next contact's data in registers.  A patch or tile colour-round
// costs one L2 round trip for the contact's normal, forcing, Delassus block, mu and impulse when
// they are loaded after the barrier; here each thread loads its first contact of the next colour
// before the barrier that ends the current one (contact data do not change during a solve, and a
// contact's impulse is written only by the thread that sweeps it), so that after the barrier only
// the shared-memory velocities remain to be read.  The update of an isotropic disc block spends
// about half the FP64 operations of gs_update64_local (fused multiply-adds, the increment in
// FP32); checks and results stay FP64.
struct C64 {
  int k, la, lb;
  double2 n, c, r;
  double w00, w01, w11, mu;
};

// sab non-null: the group is the remainder, whose body slots come packed from shared memory
// (sab[q - sab0] = slot of a | slot of b << 16); otherwise from the packed pairs B.ab.
__device__ __forceinline__ void load64(const GsArgs& A, const Gs32Args& B, const PatchArgs& Q, int q, C64& x,
                                       const unsigned* sab, int sab0) {
  if (sab) {
    const unsigned ab = sab[q - sab0];
    x.la = (int)(ab & 0xffffu);
    x.lb = (int)(ab >> 16);
  } else {
    const int2 ab = B.ab[q];
    x.la = ab.x;
    x.lb = ab.y;
  }
  x.k = Q.order[q];
  x.n = A.n[x.k];
  x.c = A.c[x.k];
  x.w00 = A.W[3 * x.k];
  x.w01 = A.W[3 * x.k + 1];
  x.w11 = A.W[3 * x.k + 2];
  x.mu = A.mu[x.k];
  x.r = __ldcg(&A.r[x.k]);
}

// The local solve of a block that is not isotropic (none in a disc scene: the Delassus block of
// two discs or of a disc and a plane is a multiple of the identity), kept out of line so that its
// registers do not count against the sweeps'.
__device__ __noinline__ double2 general_local64(double2 n, double2 c, double2 r, double w00, double w01,
                                                double w11, double mu, double2 va, bool has_b, double2 vb) {
  double u0, u1, rn0, rn1;
  local_velocity(n, c, va, has_b, vb, u0, u1);
  const double bt0 = u0 - (w00 * r.x + w01 * r.y);
  const double bt1 = u1 - (w01 * r.x + w11 * r.y);
  local_solve_2d(w00, w01, w11, bt0, bt1, mu, rn0, rn1);
  return make_double2(rn0, rn1);
}

__device__ __forceinline__ void update64(const GsArgs& A, const C64& x, double2* sv, const double* sm) {
  const double2 va = sv[x.la];
  const bool has_b = x.lb >= 0;
  const double2 vb = has_b ? sv[x.lb] : make_double2(0.0, 0.0);
  double rn0, rn1;
  const double r0 = x.r.x, r1 = x.r.y;
  const double nx = x.n.x, ny = x.n.y;
  if (x.w01 == 0.0 && x.w00 == x.w11) {
    // Isotropic block: r_new = proj_cone(r - u / w).  GB300's FP64 pipe bounds these sweeps, so
    // u is formed with fused multiply-adds and the increment u / w in FP32 (near the solution u is
    // residual-sized, and its relative rounding, 6e-8, is far below what the FP64 check resolves);
    // the impulse and the velocities stay FP64.
    const double dvx = va.x - vb.x, dvy = va.y - vb.y;
    const double u0 = fma(nx, dvx, fma(ny, dvy, x.c.x));
    const double u1 = fma(-ny, dvx, fma(nx, dvy, x.c.y));
    const float iw = 1.0f / (float)x.w00;
    const double rn = r0 - (double)((float)u0 * iw);
    rn0 = rn > 0.0 ? rn : 0.0;
    const double rt = r1 - (double)((float)u1 * iw);
    const double lim = x.mu * rn0;
    rn1 = fabs(rt) <= lim ? rt : copysign(lim, rt);
  } else {
    const double2 rn = general_local64(x.n, x.c, x.r, x.w00, x.w01, x.w11, x.mu, va, has_b, vb);
    rn0 = rn.x;
    rn1 = rn.y;
  }
  const double d0 = rn0 - r0, d1 = rn1 - r1;
  const double px = fma(nx, d0, -ny * d1);
  const double py = fma(ny, d0, nx * d1);
  const double ma = sm[x.la];
  sv[x.la] = make_double2(fma(ma, px, va.x), fma(ma, py, va.y));
  if (has_b) {
    const double mb = sm[x.lb];
    sv[x.lb] = make_double2(fma(-mb, px, vb.x), fma(-mb, py, vb.y));
  }
  A.r[x.k] = make_double2(rn0, rn1);
}

// One group's colours on shared-memory velocities: off[0..ncol] are its (group, colour) runs.  A
// thread's contacts are loaded one ahead: the next colour's first before this colour's barrier,
// and within a colour each next one before the update of the one before it (contact data do not
// depend on the velocities).
__device__ __forceinline__ void sweep_group64(const GsArgs& A, const Gs32Args& B, const PatchArgs& Q,
                                              const int* off, int ncol, double2* sv, const double* sm,
                                              const unsigned* sab = nullptr, int sab0 = 0) {
  C64 nxt;
  bool have = false;
  if (ncol > 0 && off[0] + (int)threadIdx.x < off[1]) {
    load64(A, B, Q, off[0] + threadIdx.x, nxt, sab, sab0);
    have = true;
  }
  for (int col = 0; col < ncol; ++col) {
    const int e = off[col + 1];
    const int qn = (col + 1 < ncol) ? off[col + 1] + threadIdx.x : e;
    const bool have_n = col + 1 < ncol && qn < off[col + 2];
    if (have) {
      C64 cur = nxt;
      for (int q = off[col] + threadIdx.x + blockDim.x; q < e; q += blockDim.x) {
        C64 x;
        load64(A, B, Q, q, x, sab, sab0);
        update64(A, cur, sv, sm);
        cur = x;
      }
      update64(A, cur, sv, sm);
    }
    have = have_n;
    if (have) load64(A, B, Q, qn, nxt, sab, sab0);
    __syncthreads();
  }
}

// 256 threads: the FP64 pipe, not the thread count, bounds a colour-round, and 256 threads leave
// room for the prefetched contact in registers.
constexpr int kPatch64Block = 256;

__global__ void __launch_bounds__(kPatch64Block, 1) k_gs_patch64(GsArgs A, Gs32Args B, PatchArgs Q) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nthr = gridDim.x * blockDim.x;
  if (*((volatile int*)&A.st->status) != 0) return;
  extern __shared__ __align__(16) double2 sv64[];
  double* sm64 = reinterpret_cast<double*>(sv64 + Q.cap);
  double2* svq64 = reinterpret_cast<double2*>(sm64 + Q.cap);
  double* smq64 = reinterpret_cast<double*>(svq64 + Q.capq);
  // Block 0's copy of the remainder: its bodies' velocities and inverse masses (slots as cslot
  // numbers them), then each remaining contact's two slots packed in 32 bits.
  const int capc64 = (Q.rest64 + 1) & ~1;
  double2* svc64 = reinterpret_cast<double2*>(smq64 + Q.capq);
  double* smc64 = reinterpret_cast<double*>(svc64 + capc64);
  unsigned* sab64 = reinterpret_cast<unsigned*>(smc64 + capc64);
  __shared__ int s_goff[kMaxColors + 1];
  __shared__ int s_hoff[kMaxColors + 1];
  __shared__ int s_boff[kMaxColors + 1];
  const int P = Q.ps->P, Pb = Q.ps->Pb;
  const bool has_p = blockIdx.x < P, has_q = blockIdx.x < Pb;
  const int pb0 = has_p ? Q.pstart[blockIdx.x] : 0;
  const int pb1 = has_p ? Q.pstart[blockIdx.x + 1] : 0;
  const int pbe = pb0 + (has_p ? Q.pband[blockIdx.x] : 0);  // band bodies: [pb0, pbe)
  const int qb0 = has_q ? Q.qstart[blockIdx.x] : 0;
  const int qb1 = has_q ? Q.qstart[blockIdx.x + 1] : 0;
  for (int c = threadIdx.x; c <= kMaxColors; c += blockDim.x) {
    s_goff[c] = has_p ? Q.goff[blockIdx.x * kMaxColors + c] : 0;
    s_hoff[c] = has_q ? Q.goff[(P + blockIdx.x) * kMaxColors + c] : 0;
    s_boff[c] = Q.goff[(P + Pb) * kMaxColors + c];
  }
  for (int j = pb0 + threadIdx.x; j < pb1; j += blockDim.x) {
    sm64[j - pb0] = A.minv[Q.pbody[j]];
    sv64[j - pb0] = __ldcg(&A.v[Q.pbody[j]]);
  }
  for (int j = qb0 + threadIdx.x; j < qb1; j += blockDim.x) smq64[j - qb0] = A.minv[Q.qbody[j]];
  __syncthreads();
  const int ncol_p = group_colors(s_goff), ncol_q = group_colors(s_hoff), ncol_r = group_colors(s_boff);
  // The remainder's colours: the large leading ones over the grid (one grid barrier each), the
  // small trailing ones by block 0 (staged in its shared memory when the host found room).
  int btail = ncol_r;
  while (btail > 0 && s_boff[btail] - s_boff[btail - 1] <= 2 * (int)blockDim.x) --btail;
  const int sc0 = s_boff[btail], nrest_tail = s_boff[ncol_r] - sc0;
  const bool rest_staged = Q.rest64 > 0 && nrest_tail > 0;
  if (rest_staged && blockIdx.x == 0) {
    for (int j = threadIdx.x; j < Q.rest64; j += blockDim.x) smc64[j] = A.minv[Q.cbody[j]];
    for (int q = sc0 + threadIdx.x; q < sc0 + nrest_tail; q += blockDim.x) {
      const int2 ab = B.ab[q];
      sab64[q - sc0] = (unsigned)Q.cslot[ab.x] | ((unsigned)Q.cslot[ab.y] << 16);
    }
  }
  __syncthreads();
  const unsigned eval64 = A.eval_every ? A.eval_every : 1u;
  double2* best = A.r_a;
  double2* cand = A.r_b;
  double err_best = INFINITY;
  bool converged = false;
  unsigned it = 0, n_eval = 0, s64 = 0;
  // Checks as in k_gs_patch's FP64 phase: where the residual's rate predicts tol, at most
  // 16 eval64 apart, the gap doubling where the residual did not decrease.
  unsigned next64 = eval64, interval64 = eval64, prev64_it = 0;
  double prev64_err = INFINITY;
  // Block 0's phase times (globaltimer): [0] patch interior, [1] the barrier after it and the
  // shifted tile, [2] the barrier after that and the remainder, [3] checks.
  // In shared memory, so that they take no registers from the sweeps; [4] is the running mark.
  __shared__ unsigned long long t_ph[5];
  const bool timer = tid == 0;
  if (timer) t_ph[0] = t_ph[1] = t_ph[2] = t_ph[3] = t_ph[4] = 0ull;
  for (it = 1; it <= A.max_iters; ++it) {
    const bool do_eval = it >= next64 || it == A.max_iters;
    if (timer) t_ph[4] = globaltimer_ns();
    // The patch's interior (band bodies reloaded: tiles and the remainder touched them).
    if (it > 1)
      for (int j = pb0 + threadIdx.x; j < pbe; j += blockDim.x) sv64[j - pb0] = __ldcg(&A.v[Q.pbody[j]]);
    __syncthreads();
    sweep_group64(A, B, Q, s_goff, ncol_p, sv64, sm64);
    if (timer) {
      const unsigned long long t = globaltimer_ns();
      t_ph[0] += t - t_ph[4];
      t_ph[4] = t;
    }
    const int wend = do_eval ? pb1 : pbe;
    for (int j = pb0 + threadIdx.x; j < wend; j += blockDim.x) A.v[Q.pbody[j]] = sv64[j - pb0];
    if (!grid_sync(A.gb, A.spin)) {
      if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
      return;
    }
    // The shifted tile's contacts between patches.
    if (qb1 > qb0) {
      for (int j = qb0 + threadIdx.x; j < qb1; j += blockDim.x) svq64[j - qb0] = __ldcg(&A.v[Q.qbody[j]]);
      __syncthreads();
      sweep_group64(A, B, Q, s_hoff, ncol_q, svq64, smq64);
      for (int j = qb0 + threadIdx.x; j < qb1; j += blockDim.x) A.v[Q.qbody[j]] = svq64[j - qb0];
    }
    if (timer) {
      const unsigned long long t = globaltimer_ns();
      t_ph[1] += t - t_ph[4];
      t_ph[4] = t;
    }
    if (!grid_sync(A.gb, A.spin)) {
      if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
      return;
    }
    // The remainder: large colours over the grid on global velocities, then the small trailing
    // ones by block 0, on shared-memory velocities when staged.
    for (int col = 0; col < btail; ++col) {
      const int b0 = s_boff[col], e = s_boff[col + 1];
      if (b0 == e) continue;
      for (int q = b0 + tid; q < e; q += nthr) gs_update(A, Q.order[q]);
      if (!grid_sync(A.gb, A.spin)) {
        if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
        return;
      }
    }
    if (nrest_tail > 0) {
      if (blockIdx.x == 0) {
        if (rest_staged) {
          for (int j = threadIdx.x; j < Q.rest64; j += blockDim.x) svc64[j] = __ldcg(&A.v[Q.cbody[j]]);
          __syncthreads();
          sweep_group64(A, B, Q, s_boff + btail, ncol_r - btail, svc64, smc64, sab64, sc0);
          for (int j = threadIdx.x; j < Q.rest64; j += blockDim.x) A.v[Q.cbody[j]] = svc64[j];
        } else {
          for (int col = btail; col < ncol_r; ++col) {
            for (int q = s_boff[col] + threadIdx.x; q < s_boff[col + 1]; q += blockDim.x) gs_update(A, Q.order[q]);
            __syncthreads();
          }
        }
      }
      if (!grid_sync(A.gb, A.spin)) {
        if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
        return;
      }
    }
    ++s64;
    if (timer) {
      const unsigned long long t = globaltimer_ns();
      t_ph[2] += t - t_ph[4];
      t_ph[4] = t;
    }
    if (!do_eval) continue;
    double emax = 0.0;
    for (int k = tid; k < A.nc; k += nthr) {
      const int a = A.ia[k], b = A.ib[k];
      const bool has_b = b >= 0;
      const double2 va = __ldcg(&A.v[a]);
      const double2 vb = has_b ? __ldcg(&A.v[b]) : make_double2(0.0, 0.0);
      double u0, u1;
      local_velocity(A.n[k], A.c[k], va, has_b, vb, u0, u1);
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
    if (timer) t_ph[3] += globaltimer_ns() - t_ph[4];
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
    if (err < prev64_err && prev64_err < INFINITY && err > 0.0) {
      const double per_sweep = (log(err) - log(prev64_err)) / (double)(it - prev64_it);
      const double need = (log(A.tol) - log(err)) / per_sweep;
      interval64 = need >= (double)(16u * eval64) ? 16u * eval64 : max(eval64, (unsigned)need);
    } else {
      interval64 = min(2u * interval64, 16u * eval64);
    }
    prev64_err = err;
    prev64_it = it;
    next64 = it + interval64;
  }
  if (it > A.max_iters) it = A.max_iters;
  if (!converged && err_best < INFINITY)
    for (int k = tid; k < A.nc; k += nthr) A.r[k] = __ldcg(&best[k]);
  if (tid == 0) {
    A.st->iterations = it;
    A.st->converged = converged ? 1 : 0;
    A.st->error = err_best;
    A.st->sweeps32 = 0;
    A.st->sweeps64 = s64;
    A.st->evals = n_eval;
    A.st->lifts = 0;
    A.st->boundary_contacts = Q.goff[(P + Pb + 1) * kMaxColors] - Q.goff[P * kMaxColors];
    int nbc = 0;
    for (int c = 0; c < ncol_r; ++c) nbc += s_boff[c + 1] > s_boff[c];
    A.st->boundary_colors = nbc;
    // Profile fields: interior; the barrier after it and the tile; the barrier after that, the
    // remainder and the checks.
    A.st->phase_ns[0] = t_ph[0];
    A.st->phase_ns[1] = t_ph[1];
    A.st->phase_ns[2] = t_ph[2] + t_ph[3];
  }
}

// ---------------------------------------------------------------------------
// FP64 continuation on the two-level partition in float-float arithmetic (k_gs_patch_ff).
//
// GB300 issues FP64 at a small fraction of its FP32 rate, and k_gs_patch64's patch sweeps are
// bound by that pipe.  Here the sweep state (body velocities and contact impulses) is held as
// float-float pairs (hi + lo, 48 significant bits) and updated on the FP32 pipe: error-free sums
// and products (Knuth's two-sum, FMA two-product) as in the double-double arithmetic of Dekker
// (1971) and of Hida, Li and Bailey's QD library, restated for pairs of floats.  The contact data
// (normal, forcing, mu, 1/m) are split into pairs too, so that the iteration solves the FP64
// problem to about 2^-46 of its magnitudes; only the increment u / w of the isotropic local solve
// is an FP32 product, as in k_gs_patch64.  Velocities follow the impulses through float-float
// updates.  Each check converts the impulses to FP64, recomputes the velocities from them in FP64
// (v = v0 + M^-1 H^T r), evaluates the residual in FP64 as every other kernel, and restarts the
// pairs from those velocities: the residual reported is that of the returned impulses, and the
// pairs' rounding (amplified by 1/m where small discs carry large impulses) never accumulates past
// a check.  Ball2D contacts only: their Delassus blocks are isotropic by construction (w01 = 0,
// w00 = w11).
struct FfArgs {
  float4* n;     // per packed contact: nx, ny as pairs (hi, lo, hi, lo)
  float4* c;     // forcing c as pairs
  float4* m;     // mu as a pair, 1 / w00 in FP32, unused
  float4* r;     // impulse as pairs (the sweep state)
  float4* v;     // per body: velocity as pairs (the state between phases)
  float2* minv;  // per body: 1 / m as a pair
};

// Sweep data of one packed contact (a C64 in pairs).
struct CFF {
  int q, la, lb;
  float4 n, c, m, r;
};

__device__ __forceinline__ void load_ff(const Gs32Args& B, const FfArgs& F, int q, CFF& x, const unsigned* sab,
                                        int sab0) {
  if (sab) {
    const unsigned ab = sab[q - sab0];
    x.la = (int)(ab & 0xffffu);
    x.lb = (int)(ab >> 16);
  } else {
    const int2 ab = B.ab[q];
    x.la = ab.x;
    x.lb = ab.y;
  }
  x.q = q;
  x.n = F.n[q];
  x.c = F.c[q];
  x.m = F.m[q];
  x.r = __ldcg(&F.r[q]);
}

// The isotropic update of update64 in pairs: u = H v + c, r_new = proj_cone(r - u / w) with the
// increment u / w in FP32, then v += M^-1 H^T (r_new - r).  kGlobal: the velocities are the
// global pairs of F.v (read at L2: other SMs wrote them before the last grid barrier).
template <bool kGlobal>
__device__ __forceinline__ void update_ff(const FfArgs& F, const CFF& x, float4* sv, const float2* sm) {
  const float4 a4 = kGlobal ? __ldcg(&sv[x.la]) : sv[x.la];
  const bool has_b = x.lb >= 0;
  const float4 b4 = has_b ? (kGlobal ? __ldcg(&sv[x.lb]) : sv[x.lb]) : make_float4(0.f, 0.f, 0.f, 0.f);
  const FF nx = ff_make(x.n.x, x.n.y), ny = ff_make(x.n.z, x.n.w);
  const FF dvx = ff_sub(ff_make(a4.x, a4.y), ff_make(b4.x, b4.y));
  const FF dvy = ff_sub(ff_make(a4.z, a4.w), ff_make(b4.z, b4.w));
  const FF u0 = ff_add(ff_add(ff_mul(nx, dvx), ff_mul(ny, dvy)), ff_make(x.c.x, x.c.y));
  const FF u1 = ff_add(ff_sub(ff_mul(nx, dvy), ff_mul(ny, dvx)), ff_make(x.c.z, x.c.w));
  const float iw = x.m.z;
  const FF r0 = ff_make(x.r.x, x.r.y), r1 = ff_make(x.r.z, x.r.w);
  const FF rn = ff_add_f(r0, -__fmul_rn(u0.hi, iw));
  const FF rn0 = rn.hi > 0.f ? rn : ff_make(0.f, 0.f);
  const FF rt = ff_add_f(r1, -__fmul_rn(u1.hi, iw));
  const FF lim = ff_mul(ff_make(x.m.x, x.m.y), rn0);
  const bool neg = signbit(rt.hi);
  const FF art = neg ? ff_neg(rt) : rt;
  const bool inside = art.hi < lim.hi || (art.hi == lim.hi && art.lo <= lim.lo);
  const FF rn1 = inside ? rt : (neg ? ff_neg(lim) : lim);
  const FF d0 = ff_sub(rn0, r0), d1 = ff_sub(rn1, r1);
  const FF px = ff_sub(ff_mul(nx, d0), ff_mul(ny, d1));
  const FF py = ff_add(ff_mul(ny, d0), ff_mul(nx, d1));
  const float2 ma2 = sm[x.la];
  const FF ma = ff_make(ma2.x, ma2.y);
  const FF vax = ff_add(ff_make(a4.x, a4.y), ff_mul(ma, px));
  const FF vay = ff_add(ff_make(a4.z, a4.w), ff_mul(ma, py));
  sv[x.la] = make_float4(vax.hi, vax.lo, vay.hi, vay.lo);
  if (has_b) {
    const float2 mb2 = sm[x.lb];
    const FF mb = ff_make(mb2.x, mb2.y);
    const FF vbx = ff_sub(ff_make(b4.x, b4.y), ff_mul(mb, px));
    const FF vby = ff_sub(ff_make(b4.z, b4.w), ff_mul(mb, py));
    sv[x.lb] = make_float4(vbx.hi, vbx.lo, vby.hi, vby.lo);
  }
  F.r[x.q] = make_float4(rn0.hi, rn0.lo, rn1.hi, rn1.lo);
}

// sweep_group64 in pairs.
__device__ __forceinline__ void sweep_group_ff(const Gs32Args& B, const FfArgs& F, const int* off, int ncol,
                                               float4* sv, const float2* sm, const unsigned* sab = nullptr,
                                               int sab0 = 0) {
  CFF nxt;
  bool have = false;
  if (ncol > 0 && off[0] + (int)threadIdx.x < off[1]) {
    load_ff(B, F, off[0] + threadIdx.x, nxt, sab, sab0);
    have = true;
  }
  for (int col = 0; col < ncol; ++col) {
    const int e = off[col + 1];
    const int qn = (col + 1 < ncol) ? off[col + 1] + threadIdx.x : e;
    const bool have_n = col + 1 < ncol && qn < off[col + 2];
    if (have) {
      CFF cur = nxt;
      for (int q = off[col] + threadIdx.x + blockDim.x; q < e; q += blockDim.x) {
        CFF x;
        load_ff(B, F, q, x, sab, sab0);
        update_ff<false>(F, cur, sv, sm);
        cur = x;
      }
      update_ff<false>(F, cur, sv, sm);
    }
    have = have_n;
    if (have) load_ff(B, F, qn, nxt, sab, sab0);
    __syncthreads();
  }
}

// The FP64 state split into pairs, by packed position (contacts; by contact index when order is
// null) and by body.
__global__ void k_pack_ff(int nc, int nb, const int* __restrict__ order, const double2* __restrict__ n,
                          const double2* __restrict__ c, const double* __restrict__ W, const double* __restrict__ mu,
                          const double2* __restrict__ r, const double2* __restrict__ v,
                          const double* __restrict__ minv, FfArgs F) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nc) {
    const int k = order ? order[t] : t;
    const double2 nk = n[k], ck = c[k], rk = r[k];
    const FF nx = ff_split(nk.x), ny = ff_split(nk.y), cx = ff_split(ck.x), cy = ff_split(ck.y);
    const FF m = ff_split(mu[k]), r0 = ff_split(rk.x), r1 = ff_split(rk.y);
    F.n[t] = make_float4(nx.hi, nx.lo, ny.hi, ny.lo);
    F.c[t] = make_float4(cx.hi, cx.lo, cy.hi, cy.lo);
    F.m[t] = make_float4(m.hi, m.lo, __double2float_rn(1.0 / W[3 * k]), 0.f);
    F.r[t] = make_float4(r0.hi, r0.lo, r1.hi, r1.lo);
  }
  if (t < nb) {
    const double2 vi = v[t];
    const FF vx = ff_split(vi.x), vy = ff_split(vi.y), mi = ff_split(minv[t]);
    F.v[t] = make_float4(vx.hi, vx.lo, vy.hi, vy.lo);
    F.minv[t] = make_float2(mi.hi, mi.lo);
  }
}

// One-level FP64-precision sweeps in float-float pairs (k_gs_mixed's FP64 sweeps in the pairs of
// k_gs_patch_ff): the global colour order over all contacts, velocities as pairs in global memory,
// contact data and impulses as pairs by contact index; checks as in k_gs_patch_ff.  The FP32
// form's one-level FP64 continuation for discs.
constexpr int kGsFf1Block = 256;

__global__ void __launch_bounds__(kGsFf1Block, 1) k_gs_ff1(GsArgs A, Gs32Args B, FfArgs F) {
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
  double2* best = A.r_a;
  double2* cand = A.r_b;
  double err_best = INFINITY;
  bool converged = false;
  unsigned it = 0, n_eval = 0;
  unsigned next64 = eval64, interval64 = eval64, prev64_it = 0;
  double prev64_err = INFINITY;
  for (it = 1; it <= A.max_iters; ++it) {
    for (int col = 0; col < ncol; ++col) {
      const int e = s_off[col + 1];
      for (int s = s_off[col] + tid; s < e; s += nthr) {
        const int k = A.perm[s];
        CFF x;
        x.q = k;
        x.la = A.ia[k];
        x.lb = A.ib[k];
        x.n = F.n[k];
        x.c = F.c[k];
        x.m = F.m[k];
        x.r = __ldcg(&F.r[k]);
        update_ff<true>(F, x, F.v, F.minv);
      }
      if (!grid_sync(A.gb, A.spin)) {
        if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
        return;
      }
    }
    if (!(it >= next64 || it == A.max_iters)) continue;
    for (int k = tid; k < A.nc; k += nthr) {
      const float4 w = __ldcg(&F.r[k]);
      A.r[k] = make_double2(ff_value(ff_make(w.x, w.y)), ff_value(ff_make(w.z, w.w)));
    }
    if (!grid_sync(A.gb, A.spin)) {
      if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
      return;
    }
    for (int i = tid; i < B.nb; i += nthr) {
      double hx = 0.0, hy = 0.0;
      const int e = B.body_off[i + 1];
      for (int p = B.body_off[i]; p < e; ++p) {
        const int k = B.body_adj[p];
        const double sgn = (A.ia[k] == i) ? 1.0 : -1.0;
        const double2 nk = A.n[k], rk = __ldcg(&A.r[k]);
        const double px = nk.x * rk.x + (-nk.y) * rk.y;
        const double py = nk.y * rk.x + nk.x * rk.y;
        hx = hx + sgn * px;
        hy = hy + sgn * py;
      }
      const double2 a = B.v0[i];
      const double mi = B.minv64[i];
      const double2 vi = make_double2(a.x + mi * hx, a.y + mi * hy);
      A.v[i] = vi;
      const FF vx = ff_split(vi.x), vy = ff_split(vi.y);
      F.v[i] = make_float4(vx.hi, vx.lo, vy.hi, vy.lo);
    }
    if (!grid_sync(A.gb, A.spin)) {
      if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
      return;
    }
    double emax = 0.0;
    for (int k = tid; k < A.nc; k += nthr) {
      const int a = A.ia[k], b = A.ib[k];
      const bool has_b = b >= 0;
      const double2 va = __ldcg(&A.v[a]);
      const double2 vb = has_b ? __ldcg(&A.v[b]) : make_double2(0.0, 0.0);
      double u0, u1;
      local_velocity(A.n[k], A.c[k], va, has_b, vb, u0, u1);
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
    if (err < prev64_err && prev64_err < INFINITY && err > 0.0) {
      const double per_sweep = (log(err) - log(prev64_err)) / (double)(it - prev64_it);
      const double need = (log(A.tol) - log(err)) / per_sweep;
      interval64 = need >= (double)(16u * eval64) ? 16u * eval64 : max(eval64, (unsigned)need);
    } else {
      interval64 = min(2u * interval64, 16u * eval64);
    }
    prev64_err = err;
    prev64_it = it;
    next64 = it + interval64;
  }
  if (it > A.max_iters) it = A.max_iters;
  if (!converged && err_best < INFINITY)
    for (int k = tid; k < A.nc; k += nthr) A.r[k] = __ldcg(&best[k]);
  if (tid == 0) {
    A.st->iterations = it;
    A.st->converged = converged ? 1 : 0;
    A.st->error = err_best;
    A.st->sweeps32 = 0;
    A.st->sweeps64 = it;
    A.st->evals = n_eval;
    A.st->lifts = 0;
  }
}


__global__ void __launch_bounds__(kPatch64Block, 1) k_gs_patch_ff(GsArgs A, Gs32Args B, PatchArgs Q, FfArgs F) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nthr = gridDim.x * blockDim.x;
  if (*((volatile int*)&A.st->status) != 0) return;
  extern __shared__ __align__(16) float4 svf[];
  float2* smf = reinterpret_cast<float2*>(svf + Q.cap);
  float4* svqf = reinterpret_cast<float4*>(smf + Q.cap);
  float2* smqf = reinterpret_cast<float2*>(svqf + Q.capq);
  const int capc = (Q.rest64 + 1) & ~1;
  float4* svcf = reinterpret_cast<float4*>(smqf + Q.capq);
  float2* smcf = reinterpret_cast<float2*>(svcf + capc);
  unsigned* sabf = reinterpret_cast<unsigned*>(smcf + capc);
  __shared__ int s_goff[kMaxColors + 1];
  __shared__ int s_hoff[kMaxColors + 1];
  __shared__ int s_boff[kMaxColors + 1];
  const int P = Q.ps->P, Pb = Q.ps->Pb;
  const bool has_p = blockIdx.x < P, has_q = blockIdx.x < Pb;
  const int pb0 = has_p ? Q.pstart[blockIdx.x] : 0;
  const int pb1 = has_p ? Q.pstart[blockIdx.x + 1] : 0;
  const int pbe = pb0 + (has_p ? Q.pband[blockIdx.x] : 0);  // band bodies: [pb0, pbe)
  const int qb0 = has_q ? Q.qstart[blockIdx.x] : 0;
  const int qb1 = has_q ? Q.qstart[blockIdx.x + 1] : 0;
  for (int c = threadIdx.x; c <= kMaxColors; c += blockDim.x) {
    s_goff[c] = has_p ? Q.goff[blockIdx.x * kMaxColors + c] : 0;
    s_hoff[c] = has_q ? Q.goff[(P + blockIdx.x) * kMaxColors + c] : 0;
    s_boff[c] = Q.goff[(P + Pb) * kMaxColors + c];
  }
  for (int j = pb0 + threadIdx.x; j < pb1; j += blockDim.x) {
    smf[j - pb0] = F.minv[Q.pbody[j]];
    svf[j - pb0] = __ldcg(&F.v[Q.pbody[j]]);
  }
  for (int j = qb0 + threadIdx.x; j < qb1; j += blockDim.x) smqf[j - qb0] = F.minv[Q.qbody[j]];
  __syncthreads();
  const int ncol_p = group_colors(s_goff), ncol_q = group_colors(s_hoff), ncol_r = group_colors(s_boff);
  int btail = ncol_r;
  while (btail > 0 && s_boff[btail] - s_boff[btail - 1] <= 2 * (int)blockDim.x) --btail;
  const int sc0 = s_boff[btail], nrest_tail = s_boff[ncol_r] - sc0;
  const bool rest_staged = Q.rest64 > 0 && nrest_tail > 0;
  if (rest_staged && blockIdx.x == 0) {
    for (int j = threadIdx.x; j < Q.rest64; j += blockDim.x) smcf[j] = F.minv[Q.cbody[j]];
    for (int q = sc0 + threadIdx.x; q < sc0 + nrest_tail; q += blockDim.x) {
      const int2 ab = B.ab[q];
      sabf[q - sc0] = (unsigned)Q.cslot[ab.x] | ((unsigned)Q.cslot[ab.y] << 16);
    }
  }
  __syncthreads();
  const unsigned eval64 = A.eval_every ? A.eval_every : 1u;
  double2* best = A.r_a;
  double2* cand = A.r_b;
  double err_best = INFINITY;
  bool converged = false;
  unsigned it = 0, n_eval = 0, s64 = 0;
  unsigned next64 = eval64, interval64 = eval64, prev64_it = 0;
  double prev64_err = INFINITY;
  __shared__ unsigned long long t_ph[5];
  const bool timer = tid == 0;
  if (timer) t_ph[0] = t_ph[1] = t_ph[2] = t_ph[3] = t_ph[4] = 0ull;
  // After a check every velocity was recomputed from the impulses: the next sweep reloads them all.
  bool reload_all = false;
  for (it = 1; it <= A.max_iters; ++it) {
    const bool do_eval = it >= next64 || it == A.max_iters;
    if (timer) t_ph[4] = globaltimer_ns();
    if (it > 1) {
      const int lend = reload_all ? pb1 : pbe;
      for (int j = pb0 + threadIdx.x; j < lend; j += blockDim.x) svf[j - pb0] = __ldcg(&F.v[Q.pbody[j]]);
      reload_all = false;
    }
    __syncthreads();
    sweep_group_ff(B, F, s_goff, ncol_p, svf, smf);
    if (timer) {
      const unsigned long long t = globaltimer_ns();
      t_ph[0] += t - t_ph[4];
      t_ph[4] = t;
    }
    const int wend = do_eval ? pb1 : pbe;
    for (int j = pb0 + threadIdx.x; j < wend; j += blockDim.x) F.v[Q.pbody[j]] = svf[j - pb0];
    if (!grid_sync(A.gb, A.spin)) {
      if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
      return;
    }
    if (qb1 > qb0) {
      for (int j = qb0 + threadIdx.x; j < qb1; j += blockDim.x) svqf[j - qb0] = __ldcg(&F.v[Q.qbody[j]]);
      __syncthreads();
      sweep_group_ff(B, F, s_hoff, ncol_q, svqf, smqf);
      for (int j = qb0 + threadIdx.x; j < qb1; j += blockDim.x) F.v[Q.qbody[j]] = svqf[j - qb0];
    }
    if (timer) {
      const unsigned long long t = globaltimer_ns();
      t_ph[1] += t - t_ph[4];
      t_ph[4] = t;
    }
    if (!grid_sync(A.gb, A.spin)) {
      if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
      return;
    }
    for (int col = 0; col < btail; ++col) {
      const int b0 = s_boff[col], e = s_boff[col + 1];
      if (b0 == e) continue;
      for (int q = b0 + tid; q < e; q += nthr) {
        CFF x;
        load_ff(B, F, q, x, nullptr, 0);
        update_ff<true>(F, x, F.v, F.minv);
      }
      if (!grid_sync(A.gb, A.spin)) {
        if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
        return;
      }
    }
    if (nrest_tail > 0) {
      if (blockIdx.x == 0) {
        if (rest_staged) {
          for (int j = threadIdx.x; j < Q.rest64; j += blockDim.x) svcf[j] = __ldcg(&F.v[Q.cbody[j]]);
          __syncthreads();
          sweep_group_ff(B, F, s_boff + btail, ncol_r - btail, svcf, smcf, sabf, sc0);
          for (int j = threadIdx.x; j < Q.rest64; j += blockDim.x) F.v[Q.cbody[j]] = svcf[j];
        } else {
          for (int col = btail; col < ncol_r; ++col) {
            for (int q = s_boff[col] + threadIdx.x; q < s_boff[col + 1]; q += blockDim.x) {
              CFF x;
              load_ff(B, F, q, x, nullptr, 0);
              update_ff<true>(F, x, F.v, F.minv);
            }
            __syncthreads();
          }
        }
      }
      if (!grid_sync(A.gb, A.spin)) {
        if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
        return;
      }
    }
    ++s64;
    if (timer) {
      const unsigned long long t = globaltimer_ns();
      t_ph[2] += t - t_ph[4];
      t_ph[4] = t;
    }
    if (!do_eval) continue;
    // The impulses in FP64, then the velocities recomputed from them in FP64 (v = v0 + M^-1 H^T r,
    // as k_gs_mixed's lift), so that the check evaluates exactly the returned impulses, and the
    // pairs restarted from those velocities; then the FP64 check.
    for (int q = tid; q < A.nc; q += nthr) {
      const float4 w = __ldcg(&F.r[q]);
      A.r[Q.order[q]] = make_double2(ff_value(ff_make(w.x, w.y)), ff_value(ff_make(w.z, w.w)));
    }
    if (!grid_sync(A.gb, A.spin)) {
      if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
      return;
    }
    for (int i = tid; i < B.nb; i += nthr) {
      double hx = 0.0, hy = 0.0;
      const int e = B.body_off[i + 1];
      for (int p = B.body_off[i]; p < e; ++p) {
        const int k = B.body_adj[p];
        const double sgn = (A.ia[k] == i) ? 1.0 : -1.0;
        const double2 nk = A.n[k], rk = __ldcg(&A.r[k]);
        const double px = nk.x * rk.x + (-nk.y) * rk.y;
        const double py = nk.y * rk.x + nk.x * rk.y;
        hx = hx + sgn * px;
        hy = hy + sgn * py;
      }
      const double2 a = B.v0[i];
      const double mi = B.minv64[i];
      const double2 vi = make_double2(a.x + mi * hx, a.y + mi * hy);
      A.v[i] = vi;
      const FF vx = ff_split(vi.x), vy = ff_split(vi.y);
      F.v[i] = make_float4(vx.hi, vx.lo, vy.hi, vy.lo);
    }
    reload_all = true;
    if (!grid_sync(A.gb, A.spin)) {
      if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
      return;
    }
    double emax = 0.0;
    for (int k = tid; k < A.nc; k += nthr) {
      const int a = A.ia[k], b = A.ib[k];
      const bool has_b = b >= 0;
      const double2 va = __ldcg(&A.v[a]);
      const double2 vb = has_b ? __ldcg(&A.v[b]) : make_double2(0.0, 0.0);
      double u0, u1;
      local_velocity(A.n[k], A.c[k], va, has_b, vb, u0, u1);
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
    if (timer) t_ph[3] += globaltimer_ns() - t_ph[4];
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
    // A check (impulses to FP64, velocities recomputed, the residual) costs several of these
    // sweeps: the gap may grow to 64 eval64 in a long solve, at most a quarter of the sweeps done.
    const unsigned cap64 = min(64u * eval64, max(16u * eval64, it / 4u));
    if (err < prev64_err && prev64_err < INFINITY && err > 0.0) {
      const double per_sweep = (log(err) - log(prev64_err)) / (double)(it - prev64_it);
      const double need = (log(A.tol) - log(err)) / per_sweep;
      interval64 = need >= (double)cap64 ? cap64 : max(eval64, (unsigned)need);
    } else {
      interval64 = min(2u * interval64, cap64);
    }
    prev64_err = err;
    prev64_it = it;
    next64 = it + interval64;
  }
  if (it > A.max_iters) it = A.max_iters;
  if (!converged && err_best < INFINITY)
    for (int k = tid; k < A.nc; k += nthr) A.r[k] = __ldcg(&best[k]);
  if (tid == 0) {
    A.st->iterations = it;
    A.st->converged = converged ? 1 : 0;
    A.st->error = err_best;
    A.st->sweeps32 = 0;
    A.st->sweeps64 = s64;
    A.st->evals = n_eval;
    A.st->lifts = 0;
    A.st->boundary_contacts = Q.goff[(P + Pb + 1) * kMaxColors] - Q.goff[P * kMaxColors];
    int nbc = 0;
    for (int c = 0; c < ncol_r; ++c) nbc += s_boff[c + 1] > s_boff[c];
    A.st->boundary_colors = nbc;
    A.st->phase_ns[0] = t_ph[0];
    A.st->phase_ns[1] = t_ph[1];
    A.st->phase_ns[2] = t_ph[2] + t_ph[3];
  }
}

// FP64 Coulomb residual of a start impulse r at running velocities v (one residual
// evaluation of k_gs), maximum into *slot (ordered encoding).
__global__ void k_start_err(int nc, const int* __restrict__ ia, const int* __restrict__ ib,
                            const double2* __restrict__ n, const double2* __restrict__ c,
                            const double* __restrict__ mu, const double2* __restrict__ r,
                            const double2* __restrict__ v, unsigned long long* slot) {
  double emax = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nc; k += gridDim.x * blockDim.x) {
    const int a = ia[k], b = ib[k];
    const bool has_b = b >= 0;
    const double2 va = v[a];
    const double2 vb = has_b ? v[b] : make_double2(0.0, 0.0);
    double u0, u1;
    local_velocity(n[k], c[k], va, has_b, vb, u0, u1);
    const double2 rk = r[k];
    emax = nanmax(emax, fb_error_2d(rk.x, rk.y, u0, u1, mu[k]));
  }
  emax = block_nanmax(emax);
  if (threadIdx.x == 0) atomicMax(slot, f64_to_ordered(emax));
}

// Keeps the start with the smaller residual (slot[0]: current, slot[1]: network).
__global__ void k_select_start(int nc, double2* __restrict__ r, const double2* __restrict__ r_alt,
                               const unsigned long long* __restrict__ slot, unsigned long long* chosen) {
  const double e_cur = ordered_to_f64(slot[0]), e_alt = ordered_to_f64(slot[1]);
  const bool take = e_alt < e_cur;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k == 0 && take) *chosen += 1ull;
  if (k < nc && take) r[k] = r_alt[k];
}

// ---------------------------------------------------------------------------
// Batched scenes with FP32 sweeps: every scene is in one of three modes, FP32 sweeping,
// FP64 sweeping (refinement) or done, and moves between them on its own FP64 residual
// exactly as a single scene does in k_gs_mixed (FP64 hand-over when FP32 reached tol or
// hit its rounding floor; done when an FP64 residual is below tol).  FP32 scenes are
// checked on a common schedule (sweeps 1, 2, 4, ... eval32, then an interval that grows
// while the largest FP32-scene residual is far above tol); FP64 scenes every eval_every
// sweeps.  A contact's colour slot runs the update of its scene's mode.
struct GsMixedBatchArgs {
  GsBatchArgs X;          // per-scene state (err_slot, best, bestbuf, done, iters, done_count)
  const int* pscene;      // scene of each packed contact
  const int* scene_of;    // scene of each body
  int* mode;              // S: 0 FP32, 1 FP64
  unsigned* since;        // S: checks since the scene's best
  unsigned long long* exc_slot;  // 3 S: FP32 rounding-floor excess per scene
  unsigned long long* gmax;      // 3: largest residual of the FP32 scenes per check
  int* n64;                      // scenes in FP64 mode
  unsigned long long* work;      // [0] FP32 contact updates, [1] FP64 contact updates, [2] contact
                                 // evaluations, [3] contact lifts, [4] body lifts
};

__global__ void __launch_bounds__(kGs32Block, 1) k_gs_mixed_batch(GsMixedBatchArgs M, Gs32Args B) {
  GsBatchArgs& X = M.X;
  const GsArgs& A = X.g;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nthr = gridDim.x * blockDim.x;
  if (*((volatile int*)&A.st->status) != 0) return;
  __shared__ int s_off[kMaxColors + 1];
  __shared__ int s_ncol;
  if (threadIdx.x == 0) s_ncol = A.st->n_colors;
  for (int c = threadIdx.x; c <= kMaxColors; c += blockDim.x) s_off[c] = A.st->color_off[c];
  const int nc = *X.nc_dev;
  const int S = X.S;
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
  double2* bufs[2] = {A.r_a, A.r_b};
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
        for (int s = s_off[col] + tid; s < e; s += nthr) {
          const int sc = M.pscene[s];
          if (__ldcg(&X.done[sc])) continue;
          if (__ldcg(&M.mode[sc]) == 0) {
            gs_update32(B, s);
            ++n32;
          } else {
            gs_update(A, A.perm[s]);
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
        // Lift the FP32 scenes' iterates to FP64 and resynchronise their FP32 velocities.
        for (int s = tid; s < nc; s += nthr) {
          const int sc = M.pscene[s];
          if (__ldcg(&X.done[sc]) || __ldcg(&M.mode[sc]) != 0) continue;
          const float2 r32 = __ldcg(&B.r[s]);
          A.r[A.perm[s]] = make_double2((double)r32.x, (double)r32.y);
          ++nlc;
        }
        if (!grid_sync(A.gb, A.spin)) {
          if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
          return;
        }
        for (int i = tid; i < B.nb; i += nthr) {
          const int sc = M.scene_of[i];
          if (__ldcg(&X.done[sc]) || __ldcg(&M.mode[sc]) != 0) continue;
          double hx = 0.0, hy = 0.0;
          const int e = B.body_off[i + 1];
          for (int p = B.body_off[i]; p < e; ++p) {
            const int k = B.body_adj[p];
            const double sgn = (A.ia[k] == i) ? 1.0 : -1.0;
            const double2 nk = A.n[k], rk = __ldcg(&A.r[k]);
            const double px = nk.x * rk.x + (-nk.y) * rk.y;
            const double py = nk.y * rk.x + nk.x * rk.y;
            hx = hx + sgn * px;
            hy = hy + sgn * py;
          }
          const double2 a = B.v0[i];
          const double mi = B.minv64[i];
          const double2 vi = make_double2(a.x + mi * hx, a.y + mi * hy);
          A.v[i] = vi;
          B.v[i] = make_float2((float)vi.x, (float)vi.y);
          ++nlb;
        }
        if (!grid_sync(A.gb, A.spin)) {
          if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
          return;
        }
      }
      // FP64 residual and FP32 floor excess of every due scene.
      const int slot = n_eval % 3;
      unsigned long long* eslots = X.err_slot + (size_t)slot * S;
      unsigned long long* xslots = M.exc_slot + (size_t)slot * S;
      const int lane = threadIdx.x & 31;
      for (int k0 = tid - lane; k0 < nc; k0 += nthr) {
        const int k = k0 + lane;
        int key = -1;
        unsigned long long ve = 0ull, vx = 0ull;
        if (k < nc) {
          const int sc = X.cscene[k];
          const int md = __ldcg(&M.mode[sc]);
          if (!__ldcg(&X.done[sc]) && ((md == 0 && due32) || (md == 1 && due64))) {
            const int a = A.ia[k], b = A.ib[k];
            const bool has_b = b >= 0;
            const double2 va = __ldcg(&A.v[a]);
            const double2 vb = has_b ? __ldcg(&A.v[b]) : make_double2(0.0, 0.0);
            const double2 ck = A.c[k];
            double u0, u1;
            local_velocity(A.n[k], ck, va, has_b, vb, u0, u1);
            const double2 rk = __ldcg(&A.r[k]);
            bufs[1 - __ldcg(&X.bestbuf[sc])][k] = rk;
            const double ek = fb_error_2d(rk.x, rk.y, u0, u1, A.mu[k]);
            const double scale = fabs(va.x) + fabs(va.y) + fabs(vb.x) + fabs(vb.y) + fabs(ck.x) + fabs(ck.y) +
                                 fabs(rk.x) + fabs(rk.y);
            ve = f64_to_ordered(ek);
            vx = f64_to_ordered(ek - 64.0 * 1.1920929e-7 * scale);
            key = sc;
            ++nev;
          }
        }
        run_max_atomic(ve, key, eslots);
        run_max_atomic(vx, key, xslots);
      }
      if (!grid_sync(A.gb, A.spin)) {
        if (tid == 0) atomicExch(&A.st->status, (int)SG_DEVICE_TIMEOUT);
        return;
      }
      // Per-scene decisions (one thread per scene).
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
    const int sc = X.cscene[k];
    if (__ldcg(&X.done[sc])) continue;
    if (__ldcg(&X.best[sc]) < INFINITY) A.r[k] = __ldcg(&bufs[__ldcg(&X.bestbuf[sc])][k]);
  }
  for (int sc = tid; sc < S; sc += nthr)
    if (!__ldcg(&X.done[sc])) X.iters[sc] = A.max_iters;
  if (tid == 0) *X.unconverged += (unsigned long long)(S - *((volatile int*)X.done_count));
  atomicAdd(&M.work[0], n32);
  atomicAdd(&M.work[1], n64);
  atomicAdd(&M.work[2], nev);
  atomicAdd(&M.work[3], nlc);
  atomicAdd(&M.work[4], nlb);
  if (tid == 0) {
    A.st->iterations = it > A.max_iters ? A.max_iters : it;
    A.st->evals = n_eval;
  }
}

// ---------------------------------------------------------------------------
// Batched scenes, one scene per block.  A scene's bodies fit in a block's shared memory, so the
// block sweeps the scene's contacts colour by colour (the global colouring restricted to the scene:
// contacts ordered by (scene, colour)) with block barriers only, keeps the running velocities in
// shared memory, evaluates the scene's own residual, keeps its best iterate and stops at tol or
// max_iters.  Blocks take scenes from a largest-first work list.
//
// kMixed = false: FP64 sweeps, each scene seeing k_gs_batch's update sequence (the same results).
// kMixed = true (SG_PRECISION_FP32_REFINE): FP32 sweeps over colour-packed FP32 copies; on a
// doubling-then-adaptive schedule the FP32 iterate is lifted to FP64 (impulses, then velocities
// gathered from v0 and the impulses), its FP64 residual evaluated, and the scene turns to FP64
// sweeps once the residual reaches tol or the FP32 rounding floor (as k_gs_mixed_batch per scene).
constexpr int kSceneBlock = 256;

struct SceneBlockArgs {
  GsArgs g;                 // FP64 contacts, impulses (g.r), snapshot buffers g.r_a / g.r_b
  Gs32Args f;               // FP32 copies in (scene, colour) order (kMixed), v0, minv64, body adjacency
  const double2* v;         // running velocities at the start (warm start)
  const int* sb_off;        // S + 1 body offsets
  const int* sc_off;        // S + 1 contact offsets
  const int* nc_dev;        // contacts written this step (0 when the capacity overflowed: nothing is swept)
  const int* key_start;     // S * kMaxColors + 1: (scene, colour) runs of sperm
  const int* sperm;         // contacts by (scene, colour)
  const int* order;         // scenes, largest first
  int* next;                // work-list counter
  int S;
  int smax;                 // shared-memory body slots (the largest scene)
  double* best;
  int* done;
  unsigned* iters;
  unsigned long long* unconverged;
  unsigned long long* work;  // [0] FP32 updates, [1] FP64 updates, [2] evaluations, [3] contact lifts, [4] body lifts
};

// gs_update's arithmetic on shared-memory velocities (la, lb: the bodies' slots; lb < 0 for a plane).
__device__ __forceinline__ void gs_update_sv(const GsArgs& A, int k, int a, int b, int la, int lb, double2* sv) {
  const double2 nk = A.n[k], ck = A.c[k];
  const double2 va = sv[la];
  const bool has_b = lb >= 0;
  const double2 vb = has_b ? sv[lb] : make_double2(0.0, 0.0);
  double u0, u1;
  local_velocity(nk, ck, va, has_b, vb, u0, u1);
  const double2 rk = A.r[k];
  const double r0 = rk.x, r1 = rk.y;
  const double w00 = A.W[3 * k], w01 = A.W[3 * k + 1], w11 = A.W[3 * k + 2];
  const double bt0 = u0 - (w00 * r0 + w01 * r1);
  const double bt1 = u1 - (w01 * r0 + w11 * r1);
  double rn0, rn1;
  local_solve_2d(w00, w01, w11, bt0, bt1, A.mu[k], rn0, rn1);
  const double d0 = rn0 - r0, d1 = rn1 - r1;
  const double nx = nk.x, ny = nk.y, tx = -ny, ty = nx;
  const double px = nx * d0 + tx * d1;
  const double py = ny * d0 + ty * d1;
  const double ma = A.minv[a];
  sv[la] = make_double2(va.x + ma * px, va.y + ma * py);
  if (has_b) {
    const double mb = A.minv[b];
    sv[lb] = make_double2(vb.x - mb * px, vb.y - mb * py);
  }
  A.r[k] = make_double2(rn0, rn1);
}

// gs_update32's arithmetic on shared-memory FP32 velocities; q indexes the (scene, colour) packing.
__device__ __forceinline__ void gs_update32_sv(const Gs32Args& B, int q, int b0, float2* sv) {
  const int2 ab = B.ab[q];
  const float2 nk = B.n[q], ck = B.c[q];
  const float4 w = B.w[q];
  const int la = ab.x - b0;
  const bool has_b = ab.y >= 0;
  const int lb = has_b ? ab.y - b0 : -1;
  const float2 va = sv[la];
  const float2 vb = has_b ? sv[lb] : make_float2(0.0f, 0.0f);
  const float nx = nk.x, ny = nk.y, tx = -ny, ty = nx;
  float hn = nx * va.x + ny * va.y;
  float ht = tx * va.x + ty * va.y;
  if (has_b) {
    hn -= nx * vb.x + ny * vb.y;
    ht -= tx * vb.x + ty * vb.y;
  }
  const float u0 = hn + ck.x, u1 = ht + ck.y;
  const float2 rk = B.r[q];
  const float bt0 = u0 - (w.x * rk.x + w.y * rk.y);
  const float bt1 = u1 - (w.y * rk.x + w.z * rk.y);
  float rn0, rn1;
  local_solve_2d_f(w.x, w.y, w.z, bt0, bt1, w.w, rn0, rn1);
  const float d0 = rn0 - rk.x, d1 = rn1 - rk.y;
  const float px = nx * d0 + tx * d1, py = ny * d0 + ty * d1;
  const float ma = B.minv[ab.x];
  sv[la] = make_float2(va.x + ma * px, va.y + ma * py);
  if (has_b) {
    const float mb = B.minv[ab.y];
    sv[lb] = make_float2(vb.x - mb * px, vb.y - mb * py);
  }
  B.r[q] = make_float2(rn0, rn1);
}

// Block-wide nanmax of a (residual) and plain max of x (floor excess); every thread gets both.
__device__ __forceinline__ void block_max2(double& a, double& x, double* s_red) {
  for (int o = 16; o > 0; o >>= 1) {
    a = nanmax(a, __shfl_down_sync(0xffffffffu, a, o));
    x = fmax(x, __shfl_down_sync(0xffffffffu, x, o));
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if (lane == 0) {
    s_red[wid] = a;
    s_red[32 + wid] = x;
  }
  __syncthreads();
  if (wid == 0) {
    a = lane < nw ? s_red[lane] : 0.0;
    x = lane < nw ? s_red[32 + lane] : -INFINITY;
    for (int o = 16; o > 0; o >>= 1) {
      a = nanmax(a, __shfl_down_sync(0xffffffffu, a, o));
      x = fmax(x, __shfl_down_sync(0xffffffffu, x, o));
    }
    if (lane == 0) {
      s_red[64] = a;
      s_red[65] = x;
    }
  }
  __syncthreads();
  a = s_red[64];
  x = s_red[65];
  __syncthreads();
}

template <bool kMixed>
__global__ void __launch_bounds__(kSceneBlock) k_gs_scenes(SceneBlockArgs Z) {
  const GsArgs& A = Z.g;
  const Gs32Args& F = Z.f;
  extern __shared__ __align__(16) double2 sv64[];
  float2* sv32 = reinterpret_cast<float2*>(sv64 + Z.smax);
  __shared__ int s_w;
  __shared__ int s_off[kMaxColors + 1];
  __shared__ double s_red[66];
  if (*((volatile int*)&A.st->status) != 0) return;  // the colouring failed
  const unsigned eval64 = A.eval_every ? A.eval_every : 1u;
  const unsigned eval32 = F.eval32 ? F.eval32 : 1u;
  double2* bufs[2] = {A.r_a, A.r_b};
  unsigned long long n32 = 0, n64 = 0, nev = 0, nlc = 0, nlb = 0;
  // Scene offsets count every detected contact; after a capacity overflow none was written.
  const int ncv = *Z.nc_dev;
  for (;;) {
    if (threadIdx.x == 0) s_w = atomicAdd(Z.next, 1);
    __syncthreads();
    const int w = s_w;
    __syncthreads();
    if (w >= Z.S) break;
    const int sc = Z.order[w];
    const int b0 = Z.sb_off[sc], nbs = Z.sb_off[sc + 1] - b0;
    const int c0 = min(Z.sc_off[sc], ncv), c1 = min(Z.sc_off[sc + 1], ncv);
    if (c1 == c0) {
      if (threadIdx.x == 0) {
        Z.done[sc] = 1;
        Z.iters[sc] = 0;
        Z.best[sc] = INFINITY;
      }
      continue;
    }
    for (int j = threadIdx.x; j < nbs; j += blockDim.x) {
      const double2 vj = Z.v[b0 + j];
      sv64[j] = vj;
      if (kMixed) sv32[j] = make_float2((float)vj.x, (float)vj.y);
    }
    for (int c = threadIdx.x; c <= kMaxColors; c += blockDim.x)
      s_off[c] = c < kMaxColors ? Z.key_start[sc * kMaxColors + c] : Z.key_start[(sc + 1) * kMaxColors];
    __syncthreads();
    int ncol = kMaxColors;
    while (ncol > 0 && s_off[ncol] == s_off[ncol - 1]) --ncol;
    // Per-scene state, the same in every thread.
    double err_best = INFINITY;
    int bestbuf = 0;
    bool converged = false;
    int mode = kMixed ? 0 : 1;
    unsigned since = 0, next_eval = 1, interval = eval32;
    unsigned it;
    for (it = 1; it <= A.max_iters; ++it) {
      for (int col = 0; col < ncol; ++col) {
        const int e = s_off[col + 1];
        if (mode == 0) {
          for (int q = s_off[col] + threadIdx.x; q < e; q += blockDim.x) {
            gs_update32_sv(F, q, b0, sv32);
            ++n32;
          }
        } else {
          for (int q = s_off[col] + threadIdx.x; q < e; q += blockDim.x) {
            const int k = Z.sperm[q];
            const int a = A.ia[k], b = A.ib[k];
            gs_update_sv(A, k, a, b, a - b0, b >= 0 ? b - b0 : -1, sv64);
            ++n64;
          }
        }
        __syncthreads();
      }
      const bool due = mode == 0 ? (it == next_eval || it == A.max_iters)
                                 : (it % eval64 == 0 || (kMixed && it == A.max_iters));
      if (!due) continue;
      if (mode == 0) {
        // Lift: FP64 impulses from the FP32 ones, then each body's FP64 velocity from v0 and them.
        for (int q = s_off[0] + threadIdx.x; q < s_off[ncol]; q += blockDim.x) {
          const float2 r32 = F.r[q];
          A.r[Z.sperm[q]] = make_double2((double)r32.x, (double)r32.y);
          ++nlc;
        }
        __syncthreads();
        for (int j = threadIdx.x; j < nbs; j += blockDim.x) {
          const int i = b0 + j;
          double hx = 0.0, hy = 0.0;
          const int e = F.body_off[i + 1];
          for (int p = F.body_off[i]; p < e; ++p) {
            const int k = F.body_adj[p];
            const double sgn = (A.ia[k] == i) ? 1.0 : -1.0;
            const double2 nk = A.n[k], rk = A.r[k];
            const double px = nk.x * rk.x + (-nk.y) * rk.y;
            const double py = nk.y * rk.x + nk.x * rk.y;
            hx = hx + sgn * px;
            hy = hy + sgn * py;
          }
          const double2 a0 = F.v0[i];
          const double mi = F.minv64[i];
          const double2 vi = make_double2(a0.x + mi * hx, a0.y + mi * hy);
          sv64[j] = vi;
          sv32[j] = make_float2((float)vi.x, (float)vi.y);
          ++nlb;
        }
        __syncthreads();
      }
      // FP64 residual of the scene (and, in FP32 mode, its excess over the FP32 rounding floor).
      double emax = 0.0, xmax = -INFINITY;
      double2* cand = bufs[1 - bestbuf];
      for (int k = c0 + threadIdx.x; k < c1; k += blockDim.x) {
        const int a = A.ia[k], b = A.ib[k];
        const bool has_b = b >= 0;
        const double2 va = sv64[a - b0];
        const double2 vb = has_b ? sv64[b - b0] : make_double2(0.0, 0.0);
        const double2 ck = A.c[k];
        double u0, u1;
        local_velocity(A.n[k], ck, va, has_b, vb, u0, u1);
        const double2 rk = A.r[k];
        cand[k] = rk;
        const double ek = fb_error_2d(rk.x, rk.y, u0, u1, A.mu[k]);
        emax = nanmax(emax, ek);
        if (kMixed && mode == 0) {
          const double scale = fabs(va.x) + fabs(va.y) + fabs(vb.x) + fabs(vb.y) + fabs(ck.x) + fabs(ck.y) +
                               fabs(rk.x) + fabs(rk.y);
          xmax = fmax(xmax, ek - 64.0 * 1.1920929e-7 * scale);
        }
        ++nev;
      }
      block_max2(emax, xmax, s_red);
      const double err = emax;
      if (err < err_best) {
        err_best = err;
        bestbuf ^= 1;
        since = 0;
      } else {
        ++since;
      }
      if (mode == 1) {
        if (err < A.tol) {
          converged = true;
          break;
        }
      } else {
        if (err < A.tol || xmax <= A.tol || (since >= 16 && xmax <= 16.0 * A.tol)) {
          mode = 1;
        } else if (it < eval32) {
          next_eval = 2 * it;
        } else {
          interval = (err > 1e3 * A.tol) ? min(2u * interval, 16u * eval32) : (err > 10.0 * A.tol ? interval : eval32);
          next_eval = it + interval;
        }
      }
    }
    if (!converged) {
      if (err_best < INFINITY)
        for (int k = c0 + threadIdx.x; k < c1; k += blockDim.x) A.r[k] = bufs[bestbuf][k];
      it = A.max_iters;
    }
    if (threadIdx.x == 0) {
      Z.done[sc] = converged ? 1 : 0;
      Z.iters[sc] = it;
      Z.best[sc] = err_best;
      if (!converged) atomicAdd(Z.unconverged, 1ull);
      atomicMax(&A.st->iterations, it);
    }
    __syncthreads();
  }
  n32 = warp_sum(n32);
  n64 = warp_sum(n64);
  nev = warp_sum(nev);
  nlc = warp_sum(nlc);
  nlb = warp_sum(nlb);
  if ((threadIdx.x & 31) == 0) {
    if (n32) atomicAdd(&Z.work[0], n32);
    atomicAdd(&Z.work[1], n64);
    atomicAdd(&Z.work[2], nev);
    if (nlc) atomicAdd(&Z.work[3], nlc);
    if (nlb) atomicAdd(&Z.work[4], nlb);
  }
}

// (scene, colour) runs of a batch's contacts.
__global__ void k_scene_color_count(const int* __restrict__ nc_dev, const int* __restrict__ cscene,
                                    const int* __restrict__ color, int* __restrict__ cnt) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= *nc_dev) return;
  const int c = color[k];
  if (c < 0 || c >= kMaxColors) return;  // a failed colouring (its status ends the solve)
  atomicAdd(&cnt[cscene[k] * kMaxColors + c], 1);
}

__global__ void k_scene_color_scatter(const int* __restrict__ nc_dev, const int* __restrict__ cscene,
                                      const int* __restrict__ color, const int* __restrict__ start,
                                      int* __restrict__ fill, int* __restrict__ sperm) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= *nc_dev) return;
  const int c = color[k];
  if (c < 0 || c >= kMaxColors) return;
  const int key = cscene[k] * kMaxColors + c;
  sperm[start[key] + atomicAdd(&fill[key], 1)] = k;
}

// FP32 copies of the contacts in (scene, colour) order (position q holds contact sperm[q]).
__global__ void k_pack32_scenes(const int* __restrict__ n_dev, const int* __restrict__ sperm,
                                const int* __restrict__ ia, const int* __restrict__ ib,
                                const double2* __restrict__ n, const double2* __restrict__ c,
                                const double* __restrict__ W, const double* __restrict__ mu,
                                const double2* __restrict__ r, int2* __restrict__ ab, float2* __restrict__ n32,
                                float2* __restrict__ c32, float4* __restrict__ w32, float2* __restrict__ r32) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= *n_dev) return;
  const int k = sperm[q];
  const int b = ib[k];
  ab[q] = make_int2(ia[k], b >= 0 ? b : -1);
  const double2 nk = n[k], ck = c[k], rk = r[k];
  n32[q] = make_float2((float)nk.x, (float)nk.y);
  c32[q] = make_float2((float)ck.x, (float)ck.y);
  w32[q] = make_float4((float)W[3 * k], (float)W[3 * k + 1], (float)W[3 * k + 2], (float)mu[k]);
  r32[q] = make_float2((float)rk.x, (float)rk.y);
}

__global__ void k_wait_flag(const int* flag, int* status, unsigned long long spin) {
  volatile const int* f = flag;
  unsigned long long n = 0;
  while (*f == 0) {
    if (++n > spin) {
      *status = SG_DEVICE_TIMEOUT;
      return;
    }
    __nanosleep(32);
  }
  *status = SG_OK;
}

}  // namespace

int ensure_solver_capacity(sg_ctx* ctx, int nb, int nc) {
  const size_t ncs = (size_t)std::max(nc, 1), nbs = (size_t)std::max(nb, 1);
  if (int r = grow(ctx->color, sizeof(int) * ncs)) return r;
  if (int r = grow(ctx->perm, sizeof(int) * ncs)) return r;
  if (int r = grow(ctx->body_cnt, sizeof(int) * (nbs + 1))) return r;
  if (int r = grow(ctx->body_off, sizeof(int) * (nbs + 1))) return r;
  if (int r = grow(ctx->body_fill, sizeof(int) * (nbs + 1))) return r;
  if (int r = grow(ctx->body_adj, sizeof(int) * 2 * ncs)) return r;
  if (int r = grow(ctx->v_run, sizeof(double) * 2 * nbs)) return r;
  if (int r = grow(ctx->r_cand, sizeof(double) * 2 * ncs)) return r;
  if (int r = grow(ctx->r_best, sizeof(double) * 2 * ncs)) return r;
  if (int r = grow(ctx->stats, sizeof(SolveStats))) return r;
  if (int r = grow(ctx->barrier, sizeof(GridBarrier))) return r;
  return SG_OK;
}

int prepare_contact_graph(sg_ctx* ctx, int nb, int nc, const int* ia, const int* ib, const int* nc_dev,
                          const int* warm_color) {
  cudaStream_t s = ctx->stream;
  int* cnt = ctx->body_cnt.as<int>();
  int* off = ctx->body_off.as<int>();
  int* fill = ctx->body_fill.as<int>();
  int* adj = ctx->body_adj.as<int>();
  SolveStats* st = ctx->stats.as<SolveStats>();
  GridBarrier* gb = ctx->barrier.as<GridBarrier>();
  SG_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int) * (size_t)(nb + 1), s));
  SG_CUDA_TRY(cudaMemsetAsync(fill, 0, sizeof(int) * (size_t)(nb + 1), s));
  SG_CUDA_TRY(cudaMemsetAsync(st, 0, sizeof(SolveStats), s));
  if (nc > 0) {
    k_body_count<<<blocks_for(nc), kBlock, 0, s>>>(nc, nc_dev, ia, ib, cnt);
    SG_CUDA_TRY(cudaGetLastError());
  }
  if (int r = scan_exclusive(ctx, cnt, off, nb)) return r;
  ctx->kernel_launches += nb > 0 ? 3 : 0;
  if (nc == 0) return SG_OK;
  k_body_fill<<<blocks_for(nc), kBlock, 0, s>>>(nc, nc_dev, ia, ib, off, fill, adj);
  k_body_sort<<<blocks_for(nb), kBlock, 0, s>>>(nb, off, adj);
  SG_CUDA_TRY(cudaGetLastError());
  if (warm_color)
    SG_CUDA_TRY(cudaMemcpyAsync(ctx->color.p, warm_color, sizeof(int) * (size_t)nc, cudaMemcpyDeviceToDevice, s));
  else
    SG_CUDA_TRY(cudaMemsetAsync(ctx->color.p, 0xff, sizeof(int) * (size_t)nc, s));
  SG_CUDA_TRY(cudaMemsetAsync(gb, 0, sizeof(GridBarrier), s));
  ColorArgs CA{nc, nc_dev, ia, ib, off, adj, ctx->color.as<int>(), ctx->perm.as<int>(), st, gb, ctx->spin_limit,
               4096};
  if (warm_color) {
    // The carried colours need no Jones-Plassmann round; one recolouring pass keeps the count
    // from creeping up as new contacts take the first free colour.
    CA.first_round = 1;
    CA.ig_passes = 1;
  }
  void* args[] = {&CA};
  // One 1,024-thread block per SM: the colouring is a chain of grid barriers (a Jones-Plassmann
  // round each, a colour class each in the recolouring passes), and a barrier's cost grows with the
  // blocks arriving at it.
  const int g = coop_grid(ctx, k_color_jp, nc, kColorBlock, 1);
  SG_CUDA_TRY(launch_cooperative((const void*)k_color_jp, g, kColorBlock, args, s));
  ctx->kernel_launches += 4;  // body_count, body_fill, body_sort, colouring
  return SG_OK;
}

int solve_contacts(sg_ctx* ctx, const ContactProblem& P, const SolveParams& sp) {
  const int nb = P.nb, nc = P.nc;
  cudaStream_t s = ctx->stream;
  if (int r = ensure_solver_capacity(ctx, nb, nc)) return r;
  int* off = ctx->body_off.as<int>();
  int* adj = ctx->body_adj.as<int>();
  SolveStats* st = ctx->stats.as<SolveStats>();
  GridBarrier* gb = ctx->barrier.as<GridBarrier>();
  bool patched_run = false;
  const double2* n2 = reinterpret_cast<const double2*>(P.n);
  double2* r2 = reinterpret_cast<double2*>(P.r);

  // Adjacency and colouring first: the velocity initialisation reads the adjacency.
  if (int r = prepare_contact_graph(ctx, nb, nc, P.ia, P.ib, nullptr, P.warm_color)) return r;
  stage_mark(ctx, 4);
  double2* vrun = ctx->v_run.as<double2>();
  if (sp.learned && nc > 0 && (ctx->mlp_on || ctx->mlp_record)) {
    if (int r = mlp_features(ctx, P)) return r;
    if (ctx->mlp_on) {
      // Network start into the (not yet used) candidate buffer; the start with the smaller
      // FP64 residual goes to the solve.
      double2* r_alt = ctx->r_cand.as<double2>();
      if (int r = mlp_predict(ctx, P, reinterpret_cast<double*>(r_alt))) return r;
      if (int r = grow(ctx->mlp_slots, 2 * sizeof(unsigned long long))) return r;
      if (!ctx->mlp_choice.p) {
        if (int r = grow(ctx->mlp_choice, sizeof(unsigned long long))) return r;
        SG_CUDA_TRY(cudaMemsetAsync(ctx->mlp_choice.p, 0, sizeof(unsigned long long), s));
      }
      unsigned long long* slots = ctx->mlp_slots.as<unsigned long long>();
      SG_CUDA_TRY(cudaMemsetAsync(slots, 0, 2 * sizeof(unsigned long long), s));
      const int eb = std::max(1, std::min(blocks_for(nc), ctx->num_sms * 8));
      const double2* starts[2] = {r2, r_alt};
      for (int w = 0; w < 2; ++w) {
        k_vel_init<<<blocks_for(nb), kBlock, 0, s>>>(nb, off, adj, P.ia, n2, starts[w],
                                                     reinterpret_cast<const double2*>(P.v0), P.minv, vrun);
        k_start_err<<<eb, kBlock, 0, s>>>(nc, P.ia, P.ib, n2, reinterpret_cast<const double2*>(P.c), P.mu, starts[w],
                                          vrun, slots + w);
      }
      k_select_start<<<blocks_for(nc), kBlock, 0, s>>>(nc, r2, r_alt, slots, ctx->mlp_choice.as<unsigned long long>());
      SG_CUDA_TRY(cudaGetLastError());
      ctx->mlp_evals += 1;
      ctx->kernel_launches += 5;
    }
  }
  k_vel_init<<<blocks_for(nb), kBlock, 0, s>>>(nb, off, adj, P.ia, n2, r2, reinterpret_cast<const double2*>(P.v0),
                                               P.minv, vrun);
  SG_CUDA_TRY(cudaGetLastError());

  // FP32 form: a probe of up to kFp64Probe one-level FP64 sweeps first (isotropic closed form; a
  // warm start on a settled scene converges within them, for less than the two-level partition's
  // setup costs).  If it has not converged, its residual decides the arithmetic: within
  // fp64_factor tol of the tolerance the solve goes on in FP64 (on the two-level partition for a
  // large scene), because FP32 sweeps would only add their rounding, whose floor lies near tol
  // where the impulses of deep stacks reach hundreds of times the velocity scale; further away,
  // FP32 sweeps with FP64 checks and refinement.
  const bool fp32_form = sp.precision == SG_PRECISION_FP32_REFINE;
  bool fp64_start = false;
  bool fp32_sweeps = fp32_form;
  unsigned probe_iters = 0, probe_evals = 0;

  if (nc > 0) {
    // Gauss-Seidel.
    SG_CUDA_TRY(cudaMemsetAsync(gb, 0, sizeof(GridBarrier), s));
    GsArgs GA;
    GA.nc = nc;
    GA.ia = P.ia;
    GA.ib = P.ib;
    GA.n = n2;
    GA.c = reinterpret_cast<const double2*>(P.c);
    GA.W = P.W;
    GA.mu = P.mu;
    GA.minv = P.minv;
    GA.perm = ctx->perm.as<int>();
    GA.r = r2;
    GA.r_a = ctx->r_cand.as<double2>();
    GA.r_b = ctx->r_best.as<double2>();
    GA.v = vrun;
    GA.st = st;
    GA.gb = gb;
    GA.spin = ctx->spin_limit;
    GA.tol = sp.tol;
    GA.max_iters = sp.max_iters;
    GA.eval_every = sp.eval_every;
    GA.iso = fp32_form ? 1 : 0;
    if (fp32_form && ctx->fp64_factor > 0) {  // fp64_factor 0: FP32 sweeps from the start
      GsArgs GP = GA;
      const bool probe = sp.max_iters > kFp64Probe;
      if (probe) GP.max_iters = kFp64Probe;
      // A warm start rarely converges in one sweep, and a residual check costs about three FP64
      // sweeps on GB300: the first check follows the second sweep, and after the fourth every
      // second sweep is checked.
      GP.first_eval = GP.max_iters >= 2 ? 2u : 1u;
      GP.eval_stride = 2;
      void* pargs[] = {&GP};
      const int g = coop_grid(ctx, k_gs, nc, kGsBlock, 1);
      stage_mark(ctx, 5);
      if (ctx->profile) SG_CUDA_TRY(cudaEventRecord(ctx->ev_gs0, s));
      SG_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_gs, dim3(g), dim3(kGsBlock), pargs, 0, s));
      if (ctx->profile) SG_CUDA_TRY(cudaEventRecord(ctx->ev_gs1, s));
      stage_mark(ctx, 6);
      ctx->kernel_launches += 1;
      fp32_sweeps = false;
      if (probe) {
        SolveStats hp{};
        SG_CUDA_TRY(cudaMemcpyAsync(&hp, st, sizeof(SolveStats), cudaMemcpyDeviceToHost, s));
        SG_CUDA_TRY(cudaStreamSynchronize(s));
        if (hp.converged) ctx->fp64_start_solves += 1;
        if (!hp.converged && hp.status == 0) {
          // Not converged in the probe: on from its best iterate, within the remaining sweeps, in
          // FP64 or in the FP32 form as its residual says; the residual slots start afresh.
          fp64_start = hp.error < (double)ctx->fp64_factor * sp.tol;
          if (fp64_start) ctx->fp64_start_solves += 1;
          if (ctx->profile) {
            float ms = 0.f;
            SG_CUDA_TRY(cudaEventElapsedTime(&ms, ctx->ev_gs0, ctx->ev_gs1));
            ctx->gs_ms += ms;
          }
          probe_iters = hp.iterations;
          probe_evals = hp.evals;
          k_vel_init<<<blocks_for(nb), kBlock, 0, s>>>(nb, off, adj, P.ia, n2, r2,
                                                       reinterpret_cast<const double2*>(P.v0), P.minv, vrun);
          SG_CUDA_TRY(cudaGetLastError());
          SG_CUDA_TRY(cudaMemsetAsync(st->err_slot, 0, sizeof(st->err_slot), s));
          SG_CUDA_TRY(cudaMemsetAsync(st->mag_slot, 0, sizeof(st->mag_slot), s));
          SG_CUDA_TRY(cudaMemsetAsync(gb, 0, sizeof(GridBarrier), s));
          GA.max_iters = sp.max_iters - probe_iters;
          fp32_sweeps = true;
          ctx->kernel_launches += 1;
        }
      }
    }
    if (fp32_sweeps) {
      // A solve the probe leaves near tol under two_level 1: up to kOneLevel64 one-level FP64
      // sweeps first, then, unconverged, the two-level partition for the rest.  Near tol the
      // two-level order, which sweeps the contacts between patches after the patches, can hold
      // the residual on a plateau just above tol for hundreds of sweeps that the colour order
      // crosses in tens; a solve that needs thousands of sweeps either way gets the two-level
      // sweeps' lower cost for all but the first kOneLevel64.
      const bool eligible = sp.learned && ctx->patches && ctx->dim == 2 && ctx->n_scenes == 0 &&
                            nc >= ctx->two_level_min_contacts;
      bool second_pass = false;
      for (int pass = 0;; ++pass) {
        const bool one_level = pass == 0 && fp64_start && ctx->patches == 1;
        const bool one_level_first = one_level && eligible && GA.max_iters > kOneLevel64;
        const unsigned remaining = GA.max_iters;
        if (one_level_first) GA.max_iters = kOneLevel64;
        const size_t c = (size_t)nc, b = (size_t)std::max(nb, 1);
        if (int r = grow(ctx->pk_ab, sizeof(int2) * c)) return r;
        if (int r = grow(ctx->pk_n, sizeof(float2) * c)) return r;
        if (int r = grow(ctx->pk_c, sizeof(float2) * c)) return r;
        if (int r = grow(ctx->pk_w, sizeof(float4) * c)) return r;
        if (int r = grow(ctx->pk_r, sizeof(float2) * c)) return r;
        if (int r = grow(ctx->v32, sizeof(float2) * b)) return r;
        if (int r = grow(ctx->minv32, sizeof(float) * b)) return r;
        // Two-level sweeps for large scene steps (the broad phase's grid gives the patches).
        int pmax = 0;
        const int maxP = ctx->num_sms;
        const bool try_patches = eligible && !one_level;
        int pmaxq = 0, cmax_p = 0, cmax_q = 0, nrest = 0, nrest_bodies = 0;
        PatchSetup hps{};
        if (try_patches) {
          // Groups: at most maxP patches, maxP shifted tiles and the remainder (a degenerate
          // setup is rejected below before any launch uses it).
          const int groups = 2 * maxP + 8;
          const size_t keys = (size_t)groups * kMaxColors + 1;
          const size_t gsz = sizeof(int) * (size_t)(groups + 1);
          if (int r = grow(ctx->pt_setup, sizeof(PatchSetup))) return r;
          if (int r = grow(ctx->pt_patch, sizeof(int) * b)) return r;
          if (int r = grow(ctx->pt_qpatch, sizeof(int) * b)) return r;
          if (int r = grow(ctx->pt_band, sizeof(int) * b)) return r;
          if (int r = grow(ctx->pt_lidx, sizeof(int) * b)) return r;
          if (int r = grow(ctx->pt_lidxq, sizeof(int) * b)) return r;
          if (int r = grow(ctx->pt_body, sizeof(int) * b)) return r;
          if (int r = grow(ctx->pt_qbody, sizeof(int) * b)) return r;
          if (int r = grow(ctx->pt_cnt, gsz)) return r;
          if (int r = grow(ctx->pt_start, gsz)) return r;
          if (int r = grow(ctx->pt_fill, gsz)) return r;
          if (int r = grow(ctx->pt_bcnt, gsz)) return r;
          if (int r = grow(ctx->pt_nfill, gsz)) return r;
          if (int r = grow(ctx->pt_qcnt, gsz)) return r;
          if (int r = grow(ctx->pt_qstart, gsz)) return r;
          if (int r = grow(ctx->pt_qfill, gsz)) return r;
          if (int r = grow(ctx->pt_key, sizeof(int) * c)) return r;
          if (int r = grow(ctx->pt_kcnt, sizeof(int) * keys)) return r;
          if (int r = grow(ctx->pt_kstart, sizeof(int) * keys)) return r;
          if (int r = grow(ctx->pt_kfill, sizeof(int) * keys)) return r;
          if (int r = grow(ctx->pt_order, sizeof(int) * c)) return r;
          if (int r = grow(ctx->pt_max, 7 * sizeof(int))) return r;
          // Cell columns and rows number at most the broad phase's cell capacity (4 nb + 64).
          const size_t gcap = 4 * (size_t)nb + 64;
          if (int r = grow(ctx->pt_hist, 2 * sizeof(int) * gcap)) return r;
          if (int r = grow(ctx->pt_pref, 2 * sizeof(int) * (gcap + 1))) return r;
          if (int r = grow(ctx->pt_cuts, 2 * sizeof(int) * (size_t)(maxP + 2))) return r;
          if (int r = grow(ctx->pt_maps, 4 * sizeof(int) * gcap)) return r;
          if (int r = grow(ctx->pt_cflag, sizeof(int) * b)) return r;
          if (int r = grow(ctx->pt_cpos, sizeof(int) * (b + 1))) return r;
          if (int r = grow(ctx->pt_cbody, sizeof(int) * b)) return r;
          if (int r = grow(ctx->pt_bcolor, sizeof(int) * c)) return r;
          if (int r = grow(ctx->pt_rem, 4 * sizeof(int))) return r;
          PatchSetup* ps = ctx->pt_setup.as<PatchSetup>();
          k_patch_setup<<<1, 1, 0, s>>>(ctx->grid.as<GridParams>(), maxP, ps);
          for (Buf* z : {&ctx->pt_cnt, &ctx->pt_fill, &ctx->pt_bcnt, &ctx->pt_nfill, &ctx->pt_qcnt, &ctx->pt_qfill})
            SG_CUDA_TRY(cudaMemsetAsync(z->p, 0, gsz, s));
          SG_CUDA_TRY(cudaMemsetAsync(ctx->pt_kcnt.p, 0, sizeof(int) * keys, s));
          SG_CUDA_TRY(cudaMemsetAsync(ctx->pt_kfill.p, 0, sizeof(int) * keys, s));
          SG_CUDA_TRY(cudaMemsetAsync(ctx->pt_max.p, 0, 7 * sizeof(int), s));
          SG_CUDA_TRY(cudaMemsetAsync(ctx->pt_cflag.p, 0, sizeof(int) * b, s));
          SG_CUDA_TRY(cudaMemsetAsync(ctx->pt_band.p, 0, sizeof(int) * b, s));
          {
            int* hx = ctx->pt_hist.as<int>();
            int* hy = hx + gcap;
            int* px = ctx->pt_pref.as<int>();
            int* py = px + gcap + 1;
            int* cx = ctx->pt_cuts.as<int>();
            int* cy = cx + maxP + 2;
            int* maps = ctx->pt_maps.as<int>();
            SG_CUDA_TRY(cudaMemsetAsync(hx, 0, 2 * sizeof(int) * gcap, s));
            k_patch_hist<<<blocks_for((long)nc + nb), kBlock, 0, s>>>(nc, nb, P.ia, ctx->cell_of.as<int>(), ps, hx, hy);
            SG_CUDA_TRY(cudaGetLastError());
            if (int r = scan_exclusive(ctx, hx, px, (int)gcap)) return r;
            if (int r = scan_exclusive(ctx, hy, py, (int)gcap)) return r;
            k_patch_cuts<<<1, kBlock, 0, s>>>(ps, px, py, cx, cy);
            k_patch_maps<<<blocks_for((long)gcap), kBlock, 0, s>>>(ps, cx, cy, maps, maps + gcap, maps + 2 * gcap,
                                                                 maps + 3 * gcap);
            k_patch_of_body<<<blocks_for(nb), kBlock, 0, s>>>(nb, ctx->cell_of.as<int>(), ps, maps, maps + gcap,
                                                             maps + 2 * gcap, maps + 3 * gcap, ctx->pt_patch.as<int>(),
                                                             ctx->pt_qpatch.as<int>(), ctx->pt_cnt.as<int>());
          }
          SG_CUDA_TRY(cudaGetLastError());
          int* cpatch = ctx->pt_order.as<int>();  // scratch until the order is built
          int* bcolor = ctx->pt_bcolor.as<int>();
          k_contact_side<<<blocks_for(nc), kBlock, 0, s>>>(nc, P.ia, P.ib, ctx->pt_patch.as<int>(),
                                                           ctx->pt_qpatch.as<int>(), ps, cpatch, bcolor,
                                                           ctx->pt_band.as<int>());
          k_rest_mark<<<blocks_for(nc), kBlock, 0, s>>>(nc, P.ia, P.ib, cpatch, ps, ctx->pt_cflag.as<int>());
          SG_CUDA_TRY(cudaGetLastError());
          if (int r = scan_exclusive(ctx, ctx->pt_cflag.as<int>(), ctx->pt_cpos.as<int>(), nb)) return r;
          k_rest_scatter<<<blocks_for(nb), kBlock, 0, s>>>(nb, ctx->pt_cflag.as<int>(), ctx->pt_cpos.as<int>(),
                                                          ctx->pt_cbody.as<int>());
          SG_CUDA_TRY(cudaMemcpyAsync(ctx->pt_max.as<int>() + 6, ctx->pt_cpos.as<int>() + nb, sizeof(int),
                                      cudaMemcpyDeviceToDevice, s));
          k_band_count<<<blocks_for(nb), kBlock, 0, s>>>(nb, ctx->pt_band.as<int>(), ctx->pt_patch.as<int>(),
                                                         ctx->pt_qpatch.as<int>(), ctx->pt_bcnt.as<int>(),
                                                         ctx->pt_qcnt.as<int>());
          SG_CUDA_TRY(cudaGetLastError());
          if (int r = scan_exclusive(ctx, ctx->pt_cnt.as<int>(), ctx->pt_start.as<int>(), groups)) return r;
          if (int r = scan_exclusive(ctx, ctx->pt_qcnt.as<int>(), ctx->pt_qstart.as<int>(), groups)) return r;
          k_patch_scatter<<<blocks_for(nb), kBlock, 0, s>>>(
              nb, ctx->pt_patch.as<int>(), ctx->pt_qpatch.as<int>(), ctx->pt_band.as<int>(), ctx->pt_start.as<int>(),
              ctx->pt_bcnt.as<int>(), ctx->pt_fill.as<int>(), ctx->pt_nfill.as<int>(), ctx->pt_body.as<int>(),
              ctx->pt_lidx.as<int>(), ctx->pt_qstart.as<int>(), ctx->pt_qfill.as<int>(), ctx->pt_qbody.as<int>(),
              ctx->pt_lidxq.as<int>());
          k_patch_max<<<1, kBlock, 0, s>>>(groups, ctx->pt_cnt.as<int>(), ctx->pt_max.as<int>());
          k_patch_max<<<1, kBlock, 0, s>>>(groups, ctx->pt_qcnt.as<int>(), ctx->pt_max.as<int>() + 1);
          SG_CUDA_TRY(cudaGetLastError());
          SG_CUDA_TRY(cudaMemsetAsync(gb, 0, sizeof(GridBarrier), s));
          SG_CUDA_TRY(cudaMemsetAsync(ctx->pt_rem.p, 0, 4 * sizeof(int), s));
          {
            BColorArgs BA{nc, P.ia, P.ib, off, adj, cpatch, ps, bcolor, ctx->pt_rem.as<int>(), &st->status, gb,
                          ctx->spin_limit, 4096};
            void* bargs[] = {&BA};
            const int g = coop_grid(ctx, k_color_boundary, nc, kBlock);
            SG_CUDA_TRY(launch_cooperative((const void*)k_color_boundary, g, kBlock, bargs, s));
          }
          k_group_color_init<<<blocks_for(nc), kBlock, 0, s>>>(nc, ctx->color.as<int>(), cpatch, ps, bcolor,
                                                              ctx->pt_max.as<int>() + 2);
          SG_CUDA_TRY(cudaGetLastError());
          SG_CUDA_TRY(cudaMemsetAsync(gb, 0, sizeof(GridBarrier), s));
          {
            RecolorArgs RA{nc, P.ia, P.ib, off, adj, cpatch, bcolor, ctx->pt_max.as<int>() + 2, &st->status, gb,
                           ctx->spin_limit};
            void* rargs[] = {&RA};
            const int g = coop_grid(ctx, k_recolor_groups, nc, kBlock);
            SG_CUDA_TRY(launch_cooperative((const void*)k_recolor_groups, g, kBlock, rargs, s));
          }
          k_contact_key<<<blocks_for(nc), kBlock, 0, s>>>(nc, bcolor, cpatch, ctx->pt_key.as<int>(),
                                                         ctx->pt_kcnt.as<int>());
          SG_CUDA_TRY(cudaGetLastError());
          if (int r = scan_exclusive(ctx, ctx->pt_kcnt.as<int>(), ctx->pt_kstart.as<int>(), (int)(keys - 1))) return r;
          k_contact_scatter<<<blocks_for(nc), kBlock, 0, s>>>(nc, ctx->pt_key.as<int>(), ctx->pt_kstart.as<int>(),
                                                             ctx->pt_kfill.as<int>(), ctx->pt_order.as<int>());
          k_group_max<<<1, kBlock, 0, s>>>(ps, ctx->pt_kstart.as<int>(), ctx->pt_max.as<int>() + 3);
          SG_CUDA_TRY(cudaGetLastError());
          int hmax[7] = {0, 0, 0, 0, 0, 0, 0};
          SG_CUDA_TRY(cudaMemcpyAsync(hmax, ctx->pt_max.p, 7 * sizeof(int), cudaMemcpyDeviceToHost, s));
          SG_CUDA_TRY(cudaMemcpyAsync(&hps, ps, sizeof(PatchSetup), cudaMemcpyDeviceToHost, s));
          SG_CUDA_TRY(cudaStreamSynchronize(s));
          pmax = hmax[0];
          pmaxq = hmax[1];
          cmax_p = hmax[3];
          cmax_q = hmax[4];
          nrest = hmax[5];
          nrest_bodies = hmax[6];
          // setup, hist, 2 x 3 scan, cuts, maps, of_body, side, rest mark, 3 scan, rest scatter,
          // band_count, 2 x 3 scan, scatter, 2 max, colour, colour init, recolour, key, 3 scan,
          // scatter, group max
          ctx->kernel_launches += 36;
        }
        // Shared-memory slots rounded up to even counts (8-byte alignment of the second block).
        const int capp = (pmax + 1) & ~1, capq = (pmaxq + 1) & ~1;
        // Body slots must fit in shared memory beside the kernel's static arrays (12 B each).
        const bool patched = try_patches && hps.P >= 2 && hps.Pb <= maxP && pmax > 0 &&
                             capp + capq <= kPatchBodyCap;
        patched_run = patched;
        ctx->last_patched = patched;
        if (patched) {
          ctx->last_patch_P = hps.P;
          ctx->last_patch_Pb = hps.Pb;
        }
        if (patched)
          k_pack32_patch<<<blocks_for(nc), kBlock, 0, s>>>(nc, ctx->pt_order.as<int>(), ctx->pt_key.as<int>(),
                                                           ctx->pt_setup.as<PatchSetup>(), P.ia, P.ib,
                                                           ctx->pt_lidx.as<int>(), ctx->pt_lidxq.as<int>(), n2, reinterpret_cast<const double2*>(P.c),
                                                           P.W, P.mu, r2, ctx->pk_ab.as<int2>(), ctx->pk_n.as<float2>(),
                                                           ctx->pk_c.as<float2>(), ctx->pk_w.as<float4>(),
                                                           ctx->pk_r.as<float2>());
        else
          k_pack32<<<blocks_for(nc), kBlock, 0, s>>>(nc, ctx->perm.as<int>(), P.ia, P.ib, n2,
                                                     reinterpret_cast<const double2*>(P.c), P.W, P.mu, r2,
                                                     ctx->pk_ab.as<int2>(), ctx->pk_n.as<float2>(), ctx->pk_c.as<float2>(),
                                                     ctx->pk_w.as<float4>(), ctx->pk_r.as<float2>());
        k_vel32<<<blocks_for(nb), kBlock, 0, s>>>(nb, vrun, P.minv, ctx->v32.as<float2>(), ctx->minv32.as<float>());
        SG_CUDA_TRY(cudaGetLastError());
        Gs32Args GB;
        GB.ab = ctx->pk_ab.as<int2>();
        GB.n = ctx->pk_n.as<float2>();
        GB.c = ctx->pk_c.as<float2>();
        GB.w = ctx->pk_w.as<float4>();
        GB.r = ctx->pk_r.as<float2>();
        GB.v = ctx->v32.as<float2>();
        GB.minv = ctx->minv32.as<float>();
        GB.minv64 = P.minv;
        GB.v0 = reinterpret_cast<const double2*>(P.v0);
        GB.body_off = off;
        GB.body_adj = adj;
        GB.nb = nb;
        GB.eval32 = (unsigned)ctx->check_interval;
        GB.fp64_below = (double)ctx->fp64_factor * sp.tol;
        GB.fp64_start = fp64_start ? 1 : 0;
        if (patched) {
          // Dynamic shared memory: the body slots, then as many of the patch's and the tile's
          // contacts as fit (the patch's first), 32 B each.
          if (ctx->patch_smem_budget < 0) {
            int optin = 0;
            SG_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
            cudaFuncAttributes fa{};
            SG_CUDA_TRY(cudaFuncGetAttributes(&fa, k_gs_patch));
            const int budget = optin - (int)fa.sharedSizeBytes;
            SG_CUDA_TRY(cudaFuncSetAttribute(k_gs_patch, cudaFuncAttributeMaxDynamicSharedMemorySize, budget));
            ctx->patch_smem_budget = budget;
          }
          const int dyn_budget = ctx->patch_smem_budget;
          const int body_bytes = 12 * (capp + capq);
          // The remainder first (block 0 sweeps it whole or not at all), then the patch, the tile.
          int capc = (nrest_bodies + 1) & ~1, stage_c = nrest;
          int rest_bytes = 12 * capc + 32 * stage_c;
          if (nrest == 0 || nrest_bodies > kPatchBodyCap || rest_bytes > dyn_budget - body_bytes) {
            capc = stage_c = rest_bytes = 0;
          }
          const int avail = std::max(0, dyn_budget - body_bytes - rest_bytes) / 32;
          const int stage_p = std::min(cmax_p, avail);
          const int stage_q = std::min(cmax_q, avail - stage_p);
          PatchArgs Q{ctx->pt_setup.as<PatchSetup>(), ctx->pt_start.as<int>(), ctx->pt_body.as<int>(),
                      ctx->pt_bcnt.as<int>(), ctx->pt_qstart.as<int>(), ctx->pt_qbody.as<int>(),
                      ctx->pt_kstart.as<int>(), ctx->pt_order.as<int>(), capp, capq, stage_p, stage_q,
                      ctx->pt_cbody.as<int>(), ctx->pt_cpos.as<int>(), capc, capc ? nrest_bodies : 0, stage_c, 0};
          size_t smem = (size_t)body_bytes + (size_t)32 * (size_t)(stage_p + stage_q) + (size_t)rest_bytes;
          // The FP64 sweeps reuse the same shared memory for the patch's and the tile's FP64
          // velocities and inverse masses (24 B per body) when they fit.
          size_t smem64 = (size_t)24 * (size_t)(capp + capq);
          GB.fp64_local = smem64 <= (size_t)dyn_budget ? 1 : 0;
          if (GB.fp64_local && smem64 > smem) smem = smem64;
          // k_gs_patch64 also holds the remainder in block 0 (24 B per body, 4 B per contact) when
          // that fits beside the patch and the tile.
          const size_t rest64_bytes = (size_t)24 * (size_t)((nrest_bodies + 1) & ~1) + (size_t)4 * (size_t)nrest;
          if (GB.fp64_local && nrest > 0 && nrest_bodies <= kPatchBodyCap &&
              smem64 + rest64_bytes <= (size_t)dyn_budget) {
            Q.rest64 = nrest_bodies;
            smem64 += rest64_bytes;
          }
          ctx->patch_staged += (uint64_t)stage_p;
          // A solve that stays in FP64 takes the FP64 kernel (its velocities fit shared memory): for
          // Ball2D discs the float-float one (k_gs_patch_ff), unless sg_set_fp64_pairs turned it off.
          const bool only64 = fp64_start && GB.fp64_local;
          const bool pairs = only64 && !ctx->rb2d && ctx->fp64_pairs;
          FfArgs FA{};
          if (pairs) {
            const size_t c4 = sizeof(float4) * (size_t)nc, b = (size_t)std::max(nb, 1);
            if (int r = grow(ctx->ff_n, c4)) return r;
            if (int r = grow(ctx->ff_c, c4)) return r;
            if (int r = grow(ctx->ff_m, c4)) return r;
            if (int r = grow(ctx->ff_r, c4)) return r;
            if (int r = grow(ctx->ff_v, sizeof(float4) * b)) return r;
            if (int r = grow(ctx->ff_minv, sizeof(float2) * b)) return r;
            FA = FfArgs{ctx->ff_n.as<float4>(), ctx->ff_c.as<float4>(), ctx->ff_m.as<float4>(),
                        ctx->ff_r.as<float4>(), ctx->ff_v.as<float4>(), ctx->ff_minv.as<float2>()};
            k_pack_ff<<<blocks_for(std::max(nc, nb)), kBlock, 0, s>>>(nc, nb, Q.order, n2, GA.c, GA.W, GA.mu, r2, vrun,
                                                                     P.minv, FA);
            SG_CUDA_TRY(cudaGetLastError());
            ctx->kernel_launches += 1;
          }
          void* args[] = {&GA, &GB, &Q, &FA};
          // The boundary colouring used the barrier: start it afresh for this grid.
          SG_CUDA_TRY(cudaMemsetAsync(gb, 0, sizeof(GridBarrier), s));
          if (!second_pass) stage_mark(ctx, 5);
          if (ctx->profile) SG_CUDA_TRY(cudaEventRecord(ctx->ev_gs0, s));
          if (only64 && !ctx->patch64_ready) {
            SG_CUDA_TRY(cudaFuncSetAttribute(k_gs_patch64, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_budget));
            SG_CUDA_TRY(cudaFuncSetAttribute(k_gs_patch_ff, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_budget));
            ctx->patch64_ready = true;
          }
          cudaLaunchConfig_t lc = {};
          lc.gridDim = dim3(maxP);
          lc.blockDim = dim3(only64 ? kPatch64Block : kPatchBlock);
          lc.dynamicSmemBytes = only64 ? smem64 : smem;
          lc.stream = s;
          cudaLaunchAttribute at[1];
          at[0].id = cudaLaunchAttributeCooperative;
          at[0].val.cooperative = 1;
          lc.attrs = at;
          lc.numAttrs = 1;
          const void* kfn = pairs ? (const void*)k_gs_patch_ff : only64 ? (const void*)k_gs_patch64 : (const void*)k_gs_patch;
          SG_CUDA_TRY(cudaLaunchKernelExC(&lc, kfn, args));
          if (ctx->profile) SG_CUDA_TRY(cudaEventRecord(ctx->ev_gs1, s));
          stage_mark(ctx, 6);
          ctx->patched_solves += 1;
        } else if (fp64_start && !ctx->rb2d && ctx->fp64_pairs) {
          // A disc solve going on in one-level FP64 sweeps: in float-float pairs (k_gs_ff1).
          const size_t c4 = sizeof(float4) * (size_t)nc, b = (size_t)std::max(nb, 1);
          if (int r = grow(ctx->ff_n, c4)) return r;
          if (int r = grow(ctx->ff_c, c4)) return r;
          if (int r = grow(ctx->ff_m, c4)) return r;
          if (int r = grow(ctx->ff_r, c4)) return r;
          if (int r = grow(ctx->ff_v, sizeof(float4) * b)) return r;
          if (int r = grow(ctx->ff_minv, sizeof(float2) * b)) return r;
          FfArgs FA{ctx->ff_n.as<float4>(), ctx->ff_c.as<float4>(), ctx->ff_m.as<float4>(), ctx->ff_r.as<float4>(),
                    ctx->ff_v.as<float4>(), ctx->ff_minv.as<float2>()};
          k_pack_ff<<<blocks_for(std::max(nc, nb)), kBlock, 0, s>>>(nc, nb, nullptr, n2, GA.c, GA.W, GA.mu, r2, vrun,
                                                                   P.minv, FA);
          SG_CUDA_TRY(cudaGetLastError());
          ctx->kernel_launches += 1;
          void* args[] = {&GA, &GB, &FA};
          const int g = coop_grid(ctx, k_gs_ff1, nc, kGsFf1Block, 1);
          SG_CUDA_TRY(cudaMemsetAsync(gb, 0, sizeof(GridBarrier), s));
          if (!second_pass) stage_mark(ctx, 5);
          if (ctx->profile) SG_CUDA_TRY(cudaEventRecord(ctx->ev_gs0, s));
          SG_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_gs_ff1, dim3(g), dim3(kGsFf1Block), args, 0, s));
          if (ctx->profile) SG_CUDA_TRY(cudaEventRecord(ctx->ev_gs1, s));
          stage_mark(ctx, 6);
        } else {
          void* args[] = {&GA, &GB};
          const int g = coop_grid(ctx, k_gs_mixed, std::max(nc, nb), kGs32Block, 1);
          // The patch setup's colouring kernels used the barrier with their own grid: reset it.
          SG_CUDA_TRY(cudaMemsetAsync(gb, 0, sizeof(GridBarrier), s));
          if (!second_pass) stage_mark(ctx, 5);
          if (ctx->profile) SG_CUDA_TRY(cudaEventRecord(ctx->ev_gs0, s));
          SG_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_gs_mixed, dim3(g), dim3(kGs32Block), args, 0, s));
          if (ctx->profile) SG_CUDA_TRY(cudaEventRecord(ctx->ev_gs1, s));
          stage_mark(ctx, 6);
        }
        ctx->kernel_launches += 2;
        if (!one_level_first) break;
        SolveStats h1{};
        SG_CUDA_TRY(cudaMemcpyAsync(&h1, st, sizeof(SolveStats), cudaMemcpyDeviceToHost, s));
        SG_CUDA_TRY(cudaStreamSynchronize(s));
        if (h1.converged || h1.status != 0) break;
        // On from the one-level sweeps' best iterate (velocities recomputed from it) on the
        // two-level partition, within the remaining sweeps; the residual slots start afresh.
        if (ctx->profile) {
          float ms = 0.f;
          SG_CUDA_TRY(cudaEventElapsedTime(&ms, ctx->ev_gs0, ctx->ev_gs1));
          ctx->gs_ms += ms;
        }
        probe_iters += h1.iterations;
        probe_evals += h1.evals;
        GA.max_iters = remaining - h1.iterations;
        k_vel_init<<<blocks_for(nb), kBlock, 0, s>>>(nb, off, adj, P.ia, n2, r2,
                                                     reinterpret_cast<const double2*>(P.v0), P.minv, vrun);
        SG_CUDA_TRY(cudaGetLastError());
        SG_CUDA_TRY(cudaMemsetAsync(st->err_slot, 0, sizeof(st->err_slot), s));
        SG_CUDA_TRY(cudaMemsetAsync(st->mag_slot, 0, sizeof(st->mag_slot), s));
        SG_CUDA_TRY(cudaMemsetAsync(gb, 0, sizeof(GridBarrier), s));
        ctx->kernel_launches += 1;
        second_pass = true;
      }
    } else if (!fp32_form) {
      void* args[] = {&GA};
      const int g = coop_grid(ctx, k_gs, nc, kGsBlock, 1);
      stage_mark(ctx, 5);
        if (ctx->profile) SG_CUDA_TRY(cudaEventRecord(ctx->ev_gs0, s));
      SG_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_gs, dim3(g), dim3(kGsBlock), args, 0, s));
      if (ctx->profile) SG_CUDA_TRY(cudaEventRecord(ctx->ev_gs1, s));
        stage_mark(ctx, 6);
    }
    ctx->kernel_launches += 1;  // gs
  }
  ctx->kernel_launches += 2;  // vel_init, final_velocity
  k_final_velocity<<<blocks_for(nb), kBlock, 0, s>>>(nb, off, adj, P.ia, n2, r2, reinterpret_cast<const double2*>(P.v0),
                                                     P.m, P.minv, reinterpret_cast<double2*>(P.v2));
  SG_CUDA_TRY(cudaGetLastError());
  stage_mark(ctx, 7);
  if (sp.learned && ctx->mlp_record) {
    if (int r = mlp_targets(ctx, P)) return r;
    ctx->mlp_last_n = nc;
  }
  SG_CUDA_TRY(cudaMemcpyAsync(&ctx->h_stats, st, sizeof(SolveStats), cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaStreamSynchronize(s));
  if (probe_iters > 0) {  // the one-level FP64 sweeps before the two-level ones
    ctx->h_stats.iterations += probe_iters;
    ctx->h_stats.sweeps64 += probe_iters;
    ctx->h_stats.evals += probe_evals;
  }
  if (nc == 0) {
    ctx->h_stats.iterations = 0;
    ctx->h_stats.converged = 1;
    ctx->h_stats.error = 0.0;
  } else if (ctx->h_stats.status == 0) {
    ctx->gs_launches += 1;
    ctx->contact_sweeps += (uint64_t)ctx->h_stats.sweeps64 * (uint64_t)nc;
    ctx->contact_sweeps32 += (uint64_t)ctx->h_stats.sweeps32 * (uint64_t)nc;
    ctx->contact_evals += (uint64_t)ctx->h_stats.evals * (uint64_t)nc;
    ctx->contact_lifts += (uint64_t)ctx->h_stats.lifts * (uint64_t)nc;
    ctx->body_lifts += (uint64_t)ctx->h_stats.lifts * (uint64_t)nb;
    if (patched_run) {
      for (int q = 0; q < 3; ++q) ctx->patch_phase_ns[q] += ctx->h_stats.phase_ns[q];
      ctx->patch_interior_max_ns += ctx->h_stats.interior_max >> 8;
      ctx->patch_slowest_block = (int)(ctx->h_stats.interior_max & 255ull);
      ctx->patch_boundary_contacts += (uint64_t)ctx->h_stats.boundary_contacts;
      ctx->patch_boundary_colors += (uint64_t)ctx->h_stats.boundary_colors;
    }
    if (ctx->profile) {
      float ms = 0.f;
      SG_CUDA_TRY(cudaEventElapsedTime(&ms, ctx->ev_gs0, ctx->ev_gs1));
      ctx->gs_ms += ms;
    }
  }
  if (ctx->h_stats.status == SG_DEVICE_TIMEOUT) {
    set_error("a device-side wait exceeded its spin limit");
    return SG_DEVICE_TIMEOUT;
  }
  if (ctx->h_stats.status == SG_CAPACITY) {
    set_error("contact colouring exceeded 64 colours or its round limit");
    return SG_CAPACITY;
  }
  return ctx->h_stats.converged ? SG_OK : SG_NOT_CONVERGED;
}

int solve_contacts_batch(sg_ctx* ctx, const ContactProblem& P, const SolveParams& sp, const BatchSolve& X) {
  const int nb = P.nb, cap = P.nc;
  cudaStream_t s = ctx->stream;
  int* off = ctx->body_off.as<int>();
  int* adj = ctx->body_adj.as<int>();
  SolveStats* st = ctx->stats.as<SolveStats>();
  GridBarrier* gb = ctx->barrier.as<GridBarrier>();
  const double2* n2 = reinterpret_cast<const double2*>(P.n);
  double2* r2 = reinterpret_cast<double2*>(P.r);
  if (int r = prepare_contact_graph(ctx, nb, cap, P.ia, P.ib, X.nc_dev)) return r;
  double2* vrun = ctx->v_run.as<double2>();
  k_vel_init<<<blocks_for(nb), kBlock, 0, s>>>(nb, off, adj, P.ia, n2, r2, reinterpret_cast<const double2*>(P.v0),
                                               P.minv, vrun);
  SG_CUDA_TRY(cudaGetLastError());
  SG_CUDA_TRY(cudaMemsetAsync(gb, 0, sizeof(GridBarrier), s));
  SG_CUDA_TRY(cudaMemsetAsync(X.err_slot, 0, sizeof(unsigned long long) * 3 * (size_t)X.S, s));
  SG_CUDA_TRY(cudaMemsetAsync(X.done_count, 0, sizeof(int), s));
  GsBatchArgs B;
  GsArgs& GA = B.g;
  GA.nc = cap;
  GA.ia = P.ia;
  GA.ib = P.ib;
  GA.n = n2;
  GA.c = reinterpret_cast<const double2*>(P.c);
  GA.W = P.W;
  GA.mu = P.mu;
  GA.minv = P.minv;
  GA.perm = ctx->perm.as<int>();
  GA.r = r2;
  GA.r_a = ctx->r_cand.as<double2>();
  GA.r_b = ctx->r_best.as<double2>();
  GA.v = vrun;
  GA.st = st;
  GA.gb = gb;
  GA.spin = ctx->spin_limit;
  GA.tol = sp.tol;
  GA.max_iters = sp.max_iters;
  GA.eval_every = sp.eval_every;
  B.nc_dev = X.nc_dev;
  B.cscene = X.cscene;
  B.sc_off = X.sc_off;
  B.S = X.S;
  B.err_slot = X.err_slot;
  B.best = X.best;
  B.bestbuf = X.bestbuf;
  B.done = X.done;
  B.iters = X.iters;
  B.done_count = X.done_count;
  B.unconverged = X.unconverged;
  B.work = X.work;
  if (X.scene_blocks) {
    // One block per scene: contacts ordered by (scene, colour), then the persistent per-scene sweeps.
    const bool mixed = sp.precision == SG_PRECISION_FP32_REFINE;
    const size_t keys = (size_t)X.S * kMaxColors;
    SG_CUDA_TRY(cudaMemsetAsync(X.key_cnt, 0, sizeof(int) * (keys + 1), s));
    SG_CUDA_TRY(cudaMemsetAsync(X.key_fill, 0, sizeof(int) * (keys + 1), s));
    SG_CUDA_TRY(cudaMemsetAsync(X.next, 0, sizeof(int), s));
    k_scene_color_count<<<blocks_for(cap), kBlock, 0, s>>>(X.nc_dev, X.cscene, ctx->color.as<int>(), X.key_cnt);
    SG_CUDA_TRY(cudaGetLastError());
    if (int r = scan_exclusive(ctx, X.key_cnt, X.key_start, (int)keys)) return r;
    k_scene_color_scatter<<<blocks_for(cap), kBlock, 0, s>>>(X.nc_dev, X.cscene, ctx->color.as<int>(), X.key_start,
                                                            X.key_fill, X.sperm);
    SG_CUDA_TRY(cudaGetLastError());
    SceneBlockArgs Z;
    Z.g = GA;
    if (mixed) {
      k_pack32_scenes<<<blocks_for(cap), kBlock, 0, s>>>(X.key_start + keys, X.sperm, P.ia, P.ib, n2,
                                                         reinterpret_cast<const double2*>(P.c), P.W, P.mu, r2,
                                                         ctx->pk_ab.as<int2>(), ctx->pk_n.as<float2>(),
                                                         ctx->pk_c.as<float2>(), ctx->pk_w.as<float4>(),
                                                         ctx->pk_r.as<float2>());
      k_vel32<<<blocks_for(nb), kBlock, 0, s>>>(nb, vrun, P.minv, ctx->v32.as<float2>(), ctx->minv32.as<float>());
      SG_CUDA_TRY(cudaGetLastError());
      ctx->kernel_launches += 2;
    }
    Z.f.ab = ctx->pk_ab.as<int2>();
    Z.f.n = ctx->pk_n.as<float2>();
    Z.f.c = ctx->pk_c.as<float2>();
    Z.f.w = ctx->pk_w.as<float4>();
    Z.f.r = ctx->pk_r.as<float2>();
    Z.f.v = ctx->v32.as<float2>();
    Z.f.minv = ctx->minv32.as<float>();
    Z.f.minv64 = P.minv;
    Z.f.v0 = reinterpret_cast<const double2*>(P.v0);
    Z.f.body_off = off;
    Z.f.body_adj = adj;
    Z.f.nb = nb;
    Z.f.eval32 = (unsigned)ctx->check_interval;
    Z.v = vrun;
    Z.sb_off = X.sb_off;
    Z.sc_off = X.sc_off;
    Z.nc_dev = X.nc_dev;
    Z.key_start = X.key_start;
    Z.sperm = X.sperm;
    Z.order = X.order;
    Z.next = X.next;
    Z.S = X.S;
    Z.smax = X.smax;
    Z.best = X.best;
    Z.done = X.done;
    Z.iters = X.iters;
    Z.unconverged = X.unconverged;
    Z.work = X.work;
    const size_t smem = (size_t)(mixed ? 24 : 16) * (size_t)X.smax;
    const void* kern = mixed ? (const void*)k_gs_scenes<true> : (const void*)k_gs_scenes<false>;
    int bps = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, kSceneBlock, smem) != cudaSuccess || bps < 1) bps = 1;
    const int g = std::max(1, std::min(ctx->num_sms * bps, X.S));
    void* args[] = {&Z};
    SG_CUDA_TRY(cudaLaunchKernel(kern, dim3(g), dim3(kSceneBlock), args, smem, s));
    ctx->kernel_launches += 5;  // count, 3 scan, scatter
  } else if (sp.precision == SG_PRECISION_FP32_REFINE) {
    k_pack32_b<<<blocks_for(cap), kBlock, 0, s>>>(X.nc_dev, ctx->perm.as<int>(), P.ia, P.ib, n2,
                                                 reinterpret_cast<const double2*>(P.c), P.W, P.mu, r2, X.cscene,
                                                 ctx->pk_ab.as<int2>(), ctx->pk_n.as<float2>(), ctx->pk_c.as<float2>(),
                                                 ctx->pk_w.as<float4>(), ctx->pk_r.as<float2>(), X.pscene);
    k_vel32<<<blocks_for(nb), kBlock, 0, s>>>(nb, vrun, P.minv, ctx->v32.as<float2>(), ctx->minv32.as<float>());
    SG_CUDA_TRY(cudaGetLastError());
    SG_CUDA_TRY(cudaMemsetAsync(X.exc_slot, 0, sizeof(unsigned long long) * 3 * (size_t)X.S, s));
    SG_CUDA_TRY(cudaMemsetAsync(X.gmax, 0, sizeof(unsigned long long) * 3, s));
    Gs32Args GB;
    GB.ab = ctx->pk_ab.as<int2>();
    GB.n = ctx->pk_n.as<float2>();
    GB.c = ctx->pk_c.as<float2>();
    GB.w = ctx->pk_w.as<float4>();
    GB.r = ctx->pk_r.as<float2>();
    GB.v = ctx->v32.as<float2>();
    GB.minv = ctx->minv32.as<float>();
    GB.minv64 = P.minv;
    GB.v0 = reinterpret_cast<const double2*>(P.v0);
    GB.body_off = off;
    GB.body_adj = adj;
    GB.nb = nb;
    GB.eval32 = (unsigned)ctx->check_interval;
    GsMixedBatchArgs M;
    M.X = B;
    M.pscene = X.pscene;
    M.scene_of = X.scene_of;
    M.mode = X.mode;
    M.since = X.since;
    M.exc_slot = X.exc_slot;
    M.gmax = X.gmax;
    M.work = X.work;
    M.n64 = X.n64;
    SG_CUDA_TRY(cudaMemsetAsync(X.n64, 0, sizeof(int), s));
    void* args[] = {&M, &GB};
    const int g = coop_grid(ctx, k_gs_mixed_batch, std::max(std::max(cap, X.S), nb), kGs32Block, 1);
    SG_CUDA_TRY(launch_cooperative((const void*)k_gs_mixed_batch, g, kGs32Block, args, s));
    ctx->kernel_launches += 2;  // pack, vel32
  } else {
    void* args[] = {&B};
    const int g = coop_grid(ctx, k_gs_batch, std::max(cap, X.S), kGsBlock, 1);
    SG_CUDA_TRY(launch_cooperative((const void*)k_gs_batch, g, kGsBlock, args, s));
  }
  k_final_velocity<<<blocks_for(nb), kBlock, 0, s>>>(nb, off, adj, P.ia, n2, r2, reinterpret_cast<const double2*>(P.v0),
                                                     P.m, P.minv, reinterpret_cast<double2*>(P.v2));
  SG_CUDA_TRY(cudaGetLastError());
  ctx->kernel_launches += 3;  // vel_init, gs, final velocity
  return SG_OK;
}

int scene_blocks_prepare(int smax) {
  SG_CUDA_TRY(cudaFuncSetAttribute(k_gs_scenes<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   std::max(16 * smax, 48 * 1024)));
  SG_CUDA_TRY(cudaFuncSetAttribute(k_gs_scenes<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   std::max(24 * smax, 48 * 1024)));
  return SG_OK;
}

int wait_timeout_selftest(sg_ctx* ctx) {
  Buf flag;
  if (int r = grow(flag, 2 * sizeof(int))) return r;
  SG_CUDA_TRY(cudaMemsetAsync(flag.p, 0, 2 * sizeof(int), ctx->stream));
  int* f = flag.as<int>();
  k_wait_flag<<<1, 1, 0, ctx->stream>>>(f, f + 1, ctx->spin_limit);
  SG_CUDA_TRY(cudaGetLastError());
  int status = -1;
  SG_CUDA_TRY(cudaMemcpyAsync(&status, f + 1, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  SG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  release(flag);
  return status;
}

// ===========================================================================
// Allocation-free FrictionSolver entry (sg_sobogus_solve_2d_noalloc).
//
// For callers that cannot call cudaMalloc -- code running where the device
// allocator must not be touched (inside another runtime's memory pool or a
// real-time loop, or under a policy that forbids allocation after start-up) -- the
// whole solve runs on the caller's device buffers plus one fixed scratch array
// declared at file scope below.  Every GPU that loads the library holds the array
// (kNoAllocScratchBytes, about 8.1 MB) until the process exits.  It bounds the
// problem size to kNoAllocMaxBodies bodies and kNoAllocMaxContacts contacts.
namespace {

constexpr int kNoAllocMaxBodies = 16384;
constexpr int kNoAllocMaxContacts = 65536;
constexpr size_t na_align(size_t x) { return (x + 255) & ~size_t(255); }
// Scratch layout (byte offsets, each region 256-byte aligned).
constexpr size_t kNaStats = 0;
constexpr size_t kNaBarrier = na_align(kNaStats + sizeof(SolveStats));
constexpr size_t kNaFlag = na_align(kNaBarrier + sizeof(GridBarrier));
constexpr size_t kNaCnt = na_align(kNaFlag + sizeof(int));
constexpr size_t kNaOff = na_align(kNaCnt + sizeof(int) * (kNoAllocMaxBodies + 1));
constexpr size_t kNaFill = na_align(kNaOff + sizeof(int) * (kNoAllocMaxBodies + 1));
constexpr size_t kNaTiles = na_align(kNaFill + sizeof(int) * (kNoAllocMaxBodies + 1));
constexpr size_t kNaMinv = na_align(kNaTiles + sizeof(int) * 64);
constexpr size_t kNaVrun = na_align(kNaMinv + sizeof(double) * kNoAllocMaxBodies);
constexpr size_t kNaAdj = na_align(kNaVrun + sizeof(double2) * kNoAllocMaxBodies);
constexpr size_t kNaColor = na_align(kNaAdj + sizeof(int) * 2 * kNoAllocMaxContacts);
constexpr size_t kNaPerm = na_align(kNaColor + sizeof(int) * kNoAllocMaxContacts);
constexpr size_t kNaN = na_align(kNaPerm + sizeof(int) * kNoAllocMaxContacts);
constexpr size_t kNaC = na_align(kNaN + sizeof(double2) * kNoAllocMaxContacts);
constexpr size_t kNaW = na_align(kNaC + sizeof(double2) * kNoAllocMaxContacts);
constexpr size_t kNaR = na_align(kNaW + sizeof(double) * 3 * kNoAllocMaxContacts);
constexpr size_t kNaRa = na_align(kNaR + sizeof(double2) * kNoAllocMaxContacts);
constexpr size_t kNaRb = na_align(kNaRa + sizeof(double2) * kNoAllocMaxContacts);
constexpr size_t kNoAllocScratchBytes = na_align(kNaRb + sizeof(double2) * kNoAllocMaxContacts);
static_assert(kNoAllocScratchBytes < 9u * 1024u * 1024u, "scratch must stay modest");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of g_noalloc_scratch, looked up per device and per context: the cache keeps it
// with the identity of the context it was looked up in (cuCtxGetId, reached through the runtime's
// driver entry points so that the library needs no link to the driver library) and looks it up
// again when another context is current, e.g. after cudaDeviceReset re-created the primary context.
constexpr int kNaMaxDevices = 64;
DeviceAddressCache<kNaMaxDevices> g_na_cache;

typedef CUresult (*PfnCtxGetCurrent)(CUcontext*);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long*);

struct NaDriverFns {
  PfnCtxGetCurrent get_current = nullptr;
  PfnCtxGetId get_id = nullptr;
  NaDriverFns() {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<PfnCtxGetCurrent>(p);
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<PfnCtxGetId>(p);
  }
};

// Identity of the context current on this thread; false when there is none or it is unknown.
bool na_current_ctx_id(unsigned long long* id) {
  static const NaDriverFns fns;  // resolved once (thread-safe initialisation)
  *id = 0;
  if (!fns.get_current || !fns.get_id) return false;
  CUcontext c = nullptr;
  if (fns.get_current(&c) != CUDA_SUCCESS || c == nullptr) return false;
  return fns.get_id(c, id) == CUDA_SUCCESS && *id != 0;
}

int na_scratch_address(unsigned char** out) {
  int dev = -1;
  SG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNaMaxDevices) {
    set_error("sg_sobogus_solve_2d_noalloc: device ordinal beyond 63");
    return SG_BAD_INPUT;
  }
  void* p = nullptr;
  const int r = g_na_cache.get(
      dev, na_current_ctx_id,
      [](void** addr) {
        const cudaError_t e = cudaGetSymbolAddress(addr, g_noalloc_scratch);
        if (e != cudaSuccess || !*addr) {
          set_error(std::string("cudaGetSymbolAddress(g_noalloc_scratch) failed: ") + cudaGetErrorString(e));
          return (int)SG_CUDA_ERROR;
        }
        return (int)SG_OK;
      },
      &p);
  if (r != SG_OK) return r;
  *out = static_cast<unsigned char*>(p);
  return SG_OK;
}

__global__ void k_na_minv(int nb, const double* __restrict__ m, double* __restrict__ minv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nb) minv[i] = 1.0 / m[i];
}

// Per-contact assembly of sg_sobogus_solve_2d, on the device, with the same
// operation order; invalid contacts raise *flag and touch nothing else.
__global__ void k_na_assemble(int nb, int nc, const double* __restrict__ minv, const double2* __restrict__ v0,
                              const int* __restrict__ ia, const int* __restrict__ ib, const double* __restrict__ bases,
                              const double* __restrict__ CoR, const double* __restrict__ alpha,
                              const double* __restrict__ beta, double2* __restrict__ n, double2* __restrict__ c,
                              double* __restrict__ W, double2* __restrict__ r, int* flag) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nc) return;
  const int a = ia[k], b = ib[k];
  const double nx = bases[4 * k], ny = bases[4 * k + 1], tx = bases[4 * k + 2], ty = bases[4 * k + 3];
  if (a < 0 || a >= nb || b < -1 || b >= nb || b == a || tx != -ny || ty != nx) {
    atomicExch(flag, 1);
    return;
  }
  const double2 va = v0[a];
  double vrx = va.x, vry = va.y;
  if (b >= 0) {
    const double2 vb = v0[b];
    vrx = vrx - vb.x;
    vry = vry - vb.y;
  } else {
    vrx = vrx - 0.0;
    vry = vry - 0.0;
  }
  const double ndotv = nx * vrx + ny * vry;
  const double nrel = -(0.0 * nx + 0.0 * ny);
  const double drel = -(0.0 * tx + 0.0 * ty);
  const double sc = CoR[k] * ndotv + nrel;
  const double wx = (0.0 + nx * sc) + tx * drel;
  const double wy = (0.0 + ny * sc) + ty * drel;
  n[k] = make_double2(nx, ny);
  c[k] = make_double2(nx * wx + ny * wy, tx * wx + ty * wy);
  const double nn = nx * nx + ny * ny, nt = nx * tx + ny * ty, tt = tx * tx + ty * ty;
  double w00 = minv[a] * nn, w01 = minv[a] * nt, w11 = minv[a] * tt;
  if (b >= 0) {
    w00 = w00 + minv[b] * nn;
    w01 = w01 + minv[b] * nt;
    w11 = w11 + minv[b] * tt;
  }
  W[3 * k] = w00;
  W[3 * k + 1] = w01;
  W[3 * k + 2] = w11;
  const double rwx = alpha[k] * nx + beta[k] * tx;
  const double rwy = alpha[k] * ny + beta[k] * ty;
  r[k] = make_double2(nx * rwx + ny * rwy, tx * rwx + ty * rwy);
}

__global__ void k_na_extract(int nc, const double2* __restrict__ n, const double2* __restrict__ r,
                             const double* __restrict__ mu, double* __restrict__ alpha, double* __restrict__ beta) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nc) return;
  const double2 nk = n[k], rk = r[k];
  const double nx = nk.x, ny = nk.y, tx = -ny, ty = nx;
  const double rwx = nx * rk.x + tx * rk.y;
  const double rwy = ny * rk.x + ty * rk.y;
  alpha[k] = rwx * nx + rwy * ny;
  beta[k] = (mu[k] == 0.0) ? 0.0 : (rwx * tx + rwy * ty);
}

// Friction force per body, summed over its contacts in ascending contact order.
__global__ void k_na_force(int nb, const int* __restrict__ off, const int* __restrict__ adj, const int* __restrict__ ia,
                           const double2* __restrict__ n, const double* __restrict__ beta, double2* __restrict__ f) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  double fx = 0.0, fy = 0.0;
  const int e = off[i + 1];
  for (int p = off[i]; p < e; ++p) {
    const int k = adj[p];
    const double2 nk = n[k];
    const double f0x = beta[k] * -nk.y, f0y = beta[k] * nk.x;
    if (ia[k] == i) {
      fx += f0x;
      fy += f0y;
    } else {
      fx -= f0x;
      fy -= f0y;
    }
  }
  f[i] = make_double2(fx, fy);
}

}  // namespace

int sobogus_solve_2d_noalloc(int32_t nb, const double* m, const double* v0, int32_t nc, const int32_t* ia,
                             const int32_t* ib, const double* bases, const double* CoR, const double* mu,
                             uint32_t max_iters, double tol, uint32_t eval_every, double* alpha, double* beta,
                             double* v2, double* f, void* stream, double* error, uint32_t* iterations) {
  if (nb < 0 || nc < 0 || (nb > 0 && (!m || !v0 || !v2 || !f)) ||
      (nc > 0 && (!ia || !ib || !bases || !CoR || !mu || !alpha || !beta)) || !(tol >= 0.0)) {
    set_error("sg_sobogus_solve_2d_noalloc: invalid arguments");
    return SG_BAD_INPUT;
  }
  if (nb > kNoAllocMaxBodies || nc > kNoAllocMaxContacts) {
    set_error("sg_sobogus_solve_2d_noalloc: " + std::to_string(nb) + " bodies / " + std::to_string(nc) +
              " contacts exceed the fixed scratch limits of " + std::to_string(kNoAllocMaxBodies) + " bodies and " +
              std::to_string(kNoAllocMaxContacts) + " contacts");
    return SG_CAPACITY;
  }
  unsigned char* base = nullptr;
  if (int r = na_scratch_address(&base)) return r;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  SolveStats* st = reinterpret_cast<SolveStats*>(base + kNaStats);
  GridBarrier* gb = reinterpret_cast<GridBarrier*>(base + kNaBarrier);
  int* flag = reinterpret_cast<int*>(base + kNaFlag);
  int* cnt = reinterpret_cast<int*>(base + kNaCnt);
  int* off = reinterpret_cast<int*>(base + kNaOff);
  int* fill = reinterpret_cast<int*>(base + kNaFill);
  int* tiles = reinterpret_cast<int*>(base + kNaTiles);
  double* minv = reinterpret_cast<double*>(base + kNaMinv);
  double2* vrun = reinterpret_cast<double2*>(base + kNaVrun);
  int* adj = reinterpret_cast<int*>(base + kNaAdj);
  int* color = reinterpret_cast<int*>(base + kNaColor);
  int* perm = reinterpret_cast<int*>(base + kNaPerm);
  double2* n2 = reinterpret_cast<double2*>(base + kNaN);
  double2* c2 = reinterpret_cast<double2*>(base + kNaC);
  double* W = reinterpret_cast<double*>(base + kNaW);
  double2* r2 = reinterpret_cast<double2*>(base + kNaR);
  double2* ra = reinterpret_cast<double2*>(base + kNaRa);
  double2* rb = reinterpret_cast<double2*>(base + kNaRb);

  // The array keeps the previous call's contents: clear what must start at zero.
  SG_CUDA_TRY(cudaMemsetAsync(base, 0, kNaCnt, s));  // stats, barrier, flag
  SG_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int) * (size_t)(nb + 1), s));
  SG_CUDA_TRY(cudaMemsetAsync(fill, 0, sizeof(int) * (size_t)(nb + 1), s));
  if (nb > 0) k_na_minv<<<blocks_for(nb), kBlock, 0, s>>>(nb, m, minv);
  if (nc > 0) {
    k_na_assemble<<<blocks_for(nc), kBlock, 0, s>>>(nb, nc, minv, reinterpret_cast<const double2*>(v0), ia, ib, bases,
                                                    CoR, alpha, beta, n2, c2, W, r2, flag);
    SG_CUDA_TRY(cudaGetLastError());
    int h_flag = 0;
    SG_CUDA_TRY(cudaMemcpyAsync(&h_flag, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    SG_CUDA_TRY(cudaStreamSynchronize(s));
    if (h_flag) {
      set_error("sg_sobogus_solve_2d_noalloc: contact body index out of range or tangent not (-n_y, n_x)");
      return SG_BAD_INPUT;
    }
    k_body_count<<<blocks_for(nc), kBlock, 0, s>>>(nc, nullptr, ia, ib, cnt);
  }
  if (int r = scan_exclusive_raw(cnt, off, nb, tiles, s)) return r;
  if (nc > 0) {
    k_body_fill<<<blocks_for(nc), kBlock, 0, s>>>(nc, nullptr, ia, ib, off, fill, adj);
    k_body_sort<<<blocks_for(nb), kBlock, 0, s>>>(nb, off, adj);
  }
  if (nb > 0)
    k_vel_init<<<blocks_for(nb), kBlock, 0, s>>>(nb, off, adj, ia, n2, r2, reinterpret_cast<const double2*>(v0), minv,
                                                 vrun);
  SG_CUDA_TRY(cudaGetLastError());
  int dev = 0, sms = 0;
  SG_CUDA_TRY(cudaGetDevice(&dev));
  SG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  auto grid_for = [&](auto kernel) {
    int bps = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kernel, kBlock, 0) != cudaSuccess || bps < 1) bps = 1;
    const long need = std::max(1L, ((long)nc + kBlock - 1) / kBlock);
    return (int)std::min((long)bps * sms, need);
  };
  const unsigned long long spin = 1ull << 22;  // about a second of barrier polls
  if (nc > 0) {
    SG_CUDA_TRY(cudaMemsetAsync(color, 0xff, sizeof(int) * (size_t)nc, s));
    ColorArgs CA{nc, nullptr, ia, ib, off, adj, color, perm, st, gb, spin, 4096};
    void* cargs[] = {&CA};
    SG_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_color_jp, dim3(grid_for(k_color_jp)), dim3(kBlock), cargs, 0, s));
    SG_CUDA_TRY(cudaMemsetAsync(gb, 0, sizeof(GridBarrier), s));
    GsArgs GA;
    GA.nc = nc;
    GA.ia = ia;
    GA.ib = ib;
    GA.n = n2;
    GA.c = c2;
    GA.W = W;
    GA.mu = mu;
    GA.minv = minv;
    GA.perm = perm;
    GA.r = r2;
    GA.r_a = ra;
    GA.r_b = rb;
    GA.v = vrun;
    GA.st = st;
    GA.gb = gb;
    GA.spin = spin;
    GA.tol = tol;
    GA.max_iters = max_iters;
    GA.eval_every = eval_every;
    void* gargs[] = {&GA};
    SG_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_gs, dim3(grid_for(k_gs)), dim3(kBlock), gargs, 0, s));
  }
  if (nb > 0)
    k_final_velocity<<<blocks_for(nb), kBlock, 0, s>>>(nb, off, adj, ia, n2, r2, reinterpret_cast<const double2*>(v0),
                                                       m, minv, reinterpret_cast<double2*>(v2));
  if (nc > 0) k_na_extract<<<blocks_for(nc), kBlock, 0, s>>>(nc, n2, r2, mu, alpha, beta);
  if (nb > 0)
    k_na_force<<<blocks_for(nb), kBlock, 0, s>>>(nb, off, adj, ia, n2, beta, reinterpret_cast<double2*>(f));
  SG_CUDA_TRY(cudaGetLastError());
  SolveStats h{};
  SG_CUDA_TRY(cudaMemcpyAsync(&h, st, sizeof(SolveStats), cudaMemcpyDeviceToHost, s));
  SG_CUDA_TRY(cudaStreamSynchronize(s));
  if (nc == 0) {
    h.iterations = 0;
    h.converged = 1;
    h.error = 0.0;
  }
  if (error) *error = h.error;
  if (iterations) *iterations = h.iterations;
  if (h.status == SG_DEVICE_TIMEOUT) {
    set_error("a device-side wait exceeded its spin limit");
    return SG_DEVICE_TIMEOUT;
  }
  if (h.status == SG_CAPACITY) {
    set_error("contact colouring exceeded 64 colours or its round limit");
    return SG_CAPACITY;
  }
  return h.converged ? SG_OK : SG_NOT_CONVERGED;
}

}  // namespace sg

extern "C" int sg_sobogus_solve_2d_noalloc(int32_t nb, const double* m, const double* v0, int32_t nc,
                                           const int32_t* ia, const int32_t* ib, const double* bases,
                                           const double* CoR, const double* mu, uint32_t max_iters, double tol,
                                           uint32_t eval_every, double* alpha, double* beta, double* v2, double* f,
                                           void* stream, double* error, uint32_t* iterations) {
  return sg::sobogus_solve_2d_noalloc(nb, m, v0, nc, ia, ib, bases, CoR, mu, max_iters, tol, eval_every, alpha, beta,
                                      v2, f, stream, error, iterations);
}
