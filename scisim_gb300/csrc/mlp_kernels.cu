// mlp_kernels.cu -- learned per-contact warm start for the Ball2D Gauss-Seidel solve.
//
// No counterpart in the reference: SCISim starts each solve from its impulse cache
// (initializeImpulses, scisim/ConstrainedMaps/GeometricImpactFrictionMap.cpp:174-220).  Here a
// 12 -> 64 -> 64 -> 3 network (GELU) maps local contact features to a start impulse; the
// plain solver still iterates to the same tolerance from whichever start (network or cache)
// has the smaller FP64 Coulomb residual, so the network can only change how many sweeps a
// step takes, never the tolerance a step reaches.
//
//   k_mlp_features   12 features per contact (FP32), from the assembled contact data
//   k_mlp_targets    training targets from the converged impulses of a step
//   k_mlp_fwdbwd     forward + backward of one block of 128 samples (FP32, shared memory),
//                    gradients summed per block then added to the global gradient
//   k_mlp_adam       Adam update (and gradient reset)
//   k_mlp_infer_tc   inference on the tensor cores: BF16 mma.sync m16n8k16 with FP32
//                    accumulation, one warp per 16 contacts, weights staged in shared memory
//   k_mlp_infer_ref  the same network in FP32 on the CUDA cores (error reference for tests)
//
// Features (vs = |g| dt, m_eff = 1 / W_nn, t = (-n_y, n_x), local impulses r = (r_n, r_t);
// velocities, gaps and impulses enter through asinh, which keeps impacts from dominating):
//   0 asinh(n.(v_a - v_b)/vs)   1 asinh(t.(v_a - v_b)/vs)   2 asinh(gap/(vs dt))
//   3 m_b^-1/(m_a^-1 + m_b^-1)   4 g.n/|g|   5 g.t/|g|   6 mu   7 CoR
//   8 asinh(r_n,cache/(m_eff vs))   9 asinh(r_t,cache/(m_eff vs))   10 cache hit
//   11 (contacts of a + contacts of b)/8
// Outputs: y0 ~ asinh(r_n/(m_eff vs)), y1 ~ asinh(r_t/(m_eff vs)), y2 = logit of "the contact
// carries load".  Start impulse: r_n = y2 > 0 ? max(sinh(y0), 0) m_eff vs : 0,
// r_t = clamp(sinh(y1) m_eff vs, -mu r_n, mu r_n) for contacts the impulse cache missed;
// contacts it hit keep the cached impulse (the network fills the cache's gaps).
#include "ctx.hpp"

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <vector>

namespace sg {
namespace {

constexpr int kIn = 12, kH = 64, kOut = 3;
constexpr int oW1 = 0, oB1 = oW1 + kH * kIn, oW2 = oB1 + kH, oB2 = oW2 + kH * kH, oW3 = oB2 + kH,
              oB3 = oW3 + kOut * kH, kParams = oB3 + kOut;
constexpr int kBlock = 256;
constexpr int kTrainBlock = 128;
constexpr int kLd = kH + 1;  // padded row of the per-sample activation tiles (bank-conflict free)
inline int blocks_for(long n, int b = kBlock) { return (int)((n + b - 1) / b); }

__device__ __forceinline__ float gelu_f(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_df(float z) {
  return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * expf(-0.5f * z * z) * 0.39894228040143268f;
}

// ---------------------------------------------------------------------------
struct FeatArgs {
  int nc;
  const int* ia;
  const int* ib;
  const double2* q0;
  const double2* v0;
  const double* rad;
  const double* minv;
  const double2* n;
  const double* W;
  const double* mu;
  const double2* plane_x;
  const double2* r_warm;
  const int* body_off;
  double dt, gx, gy, CoR;
  float* feat;
};

__global__ void k_mlp_features(FeatArgs A) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= A.nc) return;
  const int a = A.ia[k], b = A.ib[k];
  const double2 nk = A.n[k];
  const double tx = -nk.y, ty = nk.x;
  const double2 va = A.v0[a];
  double vrx = va.x, vry = va.y, gap, mratio = 0.0;
  const double2 xa = A.q0[a];
  int deg = A.body_off[a + 1] - A.body_off[a];
  if (b >= 0) {
    const double2 vb = A.v0[b], xb = A.q0[b];
    vrx -= vb.x;
    vry -= vb.y;
    const double dx = xa.x - xb.x, dy = xa.y - xb.y;
    gap = sqrt(dx * dx + dy * dy) - A.rad[a] - A.rad[b];
    mratio = A.minv[b] / (A.minv[a] + A.minv[b]);
    deg += A.body_off[b + 1] - A.body_off[b];
  } else {
    const double2 xp = A.plane_x[-1 - b];
    gap = nk.x * (xa.x - xp.x) + nk.y * (xa.y - xp.y) - A.rad[a];
  }
  const double gn = sqrt(A.gx * A.gx + A.gy * A.gy);
  const double gs = gn > 0.0 ? gn : 1.0;
  double vs = gn * A.dt;
  if (!(vs > 0.0)) vs = 1.0;
  const double meff = 1.0 / A.W[3 * k];
  const double2 rw = A.r_warm[k];
  float* f = A.feat + (size_t)kIn * k;
  f[0] = (float)asinh((nk.x * vrx + nk.y * vry) / vs);
  f[1] = (float)asinh((tx * vrx + ty * vry) / vs);
  f[2] = (float)asinh(gap / (vs * A.dt));
  f[3] = (float)mratio;
  f[4] = (float)((A.gx * nk.x + A.gy * nk.y) / gs);
  f[5] = (float)((A.gx * tx + A.gy * ty) / gs);
  f[6] = (float)A.mu[k];
  f[7] = (float)A.CoR;
  f[8] = (float)asinh(rw.x / (meff * vs));
  f[9] = (float)asinh(rw.y / (meff * vs));
  f[10] = (rw.x != 0.0 || rw.y != 0.0) ? 1.0f : 0.0f;
  f[11] = (float)(deg * 0.125);
}

__global__ void k_mlp_targets(int nc, const double2* __restrict__ r, const double* __restrict__ W, double vs,
                              float* __restrict__ tgt) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nc) return;
  const double meff = 1.0 / W[3 * k];
  const double2 rk = r[k];
  tgt[3 * (size_t)k] = (float)asinh(rk.x / (meff * vs));
  tgt[3 * (size_t)k + 1] = (float)asinh(rk.y / (meff * vs));
  tgt[3 * (size_t)k + 2] = rk.x > 0.0 ? 1.0f : 0.0f;
}

// ---------------------------------------------------------------------------
// Training: one block = 128 samples; activations of the block in shared memory.
// Samples are taken in the order idx(i) = (i * stride + offset) mod n (a permutation when
// gcd(stride, n) = 1), from position `first`; `count` samples per call.
struct TrainArgs {
  const float* p;
  const float* x;
  const float* t;
  long n;
  long first, count;
  unsigned long long stride, offset;
  float inv_batch;
  float* grad;
  double* loss;
};

__global__ void __launch_bounds__(kTrainBlock) k_mlp_fwdbwd(TrainArgs A) {
  extern __shared__ float sm[];
  float* P = sm;                          // kParams
  float* X = P + kParams;                 // 128 x 12
  float* H1 = X + kTrainBlock * kIn;      // 128 x kLd
  float* Z1 = H1 + kTrainBlock * kLd;     // 128 x kLd
  float* Z2 = Z1 + kTrainBlock * kLd;     // 128 x kLd (later dZ1)
  float* D = Z2 + kTrainBlock * kLd;      // 128 x kLd (dZ2)
  float* DY = D + kTrainBlock * kLd;      // 128 x 3
  float* G = DY + kTrainBlock * kOut;     // kParams (block gradient)
  __shared__ double s_loss[kTrainBlock / 32];
  const int tid = threadIdx.x;
  for (int i = tid; i < kParams; i += blockDim.x) {
    P[i] = A.p[i];
    G[i] = 0.0f;
  }
  const long pos = A.first + (long)blockIdx.x * kTrainBlock + tid;
  const bool valid = pos < A.first + A.count;
  long s = 0;
  if (valid) s = (long)(((unsigned long long)pos * A.stride + A.offset) % (unsigned long long)A.n);
  for (int i = 0; i < kIn; ++i) X[tid * kIn + i] = valid ? A.x[s * kIn + i] : 0.0f;
  __syncthreads();
  // Forward (thread per sample).
  const float* xs = X + tid * kIn;
  for (int j = 0; j < kH; ++j) {
    float z = P[oB1 + j];
    for (int i = 0; i < kIn; ++i) z += P[oW1 + j * kIn + i] * xs[i];
    Z1[tid * kLd + j] = z;
    H1[tid * kLd + j] = gelu_f(z);
  }
  for (int j = 0; j < kH; ++j) {
    float z = P[oB2 + j];
    for (int i = 0; i < kH; ++i) z += P[oW2 + j * kH + i] * H1[tid * kLd + i];
    Z2[tid * kLd + j] = z;
  }
  float y[kOut];
  for (int j = 0; j < kOut; ++j) {
    float z = P[oB3 + j];
    for (int i = 0; i < kH; ++i) z += P[oW3 + j * kH + i] * gelu_f(Z2[tid * kLd + i]);
    y[j] = z;
  }
  double l = 0.0;
  if (valid) {
    const float* ts = A.t + s * kOut;
    const float e0 = y[0] - ts[0], e1 = y[1] - ts[1];
    const float sp = y[2] > 0.0f ? y[2] + log1pf(expf(-y[2])) : log1pf(expf(y[2]));
    l = 0.5 * (double)e0 * e0 + 0.5 * (double)e1 * e1 + (double)sp - (double)ts[2] * y[2];
    DY[tid * kOut] = e0 * A.inv_batch;
    DY[tid * kOut + 1] = e1 * A.inv_batch;
    DY[tid * kOut + 2] = (1.0f / (1.0f + expf(-y[2])) - ts[2]) * A.inv_batch;
  } else {
    DY[tid * kOut] = DY[tid * kOut + 1] = DY[tid * kOut + 2] = 0.0f;
  }
  // dZ2 = (W3^T dy) * gelu'(z2)
  for (int i = 0; i < kH; ++i) {
    float d = 0.0f;
    for (int j = 0; j < kOut; ++j) d += P[oW3 + j * kH + i] * DY[tid * kOut + j];
    D[tid * kLd + i] = d * gelu_df(Z2[tid * kLd + i]);
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
  if ((tid & 31) == 0) s_loss[tid >> 5] = l;
  __syncthreads();
  // Layer-3 and layer-2 gradients: sums over the block's samples.
  for (int e = tid; e < kOut * kH; e += blockDim.x) {
    const int j = e / kH, i = e % kH;
    float g = 0.0f;
    for (int q = 0; q < kTrainBlock; ++q) g += DY[q * kOut + j] * gelu_f(Z2[q * kLd + i]);
    G[oW3 + e] = g;
  }
  if (tid < kOut) {
    float g = 0.0f;
    for (int q = 0; q < kTrainBlock; ++q) g += DY[q * kOut + tid];
    G[oB3 + tid] = g;
  }
  for (int e = tid; e < kH * kH; e += blockDim.x) {
    const int j = e / kH, i = e % kH;
    float g = 0.0f;
    for (int q = 0; q < kTrainBlock; ++q) g += D[q * kLd + j] * H1[q * kLd + i];
    G[oW2 + e] = g;
  }
  if (tid < kH) {
    float g = 0.0f;
    for (int q = 0; q < kTrainBlock; ++q) g += D[q * kLd + tid];
    G[oB2 + tid] = g;
  }
  // dZ1 = (W2^T dZ2) * gelu'(z1), into Z2's rows once every thread is done reading Z2.
  __syncthreads();
  for (int i = 0; i < kH; ++i) {
    float d = 0.0f;
    for (int j = 0; j < kH; ++j) d += P[oW2 + j * kH + i] * D[tid * kLd + j];
    Z2[tid * kLd + i] = d * gelu_df(Z1[tid * kLd + i]);
  }
  __syncthreads();
  for (int e = tid; e < kH * kIn; e += blockDim.x) {
    const int j = e / kIn, i = e % kIn;
    float g = 0.0f;
    for (int q = 0; q < kTrainBlock; ++q) g += Z2[q * kLd + j] * X[q * kIn + i];
    G[oW1 + e] = g;
  }
  if (tid < kH) {
    float g = 0.0f;
    for (int q = 0; q < kTrainBlock; ++q) g += Z2[q * kLd + tid];
    G[oB1 + tid] = g;
  }
  __syncthreads();
  for (int i = tid; i < kParams; i += blockDim.x) atomicAdd(&A.grad[i], G[i]);
  if (tid == 0) {
    double bl = 0.0;
    for (int w = 0; w < kTrainBlock / 32; ++w) bl += s_loss[w];
    atomicAdd(A.loss, bl);
  }
}

__global__ void k_mlp_adam(float* __restrict__ p, float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                           float lr, float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kParams) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.0f - b1) * gi;
  const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  g[i] = 0.0f;
}

// ---------------------------------------------------------------------------
// Inference.
__device__ __forceinline__ void start_from_output(float y0, float y1, float y2, double meff, double vs, double mu,
                                                  double2& r) {
  double rn = (y2 > 0.0f && y0 > 0.0f) ? sinh((double)y0) * meff * vs : 0.0;
  double rt = sinh((double)y1) * meff * vs;
  const double lim = mu * rn;
  rt = rt > lim ? lim : (rt < -lim ? -lim : rt);
  r = make_double2(rn, rt);
}

__global__ void k_mlp_infer_ref(const float* __restrict__ p, int n, const float* __restrict__ x, float* __restrict__ y) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  float h1[kH];
  for (int j = 0; j < kH; ++j) {
    float z = p[oB1 + j];
    for (int i = 0; i < kIn; ++i) z += p[oW1 + j * kIn + i] * x[(size_t)s * kIn + i];
    h1[j] = gelu_f(z);
  }
  float out[kOut];
  for (int j = 0; j < kOut; ++j) out[j] = p[oB3 + j];
  for (int j = 0; j < kH; ++j) {
    float z = p[oB2 + j];
    for (int i = 0; i < kH; ++i) z += p[oW2 + j * kH + i] * h1[i];
    const float h = gelu_f(z);
    for (int o = 0; o < kOut; ++o) out[o] += p[oW3 + o * kH + j] * h;
  }
  for (int o = 0; o < kOut; ++o) y[(size_t)s * kOut + o] = out[o];
}

__device__ __forceinline__ unsigned pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const unsigned*>(&v);
}

__device__ __forceinline__ void mma_bf16(float* d, unsigned a0, unsigned a1, unsigned a2, unsigned a3, unsigned b0,
                                         unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Shared-memory image of the network in BF16: W1 padded to 16 inputs, W3 padded to 8 outputs.
constexpr int kW1s = kH * 16, kW2s = kH * kH, kW3s = 8 * kH;

struct InferArgs {
  const float* p;     // FP32 parameters (biases are read in FP32)
  int n;
  const float* x;     // features
  float* y;           // optional raw outputs (3 per contact)
  double2* r;         // optional start impulses
  const double2* r_warm;  // cached start (kept where the cache hit, feature 10)
  const double* W;    // Delassus blocks (m_eff) for r
  const double* mu;
  double vs;
};

// One warp per 16 contacts.  Fragment layouts of mma.m16n8k16 (PTX ISA): with g = lane / 4,
// c = lane % 4, A holds rows g and g + 8 at columns 2c, 2c + 1 (+8), B holds rows 2c, 2c + 1
// (+8) at column g, and the accumulator holds rows g and g + 8 at columns 2c, 2c + 1.  The
// accumulators of n-tiles 2j and 2j + 1 are therefore exactly the A fragment of k-block j
// of the next layer.
__global__ void __launch_bounds__(128) k_mlp_infer_tc(InferArgs A) {
  __shared__ __align__(16) __nv_bfloat16 w1[kW1s];
  __shared__ __align__(16) __nv_bfloat16 w2[kW2s];
  __shared__ __align__(16) __nv_bfloat16 w3[kW3s];
  __shared__ float bias[kH + kH + 8];
  for (int e = threadIdx.x; e < kW1s; e += blockDim.x) {
    const int j = e / 16, i = e % 16;
    w1[e] = __float2bfloat16_rn(i < kIn ? A.p[oW1 + j * kIn + i] : 0.0f);
  }
  for (int e = threadIdx.x; e < kW2s; e += blockDim.x) w2[e] = __float2bfloat16_rn(A.p[oW2 + e]);
  for (int e = threadIdx.x; e < kW3s; e += blockDim.x) {
    const int j = e / kH, i = e % kH;
    w3[e] = __float2bfloat16_rn(j < kOut ? A.p[oW3 + j * kH + i] : 0.0f);
  }
  for (int e = threadIdx.x; e < kH + kH + 8; e += blockDim.x) {
    float b = 0.0f;
    if (e < kH)
      b = A.p[oB1 + e];
    else if (e < 2 * kH)
      b = A.p[oB2 + e - kH];
    else if (e - 2 * kH < kOut)
      b = A.p[oB3 + e - 2 * kH];
    bias[e] = b;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int g = lane >> 2, c = lane & 3;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  const unsigned* w1u = reinterpret_cast<const unsigned*>(w1);
  const unsigned* w2u = reinterpret_cast<const unsigned*>(w2);
  const unsigned* w3u = reinterpret_cast<const unsigned*>(w3);
  for (int tile = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; tile * 16 < A.n; tile += warps) {
    const int r0 = tile * 16 + g, r1 = r0 + 8;
    auto feat = [&](int row, int col) -> float {
      return (row < A.n && col < kIn) ? A.x[(size_t)row * kIn + col] : 0.0f;
    };
    // Layer 1: [16 x 16] x [16 x 64].
    const unsigned a0 = pack_bf16(feat(r0, 2 * c), feat(r0, 2 * c + 1));
    const unsigned a1 = pack_bf16(feat(r1, 2 * c), feat(r1, 2 * c + 1));
    const unsigned a2 = pack_bf16(feat(r0, 2 * c + 8), feat(r0, 2 * c + 9));
    const unsigned a3 = pack_bf16(feat(r1, 2 * c + 8), feat(r1, 2 * c + 9));
    float acc[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      const int col = nt * 8 + 2 * c;
      acc[nt][0] = acc[nt][2] = bias[col];
      acc[nt][1] = acc[nt][3] = bias[col + 1];
      const int wrow = nt * 8 + g;  // output neuron = column of B
      mma_bf16(acc[nt], a0, a1, a2, a3, w1u[(wrow * 16 + 2 * c) >> 1], w1u[(wrow * 16 + 2 * c + 8) >> 1]);
    }
    unsigned h[4][4];
#pragma unroll
    for (int kb = 0; kb < 4; ++kb) {
      h[kb][0] = pack_bf16(gelu_f(acc[2 * kb][0]), gelu_f(acc[2 * kb][1]));
      h[kb][1] = pack_bf16(gelu_f(acc[2 * kb][2]), gelu_f(acc[2 * kb][3]));
      h[kb][2] = pack_bf16(gelu_f(acc[2 * kb + 1][0]), gelu_f(acc[2 * kb + 1][1]));
      h[kb][3] = pack_bf16(gelu_f(acc[2 * kb + 1][2]), gelu_f(acc[2 * kb + 1][3]));
    }
    // Layer 2: [16 x 64] x [64 x 64].
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      const int col = nt * 8 + 2 * c;
      acc[nt][0] = acc[nt][2] = bias[kH + col];
      acc[nt][1] = acc[nt][3] = bias[kH + col + 1];
      const int wrow = nt * 8 + g;
#pragma unroll
      for (int kb = 0; kb < 4; ++kb)
        mma_bf16(acc[nt], h[kb][0], h[kb][1], h[kb][2], h[kb][3], w2u[(wrow * kH + kb * 16 + 2 * c) >> 1],
                 w2u[(wrow * kH + kb * 16 + 2 * c + 8) >> 1]);
    }
#pragma unroll
    for (int kb = 0; kb < 4; ++kb) {
      h[kb][0] = pack_bf16(gelu_f(acc[2 * kb][0]), gelu_f(acc[2 * kb][1]));
      h[kb][1] = pack_bf16(gelu_f(acc[2 * kb][2]), gelu_f(acc[2 * kb][3]));
      h[kb][2] = pack_bf16(gelu_f(acc[2 * kb + 1][0]), gelu_f(acc[2 * kb + 1][1]));
      h[kb][3] = pack_bf16(gelu_f(acc[2 * kb + 1][2]), gelu_f(acc[2 * kb + 1][3]));
    }
    // Layer 3: [16 x 64] x [64 x 8] (3 outputs used).
    float o[4];
    o[0] = o[2] = bias[2 * kH + 2 * c];
    o[1] = o[3] = bias[2 * kH + 2 * c + 1];
#pragma unroll
    for (int kb = 0; kb < 4; ++kb)
      mma_bf16(o, h[kb][0], h[kb][1], h[kb][2], h[kb][3], w3u[(g * kH + kb * 16 + 2 * c) >> 1],
               w3u[(g * kH + kb * 16 + 2 * c + 8) >> 1]);
    // Outputs of row r0 sit in lanes 4g (y0, y1) and 4g + 1 (y2); row r1 likewise in o[2], o[3].
    const float y2_r0 = __shfl_down_sync(0xffffffffu, o[0], 1);
    const float y2_r1 = __shfl_down_sync(0xffffffffu, o[2], 1);
    if (c == 0) {
      if (r0 < A.n) {
        if (A.y) {
          A.y[(size_t)r0 * kOut] = o[0];
          A.y[(size_t)r0 * kOut + 1] = o[1];
          A.y[(size_t)r0 * kOut + 2] = y2_r0;
        }
        if (A.r) {
          if (A.x[(size_t)r0 * kIn + 10] > 0.5f)
            A.r[r0] = A.r_warm[r0];
          else
            start_from_output(o[0], o[1], y2_r0, 1.0 / A.W[3 * r0], A.vs, A.mu[r0], A.r[r0]);
        }
      }
      if (r1 < A.n) {
        if (A.y) {
          A.y[(size_t)r1 * kOut] = o[2];
          A.y[(size_t)r1 * kOut + 1] = o[3];
          A.y[(size_t)r1 * kOut + 2] = y2_r1;
        }
        if (A.r) {
          if (A.x[(size_t)r1 * kIn + 10] > 0.5f)
            A.r[r1] = A.r_warm[r1];
          else
            start_from_output(o[2], o[3], y2_r1, 1.0 / A.W[3 * r1], A.vs, A.mu[r1], A.r[r1]);
        }
      }
    }
  }
}

size_t train_smem_bytes() {
  return sizeof(float) * ((size_t)2 * kParams + kTrainBlock * kIn + 4 * kTrainBlock * kLd + kTrainBlock * kOut);
}

double velocity_scale(const sg_ctx* ctx) {
  const double gn = std::sqrt(ctx->cfg.gravity[0] * ctx->cfg.gravity[0] + ctx->cfg.gravity[1] * ctx->cfg.gravity[1]);
  const double vs = gn * ctx->cfg.dt;
  return vs > 0.0 ? vs : 1.0;
}

}  // namespace

int mlp_param_count() { return kParams; }

int mlp_load(sg_ctx* ctx, const float* params) {
  if (int r = grow(ctx->mlp_p, sizeof(float) * kParams)) return r;
  SG_CUDA_TRY(cudaMemcpyAsync(ctx->mlp_p.p, params, sizeof(float) * kParams, cudaMemcpyHostToDevice, ctx->stream));
  SG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  ctx->mlp_loaded = true;
  return SG_OK;
}

// Features of the assembled contacts (adjacency built), into ctx->mlp_feat.
int mlp_features(sg_ctx* ctx, const ContactProblem& P) {
  if (int r = grow(ctx->mlp_feat, sizeof(float) * kIn * (size_t)std::max(P.nc, 1))) return r;
  if (P.nc == 0) return SG_OK;
  FeatArgs A;
  A.nc = P.nc;
  A.ia = P.ia;
  A.ib = P.ib;
  A.q0 = ctx->q.as<double2>();
  A.v0 = reinterpret_cast<const double2*>(P.v0);
  A.rad = ctx->r.as<double>();
  A.minv = P.minv;
  A.n = reinterpret_cast<const double2*>(P.n);
  A.W = P.W;
  A.mu = P.mu;
  A.plane_x = ctx->plane_x.as<double2>();
  A.r_warm = reinterpret_cast<const double2*>(P.r);
  A.body_off = ctx->body_off.as<int>();
  A.dt = ctx->cfg.dt;
  A.gx = ctx->cfg.gravity[0];
  A.gy = ctx->cfg.gravity[1];
  A.CoR = ctx->cfg.CoR;
  A.feat = ctx->mlp_feat.as<float>();
  k_mlp_features<<<blocks_for(P.nc), kBlock, 0, ctx->stream>>>(A);
  SG_CUDA_TRY(cudaGetLastError());
  ctx->kernel_launches += 1;
  return SG_OK;
}

// Start impulses predicted for the assembled contacts, into r_alt (double2 per contact).
int mlp_predict(sg_ctx* ctx, const ContactProblem& P, double* r_alt) {
  if (P.nc == 0) return SG_OK;
  InferArgs A;
  A.p = ctx->mlp_p.as<float>();
  A.n = P.nc;
  A.x = ctx->mlp_feat.as<float>();
  A.y = nullptr;
  A.r = reinterpret_cast<double2*>(r_alt);
  A.r_warm = reinterpret_cast<const double2*>(P.r);
  A.W = P.W;
  A.mu = P.mu;
  A.vs = velocity_scale(ctx);
  const int tiles = (P.nc + 15) / 16;
  k_mlp_infer_tc<<<std::max(1, std::min(blocks_for(tiles, 4), ctx->num_sms * 16)), 128, 0, ctx->stream>>>(A);
  SG_CUDA_TRY(cudaGetLastError());
  ctx->kernel_launches += 1;
  return SG_OK;
}

int mlp_targets(sg_ctx* ctx, const ContactProblem& P) {
  if (int r = grow(ctx->mlp_tgt, sizeof(float) * kOut * (size_t)std::max(P.nc, 1))) return r;
  if (P.nc == 0) return SG_OK;
  k_mlp_targets<<<blocks_for(P.nc), kBlock, 0, ctx->stream>>>(P.nc, reinterpret_cast<const double2*>(P.r), P.W,
                                                             velocity_scale(ctx), ctx->mlp_tgt.as<float>());
  SG_CUDA_TRY(cudaGetLastError());
  ctx->kernel_launches += 1;
  return SG_OK;
}

}  // namespace sg

using namespace sg;

namespace {

unsigned long long gcd_u64(unsigned long long a, unsigned long long b) {
  while (b) {
    const unsigned long long t = a % b;
    a = b;
    b = t;
  }
  return a;
}

// splitmix64
unsigned long long mix64(unsigned long long& s) {
  unsigned long long z = (s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

int upload_samples(sg_ctx* ctx, long n, const float* x, const float* t) {
  if (int r = grow(ctx->mlp_x, sizeof(float) * kIn * (size_t)n)) return r;
  if (int r = grow(ctx->mlp_t, sizeof(float) * kOut * (size_t)n)) return r;
  SG_CUDA_TRY(cudaMemcpyAsync(ctx->mlp_x.p, x, sizeof(float) * kIn * (size_t)n, cudaMemcpyHostToDevice, ctx->stream));
  if (t)
    SG_CUDA_TRY(cudaMemcpyAsync(ctx->mlp_t.p, t, sizeof(float) * kOut * (size_t)n, cudaMemcpyHostToDevice, ctx->stream));
  return SG_OK;
}

int launch_fwdbwd(sg_ctx* ctx, const float* p, long n, long first, long count, unsigned long long stride,
                  unsigned long long offset, float inv_batch, float* grad, double* loss) {
  TrainArgs A{p, ctx->mlp_x.as<float>(), ctx->mlp_t.as<float>(), n, first, count, stride, offset, inv_batch, grad, loss};
  const size_t smem = train_smem_bytes();
  if (!ctx->mlp_smem_set) {
    SG_CUDA_TRY(cudaFuncSetAttribute(k_mlp_fwdbwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    ctx->mlp_smem_set = true;
  }
  k_mlp_fwdbwd<<<blocks_for(count, kTrainBlock), kTrainBlock, smem, ctx->stream>>>(A);
  SG_CUDA_TRY(cudaGetLastError());
  return SG_OK;
}

}  // namespace

extern "C" {

int sg_mlp_param_count(void) { return kParams; }

int sg_mlp_load(sg_ctx* ctx, const float* params, int32_t n_params) {
  if (!ctx || !params || n_params != kParams) return SG_BAD_INPUT;
  SG_CUDA_TRY(cudaSetDevice(ctx->device));
  return mlp_load(ctx, params);
}

int sg_mlp_enable(sg_ctx* ctx, int32_t warm_start, int32_t record) {
  if (!ctx || (warm_start && !ctx->mlp_loaded)) {
    set_error("sg_mlp_enable: load the network first (sg_mlp_load)");
    return SG_BAD_INPUT;
  }
  if (ctx->n_scenes > 0 || ctx->dim != 2) {
    set_error("sg_mlp_enable: the learned warm start serves single Ball2D scenes");
    return SG_BAD_INPUT;
  }
  ctx->mlp_on = warm_start != 0;
  ctx->mlp_record = record != 0;
  return SG_OK;
}

int64_t sg_mlp_last_samples(sg_ctx* ctx, int64_t cap, float* x, float* t) {
  if (!ctx || !ctx->mlp_record) return INT64_MIN;
  const int64_t n = ctx->mlp_last_n;
  if (n > cap) return -(n + 1);
  if (n == 0) return 0;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return INT64_MIN;
  if (x) cudaMemcpyAsync(x, ctx->mlp_feat.p, sizeof(float) * kIn * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream);
  if (t) cudaMemcpyAsync(t, ctx->mlp_tgt.p, sizeof(float) * kOut * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream);
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return INT64_MIN;
  return n;
}

int sg_mlp_grad(sg_ctx* ctx, const float* params, int32_t n, const float* x, const float* t, float* grad,
                double* loss) {
  if (!ctx || !params || n <= 0 || !x || !t || !grad) return SG_BAD_INPUT;
  SG_CUDA_TRY(cudaSetDevice(ctx->device));
  if (int r = upload_samples(ctx, n, x, t)) return r;
  Buf p, g, l;
  int rc = grow(p, sizeof(float) * kParams);
  if (!rc) rc = grow(g, sizeof(float) * kParams);
  if (!rc) rc = grow(l, sizeof(double));
  if (!rc) {
    cudaMemcpyAsync(p.p, params, sizeof(float) * kParams, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemsetAsync(g.p, 0, sizeof(float) * kParams, ctx->stream);
    cudaMemsetAsync(l.p, 0, sizeof(double), ctx->stream);
    rc = launch_fwdbwd(ctx, p.as<float>(), n, 0, n, 1, 0, 1.0f / (float)n, g.as<float>(), l.as<double>());
  }
  double lh = 0.0;
  if (!rc) {
    cudaMemcpyAsync(grad, g.p, sizeof(float) * kParams, cudaMemcpyDeviceToHost, ctx->stream);
    cudaMemcpyAsync(&lh, l.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) rc = SG_CUDA_ERROR;
  }
  if (loss) *loss = lh / n;
  release(p);
  release(g);
  release(l);
  return rc;
}

int sg_mlp_train(sg_ctx* ctx, int64_t n, const float* x, const float* t, int32_t epochs, int32_t batch, float lr,
                 uint64_t seed, float* params, double* epoch_loss) {
  if (!ctx || n <= 0 || !x || !t || !params || epochs <= 0 || batch <= 0) return SG_BAD_INPUT;
  SG_CUDA_TRY(cudaSetDevice(ctx->device));
  if (int r = upload_samples(ctx, n, x, t)) return r;
  Buf p, g, m, v, l;
  int rc = grow(p, sizeof(float) * kParams);
  if (!rc) rc = grow(g, sizeof(float) * kParams);
  if (!rc) rc = grow(m, sizeof(float) * kParams);
  if (!rc) rc = grow(v, sizeof(float) * kParams);
  if (!rc) rc = grow(l, sizeof(double) * (size_t)epochs);
  cudaStream_t s = ctx->stream;
  if (!rc) {
    cudaMemcpyAsync(p.p, params, sizeof(float) * kParams, cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(g.p, 0, sizeof(float) * kParams, s);
    cudaMemsetAsync(m.p, 0, sizeof(float) * kParams, s);
    cudaMemsetAsync(v.p, 0, sizeof(float) * kParams, s);
    cudaMemsetAsync(l.p, 0, sizeof(double) * (size_t)epochs, s);
  }
  unsigned long long state = seed;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  float p1 = 1.0f, p2 = 1.0f;
  for (int e = 0; e < epochs && !rc; ++e) {
    // A fresh permutation of the samples every epoch: i -> (i * stride + offset) mod n.
    unsigned long long stride = (mix64(state) % (unsigned long long)n) | 1ull;
    while (gcd_u64(stride, (unsigned long long)n) != 1ull) stride = (stride + 2) % (unsigned long long)n | 1ull;
    const unsigned long long offset = mix64(state) % (unsigned long long)n;
    for (long first = 0; first < n && !rc; first += batch) {
      const long count = std::min<long>(batch, n - first);
      rc = launch_fwdbwd(ctx, p.as<float>(), n, first, count, stride, offset, 1.0f / (float)count, g.as<float>(),
                         l.as<double>() + e);
      p1 *= b1;
      p2 *= b2;
      if (!rc) {
        k_mlp_adam<<<blocks_for(kParams), kBlock, 0, s>>>(p.as<float>(), g.as<float>(), m.as<float>(), v.as<float>(), lr,
                                                         b1, b2, eps, 1.0f - p1, 1.0f - p2);
        if (cudaGetLastError() != cudaSuccess) rc = SG_CUDA_ERROR;
      }
      ctx->kernel_launches += 2;
    }
  }
  std::vector<double> lh((size_t)epochs);
  if (!rc) {
    cudaMemcpyAsync(params, p.p, sizeof(float) * kParams, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(lh.data(), l.p, sizeof(double) * (size_t)epochs, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) rc = SG_CUDA_ERROR;
  }
  if (!rc && epoch_loss)
    for (int e = 0; e < epochs; ++e) epoch_loss[e] = lh[e] / (double)n;
  release(p);
  release(g);
  release(m);
  release(v);
  release(l);
  return rc;
}

int sg_mlp_infer(sg_ctx* ctx, const float* params, int32_t n, const float* x, float* y, int32_t tensor_cores) {
  if (!ctx || !params || n <= 0 || !x || !y) return SG_BAD_INPUT;
  SG_CUDA_TRY(cudaSetDevice(ctx->device));
  if (int r = upload_samples(ctx, n, x, nullptr)) return r;
  Buf p, out;
  int rc = grow(p, sizeof(float) * kParams);
  if (!rc) rc = grow(out, sizeof(float) * kOut * (size_t)n);
  if (!rc) {
    cudaMemcpyAsync(p.p, params, sizeof(float) * kParams, cudaMemcpyHostToDevice, ctx->stream);
    if (tensor_cores) {
      InferArgs A{p.as<float>(), n, ctx->mlp_x.as<float>(), out.as<float>(), nullptr, nullptr, nullptr, nullptr, 1.0};
      const int tiles = (n + 15) / 16;
      k_mlp_infer_tc<<<std::max(1, std::min(blocks_for(tiles, 4), ctx->num_sms * 16)), 128, 0, ctx->stream>>>(A);
    } else {
      k_mlp_infer_ref<<<blocks_for(n), kBlock, 0, ctx->stream>>>(p.as<float>(), n, ctx->mlp_x.as<float>(),
                                                                out.as<float>());
    }
    if (cudaGetLastError() != cudaSuccess) rc = SG_CUDA_ERROR;
  }
  if (!rc) {
    cudaMemcpyAsync(y, out.p, sizeof(float) * kOut * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream);
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) rc = SG_CUDA_ERROR;
  }
  release(p);
  release(out);
  return rc;
}

int sg_mlp_stats(sg_ctx* ctx, uint64_t* steps_evaluated, uint64_t* steps_network_start) {
  if (!ctx) return SG_BAD_INPUT;
  SG_CUDA_TRY(cudaSetDevice(ctx->device));
  unsigned long long chosen = 0;
  if (ctx->mlp_choice.p) {
    SG_CUDA_TRY(cudaMemcpyAsync(&chosen, ctx->mlp_choice.p, sizeof chosen, cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  }
  if (steps_evaluated) *steps_evaluated = ctx->mlp_evals;
  if (steps_network_start) *steps_network_start = chosen;
  return SG_OK;
}

}  // extern "C"
