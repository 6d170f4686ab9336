// common.cuh -- device utilities shared by the SCISim GB300 kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>

namespace sg {

constexpr int kMaxColors = 64;

// ---------------------------------------------------------------------------
// Order-preserving map of FP64 onto uint64, so that atomicMin/atomicMax on the
// image give the exact (order-independent) FP64 min/max.  NaN maps above +inf.
__device__ __forceinline__ unsigned long long f64_to_ordered(double x) {
  unsigned long long u = (unsigned long long)__double_as_longlong(x);
  return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double ordered_to_f64(unsigned long long u) {
  u = (u & 0x8000000000000000ull) ? (u & 0x7fffffffffffffffull) : ~u;
  return __longlong_as_double((long long)u);
}
__host__ __device__ constexpr unsigned long long ordered_neg_inf_floor() { return 0ull; }

// Max over non-negative errors, NaN wins.
__device__ __forceinline__ double nanmax(double a, double b) { return (b > a || b != b) ? b : a; }

// ---------------------------------------------------------------------------
// Bounded grid barrier for cooperative launches.  Every wait gives up after
// spin_limit polls, raises `error` and returns false; callers return at once.
struct GridBarrier {
  unsigned int count;
  unsigned int gen;
  int error;
  int pad;
};

// Monotonic counter: barrier number b is complete when count reaches (b + 1) * gridDim.x,
// so each arrival is one atomic and the release needs no reset.  The counter starts
// at zero for every launch (the host clears the struct) and 2^31 arrivals are far
// beyond any launch here.  An error (a wait that ran out) sets the counter's top bit,
// so waiters see it in the word they poll and the release costs no further read;
// `error` mirrors it for the host side.
constexpr unsigned int kBarrierError = 0x80000000u;

__device__ __forceinline__ bool grid_sync(GridBarrier* gb, unsigned long long spin_limit) {
  __syncthreads();
  __shared__ int s_ok;
  if (threadIdx.x == 0) {
    volatile unsigned int* vcount = &gb->count;
    __threadfence();
    const unsigned int old = atomicAdd(&gb->count, 1u);
    int ok = (old & kBarrierError) ? 0 : 1;
    const unsigned int target = ((old & ~kBarrierError) / gridDim.x + 1u) * gridDim.x;
    unsigned long long spins = 0;
    while (ok) {
      const unsigned int v = *vcount;
      if (v & kBarrierError) {
        ok = 0;
      } else if ((int)(v - target) >= 0) {
        break;
      } else if ((++spins & 255ull) == 0ull && spins > spin_limit) {
        atomicOr(&gb->count, kBarrierError);
        atomicExch(&gb->error, 1);
        ok = 0;
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_nanmax(double v) {
  for (int o = 16; o > 0; o >>= 1) v = nanmax(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}

// Block-wide nanmax; result valid in thread 0.  blockDim.x <= 1024.
__device__ __forceinline__ double block_nanmax(double v) {
  __shared__ double s[32];
  v = warp_nanmax(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) s[wid] = v;
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    v = lane < nw ? s[lane] : 0.0;
    v = warp_nanmax(v);
  }
  return v;
}

}  // namespace sg

// ---------------------------------------------------------------------------
// Host-side error plumbing.
namespace sg {
void set_error(const std::string& msg);
}

#define SG_CUDA_TRY(expr)                                                                        \
  do {                                                                                           \
    cudaError_t _e = (expr);                                                                     \
    if (_e != cudaSuccess) {                                                                     \
      ::sg::set_error(std::string(#expr) + ": " + cudaGetErrorString(_e) + " (" __FILE__ ":" +   \
                      std::to_string(__LINE__) + ")");                                          \
      return SG_CUDA_ERROR;                                                                      \
    }                                                                                            \
  } while (0)
