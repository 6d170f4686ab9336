// scan.cu -- device-wide exclusive prefix sum over int32 counts.
//
// Reduce-then-scan in three launches: per-tile sums (2048 items per 256-thread
// block), one block scanning the tile sums, then per-tile scans with the tile
// offset.  Used for cell starts, pair offsets, plane-contact offsets and body
// adjacency offsets.
#include "ctx.hpp"

namespace sg {
namespace {

constexpr int kThreads = 256;
constexpr int kItems = 8;
constexpr int kTile = kThreads * kItems;

__device__ __forceinline__ int block_exclusive_scan(int x, int* total) {
  __shared__ int warp_tot[kThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int incl = x;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warp_tot[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int w = lane < kThreads / 32 ? warp_tot[lane] : 0;
    int wi = w;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += y;
    }
    if (lane < kThreads / 32) warp_tot[lane] = wi - w;
    if (lane == kThreads / 32 - 1) *total = wi;
  }
  __syncthreads();
  const int res = warp_tot[wid] + incl - x;
  __syncthreads();
  return res;
}

__global__ void k_tile_reduce(const int* __restrict__ in, int n, int* __restrict__ tile_sums) {
  const long base = (long)blockIdx.x * kTile;
  int s = 0;
#pragma unroll
  for (int i = 0; i < kItems; ++i) {
    const long idx = base + (long)i * kThreads + threadIdx.x;
    if (idx < n) s += in[idx];
  }
  s = warp_sum(s);
  __shared__ int ws[kThreads / 32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < kThreads / 32; ++w) t += ws[w];
    tile_sums[blockIdx.x] = t;
  }
}

// One block: exclusive scan of tile sums in place, total written to *total.
__global__ void k_scan_tile_sums(int* tile_sums, int ntiles, int* total) {
  __shared__ int carry;
  __shared__ int chunk_total;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < ntiles; base += kThreads) {
    const int idx = base + threadIdx.x;
    const int x = idx < ntiles ? tile_sums[idx] : 0;
    const int ex = block_exclusive_scan(x, &chunk_total);
    if (idx < ntiles) tile_sums[idx] = carry + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry += chunk_total;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void k_tile_scan(const int* __restrict__ in, int n, const int* __restrict__ tile_off,
                            int* __restrict__ out) {
  // Each thread owns kItems consecutive items of the tile.
  const long base = (long)blockIdx.x * kTile + (long)threadIdx.x * kItems;
  int vals[kItems];
  int s = 0;
#pragma unroll
  for (int i = 0; i < kItems; ++i) {
    const long idx = base + i;
    vals[i] = idx < n ? in[idx] : 0;
    s += vals[i];
  }
  __shared__ int tot;
  int run = block_exclusive_scan(s, &tot) + tile_off[blockIdx.x];
#pragma unroll
  for (int i = 0; i < kItems; ++i) {
    const long idx = base + i;
    if (idx < n) out[idx] = run;
    run += vals[i];
  }
}

}  // namespace

int scan_exclusive(sg_ctx* ctx, const int* in, int* out, int n) {
  const int ntiles = (n + kTile - 1) / kTile;
  if (n <= 0) {
    SG_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(int), ctx->stream));
    return SG_OK;
  }
  if (int r = grow(ctx->scan_tmp, sizeof(int) * (size_t)(ntiles + 1))) return r;
  int* tiles = ctx->scan_tmp.as<int>();
  k_tile_reduce<<<ntiles, kThreads, 0, ctx->stream>>>(in, n, tiles);
  k_scan_tile_sums<<<1, kThreads, 0, ctx->stream>>>(tiles, ntiles, out + n);
  k_tile_scan<<<ntiles, kThreads, 0, ctx->stream>>>(in, n, tiles, out);
  SG_CUDA_TRY(cudaGetLastError());
  return SG_OK;
}

// The same scan with a caller-provided tile buffer of scan_tile_count(n) + 1 ints
// (no allocation).
int scan_tile_count(int n) { return n <= 0 ? 0 : (n + kTile - 1) / kTile; }

int scan_exclusive_raw(const int* in, int* out, int n, int* tiles, cudaStream_t stream) {
  const int ntiles = scan_tile_count(n);
  if (n <= 0) {
    SG_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(int), stream));
    return SG_OK;
  }
  k_tile_reduce<<<ntiles, kThreads, 0, stream>>>(in, n, tiles);
  k_scan_tile_sums<<<1, kThreads, 0, stream>>>(tiles, ntiles, out + n);
  k_tile_scan<<<ntiles, kThreads, 0, stream>>>(in, n, tiles, out);
  SG_CUDA_TRY(cudaGetLastError());
  return SG_OK;
}

}  // namespace sg
