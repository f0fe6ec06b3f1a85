// reorder.cu -- coherence reordering of a ray batch before traversal.
//
// Rays are bucketed by a 12-bit Morton code of their origin inside the scene's
// root box (16 cells per axis) with a counting sort; the trace kernel then
// takes rays in bucket order through the permutation, so that a warp's rays
// start in the same cell and share the top of their traversals.  Order inside
// a bucket is arbitrary and hits are written back to each ray's own slot, so
// results are unchanged.
//
//   k_bucket_hist    per-block shared-memory histogram; each ray's key and its
//                    rank inside its (block, bucket) are saved, the block's
//                    counts are saved, and one global atomicAdd per (block,
//                    bucket) forms the bucket totals
//   k_bucket_scan    exclusive scan of the 4096 bucket totals (one block)
//   k_bucket_scatter per block: reserve a range per bucket with one global
//                    atomicAdd, then place each ray at its range + its rank
#include <cuda_runtime.h>

#include "rt_internal.h"

namespace rtgb {
namespace {

constexpr int kBuckets = 4096;
constexpr int kSortThreads = 512;

__device__ __forceinline__ uint32_t spread4(uint32_t v) {  // 4 bits -> every third bit
  v &= 0xFu;
  v = (v | (v << 4)) & 0x0C3u;
  v = (v | (v << 2)) & 0x249u;
  return v;
}

__device__ __forceinline__ uint32_t bucket_of(const float4 o, const float3 lo, const float3 inv) {
  const float fx = fminf(fmaxf((o.x - lo.x) * inv.x, 0.0f), 15.0f);
  const float fy = fminf(fmaxf((o.y - lo.y) * inv.y, 0.0f), 15.0f);
  const float fz = fminf(fmaxf((o.z - lo.z) * inv.z, 0.0f), 15.0f);
  return spread4((uint32_t)fx) | (spread4((uint32_t)fy) << 1) | (spread4((uint32_t)fz) << 2);
}

__global__ void __launch_bounds__(kSortThreads) k_bucket_hist(const float4* __restrict__ rays, uint32_t n, float3 lo,
                                                              float3 inv, uint16_t* __restrict__ keys,
                                                              uint32_t* __restrict__ ranks, uint32_t* __restrict__ hist,
                                                              uint32_t* __restrict__ block_hist) {
  __shared__ uint32_t h[kBuckets];
  for (int i = threadIdx.x; i < kBuckets; i += blockDim.x) h[i] = 0u;
  __syncthreads();
  const uint32_t per = (n + gridDim.x - 1) / gridDim.x;
  const uint32_t b = blockIdx.x * per, e = min(n, b + per);
  for (uint32_t i = b + threadIdx.x; i < e; i += blockDim.x) {
    const uint32_t k = bucket_of(__ldg(&rays[2u * i]), lo, inv);
    keys[i] = (uint16_t)k;
    ranks[i] = atomicAdd(&h[k], 1u);
  }
  __syncthreads();
  uint32_t* mine = block_hist + (size_t)blockIdx.x * kBuckets;
  for (int i = threadIdx.x; i < kBuckets; i += blockDim.x) {
    const uint32_t v = h[i];
    mine[i] = v;
    if (v) atomicAdd(&hist[i], v);
  }
}

__global__ void __launch_bounds__(1024) k_bucket_scan(uint32_t* __restrict__ hist) {
  __shared__ uint32_t part[1024];
  const int t = threadIdx.x;
  uint32_t v[kBuckets / 1024];
  uint32_t sum = 0;
  for (int k = 0; k < kBuckets / 1024; ++k) {
    v[k] = hist[t * (kBuckets / 1024) + k];
    sum += v[k];
  }
  part[t] = sum;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {  // inclusive Hillis-Steele scan
    const uint32_t x = t >= off ? part[t - off] : 0u;
    __syncthreads();
    part[t] += x;
    __syncthreads();
  }
  uint32_t run = part[t] - sum;  // exclusive
  for (int k = 0; k < kBuckets / 1024; ++k) {
    hist[t * (kBuckets / 1024) + k] = run;
    run += v[k];
  }
}

__global__ void __launch_bounds__(kSortThreads) k_bucket_scatter(const uint16_t* __restrict__ keys,
                                                                 const uint32_t* __restrict__ ranks, uint32_t n,
                                                                 uint32_t* __restrict__ offsets,
                                                                 const uint32_t* __restrict__ block_hist,
                                                                 uint32_t* __restrict__ order) {
  __shared__ uint32_t base[kBuckets];
  const uint32_t* mine = block_hist + (size_t)blockIdx.x * kBuckets;
  for (int i = threadIdx.x; i < kBuckets; i += blockDim.x) {
    const uint32_t v = mine[i];
    base[i] = v ? atomicAdd(&offsets[i], v) : 0u;
  }
  __syncthreads();
  const uint32_t per = (n + gridDim.x - 1) / gridDim.x;
  const uint32_t b = blockIdx.x * per, e = min(n, b + per);
  for (uint32_t i = b + threadIdx.x; i < e; i += blockDim.x) order[base[keys[i]] + ranks[i]] = i;
}

}  // namespace

// Blocks of the histogram and scatter passes (the same grid for both).
static uint32_t sort_blocks(uint32_t n) {
  uint32_t blocks = (uint32_t)device_sm_count() * 2u;
  const uint32_t need = (uint32_t)(((uint64_t)n + kSortThreads * 8 - 1) / (kSortThreads * 8));
  if (blocks > need) blocks = need;
  return blocks == 0 ? 1u : blocks;
}

static size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

// hist[4096] | block_hist[blocks * 4096] | keys u16[n] | ranks u32[n] | order u32[n]
size_t reorder_scratch_bytes(uint32_t n) {
  return al256((size_t)kBuckets * 4) + al256((size_t)sort_blocks(n) * kBuckets * 4) + al256((size_t)n * 2) +
         al256((size_t)n * 4) + (size_t)n * 4;
}

cudaError_t launch_reorder(const DeviceScene& S, const RtRay* rays, uint32_t n, void* scratch, uint32_t** order_out,
                           void* stream) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const uint32_t blocks = sort_blocks(n);
  char* p = static_cast<char*>(scratch);
  uint32_t* hist = reinterpret_cast<uint32_t*>(p);
  p += al256((size_t)kBuckets * 4);
  uint32_t* block_hist = reinterpret_cast<uint32_t*>(p);
  p += al256((size_t)blocks * kBuckets * 4);
  uint16_t* keys = reinterpret_cast<uint16_t*>(p);
  p += al256((size_t)n * 2);
  uint32_t* ranks = reinterpret_cast<uint32_t*>(p);
  p += al256((size_t)n * 4);
  uint32_t* order = reinterpret_cast<uint32_t*>(p);
  *order_out = order;
  cudaError_t e = cudaMemsetAsync(hist, 0, (size_t)kBuckets * 4, st);
  if (e != cudaSuccess) return e;
  float3 lo = make_float3(S.box[0], S.box[1], S.box[2]);
  float3 inv;
  inv.x = 16.0f / fmaxf(S.box[3] - S.box[0], 1e-30f);
  inv.y = 16.0f / fmaxf(S.box[4] - S.box[1], 1e-30f);
  inv.z = 16.0f / fmaxf(S.box[5] - S.box[2], 1e-30f);
  k_bucket_hist<<<blocks, kSortThreads, 0, st>>>(reinterpret_cast<const float4*>(rays), n, lo, inv, keys, ranks, hist,
                                                 block_hist);
  k_bucket_scan<<<1, 1024, 0, st>>>(hist);
  k_bucket_scatter<<<blocks, kSortThreads, 0, st>>>(keys, ranks, n, hist, block_hist, order);
  return cudaGetLastError();
}

}  // namespace rtgb
