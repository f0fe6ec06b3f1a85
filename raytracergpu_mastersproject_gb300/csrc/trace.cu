// trace.cu -- ray-query kernels (closest hit / any hit) for sm_103a.
//
// Replaces hitBVH/sceneHit (raytraceBVH.comp:195-274) for batches of
// independent rays.  Persistent warps: each warp takes rays 32 at a time from
// a global counter (one atomicAdd per refill), traverses them with the
// near-first while-while loop of trace_core.cuh, and hands new rays to lanes
// that finished whenever fewer than kRefill lanes are still busy.
#include <cuda_runtime.h>

#include "trace_core.cuh"

namespace rtgb {
namespace {

constexpr int kThreads = 128;
constexpr int kRefill = 20;

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

template <bool ANY, int STACK>
__global__ void __launch_bounds__(kThreads) k_trace(DeviceScene S, const float4* __restrict__ rays, uint32_t n,
                                                    uint2* __restrict__ hits, uint32_t* __restrict__ counter) {
  uint32_t stack[STACK];
  dev::Trav s;
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t ray = 0xFFFFFFFFu;
  bool exhausted = false;
  for (;;) {
    const bool idle = ray == 0xFFFFFFFFu;
    const uint32_t m = __ballot_sync(0xFFFFFFFFu, idle);
    if (m != 0u && !exhausted) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(counter, (uint32_t)__popc(m));
      base = __shfl_sync(0xFFFFFFFFu, base, 0);
      if (base + (uint32_t)__popc(m) >= n) exhausted = true;
      if (idle) {
        const uint32_t id = base + (uint32_t)__popc(m & lanemask_lt());
        if (id < n) {
          ray = id;
          dev::trav_init(s, __ldg(&rays[2u * id]), __ldg(&rays[2u * id + 1u]), S.root, stack);
        }
      }
    }
    if (__all_sync(0xFFFFFFFFu, ray == 0xFFFFFFFFu)) break;
    if (ray != 0xFFFFFFFFu) {
      const bool done = dev::trav_run<ANY, STACK>(S, s, stack, exhausted ? 0 : kRefill);
      if (done || s.sp < 0) {
        uint2 h;
        if (s.sp < 0 || s.best == dev::kNoBest) {
          h.x = RT_NO_HIT;
          h.y = __float_as_uint(__int_as_float(0x7f800000));
        } else if (s.best & kSphereBit) {
          h.x = (s.best & kSphereMask) | RT_HIT_SPHERE_BIT;
          h.y = __float_as_uint(s.tclose);
        } else {
          h.x = __ldg(&S.tri_ids[s.best & kSlotMask]);
          h.y = __float_as_uint(s.tclose);
        }
        hits[ray] = h;
        ray = 0xFFFFFFFFu;
      }
    }
  }
}

template <bool ANY, int STACK>
cudaError_t launch_variant(const DeviceScene& S, const RtRay* rays, uint32_t n, RtHit* hits, uint32_t* counter,
                           cudaStream_t st) {
  static int blocks_per_sm = -1;
  if (blocks_per_sm < 0) {
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_trace<ANY, STACK>, kThreads, 0);
    if (e != cudaSuccess) return e;
    if (blocks_per_sm < 1) blocks_per_sm = 1;
  }
  const uint32_t warps_needed = (n + 31u) / 32u;
  uint32_t blocks = (uint32_t)(device_sm_count() * blocks_per_sm);
  const uint32_t blocks_needed = (warps_needed + (kThreads / 32) - 1) / (kThreads / 32);
  if (blocks > blocks_needed) blocks = blocks_needed;
  if (blocks == 0) blocks = 1;
  k_trace<ANY, STACK><<<blocks, kThreads, 0, st>>>(S, reinterpret_cast<const float4*>(rays), n,
                                                   reinterpret_cast<uint2*>(hits), counter);
  return cudaGetLastError();
}

}  // namespace

int device_sm_count() {
  static int sms = -1;
  if (sms < 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) sms = 1;
  }
  return sms;
}

cudaError_t launch_trace(const DeviceScene& s, const RtRay* rays, uint32_t n, RtHit* hits, uint32_t flags,
                         uint32_t* counter, void* stream) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const bool any = (flags & RT_TRACE_ANY) != 0;
  if (s.depth < 64u) {
    return any ? launch_variant<true, 64>(s, rays, n, hits, counter, st)
               : launch_variant<false, 64>(s, rays, n, hits, counter, st);
  }
  return any ? launch_variant<true, 128>(s, rays, n, hits, counter, st)
             : launch_variant<false, 128>(s, rays, n, hits, counter, st);
}

}  // namespace rtgb
