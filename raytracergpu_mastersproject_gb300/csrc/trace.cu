// trace.cu -- ray-query kernels (closest hit / any hit) for sm_103a.
//
// Replaces hitBVH/sceneHit (raytraceBVH.comp:195-274) for batches of
// independent rays.  Persistent warps: each warp takes rays 32 at a time from
// a global counter (one atomicAdd per refill), traverses them with the
// near-first while-while loop of trace_core.cuh, and hands new rays to lanes
// that finished whenever fewer than kRefill lanes are still busy.
#include <cuda_runtime.h>

#include <mutex>

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

// ---- allocation-free ray queries (rt_trace_noalloc) ----
// Scratch of rt_trace_noalloc: word 0 is the persistent kernel's ray-queue
// counter, word 1 a status word.  Every device that loads the library holds
// this array until the process exits; all calls share it.
static __device__ __align__(256) uint32_t g_noalloc_scratch[RT_NOALLOC_SCRATCH_BYTES / sizeof(uint32_t)];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
uint32_t* g_noalloc_ptr[kMaxDevices] = {};
}  // namespace

const DeviceScene* scene_device(const rt_scene* scene);
void set_error(const std::string& msg);

}  // namespace rtgb

extern "C" rt_status rt_trace_noalloc(rt_scene* scene, const RtRay* d_rays, uint32_t n, RtHit* d_hits,
                                      uint32_t flags, void* stream) {
  using namespace rtgb;
  if (!scene || (n && (!d_rays || !d_hits)) || flags > RT_TRACE_ANY) {
    set_error("rt_trace_noalloc: bad argument");
    return RT_EINVAL;
  }
  if (n > RT_NOALLOC_MAX_RAYS) {
    set_error("rt_trace_noalloc: " + std::to_string(n) + " rays exceed the maximum of " +
              std::to_string(RT_NOALLOC_MAX_RAYS) + " per call (the scratch ray-queue counter is 32-bit)");
    return RT_EINVAL;
  }
  if (n == 0) return RT_OK;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_error(std::string("rt_trace_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
    return RT_ECUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("rt_trace_noalloc: device ordinal above 63");
    return RT_EINVAL;
  }
  uint32_t* scratch = nullptr;
  {
    // Set-up, once per device, with that device current: the host-side name
    // g_noalloc_scratch is not a device address, so resolve the symbol.
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        set_error(std::string("rt_trace_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        return RT_ECUDA;
      }
      g_noalloc_ptr[dev] = static_cast<uint32_t*>(p);
    }
    scratch = g_noalloc_ptr[dev];
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  // The array keeps the previous call's contents: the queue counter and the
  // status word must start at zero.
  e = cudaMemsetAsync(scratch, 0, 2 * sizeof(uint32_t), st);
  if (e != cudaSuccess) {
    set_error(std::string("rt_trace_noalloc: memset: ") + cudaGetErrorString(e));
    return RT_ECUDA;
  }
  e = launch_trace(*scene_device(scene), d_rays, n, d_hits, flags, scratch, stream);
  if (e != cudaSuccess) {
    set_error(std::string("rt_trace_noalloc: launch: ") + cudaGetErrorString(e));
    return RT_ECUDA;
  }
  return RT_OK;
}
