// trace.cu -- ray-query kernels (closest hit / any hit) for sm_103a.
//
// Replaces hitBVH/sceneHit (raytraceBVH.comp:195-274) for batches of
// independent rays.  Persistent warps take rays from a global counter (one
// atomicAdd per refill, indices handed out with __ballot_sync/__popc/
// __shfl_sync).  Two loop shapes:
//   k_trace       near-first while-while loop with postponed leaves (binary
//                 and 4-wide trees); idle lanes are refilled when fewer than
//                 `refill` lanes still traverse.
//   k_trace_step  4-wide trees: one traversal step per lane per iteration and
//                 refill as soon as `refill` lanes are idle (the default, with
//                 the top 16 stack entries of each lane in shared memory).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <type_traits>

#include "trace_core.cuh"

namespace rtgb {
namespace {

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// THREADS per block and MINB resident blocks per SM (the register cap) are
// launch-shape knobs; `refill` is the lane count below which a warp stops to
// hand new rays to its idle lanes (0: only when all lanes are idle).
template <bool ANY, int STACK, int THREADS, int MINB, int W, bool STATS, bool MT = false>
__global__ void __launch_bounds__(THREADS, MINB)
    k_trace(DeviceScene S, const float4* __restrict__ rays, uint32_t n, uint2* __restrict__ hits,
            uint32_t* __restrict__ counter, int refill, unsigned long long* __restrict__ stats,
            const uint32_t* __restrict__ order) {
  using StackT = typename std::conditional<W == 2, uint32_t, uint2>::type;
  StackT stack[STACK];
  dev::Trav s;
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t ray = 0xFFFFFFFFu;
  bool exhausted = false;
  unsigned long long vis = 0, tests = 0;
  const bool rays_al32 = dev::aligned32(rays);
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
          ray = order ? __ldg(&order[id]) : id;
          if (dev::chk(S.check, ray >= n, dev::kChkRay, ray)) {
            ray = 0xFFFFFFFFu;
          } else {
            float4 ro, rd;
            dev::load_ray(rays, ray, rays_al32, ro, rd);
            dev::trav_init_ray(s, ro, rd, S.root);
            if constexpr (W == 2) stack[0] = kSentinel;
          }
        }
      }
    }
    if (__all_sync(0xFFFFFFFFu, ray == 0xFFFFFFFFu)) break;
    if (ray != 0xFFFFFFFFu) {
      bool done;
      if constexpr (W == 2)
        done = dev::trav_run<ANY, STACK, MT>(S, s, stack, exhausted ? 0 : refill);
      else
        done = dev::trav_run_wide<ANY, STACK>(S, s, stack, exhausted ? 0 : refill);
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
        __stcs(&hits[ray], h);
        if constexpr (STATS) {
          vis += s.nvis;
          tests += s.ntest;
        }
        ray = 0xFFFFFFFFu;
      }
    }
  }
  if constexpr (STATS) {
    for (int o = 16; o > 0; o >>= 1) {
      vis += __shfl_down_sync(0xFFFFFFFFu, vis, o);
      tests += __shfl_down_sync(0xFFFFFFFFu, tests, o);
    }
    if (lane == 0) {
      atomicAdd(&stats[0], vis);
      atomicAdd(&stats[1], tests);
    }
  }
}

// Per-step variant for 4-wide trees: every iteration each lane advances its
// ray by one step -- one inner node, then the leaf that node led to if any,
// or one leaf -- and lanes whose ray finished take new rays as soon as
// `refill` of them are idle.  The heavy inner-node step then runs with nearly
// all lanes active.  Some lane needs the leaf code in nearly every iteration,
// so a lane that reaches a leaf tests it at once instead of in an iteration
// of its own (config 3: 14.2 -> 13.4 ms).
//
// RAW (the path tracer's queries): n == 0xFFFFFFFF reads the ray count from
// counter[2], written by the kernel that produced the rays; each hit is the
// traversal's own result -- the leaf-style ref of the closest primitive (0:
// none, kRawOverflow: stack overflow) and t -- so that shading needs no id map.
//
// RING > 0 keeps the top RING stack entries of each lane in shared memory
// (RING * THREADS * 4 bytes per block: refs only), the rest in local memory.
//
// TILE > 0 stages the tree's first TILE nodes -- its top levels, numbered
// first in breadth-first order -- in shared memory per block (plain loads at
// block start), and node visits read them from there.
//
// VISITS > 1 makes up to VISITS node visits per iteration (the later ones
// for lanes still at an inner node) before the leaf step: fewer iterations,
// so the leaf code, which some lane needs in nearly every iteration, and the
// loop's own work run less often (four is the default: config 3 13.24 ->
// 11.78 ms per step against one).
template <bool ANY, int STACK, int THREADS, int MINB, bool STATS, bool RAW = false, int RING = 0, bool MT = false,
          int TILE = 0, int VISITS = 1>
__global__ void __launch_bounds__(THREADS, MINB)
    k_trace_step(DeviceScene S, const float4* __restrict__ rays, uint32_t n, uint2* __restrict__ hits,
                 uint32_t* __restrict__ counter, int refill, unsigned long long* __restrict__ stats,
            const uint32_t* __restrict__ order) {
  dev::StepEntry stack[STACK];
  using Stk = typename std::conditional<(RING > 0), dev::RingStack<(RING > 0 ? RING : 1), THREADS, dev::StepEntry>,
                                        dev::LocalStackT<dev::StepEntry>>::type;
  Stk stk;
  if constexpr (RING > 0) {
    __shared__ dev::StepEntry ring[RING * THREADS];
    stk.ring = ring + threadIdx.x;
    stk.spill = stack;
    stk.lo = 0;
  } else {
    stk.a = stack;
  }
  using Fetch = typename std::conditional<(TILE > 0), dev::TiledNodes<(TILE > 0 ? TILE : 1)>, dev::GlobalNodes>::type;
  Fetch fetch;
  if constexpr (TILE > 0) {
    __shared__ float4 tile[4 * TILE];
    // node indices are below n_inner, so slots at and past it are never read
    const uint32_t words = 4u * min((uint32_t)TILE, S.n_inner);
    for (uint32_t i = threadIdx.x; i < words; i += THREADS) tile[i] = dev::ldg4(S.inner, i);
    __syncthreads();
    fetch.tile = tile;
    fetch.base = 0u;
  }
  dev::Trav s;
  const uint32_t lane = threadIdx.x & 31u;
  if (RAW && n == 0xFFFFFFFFu) n = *reinterpret_cast<volatile uint32_t*>(counter + 2);
  uint32_t ray = 0xFFFFFFFFu;
  bool exhausted = false;
  unsigned long long vis = 0, tests = 0;
  const int min_idle = refill < 1 ? 1 : (refill > 32 ? 32 : refill);
  const bool rays_al32 = dev::aligned32(rays);
  for (;;) {
    const uint32_t idle = __ballot_sync(0xFFFFFFFFu, ray == 0xFFFFFFFFu);
    if (exhausted && idle == 0xFFFFFFFFu) break;
    if (!exhausted && __popc(idle) >= min_idle) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(counter, (uint32_t)__popc(idle));
      base = __shfl_sync(0xFFFFFFFFu, base, 0);
      if (base + (uint32_t)__popc(idle) >= n) exhausted = true;
      if (ray == 0xFFFFFFFFu) {
        const uint32_t id = base + (uint32_t)__popc(idle & lanemask_lt());
        if (id < n && !dev::chk(S.check, order && __ldg(&order[id]) >= n, dev::kChkRay, order ? __ldg(&order[id]) : id)) {
          ray = order ? __ldg(&order[id]) : id;
          float4 ro, rd;
          dev::load_ray(rays, ray, rays_al32, ro, rd);
          dev::trav_init_ray(s, ro, rd, S.root);
          stk.reset();
          if (s.leaf != 0u) {  // the whole tree is one leaf
            s.node = s.leaf;
            s.leaf = 0u;
          }
        }
      }
    }
    if (ray == 0xFFFFFFFFu) continue;
    bool done = false;
    // a node visit, then in the same iteration the leaf it led to (the warp
    // runs the leaf code in nearly every iteration for some lane anyway)
    if (dev::is_inner(s.node)) {
      if (!dev::visit_wide_stk<STACK>(S, s, stk, fetch)) done = true;
    }
#pragma unroll
    for (int v = 1; v < VISITS; ++v) {
      if (!done && dev::is_inner(s.node)) {
        if (!dev::visit_wide_stk<STACK>(S, s, stk, fetch)) done = true;
      }
    }
    if (!done && dev::is_leaf(s.node)) {
      if (dev::leaf_visit<ANY, MT>(S, s, s.node))
        done = true;
      else
        s.node = stk.pop(s);
    }
    if (done || s.node == kSentinel) {
      uint2 h;
      if (RAW) {
        h.x = s.sp < 0 ? kRawOverflow : s.best;
        h.y = __float_as_uint(s.tclose);
      } else if (s.sp < 0 || s.best == dev::kNoBest) {
        h.x = RT_NO_HIT;
        h.y = __float_as_uint(__int_as_float(0x7f800000));
      } else if (s.best & kSphereBit) {
        h.x = (s.best & kSphereMask) | RT_HIT_SPHERE_BIT;
        h.y = __float_as_uint(s.tclose);
      } else {
        h.x = __ldg(&S.tri_ids[s.best & kSlotMask]);
        h.y = __float_as_uint(s.tclose);
      }
      if (RAW)
        hits[ray] = h;  // read back by the shading kernel next
      else
        __stcs(&hits[ray], h);  // written once: evict-first
      if constexpr (STATS) {
        vis += s.nvis;
        tests += s.ntest;
      }
      ray = 0xFFFFFFFFu;
    }
  }
  if constexpr (STATS) {
    for (int o = 16; o > 0; o >>= 1) {
      vis += __shfl_down_sync(0xFFFFFFFFu, vis, o);
      tests += __shfl_down_sync(0xFFFFFFFFu, tests, o);
    }
    if (lane == 0) {
      atomicAdd(&stats[0], vis);
      atomicAdd(&stats[1], tests);
    }
  }
}

using TraceKernel = void (*)(DeviceScene, const float4*, uint32_t, uint2*, uint32_t*, int, unsigned long long*,
                             const uint32_t*);

// Stack capacities: binary trees 64 or 128 refs (depth + sentinel); 4-wide
// trees 64 or 192 entries (worst-case pushes along a path; (ref, t_near) in
// the while-while loop, the ref alone in the step loop).
struct Variant {
  int threads, minb;
  TraceKernel k[2][2][2][2];  // [stats][wide][any][big stack]
  int blocks_per_sm[2][2][2][2];
};

template <int T, int M, bool ST>
void fill_variant(Variant& v) {
  v.k[ST][0][0][0] = k_trace<false, 64, T, M, 2, ST>;
  v.k[ST][0][0][1] = k_trace<false, 128, T, M, 2, ST>;
  v.k[ST][0][1][0] = k_trace<true, 64, T, M, 2, ST>;
  v.k[ST][0][1][1] = k_trace<true, 128, T, M, 2, ST>;
  v.k[ST][1][0][0] = k_trace<false, 64, T, M, 4, ST>;
  v.k[ST][1][0][1] = k_trace<false, 192, T, M, 4, ST>;
  v.k[ST][1][1][0] = k_trace<true, 64, T, M, 4, ST>;
  v.k[ST][1][1][1] = k_trace<true, 192, T, M, 4, ST>;
}

template <int T, int M, bool ST, int RING, int VISITS>
void fill_step_variant(Variant& v) {
  fill_variant<T, M, ST>(v);  // binary trees keep the while-while loop
  v.k[ST][1][0][0] = k_trace_step<false, 64, T, M, ST, false, RING, false, 0, VISITS>;
  v.k[ST][1][0][1] = k_trace_step<false, 192, T, M, ST, false, RING, false, 0, VISITS>;
  v.k[ST][1][1][0] = k_trace_step<true, 64, T, M, ST, false, RING, false, 0, VISITS>;
  v.k[ST][1][1][1] = k_trace_step<true, 192, T, M, ST, false, RING, false, 0, VISITS>;
}

template <int T, int M, bool STEP, int RING = 0, int VISITS = 1>
Variant make_variant() {
  Variant v;
  v.threads = T;
  v.minb = M;
  if constexpr (STEP) {
    fill_step_variant<T, M, false, RING, VISITS>(v);
    fill_step_variant<T, M, true, RING, VISITS>(v);
  } else {
    fill_variant<T, M, false>(v);
    fill_variant<T, M, true>(v);
  }
  for (auto& a : v.blocks_per_sm)
    for (auto& b : a)
      for (auto& c : b)
        for (int& d : c) d = -1;
  return v;
}

// Launch shapes (RT_TRACE_VARIANT selects one; RT_TRACE_REFILL sets the refill
// threshold): 0-2 while-while loop at 12 / 10 / 1 blocks per SM, 3-5 step
// loop with the stack in local memory, 6 step loop at 10 blocks of 128
// threads with a 16-entry shared ring, 7 the same as 5 blocks of 256; 8-9,
// 10-11 and 12-13 are the shapes of 6 and 7 with up to two, three and four
// node visits per iteration; 14-15 the four-visit shapes with the whole
// stack in local memory (no ring: all of L1 stays cache).  12 is the default
// (config 3: 11.78 ms per step against 13.24 with one visit; six and eight
// visits were slower again).
// Binary trees always use the while-while loop of the chosen shape.
Variant g_variants[] = {make_variant<128, 12, false>(), make_variant<128, 10, false>(), make_variant<128, 1, false>(),
                        make_variant<128, 12, true>(),  make_variant<128, 10, true>(),  make_variant<128, 1, true>(),
                        make_variant<128, 10, true, 16>(), make_variant<256, 5, true, 16>(),
                        make_variant<128, 10, true, 16, 2>(), make_variant<256, 5, true, 16, 2>(),
                        make_variant<128, 10, true, 16, 3>(), make_variant<256, 5, true, 16, 3>(),
                        make_variant<128, 10, true, 16, 4>(), make_variant<256, 5, true, 16, 4>(),
                        make_variant<128, 10, true, 0, 4>(), make_variant<256, 5, true, 0, 4>()};
constexpr int kNumVariants = sizeof(g_variants) / sizeof(g_variants[0]);

// RT_TRACE_MT: the Moller-Trumbore leaf test in the default launch shape (the
// step loop with the shared ring for 4-wide trees, the while-while loop for
// binary ones), 128 threads x 10 blocks.  [wide][any][big stack]
struct MtKernels {
  TraceKernel k[2][2][2];
  int blocks_per_sm[2][2][2];
};
MtKernels g_mt = {{{{k_trace<false, 64, 128, 10, 2, false, true>, k_trace<false, 128, 128, 10, 2, false, true>},
                    {k_trace<true, 64, 128, 10, 2, false, true>, k_trace<true, 128, 128, 10, 2, false, true>}},
                   {{k_trace_step<false, 64, 128, 10, false, false, 16, true, 0, kDefaultVisits>,
                     k_trace_step<false, 192, 128, 10, false, false, 16, true, 0, kDefaultVisits>},
                    {k_trace_step<true, 64, 128, 10, false, false, 16, true, 0, kDefaultVisits>,
                     k_trace_step<true, 192, 128, 10, false, false, 16, true, 0, kDefaultVisits>}}},
                  {{{-1, -1}, {-1, -1}}, {{-1, -1}, {-1, -1}}}};

// The default launch shape (128 threads, 10 blocks per SM, 16-entry shared
// ring, four node visits per iteration) at every tuned stack capacity and
// staging tile (closest and any hit):
// [any][kTunedStacks index][kTunedTiles index].
template <bool ANY, int STACK>
void fill_tuned_row(TraceKernel* row) {
  row[0] = k_trace_step<ANY, STACK, 128, 10, false, false, 16, false, 0, kDefaultVisits>;
  row[1] = k_trace_step<ANY, STACK, 128, 10, false, false, 16, false, 16, kDefaultVisits>;
  row[2] = k_trace_step<ANY, STACK, 128, 10, false, false, 16, false, 64, kDefaultVisits>;
}
struct TunedKernels {
  TraceKernel k[2][4][3];
  int bps[2][4][3];
  TunedKernels() {
    fill_tuned_row<false, 48>(k[0][0]);
    fill_tuned_row<false, 64>(k[0][1]);
    fill_tuned_row<false, 96>(k[0][2]);
    fill_tuned_row<false, 192>(k[0][3]);
    fill_tuned_row<true, 48>(k[1][0]);
    fill_tuned_row<true, 64>(k[1][1]);
    fill_tuned_row<true, 96>(k[1][2]);
    fill_tuned_row<true, 192>(k[1][3]);
    for (auto& a : bps)
      for (auto& b : a)
        for (int& c : b) c = -1;
  }
};
TunedKernels g_tuned;

int tuned_index(const int* table, int n, int v) {
  for (int i = 0; i < n; ++i)
    if (table[i] == v) return i;
  return -1;
}

int env_int(const char* name, int dflt) {
  const char* e = std::getenv(name);
  return e ? std::atoi(e) : dflt;
}

}  // namespace

TraceTuning default_tuning() {
  static TraceTuning t = [] {
    TraceTuning d;
    d.variant = env_int("RT_TRACE_VARIANT", kTunedVariant);
    d.refill = env_int("RT_TRACE_REFILL", 5);
    d.grid_scale = env_int("RT_TRACE_GRID_PCT", 100);
    return d;
  }();
  return t;
}

int num_trace_variants() { return kNumVariants; }

bool tuning_supported(const TraceTuning& t, uint32_t width, uint32_t stack_need, uint32_t flags) {
  if (t.variant < 0 || t.variant >= kNumVariants || t.refill < 0 || t.refill > 32) return false;
  if (t.stack == 0 && t.tile == 0) return true;
  if (t.variant != kTunedVariant || width != 4 || (flags & RT_TRACE_MT)) return false;
  const int si = t.stack == 0 ? (stack_need > 64u ? 3 : 1) : tuned_index(kTunedStacks, 4, t.stack);
  return si >= 0 && tuned_index(kTunedTiles, 3, t.tile) >= 0 && (uint32_t)kTunedStacks[si] >= stack_need;
}
void trace_variant_shape(int v, int* threads, int* minb) {
  *threads = g_variants[v].threads;
  *minb = g_variants[v].minb;
}

cudaError_t launch_trace_tuned(const DeviceScene& S, const RtRay* rays, uint32_t n, RtHit* hits, uint32_t flags,
                               uint32_t* counter, void* stream, const TraceTuning& tune, unsigned long long* stats,
                               const uint32_t* order) {
  const int vi = (tune.variant >= 0 && tune.variant < kNumVariants) ? tune.variant : 0;
  Variant& v = g_variants[vi];
  const int any = (flags & RT_TRACE_ANY) != 0 ? 1 : 0;  // RT_TRACE_SORT is handled by the caller
  const int wide = S.width == 4 ? 1 : 0;
  const int big = S.stack_need > 64u ? 1 : 0;
  const int st = stats ? 1 : 0;
  const bool mt = (flags & RT_TRACE_MT) != 0;
  if (mt && stats) return cudaErrorInvalidValue;  // no counting instantiation of the MT test
  TraceKernel k = mt ? g_mt.k[wide][any][big] : v.k[st][wide][any][big];
  const int threads = mt ? 128 : v.threads;
  int* slot = mt ? &g_mt.blocks_per_sm[wide][any][big] : &v.blocks_per_sm[st][wide][any][big];
  if (!stats && (tune.stack != 0 || tune.tile != 0)) {
    if (!tuning_supported(tune, S.width, S.stack_need, flags)) return cudaErrorInvalidValue;
    const int si = tune.stack == 0 ? (big ? 3 : 1) : tuned_index(kTunedStacks, 4, tune.stack);
    const int ti = tuned_index(kTunedTiles, 3, tune.tile);
    k = g_tuned.k[any][si][ti];
    slot = &g_tuned.bps[any][si][ti];
  }
  int bps = 0;
  if (cudaError_t e = cached_blocks_per_sm(slot, k, threads, &bps); e != cudaSuccess) return e;
  const uint32_t warps_per_block = (uint32_t)threads / 32u;
  const uint32_t warps_needed = (n + 31u) / 32u;
  uint64_t blocks = (uint64_t)device_sm_count() * (uint64_t)bps * (uint64_t)std::max(1, tune.grid_scale) / 100u;
  const uint64_t needed = (warps_needed + warps_per_block - 1) / warps_per_block;
  if (blocks > needed) blocks = needed;
  if (blocks == 0) blocks = 1;
  k<<<(uint32_t)blocks, threads, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      S, reinterpret_cast<const float4*>(rays), n, reinterpret_cast<uint2*>(hits), counter, tune.refill, stats, order);
  return cudaGetLastError();
}

int device_sm_count() {
  static int cached = -1;
  int sms = __atomic_load_n(&cached, __ATOMIC_RELAXED);
  if (sms < 1) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) sms = 1;
    __atomic_store_n(&cached, sms, __ATOMIC_RELAXED);
  }
  return sms;
}

cudaError_t launch_trace(const DeviceScene& s, const RtRay* rays, uint32_t n, RtHit* hits, uint32_t flags,
                         uint32_t* counter, void* stream, const uint32_t* order) {
  return launch_trace_tuned(s, rays, n, hits, flags, counter, stream, default_tuning(), nullptr, order);
}

cudaError_t launch_trace_raw(const DeviceScene& S, const float4* rays, uint32_t n, uint2* hits, uint32_t* counter,
                             unsigned long long* stats, cudaStream_t st) {
  constexpr int T = 128, M = 10, R = 16;  // the default ray-query shape
  const bool big = S.stack_need > 64u;
  // node visits per iteration of the bounce queries (RT_TRACE_RAW_VISITS, 1-4)
  // (config 2 extended: 3.44 against 3.51 ms per frame with two than one)
  static const int visits = std::min(4, std::max(1, env_int("RT_TRACE_RAW_VISITS", 2)));
  const int k = (big ? 1 : 0) | (stats ? 2 : 0) | ((visits - 1) << 2);
  static int bps[16] = {-1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1};
  static const TraceKernel table[16] = {
      k_trace_step<false, 64, T, M, false, true, R>,         k_trace_step<false, 192, T, M, false, true, R>,
      k_trace_step<false, 64, T, M, true, true, R>,          k_trace_step<false, 192, T, M, true, true, R>,
      k_trace_step<false, 64, T, M, false, true, R, false, 0, 2>, k_trace_step<false, 192, T, M, false, true, R, false, 0, 2>,
      k_trace_step<false, 64, T, M, true, true, R, false, 0, 2>,  k_trace_step<false, 192, T, M, true, true, R, false, 0, 2>,
      k_trace_step<false, 64, T, M, false, true, R, false, 0, 3>, k_trace_step<false, 192, T, M, false, true, R, false, 0, 3>,
      k_trace_step<false, 64, T, M, true, true, R, false, 0, 3>,  k_trace_step<false, 192, T, M, true, true, R, false, 0, 3>,
      k_trace_step<false, 64, T, M, false, true, R, false, 0, 4>, k_trace_step<false, 192, T, M, false, true, R, false, 0, 4>,
      k_trace_step<false, 64, T, M, true, true, R, false, 0, 4>,  k_trace_step<false, 192, T, M, true, true, R, false, 0, 4>};
  TraceKernel kern = table[k];
  int per_sm = 0;
  if (cudaError_t e = cached_blocks_per_sm(&bps[k], kern, T, &per_sm); e != cudaSuccess) return e;
  uint64_t blocks = (uint64_t)device_sm_count() * (uint64_t)per_sm;
  if (n != 0xFFFFFFFFu) blocks = std::min<uint64_t>(blocks, ((uint64_t)n + T - 1) / T);
  if (blocks == 0) blocks = 1;
  // The path tracer's bounce rays are short: refilling at 8 idle lanes beats
  // 4 there (config 2: 3.49 against 3.53 ms per frame).
  static const int refill = env_int("RT_TRACE_RAW_REFILL", 8);
  kern<<<(uint32_t)blocks, T, 0, st>>>(S, rays, n, hits, counter, refill, stats, nullptr);
  return cudaGetLastError();
}

// ---- allocation-free ray queries (rt_trace_noalloc) ----
// Scratch of rt_trace_noalloc: word 0 is the persistent kernel's ray-queue
// counter; the rest of the array is unused.  Every device that loads the
// library holds this array until the process exits; all calls share it.
static __device__ __align__(256) uint32_t g_noalloc_scratch[RT_NOALLOC_SCRATCH_BYTES / sizeof(uint32_t)];

const DeviceScene* scene_device(const rt_scene* scene);
void set_error(const std::string& msg);

}  // namespace rtgb

extern "C" rt_status rt_trace_noalloc(rt_scene* scene, const RtRay* d_rays, uint32_t n, RtHit* d_hits,
                                      uint32_t flags, void* stream) {
  rtgb::NvtxRange nvtx_range("rt_trace_noalloc");
  using namespace rtgb;
  if (!scene || (n && (!d_rays || !d_hits)) || (flags & ~(uint32_t)(RT_TRACE_ANY | RT_TRACE_MT)) ||
      (reinterpret_cast<uintptr_t>(d_rays) & 15u) != 0u || (reinterpret_cast<uintptr_t>(d_hits) & 7u) != 0u) {
    set_error("rt_trace_noalloc: bad argument (rays must be 16-byte aligned, hits 8-byte aligned)");
    return RT_EINVAL;
  }
  if (n > RT_NOALLOC_MAX_RAYS) {
    set_error("rt_trace_noalloc: " + std::to_string(n) + " rays exceed the maximum of " +
              std::to_string(RT_NOALLOC_MAX_RAYS) + " per call (the scratch ray-queue counter is 32-bit)");
    return RT_EINVAL;
  }
  if (n == 0) return RT_OK;
  // The host-side name g_noalloc_scratch is not a device address: resolve
  // the symbol on the current device, every call (no cached address can go
  // stale when a context is torn down and rebuilt; no allocation either).
  uint32_t* scratch = nullptr;
  cudaError_t e;
  {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      set_error(std::string("rt_trace_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      return RT_ECUDA;
    }
    scratch = static_cast<uint32_t*>(p);
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  // The array keeps the previous call's contents: the queue counter must
  // start at zero.
  e = cudaMemsetAsync(scratch, 0, sizeof(uint32_t), st);
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
