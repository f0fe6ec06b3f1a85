// pool.cu -- resident scenes in one device arena, traced together.
//
// The batched form of rt_trace: many scenes of uneven size, each with its own
// ray batch, traced by one persistent launch that takes rays from a single
// queue spanning every job.  All scenes of a pool live in one arena -- one
// array of 4-wide inner nodes, one of triangle records, one of triangle ids --
// and their child refs are rebased at upload, so a ray only needs its scene's
// root ref; nothing else in the traversal depends on the scene.
//
// Arena ranges are handed out first-fit from free lists and the arrays grow by
// doubling; refs are indices, so growing (copy to a larger array) keeps them
// valid.  Scene bytes are accounted against a budget (admission control).
// Per stream, two launch slots alternate: each holds a pinned job table, its
// device copy and a captured CUDA graph (table upload, queue reset, kernel).
#include <cuda_runtime.h>

#include <type_traits>

#include <chrono>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <unordered_map>

#include "trace_core.cuh"

namespace rtgb {

void set_error(const std::string& msg);
rt_status device_build_to_host(const RtTriangle64* tris, uint32_t nt, const RtSphere32* sph, uint32_t ns,
                               uint32_t mode, std::vector<RtBVHNode40>& out);

namespace {

struct DJob {
  const float4* rays;
  uint2* hits;
  uint32_t start;
  uint32_t count;
  uint32_t root;
  uint32_t nodes;  // the scene's 4-wide nodes [root, root + nodes) in the arena
};
static_assert(sizeof(DJob) == 32, "job record is 32 bytes");

// Table: header (num_jobs, total, 6 pad words) then the jobs.
constexpr uint32_t kMaxJobs = 8192;
constexpr size_t kTableBytes = sizeof(DJob) * (kMaxJobs + 1);

__device__ __forceinline__ uint32_t lanemask_lt_p() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ uint32_t find_job(const DJob* __restrict__ jobs, uint32_t num, uint32_t g) {
  uint32_t lo = 0, hi = num;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(&jobs[mid].start) <= g) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Jobs whose scenes' top nodes a block can stage (TILE > 0); batches with
// more jobs run without the tile.
constexpr uint32_t kTileJobs = 256;

// Node fetch of k_pool_step with a staged tile: the first `count` nodes of the
// lane's scene, [base, base + count), from shared memory.
struct PoolTiledNodes {
  const float4* tile;
  uint32_t base, count;
  __device__ __forceinline__ void operator()(const DeviceScene& S, uint32_t node, float4& h, float4& r, float4& qa,
                                             float4& qb) const {
    const uint32_t i = node - base;
    if (i < count) {
      h = tile[4u * i + 0u];
      r = tile[4u * i + 1u];
      qa = tile[4u * i + 2u];
      qb = tile[4u * i + 3u];
    } else {
      dev::GlobalNodes()(S, node, h, r, qa, qb);
    }
  }
};

// k_trace_step over a job table (see trace.cu): each lane keeps (job, local
// ray index) and its job's root; hits go to the job's own hit array.
// RING > 0: the top RING stack entries of each lane in shared memory (see
// dev::RingStack).  TILE > 0: each block stages the first TILE nodes of
// every job's scene -- its top levels, which the builder numbers first in
// breadth-first order -- in shared memory (plain loads at block start), when
// the batch has at most kTileJobs jobs.
// VISITS > 1: up to VISITS node visits per iteration before the leaf step
// (see k_trace_step).
template <bool ANY, int STACK, int THREADS, int MINB, int RING, int TILE = 0, int VISITS = 1>
__global__ void __launch_bounds__(THREADS, MINB)
    k_pool_step(DeviceScene S, const DJob* __restrict__ table, uint32_t* __restrict__ counter, int refill) {
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
  dev::Trav s;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t num_jobs = __ldg(reinterpret_cast<const uint32_t*>(table));
  const uint32_t total = __ldg(reinterpret_cast<const uint32_t*>(table) + 1);
  const DJob* jobs = table + 1;
  using Fetch = typename std::conditional<(TILE > 0), PoolTiledNodes, dev::GlobalNodes>::type;
  Fetch fetch;
  [[maybe_unused]] const float4* tile_base = nullptr;
  [[maybe_unused]] const bool tiled = TILE > 0 && num_jobs <= kTileJobs;
  if constexpr (TILE > 0) {
    __shared__ float4 tile[kTileJobs * TILE * 4];
    if (tiled) {
      for (uint32_t i = threadIdx.x; i < num_jobs * TILE * 4u; i += THREADS) {
        const uint32_t j = i / (TILE * 4u), w = i % (TILE * 4u);
        const uint32_t root = __ldg(&jobs[j].root), nn = __ldg(&jobs[j].nodes);
        if (root < kSentinel && w / 4u < nn) tile[i] = dev::ldg4(S.inner, 4u * root + w);
      }
    }
    __syncthreads();
    tile_base = tile;
    fetch.tile = tile;
    fetch.base = 0u;
    fetch.count = 0u;
  }
  uint32_t job = 0, local = 0xFFFFFFFFu;
  bool exhausted = total == 0;
  const int min_idle = refill < 1 ? 1 : (refill > 32 ? 32 : refill);
  for (;;) {
    const uint32_t idle = __ballot_sync(0xFFFFFFFFu, local == 0xFFFFFFFFu);
    if (exhausted && idle == 0xFFFFFFFFu) break;
    if (!exhausted && __popc(idle) >= min_idle) {
      // One binary search per refill, for the first ray handed out; the
      // warp's other new rays follow it in the queue, so each lane walks on
      // from that job (jobs hold thousands of rays: rarely a step, and
      // never more than 8 before it searches for itself).
      uint32_t base = 0, first_job = 0;
      if (lane == 0) {
        base = atomicAdd(counter, (uint32_t)__popc(idle));
        if (base < total) first_job = find_job(jobs, num_jobs, base);
      }
      base = __shfl_sync(0xFFFFFFFFu, base, 0);
      first_job = __shfl_sync(0xFFFFFFFFu, first_job, 0);
      if (base + (uint32_t)__popc(idle) >= total) exhausted = true;
      if (local == 0xFFFFFFFFu) {
        const uint32_t g = base + (uint32_t)__popc(idle & lanemask_lt_p());
        if (g < total) {
          job = first_job;
          for (int k = 0; job + 1u < num_jobs && __ldg(&jobs[job + 1u].start) <= g; ++k) {
            if (k == 8) {
              job = find_job(jobs, num_jobs, g);
              break;
            }
            ++job;
          }
          local = g - __ldg(&jobs[job].start);
          const float4* rays = jobs[job].rays;
          const uint32_t root = __ldg(&jobs[job].root);
          float4 ro, rd;
          dev::load_ray(rays, local, dev::aligned32(rays), ro, rd);
          dev::trav_init_ray(s, ro, rd, root);
          if constexpr (TILE > 0) {
            fetch.tile = tile_base + 4u * TILE * job;
            fetch.base = root;
            fetch.count = tiled && root < kSentinel ? min((uint32_t)TILE, __ldg(&jobs[job].nodes)) : 0u;
          }
          stk.reset();
          if (s.leaf != 0u) {
            s.node = s.leaf;
            s.leaf = 0u;
          }
        }
      }
    }
    if (local == 0xFFFFFFFFu) continue;
    bool done = false;
    // a node visit, then in the same iteration the leaf it led to
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
      if (dev::leaf_visit<ANY>(S, s, s.node))
        done = true;
      else
        s.node = stk.pop(s);
    }
    if (done || s.node == kSentinel) {
      uint2 h;
      if (s.sp < 0 || s.best == dev::kNoBest) {
        h.x = RT_NO_HIT;
        h.y = __float_as_uint(__int_as_float(0x7f800000));
      } else {
        h.x = __ldg(&S.tri_ids[s.best & kSlotMask]);
        h.y = __float_as_uint(s.tclose);
      }
      __stcs(&jobs[job].hits[local], h);  // written once: evict-first
      local = 0xFFFFFFFFu;
    }
  }
}

using PoolKernel = void (*)(DeviceScene, const DJob*, uint32_t*, int);

struct PoolVariant {
  int threads, minb, ring;
  PoolKernel k[2][2];  // [any][stack 192]
  int bps[2][2];
};

template <int T, int M, int R, int V = 1>
PoolVariant make_pool_variant() {
  PoolVariant v{T, M, R, {{k_pool_step<false, 64, T, M, R, 0, V>, k_pool_step<false, 192, T, M, R, 0, V>},
                          {k_pool_step<true, 64, T, M, R, 0, V>, k_pool_step<true, 192, T, M, R, 0, V>}},
                {{-1, -1}, {-1, -1}}};
  return v;
}

// Variants 5 and 6 are the shapes of 0 and 3 with up to four node visits
// per iteration; 5 is the default before rt_pool_autotune.
PoolVariant g_pool_variants[] = {make_pool_variant<128, 10, 16>(), make_pool_variant<256, 5, 16>(),
                                 make_pool_variant<128, 12, 0>(), make_pool_variant<128, 10, 0>(),
                                 make_pool_variant<256, 6, 0>(), make_pool_variant<128, 10, 16, kDefaultVisits>(),
                                 make_pool_variant<128, 10, 0, kDefaultVisits>()};
constexpr int kDefaultPoolVariant = 5;
constexpr int kNumPoolVariants = sizeof(g_pool_variants) / sizeof(g_pool_variants[0]);

// The tuner's further dimensions, on the two 128 x 10 shapes with four node
// visits per iteration (variant 5 with the 16-entry shared ring, variant 6
// with the stack in local memory): traversal stack capacity and the
// top-of-tree nodes staged per job.
constexpr int kPoolStacks[] = {48, 64, 96, 192};
constexpr int kPoolTiles[] = {0, 1, 2};
template <bool ANY, int STACK, int RING>
void fill_pool_tuned_row(PoolKernel* row) {
  row[0] = k_pool_step<ANY, STACK, 128, 10, RING, 0, kDefaultVisits>;
  row[1] = k_pool_step<ANY, STACK, 128, 10, RING, 1, kDefaultVisits>;
  row[2] = k_pool_step<ANY, STACK, 128, 10, RING, 2, kDefaultVisits>;
}
template <bool ANY, int RING>
void fill_pool_tuned_shape(PoolKernel (*rows)[3]) {
  fill_pool_tuned_row<ANY, 48, RING>(rows[0]);
  fill_pool_tuned_row<ANY, 64, RING>(rows[1]);
  fill_pool_tuned_row<ANY, 96, RING>(rows[2]);
  fill_pool_tuned_row<ANY, 192, RING>(rows[3]);
}
struct PoolTuned {
  PoolKernel k[2][2][4][3];  // [shape: variant 5, variant 6][any][stack][tile]
  int bps[2][2][4][3];
  PoolTuned() {
    fill_pool_tuned_shape<false, 16>(k[0][0]);
    fill_pool_tuned_shape<true, 16>(k[0][1]);
    fill_pool_tuned_shape<false, 0>(k[1][0]);
    fill_pool_tuned_shape<true, 0>(k[1][1]);
    for (auto& a : bps)
      for (auto& b : a)
        for (auto& c : b)
          for (int& d : c) d = -1;
  }
};
PoolTuned g_pool_tuned;

int pool_index(const int* table, int n, int v) {
  for (int i = 0; i < n; ++i)
    if (table[i] == v) return i;
  return -1;
}

// The kernel of (variant, stack, tile) or null when the pool cannot run it.
PoolKernel pool_kernel(int variant, int any, int big, int stack, int tile, uint32_t need, int** bps_slot,
                       int* threads) {
  if (variant < 0 || variant >= kNumPoolVariants) return nullptr;
  PoolVariant& v = g_pool_variants[variant];
  *threads = v.threads;
  if (stack == 0 && tile == 0) {
    *bps_slot = &v.bps[any][big];
    return v.k[any][big];
  }
  const int shape = variant == 5 ? 0 : (variant == 6 ? 1 : -1);
  const int si = stack == 0 ? (big ? 3 : 1) : pool_index(kPoolStacks, 4, stack);
  const int ti = pool_index(kPoolTiles, 3, tile);
  if (shape < 0 || si < 0 || ti < 0 || (uint32_t)kPoolStacks[si] < need) return nullptr;
  *bps_slot = &g_pool_tuned.bps[shape][any][si][ti];
  return g_pool_tuned.k[shape][any][si][ti];
}

// First-fit range allocator over [0, capacity) with coalescing frees.
class RangeAlloc {
 public:
  uint64_t capacity = 0;
  std::map<uint64_t, uint64_t> free_;  // offset -> size
  bool alloc(uint64_t n, uint64_t* off) {
    if (n == 0) {
      *off = 0;
      return true;
    }
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= n) {
        *off = it->first;
        const uint64_t rest = it->second - n, at = it->first + n;
        free_.erase(it);
        if (rest) free_[at] = rest;
        return true;
      }
    }
    return false;
  }
  void release(uint64_t off, uint64_t n) {
    if (n == 0) return;
    auto it = free_.emplace(off, n).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
  void grow(uint64_t new_cap) {  // adds [capacity, new_cap) as free
    const uint64_t old = capacity;
    capacity = new_cap;
    release(old, new_cap - old);
  }
};

}  // namespace

struct PoolScene {
  uint32_t root = kSentinel;
  uint64_t node_off = 0, node_cnt = 0;
  uint64_t tri_off = 0, tri_cnt = 0;
  uint64_t bytes = 0;
  uint32_t stack_need = 1;
  bool live = false;
};

struct LaunchSlot {
  DJob* host = nullptr;   // pinned
  DJob* dev = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  cudaEvent_t done = nullptr;
  bool used = false;
  // what the graph was captured with
  uint64_t generation = ~0ull;
  int variant = -1, any = -1, big = -1, refill = -1, stack = -1, tile = -1;
};

struct StreamState {
  uint32_t* counter = nullptr;
  LaunchSlot slot[2];
  int next = 0;
};

}  // namespace rtgb

struct rt_pool {
  std::mutex mu;
  uint64_t budget = 0;
  uint32_t max_scenes = 0;
  uint64_t used = 0;
  // arena
  float4* inner = nullptr;
  float4* tris = nullptr;
  uint32_t* ids = nullptr;
  rtgb::RangeAlloc nodes_alloc, tris_alloc;
  uint64_t generation = 0;  // bumps whenever the arena arrays move
  std::vector<rtgb::PoolScene> scenes;
  uint32_t max_stack_need = 1;
  int variant = rtgb::kDefaultPoolVariant;
  int refill = 4;
  int stack = 0;  // 0: 64 or 192 entries by the pooled scenes' worst case
  int tile = 0;   // top-of-tree nodes staged per job (variants 0 and 3)
  std::unordered_map<cudaStream_t, rtgb::StreamState*> streams;
};

namespace rtgb {
namespace {

rt_status cuda_err(cudaError_t e, const char* what) {
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return RT_ECUDA;
}

// Grows an arena array of `elem` bytes per entry from old_cap to new_cap entries.
template <class T>
cudaError_t grow_array(T** arr, uint64_t old_cap, uint64_t new_cap, size_t elem) {
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, new_cap * elem);
  if (e != cudaSuccess) return e;
  if (*arr && old_cap) {
    e = cudaMemcpy(p, *arr, old_cap * elem, cudaMemcpyDeviceToDevice);
    if (e != cudaSuccess) {
      cudaFree(p);
      return e;
    }
  }
  if (*arr) cudaFree(*arr);
  *arr = static_cast<T*>(p);
  return cudaSuccess;
}

DeviceScene arena_view(const rt_pool* P) {
  DeviceScene d;
  d.inner = P->inner;
  d.tris = P->tris;
  d.tri_ids = P->ids;
  d.n_tris = (uint32_t)P->tris_alloc.capacity;
  d.width = 4;
  d.stack_need = P->max_stack_need;
  return d;
}

StreamState* stream_state(rt_pool* P, cudaStream_t st, rt_status* status) {
  auto it = P->streams.find(st);
  if (it != P->streams.end()) return it->second;
  std::unique_ptr<StreamState> ss(new StreamState());
  cudaError_t e = cudaMalloc(&ss->counter, 256);
  for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
    e = cudaMallocHost(&ss->slot[i].host, kTableBytes);
    if (e == cudaSuccess) e = cudaMalloc(&ss->slot[i].dev, kTableBytes);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ss->slot[i].done, cudaEventDisableTiming);
  }
  if (e != cudaSuccess) {
    *status = cuda_err(e, "rt_pool: stream state");
    return nullptr;
  }
  StreamState* raw = ss.release();
  P->streams[st] = raw;
  return raw;
}

// Builds the job table in the slot's pinned buffer; returns the ray total.
rt_status fill_table(rt_pool* P, const RtJob* jobs, uint32_t num_jobs, DJob* host, uint64_t* total_out) {
  uint64_t total = 0;
  DJob* out = host + 1;
  for (uint32_t j = 0; j < num_jobs; ++j) {
    const RtJob& J = jobs[j];
    if (J.scene_id >= P->scenes.size() || !P->scenes[J.scene_id].live) {
      set_error("rt_pool_trace: job " + std::to_string(j) + " names an unknown scene");
      return RT_ENOTFOUND;
    }
    if (J.num_rays && (!J.d_rays || !J.d_hits)) {
      set_error("rt_pool_trace: job " + std::to_string(j) + " has null ray/hit buffers");
      return RT_EINVAL;
    }
    if ((reinterpret_cast<uintptr_t>(J.d_rays) & 15u) != 0u || (reinterpret_cast<uintptr_t>(J.d_hits) & 7u) != 0u) {
      set_error("rt_pool_trace: job " + std::to_string(j) + ": rays must be 16-byte aligned, hits 8-byte aligned");
      return RT_EINVAL;
    }
    out[j].rays = reinterpret_cast<const float4*>(J.d_rays);
    out[j].hits = reinterpret_cast<uint2*>(J.d_hits);
    out[j].start = (uint32_t)total;
    out[j].count = J.num_rays;
    out[j].root = P->scenes[J.scene_id].root;
    out[j].nodes = (uint32_t)P->scenes[J.scene_id].node_cnt;
    total += J.num_rays;
    if (total > 0x80000000ull) {
      set_error("rt_pool_trace: more than 2^31 rays in one batch");
      return RT_EINVAL;
    }
  }
  uint32_t* hdr = reinterpret_cast<uint32_t*>(host);
  std::memset(hdr, 0, sizeof(DJob));
  hdr[0] = num_jobs;
  hdr[1] = (uint32_t)total;
  *total_out = total;
  return RT_OK;
}

// Captures (table upload, queue reset, kernel) into the slot's graph.
rt_status capture(rt_pool* P, LaunchSlot& sl, uint32_t* counter, int variant, int any, int big, int refill,
                  int stack, int tile) {
  if (sl.exec) cudaGraphExecDestroy(sl.exec);
  if (sl.graph) cudaGraphDestroy(sl.graph);
  sl.exec = nullptr;
  sl.graph = nullptr;
  int* bps_slot = nullptr;
  int threads = 0;
  PoolKernel k = pool_kernel(variant, any, big, stack, tile, P->max_stack_need, &bps_slot, &threads);
  if (!k) {
    set_error("rt_pool: launch shape, stack capacity or tile not available for this pool");
    return RT_EINVAL;
  }
  int bps = 0;
  if (cudaError_t oe = cached_blocks_per_sm(bps_slot, k, threads, &bps); oe != cudaSuccess)
    return cuda_err(oe, "rt_pool: occupancy");
  cudaStream_t cs;
  cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cuda_err(e, "rt_pool: capture stream");
  e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) e = cudaMemcpyAsync(sl.dev, sl.host, kTableBytes, cudaMemcpyHostToDevice, cs);
  if (e == cudaSuccess) e = cudaMemsetAsync(counter, 0, 8, cs);
  if (e == cudaSuccess) {
    const uint32_t blocks = (uint32_t)(device_sm_count() * bps);
    k<<<blocks, threads, 0, cs>>>(arena_view(P), sl.dev, counter, refill);
    e = cudaGetLastError();
  }
  cudaGraph_t g = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(cs, &g);
  if (e == cudaSuccess) e = e2;
  if (e == cudaSuccess) e = cudaGraphInstantiate(&sl.exec, g, 0);
  sl.graph = g;
  cudaStreamDestroy(cs);
  if (e != cudaSuccess) return cuda_err(e, "rt_pool: graph capture");
  sl.generation = P->generation;
  sl.variant = variant;
  sl.any = any;
  sl.big = big;
  sl.refill = refill;
  sl.stack = stack;
  sl.tile = tile;
  return RT_OK;
}

rt_status pool_trace_locked(rt_pool* P, const RtJob* jobs, uint32_t num_jobs, uint32_t flags, cudaStream_t st,
                            int variant, int refill, int stack, int tile) {
  rt_status status = RT_OK;
  StreamState* ss = stream_state(P, st, &status);
  if (!ss) return status;
  LaunchSlot& sl = ss->slot[ss->next];
  ss->next ^= 1;
  // the slot's pinned table may still be read by its previous launch
  if (sl.used) {
    cudaError_t e = cudaEventSynchronize(sl.done);
    if (e != cudaSuccess) return cuda_err(e, "rt_pool_trace: slot wait");
  }
  uint64_t total = 0;
  if ((status = fill_table(P, jobs, num_jobs, sl.host, &total)) != RT_OK) return status;
  const int any = (flags & RT_TRACE_ANY) ? 1 : 0;
  const int big = P->max_stack_need > 64u ? 1 : 0;
  if (!sl.exec || sl.generation != P->generation || sl.variant != variant || sl.any != any || sl.big != big ||
      sl.refill != refill || sl.stack != stack || sl.tile != tile) {
    if ((status = capture(P, sl, ss->counter, variant, any, big, refill, stack, tile)) != RT_OK) return status;
  }
  cudaError_t e = cudaGraphLaunch(sl.exec, st);
  if (e == cudaSuccess) e = cudaEventRecord(sl.done, st);
  if (e != cudaSuccess) return cuda_err(e, "rt_pool_trace: graph launch");
  sl.used = true;
  return RT_OK;
}

}  // namespace

// Rebases a converted scene's refs into the arena: inner refs by node_off,
// triangle slots by tri_off (the count bits are kept).
static void rebase(HostDeviceBVH& hb, uint32_t node_off, uint32_t tri_off) {
  auto fix = [&](uint32_t r) -> uint32_t {
    if (r == kSentinel) return r;
    if (r < kSentinel) return r + node_off;
    if (r & kSphereBit) return r;  // pools hold triangles only; unused slots stay empty
    return (r & ~kSlotMask) | ((r & kSlotMask) + tri_off);
  };
  const size_t nn = hb.inner.size() / 16;
  parallel_for(nn, [&](size_t b, size_t e, unsigned) {
    for (size_t i = b; i < e; ++i)
      for (int k = 4; k < 8; ++k) {
        uint32_t u;
        std::memcpy(&u, &hb.inner[16 * i + k], 4);
        u = fix(u);
        std::memcpy(&hb.inner[16 * i + k], &u, 4);
      }
  });
  hb.root = fix(hb.root);
}

}  // namespace rtgb

using namespace rtgb;

extern "C" {

rt_status rt_pool_create(const RtPoolOptions* opt, rt_pool** out) {
  if (!out) {
    set_error("rt_pool_create: null argument");
    return RT_EINVAL;
  }
  *out = nullptr;
  rt_pool* P = new rt_pool();
  P->budget = (opt && opt->budget_bytes) ? opt->budget_bytes : (8ull << 30);
  P->max_scenes = (opt && opt->max_scenes) ? opt->max_scenes : 4096u;
  *out = P;
  return RT_OK;
}

rt_status rt_pool_destroy(rt_pool* P) {
  if (!P) return RT_OK;
  cudaDeviceSynchronize();
  for (auto& kv : P->streams) {
    StreamState* ss = kv.second;
    for (auto& sl : ss->slot) {
      if (sl.exec) cudaGraphExecDestroy(sl.exec);
      if (sl.graph) cudaGraphDestroy(sl.graph);
      if (sl.host) cudaFreeHost(sl.host);
      if (sl.dev) cudaFree(sl.dev);
      if (sl.done) cudaEventDestroy(sl.done);
    }
    if (ss->counter) cudaFree(ss->counter);
    delete ss;
  }
  if (P->inner) cudaFree(P->inner);
  if (P->tris) cudaFree(P->tris);
  if (P->ids) cudaFree(P->ids);
  delete P;
  return RT_OK;
}

rt_status rt_pool_add_scene(rt_pool* P, const RtSceneDesc* desc, uint32_t* out_id) {
  NvtxRange nvtx_range("rt_pool_add_scene");
  if (!P || !desc || !out_id) {
    set_error("rt_pool_add_scene: null argument");
    return RT_EINVAL;
  }
  if (desc->num_spheres) {
    set_error("rt_pool_add_scene: pooled scenes hold triangles only");
    return RT_EUNSUPPORTED;
  }
  if (desc->num_triangles && !desc->triangles) {
    set_error("rt_pool_add_scene: null triangles");
    return RT_EINVAL;
  }
  if (desc->bvh_mode != RT_BVH_SORTED && desc->bvh_mode != RT_BVH_REFERENCE) {
    set_error("rt_pool_add_scene: unknown bvh_mode");
    return RT_EINVAL;
  }
  const uint32_t nt = desc->num_triangles;
  if (desc->nodes && nt && desc->num_nodes != 2 * (uint64_t)nt - 1) {
    set_error("rt_pool_add_scene: num_nodes must be 2*triangles-1");
    return RT_EINVAL;
  }
  // Host work outside the lock: world space, BVH, device form.
  std::vector<RtTriangle64> wt;
  std::vector<RtSphere32> ws;
  std::string msg;
  if (!world_space(desc->triangles, nt, nullptr, 0, desc->models, desc->num_models, wt, ws, msg)) {
    set_error("rt_pool_add_scene: " + msg);
    return RT_EINVAL;
  }
  // The traversal tree, as in rt_scene_create_ex: a binned-SAH tree when the
  // library builds in sorted mode on the host (the pool exports no S1 nodes,
  // so none are built then), else the S1 array.
  const bool use_sah = !desc->nodes && !(desc->build_flags & (RT_BUILD_ON_DEVICE | RT_BUILD_TRAVERSE_S1)) &&
                       desc->bvh_mode == RT_BVH_SORTED && nt > 1;
  std::vector<RtBVHNode40> nodes;
  std::unique_ptr<RtBVHNode40[]> sah(use_sah ? new RtBVHNode40[2 * (size_t)nt - 1] : nullptr);
  if (desc->nodes) {
    nodes.assign(desc->nodes, desc->nodes + (nt ? 2 * (size_t)nt - 1 : 0));
  } else if ((desc->build_flags & RT_BUILD_ON_DEVICE) && nt) {
    rt_status bs = device_build_to_host(wt.data(), nt, nullptr, 0, desc->bvh_mode, nodes);
    if (bs != RT_OK) return bs;
  } else if (use_sah) {
    build_sah(wt.data(), nt, nullptr, 0, sah.get());
  } else {
    build_bvh(wt.data(), nt, nullptr, 0, desc->bvh_mode, nodes);
  }
  const RtBVHNode40* trav = use_sah ? sah.get() : nodes.data();
  const uint32_t trav_n = use_sah ? (uint32_t)(2 * (size_t)nt - 1) : (uint32_t)nodes.size();
  HostDeviceBVH hb;
  if (!convert_bvh(trav, trav_n, wt.data(), nt, nullptr, 0, nullptr, 0, desc->leaf_size, 4, hb, msg)) {
    set_error("rt_pool_add_scene: " + msg);
    return RT_EINVAL;
  }
  if (hb.width != 4 || hb.stack_need > 192u) {
    set_error("rt_pool_add_scene: BVH too deep for the pool's 4-wide traversal stack");
    return RT_ESTACK;
  }
  const uint64_t n_nodes = hb.inner.size() / 16, n_tris = hb.tri_ids.size();
  const uint64_t bytes = n_nodes * 64 + n_tris * 68;

  std::lock_guard<std::mutex> lk(P->mu);
  uint32_t live = 0;
  for (auto& s : P->scenes) live += s.live ? 1u : 0u;
  if (live >= P->max_scenes) {
    set_error("rt_pool_add_scene: scene limit reached");
    return RT_EBUSY;
  }
  if (P->used + bytes > P->budget) {
    set_error("rt_pool_add_scene: " + std::to_string(bytes) + " bytes exceed the remaining budget of " +
              std::to_string(P->budget - P->used));
    return RT_ENOMEM;
  }
  uint64_t noff = 0, toff = 0;
  bool moved = false;
  while (!P->nodes_alloc.alloc(n_nodes, &noff)) {
    const uint64_t cap = std::max<uint64_t>(2 * P->nodes_alloc.capacity, std::max<uint64_t>(n_nodes, 1u << 16));
    if (cap >= kSentinel) {
      set_error("rt_pool_add_scene: node arena full");
      return RT_ENOMEM;
    }
    cudaDeviceSynchronize();  // no launch may read the arrays while they move
    cudaError_t e = grow_array(&P->inner, P->nodes_alloc.capacity, cap, 64);
    if (e != cudaSuccess) {
      set_error(std::string("rt_pool_add_scene: node arena: ") + cudaGetErrorString(e));
      return RT_ENOMEM;
    }
    P->nodes_alloc.grow(cap);
    moved = true;
  }
  while (!P->tris_alloc.alloc(n_tris, &toff)) {
    const uint64_t cap = std::min<uint64_t>(std::max<uint64_t>(2 * P->tris_alloc.capacity,
                                                               std::max<uint64_t>(n_tris, 1u << 16)),
                                            kMaxTriangles);
    if (cap <= P->tris_alloc.capacity) {
      P->nodes_alloc.release(noff, n_nodes);
      set_error("rt_pool_add_scene: triangle arena full (2^27 triangles)");
      return RT_ENOMEM;
    }
    cudaDeviceSynchronize();
    cudaError_t e = grow_array(&P->tris, P->tris_alloc.capacity, cap, 64);
    if (e == cudaSuccess) e = grow_array(&P->ids, P->tris_alloc.capacity, cap, 4);
    if (e != cudaSuccess) {
      P->nodes_alloc.release(noff, n_nodes);
      set_error(std::string("rt_pool_add_scene: triangle arena: ") + cudaGetErrorString(e));
      return RT_ENOMEM;
    }
    P->tris_alloc.grow(cap);
    moved = true;
  }
  if (moved) P->generation++;
  rebase(hb, (uint32_t)noff, (uint32_t)toff);
  cudaError_t e = cudaSuccess;
  if (n_nodes) e = cudaMemcpy(P->inner + 4 * noff, hb.inner.data(), n_nodes * 64, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && n_tris) e = cudaMemcpy(P->tris + 4 * toff, hb.tris.data(), n_tris * 64, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && n_tris) e = cudaMemcpy(P->ids + toff, hb.tri_ids.data(), n_tris * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    P->nodes_alloc.release(noff, n_nodes);
    P->tris_alloc.release(toff, n_tris);
    return cuda_err(e, "rt_pool_add_scene: upload");
  }
  PoolScene ps;
  ps.root = hb.root;
  ps.node_off = noff;
  ps.node_cnt = n_nodes;
  ps.tri_off = toff;
  ps.tri_cnt = n_tris;
  ps.bytes = bytes;
  ps.stack_need = hb.stack_need;
  ps.live = true;
  uint32_t id = (uint32_t)P->scenes.size();
  for (uint32_t i = 0; i < P->scenes.size(); ++i)
    if (!P->scenes[i].live) {
      id = i;
      break;
    }
  if (id == P->scenes.size()) P->scenes.push_back(ps);
  else P->scenes[id] = ps;
  P->used += bytes;
  if (hb.stack_need > P->max_stack_need) P->max_stack_need = hb.stack_need;
  *out_id = id;
  return RT_OK;
}

rt_status rt_pool_remove_scene(rt_pool* P, uint32_t id) {
  if (!P) return RT_EINVAL;
  std::lock_guard<std::mutex> lk(P->mu);
  if (id >= P->scenes.size() || !P->scenes[id].live) {
    set_error("rt_pool_remove_scene: unknown scene");
    return RT_ENOTFOUND;
  }
  PoolScene& s = P->scenes[id];
  P->nodes_alloc.release(s.node_off, s.node_cnt);
  P->tris_alloc.release(s.tri_off, s.tri_cnt);
  P->used -= s.bytes;
  s = PoolScene();
  return RT_OK;
}

rt_status rt_pool_get_info(const rt_pool* Pc, RtPoolInfo* out) {
  if (!Pc || !out) return RT_EINVAL;
  rt_pool* P = const_cast<rt_pool*>(Pc);
  std::lock_guard<std::mutex> lk(P->mu);
  std::memset(out, 0, sizeof(*out));
  uint64_t tris = 0;
  for (auto& s : P->scenes)
    if (s.live) {
      out->num_scenes++;
      tris += s.tri_cnt;
    }
  out->stack_need = P->max_stack_need;
  out->used_bytes = P->used;
  out->budget_bytes = P->budget;
  out->arena_bytes = P->nodes_alloc.capacity * 64 + P->tris_alloc.capacity * 68;
  out->num_triangles = (uint32_t)tris;
  out->tuned_variant = (uint32_t)P->variant;
  out->tuned_refill = P->refill;
  out->tuned_stack = P->stack ? (uint32_t)P->stack : (P->max_stack_need > 64u ? 192u : 64u);
  out->tuned_tile = (uint32_t)P->tile;
  return RT_OK;
}

rt_status rt_pool_trace(rt_pool* P, const RtJob* jobs, uint32_t num_jobs, uint32_t flags, void* stream) {
  NvtxRange nvtx_range("rt_pool_trace");
  if (!P || (num_jobs && !jobs) || num_jobs > kMaxJobs || flags > RT_TRACE_ANY) {
    set_error("rt_pool_trace: bad argument (at most 8192 jobs; flags closest or any)");
    return RT_EINVAL;
  }
  std::lock_guard<std::mutex> lk(P->mu);
  // a pool that grew a deeper scene since tuning falls back to the default capacity
  int stack = P->stack, tile = P->tile;
  if (stack && (uint32_t)stack < P->max_stack_need) stack = 0, tile = 0;
  return pool_trace_locked(P, jobs, num_jobs, flags, reinterpret_cast<cudaStream_t>(stream), P->variant, P->refill,
                           stack, tile);
}

rt_status rt_pool_autotune(rt_pool* P, const RtJob* jobs, uint32_t num_jobs, uint32_t flags, void* stream,
                           uint32_t repeats) {
  NvtxRange nvtx_range("rt_pool_autotune");
  if (!P || (num_jobs && !jobs) || num_jobs > kMaxJobs || flags > RT_TRACE_ANY) {
    set_error("rt_pool_autotune: bad argument");
    return RT_EINVAL;
  }
  if (repeats == 0) repeats = 3;
  std::lock_guard<std::mutex> lk(P->mu);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  static const int refills[] = {1, 4, 8, 16};
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  float best = 3.4e38f;
  int bv = P->variant, br = P->refill, bs = 0, bt = 0;
  rt_status status = RT_OK;
  auto time_one = [&](int v, int r, int sc, int tl) -> rt_status {
    // warm-up: captures the graphs of both launch slots outside the timing
    rt_status rs = pool_trace_locked(P, jobs, num_jobs, flags, st, v, r, sc, tl);
    if (rs == RT_OK) rs = pool_trace_locked(P, jobs, num_jobs, flags, st, v, r, sc, tl);
    if (rs != RT_OK) return rs;
    cudaEventRecord(a, st);
    for (uint32_t k = 0; k < repeats && rs == RT_OK; ++k) rs = pool_trace_locked(P, jobs, num_jobs, flags, st, v, r, sc, tl);
    cudaEventRecord(b, st);
    if (rs != RT_OK) return rs;
    if (cudaEventSynchronize(b) != cudaSuccess) return cuda_err(cudaGetLastError(), "rt_pool_autotune");
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, b);
    if (ms < best) {
      best = ms;
      bv = v;
      br = r;
      bs = sc;
      bt = tl;
    }
    return RT_OK;
  };
  // 1. launch shape x refill threshold
  for (int v = 0; v < kNumPoolVariants && status == RT_OK; ++v)
    for (int r : refills) {
      if ((status = time_one(v, r, 0, 0)) != RT_OK) break;
    }
  // 2. on the 128 x 10 four-visit shapes: stack capacity x top-of-tree tile per job
  if (status == RT_OK && (bv == 5 || bv == 6)) {
    const int v = bv, r = br;
    for (int sc : kPoolStacks)
      for (int tl : kPoolTiles) {
        if (status != RT_OK || (uint32_t)sc < P->max_stack_need) continue;
        status = time_one(v, r, sc, tl);
      }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (status != RT_OK) return status;
  P->variant = bv;
  P->refill = br;
  P->stack = bs;
  P->tile = bt;
  return RT_OK;
}

rt_status rt_pool_set_tuning(rt_pool* P, uint32_t variant, int32_t refill, uint32_t stack_entries,
                             uint32_t tile_nodes) {
  if (!P) return RT_EINVAL;
  std::lock_guard<std::mutex> lk(P->mu);
  const int big = P->max_stack_need > 64u ? 1 : 0;
  int stack = (int)stack_entries, tile = (int)tile_nodes;
  if (stack == (big ? 192 : 64) && tile == 0) stack = 0;  // the shape's default capacity
  int* slot = nullptr;
  int threads = 0;
  if (refill < 0 || refill > 32 || !pool_kernel((int)variant, 0, big, stack, tile, P->max_stack_need, &slot, &threads)) {
    set_error("rt_pool_set_tuning: unknown launch shape, refill, stack capacity below the pool's need, or a tile on "
              "a shape without one");
    return RT_EINVAL;
  }
  P->variant = (int)variant;
  P->refill = refill;
  P->stack = stack;
  P->tile = tile;
  return RT_OK;
}

rt_status rt_pool_describe_variant(uint32_t v, uint32_t* threads, uint32_t* min_blocks, uint32_t* stack_ring) {
  if (v >= (uint32_t)kNumPoolVariants || !threads || !min_blocks) return RT_EINVAL;
  *threads = (uint32_t)g_pool_variants[v].threads;
  *min_blocks = (uint32_t)g_pool_variants[v].minb;
  if (stack_ring) *stack_ring = (uint32_t)g_pool_variants[v].ring;
  return RT_OK;
}

}  // extern "C"
