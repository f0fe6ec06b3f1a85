// rt_internal.h -- internal types shared by the host C++ and the CUDA sources.
//
// Device form of a scene (all arrays in HBM, read through the non-coherent path):
//
//   inner   : one 64-byte record per internal node of the binary BVH; the node
//             stores the boxes of its two children, so one fetch decides which
//             children a ray enters and in which order.
//               float4 a = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)
//               float4 b = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)
//               float4 c = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)
//               uint4  d = (ref0, ref1, 0, 0)
//   tris    : one 64-byte record per triangle, in BVH leaf order, holding the
//             values triangleHit (raytraceBVH.comp:118-149) derives from the
//             vertices, computed once with the same binary32 operations:
//               float4 (n.x, n.y, n.z, D)   n = normalize(cross(u,v)), D = dot(n,v0)
//               float4 (w.x, w.y, w.z, v0.x) w = N / dot(N,N)
//               float4 (v0.y, v0.z, u.x, u.y)
//               float4 (u.z, v.x, v.y, v.z)
//   tri_ids : leaf slot -> caller's triangle index
//   tri_mat : leaf slot -> material index
//   spheres : 32 B each, caller order: float4 (c.xyz, r), uint4 (material, ...)
//   mats    : 32 B each: float4 albedo, float4 (type bits, fuzz, ior, 0)
//
// A child reference ("ref") is a uint32:
//   bit31 = 0            internal node index
//   bit31 = 1, bit30 = 0 triangle leaf: bits 27..29 = count-1, bits 0..26 = first slot
//   bit31 = 1, bit30 = 1 sphere leaf: bits 0..29 = sphere index
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/rt_gb300.h"

#include <nvtx3/nvToolsExt.h>

namespace rtgb {

// Resident blocks per SM of `kernel` at `threads` per block, computed once per
// cache slot.  Host threads may race to fill a slot; they compute the same
// value, and the slot is read and written atomically.
template <class K>
cudaError_t cached_blocks_per_sm(int* slot, K kernel, int threads, int* out) {
  int v = __atomic_load_n(slot, __ATOMIC_RELAXED);
  if (v < 1) {
    int b = 0;
    const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, threads, 0);
    if (e != cudaSuccess) return e;
    v = b < 1 ? 1 : b;
    __atomic_store_n(slot, v, __ATOMIC_RELAXED);
  }
  *out = v;
  return cudaSuccess;
}

// An NVTX range over a library entry point (shown by Nsight Systems and
// usable as an ncu --nvtx filter); costs a function-pointer test when no tool
// is attached.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

constexpr uint32_t kLeafBit = 0x80000000u;
constexpr uint32_t kSphereBit = 0x40000000u;
constexpr uint32_t kCountShift = 27;
constexpr uint32_t kSlotMask = (1u << 27) - 1u;
constexpr uint32_t kSphereMask = (1u << 30) - 1u;
constexpr uint32_t kMaxLeafSize = 8;
constexpr uint32_t kMaxTriangles = 1u << 27;
constexpr uint32_t kSentinel = 0x7FFFFFFFu;  // stack bottom, never a node index
constexpr uint32_t kDefaultLeafSize = 1;
constexpr uint32_t kDefaultWidth = 4;
// Largest quantisation step exponent of a 4-wide node: the kernels scale by
// 2^(e+15) / d with |1/d| <= 2^64, which must stay below 2^128.
constexpr int kMaxWideExp = 48;
// The first kTopNodes 4-wide nodes of a tree are its top levels in
// breadth-first order (the rest follow in preorder), so that the kernels can
// stage the top of the tree in shared memory as one contiguous range.
constexpr uint32_t kTopNodes = 64;

struct DeviceScene {
  const void* inner = nullptr;     // float4[4 * n_inner]
  const void* tris = nullptr;      // float4[4 * n_tris]
  const uint32_t* tri_ids = nullptr;
  const uint32_t* tri_mat = nullptr;
  const void* spheres = nullptr;   // float4[2 * n_spheres]
  const void* mats = nullptr;      // float4[2 * n_mats]
  uint32_t root = kSentinel;       // ref of the root (kSentinel: empty scene)
  uint32_t n_inner = 0;
  uint32_t n_tris = 0;
  uint32_t n_spheres = 0;
  uint32_t n_mats = 0;
  uint32_t depth = 0;
  uint32_t width = 2;       // 2: binary child-box nodes; 4: quantised 4-wide nodes
  uint32_t stack_need = 0;  // worst-case traversal stack entries
  float box[6] = {0, 0, 0, 0, 0, 0};  // root box: lo xyz, hi xyz
  // Checked builds (RT_DEVICE_CHECKS=1): word 0 collects the kChk* bits of
  // out-of-range indices, word 1 the first bad index | 2^31.  May be null.
  uint32_t* check = nullptr;
};

// Host-side result of the BVH conversion, ready to upload.
struct HostDeviceBVH {
  std::vector<float> inner;        // 16 floats per internal node
  std::vector<float> tris;         // 16 floats per triangle slot
  std::vector<uint32_t> tri_ids;
  std::vector<uint32_t> tri_mat;
  std::vector<float> spheres;      // 8 floats per sphere
  std::vector<float> mats;         // 8 floats per material
  uint32_t root = kSentinel;
  uint32_t depth = 0;
  uint32_t width = 2;
  uint32_t stack_need = 1;
};

// ---- host BVH builder (host_bvh.cpp) ----
// Applies ModelSpaceToWorldSpace when models != nullptr (in place on copies).
// Returns false with msg on invalid input.
bool world_space(const RtTriangle64* tris, uint32_t nt, const RtSphere32* sph, uint32_t ns,
                 const RtModel64* models, uint32_t nm, std::vector<RtTriangle64>& out_t,
                 std::vector<RtSphere32>& out_s, std::string& msg);
// The six S1 passes; nodes gets 2N-1 records.
void build_bvh(const RtTriangle64* tris, uint32_t nt, const RtSphere32* sph, uint32_t ns,
               uint32_t mode, std::vector<RtBVHNode40>& nodes);
// Validates a reference-layout tree and converts it to the device form.
bool convert_bvh(const RtBVHNode40* nodes, uint32_t nn, const RtTriangle64* tris, uint32_t nt,
                 const RtSphere32* sph, uint32_t ns, const RtMaterial32* mats, uint32_t nm,
                 uint32_t leaf_size, uint32_t width, HostDeviceBVH& out, std::string& msg);
// Binned-SAH traversal tree over the same primitives (triangles, then
// spheres) in the node form convert_bvh reads; not the reference layout.
// Writes 2 * (nt + ns) - 1 nodes to out.
void build_sah(const RtTriangle64* tris, uint32_t nt, const RtSphere32* sph, uint32_t ns, RtBVHNode40* out);
// Camera of raytraceBVH.comp:50-81: out = camPos, pixel00, pixelDeltaU, pixelDeltaV.
void camera_setup(const RtRaytraceUBO& ubo, uint32_t width, uint32_t height, float out[12]);

unsigned host_threads();

// Runs f(begin, end, chunk) over [0, n) split into at most host_threads()
// contiguous chunks.
template <class F>
void parallel_for(size_t n, F&& f, size_t grain = 8192) {
  unsigned T = host_threads();
  if (T <= 1 || n < 2 * grain) {
    f((size_t)0, n, 0u);
    return;
  }
  size_t chunks = std::min<size_t>(T, (n + grain - 1) / grain);
  size_t per = (n + chunks - 1) / chunks;
  std::vector<std::thread> th;
  th.reserve(chunks);
  for (size_t c = 0; c < chunks; ++c) {
    size_t b = c * per, e = std::min(n, b + per);
    if (b >= e) break;
    th.emplace_back([&f, b, e, c] { f(b, e, (unsigned)c); });
  }
  for (auto& t : th) t.join();
}

// ---- device side (trace.cu / render.cu) ----
struct LaunchCfg {
  int blocks = 0;
  int threads = 0;
};
// Launch shape of the ray-query kernel: variant = (threads per block, min
// resident blocks) pair from a fixed table, refill threshold, grid size in
// percent of the resident-block count.
struct TraceTuning {
  int variant = 0;
  int refill = 20;
  int grid_scale = 100;
  // Default launch shape only (variant kTunedVariant): traversal stack
  // capacity per lane (0: 64 or 192 by the scene's worst-case need) and the
  // number of top-of-tree nodes staged in shared memory per block (0: none).
  int stack = 0;
  int tile = 0;
};
constexpr int kTunedVariant = 12;  // the default launch shape (see trace.cu)
constexpr int kDefaultVisits = 4;  // node visits per iteration of the default shape
constexpr int kTunedStacks[] = {48, 64, 96, 192};
constexpr int kTunedTiles[] = {0, 16, 64};
TraceTuning default_tuning();
int num_trace_variants();
void trace_variant_shape(int v, int* threads, int* minb);
// Whether the tuning can run a scene whose traversal needs `stack_need`
// entries with `flags` (RT_TRACE_*), and with what stack capacity.
bool tuning_supported(const TraceTuning& t, uint32_t width, uint32_t stack_need, uint32_t flags);
cudaError_t launch_trace_tuned(const DeviceScene& s, const RtRay* rays, uint32_t n, RtHit* hits, uint32_t flags,
                               uint32_t* counter, void* stream, const TraceTuning& tune,
                               unsigned long long* stats, const uint32_t* order);
// Coherence reordering (reorder.cu): bytes of scratch for n rays, and the
// launch that leaves the ray order (a permutation of 0..n-1) in *order_out.
size_t reorder_scratch_bytes(uint32_t n);
cudaError_t launch_reorder(const DeviceScene& s, const RtRay* rays, uint32_t n, void* scratch, uint32_t** order_out,
                           void* stream);
// Kernels launch on the given stream; counter is a device uint32 zeroed by the caller.
cudaError_t launch_trace(const DeviceScene& s, const RtRay* rays, uint32_t n, RtHit* hits, uint32_t flags,
                         uint32_t* counter, void* stream, const uint32_t* order = nullptr);
// Path-tracer queries (render.cu): hits[i] = (leaf-style ref of the closest
// primitive, 0: none, or kRawOverflow; t bits).  n == 0xFFFFFFFF takes the
// count from counter[2]; counter[0] must be zero.
constexpr uint32_t kRawOverflow = 0xFFFFFFFEu;
cudaError_t launch_trace_raw(const DeviceScene& s, const float4* rays, uint32_t n, uint2* hits, uint32_t* counter,
                             unsigned long long* stats, cudaStream_t stream);
// launch_render mode bits
constexpr uint32_t kRenderExtended = 1u;            // RT_SHADE_EXTENDED
constexpr uint32_t kRenderTraceEveryPrimary = 2u;   // RT_RENDER_TRACE_EVERY_PRIMARY
// Extra streams for the wavefront renderer (pixel chunks rotate over the
// caller's stream and these), with an event to fork them from the caller's
// stream and one per extra stream to join them back (none: one stream).
struct RenderStreams {
  int extra = 0;  // at most 3
  cudaStream_t streams[3] = {nullptr, nullptr, nullptr};
  cudaEvent_t fork = nullptr;
  cudaEvent_t join[3] = {nullptr, nullptr, nullptr};
};
cudaError_t launch_render(const DeviceScene& s, const float cam[12], uint32_t depth, uint32_t random_state,
                          float* accum, uint32_t w, uint32_t h, uint32_t spp, uint32_t mode,
                          const float bg[3], uint32_t* counter, void* stream,
                          unsigned long long* stats = nullptr,  // stats: queries, nodes, primitives
                          void* scratch = nullptr, uint64_t scratch_paths = 0, const RenderStreams* rs = nullptr);
// The wavefront renderer (4-wide trees) needs scratch of render_scratch_bytes
// for up to `paths` paths in flight, split in one part per stream (up to
// kWaveLanes) so that pixel chunks run their bounce levels on several streams
// at once; the frame is split into chunks that fit.
constexpr int kWaveLanes = 3;
bool render_uses_scratch(const DeviceScene& s, uint32_t depth);
size_t render_scratch_bytes(uint64_t paths, uint32_t depth);
cudaError_t launch_accum_clear(float* accum, uint32_t w, uint32_t h, void* stream);
cudaError_t launch_resolve(const float* accum, uint32_t w, uint32_t h, uint32_t spp, float* out, void* stream);
int device_sm_count();
// GPU LBVH build (gpu_build.cu)
size_t device_build_scratch_bytes(uint32_t n);
cudaError_t launch_device_build(const RtTriangle64* tris, uint32_t nt, const RtSphere32* sph, uint32_t ns,
                                uint32_t mode, RtBVHNode40* nodes, void* scratch, cudaStream_t st);

}  // namespace rtgb
