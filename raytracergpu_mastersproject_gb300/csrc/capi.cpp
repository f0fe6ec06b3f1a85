// capi.cpp -- the extern "C" entry points of include/rt_gb300.h.
//
// Ownership: a scene owns one device allocation holding every array of its
// device form (see rt_internal.h) and a host copy of its reference-layout
// nodes.  Per-stream work counters (the persistent kernels' ray/pixel
// queues) live in a small per-(device, stream) workspace created on first use.
#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <thread>

#include <cuda_runtime.h>

#include "rt_internal.h"

#ifndef RT_DEVICE_CHECKS
#define RT_DEVICE_CHECKS 0
#endif

struct rt_scene {
  rtgb::DeviceScene d;
  void* mem = nullptr;
  size_t bytes = 0;
  std::vector<RtBVHNode40> nodes40;
  RtSceneInfo info{};
  uint32_t max_material = 0;  // largest material index referenced (+1), 0 if none
  int device = 0;
  rtgb::TraceTuning tune = rtgb::default_tuning();  // launch of rt_trace / rt_trace_host (rt_trace_autotune)
};

namespace rtgb {

static thread_local std::string g_error;
void set_error(const std::string& msg) { g_error = msg; }
const DeviceScene* scene_device(const rt_scene* scene) { return &scene->d; }

static rt_status cuda_fail(cudaError_t e, const char* what) {
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return RT_ECUDA;
}

// ---- per-stream workspace ----
struct Workspace {
  uint32_t* counters = nullptr;  // 64 words
  // staging for rt_trace_host
  void* stage = nullptr;
  size_t stage_bytes = 0;
  // scratch of the coherence reordering
  void* sort = nullptr;
  size_t sort_bytes = 0;
  cudaStream_t copy_in = nullptr, copy_out = nullptr;
  cudaStream_t trace2 = nullptr;  // second trace stream of rt_trace_host
  cudaEvent_t ev[8] = {};
  // path state and ray lists of the wavefront renderer
  void* wave = nullptr;
  size_t wave_bytes = 0;
};
static std::mutex g_ws_mu;
static std::map<std::pair<int, cudaStream_t>, Workspace*> g_ws;

static rt_status workspace(cudaStream_t st, Workspace** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  std::lock_guard<std::mutex> lk(g_ws_mu);
  auto key = std::make_pair(dev, st);
  auto it = g_ws.find(key);
  if (it != g_ws.end()) {
    *out = it->second;
    return RT_OK;
  }
  Workspace* w = new Workspace();
  e = cudaMalloc(&w->counters, 64 * sizeof(uint32_t));
  if (e != cudaSuccess) {
    delete w;
    return cuda_fail(e, "cudaMalloc(workspace)");
  }
  g_ws[key] = w;
  *out = w;
  return RT_OK;
}

// Builds the node array on the GPU from host primitives and copies it back.
rt_status device_build_to_host(const RtTriangle64* tris, uint32_t nt, const RtSphere32* sph, uint32_t ns,
                               uint32_t mode, std::vector<RtBVHNode40>& out) {
  const uint64_t N = (uint64_t)nt + ns;
  RtTriangle64* d_t = nullptr;
  RtSphere32* d_s = nullptr;
  RtBVHNode40* d_n = nullptr;
  cudaError_t e = cudaMalloc(&d_t, sizeof(RtTriangle64) * (nt ? nt : 1));
  if (e == cudaSuccess) e = cudaMalloc(&d_s, sizeof(RtSphere32) * (ns ? ns : 1));
  if (e == cudaSuccess) e = cudaMalloc(&d_n, sizeof(RtBVHNode40) * (2 * N - 1));
  if (e == cudaSuccess && nt) e = cudaMemcpy(d_t, tris, sizeof(RtTriangle64) * nt, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && ns) e = cudaMemcpy(d_s, sph, sizeof(RtSphere32) * ns, cudaMemcpyHostToDevice);
  rt_status st = RT_OK;
  if (e == cudaSuccess) st = rt_build_bvh_device(d_t, nt, d_s, ns, mode, d_n, nullptr);
  if (e == cudaSuccess && st == RT_OK) {
    out.resize(2 * N - 1);
    e = cudaMemcpy(out.data(), d_n, sizeof(RtBVHNode40) * (2 * N - 1), cudaMemcpyDeviceToHost);
  }
  cudaFree(d_t);
  cudaFree(d_s);
  cudaFree(d_n);
  if (st != RT_OK) return st;
  return e == cudaSuccess ? RT_OK : cuda_fail(e, "device BVH build");
}

static rt_status ensure_sort_scratch(Workspace* w, size_t need) {
  if (w->sort_bytes >= need) return RT_OK;
  if (w->sort) cudaFree(w->sort);
  w->sort = nullptr;
  w->sort_bytes = 0;
  cudaError_t e = cudaMalloc(&w->sort, need);
  if (e != cudaSuccess) {
    set_error(std::string("reorder scratch: cudaMalloc: ") + cudaGetErrorString(e));
    return RT_ENOMEM;
  }
  w->sort_bytes = need;
  return RT_OK;
}

// The helper streams and events of rt_trace_host and the wavefront renderer,
// created on first use.
static rt_status ensure_helpers(Workspace* w) {
  if (w->copy_in) return RT_OK;
  cudaError_t e;
  if ((e = cudaStreamCreateWithFlags(&w->copy_in, cudaStreamNonBlocking)) != cudaSuccess) return cuda_fail(e, "stream");
  if ((e = cudaStreamCreateWithFlags(&w->copy_out, cudaStreamNonBlocking)) != cudaSuccess) return cuda_fail(e, "stream");
  if ((e = cudaStreamCreateWithFlags(&w->trace2, cudaStreamNonBlocking)) != cudaSuccess) return cuda_fail(e, "stream");
  for (auto& ev : w->ev)
    if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess) return cuda_fail(e, "event");
  return RT_OK;
}

static size_t sort_slot_bytes(uint32_t n) { return (reorder_scratch_bytes(n) + 255) & ~(size_t)255; }

// Reorders the batch when RT_TRACE_SORT is set; *order = nullptr otherwise.
// The scratch starts `offset` bytes into the workspace's sort buffer, so that
// batches in flight on two streams use disjoint regions.
static rt_status maybe_reorder(Workspace* w, const DeviceScene& d, const RtRay* rays, uint32_t n, uint32_t flags,
                               cudaStream_t st, uint32_t** order, size_t offset = 0) {
  *order = nullptr;
  if (!(flags & RT_TRACE_SORT) || d.root == kSentinel) return RT_OK;
  rt_status s = ensure_sort_scratch(w, offset + reorder_scratch_bytes(n));
  if (s != RT_OK) return s;
  cudaError_t e = launch_reorder(d, rays, n, static_cast<char*>(w->sort) + offset, order, st);
  return e == cudaSuccess ? RT_OK : cuda_fail(e, "reorder");
}

}  // namespace rtgb

using namespace rtgb;

extern "C" {

const char* rt_last_error_string(void) { return g_error.c_str(); }

rt_status rt_device_alloc(size_t bytes, void** d_out) {
  if (!d_out) return RT_EINVAL;
  *d_out = nullptr;
  cudaError_t e = cudaMalloc(d_out, bytes ? bytes : 1);
  if (e != cudaSuccess) {
    set_error(std::string("rt_device_alloc: ") + cudaGetErrorString(e));
    return RT_ENOMEM;
  }
  return RT_OK;
}

rt_status rt_device_free(void* d_ptr) {
  cudaError_t e = cudaFree(d_ptr);
  return e == cudaSuccess ? RT_OK : cuda_fail(e, "rt_device_free");
}

rt_status rt_copy(void* dst, const void* src, size_t bytes, void* stream) {
  if ((!dst || !src) && bytes) return RT_EINVAL;
  if (!bytes) return RT_OK;
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, reinterpret_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? RT_OK : cuda_fail(e, "rt_copy");
}
uint32_t rt_abi_version(void) { return RT_ABI_VERSION; }

rt_status rt_stream_wait(void* stream, double timeout_seconds) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const auto t0 = std::chrono::steady_clock::now();
  for (;;) {
    cudaError_t e = cudaStreamQuery(st);
    if (e == cudaSuccess) return RT_OK;
    if (e != cudaErrorNotReady) return cuda_fail(e, "cudaStreamQuery");
    const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (el >= timeout_seconds) {
      set_error("rt_stream_wait: deadline passed");
      return RT_ETIMEOUT;
    }
    std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
}

uint32_t rt_device_checks_compiled(void) { return RT_DEVICE_CHECKS; }

rt_status rt_scene_device_checks(rt_scene* scene, uint32_t* bits, uint32_t* first_index) {
  if (!scene || !bits) {
    set_error("rt_scene_device_checks: bad argument");
    return RT_EINVAL;
  }
  uint32_t w[2] = {0, 0};
  cudaError_t e = cudaMemcpy(w, scene->d.check, sizeof(w), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemset(scene->d.check, 0, sizeof(w));
  if (e != cudaSuccess) return cuda_fail(e, "rt_scene_device_checks");
  *bits = w[0];
  if (first_index) *first_index = w[1] & 0x7FFFFFFFu;
  return RT_OK;
}

uint32_t rt_workspace_count(void) {
  std::lock_guard<std::mutex> lk(g_ws_mu);
  return (uint32_t)g_ws.size();
}

rt_status rt_stream_release(void* stream) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "rt_stream_release: cudaGetDevice");
  Workspace* w = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_ws_mu);
    auto it = g_ws.find(std::make_pair(dev, st));
    if (it == g_ws.end()) return RT_OK;
    w = it->second;
    g_ws.erase(it);
  }
  // the library's work on the stream (and on its helper streams) ends first
  e = cudaStreamSynchronize(st);
  for (cudaStream_t h : {w->copy_in, w->copy_out, w->trace2})
    if (h) {
      const cudaError_t e2 = cudaStreamSynchronize(h);
      if (e == cudaSuccess) e = e2;
      cudaStreamDestroy(h);
    }
  for (cudaEvent_t ev : w->ev)
    if (ev) cudaEventDestroy(ev);
  for (void* p : {static_cast<void*>(w->counters), w->stage, w->sort, w->wave})
    if (p) cudaFree(p);
  delete w;
  return e == cudaSuccess ? RT_OK : cuda_fail(e, "rt_stream_release");
}

rt_status rt_build_bvh(const RtTriangle64* triangles, uint32_t num_triangles, const RtSphere32* spheres,
                       uint32_t num_spheres, const RtModel64* models, uint32_t num_models, uint32_t bvh_mode,
                       RtBVHNode40* out_nodes) {
  rtgb::NvtxRange nvtx_range("rt_build_bvh");
  const uint64_t N = (uint64_t)num_triangles + num_spheres;
  if ((num_triangles && !triangles) || (num_spheres && !spheres) || (N && !out_nodes) ||
      (bvh_mode != RT_BVH_SORTED && bvh_mode != RT_BVH_REFERENCE) || N > kMaxTriangles) {
    set_error("rt_build_bvh: bad argument");
    return RT_EINVAL;
  }
  std::vector<RtTriangle64> wt;
  std::vector<RtSphere32> ws;
  std::string msg;
  if (!world_space(triangles, num_triangles, spheres, num_spheres, models, num_models, wt, ws, msg)) {
    set_error("rt_build_bvh: " + msg);
    return RT_EINVAL;
  }
  std::vector<RtBVHNode40> nodes;
  build_bvh(wt.data(), num_triangles, ws.data(), num_spheres, bvh_mode, nodes);
  if (!nodes.empty()) std::memcpy(out_nodes, nodes.data(), nodes.size() * sizeof(RtBVHNode40));
  return RT_OK;
}

rt_status rt_build_bvh_sah(const RtTriangle64* triangles, uint32_t num_triangles, const RtSphere32* spheres,
                           uint32_t num_spheres, const RtModel64* models, uint32_t num_models,
                           RtBVHNode40* out_nodes) {
  rtgb::NvtxRange nvtx_range("rt_build_bvh_sah");
  const uint64_t N = (uint64_t)num_triangles + num_spheres;
  if ((num_triangles && !triangles) || (num_spheres && !spheres) || (N && !out_nodes) || N > kMaxTriangles) {
    set_error("rt_build_bvh_sah: bad argument");
    return RT_EINVAL;
  }
  std::vector<RtTriangle64> wt;
  std::vector<RtSphere32> ws;
  std::string msg;
  if (!world_space(triangles, num_triangles, spheres, num_spheres, models, num_models, wt, ws, msg)) {
    set_error("rt_build_bvh_sah: " + msg);
    return RT_EINVAL;
  }
  build_sah(wt.data(), num_triangles, ws.data(), num_spheres, out_nodes);
  return RT_OK;
}

rt_status rt_scene_create_ex(const RtSceneDesc* desc, rt_scene** out_scene) {
  rtgb::NvtxRange nvtx_range("rt_scene_create_ex");
  if (!desc || !out_scene) {
    set_error("rt_scene_create_ex: null argument");
    return RT_EINVAL;
  }
  *out_scene = nullptr;
  const uint32_t nt = desc->num_triangles, ns = desc->num_spheres, nm = desc->num_materials;
  const uint64_t N = (uint64_t)nt + ns;
  if ((nt && !desc->triangles) || (ns && !desc->spheres) || (nm && !desc->materials)) {
    set_error("rt_scene_create_ex: null array with non-zero count");
    return RT_EINVAL;
  }
  if (N > kMaxTriangles) {
    set_error("rt_scene_create_ex: more than 2^27 primitives");
    return RT_EINVAL;
  }
  if (desc->bvh_mode != RT_BVH_SORTED && desc->bvh_mode != RT_BVH_REFERENCE) {
    set_error("rt_scene_create_ex: unknown bvh_mode");
    return RT_EINVAL;
  }
  if (desc->nodes && N && desc->num_nodes != 2 * N - 1) {
    set_error("rt_scene_create_ex: num_nodes must be 2*(triangles+spheres)-1");
    return RT_EINVAL;
  }
  if (desc->build_flags & ~(RT_BUILD_ON_DEVICE | RT_BUILD_TRAVERSE_S1)) {
    set_error("rt_scene_create_ex: unknown build_flags");
    return RT_EINVAL;
  }
  const auto t0 = std::chrono::steady_clock::now();
  std::unique_ptr<rt_scene> sc(new rt_scene());
  cudaGetDevice(&sc->device);
  std::vector<RtTriangle64> wt;
  std::vector<RtSphere32> ws;
  std::string msg;
  if (!world_space(desc->triangles, nt, desc->spheres, ns, desc->models, desc->num_models, wt, ws, msg)) {
    set_error("rt_scene_create_ex: " + msg);
    return RT_EINVAL;
  }
  if (desc->nodes) {
    sc->nodes40.assign(desc->nodes, desc->nodes + (N ? 2 * N - 1 : 0));
  } else if ((desc->build_flags & RT_BUILD_ON_DEVICE) && N) {
    rt_status bs = device_build_to_host(wt.data(), nt, ws.data(), ns, desc->bvh_mode, sc->nodes40);
    if (bs != RT_OK) return bs;
  } else {
    build_bvh(wt.data(), nt, ws.data(), ns, desc->bvh_mode, sc->nodes40);
  }
  HostDeviceBVH hb;
  // 0 lets the conversion choose (4-wide unless the scene is too wide for it)
  const uint32_t width = desc->node_width;
  if (width != 0 && width != 2 && width != 4) {
    set_error("rt_scene_create_ex: node_width must be 0, 2 or 4");
    return RT_EINVAL;
  }
  // the traversal tree: SAH for library-built sorted-mode scenes, else S1
  const bool use_sah = !desc->nodes && !(desc->build_flags & (RT_BUILD_ON_DEVICE | RT_BUILD_TRAVERSE_S1)) &&
                       desc->bvh_mode == RT_BVH_SORTED && N > 1;
  std::unique_ptr<RtBVHNode40[]> sah(use_sah ? new RtBVHNode40[2 * N - 1] : nullptr);
  if (use_sah) build_sah(wt.data(), nt, ws.data(), ns, sah.get());
  const RtBVHNode40* trav = use_sah ? sah.get() : sc->nodes40.data();
  const uint32_t trav_n = use_sah ? (uint32_t)(2 * N - 1) : (uint32_t)sc->nodes40.size();
  if (!convert_bvh(trav, trav_n, wt.data(), nt, ws.data(), ns, desc->materials, nm,
                   desc->leaf_size, width, hb, msg)) {
    set_error("rt_scene_create_ex: " + msg);
    return RT_EINVAL;
  }
  if (hb.width == 4 && hb.stack_need > 192u) {  // too deep for the wide stack: binary form
    if (!convert_bvh(trav, trav_n, wt.data(), nt, ws.data(), ns, desc->materials,
                     nm, desc->leaf_size, 2, hb, msg)) {
      set_error("rt_scene_create_ex: " + msg);
      return RT_EINVAL;
    }
  }
  if (hb.width == 2 && hb.stack_need > 128u) {
    set_error("rt_scene_create_ex: BVH depth " + std::to_string(hb.depth) + " exceeds the 127-level stack");
    return RT_ESTACK;
  }
  uint32_t maxm = 0;
  for (uint32_t i = 0; i < nt; ++i) maxm = std::max(maxm, wt[i].materialIndex + 1u);
  for (uint32_t i = 0; i < ns; ++i) maxm = std::max(maxm, ws[i].materialIndex + 1u);
  sc->max_material = maxm;

  // One device allocation, 256-byte aligned sub-arrays.
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t b_inner = hb.inner.size() * 4, b_tris = hb.tris.size() * 4, b_ids = hb.tri_ids.size() * 4,
               b_mat = hb.tri_mat.size() * 4, b_sph = hb.spheres.size() * 4, b_mats = hb.mats.size() * 4;
  const size_t total = al(b_inner) + al(b_tris) + al(b_ids) + al(b_mat) + al(b_sph) + al(b_mats) + 256;
  cudaError_t e = cudaMalloc(&sc->mem, total);
  if (e != cudaSuccess) {
    set_error(std::string("rt_scene_create_ex: cudaMalloc: ") + cudaGetErrorString(e));
    return RT_ENOMEM;
  }
  sc->bytes = total;
  char* p = static_cast<char*>(sc->mem);
  auto put = [&](const void* src, size_t bytes) -> const void* {
    void* dst = p;
    if (bytes) {
      cudaError_t ce = cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
      if (ce != cudaSuccess) e = ce;
    }
    p += al(bytes);
    return dst;
  };
  sc->d.inner = put(hb.inner.data(), b_inner);
  sc->d.tris = put(hb.tris.data(), b_tris);
  sc->d.tri_ids = static_cast<const uint32_t*>(put(hb.tri_ids.data(), b_ids));
  sc->d.tri_mat = static_cast<const uint32_t*>(put(hb.tri_mat.data(), b_mat));
  sc->d.spheres = put(hb.spheres.data(), b_sph);
  sc->d.mats = put(hb.mats.data(), b_mats);
  sc->d.check = reinterpret_cast<uint32_t*>(p);  // the trailing 256 bytes
  if (e == cudaSuccess) e = cudaMemset(p, 0, 8);
  if (e != cudaSuccess) {
    cudaFree(sc->mem);
    sc->mem = nullptr;
    return cuda_fail(e, "rt_scene_create_ex: upload");
  }
  sc->d.root = hb.root;
  sc->d.n_inner = (uint32_t)(hb.inner.size() / 16);
  sc->d.n_tris = (uint32_t)hb.tri_ids.size();
  sc->d.n_spheres = ns;
  sc->d.n_mats = nm;
  sc->d.depth = hb.depth;
  sc->d.width = hb.width;
  sc->d.stack_need = hb.stack_need;
  if (!sc->nodes40.empty()) {
    const RtBVHNode40& r = sc->nodes40[0];
    const float b[6] = {r.minX, r.minY, r.minZ, r.maxX, r.maxY, r.maxZ};
    for (int k = 0; k < 6; ++k) sc->d.box[k] = b[k];
  }
  RtSceneInfo& inf = sc->info;
  inf.num_triangles = nt;
  inf.num_spheres = ns;
  inf.num_materials = nm;
  inf.num_nodes = (uint32_t)sc->nodes40.size();
  inf.device_nodes = sc->d.n_inner;
  inf.depth = hb.depth;
  inf.leaf_size = desc->leaf_size ? desc->leaf_size : kDefaultLeafSize;
  inf.bvh_mode = desc->bvh_mode;
  inf.device_bytes = total;
  inf.build_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  inf.node_width = hb.width;
  inf.stack_need = hb.stack_need;
  inf.traversal_sah = use_sah ? 1u : 0u;
  *out_scene = sc.release();
  return RT_OK;
}

rt_status rt_scene_create(const RtTriangle64* triangles, uint32_t num_triangles, const RtSphere32* spheres,
                          uint32_t num_spheres, const RtMaterial32* materials, uint32_t num_materials,
                          const RtBVHNode40* nodes, rt_scene** out_scene) {
  RtSceneDesc d;
  std::memset(&d, 0, sizeof(d));
  d.triangles = triangles;
  d.num_triangles = num_triangles;
  d.spheres = spheres;
  d.num_spheres = num_spheres;
  d.materials = materials;
  d.num_materials = num_materials;
  d.nodes = nodes;
  const uint64_t N = (uint64_t)num_triangles + num_spheres;
  d.num_nodes = nodes && N ? (uint32_t)(2 * N - 1) : 0;
  d.bvh_mode = RT_BVH_SORTED;
  return rt_scene_create_ex(&d, out_scene);
}

rt_status rt_scene_destroy(rt_scene* scene) {
  if (!scene) return RT_OK;
  if (scene->mem) cudaFree(scene->mem);
  delete scene;
  return RT_OK;
}

rt_status rt_scene_get_info(const rt_scene* scene, RtSceneInfo* out_info) {
  if (!scene || !out_info) {
    set_error("rt_scene_get_info: null argument");
    return RT_EINVAL;
  }
  *out_info = scene->info;
  return RT_OK;
}

rt_status rt_scene_get_nodes(const rt_scene* scene, RtBVHNode40* h_out, uint32_t capacity) {
  if (!scene || (!h_out && !scene->nodes40.empty())) {
    set_error("rt_scene_get_nodes: null argument");
    return RT_EINVAL;
  }
  if (capacity < scene->nodes40.size()) {
    set_error("rt_scene_get_nodes: capacity below num_nodes");
    return RT_EINVAL;
  }
  if (!scene->nodes40.empty())
    std::memcpy(h_out, scene->nodes40.data(), scene->nodes40.size() * sizeof(RtBVHNode40));
  return RT_OK;
}

// Device ray and hit arrays must sit at their records' natural vector
// alignment: the kernels read a ray as float4 pairs (16 bytes) and write a hit
// as one 8-byte store.  Any cudaMalloc'd array of RtRay / RtHit, or a slice of
// one, satisfies it; a byte offset that breaks it is refused rather than
// faulting on the device.
static bool misaligned(const void* rays, const void* hits) {
  return (reinterpret_cast<uintptr_t>(rays) & 15u) != 0u || (reinterpret_cast<uintptr_t>(hits) & 7u) != 0u;
}

rt_status rt_trace(rt_scene* scene, const RtRay* d_rays, uint32_t n, RtHit* d_hits, uint32_t flags, void* stream) {
  rtgb::NvtxRange nvtx_range("rt_trace");
  if (!scene || (n && (!d_rays || !d_hits)) || flags > (RT_TRACE_ANY | RT_TRACE_SORT | RT_TRACE_MT) ||
      n > 0x80000000u || misaligned(d_rays, d_hits)) {
    set_error("rt_trace: bad argument (rays must be 16-byte aligned, hits 8-byte aligned)");
    return RT_EINVAL;
  }
  if (n == 0) return RT_OK;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  Workspace* w = nullptr;
  rt_status s = workspace(st, &w);
  if (s != RT_OK) return s;
  uint32_t* order = nullptr;
  if ((s = maybe_reorder(w, scene->d, d_rays, n, flags, st, &order)) != RT_OK) return s;
  cudaError_t e = cudaMemsetAsync(w->counters, 0, 2 * sizeof(uint32_t), st);
  if (e != cudaSuccess) return cuda_fail(e, "rt_trace: memset");
  e = launch_trace_tuned(scene->d, d_rays, n, d_hits, flags, w->counters, stream,
                         (flags & RT_TRACE_MT) ? default_tuning() : scene->tune, nullptr, order);
  if (e != cudaSuccess) return cuda_fail(e, "rt_trace: launch");
  return RT_OK;
}

rt_status rt_trace_count(rt_scene* scene, const RtRay* d_rays, uint32_t n, RtHit* d_hits, uint32_t flags,
                         void* stream, uint64_t* h_counts) {
  rtgb::NvtxRange nvtx_range("rt_trace_count");
  if (!scene || !h_counts || (n && (!d_rays || !d_hits)) || flags > (RT_TRACE_ANY | RT_TRACE_SORT) ||
      n > 0x80000000u || misaligned(d_rays, d_hits)) {
    set_error("rt_trace_count: bad argument (rays must be 16-byte aligned, hits 8-byte aligned)");
    return RT_EINVAL;
  }
  h_counts[0] = h_counts[1] = 0;
  if (n == 0) return RT_OK;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  Workspace* w = nullptr;
  rt_status s = workspace(st, &w);
  if (s != RT_OK) return s;
  cudaError_t e = cudaMemsetAsync(w->counters, 0, 64 * sizeof(uint32_t), st);
  if (e != cudaSuccess) return cuda_fail(e, "rt_trace_count: memset");
  unsigned long long* stats = reinterpret_cast<unsigned long long*>(w->counters + 8);
  uint32_t* order = nullptr;
  if ((s = maybe_reorder(w, scene->d, d_rays, n, flags, st, &order)) != RT_OK) return s;
  e = launch_trace_tuned(scene->d, d_rays, n, d_hits, flags, w->counters, stream, default_tuning(), stats, order);
  if (e != cudaSuccess) return cuda_fail(e, "rt_trace_count: launch");
  unsigned long long hc[2] = {0, 0};
  e = cudaMemcpyAsync(hc, stats, sizeof(hc), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "rt_trace_count: read counters");
  h_counts[0] = hc[0];
  h_counts[1] = hc[1];
  return RT_OK;
}

rt_status rt_trace_autotune(rt_scene* scene, const RtRay* d_rays, uint32_t n, RtHit* d_hits, uint32_t flags,
                            void* stream, uint32_t repeats, RtTraceTuning* out) {
  rtgb::NvtxRange nvtx_range("rt_trace_autotune");
  if (!scene || !d_rays || !d_hits || n == 0 || n > 0x80000000u || (flags & ~(uint32_t)(RT_TRACE_ANY | RT_TRACE_SORT)) ||
      misaligned(d_rays, d_hits)) {
    set_error("rt_trace_autotune: bad argument (rays and hits required, 16- and 8-byte aligned; flags RT_TRACE_ANY / "
              "RT_TRACE_SORT)");
    return RT_EINVAL;
  }
  if (repeats == 0) repeats = 3;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  Workspace* w = nullptr;
  rt_status s = workspace(st, &w);
  if (s != RT_OK) return s;
  uint32_t* order = nullptr;
  if ((s = maybe_reorder(w, scene->d, d_rays, n, flags, st, &order)) != RT_OK) return s;
  cudaEvent_t a = nullptr, b = nullptr;
  cudaError_t e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  if (e != cudaSuccess) return cuda_fail(e, "rt_trace_autotune: events");
  // one warm-up launch, then `repeats` timed launches of one candidate
  auto time_one = [&](const TraceTuning& t, float* ms) -> cudaError_t {
    cudaError_t r = cudaSuccess;
    for (uint32_t k = 0; k <= repeats && r == cudaSuccess; ++k) {
      if (k == 1) r = cudaEventRecord(a, st);
      if (r == cudaSuccess) r = cudaMemsetAsync(w->counters, 0, 2 * sizeof(uint32_t), st);
      if (r == cudaSuccess) r = launch_trace_tuned(scene->d, d_rays, n, d_hits, flags, w->counters, stream, t, nullptr, order);
    }
    if (r == cudaSuccess) r = cudaEventRecord(b, st);
    if (r == cudaSuccess) r = cudaEventSynchronize(b);
    if (r == cudaSuccess) r = cudaEventElapsedTime(ms, a, b);
    if (r == cudaSuccess) *ms /= (float)repeats;
    return r;
  };
  TraceTuning best = scene->tune;
  float best_ms = 3.4e38f;
  auto consider = [&](const TraceTuning& t) -> cudaError_t {
    if (!tuning_supported(t, scene->d.width, scene->d.stack_need, flags)) return cudaSuccess;
    float ms = 0.0f;
    const cudaError_t r = time_one(t, &ms);
    if (r == cudaSuccess && ms < best_ms) {
      best_ms = ms;
      best = t;
    }
    return r;
  };
  // 1. launch shape x refill threshold; 2. at the default shape, the stack
  // capacity and the top-of-tree staging tile.
  static const int shapes[] = {kTunedVariant, 13, 14, 15, 10, 11, 8, 9, 6, 7, 3, 4};
  static const int refills[] = {3, 5, 8};
  TraceTuning t = default_tuning();
  t.stack = 0;
  t.tile = 0;
  e = consider(scene->tune);
  for (int v : shapes)
    for (int r : refills) {
      if (e != cudaSuccess) break;
      t.variant = v;
      t.refill = r;
      e = consider(t);
    }
  if (e == cudaSuccess && best.variant == kTunedVariant && scene->d.width == 4) {
    t = best;
    for (int sc : kTunedStacks)
      for (int tl : kTunedTiles) {
        if (e != cudaSuccess) break;
        t.stack = sc;
        t.tile = tl;
        e = consider(t);
      }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (e != cudaSuccess) return cuda_fail(e, "rt_trace_autotune");
  scene->tune = best;
  if (out) {
    out->launch_shape = (uint32_t)best.variant;
    out->refill = (uint32_t)best.refill;
    out->stack_entries = best.stack ? (uint32_t)best.stack : (scene->d.stack_need > 64u ? 192u : 64u);
    out->tile_nodes = (uint32_t)best.tile;
    out->best_ms = best_ms;
  }
  return RT_OK;
}

rt_status rt_scene_get_tuning(const rt_scene* scene, RtTraceTuning* out) {
  if (!scene || !out) {
    set_error("rt_scene_get_tuning: null argument");
    return RT_EINVAL;
  }
  out->launch_shape = (uint32_t)scene->tune.variant;
  out->refill = (uint32_t)scene->tune.refill;
  out->stack_entries = scene->tune.stack ? (uint32_t)scene->tune.stack : (scene->d.stack_need > 64u ? 192u : 64u);
  out->tile_nodes = (uint32_t)scene->tune.tile;
  out->best_ms = 0.0f;
  return RT_OK;
}

rt_status rt_scene_set_tuning(rt_scene* scene, const RtTraceTuning* in) {
  if (!scene || !in) {
    set_error("rt_scene_set_tuning: null argument");
    return RT_EINVAL;
  }
  TraceTuning t = default_tuning();
  t.variant = (int)in->launch_shape;
  t.refill = (int)in->refill;
  t.stack = (int)in->stack_entries;
  t.tile = (int)in->tile_nodes;
  const int need_cap = scene->d.stack_need > 64u ? 192 : 64;
  if (t.stack == need_cap && t.tile == 0) t.stack = 0;  // the default capacity of the shape
  if (!tuning_supported(t, scene->d.width, scene->d.stack_need, 0)) {
    set_error("rt_scene_set_tuning: unsupported launch shape, refill, stack capacity or tile for this scene");
    return RT_EINVAL;
  }
  scene->tune = t;
  return RT_OK;
}

rt_status rt_trace_host(rt_scene* scene, const RtRay* h_rays, uint32_t n, RtHit* h_hits, uint32_t flags,
                        void* stream) {
  rtgb::NvtxRange nvtx_range("rt_trace_host");
  if (!scene || (n && (!h_rays || !h_hits)) || flags > (RT_TRACE_ANY | RT_TRACE_SORT | RT_TRACE_MT) ||
      n > 0x80000000u) {
    set_error("rt_trace_host: bad argument");
    return RT_EINVAL;
  }
  if (n == 0) return RT_OK;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  Workspace* w = nullptr;
  rt_status s = workspace(st, &w);
  if (s != RT_OK) return s;
  // Chunks alternate between two ray buffers and two trace streams (the
  // caller's and trace2), each with its own counters and reorder scratch;
  // copy-in runs on a stream of its own, so chunk i+1 uploads while chunk i
  // traces, and chunk i+1's blocks take the SMs that chunk i's last rays
  // leave idle.  Every launch still ends with a drain of its in-flight rays at
  // falling SIMT efficiency, so chunks are few and large: the first is the
  // smallest (its upload is not overlapped) and each next one several times
  // larger.
  //
  // Hits are staged in device memory and downloaded per chunk on a third
  // stream; chunks start at 2 Mi rays and grow 4x, and the plan ends with a
  // small chunk, so that the one download that overlaps nothing is short.
  // With RT_HOST_DIRECT_HITS=1 and page-locked h_hits the kernels instead
  // write the hits there directly over the host link (scattered 8-byte
  // stores, overlapped with tracing) and chunks grow 8x; on GB300 that
  // measured no faster than staging (config 3: 12.55-13.03 ms against
  // 12.36-12.55 ms per 16 Mi rays on the same boxes).
  static const uint32_t kFirstChunk = [] {
    const char* e = std::getenv("RT_HOST_FIRST_CHUNK_RAYS");
    const long v = e ? std::atol(e) : 0;
    return v >= 4096 && v <= (1l << 30) ? (uint32_t)v : (1u << 21);
  }();
  static const uint32_t kLastChunk = [] {
    const char* e = std::getenv("RT_HOST_LAST_CHUNK_RAYS");
    if (!e) return 1u << 19;
    const long v = std::atol(e);
    return v >= 0 && v <= (1l << 30) ? (uint32_t)v : (1u << 19);
  }();
  RtHit* direct = nullptr;
  static const bool kDirectHits = [] {
    const char* e = std::getenv("RT_HOST_DIRECT_HITS");
    return e && e[0] == '1';
  }();
  if (kDirectHits) {
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, h_hits) == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer &&
        !misaligned(nullptr, pa.devicePointer))
      direct = static_cast<RtHit*>(pa.devicePointer);
    else
      cudaGetLastError();  // an unregistered pointer is not an error here
  }
  static const uint32_t kGrowth = [] {
    const char* e = std::getenv("RT_HOST_CHUNK_GROWTH");
    const long v = e ? std::atol(e) : 0;
    return v >= 2 && v <= 64 ? (uint32_t)v : 0u;
  }();
  const uint32_t growth = kGrowth ? kGrowth : (direct ? 8u : 4u);
  const uint32_t chunk = std::min<uint32_t>(n, direct ? (1u << 24) : (1u << 23));  // buffer capacity
  const size_t ray_bytes = (size_t)chunk * sizeof(RtRay), hit_bytes = direct ? 0 : (size_t)chunk * sizeof(RtHit);
  const size_t per = ray_bytes + hit_bytes;
  const size_t need = 2 * per;
  cudaError_t e;
  if (w->stage_bytes < need) {
    if (w->stage) cudaFree(w->stage);
    w->stage = nullptr;
    w->stage_bytes = 0;
    e = cudaMalloc(&w->stage, need);
    if (e != cudaSuccess) {
      set_error(std::string("rt_trace_host: staging cudaMalloc: ") + cudaGetErrorString(e));
      return RT_ENOMEM;
    }
    w->stage_bytes = need;
  }
  const size_t slot = sort_slot_bytes(chunk);
  if ((flags & RT_TRACE_SORT) && (s = ensure_sort_scratch(w, 2 * slot)) != RT_OK) return s;
  if ((s = ensure_helpers(w)) != RT_OK) return s;
  char* base = static_cast<char*>(w->stage);
  RtRay* drays[2] = {reinterpret_cast<RtRay*>(base), reinterpret_cast<RtRay*>(base + per)};
  RtHit* dhits[2] = {reinterpret_cast<RtHit*>(base + ray_bytes), reinterpret_cast<RtHit*>(base + per + ray_bytes)};
  cudaStream_t tst[2] = {st, w->trace2};
  uint32_t* counters[2] = {w->counters, w->counters + 4};
  cudaEvent_t* in_done = &w->ev[0];
  cudaEvent_t* trace_done = &w->ev[2];
  cudaEvent_t* out_done = &w->ev[4];
  // buffers b are free again once chunk c-2 is traced (direct) or downloaded
  cudaEvent_t* free_again = direct ? trace_done : out_done;
  // Every error return from here on first waits for the helper streams and
  // the caller's stream: nothing this call enqueued may still touch h_rays
  // or h_hits after it returns.
  auto drain = [&](rt_status rs) {
    for (cudaStream_t h : {w->copy_in, w->trace2, w->copy_out, st}) cudaStreamSynchronize(h);
    return rs;
  };
  // the caller's earlier work on `stream` comes first (trace2 follows it
  // through copy_in's events)
  if ((e = cudaEventRecord(w->ev[6], st)) != cudaSuccess) return drain(cuda_fail(e, "event"));
  if ((e = cudaStreamWaitEvent(w->copy_in, w->ev[6], 0)) != cudaSuccess) return drain(cuda_fail(e, "wait"));
  uint32_t chunks = 0;
  auto enqueue = [&]() -> rt_status {
    uint32_t size = std::min(chunk, kFirstChunk);
    for (uint32_t c = 0, off = 0, cnt = 0; off < n;
         ++c, off += cnt, size = (uint32_t)std::min<uint64_t>((uint64_t)growth * size, chunk)) {
      const uint32_t b = c & 1u;
      cnt = std::min(size, n - off);
      // staged: leave exactly kLastChunk rays for the last chunk
      if (!direct && kLastChunk && n - off > kLastChunk && n - off - cnt < kLastChunk) cnt = n - off - kLastChunk;
      chunks = c + 1;
      if (c >= 2 && (e = cudaStreamWaitEvent(w->copy_in, free_again[b], 0)) != cudaSuccess)
        return cuda_fail(e, "wait");
      if ((e = cudaMemcpyAsync(drays[b], h_rays + off, (size_t)cnt * sizeof(RtRay), cudaMemcpyHostToDevice,
                               w->copy_in)) != cudaSuccess)
        return cuda_fail(e, "rt_trace_host: H2D");
      if ((e = cudaEventRecord(in_done[b], w->copy_in)) != cudaSuccess) return cuda_fail(e, "event");
      if ((e = cudaStreamWaitEvent(tst[b], in_done[b], 0)) != cudaSuccess) return cuda_fail(e, "wait");
      uint32_t* order = nullptr;
      rt_status rs = maybe_reorder(w, scene->d, drays[b], cnt, flags, tst[b], &order, b * slot);
      if (rs != RT_OK) return rs;
      if ((e = cudaMemsetAsync(counters[b], 0, 2 * sizeof(uint32_t), tst[b])) != cudaSuccess)
        return cuda_fail(e, "memset");
      RtHit* out = direct ? direct + off : dhits[b];
      if ((e = launch_trace_tuned(scene->d, drays[b], cnt, out, flags, counters[b], tst[b],
                                  (flags & RT_TRACE_MT) ? default_tuning() : scene->tune, nullptr, order)) != cudaSuccess)
        return cuda_fail(e, "rt_trace_host: launch");
      if ((e = cudaEventRecord(trace_done[b], tst[b])) != cudaSuccess) return cuda_fail(e, "event");
      if (direct) continue;
      if ((e = cudaStreamWaitEvent(w->copy_out, trace_done[b], 0)) != cudaSuccess) return cuda_fail(e, "wait");
      if ((e = cudaMemcpyAsync(h_hits + off, dhits[b], (size_t)cnt * sizeof(RtHit), cudaMemcpyDeviceToHost,
                               w->copy_out)) != cudaSuccess)
        return cuda_fail(e, "rt_trace_host: D2H");
      if ((e = cudaEventRecord(out_done[b], w->copy_out)) != cudaSuccess) return cuda_fail(e, "event");
    }
    return RT_OK;
  };
  if ((s = enqueue()) != RT_OK) return drain(s);
  if (direct) {
    // the caller's stream continues after trace2's last chunk; its own chunks
    // are already in order on it
    if (chunks >= 2 && (e = cudaStreamWaitEvent(st, trace_done[1], 0)) != cudaSuccess)
      return drain(cuda_fail(e, "wait"));
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return drain(cuda_fail(e, "rt_trace_host: sync"));
    return RT_OK;
  }
  // the caller's stream continues after the last download (every chunk's
  // download waited for its trace, so trace2 is drained too)
  if ((e = cudaEventRecord(w->ev[7], w->copy_out)) != cudaSuccess) return drain(cuda_fail(e, "event"));
  if ((e = cudaStreamWaitEvent(st, w->ev[7], 0)) != cudaSuccess) return drain(cuda_fail(e, "wait"));
  if ((e = cudaStreamSynchronize(w->copy_out)) != cudaSuccess) return drain(cuda_fail(e, "rt_trace_host: sync"));
  return RT_OK;
}

static rt_status render_impl(rt_scene* scene, const RtRaytraceUBO* ubo, float* d_accum, uint32_t width,
                             uint32_t height, uint32_t spp, const RtRenderOptions* opt, void* stream,
                             uint64_t* h_counts, const char* who) {
  if (!scene || !ubo || !d_accum || width == 0 || height == 0 || (uint64_t)width * height > 0x40000000ull) {
    set_error(std::string(who) + ": bad argument");
    return RT_EINVAL;
  }
  if (scene->max_material > scene->d.n_mats) {
    set_error(std::string(who) + ": a primitive names a material index >= num_materials");
    return RT_EINVAL;
  }
  RtRenderOptions o;
  std::memset(&o, 0, sizeof(o));
  if (opt) o = *opt;
  if (o.shade_mode != RT_SHADE_REFERENCE && o.shade_mode != RT_SHADE_EXTENDED) {
    set_error(std::string(who) + ": unknown shade_mode");
    return RT_EINVAL;
  }
  if (o.flags & ~RT_RENDER_TRACE_EVERY_PRIMARY) {
    set_error(std::string(who) + ": unknown flags");
    return RT_EINVAL;
  }
  if (h_counts) h_counts[0] = h_counts[1] = h_counts[2] = 0;
  if (spp == 0) return RT_OK;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  Workspace* w = nullptr;
  rt_status s = workspace(st, &w);
  if (s != RT_OK) return s;
  float cam[12];
  camera_setup(*ubo, width, height, cam);
  // Paths in flight of the wavefront renderer: the whole frame up to 16 Mi
  // paths (about 1.9 GB of scratch); larger frames run in passes.
  static const uint64_t kMaxWavePaths = [] {
    const char* v = std::getenv("RT_RENDER_WAVE_PATHS");
    const long long x = v ? std::atoll(v) : 0;
    return x >= 1 && x <= (1ll << 30) ? (uint64_t)x : (uint64_t)1 << 24;
  }();
  uint64_t wave_paths = 0;
  if (render_uses_scratch(scene->d, ubo->maxRayTraceDepth)) {
    wave_paths = std::min<uint64_t>((uint64_t)width * height * spp, kMaxWavePaths);
    const size_t need = render_scratch_bytes(wave_paths, ubo->maxRayTraceDepth);
    if (w->wave_bytes < need) {
      if (w->wave) cudaFree(w->wave);
      w->wave = nullptr;
      w->wave_bytes = 0;
      cudaError_t e = cudaMalloc(&w->wave, need);
      if (e != cudaSuccess) {
        set_error(std::string(who) + ": wavefront scratch cudaMalloc: " + cudaGetErrorString(e));
        return RT_ENOMEM;
      }
      w->wave_bytes = need;
    }
  }
  cudaError_t e = cudaMemsetAsync(w->counters, 0, (h_counts ? 16 : 2) * sizeof(uint32_t), st);
  if (e != cudaSuccess) return cuda_fail(e, "rt_render: memset");
  unsigned long long* stats = h_counts ? reinterpret_cast<unsigned long long*>(w->counters + 8) : nullptr;
  const uint32_t mode = (o.shade_mode == RT_SHADE_EXTENDED ? kRenderExtended : 0u) |
                        ((o.flags & RT_RENDER_TRACE_EVERY_PRIMARY) ? kRenderTraceEveryPrimary : 0u);
  RenderStreams rs;
  if (wave_paths) {
    if ((s = ensure_helpers(w)) != RT_OK) return s;
    static const int kLanes = [] {
      const char* v = std::getenv("RT_RENDER_LANES");
      const int x = v ? std::atoi(v) : 0;
      return x >= 1 && x <= kWaveLanes ? x : 2;
    }();
    rs.extra = kLanes - 1;
    rs.streams[0] = w->trace2;
    rs.streams[1] = w->copy_out;
    rs.fork = w->ev[6];
    rs.join[0] = w->ev[7];
    rs.join[1] = w->ev[5];
  }
  e = launch_render(scene->d, cam, ubo->maxRayTraceDepth, ubo->randomState, d_accum, width, height, spp, mode,
                    o.background, w->counters, stream, stats, w->wave, wave_paths, &rs);
  if (e != cudaSuccess) return cuda_fail(e, "rt_render: launch");
  if (h_counts) {
    unsigned long long hc[3] = {0, 0, 0};
    e = cudaMemcpyAsync(hc, stats, sizeof(hc), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "rt_render_count: read counters");
    for (int k = 0; k < 3; ++k) h_counts[k] = hc[k];
  }
  return RT_OK;
}

rt_status rt_render(rt_scene* scene, const RtRaytraceUBO* ubo, float* d_accum, uint32_t width, uint32_t height,
                    uint32_t spp, const RtRenderOptions* opt, void* stream) {
  rtgb::NvtxRange nvtx_range("rt_render");
  return render_impl(scene, ubo, d_accum, width, height, spp, opt, stream, nullptr, "rt_render");
}

rt_status rt_render_count(rt_scene* scene, const RtRaytraceUBO* ubo, float* d_accum, uint32_t width, uint32_t height,
                          uint32_t spp, const RtRenderOptions* opt, void* stream, uint64_t* h_counts) {
  rtgb::NvtxRange nvtx_range("rt_render_count");
  if (!h_counts) {
    set_error("rt_render_count: bad argument");
    return RT_EINVAL;
  }
  return render_impl(scene, ubo, d_accum, width, height, spp, opt, stream, h_counts, "rt_render_count");
}

rt_status rt_accum_clear(float* d_accum, uint32_t width, uint32_t height, void* stream) {
  rtgb::NvtxRange nvtx_range("rt_accum_clear");
  if (!d_accum || (uint64_t)width * height > 0x40000000ull) {
    set_error("rt_accum_clear: bad argument");
    return RT_EINVAL;
  }
  cudaError_t e = launch_accum_clear(d_accum, width, height, stream);
  return e == cudaSuccess ? RT_OK : cuda_fail(e, "rt_accum_clear");
}

rt_status rt_resolve(const float* d_accum, uint32_t width, uint32_t height, uint32_t spp, float* d_out, void* stream) {
  rtgb::NvtxRange nvtx_range("rt_resolve");
  if (!d_accum || !d_out || spp == 0 || (uint64_t)width * height > 0x40000000ull) {
    set_error("rt_resolve: bad argument");
    return RT_EINVAL;
  }
  cudaError_t e = launch_resolve(d_accum, width, height, spp, d_out, stream);
  return e == cudaSuccess ? RT_OK : cuda_fail(e, "rt_resolve");
}

}  // extern "C"
