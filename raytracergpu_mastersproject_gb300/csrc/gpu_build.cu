// gpu_build.cu -- the reference's S1 pass (RaytracerBVH.cpp:778-991) on the GPU.
//
// Same node layout and the same binary32 operations as the host builder
// (host_bvh.cpp), so the two emit identical 40-byte node arrays:
//   k_centroid_box   centroids ((v0+v1)+v2)/3, min/max fold from +-1e9
//                    (GetEnclosingAABB.comp:64-109); block reduction, then
//                    atomicMin/Max on order-preserving integer images of floats
//   k_pad_box        the padding of :105-109, one thread
//   k_morton         30-bit codes (GenerateMortonCodesOfPrimitives.comp:52-93)
//   radix sort       stable LSD sort of (code, index), 4 passes of 8 bits like
//                    RadixSortSimple.comp:8-13: per-tile histograms, a scan, and
//                    a scatter whose ranks keep input order (warp multi-split)
//   k_leaves         padded leaf boxes (ConstructHLBVH.comp:117-169)
//   k_karras         internal nodes: range and split (ConstructHLBVH.comp:72-209)
//   k_bottom_up      box unions, second arriving child continues upward
//                    (ConstructAABBsOfInternalNodes.comp:38-64)
#include <cuda_runtime.h>

#include <cstring>

#include "rt_internal.h"

namespace rtgb {

void set_error(const std::string& msg);

namespace {

constexpr int kT = 256;            // threads per block
constexpr int kItems = 16;         // keys per thread in the sort tiles
constexpr int kTile = kT * kItems;  // 4096 keys per tile
constexpr int kBins = 256;

__device__ __forceinline__ uint32_t f2ord(float f) {  // order-preserving float -> uint
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

__device__ __forceinline__ void centroid(const RtTriangle64* tris, const RtSphere32* sph, uint32_t nt, uint32_t i,
                                         float c[3]) {
  if (i < nt) {
    const RtTriangle64& t = tris[i];
    for (int k = 0; k < 3; ++k) c[k] = (t.v0[k] + t.v1[k] + t.v2[k]) / 3.0f;
  } else {
    const RtSphere32& s = sph[i - nt];
    for (int k = 0; k < 3; ++k) c[k] = s.center[k];
  }
}

__global__ void k_centroid_box(const RtTriangle64* tris, const RtSphere32* sph, uint32_t nt, uint32_t n,
                               uint32_t* box /* ord: min xyz, max xyz */) {
  float mn[3] = {1000000000.0f, 1000000000.0f, 1000000000.0f};
  float mx[3] = {-1000000000.0f, -1000000000.0f, -1000000000.0f};
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float c[3];
    centroid(tris, sph, nt, i, c);
    for (int k = 0; k < 3; ++k) {
      mn[k] = fminf(mn[k], c[k]);
      mx[k] = fmaxf(mx[k], c[k]);
    }
  }
  for (int k = 0; k < 3; ++k)
    for (int o = 16; o > 0; o >>= 1) {
      mn[k] = fminf(mn[k], __shfl_down_sync(0xFFFFFFFFu, mn[k], o));
      mx[k] = fmaxf(mx[k], __shfl_down_sync(0xFFFFFFFFu, mx[k], o));
    }
  if ((threadIdx.x & 31u) == 0)
    for (int k = 0; k < 3; ++k) {
      atomicMin(&box[k], f2ord(mn[k]));
      atomicMax(&box[3 + k], f2ord(mx[k]));
    }
}

__global__ void k_pad_box(const uint32_t* ordbox, float* box) {
  const float delta = 0.001f, padding = delta / 2.0f;
  for (int k = 0; k < 3; ++k) {
    float mn = ord2f(ordbox[k]), mx = ord2f(ordbox[3 + k]);
    if (mx - mn < delta) {
      mn -= padding;
      mx += padding;
    }
    box[k] = mn;
    box[3 + k] = mx;
  }
}

__device__ __forceinline__ uint32_t f2u_sat(float f) { return __float2uint_rz(f); }

__device__ __forceinline__ uint32_t spread3(uint32_t v) {
  if (v == 1024u) v--;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

__global__ void k_morton(const RtTriangle64* tris, const RtSphere32* sph, uint32_t nt, uint32_t n, const float* box,
                         uint32_t mode, uint32_t* codes, uint32_t* idx) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float c[3];
  centroid(tris, sph, nt, i, c);
  uint32_t q[3];
  for (int k = 0; k < 3; ++k) {
    const float span = box[3 + k] - box[k];
    const float off = mode == RT_BVH_REFERENCE ? c[k] / span : (c[k] - box[k]) / span;
    q[k] = f2u_sat(off * 1024.0f);
  }
  codes[i] = (spread3(q[2]) << 2) | (spread3(q[1]) << 1) | spread3(q[0]);
  idx[i] = i;
}

// ---- stable LSD radix sort, 8-bit digits ----
// hist layout: [bin][tile], so an exclusive scan in that order gives each
// (bin, tile) its output base.
__global__ void __launch_bounds__(kT) k_rs_hist(const uint32_t* keys, uint32_t n, uint32_t shift, uint32_t* hist,
                                                uint32_t tiles) {
  __shared__ uint32_t h[kBins];
  h[threadIdx.x] = 0u;
  __syncthreads();
  const uint32_t base = blockIdx.x * kTile;
  for (int j = 0; j < kItems; ++j) {
    const uint32_t i = base + j * kT + threadIdx.x;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of `len` counts in place, one block of 1024 threads, in
// chunks of 8192: each thread sums 8 consecutive counts, a warp scan with
// __shfl_up_sync and a scan of the 32 warp totals give each thread its
// starting offset, and a running carry links the chunks.  (Loads of
// consecutive threads stay within the same sectors; a thread-per-stretch
// serial scan made every load of a warp touch 32 lines.)
__global__ void __launch_bounds__(1024) k_scan_inplace(uint32_t* a, uint32_t len) {
  __shared__ uint32_t warp_sums[32];
  const uint32_t t = threadIdx.x, lane = t & 31u, w = t >> 5;
  uint32_t carry = 0;
  for (uint32_t base = 0; base < len; base += 8192u) {
    const uint32_t i0 = base + 8u * t;
    uint32_t v[8], sum = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      v[k] = i0 + k < len ? a[i0 + k] : 0u;
      sum += v[k];
    }
    uint32_t x = sum;  // inclusive scan over the warp
#pragma unroll
    for (uint32_t off = 1; off < 32; off <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, off);
      if (lane >= off) x += y;
    }
    if (lane == 31u) warp_sums[w] = x;
    __syncthreads();
    if (w == 0) {
      uint32_t z = warp_sums[lane];
#pragma unroll
      for (uint32_t off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, z, off);
        if (lane >= off) z += y;
      }
      warp_sums[lane] = z;  // inclusive prefix of the warp totals
    }
    __syncthreads();
    uint32_t run = carry + (w ? warp_sums[w - 1] : 0u) + x - sum;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (i0 + k < len) a[i0 + k] = run;
      run += v[k];
    }
    carry += warp_sums[31];
    __syncthreads();  // warp_sums is rewritten by the next chunk
  }
}

// Each warp owns a contiguous 512-key stretch of the tile and walks it in
// order, 32 keys at a time; equal digits within a step are ranked by lane
// (__match_any_sync), and per-warp running counts keep earlier steps ahead.
__global__ void __launch_bounds__(kT) k_rs_scatter(const uint32_t* keys, const uint32_t* vals, uint32_t n,
                                                   uint32_t shift, const uint32_t* offs, uint32_t tiles,
                                                   uint32_t* keys_out, uint32_t* vals_out) {
  constexpr int kWarps = kT / 32;
  constexpr int kPerWarp = kTile / kWarps;  // 512
  __shared__ uint32_t cnt[kWarps][kBins];
  const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
  for (int b = lane; b < kBins; b += 32) cnt[w][b] = 0u;
  __syncwarp();
  const uint32_t base = blockIdx.x * kTile + w * kPerWarp;
  // pass 1: this warp's digit counts
  for (int s = 0; s < kPerWarp; s += 32) {
    const uint32_t i = base + s + lane;
    const bool ok = i < n;
    const uint32_t d = ok ? (keys[i] >> shift) & 255u : 256u;
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
    if (ok && lane == (uint32_t)(__ffs(peers) - 1)) cnt[w][d] += (uint32_t)__popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // per bin: global base of this tile + counts of earlier warps
  {
    const uint32_t b = threadIdx.x;  // kT == kBins
    uint32_t run = offs[b * tiles + blockIdx.x];
    for (int ww = 0; ww < kWarps; ++ww) {
      const uint32_t c = cnt[ww][b];
      cnt[ww][b] = run;
      run += c;
    }
  }
  __syncthreads();
  // pass 2: place keys in order
  for (int s = 0; s < kPerWarp; s += 32) {
    const uint32_t i = base + s + lane;
    const bool ok = i < n;
    const uint32_t k = ok ? keys[i] : 0u;
    const uint32_t d = ok ? (k >> shift) & 255u : 256u;
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
    const uint32_t lt = peers & ((1u << lane) - 1u);
    if (ok) {
      const uint32_t pos = cnt[w][d] + (uint32_t)__popc(lt);
      keys_out[pos] = k;
      vals_out[pos] = vals[i];
    }
    __syncwarp();
    if (ok && lane == (uint32_t)(__ffs(peers) - 1)) cnt[w][d] += (uint32_t)__popc(peers);
    __syncwarp();
  }
}

__device__ __forceinline__ void pad_axis(float& mn, float& mx) {
  const float delta = 0.001f, padding = delta / 2.0f;
  if (mx - mn < delta) {
    mn -= padding;
    mx += padding;
  }
}

__global__ void k_leaves(const RtTriangle64* tris, const RtSphere32* sph, uint32_t nt, uint32_t n, uint32_t mode,
                         const uint32_t* order, RtBVHNode40* nodes) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t g = mode == RT_BVH_REFERENCE ? k : order[k];
  RtBVHNode40 nd;
  if (g < nt) {
    const RtTriangle64& t = tris[g];
    nd.minX = fminf(t.v0[0], fminf(t.v1[0], t.v2[0]));
    nd.maxX = fmaxf(t.v0[0], fmaxf(t.v1[0], t.v2[0]));
    nd.minY = fminf(t.v0[1], fminf(t.v1[1], t.v2[1]));
    nd.maxY = fmaxf(t.v0[1], fmaxf(t.v1[1], t.v2[1]));
    nd.minZ = fminf(t.v0[2], fminf(t.v1[2], t.v2[2]));
    nd.maxZ = fmaxf(t.v0[2], fmaxf(t.v1[2], t.v2[2]));
    nd.primitiveIndex = g;
    nd.primitiveType = RT_PRIM_TRIANGLE;
  } else {
    const RtSphere32& s = sph[g - nt];
    float l[3], r[3];
    for (int a = 0; a < 3; ++a) {
      l[a] = s.center[a] - s.radius;
      r[a] = s.center[a] + s.radius;
    }
    nd.minX = fminf(l[0], r[0]);
    nd.maxX = fmaxf(l[0], r[0]);
    nd.minY = fminf(l[1], r[1]);
    nd.maxY = fmaxf(l[1], r[1]);
    nd.minZ = fminf(l[2], r[2]);
    nd.maxZ = fmaxf(l[2], r[2]);
    nd.primitiveIndex = g - nt;
    nd.primitiveType = RT_PRIM_SPHERE;
  }
  pad_axis(nd.minX, nd.maxX);
  pad_axis(nd.minY, nd.maxY);
  pad_axis(nd.minZ, nd.maxZ);
  nd.left = 0;
  nd.right = 0;
  nodes[(n - 1) + k] = nd;
}

__device__ __forceinline__ int delta(const uint32_t* codes, int n, int i, int j) {
  if (j < 0 || j > n - 1) return -1;
  const uint32_t ci = codes[i], cj = codes[j];
  if (ci == cj) return 32 + __clz((int)((uint32_t)i ^ (uint32_t)j));
  return __clz((int)(ci ^ cj));
}

__global__ void k_karras(const uint32_t* codes, uint32_t N, RtBVHNode40* nodes, uint32_t* parent, int* visits) {
  const int id = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int n = (int)N;
  if (id >= n - 1) return;
  const int dl = delta(codes, n, id, id - 1), dr = delta(codes, n, id, id + 1);
  const int dir = dr >= dl ? 1 : -1;
  const int dmin = min(dl, dr);
  int lmax = 2;
  while (delta(codes, n, id, id + lmax * dir) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t > 0; t >>= 1)
    if (delta(codes, n, id, id + (l + t) * dir) > dmin) l += t;
  const int end = id + l * dir;
  const int first = min(id, end), last = max(id, end);
  const int common = delta(codes, n, first, last);
  int split = first, stride = last - first;
  do {
    stride = (stride + 1) >> 1;
    const int ns = split + stride;
    if (ns < last && delta(codes, n, first, ns) > common) split = ns;
  } while (stride > 1);
  const uint32_t leaf_off = N - 1;
  const uint32_t lc = (uint32_t)(split == first ? (int)leaf_off + split : split);
  const uint32_t rc = (uint32_t)(split + 1 == last ? (int)leaf_off + split + 1 : split + 1);
  RtBVHNode40 nd;
  nd.minX = nd.maxX = nd.minY = nd.maxY = nd.minZ = nd.maxZ = 0.0f;
  nd.left = lc;
  nd.right = rc;
  nd.primitiveIndex = 0;
  nd.primitiveType = 0;
  nodes[id] = nd;
  parent[lc] = (uint32_t)id;
  parent[rc] = (uint32_t)id;
  visits[id] = 0;
}

// Children's boxes are read with ld.global.cg (L2, not a stale L1 line).
__global__ void k_bottom_up(uint32_t N, RtBVHNode40* nodes, const uint32_t* parent, int* visits) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N || N < 2) return;
  uint32_t node = parent[(N - 1) + i];
  for (;;) {
    __threadfence();
    const int v = atomicAdd(&visits[node], 1);
    if (v < 1) return;
    RtBVHNode40* nd = &nodes[node];
    const uint32_t L = __ldcg(&nd->left), R = __ldcg(&nd->right);
    const float* a = reinterpret_cast<const float*>(&nodes[L]);
    const float* b = reinterpret_cast<const float*>(&nodes[R]);
    float r[6];
    for (int k = 0; k < 6; ++k) {
      const float x = __ldcg(&a[k]), y = __ldcg(&b[k]);
      r[k] = (k & 1) ? fmaxf(x, y) : fminf(x, y);
    }
    nd->minX = r[0]; nd->maxX = r[1]; nd->minY = r[2]; nd->maxY = r[3]; nd->minZ = r[4]; nd->maxZ = r[5];
    if (node == 0) return;
    node = parent[node];
  }
}

}  // namespace

size_t device_build_scratch_bytes(uint32_t n) {
  const uint32_t tiles = (n + kTile - 1) / kTile;
  return 256 + (size_t)n * 4 * 4 + (size_t)kBins * tiles * 4 + (size_t)(2 * (size_t)n) * 4 * 2;
}

// nodes: 2n-1 records; scratch: device_build_scratch_bytes(n).
cudaError_t launch_device_build(const RtTriangle64* tris, uint32_t nt, const RtSphere32* sph, uint32_t ns,
                                uint32_t mode, RtBVHNode40* nodes, void* scratch, cudaStream_t st) {
  const uint32_t n = nt + ns;
  if (n == 0) return cudaSuccess;
  char* p = static_cast<char*>(scratch);
  uint32_t* ordbox = reinterpret_cast<uint32_t*>(p);
  float* box = reinterpret_cast<float*>(p + 64);
  p += 256;
  uint32_t* ka = reinterpret_cast<uint32_t*>(p);
  p += (size_t)n * 4;
  uint32_t* va = reinterpret_cast<uint32_t*>(p);
  p += (size_t)n * 4;
  uint32_t* kb = reinterpret_cast<uint32_t*>(p);
  p += (size_t)n * 4;
  uint32_t* vb = reinterpret_cast<uint32_t*>(p);
  p += (size_t)n * 4;
  const uint32_t tiles = (n + kTile - 1) / kTile;
  uint32_t* hist = reinterpret_cast<uint32_t*>(p);
  p += (size_t)kBins * tiles * 4;
  uint32_t* parent = reinterpret_cast<uint32_t*>(p);
  p += (size_t)(2 * (size_t)n) * 4;
  int* visits = reinterpret_cast<int*>(p);

  uint32_t init[6] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u};
  cudaError_t e = cudaMemcpyAsync(ordbox, init, sizeof(init), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  const uint32_t gb = (n + kT - 1) / kT;
  k_centroid_box<<<std::min<uint32_t>(gb, 1024u), kT, 0, st>>>(tris, sph, nt, n, ordbox);
  k_pad_box<<<1, 1, 0, st>>>(ordbox, box);
  k_morton<<<gb, kT, 0, st>>>(tris, sph, nt, n, box, mode, ka, va);
  uint32_t *kin = ka, *vin = va, *kout = kb, *vout = vb;
  for (int pass = 0; pass < 4; ++pass) {
    const uint32_t shift = 8u * (uint32_t)pass;
    k_rs_hist<<<tiles, kT, 0, st>>>(kin, n, shift, hist, tiles);
    k_scan_inplace<<<1, 1024, 0, st>>>(hist, kBins * tiles);
    k_rs_scatter<<<tiles, kT, 0, st>>>(kin, vin, n, shift, hist, tiles, kout, vout);
    std::swap(kin, kout);
    std::swap(vin, vout);
  }
  k_leaves<<<gb, kT, 0, st>>>(tris, sph, nt, n, mode, vin, nodes);
  if (n > 1) {
    k_karras<<<gb, kT, 0, st>>>(kin, n, nodes, parent, visits);
    k_bottom_up<<<gb, kT, 0, st>>>(n, nodes, parent, visits);
  }
  return cudaGetLastError();
}

}  // namespace rtgb

using namespace rtgb;

extern "C" rt_status rt_build_bvh_device(const RtTriangle64* d_triangles, uint32_t num_triangles,
                                         const RtSphere32* d_spheres, uint32_t num_spheres, uint32_t bvh_mode,
                                         RtBVHNode40* d_nodes, void* stream) {
  const uint64_t n = (uint64_t)num_triangles + num_spheres;
  if ((num_triangles && !d_triangles) || (num_spheres && !d_spheres) || (n && !d_nodes) ||
      (bvh_mode != RT_BVH_SORTED && bvh_mode != RT_BVH_REFERENCE) || n > kMaxTriangles) {
    set_error("rt_build_bvh_device: bad argument");
    return RT_EINVAL;
  }
  if (n == 0) return RT_OK;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  void* scratch = nullptr;
  cudaError_t e = cudaMallocAsync(&scratch, device_build_scratch_bytes((uint32_t)n), st);
  if (e != cudaSuccess) {
    set_error(std::string("rt_build_bvh_device: scratch: ") + cudaGetErrorString(e));
    return RT_ENOMEM;
  }
  e = launch_device_build(d_triangles, num_triangles, d_spheres, num_spheres, bvh_mode, d_nodes, scratch, st);
  cudaError_t e2 = cudaFreeAsync(scratch, st);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) {
    set_error(std::string("rt_build_bvh_device: ") + cudaGetErrorString(e));
    return RT_ECUDA;
  }
  return RT_OK;
}
