// host_bvh.cpp -- host BVH build in the reference node layout, and its
// conversion to the device form.
//
// The build reproduces the six S1 compute passes of the reference
// (RaytracerBVH.cpp:778-991) on the host, multi-threaded:
//   ModelSpaceToWorldSpace.comp:32-48          world_space()
//   GetEnclosingAABB.comp:64-109               centroid box, padded
//   GenerateMortonCodesOfPrimitives.comp:52-93 30-bit codes
//   RadixSortSimple.comp:59-157                stable LSD sort, 4 x 8 bits
//   ConstructHLBVH.comp:145-214                Karras internal nodes + leaves
//   ConstructAABBsOfInternalNodes.comp:38-64   bottom-up box union
// Mode RT_BVH_REFERENCE keeps the reference's two quirks: Morton quantisation
// of coord/span instead of (coord-min)/span (:60-65), and leaf slot k holding
// primitive k rather than the k-th sorted primitive (ConstructHLBVH.comp:152-169).
// Mode RT_BVH_SORTED corrects both; its node array has the same layout.
//
// This translation unit is compiled with -ffp-contract=off: every binary32
// operation is rounded on its own, in the order written, as the shaders state.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <thread>

#include "rt_internal.h"

namespace rtgb {

unsigned host_threads() {
  static unsigned cached = [] {
    unsigned n = std::thread::hardware_concurrency();
    if (const char* e = std::getenv("RT_HOST_THREADS")) {
      long v = std::strtol(e, nullptr, 10);
      if (v > 0) n = (unsigned)v;
    }
    if (n == 0) n = 1;
    if (n > 128) n = 128;
    return n;
  }();
  return cached;
}

static inline uint32_t f2u_sat(float f) {
  if (!(f > 0.0f)) return 0u;
  if (f >= 4294967296.0f) return 0xFFFFFFFFu;
  return (uint32_t)f;
}

// GenerateMortonCodesOfPrimitives.comp:41-50
static inline uint32_t spread3(uint32_t v) {
  if (v == 1024u) v--;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

static inline void pad_axis(float& mn, float& mx) {
  const float delta = 0.001f, padding = delta / 2.0f;  // ConstructHLBVH.comp:38-39
  if (mx - mn < delta) {
    mn -= padding;
    mx += padding;
  }
}

bool world_space(const RtTriangle64* tris, uint32_t nt, const RtSphere32* sph, uint32_t ns,
                 const RtModel64* models, uint32_t nm, std::vector<RtTriangle64>& out_t,
                 std::vector<RtSphere32>& out_s, std::string& msg) {
  out_t.assign(tris, tris + nt);
  out_s.assign(sph, sph + ns);
  if (!models) return true;
  for (uint32_t i = 0; i < nt; ++i)
    if (tris[i].modelIndex >= nm) {
      msg = "triangle " + std::to_string(i) + " has modelIndex out of range";
      return false;
    }
  for (uint32_t i = 0; i < ns; ++i)
    if (sph[i].modelIndex >= nm) {
      msg = "sphere " + std::to_string(i) + " has modelIndex out of range";
      return false;
    }
  // ModelSpaceToWorldSpace.comp:37-45: v' = M * vec4(v.xyz, 1), column-major M.
  auto xform = [](const float* m, float* v) {
    float x = v[0], y = v[1], z = v[2], w = 1.0f;
    float r[4];
    for (int row = 0; row < 4; ++row) r[row] = m[0 + row] * x + m[4 + row] * y + m[8 + row] * z + m[12 + row] * w;
    std::memcpy(v, r, sizeof(r));
  };
  parallel_for(nt, [&](size_t b, size_t e, unsigned) {
    for (size_t i = b; i < e; ++i) {
      const float* m = models[out_t[i].modelIndex].m;
      xform(m, out_t[i].v0);
      xform(m, out_t[i].v1);
      xform(m, out_t[i].v2);
    }
  });
  for (uint32_t i = 0; i < ns; ++i) xform(models[out_s[i].modelIndex].m, out_s[i].center);
  return true;
}

// Stable LSD radix sort of (key, value) by key, 4 passes of 8 bits
// (the bin width of RadixSortSimple.comp:8-13), parallel over chunks with
// per-chunk histograms so that equal keys keep their input order.
static void radix_sort_pairs(std::vector<uint32_t>& keys, std::vector<uint32_t>& vals) {
  size_t n = keys.size();
  std::vector<uint32_t> k2(n), v2(n);
  unsigned T = std::min<unsigned>(host_threads(), (unsigned)std::max<size_t>(1, n / 65536));
  if (T == 0) T = 1;
  size_t per = (n + T - 1) / T;
  std::vector<uint32_t> hist((size_t)T * 256);
  for (int pass = 0; pass < 4; ++pass) {
    uint32_t shift = 8u * (uint32_t)pass;
    std::fill(hist.begin(), hist.end(), 0u);
    auto count = [&](unsigned t) {
      size_t b = t * per, e = std::min(n, b + per);
      uint32_t* h = &hist[(size_t)t * 256];
      for (size_t i = b; i < e; ++i) h[(keys[i] >> shift) & 255u]++;
    };
    std::vector<std::thread> th;
    for (unsigned t = 1; t < T; ++t) th.emplace_back(count, t);
    count(0);
    for (auto& x : th) x.join();
    th.clear();
    uint32_t acc = 0;
    for (int bin = 0; bin < 256; ++bin)
      for (unsigned t = 0; t < T; ++t) {
        uint32_t c = hist[(size_t)t * 256 + bin];
        hist[(size_t)t * 256 + bin] = acc;
        acc += c;
      }
    auto scatter = [&](unsigned t) {
      size_t b = t * per, e = std::min(n, b + per);
      uint32_t* h = &hist[(size_t)t * 256];
      for (size_t i = b; i < e; ++i) {
        uint32_t dst = h[(keys[i] >> shift) & 255u]++;
        k2[dst] = keys[i];
        v2[dst] = vals[i];
      }
    };
    for (unsigned t = 1; t < T; ++t) th.emplace_back(scatter, t);
    scatter(0);
    for (auto& x : th) x.join();
    keys.swap(k2);
    vals.swap(v2);
  }
}

// ConstructHLBVH.comp:58-70
static inline int delta(const uint32_t* codes, int n, int i, int j) {
  if (j < 0 || j > n - 1) return -1;
  uint32_t ci = codes[i], cj = codes[j];
  if (ci == cj) return 32 + __builtin_clz((uint32_t)i ^ (uint32_t)j);
  return __builtin_clz(ci ^ cj);
}

void build_bvh(const RtTriangle64* tris, uint32_t nt, const RtSphere32* sph, uint32_t ns, uint32_t mode,
               std::vector<RtBVHNode40>& nodes) {
  const uint32_t N = nt + ns;
  nodes.clear();
  if (N == 0) return;
  nodes.resize(2 * (size_t)N - 1);

  // Centroids (GetEnclosingAABB.comp:40-42): ((v0 + v1 + v2) / 3).xyz
  std::vector<float> cen(3 * (size_t)N);
  parallel_for(N, [&](size_t b, size_t e, unsigned) {
    for (size_t i = b; i < e; ++i) {
      if (i < nt) {
        const RtTriangle64& t = tris[i];
        for (int k = 0; k < 3; ++k) cen[3 * i + k] = (t.v0[k] + t.v1[k] + t.v2[k]) / 3.0f;
      } else {
        const RtSphere32& s = sph[i - nt];
        for (int k = 0; k < 3; ++k) cen[3 * i + k] = s.center[k];
      }
    }
  });

  // Enclosing box of the centroids, preset to +-1e9 (GetEnclosingAABB.comp:72-76),
  // then padded (:105-109).
  unsigned T = host_threads();
  std::vector<float> part(6 * (size_t)T);
  for (unsigned t = 0; t < T; ++t)
    for (int k = 0; k < 3; ++k) {
      part[6 * t + k] = 1000000000.0f;
      part[6 * t + 3 + k] = -1000000000.0f;
    }
  parallel_for(N, [&](size_t b, size_t e, unsigned t) {
    float* p = &part[6 * (size_t)t];
    for (size_t i = b; i < e; ++i)
      for (int k = 0; k < 3; ++k) {
        p[k] = std::fmin(p[k], cen[3 * i + k]);
        p[3 + k] = std::fmax(p[3 + k], cen[3 * i + k]);
      }
  });
  float emin[3], emax[3];
  for (int k = 0; k < 3; ++k) {
    emin[k] = 1000000000.0f;
    emax[k] = -1000000000.0f;
    for (unsigned t = 0; t < T; ++t) {
      emin[k] = std::fmin(emin[k], part[6 * t + k]);
      emax[k] = std::fmax(emax[k], part[6 * t + 3 + k]);
    }
    pad_axis(emin[k], emax[k]);
  }

  // Morton codes (GenerateMortonCodesOfPrimitives.comp:60-65, 88-90).
  std::vector<uint32_t> codes(N), order(N);
  parallel_for(N, [&](size_t b, size_t e, unsigned) {
    for (size_t i = b; i < e; ++i) {
      uint32_t q[3];
      for (int k = 0; k < 3; ++k) {
        float span = emax[k] - emin[k];
        float off = mode == RT_BVH_REFERENCE ? cen[3 * i + k] / span : (cen[3 * i + k] - emin[k]) / span;
        q[k] = f2u_sat(off * 1024.0f);
      }
      codes[i] = (spread3(q[2]) << 2) | (spread3(q[1]) << 1) | spread3(q[0]);
      order[i] = (uint32_t)i;
    }
  });
  radix_sort_pairs(codes, order);

  // Leaves (ConstructHLBVH.comp:151-169), padded boxes (:41-54, 117-143).
  const uint32_t leaf_off = N - 1;
  parallel_for(N, [&](size_t b, size_t e, unsigned) {
    for (size_t k = b; k < e; ++k) {
      uint32_t g = mode == RT_BVH_REFERENCE ? (uint32_t)k : order[k];
      RtBVHNode40& nd = nodes[leaf_off + k];
      if (g < nt) {
        const RtTriangle64& t = tris[g];
        nd.minX = std::fmin(t.v0[0], std::fmin(t.v1[0], t.v2[0]));
        nd.maxX = std::fmax(t.v0[0], std::fmax(t.v1[0], t.v2[0]));
        nd.minY = std::fmin(t.v0[1], std::fmin(t.v1[1], t.v2[1]));
        nd.maxY = std::fmax(t.v0[1], std::fmax(t.v1[1], t.v2[1]));
        nd.minZ = std::fmin(t.v0[2], std::fmin(t.v1[2], t.v2[2]));
        nd.maxZ = std::fmax(t.v0[2], std::fmax(t.v1[2], t.v2[2]));
        nd.primitiveIndex = g;
        nd.primitiveType = RT_PRIM_TRIANGLE;
      } else {
        const RtSphere32& s = sph[g - nt];
        float l[3], r[3];
        for (int a = 0; a < 3; ++a) {
          l[a] = s.center[a] - s.radius;
          r[a] = s.center[a] + s.radius;
        }
        nd.minX = std::fmin(l[0], r[0]);
        nd.maxX = std::fmax(l[0], r[0]);
        nd.minY = std::fmin(l[1], r[1]);
        nd.maxY = std::fmax(l[1], r[1]);
        nd.minZ = std::fmin(l[2], r[2]);
        nd.maxZ = std::fmax(l[2], r[2]);
        nd.primitiveIndex = g - nt;
        nd.primitiveType = RT_PRIM_SPHERE;
      }
      pad_axis(nd.minX, nd.maxX);
      pad_axis(nd.minY, nd.maxY);
      pad_axis(nd.minZ, nd.maxZ);
      nd.left = 0;
      nd.right = 0;
    }
  });

  // Internal nodes: Karras range + split (ConstructHLBVH.comp:72-115, 171-209).
  std::vector<uint32_t> parent(2 * (size_t)N - 1, 0u);
  const uint32_t* C = codes.data();
  const int n = (int)N;
  parallel_for(N > 0 ? N - 1 : 0, [&](size_t b, size_t e, unsigned) {
    for (size_t ii = b; ii < e; ++ii) {
      int id = (int)ii;
      int dl = delta(C, n, id, id - 1), dr = delta(C, n, id, id + 1);
      int dir = dr >= dl ? 1 : -1;
      int dmin = std::min(dl, dr);
      int lmax = 2;
      while (delta(C, n, id, id + lmax * dir) > dmin) lmax <<= 1;
      int l = 0;
      for (int t = lmax >> 1; t > 0; t >>= 1)
        if (delta(C, n, id, id + (l + t) * dir) > dmin) l += t;
      int end = id + l * dir;
      int first = std::min(id, end), last = std::max(id, end);
      int common = delta(C, n, first, last);
      int split = first, stride = last - first;
      do {
        stride = (stride + 1) >> 1;
        int ns2 = split + stride;
        if (ns2 < last && delta(C, n, first, ns2) > common) split = ns2;
      } while (stride > 1);
      uint32_t lc = (uint32_t)(split == first ? (int)leaf_off + split : split);
      uint32_t rc = (uint32_t)(split + 1 == last ? (int)leaf_off + split + 1 : split + 1);
      RtBVHNode40& nd = nodes[ii];
      nd.minX = nd.maxX = nd.minY = nd.maxY = nd.minZ = nd.maxZ = 0.0f;
      nd.left = lc;
      nd.right = rc;
      nd.primitiveIndex = 0;
      nd.primitiveType = 0;
      parent[lc] = (uint32_t)ii;
      parent[rc] = (uint32_t)ii;
    }
  });
  if (N == 1) return;

  // Bottom-up boxes (ConstructAABBsOfInternalNodes.comp:38-64): the second
  // child to arrive at a node forms the union and continues upward.
  std::vector<std::atomic<int>> visits(N - 1);
  for (auto& v : visits) v.store(0, std::memory_order_relaxed);
  parallel_for(N, [&](size_t b, size_t e, unsigned) {
    for (size_t i = b; i < e; ++i) {
      uint32_t node = parent[leaf_off + i];
      for (;;) {
        int v = visits[node].fetch_add(1, std::memory_order_acq_rel);
        if (v < 1) break;
        RtBVHNode40& nd = nodes[node];
        const RtBVHNode40& L = nodes[nd.left];
        const RtBVHNode40& R = nodes[nd.right];
        nd.minX = std::fmin(L.minX, R.minX);
        nd.maxX = std::fmax(L.maxX, R.maxX);
        nd.minY = std::fmin(L.minY, R.minY);
        nd.maxY = std::fmax(L.maxY, R.maxY);
        nd.minZ = std::fmin(L.minZ, R.minZ);
        nd.maxZ = std::fmax(L.maxZ, R.maxZ);
        std::atomic_thread_fence(std::memory_order_release);
        if (node == 0) break;
        node = parent[node];
      }
    }
  });
}

// triangleHit's vertex-only values (raytraceBVH.comp:119-125), binary32.
// ------------------------------------------------ SAH traversal tree ----
// A binned surface-area-heuristic tree over the same primitives, in the node
// form convert_bvh reads (root 0, leaves with left == right == 0, one
// primitive per leaf, no leaf box flat).  Used for traversal only: closest hits do not depend
// on the tree, and the scene keeps the reference-layout nodes for export.
//
// Primitive records (bounds, centroid, id) are kept in tree order and
// partitioned in place, so every pass streams through memory.  A split bins
// the range's centroids into kSahBins bins on all three axes and takes the
// bin boundary of least  area(L) * |L| + area(R) * |R|; ranges of at most
// kSahSweep primitives are sorted along their widest centroid axis and take
// the exact split of that axis; a range whose centroids coincide is split in
// the middle, and past kSahDepth levels every split is at the centroid
// median, which bounds the depth.  The top of the tree is built with binning
// and partitioning spread over the host threads, subtrees below kSahTask
// primitives as parallel tasks.
namespace {

constexpr int kSahBins = 32;
constexpr size_t kSahTask = 1u << 15;
constexpr int kSahDepth = 48;
constexpr size_t kSahSweep = 16;

struct SahRec {
  float lo[3], hi[3], c[3];
  uint32_t id;
};

struct SahBox {
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  void grow(const float* l, const float* h) {
    for (int a = 0; a < 3; ++a) {
      lo[a] = l[a] < lo[a] ? l[a] : lo[a];
      hi[a] = h[a] > hi[a] ? h[a] : hi[a];
    }
  }
  void grow(const SahBox& b) { grow(b.lo, b.hi); }
  double area() const {
    const double dx = std::fmax(0.0, (double)hi[0] - lo[0]), dy = std::fmax(0.0, (double)hi[1] - lo[1]),
                 dz = std::fmax(0.0, (double)hi[2] - lo[2]);
    return dx * dy + dy * dz + dz * dx;
  }
};

struct SahBin {
  SahBox box;
  uint32_t count = 0;
};

struct SahBuild {
  uint32_t nt = 0;
  // uninitialised (no zero fill): every record and node is written before it
  // is read, by the threads that build, so the first-touch faults spread too
  std::unique_ptr<SahRec[]> rec, tmp;
  RtBVHNode40* out = nullptr;
  std::atomic<uint32_t> next{1};

  static void set_box(RtBVHNode40& nd, const SahBox& b) {
    nd.minX = b.lo[0]; nd.maxX = b.hi[0];
    nd.minY = b.lo[1]; nd.maxY = b.hi[1];
    nd.minZ = b.lo[2]; nd.maxZ = b.hi[2];
  }
  void leaf(uint32_t node, const SahRec& r) {
    RtBVHNode40& nd = out[node];
    SahBox b;
    b.grow(r.lo, r.hi);
    set_box(nd, b);
    nd.left = nd.right = 0;
    if (r.id < nt) {
      nd.primitiveIndex = r.id;
      nd.primitiveType = RT_PRIM_TRIANGLE;
    } else {
      nd.primitiveIndex = r.id - nt;
      nd.primitiveType = RT_PRIM_SPHERE;
    }
  }
  void bounds(size_t b, size_t e, bool par, SahBox& box, SahBox& cb) const {
    auto part = [&](size_t i0, size_t i1, SahBox& bx, SahBox& cx) {
      for (size_t i = i0; i < i1; ++i) {
        bx.grow(rec[i].lo, rec[i].hi);
        cx.grow(rec[i].c, rec[i].c);
      }
    };
    if (!par) {
      part(b, e, box, cb);
      return;
    }
    std::vector<SahBox> bx(host_threads()), cx(host_threads());
    parallel_for(e - b, [&](size_t i0, size_t i1, unsigned t) { part(b + i0, b + i1, bx[t], cx[t]); });
    for (size_t t = 0; t < bx.size(); ++t) {
      box.grow(bx[t]);
      cb.grow(cx[t]);
    }
  }
  // Moves the records of [b, e) for which `left` holds to the front, in
  // parallel through the scratch array when `par`; returns the split point.
  template <class P>
  size_t partition(size_t b, size_t e, bool par, P left) {
    if (!par) {
      SahRec* m = std::partition(rec.get() + b, rec.get() + e, left);
      return (size_t)(m - rec.get());
    }
    const unsigned T = host_threads();
    const size_t n = e - b, per = (n + T - 1) / T;
    std::vector<size_t> nl(T, 0), nr(T, 0);
    std::vector<std::thread> th;
    for (unsigned t = 0; t < T; ++t)
      th.emplace_back([&, t] {
        const size_t i0 = b + std::min(n, t * per), i1 = b + std::min(n, (t + 1) * per);
        for (size_t i = i0; i < i1; ++i) (left(rec[i]) ? nl[t] : nr[t])++;
      });
    for (auto& x : th) x.join();
    th.clear();
    size_t total_l = 0;
    for (unsigned t = 0; t < T; ++t) total_l += nl[t];
    std::vector<size_t> ol(T), orr(T);
    size_t accl = b, accr = b + total_l;
    for (unsigned t = 0; t < T; ++t) {
      ol[t] = accl;
      orr[t] = accr;
      accl += nl[t];
      accr += nr[t];
    }
    for (unsigned t = 0; t < T; ++t)
      th.emplace_back([&, t] {
        const size_t i0 = b + std::min(n, t * per), i1 = b + std::min(n, (t + 1) * per);
        size_t l = ol[t], r = orr[t];
        for (size_t i = i0; i < i1; ++i) tmp[left(rec[i]) ? l++ : r++] = rec[i];
      });
    for (auto& x : th) x.join();
    parallel_for(n, [&](size_t i0, size_t i1, unsigned) {
      std::memcpy(&rec[b + i0], &tmp[b + i0], (i1 - i0) * sizeof(SahRec));
    });
    return b + total_l;
  }
  // Splits [b, e), fills the node's box and returns the split point.
  size_t split(uint32_t node, size_t b, size_t e, bool par, int depth) {
    SahBox box, cb;
    bounds(b, e, par, box, cb);
    set_box(out[node], box);
    const size_t n = e - b;
    int wide = 0;
    for (int k = 1; k < 3; ++k)
      if (cb.hi[k] - cb.lo[k] > cb.hi[wide] - cb.lo[wide]) wide = k;
    auto by_axis = [wide](const SahRec& p, const SahRec& q) { return p.c[wide] < q.c[wide]; };
    if (depth >= kSahDepth) {
      const size_t mid = b + n / 2;
      std::nth_element(rec.get() + (ptrdiff_t)b, rec.get() + (ptrdiff_t)mid, rec.get() + (ptrdiff_t)e, by_axis);
      return mid;
    }
    if (n <= kSahSweep) {
      std::sort(rec.get() + (ptrdiff_t)b, rec.get() + (ptrdiff_t)e, by_axis);
      double right[kSahSweep];
      SahBox acc;
      for (size_t i = n - 1; i > 0; --i) {
        acc.grow(rec[b + i].lo, rec[b + i].hi);
        right[i] = acc.area() * (double)(n - i);
      }
      acc = SahBox();
      double best = INFINITY;
      size_t at = n / 2;
      for (size_t i = 1; i < n; ++i) {
        acc.grow(rec[b + i - 1].lo, rec[b + i - 1].hi);
        const double c = acc.area() * (double)i + right[i];
        if (c < best) {
          best = c;
          at = i;
        }
      }
      return b + at;
    }
    float scale[3];
    for (int a = 0; a < 3; ++a) {
      const float ext = cb.hi[a] - cb.lo[a];
      scale[a] = ext > 0.0f ? (float)kSahBins / ext : 0.0f;
    }
    auto bin_of = [&](const SahRec& p, int a) {
      const int k = (int)((p.c[a] - cb.lo[a]) * scale[a]);
      return k < 0 ? 0 : (k >= kSahBins ? kSahBins - 1 : k);
    };
    auto fill = [&](size_t i0, size_t i1, SahBin (*bins)[kSahBins]) {
      for (size_t i = i0; i < i1; ++i)
        for (int a = 0; a < 3; ++a)
          if (scale[a] > 0.0f) {
            SahBin& bn = bins[a][bin_of(rec[i], a)];
            bn.box.grow(rec[i].lo, rec[i].hi);
            bn.count++;
          }
    };
    SahBin bins[3][kSahBins];
    if (!par) {
      fill(b, e, bins);
    } else {
      std::vector<SahBin> tb((size_t)host_threads() * 3 * kSahBins);
      parallel_for(n, [&](size_t i0, size_t i1, unsigned t) {
        fill(b + i0, b + i1, reinterpret_cast<SahBin(*)[kSahBins]>(&tb[(size_t)t * 3 * kSahBins]));
      });
      for (unsigned t = 0; t < host_threads(); ++t)
        for (int a = 0; a < 3; ++a)
          for (int k = 0; k < kSahBins; ++k) {
            const SahBin& x = tb[((size_t)t * 3 + a) * kSahBins + k];
            if (x.count) {
              bins[a][k].box.grow(x.box);
              bins[a][k].count += x.count;
            }
          }
    }
    double best = INFINITY;
    int best_axis = -1, best_k = 0;
    for (int a = 0; a < 3; ++a) {
      if (scale[a] <= 0.0f) continue;
      double right_area[kSahBins];
      uint32_t right_count[kSahBins];
      SahBox acc;
      uint32_t cnt = 0;
      for (int k = kSahBins - 1; k > 0; --k) {
        if (bins[a][k].count) acc.grow(bins[a][k].box);
        cnt += bins[a][k].count;
        right_area[k] = acc.area();
        right_count[k] = cnt;
      }
      acc = SahBox();
      cnt = 0;
      for (int k = 0; k < kSahBins - 1; ++k) {
        if (bins[a][k].count) acc.grow(bins[a][k].box);
        cnt += bins[a][k].count;
        if (cnt == 0 || right_count[k + 1] == 0) continue;
        const double c = acc.area() * cnt + right_area[k + 1] * right_count[k + 1];
        if (c < best) {
          best = c;
          best_axis = a;
          best_k = k;
        }
      }
    }
    if (best_axis < 0) return b + n / 2;  // coincident centroids
    const int a = best_axis, k = best_k;
    const size_t mid = partition(b, e, par, [&](const SahRec& p) { return bin_of(p, a) <= k; });
    return mid == b || mid == e ? b + n / 2 : mid;
  }
  void children(uint32_t node, uint32_t& l, uint32_t& r) {
    const uint32_t c = next.fetch_add(2);
    l = c;
    r = c + 1;
    out[node].left = l;
    out[node].right = r;
    out[node].primitiveIndex = 0;
    out[node].primitiveType = 0;
  }
  void build_serial(uint32_t node, size_t b, size_t e, int depth) {
    if (e - b == 1) {
      leaf(node, rec[b]);
      return;
    }
    const size_t mid = split(node, b, e, false, depth);
    uint32_t l, r;
    children(node, l, r);
    build_serial(l, b, mid, depth + 1);
    build_serial(r, mid, e, depth + 1);
  }
};

}  // namespace

void build_sah(const RtTriangle64* tris, uint32_t nt, const RtSphere32* sph, uint32_t ns, RtBVHNode40* out) {
  const size_t N = (size_t)nt + ns;
  if (N == 0) return;
  SahBuild B;
  B.nt = nt;
  B.out = out;
  B.rec.reset(new SahRec[N]);
  if (N > kSahTask) B.tmp.reset(new SahRec[N]);
  parallel_for(N, [&](size_t b, size_t e, unsigned) {
    for (size_t i = b; i < e; ++i) {
      SahRec& r = B.rec[i];
      if (i < nt) {
        const RtTriangle64& T = tris[i];
        for (int a = 0; a < 3; ++a) {
          r.lo[a] = std::fmin(std::fmin(T.v0[a], T.v1[a]), T.v2[a]);
          r.hi[a] = std::fmax(std::fmax(T.v0[a], T.v1[a]), T.v2[a]);
        }
      } else {
        const RtSphere32& S = sph[i - nt];
        for (int a = 0; a < 3; ++a) {
          const float l = S.center[a] - S.radius, h = S.center[a] + S.radius;
          r.lo[a] = std::fmin(l, h);
          r.hi[a] = std::fmax(l, h);
        }
      }
      for (int a = 0; a < 3; ++a) r.c[a] = 0.5f * r.lo[a] + 0.5f * r.hi[a];
      // An exactly flat axis (an axis-aligned triangle) gets 2^-20 of its
      // magnitude on each side, so that a strict slab test (tNear < tFar)
      // can enter the box; no other box is changed.
      for (int a = 0; a < 3; ++a)
        if (r.hi[a] == r.lo[a]) {
          const float e = std::fmax(std::fabs(r.lo[a]), 1e-30f) * 9.5367431640625e-07f;
          r.lo[a] -= e;
          r.hi[a] += e;
        }
      r.id = (uint32_t)i;
    }
  });
  // Top of the tree: breadth-first with the passes spread over the threads,
  // until every open range is small enough to be a task of its own.
  struct Range {
    uint32_t node;
    size_t b, e;
    int depth;
  };
  std::vector<Range> open{{0u, 0, N, 0}}, tasks;
  const unsigned T = std::max(1u, host_threads());
  while (!open.empty()) {
    std::vector<Range> big;
    for (const Range& r : open) (r.e - r.b <= kSahTask ? tasks : big).push_back(r);
    std::vector<Range> nxt(2 * big.size());
    auto one = [&](size_t i, bool par) {
      const Range& r = big[i];
      const size_t mid = B.split(r.node, r.b, r.e, par, r.depth);
      uint32_t l, rr;
      B.children(r.node, l, rr);
      nxt[2 * i] = {l, r.b, mid, r.depth + 1};
      nxt[2 * i + 1] = {rr, mid, r.e, r.depth + 1};
    };
    if (big.size() >= T) {  // a range per thread, each split serially
      std::atomic<size_t> ri{0};
      std::vector<std::thread> th;
      for (unsigned t = 0; t < T; ++t)
        th.emplace_back([&] {
          for (size_t k; (k = ri.fetch_add(1)) < big.size();) one(k, false);
        });
      for (auto& x : th) x.join();
    } else {  // few ranges: each split's passes spread over the threads
      for (size_t i = 0; i < big.size(); ++i) one(i, true);
    }
    open.swap(nxt);
  }
  std::sort(tasks.begin(), tasks.end(), [](const Range& a, const Range& b) { return a.e - a.b > b.e - b.b; });
  std::atomic<size_t> ti{0};
  std::vector<std::thread> th;
  for (unsigned t = 0; t < T; ++t)
    th.emplace_back([&] {
      for (size_t k; (k = ti.fetch_add(1)) < tasks.size();)
        B.build_serial(tasks[k].node, tasks[k].b, tasks[k].e, tasks[k].depth);
    });
  for (auto& x : th) x.join();
}

static void precompute_triangle(const RtTriangle64& T, float* r) {
  float v0x = T.v0[0], v0y = T.v0[1], v0z = T.v0[2];
  float ux = T.v1[0] - v0x, uy = T.v1[1] - v0y, uz = T.v1[2] - v0z;
  float vx = T.v2[0] - v0x, vy = T.v2[1] - v0y, vz = T.v2[2] - v0z;
  float Nx = uy * vz - uz * vy, Ny = uz * vx - ux * vz, Nz = ux * vy - uy * vx;
  float nn = Nx * Nx + Ny * Ny + Nz * Nz;
  float len = std::sqrt(nn);
  float nx = Nx / len, ny = Ny / len, nz = Nz / len;
  float D = nx * v0x + ny * v0y + nz * v0z;
  float wx = Nx / nn, wy = Ny / nn, wz = Nz / nn;
  float vals[16] = {nx, ny, nz, D, wx, wy, wz, v0x, v0y, v0z, ux, uy, uz, vx, vy, vz};
  std::memcpy(r, vals, sizeof(vals));
}

static inline float bits_f(uint32_t u) {
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

bool convert_bvh(const RtBVHNode40* nodes, uint32_t nn, const RtTriangle64* tris, uint32_t nt,
                 const RtSphere32* sph, uint32_t ns, const RtMaterial32* mats, uint32_t nm,
                 uint32_t leaf_size, uint32_t width, HostDeviceBVH& out, std::string& msg) {
  out = HostDeviceBVH();
  // 4-wide nodes store per-axis steps 2^e with e <= kMaxWideExp (the kernels
  // scale by 2^(e+15)); a root box wider than 255 * 2^kMaxWideExp (7.2e16)
  // keeps the binary layout, or is rejected when 4-wide nodes were asked for.
  bool too_wide = false;
  if (nn > 0) {
    const RtBVHNode40& r = nodes[0];
    const double lim = 255.0 * std::ldexp(1.0, kMaxWideExp);
    too_wide = (double)r.maxX - r.minX > lim || (double)r.maxY - r.minY > lim || (double)r.maxZ - r.minZ > lim;
  }
  if (width == 0) width = too_wide ? 2u : kDefaultWidth;
  if (width != 2 && width != 4) {
    msg = "node width must be 2 or 4";
    return false;
  }
  if (width == 4 && too_wide) {
    msg = "scene extent beyond 255 * 2^48 (7.2e16) needs node width 2";
    return false;
  }
  if (leaf_size == 0) leaf_size = kDefaultLeafSize;
  if (leaf_size > kMaxLeafSize) {
    msg = "leaf_size above " + std::to_string(kMaxLeafSize);
    return false;
  }
  // spheres and materials in caller order
  out.spheres.resize(8 * (size_t)ns);
  for (uint32_t i = 0; i < ns; ++i) {
    float* s = &out.spheres[8 * (size_t)i];
    s[0] = sph[i].center[0]; s[1] = sph[i].center[1]; s[2] = sph[i].center[2]; s[3] = sph[i].radius;
    s[4] = bits_f(sph[i].materialIndex); s[5] = 0.0f; s[6] = 0.0f; s[7] = 0.0f;
  }
  out.mats.resize(8 * (size_t)nm);
  for (uint32_t i = 0; i < nm; ++i) {
    float* m = &out.mats[8 * (size_t)i];
    m[0] = mats[i].albedo[0]; m[1] = mats[i].albedo[1]; m[2] = mats[i].albedo[2]; m[3] = 0.0f;
    m[4] = bits_f(mats[i].materialType); m[5] = mats[i].fuzz; m[6] = mats[i].ior; m[7] = 0.0f;
  }
  if (nn == 0) return true;

  // Pass A: left-first DFS from node 0; triangle leaves get slots in visit order.
  const uint32_t NONE = 0xFFFFFFFFu;
  std::vector<uint32_t> pre;
  pre.reserve(nn);
  std::vector<uint8_t> seen(nn, 0);
  std::vector<uint32_t> slot(nn, NONE);
  std::vector<uint32_t> stack;
  stack.push_back(0);
  while (!stack.empty()) {
    uint32_t x = stack.back();
    stack.pop_back();
    if (x >= nn) {
      msg = "node index " + std::to_string(x) + " out of range";
      return false;
    }
    if (seen[x]) {
      msg = "node " + std::to_string(x) + " reached twice: not a tree";
      return false;
    }
    seen[x] = 1;
    pre.push_back(x);
    const RtBVHNode40& nd = nodes[x];
    if (nd.left == 0u && nd.right == 0u) {
      if (nd.primitiveType == RT_PRIM_TRIANGLE) {
        if (nd.primitiveIndex >= nt) {
          msg = "leaf " + std::to_string(x) + " names triangle out of range";
          return false;
        }
        slot[x] = (uint32_t)out.tri_ids.size();
        out.tri_ids.push_back(nd.primitiveIndex);
      } else if (nd.primitiveType == RT_PRIM_SPHERE) {
        if (nd.primitiveIndex >= ns) {
          msg = "leaf " + std::to_string(x) + " names sphere out of range";
          return false;
        }
      }
    } else {
      stack.push_back(nd.right);
      stack.push_back(nd.left);
    }
  }
  const uint32_t nslots = (uint32_t)out.tri_ids.size();
  if (nslots > kMaxTriangles) {
    msg = "more than 2^27 triangle leaves";
    return false;
  }

  // Pass B: subtree triangle counts, sphere presence, first slot.
  std::vector<uint32_t> cnt(nn, 0), first(nn, NONE);
  std::vector<uint8_t> has_sph(nn, 0), other(nn, 0);
  for (size_t k = pre.size(); k-- > 0;) {
    uint32_t x = pre[k];
    const RtBVHNode40& nd = nodes[x];
    if (nd.left == 0u && nd.right == 0u) {
      if (nd.primitiveType == RT_PRIM_TRIANGLE) {
        cnt[x] = 1;
        first[x] = slot[x];
      } else if (nd.primitiveType == RT_PRIM_SPHERE) {
        has_sph[x] = 1;
      } else {
        other[x] = 1;
      }
    } else {
      cnt[x] = cnt[nd.left] + cnt[nd.right];
      has_sph[x] = has_sph[nd.left] | has_sph[nd.right];
      other[x] = other[nd.left] | other[nd.right];
      first[x] = first[nd.left] != NONE ? first[nd.left] : first[nd.right];
    }
  }
  auto is_leaf = [&](uint32_t x) { return nodes[x].left == 0u && nodes[x].right == 0u; };
  auto collapsible = [&](uint32_t x) {
    return !is_leaf(x) && cnt[x] >= 1 && cnt[x] <= leaf_size && !has_sph[x] && !other[x];
  };
  const uint32_t EMPTY = kLeafBit | kSphereBit | kSphereMask;
  auto leaf_ref = [&](uint32_t x) -> uint32_t {
    const RtBVHNode40& nd = nodes[x];
    if (nd.primitiveType == RT_PRIM_TRIANGLE) return kLeafBit | slot[x];
    if (nd.primitiveType == RT_PRIM_SPHERE) return kLeafBit | kSphereBit | nd.primitiveIndex;
    return EMPTY;
  };

  auto ref_of = [&](uint32_t x, const std::vector<uint32_t>& dev) -> uint32_t {
    if (is_leaf(x)) return leaf_ref(x);
    if (collapsible(x)) return kLeafBit | ((cnt[x] - 1u) << kCountShift) | first[x];
    return dev[x];
  };
  auto expandable = [&](uint32_t x) { return !is_leaf(x) && !collapsible(x); };
  std::vector<uint32_t> dev(nn, NONE);
  out.width = width;
  if (!expandable(0)) {
    out.root = ref_of(0, dev);
    out.depth = 0;
    out.stack_need = 1;
  } else if (width == 2) {
    // Binary device tree: the kept internal nodes in left-first preorder.
    std::vector<uint32_t> kept;
    std::vector<std::pair<uint32_t, uint32_t>> st2;  // (node, depth)
    uint32_t maxdepth = 0;
    st2.push_back({0u, 1u});
    while (!st2.empty()) {
      auto [x, d] = st2.back();
      st2.pop_back();
      dev[x] = (uint32_t)kept.size();
      kept.push_back(x);
      maxdepth = std::max(maxdepth, d);
      const RtBVHNode40& nd = nodes[x];
      if (expandable(nd.right)) st2.push_back({nd.right, d + 1});
      if (expandable(nd.left)) st2.push_back({nd.left, d + 1});
    }
    out.root = 0;
    out.depth = maxdepth;
    out.stack_need = maxdepth + 1;
    out.inner.resize(16 * kept.size());
    parallel_for(kept.size(), [&](size_t b, size_t e, unsigned) {
      for (size_t i = b; i < e; ++i) {
        const RtBVHNode40& nd = nodes[kept[i]];
        const RtBVHNode40& L = nodes[nd.left];
        const RtBVHNode40& R = nodes[nd.right];
        float* o = &out.inner[16 * i];
        o[0] = L.minX; o[1] = L.maxX; o[2] = L.minY; o[3] = L.maxY;
        o[4] = R.minX; o[5] = R.maxX; o[6] = R.minY; o[7] = R.maxY;
        o[8] = L.minZ; o[9] = L.maxZ; o[10] = R.minZ; o[11] = R.maxZ;
        o[12] = bits_f(ref_of(nd.left, dev));
        o[13] = bits_f(ref_of(nd.right, dev));
        o[14] = 0.0f;
        o[15] = 0.0f;
      }
    });
  } else {
    // 4-wide device tree: each wide node takes a binary node's two children
    // and splits the child with the largest surface area until it has four,
    // keeping left-to-right order (so leaf slots stay contiguous per subtree).
    struct Wide {
      uint32_t ch[4];
      uint32_t count;
    };
    auto area = [&](uint32_t x) {
      const RtBVHNode40& n = nodes[x];
      const double dx = (double)n.maxX - n.minX, dy = (double)n.maxY - n.minY, dz = (double)n.maxZ - n.minZ;
      return dx * dy + dy * dz + dz * dx;
    };
    std::vector<Wide> wn;
    std::vector<uint32_t> todo{0u};
    while (!todo.empty()) {
      const uint32_t x = todo.back();
      todo.pop_back();
      Wide w;
      w.ch[0] = nodes[x].left;
      w.ch[1] = nodes[x].right;
      w.count = 2;
      while (w.count < 4) {
        int best = -1;
        double ba = -1.0;
        for (uint32_t j = 0; j < w.count; ++j)
          if (expandable(w.ch[j])) {
            const double a = area(w.ch[j]);
            if (a > ba) { ba = a; best = (int)j; }
          }
        if (best < 0) break;
        const uint32_t c = w.ch[best];
        for (uint32_t j = w.count; j > (uint32_t)best + 1; --j) w.ch[j] = w.ch[j - 1];
        w.ch[best] = nodes[c].left;
        w.ch[best + 1] = nodes[c].right;
        w.count++;
      }
      dev[x] = (uint32_t)wn.size();
      wn.push_back(w);
      for (int j = (int)w.count - 1; j >= 0; --j)
        if (expandable(w.ch[j])) todo.push_back(w.ch[j]);
    }
    // depth and worst-case stack use (a visit pushes at most count-1 entries)
    std::vector<uint32_t> need(wn.size()), dep(wn.size());
    for (size_t k = wn.size(); k-- > 0;) {
      uint32_t nd = 0, dd = 0;
      for (uint32_t j = 0; j < wn[k].count; ++j)
        if (expandable(wn[k].ch[j])) {
          nd = std::max(nd, need[dev[wn[k].ch[j]]]);
          dd = std::max(dd, dep[dev[wn[k].ch[j]]]);
        }
      need[k] = nd + wn[k].count - 1u;
      dep[k] = dd + 1u;
    }
    out.root = 0;
    out.depth = dep[0];
    out.stack_need = need[0] + 1u;
    // Renumber: the top kTopNodes wide nodes in breadth-first order first (so
    // a kernel can stage the top levels of the tree as one contiguous range
    // [root, root + K)), the rest in their left-first preorder.
    {
      const size_t top = std::min<size_t>(kTopNodes, wn.size());
      std::vector<uint32_t> perm(wn.size(), NONE);
      std::vector<uint32_t> bfs{0u};
      for (size_t h = 0; h < bfs.size() && bfs.size() < top; ++h)
        for (uint32_t j = 0; j < wn[bfs[h]].count && bfs.size() < top; ++j)
          if (expandable(wn[bfs[h]].ch[j])) bfs.push_back(dev[wn[bfs[h]].ch[j]]);
      uint32_t next = 0;
      for (uint32_t k : bfs) perm[k] = next++;
      for (size_t k = 0; k < wn.size(); ++k)
        if (perm[k] == NONE) perm[k] = next++;
      std::vector<Wide> wn2(wn.size());
      for (size_t k = 0; k < wn.size(); ++k) wn2[perm[k]] = wn[k];
      wn.swap(wn2);
      for (auto& d : dev)
        if (d != NONE) d = perm[d];
    }
    // Quantised child boxes: node origin p = min of the child boxes; per axis a
    // power-of-two step s = 2^e with 255*s >= extent; child bounds rounded
    // outward to multiples of s, so p + q*s encloses every child box.
    out.inner.resize(16 * wn.size());
    parallel_for(wn.size(), [&](size_t b, size_t e, unsigned) {
      for (size_t i = b; i < e; ++i) {
        const Wide& w = wn[i];
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (uint32_t j = 0; j < w.count; ++j) {
          const RtBVHNode40& c = nodes[w.ch[j]];
          const float cl[3] = {c.minX, c.minY, c.minZ}, chh[3] = {c.maxX, c.maxY, c.maxZ};
          for (int a = 0; a < 3; ++a) {
            lo[a] = std::fmin(lo[a], cl[a]);
            hi[a] = std::fmax(hi[a], chh[a]);
          }
        }
        int ex[3];
        for (int a = 0; a < 3; ++a) {
          const double ext = (double)hi[a] - (double)lo[a];
          int e2 = -126;
          if (ext > 0.0) {
            e2 = (int)std::ceil(std::log2(ext / 255.0));
            while (255.0 * std::ldexp(1.0, e2) < ext) ++e2;
            while (e2 > -126 && 255.0 * std::ldexp(1.0, e2 - 1) >= ext) --e2;
          }
          ex[a] = std::max(-126, std::min(kMaxWideExp, e2));
        }
        uint32_t q[6] = {0, 0, 0, 0, 0, 0};  // qlo_x, qhi_x, qlo_y, qhi_y, qlo_z, qhi_z
        for (uint32_t j = w.count; j < 4; ++j)  // unused slot: qlo 255 > qhi 0, empty for any ray
          for (int a = 0; a < 3; ++a) q[2 * a] |= 255u << (8 * j);
        for (uint32_t j = 0; j < w.count; ++j) {
          const RtBVHNode40& c = nodes[w.ch[j]];
          const float cl[3] = {c.minX, c.minY, c.minZ}, chh[3] = {c.maxX, c.maxY, c.maxZ};
          for (int a = 0; a < 3; ++a) {
            const double st = std::ldexp(1.0, ex[a]);
            double ql = std::floor(((double)cl[a] - (double)lo[a]) / st);
            double qh = std::ceil(((double)chh[a] - (double)lo[a]) / st);
            ql = std::min(255.0, std::max(0.0, ql));
            qh = std::min(255.0, std::max(0.0, qh));
            q[2 * a] |= (uint32_t)ql << (8 * j);
            q[2 * a + 1] |= (uint32_t)qh << (8 * j);
          }
        }
        float* o = &out.inner[16 * i];
        o[0] = lo[0]; o[1] = lo[1]; o[2] = lo[2];
        // the per-axis scales 2^(e+15) as floats (exact powers of two), which the
        // kernels multiply by 1/d: x in word 3, y and z in words 14 and 15
        o[3] = std::ldexp(1.0f, ex[0] + 15);
        for (uint32_t j = 0; j < 4; ++j)
          o[4 + j] = bits_f(j < w.count ? ref_of(w.ch[j], dev) : (kLeafBit | kSphereBit | kSphereMask));
        for (int k = 0; k < 6; ++k) o[8 + k] = bits_f(q[k]);
        o[14] = std::ldexp(1.0f, ex[1] + 15);
        o[15] = std::ldexp(1.0f, ex[2] + 15);
      }
    });
  }

  // Triangle records in slot order.
  out.tris.resize(16 * (size_t)nslots);
  out.tri_mat.resize(nslots);
  parallel_for(nslots, [&](size_t b, size_t e, unsigned) {
    for (size_t s = b; s < e; ++s) {
      const RtTriangle64& T = tris[out.tri_ids[s]];
      precompute_triangle(T, &out.tris[16 * s]);
      out.tri_mat[s] = T.materialIndex;
    }
  });
  return true;
}

// raytraceBVH.comp:54-76 evaluated once per frame.
void camera_setup(const RtRaytraceUBO& ubo, uint32_t width, uint32_t height, float out[12]) {
  auto normalize3 = [](float* v) {
    float l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] = v[0] / l; v[1] = v[1] / l; v[2] = v[2] / l;
  };
  auto cross3 = [](const float* a, const float* b, float* r) {
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
  };
  float W = (float)width, H = (float)height;
  float aspect = W / H;
  float theta = ubo.verticalFOV * 0x1.1df46ap-6f;  // radians()
  float h = (float)std::tan((double)(theta / 2.0f));
  float vh = 2.0f * h * 10.0f;                      // _FOCAL_DISTANCE = 10
  float vw = vh * aspect;
  float w[3] = {ubo.camPos[0] - ubo.camLookAt[0], ubo.camPos[1] - ubo.camLookAt[1], ubo.camPos[2] - ubo.camLookAt[2]};
  normalize3(w);
  float u[3];
  cross3(ubo.camUpDir, w, u);
  normalize3(u);
  float v[3];
  cross3(w, u, v);
  float vpu[3], vpv[3], pdu[3], pdv[3], p00[3];
  for (int k = 0; k < 3; ++k) {
    vpu[k] = u[k] * vw;
    vpv[k] = -v[k] * vh;
    pdu[k] = vpu[k] / W;
    pdv[k] = vpv[k] / H;
  }
  for (int k = 0; k < 3; ++k) {
    float ul = ((ubo.camPos[k] - w[k] * 10.0f) - vpu[k] / 2.0f) - vpv[k] / 2.0f;
    p00[k] = ul + (pdu[k] + pdv[k]) * 0.5f;
  }
  float vals[12] = {ubo.camPos[0], ubo.camPos[1], ubo.camPos[2], p00[0], p00[1], p00[2],
                    pdu[0], pdu[1], pdu[2], pdv[0], pdv[1], pdv[2]};
  std::memcpy(out, vals, sizeof(vals));
}

}  // namespace rtgb
