// trace_core.cuh -- device traversal and intersection shared by the ray-query
// and path-tracing kernels.
//
// Arithmetic contract: the translation units that include this header are
// compiled with -fmad=false and IEEE division/square root, so each binary32
// operation below rounds on its own in the order written -- the same contract
// the reference's shader expressions are restated under on the host.  FMAs
// appear only where written explicitly (fmaf), and only in box tests, whose
// results are widened to stay conservative.
#pragma once

#include <cstdint>

#include "rt_internal.h"

namespace rtgb {
namespace dev {

constexpr uint32_t kNoBest = 0u;  // "no hit yet" (every leaf ref has bit31 set)

// ---------------------------------------------------------------- loads ---
__device__ __forceinline__ float4 ldg4(const void* base, uint32_t idx) {
  return __ldg(reinterpret_cast<const float4*>(base) + idx);
}
__device__ __forceinline__ uint32_t fbits(float f) { return __float_as_uint(f); }
// Two consecutive float4 (32 bytes, 32-byte aligned) in one 256-bit load
// through the read-only path (sm_100 and later): a node or triangle record
// takes two loads instead of four, each one whole 32-byte sector (config 3:
// 11.28 -> 10.2 ms per step).  idx2 counts 32-byte units.
__device__ __forceinline__ void ldg8(const void* base, uint32_t idx2, float4& a, float4& b) {
  const float4* p = reinterpret_cast<const float4*>(base) + 2u * idx2;
  asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
      : "l"(p));
}
// The same for tree nodes, marked to stay in L2 ahead of streamed data
// (rays, hits), which is marked evict-first.
__device__ __forceinline__ void ldg8_keep(const void* base, uint32_t idx2, float4& a, float4& b) {
  const float4* p = reinterpret_cast<const float4*>(base) + 2u * idx2;
  asm("ld.global.nc.L2::evict_last.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
      : "l"(p));
}
// One 32-byte ray record (origin, tmin | direction, tmax), read once: a
// single 256-bit load that skips L1 and leaves L2 first when the caller's
// array is 32-byte aligned (`al32`, uniform per launch), else two loads.
__device__ __forceinline__ void load_ray(const float4* rays, uint32_t i, bool al32, float4& o, float4& d) {
  if (al32) {
    asm("ld.global.nc.L1::no_allocate.L2::evict_first.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(o.x), "=f"(o.y), "=f"(o.z), "=f"(o.w), "=f"(d.x), "=f"(d.y), "=f"(d.z), "=f"(d.w)
        : "l"(rays + 2u * i));
  } else {
    o = __ldg(&rays[2u * i]);
    d = __ldg(&rays[2u * i + 1u]);
  }
}
__device__ __forceinline__ bool aligned32(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 31u) == 0u; }

// ------------------------------------------------------- triangle test ----
// triangleHit (raytraceBVH.comp:118-149) on a precomputed 64-byte record;
// returns true and t for a hit in [tmin, tmax].  A NaN t never hits.
__device__ __forceinline__ bool tri_test(const void* tris, uint32_t slot, float ox, float oy, float oz,
                                         float dx, float dy, float dz, float tmin, float tmax, float& t_out) {
  float4 r0, r1, r2, r3;
  ldg8(tris, 2u * slot + 0u, r0, r1);  // n.xyz, D | w.xyz, v0.x
  const float denom = r0.x * dx + r0.y * dy + r0.z * dz;
  if (fabsf(denom) < 0.0001f) return false;
  const float t = (r0.w - (r0.x * ox + r0.y * oy + r0.z * oz)) / denom;
  if (!(t >= tmin && t <= tmax)) return false;  // a NaN t misses
  ldg8(tris, 2u * slot + 1u, r2, r3);  // v0.y, v0.z, u.x, u.y | u.z, v.x, v.y, v.z
  const float px = ox + t * dx, py = oy + t * dy, pz = oz + t * dz;
  const float qx = px - r1.w, qy = py - r2.x, qz = pz - r2.y;
  const float ux = r2.z, uy = r2.w, uz = r3.x;
  const float vx = r3.y, vy = r3.z, vz = r3.w;
  // a = dot(w, cross(q, v)); b = dot(w, cross(u, q))
  const float cqx = qy * vz - qz * vy, cqy = qz * vx - qx * vz, cqz = qx * vy - qy * vx;
  const float a = r1.x * cqx + r1.y * cqy + r1.z * cqz;
  const float cux = uy * qz - uz * qy, cuy = uz * qx - ux * qz, cuz = ux * qy - uy * qx;
  const float b = r1.x * cux + r1.y * cuy + r1.z * cuz;
  if (a < 0.0f || b < 0.0f || a + b > 1.0f) return false;
  t_out = t;
  return true;
}

// Moller & Trumbore, "Fast, minimum storage ray-triangle intersection",
// J. Graphics Tools 2(1), 1997, on the same record (v0, e1 = v1 - v0,
// e2 = v2 - v0) under the same arithmetic contract: p = d x e2,
// det = e1 . p (0: the ray is parallel, a miss), u = (o - v0) . p / det,
// q = (o - v0) x e1, v = d . q / det, t = e2 . q / det.  An optional mode
// (RT_TRACE_MT), not the reference's test.
__device__ __forceinline__ bool tri_test_mt(const void* tris, uint32_t slot, float ox, float oy, float oz,
                                            float dx, float dy, float dz, float tmin, float tmax, float& t_out) {
  float4 r0, r1, r2, r3;
  ldg8(tris, 2u * slot + 0u, r0, r1);  // (n, D: unused) | w.xyz, v0.x
  ldg8(tris, 2u * slot + 1u, r2, r3);  // v0.y, v0.z, e1.x, e1.y | e1.z, e2.x, e2.y, e2.z
  (void)r0;
  const float e1x = r2.z, e1y = r2.w, e1z = r3.x;
  const float e2x = r3.y, e2y = r3.z, e2z = r3.w;
  const float px = dy * e2z - dz * e2y, py = dz * e2x - dx * e2z, pz = dx * e2y - dy * e2x;
  const float det = e1x * px + e1y * py + e1z * pz;
  if (!(fabsf(det) > 0.0f)) return false;  // parallel (or NaN)
  const float inv = 1.0f / det;
  const float tx = ox - r1.w, ty = oy - r2.x, tz = oz - r2.y;
  const float u = (tx * px + ty * py + tz * pz) * inv;
  if (!(u >= 0.0f && u <= 1.0f)) return false;
  const float qx = ty * e1z - tz * e1y, qy = tz * e1x - tx * e1z, qz = tx * e1y - ty * e1x;
  const float v = (dx * qx + dy * qy + dz * qz) * inv;
  if (!(v >= 0.0f && u + v <= 1.0f)) return false;
  const float t = (e2x * qx + e2y * qy + e2z * qz) * inv;
  if (!(t >= tmin && t <= tmax)) return false;
  t_out = t;
  return true;
}

// sphereHit (raytraceBVH.comp:152-181) -- root only; the hit record is rebuilt
// by the caller when it needs the normal.
__device__ __forceinline__ bool sphere_test(const void* spheres, uint32_t idx, float ox, float oy, float oz,
                                            float dx, float dy, float dz, float tmin, float tmax, float& t_out) {
  const float4 s = ldg4(spheres, 2u * idx);
  const float ocx = ox - s.x, ocy = oy - s.y, ocz = oz - s.z;
  const float a = dx * dx + dy * dy + dz * dz;
  const float halfB = ocx * dx + ocy * dy + ocz * dz;
  const float c = (ocx * ocx + ocy * ocy + ocz * ocz) - (s.w * s.w);
  const float under = (halfB * halfB) - (a * c);
  if (under < 0.0f) return false;
  const float rad = sqrtf(under);
  float root = (-halfB - rad) / a;
  if (root < tmin || root > tmax) {
    root = (-halfB + rad) / a;
    if (root < tmin || root > tmax) return false;
  }
  t_out = root;
  return true;
}

// ---------------------------------------------------------- traversal ----
// One ray's traversal state; kept in registers across warp refills.
#ifndef RT_DEVICE_CHECKS
#define RT_DEVICE_CHECKS 0
#endif
// Device-side index checks of the checked build (RT_DEVICE_CHECKS=1), in
// place of a sanitizer: an index outside its array sets a bit in the scene's
// check word, records the first bad index, and the access is skipped (the
// ray ends as a miss).  In the normal build chk() is constant false.
enum : uint32_t { kChkNode = 1u, kChkTri = 2u, kChkSphere = 4u, kChkRay = 8u, kChkMat = 16u, kChkPath = 32u };
__device__ __forceinline__ bool chk(uint32_t* word, bool bad, uint32_t bit, uint32_t value) {
#if RT_DEVICE_CHECKS
  if (bad && word) {
    atomicOr(word, bit);
    atomicCAS(word + 1, 0u, value | 0x80000000u);
  }
  return bad;
#else
  (void)word; (void)bad; (void)bit; (void)value;
  return false;
#endif
}

struct Trav {
  float ox, oy, oz, dx, dy, dz;  // the ray exactly as given (triangle tests)
  float ix, iy, iz;              // 1/d, with zero components replaced
  float tmin, tclose;            // interval; tclose = closest hit so far
  float cull_lo, cull_hi;        // widened interval for box culling
  uint32_t best;                 // leaf-style ref of the closest hit (kNoBest: none)
  uint32_t node;                 // next node to visit, or a leaf, or kSentinel
  uint32_t leaf;                 // postponed leaf (0: none)
  int sp;                        // stack top index; stack[0] = kSentinel
  uint32_t nvis, ntest;          // inner nodes fetched, primitives tested
};

// Box culling margin: wider than the binary32 rounding of box and triangle
// t values, so that a box is skipped only when it cannot hold a closer hit
// except within the margin (a near-tie).
constexpr float kCullRel = 1.52587890625e-05f;  // 2^-16
constexpr float kSlabWiden = 4.76837158203125e-07f;  // 2^-21: > 3 ulps of (b-o)*(1/d)

__device__ __forceinline__ void trav_set_close(Trav& s, float t) {
  s.tclose = t;
  s.cull_hi = fmaf(fabsf(t), kCullRel, t);
}

// Loads one ray into the state; the caller prepares its stack.
__device__ __forceinline__ void trav_init_ray(Trav& s, const float4 o_tmin, const float4 d_tmax, uint32_t root) {
  // A NaN bound rejects nothing in the reference's t < tMin || tMax < t, as
  // -inf / +inf do, which keeps the tests below NaN-free.
  const float inf = __int_as_float(0x7f800000);
  s.ox = o_tmin.x; s.oy = o_tmin.y; s.oz = o_tmin.z; s.tmin = o_tmin.w == o_tmin.w ? o_tmin.w : -inf;
  s.dx = d_tmax.x; s.dy = d_tmax.y; s.dz = d_tmax.z;
  // Zero (or smaller) direction components become +-2^-64, so 1/d stays
  // within 2^64: with 4-wide steps up to 2^kMaxWideExp the node scale
  // 2^(e+15)/d stays finite.
  const float eps = 5.42101086242752217e-20f;  // 2^-64
  s.ix = 1.0f / (fabsf(s.dx) > eps ? s.dx : copysignf(eps, s.dx));
  s.iy = 1.0f / (fabsf(s.dy) > eps ? s.dy : copysignf(eps, s.dy));
  s.iz = 1.0f / (fabsf(s.dz) > eps ? s.dz : copysignf(eps, s.dz));
  s.cull_lo = fmaf(-fabsf(s.tmin), kCullRel, s.tmin);
  trav_set_close(s, d_tmax.w == d_tmax.w ? d_tmax.w : inf);
  s.best = kNoBest;
  s.node = root;
  s.leaf = 0u;
  if (root > kSentinel) {  // the whole tree is one leaf
    s.leaf = root;
    s.node = kSentinel;
  }
  // A non-finite origin or direction component fails the reference's root
  // box test (its slab parameters are infinite or NaN), so the ray misses.
  const float big = 3.40282347e+38f;
  if (!(fabsf(s.ox) <= big && fabsf(s.oy) <= big && fabsf(s.oz) <= big && fabsf(s.dx) <= big &&
        fabsf(s.dy) <= big && fabsf(s.dz) <= big)) {
    s.node = kSentinel;
    s.leaf = 0u;
  }
  s.sp = 0;
  s.nvis = 0;
  s.ntest = 0;
}

// Binary-tree stack: stack[0] holds the sentinel, sp is the top index.
__device__ __forceinline__ void trav_init(Trav& s, const float4 o_tmin, const float4 d_tmax, uint32_t root,
                                          uint32_t* stack) {
  trav_init_ray(s, o_tmin, d_tmax, root);
  stack[0] = kSentinel;
}

// Near/far parameters of one child box, robust form (b - o) * (1/d), widened.
__device__ __forceinline__ void slab(const Trav& s, float lox, float hix, float loy, float hiy, float loz,
                                     float hiz, float& tn, float& tf) {
  const float x0 = (lox - s.ox) * s.ix, x1 = (hix - s.ox) * s.ix;
  const float y0 = (loy - s.oy) * s.iy, y1 = (hiy - s.oy) * s.iy;
  const float z0 = (loz - s.oz) * s.iz, z1 = (hiz - s.oz) * s.iz;
  const float n = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fminf(z0, z1));
  const float f = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fmaxf(z0, z1));
  tn = fmaf(-fabsf(n), kSlabWiden, n);
  tf = fmaf(fabsf(f), kSlabWiden, f);
}

__device__ __forceinline__ bool is_inner(uint32_t r) { return r < kSentinel; }
__device__ __forceinline__ bool is_leaf(uint32_t r) { return r > kSentinel; }

// Tests the primitives of one leaf ref; returns true when the ray is done
// (any-hit found).  MT: the Moller-Trumbore triangle test (RT_TRACE_MT).
template <bool ANY, bool MT = false>
__device__ __forceinline__ bool leaf_visit(const DeviceScene& S, Trav& s, uint32_t leaf) {
  if (leaf & kSphereBit) {
    const uint32_t idx = leaf & kSphereMask;
    if (chk(S.check, idx >= S.n_spheres, kChkSphere, idx)) return false;
    float t;
    s.ntest++;
    if (idx < S.n_spheres && sphere_test(S.spheres, idx, s.ox, s.oy, s.oz, s.dx, s.dy, s.dz, s.tmin, s.tclose, t)) {
      trav_set_close(s, t);
      s.best = leaf;
      if (ANY) return true;
    }
    return false;
  }
  const uint32_t first = leaf & kSlotMask;
  const uint32_t count = ((leaf >> kCountShift) & 7u) + 1u;
  if (chk(S.check, first + count > S.n_tris, kChkTri, first)) return false;
  for (uint32_t k = 0; k < count; ++k) {
    float t;
    s.ntest++;
    const bool hit = MT ? tri_test_mt(S.tris, first + k, s.ox, s.oy, s.oz, s.dx, s.dy, s.dz, s.tmin, s.tclose, t)
                        : tri_test(S.tris, first + k, s.ox, s.oy, s.oz, s.dx, s.dy, s.dz, s.tmin, s.tclose, t);
    if (hit) {
      trav_set_close(s, t);
      s.best = kLeafBit | (first + k);
      if (ANY) return true;
    }
  }
  return false;
}

// Advances the traversal.  Returns true when the ray is finished.  Returns
// false early when fewer than `refill` lanes of the warp are still traversing,
// so that the warp can hand new rays to its idle lanes (state is kept).
// Returns false with s.sp == -1 on stack overflow (the ray is abandoned).
template <bool ANY, int STACK, bool MT = false>
__device__ __forceinline__ bool trav_run(const DeviceScene& S, Trav& s, uint32_t* stack, int refill) {
  for (;;) {
    // Inner nodes: descend, postponing the first leaf found.
    while (is_inner(s.node)) {
      if (chk(S.check, s.node >= S.n_inner, kChkNode, s.node)) {
        s.sp = -1;
        return false;
      }
      s.nvis++;
      float4 a, b, c, d;
      ldg8_keep(S.inner, 2u * s.node + 0u, a, b);
      ldg8_keep(S.inner, 2u * s.node + 1u, c, d);
      float n0, f0, n1, f1;
      slab(s, a.x, a.y, a.z, a.w, c.x, c.y, n0, f0);
      slab(s, b.x, b.y, b.z, b.w, c.z, c.w, n1, f1);
      const bool h0 = fmaxf(n0, s.cull_lo) <= fminf(f0, s.cull_hi);
      const bool h1 = fmaxf(n1, s.cull_lo) <= fminf(f1, s.cull_hi);
      const uint32_t r0 = fbits(d.x), r1 = fbits(d.y);
      if (!h0 && !h1) {
        s.node = stack[s.sp];
        s.sp = s.sp > 0 ? s.sp - 1 : 0;
      } else {
        uint32_t first = h0 ? r0 : r1;
        if (h0 && h1) {
          uint32_t second = r1;
          if (n1 < n0) {
            first = r1;
            second = r0;
          }
          if (s.sp + 1 >= STACK) {
            s.sp = -1;
            return false;
          }
          stack[++s.sp] = second;
        }
        s.node = first;
      }
      if (is_leaf(s.node) && s.leaf == 0u) {
        s.leaf = s.node;
        s.node = stack[s.sp];
        s.sp = s.sp > 0 ? s.sp - 1 : 0;
      }
      if (__all_sync(__activemask(), s.leaf != 0u)) break;
    }
    // Leaves: test the postponed leaf, then any leaves popped in sequence.
    while (s.leaf != 0u) {
      if (leaf_visit<ANY, MT>(S, s, s.leaf)) {
        s.leaf = 0u;
        s.node = kSentinel;
        return true;
      }
      s.leaf = 0u;
      if (is_leaf(s.node)) {
        s.leaf = s.node;
        s.node = stack[s.sp];
        s.sp = s.sp > 0 ? s.sp - 1 : 0;
      }
    }
    if (s.node == kSentinel) return true;
    if (refill > 0 && __popc(__activemask()) < refill) return false;
  }
}

// ------------------------------------------------------ 4-wide nodes ----
// Node (64 B): float4 (p.xyz, 2^(e_x+15)), uint4 refs, uint4 (qlo_x, qhi_x,
// qlo_y, qhi_y), uint4 (qlo_z, qhi_z, 2^(e_y+15), 2^(e_z+15)) -- the three
// per-axis scales stored as floats.  Child i spans p + q*2^e per axis, with q
// the i-th byte of the matching word.
//
// A plane's parameter t = (p + q*2^e - o)/d is evaluated as one fma,
// fma(Q, A, C) with Q = 1 + q*2^-15 (the byte placed in the mantissa under
// 1.0f: one byte permute, exact), A = 2^(e+15)/d (exact scaling of 1/d) and
// C = (p - o)/d - A per axis and node.  With B = (p - o)/d, the rounding of
// 1/d, p - o, the product, B - A and the fma keep it within
// 2^-24 (4|B| + 3|C| + 2.02|A|) of the exact value (|t| <= |C| + 1.008|A|).
// Each axis therefore uses C - M for its near plane and C + M for its far
// plane, with M = (|B| + |A|) * 2^-20: since |C| <= (|B| + |A|)(1 + 2^-24) the
// bound is below 2^-24 (7.01|B| + 5.03|A|), so M is twice the bound and more
// (the rounding of |B| + |A| and of the fma C -+ M fit in the rest), and at
// most 1/32 of a quantisation step (|A| * 2^-20 = 2^e/|d| * 2^-5) beyond the
// distance-relative terms.  The near plane of an axis is the low bound when
// d >= 0 and the high bound otherwise, so no per-axis min/max is needed.
constexpr float kWideWiden = 9.5367431640625e-07f;  // 2^-20

// Stack entries of the while-while loop are (ref, t_near): pop_wide drops an
// entry that starts beyond the closest hit without fetching it.  The step
// loop's stacks below take the top entry as it is: a node beyond the closest
// hit is then visited and culls all of its children, which costs the warp
// less than a per-lane loop over culled entries, where every lane loops a
// different number of times (config 3: 10.15 -> 9.68 ms per step, the same
// hits).  sp counts entries.
__device__ __forceinline__ uint32_t pop_wide(Trav& s, const uint2* stack) {
  while (s.sp > 0) {
    const uint2 e = stack[--s.sp];
    if (__uint_as_float(e.y) <= s.cull_hi) return e.x;
  }
  return kSentinel;
}

// A stack entry of the step loop's stacks: (ref, t_near) as uint2, or the
// ref alone as uint32_t (their pops never look at t_near).
__device__ __forceinline__ uint32_t entry_ref(uint2 e) { return e.x; }
__device__ __forceinline__ uint32_t entry_ref(uint32_t e) { return e; }
template <class E>
__device__ __forceinline__ E make_entry(uint32_t ref, float t);
template <>
__device__ __forceinline__ uint2 make_entry<uint2>(uint32_t ref, float t) {
  return make_uint2(ref, __float_as_uint(t));
}
template <>
__device__ __forceinline__ uint32_t make_entry<uint32_t>(uint32_t ref, float) {
  return ref;
}

// The 4-wide traversal stack in the thread's local memory.
template <class E = uint2>
struct LocalStackT {
  E* a;
  __device__ __forceinline__ void reset() {}
  // pushes the entries whose flag is set, in argument order (np of them)
  __device__ __forceinline__ void push3(Trav& s, int np, bool va, uint32_t ra, float ta, bool vb, uint32_t rb,
                                        float tb, bool vc, uint32_t rc, float tc) {
    (void)np;
    if (va) a[s.sp++] = make_entry<E>(ra, ta);
    if (vb) a[s.sp++] = make_entry<E>(rb, tb);
    if (vc) a[s.sp++] = make_entry<E>(rc, tc);
  }
  __device__ __forceinline__ uint32_t pop(Trav& s) { return s.sp > 0 ? entry_ref(a[--s.sp]) : kSentinel; }
};
using LocalStack = LocalStackT<uint2>;
// Entry type of the step loop's stacks (k_trace_step, k_pool_step): the ref
// alone, since their pops never look at t_near.  Four bytes instead of eight
// halve the shared-memory ring and its stores (config 3: 9.70 -> 9.58 ms).
using StepEntry = uint32_t;

// The same stack with its top K entries in a shared-memory ring (this
// thread's slot j at ring[j * T], so that a warp's lanes hit consecutive
// words) and older entries in local memory: pushes and pops, which sit on
// the path from one node to the next, stay on chip.  The ring holds the
// logical entries [lo, sp); a push into a full ring first moves entry lo out
// to local memory, a pop below lo reads it back from there.
template <int K, int T, class E = uint2>
struct RingStack {
  static_assert((K & (K - 1)) == 0, "ring size must be a power of two");
  E* ring;   // &shared[threadIdx.x]
  E* spill;  // local array of the full stack capacity
  int lo;
  __device__ __forceinline__ void reset() { lo = 0; }
  // pushes the entries whose flag is set, in argument order (np of them):
  // one check for room in the ring, then the stores
  __device__ __forceinline__ void push3(Trav& s, int np, bool va, uint32_t ra, float ta, bool vb, uint32_t rb,
                                        float tb, bool vc, uint32_t rc, float tc) {
    while (s.sp + np - lo > K) {
      spill[lo] = ring[(lo & (K - 1)) * T];
      ++lo;
    }
    int p = s.sp;
    if (va) ring[(p++ & (K - 1)) * T] = make_entry<E>(ra, ta);
    if (vb) ring[(p++ & (K - 1)) * T] = make_entry<E>(rb, tb);
    if (vc) ring[(p++ & (K - 1)) * T] = make_entry<E>(rc, tc);
    s.sp = p;
  }
  __device__ __forceinline__ uint32_t pop(Trav& s) {
    if (s.sp == 0) return kSentinel;
    --s.sp;
    if (s.sp >= lo) return entry_ref(ring[(s.sp & (K - 1)) * T]);
    lo = s.sp;
    return entry_ref(spill[s.sp]);
  }
};

// 3-input max / min (a PTX form of sm_100 and later).
__device__ __forceinline__ float fmax3(float a, float b, float c) {
  float d;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}
__device__ __forceinline__ float fmin3(float a, float b, float c) {
  float d;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}

// 1 + (byte I of w) * 2^-15: the byte becomes mantissa bits 8-15 under the
// bits of 1.0f (0x3F800000), so the value is exact.
template <int I>
__device__ __forceinline__ float qbyte(uint32_t w) {
  return __uint_as_float(__byte_perm(w, 0x3F800000u, 0x7604u | ((uint32_t)I << 4)));
}

// Where a 4-wide node's four float4 come from: global memory through the
// read-only path ...
struct GlobalNodes {
  __device__ __forceinline__ void operator()(const DeviceScene& S, uint32_t node, float4& h, float4& r, float4& qa,
                                             float4& qb) const {
    ldg8_keep(S.inner, 2u * node + 0u, h, r);
    ldg8_keep(S.inner, 2u * node + 1u, qa, qb);
  }
};
// ... or, for the K nodes [base, base + K) -- the top levels of a tree, which
// the builder numbers first in breadth-first order -- a copy staged in shared
// memory (4 float4 per node from `tile`).
template <int K>
struct TiledNodes {
  const float4* tile;
  uint32_t base;
  __device__ __forceinline__ void operator()(const DeviceScene& S, uint32_t node, float4& h, float4& r, float4& qa,
                                             float4& qb) const {
    const uint32_t i = node - base;
    if (i < (uint32_t)K) {
      h = tile[4u * i + 0u];
      r = tile[4u * i + 1u];
      qa = tile[4u * i + 2u];
      qb = tile[4u * i + 3u];
    } else {
      GlobalNodes()(S, node, h, r, qa, qb);
    }
  }
};

// One 4-wide inner node: tests its children, pushes all hit children but the
// nearest, and moves to the nearest (or pops).  Returns false on stack
// overflow (s.sp = -1).
template <int STACK, class Stk, class Fetch = GlobalNodes>
__device__ __forceinline__ bool visit_wide_stk(const DeviceScene& S, Trav& s, Stk& stk, const Fetch& fetch = Fetch()) {
  if (chk(S.check, s.node >= S.n_inner, kChkNode, s.node)) {
    s.sp = -1;  // ends the ray like a stack overflow
    return false;
  }
  s.nvis++;
  float4 h, r, qa, qb;
  fetch(S, s.node, h, r, qa, qb);
  const float ax = h.w * s.ix, ay = qb.z * s.iy, az = qb.w * s.iz;
  const float bx = (h.x - s.ox) * s.ix, by = (h.y - s.oy) * s.iy, bz = (h.z - s.oz) * s.iz;
  const float cx = bx - ax, cy = by - ay, cz = bz - az;
  const float mx = fabsf(bx) + fabsf(ax), my = fabsf(by) + fabsf(ay), mz = fabsf(bz) + fabsf(az);
  const float bxn = fmaf(mx, -kWideWiden, cx), bxf = fmaf(mx, kWideWiden, cx);
  const float byn = fmaf(my, -kWideWiden, cy), byf = fmaf(my, kWideWiden, cy);
  const float bzn = fmaf(mz, -kWideWiden, cz), bzf = fmaf(mz, kWideWiden, cz);
  // near/far words per axis from the direction's sign; unused child slots
  // hold qlo = 255 > qhi = 0, an empty interval for either sign.
  const uint32_t nx = s.ix >= 0.0f ? fbits(qa.x) : fbits(qa.y), fx = s.ix >= 0.0f ? fbits(qa.y) : fbits(qa.x);
  const uint32_t ny = s.iy >= 0.0f ? fbits(qa.z) : fbits(qa.w), fy = s.iy >= 0.0f ? fbits(qa.w) : fbits(qa.z);
  const uint32_t nz = s.iz >= 0.0f ? fbits(qb.x) : fbits(qb.y), fz = s.iz >= 0.0f ? fbits(qb.y) : fbits(qb.x);
  const float inf = __int_as_float(0x7f800000);
  float t0, t1, t2, t3;
  uint32_t r0 = fbits(r.x), r1 = fbits(r.y), r2 = fbits(r.z), r3 = fbits(r.w);
#define RT_CHILD(I, T)                                                                            \
  {                                                                                               \
    float n = fmax3(fmaf(qbyte<I>(nx), ax, bxn), fmaf(qbyte<I>(ny), ay, byn), fmaf(qbyte<I>(nz), az, bzn)); \
    float f = fmin3(fmaf(qbyte<I>(fx), ax, bxf), fmaf(qbyte<I>(fy), ay, byf), fmaf(qbyte<I>(fz), az, bzf)); \
    n = fmaxf(n, s.cull_lo);                                                                      \
    f = fminf(f, s.cull_hi);                                                                      \
    T = n <= f ? n : inf;                                                                         \
  }
  RT_CHILD(0, t0) RT_CHILD(1, t1) RT_CHILD(2, t2) RT_CHILD(3, t3)
#undef RT_CHILD
  // nearest child next; the others go on the stack, the runner-up last
#define RT_SWAP(ta, ra, tb, rb)                       \
  if (tb < ta) {                                      \
    const float tt = ta; ta = tb; tb = tt;            \
    const uint32_t rr = ra; ra = rb; rb = rr;         \
  }
  RT_SWAP(t0, r0, t1, r1) RT_SWAP(t2, r2, t3, r3) RT_SWAP(t0, r0, t2, r2)
#undef RT_SWAP
  // t0 is the minimum (inf: no child hit); t2 (the other pair's minimum) is
  // pushed last
  if (!(t0 < inf)) {
    s.node = stk.pop(s);
  } else {
    const bool v3 = t3 < inf, v1 = t1 < inf, v2 = t2 < inf;
    const int np = (int)v3 + (int)v1 + (int)v2;
    if (s.sp + np > STACK) {
      s.sp = -1;
      return false;
    }
    stk.push3(s, np, v3, r3, t3, v1, r1, t1, v2, r2, t2);
    s.node = r0;
  }
  return true;
}

template <int STACK>
__device__ __forceinline__ bool visit_wide(const DeviceScene& S, Trav& s, uint2* stack) {
  LocalStack stk{stack};
  return visit_wide_stk<STACK>(S, s, stk);
}

template <bool ANY, int STACK>
__device__ __forceinline__ bool trav_run_wide(const DeviceScene& S, Trav& s, uint2* stack, int refill) {
  for (;;) {
    while (is_inner(s.node)) {
      if (!visit_wide<STACK>(S, s, stack)) return false;
      if (is_leaf(s.node) && s.leaf == 0u) {
        s.leaf = s.node;
        s.node = pop_wide(s, stack);
      }
      if (__all_sync(__activemask(), s.leaf != 0u)) break;
    }
    while (s.leaf != 0u) {
      if (leaf_visit<ANY>(S, s, s.leaf)) {
        s.leaf = 0u;
        s.node = kSentinel;
        return true;
      }
      s.leaf = 0u;
      if (is_leaf(s.node)) {
        s.leaf = s.node;
        s.node = pop_wide(s, stack);
      }
    }
    if (s.node == kSentinel) return true;
    if (refill > 0 && __popc(__activemask()) < refill) return false;
  }
}

}  // namespace dev
}  // namespace rtgb
