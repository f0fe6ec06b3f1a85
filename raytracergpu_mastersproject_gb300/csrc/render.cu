// render.cu -- the S2 pass: per-pixel path tracing with the reference RNG.
//
// One call renders spp samples of raytraceBVH.comp:main (:345-375) for every
// pixel.  The reference records spp dispatches with an image barrier between
// them (RaytracerBVH.cpp:1025-1050); a pixel's sample s+1 depends only on that
// pixel's accumulator after sample s (the RNG carry lives in alpha), so here
// one lane runs a pixel's samples back to back and the accumulator is read
// and written once.  Three schedules: the wavefront renderer (4-wide trees,
// the default: each bounce level traced by the ray-query step kernel, then
// shaded in its own pass), k_render_step (4-wide trees; one traversal or
// shading step per lane per iteration, idle lanes refilled with new pixels)
// and k_render (binary trees, or depth 0; persistent warps take 32 pixels at
// a time and run whole traversals).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <type_traits>

#include "trace_core.cuh"

namespace rtgb {
namespace {

constexpr int kThreads = 128;

struct Cam {
  float v[12];  // camPos, pixel00, pixelDeltaU, pixelDeltaV
};

struct f3 {
  float x, y, z;
};
__device__ __forceinline__ f3 mk(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 add(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 sub(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 mul(f3 a, f3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ f3 scale(f3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ f3 divs(f3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 normalize(f3 a) { return divs(a, sqrtf(dot(a, a))); }
__device__ __forceinline__ f3 reflect(f3 v, f3 n) { return sub(v, scale(n, 2.0f * dot(v, n))); }

// ---- RNG, random.glsl:10-62 ----
__device__ __forceinline__ float rng_next(uint32_t& s) {
  s = s * 747796405u + 1u;
  uint32_t word = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
  word = (word >> 22u) ^ word;
  return (float)word / 4294967295.0f;
}

// Portable sine/cosine: Cody-Waite reduction by pi/2 (three binary32 parts)
// and Taylor polynomials of degree 9 / 10 on [-pi/4, pi/4]; every operation
// rounds separately, so host and device produce the same bits.
__device__ __forceinline__ void rt_sincos(float x, float& so, float& co) {
  const float kf = rintf(x * 0x1.45f306p-1f);
  const int k = (int)kf;
  float r = x - kf * 0x1.92p+0f;
  r = r - kf * 0x1.fb6p-12f;
  r = r - kf * -0x1.777a5cp-25f;
  const float r2 = r * r;
  float ps = 0x1.71de3ap-19f;
  ps = ps * r2 + -0x1.a01a02p-13f;
  ps = ps * r2 + 0x1.111112p-7f;
  ps = ps * r2 + -0x1.555556p-3f;
  const float s = r + r * (r2 * ps);
  float pc = -0x1.27e4fcp-22f;
  pc = pc * r2 + 0x1.a01a02p-16f;
  pc = pc * r2 + -0x1.6c16c2p-10f;
  pc = pc * r2 + 0x1.555556p-5f;
  pc = pc * r2 + -0x1p-1f;
  const float c = 1.0f + r2 * pc;
  switch (k & 3) {
    case 0: so = s; co = c; break;
    case 1: so = c; co = -s; break;
    case 2: so = -s; co = -c; break;
    default: so = -c; co = s; break;
  }
}

__device__ __forceinline__ f3 random_unit_vector(uint32_t& rng) {
  const float pi = 0x1.921fb6p+1f;
  const float rho = rng_next(rng);
  const float theta = 0.0f + (2.0f * pi - 0.0f) * rng_next(rng);
  const float phi = 0.0f + (pi - 0.0f) * rng_next(rng);
  float sp, cp, st, ct;
  rt_sincos(phi, sp, cp);
  rt_sincos(theta, st, ct);
  return normalize(mk(rho * sp * ct, rho * sp * st, rho * cp));
}

// One bounce of rayColor (raytraceBVH.comp:276-315) after its closest-hit
// query: adds the background (miss) or the emitted light, and scatters.
// Returns true when the path continues from (co, cd).  A traversal that
// overflowed its stack (s.sp < 0) sets status bit 0 and counts as a miss.
__device__ __forceinline__ bool bounce(const DeviceScene& S, const dev::Trav& s, f3& co, f3& cd, f3& color, f3& gatt,
                                       uint32_t& rng, bool extended, f3 bg, uint32_t& status) {
  if (s.sp < 0) status |= 1u;
  if (s.best == dev::kNoBest || s.sp < 0) {
    const f3 b = extended ? bg : mk(0.0f, 0.0f, 0.0f);
    color = add(color, mul(b, gatt));
    return false;
  }
  const float t = s.tclose;
  f3 p, n;
  uint32_t mat;
  if (dev::chk(S.check, (s.best & kSphereBit) ? (s.best & kSphereMask) >= S.n_spheres : (s.best & kSlotMask) >= S.n_tris,
               (s.best & kSphereBit) ? dev::kChkSphere : dev::kChkTri, s.best))
    return false;
  if (s.best & kSphereBit) {
    const uint32_t idx = s.best & kSphereMask;
    const float4 c0 = dev::ldg4(S.spheres, 2u * idx);
    const float4 c1 = dev::ldg4(S.spheres, 2u * idx + 1u);
    p = add(co, scale(cd, t));
    n = divs(sub(p, mk(c0.x, c0.y, c0.z)), c0.w);
    mat = __float_as_uint(c1.x);
  } else {
    const uint32_t slot = s.best & kSlotMask;
    const float4 r0 = dev::ldg4(S.tris, 4u * slot);
    p = add(co, scale(cd, t));
    n = mk(r0.x, r0.y, r0.z);
    mat = __ldg(&S.tri_mat[slot]);
  }
  if (dev::chk(S.check, mat >= S.n_mats, dev::kChkMat, mat)) return false;
  const int back = dot(cd, n) > 0.0f ? 1 : 0;
  n = scale(n, (float)(1 - 2 * back));
  const float4 m0 = dev::ldg4(S.mats, 2u * mat);
  const float4 m1 = dev::ldg4(S.mats, 2u * mat + 1u);
  const uint32_t type = __float_as_uint(m1.x);
  const f3 albedo = mk(m0.x, m0.y, m0.z);
  const f3 em = type == RT_MAT_LIGHT ? albedo : mk(0.0f, 0.0f, 0.0f);
  color = add(color, mul(em, gatt));
  f3 att, nd;
  bool scattered = false;
  if (type == RT_MAT_DIFFUSE) {
    att = albedo;
    nd = normalize(add(n, random_unit_vector(rng)));
    scattered = true;
  } else if (extended && type == RT_MAT_METALLIC) {
    const f3 refl = normalize(reflect(cd, n));
    nd = normalize(add(refl, scale(random_unit_vector(rng), m1.y)));
    att = albedo;
    scattered = dot(nd, n) > 0.0f;
  } else if (extended && type == RT_MAT_DIELECTRIC) {
    const float ior = m1.z;
    const float ri = back ? ior : 1.0f / ior;
    const float cosv = fminf(-dot(cd, n), 1.0f);
    const float sinv = sqrtf(1.0f - cosv * cosv);
    float r0 = (1.0f - ri) / (1.0f + ri);
    r0 = r0 * r0;
    const float x = 1.0f - cosv;
    const float x2 = x * x;
    const float refl = r0 + (1.0f - r0) * (x2 * x2 * x);
    const float rnd = rng_next(rng);
    f3 dir;
    if (ri * sinv > 1.0f || refl > rnd) {
      dir = reflect(cd, n);
    } else {
      const f3 perp = scale(add(cd, scale(n, cosv)), ri);
      const f3 par = scale(n, -sqrtf(fabsf(1.0f - dot(perp, perp))));
      dir = add(perp, par);
    }
    att = mk(1.0f, 1.0f, 1.0f);
    nd = normalize(dir);
    scattered = true;
  }
  if (!scattered) return false;
  gatt = mul(gatt, att);
  co = p;
  cd = nd;
  return true;
}

// rayColor with the whole traversal of each bounce in one call.
template <int W, int STACK, typename StackT, typename WC>
__device__ f3 ray_color(const DeviceScene& S, f3 o, f3 d, uint32_t depth, uint32_t& rng, bool extended, f3 bg,
                        StackT* stack, uint32_t& status, WC& wc) {
  f3 color = mk(0.0f, 0.0f, 0.0f);
  f3 gatt = mk(1.0f, 1.0f, 1.0f);
  f3 co = o, cd = normalize(d);
  for (uint32_t i = 0; i < depth; ++i) {
    dev::Trav s;
    dev::trav_init_ray(s, make_float4(co.x, co.y, co.z, 0.001f), make_float4(cd.x, cd.y, cd.z, 10000000.0f), S.root);
    if constexpr (W == 2) {
      stack[0] = kSentinel;
      dev::trav_run<false, STACK>(S, s, stack, 0);
    } else {
      dev::trav_run_wide<false, STACK>(S, s, stack, 0);
    }
    wc.add(s);
    if (!bounce(S, s, co, cd, color, gatt, rng, extended, bg, status)) break;
  }
  return color;
}

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Work counters of rt_render_count: closest-hit queries, inner nodes fetched,
// primitives tested.  Kernels without STATS never store them, so the adds
// are dead code there.
struct WorkCount {
  unsigned long long queries = 0, nodes = 0, prims = 0;
  __device__ __forceinline__ void add(const dev::Trav& s) {
    queries += 1;
    nodes += s.nvis;
    prims += s.ntest;
  }
  __device__ __forceinline__ void flush(unsigned long long* stats) {
    for (int o = 16; o > 0; o >>= 1) {
      queries += __shfl_down_sync(0xFFFFFFFFu, queries, o);
      nodes += __shfl_down_sync(0xFFFFFFFFu, nodes, o);
      prims += __shfl_down_sync(0xFFFFFFFFu, prims, o);
    }
    if ((threadIdx.x & 31u) == 0u) {
      atomicAdd(&stats[0], queries);
      atomicAdd(&stats[1], nodes);
      atomicAdd(&stats[2], prims);
    }
  }
};

template <int W, int STACK, bool STATS>
__global__ void __launch_bounds__(kThreads) k_render(DeviceScene S, Cam cam, uint32_t depth, uint32_t random_state,
                                                     float4* __restrict__ accum, uint32_t Wd, uint32_t H, uint32_t spp,
                                                     uint32_t mode, float bgx, float bgy, float bgz,
                                                     uint32_t* __restrict__ counter,
                                                     unsigned long long* __restrict__ stats) {
  WorkCount wc;
  using StackT = typename std::conditional<W == 2, uint32_t, uint2>::type;
  StackT stack[STACK];
  const uint32_t total = Wd * H;
  const uint32_t lane = threadIdx.x & 31u;
  const f3 pos = mk(cam.v[0], cam.v[1], cam.v[2]);
  const f3 p00 = mk(cam.v[3], cam.v[4], cam.v[5]);
  const f3 pdu = mk(cam.v[6], cam.v[7], cam.v[8]);
  const f3 pdv = mk(cam.v[9], cam.v[10], cam.v[11]);
  const f3 bg = mk(bgx, bgy, bgz);
  uint32_t status = 0;
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(counter, 32u);
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
    if (base >= total) break;
    const uint32_t i = base + lane;
    if (i < total) {
      const uint32_t x = i % Wd, y = i / Wd;
      float4 px = accum[i];
      for (uint32_t smp = 0; smp < spp; ++smp) {
        uint32_t rng = (600u * x + y) * (random_state + 1u);  // random.glsl:9
        rng += __float2uint_rz(px.w * 4294967294.0f);         // :350, saturating
        const float next = rng_next(rng);                     // :352 (:351 is a no-op)
        const f3 sample = add(add(p00, scale(pdu, (float)x)), scale(pdv, (float)y));
        const f3 d = normalize(sub(sample, pos));
        const f3 c = ray_color<W, STACK>(S, pos, d, depth, rng, (mode & kRenderExtended) != 0u, bg, stack, status, wc);
        px.x = c.x + px.x;
        px.y = c.y + px.y;
        px.z = c.z + px.z;
        px.w = next;
      }
      accum[i] = px;
    }
  }
  if (status) atomicOr(counter + 1, status);
  if constexpr (STATS) wc.flush(stats);
}

// 4-wide trees: every lane is a small state machine that makes one move per
// iteration of the warp's loop -- one node visit, one leaf test, or the
// shading of a finished bounce followed by the start of the next bounce, the
// next sample or the end of the pixel.  Lanes of a warp thus stay busy while
// their paths have different lengths, and a warp takes new pixels for its
// idle lanes once `refill` lanes are idle.  A lane still runs its pixel's
// samples in order, so the accumulator sums are the same as k_render's.  Each
// phase's code appears once in the loop, which keeps the kernel small enough
// for the instruction cache.
template <int STACK, int THREADS, int MINB, bool STATS>
__global__ void __launch_bounds__(THREADS, MINB)
    k_render_step(DeviceScene S, Cam cam, uint32_t depth, uint32_t random_state, float4* __restrict__ accum,
                  uint32_t Wd, uint32_t H, uint32_t spp, uint32_t mode, float bgx, float bgy, float bgz,
                  uint32_t* __restrict__ counter, int refill, unsigned long long* __restrict__ stats) {
  WorkCount wc;
  enum : uint32_t { kIdle, kTraverse, kShade, kNewSample };
  uint2 stack[STACK];
  dev::Trav s;
  const uint32_t total = Wd * H;
  const uint32_t lane = threadIdx.x & 31u;
  const f3 bg = mk(bgx, bgy, bgz);
  const int min_idle = refill < 1 ? 1 : (refill > 32 ? 32 : refill);
  const bool extended = (mode & kRenderExtended) != 0u;
  const bool share = (mode & kRenderTraceEveryPrimary) == 0u;
  uint32_t status = 0;
  uint32_t phase = kIdle, pix = 0, smp = 0, nb = 0, rng = 0;
  uint32_t first_best = 0;  // the pixel's first hit (sample 0, bounce 0)
  float first_t = 0.0f;
  int first_sp = 0;
  float4 px = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  f3 color = mk(0.0f, 0.0f, 0.0f), gatt = mk(1.0f, 1.0f, 1.0f), co = color, cd = color;
  bool exhausted = spp == 0u;
  for (;;) {
    const uint32_t idle = __ballot_sync(0xFFFFFFFFu, phase == kIdle);
    if (exhausted && idle == 0xFFFFFFFFu) break;
    if (!exhausted && __popc(idle) >= min_idle) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(counter, (uint32_t)__popc(idle));
      base = __shfl_sync(0xFFFFFFFFu, base, 0);
      if (base + (uint32_t)__popc(idle) >= total) exhausted = true;
      if (phase == kIdle) {
        const uint32_t id = base + (uint32_t)__popc(idle & lanemask_lt());
        if (id < total) {
          pix = id;
          px = accum[id];
          smp = 0;
          phase = kNewSample;
        }
      }
    }
    if (phase == kTraverse) {
      if (dev::is_inner(s.node)) {
        if (!dev::visit_wide<STACK>(S, s, stack)) s.node = kSentinel;  // overflow: s.sp = -1
      } else if (dev::is_leaf(s.node)) {
        dev::leaf_visit<false>(S, s, s.node);
        s.node = dev::pop_wide(s, stack);
      }
      if (s.node != kSentinel) continue;
      phase = kShade;  // the query is done: shade in this iteration
    }
    bool trace = false;
    if (phase == kShade) {
      if (nb == 0u && smp == 0u) {  // keep the pixel's first hit for its later samples
        first_best = s.best;
        first_t = s.tclose;
        first_sp = s.sp;
      }
      if (STATS && (nb != 0u || smp == 0u || !share)) wc.add(s);
      if (bounce(S, s, co, cd, color, gatt, rng, extended, bg, status) && ++nb < depth) {
        trace = true;
      } else {  // the sample is done
        px.x = color.x + px.x;
        px.y = color.y + px.y;
        px.z = color.z + px.z;
        if (++smp < spp) {
          phase = kNewSample;
        } else {
          accum[pix] = px;
          phase = kIdle;
        }
      }
    }
    if (phase == kNewSample) {  // raytraceBVH.comp:345-375 up to the first query
      const uint32_t x = pix % Wd, y = pix / Wd;
      rng = (600u * x + y) * (random_state + 1u);  // random.glsl:9
      rng += __float2uint_rz(px.w * 4294967294.0f);  // :350, saturating
      px.w = rng_next(rng);                          // :352 (:351 is a no-op); read by the next sample
      const f3 pos = mk(cam.v[0], cam.v[1], cam.v[2]);
      const f3 sample = add(add(mk(cam.v[3], cam.v[4], cam.v[5]), scale(mk(cam.v[6], cam.v[7], cam.v[8]), (float)x)),
                            scale(mk(cam.v[9], cam.v[10], cam.v[11]), (float)y));
      const f3 d = normalize(sub(sample, pos));
      color = mk(0.0f, 0.0f, 0.0f);
      gatt = mk(1.0f, 1.0f, 1.0f);
      co = pos;
      cd = normalize(d);
      nb = 0;
      if (share && smp > 0u) {  // the same primary ray: its first hit is known
        s.best = first_best;
        s.tclose = first_t;
        s.sp = first_sp < 0 ? -1 : 0;
        phase = kShade;
      } else {
        trace = true;  // depth >= 1 (the launcher sends depth 0 to k_render)
      }
    }
    if (trace) {
      dev::trav_init_ray(s, make_float4(co.x, co.y, co.z, 0.001f), make_float4(cd.x, cd.y, cd.z, 10000000.0f), S.root);
      if (s.leaf != 0u) {  // the whole tree is one leaf
        s.node = s.leaf;
        s.leaf = 0u;
      }
      phase = kTraverse;
    }
  }
  if (status) atomicOr(counter + 1, status);
  if constexpr (STATS) wc.flush(stats);
}

// ---------------------------------------------------------- wavefront ----
// 4-wide trees: the frame runs level by level (bounce 0, 1, ...).  Each level
// traces all of its rays with the ray-query step kernel (RAW hits) and then
// shades them in a separate pass, one path per thread, which appends the
// continuing paths and their next rays to the next level's list.  Traversal
// and shading thus each run with the lanes of a warp doing the same kind of
// work.  A path's RNG state starts from the pixel's alpha carry chain, which
// needs no tracing (k_wave_seed), and each pixel adds its samples' colours in
// sample order at the end (k_wave_accum), so the accumulator is the same as
// with one lane running the pixel's samples back to back.
//
// Path p of a pass over npix pixels x ns samples is sample p % ns of pixel
// p / ns: a pixel's samples start from the same hit point, and kept adjacent
// they keep their next rays in the same warps.  The starting RNG states are
// stored sample-major (rng0[k * npix + q]) so that k_wave_seed's stores are
// coalesced.  Scratch per path: state (color.xyz, rng | gatt.xyz, -) 32 B,
// the starting RNG state 4 B, two ray buffers 2 x 32 B, two path lists
// 2 x 4 B, hits 8 B.
struct WaveBufs {
  float4* state;  // 2 float4 per path
  uint32_t* rng0;
  float4* rays[2];
  uint32_t* list[2];
  uint2* hits;
  uint32_t* cnt;  // 4 words per level: trace queue, -, ray count, -
};

__global__ void k_wave_seed(Cam cam, uint32_t random_state, float4* __restrict__ accum, uint32_t Wd, uint32_t pix0,
                            uint32_t npix, uint32_t ns, uint32_t per_path, uint32_t* __restrict__ rng0,
                            float4* __restrict__ rays) {
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < npix; q += gridDim.x * blockDim.x) {
    const uint32_t pix = pix0 + q;
    const uint32_t x = pix % Wd, y = pix / Wd;
    float4 px = accum[pix];
    for (uint32_t k = 0; k < ns; ++k) {
      uint32_t rng = (600u * x + y) * (random_state + 1u);  // random.glsl:9
      rng += __float2uint_rz(px.w * 4294967294.0f);         // raytraceBVH.comp:350, saturating
      px.w = rng_next(rng);                                 // :352 (:351 is a no-op)
      rng0[(size_t)k * npix + q] = rng;
    }
    accum[pix] = px;  // the carry after these samples; the colours are added by k_wave_accum
    const f3 pos = mk(cam.v[0], cam.v[1], cam.v[2]);
    const f3 sample = add(add(mk(cam.v[3], cam.v[4], cam.v[5]), scale(mk(cam.v[6], cam.v[7], cam.v[8]), (float)x)),
                          scale(mk(cam.v[9], cam.v[10], cam.v[11]), (float)y));
    const f3 cd = normalize(normalize(sub(sample, pos)));  // getRay, then rayColor's normalize
    const float4 o = make_float4(pos.x, pos.y, pos.z, 0.001f);
    const float4 d = make_float4(cd.x, cd.y, cd.z, 10000000.0f);
    if (per_path) {
      for (uint32_t k = 0; k < ns; ++k) {
        const size_t p = (size_t)q * ns + k;
        rays[2 * p] = o;
        rays[2 * p + 1] = d;
      }
    } else {
      rays[2 * (size_t)q] = o;
      rays[2 * (size_t)q + 1] = d;
    }
  }
}

// Shades level `level`: n0 = npix * ns paths at level 0 (path p's ray is
// rays[p] or, when the pixel's first hit is shared, rays[p / ns]; colour 0,
// throughput 1, RNG from rng0); later levels take the count from the level's
// counter block and path ids from `list`.
template <bool STATS>
__global__ void k_wave_shade(DeviceScene S, uint32_t level, uint32_t depth, uint32_t n0, uint32_t npix, uint32_t ns,
                             uint32_t per_path, uint32_t mode, float bgx, float bgy, float bgz,
                             float4* __restrict__ state, const uint32_t* __restrict__ rng0,
                             const float4* __restrict__ rays, const uint32_t* __restrict__ list,
                             const uint2* __restrict__ hits, float4* __restrict__ next_rays,
                             uint32_t* __restrict__ next_list, uint32_t* __restrict__ cnt,
                             uint32_t* __restrict__ status_word, unsigned long long* __restrict__ stats) {
  const uint32_t n = level == 0 ? n0 : *reinterpret_cast<volatile uint32_t*>(cnt + 4u * level + 2u);
  if (STATS && level == 0 && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&stats[0], (unsigned long long)(per_path ? n0 : npix));
  if (STATS && level > 0 && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&stats[0], (unsigned long long)n);
  const bool extended = (mode & kRenderExtended) != 0u;
  const f3 bg = mk(bgx, bgy, bgz);
  uint32_t status = 0;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < n; i0 += stride) {  // warp-uniform trip count
    const uint32_t i = i0 + threadIdx.x;
    bool more = false;
    uint32_t p = 0;
    f3 co = mk(0.0f, 0.0f, 0.0f), cd = co;
    if (i < n && !dev::chk(S.check, level > 0 && list[i] >= n0, dev::kChkPath, level > 0 ? list[i] : i)) {
      p = level == 0 ? i : list[i];
      const uint32_t r = level == 0 ? (per_path ? i : i / ns) : i;
      const float4 o = rays[2 * (size_t)r], d = rays[2 * (size_t)r + 1];
      const uint2 h = hits[r];
      dev::Trav s;
      s.best = h.x == kRawOverflow ? 0u : h.x;
      s.sp = h.x == kRawOverflow ? -1 : 0;
      s.tclose = __uint_as_float(h.y);
      f3 color = mk(0.0f, 0.0f, 0.0f), gatt = mk(1.0f, 1.0f, 1.0f);
      uint32_t rng;
      if (level == 0) {
        rng = rng0[(size_t)(p % ns) * npix + p / ns];
      } else {
        const float4 a = state[2 * (size_t)p], g = state[2 * (size_t)p + 1];
        color = mk(a.x, a.y, a.z);
        gatt = mk(g.x, g.y, g.z);
        rng = __float_as_uint(a.w);
      }
      co = mk(o.x, o.y, o.z);
      cd = mk(d.x, d.y, d.z);
      more = bounce(S, s, co, cd, color, gatt, rng, extended, bg, status) && level + 1u < depth;
      state[2 * (size_t)p] = make_float4(color.x, color.y, color.z, __uint_as_float(rng));
      state[2 * (size_t)p + 1] = make_float4(gatt.x, gatt.y, gatt.z, 0.0f);
    }
    // append the continuing paths: one atomicAdd per warp
    const uint32_t m = __ballot_sync(0xFFFFFFFFu, more);
    if (m) {
      const uint32_t lane = threadIdx.x & 31u;
      uint32_t base = 0;
      if (lane == (uint32_t)(__ffs(m) - 1)) base = atomicAdd(cnt + 4u * (level + 1u) + 2u, (uint32_t)__popc(m));
      base = __shfl_sync(0xFFFFFFFFu, base, __ffs(m) - 1);
      if (more) {
        const uint32_t j = base + (uint32_t)__popc(m & lanemask_lt());
        next_list[j] = p;
        next_rays[2 * (size_t)j] = make_float4(co.x, co.y, co.z, 0.001f);
        next_rays[2 * (size_t)j + 1] = make_float4(cd.x, cd.y, cd.z, 10000000.0f);
      }
    }
  }
  if (status) atomicOr(status_word, status);
}

__global__ void k_wave_accum(float4* __restrict__ accum, uint32_t pix0, uint32_t npix, uint32_t ns,
                             const float4* __restrict__ state) {
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < npix; q += gridDim.x * blockDim.x) {
    float4 px = accum[pix0 + q];
    for (uint32_t k = 0; k < ns; ++k) {
      const float4 c = state[2 * ((size_t)q * ns + k)];
      px.x = c.x + px.x;
      px.y = c.y + px.y;
      px.z = c.z + px.z;
    }
    accum[pix0 + q] = px;
  }
}

constexpr size_t kWaveBytesPerPath = 32 + 4 + 64 + 8 + 8;
// Two launches per level: deeper paths go to k_render_step instead.
constexpr uint32_t kWaveMaxDepth = 64;

WaveBufs wave_bufs(void* scratch, uint64_t paths, uint32_t depth) {
  auto up = [](size_t v) { return (v + 255) & ~(size_t)255; };
  char* b = static_cast<char*>(scratch);
  WaveBufs w;
  size_t off = 0;
  w.state = reinterpret_cast<float4*>(b + off);
  off += up(paths * 32);
  w.rng0 = reinterpret_cast<uint32_t*>(b + off);
  off += up(paths * 4);
  w.rays[0] = reinterpret_cast<float4*>(b + off);
  off += up(paths * 32);
  w.rays[1] = reinterpret_cast<float4*>(b + off);
  off += up(paths * 32);
  w.list[0] = reinterpret_cast<uint32_t*>(b + off);
  off += up(paths * 4);
  w.list[1] = reinterpret_cast<uint32_t*>(b + off);
  off += up(paths * 4);
  w.hits = reinterpret_cast<uint2*>(b + off);
  off += up(paths * 8);
  w.cnt = reinterpret_cast<uint32_t*>(b + off);
  (void)depth;
  return w;
}

// Scratch of one stream's part for `paths` paths.
size_t wave_part_bytes(uint64_t paths, uint32_t depth) {
  const size_t b = (size_t)paths * kWaveBytesPerPath + 8 * 256 + 16 * ((size_t)depth + 1);
  return (b + 255) & ~(size_t)255;  // the next stream's part starts 256-byte aligned
}

// A frame below this many paths per chunk stays one chunk on one stream.
constexpr uint64_t kWaveMinChunkPaths = 1u << 16;

// Pixel chunks rotate over the caller's stream and the extra streams given,
// each stream with its own part of the scratch: chunk c+1's bounce levels run
// while chunk c's are in flight, so one chunk's launch tails (the drain of a
// persistent trace grid, a short shading pass) overlap another's work.  All
// samples of a pixel stay in one chunk, in order, so the accumulator and its
// RNG carry are the same as with one stream.
template <bool STATS>
cudaError_t launch_render_wave(const DeviceScene& S, const Cam& cam, uint32_t depth, uint32_t rs, float* accum_f,
                               uint32_t Wd, uint32_t H, uint32_t spp, uint32_t mode, const float bg[3],
                               uint32_t* counter, unsigned long long* stats, void* scratch, uint64_t max_paths,
                               cudaStream_t st, const RenderStreams* streams) {
  float4* accum = reinterpret_cast<float4*>(accum_f);
  const uint32_t total = Wd * H;
  const uint32_t per_path = (mode & kRenderTraceEveryPrimary) ? 1u : 0u;
  // Streams used: all given, unless the whole frame fits the scratch and
  // splitting it would leave chunks below kWaveMinChunkPaths.
  const uint64_t frame_paths = (uint64_t)total * spp;
  int used = 1 + (streams ? std::min(streams->extra, kWaveLanes - 1) : 0);
  while (used > 1 && frame_paths <= max_paths && frame_paths < (uint64_t)used * kWaveMinChunkPaths) --used;
  const uint64_t cap = (max_paths + used - 1) / used;  // paths per stream's scratch part
  const uint32_t ns_pass = (uint32_t)std::min<uint64_t>(spp, cap);
  const uint32_t q_cap = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(total, cap / ns_pass));
  // equal chunks, as many as the capacity needs, a multiple of the streams
  uint64_t n_chunks = std::max<uint64_t>(((uint64_t)total + q_cap - 1) / q_cap, (uint64_t)used);
  n_chunks = (n_chunks + used - 1) / used * used;
  const uint32_t q_chunk = (uint32_t)(((uint64_t)total + n_chunks - 1) / n_chunks);
  WaveBufs Bs[kWaveLanes];
  cudaStream_t sts[kWaveLanes];
  for (int k = 0; k < used; ++k) {
    Bs[k] = wave_bufs(static_cast<char*>(scratch) + (size_t)k * wave_part_bytes(cap, depth), cap, depth);
    sts[k] = k == 0 ? st : streams->streams[k - 1];
  }
  const uint32_t sms = (uint32_t)device_sm_count();
  unsigned long long* trace_stats = STATS ? stats + 1 : nullptr;
  cudaError_t e;
  if (used > 1) {
    if ((e = cudaEventRecord(streams->fork, st)) != cudaSuccess) return e;
    for (int k = 1; k < used; ++k)
      if ((e = cudaStreamWaitEvent(sts[k], streams->fork, 0)) != cudaSuccess) return e;
  }
  auto chunks = [&]() -> cudaError_t {
    cudaError_t e2;
    uint32_t chunk = 0;
    for (uint32_t pix0 = 0; pix0 < total; pix0 += q_chunk, ++chunk) {
      const uint32_t q = std::min(q_chunk, total - pix0);
      const WaveBufs& B = Bs[chunk % (uint32_t)used];
      const cudaStream_t cs = sts[chunk % (uint32_t)used];
      for (uint32_t s0 = 0; s0 < spp; s0 += ns_pass) {
        const uint32_t ns = std::min(ns_pass, spp - s0);
        const uint32_t np = q * ns;
        if ((e2 = cudaMemsetAsync(B.cnt, 0, 16 * ((size_t)depth + 1), cs)) != cudaSuccess) return e2;
        const uint32_t gb = std::min<uint32_t>(sms * 8, (q + 255) / 256);
        k_wave_seed<<<gb, 256, 0, cs>>>(cam, rs, accum, Wd, pix0, q, ns, per_path, B.rng0, B.rays[0]);
        for (uint32_t l = 0; l < depth; ++l) {
          const float4* r = B.rays[l & 1u];
          if ((e2 = launch_trace_raw(S, r, l == 0 ? (per_path ? np : q) : 0xFFFFFFFFu, B.hits, B.cnt + 4u * l,
                                     trace_stats, cs)) != cudaSuccess)
            return e2;
          const uint32_t gs = l == 0 ? std::min<uint32_t>(sms * 8, (np + 255) / 256) : sms * 8;
          k_wave_shade<STATS><<<gs, 256, 0, cs>>>(S, l, depth, np, q, ns, per_path, mode, bg[0], bg[1], bg[2],
                                                  B.state, B.rng0, r, B.list[l & 1u], B.hits,
                                                  B.rays[(l + 1u) & 1u], B.list[(l + 1u) & 1u], B.cnt,
                                                  counter + 1, stats);
        }
        k_wave_accum<<<gb, 256, 0, cs>>>(accum, pix0, q, ns, B.state);
        if ((e2 = cudaGetLastError()) != cudaSuccess) return e2;
      }
    }
    return cudaSuccess;
  };
  e = chunks();
  // the caller's stream waits for every extra stream, also after a failed
  // launch, so that nothing of this call is left unordered behind it
  for (int k = 1; k < used; ++k) {
    cudaError_t ej = cudaEventRecord(streams->join[k - 1], sts[k]);
    if (ej == cudaSuccess) ej = cudaStreamWaitEvent(st, streams->join[k - 1], 0);
    if (e == cudaSuccess) e = ej;
  }
  return e != cudaSuccess ? e : cudaGetLastError();
}

__global__ void k_clear(float4* accum, uint32_t total) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x)
    accum[i] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
}

// SingleTriangleFullScreen.frag:13-18
__global__ void k_resolve(const float4* accum, uint32_t total, float inv_spp_den, float4* out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const float4 a = accum[i];
    float4 r;
    r.x = fminf(fmaxf(sqrtf(a.x / inv_spp_den), 0.0f), 1.0f);
    r.y = fminf(fmaxf(sqrtf(a.y / inv_spp_den), 0.0f), 1.0f);
    r.z = fminf(fmaxf(sqrtf(a.z / inv_spp_den), 0.0f), 1.0f);
    r.w = 1.0f;
    out[i] = r;
  }
}

template <int W, int STACK, bool STATS>
cudaError_t launch_render_variant(const DeviceScene& S, const Cam& cam, uint32_t depth, uint32_t rs, float* accum,
                                  uint32_t w, uint32_t h, uint32_t spp, uint32_t shade, const float bg[3],
                                  uint32_t* counter, unsigned long long* stats, cudaStream_t st) {
  static int cache = -1;
  int blocks_per_sm = 0;
  if (cudaError_t e = cached_blocks_per_sm(&cache, k_render<W, STACK, STATS>, kThreads, &blocks_per_sm);
      e != cudaSuccess)
    return e;
  const uint32_t total = w * h;
  uint32_t blocks = (uint32_t)(device_sm_count() * blocks_per_sm);
  const uint32_t needed = (total + kThreads - 1) / kThreads;
  if (blocks > needed) blocks = needed;
  if (blocks == 0) blocks = 1;
  k_render<W, STACK, STATS><<<blocks, kThreads, 0, st>>>(S, cam, depth, rs, reinterpret_cast<float4*>(accum), w, h,
                                                         spp, shade, bg[0], bg[1],
                                                         bg[2], counter, stats);
  return cudaGetLastError();
}

template <int STACK, int T, int M, bool STATS>
cudaError_t launch_render_step(const DeviceScene& S, const Cam& cam, uint32_t depth, uint32_t rs, float* accum,
                               uint32_t w, uint32_t h, uint32_t spp, uint32_t shade, const float bg[3],
                               uint32_t* counter, int refill, unsigned long long* stats, cudaStream_t st) {
  static int cache = -1;
  int blocks_per_sm = 0;
  if (cudaError_t e = cached_blocks_per_sm(&cache, k_render_step<STACK, T, M, STATS>, T, &blocks_per_sm);
      e != cudaSuccess)
    return e;
  const uint32_t total = w * h;
  uint32_t blocks = (uint32_t)(device_sm_count() * blocks_per_sm);
  const uint32_t needed = (total + T - 1) / T;
  if (blocks > needed) blocks = needed;
  if (blocks == 0) blocks = 1;
  k_render_step<STACK, T, M, STATS><<<blocks, T, 0, st>>>(S, cam, depth, rs, reinterpret_cast<float4*>(accum), w, h,
                                                          spp, shade, bg[0], bg[1],
                                                          bg[2], counter, refill, stats);
  return cudaGetLastError();
}

int env_int(const char* name, int dflt) {
  const char* e = std::getenv(name);
  return e ? std::atoi(e) : dflt;
}

// 0: k_render (one thread per pixel, whole traversals); 1-3: k_render_step
// with 128 threads and at least 8, 6 or 10 blocks per SM (6: 72 registers, no
// spills; 8 and 10 spill); 4: the wavefront renderer (the default; depth up
// to kWaveMaxDepth, deeper frames use variant 2).
struct RenderTuning {
  int variant, refill;
};
const RenderTuning& render_tuning() {
  static const RenderTuning t{env_int("RT_RENDER_VARIANT", 4), env_int("RT_RENDER_REFILL", 8)};
  return t;
}

template <bool STATS>
cudaError_t launch_render_impl(const DeviceScene& s, const Cam& c, uint32_t depth, uint32_t random_state, float* accum,
                               uint32_t w, uint32_t h, uint32_t spp, uint32_t mode, const float bg[3],
                               uint32_t* counter, unsigned long long* stats, void* scratch, uint64_t scratch_paths,
                               cudaStream_t st, const RenderStreams* rs) {
  const RenderTuning& tn = render_tuning();
  if (s.width == 4 && depth > 0u && depth <= kWaveMaxDepth && tn.variant == 4 && scratch && scratch_paths > 0)
    return launch_render_wave<STATS>(s, c, depth, random_state, accum, w, h, spp, mode, bg, counter, stats, scratch,
                                     scratch_paths, st, rs);
  if (s.width == 4 && depth > 0u && tn.variant >= 1 && tn.variant <= 4) {  // 4: depth beyond the wavefront's
    const bool big = s.stack_need > 64u;
#define RT_STEP(STK, T, M)                                                                                         \
  launch_render_step<STK, T, M, STATS>(s, c, depth, random_state, accum, w, h, spp, mode, bg, counter, \
                                       tn.refill, stats, st)
    if (tn.variant == 2 || tn.variant == 4) return big ? RT_STEP(192, 128, 6) : RT_STEP(64, 128, 6);
    if (tn.variant == 3) return big ? RT_STEP(192, 128, 10) : RT_STEP(64, 128, 10);
    return big ? RT_STEP(192, 128, 8) : RT_STEP(64, 128, 8);
#undef RT_STEP
  }
#define RT_PIX(W, STK) \
  launch_render_variant<W, STK, STATS>(s, c, depth, random_state, accum, w, h, spp, mode, bg, counter, stats, st)
  if (s.width == 4) return s.stack_need <= 64u ? RT_PIX(4, 64) : RT_PIX(4, 192);
  return s.stack_need <= 64u ? RT_PIX(2, 64) : RT_PIX(2, 128);
#undef RT_PIX
}

}  // namespace

cudaError_t launch_render(const DeviceScene& s, const float cam[12], uint32_t depth, uint32_t random_state,
                          float* accum, uint32_t w, uint32_t h, uint32_t spp, uint32_t mode, const float bg[3],
                          uint32_t* counter, void* stream, unsigned long long* stats, void* scratch,
                          uint64_t scratch_paths, const RenderStreams* rs) {
  Cam c;
  for (int k = 0; k < 12; ++k) c.v[k] = cam[k];
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (stats)
    return launch_render_impl<true>(s, c, depth, random_state, accum, w, h, spp, mode, bg, counter, stats, scratch,
                                    scratch_paths, st, rs);
  return launch_render_impl<false>(s, c, depth, random_state, accum, w, h, spp, mode, bg, counter, nullptr, scratch,
                                   scratch_paths, st, rs);
}

bool render_uses_scratch(const DeviceScene& s, uint32_t depth) {
  return s.width == 4 && depth > 0u && depth <= kWaveMaxDepth && render_tuning().variant == 4;
}

size_t render_scratch_bytes(uint64_t paths, uint32_t depth) {
  size_t most = 0;  // any split of the paths over 1..kWaveLanes streams fits
  for (uint64_t k = 1; k <= (uint64_t)kWaveLanes; ++k)
    most = std::max(most, (size_t)k * wave_part_bytes((paths + k - 1) / k, depth));
  return most;
}

cudaError_t launch_accum_clear(float* accum, uint32_t w, uint32_t h, void* stream) {
  const uint32_t total = w * h;
  uint32_t blocks = (total + 255u) / 256u;
  if (blocks > 4096u) blocks = 4096u;
  if (blocks == 0) return cudaSuccess;
  k_clear<<<blocks, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(reinterpret_cast<float4*>(accum), total);
  return cudaGetLastError();
}

cudaError_t launch_resolve(const float* accum, uint32_t w, uint32_t h, uint32_t spp, float* out, void* stream) {
  const uint32_t total = w * h;
  uint32_t blocks = (total + 255u) / 256u;
  if (blocks > 4096u) blocks = 4096u;
  if (blocks == 0) return cudaSuccess;
  k_resolve<<<blocks, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(reinterpret_cast<const float4*>(accum), total,
                                                                        (float)spp, reinterpret_cast<float4*>(out));
  return cudaGetLastError();
}

}  // namespace rtgb
