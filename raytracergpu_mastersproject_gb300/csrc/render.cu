// render.cu -- the S2 pass: per-pixel path tracing with the reference RNG.
//
// One call renders spp samples of raytraceBVH.comp:main (:345-375) for every
// pixel.  The reference records spp dispatches with an image barrier between
// them (RaytracerBVH.cpp:1025-1050); a pixel's sample s+1 depends only on that
// pixel's accumulator after sample s (the RNG carry lives in alpha), so here
// one lane runs a pixel's samples back to back and the accumulator is read
// and written once.  Two kernels: k_render_step (4-wide trees; one traversal
// or shading step per lane per iteration, idle lanes refilled with new
// pixels) and k_render (binary trees, or depth 0; persistent warps take 32
// pixels at a time and run whole traversals).
#include <cuda_runtime.h>

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
template <int W, int STACK, typename StackT>
__device__ f3 ray_color(const DeviceScene& S, f3 o, f3 d, uint32_t depth, uint32_t& rng, bool extended, f3 bg,
                        StackT* stack, uint32_t& status) {
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
    if (!bounce(S, s, co, cd, color, gatt, rng, extended, bg, status)) break;
  }
  return color;
}

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

template <int W, int STACK>
__global__ void __launch_bounds__(kThreads) k_render(DeviceScene S, Cam cam, uint32_t depth, uint32_t random_state,
                                                     float4* __restrict__ accum, uint32_t Wd, uint32_t H, uint32_t spp,
                                                     uint32_t extended, float bgx, float bgy, float bgz,
                                                     uint32_t* __restrict__ counter) {
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
        const f3 c = ray_color<W, STACK>(S, pos, d, depth, rng, extended != 0u, bg, stack, status);
        px.x = c.x + px.x;
        px.y = c.y + px.y;
        px.z = c.z + px.z;
        px.w = next;
      }
      accum[i] = px;
    }
  }
  if (status) atomicOr(counter + 1, status);
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
template <int STACK, int THREADS, int MINB>
__global__ void __launch_bounds__(THREADS, MINB)
    k_render_step(DeviceScene S, Cam cam, uint32_t depth, uint32_t random_state, float4* __restrict__ accum,
                  uint32_t Wd, uint32_t H, uint32_t spp, uint32_t extended, float bgx, float bgy, float bgz,
                  uint32_t* __restrict__ counter, int refill) {
  enum : uint32_t { kIdle, kTraverse, kShade, kNewSample };
  uint2 stack[STACK];
  dev::Trav s;
  const uint32_t total = Wd * H;
  const uint32_t lane = threadIdx.x & 31u;
  const f3 bg = mk(bgx, bgy, bgz);
  const int min_idle = refill < 1 ? 1 : (refill > 32 ? 32 : refill);
  uint32_t status = 0;
  uint32_t phase = kIdle, pix = 0, smp = 0, nb = 0, rng = 0;
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
      if (bounce(S, s, co, cd, color, gatt, rng, extended != 0u, bg, status) && ++nb < depth) {
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
      trace = true;  // depth >= 1 (the launcher sends depth 0 to k_render)
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

template <int W, int STACK>
cudaError_t launch_render_variant(const DeviceScene& S, const Cam& cam, uint32_t depth, uint32_t rs, float* accum,
                                  uint32_t w, uint32_t h, uint32_t spp, uint32_t shade, const float bg[3],
                                  uint32_t* counter, cudaStream_t st) {
  static int blocks_per_sm = -1;
  if (blocks_per_sm < 0) {
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_render<W, STACK>, kThreads, 0);
    if (e != cudaSuccess) return e;
    if (blocks_per_sm < 1) blocks_per_sm = 1;
  }
  const uint32_t total = w * h;
  uint32_t blocks = (uint32_t)(device_sm_count() * blocks_per_sm);
  const uint32_t needed = (total + kThreads - 1) / kThreads;
  if (blocks > needed) blocks = needed;
  if (blocks == 0) blocks = 1;
  k_render<W, STACK><<<blocks, kThreads, 0, st>>>(S, cam, depth, rs, reinterpret_cast<float4*>(accum), w, h, spp,
                                               shade == RT_SHADE_EXTENDED ? 1u : 0u, bg[0], bg[1], bg[2], counter);
  return cudaGetLastError();
}

template <int STACK, int T, int M>
cudaError_t launch_render_step(const DeviceScene& S, const Cam& cam, uint32_t depth, uint32_t rs, float* accum,
                               uint32_t w, uint32_t h, uint32_t spp, uint32_t shade, const float bg[3],
                               uint32_t* counter, int refill, cudaStream_t st) {
  static int blocks_per_sm = -1;
  if (blocks_per_sm < 0) {
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_render_step<STACK, T, M>, T, 0);
    if (e != cudaSuccess) return e;
    if (blocks_per_sm < 1) blocks_per_sm = 1;
  }
  const uint32_t total = w * h;
  uint32_t blocks = (uint32_t)(device_sm_count() * blocks_per_sm);
  const uint32_t needed = (total + T - 1) / T;
  if (blocks > needed) blocks = needed;
  if (blocks == 0) blocks = 1;
  k_render_step<STACK, T, M><<<blocks, T, 0, st>>>(S, cam, depth, rs, reinterpret_cast<float4*>(accum), w, h, spp,
                                                   shade == RT_SHADE_EXTENDED ? 1u : 0u, bg[0], bg[1], bg[2], counter,
                                                   refill);
  return cudaGetLastError();
}

int env_int(const char* name, int dflt) {
  const char* e = std::getenv(name);
  return e ? std::atoi(e) : dflt;
}

// 0: k_render (one thread per pixel, whole traversals); 1-3: k_render_step
// with 128 threads and at least 8, 6 or 10 blocks per SM (6: 72 registers, no
// spills -- the default; 8 and 10 spill).
struct RenderTuning {
  int variant, refill;
};
const RenderTuning& render_tuning() {
  static const RenderTuning t{env_int("RT_RENDER_VARIANT", 2), env_int("RT_RENDER_REFILL", 8)};
  return t;
}

}  // namespace

cudaError_t launch_render(const DeviceScene& s, const float cam[12], uint32_t depth, uint32_t random_state,
                          float* accum, uint32_t w, uint32_t h, uint32_t spp, uint32_t shade_mode, const float bg[3],
                          uint32_t* counter, void* stream) {
  Cam c;
  for (int k = 0; k < 12; ++k) c.v[k] = cam[k];
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const RenderTuning& tn = render_tuning();
  if (s.width == 4 && depth > 0u && tn.variant >= 1 && tn.variant <= 3) {
    const bool big = s.stack_need > 64u;
#define RT_STEP(STK, T, M) \
  launch_render_step<STK, T, M>(s, c, depth, random_state, accum, w, h, spp, shade_mode, bg, counter, tn.refill, st)
    if (tn.variant == 2) return big ? RT_STEP(192, 128, 6) : RT_STEP(64, 128, 6);
    if (tn.variant == 3) return big ? RT_STEP(192, 128, 10) : RT_STEP(64, 128, 10);
    return big ? RT_STEP(192, 128, 8) : RT_STEP(64, 128, 8);
#undef RT_STEP
  }
  if (s.width == 4) {
    if (s.stack_need <= 64u)
      return launch_render_variant<4, 64>(s, c, depth, random_state, accum, w, h, spp, shade_mode, bg, counter, st);
    return launch_render_variant<4, 192>(s, c, depth, random_state, accum, w, h, spp, shade_mode, bg, counter, st);
  }
  if (s.stack_need <= 64u)
    return launch_render_variant<2, 64>(s, c, depth, random_state, accum, w, h, spp, shade_mode, bg, counter, st);
  return launch_render_variant<2, 128>(s, c, depth, random_state, accum, w, h, spp, shade_mode, bg, counter, st);
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
