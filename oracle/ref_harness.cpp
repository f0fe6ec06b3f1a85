// ref_harness.cpp -- dispatch entry points over the reference's own compute
// shaders compiled as C++ (oracle/ref_glsl.py generates the k_*.inc classes).
//
// TEST INFRASTRUCTURE ONLY: tests/ use it to pin the oracle
// (oracle/rt_oracle.c) to the reference, and bench.py's reference arm times
// ref_trace on the host cores.  The product never links it.
//
// Each entry point binds buffers by the binding numbers of the shader's
// descriptor set and dispatches the shader's main() (or calls one of its
// functions) the way RaytracerBVH.cpp records the passes:
//   S1 (RaytracerBVH.cpp:778-991): ModelSpaceToWorldSpace, GetEnclosingAABB,
//      GenerateMortonCodesOfPrimitives, RadixSortSimple, ConstructHLBVH,
//      ConstructAABBsOfInternalNodes, with the dispatch sizes recorded there;
//   S2 (RaytracerBVH.cpp:1025-1050): raytraceBVH.comp over
//      (W/32+1) x (H/32+1) workgroups of 32x32, once per sample.
// Invocations of a dispatch without barriers run one after another (or, for
// the raytrace pass, in parallel over pixel rows: each invocation touches
// only its own pixel); dispatches with barriers run each invocation of the
// workgroup on its own thread (glsl::Workgroup).
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "ref_shim.hpp"

#include "k_raytraceBVH.inc"
#include "k_ModelSpaceToWorldSpace.inc"
#include "k_GetEnclosingAABB.inc"
#include "k_GenerateMortonCodesOfPrimitives.inc"
#include "k_RadixSortSimple.inc"
#include "k_ConstructHLBVH.inc"
#include "k_ConstructAABBsOfInternalNodes.inc"

using namespace glsl;

namespace {

using RT = k_raytraceBVH::Invocation;
static_assert(sizeof(RT::Triangle) == 64 && sizeof(RT::Sphere) == 32 && sizeof(RT::Material) == 32 &&
                  sizeof(RT::HLBVHNode) == 40 && sizeof(RT::MortonPrimitive) == 12 && sizeof(RT::Model) == 64 &&
                  sizeof(RT::HLBVHAABBConstructionInfo) == 8,
              "std430 record sizes (definitions.glsl)");
static_assert(offsetof(RT::Triangle, materialIndex) == 48 && offsetof(RT::Sphere, radius) == 16,
              "std430 record offsets");
static_assert(sizeof(RT::ParameterUBO) == 80 && offsetof(RT::ParameterUBO, verticalFOV) == 48 &&
                  offsetof(RT::ParameterUBO, randomState) == 72,
              "std140 ParameterUBO (raytraceBVH.comp:7-18)");

// Runs f(i) for i in [0, n) over up to nthreads threads, in chunks.
template <class F>
void parallel_for(uint32_t n, uint32_t nthreads, uint32_t chunk, F f) {
  if (nthreads <= 1 || n <= chunk) {
    for (uint32_t i = 0; i < n; ++i) f(i, 0u);
    return;
  }
  std::atomic<uint32_t> next{0};
  std::vector<std::thread> th;
  for (uint32_t t = 0; t < nthreads; ++t)
    th.emplace_back([&, t] {
      for (;;) {
        const uint32_t b = next.fetch_add(chunk);
        if (b >= n) break;
        const uint32_t e = b + chunk < n ? b + chunk : n;
        for (uint32_t i = b; i < e; ++i) f(i, t);
      }
    });
  for (auto& x : th) x.join();
}

// Every invocation of `groups` workgroups, one after another, in workgroup
// order and then local-index order.
template <class K>
void dispatch_serial(const Env& env, uint32_t groups_x) {
  for (uint32_t g = 0; g < groups_x; ++g)
    for (uint32_t l = 0; l < K::kLocalSizeX; ++l) {
      K inv(env, uvec3(g * K::kLocalSizeX + l, 0u, 0u), uvec3(l, 0u, 0u), uvec3(g, 0u, 0u));
      inv.main();
    }
}

// One workgroup whose invocations synchronise: each runs on its own thread.
template <class K>
void dispatch_workgroup(const Env& env_in) {
  constexpr uint32_t n = K::kLocalSizeX;
  Workgroup wg((int)n);
  Env env = env_in;
  env.wg = &wg;
  std::vector<std::thread> th;
  th.reserve(n);
  for (uint32_t l = 0; l < n; ++l)
    th.emplace_back([&env, l] {
      K inv(env, uvec3(l, 0u, 0u), uvec3(l, 0u, 0u), uvec3(0u, 0u, 0u));
      inv.main();
    });
  for (auto& x : th) x.join();
}

RT::ParameterUBO make_ubo(uint32_t nt, uint32_t ns) {
  RT::ParameterUBO u;
  std::memset(&u, 0, sizeof(u));
  u.verticalFOV = 60.0f;
  u.numTriangles = nt;
  u.numSpheres = ns;
  u.maxRayTraceDepth = 1u;
  return u;
}

struct RayIn { float o[3]; float tmin; float d[3]; float tmax; };
struct HitOut { uint32_t prim; float t; };

}  // namespace

extern "C" {

uint32_t ref_abi(void) { return 1u; }

// ----------------------------------------------------------------- S2 ----
// hitBVH (raytraceBVH.comp:195-265) on each ray with the ray's own interval.
// The hit primitive is read back through HitRecord.materialIndex, which
// triangleHit / sphereHit copy from the primitive: the harness binds copies
// of the triangle and sphere buffers whose materialIndex is the triangle's
// index, or 0x80000000 | the sphere's index.
int ref_trace(const void* nodes, uint32_t nn, const void* tris, uint32_t nt, const void* sph, uint32_t ns,
              const void* rays, uint32_t n, void* hits, uint32_t nthreads) {
  if (nn == 0) return -1;
  std::vector<RT::Triangle> T(nt ? nt : 1);
  std::vector<RT::Sphere> S(ns ? ns : 1);
  if (nt) std::memcpy(T.data(), tris, sizeof(RT::Triangle) * nt);
  if (ns) std::memcpy(S.data(), sph, sizeof(RT::Sphere) * ns);
  for (uint32_t i = 0; i < nt; ++i) T[i].materialIndex = i;
  for (uint32_t i = 0; i < ns; ++i) S[i].materialIndex = 0x80000000u | i;
  RT::Material M{};
  RT::ParameterUBO ubo = make_ubo(nt, ns);
  float pixel[4] = {0, 0, 0, 1};
  image2D img{pixel, 1, 1};
  const RayIn* R = static_cast<const RayIn*>(rays);
  HitOut* H = static_cast<HitOut*>(hits);
  const uint32_t nth = nthreads ? nthreads : 1u;
  std::vector<std::vector<float>> scratch(nth, std::vector<float>(64, 0.0f));
  parallel_for(n, nth, 256u, [&](uint32_t i, uint32_t t) {
    Env env{};
    env.bind[0] = &ubo;
    env.bind[1] = &img;
    env.bind[2] = T.data();
    env.bind[3] = S.data();
    env.bind[4] = &M;
    env.bind[5] = const_cast<void*>(nodes);
    env.bind[6] = scratch[t].data();
    RT inv(env, uvec3(0u, 0u, 0u), uvec3(0u, 0u, 0u), uvec3(0u, 0u, 0u));
    RT::Ray r{vec3(R[i].o[0], R[i].o[1], R[i].o[2]), vec3(R[i].d[0], R[i].d[1], R[i].d[2])};
    RT::HitRecord rec;
    if (inv.hitBVH(r, R[i].tmin, R[i].tmax, rec)) {
      H[i].prim = rec.materialIndex;
      H[i].t = rec.t;
    } else {
      H[i].prim = 0xFFFFFFFFu;
      H[i].t = std::numeric_limits<float>::infinity();
    }
  });
  return 0;
}

// The raytrace pass: spp dispatches of main() (raytraceBVH.comp:345-375)
// over the accumulator (W*H RGBA32F texels, updated in place).
int ref_render(const void* ubo80, float* accum, uint32_t W, uint32_t H, uint32_t spp, const void* tris, uint32_t nt,
               const void* sph, uint32_t ns, const void* mats, uint32_t nm, const void* nodes, uint32_t nn,
               uint32_t nthreads) {
  (void)nt; (void)ns; (void)nm; (void)nn;
  RT::ParameterUBO ubo;
  std::memcpy(&ubo, ubo80, sizeof(ubo));
  image2D img{accum, (int)W, (int)H};
  const uint32_t gx = W / 32u + 1u, gy = H / 32u + 1u;
  const uint32_t nth = nthreads ? nthreads : 1u;
  std::vector<std::vector<float>> scratch(nth, std::vector<float>(64, 0.0f));
  for (uint32_t s = 0; s < spp; ++s) {
    parallel_for(gy * 32u, nth, 4u, [&](uint32_t y, uint32_t t) {
      Env env{};
      env.bind[0] = &ubo;
      env.bind[1] = &img;
      env.bind[2] = const_cast<void*>(tris);
      env.bind[3] = const_cast<void*>(sph);
      env.bind[4] = const_cast<void*>(mats);
      env.bind[5] = const_cast<void*>(nodes);
      env.bind[6] = scratch[t].data();
      for (uint32_t x = 0; x < gx * 32u; ++x) {
        RT inv(env, uvec3(x, y, 0u), uvec3(x % 32u, y % 32u, 0u), uvec3(x / 32u, y / 32u, 0u));
        inv.main();
      }
    });
  }
  return 0;
}

// Camera of the raytrace pass for a W x H image: the globals of
// raytraceBVH.comp:54-76 as one invocation computes them.
// out[0..11] = camPos, pixel00Location, pixelDeltaU, pixelDeltaV.
void ref_camera(const void* ubo80, uint32_t W, uint32_t H, float* out) {
  RT::ParameterUBO ubo;
  std::memcpy(&ubo, ubo80, sizeof(ubo));
  float pixel[4] = {0, 0, 0, 1};
  std::vector<float> tex((size_t)W * H * 4u + 4u, 0.0f);
  image2D img{tex.data(), (int)W, (int)H};
  Env env{};
  env.bind[0] = &ubo;
  env.bind[1] = &img;
  (void)pixel;
  RT inv(env, uvec3(0u, 0u, 0u), uvec3(0u, 0u, 0u), uvec3(0u, 0u, 0u));
  const vec3 p = ubo.camPos.xyz;
  const vec3 v[4] = {p, inv._pixel00Location, inv._pixelDeltaU, inv._pixelDeltaV};
  for (int i = 0; i < 4; ++i) {
    out[3 * i] = v[i].x;
    out[3 * i + 1] = v[i].y;
    out[3 * i + 2] = v[i].z;
  }
}

// getRay (raytraceBVH.comp:329-342) for every pixel; rays[i] = {o, d} with
// tmin/tmax of sceneHit (:268-269).
void ref_get_rays(const void* ubo80, uint32_t W, uint32_t H, void* rays_out) {
  RT::ParameterUBO ubo;
  std::memcpy(&ubo, ubo80, sizeof(ubo));
  std::vector<float> tex((size_t)W * H * 4u, 0.0f);
  image2D img{tex.data(), (int)W, (int)H};
  Env env{};
  env.bind[0] = &ubo;
  env.bind[1] = &img;
  RayIn* R = static_cast<RayIn*>(rays_out);
  for (uint32_t y = 0; y < H; ++y)
    for (uint32_t x = 0; x < W; ++x) {
      RT inv(env, uvec3(x, y, 0u), uvec3(x % 32u, y % 32u, 0u), uvec3(x / 32u, y / 32u, 0u));
      const RT::Ray r = inv.getRay(uvec2{x, y});
      RayIn& o = R[(size_t)y * W + x];
      o.o[0] = r.origin.x; o.o[1] = r.origin.y; o.o[2] = r.origin.z;
      o.d[0] = r.direction.x; o.d[1] = r.direction.y; o.d[2] = r.direction.z;
      o.tmin = 0.001f;
      o.tmax = 10000000.0f;
    }
}

// The per-invocation RNG seed (random.glsl:10).
uint32_t ref_seed(uint32_t x, uint32_t y, uint32_t random_state) {
  RT::ParameterUBO ubo = make_ubo(0, 0);
  ubo.randomState = random_state;
  float pixel[4] = {0, 0, 0, 1};
  image2D img{pixel, 1, 1};
  Env env{};
  env.bind[0] = &ubo;
  env.bind[1] = &img;
  RT inv(env, uvec3(x, y, 0u), uvec3(0u, 0u, 0u), uvec3(0u, 0u, 0u));
  return inv.rngState;
}

static RT* rng_invocation(Env& env, RT::ParameterUBO& ubo, image2D& img) {
  env.bind[0] = &ubo;
  env.bind[1] = &img;
  return new RT(env, uvec3(0u, 0u, 0u), uvec3(0u, 0u, 0u), uvec3(0u, 0u, 0u));
}

// n draws of random() (random.glsl:25-27) from state s: floats and states.
void ref_random_stream(uint32_t s, uint32_t n, float* out, uint32_t* states) {
  RT::ParameterUBO ubo = make_ubo(0, 0);
  float pixel[4] = {0, 0, 0, 1};
  image2D img{pixel, 1, 1};
  Env env{};
  RT* inv = rng_invocation(env, ubo, img);
  inv->rngState = s;
  for (uint32_t i = 0; i < n; ++i) {
    out[i] = inv->random();
    if (states) states[i] = inv->rngState;
  }
  delete inv;
}

// n draws of randomUnitVector() (random.glsl:60-62) from state s.
void ref_random_unit_vectors(uint32_t s, uint32_t n, float* out3) {
  RT::ParameterUBO ubo = make_ubo(0, 0);
  float pixel[4] = {0, 0, 0, 1};
  image2D img{pixel, 1, 1};
  Env env{};
  RT* inv = rng_invocation(env, ubo, img);
  inv->rngState = s;
  for (uint32_t i = 0; i < n; ++i) {
    const vec3 v = inv->randomUnitVector();
    out3[3 * i] = v.x;
    out3[3 * i + 1] = v.y;
    out3[3 * i + 2] = v.z;
  }
  delete inv;
}

// ----------------------------------------------------------------- S1 ----
// The six BVH-build passes in the order and with the dispatch sizes of
// recordComputeS1CommandBuffer (RaytracerBVH.cpp:778-991), on copies of the
// caller's triangles and spheres (pass 1 transforms them in place).
// models: nmodels column-major 4x4 matrices (the Model buffer).
// Outputs (each may be NULL but nodes): nodes[2N-1], the sorted Morton codes
// [N], the sorted primitives [N] (index | 0x80000000 for spheres), and the
// padded enclosing box of the centroids (min xyz, max xyz).
int ref_build_bvh(const void* tris, uint32_t nt, const void* sph, uint32_t ns, const float* models,
                  uint32_t nmodels, void* nodes_out, uint32_t* codes_out, uint32_t* prims_out,
                  float* enclosing_out) {
  using MS = k_ModelSpaceToWorldSpace::Invocation;
  using EA = k_GetEnclosingAABB::Invocation;
  using MC = k_GenerateMortonCodesOfPrimitives::Invocation;
  using RS = k_RadixSortSimple::Invocation;
  using CH = k_ConstructHLBVH::Invocation;
  using CA = k_ConstructAABBsOfInternalNodes::Invocation;
  const uint32_t N = nt + ns;
  if (N == 0 || nmodels == 0 || !models) return -1;
  std::vector<RT::Triangle> T(nt ? nt : 1);
  std::vector<RT::Sphere> S(ns ? ns : 1);
  if (nt) std::memcpy(T.data(), tris, sizeof(RT::Triangle) * nt);
  if (ns) std::memcpy(S.data(), sph, sizeof(RT::Sphere) * ns);
  for (uint32_t i = 0; i < nt; ++i)
    if (T[i].modelIndex >= nmodels) return -2;
  for (uint32_t i = 0; i < ns; ++i)
    if (S[i].modelIndex >= nmodels) return -2;
  std::vector<mat4> Mo(nmodels);
  std::memcpy(Mo.data(), models, sizeof(mat4) * nmodels);
  RT::ParameterUBO ubo = make_ubo(nt, ns);
  vec4 enclosing[2] = {vec4(0.0f), vec4(0.0f)};
  std::vector<RT::MortonPrimitive> m1(N), m2(N);
  std::vector<RT::HLBVHNode> nodes(2 * N - 1);
  std::vector<RT::HLBVHAABBConstructionInfo> info(2 * N - 1);
  std::memset(nodes.data(), 0, sizeof(RT::HLBVHNode) * nodes.size());
  std::memset(info.data(), 0, sizeof(RT::HLBVHAABBConstructionInfo) * info.size());
  std::vector<float> scratch(64, 0.0f);

  Env e{};
  e.bind[0] = &ubo;
  // 1. ModelSpaceToWorldSpace (:778-789), (N/32)+1 groups of 32
  e.bind[1] = Mo.data(); e.bind[2] = T.data(); e.bind[3] = S.data();
  dispatch_serial<MS>(e, N / 32u + 1u);
  // 2. GetEnclosingAABB (:831-842), one workgroup of 256
  e = Env{}; e.bind[0] = &ubo;
  e.bind[1] = enclosing; e.bind[2] = T.data(); e.bind[3] = S.data(); e.bind[4] = scratch.data();
  dispatch_workgroup<EA>(e);
  // 3. GenerateMortonCodesOfPrimitives (:868-879), (N/32)+1 groups of 32
  e = Env{}; e.bind[0] = &ubo;
  e.bind[1] = enclosing; e.bind[2] = T.data(); e.bind[3] = S.data(); e.bind[4] = m1.data(); e.bind[5] = scratch.data();
  dispatch_serial<MC>(e, N / 32u + 1u);
  // 4. RadixSortSimple (:905-916), one workgroup of 256
  e = Env{}; e.bind[0] = &ubo;
  e.bind[1] = m1.data(); e.bind[2] = m2.data();
  dispatch_workgroup<RS>(e);
  // 5. ConstructHLBVH (:943-954), (N/256)+1 groups of 256
  e = Env{}; e.bind[0] = &ubo;
  e.bind[1] = T.data(); e.bind[2] = S.data(); e.bind[3] = m1.data(); e.bind[4] = nodes.data(); e.bind[5] = info.data();
  dispatch_serial<CH>(e, N / 256u + 1u);
  // 6. ConstructAABBsOfInternalNodes (:980-991), (N/32)+1 groups of 32
  e = Env{}; e.bind[0] = &ubo;
  e.bind[1] = nodes.data(); e.bind[2] = info.data();
  dispatch_serial<CA>(e, N / 32u + 1u);

  std::memcpy(nodes_out, nodes.data(), sizeof(RT::HLBVHNode) * nodes.size());
  for (uint32_t i = 0; i < N; ++i) {
    if (codes_out) codes_out[i] = m1[i].code;
    if (prims_out) prims_out[i] = m1[i].primitiveIndex | (m1[i].primitiveType == 0u ? 0x80000000u : 0u);
  }
  if (enclosing_out) {
    enclosing_out[0] = enclosing[0].x; enclosing_out[1] = enclosing[0].y; enclosing_out[2] = enclosing[0].z;
    enclosing_out[3] = enclosing[1].x; enclosing_out[4] = enclosing[1].y; enclosing_out[5] = enclosing[1].z;
  }
  return 0;
}

}  // extern "C"
