// ref_shim.hpp -- GLSL 450 types, built-ins and a compute-workgroup model in
// C++, so that the reference's compute shaders compile unmodified in meaning
// as host C++ (oracle/ref_glsl.py rewrites only GLSL-only syntax around them).
//
// TEST INFRASTRUCTURE ONLY: the library built from this header
// (oracle/_ref/libref_glsl*.so) is the reference's own shader code run on
// the CPU.  It pins the oracle (oracle/rt_oracle.c); the product never
// links it.
//
// Semantics chosen where GLSL leaves them open (the oracle and the CUDA
// kernels make the same choices):
//   * every + - * / sqrt is one IEEE-754 binary32 operation in the order
//     written (the recipe compiles with -ffp-contract=off);
//     dot(a,b) = (a.x*b.x + a.y*b.y) + a.z*b.z, normalize(v) = v / sqrt(dot(v,v))
//     per component, mat4*vec4 sums the columns left to right;
//   * min/max ignore a NaN operand (fminf/fmaxf); GLSL leaves NaN undefined;
//   * float -> uint conversion saturates (NaN and negatives -> 0, >= 2^32 ->
//     0xFFFFFFFF); GLSL leaves out-of-range conversions undefined;
//   * an uninitialised vec3 local reads as NaN, so that the min/max folds of
//     GetEnclosingAABB.comp:69-91, which start from uninitialised locals,
//     fold over the data alone;
//   * tan() is evaluated in binary64 and rounded; sin()/cos() are libm's
//     sinf/cosf, or, with REF_PORTABLE_SINCOS, the portable binary32
//     sin/cos of oracle/rt_sincos.h that the oracle and the CUDA kernels use;
//   * radians(x) = x * (pi/180 rounded to binary32).
// Workgroup model: with barriers, each invocation of a workgroup is its own
// host thread; barrier() is a std::barrier over the workgroup; subgroups are
// 32 consecutive invocations and subgroup operations are collective over
// them (they are only called in uniform control flow in these shaders);
// subgroupElect() is true on invocation 0 of the subgroup.  A `shared uint`
// is a sequentially consistent atomic word, so that spin loops on shared
// memory (GetEnclosingAABB.comp:98) observe other invocations' writes.
#pragma once

#include <atomic>
#include <barrier>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <thread>

#ifdef REF_PORTABLE_SINCOS
extern "C" {
#include "rt_sincos.h"
}
#endif

namespace glsl {

typedef uint32_t uint;

// ------------------------------------------------------------------ types --
struct swz2 { float x, y; };
struct swz3 { float x, y, z; };  // a .xyz / .rgb view of a vec4 (trivial)

struct uvec2 { uint x, y; };
struct ivec2 {
  int x, y;
  ivec2() = default;
  ivec2(int a, int b) : x(a), y(b) {}
  explicit ivec2(uvec2 u) : x((int)u.x), y((int)u.y) {}
};
struct vec2 {
  float x, y;
  vec2() = default;
  vec2(float a, float b) : x(a), y(b) {}
  explicit vec2(ivec2 v) : x((float)v.x), y((float)v.y) {}
  vec2(uvec2 v) : x((float)v.x), y((float)v.y) {}  // GLSL converts uint -> float implicitly
};

struct vec3 {
  float x, y, z;
  vec3() : x(std::numeric_limits<float>::quiet_NaN()), y(x), z(x) {}
  explicit vec3(float s) : x(s), y(s), z(s) {}
  vec3(float a, float b, float c) : x(a), y(b), z(c) {}
  vec3(const swz3& s) : x(s.x), y(s.y), z(s.z) {}
};

struct alignas(16) vec4 {
  union {
    struct { float x, y, z, w; };
    struct { float r, g, b, a; };
    swz3 xyz;
    swz3 rgb;
    swz2 xy;
    float v[4];
  };
  vec4() = default;
  explicit vec4(float s) { v[0] = v[1] = v[2] = v[3] = s; }
  vec4(float a_, float b_, float c_, float d_) { v[0] = a_; v[1] = b_; v[2] = c_; v[3] = d_; }
  vec4(const vec3& p, float q) { v[0] = p.x; v[1] = p.y; v[2] = p.z; v[3] = q; }
};

struct uvec3 {
  union {
    struct { uint x, y, z; };
    uvec2 xy;
  };
  uvec3() = default;
  uvec3(uint a, uint b, uint c) { x = a; y = b; z = c; }
  explicit uvec3(const vec3& f);
};

struct alignas(16) mat4 { vec4 col[4]; };

// ------------------------------------------------------------ arithmetic --
inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator/(const vec3& a, const vec3& b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline vec3 operator+(const vec3& a, float s) { return vec3(a.x + s, a.y + s, a.z + s); }
inline vec3 operator-(const vec3& a, float s) { return vec3(a.x - s, a.y - s, a.z - s); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator*(float s, const vec3& a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3& operator+=(vec3& a, const vec3& b) { return a = a + b; }
inline vec3& operator-=(vec3& a, const vec3& b) { return a = a - b; }
inline vec3& operator*=(vec3& a, const vec3& b) { return a = a * b; }
inline vec3& operator*=(vec3& a, float s) { return a = a * s; }
inline vec3& operator/=(vec3& a, float s) { return a = a / s; }

inline vec4 operator+(const vec4& a, const vec4& b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline vec4 operator-(const vec4& a, const vec4& b) { return vec4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
inline vec4 operator*(const vec4& a, float s) { return vec4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline vec4 operator/(const vec4& a, float s) { return vec4(a.x / s, a.y / s, a.z / s, a.w / s); }

inline vec4 operator*(const mat4& m, const vec4& p) {
  vec4 r;
  for (int row = 0; row < 4; ++row)
    r.v[row] = m.col[0].v[row] * p.x + m.col[1].v[row] * p.y + m.col[2].v[row] * p.z + m.col[3].v[row] * p.w;
  return r;
}

// ------------------------------------------------------------- built-ins --
inline float dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3 cross(const vec3& a, const vec3& b) {
  return vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float sqrt(float x) { return ::sqrtf(x); }
inline vec3 normalize(const vec3& a) { return a / glsl::sqrt(dot(a, a)); }
inline float abs(float x) { return ::fabsf(x); }
inline int abs(int x) { return x < 0 ? -x : x; }
inline float min(float a, float b) { return ::fminf(a, b); }
inline float max(float a, float b) { return ::fmaxf(a, b); }
inline int min(int a, int b) { return b < a ? b : a; }
inline int max(int a, int b) { return a < b ? b : a; }
inline uint min(uint a, uint b) { return b < a ? b : a; }
inline uint max(uint a, uint b) { return a < b ? b : a; }
inline vec3 min(const vec3& a, const vec3& b) { return vec3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline vec3 max(const vec3& a, const vec3& b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline vec4 min(const vec4& a, const vec4& b) { return vec4(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z), min(a.w, b.w)); }
inline vec4 max(const vec4& a, const vec4& b) { return vec4(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z), max(a.w, b.w)); }
inline float radians(float deg) { return deg * 0.01745329251994329577f; }
inline float tan(float x) { return (float)::tan((double)x); }
#ifdef REF_PORTABLE_SINCOS
inline float sin(float x) { float s, c; rt_sincos(x, &s, &c); return s; }
inline float cos(float x) { float s, c; rt_sincos(x, &s, &c); return c; }
#else
inline float sin(float x) { return ::sinf(x); }
inline float cos(float x) { return ::cosf(x); }
#endif
inline float atan(float y, float x) { return ::atan2f(y, x); }
inline float acos(float x) { return ::acosf(x); }
inline int findMSB(uint v) { return v == 0u ? -1 : 31 - __builtin_clz(v); }
inline int bitCount(uint v) { return __builtin_popcount(v); }

// uint(x): saturating from float, plain from integers.
inline uint glsl_uint(float f) {
  if (!(f > 0.0f)) return 0u;
  if (f >= 4294967296.0f) return 0xFFFFFFFFu;
  return (uint)f;
}
inline uint glsl_uint(double f) { return glsl_uint((float)f); }
inline uint glsl_uint(uint u) { return u; }
inline uint glsl_uint(int i) { return (uint)i; }
inline uvec3::uvec3(const vec3& f) { x = glsl_uint(f.x); y = glsl_uint(f.y); z = glsl_uint(f.z); }

// s.xxx on a scalar or a vector
inline vec3 glsl_xxx(float s) { return vec3(s, s, s); }
inline vec3 glsl_xxx(const vec3& v) { return vec3(v.x, v.x, v.x); }
inline vec3 glsl_xxx(const vec4& v) { return vec3(v.x, v.x, v.x); }

// --------------------------------------------------------------- atomics --
inline void spin_hint() {
  thread_local unsigned n = 0;
  if ((++n & 63u) == 0u) std::this_thread::yield();
}
struct shared_u32 {
  std::atomic<uint> a{0u};
  operator uint() const { spin_hint(); return a.load(); }
  shared_u32& operator=(uint x) { a.store(x); return *this; }
};
inline uint atomicAdd(shared_u32& s, uint v) { return s.a.fetch_add(v); }
inline uint atomicAnd(shared_u32& s, uint v) { return s.a.fetch_and(v); }
inline uint atomicAdd(uint& s, uint v) { return std::atomic_ref<uint>(s).fetch_add(v); }
inline uint atomicAnd(uint& s, uint v) { return std::atomic_ref<uint>(s).fetch_and(v); }
inline int atomicAdd(int& s, int v) { return std::atomic_ref<int>(s).fetch_add(v); }

// ----------------------------------------------------------------- image --
// The raytrace pass's accumulator: RGBA32F texels, row-major (the format the
// reference allocates, RaytracerBVH.cpp:408; the shader's rgba8 qualifier on
// that image is undefined, and float storage is used).
struct image2D {
  float* texels;
  int width, height;
};
struct texel_read { vec4 rgba; };
inline ivec2 imageSize(const image2D& im) { return ivec2(im.width, im.height); }
inline texel_read imageLoad(const image2D& im, ivec2 p) {
  const float* t = im.texels + ((size_t)p.y * (size_t)im.width + (size_t)p.x) * 4u;
  return texel_read{vec4(t[0], t[1], t[2], t[3])};
}
inline void imageStore(image2D& im, ivec2 p, const vec4& c) {
  float* t = im.texels + ((size_t)p.y * (size_t)im.width + (size_t)p.x) * 4u;
  t[0] = c.x; t[1] = c.y; t[2] = c.z; t[3] = c.w;
}

// ------------------------------------------------------------- workgroup --
constexpr int kSubgroupSize = 32;

struct Subgroup {
  std::barrier<> bar{kSubgroupSize};
  alignas(16) unsigned char slot[kSubgroupSize][16];
};

struct Workgroup {
  std::barrier<> bar;
  Subgroup* sub;
  int nsub;
  explicit Workgroup(int size) : bar(size), sub(new Subgroup[(size + kSubgroupSize - 1) / kSubgroupSize]),
                                 nsub((size + kSubgroupSize - 1) / kSubgroupSize) {}
  ~Workgroup() { delete[] sub; }
  Workgroup(const Workgroup&) = delete;
  Workgroup& operator=(const Workgroup&) = delete;
};

// Descriptor bindings (by binding number) and the workgroup of a dispatch.
struct Env {
  void* bind[16];
  Workgroup* wg;  // null when the kernel is run without barriers
};

// What every translated shader class derives from: the invocation's
// built-in variables and the collective built-ins.
struct InvocationBase {
  const Env& env;
  uvec3 gl_GlobalInvocationID;
  uvec3 gl_LocalInvocationID;
  uvec3 gl_WorkGroupID;
  uint gl_SubgroupID;
  uint gl_SubgroupInvocationID;

  InvocationBase(const Env& e, uvec3 gid, uvec3 lid, uvec3 wid)
      : env(e), gl_GlobalInvocationID(gid), gl_LocalInvocationID(lid), gl_WorkGroupID(wid),
        gl_SubgroupID(lid.x / (uint)kSubgroupSize), gl_SubgroupInvocationID(lid.x % (uint)kSubgroupSize) {}

  void barrier() const { env.wg->bar.arrive_and_wait(); }

  template <class T, class Fold>
  T sub_collective(const T& v, Fold fold) const {
    Subgroup& sg = env.wg->sub[gl_SubgroupID];
    static_assert(sizeof(T) <= 16, "subgroup slot");
    std::memcpy(sg.slot[gl_SubgroupInvocationID], &v, sizeof(T));
    sg.bar.arrive_and_wait();
    T out = fold(sg);
    sg.bar.arrive_and_wait();  // slots may be reused afterwards
    return out;
  }
  static uint slot_u(const Subgroup& sg, int lane) { uint u; std::memcpy(&u, sg.slot[lane], 4); return u; }
  static vec3 slot_v3(const Subgroup& sg, int lane) { vec3 v; std::memcpy(&v, sg.slot[lane], sizeof(vec3)); return v; }

  vec3 subgroupMin(const vec3& v) const {
    return sub_collective(v, [](const Subgroup& sg) {
      vec3 r = slot_v3(sg, 0);
      for (int l = 1; l < kSubgroupSize; ++l) r = min(r, slot_v3(sg, l));
      return r;
    });
  }
  vec3 subgroupMax(const vec3& v) const {
    return sub_collective(v, [](const Subgroup& sg) {
      vec3 r = slot_v3(sg, 0);
      for (int l = 1; l < kSubgroupSize; ++l) r = max(r, slot_v3(sg, l));
      return r;
    });
  }
  uint subgroupAdd(uint v) const {
    return sub_collective(v, [](const Subgroup& sg) {
      uint r = 0;
      for (int l = 0; l < kSubgroupSize; ++l) r += slot_u(sg, l);
      return r;
    });
  }
  uint subgroupExclusiveAdd(uint v) const {
    const int me = (int)gl_SubgroupInvocationID;
    return sub_collective(v, [me](const Subgroup& sg) {
      uint r = 0;
      for (int l = 0; l < me; ++l) r += slot_u(sg, l);
      return r;
    });
  }
  bool subgroupElect() const { return gl_SubgroupInvocationID == 0u; }
};

}  // namespace glsl
