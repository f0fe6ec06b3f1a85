// scenes.cpp -- seeded synthetic workloads (see include/rt_gb300_workloads.h).
// Compiled with -ffp-contract=off like the rest of the host code.
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/rt_gb300_workloads.h"
#include "rt_internal.h"

namespace rtgb {
void set_error(const std::string& msg);
}

namespace {

using rtgb::parallel_for;

inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
inline uint64_t stream_key(uint64_t seed, uint64_t stream) {
  return splitmix64(splitmix64(seed) ^ (stream * 0xD1B54A32D192ED03ull));
}
inline double u01(uint64_t key, uint64_t i) { return (double)(splitmix64(key + i) >> 11) * 0x1p-53; }
inline double gauss(uint64_t key, uint64_t i) {
  const double u1 = u01(key, 2 * i), u2 = u01(key, 2 * i + 1);
  return std::sqrt(-2.0 * std::log(1.0 - u1)) * std::cos(6.283185307179586 * u2);
}

void set_tri(RtTriangle64& t, const double* a, const double* b, const double* c, uint32_t mat) {
  std::memset(&t, 0, sizeof(t));
  for (int k = 0; k < 3; ++k) {
    t.v0[k] = (float)a[k];
    t.v1[k] = (float)b[k];
    t.v2[k] = (float)c[k];
  }
  t.materialIndex = mat;
}

// Icosahedron (12 unit vertices, 20 faces) split `subdiv` times; each face
// (a,b,c) becomes (a,ab,ca), (b,bc,ab), (c,ca,bc), (ab,bc,ca) with edge
// midpoints projected to the sphere.  Shared edges give identical midpoints.
std::vector<double> icosphere_unit(uint32_t subdiv) {
  const double p = (1.0 + std::sqrt(5.0)) / 2.0;
  const double base[12][3] = {{-1, p, 0}, {1, p, 0}, {-1, -p, 0}, {1, -p, 0}, {0, -1, p}, {0, 1, p},
                              {0, -1, -p}, {0, 1, -p}, {p, 0, -1}, {p, 0, 1}, {-p, 0, -1}, {-p, 0, 1}};
  const int faces[20][3] = {{0, 11, 5}, {0, 5, 1},  {0, 1, 7},   {0, 7, 10}, {0, 10, 11}, {1, 5, 9},  {5, 11, 4},
                            {11, 10, 2}, {10, 7, 6}, {7, 1, 8},   {3, 9, 4},  {3, 4, 2},   {3, 2, 6},  {3, 6, 8},
                            {3, 8, 9},  {4, 9, 5},  {2, 4, 11}, {6, 2, 10}, {8, 6, 7},   {9, 8, 1}};
  auto unit = [](const double* v, double* o) {
    double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    o[0] = v[0] / l; o[1] = v[1] / l; o[2] = v[2] / l;
  };
  std::vector<double> cur(20 * 9);
  for (int f = 0; f < 20; ++f)
    for (int k = 0; k < 3; ++k) unit(base[faces[f][k]], &cur[9 * f + 3 * k]);
  for (uint32_t s = 0; s < subdiv; ++s) {
    std::vector<double> nxt(cur.size() * 4);
    size_t nf = cur.size() / 9;
    for (size_t f = 0; f < nf; ++f) {
      const double* a = &cur[9 * f];
      const double* b = a + 3;
      const double* c = a + 6;
      double ab[3], bc[3], ca[3], t[3];
      for (int k = 0; k < 3; ++k) t[k] = (a[k] + b[k]) * 0.5;
      unit(t, ab);
      for (int k = 0; k < 3; ++k) t[k] = (b[k] + c[k]) * 0.5;
      unit(t, bc);
      for (int k = 0; k < 3; ++k) t[k] = (c[k] + a[k]) * 0.5;
      unit(t, ca);
      const double* out[4][3] = {{a, ab, ca}, {b, bc, ab}, {c, ca, bc}, {ab, bc, ca}};
      for (int q = 0; q < 4; ++q)
        for (int v = 0; v < 3; ++v)
          for (int k = 0; k < 3; ++k) nxt[9 * (4 * f + q) + 3 * v + k] = out[q][v][k];
    }
    cur.swap(nxt);
  }
  return cur;
}

// Seeded 3-D value noise in [0,1): hashed lattice values, trilinear blend with
// smoothstep weights.
double value_noise(uint64_t key, double x, double y, double z) {
  const double fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
  const int64_t ix = (int64_t)fx, iy = (int64_t)fy, iz = (int64_t)fz;
  double tx = x - fx, ty = y - fy, tz = z - fz;
  tx = tx * tx * (3.0 - 2.0 * tx);
  ty = ty * ty * (3.0 - 2.0 * ty);
  tz = tz * tz * (3.0 - 2.0 * tz);
  auto lat = [&](int64_t i, int64_t j, int64_t k) {
    uint64_t h = ((uint64_t)(i & 0x1FFFFF)) | ((uint64_t)(j & 0x1FFFFF) << 21) | ((uint64_t)(k & 0x1FFFFF) << 42);
    return (double)(splitmix64(key ^ splitmix64(h)) >> 11) * 0x1p-53;
  };
  double c[2][2][2];
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b)
      for (int d = 0; d < 2; ++d) c[a][b][d] = lat(ix + a, iy + b, iz + d);
  double x00 = c[0][0][0] + (c[1][0][0] - c[0][0][0]) * tx;
  double x10 = c[0][1][0] + (c[1][1][0] - c[0][1][0]) * tx;
  double x01 = c[0][0][1] + (c[1][0][1] - c[0][0][1]) * tx;
  double x11 = c[0][1][1] + (c[1][1][1] - c[0][1][1]) * tx;
  double y0 = x00 + (x10 - x00) * ty;
  double y1 = x01 + (x11 - x01) * ty;
  return y0 + (y1 - y0) * tz;
}

}  // namespace

extern "C" {

rt_status rt_gen_uniform(uint64_t seed, uint64_t stream, uint64_t n, double* out) {
  if (!out && n) return RT_EINVAL;
  const uint64_t key = stream_key(seed, stream);
  for (uint64_t i = 0; i < n; ++i) out[i] = u01(key, i);
  return RT_OK;
}

rt_status rt_gen_icosphere(uint32_t subdiv, const float center[3], float radius, uint32_t material,
                           RtTriangle64* out, uint64_t capacity, uint64_t* count) {
  if (subdiv > 9 || !center) {
    rtgb::set_error("rt_gen_icosphere: subdiv must be <= 9 and center non-null");
    return RT_EINVAL;
  }
  const uint64_t nf = 20ull << (2 * subdiv);
  if (count) *count = nf;
  if (!out) return RT_OK;
  if (capacity < nf) {
    rtgb::set_error("rt_gen_icosphere: capacity too small");
    return RT_EINVAL;
  }
  std::vector<double> u = icosphere_unit(subdiv);
  for (uint64_t f = 0; f < nf; ++f) {
    double v[3][3];
    for (int a = 0; a < 3; ++a)
      for (int k = 0; k < 3; ++k) v[a][k] = (double)center[k] + (double)radius * u[9 * f + 3 * a + k];
    set_tri(out[f], v[0], v[1], v[2], material);
  }
  return RT_OK;
}

rt_status rt_gen_camera_rays(const RtRaytraceUBO* ubo, uint32_t width, uint32_t height, RtRay* out) {
  if (!ubo || !out || width == 0 || height == 0) {
    rtgb::set_error("rt_gen_camera_rays: bad argument");
    return RT_EINVAL;
  }
  float cam[12];
  rtgb::camera_setup(*ubo, width, height, cam);
  parallel_for((size_t)width * height, [&](size_t b, size_t e, unsigned) {
    for (size_t i = b; i < e; ++i) {
      const float fx = (float)(uint32_t)(i % width), fy = (float)(uint32_t)(i / width);
      float s[3], d[3];
      for (int k = 0; k < 3; ++k) s[k] = (cam[3 + k] + cam[6 + k] * fx) + cam[9 + k] * fy;
      for (int k = 0; k < 3; ++k) d[k] = s[k] - cam[k];
      for (int pass = 0; pass < 2; ++pass) {  // getRay normalises, rayColor again
        float l = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        d[0] = d[0] / l; d[1] = d[1] / l; d[2] = d[2] / l;
      }
      RtRay& r = out[i];
      r.org[0] = cam[0]; r.org[1] = cam[1]; r.org[2] = cam[2];
      r.dir[0] = d[0]; r.dir[1] = d[1]; r.dir[2] = d[2];
      r.tmin = 0.001f;
      r.tmax = 10000000.0f;
    }
  });
  return RT_OK;
}

rt_status rt_gen_config1(RtTriangle64* tris, RtRaytraceUBO* ubo, RtRay* rays) {
  RtRaytraceUBO u;
  std::memset(&u, 0, sizeof(u));
  u.camPos[0] = 0.0f; u.camPos[1] = 0.5f; u.camPos[2] = 4.0f;
  u.camUpDir[1] = 1.0f;
  u.verticalFOV = 60.0f;
  u.numTriangles = 20482;
  u.numSpheres = 0;
  u.numMaterials = 2;
  u.maxRayTraceDepth = 8;
  u.randomState = 0;
  if (ubo) *ubo = u;
  if (tris) {
    const float c[3] = {0.0f, 0.0f, 0.0f};
    rt_status st = rt_gen_icosphere(5, c, 1.0f, 0u, tris, 20480, nullptr);
    if (st != RT_OK) return st;
    const double q[4][3] = {{-10, -1, -10}, {10, -1, -10}, {10, -1, 10}, {-10, -1, 10}};
    set_tri(tris[20480], q[0], q[1], q[2], 1u);
    set_tri(tris[20481], q[0], q[2], q[3], 1u);
  }
  if (rays) return rt_gen_camera_rays(&u, 640, 360, rays);
  return RT_OK;
}

rt_status rt_gen_soup(uint64_t seed, uint64_t stream, uint32_t n, float side, float sigma, uint32_t material,
                      RtTriangle64* out) {
  if (!out && n) return RT_EINVAL;
  const uint64_t kc = stream_key(seed, 4 * stream + 0), kv = stream_key(seed, 4 * stream + 1);
  parallel_for(n, [&](size_t b, size_t e, unsigned) {
    for (size_t i = b; i < e; ++i) {
      double c[3], v[3][3];
      for (int k = 0; k < 3; ++k) c[k] = u01(kc, 3 * i + k) * (double)side;
      for (int m = 0; m < 3; ++m)
        for (int k = 0; k < 3; ++k) v[m][k] = c[k] + (double)sigma * gauss(kv, 9 * i + 3 * m + k);
      set_tri(out[i], v[0], v[1], v[2], material);
    }
  });
  return RT_OK;
}

rt_status rt_gen_rays(uint64_t seed, uint64_t stream, uint32_t n, float side, float tmin, float tmax, RtRay* out) {
  if (!out && n) return RT_EINVAL;
  const uint64_t ko = stream_key(seed, 4 * stream + 2), kd = stream_key(seed, 4 * stream + 3);
  parallel_for(n, [&](size_t b, size_t e, unsigned) {
    for (size_t i = b; i < e; ++i) {
      RtRay& r = out[i];
      double g[3];
      for (int k = 0; k < 3; ++k) {
        r.org[k] = (float)(u01(ko, 3 * i + k) * (double)side);
        g[k] = gauss(kd, 3 * i + k);
      }
      double l = std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
      if (l == 0.0) {
        g[0] = 1.0;
        l = 1.0;
      }
      for (int k = 0; k < 3; ++k) r.dir[k] = (float)(g[k] / l);
      r.tmin = tmin;
      r.tmax = tmax;
    }
  });
  return RT_OK;
}

rt_status rt_gen_spheres_scene(uint64_t seed, uint32_t count, uint32_t subdiv, float amp, RtTriangle64* tris,
                               RtMaterial32* mats) {
  if (subdiv > 8 || (!tris && count)) {
    rtgb::set_error("rt_gen_spheres_scene: bad argument");
    return RT_EINVAL;
  }
  const uint64_t per = 20ull << (2 * subdiv);
  std::vector<double> u = icosphere_unit(subdiv);
  const uint64_t ks = stream_key(seed, 1000);
  for (uint32_t s = 0; s < count; ++s) {
    double c[3];
    for (int k = 0; k < 3; ++k) c[k] = -8.0 + 16.0 * u01(ks, 16ull * s + k);
    const double r = 0.3 + 1.2 * u01(ks, 16ull * s + 3);
    const double which = u01(ks, 16ull * s + 4);
    const uint64_t knoise = stream_key(seed, 2000 + s);
    parallel_for(per, [&](size_t b, size_t e, unsigned) {
      for (size_t f = b; f < e; ++f) {
        double v[3][3];
        for (int a = 0; a < 3; ++a) {
          const double* un = &u[9 * f + 3 * a];
          const double nz = value_noise(knoise, 4.0 * un[0], 4.0 * un[1], 4.0 * un[2]);
          const double rr = r + (double)amp * (2.0 * nz - 1.0);
          for (int k = 0; k < 3; ++k) v[a][k] = c[k] + rr * un[k];
        }
        set_tri(tris[(uint64_t)s * per + f], v[0], v[1], v[2], s);
      }
    });
    if (mats) {
      RtMaterial32& m = mats[s];
      std::memset(&m, 0, sizeof(m));
      if (which < 1.0 / 3.0) {
        m.materialType = RT_MAT_DIFFUSE;
        for (int k = 0; k < 3; ++k) m.albedo[k] = (float)(0.1 + 0.8 * u01(ks, 16ull * s + 5 + k));
      } else if (which < 2.0 / 3.0) {
        m.materialType = RT_MAT_METALLIC;
        for (int k = 0; k < 3; ++k) m.albedo[k] = (float)(0.5 + 0.5 * u01(ks, 16ull * s + 5 + k));
        m.fuzz = (float)(0.3 * u01(ks, 16ull * s + 8));
      } else {
        m.materialType = RT_MAT_DIELECTRIC;
        m.albedo[0] = m.albedo[1] = m.albedo[2] = 1.0f;
        m.ior = 1.5f;
      }
    }
  }
  return RT_OK;
}

}  // extern "C"
