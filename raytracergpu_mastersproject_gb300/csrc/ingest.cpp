// ingest.cpp -- scene ingestion and image output on the host.
//
//   rt_obj_load      Wavefront OBJ -> triangle records.  The reference loads
//                    models with tinyobjloader (RTModel.cpp:47-108): vertex
//                    positions of each face, faces triangulated as a fan from
//                    their first vertex, shapes in file order.  This reader
//                    does the same for the `v` and `f` statements (index forms
//                    i, i/j, i/j/k, i//k, negative = relative); other
//                    statements are ignored.
//   rt_model_matrix  TransformComponent::mat4 (TransformComponent.cpp:9-45):
//                    translate * Ry * Rx * Rz * scale, column-major.
//   rt_write_ppm / rt_write_pfm   the resolved frame to a file, in place of
//                    the swapchain present (SingleTriangleFullScreen.frag).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "rt_internal.h"

namespace rtgb {
void set_error(const std::string& msg);
}

namespace {

bool parse_index(const char* tok, long nverts, long* out) {
  char* end = nullptr;
  const long v = std::strtol(tok, &end, 10);
  if (end == tok || v == 0) return false;
  const long idx = v > 0 ? v - 1 : nverts + v;
  if (idx < 0 || idx >= nverts) return false;
  *out = idx;
  return true;
}

}  // namespace

extern "C" {

rt_status rt_obj_load(const char* path, uint32_t material, RtTriangle64* out, uint64_t capacity, uint64_t* count) {
  if (!path || !count) {
    rtgb::set_error("rt_obj_load: null argument");
    return RT_EINVAL;
  }
  FILE* f = std::fopen(path, "rb");
  if (!f) {
    rtgb::set_error(std::string("rt_obj_load: cannot open ") + path);
    return RT_ENOTFOUND;
  }
  std::vector<float> v;
  uint64_t n = 0;
  std::vector<long> poly;
  char line[4096];
  long lineno = 0;
  rt_status st = RT_OK;
  while (std::fgets(line, sizeof(line), f)) {
    ++lineno;
    char* p = line;
    while (*p == ' ' || *p == '\t') ++p;
    if (p[0] == 'v' && (p[1] == ' ' || p[1] == '\t')) {
      float xyz[3] = {0, 0, 0};
      char* q = p + 2;
      for (int k = 0; k < 3; ++k) {
        char* e = nullptr;
        xyz[k] = std::strtof(q, &e);
        if (e == q) {
          st = RT_EINVAL;
          break;
        }
        q = e;
      }
      if (st != RT_OK) {
        rtgb::set_error("rt_obj_load: bad vertex at line " + std::to_string(lineno));
        break;
      }
      v.insert(v.end(), xyz, xyz + 3);
    } else if (p[0] == 'f' && (p[1] == ' ' || p[1] == '\t')) {
      poly.clear();
      const long nverts = (long)(v.size() / 3);
      char* save = nullptr;
      for (char* tok = strtok_r(p + 2, " \t\r\n", &save); tok; tok = strtok_r(nullptr, " \t\r\n", &save)) {
        long idx;
        if (!parse_index(tok, nverts, &idx)) {
          st = RT_EINVAL;
          break;
        }
        poly.push_back(idx);
      }
      if (st != RT_OK || poly.size() < 3) {
        rtgb::set_error("rt_obj_load: bad face at line " + std::to_string(lineno));
        st = RT_EINVAL;
        break;
      }
      for (size_t k = 1; k + 1 < poly.size(); ++k) {
        if (out && n < capacity) {
          RtTriangle64& t = out[n];
          std::memset(&t, 0, sizeof(t));
          const long ids[3] = {poly[0], poly[k], poly[k + 1]};
          float* dst[3] = {t.v0, t.v1, t.v2};
          for (int a = 0; a < 3; ++a)
            for (int c = 0; c < 3; ++c) dst[a][c] = v[3 * (size_t)ids[a] + c];
          t.materialIndex = material;
        }
        ++n;
      }
    }
  }
  std::fclose(f);
  if (st != RT_OK) return st;
  *count = n;
  if (out && n > capacity) {
    rtgb::set_error("rt_obj_load: capacity below the triangle count");
    return RT_EINVAL;
  }
  return RT_OK;
}

rt_status rt_model_matrix(const float translation[3], const float rotation[3], const float scale[3],
                          RtModel64* out) {
  if (!translation || !rotation || !scale || !out) return RT_EINVAL;
  const float c3 = std::cos(rotation[2]), s3 = std::sin(rotation[2]);
  const float c2 = std::cos(rotation[0]), s2 = std::sin(rotation[0]);
  const float c1 = std::cos(rotation[1]), s1 = std::sin(rotation[1]);
  const float m[16] = {scale[0] * (c1 * c3 + s1 * s2 * s3), scale[0] * (c2 * s3), scale[0] * (c1 * s2 * s3 - c3 * s1),
                       0.0f,
                       scale[1] * (c3 * s1 * s2 - c1 * s3), scale[1] * (c2 * c3), scale[1] * (c1 * c3 * s2 + s1 * s3),
                       0.0f,
                       scale[2] * (c2 * s1), scale[2] * (-s2), scale[2] * (c1 * c2), 0.0f,
                       translation[0], translation[1], translation[2], 1.0f};
  std::memcpy(out->m, m, sizeof(m));
  return RT_OK;
}

// Binary PPM (P6), rows top to bottom; rgba in [0,1] (e.g. rt_resolve output).
rt_status rt_write_ppm(const char* path, const float* rgba, uint32_t width, uint32_t height) {
  if (!path || !rgba || !width || !height) return RT_EINVAL;
  FILE* f = std::fopen(path, "wb");
  if (!f) {
    rtgb::set_error(std::string("rt_write_ppm: cannot open ") + path);
    return RT_EINVAL;
  }
  std::fprintf(f, "P6\n%u %u\n255\n", width, height);
  std::vector<unsigned char> row(3 * (size_t)width);
  for (uint32_t y = 0; y < height; ++y) {
    for (uint32_t x = 0; x < width; ++x)
      for (int c = 0; c < 3; ++c) {
        float v = rgba[4 * ((size_t)y * width + x) + c];
        v = v != v ? 0.0f : std::fmin(std::fmax(v, 0.0f), 1.0f);
        row[3 * (size_t)x + c] = (unsigned char)std::lround(v * 255.0f);
      }
    std::fwrite(row.data(), 1, row.size(), f);
  }
  std::fclose(f);
  return RT_OK;
}

// Little-endian PFM (PF, scale -1), rows bottom to top as the format requires.
rt_status rt_write_pfm(const char* path, const float* rgba, uint32_t width, uint32_t height) {
  if (!path || !rgba || !width || !height) return RT_EINVAL;
  FILE* f = std::fopen(path, "wb");
  if (!f) {
    rtgb::set_error(std::string("rt_write_pfm: cannot open ") + path);
    return RT_EINVAL;
  }
  std::fprintf(f, "PF\n%u %u\n-1.0\n", width, height);
  std::vector<float> row(3 * (size_t)width);
  for (uint32_t yy = 0; yy < height; ++yy) {
    const uint32_t y = height - 1 - yy;
    for (uint32_t x = 0; x < width; ++x)
      for (int c = 0; c < 3; ++c) row[3 * (size_t)x + c] = rgba[4 * ((size_t)y * width + x) + c];
    std::fwrite(row.data(), sizeof(float), row.size(), f);
  }
  std::fclose(f);
  return RT_OK;
}

}  // extern "C"
