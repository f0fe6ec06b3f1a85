// Exercises the C++ host interface (include/rt_gb300.hpp) the way the
// reference's Raytracer uses RaytraceScene: game objects with transforms and
// models, flattening, prepForRender, one frame of the raytrace pass.
//   host_api_test cpu            flatten only; prints counts and a checksum
//   host_api_test gpu <out.bin>  renders a frame; writes the accumulator
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "rt_gb300.hpp"
#include "rt_gb300_workloads.h"

static rtgb::RaytraceScene* make_scene() {
  auto* scene = new rtgb::RaytraceScene();
  uint64_t n = 0;
  const float c[3] = {0.0f, 0.0f, 0.0f};
  rtgb::check(rt_gen_icosphere(2, c, 1.0f, 0, nullptr, 0, &n), "icosphere");
  std::vector<RtTriangle64> ico(n);
  rtgb::check(rt_gen_icosphere(2, c, 1.0f, 0, ico.data(), n, &n), "icosphere");
  rtgb::GameObject a;
  a.model = rtgb::RTModel::Triangles(ico, rtgb::make_material(0.73f, 0.33f, 0.25f, RT_MAT_DIFFUSE));
  a.transform.translation[1] = 0.1f;
  a.transform.rotation[1] = 0.4f;
  scene->addGameObject(std::move(a));

  std::vector<RtTriangle64> quad(2);
  std::memset(quad.data(), 0, sizeof(RtTriangle64) * 2);
  const float q[4][3] = {{-1, 0, -1}, {1, 0, -1}, {1, 0, 1}, {-1, 0, 1}};
  const int tri[2][3] = {{0, 1, 2}, {0, 2, 3}};
  for (int t = 0; t < 2; ++t)
    for (int k = 0; k < 3; ++k) {
      float* dst = k == 0 ? quad[t].v0 : (k == 1 ? quad[t].v1 : quad[t].v2);
      std::memcpy(dst, q[tri[t][k]], 12);
    }
  rtgb::GameObject ground;
  ground.model = rtgb::RTModel::Triangles(quad, rtgb::make_material(3.0f, 3.0f, 3.0f, RT_MAT_LIGHT));
  ground.transform.translation[1] = -1.0f;
  ground.transform.scale[0] = ground.transform.scale[2] = 10.0f;
  scene->addGameObject(std::move(ground));

  rtgb::GameObject ball;
  ball.model = rtgb::RTModel::Sphere(0.5f, rtgb::make_material(0.2f, 0.6f, 0.3f, RT_MAT_DIFFUSE));
  ball.transform.translation[0] = 1.5f;
  ball.transform.translation[2] = 0.5f;
  scene->addGameObject(std::move(ball));
  scene->setMaxRaytraceDepth(4);
  scene->setRaysPerPixel(3);
  return scene;
}

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  rtgb::RaytraceScene* scene = make_scene();
  if (std::strcmp(argv[1], "cpu") == 0) {
    scene->moveGameObjectsToHostVectors();
    double sum = 0.0;
    for (const RtTriangle64& t : scene->triangles()) sum += t.v0[0] + 2.0 * t.v1[1] + 3.0 * t.v2[2] + t.modelIndex;
    std::printf("models %u triangles %u spheres %u materials %u checksum %.6f\n", scene->getModelCount(),
                scene->getTriangleCount(), scene->getSphereCount(), scene->getMaterialCount(), sum);
    bool threw = false;
    try {
      scene->handle();
    } catch (const std::runtime_error&) {
      threw = true;
    }
    std::printf("handle-before-prep-throws %d\n", threw ? 1 : 0);
    delete scene;
    return 0;
  }
  if (std::strcmp(argv[1], "gpu") == 0 && argc >= 3) {
    const uint32_t w = 64, h = 36;
    rtgb::RaytracePass pass(w, h);
    const float pos[3] = {0.0f, 0.5f, 4.0f}, look[3] = {0.0f, 0.0f, 0.0f}, up[3] = {0.0f, 1.0f, 0.0f};
    pass.doIteration(*scene, pos, look, up, 60.0f, 77u);
    std::vector<float> acc = pass.accumulator();
    FILE* f = std::fopen(argv[2], "wb");
    if (!f) return 3;
    std::fwrite(acc.data(), sizeof(float), acc.size(), f);
    std::fclose(f);
    pass.writeImage(std::string(argv[2]) + ".ppm");
    std::printf("rendered %u x %u, %u samples\n", w, h, scene->getRaysPerPixel());
    delete scene;
    return 0;
  }
  return 2;
}
