// rt_gb300.hpp -- C++ host interface over the C ABI, shaped like the
// reference's own host classes for this path, so that its callers keep their
// structure:
//
//   rtgb::TransformComponent  TransformComponent (components/TransformComponent.cpp:9-45)
//   rtgb::RTModel             RTModel_Triangles / RTModel_Sphere, loadModel (RTModel.cpp:47-112)
//   rtgb::GameObject          GameObject: transform + model
//   rtgb::RaytraceScene       RaytraceScene (RaytraceScene.hpp:64-102): addGameObject,
//                             prepForRender, updateScene, get*Count,
//                             set/getMaxRaytraceDepth, set/getRaysPerPixel
//   rtgb::RaytracePass        the S2 pass of RaytracerBVH (RaytracerBVH.cpp:998-1078):
//                             the RGBA32F accumulator, its clear (:772-776), spp
//                             samples per frame, and the present pass's resolve
//
// Errors throw std::runtime_error with rt_last_error_string(), as the
// reference throws on a failed VkResult (RaytracerBVH.hpp:399-404).
// Header-only; link librt_gb300.so.  No CUDA headers needed.
#pragma once

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "rt_gb300.h"

namespace rtgb {

inline void check(rt_status s, const char* where) {
  if (s != RT_OK) throw std::runtime_error(std::string(where) + ": " + rt_last_error_string());
}

struct TransformComponent {
  float translation[3] = {0.0f, 0.0f, 0.0f};
  float rotation[3] = {0.0f, 0.0f, 0.0f};  // radians, Tait-Bryan Y-X-Z
  float scale[3] = {1.0f, 1.0f, 1.0f};
  RtModel64 mat4() const {
    RtModel64 m;
    check(rt_model_matrix(translation, rotation, scale, &m), "TransformComponent::mat4");
    return m;
  }
};

// Model-space geometry with one material: a triangle list or a sphere of the
// given radius at the origin.
struct RTModel {
  std::vector<RtTriangle64> triangles;
  bool is_sphere = false;
  float radius = 0.0f;
  RtMaterial32 material{};

  static RTModel Triangles(std::vector<RtTriangle64> tris, const RtMaterial32& mat) {
    RTModel m;
    m.triangles = std::move(tris);
    m.material = mat;
    return m;
  }
  static RTModel Sphere(float radius, const RtMaterial32& mat) {
    RTModel m;
    m.is_sphere = true;
    m.radius = radius;
    m.material = mat;
    return m;
  }
  // loadModel(filepath, material)
  static RTModel FromObj(const std::string& path, const RtMaterial32& mat) {
    uint64_t n = 0;
    check(rt_obj_load(path.c_str(), 0, nullptr, 0, &n), "loadModel");
    std::vector<RtTriangle64> tris(n);
    check(rt_obj_load(path.c_str(), 0, tris.data(), n, &n), "loadModel");
    return Triangles(std::move(tris), mat);
  }
};

inline RtMaterial32 make_material(float r, float g, float b, uint32_t type, float fuzz = 0.0f, float ior = 1.5f) {
  RtMaterial32 m{};
  m.albedo[0] = r;
  m.albedo[1] = g;
  m.albedo[2] = b;
  m.materialType = type;
  m.fuzz = fuzz;
  m.ior = ior;
  return m;
}

struct GameObject {
  TransformComponent transform;
  RTModel model;
};

class RaytraceScene {
 public:
  RaytraceScene() = default;
  RaytraceScene(const RaytraceScene&) = delete;
  RaytraceScene& operator=(const RaytraceScene&) = delete;
  ~RaytraceScene() { release(); }

  void addGameObject(GameObject&& go) {
    objects_.push_back(std::move(go));
    dirty_ = true;
  }
  bool removeGameObject(size_t index) {
    if (index >= objects_.size()) return false;
    objects_.erase(objects_.begin() + (std::ptrdiff_t)index);
    dirty_ = true;
    return true;
  }
  size_t gameObjectCount() const { return objects_.size(); }

  void setMaxRaytraceDepth(uint32_t d) { depth_ = d; }
  void setRaysPerPixel(uint32_t s) { spp_ = s; }
  uint32_t getMaxRaytraceDepth() const { return depth_; }
  uint32_t getRaysPerPixel() const { return spp_; }
  void setBvhMode(uint32_t mode) { bvh_mode_ = mode; dirty_ = true; }

  // moveGameObjectsToHostVectors (RaytraceScene.cpp:157-200): one model
  // matrix per game object in order; each object appends its material and
  // its triangles (or its sphere) with that material and model index.
  void moveGameObjectsToHostVectors() {
    models_.clear();
    triangles_.clear();
    spheres_.clear();
    materials_.clear();
    for (size_t i = 0; i < objects_.size(); ++i) {
      const GameObject& go = objects_[i];
      const uint32_t model_index = (uint32_t)models_.size();
      models_.push_back(go.transform.mat4());
      const uint32_t material_index = (uint32_t)materials_.size();
      materials_.push_back(go.model.material);
      if (go.model.is_sphere) {
        RtSphere32 s{};
        s.radius = go.model.radius;
        s.materialIndex = material_index;
        s.modelIndex = model_index;
        spheres_.push_back(s);
      } else {
        for (RtTriangle64 t : go.model.triangles) {
          t.materialIndex = material_index;
          t.modelIndex = model_index;
          triangles_.push_back(t);
        }
      }
    }
  }

  // Flattens, applies the model matrices, builds the BVH and uploads.
  void prepForRender() {
    moveGameObjectsToHostVectors();
    release();
    RtSceneDesc d{};
    d.triangles = triangles_.data();
    d.num_triangles = (uint32_t)triangles_.size();
    d.spheres = spheres_.data();
    d.num_spheres = (uint32_t)spheres_.size();
    d.materials = materials_.data();
    d.num_materials = (uint32_t)materials_.size();
    d.models = models_.data();
    d.num_models = (uint32_t)models_.size();
    d.bvh_mode = bvh_mode_;
    check(rt_scene_create_ex(&d, &scene_), "RaytraceScene::prepForRender");
    dirty_ = false;
  }
  // The reference re-uploads every frame (RaytraceScene.cpp:78-113); here the
  // device scene is rebuilt only when game objects changed.
  void updateScene() {
    if (dirty_ || !scene_) prepForRender();
  }

  uint32_t getModelCount() const { return (uint32_t)models_.size(); }
  uint32_t getTriangleCount() const { return (uint32_t)triangles_.size(); }
  uint32_t getSphereCount() const { return (uint32_t)spheres_.size(); }
  uint32_t getMaterialCount() const { return (uint32_t)materials_.size(); }
  const std::vector<RtTriangle64>& triangles() const { return triangles_; }
  const std::vector<RtSphere32>& spheres() const { return spheres_; }
  const std::vector<RtMaterial32>& materials() const { return materials_; }
  const std::vector<RtModel64>& models() const { return models_; }
  rt_scene* handle() {
    if (!scene_) throw std::runtime_error("RaytraceScene: prepForRender has not run");
    return scene_;
  }

 private:
  void release() {
    if (scene_) rt_scene_destroy(scene_);
    scene_ = nullptr;
  }
  std::vector<GameObject> objects_;
  std::vector<RtModel64> models_;
  std::vector<RtTriangle64> triangles_;
  std::vector<RtSphere32> spheres_;
  std::vector<RtMaterial32> materials_;
  rt_scene* scene_ = nullptr;
  uint32_t depth_ = 8, spp_ = 1, bvh_mode_ = RT_BVH_SORTED;
  bool dirty_ = true;
};

// The raytrace pass over an accumulator of width x height pixels.
class RaytracePass {
 public:
  RaytracePass(uint32_t width, uint32_t height) : w_(width), h_(height) {
    check(rt_device_alloc((size_t)width * height * 16, reinterpret_cast<void**>(&accum_)), "RaytracePass");
    check(rt_device_alloc((size_t)width * height * 16, reinterpret_cast<void**>(&resolved_)), "RaytracePass");
  }
  RaytracePass(const RaytracePass&) = delete;
  RaytracePass& operator=(const RaytracePass&) = delete;
  ~RaytracePass() {
    rt_device_free(accum_);
    rt_device_free(resolved_);
  }

  // One frame: clear, then getRaysPerPixel() samples of every pixel with the
  // given camera and random state (the UBO of RaytracerBVH.hpp:340-352).
  void doIteration(RaytraceScene& scene, const float cam_pos[3], const float look_at[3], const float up[3],
                   float vertical_fov, uint32_t random_state, const RtRenderOptions* opt = nullptr) {
    scene.updateScene();
    RtRaytraceUBO ubo{};
    for (int k = 0; k < 3; ++k) {
      ubo.camPos[k] = cam_pos[k];
      ubo.camLookAt[k] = look_at[k];
      ubo.camUpDir[k] = up[k];
    }
    ubo.verticalFOV = vertical_fov;
    ubo.numTriangles = scene.getTriangleCount();
    ubo.numSpheres = scene.getSphereCount();
    ubo.numMaterials = scene.getMaterialCount();
    ubo.maxRayTraceDepth = scene.getMaxRaytraceDepth();
    ubo.randomState = random_state;
    check(rt_accum_clear(accum_, w_, h_, nullptr), "RaytracePass::clear");
    check(rt_render(scene.handle(), &ubo, accum_, w_, h_, scene.getRaysPerPixel(), opt, nullptr), "RaytracePass::render");
    spp_ = scene.getRaysPerPixel();
  }

  // The accumulator (RGB sums, alpha = RNG carry) on the host.
  std::vector<float> accumulator() const {
    std::vector<float> out((size_t)w_ * h_ * 4);
    check(rt_copy(out.data(), accum_, out.size() * 4, nullptr), "RaytracePass::accumulator");
    check(rt_stream_wait(nullptr, 60.0), "RaytracePass::accumulator");
    return out;
  }
  // clamp(sqrt(sum / spp), 0, 1), the present pass's colour.
  std::vector<float> resolve() const {
    check(rt_resolve(accum_, w_, h_, spp_ ? spp_ : 1, resolved_, nullptr), "RaytracePass::resolve");
    std::vector<float> out((size_t)w_ * h_ * 4);
    check(rt_copy(out.data(), resolved_, out.size() * 4, nullptr), "RaytracePass::resolve");
    check(rt_stream_wait(nullptr, 60.0), "RaytracePass::resolve");
    return out;
  }
  void writeImage(const std::string& path) const {
    const std::vector<float> img = resolve();
    const bool pfm = path.size() > 4 && path.compare(path.size() - 4, 4, ".pfm") == 0;
    check(pfm ? rt_write_pfm(path.c_str(), img.data(), w_, h_) : rt_write_ppm(path.c_str(), img.data(), w_, h_),
          "RaytracePass::writeImage");
  }

 private:
  uint32_t w_, h_, spp_ = 1;
  float* accum_ = nullptr;
  float* resolved_ = nullptr;
};

}  // namespace rtgb
