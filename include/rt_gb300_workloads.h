/*
 * rt_gb300_workloads.h -- seeded synthetic scenes and ray batches.
 *
 * No counterpart in the reference: its scenes load .obj files that are not in
 * the repository (Scenes.cpp:105-122, 342-345).  These generators stand in for
 * them with the shapes and sizes of the benchmark configurations:
 *   config 1  icosphere subdiv 5 (20,480 tris, r=1) + 2-triangle ground quad at
 *             y=-1, camera (0,0.5,4)->(0,0,0), vFOV 60, 640x360, 1 ray/pixel
 *   config 2  64 displaced icospheres subdiv 6 (5,242,880 tris), mixed materials
 *   config 3  4,194,304-triangle soup in the unit cube (vertex offsets
 *             N(0, 0.002^2)), 16,777,216 rays (origins in the cube, directions
 *             uniform on the sphere, tmin 1e-4, tmax +inf)
 *   configs 4/5  soups of other sizes in cubes scaled to keep config 3's density
 *
 * Every value is a pure function of (seed, stream, index): splitmix64 of a
 * counter, uniform doubles from its top 53 bits, normals by Box-Muller in
 * binary64, rounded to binary32 at the end.  Outputs are identical for any
 * thread count.
 */
#ifndef RT_GB300_WORKLOADS_H
#define RT_GB300_WORKLOADS_H

#include "rt_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* n uniform doubles in [0,1) of stream (seed, stream). */
rt_status rt_gen_uniform(uint64_t seed, uint64_t stream, uint64_t n, double* out);

/* Icosphere: icosahedron split subdiv times, vertices on the sphere.
 * Writes 20*4^subdiv triangles (capacity checked). */
rt_status rt_gen_icosphere(uint32_t subdiv, const float center[3], float radius, uint32_t material,
                           RtTriangle64* out, uint64_t capacity, uint64_t* count);

/* Config 1: triangles (20,482: sphere with material 0, ground quad with
 * material 1), the UBO (camera, depth 1, randomState 0) and 640x360 primary
 * rays.  Any output pointer may be NULL. */
rt_status rt_gen_config1(RtTriangle64* tris, RtRaytraceUBO* ubo, RtRay* rays);

/* Primary rays of the reference camera (raytraceBVH.comp:50-81, 329-342;
 * rayColor's normalisation :280): origin camPos, interval [0.001, 1e7]. */
rt_status rt_gen_camera_rays(const RtRaytraceUBO* ubo, uint32_t width, uint32_t height, RtRay* out);

/* Triangle soup: n triangles, centroids uniform in [0,side]^3, each vertex =
 * centroid + N(0, sigma^2) per axis.  Stream ids: seed, stream. */
rt_status rt_gen_soup(uint64_t seed, uint64_t stream, uint32_t n, float side, float sigma, uint32_t material,
                      RtTriangle64* out);

/* Rays: origins uniform in [0,side]^3, directions uniform on the unit sphere. */
rt_status rt_gen_rays(uint64_t seed, uint64_t stream, uint32_t n, float side, float tmin, float tmax, RtRay* out);

/* Config 2 geometry: count icospheres of the given subdiv, centres uniform
 * in [-8,8]^3, radii U(0.3,1.5), vertices displaced radially by seeded value
 * noise of amplitude amp; one material per sphere (lambertian albedo
 * U(0.1,0.9)^3, metal albedo U(0.5,1)^3 fuzz U(0,0.3), dielectric ior 1.5,
 * each with probability 1/3).  tris holds count*20*4^subdiv records, mats
 * holds count records. */
rt_status rt_gen_spheres_scene(uint64_t seed, uint32_t count, uint32_t subdiv, float amp, RtTriangle64* tris,
                               RtMaterial32* mats);

#ifdef __cplusplus
}
#endif

#endif /* RT_GB300_WORKLOADS_H */
