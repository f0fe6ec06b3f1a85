/*
 * rt_gb300.h -- C ABI of the GB300 (sm_103a) ray-tracing hot path.
 *
 * This header is the drop-in boundary for the raytrace compute pass of
 * RaytracerGPU_MastersProject (Vulkan).  In the reference, C++ host code fills a
 * descriptor set (RaytracerBVH.cpp:202-238, 677-685):
 *
 *   b0 ParameterUBO       camera, counts, depth, randomState   (raytraceBVH.comp:7-18)
 *   b1 storage image      RGBA32F accumulator, RNG carry in a   (raytraceBVH.comp:22, 349-374)
 *   b2 Triangle SSBO      64-byte records                      (definitions.glsl:15-21)
 *   b3 Sphere SSBO        32-byte records                      (definitions.glsl:23-28)
 *   b4 Material SSBO      32-byte records                      (definitions.glsl:10-13)
 *   b5 HLBVHNode SSBO     40-byte nodes, 2N-1 of them           (definitions.glsl:66-72)
 *
 * and records vkCmdDispatch((W/32)+1, (H/32)+1, 1) once per ray per pixel
 * (RaytracerBVH.cpp:1025-1050).  Here the same buffers are handed to
 * rt_scene_create / rt_render, and the dispatch becomes one stream-ordered call.
 * The BVH is built on the host in the reference node layout when no node
 * buffer is supplied.
 *
 * Conventions
 *   - Every entry point returns rt_status; nothing throws across the ABI.
 *     rt_last_error_string() describes the last failure of the calling thread.
 *   - "stream" is a cudaStream_t passed as void* (NULL = legacy default stream).
 *   - Pointers named d_* are device pointers; h_* are host pointers.
 *   - Scenes are immutable after creation; tracing one scene from several
 *     streams at once is safe.
 */
#ifndef RT_GB300_H
#define RT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RT_ABI_VERSION 1u

/* ---------------------------------------------------------------- status */
typedef enum rt_status {
  RT_OK = 0,
  RT_EINVAL = 1,      /* bad argument (null pointer, size, index out of range) */
  RT_ENOMEM = 2,      /* device or host allocation failed / over budget       */
  RT_ETIMEOUT = 3,    /* bounded host wait ran out                            */
  RT_ESTACK = 4,      /* BVH deeper than the traversal stack                  */
  RT_ECUDA = 5,       /* CUDA runtime error                                   */
  RT_EBUSY = 6,       /* admission refused for now (serving)                  */
  RT_ECANCELED = 7,   /* request cancelled                                    */
  RT_ENOTFOUND = 8,   /* unknown scene / request id                           */
  RT_EUNSUPPORTED = 9 /* option not supported by this library                 */
} rt_status;

/* ------------------------------------------------ enums of the reference */
/* Material types: definitions.glsl:79-82, SceneTypes.hpp:14-19. */
enum { RT_MAT_LIGHT = 0, RT_MAT_DIFFUSE = 1, RT_MAT_METALLIC = 2, RT_MAT_DIELECTRIC = 3 };
/* Primitive types: definitions.glsl:84-85. */
enum { RT_PRIM_SPHERE = 0, RT_PRIM_TRIANGLE = 1 };

/* ------------------------------------------------- records (std430 size) */
/* Triangle, 64 B: vec4 v0,v1,v2 (w unused), materialIndex@48, modelIndex@52.
 * definitions.glsl:15-21, SceneTypes.hpp:41-47. */
typedef struct RtTriangle64 {
  float v0[4];
  float v1[4];
  float v2[4];
  uint32_t materialIndex;
  uint32_t modelIndex;
  uint32_t _pad[2];
} RtTriangle64;

/* Sphere, 32 B: vec4 center, radius@16, materialIndex@20, modelIndex@24.
 * definitions.glsl:23-28, SceneTypes.hpp:62-66. */
typedef struct RtSphere32 {
  float center[4];
  float radius;
  uint32_t materialIndex;
  uint32_t modelIndex;
  uint32_t _pad;
} RtSphere32;

/* Material, 32 B: vec4 albedo, materialType@16 (definitions.glsl:10-13,
 * SceneTypes.hpp:82-84).  fuzz@20 and ior@24 sit in the record's std430 tail
 * padding; the reference never reads them.  Only RT_SHADE_EXTENDED uses them. */
typedef struct RtMaterial32 {
  float albedo[4];
  uint32_t materialType;
  float fuzz;
  float ior;
  uint32_t _pad;
} RtMaterial32;

/* Model matrix, 64 B, column-major mat4 (definitions.glsl:6-8, SceneTypes.hpp:32-33). */
typedef struct RtModel64 {
  float m[16];
} RtModel64;

/* BVH node, 40 B (definitions.glsl:52-56,66-72; SceneTypes.hpp:107-123).
 * Leaf <=> left == 0 && right == 0 (raytraceBVH.comp:213).  Node 0 is the root. */
typedef struct RtBVHNode40 {
  float minX, maxX, minY, maxY, minZ, maxZ;
  uint32_t left;
  uint32_t right;
  uint32_t primitiveIndex;
  uint32_t primitiveType;
} RtBVHNode40;

/* ParameterUBO, std140 (raytraceBVH.comp:7-18; RaytracerBVH.hpp:31-42):
 * camPos@0 camLookAt@16 camUpDir@32 verticalFOV@48 numTriangles@52
 * numSpheres@56 numMaterials@60 numLights@64 maxRayTraceDepth@68
 * randomState@72; padded to 80 B like the C++ struct. */
typedef struct RtRaytraceUBO {
  float camPos[4];
  float camLookAt[4];
  float camUpDir[4];
  float verticalFOV;
  uint32_t numTriangles;
  uint32_t numSpheres;
  uint32_t numMaterials;
  uint32_t numLights;
  uint32_t maxRayTraceDepth;
  uint32_t randomState;
  uint32_t _pad;
} RtRaytraceUBO;

/* A ray query, 32 B: origin, tmin, direction, tmax.  Struct Ray of
 * definitions.glsl:35-38 plus the interval that sceneHit fixes at
 * [0.001, 1e7] (raytraceBVH.comp:267-274). */
typedef struct RtRay {
  float org[3];
  float tmin;
  float dir[3];
  float tmax;
} RtRay;

/* A hit, 8 B.  prim = triangle index, or (sphere index | RT_HIT_SPHERE_BIT),
 * or RT_NO_HIT; t = ray parameter of the hit (+inf on a miss). */
typedef struct RtHit {
  uint32_t prim;
  float t;
} RtHit;

#define RT_NO_HIT 0xFFFFFFFFu
#define RT_HIT_SPHERE_BIT 0x80000000u

/* ------------------------------------------------------------------ scene */
typedef struct rt_scene rt_scene;

enum {
  RT_BVH_SORTED = 0,    /* leaf k holds the k-th Morton-sorted primitive (default) */
  RT_BVH_REFERENCE = 1  /* leaf k holds primitive k, as ConstructHLBVH.comp:152-169 */
};

typedef struct RtSceneDesc {
  const RtTriangle64* triangles;  /* host, num_triangles records */
  uint32_t num_triangles;
  const RtSphere32* spheres;      /* host, may be NULL if num_spheres == 0 */
  uint32_t num_spheres;
  const RtMaterial32* materials;  /* host, may be NULL if num_materials == 0 */
  uint32_t num_materials;
  const RtModel64* models;        /* host; NULL = vertices are already in world space */
  uint32_t num_models;
  const RtBVHNode40* nodes;       /* host; NULL = build on the host (bvh_mode) */
  uint32_t num_nodes;             /* 2*(num_triangles+num_spheres)-1 when nodes != NULL */
  uint32_t bvh_mode;              /* RT_BVH_SORTED | RT_BVH_REFERENCE */
  uint32_t leaf_size;             /* max triangles per device leaf after collapsing; 0 = default (1) */
  uint32_t node_width;            /* device BVH width: 2 (binary) or 4 (quantised); 0 = default (4) */
  uint32_t build_flags;           /* RT_BUILD_ON_DEVICE | RT_BUILD_TRAVERSE_S1 */
} RtSceneDesc;

/* Build the node array with rt_build_bvh_device (the S1 passes on the GPU). */
#define RT_BUILD_ON_DEVICE 1u
/* Which tree the device traverses.  The scene always keeps the S1 node array
 * (rt_scene_get_nodes).  When the library builds that array on the host in
 * RT_BVH_SORTED mode, the device by default traverses a binned-SAH tree over
 * the same primitives instead, built on the host: about 10% fewer box tests
 * per ray, and the same hits (closest hits do not depend on the tree).  With
 * this flag, and always for caller-supplied nodes, RT_BVH_REFERENCE or
 * RT_BUILD_ON_DEVICE, it traverses the S1 array itself. */
#define RT_BUILD_TRAVERSE_S1 2u

typedef struct RtSceneInfo {
  uint32_t num_triangles;
  uint32_t num_spheres;
  uint32_t num_materials;
  uint32_t num_nodes;          /* reference-layout node count, 2N-1 */
  uint32_t device_nodes;       /* internal nodes of the device BVH */
  uint32_t depth;              /* longest root-to-leaf path of the device BVH (inner nodes) */
  uint32_t leaf_size;
  uint32_t bvh_mode;
  uint64_t device_bytes;       /* device memory held by the scene */
  double build_seconds;        /* host BVH build + conversion time */
  uint32_t node_width;         /* 2 or 4 */
  uint32_t stack_need;         /* worst-case traversal stack entries */
  uint32_t traversal_sah;      /* 1: the device traverses the SAH tree; 0: the S1 array */
  uint32_t _reserved;
} RtSceneInfo;

/* Replaces the scene upload + S1 BVH build of the reference
 * (RaytraceScene.cpp:157-248, RaytracerBVH.cpp:479-550, 734-997).
 * Copies the host arrays, builds the BVH on the host when nodes == NULL,
 * and uploads the device form.  The caller keeps ownership of its arrays. */
rt_status rt_scene_create(const RtTriangle64* triangles, uint32_t num_triangles,
                          const RtSphere32* spheres, uint32_t num_spheres,
                          const RtMaterial32* materials, uint32_t num_materials,
                          const RtBVHNode40* nodes, rt_scene** out_scene);
rt_status rt_scene_create_ex(const RtSceneDesc* desc, rt_scene** out_scene);
rt_status rt_scene_destroy(rt_scene* scene);
rt_status rt_scene_get_info(const rt_scene* scene, RtSceneInfo* out_info);
/* Copies the reference-layout node array (2N-1 records) the scene was built
 * from, i.e. the content of the HLBVHNode SSBO (RaytracerBVH.cpp:536-542). */
rt_status rt_scene_get_nodes(const rt_scene* scene, RtBVHNode40* h_out, uint32_t capacity);

/* Host BVH build alone (no device work): the six S1 passes of
 * RaytracerBVH.cpp:778-991 in the reference node layout.  out_nodes holds
 * 2*(num_triangles+num_spheres)-1 records.  models may be NULL. */
rt_status rt_build_bvh(const RtTriangle64* triangles, uint32_t num_triangles,
                       const RtSphere32* spheres, uint32_t num_spheres,
                       const RtModel64* models, uint32_t num_models,
                       uint32_t bvh_mode, RtBVHNode40* out_nodes);
/* A binned surface-area-heuristic tree over the same primitives (triangles,
 * then spheres; world space when models are given), 2N-1 nodes in the
 * RtBVHNode40 form: root 0, leaves with left == right == 0 holding one
 * primitive each.  Not the reference's leaf layout -- it is the tree the
 * device traverses by default; passing it as RtSceneDesc.nodes traverses it
 * too.  No counterpart in the reference. */
rt_status rt_build_bvh_sah(const RtTriangle64* triangles, uint32_t num_triangles, const RtSphere32* spheres,
                           uint32_t num_spheres, const RtModel64* models, uint32_t num_models,
                           RtBVHNode40* out_nodes);

/* The same six S1 passes on the GPU (device in, device out), bit-identical to
 * rt_build_bvh: centroid box, 30-bit Morton codes, stable radix sort of
 * (code, index) in four 8-bit passes, Karras hierarchy, bottom-up boxes.
 * d_nodes holds 2*(num_triangles+num_spheres)-1 records.  Stream-ordered;
 * its scratch comes from the stream-ordered allocator (cudaMallocAsync). */
rt_status rt_build_bvh_device(const RtTriangle64* d_triangles, uint32_t num_triangles,
                              const RtSphere32* d_spheres, uint32_t num_spheres, uint32_t bvh_mode,
                              RtBVHNode40* d_nodes, void* stream);

/* ------------------------------------------------------------------ trace */
enum {
  RT_TRACE_CLOSEST = 0,  /* closest hit in [tmin, tmax] (hitBVH, raytraceBVH.comp:195-265) */
  RT_TRACE_ANY = 1,      /* any hit in [tmin, tmax] (occlusion) */
  RT_TRACE_SORT = 2,     /* or'ed in: trace the batch in an order bucketed by ray origin
                            (coherence); hits are unchanged and still land in ray order.
                            Uses a per-stream device workspace of about 10 bytes per ray. */
  RT_TRACE_MT = 4        /* or'ed in (rt_trace, rt_trace_host): the Moller-Trumbore
                            ray-triangle test (J. Graphics Tools 2(1), 1997) in binary32
                            instead of the reference's plane test (raytraceBVH.comp:118-149).
                            Not the reference's arithmetic: it also hits rays within
                            |n.d| < 1e-4 of the plane, which the reference rejects, and
                            its t and edge decisions round differently. */
};

/* Traces n rays resident on the device; writes n hits.  Stream-ordered.
 * d_rays must be 16-byte aligned and d_hits 8-byte aligned (RT_EINVAL
 * otherwise), as any cudaMalloc'd RtRay / RtHit array or slice of one is;
 * the same holds for every entry point that takes device rays and hits. */
rt_status rt_trace(rt_scene* scene, const RtRay* d_rays, uint32_t n, RtHit* d_hits,
                   uint32_t flags, void* stream);
/* Same with host buffers (pinned or pageable): the library stages the rays
 * through the device in chunks, overlapping copies with tracing, and returns
 * when h_hits is filled. */
rt_status rt_trace_host(rt_scene* scene, const RtRay* h_rays, uint32_t n, RtHit* h_hits,
                        uint32_t flags, void* stream);

/* rt_trace plus work counters, for measurement (no counterpart in the
 * reference): h_counts[0] = inner BVH nodes fetched, h_counts[1] = primitives
 * tested, summed over the n rays.  Synchronous. */
rt_status rt_trace_count(rt_scene* scene, const RtRay* d_rays, uint32_t n, RtHit* d_hits, uint32_t flags,
                         void* stream, uint64_t* h_counts);

/* The launch of rt_trace / rt_trace_host for one scene.  No counterpart in the
 * reference, whose dispatch size is fixed (RaytracerBVH.cpp:1025-1050). */
typedef struct RtTraceTuning {
  uint32_t launch_shape;   /* ray-query launch shape (threads per block x resident blocks,
                              traversal-stack ring in shared memory); index into the
                              table RT_TRACE_VARIANT selects from */
  uint32_t refill;         /* idle lanes of a warp that make it take new rays */
  uint32_t stack_entries;  /* traversal stack capacity per lane (>= the tree's worst case) */
  uint32_t tile_nodes;     /* top-of-tree nodes staged in shared memory per block (0: none) */
  float best_ms;           /* rt_trace_autotune: the best launch time measured */
} RtTraceTuning;
/* Times rt_trace's launch shapes, refill thresholds, stack capacities and
 * top-of-tree staging tiles on the caller's batch (flags RT_TRACE_ANY and
 * RT_TRACE_SORT as for rt_trace), keeps the fastest for the scene (used by
 * later rt_trace and rt_trace_host calls; hits do not depend on it) and
 * reports it in *out (may be NULL).  d_hits receives the batch's hits.
 * Synchronous; launches each candidate 1 + repeats times (repeats 0: 3). */
rt_status rt_trace_autotune(rt_scene* scene, const RtRay* d_rays, uint32_t n, RtHit* d_hits, uint32_t flags,
                            void* stream, uint32_t repeats, RtTraceTuning* out);
rt_status rt_scene_get_tuning(const rt_scene* scene, RtTraceTuning* out);
/* RT_EINVAL when the scene cannot run the given launch (an unknown shape, a
 * stack capacity below the tree's worst case, a tile on a shape without one). */
rt_status rt_scene_set_tuning(rt_scene* scene, const RtTraceTuning* tuning);

/* rt_trace without any device allocation.  No counterpart in the reference.
 *
 * Who needs it: host applications that must not call cudaMalloc while they
 * trace -- an engine that reserves the device's memory up front and hands
 * every byte out from its own pool, or a frame loop that cannot afford the
 * device-wide synchronisation a cudaMalloc may cause.  rt_trace allocates a
 * small per-stream workspace (its ray-queue counter) with cudaMalloc the
 * first time it sees a stream; this entry point never allocates.  The scene
 * (created beforehand; creation does allocate), the rays and the hits are
 * the caller's, as for rt_trace, and the results are identical.
 *
 * Its scratch is a file-scope device array of RT_NOALLOC_SCRATCH_BYTES that
 * every GPU which loads the library holds until the process exits; the
 * kernel uses its first word, the ray-queue counter.  Every call looks up
 * the array's address on the current device (cudaGetSymbolAddress), so no
 * address is kept across a cudaDeviceReset; the first call on a device loads
 * the library's device code, so make it before any stream capture.  All calls
 * share the one array and it keeps the last call's
 * contents (each call zeroes the counter first): calls that overlap on the
 * GPU -- on different streams or from different host threads -- race and
 * must be serialised by the caller.
 * Limit: n <= RT_NOALLOC_MAX_RAYS per call (the scratch counter is 32-bit);
 * larger n returns RT_EINVAL. */
#define RT_NOALLOC_SCRATCH_BYTES 256u
#define RT_NOALLOC_MAX_RAYS 0x80000000u
rt_status rt_trace_noalloc(rt_scene* scene, const RtRay* d_rays, uint32_t n, RtHit* d_hits,
                           uint32_t flags, void* stream);

/* ------------------------------------------------------------ scene pool */
/* Resident scenes sharing one device arena, traced together in one launch.
 * No counterpart in the reference, which traces one scene per frame; this is
 * the batched form of rt_trace: many scenes of uneven size, each with its own
 * ray batch, traced by one persistent launch replayed from a captured CUDA
 * graph, with the launch shape picked by rt_pool_autotune.  Pooled scenes hold
 * triangles only and use the 4-wide device BVH; at most 2^27 triangles per pool. */
typedef struct rt_pool rt_pool;

typedef struct RtPoolOptions {
  uint64_t budget_bytes;  /* device bytes the scenes may occupy (nodes + triangles); 0 = 8 GiB */
  uint32_t max_scenes;    /* 0 = 4096 */
  uint32_t _reserved;
} RtPoolOptions;

typedef struct RtPoolInfo {
  uint32_t num_scenes;
  uint32_t stack_need;    /* worst-case traversal stack over the pooled scenes */
  uint64_t used_bytes;    /* scene bytes accounted against the budget */
  uint64_t budget_bytes;
  uint64_t arena_bytes;   /* device memory the arena holds */
  uint32_t num_triangles;
  uint32_t tuned_variant; /* launch shape in use (see rt_pool_describe_variant) */
  int32_t tuned_refill;   /* idle lanes that trigger a ray refill */
  uint32_t tuned_stack;   /* traversal stack capacity per lane */
  uint32_t tuned_tile;    /* top-of-tree nodes of each job's scene staged in shared memory (0: none) */
  uint32_t _pad;
} RtPoolInfo;

typedef struct RtJob {    /* one scene's ray batch */
  uint32_t scene_id;
  uint32_t num_rays;
  const RtRay* d_rays;    /* device */
  RtHit* d_hits;          /* device */
} RtJob;

rt_status rt_pool_create(const RtPoolOptions* opt, rt_pool** out_pool);
rt_status rt_pool_destroy(rt_pool* pool);
/* Builds the scene's BVH on the host like rt_scene_create_ex and uploads it
 * into the arena.  RT_ENOMEM when it would exceed the budget, RT_EBUSY at the
 * scene limit, RT_EUNSUPPORTED for spheres. */
rt_status rt_pool_add_scene(rt_pool* pool, const RtSceneDesc* desc, uint32_t* out_scene_id);
/* Frees the scene's arena ranges; no batch using it may still be in flight. */
rt_status rt_pool_remove_scene(rt_pool* pool, uint32_t scene_id);
rt_status rt_pool_get_info(const rt_pool* pool, RtPoolInfo* out_info);
/* Traces all jobs (at most 8192, 2^31 rays) in one persistent launch, stream-
 * ordered.  flags: RT_TRACE_CLOSEST or RT_TRACE_ANY for every job.  Hits are
 * identical to rt_trace on each scene alone. */
rt_status rt_pool_trace(rt_pool* pool, const RtJob* jobs, uint32_t num_jobs, uint32_t flags, void* stream);
/* Times the jobs under every launch shape (threads per block, register cap)
 * and refill threshold, then, on the two shapes of 128 threads x 10 blocks
 * with four node visits per iteration (variants 5 and 6),
 * every traversal stack capacity (48, 64, 96, 192 entries, at least the pooled
 * scenes' worst case) and top-of-tree tile (0, 1 or 2 nodes of each job's
 * scene staged in shared memory per block, for batches of up to 256 jobs),
 * `repeats` launches each, and keeps the fastest for later rt_pool_trace
 * calls (rt_pool_get_info reports it).  Synchronous. */
rt_status rt_pool_autotune(rt_pool* pool, const RtJob* jobs, uint32_t num_jobs, uint32_t flags, void* stream,
                           uint32_t repeats);
/* Sets the launch rt_pool_trace uses (what rt_pool_autotune would choose):
 * launch shape, refill threshold, stack capacity (0: 64 or 192 by the pooled
 * scenes' worst case) and top-of-tree tile per job (0, 1 or 2; variants 5
 * and 6 only).  RT_EINVAL for a combination the pool cannot run. */
rt_status rt_pool_set_tuning(rt_pool* pool, uint32_t variant, int32_t refill, uint32_t stack_entries,
                             uint32_t tile_nodes);
/* Launch shape of a variant: threads per block, minimum resident blocks per
 * SM (the register cap), and the traversal-stack entries kept in shared
 * memory per lane (0: all in local memory).  stack_ring may be NULL.
 * Variants 5 (the default) and 6 have the shapes of 0 and 3 and make up to
 * four node visits per loop iteration. */
rt_status rt_pool_describe_variant(uint32_t variant, uint32_t* threads, uint32_t* min_blocks,
                                   uint32_t* stack_ring);

/* ---------------------------------------------------------------- serving */
/* A request loop over a scene pool (no counterpart in the reference): keeps
 * scenes resident on the device, admits ray queries and scene uploads, and
 * batches queries continuously -- queries that arrive while earlier batches
 * run are staged and launched on further streams (up to max_inflight batches
 * on the device at once) as staging memory frees up.  Uploads are admitted
 * against the byte budget, evicting least-recently-used idle scenes.
 * Host ray/hit buffers and upload arrays must stay valid until the request
 * completes; pinned host memory lets the copies run asynchronously. */
typedef struct rt_server rt_server;

typedef struct RtServerOptions {
  uint64_t budget_bytes;    /* resident scene bytes; 0 = 8 GiB */
  uint32_t max_scenes;      /* 0 = 4096 */
  uint32_t stage_rays;      /* device staging capacity in rays (40 B each); 0 = 2^25 */
  uint32_t max_batch_rays;  /* rays per batch launch; 0 = 2^23 */
  uint32_t max_batch_jobs;  /* queries per batch launch (<= 8192); 0 = 1024 */
  uint32_t max_inflight;    /* batches on the device at once (<= 16); 0 = 3 */
  uint32_t _pad;
} RtServerOptions;

typedef struct RtServerStats {
  uint64_t requests_done;
  uint64_t rays_done;
  uint64_t uploads_done;
  uint64_t batches;
  uint64_t evictions;
  uint32_t pending;
  uint32_t inflight_batches;
  uint32_t resident_scenes;
  uint32_t _pad;
  uint64_t resident_bytes;
} RtServerStats;

typedef struct RtRequestResult {
  int32_t status;           /* rt_status of the request */
  uint32_t scene_id;        /* the query's scene, or the id an upload received */
  uint32_t num_rays;
  uint32_t batch_jobs;      /* queries in the batch that carried this one */
  double latency_seconds;   /* submit -> completion */
  double queue_seconds;     /* submit -> start */
} RtRequestResult;

rt_status rt_server_create(const RtServerOptions* opt, rt_server** out_server);
/* Cancels queued requests, waits for running ones, frees everything. */
rt_status rt_server_destroy(rt_server* server);
/* Queues a scene upload (BVH built on the host by the server). */
rt_status rt_server_upload(rt_server* server, const RtSceneDesc* desc, uint64_t* out_request);
/* Queues a closest/any-hit query of n host rays into host hits. */
rt_status rt_server_submit(rt_server* server, uint32_t scene_id, const RtRay* h_rays, uint32_t n, RtHit* h_hits,
                           uint32_t flags, uint64_t* out_request);
/* Cancels a request that has not started (RT_EBUSY once it runs). */
rt_status rt_server_cancel(rt_server* server, uint64_t request);
/* Waits up to timeout_seconds; RT_ETIMEOUT leaves the request queryable.
 * Returns the request's status and forgets it. */
rt_status rt_server_wait(rt_server* server, uint64_t request, double timeout_seconds, RtRequestResult* out);
rt_status rt_server_remove_scene(rt_server* server, uint32_t scene_id);
rt_status rt_server_get_stats(rt_server* server, RtServerStats* out);
/* Changes the batching policy of a running server: queries per launch and
 * batches on the device at once (at most the max_inflight it was created with).
 * max_batch_jobs = max_inflight = 1 gives plain sequential service. */
rt_status rt_server_set_batching(rt_server* server, uint32_t max_batch_jobs, uint32_t max_inflight);
/* Runs the pool autotuner on one resident scene's device ray batch. */
rt_status rt_server_autotune(rt_server* server, uint32_t scene_id, const RtRay* d_rays, uint32_t n, RtHit* d_hits);

/* ----------------------------------------------------------------- render */
enum {
  RT_SHADE_REFERENCE = 0, /* LIGHT emits, DIFFUSE scatters, others terminate, background 0 */
  RT_SHADE_EXTENDED = 1   /* + metal (fuzz), dielectric (ior), background colour */
};

/* RtRenderOptions.flags.  The reference camera has no jitter
 * (raytraceBVH.comp:329-342), so every sample of a pixel starts with the same
 * primary ray and meets the same first hit; by default the first hit is found
 * once per pixel and call and shared by the pixel's samples (the result is the
 * same bit for bit).  This flag traces every sample's primary ray instead, as
 * the reference's spp dispatches do. */
#define RT_RENDER_TRACE_EVERY_PRIMARY 1u

typedef struct RtRenderOptions {
  uint32_t shade_mode;     /* RT_SHADE_REFERENCE | RT_SHADE_EXTENDED */
  float background[3];     /* used by RT_SHADE_EXTENDED only */
  uint32_t flags;          /* RT_RENDER_TRACE_EVERY_PRIMARY or 0 */
} RtRenderOptions;

/* The S2 pass (RaytracerBVH.cpp:998-1078): spp samples per pixel of
 * raytraceBVH.comp:main, each adding its colour to d_accum (W*H float4,
 * row-major, pixel (x,y) at index y*W+x) and leaving the RNG carry in alpha,
 * exactly as spp back-to-back dispatches would.  opt may be NULL (reference).
 * Stream-ordered on `stream`: the library may fork part of the frame onto a
 * helper stream of its own, which waits for `stream` first and which
 * `stream` waits for before anything enqueued after this call (an event
 * fork/join). */
rt_status rt_render(rt_scene* scene, const RtRaytraceUBO* ubo, float* d_accum,
                    uint32_t width, uint32_t height, uint32_t spp,
                    const RtRenderOptions* opt, void* stream);
/* rt_render plus work counters, for measurement (no counterpart in the
 * reference): h_counts[0] = closest-hit queries (bounces traced),
 * h_counts[1] = inner BVH nodes fetched, h_counts[2] = primitives tested,
 * summed over the frame.  Synchronous. */
rt_status rt_render_count(rt_scene* scene, const RtRaytraceUBO* ubo, float* d_accum,
                          uint32_t width, uint32_t height, uint32_t spp,
                          const RtRenderOptions* opt, void* stream, uint64_t* h_counts);
/* The per-frame clear of the accumulator to (0,0,0,1) (RaytracerBVH.cpp:772-776). */
rt_status rt_accum_clear(float* d_accum, uint32_t width, uint32_t height, void* stream);
/* The present pass's colour math, clamp(sqrt(sum/spp), 0, 1)
 * (SingleTriangleFullScreen.frag:13-18), into a W*H float4 device buffer. */
rt_status rt_resolve(const float* d_accum, uint32_t width, uint32_t height, uint32_t spp,
                     float* d_out, void* stream);

/* ------------------------------------------------------- scene ingestion */
/* Wavefront OBJ -> triangles, as the reference's loadModel (RTModel.cpp:47-108,
 * tinyobjloader): face vertex positions, polygons fanned from their first
 * vertex, file order.  Call with out = NULL to get the count. */
rt_status rt_obj_load(const char* path, uint32_t material, RtTriangle64* out, uint64_t capacity, uint64_t* count);
/* TransformComponent::mat4 (TransformComponent.cpp:9-45): translate * Ry * Rx * Rz * scale,
 * Tait-Bryan Y-X-Z angles in radians, column-major. */
rt_status rt_model_matrix(const float translation[3], const float rotation[3], const float scale[3],
                          RtModel64* out);
/* Headless stand-ins for the present pass: a W*H RGBA float image (e.g. from
 * rt_resolve, copied to the host) to binary PPM (8-bit, top row first) or PFM. */
rt_status rt_write_ppm(const char* path, const float* h_rgba, uint32_t width, uint32_t height);
rt_status rt_write_pfm(const char* path, const float* h_rgba, uint32_t width, uint32_t height);

/* --------------------------------------------------------------- utility */
/* Device memory for callers without CUDA headers (the C++ mirror uses these). */
rt_status rt_device_alloc(size_t bytes, void** d_out);
rt_status rt_device_free(void* d_ptr);
/* Stream-ordered copies; host memory pinned or pageable. */
rt_status rt_copy(void* dst, const void* src, size_t bytes, void* stream);
const char* rt_last_error_string(void);
uint32_t rt_abi_version(void);
/* Waits for the stream with a deadline; RT_ETIMEOUT when it runs out. */
rt_status rt_stream_wait(void* stream, double timeout_seconds);
/* Device-side index checks (no counterpart in the reference).  A library
 * built with RT_DEVICE_CHECKS=1 (librt_gb300_checked.so) checks every node,
 * primitive, ray, material and path index its kernels use against the
 * scene's arrays; an index out of range sets a bit in the scene's check word
 * (1 node, 2 triangle, 4 sphere, 8 ray, 16 material, 32 path), records the
 * first bad index, and the access is skipped.  rt_scene_device_checks reads
 * and clears the word (synchronous; always 0 in the normal build). */
uint32_t rt_device_checks_compiled(void);
rt_status rt_scene_device_checks(rt_scene* scene, uint32_t* bits, uint32_t* first_index);
/* Frees the device workspace the library keeps for this stream on the current
 * device (work counters, ray staging, reorder and path-tracing scratch), after
 * the stream's work has finished.  No call on the stream may run concurrently;
 * a later call on it allocates a new workspace.  No counterpart in the
 * reference. */
rt_status rt_stream_release(void* stream);
/* How many per-(device, stream) workspaces the library holds: each is created
 * with cudaMalloc the first time rt_trace, rt_trace_host, rt_trace_count or
 * rt_render sees a stream, and freed by rt_stream_release.  A diagnostic of
 * the library's own device allocations.  No counterpart in the reference. */
uint32_t rt_workspace_count(void);

#ifdef __cplusplus
}
#endif

#endif /* RT_GB300_H */
