"""GB300 (sm_103a) ray-tracing hot path of RaytracerGPU_MastersProject.

Python host mirror of the C ABI in include/rt_gb300.h.  The reference's host
interface for this path is the raytrace pass of RaytracerBVHRenderer::Raytracer
(RaytracerBVH.hpp:206-496): a RaytraceScene whose triangle, sphere, material
and BVH-node buffers, plus a ParameterUBO and an RGBA32F accumulator, feed one
compute dispatch per ray per pixel.  Here:

  Scene(...)        RaytraceScene::prepForRender + S1 BVH build  (rt_scene_create_ex)
  Scene.trace(...)  hitBVH over a batch of rays                    (rt_trace)
  Scene.render(...) the S2 pass, spp samples into the accumulator  (rt_render)

Every call goes to librt_gb300.so.  There is no CPU fallback: importing this
package without the built library raises, and so does calling a GPU entry
point without a GPU.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "librt_gb300.so"

# ------------------------------------------------------------------ records
TRIANGLE_DTYPE = np.dtype([("v0", "<f4", 4), ("v1", "<f4", 4), ("v2", "<f4", 4), ("materialIndex", "<u4"),
                           ("modelIndex", "<u4"), ("_pad", "<u4", 2)])
SPHERE_DTYPE = np.dtype([("center", "<f4", 4), ("radius", "<f4"), ("materialIndex", "<u4"),
                         ("modelIndex", "<u4"), ("_pad", "<u4")])
MATERIAL_DTYPE = np.dtype([("albedo", "<f4", 4), ("materialType", "<u4"), ("fuzz", "<f4"), ("ior", "<f4"),
                           ("_pad", "<u4")])
NODE_DTYPE = np.dtype([("minX", "<f4"), ("maxX", "<f4"), ("minY", "<f4"), ("maxY", "<f4"), ("minZ", "<f4"),
                       ("maxZ", "<f4"), ("left", "<u4"), ("right", "<u4"), ("primitiveIndex", "<u4"),
                       ("primitiveType", "<u4")])
MODEL_DTYPE = np.dtype([("m", "<f4", 16)])
RAY_DTYPE = np.dtype([("org", "<f4", 3), ("tmin", "<f4"), ("dir", "<f4", 3), ("tmax", "<f4")])
HIT_DTYPE = np.dtype([("prim", "<u4"), ("t", "<f4")])
assert TRIANGLE_DTYPE.itemsize == 64 and SPHERE_DTYPE.itemsize == 32 and MATERIAL_DTYPE.itemsize == 32
assert NODE_DTYPE.itemsize == 40 and RAY_DTYPE.itemsize == 32 and HIT_DTYPE.itemsize == 8

MAT_LIGHT, MAT_DIFFUSE, MAT_METALLIC, MAT_DIELECTRIC = 0, 1, 2, 3
PRIM_SPHERE, PRIM_TRIANGLE = 0, 1
BVH_SORTED, BVH_REFERENCE = 0, 1
TRACE_CLOSEST, TRACE_ANY, TRACE_SORT, TRACE_MT = 0, 1, 2, 4
SHADE_REFERENCE, SHADE_EXTENDED = 0, 1
NO_HIT = 0xFFFFFFFF
HIT_SPHERE_BIT = 0x80000000

STATUS = {0: "RT_OK", 1: "RT_EINVAL", 2: "RT_ENOMEM", 3: "RT_ETIMEOUT", 4: "RT_ESTACK", 5: "RT_ECUDA",
          6: "RT_EBUSY", 7: "RT_ECANCELED", 8: "RT_ENOTFOUND", 9: "RT_EUNSUPPORTED"}


class RtError(RuntimeError):
    def __init__(self, status: int, where: str, msg: str):
        self.status = status
        super().__init__(f"{where}: {STATUS.get(status, status)}: {msg}")


class RaytracingUBO(C.Structure):
    """ParameterUBO (raytraceBVH.comp:7-18; RaytracerBVH.hpp:31-42), 80 bytes."""
    _fields_ = [("camPos", C.c_float * 4), ("camLookAt", C.c_float * 4), ("camUpDir", C.c_float * 4),
                ("verticalFOV", C.c_float), ("numTriangles", C.c_uint32), ("numSpheres", C.c_uint32),
                ("numMaterials", C.c_uint32), ("numLights", C.c_uint32), ("maxRayTraceDepth", C.c_uint32),
                ("randomState", C.c_uint32), ("_pad", C.c_uint32)]


class TraceTuning(C.Structure):
    """RtTraceTuning: the launch of rt_trace / rt_trace_host for one scene."""
    _fields_ = [("launch_shape", C.c_uint32), ("refill", C.c_uint32), ("stack_entries", C.c_uint32),
                ("tile_nodes", C.c_uint32), ("best_ms", C.c_float)]

    def as_dict(self) -> dict:
        return {"launch_shape": self.launch_shape, "refill": self.refill, "stack_entries": self.stack_entries,
                "tile_nodes": self.tile_nodes, "best_ms": self.best_ms}


class _SceneDesc(C.Structure):
    _fields_ = [("triangles", C.c_void_p), ("num_triangles", C.c_uint32), ("spheres", C.c_void_p),
                ("num_spheres", C.c_uint32), ("materials", C.c_void_p), ("num_materials", C.c_uint32),
                ("models", C.c_void_p), ("num_models", C.c_uint32), ("nodes", C.c_void_p),
                ("num_nodes", C.c_uint32), ("bvh_mode", C.c_uint32), ("leaf_size", C.c_uint32),
                ("node_width", C.c_uint32), ("build_flags", C.c_uint32)]

BUILD_ON_DEVICE = 1
BUILD_TRAVERSE_S1 = 2


class SceneInfo(C.Structure):
    _fields_ = [("num_triangles", C.c_uint32), ("num_spheres", C.c_uint32), ("num_materials", C.c_uint32),
                ("num_nodes", C.c_uint32), ("device_nodes", C.c_uint32), ("depth", C.c_uint32),
                ("leaf_size", C.c_uint32), ("bvh_mode", C.c_uint32), ("device_bytes", C.c_uint64),
                ("build_seconds", C.c_double), ("node_width", C.c_uint32), ("stack_need", C.c_uint32),
                ("traversal_sah", C.c_uint32), ("_reserved", C.c_uint32)]


class PoolOptions(C.Structure):
    _fields_ = [("budget_bytes", C.c_uint64), ("max_scenes", C.c_uint32), ("_reserved", C.c_uint32)]


class PoolInfo(C.Structure):
    _fields_ = [("num_scenes", C.c_uint32), ("stack_need", C.c_uint32), ("used_bytes", C.c_uint64),
                ("budget_bytes", C.c_uint64), ("arena_bytes", C.c_uint64), ("num_triangles", C.c_uint32),
                ("tuned_variant", C.c_uint32), ("tuned_refill", C.c_int32), ("tuned_stack", C.c_uint32),
                ("tuned_tile", C.c_uint32), ("_pad", C.c_uint32)]


class Job(C.Structure):
    """RtJob: one scene's ray batch (device buffers)."""
    _fields_ = [("scene_id", C.c_uint32), ("num_rays", C.c_uint32), ("d_rays", C.c_void_p), ("d_hits", C.c_void_p)]


class ServerOptions(C.Structure):
    _fields_ = [("budget_bytes", C.c_uint64), ("max_scenes", C.c_uint32), ("stage_rays", C.c_uint32),
                ("max_batch_rays", C.c_uint32), ("max_batch_jobs", C.c_uint32), ("max_inflight", C.c_uint32),
                ("_pad", C.c_uint32)]


class ServerStats(C.Structure):
    _fields_ = [("requests_done", C.c_uint64), ("rays_done", C.c_uint64), ("uploads_done", C.c_uint64),
                ("batches", C.c_uint64), ("evictions", C.c_uint64), ("pending", C.c_uint32),
                ("inflight_batches", C.c_uint32), ("resident_scenes", C.c_uint32), ("_pad", C.c_uint32),
                ("resident_bytes", C.c_uint64)]


class RequestResult(C.Structure):
    _fields_ = [("status", C.c_int32), ("scene_id", C.c_uint32), ("num_rays", C.c_uint32),
                ("batch_jobs", C.c_uint32), ("latency_seconds", C.c_double), ("queue_seconds", C.c_double)]


class _RenderOptions(C.Structure):
    _fields_ = [("shade_mode", C.c_uint32), ("background", C.c_float * 3), ("flags", C.c_uint32)]


RENDER_TRACE_EVERY_PRIMARY = 1


assert C.sizeof(RaytracingUBO) == 80

# ------------------------------------------------------------------ loading
_lib = None

# Every symbol the library must export, with (restype, argtypes).
_P, _U32, _U64, _F, _D, _I = C.c_void_p, C.c_uint32, C.c_uint64, C.c_float, C.c_double, C.c_int
SIGNATURES = {
    "rt_scene_create": (_I, [_P, _U32, _P, _U32, _P, _U32, _P, C.POINTER(C.c_void_p)]),
    "rt_scene_create_ex": (_I, [C.POINTER(_SceneDesc), C.POINTER(C.c_void_p)]),
    "rt_scene_destroy": (_I, [_P]),
    "rt_scene_get_info": (_I, [_P, C.POINTER(SceneInfo)]),
    "rt_scene_get_nodes": (_I, [_P, _P, _U32]),
    "rt_build_bvh": (_I, [_P, _U32, _P, _U32, _P, _U32, _U32, _P]),
    "rt_build_bvh_sah": (_I, [_P, _U32, _P, _U32, _P, _U32, _P]),
    "rt_build_bvh_device": (_I, [_P, _U32, _P, _U32, _U32, _P, _P]),
    "rt_trace": (_I, [_P, _P, _U32, _P, _U32, _P]),
    "rt_trace_host": (_I, [_P, _P, _U32, _P, _U32, _P]),
    "rt_trace_count": (_I, [_P, _P, _U32, _P, _U32, _P, C.POINTER(_U64)]),
    "rt_render": (_I, [_P, C.POINTER(RaytracingUBO), _P, _U32, _U32, _U32, C.POINTER(_RenderOptions), _P]),
    "rt_render_count": (_I, [_P, C.POINTER(RaytracingUBO), _P, _U32, _U32, _U32, C.POINTER(_RenderOptions), _P,
                             C.POINTER(_U64)]),
    "rt_accum_clear": (_I, [_P, _U32, _U32, _P]),
    "rt_resolve": (_I, [_P, _U32, _U32, _U32, _P, _P]),
    "rt_last_error_string": (C.c_char_p, []),
    "rt_abi_version": (_U32, []),
    "rt_stream_wait": (_I, [_P, _D]),
    "rt_device_checks_compiled": (_U32, []),
    "rt_scene_device_checks": (_I, [_P, C.POINTER(_U32), C.POINTER(_U32)]),
    "rt_stream_release": (_I, [_P]),
    "rt_workspace_count": (_U32, []),
    "rt_trace_autotune": (_I, [_P, _P, _U32, _P, _U32, _P, _U32, C.POINTER(TraceTuning)]),
    "rt_scene_get_tuning": (_I, [_P, C.POINTER(TraceTuning)]),
    "rt_scene_set_tuning": (_I, [_P, C.POINTER(TraceTuning)]),
    "rt_pool_create": (_I, [C.POINTER(PoolOptions), C.POINTER(C.c_void_p)]),
    "rt_pool_destroy": (_I, [_P]),
    "rt_pool_add_scene": (_I, [_P, C.POINTER(_SceneDesc), C.POINTER(_U32)]),
    "rt_pool_remove_scene": (_I, [_P, _U32]),
    "rt_pool_get_info": (_I, [_P, C.POINTER(PoolInfo)]),
    "rt_pool_trace": (_I, [_P, C.POINTER(Job), _U32, _U32, _P]),
    "rt_pool_autotune": (_I, [_P, C.POINTER(Job), _U32, _U32, _P, _U32]),
    "rt_pool_describe_variant": (_I, [_U32, C.POINTER(_U32), C.POINTER(_U32), C.POINTER(_U32)]),
    "rt_pool_set_tuning": (_I, [_P, _U32, C.c_int32, _U32, _U32]),
    "rt_server_create": (_I, [C.POINTER(ServerOptions), C.POINTER(C.c_void_p)]),
    "rt_server_destroy": (_I, [_P]),
    "rt_server_upload": (_I, [_P, C.POINTER(_SceneDesc), C.POINTER(_U64)]),
    "rt_server_submit": (_I, [_P, _U32, _P, _U32, _P, _U32, C.POINTER(_U64)]),
    "rt_server_cancel": (_I, [_P, _U64]),
    "rt_server_wait": (_I, [_P, _U64, _D, C.POINTER(RequestResult)]),
    "rt_server_remove_scene": (_I, [_P, _U32]),
    "rt_server_get_stats": (_I, [_P, C.POINTER(ServerStats)]),
    "rt_server_autotune": (_I, [_P, _U32, _P, _U32, _P]),
    "rt_server_set_batching": (_I, [_P, _U32, _U32]),
    "rt_obj_load": (_I, [C.c_char_p, _U32, _P, _U64, C.POINTER(_U64)]),
    "rt_model_matrix": (_I, [_P, _P, _P, _P]),
    "rt_write_ppm": (_I, [C.c_char_p, _P, _U32, _U32]),
    "rt_write_pfm": (_I, [C.c_char_p, _P, _U32, _U32]),
    "rt_gen_uniform": (_I, [_U64, _U64, _U64, _P]),
    "rt_gen_icosphere": (_I, [_U32, _P, _F, _U32, _P, _U64, C.POINTER(_U64)]),
    "rt_gen_config1": (_I, [_P, C.POINTER(RaytracingUBO), _P]),
    "rt_gen_camera_rays": (_I, [C.POINTER(RaytracingUBO), _U32, _U32, _P]),
    "rt_gen_soup": (_I, [_U64, _U64, _U32, _F, _F, _U32, _P]),
    "rt_gen_rays": (_I, [_U64, _U64, _U32, _F, _F, _F, _P]),
    "rt_gen_spheres_scene": (_I, [_U64, _U32, _U32, _F, _P, _P]),
}


def lib() -> C.CDLL:
    """Loads librt_gb300.so (built by __graft_entry__.build()); raises if absent."""
    global _lib
    if _lib is None:
        path = Path(os.environ.get("RT_GB300_LIB", LIB_PATH))
        if not path.exists():
            raise ImportError(f"{path} is not built: run python -c 'import __graft_entry__ as g; g.build()'")
        L = C.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(status: int, where: str) -> None:
    if status != 0:
        raise RtError(status, where, lib().rt_last_error_string().decode(errors="replace"))


def _ptr(a) -> int | None:
    """Address of a numpy array or torch tensor (None for None/empty)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if a.size == 0:
            return None
        assert a.flags["C_CONTIGUOUS"], "arrays passed to the ABI must be C-contiguous"
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        assert a.is_contiguous(), "tensors passed to the ABI must be contiguous"
        return a.data_ptr() or None
    raise TypeError(f"cannot take the address of {type(a)}")


def _stream_handle(stream) -> int | None:
    if stream is None:
        try:
            import torch
            if torch.cuda.is_available():
                return torch.cuda.current_stream().cuda_stream or None
        except ImportError:
            pass
        return None
    if isinstance(stream, int):
        return stream or None
    return stream.cuda_stream or None


# ------------------------------------------------------------------- scene
class Scene:
    """A scene resident on the device: RaytraceScene's buffers + the BVH.

    triangles: TRIANGLE_DTYPE array (world space unless models is given)
    spheres, materials, models, nodes: optional arrays of the record dtypes
    bvh_mode: BVH_SORTED (default) or BVH_REFERENCE (the reference's leaf order)
    leaf_size: max triangles per device leaf (1..8); 0 = library default
    node_width: device BVH width, 2 (binary) or 4 (quantised 4-wide); 0 = library default
    build_on_device: build the S1 node array on the GPU (rt_build_bvh_device)
    traverse_s1: traverse the S1 node array instead of the binned-SAH tree the
        library otherwise builds for sorted-mode scenes (same hits)
    """

    def __init__(self, triangles, spheres=None, materials=None, models=None, nodes=None,
                 bvh_mode: int = BVH_SORTED, leaf_size: int = 0, node_width: int = 0, build_on_device: bool = False,
                 traverse_s1: bool = False):
        L = lib()
        tri = np.ascontiguousarray(triangles, dtype=TRIANGLE_DTYPE) if triangles is not None else np.zeros(0, TRIANGLE_DTYPE)
        sph = np.ascontiguousarray(spheres, dtype=SPHERE_DTYPE) if spheres is not None else np.zeros(0, SPHERE_DTYPE)
        mat = np.ascontiguousarray(materials, dtype=MATERIAL_DTYPE) if materials is not None else np.zeros(0, MATERIAL_DTYPE)
        mod = np.ascontiguousarray(models, dtype=MODEL_DTYPE) if models is not None else None
        nod = np.ascontiguousarray(nodes, dtype=NODE_DTYPE) if nodes is not None else None
        d = _SceneDesc(_ptr(tri), len(tri), _ptr(sph), len(sph), _ptr(mat), len(mat),
                       _ptr(mod), 0 if mod is None else len(mod), _ptr(nod), 0 if nod is None else len(nod),
                       bvh_mode, leaf_size, node_width,
                       (BUILD_ON_DEVICE if build_on_device else 0) | (BUILD_TRAVERSE_S1 if traverse_s1 else 0))
        h = C.c_void_p()
        _check(L.rt_scene_create_ex(C.byref(d), C.byref(h)), "rt_scene_create_ex")
        self._h = h
        self.num_triangles = len(tri)
        self.num_spheres = len(sph)

    @property
    def handle(self) -> int:
        if self._h is None:
            raise ValueError("scene destroyed")
        return self._h.value

    def info(self) -> SceneInfo:
        inf = SceneInfo()
        _check(lib().rt_scene_get_info(self.handle, C.byref(inf)), "rt_scene_get_info")
        return inf

    def nodes(self) -> np.ndarray:
        n = self.info().num_nodes
        out = np.zeros(n, NODE_DTYPE)
        _check(lib().rt_scene_get_nodes(self.handle, _ptr(out), n), "rt_scene_get_nodes")
        return out

    def trace(self, rays, hits, n: int | None = None, any_hit: bool = False, sort: bool = False, stream=None,
              mt: bool = False) -> None:
        """rays/hits: device tensors holding RtRay / RtHit records (stream-ordered).
        sort: trace in an origin-bucketed order for coherence (same results).
        mt: the Moller-Trumbore triangle test instead of the reference's plane test."""
        if n is None:
            n = rays.numel() * rays.element_size() // RAY_DTYPE.itemsize
        flags = (TRACE_ANY if any_hit else TRACE_CLOSEST) | (TRACE_SORT if sort else 0) | (TRACE_MT if mt else 0)
        _check(lib().rt_trace(self.handle, _ptr(rays), n, _ptr(hits), flags, _stream_handle(stream)), "rt_trace")

    def autotune(self, rays, hits, n: int | None = None, any_hit: bool = False, sort: bool = False, stream=None,
                 repeats: int = 3) -> TraceTuning:
        """rt_trace_autotune: times the launch options on this batch and keeps the fastest."""
        if n is None:
            n = rays.numel() * rays.element_size() // RAY_DTYPE.itemsize
        flags = (TRACE_ANY if any_hit else TRACE_CLOSEST) | (TRACE_SORT if sort else 0)
        out = TraceTuning()
        _check(lib().rt_trace_autotune(self.handle, _ptr(rays), n, _ptr(hits), flags, _stream_handle(stream),
                                       repeats, C.byref(out)), "rt_trace_autotune")
        return out

    def tuning(self) -> TraceTuning:
        out = TraceTuning()
        _check(lib().rt_scene_get_tuning(self.handle, C.byref(out)), "rt_scene_get_tuning")
        return out

    def set_tuning(self, t: TraceTuning) -> None:
        _check(lib().rt_scene_set_tuning(self.handle, C.byref(t)), "rt_scene_set_tuning")

    def trace_count(self, rays, hits, n: int | None = None, any_hit: bool = False, sort: bool = False,
                    stream=None) -> tuple[int, int]:
        """rt_trace with work counters -> (inner nodes fetched, primitives tested)."""
        if n is None:
            n = rays.numel() * rays.element_size() // RAY_DTYPE.itemsize
        c = (_U64 * 2)()
        flags = (TRACE_ANY if any_hit else TRACE_CLOSEST) | (TRACE_SORT if sort else 0)
        _check(lib().rt_trace_count(self.handle, _ptr(rays), n, _ptr(hits), flags, _stream_handle(stream), c),
               "rt_trace_count")
        return int(c[0]), int(c[1])

    def trace_host(self, rays: np.ndarray, any_hit: bool = False, out: np.ndarray | None = None, sort: bool = False,
                   stream=None, mt: bool = False) -> np.ndarray:
        """Host rays in, host hits out; copies overlap with tracing inside the library."""
        rays = np.ascontiguousarray(rays, dtype=RAY_DTYPE)
        if out is None:
            out = np.empty(len(rays), HIT_DTYPE)
        flags = (TRACE_ANY if any_hit else TRACE_CLOSEST) | (TRACE_SORT if sort else 0) | (TRACE_MT if mt else 0)
        _check(lib().rt_trace_host(self.handle, _ptr(rays), len(rays), _ptr(out), flags, _stream_handle(stream)),
               "rt_trace_host")
        return out

    def render(self, ubo: RaytracingUBO, accum, width: int, height: int, spp: int,
               shade_mode: int = SHADE_REFERENCE, background=(0.0, 0.0, 0.0), stream=None,
               trace_every_primary: bool = False) -> None:
        """accum: device float32 tensor of width*height*4 (RGBA32F, alpha = RNG carry).
        trace_every_primary: trace each sample's primary ray instead of sharing a
        pixel's first hit between its samples (same result)."""
        opt = _RenderOptions(shade_mode, (C.c_float * 3)(*background),
                             RENDER_TRACE_EVERY_PRIMARY if trace_every_primary else 0)
        _check(lib().rt_render(self.handle, C.byref(ubo), _ptr(accum), width, height, spp, C.byref(opt),
                               _stream_handle(stream)), "rt_render")

    def render_count(self, ubo: RaytracingUBO, accum, width: int, height: int, spp: int,
                     shade_mode: int = SHADE_REFERENCE, background=(0.0, 0.0, 0.0), stream=None,
                     trace_every_primary: bool = False) -> tuple[int, int, int]:
        """render with work counters -> (closest-hit queries traced, inner nodes fetched, primitives tested)."""
        opt = _RenderOptions(shade_mode, (C.c_float * 3)(*background),
                             RENDER_TRACE_EVERY_PRIMARY if trace_every_primary else 0)
        c = (_U64 * 3)()
        _check(lib().rt_render_count(self.handle, C.byref(ubo), _ptr(accum), width, height, spp, C.byref(opt),
                                     _stream_handle(stream), c), "rt_render_count")
        return int(c[0]), int(c[1]), int(c[2])

    def device_checks(self) -> tuple[int, int]:
        """Reads and clears the checked build's index-check word -> (bits, first bad index)."""
        b, f = C.c_uint32(), C.c_uint32()
        _check(lib().rt_scene_device_checks(self.handle, C.byref(b), C.byref(f)), "rt_scene_device_checks")
        return b.value, f.value

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().rt_scene_destroy(self._h.value)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def _desc(triangles, models=None, nodes=None, bvh_mode=BVH_SORTED, leaf_size=0, node_width=0, build_flags=0):
    tri = np.ascontiguousarray(triangles, dtype=TRIANGLE_DTYPE)
    mod = np.ascontiguousarray(models, dtype=MODEL_DTYPE) if models is not None else None
    nod = np.ascontiguousarray(nodes, dtype=NODE_DTYPE) if nodes is not None else None
    d = _SceneDesc(_ptr(tri), len(tri), None, 0, None, 0, _ptr(mod), 0 if mod is None else len(mod),
                   _ptr(nod), 0 if nod is None else len(nod), bvh_mode, leaf_size, node_width, build_flags)
    return d, (tri, mod, nod)


class Pool:
    """Resident scenes in one device arena, traced together (rt_pool_*).

    add_scene() admits a scene against the byte budget; trace() runs every
    job -- (scene_id, device rays, device hits[, n]) -- in one persistent,
    graph-replayed launch; autotune() picks the launch shape for a batch."""

    def __init__(self, budget_bytes: int = 0, max_scenes: int = 0):
        opt = PoolOptions(budget_bytes, max_scenes, 0)
        h = C.c_void_p()
        _check(lib().rt_pool_create(C.byref(opt), C.byref(h)), "rt_pool_create")
        self._h = h

    @property
    def handle(self) -> int:
        if self._h is None:
            raise ValueError("pool destroyed")
        return self._h.value

    def add_scene(self, triangles, models=None, nodes=None, bvh_mode: int = BVH_SORTED, leaf_size: int = 0,
                  build_on_device: bool = False) -> int:
        d, keep = _desc(triangles, models, nodes, bvh_mode, leaf_size, 4, BUILD_ON_DEVICE if build_on_device else 0)
        sid = C.c_uint32()
        _check(lib().rt_pool_add_scene(self.handle, C.byref(d), C.byref(sid)), "rt_pool_add_scene")
        return sid.value

    def remove_scene(self, scene_id: int) -> None:
        _check(lib().rt_pool_remove_scene(self.handle, scene_id), "rt_pool_remove_scene")

    def info(self) -> PoolInfo:
        inf = PoolInfo()
        _check(lib().rt_pool_get_info(self.handle, C.byref(inf)), "rt_pool_get_info")
        return inf

    @staticmethod
    def _jobs(jobs):
        arr = (Job * max(len(jobs), 1))()
        for i, j in enumerate(jobs):
            sid, rays, hits = j[0], j[1], j[2]
            n = j[3] if len(j) > 3 else rays.numel() * rays.element_size() // RAY_DTYPE.itemsize
            arr[i] = Job(sid, n, _ptr(rays), _ptr(hits))
        return arr

    def trace(self, jobs, any_hit: bool = False, stream=None) -> None:
        arr = self._jobs(jobs)
        _check(lib().rt_pool_trace(self.handle, arr, len(jobs), TRACE_ANY if any_hit else TRACE_CLOSEST,
                                   _stream_handle(stream)), "rt_pool_trace")

    def autotune(self, jobs, any_hit: bool = False, repeats: int = 3, stream=None) -> tuple[int, int]:
        """-> (launch shape, refill); info() also reports the stack capacity and tile chosen."""
        arr = self._jobs(jobs)
        _check(lib().rt_pool_autotune(self.handle, arr, len(jobs), TRACE_ANY if any_hit else TRACE_CLOSEST,
                                      _stream_handle(stream), repeats), "rt_pool_autotune")
        inf = self.info()
        return inf.tuned_variant, inf.tuned_refill

    def set_tuning(self, variant: int, refill: int, stack_entries: int = 0, tile_nodes: int = 0) -> None:
        _check(lib().rt_pool_set_tuning(self.handle, variant, refill, stack_entries, tile_nodes), "rt_pool_set_tuning")

    def render_count(self, ubo: RaytracingUBO, accum, width: int, height: int, spp: int,
                     shade_mode: int = SHADE_REFERENCE, background=(0.0, 0.0, 0.0), stream=None,
                     trace_every_primary: bool = False) -> tuple[int, int, int]:
        """render with work counters -> (closest-hit queries traced, inner nodes fetched, primitives tested)."""
        opt = _RenderOptions(shade_mode, (C.c_float * 3)(*background),
                             RENDER_TRACE_EVERY_PRIMARY if trace_every_primary else 0)
        c = (_U64 * 3)()
        _check(lib().rt_render_count(self.handle, C.byref(ubo), _ptr(accum), width, height, spp, C.byref(opt),
                                     _stream_handle(stream), c), "rt_render_count")
        return int(c[0]), int(c[1]), int(c[2])

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().rt_pool_destroy(self._h.value)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Server:
    """Serving loop over resident scenes (rt_server_*).

    upload() and submit() queue requests and return their ids at once; wait()
    returns the RequestResult (status, latency, batch size) and raises on an
    error status.  Host arrays handed to upload()/submit() are kept alive here
    until their request is waited for."""

    def __init__(self, budget_bytes: int = 0, max_scenes: int = 0, stage_rays: int = 0, max_batch_rays: int = 0,
                 max_batch_jobs: int = 0, max_inflight: int = 0):
        opt = ServerOptions(budget_bytes, max_scenes, stage_rays, max_batch_rays, max_batch_jobs, max_inflight, 0)
        h = C.c_void_p()
        _check(lib().rt_server_create(C.byref(opt), C.byref(h)), "rt_server_create")
        self._h = h
        self._keep = {}

    @property
    def handle(self) -> int:
        if self._h is None:
            raise ValueError("server destroyed")
        return self._h.value

    def upload(self, triangles, models=None, bvh_mode: int = BVH_SORTED, build_on_device: bool = False) -> int:
        d, keep = _desc(triangles, models, None, bvh_mode, 0, 4, BUILD_ON_DEVICE if build_on_device else 0)
        rid = C.c_uint64()
        _check(lib().rt_server_upload(self.handle, C.byref(d), C.byref(rid)), "rt_server_upload")
        self._keep[rid.value] = (d, keep)
        return rid.value

    def submit(self, scene_id: int, rays: np.ndarray, hits: np.ndarray | None = None, any_hit: bool = False) -> int:
        """rays/hits: host arrays (pinned memory makes the copies asynchronous)."""
        if hits is None:
            hits = np.empty(len(rays), HIT_DTYPE)
        rid = C.c_uint64()
        _check(lib().rt_server_submit(self.handle, scene_id, _ptr(rays), len(rays), _ptr(hits),
                                      TRACE_ANY if any_hit else TRACE_CLOSEST, C.byref(rid)), "rt_server_submit")
        self._keep[rid.value] = (rays, hits)
        return rid.value

    def hits(self, request_id: int):
        return self._keep[request_id][1]

    def cancel(self, request_id: int) -> None:
        _check(lib().rt_server_cancel(self.handle, request_id), "rt_server_cancel")

    def wait(self, request_id: int, timeout: float = 60.0) -> RequestResult:
        res = RequestResult()
        st = lib().rt_server_wait(self.handle, request_id, timeout, C.byref(res))
        if st != 3:  # RT_ETIMEOUT keeps the request (and its arrays) alive
            self._keep.pop(request_id, None)
        _check(st, "rt_server_wait")
        return res

    def remove_scene(self, scene_id: int) -> None:
        _check(lib().rt_server_remove_scene(self.handle, scene_id), "rt_server_remove_scene")

    def set_batching(self, max_batch_jobs: int, max_inflight: int) -> None:
        _check(lib().rt_server_set_batching(self.handle, max_batch_jobs, max_inflight), "rt_server_set_batching")

    def stats(self) -> ServerStats:
        st = ServerStats()
        _check(lib().rt_server_get_stats(self.handle, C.byref(st)), "rt_server_get_stats")
        return st

    def autotune(self, scene_id: int, d_rays, d_hits, n: int | None = None) -> None:
        if n is None:
            n = d_rays.numel() * d_rays.element_size() // RAY_DTYPE.itemsize
        _check(lib().rt_server_autotune(self.handle, scene_id, _ptr(d_rays), n, _ptr(d_hits)), "rt_server_autotune")

    def render_count(self, ubo: RaytracingUBO, accum, width: int, height: int, spp: int,
                     shade_mode: int = SHADE_REFERENCE, background=(0.0, 0.0, 0.0), stream=None,
                     trace_every_primary: bool = False) -> tuple[int, int, int]:
        """render with work counters -> (closest-hit queries traced, inner nodes fetched, primitives tested)."""
        opt = _RenderOptions(shade_mode, (C.c_float * 3)(*background),
                             RENDER_TRACE_EVERY_PRIMARY if trace_every_primary else 0)
        c = (_U64 * 3)()
        _check(lib().rt_render_count(self.handle, C.byref(ubo), _ptr(accum), width, height, spp, C.byref(opt),
                                     _stream_handle(stream), c), "rt_render_count")
        return int(c[0]), int(c[1]), int(c[2])

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().rt_server_destroy(self._h.value)
        self._h = None
        self._keep = {}

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def device_checks_compiled() -> bool:
    """True for the checked build (RT_DEVICE_CHECKS=1)."""
    return bool(lib().rt_device_checks_compiled())


def workspace_count() -> int:
    """Per-(device, stream) workspaces the library holds (each made by cudaMalloc)."""
    return int(lib().rt_workspace_count())


def release_stream(stream=None) -> None:
    """Frees the library's device workspace for `stream` (after its work ends)."""
    _check(lib().rt_stream_release(_stream_handle(stream)), "rt_stream_release")


def describe_pool_variant(v: int) -> tuple[int, int, int]:
    """-> (threads per block, minimum blocks per SM, stack entries per lane in shared memory)."""
    t, m, r = C.c_uint32(), C.c_uint32(), C.c_uint32()
    _check(lib().rt_pool_describe_variant(v, C.byref(t), C.byref(m), C.byref(r)), "rt_pool_describe_variant")
    return t.value, m.value, r.value


def build_bvh(triangles, spheres=None, models=None, bvh_mode: int = BVH_SORTED) -> np.ndarray:
    """Host BVH build alone (the six S1 passes) -> NODE_DTYPE array of 2N-1 nodes."""
    tri = np.ascontiguousarray(triangles, dtype=TRIANGLE_DTYPE)
    sph = np.ascontiguousarray(spheres, dtype=SPHERE_DTYPE) if spheres is not None else np.zeros(0, SPHERE_DTYPE)
    mod = np.ascontiguousarray(models, dtype=MODEL_DTYPE) if models is not None else None
    n = len(tri) + len(sph)
    out = np.zeros(max(2 * n - 1, 0), NODE_DTYPE)
    _check(lib().rt_build_bvh(_ptr(tri), len(tri), _ptr(sph), len(sph), _ptr(mod), 0 if mod is None else len(mod),
                              bvh_mode, _ptr(out)), "rt_build_bvh")
    return out


def build_bvh_sah(triangles, spheres=None, models=None) -> np.ndarray:
    """The binned-SAH traversal tree -> NODE_DTYPE array of 2N-1 nodes (root 0;
    not the reference's leaf layout)."""
    tri = np.ascontiguousarray(triangles, dtype=TRIANGLE_DTYPE)
    sph = np.ascontiguousarray(spheres, dtype=SPHERE_DTYPE) if spheres is not None else np.zeros(0, SPHERE_DTYPE)
    mod = np.ascontiguousarray(models, dtype=MODEL_DTYPE) if models is not None else None
    n = len(tri) + len(sph)
    out = np.zeros(max(2 * n - 1, 0), NODE_DTYPE)
    _check(lib().rt_build_bvh_sah(_ptr(tri), len(tri), _ptr(sph), len(sph), _ptr(mod),
                                  0 if mod is None else len(mod), _ptr(out)), "rt_build_bvh_sah")
    return out


def build_bvh_device(d_triangles, num_triangles: int, d_spheres=None, num_spheres: int = 0, d_nodes=None,
                     bvh_mode: int = BVH_SORTED, stream=None):
    """rt_build_bvh_device on device buffers (torch tensors); returns d_nodes."""
    _check(lib().rt_build_bvh_device(_ptr(d_triangles), num_triangles, _ptr(d_spheres), num_spheres, bvh_mode,
                                     _ptr(d_nodes), _stream_handle(stream)), "rt_build_bvh_device")
    return d_nodes


def load_obj(path, material: int = 0) -> np.ndarray:
    """Triangles of an OBJ file (positions, fan-triangulated faces, file order)."""
    cnt = C.c_uint64()
    _check(lib().rt_obj_load(str(path).encode(), material, None, 0, C.byref(cnt)), "rt_obj_load")
    out = np.zeros(cnt.value, TRIANGLE_DTYPE)
    _check(lib().rt_obj_load(str(path).encode(), material, _ptr(out), cnt.value, C.byref(cnt)), "rt_obj_load")
    return out


def model_matrix(translation=(0.0, 0.0, 0.0), rotation=(0.0, 0.0, 0.0), scale=(1.0, 1.0, 1.0)) -> np.ndarray:
    """TransformComponent::mat4 as a MODEL_DTYPE record (column-major)."""
    t = np.asarray(translation, np.float32)
    r = np.asarray(rotation, np.float32)
    s = np.asarray(scale, np.float32)
    out = np.zeros(1, MODEL_DTYPE)
    _check(lib().rt_model_matrix(_ptr(t), _ptr(r), _ptr(s), _ptr(out)), "rt_model_matrix")
    return out


def write_image(path, rgba: np.ndarray, width: int, height: int) -> None:
    """RGBA float image (host) to .ppm (8-bit) or .pfm (float)."""
    rgba = np.ascontiguousarray(rgba, dtype=np.float32)
    fn = lib().rt_write_pfm if str(path).endswith(".pfm") else lib().rt_write_ppm
    _check(fn(str(path).encode(), _ptr(rgba), width, height), "rt_write_image")


def accum_clear(accum, width: int, height: int, stream=None) -> None:
    _check(lib().rt_accum_clear(_ptr(accum), width, height, _stream_handle(stream)), "rt_accum_clear")


def resolve(accum, width: int, height: int, spp: int, out, stream=None) -> None:
    _check(lib().rt_resolve(_ptr(accum), width, height, spp, _ptr(out), _stream_handle(stream)), "rt_resolve")


# --------------------------------------------------------------- workloads
def gen_uniform(seed: int, stream: int, n: int) -> np.ndarray:
    out = np.empty(n, np.float64)
    _check(lib().rt_gen_uniform(seed, stream, n, _ptr(out)), "rt_gen_uniform")
    return out


def gen_icosphere(subdiv: int, center=(0.0, 0.0, 0.0), radius: float = 1.0, material: int = 0) -> np.ndarray:
    n = 20 * 4 ** subdiv
    out = np.zeros(n, TRIANGLE_DTYPE)
    c = (C.c_float * 3)(*center)
    cnt = C.c_uint64()
    _check(lib().rt_gen_icosphere(subdiv, C.cast(c, C.c_void_p), radius, material, _ptr(out), n, C.byref(cnt)),
           "rt_gen_icosphere")
    return out


def gen_config1():
    """-> (triangles[20482], ubo, rays[640*360])"""
    tris = np.zeros(20482, TRIANGLE_DTYPE)
    rays = np.zeros(640 * 360, RAY_DTYPE)
    ubo = RaytracingUBO()
    _check(lib().rt_gen_config1(_ptr(tris), C.byref(ubo), _ptr(rays)), "rt_gen_config1")
    return tris, ubo, rays


def gen_camera_rays(ubo: RaytracingUBO, width: int, height: int) -> np.ndarray:
    out = np.zeros(width * height, RAY_DTYPE)
    _check(lib().rt_gen_camera_rays(C.byref(ubo), width, height, _ptr(out)), "rt_gen_camera_rays")
    return out


def gen_soup(seed: int, stream: int, n: int, side: float = 1.0, sigma: float = 0.002, material: int = 0) -> np.ndarray:
    out = np.zeros(n, TRIANGLE_DTYPE)
    _check(lib().rt_gen_soup(seed, stream, n, side, sigma, material, _ptr(out)), "rt_gen_soup")
    return out


def gen_rays(seed: int, stream: int, n: int, side: float = 1.0, tmin: float = 1e-4,
             tmax: float = float("inf")) -> np.ndarray:
    out = np.zeros(n, RAY_DTYPE)
    _check(lib().rt_gen_rays(seed, stream, n, side, tmin, tmax, _ptr(out)), "rt_gen_rays")
    return out


def gen_spheres_scene(seed: int, count: int, subdiv: int, amp: float = 0.05):
    """-> (triangles, materials) of config 2's displaced icospheres."""
    tris = np.zeros(count * 20 * 4 ** subdiv, TRIANGLE_DTYPE)
    mats = np.zeros(count, MATERIAL_DTYPE)
    _check(lib().rt_gen_spheres_scene(seed, count, subdiv, amp, _ptr(tris), _ptr(mats)), "rt_gen_spheres_scene")
    return tris, mats


def make_ubo(cam_pos, look_at, up=(0.0, 1.0, 0.0), fov: float = 60.0, depth: int = 8, random_state: int = 0,
             num_triangles: int = 0, num_spheres: int = 0, num_materials: int = 0) -> RaytracingUBO:
    u = RaytracingUBO()
    u.camPos[:3] = list(cam_pos)
    u.camLookAt[:3] = list(look_at)
    u.camUpDir[:3] = list(up)
    u.verticalFOV = fov
    u.numTriangles, u.numSpheres, u.numMaterials = num_triangles, num_spheres, num_materials
    u.maxRayTraceDepth = depth
    u.randomState = random_state
    return u
