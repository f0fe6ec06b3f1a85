"""ctypes binding of the CPU oracle (oracle/rt_oracle.c).

TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's CPU
baseline load this as the checker.  The product library never does.
The reference has no tests, fixtures or golden vectors and its Vulkan/GLSL
path cannot run here; the oracle is pinned to the reference's own shaders
compiled for the host (oracle/ref_glsl.py, tests/test_ref_pin_cpu.py).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"

TRI = np.dtype([("v0", "<f4", 4), ("v1", "<f4", 4), ("v2", "<f4", 4), ("materialIndex", "<u4"),
                ("modelIndex", "<u4"), ("_pad", "<u4", 2)])
SPH = np.dtype([("center", "<f4", 4), ("radius", "<f4"), ("materialIndex", "<u4"), ("modelIndex", "<u4"),
                ("_pad", "<u4")])
MAT = np.dtype([("albedo", "<f4", 4), ("materialType", "<u4"), ("fuzz", "<f4"), ("ior", "<f4"), ("_pad", "<u4")])
NODE = np.dtype([("minX", "<f4"), ("maxX", "<f4"), ("minY", "<f4"), ("maxY", "<f4"), ("minZ", "<f4"),
                 ("maxZ", "<f4"), ("left", "<u4"), ("right", "<u4"), ("primitiveIndex", "<u4"),
                 ("primitiveType", "<u4")])
RAY = np.dtype([("org", "<f4", 3), ("tmin", "<f4"), ("dir", "<f4", 3), ("tmax", "<f4")])
HIT = np.dtype([("prim", "<u4"), ("t", "<f4")])
NO_HIT = 0xFFFFFFFF


class OScene(C.Structure):
    _fields_ = [("tris", C.c_void_p), ("nt", C.c_uint32), ("sph", C.c_void_p), ("ns", C.c_uint32),
                ("mats", C.c_void_p), ("nm", C.c_uint32), ("nodes", C.c_void_p), ("nn", C.c_uint32)]


_lib = None


def build() -> Path:
    newest = max((HERE / f).stat().st_mtime for f in ("rt_oracle.c", "rt_sincos.h", "build.sh"))
    if not LIB.exists() or LIB.stat().st_mtime < newest:
        subprocess.run(["sh", str(HERE / "build.sh")], check=True, capture_output=True)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        P, U, U64, F, D = C.c_void_p, C.c_uint32, C.c_uint64, C.c_float, C.c_double
        sig = {
            "orc_trace": (C.c_int, [C.POINTER(OScene), P, U, P, U, U, P]),
            "orc_render": (C.c_int, [C.POINTER(OScene), P, P, U, U, U, U, P, U, U, U]),
            "orc_resolve": (None, [P, U, U, U, P]),
            "orc_build_bvh": (C.c_int, [P, U, P, U, P, U, U, P, P, P, P]),
            "orc_karras": (None, [P, U, P, P]),
            "orc_separate_bits_by_3": (U, [U]),
            "orc_camera": (None, [P, U, U, P]),
            "orc_primary_rays": (None, [P, U, U, P]),
            "orc_random_stream": (None, [U, U, P, P]),
            "orc_random_unit_vectors": (None, [U, U, P]),
            "orc_seed": (U, [U, U, U]),
            "orc_step_rng": (U, [U]),
            "orc_sin": (F, [F]),
            "orc_cos": (F, [F]),
            "orc_triangle_test": (C.c_int, [P, P, F, C.POINTER(F)]),
            "orc_triangle_t64": (D, [P, P, C.POINTER(C.c_int)]),
            "orc_all_hits": (U, [C.POINTER(OScene), P, P, P, U]),
            "orc_gen_soup": (None, [U64, U64, U64, U, F, F, U, P]),
            "orc_gen_rays": (None, [U64, U64, U64, U, F, F, F, P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(a):
    if a is None or (isinstance(a, np.ndarray) and a.size == 0):
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


class Scene:
    """Arrays kept alive with the OScene that points at them."""

    def __init__(self, tris, nodes, spheres=None, mats=None):
        self.tris = np.ascontiguousarray(tris, dtype=TRI)
        self.nodes = np.ascontiguousarray(nodes, dtype=NODE)
        self.sph = np.ascontiguousarray(spheres if spheres is not None else np.zeros(0, SPH), dtype=SPH)
        self.mats = np.ascontiguousarray(mats if mats is not None else np.zeros(0, MAT), dtype=MAT)
        self.s = OScene(_p(self.tris), len(self.tris), _p(self.sph), len(self.sph), _p(self.mats), len(self.mats),
                        _p(self.nodes), len(self.nodes))


def threads() -> int:
    return int(os.environ.get("RT_ORACLE_THREADS", os.cpu_count() or 1))


def build_bvh(tris, spheres=None, mode: int = 0, models=None):
    """-> (nodes, sorted codes, sorted prims, enclosing box[6])"""
    tris = np.ascontiguousarray(tris, dtype=TRI)
    sph = np.ascontiguousarray(spheres if spheres is not None else np.zeros(0, SPH), dtype=SPH)
    n = len(tris) + len(sph)
    nodes = np.zeros(max(2 * n - 1, 0), NODE)
    codes = np.zeros(n, np.uint32)
    prims = np.zeros(n, np.uint32)
    enc = np.zeros(6, np.float32)
    mod = None if models is None else np.ascontiguousarray(models, dtype=np.float32).reshape(-1, 16)
    rc = lib().orc_build_bvh(_p(tris), len(tris), _p(sph), len(sph), _p(mod), 0 if mod is None else len(mod),
                             mode, _p(nodes), _p(codes), _p(prims), _p(enc))
    if rc != 0:
        raise ValueError(f"orc_build_bvh failed: {rc}")
    return nodes, codes, prims, enc


def trace(scene: Scene, rays, any_hit: bool = False, canonical: bool = False, nthreads: int | None = None,
          mt: bool = False):
    """-> (hits, stats[5]: boxes, tris, spheres, inner, status).  mt: the
    Moller-Trumbore triangle test (the library's RT_TRACE_MT) instead of the
    reference's plane test."""
    rays = np.ascontiguousarray(rays, dtype=RAY)
    hits = np.zeros(len(rays), HIT)
    stats = np.zeros(5, np.uint64)
    flags = (1 if any_hit else 0) | (2 if canonical else 0) | (4 if mt else 0)
    lib().orc_trace(C.byref(scene.s), _p(rays), len(rays), _p(hits), flags,
                    nthreads if nthreads is not None else threads(), _p(stats))
    return hits, stats


def render(scene: Scene, ubo, accum: np.ndarray, width: int, height: int, spp: int, extended: bool = False,
           background=(0.0, 0.0, 0.0), nthreads: int | None = None, rows: tuple[int, int] | None = None,
           canonical: bool = False) -> int:
    """accum: float32 [H*W*4], updated in place (only pixel rows
    rows[0]..rows[1]-1 when given); returns the status bits.  canonical: the
    culled near-first traversal (same hits except exact ties of t), for
    frames too large for the reference order."""
    assert accum.dtype == np.float32 and accum.flags["C_CONTIGUOUS"]
    bg = np.asarray(background, np.float32)
    y0, y1 = rows if rows is not None else (0, height)
    flags = (1 if extended else 0) | (2 if canonical else 0)
    return lib().orc_render(C.byref(scene.s), C.addressof(ubo), _p(accum), width, height, spp, flags,
                            _p(bg), nthreads if nthreads is not None else threads(), y0, y1)


def resolve(accum: np.ndarray, width: int, height: int, spp: int) -> np.ndarray:
    out = np.zeros(width * height * 4, np.float32)
    lib().orc_resolve(_p(accum), width, height, spp, _p(out))
    return out


def primary_rays(ubo, width: int, height: int) -> np.ndarray:
    out = np.zeros(width * height, RAY)
    lib().orc_primary_rays(C.addressof(ubo), width, height, _p(out))
    return out


def camera(ubo, width: int, height: int) -> np.ndarray:
    out = np.zeros(12, np.float32)
    lib().orc_camera(C.addressof(ubo), width, height, _p(out))
    return out


def random_stream(state: int, n: int):
    out = np.zeros(n, np.float32)
    st = np.zeros(n, np.uint32)
    lib().orc_random_stream(state, n, _p(out), _p(st))
    return out, st


def random_unit_vectors(state: int, n: int) -> np.ndarray:
    out = np.zeros(3 * n, np.float32)
    lib().orc_random_unit_vectors(state, n, _p(out))
    return out.reshape(n, 3)


def gen_soup(seed: int, stream: int, n: int, side: float = 1.0, sigma: float = 0.002, material: int = 0,
             first: int = 0) -> np.ndarray:
    """Triangles first..first+n-1 of the library's seeded soup generator."""
    out = np.zeros(n, TRI)
    lib().orc_gen_soup(seed, stream, first, n, side, sigma, material, _p(out))
    return out


def gen_rays(seed: int, stream: int, n: int, side: float = 1.0, tmin: float = 1e-4, tmax: float = float("inf"),
             first: int = 0) -> np.ndarray:
    """Rays first..first+n-1 of the library's seeded ray generator."""
    out = np.zeros(n, RAY)
    lib().orc_gen_rays(seed, stream, first, n, side, tmin, tmax, _p(out))
    return out


def karras(codes) -> tuple[np.ndarray, np.ndarray]:
    codes = np.ascontiguousarray(codes, dtype=np.uint32)
    n = len(codes)
    left = np.zeros(max(n - 1, 0), np.uint32)
    right = np.zeros(max(n - 1, 0), np.uint32)
    lib().orc_karras(_p(codes), n, _p(left), _p(right))
    return left, right


def triangle_test(tri, ray, tmax=None):
    """Reference binary32 test of one triangle record against one ray -> t or None."""
    tri = np.ascontiguousarray(tri, dtype=TRI).reshape(1)
    ray = np.ascontiguousarray(ray, dtype=RAY).reshape(1)
    t = C.c_float()
    tm = float(ray["tmax"][0]) if tmax is None else tmax
    ok = lib().orc_triangle_test(_p(tri), _p(ray), tm, C.byref(t))
    return t.value if ok else None


def triangle_t64(tri, ray):
    """Binary64 plane parameter and inside flag -> (t, inside)."""
    tri = np.ascontiguousarray(tri, dtype=TRI).reshape(1)
    ray = np.ascontiguousarray(ray, dtype=RAY).reshape(1)
    inside = C.c_int()
    t = lib().orc_triangle_t64(_p(tri), _p(ray), C.byref(inside))
    return t, bool(inside.value)


def all_hits(scene: Scene, ray, cap: int = 64):
    ray = np.ascontiguousarray(ray, dtype=RAY).reshape(1)
    ids = np.zeros(cap, np.uint32)
    ts = np.zeros(cap, np.float32)
    n = lib().orc_all_hits(C.byref(scene.s), _p(ray), _p(ids), _p(ts), cap)
    return ids[:min(n, cap)], ts[:min(n, cap)]


def arbitrate(tris, rays, ref_hits, gpu_hits, rel: float = 1e-6) -> dict:
    """Classifies every ray whose GPU hit differs from the oracle's.

    A difference is accepted (near-tie, arbitrated in binary64) when both
    candidates pass the reference's binary32 triangle test and the GPU's
    candidate is not farther than the oracle's in binary64 beyond `rel`.
    Returns counts and the indices of unexplained differences.
    """
    tris = np.ascontiguousarray(tris, dtype=TRI)
    diff = np.nonzero(ref_hits["prim"] != gpu_hits["prim"])[0]
    out = {"mismatch": int(len(diff)), "near_tie": 0, "gpu_closer": 0, "unexplained": []}
    for i in diff:
        r, g = int(ref_hits["prim"][i]), int(gpu_hits["prim"][i])
        if r == NO_HIT or g == NO_HIT or (r & 0x80000000) or (g & 0x80000000):
            out["unexplained"].append(int(i))
            continue
        ray = rays[i:i + 1]
        tr = triangle_test(tris[r], ray)
        tg = triangle_test(tris[g], ray)
        if tr is None or tg is None:
            out["unexplained"].append(int(i))
            continue
        t64r, _ = triangle_t64(tris[r], ray)
        t64g, _ = triangle_t64(tris[g], ray)
        if abs(t64g - t64r) <= rel * abs(t64r) or abs(tg - tr) <= rel * abs(tr):
            out["near_tie"] += 1
        elif t64g <= t64r:
            out["gpu_closer"] += 1
        else:
            out["unexplained"].append(int(i))
    return out
