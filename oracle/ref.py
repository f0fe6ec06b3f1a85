"""ctypes binding of the reference's own compute shaders compiled for the host
(oracle/_ref/libref_glsl*.so, built by oracle/ref_glsl.py).

TEST INFRASTRUCTURE ONLY: tests/ use it to pin the oracle to the reference,
and bench.py's reference arm times `trace` (the reference's hitBVH) on the
host cores.  `available()` is False where neither the reference checkout nor
previously generated sources exist.

Two builds: `portable=True` (default) evaluates the shaders' sin/cos with the
oracle's portable binary32 functions, under which the oracle must agree bit
for bit; `portable=False` uses libm's sinf/cosf.
"""
from __future__ import annotations

import ctypes as C
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
if str(HERE.parent) not in sys.path:
    sys.path.insert(0, str(HERE.parent))

from oracle import oracle as orc  # noqa: E402

_libs: dict[bool, C.CDLL] = {}
_built: list[Path] | None = None


def build() -> list[Path]:
    global _built
    if _built is None:
        r = subprocess.run([sys.executable, str(HERE / "ref_glsl.py")], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle/ref_glsl.py failed:\n{r.stdout}\n{r.stderr}")
        _built = [p for p in (HERE / "_ref" / n for n in ("libref_glsl.so", "libref_glsl_portable.so")) if p.exists()]
    return _built


def available() -> bool:
    return len(build()) == 2


def lib(portable: bool = True) -> C.CDLL:
    if portable not in _libs:
        if not available():
            raise RuntimeError("the reference's shaders are not available to compile")
        L = C.CDLL(str(HERE / "_ref" / ("libref_glsl_portable.so" if portable else "libref_glsl.so")))
        P, U, F = C.c_void_p, C.c_uint32, C.POINTER(C.c_float)
        sig = {
            "ref_trace": (C.c_int, [P, U, P, U, P, U, P, U, P, U]),
            "ref_render": (C.c_int, [P, P, U, U, U, P, U, P, U, P, U, P, U, U]),
            "ref_camera": (None, [P, U, U, P]),
            "ref_get_rays": (None, [P, U, U, P]),
            "ref_seed": (U, [U, U, U]),
            "ref_random_stream": (None, [U, U, P, P]),
            "ref_random_unit_vectors": (None, [U, U, P]),
            "ref_build_bvh": (C.c_int, [P, U, P, U, P, U, P, P, P, P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _libs[portable] = L
    return _libs[portable]


_p = orc._p


def trace(scene: "orc.Scene", rays, nthreads: int | None = None, portable: bool = True) -> np.ndarray:
    """hitBVH (raytraceBVH.comp:195-265) on every ray with its own interval,
    over the scene's reference-layout node array -> HIT records."""
    rays = np.ascontiguousarray(rays, dtype=orc.RAY)
    hits = np.zeros(len(rays), orc.HIT)
    rc = lib(portable).ref_trace(_p(scene.nodes), len(scene.nodes), _p(scene.tris), len(scene.tris),
                                 _p(scene.sph), len(scene.sph), _p(rays), len(rays), _p(hits),
                                 nthreads if nthreads is not None else orc.threads())
    if rc != 0:
        raise ValueError(f"ref_trace failed: {rc}")
    return hits


def render(scene: "orc.Scene", ubo, accum: np.ndarray, width: int, height: int, spp: int,
           nthreads: int | None = None, portable: bool = True) -> None:
    """spp dispatches of raytraceBVH.comp's main() over accum (float32
    [H*W*4], updated in place)."""
    assert accum.dtype == np.float32 and accum.flags["C_CONTIGUOUS"] and accum.size == width * height * 4
    mats = scene.mats if len(scene.mats) else np.zeros(1, orc.MAT)
    sph = scene.sph if len(scene.sph) else np.zeros(1, orc.SPH)
    lib(portable).ref_render(C.addressof(ubo), _p(accum), width, height, spp, _p(scene.tris), len(scene.tris),
                             _p(sph), len(scene.sph), _p(mats), len(scene.mats), _p(scene.nodes),
                             len(scene.nodes), nthreads if nthreads is not None else orc.threads())


def camera(ubo, width: int, height: int) -> np.ndarray:
    out = np.zeros(12, np.float32)
    lib().ref_camera(C.addressof(ubo), width, height, _p(out))
    return out


def get_rays(ubo, width: int, height: int) -> np.ndarray:
    out = np.zeros(width * height, orc.RAY)
    lib().ref_get_rays(C.addressof(ubo), width, height, _p(out))
    return out


def seed(x: int, y: int, random_state: int) -> int:
    return int(lib().ref_seed(x, y, random_state))


def random_stream(state: int, n: int):
    out = np.zeros(n, np.float32)
    st = np.zeros(n, np.uint32)
    lib().ref_random_stream(state, n, _p(out), _p(st))
    return out, st


def random_unit_vectors(state: int, n: int, portable: bool = True) -> np.ndarray:
    out = np.zeros(3 * n, np.float32)
    lib(portable).ref_random_unit_vectors(state, n, _p(out))
    return out.reshape(n, 3)


def build_bvh(tris, spheres=None, models=None):
    """The six S1 passes of the reference -> (nodes, sorted codes, sorted
    prims (index | 0x80000000 for spheres), enclosing box[6]).  models:
    column-major 4x4 matrices (identity when None)."""
    tris = np.ascontiguousarray(tris, dtype=orc.TRI)
    sph = np.ascontiguousarray(spheres if spheres is not None else np.zeros(0, orc.SPH), dtype=orc.SPH)
    mod = np.eye(4, dtype=np.float32).reshape(1, 16) if models is None else \
        np.ascontiguousarray(models, dtype=np.float32).reshape(-1, 16)
    n = len(tris) + len(sph)
    nodes = np.zeros(max(2 * n - 1, 0), orc.NODE)
    codes = np.zeros(n, np.uint32)
    prims = np.zeros(n, np.uint32)
    enc = np.zeros(6, np.float32)
    rc = lib().ref_build_bvh(_p(tris), len(tris), _p(sph), len(sph), _p(mod), len(mod), _p(nodes), _p(codes),
                             _p(prims), _p(enc))
    if rc != 0:
        raise ValueError(f"ref_build_bvh failed: {rc}")
    return nodes, codes, prims, enc
