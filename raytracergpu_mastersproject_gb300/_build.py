"""Build recipe for the native library (in-tree, no cmake).

Compiles every source under csrc/ with nvcc for sm_103a in parallel and links
librt_gb300.so next to this file.  Host C++ is compiled with
-ffp-contract=off and device code with -fmad=false: the binary32 arithmetic
of the reference's shader expressions is reproduced one rounding per
operation on both sides.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
BUILD = PKG / "_build"
LIB = PKG / "librt_gb300.so"
# The checked build: device-side index checks (RT_DEVICE_CHECKS=1).
BUILD_CHECKED = PKG / "_build_checked"
LIB_CHECKED = PKG / "librt_gb300_checked.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "--expt-relaxed-constexpr",
          "-Xcompiler", "-fPIC,-pthread,-ffp-contract=off,-fno-fast-math",
          f"-I{INCLUDE}", f"-I{CSRC}"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build librt_gb300.so")


def sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _stale(lib: Path, deps: list[Path]) -> bool:
    if not lib.exists():
        return True
    t = lib.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None,
          checked: bool = False) -> Path:
    """Compiles and links librt_gb300.so (librt_gb300_checked.so with the
    device-side index checks when `checked`); returns its path."""
    lib_path, bdir = (LIB_CHECKED, BUILD_CHECKED) if checked else (LIB, BUILD)
    srcs = sources()
    deps = srcs + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h")) + [Path(__file__)]
    if not force and not _stale(lib_path, deps):
        return lib_path
    bdir.mkdir(exist_ok=True)
    cc = nvcc()
    flags = COMMON + ARCH + list(extra_flags or []) + (["-DRT_DEVICE_CHECKS=1"] if checked else [])

    def compile_one(src: Path) -> Path:
        obj = bdir / (src.name + ".o")
        cmd = [cc, *flags, "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = lib_path.with_suffix(".so.tmp")
    cmd = [cc, "-shared", *ARCH, "-Xcompiler", "-pthread", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, checked="--checked" in sys.argv))
