"""The quantised 4-wide node encoding, checked on the CPU by a C++ program
linked against the library (tests/cpp/wide_nodes_test.cpp): for scenes at
awkward scales and offsets (1e-40 to 1e17, flat, tiny boxes far from 0),
every child slot's planes enclose its primitives exactly, and the kernels'
node-visit arithmetic, restated op for op in binary32, keeps every point of
a child box on a ray inside the interval it computes."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def exe(rt, tmp_path_factory):
    from raytracergpu_mastersproject_gb300 import _build
    cuda_inc = Path(_build.nvcc()).resolve().parent.parent / "include"
    pkg = ROOT / "raytracergpu_mastersproject_gb300"
    out = tmp_path_factory.mktemp("wide") / "wide_nodes_test"
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-Wall",
           "-I", str(ROOT / "include"), "-I", str(pkg / "csrc"), "-I", str(cuda_inc),
           str(ROOT / "tests" / "cpp" / "wide_nodes_test.cpp"), "-o", str(out), "-L", str(pkg), "-lrt_gb300",
           f"-Wl,-rpath,{pkg}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_wide_node_encoding_and_visit_are_conservative(exe):
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = r.stdout.splitlines()
    names = [ln.split()[1] for ln in lines if ln.startswith("ok ")]
    assert names == ["unit-soup", "offset-1e7", "tiny-at-1", "flat-z", "huge-1e17", "signed", "subnormal",
                     "wide-1e9", "wide-1e17"], r.stdout
