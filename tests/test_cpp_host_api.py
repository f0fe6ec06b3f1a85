"""The C++ host interface (include/rt_gb300.hpp): compiled with g++ against
the library; its flattening matches RaytraceScene's rules on the CPU, and its
frame matches the Python path bit for bit on the GPU."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def exe(rt, tmp_path_factory):
    out = tmp_path_factory.mktemp("cpp") / "host_api_test"
    pkg = ROOT / "raytracergpu_mastersproject_gb300"
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", str(ROOT / "include"),
           str(ROOT / "tests" / "cpp" / "host_api_test.cpp"), "-o", str(out), "-L", str(pkg), "-lrt_gb300",
           f"-Wl,-rpath,{pkg}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def python_scene(rt):
    ico = rt.gen_icosphere(2, (0, 0, 0), 1.0, 0)
    quad = np.zeros(2, rt.TRIANGLE_DTYPE)
    q = [(-1, 0, -1), (1, 0, -1), (1, 0, 1), (-1, 0, 1)]
    for t, (a, b, c) in enumerate([(0, 1, 2), (0, 2, 3)]):
        quad[t]["v0"][:3], quad[t]["v1"][:3], quad[t]["v2"][:3] = q[a], q[b], q[c]
    ico["materialIndex"], ico["modelIndex"] = 0, 0
    quad["materialIndex"], quad["modelIndex"] = 1, 1
    tris = np.concatenate([ico, quad])
    sph = np.zeros(1, rt.SPHERE_DTYPE)
    sph["radius"], sph["materialIndex"], sph["modelIndex"] = 0.5, 2, 2
    mats = np.zeros(3, rt.MATERIAL_DTYPE)
    for i, (alb, ty) in enumerate([((0.73, 0.33, 0.25), 1), ((3.0, 3.0, 3.0), 0), ((0.2, 0.6, 0.3), 1)]):
        mats[i]["albedo"][:3], mats[i]["materialType"], mats[i]["ior"] = alb, ty, 1.5
    models = np.concatenate([rt.model_matrix((0, 0.1, 0), (0, 0.4, 0)),
                             rt.model_matrix((0, -1.0, 0), (0, 0, 0), (10.0, 1.0, 10.0)),
                             rt.model_matrix((1.5, 0, 0.5))])
    return tris, sph, mats, models


def test_cpp_flattening_on_cpu(rt, exe):
    r = subprocess.run([str(exe), "cpu"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    words = r.stdout.split()
    assert words[:8] == ["models", "3", "triangles", "322", "spheres", "1", "materials", "3"]
    tris, sph, mats, models = python_scene(rt)
    chk = float(np.sum(tris["v0"][:, 0].astype(np.float64) + 2.0 * tris["v1"][:, 1] + 3.0 * tris["v2"][:, 2]
                       + tris["modelIndex"]))
    assert abs(float(words[9]) - chk) < 1e-3
    assert "handle-before-prep-throws 1" in r.stdout


@pytest.mark.gpu
def test_cpp_frame_matches_python(rt, exe, cuda, tmp_path):
    out = tmp_path / "acc.bin"
    r = subprocess.run([str(exe), "gpu", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr + r.stdout
    acc = np.fromfile(out, np.float32)
    tris, sph, mats, models = python_scene(rt)
    ubo = rt.make_ubo((0.0, 0.5, 4.0), (0.0, 0.0, 0.0), fov=60.0, depth=4, random_state=77)
    with rt.Scene(tris, spheres=sph, materials=mats, models=models) as sc:
        d = cuda.empty(64 * 36 * 4, dtype=cuda.float32, device="cuda")
        rt.accum_clear(d, 64, 36)
        sc.render(ubo, d, 64, 36, 3)
        cuda.cuda.synchronize()
        ref = d.cpu().numpy()
    assert np.array_equal(acc.view(np.uint32), ref.view(np.uint32))
    assert acc[0::4].max() > 0.1
    assert (tmp_path / "acc.bin.ppm").read_bytes().startswith(b"P6\n64 36\n255\n")
