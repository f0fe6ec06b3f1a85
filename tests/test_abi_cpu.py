"""CPU checks of the product library: it loads, exports every declared entry
point, its host BVH builder equals the oracle's transcription byte for byte,
its workload generators are deterministic, and invalid input is rejected."""
import ctypes as C
import os
import re
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:rt_status|const char\s*\*|uint32_t)\s+(rt_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_every_declared_symbol_is_exported(rt):
    names = declared_functions()
    assert len(names) >= 20
    L = rt.lib()
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(rt.SIGNATURES) <= set(names)


def test_abi_version_and_record_sizes(rt):
    assert rt.lib().rt_abi_version() == 1
    assert C.sizeof(rt.RaytracingUBO) == 80
    assert rt.TRIANGLE_DTYPE.itemsize == 64 and rt.NODE_DTYPE.itemsize == 40


@pytest.mark.parametrize("mode", [0, 1])
def test_host_builder_matches_oracle(rt, orc, mode):
    tris, ubo, rays = rt.gen_config1()
    a = rt.build_bvh(tris, bvh_mode=mode)
    b, _, _, _ = orc.build_bvh(tris, mode=mode)
    assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
    soup = rt.gen_soup(4, 0, 300_000, 1.0, 0.002)
    sph = np.zeros(11, rt.SPHERE_DTYPE)
    sph["center"][:, :3] = np.random.default_rng(1).random((11, 3)).astype(np.float32)
    sph["radius"] = np.float32(0.01)
    a = rt.build_bvh(soup, sph, bvh_mode=mode)
    b, _, _, _ = orc.build_bvh(soup, sph, mode=mode)
    assert np.array_equal(a.view(np.uint8), b.view(np.uint8))


def test_host_builder_edge_cases(rt, orc):
    t = rt.gen_soup(3, 5, 64, 1.0, 0.01)
    for n in (1, 2, 3, 17):
        for mode in (0, 1):
            a = rt.build_bvh(t[:n], bvh_mode=mode)
            b, _, _, _ = orc.build_bvh(t[:n], mode=mode)
            assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
    same = np.repeat(t[:1], 1000)  # all codes equal: index tie-break of ConstructHLBVH.comp:64-68
    a = rt.build_bvh(same)
    b, _, _, _ = orc.build_bvh(same)
    assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
    assert len(rt.build_bvh(np.zeros(0, rt.TRIANGLE_DTYPE))) == 0


def test_host_builder_models(rt, orc):
    tris = rt.gen_icosphere(2, (0, 0, 0), 1.0, 0)
    tris["modelIndex"] = np.arange(len(tris)) % 2
    m = np.zeros(2, rt.MODEL_DTYPE)
    m0 = np.eye(4, dtype=np.float32)
    m1 = np.array([[0.5, -0.2, 0, 3], [0.1, 1.5, 0.3, -1], [0, 0.2, 2.0, 0.5], [0, 0, 0, 1]], np.float32)
    m[0]["m"] = m0.T.ravel()
    m[1]["m"] = m1.T.ravel()
    a = rt.build_bvh(tris, models=m)
    b, _, _, _ = orc.build_bvh(tris, mode=0, models=m["m"])
    assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
    bad = tris.copy()
    bad["modelIndex"][3] = 5
    with pytest.raises(rt.RtError):
        rt.build_bvh(bad, models=m)


def test_camera_rays_match_oracle(rt, orc):
    for pos, look, fov, w, h in [((0, 0.5, 4), (0, 0, 0), 60.0, 640, 360), ((275, 275, -800), (275, 275, 0), 40.0, 320, 200),
                                 ((1, 2, 3), (-1, 0.5, 0), 90.0, 33, 17)]:
        ubo = rt.make_ubo(pos, look, fov=fov)
        a = rt.gen_camera_rays(ubo, w, h)
        b = orc.primary_rays(ubo, w, h)
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8))


def test_generators_deterministic_across_thread_counts(rt):
    code = ("import sys, hashlib; sys.path.insert(0, %r); import raytracergpu_mastersproject_gb300 as rt;"
            "a = rt.gen_soup(3, 0, 200000); b = rt.gen_rays(3, 0, 300000);"
            "print(hashlib.sha256(a.tobytes() + b.tobytes()).hexdigest())") % str(ROOT)
    outs = []
    for th in ("1", "7"):
        env = dict(os.environ, RT_HOST_THREADS=th)
        r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, check=True)
        outs.append(r.stdout.strip())
    assert outs[0] == outs[1]


def test_generator_shapes(rt):
    tris, ubo, rays = rt.gen_config1()
    assert len(tris) == 20482 and len(rays) == 640 * 360
    assert ubo.verticalFOV == 60.0 and tuple(ubo.camPos[:3]) == (0.0, 0.5, 4.0)
    ico = rt.gen_icosphere(5)
    r = np.linalg.norm(np.stack([ico["v0"][:, :3], ico["v1"][:, :3], ico["v2"][:, :3]]).astype(np.float64), axis=-1)
    assert np.allclose(r, 1.0, atol=1e-6)
    rays = rt.gen_rays(3, 0, 100_000)
    d = np.linalg.norm(rays["dir"].astype(np.float64), axis=1)
    assert np.allclose(d, 1.0, atol=1e-6)
    assert rays["org"].min() >= 0 and rays["org"].max() < 1
    assert np.all(np.isinf(rays["tmax"])) and np.all(rays["tmin"] == np.float32(1e-4))
    soup = rt.gen_soup(3, 0, 100_000)
    c = (soup["v0"][:, :3] + soup["v1"][:, :3] + soup["v2"][:, :3]) / 3
    assert 0.45 < c.mean() < 0.55
    off = (soup["v1"][:, :3] - soup["v0"][:, :3]).astype(np.float64).std()
    assert abs(off - 0.002 * np.sqrt(2)) < 2e-4
    t2, m2 = rt.gen_spheres_scene(2, 4, 1)
    assert len(t2) == 4 * 80 and len(m2) == 4
    assert set(m2["materialType"]) <= {1, 2, 3}


def test_invalid_arguments_rejected_without_a_gpu(rt, orc):
    tris, ubo, rays = rt.gen_config1()
    with pytest.raises(rt.RtError) as e:
        rt.build_bvh(tris, bvh_mode=7)
    assert e.value.status == 1
    with pytest.raises(rt.RtError) as e:
        rt.Scene(tris, bvh_mode=3)
    assert e.value.status == 1
    with pytest.raises(rt.RtError) as e:
        rt.Scene(tris, leaf_size=9)
    assert e.value.status == 1
    nodes, _, _, _ = orc.build_bvh(tris, mode=0)
    with pytest.raises(rt.RtError) as e:
        rt.Scene(tris, nodes=nodes[:-1])
    assert e.value.status == 1
    cyc = nodes.copy()
    cyc[1]["left"] = 0  # node 0 reachable twice: not a tree
    with pytest.raises(rt.RtError) as e:
        rt.Scene(tris, nodes=cyc)
    assert e.value.status == 1 and "tree" in str(e.value)
    oob = nodes.copy()
    leaf = np.nonzero((oob["left"] == 0) & (oob["right"] == 0))[0][0]
    oob[leaf]["primitiveIndex"] = 10 ** 6
    with pytest.raises(rt.RtError) as e:
        rt.Scene(tris, nodes=oob)
    assert e.value.status == 1
    # a chain of depth > 127 cannot be traversed with the kernel's stack
    n = 200
    chain = np.zeros(2 * n - 1, rt.NODE_DTYPE)
    for i in range(n - 1):
        chain[i]["left"] = n - 1 + i
        chain[i]["right"] = i + 1 if i + 1 < n - 1 else 2 * n - 2
    for k in range(n):
        chain[n - 1 + k]["primitiveIndex"] = k
        chain[n - 1 + k]["primitiveType"] = 1
    for f in ("minX", "minY", "minZ"):
        chain[f] = -1
    for f in ("maxX", "maxY", "maxZ"):
        chain[f] = 1
    soup = rt.gen_soup(1, 1, n)
    with pytest.raises(rt.RtError) as e:
        rt.Scene(soup, nodes=chain)
    assert e.value.status == 4  # RT_ESTACK


def test_library_refuses_to_load_when_missing(tmp_path):
    code = ("import os, sys; os.environ['RT_GB300_LIB'] = %r; sys.path.insert(0, %r);"
            "import raytracergpu_mastersproject_gb300 as rt\n"
            "try:\n    rt.lib()\nexcept ImportError as e:\n    print('refused', e)\n") % (str(tmp_path / "none.so"), str(ROOT))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True)
    assert "refused" in r.stdout


def test_pool_admission_without_a_gpu(rt):
    """Admission and validation happen before any device work."""
    soup = rt.gen_soup(8, 0, 20_000)
    with rt.Pool(budget_bytes=1000) as pool:
        with pytest.raises(rt.RtError) as e:
            pool.add_scene(soup)
        assert e.value.status == 2 and "budget" in str(e.value)
        assert pool.info().num_scenes == 0 and pool.info().used_bytes == 0
    with rt.Pool() as pool:
        with pytest.raises(rt.RtError) as e:
            pool.add_scene(soup, bvh_mode=5)
        assert e.value.status == 1
        with pytest.raises(rt.RtError) as e:
            pool.trace([(0, None, None, 0)] * 9000)
        assert e.value.status == 1
    assert rt.describe_pool_variant(0) == (128, 10, 16)
    assert rt.describe_pool_variant(2) == (128, 12, 0)
