"""GPU parity of the path-tracing pass (rt_render) against the CPU oracle.

rt_render runs spp samples of raytraceBVH.comp:main per pixel with the
reference RNG (random.glsl) and its alpha-channel carry; images must agree
with the oracle within per-pixel RMSE 1e-3 at identical RNG streams.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def lit_scene(rt):
    sph = rt.gen_icosphere(3, (0.0, 0.0, 0.0), 1.0, 0)
    ground = rt.gen_config1()[0][-2:]
    tris = np.concatenate([sph, ground])
    mats = np.zeros(2, rt.MATERIAL_DTYPE)
    mats[0]["albedo"][:3] = (0.73, 0.33, 0.25)
    mats[0]["materialType"] = rt.MAT_DIFFUSE
    mats[1]["albedo"][:3] = (3.0, 3.0, 3.0)
    mats[1]["materialType"] = rt.MAT_LIGHT
    return tris, mats


def gpu_render(rt, torch, scene, ubo, w, h, spp, calls=1, **kw):
    acc = torch.empty(w * h * 4, dtype=torch.float32, device="cuda")
    rt.accum_clear(acc, w, h)
    for _ in range(calls):
        scene.render(ubo, acc, w, h, spp, **kw)
    torch.cuda.synchronize()
    return acc.cpu().numpy()


def oracle_render(orc, tris, nodes, mats, ubo, w, h, spp, spheres=None, **kw):
    acc = np.tile(np.array([0, 0, 0, 1], np.float32), w * h)
    status = orc.render(orc.Scene(tris, nodes, spheres=spheres, mats=mats), ubo, acc, w, h, spp, **kw)
    assert status == 0
    return acc


def rmse(a, b):
    return float(np.sqrt(np.mean((a.astype(np.float64) - b.astype(np.float64)) ** 2)))


@pytest.mark.parametrize("width", [2, 4])
@pytest.mark.parametrize("mode", [0, 1], ids=["sorted", "reference"])
def test_reference_shading(rt, orc, cuda, mode, width):
    tris, mats = lit_scene(rt)
    ubo = rt.make_ubo((0.0, 0.5, 4.0), (0.0, 0.0, 0.0), fov=60.0, depth=5, random_state=12345)
    w, h, spp = 96, 54, 4
    with rt.Scene(tris, materials=mats, bvh_mode=mode, node_width=width) as sc:
        img = gpu_render(rt, cuda, sc, ubo, w, h, spp)
        ref = oracle_render(orc, tris, sc.nodes(), mats, ubo, w, h, spp)
    assert rmse(img, ref) <= 1e-3
    assert np.mean(img == ref) > 0.99  # bit-identical except pixels whose paths met a near-tie
    assert img[0::4].max() > 0.1       # the light reaches the camera


def test_config2_frame(rt, orc, cuda):
    """Config 2's own frame, built as the bench builds it: 64 displaced
    subdiv-6 icospheres (5,242,880 triangles) with lambertian, metal and glass
    materials, camera (0,3,28) -> 0, FOV 40, 1280x720, 16 spp, depth 8.  Both
    shadings, with the first hit shared by a pixel's samples (the default) and
    with every sample's primary ray traced, against the oracle's whole frame
    (raytraceBVH.comp:276-315, 345-375 in the reference's traversal order)."""
    tris, mats = rt.gen_spheres_scene(2, 64, 6, 0.05)
    assert len(tris) == 5_242_880
    w, h, spp = 1280, 720, 16
    ubo = rt.make_ubo((0.0, 3.0, 28.0), (0.0, 0.0, 0.0), fov=40.0, depth=8, random_state=2,
                      num_triangles=len(tris), num_materials=len(mats))
    bg = (0.6, 0.7, 1.0)
    with rt.Scene(tris, materials=mats) as sc:
        nodes = sc.nodes()
        for mode, ext in ((rt.SHADE_EXTENDED, True), (rt.SHADE_REFERENCE, False)):
            imgs = [gpu_render(rt, cuda, sc, ubo, w, h, spp, shade_mode=mode, background=bg,
                               trace_every_primary=every) for every in (False, True)]
            ref = oracle_render(orc, tris, nodes, mats, ubo, w, h, spp, extended=ext, background=bg)
            assert np.array_equal(imgs[0], imgs[1])  # sharing the first hit changes nothing
            img = imgs[0]
            assert rmse(img, ref) <= 1e-3
            assert np.mean(np.all(img.reshape(-1, 4) == ref.reshape(-1, 4), axis=1)) > 0.98
            assert np.array_equal(img[3::4].view(np.uint32), ref[3::4].view(np.uint32))  # alpha RNG carry
            if ext:
                assert img[0::4].mean() / spp > 0.2  # sky and lit spheres, not a black frame


def test_samples_split_across_calls(rt, cuda):
    """Alpha carries the RNG between samples (raytraceBVH.comp:350-372), so
    two calls of 2 samples equal one call of 4."""
    tris, mats = lit_scene(rt)
    ubo = rt.make_ubo((0.0, 0.5, 4.0), (0.0, 0.0, 0.0), fov=60.0, depth=4, random_state=99)
    with rt.Scene(tris, materials=mats) as sc:
        a = gpu_render(rt, cuda, sc, ubo, 64, 36, 4)
        b = gpu_render(rt, cuda, sc, ubo, 64, 36, 2, calls=2)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("width", [2, 4])
def test_extended_materials_and_spheres(rt, orc, cuda, width):
    tris, mats = rt.gen_spheres_scene(21, 6, 2, 0.05)
    ground = rt.gen_config1()[0][-2:].copy()
    ground["v0"][:, 1] = ground["v1"][:, 1] = ground["v2"][:, 1] = -9.0
    ground["materialIndex"] = len(mats)
    lam = np.zeros(1, rt.MATERIAL_DTYPE)
    lam["albedo"][0][:3] = (0.5, 0.5, 0.5)
    lam["materialType"] = rt.MAT_DIFFUSE
    sph = np.zeros(2, rt.SPHERE_DTYPE)
    sph["center"][:, :3] = [(0.0, 0.0, 0.0), (3.0, 1.0, 2.0)]
    sph["radius"] = [1.5, 1.0]
    sph["materialIndex"] = [len(mats) + 1, 2]
    glass = np.zeros(1, rt.MATERIAL_DTYPE)
    glass["albedo"][0][:3] = 1.0
    glass["materialType"] = rt.MAT_DIELECTRIC
    glass["ior"] = 1.5
    allm = np.concatenate([mats, lam, glass])
    allt = np.concatenate([tris, ground])
    ubo = rt.make_ubo((0.0, 3.0, 28.0), (0.0, 0.0, 0.0), fov=40.0, depth=8, random_state=7)
    w, h, spp = 80, 45, 3
    bg = (0.6, 0.7, 1.0)
    with rt.Scene(allt, spheres=sph, materials=allm, node_width=width) as sc:
        img = gpu_render(rt, cuda, sc, ubo, w, h, spp, shade_mode=rt.SHADE_EXTENDED, background=bg)
        ref = oracle_render(orc, allt, sc.nodes(), allm, ubo, w, h, spp, spheres=sph, extended=True, background=bg)
        img_ref_mode = gpu_render(rt, cuda, sc, ubo, w, h, spp)
        ref_ref_mode = oracle_render(orc, allt, sc.nodes(), allm, ubo, w, h, spp, spheres=sph)
    assert rmse(img, ref) <= 1e-3
    assert np.mean(img == ref) > 0.99
    assert rmse(img_ref_mode, ref_ref_mode) <= 1e-3
    assert img[0::4].max() > 0.1


def test_resolve_and_clear(rt, orc, cuda):
    tris, mats = lit_scene(rt)
    ubo = rt.make_ubo((0.0, 0.5, 4.0), (0.0, 0.0, 0.0), depth=3, random_state=3)
    w, h, spp = 48, 27, 2
    with rt.Scene(tris, materials=mats) as sc:
        acc = cuda.empty(w * h * 4, dtype=cuda.float32, device="cuda")
        rt.accum_clear(acc, w, h)
        cleared = acc.cpu().numpy().reshape(-1, 4)
        assert np.all(cleared == np.array([0, 0, 0, 1], np.float32))
        sc.render(ubo, acc, w, h, spp)
        out = cuda.empty_like(acc)
        rt.resolve(acc, w, h, spp, out)
        cuda.cuda.synchronize()
        ref = orc.resolve(acc.cpu().numpy(), w, h, spp)
    assert np.array_equal(out.cpu().numpy(), ref)


def test_render_rejects_bad_material(rt, cuda):
    tris, mats = lit_scene(rt)
    ubo = rt.make_ubo((0.0, 0.5, 4.0), (0.0, 0.0, 0.0))
    with rt.Scene(tris, materials=mats[:1]) as sc:
        acc = cuda.empty(16 * 9 * 4, dtype=cuda.float32, device="cuda")
        with pytest.raises(rt.RtError) as e:
            sc.render(ubo, acc, 16, 9, 1)
        assert e.value.status == 1


def test_golden_accumulator_on_gpu(rt, cuda):
    from pathlib import Path

    g = np.load(Path(__file__).resolve().parent / "golden" / "small_scene.npz")
    tris = g["tris"].view(rt.TRIANGLE_DTYPE)
    mats = g["mats"].view(rt.MATERIAL_DTYPE)
    ubo = rt.RaytracingUBO.from_buffer_copy(g["ubo"].tobytes())
    w, h, spp = (int(v) for v in g["render_wh_spp"])
    with rt.Scene(tris, materials=mats) as sc:
        img = gpu_render(rt, cuda, sc, ubo, w, h, spp)
    assert rmse(img, g["accum"]) <= 1e-3


@pytest.mark.parametrize("mode", ["reference", "extended"])
def test_step_render_matches_per_pixel_render(rt, cuda, mode):
    """4-wide trees render with the per-lane step kernel, binary trees with
    one thread per pixel and whole traversals.  Hits do not depend on the
    traversal, and each pixel's samples are summed in order by both, so the
    accumulators are bit-identical."""
    tris, mats = rt.gen_spheres_scene(2, 64, 3, 0.05)
    ubo = rt.make_ubo((0.0, 3.0, 28.0), (0.0, 0.0, 0.0), fov=40.0, depth=8, random_state=2,
                      num_triangles=len(tris), num_materials=len(mats))
    w, h, spp = 160, 90, 4
    kw = {"shade_mode": rt.SHADE_EXTENDED, "background": (0.6, 0.7, 1.0)} if mode == "extended" else {}
    with rt.Scene(tris, materials=mats, node_width=2) as s2, rt.Scene(tris, materials=mats, node_width=4) as s4:
        a = gpu_render(rt, cuda, s2, ubo, w, h, spp, **kw)
        b = gpu_render(rt, cuda, s4, ubo, w, h, spp, **kw)
        c = gpu_render(rt, cuda, s4, ubo, w, h, 1, calls=spp, **kw)
    assert np.array_equal(a, b)
    assert np.array_equal(b, c)
    if mode == "extended":
        assert a[0::4].max() > 0.1


def test_depth_zero_advances_rng_only(rt, cuda):
    """maxRayTraceDepth 0: rayColor returns black, but every sample still
    advances the alpha carry (raytraceBVH.comp:350-372)."""
    tris, mats = lit_scene(rt)
    ubo = rt.make_ubo((0.0, 0.5, 4.0), (0.0, 0.0, 0.0), depth=0, random_state=5)
    with rt.Scene(tris, materials=mats, node_width=2) as s2, rt.Scene(tris, materials=mats, node_width=4) as s4:
        a = gpu_render(rt, cuda, s2, ubo, 40, 20, 3)
        b = gpu_render(rt, cuda, s4, ubo, 40, 20, 3)
    assert np.array_equal(a, b)
    px = a.reshape(-1, 4)
    assert np.all(px[:, :3] == 0.0)
    assert np.all(px[:, 3] != 1.0)


def test_render_count_matches_render(rt, cuda):
    """rt_render_count renders the same frame as rt_render and counts one
    closest-hit query per traced bounce; both kernels count the same queries."""
    tris, mats = rt.gen_spheres_scene(2, 64, 3, 0.05)
    ubo = rt.make_ubo((0.0, 3.0, 28.0), (0.0, 0.0, 0.0), fov=40.0, depth=8, random_state=2,
                      num_triangles=len(tris), num_materials=len(mats))
    w, h, spp = 96, 54, 2
    kw = {"shade_mode": rt.SHADE_EXTENDED, "background": (0.6, 0.7, 1.0)}
    counts = {}
    for width in (2, 4):
        with rt.Scene(tris, materials=mats, node_width=width) as sc:
            a = gpu_render(rt, cuda, sc, ubo, w, h, spp, **kw)
            for every in (False, True):
                acc = cuda.empty(w * h * 4, dtype=cuda.float32, device="cuda")
                rt.accum_clear(acc, w, h)
                counts[width, every] = sc.render_count(ubo, acc, w, h, spp, trace_every_primary=every, **kw)
                cuda.cuda.synchronize()
                assert np.array_equal(acc.cpu().numpy(), a)
    q2, n2, p2 = counts[2, True]
    q4, n4, p4 = counts[4, True]
    assert counts[2, False] == counts[2, True]  # the per-pixel kernel traces every primary ray
    assert q2 == q4
    assert w * h * spp <= q4 <= w * h * spp * 8
    assert n4 > 0 and p4 > 0 and n2 > n4
    # sharing the first hit saves exactly one query per pixel and later sample
    assert counts[4, False][0] == q4 - w * h * (spp - 1)


def test_shared_first_hit_is_exact(rt, cuda):
    """Samples 1.. of a pixel reuse sample 0's first hit (the camera has no
    jitter); the frame equals the one that traces every primary ray."""
    tris, mats = rt.gen_spheres_scene(5, 16, 3, 0.05)
    ubo = rt.make_ubo((0.0, 3.0, 28.0), (0.0, 0.0, 0.0), fov=40.0, depth=6, random_state=11,
                      num_triangles=len(tris), num_materials=len(mats))
    w, h = 120, 68
    for kw in ({}, {"shade_mode": rt.SHADE_EXTENDED, "background": (0.6, 0.7, 1.0)}):
        with rt.Scene(tris, materials=mats, node_width=4) as sc:
            a = gpu_render(rt, cuda, sc, ubo, w, h, 5, **kw)
            b = gpu_render(rt, cuda, sc, ubo, w, h, 5, trace_every_primary=True, **kw)
            c = gpu_render(rt, cuda, sc, ubo, w, h, 1, calls=5, **kw)
        assert np.array_equal(a, b)
        assert np.array_equal(a, c)


@pytest.mark.parametrize("paths", ["777", "4"])
def test_wavefront_passes_match(rt, cuda, tmp_path, paths):
    """The wavefront renderer splits a frame into pixel chunks when its paths
    do not fit the scratch, alternating two scratch halves and two streams:
    room for 777 paths gives chunks of 43 pixels x 9 samples; room for 4 gives
    one pixel at a time in sample passes of 2, 2, 2, 2 and 1 (the alpha carry
    links the passes).  The frame is unchanged either way (the reference frame
    here, 13,833 paths, runs as one chunk on one stream)."""
    import os
    import subprocess
    import sys

    tris, mats = lit_scene(rt)
    ubo = rt.make_ubo((0.0, 0.5, 4.0), (0.0, 0.0, 0.0), fov=60.0, depth=5, random_state=77)
    w, h = 53, 29
    with rt.Scene(tris, materials=mats, node_width=4) as sc:
        a = gpu_render(rt, cuda, sc, ubo, w, h, 9, shade_mode=rt.SHADE_EXTENDED, background=(0.3, 0.4, 0.5))
    np.save(tmp_path / "a.npy", a)
    code = f"""
import numpy as np, torch, sys
sys.path.insert(0, {repr(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))})
import raytracergpu_mastersproject_gb300 as rt
sph = rt.gen_icosphere(3, (0.0, 0.0, 0.0), 1.0, 0)
tris = np.concatenate([sph, rt.gen_config1()[0][-2:]])
mats = np.zeros(2, rt.MATERIAL_DTYPE)
mats[0]["albedo"][:3] = (0.73, 0.33, 0.25); mats[0]["materialType"] = rt.MAT_DIFFUSE
mats[1]["albedo"][:3] = (3.0, 3.0, 3.0); mats[1]["materialType"] = rt.MAT_LIGHT
ubo = rt.make_ubo((0.0, 0.5, 4.0), (0.0, 0.0, 0.0), fov=60.0, depth=5, random_state=77)
acc = torch.empty({w} * {h} * 4, dtype=torch.float32, device="cuda")
rt.accum_clear(acc, {w}, {h})
with rt.Scene(tris, materials=mats, node_width=4) as sc:
    sc.render(ubo, acc, {w}, {h}, 9, shade_mode=rt.SHADE_EXTENDED, background=(0.3, 0.4, 0.5))
torch.cuda.synchronize()
np.save({repr(str(tmp_path / "b.npy"))}, acc.cpu().numpy())
"""
    env = dict(os.environ, RT_RENDER_WAVE_PATHS=paths)
    p = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    assert np.array_equal(np.load(tmp_path / "b.npy"), a)


@pytest.mark.parametrize("lanes", ["1", "3"])
def test_render_lanes_match(rt, cuda, tmp_path, lanes):
    """A frame of 230,400 paths is split into pixel chunks over two streams by
    default; one stream (RT_RENDER_LANES=1) or three give the same frame bit
    for bit, and so do the work counters of rt_render_count."""
    import os
    import subprocess
    import sys

    w, h, spp = 320, 180, 4
    tris, mats = lit_scene(rt)
    ubo = rt.make_ubo((0.0, 0.5, 4.0), (0.0, 0.0, 0.0), fov=60.0, depth=6, random_state=5)
    kw = {"shade_mode": rt.SHADE_EXTENDED, "background": (0.3, 0.4, 0.5)}
    with rt.Scene(tris, materials=mats, node_width=4) as sc:
        a = gpu_render(rt, cuda, sc, ubo, w, h, spp, **kw)
        acc = cuda.empty(w * h * 4, dtype=cuda.float32, device="cuda")
        rt.accum_clear(acc, w, h)
        counts = sc.render_count(ubo, acc, w, h, spp, **kw)
        cuda.cuda.synchronize()
        assert np.array_equal(acc.cpu().numpy(), a)
    code = f"""
import numpy as np, torch, sys
sys.path.insert(0, {repr(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))})
import raytracergpu_mastersproject_gb300 as rt
sph = rt.gen_icosphere(3, (0.0, 0.0, 0.0), 1.0, 0)
tris = np.concatenate([sph, rt.gen_config1()[0][-2:]])
mats = np.zeros(2, rt.MATERIAL_DTYPE)
mats[0]["albedo"][:3] = (0.73, 0.33, 0.25); mats[0]["materialType"] = rt.MAT_DIFFUSE
mats[1]["albedo"][:3] = (3.0, 3.0, 3.0); mats[1]["materialType"] = rt.MAT_LIGHT
ubo = rt.make_ubo((0.0, 0.5, 4.0), (0.0, 0.0, 0.0), fov=60.0, depth=6, random_state=5)
kw = dict(shade_mode=rt.SHADE_EXTENDED, background=(0.3, 0.4, 0.5))
acc = torch.empty({w} * {h} * 4, dtype=torch.float32, device="cuda")
with rt.Scene(tris, materials=mats, node_width=4) as sc:
    rt.accum_clear(acc, {w}, {h})
    sc.render(ubo, acc, {w}, {h}, {spp}, **kw)
    torch.cuda.synchronize()
    np.save({repr(str(tmp_path / "b.npy"))}, acc.cpu().numpy())
    rt.accum_clear(acc, {w}, {h})
    c = sc.render_count(ubo, acc, {w}, {h}, {spp}, **kw)
    np.save({repr(str(tmp_path / "c.npy"))}, np.array(c, dtype=np.uint64))
"""
    env = dict(os.environ, RT_RENDER_LANES=lanes)
    p = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    assert np.array_equal(np.load(tmp_path / "b.npy"), a)
    assert tuple(int(x) for x in np.load(tmp_path / "c.npy")) == tuple(counts)


def test_deep_stack_render_matches_per_pixel(rt, cuda):
    """A dense cluster of large triangles keeps traversal stacks far past the
    shared-memory ring; the wavefront frame equals the binary per-pixel one."""
    rng = np.random.default_rng(8)
    n = 20_000
    tris = np.zeros(n, rt.TRIANGLE_DTYPE)
    c = rng.normal(0.0, 0.05, (n, 3)).astype(np.float32)
    for k in ("v0", "v1", "v2"):
        tris[k][:, :3] = c + rng.normal(0.0, 0.5, (n, 3)).astype(np.float32)
    tris["materialIndex"] = rng.integers(0, 2, n)
    mats = np.zeros(2, rt.MATERIAL_DTYPE)
    mats[0]["albedo"][:3] = (0.6, 0.5, 0.4)
    mats[0]["materialType"] = rt.MAT_DIFFUSE
    mats[1]["albedo"][:3] = (2.0, 2.0, 2.0)
    mats[1]["materialType"] = rt.MAT_LIGHT
    ubo = rt.make_ubo((0.0, 0.0, 4.0), (0.0, 0.0, 0.0), fov=40.0, depth=4, random_state=9)
    with rt.Scene(tris, materials=mats, node_width=2) as s2, rt.Scene(tris, materials=mats, node_width=4) as s4:
        a = gpu_render(rt, cuda, s2, ubo, 64, 48, 3)
        b = gpu_render(rt, cuda, s4, ubo, 64, 48, 3)
    assert np.array_equal(a, b)
    assert a[0::4].max() > 0.1


def test_stream_release_frees_and_recreates_workspace(rt, cuda):
    """rt_stream_release drops the stream's workspace (including the path
    tracer's scratch); the next call on the stream allocates a new one and
    renders the same frame."""
    tris, mats = lit_scene(rt)
    ubo = rt.make_ubo((0.0, 0.5, 4.0), (0.0, 0.0, 0.0), fov=60.0, depth=4, random_state=21)
    st = cuda.cuda.Stream()
    w, h = 80, 45

    def frame(sc):
        acc = cuda.empty(w * h * 4, dtype=cuda.float32, device="cuda")
        cuda.cuda.synchronize()
        rt.accum_clear(acc, w, h, stream=st)
        sc.render(ubo, acc, w, h, 4, stream=st)
        st.synchronize()
        return acc.cpu().numpy()

    with rt.Scene(tris, materials=mats) as sc:
        a = frame(sc)
        free0 = cuda.cuda.mem_get_info()[0]
        rt.release_stream(st)
        free1 = cuda.cuda.mem_get_info()[0]
        b = frame(sc)
        rt.release_stream(st)
        rt.release_stream(st)  # nothing left to free
    assert np.array_equal(a, b)
    assert free1 >= free0


@pytest.mark.parametrize("depth", [64, 70])
def test_deep_paths_wavefront_and_step_kernel(rt, cuda, depth):
    """Depth up to 64 runs the wavefront renderer, deeper frames the per-lane
    step kernel; both equal the binary per-pixel kernel bit for bit.  Glass
    spheres keep paths bouncing to the depth limit."""
    tris, mats = rt.gen_spheres_scene(9, 8, 3, 0.05)
    mats["materialType"] = rt.MAT_DIELECTRIC
    mats["ior"] = 1.5
    mats["albedo"][:, :3] = 1.0
    ubo = rt.make_ubo((0.0, 3.0, 28.0), (0.0, 0.0, 0.0), fov=40.0, depth=depth, random_state=4,
                      num_triangles=len(tris), num_materials=len(mats))
    kw = {"shade_mode": rt.SHADE_EXTENDED, "background": (0.6, 0.7, 1.0)}
    with rt.Scene(tris, materials=mats, node_width=2) as s2, rt.Scene(tris, materials=mats, node_width=4) as s4:
        a = gpu_render(rt, cuda, s2, ubo, 48, 27, 2, **kw)
        b = gpu_render(rt, cuda, s4, ubo, 48, 27, 2, **kw)
    assert np.array_equal(a, b)
    assert a[0::4].max() > 0.1
