"""The oracle against the reference's own shaders, compiled for the host.

oracle/ref_glsl.py compiles raytraceBVH.comp (with random.glsl and
definitions.glsl) and the six S1 build shaders as C++, unchanged in meaning
(oracle/ref_shim.hpp supplies the GLSL types and built-ins).  These tests
require oracle/rt_oracle.c -- which the GPU parity tests use as the checker --
to agree with that code bit for bit: RNG streams, seeds, camera and primary
rays, the six build passes (nodes, Morton codes, sort order, enclosing box),
hitBVH on whole ray batches, and whole path-traced frames (accumulator and
alpha RNG carry).  Where the oracle defines what the reference leaves
undefined (a zero-area triangle's NaN t), the divergence is shown and
confined.
"""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def ref(orc):
    from oracle import ref as ref_mod

    if not ref_mod.available():
        pytest.skip("reference shaders not present on this host (no checkout, no generated sources)")
    return ref_mod


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


# ------------------------------------------------------------------- RNG ---
@pytest.mark.parametrize("seed", [0, 1, 7, 600 * 639 + 359, 0x9E3779B9, 0xFFFFFFFF])
def test_random_stream(orc, ref, seed):
    f, st = ref.random_stream(seed, 500)
    of, ost = orc.random_stream(seed, 500)
    assert np.array_equal(st, ost)
    assert np.array_equal(bits(f), bits(of))


@pytest.mark.parametrize("seed", [0, 3, 12345, 0xDEADBEEF])
def test_random_unit_vectors(orc, ref, seed):
    u = ref.random_unit_vectors(seed, 2000)
    assert np.array_equal(bits(u), bits(orc.random_unit_vectors(seed, 2000)))
    # with libm's sinf/cosf in the shader the draws move by at most a few ulps
    lm = ref.random_unit_vectors(seed, 2000, portable=False)
    assert np.max(np.abs(lm - u)) <= 4.8e-7


def test_seed(orc, ref):
    for x, y, r in [(0, 0, 0), (175, 650, 1), (639, 359, 0), (1279, 719, 0xFFFFFFFE), (5, 7, 123456789)]:
        assert ref.seed(x, y, r) == orc.lib().orc_seed(x, y, r)


# ---------------------------------------------------------------- camera ---
@pytest.mark.parametrize("cam,size", [(((0.0, 0.5, 4.0), (0.0, 0.0, 0.0), 60.0), (640, 360)),
                                      (((0.0, 3.0, 28.0), (0.0, 0.0, 0.0), 40.0), (1280, 720)),
                                      (((2.0, -1.0, 3.0), (0.5, 0.2, -1.0), 75.0), (33, 17))])
def test_camera_and_primary_rays(rt, orc, ref, cam, size):
    pos, look, fov = cam
    w, h = size
    ubo = rt.make_ubo(pos, look, fov=fov, depth=8, random_state=0)
    assert np.array_equal(bits(ref.camera(ubo, w, h)), bits(orc.camera(ubo, w, h)))
    rr = ref.get_rays(ubo, w, h)
    orays = orc.primary_rays(ubo, w, h)
    assert np.array_equal(bits(rr["org"]), bits(orays["org"]))
    # getRay normalises, rayColor (raytraceBVH.comp:280) normalises again
    d = rr["dir"].astype(np.float32)
    n = np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]).astype(np.float32)
    assert np.array_equal(bits((d / n[:, None]).astype(np.float32)), bits(orays["dir"]))


# -------------------------------------------------------------- S1 build ---
def _soup_with_spheres(rt, orc, seed, nt, ns, side=1.0):
    tris = rt.gen_soup(seed, 0, nt, side, 0.004) if nt else np.zeros(0, orc.TRI)
    sph = np.zeros(ns, orc.SPH)
    if ns:
        u = rt.gen_uniform(seed, 7, 4 * ns).reshape(ns, 4)
        sph["center"][:, :3] = u[:, :3] * side
        sph["radius"] = 0.01 + 0.05 * u[:, 3]
    return tris, sph


def _check_build(orc, ref, tris, sph=None, models=None):
    mod = np.eye(4, dtype=np.float32).reshape(1, 16) if models is None else models
    a = orc.build_bvh(tris, spheres=sph, mode=1, models=mod)
    b = ref.build_bvh(tris, spheres=sph, models=mod)
    assert np.array_equal(a[0].view(np.uint8), b[0].view(np.uint8)), "node arrays differ"
    assert np.array_equal(a[1], b[1]), "sorted Morton codes differ"
    assert np.array_equal(a[2], b[2]), "sort order differs"
    assert np.array_equal(bits(a[3]), bits(b[3])), "enclosing box differs"
    return b


def test_build_config1(rt, orc, ref):
    tris = rt.gen_config1()[0]
    _check_build(orc, ref, tris)


@pytest.mark.parametrize("nt,ns", [(1, 0), (0, 1), (2, 0), (1, 1), (31, 2), (200, 57), (255, 1), (256, 1),
                                   (3000, 300)])
def test_build_small_sizes_and_spheres(rt, orc, ref, nt, ns):
    tris, sph = _soup_with_spheres(rt, orc, 20 + nt + ns, nt, ns)
    _check_build(orc, ref, tris, sph)


def test_build_duplicate_codes(rt, orc, ref):
    # many identical centroids: equal Morton codes take the index tie-break
    # (ConstructHLBVH.comp:64-68) and the stable sort keeps input order
    base = rt.gen_soup(31, 0, 64, 1.0, 0.004)
    tris = np.concatenate([base] * 8)
    _check_build(orc, ref, tris)


def test_build_with_models(rt, orc, ref):
    # ModelSpaceToWorldSpace (pass 1) with three model matrices
    tris, sph = _soup_with_spheres(rt, orc, 41, 5000, 40)
    tris["modelIndex"] = np.arange(len(tris)) % 3
    sph["modelIndex"] = np.arange(len(sph)) % 3
    models = np.stack([np.eye(4, dtype=np.float32).reshape(16),
                       rt.model_matrix((1.0, -2.0, 0.5), (0.3, 1.1, -0.4), (2.0, 0.5, 1.0))["m"].reshape(16),
                       rt.model_matrix((-3.0, 0.0, 4.0), (0.0, 0.0, 0.7), (0.1, 0.1, 0.1))["m"].reshape(16)])
    _check_build(orc, ref, tris, sph, models)


# -------------------------------------------------------------- hitBVH ----
def _assert_same_hits(a, b):
    assert np.array_equal(a["prim"], b["prim"]), f"{int((a['prim'] != b['prim']).sum())} ids differ"
    assert np.array_equal(bits(a["t"]), bits(b["t"])), "t differs"


@pytest.mark.parametrize("mode", [0, 1], ids=["sorted", "reference"])
def test_trace_config1(rt, orc, ref, mode):
    tris, ubo, rays = rt.gen_config1()
    S = orc.Scene(tris, orc.build_bvh(tris, mode=mode)[0])
    got = ref.trace(S, rays)
    want, st = orc.trace(S, rays)
    assert st[4] == 0
    _assert_same_hits(got, want)
    assert (got["prim"] != orc.NO_HIT).sum() > 100000


def test_trace_soup_and_spheres(rt, orc, ref):
    tris, sph = _soup_with_spheres(rt, orc, 51, 200_000, 500)
    rays = rt.gen_rays(51, 0, 60_000, 1.0, 1e-4, float("inf"))
    S = orc.Scene(tris, orc.build_bvh(tris, spheres=sph, mode=0)[0], spheres=sph)
    got = ref.trace(S, rays)
    want, _ = orc.trace(S, rays)
    _assert_same_hits(got, want)
    assert ((got["prim"] & 0x80000000) != 0).sum() > 100  # sphere hits are covered
    assert ((got["prim"] != orc.NO_HIT) & ((got["prim"] & 0x80000000) == 0)).sum() > 10000


def test_trace_config3_sample(rt, orc, ref):
    """The first 131,072 rays of config 3 on its full 4,194,304-triangle soup."""
    from raytracergpu_mastersproject_gb300 import workloads

    tris, rays = workloads.config3(n_rays=131_072)
    S = orc.Scene(tris, orc.build_bvh(tris, mode=0)[0])
    _assert_same_hits(ref.trace(S, rays), orc.trace(S, rays)[0])


def test_trace_interval_edges(rt, orc, ref):
    # negative tmin, empty and point intervals, axis-parallel directions
    tris = rt.gen_soup(61, 0, 20_000, 1.0, 0.004)
    rays = rt.gen_rays(61, 0, 20_000, 1.0, 1e-4, float("inf"))
    rays["tmin"][0::4] = -0.5
    rays["tmax"][1::4] = rays["tmin"][1::4]
    rays["tmax"][2::4] = 0.05
    ax = rays[3::8]
    ax["dir"] = np.array([0.0, 0.0, 1.0], np.float32)
    rays[3::8] = ax
    S = orc.Scene(tris, orc.build_bvh(tris, mode=0)[0])
    _assert_same_hits(ref.trace(S, rays), orc.trace(S, rays)[0])


def test_zero_area_triangle_divergence_is_confined(rt, orc, ref):
    """The reference accepts a zero-area triangle's NaN t as a hit
    (triangleHit's tests are all false on NaN, raytraceBVH.comp:127-136); the
    oracle and the kernels define it as a miss.  Only rays whose reference
    result is such a NaN-t hit, or that the NaN bound then let reach a farther
    triangle, may differ."""
    tris = rt.gen_soup(71, 0, 5_000, 1.0, 0.01)
    flat = tris[::50].copy()
    flat["v1"] = flat["v0"]
    flat["v2"] = flat["v0"]
    tris[::50] = flat
    rays = rt.gen_rays(71, 0, 50_000, 1.0, 1e-4, float("inf"))
    S = orc.Scene(tris, orc.build_bvh(tris, mode=0)[0])
    got = ref.trace(S, rays)
    want, _ = orc.trace(S, rays)
    diff = np.nonzero((got["prim"] != want["prim"]) | (bits(got["t"]) != bits(want["t"])))[0]
    assert 0 < len(diff) < len(rays) // 20
    is_flat = np.zeros(len(tris), bool)
    is_flat[::50] = True
    flat_pts = tris["v0"][::50, :3].astype(np.float64)
    for i in diff:
        # the ray entered the padded leaf box (+-0.0005) of a zero-area triangle
        o, d = rays["org"][i].astype(np.float64), rays["dir"][i].astype(np.float64)
        v = flat_pts - o
        off = v - np.outer(v @ d / (d @ d), d)
        assert (np.linalg.norm(off, axis=1) < 0.0009).any(), i
        p = int(got["prim"][i])
        if np.isnan(got["t"][i]):
            assert is_flat[p]
        else:  # a farther triangle accepted after the NaN bound: a real hit, never closer
            assert not is_flat[p] and orc.triangle_test(tris[p], rays[i:i + 1]) is not None
            assert want["prim"][i] != orc.NO_HIT and want["t"][i] <= got["t"][i]
    same = np.setdiff1d(np.arange(len(rays)), diff)
    assert np.array_equal(got["prim"][same], want["prim"][same])


# -------------------------------------------------------------- render ----
def _lit_scene(rt, orc, subdiv=3):
    sph = rt.gen_icosphere(subdiv, (0.0, 0.0, 0.0), 1.0, 0)
    ground = rt.gen_config1()[0][-2:].copy()
    ground["materialIndex"] = 1
    tris = np.concatenate([sph, ground])
    mats = np.zeros(2, orc.MAT)
    mats[0]["albedo"][:3] = (0.7, 0.4, 0.3)
    mats[0]["materialType"] = 1
    mats[1]["albedo"][:3] = (2.0, 2.0, 2.0)
    mats[1]["materialType"] = 0
    return tris, mats


@pytest.mark.parametrize("mode", [0, 1], ids=["sorted", "reference"])
@pytest.mark.parametrize("depth,spp", [(1, 2), (6, 5), (12, 3)])
def test_render_lit_scene(rt, orc, ref, mode, depth, spp):
    tris, mats = _lit_scene(rt, orc)
    ubo = rt.make_ubo((0.0, 0.5, 4.0), (0.0, 0.0, 0.0), fov=60.0, depth=depth, random_state=7)
    S = orc.Scene(tris, orc.build_bvh(tris, mode=mode)[0], mats=mats)
    w, h = 96, 54
    a = np.tile(np.array([0, 0, 0, 1], np.float32), w * h)  # the clear of RaytracerBVH.cpp:772-776
    b = a.copy()
    assert orc.render(S, ubo, a, w, h, spp) == 0
    ref.render(S, ubo, b, w, h, spp)
    assert np.array_equal(bits(a), bits(b)), "accumulators differ"
    assert (a.reshape(-1, 4)[:, :3].sum(1) > 0).mean() > 0.3


def test_render_spheres_and_materials(rt, orc, ref):
    """Lights, diffuse triangles, sphere records and metal/glass materials
    (which the reference's scatter() terminates); split dispatches carry the
    RNG through alpha exactly like one call."""
    tris, mats = _lit_scene(rt, orc, subdiv=2)
    mats = np.concatenate([mats, np.zeros(3, orc.MAT)])
    mats[2]["albedo"][:3] = (0.9, 0.9, 0.9)
    mats[2]["materialType"] = 2
    mats[3]["albedo"][:3] = (1.0, 1.0, 1.0)
    mats[3]["materialType"] = 3
    mats[4]["albedo"][:3] = (0.2, 0.8, 0.3)
    mats[4]["materialType"] = 1
    sph = np.zeros(4, orc.SPH)
    sph["center"][:, :3] = [(1.5, 0.0, 0.0), (-1.5, 0.2, 0.5), (0.0, 1.4, -0.5), (0.0, -0.6, 1.5)]
    sph["radius"] = [0.4, 0.5, 0.3, 0.25]
    sph["materialIndex"] = [2, 3, 4, 0]
    tris["materialIndex"][:40] = 4
    ubo = rt.make_ubo((0.3, 0.8, 4.5), (0.0, 0.0, 0.0), fov=55.0, depth=8, random_state=3)
    S = orc.Scene(tris, orc.build_bvh(tris, spheres=sph, mode=0)[0], spheres=sph, mats=mats)
    w, h = 80, 45
    a = np.tile(np.array([0, 0, 0, 1], np.float32), w * h)
    b = a.copy()
    orc.render(S, ubo, a, w, h, 4)
    ref.render(S, ubo, b, w, h, 1)
    ref.render(S, ubo, b, w, h, 3)
    assert np.array_equal(bits(a), bits(b))
