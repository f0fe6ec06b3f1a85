"""Seeded random parity sweep of the ray-query path against the CPU oracle.

Each case draws a scene and a ray batch with the awkward shapes the other
tests cover one at a time: zero-area and axis-aligned triangles, duplicated
triangles (exact ties), spheres (some of zero radius), scenes of one
primitive, rays with zero direction components, empty [tmin, tmax] intervals
and tmin below zero, origins inside and outside the scene.  Scene options are
drawn too: node width, leaf size, build mode, device build, S1 traversal.
Closest hit must match the oracle's restatement (hitBVH, raytraceBVH.comp:
195-265) up to near-ties the binary64 arbiter explains, any hit must agree
on which rays hit, and the Moller-Trumbore mode must match the oracle's.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def random_case(rt, seed):
    g = np.random.default_rng(seed)
    n_tri = int(g.choice([1, 2, 7, 64, 1000, 20_000]))
    n_sph = int(g.choice([0, 0, 1, 5, 40]))
    scale = float(g.choice([1e-3, 1.0, 1e3]))
    tris = np.zeros(n_tri, rt.TRIANGLE_DTYPE)
    c = g.uniform(-1, 1, (n_tri, 3)) * scale
    size = scale * float(g.choice([0.01, 0.05, 0.3]))
    for k in ("v0", "v1", "v2"):
        tris[k][:, :3] = (c + g.normal(0, size, (n_tri, 3))).astype(np.float32)
    kinds = g.integers(0, 10, n_tri)
    flat = kinds == 0  # axis-aligned: all three vertices share y
    for k in ("v1", "v2"):
        tris[k][flat, 1] = tris["v0"][flat, 1]
    zero = kinds == 1  # zero area: v2 == v1
    tris["v2"][zero] = tris["v1"][zero]
    dup = np.nonzero(kinds == 2)[0]  # exact duplicates of another triangle
    if len(dup) and n_tri > 1:
        src = g.integers(0, n_tri, len(dup))
        for k in ("v0", "v1", "v2"):
            tris[k][dup] = tris[k][src]
    sph = np.zeros(n_sph, rt.SPHERE_DTYPE)
    if n_sph:
        sph["center"][:, :3] = (g.uniform(-1, 1, (n_sph, 3)) * scale).astype(np.float32)
        sph["radius"] = (g.uniform(0, 0.1, n_sph) * scale).astype(np.float32)
        sph["radius"][g.integers(0, 4, n_sph) == 0] = 0.0
    n_ray = int(g.choice([1, 31, 4096, 50_000]))
    rays = np.zeros(n_ray, rt.RAY_DTYPE)
    rays["org"] = (g.uniform(-1.5, 1.5, (n_ray, 3)) * scale).astype(np.float32)
    d = g.normal(0, 1, (n_ray, 3))
    axis = g.integers(0, 6, n_ray)
    for a in range(3):
        d[axis == a, a] = 0.0  # one zero component
        d[axis == 3 + a] = 0.0
        d[axis == 3 + a, a] = 1.0  # axis-parallel
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays["dir"] = d.astype(np.float32)
    rays["tmin"] = np.float32(g.choice([1e-4, 0.0, -1.0]) * scale)
    rays["tmax"] = np.float32(np.inf)
    short = g.integers(0, 5, n_ray) == 0
    rays["tmax"][short] = (g.uniform(0, 2, short.sum()) * scale).astype(np.float32)
    empty = g.integers(0, 20, n_ray) == 0
    rays["tmax"][empty] = rays["tmin"][empty] - np.float32(scale)
    opts = {
        "node_width": int(g.choice([2, 4])),
        "leaf_size": int(g.choice([0, 1, 2, 8])),
        "bvh_mode": int(g.choice([rt.BVH_SORTED, rt.BVH_REFERENCE])),
    }
    pick = int(g.integers(0, 3))
    if pick == 1:
        opts["build_on_device"] = True
    elif pick == 2:
        opts["traverse_s1"] = True
    return tris, sph, rays, opts


def trace(cuda, rt, sc, rays, **kw):
    d_rays = cuda.from_numpy(np.ascontiguousarray(rays).view(np.uint8)).cuda()
    d_hits = cuda.empty(len(rays) * 8, dtype=cuda.uint8, device="cuda")
    sc.trace(d_rays, d_hits, n=len(rays), **kw)
    cuda.cuda.synchronize()
    return d_hits.cpu().numpy().view(rt.HIT_DTYPE).copy()


@pytest.mark.parametrize("seed", range(64))
def test_random_scenes_match_oracle(rt, orc, cuda, seed):
    tris, sph, rays, opts = random_case(rt, 1000 + seed)
    with rt.Scene(tris, spheres=sph, **opts) as sc:
        closest = trace(cuda, rt, sc, rays, sort=bool(seed % 2))
        anyh = trace(cuda, rt, sc, rays, any_hit=True)
        mt = trace(cuda, rt, sc, rays, mt=True)
        host = sc.trace_host(rays, sort=bool(seed % 2))
        nodes = sc.nodes()
    assert np.array_equal(host.view(np.uint64), closest.view(np.uint64))
    S = orc.Scene(tris, nodes, spheres=sph)
    ref, st = orc.trace(S, rays, canonical=True)
    assert st[4] == 0
    arb = orc.arbitrate(tris, rays, ref, closest)
    assert not arb["unexplained"], (opts, arb)
    same = (ref["prim"] == closest["prim"]) & (ref["prim"] != orc.NO_HIT)
    assert np.array_equal(ref["t"][same].view(np.uint32), closest["t"][same].view(np.uint32))
    assert np.array_equal(anyh["prim"] != orc.NO_HIT, ref["prim"] != orc.NO_HIT), opts
    ref_mt, _ = orc.trace(S, rays, canonical=True, mt=True)
    diff = np.nonzero(ref_mt["prim"] != mt["prim"])[0]
    for i in diff:  # near-ties only: both hit at the same t within 1e-6
        assert ref_mt["prim"][i] != orc.NO_HIT and mt["prim"][i] != orc.NO_HIT, (opts, i)
        assert abs(float(ref_mt["t"][i]) - float(mt["t"][i])) <= 1e-6 * abs(float(ref_mt["t"][i])), (opts, i)
    same = (ref_mt["prim"] == mt["prim"]) & (mt["prim"] != orc.NO_HIT)
    assert np.array_equal(ref_mt["t"][same].view(np.uint32), mt["t"][same].view(np.uint32))


@pytest.mark.parametrize("seed", range(16))
def test_random_frames_match_oracle(rt, orc, cuda, seed):
    """Path-traced frames of random sphere scenes (lights, diffuse, metal,
    glass, a sphere record), cameras, depths 1-12, 1-5 samples, both
    shadings and both primary-ray settings, against the oracle's restatement
    of raytraceBVH.comp: per-pixel RMSE within 1e-3 at identical RNG streams,
    nearly all pixels bit for bit (a path that meets a near-tie may differ)."""
    g = np.random.default_rng(2000 + seed)
    tris, mats = rt.gen_spheres_scene(int(g.integers(1, 1 << 30)), int(g.integers(1, 9)), int(g.integers(0, 3)),
                                      float(g.choice([0.0, 0.05])))
    lights = g.integers(0, 3, len(mats)) == 0
    mats["materialType"][lights] = rt.MAT_LIGHT
    mats["albedo"][lights, :3] = 3.0
    sph = np.zeros(1, rt.SPHERE_DTYPE)
    sph["center"][0, :3] = g.uniform(-6, 6, 3).astype(np.float32)
    sph["radius"] = np.float32(g.uniform(0.5, 2.0))
    sph["materialIndex"] = int(g.integers(0, len(mats)))
    cam = tuple(float(x) for x in g.uniform(-30, 30, 3))
    depth = int(g.integers(1, 13))
    ubo = rt.make_ubo(cam, (0.0, 0.0, 0.0), fov=float(g.uniform(20, 90)), depth=depth,
                      random_state=int(g.integers(0, 1 << 31)), num_triangles=len(tris), num_materials=len(mats))
    w, h, spp = int(g.integers(16, 97)), int(g.integers(9, 55)), int(g.integers(1, 6))
    extended = bool(g.integers(0, 2))
    bg = tuple(float(x) for x in g.uniform(0, 1, 3)) if extended else (0.0, 0.0, 0.0)
    every = bool(g.integers(0, 2))
    kw = {"shade_mode": rt.SHADE_EXTENDED if extended else rt.SHADE_REFERENCE, "background": bg,
          "trace_every_primary": every}
    with rt.Scene(tris, spheres=sph, materials=mats, node_width=int(g.choice([2, 4]))) as sc:
        acc = cuda.empty(w * h * 4, dtype=cuda.float32, device="cuda")
        rt.accum_clear(acc, w, h)
        sc.render(ubo, acc, w, h, spp, **kw)
        cuda.cuda.synchronize()
        img = acc.cpu().numpy()
        nodes = sc.nodes()
    ref = np.tile(np.array([0, 0, 0, 1], np.float32), w * h)
    assert orc.render(orc.Scene(tris, nodes, spheres=sph, mats=mats), ubo, ref, w, h, spp, extended=extended,
                      background=bg) == 0
    err = np.sqrt(np.mean((img.astype(np.float64) - ref.astype(np.float64)) ** 2))
    assert err <= 1e-3, (seed, err)
    assert np.mean(img == ref) > 0.98, seed
    assert np.array_equal(img[3::4], ref[3::4])  # the alpha RNG carry needs no tracing
