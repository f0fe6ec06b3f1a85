"""CPU checks of the oracle: restatements, published examples, golden fixtures."""
import math
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


# ------------------------------------------------------------------ RNG ---
def py_random_stream(state: int, n: int):
    """Independent restatement of random.glsl:12-22 with Python ints."""
    out, states = [], []
    s = state & 0xFFFFFFFF
    for _ in range(n):
        s = (s * 747796405 + 1) & 0xFFFFFFFF
        word = (((s >> ((s >> 28) + 4)) ^ s) * 277803737) & 0xFFFFFFFF
        word = ((word >> 22) ^ word) & 0xFFFFFFFF
        out.append(np.float32(np.float32(word) / np.float32(4294967295.0)))
        states.append(s)
    return np.array(out, np.float32), np.array(states, np.uint32)


@pytest.mark.parametrize("seed", [0, 1, 7, 600 * 639 + 359, 0xFFFFFFFF])
def test_rng_matches_independent_restatement(orc, seed):
    f, st = orc.random_stream(seed, 200)
    pf, pst = py_random_stream(seed, 200)
    assert np.array_equal(st, pst)
    assert np.array_equal(f.view(np.uint32), pf.view(np.uint32))


def test_seed_formula(orc):
    # random.glsl:9: (600*x + y) * (randomState + 1), 32-bit wrap
    for x, y, r in [(0, 0, 0), (639, 359, 0), (1279, 719, 0xFFFFFFFE), (5, 7, 123456789)]:
        assert orc.lib().orc_seed(x, y, r) == ((600 * x + y) * (r + 1)) & 0xFFFFFFFF


def test_rng_golden(orc):
    g = np.load(GOLDEN / "rng.npz")
    for i, s in enumerate(g["seeds"]):
        f, st = orc.random_stream(int(s), 64)
        assert np.array_equal(f.view(np.uint32), g["floats"][i].view(np.uint32))
        assert np.array_equal(st, g["states"][i])
        u = orc.random_unit_vectors(int(s), 16)
        assert np.array_equal(u.view(np.uint32), g["units"][i].view(np.uint32))


def test_sincos_accuracy_and_golden(orc):
    g = np.load(GOLDEN / "sincos.npz")
    for x, s, c in zip(g["x"], g["sin"], g["cos"]):
        gs, gc = np.float32(orc.lib().orc_sin(float(x))), np.float32(orc.lib().orc_cos(float(x)))
        assert gs.view(np.uint32) == s.view(np.uint32) and gc.view(np.uint32) == c.view(np.uint32)
        assert abs(float(gs) - math.sin(float(x))) <= 3e-7
        assert abs(float(gc) - math.cos(float(x))) <= 3e-7


def test_unit_vectors_are_unit(orc):
    u = orc.random_unit_vectors(99, 1000).astype(np.float64)
    assert np.allclose(np.linalg.norm(u, axis=1), 1.0, atol=1e-6)


# -------------------------------------------------------------- Morton ----
def test_spread_masks_match_their_binary_comments(orc):
    # GenerateMortonCodesOfPrimitives.comp:45-48 gives each mask in binary
    assert 50331903 == 0b00000011000000000000000011111111
    assert 50393103 == 0b00000011000000001111000000001111
    assert 51130563 == 0b00000011000011000011000011000011
    assert 153391689 == 0b00001001001001001001001001001001
    f = orc.lib().orc_separate_bits_by_3
    for v in [0, 1, 2, 3, 5, 511, 1023]:
        expect = 0
        for b in range(10):
            if v >> b & 1:
                expect |= 1 << (3 * b)
        assert f(v) == expect
    assert f(1024) == f(1023)  # the ==MORTON_SCALE clamp (:42-44)


def test_karras_2012_figure3(orc):
    """Worked example of Karras, "Maximizing Parallelism in the Construction of
    BVHs, Octrees, and k-d Trees" (HPG 2012), Fig. 3: 8 sorted 5-bit keys."""
    codes = [0b00001, 0b00010, 0b00100, 0b00101, 0b10011, 0b11000, 0b11001, 0b11110]
    left, right = orc.karras(codes)
    leaf = lambda k: 7 + k  # leaves sit at N-1+k (ConstructHLBVH.comp:149-168)
    assert list(left) == [3, leaf(0), leaf(2), 1, leaf(4), 6, leaf(5)]
    assert list(right) == [4, leaf(1), leaf(3), 2, 5, leaf(7), leaf(6)]


# ------------------------------------------------------------- BVH build --
def check_tree(orc, nodes, nt, ns):
    n = nt + ns
    assert len(nodes) == 2 * n - 1
    seen_prim = set()
    seen = np.zeros(len(nodes), bool)
    stack = [0]
    while stack:
        x = stack.pop()
        assert not seen[x]
        seen[x] = True
        nd = nodes[x]
        if nd["left"] == 0 and nd["right"] == 0:
            key = (int(nd["primitiveType"]), int(nd["primitiveIndex"]))
            assert key not in seen_prim
            seen_prim.add(key)
            for a in "XYZ":
                assert nd[f"max{a}"] - nd[f"min{a}"] >= np.float32(0.001) or nd[f"max{a}"] > nd[f"min{a}"]
        else:
            for c in (nd["left"], nd["right"]):
                ch = nodes[c]
                for a in "XYZ":
                    assert nd[f"min{a}"] <= ch[f"min{a}"] and nd[f"max{a}"] >= ch[f"max{a}"]
                stack.append(int(c))
    assert seen.all()
    assert len(seen_prim) == n


@pytest.mark.parametrize("mode", [0, 1])
def test_bvh_invariants(rt, orc, mode):
    tris, ubo, rays = rt.gen_config1()
    nodes, codes, prims, enc = orc.build_bvh(tris, mode=mode)
    check_tree(orc, nodes, len(tris), 0)
    assert np.all(np.diff(codes.astype(np.int64)) >= 0)
    soup = rt.gen_soup(5, 0, 5000, 1.0, 0.01)
    sph = np.zeros(7, orc.SPH)
    sph["center"][:, :3] = np.random.default_rng(0).random((7, 3))
    sph["radius"] = 0.05
    nodes, _, _, _ = orc.build_bvh(soup, sph, mode=mode)
    check_tree(orc, nodes, len(soup), len(sph))


def test_golden_small_scene(orc):
    g = np.load(GOLDEN / "small_scene.npz")
    tris = g["tris"].view(orc.TRI)
    rays = g["rays"].view(orc.RAY)
    for mode, key in ((0, "sorted"), (1, "reference")):
        nodes, codes, _, _ = orc.build_bvh(tris, mode=mode)
        assert np.array_equal(nodes.view(np.uint8), g[f"nodes_{key}"])
        assert np.array_equal(codes, g[f"codes_{key}"])
        hits, st = orc.trace(orc.Scene(tris, nodes), rays)
        assert st[4] == 0
        assert np.array_equal(hits.view(np.uint8), g[f"hits_{key}"])
    mats = g["mats"].view(orc.MAT)
    nodes = g["nodes_sorted"].view(orc.NODE)
    hany, _ = orc.trace(orc.Scene(tris, nodes), rays, any_hit=True)
    assert np.array_equal(hany.view(np.uint8), g["hits_any"])
    import ctypes as C
    from raytracergpu_mastersproject_gb300 import RaytracingUBO
    ubo = RaytracingUBO.from_buffer_copy(g["ubo"].tobytes())
    w, h, spp = (int(v) for v in g["render_wh_spp"])
    acc = np.tile(np.array([0, 0, 0, 1], np.float32), w * h)
    orc.render(orc.Scene(tris, nodes, mats=mats), ubo, acc, w, h, spp)
    assert np.array_equal(acc.view(np.uint32), g["accum"].view(np.uint32))


def test_golden_soup(orc):
    g = np.load(GOLDEN / "soup_small.npz")
    tris, rays = g["tris"].view(orc.TRI), g["rays"].view(orc.RAY)
    nodes, _, _, _ = orc.build_bvh(tris, mode=0)
    assert np.array_equal(nodes.view(np.uint8), g["nodes"])
    hits, _ = orc.trace(orc.Scene(tris, nodes), rays)
    assert np.array_equal(hits.view(np.uint8), g["hits"])


def test_golden_soup_moller_trumbore(orc):
    g = np.load(GOLDEN / "soup_small.npz")
    m = np.load(GOLDEN / "soup_small_mt.npz")
    tris, rays, nodes = g["tris"].view(orc.TRI), g["rays"].view(orc.RAY), g["nodes"].view(orc.NODE)
    hits, _ = orc.trace(orc.Scene(tris, nodes), rays, mt=True)
    assert np.array_equal(hits.view(np.uint8), m["hits"])
    assert (hits["prim"] != orc.NO_HIT).sum() > 100


# --------------------------------------------------------- traversal ------
def test_reference_and_canonical_orders_agree(rt, orc):
    tris, ubo, rays = rt.gen_config1()
    for mode in (0, 1):
        nodes, _, _, _ = orc.build_bvh(tris, mode=mode)
        S = orc.Scene(tris, nodes)
        a, sa = orc.trace(S, rays[::7])
        b, sb = orc.trace(S, rays[::7], canonical=True)
        assert np.array_equal(a["prim"], b["prim"])
        assert np.array_equal(a["t"].view(np.uint32), b["t"].view(np.uint32))
        assert sb[0] < sa[0]  # culling does less work
    soup = rt.gen_soup(9, 0, 40_000, 1.0, 0.004)
    rays = rt.gen_rays(9, 0, 20_000, 1.0, 1e-4, float("inf"))
    nodes, _, _, _ = orc.build_bvh(soup, mode=0)
    S = orc.Scene(soup, nodes)
    a, _ = orc.trace(S, rays)
    b, _ = orc.trace(S, rays, canonical=True)
    arb = orc.arbitrate(soup, rays, a, b)
    assert not arb["unexplained"]


def test_arbiter_flags_a_planted_mistake(rt, orc):
    """A wrong id planted into the oracle's own answer must be caught."""
    soup = rt.gen_soup(9, 0, 20_000, 1.0, 0.004)
    rays = rt.gen_rays(9, 0, 5_000, 1.0, 1e-4, float("inf"))
    nodes, _, _, _ = orc.build_bvh(soup, mode=0)
    a, _ = orc.trace(orc.Scene(soup, nodes), rays)
    bad = a.copy()
    hit = np.nonzero(a["prim"] != orc.NO_HIT)[0][:5]
    bad["prim"][hit] = (bad["prim"][hit] + 1) % len(soup)
    arb = orc.arbitrate(soup, rays, a, bad)
    assert len(arb["unexplained"]) == 5


def test_any_hit_reports_a_real_hit(rt, orc):
    soup = rt.gen_soup(10, 0, 20_000, 1.0, 0.004)
    rays = rt.gen_rays(10, 0, 4_000, 1.0, 1e-4, 0.2)
    nodes, _, _, _ = orc.build_bvh(soup, mode=0)
    S = orc.Scene(soup, nodes)
    c, _ = orc.trace(S, rays)
    a, _ = orc.trace(S, rays, any_hit=True)
    assert np.array_equal(c["prim"] != orc.NO_HIT, a["prim"] != orc.NO_HIT)
    for i in np.nonzero(a["prim"] != orc.NO_HIT)[0][:200]:
        t = orc.triangle_test(soup[a["prim"][i]], rays[i:i + 1])
        assert t is not None and np.float32(t) == a["t"][i] and a["t"][i] >= c["t"][i]


# ------------------------------------------------- Moller-Trumbore mode ----
def _mt_numpy(tris, ray):
    """Moller-Trumbore in numpy binary32 (one rounding per operation, the
    oracle's evaluation order) against every triangle -> (t per triangle, hit mask)."""
    f = np.float32
    v0, v1, v2 = (tris[k][:, :3].astype(f) for k in ("v0", "v1", "v2"))
    o, d = ray["org"][0].astype(f), ray["dir"][0].astype(f)
    e1, e2 = v1 - v0, v2 - v0
    px = d[1] * e2[:, 2] - d[2] * e2[:, 1]
    py = d[2] * e2[:, 0] - d[0] * e2[:, 2]
    pz = d[0] * e2[:, 1] - d[1] * e2[:, 0]
    det = (e1[:, 0] * px + e1[:, 1] * py) + e1[:, 2] * pz
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = f(1.0) / det
        s = o - v0
        u = ((s[:, 0] * px + s[:, 1] * py) + s[:, 2] * pz) * inv
        qx = s[:, 1] * e1[:, 2] - s[:, 2] * e1[:, 1]
        qy = s[:, 2] * e1[:, 0] - s[:, 0] * e1[:, 2]
        qz = s[:, 0] * e1[:, 1] - s[:, 1] * e1[:, 0]
        v = ((d[0] * qx + d[1] * qy) + d[2] * qz) * inv
        t = ((e2[:, 0] * qx + e2[:, 1] * qy) + e2[:, 2] * qz) * inv
        ok = (np.abs(det) > 0) & (u >= 0) & (u <= 1) & (v >= 0) & (u + v <= 1)
        ok &= (t >= ray["tmin"][0]) & (t <= ray["tmax"][0])
    return t, ok


def test_mt_restatement_matches_numpy(rt, orc):
    """The oracle's Moller-Trumbore mode against an independent numpy
    binary32 restatement over every triangle: the same closest t bit for bit
    (the same id unless another triangle has exactly that t)."""
    soup = rt.gen_soup(21, 0, 3_000, 1.0, 0.02)
    rays = rt.gen_rays(21, 0, 400, 1.0, 1e-4, float("inf"))
    nodes, _, _, _ = orc.build_bvh(soup, mode=0)
    got, _ = orc.trace(orc.Scene(soup, nodes), rays, mt=True)
    hits = 0
    for i in range(len(rays)):
        t, ok = _mt_numpy(soup, rays[i:i + 1])
        if not ok.any():
            assert got["prim"][i] == orc.NO_HIT
            continue
        hits += 1
        tmin = t[ok].min()
        assert got["prim"][i] != orc.NO_HIT and got["t"][i].view(np.uint32) == np.float32(tmin).view(np.uint32)
        assert t[got["prim"][i]] == tmin and ok[got["prim"][i]]
    assert hits > 100


def _mt_explained(tri, ray, t_mt, t_plane, extent):
    """Why a Moller-Trumbore hit can differ from the plane test's: the ray
    grazes the plane (|n.d| < 1e-4, rejected by the reference), the hit lies on
    an edge (in binary64 a barycentric within 1e-4 / |n.d| of 0, or u+v of 1:
    both tests round the hit point at the scale of the coordinates, not of the
    triangle, and the plane test's point moves along the ray by t's error), or
    the two answers are a near-tie in t."""
    v0, v1, v2 = (tri[k][:3].astype(np.float64) for k in ("v0", "v1", "v2"))
    o, d = ray["org"][0].astype(np.float64), ray["dir"][0].astype(np.float64)
    n = np.cross(v1 - v0, v2 - v0)
    if np.linalg.norm(n) == 0:
        return "degenerate"
    n /= np.linalg.norm(n)
    if abs(n @ d) < 1.01e-4:
        return "grazing"
    t = ((v0 - o) @ n) / (n @ d)
    p = o + t * d
    e1, e2, q = v1 - v0, v2 - v0, p - v0
    m = np.array([[e1 @ e1, e1 @ e2], [e1 @ e2, e2 @ e2]])
    u, v = np.linalg.solve(m, np.array([q @ e1, q @ e2]))
    if min(abs(u), abs(v), abs(1 - u - v)) < 1e-4 / max(abs(n @ d), 1e-4):
        return "edge"
    if np.isfinite(t_plane) and abs(t_mt - t_plane) <= 1e-5 * max(abs(t_mt), extent):
        return "near-tie"
    return None


def test_mt_divergence_set(rt, orc):
    """The Moller-Trumbore mode against the reference's plane test: hit ids
    agree except on grazing rays, edge hits and near-ties; matching hits agree
    in t within 1e-5 of max(t, scene extent) plus 1e-7 / |n.d| (the plane
    test's t cancels for hits near the ray origin and near grazing).  Config 1, a soup, and the first 131,072 rays of
    config 3 (about 1 in 12,000 of them differ there, every one at an edge)."""
    cases = []
    tris, _, rays = rt.gen_config1()
    cases.append((tris, rays[::3], 20.0, False))
    soup = rt.gen_soup(22, 0, 50_000, 1.0, 0.004)
    cases.append((soup, rt.gen_rays(22, 0, 20_000, 1.0, 1e-4, float("inf")), 1.0, False))
    soup3 = rt.gen_soup(3, 0, 4_194_304, 1.0, 0.002)
    cases.append((soup3, rt.gen_rays(3, 0, 131_072, 1.0, 1e-4, float("inf")), 1.0, True))
    for tris, rays, extent, sah in cases:
        nodes = rt.build_bvh_sah(tris) if sah else orc.build_bvh(tris, mode=0)[0]
        S = orc.Scene(tris, nodes)
        plane, _ = orc.trace(S, rays, canonical=True)
        mt, _ = orc.trace(S, rays, canonical=True, mt=True)
        same = plane["prim"] == mt["prim"]
        both = same & (plane["prim"] != orc.NO_HIT)
        assert both.sum() > 0.1 * len(rays)
        dt = np.abs(plane["t"][both].astype(np.float64) - mt["t"][both])
        # the plane test's t = (D - n.o) / (n.d) carries D - n.o's absolute
        # rounding divided by n.d, so the bound grows as the ray grazes
        hit = tris[plane["prim"][both]]
        v0, v1, v2 = (hit[k][:, :3].astype(np.float64) for k in ("v0", "v1", "v2"))
        n = np.cross(v1 - v0, v2 - v0)
        n /= np.linalg.norm(n, axis=1, keepdims=True)
        nd = np.abs(np.sum(n * rays["dir"][both].astype(np.float64), axis=1))
        assert np.all(dt <= 1e-5 * np.maximum(np.abs(mt["t"][both]), extent) + 1e-7 / nd)
        diff = np.nonzero(~same)[0]
        assert len(diff) <= 0.01 * len(rays)
        for i in diff:
            r = rays[i:i + 1]
            if mt["prim"][i] == orc.NO_HIT:  # the plane test hit where MT missed: an edge or near-tie
                why = _mt_explained(tris[plane["prim"][i]], r, np.inf, plane["t"][i], extent) or "mt-miss"
                assert why in ("edge", "grazing", "degenerate"), (i, why)
                continue
            why = _mt_explained(tris[mt["prim"][i]], r, mt["t"][i], plane["t"][i], extent)
            if why is None and plane["prim"][i] != orc.NO_HIT:
                why = _mt_explained(tris[plane["prim"][i]], r, mt["t"][i], plane["t"][i], extent)
            assert why is not None, (i, mt[i], plane[i])


def test_resolve_formula(orc):
    acc = np.array([0.0, 0.25, 4.0, 1.0, -1.0, 1e-8, 2.0, 0.5], np.float32)
    out = orc.resolve(acc, 2, 1, 4)
    expect = np.clip(np.sqrt(np.maximum(acc.reshape(2, 4)[:, :3] / np.float32(4), 0)), 0, 1)
    assert np.allclose(out.reshape(2, 4)[:, :3], expect, atol=0)
    assert np.all(out.reshape(2, 4)[:, 3] == 1.0)


# ------------------------------------------------------ workload inputs ---
@pytest.mark.parametrize("seed,stream,n,side,sigma", [(3, 0, 50_000, 1.0, 0.002), (4, 17, 3_000, 0.3, 0.002),
                                                      (11, 0, 1_000, 1.0, 0.004)])
def test_workload_generators_match_library(rt, orc, seed, stream, n, side, sigma):
    """The oracle's copy of the seeded generators (the CPU reference arm's
    inputs) gives the library's triangles and rays byte for byte, also from
    an offset into the sequence."""
    a = rt.gen_soup(seed, stream, n, side, sigma)
    assert np.array_equal(a.view(np.uint8), orc.gen_soup(seed, stream, n, side, sigma).view(np.uint8))
    tail = orc.gen_soup(seed, stream, 100, side, sigma, first=n - 100)
    assert np.array_equal(a[-100:].view(np.uint8), tail.view(np.uint8))
    r = rt.gen_rays(seed, stream, n, side, 1e-4, float("inf"))
    assert np.array_equal(r.view(np.uint8), orc.gen_rays(seed, stream, n, side, 1e-4, float("inf")).view(np.uint8))
    rtail = orc.gen_rays(seed, stream, 64, side, 1e-4, float("inf"), first=n - 64)
    assert np.array_equal(r[-64:].view(np.uint8), rtail.view(np.uint8))
