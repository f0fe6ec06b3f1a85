"""The binned-SAH traversal tree (rt_build_bvh_sah) on the CPU: a valid
binary tree over every primitive, the same hits as the S1 tree through the
oracle's traversal, and fewer box tests per ray on a config-3-style soup."""
import numpy as np
import pytest


def check_tree(rt, nodes, n_tris, n_sph, tris, sph):
    n = n_tris + n_sph
    assert len(nodes) == 2 * n - 1
    seen_t = np.zeros(n_tris, int)
    seen_s = np.zeros(n_sph, int)
    stack = [0]
    visited = 0
    while stack:
        i = stack.pop()
        visited += 1
        nd = nodes[i]
        box = np.array([nd["minX"], nd["maxX"], nd["minY"], nd["maxY"], nd["minZ"], nd["maxZ"]])
        if nd["left"] == 0 and nd["right"] == 0:
            p = nd["primitiveIndex"]
            if nd["primitiveType"] == rt.PRIM_TRIANGLE:
                seen_t[p] += 1
                v = np.stack([tris["v0"][p, :3], tris["v1"][p, :3], tris["v2"][p, :3]])
                lo, hi = v.min(0), v.max(0)
            else:
                seen_s[p] += 1
                lo = sph["center"][p, :3] - sph["radius"][p]
                hi = sph["center"][p, :3] + sph["radius"][p]
            assert np.all(box[0::2] <= lo) and np.all(box[1::2] >= hi)
            continue
        for c in (nd["left"], nd["right"]):
            ch = nodes[c]
            cb = np.array([ch["minX"], ch["maxX"], ch["minY"], ch["maxY"], ch["minZ"], ch["maxZ"]])
            assert np.all(box[0::2] <= cb[0::2]) and np.all(box[1::2] >= cb[1::2])
            stack.append(c)
    assert visited == len(nodes)
    assert np.all(seen_t == 1) and np.all(seen_s == 1)


def test_sah_tree_is_valid_and_matches_s1_hits(rt, orc):
    n = 65_536
    side = (n / 4_194_304) ** (1 / 3)
    tris = rt.gen_soup(3, 0, n, side, 0.002)
    rays = rt.gen_rays(3, 0, 20_000, side, 1e-4, float("inf"))
    sah = rt.build_bvh_sah(tris)
    s1 = rt.build_bvh(tris)
    check_tree(rt, sah, n, 0, tris, None)
    h_sah, st_sah = orc.trace(orc.Scene(tris, sah), rays, canonical=True)
    h_s1, st_s1 = orc.trace(orc.Scene(tris, s1), rays, canonical=True)
    assert np.array_equal(h_sah["prim"], h_s1["prim"])
    assert np.array_equal(h_sah["t"].view(np.uint32), h_s1["t"].view(np.uint32))
    assert (h_sah["prim"] != orc.NO_HIT).sum() > 10_000
    assert st_sah[0] < 0.95 * st_s1[0]  # box tests: about 10% fewer


def test_sah_tree_with_spheres_and_degenerate_inputs(rt, orc):
    rng = np.random.default_rng(1)
    tris = rt.gen_soup(5, 0, 3_000, 1.0, 0.01)
    tris = np.concatenate([tris, np.repeat(tris[:1], 500)])  # 501 coincident triangles
    sph = np.zeros(40, rt.SPHERE_DTYPE)
    sph["center"][:, :3] = rng.uniform(0.0, 1.0, (40, 3))
    sph["radius"] = rng.uniform(0.01, 0.05, 40)
    nodes = rt.build_bvh_sah(tris, spheres=sph)
    check_tree(rt, nodes, len(tris), len(sph), tris, sph)
    rays = rt.gen_rays(5, 0, 5_000, 1.0, 1e-4, float("inf"))
    a, _ = orc.trace(orc.Scene(tris, nodes, spheres=sph), rays, canonical=True)
    b, _ = orc.trace(orc.Scene(tris, rt.build_bvh(tris, spheres=sph), spheres=sph), rays, canonical=True)
    # the closest t never depends on the tree; the id may only differ between
    # the coincident copies of triangle 0 (an exact tie)
    assert np.array_equal(a["t"].view(np.uint32), b["t"].view(np.uint32))
    copies = {0} | set(range(3_000, 3_500))
    diff = np.nonzero(a["prim"] != b["prim"])[0]
    assert all(int(a["prim"][i]) in copies and int(b["prim"][i]) in copies for i in diff)
    assert (a["prim"] != orc.NO_HIT).sum() > 500


@pytest.mark.parametrize("n", [0, 1, 2])
def test_sah_tiny_inputs(rt, n):
    tris = rt.gen_soup(6, 0, n, 1.0, 0.01) if n else np.zeros(0, rt.TRIANGLE_DTYPE)
    nodes = rt.build_bvh_sah(tris)
    assert len(nodes) == max(2 * n - 1, 0)
    if n == 1:
        assert nodes[0]["left"] == 0 and nodes[0]["right"] == 0 and nodes[0]["primitiveType"] == rt.PRIM_TRIANGLE


def test_sah_flat_leaves_are_widened(rt, orc):
    """An axis-aligned quad has a flat box; the reference pads such leaf boxes
    (ConstructHLBVH.comp:38-54) so that its strict slab test can enter them.
    The SAH tree widens exactly flat axes by 2^-20 of their magnitude: config
    1's ground quad is hit through it exactly as through the S1 tree through
    the oracle's strict test, and no SAH box is flat."""
    tris, _, rays = rt.gen_config1()
    sah = rt.build_bvh_sah(tris)
    s1, _, _, _ = orc.build_bvh(tris, mode=0)
    for ax in ("X", "Y", "Z"):
        assert np.all(sah["max" + ax] - sah["min" + ax] > 0)
    a, _ = orc.trace(orc.Scene(tris, s1), rays[::5], canonical=True)
    b, _ = orc.trace(orc.Scene(tris, sah), rays[::5], canonical=True)
    assert np.array_equal(a["prim"], b["prim"])
    assert np.array_equal(a["t"].view(np.uint32), b["t"].view(np.uint32))
    ground = len(tris) - 2
    assert (a["prim"] >= ground).sum() > 1000
