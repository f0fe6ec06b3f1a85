"""GPU parity of the ray-query path (rt_trace / rt_trace_host) against the CPU oracle.

The oracle restates hitBVH (raytraceBVH.comp:195-265) and triangleHit
(:118-149).  Hit ids must match on every ray except near-ties, which the
binary64 arbiter (oracle.arbitrate) accepts; matching hits must carry the
bit-identical binary32 t.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def dev_trace(rt, torch, scene, rays, any_hit=False, sort=False):
    rays = np.ascontiguousarray(rays, dtype=rt.RAY_DTYPE)
    d_rays = torch.from_numpy(rays.view(np.uint8)).cuda()
    d_hits = torch.full((max(len(rays), 1) * 8,), 0xAB, dtype=torch.uint8, device="cuda")
    scene.trace(d_rays, d_hits, n=len(rays), any_hit=any_hit, sort=sort)
    torch.cuda.synchronize()
    return d_hits.cpu().numpy().view(rt.HIT_DTYPE)[: len(rays)]


def assert_parity(orc, tris, rays, ref, got):
    arb = orc.arbitrate(tris, rays, ref, got)
    assert not arb["unexplained"], f"unexplained mismatches at rays {arb['unexplained'][:10]} ({arb})"
    same = ref["prim"] == got["prim"]
    hit = same & (ref["prim"] != orc.NO_HIT)
    assert np.array_equal(ref["t"][hit].view(np.uint32), got["t"][hit].view(np.uint32)), "t differs on matching hits"
    miss = got["prim"] == orc.NO_HIT
    assert np.all(np.isinf(got["t"][miss]))
    return arb


@pytest.mark.parametrize("width", [2, 4])
@pytest.mark.parametrize("mode", [0, 1], ids=["sorted", "reference"])
def test_config1_matches_reference_order(rt, orc, cuda, mode, width):
    tris, ubo, rays = rt.gen_config1()
    with rt.Scene(tris, bvh_mode=mode, node_width=width) as sc:
        assert sc.info().node_width == width
        got = dev_trace(rt, cuda, sc, rays)
        ref, st = orc.trace(orc.Scene(tris, sc.nodes()), rays)
    assert st[4] == 0
    arb = assert_parity(orc, tris, rays, ref, got)
    assert (got["prim"] != orc.NO_HIT).sum() > 100000
    assert arb["mismatch"] <= 20


@pytest.mark.parametrize("width", [2, 4])
@pytest.mark.parametrize("leaf", [2, 4, 8])
def test_collapsed_leaves_same_hits(rt, orc, cuda, leaf, width):
    tris, ubo, rays = rt.gen_config1()
    with rt.Scene(tris, node_width=width) as base, rt.Scene(tris, leaf_size=leaf, node_width=width) as sc:
        a = dev_trace(rt, cuda, base, rays)
        b = dev_trace(rt, cuda, sc, rays)
        assert sc.info().device_nodes < base.info().device_nodes
        ref, _ = orc.trace(orc.Scene(tris, sc.nodes()), rays)
    assert_parity(orc, tris, rays, ref, b)
    assert_parity(orc, tris, rays, a, b)


@pytest.mark.parametrize("width", [2, 4])
def test_soup_matches_oracle(rt, orc, cuda, width):
    tris = rt.gen_soup(11, 0, 200_000, 1.0, 0.004)
    rays = rt.gen_rays(11, 0, 300_000, 1.0, 1e-4, float("inf"))
    with rt.Scene(tris, node_width=width) as sc:
        got = dev_trace(rt, cuda, sc, rays)
        S = orc.Scene(tris, sc.nodes())
    can, _ = orc.trace(S, rays, canonical=True)
    assert_parity(orc, tris, rays, can, got)
    ref, _ = orc.trace(S, rays[:20000])
    assert_parity(orc, tris, rays[:20000], ref, got[:20000])


@pytest.mark.parametrize("width", [2, 4])
def test_any_hit_semantics(rt, orc, cuda, width):
    tris = rt.gen_soup(12, 0, 100_000, 1.0, 0.004)
    rays = rt.gen_rays(12, 0, 100_000, 1.0, 1e-4, 0.05)
    with rt.Scene(tris, node_width=width) as sc:
        anyh = dev_trace(rt, cuda, sc, rays, any_hit=True)
        close = dev_trace(rt, cuda, sc, rays)
        ref, _ = orc.trace(orc.Scene(tris, sc.nodes()), rays, canonical=True)
    assert np.array_equal(anyh["prim"] != orc.NO_HIT, ref["prim"] != orc.NO_HIT)
    assert np.array_equal(close["prim"] != orc.NO_HIT, ref["prim"] != orc.NO_HIT)
    idx = np.nonzero(anyh["prim"] != orc.NO_HIT)[0]
    for i in idx[:: max(1, len(idx) // 500)]:
        t = orc.triangle_test(tris[anyh["prim"][i]], rays[i:i + 1])
        assert t is not None and np.float32(t) == anyh["t"][i]
        assert anyh["t"][i] >= close["t"][i]


def test_config3_full_size(rt, orc, cuda):
    """4,194,304 triangles, 16,777,216 rays: every ray against the oracle's
    canonical traversal, and the first 2,097,152 against the reference's own
    order (push left, go right, no culling: raytraceBVH.comp:236-244) with
    binary64 arbitration; any-hit agrees with closest-hit on which rays hit;
    a second run is bit-identical."""
    tris = rt.gen_soup(3, 0, 4_194_304, 1.0, 0.002)
    rays = rt.gen_rays(3, 0, 16_777_216, 1.0, 1e-4, float("inf"))
    with rt.Scene(tris) as sc:
        got = dev_trace(rt, cuda, sc, rays)
        again = dev_trace(rt, cuda, sc, rays, sort=True)
        anyh = dev_trace(rt, cuda, sc, rays, any_hit=True, sort=True)
        S = orc.Scene(tris, sc.nodes())
    assert np.array_equal(got.view(np.uint64), again.view(np.uint64))  # reordering changes nothing
    assert np.array_equal(got["prim"] != orc.NO_HIT, anyh["prim"] != orc.NO_HIT)
    can, _ = orc.trace(S, rays, canonical=True)
    arb = assert_parity(orc, tris, rays, can, got)
    assert arb["mismatch"] < 1000
    k = 2_097_152
    ref, st = orc.trace(S, rays[:k])
    assert st[4] == 0
    arb = assert_parity(orc, tris, rays[:k], ref, got[:k])
    assert arb["mismatch"] < 200


def test_trace_host_matches_device(rt, cuda):
    tris = rt.gen_soup(13, 0, 50_000, 1.0, 0.004)
    rays = rt.gen_rays(13, 0, 5_000_000, 1.0, 1e-4, float("inf"))
    with rt.Scene(tris) as sc:
        a = dev_trace(rt, cuda, sc, rays)
        b = sc.trace_host(rays)
        pinned = cuda.from_numpy(rays.view(np.uint8)).pin_memory()
        c = sc.trace_host(pinned.numpy().view(rt.RAY_DTYPE))
        # 5 M rays: chunks of 2 Mi, the rest but 512 Ki, and 512 Ki, on both buffers and both trace streams
        d = sc.trace_host(pinned.numpy().view(rt.RAY_DTYPE), sort=True)
        e = sc.trace_host(pinned.numpy().view(rt.RAY_DTYPE), any_hit=True)
        f = dev_trace(rt, cuda, sc, rays, any_hit=True)
        # page-locked hits: staged by default; with RT_HOST_DIRECT_HITS=1 the kernels write them directly
        out_t = cuda.full((len(rays) * 8,), 0xCD, dtype=cuda.uint8).pin_memory()
        out = out_t.numpy().view(rt.HIT_DTYPE)
        g = sc.trace_host(pinned.numpy().view(rt.RAY_DTYPE), out=out, sort=True).copy()
        out_t.fill_(0xCD)
        h = sc.trace_host(rays, out=out, any_hit=True).copy()
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
    assert np.array_equal(a.view(np.uint64), c.view(np.uint64))
    assert np.array_equal(a.view(np.uint64), d.view(np.uint64))
    assert np.array_equal(e.view(np.uint64), f.view(np.uint64))
    assert np.array_equal(a.view(np.uint64), g.view(np.uint64))
    assert np.array_equal(f.view(np.uint64), h.view(np.uint64))


def test_caller_supplied_nodes(rt, orc, cuda):
    tris, ubo, rays = rt.gen_config1()
    nodes, _, _, _ = orc.build_bvh(tris, mode=1)
    with rt.Scene(tris, nodes=nodes) as sc, rt.Scene(tris, bvh_mode=1) as sc2:
        assert np.array_equal(sc.nodes().view(np.uint8), nodes.view(np.uint8))
        a = dev_trace(rt, cuda, sc, rays)
        b = dev_trace(rt, cuda, sc2, rays)
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


@pytest.mark.parametrize("width", [2, 4])
def test_spheres_and_models(rt, orc, cuda, width):
    tris = rt.gen_icosphere(2, (0.0, 0.0, 0.0), 1.0, 0)
    tris["modelIndex"] = 0
    sph = np.zeros(3, rt.SPHERE_DTYPE)
    sph["center"][:, :3] = [(2.5, 0, 0), (-2.5, 0.5, 0), (0, 2.5, -1)]
    sph["radius"] = [0.7, 0.5, 0.9]
    sph["modelIndex"] = [1, 1, 0]
    models = np.zeros(2, rt.MODEL_DTYPE)
    models[0]["m"] = np.eye(4, dtype=np.float32).T.ravel()
    m = np.eye(4, dtype=np.float32)
    m[:3, 3] = (0.25, -0.5, 0.125)
    m[0, 0] = 1.5
    models[1]["m"] = m.T.ravel()  # column-major
    ubo = rt.make_ubo((0.0, 0.5, 6.0), (0.0, 0.0, 0.0), fov=70.0)
    rays = rt.gen_camera_rays(ubo, 160, 90)
    with rt.Scene(tris, spheres=sph, models=models, node_width=width) as sc:
        got = dev_trace(rt, cuda, sc, rays)
        nodes = sc.nodes()
    onodes, _, _, _ = orc.build_bvh(tris, sph, mode=0, models=models["m"])
    assert np.array_equal(nodes.view(np.uint8), onodes.view(np.uint8))
    # the oracle traces world-space records: transform them the same way
    wt, ws = world(rt, tris, sph, models)
    ref, _ = orc.trace(orc.Scene(wt, nodes, spheres=ws), rays)
    assert np.array_equal(ref["prim"], got["prim"])
    hit = ref["prim"] != orc.NO_HIT
    assert np.array_equal(ref["t"][hit].view(np.uint32), got["t"][hit].view(np.uint32))
    assert ((got["prim"] & rt.HIT_SPHERE_BIT) != 0).sum() > 100


def world(rt, tris, sph, models):
    """ModelSpaceToWorldSpace.comp:32-48 in numpy binary32, left-to-right sums."""
    M = models["m"].reshape(-1, 4, 4)  # [model][column][row]

    def xf(m, v):
        out = np.zeros(4, np.float32)
        for r in range(4):
            acc = np.float32(m[0, r] * v[0])
            acc = np.float32(acc + np.float32(m[1, r] * v[1]))
            acc = np.float32(acc + np.float32(m[2, r] * v[2]))
            acc = np.float32(acc + np.float32(m[3, r] * np.float32(1.0)))
            out[r] = acc
        return out

    wt = tris.copy()
    for i in range(len(wt)):
        for k in ("v0", "v1", "v2"):
            wt[i][k] = xf(M[wt[i]["modelIndex"]], wt[i][k])
    ws = sph.copy()
    for i in range(len(ws)):
        ws[i]["center"] = xf(M[ws[i]["modelIndex"]], ws[i]["center"])
    return wt, ws


@pytest.mark.parametrize("width", [2, 4])
def test_edge_cases(rt, orc, cuda, width):
    # one triangle; axis-aligned and grazing rays; ray starting on the triangle; tmax < tmin
    t = np.zeros(2, rt.TRIANGLE_DTYPE)
    t[0]["v0"][:3] = (0, 0, 0)
    t[0]["v1"][:3] = (1, 0, 0)
    t[0]["v2"][:3] = (0, 1, 0)
    t[1]["v0"][:3] = (5, 5, 5)  # zero-area: defined as never hit
    t[1]["v1"][:3] = (5, 5, 5)
    t[1]["v2"][:3] = (6, 6, 6)
    r = np.zeros(8, rt.RAY_DTYPE)
    r["tmin"] = 0.0
    r["tmax"] = np.inf
    r[0]["org"], r[0]["dir"] = (0.25, 0.25, 1.0), (0, 0, -1)      # straight down the z axis
    r[1]["org"], r[1]["dir"] = (0.25, 0.25, -1.0), (0, 0, 1)      # from below
    r[2]["org"], r[2]["dir"] = (-1, 0.5, 0.0), (1, 0, 0)          # in the plane: parallel
    r[3]["org"], r[3]["dir"] = (0.2, 0.2, 0.0), (0, 0, 1)         # starts on the triangle
    r[4]["org"], r[4]["dir"] = (0.25, 0.25, 1.0), (0, 0, -1)
    r[4]["tmax"] = 0.5                                            # hit beyond tmax
    r[5]["org"], r[5]["dir"] = (0.25, 0.25, 1.0), (0, 0, -1)
    r[5]["tmin"], r[5]["tmax"] = 2.0, 1.0                         # empty interval
    r[6]["org"], r[6]["dir"] = (5.5, 5.5, 4.0), (0, 0, 1)         # through the zero-area one
    r[7]["org"], r[7]["dir"] = (1.0, 0.0, 1.0), (0, 0, -1)        # exactly on a vertex
    with rt.Scene(t, node_width=width) as sc:
        got = dev_trace(rt, cuda, sc, r)
        ref, _ = orc.trace(orc.Scene(t, sc.nodes()), r)
    # Ray 7 lies in the plane x = 1 of the leaf box's face with d.x = 0: the
    # reference's slab test computes 0/0 there and rejects the box, the kernels
    # keep a box whose face the ray touches.  The vertex hit they may report
    # must pass the reference's own triangle test.
    if got["prim"][7] != ref["prim"][7]:
        assert ref["prim"][7] == orc.NO_HIT and orc.triangle_test(t[got["prim"][7]], r[7:8]) == got["t"][7]
    keep = np.arange(len(r)) != 7
    assert np.array_equal(got["prim"][keep], ref["prim"][keep]), (got, ref)
    assert list(got["prim"][:2]) == [0, 0]
    assert got["prim"][2] == orc.NO_HIT and got["prim"][4] == orc.NO_HIT and got["prim"][5] == orc.NO_HIT
    assert got["prim"][6] == orc.NO_HIT
    hit = (ref["prim"] != orc.NO_HIT) & keep
    assert np.array_equal(got["t"][hit], ref["t"][hit])
    # empty scene: every ray misses; zero rays is a no-op
    with rt.Scene(np.zeros(0, rt.TRIANGLE_DTYPE), node_width=width) as empty:
        g = dev_trace(rt, cuda, empty, r)
        assert np.all(g["prim"] == orc.NO_HIT)
        empty.trace(cuda.empty(0, dtype=cuda.uint8, device="cuda"), cuda.empty(0, dtype=cuda.uint8, device="cuda"), n=0)


def test_golden_fixtures_on_gpu(rt, orc, cuda):
    from pathlib import Path

    g = np.load(Path(__file__).resolve().parent / "golden" / "small_scene.npz")
    tris = g["tris"].view(rt.TRIANGLE_DTYPE)
    rays = g["rays"].view(rt.RAY_DTYPE)
    for mode, key in ((0, "sorted"), (1, "reference")):
        with rt.Scene(tris, bvh_mode=mode) as sc:
            assert np.array_equal(sc.nodes().view(np.uint8), g[f"nodes_{key}"])
            got = dev_trace(rt, cuda, sc, rays)
            want = g[f"hits_{key}"].view(rt.HIT_DTYPE)
            assert_parity(orc, tris, rays, want, got)
            anyh = dev_trace(rt, cuda, sc, rays, any_hit=True)
            assert np.array_equal(anyh["prim"] != rt.NO_HIT, want["prim"] != rt.NO_HIT)
    s = np.load(Path(__file__).resolve().parent / "golden" / "soup_small.npz")
    st, sr = s["tris"].view(rt.TRIANGLE_DTYPE), s["rays"].view(rt.RAY_DTYPE)
    with rt.Scene(st) as sc:
        got = dev_trace(rt, cuda, sc, sr)
        d_rays = cuda.from_numpy(np.ascontiguousarray(sr).view(np.uint8)).cuda()
        d_hits = cuda.empty(len(sr) * 8, dtype=cuda.uint8, device="cuda")
        sc.trace(d_rays, d_hits, mt=True)
        cuda.cuda.synchronize()
        got_mt = d_hits.cpu().numpy().view(rt.HIT_DTYPE).copy()
    assert_parity(orc, st, sr, s["hits"].view(rt.HIT_DTYPE), got)
    m = np.load(Path(__file__).resolve().parent / "golden" / "soup_small_mt.npz")
    assert_mt_parity(orc, m["hits"].view(rt.HIT_DTYPE), got_mt)


@pytest.mark.parametrize("width", [2, 4])
def test_work_counters(rt, cuda, width):
    tris = rt.gen_soup(14, 0, 100_000, 1.0, 0.004)
    rays = rt.gen_rays(14, 0, 200_000, 1.0, 1e-4, float("inf"))
    with rt.Scene(tris, node_width=width) as sc:
        d_rays = cuda.from_numpy(rays.view(np.uint8)).cuda()
        a = cuda.empty(len(rays) * 8, dtype=cuda.uint8, device="cuda")
        b = cuda.empty_like(a)
        sc.trace(d_rays, a)
        nodes, tests = sc.trace_count(d_rays, b)
    assert cuda.equal(a, b)
    assert nodes > len(rays) and tests > len(rays) // 2


@pytest.mark.parametrize("width", [2, 4])
def test_sorted_order_same_hits(rt, cuda, width):
    tris = rt.gen_soup(15, 0, 150_000, 1.0, 0.004)
    rays = rt.gen_rays(15, 0, 1_000_003, 1.0, 1e-4, float("inf"))
    cam_tris, ubo, cam_rays = rt.gen_config1()
    with rt.Scene(tris, node_width=width) as sc, rt.Scene(cam_tris, node_width=width) as cam:
        for anyh in (False, True):
            a = dev_trace(rt, cuda, sc, rays, any_hit=anyh)
            b = dev_trace(rt, cuda, sc, rays, any_hit=anyh, sort=True)
            assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
        # every camera ray starts at one point: a single bucket
        a = dev_trace(rt, cuda, cam, cam_rays)
        b = dev_trace(rt, cuda, cam, cam_rays, sort=True)
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
        c = sc.trace_host(rays[:300_000], sort=True)
        assert np.array_equal(c.view(np.uint64), dev_trace(rt, cuda, sc, rays[:300_000]).view(np.uint64))


def _axis_rays(rt, n, scale, seed):
    """Rays inside a cube of side `scale`, half of them along +-x/y/z exactly
    (two zero direction components), the rest with one zero component."""
    rng = np.random.default_rng(seed)
    rays = np.zeros(n, rt.RAY_DTYPE)
    o = rng.uniform(0.0, scale, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    axis = rng.integers(0, 3, n)
    half = n // 2
    d[:half] = 0.0
    d[np.arange(half), axis[:half]] = rng.choice([-1.0, 1.0], half)
    d[np.arange(half, n), axis[half:]] = 0.0
    d /= np.sqrt((d.astype(np.float64) ** 2).sum(1, keepdims=True)).astype(np.float32)
    rays["org"] = o
    rays["tmin"] = 0.0
    rays["dir"] = d
    rays["tmax"] = np.float32(np.inf)
    return rays


@pytest.mark.parametrize("scale", [1.0, 1.0e7, 1.0e9])
def test_axis_parallel_rays_at_large_scales(rt, orc, cuda, scale):
    """Direction components of exactly 0 in scenes up to 1e9 wide (4-wide
    steps up to 2^22; far beyond that the reference's own triangle test
    overflows binary32): the node step's scale A = 2^(e+15)/d stays finite
    and conservative, and both layouts match the oracle."""
    tris = rt.gen_soup(31, 0, 30_000, 1.0, 0.01)
    for k in ("v0", "v1", "v2"):
        tris[k][:, :3] *= np.float32(scale)
    rays = _axis_rays(rt, 40_000, scale, 5)
    with rt.Scene(tris, node_width=4) as s4, rt.Scene(tris, node_width=2) as s2:
        assert s4.info().node_width == 4
        got4 = dev_trace(rt, cuda, s4, rays)
        got2 = dev_trace(rt, cuda, s2, rays)
        ref, _ = orc.trace(orc.Scene(tris, s4.nodes()), rays, canonical=True)
    assert (ref["prim"] != orc.NO_HIT).sum() > 1000
    assert_parity(orc, tris, rays, ref, got4)
    assert_parity(orc, tris, rays, ref, got2)


def test_extent_beyond_wide_range_uses_binary_nodes(rt, orc, cuda):
    """Beyond 255 * 2^48 the 4-wide quantisation is not used: the default
    layout falls back to binary nodes and an explicit width of 4 is refused."""
    tris = rt.gen_soup(32, 0, 5_000, 1.0, 0.01)
    for k in ("v0", "v1", "v2"):
        tris[k][:, :3] *= np.float32(1.0e17)
    rays = _axis_rays(rt, 10_000, 1.0e17, 6)
    with rt.Scene(tris) as sc:
        assert sc.info().node_width == 2
        got = dev_trace(rt, cuda, sc, rays)
        ref, _ = orc.trace(orc.Scene(tris, sc.nodes()), rays)
    assert_parity(orc, tris, rays, ref, got)
    with pytest.raises(rt.RtError) as e:
        rt.Scene(tris, node_width=4)
    assert e.value.status == 1


def _dense_cluster(rt, n, seed):
    """n large triangles crossing one small region: rays through it test
    thousands of boxes and keep deep traversal stacks."""
    rng = np.random.default_rng(seed)
    tris = np.zeros(n, rt.TRIANGLE_DTYPE)
    c = rng.normal(0.0, 0.05, (n, 3)).astype(np.float32)
    for k in ("v0", "v1", "v2"):
        tris[k][:, :3] = c + rng.normal(0.0, 0.5, (n, 3)).astype(np.float32)
    return tris


def _rays_at_origin(rt, n, seed):
    rng = np.random.default_rng(seed)
    rays = np.zeros(n, rt.RAY_DTYPE)
    o = rng.uniform(-3.0, 3.0, (n, 3)).astype(np.float32)
    d = (-o + rng.normal(0.0, 0.1, (n, 3))).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays["org"], rays["dir"], rays["tmin"], rays["tmax"] = o, d, 0.0, np.float32(np.inf)
    return rays


def test_deep_stacks_spill_the_shared_ring(rt, orc, cuda):
    """About 5,500 box tests and 400 triangle tests per ray: traversal stacks
    run far past the 16 entries each lane keeps in shared memory, so entries
    move out to local memory and back.  Hits match the oracle for both ray
    kinds, both node layouts and the sorted order."""
    tris = _dense_cluster(rt, 20_000, 3)
    rays = _rays_at_origin(rt, 20_000, 4)
    with rt.Scene(tris, node_width=4) as s4, rt.Scene(tris, node_width=2) as s2:
        assert s4.info().stack_need > 16
        closest4 = dev_trace(rt, cuda, s4, rays)
        sorted4 = dev_trace(rt, cuda, s4, rays, sort=True)
        closest2 = dev_trace(rt, cuda, s2, rays)
        any4 = dev_trace(rt, cuda, s4, rays, any_hit=True)
        ref, st = orc.trace(orc.Scene(tris, s4.nodes()), rays, canonical=True)
    assert st[0] / len(rays) > 1000  # boxes tested per ray
    assert_parity(orc, tris, rays, ref, closest4)
    assert_parity(orc, tris, rays, ref, closest2)
    assert np.array_equal(closest4.view(np.uint64), sorted4.view(np.uint64))
    hit = ref["prim"] != orc.NO_HIT
    assert np.array_equal(any4["prim"] != orc.NO_HIT, hit)  # any-hit finds a hit exactly where one exists


def _t64_errors(orc, tris, rays, hits):
    i = np.nonzero(hits["prim"] != orc.NO_HIT)[0]
    t64 = np.array([orc.triangle_t64(tris[hits["prim"][k]], rays[k])[0] for k in i])
    return i, t64, np.abs(hits["t"][i].astype(np.float64) - t64)


def test_hit_t_against_fp64(rt, orc, cuda):
    """Hit t against the same triangle intersected in binary64.  Config 1:
    within 1e-5 relative on every hit.  A config-3 soup: the reference's
    binary32 plane test, D - dot(n, o), cancels for short hits, so the bound
    there is 1e-5 of max(t, scene extent 1); the kernels return the
    reference's binary32 t bit for bit either way."""
    tris, ubo, rays = rt.gen_config1()
    with rt.Scene(tris) as sc:
        got = dev_trace(rt, cuda, sc, rays[::2])
    i, t64, err = _t64_errors(orc, tris, rays[::2], got)
    assert len(i) > 50_000
    assert np.all(err <= 1e-5 * np.abs(t64))

    from raytracergpu_mastersproject_gb300 import workloads as W
    tris3, rays3 = W.config3(262_144, 50_000)
    with rt.Scene(tris3) as sc:
        got3 = dev_trace(rt, cuda, sc, rays3)
    i3, t3, err3 = _t64_errors(orc, tris3, rays3, got3)
    assert len(i3) > 10_000
    assert np.all(err3 <= 1e-5 * np.maximum(np.abs(t3), 1.0))


def test_degenerate_rays(rt, orc, cuda):
    """NaN and infinite components, an all-zero direction, tmin > tmax, an
    empty interval and negative tmin: no fault, and the same answer as the
    oracle's restatement.  A NaN origin or direction gives NaN parameters,
    which never hit; a NaN tmax rejects nothing, as in the reference's
    `t < tMin || tMax < t`, so it acts as +inf."""
    tris = rt.gen_soup(41, 0, 20_000, 1.0, 0.01)
    base = rt.gen_rays(41, 0, 4_096, 1.0, 1e-4, float("inf"))
    rays = np.concatenate([base] * 8)
    k = len(base)
    nan, inf = np.float32(np.nan), np.float32(np.inf)
    rays["org"][0 * k:1 * k, 0] = nan
    rays["dir"][1 * k:2 * k, 1] = nan
    rays["dir"][2 * k:3 * k] = 0.0
    rays["tmin"][3 * k:4 * k] = 2.0
    rays["tmax"][3 * k:4 * k] = 1.0
    rays["tmin"][4 * k:5 * k] = 0.25
    rays["tmax"][4 * k:5 * k] = 0.25
    rays["tmin"][5 * k:6 * k] = -1.0
    rays["org"][6 * k:7 * k, 2] = inf
    rays["tmax"][7 * k:8 * k] = nan
    with rt.Scene(tris, node_width=4) as s4, rt.Scene(tris, node_width=2) as s2:
        got4 = dev_trace(rt, cuda, s4, rays)
        got4s = dev_trace(rt, cuda, s4, rays, sort=True)
        got2 = dev_trace(rt, cuda, s2, rays)
        any4 = dev_trace(rt, cuda, s4, rays, any_hit=True)
        ref, _ = orc.trace(orc.Scene(tris, s4.nodes()), rays, canonical=True)
    for got in (got4, got2):
        assert_parity(orc, tris, rays, ref, got)
    assert np.array_equal(got4.view(np.uint64), got4s.view(np.uint64))
    assert np.array_equal(any4["prim"] != orc.NO_HIT, ref["prim"] != orc.NO_HIT)
    for blk in (0, 1, 2, 3):  # NaN origin/direction, zero direction, tmin > tmax
        assert np.all(got4["prim"][blk * k:(blk + 1) * k] == orc.NO_HIT), blk
    # NaN tmax behaves as +inf: the same hits as the unmodified rays
    base_hits = dev_trace(rt, cuda, rt.Scene(tris, node_width=4), base)
    assert np.array_equal(got4[7 * k:].view(np.uint64), base_hits.view(np.uint64))


def assert_mt_parity(orc, ref, got):
    """Moller-Trumbore results against the oracle's MT mode: ids equal except
    where both answers have the same t within 1e-6 (a near-tie); matching
    hits carry the bit-identical binary32 t."""
    diff = np.nonzero(ref["prim"] != got["prim"])[0]
    for i in diff:
        a, b = float(ref["t"][i]), float(got["t"][i])
        assert ref["prim"][i] != orc.NO_HIT and got["prim"][i] != orc.NO_HIT, (i, ref[i], got[i])
        assert abs(a - b) <= 1e-6 * abs(a), (i, ref[i], got[i])
    same = (ref["prim"] == got["prim"]) & (ref["prim"] != orc.NO_HIT)
    assert np.array_equal(ref["t"][same].view(np.uint32), got["t"][same].view(np.uint32))
    return len(diff)


@pytest.mark.parametrize("width", [2, 4])
def test_mt_mode_matches_oracle(rt, orc, cuda, width):
    """RT_TRACE_MT against the oracle's Moller-Trumbore restatement: config 1
    and a soup, closest hit (plain, sorted, host buffers) and any hit."""
    tris, _, rays = rt.gen_config1()
    soup = rt.gen_soup(31, 0, 200_000, 1.0, 0.004)
    srays = rt.gen_rays(31, 0, 200_000, 1.0, 1e-4, float("inf"))
    for t, r in ((tris, rays), (soup, srays)):
        with rt.Scene(t, node_width=width) as sc:
            assert sc.info().node_width == width
            d_rays = cuda.from_numpy(np.ascontiguousarray(r).view(np.uint8)).cuda()
            d_hits = cuda.empty(len(r) * 8, dtype=cuda.uint8, device="cuda")
            sc.trace(d_rays, d_hits, mt=True)
            cuda.cuda.synchronize()
            got = d_hits.cpu().numpy().view(rt.HIT_DTYPE).copy()
            sc.trace(d_rays, d_hits, mt=True, sort=True)
            cuda.cuda.synchronize()
            again = d_hits.cpu().numpy().view(rt.HIT_DTYPE).copy()
            host = sc.trace_host(r, mt=True, sort=True)
            sc.trace(d_rays, d_hits, mt=True, any_hit=True)
            cuda.cuda.synchronize()
            anyh = d_hits.cpu().numpy().view(rt.HIT_DTYPE).copy()
            ref, st = orc.trace(orc.Scene(t, sc.nodes()), r, canonical=True, mt=True)
        assert st[4] == 0
        assert (ref["prim"] != orc.NO_HIT).sum() > 0.1 * len(r)
        assert assert_mt_parity(orc, ref, got) <= 0.001 * len(r)
        assert np.array_equal(got.view(np.uint64), again.view(np.uint64))
        assert np.array_equal(got.view(np.uint64), host.view(np.uint64))
        assert np.array_equal(anyh["prim"] != orc.NO_HIT, ref["prim"] != orc.NO_HIT)
        hit = np.nonzero(anyh["prim"] != orc.NO_HIT)[0]
        assert np.all(anyh["t"][hit] >= got["t"][hit])


def test_mt_mode_rejected_where_unsupported(rt, cuda):
    """rt_trace_count and the pool have no Moller-Trumbore instantiation: the
    flag is refused with RT_EINVAL, not ignored."""
    tris, _, rays = rt.gen_config1()
    with rt.Scene(tris) as sc:
        d_rays = cuda.from_numpy(np.ascontiguousarray(rays[:1024]).view(np.uint8)).cuda()
        d_hits = cuda.empty(1024 * 8, dtype=cuda.uint8, device="cuda")
        c = (C.c_uint64 * 2)()
        st = rt.lib().rt_trace_count(sc.handle, d_rays.data_ptr(), 1024, d_hits.data_ptr(), rt.TRACE_MT, None, c)
        assert rt.STATUS[st] == "RT_EINVAL"


def test_autotune_and_every_tuning_same_hits(rt, orc, cuda):
    """rt_trace_autotune picks a launch (shape, refill, stack capacity, staged
    top-of-tree tile) on the caller's batch; every tuning gives the same hits,
    bit for bit, and settings a scene cannot run are refused."""
    tris = rt.gen_soup(31, 0, 200_000, 1.0, 0.002)
    rays = rt.gen_rays(31, 0, 400_000, 1.0, 1e-4, float("inf"))
    with rt.Scene(tris) as sc:
        base = dev_trace(rt, cuda, sc, rays)
        base_any = dev_trace(rt, cuda, sc, rays, any_hit=True)
        d_rays = cuda.from_numpy(rays.view(np.uint8)).cuda()
        d_hits = cuda.empty(len(rays) * 8, dtype=cuda.uint8, device="cuda")
        t = sc.autotune(d_rays, d_hits, sort=True, repeats=1)
        assert t.best_ms > 0 and t.stack_entries >= sc.info().stack_need
        got = sc.tuning()
        assert (got.launch_shape, got.refill, got.stack_entries, got.tile_nodes) == \
               (t.launch_shape, t.refill, t.stack_entries, t.tile_nodes)
        assert np.array_equal(dev_trace(rt, cuda, sc, rays, sort=True).view(np.uint64), base.view(np.uint64))
        need = sc.info().stack_need
        for stack in (48, 64, 96, 192):
            for tile in (0, 16, 64):
                if stack < need:
                    with pytest.raises(rt.RtError):
                        sc.set_tuning(rt.TraceTuning(12, 5, stack, tile, 0.0))
                    continue
                sc.set_tuning(rt.TraceTuning(12, 5, stack, tile, 0.0))
                assert np.array_equal(dev_trace(rt, cuda, sc, rays).view(np.uint64), base.view(np.uint64)), (stack, tile)
                assert np.array_equal(dev_trace(rt, cuda, sc, rays, any_hit=True).view(np.uint64),
                                      base_any.view(np.uint64)), (stack, tile)
        host = sc.trace_host(rays)
        assert np.array_equal(host.view(np.uint64), base.view(np.uint64))
        shapes = 0
        while True:  # every launch shape the library has, until the first unknown one
            try:
                sc.set_tuning(rt.TraceTuning(shapes, 5, 0, 0, 0.0))
            except rt.RtError:
                break
            assert np.array_equal(dev_trace(rt, cuda, sc, rays, sort=True).view(np.uint64),
                                  base.view(np.uint64)), shapes
            assert np.array_equal(dev_trace(rt, cuda, sc, rays, any_hit=True).view(np.uint64),
                                  base_any.view(np.uint64)), shapes
            shapes += 1
        assert shapes >= 16
        with pytest.raises(rt.RtError):
            sc.set_tuning(rt.TraceTuning(12, 5, 8, 0, 0.0))    # below the tree's worst case
        with pytest.raises(rt.RtError):
            sc.set_tuning(rt.TraceTuning(3, 5, 64, 16, 0.0))  # tiles only on the default shape
    ref, _ = orc.trace(orc.Scene(tris, orc.build_bvh(tris, mode=0)[0]), rays[:50_000], canonical=True)
    assert_parity(orc, tris, rays[:50_000], ref, base[:50_000])


def test_ray_and_hit_alignment(rt, orc, cuda):
    """Rays are read as one 32-byte load when the array is 32-byte aligned and
    as two 16-byte loads otherwise, with the same hits; a ray array off a
    16-byte boundary or a hit array off an 8-byte boundary is refused with
    RT_EINVAL before anything is launched."""
    tris = rt.gen_soup(5, 0, 20_000, 1.0, 0.01)
    rays = rt.gen_rays(5, 0, 30_000, 1.0, 1e-4, float("inf"))
    n = len(rays)
    f = rt.lib().rt_trace
    with rt.Scene(tris) as sc:
        ref = dev_trace(rt, cuda, sc, rays)
        raw = cuda.from_numpy(rays.view(np.uint8)).cuda()
        buf = cuda.zeros(n * 32 + 64, dtype=cuda.uint8, device="cuda")
        hits = cuda.full((n * 8 + 64,), 0xAB, dtype=cuda.uint8, device="cuda")
        assert buf.data_ptr() % 256 == 0 and hits.data_ptr() % 256 == 0
        st = cuda.cuda.current_stream().cuda_stream
        for flags in (0, 2):  # as given, and origin-bucketed
            for off in (16, 32, 48):  # 16-byte aligned, not always 32
                buf[off:off + n * 32].copy_(raw)
                hits.fill_(0xAB)
                assert f(sc.handle, buf.data_ptr() + off, n, hits.data_ptr() + 8, flags, st) == 0
                cuda.cuda.synchronize()
                got = hits[8:8 + n * 8].cpu().numpy().view(rt.HIT_DTYPE)
                assert np.array_equal(got.view(np.uint64), ref.view(np.uint64)), (flags, off)
        for roff, hoff in ((4, 0), (8, 0), (0, 4)):
            assert f(sc.handle, buf.data_ptr() + roff, n, hits.data_ptr() + hoff, 0, st) == 1  # RT_EINVAL
            assert b"aligned" in rt.lib().rt_last_error_string()
    assert (ref["prim"] != orc.NO_HIT).sum() > n // 10
