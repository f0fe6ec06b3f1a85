"""The GPU LBVH build (rt_build_bvh_device) must emit exactly the node array
of the oracle's transcription of the six S1 passes (ModelSpaceToWorldSpace.comp
to ConstructAABBsOfInternalNodes.comp), and of the host build."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def device_build(rt, torch, tris, spheres=None, mode=0):
    tris = np.ascontiguousarray(tris, dtype=rt.TRIANGLE_DTYPE)
    n = len(tris) + (0 if spheres is None else len(spheres))
    d_t = torch.from_numpy(tris.view(np.uint8)).cuda() if len(tris) else None
    d_s = None if spheres is None else torch.from_numpy(np.ascontiguousarray(spheres).view(np.uint8)).cuda()
    d_n = torch.full((max(2 * n - 1, 1) * 40,), 0xCC, dtype=torch.uint8, device="cuda")
    rt.build_bvh_device(d_t, len(tris), d_s, 0 if spheres is None else len(spheres), d_n, bvh_mode=mode)
    torch.cuda.synchronize()
    return d_n.cpu().numpy().view(rt.NODE_DTYPE)[: 2 * n - 1]


@pytest.mark.parametrize("mode", [0, 1])
def test_device_build_matches_host(rt, cuda, mode):
    tris, _, _ = rt.gen_config1()
    assert np.array_equal(device_build(rt, cuda, tris, mode=mode).view(np.uint8),
                          rt.build_bvh(tris, bvh_mode=mode).view(np.uint8))
    soup = rt.gen_soup(6, 0, 300_000, 1.0, 0.002)
    sph = np.zeros(13, rt.SPHERE_DTYPE)
    sph["center"][:, :3] = np.random.default_rng(3).random((13, 3)).astype(np.float32)
    sph["radius"] = np.float32(0.02)
    assert np.array_equal(device_build(rt, cuda, soup, sph, mode).view(np.uint8),
                          rt.build_bvh(soup, sph, bvh_mode=mode).view(np.uint8))


def test_device_build_edge_cases(rt, cuda):
    t = rt.gen_soup(3, 5, 70_000, 1.0, 0.01)
    for n in (1, 2, 3, 255, 4096, 4097, 65_537):
        for mode in (0, 1):
            assert np.array_equal(device_build(rt, cuda, t[:n], mode=mode).view(np.uint8),
                                  rt.build_bvh(t[:n], bvh_mode=mode).view(np.uint8)), n
    same = np.repeat(t[:1], 5000)  # equal codes everywhere: index tie-break
    assert np.array_equal(device_build(rt, cuda, same).view(np.uint8), rt.build_bvh(same).view(np.uint8))


def test_device_build_config3_and_scene(rt, cuda):
    tris = rt.gen_soup(3, 0, 4_194_304, 1.0, 0.002)
    host = rt.build_bvh(tris)
    assert np.array_equal(device_build(rt, cuda, tris).view(np.uint8), host.view(np.uint8))
    with rt.Scene(tris[:200_000], build_on_device=True) as a, rt.Scene(tris[:200_000]) as b:
        assert np.array_equal(a.nodes().view(np.uint8), b.nodes().view(np.uint8))


@pytest.mark.parametrize("mode", [0, 1], ids=["sorted", "reference"])
def test_device_build_matches_oracle(rt, orc, cuda, mode):
    """The device build against the oracle's transcription of the S1 passes
    (which the CPU suite pins to the reference's own shaders in reference
    mode): config 1, a soup with spheres, duplicate centroids, the full
    config-3 soup, and sizes around the device kernels' block sizes."""
    tris, _, _ = rt.gen_config1()
    assert np.array_equal(device_build(rt, cuda, tris, mode=mode).view(np.uint8),
                          orc.build_bvh(tris, mode=mode)[0].view(np.uint8))
    soup = rt.gen_soup(8, 0, 200_000, 1.0, 0.002)
    sph = np.zeros(40, rt.SPHERE_DTYPE)
    sph["center"][:, :3] = np.random.default_rng(8).random((40, 3)).astype(np.float32)
    sph["radius"] = np.float32(0.01)
    assert np.array_equal(device_build(rt, cuda, soup, sph, mode).view(np.uint8),
                          orc.build_bvh(soup, spheres=sph, mode=mode)[0].view(np.uint8))
    dup = np.concatenate([soup[:500]] * 6)
    assert np.array_equal(device_build(rt, cuda, dup, mode=mode).view(np.uint8),
                          orc.build_bvh(dup, mode=mode)[0].view(np.uint8))
    for n in (1, 2, 255, 256, 257, 1023, 1025):
        assert np.array_equal(device_build(rt, cuda, soup[:n], mode=mode).view(np.uint8),
                              orc.build_bvh(soup[:n], mode=mode)[0].view(np.uint8)), n
    big = rt.gen_soup(3, 0, 4_194_304, 1.0, 0.002)
    assert np.array_equal(device_build(rt, cuda, big, mode=mode).view(np.uint8),
                          orc.build_bvh(big, mode=mode)[0].view(np.uint8))
