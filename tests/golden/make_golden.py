"""Generates the golden fixtures in this directory from the CPU oracle.

The reference ships no test vectors and cannot run here, so these fixtures
freeze the oracle's own outputs (RNG streams, sin/cos, BVH node arrays,
closest/any hits, the Moller-Trumbore mode's hits, a small path-traced
accumulator) on small inputs that are stored alongside, so the checks do not
depend on the generators' libm.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from oracle import oracle as orc  # noqa: E402


def small_scene():
    import raytracergpu_mastersproject_gb300 as rt

    sph = rt.gen_icosphere(2, (0.0, 0.0, 0.0), 1.0, 0)
    ground = rt.gen_config1()[0][-2:]
    tris = np.concatenate([sph, ground])
    ubo = rt.make_ubo((0.0, 0.5, 4.0), (0.0, 0.0, 0.0), fov=60.0, depth=4, random_state=2024)
    rays = rt.gen_camera_rays(ubo, 64, 36)
    mats = np.zeros(2, orc.MAT)
    mats[0]["albedo"][:3] = (0.73, 0.33, 0.25)
    mats[0]["materialType"] = 1
    mats[1]["albedo"][:3] = (3.0, 3.0, 3.0)
    mats[1]["materialType"] = 0
    return tris, ubo, rays, mats


def main():
    import raytracergpu_mastersproject_gb300 as rt

    seeds = np.array([0, 1, 12345, 0xFFFFFFFF, 0x9E3779B9], np.uint32)
    floats, states, units = [], [], []
    for s in seeds:
        f, st = orc.random_stream(int(s), 64)
        floats.append(f)
        states.append(st)
        units.append(orc.random_unit_vectors(int(s), 16))
    np.savez_compressed(HERE / "rng.npz", seeds=seeds, floats=np.array(floats), states=np.array(states),
                        units=np.array(units))

    x = np.linspace(0.0, 2.0 * np.float32(np.pi), 257, dtype=np.float32)
    s = np.array([orc.lib().orc_sin(float(v)) for v in x], np.float32)
    c = np.array([orc.lib().orc_cos(float(v)) for v in x], np.float32)
    np.savez_compressed(HERE / "sincos.npz", x=x, sin=s, cos=c)

    tris, ubo, rays, mats = small_scene()
    n0, codes0, prims0, enc0 = orc.build_bvh(tris, mode=0)
    n1, codes1, prims1, enc1 = orc.build_bvh(tris, mode=1)
    S0 = orc.Scene(tris, n0, mats=mats)
    h0, _ = orc.trace(S0, rays)
    h1, _ = orc.trace(orc.Scene(tris, n1), rays)
    hany, _ = orc.trace(S0, rays, any_hit=True)
    ubo_bytes = np.frombuffer(bytes(ubo), np.uint8)
    w, h, spp = 24, 14, 2
    acc = np.tile(np.array([0, 0, 0, 1], np.float32), w * h)
    assert orc.render(S0, ubo, acc, w, h, spp) == 0
    np.savez_compressed(HERE / "small_scene.npz", tris=tris.view(np.uint8), rays=rays.view(np.uint8),
                        mats=mats.view(np.uint8), ubo=ubo_bytes, nodes_sorted=n0.view(np.uint8),
                        nodes_reference=n1.view(np.uint8), codes_sorted=codes0, codes_reference=codes1,
                        enclosing=enc0, hits_sorted=h0.view(np.uint8), hits_reference=h1.view(np.uint8),
                        hits_any=hany.view(np.uint8), accum=acc, render_wh_spp=np.array([w, h, spp]))

    soup = rt.gen_soup(7, 0, 3000, 1.0, 0.01)
    srays = rt.gen_rays(7, 0, 4096, 1.0, 1e-4, float("inf"))
    sn, _, _, _ = orc.build_bvh(soup, mode=0)
    sh, _ = orc.trace(orc.Scene(soup, sn), srays)
    np.savez_compressed(HERE / "soup_small.npz", tris=soup.view(np.uint8), rays=srays.view(np.uint8),
                        nodes=sn.view(np.uint8), hits=sh.view(np.uint8))
    mt_fixture()
    print("fixtures written to", HERE)


def mt_fixture():
    """The Moller-Trumbore mode's closest hits on the soup_small inputs."""
    g = np.load(HERE / "soup_small.npz")
    soup, srays, sn = g["tris"].view(orc.TRI), g["rays"].view(orc.RAY), g["nodes"].view(orc.NODE)
    mh, _ = orc.trace(orc.Scene(soup, sn), srays, mt=True)
    np.savez_compressed(HERE / "soup_small_mt.npz", hits=mh.view(np.uint8))


if __name__ == "__main__":
    main()
