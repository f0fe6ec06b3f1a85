"""Seeded synthetic workloads of the benchmark configurations 3-5.

Every draw comes from the library's counter-based generators (splitmix64 of
seed/stream/index), so each workload is identical on every machine and for
any thread count.

  config 3  one 4,194,304-triangle soup in the unit cube, 16,777,216 rays
  config 4  256 soups, triangle counts log-uniform in [1K, 256K], each with
            a ray batch log-uniform in [4K, 1M]; each soup fills a cube of
            side (n/4,194,304)^(1/3), so triangle size and density match
            config 3
  config 5  64 resident soups with counts log-uniform in [64K, 4M], built the
            same way; requests draw ray counts log-uniform in [1K, 2M]
"""
from __future__ import annotations

import numpy as np

from . import gen_rays, gen_soup, gen_uniform

CONFIG3_TRIS = 4_194_304
CONFIG3_RAYS = 16_777_216


def log_uniform(u, lo: float, hi: float):
    return np.exp(np.log(lo) + (np.log(hi) - np.log(lo)) * np.asarray(u))


def soup_side(n_tris: int) -> float:
    """Cube side that keeps config 3's triangle density."""
    return float((n_tris / CONFIG3_TRIS) ** (1.0 / 3.0))


def config3(n_tris: int = CONFIG3_TRIS, n_rays: int = CONFIG3_RAYS):
    return gen_soup(3, 0, n_tris, 1.0, 0.002), gen_rays(3, 0, n_rays, 1.0, 1e-4, float("inf"))


def config4_sizes(count: int = 256, tri_range=(1_000, 256_000), ray_range=(4_000, 1_000_000)):
    u = gen_uniform(4, 99, 2 * count)
    tris = np.rint(log_uniform(u[0::2], *tri_range)).astype(np.int64)
    rays = np.rint(log_uniform(u[1::2], *ray_range)).astype(np.int64)
    return tris, rays


def config4(count: int = 256, tri_range=(1_000, 256_000), ray_range=(4_000, 1_000_000)):
    """-> list of (triangles, rays) per scene."""
    nt, nr = config4_sizes(count, tri_range, ray_range)
    out = []
    for i in range(count):
        side = soup_side(int(nt[i]))
        out.append((gen_soup(4, i + 1, int(nt[i]), side, 0.002),
                    gen_rays(4, i + 1, int(nr[i]), side, 1e-4, float("inf"))))
    return out


def config5_scene(i: int, tri_range=(64_000, 4_000_000)):
    """Scene i of the serving workload (resident scenes and later uploads).

    Stored scaled to the unit cube: n triangles with vertex offsets
    N(0, (0.002/s)^2), s = soup_side(n) -- config 4's construction divided by s,
    so that one batch of unit-cube rays serves every scene.  Traversal work is
    invariant under the uniform scaling; t values scale by 1/s."""
    u = gen_uniform(5, 1_000_000 + i, 1)
    nt = int(np.rint(log_uniform(u[0], *tri_range)))
    return gen_soup(5, i + 1, nt, 1.0, 0.002 / soup_side(nt))


def config5_requests(count: int, rate: float, n_scenes: int, upload_frac: float = 0.1,
                     ray_range=(1_000, 2_000_000), seed_stream: int = 0):
    """Poisson arrivals: -> list of (t_arrival, kind, scene_or_upload_index, n_rays, ray_offset)."""
    u = gen_uniform(5, 4_000_000 + seed_stream, 5 * count)
    t = 0.0
    out = []
    up = 0
    for k in range(count):
        t += -np.log(1.0 - u[5 * k]) / rate
        if u[5 * k + 1] < upload_frac:
            out.append((t, "upload", up, 0, 0))
            up += 1
        else:
            n = int(np.rint(log_uniform(u[5 * k + 2], *ray_range)))
            sid = min(int(u[5 * k + 3] * n_scenes), n_scenes - 1)
            off = int(u[5 * k + 4] * (ray_range[1] - n + 1))
            out.append((t, "rays", sid, n, off))
    return out
