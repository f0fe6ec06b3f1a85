"""GPU tests of the serving loop (rt_server_*): continuous batching must not
change any query's result; admission, eviction, cancellation and deadlines
are exercised on the host (no GPU fault is involved)."""
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def scene_data(rt, seed, k, nt, nr):
    side = (nt / 4_194_304) ** (1 / 3)
    return rt.gen_soup(seed, k + 1, nt, side, 0.002), rt.gen_rays(seed, k + 1, nr, side, 1e-4, float("inf"))


def alone(rt, torch, tris, rays):
    with rt.Scene(tris) as sc:
        d_rays = torch.from_numpy(rays.view(np.uint8)).cuda()
        d_hits = torch.empty(len(rays) * 8, dtype=torch.uint8, device="cuda")
        sc.trace(d_rays, d_hits)
        torch.cuda.synchronize()
        return d_hits.cpu().numpy().view(rt.HIT_DTYPE)


def pinned(torch, a):
    t = torch.from_numpy(np.ascontiguousarray(a).view(np.uint8)).pin_memory()
    return t, t.numpy().view(a.dtype)


def test_results_same_alone_and_in_the_mix(rt, cuda):
    scenes = [scene_data(rt, 51, k, nt, 1)[0] for k, nt in enumerate([30_000, 120_000, 5_000, 400_000, 60_000, 9_000])]
    u = rt.gen_uniform(51, 7, 120)
    reqs = []
    for i in range(60):
        sid = int(u[2 * i] * len(scenes))
        nr = int(np.exp(np.log(1_000) + (np.log(300_000) - np.log(1_000)) * u[2 * i + 1]))
        side = (len(scenes[sid]) / 4_194_304) ** (1 / 3)
        reqs.append((sid, rt.gen_rays(51, 100 + i, nr, side, 1e-4, float("inf"))))
    bufs = []
    for sid, r in reqs:  # pin everything first, so the submissions come in a burst
        tr, hr = pinned(cuda, r)
        th, hh = pinned(cuda, np.zeros(len(r), rt.HIT_DTYPE))
        bufs.append((tr, hr, th, hh))
    with rt.Server(max_batch_rays=1 << 20, max_inflight=2) as srv:
        ids = [srv.wait(srv.upload(t)).scene_id for t in scenes]
        out = [None] * len(reqs)

        def submitter(lo, hi):
            for i in range(lo, hi):
                sid, _ = reqs[i]
                out[i] = (srv.submit(ids[sid], bufs[i][1], bufs[i][3]), bufs[i][3])

        ts = [threading.Thread(target=submitter, args=(0, 30)), threading.Thread(target=submitter, args=(30, 60))]
        [t.start() for t in ts]
        [t.join() for t in ts]
        results = [srv.wait(rid, 120.0) for rid, _ in out]
        st = srv.stats()
    assert all(r.status == 0 for r in results)
    assert st.requests_done == 60 and st.batches < 60  # queries shared launches
    assert max(r.batch_jobs for r in results) > 1
    for (sid, r), (_, hh) in zip(reqs, out):
        assert np.array_equal(hh.view(np.uint64), alone(rt, cuda, scenes[sid], r).view(np.uint64))


def test_eviction_under_budget(rt, cuda):
    scenes = [scene_data(rt, 52, k, 100_000, 1)[0] for k in range(3)]
    side = (100_000 / 4_194_304) ** (1 / 3)
    rays = rt.gen_rays(52, 9, 200_000, side, 1e-4, float("inf"))
    with rt.Server(budget_bytes=25_000_000) as srv:
        a = srv.wait(srv.upload(scenes[0])).scene_id
        b = srv.wait(srv.upload(scenes[1])).scene_id
        hits = np.zeros(len(rays), rt.HIT_DTYPE)
        rid = srv.submit(b, rays, hits)  # keeps b busy (or recently used)
        c = srv.wait(srv.upload(scenes[2])).scene_id  # needs room: the idle, older scene a goes
        assert c not in (a, b)  # server scene ids are never reused
        assert srv.stats().evictions >= 1
        assert srv.wait(rid).status == 0
        assert np.array_equal(hits.view(np.uint64), alone(rt, cuda, scenes[1], rays).view(np.uint64))
        with pytest.raises(rt.RtError) as e:
            srv.submit(a, rays)
        assert e.value.status == 8  # evicted: RT_ENOTFOUND
        too_big = scene_data(rt, 52, 9, 600_000, 1)[0]
        with pytest.raises(rt.RtError) as e:
            srv.wait(srv.upload(too_big))
        assert e.value.status == 2  # RT_ENOMEM even with every idle scene evicted


def test_cancel_deadline_and_errors(rt, cuda):
    tris, _ = scene_data(rt, 53, 0, 50_000, 1)
    side = (50_000 / 4_194_304) ** (1 / 3)
    big = rt.gen_rays(53, 1, 3_000_000, side, 1e-4, float("inf"))
    with rt.Server(max_inflight=1, max_batch_rays=1 << 16) as srv:
        sid = srv.wait(srv.upload(tris)).scene_id
        ids = [srv.submit(sid, big) for _ in range(4)]
        # one batch at a time, one query per batch: the last is still queued
        srv.cancel(ids[3])
        with pytest.raises(rt.RtError) as e:
            srv.wait(ids[2], timeout=0.0)
        assert e.value.status == 3  # RT_ETIMEOUT; the request stays queryable
        for rid in ids[:3]:
            assert srv.wait(rid, 120.0).status == 0
        with pytest.raises(rt.RtError) as e:
            srv.wait(ids[3])
        assert e.value.status == 7  # RT_ECANCELED
        with pytest.raises(rt.RtError) as e:
            srv.cancel(ids[0])  # already waited for and forgotten
        assert e.value.status == 8
        with pytest.raises(rt.RtError) as e:
            srv.submit(12345, big[:10])
        assert e.value.status == 8
        with pytest.raises(rt.RtError) as e:
            srv.wait(987654321)
        assert e.value.status == 8
