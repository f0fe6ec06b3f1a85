"""GPU tests of the scene pool (rt_pool_*): one launch over many scenes must
return exactly what rt_trace returns on each scene alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def soups(rt, seed, count, lo=1_000, hi=60_000):
    u = rt.gen_uniform(seed, 99, 2 * count)
    out = []
    for i in range(count):
        nt = int(round(np.exp(np.log(lo) + (np.log(hi) - np.log(lo)) * u[2 * i])))
        nr = int(round(np.exp(np.log(2_000) + (np.log(80_000) - np.log(2_000)) * u[2 * i + 1])))
        side = (nt / 4_194_304) ** (1 / 3)
        out.append((rt.gen_soup(seed, i + 1, nt, side, 0.002), rt.gen_rays(seed, i + 1, nr, side, 1e-4, float("inf"))))
    return out


def alone(rt, torch, tris, rays, any_hit=False):
    with rt.Scene(tris) as sc:
        d_rays = torch.from_numpy(rays.view(np.uint8)).cuda()
        d_hits = torch.empty(len(rays) * 8, dtype=torch.uint8, device="cuda")
        sc.trace(d_rays, d_hits, any_hit=any_hit)
        torch.cuda.synchronize()
        return d_hits.cpu().numpy().view(rt.HIT_DTYPE)


def run_pool(rt, torch, pool, ids, data, any_hit=False, autotune=False):
    dr = [torch.from_numpy(r.view(np.uint8)).cuda() for _, r in data]
    dh = [torch.full((len(r) * 8,), 0xEE, dtype=torch.uint8, device="cuda") for _, r in data]
    jobs = [(sid, a, b) for sid, a, b in zip(ids, dr, dh)]
    if autotune:
        pool.autotune(jobs, any_hit=any_hit, repeats=1)
    pool.trace(jobs, any_hit=any_hit)
    torch.cuda.synchronize()
    return [h.cpu().numpy().view(rt.HIT_DTYPE) for h in dh]


def test_pool_matches_individual_scenes(rt, cuda):
    data = soups(rt, 41, 24)
    with rt.Pool() as pool:
        ids = [pool.add_scene(t) for t, _ in data]
        assert pool.info().num_scenes == 24
        for anyh in (False, True):
            got = run_pool(rt, cuda, pool, ids, data, any_hit=anyh)
            for (t, r), g in zip(data, got):
                assert np.array_equal(g.view(np.uint64), alone(rt, cuda, t, r, any_hit=anyh).view(np.uint64))
        # a second launch on the same stream (other launch slot) and an autotuned one
        got = run_pool(rt, cuda, pool, ids[::-1], data[::-1], autotune=True)
        for (t, r), g in zip(data[::-1], got):
            assert np.array_equal(g.view(np.uint64), alone(rt, cuda, t, r).view(np.uint64))


def test_pool_runs_of_empty_jobs(rt, cuda):
    """Jobs with no rays between and around real ones: a refill's new rays
    walk from the first ray's job over empty jobs, and past 8 of them search
    the job table instead.  Every real job gets exactly its own hits."""
    data = soups(rt, 44, 4, lo=5_000, hi=20_000)
    with rt.Pool() as pool:
        ids = [pool.add_scene(t) for t, _ in data]
        zero = cuda.empty(8, dtype=cuda.uint8, device="cuda")
        dr = [cuda.from_numpy(r.view(np.uint8)).cuda() for _, r in data]
        dh = [cuda.full((len(r) * 8,), 0xEE, dtype=cuda.uint8, device="cuda") for _, r in data]
        jobs = []
        for k, (sid, a, b) in enumerate(zip(ids, dr, dh)):
            jobs += [(sid, zero, zero, 0)] * (3 + 9 * k)  # 3, 12, 21, 30 empty jobs before each
            jobs.append((sid, a, b))
        jobs += [(ids[0], zero, zero, 0)] * 5
        for variant in (5, 6):  # with and without the shared-memory ring
            for h in dh:
                h.fill_(0xEE)
            pool.set_tuning(variant, 4)
            pool.trace(jobs)
            cuda.cuda.synchronize()
            for (t, r), h in zip(data, dh):
                got = h.cpu().numpy().view(rt.HIT_DTYPE)
                assert np.array_equal(got.view(np.uint64), alone(rt, cuda, t, r).view(np.uint64)), variant


def test_pool_remove_reuse_and_growth(rt, cuda):
    data = soups(rt, 42, 40, lo=20_000, hi=120_000)
    with rt.Pool() as pool:
        ids = [pool.add_scene(t) for t, _ in data[:10]]
        arena0 = pool.info().arena_bytes
        for k in (1, 4, 7):
            pool.remove_scene(ids[k])
        with pytest.raises(rt.RtError) as e:
            pool.remove_scene(ids[4])
        assert e.value.status == 8  # RT_ENOTFOUND
        more = [pool.add_scene(t) for t, _ in data[10:]]  # fills the holes, then grows the arena
        assert pool.info().arena_bytes > arena0
        keep = [i for i in range(10) if i not in (1, 4, 7)]
        sel_ids = [ids[i] for i in keep] + more
        sel = [data[i] for i in keep] + data[10:]
        got = run_pool(rt, cuda, pool, sel_ids, sel)
        for (t, r), g in zip(sel, got):
            assert np.array_equal(g.view(np.uint64), alone(rt, cuda, t, r).view(np.uint64))


def test_pool_budget_and_empty_jobs(rt, cuda):
    data = soups(rt, 43, 3, lo=50_000, hi=50_001)
    with rt.Pool(budget_bytes=9_000_000) as pool:
        a = pool.add_scene(data[0][0])
        with pytest.raises(rt.RtError) as e:
            pool.add_scene(data[1][0])
            pool.add_scene(data[2][0])
        assert e.value.status == 2  # RT_ENOMEM
        used = pool.info().used_bytes
        assert used <= 9_000_000
        pool.remove_scene(a)
        b = pool.add_scene(data[1][0])
        t, r = data[1]
        zero = cuda.empty(8, dtype=cuda.uint8, device="cuda")
        d_rays = cuda.from_numpy(r.view(np.uint8)).cuda()
        d_hits = cuda.empty(len(r) * 8, dtype=cuda.uint8, device="cuda")
        pool.trace([(b, zero, zero, 0), (b, d_rays, d_hits), (b, zero, zero, 0)])
        cuda.cuda.synchronize()
        assert np.array_equal(d_hits.cpu().numpy().view(np.uint64), alone(rt, cuda, t, r).view(np.uint64))
        pool.trace([])
        with pytest.raises(rt.RtError):
            pool.trace([(999, d_rays, d_hits)])
        # a job whose rays are off a 16-byte boundary, or hits off an 8-byte
        # one, is refused before anything is launched
        n = len(r) - 1
        for rays_view, hits_view in ((d_rays[4:4 + n * 32], d_hits), (d_rays, d_hits[4:4 + n * 8])):
            with pytest.raises(rt.RtError) as e:
                pool.trace([(b, rays_view, hits_view, n)])
            assert e.value.status == 1 and "aligned" in str(e.value)


def test_pool_every_tuning_same_hits(rt, cuda):
    """Every stack capacity and top-of-tree tile the pool tuner searches (on
    the two 128 x 10 four-visit launch shapes) returns exactly the hits of each scene
    traced alone; the tuner reports what it chose; settings the pool cannot
    run are refused.  Also with more jobs than a block can stage (no tile)."""
    data = soups(rt, 43, 40, hi=30_000)
    ref = [alone(rt, cuda, t, r) for t, r in data]
    with rt.Pool() as pool:
        ids = [pool.add_scene(t) for t, _ in data]
        need = pool.info().stack_need
        for variant in (5, 6):
            for stack in (48, 64, 96, 192):
                for tile in (0, 1, 2):
                    if stack < need:
                        with pytest.raises(rt.RtError):
                            pool.set_tuning(variant, 4, stack, tile)
                        continue
                    pool.set_tuning(variant, 4, stack, tile)
                    info = pool.info()
                    assert (info.tuned_variant, info.tuned_stack, info.tuned_tile) == (variant, stack, tile)
                    got = run_pool(rt, cuda, pool, ids, data)
                    for g, want in zip(got, ref):
                        assert np.array_equal(g.view(np.uint64), want.view(np.uint64)), (variant, stack, tile)
        with pytest.raises(rt.RtError):
            pool.set_tuning(1, 4, 64, 1)  # tiles only on the 128 x 10 shapes
        run_pool(rt, cuda, pool, ids, data, autotune=True)
        info = pool.info()
        assert info.tuned_stack >= need and info.tuned_tile in (0, 1, 2)
        # 300 jobs (above the 256 a block stages): the tile is skipped, hits unchanged
        if info.tuned_variant in (5, 6):
            pool.set_tuning(info.tuned_variant, 4, 64 if need <= 64 else 192, 2)
        many = [(ids[i % len(ids)], data[i % len(data)]) for i in range(300)]
        got = run_pool(rt, cuda, pool, [m[0] for m in many], [m[1] for m in many])
        for k, g in enumerate(got):
            assert np.array_equal(g.view(np.uint64), ref[k % len(ref)].view(np.uint64))
