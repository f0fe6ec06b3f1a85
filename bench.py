#!/usr/bin/env python3
"""Benchmark of the ray-query hot path on one GB300.

Workload (a "step"): config 3 -- closest-hit traversal of 16,777,216
incoherent rays (origins uniform in the unit cube, directions uniform on the
sphere, tmin 1e-4, tmax inf) through a 4,194,304-triangle soup (centroids
uniform in the cube, vertex offsets N(0, 0.002^2)), BVH built on the host in
the reference node layout (sorted leaves).  Synthetic, seeded inputs.

value  : rays/s with rays and hits resident in HBM (one rt_trace per step)
e2e    : the same through rt_trace_host with pinned host buffers, so every
         step includes the 512 MiB ray upload and 128 MiB hit download
roofline: algorithmic bytes per ray (32 ray + 8 hit + 32 per node box tested
         + 48 per triangle tested, counts of the canonical traversal) times
         rays per launch over the kernel's event-timed launch duration,
         against the measured HBM copy bandwidth
cpu_baseline: the reference's traversal (raytraceBVH.comp:195-265,
         push-left/go-right, no culling) on the host cores -- its own GLSL
         compiled as C++ (oracle/ref_glsl.py) where available, else the
         oracle's restatement -- on a bounded sample of the same rays, all
         host threads

--impl reference runs that CPU traversal alone as the reference arm.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "closest-hit Grays/s batched vs plain per-call launch; served p50/p99 latency"
UNIT = "Grays/s"
L2_BYTES = 129 * 10**6
N_TRIS = 4_194_304
N_RAYS = 16_777_216
SEED = 3
CPU_SAMPLE = 2_097_152
# DRAM bytes per ray of k_trace_step on the full config-3 BVH: one ncu capture
# of a 2,097,152-ray launch, dram__bytes_read.sum + dram__bytes_write.sum.
DRAM_BYTES_PER_RAY = (1.306393e9 + 58.430976e6) / 2_097_152  # ncu, 2 Mi-ray launch on the config-3 tree
# The same capture: L2 -> L1 bytes per ray (missed global-load sectors x 32 B)
# and the FP32 (FMA) and ALU pipe activity of the kernel.
L2_TO_L1_BYTES_PER_RAY = 188_542_810 * 32 / 2_097_152
FMA_PIPE_PCT, ALU_PIPE_PCT = 31.5, 67.1
NOMINAL_HBM_GBS = 8000.0  # GB300 HBM3e, nominal


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=40)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--tris", type=int, default=N_TRIS)
    p.add_argument("--rays", type=int, default=N_RAYS)
    p.add_argument("--leaf-size", type=int, default=0)
    p.add_argument("--node-width", type=int, default=0, help="device BVH width (2 or 4; 0 = library default)")
    p.add_argument("--cpu-sample", type=int, default=CPU_SAMPLE)
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-sort", action="store_true", help="trace in the given ray order (no RT_TRACE_SORT)")
    p.add_argument("--no-tune", action="store_true", help="skip rt_trace_autotune (default launch)")
    p.add_argument("--no-batched", action="store_true", help="skip the config-4 batched comparison")
    p.add_argument("--no-served", action="store_true", help="skip the config-5 serving run")
    p.add_argument("--no-render", action="store_true", help="skip the config-2 path-tracing run")
    p.add_argument("--render-spp", type=int, default=16, help="samples per pixel of the config-2 frame")
    p.add_argument("--serve-requests", type=int, default=200)
    p.add_argument("--serve-inflight", type=int, default=3, help="batches in flight at once (continuous batching)")
    p.add_argument("--serve-rates", type=str, default="250,500,1000,2000,4000,8000,16000",
                   help="Poisson arrival rates (requests/s), swept in order")
    return p.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def l2_note(n_rays: int, info) -> str:
    """Whether the timed inputs exceed the 129 MB L2 (no flush between steps then)."""
    ray_b = n_rays * 32
    scene_b = info.device_nodes * 64 + info.num_triangles * 64
    big = ray_b + n_rays * 8 > L2_BYTES and scene_b > L2_BYTES
    return (f"rays {ray_b / 2**20:.0f} MiB + hits {n_rays * 8 / 2**20:.0f} MiB, nodes+triangles "
            f"{scene_b / 2**20:.0f} MiB; " + ("both larger than L2, no flush" if big else
                                               "not both larger than L2 (a parity/shape run, not a bench value)"))


def reduce_max(x: float, dist=None, device="cpu") -> float:
    """The largest x over all ranks: the slowest replica sets the job time."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job(total_ms: float, steps: int, units_per_rank: int, world: int):
    """-> (ms per step, units per second of all ranks).  Every rank processes
    its own full batch (replicas), so the job's work grows with the world size."""
    ms_step = total_ms / steps
    return ms_step, units_per_rank * world / (ms_step / 1e3)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 8:
                self.rows.append((time.time(), parts))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, t0: float, t1: float) -> dict:
        rows = [r for (t, r) in self.rows if t0 <= t <= t1] or [r for (_, r) in self.rows]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[0]) for r in rows if num(r[0]) is not None]
        mx = [num(r[1]) for r in rows if num(r[1]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[4 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max((num(r[2]) or 0.0) for r in rows)}


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return 6800.0, "fallback"


def workload(n_tris: int, n_rays: int):
    import raytracergpu_mastersproject_gb300 as rt

    tris = rt.gen_soup(SEED, 0, n_tris, 1.0, 0.002)
    rays = rt.gen_rays(SEED, 0, n_rays, 1.0, 1e-4, float("inf"))
    return tris, rays


def cpu_leg(tris, nodes, rays, sample: int, trav_nodes=None) -> tuple[dict, dict]:
    """CPU baseline: the oracle's reference-order traversal of the S1 tree
    (`nodes`, the reference's own) with every host thread, the median of 5
    timed runs on a quarter of `sample` rays, plus one run over all `sample`
    rays whose hits check the GPU's; single-thread rates on small samples;
    canonical traversal counts (work per ray) on the tree the kernel traverses
    (`trav_nodes`, default the S1 tree)."""
    from oracle import oracle as orc

    trace, kind, what = reference_tracer()
    S = orc.Scene(tris, nodes)
    cores = os.cpu_count() or 1
    sub = np.ascontiguousarray(rays[:sample])

    def rate(scene, r, canonical, threads):
        t0 = time.perf_counter()
        if canonical:
            orc.trace(scene, r, canonical=True, nthreads=threads)
        else:
            trace(scene, r, threads)
        return len(r) / (time.perf_counter() - t0) / 1e9

    quarter = np.ascontiguousarray(rays[:max(1, sample // 4)])
    runs = [rate(S, quarter, False, cores) for _ in range(5)]
    t0 = time.perf_counter()
    ref_hits = trace(S, sub, cores)
    dt = time.perf_counter() - t0
    cnt = sub
    St = S if trav_nodes is None else orc.Scene(tris, trav_nodes)
    t1 = time.perf_counter()
    can_hits, cst = orc.trace(St, cnt, canonical=True, nthreads=cores)
    dt_can = time.perf_counter() - t1
    one_ref = np.ascontiguousarray(rays[:max(1, sample // 32)])
    one_can = np.ascontiguousarray(rays[:max(1, sample // 16)])
    single = {"reference_order": rate(S, one_ref, False, 1), "reference_order_rays": len(one_ref),
              "canonical": rate(St, one_can, True, 1), "canonical_rays": len(one_can), "unit": UNIT}
    counts = {"node_boxes_per_ray": float(cst[0]) / len(cnt), "tri_tests_per_ray": float(cst[1]) / len(cnt),
              "sample": len(cnt)}
    base = {"value": float(np.median(runs)), "unit": UNIT, "cores": cores, "kind": kind,
            "sample": f"median of 5 runs over the first {len(quarter)} rays of the config-3 batch, {what} "
                      f"(reference order, no culling, sorted-leaf S1 tree), {cores} threads",
            "runs": runs,
            "full_sample": {"rays": len(sub), "value": len(sub) / dt / 1e9, "seconds": dt},
            "single_thread": single,
            "canonical": {"value": len(cnt) / dt_can / 1e9, "unit": UNIT, "cores": cores,
                          "sample": f"first {len(cnt)} rays, the same restatement with near-child-first "
                                    f"order and interval culling (the kernels' order; same hits) over "
                                    f"{'the binned-SAH tree the kernel traverses' if trav_nodes is not None else 'the S1 tree'}"
                                    f", {dt_can:.2f} s"}}
    return base, {"counts": counts, "ref_hits": ref_hits, "can_hits": can_hits}


def _time_events(torch, fn, warmup: int = 2, reps: int = 5) -> float:
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def run_batched(torch, rt) -> dict:
    """Config 4: 256 soups with their own ray batches -- 256 plain rt_trace
    calls vs one autotuned pool launch replayed from a CUDA graph."""
    from raytracergpu_mastersproject_gb300 import workloads as wl

    data = wl.config4()
    nt = int(sum(len(t) for t, _ in data))
    nr = int(sum(len(r) for _, r in data))
    scenes = [rt.Scene(t) for t, _ in data]
    pool = rt.Pool(budget_bytes=32 << 30)
    ids = [pool.add_scene(t) for t, _ in data]
    dr = [torch.from_numpy(r.view(np.uint8)).cuda() for _, r in data]
    dh_plain = [torch.empty(len(r) * 8, dtype=torch.uint8, device="cuda") for _, r in data]
    dh_batch = [torch.empty(len(r) * 8, dtype=torch.uint8, device="cuda") for _, r in data]
    jobs = list(zip(ids, dr, dh_batch))

    def plain():
        for sc, a, b in zip(scenes, dr, dh_plain):
            sc.trace(a, b)

    def batched():
        pool.trace(jobs)

    ms_plain = _time_events(torch, plain)
    ms_untuned = _time_events(torch, batched)
    variant, refill = pool.autotune(jobs, repeats=2)
    ms_batch = _time_events(torch, batched)
    plain()
    batched()
    torch.cuda.synchronize()
    same = all(torch.equal(a, b) for a, b in zip(dh_plain, dh_batch))
    thr, minb, ring = rt.describe_pool_variant(variant)
    pinfo = pool.info()
    out = {"workload": "config 4: 256 triangle soups, counts log-uniform in [1K, 256K], each with a ray batch "
                       "log-uniform in [4K, 1M] rays, closest-hit",
           "triangles": nt, "rays": nr, "unit": UNIT,
           "plain": {"value": nr / ms_plain / 1e6, "ms": ms_plain, "launches": 256,
                     "path": "one rt_trace per scene"},
           "batched": {"value": nr / ms_batch / 1e6, "ms": ms_batch, "launches": 1, "cuda_graph": True,
                       "untuned_ms": ms_untuned,
                       "autotuned": {"threads_per_block": thr, "min_blocks_per_sm": minb,
                                     "stack_entries_in_shared_memory": ring, "refill": refill,
                                     "stack_entries": int(pinfo.tuned_stack),
                                     "tile_nodes_per_scene": int(pinfo.tuned_tile)}},
           "speedup": ms_plain / ms_batch, "identical_hits": bool(same)}
    pool.close()
    for sc in scenes:
        sc.close()
    return out


def run_extras(torch, rt, scene, tris, d_rays, n: int) -> dict:
    """Config 3 any-hit and Moller-Trumbore closest-hit, the BVH build on host
    vs device, config 1 closest-hit."""
    d_hits = torch.empty(n * 8, dtype=torch.uint8, device="cuda")
    ms_any = _time_events(torch, lambda: scene.trace(d_rays, d_hits, any_hit=True, sort=True), warmup=2, reps=10)
    ms_mt = _time_events(torch, lambda: scene.trace(d_rays, d_hits, sort=True, mt=True), warmup=2, reps=10)
    t0 = time.perf_counter()
    rt.build_bvh(tris)
    host_s = time.perf_counter() - t0
    d_t = torch.from_numpy(tris.view(np.uint8)).cuda()
    d_n = torch.empty((2 * len(tris) - 1) * 40, dtype=torch.uint8, device="cuda")
    ms_dev = _time_events(torch, lambda: rt.build_bvh_device(d_t, len(tris), None, 0, d_n), warmup=1, reps=5)
    c1_tris, _, c1_rays = rt.gen_config1()
    out = {"config3_any_hit": {"value": n / ms_any / 1e6, "unit": UNIT, "ms": ms_any},
           "config3_closest_hit_moller_trumbore": {
               "value": n / ms_mt / 1e6, "unit": UNIT, "ms": ms_mt,
               "note": "RT_TRACE_MT: not the reference's plane test; ids differ on edge hits (about 1 ray in 12,000)"},
           "bvh_build_config3": {"host_s": host_s, "host_threads": os.cpu_count(), "device_ms": ms_dev,
                                 "note": "2N-1 reference-layout nodes, identical bytes from both builders"}}
    with rt.Scene(c1_tris, bvh_mode=rt.BVH_REFERENCE) as s1:
        r1 = torch.from_numpy(c1_rays.view(np.uint8)).cuda()
        h1 = torch.empty(len(c1_rays) * 8, dtype=torch.uint8, device="cuda")
        ms1 = _time_events(torch, lambda: s1.trace(r1, h1), warmup=2, reps=20)
    out["config1_closest_hit"] = {"value": len(c1_rays) / ms1 / 1e6, "unit": UNIT, "ms": ms1,
                                  "bvh": "reference leaf order (ConstructHLBVH.comp:152-169)"}
    return out


def run_render(torch, rt, spp: int = 16) -> dict:
    """Config 2: 64 displaced icospheres (subdiv 6), 1280x720, 16 samples,
    depth 8, one rt_render call (all samples), extended shading (metal,
    dielectric, sky colour) and reference shading."""
    tris, mats = rt.gen_spheres_scene(2, 64, 6, 0.05)
    w, h = 1280, 720
    ubo = rt.make_ubo((0.0, 3.0, 28.0), (0.0, 0.0, 0.0), fov=40.0, depth=8, random_state=2,
                      num_triangles=len(tris), num_materials=len(mats))
    out = {"workload": "config 2: 64 icospheres subdiv 6 (5,242,880 triangles), radial value-noise displacement "
                       f"0.05, lambertian/metal/dielectric, 1280x720, {spp} spp, depth 8",
           "triangles": int(len(tris)), "paths": w * h * spp, "unit": "Mpaths/s"}
    with rt.Scene(tris, materials=mats) as sc:
        acc = torch.empty(w * h * 4, dtype=torch.float32, device="cuda")
        for mode, name in ((rt.SHADE_EXTENDED, "extended"), (rt.SHADE_REFERENCE, "reference")):
            for every in (False, True):
                def frame():
                    rt.accum_clear(acc, w, h)
                    sc.render(ubo, acc, w, h, spp, shade_mode=mode, background=(0.6, 0.7, 1.0),
                              trace_every_primary=every)
                ms = _time_events(torch, frame, warmup=1, reps=3)
                img = acc.cpu().numpy().reshape(h, w, 4)
                rt.accum_clear(acc, w, h)
                q, nodes, prims = sc.render_count(ubo, acc, w, h, spp, shade_mode=mode, background=(0.6, 0.7, 1.0),
                                                  trace_every_primary=every)
                r = {"value": w * h * spp / ms / 1e3, "ms_per_frame": ms,
                     "mean_rgb": [float(img[..., k].mean() / spp) for k in range(3)],
                     "queries_per_path": q / (w * h * spp), "Gqueries_per_s": q / ms / 1e6,
                     "nodes_per_query": nodes / max(q, 1), "prims_per_query": prims / max(q, 1)}
                if every:
                    r["note"] = "every sample traces its primary ray, as the reference's spp dispatches do"
                    out[name]["every_sample_traces_primary"] = r
                else:
                    r["note"] = ("default: a pixel's first hit is found once and shared by its samples (no camera "
                                 "jitter, so every sample starts with the same ray); the image is the same bit for bit")
                    out[name] = r
    return out


def sustained(m: dict) -> bool:
    """A rate is sustained when the queue does not build up over the run: the
    later third of the queries wait at most twice as long (plus 2 ms) as the
    first third, and queries complete at least at 80 % of the offered rate."""
    return bool(m["late_over_early_p50"] <= 2.0 + 2.0 / max(m["p50_ms"], 1e-3)
                and m["completed_queries_per_s"] >= 0.8 * m["offered_queries_per_s"])


def serving_summary(runs: list[dict]) -> dict:
    """Per mode the highest swept rate it sustains (with every lower rate), and
    the latencies of both modes at the highest rate both sustain."""
    out = {}
    for mode in ("batched", "sequential"):
        best = None
        for r in runs:
            if not r[mode]["sustained"]:
                break
            best = r["rate_per_s"]
        out[f"{mode}_max_sustained_req_per_s"] = best
    both = [r for r in runs if r["batched"]["sustained"] and r["sequential"]["sustained"]]
    if both:
        r = both[-1]
        out["at_rate_both_sustain"] = {"rate_per_s": r["rate_per_s"],
                                       "batched_p50_p99_ms": [round(r["batched"]["p50_ms"], 3), round(r["batched"]["p99_ms"], 3)],
                                       "sequential_p50_p99_ms": [round(r["sequential"]["p50_ms"], 3),
                                                                 round(r["sequential"]["p99_ms"], 3)]}
    out["p99_ms_by_rate"] = {str(int(r["rate_per_s"])): [round(r["batched"]["p99_ms"], 2), round(r["sequential"]["p99_ms"], 2)]
                             for r in runs}
    out["Grays_by_rate"] = {str(int(r["rate_per_s"])): [round(r["batched"]["Grays_per_s"], 3),
                                                        round(r["sequential"]["Grays_per_s"], 3)] for r in runs}
    return out


def run_served(torch, rt, n_requests: int, rates: list[float], inflight: int = 3) -> dict:
    """Config 5: 64 resident scenes, Poisson arrivals; 90% ray queries
    (log-uniform [1K, 2M] rays, closest-hit), 10% new-scene uploads; latency
    p50/p99 and rays/s with continuous batching vs plain sequential service."""
    from raytracergpu_mastersproject_gb300 import workloads as wl

    n_scenes = 64
    t0 = time.perf_counter()
    resident = [wl.config5_scene(i) for i in range(n_scenes)]
    ray_pool_t = torch.from_numpy(rt.gen_rays(5, 0, 2_000_000, 1.0, 1e-4, float("inf")).view(np.uint8)).pin_memory()
    ray_pool = ray_pool_t.numpy().view(rt.RAY_DTYPE)
    srv = rt.Server(budget_bytes=150 << 30, max_inflight=inflight, max_batch_rays=1 << 23)
    sids = [srv.wait(srv.upload(t, build_on_device=True), 600.0).scene_id for t in resident]
    setup_s = time.perf_counter() - t0
    res_tris = int(sum(len(t) for t in resident))
    runs = []
    for ri, rate in enumerate(rates):
        reqs = wl.config5_requests(n_requests, rate, n_scenes, seed_stream=ri)
        uploads = [wl.config5_scene(1000 + 100 * ri + k) for k in range(sum(1 for r in reqs if r[1] == "upload"))]
        tot_rays = sum(r[3] for r in reqs)
        hits_t = torch.empty(max(tot_rays, 1) * 8, dtype=torch.uint8).pin_memory()
        hits = hits_t.numpy().view(rt.HIT_DTYPE)
        entry = {"rate_per_s": rate, "requests": n_requests, "ray_requests": sum(1 for r in reqs if r[1] == "rays"),
                 "uploads": len(uploads), "rays": tot_rays}
        for mode in ("batched", "sequential"):
            if mode == "batched":
                srv.set_batching(1024, inflight)
            else:
                srv.set_batching(1, 1)
            ids, kinds, new_scenes = [], [], []
            hoff = 0
            start = time.perf_counter()
            for (t_arr, kind, idx, n, off) in reqs:
                delay = start + t_arr - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                if kind == "upload":
                    ids.append(srv.upload(uploads[idx], build_on_device=True))
                else:
                    ids.append(srv.submit(sids[idx], ray_pool[off:off + n], hits[hoff:hoff + n]))
                    hoff += n
                kinds.append(kind)
            lat, up_lat, batch_jobs = [], [], []
            first_arr, last_done = None, 0.0
            for rid, kind, rq in zip(ids, kinds, reqs):
                r = srv.wait(rid, 600.0)
                if kind == "rays":
                    lat.append(r.latency_seconds)
                    batch_jobs.append(r.batch_jobs)
                    first_arr = rq[0] if first_arr is None else min(first_arr, rq[0])
                    last_done = max(last_done, rq[0] + r.latency_seconds)
                else:
                    up_lat.append(r.latency_seconds)
                    new_scenes.append(r.scene_id)
            wall = max(last_done - (first_arr or 0.0), 1e-9)  # span of the ray queries
            for sid in new_scenes:
                srv.remove_scene(sid)
            lat_ms = np.array(lat) * 1e3
            arr = np.array([rq[0] for rq in reqs if rq[1] == "rays"])
            third = max(1, len(lat_ms) // 3)
            entry[mode] = {"p50_ms": float(np.percentile(lat_ms, 50)), "p99_ms": float(np.percentile(lat_ms, 99)),
                           "mean_ms": float(lat_ms.mean()), "rays_per_s": tot_rays / wall,
                           "Grays_per_s": tot_rays / wall / 1e9, "query_span_s": wall,
                           "offered_queries_per_s": len(arr) / max(float(arr[-1] - arr[0]), 1e-9),
                           "completed_queries_per_s": len(arr) / wall,
                           "late_over_early_p50": float(np.median(lat_ms[-third:]) / max(np.median(lat_ms[:third]), 1e-6)),
                           "mean_queries_per_launch": float(np.mean(batch_jobs)),
                           "upload_p50_s": float(np.median(up_lat)) if up_lat else None}
            entry[mode]["sustained"] = sustained(entry[mode])
        runs.append(entry)
    st = srv.stats()
    srv.close()
    return {"workload": "config 5: 64 resident soups (counts log-uniform in [64K, 4M]), Poisson arrivals, "
                        "90% closest-hit queries of log-uniform [1K, 2M] rays from pinned host memory, "
                        "10% new-scene uploads (BVH built on the GPU); HBM budget 150 GB",
            "resident_triangles": res_tris, "setup_s": setup_s, "runs": runs,
            "summary": serving_summary(runs),
            "batches_total": int(st.batches), "evictions": int(st.evictions),
            "latency": "submit of the host request to its hits back in host memory",
            "sequential": "same server, one query per launch, one launch at a time"}


def reference_tracer():
    """-> (trace(scene, rays, nthreads) -> hits, kind, description) of the
    reference's traversal on the host: its own hitBVH (raytraceBVH.comp:195-265)
    compiled from the shader source when oracle/_ref has it, else the oracle's
    line-by-line restatement."""
    from oracle import oracle as orc

    orc.build()
    try:
        from oracle import ref

        if ref.available():
            return (lambda S, r, nth: ref.trace(S, r, nthreads=nth), "reference",
                    "the reference's own hitBVH (raytraceBVH.comp:195-265) compiled from its GLSL source as host "
                    "C++ (oracle/ref_glsl.py)")
    except (ImportError, OSError, RuntimeError):
        pass
    return (lambda S, r, nth: orc.trace(S, r, nthreads=nth)[0], "port",
            "oracle restatement of hitBVH (raytraceBVH.comp:195-265)")


def run_reference(args):
    """Reference arm: the reference's traversal on the host cores, timed on
    bounded samples.  Inputs come from the oracle's copy of the generators and
    the BVH from the oracle's transcription of the six S1 passes, so this arm
    loads nothing of the product library."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as orc

    trace, kind, what = reference_tracer()
    tris = orc.gen_soup(SEED, 0, args.tris, 1.0, 0.002)
    nodes = orc.build_bvh(tris, mode=0)[0]
    S = orc.Scene(tris, nodes)
    cores = os.cpu_count() or 1
    per = max(1024, min(args.cpu_sample, 65_536))
    total = per * (args.warmup + args.steps)
    rays = orc.gen_rays(SEED, 0, min(total, args.rays), 1.0, 1e-4, float("inf"))
    off = 0

    def step():
        nonlocal off
        if off + per > len(rays):
            off = 0
        trace(S, rays[off:off + per], cores)
        off += per

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t0
    v = per * args.steps / dt / 1e9
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": f"config 3: {args.tris}-triangle soup, incoherent rays, closest-hit; "
                                   f"each step traces a bounded sample of {per} rays on the host cores",
                       "triangles": args.tris, "rays_per_step": per},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": kind,
                             "sample": f"{per} consecutive rays of the config-3 batch per step, {what}, over the "
                                       f"sorted-leaf S1 tree, {cores} threads"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch

    import raytracergpu_mastersproject_gb300 as rt

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    tris, rays = workload(args.tris, args.rays)
    scene = rt.Scene(tris, leaf_size=args.leaf_size, node_width=args.node_width)
    info = scene.info()
    n = len(rays)
    d_rays = torch.from_numpy(rays.view(np.uint8)).cuda()
    d_hits = torch.empty(n * 8, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    def barrier():
        if dist is not None:
            dist.barrier()

    sort = not args.no_sort
    for _ in range(args.warmup):
        scene.trace(d_rays, d_hits, sort=sort)
    torch.cuda.synchronize()
    # rt_trace_autotune on this batch: launch shape, refill, stack capacity and
    # staged top-of-tree tile; the timed steps run with what it keeps
    tuned = None if args.no_tune else scene.autotune(d_rays, d_hits, sort=sort, repeats=2).as_dict()
    torch.cuda.synchronize()
    gpu_nodes, gpu_tests = scene.trace_count(d_rays, d_hits, sort=sort)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.5)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier()
    torch.cuda.synchronize()
    t_start = time.time()
    g0 = torch.cuda.Event(enable_timing=True)
    g1 = torch.cuda.Event(enable_timing=True)
    g0.record(stream)
    for s in range(args.steps):
        evs[s][0].record(stream)
        scene.trace(d_rays, d_hits, sort=sort, stream=stream)
        evs[s][1].record(stream)
    g1.record(stream)
    torch.cuda.synchronize()
    barrier()
    t_end = time.time()
    total_ms = reduce_max(g0.elapsed_time(g1), dist, "cuda")
    launch_ms = [a.elapsed_time(b) for a, b in evs]
    ms_step, rays_per_s = whole_job(total_ms, args.steps, n, ws)
    value = rays_per_s / 1e9

    e2e = None
    if not args.no_e2e:
        h_rays = torch.from_numpy(rays.view(np.uint8)).pin_memory()
        h_hits = torch.empty(n * 8, dtype=torch.uint8).pin_memory()
        hr = h_rays.numpy().view(rt.RAY_DTYPE)
        hh = h_hits.numpy().view(rt.HIT_DTYPE)
        # The first calls on fresh page-locked buffers run slower (up to 13
        # against 10.6 ms per call on config 3), so the warm-up calls come
        # first and the value is the median of three timed blocks.
        for _ in range(max(3, args.warmup)):
            scene.trace_host(hr, out=hh, sort=sort)
        k = max(3, min(args.steps, 10))
        blocks = []
        for _ in range(3):
            barrier()
            t0 = time.perf_counter()
            for _ in range(k):
                scene.trace_host(hr, out=hh, sort=sort)
            blocks.append(reduce_max(time.perf_counter() - t0, dist, "cuda") / k)
        barrier()
        per = statistics.median(blocks)
        e2e = {"value": n * ws / per / 1e9, "unit": UNIT, "h2d_bytes_per_step": n * 32,
               "d2h_bytes_per_step": n * 8, "steps": 3 * k, "ms_per_step": per * 1e3,
               "block_ms_per_step": [round(b * 1e3, 3) for b in blocks],
               "timing": f"wall clock around each of 3 blocks of {k} calls after {max(3, args.warmup)} warm-up "
                         "calls; the median block",
               "path": "rt_trace_host, pinned host buffers: rays in chunks of 2 Mi, 8 Mi, the rest but "
                       "512 Ki, and 512 Ki, each uploaded on a copy stream while the one before traces (two trace "
                       "streams); hits staged in HBM and downloaded per chunk on a third stream"}
        hits_dev = d_hits.cpu().numpy().view(rt.HIT_DTYPE)
        assert np.array_equal(hits_dev.view(np.uint64), hh.view(np.uint64)), "e2e hits differ from device hits"
    clocks.stop()
    clk = clocks.summary(t_start, t_end)

    if rank != 0:
        return
    extras = run_extras(torch, rt, scene, tris, d_rays, n) if (args.tris, args.rays) == (N_TRIS, N_RAYS) else None
    batched = None if args.no_batched else run_batched(torch, rt)
    render = None if args.no_render else run_render(torch, rt, args.render_spp)
    served = None if args.no_served else run_served(
        torch, rt, args.serve_requests, [float(x) for x in args.serve_rates.split(",") if x], args.serve_inflight)
    peak, peak_kind = measured_peak()
    cpu_base, counts, parity = None, None, None
    if not args.no_cpu:
        nodes = scene.nodes()
        trav = rt.build_bvh_sah(tris) if info.traversal_sah else None
        cpu_base, extra = cpu_leg(tris, nodes, rays, min(args.cpu_sample, n), trav)
        counts = extra["counts"]
        got = d_hits.cpu().numpy().view(rt.HIT_DTYPE)
        k = len(extra["ref_hits"])
        parity = {"rays_checked": k, "id_mismatches_vs_reference_order": int((got["prim"][:k] != extra["ref_hits"]["prim"]).sum())}
    roof = None
    if counts:
        b_ray = 32 + 8 + 32 * counts["node_boxes_per_ray"] + 48 * counts["tri_tests_per_ray"]
        avg_launch = statistics.mean(launch_ms) / 1e3
        achieved = b_ray * n / avg_launch / 1e9
        full3 = (args.tris, n) == (N_TRIS, N_RAYS) and sort and info.node_width == 4
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": DRAM_BYTES_PER_RAY * n if full3 else None,
                "traffic_note": "ncu dram bytes of a 2,097,152-ray launch on the same BVH, scaled by rays"
                                if full3 else "not captured for this shape",
                "peak_kind": peak_kind,
                "bytes_per_ray": b_ray, "node_boxes_per_ray": counts["node_boxes_per_ray"],
                "tri_tests_per_ray": counts["tri_tests_per_ray"],
                "kernel": f"k_trace_step<closest> (persistent warps, {info.node_width}-wide nodes)"
                          + ("; the step also runs the 3 reorder kernels" if sort else ""),
                "gpu_node_fetches_per_ray": gpu_nodes / n, "gpu_prim_tests_per_ray": gpu_tests / n,
                "fetched_bytes_per_ray": 40 + 64 * gpu_nodes / n + 64 * gpu_tests / n,
                "avg_launch_ms": avg_launch * 1e3,
                "frac_of_nominal_8TBps": achieved / NOMINAL_HBM_GBS}
        # the same launch measured in the bytes the kernel itself fetches (its
        # own node and triangle fetches, GPU counters), and in DRAM bytes
        fetched = roof["fetched_bytes_per_ray"] * n / avg_launch / 1e9
        roof["fetched_GBps"], roof["fetched_frac"] = fetched, fetched / peak
        if full3:
            dram = DRAM_BYTES_PER_RAY * n / avg_launch / 1e9
            roof["dram_GBps"], roof["dram_frac"] = dram, dram / peak
        if full3:
            roof["ncu_2Mi_ray_launch"] = {"l2_to_l1_bytes_per_ray": L2_TO_L1_BYTES_PER_RAY,
                                          "dram_bytes_per_ray": DRAM_BYTES_PER_RAY,
                                          "fp32_fma_pipe_active_pct": FMA_PIPE_PCT,
                                          "alu_pipe_active_pct": ALU_PIPE_PCT}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "config 3: 4,194,304-triangle soup, 16,777,216 incoherent rays, closest-hit"
                       if (args.tris, args.rays) == (N_TRIS, N_RAYS) else
                       f"config-3 shape: {args.tris} triangles, {args.rays} rays, closest-hit",
                       "triangles": args.tris, "rays": n, "bvh": ("S1 nodes: host LBVH, sorted leaves; traversed: binned-SAH tree over the same triangles"
                               if info.traversal_sah else "host LBVH, sorted leaves (traversed as built)"),
                       "leaf_size": info.leaf_size, "node_width": info.node_width,
                       "device_nodes": info.device_nodes, "bvh_depth": info.depth, "stack_need": info.stack_need,
                       "l2": l2_note(n, info),
                       "ray_order": "origin-bucketed inside the step (RT_TRACE_SORT)" if sort else "as given",
                       "launch": tuned if tuned else "default (not tuned)",
                       "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"},
            "roofline": roof, "cpu_baseline": cpu_base, "e2e": e2e, "clocks": clk,
            "batched": batched, "served": served, "render": render, "extras": extras,
            "gpu_launches": args.steps * (4 if sort else 1), "parity_sample": parity,
            "scene_build_s": info.build_seconds}
    # the headline figures of the long blocks above, last on the line, so
    # that a tail of the output still holds them
    summary = {}
    if tuned:
        summary["launch_config3"] = {k: (round(v, 3) if isinstance(v, float) else v) for k, v in tuned.items()}
    if batched:
        summary["batched_config4"] = {"plain_Grays_per_s": round(batched["plain"]["value"], 3),
                                      "batched_Grays_per_s": round(batched["batched"]["value"], 3),
                                      "speedup": round(batched["speedup"], 3), "identical_hits": batched["identical_hits"],
                                      "autotuned": batched["batched"]["autotuned"]}
    if render:
        summary["render_config2_Mpaths_per_s"] = {"extended": round(render["extended"]["value"], 1),
                                                  "reference": round(render["reference"]["value"], 1)}
    if served:
        summary["served_config5"] = served["summary"]
    line["summary"] = summary
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
