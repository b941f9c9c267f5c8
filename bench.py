#!/usr/bin/env python
"""Benchmark: Msamples/s of the plain one-image-per-launch GPU path.

Workload (single larger scene): 1.0M FP32 triangles from 64 seeded UV-spheres and
displaced grids, 40% Lambert / 40% GGX / 20% glass, a 2048x1024 procedural
equirect sky, 1920x1080, 64 spp, max 16 bounces, MIS next-event estimation
(PathTracing semantics). Synthetic, seeded. A step = one full render of that
image (132.7M samples) with the scene resident in HBM.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 runs independent replicas, one per GPU (each renders its own image with
its own seed; no data exchange): "scaling": "weak".
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

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

WORKLOAD = "spheres_grids_1M_1080p_64spp_pt16"
STRESS_WORKLOAD = "terrain_rocks_20M_2160p_256spp_pt12"
METRIC = "render_msamples_per_s"
UNIT = "Msamples/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--small", action="store_true", help="reduced workload for quick checks")
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="target CPU time of the CPU-baseline sample")
    ap.add_argument("--width", type=int, default=0, help="override (profiling runs only)")
    ap.add_argument("--height", type=int, default=0, help="override (profiling runs only)")
    ap.add_argument("--spp", type=int, default=0, help="override (profiling runs only)")
    ap.add_argument("--ref-seconds", type=float, default=20.0,
                    help="CPU seconds of the reference arm's sample per step (--impl reference)")
    ap.add_argument("--stress", action="store_true",
                    help="memory-bound stress scene: 20M triangles, 3840x2160, 256 spp, 8192x4096 env")
    ap.add_argument("--batch", action="store_true",
                    help="batched uneven instances: 64 scenes in shared waves vs 64 plain launches")
    ap.add_argument("--serve", action="store_true",
                    help="serving loop: Poisson request stream, p50/p99 latency vs the plain path")
    ap.add_argument("--requests", type=int, default=100, help="requests per arrival rate (--serve)")
    ap.add_argument("--wave-paths", type=int, default=0, help="serving wave size (0: auto)")
    ap.add_argument("--env-sampling", default="reference", choices=["reference", "alias"],
                    help="environment next-event sampler: the reference's tables, or the opt-in "
                         "alias table (a different, unbiased estimator)")
    return ap.parse_args()


def make_scene(args):
    import dataclasses
    from petrichor_gb300 import synth
    if args.stress:
        sc = synth.terrain_rocks()  # 20M tris, 3840x2160, 256 spp, 12 bounces, 8192x4096 env
    elif args.small:
        sc = synth.spheres_grids(tri_budget=100_000, width=480, height=270, spp=16, max_bounces=16,
                                 env_width=512, env_height=256)
    else:
        sc = synth.spheres_grids()  # 1.0M tris, 1920x1080, 64 spp, 16 bounces, 2048x1024 env
    over = {k: v for k, v in (("width", args.width), ("height", args.height), ("spp", args.spp)) if v}
    if over:
        sc = sc.copy_with(settings=dataclasses.replace(sc.settings, **over))
    return sc


def workload_name(args):
    if args.stress:
        name = STRESS_WORKLOAD
    else:
        name = WORKLOAD + ("_SMALL" if args.small else "")
    if args.width or args.height or args.spp:
        name += "_OVERRIDE"
    if getattr(args, "env_sampling", "reference") == "alias":
        name += "_ENV_ALIAS"
    return name


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4)
                          if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def cpu_baseline(scene, seconds: float, threads: int = 0):
    """The CPU oracle (a restatement of the reference renderer) on the host cores, on a
    bounded sample of the same workload: tiles spread evenly over the image at full spp."""
    import numpy as np
    import oracle
    o = oracle.OracleScene(scene)
    t0 = time.perf_counter()
    o.build_bvh()
    bvh_s = time.perf_counter() - t0
    n_tiles = o.num_tiles()
    ncores = threads or os.cpu_count() or 1
    # probe with one tile per core, then size the sample to the time target
    order = np.random.default_rng(0).permutation(n_tiles)
    probe = order[:ncores]
    _, secs, px = o.render_tiles(probe, threads)
    per_tile = secs / max(1, len(probe)) * ncores
    n = int(min(n_tiles, max(len(probe), seconds / max(per_tile, 1e-6) * ncores)))
    tiles = order[:n]
    _, secs, px = o.render_tiles(tiles, threads)
    samples = px * scene.settings.spp
    return {"value": samples / secs / 1e6, "unit": UNIT, "cores": ncores, "kind": "port",
            "sample": f"{len(tiles)} of {n_tiles} 16x16 tiles (random spread) at the full "
                      f"{scene.settings.spp} spp: {samples} samples in {secs:.2f} s; BVH build "
                      f"{bvh_s:.2f} s not included",
            "bvh_build_s": bvh_s}


def run_reference_arm(args):
    from petrichor_gb300 import replicas
    rank, world, local = replicas.rank_world_local()
    if rank != 0:  # the reference arm runs once, on rank 0's host cores
        return
    if args.env_sampling == "alias":
        print(json.dumps({"impl": "reference", "unavailable": "the reference has no alias-table "
                          "environment sampler (its AliasMethod is never called on the render path)"}))
        return
    scene = make_scene(args)
    import numpy as np
    import oracle
    o = oracle.OracleScene(scene)
    o.build_bvh()
    n_tiles = o.num_tiles()
    ncores = os.cpu_count() or 1
    order = np.random.default_rng(0).permutation(n_tiles)
    _, secs, _ = o.render_tiles(order[:ncores])
    per_tile = secs
    n = int(min(n_tiles, max(ncores, args.ref_seconds / max(per_tile, 1e-6) * ncores)))
    tiles = order[:n]
    for _ in range(args.warmup):
        o.render_tiles(tiles[:ncores])
    times = []
    px = 0
    for _ in range(args.steps):
        _, secs, px = o.render_tiles(tiles)
        times.append(secs)
    samples = px * scene.settings.spp
    ms = statistics.mean(times) * 1e3
    v = samples / (ms / 1e3) / 1e6
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload_name(args), "integrator": "PathTracing (MIS NEE)",
                   "sample_per_step": f"{len(tiles)} of {n_tiles} tiles at full spp"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": ncores, "kind": "port",
                         "sample": f"{len(tiles)} random 16x16 tiles x {scene.settings.spp} spp "
                                   f"per step ({samples} samples)"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def run_batch(args):
    """64 uneven scenes (triangles log-uniform 10k-2M, pixels log-uniform 256^2-1024^2,
    aspect 0.5-2, spp in {4,16,64,256}, own 1024x512 skies): one pt_batch_render vs
    64 sequential pt_render_device launches; films checked identical."""
    import numpy as np
    import torch
    from petrichor_gb300 import capi, synth
    t0 = time.perf_counter()
    scenes = synth.batch_instances()
    gen_s = time.perf_counter() - t0
    ctx = capi.Context(0)
    t0 = time.perf_counter()
    sids = [ctx.upload(s) for s in scenes]
    upload_s = time.perf_counter() - t0
    jobs = []
    for k, (sc, sid) in enumerate(zip(scenes, sids)):
        st = capi.settings_from_scene(sc, capi.MODE_WAVEFRONT, seed=k + 1)
        film = torch.empty(st.width * st.height * 3, dtype=torch.float32, device="cuda")
        jobs.append((sid, capi.camera_from_scene(sc), st, film))
    samples = sum(j[2].width * j[2].height * j[2].spp for j in jobs)
    tris = sum(s.num_triangles for s in scenes)
    stream = torch.cuda.Stream()
    plain = [torch.empty_like(j[3]) for j in jobs]

    def run_plain():
        for (sid, cam, st, _), f in zip(jobs, plain):
            ctx.render_device(sid, cam, st, f.data_ptr(), stream.cuda_stream)

    def run_batched():
        ctx.batch_render([(sid, cam, st, f.data_ptr()) for sid, cam, st, f in jobs], stream.cuda_stream)

    # autotuned launch configuration (grid, pixel bands, graph replay), probed on the
    # job with the most samples; both arms then run with it
    t0 = time.perf_counter()
    big = max(jobs, key=lambda j: j[2].width * j[2].height * j[2].spp)
    tuning = ctx.autotune(big[0], big[1], big[2], probe_spp=4).as_dict()
    tune_s = time.perf_counter() - t0

    def run_batched_ungraphed():
        t = ctx.get_tuning()
        ctx.set_tuning(t.wave_paths, t.blocks_per_sm, t.band_rows, 0)
        run_batched()
        torch.cuda.synchronize()
        ctx.set_tuning(t.wave_paths, t.blocks_per_sm, t.band_rows, t.use_graphs)

    for _ in range(max(1, args.warmup)):
        run_plain()
        run_batched()
    torch.cuda.synchronize()
    res = {}
    for name, fn in (("plain", run_plain), ("batched", run_batched),
                     ("batched_without_graphs", run_batched_ungraphed)):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        launches0 = ctx.stats().kernel_launches
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        secs = e0.elapsed_time(e1) / 1e3 / args.steps
        res[name] = {"ms_per_batch": secs * 1e3, "msamples_per_s": samples / secs / 1e6,
                     "gpu_launches_per_batch": (ctx.stats().kernel_launches - launches0) / args.steps}
    same = all(torch.equal(a[3], b) for a, b in zip(jobs, plain))
    print(json.dumps({
        "metric": "batched_msamples_per_s", "value": res["batched"]["msamples_per_s"], "unit": UNIT,
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": res["batched"]["ms_per_batch"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "batch_64_uneven_spheres_grids", "scenes": len(scenes),
                   "triangles_total": tris, "samples_per_batch": samples,
                   "scene_gen_s": round(gen_s, 1), "upload_s": round(upload_s, 1),
                   "autotuned": tuning, "autotune_s": round(tune_s, 2)},
        "plain_sequential": res["plain"], "batched": res["batched"],
        "batched_without_graphs": res["batched_without_graphs"],
        "speedup_vs_plain": res["batched"]["msamples_per_s"] / res["plain"]["msamples_per_s"],
        "films_identical_to_plain": bool(same),
    }))
    ctx.close()


def run_serve(args):
    """8 resident scenes (100k-4M triangles, 8192x4096 skies); Poisson arrivals at
    20/100/500 requests/s; per request resolution log-uniform 128^2-2048^2 (aspect
    0.5-2), spp in {1,8,32,128}, depth 4-16. The continuous-batching server vs the
    plain path serving the same stream one request at a time."""
    import numpy as np
    import torch
    from petrichor_gb300 import capi, synth
    t0 = time.perf_counter()
    scenes = synth.serving_scenes()
    gen_s = time.perf_counter() - t0
    ctx = capi.Context(0)
    sids = [ctx.upload(s) for s in scenes]
    resident = sum(ctx.scene_info(sid).device_bytes for sid in sids)
    cams = [capi.camera_from_scene(s) for s in scenes]
    out = {"metric": "serve_msamples_per_s", "unit": UNIT, "n_gpus": 1, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": "serve_8_scenes_poisson", "scenes": len(scenes),
                      "triangles": [s.num_triangles for s in scenes],
                      "resident_bytes": int(resident), "requests_per_rate": args.requests,
                      "state_budget_bytes": 150 * 2**30, "scene_gen_s": round(gen_s, 1)},
           "rates": {}}
    max_px = 2048 * 2048 * 2
    pinned = [torch.empty(max_px * 3, dtype=torch.float32, pin_memory=True) for _ in range(4)]

    def settings(w, h, spp, depth, seed):
        st = capi.settings_from_scene(scenes[0], capi.MODE_WAVEFRONT, seed=seed, width=w, height=h,
                                      spp=spp, max_bounces=depth)
        return st

    for rate in (20.0, 100.0, 500.0):
        stream_ = synth.request_stream(int(rate), rate, args.requests)
        samples = sum(w * h * spp for _, _, w, h, spp, _ in stream_)
        res = {}
        # ---- continuous-batching server
        ctx.serve_start(wave_paths=args.wave_paths, max_active=512, state_budget=150 * 2**30)
        # pinned host films, as for the plain path
        films = [torch.empty(h * w * 3, dtype=torch.float32, pin_memory=True).numpy().reshape(h, w, 3)
                 for _, _, w, h, _, _ in stream_]
        rids = []
        t_start = time.perf_counter()
        for k, (t, sc, w, h, spp, depth) in enumerate(stream_):
            dt = t_start + t - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            rids.append(ctx.serve_submit(sids[sc], cams[sc], settings(w, h, spp, depth, k + 1),
                                         film_host=films[k]))
        sts = [ctx.serve_wait(r, 600) for r in rids]
        ctx.serve_stop()
        lat = np.array([s.done_s - s.submit_s for s in sts])
        first = min(s.submit_s for s in sts)
        last = max(s.done_s for s in sts)
        res["batched_serve"] = {"msamples_per_s": samples / (last - first) / 1e6,
                                "p50_ms": float(np.percentile(lat, 50) * 1e3),
                                "p99_ms": float(np.percentile(lat, 99) * 1e3),
                                "completed": sum(s.state == capi.REQ_DONE for s in sts)}
        # ---- plain path: one pt_render per request, in arrival order
        lat_p = []
        t_start = time.perf_counter()
        t_first = None
        for k, (t, sc, w, h, spp, depth) in enumerate(stream_):
            now = time.perf_counter()
            if t_start + t > now:
                time.sleep(t_start + t - now)
            arrival = t_start + t
            t_first = t_first or arrival
            film = pinned[k % 4][: w * h * 3].numpy().reshape(h, w, 3)
            ctx.render(sids[sc], cams[sc], settings(w, h, spp, depth, k + 1), out=film)
            lat_p.append(time.perf_counter() - arrival)
            if k == 0:
                same_first = bool(np.array_equal(film.view(np.uint32), films[0].view(np.uint32)))
        t_end = time.perf_counter()
        lat_p = np.array(lat_p)
        res["plain"] = {"msamples_per_s": samples / (t_end - t_first) / 1e6,
                        "p50_ms": float(np.percentile(lat_p, 50) * 1e3),
                        "p99_ms": float(np.percentile(lat_p, 99) * 1e3)}
        res["speedup_vs_plain"] = res["batched_serve"]["msamples_per_s"] / res["plain"]["msamples_per_s"]
        res["first_film_identical_to_plain"] = same_first
        res["samples"] = samples
        out["rates"][str(int(rate))] = res
    top = out["rates"]["500"]
    out["value"] = top["batched_serve"]["msamples_per_s"]
    out["p50_ms"] = top["batched_serve"]["p50_ms"]
    out["p99_ms"] = top["batched_serve"]["p99_ms"]
    print(json.dumps(out))
    ctx.close()


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.batch:
        return run_batch(args)
    if args.serve:
        return run_serve(args)
    import numpy as np
    import torch
    from petrichor_gb300 import capi

    from petrichor_gb300 import replicas
    rank, world, local = replicas.rank_world_local()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()

    t0 = time.perf_counter()
    scene = make_scene(args)
    gen_s = time.perf_counter() - t0
    st = scene.settings
    ctx = capi.Context(local)
    t0 = time.perf_counter()
    sid = ctx.upload(scene)
    upload_s = time.perf_counter() - t0
    info = ctx.scene_info(sid)
    cam = capi.camera_from_scene(scene)
    env = capi.ENV_SAMPLING_ALIAS if args.env_sampling == "alias" else capi.ENV_SAMPLING_REFERENCE
    sets = capi.settings_from_scene(scene, capi.MODE_WAVEFRONT, seed=replicas.replica_seed(1, rank),
                                    env_sampling=env)
    npx = st.width * st.height
    samples_per_step = npx * st.spp
    film = torch.empty(npx * 3, dtype=torch.float32, device="cuda")
    # a real stream (not the legacy default stream, whose handle is 0): the
    # renders and the timing events are enqueued on it
    stream = torch.cuda.Stream()

    def step():
        ctx.render_device(sid, cam, sets, film.data_ptr(), stream.cuda_stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    launches0 = ctx.stats().kernel_launches
    clocks = ClockSampler(local)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    clocks.stop()
    barrier()
    secs = e0.elapsed_time(e1) / 1e3
    launches = ctx.stats().kernel_launches - launches0
    secs = replicas.max_over_ranks(secs, dist, "cuda")
    value = replicas.job_throughput(world, samples_per_step * args.steps, secs) / 1e6

    # ---- end to end through the C ABI with a host film (pinned): per step the
    # camera + settings go in (kernel arguments) and the film comes back.
    host = torch.empty(npx * 3, dtype=torch.float32, pin_memory=True)
    host_np = host.numpy().reshape(st.height, st.width, 3)
    ctx.render(sid, cam, sets, out=host_np)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.render(sid, cam, sets, out=host_np)
        _ = float(host_np[0, 0, 0])
    e2e_s = time.perf_counter() - t0
    e2e_s = replicas.max_over_ranks(e2e_s, dist, "cuda")
    e2e = replicas.job_throughput(world, samples_per_step * args.steps, e2e_s) / 1e6
    img_mean = float(host_np.mean())

    # ---- roofline of the dominant kernel (CUDA events around every stage launch)
    prof = ctx.render_profile(sid, cam, sets, film.data_ptr(), count_reference=True).as_dict()
    prof2 = ctx.render_profile(sid, cam, sets, film.data_ptr(), count_reference=False).as_dict()
    stages = {k: prof2[k] for k in ("raygen_ms", "extend_ms", "shade_ms", "shadow_ms", "accumulate_ms")}
    dominant = max(stages, key=stages.get)
    # algorithmic bytes of a traced ray (reference traversal order): 32 B per node
    # popped and slab-tested, 48 B per triangle test, 32 B ray in, 16 B hit out
    rays = max(1, prof["ref_rays"])
    bytes_per_ray = (32.0 * prof["ref_node_tests"] + 48.0 * prof["ref_tri_tests"]) / rays + 48.0
    ext_launches = max(1, prof2["extend_launches"])
    bytes_per_launch = bytes_per_ray * prof2["extend_rays"] / ext_launches
    avg_launch_s = prof2["extend_ms"] / 1e3 / ext_launches
    achieved = bytes_per_launch / avg_launch_s / 1e9
    peaks_path = os.path.join(HERE, "MEASURED_PEAKS.json")
    peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        with open(peaks_path) as fh:
            peak, peak_src = float(json.load(fh)["hbm_gbs"]), "measured"
    traffic = None
    # measured DRAM bytes per extension ray (ncu launch list) of the named workloads only
    traffic_files = {WORKLOAD: "extend_kernel_traffic_spheres_grids_1M_1080p_64spp.json",
                     STRESS_WORKLOAD: "extend_kernel_traffic_terrain_rocks_20M_2160p_256spp.json"}
    tp = os.path.join(HERE, "profiles", traffic_files.get(workload_name(args), "-"))
    if os.path.exists(tp):
        with open(tp) as fh:
            t = json.load(fh)
        traffic = t["dram_bytes_per_ray"] * prof2["extend_rays"] / ext_launches

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": secs / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload_name(args),
                   "triangles": info.num_triangles, "bvh_nodes": info.num_nodes,
                   "resolution": [st.width, st.height], "spp": st.spp, "max_bounces": st.max_bounces,
                   "env": list(scene.env.texture.shape[:2][::-1]), "mode": "wavefront",
                   "env_sampling": args.env_sampling,
                   "parallelism": f"replicas{world}",
                   "l2": "working set > L2 (scene ~%.0f MB resident + wave state)" % (
                       info.device_bytes / 1e6),
                   "scene_gen_s": round(gen_s, 2), "scene_upload_s": round(upload_s, 2),
                   "bvh_build_s": round(info.build_seconds, 2)},
        "e2e": {"value": e2e, "unit": UNIT,
                "h2d_bytes_per_step": 64 + 48, "d2h_bytes_per_step": npx * 12},
        "gpu_launches": int(launches),
        "clocks": clocks.summary(),
        "roofline": {"bound": "hbm", "kernel": "ExtendKernel (closest-hit traversal)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_source": peak_src,
                     "bytes_per_ray": bytes_per_ray,
                     "ref_nodes_per_ray": prof["ref_node_tests"] / rays,
                     "ref_tris_per_ray": prof["ref_tri_tests"] / rays,
                     "dominant_stage": dominant, "stage_ms": stages,
                     "rays_extended": prof2["extend_rays"], "shadow_rays": prof2["shadow_rays"],
                     "mrays_per_s": (prof2["extend_rays"] + prof2["shadow_rays"]) /
                                    (sum(stages.values()) / 1e3) / 1e6},
        "image_mean": img_mean,
    }
    if rank == 0 and world == 1:
        line["cpu_baseline"] = cpu_baseline(scene, args.cpu_seconds)
    ctx.release(sid)
    ctx.close()
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
