#!/usr/bin/env python
"""Benchmark: Msamples/s of the GPU path-tracing core, plain and in its batched and
serving forms.

Default line (one JSON line, N=1 unless --gpus):
* plain path, the single larger scene: 1.0M FP32 triangles from 64 seeded UV-spheres and
  displaced grids, 40% Lambert / 40% GGX / 20% glass, a 2048x1024 procedural equirect sky,
  1920x1080, 64 spp, max 16 bounces, MIS next-event estimation (PathTracing semantics).
  Synthetic, seeded. A step = one full render of that image (132.7M samples) with the
  scene resident in HBM. `value` times the device render; `e2e` goes through pt_render
  with a host film; `e2e_dropin` through the C++ Petrichor::Render(const Scene&), which
  flattens, uploads, builds the BVH, renders and copies back on every call.
* `image_error`: the GPU image mean against the CPU oracle's (the reference's estimator)
  on the tiles the CPU-baseline leg renders, with standard errors from replicates.
* `serve`: the continuous-batching server against the plain path on a Poisson request
  stream over 8 resident scenes (about 12 GB), with p50/p99 latency, per-request error
  and the attainable speed-up of that stream.
* `batch`: 64 uneven scenes in one batched launch against 64 plain launches.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--plain-only] [--batch] [--serve] [--stress] [--small]

N > 1 runs independent replicas, one per GPU (each renders its own image with its own
seed; no data exchange): "scaling": "weak". The serve and batch objects run on rank 0's
GPU only when N = 1.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

WORKLOAD = "spheres_grids_1M_1080p_64spp_pt16"
STRESS_WORKLOAD = "terrain_rocks_20M_2160p_256spp_pt12"
METRIC = "render_msamples_per_s"
UNIT = "Msamples/s"
L2_NOTE = "inputs larger than L2 (scene + wave state); no flush between steps"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--small", action="store_true", help="reduced workload for quick checks")
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="target CPU time of the CPU-baseline sample")
    ap.add_argument("--err-seconds", type=float, default=24.0,
                    help="CPU time of the oracle replicates behind image_error")
    ap.add_argument("--width", type=int, default=0, help="override (profiling runs only)")
    ap.add_argument("--height", type=int, default=0, help="override (profiling runs only)")
    ap.add_argument("--spp", type=int, default=0, help="override (profiling runs only)")
    ap.add_argument("--max-bounces", type=int, default=0, help="override (profiling runs only)")
    ap.add_argument("--ref-seconds", type=float, default=20.0,
                    help="CPU seconds of the reference arm's sample per step (--impl reference)")
    ap.add_argument("--stress", action="store_true",
                    help="memory-bound stress scene: 20M triangles, 3840x2160, 256 spp, 8192x4096 env")
    ap.add_argument("--batch", action="store_true",
                    help="only the batched form: 64 scenes in shared waves vs 64 plain launches")
    ap.add_argument("--serve", action="store_true",
                    help="only the serving loop at 20/100/500 requests/s vs the plain path")
    ap.add_argument("--stress-forms", action="store_true",
                    help="the stress scene's frame as 4 requests of a quarter of its spp: served, "
                         "batched and plain, against one plain render of the whole frame")
    ap.add_argument("--plain-only", action="store_true",
                    help="the plain line alone (no image error, drop-in, serve or batch objects)")
    ap.add_argument("--no-cpu-baseline", action="store_true",
                    help="skip the CPU-baseline leg (profiling and A/B runs only)")
    ap.add_argument("--trace-primary", action="store_true",
                    help="trace the first bounce through the BVH instead of rasterising it "
                         "(A/B runs; the films are the same)")
    ap.add_argument("--tuning", default="",
                    help="pt_tuning fields of the plain line, k=v,... (A/B runs; films are the same)")
    ap.add_argument("--requests", type=int, default=100, help="requests per arrival rate (serve)")
    ap.add_argument("--serve-rates", default="",
                    help="comma-separated arrival rates of the serve object (default 500; "
                         "--serve: 20,100,500)")
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
    over = {k: v for k, v in (("width", args.width), ("height", args.height), ("spp", args.spp),
                              ("max_bounces", args.max_bounces)) if v}
    if over:
        sc = sc.copy_with(settings=dataclasses.replace(sc.settings, **over))
    return sc


def workload_name(args):
    if args.stress:
        name = STRESS_WORKLOAD
    else:
        name = WORKLOAD + ("_SMALL" if args.small else "")
    if args.width or args.height or args.spp or args.max_bounces:
        name += "_OVERRIDE"
    if getattr(args, "env_sampling", "reference") == "alias":
        name += "_ENV_ALIAS"
    return name


def workload_config(args, scene, world):
    """The `config` object, identical in both arms (same workload, same keys)."""
    st = scene.settings
    env = scene.env.texture
    return {"workload": workload_name(args), "triangles": scene.num_triangles,
            "resolution": [st.width, st.height], "spp": st.spp, "max_bounces": st.max_bounces,
            "env": list(env.shape[:2][::-1]) if env is not None else None,
            "integrator": "PathTracing (MIS NEE)" if st.integrator == 1 else "SimplePathTracing",
            "env_sampling": args.env_sampling, "parallelism": f"replicas{world}", "l2": L2_NOTE}


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


# ------------------------------------------------------------------ CPU baseline (oracle)
def cpu_baseline(scene, seconds: float, threads: int = 0):
    """The CPU oracle (a restatement of the reference renderer) on the host cores, on a
    bounded sample of the same workload: tiles spread evenly over the image at full spp.
    Returns (baseline dict, oracle scene, film, rendered tile list, per-tile seconds)."""
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
    film, secs, px = o.render_tiles(tiles, threads)
    samples = px * scene.settings.spp
    info = {"value": samples / secs / 1e6, "unit": UNIT, "cores": ncores, "kind": "port",
            "sample": f"{len(tiles)} of {n_tiles} 16x16 tiles (random spread) at the full "
                      f"{scene.settings.spp} spp: {samples} samples in {secs:.2f} s; BVH build "
                      f"{bvh_s:.2f} s not included",
            "bvh_build_s": bvh_s}
    return info, o, film, tiles, secs / max(1, len(tiles)) * ncores, order


def run_reference_arm(args):
    from petrichor_gb300 import replicas
    rank, world, local = replicas.rank_world_local()
    if rank != 0:  # the reference arm runs once, on rank 0's host cores
        return
    if args.env_sampling == "alias":
        print(json.dumps({"impl": "reference", "unavailable": "the reference has no alias-table "
                          "environment sampler (its AliasMethod is never called on the render path)"}))
        return
    if args.batch or args.serve or args.stress_forms:
        print(json.dumps({"impl": "reference", "unavailable": "the reference has no batched or "
                          "serving form; its arm times the plain render workload only"}))
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
        "config": workload_config(args, scene, world),
        "sample_per_step": f"{len(tiles)} of {n_tiles} tiles at full spp",
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": ncores, "kind": "port",
                         "sample": f"{len(tiles)} random 16x16 tiles x {scene.settings.spp} spp "
                                   f"per step ({samples} samples)"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


# ------------------------------------------------------------------ measurements
def l2_read_peak(ctx):
    """Measured L2 read bandwidth (pt_probe_bandwidth): the roofline denominator of the
    traversal kernels, whose algorithmic bytes are served mostly from L2."""
    mib, passes, reps = 32, 16, 10
    return {"gbs": ctx.probe_l2_read_gbs(mib << 20, passes, reps),
            "method": f"pt_probe_bandwidth: a {mib} MiB buffer (L2-resident) read {passes} times "
                      f"per launch with 16-byte L1-bypassing loads by 4 blocks of 512 threads per "
                      f"SM, {reps} launches between CUDA events after one warm-up"}


def counters_profile(name):
    """Small-case ncu counters of ExtendKernel committed under profiles/ (None if absent)."""
    p = os.path.join(HERE, "profiles", name)
    if not os.path.exists(p):
        return None
    with open(p) as fh:
        return json.load(fh)


def image_error(ctx, sid, cam, sets, scene, film_t, stream, o, cpu_film, cpu_tiles, order,
                per_tile_s, seconds, torch):
    """Image mean of the throughput path against the reference's estimator (the oracle).

    * independent-stream comparison: R oracle replicates with decorrelated per-tile
      streams over a random spread of tiles U, against S GPU renders with distinct
      seeds over the same tiles; the standard error pools both sets' replicate variance
      (the same estimator, so the same variance);
    * reference-stream comparison: the CPU-baseline leg's film (the reference's own
      random streams) against the mean GPU image over the same tiles T (one replicate of
      the reference estimator, so no standard error of its own)."""
    import ctypes
    import numpy as np
    from petrichor_gb300 import capi
    S, R = 8, 3
    st = scene.settings
    ncores = os.cpu_count() or 1
    n_u = int(min(len(order), max(ncores, seconds / R / max(per_tile_s, 1e-6) * ncores)))
    tiles_u = order[:n_u]
    mask_u = o.tile_mask(tiles_u)
    mask_t = o.tile_mask(cpu_tiles)
    host = torch.empty(st.width * st.height * 3, dtype=torch.float32, pin_memory=True)
    g_u, g_t = [], []
    for s in range(S):
        seeded = capi.settings_from_scene(scene, capi.MODE_WAVEFRONT, seed=9001 + s,
                                          env_sampling=sets.env_sampling)
        ctx.render_device(sid, cam, seeded, film_t.data_ptr(), stream.cuda_stream)
        host.copy_(film_t, non_blocking=True)
        torch.cuda.synchronize()
        img = host.numpy().reshape(st.height, st.width, 3)
        g_u.append(float(img[mask_u].mean()))
        g_t.append(float(img[mask_t].mean()))
    t0 = time.perf_counter()
    o_u = [float(o.render_tiles_decorrelated(tiles_u, seed=101 + r)[0][mask_u].mean())
           for r in range(R)]
    o_secs = time.perf_counter() - t0
    g_u, o_u = np.array(g_u), np.array(o_u)
    pooled = (((g_u - g_u.mean()) ** 2).sum() + ((o_u - o_u.mean()) ** 2).sum()) / (S - 1 + R - 1)
    se = math.sqrt(pooled * (1.0 / S + 1.0 / R))
    ref_mean = float(o_u.mean())
    rel = abs(float(g_u.mean()) - ref_mean) / ref_mean
    ref_t = float(cpu_film[mask_t].mean())
    # independent-stream spread scaled to T's sample count: one reference replicate plus
    # the mean of S GPU seeds (the reference's correlated streams spread wider, so the
    # z below overstates the deviation)
    var_t = pooled * float(mask_u.sum()) / max(1.0, float(mask_t.sum()))
    se_t = math.sqrt(var_t * (1.0 + 1.0 / S))
    g_t_mean = float(np.mean(g_t))
    return {
        "rel": rel, "sigma_rel": se / ref_mean, "z": rel * ref_mean / se if se > 0 else None,
        "pass": bool(rel <= 0.005 or rel <= 4.5 * se / ref_mean),
        "gpu_mean": float(g_u.mean()), "oracle_mean": ref_mean,
        "gpu_seeds": S, "oracle_replicates": R, "tiles": int(n_u), "of_tiles": int(len(order)),
        "samples_per_replicate": int(mask_u.sum()) * st.spp, "oracle_seconds": round(o_secs, 2),
        "rule": "rel <= 0.5% or within 4.5 sigma; sigma from pooled replicate variance",
        "reference_stream": {"tiles": int(len(cpu_tiles)), "oracle_mean": ref_t,
                             "gpu_mean": g_t_mean, "rel": abs(g_t_mean - ref_t) / ref_t,
                             "sigma_rel": se_t / ref_t,
                             "z": abs(g_t_mean - ref_t) / se_t if se_t > 0 else None,
                             "note": "one replicate of the reference's own streams (the CPU "
                                     "baseline's film) against the mean of the GPU seeds; sigma "
                                     "from the independent-stream spread, which the reference's "
                                     "correlated streams exceed"},
    }


def dropin_client():
    """Builds the C++ drop-in client (tests/cpp/drop_in_render.cpp) against the library."""
    from petrichor_gb300 import _build
    lib = _build.build()
    libdir = os.path.dirname(lib)
    exe = os.path.join(libdir, "drop_in_render")
    src = os.path.join(HERE, "tests", "cpp", "drop_in_render.cpp")
    if not os.path.exists(exe) or os.path.getmtime(exe) < max(os.path.getmtime(src),
                                                               os.path.getmtime(lib)):
        subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(HERE, "include"), src,
                        "-L", libdir, "-lpetrichor_gb300", f"-Wl,-rpath,{libdir}", "-o", exe],
                       check=True, capture_output=True)
    return exe


def e2e_dropin(scene, steps):
    """Petrichor::Render(const Scene&) through the C++ API (wavefront mode): per call it
    flattens the scene, uploads it, builds the BVH on the device, renders, copies the
    film into the Texture2D and releases the scene. Wall time of each call."""
    from petrichor_gb300 import scene_io
    st = scene.settings
    try:
        exe = dropin_client()
    except (subprocess.CalledProcessError, OSError) as e:
        return {"unavailable": f"C++ client did not build: {str(e)[:200]}"}
    with tempfile.TemporaryDirectory() as td:
        sp = os.path.join(td, "scene.ptscene")
        with open(sp, "wb") as fh:
            fh.write(scene_io.scene_bytes(scene))
        r = subprocess.run([exe, sp, os.path.join(td, "film.bin"), "wavefront", "--repeat",
                            str(steps)], capture_output=True, text=True, timeout=1200)
    if r.returncode != 0:
        return {"unavailable": f"client exit {r.returncode}: {(r.stdout + r.stderr)[-300:]}"}
    out = json.loads(r.stdout.strip().splitlines()[-1])
    calls = out["call_seconds"]
    samples = st.width * st.height * st.spp
    h2d = sum(a.nbytes for a in (scene.positions, scene.normals, scene.uvs, scene.indices,
                                 scene.tri_material, scene.tri_shading))
    if scene.env.texture is not None:
        h2d += scene.env.texture.size * 4
    return {"value": samples / statistics.mean(calls) / 1e6, "unit": UNIT,
            "call_seconds": calls, "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": st.width * st.height * 12,
            "path": "C++ Petrichor::Render(const Scene&): flatten + upload + device BVH build + "
                    "render + film copy + release per call"}


# ------------------------------------------------------------------ batched form
def batch_summary(args, steps: int, warmup: int):
    """64 uneven scenes (triangles log-uniform 10k-2M, pixels log-uniform 256^2-1024^2,
    aspect 0.5-2, spp in {4,16,64,256}, own 1024x512 skies): one pt_batch_render vs
    64 sequential pt_render_device launches; films checked identical."""
    import torch
    from petrichor_gb300 import capi, synth
    t0 = time.perf_counter()
    scenes = synth.batch_instances()
    gen_s = time.perf_counter() - t0
    ctx = capi.Context(0)
    try:
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
            ctx.batch_render([(sid, cam, st, f.data_ptr()) for sid, cam, st, f in jobs],
                             stream.cuda_stream)

        # autotuned launch configuration (grid, pixel bands, graph replay), probed on the
        # job with the most samples; both arms then run with it
        t0 = time.perf_counter()
        big = max(jobs, key=lambda j: j[2].width * j[2].height * j[2].spp)
        tuning = ctx.autotune(big[0], big[1], big[2], probe_spp=4).as_dict()
        tune_s = time.perf_counter() - t0

        def run_batched_ungraphed():
            t = ctx.get_tuning()
            keep = dict(wave_paths=t.wave_paths, blocks_per_sm=t.blocks_per_sm, band_rows=t.band_rows,
                        sort_rays=t.sort_rays, tail_bounce=t.tail_bounce,
                        primary_traversal=t.primary_traversal)
            ctx.set_tuning(use_graphs=0, **keep)
            run_batched()
            torch.cuda.synchronize()
            ctx.set_tuning(use_graphs=t.use_graphs, **keep)

        for _ in range(max(1, warmup)):
            run_plain()
            run_batched()
        torch.cuda.synchronize()
        res = {}
        for name, fn in (("plain", run_plain), ("batched", run_batched),
                         ("batched_without_graphs", run_batched_ungraphed)):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            launches0 = ctx.stats().kernel_launches
            e0.record(stream)
            for _ in range(steps):
                fn()
            e1.record(stream)
            torch.cuda.synchronize()
            secs = e0.elapsed_time(e1) / 1e3 / steps
            res[name] = {"ms_per_batch": secs * 1e3, "msamples_per_s": samples / secs / 1e6,
                         "gpu_launches_per_batch": (ctx.stats().kernel_launches - launches0) / steps}
        same = all(torch.equal(a[3], b) for a, b in zip(jobs, plain))
    finally:
        ctx.close()
    return {
        "workload": "batch_64_uneven_spheres_grids", "scenes": len(scenes),
        "triangles_total": tris, "samples_per_batch": samples, "steps": steps,
        "msamples_per_s": res["batched"]["msamples_per_s"],
        "plain_msamples_per_s": res["plain"]["msamples_per_s"],
        "speedup_vs_plain": res["batched"]["msamples_per_s"] / res["plain"]["msamples_per_s"],
        "kernels_per_batch": res["batched"]["gpu_launches_per_batch"],
        "plain_sequential": res["plain"], "batched": res["batched"],
        "batched_without_graphs": res["batched_without_graphs"],
        "films_identical_to_plain": bool(same),
        "scene_gen_s": round(gen_s, 1), "upload_s": round(upload_s, 1),
        "autotuned": tuning, "autotune_s": round(tune_s, 2),
    }


def run_batch(args):
    b = batch_summary(args, args.steps, args.warmup)
    print(json.dumps({
        "metric": "batched_msamples_per_s", "value": b["msamples_per_s"], "unit": UNIT,
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": b["batched"]["ms_per_batch"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": b["workload"], "scenes": b["scenes"],
                   "triangles_total": b["triangles_total"], "samples_per_batch": b["samples_per_batch"],
                   "l2": L2_NOTE},
        "batch": b}))


# ------------------------------------------------------------------ serving form
def full_rate_probe(ctx, sid, cam, scene, depth, film_ptr, stream, torch, cache):
    """Msamples/s of the plain path on one whole-GPU wave of this scene at this depth
    (2048x2048 at 32 spp = 2^27 paths, the largest wave, whose first bounce is
    rasterised on every serving scene): the rate a request's samples could reach if
    the GPU were always full. Cached per (scene, depth)."""
    from petrichor_gb300 import capi
    key = (sid, depth)
    if key not in cache:
        st = capi.settings_from_scene(scene, capi.MODE_WAVEFRONT, seed=77, width=2048,
                                      height=2048, spp=32, max_bounces=depth)
        ctx.render_device(sid, cam, st, film_ptr, stream.cuda_stream)  # warm
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.render_device(sid, cam, st, film_ptr, stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        cache[key] = 2048 * 2048 * 32 / (e0.elapsed_time(e1) / 1e3) / 1e6
    return cache[key]


def serve_summary(args, rates, count: int, oracle_checks: int = 3):
    """8 resident scenes (100k-4M triangles, own 8192x4096 skies and 4096^2 material maps:
    about 12 GB resident); Poisson arrivals; per request resolution log-uniform
    128^2-2048^2 (aspect 0.5-2), spp in {1,8,32,128}, depth 4-16. The continuous-batching
    server against the plain path serving the same stream one request at a time."""
    import numpy as np
    import torch
    from petrichor_gb300 import capi, synth
    t0 = time.perf_counter()
    scenes = synth.serving_scenes()
    gen_s = time.perf_counter() - t0
    ctx = capi.Context(0)
    out = {}
    try:
        t0 = time.perf_counter()
        sids = [ctx.upload(s) for s in scenes]
        upload_s = time.perf_counter() - t0
        resident = sum(ctx.scene_info(sid).device_bytes for sid in sids)
        cams = [capi.camera_from_scene(s) for s in scenes]
        out["config"] = {"workload": "serve_8_scenes_poisson", "scenes": len(scenes),
                         "triangles": [s.num_triangles for s in scenes],
                         "resident_bytes": int(resident), "requests_per_rate": count,
                         "state_budget_bytes": 150 * 2 ** 30, "scene_gen_s": round(gen_s, 1),
                         "upload_s": round(upload_s, 1)}
        max_px = max(w * h for r in rates for _, _, w, h, _, _ in synth.request_stream(int(r), r, count))
        pinned = [torch.empty(max_px * 3, dtype=torch.float32, pin_memory=True) for _ in range(2)]
        probe_film = torch.empty(2048 * 2048 * 3, dtype=torch.float32, device="cuda")
        probe_stream = torch.cuda.Stream()
        rate_cache = {}

        def settings(w, h, spp, depth, seed):
            return capi.settings_from_scene(scenes[0], capi.MODE_WAVEFRONT, seed=seed, width=w,
                                            height=h, spp=spp, max_bounces=depth)

        out["rates"] = {}
        for rate in rates:
            stream_ = synth.request_stream(int(rate), rate, count)
            samples = sum(w * h * spp for _, _, w, h, spp, _ in stream_)
            res = {"samples": samples}
            # ---- continuous-batching server, host films (pinned, as for the plain path)
            ctx.serve_start(wave_paths=args.wave_paths, max_active=512, state_budget=150 * 2 ** 30)
            films = [torch.empty(h * w * 3, dtype=torch.float32, pin_memory=True).numpy().reshape(h, w, 3)
                     for _, _, w, h, _, _ in stream_]
            rids = []
            launches0 = ctx.stats().kernel_launches
            t_start = time.perf_counter()
            for k, (t, sc, w, h, spp, depth) in enumerate(stream_):
                dt = t_start + t - time.perf_counter()
                if dt > 0:
                    time.sleep(dt)
                rids.append(ctx.serve_submit(sids[sc], cams[sc], settings(w, h, spp, depth, k + 1),
                                             film_host=films[k]))
            sts = [ctx.serve_wait(r, 600) for r in rids]
            ctx.serve_stop()
            serve_launches = ctx.stats().kernel_launches - launches0
            lat = np.array([s.done_s - s.submit_s for s in sts])
            first = min(s.submit_s for s in sts)
            last = max(s.done_s for s in sts)
            res["batched_serve"] = {"msamples_per_s": samples / (last - first) / 1e6,
                                    "p50_ms": float(np.percentile(lat, 50) * 1e3),
                                    "p99_ms": float(np.percentile(lat, 99) * 1e3),
                                    "completed": sum(s.state == capi.REQ_DONE for s in sts),
                                    "gpu_launches": int(serve_launches)}
            # ---- plain path: one pt_render per request, in arrival order; each film is
            # compared with the served film of the same request
            lat_p, service, errs, identical = [], [], [], 0
            t_start = time.perf_counter()
            t_first = None
            for k, (t, sc, w, h, spp, depth) in enumerate(stream_):
                now = time.perf_counter()
                if t_start + t > now:
                    time.sleep(t_start + t - now)
                arrival = t_start + t
                t_first = t_first or arrival
                film = pinned[k % 2][: w * h * 3].numpy().reshape(h, w, 3)
                t1 = time.perf_counter()
                ctx.render(sids[sc], cams[sc], settings(w, h, spp, depth, k + 1), out=film)
                t2 = time.perf_counter()
                service.append(t2 - t1)
                lat_p.append(t2 - arrival)
                if np.array_equal(film.view(np.uint32), films[k].view(np.uint32)):
                    identical += 1
                    errs.append(0.0)
                else:
                    m = float(film.mean())
                    errs.append(abs(float(films[k].mean()) - m) / max(abs(m), 1e-30))
            t_end = time.perf_counter()
            lat_p = np.array(lat_p)
            plain_msps = samples / (t_end - t_first) / 1e6
            res["plain"] = {"msamples_per_s": plain_msps,
                            "p50_ms": float(np.percentile(lat_p, 50) * 1e3),
                            "p99_ms": float(np.percentile(lat_p, 99) * 1e3)}
            res["speedup_vs_plain"] = res["batched_serve"]["msamples_per_s"] / plain_msps
            res["films_identical_to_plain"] = f"{identical} of {len(stream_)}"
            res["max_request_error"] = float(max(errs))
            # ---- what this stream allows: every request's samples at the full-GPU path
            # rate of its scene and depth, and no request served before it arrives
            ideal = [w * h * spp / (full_rate_probe(ctx, sids[sc], cams[sc], scenes[sc], depth,
                                                    probe_film.data_ptr(), probe_stream, torch,
                                                    rate_cache) * 1e6)
                     for _, sc, w, h, spp, depth in stream_]
            span = stream_[-1][0] - stream_[0][0]
            best_makespan = max(sum(ideal), span + ideal[-1])
            res["attainable"] = {
                "plain_service_s": float(sum(service)), "full_rate_service_s": float(sum(ideal)),
                "arrival_span_s": float(span),
                "gpu_bound_speedup": float(sum(service) / sum(ideal)),
                "msamples_per_s_bound": samples / best_makespan / 1e6,
                "speedup_bound": samples / best_makespan / 1e6 / plain_msps,
                "method": "each request's samples at the plain path's rate on a whole-GPU wave "
                          "(2048x2048 x 32 spp, 2^27 paths) of its scene and depth; makespan >= "
                          "max(sum of those times, arrival span + the last request's time)"}
            out["rates"][str(int(rate))] = res
            del films
        # ---- per-request error against the oracle (the reference's estimator) on the
        # first requests of the stream small enough for the CPU: 8 GPU seeds against 3
        # decorrelated oracle replicates at the request's own resolution, spp and depth
        out["oracle_checks"] = serve_oracle_checks(ctx, sids, cams, scenes, rates[-1], count,
                                                   oracle_checks)
    finally:
        ctx.close()
    return out


def serve_oracle_checks(ctx, sids, cams, scenes, rate, count, n_checks):
    import dataclasses
    import numpy as np
    import oracle
    from petrichor_gb300 import capi, synth
    checks = []
    for k, (_, sc, w, h, spp, depth) in enumerate(synth.request_stream(int(rate), rate, count)):
        if len(checks) >= n_checks:
            break
        if w * h * spp > 1_000_000 or scenes[sc].num_triangles > 1_500_000:
            continue
        scene = scenes[sc].copy_with(settings=dataclasses.replace(
            scenes[sc].settings, width=w, height=h, spp=spp, max_bounces=depth))
        g = np.array([ctx.render(sids[sc], cams[sc], capi.settings_from_scene(
            scene, capi.MODE_WAVEFRONT, seed=500 + s)).mean() for s in range(8)])
        o = oracle.OracleScene(scene)
        d = np.array([o.render_decorrelated(31 + r)[0].mean() for r in range(3)])
        pooled = (((g - g.mean()) ** 2).sum() + ((d - d.mean()) ** 2).sum()) / (7 + 2)
        se = math.sqrt(pooled * (1 / 8 + 1 / 3))
        rel = abs(float(g.mean()) - float(d.mean())) / float(d.mean())
        checks.append({"request": k, "scene": int(sc), "resolution": [w, h], "spp": spp,
                       "max_bounces": depth, "rel": rel, "sigma_rel": se / float(d.mean()),
                       "pass": bool(rel <= 0.005 or rel <= 4.5 * se / float(d.mean()))})
    return checks


def run_serve(args):
    rates = [float(r) for r in (args.serve_rates or "20,100,500").split(",")]
    s = serve_summary(args, rates, args.requests)
    top = s["rates"][str(int(rates[-1]))]
    print(json.dumps({"metric": "serve_msamples_per_s", "value": top["batched_serve"]["msamples_per_s"],
                      "unit": UNIT, "n_gpus": 1, "higher_is_better": True, "scaling": "weak",
                      "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                      "config": s["config"], "p50_ms": top["batched_serve"]["p50_ms"],
                      "p99_ms": top["batched_serve"]["p99_ms"], "serve": s}))


def serve_object(s, rate):
    """The serve object of the default line: the top rate's numbers up front."""
    r = s["rates"][str(int(rate))]
    return {"rate_per_s": rate, "msamples_per_s": r["batched_serve"]["msamples_per_s"],
            "p50_ms": r["batched_serve"]["p50_ms"], "p99_ms": r["batched_serve"]["p99_ms"],
            "plain_msamples_per_s": r["plain"]["msamples_per_s"],
            "plain_p50_ms": r["plain"]["p50_ms"], "plain_p99_ms": r["plain"]["p99_ms"],
            "speedup_vs_plain": r["speedup_vs_plain"], "max_request_error": r["max_request_error"],
            "films_identical_to_plain": r["films_identical_to_plain"],
            "attainable": r["attainable"], "oracle_checks": s["oracle_checks"],
            "config": s["config"]}


# ------------------------------------------------------------------ stress scene, all forms
def run_stress_forms(args):
    """The memory-bound stress workload (20M triangles, 3840x2160, 256 spp, 12 bounces,
    8192x4096 sky) rendered four ways with the same samples: one plain render at 256 spp;
    four requests of 64 spp (seeds 1-4) through the serving loop, through one batched
    launch, and as four plain renders. Device time from CUDA events (serve: submission to
    the last completion, host clock)."""
    import torch
    from petrichor_gb300 import capi, synth
    t0 = time.perf_counter()
    scene = synth.terrain_rocks()
    gen_s = time.perf_counter() - t0
    st = scene.settings
    ctx = capi.Context(0)
    res = {}
    try:
        sid = ctx.upload(scene)
        cam = capi.camera_from_scene(scene)
        npx = st.width * st.height
        q = 4
        whole = capi.settings_from_scene(scene, capi.MODE_WAVEFRONT, seed=1)
        parts = [capi.settings_from_scene(scene, capi.MODE_WAVEFRONT, seed=k + 1, spp=st.spp // q)
                 for k in range(q)]
        films = [torch.empty(npx * 3, dtype=torch.float32, device="cuda") for _ in range(q)]
        stream = torch.cuda.Stream()
        samples = npx * st.spp

        def timed(fn):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            l0 = ctx.stats().kernel_launches
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            secs = e0.elapsed_time(e1) / 1e3
            return {"seconds": secs, "msamples_per_s": samples / secs / 1e6,
                    "gpu_launches": int(ctx.stats().kernel_launches - l0)}

        ctx.render_device(sid, cam, parts[0], films[0].data_ptr(), stream.cuda_stream)  # warm
        res["plain_whole_frame"] = timed(
            lambda: ctx.render_device(sid, cam, whole, films[0].data_ptr(), stream.cuda_stream))
        res["plain_4_requests"] = timed(lambda: [
            ctx.render_device(sid, cam, parts[k], films[k].data_ptr(), stream.cuda_stream)
            for k in range(q)])
        res["batched_4_requests"] = timed(lambda: ctx.batch_render(
            [(sid, cam, parts[k], films[k].data_ptr()) for k in range(q)], stream.cuda_stream))
        ctx.serve_start(wave_paths=args.wave_paths, max_active=64, state_budget=150 * 2 ** 30)
        torch.cuda.synchronize()
        rids = [ctx.serve_submit(sid, cam, parts[k], film_device=films[k].data_ptr())
                for k in range(q)]
        sts = [ctx.serve_wait(r, 600) for r in rids]
        secs = max(x.done_s for x in sts) - min(x.submit_s for x in sts)
        ctx.serve_stop()
        res["served_4_requests"] = {"seconds": secs, "msamples_per_s": samples / secs / 1e6,
                                    "completed": sum(x.state == capi.REQ_DONE for x in sts)}
        prof = ctx.render_profile(sid, cam, whole, films[0].data_ptr(), count_reference=False).as_dict()
        ctx.release(sid)
    finally:
        ctx.close()
    base = res["plain_whole_frame"]["msamples_per_s"]
    for k in ("plain_4_requests", "batched_4_requests", "served_4_requests"):
        res[k]["vs_plain_whole_frame"] = res[k]["msamples_per_s"] / base
    print(json.dumps({"metric": "stress_forms_msamples_per_s", "unit": UNIT, "n_gpus": 1,
                      "higher_is_better": True, "dtype": "f32", "data": "synthetic",
                      "config": {"workload": STRESS_WORKLOAD, "triangles": scene.num_triangles,
                                 "resolution": [st.width, st.height], "spp": st.spp,
                                 "max_bounces": st.max_bounces, "requests": q,
                                 "scene_gen_s": round(gen_s, 1)},
                      "forms": res,
                      "stage_ms_whole_frame": {k: prof[k] for k in
                                               ("raygen_ms", "extend_ms", "shade_ms", "shadow_ms",
                                                "accumulate_ms")}}))


# ------------------------------------------------------------------ plain path (default)
def main():
    args = parse()
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.batch:
        return run_batch(args)
    if args.serve:
        return run_serve(args)
    if args.stress_forms:
        return run_stress_forms(args)
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
    tuning = {k: int(v) for k, v in (kv.split("=") for kv in args.tuning.split(",") if kv)}
    if args.trace_primary:
        tuning["primary_traversal"] = 1
    if tuning:
        ctx.set_tuning(**tuning)
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
    stages = {k: prof2[k] for k in ("raygen_ms", "extend_ms", "raster_ms", "shade_ms", "shadow_ms",
                                     "accumulate_ms")}
    dominant = max(stages, key=stages.get)
    # extension rays of the first four bounces (renders cut after bounce b, differenced):
    # the units behind one ExtendKernel launch of a profiler capture; bounce 0 counted in
    # the reference's traversal order too (its rays are rasterised, not traced)
    rays_per_bounce, prev, prof0 = [], 0, None
    for b in range(4):
        sb = capi.settings_from_scene(scene, capi.MODE_WAVEFRONT, seed=replicas.replica_seed(1, rank),
                                      env_sampling=env, max_bounces=b)
        n = ctx.render_profile(sid, cam, sb, film.data_ptr(), count_reference=(b == 0)).as_dict()
        if b == 0:
            prof0 = n
        rays_per_bounce.append(int(n["extend_rays"] - prev))
        prev = n["extend_rays"]
    # ExtendKernel alone: the rays it traces (every extension ray but the rasterised
    # first-bounce ones) over its own time (the raster kernels are timed apart).
    # Algorithmic bytes of a traced ray (reference traversal order): 32 B per node popped
    # and slab-tested, 48 B per triangle test, 32 B ray in, 16 B hit out
    share0 = prof2["raster_paths"] / max(1, prof0["ref_rays"])  # of bounce 0 rasterised
    nodes = prof["ref_node_tests"] - share0 * prof0["ref_node_tests"]
    tris = prof["ref_tri_tests"] - share0 * prof0["ref_tri_tests"]
    traced = max(1, prof2["extend_rays"] - prof2["raster_paths"])
    bytes_per_ray = (32.0 * nodes + 48.0 * tris) / traced + 48.0
    ext_launches = max(1, prof2["extend_launches"])
    busy_launches = ext_launches - (1 if prof2["raster_paths"] >= prof0["ref_rays"] > 0 else 0)
    bytes_per_launch = bytes_per_ray * traced / ext_launches
    avg_launch_s = prof2["extend_ms"] / 1e3 / ext_launches
    achieved = bytes_per_launch / avg_launch_s / 1e9
    peaks_path = os.path.join(HERE, "MEASURED_PEAKS.json")
    peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        with open(peaks_path) as fh:
            peak, peak_src = float(json.load(fh)["hbm_gbs"]), "measured"
    l2 = l2_read_peak(ctx)
    # single-kernel ncu counters of ExtendKernel on the same scene at 1920x1080 and 2 / 4
    # spp: DRAM bytes = fixed part per launch + bytes per ray, SIMT efficiency, issue use
    cnt = counters_profile("extend_kernel_counters_spheres_grids_1M_1080p_2_4spp.json") \
        if workload_name(args) == WORKLOAD else None
    traffic = None
    if cnt is not None:
        traffic = (cnt["dram_bytes_per_ray"] * traced +
                   cnt["dram_bytes_fixed_per_launch"] * busy_launches) / ext_launches
    raster_stage = None
    if prof2["raster_paths"] > 0:
        raster_stage = {"kernels": "RasterSetupKernel, RasterVisitKernel, RasterFinishKernel",
                        "ms": prof2["raster_ms"], "paths": prof2["raster_paths"],
                        "mpaths_per_s": prof2["raster_paths"] / (prof2["raster_ms"] / 1e3) / 1e6}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": secs / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(args, scene, world),
        "setup": {"bvh_nodes": info.num_nodes, "mode": "wavefront",
                  "resident_bytes": int(info.device_bytes),
                  "scene_gen_s": round(gen_s, 2), "scene_upload_s": round(upload_s, 2),
                  "bvh_build_s": round(info.build_seconds, 2), "tuning": tuning or "default"},
        "e2e": {"value": e2e, "unit": UNIT,
                "h2d_bytes_per_step": 64 + 48, "d2h_bytes_per_step": npx * 12,
                "path": "pt_render (C ABI) with the scene resident, film into pinned host memory"},
        "gpu_launches": int(launches),
        "clocks": clocks.summary(),
        "roofline": {"bound": "issue/latency", "kernel": "ExtendKernel (closest-hit traversal)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "frac_hbm": achieved / peak,
                     "frac_l2": achieved / l2["gbs"], "l2_peak": l2["gbs"],
                     "l2_peak_method": l2["method"], "traffic": traffic, "peak_source": peak_src,
                     "simt_eff": cnt.get("simt_eff") if cnt else None,
                     "issue_active": cnt.get("issue_active") if cnt else None,
                     "counters_source": cnt.get("source") if cnt else None,
                     "note": "achieved = algorithmic bytes of the rays ExtendKernel traces "
                             "(reference traversal order) / ExtendKernel time; served mostly "
                             "from L1/L2, so the limiter is issue rate at the stated SIMT "
                             "efficiency, not DRAM; traffic = the counters' DRAM model at this "
                             "frame's rays per launch",
                     "bytes_per_ray": bytes_per_ray,
                     "traced_rays": int(traced),
                     "ref_nodes_per_ray": nodes / traced,
                     "ref_tris_per_ray": tris / traced,
                     "raster_stage": raster_stage,
                     "dominant_stage": dominant, "stage_ms": stages,
                     "rays_extended": prof2["extend_rays"], "shadow_rays": prof2["shadow_rays"],
                     "rays_per_bounce_0_3": rays_per_bounce,
                     "mrays_per_s": (prof2["extend_rays"] + prof2["shadow_rays"]) /
                                    (sum(stages.values()) / 1e3) / 1e6},
        "image_mean": img_mean,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        base, o, cpu_film, cpu_tiles, per_tile_s, order = cpu_baseline(scene, args.cpu_seconds)
        line["cpu_baseline"] = base
        if not args.plain_only:
            line["image_error"] = image_error(ctx, sid, cam, sets, scene, film, stream, o, cpu_film,
                                              cpu_tiles, order, per_tile_s, args.err_seconds, torch)
        del o
    ctx.release(sid)
    ctx.close()
    del film
    torch.cuda.empty_cache()
    if rank == 0 and world == 1 and not args.plain_only:
        line["e2e_dropin"] = e2e_dropin(scene, args.steps)
        if not args.small and not args.stress:
            # the plain line stands on its own: a failure of a form is recorded in its
            # object and on stderr, not allowed to swallow the line
            rate = float((args.serve_rates or "500").split(",")[-1])
            try:
                line["serve"] = serve_object(serve_summary(args, [rate], args.requests), rate)
            except Exception as e:  # noqa: BLE001
                line["serve"] = {"error": f"{type(e).__name__}: {e}"}
                print(f"serve form failed: {line['serve']['error']}", file=sys.stderr)
            torch.cuda.empty_cache()
            try:
                line["batch"] = batch_summary(args, steps=1, warmup=1)
            except Exception as e:  # noqa: BLE001
                line["batch"] = {"error": f"{type(e).__name__}: {e}"}
                print(f"batch form failed: {line['batch']['error']}", file=sys.stderr)
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
