"""Benchmark of the GB300 raster backend on the single-large-scene workload:
a 2048x2048 premultiplied RGBA8 canvas cleared to white, 20,000 seeded
synthetic paths of 3-64 verbs (50% lines / 25% quads / 25% cubics,
coordinates uniform in [-64, 2112]^2), 30% even-odd, 50% solid / 25% linear
/ 25% radial gradients, 20% stroked (width 1-8, all caps and joins), one
DrawPath per path, one Flush (skity_gb300.scene.config2).

One step = rendering the whole scene (every DrawPath + Flush).
  value: paths/s with the scene resident in device memory (CUDA events
         around each render on the library's stream), summed over ranks;
  e2e:   the same through skity_cuda_render_streams with host buffers: the
         scene stream uploaded and the pixels read back inside every step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

Multi-GPU: every rank renders its own replica (independent canvases, no
collective on the data path); the timing is the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = ("Mpix/s & paths/s, batched vs per-draw GPU vs CPU, ≤1 LSB; p50/p99 ms")
WORKLOAD = ("config2: 2048x2048 RGBA8 canvas, 20,000 seeded paths (3-64 verbs line/quad/cubic, "
            "coords U[-64,2112]^2, 30% even-odd, 25% linear + 25% radial gradients 2-8 stops, "
            "20% stroked w U[1,8] all caps x joins), one DrawPath per path, one Flush")


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def measured_peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = os.path.join("/tmp", f"skity_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx.append(float(f[2]))
                except ValueError:
                    continue
                for n, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
            os.unlink(self.path)
        except Exception:
            pass
        loaded = [s for s in sm if s > 0.5 * (max(mx) if mx else 0)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


# Integer ops per fragment, counted from the reference's formulas: coverage
# AlphaMulQ 9 + PMSrcOver 14 (color_priv.hpp:62-72) for every fragment; a
# linear gradient adds the mapping 4, stop search and lerp ~26, Color4fToColor
# 16 and premultiply 18 (sw_span_brush.cc:239-320, color.cc:53-59,
# color_priv.hpp:47-58); radial adds the second coordinate and the length 8;
# the blur composite's image brush adds the mapping and a nearest sample 12.
OPS_PER_FRAGMENT = (23, 93, 101, 35)  # solid, linear, radial, image


def issue_roofline(st, frame_ms, composite_ms, clk):
    """Fragment work against the int32 issue peak (152 SMs x 128 lanes x the
    SM clock sampled during the timed region): over the whole frame and over
    the compositing stage, where the fragments are shaded and blended."""
    frags = st.get("fragments_by_brush") or [st["fragments"], 0, 0, 0]
    ops = sum(o * f for o, f in zip(OPS_PER_FRAGMENT, frags))
    mhz = clk.get("sm_mhz") or 2070.0
    peak = 152 * 128 * mhz * 1e6
    return {"ops_per_frame": ops, "peak_ops_per_s": peak, "sm_mhz": mhz,
            "frac_frame": ops / (frame_ms / 1e3) / peak if frame_ms else None,
            "frac_composite": ops / (composite_ms / 1e3) / peak if composite_ms else None,
            "fragments_by_brush": dict(zip(("solid", "linear", "radial", "image"), frags))}


def load_scene():
    from skity_gb300 import scene as S
    cache = os.path.join("/tmp", "skity_config2_v1.bin")
    try:
        with open(cache, "rb") as f:
            return S.Scene.from_bytes(f.read())
    except Exception:
        sc = S.config2()
        try:
            with open(cache, "wb") as f:
                f.write(sc.to_bytes())
        except Exception:
            pass
        return sc


def load_config3():
    from skity_gb300 import scene as S
    cache = os.path.join("/tmp", "skity_config3_v1.bin")
    try:
        with open(cache, "rb") as f:
            buf = f.read()
        scenes, o = [], 0
        while o < len(buf):
            n = int.from_bytes(buf[o:o + 8], "little")
            scenes.append(S.Scene.from_bytes(buf[o + 8:o + 8 + n]))
            o += 8 + n
        if len(scenes) == 256:
            return scenes
    except Exception:
        pass
    scenes = S.config3()
    try:
        with open(cache, "wb") as f:
            for sc in scenes:
                b = sc.to_bytes()
                f.write(len(b).to_bytes(8, "little") + b)
    except Exception:
        pass
    return scenes


def batch_forms(ctx, steps: int, warmup: int, sample: int, cpu_sample: int = 64):
    """The 256-canvas batching workload (log-uniform sides in [64,1024],
    log-uniform 50-2,000 paths each, drawn as in the 512x512 scene) in three
    forms: the batched form (one planned batch, re-rendered by CUDA graph
    replay), the plain per-draw form (one launch sequence per DrawPath onto a
    device canvas, skity_cuda_draw_path_static) on the first `sample`
    canvases, and the CPU oracle on all host cores over the first
    `cpu_sample` canvases, dealt largest first to a pool of one thread per
    core (each thread takes the next canvas when it finishes one), so that
    every core stays busy to the end.  The per-draw result is compared with
    the batched one on its sample."""
    import numpy as np
    import torch
    from concurrent.futures import ThreadPoolExecutor
    from oracle import oracle
    from skity_gb300.canvas import Batch, DeviceCanvas

    scenes = load_config3()
    pix = sum(sc.width * sc.height for sc in scenes)
    paths = sum(sc.n_draws for sc in scenes)
    batch = Batch(ctx, scenes)
    from skity_gb300 import autotune
    tuned = autotune.tune(batch, autotune.signature(scenes, "GB300"), reps=2)
    for _ in range(max(warmup, 1)):
        batch.render()
    ms = []
    for _ in range(steps):
        st = batch.render()
        ms.append(st["device_ms"])
    bms = statistics.mean(ms)
    stage = {k: st[k] for k in ("geometry_ms", "sweep_emit_ms", "composite_ms", "blur_ms")}
    out = {"workload": "256 canvases, sides log-uniform [64,1024], 50-2,000 paths each "
                       "(3-32 verbs line/quad/cubic, nonzero, solid colours)",
           "canvases": len(scenes), "paths": paths, "mpix": pix / 1e6,
           "batched": {"ms": bms, "mpix_per_s": pix / 1e3 / bms, "paths_per_s": paths * 1e3 / bms,
                       "graph_replays": int(st["graph_replays"]), "stage_ms": stage,
                       "raster_config": tuned["config"], "autotune_cached": tuned["cached"],
                       "autotune_trials": len(tuned.get("trials", [])),
                       "spans": st["spans"], "fragments": st["fragments"],
                       "form": "one planned batch, "
                       "CUDA-graph replay (geometry, sweeps, composites)"}}
    # per-draw form on a sample of canvases
    sub = scenes[:sample]
    spix = sum(sc.width * sc.height for sc in sub)
    spaths = sum(sc.n_draws for sc in sub)
    stream = torch.cuda.current_stream()
    canv = [torch.full((sc.height, sc.width, 4), 255, dtype=torch.uint8, device="cuda")
            for sc in sub]
    dcs = [DeviceCanvas(c.data_ptr(), sc.width, sc.height, device=torch.cuda.current_device(),
                        stream=stream.cuda_stream) for c, sc in zip(canv, sub)]
    dcs[0].draw_scene(sub[0].subset(0, 8))  # first call: one-time set-up
    for c in canv:
        c.fill_(255)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for dc, sc in zip(dcs, sub):
        dc.draw_scene(sc)
    torch.cuda.synchronize()
    pd_s = time.perf_counter() - t0
    exact = all(np.array_equal(c.cpu().numpy(), batch.read(i)) for i, c in enumerate(canv))
    out["per_draw"] = {"ms_per_canvas": 1e3 * pd_s / len(sub), "mpix_per_s": spix / 1e6 / pd_s,
                       "paths_per_s": spaths / pd_s, "sample": f"first {len(sub)} canvases, "
                       f"{spaths} paths", "matches_batched": exact,
                       "form": "skity_cuda_draw_path_static per DrawPath on a device canvas"}
    # CPU oracle on all host cores: a pool of one thread per core, canvases
    # dealt largest first (paths x rows), each thread taking the next canvas
    threads = os.cpu_count() or 1
    oracle.build()
    csub = sorted(scenes[:cpu_sample], key=lambda sc: -sc.n_draws * sc.height)
    cpix = sum(sc.width * sc.height for sc in csub)
    cpaths = sum(sc.n_draws for sc in csub)

    def one(sc):
        t = time.perf_counter()
        oracle.render(sc)
        return time.perf_counter() - t

    t0 = time.perf_counter()
    with ThreadPoolExecutor(threads) as ex:
        busy = sum(ex.map(one, csub))
    cpu_s = time.perf_counter() - t0
    out["cpu"] = {"mpix_per_s": cpix / 1e6 / cpu_s, "paths_per_s": cpaths / cpu_s, "cores": threads,
                  "kind": "port", "seconds": cpu_s, "core_busy": busy / (threads * cpu_s),
                  "sample": f"first {len(csub)} canvases ({cpaths} paths), largest first on a "
                            f"{threads}-thread pool"}
    out["batched_over_per_draw"] = out["batched"]["paths_per_s"] / out["per_draw"]["paths_per_s"]
    out["batched_over_cpu"] = out["batched"]["paths_per_s"] / out["cpu"]["paths_per_s"]
    batch.close()
    return out


def serving_pool(n: int = 64):
    """Request scenes of the serving workload: one canvas each, sides
    log-uniform in [128, 2048], log-uniform 10-5,000 paths drawn as in the
    512x512 scene; arrivals cycle through this seeded pool."""
    from skity_gb300 import scene as S
    cache = os.path.join("/tmp", f"skity_serving_pool_v1_{n}.bin")
    try:
        with open(cache, "rb") as f:
            buf = f.read()
        out, o = [], 0
        while o < len(buf):
            k = int.from_bytes(buf[o:o + 8], "little")
            out.append(buf[o + 8:o + 8 + k])
            o += 8 + k
        if len(out) == n:
            return out
    except Exception:
        pass
    R = S.random_streams(S.SEED_BASE + 5, n, 4)
    out = []
    for i in range(n):
        w = int(round(float(S.loguniform(R[i, 0], 128, 2048))))
        h = int(round(float(S.loguniform(R[i, 1], 128, 2048))))
        k = max(1, int(round(float(S.loguniform(R[i, 2], 10, 5000)))))
        out.append(S.random_paths_scene(int(R[i, 3]), w, h, k, 3, 32).to_bytes())
    try:
        with open(cache, "wb") as f:
            for b in out:
                f.write(len(b).to_bytes(8, "little") + b)
    except Exception:
        pass
    return out


def serving(ctx, rates, seconds: float, device: int, max_outstanding: int = 512):
    """Poisson request streams against the serving loop: for each rate,
    arrivals for `seconds` seconds (seeded exponential gaps), requests
    drawn in turn from the pool; latency = submit -> pixels on the host.
    Clients give up on an arrival while `max_outstanding` requests are
    already waiting (counted as shed), which bounds the drain of a rate
    beyond capacity.  Beside them, the offline batched form on the pool."""
    import random
    import threading
    from skity_gb300 import scene as S
    from skity_gb300.canvas import Batch, Server

    pool = serving_pool()
    scenes = [S.Scene.from_bytes(b) for b in pool]
    paths = [sc.n_draws for sc in scenes]
    off = Batch(ctx, scenes)
    off.render()
    st = off.render()
    off.close()
    offline = {"paths_per_s": sum(paths) * 1e3 / st["device_ms"],
               "requests_per_s": len(pool) * 1e3 / st["device_ms"], "ms": st["device_ms"]}
    results = []
    for rate in rates:
        srv = Server(device, workers=2, max_batch=64)
        rng = random.Random(0x5EED0005 + int(rate))
        tickets = []
        lock = threading.Lock()
        done = threading.Event()
        shed = [0]
        waited = [0]

        def submitter():
            t0 = time.perf_counter()
            t_next, i = 0.0, 0
            while t_next < seconds:
                now = time.perf_counter() - t0
                if now < t_next:
                    time.sleep(min(t_next - now, 0.002))
                    continue
                k = i % len(pool)
                with lock:
                    outstanding = len(tickets) - waited[0]
                if outstanding >= max_outstanding:
                    shed[0] += 1
                else:
                    tk = srv.submit(stream=pool[k])
                    with lock:
                        tickets.append((tk, k))
                i += 1
                t_next += rng.expovariate(rate)
            done.set()

        lat, queue_ms, sizes, npaths = [], [], [], 0
        t_start = time.perf_counter()
        th = threading.Thread(target=submitter)
        th.start()
        j = 0
        while True:
            with lock:
                have = len(tickets)
            if j >= have:
                if done.is_set():
                    with lock:
                        if j >= len(tickets):
                            break
                time.sleep(0.0005)
                continue
            tk, k = tickets[j]
            _, info = srv.wait(tk, 600000, want_pixels=False)
            lat.append(info["latency_ms"])
            queue_ms.append(info["queue_ms"])
            sizes.append(info["batch_size"])
            npaths += paths[k]
            j += 1
            with lock:
                waited[0] = j
        wall = time.perf_counter() - t_start
        th.join()
        srv.close()
        lat.sort()
        q = lambda f: lat[min(len(lat) - 1, int(f * len(lat)))]
        results.append({"rate_rps": rate, "seconds": seconds, "requests": len(lat),
                        "shed": shed[0], "max_outstanding": max_outstanding,
                        "achieved_rps": len(lat) / wall, "paths_per_s": npaths / wall,
                        "p50_ms": q(0.50), "p99_ms": q(0.99), "max_ms": lat[-1],
                        "mean_queue_ms": statistics.mean(queue_ms),
                        "mean_batch": statistics.mean(sizes),
                        "vs_offline_paths": (npaths / wall) / offline["paths_per_s"]})
    return {"workload": "Poisson arrivals; requests cycle through 64 seeded canvases (sides "
                        "log-uniform [128,2048], 10-5,000 paths, solid fills); admission budget "
                        "40 GiB; 2 workers, up to 64 requests per batch",
            "offline_batched": offline, "rates": results}


def load_config4():
    from skity_gb300 import scene as S
    cache = os.path.join("/tmp", "skity_config4_v1.bin")
    try:
        with open(cache, "rb") as f:
            return S.Scene.from_bytes(f.read())
    except Exception:
        sc = S.config4()
        try:
            with open(cache, "wb") as f:
                f.write(sc.to_bytes())
        except Exception:
            pass
        return sc


def other_workloads(ctx, steps: int):
    """The 512x512 scene (1,000 fills) and the glyph-dense scene (4096x4096,
    100,000 small even-odd outlines, a tenth with a kNormal blur): resident
    batch renders (CUDA-graph replays) against the CPU oracle on one core
    over the whole scene (a single canvas has no parallelism in the
    reference)."""
    from oracle import oracle
    from skity_gb300 import scene as S
    from skity_gb300.canvas import Batch
    out = {}
    for name, sc, desc in [
            ("config1", S.config1(), "512x512, 1,000 fills of 3-32 verbs, nonzero, solid"),
            ("config4", load_config4(), "4096x4096, 100,000 outlines (1-3 contours, 8-48 px), "
                                        "even-odd, 10% kNormal blur sigma 2-20")]:
        b = Batch(ctx, [sc])
        for _ in range(3):
            b.render()
        ms = [b.render()["device_ms"] for _ in range(steps)]
        st = ctx.stats()
        b.close()
        gms = statistics.mean(ms)
        _, cst = oracle.render(sc)
        px = sc.width * sc.height
        out[name] = {"workload": desc, "paths": sc.n_draws,
                     "gpu": {"ms": gms, "paths_per_s": sc.n_draws * 1e3 / gms,
                             "mpix_per_s": px / 1e3 / gms,
                             "stage_ms": {k: st[k] for k in ("geometry_ms", "sweep_emit_ms",
                                                             "composite_ms", "blur_ms")}},
                     "cpu": {"s": cst.seconds, "paths_per_s": sc.n_draws / cst.seconds,
                             "cores": 1, "kind": "port", "sample": "whole scene"},
                     "gpu_over_cpu": (sc.n_draws * 1e3 / gms) / (sc.n_draws / cst.seconds)}
    return out


def cpu_baseline(scene, threads: int, sample_paths: int, steps: int = 1):
    """The oracle (CPU restatement of the reference path) on the first
    `sample_paths` draws; paths/s over `steps` repetitions."""
    from oracle import oracle
    oracle.build()
    secs = []
    for _ in range(steps):
        if threads == 1:
            _, st = oracle.render(scene, 0, sample_paths)
        else:
            _, st = oracle.render_mt(scene, threads, 0, sample_paths)
        secs.append(st.seconds)
    return sample_paths / statistics.mean(secs), secs


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    scene = load_scene()
    threads = os.cpu_count() or 1
    sample = args.ref_sample_paths
    # warm-up (untimed), then timed steps, each a bounded sample of the scene
    for _ in range(args.warmup):
        cpu_baseline(scene, threads, min(sample, 50))
    value, secs = cpu_baseline(scene, threads, sample, steps=args.steps)
    line = {
        "metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(secs) * scene.n_draws / sample,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8/int32/f32",
        "data": "synthetic (seeded)", "impl": "reference",
        "config": {"workload": WORKLOAD, "canvas": "2048x2048", "paths": scene.n_draws},
        "cpu_baseline": {"value": value, "unit": "paths/s", "cores": threads, "kind": "port",
                         "sample": f"first {sample} of {scene.n_draws} paths per step, banded rows "
                                   f"on {threads} threads (identical pixels)"},
        "e2e": {"value": value, "unit": "paths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_gpu(args, rank, world, local):
    import torch
    import torch.distributed as dist
    torch.cuda.set_device(local)
    if world > 1 and not dist.is_initialized():
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from skity_gb300.canvas import Batch, Context

    scene = load_scene()
    if args.paths:
        scene = scene.subset(0, args.paths)
    ctx = Context(local)
    batch = Batch(ctx, [scene])
    flush_buf = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB L2

    for _ in range(max(args.warmup, 1)):
        batch.render()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    step_ms, stages = [], []
    t0 = time.perf_counter()
    for k in range(args.steps):
        flush_buf.fill_(k & 0xFF)
        torch.cuda.synchronize()
        st = batch.render()
        step_ms.append(st["device_ms"])
        stages.append(st)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    if world > 1:
        dist.barrier()
    clk = clocks.stop()
    total_ms = torch.tensor([sum(step_ms)], dtype=torch.float64, device="cuda")
    if world > 1:
        dist.all_reduce(total_ms, op=dist.ReduceOp.MAX)
    ms_per_step = total_ms.item() / args.steps
    paths = scene.n_draws
    value = world * paths / (ms_per_step / 1e3)
    mpix = world * scene.width * scene.height / (ms_per_step / 1e3) / 1e6
    last = stages[-1]

    # end to end through the C ABI with host buffers (upload + render + readback)
    e2e_ms = []
    if not args.no_e2e:
        ctx.render_streams([scene])  # warm
        for _ in range(max(1, min(args.steps, 3))):
            ctx.render_streams([scene])
            e2e_ms.append(ctx.stats()["total_ms"])
    e2e_ms_mean = statistics.mean(e2e_ms) if e2e_ms else None

    # roofline of the dominant stage
    stage_ms = {k: statistics.mean(s[k] for s in stages)
                for k in ("geometry_ms", "sweep_count_ms", "sweep_emit_ms", "composite_ms", "blur_ms")}
    dom = max(stage_ms, key=stage_ms.get)
    peak, peak_kind = measured_peaks()
    spans, frags, pixels, edges = last["spans"], last["fragments"], last["pixels"], last["edges"]
    # algorithmic bytes per launch of each stage (measurement section)
    alg = {
        "composite_ms": spans * 8 + pixels * 4 * 2 + last["passes"] * 24,
        "sweep_emit_ms": spans * 8 + edges * 84 * 2,
        "sweep_count_ms": edges * 84 * 2,
        "geometry_ms": edges * 84 * 2,
        "blur_ms": 0,
    }[dom]
    achieved = alg / (stage_ms[dom] / 1e3) / 1e9 if stage_ms[dom] > 0 else 0.0
    line = {
        "metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8/int32/f32",
        "data": "synthetic (seeded, skity_gb300.scene.config2)",
        "config": {"workload": WORKLOAD, "canvas": "2048x2048", "paths": paths,
                   "l2": "flushed between steps (256 MiB device write)",
                   "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"},
        "mpix_per_s": mpix,
        "stage_ms": stage_ms,
        "work": {"passes": last["passes"], "edges": edges, "spans": spans, "fragments": frags,
                 "fragments_per_s": world * frags / (ms_per_step / 1e3)},
        "gpu_launches": int(sum(s["kernel_launches"] for s in stages)),
        "clocks": clk,
        "roofline": {"kernel": dom.replace("_ms", ""), "bound": "hbm", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak if peak else None,
                     "peak_source": peak_kind, "traffic": None},
        "issue_roofline": issue_roofline(last, ms_per_step, stage_ms["composite_ms"], clk),
        "e2e": {"value": (world * paths / (e2e_ms_mean / 1e3)) if e2e_ms_mean else None,
                "unit": "paths/s", "h2d_bytes_per_step": len(scene.to_bytes()),
                "d2h_bytes_per_step": scene.width * scene.height * 4,
                "ms_per_step": e2e_ms_mean},
        "wall_s": wall,
    }
    if rank == 0 and not args.no_others:
        line["other_workloads"] = other_workloads(ctx, max(1, min(args.steps, 5)))
    if rank == 0 and args.serve_seconds > 0:
        line["serving"] = serving(ctx, [float(r) for r in args.serve_rates.split(",")],
                                  args.serve_seconds, local)
    if rank == 0 and not args.no_forms:
        line["batching"] = batch_forms(ctx, max(1, min(args.steps, 5)), 3, args.per_draw_sample)
    if rank == 0 and not args.no_cpu:
        v, secs = cpu_baseline(scene, 1, args.cpu_sample_paths)
        line["cpu_baseline"] = {"value": v, "unit": "paths/s", "cores": 1, "kind": "port",
                                "sample": f"first {args.cpu_sample_paths} of {paths} paths, "
                                          f"{secs[0]:.1f} s single-threaded"}
    batch.close()
    ctx.close()
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--cpu-sample-paths", type=int, default=400)
    ap.add_argument("--ref-sample-paths", type=int, default=800)
    ap.add_argument("--paths", type=int, default=0,
                    help="render only the first N paths of the scene (small profiling case)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the 256-canvas batched / per-draw / CPU comparison")
    ap.add_argument("--per-draw-sample", type=int, default=16)
    ap.add_argument("--no-others", action="store_true",
                    help="skip the 512x512 and glyph-dense scenes")
    ap.add_argument("--serve-rates", default="200,1000,5000",
                    help="Poisson request rates (requests/s) of the serving runs")
    ap.add_argument("--serve-seconds", type=float, default=5.0,
                    help="arrival window per rate (the serving workload specifies 60 s); 0 skips")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    from skity_gb300 import build
    build.build()
    return run_gpu(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
