"""Benchmark of the GB300 raster backend on the batching workload: 256
independent canvases with log-uniform sides in [64, 1024] px (non-square),
each cleared to white with a log-uniform 50-2,000 seeded paths of 3-32
verbs (50% lines / 25% quads / 25% cubics, control points uniform over the
canvas, nonzero fill, solid colours with alpha in [0.3, 1]), one DrawPath per
path and one Flush per canvas (skity_gb300.scene.config3).

One step = rendering all 256 canvases.
  value: paths/s of the batched form with the batch resident in device
         memory (its planned launches replayed from CUDA graphs; CUDA events
         around each render on the library's stream), summed over ranks;
  e2e:   the same through skity_cuda_render_streams with host buffers: the
         scene streams uploaded, planned and rendered, and every canvas read
         back inside every step;
  per_draw: the plain per-draw form of the same canvases (every DrawPath
         rasterised and blended on its own, skity_cuda_batch_render_per_draw);
  parity: the pixels of the last timed render against the oracle (the CPU
         restatement of the reference's software backend), every canvas;
  cpu_baseline: that oracle run, timed on all host cores (a pool of one
         thread per core, canvases dealt largest first).
The other workloads (the 512x512 and 2048x2048 scenes, the glyph-dense
4096x4096 scene with blur) and the serving runs are reported beside it, each
checked against the oracle's committed pixel digests.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

Multi-GPU: every rank renders its own replica (independent canvases, no
collective on the data path); the timing is the max over ranks.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import statistics
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "Mpix/s & paths/s, batched vs per-draw GPU vs CPU, ≤1 LSB; p50/p99 ms"
WORKLOAD = ("256 canvases, sides log-uniform [64,1024] px, 50-2,000 seeded paths each (3-32 verbs "
            "line/quad/cubic, nonzero, solid colours, alpha U[0.3,1]), one DrawPath per path, "
            "one Flush per canvas")
TOL_LSB, MIN_EXACT = 1, 0.999


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def bench_config(scenes, world: int) -> dict:
    """The `config` of both arms' lines (identical by construction)."""
    return {"workload": WORKLOAD, "canvases": len(scenes),
            "paths": sum(sc.n_draws for sc in scenes),
            "mpix": round(sum(sc.width * sc.height for sc in scenes) / 1e6, 3),
            "l2": "flushed between GPU steps (256 MiB device write)",
            "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"}


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


def issue_roofline(st, frame_ms, composite_ms, clk, sms):
    """Fragment work against the int32 issue peak (SMs x 128 lanes x the SM
    clock sampled during the timed region): over the whole frame and over the
    compositing stage, where the fragments are shaded and blended."""
    frags = st.get("fragments_by_brush") or [st["fragments"], 0, 0, 0]
    ops = sum(o * f for o, f in zip(OPS_PER_FRAGMENT, frags))
    mhz = clk.get("sm_mhz") or 2070.0
    peak = sms * 128 * mhz * 1e6
    return {"ops_per_frame": ops, "peak_ops_per_s": peak, "sm_mhz": mhz, "sms": sms,
            "frac_frame": ops / (frame_ms / 1e3) / peak if frame_ms else None,
            "frac_composite": ops / (composite_ms / 1e3) / peak if composite_ms else None,
            "fragments_by_brush": dict(zip(("solid", "linear", "radial", "image"), frags))}


# The sweep stage's counters per emitted span, from an ncu capture of the
# 256-canvas workload's first 64 canvases (profiles/k_sweep_reg_config3_64canvases.md):
# warp instructions executed and DRAM bytes (read + write) of the five sweep
# launches of one render (17.440 G instructions, 1.854 GB) over the
# 165,827,810 spans they emit.  Multiplied by the spans of the timed render
# (the units one launch processes) they give the per-render figures.
SWEEP_PER_SPAN = {"warp_inst": 105.17, "dram_bytes": 11.18}


def sweep_roofline(st, sweep_ms, clk, sms, hbm_peak, hbm_kind):
    """Roofline of the dominant kernel, the AAA sweep.  It is neither
    HBM- nor tensor-bound: one warp per path walks the path's rows in order,
    so its bound is instruction issue (SMs x 4 schedulers x 1 warp
    instruction per cycle at the sampled SM clock).  achieved = the sweep's
    warp instructions per render (ncu count per span x the render's spans)
    / the sweep stage's CUDA-event time; traffic = its DRAM bytes per render
    (ncu, scaled the same way).  Beside it, the HBM view: the sweep's
    algorithmic bytes (84-byte edges read and written, 8-byte spans
    written) over the same time against the measured copy bandwidth."""
    mhz = clk.get("sm_mhz") or 2070.0
    spans, edges = st["spans"], st["edges"]
    alg = spans * 8 + edges * 84 * 2
    hbm = {"algorithmic_bytes": alg, "achieved_gbs": alg / (sweep_ms / 1e3) / 1e9,
           "peak_gbs": hbm_peak, "peak_source": hbm_kind}
    hbm["frac"] = hbm["achieved_gbs"] / hbm_peak
    out = {"kernel": "sweep (k_sweep_reg<32/64/128>, k_sweep, k_sweep_retry)", "sweep_ms": sweep_ms, "hbm": hbm}
    if SWEEP_PER_SPAN["warp_inst"]:
        inst = SWEEP_PER_SPAN["warp_inst"] * spans
        peak = sms * 4 * mhz * 1e6 / 1e9
        ach = inst / (sweep_ms / 1e3) / 1e9
        out.update({"bound": "issue", "achieved": ach, "peak": peak, "unit": "Gwarp-inst/s",
                    "frac": ach / peak, "peak_source": f"{sms} SMs x 4 issue slots x {mhz:.0f} MHz",
                    "traffic": SWEEP_PER_SPAN["dram_bytes"] * spans
                    if SWEEP_PER_SPAN["dram_bytes"] else None})
    else:
        out.update({"bound": "hbm", "achieved": hbm["achieved_gbs"], "peak": hbm_peak,
                    "unit": "GB/s", "frac": hbm["frac"], "peak_source": hbm_kind, "traffic": None})
    return out


def _cached_scenes(name, make):
    from skity_gb300 import scene as S
    cache = os.path.join("/tmp", f"skity_{name}_v1.bin")
    try:
        with open(cache, "rb") as f:
            buf = f.read()
        scenes, o = [], 0
        while o < len(buf):
            n = int.from_bytes(buf[o:o + 8], "little")
            scenes.append(S.Scene.from_bytes(buf[o + 8:o + 8 + n]))
            o += 8 + n
        if scenes:
            return scenes
    except Exception:
        pass
    scenes = make()
    try:
        with open(cache, "wb") as f:
            for sc in scenes:
                b = sc.to_bytes()
                f.write(len(b).to_bytes(8, "little") + b)
    except Exception:
        pass
    return scenes


def load_config3():
    from skity_gb300 import scene as S
    return _cached_scenes("config3", S.config3)


def load_config2():
    from skity_gb300 import scene as S
    return _cached_scenes("config2", lambda: [S.config2()])[0]


def load_config4():
    from skity_gb300 import scene as S
    return _cached_scenes("config4", lambda: [S.config4()])[0]


def committed_digests() -> dict:
    try:
        with open(os.path.join(HERE, "tests", "golden", "full_digests.json")) as f:
            return json.load(f)
    except Exception:
        return {}


def digest(px) -> str:
    return hashlib.sha256(px.tobytes()).hexdigest()


def oracle_pool(scenes, threads: int):
    """The oracle on `threads` host threads, one canvas per thread at a time,
    canvases dealt largest first: pixels per canvas and the wall time."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle import oracle
    oracle.build()
    order = sorted(range(len(scenes)), key=lambda i: -scenes[i].n_draws * scenes[i].height)
    out = [None] * len(scenes)

    def one(i):
        out[i] = oracle.render(scenes[i])[0]

    t0 = time.perf_counter()
    with ThreadPoolExecutor(threads) as ex:
        list(ex.map(one, order))
    return out, time.perf_counter() - t0


def parity(got: list, want: list) -> dict:
    from oracle import oracle
    worst, bad, px = 0, 0, 0
    for g, w in zip(got, want):
        c = oracle.compare(g, w)
        worst = max(worst, c["max_abs_diff"])
        bad += c["bad_pixels"]
        px += g.shape[0] * g.shape[1]
    exact = 1.0 - bad / max(px, 1)
    return {"max_abs_diff": worst, "exact_frac": exact, "bad_pixels": bad, "pixels": px,
            "pass": worst <= TOL_LSB and exact >= MIN_EXACT, "against": "oracle pixels"}


def parity_by_digest(name: str, got: list, scenes, threads: int) -> dict:
    """Pixels against the committed oracle digests of the workload; on a
    mismatch the oracle renders the canvases and the difference is
    measured."""
    want = committed_digests().get(name)
    if want and len(want) == len(got) and all(digest(g) == w for g, w in zip(got, want)):
        return {"max_abs_diff": 0, "exact_frac": 1.0, "bad_pixels": 0,
                "pixels": sum(g.shape[0] * g.shape[1] for g in got), "pass": True,
                "against": "committed oracle digests (tests/golden/full_digests.json)"}
    from oracle import oracle
    ref = [oracle.render_mt(sc, threads)[0] for sc in scenes]
    return parity(got, ref)


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


def serving(ctx, rates, seconds: float, device: int, max_outstanding: int = 512,
            workers: int = 2):
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
        srv = Server(device, workers=workers, max_batch=64)
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
                        f"40 GiB; {workers} workers, up to 64 requests per batch",
            "offline_batched": offline, "rates": results}




def other_workloads(ctx, steps: int, threads: int):
    """The 512x512 scene (1,000 fills), the single large scene (2048x2048,
    20,000 paths with gradients, strokes and both fill rules), the
    glyph-dense scene (4096x4096, 100,000 small even-odd outlines, a tenth
    with a kNormal blur) and the imported tiger picture: resident batch
    renders (CUDA-graph replays), their
    pixels checked against the committed oracle digests, and the oracle
    timed on one core (a single canvas has no parallelism in the reference)
    -- over the whole scene, or the first paths of the 2048x2048 one."""
    from oracle import oracle
    from skity_gb300 import scene as S
    from skity_gb300.canvas import Batch
    out = {}
    for name, sc, desc, cpu_paths in [
            ("config1", S.config1(), "512x512, 1,000 fills of 3-32 verbs, nonzero, solid", None),
            ("config2", load_config2(), "2048x2048, 20,000 paths of 3-64 verbs over [-64,2112]^2, "
             "30% even-odd, 25% linear + 25% radial gradients, 20% stroked", 400),
            ("config4", load_config4(), "4096x4096, 100,000 outlines (1-3 contours, 8-48 px), "
                                        "even-odd, 10% kNormal blur sigma 2-20", None),
            ("skp_tiger", load_tiger(), "the reference's resources/skp/tiger.skp imported "
             "(skity_gb300/skp.py): 2560x1920, 305 fills and strokes under a canvas matrix",
             None)]:
        b = Batch(ctx, [sc])
        for _ in range(3):
            b.render()
        sts = [b.render() for _ in range(steps)]
        st = sts[-1]
        pix = b.read(0)
        b.close()
        gms = statistics.mean(s["device_ms"] for s in sts)
        n = sc.n_draws if cpu_paths is None else cpu_paths
        _, cst = oracle.render(sc, 0, n)
        cpu_ps = n / cst.seconds
        px = sc.width * sc.height
        out[name] = {"workload": desc, "paths": sc.n_draws,
                     "gpu": {"ms": gms, "paths_per_s": sc.n_draws * 1e3 / gms,
                             "mpix_per_s": px / 1e3 / gms,
                             "stage_ms": {k: st[k] for k in ("geometry_ms", "plan_ms",
                                                             "sweep_emit_ms", "composite_ms",
                                                             "blur_ms")},
                             "spans": st["spans"], "fragments": st["fragments"]},
                     "cpu": {"paths_per_s": cpu_ps, "cores": 1, "kind": "port",
                             "sample": "whole scene" if cpu_paths is None
                             else f"first {n} of {sc.n_draws} paths, {cst.seconds:.1f} s"},
                     "gpu_over_cpu": (sc.n_draws * 1e3 / gms) / cpu_ps,
                     "parity": (parity_by_digest(name, [pix], [sc], threads)
                                if name != "skp_tiger" else tiger_parity(pix, sc, threads)),
                     "coverage": coverage_report(ctx, sc, 16)}
    return out


def load_tiger():
    """The tiger picture as the SKP importer wrote it (tests/golden/tiger_scene.bin.gz)."""
    import gzip
    from skity_gb300 import scene as S
    with gzip.open(os.path.join(HERE, "tests", "golden", "tiger_scene.bin.gz"), "rb") as f:
        return S.Scene.from_bytes(f.read())


def tiger_parity(pix, sc, threads: int) -> dict:
    """The tiger's pixels against the digest of the reference IO module's own
    playback of the SKP (tests/golden/skp_digests.json)."""
    with open(os.path.join(HERE, "tests", "golden", "skp_digests.json")) as f:
        want = json.load(f)["tiger"]["pixels_sha256"]
    if digest(pix) == want:
        return {"max_abs_diff": 0, "exact_frac": 1.0, "bad_pixels": 0,
                "pixels": pix.shape[0] * pix.shape[1], "pass": True,
                "against": "the reference's playback of the SKP (tests/golden/skp_digests.json)"}
    from oracle import oracle
    return parity([pix], [oracle.render_mt(sc, threads)[0]])


def coverage_report(ctx, scene, n_draws: int) -> dict:
    """The FP64 exact-area coverage report (oracle/exact_area.cc) of the
    first `n_draws` fill draws of a workload: each fill rendered alone (opaque
    white on transparent) by the GPU and by the oracle, its alpha against the
    path's true area -- max and mean error in 1/255 units over the pixels
    either touches."""
    from oracle import oracle
    cs = oracle.coverage_scenes(scene.subset(0, min(scene.n_draws, 4 * n_draws)))[:n_draws]
    gpu = ctx.render_streams([s for _, s in cs])
    ref = [oracle.render(s)[0] for _, s in cs]
    sub = scene.subset(0, min(scene.n_draws, 4 * n_draws))
    rg = oracle.coverage_error(sub, [g[..., 3] for g in gpu])
    rr = oracle.coverage_error(sub, [r[..., 3] for r in ref])
    return {"draws": len(cs), "gpu": rg, "reference": rr,
            "same_pixels": all(bool((g == r).all()) for g, r in zip(gpu, ref))}


def run_reference(args, rank, world):
    """The reference arm: the reference's CPU software path -- its restatement
    in oracle/, pinned pixel for pixel to the reference's own build -- on the
    same 256 canvases, on every host core (a pool of one thread per core,
    canvases largest first).  Each step renders every canvas."""
    if rank != 0:
        return 0
    scenes = load_config3()
    if args.ref_canvases:
        scenes = scenes[:args.ref_canvases]
    threads = os.cpu_count() or 1
    paths = sum(sc.n_draws for sc in scenes)
    for _ in range(args.warmup):
        oracle_pool(scenes, threads)
    secs = [oracle_pool(scenes, threads)[1] for _ in range(args.steps)]
    ms = 1e3 * statistics.mean(secs)
    value = paths / (ms / 1e3)
    line = {
        "metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8/int32/f32", "data": "synthetic (seeded)",
        "impl": "reference", "config": bench_config(scenes, world),
        "mpix_per_s": sum(sc.width * sc.height for sc in scenes) / 1e6 / (ms / 1e3),
        "cpu_baseline": {"value": value, "unit": "paths/s", "cores": threads, "kind": "port",
                         "sample": f"every step: all {len(scenes)} canvases ({paths} paths) on a "
                                   f"{threads}-thread pool, largest first"},
        "e2e": {"value": value, "unit": "paths/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def workload_scenes(args):
    """The timed workload: the 256-canvas batch (or its first --canvases);
    --workload picks one of the single-canvas scenes instead, cut to its
    first --paths draws -- small cases for profiling single kernels."""
    if args.workload == "config3":
        scenes = load_config3()
        return scenes[:args.canvases] if args.canvases else scenes
    from skity_gb300 import scene as S
    sc = {"config1": S.config1, "config2": load_config2, "config4": load_config4,
          "tiger": load_tiger}[args.workload]()
    return [sc.subset(0, args.paths) if args.paths else sc]


def run_gpu(args, rank, world, local):
    import torch
    import torch.distributed as dist
    torch.cuda.set_device(local)
    if world > 1 and not dist.is_initialized():
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from skity_gb300 import autotune
    from skity_gb300.canvas import Batch, Context

    scenes = workload_scenes(args)
    paths = sum(sc.n_draws for sc in scenes)
    pix = sum(sc.width * sc.height for sc in scenes)
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    threads = os.cpu_count() or 1
    ctx = Context(local)
    batch = Batch(ctx, scenes)
    tuned = (autotune.tune(batch, autotune.signature(scenes, "GB300"), reps=2)
             if not args.no_tune else {"config": batch.config(), "cached": False, "trials": []})
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
    value = world * paths / (ms_per_step / 1e3)
    last = stages[-1]
    got = [batch.read(i) for i in range(len(scenes))]

    # end to end through the C ABI with host buffers: every step uploads the
    # scene streams, plans and renders on the device, and reads every canvas back
    e2e_ms, e2e_parts = [], []
    if not args.no_e2e:
        # the canvases land in page-locked host memory, as a renderer handing
        # frames to a compositor or an encoder would keep them
        pinned = [torch.empty((sc.height, sc.width, 4), dtype=torch.uint8,
                              pin_memory=True).numpy() for sc in scenes]
        ctx.render_streams(scenes, pinned)  # warm
        for _ in range(max(1, min(args.steps, 5))):
            e2e_out = ctx.render_streams(scenes, pinned)
            est = ctx.stats()
            e2e_ms.append(est["total_ms"])
            e2e_parts.append(est)
        e2e_same = all(bool((a == b).all()) for a, b in zip(e2e_out, got))
    e2e_ms_mean = statistics.mean(e2e_ms) if e2e_ms else None

    stage_ms = {k: statistics.mean(s[k] for s in stages)
                for k in ("geometry_ms", "plan_ms", "sweep_count_ms", "sweep_emit_ms",
                          "composite_ms", "blur_ms")}
    peak, peak_kind = measured_peaks()
    line = {
        "metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8/int32/f32",
        "data": "synthetic (seeded, skity_gb300.scene.config3)",
        "config": bench_config(scenes, world),
        "mpix_per_s": world * pix / 1e6 / (ms_per_step / 1e3),
        "stage_ms": stage_ms,
        "raster_config": tuned["config"], "autotune_cached": tuned.get("cached"),
        "work": {"passes": last["passes"], "edges": last["edges"], "spans": last["spans"],
                 "fragments": last["fragments"],
                 "fragments_per_s": world * last["fragments"] / (ms_per_step / 1e3)},
        "gpu_launches": int(sum(s["kernel_launches"] for s in stages)),
        "host_syncs_per_step": int(last["host_syncs"]),
        "clocks": clk,
        "roofline": sweep_roofline(last, stage_ms["sweep_emit_ms"], clk, sms, peak, peak_kind),
        "issue_roofline": issue_roofline(last, ms_per_step, stage_ms["composite_ms"], clk, sms),
        "e2e": {"value": (world * paths / (e2e_ms_mean / 1e3)) if e2e_ms_mean else None,
                "unit": "paths/s",
                "h2d_bytes_per_step": sum(len(sc.to_bytes()) for sc in scenes),
                "d2h_bytes_per_step": pix * 4, "ms_per_step": e2e_ms_mean,
                "stage_ms": ({k: statistics.mean(p[k] for p in e2e_parts)
                              for k in ("parse_ms", "upload_ms", "device_ms", "readback_ms")}
                             if e2e_parts else None),
                "same_pixels": e2e_same if e2e_ms else None},
        "wall_s": wall,
    }
    if rank == 0 and not args.no_per_draw:
        # the per-draw form runs each path's sequential work alone (about
        # 1.6 ms a draw), so it is timed on the first canvases only
        sub = scenes[:args.per_draw_canvases]
        spaths = sum(sc.n_draws for sc in sub)
        spix = sum(sc.width * sc.height for sc in sub)
        pb = Batch(ctx, sub)
        pst = pb.render_per_draw()  # capacities found on the way (its time: the last attempt)
        pd_same = all(bool((pb.read(i) == g).all()) for i, g in enumerate(got[:len(sub)]))
        pb.close()
        line["per_draw"] = {"ms": pst["device_ms"], "paths_per_s": spaths * 1e3 / pst["device_ms"],
                            "mpix_per_s": spix / 1e3 / pst["device_ms"],
                            "ms_per_draw": pst["device_ms"] / spaths,
                            "kernel_launches": int(pst["kernel_launches"]),
                            "host_syncs": int(pst["host_syncs"]), "same_pixels": pd_same,
                            "sample": f"first {len(sub)} canvases ({spaths} paths)",
                            "form": "skity_cuda_batch_render_per_draw: geometry, plan, sweep and "
                                    "composite launches per DrawPath, one stream, no host sync "
                                    "until the end"}
        line["batched_over_per_draw"] = value / world / line["per_draw"]["paths_per_s"]
    if rank == 0 and not args.no_cpu:
        ref, cpu_s = oracle_pool(scenes, threads)
        line["parity"] = parity(got, ref)
        line["cpu_baseline"] = {"value": paths / cpu_s, "unit": "paths/s", "cores": threads,
                                "kind": "port", "seconds": cpu_s,
                                "sample": f"all {len(scenes)} canvases ({paths} paths) on a "
                                          f"{threads}-thread pool, largest first"}
        line["batched_over_cpu"] = value / world / (paths / cpu_s)
        line["coverage"] = coverage_report(ctx, scenes[0], 32)
        if e2e_ms_mean:
            line["e2e_over_cpu"] = (paths / (e2e_ms_mean / 1e3)) / (paths / cpu_s)
    if rank == 0 and not args.no_others:
        line["other_workloads"] = other_workloads(ctx, max(1, min(args.steps, 5)), threads)
    if rank == 0 and args.serve_seconds > 0:
        line["serving"] = serving(ctx, [float(r) for r in args.serve_rates.split(",")],
                                  args.serve_seconds, local, workers=args.serve_workers)
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
    ap.add_argument("--canvases", type=int, default=0,
                    help="render only the first N canvases (small profiling case)")
    ap.add_argument("--workload", default="config3",
                    choices=["config3", "config1", "config2", "config4", "tiger"],
                    help="profiling: time one of the single-canvas scenes instead of the batch")
    ap.add_argument("--paths", type=int, default=0,
                    help="profiling: the first N draws of a single-canvas --workload")
    ap.add_argument("--ref-canvases", type=int, default=0,
                    help="reference arm: the first N canvases per step (default all)")
    ap.add_argument("--no-tune", action="store_true", help="default raster config, no autotuning")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-per-draw", action="store_true")
    ap.add_argument("--per-draw-canvases", type=int, default=8,
                    help="canvases the per-draw form is timed on")
    ap.add_argument("--no-others", action="store_true",
                    help="skip the 512x512, 2048x2048 and glyph-dense scenes")
    ap.add_argument("--serve-rates", default="200,1000,5000",
                    help="Poisson request rates (requests/s) of the serving runs")
    ap.add_argument("--serve-workers", type=int, default=2,
                    help="serving loop workers (concurrent batches, each its own stream)")
    ap.add_argument("--serve-seconds", type=float, default=60.0,
                    help="arrival window per rate (the serving workload's 60 s); 0 skips")
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
