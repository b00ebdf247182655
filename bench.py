#!/usr/bin/env python3
"""Headline benchmark: Msamples/s of the NEE+MIS path tracer on the
environment-map Cornell box (512x512, 256 spp, max path length 12, Russian
roulette after 3 bounces, synthetic 1024x512 sky), one JSON line on stdout.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

A step renders the whole workload once (512*512*256 = 67,108,864 camera paths).
* value    device time (CUDA events on the library's stream) of K steps, inputs
           resident in HBM, L2 flushed between steps (a 256 MiB memset outside
           the timed events);
* e2e      the same metric through the C ABI as a user calls it with host
           buffers: create (scene + environment map host->device), render,
           read the framebuffer (device->host), destroy -- per step;
* roofline algorithmic bytes of the path kernel per launch (per segment 360 B,
           per path 72 B start + 36 B end, the wavefront record sizes) over its
           event-timed launch duration, against the measured HBM copy peak;
* cpu_baseline the reference's own CPU renderer (oracle/_ref, built from the
           reference sources) on all host cores over a bounded sample.
* secondary the other two parts of the metric, on their own workloads: batched
           scenes/s (64 seeded variants in one persistent launch vs a loop of
           single-scene launches), forward+adjoint ms/iteration with a
           finite-difference check of the gradient, and the inverse-rendering loop
           (500 Adam steps, one CUDA graph per iteration); and the headline
           workload's variants: the LBVH on a mesh, one call per iteration, the
           adaptive triangulation, the CDF and cosine samplers, with the
           equal-quality speedup of every GPU sampler against the reference's
           steerable and CDF samplers.
--impl reference times that CPU renderer alone as the main line.
With N > 1 (torchrun) every rank renders its own sample range of the same
workload (weak scaling, no collective on the data path).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Msamples/s at matched rel-MSE vs CPU"
UNIT = "Msamples/s"
WIDTH = HEIGHT = 512
SPP = 256
MESH_SIDE, MESH_SPP = 512, 64
MAX_PATH = 12
RR_FROM = 4            # Russian roulette from path length 4, i.e. after 3 bounces
EM_W, EM_H = 1024, 512
# per-unit algorithmic bytes of the wavefront record layout (ray 32, hit 16, state 40, shadow 48)
BYTES_PER_SEGMENT = 360
BYTES_PER_PATH = 72 + 36
# DRAM bytes (read + write) per camera path of one launch chunk, measured by ncu over all stage
# kernels of one step of the 128x128 x 64 spp case of this workload (one chunk of 2^20 paths);
# the chunk's traffic grows with its paths.
NCU_TRAFFIC_PER_PATH = 954.4


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--sampler", default="auto", choices=["auto", "steerable", "cdf", "cosine"])
    ap.add_argument("--pipeline", default="auto", choices=["auto", "megakernel", "wavefront"])
    ap.add_argument("--steer-weights", default="projected", choices=["point", "projected"],
                    help="vertex luminance of the steerable sampler: the map's value at the vertex (the "
                         "reference's build) or its projection onto the vertex's hat function")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=None)
    # smaller cases of the same workload (profiling captures); the headline uses the defaults
    ap.add_argument("--width", type=int, default=512)
    ap.add_argument("--spp", type=int, default=256)
    ap.add_argument("--cpu-iters", type=int, default=12)
    ap.add_argument("--paths-in-flight", type=int, default=0, help="wavefront chunk size (0: automatic)")
    ap.add_argument("--no-secondary", action="store_true",
                    help="skip the batched (64 scenes), forward+adjoint and inverse-rendering measurements")
    ap.add_argument("--only-secondary", default=None,
                    choices=["batched", "differentiable", "inverse_rendering", "mesh_bvh", "per_iteration",
                             "adaptive_sampler", "samplers"],
                    help="run one secondary measurement alone and print its JSON (profiling captures)")
    ap.add_argument("--mesh-side", type=int, default=512, help="image side of the LBVH mesh measurement")
    ap.add_argument("--mesh-spp", type=int, default=64, help="samples per pixel of the LBVH mesh measurement")
    a = ap.parse_args()
    global WIDTH, HEIGHT, SPP, MESH_SIDE, MESH_SPP
    WIDTH = HEIGHT = a.width
    SPP = a.spp
    MESH_SIDE, MESH_SPP = a.mesh_side, a.mesh_spp
    return a


def build_scene():
    from pg3render_gb300 import scene as S
    return S.cornell_env(WIDTH, HEIGHT, EM_W, EM_H, em_seed=7)


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples (200 ms) of SM clock and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------------- CPU baseline
def cpu_baseline(scene, sampler, threads=None, iters=1):
    """The reference's own CPU renderer (oracle/_ref) on the same scene, all host cores,
    `threads` renderers x `iters` iterations at 512x512; falls back to the oracle port."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    threads = threads or os.cpu_count() or 1
    ref_sampler = {"steerable": "steerable", "cdf": "cdf", "cosine": "cosine"}[sampler]
    with tempfile.TemporaryDirectory() as td:
        em = os.path.join(td, "em.bin")
        scene.write_env_map(em)
        text = scene.to_text(em_path=em, max_path_length=MAX_PATH)
        if O.reference_binary(ref_sampler):
            extra = ["--em-params", "5", "3", "3"] if ref_sampler == "steerable" else []
            r = O.reference_render(text, renderers=threads, iters=iters, threads=threads, seed=1,
                                   em_sampler=ref_sampler, time_only=True, extra=extra)
            t = r["timing"]
            return {"value": t["msamples_per_s"], "unit": UNIT, "cores": t["threads"], "kind": "reference",
                    "sample": "%d renderers x %d iteration(s) of the %dx%d scene (%.1f M paths, %.1f s), max path "
                              "length %d without roulette (the reference applies roulette only without a length "
                              "limit), %s sampler" % (threads, iters, WIDTH, HEIGHT, t["samples"] / 1e6,
                                                      t["seconds"], MAX_PATH, ref_sampler)}
        # oracle port (C++ restatement) -- CDF / cosine only
        t0 = time.perf_counter()
        spp = max(1, iters * threads // 8)
        O.render(text, WIDTH, HEIGHT, seed=1, spp=spp, em_sampler=0 if sampler == "cdf" else 1,
                 rr_min_path_length=RR_FROM, threads=threads)
        dt = time.perf_counter() - t0
        return {"value": WIDTH * HEIGHT * spp / dt / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
                "sample": "%d spp of the %dx%d scene" % (spp, WIDTH, HEIGHT)}


ADAPTIVE_DEFAULT = (4, 9, 5.0)   # the reference's default steerable build: levels 4-9, error 5


def adaptive_kw(levels):
    if not levels:
        return {}
    return dict(steer_subdiv_level=levels[0], steer_max_subdiv_level=levels[1], steer_max_approx_error=levels[2])


def matched_quality(gpu_value, cpu_value, steer_weights, spps=(16, 256), renders=(16, 8)):
    """Per-sample quality of the two renderers on the headline scene (its full 1024x512 sky) at
    64x64 pixels: the relative MSE, mean over pixel channels of (x - c)^2 / (c^2 + 0.01), of
    images of spp samples against the converged image c, averaged over independent images. c is
    the reference's own CPU renderer at 65536 samples per pixel (CDF sampler, max length 12;
    the committed fixture tests/golden/cornell_env_64_sky1024_cdf.npz, made by
    tests/golden/make_golden.py). Measured for the GPU path (roulette from length 4; steerable
    sampler with both vertex weightings, and the CDF sampler) and for the reference's own CPU
    renderer (max length 12 without roulette; its steerable sampler at 1280 triangles and its
    CDF sampler). The reference's steerable sampler evaluates its pdf from the map instead of
    the density it samples, so its images converge to a darker limit (bias). At the benchmark's
    256 samples per pixel, the ratio of the relative MSEs turns the Msamples/s ratio into an
    equal-quality speedup: the GPU renders the samples that reach the reference's error in that
    many times less time."""
    import numpy as np
    import pg3render_gb300 as P
    from pg3render_gb300 import scene as S
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    R = P.renderer
    golden = np.load(os.path.join(ROOT, "tests", "golden", "cornell_env_64_sky1024_cdf.npz"))
    conv = golden["mean"]
    side = conv.shape[0]
    sc = S.cornell_env(side, side, EM_W, EM_H, em_seed=7)
    sc.env_map = golden["env_map"]   # the map the reference rendered (bit for bit)
    # the third entry: an adaptive triangulation with the reference's default build parameters
    # (levels 4-9, error 5) instead of the uniform 1280 triangles
    gpu_cfgs = {"steerable_point": (R.EM_STEERABLE, R.STEER_WEIGHTS_POINT, None),
                "steerable_projected": (R.EM_STEERABLE, R.STEER_WEIGHTS_PROJECTED, None),
                "steerable_adaptive_projected": (R.EM_STEERABLE, R.STEER_WEIGHTS_PROJECTED, ADAPTIVE_DEFAULT),
                "cdf": (R.EM_CDF, 0, None),
                "cosine": (R.EM_COSINE, 0, None)}

    def gpu_image(key, seed, n):
        em, w, ad = gpu_cfgs[key]
        cfg = P.Config(scene=sc, max_path_length=MAX_PATH, rr_min_path_length=RR_FROM, em_sampler=em,
                       steer_weights=w, **adaptive_kw(ad))
        with P.GpuPathTracer(cfg, seed=seed) as r:
            r.RunIteration(R.kPathTracing, 0, n)
            return r.framebuffer()[0]

    def rel_mse(img):
        return float(np.mean((img - conv) ** 2 / (conv ** 2 + 0.01)))

    out = {"side": side, "converged": "the reference's CPU renderer, CDF sampler, %d spp (max path length 12)"
           % int(golden["spp"])}
    with tempfile.TemporaryDirectory() as td:
        em_path = os.path.join(td, "em.bin")
        sc.write_env_map(em_path)
        text = sc.to_text(em_path=em_path, max_path_length=MAX_PATH)
        for spp, reps in zip(spps, renders):
            row = {"renders": reps}
            for key in gpu_cfgs:
                row["gpu_" + key] = round(statistics.mean(rel_mse(gpu_image(key, 1000 + k, spp))
                                                          for k in range(reps)), 6)
            for name in ("steerable", "cdf"):
                if O.reference_binary(name):
                    extra = ["--em-params", "5", "3", "3"] if name == "steerable" else []
                    row["cpu_reference_" + name] = round(statistics.mean(
                        rel_mse(O.reference_render(text, renderers=spp, iters=1, seed=2000 + k, em_sampler=name,
                                                   extra=extra)["mean"]) for k in range(reps)), 6)
            out["rel_mse_at_%dspp" % spp] = row
    last = out["rel_mse_at_%dspp" % spps[-1]]
    mine = last["gpu_steerable_" + steer_weights]
    if "cpu_reference_steerable" in last and cpu_value and mine > 0:
        ratio = last["cpu_reference_steerable"] / mine
        out["headline_sampler"] = "steerable_" + steer_weights
        out["rel_mse_ratio_cpu_over_gpu_at_%dspp" % spps[-1]] = round(ratio, 4)
        out["equal_quality_speedup"] = round(gpu_value / cpu_value * ratio, 2)
    return out


# ----------------------------------------------------------------------------- ranks
SAMPLES_PER_RANK = 1 << 24   # sample-index stride between ranks: disjoint random streams


def rank_sample_base(rank):
    """First sample index a rank renders. Ranks render disjoint sample ranges of the same
    workload (weak scaling, no collective on the data path)."""
    return rank * SAMPLES_PER_RANK


def max_over_ranks(x, device):
    """The slowest rank's value (the timing rule: max over ranks)."""
    import torch
    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def whole_job_value(world, steps, paths_per_step, total_s):
    """Msamples/s of the whole job: every rank renders paths_per_step per step."""
    return world * steps * paths_per_step / total_s / 1e6


# ----------------------------------------------------------------------------- GPU arm
def run_gpu(args, rank, world, local_rank):
    import torch
    import pg3render_gb300 as P
    from pg3render_gb300 import _lib
    from pg3render_gb300 import renderer as R

    torch.cuda.set_device(local_rank)
    scene = build_scene()
    sampler = args.sampler
    if sampler == "auto":
        sampler = "steerable"   # the workload's light sampler (icosahedron subdivided to 1280 triangles)
    em_sampler = {"steerable": R.EM_STEERABLE, "cdf": R.EM_CDF, "cosine": R.EM_COSINE}[sampler]
    pipeline = {"auto": R.PIPELINE_AUTO, "megakernel": R.PIPELINE_MEGAKERNEL,
                "wavefront": R.PIPELINE_WAVEFRONT}[args.pipeline]
    steer_weights = {"point": R.STEER_WEIGHTS_POINT, "projected": R.STEER_WEIGHTS_PROJECTED}[args.steer_weights]
    cfg = P.Config(scene=scene, algorithm=R.kPathTracing, max_path_length=MAX_PATH, rr_min_path_length=RR_FROM,
                   em_sampler=em_sampler, pipeline=pipeline, base_seed=1234,
                   max_paths_in_flight=args.paths_in_flight, steer_weights=steer_weights)
    npix = WIDTH * HEIGHT
    paths_per_step = npix * SPP
    sample_base = rank_sample_base(rank)
    if (args.warmup + args.steps) * SPP > SAMPLES_PER_RANK:
        raise ValueError("warmup + steps exceed the sample range of a rank")

    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    r = P.GpuPathTracer(cfg, device=local_rank)
    for w in range(args.warmup):
        r.RunIteration(R.kPathTracing, sample_base + w * SPP, SPP)
    r.synchronize()
    r.reset_stats()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    stops = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with ClockSampler(local_rank) as clk:
        for k in range(args.steps):
            flush.zero_()                                  # L2 flush, outside the events
            starts[k].record()
            r.RunIteration(R.kPathTracing, sample_base + (args.warmup + k) * SPP, SPP)
            stops[k].record()
        torch.cuda.synchronize()
    r.synchronize()
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, stops)]
    total_s = sum(step_ms) / 1e3
    st = r.stats()
    if world > 1:
        total_s = max_over_ranks(total_s, "cuda")
        torch.distributed.barrier()
    value = whole_job_value(world, args.steps, paths_per_step, total_s)

    # roofline of the path kernel
    launches = max(1, st["path_kernel_launches"])
    launch_ms = st["path_kernel_ms"] / launches
    alg_bytes = (BYTES_PER_SEGMENT * st["extension_rays"] + BYTES_PER_PATH * st["paths"]) / launches
    peak, peak_kind = load_peaks()
    achieved = alg_bytes / (launch_ms / 1e3) / 1e9
    traffic = (NCU_TRAFFIC_PER_PATH * st["paths"] / launches) if NCU_TRAFFIC_PER_PATH else None
    roofline = {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 5), "traffic": traffic, "peak_source": peak_kind,
                "kernel": "megakernel" if args.pipeline == "megakernel" else "wavefront (all stage kernels of a chunk)",
                "launch_ms": round(launch_ms, 4), "algorithmic_bytes_per_launch": int(alg_bytes),
                "segments_per_path": round(st["extension_rays"] / max(1, st["paths"]), 4),
                "shadow_rays_per_path": round(st["shadow_rays"] / max(1, st["paths"]), 4)}
    gpu_launches = int(st["kernel_launches"])
    r.close()

    # end to end through the C ABI with host buffers
    e2e_steps = args.e2e_steps if args.e2e_steps is not None else max(1, min(args.steps, 5))
    desc_bytes = (scene.env_map.nbytes + 40 * len(scene.triangles) + 20 * len(scene.spheres)
                  + 32 * len(scene.materials) + 16 * len(scene.area_lights))
    d2h = npix * 3 * 8
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    img = None
    for k in range(e2e_steps):
        with P.GpuPathTracer(cfg, device=local_rank) as rr:
            rr.RunIteration(R.kPathTracing, sample_base + k * SPP, SPP)
            img = rr.GetFramebuffer()
    torch.cuda.synchronize()
    e2e_s = max(time.perf_counter() - t0, 1e-9)
    if world > 1:
        e2e_s = max_over_ranks(e2e_s, "cuda")
    e2e = None
    if e2e_steps > 0:
        e2e = {"value": round(whole_job_value(world, e2e_steps, paths_per_step, e2e_s), 3), "unit": UNIT,
               "h2d_bytes_per_step": int(desc_bytes), "d2h_bytes_per_step": int(d2h), "steps": e2e_steps,
               "image_mean": [round(float(x), 5) for x in img.mean(axis=(0, 1))]}
        # where an end-to-end step's time goes (measured after the timed loop, host clock): create
        # (scene and map upload, sampler tables), render + framebuffer readback, destroy
        parts = {"create_ms": [], "render_and_read_ms": [], "destroy_ms": []}
        for k in range(2):
            t0 = time.perf_counter()
            rr = P.GpuPathTracer(cfg, device=local_rank)
            t1 = time.perf_counter()
            rr.RunIteration(R.kPathTracing, sample_base + k * SPP, SPP)
            rr.GetFramebuffer()
            t2 = time.perf_counter()
            rr.close()
            t3 = time.perf_counter()
            parts["create_ms"].append((t1 - t0) * 1e3)
            parts["render_and_read_ms"].append((t2 - t1) * 1e3)
            parts["destroy_ms"].append((t3 - t2) * 1e3)
        e2e["breakdown"] = {k: round(statistics.median(v), 3) for k, v in parts.items()}

    if rank != 0:
        return None
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_s * 1e3 / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "cornell_env_%dx%d_%dspp_maxpl12_rr3_em1024x512_%s" % (WIDTH, HEIGHT, SPP, sampler),
                   "width": WIDTH, "height": HEIGHT, "spp": SPP, "max_path_length": MAX_PATH,
                   "rr_min_path_length": RR_FROM, "env_map": [EM_W, EM_H], "em_sampler": sampler,
                   "steer_weights": args.steer_weights if sampler == "steerable" else None,
                   "pipeline": args.pipeline, "paths_per_step": paths_per_step,
                   "l2": "flushed between steps (256 MiB memset outside the timed events)",
                   "parallelism": "replicas over sample ranges" if world > 1 else "single GPU"},
        "e2e": e2e, "roofline": roofline, "gpu_launches": gpu_launches,
        "step_ms": [round(x, 3) for x in step_ms],
    }
    line["clocks"] = clk.summary()
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(scene, sampler, iters=args.cpu_iters)
        if sampler == "steerable" and not args.no_secondary:
            # the reference's CDF sampler on the same cores, for the per-sampler comparison
            try:
                line["cpu_baseline"]["cdf_value"] = cpu_baseline(scene, "cdf", iters=max(1, args.cpu_iters // 2))["value"]
            except Exception as e:   # reported, never hidden
                line["cpu_baseline"]["cdf_value"] = None
                line["cpu_baseline"]["cdf_error"] = "%s: %s" % (type(e).__name__, e)
        if sampler == "steerable":
            try:
                line["cpu_baseline"]["matched_quality"] = matched_quality(value, line["cpu_baseline"]["value"],
                                                                          args.steer_weights)
            except Exception as e:   # reported, never hidden
                line["cpu_baseline"]["matched_quality"] = {"error": "%s: %s" % (type(e).__name__, e)}
    if world == 1 and not args.no_secondary:
        line["secondary"] = secondary_metrics()
        # the same equal-quality figure for the adaptive triangulation: its own Msamples/s and its
        # relative MSE at the benchmark's samples per pixel
        mq = line.get("cpu_baseline", {}).get("matched_quality", {})
        ad = line["secondary"].get("adaptive_sampler", {})
        last = mq.get("rel_mse_at_%dspp" % SPP, {})
        if ad.get("msamples_per_s") and last.get("gpu_steerable_adaptive_projected") and \
                last.get("cpu_reference_steerable"):
            ratio = last["cpu_reference_steerable"] / last["gpu_steerable_adaptive_projected"]
            ad["rel_mse_ratio_cpu_over_gpu_at_%dspp" % SPP] = round(ratio, 4)
            ad["equal_quality_speedup"] = round(ad["msamples_per_s"] / line["cpu_baseline"]["value"] * ratio, 2)
        if "cpu_baseline" in line and sampler == "steerable":
            line["secondary"]["sampler_comparison"] = sampler_comparison(line)
    return line


# ----------------------------------------------------------------------------- secondary metrics
def _events():
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def batched_metric(reps=3):
    """64 seeded Cornell-box variants (side 64..512 log-uniform, 4..64 spp, 0..8 spheres, half
    area light / half 256x128 sky, Russian roulette path lengths): one autotuned batch run (one
    CUDA graph launch) against a loop of plain single-scene launches of the same scenes."""
    import torch
    import pg3render_gb300 as P
    from pg3render_gb300 import scene as S
    R = P.renderer
    cfgs, spps = [], []
    for i in range(64):
        s, k = S.random_variant(i)
        cfgs.append(P.Config(scene=s, max_path_length=0, base_seed=1000 + i, max_paths_in_flight=1 << 21))
        spps.append(k)
    paths = sum(c.scene.camera.width * c.scene.camera.height * k for c, k in zip(cfgs, spps))
    ctxs = [P.GpuPathTracer(c) for c in cfgs]
    for r, k in zip(ctxs, spps):
        r.RunIteration(R.kPathTracing, 0, k)
    for r in ctxs:
        r.synchronize()
    loop = []
    for rep in range(reps):
        t0 = time.perf_counter()
        for r, k in zip(ctxs, spps):
            r.RunIteration(R.kPathTracing, (rep + 1) * k, k)
        for r in ctxs:
            r.synchronize()
        loop.append(time.perf_counter() - t0)
    for r in ctxs:
        r.close()
    b = P.GpuBatch(cfgs, spps)
    t0 = time.perf_counter()
    tuning = b.autotune(16)
    tune_s = time.perf_counter() - t0
    b.run()
    b.synchronize()
    batch, dev = [], []
    for rep in range(reps):
        t0 = time.perf_counter()
        b.run()
        b.synchronize()
        batch.append(time.perf_counter() - t0)
        dev.append(b.stats()["last_iteration_ms"])
    st = b.stats()
    b.close()
    lt, bt = statistics.median(loop), statistics.median(batch)
    return {"metric": "batched scenes/s", "scenes": 64, "paths_per_run": paths,
            "batched_scenes_per_s": round(64 / bt, 2), "loop_scenes_per_s": round(64 / lt, 2),
            "speedup_vs_loop": round(lt / bt, 2), "batch_run_ms": round(bt * 1e3, 2),
            "batch_device_ms": round(statistics.median(dev), 2), "loop_run_ms": round(lt * 1e3, 2),
            "batch_msamples_per_s": round(paths / bt / 1e6, 1), "tuning": tuning, "autotune_s": round(tune_s, 2),
            "timing": "host wall clock of whole runs incl. synchronisation, median of %d" % reps,
            "paths_counted": int(st["paths"])}


def differentiable_metric(steps=5):
    """The gradient configuration: the environment-lit box with 4 Lambert and 4 GGX materials at
    256x256, 64 spp, 512x256 map, max path length 12, roulette after 3 bounces; L2 loss against a
    fixed target. Reports forward+adjoint ms/iteration against the plain forward, and the
    adjoint against central differences (step 1e-3, common random numbers, sampling held fixed)
    of the loss restricted to a 32x32 crop."""
    import numpy as np
    import torch
    import pg3render_gb300 as P
    from pg3render_gb300 import scene as S, _lib
    R = P.renderer
    sc = S.cornell_env_diff(256, 256, 512, 256)
    cfg = P.Config(scene=sc, max_path_length=MAX_PATH, rr_min_path_length=RR_FROM, em_sampler=_lib.EM_STEERABLE,
                   base_seed=3)
    spp = 64
    out = {"metric": "fwd+adjoint ms/iter", "workload": "cornell_env_diff_256x256_64spp_maxpl12_rr3_em512x256_steerable",
           "paths": 256 * 256 * spp}
    with P.diff.DiffRenderer(cfg) as dr:
        dr.use_torch_stream()
        for _ in range(3):
            dr.RunIteration(R.kPathTracing, 0, spp)
        a, b = _events()
        torch.cuda.synchronize()
        a.record()
        for k in range(steps):
            dr.RunIteration(R.kPathTracing, 0, spp)
        b.record()
        torch.cuda.synchronize()
        fwd = a.elapsed_time(b) / steps
        img = torch.empty((256, 256, 3), device="cuda")
        target = torch.full_like(img, 0.25)
        crop = torch.zeros_like(img)
        crop[112:144, 112:144] = 1
        gm = torch.zeros((len(sc.materials), 4), device="cuda")
        ge = torch.zeros((256, 512, 3), device="cuda")
        for _ in range(3):
            dr.forward_into(img, 0, spp)
            dr.adjoint_into(2 * (img - target), gm, ge)
        torch.cuda.synchronize()
        a, b = _events()
        a.record()
        for k in range(steps):
            dr.forward_into(img, 0, spp)
            dr.adjoint_into(2 * (img - target), gm, ge)
        b.record()
        torch.cuda.synchronize()
        fa = a.elapsed_time(b) / steps
        out.update(plain_forward_ms=round(fwd, 3), fwd_adjoint_ms=round(fa, 3), ratio_to_forward=round(fa / fwd, 3))
        # gradient check on the crop
        dr.forward_into(img, 0, spp)
        dl = (2 * (img - target) * crop).contiguous()
        gm.zero_()
        dr.adjoint_into(dl, gm, None)
        torch.cuda.synchronize()
        adj = gm.cpu().numpy().astype(np.float64)
        base, _ = dr.get_params()
        errs, h = [], 1e-3

        def loss_at(p):
            dr.set_params(p, None, keep_sampling=True)
            dr.forward_into(img, 0, spp)
            torch.cuda.synchronize()
            return float((((img - target) ** 2) * crop).double().sum())
        names = []
        for i, m in enumerate(sc.materials):
            cols = [0, 1, 2] if m.kind == S.MAT_LAMBERT else [3]
            for c in cols:
                p1, p2 = base.copy(), base.copy()
                p1[i, c] += h
                p2[i, c] -= h
                fd = (loss_at(p1) - loss_at(p2)) / (2 * h)
                errs.append((abs(adj[i, c] - fd), abs(fd), adj[i, c], fd))
                names.append("%s%d.%s" % ("albedo" if c < 3 else "alpha", i, "rgba"[c]))
        dr.set_params(base, None)
        scale = max(e[1] for e in errs)
        big = [e for e in errs if e[1] > 0.02 * scale]
        out["gradient_check"] = {
            "params": len(errs), "crop": [32, 32], "step": h,
            "max_rel_err": round(max(e[0] / e[1] for e in big), 5),
            "median_rel_err": round(statistics.median(e[0] / e[1] for e in big), 6),
            "params_compared": len(big), "note": "relative errors over parameters whose derivative exceeds 2% of the "
                                                 "largest; sampling held fixed (detached estimator)"}
    return out


ENV_SMOOTHNESS = 1.0   # weight of the log-texel smoothness penalty in the third inverse-rendering run


def inverse_metric():
    """The inverse-rendering configuration (128x128 x 16 spp forward + adjoint per iteration, 500
    Adam steps, one CUDA graph per iteration) three ways: map and materials jointly (the
    configuration), materials with the map at its hidden values (the materials are then
    identifiable: albedo times illumination is a scale ambiguity), with the primal residual and the
    adjoint on independent samples (the L2 loss of one noisy render favours darker renders), and
    jointly with a smoothness penalty on the log texels."""
    from pg3render_gb300 import inverse
    r = inverse.run()
    r["metric"] = "inverse rendering: 500 Adam steps, one CUDA graph per iteration"
    r.pop("loss_trace", None)
    for key, kw in (("materials_with_hidden_map", dict(optimize_env=False)),
                    ("materials_with_hidden_map_decorrelated", dict(optimize_env=False, decorrelate=True)),
                    ("joint_smooth_map_decorrelated", dict(env_smoothness=ENV_SMOOTHNESS, decorrelate=True))):
        x = inverse.run(**kw)
        r[key] = {k: x[k] for k in ("before", "after", "iteration_ms", "materials_true", "materials_found")}
        r[key]["errors_fall"] = {g: x["after"][g] < x["before"][g] for g in ("albedo_mae", "alpha_abs_err", "env_rel_l1")
                                 if kw.get("optimize_env", True) or g != "env_rel_l1"}
    return r


def mesh_metric(reps=3):
    """The environment-map box with its spheres as triangle meshes (two icospheres of 20480
    triangles each, 40968 triangles in all), 512x512 x 64 spp by default, steerable sampler: every
    closest-hit and any-hit query runs through a BVH built on the device (the list loop would test
    every triangle): the binary LBVH (the default) and the 4-wide BVH collapsed from it."""
    import torch
    import pg3render_gb300 as P
    from pg3render_gb300 import scene as S
    R = P.renderer
    side = MESH_SIDE
    sc = S.cornell_env_mesh(side, side, 1024, 512, level=5)
    spp = MESH_SPP
    paths = side * side * spp
    out = {"metric": "Msamples/s (BVH traversal)", "triangles": len(sc.triangles), "side": side, "spp": spp,
           "timing": "host wall clock of whole runs incl. synchronisation, median of %d" % reps}
    for name, trav in (("lbvh_binary", R.TRAVERSAL_BVH), ("bvh4", R.TRAVERSAL_BVH4)):
        cfg = P.Config(scene=sc, max_path_length=12, rr_min_path_length=4, em_sampler=R.EM_STEERABLE,
                       traversal=trav)
        with P.GpuPathTracer(cfg) as r:
            r.RunIteration(R.kPathTracing, 0, spp)
            r.synchronize()
            ts = []
            for rep in range(reps):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                r.RunIteration(R.kPathTracing, (rep + 1) * spp, spp)
                r.synchronize()
                ts.append(time.perf_counter() - t0)
            st = r.stats()
        t = statistics.median(ts)
        out[name] = {"msamples_per_s": round(paths / t / 1e6, 1), "ms_per_run": round(t * 1e3, 2),
                     "segments_per_path": round(st["extension_rays"] / max(1, st["paths"]), 3)}
    out["msamples_per_s"] = out["lbvh_binary"]["msamples_per_s"]
    return out


def per_iteration_metric(iters=256, reps=3):
    """The call pattern of the reference's own render loop: one pg3gpu_run_iteration per
    iteration, one sample per pixel each (RunIteration, src/pg3render.cxx:112-128), on the
    headline scene at 512x512 (the headline's 256 iterations), against one call of all 256.
    Also the reference's own program with the GPU renderer (oracle/_ref/pg3render_gpu: its
    Config, its LoadCornellBox scene -s 12 at its fixed 512x512, GpuPathTracer::RunIteration
    per iteration) where that program is built."""
    import torch
    import pg3render_gb300 as P
    R = P.renderer
    sc = build_scene()
    cfg = P.Config(scene=sc, max_path_length=MAX_PATH, rr_min_path_length=RR_FROM, em_sampler=R.EM_STEERABLE)
    paths = WIDTH * HEIGHT * iters
    out = {"metric": "Msamples/s, one sample per pixel per call", "side": WIDTH, "iterations": iters}
    with P.GpuPathTracer(cfg) as r:
        for k in range(8):
            r.RunIteration(R.kPathTracing, k, 1)
        r.RunIteration(R.kPathTracing, 8, iters)
        r.synchronize()
        r.reset_stats()
        for k in range(16):
            r.RunIteration(R.kPathTracing, 500 + k, 1)
        launches = r.stats()["kernel_launches"] / 16
        per, whole = [], []
        for rep in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for k in range(iters):
                r.RunIteration(R.kPathTracing, (rep + 1) * 1000 + k, 1)
            r.synchronize()
            per.append(time.perf_counter() - t0)
            t0 = time.perf_counter()
            r.RunIteration(R.kPathTracing, (rep + 1) * 1000, iters)
            r.synchronize()
            whole.append(time.perf_counter() - t0)
    tp, tw = statistics.median(per), statistics.median(whole)
    out.update(per_call_msamples_per_s=round(paths / tp / 1e6, 1), one_call_msamples_per_s=round(paths / tw / 1e6, 1),
               per_call_us=round(tp / iters * 1e6, 1), launches_per_call=round(launches, 1),
               timing="host wall clock of %d calls incl. the final synchronisation, median of %d" % (iters, reps))
    exe = os.path.join(ROOT, "oracle", "_ref", "pg3render_gpu")
    if os.path.exists(exe):
        prog = {}
        for batch in (1, iters):
            res = subprocess.run([exe, "-s", "12", "-a", "pt", "-minpl", "1", "-maxpl", "8", "-sb", "1", "-iic", "0",
                                  "-i", str(iters), "-q", "--batch", str(batch)], capture_output=True, text=True)
            if res.returncode != 0:
                prog["error"] = res.stderr.strip()[-300:]
                break
            prog["batch_%d" % batch] = json.loads(res.stdout.strip().splitlines()[-1])
        out["reference_program"] = prog
    return out


def adaptive_sampler_metric(reps=3):
    """The headline scene and workload (512x512 x 256 spp, max path length 12, roulette from length
    4, the 1024x512 sky) with the steerable sampler over the reference's default adaptive
    triangulation (levels 4-9, error 5, projected vertex weights) instead of 1280 uniform triangles;
    device time of one call, median of reps; the triangulation's build is part of create."""
    import torch
    import pg3render_gb300 as P
    R = P.renderer
    sc = build_scene()
    cfg = P.Config(scene=sc, max_path_length=MAX_PATH, rr_min_path_length=RR_FROM, em_sampler=R.EM_STEERABLE,
                   steer_weights=R.STEER_WEIGHTS_PROJECTED, **adaptive_kw(ADAPTIVE_DEFAULT))
    t0 = time.perf_counter()
    r = P.GpuPathTracer(cfg)
    create_ms = (time.perf_counter() - t0) * 1e3
    try:
        r.RunIteration(R.kPathTracing, 0, SPP)
        r.synchronize()
        ts = []
        for rep in range(reps):
            a, b = _events()
            a.record()
            r.RunIteration(R.kPathTracing, (rep + 1) * SPP, SPP)
            b.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
    finally:
        r.close()
    ms = statistics.median(ts)
    return {"metric": "Msamples/s (adaptive steerable triangulation)", "levels": list(ADAPTIVE_DEFAULT),
            "msamples_per_s": round(WIDTH * HEIGHT * SPP / ms / 1e3, 1), "ms_per_run": round(ms, 3),
            "create_ms": round(create_ms, 2)}


def sampler_metric(reps=3):
    """The headline workload (512x512 x 256 spp, max path length 12, roulette from length 4, the
    1024x512 sky) with the CDF and the cosine environment-map samplers instead of the steerable one:
    device time of one call, median of reps."""
    import torch
    import pg3render_gb300 as P
    R = P.renderer
    sc = build_scene()
    out = {"metric": "Msamples/s per environment-map sampler (headline workload)"}
    for name, em in (("cdf", R.EM_CDF), ("cosine", R.EM_COSINE)):
        cfg = P.Config(scene=sc, max_path_length=MAX_PATH, rr_min_path_length=RR_FROM, em_sampler=em)
        with P.GpuPathTracer(cfg) as r:
            r.RunIteration(R.kPathTracing, 0, SPP)
            r.synchronize()
            ts = []
            for rep in range(reps):
                a, b = _events()
                a.record()
                r.RunIteration(R.kPathTracing, (rep + 1) * SPP, SPP)
                b.record()
                torch.cuda.synchronize()
                ts.append(a.elapsed_time(b))
        out[name] = {"msamples_per_s": round(WIDTH * HEIGHT * SPP / statistics.median(ts) / 1e3, 1)}
    return out


def sampler_comparison(line):
    """Equal-quality speedups per sampler from the bench line's parts: each GPU sampler's
    Msamples/s and relative MSE at the benchmark's samples per pixel against the reference's CPU
    renderer with the same sampler (steerable, CDF) and with the configured steerable sampler."""
    cb = line.get("cpu_baseline", {})
    mq = cb.get("matched_quality", {})
    last = mq.get("rel_mse_at_%dspp" % SPP, {})
    sec = line.get("secondary", {})
    gpu = {"steerable": line["value"],
           "steerable_adaptive": sec.get("adaptive_sampler", {}).get("msamples_per_s"),
           "cdf": sec.get("samplers", {}).get("cdf", {}).get("msamples_per_s"),
           "cosine": sec.get("samplers", {}).get("cosine", {}).get("msamples_per_s")}
    mse = {"steerable": last.get("gpu_steerable_" + line["config"].get("steer_weights", "projected")),
           "steerable_adaptive": last.get("gpu_steerable_adaptive_projected"),
           "cdf": last.get("gpu_cdf"), "cosine": last.get("gpu_cosine")}
    cpu = {"steerable": (cb.get("value"), last.get("cpu_reference_steerable")),
           "cdf": (cb.get("cdf_value"), last.get("cpu_reference_cdf"))}
    out = {"gpu_msamples_per_s": gpu, "gpu_rel_mse": mse,
           "cpu_msamples_per_s": {k: v[0] for k, v in cpu.items()},
           "cpu_rel_mse": {k: v[1] for k, v in cpu.items()},
           "equal_quality_speedup": {}}
    for g in gpu:
        for c in cpu:
            if gpu[g] and mse[g] and cpu[c][0] and cpu[c][1]:
                out["equal_quality_speedup"]["gpu_%s_vs_cpu_%s" % (g, c)] = round(
                    gpu[g] / cpu[c][0] * cpu[c][1] / mse[g], 1)
    return out


def secondary_metrics(only=None):
    out = {}
    for name, fn in (("batched", batched_metric), ("differentiable", differentiable_metric),
                     ("inverse_rendering", inverse_metric), ("mesh_bvh", mesh_metric),
                     ("per_iteration", per_iteration_metric), ("adaptive_sampler", adaptive_sampler_metric),
                     ("samplers", sampler_metric)):
        if only and name != only:
            continue
        try:
            out[name] = fn()
        except Exception as e:   # reported, never hidden
            out[name] = {"error": "%s: %s" % (type(e).__name__, e)}
    return out


# ----------------------------------------------------------------------------- reference arm
def run_reference(args, rank, world):
    if rank != 0:
        return None
    scene = build_scene()
    sampler = args.sampler if args.sampler != "auto" else "steerable"
    threads = os.cpu_count() or 1
    for _ in range(max(0, args.warmup)):
        cpu_baseline(scene, sampler, threads=threads)
    vals, secs = [], []
    last = None
    for _ in range(args.steps):
        t0 = time.perf_counter()
        last = cpu_baseline(scene, sampler, threads=threads)
        secs.append(time.perf_counter() - t0)
        vals.append(last["value"])
    value = statistics.mean(vals)
    cb = dict(last)
    cb["value"] = round(value, 4)
    return {"impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * statistics.mean(secs), 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "cornell_env_%dx%d_%dspp_maxpl12_rr3_em1024x512_%s" % (WIDTH, HEIGHT, SPP, sampler),
                       "width": WIDTH, "height": HEIGHT, "em_sampler": sampler,
                       "step": "bounded sample: one iteration per host thread"},
            "cpu_baseline": cb,
            "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        line = run_reference(args, rank, world)
    elif args.only_secondary:
        line = secondary_metrics(args.only_secondary) if rank == 0 else None
    else:
        if world > 1:
            import torch
            torch.cuda.set_device(local_rank)
            torch.distributed.init_process_group("nccl")
        line = run_gpu(args, rank, world, local_rank)
        if world > 1:
            import torch
            torch.distributed.destroy_process_group()
    if line is not None:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
