"""Benchmark: Mrays/s of the path tracer on the large single-mesh workload.

Workload (one GPU): a displaced icosphere of 1,310,720 triangles (level-8
subdivision, seeded 6-octave value noise of amplitude 0.08 r, dielectric
n = 1.5) inside the Cornell box, 1024 x 1024 pixels, 8 bounces, compat
estimator.  One step = one progressive launch of 16 samples per pixel over
the whole frame (16 steps = the 256-spp frame), inputs resident in HBM.

Metric: rays actually traced (primary + bounce + shadow) per second of
device time, in millions.  Multi-GPU: each rank renders its own disjoint
range of sample indices of the same frame (weak scaling, no collective on
the data path; a barrier and a max-reduce of the time only).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

The line also carries `quality`: the equal-time relMSE of MLP-guided vs
plain sampling on the hard-indirect scene (1024 x 1024, 256 spp, physically
based estimator) against a 4,096-spp FP64 reference, measured in the same
run after the timed region; and `optix`: the reference's own OptiX render
(baseline/optix_harness.cc, the reference's shader.cu and OptiX set-up) of
the same workload on the same GPU, 16 spp per launch.

--impl reference times the reference's own estimator code on the host
cores: src/LiSA/src/shader.cu compiled for the CPU (oracle/ref_shader_run.cc,
closest hits from the oracle's CPU BVH) on all host threads, on a bounded
sample of the same workload; where it was not built, the oracle's
restatement of it.  --impl optix prints the OptiX render's own line.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = ("displaced icosphere 1,310,720 tris (dielectric n=1.5) in Cornell box, 1024x1024, 8 bounces, "
            "16 spp per step (256-spp frame = 16 steps), compat estimator")
METRIC = "Mrays/s (primary+bounce+shadow rays of the reference estimator, counted as its shader.cu traces them)"


def dist_init(gpus: int):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return rank, ws, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, ws: int) -> float:
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x: float, ws: int) -> float:
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for k, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(k)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_bf16(sustained=True):
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["bf16_tflops_sustained" if sustained else "bf16_tflops"]), "of measured"
    except (OSError, KeyError, ValueError):
        return (1700.0 if sustained else 1900.0), "of fallback"


# guide network FLOPs per sample (N = 40 outputs, unpadded): forward
# 2*(4*64*64 + 64*40); a training sample runs the forward pass and the
# backward pass (twice the forward's products)
MLP_FWD_FLOP = 2 * (4 * 64 * 64 + 64 * 40)
MLP_TRAIN_FLOP = 3 * MLP_FWD_FLOP


def mlp_roofline(guided_row):
    """Tensor-pipe roofline of the guide's kernels inside the guided render:
    inference (k_guided_infer: the network on every emitter-queue entry of a
    guided depth, fused with the guided bounce) and training (sample
    collection, then k_guide_train_rounds: every Adam round of a wave in one
    cooperative launch), from the renderer's stage timers and
    its work counters, against the sustained bf16 peak (the kernels run
    inside a long render)."""
    peak, kind = measured_peak_bf16(sustained=True)
    out = {}
    for key, unit_key, flop in (("guide_infer", "rows", MLP_FWD_FLOP), ("guide_train", "samples", MLP_TRAIN_FLOP)):
        g = guided_row.get(key) or {}
        ms, units = g.get("ms", 0.0), g.get(unit_key, 0)
        tf = units * flop / (ms * 1e-3) / 1e12 if ms > 0 else 0.0
        out[key] = {"bound": "tensor", "achieved": tf, "peak": peak, "unit": "TFLOP/s", "frac": tf / peak,
                    "peak_kind": kind, unit_key: units, "ms": ms, "flop_per_unit": flop}
    return out


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "of measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "of fallback"


TRAFFIC_FILE = os.path.join("profiles", "dram_traffic_icosphere1310k_1024px.md")


def profile_traffic():
    """DRAM bytes per unit of the path's kernels, measured by ncu on this
    workload (the committed summary's key = value lines), or {}."""
    try:
        kv = {}
        with open(os.path.join(ROOT, TRAFFIC_FILE)) as f:
            for ln in f:
                k, sep, v = ln.partition(" = ")
                if not sep or " " in k.strip() or not k.strip().startswith("k_"):
                    continue
                v = v.strip()
                try:
                    kv[k.strip()] = float(v)
                except ValueError:
                    kv[k.strip()] = v
        return kv
    except OSError:
        return {}


def make_scene(level=8, res=1024):
    from lisa_gb300 import scenes

    return scenes.icosphere_box(level=level, width=res, height=res, num_samples=256, num_bounces=8)


# Algorithmic bytes.  Closest-hit kernel (k_trace), per radiance ray: the
# queued ray read (32 B) and its hit written (8 B); per node visit 80 B; per
# triangle test 48 B.  Emitter-search kernel (k_nee), per opaque vertex: the
# queue entry (48 B) + path state read and written back (36 + 36 B) + the
# continuation ray (32 B); per shadow ray that walks a BVH the material
# look-up of its hit (16 B); node visits and triangle tests as above.  (A try
# that cannot change the search's result moves no bytes.)
TRACE_B_RAY = 32 + 8
NEE_B_VERTEX = 48 + 36 + 36 + 32
NEE_B_RAY = 16
B_NODE = 80
B_TRI = 48


def kernel_roofline(name, ms_total, launches, bytes_step, launches_counted, peak, peak_kind, dram_per_unit,
                    units_step, limiter, extra):
    """HBM roofline of one kernel: algorithmic bytes per launch (the counting
    pass's per-step counts x the per-unit bytes, over its launches) over the
    kernel's average CUDA-event launch time; traffic = ncu's DRAM bytes per
    unit on this workload x the units of a launch (a measured rate scaled to
    the launch, not a capture of this run)."""
    bytes_launch = bytes_step / max(launches_counted, 1)
    avg_s = ms_total / 1e3 / max(launches, 1)
    achieved = bytes_launch / avg_s / 1e9 if avg_s > 0 else 0.0
    traffic = None if dram_per_unit is None else dram_per_unit * units_step / max(launches_counted, 1)
    out = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
           "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
           "traffic_kind": "ncu DRAM bytes per unit on this workload, scaled to a launch",
           "dram_gbs_from_traffic": (traffic / avg_s / 1e9) if (traffic and avg_s > 0) else None,
           "limiter": limiter, "bytes_per_launch": bytes_launch, "avg_launch_ms": avg_s * 1e3,
           "ms_in_timed_region": ms_total}
    out.update(extra)
    return out


def cpu_sample(scene, spp, budget_s=12.0, threads=0, seed=0):
    """Time the CPU oracle on a bounded sample of the workload: bands of
    pixels spread over the frame, `spp` samples each.  Returns (Mrays/s,
    description, cores)."""
    import oracle as O

    osc = O.Scene.from_scene(scene, spp=spp, seed=seed)
    osc.render(0, 1, use_bvh=True, threads=threads)  # builds the CPU BVH once
    w, h = scene.width, scene.height
    cores = threads or os.cpu_count()
    npx = 64
    rays_tot, t_tot, px_tot = 0, 0.0, 0
    bands = 0
    for y in np.linspace(0, h - 1, 64).astype(int).tolist():
        x0 = (bands * 97) % (w - npx)
        p0 = y * w + x0
        t0 = time.perf_counter()
        _, _, rays = osc.render(p0, p0 + npx, use_bvh=True, threads=threads)
        t_tot += time.perf_counter() - t0
        rays_tot += int(rays.sum())
        px_tot += npx
        bands += 1
        if t_tot > budget_s:
            break
    return (rays_tot / max(t_tot, 1e-9) / 1e6,
            f"{px_tot} pixels in {bands} bands x {spp} spp of the same frame (CPU BVH built once, not timed)", cores)


REF_SHADER = os.path.join(ROOT, "oracle", "_ref", "ref_shader_run")


class RefShaderSample:
    """The reference's own estimator (shader.cu compiled for the host,
    oracle/ref_shader_run.cc) timed on a sample of the workload: 64 rows
    spread over the frame, 64 pixels of each, on all host threads.  The scene
    is written once as a raw soup; the CPU BVH is built outside the timed
    region."""

    def __init__(self, scene, rows=64, band=64, threads=0):
        import tempfile

        sys.path.insert(0, os.path.join(ROOT, "baseline"))
        import optix_run

        self.dir = tempfile.TemporaryDirectory()
        self.path = os.path.join(self.dir.name, "scene.soup")
        optix_run.write_soup(scene, self.path)
        self.rows, self.band, self.threads = rows, band, threads

    def __call__(self, spp):
        cmd = [REF_SHADER, "--soup", self.path, "--spp", str(spp), "--rows", str(self.rows), "--band",
               str(self.band)]
        if self.threads:
            cmd += ["--threads", str(self.threads)]
        d = json.loads(subprocess.run(cmd, capture_output=True, text=True, check=True).stdout.strip().splitlines()[-1])
        rays = d["rays_radiance"] + d["rays_occlusion"]
        desc = (f"{d['pixels']} pixels ({self.rows} rows x {self.band}) x {spp} spp of the same frame; the "
                f"reference's shader.cu compiled for the host, every trace counted (CPU BVH built once, not timed)")
        return rays / d["seconds"] / 1e6, desc, d["threads"]


def cpu_reference(scene, spp, steps=1, seed=0, budget_s=12.0):
    """(Mrays/s per step, description, cores, kind) of the CPU baseline:
    the reference's own estimator code where it was built, else the oracle's
    restatement."""
    if os.path.exists(REF_SHADER):
        run = RefShaderSample(scene)
        out = [run(spp) for _ in range(steps)]
        return [o[0] for o in out], out[-1][1], out[-1][2], "reference"
    vals = []
    for i in range(steps):
        v, desc, cores = cpu_sample(scene, spp=spp, budget_s=budget_s, seed=seed + i)
        vals.append(v)
    return vals, desc, cores, "port"


def optix_reference(scene, spp, warmup=2, reps=5):
    """The reference's OptiX render of `scene` on this GPU
    (baseline/optix_harness.cc), or {"unavailable": why}."""
    sys.path.insert(0, os.path.join(ROOT, "baseline"))
    import optix_run

    why = optix_run.available()
    if why:
        return {"unavailable": why}
    try:
        r = optix_run.run(scene, spp=spp, warmup=warmup, reps=reps, count=True)
    except Exception as e:  # noqa: BLE001 - reported, not fatal to our own line
        return {"unavailable": f"OptiX harness failed: {str(e)[-300:]}"}
    return {"value": r["mrays_per_s"], "unit": "Mrays/s", "ms_per_launch": r["ms_per_launch"],
            "rays_per_launch": r["rays"], "rays_radiance": r["rays_radiance"], "rays_occlusion": r["rays_occlusion"],
            "spp_per_launch": r["spp"], "launches_timed": r["reps"],
            "what": "the reference's own OptiX pipeline (optix_wrapper.cc set-up, shader.cu compiled with its "
                    "--use_fast_math flags), one optixLaunch of width x height per step, CUDA events on its "
                    "stream; rays counted by an instrumented copy of shader.cu in a separate untimed launch"}


def soup_leg(args, local, spp=4, steps=3):
    """The triangle-soup stress workload: 20,000 UV spheres of 16 x 8
    segments (224 triangles each: the pole rows are triangles; 4,480,000 in
    all), 10 % emissive, in a 100^3 box; 1920 x 1080, 12 bounces, reference
    estimator; `spp` samples per step, L2 flushed before each step.  Also the
    reference's OptiX render of the same scene where it runs."""
    import torch

    import lisa_gb300 as L
    from lisa_gb300 import scenes

    sc = scenes.sphere_soup()
    r = L.Renderer(L.params_from_scene(sc), L.default_options(stage_timing=1))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    stats = []
    for i in range(steps + 1):
        flush.zero_()
        torch.cuda.synchronize()
        st = r.render_progressive(spp)
        if i:
            stats.append(st)
    ms = sum(s.ms_device for s in stats) / len(stats)
    rays = sum(s.rays for s in stats) / len(stats)
    out = {"workload": "20,000 UV spheres 16x8 (224 tris each, 4,480,000 tris, 20,000 materials, 10% emissive) in a "
                       "100^3 box, 1920x1080, 12 bounces, compat estimator",
           "spp_per_step": spp, "steps": steps, "value": rays / ms / 1e3, "unit": "Mrays/s", "ms_per_step": ms,
           "rays_per_step": rays,
           "shadow_traversals_per_step": sum(s.shadow_traversals for s in stats) / len(stats),
           "stages_ms_per_step": {"trace": sum(s.ms_trace for s in stats) / len(stats),
                                  "shade": sum(s.ms_shade for s in stats) / len(stats),
                                  "nee": sum(s.ms_nee for s in stats) / len(stats)},
           "bvh": r.bvh_info()}
    r.close()
    del flush
    if not args.no_optix:
        o = optix_reference(sc, spp, warmup=1, reps=steps)
        out["optix"] = o
        if "ms_per_launch" in o:
            out["optix"]["time_over_ours"] = o["ms_per_launch"] / ms
    return out


def run_reference(args, rank, ws):
    if rank != 0:
        return
    sc = make_scene(res=args.res)
    vals, desc, cores, kind = cpu_reference(sc, args.spp_per_step, steps=args.warmup + args.steps,
                                            budget_s=args.ref_budget)
    value = float(np.mean(vals[args.warmup:]))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "l2": "host-side run"},
            "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": cores, "kind": kind, "sample": desc},
            "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_optix(args, rank, ws):
    if rank != 0:
        return
    sc = make_scene(res=args.res)
    o = optix_reference(sc, args.spp_per_step, warmup=args.warmup, reps=args.steps)
    if "unavailable" in o:
        print(json.dumps({"impl": "optix", "unavailable": o["unavailable"]}), flush=True)
        return
    line = {"impl": "optix", "metric": METRIC, "value": o["value"], "unit": "Mrays/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": o["ms_per_launch"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": {"workload": WORKLOAD}, "optix": o}
    print(json.dumps(line), flush=True)


def run_ours(args, rank, ws, local):
    import torch

    import lisa_gb300 as L

    sc = make_scene(res=args.res)
    params = L.params_from_scene(sc)
    # each rank renders its own range of sample indices of the frame
    # (lisa_gb300.shard); one rank renders samples 0, 1, 2, ...
    shard_first = rank * (1 << 20)
    # queue and block sizes from the autotuner (short renders of this
    # workload, before and outside the timed region)
    tuning = None
    base = L.default_options(paths_in_flight=args.paths)
    if not args.no_tune:
        import tempfile

        with tempfile.TemporaryDirectory() as td:
            tuning = L.autotune(params, base, cache=os.path.join(td, "tune.json"))
        base = L.apply_tuning(tuning, base)
    tuned = {k: getattr(base, k) for k in ("paths_in_flight", "threads_per_block", "blocks_per_sm", "refill_idle")}
    opts = L.default_options(stage_timing=1, **tuned)
    r = L.Renderer(params, opts)
    r.set_sample_offset(shard_first)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    def step():
        flush.zero_()
        torch.cuda.synchronize()
        return r.render_progressive(args.spp_per_step)

    for _ in range(args.warmup):
        step()
    barrier(ws)
    torch.cuda.synchronize()
    clk = ClockSampler(local)
    clk.start()
    t0 = time.perf_counter()
    stats = [step() for _ in range(args.steps)]
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clocks = clk.stop()
    barrier(ws)
    dev_s = sum(s.ms_device for s in stats) / 1e3
    rays = sum(s.rays for s in stats)
    t_max = max_over_ranks(dev_s, ws)
    rays_all = sum_over_ranks(float(rays), ws)
    value = rays_all / t_max / 1e6
    # dominant kernel: the emitter search (k_nee); per-launch device time
    nee_ms = sum(s.ms_nee for s in stats)
    nee_launches = sum(s.launches_nee for s in stats)
    trace_ms = sum(s.ms_trace for s in stats)
    shade_ms = sum(s.ms_shade for s in stats)
    other_ms = sum(s.ms_other for s in stats)
    launches = sum(s.launches_total for s in stats)
    # counting pass (same seeds, one step) for the algorithmic bytes per launch
    copts = L.default_options(count_traversal=1, **tuned)
    rc = L.Renderer(params, copts)
    rc.set_sample_offset(shard_first)
    cs = rc.render_progressive(args.spp_per_step)
    peak, peak_kind = measured_peak_hbm()
    dram = profile_traffic()
    radiance = cs.rays_primary + cs.rays_bounce
    kernels = {
        "k_trace": kernel_roofline(
            "k_trace (closest hit of radiance rays)", trace_ms, sum(s.launches_trace for s in stats),
            radiance * TRACE_B_RAY + cs.node_visits_trace * B_NODE + cs.tri_tests_trace * B_TRI,
            cs.launches_trace, peak, peak_kind, dram.get("k_trace_dram_bytes_per_ray"), radiance,
            dram.get("k_trace_limiter"),
            {"per_unit": {"ray_B": TRACE_B_RAY, "node_B": B_NODE, "tri_B": B_TRI},
             "counts_per_step": {"rays": radiance, "node_visits": cs.node_visits_trace,
                                 "tri_tests": cs.tri_tests_trace}}),
        "k_nee": kernel_roofline(
            "k_nee (30-try emitter search + bounce)", nee_ms, nee_launches,
            cs.nee_vertices * NEE_B_VERTEX + cs.shadow_traversals * NEE_B_RAY + cs.node_visits_nee * B_NODE +
            cs.tri_tests_nee * B_TRI, cs.launches_nee, peak, peak_kind,
            dram.get("k_nee_dram_bytes_per_vertex"), cs.nee_vertices, dram.get("k_nee_limiter"),
            {"per_unit": {"vertex_B": NEE_B_VERTEX, "walked_shadow_ray_B": NEE_B_RAY, "node_B": B_NODE,
                          "tri_B": B_TRI},
             "counts_per_step": {"nee_vertices": cs.nee_vertices, "shadow_rays": cs.rays_shadow,
                                 "shadow_traversals": cs.shadow_traversals, "node_visits": cs.node_visits_nee,
                                 "tri_tests": cs.tri_tests_nee}}),
    }
    dominant = max(kernels, key=lambda k: kernels[k]["ms_in_timed_region"])
    rc.close()
    del rc
    # end to end through the C ABI with host buffers: upload + BVH build +
    # render + image read-back, per step
    v, n, mi = sc.soup()
    mats = sc.material_table()
    h2d = v.nbytes + n.nbytes + mi.nbytes + 40 * mats.shape[0]
    d2h = sc.width * sc.height * 3 * 4
    e2e_steps = 0 if args.quick else max(2, min(args.steps, 4))
    e2e_rays, e2e_t = 0, 0.0
    for i in range(e2e_steps + 1 if e2e_steps else 0):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        p2 = L.params_from_arrays(v, n, mi, mats, sc.width, sc.height, sc.eye, sc.look_at, sc.fov, 256, 8)
        r2 = L.Renderer(p2, L.default_options(**tuned))
        r2.set_sample_offset(shard_first + (i + 1) * 4096)
        s2 = r2.render_progressive(args.spp_per_step)
        img = r2.image()
        r2.close()
        dt = time.perf_counter() - t0
        if i > 0:  # first one warms the allocator
            e2e_rays += s2.rays
            e2e_t += dt
    e2e_val = sum_over_ranks(float(e2e_rays), ws) / max(max_over_ranks(e2e_t, ws), 1e-9) / 1e6
    info = r.bvh_info()
    # equal-time relMSE of guided vs plain sampling (hard-indirect scene,
    # 1024x1024, 256 spp, physically based estimator) against a 4,096-spp
    # FP64 reference whose own variance is removed from the figures
    quality = None
    if rank == 0 and not (args.quick or args.no_quality):
        from lisa_gb300 import study

        qa = argparse.Namespace(res=1024, level=8, spp=256, ref_spp=4096, ref_chunk=256, estimator="physical")
        q = study.hard_indirect(qa)[0]
        quality = {"workload": "hard-indirect scene (C2 mesh, 0.02 light behind a baffle), 1024x1024, 256 spp, "
                               "physically based estimator",
                   "reference": "4096 spp plain, FP64 accumulation; relMSE with its variance removed",
                   "relmse_plain": q["plain"]["relmse_corrected"], "relmse_guided": q["guided"]["relmse_corrected"],
                   "ms_plain": q["plain"]["ms"], "ms_guided": q["guided"]["ms"],
                   "equal_time_relmse_guided_over_plain": q["equal_time_relmse"]["guided"] / q["equal_time_relmse"]["plain"],
                   "guided_time_to_plain_error": q["time_to_plain_error"],
                   "mlp": mlp_roofline(q["guided"])}
    soup = None
    if rank == 0 and not (args.quick or args.no_soup):
        soup = soup_leg(args, local)
    cpu = None
    if rank == 0 and not (args.no_cpu or args.quick):
        cv, cdesc, ccores, ckind = cpu_reference(sc, args.spp_per_step, steps=1, budget_s=args.cpu_budget)
        cpu = {"value": cv[0], "unit": "Mrays/s", "cores": ccores, "kind": ckind, "sample": cdesc}
    optix = None
    if rank == 0 and not (args.quick or args.no_optix):
        optix = optix_reference(sc, args.spp_per_step)
        if "value" in optix:
            optix["plain_over_optix"] = value / optix["value"]
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "triangles": sc.num_triangles, "width": sc.width,
                       "height": sc.height, "spp_per_step": args.spp_per_step, "bounces": sc.num_bounces,
                       "paths_in_flight": r.options.paths_in_flight or None,
                       "tuning": None if tuning is None else {**tuned, "candidates": tuning.candidates,
                                                               "probe_mrays_per_s": tuning.mrays_per_s},
                       "l2": "working set > L2 (BVH+triangles+queues) and a 256 MB L2 flush before every step",
                       "bvh": info, "sharding": "disjoint sample ranges per rank"},
            "roofline": kernels[dominant],
            "kernels": kernels,
            "rays_traversed_per_step": (cs.rays_primary + cs.rays_bounce + cs.shadow_traversals),
            "stages_ms_per_step": {"trace": trace_ms / args.steps, "shade": shade_ms / args.steps,
                                   "nee": nee_ms / args.steps, "other": other_ms / args.steps},
            "rays_per_step": rays / args.steps,
            "traversal_per_ray": {
                "shadow": {"nodes": cs.node_visits_nee / max(cs.rays_shadow, 1),
                           "tris": cs.tri_tests_nee / max(cs.rays_shadow, 1)},
                "radiance": {"nodes": cs.node_visits_trace / max(cs.rays_primary + cs.rays_bounce, 1),
                             "tris": cs.tri_tests_trace / max(cs.rays_primary + cs.rays_bounce, 1)}},
            "wall_s": wall,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_val, "unit": "Mrays/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h),
                    "what": "Renderer create (H2D soup + GPU BVH build) + 16-spp render + FP32 image D2H"},
            "clocks": clocks,
            "gpu_launches": int(launches),
            "quality": quality,
            "optix": optix,
            "soup": soup,
        }
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference", "optix"])
    ap.add_argument("--spp-per-step", type=int, default=16)
    ap.add_argument("--paths", type=int, default=0, help="paths in flight (0 = library default)")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--ref-budget", type=float, default=6.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--res", type=int, default=1024, help="square resolution (profiling cases use less)")
    ap.add_argument("--quick", action="store_true", help="skip the CPU baseline, the end-to-end leg and the quality leg")
    ap.add_argument("--no-quality", action="store_true", help="skip the guided-vs-plain relMSE leg")
    ap.add_argument("--no-optix", action="store_true", help="skip the reference's OptiX render leg")
    ap.add_argument("--no-soup", action="store_true", help="skip the triangle-soup stress leg")
    ap.add_argument("--no-tune", action="store_true", help="library default queue and block sizes")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, ws, local = dist_init(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, ws)
    elif args.impl == "optix":
        run_optix(args, rank, ws)
    else:
        run_ours(args, rank, ws, local)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
