#!/usr/bin/env python
"""Headline benchmark: Msamples/s (and Grays/s) of the GB300 wavefront path tracer on the
1M-triangle soup, 1920x1080, 64 spp, path length 8, NEE + Russian roulette from depth 3.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gbpt|reference]

A step is one frame (1920*1080*64 path samples) rendered through the C ABI. `value` times
gbpt_render_device with the scene and output resident in HBM; `e2e` times gbpt_render, which
copies the frame's result to pinned host memory inside the call. Under torchrun every rank renders
its own frame (frame seed = rank, weak scaling, no collective on the data path); the timing is the
max over ranks. `--impl reference` times the CPU restatement of merian's `pt` (oracle/, FP32,
every host thread) on the same workload, since the reference's Vulkan/Slang path cannot run here.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Msamples/s and Grays/s at equal RMSE vs FP64; served p50/p99 latency, 1 GB300"
WORKLOAD = "soup-1m-1080p-64spp"
L2_FLUSH_BYTES = 256 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=None)
    ap.add_argument("--impl", default="gbpt", choices=["gbpt", "reference"])
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--tuning", default=None,
                    help="WAVE_PATHS,SORT[,STREAMS[,REFILL,POSTPONE,BLOCKS_PER_SM]]: a fixed "
                         "schedule instead of the autotuner's (0 = default)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default schedule instead of gbpt_autotune's choice of tick "
                         "size and material sorting (made before the warm-up, untimed)")
    # the mixed workloads (--workload batch-256 | served-stream)
    ap.add_argument("--scenes", type=int, default=None, help="scenes of a mixed workload")
    ap.add_argument("--requests", type=int, default=None,
                    help="requests per served rate (served-stream 96, served-small 512)")
    ap.add_argument("--rates", default=None,
                    help="served arrival rates, req/s (served-stream 50,200,2000; served-small "
                         "2000,10000,50000)")
    return ap.parse_args()


def dist_info():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)),
            int(os.environ.get("WORLD_SIZE", 1)))


def rank_max(values, world):
    """Each value's maximum over the ranks (host all_reduce over the process group): the timing
    rule for N > 1. Identity for one rank."""
    if world <= 1:
        return [float(v) for v in values]
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v) for v in values], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t]


def whole_job(world, units_per_rank, ms):
    """Millions of units per second of the whole job: every rank's units over the slowest
    rank's time (replicas with fixed work per rank: weak scaling)."""
    return world * units_per_rank / (ms / 1e3) / 1e6


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic_per_ray():
    """DRAM bytes per closest-hit ray from the committed ncu summary of the traversal kernel."""
    for f in sorted((ROOT / "profiles").glob("*.md")):
        m = re.search(r"dram_bytes_per_ray:\s*([0-9.eE+-]+)", f.read_text())
        if m:
            return float(m.group(1)), f.name
    return None, None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self.t = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.t:
                self.t.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def host_threads() -> int:
    """Every host thread this process may run on (torchrun's OMP_NUM_THREADS=1 is overridden:
    the CPU legs use the whole host)."""
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_baseline(scene, camera, w, cpu_seconds: float, kind_label: str = "port"):
    """FP32 oracle on every host thread, on a bounded pixel sample of the same workload."""
    from merian_gb300 import scene as S
    from oracle import binding as O
    osc = O.OracleScene(scene)
    rng = np.random.default_rng(0xC0FFEE)
    n_total = w["width"] * w["height"]
    probe = np.sort(rng.choice(n_total, 32, replace=False)).astype(np.uint32)
    p, keep = S.render_params(w["width"], w["height"], w["spp"], w["max_path_length"],
                              pixels=probe, nee=w["nee"], rr_depth=w["rr_depth"], frame=0)
    t0 = time.perf_counter()
    osc.render(camera, p, fp64=False, threads=host_threads())
    dt = time.perf_counter() - t0
    n_px = int(min(n_total, max(32, 32 * cpu_seconds / max(dt, 1e-3))))
    pix = np.sort(rng.choice(n_total, n_px, replace=False)).astype(np.uint32)
    p, keep = S.render_params(w["width"], w["height"], w["spp"], w["max_path_length"],
                              pixels=pix, nee=w["nee"], rr_depth=w["rr_depth"], frame=0)
    t0 = time.perf_counter()
    _, _, rays = osc.render(camera, p, fp64=False, threads=host_threads())
    dt = time.perf_counter() - t0
    samples = n_px * w["spp"]
    threads = O.num_threads()
    osc.close()
    return {"value": round(samples / dt / 1e6, 4), "unit": "Msamples/s", "cores": threads,
            "kind": kind_label,
            "sample": f"{n_px} random pixels x {w['spp']} spp of the same frame "
                      f"({samples} samples, {rays} rays, {dt:.1f} s, FP32 oracle, "
                      f"{threads} threads)",
            "grays_per_s": round(rays / dt / 1e9, 6)}


def cwbvh_walk_sample(scene, camera, w, frac: float = 0.01):
    """CWBVH nodes visited and triangles tested per closest-hit bounce ray, from a host walk
    (the oracle's restatement of the device traversal) of the same tree the device traverses
    (gbpt_bvh_build), over the bounce rays the FP32 oracle traces for a seeded `frac` of the
    frame's pixels at the workload's spp and estimator."""
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    from oracle import binding as O
    t0 = time.perf_counter()
    nodes, tris, _ = S.build_bvh(scene)
    osc = O.OracleScene(scene)
    n_total = w["width"] * w["height"]
    rng = np.random.default_rng(0x5EED)
    pix = np.sort(rng.choice(n_total, max(1, int(n_total * frac)), replace=False)).astype(np.uint32)
    p, keep = S.render_params(w["width"], w["height"], w["spp"], w["max_path_length"],
                              pixels=pix, nee=w["nee"], rr_depth=w["rr_depth"], frame=0)
    rays = O.bounce_rays(osc, camera, p, N.RAY_DTYPE)
    _, counts = O.cwbvh_trace(nodes, tris, rays, hit_dtype=N.HIT_DTYPE)
    osc.close()
    return {"nodes_per_ray": float(counts[:, 0].mean()), "tris_per_ray": float(counts[:, 1].mean()),
            "rays": int(len(rays)), "pixels": int(len(pix)),
            "seconds": round(time.perf_counter() - t0, 1)}


def parity_vs_fixtures(ctx, sid, cam, w):
    """Relative RMSE of the GPU estimate (headline estimator: NEE + roulette) against the FP64
    oracle fixtures of this workload (tests/golden, BSDF-only estimator: the reference's), on the
    fixtures' seeded pixels, untimed:
      * frame: one frame at the workload's spp on the 1,024 pixels of soup_1m.npz (65,536 spp);
      * converged: the 64 pixels of soup_1m_deep.npz (2^22 spp each) at the same 2^22 spp.
    `oracle_noise` is the relative RMSE the fixture's own sampling noise explains; relative RMSE
    is RMSE over the pixels' rgb divided by the fixture's mean."""
    from merian_gb300 import scene as S
    out = {}
    gold = ROOT / "tests" / "golden"
    for key, fname, spp, frame in (("frame", "soup_1m.npz", w["spp"], 777),
                                   ("converged", "soup_1m_deep.npz", None, 778)):
        f = gold / fname
        if not f.exists():
            continue
        g = np.load(f)
        pix = g["pixels"].astype(np.uint32)
        n_spp = int(g["spp"]) if spp is None else spp
        p, keep = S.render_params(int(g["width"]), int(g["height"]), n_spp,
                                  int(g["max_path_length"]), pixels=pix, nee=w["nee"],
                                  rr_depth=w["rr_depth"], frame=frame)
        est = ctx.render(sid, cam, p)[:, :3].astype(np.float64)
        scale = float(np.mean(g["mean"]))
        out[key] = {"fixture": fname, "pixels": int(len(pix)), "spp": n_spp,
                    "fixture_spp": int(g["spp"]),
                    "rel_rmse": round(float(np.sqrt(np.mean((est - g["mean"]) ** 2)) / scale), 5),
                    "oracle_noise": round(float(np.sqrt(np.mean(g["var"] / int(g["spp"])))
                                                / scale), 5)}
    return out


def tuning_dict(t) -> dict:
    """The schedule a gbpt_tuning selects, as reported in config.tuning (0 = default)."""
    return {"wave_paths": t.wave_paths, "sort_materials": t.sort_materials,
            "streams": t.streams or 2, "trace_refill_lanes": t.trace_refill_lanes or 20,
            "trace_postpone_lanes": t.trace_postpone_lanes or 6,
            "trace_blocks_per_sm": t.trace_blocks_per_sm or "all resident"}


def build_workload(name):
    from merian_gb300 import scene as S
    w = S.WORKLOADS[name]
    sc = S.workload_scene(name)
    cam = S.workload_camera(name)
    return w, sc, cam


def run_reference(args):
    rank, _, world = dist_info()
    if rank != 0:
        return
    from oracle import binding as O
    from merian_gb300 import scene as S
    # the scene and camera come from the oracle library (its own camera basis and the seeded
    # generators compiled into it): this arm maps no CUDA library of the package
    w = S.WORKLOADS[args.workload]
    sc = S.workload_scene(args.workload, lib=O.generator())
    cam = O.workload_camera(args.workload)
    osc = O.OracleScene(sc)
    n_total = w["width"] * w["height"]
    rng = np.random.default_rng(7)
    # size one step as a bounded sample: ~ cpu_seconds / (steps + warmup) of CPU work each
    probe = np.sort(rng.choice(n_total, 16, replace=False)).astype(np.uint32)
    p, keep = S.render_params(w["width"], w["height"], w["spp"], w["max_path_length"],
                              pixels=probe, nee=w["nee"], rr_depth=w["rr_depth"])
    t0 = time.perf_counter()
    osc.render(cam, p, fp64=False, threads=host_threads())
    per_px = (time.perf_counter() - t0) / 16
    # about 4 x --cpu-seconds of CPU work over the whole run (60 s by default)
    budget = max(0.5, 4.0 * args.cpu_seconds / max(1, args.steps + args.warmup))
    n_px = int(min(n_total, max(16, budget / max(per_px, 1e-6))))
    times, rays_total = [], 0
    for i in range(args.warmup + args.steps):
        pix = np.sort(rng.choice(n_total, n_px, replace=False)).astype(np.uint32)
        p, keep = S.render_params(w["width"], w["height"], w["spp"], w["max_path_length"],
                                  pixels=pix, nee=w["nee"], rr_depth=w["rr_depth"], frame=i)
        t0 = time.perf_counter()
        _, _, rays = osc.render(cam, p, fp64=False, threads=host_threads())
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(dt)
            rays_total += rays
    samples = n_px * w["spp"]
    ms = 1e3 * float(np.mean(times))
    value = samples / (ms / 1e3) / 1e6
    threads = O.num_threads()
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "Msamples/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.workload, "triangles": sc.triangle_count,
                   "width": w["width"], "height": w["height"], "spp": w["spp"],
                   "max_path_length": w["max_path_length"], "nee": w["nee"],
                   "rr_depth": w["rr_depth"], "step": f"{n_px} random pixels x {w['spp']} spp"},
        "grays_per_s": round(rays_total / sum(times) / 1e9, 6),
        "cpu_baseline": {"value": round(value, 4), "unit": "Msamples/s", "cores": threads,
                         "kind": "port",
                         "sample": f"{n_px} random pixels x {w['spp']} spp per step, FP32 "
                                   "restatement of merian's pt (the Vulkan reference cannot "
                                   "run on this box)"},
        "e2e": {"value": round(value, 4), "unit": "Msamples/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gbpt(args):
    import torch
    rank, local_rank, world = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    torch.cuda.set_device(local_rank)
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S

    w, sc, cam = build_workload(args.workload)
    # the context renders on this stream (gbpt_create with 0 would make a private one): events
    # recorded on it order with every launch of a step, including the second tick stream's
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = S.Context(local_rank, stream.cuda_stream)
    sid = ctx.upload(sc)
    bvh = ctx.scene_stats(sid)
    W, H = w["width"], w["height"]
    n_pix = W * H
    out = torch.empty((n_pix, 4), dtype=torch.float32, device="cuda")
    host_out = torch.empty((n_pix, 4), dtype=torch.float32, pin_memory=True)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    def params(frame):
        p, _ = S.render_params(W, H, w["spp"], w["max_path_length"], nee=w["nee"],
                               rr_depth=w["rr_depth"], frame=frame)
        return p

    frame_base = 1_000_000 * rank
    tuning = None
    if args.tuning:
        wave, sort, *more = (int(x) for x in args.tuning.split(","))
        more += [0] * (4 - len(more))
        streams, refill, postpone, bps = more[:4]
        ctx.set_tuning(wave, sort, streams=streams, refill_lanes=refill,
                       postpone_lanes=postpone, blocks_per_sm=bps)
        tuning = dict(tuning_dict(ctx.get_tuning()), fixed=True)
    elif not args.no_autotune:
        t, cand_ms = ctx.autotune(sid, cam, params(frame_base + 998))
        tuning = dict(tuning_dict(t), candidates_ms=[round(m, 2) for m in cand_ms])
    for i in range(args.warmup):
        ctx.render_device(sid, cam, params(frame_base + i), out.data_ptr())
    torch.cuda.synchronize()

    # the timed steps: the render as a user runs it (no profiling: ticks alternate over two
    # streams); then the same number of profiled steps (per-launch CUDA events, one stream) give
    # the kernel split and the traversal launch durations of the roofline
    ctx.set_profiling(0)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    step_ms = []
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank if "CUDA_VISIBLE_DEVICES" not in os.environ else 0) as clk:
        for i in range(args.steps):
            flush.zero_()                       # L2 flush outside the timed events
            ev0.record(stream)
            ctx.render_device(sid, cam, params(frame_base + args.warmup + i), out.data_ptr())
            ev1.record(stream)
            torch.cuda.synchronize()
            step_ms.append(ev0.elapsed_time(ev1))
    torch.cuda.synchronize()
    ms = float(np.mean(step_ms))

    # untimed instrumented pass: CWBVH nodes / triangles per closest-hit ray of this workload by
    # the kernel's own counters (with its postponed triangle groups)
    ctx.set_profiling(2)
    cst = ctx.render_device(sid, cam, params(frame_base + 999), out.data_ptr(), stats=True)
    kernel_nodes_per_ray = cst.nodes_visited / max(cst.trace_rays, 1)
    kernel_tris_per_ray = cst.tris_tested / max(cst.trace_rays, 1)
    # the roofline's per-ray counts: a host walk of the same tree over a 1 % pixel sample's
    # bounce rays (rank 0 at N = 1 with the CPU legs; else the kernel's counters)
    walk = None
    if world == 1 and not args.no_cpu_baseline:
        walk = cwbvh_walk_sample(sc, cam, w)
    nodes_per_ray = walk["nodes_per_ray"] if walk else kernel_nodes_per_ray
    tris_per_ray = walk["tris_per_ray"] if walk else kernel_tris_per_ray
    simt = {"node_lanes_per_step": round(cst.node_lanes / max(cst.node_steps, 1), 2),
            "tri_lanes_per_step": round(cst.tri_lanes / max(cst.tri_steps, 1), 2),
            "node_steps_per_ray": round(cst.node_steps / max(cst.trace_rays, 1), 3),
            "tri_steps_per_ray": round(cst.tri_steps / max(cst.trace_rays, 1), 3)}
    bytes_per_ray = 48.0 + 80.0 * nodes_per_ray + 48.0 * tris_per_ray
    ctx.set_profiling(1)

    torch.cuda.synchronize()
    prof_ms, trace_ms, trace_rays, trace_launches, launches, rays = [], 0.0, 0, 0, 0, 0
    cls_ms = {"trace": 0.0, "shade": 0.0, "shadow": 0.0, "primary_finalize": 0.0}
    for i in range(args.steps):
        flush.zero_()
        ev0.record(stream)
        st = ctx.render_device(sid, cam, params(frame_base + args.warmup + i),
                               out.data_ptr(), stats=True)
        ev1.record(stream)
        torch.cuda.synchronize()
        prof_ms.append(ev0.elapsed_time(ev1))
        trace_ms += st.trace_ms
        cls_ms["trace"] += st.trace_ms
        cls_ms["shade"] += st.shade_ms
        cls_ms["shadow"] += st.shadow_ms
        cls_ms["primary_finalize"] += st.other_ms
        trace_rays += st.trace_rays
        trace_launches += st.trace_launches
        launches += st.kernel_launches
        rays += st.rays
    torch.cuda.synchronize()

    parity = parity_vs_fixtures(ctx, sid, cam, w) if args.workload == WORKLOAD else None

    # end to end through the public API with a host output buffer (D2H inside the call)
    ctx.set_profiling(0)
    e2e_ms = []
    for i in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        p = params(frame_base + 5000 + i)
        N.check(ctx.lib.gbpt_render(ctx.handle, sid, N.C.byref(cam), N.C.byref(p),
                                    host_out.data_ptr(), None))
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    e2e = float(np.mean(e2e_ms))

    ms, e2e = rank_max([ms, e2e], world)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()

    samples_per_step = n_pix * w["spp"]
    value = whole_job(world, samples_per_step, ms)
    e2e_value = whole_job(world, samples_per_step, e2e)
    peak, peak_kind = measured_peaks()
    achieved = (trace_rays * bytes_per_ray) / (trace_ms / 1e3) / 1e9 if trace_ms > 0 else None
    tpr, tsrc = ncu_traffic_per_ray()
    traffic = None
    if tpr is not None and trace_launches:
        traffic = tpr * trace_rays / trace_launches
    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "Msamples/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator, same shapes and distributions as the config)",
            "config": {"workload": args.workload, "triangles": sc.triangle_count,
                       "width": W, "height": H, "spp": w["spp"],
                       "max_path_length": w["max_path_length"], "nee": w["nee"],
                       "rr_depth": w["rr_depth"], "env": "2048x1024 RGBA32F, 8 Gaussian lobes",
                       "bvh_nodes": bvh["nodes"], "bvh_depth": bvh["depth"],
                       "l2": "flushed between timed steps (256 MiB write)",
                       "parallelism": f"{world} replica(s): one frame per rank, frame seed = rank"},
            "grays_per_s": round(world * rays / args.steps / (ms / 1e3) / 1e9, 4),
            "rays_per_sample": round(rays / args.steps / samples_per_step, 4),
            "clocks": clk.summary(),
            "e2e": {"value": round(e2e_value, 3), "unit": "Msamples/s",
                    "h2d_bytes_per_step": N.C.sizeof(N.Camera) + N.C.sizeof(N.RenderParams),
                    "d2h_bytes_per_step": n_pix * 16},
            "gpu_launches": int(launches),
            "kernel_ms_per_step": {k: round(v / args.steps, 3) for k, v in cls_ms.items()},
            "roofline": {"kernel": "k_trace (CWBVH closest-hit traversal, bounce loop)",
                         "bound": "hbm", "achieved": None if achieved is None else round(achieved, 1),
                         "peak": peak, "unit": "GB/s",
                         "frac": None if achieved is None else round(achieved / peak, 4),
                         "peak_kind": f"{peak_kind} HBM copy bandwidth",
                         "traffic": None if traffic is None else round(traffic),
                         "traffic_source": tsrc,
                         "bytes_per_ray": round(bytes_per_ray, 1),
                         "nodes_per_ray": round(nodes_per_ray, 3),
                         "tris_per_ray": round(tris_per_ray, 3),
                         "counts_source": (f"host walk of the same CWBVH, {walk['rays']} bounce "
                                           f"rays of {walk['pixels']} pixels (1 %)" if walk else
                                           "kernel counters"),
                         "kernel_nodes_per_ray": round(kernel_nodes_per_ray, 3),
                         "kernel_tris_per_ray": round(kernel_tris_per_ray, 3),
                         "simt": simt,
                         "launches_per_step": trace_launches // max(args.steps, 1),
                         "trace_rays_per_step": trace_rays // max(args.steps, 1),
                         "trace_share_of_step": round(trace_ms / float(np.sum(prof_ms)), 4),
                         "kernel_times": "CUDA events per launch over the profiled steps "
                                         "(one stream)"},
            "profiled_ms_per_step": round(float(np.mean(prof_ms)), 3),
        }
        if tuning is not None:
            line["config"]["tuning"] = tuning
        if parity:
            line["rel_rmse_vs_fp64"] = parity
        if world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(sc, cam, w, args.cpu_seconds)
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def _flush_l2(torch, buf):
    buf.zero_()
    torch.cuda.synchronize()


def run_batch_mix(args):
    """Config 3: independent scenes (triangles log-uniform 1k-2M), one request each, rendered
    by plain per-request gbpt_render_device launches and by one gbpt_render_batch call (with and
    without CUDA-graph replay of the ticks). All outputs stay in HBM; the outputs of both paths
    are compared bit for bit. batch-256: requests of 256^2-1024^2 at 1-64 spp; batch-small: the
    same scenes with requests of 64^2-512^2 at 1-4 spp, where one request alone cannot fill the
    GPU, timed per resolution bucket as well."""
    import torch
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    from merian_gb300 import workloads as WL
    torch.cuda.set_device(0)
    n = args.scenes or 256
    small = args.workload == "batch-small"
    specs, reqs = (WL.batch_small if small else WL.batch_mix)(S.BASE_SEED, n)
    # the context renders on this stream (gbpt_create with 0 would make a private one): events
    # recorded on it order with every launch of a step, including the second tick stream's
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = S.Context(0, stream.cuda_stream)
    t0 = time.perf_counter()
    sids = WL.upload_all(ctx, specs)
    setup_s = time.perf_counter() - t0
    jobs, out_plain, out_batch = [], [], []
    for r in reqs:
        kind = specs[r.scene].kind
        jobs.append((sids[r.scene], WL.camera(kind, r.width, r.height), WL.params(kind, r)))
        out_plain.append(torch.empty((r.width * r.height, 4), device="cuda"))
        out_batch.append(torch.empty((r.width * r.height, 4), device="cuda"))
    samples = sum(r.width * r.height * r.spp for r in reqs)
    creqs = (N.Request * n)()
    for i, (sid, cam, p) in enumerate(jobs):
        creqs[i] = ctx.request(sid, cam, p, out_device=out_batch[i].data_ptr())
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    tuning = None
    if not args.no_autotune:
        # one schedule for both arms, tuned on the batch's largest whole-frame request
        k = max(range(n), key=lambda i: reqs[i].width * reqs[i].height * reqs[i].spp)
        t, cand = ctx.autotune(*jobs[k])
        tuning = dict(tuning_dict(t), tuned_on_request=k,
                      candidates_ms=[round(m, 2) for m in cand])

    def plain(sel=None):
        for i in (range(n) if sel is None else sel):
            sid, cam, p = jobs[i]
            ctx.render_device(sid, cam, p, out_plain[i].data_ptr())

    def batched(sel=None):
        if sel is None:
            N.check(ctx.lib.gbpt_render_batch(ctx.handle, creqs, n, None))
            return
        sub = (N.Request * len(sel))(*[creqs[i] for i in sel])
        N.check(ctx.lib.gbpt_render_batch(ctx.handle, sub, len(sel), None))

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(args.steps):
            _flush_l2(torch, flush)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.mean(ts))

    per_bucket = {}
    with ClockSampler(0) as clk:
        ms_plain = timed(plain)
        ms_batch = timed(batched)
        ctx.set_graphs(True)
        ms_graph = timed(batched)
        ctx.set_graphs(False)
        if small:
            for res in WL.SMALL_RESOLUTIONS:
                sel = [i for i, r in enumerate(reqs) if (r.width, r.height) == res]
                if not sel:
                    continue
                smp = sum(reqs[i].width * reqs[i].height * reqs[i].spp for i in sel)
                bp = timed(lambda: plain(sel))
                bb = timed(lambda: batched(sel))
                ctx.set_graphs(True)
                bg = timed(lambda: batched(sel))
                ctx.set_graphs(False)
                rate = lambda ms: round(smp / (ms / 1e3) / 1e6, 3)
                per_bucket[f"{res[0]}x{res[1]}"] = {
                    "requests": len(sel), "samples": smp,
                    "plain": {"value": rate(bp), "ms": round(bp, 3)},
                    "batched": {"value": rate(bb), "ms": round(bb, 3)},
                    "batched_graphs": {"value": rate(bg), "ms": round(bg, 3)},
                    "speedup_vs_plain": round(bp / min(bb, bg), 3)}
    identical = all(torch.equal(a.view(torch.int32), b.view(torch.int32))
                    for a, b in zip(out_plain, out_batch))
    mps = lambda ms: round(samples / (ms / 1e3) / 1e6, 3)
    best = min(ms_batch, ms_graph)
    line = {
        "metric": "Msamples/s of a request batch: one tick engine for all requests vs plain "
                  "per-request launches (same outputs, bit for bit)",
        "workload": args.workload, "value": mps(best), "unit": "Msamples/s",
        "higher_is_better": True, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(best, 3), "dtype": "f32", "data": "synthetic",
        "plain": {"value": mps(ms_plain), "ms_per_step": round(ms_plain, 3)},
        "batched": {"value": mps(ms_batch), "ms_per_step": round(ms_batch, 3)},
        "batched_graphs": {"value": mps(ms_graph), "ms_per_step": round(ms_graph, 3)},
        "speedup_vs_plain": round(ms_plain / best, 3),
        "target": "batched >= 2x plain samples/s",
        "outputs_identical": identical,
        "clocks": clk.summary(),
        "config": {"workload": args.workload, "scenes": n, "requests": n,
                   "triangles_total": sum(s.triangles for s in specs),
                   "cornell_scenes": sum(s.kind == "cornell" for s in specs),
                   "samples_per_step": samples,
                   "resolutions": ("64^2 / 128^2 / 256^2 / 512^2" if small
                                   else "256^2 / 512^2 / 1024^2"),
                   "spp": "1 / 2 / 4" if small else "uniform 1..64",
                   "estimator": "NEE + RR from 3; path length 5 (Cornell) / 8 (soup)",
                   "scene_setup_s": round(setup_s, 1),
                   "l2": "flushed between timed steps (256 MiB write)",
                   "tuning": tuning},
    }
    if per_bucket:
        line["per_resolution"] = per_bucket
    print(json.dumps(line), flush=True)
    ctx.close()


def run_instanced(args):
    """Config 5: 1,000 instances of 50 distinct 50k-triangle meshes (50M instanced triangles)
    under random affine transforms, 256 sRGB RGBA8 512^2 albedo textures, Lambert / GGX-Lambert
    materials, a Gaussian-lobe environment; 3840x2160, progressive 256 spp as 16 frames of 16 spp
    accumulated on the device (gbpt_accumulate, running mean), path length 16, NEE and Russian
    roulette from depth 3. A step is the whole progressive image."""
    import torch
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    from merian_gb300 import workloads as W
    torch.cuda.set_device(0)
    W_, H_, frames, spp, L = 3840, 2160, 16, 16, 16
    t0 = time.perf_counter()
    sc = W.instanced_scene(S.BASE_SEED)
    # the context renders on this stream (gbpt_create with 0 would make a private one): events
    # recorded on it order with every launch of a step, including the second tick stream's
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = S.Context(0, stream.cuda_stream)
    sid = ctx.upload(sc)
    setup_s = time.perf_counter() - t0
    st = ctx.scene_stats(sid)
    cam = W.instanced_camera(W_, H_)
    n = W_ * H_
    frame = torch.empty((n, 4), device="cuda")
    acc = torch.zeros((n, 4), device="cuda")
    hist = torch.zeros(n, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    tuning = None
    if not args.no_autotune:
        p0, _ = S.render_params(W_, H_, spp, L, nee=True, rr_depth=3, frame=999_999)
        t, cand = ctx.autotune(sid, cam, p0)
        tuning = dict(tuning_dict(t), candidates_ms=[round(m, 2) for m in cand])

    def step(base):
        for f in range(frames):
            p, _ = S.render_params(W_, H_, spp, L, nee=True, rr_depth=3, frame=base + f)
            ctx.render_device(sid, cam, p, frame.data_ptr())
            N.check(ctx.lib.gbpt_accumulate(ctx.handle, frame.data_ptr(), acc.data_ptr(),
                                            hist.data_ptr(), n, 1.0, float("inf"), int(f == 0)))

    for i in range(args.warmup):
        step(1000 * i)
    torch.cuda.synchronize()
    ts, rays = [], 0
    with ClockSampler(0) as clk:
        for i in range(args.steps):
            _flush_l2(torch, flush)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step(100000 + 1000 * i)
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
    ms = float(np.mean(ts))
    samples = n * spp * frames
    img = acc.cpu().numpy()
    line = {
        "metric": "Msamples/s, progressive render of the instanced scene", "workload": "instanced-4k",
        "value": round(samples / (ms / 1e3) / 1e6, 3), "unit": "Msamples/s",
        "higher_is_better": True, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms, 3), "dtype": "f32", "data": "synthetic",
        "clocks": clk.summary(),
        "image_mean_rgb": [round(float(x), 5) for x in img[:, :3].mean(axis=0)],
        "image_finite": bool(np.all(np.isfinite(img))),
        "config": {"workload": "instanced-4k", "meshes": 50, "triangles_per_mesh": 50000,
                   "instances": len(sc.instances),
                   "instanced_triangles": int(sum(sc.geometries["triangle_count"][
                       sc.blas_ranges["first_geometry"][b]:sc.blas_ranges["first_geometry"][b] +
                       sc.blas_ranges["geometry_count"][b]].sum() for b in sc.instances["blas"])),
                   "textures": len(sc.textures), "width": W_, "height": H_,
                   "spp": spp * frames, "frames": frames, "max_path_length": L,
                   "nee": True, "rr_depth": 3, "bvh_nodes": st["nodes"], "bvh_depth": st["depth"],
                   "scene_setup_s": round(setup_s, 1),
                   "l2": "flushed between timed steps (256 MiB write)", "tuning": tuning},
    }
    print(json.dumps(line), flush=True)
    ctx.close()


def _percentile(xs, q):
    return float(np.percentile(np.asarray(xs), q)) if xs else None


def run_served(args):
    """Config 4: Poisson arrivals over resident scenes (triangles log-uniform 10k-5M), 5 % of
    requests bringing a new 100k-triangle scene; each rate is served by the request server
    (continuous batching) and, with the same arrivals, by a serial queue of plain gbpt_render
    calls. Latency = completion - scheduled arrival; outputs go to host memory."""
    import torch
    from merian_gb300 import _native as N
    from merian_gb300 import scene as S
    from merian_gb300 import workloads as WL
    torch.cuda.set_device(0)
    n_scenes = args.scenes or 32
    small = args.workload == "served-small"
    rates = [float(x) for x in (args.rates or ("2000,10000,50000" if small else "50,200,2000"))
             .split(",") if x]
    n_requests = args.requests or (512 if small else 96)
    mix = WL.served_small if small else WL.served_stream
    specs, _ = WL.served_stream(S.BASE_SEED, n_scenes, 0)
    ctx = S.Context(0)
    t0 = time.perf_counter()
    sids = WL.upload_all(ctx, specs)
    setup_s = time.perf_counter() - t0
    results = []

    def prepare(rate):
        _, reqs = mix(S.BASE_SEED, n_scenes, n_requests, rate)
        new_scenes = {i: r.upload.build() for i, r in enumerate(reqs) if r.upload}
        return reqs, new_scenes

    def job(r, sid):
        kind = "soup" if r.upload else specs[r.scene].kind
        return sid, WL.camera(kind, r.width, r.height), WL.params(kind, r)

    tuning = None
    if not args.no_autotune:
        # one schedule for the server and the serial queue, tuned on the largest request
        _, reqs0 = mix(S.BASE_SEED, n_scenes, n_requests, rates[0])
        big = max((r for r in reqs0 if not r.upload), key=lambda r: r.width * r.height * r.spp)
        t, cand = ctx.autotune(*job(big, sids[big.scene]))
        tuning = dict(tuning_dict(t), candidates_ms=[round(m, 2) for m in cand])

    with ClockSampler(0) as clk:
        for rate in rates:
            reqs, new_scenes = prepare(rate)
            samples = sum(r.width * r.height * r.spp for r in reqs)
            row = {"rate_req_s": rate, "requests": len(reqs),
                   "uploads": len(new_scenes), "samples": samples}
            for mode in ("served", "plain"):
                outs = [np.empty((r.width * r.height, 4), np.float32) for r in reqs]
                made = []
                lat = [None] * len(reqs)
                if mode == "served":
                    ctx.server_start()
                start = ctx.clock() + 0.05
                tickets = [None] * len(reqs)
                for i, r in enumerate(reqs):
                    delay = start + r.arrival_s - ctx.clock()
                    if delay > 0:
                        time.sleep(delay)
                    sid = sids[r.scene]
                    if r.upload:
                        sid = ctx.upload(new_scenes[i])
                        made.append(sid)
                    sid, cam, p = job(r, sid)
                    if mode == "served":
                        tickets[i] = ctx.submit(sid, cam, p, out_host=outs[i])
                    else:
                        N.check(ctx.lib.gbpt_render(ctx.handle, sid, N.C.byref(cam),
                                                    N.C.byref(p), N.ptr(outs[i]), None))
                        lat[i] = ctx.clock() - (start + r.arrival_s)
                end = ctx.clock()
                if mode == "served":
                    for i, t in enumerate(tickets):
                        rc, st = ctx.wait(t, -1.0)
                        if rc != 0:
                            raise RuntimeError(f"served request {i} failed: {rc}")
                        lat[i] = st.done_s - (start + reqs[i].arrival_s)
                        end = max(end, st.done_s)
                    info = ctx.server_info()
                    ctx.server_stop()
                for sid in made:
                    ctx.destroy_scene(sid)
                span = end - start
                row[mode] = {"p50_ms": round(1e3 * _percentile(lat, 50), 1),
                             "p99_ms": round(1e3 * _percentile(lat, 99), 1),
                             "mean_ms": round(1e3 * float(np.mean(lat)), 1),
                             "makespan_s": round(span, 3),
                             "msamples_per_s": round(samples / span / 1e6, 3)}
                if mode == "served":
                    row[mode]["ticks"] = info["ticks"]
            row["throughput_ratio"] = round(row["served"]["msamples_per_s"] /
                                            row["plain"]["msamples_per_s"], 3)
            results.append(row)
    best = max(results, key=lambda r: r["served"]["msamples_per_s"])
    line = {
        "metric": "served p50/p99 latency and Msamples/s: request server (continuous batching) "
                  "vs a serial queue of plain gbpt_render calls, same arrivals",
        "workload": args.workload, "value": best["served"]["msamples_per_s"],
        "unit": "Msamples/s", "higher_is_better": True, "n_gpus": 1, "dtype": "f32",
        "data": "synthetic", "rates": results, "clocks": clk.summary(),
        "target": "served >= 2x the serial plain queue's samples/s",
        "config": {"workload": args.workload, "resident_scenes": n_scenes,
                   "triangles_resident": sum(s.triangles for s in specs),
                   "requests_per_rate": n_requests,
                   "resolutions": ("64^2 / 128^2 / 256^2 / 512^2" if small
                                   else "512^2 / 1024^2 / 1920x1080"),
                   "spp": "1 / 2 / 4" if small else "1 / 4 / 16 / 64",
                   "uploads": ("none" if small else
                               "5 % of requests bring a new 100k-triangle soup (BVH build + "
                               "upload inside the request's latency)"),
                   "estimator": "NEE + RR from 3; path length 5 (Cornell) / 8 (soup)",
                   "scene_setup_s": round(setup_s, 1), "tuning": tuning},
    }
    print(json.dumps(line), flush=True)
    ctx.close()


def _free_port() -> int:
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def launch_ranks(args) -> int | None:
    """--gpus N outside torchrun: start N ranks of this script with torch.distributed.run (one
    process per GPU, rendezvous on 127.0.0.1) and return their exit status. Under torchrun,
    --gpus must equal WORLD_SIZE. None: run this process as the only rank."""
    world_env = os.environ.get("WORLD_SIZE")
    if world_env is not None:
        if int(world_env) != args.gpus:
            print(f"bench.py: --gpus {args.gpus} but WORLD_SIZE={world_env}", file=sys.stderr)
            return 2
        return None
    if args.gpus <= 1:
        return None
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
           f"--nproc-per-node={args.gpus}", "--master-addr", "127.0.0.1",
           "--master-port", str(_free_port()), str(Path(__file__).resolve()), *sys.argv[1:]]
    return subprocess.call(cmd)


def main():
    args = parse()
    rc = launch_ranks(args)
    if rc is not None:
        sys.exit(rc)
    mixed = args.workload in ("batch-256", "batch-small", "served-stream", "served-small",
                              "instanced-4k")
    if args.steps is None:
        args.steps = 1 if mixed else 5
    if args.warmup is None:
        args.warmup = 1 if mixed else 3
    if args.impl == "reference":
        if mixed:  # the CPU reference is timed on the headline frame only
            args.workload = WORKLOAD
        run_reference(args)
    elif args.workload in ("batch-256", "batch-small"):
        run_batch_mix(args)
    elif args.workload in ("served-stream", "served-small"):
        run_served(args)
    elif args.workload == "instanced-4k":
        run_instanced(args)
    else:
        run_gbpt(args)


if __name__ == "__main__":
    main()
