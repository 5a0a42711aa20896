#!/usr/bin/env python
"""Benchmark of the sculpt-brush dab path: vertices displaced per second.

Default workload (one GPU): the masked, X-mirrored smooth-brush stroke of 128
dabs on a noisy level-8 icosphere (655,362 vertices, 1,310,720 looptris,
PBVH leaf limit 5000 looptris), seeded synthetic input.  A step is that whole
stroke: per dab and symmetry pass the node search and the brush, then the
normal update and bounding-box refit, as the reference's stroke does.

  value  : device-resident throughput — Sum(vertices displaced) / Sum(stroke
           time), stroke time from CUDA events on the mesh stream; the stroke
           runs as one launch of the persistent stroke kernel (cluster size
           picked by the autotuner); positions, normals and node boxes are
           restored from a device snapshot and L2 flushed (256 MiB write, then a
           256 MiB read of another buffer)
           before every step, both outside the timed region.
  e2e    : the same through sgpu_stroke_host with page-locked host buffers:
           H2D of positions and normals, full box refit, stroke, D2H of
           positions, all inside the event-timed region.
  roofline: k_team_stroke (the only kernel of a step): algorithmic bytes per
           launch (the kernel's own counters, an instrumented run) / mean
           step time of the timed run, against the measured HBM copy
           bandwidth.
  plain_graph / plain_eager: the same stroke through the per-call kernels
           (one kernel per reference call), replayed as a CUDA graph / eager.
  batch  : the 64-mesh uneven batch, one persistent launch versus 64
           sequential plain strokes.
  cpu_baseline: the FP32 CPU restatement (oracle, OpenMP over PBVH nodes) on
           the host cores, same stroke.

--quick runs three persistent strokes of the workload and exits (the
command profiled with ncu).  --phases prints the persistent kernel's per-dab
phase profile on all five workloads.

--impl reference times the CPU restatement of the reference path (the
reference cannot run the path: its brush code and public headers are missing).
Under torchrun (N>1) each rank runs an independent replica (the path does not
shard within a mesh); rank 0 prints max-over-ranks timing.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "vertices displaced/sec"
UNIT = "verts/s"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--cpu-sample-dabs", type=int, default=0,
                    help="dabs of the stroke in the CPU sample (0 = whole stroke)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-mesh batch comparison")
    ap.add_argument("--quick", action="store_true",
                    help="three persistent strokes of the workload, no report (for ncu)")
    ap.add_argument("--cluster", type=int, default=16, help="cluster size for --quick")
    ap.add_argument("--raycast-only", action="store_true",
                    help="1024-ray sgpu_raycast batches on the workload mesh and on the "
                         "multires torus, one JSON line, and exit (the command profiled "
                         "with ncu for the ray kernels)")
    ap.add_argument("--raycast-mesh", choices=["faces", "grids", "both"], default="both",
                    help="meshes of --raycast-only")
    ap.add_argument("--draw-only", action="store_true",
                    help="full draw-buffer refreshes on the workload mesh and on the multires "
                         "torus, one JSON line, and exit (the command profiled with ncu for "
                         "the draw kernels)")
    ap.add_argument("--draw-mesh", choices=["faces", "grids", "both"], default="both",
                    help="meshes of --draw-only")
    ap.add_argument("--phases", action="store_true",
                    help="per-phase profile of the persistent stroke on the five workloads "
                         "and the stroke-start brushes "
                         "(one JSON line each), no report")
    return ap.parse_args()


def run_quick(args):
    from dune_sculpt_gb300 import build as libbuild

    libbuild.build()
    from dune_sculpt_gb300.sculpt import PBVH, STROKE_TEAM

    m, st, leaf_limit, _ = workload()
    g = PBVH.build_mesh(m, leaf_limit)
    g.snapshot()
    g.set_team(args.cluster)
    for _ in range(3):
        g.restore()
        s = g.stroke(st, mode=STROKE_TEAM)
    print(f"quick: {s.verts_displaced} vertices displaced, {s.gpu_ms:.3f} ms")
    return 0


def run_phases(args):
    """Per-dab phase times of the persistent stroke kernel on the five workloads:
    the autotuned cluster, the best of three L2-flushed strokes, then one
    instrumented stroke (phase timers of the team's first thread)."""
    from dune_sculpt_gb300 import build as libbuild

    libbuild.build()
    from dune_sculpt_gb300 import synth
    from dune_sculpt_gb300.sculpt import PBVH, STROKE_GRAPH, STROKE_TEAM

    def one(name, g, st, tools=None, graph=False):
        g.snapshot()
        best, _ = g.autotune_team(st, dab_tools=tools)
        times = []
        for _ in range(3):
            g.restore()
            g.flush_l2()
            times.append(g.stroke(st, mode=STROKE_TEAM, dab_tools=tools).gpu_ms)
        extra = {}
        if graph:  # the same stroke replayed from a CUDA graph of the per-call kernels
            gt = []
            for _ in range(3):
                g.restore()
                g.flush_l2()
                gt.append(g.stroke(st, mode=STROKE_GRAPH, dab_tools=tools).gpu_ms)
            extra["graph_ms_per_stroke"] = round(min(gt), 3)
        g.restore()
        g.flush_l2()
        ph, _, stats = g.stroke_team_profile(st, dab_tools=tools)
        nd = st.dabs.shape[0]
        print(json.dumps({
            "workload": name, "cluster": best, "ms_per_stroke": round(min(times), 3),
            "us_per_dab": round(1000 * min(times) / nd, 2),
            "verts_displaced": stats.verts_displaced, **extra,
            "phase_us_per_dab": {k: round(1000 * v["ms"] / nd, 2) for k, v in ph.items()},
            "phase_alg_MB_per_stroke": {k: round(v["bytes"] / 1e6, 2) for k, v in ph.items()}}),
            flush=True)
        g.free()

    m, st, ll = synth.cfg1_grid_draw()
    one("grid513_draw", PBVH.build_mesh(m, ll), st)
    m, st, ll = synth.cfg2_icosphere_smooth()
    one("icosphere8_smooth_masked_xmirror", PBVH.build_mesh(m, ll), st)
    m, st, ll = synth.cfg3_sphere_clay()
    one("uvsphere2048_clay_strips_xmirror", PBVH.build_mesh(m, ll), st)
    g, dabs = synth.cfg5_multires()
    tools = np.array([(synth.TOOL_DRAW, synth.TOOL_SMOOTH, synth.TOOL_INFLATE)[d % 3]
                      for d in range(dabs.shape[0])], dtype=np.int32)
    st = synth.Stroke(synth.TOOL_DRAW, 0.04, 0.6, synth.CURVE_SMOOTH, 0, dabs)
    one("multires_torus_50000x17x17_mixed", PBVH.build_grids(g), st, tools)
    # the stroke-start brushes on the icosphere of the bench workload (128
    # dabs, X mirror): persistent and graph-replayed
    m, st, ll = synth.cfg2_icosphere_smooth()
    grab = synth.grab_dabs(synth.SEED_BASE + 40, st.dabs.shape[0], 0.0005)
    for name, tool, dabs, kw in (
            ("grab", synth.TOOL_GRAB, grab, {}),
            ("layer", synth.TOOL_LAYER, st.dabs, {"height": 0.3})):
        so = synth.Stroke(tool, st.radius, st.strength, synth.CURVE_SMOOTH, synth.SYMM_X, dabs, **kw)
        one(f"icosphere8_{name}_xmirror", PBVH.build_mesh(m, ll), so, graph=True)
    return 0


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def workload():
    from dune_sculpt_gb300 import synth

    m, st, leaf_limit = synth.cfg2_icosphere_smooth()
    cfg = {"workload": "icosphere8_smooth_masked_xmirror", "verts": int(m.totvert),
           "looptris": int(m.looptris.shape[0]), "dabs": int(st.dabs.shape[0]),
           "radius": st.radius, "strength": st.strength, "symmetry": "X",
           "curve": "smooth", "leaf_limit": leaf_limit, "mask": "seeded smooth noise",
           "l2": "flushed before every step (256 MiB device write, then 256 MiB read)"}
    return m, st, leaf_limit, cfg


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None
        self.gpu = gpu_index
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def wait_first(self, timeout: float = 5.0):
        """Blocks until the first sample is written, so that sampling covers
        the timed region from its start."""
        t0 = time.perf_counter()
        while self.proc is not None and time.perf_counter() - t0 < timeout:
            self.f.flush()
            if os.path.getsize(self.path) > 0:
                return
            time.sleep(0.02)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sms, maxes, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sms.append(float(parts[1]))
                    maxes.append(float(parts[2]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sms) if sms else None,
                "sm_max_mhz": max(maxes) if maxes else None, "samples": len(sms),
                "reasons": sorted(reasons)}


def cpu_baseline(m, st, leaf_limit, sample_dabs: int):
    """FP32 CPU restatement (oracle) on all host cores: a bounded sample of the
    same stroke (the first sample_dabs dabs, or the whole stroke)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    pyoracle.build()
    o = pyoracle.OracleMesh.faces(m, leaf_limit)
    o.recalc_all_normals()
    dabs = st.dabs if not sample_dabs else st.dabs[:sample_dabs]
    threads = pyoracle.max_threads()
    t0 = time.perf_counter()
    tot, _ = o.stroke(st, which=1, nthreads=threads, dabs=dabs)
    dt = time.perf_counter() - t0
    o.close()
    return {"value": tot / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{dabs.shape[0]} of {st.dabs.shape[0]} dabs of the same stroke, "
                      f"{tot} vertices displaced in {dt:.3f} s (FP32 restatement, OpenMP "
                      f"over PBVH nodes)", "seconds": dt}


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    m, st, leaf_limit, cfg = workload()
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    pyoracle.build()
    sample = args.cpu_sample_dabs or 32
    dabs = st.dabs[:sample]
    threads = pyoracle.max_threads()

    def fresh():
        o = pyoracle.OracleMesh.faces(m, leaf_limit)
        o.recalc_all_normals()
        return o

    for _ in range(args.warmup):
        fresh().stroke(st, which=1, nthreads=threads, dabs=dabs)
    total_v, total_s = 0, 0.0
    for _ in range(args.steps):
        o = fresh()  # every step starts from the same mesh state (untimed)
        t0 = time.perf_counter()
        tot, _ = o.stroke(st, which=1, nthreads=threads, dabs=dabs)
        total_s += time.perf_counter() - t0
        total_v += tot
        o.close()
    value = total_v / total_s
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * total_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)", "config": cfg,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"first {sample} of {st.dabs.shape[0]} dabs per step "
                                       "(FP32 CPU restatement of the reference path: the "
                                       "reference has no brush code to run)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def combine_ranks(dist, total_ms, e2e_ms, total_v, e2e_v):
    """Replicas: the slowest rank's times (max) and every rank's vertices
    (sum), so that value = all vertices / the job's time."""
    import torch

    t = torch.tensor([total_ms, e2e_ms], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    c = torch.tensor([total_v, e2e_v], dtype=torch.float64)
    dist.all_reduce(c, op=dist.ReduceOp.SUM)
    return float(t[0]), float(t[1]), int(c[0]), int(c[1])


def run_gpu(args):
    world, rank, local = dist_env()
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
        import torch.distributed as dist

        dist.init_process_group("gloo")
    from dune_sculpt_gb300 import build as libbuild

    libbuild.build()
    from dune_sculpt_gb300 import synth
    from dune_sculpt_gb300.sculpt import (BATCH_SEQUENTIAL, BATCH_TEAM, PBVH, STROKE_EAGER,
                                          STROKE_GRAPH, STROKE_TEAM, PinnedArray, batch_stroke)

    m, st, leaf_limit, cfg = workload()
    g = PBVH.build_mesh(m, leaf_limit)
    g.snapshot()
    cluster, tune_ms = g.autotune_team(st)  # restores the snapshot

    def barrier():
        if world > 1:
            dist.barrier()

    for _ in range(args.warmup):
        g.restore()
        g.stroke(st, mode=STROKE_TEAM)
    barrier()
    clocks = ClockSampler(local) if rank == 0 else None
    if clocks:
        clocks.wait_first()
    total_ms, total_v, launches = 0.0, 0, 0
    for _ in range(args.steps):
        g.restore()
        g.flush_l2()
        s = g.stroke(st, mode=STROKE_TEAM)
        total_ms += s.gpu_ms
        total_v += s.verts_displaced
        launches += s.kernel_launches
    g.sync()
    barrier()
    clk = clocks.stop() if clocks else None

    # the same stroke through the per-call kernels: captured graph, and eager
    def plain(mode, n=2):
        ms, v = 0.0, 0
        for _ in range(n):
            g.restore()
            g.flush_l2()
            se = g.stroke(st, mode=mode)
            ms += se.gpu_ms
            v += se.verts_displaced
        return {"value": v / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / n}

    g.restore()
    g.stroke(st, mode=STROKE_GRAPH)  # graph capture outside the timing
    plain_graph = plain(STROKE_GRAPH)
    plain_eager = plain(STROKE_EAGER)

    # e2e through the host-buffer entry point with page-locked buffers
    V = m.totvert
    vin = PinnedArray((V,), m.verts.dtype)
    vin.array[:] = m.verts
    g.restore()
    nin = PinnedArray((V, 3), np.float32)
    nin.array[:] = g.normals()
    vout = PinnedArray((V,), m.verts.dtype)
    g.restore()
    g.stroke_host(st, vin.array, vout.array, nin.array, mode=STROKE_TEAM)
    e2e_ms, e2e_v = 0.0, 0
    for _ in range(args.steps):
        g.restore()
        g.flush_l2()
        s2 = g.stroke_host(st, vin.array, vout.array, nin.array, mode=STROKE_TEAM)
        e2e_ms += s2.gpu_ms
        e2e_v += s2.verts_displaced

    # phase profile of the persistent kernel (instrumented run, not timed)
    g.restore()
    g.flush_l2()
    phases, prof_ms, _ = g.stroke_team_profile(st)
    alg_bytes = sum(p["bytes"] for p in phases.values())

    batch = None if args.no_batch else run_batch(args, synth, PBVH, batch_stroke, BATCH_TEAM,
                                                  BATCH_SEQUENTIAL)
    g.restore()
    ray = run_raycast_leg(g, m, leaf_limit, args.no_cpu)
    g.restore()
    draw = run_draw_leg(g, m, st, leaf_limit, args.no_cpu, peak=measured_peaks()[0])

    if world > 1:
        total_ms, e2e_ms, total_v, e2e_v = combine_ranks(dist, total_ms, e2e_ms, total_v, e2e_v)
    if rank != 0:
        return 0

    peak, peak_kind = measured_peaks()
    step_ms = total_ms / args.steps
    achieved = alg_bytes / (step_ms / 1e3) / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic_per_launch.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            traffic = json.load(f).get(cfg["workload"], {}).get("k_team_stroke")
    cpu = None
    if not args.no_cpu:
        cpu = cpu_baseline(m, st, leaf_limit, args.cpu_sample_dabs)
    value = total_v / (total_ms / 1e3)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded icosphere, Gaussian radial noise, smooth-noise mask)",
        "config": dict(cfg, parallelism=f"replicas{world}",
                       mode=f"persistent stroke kernel, cluster of {cluster} CTAs (autotuned)"),
        "e2e": {"value": e2e_v / (e2e_ms / 1e3), "unit": UNIT,
                "h2d_bytes_per_step": int(V * 16 + V * 12), "d2h_bytes_per_step": int(V * 16)},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": "k_team_stroke", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS hbm_gbs)",
                     "alg_bytes_per_launch": alg_bytes, "mean_launch_ms": step_ms,
                     "traffic": traffic},
        "team_phases_ms": {k: round(v["ms"], 4) for k, v in phases.items()},
        "team_phases_bytes": {k: v["bytes"] for k, v in phases.items()},
        "autotune_ms": tune_ms,
        "plain_graph": plain_graph,
        "plain_eager": plain_eager,
        "batch": batch,
        "raycast": ray,
        "draw_buffers": draw,
        "cpu_baseline": ({k: v for k, v in cpu.items() if k != "seconds"} if cpu else None),
        "clocks": clk,
    }
    print(json.dumps(line))
    return 0


def draw_alg_bytes(g, masked: bool) -> int:
    """Algorithmic bytes of a full draw-buffer refresh: the vertex buffer
    written once (36 B per vertex) and each input read once: FACES per visible
    looptri its corner record (16 B) and per mesh vertex its
    position, normal (float4 each) and mask; GRIDS per element the same three."""
    lay = g.draw_buffers_layout()
    nverts = int(lay["vert_off"][-1])
    per_vert_in = 16 + 16 + (4 if masked else 0)
    if g.info.type == 0:
        tris = int(lay["tot_tri"].sum())
        return nverts * 36 + tris * 16 + g.num_verts * per_vert_in
    return nverts * 36 + g.num_verts * per_vert_in


def time_draw(g, reps: int = 20):
    """Full refreshes (every leaf flagged) timed with CUDA events; L2 flushed
    before each.  Returns the per-call times in ms."""
    g.draw_buffers_update_timed(all_leaves=True)
    out = []
    for _ in range(reps):
        g.flush_l2()
        out.append(g.draw_buffers_update_timed(all_leaves=True))
    return out


def run_draw_leg(g, m, st, leaf_limit, no_cpu, peak):
    """Headless draw buffers (pbvh_update_draw_buffers without GL) on the
    workload mesh: seeded face sets 1..8 on every poly, the mesh's mask,
    smooth shading.  A full refresh (all leaves) and the refresh after one
    stroke (the leaves it touched), CUDA-event timed; the oracle's full
    refresh on one host core."""
    from dune_sculpt_gb300.sculpt import STROKE_TEAM

    rng = np.random.default_rng(0x5EED0000 + 9)
    fs = rng.integers(1, 9, size=m.polys.shape[0]).astype(np.int32)
    t0 = time.perf_counter()
    g.draw_buffers_build(face_sets=fs, seed=3, color_default=1)
    build_s = time.perf_counter() - t0
    times = time_draw(g)
    ms = statistics.median(times)
    alg = draw_alg_bytes(g, m.mask is not None)
    achieved = alg / (ms / 1e3) / 1e9
    g.restore()
    g.draw_buffers_update_timed(all_leaves=False)  # consumes the flags the restore brought back
    g.stroke(st, mode=STROKE_TEAM)
    touched = int(np.count_nonzero(g.nodes()["flag"] & 16))
    g.flush_l2()
    partial_ms = g.draw_buffers_update_timed(all_leaves=False)
    lay = g.draw_buffers_layout()
    out = {"workload": "icosphere level 8, face sets 1..8, masked, smooth",
           "vertices": int(lay["vert_off"][-1]), "bytes_written": int(lay["vert_off"][-1]) * 36,
           "full_refresh_ms": ms, "full_refresh_min_ms": min(times),
           "roofline": {"bound": "hbm", "kernel": "k_draw_faces", "alg_bytes": alg,
                        "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": achieved / peak},
           "after_stroke": {"leaves_refilled": touched, "ms": partial_ms},
           "layout_build_s": build_s,
           "timing": "CUDA events on the mesh stream, L2 flushed before each refresh"}
    if not no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle

        o = pyoracle.OracleMesh.faces(m, leaf_limit)
        o.recalc_all_normals()
        L = o.draw_build(face_sets=fs, seed=3, color_default=1, vert_flag=m.verts["flag"])
        vbo = np.zeros(int(L["vert_off"][-1]) * 36, dtype=np.uint8)
        t0 = time.perf_counter()
        o.draw_update(vbo)
        cpu_s = time.perf_counter() - t0
        out["cpu_baseline"] = {"full_refresh_ms": 1e3 * cpu_s, "cores": 1, "kind": "port",
                               "sample": "one full refresh, FP32 restatement, one thread"}
        o.close()
    return out


def run_draw_grids(synth, PBVH, peak):
    """Full draw-buffer refresh on the multires torus (50,000 grids of 17x17),
    smooth, masked, face sets per base face."""
    g5, _ = synth.cfg5_multires()
    gp = PBVH.build_grids(g5)
    fs = ((np.arange(g5.num_faces) % 8) + 1).astype(np.int32)
    gp.draw_buffers_build(face_sets=fs, seed=3, color_default=1)
    times = time_draw(gp)
    ms = statistics.median(times)
    alg = draw_alg_bytes(gp, g5.mask is not None)
    achieved = alg / (ms / 1e3) / 1e9
    return {"workload": "multires torus 50,000 grids of 17x17, smooth, masked",
            "vertices": int(gp.draw_buffers_layout()["vert_off"][-1]),
            "full_refresh_ms": ms, "full_refresh_min_ms": min(times),
            "roofline": {"bound": "hbm", "kernel": "k_draw_grids", "alg_bytes": alg,
                         "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak}}


def time_raycast(g, starts, dirs, reps=20, one=200):
    """Wall-clock seconds per batch call and per one-ray call of
    sgpu_raycast (host arrays), and the batch's hit count."""
    n = starts.shape[0]
    g.raycast(starts, dirs)  # batch buffers allocated outside the timing
    t0 = time.perf_counter()
    for _ in range(reps):
        hit, _, _, _, _ = g.raycast(starts, dirs)
    batch_s = (time.perf_counter() - t0) / reps
    t0 = time.perf_counter()
    for k in range(one):
        g.raycast(starts[k % n:k % n + 1], dirs[k % n:k % n + 1])
    single_s = (time.perf_counter() - t0) / one
    return batch_s, single_s, int(hit.sum())


def run_raycast_grids(synth, PBVH):
    """Multires ray cast on the 50,000-grid torus (17x17 elements per grid):
    1024 seeded rays from radius 3 aimed at seeded grid elements."""
    g5, _ = synth.cfg5_multires()
    gp = PBVH.build_grids(g5)
    rng = np.random.default_rng(0x5EED0000 + 8)
    n = 1024
    s = rng.normal(size=(n, 3))
    starts = (3.0 * s / np.linalg.norm(s, axis=1, keepdims=True)).astype(np.float32)
    tgt = g5.co[rng.integers(0, g5.co.shape[0], size=n)].astype(np.float64)
    d = tgt - starts
    dirs = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    best = None
    for _ in range(3):
        r = time_raycast(gp, starts, dirs)
        best = r if best is None or r[0] < best[0] else best
    batch_s, single_s, nhit = best
    return {"workload": "1024 rays from radius 3 at seeded grid elements, multires torus "
            "50,000 grids of 17x17", "hits": nhit, "rays_per_s": n / batch_s,
            "ms_per_1024_rays": 1e3 * batch_s, "single_ray_us": 1e6 * single_s}


def run_raycast_leg(g, m, leaf_limit, no_cpu):
    """Ray cast (BKE_pbvh_raycast with the sculpt callback) on the workload's
    mesh: 1024 seeded rays from a sphere of radius 3 towards points near the
    centre, through sgpu_raycast with host arrays (upload, three kernels,
    read-back in the timed region); one ray per call for the latency; the
    oracle's restatement on one host core for 128 of the rays."""
    rng = np.random.default_rng(0x5EED0000 + 7)
    n = 1024
    s = rng.normal(size=(n, 3))
    starts = (3.0 * s / np.linalg.norm(s, axis=1, keepdims=True)).astype(np.float32)
    tgt = rng.normal(size=(n, 3)) * 0.3
    d = tgt - starts
    dirs = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    batch_s, single_s, nhit = time_raycast(g, starts, dirs)
    out = {"workload": "1024 rays from radius 3 towards the centre (+/-0.3), icosphere level 8",
           "hits": nhit, "rays_per_s": n / batch_s, "ms_per_1024_rays": 1e3 * batch_s,
           "single_ray_us": 1e6 * single_s, "timing": "wall clock around sgpu_raycast "
           "(host arrays in and out)"}
    if not no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle

        o = pyoracle.OracleMesh.faces(m, leaf_limit)
        o.recalc_all_normals()
        k = 128
        t0 = time.perf_counter()
        for r in range(k):
            o.raycast(starts[r], dirs[r])
        cpu_s = time.perf_counter() - t0
        out["cpu_baseline"] = {"rays_per_s": k / cpu_s, "cores": 1, "kind": "port",
                               "sample": f"{k} of the rays, FP32 restatement, one thread"}
        o.close()
    return out


def run_batch(args, synth, PBVH, batch_stroke, BATCH_TEAM, BATCH_SEQUENTIAL):
    """The 64-mesh uneven batch: one persistent launch versus 64 sequential
    plain strokes (each a CUDA graph of per-call kernels)."""
    batch = synth.cfg4_batch()
    gs = [PBVH.build_mesh(mm, ll) for (mm, _, ll) in batch]
    strokes = [s for (_, s, _) in batch]
    for p in gs:
        p.snapshot()
    nverts = sum(mm.totvert for (mm, _, _) in batch)
    best = None
    for cl in (4, 8, 16):
        for p in gs:
            p.restore()
        batch_stroke(gs, strokes, mode=BATCH_TEAM, cluster=cl)
        ms_l = []
        for _ in range(3):
            for p in gs:
                p.restore()
            gs[0].flush_l2()
            stats, ms = batch_stroke(gs, strokes, mode=BATCH_TEAM, cluster=cl)
            ms_l.append(ms)
        disp = sum(s.verts_displaced for s in stats)
        ms = statistics.median(ms_l)
        if best is None or ms < best["ms_per_step"]:
            best = {"cluster": cl, "ms_per_step": ms, "value": disp / (ms / 1e3)}
    for p in gs:
        p.restore()
    batch_stroke(gs, strokes, mode=BATCH_SEQUENTIAL)  # graph captures
    for p in gs:
        p.restore()
    t0 = time.perf_counter()
    stats, seq_ms = batch_stroke(gs, strokes, mode=BATCH_SEQUENTIAL)
    wall = (time.perf_counter() - t0) * 1e3
    disp = sum(s.verts_displaced for s in stats)
    return {"workload": "64 meshes (grid/uv-sphere alternating, log-uniform 1e4-5e5 verts, "
                        f"{nverts} verts total), 32-dab draw/inflate strokes",
            "persistent": {"value": best["value"], "unit": UNIT, "ms_per_step": best["ms_per_step"],
                           "cluster": best["cluster"]},
            "sequential_plain": {"value": disp / (seq_ms / 1e3), "unit": UNIT,
                                 "ms_per_step": seq_ms, "wall_ms": wall},
            "speedup": best["value"] / (disp / (seq_ms / 1e3))}


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.quick:
        return run_quick(args)
    if args.phases:
        return run_phases(args)
    if args.draw_only:
        from dune_sculpt_gb300 import build as libbuild

        libbuild.build()
        from dune_sculpt_gb300 import synth
        from dune_sculpt_gb300.sculpt import PBVH

        peak = measured_peaks()[0]
        out = {}
        if args.draw_mesh in ("faces", "both"):
            m, st, leaf_limit, _ = workload()
            g = PBVH.build_mesh(m, leaf_limit)
            g.snapshot()
            out["draw_faces"] = run_draw_leg(g, m, st, leaf_limit, True, peak)
            g.free()
        if args.draw_mesh in ("grids", "both"):
            out["draw_grids"] = run_draw_grids(synth, PBVH, peak)
        print(json.dumps(out))
        return 0
    if args.raycast_only:
        from dune_sculpt_gb300 import build as libbuild

        libbuild.build()
        from dune_sculpt_gb300 import synth
        from dune_sculpt_gb300.sculpt import PBVH

        out = {}
        if args.raycast_mesh in ("faces", "both"):
            m, _, leaf_limit, _ = workload()
            g = PBVH.build_mesh(m, leaf_limit)
            for _ in range(3):
                out["raycast_faces"] = run_raycast_leg(g, m, leaf_limit, True)
            g.free()
        if args.raycast_mesh in ("grids", "both"):
            out["raycast_grids"] = run_raycast_grids(synth, PBVH)
        print(json.dumps(out))
        return 0
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
