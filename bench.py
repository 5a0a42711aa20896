#!/usr/bin/env python
"""Benchmark of the sculpt-brush dab path: vertices displaced per second.

Default workload (one GPU): the masked, X-mirrored smooth-brush stroke of 128
dabs on a noisy level-8 icosphere (655,362 vertices, 1,310,720 looptris,
PBVH leaf limit 5000 looptris), seeded synthetic input.  A step is that whole
stroke: per dab and symmetry pass the node search and the brush, then the
normal update and bounding-box refit, as the reference's stroke does.

  value  : device-resident throughput — Sum(vertices displaced) / Sum(stroke
           time), stroke time from CUDA events on the mesh stream, the stroke
           replayed from its captured CUDA graph; positions, normals and node
           boxes restored from a device snapshot and L2 flushed (256 MiB write)
           before every step, both outside the timed region.
  e2e    : the same through sgpu_stroke_host with page-locked host buffers:
           H2D of positions and normals, full box refit, stroke, D2H of
           positions, all inside the event-timed region.
  roofline: the dominant kernel of an event-profiled eager run: algorithmic
           bytes per launch / mean launch time, against the measured HBM copy
           bandwidth.
  cpu_baseline: the FP32 CPU restatement (oracle, OpenMP over PBVH nodes) on
           the host cores, same stroke.

--impl reference times the CPU restatement of the reference path (the
reference itself does not build: its headers and brush code are missing).
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
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--cpu-sample-dabs", type=int, default=0,
                    help="dabs of the stroke in the CPU sample (0 = whole stroke)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    return ap.parse_args()


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
           "l2": "flushed before every step (256 MiB device write)"}
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
    o = pyoracle.OracleMesh.faces(m, leaf_limit)
    o.recalc_all_normals()
    threads = pyoracle.max_threads()
    co0 = o.co()
    for _ in range(args.warmup):
        o.set_co(co0)
        o.stroke(st, which=1, nthreads=threads, dabs=dabs)
    total_v, total_s = 0, 0.0
    for _ in range(args.steps):
        o.set_co(co0)
        t0 = time.perf_counter()
        tot, _ = o.stroke(st, which=1, nthreads=threads, dabs=dabs)
        total_s += time.perf_counter() - t0
        total_v += tot
    value = total_v / total_s
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * total_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)", "config": cfg,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"first {sample} of {st.dabs.shape[0]} dabs per step "
                                       "(FP32 CPU restatement of the reference path; the "
                                       "reference itself does not compile)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_gpu(args):
    world, rank, local = dist_env()
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
        import torch.distributed as dist

        dist.init_process_group("gloo")
    from dune_sculpt_gb300 import build as libbuild

    libbuild.build()
    from dune_sculpt_gb300 import sculpt
    from dune_sculpt_gb300.sculpt import PBVH, STROKE_EAGER, STROKE_GRAPH, PinnedArray

    m, st, leaf_limit, cfg = workload()
    g = PBVH.build_mesh(m, leaf_limit)
    g.snapshot()

    def barrier():
        if world > 1:
            dist.barrier()

    # warm-up (graph capture happens on the first call)
    for _ in range(args.warmup):
        g.restore()
        g.stroke(st, mode=STROKE_GRAPH)
    barrier()
    clocks = ClockSampler(local) if rank == 0 else None
    total_ms, total_v, launches = 0.0, 0, 0
    for _ in range(args.steps):
        g.restore()
        g.flush_l2()
        s = g.stroke(st, mode=STROKE_GRAPH)
        total_ms += s.gpu_ms
        total_v += s.verts_displaced
        launches += s.kernel_launches
    g.sync()
    barrier()
    clk = clocks.stop() if clocks else None
    graph_nodes = s.graph_nodes

    # plain (call-by-call) launches of the same stroke, for comparison
    eager_ms, eager_v = 0.0, 0
    for _ in range(2):
        g.restore()
        g.flush_l2()
        se = g.stroke(st, mode=STROKE_EAGER)
        eager_ms += se.gpu_ms
        eager_v += se.verts_displaced

    # e2e through the host-buffer entry point with page-locked buffers
    V = m.totvert
    vin = PinnedArray((V,), m.verts.dtype)
    vin.array[:] = m.verts
    g.restore()
    nin = PinnedArray((V, 3), np.float32)
    nin.array[:] = g.normals()
    vout = PinnedArray((V,), m.verts.dtype)
    g.restore()
    g.stroke_host(st, vin.array, vout.array, nin.array)  # warm (graph capture)
    e2e_ms, e2e_v = 0.0, 0
    for _ in range(args.steps):
        g.restore()
        g.flush_l2()
        s2 = g.stroke_host(st, vin.array, vout.array, nin.array)
        e2e_ms += s2.gpu_ms
        e2e_v += s2.verts_displaced

    # kernel profile (event-bracketed eager run with algorithmic-byte counters)
    g.restore()
    g.flush_l2()
    prof, _ = g.stroke_profile(st)

    # max over ranks
    if world > 1:
        import torch

        t = torch.tensor([total_ms, e2e_ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms, e2e_ms = float(t[0]), float(t[1])
        c = torch.tensor([total_v, e2e_v], dtype=torch.float64)
        dist.all_reduce(c, op=dist.ReduceOp.SUM)
        total_v, e2e_v = int(c[0]), int(c[1])
    if rank != 0:
        return 0

    peak, peak_kind = measured_peaks()
    dom = max(prof.items(), key=lambda kv: kv[1]["total_ms"])
    dname, d = dom
    achieved = d["alg_bytes"] / (d["total_ms"] / 1e3) / 1e9 if d["total_ms"] > 0 else 0.0
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic_per_launch.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            traffic = json.load(f).get(cfg["workload"], {}).get(dname)
    cpu = None
    if not args.no_cpu:
        cpu = cpu_baseline(m, st, leaf_limit, args.cpu_sample_dabs)
    value = total_v / (total_ms / 1e3)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded icosphere, Gaussian radial noise, smooth-noise mask)",
        "config": dict(cfg, parallelism=f"replicas{world}", mode="CUDA graph per stroke"),
        "e2e": {"value": e2e_v / (e2e_ms / 1e3), "unit": UNIT,
                "h2d_bytes_per_step": int(V * 16 + V * 12), "d2h_bytes_per_step": int(V * 16)},
        "gpu_launches": launches,
        "graph_nodes_per_step": graph_nodes,
        "roofline": {"bound": "hbm", "kernel": dname, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                     "alg_bytes_per_launch": d["alg_bytes"] / d["launches"],
                     "mean_launch_us": 1e3 * d["total_ms"] / d["launches"],
                     "traffic": traffic},
        "kernels": {k: {"launches": v["launches"], "total_ms": round(v["total_ms"], 4),
                        "GBps": (v["alg_bytes"] / (v["total_ms"] / 1e3) / 1e9)
                        if v["total_ms"] > 0 else None} for k, v in prof.items()},
        "plain_eager": {"value": eager_v / (eager_ms / 1e3), "unit": UNIT,
                        "ms_per_step": eager_ms / 2},
        "cpu_baseline": ({k: v for k, v in cpu.items() if k != "seconds"} if cpu else None),
        "clocks": clk,
    }
    print(json.dumps(line))
    return 0


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
