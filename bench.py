#!/usr/bin/env python
"""Benchmark of the sculpt-brush dab path: vertices displaced per second.

Default workload (one GPU, --workload multires): the multires (PBVH_GRIDS)
stroke of the fifth configuration, the largest single-GPU one: 50,000 grids of
17x17 elements (14.45 M) on a seeded noise-displaced torus (R=1, r=0.35), a
seeded value-noise mask, 256 dabs alternating draw / smooth / inflate, radius
0.04, strength 0.6; per dab the node search and the brush, then the grid
normal update with seam stitching and the bounding-box refit, as the
reference's stroke does.  Seeded synthetic input (no dataset).  A step is that
whole stroke.  --workload icosphere (masked X-mirrored smooth, 655,362 verts,
128 dabs), clay (clay strips on a 4,194,304-vertex sphere, X mirror, 256
dabs) and grid (draw on a 513x513 grid, 64 dabs) select the other
single-mesh configurations.

  value  : device-resident throughput, Sum(vertices displaced) / Sum(stroke
           time); the stroke is one launch of the persistent stroke kernel on
           the autotuned team (the whole GPU or a cluster), CUDA events on the
           mesh stream; positions, normals, masks and node boxes are restored
           from a device snapshot and L2 is flushed (256 MiB write, then a
           256 MiB read of another buffer) before every step, both outside the
           timed region.
  e2e    : the same stroke through the host-buffer entry point
           (sgpu_stroke_host_grids / sgpu_stroke_host) with page-locked
           buffers: positions and normals in, every leaf box refit, the
           stroke, positions out, all inside the event-timed region.
  roofline: k_team_stroke, the only kernel of a step: its algorithmic bytes
           per launch (the kernel's own counters, an instrumented run) / the
           mean step time of the timed run, against the measured HBM copy
           bandwidth.
  max_rel_err: the GPU's positions after the timed strokes against the FP32
           restatement (bit for bit), and the restatement's error against FP64
           per dab (each stage from the same input) and over the whole stroke.
  batch  : the 64-mesh uneven batch (fourth configuration), one persistent
           launch on the batch autotuner's team versus 64 sequential plain
           strokes; algorithmic bytes and HBM fraction.
  batched_clay / batched_multires: K independent seeded strokes on K meshes
           of the clay / multires workload in one persistent launch (the
           batched form), with their HBM fraction.
  cpu_baseline: the FP32 restatement (oracle, OpenMP over PBVH nodes) of the
           same whole stroke on all host cores.

--quick runs three persistent strokes of the workload and exits (the command
profiled with ncu).  --phases prints the persistent kernel's per-dab phase
profile on the single-mesh workloads.

--impl reference times the CPU restatement of the reference path on the same
workload and config (the reference cannot run the path: its brush code and
public headers are missing), the whole stroke per step.  Under torchrun (N>1)
each rank runs an independent replica (the path does not shard within a
mesh); rank 0 prints max-over-ranks timing.
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
from dataclasses import dataclass

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "vertices displaced/sec"
UNIT = "verts/s"
L2_NOTE = "flushed before every step (256 MiB device write, then 256 MiB read)"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--workload", choices=["multires", "icosphere", "clay", "grid"],
                    default="multires")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline and checks")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-mesh batch leg")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the batched clay / multires legs")
    ap.add_argument("--batched-k", type=int, default=8,
                    help="strokes (meshes) of the batched clay / multires legs")
    ap.add_argument("--no-legs", action="store_true", help="skip the ray-cast and draw legs")
    ap.add_argument("--quick", action="store_true",
                    help="three persistent strokes of the workload, no report (for ncu)")
    ap.add_argument("--team", type=int, default=0,
                    help="team for --quick: cluster size, -1 for the whole GPU, 0 autotuned; "
                         "for --quick-batch: cluster size, -1, or -2 for the lockstep launch")
    ap.add_argument("--quick-dabs", type=int, default=0,
                    help="--quick strokes only N dabs (a shorter launch for a full ncu "
                         "capture); 0: every dab")
    ap.add_argument("--quick-from", type=int, default=0,
                    help="first dab of the --quick-dabs slice (the multires stroke's first 23 "
                         "dabs fall on fully masked elements: they search, update and refit "
                         "but move nothing)")
    ap.add_argument("--quick-batch", action="store_true",
                    help="three launches of the 64-mesh batch on --team (8 when 0), no report "
                         "(the command profiled with ncu for the batch kernels)")
    ap.add_argument("--raycast-only", action="store_true",
                    help="1024-ray sgpu_raycast batches on the icosphere and on the multires "
                         "torus, one JSON line, and exit (the command profiled with ncu for "
                         "the ray kernels)")
    ap.add_argument("--raycast-mesh", choices=["faces", "grids", "both"], default="both",
                    help="meshes of --raycast-only")
    ap.add_argument("--draw-only", action="store_true",
                    help="full draw-buffer refreshes on the icosphere and on the multires "
                         "torus, one JSON line, and exit (the command profiled with ncu for "
                         "the draw kernels)")
    ap.add_argument("--draw-mesh", choices=["faces", "grids", "both"], default="both",
                    help="meshes of --draw-only")
    ap.add_argument("--phases", action="store_true",
                    help="per-phase profile of the persistent stroke on the single-mesh "
                         "workloads (one JSON line each), no report")
    ap.add_argument("--batched-only", action="store_true",
                    help="the batched clay / multires legs only, one JSON line")
    ap.add_argument("--batch-only", action="store_true",
                    help="the 64-mesh batch leg only (no CPU baseline), one JSON line")
    ap.add_argument("--batch-phases", action="store_true",
                    help="per-dab phase profile of the batch launches (64-mesh batch, K clay and "
                         "K multires strokes) on several team shapes, one JSON line each")
    return ap.parse_args()


@dataclass
class Workload:
    name: str
    kind: str            # "faces" or "grids"
    mesh: object         # synth.FacesMesh or synth.GridsMesh
    stroke: object       # synth.Stroke
    tools: object        # per-dab tools or None
    leaf_limit: int
    cfg: dict

    @property
    def nverts(self) -> int:
        return int(self.mesh.co.shape[0]) if self.kind == "grids" else int(self.mesh.totvert)


def multires_tools(synth, n):
    return np.array([(synth.TOOL_DRAW, synth.TOOL_SMOOTH, synth.TOOL_INFLATE)[d % 3]
                     for d in range(n)], dtype=np.int32)


def workload(name: str = "multires") -> Workload:
    """The single-mesh configurations; cfg is the same dict in both arms."""
    from dune_sculpt_gb300 import synth

    if name == "multires":
        g, dabs = synth.cfg5_multires()
        st = synth.Stroke(synth.TOOL_DRAW, 0.04, 0.6, synth.CURVE_SMOOTH, 0, dabs)
        cfg = {"workload": "multires_torus_50000x17x17_mixed", "grids": g.num_grids,
               "grid_size": g.grid_size, "elements": int(g.co.shape[0]),
               "dabs": int(dabs.shape[0]), "tools": "draw/smooth/inflate alternating",
               "radius": 0.04, "strength": 0.6, "symmetry": "none", "curve": "smooth",
               "mask": "seeded value noise", "leaf_limit": "34 grids (10000 // 289)",
               "l2": L2_NOTE}
        return Workload(name, "grids", g, st, multires_tools(synth, dabs.shape[0]), 0, cfg)
    if name == "clay":
        m, st, ll = synth.cfg3_sphere_clay()
        cfg = {"workload": "uvsphere2048_clay_strips_xmirror", "verts": int(m.totvert),
               "looptris": int(m.looptris.shape[0]), "dabs": int(st.dabs.shape[0]),
               "radius": st.radius, "strength": st.strength, "symmetry": "X", "curve": "sharp",
               "leaf_limit": ll, "l2": L2_NOTE}
        return Workload(name, "faces", m, st, None, ll, cfg)
    if name == "grid":
        m, st, ll = synth.cfg1_grid_draw()
        cfg = {"workload": "grid513_draw", "verts": int(m.totvert),
               "looptris": int(m.looptris.shape[0]), "dabs": int(st.dabs.shape[0]),
               "radius": st.radius, "strength": st.strength, "symmetry": "none",
               "curve": "smooth", "leaf_limit": ll, "l2": L2_NOTE}
        return Workload(name, "faces", m, st, None, ll, cfg)
    m, st, ll = synth.cfg2_icosphere_smooth()
    cfg = {"workload": "icosphere8_smooth_masked_xmirror", "verts": int(m.totvert),
           "looptris": int(m.looptris.shape[0]), "dabs": int(st.dabs.shape[0]),
           "radius": st.radius, "strength": st.strength, "symmetry": "X", "curve": "smooth",
           "leaf_limit": ll, "mask": "seeded smooth noise", "l2": L2_NOTE}
    return Workload("icosphere", "faces", m, st, None, ll, cfg)


def build_gpu(W: Workload):
    from dune_sculpt_gb300.sculpt import PBVH

    if W.kind == "grids":
        return PBVH.build_grids(W.mesh, W.leaf_limit)
    return PBVH.build_mesh(W.mesh, W.leaf_limit)


def build_oracle(W: Workload):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    pyoracle.build()
    o = (pyoracle.OracleMesh.grids(W.mesh, W.leaf_limit) if W.kind == "grids"
         else pyoracle.OracleMesh.faces(W.mesh, W.leaf_limit))
    o.recalc_all_normals()
    return o


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


def traffic_for(workload_name: str):
    tpath = os.path.join(ROOT, "profiles", "traffic_per_launch.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            return json.load(f).get(workload_name, {}).get("k_team_stroke")
    return None


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



def combine_ranks(dist, total_ms, e2e_ms, total_v, e2e_v):
    """Replicas: the slowest rank's times (max) and every rank's vertices
    (sum), so that value = all vertices / the job's time."""
    import torch

    t = torch.tensor([total_ms, e2e_ms], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    c = torch.tensor([total_v, e2e_v], dtype=torch.float64)
    dist.all_reduce(c, op=dist.ReduceOp.SUM)
    return float(t[0]), float(t[1]), int(c[0]), int(c[1])



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



def rel_err(x, ref) -> float:
    """Norm-wise relative error max|x - ref| / max|ref|."""
    ref = np.asarray(ref, dtype=np.float64)
    return float(np.abs(np.asarray(x, dtype=np.float64) - ref).max() /
                 max(np.abs(ref).max(), 1e-30))


def cpu_baseline(W: Workload, gpu_positions=None, fp64_stride: int = 16):
    """The FP32 restatement (oracle) of the same whole stroke on all host cores,
    timed; then, as the checker, the GPU's positions against it and the
    restatement's error against FP64 (per dab, each stage from the same input,
    every fp64_stride-th dab; and an independent FP64 stroke)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    o = build_oracle(W)
    threads = pyoracle.max_threads()
    t0 = time.perf_counter()
    tot, _ = o.stroke(W.stroke, which=1, nthreads=threads, dab_tools=W.tools)
    dt = time.perf_counter() - t0
    out = {"value": tot / dt, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"the whole stroke ({W.stroke.dabs.shape[0]} dabs), {tot} vertices "
                     f"displaced in {dt:.3f} s (FP32 restatement, OpenMP over PBVH nodes)",
           "seconds": dt}
    err = {}
    if gpu_positions is not None:
        co = o.co()
        err["positions_bit_exact_vs_fp32_restatement"] = bool(
            np.array_equal(np.ascontiguousarray(gpu_positions).view(np.uint32),
                           np.ascontiguousarray(co).view(np.uint32)))
        err["vs_fp32_restatement"] = rel_err(gpu_positions, co)
    o.close()
    o = build_oracle(W)
    _, local = o.stroke_local_error(W.stroke, dab_tools=W.tools, stride=fp64_stride,
                                    nthreads=threads)
    o.close()
    err["vs_fp64_per_dab"] = {k: float(f"{v:.3g}") for k, v in local.items()}
    err["vs_fp64_per_dab_measured_dabs"] = f"every {fp64_stride}th"
    o = build_oracle(W)
    o.stroke(W.stroke, which=3, nthreads=threads, dab_tools=W.tools)
    err["vs_fp64_whole_stroke"] = {"co": float(f"{rel_err(o.co(), o.co64()):.3g}"),
                                   "no": float(f"{np.abs(o.no() - o.no64()).max():.3g}")}
    o.close()
    err["note"] = ("positions: norm-wise relative max|x - ref| / max|ref|; normals, area: "
                   "absolute; per dab: each stage (brush, normal update, refit) from the same "
                   "input in both precisions; whole stroke: independent FP32 and FP64 strokes")
    return out, err


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    W = workload(args.workload)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    pyoracle.build()
    threads = pyoracle.max_threads()
    for _ in range(args.warmup):
        o = build_oracle(W)
        o.stroke(W.stroke, which=1, nthreads=threads, dab_tools=W.tools)
        o.close()
    total_v, total_s = 0, 0.0
    for _ in range(args.steps):
        o = build_oracle(W)  # every step starts from the same mesh state (untimed)
        t0 = time.perf_counter()
        tot, _ = o.stroke(W.stroke, which=1, nthreads=threads, dab_tools=W.tools)
        total_s += time.perf_counter() - t0
        total_v += tot
        o.close()
    value = total_v / total_s
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * total_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)", "config": W.cfg,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"the whole stroke ({W.stroke.dabs.shape[0]} dabs) per "
                                       "step (FP32 CPU restatement of the reference path: the "
                                       "reference has no brush code to run)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def team_label(team: int) -> str:
    return "whole GPU (one CTA per SM)" if team == -1 else f"cluster of {team} CTAs"


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
                                          STROKE_GRAPH, STROKE_TEAM, PinnedArray, autotune_batch,
                                          batch_stroke)

    W = workload(args.workload)
    st, tools = W.stroke, W.tools
    g = build_gpu(W)
    g.snapshot()
    team, tune_ms = g.autotune_team(st, dab_tools=tools)  # restores the snapshot

    def barrier():
        if world > 1:
            dist.barrier()

    for _ in range(args.warmup):
        g.restore()
        g.stroke(st, mode=STROKE_TEAM, dab_tools=tools)
    barrier()
    clocks = ClockSampler(local) if rank == 0 else None
    if clocks:
        clocks.wait_first()
    total_ms, total_v, launches = 0.0, 0, 0
    for _ in range(args.steps):
        g.restore()
        g.flush_l2()
        s = g.stroke(st, mode=STROKE_TEAM, dab_tools=tools)
        total_ms += s.gpu_ms
        total_v += s.verts_displaced
        launches += s.kernel_launches
    g.sync()
    barrier()
    clk = clocks.stop() if clocks else None
    final_positions = g.positions()

    # the same stroke through the per-call kernels: captured graph, and eager
    def plain(mode, n=2):
        ms, v = 0.0, 0
        for _ in range(n):
            g.restore()
            g.flush_l2()
            se = g.stroke(st, mode=mode, dab_tools=tools)
            ms += se.gpu_ms
            v += se.verts_displaced
        return {"value": v / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / n}

    g.restore()
    g.stroke(st, mode=STROKE_GRAPH, dab_tools=tools)  # graph capture outside the timing
    plain_graph = plain(STROKE_GRAPH)
    plain_eager = plain(STROKE_EAGER)

    # e2e through the host-buffer entry point with page-locked buffers
    V = W.nverts
    g.restore()
    nin = PinnedArray((V, 3), np.float32)
    nin.array[:] = g.normals()
    if W.kind == "grids":
        cin = PinnedArray((V, 3), np.float32)
        cin.array[:] = W.mesh.co
        cout = PinnedArray((V, 3), np.float32)

        def host_stroke():
            return g.stroke_host_grids(st, cin.array, cout.array, nin.array, dab_tools=tools,
                                       mode=STROKE_TEAM)

        h2d, d2h = V * 12 + V * 12, V * 12
    else:
        cin = PinnedArray((V,), W.mesh.verts.dtype)
        cin.array[:] = W.mesh.verts
        cout = PinnedArray((V,), W.mesh.verts.dtype)

        def host_stroke():
            return g.stroke_host(st, cin.array, cout.array, nin.array, dab_tools=tools,
                                 mode=STROKE_TEAM)

        h2d, d2h = V * 16 + V * 12, V * 16
    g.restore()
    host_stroke()
    e2e_ms, e2e_v = 0.0, 0
    for _ in range(args.steps):
        g.restore()
        g.flush_l2()
        s2 = host_stroke()
        e2e_ms += s2.gpu_ms
        e2e_v += s2.verts_displaced
    if W.kind != "grids":
        # blocks of 256 vertices the stroke changed (the record's 16 bytes),
        # written by the device into the page-locked output
        rec = np.ascontiguousarray(cout.array).view(np.uint32).reshape(V, -1)
        ref = np.ascontiguousarray(cin.array).view(np.uint32).reshape(V, -1)
        diff = np.any(rec != ref, axis=1)
        nblk = (V + 255) // 256
        changed = np.zeros(nblk * 256, dtype=bool)
        changed[:V] = diff
        changed = changed.reshape(nblk, 256).any(axis=1)
        d2h = int(sum(min(256, V - 256 * b) for b in np.nonzero(changed)[0])) * 16
        d2h_note = (f"the {int(changed.sum())} of {nblk} blocks of 256 vertices the stroke changed, "
                    "written by the device into the page-locked output; the others copied from the "
                    "input by host threads during the stroke (inside the timed call)")
    if W.kind == "grids":
        # the page-locked output takes only the grids the stroke changed from
        # the device (bitwise against the input); the rest arrives from the
        # input, copied by host threads while the stroke runs
        area = W.mesh.grid_size * W.mesh.grid_size
        changed = np.any((cout.array.view(np.uint32) != cin.array.view(np.uint32)).reshape(-1, 3 * area),
                         axis=1)
        d2h = int(changed.sum()) * area * 12
        d2h_note = (f"the {int(changed.sum())} of {changed.size} grids the stroke changed, written by the "
                    "device into the page-locked output; the other grids copied from the input by host "
                    "threads during the stroke (inside the timed call)")

    # phase profile of the persistent kernel (instrumented run, not timed)
    g.restore()
    g.flush_l2()
    phases, _, _ = g.stroke_team_profile(st, dab_tools=tools)
    alg_bytes = sum(p["bytes"] for p in phases.values())
    g.free()

    peak, peak_kind = measured_peaks()
    batch = None if args.no_batch else run_batch(synth, PBVH, batch_stroke, autotune_batch,
                                                  BATCH_TEAM, BATCH_SEQUENTIAL, peak,
                                                  no_cpu=args.no_cpu)
    batched = None if args.no_batched else run_batched(args.batched_k, peak, no_cpu=args.no_cpu)
    ray = draw = None
    if not args.no_legs:
        Wi = workload("icosphere")
        gi = build_gpu(Wi)
        gi.snapshot()
        ray = run_raycast_leg(gi, Wi.mesh, Wi.leaf_limit, args.no_cpu)
        gi.restore()
        draw = run_draw_leg(gi, Wi.mesh, Wi.stroke, Wi.leaf_limit, args.no_cpu, peak=peak)
        gi.free()

    if world > 1:
        total_ms, e2e_ms, total_v, e2e_v = combine_ranks(dist, total_ms, e2e_ms, total_v, e2e_v)
    if rank != 0:
        return 0

    step_ms = total_ms / args.steps
    achieved = alg_bytes / (step_ms / 1e3) / 1e9
    cpu, err = (None, None)
    if not args.no_cpu:
        cpu, err = cpu_baseline(W, final_positions)
    value = total_v / (total_ms / 1e3)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded; no dataset)", "config": W.cfg,
        "parallelism": f"replicas{world}",
        "mode": f"persistent stroke kernel, {team_label(team)} (autotuned)",
        "e2e": {"value": e2e_v / (e2e_ms / 1e3), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "d2h": d2h_note,
                "path": "sgpu_stroke_host_grids" if W.kind == "grids" else "sgpu_stroke_host"},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": "k_team_stroke", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS hbm_gbs)",
                     "alg_bytes_per_launch": alg_bytes, "mean_launch_ms": step_ms,
                     "traffic": traffic_for(W.cfg["workload"])},
        "max_rel_err": err,
        "team_phases_us_per_dab": {k: round(1e3 * v["ms"] / st.dabs.shape[0], 2)
                                   for k, v in phases.items()},
        "team_phases_alg_MB": {k: round(v["bytes"] / 1e6, 3) for k, v in phases.items()},
        "autotune_ms": {str(k): round(v, 3) for k, v in tune_ms.items()},
        "plain_graph": plain_graph,
        "plain_eager": plain_eager,
        "batch": batch,
        "batched": batched,
        "raycast": ray,
        "draw_buffers": draw,
        "cpu_baseline": ({k: v for k, v in cpu.items() if k != "seconds"} if cpu else None),
        "clocks": clk,
    }
    print(json.dumps(line))
    return 0


def stroke_alg_bytes(g, st, tools=None) -> float:
    """Algorithmic bytes of one persistent stroke of g (instrumented run; the
    caller restores the mesh before and after)."""
    phases, _, _ = g.stroke_team_profile(st, dab_tools=tools)
    return sum(p["bytes"] for p in phases.values())


def _team_kernel(shape) -> str:
    """The kernel a batch team shape launches."""
    from dune_sculpt_gb300.sculpt import TEAM_LOCKSTEP
    return "k_lock_stroke" if shape[0] == TEAM_LOCKSTEP else "k_team_stroke"


def run_batch(synth, PBVH, batch_stroke, autotune_batch, BATCH_TEAM, BATCH_SEQUENTIAL, peak,
              no_cpu=False, steps: int = 5):
    """The 64-mesh uneven batch: one persistent launch on the batch autotuner's
    team versus 64 sequential plain strokes (each a CUDA graph of per-call
    kernels); algorithmic bytes from each mesh's instrumented stroke."""
    batch = synth.cfg4_batch()
    gs = [PBVH.build_mesh(mm, ll) for (mm, _, ll) in batch]
    strokes = [s for (_, s, _) in batch]
    for p in gs:
        p.snapshot()
    nverts = sum(mm.totvert for (mm, _, _) in batch)
    shape, tune = autotune_batch(gs, strokes)  # restores every mesh
    alg = 0.0
    for p, s in zip(gs, strokes):
        p.restore()
        alg += stroke_alg_bytes(p, s)
        p.restore()
    ms_l, disp = [], 0
    for _ in range(steps):
        for p in gs:
            p.restore()
        gs[0].flush_l2()
        stats, ms = batch_stroke(gs, strokes, mode=BATCH_TEAM, cluster=0)
        ms_l.append(ms)
        disp = sum(s.verts_displaced for s in stats)
    ms = statistics.median(ms_l)
    for p in gs:
        p.restore()
    batch_stroke(gs, strokes, mode=BATCH_SEQUENTIAL)  # graph captures
    for p in gs:
        p.restore()
    stats, seq_ms = batch_stroke(gs, strokes, mode=BATCH_SEQUENTIAL)
    seq_disp = sum(s.verts_displaced for s in stats)
    achieved = alg / (ms / 1e3) / 1e9
    out = {"workload": "64 meshes (grid/uv-sphere alternating, log-uniform 1e4-5e5 verts, "
                       f"{nverts} verts total), 32-dab draw/inflate strokes",
           "persistent": {"value": disp / (ms / 1e3), "unit": UNIT, "ms_per_step": ms,
                          "team": {"cluster": shape[0], "ctas_per_sm": shape[1]},
                          "steps": steps},
           "sequential_plain": {"value": seq_disp / (seq_ms / 1e3), "unit": UNIT,
                                "ms_per_step": seq_ms},
           "speedup": (disp / ms) / (seq_disp / seq_ms),
           "roofline": {"bound": "hbm", "kernel": _team_kernel(shape), "alg_bytes": alg,
                        "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": achieved / peak},
           "autotune_ms": {f"{c[0]}x{c[1]}": round(t, 3) for c, t in tune.items()}}
    for p in gs:
        p.free()
    if not no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle

        pyoracle.build()
        threads = pyoracle.max_threads()
        k, tot, dt = 8, 0, 0.0
        for mm, s, ll in batch[:k]:
            o = pyoracle.OracleMesh.faces(mm, ll)
            o.recalc_all_normals()
            t0 = time.perf_counter()
            n, _ = o.stroke(s, which=1, nthreads=threads)
            dt += time.perf_counter() - t0
            tot += n
            o.close()
        out["cpu_baseline"] = {"value": tot / dt, "unit": UNIT, "cores": threads, "kind": "port",
                               "sample": f"the first {k} of the 64 strokes, one after another "
                                         "(FP32 restatement, OpenMP over PBVH nodes)"}
    return out


def run_batched(K: int, peak, no_cpu=False, steps: int = 3):
    """The batched form of the clay-strips and multires workloads: K
    independent seeded strokes on K meshes of that workload (same geometry,
    separate handles), in one persistent launch on the batch autotuner's team;
    against the K strokes run one after another on the single-stroke team."""
    from dune_sculpt_gb300 import synth
    from dune_sculpt_gb300.sculpt import (BATCH_TEAM, STROKE_TEAM, autotune_batch,
                                          batch_stroke)

    out = {}
    for name in ("clay", "multires"):
        W = workload(name)
        strokes, tools = [], None
        for k in range(K):
            if name == "clay":
                dabs = synth.arc_dabs(synth.SEED_BASE + 200 + k, W.stroke.dabs.shape[0],
                                      0.1 * 2 * W.stroke.radius)
            else:
                dabs = synth.torus_dabs(synth.SEED_BASE + 200 + k, W.stroke.dabs.shape[0],
                                        W.stroke.radius)
            s = synth.Stroke(W.stroke.tool, W.stroke.radius, W.stroke.strength,
                             W.stroke.curve_preset, W.stroke.symmetry, dabs)
            strokes.append(s)
        if W.tools is not None:
            tools = np.concatenate([W.tools] * K)
        gs = [build_gpu(W) for _ in range(K)]
        for p in gs:
            p.snapshot()
        shape, tune = autotune_batch(gs, strokes, dab_tools=tools)
        alg, single_ms, single_v = 0.0, 0.0, 0
        best_single, _ = gs[0].autotune_team(strokes[0], dab_tools=W.tools)
        for p, s in zip(gs, strokes):
            p.set_team(best_single)
            p.restore()
            alg += stroke_alg_bytes(p, s, W.tools)
            p.restore()
            p.flush_l2()
            r = p.stroke(s, mode=STROKE_TEAM, dab_tools=W.tools)
            single_ms += r.gpu_ms
            single_v += r.verts_displaced
            p.restore()
        ms_l, disp = [], 0
        for _ in range(steps):
            for p in gs:
                p.restore()
            gs[0].flush_l2()
            stats, ms = batch_stroke(gs, strokes, mode=BATCH_TEAM, cluster=0, dab_tools=tools)
            ms_l.append(ms)
            disp = sum(s.verts_displaced for s in stats)
        ms = statistics.median(ms_l)
        achieved = alg / (ms / 1e3) / 1e9
        out[name] = {"workload": f"{K} independent seeded strokes of the {W.cfg['workload']} "
                                 "workload on K meshes, one persistent launch",
                     "strokes": K, "value": disp / (ms / 1e3), "unit": UNIT,
                     "ms_per_batch": ms,
                     "team": {"cluster": shape[0], "ctas_per_sm": shape[1]},
                     "roofline": {"bound": "hbm", "kernel": _team_kernel(shape), "alg_bytes": alg,
                                  "achieved": achieved, "peak": peak, "unit": "GB/s",
                                  "frac": achieved / peak},
                     "one_after_another": {"value": single_v / (single_ms / 1e3), "unit": UNIT,
                                           "ms": single_ms, "team": best_single},
                     "speedup_vs_one_after_another": (disp / ms) / (single_v / single_ms),
                     "autotune_ms": {f"{c[0]}x{c[1]}": round(t, 3) for c, t in tune.items()}}
        for p in gs:
            p.free()
    return out


def run_quick(args):
    from dune_sculpt_gb300 import build as libbuild

    libbuild.build()
    from dune_sculpt_gb300.sculpt import STROKE_TEAM

    W = workload(args.workload)
    st, tools = W.stroke, W.tools
    if args.quick_dabs > 0:
        from dataclasses import replace

        lo, hi = args.quick_from, args.quick_from + args.quick_dabs
        st = replace(st, dabs=st.dabs[lo:hi])
        tools = None if tools is None else tools[lo:hi]
    g = build_gpu(W)
    g.snapshot()
    if args.team:
        g.set_team(args.team)
    else:
        g.autotune_team(st, dab_tools=tools)
    for _ in range(3):
        g.restore()
        s = g.stroke(st, mode=STROKE_TEAM, dab_tools=tools)
    print(f"quick: {s.verts_displaced} vertices displaced, {s.gpu_ms:.3f} ms, team {g.team()}")
    return 0


def run_quick_batch(args):
    """Three launches of the 64-mesh batch on one team shape."""
    from dune_sculpt_gb300 import build as libbuild

    libbuild.build()
    from dune_sculpt_gb300 import synth
    from dune_sculpt_gb300.sculpt import BATCH_TEAM, PBVH, batch_stroke

    batch = synth.cfg4_batch()
    gs = [PBVH.build_mesh(m, ll) for (m, _, ll) in batch]
    strokes = [st for (_, st, _) in batch]
    for p in gs:
        p.snapshot()
    team = args.team or 8
    for _ in range(3):
        for p in gs:
            p.restore()
        stats, ms = batch_stroke(gs, strokes, mode=BATCH_TEAM, cluster=team)
    print(f"quick batch: {sum(x.verts_displaced for x in stats)} vertices displaced, "
          f"{ms:.3f} ms, team {team}")
    return 0


def run_phases(args):
    """Per-dab phase times of the persistent stroke kernel on the single-mesh
    workloads: the autotuned team, the best of three L2-flushed strokes, then
    one instrumented stroke (phase timers of the team's first thread)."""
    from dune_sculpt_gb300 import build as libbuild

    libbuild.build()
    from dune_sculpt_gb300 import synth
    from dune_sculpt_gb300.sculpt import STROKE_GRAPH, STROKE_TEAM

    def one(name, g, st, tools=None, graph=False):
        g.snapshot()
        best, tune = g.autotune_team(st, dab_tools=tools)
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
            "workload": name, "team": best, "ms_per_stroke": round(min(times), 3),
            "us_per_dab": round(1000 * min(times) / nd, 2),
            "verts_displaced": stats.verts_displaced, **extra,
            "autotune_ms": {str(k): round(v, 3) for k, v in tune.items()},
            "phase_us_per_dab": {k: round(1000 * v["ms"] / nd, 2) for k, v in ph.items()},
            "phase_alg_MB_per_stroke": {k: round(v["bytes"] / 1e6, 2) for k, v in ph.items()}}),
            flush=True)
        g.free()

    for name in ("grid", "icosphere", "clay", "multires"):
        W = workload(name)
        one(W.cfg["workload"], build_gpu(W), W.stroke, W.tools)
    # the stroke-start brushes on the icosphere (128 dabs, X mirror):
    # persistent and graph-replayed
    W = workload("icosphere")
    st = W.stroke
    grab = synth.grab_dabs(synth.SEED_BASE + 40, st.dabs.shape[0], 0.0005)
    for name, tool, dabs, kw in (
            ("grab", synth.TOOL_GRAB, grab, {}),
            ("layer", synth.TOOL_LAYER, st.dabs, {"height": 0.3}),
            ("elastic_deform", synth.TOOL_ELASTIC_DEFORM, grab, {})):
        so = synth.Stroke(tool, st.radius, st.strength, synth.CURVE_SMOOTH, synth.SYMM_X, dabs, **kw)
        one(f"icosphere8_{name}_xmirror", build_gpu(W), so, graph=True)
    return 0


def batched_strokes(synth, W, K: int):
    """K independent seeded strokes of a single-mesh workload (the batched form)."""
    strokes = []
    for k in range(K):
        if W.name == "clay":
            dabs = synth.arc_dabs(synth.SEED_BASE + 200 + k, W.stroke.dabs.shape[0],
                                  0.1 * 2 * W.stroke.radius)
        else:
            dabs = synth.torus_dabs(synth.SEED_BASE + 200 + k, W.stroke.dabs.shape[0],
                                    W.stroke.radius)
        strokes.append(synth.Stroke(W.stroke.tool, W.stroke.radius, W.stroke.strength,
                                    W.stroke.curve_preset, W.stroke.symmetry, dabs))
    return strokes


def run_batch_phases(args):
    """Per-dab phase times of the batch launches: the 64-mesh batch and the K
    clay / multires strokes, each on 8-CTA clusters (two per SM), 16-CTA
    clusters and the lockstep launch (one and two CTAs per SM); best of three
    instrumented launches (phase timers of the launch's first thread)."""
    from dune_sculpt_gb300 import build as libbuild

    libbuild.build()
    from dune_sculpt_gb300 import synth
    from dune_sculpt_gb300.sculpt import (DEBUG_LOCKSTEP_PER_SM, PBVH, TEAM_LOCKSTEP,
                                          SculptGPUError, batch_team_profile, debug_inject)

    def profile(name, gs, strokes, tools, ndabs):
        for p in gs:
            p.snapshot()
        for label, cl, per in (("cluster8", 8, 0), ("cluster16", 16, 0),
                               ("lockstep_1_per_sm", TEAM_LOCKSTEP, 1),
                               ("lockstep_2_per_sm", TEAM_LOCKSTEP, 2)):
            best = None
            try:
                for _ in range(3):
                    for p in gs:
                        p.restore()
                    gs[0].flush_l2()
                    debug_inject(DEBUG_LOCKSTEP_PER_SM, per)
                    try:
                        ph, ms, st = batch_team_profile(gs, strokes, cluster=cl, dab_tools=tools)
                    finally:
                        debug_inject(DEBUG_LOCKSTEP_PER_SM, 0)
                    if best is None or ms < best[1]:
                        best = (ph, ms, st)
            except SculptGPUError as e:
                print(json.dumps({"batch": name, "team": label, "unavailable": str(e)}), flush=True)
                continue
            ph, ms, st = best
            print(json.dumps({"batch": name, "team": label, "ms": round(ms, 3),
                              "verts_displaced": sum(x.verts_displaced for x in st),
                              "phase_us_per_dab": {k: round(1000 * v / ndabs, 2)
                                                   for k, v in ph.items()}}), flush=True)
        for p in gs:
            p.restore()
            p.free()

    batch = synth.cfg4_batch()
    profile("64_meshes_cfg4", [PBVH.build_mesh(m, ll) for (m, _, ll) in batch],
            [st for (_, st, _) in batch], None, batch[0][1].dabs.shape[0])
    for name in ("clay", "multires"):
        W = workload(name)
        K = args.batched_k
        tools = np.concatenate([W.tools] * K) if W.tools is not None else None
        profile(f"{K}x_{W.cfg['workload']}", [build_gpu(W) for _ in range(K)],
                batched_strokes(synth, W, K), tools, W.stroke.dabs.shape[0])
    return 0


def main():
    args = parse_args()
    if args.batch_phases:
        return run_batch_phases(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.quick:
        return run_quick(args)
    if args.quick_batch:
        return run_quick_batch(args)
    if args.phases:
        return run_phases(args)
    if args.batch_only:
        from dune_sculpt_gb300 import build as libbuild

        libbuild.build()
        from dune_sculpt_gb300 import synth
        from dune_sculpt_gb300.sculpt import (BATCH_SEQUENTIAL, BATCH_TEAM, PBVH, autotune_batch,
                                              batch_stroke)

        print(json.dumps(run_batch(synth, PBVH, batch_stroke, autotune_batch, BATCH_TEAM,
                                   BATCH_SEQUENTIAL, measured_peaks()[0], no_cpu=True)))
        return 0
    if args.batched_only:
        from dune_sculpt_gb300 import build as libbuild

        libbuild.build()
        print(json.dumps(run_batched(args.batched_k, measured_peaks()[0], no_cpu=True)))
        return 0
    if args.draw_only:
        from dune_sculpt_gb300 import build as libbuild

        libbuild.build()
        from dune_sculpt_gb300 import synth
        from dune_sculpt_gb300.sculpt import PBVH

        peak = measured_peaks()[0]
        out = {}
        if args.draw_mesh in ("faces", "both"):
            W = workload("icosphere")
            g = build_gpu(W)
            g.snapshot()
            out["draw_faces"] = run_draw_leg(g, W.mesh, W.stroke, W.leaf_limit, True, peak)
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
            W = workload("icosphere")
            g = build_gpu(W)
            for _ in range(3):
                out["raycast_faces"] = run_raycast_leg(g, W.mesh, W.leaf_limit, True)
            g.free()
        if args.raycast_mesh in ("grids", "both"):
            out["raycast_grids"] = run_raycast_grids(synth, PBVH)
        print(json.dumps(out))
        return 0
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
