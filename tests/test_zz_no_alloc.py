"""The allocation-free smooth dab (sgpu_smooth_dab_noalloc) against the
handle-based smooth brush (sgpu_do_smooth_brush) through the C ABI.

The caller of the allocation-free entry point owns its device arrays; this test
plays that caller by allocating them itself through the CUDA runtime, then
checks that two calls in a row move the vertices exactly as the existing entry
point does (bit for bit, the tolerance of every parity test here).  Collected
last so that a run stopping at the first failure has run everything else.
"""
import ctypes as C
import ctypes.util
import glob
import os

import numpy as np
import pytest

from dune_sculpt_gb300 import synth
from dune_sculpt_gb300.sculpt import PBVH, make_brush

from helpers import bits_equal, first_diff, small_icosphere

pytestmark = pytest.mark.gpu

H2D, D2H = 1, 2


def _cudart():
    names = [ctypes.util.find_library("cudart")]
    names += sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*"))
    names += sorted(glob.glob("/usr/local/cuda/targets/*/lib/libcudart.so*"))
    for n in names:
        if n:
            try:
                rt = C.CDLL(n)
                rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
                rt.cudaFree.argtypes = [C.c_void_p]
                rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
                return rt
            except OSError:
                continue
    pytest.fail("CUDA runtime library not found")


class DevArray:
    """Device memory owned by the caller (not by libsculptgpu)."""

    def __init__(self, rt, host: np.ndarray):
        self.rt = rt
        self.nbytes = max(host.nbytes, 16)
        self.ptr = C.c_void_p()
        assert rt.cudaMalloc(C.byref(self.ptr), self.nbytes) == 0
        self.upload(host)

    def upload(self, host):
        h = np.ascontiguousarray(host)
        if h.nbytes:
            assert self.rt.cudaMemcpy(self.ptr, h.ctypes.data_as(C.c_void_p), h.nbytes, H2D) == 0

    def download(self, like: np.ndarray) -> np.ndarray:
        out = np.empty_like(like)
        assert self.rt.cudaMemcpy(out.ctypes.data_as(C.c_void_p), self.ptr, out.nbytes, D2H) == 0
        return out

    def free(self):
        if self.ptr:
            self.rt.cudaFree(self.ptr)
            self.ptr = None


def one_ring(m):
    """The one-ring in CSR form: per polygon around a vertex (ascending), the
    previous then the next corner vertex, first occurrences only."""
    V = m.totvert
    ls = m.polys["loopstart"]
    tl = m.polys["totloop"]
    lv = m.loops["v"].astype(np.int64)
    around = [[] for _ in range(V)]
    for p in range(m.polys.shape[0]):
        c = lv[ls[p]:ls[p] + tl[p]]
        n = len(c)
        for k in range(n):
            around[c[k]].append((c[(k - 1) % n], c[(k + 1) % n]))
    off = np.zeros(V + 1, dtype=np.int32)
    idx = []
    for v in range(V):
        seen = []
        for a, b in around[v]:
            for u in (a, b):
                if u != v and u not in seen:
                    seen.append(u)
        idx += seen
        off[v + 1] = len(idx)
    return off, np.asarray(idx, dtype=np.int32)


def candidates(pbvh, nodes):
    nd = pbvh.nodes()
    vi = pbvh.vert_indices()
    parts = [vi[nd["vert_off"][n]:nd["vert_off"][n] + nd["uniq"][n]] for n in nodes]
    return np.concatenate(parts).astype(np.int32) if parts else np.zeros(0, np.int32)


def _noalloc_lib(gpu):
    lib = gpu.load()
    lib.sgpu_smooth_dab_noalloc.argtypes = [C.c_void_p] * 7 + [C.c_int, C.c_void_p,
                                                                C.c_void_p, C.c_void_p]
    return lib


@pytest.mark.parametrize("strength,frontface", [(0.7, False), (0.25, False), (1.0, False),
                                                (0.7, True)])
def test_noalloc_smooth_matches_handle_path(gpu, strength, frontface):
    """Two calls in a row equal sgpu_do_smooth_brush bit for bit: strength 0.7
    (two full sweeps and a fractional one), 0.25 (one full sweep and a last
    one of strength zero), 1.0 (four full sweeps and a last zero one), and the
    front-face falloff, which reads the normals, with an automask."""
    lib = _noalloc_lib(gpu)
    rt = _cudart()
    m = small_icosphere(4)
    automask = None
    if frontface:
        automask = (0.25 + 0.75 * synth.value_noise(synth.SEED_BASE + 71, 3,
                                                    m.verts["co"].astype(np.float64), 3.0))
        automask = automask.astype(np.float32)
    g = PBVH.build_mesh(m, 200, automask=automask)
    verts0 = g.verts()
    off, idx = one_ring(m)
    d_co = DevArray(rt, verts0)
    d_mask = DevArray(rt, m.mask)
    d_off = DevArray(rt, off)
    d_idx = DevArray(rt, idx)
    d_no = d_am = None
    if frontface:
        no4 = np.zeros((m.totvert, 4), np.float32)
        no4[:, :3] = g.normals()
        d_no = DevArray(rt, no4)
        d_am = DevArray(rt, automask)
    view = (0.3, -0.4, 0.866)
    st = synth.Stroke(synth.TOOL_SMOOTH, 0.18, strength, synth.CURVE_SMOOTH, 0, None,
                      flag=(1 << 27) if frontface else 0, view_normal=view)
    brush = make_brush(st)
    co = g.positions()
    try:
        for call, vid in enumerate((17, 300)):  # two calls in a row
            center = np.ascontiguousarray(co[vid], dtype=np.float32)
            rsq = float(np.float32(np.float32(st.radius) * np.float32(st.radius)))
            nodes = g.search_gather_sphere(center, rsq)
            cand = candidates(g, nodes)
            assert 0 < cand.size <= 65536
            d_verts = DevArray(rt, cand)
            g.do_smooth_brush(st, center, [1.0, 0.0, 0.0], nodes)
            rc = lib.sgpu_smooth_dab_noalloc(d_co.ptr, d_no.ptr if d_no else None, d_mask.ptr,
                                             d_am.ptr if d_am else None, d_off.ptr, d_idx.ptr,
                                             d_verts.ptr, cand.size, C.byref(brush),
                                             center.ctypes.data_as(C.c_void_p), None)
            d_verts.free()
            assert rc == 0, lib.sgpu_last_error()
            got = d_co.download(verts0)
            want = g.verts()
            assert bits_equal(got["co"], want["co"]), f"call {call}: " + first_diff(got["co"], want["co"])
            assert np.array_equal(got["flag"], want["flag"])
            moved = np.abs(got["co"] - verts0["co"]).max()
            assert moved > 0.0
        # sizes beyond the fixed scratch are rejected before any launch
        rc = lib.sgpu_smooth_dab_noalloc(d_co.ptr, None, None, None, d_off.ptr, d_idx.ptr,
                                         d_off.ptr, 65537, C.byref(brush),
                                         np.zeros(3, np.float32).ctypes.data_as(C.c_void_p), None)
        assert rc == 1 and b"65536" in lib.sgpu_last_error()
    finally:
        for a in (d_co, d_mask, d_off, d_idx, d_no, d_am):
            if a is not None:
                a.free()


def test_noalloc_empty_call_and_front_face_without_normals(gpu):
    """nverts = 0 returns SGPU_OK and leaves the positions alone (it only looks
    up the scratch address: the warm-up call a caller makes at set-up); the
    front-face falloff without normals is rejected."""
    lib = _noalloc_lib(gpu)
    rt = _cudart()
    m = small_icosphere(3)
    verts0 = np.ascontiguousarray(m.verts)
    off, idx = one_ring(m)
    d_co = DevArray(rt, verts0)
    d_off = DevArray(rt, off)
    d_idx = DevArray(rt, idx)
    brush = make_brush(synth.Stroke(synth.TOOL_SMOOTH, 0.2, 0.5, synth.CURVE_SMOOTH, 0, None))
    loc = np.zeros(3, np.float32)
    try:
        rc = lib.sgpu_smooth_dab_noalloc(d_co.ptr, None, None, None, d_off.ptr, d_idx.ptr, None,
                                         0, C.byref(brush), loc.ctypes.data_as(C.c_void_p), None)
        assert rc == 0, lib.sgpu_last_error()
        assert bits_equal(d_co.download(verts0)["co"], verts0["co"])
        ff = make_brush(synth.Stroke(synth.TOOL_SMOOTH, 0.2, 0.5, synth.CURVE_SMOOTH, 0, None,
                                     flag=1 << 27))
        rc = lib.sgpu_smooth_dab_noalloc(d_co.ptr, None, None, None, d_off.ptr, d_idx.ptr,
                                         d_off.ptr, 1, C.byref(ff),
                                         loc.ctypes.data_as(C.c_void_p), None)
        assert rc == 1 and b"normals" in lib.sgpu_last_error()
        assert bits_equal(d_co.download(verts0)["co"], verts0["co"])
    finally:
        for a in (d_co, d_off, d_idx):
            a.free()
