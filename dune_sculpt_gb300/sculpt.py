"""Python binding of libsculptgpu (the C ABI declared in include/sculpt_gpu.h).

``PBVH`` mirrors the reference's PBVH call surface for the sculpt dab path
(source/dune/kernel/intern/pbvh.c): ``build_mesh`` / ``build_grids``
(BKE_pbvh_build_mesh / _grids), ``search_gather_sphere``
(BKE_pbvh_search_gather with the sculpt sphere callback), ``do_draw_brush`` and
the other ``do_*_brush`` entry points, ``update_normals``
(BKE_pbvh_update_normals), ``update_bounds`` (BKE_pbvh_update_bounds) and
``node_mark_update``.  Errors raise ``SculptGPUError`` with the library's status
code, as the C entry points return it.  There is no CPU fallback: without the
compiled library or a GPU every call fails.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import synth

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libsculptgpu.so")

OK, ERR_INVALID_ARG, ERR_OOM, ERR_CUDA, ERR_TIMEOUT, ERR_BOUNDS, ERR_UNSUPPORTED = range(7)
PBVH_Leaf, PBVH_UpdateNormals, PBVH_UpdateBB, PBVH_UpdateOriginalBB = 1, 2, 4, 8
PBVH_UpdateDrawBuffers, PBVH_UpdateRedraw = 16, 32
STROKE_EAGER, STROKE_GRAPH, STROKE_TEAM = 0, 1, 2
BATCH_SEQUENTIAL, BATCH_TEAM = 0, 1
TEAM_GRID = -1  # SGPU_TEAM_GRID: every SM of the GPU works on one stroke
TEAM_LOCKSTEP = -2  # SGPU_TEAM_LOCKSTEP: every SM on every stroke of a batch, phase work pooled
TEAM_SIZES = (TEAM_GRID, 1, 2, 4, 8, 16)  # sgpu_autotune_team's candidates, in order
BATCH_TEAM_CANDIDATES = ((16, 1), (8, 1), (8, 2), (4, 1), (4, 2), (2, 2), (TEAM_GRID, 1),
                         (TEAM_LOCKSTEP, 1), (TEAM_LOCKSTEP, 2))
INJECT_ALLOC_FAIL, INJECT_WAIT_NS, INJECT_BARRIER_EXTRA = 1, 2, 3
DEBUG_LOCKSTEP_PER_SM = 4  # test hook: CTAs per SM of lockstep launches (0: the team shape's)


class SculptGPUError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"libsculptgpu error {code}: {msg}")
        self.code = code


class SGPU_Brush(C.Structure):
    _fields_ = [("sculpt_tool", C.c_int), ("flag", C.c_int), ("symmetry", C.c_int),
                ("curve_preset", C.c_int), ("radius", C.c_float), ("strength", C.c_float),
                ("normal_radius_factor", C.c_float), ("area_radius_factor", C.c_float),
                ("plane_offset", C.c_float), ("view_normal", C.c_float * 3),
                ("use_original_bb", C.c_int), ("crease_pinch_factor", C.c_float),
                ("elastic_deform_type", C.c_int),
                ("elastic_deform_volume_preservation", C.c_float), ("height", C.c_float)]


class SGPU_MeshInfo(C.Structure):
    _fields_ = [("type", C.c_int), ("totvert", C.c_int), ("totnode", C.c_int),
                ("totleaf", C.c_int), ("leaf_limit", C.c_int), ("totprim", C.c_int),
                ("leaf_vert_entries", C.c_int), ("grid_size", C.c_int)]


class SGPU_StrokeStats(C.Structure):
    _fields_ = [("verts_displaced", C.c_int64), ("gpu_ms", C.c_float),
                ("kernel_launches", C.c_int), ("graph_nodes", C.c_int)]


KERNEL_KINDS = 10


class SGPU_KernelProfile(C.Structure):
    _fields_ = [("name", C.c_char * 24), ("launches", C.c_int), ("total_ms", C.c_float),
                ("alg_bytes", C.c_double)]


TEAM_PHASES = ("search", "area", "brush", "smooth_apply", "normals_refit", "flush", "job",
               "grid_faces", "grid_seams")


class SGPU_TeamProfile(C.Structure):
    _fields_ = [("total_ms", C.c_float), ("phase_ms", C.c_double * 9),
                ("phase_bytes", C.c_double * 9)]


# Every exported symbol, as declared in include/sculpt_gpu.h.
EXPORTS = (
    "sgpu_version", "sgpu_last_error", "sgpu_device_info", "sgpu_mesh_create_faces",
    "sgpu_mesh_create_grids", "sgpu_mesh_destroy", "sgpu_mesh_info", "sgpu_mesh_sync",
    "sgpu_mesh_stream", "sgpu_search_sphere", "sgpu_do_draw_brush", "sgpu_do_smooth_brush",
    "sgpu_do_inflate_brush", "sgpu_do_clay_strips_brush", "sgpu_do_brush",
    "sgpu_do_pinch_brush", "sgpu_do_crease_brush", "sgpu_do_grab_brush",
    "sgpu_do_elastic_deform_brush", "sgpu_mesh_store_original", "sgpu_do_layer_brush",
    "sgpu_pbvh_update_normals", "sgpu_pbvh_update_bounds", "sgpu_pbvh_node_mark_update",
    "sgpu_stroke", "sgpu_get_verts", "sgpu_set_verts", "sgpu_get_positions",
    "sgpu_set_positions", "sgpu_get_normals", "sgpu_get_mask", "sgpu_get_node_bbs",
    "sgpu_get_nodes", "sgpu_get_prim_indices", "sgpu_get_vert_indices", "sgpu_curve_table",
    "sgpu_stroke_host", "sgpu_mesh_snapshot", "sgpu_mesh_restore", "sgpu_stroke_profile",
    "sgpu_mesh_flush_l2", "sgpu_host_alloc", "sgpu_host_free", "sgpu_mesh_set_team",
    "sgpu_mesh_get_team", "sgpu_autotune_team", "sgpu_batch_stroke", "sgpu_stroke_team_profile",
    "sgpu_raycast", "sgpu_draw_buffers_build", "sgpu_draw_buffers_update",
    "sgpu_draw_buffers_layout", "sgpu_draw_buffers_overlay", "sgpu_draw_buffers_get",
    "sgpu_draw_buffers_device", "sgpu_draw_buffers_update_timed", "sgpu_debug_inject",
    "sgpu_calc_area_normal_and_center", "sgpu_stroke_host_grids", "sgpu_autotune_batch",
    "sgpu_find_nearest_to_ray", "sgpu_batch_team_profile",
)

DRAW_STRIDE = 36  # SGPU_DRAW_STRIDE
# numpy view of one vertex of the draw buffer (VertexFormat_pack of pos, nor,
# msk, ac, fset; the padding bytes named _pad*)
DRAW_VERTEX_DT = np.dtype({"names": ["pos", "nor", "msk", "ac", "fset"],
                           "formats": [("<f4", (3,)), ("<i2", (3,)), "u1", ("<u2", (4,)),
                                       ("u1", (3,))],
                           "offsets": [0, 16, 22, 24, 32], "itemsize": DRAW_STRIDE})


class SGPU_DrawSetup(C.Structure):
    _fields_ = [("face_sets", C.c_void_p), ("face_sets_color_seed", C.c_int),
                ("face_sets_color_default", C.c_int), ("loop_colors", C.c_void_p),
                ("vert_colors", C.c_void_p), ("use_sculpt_vertex_colors", C.c_int),
                ("grid_flag_mats", C.c_void_p)]

_lib = None


def load(path: str | None = None):
    """Loads libsculptgpu; raises if it is missing (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"libsculptgpu is not built ({p} missing); run __graft_entry__.build()")
    L = C.CDLL(p)
    vp, i, f = C.c_void_p, C.c_int, C.c_float
    L.sgpu_version.restype = C.c_char_p
    L.sgpu_last_error.restype = C.c_char_p
    L.sgpu_device_info.argtypes = [vp, vp, vp]
    L.sgpu_mesh_create_faces.argtypes = [vp, i, vp, i, vp, i, vp, i, vp, vp, vp, i, vp]
    L.sgpu_mesh_create_grids.argtypes = [i, i, vp, vp, vp, i, vp, vp, vp, vp, i, i, vp, i, vp]
    L.sgpu_mesh_destroy.argtypes = [vp]
    L.sgpu_mesh_info.argtypes = [vp, C.POINTER(SGPU_MeshInfo)]
    L.sgpu_mesh_sync.argtypes = [vp]
    L.sgpu_mesh_stream.argtypes = [vp]
    L.sgpu_mesh_stream.restype = vp
    L.sgpu_search_sphere.argtypes = [vp, vp, f, i, vp, vp]
    L.sgpu_raycast.argtypes = [vp, i, vp, vp, vp, i, vp, vp, vp, vp, vp]
    for name in ("sgpu_do_draw_brush", "sgpu_do_smooth_brush", "sgpu_do_inflate_brush",
                 "sgpu_do_clay_strips_brush", "sgpu_do_brush", "sgpu_do_pinch_brush",
                 "sgpu_do_crease_brush", "sgpu_do_grab_brush", "sgpu_do_elastic_deform_brush",
                 "sgpu_do_layer_brush"):
        getattr(L, name).argtypes = [vp, C.POINTER(SGPU_Brush), vp, vp, vp, i]
    L.sgpu_pbvh_update_normals.argtypes = [vp]
    L.sgpu_pbvh_update_bounds.argtypes = [vp, i]
    L.sgpu_pbvh_node_mark_update.argtypes = [vp, i]
    L.sgpu_stroke.argtypes = [vp, C.POINTER(SGPU_Brush), vp, i, vp, i,
                              C.POINTER(SGPU_StrokeStats)]
    for name in ("sgpu_get_verts", "sgpu_set_verts", "sgpu_get_positions", "sgpu_set_positions",
                 "sgpu_get_normals", "sgpu_get_mask", "sgpu_get_prim_indices",
                 "sgpu_get_vert_indices"):
        getattr(L, name).argtypes = [vp, vp]
    L.sgpu_get_node_bbs.argtypes = [vp, vp, vp]
    L.sgpu_get_nodes.argtypes = [vp] + [vp] * 7
    L.sgpu_curve_table.argtypes = [i, vp, vp]
    L.sgpu_stroke_host.argtypes = [vp, C.POINTER(SGPU_Brush), vp, i, vp, vp, vp, vp, i,
                                   C.POINTER(SGPU_StrokeStats)]
    L.sgpu_stroke_team_profile.argtypes = [vp, C.POINTER(SGPU_Brush), vp, i, vp,
                                           C.POINTER(SGPU_TeamProfile),
                                           C.POINTER(SGPU_StrokeStats)]
    L.sgpu_stroke_profile.argtypes = [vp, C.POINTER(SGPU_Brush), vp, i, vp,
                                      C.POINTER(SGPU_KernelProfile),
                                      C.POINTER(SGPU_StrokeStats)]
    for name in ("sgpu_mesh_snapshot", "sgpu_mesh_restore", "sgpu_mesh_flush_l2"):
        getattr(L, name).argtypes = [vp]
    L.sgpu_host_alloc.restype = vp
    L.sgpu_host_alloc.argtypes = [C.c_size_t]
    L.sgpu_host_free.argtypes = [vp]
    L.sgpu_mesh_set_team.argtypes = [vp, i]
    L.sgpu_mesh_get_team.argtypes = [vp, vp]
    L.sgpu_autotune_team.argtypes = [vp, C.POINTER(SGPU_Brush), vp, i, vp, vp, vp]
    L.sgpu_batch_stroke.argtypes = [vp, i, vp, vp, vp, vp, i, i, vp, vp]
    L.sgpu_autotune_batch.argtypes = [vp, i, vp, vp, vp, vp, vp, vp, vp]
    L.sgpu_batch_team_profile.argtypes = [vp, i, vp, vp, vp, vp, i, C.POINTER(SGPU_TeamProfile),
                                          vp]
    L.sgpu_find_nearest_to_ray.argtypes = [vp, i, vp, vp, i, vp, vp, vp]
    L.sgpu_mesh_store_original.argtypes = [vp]
    L.sgpu_debug_inject.argtypes = [i, C.c_int64]
    L.sgpu_calc_area_normal_and_center.argtypes = [vp, C.POINTER(SGPU_Brush), vp, vp, i, vp, vp]
    L.sgpu_stroke_host_grids.argtypes = [vp, C.POINTER(SGPU_Brush), vp, i, vp, vp, vp, vp, i,
                                         C.POINTER(SGPU_StrokeStats)]
    L.sgpu_draw_buffers_build.argtypes = [vp, C.POINTER(SGPU_DrawSetup)]
    L.sgpu_draw_buffers_update.argtypes = [vp]
    L.sgpu_draw_buffers_update_timed.argtypes = [vp, i, vp]
    L.sgpu_draw_buffers_layout.argtypes = [vp, vp, vp, vp, vp]
    L.sgpu_draw_buffers_overlay.argtypes = [vp, vp]
    L.sgpu_draw_buffers_get.argtypes = [vp, vp, C.c_size_t]
    L.sgpu_draw_buffers_device.argtypes = [vp, vp, vp]
    _lib = L
    return L


def debug_inject(what: int, value: int):
    """Host-side failure injection (sgpu_debug_inject): INJECT_ALLOC_FAIL,
    INJECT_WAIT_NS or INJECT_BARRIER_EXTRA."""
    _check(load().sgpu_debug_inject(what, value))


def _batch_args(pbvhs, strokes, dab_tools):
    n = len(pbvhs)
    handles = (C.c_void_p * n)(*[p.handle for p in pbvhs])
    brushes = (SGPU_Brush * n)(*[make_brush(s) for s in strokes])
    dabs = np.ascontiguousarray(np.concatenate([s.dabs for s in strokes]), dtype=np.float32)
    offs = np.zeros(n + 1, dtype=np.int32)
    offs[1:] = np.cumsum([s.dabs.shape[0] for s in strokes])
    tools = None if dab_tools is None else np.ascontiguousarray(dab_tools, dtype=np.int32)
    return n, handles, brushes, dabs, offs, tools


def autotune_batch(pbvhs, strokes, dab_tools=None):
    """sgpu_autotune_batch: ((cluster, CTAs per SM) of the fastest team,
    {candidate: ms})."""
    n, handles, brushes, dabs, offs, tools = _batch_args(pbvhs, strokes, dab_tools)
    cl, per_sm = C.c_int(), C.c_int()
    ms = np.zeros(len(BATCH_TEAM_CANDIDATES), dtype=np.float32)
    _check(load().sgpu_autotune_batch(handles, n, brushes, _p(dabs), _p(offs), _p(tools),
                                      C.byref(cl), C.byref(per_sm), _p(ms)))
    return (cl.value, per_sm.value), {c: float(t) for c, t in zip(BATCH_TEAM_CANDIDATES, ms)}


def batch_stroke(pbvhs, strokes, mode: int = BATCH_TEAM, cluster: int = 0, dab_tools=None):
    """Strokes many independent meshes; returns (per-mesh stats list, total_ms)."""
    L = load()
    n = len(pbvhs)
    handles = (C.c_void_p * n)(*[p.handle for p in pbvhs])
    brushes = (SGPU_Brush * n)(*[make_brush(s) for s in strokes])
    dabs = np.ascontiguousarray(np.concatenate([s.dabs for s in strokes]), dtype=np.float32)
    offs = np.zeros(n + 1, dtype=np.int32)
    offs[1:] = np.cumsum([s.dabs.shape[0] for s in strokes])
    tools = None if dab_tools is None else np.ascontiguousarray(dab_tools, dtype=np.int32)
    stats = (SGPU_StrokeStats * n)()
    total = C.c_float()
    _check(L.sgpu_batch_stroke(handles, n, brushes, _p(dabs), _p(offs), _p(tools), mode,
                               cluster, stats, C.byref(total)))
    return list(stats), total.value


def batch_team_profile(pbvhs, strokes, cluster: int = 0, dab_tools=None):
    """One SGPU_BATCH_TEAM batch with phase timers (those of the launch's first
    thread).  Returns ({phase: ms}, total_ms, per-mesh stats)."""
    L = load()
    n = len(pbvhs)
    handles = (C.c_void_p * n)(*[p.handle for p in pbvhs])
    brushes = (SGPU_Brush * n)(*[make_brush(s) for s in strokes])
    dabs = np.ascontiguousarray(np.concatenate([s.dabs for s in strokes]), dtype=np.float32)
    offs = np.zeros(n + 1, dtype=np.int32)
    offs[1:] = np.cumsum([s.dabs.shape[0] for s in strokes])
    tools = None if dab_tools is None else np.ascontiguousarray(dab_tools, dtype=np.int32)
    prof = SGPU_TeamProfile()
    stats = (SGPU_StrokeStats * n)()
    _check(L.sgpu_batch_team_profile(handles, n, brushes, _p(dabs), _p(offs), _p(tools), cluster,
                                     C.byref(prof), stats))
    return ({name: prof.phase_ms[k] for k, name in enumerate(TEAM_PHASES)}, prof.total_ms,
            list(stats))


class PinnedArray:
    """A numpy array in page-locked host memory from sgpu_host_alloc."""

    def __init__(self, shape, dtype):
        dt = np.dtype(dtype)
        n = int(np.prod(shape)) * dt.itemsize
        self._ptr = load().sgpu_host_alloc(max(n, 16))
        if not self._ptr:
            raise SculptGPUError(ERR_OOM, load().sgpu_last_error().decode())
        buf = (C.c_char * n).from_address(self._ptr)
        self.array = np.frombuffer(buf, dtype=dt).reshape(shape)

    def free(self):
        if self._ptr:
            self.array = None
            load().sgpu_host_free(self._ptr)
            self._ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _check(rc: int):
    if rc != OK:
        raise SculptGPUError(rc, load().sgpu_last_error().decode())


def make_brush(st) -> SGPU_Brush:
    b = SGPU_Brush()
    b.sculpt_tool = st.tool
    b.flag = st.flag
    b.symmetry = st.symmetry
    b.curve_preset = st.curve_preset
    b.radius = st.radius
    b.strength = st.strength
    b.normal_radius_factor = st.normal_radius_factor
    b.area_radius_factor = st.area_radius_factor
    b.plane_offset = st.plane_offset
    for k in range(3):
        b.view_normal[k] = st.view_normal[k]
    b.use_original_bb = st.use_original_bb
    b.crease_pinch_factor = st.crease_pinch_factor
    b.elastic_deform_type = st.elastic_deform_type
    b.elastic_deform_volume_preservation = st.elastic_deform_volume_preservation
    b.height = st.height
    return b


def device_info() -> tuple[int, int, int]:
    L = load()
    sms, ma, mi = C.c_int(), C.c_int(), C.c_int()
    _check(L.sgpu_device_info(C.byref(sms), C.byref(ma), C.byref(mi)))
    return sms.value, ma.value, mi.value


def curve_table(preset: int):
    t = np.zeros((257, 2), dtype=np.float32)
    p = np.zeros(7, dtype=np.float32)
    _check(load().sgpu_curve_table(preset, _p(t), _p(p)))
    return t, p


class PBVH:
    """Device mirror of one PBVH and its mesh (one handle of libsculptgpu)."""

    def __init__(self, handle: C.c_void_p):
        self._h = handle
        self._info = SGPU_MeshInfo()
        _check(load().sgpu_mesh_info(self._h, C.byref(self._info)))

    # -- construction (BKE_pbvh_build_mesh / BKE_pbvh_build_grids)
    @classmethod
    def build_mesh(cls, mesh: "synth.FacesMesh", leaf_limit: int = 0, vert_normals=None,
                   automask=None) -> "PBVH":
        L = load()
        h = C.c_void_p()
        mask = None if mesh.mask is None else np.ascontiguousarray(mesh.mask, dtype=np.float32)
        no = None if vert_normals is None else np.ascontiguousarray(vert_normals, np.float32)
        am = None if automask is None else np.ascontiguousarray(automask, dtype=np.float32)
        _check(L.sgpu_mesh_create_faces(
            _p(mesh.verts), mesh.verts.shape[0], _p(mesh.polys), mesh.polys.shape[0],
            _p(mesh.loops), mesh.loops.shape[0], _p(mesh.looptris), mesh.looptris.shape[0],
            _p(no), _p(mask), _p(am), leaf_limit, C.byref(h)))
        return cls(h)

    @classmethod
    def build_grids(cls, g: "synth.GridsMesh", leaf_limit: int = 0, normals=None) -> "PBVH":
        L = load()
        h = C.c_void_p()
        co = np.ascontiguousarray(g.co, dtype=np.float32)
        no = None if normals is None else np.ascontiguousarray(normals, dtype=np.float32)
        mask = None if g.mask is None else np.ascontiguousarray(g.mask, dtype=np.float32)
        arrs = [np.ascontiguousarray(a, dtype=np.int32) for a in
                (g.face_start, g.face_ngrids, g.face_verts, g.face_edges, g.edge_verts)]
        _check(L.sgpu_mesh_create_grids(
            g.num_grids, g.grid_size, _p(co), _p(no), _p(mask), g.num_faces, _p(arrs[0]),
            _p(arrs[1]), _p(arrs[2]), _p(arrs[3]), g.num_base_verts, arrs[4].shape[0],
            _p(arrs[4]), leaf_limit, C.byref(h)))
        return cls(h)

    def free(self):
        if self._h:
            _check(load().sgpu_mesh_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    @property
    def info(self) -> SGPU_MeshInfo:
        return self._info

    @property
    def num_nodes(self) -> int:
        return self._info.totnode

    @property
    def num_leaves(self) -> int:
        return self._info.totleaf

    @property
    def num_verts(self) -> int:
        return self._info.totvert

    # -- the reference's per-call entry points
    def search_gather_sphere(self, center, radius_sq: float, original: int = 0) -> np.ndarray:
        out = np.zeros(self.num_leaves + 1, dtype=np.int32)
        tot = C.c_int()
        c = np.asarray(center, dtype=np.float32)
        _check(load().sgpu_search_sphere(self._h, _p(c), radius_sq, original, _p(out),
                                         C.byref(tot)))
        return out[:tot.value]

    def raycast(self, starts, normals, lengths=None, original: int = 0):
        """BKE_pbvh_raycast with the sculpt callback for a batch of rays.
        Returns (hit bool[n], depth float32[n], active vertex int32[n],
        active face int32[n], face normal float32[n, 3])."""
        o = np.ascontiguousarray(starts, dtype=np.float32).reshape(-1, 3)
        d = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
        n = o.shape[0]
        ln = None if lengths is None else np.ascontiguousarray(lengths, dtype=np.float32)
        dep = np.zeros(n, dtype=np.float32)
        hit = np.zeros(n, dtype=np.int32)
        av = np.zeros(n, dtype=np.int32)
        af = np.zeros(n, dtype=np.int32)
        fn = np.zeros((n, 3), dtype=np.float32)
        _check(load().sgpu_raycast(self._h, n, _p(o), _p(d), _p(ln), original, _p(dep), _p(hit),
                                   _p(av), _p(af), _p(fn)))
        return hit.astype(bool), dep, av, af, fn

    def nearest_to_ray(self, starts, normals, original: int = 0):
        """BKE_pbvh_find_nearest_to_ray with the sculpt callback for a batch of
        rays.  Returns (hit bool[n], depth float32[n], squared distance
        float32[n])."""
        o = np.ascontiguousarray(starts, dtype=np.float32).reshape(-1, 3)
        d = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
        n = o.shape[0]
        dep = np.zeros(n, dtype=np.float32)
        dsq = np.zeros(n, dtype=np.float32)
        hit = np.zeros(n, dtype=np.int32)
        _check(load().sgpu_find_nearest_to_ray(self._h, n, _p(o), _p(d), original, _p(dep),
                                               _p(dsq), _p(hit)))
        return hit.astype(bool), dep, dsq

    # -- headless draw buffers (GPU_pbvh_*_buffers_build / _update)
    def draw_buffers_build(self, face_sets=None, seed: int = 0, color_default: int = 1,
                           loop_colors=None, vert_colors=None, use_vert_colors: bool = False,
                           grid_flag_mats=None):
        """grid_flag_mats: (num_grids, 2) ints (mat_nr, flag) or None."""
        keep = []

        def arr(a, dt):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=dt)
            keep.append(a)
            return a.ctypes.data_as(C.c_void_p)

        fm = None
        if grid_flag_mats is not None:
            g = np.asarray(grid_flag_mats)
            fm = np.zeros(g.shape[0], dtype=np.dtype([("mat_nr", "<i2"), ("flag", "i1"),
                                                      ("_pad", "i1")]))
            fm["mat_nr"] = g[:, 0]
            fm["flag"] = g[:, 1]
        s = SGPU_DrawSetup(arr(face_sets, np.int32), seed, color_default,
                           arr(loop_colors, np.uint8), arr(vert_colors, np.float32),
                           int(bool(use_vert_colors)), arr(fm, fm.dtype) if fm is not None else None)
        _check(load().sgpu_draw_buffers_build(self._h, C.byref(s)))

    def draw_buffers_update(self):
        _check(load().sgpu_draw_buffers_update(self._h))

    def draw_buffers_update_timed(self, all_leaves: bool = False) -> float:
        """The update timed with CUDA events (ms); all_leaves: full refresh."""
        ms = C.c_float()
        _check(load().sgpu_draw_buffers_update_timed(self._h, int(bool(all_leaves)),
                                                     C.byref(ms)))
        return ms.value

    def draw_buffers_layout(self) -> dict:
        n = self.num_nodes
        out = {"vert_off": np.zeros(n + 1, dtype=np.int64), "tot_tri": np.zeros(n, np.int32),
               "smooth": np.zeros(n, np.int32), "material_index": np.zeros(n, np.int32)}
        _check(load().sgpu_draw_buffers_layout(self._h, _p(out["vert_off"]), _p(out["tot_tri"]),
                                               _p(out["smooth"]), _p(out["material_index"])))
        return out

    def draw_buffers_overlay(self) -> np.ndarray:
        out = np.zeros(self.num_nodes, dtype=np.int32)
        _check(load().sgpu_draw_buffers_overlay(self._h, _p(out)))
        return out

    def draw_buffers_get(self) -> np.ndarray:
        """The whole vertex buffer as bytes (vert_off[-1] * 36)."""
        n = int(self.draw_buffers_layout()["vert_off"][-1])
        out = np.zeros(max(n, 1) * DRAW_STRIDE, dtype=np.uint8)
        _check(load().sgpu_draw_buffers_get(self._h, _p(out), out.nbytes))
        return out[:n * DRAW_STRIDE]

    def search_sphere_device(self, center, radius_sq: float, original: int = 0):
        c = np.asarray(center, dtype=np.float32)
        _check(load().sgpu_search_sphere(self._h, _p(c), radius_sq, original, None, None))

    def _brush(self, fn: str, st, location, grab_delta, nodes=None):
        b = make_brush(st)
        loc = np.asarray(location, dtype=np.float32)
        gd = np.asarray(grab_delta, dtype=np.float32)
        nd = None if nodes is None else np.ascontiguousarray(nodes, dtype=np.int32)
        _check(getattr(load(), fn)(self._h, C.byref(b), _p(loc), _p(gd), _p(nd),
                                   0 if nd is None else nd.shape[0]))

    def area_normal_center(self, st, location, nodes=None):
        """sgpu_calc_area_normal_and_center: (area normal, area centre)."""
        b = make_brush(st)
        loc = np.asarray(location, dtype=np.float32)
        nd = None if nodes is None else np.ascontiguousarray(nodes, dtype=np.int32)
        no = np.zeros(3, dtype=np.float32)
        co = np.zeros(3, dtype=np.float32)
        _check(load().sgpu_calc_area_normal_and_center(
            self._h, C.byref(b), _p(loc), _p(nd), 0 if nd is None else nd.shape[0], _p(no),
            _p(co)))
        return no, co

    def do_draw_brush(self, st, location, grab_delta, nodes=None):
        self._brush("sgpu_do_draw_brush", st, location, grab_delta, nodes)

    def do_smooth_brush(self, st, location, grab_delta, nodes=None):
        self._brush("sgpu_do_smooth_brush", st, location, grab_delta, nodes)

    def do_inflate_brush(self, st, location, grab_delta, nodes=None):
        self._brush("sgpu_do_inflate_brush", st, location, grab_delta, nodes)

    def do_clay_strips_brush(self, st, location, grab_delta, nodes=None):
        self._brush("sgpu_do_clay_strips_brush", st, location, grab_delta, nodes)

    def do_pinch_brush(self, st, location, grab_delta, nodes=None):
        self._brush("sgpu_do_pinch_brush", st, location, grab_delta, nodes)

    def do_crease_brush(self, st, location, grab_delta, nodes=None):
        self._brush("sgpu_do_crease_brush", st, location, grab_delta, nodes)

    def do_layer_brush(self, st, location, grab_delta, nodes=None):
        self._brush("sgpu_do_layer_brush", st, location, grab_delta, nodes)

    def do_grab_brush(self, st, location, grab_delta):
        """One dab over all symmetry passes (the library gathers the leaves)."""
        self._brush("sgpu_do_grab_brush", st, location, grab_delta, None)

    def do_elastic_deform_brush(self, st, location, grab_delta):
        self._brush("sgpu_do_elastic_deform_brush", st, location, grab_delta, None)

    def store_original(self):
        _check(load().sgpu_mesh_store_original(self._h))

    def do_brush(self, st, location, grab_delta, nodes=None):
        self._brush("sgpu_do_brush", st, location, grab_delta, nodes)

    def update_normals(self):
        _check(load().sgpu_pbvh_update_normals(self._h))

    def update_bounds(self, flag: int):
        _check(load().sgpu_pbvh_update_bounds(self._h, flag))

    def node_mark_update(self, node: int):
        _check(load().sgpu_pbvh_node_mark_update(self._h, node))

    # -- whole strokes
    def stroke(self, st, mode: int = STROKE_GRAPH, dabs=None, dab_tools=None) -> SGPU_StrokeStats:
        b = make_brush(st)
        d = np.ascontiguousarray(st.dabs if dabs is None else dabs, dtype=np.float32)
        tools = None if dab_tools is None else np.ascontiguousarray(dab_tools, dtype=np.int32)
        stats = SGPU_StrokeStats()
        _check(load().sgpu_stroke(self._h, C.byref(b), _p(d), d.shape[0], _p(tools), mode,
                                  C.byref(stats)))
        return stats

    def stroke_host(self, st, verts_in, verts_out, normals_in=None, dabs=None,
                    dab_tools=None, mode: int = STROKE_TEAM) -> SGPU_StrokeStats:
        """Host-buffer stroke: upload, refit, stroke, download (one C-ABI call)."""
        b = make_brush(st)
        d = np.ascontiguousarray(st.dabs if dabs is None else dabs, dtype=np.float32)
        tools = None if dab_tools is None else np.ascontiguousarray(dab_tools, dtype=np.int32)
        stats = SGPU_StrokeStats()
        _check(load().sgpu_stroke_host(self._h, C.byref(b), _p(d), d.shape[0], _p(tools),
                                       _p(verts_in), _p(normals_in), _p(verts_out), mode,
                                       C.byref(stats)))
        return stats

    def stroke_host_grids(self, st, co_in, co_out, normals_in=None, dabs=None,
                          dab_tools=None, mode: int = STROKE_TEAM) -> SGPU_StrokeStats:
        """GRIDS host-buffer stroke (3 floats per element in and out)."""
        b = make_brush(st)
        d = np.ascontiguousarray(st.dabs if dabs is None else dabs, dtype=np.float32)
        tools = None if dab_tools is None else np.ascontiguousarray(dab_tools, dtype=np.int32)
        stats = SGPU_StrokeStats()
        _check(load().sgpu_stroke_host_grids(self._h, C.byref(b), _p(d), d.shape[0], _p(tools),
                                             _p(co_in), _p(normals_in), _p(co_out), mode,
                                             C.byref(stats)))
        return stats

    def stroke_team_profile(self, st, dabs=None, dab_tools=None):
        """Persistent stroke with phase timers and algorithmic-byte counters.
        Returns ({phase: {ms, bytes}}, total_ms, stats)."""
        b = make_brush(st)
        d = np.ascontiguousarray(st.dabs if dabs is None else dabs, dtype=np.float32)
        tools = None if dab_tools is None else np.ascontiguousarray(dab_tools, dtype=np.int32)
        prof = SGPU_TeamProfile()
        stats = SGPU_StrokeStats()
        _check(load().sgpu_stroke_team_profile(self._h, C.byref(b), _p(d), d.shape[0],
                                               _p(tools), C.byref(prof), C.byref(stats)))
        out = {name: {"ms": prof.phase_ms[k], "bytes": prof.phase_bytes[k]}
               for k, name in enumerate(TEAM_PHASES)}
        return out, prof.total_ms, stats

    def stroke_profile(self, st, dabs=None, dab_tools=None):
        """Eager stroke with per-launch CUDA events and algorithmic-byte counters.
        Returns ({kernel: {launches, total_ms, alg_bytes}}, stats)."""
        b = make_brush(st)
        d = np.ascontiguousarray(st.dabs if dabs is None else dabs, dtype=np.float32)
        tools = None if dab_tools is None else np.ascontiguousarray(dab_tools, dtype=np.int32)
        prof = (SGPU_KernelProfile * KERNEL_KINDS)()
        stats = SGPU_StrokeStats()
        _check(load().sgpu_stroke_profile(self._h, C.byref(b), _p(d), d.shape[0], _p(tools),
                                          prof, C.byref(stats)))
        out = {}
        for p in prof:
            if p.launches:
                out[p.name.decode()] = {"launches": p.launches, "total_ms": p.total_ms,
                                        "alg_bytes": p.alg_bytes}
        return out, stats

    def set_team(self, cluster: int):
        _check(load().sgpu_mesh_set_team(self._h, cluster))

    def team(self) -> int:
        c = C.c_int()
        _check(load().sgpu_mesh_get_team(self._h, C.byref(c)))
        return c.value

    def autotune_team(self, st, dabs=None, dab_tools=None):
        """Times the persistent stroke for each cluster size; keeps the fastest.
        Returns (best cluster size, {size: ms})."""
        b = make_brush(st)
        d = np.ascontiguousarray(st.dabs if dabs is None else dabs, dtype=np.float32)
        tools = None if dab_tools is None else np.ascontiguousarray(dab_tools, dtype=np.int32)
        best = C.c_int()
        ms = np.zeros(len(TEAM_SIZES), dtype=np.float32)
        _check(load().sgpu_autotune_team(self._h, C.byref(b), _p(d), d.shape[0], _p(tools),
                                         C.byref(best), _p(ms)))
        return best.value, {s: float(t) for s, t in zip(TEAM_SIZES, ms)}

    def snapshot(self):
        _check(load().sgpu_mesh_snapshot(self._h))

    def restore(self):
        _check(load().sgpu_mesh_restore(self._h))

    def flush_l2(self):
        _check(load().sgpu_mesh_flush_l2(self._h))

    def sync(self):
        _check(load().sgpu_mesh_sync(self._h))

    # -- data access
    def positions(self) -> np.ndarray:
        out = np.zeros((self.num_verts, 3), dtype=np.float32)
        _check(load().sgpu_get_positions(self._h, _p(out)))
        return out

    def set_positions(self, co: np.ndarray):
        co = np.ascontiguousarray(co, dtype=np.float32)
        _check(load().sgpu_set_positions(self._h, _p(co)))

    def verts(self) -> np.ndarray:
        out = np.zeros(self.num_verts, dtype=synth.MVERT_DT)
        _check(load().sgpu_get_verts(self._h, _p(out)))
        return out

    def set_verts(self, verts: np.ndarray):
        v = np.ascontiguousarray(verts)
        _check(load().sgpu_set_verts(self._h, _p(v)))

    def normals(self) -> np.ndarray:
        out = np.zeros((self.num_verts, 3), dtype=np.float32)
        _check(load().sgpu_get_normals(self._h, _p(out)))
        return out

    def mask(self) -> np.ndarray:
        out = np.zeros(self.num_verts, dtype=np.float32)
        _check(load().sgpu_get_mask(self._h, _p(out)))
        return out

    def bbs(self):
        vb = np.zeros((self.num_nodes, 6), dtype=np.float32)
        ovb = np.zeros((self.num_nodes, 6), dtype=np.float32)
        _check(load().sgpu_get_node_bbs(self._h, _p(vb), _p(ovb)))
        return vb, ovb

    def nodes(self) -> dict:
        n = self.num_nodes
        keys = ("children_offset", "flag", "prim_off", "totprim", "uniq", "face_verts",
                "vert_off")
        arrs = {k: np.zeros(n, dtype=np.int32) for k in keys}
        _check(load().sgpu_get_nodes(self._h, *[_p(arrs[k]) for k in keys]))
        return arrs

    def prim_indices(self) -> np.ndarray:
        out = np.zeros(max(self._info.totprim, 1), dtype=np.int32)
        _check(load().sgpu_get_prim_indices(self._h, _p(out)))
        return out[:self._info.totprim]

    def vert_indices(self) -> np.ndarray:
        n = self._info.leaf_vert_entries
        out = np.zeros(max(n, 1), dtype=np.int32)
        _check(load().sgpu_get_vert_indices(self._h, _p(out)))
        return out[:n]
