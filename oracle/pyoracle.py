"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: loaded by tests/, the smoke check and the CPU
baseline leg of bench.py, never by the GPU product.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None


def build() -> str:
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


class OrBrush(C.Structure):
    _fields_ = [("sculpt_tool", C.c_int), ("flag", C.c_int), ("symmetry", C.c_int),
                ("curve_preset", C.c_int), ("radius", C.c_float), ("strength", C.c_float),
                ("normal_radius_factor", C.c_float), ("area_radius_factor", C.c_float),
                ("plane_offset", C.c_float), ("view_normal", C.c_float * 3),
                ("use_original_bb", C.c_int), ("crease_pinch_factor", C.c_float),
                ("elastic_deform_type", C.c_int),
                ("elastic_deform_volume_preservation", C.c_float), ("height", C.c_float)]


class OrDrawSetup(C.Structure):
    _fields_ = [("face_sets", C.c_void_p), ("face_sets_color_seed", C.c_int),
                ("face_sets_color_default", C.c_int), ("loop_colors", C.c_void_p),
                ("vert_colors", C.c_void_p), ("use_sculpt_vertex_colors", C.c_int),
                ("grid_flag_mats", C.c_void_p), ("vert_flag", C.c_void_p),
                ("lt_loops", C.c_void_p)]


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = C.CDLL(_LIB_PATH)
        vp, i, f = C.c_void_p, C.c_int, C.c_float
        L.or_mesh_create_faces.restype = vp
        L.or_mesh_create_faces.argtypes = [vp, i, vp, i, vp, i, vp, i, vp, vp, i]
        L.or_mesh_create_grids.restype = vp
        L.or_mesh_create_grids.argtypes = [i, i, vp, vp, vp, i, vp, vp, vp, vp, i, i, vp, i]
        L.or_mesh_free.argtypes = [vp]
        for name in ("or_num_nodes", "or_num_leaves", "or_num_verts", "or_num_leaf_vert_entries"):
            getattr(L, name).restype = i
            getattr(L, name).argtypes = [vp]
        L.or_get_nodes.argtypes = [vp] + [vp] * 7
        for name in ("or_get_prim_indices", "or_get_vert_indices", "or_get_co", "or_get_no",
                     "or_get_mask", "or_get_co64", "or_get_no64", "or_set_co"):
            getattr(L, name).argtypes = [vp, vp]
        L.or_get_bbs.argtypes = [vp, vp, vp]
        L.or_get_bbs64.argtypes = [vp, vp, vp]
        L.or_search_sphere.restype = i
        L.or_search_sphere.argtypes = [vp, vp, f, i, vp]
        L.or_recalc_all_normals.argtypes = [vp]
        L.or_brush_pass.restype = i
        L.or_brush_pass.argtypes = [vp, C.POINTER(OrBrush), vp, vp, vp, i, vp]
        L.or_update_normals.argtypes = [vp]
        L.or_update_bounds.argtypes = [vp, i]
        L.or_node_mark_update.argtypes = [vp, i]
        L.or_vert_mark_update.argtypes = [vp, i]
        L.or_get_vert_tags.argtypes = [vp, vp]
        L.or_stroke.restype = C.c_int64
        L.or_stroke.argtypes = [vp, C.POINTER(OrBrush), vp, i, vp, i, i, vp]
        L.or_sync64.argtypes = [vp]
        L.or_area_normal_center.argtypes = [vp, C.POINTER(OrBrush), vp, vp, i, vp, vp]
        L.or_stroke_local_error.restype = C.c_int64
        L.or_stroke_local_error.argtypes = [vp, C.POINTER(OrBrush), vp, i, vp, i, i, vp]
        L.or_draw_build.restype = C.c_int64
        L.or_draw_build.argtypes = [vp, C.POINTER(OrDrawSetup), vp, vp, vp, vp]
        L.or_draw_update.argtypes = [vp, C.POINTER(OrDrawSetup), vp, vp, vp]
        L.or_face_set_color.argtypes = [i, i, vp]
        L.or_kelvinlet.argtypes = [i, f, f, f, vp, vp, vp, vp]
        L.or_store_original.argtypes = [vp]
        L.or_orig_dab.restype = i
        L.or_orig_dab.argtypes = [vp, C.POINTER(OrBrush), vp, vp]
        L.or_raycast.restype = i
        L.or_raycast.argtypes = [vp, vp, vp, i, vp, vp, vp, vp, vp]
        L.or_nearest_to_ray.restype = i
        L.or_nearest_to_ray.argtypes = [vp, vp, vp, i, vp, vp, vp]
        L.or_grids_special_quads.restype = i
        L.or_grids_special_quads.argtypes = [vp, vp, vp]
        L.or_curve_table.argtypes = [i, vp, vp]
        L.or_curve_strength.restype = f
        L.or_curve_strength.argtypes = [i, f, f]
        L.or_max_threads.restype = i
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def make_brush(st) -> OrBrush:
    b = OrBrush()
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


class OracleMesh:
    """The oracle's mirror of one PBVH (FP32 and FP64 states)."""

    def __init__(self, handle, keep):
        self.h = handle
        self._keep = keep

    @classmethod
    def faces(cls, m, leaf_limit: int, automask=None):
        L = lib()
        mask = None if m.mask is None else np.ascontiguousarray(m.mask, dtype=np.float32)
        am = None if automask is None else np.ascontiguousarray(automask, dtype=np.float32)
        h = L.or_mesh_create_faces(_p(m.verts), m.verts.shape[0], _p(m.polys), m.polys.shape[0],
                                   _p(m.loops), m.loops.shape[0], _p(m.looptris),
                                   m.looptris.shape[0], _p(mask), _p(am), leaf_limit)
        return cls(h, (m, mask, am))

    @classmethod
    def grids(cls, g, leaf_limit: int = 0, normals=None):
        L = lib()
        co = np.ascontiguousarray(g.co, dtype=np.float32)
        no = None if normals is None else np.ascontiguousarray(normals, dtype=np.float32)
        mask = None if g.mask is None else np.ascontiguousarray(g.mask, dtype=np.float32)
        fs = np.ascontiguousarray(g.face_start, dtype=np.int32)
        fn = np.ascontiguousarray(g.face_ngrids, dtype=np.int32)
        fv = np.ascontiguousarray(g.face_verts, dtype=np.int32)
        fe = np.ascontiguousarray(g.face_edges, dtype=np.int32)
        ev = np.ascontiguousarray(g.edge_verts, dtype=np.int32)
        h = L.or_mesh_create_grids(g.num_grids, g.grid_size, _p(co), _p(no), _p(mask),
                                   g.num_faces, _p(fs), _p(fn), _p(fv), _p(fe),
                                   g.num_base_verts, ev.shape[0], _p(ev), leaf_limit)
        return cls(h, (co, no, mask, fs, fn, fv, fe, ev))

    def close(self):
        if self.h:
            lib().or_mesh_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_nodes(self) -> int:
        return lib().or_num_nodes(self.h)

    @property
    def num_leaves(self) -> int:
        return lib().or_num_leaves(self.h)

    @property
    def num_verts(self) -> int:
        return lib().or_num_verts(self.h)

    def nodes(self) -> dict:
        n = self.num_nodes
        arrs = {k: np.zeros(n, dtype=np.int32) for k in
                ("children_offset", "flag", "prim_off", "totprim", "uniq", "face_verts",
                 "vert_off")}
        lib().or_get_nodes(self.h, *[_p(arrs[k]) for k in
                                     ("children_offset", "flag", "prim_off", "totprim", "uniq",
                                      "face_verts", "vert_off")])
        return arrs

    def prim_indices(self) -> np.ndarray:
        nd = self.nodes()
        tot = int(nd["totprim"].sum())
        out = np.zeros(max(tot, 1), dtype=np.int32)
        lib().or_get_prim_indices(self.h, _p(out))
        return out[:tot]

    def vert_indices(self) -> np.ndarray:
        n = lib().or_num_leaf_vert_entries(self.h)
        out = np.zeros(max(n, 1), dtype=np.int32)
        lib().or_get_vert_indices(self.h, _p(out))
        return out[:n]

    def bbs(self):
        n = self.num_nodes
        vb = np.zeros((n, 6), dtype=np.float32)
        ovb = np.zeros((n, 6), dtype=np.float32)
        lib().or_get_bbs(self.h, _p(vb), _p(ovb))
        return vb, ovb

    def bbs64(self):
        n = self.num_nodes
        vb = np.zeros((n, 6), dtype=np.float64)
        ovb = np.zeros((n, 6), dtype=np.float64)
        lib().or_get_bbs64(self.h, _p(vb), _p(ovb))
        return vb, ovb

    def co(self) -> np.ndarray:
        out = np.zeros((self.num_verts, 3), dtype=np.float32)
        lib().or_get_co(self.h, _p(out))
        return out

    def no(self) -> np.ndarray:
        out = np.zeros((self.num_verts, 3), dtype=np.float32)
        lib().or_get_no(self.h, _p(out))
        return out

    def mask(self) -> np.ndarray:
        out = np.zeros(self.num_verts, dtype=np.float32)
        lib().or_get_mask(self.h, _p(out))
        return out

    def co64(self) -> np.ndarray:
        out = np.zeros((self.num_verts, 3), dtype=np.float64)
        lib().or_get_co64(self.h, _p(out))
        return out

    def no64(self) -> np.ndarray:
        out = np.zeros((self.num_verts, 3), dtype=np.float64)
        lib().or_get_no64(self.h, _p(out))
        return out

    def set_co(self, co: np.ndarray):
        co = np.ascontiguousarray(co, dtype=np.float32)
        lib().or_set_co(self.h, _p(co))

    def search_sphere(self, center, radius_sq: float, original: int = 0) -> np.ndarray:
        out = np.zeros(self.num_nodes + 1, dtype=np.int32)
        c = np.asarray(center, dtype=np.float32)
        n = lib().or_search_sphere(self.h, _p(c), radius_sq, original, _p(out))
        return out[:n]

    def recalc_all_normals(self):
        lib().or_recalc_all_normals(self.h)

    def brush_pass(self, st, location, grab_delta, nodes) -> tuple[int, np.ndarray]:
        b = make_brush(st)
        loc = np.asarray(location, dtype=np.float32)
        gd = np.asarray(grab_delta, dtype=np.float32)
        nd = np.ascontiguousarray(nodes, dtype=np.int32)
        area = np.zeros(6, dtype=np.float32)
        n = lib().or_brush_pass(self.h, C.byref(b), _p(loc), _p(gd), _p(nd), nd.shape[0],
                                _p(area))
        return n, area

    def update_normals(self):
        lib().or_update_normals(self.h)

    def node_mark_update(self, node: int):
        lib().or_node_mark_update(self.h, int(node))

    def vert_mark_update(self, vertex: int):
        lib().or_vert_mark_update(self.h, int(vertex))

    def vert_tags(self) -> np.ndarray:
        out = np.zeros(self.num_verts, dtype=np.uint8)
        lib().or_get_vert_tags(self.h, _p(out))
        return out

    def update_bounds(self, flag: int):
        lib().or_update_bounds(self.h, flag)

    def store_original(self):
        lib().or_store_original(self.h)

    def orig_dab(self, st, location, grab_delta) -> int:
        """One dab of grab / elastic deform (all symmetry passes), FP32."""
        b = make_brush(st)
        loc = np.asarray(location, dtype=np.float32)
        gd = np.asarray(grab_delta, dtype=np.float32)
        return int(lib().or_orig_dab(self.h, C.byref(b), _p(loc), _p(gd)))

    def draw_build(self, face_sets=None, seed: int = 0, color_default: int = 1,
                   loop_colors=None, vert_colors=None, use_vert_colors: bool = False,
                   grid_flag_mats=None, vert_flag=None, lt_loops=None) -> dict:
        """The draw-buffer layout per node; keeps the inputs for draw_update.
        grid_flag_mats: (num_grids, 2) ints (mat_nr, flag)."""
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
        st = OrDrawSetup(arr(face_sets, np.int32), seed, color_default, arr(loop_colors, np.uint8),
                         arr(vert_colors, np.float32), int(bool(use_vert_colors)),
                         arr(fm, fm.dtype) if fm is not None else None, arr(vert_flag, np.uint8),
                         arr(lt_loops, np.int32))
        n = self.num_nodes
        out = {"vert_off": np.zeros(n + 1, dtype=np.int64), "tot_tri": np.zeros(n, np.int32),
               "smooth": np.zeros(n, np.int32), "material_index": np.zeros(n, np.int32)}
        lib().or_draw_build(self.h, C.byref(st), _p(out["vert_off"]), _p(out["tot_tri"]),
                            _p(out["smooth"]), _p(out["material_index"]))
        self._draw = (st, keep, out["vert_off"])
        return out

    def draw_update(self, vbo: np.ndarray) -> np.ndarray:
        """Fills the flagged leaves into vbo (uint8, vert_off[-1] * 36 bytes);
        returns show_overlay per node (-1 where not updated)."""
        st, _, vert_off = self._draw
        assert vbo.dtype == np.uint8 and vbo.nbytes >= int(vert_off[-1]) * 36
        ov = np.full(self.num_nodes, -1, dtype=np.int32)
        lib().or_draw_update(self.h, C.byref(st), _p(vert_off), _p(vbo), _p(ov))
        return ov

    def raycast(self, ray_start, ray_normal, depth: float = 3.4028234663852886e38,
                original: int = 0):
        """BKE_pbvh_raycast with the spec'd callback: (hit, depth, active vertex,
        active face, face normal, leaves the ray's line meets)."""
        o = np.asarray(ray_start, dtype=np.float32)
        d = np.asarray(ray_normal, dtype=np.float32)
        dep = np.array([depth], dtype=np.float32)
        av = np.array([-1], dtype=np.int32)
        af = np.array([-1], dtype=np.int32)
        fn = np.zeros(3, dtype=np.float32)
        nl = np.zeros(1, dtype=np.int32)
        hit = lib().or_raycast(self.h, _p(o), _p(d), original, _p(dep), _p(av), _p(af), _p(fn),
                               _p(nl))
        return bool(hit), dep[0], int(av[0]), int(af[0]), fn, int(nl[0])

    def nearest_to_ray(self, ray_start, ray_normal, original: int = 0):
        """(hit, depth, squared distance, leaves listed) of the nearest-to-ray query."""
        o = np.asarray(ray_start, dtype=np.float32)
        d = np.asarray(ray_normal, dtype=np.float32)
        dep = np.array([3.4028234663852886e38], dtype=np.float32)
        dsq = np.array([3.4028234663852886e38], dtype=np.float32)
        nl = np.zeros(1, dtype=np.int32)
        hit = lib().or_nearest_to_ray(self.h, _p(o), _p(d), original, _p(dep), _p(dsq), _p(nl))
        return bool(hit), dep[0], dsq[0], int(nl[0])

    def grids_special_quads(self, ray_start, ray_normal) -> int:
        o = np.asarray(ray_start, dtype=np.float32)
        d = np.asarray(ray_normal, dtype=np.float32)
        return int(lib().or_grids_special_quads(self.h, _p(o), _p(d)))

    def stroke(self, st, which: int = 3, nthreads: int = 0, dabs=None, dab_tools=None):
        b = make_brush(st)
        d = np.ascontiguousarray(st.dabs if dabs is None else dabs, dtype=np.float32)
        tools = None if dab_tools is None else np.ascontiguousarray(dab_tools, dtype=np.int32)
        per = np.zeros(d.shape[0], dtype=np.int64)
        tot = lib().or_stroke(self.h, C.byref(b), _p(d), d.shape[0], _p(tools), which, nthreads,
                              _p(per))
        return int(tot), per

    LOCAL_ERR_FIELDS = ("co", "no", "bb", "area_no", "area_co")

    def stroke_local_error(self, st, dab_tools=None, stride: int = 1, nthreads: int = 0):
        """The FP32 stroke with each measured dab's FP32-vs-FP64 error from the
        same input state (or_stroke_local_error).  Returns (vertices displaced,
        {field: max over the measured dabs})."""
        b = make_brush(st)
        d = np.ascontiguousarray(st.dabs, dtype=np.float32)
        tools = None if dab_tools is None else np.ascontiguousarray(dab_tools, dtype=np.int32)
        err = np.zeros((d.shape[0], 5), dtype=np.float64)
        tot = lib().or_stroke_local_error(self.h, C.byref(b), _p(d), d.shape[0], _p(tools),
                                          stride, nthreads, _p(err))
        measured = err[err[:, 0] >= 0]
        return int(tot), {k: float(measured[:, i].max()) if measured.size else 0.0
                          for i, k in enumerate(self.LOCAL_ERR_FIELDS)}

    def sync64(self):
        lib().or_sync64(self.h)

    def area_normal_center(self, st, location, nodes):
        """Area normal and centre over the leaves nodes at location: (FP32 6
        floats, FP64 6 doubles from the same state)."""
        b = make_brush(st)
        loc = np.asarray(location, dtype=np.float32)
        nd = np.ascontiguousarray(nodes, dtype=np.int32)
        o32 = np.zeros(6, dtype=np.float32)
        o64 = np.zeros(6, dtype=np.float64)
        lib().or_area_normal_center(self.h, C.byref(b), _p(loc), _p(nd), nd.shape[0], _p(o32),
                                    _p(o64))
        return o32, o64


def kelvinlet(kind: int, radius: float, force: float, poisson: float, co, location, dn):
    out = np.zeros(3, dtype=np.float32)
    c = np.asarray(co, dtype=np.float32)
    lo = np.asarray(location, dtype=np.float32)
    d = np.asarray(dn, dtype=np.float32)
    lib().or_kelvinlet(kind, radius, force, poisson, _p(c), _p(lo), _p(d), _p(out))
    return out


def face_set_color(face_set: int, seed: int) -> np.ndarray:
    out = np.zeros(3, dtype=np.uint8)
    lib().or_face_set_color(face_set, seed, _p(out))
    return out


def curve_table(preset: int):
    t = np.zeros((257, 2), dtype=np.float32)
    p = np.zeros(7, dtype=np.float32)
    lib().or_curve_table(preset, _p(t), _p(p))
    return t, p


def curve_strength(preset: int, dist: float, radius: float) -> float:
    return float(lib().or_curve_strength(preset, dist, radius))


def max_threads() -> int:
    return int(lib().or_max_threads())
