"""ctypes binding of the reference-pinning harness (oracle/_ref/librefpin.so).

TEST INFRASTRUCTURE ONLY.  The library is the reference's own pbvh.c (and the
poly-normal / vector-math code it calls) compiled from the reference tree by
oracle/refpin/Makefile; tests use it to check the oracle's restatement of the
PBVH build, node search, normal update and bounding-box refit against the
reference itself.  It can only be built where the reference tree is present.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_DIR = os.path.join(_HERE, "refpin")
_LIB_PATH = os.path.join(_HERE, "_ref", "librefpin.so")
REFERENCE_ROOT = os.environ.get("DUNE_SCULPT_REFERENCE", "/root/reference")
_lib = None


def available() -> bool:
    """True when the library exists or the reference tree is here to build it."""
    return os.path.exists(_LIB_PATH) or os.path.isdir(os.path.join(REFERENCE_ROOT, "source"))


def build() -> str:
    if os.path.isdir(os.path.join(REFERENCE_ROOT, "source")):
        subprocess.run(["make", "-s", "-C", _DIR, f"REF={REFERENCE_ROOT}"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        vp, i, f = C.c_void_p, C.c_int, C.c_float
        L.rp_build_faces.restype = vp
        L.rp_build_faces.argtypes = [vp, i, vp, i, vp, i, vp, i, vp, vp]
        L.rp_build_grids.restype = vp
        L.rp_build_grids.argtypes = [i, i, vp, vp, vp]
        L.rp_free.argtypes = [vp]
        L.rp_set_leaf_limit.argtypes = [i]
        for name in ("rp_num_nodes", "rp_leaf_limit"):
            getattr(L, name).restype = i
            getattr(L, name).argtypes = [vp]
        L.rp_get_nodes.argtypes = [vp] + [vp] * 6
        L.rp_get_prim_indices.argtypes = [vp, vp]
        L.rp_get_node_vert_indices.argtypes = [vp, i, vp]
        L.rp_get_node_face_vert_indices.argtypes = [vp, i, vp]
        L.rp_get_bbs.argtypes = [vp, vp, vp]
        L.rp_search_sphere.restype = i
        L.rp_search_sphere.argtypes = [vp, vp, f, i, vp]
        L.rp_set_co.argtypes = [vp, vp]
        L.rp_set_grid_co.argtypes = [vp, vp]
        L.rp_get_no.argtypes = [vp, vp]
        L.rp_node_mark_update.argtypes = [vp, i]
        L.rp_vert_mark_update.argtypes = [vp, i]
        L.rp_update_normals.argtypes = [vp]
        L.rp_update_bounds.argtypes = [vp, i]
        L.rp_node_flag.restype = i
        L.rp_node_flag.argtypes = [vp, i]
        L.rg_create.restype = vp
        L.rg_create.argtypes = [i, vp, vp, vp, vp, i, i, vp, i, vp, vp, vp, i]
        L.rg_free.argtypes = [vp]
        for name in ("rg_num_grids", "rg_num_nodes"):
            getattr(L, name).restype = i
            getattr(L, name).argtypes = [vp]
        L.rg_get_bbs.argtypes = [vp, vp, vp]
        L.rg_get.argtypes = [vp, vp, vp, vp]
        L.rg_set.argtypes = [vp, vp, vp]
        L.rg_node_mark_update.argtypes = [vp, i]
        L.rg_update_normals.argtypes = [vp]
        L.rg_update_bounds.argtypes = [vp, i]
        L.rg_edge_num_faces.restype = i
        L.rg_edge_num_faces.argtypes = [vp, i]
        L.rg_edge_coords.argtypes = [vp, i, i, vp]
        L.rg_vertex_num_faces.restype = i
        L.rg_vertex_num_faces.argtypes = [vp, i]
        L.rg_vertex_coords.argtypes = [vp, i, vp]
        L.rg_raycast.restype = i
        L.rg_raycast.argtypes = [vp, vp, vp, i, vp, vp, vp, vp]
        L.rp_raycast.restype = i
        L.rp_raycast.argtypes = [vp, vp, vp, i, vp, vp, vp, vp]
        for name in ("rp_nearest_to_ray", "rg_nearest_to_ray"):
            getattr(L, name).restype = i
            getattr(L, name).argtypes = [vp, vp, vp, i, vp, vp]
        L.rp_curve_table.argtypes = [i, vp, vp]
        L.rp_curve_evaluate.argtypes = [i, vp, i, vp]
        L.rp_pbvh.restype = vp
        L.rp_pbvh.argtypes = [vp]
        L.rg_pbvh.restype = vp
        L.rg_pbvh.argtypes = [vp]
        L.rp_draw_setup_faces.argtypes = [vp, i, vp, vp, i, vp, vp, vp, i, i, i]
        L.rp_draw_setup_grids.argtypes = [vp, vp, vp, i, i]
        L.rp_draw.argtypes = [vp]
        L.rp_draw_node_info.argtypes = [vp, i, vp]
        L.rp_draw_stride.restype = i
        L.rp_draw_node_bytes.argtypes = [vp, i, vp]
        L.rp_draw_format.argtypes = [vp, vp]
        L.rp_face_set_color.argtypes = [i, i, vp]
        L.rp_kelvinlet.argtypes = [i, f, f, f, vp, vp, vp, vp]
        L.rp_hash_int_01.restype = f
        L.rp_hash_int_01.argtypes = [C.c_uint]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def draw_format():
    """(offsets, sizes) of pos, nor, msk, ac, fset and the stride, as the
    reference's VertexFormat_pack lays them out."""
    off = np.zeros(5, dtype=np.int32)
    sz = np.zeros(5, dtype=np.int32)
    lib().rp_draw_format(_p(off), _p(sz))
    return off, sz, lib().rp_draw_stride()


def face_set_color(face_set: int, seed: int) -> np.ndarray:
    out = np.zeros(3, dtype=np.uint8)
    lib().rp_face_set_color(face_set, seed, _p(out))
    return out


def kelvinlet(kind: int, radius: float, force: float, poisson: float, co, location, dn):
    """The reference's Kelvinlet displacement (kelvinlet.c) of one element."""
    out = np.zeros(3, dtype=np.float32)
    c = np.asarray(co, dtype=np.float32)
    lo = np.asarray(location, dtype=np.float32)
    d = np.asarray(dn, dtype=np.float32)
    lib().rp_kelvinlet(kind, radius, force, poisson, _p(c), _p(lo), _p(d), _p(out))
    return out


def hash_int_01(k: int) -> float:
    return float(lib().rp_hash_int_01(k))


def _draw_collect(pbvh, num_nodes: int) -> dict:
    """BKE_pbvh_draw_cb on every node that needs an update, then per node its
    buffer: vertex count (-1: none), tot_tri, smooth, material_index,
    show_overlay, and its bytes."""
    lib().rp_draw(pbvh)
    info = np.zeros((num_nodes, 5), dtype=np.int32)
    stride = lib().rp_draw_stride()
    data = []
    for n in range(num_nodes):
        lib().rp_draw_node_info(pbvh, n, _p(info[n]))
        b = np.zeros(max(int(info[n, 0]), 0) * stride, dtype=np.uint8)
        if b.size:
            lib().rp_draw_node_bytes(pbvh, n, _p(b))
        data.append(b)
    return {"nverts": info[:, 0], "tot_tri": info[:, 1], "smooth": info[:, 2],
            "material_index": info[:, 3], "show_overlay": info[:, 4], "bytes": data}


def curve_table(preset: int):
    """The brush falloff table built by the reference's colortools.c."""
    t = np.zeros((257, 2), dtype=np.float32)
    p = np.zeros(7, dtype=np.float32)
    lib().rp_curve_table(preset, _p(t), _p(p))
    return t, p


def curve_evaluate(preset: int, values) -> np.ndarray:
    """KERNEL_curvemapping_evaluateF of the brush curve (colortools.c:964-980)."""
    v = np.ascontiguousarray(values, dtype=np.float32)
    out = np.zeros_like(v)
    lib().rp_curve_evaluate(preset, _p(v), v.shape[0], _p(out))
    return out


class RefPBVH:
    """One PBVH built and updated by the reference's own compiled code."""

    def __init__(self, handle, keep, totvert: int):
        self.h = handle
        self._keep = keep
        self.totvert = totvert

    @classmethod
    def faces(cls, m, vert_normals: np.ndarray, leaf_limit: int = 10000):
        """BKE_pbvh_build_mesh; leaf_limit replaces pbvh.c's LEAF_LIMIT (10000)."""
        lib().rp_set_leaf_limit(leaf_limit)
        no = np.ascontiguousarray(vert_normals, dtype=np.float32)
        mask = None if m.mask is None else np.ascontiguousarray(m.mask, dtype=np.float32)
        h = lib().rp_build_faces(_p(m.verts), m.verts.shape[0], _p(m.polys), m.polys.shape[0],
                                 _p(m.loops), m.loops.shape[0], _p(m.looptris),
                                 m.looptris.shape[0], _p(no), _p(mask))
        return cls(h, (m, no, mask), m.verts.shape[0])

    @classmethod
    def grids(cls, num_grids: int, grid_size: int, co, no, mask=None, leaf_limit: int = 10000):
        """BKE_pbvh_build_grids: leaves of max(leaf_limit / grid_size^2, 1) grids."""
        lib().rp_set_leaf_limit(leaf_limit)
        co = np.ascontiguousarray(co, dtype=np.float32)
        no = np.ascontiguousarray(no, dtype=np.float32)
        mask = None if mask is None else np.ascontiguousarray(mask, dtype=np.float32)
        h = lib().rp_build_grids(num_grids, grid_size, _p(co), _p(no), _p(mask))
        return cls(h, (co, no, mask), co.shape[0])

    def close(self):
        if self.h:
            lib().rp_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_nodes(self) -> int:
        return lib().rp_num_nodes(self.h)

    @property
    def leaf_limit(self) -> int:
        return lib().rp_leaf_limit(self.h)

    def nodes(self) -> dict:
        n = self.num_nodes
        keys = ("children_offset", "flag", "prim_off", "totprim", "uniq", "face_verts")
        arrs = {k: np.zeros(n, dtype=np.int32) for k in keys}
        lib().rp_get_nodes(self.h, *[_p(arrs[k]) for k in keys])
        return arrs

    def prim_indices(self) -> np.ndarray:
        tot = int(self.nodes()["totprim"].sum())
        out = np.zeros(max(tot, 1), dtype=np.int32)
        lib().rp_get_prim_indices(self.h, _p(out))
        return out[:tot]

    def node_vert_indices(self, node: int) -> np.ndarray:
        nd = self.nodes()
        n = int(nd["uniq"][node] + nd["face_verts"][node])
        out = np.zeros(max(n, 1), dtype=np.int32)
        lib().rp_get_node_vert_indices(self.h, node, _p(out))
        return out[:n]

    def node_face_vert_indices(self, node: int) -> np.ndarray:
        n = int(self.nodes()["totprim"][node])
        out = np.zeros((max(n, 1), 3), dtype=np.int32)
        lib().rp_get_node_face_vert_indices(self.h, node, _p(out))
        return out[:n]

    def bbs(self):
        n = self.num_nodes
        vb = np.zeros((n, 6), dtype=np.float32)
        ovb = np.zeros((n, 6), dtype=np.float32)
        lib().rp_get_bbs(self.h, _p(vb), _p(ovb))
        return vb, ovb

    def search_sphere(self, center, radius_sq: float, original: int = 0) -> np.ndarray:
        out = np.zeros(self.num_nodes + 1, dtype=np.int32)
        c = np.asarray(center, dtype=np.float32)
        n = lib().rp_search_sphere(self.h, _p(c), radius_sq, original, _p(out))
        return out[:n]

    def set_co(self, co: np.ndarray):
        co = np.ascontiguousarray(co, dtype=np.float32)
        lib().rp_set_co(self.h, _p(co))

    def set_grid_co(self, co: np.ndarray):
        co = np.ascontiguousarray(co, dtype=np.float32)
        lib().rp_set_grid_co(self.h, _p(co))

    def no(self) -> np.ndarray:
        out = np.zeros((self.totvert, 3), dtype=np.float32)
        lib().rp_get_no(self.h, _p(out))
        return out

    def node_mark_update(self, node: int):
        lib().rp_node_mark_update(self.h, int(node))

    def vert_mark_update(self, vertex: int):
        lib().rp_vert_mark_update(self.h, int(vertex))

    def update_normals(self):
        lib().rp_update_normals(self.h)

    def update_bounds(self, flag: int):
        lib().rp_update_bounds(self.h, flag)

    def raycast(self, ray_start, ray_normal, depth: float = 3.4028234663852886e38,
                original: int = 0):
        """BKE_pbvh_raycast with the spec'd callback: (hit, depth, active vertex,
        active face, face normal)."""
        o = np.asarray(ray_start, dtype=np.float32)
        d = np.asarray(ray_normal, dtype=np.float32)
        dep = np.array([depth], dtype=np.float32)
        av = np.array([-1], dtype=np.int32)
        af = np.array([-1], dtype=np.int32)
        fn = np.zeros(3, dtype=np.float32)
        hit = lib().rp_raycast(self.h, _p(o), _p(d), original, _p(dep), _p(av), _p(af), _p(fn))
        return bool(hit), dep[0], int(av[0]), int(af[0]), fn

    def nearest_to_ray(self, ray_start, ray_normal, original: int = 0):
        """BKE_pbvh_find_nearest_to_ray with the spec'd callback: (hit, depth,
        squared distance)."""
        o = np.asarray(ray_start, dtype=np.float32)
        d = np.asarray(ray_normal, dtype=np.float32)
        dep = np.array([3.4028234663852886e38], dtype=np.float32)
        dsq = np.array([3.4028234663852886e38], dtype=np.float32)
        hit = lib().rp_nearest_to_ray(self.h, _p(o), _p(d), original, _p(dep), _p(dsq))
        return bool(hit), dep[0], dsq[0]


def _refpbvh_draw_setup(self, m, face_sets=None, loop_colors=None, vert_colors=None,
                        use_vert_colors=False, seed: int = 0, color_default: int = 1):
    ls = np.ascontiguousarray(m.polys["loopstart"], dtype=np.int32)
    tl = np.ascontiguousarray(m.polys["totloop"], dtype=np.int32)
    fs = None if face_sets is None else np.ascontiguousarray(face_sets, dtype=np.int32)
    lc = None if loop_colors is None else np.ascontiguousarray(loop_colors, dtype=np.uint8)
    vc = None if vert_colors is None else np.ascontiguousarray(vert_colors, dtype=np.float32)
    self._draw_keep = (ls, tl, fs, lc, vc)
    lib().rp_draw_setup_faces(lib().rp_pbvh(self.h), ls.shape[0], _p(ls), _p(tl),
                              m.loops.shape[0], _p(fs), _p(lc), _p(vc), int(bool(use_vert_colors)),
                              seed, color_default)


def _refpbvh_draw(self) -> dict:
    return _draw_collect(lib().rp_pbvh(self.h), self.num_nodes)


RefPBVH.draw_setup = _refpbvh_draw_setup
RefPBVH.draw = _refpbvh_draw


class RefGrids:
    """Multires grids driven by the reference's own subdiv_ccg.c and pbvh.c:
    adjacency, PBVH, normal update with seam stitching, bounds refit."""

    def __init__(self, g, no, leaf_limit: int = 10000):
        arr = lambda a: np.ascontiguousarray(a, dtype=np.int32)  # noqa: E731
        self._keep = [arr(g.face_start), arr(g.face_ngrids), arr(g.face_verts),
                      arr(g.face_edges), arr(g.edge_verts),
                      np.ascontiguousarray(g.co, dtype=np.float32),
                      np.ascontiguousarray(no, dtype=np.float32),
                      None if g.mask is None else np.ascontiguousarray(g.mask, dtype=np.float32)]
        fs, fn, fv, fe, ev, co, nrm, mask = self._keep
        self.grid_size = g.grid_size
        self.nelem = co.shape[0]
        self.has_mask = mask is not None
        self.h = lib().rg_create(fs.shape[0], _p(fs), _p(fn), _p(fv), _p(fe), g.num_base_verts,
                                 ev.shape[0], _p(ev), g.grid_size, _p(co), _p(nrm), _p(mask),
                                 leaf_limit)

    def close(self):
        if self.h:
            lib().rg_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_nodes(self) -> int:
        return lib().rg_num_nodes(self.h)

    def bbs(self):
        n = self.num_nodes
        vb = np.zeros((n, 6), dtype=np.float32)
        ovb = np.zeros((n, 6), dtype=np.float32)
        lib().rg_get_bbs(self.h, _p(vb), _p(ovb))
        return vb, ovb

    def get(self):
        co = np.zeros((self.nelem, 3), dtype=np.float32)
        no = np.zeros((self.nelem, 3), dtype=np.float32)
        mask = np.zeros(self.nelem, dtype=np.float32)
        lib().rg_get(self.h, _p(co), _p(no), _p(mask))
        return co, no, (mask if self.has_mask else None)

    def set(self, co, mask=None):
        co = np.ascontiguousarray(co, dtype=np.float32)
        mask = None if mask is None else np.ascontiguousarray(mask, dtype=np.float32)
        lib().rg_set(self.h, _p(co), _p(mask))

    def node_mark_update(self, node: int):
        lib().rg_node_mark_update(self.h, int(node))

    def update_normals(self):
        lib().rg_update_normals(self.h)

    def update_bounds(self, flag: int):
        lib().rg_update_bounds(self.h, flag)

    def edge_coords(self, edge: int) -> np.ndarray:
        nf = lib().rg_edge_num_faces(self.h, edge)
        out = np.zeros((nf, 2 * self.grid_size, 3), dtype=np.int32)
        for f in range(nf):
            lib().rg_edge_coords(self.h, edge, f, _p(out[f]))
        return out

    def raycast(self, ray_start, ray_normal, depth: float = 3.4028234663852886e38,
                original: int = 0):
        """BKE_pbvh_raycast on the grids: (hit, depth, active element, active
        grid, face normal)."""
        o = np.asarray(ray_start, dtype=np.float32)
        d = np.asarray(ray_normal, dtype=np.float32)
        dep = np.array([depth], dtype=np.float32)
        av = np.array([-1], dtype=np.int32)
        ag = np.array([-1], dtype=np.int32)
        fn = np.zeros(3, dtype=np.float32)
        hit = lib().rg_raycast(self.h, _p(o), _p(d), original, _p(dep), _p(av), _p(ag), _p(fn))
        return bool(hit), dep[0], int(av[0]), int(ag[0]), fn

    def nearest_to_ray(self, ray_start, ray_normal, original: int = 0):
        """BKE_pbvh_find_nearest_to_ray on the grids: (hit, depth, squared distance)."""
        o = np.asarray(ray_start, dtype=np.float32)
        d = np.asarray(ray_normal, dtype=np.float32)
        dep = np.array([3.4028234663852886e38], dtype=np.float32)
        dsq = np.array([3.4028234663852886e38], dtype=np.float32)
        hit = lib().rg_nearest_to_ray(self.h, _p(o), _p(d), original, _p(dep), _p(dsq))
        return bool(hit), dep[0], dsq[0]

    def draw_setup(self, face_sets=None, grid_flag_mats=None, seed: int = 0,
                   color_default: int = 1):
        """grid_flag_mats: (num_grids, 2) ints (mat_nr, flag)."""
        fs = None if face_sets is None else np.ascontiguousarray(face_sets, dtype=np.int32)
        fm = None
        if grid_flag_mats is not None:
            g = np.asarray(grid_flag_mats)
            fm = np.zeros((g.shape[0], 4), dtype=np.uint8)
            fm[:, 0:2] = g[:, 0].astype("<i2").view(np.uint8).reshape(-1, 2)
            fm[:, 2] = g[:, 1].astype(np.uint8)
        self._draw_keep = (fs, fm)
        lib().rp_draw_setup_grids(lib().rg_pbvh(self.h), _p(fs), _p(fm), seed, color_default)

    def draw(self) -> dict:
        return _draw_collect(lib().rg_pbvh(self.h), self.num_nodes)

    def vertex_coords(self, vertex: int) -> np.ndarray:
        nf = lib().rg_vertex_num_faces(self.h, vertex)
        out = np.zeros((max(nf, 1), 3), dtype=np.int32)
        lib().rg_vertex_coords(self.h, vertex, _p(out))
        return out[:nf]
