"""Seeded inputs of the draw-buffer tests: meshes and the layers the draw
path reads (face sets, hidden vertices, colours, grid flags), shared by the
reference-pinning tests and the GPU tests."""
from __future__ import annotations

import numpy as np

from dune_sculpt_gb300 import synth
from helpers import small_icosphere

STRIDE = 36
ME_HIDE = 16

# FACES variants: name -> options
FACES_CASES = {
    "smooth-facesets": {},
    "flat-materials": {"flat": True},
    "unmasked": {"masked": False},
    "hidden-verts": {"hide": True},
    "default-set": {"default_set": True, "masked": False},
    "no-face-sets": {"no_fs": True},
    "loop-colors": {"loop_colors": True, "flat": True},
    "vert-colors": {"vert_colors": True, "hide": True},
}

GRIDS_CASES = {
    "smooth": {},
    "flat-mixed": {"flat": True},
    "unmasked-no-sets": {"masked": False, "no_fs": True},
    "flat-unmasked": {"flat": True, "masked": False},
}


def faces_case(name: str, level: int = 3):
    """(mesh, draw kwargs) for a FACES variant."""
    opt = FACES_CASES[name]
    m = small_icosphere(level, masked=opt.get("masked", True))
    rng = np.random.default_rng(0x5EED0000 + 61)
    P = m.polys.shape[0]
    if opt.get("flat"):
        m.polys["flag"][::3] = 0
        m.polys["mat_nr"] = np.arange(P) % 3
    if opt.get("hide"):
        m.verts["flag"][rng.random(m.verts.shape[0]) < 0.08] |= ME_HIDE
    fs = ((np.arange(P) % 5) + 1).astype(np.int32)
    fs[rng.random(P) < 0.1] = -2  # hidden face set
    if opt.get("default_set"):
        fs[:] = 1
    kw = {"face_sets": None if opt.get("no_fs") else fs, "seed": 7, "color_default": 1}
    if opt.get("loop_colors"):
        kw["loop_colors"] = rng.integers(0, 256, size=(m.loops.shape[0], 4)).astype(np.uint8)
    if opt.get("vert_colors"):
        kw["vert_colors"] = (rng.random((m.verts.shape[0], 4)) * 1.2 - 0.1).astype(np.float32)
        kw["use_vert_colors"] = True
    return m, kw


def grids_case(name: str, level: int = 4):
    """(grids, draw kwargs, grid flag mats or None) for a GRIDS variant."""
    opt = GRIDS_CASES[name]
    g = synth.torus_grids(16, 6, level=level)
    if not opt.get("masked", True):
        g.mask = None
    fm = None
    if opt.get("flat"):
        k = np.arange(g.num_grids)
        fm = np.stack([k % 3, (k // 7) % 2], axis=1)
    fs = ((np.arange(g.num_faces) % 4) + 1).astype(np.int32)
    kw = {"face_sets": None if opt.get("no_fs") else fs, "seed": 5, "color_default": 2}
    return g, kw, fm


def all_smooth(num_grids: int) -> np.ndarray:
    return np.stack([np.zeros(num_grids, int), np.ones(num_grids, int)], axis=1)


def oracle_faces_kw(m, kw):
    """The oracle's extra inputs (vertex flags, looptri loops)."""
    return dict(kw, vert_flag=m.verts["flag"],
                lt_loops=np.ascontiguousarray(m.looptris["tri"], dtype=np.int32))


def node_bytes(vbo: np.ndarray, vert_off: np.ndarray, n: int) -> np.ndarray:
    return vbo[int(vert_off[n]) * STRIDE:int(vert_off[n + 1]) * STRIDE]
