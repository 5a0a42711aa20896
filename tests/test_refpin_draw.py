"""The oracle's draw-buffer restatement against the reference's own compiled
draw code (CPU): gpu_buffers.c's mesh and grid buffer build / update and
gpu_vertex_format.cc's packing, run through the reference's BKE_pbvh_draw_cb
over host-array vertex buffers (oracle/refpin/refpin_draw.c).  Bit for bit:
every node's vertex bytes, tot_tri, smooth, material_index and show_overlay;
the packed format; the face-set colours (paint.c:2219-2236 with the lookup3
hash that noise.cc compiles)."""
from __future__ import annotations

import numpy as np
import pytest

import pyrefpin
from dune_sculpt_gb300.sculpt import DRAW_VERTEX_DT
from draw_cases import (FACES_CASES, GRIDS_CASES, all_smooth, faces_case, grids_case,
                        node_bytes, oracle_faces_kw)

pytestmark = pytest.mark.skipif(not pyrefpin.available(),
                                reason="reference tree absent: the pinning library cannot be built")


def test_draw_format_matches_reference():
    off, sz, stride = pyrefpin.draw_format()
    assert stride == 36 == DRAW_VERTEX_DT.itemsize
    assert list(off) == [0, 16, 22, 24, 32]
    assert list(sz) == [12, 6, 1, 8, 3]
    assert [DRAW_VERTEX_DT.fields[k][1] for k in ("pos", "nor", "msk", "ac", "fset")] == list(off)


def test_face_set_colors_match_reference(oracle):
    for seed in (0, 3, 17, 12345, -4):
        for fs in list(range(-20, 70)) + [1000, 65535, 2 ** 30]:
            a = oracle.face_set_color(fs, seed)
            b = pyrefpin.face_set_color(fs, seed)
            assert np.array_equal(a, b), (fs, seed, a, b)


def _compare(o, layout, vbo, ov, ref):
    for n in range(o.num_nodes):
        a = node_bytes(vbo, layout["vert_off"], n)
        if ref["nverts"][n] < 0:
            assert a.size == 0, n
            continue
        b = ref["bytes"][n]
        assert a.size == b.size, (n, a.size, b.size)
        assert np.array_equal(a, b), (n, np.nonzero(a != b)[0][:8])
        for k in ("tot_tri", "smooth", "material_index"):
            assert layout[k][n] == ref[k][n], (n, k)
        assert ov[n] == ref["show_overlay"][n], n


@pytest.mark.parametrize("name", list(FACES_CASES))
def test_faces_draw_buffers_match_reference(oracle, name):
    m, kw = faces_case(name)
    o = oracle.OracleMesh.faces(m, 100)
    o.recalc_all_normals()
    r = pyrefpin.RefPBVH.faces(m, o.no(), 100)
    r.draw_setup(m, **kw)
    ref = r.draw()
    layout = o.draw_build(**oracle_faces_kw(m, kw))
    vbo = np.zeros(int(layout["vert_off"][-1]) * 36, dtype=np.uint8)
    ov = o.draw_update(vbo)
    _compare(o, layout, vbo, ov, ref)
    if kw["face_sets"] is None:
        assert layout["vert_off"][-1] == 0  # nothing is visible without face sets


@pytest.mark.parametrize("name", list(GRIDS_CASES))
def test_grids_draw_buffers_match_reference(oracle, name):
    g, kw, fm = grids_case(name)
    o = oracle.OracleMesh.grids(g, 4)
    o.recalc_all_normals()
    r = pyrefpin.RefGrids(g, o.no(), 4 * g.grid_size ** 2)
    # the harness's CCG starts with zeroed DMFlagMat (flat); the oracle's and
    # the product's default (no flag mats) is every grid smooth
    r.draw_setup(grid_flag_mats=fm if fm is not None else all_smooth(g.num_grids), **kw)
    ref = r.draw()
    layout = o.draw_build(grid_flag_mats=fm, **kw)
    vbo = np.zeros(int(layout["vert_off"][-1]) * 36, dtype=np.uint8)
    ov = o.draw_update(vbo)
    _compare(o, layout, vbo, ov, ref)
    if fm is not None:
        assert 0 < layout["smooth"].sum() < (o.nodes()["flag"] & 1).sum()
