"""Headless draw buffers on the GPU (sgpu_draw_buffers_*) against the oracle's
restatement of pbvh_update_draw_buffers / GPU_pbvh_*_buffers_update (itself
pinned to the reference's compiled gpu_buffers.c in test_refpin_draw.py):
the whole vertex buffer byte for byte, the per-node layout and show_overlay,
after the build and after strokes (only the leaves a stroke touched are
refilled; the others keep their bytes)."""
import numpy as np
import pytest

from dune_sculpt_gb300 import synth
from dune_sculpt_gb300.sculpt import (DRAW_VERTEX_DT, PBVH, STROKE_GRAPH, STROKE_TEAM,
                                      SculptGPUError, _check, _p, load)

from draw_cases import FACES_CASES, GRIDS_CASES, faces_case, grids_case, oracle_faces_kw

pytestmark = pytest.mark.gpu

LEAF = 1
UPD_DRAW = 16
REBUILD_DRAW = 1 << 9


def _first_diff(a, b):
    d = np.nonzero(a != b)[0]
    if d.size == 0:
        return ""
    v = d[0] // 36
    return f"byte {d[0]} (vertex {v}, offset {d[0] % 36}): gpu {a[d[0]]} oracle {b[d[0]]}"


def _check_draw(gp, o, layout_o, vbo_o, ov_o, what):
    lay = gp.draw_buffers_layout()
    for k in ("vert_off", "tot_tri", "smooth", "material_index"):
        assert np.array_equal(lay[k], layout_o[k]), f"{what}: layout {k}"
    vbo = gp.draw_buffers_get()
    assert vbo.size == vbo_o.size, what
    assert np.array_equal(vbo, vbo_o), f"{what}: {_first_diff(vbo, vbo_o)}"
    ov = gp.draw_buffers_overlay()
    upd = ov_o >= 0
    assert np.array_equal(ov[upd], ov_o[upd]), f"{what}: show_overlay"
    # the draw flags are consumed on every leaf
    fl = gp.nodes()["flag"]
    assert not np.any(fl & (UPD_DRAW | REBUILD_DRAW)), what


@pytest.mark.parametrize("name", list(FACES_CASES))
def test_faces_draw_buffers_match_oracle(gpu, oracle, name):
    m, kw = faces_case(name, level=5)
    gp = PBVH.build_mesh(m, 600)
    o = oracle.OracleMesh.faces(m, 600)
    o.recalc_all_normals()
    gp.draw_buffers_build(**kw)
    layout_o = o.draw_build(**oracle_faces_kw(m, kw))
    gp.draw_buffers_update()
    vbo_o = np.zeros(int(layout_o["vert_off"][-1]) * 36, dtype=np.uint8)
    ov_o = o.draw_update(vbo_o)
    _check_draw(gp, o, layout_o, vbo_o, ov_o, name)
    if kw["face_sets"] is not None:
        v = gp.draw_buffers_get().view(DRAW_VERTEX_DT)
        assert v.shape[0] > 0 and np.all(np.abs(v["nor"].astype(np.int32)).max(1) > 0)


@pytest.mark.parametrize("mode", [STROKE_GRAPH, STROKE_TEAM])
def test_faces_draw_buffers_after_stroke(gpu, oracle, mode):
    m, kw = faces_case("flat-materials", level=5)
    gp = PBVH.build_mesh(m, 600)
    o = oracle.OracleMesh.faces(m, 600)
    o.recalc_all_normals()
    gp.draw_buffers_build(**kw)
    layout_o = o.draw_build(**oracle_faces_kw(m, kw))
    gp.draw_buffers_update()
    vbo_o = np.zeros(int(layout_o["vert_off"][-1]) * 36, dtype=np.uint8)
    o.draw_update(vbo_o)
    st = synth.Stroke(synth.TOOL_DRAW, 0.25, 0.8, synth.CURVE_SMOOTH, synth.SYMM_X,
                      synth.arc_dabs(5, 12, 0.1))
    gp.stroke(st, mode=mode)
    o.stroke(st, which=1)
    # the stroke flagged the leaves it touched, on both sides
    fl_g, fl_o = gp.nodes()["flag"], o.nodes()["flag"]
    touched = (fl_o & UPD_DRAW) != 0
    assert np.array_equal((fl_g & UPD_DRAW) != 0, touched)
    assert 0 < touched.sum() < (fl_o & LEAF).sum()
    before = gp.draw_buffers_get()
    gp.draw_buffers_update()
    ov_o = o.draw_update(vbo_o)
    _check_draw(gp, o, layout_o, vbo_o, ov_o, "after stroke")
    assert not np.array_equal(before, vbo_o)


@pytest.mark.parametrize("name", list(GRIDS_CASES))
def test_grids_draw_buffers_match_oracle(gpu, oracle, name):
    g, kw, fm = grids_case(name)
    gp = PBVH.build_grids(g, 4)
    o = oracle.OracleMesh.grids(g, 4)
    o.recalc_all_normals()
    gp.draw_buffers_build(grid_flag_mats=fm, **kw)
    layout_o = o.draw_build(grid_flag_mats=fm, **kw)
    gp.draw_buffers_update()
    vbo_o = np.zeros(int(layout_o["vert_off"][-1]) * 36, dtype=np.uint8)
    ov_o = o.draw_update(vbo_o)
    _check_draw(gp, o, layout_o, vbo_o, ov_o, name)


def test_grids_draw_buffers_after_stroke(gpu, oracle):
    g, kw, fm = grids_case("flat-mixed")
    gp = PBVH.build_grids(g, 4)
    o = oracle.OracleMesh.grids(g, 4)
    o.recalc_all_normals()
    gp.draw_buffers_build(grid_flag_mats=fm, **kw)
    layout_o = o.draw_build(grid_flag_mats=fm, **kw)
    gp.draw_buffers_update()
    vbo_o = np.zeros(int(layout_o["vert_off"][-1]) * 36, dtype=np.uint8)
    o.draw_update(vbo_o)
    st = synth.Stroke(synth.TOOL_INFLATE, 0.15, 0.6, synth.CURVE_SMOOTH, synth.SYMM_X,
                      synth.torus_dabs(31, 16, 0.15))
    gp.stroke(st, mode=STROKE_TEAM)
    o.stroke(st, which=1)
    gp.draw_buffers_update()
    ov_o = o.draw_update(vbo_o)
    _check_draw(gp, o, layout_o, vbo_o, ov_o, "grids after stroke")


def test_draw_buffers_errors(gpu):
    m, kw = faces_case("smooth-facesets")
    gp = PBVH.build_mesh(m, 600)
    with pytest.raises(SculptGPUError):
        gp.draw_buffers_update()  # not built
    gp.draw_buffers_build(**kw)
    gp.draw_buffers_update()
    small = np.zeros(8, dtype=np.uint8)
    with pytest.raises(SculptGPUError):
        _check(load().sgpu_draw_buffers_get(gp._h, _p(small), small.nbytes))
    # a rebuild refills every leaf at the next update
    gp.draw_buffers_build(**kw)
    assert np.all(gp.nodes()["flag"][gp.nodes()["flag"] & LEAF != 0] & UPD_DRAW)
