"""Grab, elastic deform and layer (the brushes that read the stroke-start
positions) on the GPU against the oracle, bit for bit: strokes through every
path (eager, graph, the persistent stroke kernel — elastic deform strokes of
one mesh take the graph path there — and the persistent batch),
per-call dabs after sgpu_mesh_store_original, FACES and GRIDS, symmetry, front
face and masks.
The oracle's Kelvinlet displacement is pinned to the reference's compiled
kelvinlet.c in test_refpin_kelvinlet.py."""
import numpy as np
import pytest

from dune_sculpt_gb300 import synth
from dune_sculpt_gb300.sculpt import (PBVH, STROKE_EAGER, STROKE_GRAPH, STROKE_TEAM,
                                      SculptGPUError, batch_stroke, BATCH_TEAM)

from helpers import bits_equal, first_diff, rel_err, small_icosphere

pytestmark = pytest.mark.gpu

FP64_TOL = 2e-6


def _pair(oracle, m, ll):
    g = PBVH.build_mesh(m, ll)
    o = oracle.OracleMesh.faces(m, ll)
    o.recalc_all_normals()
    return g, o


def _assert_equal(g, o, what):
    assert bits_equal(g.positions(), o.co()), what + " co " + first_diff(g.positions(), o.co())
    assert bits_equal(g.normals(), o.no()), what + " no " + first_diff(g.normals(), o.no())
    for a, b in zip(g.bbs(), o.bbs()):
        assert bits_equal(a, b), what + " bb " + first_diff(a, b)


@pytest.mark.parametrize("mode", [STROKE_EAGER, STROKE_GRAPH, STROKE_TEAM])
@pytest.mark.parametrize("frontface", [0, 1])
def test_grab_stroke(gpu, oracle, mode, frontface):
    m = small_icosphere(5)
    g, o = _pair(oracle, m, 600)
    dabs = synth.grab_dabs(3, 12, 0.02)
    view = dabs[0, :3] / np.linalg.norm(dabs[0, :3])  # looking at the anchor's side
    st = synth.Stroke(synth.TOOL_GRAB, 0.25, 0.8, synth.CURVE_SMOOTH, synth.SYMM_X, dabs,
                      flag=(1 << 27) if frontface else 0, view_normal=tuple(float(x) for x in view))
    s = g.stroke(st, mode=mode)
    tot, _ = o.stroke(st, which=3)
    assert s.verts_displaced == tot and tot > 0
    _assert_equal(g, o, f"grab mode {mode}")
    assert rel_err(g.positions(), o.co64()) < FP64_TOL
    # a second stroke starts from the new positions
    s = g.stroke(st, mode=mode)
    tot, _ = o.stroke(st, which=1)
    assert s.verts_displaced == tot
    _assert_equal(g, o, "grab second stroke")


@pytest.mark.parametrize("mode", [STROKE_GRAPH, STROKE_TEAM])
@pytest.mark.parametrize("kind", [0, 1, 2, 3, 4])
def test_elastic_deform_stroke(gpu, oracle, kind, mode):
    m = small_icosphere(4)
    g, o = _pair(oracle, m, 300)
    st = synth.Stroke(synth.TOOL_ELASTIC_DEFORM, 0.2, 0.6, synth.CURVE_SMOOTH, synth.SYMM_X,
                      synth.grab_dabs(5, 8, 0.015), view_normal=(0.0, 0.6, 0.8),
                      elastic_deform_type=kind, elastic_deform_volume_preservation=0.35)
    s = g.stroke(st, mode=mode)
    tot, _ = o.stroke(st, which=3)
    assert s.verts_displaced == tot and tot > 0
    _assert_equal(g, o, f"elastic {kind} mode {mode}")
    assert rel_err(g.positions(), o.co64()) < FP64_TOL


@pytest.mark.parametrize("mode", [STROKE_EAGER, STROKE_GRAPH, STROKE_TEAM])
def test_layer_stroke(gpu, oracle, mode):
    m = small_icosphere(5)  # masked
    g, o = _pair(oracle, m, 600)
    st = synth.Stroke(synth.TOOL_LAYER, 0.15, 0.7, synth.CURVE_SMOOTH, synth.SYMM_X,
                      synth.arc_dabs(13, 20, 0.04), height=0.3)
    s = g.stroke(st, mode=mode)
    tot, _ = o.stroke(st, which=3)
    assert s.verts_displaced == tot and tot > 0
    _assert_equal(g, o, f"layer mode {mode}")
    assert rel_err(g.positions(), o.co64()) < FP64_TOL
    gr = synth.torus_grids(16, 6, level=4)
    gp = PBVH.build_grids(gr, 4)
    og = oracle.OracleMesh.grids(gr, 4)
    og.recalc_all_normals()
    st = synth.Stroke(synth.TOOL_LAYER, 0.15, -0.5, synth.CURVE_SHARP, synth.SYMM_X,
                      synth.torus_dabs(31, 12, 0.1), height=0.2)
    s = gp.stroke(st, mode=mode)
    tot, _ = og.stroke(st, which=1)
    assert s.verts_displaced == tot and tot > 0
    assert bits_equal(gp.positions(), og.co()), first_diff(gp.positions(), og.co())


@pytest.mark.parametrize("mode", [STROKE_EAGER, STROKE_TEAM])
def test_mixed_stroke_with_grab(gpu, oracle, mode):
    """Draw, grab and smooth dabs in one stroke: the grab dabs rebuild their
    leaves from the positions stored at the stroke start."""
    m = small_icosphere(5)
    g, o = _pair(oracle, m, 600)
    dabs = synth.grab_dabs(7, 12, 0.02)
    tools = np.array([(synth.TOOL_DRAW, synth.TOOL_GRAB, synth.TOOL_SMOOTH, synth.TOOL_LAYER)[d % 4]
                      for d in range(12)], dtype=np.int32)
    st = synth.Stroke(synth.TOOL_DRAW, 0.2, 0.5, synth.CURVE_SMOOTH, synth.SYMM_X, dabs)
    s = g.stroke(st, mode=mode, dab_tools=tools)
    tot, _ = o.stroke(st, which=1, dab_tools=tools)
    assert s.verts_displaced == tot
    _assert_equal(g, o, "mixed")


@pytest.mark.parametrize("mode", [STROKE_GRAPH, STROKE_TEAM])
def test_grab_and_elastic_on_grids(gpu, oracle, mode):
    gr = synth.torus_grids(16, 6, level=4)
    for tool, kind in ((synth.TOOL_GRAB, 0), (synth.TOOL_ELASTIC_DEFORM, 2),
                       (synth.TOOL_ELASTIC_DEFORM, 4)):
        gp = PBVH.build_grids(gr, 4)
        o = oracle.OracleMesh.grids(gr, 4)
        o.recalc_all_normals()
        st = synth.Stroke(tool, 0.3, 0.7, synth.CURVE_SMOOTH, synth.SYMM_X,
                          synth.grab_dabs(9, 6, 0.02, surf_radius=1.3), elastic_deform_type=kind)
        s = gp.stroke(st, mode=mode)
        tot, _ = o.stroke(st, which=1)
        assert s.verts_displaced == tot and tot > 0
        assert bits_equal(gp.positions(), o.co()), (tool, kind, first_diff(gp.positions(), o.co()))
        assert bits_equal(gp.normals(), o.no()), (tool, kind)


def test_per_call_dabs(gpu, oracle):
    m = small_icosphere(5)
    g, o = _pair(oracle, m, 600)
    dabs = synth.grab_dabs(11, 4, 0.03)
    st = synth.Stroke(synth.TOOL_GRAB, 0.3, 0.9, synth.CURVE_SMOOTH, synth.SYMM_X, None)
    with pytest.raises(SculptGPUError):
        g.do_grab_brush(st, dabs[0, :3], dabs[0, 3:])  # no stroke-start positions yet
    g.store_original()
    o.store_original()
    for d in range(dabs.shape[0]):
        g.do_grab_brush(st, dabs[d, :3], dabs[d, 3:])
        n = o.orig_dab(st, dabs[d, :3], dabs[d, 3:])
        assert n > 0
        assert bits_equal(g.positions(), o.co()), (d, first_diff(g.positions(), o.co()))
    ste = synth.Stroke(synth.TOOL_ELASTIC_DEFORM, 0.2, 0.5, synth.CURVE_SMOOTH, 0, None,
                       elastic_deform_type=1)
    g.do_elastic_deform_brush(ste, dabs[1, :3], dabs[1, 3:])
    o.orig_dab(ste, dabs[1, :3], dabs[1, 3:])
    assert bits_equal(g.positions(), o.co())
    with pytest.raises(SculptGPUError):  # a node list is not taken
        g._brush("sgpu_do_grab_brush", st, dabs[0, :3], dabs[0, 3:], np.array([0], np.int32))


def test_batch_original_brushes(gpu, oracle):
    """Grab, elastic deform and layer strokes in one persistent launch, next
    to a draw stroke (single-mesh elastic deform strokes take the graph path,
    so the batch is where the persistent kernel runs them)."""
    m4, m5 = small_icosphere(4), small_icosphere(5)
    cases = [
        (m5, 600, synth.Stroke(synth.TOOL_GRAB, 0.25, 0.8, synth.CURVE_SMOOTH, synth.SYMM_X,
                               synth.grab_dabs(3, 12, 0.02))),
        (m4, 300, synth.Stroke(synth.TOOL_ELASTIC_DEFORM, 0.2, 0.6, synth.CURVE_SMOOTH, synth.SYMM_X,
                               synth.grab_dabs(5, 8, 0.015), view_normal=(0.0, 0.6, 0.8),
                               elastic_deform_type=3, elastic_deform_volume_preservation=0.35)),
        (m5, 600, synth.Stroke(synth.TOOL_LAYER, 0.15, 0.7, synth.CURVE_SMOOTH, synth.SYMM_X,
                               synth.arc_dabs(13, 20, 0.04), height=0.3)),
        (m4, 300, synth.Stroke(synth.TOOL_DRAW, 0.2, 0.5, synth.CURVE_SMOOTH, synth.SYMM_X,
                               synth.arc_dabs(17, 10, 0.04))),
        (m4, 300, synth.Stroke(synth.TOOL_ELASTIC_DEFORM, 0.25, 0.4, synth.CURVE_SMOOTH, 0,
                               synth.grab_dabs(19, 6, 0.02), elastic_deform_type=1,
                               elastic_deform_volume_preservation=0.2)),
    ]
    pairs = [_pair(oracle, m, ll) for m, ll, _ in cases]
    stats, _ = batch_stroke([g for g, _ in pairs], [st for _, _, st in cases], mode=BATCH_TEAM,
                            cluster=4)
    for (g, o), (_, _, st), s in zip(pairs, cases, stats):
        tot, _ = o.stroke(st, which=3)
        assert s.verts_displaced == tot and tot > 0
        _assert_equal(g, o, f"batch tool {st.tool}")


@pytest.mark.parametrize("tool", [synth.TOOL_GRAB, synth.TOOL_LAYER, synth.TOOL_ELASTIC_DEFORM])
def test_stroke_host_original_brushes(gpu, oracle, tool):
    """sgpu_stroke_host in persistent mode: the uploaded positions become the
    stroke-start positions (elastic deform runs as a graph replay there)."""
    m = small_icosphere(5)
    g, o = _pair(oracle, m, 600)
    dabs = synth.arc_dabs(13, 20, 0.04) if tool == synth.TOOL_LAYER else synth.grab_dabs(3, 12, 0.02)
    st = synth.Stroke(tool, 0.2, 0.6, synth.CURVE_SMOOTH, synth.SYMM_X, dabs, height=0.3,
                      elastic_deform_type=2)
    vin = m.verts.copy()
    vout = np.zeros_like(vin)
    nin = np.ascontiguousarray(g.normals(), dtype=np.float32)
    s = g.stroke_host(st, vin, vout, nin, mode=STROKE_TEAM)
    tot, _ = o.stroke(st, which=3)
    assert s.verts_displaced == tot and tot > 0
    co = np.ascontiguousarray(vout["co"])
    assert bits_equal(co, o.co()), first_diff(co, o.co())
    _assert_equal(g, o, f"stroke_host tool {tool}")


@pytest.mark.parametrize("tool,kind", [(synth.TOOL_GRAB, 0), (synth.TOOL_LAYER, 0),
                                       (synth.TOOL_ELASTIC_DEFORM, 0),
                                       (synth.TOOL_ELASTIC_DEFORM, 4)])
def test_grid_team_original_brushes(gpu, oracle, tool, kind):
    """The whole-GPU team runs grab, layer and elastic deform strokes itself
    (elastic deform included: every SM sweeps the mesh)."""
    from dune_sculpt_gb300.sculpt import TEAM_GRID

    m = small_icosphere(5)
    g, o = _pair(oracle, m, 600)
    g.set_team(TEAM_GRID)
    dabs = synth.arc_dabs(13, 16, 0.04) if tool == synth.TOOL_LAYER else synth.grab_dabs(3, 10, 0.02)
    st = synth.Stroke(tool, 0.2, 0.6, synth.CURVE_SMOOTH, synth.SYMM_X, dabs, height=0.3,
                      elastic_deform_type=kind, elastic_deform_volume_preservation=0.3)
    s = g.stroke(st, mode=STROKE_TEAM)
    assert s.kernel_launches == 1  # the persistent launch, not a graph replay
    tot, _ = o.stroke(st, which=1)
    assert s.verts_displaced == tot and tot > 0
    _assert_equal(g, o, f"grid team tool {tool}")
