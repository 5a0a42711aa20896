"""The lockstep batch launch (SGPU_TEAM_LOCKSTEP): every SM works on every
stroke of a batch at once, each phase's work pooled over the meshes.  Each
mesh must end bit-identical to its own stroke in the FP32 restatement
(positions, normals, masks, node boxes, node flags, vertices displaced),
whatever the mix: FACES and GRIDS meshes, different sizes, tools per dab,
symmetry, stroke lengths (none included), strengths below a quarter (smooth
with no full sweep), and leaves left flagged by per-call brushes."""
import numpy as np
import pytest

from dune_sculpt_gb300 import synth
from dune_sculpt_gb300.sculpt import (BATCH_TEAM, DEBUG_LOCKSTEP_PER_SM, ERR_INVALID_ARG,
                                      ERR_TIMEOUT, ERR_UNSUPPORTED, INJECT_BARRIER_EXTRA,
                                      INJECT_WAIT_NS, PBVH, STROKE_GRAPH,
                                      TEAM_LOCKSTEP, SculptGPUError, autotune_batch, batch_stroke,
                                      debug_inject)

from helpers import bits_equal, first_diff, small_icosphere, small_uvsphere

pytestmark = pytest.mark.gpu

MIXED = [synth.TOOL_DRAW, synth.TOOL_SMOOTH, synth.TOOL_INFLATE, synth.TOOL_CLAY_STRIPS,
         synth.TOOL_PINCH, synth.TOOL_CREASE]


def _assert_equal(g, o, what, grids=False):
    assert bits_equal(g.positions(), o.co()), what + " co " + first_diff(g.positions(), o.co())
    assert bits_equal(g.normals(), o.no()), what + " no " + first_diff(g.normals(), o.no())
    if grids:
        assert bits_equal(g.mask(), o.mask()), what + " mask " + first_diff(g.mask(), o.mask())
    for a, b in zip(g.bbs(), o.bbs()):
        assert bits_equal(a, b), what + " bb " + first_diff(a, b)
    assert np.array_equal(g.nodes()["flag"] & 15, o.nodes()["flag"] & 15), what + " flags"


def _faces_job(oracle, m, ll):
    g = PBVH.build_mesh(m, ll)
    o = oracle.OracleMesh.faces(m, ll)
    o.recalc_all_normals()
    return g, o


def _grids_job(oracle, g_mesh, ll=4):
    g = PBVH.build_grids(g_mesh, ll)
    o = oracle.OracleMesh.grids(g_mesh, ll)
    o.recalc_all_normals()
    return g, o


def _run_and_check(jobs, strokes, tools, grids_flags, what, per_sm=0):
    gs = [g for g, _ in jobs]
    all_tools = None
    if any(t is not None for t in tools):
        all_tools = np.concatenate([
            t if t is not None else np.full(st.dabs.shape[0], st.tool, dtype=np.int32)
            for t, st in zip(tools, strokes)]).astype(np.int32)
    debug_inject(DEBUG_LOCKSTEP_PER_SM, per_sm)
    try:
        stats, ms = batch_stroke(gs, strokes, mode=BATCH_TEAM, cluster=TEAM_LOCKSTEP,
                                 dab_tools=all_tools)
    finally:
        debug_inject(DEBUG_LOCKSTEP_PER_SM, 0)
    assert ms > 0
    for k, ((g, o), st, t, s, gr) in enumerate(zip(jobs, strokes, tools, stats, grids_flags)):
        tot, _ = o.stroke(st, which=1, dab_tools=t)
        assert s.verts_displaced == tot, (what, k, s.verts_displaced, tot)
        _assert_equal(g, o, f"{what} mesh {k}", grids=gr)


@pytest.mark.parametrize("per_sm", [1, 2])
def test_lockstep_faces_mixed_batch(gpu, oracle, per_sm):
    """Uneven FACES meshes; per-dab tool mixes, X and XY symmetry, strokes of
    different lengths and one without dabs."""
    batch = synth.cfg4_batch(nmesh=7, vmin=2000, vmax=30000, ndabs=12)
    jobs, strokes, tools = [], [], []
    rng = np.random.default_rng(5)
    for k, (m, st, _) in enumerate(batch):
        jobs.append(_faces_job(oracle, m, 300))
        nd = [12, 5, 0, 12, 9, 1, 12][k]
        st.dabs = st.dabs[:nd]
        st.symmetry = [0, synth.SYMM_X, 0, 3, 0, synth.SYMM_X, 0][k]  # 3: X and Y
        strokes.append(st)
        tools.append(rng.choice(MIXED, size=nd).astype(np.int32) if k % 2 == 0 else None)
    _run_and_check(jobs, strokes, tools, [False] * len(jobs), "faces", per_sm)


def test_lockstep_masked_and_weak_smooth(gpu, oracle):
    """A masked icosphere with smooth at strength 0.2 (no full sweep: the
    first sweep is the result) beside one at 0.9 (three full sweeps and a
    partial one), and a clay-strips sphere."""
    jobs = [_faces_job(oracle, small_icosphere(4), 200), _faces_job(oracle, small_icosphere(4), 200),
            _faces_job(oracle, small_uvsphere(64), 300)]
    strokes = [
        synth.Stroke(synth.TOOL_SMOOTH, 0.15, 0.2, synth.CURVE_SMOOTH, synth.SYMM_X,
                     synth.arc_dabs(3, 10, 0.03)),
        synth.Stroke(synth.TOOL_SMOOTH, 0.12, 0.9, synth.CURVE_SMOOTH, 0, synth.arc_dabs(4, 14, 0.03)),
        synth.Stroke(synth.TOOL_CLAY_STRIPS, 0.1, 0.8, synth.CURVE_SHARP, synth.SYMM_X,
                     synth.arc_dabs(6, 16, 0.03)),
    ]
    _run_and_check(jobs, strokes, [None] * 3, [False] * 3, "masked/smooth", 2)


@pytest.mark.parametrize("per_sm", [1, 2])
def test_lockstep_grids_and_faces(gpu, oracle, per_sm):
    """Multires meshes (inner normals, seams, base edges and corners through
    the pooled face items) beside FACES meshes, tools per dab."""
    jobs = [_grids_job(oracle, synth.torus_grids(16, 6, level=4, seed=synth.SEED_BASE + 4)),
            _faces_job(oracle, small_uvsphere(48), 200),
            _grids_job(oracle, synth.torus_grids(12, 5, level=3, seed=synth.SEED_BASE + 9)),
            _faces_job(oracle, small_icosphere(4), 200)]
    rng = np.random.default_rng(9)
    strokes, tools = [], []
    for k in range(4):
        dabs = synth.torus_dabs(31 + k, 14, 0.15) if k % 2 == 0 else synth.arc_dabs(40 + k, 11, 0.03)
        strokes.append(synth.Stroke(synth.TOOL_DRAW, 0.15 if k % 2 == 0 else 0.1, 0.6,
                                    synth.CURVE_SMOOTH, synth.SYMM_X if k < 2 else 0, dabs))
        tools.append(rng.choice(MIXED, size=dabs.shape[0]).astype(np.int32))
    _run_and_check(jobs, strokes, tools, [True, False, True, False], "grids+faces", per_sm)


def test_lockstep_after_pending_per_call_brush(gpu, oracle):
    """Leaves flagged by a per-call brush without its update join the first
    dab's update, as in a graph-mode stroke."""
    m = small_icosphere(4)
    ga = PBVH.build_mesh(m, 200)
    gb = PBVH.build_mesh(m, 200)
    other = PBVH.build_mesh(small_uvsphere(32), 200)
    st1 = synth.Stroke(synth.TOOL_INFLATE, 0.2, 0.5, synth.CURVE_SMOOTH, 0, None)
    c = ga.positions()[33]
    rsq = float(np.float32(np.float32(0.2) * np.float32(0.2)))
    for g in (ga, gb):
        g.search_sphere_device(c, rsq)
        g.do_inflate_brush(st1, c, [0, 0, 1])
    st2 = synth.Stroke(synth.TOOL_SMOOTH, 0.12, 0.6, synth.CURVE_SMOOTH, synth.SYMM_X,
                       synth.arc_dabs(8, 10, 0.03))
    ga.stroke(st2, mode=STROKE_GRAPH)
    st3 = synth.Stroke(synth.TOOL_DRAW, 0.1, 0.5, synth.CURVE_SMOOTH, 0, synth.arc_dabs(9, 6, 0.03))
    batch_stroke([gb, other], [st2, st3], mode=BATCH_TEAM, cluster=TEAM_LOCKSTEP)
    assert bits_equal(ga.positions(), gb.positions()), first_diff(ga.positions(), gb.positions())
    assert bits_equal(ga.normals(), gb.normals()), first_diff(ga.normals(), gb.normals())
    for x, y in zip(ga.bbs(), gb.bbs()):
        assert bits_equal(x, y), first_diff(x, y)


def test_lockstep_rejections(gpu):
    m = small_icosphere(3)
    a, b = PBVH.build_mesh(m, 200), PBVH.build_mesh(m, 200)
    draw = synth.Stroke(synth.TOOL_DRAW, 0.1, 0.5, synth.CURVE_SMOOTH, 0, synth.arc_dabs(1, 4, 0.03))
    grab = synth.Stroke(synth.TOOL_GRAB, 0.2, 0.5, synth.CURVE_SMOOTH, 0, synth.grab_dabs(2, 4, 0.02))
    with pytest.raises(SculptGPUError) as e:
        batch_stroke([a, b], [draw, grab], mode=BATCH_TEAM, cluster=TEAM_LOCKSTEP)
    assert e.value.code == ERR_UNSUPPORTED
    with pytest.raises(SculptGPUError) as e:
        batch_stroke([a, a], [draw, draw], mode=BATCH_TEAM, cluster=TEAM_LOCKSTEP)
    assert e.value.code == ERR_INVALID_ARG
    # the batch autotuner skips the lockstep candidate for such a batch
    shape, times = autotune_batch([a, b], [draw, grab])
    assert times[(TEAM_LOCKSTEP, 1)] < 0 and shape[0] != TEAM_LOCKSTEP


def test_lockstep_barrier_timeout_returns_status(gpu, oracle):
    """A barrier told to wait for one arrival more than the launch has runs
    out, the launch ends with SGPU_ERR_TIMEOUT, and the next batch runs."""
    m = small_icosphere(4)
    jobs = [_faces_job(oracle, m, 300), _faces_job(oracle, small_uvsphere(32), 200)]
    st = [synth.Stroke(synth.TOOL_DRAW, 0.15, 0.5, synth.CURVE_SMOOTH, synth.SYMM_X,
                       synth.arc_dabs(7, 6, 0.04)),
          synth.Stroke(synth.TOOL_INFLATE, 0.1, 0.5, synth.CURVE_SMOOTH, 0, synth.arc_dabs(8, 6, 0.03))]
    debug_inject(INJECT_WAIT_NS, 20_000_000)  # 20 ms
    debug_inject(INJECT_BARRIER_EXTRA, 1)
    try:
        with pytest.raises(SculptGPUError) as e:
            batch_stroke([g for g, _ in jobs], st, mode=BATCH_TEAM, cluster=TEAM_LOCKSTEP)
        assert e.value.code == ERR_TIMEOUT
    finally:
        debug_inject(INJECT_BARRIER_EXTRA, 0)
        debug_inject(INJECT_WAIT_NS, 0)
    fresh = [_faces_job(oracle, m, 300), _faces_job(oracle, small_uvsphere(32), 200)]
    _run_and_check(fresh, st, [None, None], [False, False], "after timeout")


def test_lockstep_in_batch_autotuner(gpu, oracle):
    batch = synth.cfg4_batch(nmesh=5, vmin=2000, vmax=20000, ndabs=8)
    jobs = [_faces_job(oracle, m, 300) for m, _, _ in batch]
    strokes = [st for _, st, _ in batch]
    shape, times = autotune_batch([g for g, _ in jobs], strokes)
    assert times[(TEAM_LOCKSTEP, 1)] > 0 and times[(TEAM_LOCKSTEP, 2)] > 0
    for k, (g, o) in enumerate(jobs):
        _assert_equal(g, o, f"after autotune {k}")
    _run_and_check(jobs, strokes, [None] * len(jobs), [False] * len(jobs), "tuned")
