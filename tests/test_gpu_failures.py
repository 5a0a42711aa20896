"""Failure handling without a GPU fault: an injected out-of-memory during mesh
creation returns SGPU_ERR_OOM and frees what the call had allocated; a
whole-GPU team barrier whose wait runs out (it is told to wait for one
arrival more than the launch has) ends the launch with SGPU_ERR_TIMEOUT, and
the context stays usable: the next stroke runs and matches the oracle."""
import numpy as np
import pytest

from dune_sculpt_gb300 import synth
from dune_sculpt_gb300.sculpt import (ERR_OOM, ERR_TIMEOUT, INJECT_ALLOC_FAIL,
                                      INJECT_BARRIER_EXTRA, INJECT_WAIT_NS, PBVH, STROKE_TEAM,
                                      TEAM_GRID, SculptGPUError, debug_inject)

from helpers import bits_equal, first_diff, small_icosphere

pytestmark = pytest.mark.gpu


def _free_bytes():
    torch = pytest.importorskip("torch")
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def test_injected_oom_frees_the_partial_mesh(gpu):
    m = small_icosphere(5)
    PBVH.build_mesh(m, 600).free()  # one-time set-up outside the measurement
    before = _free_bytes()
    for n in (1, 2, 5, 13, 29):
        debug_inject(INJECT_ALLOC_FAIL, n)
        with pytest.raises(SculptGPUError) as e:
            PBVH.build_mesh(m, 600)
        assert e.value.code == ERR_OOM
        assert "injected" in str(e.value)
    debug_inject(INJECT_ALLOC_FAIL, 0)
    after = _free_bytes()
    # a leaked mesh would hold about 20 MB of device memory per failed call
    assert before - after < 8 << 20, (before, after)
    g = PBVH.build_mesh(m, 600)  # creation works again
    assert g.num_verts == m.verts.shape[0]
    g.free()


def test_barrier_timeout_returns_status(gpu, oracle):
    m = small_icosphere(4)
    g = PBVH.build_mesh(m, 300)
    g.set_team(TEAM_GRID)
    st = synth.Stroke(synth.TOOL_DRAW, 0.15, 0.5, synth.CURVE_SMOOTH, synth.SYMM_X,
                      synth.arc_dabs(7, 6, 0.04))
    debug_inject(INJECT_WAIT_NS, 20_000_000)  # 20 ms
    debug_inject(INJECT_BARRIER_EXTRA, 1)
    try:
        with pytest.raises(SculptGPUError) as e:
            g.stroke(st, mode=STROKE_TEAM)
        assert e.value.code == ERR_TIMEOUT
    finally:
        debug_inject(INJECT_BARRIER_EXTRA, 0)
        debug_inject(INJECT_WAIT_NS, 0)
    # the context is usable: a fresh mesh strokes and matches the oracle
    g2 = PBVH.build_mesh(m, 300)
    g2.set_team(TEAM_GRID)
    s = g2.stroke(st, mode=STROKE_TEAM)
    o = oracle.OracleMesh.faces(m, 300)
    o.recalc_all_normals()
    tot, _ = o.stroke(st, which=1)
    assert s.verts_displaced == tot and tot > 0
    assert bits_equal(g2.positions(), o.co()), first_diff(g2.positions(), o.co())
    g.free()
    g2.free()
