"""The host-buffer strokes (sgpu_stroke_host for PBVH_FACES,
sgpu_stroke_host_grids for PBVH_GRIDS): given the handle's own positions and
normals, the positions they hand back and the vertices they report displaced
equal a device-resident stroke of the same input on the same handle, bit for
bit, in the persistent and graph modes — also into a page-locked output,
where the device writes only the changed grids (a separate buffer, and the
input buffer itself)."""
import numpy as np
import pytest

from dune_sculpt_gb300 import synth
from dune_sculpt_gb300.sculpt import PBVH, STROKE_GRAPH, STROKE_TEAM, TEAM_GRID, PinnedArray

from helpers import bits_equal, first_diff, small_icosphere

pytestmark = pytest.mark.gpu

MIXED = [synth.TOOL_DRAW, synth.TOOL_SMOOTH, synth.TOOL_INFLATE]


@pytest.mark.parametrize("mode", [STROKE_TEAM, STROKE_GRAPH])
@pytest.mark.parametrize("team", [8, TEAM_GRID])
def test_grids_host_stroke_matches_device_stroke(gpu, mode, team):
    gm = synth.torus_grids(24, 8, level=4, seed=synth.SEED_BASE + 4)
    gp = PBVH.build_grids(gm, 4)
    gp.set_team(team)
    gp.snapshot()
    co0, no0 = gp.positions(), gp.normals()
    dabs = synth.torus_dabs(31, 24, 0.12)
    tools = np.array([MIXED[d % 3] for d in range(dabs.shape[0])], dtype=np.int32)
    st = synth.Stroke(synth.TOOL_DRAW, 0.12, 0.6, synth.CURVE_SMOOTH, synth.SYMM_X, dabs)
    s1 = gp.stroke(st, mode=mode, dab_tools=tools)
    want = gp.positions()
    assert s1.verts_displaced > 0
    for _ in range(2):  # twice: the second call starts from the first one's leftovers
        gp.restore()
        out = np.zeros_like(co0)
        s2 = gp.stroke_host_grids(st, co0, out, no0, dab_tools=tools, mode=mode)
        assert s2.verts_displaced == s1.verts_displaced, (s2.verts_displaced, s1.verts_displaced)
        assert bits_equal(out, want), first_diff(out, want)
        assert bits_equal(gp.positions(), want)


@pytest.mark.parametrize("mode", [STROKE_TEAM, STROKE_GRAPH])
def test_faces_host_stroke_matches_device_stroke(gpu, mode):
    m = small_icosphere(5)
    g = PBVH.build_mesh(m, 600)
    g.set_team(TEAM_GRID)
    g.snapshot()
    verts0 = g.verts()
    no0 = g.normals()
    st = synth.Stroke(synth.TOOL_DRAW, 0.15, 0.6, synth.CURVE_SMOOTH, synth.SYMM_X,
                      synth.arc_dabs(13, 20, 0.04))
    s1 = g.stroke(st, mode=mode)
    want = g.verts()
    for _ in range(2):
        g.restore()
        out = np.zeros_like(verts0)
        s2 = g.stroke_host(st, verts0, out, no0, mode=mode)
        assert s2.verts_displaced == s1.verts_displaced
        got, ref = np.ascontiguousarray(out["co"]), np.ascontiguousarray(want["co"])
        assert bits_equal(got, ref), first_diff(got, ref)


@pytest.mark.parametrize("in_place", [False, True])
def test_grids_host_stroke_into_page_locked_output(gpu, in_place):
    gm = synth.torus_grids(24, 8, level=4, seed=synth.SEED_BASE + 4)
    gp = PBVH.build_grids(gm, 4)
    gp.set_team(TEAM_GRID)
    gp.snapshot()
    co0, no0 = gp.positions(), gp.normals()
    dabs = synth.torus_dabs(31, 24, 0.12)
    tools = np.array([MIXED[d % 3] for d in range(dabs.shape[0])], dtype=np.int32)
    st = synth.Stroke(synth.TOOL_DRAW, 0.12, 0.6, synth.CURVE_SMOOTH, synth.SYMM_X, dabs)
    s1 = gp.stroke(st, mode=STROKE_TEAM, dab_tools=tools)
    want = gp.positions()
    changed = np.any((want != co0).reshape(-1, gm.grid_size * gm.grid_size * 3), axis=1)
    assert 0 < changed.sum() < changed.size  # some grids change, some do not
    cin = PinnedArray(co0.shape, np.float32)
    cout = cin if in_place else PinnedArray(co0.shape, np.float32)
    nin = PinnedArray(no0.shape, np.float32)
    nin.array[:] = no0
    for rep in range(2):
        gp.restore()
        cin.array[:] = co0
        if not in_place:
            cout.array[:] = np.float32(7.0)  # stale contents the call must replace
        s2 = gp.stroke_host_grids(st, cin.array, cout.array, nin.array, dab_tools=tools,
                                  mode=STROKE_TEAM)
        assert s2.verts_displaced == s1.verts_displaced
        assert bits_equal(cout.array, want), (rep, first_diff(cout.array, want))
        assert bits_equal(gp.positions(), want)
    for a in {id(x): x for x in (cin, cout, nin)}.values():
        a.free()


@pytest.mark.parametrize("in_place", [False, True])
def test_faces_host_stroke_into_page_locked_output(gpu, in_place):
    m = small_icosphere(5)
    g = PBVH.build_mesh(m, 600)
    g.set_team(TEAM_GRID)
    g.snapshot()
    verts0 = g.verts()
    no0 = g.normals()
    st = synth.Stroke(synth.TOOL_DRAW, 0.15, 0.6, synth.CURVE_SMOOTH, synth.SYMM_X,
                      synth.arc_dabs(13, 20, 0.04))
    s1 = g.stroke(st, mode=STROKE_TEAM)
    want = g.verts()
    vin = PinnedArray(verts0.shape, verts0.dtype)
    vout = vin if in_place else PinnedArray(verts0.shape, verts0.dtype)
    nin = PinnedArray(no0.shape, np.float32)
    nin.array[:] = no0
    for rep in range(2):
        g.restore()
        vin.array[:] = verts0
        if not in_place:
            vout.array["co"] = np.float32(7.0)  # stale contents the call must replace
        s2 = g.stroke_host(st, vin.array, vout.array, nin.array, mode=STROKE_TEAM)
        assert s2.verts_displaced == s1.verts_displaced
        got, ref = np.ascontiguousarray(vout.array["co"]), np.ascontiguousarray(want["co"])
        assert bits_equal(got, ref), (rep, first_diff(got, ref))
        assert vout.array.tobytes() == want.tobytes()
    for a in {id(x): x for x in (vin, vout, nin)}.values():
        a.free()
