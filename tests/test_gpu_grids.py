"""GPU parity for PBVH_GRIDS (multires): build, brushes, inner grid normals and
seam stitching (subdiv_ccg.c:670-1287) against the CPU oracle, bit for bit."""
import numpy as np
import pytest

from dune_sculpt_gb300 import synth
from dune_sculpt_gb300.sculpt import PBVH, STROKE_EAGER, STROKE_GRAPH

from helpers import bits_equal, first_diff, rel_err

pytestmark = pytest.mark.gpu

# FP32 vs FP64 positions, norm-wise relative.  The GPU equals the FP32
# restatement bit for bit; the FP32 arithmetic itself (seam averages, grid
# normals feeding draw/inflate) drifts up to ~1.1e-6 from FP64 over these
# strokes, so the bound here is 2e-6 (FACES strokes stay under 1e-6).
FP64_TOL_GRIDS = 2e-6

TOOLS = [synth.TOOL_DRAW, synth.TOOL_SMOOTH, synth.TOOL_INFLATE, synth.TOOL_CLAY_STRIPS,
         synth.TOOL_PINCH, synth.TOOL_CREASE]


def small_torus(level=4):
    return synth.torus_grids(16, 6, level=level, seed=synth.SEED_BASE + 4)


def _pair(oracle, g, leaf_limit=4):
    gp = PBVH.build_grids(g, leaf_limit)
    o = oracle.OracleMesh.grids(g, leaf_limit)
    o.recalc_all_normals()
    return gp, o


def _assert_equal(gp, o, what):
    assert bits_equal(gp.positions(), o.co()), what + " co " + first_diff(gp.positions(), o.co())
    assert bits_equal(gp.normals(), o.no()), what + " no " + first_diff(gp.normals(), o.no())
    assert bits_equal(gp.mask(), o.mask()), what + " mask " + first_diff(gp.mask(), o.mask())
    for a, b in zip(gp.bbs(), o.bbs()):
        assert bits_equal(a, b), what + " bb " + first_diff(a, b)


def test_grids_build_and_normals(gpu, oracle):
    g = small_torus()
    gp, o = _pair(oracle, g)
    gn, on = gp.nodes(), o.nodes()
    for k in ("children_offset", "prim_off", "totprim"):
        assert np.array_equal(gn[k], on[k]), k
    assert np.array_equal(gp.prim_indices(), o.prim_indices())
    _assert_equal(gp, o, "build")
    # outward unit-ish normals on the torus
    no = gp.normals().astype(np.float64)
    assert np.all(np.linalg.norm(no, axis=1) > 0.9)


def _seam_consistent(g, co):
    """Every element a base edge or base vertex shares across faces holds one
    position after stitching."""
    gs = g.grid_size
    area = gs * gs
    F = g.num_faces
    # compare corner elements (gs-1, gs-1) of grids around each base vertex
    corners = {}
    for f in range(F):
        for c in range(4):
            v = g.face_verts[4 * f + c]
            corners.setdefault(v, []).append((4 * f + c) * area + (gs - 1) * gs + (gs - 1))
    for els in corners.values():
        ref = co[els[0]]
        for e in els[1:]:
            assert np.array_equal(co[e], ref)
    # centre element shared by a face's grids
    for f in range(F):
        els = [(4 * f + c) * area for c in range(4)]
        for e in els[1:]:
            assert np.array_equal(co[e], co[els[0]])


@pytest.mark.parametrize("tool", TOOLS)
@pytest.mark.parametrize("mode", [STROKE_EAGER, STROKE_GRAPH])
def test_grids_stroke_parity(gpu, oracle, tool, mode):
    g = small_torus()
    gp, o = _pair(oracle, g)
    dabs = synth.torus_dabs(31, 16, 0.15)
    st = synth.Stroke(tool, 0.15, 0.6, synth.CURVE_SMOOTH, synth.SYMM_X, dabs)
    s = gp.stroke(st, mode=mode)
    tot, _ = o.stroke(st, which=3)
    assert s.verts_displaced == tot and tot > 0
    _assert_equal(gp, o, f"tool {tool}")
    assert rel_err(gp.positions(), o.co64()) < FP64_TOL_GRIDS
    _seam_consistent(g, gp.positions())


def test_grids_mixed_stroke(gpu, oracle):
    """Alternating draw / smooth / inflate dabs with a noise mask (the multires
    workload's stroke, small)."""
    g = small_torus(5)
    gp, o = _pair(oracle, g, leaf_limit=8)
    dabs = synth.torus_dabs(41, 24, 0.12)
    tools = np.array([(synth.TOOL_DRAW, synth.TOOL_SMOOTH, synth.TOOL_INFLATE)[d % 3]
                      for d in range(dabs.shape[0])], dtype=np.int32)
    st = synth.Stroke(synth.TOOL_DRAW, 0.12, 0.6, synth.CURVE_SMOOTH, 0, dabs)
    s = gp.stroke(st, mode=STROKE_GRAPH, dab_tools=tools)
    tot, _ = o.stroke(st, which=3, dab_tools=tools)
    assert s.verts_displaced == tot
    _assert_equal(gp, o, "mixed")
    assert rel_err(gp.positions(), o.co64()) < FP64_TOL_GRIDS


@pytest.mark.parametrize("cluster", [1, 8, -1])
def test_grids_team_stroke(gpu, oracle, cluster):
    """The persistent stroke kernel on multires grids, mixed tools, X mirror."""
    from dune_sculpt_gb300.sculpt import STROKE_TEAM

    g = small_torus(5)
    gp, o = _pair(oracle, g, leaf_limit=8)
    gp.set_team(cluster)
    dabs = synth.torus_dabs(43, 24, 0.12)
    tools = np.array([(synth.TOOL_DRAW, synth.TOOL_SMOOTH, synth.TOOL_INFLATE,
                       synth.TOOL_CLAY_STRIPS)[d % 4] for d in range(dabs.shape[0])],
                     dtype=np.int32)
    st = synth.Stroke(synth.TOOL_DRAW, 0.12, 0.6, synth.CURVE_SMOOTH, synth.SYMM_X, dabs)
    s = gp.stroke(st, mode=STROKE_TEAM, dab_tools=tools)
    tot, _ = o.stroke(st, which=1, dab_tools=tools)
    assert s.verts_displaced == tot and tot > 0
    _assert_equal(gp, o, f"team{cluster}")
    _seam_consistent(g, gp.positions())
    # a second stroke continues from the first (epochs, flags, counters)
    s = gp.stroke(st, mode=STROKE_TEAM, dab_tools=tools)
    tot, _ = o.stroke(st, which=1, dab_tools=tools)
    assert s.verts_displaced == tot
    _assert_equal(gp, o, f"team{cluster} second")


@pytest.mark.parametrize("team", [16, -1])
def test_grids_persistent_stroke_unstaged_grids(gpu, oracle, team):
    """Grids of 65x65 do not fit the persistent kernel's shared-memory stage:
    inner normals and face seams per element, then the base edges and corners
    with their owner records made in that phase."""
    from dune_sculpt_gb300.sculpt import STROKE_TEAM

    g = synth.torus_grids(8, 4, level=7, seed=synth.SEED_BASE + 7)
    assert g.grid_size == 65
    gp, o = _pair(oracle, g, 2)
    gp.set_team(team)
    dabs = synth.torus_dabs(5, 10, 0.2)
    tools = np.array([TOOLS[d % len(TOOLS)] for d in range(dabs.shape[0])], dtype=np.int32)
    st = synth.Stroke(synth.TOOL_DRAW, 0.2, 0.6, synth.CURVE_SMOOTH, synth.SYMM_X, dabs)
    s = gp.stroke(st, mode=STROKE_TEAM, dab_tools=tools)
    tot, _ = o.stroke(st, which=1, dab_tools=tools)
    assert s.verts_displaced == tot and tot > 0
    _assert_equal(gp, o, f"unstaged team {team}")
