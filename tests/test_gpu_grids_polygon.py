"""GPU parity for multires grids over triangle and pentagon base faces whose
base vertices join three or five faces (the other multires tests use quad
tori, four faces a vertex): build with its normals, then whole strokes through
the per-call kernels (graph replay) and the persistent kernel, bit for bit
against the oracle.  The oracle is pinned to the reference on the same meshes
(test_refpin.py::test_grids_polygon_base_match_reference).

Triangles (3 grids of 9x9) fit the persistent kernel's face stage and take its
prefetched base-edge and corner items; pentagons (5 grids) do not and take the
unstaged seams; the icosahedron's base-vertex sets (5 corner elements) take
the record path of the corner items."""
import numpy as np
import pytest

from dune_sculpt_gb300 import synth
from dune_sculpt_gb300.sculpt import PBVH, STROKE_GRAPH, STROKE_TEAM

from helpers import bits_equal, first_diff

pytestmark = pytest.mark.gpu


def _mesh(base):
    if base == "icosahedron":
        co, tris = synth.icosphere(0)
        return synth.polygon_grids(co, [list(t) for t in tris], 4)
    co, polys = synth.pentagonal_prism()
    return synth.polygon_grids(co, polys, 4)


def _assert_equal(gp, o, what):
    assert bits_equal(gp.positions(), o.co()), what + " co " + first_diff(gp.positions(), o.co())
    assert bits_equal(gp.normals(), o.no()), what + " no " + first_diff(gp.normals(), o.no())
    assert bits_equal(gp.mask(), o.mask()), what + " mask " + first_diff(gp.mask(), o.mask())
    for a, b in zip(gp.bbs(), o.bbs()):
        assert bits_equal(a, b), what + " bb " + first_diff(a, b)


CASES = [(STROKE_GRAPH, 0, synth.SYMM_X), (STROKE_TEAM, -1, 0), (STROKE_TEAM, -1, synth.SYMM_X),
         (STROKE_TEAM, 8, synth.SYMM_X)]


@pytest.mark.parametrize("case", CASES, ids=["graph", "grid", "grid-xmirror", "cluster8-xmirror"])
@pytest.mark.parametrize("base", ["icosahedron", "pentagonal_prism"])
def test_polygon_base_stroke(gpu, oracle, base, case):
    mode, team, symm = case
    g = _mesh(base)
    gp = PBVH.build_grids(g, 4)
    o = oracle.OracleMesh.grids(g, 4)
    o.recalc_all_normals()
    _assert_equal(gp, o, "build")
    if mode == STROKE_TEAM:
        gp.set_team(team)
    dabs = synth.arc_dabs(synth.SEED_BASE + 11, 16, 0.25, 0.85)
    tools = np.array([(synth.TOOL_DRAW, synth.TOOL_SMOOTH, synth.TOOL_INFLATE,
                       synth.TOOL_CLAY_STRIPS)[d % 4] for d in range(dabs.shape[0])],
                     dtype=np.int32)
    st = synth.Stroke(synth.TOOL_DRAW, 0.3, 0.6, synth.CURVE_SMOOTH, symm, dabs)
    for k in range(2):  # a second stroke continues from the first
        s = gp.stroke(st, mode=mode, dab_tools=tools)
        tot, _ = o.stroke(st, which=1, dab_tools=tools)
        assert s.verts_displaced == tot and tot > 0
        _assert_equal(gp, o, f"{base} stroke {k}")
