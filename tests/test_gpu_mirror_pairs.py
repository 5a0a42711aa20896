"""Paired symmetry passes in the persistent stroke kernel.  With a single-axis
symmetry one node search lists the leaves of both passes; lists without a
common leaf under draw, inflate, pinch, crease or clay strips run as one pass
pair (one area phase with a pairwise tree per pass, one sweep), overlapping
lists and the smooth brush run the passes one after the other from the stored
second list, and lists too long to store both make the second pass search
again.  Every case must equal the FP32 restatement's passes, run one after the
other, bit for bit (positions, normals, boxes, node flags, vertices moved)."""
import numpy as np
import pytest

from dune_sculpt_gb300 import synth
from dune_sculpt_gb300.sculpt import BATCH_TEAM, PBVH, STROKE_TEAM, TEAM_GRID, batch_stroke

from helpers import bits_equal, first_diff, small_icosphere, small_uvsphere

pytestmark = pytest.mark.gpu

JOINABLE = [synth.TOOL_DRAW, synth.TOOL_INFLATE, synth.TOOL_PINCH, synth.TOOL_CREASE,
            synth.TOOL_CLAY_STRIPS]
SYMM_Y, SYMM_Z = 2, 4


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
    assert np.array_equal(g.nodes()["flag"] & 15, o.nodes()["flag"] & 15), what + " flags"


def _arc_near(centre, n, step, seed):
    """n dabs on the unit sphere along a short arc through the direction centre."""
    c = np.asarray(centre, dtype=np.float64)
    c /= np.linalg.norm(c)
    g = synth.gaussian(seed, 5, 3)
    u = np.cross(c, g)
    u /= np.linalg.norm(u)
    pts = np.array([c + step * (k - n / 2) * u for k in range(n)])
    pts /= np.linalg.norm(pts, axis=1)[:, None]
    return synth._dabs_from_points(pts)


def _mirror(loc, sym):
    out = np.array(loc, dtype=np.float32)
    for k in range(3):
        if (sym >> k) & 1:
            out[k] = -out[k]
    return out


def _cull_rsq(st, tool):
    r = np.float32(st.radius)
    if tool == synth.TOOL_CLAY_STRIPS:
        r = np.float32(r * np.float32(1.41421356237309504880))
    return float(np.float32(r * r))


def _overlaps(o, st, tools):
    """Per dab: do the two passes' leaf lists share a leaf (at the stroke start)?"""
    out = []
    for d, t in zip(st.dabs, tools):
        rsq = _cull_rsq(st, t)
        a = set(o.search_sphere(d[:3], rsq).tolist())
        b = set(o.search_sphere(_mirror(d[:3], st.symmetry), rsq).tolist())
        out.append(bool(a & b))
    return out


@pytest.mark.parametrize("team", [16, TEAM_GRID])
@pytest.mark.parametrize("sym", [synth.SYMM_X, SYMM_Y, SYMM_Z])
def test_disjoint_pairs_per_tool(gpu, oracle, team, sym):
    """Dabs far from every mirror plane: the joinable tools run as pass pairs,
    smooth runs its passes in turn from the stored list; tools change per dab."""
    m = small_uvsphere(64)
    g, o = _pair(oracle, m, 300)
    g.set_team(team)
    dabs = _arc_near([0.6, 0.55, 0.58], 18, 0.03, seed=7)
    cycle = JOINABLE + [synth.TOOL_SMOOTH]
    tools = np.array([cycle[d % len(cycle)] for d in range(dabs.shape[0])], dtype=np.int32)
    st = synth.Stroke(synth.TOOL_DRAW, 0.1, 0.7, synth.CURVE_SMOOTH, sym, dabs)
    assert not any(_overlaps(o, st, tools))
    s = g.stroke(st, mode=STROKE_TEAM, dab_tools=tools)
    tot, _ = o.stroke(st, which=1, dab_tools=tools)
    assert s.verts_displaced == tot and tot > 0
    _assert_equal(g, o, f"sym {sym} team {team}")


@pytest.mark.parametrize("team", [16, TEAM_GRID])
def test_overlapping_pairs(gpu, oracle, team):
    """A stroke across the mirror plane: some dabs' lists share leaves (the
    passes run in turn), others do not (pairs)."""
    m = small_uvsphere(64)
    g, o = _pair(oracle, m, 300)
    g.set_team(team)
    dabs = _arc_near([0.0, 0.3, 0.95], 30, 0.04, seed=8)
    tools = np.array([JOINABLE[d % len(JOINABLE)] for d in range(dabs.shape[0])], dtype=np.int32)
    st = synth.Stroke(synth.TOOL_CLAY_STRIPS, 0.08, 0.6, synth.CURVE_SHARP, synth.SYMM_X, dabs)
    ov = _overlaps(o, st, tools)
    assert any(ov) and not all(ov)
    s = g.stroke(st, mode=STROKE_TEAM, dab_tools=tools)
    tot, _ = o.stroke(st, which=1, dab_tools=tools)
    assert s.verts_displaced == tot
    _assert_equal(g, o, f"overlapping team {team}")


@pytest.mark.parametrize("tool", [synth.TOOL_DRAW, synth.TOOL_SMOOTH])
def test_pair_lists_too_long_to_store(gpu, oracle, tool):
    """A radius that lists every leaf in both passes: the two lists do not
    fit the list arrays together, so the second pass searches again."""
    m = small_icosphere(3)
    g, o = _pair(oracle, m, 40)
    g.set_team(TEAM_GRID)
    assert o.num_leaves > 2
    st = synth.Stroke(tool, 2.5, 0.3, synth.CURVE_SMOOTH, synth.SYMM_X,
                      _arc_near([0.5, 0.5, 0.7], 4, 0.05, seed=9))
    s = g.stroke(st, mode=STROKE_TEAM)
    tot, _ = o.stroke(st, which=1)
    assert s.verts_displaced == tot
    _assert_equal(g, o, f"full cover tool {tool}")


@pytest.mark.parametrize("cluster", [8, 16])
def test_pairs_in_cluster_batch(gpu, oracle, cluster):
    """Cluster teams of a batch with X-mirrored strokes beside one without."""
    meshes = [(small_uvsphere(48), 300), (small_icosphere(4), 200), (small_uvsphere(40), 200)]
    jobs = [_pair(oracle, m, ll) for m, ll in meshes]
    strokes = [
        synth.Stroke(synth.TOOL_CLAY_STRIPS, 0.1, 0.8, synth.CURVE_SHARP, synth.SYMM_X,
                     _arc_near([0.6, 0.5, 0.6], 12, 0.03, seed=10)),
        synth.Stroke(synth.TOOL_DRAW, 0.12, 0.6, synth.CURVE_SMOOTH, synth.SYMM_X,
                     _arc_near([0.05, 0.6, 0.8], 12, 0.04, seed=11)),
        synth.Stroke(synth.TOOL_INFLATE, 0.1, 0.5, synth.CURVE_SMOOTH, 0,
                     _arc_near([0.6, 0.5, 0.6], 12, 0.03, seed=12)),
    ]
    stats, ms = batch_stroke([g for g, _ in jobs], strokes, mode=BATCH_TEAM, cluster=cluster)
    assert ms > 0
    for k, ((g, o), st, s) in enumerate(zip(jobs, strokes, stats)):
        tot, _ = o.stroke(st, which=1)
        assert s.verts_displaced == tot, (k, s.verts_displaced, tot)
        _assert_equal(g, o, f"batch mesh {k}")


@pytest.mark.parametrize("team", [16, TEAM_GRID])
@pytest.mark.parametrize("strength", [0.2, 0.6, 0.95])
def test_smooth_pairs(gpu, oracle, team, strength):
    """Smooth with X symmetry: dabs far from the mirror plane pair their
    passes (no leaf of one pass joined to a leaf of the other by an edge),
    dabs near it run the passes in turn; strengths give no full sweep, two
    and three."""
    m = small_icosphere(4)
    g, o = _pair(oracle, m, 200)
    g.set_team(team)
    far = _arc_near([0.7, 0.4, 0.6], 10, 0.03, seed=13)
    near = _arc_near([0.03, 0.5, 0.86], 10, 0.03, seed=14)
    dabs = np.concatenate([far, near, far[::-1]])
    st = synth.Stroke(synth.TOOL_SMOOTH, 0.12, strength, synth.CURVE_SMOOTH, synth.SYMM_X, dabs)
    s = g.stroke(st, mode=STROKE_TEAM)
    tot, _ = o.stroke(st, which=1)
    assert s.verts_displaced == tot and tot > 0
    _assert_equal(g, o, f"smooth {strength} team {team}")


@pytest.mark.parametrize("team", [8, TEAM_GRID])
def test_grids_pairs(gpu, oracle, team):
    """Multires: a stroke around the torus with X symmetry crosses the mirror
    plane (passes in turn) and runs far from it (pairs; smooth pairs on
    disjoint leaves alone, its neighbours being in-grid); draw, smooth and
    inflate by turns, positions, normals, masks and boxes bit for bit."""
    gm = synth.torus_grids(16, 6, level=4, seed=synth.SEED_BASE + 4)
    g = PBVH.build_grids(gm, 4)
    o = oracle.OracleMesh.grids(gm, 4)
    o.recalc_all_normals()
    g.set_team(team)
    # on the ring (torus_grids: R 1, r 0.35) at tube angle 0.3: u 1.2..1.9
    # crosses the plane x = 0, u -0.3..0.3 stays far from it
    ring = 1.0 + 0.35 * np.cos(0.3)
    u = np.concatenate([np.linspace(1.2, 1.9, 20), np.linspace(-0.3, 0.3, 20)])
    pts = np.stack([ring * np.cos(u), ring * np.sin(u), np.full(u.size, 0.35 * np.sin(0.3))], 1)
    dabs = synth._dabs_from_points(pts)
    mixed = [synth.TOOL_DRAW, synth.TOOL_SMOOTH, synth.TOOL_INFLATE]
    tools = np.array([mixed[d % 3] for d in range(dabs.shape[0])], dtype=np.int32)
    st = synth.Stroke(synth.TOOL_DRAW, 0.12, 0.6, synth.CURVE_SMOOTH, synth.SYMM_X, dabs)
    ov = _overlaps(o, st, tools)
    assert any(ov) and not all(ov)
    s = g.stroke(st, mode=STROKE_TEAM, dab_tools=tools)
    tot, _ = o.stroke(st, which=1, dab_tools=tools)
    assert s.verts_displaced == tot
    _assert_equal(g, o, f"grids team {team}")
    assert bits_equal(g.mask(), o.mask())
