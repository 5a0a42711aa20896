"""Ray cast on the GPU (sgpu_raycast) against the oracle's restatement of
BKE_pbvh_raycast with the sculpt callback (itself pinned to the reference's
compiled ray cast in test_refpin.py): hit flag, depth, active vertex, active
face and face normal bit for bit, over vb and orig_vb, bounded and unbounded
ray lengths, axis-aligned directions, and after strokes have moved the mesh."""
import numpy as np
import pytest

from dune_sculpt_gb300 import synth
from dune_sculpt_gb300.sculpt import PBVH, STROKE_TEAM

from helpers import bits_equal, small_grid, small_icosphere, small_uvsphere

pytestmark = pytest.mark.gpu

FLT_MAX = np.float32(3.4028235e38)


def rays(seed, n, center, radius):
    rng = np.random.default_rng(seed)
    starts, dirs = [], []
    for k in range(n):
        s = rng.normal(size=3)
        s = center + s / np.linalg.norm(s) * radius
        if k % 7 == 0:
            d = np.zeros(3)
            ax = k % 3
            d[ax] = -1.0 if s[ax] > center[ax] else 1.0
        else:
            t = center + rng.normal(size=3) * 0.1 * radius
            d = (t - s) / np.linalg.norm(t - s)
        starts.append(s)
        dirs.append(d)
    return np.asarray(starts, np.float32), np.asarray(dirs, np.float32)


def compare(gp, o, starts, dirs, lengths, original):
    hit, dep, av, af, fn = gp.raycast(starts, dirs, lengths, original)
    nhit = 0
    for r in range(starts.shape[0]):
        length = FLT_MAX if lengths is None else lengths[r]
        h, d, a, f, n, _ = o.raycast(starts[r], dirs[r], length, original)
        assert hit[r] == h, r
        assert bits_equal(np.float32(dep[r]).reshape(1), np.float32(d).reshape(1)), (r, dep[r], d)
        assert av[r] == a and af[r] == f, (r, av[r], a, af[r], f)
        assert bits_equal(fn[r], n), (r, fn[r], n)
        nhit += h
    return nhit


@pytest.mark.parametrize("kind", ["grid", "icosphere", "uvsphere"])
def test_raycast_matches_oracle(gpu, oracle, kind):
    m = {"grid": lambda: small_grid(96), "icosphere": lambda: small_icosphere(5),
         "uvsphere": lambda: small_uvsphere(80)}[kind]()
    gp = PBVH.build_mesh(m, 600)
    o = oracle.OracleMesh.faces(m, 600)
    o.recalc_all_normals()
    co = o.co()
    center = (co.min(0) + co.max(0)) / 2
    radius = float(np.linalg.norm(co.max(0) - co.min(0)))
    starts, dirs = rays(3, 257, center, radius)
    lengths = np.where(np.arange(257) % 3 == 0, np.float32(0.8 * radius), FLT_MAX).astype(np.float32)
    assert compare(gp, o, starts, dirs, None, 0) > 50
    compare(gp, o, starts, dirs, lengths, 1)
    # one ray at a time gives the same as the batch
    compare(gp, o, starts[:5], dirs[:5], None, 0)


def test_raycast_after_stroke(gpu, oracle):
    m = small_icosphere(5)
    st = synth.Stroke(synth.TOOL_INFLATE, 0.2, 0.8, synth.CURVE_SMOOTH, synth.SYMM_X,
                      synth.arc_dabs(7, 24, 0.1))
    gp = PBVH.build_mesh(m, 600)
    gp.stroke(st, mode=STROKE_TEAM)
    o = oracle.OracleMesh.faces(m, 600)
    o.recalc_all_normals()
    o.stroke(st, which=1)
    starts, dirs = rays(11, 200, np.zeros(3), 3.0)
    assert compare(gp, o, starts, dirs, None, 0) > 50
    compare(gp, o, starts, dirs, None, 1)


def test_raycast_edge_cases(gpu, oracle):
    m = small_grid(32)
    gp = PBVH.build_mesh(m, 300)
    o = oracle.OracleMesh.faces(m, 300)
    o.recalc_all_normals()
    # rays along the grid plane, through vertices and edges, from above, missing
    starts = np.array([[0.5, 0.5, 1.0], [0.25, 0.25, 2.0], [-1.0, 0.5, 0.0], [2.0, 2.0, 1.0],
                       [0.5, 0.5, -1.0], [0.03125, 0.0625, 0.5]], np.float32)
    dirs = np.array([[0, 0, -1], [0, 0, -1], [1, 0, 0], [0, 0, -1], [0, 0, 1], [0, 0, -1]],
                    np.float32)
    compare(gp, o, starts, dirs, None, 0)
    # zero rays is a no-op
    hit, dep, _, _, _ = gp.raycast(np.zeros((0, 3)), np.zeros((0, 3)))
    assert hit.shape == (0,)


def _torus_rays(seed, n):
    rng = np.random.default_rng(seed)
    starts, dirs = [], []
    for _ in range(n):
        s = rng.normal(size=3)
        s = 2.5 * s / np.linalg.norm(s)
        t = rng.normal(size=3) * 0.6
        starts.append(s)
        dirs.append((t - s) / np.linalg.norm(t - s))
    return np.asarray(starts, np.float32), np.asarray(dirs, np.float32)


@pytest.mark.parametrize("level,leaf_limit,jitter", [(4, 0, 0.0), (4, 0, 0.02), (5, 4, 0.01),
                                                     (3, 1, 0.03)])
def test_grids_raycast_matches_oracle(gpu, oracle, level, leaf_limit, jitter):
    """PBVH_GRIDS (pbvh_grids_node_raycast, pbvh.c:4110-4201): the jittered
    tori hold folded quads whose second triangle is the closer hit, which the
    GPU replays in order; the active vertex is the grid element, the face the
    grid."""
    g = synth.torus_grids(16, 6, level=level)
    if jitter:
        rng = np.random.default_rng(9)
        g.co = (g.co + rng.normal(size=g.co.shape) * jitter).astype(np.float32)
    gp = PBVH.build_grids(g, leaf_limit)
    o = oracle.OracleMesh.grids(g, leaf_limit)
    o.recalc_all_normals()
    starts, dirs = _torus_rays(5, 300)
    lengths = np.where(np.arange(300) % 3 == 0, np.float32(2.4), FLT_MAX).astype(np.float32)
    assert compare(gp, o, starts, dirs, None, 0) > 100
    compare(gp, o, starts, dirs, lengths, 1)
    if jitter:
        special = sum(o.grids_special_quads(starts[r], dirs[r]) > 0 for r in range(300))
        assert special > 20
    compare(gp, o, starts[:3], dirs[:3], None, 0)


def test_grids_raycast_after_stroke(gpu, oracle):
    g = synth.torus_grids(16, 6, level=4)
    st = synth.Stroke(synth.TOOL_DRAW, 0.15, 0.9, synth.CURVE_SMOOTH, synth.SYMM_X,
                      synth.torus_dabs(31, 16, 0.15))
    gp = PBVH.build_grids(g, 4)
    gp.stroke(st, mode=STROKE_TEAM)
    o = oracle.OracleMesh.grids(g, 4)
    o.recalc_all_normals()
    o.stroke(st, which=1)
    assert bits_equal(gp.positions(), o.co())
    starts, dirs = _torus_rays(13, 200)
    assert compare(gp, o, starts, dirs, None, 0) > 80
    compare(gp, o, starts, dirs, None, 1)
