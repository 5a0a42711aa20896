"""Nearest to ray on the GPU (sgpu_find_nearest_to_ray) against the oracle's
restatement of BKE_pbvh_find_nearest_to_ray with the sculpt callback (itself
pinned to the reference's compiled query in test_refpin.py): hit flag, depth
and squared distance bit for bit, PBVH_FACES and PBVH_GRIDS (smooth and
jittered grids), over vb and orig_vb, one ray per call and batches (the
front-to-back two-round path), and after a stroke has moved the mesh."""
import numpy as np
import pytest

from dune_sculpt_gb300 import synth
from dune_sculpt_gb300.sculpt import PBVH, STROKE_TEAM

from helpers import bits_equal, ngon_mesh, small_grid, small_icosphere, small_uvsphere

pytestmark = pytest.mark.gpu


def near_rays(seed, n, center, radius):
    """Rays from a sphere around the mesh towards points scattered about its
    middle: many pass beside the surface; every seventh axis-aligned."""
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
            t = center + rng.normal(size=3) * 0.45 * radius
            d = (t - s) / np.linalg.norm(t - s)
        starts.append(s)
        dirs.append(d)
    return np.asarray(starts, np.float32), np.asarray(dirs, np.float32)


def compare(gp, o, starts, dirs, original):
    hit, dep, dsq = gp.nearest_to_ray(starts, dirs, original)
    nhit = 0
    for r in range(starts.shape[0]):
        h, d, q, _ = o.nearest_to_ray(starts[r], dirs[r], original)
        assert hit[r] == h, r
        assert bits_equal(np.float32(dep[r]).reshape(1), np.float32(d).reshape(1)), (r, dep[r], d)
        assert bits_equal(np.float32(dsq[r]).reshape(1), np.float32(q).reshape(1)), (r, dsq[r], q)
        nhit += h
    return nhit


def _center_radius(o):
    co = o.co()
    return (co.min(0) + co.max(0)) / 2, float(np.linalg.norm(co.max(0) - co.min(0)))


@pytest.mark.parametrize("kind", ["grid", "icosphere", "uvsphere", "ngon"])
def test_nearest_matches_oracle_faces(gpu, oracle, kind):
    m = {"grid": lambda: small_grid(96), "icosphere": lambda: small_icosphere(5),
         "uvsphere": lambda: small_uvsphere(80), "ngon": lambda: ngon_mesh(60)}[kind]()
    gp = PBVH.build_mesh(m, 600)
    o = oracle.OracleMesh.faces(m, 600)
    o.recalc_all_normals()
    center, radius = _center_radius(o)
    starts, dirs = near_rays(3, 200, center, radius)
    assert compare(gp, o, starts, dirs, 0) > 50
    assert compare(gp, o, starts, dirs, 1) > 50
    for r in range(8):  # one ray per call (one round)
        compare(gp, o, starts[r:r + 1], dirs[r:r + 1], 0)
    # after a stroke (boxes refit, orig_vb from the stroke's end)
    st = synth.Stroke(synth.TOOL_DRAW, 0.15 * radius, 0.8, synth.CURVE_SMOOTH, synth.SYMM_X,
                      synth.arc_dabs(5, 12, 0.05) if kind != "grid" else synth.line_dabs(5, 12))
    gp.stroke(st, mode=STROKE_TEAM)
    o.stroke(st, which=1)
    assert bits_equal(gp.positions(), o.co())
    compare(gp, o, starts, dirs, 0)


@pytest.mark.parametrize("jitter", [0.0, 0.02])
def test_nearest_matches_oracle_grids(gpu, oracle, jitter):
    g = synth.torus_grids(16, 6, level=4)
    rng = np.random.default_rng(5)
    if jitter:
        g.co = (g.co + rng.normal(size=g.co.shape) * jitter).astype(np.float32)
    gp = PBVH.build_grids(g, 4)
    o = oracle.OracleMesh.grids(g, 4)
    o.recalc_all_normals()
    starts, dirs = near_rays(7, 200, np.zeros(3), 2.5)
    assert compare(gp, o, starts, dirs, 0) > 50
    compare(gp, o, starts[:6], dirs[:6], 1)
    for r in range(4):
        compare(gp, o, starts[r:r + 1], dirs[r:r + 1], 0)
