"""Known-answer tests that pin the CPU oracle to the reference's definitions.

The reference ships no test, fixture or golden vector for this path (and does
not compile), so the oracle is pinned by answers that follow from the
reference's own code: curve-table end points of the presets
(colortools.c:298-316), flat-grid normals, radial sphere normals, the
bounding-box union invariant of the build (pbvh.c:2240-2247, 3287-3317), the
DFS search order (pbvh.c:2664-2705), an analytic draw displacement on a flat
grid (draw, pinch, crease), and a zero-strength no-op.
"""
import math

import numpy as np
import pytest

from dune_sculpt_gb300 import synth

from helpers import small_grid, small_icosphere


def test_curve_tables_endpoints(oracle):
    for preset in (synth.CURVE_SMOOTH, synth.CURVE_SHARP):
        t, p = oracle.curve_table(preset)
        assert t[0, 0] == 0.0 and t[0, 1] == 1.0
        assert abs(t[256, 0] - 1.0) < 1e-6 and abs(t[256, 1]) < 1e-6
        assert p[0] == 0.0 and p[1] == 1.0 and p[2] == 256.0
        # auto handles overshoot the end values slightly (sharp: -7e-4 near x=1),
        # which evaluation clips; otherwise the falloff is non-increasing
        assert np.all(np.diff(t[:, 1]) <= 1e-4)
        assert t[:, 1].max() <= 1.0 + 1e-4 and t[:, 1].min() >= -1e-3
        ev = [oracle.curve_strength(preset, x, 1.0) for x in np.linspace(0, 1, 101)]
        assert min(ev) >= 0.0 and max(ev) <= 1.0
        assert oracle.curve_strength(preset, 0.0, 1.0) == 1.0
        assert oracle.curve_strength(preset, 1.0, 1.0) == 0.0
        assert oracle.curve_strength(preset, 2.0, 1.0) == 0.0
    # the smooth preset passes (near) its control points
    assert abs(oracle.curve_strength(synth.CURVE_SMOOTH, 0.25, 1.0) - 0.94) < 0.02
    assert abs(oracle.curve_strength(synth.CURVE_SMOOTH, 0.75, 1.0) - 0.06) < 0.02
    # MAX preset is flat at 1; LINE goes 1 -> 0 linearly
    t, _ = oracle.curve_table(3)
    assert np.all(t[:, 1] == 1.0)
    t, _ = oracle.curve_table(0)
    assert np.allclose(t[:, 1], 1.0 - t[:, 0], atol=2e-3)


def test_flat_grid_normals_and_bbs(oracle):
    m = small_grid(32)
    om = oracle.OracleMesh.faces(m, 200)
    om.recalc_all_normals()
    no = om.no()
    assert np.all(no[:, 2] == 1.0) and np.all(no[:, :2] == 0.0)
    nd = om.nodes()
    vb, ovb = om.bbs()
    co = om.co()
    vi = om.vert_indices()
    for n in range(om.num_nodes):
        if nd["children_offset"][n] >= 0:
            c = nd["children_offset"][n]
            union = np.concatenate([np.minimum(vb[c, :3], vb[c + 1, :3]),
                                    np.maximum(vb[c, 3:], vb[c + 1, 3:])])
            assert np.array_equal(vb[n], union)
        else:
            idx = vi[nd["vert_off"][n]:nd["vert_off"][n] + nd["uniq"][n] + nd["face_verts"][n]]
            pts = co[idx]
            assert np.array_equal(vb[n, :3], pts.min(0)) and np.array_equal(vb[n, 3:], pts.max(0))
    assert np.array_equal(vb, ovb)
    # every vertex is unique to exactly one leaf
    uniq = np.concatenate([vi[nd["vert_off"][n]:nd["vert_off"][n] + nd["uniq"][n]]
                           for n in range(om.num_nodes) if nd["children_offset"][n] < 0])
    assert np.array_equal(np.sort(uniq), np.arange(m.totvert))
    # leaf primitive counts respect the leaf limit and cover every looptri
    prims = om.prim_indices()
    assert np.array_equal(np.sort(prims), np.arange(m.looptris.shape[0]))
    assert nd["totprim"].max() <= 200


def test_icosphere_normals_radial(oracle):
    m = synth._faces_from_polys(*synth.icosphere(4))
    om = oracle.OracleMesh.faces(m, 300)
    om.recalc_all_normals()
    co = om.co().astype(np.float64)
    no = om.no().astype(np.float64)
    radial = co / np.linalg.norm(co, axis=1, keepdims=True)
    assert np.abs(np.einsum("ij,ij->i", no, radial) - 1.0).max() < 1e-3
    assert np.abs(np.linalg.norm(no, axis=1) - 1.0).max() < 1e-6


def _dfs_leaves(nd):
    out, stack = [], [0]
    while stack:
        n = stack.pop()
        if nd["children_offset"][n] < 0:
            out.append(n)
        else:
            stack += [nd["children_offset"][n] + 1, nd["children_offset"][n]]
    return out


def test_search_order_and_pruning(oracle):
    m = small_icosphere(4)
    om = oracle.OracleMesh.faces(m, 150)
    nd = om.nodes()
    vb, _ = om.bbs()
    parent = {}
    for n in range(om.num_nodes):
        if nd["children_offset"][n] >= 0:
            parent[nd["children_offset"][n]] = n
            parent[nd["children_offset"][n] + 1] = n
    order = _dfs_leaves(nd)
    rng = np.random.default_rng(5)
    for _ in range(40):
        c = rng.normal(size=3)
        c = (c / np.linalg.norm(c)).astype(np.float32)
        r = np.float32(rng.uniform(0.02, 0.6))
        got = om.search_sphere(c, float(r * r))

        def hits(n):
            near = np.clip(c, vb[n, :3], vb[n, 3:])
            t = (c - near).astype(np.float32)
            return float(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]) < float(r * r)

        want = []
        for leaf in order:
            ok, n = hits(leaf), leaf
            while ok and n in parent:
                n = parent[n]
                ok = hits(n)
            if ok:
                want.append(leaf)
        assert list(got) == want


def test_flat_grid_draw_analytic(oracle):
    """Draw on a flat +Z grid: area normal is +Z, so each vertex within the radius
    moves by radius*strength*falloff(dist/radius) along z; x, y stay put."""
    m = small_grid(64)
    st = synth.Stroke(synth.TOOL_DRAW, 0.1, 0.5, synth.CURVE_SMOOTH, 0,
                      np.array([[0.5, 0.5, 0.0, 1.0, 0.0, 0.0]], dtype=np.float32))
    om = oracle.OracleMesh.faces(m, 400)
    om.recalc_all_normals()
    co0 = om.co().astype(np.float64)
    tot, _ = om.stroke(st, which=3)
    co = om.co64()
    d = np.linalg.norm(co0 - [0.5, 0.5, 0.0], axis=1)
    t, _ = oracle.curve_table(synth.CURVE_SMOOTH)
    p = d / 0.1
    fi = p * 256.0
    i = np.minimum(fi.astype(int), 255)
    f = fi - i
    fall = np.where(d < 0.1, (1 - f) * t[i, 1] + f * t[np.minimum(i + 1, 256), 1], 0.0)
    fall = np.clip(fall, 0, 1)
    assert np.abs(co[:, :2] - co0[:, :2]).max() == 0.0
    assert np.abs(co[:, 2] - 0.1 * 0.5 * fall).max() < 1e-6
    assert tot == int(np.count_nonzero(fall > 0))


def _flat_fall(oracle, co0, c, r):
    d = np.linalg.norm(co0 - c, axis=1)
    t, _ = oracle.curve_table(synth.CURVE_SMOOTH)
    fi = d / r * 256.0
    i = np.minimum(fi.astype(int), 255)
    f = fi - i
    fall = np.where(d < r, (1 - f) * t[i, 1] + f * t[np.minimum(i + 1, 256), 1], 0.0)
    return np.clip(fall, 0, 1)


def test_flat_grid_pinch_analytic(oracle):
    """Pinch on a flat +Z grid with the stroke along +X: the side axis is
    z x delta = +Y, so each vertex within the radius moves along y toward the
    brush centre by strength * falloff of its offset; x and z stay put."""
    m = small_grid(64)
    st = synth.Stroke(synth.TOOL_PINCH, 0.1, 0.5, synth.CURVE_SMOOTH, 0,
                      np.array([[0.5, 0.5, 0.0, 1.0, 0.0, 0.0]], dtype=np.float32))
    om = oracle.OracleMesh.faces(m, 400)
    om.recalc_all_normals()
    co0 = om.co().astype(np.float64)
    tot, _ = om.stroke(st, which=3)
    co = om.co64()
    fall = _flat_fall(oracle, co0, [0.5, 0.5, 0.0], 0.1)
    assert np.abs(co[:, [0, 2]] - co0[:, [0, 2]]).max() == 0.0
    assert np.abs(co[:, 1] - (co0[:, 1] + (0.5 - co0[:, 1]) * 0.5 * fall)).max() < 1e-6
    assert tot == int(np.count_nonzero(fall > 0))


def test_flat_grid_crease_analytic(oracle):
    """Crease on a flat +Z grid: the draw offset along z (radius * strength *
    falloff) plus an in-plane pull toward the centre by
    crease_pinch_factor^2 * strength * falloff."""
    m = small_grid(64)
    st = synth.Stroke(synth.TOOL_CREASE, 0.1, 0.5, synth.CURVE_SMOOTH, 0,
                      np.array([[0.5, 0.5, 0.0, 0.0, 1.0, 0.0]], dtype=np.float32),
                      crease_pinch_factor=0.6)
    om = oracle.OracleMesh.faces(m, 400)
    om.recalc_all_normals()
    co0 = om.co().astype(np.float64)
    om.stroke(st, which=3)
    co = om.co64()
    fall = _flat_fall(oracle, co0, [0.5, 0.5, 0.0], 0.1)
    k = 0.36 * 0.5 * fall
    assert np.abs(co[:, 0] - (co0[:, 0] + (0.5 - co0[:, 0]) * k)).max() < 1e-6
    assert np.abs(co[:, 1] - (co0[:, 1] + (0.5 - co0[:, 1]) * k)).max() < 1e-6
    assert np.abs(co[:, 2] - 0.1 * 0.5 * fall).max() < 1e-6


def test_flat_grid_grab_analytic(oracle):
    """Grab rebuilds each dab from the stroke-start positions: on a flat grid
    every vertex within the radius of the anchor ends at
    orig + delta_last * strength * falloff(|orig - anchor|), whatever the
    earlier dabs did."""
    m = small_grid(64)
    d1 = [0.01, 0.0, 0.02]
    d2 = [0.02, -0.01, 0.05]
    dabs = np.array([[0.5, 0.5, 0.0] + d1, [0.5, 0.5, 0.0] + d2], dtype=np.float32)
    st = synth.Stroke(synth.TOOL_GRAB, 0.1, 0.5, synth.CURVE_SMOOTH, 0, dabs)
    om = oracle.OracleMesh.faces(m, 400)
    om.recalc_all_normals()
    co0 = om.co().astype(np.float64)
    tot, per = om.stroke(st, which=3)
    co = om.co64()
    fall = _flat_fall(oracle, co0, [0.5, 0.5, 0.0], 0.1)
    want = co0 + np.outer(0.5 * fall, np.asarray(d2, np.float32).astype(np.float64))
    assert np.abs(co - want).max() < 1e-6
    assert per[0] == per[1] == int(np.count_nonzero(fall > 0))


def test_flat_grid_layer_analytic(oracle):
    """Layer on a flat +Z grid, one dab: the layer height becomes
    fade * strength * 1.05 and each vertex moves |fade| of the way to
    orig + normal * brush_height * layer, i.e. z = height * 0.525 * fade^2
    for strength 0.5."""
    m = small_grid(64)
    st = synth.Stroke(synth.TOOL_LAYER, 0.1, 0.5, synth.CURVE_SMOOTH, 0,
                      np.array([[0.5, 0.5, 0.0, 1.0, 0.0, 0.0]], dtype=np.float32), height=0.5)
    om = oracle.OracleMesh.faces(m, 400)
    om.recalc_all_normals()
    co0 = om.co().astype(np.float64)
    om.stroke(st, which=3)
    co = om.co64()
    fall = _flat_fall(oracle, co0, [0.5, 0.5, 0.0], 0.1)
    assert np.abs(co[:, :2] - co0[:, :2]).max() == 0.0
    assert np.abs(co[:, 2] - 0.5 * (0.5 * 1.05 * fall) * fall).max() < 1e-6


@pytest.mark.parametrize("kind", [0, 1, 2, 3, 4])
def test_flat_grid_elastic_deform(oracle, kind):
    """Elastic deform moves every vertex (all leaves) by the Kelvinlet
    displacement of its stroke-start position (grab types scaled by
    strength * 20); scale and twist about the +Z normal keep a flat grid flat."""
    m = small_grid(32)
    delta = [0.02, 0.01, 0.0] if kind >= 3 else [0.01, 0.0, 0.02]
    dabs = np.array([[0.5, 0.5, 0.0] + delta], dtype=np.float32)
    st = synth.Stroke(synth.TOOL_ELASTIC_DEFORM, 0.1, 0.5, synth.CURVE_SMOOTH, 0, dabs,
                      view_normal=(0.0, 0.0, 1.0), elastic_deform_type=kind)
    om = oracle.OracleMesh.faces(m, 100)
    om.recalc_all_normals()
    co0 = om.co().copy()
    tot, _ = om.stroke(st, which=1)
    co = om.co()
    force = np.float32(np.float32(np.linalg.norm(np.asarray(delta, np.float32))) * np.float32(0.5))
    dn = np.asarray(delta if kind <= 2 else st.view_normal, np.float32)
    for v in range(0, co0.shape[0], 37):
        k = oracle.kelvinlet(kind, 0.1, force, 0.4, co0[v], dabs[0, :3], dn)
        if kind <= 2:
            k = k * np.float32(np.float32(0.5) * np.float32(20.0))
        assert np.array_equal((co0[v] + k).view(np.uint32), co[v].view(np.uint32)), v
    assert tot == co0.shape[0] - 1 or tot == co0.shape[0]  # all but the centre may move
    if kind >= 3:
        assert np.abs(co[:, 2]).max() == 0.0


def test_zero_strength_is_noop(oracle):
    m = small_icosphere(3)
    om = oracle.OracleMesh.faces(m, 150)
    om.recalc_all_normals()
    co0 = om.co().copy()
    for tool in (synth.TOOL_DRAW, synth.TOOL_INFLATE, synth.TOOL_SMOOTH, synth.TOOL_CLAY_STRIPS,
                 synth.TOOL_PINCH, synth.TOOL_CREASE):
        st = synth.Stroke(tool, 0.2, 0.0, synth.CURVE_SMOOTH, synth.SYMM_X,
                          synth.arc_dabs(1, 4, 0.05))
        om.stroke(st, which=1)
        assert np.array_equal(om.co().view(np.uint32), co0.view(np.uint32)), tool


def test_fp32_restatement_close_to_fp64(oracle):
    m = small_icosphere(4)
    st = synth.Stroke(synth.TOOL_SMOOTH, 0.15, 0.7, synth.CURVE_SMOOTH, synth.SYMM_X,
                      synth.arc_dabs(3, 16, 0.03))
    om = oracle.OracleMesh.faces(m, 300)
    om.recalc_all_normals()
    tot, _ = om.stroke(st, which=3)
    assert tot > 0
    err = np.abs(om.co().astype(np.float64) - om.co64()).max()
    assert err < 1e-6, err
