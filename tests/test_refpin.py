"""The oracle against the reference's own compiled PBVH code (CPU).

oracle/refpin compiles the reference's pbvh.c (complete copy, pbvh.c:1913-4986),
subdiv_ccg.c, BKE_mesh_calc_poly_normal (mesh_evaluate.c:39-86), normal_tri_v3 /
normal_quad_v3 (math_geom.cc:31-68), its inline vector math and the falloff
curve code of colortools.c from the reference tree, behind stand-ins for the
headers the reference does not ship.
These tests check, on the same inputs, that the oracle's restatement gives

* the same PBVH (BKE_pbvh_build_mesh / _build_grids): node table, prim order,
  per-leaf vertex lists with the unique/shared split, node boxes — bit for bit;
* the same node lists from BKE_pbvh_search_gather with the sphere callback,
  over vb and orig_vb — exactly;
* the same boxes after BKE_pbvh_update_bounds (UpdateBB, UpdateOriginalBB) —
  bit for bit;
* the same vertex normals after BKE_pbvh_update_normals within 1e-6 absolute
  (unit vectors): the reference adds face normals with float atomics in task
  order, the oracle in ascending looptri order with compensated sums, so the
  last bit may differ.

* the same multires normals, seam-stitched positions and masks after
  KERNEL_subdiv_ccg_update_normals (the reference builds its own edge / corner
  adjacency) — bit for bit;
* the same falloff tables and curve values — bit for bit.

The replay tests drive whole oracle strokes (draw, smooth, inflate, clay
strips; X symmetry) and, after every dab, hand the oracle's positions, vertex
tags and culled nodes to the reference's update code.

They need the reference tree (to build oracle/_ref/librefpin.so) and skip
without it.
"""
from __future__ import annotations

import numpy as np
import pytest

import pyrefpin
from dune_sculpt_gb300 import synth
from helpers import bits_equal, first_diff, material_grid, ngon_mesh, small_icosphere, small_uvsphere

pytestmark = pytest.mark.skipif(not pyrefpin.available(),
                                reason="reference tree absent: the pinning library cannot be built")

LEAF = 1          # PBVH_Leaf
UPD_BB = 4        # PBVH_UpdateBB
UPD_ORIG_BB = 8   # PBVH_UpdateOriginalBB
NORMAL_ATOL = 1e-6


MESHES = {
    "grid": lambda: synth.grid_mesh(160),
    "icosphere": lambda: small_icosphere(6),
    "uvsphere": lambda: small_uvsphere(180),
    "ngon": lambda: ngon_mesh(120),
    "materials": lambda: material_grid(96),
}


def _pair(oracle, name, leaf_limit):
    m = MESHES[name]()
    o = oracle.OracleMesh.faces(m, leaf_limit)
    o.recalc_all_normals()
    r = pyrefpin.RefPBVH.faces(m, o.no(), leaf_limit)
    return m, o, r


def _assert_same_tree(o, r):
    on, rn = o.nodes(), r.nodes()
    assert o.num_nodes == r.num_nodes
    for k in ("children_offset", "prim_off", "totprim", "uniq", "face_verts"):
        assert np.array_equal(on[k], rn[k]), k
    assert np.array_equal(on["flag"] & LEAF, rn["flag"] & LEAF)
    assert np.array_equal(o.prim_indices(), r.prim_indices())
    ov = o.vert_indices()
    for n in np.nonzero(on["flag"] & LEAF)[0]:
        cnt = on["uniq"][n] + on["face_verts"][n]
        a = ov[on["vert_off"][n]:on["vert_off"][n] + cnt]
        assert np.array_equal(a, r.node_vert_indices(int(n))), f"leaf {n}"
    ovb, oovb = o.bbs()
    rvb, rovb = r.bbs()
    assert bits_equal(ovb, rvb), first_diff(ovb, rvb)
    assert bits_equal(oovb, rovb), first_diff(oovb, rovb)


@pytest.mark.parametrize("leaf_limit", [10000, 5000, 700])
@pytest.mark.parametrize("name", list(MESHES))
def test_build_matches_reference(oracle, name, leaf_limit):
    _, o, r = _pair(oracle, name, leaf_limit)
    assert r.leaf_limit == leaf_limit
    _assert_same_tree(o, r)
    assert int((o.nodes()["flag"] & LEAF).sum()) > 1


@pytest.mark.parametrize("name", list(MESHES))
def test_search_matches_reference(oracle, name):
    m, o, r = _pair(oracle, name, 5000)
    co = m.verts["co"]
    lo, hi = co.min(0), co.max(0)
    rng = np.random.default_rng(7)
    hits = 0
    for _ in range(150):
        c = rng.uniform(lo - 0.1, hi + 0.1).astype(np.float32)
        rsq = np.float32(rng.uniform(0.0, 0.5 * float((hi - lo).max()))) ** 2
        for orig in (0, 1):
            a = o.search_sphere(c, rsq, orig)
            b = r.search_sphere(c, rsq, orig)
            assert np.array_equal(a, b), (c, rsq, orig, a, b)
            hits += a.size
    assert hits > 0
    # empty and all-covering spheres, a zero radius on a vertex
    assert r.search_sphere(hi + 10.0, np.float32(1.0)).size == 0
    assert o.search_sphere(hi + 10.0, np.float32(1.0)).size == 0
    big = np.float32(1e6)
    assert np.array_equal(o.search_sphere(lo, big), r.search_sphere(lo, big))
    assert np.array_equal(o.search_sphere(co[0], np.float32(0.0)),
                          r.search_sphere(co[0], np.float32(0.0)))


def _edit(o, r, co, center, rad, amp):
    """Displace the vertices inside a sphere smoothly, tag them, mark the
    culled nodes, in both; then the reference's and the oracle's updates."""
    rsq = np.float32(rad) * np.float32(rad)
    d2 = ((co - center) ** 2).sum(1)
    inside = np.nonzero(d2 < rsq)[0]
    fall = (np.float32(1) - d2[inside] / rsq).astype(np.float32)
    co = co.copy()
    co[inside] += (np.float32(amp) * fall)[:, None] * np.array([0.3, -0.2, 1.0], np.float32)
    nodes = o.search_sphere(center, rsq, 0)
    assert np.array_equal(nodes, r.search_sphere(center, rsq, 0))
    o.set_co(co)
    r.set_co(co)
    for n in nodes:
        o.node_mark_update(int(n))
        r.node_mark_update(int(n))
    for v in inside:
        o.vert_mark_update(int(v))
        r.vert_mark_update(int(v))
    return co, inside


@pytest.mark.parametrize("name", list(MESHES))
def test_update_normals_and_bounds_match_reference(oracle, name):
    m, o, r = _pair(oracle, name, 5000)
    co = o.co()
    lo, hi = co.min(0), co.max(0)
    rng = np.random.default_rng(11)
    for step in range(4):
        center = rng.uniform(lo, hi).astype(np.float32)
        rad = 0.15 * float((hi - lo).max())
        co, inside = _edit(o, r, co, center, rad, 0.02)
        o.update_normals()
        r.update_normals()
        no_o, no_r = o.no(), r.no()
        err = float(np.abs(no_o - no_r).max())
        assert err <= NORMAL_ATOL, (step, err)
        o.update_bounds(UPD_BB)
        r.update_bounds(UPD_BB)
        ovb, oovb = o.bbs()
        rvb, rovb = r.bbs()
        assert bits_equal(ovb, rvb), first_diff(ovb, rvb)
        assert bits_equal(oovb, rovb), first_diff(oovb, rovb)
        assert np.array_equal(o.nodes()["flag"] & 0xF, r.nodes()["flag"] & 0xF)
    o.update_bounds(UPD_ORIG_BB)
    r.update_bounds(UPD_ORIG_BB)
    ovb, oovb = o.bbs()
    rvb, rovb = r.bbs()
    assert bits_equal(oovb, rovb), first_diff(oovb, rovb)
    assert bits_equal(ovb, rvb)


REPLAY = [
    ("grid", synth.TOOL_DRAW, 0.05, 0.5, synth.CURVE_SMOOTH, 0),
    ("icosphere", synth.TOOL_SMOOTH, 0.12, 0.7, synth.CURVE_SMOOTH, synth.SYMM_X),
    ("uvsphere", synth.TOOL_CLAY_STRIPS, 0.1, 0.8, synth.CURVE_SHARP, synth.SYMM_X),
    ("icosphere", synth.TOOL_INFLATE, 0.1, 0.6, synth.CURVE_SMOOTH, synth.SYMM_X),
    ("ngon", synth.TOOL_DRAW, 0.06, 0.9, synth.CURVE_SHARP, synth.SYMM_X),
    ("icosphere", synth.TOOL_PINCH, 0.1, 0.6, synth.CURVE_SMOOTH, synth.SYMM_X),
    ("uvsphere", synth.TOOL_CREASE, 0.1, 0.7, synth.CURVE_SHARP, synth.SYMM_X),
    ("icosphere", synth.TOOL_LAYER, 0.12, 0.6, synth.CURVE_SMOOTH, synth.SYMM_X),
]


@pytest.mark.parametrize("case", REPLAY, ids=[f"{c[0]}-tool{c[1]}" for c in REPLAY])
def test_stroke_replay_in_reference(oracle, case):
    """Every PBVH step of an oracle stroke re-run by the reference's code."""
    name, tool, radius, strength, curve, symm = case
    m, o, r = _pair(oracle, name, 5000)
    if m.kind == "grid" or m.kind == "ngon":
        dabs = synth.line_dabs(synth.SEED_BASE, 12)
    else:
        dabs = synth.arc_dabs(synth.SEED_BASE + 1, 12, 0.5 * radius)
    st = synth.Stroke(tool, radius, strength, curve, symm, dabs)
    scale = np.float32(1.41421356237309504880) if tool == synth.TOOL_CLAY_STRIPS else np.float32(1)
    rr = np.float32(radius) * scale
    rsq = rr * rr
    moved = 0
    original = 1 if tool == synth.TOOL_LAYER else 0  # layer culls on the original boxes
    if tool == synth.TOOL_LAYER:
        o.store_original()
    for d in range(dabs.shape[0]):
        for p in range(8):
            if p & ~symm:
                continue
            sgn = np.array([-1 if p & (1 << k) else 1 for k in range(3)], np.float32)
            loc = dabs[d, :3] * sgn
            delta = dabs[d, 3:] * sgn
            nodes = o.search_sphere(loc, rsq, original)
            assert np.array_equal(nodes, r.search_sphere(loc, rsq, original)), (d, p)
            n, _ = o.brush_pass(st, loc, delta, nodes)
            moved += n
            for nd in nodes:
                r.node_mark_update(int(nd))
        r.set_co(o.co())
        for v in np.nonzero(o.vert_tags())[0]:
            r.vert_mark_update(int(v))
        o.update_normals()
        r.update_normals()
        err = float(np.abs(o.no() - r.no()).max())
        assert err <= NORMAL_ATOL, (d, err)
        o.update_bounds(UPD_BB)
        r.update_bounds(UPD_BB)
        ovb, _ = o.bbs()
        rvb, _ = r.bbs()
        assert bits_equal(ovb, rvb), (d, first_diff(ovb, rvb))
    o.update_bounds(UPD_ORIG_BB)
    r.update_bounds(UPD_ORIG_BB)
    _, oovb = o.bbs()
    _, rovb = r.bbs()
    assert bits_equal(oovb, rovb)
    assert moved > 0


def test_grids_build_search_bounds_match_reference(oracle):
    """BKE_pbvh_build_grids (leaf = max(limit / 17^2, 1) grids), search and the
    grid-element refit, against the oracle on a multires torus."""
    g = synth.torus_grids(40, 12, 5)
    o = oracle.OracleMesh.grids(g, 0)
    o.recalc_all_normals()
    no = o.no()
    r = pyrefpin.RefPBVH.grids(g.num_grids, g.grid_size, g.co, no, g.mask)
    assert r.leaf_limit == max(10000 // (g.grid_size ** 2), 1)
    on, rn = o.nodes(), r.nodes()
    assert o.num_nodes == r.num_nodes
    for k in ("children_offset", "prim_off", "totprim"):
        assert np.array_equal(on[k], rn[k]), k
    assert np.array_equal(o.prim_indices(), r.prim_indices())
    ovb, oovb = o.bbs()
    rvb, rovb = r.bbs()
    assert bits_equal(ovb, rvb) and bits_equal(oovb, rovb)
    rng = np.random.default_rng(3)
    for _ in range(100):
        c = rng.uniform(-1.4, 1.4, 3).astype(np.float32)
        rsq = np.float32(rng.uniform(0.0, 0.5)) ** 2
        assert np.array_equal(o.search_sphere(c, rsq), r.search_sphere(c, rsq))
    co = g.co.copy()
    center = co[co.shape[0] // 3]
    d2 = ((co - center) ** 2).sum(1)
    inside = d2 < np.float32(0.04)
    co[inside] *= np.float32(1.03)
    nodes = o.search_sphere(center, np.float32(0.04))
    o.set_co(co)
    r.set_grid_co(co)
    for n in nodes:
        o.node_mark_update(int(n))
        r.node_mark_update(int(n))
    o.update_bounds(UPD_BB)
    r.update_bounds(UPD_BB)
    ovb, _ = o.bbs()
    rvb, _ = r.bbs()
    assert bits_equal(ovb, rvb), first_diff(ovb, rvb)


@pytest.mark.parametrize("preset", [0, 1, 2, 3, 5, 6])
def test_curve_table_matches_reference(oracle, preset):
    """Falloff table (KERNEL_curvemap_reset + KERNEL_curvemapping_changed ->
    curvemap_make_table, colortools.c:249-416, 597-771, 846-922) and its
    evaluation (KERNEL_curvemapping_evaluateF, :942-980), bit for bit."""
    t_o, p_o = oracle.curve_table(preset)
    t_r, p_r = pyrefpin.curve_table(preset)
    assert bits_equal(t_o, t_r), first_diff(t_o, t_r)
    assert bits_equal(p_o, p_r), first_diff(p_o, p_r)
    v = np.linspace(0.0, 1.0, 4097, dtype=np.float32)[:-1]
    got = np.array([oracle.curve_strength(preset, float(x), 1.0) for x in v], dtype=np.float32)
    ref = pyrefpin.curve_evaluate(preset, v)
    assert bits_equal(got, ref), first_diff(got, ref)


def _grid_pair(oracle, nu=24, nv=8):
    g = synth.torus_grids(nu, nv, 5)
    o = oracle.OracleMesh.grids(g, 0)
    r = pyrefpin.RefGrids(g, np.zeros_like(g.co))
    assert o.num_nodes == r.num_nodes
    return g, o, r


def _assert_same_grids(o, r, what):
    co_r, no_r, m_r = r.get()
    assert bits_equal(o.co(), co_r), (what, "co", first_diff(o.co(), co_r))
    assert bits_equal(o.no(), no_r), (what, "no", first_diff(o.no(), no_r))
    assert bits_equal(o.mask(), m_r), (what, "mask", first_diff(o.mask(), m_r))


def test_grids_normals_and_stitching_match_reference(oracle):
    """Every grid normal recomputed with all seams stitched (subdiv_ccg.c
    normal update: inner quad normals, face-internal seams and centres, base
    edges and corners — positions, normals and masks averaged), bit for bit;
    the reference builds its own edge/corner adjacency from the base topology
    (subdiv_ccg.c:397-540)."""
    g, o, r = _grid_pair(oracle)
    o.recalc_all_normals()
    for n in np.nonzero(o.nodes()["flag"] & LEAF)[0]:
        r.node_mark_update(int(n))
    r.update_normals()
    _assert_same_grids(o, r, "full update")


def test_grids_stroke_replay_in_reference(oracle):
    """A mixed draw / smooth / inflate oracle stroke on multires grids with X
    symmetry; after every dab the reference's normal update (with seam
    stitching) and refit run on the oracle's brushed grids and give the same
    positions, normals, masks and boxes bit for bit."""
    g, o, r = _grid_pair(oracle)
    o.recalc_all_normals()
    for n in np.nonzero(o.nodes()["flag"] & LEAF)[0]:
        r.node_mark_update(int(n))
    r.update_normals()
    dabs = synth.torus_dabs(synth.SEED_BASE + 4, 18, 0.12)
    tools = (synth.TOOL_DRAW, synth.TOOL_SMOOTH, synth.TOOL_INFLATE)
    moved = 0
    for d in range(dabs.shape[0]):
        st = synth.Stroke(tools[d % 3], 0.12, 0.6, synth.CURVE_SMOOTH, synth.SYMM_X, dabs)
        rsq = np.float32(0.12) * np.float32(0.12)
        for p in (0, 1):
            sgn = np.array([-1 if p & 1 else 1, 1, 1], np.float32)
            loc = dabs[d, :3] * sgn
            delta = dabs[d, 3:] * sgn
            nodes = o.search_sphere(loc, rsq, 0)
            n, _ = o.brush_pass(st, loc, delta, nodes)
            moved += n
            for nd in nodes:
                r.node_mark_update(int(nd))
        r.set(o.co(), o.mask())
        o.update_normals()
        r.update_normals()
        _assert_same_grids(o, r, f"dab {d}")
        o.update_bounds(UPD_BB)
        r.update_bounds(UPD_BB)
        ovb, _ = o.bbs()
        rvb, _ = r.bbs()
        assert bits_equal(ovb, rvb), (d, first_diff(ovb, rvb))
    assert moved > 0


def _polygon_base(name):
    if name == "icosahedron":  # triangles; every base vertex joins five faces
        co, tris = synth.icosphere(0)
        return co, [list(t) for t in tris]
    return synth.pentagonal_prism()  # pentagons and quads; three faces a vertex


@pytest.mark.parametrize("base", ["icosahedron", "pentagonal_prism"])
def test_grids_polygon_base_match_reference(oracle, base):
    """Multires grids over triangles and pentagons, base vertices joining three
    or five faces (the tori elsewhere have quads and four): the full normal
    update with seam stitching, then a mixed X-mirrored stroke with the
    reference's normal update and refit after every dab, bit for bit."""
    co, polys = _polygon_base(base)
    g = synth.polygon_grids(co, polys, 4)
    # 4 grids of 9x9 a leaf: the oracle counts grids, the reference elements
    o = oracle.OracleMesh.grids(g, 4)
    r = pyrefpin.RefGrids(g, np.zeros_like(g.co), 4 * 81)
    assert o.num_nodes == r.num_nodes > 1
    o.recalc_all_normals()
    for n in np.nonzero(o.nodes()["flag"] & LEAF)[0]:
        r.node_mark_update(int(n))
    r.update_normals()
    _assert_same_grids(o, r, "full update")
    # seam elements computed from two grids' bilinear maps can differ by an
    # ulp, so the stitching moves them: a second update of every leaf and a
    # refit in both before the stroke
    for n in np.nonzero(o.nodes()["flag"] & LEAF)[0]:
        o.node_mark_update(int(n))
        r.node_mark_update(int(n))
    o.update_normals()
    r.update_normals()
    _assert_same_grids(o, r, "second update")
    o.update_bounds(UPD_BB)
    r.update_bounds(UPD_BB)
    assert bits_equal(o.bbs()[0], r.bbs()[0])
    dabs = synth.arc_dabs(synth.SEED_BASE + 11, 12, 0.25, 0.85)
    tools = (synth.TOOL_DRAW, synth.TOOL_SMOOTH, synth.TOOL_INFLATE)
    moved = 0
    for d in range(dabs.shape[0]):
        st = synth.Stroke(tools[d % 3], 0.3, 0.6, synth.CURVE_SMOOTH, synth.SYMM_X, dabs)
        rsq = np.float32(0.3) * np.float32(0.3)
        for p in (0, 1):
            sgn = np.array([-1 if p & 1 else 1, 1, 1], np.float32)
            nodes = o.search_sphere(dabs[d, :3] * sgn, rsq, 0)
            n, _ = o.brush_pass(st, dabs[d, :3] * sgn, dabs[d, 3:] * sgn, nodes)
            moved += n
            for nd in nodes:
                r.node_mark_update(int(nd))
        r.set(o.co(), o.mask())
        o.update_normals()
        r.update_normals()
        _assert_same_grids(o, r, f"dab {d}")
        o.update_bounds(UPD_BB)
        r.update_bounds(UPD_BB)
        assert bits_equal(o.bbs()[0], r.bbs()[0]), d
    assert moved > 0


def _rays(rng, n, center, radius):
    """Rays from a sphere around the mesh towards points near its middle; every
    seventh one axis-aligned (exercises the 1/0 slabs of the box test)."""
    out = []
    for k in range(n):
        s = rng.normal(size=3)
        s = (center + s / np.linalg.norm(s) * radius).astype(np.float32)
        if k % 7 == 0:
            ax = k % 3
            d = np.zeros(3, np.float32)
            d[ax] = -1.0 if s[ax] > center[ax] else 1.0
        else:
            t = center + rng.normal(size=3) * 0.3 * radius / 3.0
            d = (t - s) / np.linalg.norm(t - s)
        out.append((s, d.astype(np.float32)))
    return out


def _same_hit(a, b):
    return (a[0] == b[0] and np.float32(a[1]).view(np.uint32) == np.float32(b[1]).view(np.uint32)
            and a[2] == b[2] and a[3] == b[3] and bits_equal(a[4], b[4]))


@pytest.mark.parametrize("name", ["grid", "icosphere", "uvsphere", "ngon"])
def test_raycast_matches_reference(oracle, name):
    """BKE_pbvh_raycast (pbvh.c:3916) + BKE_pbvh_node_raycast with the spec'd
    sculpt callback: hit flag, depth, active vertex, active face and face normal
    bit for bit, over vb and orig_vb, with finite and unbounded ray lengths,
    before and after brushing."""
    m, o, r = _pair(oracle, name, 5000)
    co = o.co()
    center = (co.min(0) + co.max(0)) / 2
    radius = float(np.linalg.norm(co.max(0) - co.min(0)))
    rng = np.random.default_rng(17)
    hits = 0
    for k, (s, d) in enumerate(_rays(rng, 300, center, radius)):
        depth = np.float32(3.4028235e38) if k % 3 else np.float32(radius * 0.8)
        a = o.raycast(s, d, depth, original=k % 2)
        b = r.raycast(s, d, depth, original=k % 2)
        assert _same_hit(a[:5], b), (k, a, b)
        hits += a[0]
    assert hits > 50
    # after an edit (boxes refit, orig_vb kept) the same holds
    co2, _ = _edit(o, r, co, center.astype(np.float32), 0.3 * radius, 0.05 * radius)
    o.update_normals()
    r.update_normals()
    o.update_bounds(UPD_BB)
    r.update_bounds(UPD_BB)
    for k, (s, d) in enumerate(_rays(rng, 100, center, radius)):
        a = o.raycast(s, d, original=k % 2)
        b = r.raycast(s, d, original=k % 2)
        assert _same_hit(a[:5], b), (k, a, b)


@pytest.mark.parametrize("jitter", [0.0, 0.02])
def test_grids_raycast_matches_reference(oracle, jitter):
    """pbvh_grids_node_raycast through BKE_pbvh_raycast (pbvh.c:4110-4201):
    grid quads, the second triangle tried only when the first is not taken.
    The jittered torus has folded quads where both triangles meet the ray with
    the second closer, the case in which that order decides the result."""
    g = synth.torus_grids(16, 6, 4)
    rng = np.random.default_rng(9)
    if jitter:
        g.co = (g.co + rng.normal(size=g.co.shape) * jitter).astype(np.float32)
    o = oracle.OracleMesh.grids(g, 0)
    o.recalc_all_normals()
    r = pyrefpin.RefGrids(g, np.zeros_like(g.co))
    for n in np.nonzero(o.nodes()["flag"] & LEAF)[0]:
        r.node_mark_update(int(n))
    r.update_normals()
    r.update_bounds(UPD_BB)
    hits = special = 0
    for k in range(300):
        s = rng.normal(size=3)
        s = (2.5 * s / np.linalg.norm(s)).astype(np.float32)
        t = rng.normal(size=3) * 0.6
        d = ((t - s) / np.linalg.norm(t - s)).astype(np.float32)
        length = np.float32(3.4028235e38) if k % 3 else np.float32(2.4)
        a = o.raycast(s, d, length, original=k % 2)
        b = r.raycast(s, d, length, original=k % 2)
        assert _same_hit(a[:5], b), (k, a, b)
        hits += a[0]
        special += o.grids_special_quads(s, d) > 0
    assert hits > 100
    if jitter:
        assert special > 20


def _near_rays(rng, n, center, radius):
    """Rays from a sphere around the mesh towards points scattered up to about
    the mesh's size from its middle: many pass beside the surface, the case
    the nearest-to-ray query serves; every seventh one axis-aligned."""
    out = []
    for k in range(n):
        s = rng.normal(size=3)
        s = (center + s / np.linalg.norm(s) * radius).astype(np.float32)
        if k % 7 == 0:
            ax = k % 3
            d = np.zeros(3, np.float32)
            d[ax] = -1.0 if s[ax] > center[ax] else 1.0
        else:
            t = center + rng.normal(size=3) * 0.45 * radius
            d = (t - s) / np.linalg.norm(t - s)
        out.append((s, d.astype(np.float32)))
    return out


def _same_near(a, b):
    f = lambda x: np.float32(x).view(np.uint32)  # noqa: E731
    return a[0] == b[0] and f(a[1]) == f(b[1]) and f(a[2]) == f(b[2])


@pytest.mark.parametrize("name", ["grid", "icosphere", "uvsphere", "ngon"])
def test_nearest_to_ray_matches_reference(oracle, name):
    """BKE_pbvh_find_nearest_to_ray (pbvh.c:4339-4352) with the spec'd sculpt
    callback, pbvh_faces_node_nearest_to_ray, dist_squared_ray_to_tri_v3_fast
    and the math_geom.cc ray / segment / box distances: hit flag, depth and
    squared distance bit for bit, over vb and orig_vb, before and after an
    edit."""
    m, o, r = _pair(oracle, name, 5000)
    co = o.co()
    center = (co.min(0) + co.max(0)) / 2
    radius = float(np.linalg.norm(co.max(0) - co.min(0)))
    rng = np.random.default_rng(23)
    hits = 0
    for k, (s, d) in enumerate(_near_rays(rng, 300, center, radius)):
        a = o.nearest_to_ray(s, d, original=k % 2)
        b = r.nearest_to_ray(s, d, original=k % 2)
        assert _same_near(a, b), (k, a, b)
        hits += a[0]
    assert hits > 100
    co2, _ = _edit(o, r, co, center.astype(np.float32), 0.3 * radius, 0.05 * radius)
    o.update_normals()
    r.update_normals()
    o.update_bounds(UPD_BB)
    r.update_bounds(UPD_BB)
    for k, (s, d) in enumerate(_near_rays(rng, 100, center, radius)):
        a = o.nearest_to_ray(s, d, original=k % 2)
        b = r.nearest_to_ray(s, d, original=k % 2)
        assert _same_near(a, b), (k, a, b)


@pytest.mark.parametrize("jitter", [0.0, 0.02])
def test_grids_nearest_to_ray_matches_reference(oracle, jitter):
    """pbvh_grids_node_nearest_to_ray (pbvh.c:4402-4460): grid quads, the
    second triangle tested only when the first is taken (ray_face_nearest_quad,
    pbvh.c:3991-4017), on a smooth and a jittered torus."""
    g = synth.torus_grids(16, 6, 4)
    rng = np.random.default_rng(31)
    if jitter:
        g.co = (g.co + rng.normal(size=g.co.shape) * jitter).astype(np.float32)
    o = oracle.OracleMesh.grids(g, 0)
    o.recalc_all_normals()
    r = pyrefpin.RefGrids(g, np.zeros_like(g.co))
    for n in np.nonzero(o.nodes()["flag"] & LEAF)[0]:
        r.node_mark_update(int(n))
    r.update_normals()
    r.update_bounds(UPD_BB)
    hits = 0
    for k in range(300):
        s = rng.normal(size=3)
        s = (2.5 * s / np.linalg.norm(s)).astype(np.float32)
        t = rng.normal(size=3) * 1.2
        d = ((t - s) / np.linalg.norm(t - s)).astype(np.float32)
        a = o.nearest_to_ray(s, d, original=k % 2)
        b = r.nearest_to_ray(s, d, original=k % 2)
        assert _same_near(a, b), (k, a, b)
        hits += a[0]
    assert hits > 100
