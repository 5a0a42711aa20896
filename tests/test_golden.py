"""The oracle and the GPU path against golden outputs of the reference's own
compiled code (tests/golden/reference_golden.npz, made by
tests/golden/make_golden.py from the reference tree).  These run without the
reference tree, so they pin parity wherever the tests run.

Bit for bit: falloff tables and values, PBVH node tables, prim order, leaf
vertex lists, node boxes, search lists, boxes after an edit, ray-cast results,
multires positions / normals / masks after a full normal update with seam
stitching (as SHA-256 digests).  Within 1e-6: FACES vertex normals after an
edit (the reference adds face normals with float atomics in task order, the
oracle and GPU in looptri order with compensated sums).
"""
import hashlib
import os

import numpy as np
import pytest

import golden_inputs as gi
from helpers import bits_equal, first_diff

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_golden.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def digest(a):
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest(), np.uint8)


def _search_lists(flat):
    out, i = [], 0
    while i < flat.shape[0]:
        n = int(flat[i])
        out.append(flat[i + 1:i + 1 + n])
        i += 1 + n
    return out


def _ray_row(h, dep, av, af, fn):
    return np.array([float(h), dep, float(av), float(af), fn[0], fn[1], fn[2]], np.float32)


# ---------------------------------------------------------------- oracle (CPU)

@pytest.mark.parametrize("preset", gi.CURVE_PRESETS)
def test_oracle_curves_match_golden(oracle, gold, preset):
    t, p = oracle.curve_table(preset)
    assert bits_equal(t, gold[f"curve{preset}_table"])
    assert bits_equal(p, gold[f"curve{preset}_params"])
    v = np.array([oracle.curve_strength(preset, float(x), 1.0) for x in gi.curve_points()],
                 np.float32)
    assert bits_equal(v, gold[f"curve{preset}_eval"]), first_diff(v, gold[f"curve{preset}_eval"])


@pytest.mark.parametrize("name", gi.FACES_MESHES)
def test_oracle_faces_match_golden(oracle, gold, name):
    m = gi.faces_mesh(name, gold)
    o = oracle.OracleMesh.faces(m, gi.LEAF_LIMIT)
    nd = o.nodes()
    for k in ("children_offset", "prim_off", "totprim", "uniq", "face_verts"):
        assert np.array_equal(nd[k], gold[f"{name}_{k}"]), k
    assert np.array_equal(nd["flag"] & 1, gold[f"{name}_leaf"])
    assert np.array_equal(o.prim_indices(), gold[f"{name}_prims"])
    vi = o.vert_indices()
    leaves = np.nonzero(nd["flag"] & 1)[0]
    mine = np.concatenate([vi[nd["vert_off"][n]:nd["vert_off"][n] + nd["uniq"][n] + nd["face_verts"][n]]
                           for n in leaves])
    assert np.array_equal(mine, gold[f"{name}_verts"])
    assert bits_equal(o.bbs()[0], gold[f"{name}_vb"])
    spheres = gi.unpack_spheres(gold[f"{name}_in_spheres"])
    for (c, rsq, orig), ref in zip(spheres, _search_lists(gold[f"{name}_search"])):
        assert np.array_equal(o.search_sphere(c, rsq, orig), ref)
    rays = gi.unpack_rays(gold[f"{name}_in_rays"])
    rows = [_ray_row(*o.raycast(s, d, length, orig)[:5]) for s, d, length, orig in rays]
    assert bits_equal(np.asarray(rows), gold[f"{name}_rays"])
    _, _, nodes = gi.edit(m, lambda c, rsq, orig: o.search_sphere(c, rsq, orig))
    co2, tags = gold[f"{name}_in_edit_co"], gold[f"{name}_in_edit_tags"]
    o.set_co(co2)
    for n in nodes:
        o.node_mark_update(int(n))
    for v in tags:
        o.vert_mark_update(int(v))
    o.update_normals()
    o.update_bounds(4)
    err = np.abs(o.no()[tags] - gold[f"{name}_edit_no"][tags]).max()
    assert err <= 1e-6, err
    assert bits_equal(o.bbs()[0], gold[f"{name}_edit_vb"])


def test_oracle_grids_match_golden(oracle, gold):
    g = gi.grids_mesh(gold)
    o = oracle.OracleMesh.grids(g, 0)
    o.recalc_all_normals()
    assert np.array_equal(digest(o.co()), gold["grids_co_sha"])
    assert np.array_equal(digest(o.no()), gold["grids_no_sha"])
    assert np.array_equal(digest(o.mask()), gold["grids_mask_sha"])
    assert bits_equal(o.bbs()[0], gold["grids_vb"])


# ---------------------------------------------------------------- GPU

@pytest.mark.gpu
@pytest.mark.parametrize("preset", gi.CURVE_PRESETS)
def test_gpu_curves_match_golden(gpu, gold, preset):
    t, p = gpu.curve_table(preset)
    assert bits_equal(t, gold[f"curve{preset}_table"])
    assert bits_equal(p, gold[f"curve{preset}_params"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", gi.FACES_MESHES)
def test_gpu_faces_match_golden(gpu, gold, name):
    m = gi.faces_mesh(name, gold)
    g = gpu.PBVH.build_mesh(m, gi.LEAF_LIMIT)
    nd = g.nodes()
    for k in ("children_offset", "prim_off", "totprim", "uniq", "face_verts"):
        assert np.array_equal(nd[k], gold[f"{name}_{k}"]), k
    assert np.array_equal(g.prim_indices(), gold[f"{name}_prims"])
    vi = g.vert_indices()
    leaves = np.nonzero(nd["flag"] & 1)[0]
    mine = np.concatenate([vi[nd["vert_off"][n]:nd["vert_off"][n] + nd["uniq"][n] + nd["face_verts"][n]]
                           for n in leaves])
    assert np.array_equal(mine, gold[f"{name}_verts"])
    assert bits_equal(g.bbs()[0], gold[f"{name}_vb"])
    spheres = gi.unpack_spheres(gold[f"{name}_in_spheres"])
    for (c, rsq, orig), ref in zip(spheres, _search_lists(gold[f"{name}_search"])):
        assert np.array_equal(g.search_gather_sphere(c, rsq, orig), ref)
    rays = gi.unpack_rays(gold[f"{name}_in_rays"])
    starts = np.array([r[0] for r in rays])
    dirs = np.array([r[1] for r in rays])
    lengths = np.array([r[2] for r in rays], np.float32)
    for orig in (0, 1):
        sel = [k for k, r in enumerate(rays) if r[3] == orig]
        hit, dep, av, af, fn = g.raycast(starts[sel], dirs[sel], lengths[sel], orig)
        rows = np.array([_ray_row(hit[i], dep[i], av[i], af[i], fn[i]) for i in range(len(sel))])
        assert bits_equal(rows, gold[f"{name}_rays"][sel]), orig
    g.free()


@pytest.mark.gpu
def test_gpu_grids_match_golden(gpu, gold):
    g = gi.grids_mesh(gold)
    gp = gpu.PBVH.build_grids(g)
    assert np.array_equal(digest(gp.positions()), gold["grids_co_sha"])
    assert np.array_equal(digest(gp.normals()), gold["grids_no_sha"])
    assert np.array_equal(digest(gp.mask()), gold["grids_mask_sha"])
    assert bits_equal(gp.bbs()[0], gold["grids_vb"])
