"""Generates tests/golden/reference_golden.npz from the reference's own code.

Run where the reference tree is present (it builds oracle/_ref/librefpin.so,
the reference's pbvh.c, subdiv_ccg.c, colortools.c and math code compiled from
that tree by oracle/refpin/Makefile):

    python tests/golden/make_golden.py

Every input is a seeded synthetic mesh or query from dune_sculpt_gb300.synth,
so the tests regenerate the inputs anywhere and compare with the outputs
stored here.  Small outputs are stored whole; large float arrays as SHA-256
digests of their bytes.
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)

import golden_inputs as gi  # noqa: E402


def digest(a: np.ndarray) -> np.ndarray:
    h = hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest()
    return np.frombuffer(h, dtype=np.uint8).copy()


def main():
    import pyrefpin

    out = {}
    # falloff curves: table, params, values
    for preset in gi.CURVE_PRESETS:
        t, p = pyrefpin.curve_table(preset)
        out[f"curve{preset}_table"] = t
        out[f"curve{preset}_params"] = p
        out[f"curve{preset}_eval"] = pyrefpin.curve_evaluate(preset, gi.curve_points())
    # FACES meshes: build, search, one edit's update, ray cast
    for name in gi.FACES_MESHES:
        m = gi.faces_mesh(name)
        out[f"{name}_in_co"] = m.verts["co"].copy()
        if m.mask is not None:
            out[f"{name}_in_mask"] = m.mask.copy()
        out[f"{name}_in_spheres"] = gi.pack_spheres(gi.spheres(m))
        out[f"{name}_in_rays"] = gi.pack_rays(gi.rays(m))
        no0 = gi.initial_normals(m)
        r = pyrefpin.RefPBVH.faces(m, no0, gi.LEAF_LIMIT)
        nd = r.nodes()
        for k in ("children_offset", "prim_off", "totprim", "uniq", "face_verts"):
            out[f"{name}_{k}"] = nd[k]
        out[f"{name}_leaf"] = (nd["flag"] & 1).astype(np.int32)
        out[f"{name}_prims"] = r.prim_indices()
        out[f"{name}_verts"] = np.concatenate(
            [r.node_vert_indices(int(n)) for n in np.nonzero(nd["flag"] & 1)[0]])
        vb, ovb = r.bbs()
        out[f"{name}_vb"] = vb
        lists = []
        for c, rsq, orig in gi.unpack_spheres(out[f"{name}_in_spheres"]):
            lists.append(np.concatenate([[len(x := r.search_sphere(c, rsq, orig))], x]))
        out[f"{name}_search"] = np.concatenate(lists).astype(np.int32)
        hits = []
        for s, d, length, orig in gi.unpack_rays(out[f"{name}_in_rays"]):
            h, dep, av, af, fn = r.raycast(s, d, length, orig)
            hits.append([float(h), dep, float(av), float(af), fn[0], fn[1], fn[2]])
        out[f"{name}_rays"] = np.asarray(hits, dtype=np.float32)
        co2, tags, nodes = gi.edit(m, r.search_sphere)
        out[f"{name}_in_edit_co"] = co2
        out[f"{name}_in_edit_tags"] = tags.astype(np.int32)
        r.set_co(co2)
        for n in nodes:
            r.node_mark_update(int(n))
        for v in tags:
            r.vert_mark_update(int(v))
        r.update_normals()
        r.update_bounds(4)
        out[f"{name}_edit_no"] = r.no()
        out[f"{name}_edit_vb"] = r.bbs()[0]
        r.close()
    # GRIDS: full normal update with seam stitching, then an edit's update
    g = gi.grids_mesh()
    out["grids_in_co"] = g.co.copy()
    out["grids_in_mask"] = g.mask.copy()
    rg = pyrefpin.RefGrids(g, np.zeros_like(g.co))
    for n in range(rg.num_nodes):
        rg.node_mark_update(n)  # non-leaf marks are ignored by the update
    rg.update_normals()
    co, no, mask = rg.get()
    out["grids_co_sha"] = digest(co)
    out["grids_no_sha"] = digest(no)
    out["grids_mask_sha"] = digest(mask)
    out["grids_vb"] = rg.bbs()[0]
    np.savez_compressed(os.path.join(HERE, "reference_golden.npz"), **out)
    total = sum(v.nbytes for v in out.values())
    print(f"{len(out)} arrays, {total} bytes uncompressed")


if __name__ == "__main__":
    main()
