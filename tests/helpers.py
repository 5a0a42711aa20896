"""Shared helpers of the parity tests: small seeded meshes and comparisons."""
from __future__ import annotations

import numpy as np

from dune_sculpt_gb300 import synth


def small_grid(nq=48):
    return synth.grid_mesh(nq)


def small_icosphere(level=4, seed=synth.SEED_BASE + 1, masked=True):
    co, tris = synth.icosphere(level)
    r = 1.0 + 0.01 * synth.gaussian(seed, 1, co.shape[0])
    co = co * r[:, None]
    m = synth._faces_from_polys(co, tris)
    if masked:
        nz = synth.value_noise(seed, 2, co, 2.0)
        m.mask = synth._f32(np.clip(1.5 * nz - 0.25, 0.0, 1.0))
    return m


def small_uvsphere(n=64, seed=synth.SEED_BASE + 2):
    co, corners = synth.uv_sphere(n, n)
    disp = 1.0 + 0.02 * (synth.value_noise(seed, 3, co, 2.0) - 0.5)
    return synth._faces_from_polys(co * disp[:, None], corners)


def bits_equal(a: np.ndarray, b: np.ndarray) -> bool:
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def first_diff(a: np.ndarray, b: np.ndarray) -> str:
    a = np.asarray(a).reshape(-1)
    b = np.asarray(b).reshape(-1)
    if a.shape != b.shape:
        return f"shape {a.shape} vs {b.shape}"
    d = np.nonzero(a.view(np.uint32) != b.view(np.uint32))[0]
    if d.size == 0:
        return "equal"
    i = d[0]
    return f"{d.size} differ; first at {i}: {a[i]!r} vs {b[i]!r}"


def rel_err(x: np.ndarray, ref: np.ndarray) -> float:
    """Norm-wise relative error max|x - ref| / max|ref| (positions are O(1))."""
    ref = np.asarray(ref, dtype=np.float64)
    return float(np.abs(np.asarray(x, dtype=np.float64) - ref).max() / max(np.abs(ref).max(), 1e-30))


def ngon_mesh(nq: int = 120) -> synth.FacesMesh:
    """A grid whose quads are merged in pairs into hexagons (n-gon polys,
    fan looptris), with a few triangles and quads left over at the row ends,
    and a smooth height field so the Newell normals are not all +Z."""
    n = nq + 1
    j, i = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    x = i.reshape(-1) / nq
    y = j.reshape(-1) / nq
    z = 0.05 * np.sin(6.0 * x) * np.cos(5.0 * y)
    co = synth._f32(np.stack([x, y, z], 1))
    polys = []
    for qj in range(nq):
        qi = 0
        while qi < nq:
            v00 = qj * n + qi
            if qi + 1 < nq and (qi + qj) % 5 != 4:
                polys.append([v00, v00 + 1, v00 + 2, v00 + 2 + n, v00 + 1 + n, v00 + n])
                qi += 2
            else:
                polys.append([v00, v00 + 1, v00 + 1 + n])
                polys.append([v00, v00 + 1 + n, v00 + n])
                qi += 1
    P = len(polys)
    sizes = np.array([len(p) for p in polys], dtype=np.int32)
    verts = np.zeros(n * n, dtype=synth.MVERT_DT)
    verts["co"] = co
    mp = np.zeros(P, dtype=synth.MPOLY_DT)
    mp["totloop"] = sizes
    mp["loopstart"] = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int32)
    mp["flag"] = 1
    loops = np.zeros(int(sizes.sum()), dtype=synth.MLOOP_DT)
    loops["v"] = np.concatenate(polys).astype(np.uint32)
    tris = []
    for p, ls in enumerate(mp["loopstart"]):
        for k in range(1, sizes[p] - 1):
            tris.append((ls, ls + k, ls + k + 1, p))
    lt = np.zeros(len(tris), dtype=synth.MLOOPTRI_DT)
    t = np.array(tris, dtype=np.uint32)
    lt["tri"] = t[:, :3]
    lt["poly"] = t[:, 3]
    return synth.FacesMesh(verts=verts, polys=mp, loops=loops, looptris=lt, kind="ngon")


def material_grid(nq: int = 96) -> synth.FacesMesh:
    """A flat grid whose polys carry four materials in stripes and a flat/smooth
    checker, so leaves are split by material (partition_indices_material)."""
    m = synth.grid_mesh(nq)
    p = np.arange(m.polys.shape[0])
    m.polys["mat_nr"] = ((p % nq) * 4 // nq).astype(np.int16)
    m.polys["flag"] = np.where((p // (nq * 8)) % 2 == 0, 1, 0).astype(m.polys["flag"].dtype)
    return m
