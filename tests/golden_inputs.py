"""Seeded inputs of the golden fixtures (tests/golden/reference_golden.npz).

The generator builds them here and stores every floating-point input it used
(positions, masks, rays, spheres, edited positions) next to the outputs: float64
library arithmetic (norms, sin / cos) rounds differently on different CPUs, so
the tests take the stored floats and rebuild only the integer topology here."""
from __future__ import annotations

import numpy as np

from dune_sculpt_gb300 import synth

LEAF_LIMIT = 300
CURVE_PRESETS = (0, 1, 2, 3, 5, 6)
FACES_MESHES = ("grid", "icosphere", "uvsphere")
FLT_MAX = np.float32(3.4028235e38)


def curve_points() -> np.ndarray:
    return np.linspace(0.0, 1.0, 129, dtype=np.float32)[:-1]


def faces_mesh(name: str, gold=None) -> synth.FacesMesh:
    """The mesh; with gold (the loaded fixture) its stored positions and mask."""
    m = _faces_mesh(name)
    if gold is not None:
        m.verts["co"] = gold[f"{name}_in_co"]
        if f"{name}_in_mask" in gold:
            m.mask = gold[f"{name}_in_mask"]
    return m


def _faces_mesh(name: str) -> synth.FacesMesh:
    if name == "grid":
        m = synth.grid_mesh(40)
        co = m.verts["co"].astype(np.float64)
        co[:, 2] = 0.05 * np.sin(7.0 * co[:, 0]) * np.cos(6.0 * co[:, 1])
        m.verts["co"] = synth._f32(co)
        return m
    if name == "icosphere":
        co, tris = synth.icosphere(4)
        r = 1.0 + 0.01 * synth.gaussian(synth.SEED_BASE + 21, 1, co.shape[0])
        m = synth._faces_from_polys(co * r[:, None], tris)
        nz = synth.value_noise(synth.SEED_BASE + 21, 2, co, 2.0)
        m.mask = synth._f32(np.clip(1.5 * nz - 0.25, 0.0, 1.0))
        return m
    co, corners = synth.uv_sphere(48, 32)
    disp = 1.0 + 0.02 * (synth.value_noise(synth.SEED_BASE + 22, 3, co, 2.0) - 0.5)
    return synth._faces_from_polys(co * disp[:, None], corners)


def initial_normals(m: synth.FacesMesh) -> np.ndarray:
    """Any fixed per-vertex normals (the update recomputes the tagged ones)."""
    co = m.verts["co"].astype(np.float64)
    n = co - co.mean(0)
    n /= np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-12)
    return synth._f32(n)


def _box(m):
    co = m.verts["co"]
    return co.min(0), co.max(0)


def spheres(m):
    lo, hi = _box(m)
    rng = np.random.default_rng(31)
    out = []
    for k in range(24):
        c = rng.uniform(lo - 0.1, hi + 0.1).astype(np.float32)
        rsq = np.float32(rng.uniform(0.0, 0.5 * float((hi - lo).max()))) ** 2
        out.append((c, rsq, k % 2))
    return out


def edit(m, search):
    """A smooth displacement inside a sphere: new positions, the moved
    vertices (tags) and the nodes the sphere culls (marked)."""
    co = m.verts["co"].copy()
    lo, hi = _box(m)
    c = ((lo + hi) / 2 + 0.13 * (hi - lo)).astype(np.float32)
    rad = np.float32(0.3 * float((hi - lo).max()))
    rsq = rad * rad
    d2 = ((co - c) ** 2).sum(1)
    inside = np.nonzero(d2 < rsq)[0]
    fall = (np.float32(1) - d2[inside] / rsq).astype(np.float32)
    co[inside] += (np.float32(0.04) * fall)[:, None] * np.array([0.3, -0.2, 1.0], np.float32)
    return co, inside, search(c, rsq, 0)


def rays(m):
    lo, hi = _box(m)
    center = (lo + hi) / 2
    radius = float(np.linalg.norm(hi - lo))
    rng = np.random.default_rng(37)
    out = []
    for k in range(48):
        s = rng.normal(size=3)
        s = (center + s / np.linalg.norm(s) * radius).astype(np.float32)
        if k % 6 == 0:
            d = np.zeros(3, np.float32)
            d[k % 3] = -1.0 if s[k % 3] > center[k % 3] else 1.0
        else:
            t = center + rng.normal(size=3) * 0.1 * radius
            d = ((t - s) / np.linalg.norm(t - s)).astype(np.float32)
        length = FLT_MAX if k % 4 else np.float32(0.8 * radius)
        out.append((s, d, length, k % 2))
    return out


def grids_mesh(gold=None):
    g = synth.torus_grids(12, 4, 4)
    if gold is not None:
        g.co = gold["grids_in_co"]
        g.mask = gold["grids_in_mask"]
    return g


def pack_rays(rays_list) -> np.ndarray:
    return np.array([[*s, *d, length, orig] for s, d, length, orig in rays_list], np.float32)


def unpack_rays(a):
    return [(r[0:3].copy(), r[3:6].copy(), np.float32(r[6]), int(r[7])) for r in a]


def pack_spheres(sph) -> np.ndarray:
    return np.array([[*c, rsq, orig] for c, rsq, orig in sph], np.float32)


def unpack_spheres(a):
    return [(r[0:3].copy(), np.float32(r[3]), int(r[4])) for r in a]
