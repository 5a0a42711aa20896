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
