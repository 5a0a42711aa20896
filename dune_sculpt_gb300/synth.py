"""Seeded synthetic meshes and strokes for the five sculpt workloads.

No public dataset exists for this path; every input is generated here from a
seed (``0x5EED0000 + workload index``).  Noise is a splitmix64 counter hash,
Gaussians use Box-Muller, and "smooth noise" is value noise with trilinear
interpolation on a seeded lattice that repeats every 8 cells.  Geometry is
computed in float64 and rounded to float32; negative zeros are canonicalised
to +0 so that bounding-box min/max stay order independent.

Mesh arrays follow the reference's element layouts
(source/dune/types/types_meshdata.h):
  MVert    16 B: float co[3]; char flag, bweight, _pad[2]       (:13-17)
  MPoly    12 B: int loopstart, totloop; short mat_nr; char flag, _pad (:50-56)
  MLoop     8 B: uint v, e                                       (:69-74)
  MLoopTri 16 B: uint tri[3] (loop indices), uint poly          (:178-181)
Quads are split into looptris (0,1,2) and (0,2,3) as the reference's
tessellation does (kernel/intern/mesh_tessellate.c:232-240).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

MVERT_DT = np.dtype([("co", "<f4", (3,)), ("flag", "i1"), ("bweight", "i1"), ("pad", "i1", (2,))])
MPOLY_DT = np.dtype([("loopstart", "<i4"), ("totloop", "<i4"), ("mat_nr", "<i2"),
                     ("flag", "i1"), ("pad", "i1")])
MLOOP_DT = np.dtype([("v", "<u4"), ("e", "<u4")])
MLOOPTRI_DT = np.dtype([("tri", "<u4", (3,)), ("poly", "<u4")])

SEED_BASE = 0x5EED0000
_M64 = (1 << 64) - 1


def splitmix64(x: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser on a uint64 counter array."""
    x = np.asarray(x, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = x + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def hash_u01(seed: int, stream: int, idx) -> np.ndarray:
    """Uniform [0,1) doubles from (seed, stream, counter)."""
    idx = np.asarray(idx, dtype=np.uint64)
    with np.errstate(over="ignore"):
        key = splitmix64(np.uint64(seed & _M64) ^ np.uint64((stream * 0x632BE59BD9B4E019) & _M64))
        h = splitmix64(idx ^ key)
    return (h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def gaussian(seed: int, stream: int, n: int) -> np.ndarray:
    """Box-Muller standard normals."""
    i = np.arange(n, dtype=np.uint64)
    u1 = hash_u01(seed, stream, 2 * i)
    u2 = hash_u01(seed, stream, 2 * i + 1)
    u1 = np.maximum(u1, 1e-300)
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


def value_noise(seed: int, stream: int, p: np.ndarray, freq: float) -> np.ndarray:
    """Trilinear value noise in [0,1) on a lattice of period 8 cells."""
    q = np.asarray(p, dtype=np.float64) * freq
    i0 = np.floor(q)
    f = q - i0
    i0 = i0.astype(np.int64)
    table = hash_u01(seed, stream, np.arange(512, dtype=np.uint64))  # the 8^3 lattice values
    # per axis: lattice index mod 8 (x & 7 == x % 8 for two's-complement
    # integers) and weight of the lower and upper corner
    ii = [[(np.ascontiguousarray(i0[:, a]) + d) & 7 for d in (0, 1)] for a in range(3)]
    ww = [[1.0 - np.ascontiguousarray(f[:, a]), np.ascontiguousarray(f[:, a])] for a in range(3)]
    out = np.zeros(q.shape[0], dtype=np.float64)
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                lat = table[ii[0][dx] * 64 + ii[1][dy] * 8 + ii[2][dz]]
                w = ww[0][dx] * ww[1][dy] * ww[2][dz]
                out += w * lat
    return out


def _f32(a: np.ndarray) -> np.ndarray:
    a = np.asarray(a, dtype=np.float32)
    return a + np.float32(0.0)  # -0.0 + 0.0 == +0.0


@dataclass
class FacesMesh:
    """A PBVH_FACES input mesh in the reference's element layouts."""
    verts: np.ndarray
    polys: np.ndarray
    loops: np.ndarray
    looptris: np.ndarray
    mask: np.ndarray | None = None
    name: str = ""
    kind: str = ""

    @property
    def totvert(self) -> int:
        return int(self.verts.shape[0])


def _faces_from_polys(co: np.ndarray, poly_corners: np.ndarray) -> FacesMesh:
    """co: (V,3) float64; poly_corners: (P,k) int vertex indices, k = 3 or 4."""
    V = co.shape[0]
    P, k = poly_corners.shape
    verts = np.zeros(V, dtype=MVERT_DT)
    verts["co"] = _f32(co)
    polys = np.zeros(P, dtype=MPOLY_DT)
    polys["loopstart"] = np.arange(P, dtype=np.int32) * k
    polys["totloop"] = k
    polys["flag"] = 1  # ME_SMOOTH
    loops = np.zeros(P * k, dtype=MLOOP_DT)
    loops["v"] = poly_corners.reshape(-1).astype(np.uint32)
    ls = np.arange(P, dtype=np.uint32) * k
    if k == 3:
        lt = np.zeros(P, dtype=MLOOPTRI_DT)
        lt["tri"] = np.stack([ls, ls + 1, ls + 2], axis=1)
        lt["poly"] = np.arange(P, dtype=np.uint32)
    else:
        lt = np.zeros(2 * P, dtype=MLOOPTRI_DT)
        tri = np.empty((P, 2, 3), dtype=np.uint32)
        tri[:, 0] = np.stack([ls, ls + 1, ls + 2], axis=1)
        tri[:, 1] = np.stack([ls, ls + 2, ls + 3], axis=1)
        lt["tri"] = tri.reshape(-1, 3)
        lt["poly"] = np.repeat(np.arange(P, dtype=np.uint32), 2)
    return FacesMesh(verts=verts, polys=polys, loops=loops, looptris=lt)


def grid_mesh(nq: int) -> FacesMesh:
    """(nq+1)^2 vertices on [0,1]^2 at z=0, nq^2 quads facing +Z."""
    n = nq + 1
    j, i = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    co = np.stack([i.reshape(-1) / nq, j.reshape(-1) / nq, np.zeros(n * n)], axis=1)
    qj, qi = np.meshgrid(np.arange(nq), np.arange(nq), indexing="ij")
    v00 = (qj * n + qi).reshape(-1)
    corners = np.stack([v00, v00 + 1, v00 + 1 + n, v00 + n], axis=1)
    m = _faces_from_polys(co, corners)
    m.kind = "grid"
    return m


def icosphere(level: int) -> tuple[np.ndarray, np.ndarray]:
    """Unit icosphere by midpoint subdivision; returns (co float64, tris int64)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    co = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
                   [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]],
                  dtype=np.float64)
    co /= np.linalg.norm(co, axis=1, keepdims=True)
    tris = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9],
                     [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2],
                     [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10],
                     [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    for _ in range(level):
        V = co.shape[0]
        e = np.concatenate([tris[:, [0, 1]], tris[:, [1, 2]], tris[:, [2, 0]]], axis=0)
        key = np.minimum(e[:, 0], e[:, 1]) * V + np.maximum(e[:, 0], e[:, 1])
        uk, inv = np.unique(key, return_inverse=True)
        a = uk // V
        b = uk % V
        mid = co[a] + co[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        T = tris.shape[0]
        mids = (inv + V).reshape(3, T)
        m01, m12, m20 = mids[0], mids[1], mids[2]
        v0, v1, v2 = tris[:, 0], tris[:, 1], tris[:, 2]
        tris = np.stack([np.stack([v0, m01, m20], 1), np.stack([v1, m12, m01], 1),
                         np.stack([v2, m20, m12], 1), np.stack([m01, m12, m20], 1)],
                        axis=1).reshape(-1, 3)
        co = np.concatenate([co, mid], axis=0)
    return co, tris


def uv_sphere(n_lon: int, n_lat: int) -> tuple[np.ndarray, np.ndarray]:
    """Grid-mapped unit sphere: n_lat rings (poles left open) x n_lon columns of quads,
    n_lon*n_lat vertices, outward-facing quads."""
    jj, ii = np.meshgrid(np.arange(n_lat), np.arange(n_lon), indexing="ij")
    theta = np.pi * (jj.reshape(-1) + 0.5) / n_lat
    phi = 2.0 * np.pi * ii.reshape(-1) / n_lon
    co = np.stack([np.sin(theta) * np.cos(phi), np.sin(theta) * np.sin(phi), np.cos(theta)], 1)
    qj, qi = np.meshgrid(np.arange(n_lat - 1), np.arange(n_lon), indexing="ij")
    a = qj * n_lon + qi
    b = qj * n_lon + (qi + 1) % n_lon
    c = (qj + 1) * n_lon + (qi + 1) % n_lon
    d = (qj + 1) * n_lon + qi
    corners = np.stack([a.reshape(-1), d.reshape(-1), c.reshape(-1), b.reshape(-1)], 1)
    return co, corners


@dataclass
class Stroke:
    """A brush and its dab sequence (location xyz, grab delta xyz per dab)."""
    tool: int
    radius: float
    strength: float
    curve_preset: int
    symmetry: int
    dabs: np.ndarray  # (n, 6) float32
    normal_radius_factor: float = 0.5
    area_radius_factor: float = 0.5
    plane_offset: float = 0.0
    flag: int = 0
    view_normal: tuple = (0.0, 0.0, 1.0)
    use_original_bb: int = 0
    crease_pinch_factor: float = 0.5  # types_brush_defaults.h:23
    elastic_deform_type: int = 0      # BRUSH_ELASTIC_DEFORM_GRAB
    elastic_deform_volume_preservation: float = 0.4
    height: float = 0.5  # Brush.height (layer)


TOOL_DRAW, TOOL_SMOOTH, TOOL_INFLATE, TOOL_CLAY_STRIPS = 1, 2, 4, 18
TOOL_PINCH, TOOL_CREASE = 3, 16
TOOL_GRAB, TOOL_ELASTIC_DEFORM, TOOL_LAYER = 5, 21, 6
CURVE_SHARP, CURVE_SMOOTH = 1, 2
SYMM_X = 1


def _dabs_from_points(pts: np.ndarray) -> np.ndarray:
    pts = np.asarray(pts, dtype=np.float64)
    delta = np.zeros_like(pts)
    if len(pts) > 1:
        delta[1:] = pts[1:] - pts[:-1]
        delta[0] = pts[1] - pts[0]
    return _f32(np.concatenate([pts, delta], axis=1))


def line_dabs(seed: int, n: int, lo: float = 0.1, hi: float = 0.9) -> np.ndarray:
    u = hash_u01(seed, 7, np.arange(4))
    p0 = lo + (hi - lo) * u[:2]
    p1 = lo + (hi - lo) * u[2:]
    t = np.linspace(0.0, 1.0, n)[:, None]
    pts = np.concatenate([p0 + (p1 - p0) * t, np.zeros((n, 1))], axis=1)
    return _dabs_from_points(pts)


def arc_dabs(seed: int, n: int, step: float, surf_radius: float = 1.0) -> np.ndarray:
    g = gaussian(seed, 9, 6)
    axis = g[:3] / np.linalg.norm(g[:3])
    p0 = np.cross(axis, g[3:])
    p0 /= np.linalg.norm(p0)
    q = np.cross(axis, p0)
    ang = step * np.arange(n)[:, None]
    pts = (np.cos(ang) * p0 + np.sin(ang) * q) * surf_radius
    return _dabs_from_points(pts)


def grab_dabs(seed: int, n: int, step: float, surf_radius: float = 1.0) -> np.ndarray:
    """A grab stroke: the location stays at the anchor on a sphere of
    surf_radius, the grab delta grows by step per dab along a seeded
    direction (the reference's grab keeps the stroke's first location and
    accumulates the delta)."""
    g = gaussian(seed, 10, 6)
    p = g[:3] / np.linalg.norm(g[:3]) * surf_radius
    d = g[3:] / np.linalg.norm(g[3:])
    out = np.zeros((n, 6), dtype=np.float64)
    out[:, :3] = p
    out[:, 3:] = d[None, :] * (step * (np.arange(n)[:, None] + 1))
    return _f32(out)


# ---------------------------------------------------------------------------
# The five workloads


def cfg1_grid_draw(nq: int = 512, ndabs: int = 64) -> tuple[FacesMesh, Stroke, int]:
    """Draw brush on a flat grid of nq x nq quads; 64 dabs along a seeded line."""
    seed = SEED_BASE + 0
    m = grid_mesh(nq)
    m.name = f"grid{nq + 1}x{nq + 1}_draw"
    st = Stroke(TOOL_DRAW, 0.05, 0.5, CURVE_SMOOTH, 0, line_dabs(seed, ndabs))
    return m, st, 5000


def cfg2_icosphere_smooth(level: int = 8, ndabs: int = 128) -> tuple[FacesMesh, Stroke, int]:
    """Masked, X-mirrored smooth brush on a noisy icosphere."""
    seed = SEED_BASE + 1
    co, tris = icosphere(level)
    r = 1.0 + 0.01 * gaussian(seed, 1, co.shape[0])
    co = co * r[:, None]
    m = _faces_from_polys(co, tris)
    m.kind = "icosphere"
    m.name = f"icosphere{level}_smooth"
    nz = value_noise(seed, 2, co, 2.0)
    m.mask = _f32(np.clip(1.5 * nz - 0.25, 0.0, 1.0))
    radius = 0.08
    st = Stroke(TOOL_SMOOTH, radius, 0.7, CURVE_SMOOTH, SYMM_X,
                arc_dabs(seed, ndabs, 0.1 * 2 * radius))
    return m, st, 5000


def cfg3_sphere_clay(n: int = 2048, ndabs: int = 256) -> tuple[FacesMesh, Stroke, int]:
    """Clay strips on a displaced n x n grid-mapped sphere, X symmetry."""
    seed = SEED_BASE + 2
    co, corners = uv_sphere(n, n)
    disp = 1.0 + 0.02 * (value_noise(seed, 3, co, 2.0) - 0.5)
    co = co * disp[:, None]
    m = _faces_from_polys(co, corners)
    m.kind = "uvsphere"
    m.name = f"uvsphere{n}x{n}_clay"
    radius = 0.06
    st = Stroke(TOOL_CLAY_STRIPS, radius, 0.8, CURVE_SHARP, SYMM_X,
                arc_dabs(seed, ndabs, 0.1 * 2 * radius))
    return m, st, 5000


def cfg4_batch(nmesh: int = 64, vmin: float = 1e4, vmax: float = 5e5, ndabs: int = 32,
               ) -> list[tuple[FacesMesh, Stroke, int]]:
    """Uneven batch: alternating grid / sphere meshes, log-uniform sizes, own strokes."""
    seed = SEED_BASE + 3
    u = hash_u01(seed, 11, np.arange(4 * nmesh)).reshape(nmesh, 4)
    out = []
    for k in range(nmesh):
        V = math.exp(math.log(vmin) + (math.log(vmax) - math.log(vmin)) * u[k, 0])
        side = max(8, int(round(math.sqrt(V))))
        radius = 0.03 + 0.07 * u[k, 1]
        strength = 0.2 + 0.8 * u[k, 2]
        tool = TOOL_DRAW if u[k, 3] < 0.5 else TOOL_INFLATE
        if k % 2 == 0:
            m = grid_mesh(side - 1)
            dabs = line_dabs(seed + 1000 + k, ndabs)
        else:
            co, corners = uv_sphere(side, side)
            m = _faces_from_polys(co, corners)
            m.kind = "uvsphere"
            dabs = arc_dabs(seed + 1000 + k, ndabs, 0.2 * radius)
        m.name = f"batch{k}"
        out.append((m, Stroke(tool, radius, strength, CURVE_SMOOTH, 0, dabs), 5000))
    return out


# ---------------------------------------------------------------------------
# PBVH_GRIDS (multires) torus


@dataclass
class GridsMesh:
    """Multires grids in the CCG layout: per element co[3] | mask | no[3] (28 B),
    stored here as separate arrays; base topology for the seam adjacency."""
    grid_size: int
    co: np.ndarray          # (num_grids*gs*gs, 3) float32
    mask: np.ndarray        # (num_grids*gs*gs,) float32
    face_start: np.ndarray  # (F,) int32
    face_ngrids: np.ndarray
    face_verts: np.ndarray  # (4F,) int32, per corner
    face_edges: np.ndarray  # (4F,) int32, edge from corner c to c+1
    edge_verts: np.ndarray  # (E, 2) int32
    num_base_verts: int
    name: str = ""

    @property
    def num_grids(self) -> int:
        return int(self.face_ngrids.sum())

    @property
    def num_faces(self) -> int:
        return int(self.face_start.shape[0])


def torus_grids(nu: int, nv: int, level: int = 5, seed: int = SEED_BASE + 4,
                R: float = 1.0, r: float = 0.35, amp: float = 0.01) -> GridsMesh:
    gs = (1 << (level - 1)) + 1
    L = 2 * (gs - 1)
    F = nu * nv
    fj, fi = np.meshgrid(np.arange(nv), np.arange(nu), indexing="ij")
    fi = fi.reshape(-1)
    fj = fj.reshape(-1)
    vid = lambda i, j: (j % nv) * nu + (i % nu)  # noqa: E731
    c0, c1, c2, c3 = vid(fi, fj), vid(fi + 1, fj), vid(fi + 1, fj + 1), vid(fi, fj + 1)
    face_verts = np.stack([c0, c1, c2, c3], 1).reshape(-1).astype(np.int32)
    h = lambda i, j: (j % nv) * nu + (i % nu)  # noqa: E731  horizontal edge (i,j)-(i+1,j)
    v = lambda i, j: nu * nv + (j % nv) * nu + (i % nu)  # noqa: E731 vertical (i,j)-(i,j+1)
    face_edges = np.stack([h(fi, fj), v(fi + 1, fj), h(fi, fj + 1), v(fi, fj)], 1)
    face_edges = face_edges.reshape(-1).astype(np.int32)
    ej, ei = np.meshgrid(np.arange(nv), np.arange(nu), indexing="ij")
    ei = ei.reshape(-1)
    ej = ej.reshape(-1)
    edge_verts = np.concatenate([np.stack([vid(ei, ej), vid(ei + 1, ej)], 1),
                                 np.stack([vid(ei, ej), vid(ei, ej + 1)], 1)], 0).astype(np.int32)
    # element lattice coordinates inside the face, per corner grid
    yy, xx = np.meshgrid(np.arange(gs), np.arange(gs), indexing="ij")
    xx = xx.reshape(-1)
    yy = yy.reshape(-1)
    half = L // 2
    px = np.stack([half - yy, half + xx, half + yy, half - xx], 0)  # (4, gs*gs)
    py = np.stack([half - xx, half - yy, half + xx, half + yy], 0)
    U = (fi[:, None, None] * L + px[None]) % (nu * L)
    Vv = (fj[:, None, None] * L + py[None]) % (nv * L)
    u = 2.0 * np.pi * U.reshape(-1) / (nu * L)
    w = 2.0 * np.pi * Vv.reshape(-1) / (nv * L)
    ring = R + r * np.cos(w)
    pos = np.stack([ring * np.cos(u), ring * np.sin(u), r * np.sin(w)], 1)
    nrm = np.stack([np.cos(w) * np.cos(u), np.cos(w) * np.sin(u), np.sin(w)], 1)
    disp = amp * (value_noise(seed, 5, pos, 3.0) - 0.5)
    pos = pos + nrm * disp[:, None]
    mask = np.clip(1.5 * value_noise(seed, 6, pos, 2.0) - 0.25, 0.0, 1.0)
    return GridsMesh(grid_size=gs, co=_f32(pos), mask=_f32(mask),
                     face_start=(np.arange(F, dtype=np.int32) * 4),
                     face_ngrids=np.full(F, 4, dtype=np.int32), face_verts=face_verts,
                     face_edges=face_edges, edge_verts=edge_verts, num_base_verts=nu * nv,
                     name=f"torus{nu}x{nv}_L{level}")


def polygon_grids(co: np.ndarray, polys: list, level: int = 4, seed: int = SEED_BASE + 11,
                  amp: float = 0.01) -> GridsMesh:
    """Multires grids over any closed polygon base mesh: one grid per face
    corner, element (0, 0) at the face centre, (gs-1, 0) at the midpoint of
    the edge from this corner to the next, (0, gs-1) at the midpoint of the
    edge from the previous corner, (gs-1, gs-1) at the corner (the layout of
    torus_grids); positions bilinear over that quad, displaced along the
    radial direction by seeded noise, with a seeded noise mask."""
    co = np.asarray(co, dtype=np.float64)
    gs = (1 << (level - 1)) + 1
    edges: dict = {}
    face_start, face_ngrids, face_verts, face_edges = [], [], [], []
    pos = []
    t = np.arange(gs, dtype=np.float64) / (gs - 1)
    uu, ww = np.meshgrid(t, t, indexing="xy")  # [y, x]: u along x, w along y
    uu = uu.reshape(-1, 1)
    ww = ww.reshape(-1, 1)
    g = 0
    for poly in polys:
        n = len(poly)
        face_start.append(g)
        face_ngrids.append(n)
        centre = co[list(poly)].mean(axis=0)
        for c in range(n):
            a_, b_ = int(poly[c]), int(poly[(c + 1) % n])
            key = (min(a_, b_), max(a_, b_))
            if key not in edges:
                edges[key] = len(edges)
            face_verts.append(a_)
            face_edges.append(edges[key])
            m_next = 0.5 * (co[a_] + co[b_])
            m_prev = 0.5 * (co[int(poly[c - 1])] + co[a_])
            pos.append((1 - uu) * (1 - ww) * centre + uu * (1 - ww) * m_next + uu * ww * co[a_]
                       + (1 - uu) * ww * m_prev)
            g += 1
    pos = np.concatenate(pos, axis=0)
    radial = pos / np.linalg.norm(pos, axis=1, keepdims=True)
    pos = pos + radial * (amp * (value_noise(seed, 5, pos, 3.0) - 0.5))[:, None]
    mask = np.clip(1.5 * value_noise(seed, 6, pos, 2.0) - 0.25, 0.0, 1.0)
    edge_verts = np.zeros((len(edges), 2), dtype=np.int32)
    for (a_, b_), e in edges.items():
        edge_verts[e] = (a_, b_)
    return GridsMesh(grid_size=gs, co=_f32(pos), mask=_f32(mask),
                     face_start=np.asarray(face_start, dtype=np.int32),
                     face_ngrids=np.asarray(face_ngrids, dtype=np.int32),
                     face_verts=np.asarray(face_verts, dtype=np.int32),
                     face_edges=np.asarray(face_edges, dtype=np.int32), edge_verts=edge_verts,
                     num_base_verts=int(co.shape[0]), name=f"polygons{len(polys)}_L{level}")


def pentagonal_prism() -> tuple[np.ndarray, list]:
    """Closed prism over a regular pentagon: 2 pentagons and 5 quads, every
    vertex joining three faces."""
    ang = 2.0 * np.pi * np.arange(5) / 5.0
    ring = np.stack([np.cos(ang), np.sin(ang)], 1)
    co = np.concatenate([np.concatenate([ring, np.full((5, 1), -0.6)], 1),
                         np.concatenate([ring, np.full((5, 1), 0.6)], 1)], 0)
    polys = [[4, 3, 2, 1, 0], [5, 6, 7, 8, 9]]
    polys += [[i, (i + 1) % 5, 5 + (i + 1) % 5, 5 + i] for i in range(5)]
    return co, polys


def torus_dabs(seed: int, n: int, radius: float, R: float = 1.0, r: float = 0.35) -> np.ndarray:
    u0 = hash_u01(seed, 13, np.arange(2))
    w0 = 2.0 * np.pi * u0[1]
    ring = R + r * math.cos(w0)
    u = 2.0 * np.pi * u0[0] + (0.2 * radius / ring) * np.arange(n)
    pts = np.stack([ring * np.cos(u), ring * np.sin(u), np.full(n, r * math.sin(w0))], 1)
    return _dabs_from_points(pts)


def cfg5_multires(nu: int = 250, nv: int = 50, level: int = 5, ndabs: int = 256):
    """Mixed draw / smooth / inflate stroke on a multires torus (50,000 grids of 17x17)."""
    seed = SEED_BASE + 4
    g = torus_grids(nu, nv, level, seed)
    dabs = torus_dabs(seed, ndabs, 0.04)
    return g, dabs
