"""Seeded synthetic control cages for the evaluation workloads.

Every cage is returned as a :class:`Cage`: float32 positions, the face list in the
``Far::TopologyDescriptor`` layout (``numVertsPerFace`` + flat ``vertIndicesPerFace``,
far/topologyDescriptor.h:49-85), optional crease edges with sharpness, and the subdivision
scheme (0 bilinear, 1 Catmull-Clark, 2 Loop -- ``Sdc::SchemeType``, sdc/types.h:37-40).

All cages here are closed 2-manifolds unless stated; ``grid`` is the one open surface and is
used to exercise boundary patches.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

BILINEAR, CATMARK, LOOP = 0, 1, 2


@dataclass
class Cage:
    positions: np.ndarray                # float32 [nverts, 3]
    verts_per_face: np.ndarray           # int32 [nfaces]
    face_verts: np.ndarray               # int32 [sum(verts_per_face)]
    scheme: int = CATMARK
    crease_verts: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.int32))
    crease_sharpness: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    name: str = ""

    @property
    def num_vertices(self) -> int:
        return int(self.positions.shape[0])

    @property
    def num_faces(self) -> int:
        return int(self.verts_per_face.shape[0])

    def bbox_diagonal(self) -> float:
        p = self.positions.astype(np.float64)
        return float(np.linalg.norm(p.max(0) - p.min(0)))

    def ptex_face_offsets(self) -> np.ndarray:
        """First ptex face of every coarse face; regular faces own one ptex face and irregular
        faces one per corner (far/ptexIndices.cpp:47-63).  Entry nfaces is the total."""
        reg = 3 if self.scheme == LOOP else 4
        per = np.where(self.verts_per_face == reg, 1, self.verts_per_face)
        out = np.zeros(self.num_faces + 1, np.int32)
        np.cumsum(per, out=out[1:])
        return out


def _edges_of(verts_per_face: np.ndarray, face_verts: np.ndarray) -> np.ndarray:
    """Unique undirected edges (sorted pairs) in first-seen order."""
    starts = np.zeros(len(verts_per_face) + 1, np.int64)
    np.cumsum(verts_per_face, out=starts[1:])
    a = face_verts
    nxt = np.empty_like(a)
    for n in np.unique(verts_per_face):
        sel = np.nonzero(verts_per_face == n)[0]
        base = starts[sel][:, None] + np.arange(n)[None, :]
        nxt[base] = a[starts[sel][:, None] + (np.arange(n)[None, :] + 1) % n]
    e = np.stack([np.minimum(a, nxt), np.maximum(a, nxt)], 1)
    _, first = np.unique(e[:, 0].astype(np.int64) * (1 << 32) + e[:, 1], return_index=True)
    return e[np.sort(first)].astype(np.int32)


def torus(nu: int = 512, nv: int = 256, R: float = 1.0, r: float = 0.3,
          tri_fraction: float = 0.0, crease_fraction: float = 0.0, max_sharpness: float = 4.0,
          noise: float = 0.0, seed: int = 0, scheme: int = CATMARK) -> Cage:
    """Quad torus with nu x nv vertices.  A seeded ``tri_fraction`` of the quads is split
    into two triangles along a random diagonal and a seeded ``crease_fraction`` of the edges
    gets sharpness U[0, max_sharpness].  With scheme=LOOP every quad is split (random
    diagonal) so the cage is all triangles."""
    rng = np.random.default_rng(seed)
    th = 2.0 * np.pi * np.arange(nu) / nu
    ph = 2.0 * np.pi * np.arange(nv) / nv
    T, P = np.meshgrid(th, ph, indexing="ij")
    pos = np.stack([(R + r * np.cos(P)) * np.cos(T), (R + r * np.cos(P)) * np.sin(T),
                    r * np.sin(P)], -1).reshape(-1, 3)
    if noise > 0:
        pos = pos + rng.normal(0.0, noise, pos.shape)
    i, j = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    i, j = i.ravel(), j.ravel()
    v0 = i * nv + j
    v1 = ((i + 1) % nu) * nv + j
    v2 = ((i + 1) % nu) * nv + (j + 1) % nv
    v3 = i * nv + (j + 1) % nv
    quads = np.stack([v0, v1, v2, v3], 1)
    nq = quads.shape[0]
    split = rng.random(nq) < (1.0 if scheme == LOOP else tri_fraction)
    diag = rng.random(nq) < 0.5
    vpf, fv = [], []
    for q in range(nq):
        a, b, c, d = quads[q]
        if not split[q]:
            vpf.append(4); fv.extend((a, b, c, d))
        elif diag[q]:
            vpf.extend((3, 3)); fv.extend((a, b, c, a, c, d))
        else:
            vpf.extend((3, 3)); fv.extend((a, b, d, b, c, d))
    vpf = np.asarray(vpf, np.int32)
    fv = np.asarray(fv, np.int32)
    cage = Cage(pos.astype(np.float32), vpf, fv, scheme=scheme, name=f"torus{nu}x{nv}")
    if crease_fraction > 0:
        edges = _edges_of(vpf, fv)
        pick = rng.random(len(edges)) < crease_fraction
        cage.crease_verts = edges[pick].astype(np.int32)
        cage.crease_sharpness = rng.uniform(0.0, max_sharpness, int(pick.sum())).astype(np.float32)
    return cage


def cube(n: int = 8, noise: float = 0.01, seed: int = 0, scheme: int = CATMARK) -> Cage:
    """Unit cube [-0.5, 0.5]^3 with every face split into n x n quads (6n^2+2 vertices,
    eight valence-3 corners).  scheme=LOOP splits every quad into two triangles.  Vertices are
    numbered in the order the quads first visit them (cube faces by axis, then sign; quads by
    x, then y; corners (0,0), (1,0), (1,1), (0,1))."""
    rng = np.random.default_rng(seed)
    g = np.linspace(-0.5, 0.5, n + 1)
    corners = np.array([(0, 0), (1, 0), (1, 1), (0, 1)])
    xs, ys = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    blocks = []
    # each cube face: fixed axis, sign, two in-plane axes ordered for outward orientation
    for axis in range(3):
        for sign in (-1.0, 1.0):
            a1, a2 = [(axis + 1) % 3, (axis + 2) % 3]
            if sign < 0:
                a1, a2 = a2, a1
            p = np.zeros((n, n, 4, 3))
            p[..., axis] = 0.5 * sign
            p[..., a1] = g[xs[..., None] + corners[:, 0]]
            p[..., a2] = g[ys[..., None] + corners[:, 1]]
            blocks.append(p.reshape(-1, 3))
    visits = np.concatenate(blocks)                       # corner points in visit order
    k = np.rint(visits * 2 * n).astype(np.int64) + n     # grid coordinates in [0, 2n]
    keys = (k[:, 0] * (2 * n + 1) + k[:, 1]) * (2 * n + 1) + k[:, 2]
    _, first, inverse = np.unique(keys, return_index=True, return_inverse=True)
    order = np.argsort(first, kind="stable")              # unique points by first visit
    rank = np.empty_like(order)
    rank[order] = np.arange(len(order))
    quads = rank[inverse.ravel()].reshape(-1, 4)
    pos = visits[first[order]]
    if noise > 0:
        pos = pos + rng.normal(0.0, noise, pos.shape)
    if scheme == LOOP:
        split = rng.random(len(quads)) < 0.5
        a, b, c, d = quads.T
        tri = np.where(split[:, None], np.stack([a, b, c, a, c, d], 1),
                       np.stack([a, b, d, b, c, d], 1))
        vpf = np.full(2 * len(quads), 3, np.int32)
        fv = tri.reshape(-1)
    else:
        vpf = np.full(len(quads), 4, np.int32)
        fv = quads.reshape(-1)
    return Cage(pos.astype(np.float32), vpf, np.asarray(fv, np.int32), scheme=scheme,
                name=f"cube{n}")


def icosphere(subdivisions: int = 6, noise: float = 0.005, seed: int = 0) -> Cage:
    """Loop-scheme icosphere: an icosahedron split 4:1 ``subdivisions`` times with new points
    projected to the unit sphere (10*4^k + 2 vertices), then seeded Gaussian noise."""
    rng = np.random.default_rng(seed)
    t = (1.0 + 5 ** 0.5) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t),
             (0, -1, -t), (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.asarray(v, np.float64) / np.linalg.norm(v) for v in verts]
    tris = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
            (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
            (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdivisions):
        mid = {}

        def m(a, b):
            k = (a, b) if a < b else (b, a)
            if k not in mid:
                p = verts[a] + verts[b]
                verts.append(p / np.linalg.norm(p))
                mid[k] = len(verts) - 1
            return mid[k]

        nt = []
        for a, b, c in tris:
            ab, bc, ca = m(a, b), m(b, c), m(c, a)
            nt.extend(((a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)))
        tris = nt
    pos = np.asarray(verts)
    if noise > 0:
        pos = pos + rng.normal(0.0, noise, pos.shape)
    return Cage(pos.astype(np.float32), np.full(len(tris), 3, np.int32),
                np.asarray(tris, np.int32).ravel(), scheme=LOOP, name=f"icosphere{subdivisions}")


def bipyramid(n: int = 360, height: float = 1.0, scheme: int = CATMARK) -> Cage:
    """A closed double cone: a ring of n vertices and two poles of valence n joined by 2n
    triangles -- the extraordinary-vertex stress case (rows of hundreds of entries)."""
    a = np.arange(n) * (2.0 * np.pi / n)
    ring = np.stack([np.cos(a), np.sin(a), np.zeros(n)], 1)
    pos = np.concatenate([ring, [[0.0, 0.0, height], [0.0, 0.0, -height]]])
    top, bot = n, n + 1
    i = np.arange(n)
    j = (i + 1) % n
    tris = np.concatenate([np.stack([np.full(n, top), i, j], 1),
                           np.stack([np.full(n, bot), j, i], 1)])
    return Cage(pos.astype(np.float32), np.full(2 * n, 3, np.int32),
                tris.astype(np.int32).ravel(), scheme=scheme, name=f"bipyramid{n}")


def grid(nx: int = 6, ny: int = 6, noise: float = 0.02, seed: int = 0,
         scheme: int = CATMARK) -> Cage:
    """Open (nx x ny)-quad planar grid with a height field; has boundary edges and corners.
    scheme=LOOP splits quads into triangles."""
    rng = np.random.default_rng(seed)
    x, y = np.meshgrid(np.linspace(0, 1, nx + 1), np.linspace(0, 1, ny + 1), indexing="ij")
    z = 0.1 * np.sin(3 * x) * np.cos(2 * y)
    pos = np.stack([x, y, z], -1).reshape(-1, 3)
    pos = pos + rng.normal(0.0, noise, pos.shape)
    vpf, fv = [], []
    for i in range(nx):
        for j in range(ny):
            a = i * (ny + 1) + j
            b = (i + 1) * (ny + 1) + j
            c = (i + 1) * (ny + 1) + j + 1
            d = i * (ny + 1) + j + 1
            if scheme == LOOP:
                vpf.extend((3, 3)); fv.extend((a, b, c, a, c, d))
            else:
                vpf.append(4); fv.extend((a, b, c, d))
    return Cage(pos.astype(np.float32), np.asarray(vpf, np.int32), np.asarray(fv, np.int32),
                scheme=scheme, name=f"grid{nx}x{ny}")


def uniform_locations(cage: Cage, n: int, seed: int = 0):
    """n seeded limit-surface locations (ptex face, u, v), uniform over ptex faces with
    u, v ~ U[0, 1].  Loop (triangular) locations are folded into u + v <= 1 the way
    examples/glStencilViewer/glStencilViewer.cpp:367-370 does."""
    rng = np.random.default_rng(seed)
    nptex = int(cage.ptex_face_offsets()[-1])
    face = rng.integers(0, nptex, n).astype(np.int32)
    u = rng.random(n).astype(np.float32)
    v = rng.random(n).astype(np.float32)
    if cage.scheme == LOOP:
        fold = (u + v) > 1.0
        u[fold] = 1.0 - u[fold]
        v[fold] = 1.0 - v[fold]
    return face, u, v
