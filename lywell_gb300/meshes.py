"""Synthetic PEC bodies as triangle soups, and ASCII STL I/O.

The MLFMAxwell driver reads an ASCII STL file (modReadStl.f90:1378-1442,
``obtener_p_t``) and deduplicates its nodes by exact coordinate equality
(modReadStl.f90:1444-1533, ``limpiarnodos``).  The bodies here are written as
triangle soups ``tris[T, 3, 3]`` (triangle, vertex, xyz) in the order an STL
file would list them, so the same array can feed this library's RWG builder
and, written with :func:`write_stl`, the reference program.

Meshes:
  * :func:`icosphere`            — icosahedron subdivided ``level`` times and
                                   projected to a sphere (20·4^level triangles).
  * :func:`spheroid`             — icosphere affinely mapped to semi-axes
                                   (a, b, c), with an optional seeded radial
                                   perturbation smoothed over 2-ring neighbours.
  * :func:`superellipsoid`       — icosphere vertices pushed onto
                                   |x/a|^e + |y/b|^e + |z/c|^e = 1.

``quantum`` rounds every coordinate to a multiple of ``quantum`` (a power of
two), so that a decimal print with enough fractional digits is parsed back
exactly by any reader, including one that divides an integer mantissa by a
power of ten.
"""
from __future__ import annotations

import numpy as np

__all__ = ["icosphere", "spheroid", "superellipsoid", "write_stl", "read_stl",
           "quantize", "mean_edge"]


def _icosahedron():
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([
        [-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
        [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
        [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([
        [0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
        [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
        [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
        [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    return v, f


def _subdivide(v, f):
    """Split every triangle into four; new vertices are unit-normalised edge midpoints."""
    verts = [tuple(x) for x in v]
    cache = {}

    def mid(a, b):
        key = (a, b) if a < b else (b, a)
        if key in cache:
            return cache[key]
        m = (np.asarray(verts[a]) + np.asarray(verts[b])) * 0.5
        m /= np.linalg.norm(m)
        verts.append(tuple(m))
        cache[key] = len(verts) - 1
        return cache[key]

    out = []
    for a, b, c in f:
        ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
        out += [[a, ab, ca], [b, bc, ab], [c, ca, bc], [ab, bc, ca]]
    return np.asarray(verts, dtype=np.float64), np.asarray(out, dtype=np.int64)


def icosphere_indexed(level: int):
    """Unit icosphere as (vertices[P,3], faces[T,3]) with outward orientation."""
    v, f = _icosahedron()
    for _ in range(level):
        v, f = _subdivide(v, f)
    return v, f


def quantize(x: np.ndarray, quantum: float | None) -> np.ndarray:
    if not quantum:
        return x
    return np.round(x / quantum) * quantum


def _soup(v, f, quantum):
    v = quantize(v, quantum)
    return np.ascontiguousarray(v[f])  # [T, 3, 3]


def icosphere(level: int, radius: float = 1.0, quantum: float | None = None) -> np.ndarray:
    """Triangle soup of an icosphere: 20·4^level triangles, 30·4^level RWG edges."""
    v, f = icosphere_indexed(level)
    return _soup(v * radius, f, quantum)


def _ring_neighbours(nv, f):
    nb = [set() for _ in range(nv)]
    for a, b, c in f:
        nb[a].update((b, c)); nb[b].update((a, c)); nb[c].update((a, b))
    return nb


def spheroid(level: int, axes=(3.0, 0.75, 0.75), noise: float = 0.0, seed: int = 1234,
             quantum: float | None = None) -> np.ndarray:
    """Icosphere mapped to an ellipsoid with semi-axes ``axes``.

    With ``noise`` > 0 every vertex is moved radially by ``noise`` times a
    uniform U(-1, 1) sample (``numpy.random.default_rng(seed)``) averaged over
    the vertex and its 2-ring neighbours.
    """
    v, f = icosphere_indexed(level)
    p = v * np.asarray(axes, dtype=np.float64)
    if noise:
        rng = np.random.default_rng(seed)
        u = rng.uniform(-1.0, 1.0, size=len(v))
        nb1 = _ring_neighbours(len(v), f)
        sm = np.empty_like(u)
        for i in range(len(v)):
            ring = set(nb1[i])
            for j in nb1[i]:
                ring |= nb1[j]
            ring.add(i)
            idx = np.fromiter(ring, dtype=np.int64)
            sm[i] = u[idx].mean()
        rhat = p / np.linalg.norm(p, axis=1, keepdims=True)
        p = p + (noise * sm)[:, None] * rhat
    return _soup(p, f, quantum)


def superellipsoid(level: int, axes=(4.0, 2.0, 2.0), exponent: float = 4.0,
                   quantum: float | None = None) -> np.ndarray:
    """Icosphere directions scaled onto |x/a|^e + |y/b|^e + |z/c|^e = 1."""
    v, f = icosphere_indexed(level)
    a = np.asarray(axes, dtype=np.float64)
    s = (np.abs(v / a) ** exponent).sum(axis=1) ** (-1.0 / exponent)
    p = v * s[:, None]
    return _soup(p, f, quantum)


def mean_edge(tris: np.ndarray) -> float:
    e = np.concatenate([tris[:, 1] - tris[:, 0], tris[:, 2] - tris[:, 1], tris[:, 0] - tris[:, 2]])
    return float(np.linalg.norm(e, axis=1).mean())


def write_stl(path: str, tris: np.ndarray, digits: int = 12, name: str = "body") -> None:
    """Write an ASCII STL; coordinates use fixed-point with ``digits`` decimals."""
    fmt = "%." + str(digits) + "f"
    n = np.cross(tris[:, 1] - tris[:, 0], tris[:, 2] - tris[:, 0])
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    lines = [f"solid {name}"]
    for t in range(tris.shape[0]):
        lines.append("  facet normal " + " ".join(fmt % x for x in n[t]))
        lines.append("    outer loop")
        for k in range(3):
            lines.append("      vertex " + " ".join(fmt % x for x in tris[t, k]))
        lines.append("    endloop")
        lines.append("  endfacet")
    lines.append(f"endsolid {name}")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def read_stl(path: str) -> np.ndarray:
    """Read an ASCII STL into a triangle soup [T, 3, 3] (vertices in file order)."""
    verts = []
    with open(path) as fh:
        for line in fh:
            w = line.split()
            if w and w[0].lower() == "vertex":
                verts.append([float(w[1]), float(w[2]), float(w[3])])
    a = np.asarray(verts, dtype=np.float64)
    return a.reshape(-1, 3, 3)
