"""ORACLE (test infrastructure): RWG basis construction restated from MLFMAxwell.

Restates, in numpy:
  * node deduplication by exact coordinate equality (limpiarnodos,
    modReadStl.f90:1444-1533).  Node *numbering* here is first-occurrence
    order; the reference relabels by swap-with-last, which changes node ids
    but no coordinate, edge or triangle, so nothing numeric depends on it;
  * edge enumeration (llenar_lados, Buscar_L_Comun, llenar_todo,
    modRWG.f90:8-131): per triangle the pairs (1,2), (1,3), (2,3); an edge is
    created at the first occurrence of a pair that occurs again later, T+ is
    the triangle of that first occurrence and T- the one of the next
    occurrence, the edge keeps the first occurrence's vertex order;
  * parametros_rwg (modRWG.f90:133-174): e_long, e_centro;
  * hallar_geometria_rwg (modRWG.f90:270-328): centroids, the nine
    sub-triangle centroids and areas, with the reference's single-precision
    literals (1./3.) and (2./3.).

All index arrays returned are 0-based.
"""
from __future__ import annotations

import numpy as np

F13 = float(np.float32(1.0) / np.float32(3.0))   # Fortran (1./3.) promoted to double
F23 = float(np.float32(2.0) / np.float32(3.0))   # Fortran (2./3.)


def dedup_nodes(tris: np.ndarray):
    v = tris.reshape(-1, 3)
    # exact equality of the three doubles (bit pattern, with -0.0 == 0.0)
    key = np.ascontiguousarray(v + 0.0).view(np.dtype((np.void, 24))).ravel()
    _, first, inv = np.unique(key, return_index=True, return_inverse=True)
    order = np.argsort(first, kind="stable")          # unique ids in first-occurrence order
    rank = np.empty_like(order)
    rank[order] = np.arange(order.size)
    node_of = rank[inv]
    p_coord = v[first[order]]
    t_p = node_of.reshape(-1, 3)
    return p_coord, t_p


def build_edges(t_p: np.ndarray):
    T = t_p.shape[0]
    lt = np.empty((3 * T, 2), dtype=np.int64)
    lt[0::3] = t_p[:, [0, 1]]
    lt[1::3] = t_p[:, [0, 2]]
    lt[2::3] = t_p[:, [1, 2]]
    lo = np.minimum(lt[:, 0], lt[:, 1])
    hi = np.maximum(lt[:, 0], lt[:, 1])
    order = np.lexsort((np.arange(3 * T), hi, lo))
    lo_s, hi_s = lo[order], hi[order]
    firsts, seconds = [], []
    i = 0
    n = order.size
    while i < n:
        j = i
        while j + 1 < n and lo_s[j + 1] == lo_s[i] and hi_s[j + 1] == hi_s[i]:
            j += 1
        grp = order[i:j + 1]          # ascending entry indices of one vertex pair
        for q in range(0, len(grp) - 1, 2):
            firsts.append(grp[q]); seconds.append(grp[q + 1])
        i = j + 1
    firsts = np.asarray(firsts, dtype=np.int64)
    seconds = np.asarray(seconds, dtype=np.int64)
    srt = np.argsort(firsts, kind="stable")
    firsts, seconds = firsts[srt], seconds[srt]
    e_p = lt[firsts]
    x = firsts // 3
    y = seconds // 3
    e_t = np.stack([x, y], axis=1)

    def opposite(tri, ep):
        t = t_p[tri]
        c1 = (t[:, 0] != ep[:, 0]) & (t[:, 0] != ep[:, 1])
        c2 = (t[:, 1] != ep[:, 0]) & (t[:, 1] != ep[:, 1])
        return np.where(c1, t[:, 0], np.where(c2, t[:, 1], t[:, 2]))

    e_po = np.stack([opposite(x, e_p), opposite(y, e_p)], axis=1)
    return e_p, e_t, e_po


def triangle_geometry(p_coord, t_p):
    p1, p2, p3 = p_coord[t_p[:, 0]], p_coord[t_p[:, 1]], p_coord[t_p[:, 2]]
    t_baric = F13 * ((p1 + p2) + p3)
    v = [None] * 11
    v[1], v[2], v[3] = p1, p2, p3
    v[4] = p1 + F13 * (p2 - p1)
    v[5] = p1 + F23 * (p2 - p1)
    v[6] = p2 + F13 * (p3 - p2)
    v[7] = p2 + F23 * (p3 - p2)
    v[8] = p3 + F13 * (p1 - p3)
    v[9] = p3 + F23 * (p1 - p3)
    v[10] = t_baric
    trip = [(1, 4, 9), (4, 5, 10), (5, 2, 6), (6, 10, 7), (7, 8, 3),
            (7, 8, 10), (8, 9, 10), (9, 4, 10), (5, 6, 10)]
    sub = np.stack([F13 * ((v[a] + v[b]) + v[c]) for a, b, c in trip], axis=1)  # [T, 9, 3]
    ba = p1 - p2
    ca = p1 - p3
    cr = np.stack([ba[:, 1] * ca[:, 2] - ba[:, 2] * ca[:, 1],
                   ba[:, 2] * ca[:, 0] - ba[:, 0] * ca[:, 2],
                   ba[:, 0] * ca[:, 1] - ba[:, 1] * ca[:, 0]], axis=1)
    t_area = 0.5 * np.sqrt((cr[:, 0] * cr[:, 0] + cr[:, 1] * cr[:, 1]) + cr[:, 2] * cr[:, 2])
    return t_baric, np.ascontiguousarray(sub), t_area


class RWG:
    """RWG geometry of a triangle soup, in the reference's basis order."""

    def __init__(self, tris: np.ndarray):
        tris = np.asarray(tris, dtype=np.float64)
        self.p_coord, self.t_p = dedup_nodes(tris)
        self.e_p, self.e_t, self.e_po = build_edges(self.t_p)
        a = self.p_coord[self.e_p[:, 0]]
        b = self.p_coord[self.e_p[:, 1]]
        d = a - b
        self.e_long = np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2])
        self.e_centro = 0.5 * (a + b)
        self.t_baric, self.t_baric_sub, self.t_area = triangle_geometry(self.p_coord, self.t_p)
        self.N = self.e_p.shape[0]
        self.T = self.t_p.shape[0]
        self.P = self.p_coord.shape[0]
