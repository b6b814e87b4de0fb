"""Test infrastructure only: a sequential CPU restatement of the reference's edge
orientation on adjacency matrices, the checker for the GPU orientation kernels.

The reference (gpucsl/pc/edge_orientation/) works on networkx graphs; this restates its
exact visiting order and update semantics without networkx:

* v-structures (v_structures.py:8-35): ordered skeleton edges (v1, v2) in column-major
  order (key v2 * p + v1), neighbours v3 of v2 ascending; an unshielded triple whose
  middle v2 is in neither sepset(v1, v3) nor sepset(v3, v1) adds v1 -> v2, v3 -> v2 and
  removes v2 -> v1, v2 -> v3 in the live graph (non-adjacency and neighbours are read
  from the skeleton);
* rules (orientation_rules.py:7-89), repeated until no rule fires: R1, then R2, then
  R3, each reading a snapshot taken before it and writing the live graph, visiting
  ordered edges in column-major order; R1 additionally requires the edge to be still
  undirected in the live graph.

D[a, b] = 1 means the directed graph has the edge a -> b (an undirected edge a - b is
both D[a, b] and D[b, a]).
"""
from __future__ import annotations

import itertools

import numpy as np


def _col_major_edges(D: np.ndarray):
    p = D.shape[0]
    a, b = np.nonzero(D)
    order = np.argsort(b * p + a, kind="stable")
    return list(zip(a[order].tolist(), b[order].tolist()))


def orient_v_structures(S: np.ndarray, sepsets: np.ndarray) -> np.ndarray:
    """v_structures.py:8-35 on the skeleton S (symmetric 0/1, zero diagonal)."""
    S = (np.asarray(S) != 0)
    p = S.shape[0]
    D = S.astype(np.uint8).copy()
    for v1, v2 in _col_major_edges(S):
        for v3 in np.nonzero(S[v2])[0].tolist():
            if v1 == v3 or S[v1, v3]:
                continue
            if v2 in sepsets[v1, v3] or v2 in sepsets[v3, v1]:
                continue
            D[v1, v2] = 1
            D[v3, v2] = 1
            D[v2, v1] = 0
            D[v2, v3] = 0
    return D


def apply_rules(D: np.ndarray) -> tuple[np.ndarray, int]:
    """orientation_rules.py:7-89; returns the final graph and the number of passes."""
    D = D.copy()
    passes = 0

    def nonadj(g, a, b):
        return not g[a, b] and not g[b, a]

    while True:
        passes += 1
        changed = False
        # R1: v1 -> v2 - v3, v1 and v3 non-adjacent: v2 -> v3
        g = D.copy()
        for v1, v2 in _col_major_edges(g):
            if g[v2, v1]:
                continue
            for v3 in np.nonzero(g[v2])[0].tolist():
                if v1 == v3:
                    continue
                if g[v3, v2] and nonadj(g, v1, v3) and D[v2, v3] and D[v3, v2]:
                    D[v2, v3] = 1
                    D[v3, v2] = 0
                    changed = True
        # R2: v1 -> v3 -> v2 and v1 - v2: v1 -> v2
        g = D.copy()
        for v1, v2 in _col_major_edges(g):
            if not g[v2, v1]:
                continue
            mids = sorted(set(np.nonzero(g[v1])[0].tolist()) & set(np.nonzero(g[:, v2])[0].tolist()))
            for v3 in mids:
                if not g[v3, v1] and not g[v2, v3]:
                    D[v1, v2] = 1
                    D[v2, v1] = 0
                    changed = True
        # R3: v1 - v3 -> v2, v1 - v4 -> v2, v3 and v4 non-adjacent, v1 - v2: v1 -> v2
        g = D.copy()
        for v1, v2 in _col_major_edges(g):
            if not g[v2, v1]:
                continue
            nb1 = set(np.nonzero(g[v1] & g[:, v1])[0].tolist())
            pr2 = set(np.nonzero(g[:, v2] & (1 - g[v2]))[0].tolist())
            C = sorted(nb1 & pr2)
            for v3, v4 in itertools.combinations(C, 2):
                if nonadj(g, v3, v4):
                    D[v1, v2] = 1
                    D[v2, v1] = 0
                    changed = True
        if not changed:
            return D, passes


def orient(S: np.ndarray, sepsets: np.ndarray) -> tuple[np.ndarray, int]:
    """edge_orientation.py:25-36: v-structures, then the rules to a fixed point."""
    return apply_rules(orient_v_structures(S, sepsets))
