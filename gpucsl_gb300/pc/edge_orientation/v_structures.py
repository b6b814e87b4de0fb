"""Unshielded-collider orientation (gpucsl/pc/edge_orientation/v_structures.py:8-35).

For every ordered skeleton edge (v1, v2), taken in column-major order (key v2 * p + v1),
and every neighbour v3 != v1 of v2 in ascending order: if v1 and v3 are not adjacent and
v2 lies in neither sepset(v1, v3) nor sepset(v3, v1), orient v1 -> v2 <- v3.
"""
from __future__ import annotations

import logging

import numpy as np


def orient_v_structure(dag, separation_sets: np.ndarray, skeleton=None) -> None:
    if skeleton is None:
        skeleton = dag.to_undirected()
    p = len(skeleton.nodes)

    def separated_by(v, a, b) -> bool:
        return v in separation_sets[a][b] or v in separation_sets[b][a]

    ordered = sorted(skeleton.to_directed().edges, key=lambda e: e[1] * p + e[0])
    for v1, v2 in ordered:
        for v3 in sorted(skeleton.neighbors(v2)):
            if v3 == v1 or skeleton.has_edge(v1, v3):
                continue
            if separated_by(v2, v1, v3):
                continue
            logging.debug(f"v: {[(v2, v1), (v2, v3)]}")
            dag.add_edges_from([(v1, v2), (v3, v2)])
            dag.remove_edges_from([(v2, v1), (v2, v3)])
