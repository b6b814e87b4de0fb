"""CPDAG from skeleton and sepsets (gpucsl/pc/edge_orientation/edge_orientation.py:25-36):
v-structures, then Meek's rules to a fixed point (Meek 1995, UAI)."""
from __future__ import annotations

import numpy as np

from ..helpers import timed
from .orientation_rules import apply_rules
from .v_structures import orient_v_structure


@timed
def orient_edges(skeleton, separation_sets: np.ndarray):
    """The reference's CPU orientation on networkx graphs (kept as-is)."""
    dag = skeleton.to_directed()
    orient_v_structure(dag, separation_sets, skeleton)
    apply_rules(dag)
    return dag


@timed
def orient_edges_gpu(skeleton, separation_sets: np.ndarray):
    """The same CPDAG from the GPU kernels (gcsl_orient_edges); `skeleton` is a networkx
    graph or a (p, p) adjacency matrix.  Returns an nx.DiGraph like orient_edges."""
    import networkx as nx

    from ...orient import orient_matrix

    if isinstance(skeleton, (nx.Graph, nx.DiGraph)):
        p = skeleton.number_of_nodes()
        A = np.zeros((p, p), np.uint8)
        for a, b in skeleton.edges:
            A[a, b] = A[b, a] = 1
    else:
        A = np.asarray(skeleton)
        p = A.shape[0]
    D, _ = orient_matrix(A, separation_sets)
    dag = nx.DiGraph()
    dag.add_nodes_from(range(p))
    dag.add_edges_from((int(a), int(b)) for a, b in zip(*np.nonzero(D)))
    return dag
