"""Meek's orientation rules R1-R3 applied to a fixed point
(gpucsl/pc/edge_orientation/orientation_rules.py:7-89).

Each pass runs R1, then R2, then R3; every rule reads a snapshot of the graph taken
before it and writes the live graph, visiting ordered edges in column-major order.
An undirected edge a - b is stored as both (a, b) and (b, a).
"""
from __future__ import annotations

import itertools
import logging


def apply_rules(dag) -> None:
    p = len(dag.nodes)

    def order(e):
        return e[1] * p + e[0]

    def adjacent(g, a, b):
        return g.has_edge(a, b) or g.has_edge(b, a)

    def both_ways(g, a, b):
        return g.has_edge(a, b) and g.has_edge(b, a)

    def orient(a, b):
        dag.add_edge(a, b)
        dag.remove_edges_from([(b, a)])

    while True:
        changed = False

        # R1: a -> b - c with a, c non-adjacent  =>  b -> c
        snap = dag.copy()
        for a, b in sorted(snap.edges, key=order):
            if snap.has_edge(b, a):
                continue
            for c in sorted(snap.successors(b)):
                if c == a:
                    continue
                if snap.has_edge(c, b) and not adjacent(snap, a, c) and both_ways(dag, b, c):
                    logging.debug(f"R1: remove ({c, b})")
                    orient(b, c)
                    changed = True

        # R2: a -> c -> b with a - b  =>  a -> b
        snap = dag.copy()
        for a, b in sorted(snap.edges, key=order):
            if not snap.has_edge(b, a):
                continue
            for c in sorted(set(snap.successors(a)).intersection(snap.predecessors(b))):
                if not snap.has_edge(c, a) and not snap.has_edge(b, c):
                    logging.debug(f"R2: remove ({b, a})")
                    orient(a, b)
                    changed = True

        # R3: a - c -> b, a - d -> b, c and d non-adjacent, a - b  =>  a -> b
        snap = dag.copy()
        for a, b in sorted(snap.edges, key=order):
            if not snap.has_edge(b, a):
                continue
            undirected_of_a = set(snap.successors(a)).intersection(snap.predecessors(a))
            parents_only_of_b = set(snap.predecessors(b)).difference(snap.successors(b))
            cands = sorted(undirected_of_a.intersection(parents_only_of_b))
            for c, d in itertools.combinations(cands, 2):
                if not adjacent(snap, c, d):
                    logging.debug(f"R3: remove ({b, a})")
                    orient(a, b)
                    changed = True

        if not changed:
            return
