"""CPDAG from skeleton and sepsets (gpucsl/pc/edge_orientation/edge_orientation.py:25-36):
v-structures, then Meek's rules to a fixed point (Meek 1995, UAI)."""
from __future__ import annotations

import numpy as np

from ..helpers import timed
from .orientation_rules import apply_rules
from .v_structures import orient_v_structure


@timed
def orient_edges(skeleton, separation_sets: np.ndarray):
    dag = skeleton.to_directed()
    orient_v_structure(dag, separation_sets, skeleton)
    apply_rules(dag)
    return dag
