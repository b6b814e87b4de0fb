"""Host helpers of the skeleton-discovery path, with the reference's names and return
types (gpucsl/pc/helpers.py)."""
from __future__ import annotations

import logging
from functools import wraps
from math import sqrt
from timeit import default_timer as timer
from typing import Any, Callable, Dict, Generic, NamedTuple, Set, Tuple, TypeVar

import numpy as np
from scipy.stats import norm

T = TypeVar("T")
U = TypeVar("U")

NUMBER_OF_THRESHOLDS = 50


class TimedReturnT(Generic[T]):
    result: T
    runtime: float


class TimedReturn(NamedTuple):
    """(result, runtime in seconds) — helpers.py:18-27."""
    result: Any
    runtime: float


def timed(f: Callable[..., U]) -> Callable[..., TimedReturnT[U]]:
    """Wrap a result into TimedReturn(result, seconds) (helpers.py:30-39)."""
    @wraps(f)
    def wrap(*args, **kw):
        start = timer()
        result = f(*args, **kw)
        return TimedReturn(result, timer() - start)

    return wrap


def get_gaussian_thresholds(data: np.ndarray, alpha: float = 0.05):
    """Fisher-z thresholds per level (helpers.py:42-50): entry l is
    |Phi^-1(alpha/2)| / sqrt(n - l - 4) for the levels the 50-entry table covers, 0.0 after."""
    from ..engine import gaussian_thresholds

    return gaussian_thresholds(data.shape[0], alpha)


def init_pc_graph(data: np.ndarray) -> np.ndarray:
    """Fully connected start graph (helpers.py:53-55)."""
    p = data.shape[1]
    return np.ones((p, p), np.uint16)


def correlation_matrix_of(data: np.ndarray) -> np.ndarray:
    """Correlation matrix of the samples (helpers.py:58-59), computed on the GPU by
    the FP64 correlation kernel; returned as a NumPy array like the reference."""
    from .. import engine

    torch = engine._torch()
    X = torch.from_numpy(np.ascontiguousarray(data)).to("cuda")
    return engine.correlation(X).cpu().numpy()


def transform_to_pmax(zmin: np.ndarray, num_samples: int) -> np.ndarray:
    """FP64 twin of the device epilogue (helpers.py:85-86)."""
    return 2 * norm.sf(np.abs(np.sqrt(num_samples - 3) * zmin))


def postprocess_pmax(pmax: np.ndarray) -> np.ndarray:
    """Lower triangle and diagonal to -1 (helpers.py:96-101)."""
    pmax[np.tril_indices(pmax.shape[0])] = -1
    return pmax


def get_max_neighbor_count(compacted_skeleton: np.ndarray, columns_per_device: int = None,
                           device_index: int = 0) -> int:
    """Max degree of a compacted skeleton (helpers.py:104-118)."""
    col = compacted_skeleton[:, 0]
    return int(col.max()) if col.size else 0


def log(message):
    logging.info(message)


def log_time(message, value, unit="s", value_spacing=40):
    spacing_length = value_spacing - len(message)
    unit_message = ""
    if unit:
        spacing_length -= len(unit) + 2
        unit_message = f"({unit})"
    log(message + " " * max(spacing_length, 1) + unit_message + ": " + f"{value:1.6f}")


class PCResult(NamedTuple):
    """helpers.py:138-144."""
    directed_graph: Any
    separation_sets: Dict[Tuple[int, int], Set[int]]
    pmax: np.ndarray
    discover_skeleton_runtime: float
    edge_orientation_runtime: float
    discover_skeleton_kernel_runtime: float


class SkeletonResult(NamedTuple):
    """helpers.py:147-151 (field name spelled as in the reference)."""
    skeleton: np.ndarray
    seperation_sets: Dict[Tuple[int, int], Set[int]]
    pmax: np.ndarray
    discover_skeleton_kernel_time: float
