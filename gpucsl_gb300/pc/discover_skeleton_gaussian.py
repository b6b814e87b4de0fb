"""Gaussian skeleton discovery, drop-in for gpucsl/pc/discover_skeleton_gaussian.py.

Same signature and result as the reference's discover_skeleton_gpu_gaussian
(discover_skeleton_gaussian.py:116-172): thresholds on the host (scipy), then the
correlation matrix (GPU kernel when none is given), the level loop and the zmin->pmax
epilogue in the sm_103a library, results returned as NumPy arrays.
"""
from __future__ import annotations

from timeit import default_timer as timer
from typing import List

import numpy as np

from .. import engine
from .helpers import SkeletonResult, get_gaussian_thresholds, log_time, timed
from .pc_validations import validate_given_devices


@timed
def discover_skeleton_gpu_gaussian(
    skeleton: np.ndarray,
    data: np.ndarray,
    correlation_matrix: np.ndarray,
    alpha: float,
    max_level: int,
    num_variables: int,
    num_observations: int,
    kernels=None,
    is_debug: bool = False,
    should_log: bool = False,
    devices: List[int] = [0],
    sync_device: int = None,
) -> SkeletonResult:
    validate_given_devices(devices, sync_device)
    torch = engine._torch()
    thresholds = get_gaussian_thresholds(data, alpha)
    dev = torch.device("cuda", devices[0])
    with torch.cuda.device(dev):
        if correlation_matrix is None:
            X = torch.from_numpy(np.ascontiguousarray(data)).to(dev)
            C = engine.correlation(X)
        else:
            C = torch.from_numpy(np.ascontiguousarray(correlation_matrix, dtype=np.float64)).to(dev)
        # is_debug: the bounds-checked build of the kernels (the reference compiles with -G)
        solver = kernels.gaussian_solver(num_variables, max_level) if kernels is not None else \
            engine.GaussianSolver(num_variables, max_level, device=dev, debug=is_debug)
        torch.cuda.synchronize(dev)
        start = timer()
        solver.run(C, num_observations, thresholds)
        computation_time = timer() - start
        log_time("Computation time", computation_time)
        final_skeleton, separation_sets, pmax = solver.to_host()
    return SkeletonResult(final_skeleton, separation_sets, pmax, computation_time)
