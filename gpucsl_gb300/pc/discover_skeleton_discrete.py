"""Discrete skeleton discovery, drop-in for gpucsl/pc/discover_skeleton_discrete.py.

Same signature and result as the reference's discover_skeleton_gpu_discrete
(discover_skeleton_discrete.py:24-128): ordinal encoding over the observed values,
column-major uint8 upload, the chi-squared level loop in the sm_103a library.
`memory_restriction` is accepted for compatibility; the working tables live in shared
memory, so no large working area is allocated.
"""
from __future__ import annotations

from timeit import default_timer as timer

import numpy as np

from .. import engine
from .helpers import SkeletonResult, log_time, timed


@timed
def discover_skeleton_gpu_discrete(
    skeleton: np.ndarray,
    data: np.ndarray,
    alpha: float,
    max_level: int,
    num_variables: int,
    num_observations: int,
    kernels=None,
    memory_restriction: int = None,
    is_debug: bool = False,
    should_log: bool = False,
) -> SkeletonResult:
    torch = engine._torch()
    codes, dims = engine.ordinal_encode(data)
    max_dim = int(dims.max()) if dims.size else 1
    solver = kernels.discrete_solver(num_variables, num_observations, max_level, max_dim) if kernels is not None \
        else engine.DiscreteSolver(num_variables, num_observations, max_level, max_dim)
    solver.load(codes, dims)
    torch.cuda.synchronize()
    start = timer()
    solver.run(alpha)
    computation_time = timer() - start
    log_time("Computation time", computation_time)
    result_skeleton, separation_sets, pmax = solver.to_host()
    return SkeletonResult(result_skeleton, separation_sets, pmax, computation_time)
