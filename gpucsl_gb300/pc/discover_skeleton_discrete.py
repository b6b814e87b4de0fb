"""Discrete skeleton discovery, drop-in for gpucsl/pc/discover_skeleton_discrete.py.

Same signature and result as the reference's discover_skeleton_gpu_discrete
(discover_skeleton_discrete.py:24-128): ordinal encoding over the observed values (on
the device for integer-valued data, gcsl_ordinal_encode; on the host otherwise),
column-major uint8 layout, the chi-squared level loop in the sm_103a library.
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
    data = np.asarray(data)
    codes_dev = dims_dev = None
    if data.dtype.kind in "iu" or (data.dtype == np.float64 and np.all(np.isfinite(data))):
        # integer-valued categories: encoded on the device (observed values ascending)
        try:
            X = torch.from_numpy(np.ascontiguousarray(data if data.dtype.kind == "f" or data.dtype == np.uint8
                                                      else data.astype(np.int64))).cuda()
            codes_dev, dims_dev = engine.ordinal_encode_device(X)
        except engine._lib.GcslError:
            codes_dev = dims_dev = None  # wide or non-integer categories: the host encoder
    if codes_dev is not None:
        dims = dims_dev.cpu().numpy()
    else:
        codes, dims = engine.ordinal_encode(data)
    max_dim = int(dims.max()) if dims.size else 1
    # is_debug: the bounds-checked build of the kernels (the reference compiles with -G)
    solver = kernels.discrete_solver(num_variables, num_observations, max_level, max_dim) if kernels is not None \
        else engine.DiscreteSolver(num_variables, num_observations, max_level, max_dim, debug=is_debug)
    if codes_dev is not None:
        solver.load(codes_dev=codes_dev[:, :num_observations], dims_dev=dims_dev)
    else:
        solver.load(codes, dims)
    torch.cuda.synchronize()
    start = timer()
    solver.run(alpha)
    computation_time = timer() - start
    log_time("Computation time", computation_time)
    result_skeleton, separation_sets, pmax = solver.to_host()
    return SkeletonResult(result_skeleton, separation_sets, pmax, computation_time)
