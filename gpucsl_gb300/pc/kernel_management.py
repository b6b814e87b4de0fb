"""`kernels=` compatibility object (gpucsl/pc/kernel_management.py:293-342).

The reference JIT-compiles one module per problem shape and lets callers pass the
compiled `Kernels` in to keep compilation out of their timings.  Here the kernels are
compiled ahead of time into libgpucsl_gb300.so; a `Kernels` object instead holds
preallocated device solvers for one shape, so passing it keeps allocation out of the
timing in the same way.
"""
from __future__ import annotations

from .. import engine


class Kernels:
    def __init__(self, kind: str, **shape):
        self.kind = kind
        self.shape = shape
        self._solver = None

    @staticmethod
    def for_gaussian_ci(variable_count: int, device_count: int = 1, max_level: int = 0, is_debug: bool = False,
                        should_log: bool = False) -> "Kernels":
        if device_count != 1:
            raise ValueError("gpucsl_gb300 runs one skeleton per GPU (device_count must be 1)")
        k = Kernels("gaussian", p=variable_count, max_level=max_level, debug=is_debug)
        k._solver = engine.GaussianSolver(variable_count, max_level, debug=is_debug)
        return k

    @staticmethod
    def for_discrete_ci(max_level: int, variable_count: int, max_dim: int, n_observations: int,
                        memory_restriction: int = None, is_debug: bool = False, should_log: bool = False) -> "Kernels":
        k = Kernels("discrete", p=variable_count, n=n_observations, max_level=max_level, max_dim=max_dim,
                    debug=is_debug)
        k._solver = engine.DiscreteSolver(variable_count, n_observations, max_level, max_dim, debug=is_debug)
        return k

    def gaussian_solver(self, p: int, max_level: int) -> engine.GaussianSolver:
        s = self._solver
        if self.kind != "gaussian" or s is None or s.p != p or s.max_level != max_level:
            s = engine.GaussianSolver(p, max_level, debug=bool(self.shape.get("debug", False)))
        return s

    def discrete_solver(self, p: int, n: int, max_level: int, max_dim: int) -> engine.DiscreteSolver:
        s = self._solver
        if self.kind != "discrete" or s is None or (s.p, s.n, s.max_level) != (p, n, max_level) or s.max_dim < max_dim:
            s = engine.DiscreteSolver(p, n, max_level, max_dim, debug=bool(self.shape.get("debug", False)))
        return s
