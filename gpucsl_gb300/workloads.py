"""Named workloads for timing and profiling a single configuration from the command line:

  python -m gpucsl_gb300.workloads --workload cfg2 [--repeat N]

cfg1   Gaussian p = 20, n = 1000, degree 2, seed 1, alpha 0.05, levels <= 3
cfg2   Gaussian p = 1000, n = 10000, degree 3, seed 2, alpha 0.01, to termination
wide   Gaussian p = 5000, n = 2000, degree 3, seed 5, alpha 0.01, levels <= 1: C (200 MB),
       zmin and pmax exceed the 129 MB L2, so level 0, compaction and the pmax kernels
       run against HBM
cfg3   discrete p = 200, n = 50000, cardinality 2..5, degree 2, seed 3, alpha 0.05, levels <= 3
cfg4   512 uneven Gaussian instances (p 50..400, n 500..20000), split precision, levels <= 4
       (--instances N: the first N of them)
orient edge orientation (v-structures and Meek's rules) of the cfg2 skeleton and sepsets
encode device ordinal encoding of the cfg3 samples (200 int64 columns, n = 50000)

Each repeat is one full solve from samples in device memory (correlation included for
the Gaussian workloads); the script prints one line per repeat with its device time.
"""
from __future__ import annotations

import argparse
import json

GAUSS = {"cfg1": (20, 1000, 2, 1, 0.05, 3), "cfg2": (1000, 10000, 3, 2, 0.01, 998),
         "wide": (5000, 2000, 3, 5, 0.01, 1)}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="cfg2", choices=sorted(list(GAUSS) + ["cfg3", "cfg4", "orient", "encode"]))
    ap.add_argument("--repeat", type=int, default=2)
    ap.add_argument("--instances", type=int, default=512,
                    help="cfg4: solve the first N of the 512 instances (smaller cases for profiling)")
    args = ap.parse_args(argv)

    import torch

    from . import engine
    from .synthetic import discrete_bn_data, gaussian_dag_data, gaussian_dag_data_device

    torch.cuda.set_device(0)

    def timed(fn):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        out = fn()
        b.record()
        torch.cuda.synchronize()
        return out, a.elapsed_time(b)

    if args.workload in GAUSS:
        p, n, deg, seed, alpha, maxl = GAUSS[args.workload]
        X = torch.from_numpy(gaussian_dag_data(p, n, deg, seed).data).cuda()
        thr = engine.gaussian_thresholds(n, alpha)
        solver = engine.GaussianSolver(p, min(maxl, p - 2) if p > 2 else 0)
        C = torch.empty((p, p), dtype=torch.float64, device="cuda")
        ws = torch.empty(int(engine._lib.lib().gcsl_corr_tc_workspace_bytes(n, p)), dtype=torch.uint8, device="cuda")

        def solve():
            engine.correlation(X, out=C, workspace=ws)
            return solver.run(C, n, thr)

        for r in range(args.repeat):
            st, ms = timed(solve)
            print(json.dumps({"workload": args.workload, "repeat": r, "ms": round(ms, 3), "tests": st.tests,
                              "levels_run": st.levels_run}), flush=True)
    elif args.workload == "orient":
        from .orient import orient_edges_device

        p, n, deg, seed, alpha, maxl = GAUSS["cfg2"]
        X = torch.from_numpy(gaussian_dag_data(p, n, deg, seed).data).cuda()
        solver = engine.GaussianSolver(p, 12)  # the cfg2 loop ends at level 10; 12 bounds the sepsets
        st = solver.run(engine.correlation(X), n, engine.gaussian_thresholds(n, alpha))
        G, sep, _ = solver.to_host()
        Gd = torch.from_numpy(G.view("int16")).cuda()
        sepd = torch.from_numpy(sep[:, :, :max(st.levels_run - 1, 1)].astype("int32")).cuda()
        for r in range(args.repeat):
            (_, passes), ms = timed(lambda: orient_edges_device(Gd, sepd))
            print(json.dumps({"workload": "orient", "repeat": r, "ms": round(ms, 3), "passes": passes}), flush=True)
    elif args.workload == "encode":
        d = discrete_bn_data(200, 50000, 2, 3)
        Xd = torch.from_numpy(d.data.astype("int64")).cuda()
        for r in range(args.repeat):
            (_, dims), ms = timed(lambda: engine.ordinal_encode_device(Xd))
            print(json.dumps({"workload": "encode", "repeat": r, "ms": round(ms, 3),
                              "max_dim": int(dims.max().item())}), flush=True)
    elif args.workload == "cfg3":
        d = discrete_bn_data(200, 50000, 2, 3)
        codes, dims = engine.ordinal_encode(d.data)
        ds = engine.DiscreteSolver(200, 50000, 3, int(dims.max()))
        ds.load(codes, dims)
        for r in range(args.repeat):
            st, ms = timed(lambda: ds.run(0.05))
            print(json.dumps({"workload": "cfg3", "repeat": r, "ms": round(ms, 3), "tests": st.tests}), flush=True)
    else:
        from .batch import GaussianBatch
        from .synthetic import batch_instance_sizes

        sizes = batch_instance_sizes(512)[:max(1, min(512, args.instances))]
        Xs = [gaussian_dag_data_device(p, n, d, s) for (p, n, d, s) in sizes]
        b = GaussianBatch([s[0] for s in sizes], [s[1] for s in sizes], 0.01, 4, "split")
        b.bind_samples(Xs)
        for r in range(args.repeat):
            _, ms = timed(lambda: b.run(graph=False, sync=False))
            res = b.collect()
            print(json.dumps({"workload": "cfg4", "repeat": r, "ms": round(ms, 3),
                              "tests": sum(x.tests for x in res)}), flush=True)


if __name__ == "__main__":
    main()
