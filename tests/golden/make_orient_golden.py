"""Generate tests/golden/orient_cases.npz: edge-orientation cases solved by the
reference's own orientation code (gpucsl/pc/edge_orientation/v_structures.py and
orientation_rules.py, loaded by file path from the reference checkout so that the
package's GPU imports are not triggered).  Run in a container that has the reference
and networkx:

    python tests/golden/make_orient_golden.py <reference checkout>

Cases: random Erdos-Renyi skeletons (p 6..28) with random separating sets, including
conflicting v-structures, and sepsets drawn so that some unshielded triples collide."""
import importlib.util
import sys
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent / "orient_cases.npz"


def load(ref: Path, name: str):
    path = ref / "gpucsl" / "pc" / "edge_orientation" / f"{name}.py"
    spec = importlib.util.spec_from_file_location(f"ref_{name}", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def make_case(rng, p, dens, L, keep_common):
    upper = np.triu(rng.random((p, p)) < dens, 1)
    S = (upper | upper.T).astype(np.uint8)
    sep = np.full((p, p, L), -1, np.int32)
    for i in range(p):
        for j in range(i + 1, p):
            if S[i, j]:
                continue
            common = np.nonzero(S[i] & S[j])[0]
            if rng.random() < keep_common:  # the middles stay in the set: no v-structure
                pick = np.sort(rng.permutation(common)[:L])
            else:
                k = int(rng.integers(0, L + 1))
                cand = np.setdiff1d(np.arange(p), [i, j])
                pool = common if (common.size and rng.random() < 0.5) else cand
                pick = np.sort(rng.choice(pool, size=min(k, pool.size), replace=False))
            sep[i, j, :pick.size] = pick
            sep[j, i, :pick.size] = pick
    return S, sep


def main():
    import networkx as nx

    if len(sys.argv) < 2:
        sys.exit("usage: python tests/golden/make_orient_golden.py <reference checkout>")
    ref = Path(sys.argv[1])
    vs = load(ref, "v_structures")
    rules = load(ref, "orientation_rules")
    rng = np.random.default_rng(2024)
    cases = {}
    for c in range(40):
        p = int(rng.integers(6, 29))
        # half the cases keep most middles in the sets: few v-structures, so the rules
        # have undirected edges to orient
        S, sep = make_case(rng, p, float(rng.uniform(0.1, 0.45)), 3, 0.0 if c % 2 else 0.9)
        g = nx.Graph()
        g.add_nodes_from(range(p))
        g.add_edges_from([(int(a), int(b)) for a, b in zip(*np.nonzero(np.triu(S, 1)))])
        dag = g.to_directed()
        vs.orient_v_structure(dag, sep, g)
        rules.apply_rules(dag)
        D = np.zeros((p, p), np.uint8)
        for a, b in dag.edges:
            D[a, b] = 1
        cases[f"S{c}"] = S
        cases[f"sep{c}"] = sep
        cases[f"D{c}"] = D
    np.savez_compressed(OUT, n=np.array(40), **cases)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
