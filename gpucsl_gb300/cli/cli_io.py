"""Input and output files of the command line (gpucsl/cli/cli_io.py:10-101), same names
and formats: `<stem>.gml` (the CPDAG, networkx GML), `<stem>_sepset.txt` (one line
`i k s1 s2 ...` per ordered pair with a separating set, row-major), `<stem>_pmax.csv`
(p x p, comma-separated, `%.4f`) and `<stem>_config.txt` (the command line).  CSV input is
read with numpy (no header, comma-separated)."""
from __future__ import annotations

import os
from pathlib import Path

import numpy as np

from .cli_util import error


def force_csv_suffix(path: Path) -> Path:
    path = Path(path)
    return path if path.suffix == ".csv" else path.parent / (path.stem + ".csv")


def get_file_name_stem(dataset_path: str) -> str:
    return Path(dataset_path).stem


def read_csv(path) -> np.ndarray:
    path = force_csv_suffix(Path(path))
    try:
        data = np.loadtxt(path.absolute(), delimiter=",", dtype=np.float64, ndmin=2)
    except FileNotFoundError as e:
        error(str(e))
    # integer-valued files stay integers (discrete categories)
    if data.size and np.all(data == np.round(data)) and np.all(np.abs(data) < 2**53):
        as_int = data.astype(np.int64)
        if np.array_equal(as_int, data):
            return as_int
    return data


def read_correlation_matrix(path):
    """None when no cached matrix is given (the correlation is then computed)."""
    return None if path is None else read_csv(path).astype(np.float64)


def write_separation_sets(output_path: Path, stem: str, sepsets: np.ndarray):
    sepsets = np.asarray(sepsets)
    with open(Path(output_path) / (stem + "_sepset.txt"), "w", newline="") as f:
        if sepsets.size == 0:  # the file exists even without separating sets
            return
        p = sepsets.shape[0]
        for i in range(p):
            for k in range(p):
                s = sepsets[i, k]
                if s[0] == -1:
                    continue
                items = s[s != -1]
                f.write(f"{i} {k} " + " ".join(str(int(v)) for v in items) + "\n")


def write_directed_graph(output_path: Path, stem: str, directed_graph):
    import networkx as nx

    nx.write_gml(directed_graph, Path(output_path) / (stem + ".gml"))


def write_pmax(output_path: Path, stem: str, pmax: np.ndarray):
    np.savetxt(Path(output_path) / (stem + "_pmax.csv"), np.asarray(pmax), delimiter=",", fmt="%.4f")


def write_configuration(output_path: Path, stem: str, command_line_arguments):
    with open(Path(output_path) / (stem + "_config.txt"), "w", newline="") as f:
        f.write(f"The output for the dataset {stem} was generated using the following given parameters: \n\n")
        f.write(" ".join(command_line_arguments))
        f.write("\n")


def write_results(output_path, stem: str, result):
    if not os.path.isdir(output_path):
        os.makedirs(output_path)
    write_directed_graph(output_path, stem, result.directed_graph)
    write_separation_sets(output_path, stem, result.separation_sets)
    write_pmax(output_path, stem, result.pmax)
    print(f"successfully wrote results to: {output_path}")


def write_results_and_config(output_directory: str, dataset_path: str, command_line_arguments, result):
    out = Path(output_directory)
    stem = get_file_name_stem(dataset_path)
    write_results(out, stem, result)
    write_configuration(out, stem, command_line_arguments)
