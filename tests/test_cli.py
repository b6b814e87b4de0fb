"""Command line and output files (mirrors the reference's tests/test_cli.py: option
validation, CSV naming, the output formats of gpucsl/cli/cli_io.py:39-101)."""
from pathlib import Path

import numpy as np
import pytest

from gpucsl_gb300.cli.cli import gpucsl_cli
from gpucsl_gb300.cli.cli_io import (force_csv_suffix, get_file_name_stem, read_correlation_matrix, read_csv,
                                     write_configuration, write_directed_graph, write_pmax,
                                     write_separation_sets)
from gpucsl_gb300.cli.cli_util import GpucslError


def test_error_on_no_parameter():
    with pytest.raises(SystemExit):
        gpucsl_cli([])


def test_error_on_missing_dataset():
    with pytest.raises(SystemExit):
        gpucsl_cli(["-l", "3", "-o", "out", "--gaussian"])


def test_error_on_missing_output_path():
    with pytest.raises(SystemExit):
        gpucsl_cli(["-d", "foobar", "-l", "3", "--gaussian"])


def test_exactly_one_of_discrete_and_gaussian():
    with pytest.raises(GpucslError):
        gpucsl_cli(["-d", "foobar", "-o", "out", "-l", "3"])
    with pytest.raises(GpucslError):
        gpucsl_cli(["-d", "foobar", "-o", "out", "-l", "3", "--gaussian", "--discrete"])


def test_error_on_discrete_with_correlation_matrix():
    with pytest.raises(GpucslError):
        gpucsl_cli(["-d", "foobar", "-o", "out", "-l", "3", "--discrete", "-c", "corr"])


def test_error_on_several_gpus():
    with pytest.raises(GpucslError):
        gpucsl_cli(["-d", "foobar", "-o", "out", "--discrete", "-g", "0", "1"])
    with pytest.raises(GpucslError):
        gpucsl_cli(["-d", "foobar", "-o", "out", "--gaussian", "-g", "0", "1"])


def test_csv_names():
    assert force_csv_suffix(Path("foobar/foo.csv")) == Path("foobar/foo.csv")
    assert force_csv_suffix(Path("foobar/foo")) == Path("foobar/foo.csv")
    assert get_file_name_stem("foobar/foo.csv") == "foo"
    assert read_correlation_matrix(None) is None


def test_read_csv_types(tmp_path):
    (tmp_path / "ints.csv").write_text("0,1,2\n2,1,0\n")
    (tmp_path / "floats.csv").write_text("0.5,1,2\n2,1,0\n")
    a = read_csv(tmp_path / "ints")
    assert a.dtype == np.int64 and a.shape == (2, 3)
    b = read_csv(tmp_path / "floats.csv")
    assert b.dtype == np.float64 and b[0, 0] == 0.5
    with pytest.raises(GpucslError):
        read_csv(tmp_path / "missing.csv")


def test_output_formats(tmp_path):
    import networkx as nx

    sep = np.full((3, 3, 2), -1, np.int32)
    sep[0, 2] = [1, -1]
    sep[2, 0] = [1, -1]
    sep[1, 2] = [0, 2]
    write_separation_sets(tmp_path, "d", sep)
    assert (tmp_path / "d_sepset.txt").read_text() == "0 2 1\n1 2 0 2\n2 0 1\n"
    write_separation_sets(tmp_path, "e", np.zeros((3, 3, 0), np.int32))
    assert (tmp_path / "e_sepset.txt").read_text() == ""
    write_pmax(tmp_path, "d", np.array([[0.0, 0.123456], [1.0, 0.5]]))
    assert (tmp_path / "d_pmax.csv").read_text() == "0.0000,0.1235\n1.0000,0.5000\n"
    g = nx.DiGraph()
    g.add_nodes_from(range(3))
    g.add_edges_from([(0, 1), (1, 0), (2, 1)])
    write_directed_graph(tmp_path, "d", g)
    back = nx.read_gml(tmp_path / "d.gml", destringizer=int)
    assert set(back.edges) == set(g.edges)
    write_configuration(tmp_path, "d", ["-d", "d.csv", "--gaussian"])
    assert (tmp_path / "d_config.txt").read_text().endswith("-d d.csv --gaussian\n")


@pytest.mark.gpu
def test_cli_end_to_end(cuda, tmp_path):
    import networkx as nx

    from gpucsl_gb300.synthetic import discrete_bn_data, gaussian_dag_data

    X = gaussian_dag_data(20, 1000, 2, 1).data
    np.savetxt(tmp_path / "gauss.csv", X, delimiter=",", fmt="%.17g")
    res = gpucsl_cli(["-d", str(tmp_path / "gauss.csv"), "--gaussian", "-l", "3", "-a", "0.05",
                      "-o", str(tmp_path / "out")])
    out = tmp_path / "out"
    assert (out / "gauss_config.txt").exists()
    g = nx.read_gml(out / "gauss.gml", destringizer=int)
    assert set(g.edges) == set(res.directed_graph.edges)
    pm = np.loadtxt(out / "gauss_pmax.csv", delimiter=",")
    assert np.allclose(pm, np.round(res.pmax, 4), atol=5e-5)
    lines = (out / "gauss_sepset.txt").read_text().splitlines()
    sep = np.asarray(res.separation_sets)
    expected = int((sep[:, :, 0] != -1).sum()) if sep.size else 0
    assert len(lines) == expected
    D = discrete_bn_data(15, 3000, 2, 3).data
    np.savetxt(tmp_path / "disc.csv", D, delimiter=",", fmt="%d")
    res_d = gpucsl_cli(["-d", str(tmp_path / "disc"), "--discrete", "-l", "2", "-o", str(out)])
    assert (out / "disc.gml").exists() and (out / "disc_pmax.csv").exists()
    assert res_d.pmax.shape == (15, 15)
