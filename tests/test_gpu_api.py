"""The reference's public surface on the GPU path: discover_skeleton_gpu_gaussian /
discover_skeleton_gpu_discrete return TimedReturn(SkeletonResult(skeleton, sepsets, pmax,
kernel_time), runtime); GaussianPC / DiscretePC.execute() return PCResult."""
import numpy as np
import pytest

from gpucsl_gb300.synthetic import discrete_bn_data, gaussian_dag_data
from oracle import gaussian as og

pytestmark = pytest.mark.gpu


def test_discover_skeleton_gpu_gaussian_signature_and_result(cuda):
    from gpucsl_gb300.pc.discover_skeleton_gaussian import discover_skeleton_gpu_gaussian
    from gpucsl_gb300.pc.helpers import init_pc_graph

    w = gaussian_dag_data(20, 1000, 2, 1)
    graph = init_pc_graph(w.data)
    res = discover_skeleton_gpu_gaussian(graph, w.data, None, 0.05, 3, 20, 1000)
    (skeleton, sepsets, pmax, kt), runtime = res
    ref = og.skeleton(og.corrcoef(w.data), 1000, 0.05, 3)
    assert skeleton.dtype == np.uint16 and skeleton.shape == (20, 20)
    assert sepsets.shape == (20, 20, 3) and sepsets.dtype == np.int32
    assert (skeleton == ref.skeleton).all()
    assert (sepsets == ref.sepsets).all()
    assert np.allclose(pmax, ref.pmax, rtol=1e-9, atol=0)
    assert runtime >= kt >= 0
    # with a caller-supplied correlation matrix
    res2 = discover_skeleton_gpu_gaussian(graph, w.data, og.corrcoef(w.data), 0.05, 3, 20, 1000)
    assert (res2.result.skeleton == ref.skeleton).all()


def test_multi_device_request_is_rejected(cuda):
    from gpucsl_gb300.pc.discover_skeleton_gaussian import discover_skeleton_gpu_gaussian
    from gpucsl_gb300.pc.pc_validations import GpucslError

    w = gaussian_dag_data(8, 200, 2, 1)
    with pytest.raises(GpucslError):
        discover_skeleton_gpu_gaussian(np.ones((8, 8), np.uint16), w.data, None, 0.05, 2, 8, 200, devices=[0, 1])


def test_discover_skeleton_gpu_discrete(cuda):
    from gpucsl_gb300.pc.discover_skeleton_discrete import discover_skeleton_gpu_discrete

    w = discrete_bn_data(15, 3000, 2, 8)
    (skeleton, sepsets, pmax, kt), runtime = discover_skeleton_gpu_discrete(
        np.ones((15, 15), np.uint16), w.data, 0.05, 3, 15, 3000)
    assert skeleton.shape == (15, 15) and sepsets.shape == (15, 15, 3)
    assert (np.diag(skeleton) == 0).all() and (skeleton == skeleton.T).all()
    iu = np.triu_indices(15, 1)
    assert ((pmax[iu] >= 0) & (pmax[iu] <= 1)).all()


def test_gaussian_pc_execute(cuda):
    pytest.importorskip("networkx")
    from gpucsl_gb300.pc.pc import GaussianPC

    w = gaussian_dag_data(15, 2000, 2, 12)
    res = GaussianPC(w.data, 3, 0.05).set_distribution_specific_options().execute()
    pc, runtime = res
    assert pc.directed_graph.number_of_nodes() == 15
    assert pc.separation_sets.shape == (15, 15, 3)
    assert pc.discover_skeleton_runtime >= pc.discover_skeleton_kernel_runtime


def test_discrete_pc_execute(cuda):
    pytest.importorskip("networkx")
    from gpucsl_gb300.pc.pc import DiscretePC

    w = discrete_bn_data(10, 4000, 2, 13)
    pc, runtime = DiscretePC(w.data, None, 0.05).set_distribution_specific_options().execute()
    assert pc.directed_graph.number_of_nodes() == 10
    assert pc.separation_sets.shape == (10, 10, 8)
