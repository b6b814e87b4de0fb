"""gpucsl_gb300: GB300-native (sm_103a) skeleton discovery for the PC-stable algorithm.

Public entry points mirror the reference package (hpi-epic/gpucsl):
    gpucsl_gb300.pc.pc.GaussianPC / DiscretePC
    gpucsl_gb300.pc.discover_skeleton_gaussian.discover_skeleton_gpu_gaussian
    gpucsl_gb300.pc.discover_skeleton_discrete.discover_skeleton_gpu_discrete
    gpucsl_gb300.pc.edge_orientation.edge_orientation.orient_edges
The compute path is libgpucsl_gb300.so (C ABI in include/gpucsl_gb300.h).
"""
__version__ = "0.1.0"
