"""Edge orientation on the GPU (C ABI gcsl_orient_edges): v-structures, then Meek's
rules R1-R3 to a fixed point, with the result of the reference's sequential code
(gpucsl/pc/edge_orientation/edge_orientation.py:25-36)."""
from __future__ import annotations

import ctypes as ct

import numpy as np

from . import _lib


def orient_edges_device(G, sepsets=None, workspace=None):
    """G: (p, p) int16/uint16 device skeleton; sepsets: (p, p, L) int32 device tensor with
    -1 padding, or None.  Returns ((p, p) uint8 device tensor D with D[a, b] = 1 for a -> b,
    rule passes)."""
    torch = _lib.require_cuda()
    L = _lib.lib()
    p = int(G.shape[0])
    if G.dim() != 2 or G.shape[1] != p:
        raise ValueError("G must be a square matrix")
    G = G.contiguous()
    sep_len = 0 if sepsets is None else int(sepsets.shape[2])
    if sepsets is not None:
        if tuple(sepsets.shape[:2]) != (p, p) or sepsets.dtype != torch.int32:
            raise ValueError("sepsets must be a (p, p, L) int32 tensor")
        sepsets = sepsets.contiguous()
    need = int(L.gcsl_orient_workspace_bytes(p))
    if workspace is None or workspace.numel() < need:
        workspace = torch.empty(need, dtype=torch.uint8, device=G.device)
    D = torch.empty((p, p), dtype=torch.uint8, device=G.device)
    passes = ct.c_int32(0)
    _lib.check(L.gcsl_orient_edges(G.data_ptr(), p, _lib.ptr(sepsets) if sep_len else None, sep_len, D.data_ptr(),
                                   ct.byref(passes), workspace.data_ptr(), workspace.numel(), _lib.stream_ptr()),
               "gcsl_orient_edges")
    return D, int(passes.value)


def orient_matrix(skeleton: np.ndarray, separation_sets: np.ndarray | None):
    """Host arrays in, host (p, p) uint8 directed adjacency out."""
    torch = _lib.require_cuda()
    S = np.ascontiguousarray(np.asarray(skeleton) != 0, dtype=np.uint16)
    np.fill_diagonal(S, 0)
    G = torch.from_numpy(S.view(np.int16)).cuda()
    sep = None
    if separation_sets is not None and np.asarray(separation_sets).ndim == 3 and np.asarray(separation_sets).shape[2]:
        sep = torch.from_numpy(np.ascontiguousarray(separation_sets, dtype=np.int32)).cuda()
    D, passes = orient_edges_device(G, sep)
    return D.cpu().numpy(), passes
