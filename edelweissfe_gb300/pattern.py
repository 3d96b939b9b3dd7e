"""CSR pattern and element-to-CSR slot maps (host side, once per mesh).

Produces the same canonical CSR pattern as `CSRGenerator.__init__`
(`edelweissfe/numerics/csrgenerator.pyx:47-98`, scipy's sorted/deduplicated CSR of the VIJ
pattern of `dofmanager.py:522-557`) without forming the VIJ index vectors: the rows of a node's
DOFs hold the DOFs of every node that shares an element with it.  Instead of the reference's
per-VIJ-entry slot map ``x[k]`` it returns one slot per element node pair: the CSR position of
(row = first DOF of node b, col = first DOF of node a); entry (j, k) of the pair lies at
``slot + k * rowLen(b) + j``.
"""

import ctypes

import numpy as np

from . import _lib as L


def build_pattern(dim, nNodes, nodeDof, nDof, conns):
    """indptr [nDof+1], indices [nnz], nodeRowLen [nNodes], slots (list of [E, n, n]) -- all int32."""
    lib = L.load()
    nodeDof = np.ascontiguousarray(nodeDof, np.int32)
    conns = [np.ascontiguousarray(c, np.int32) for c in conns]
    nG = len(conns)
    cptr = (ctypes.c_void_p * max(nG, 1))(*[c.ctypes.data for c in conns])
    nEl = np.array([len(c) for c in conns] or [0], np.int64)
    nn = np.array([c.shape[1] for c in conns] or [0], np.int32)
    indptr = np.zeros(int(nDof) + 1, np.int32)
    rowlen = np.zeros(int(nNodes), np.int32)
    nnz = lib.efe_pattern_count(
        dim, nNodes, nodeDof.ctypes.data, nG, cptr, nEl.ctypes.data, nn.ctypes.data, int(nDof), indptr.ctypes.data,
        rowlen.ctypes.data,
    )
    if nnz < 0:
        raise RuntimeError("efe_pattern_count: " + lib.efe_last_error().decode())
    indices = np.zeros(int(nnz), np.int32)
    slots = [np.zeros((len(c), c.shape[1], c.shape[1]), np.int32) for c in conns]
    sptr = (ctypes.c_void_p * max(nG, 1))(*[s.ctypes.data for s in slots])
    L.check(
        lib.efe_pattern_fill(
            dim, nNodes, nodeDof.ctypes.data, nG, cptr, nEl.ctypes.data, nn.ctypes.data, int(nDof),
            indptr.ctypes.data, indices.ctypes.data, sptr,
        ),
        "efe_pattern_fill",
    )
    return indptr, indices, rowlen, slots
