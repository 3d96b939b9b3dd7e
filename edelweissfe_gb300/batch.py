"""Batches of independent meshes of uneven size and mixed element types in one element pass.

Meshes of one dimension are concatenated into one block-diagonal system (`MeshBatch`): their
nodes, DOFs and CSR rows are stacked, so one group spans every mesh of a batch and each mesh's
DOF vectors and CSR data are contiguous slices of the batch's.  `BatchedPass` runs the element
pass of several batches (e.g. the 2D and the 3D meshes, each split into int32-indexable chunks)
either as one persistent launch (`efe_compute_elements_persistent`: the resident CTAs take tiles of
all batches from one work counter) or as one launch per batch, and can capture the whole pass
(zeroing of P, F, K and the launches) in a CUDA graph.
"""

import ctypes

import numpy as np
import torch

from . import _lib as L
from .assembly import ElementGroup, GPUAssembler


def chunk_meshes(meshes, elType, limit=2**31 - 1):
    """Split a list of meshes of one element type into consecutive chunks whose CSR patterns fit the
    int32 indexing of one batch: every element contributes at most (nodes x dim)^2 entries, so a
    chunk holds at most limit / (nodes x dim)^2 elements."""
    from .library import element_type

    et = element_type(elType)
    per = (et.nNodes * et.dim) ** 2
    cap = max(1, limit // per)
    chunks, cur, n = [], [], 0
    for m in meshes:
        e = len(m["conn"])
        if e > cap:
            raise ValueError(f"a single mesh of {e} elements exceeds the int32 CSR of one batch")
        if cur and n + e > cap:
            chunks.append(cur)
            cur, n = [], 0
        cur.append(m)
        n += e
    if cur:
        chunks.append(cur)
    return chunks


class MeshBatch:
    """meshes: list of dicts with coords [n, d], conn [E, nN], nodeDof [n], nDof, props [nP] or [E, nP],
    thickness (2D); all of one element type and material.  keep_host_pattern=False drops the host
    copies of the CSR indices and slot maps once they are on the device (large batches)."""

    def __init__(self, meshes, elType, material, precision="mixed", device=None, keep_host_pattern=True):
        node_off = np.cumsum([0] + [len(m["coords"]) for m in meshes])
        dof_off = np.cumsum([0] + [int(m["nDof"]) for m in meshes])
        el_off = np.cumsum([0] + [len(m["conn"]) for m in meshes])
        coords = np.concatenate([m["coords"] for m in meshes])
        nodeDof = np.concatenate([np.where(m["nodeDof"] >= 0, m["nodeDof"] + dof_off[i], -1)
                                  for i, m in enumerate(meshes)])  # fmt: skip
        conn = np.concatenate([m["conn"] + node_off[i] for i, m in enumerate(meshes)])
        props = np.concatenate([np.broadcast_to(np.asarray(m["props"], float), (len(m["conn"]), len(m["props"]) if
                                np.ndim(m["props"]) == 1 else np.shape(m["props"])[1])) for m in meshes])  # fmt: skip
        thickness = np.concatenate([np.broadcast_to(np.asarray(m.get("thickness", 1.0), float), (len(m["conn"]),))
                                    for m in meshes])  # fmt: skip
        self.asm = GPUAssembler(coords, nodeDof, int(dof_off[-1]),
                                [ElementGroup(elType, material, props, conn, thickness)],
                                precision=precision, device=device)  # fmt: skip
        self.nMeshes = len(meshes)
        self.dof_offsets = dof_off
        self.element_offsets = el_off
        ip = self.asm.indptr_host
        self.nnz_offsets = np.array([ip[d] for d in dof_off])
        if not keep_host_pattern:
            self.asm.indices_host = None
            self.asm._slots_host = None
            self.asm._conns_host = None
        self.nElements = int(el_off[-1])
        self.U = self.asm.constructDofVector()
        self.dU = self.asm.constructDofVector()
        self.P = self.asm.constructDofVector()
        self.F = self.asm.constructDofVector()
        self.K = self.asm.constructSystemMatrix()

    def mesh_slice(self, i):
        """(DOF slice, CSR-data slice) of mesh i in the batch vectors."""
        return (slice(int(self.dof_offsets[i]), int(self.dof_offsets[i + 1])),
                slice(int(self.nnz_offsets[i]), int(self.nnz_offsets[i + 1])))  # fmt: skip


# element types of the persistent kernel (efe_compute_elements_persistent), in its hand-out order:
# (shape, rule, kinematics, hyperelastic material) -> type index of the kernel
PERSISTENT_TYPES = {
    (L.EFE_HEXA20, L.EFE_RULE_3D_3X3X3, L.EFE_TOTAL_LAGRANGIAN, True): 0,  # e.g. C3D20TL Neo-Hooke
    (L.EFE_HEXA20, L.EFE_RULE_3D_3X3X3, L.EFE_SMALL_STRAIN, False): 1,  # C3D20 von Mises / linear elastic
    (L.EFE_HEXA8, L.EFE_RULE_3D_2X2X2, L.EFE_TOTAL_LAGRANGIAN, True): 2,  # C3D8TL Neo-Hooke
    (L.EFE_HEXA8, L.EFE_RULE_3D_2X2X2, L.EFE_SMALL_STRAIN, False): 3,  # C3D8 von Mises / linear elastic
    (L.EFE_QUAD8, L.EFE_RULE_2D_2X2, L.EFE_TOTAL_LAGRANGIAN, True): 4,  # CPE8RTL Neo-Hooke
}
PERSISTENT_MAX_GROUPS = 8


def persistent_type(elType, material):
    """Type index of an element type and material in the persistent kernel, or None."""
    from .library import element_type

    et = element_type(elType)
    hyper = material.lower().startswith("neohooke")
    if hyper and et.plane == L.EFE_PLANE_STRESS:
        return None  # the reference has no plane-stress hyperelasticity
    return PERSISTENT_TYPES.get((et.shape, et.rule, et.kinematics, hyper))


def persistent_capable(batches):
    """True if one persistent launch can run all batches: every batch of a type of the persistent
    kernel (PERSISTENT_TYPES), at most eight batches of each type, one precision."""
    kinds = [persistent_type(b.asm.groups[0].elType, b.asm.groups[0].material) for b in batches]
    if None in kinds or any(len(b.asm.groups) != 1 for b in batches):
        return False
    if any(kinds.count(k) > PERSISTENT_MAX_GROUPS for k in set(kinds)):
        return False
    # one precision for all (each type of the persistent kernel has its float-float form too)
    precs = {b.asm.kPrecision for b in batches}
    return len(precs) == 1


class BatchedPass:
    """The element pass of several MeshBatch objects: one persistent launch over all of them (when
    persistent_capable) or one launch per batch."""

    def __init__(self, batches, persistent=True):
        self.batches = list(batches)
        self.lib = L.load()
        self.can_persist = persistent_capable(self.batches)
        self.persistent = persistent and self.can_persist
        dev = self.batches[0].asm.device
        self.counter = torch.zeros(1, dtype=torch.int64, device=dev)
        self.status = torch.zeros(4, dtype=torch.int32, device=dev)
        self.graph = None
        if self.can_persist:
            n = len(self.batches)
            self._items = (L.EfeWorkItem * n)(*[
                L.EfeWorkItem(ctypes.addressof(b.asm.mesh), ctypes.addressof(b.asm._groups_c[0]), b.U.data_ptr(),
                              b.dU.data_ptr(), b.K.data_ptr(), b.P.data_ptr(), b.F.data_ptr())
                for b in self.batches
            ])  # fmt: skip
            self._prec = self.batches[0].asm.kPrecision

    def _launch(self):
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        if self.persistent:
            L.check(self.lib.efe_compute_elements_persistent(self._items, len(self.batches), self._prec,
                                                             ctypes.c_void_p(self.counter.data_ptr()),
                                                             ctypes.c_void_p(self.status.data_ptr()), stream),
                    "efe_compute_elements_persistent")  # fmt: skip
        else:
            for b in self.batches:
                a = b.asm
                L.check(self.lib.efe_compute_elements(ctypes.byref(a.mesh), a._groups_c, len(a.groups),
                                                      ctypes.c_void_p(b.U.data_ptr()), ctypes.c_void_p(b.dU.data_ptr()),
                                                      None, 0.0, a.kPrecision, ctypes.c_void_p(b.K.data_ptr()),
                                                      ctypes.c_void_p(b.P.data_ptr()), ctypes.c_void_p(b.F.data_ptr()),
                                                      ctypes.c_void_p(self.status.data_ptr()), stream),
                        "efe_compute_elements")  # fmt: skip

    def step(self):
        """One pass over every element of every batch: zero the accumulators, run the kernels."""
        for b in self.batches:
            b.P.zero_()
            b.F.zero_()
            b.K.zero_()
        self.status.zero_()
        self._launch()

    def capture(self):
        """Capture step() in a CUDA graph (warm-up on a side stream first, as torch requires)."""
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.step()
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.step()
        return self.graph

    def replay(self):
        self.graph.replay()

    def check_status(self):
        st = self.status.cpu().numpy()
        if st[0] & L.EFE_STATUS_TC_TIMEOUT:
            raise RuntimeError("the tensor-core tangent gave up waiting for its MMAs: K is incomplete")
        if st[0] & L.EFE_STATUS_BOUNDS:
            raise IndexError("device bounds check: an element indexes outside a node, DOF or CSR array")
        if st[0] & L.EFE_STATUS_CUTBACK:
            from .exceptions import CutbackRequest

            raise CutbackRequest("material point failed in the batch", 0.5)
        return st
