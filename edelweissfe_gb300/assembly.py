"""GPU element evaluation and CSR assembly behind the reference's element/assembly interface.

`GPUAssembler` is the drop-in for the two calls `NIST.solveIncrement` makes on the hot path
(`edelweissfe/solvers/nonlinearimplicitstatic.py:421, 451`):

* ``computeElements(elements, U_np, dU, P, K, F, timeStep) -> (P, K, F)``
  (NIST.computeElements, `nonlinearimplicitstatic.py:794-849`): every element's material update,
  P_e, |P_e| and K_e, with K_e scattered straight into the CSR data;
* ``assembleStiffnessCSR(K)`` (`:753-770`, CSRGenerator.updateCSR `numerics/csrgenerator.pyx:100-115`):
  the CSR matrix with the reference's canonical pattern (int32 indptr/indices, sorted columns).

plus the state calls of the elements (`acceptLastState`, `resetToLastValidState`,
`getResultArray`, `displacementelement/element.py:373-409`).

All buffers are torch tensors on the GPU; the work is done by libefe_gb300.so through its C ABI
(include/efe_gb300.h).  Quadrature-point state is kept structure-of-arrays on the device:
``state[field, element * nInt + qp]`` with fields ``[stress(6), strain(6), material state]``
in the reference's Voigt order of the element family.
"""

import ctypes
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib as L
from . import library
from .exceptions import CutbackRequest
from .pattern import build_pattern


def _upload(a, dtype, dev):
    """Row-major (C-contiguous) device copy of a host array: the C ABI indexes raw pointers."""
    return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).to(dev).contiguous()


@dataclass
class ElementGroup:
    """Elements of one type and material (a section, `sections/base/sectionbase.py:86-108`).

    conn: [E, nNodes] node indices into the mesh coordinates (reference node order of the type);
    props: material properties, [nProps] shared or [E, nProps] per element;
    thickness: 2D section thickness (`sections/plane.py:66`), scalar or [E]; ignored for solids."""

    elType: str
    material: str
    props: np.ndarray
    conn: np.ndarray
    thickness: object = 1.0
    name: str = ""
    _dev: dict = field(default_factory=dict, repr=False)


class GPUAssembler:
    """Element pass + CSR assembly on one GPU.

    coords: [nNodes, dim] reference coordinates; nodeDof: [nNodes] first DOF of each node
    (-1 for nodes without DOFs; DofManager numbering, `numerics/dofmanager.py:259-300`);
    nDof: size of the DOF vectors; groups: ElementGroup list in the reference's element order.
    precision: "fp64" (everything FP64), "mixed" (FP32 tangent, FP64 residual and state) or
    "mixed-ff" (as "mixed", with the small-strain strain increment and element residual in
    float-float arithmetic; the return map, state and global residual accumulation stay FP64)."""

    def __init__(self, coords, nodeDof, nDof, groups, precision="fp64", device=None):
        self.lib = L.load()
        if not torch.cuda.is_available():
            raise RuntimeError("GPUAssembler needs a CUDA device (there is no CPU fallback)")
        dev = torch.device(device or "cuda")
        if dev.index is None:
            dev = torch.device("cuda", torch.cuda.current_device())
        self.device = dev
        coords = np.ascontiguousarray(coords, np.float64)
        self.dim = coords.shape[1]
        self.nNodes = coords.shape[0]
        self.nDof = int(nDof)
        self.nodeDof_host = np.ascontiguousarray(nodeDof, np.int32)
        self.groups = list(groups)
        self.precision = precision
        self.kPrecision = {"fp64": L.EFE_K_FP64, "mixed": L.EFE_K_FP32, "mixed-ff": L.EFE_K_FP32_FF}[precision]
        self.kdtype = torch.float64 if precision == "fp64" else torch.float32
        self._build_pattern()
        # rows come in aligned groups of dim (a node's DOF rows, one shared column list) when every
        # node's first DOF is a multiple of dim and the nodes' DOFs fill 0 .. nDof-1
        used = self.nodeDof_host[self.nodeDof_host >= 0]
        self.rowGroup = self.dim if (self.nDof == self.dim * len(np.unique(used)) and np.all(used % self.dim == 0)
                                     and self.dim in (2, 3)) else 1  # fmt: skip
        dev = self.device
        self.coords = _upload(coords, np.float64, dev)
        self.nodeDof = _upload(self.nodeDof_host, np.int32, dev)
        self.nodeRowLen = _upload(self.nodeRowLen_host, np.int32, dev)
        self.indptr = _upload(self.indptr_host, np.int32, dev)
        self.indices = _upload(self.indices_host, np.int32, dev)
        self.status = torch.zeros(4, dtype=torch.int32, device=dev)
        self.mesh = L.EfeMesh(
            self.dim, self.nNodes, self.nDof, self.nnz, self.coords.data_ptr(), self.nodeDof.data_ptr(),
            self.nodeRowLen.data_ptr()
        )
        offset = 0
        structs = []
        for g in self.groups:
            structs.append(self._setup_group(g, offset))
            offset += len(g.conn)
        self.nElements = offset
        self._groups_c = (L.EfeGroup * len(structs))(*structs)
        # default tile (autotune.default_variant): the tensor-core tangent where it measured faster;
        # the autotuner may choose otherwise
        from .autotune import default_variant

        for i in range(len(self.groups)):
            self._groups_c[i].tileVariant = default_variant(self, i)
        self._setup_geometry()

    # ------------------------------------------------------------------ set-up
    def _build_pattern(self):
        conns = [np.ascontiguousarray(g.conn, np.int32) for g in self.groups]
        for g, c in zip(self.groups, conns):
            et = library.element_type(g.elType)
            if c.ndim != 2 or c.shape[1] != et.nNodes:
                raise ValueError(f"connectivity of {g.elType} must be [E, {et.nNodes}]")
            if et.dim != self.dim:
                raise ValueError(f"{g.elType} is {et.dim}D but the mesh is {self.dim}D")
            if len(c) and (c.min() < 0 or c.max() >= self.nNodes):
                raise ValueError("connectivity refers to a node outside the mesh")
            if len(c) and (self.nodeDof_host[c] < 0).any():
                raise ValueError("an element node has no DOFs")
        self._conns_host = conns
        self.indptr_host, self.indices_host, self.nodeRowLen_host, self._slots_host = build_pattern(
            self.dim, self.nNodes, self.nodeDof_host, self.nDof, conns
        )
        self.nnz = len(self.indices_host)

    def _setup_group(self, g, offset):
        dev = self.device
        et = library.element_type(g.elType)
        mcode, nProps, nm = library.material(g.material)
        E = len(g.conn)
        props = np.asarray(g.props, np.float64)
        if props.ndim == 1:
            props = np.broadcast_to(props, (E, len(props)))
        if props.shape[1] < nProps:
            raise ValueError(f"{g.material} needs {nProps} properties")
        th = np.broadcast_to(np.asarray(g.thickness, np.float64), (E,))
        nPts = E * et.nInt
        S = 12 + nm
        d = g._dev
        d["type"] = et
        d["conn"] = _upload(self._conns_host[self.groups.index(g)], np.int32, dev)
        d["pairSlot"] = _upload(self._slots_host[self.groups.index(g)], np.int32, dev)
        d["props"] = _upload(props, np.float64, dev)
        d["thickness"] = _upload(th, np.float64, dev)
        d["geomG"] = torch.zeros((et.dim * et.nNodes, nPts), dtype=torch.float64, device=dev)
        if self.kPrecision in (L.EFE_K_FP32, L.EFE_K_FP32_FF):
            d["geomG32"] = torch.zeros((et.dim * et.nNodes, nPts), dtype=torch.float32, device=dev)
        if self.kPrecision in (L.EFE_K_FP32, L.EFE_K_FP32_FF):
            # float-float form of dN/dX (with geomG32): read by the mixed-ff pass and by the reverse
            # small-strain pass, which forms its B-products on the FP32 pipe when it is present
            d["geomGlo"] = torch.zeros((et.dim * et.nNodes, nPts), dtype=torch.float32, device=dev)
        d["geomS"] = torch.zeros(nPts, dtype=torch.float64, device=dev)
        d["stateRef"] = torch.zeros((S, nPts), dtype=torch.float64, device=dev)
        d["stateTemp"] = torch.zeros((S, nPts), dtype=torch.float64, device=dev)
        if et.totalLagrangian:
            d["auxRef"] = torch.zeros((6, nPts), dtype=torch.float64, device=dev)
            d["auxTemp"] = torch.zeros((6, nPts), dtype=torch.float64, device=dev)
        d["offset"] = offset
        for key, t in d.items():
            if isinstance(t, torch.Tensor) and not t.is_contiguous():
                raise AssertionError(f"{key} must be contiguous for the C ABI")
        return L.EfeGroup(
            et.shape, et.rule, et.kinematics, et.plane, mcode, props.shape[1], E, offset,
            d["conn"].data_ptr(), d["pairSlot"].data_ptr(), d["props"].data_ptr(),
            d["thickness"].data_ptr() if et.dim == 2 else None,
            d["geomG"].data_ptr(), d["geomG32"].data_ptr() if "geomG32" in d else None,
            d["geomGlo"].data_ptr() if "geomGlo" in d else None, d["geomS"].data_ptr(), d["stateRef"].data_ptr(), d["stateTemp"].data_ptr(),
            d["auxRef"].data_ptr() if et.totalLagrangian else None,
            d["auxTemp"].data_ptr() if et.totalLagrangian else None,
        )  # fmt: skip

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def _setup_geometry(self):
        self.status.zero_()
        for i in range(len(self.groups)):
            L.check(
                self.lib.efe_setup_geometry(
                    ctypes.byref(self.mesh), ctypes.byref(self._groups_c[i]), ctypes.c_void_p(self.status.data_ptr()),
                    self._stream(),
                ),
                "efe_setup_geometry",
            )
        st = self.status.cpu().numpy()
        if st[0] & L.EFE_STATUS_BAD_JACOBIAN:
            raise ValueError(f"element {0x7FFFFFFF - int(st[1])} has a non-positive Jacobian determinant")

    # ------------------------------------------------------------------ parameters
    def setCoordinates(self, coords):
        """Move the nodes (same topology and DOF numbering) and recompute the element geometry
        (the reference re-runs setNodes + initializeElement, element.py:164-205)."""
        c = torch.as_tensor(coords, dtype=torch.float64).to(self.device).reshape(self.nNodes, self.dim)
        self.coords.copy_(c)
        self._setup_geometry()

    def setProperties(self, group, props):
        """Replace the material properties of one group: [nProps] shared or [E, nProps] per element."""
        d = self.groups[group]._dev["props"]
        p = torch.as_tensor(props, dtype=torch.float64).to(self.device)
        if p.dim() == 1:
            p = p[: d.shape[1]].expand_as(d)
        d.copy_(p[:, : d.shape[1]])

    def resetState(self):
        """Zero the quadrature-point history of every group (a fresh, undeformed model)."""
        for g in self.groups:
            for key in ("stateRef", "stateTemp", "auxRef", "auxTemp"):
                if key in g._dev:
                    g._dev[key].zero_()

    # ------------------------------------------------------------------ buffers
    def constructDofVector(self):
        """Zero DOF vector on the device (DofManager.constructDofVector, dofmanager.py)."""
        return torch.zeros(self.nDof, dtype=torch.float64, device=self.device)

    def constructSystemMatrix(self):
        """Zero CSR data vector (double in fp64 mode, float in mixed mode)."""
        return torch.zeros(self.nnz, dtype=self.kdtype, device=self.device)

    # ------------------------------------------------------------------ the element pass
    def _as_device(self, x):
        if isinstance(x, torch.Tensor):
            if x.device != self.device or x.dtype != torch.float64:
                x = x.to(self.device, torch.float64)
            return x.contiguous()
        return torch.as_tensor(np.asarray(x, np.float64), device=self.device)

    def launch(self, U_np, dU, P, K, F, time=None, dT=0.0, status=None):
        """Enqueue one element pass on the current stream (no synchronisation, no status check).
        status: an int32 device tensor of 4 words to report into instead of the assembler's own
        (for passes in flight at the same time); the caller zeroes it."""
        if K.dtype != self.kdtype or K.numel() != self.nnz:
            raise ValueError(f"K must be a {self.kdtype} vector of length nnz={self.nnz}")
        for v in (U_np, dU, P, F):
            if v.numel() != self.nDof or v.dtype != torch.float64 or v.device != self.device:
                raise ValueError("DOF vectors must be float64 device tensors of length nDof")
        t2 = (ctypes.c_double * 2)(*(time if time is not None else (0.0, 0.0)))
        L.check(
            self.lib.efe_compute_elements(
                ctypes.byref(self.mesh), self._groups_c, len(self.groups), ctypes.c_void_p(U_np.data_ptr()),
                ctypes.c_void_p(dU.data_ptr()), t2, float(dT), self.kPrecision, ctypes.c_void_p(K.data_ptr()),
                ctypes.c_void_p(P.data_ptr()), ctypes.c_void_p(F.data_ptr()),
                ctypes.c_void_p((self.status if status is None else status).data_ptr()), self._stream(),
            ),
            "efe_compute_elements",
        )

    def check_status(self):
        """Raise CutbackRequest if a material point failed in the last pass (synchronises)."""
        st = self.status.cpu().numpy()
        if st[0] & L.EFE_STATUS_TC_TIMEOUT:
            raise RuntimeError("the tensor-core tangent gave up waiting for its MMAs (tile variant 3): K is incomplete")
        if st[0] & L.EFE_STATUS_BOUNDS:
            raise IndexError(f"device bounds check: element {0x7FFFFFFF - int(st[1])} indexes outside a node, DOF "
                             "or CSR array (the access was skipped; P, F and K of this pass are invalid)")
        if st[0] & L.EFE_STATUS_CUTBACK:
            first = 0x7FFFFFFF - int(st[1])
            raise CutbackRequest(f"material point failed in element {first} ({int(st[2])} points)", 0.5)
        return st

    def computeElements(self, elements, U_np, dU, P, K, F, timeStep=None, check=True):
        """NIST.computeElements (nonlinearimplicitstatic.py:794-849) on the GPU.

        `elements` is accepted for signature parity; the element set is the one given at
        construction.  U_np, dU: total displacement and increment (device float64 or host arrays);
        P, K, F: device accumulators (P, F: [nDof] float64, K: CSR data [nnz]); they are added to,
        the caller zeroes them (nonlinearimplicitstatic.py:419).  Raises CutbackRequest like the
        reference's material points do."""
        U_np = self._as_device(U_np)
        dU = self._as_device(dU)
        time = None
        dT = 0.0
        if timeStep is not None:
            time = (float(timeStep.stepTime), float(timeStep.totalTime))
            dT = float(timeStep.timeIncrement)
        self.status.zero_()
        self.launch(U_np, dU, P, K, F, time, dT)
        if check:
            self.check_status()
        return P, K, F

    def assembleStiffnessCSR(self, K, host=False):
        """The assembled matrix in CSR form with the reference's pattern (CSRGenerator.updateCSR).

        host=False: torch sparse CSR tensor on the device (int32 indices); host=True: scipy
        csr_matrix, as the reference returns."""
        if host:
            import scipy.sparse as sp

            return sp.csr_matrix(
                (K.detach().double().cpu().numpy(), self.indices_host.copy(), self.indptr_host.copy()),
                shape=(self.nDof, self.nDof),
            )
        return torch.sparse_csr_tensor(self.indptr, self.indices, K, size=(self.nDof, self.nDof))

    def computeDistributedLoad(self, loadType, P, K, faceID, load, U, time, dTime):
        """Surface loads: the reference's displacement elements of this provider do not support them
        and raise (`elements/displacementelement/element.py:255-288`,
        `elements/displacementtlelement/element.py:311-344`); so does this."""
        raise Exception("Applying a distributed load is currently not possible with this element provider.")

    def computeBodyForce(self, P, force, elements=None):
        """Add the body force `force` [dim] of the given global element indices (default: all) to P
        (NIST.computeBodyForces, nonlinearimplicitstatic.py:520-557)."""
        force = (ctypes.c_double * 3)(*[float(f) for f in list(force)[: self.dim]], *([0.0] * (3 - self.dim)))
        if elements is not None:
            elements = np.asarray(elements, np.int64)
        for i, g in enumerate(self.groups):
            off, n = g._dev["offset"], len(g.conn)
            if elements is None:
                sel, ptr, cnt = None, None, n
            else:
                loc = elements[(elements >= off) & (elements < off + n)] - off
                if len(loc) == 0:
                    continue
                sel = _upload(loc, np.int32, self.device)
                ptr, cnt = ctypes.c_void_p(sel.data_ptr()), len(loc)
            L.check(
                self.lib.efe_body_force(
                    ctypes.byref(self.mesh), ctypes.byref(self._groups_c[i]), ptr, cnt, force,
                    ctypes.c_void_p(P.data_ptr()), self._stream(),
                ),
                "efe_body_force",
            )
            del sel
        return P

    def adjointTL(self, U, lam):
        """dL/dX [nNodes, dim] and per group dL/d(mu, K) [E, 2] for L = lam^T P(X, U, mu, K) of the
        total-Lagrangian Neo-Hooke groups (efe_adjoint_tl); lam must be zero on prescribed DOFs."""
        U = self._as_device(U)
        lam = self._as_device(lam)
        gX = torch.zeros((self.nNodes, self.dim), dtype=torch.float64, device=self.device)
        gP = []
        for i, g in enumerate(self.groups):
            gp = torch.zeros((len(g.conn), 2), dtype=torch.float64, device=self.device)
            L.check(
                self.lib.efe_adjoint_tl(
                    ctypes.byref(self.mesh), ctypes.byref(self._groups_c[i]), ctypes.c_void_p(U.data_ptr()),
                    ctypes.c_void_p(lam.data_ptr()), ctypes.c_void_p(gX.data_ptr()), ctypes.c_void_p(gp.data_ptr()),
                    self._stream(),
                ),
                "efe_adjoint_tl",
            )
            gP.append(gp)
        return gX, gP

    def adjointSmallStrain(self, group, stateBefore, dU, dUbar, Pbar=None, stateBarIn=None, stateBarOut=None,
                           gProps=None, gX=None):
        """Reverse mode of one small-strain pass of a group (efe_adjoint_small_strain): accumulates
        into dUbar [nDof], stateBarOut ([S, nPts], optional), gProps ([E, nProps], optional) and gX
        ([nNodes, dim], optional) the adjoints of dU, of the state before the increment, of the
        properties and of the nodal coordinates, given the seeds stateBarIn (adjoint of the new
        state) and Pbar (adjoint of the residual P).  Every buffer is checked here (dtype, device,
        contiguity, exact shape): the kernel writes through them."""
        d = self.groups[group]._dev

        def need(t, name, shape, required=False):
            if t is None:
                if required:
                    raise ValueError(f"adjointSmallStrain: {name} is required")
                return
            if (not isinstance(t, torch.Tensor) or t.dtype != torch.float64 or t.device != self.device
                    or tuple(t.shape) != tuple(shape) or not t.is_contiguous()):  # fmt: skip
                raise ValueError(f"adjointSmallStrain: {name} must be a contiguous float64 tensor of shape "
                                 f"{tuple(shape)} on {self.device}")  # fmt: skip

        S = tuple(d["stateRef"].shape)
        need(stateBefore, "stateBefore", S, True)
        need(stateBarIn, "stateBarIn", S)
        need(stateBarOut, "stateBarOut", S)
        need(dU, "dU", (self.nDof,), True)
        need(dUbar, "dUbar", (self.nDof,), True)
        need(Pbar, "Pbar", (self.nDof,))
        need(gProps, "gProps", tuple(d["props"].shape))
        need(gX, "gX", (self.nNodes, self.dim))

        def ptr(t):
            return None if t is None else ctypes.c_void_p(t.data_ptr())

        L.check(
            self.lib.efe_adjoint_small_strain(
                ctypes.byref(self.mesh), ctypes.byref(self._groups_c[group]), ptr(stateBefore), ptr(dU), ptr(Pbar),
                ptr(stateBarIn), ptr(stateBarOut), ptr(dUbar), ptr(gProps), ptr(gX), self._stream(),
            ),
            "efe_adjoint_small_strain",
        )  # fmt: skip

    # ------------------------------------------------------------------ state
    def acceptLastState(self):
        """acceptLastState of every element (element.py:373-379; TL element.py:454-461)."""
        L.check(self.lib.efe_accept_state(self._groups_c, len(self.groups), self._stream()), "efe_accept_state")

    def resetToLastValidState(self):
        """The reference elements do nothing here (element.py:381-384): stateTemp is recomputed from
        stateRef on every call."""

    def group_state(self, i, which="temp"):
        """[E, nInt, S] host copy of a group's state (reference element layout)."""
        g = self.groups[i]
        d = g._dev
        et = d["type"]
        s = d["stateTemp" if which == "temp" else "stateRef"]
        return s.T.reshape(len(g.conn), et.nInt, -1).cpu().numpy()

    def getResultArray(self, result, element, quadraturePoint, accepted=True):
        """Stress, strain or material state of one quadrature point (element.py:386-409)."""
        for g in self.groups:
            off = g._dev["offset"]
            if off <= element < off + len(g.conn):
                et = g._dev["type"]
                s = g._dev["stateRef" if accepted else "stateTemp"]
                col = (element - off) * et.nInt + quadraturePoint
                key = result.lower()
                if key == "stress":
                    return s[0:6, col].cpu().numpy()
                if key == "strain":
                    return s[6:12, col].cpu().numpy()
                if s.shape[0] > 12 and key in ("kappa", "energy", "materialstate"):
                    return s[12:, col].cpu().numpy()
                raise KeyError(result)
        raise IndexError(element)
