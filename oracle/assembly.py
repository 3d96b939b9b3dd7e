"""Global assembly: DOF numbering, VIJ pattern, canonical CSR, slot map, element loop.

Restates
* the DOF numbering of `DofManager._reserveSpaceForNodeFields` and
  `_locateNodeCouplingEntitiesInDofVector`
  (`edelweissfe/numerics/dofmanager.py:259-300, 445-471`): node-major,
  components interleaved, nodes in NodeField order;
* the VIJ (COO) pattern of `DofManager._initializeVIJPattern` (`dofmanager.py:522-557`):
  ``V[off_e + a*n + b]`` goes to global (row = idx[b], col = idx[a]);
* `CSRGenerator.__init__` / `updateCSR` (`edelweissfe/numerics/csrgenerator.pyx:47-115`):
  scipy canonical CSR (sorted, deduplicated, int32), slot map x[k], ``data[x[k]] += V[k]`` in COO order;
* `NIST.computeElements` (`edelweissfe/solvers/nonlinearimplicitstatic.py:794-849`):
  ``P[el] += Pe``, ``F[el] += abs(Pe)`` in element order.
"""

import numpy as np
import scipy.sparse as sp

from . import elements as elem
from . import library, materials
from .exceptions import CutbackRequest


def element_dofs(conn, node_dof, dim):
    """Global DOF indices [E, nN*dim] of every element, node-major, components interleaved."""
    return (node_dof[conn][:, :, None] + np.arange(dim)[None, None, :]).reshape(len(conn), -1)


def vij_pattern(dofs_list):
    """I, J (int64) of the VIJ system matrix (dofmanager.py:522-557) for a list of element DOF arrays."""
    Is, Js = [], []
    for dofs in dofs_list:
        n = dofs.shape[1]
        # I[a*n+b] = idx[b]; J[a*n+b] = idx[a]
        Is.append(np.broadcast_to(dofs[:, None, :], (len(dofs), n, n)).reshape(-1))
        Js.append(np.broadcast_to(dofs[:, :, None], (len(dofs), n, n)).reshape(-1))
    return np.concatenate(Is).astype(np.int64), np.concatenate(Js).astype(np.int64)


def csr_pattern(I, J, nDof):
    """Canonical CSR pattern as built by CSRGenerator.__init__ (csrgenerator.pyx:64-77)."""
    m = sp.csr_matrix((np.zeros(len(I)), (I, J)), (nDof, nDof))
    if not m.has_canonical_format:
        m.sum_duplicates()
    return m.indptr.astype(np.int32), m.indices.astype(np.int32)


def slot_map(I, J, indptr, indices):
    """x[k] = position of (I[k], J[k]) in the CSR data (csrgenerator.pyx:79-98)."""
    I = np.asarray(I)
    J = np.asarray(J)
    nnz = len(indices)
    rows = np.repeat(np.arange(len(indptr) - 1), np.diff(indptr))
    key_csr = rows.astype(np.int64) * (len(indptr) - 1) + indices
    key = I * (len(indptr) - 1) + J
    pos = np.searchsorted(key_csr, key)
    assert np.all(pos < nnz) and np.all(key_csr[pos] == key)
    return pos.astype(np.int32)


def update_csr(x, V, nnz):
    """data[:] = 0; data[x[k]] += V[k] sequentially (csrgenerator.pyx:100-115)."""
    return np.bincount(x, weights=V, minlength=nnz)


class Model:
    """A mesh with element groups, for the oracle.

    coords [nNodes, d]; node_dof [nNodes] (first DOF of each node, -1 for nodes without DOFs);
    groups: list of dicts with keys elType, kind, props [E,nP], conn [E,nN], thickness [E], order [E]
    (position of each element in the global element order)."""

    def __init__(self, coords, node_dof, nDof, groups):
        self.coords = np.asarray(coords, float)
        self.node_dof = np.asarray(node_dof, np.int64)
        self.nDof = int(nDof)
        self.dim = self.coords.shape[1]
        self.groups = groups
        nEl = sum(len(g["conn"]) for g in groups)
        self.nElements = nEl
        # element DOF lists in global element order
        self.dofs = [None] * nEl
        for g in groups:
            d = element_dofs(g["conn"], self.node_dof, self.dim)
            g["dofs"] = d
            for k, e in enumerate(g["order"]):
                self.dofs[e] = d[k]
        I, J = vij_pattern([d[None] for d in self.dofs])
        self.I, self.J = I, J
        self.indptr, self.indices = csr_pattern(I, J, self.nDof)
        self.x = slot_map(I, J, self.indptr, self.indices)
        self.vij_offsets = np.concatenate([[0], np.cumsum([len(d) ** 2 for d in self.dofs])])

    def initial_state(self):
        """Zero state per group (element.py:225 / displacementtlelement/element.py:283)."""
        out = []
        for g in self.groups:
            lib = library.get(g["elType"])
            S = 12 + materials.STATE_VARS[g["kind"]]
            st = dict(state=np.zeros((len(g["conn"]), lib["nInt"], S)))
            if lib["elClass"] == "DisplacementTLElement":
                d = lib["nSpatialDimensions"]
                st["Eold"] = np.zeros((len(g["conn"]), lib["nInt"], d, d))
            out.append(st)
        return out

    def compute_elements(self, U_np, dU, stateRef, time=None, dT=1.0):
        """NIST.computeElements + CSRGenerator.updateCSR for the whole model.

        Returns dict(P, F, Kdata, V, stateTemp (list per group), fail (list per group))."""
        nEl = self.nElements
        Pe_all = [None] * nEl
        V = np.zeros(self.vij_offsets[-1])
        stateTemp = []
        fails = []
        for g, st in zip(self.groups, stateRef):
            X = self.coords[g["conn"]]
            d = g["dofs"]
            lib = library.get(g["elType"])
            if lib["elClass"] == "DisplacementElement":
                Ke, Pe, sT, fail = elem.compute_small_strain(
                    g["elType"], g["kind"], g["props"], X, dU[d], st["state"], g["thickness"]
                )
                stateTemp.append(dict(state=sT))
            else:
                Ke, Pe, sT, Enew, fail = elem.compute_total_lagrangian(
                    g["elType"], g["kind"], g["props"], X, U_np[d], st["state"], st["Eold"], g["thickness"]
                )
                stateTemp.append(dict(state=sT, Eold=st["Eold"], Enew=Enew))
            fails.append(fail)
            for k, e in enumerate(g["order"]):
                Pe_all[e] = Pe[k]
                V[self.vij_offsets[e] : self.vij_offsets[e + 1]] = Ke[k].reshape(-1)
        # the reference raises at the first failing element in element order
        first = None
        for g, f in zip(self.groups, fails):
            if f.any():
                e = int(np.asarray(g["order"])[f].min())
                first = e if first is None else min(first, e)
        P = np.zeros(self.nDof)
        F = np.zeros(self.nDof)
        for e in range(nEl):  # nonlinearimplicitstatic.py:837-844
            P[self.dofs[e]] += Pe_all[e]
            F[self.dofs[e]] += np.abs(Pe_all[e])
        Kdata = update_csr(self.x, V, len(self.indices))
        return dict(P=P, F=F, Kdata=Kdata, V=V, stateTemp=stateTemp, fail=fails, first_failed_element=first)

    def body_force(self, load, elements=None):
        """External load vector of a body force `load` on the given global element indices (all by
        default): NIST.computeBodyForces (`solvers/nonlinearimplicitstatic.py:520-557`) scattering
        each element's computeBodyForce (`elem.body_force`) into the DOF vector."""
        P = np.zeros(self.nDof)
        wanted = None if elements is None else set(int(e) for e in elements)
        for g in self.groups:
            order = np.asarray(g["order"])
            pick = np.arange(len(order)) if wanted is None else np.array(
                [k for k, e in enumerate(order) if int(e) in wanted], np.int64)  # fmt: skip
            if len(pick) == 0:
                continue
            X = self.coords[np.asarray(g["conn"])[pick]]
            th = np.broadcast_to(np.asarray(g["thickness"], float), (len(order),))[pick]
            Pe = elem.body_force(g["elType"], X, load, th)
            for j, e in enumerate(order[pick]):
                P[self.dofs[e]] += Pe[j]
        return P

    def compute_elements_or_raise(self, U_np, dU, stateRef, time=None, dT=1.0):
        r = self.compute_elements(U_np, dU, stateRef, time, dT)
        if r["first_failed_element"] is not None:
            raise CutbackRequest("material point failed in element %d" % r["first_failed_element"], 0.5)
        return r

    @staticmethod
    def accept_state(stateTemp):
        """acceptLastState (element.py:373-379; TL element.py:454-461): temp -> ref, TL also E_old = E."""
        out = []
        for st in stateTemp:
            d = dict(state=st["state"].copy())
            if "Enew" in st:
                d["Eold"] = st["Enew"].copy()
            out.append(d)
        return out
