"""Wiring the GPU element path into an EdelweissFE run.

EdelweissFE extends its Newton solver by subclassing `NIST` and overriding `computeElements`
(the pattern of `solvers/nonlinearimplicitstaticparallelmk2.pyx:50,111`), registered in
`config/solvers.py:48-53` (`solverLibrary`) and selected with ``*solver, solver=<name>``.
`make_nist_gpu` builds such a subclass around `GPUAssembler`; `arrays_from_reference` converts the
reference's element objects and DofManager into the arrays the GPU path takes.

The reference package is not imported here: the functions take its objects and read only their
public state (element type tables, nodes, material parameters, section thickness, DOF indices).
"""

import numpy as np

from . import library

_MATERIALS = {
    "LinearElasticMaterial": "linearelastic",
    "VonMisesMaterial": "vonmises",
    "NeoHookeanWaMaterial": "neohookewa",
    "NeoHookeanWbMaterial": "neohookewb",
    "NeoHookeanWcMaterial": "neohookewc",
}


def element_type_of(el):
    """Library name of a reference element from its tables (class, nodes, dimension, points, plane flag)."""
    tl = type(el).__name__ == "DisplacementTLElement"
    if type(el).__name__ not in ("DisplacementElement", "DisplacementTLElement"):
        raise NotImplementedError(f"{type(el).__name__} is not an edelweiss displacement element")
    for name, et in library.ELEMENT_TYPES.items():
        if et.totalLagrangian != tl or et.nNodes != el.nNodes or et.dim != el.nSpatialDimensions:
            continue
        if et.nInt != el._nInt:
            continue
        plane = {True: "pe", False: "ps", None: "solid"}[el.planeStrain]
        if plane == {1: "pe", 2: "ps", 0: "solid"}[et.plane]:
            return name
    raise KeyError("no matching element type")


def material_of(mat):
    """(material name, property vector) of a reference material object (materials/*)."""
    name = _MATERIALS.get(type(mat).__name__)
    if name is None:
        raise NotImplementedError(f"{type(mat).__name__} is not supported by the GPU element path")
    if name == "linearelastic":
        return name, [mat._E, mat._v]
    if name == "vonmises":
        return name, [mat._E, mat._v, mat.yieldStress, mat.HLin, mat.deltaYieldStress, mat.delta]
    return name, list(np.asarray(mat.materialProperties, float)[:2])


def arrays_from_reference(elements, dofManager):
    """coords, nodeDof, nDof, groups for a list of reference elements (in the model's element order)."""
    from .assembly import ElementGroup

    elements = list(elements)
    nodes = {}
    for el in elements:
        for n in el.nodes:
            nodes.setdefault(id(n), n)
    order = list(nodes.values())
    pos = {id(n): i for i, n in enumerate(order)}
    dim = elements[0].nSpatialDimensions
    coords = np.array([n.coordinates for n in order], float)
    nodeDof = -np.ones(len(order), np.int64)
    recs = []
    for el in elements:
        idx = np.asarray(dofManager.idcsOfElementsInDofVector[el])
        conn = [pos[id(n)] for n in el.nodes]
        first = idx[0::dim]
        if not np.array_equal(idx, (first[:, None] + np.arange(dim)).ravel()):
            raise NotImplementedError("element DOFs are not node-major with interleaved components")
        nodeDof[conn] = first
        kind, props = material_of(el.material)
        recs.append((element_type_of(el), kind, props, conn, float(getattr(el, "_t", 1.0))))
    groups = []
    start = 0
    for e in range(1, len(recs) + 1):
        if e == len(recs) or recs[e][:2] != recs[start][:2] or len(recs[e][2]) != len(recs[start][2]):
            chunk = recs[start:e]
            groups.append(ElementGroup(chunk[0][0], chunk[0][1], np.array([r[2] for r in chunk]),
                                       np.array([r[3] for r in chunk]), np.array([r[4] for r in chunk])))  # fmt: skip
            start = e
    return coords, nodeDof, int(dofManager.nDof), groups


def write_back_state(asm, elements):
    """Copy the assembler's accepted quadrature-point state into the reference element objects, in
    place: `_stateVarsRef` and the rows of `_stateVarsTemp` ([nInt][12 + m] per element,
    `elements/displacementelement/element.py:222-235`, `elements/displacementtlelement/element.py`
    likewise), whose rows hold the same [stress, strain, material state] in the element family's
    Voigt order as the device state; total-Lagrangian elements also get the accepted Green-Lagrange
    strain (`_Eold` and `_E`, displacementtlelement/element.py:215-216, 454-461) from the device's
    aux fields.  Everything that reads results from the element objects --
    the persistent views of `getResultArray` (element.py:386-409), the reference's
    ElementResultCollector and field outputs, the output managers -- then sees the GPU solution.
    `elements`: the reference elements in the assembler's element order."""
    elements = list(elements)
    for gi, g in enumerate(asm.groups):
        off = g._dev["offset"]
        S = asm.group_state(gi, "ref")  # [E, nInt, 12 + m]
        Eold = _aux_tensors(g, S.shape[0], S.shape[1])
        for k in range(S.shape[0]):
            el = elements[off + k]
            if el._stateVarsRef.shape != S.shape[1:]:
                raise ValueError(f"element {off + k}: state shape {el._stateVarsRef.shape} != {S.shape[1:]}")
            el._stateVarsRef[...] = S[k]
            for q in range(S.shape[1]):  # an array, or a list of rows once computeYourself ran (element.py:320)
                el._stateVarsTemp[q][...] = S[k, q]
            if Eold is not None and hasattr(el, "_Eold"):  # TL: E_old = E after acceptance (:454-461)
                d = el._Eold.shape[-1]
                el._Eold = Eold[k, :, :d, :d].copy()
                el._E = Eold[k, :, :d, :d].copy()


# device aux fields of total-Lagrangian groups: the accepted Green-Lagrange strain per point as
# [E11, E22, E33, E12, E23, E13] (tensor components), [6][element * nInt + qp]
_AUX = ((0, 0), (1, 1), (2, 2), (0, 1), (1, 2), (0, 2))


def _aux_tensors(g, nEl, nInt):
    """[E, nInt, 3, 3] accepted Green-Lagrange strains of a total-Lagrangian group, or None."""
    aux = g._dev.get("auxRef")
    if aux is None:
        return None
    a = aux.cpu().numpy().T.reshape(nEl, nInt, 6)
    T = np.zeros((nEl, nInt, 3, 3))
    for f, (i, j) in enumerate(_AUX):
        T[:, :, i, j] = a[:, :, f]
        T[:, :, j, i] = a[:, :, f]
    return T


def read_state_from_reference(asm, elements):
    """The inverse of write_back_state: every reference element's `_stateVarsRef` (and, for
    total-Lagrangian elements, `_Eold`) into the assembler's accepted state (stateRef and stateTemp,
    [field][element * nInt + qp]; auxRef and auxTemp).  With the
    write-back on, the element objects hold the accepted state at every step boundary, so reading
    them at a step start picks up exactly what the reference's own elements would compute from,
    including states set by step actions (`stepactions/setfield.py:95`, through the field outputs'
    setResults)."""
    import torch

    elements = list(elements)
    for g in asm.groups:
        d = g._dev
        off, n, nInt = d["offset"], len(g.conn), d["type"].nInt
        host = np.stack([np.asarray(elements[off + k]._stateVarsRef, float) for k in range(n)])  # [E, nInt, S]
        if host.shape[1] != nInt or host.shape[2] != d["stateRef"].shape[0]:
            raise ValueError(f"reference state shape {host.shape[1:]} != device ({nInt}, {d['stateRef'].shape[0]})")
        soa = torch.from_numpy(np.ascontiguousarray(host.reshape(n * nInt, -1).T)).to(d["stateRef"])
        d["stateRef"].copy_(soa)
        d["stateTemp"].copy_(soa)
        if d.get("auxRef") is not None and hasattr(elements[off], "_Eold"):  # TL: the accepted E_old
            a = np.zeros((n, nInt, 6))
            for k in range(n):
                Eo = np.asarray(elements[off + k]._Eold, float)  # [nInt, d, d]
                for f, (i, j) in enumerate(_AUX):
                    if i < Eo.shape[-1] and j < Eo.shape[-1]:
                        a[k, :, f] = Eo[:, i, j]
            aux = torch.from_numpy(np.ascontiguousarray(a.reshape(n * nInt, 6).T)).to(d["auxRef"])
            d["auxRef"].copy_(aux)
            d["auxTemp"].copy_(aux)


def same_layout(asm, nodeDof, nDof, groups):
    """True when an assembler was built for the same DOF map, elements, materials and properties as
    freshly extracted arrays (NIST builds a new DofManager every step, nonlinearimplicitstatic.py:134,
    usually for the same numbering)."""
    if asm.nDof != nDof or not np.array_equal(asm.nodeDof_host, nodeDof) or len(asm.groups) != len(groups):
        return False
    return all(a.elType == b.elType and a.material == b.material and np.array_equal(a.conn, b.conn)
               and np.array_equal(np.asarray(a.props), np.asarray(b.props))
               and np.array_equal(np.asarray(a.thickness), np.asarray(b.thickness))
               for a, b in zip(asm.groups, groups))  # fmt: skip


def make_nist_gpu(NIST, precision="fp64", writeBackState=True, assemblerClass=None):
    """A NIST subclass whose element loop and CSR assembly run on the GPU.

    The reference's solveIncrement keeps its host DOF vectors: computeElements copies U_np and dU to
    the device, runs the element pass, and adds P and |P_e| back into the host vectors; the
    tangent stays on the device until assembleStiffnessCSR returns it as the scipy CSR matrix the
    linear solvers expect.  The assembler (pattern, geometry, device state) is kept across steps
    while the extracted mesh, DOF map and materials stay the same (NIST builds a new DofManager
    every step).  Accepting a converged increment (FEModel.advanceToTime) also accepts
    the device state and, with writeBackState, copies it into the reference element objects
    (write_back_state) before the field outputs and output managers of that increment read them;
    each later step then starts from the element objects' state (read_state_from_reference), as
    the reference's own elements would.  A material point's cutback request reaches the reference's
    solveStep as the CutbackRequest class that NIST's module catches
    (`solvers/nonlinearimplicitstatic.py:48-50, 247`), with the same message and cutback size.
    assemblerClass: the assembler built from the extracted arrays (default GPUAssembler; the CPU
    tests substitute one with the same interface to run the subclass's control flow)."""
    import sys

    import torch

    from .assembly import GPUAssembler
    from .exceptions import CutbackRequest

    Assembler = assemblerClass or GPUAssembler
    RefCutbackRequest = getattr(sys.modules.get(NIST.__module__), "CutbackRequest", None)

    class NISTGPU(NIST):
        identification = "NISTGPU"

        def _gpu(self, elements):
            old = getattr(self, "_gpuAssembler", None)
            if old is None or self._gpuDofManager is not self.theDofManager:
                coords, nodeDof, nDof, groups = arrays_from_reference(elements.values(), self.theDofManager)
                if old is None or not same_layout(old, nodeDof, nDof, groups):
                    if old is not None and not writeBackState:
                        raise NotImplementedError("the model changed between steps; carrying the GPU state over "
                                                  "needs writeBackState=True")  # fmt: skip
                    self._gpuAssembler = Assembler(coords, nodeDof, nDof, groups, precision=precision)
                    if old is not None:  # the element objects hold the accepted state (write-back)
                        read_state_from_reference(self._gpuAssembler, elements.values())
                self._gpuDofManager = self.theDofManager
                self._gpuElements = list(elements.values())
            return self._gpuAssembler

        def computeElements(self, elements, U_np, dU, P, K, F, timeStep):
            asm = self._gpu(elements)
            Pd, Fd = asm.constructDofVector(), asm.constructDofVector()
            self._gpuK = asm.constructSystemMatrix()
            try:
                asm.computeElements(elements, torch.as_tensor(np.asarray(U_np)), torch.as_tensor(np.asarray(dU)), Pd,
                                    self._gpuK, Fd, timeStep)  # fmt: skip
            except CutbackRequest as e:
                if RefCutbackRequest is None:
                    raise
                raise RefCutbackRequest(str(e), e.cutbackSize) from e
            P += Pd.cpu().numpy()
            F += Fd.cpu().numpy()
            return P, K, F

        def assembleStiffnessCSR(self, K):
            return self._gpuAssembler.assembleStiffnessCSR(self._gpuK, host=True)

        def solveStep(self, step, model, fieldOutputController, outputmanagers):
            if getattr(model, "constraints", None):
                # assembleConstraints (nonlinearimplicitstatic.py:851-901) adds the constraints' terms
                # to the host VIJ matrix, which this subclass does not assemble: the returned GPU
                # tangent would lack them
                raise NotImplementedError("NISTGPU: models with constraints are not supported (the GPU tangent "
                                          "carries element contributions only)")  # fmt: skip
            advance = model.advanceToTime

            def advanceToTime(time):
                advance(time)
                if getattr(self, "_gpuAssembler", None) is not None:
                    self._gpuAssembler.acceptLastState()
                    if writeBackState:
                        write_back_state(self._gpuAssembler, self._gpuElements)

            model.advanceToTime = advanceToTime
            if writeBackState and getattr(self, "_gpuAssembler", None) is not None:
                read_state_from_reference(self._gpuAssembler, self._gpuElements)
            try:
                return super().solveStep(step, model, fieldOutputController, outputmanagers)
            finally:
                model.advanceToTime = advance

    return NISTGPU
