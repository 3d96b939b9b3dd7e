"""The adapter from reference objects to the GPU path's arrays (edelweissfe_gb300.integration).

Needs the reference source tree, named by the EDELWEISSFE_ROOT environment variable; skipped when
it is unset.  No GPU: the extracted arrays are checked against the reference's own DofManager and,
through the oracle, against the reference's computeElements.
"""

import os
import sys

import numpy as np
import pytest

REF = os.environ.get("EDELWEISSFE_ROOT", "")
pytestmark = pytest.mark.skipif(not REF or not os.path.isdir(os.path.join(REF, "edelweissfe")),
                                reason="EDELWEISSFE_ROOT (the reference source tree) is not set")  # fmt: skip


@pytest.fixture(scope="module")
def ref():
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    import make_golden

    make_golden.setup_reference(REF)
    return make_golden


def _prepared(mg, dim, gen, lines, et, kind, props, jit, h, seed, lo, hi):
    from edelweissfe.journal.journal import Journal
    from edelweissfe.numerics.dofmanager import DofManager
    from edelweissfe.sets.nodeset import NodeSet

    model = mg.make_model(dim, gen, lines, et, jit, h, seed, lo, hi)
    model.nodeSets["all"] = NodeSet("all", list(model.nodes.values()))
    cls = mg.material_class(kind)
    for el in model.elements.values():
        el.setProperties(np.array([0.7]))
        el.initializeElement()
        el.setMaterial(cls(np.array(props, float)))
    model._prepareVariablesAndFields(Journal(verbose=False))
    dm = DofManager(model.nodeFields.values(), [], model.elements.values(), [], model.nodeSets.values())
    return model, dm


@pytest.mark.parametrize(
    "dim,gen,lines,et,kind,props",
    [
        (3, "boxGen", ["nX=3", "nY=2", "nZ=2"], "C3D8", "vonmises", [210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0]),
        (2, "planeRectQuad", ["nX=4", "nY=3"], "CPE8RTL", "neohookewa", [1000.0, 10000.0]),
        (3, "boxGen", ["nX=2", "nY=1", "nZ=1"], "C3D20", "linearelastic", [210000.0, 0.3]),
    ],
)
def test_arrays_from_reference_reproduce_compute_elements(ref, dim, gen, lines, et, kind, props):
    from edelweissfe.config.timing import createTimingDict
    from edelweissfe.numerics.csrgenerator import CSRGenerator
    from edelweissfe.solvers.nonlinearimplicitstatic import NIST
    from edelweissfe.timesteppers.timestep import TimeStep

    from edelweissfe_gb300.integration import arrays_from_reference
    from oracle.assembly import Model

    h = [1.0 / 3] * dim
    model, dm = _prepared(ref, dim, gen, lines, et, kind, props, 0.1, h, 5, [0] * dim, [1] * dim)
    coords, nodeDof, nDof, groups = arrays_from_reference(model.elements.values(), dm)
    assert len(groups) == 1 and groups[0].elType == et and groups[0].material == kind
    g = groups[0]
    el_dofs = (nodeDof[g.conn][:, :, None] + np.arange(dim)).reshape(len(g.conn), -1)
    assert np.array_equal(el_dofs, np.array([dm.idcsOfElementsInDofVector[el] for el in model.elements.values()]))
    # the oracle on the extracted arrays reproduces the reference's element pass
    rng = np.random.default_rng(0)
    U = dm.constructDofVector()
    U[:] = rng.uniform(-1, 1, nDof) * (0.02 if kind.startswith("neo") else 2e-3)
    P, F, K = dm.constructDofVector(), dm.constructDofVector(), dm.constructVIJSystemMatrix()
    s = type("S", (), {"computationTimes": createTimingDict()})()
    P, K, F = NIST.computeElements(s, model.elements, U, U, P, K, F, TimeStep(1, 1.0, 1.0, 1.0, 1.0, 1.0))
    Kc = CSRGenerator(K).updateCSR(K)
    om = Model(coords, nodeDof, nDof, [dict(elType=g.elType, kind=g.material, props=g.props, conn=g.conn,
                                            thickness=g.thickness, order=np.arange(len(g.conn)))])  # fmt: skip
    r = om.compute_elements(np.asarray(U), np.asarray(U), om.initial_state())
    assert np.array_equal(om.indptr, Kc.indptr) and np.array_equal(om.indices, Kc.indices)
    assert np.abs(r["P"] - P).max() <= 1e-12 * np.abs(P).max()
    assert np.abs(r["Kdata"] - Kc.data).max() <= 1e-12 * np.abs(Kc.data).max()


def test_distributed_loads_raise_like_the_reference():
    """The reference's displacement elements of the edelweiss provider raise on surface loads; the
    assembler's computeDistributedLoad does the same (no device needed to reach the raise)."""
    from edelweissfe_gb300.assembly import GPUAssembler

    with pytest.raises(Exception, match="distributed load is currently not possible"):
        GPUAssembler.computeDistributedLoad(None, "pressure", None, None, 1, [1.0], None, (0.0, 0.0), 0.1)


@pytest.mark.parametrize(
    "dim,gen,lines,et,kind,props",
    [
        (3, "boxGen", ["nX=2", "nY=2", "nZ=1"], "C3D8", "vonmises", [210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0]),
        (2, "planeRectQuad", ["nX=3", "nY=2"], "CPE8RTL", "neohookewa", [1000.0, 10000.0]),
        (3, "boxGen", ["nX=2", "nY=1", "nZ=1"], "C3D8TL", "neohookewb", [1000.0, 10000.0]),
        (3, "boxGen", ["nX=2", "nY=1", "nZ=1"], "C3D8TL", "vonmises", [210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0]),
    ],
)
def test_write_back_reproduces_the_reference_state(ref, dim, gen, lines, et, kind, props):
    """write_back_state puts an accepted state in the device layout ([field][element * nInt + qp])
    into the reference elements: after the reference's own computeElements + acceptLastState, and the
    oracle's pass over the extracted arrays written back in its place, every element's _stateVarsRef
    agrees with the reference's (1e-12), in place (persistent result views taken before see it)."""
    from types import SimpleNamespace

    import torch

    from edelweissfe.config.timing import createTimingDict
    from edelweissfe.solvers.nonlinearimplicitstatic import NIST
    from edelweissfe.timesteppers.timestep import TimeStep

    from edelweissfe_gb300.assembly import GPUAssembler
    from edelweissfe_gb300.integration import arrays_from_reference, read_state_from_reference, write_back_state
    from oracle.assembly import Model

    h = [1.0 / 3] * dim
    model, dm = _prepared(ref, dim, gen, lines, et, kind, props, 0.1, h, 6, [0] * dim, [1] * dim)
    elements = list(model.elements.values())
    coords, nodeDof, nDof, groups = arrays_from_reference(elements, dm)
    rng = np.random.default_rng(1)
    U = dm.constructDofVector()
    U[:] = rng.uniform(-1, 1, nDof) * (0.02 if kind.startswith("neo") else 4e-3)
    P, F, K = dm.constructDofVector(), dm.constructDofVector(), dm.constructVIJSystemMatrix()
    s = type("S", (), {"computationTimes": createTimingDict()})()
    NIST.computeElements(s, model.elements, U, U, P, K, F, TimeStep(1, 1.0, 1.0, 1.0, 1.0, 1.0))
    for el in elements:
        el.acceptLastState()
    want = [el._stateVarsRef.copy() for el in elements]
    want_E = [np.array(el._Eold, copy=True) for el in elements] if et.endswith("TL") else None
    assert max(np.abs(w).max() for w in want) > 0
    views = [el.getResultArray("stress", 0) for el in elements]
    collector = None
    try:  # the reference's own collector (compiled from its .pyx for the fixtures), when importable
        from edelweissfe.utils.elementresultcollector import ElementResultCollector

        collector = ElementResultCollector(elements, range(elements[0]._nInt), "stress")
    except ImportError:
        pass
    for el in elements:  # forget the reference's state
        el._stateVarsRef[...] = 0.0
        for row in el._stateVarsTemp:
            row[...] = 0.0
    g = groups[0]
    om = Model(coords, nodeDof, nDof, [dict(elType=g.elType, kind=g.material, props=g.props, conn=g.conn,
                                            thickness=g.thickness, order=np.arange(len(g.conn)))])  # fmt: skip
    temp = om.compute_elements(np.asarray(U), np.asarray(U), om.initial_state())["stateTemp"][0]
    st = temp["state"]
    E, nInt, S = st.shape
    fake = SimpleNamespace(groups=[SimpleNamespace(conn=g.conn, _dev={"offset": 0, "type": SimpleNamespace(nInt=nInt),
                                                                       "stateRef": torch.from_numpy(
                                                                           st.reshape(E * nInt, S).T.copy())})])  # fmt: skip
    fake.group_state = lambda i, which: GPUAssembler.group_state(fake, i, which)
    if want_E is not None:  # the device's aux fields: accepted E as [E11, E22, E33, E12, E23, E13]
        En = temp["Enew"]  # [E, nInt, d, d]
        d = En.shape[-1]
        aux = np.zeros((E * nInt, 6))
        for f, (i, j) in enumerate(((0, 0), (1, 1), (2, 2), (0, 1), (1, 2), (0, 2))):
            if i < d and j < d:
                aux[:, f] = En[:, :, i, j].reshape(-1)
        fake.groups[0]._dev["auxRef"] = torch.from_numpy(aux.T.copy())
        fake.groups[0]._dev["auxTemp"] = torch.from_numpy(aux.T.copy())
        for el in elements:
            el._Eold = np.zeros_like(el._Eold)
    write_back_state(fake, elements)
    if want_E is not None:
        for el, w in zip(elements, want_E):
            assert np.abs(el._Eold - w).max() <= 1e-14 * max(np.abs(np.array(want_E)).max(), 1e-300)
    scale = max(np.abs(w).max() for w in want)
    for el, w, v in zip(elements, want, views):
        assert np.abs(el._stateVarsRef - w).max() <= 1e-12 * scale
        assert np.array_equal(np.asarray(el._stateVarsTemp), el._stateVarsRef)
        assert np.array_equal(v, el._stateVarsRef[0][0:6])  # the view taken before the write-back
    if collector is not None:  # the reference's field-output path reads the written-back state
        got = np.asarray(collector.getCurrentResults())
        assert np.abs(got - np.array([w[:, 0:6] for w in want])).max() <= 1e-12 * scale
    # and back: a state set on the element objects (as a step action does) reaches the device layout
    for el in elements:
        el._stateVarsRef[:, 0] = 7.0
    g0 = fake.groups[0]._dev
    g0["stateTemp"] = torch.zeros_like(g0["stateRef"])
    if want_E is not None:  # and the accepted E back into the aux fields
        aux_before = g0["auxRef"].clone()
        g0["auxRef"].zero_()
    read_state_from_reference(fake, elements)
    if want_E is not None:
        assert torch.allclose(g0["auxRef"], aux_before, rtol=0, atol=0)
    assert torch.equal(g0["stateRef"], g0["stateTemp"])
    back = GPUAssembler.group_state(fake, 0, "ref")
    assert np.array_equal(back, np.stack([el._stateVarsRef for el in elements]))
    assert bool((g0["stateRef"][0] == 7.0).all())


@pytest.mark.parametrize(
    "dim,gen,lines,et",
    [
        (2, "planeRectQuad", ["nX=3", "nY=2"], "CPE4"),
        (2, "planeRectQuad", ["nX=3", "nY=2"], "CPS8R"),
        (3, "boxGen", ["nX=2", "nY=2", "nZ=1"], "C3D8"),
        (3, "boxGen", ["nX=2", "nY=1", "nZ=1"], "C3D20"),
        (3, "boxGen", ["nX=2", "nY=1", "nZ=1"], "C3D20TL"),
    ],
)
def test_oracle_body_force_matches_reference(ref, dim, gen, lines, et):
    """oracle.elements.body_force / Model.body_force against the reference's computeBodyForce of
    every element of a jittered mesh (computeNOperator at the library points, J as the reference
    forms it -- the Hexa20 fit included -- section thickness in 2D), scattered as
    NIST.computeBodyForces does."""
    from edelweissfe_gb300.integration import arrays_from_reference
    from oracle.assembly import Model

    kind, props = ("linearelastic", [210000.0, 0.3]) if not et.endswith("TL") else ("neohookewa", [1000.0, 10000.0])
    model, dm = _prepared(ref, dim, gen, lines, et, kind, props, 0.15, [1.0 / 3] * dim, 7, [0] * dim, [1] * dim)
    elements = list(model.elements.values())
    load = np.array([1.5, -2.0, 0.7][:dim])
    want = dm.constructDofVector()
    for el in elements:
        Pe = np.zeros(el.nDof)
        el.computeBodyForce(Pe, None, load, None, np.array([0.0, 0.0]), 1.0)
        want[dm.idcsOfElementsInDofVector[el]] += Pe
    coords, nodeDof, nDof, groups = arrays_from_reference(elements, dm)
    om = Model(coords, nodeDof, nDof, [dict(elType=g.elType, kind=g.material, props=g.props, conn=g.conn,
                                            thickness=g.thickness, order=np.arange(len(g.conn))) for g in groups])  # fmt: skip
    got = om.body_force(load)
    assert np.abs(got - np.asarray(want)).max() <= 1e-14 * np.abs(np.asarray(want)).max()
    half = om.body_force(load, elements=range(0, len(elements), 2))  # a subset, as an element set
    want_half = dm.constructDofVector()
    for el in elements[0::2]:
        Pe = np.zeros(el.nDof)
        el.computeBodyForce(Pe, None, load, None, np.array([0.0, 0.0]), 1.0)
        want_half[dm.idcsOfElementsInDofVector[el]] += Pe
    assert np.abs(half - np.asarray(want_half)).max() <= 1e-14 * np.abs(np.asarray(want)).max()


def test_result_collector_matches_the_reference_collector(ref):
    """results.ElementResultCollector over a state in the device layout against the reference's own
    ElementResultCollector (utils/elementresultcollector.pyx) over element objects holding the same
    state: stress and strain tables for a scattered element list and all points, and the material
    state against the element arrays."""
    from types import SimpleNamespace

    import torch

    from edelweissfe.config.timing import createTimingDict
    from edelweissfe.solvers.nonlinearimplicitstatic import NIST
    from edelweissfe.timesteppers.timestep import TimeStep

    from edelweissfe_gb300.integration import arrays_from_reference
    from edelweissfe_gb300.results import ElementResultCollector

    try:
        from edelweissfe.utils.elementresultcollector import ElementResultCollector as RefCollector
    except ImportError:
        pytest.skip("the reference's compiled collector is not importable")
    model, dm = _prepared(ref, 3, "boxGen", ["nX=3", "nY=2", "nZ=2"], "C3D8", "vonmises",
                          [210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0], 0.1, [1 / 3, 0.5, 0.5], 4, [0] * 3, [1] * 3)  # fmt: skip
    elements = list(model.elements.values())
    rng = np.random.default_rng(3)
    U = dm.constructDofVector()
    U[:] = rng.uniform(-1, 1, dm.nDof) * 6e-3
    P, F, K = dm.constructDofVector(), dm.constructDofVector(), dm.constructVIJSystemMatrix()
    s = type("S", (), {"computationTimes": createTimingDict()})()
    NIST.computeElements(s, model.elements, U, U, P, K, F, TimeStep(1, 1.0, 1.0, 1.0, 1.0, 1.0))
    for el in elements:
        el.acceptLastState()
    _, _, _, groups = arrays_from_reference(elements, dm)
    g = groups[0]
    nInt = elements[0]._nInt
    host = np.stack([el._stateVarsRef for el in elements])  # [E, nInt, S]
    soa = torch.from_numpy(np.ascontiguousarray(host.reshape(len(elements) * nInt, -1).T))
    g._dev.update(offset=0, type=SimpleNamespace(nInt=nInt), stateRef=soa, stateTemp=soa.clone())
    fake = SimpleNamespace(groups=[g], device=torch.device("cpu"))
    pick = rng.permutation(len(elements))[:7]
    for result in ("stress", "strain"):
        ours = ElementResultCollector(fake, pick, range(nInt), result).getCurrentResults()
        theirs = np.asarray(RefCollector([elements[i] for i in pick], range(nInt), result).getCurrentResults())
        assert ours.shape == theirs.shape and np.array_equal(ours, theirs)
    kappa = ElementResultCollector(fake, pick, range(nInt), "kappa").getCurrentResults()
    assert np.array_equal(kappa[..., 0], host[pick][:, :, 12]) and kappa.max() > 0
