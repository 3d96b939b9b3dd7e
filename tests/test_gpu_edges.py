"""Edge cases of the element pass through the C ABI: empty groups, single-element meshes (against
the oracle), an inverted element at set-up, a zero increment, non-finite input and the
reference's unsupported combination (plane-stress hyperelasticity)."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

VM = [210e3, 0.3, 250.0, 1000.0, 0.0, 0.0]


def _pass(asm, U, dU):
    P, F, K = asm.constructDofVector(), asm.constructDofVector(), asm.constructSystemMatrix()
    asm.computeElements(None, torch.as_tensor(U, device=asm.device), torch.as_tensor(dU, device=asm.device), P, K, F)
    return P.cpu().numpy(), F.cpu().numpy(), K.double().cpu().numpy()


def test_empty_group_changes_nothing():
    from edelweissfe_gb300 import ElementGroup, GPUAssembler, meshes

    coords, conn, nodeDof, nDof = meshes.box(2, 2, 1, nNodes=8)
    dU = np.random.default_rng(0).normal(0, 1e-3, nDof)
    ref = GPUAssembler(coords, nodeDof, nDof, [ElementGroup("C3D8", "vonmises", VM, conn)])
    both = GPUAssembler(coords, nodeDof, nDof, [ElementGroup("C3D8", "vonmises", VM, conn),
                                                ElementGroup("C3D8", "linearelastic", [1.0, 0.3], conn[:0])])  # fmt: skip
    # P, F and K are accumulated with atomics, whose order varies between runs: compare at rounding level
    for a, b in zip(_pass(ref, dU, dU), _pass(both, dU, dU)):
        assert np.abs(a - b).max() <= 1e-12 * np.abs(a).max()
    both.acceptLastState()
    # a model whose only group is empty: a pattern without entries, zero outputs, no error
    none = GPUAssembler(coords, nodeDof, nDof, [ElementGroup("C3D8", "vonmises", VM, conn[:0])])
    assert none.nnz == 0
    P, F, K = _pass(none, dU, dU)
    assert not P.any() and not F.any() and K.size == 0
    none.acceptLastState()


@pytest.mark.parametrize("elType,kind,props", [("C3D20", "vonmises", VM), ("CPE4", "vonmises", VM),
                                               ("C3D8TL", "neohookewa", [400.0, 4000.0]),
                                               ("CPE8RTL", "neohookewb", [400.0, 4000.0])])
def test_single_element_matches_oracle(elType, kind, props):
    from edelweissfe_gb300 import ElementGroup, GPUAssembler, meshes
    from oracle.assembly import Model

    dim = 3 if elType.startswith("C3D") else 2
    nn = {"C3D20": 20, "CPE4": 4, "C3D8TL": 8, "CPE8RTL": 8}[elType]
    if dim == 3:
        coords, conn, nodeDof, nDof = meshes.box(1, 1, 1, nNodes=nn)
    else:
        coords, conn, nodeDof, nDof = meshes.rect(1, 1, nNodes=nn)
    rng = np.random.default_rng(1)
    coords = coords + rng.uniform(-0.05, 0.05, coords.shape)
    U = rng.normal(0, 3e-3, nDof)
    asm = GPUAssembler(coords, nodeDof, nDof, [ElementGroup(elType, kind, props, conn, 1.0)])
    P, F, K = _pass(asm, U, U)
    g = dict(elType=elType, kind=kind, props=np.tile(props, (1, 1)), conn=conn.astype(np.int64),
             thickness=np.ones(1), order=np.arange(1))  # fmt: skip
    m = Model(coords, nodeDof, nDof, [g])
    r = m.compute_elements(U, U, m.initial_state())
    assert np.abs(P - r["P"]).max() <= 1e-12 * np.abs(r["P"]).max()
    assert np.abs(F - r["F"]).max() <= 1e-12 * np.abs(r["F"]).max()
    assert np.abs(K - r["Kdata"]).max() <= 1e-12 * np.abs(r["Kdata"]).max()


def test_inverted_element_is_reported_at_setup():
    from edelweissfe_gb300 import ElementGroup, GPUAssembler, meshes

    coords, conn, nodeDof, nDof = meshes.box(3, 1, 1, nNodes=8)
    bad = conn.copy()
    bad[2] = bad[2][[4, 5, 6, 7, 0, 1, 2, 3]]  # element 2 turned inside out
    with pytest.raises(ValueError, match="element 2 has a non-positive Jacobian"):
        GPUAssembler(coords, nodeDof, nDof, [ElementGroup("C3D8", "linearelastic", [1.0, 0.3], bad)])


def test_zero_increment_keeps_state_and_gives_elastic_tangent():
    from edelweissfe_gb300 import ElementGroup, GPUAssembler, meshes

    coords, conn, nodeDof, nDof = meshes.box(2, 1, 1, nNodes=8)
    asm = GPUAssembler(coords, nodeDof, nDof, [ElementGroup("C3D8", "vonmises", VM, conn)])
    el = GPUAssembler(coords, nodeDof, nDof, [ElementGroup("C3D8", "linearelastic", VM[:2], conn)])
    dU = np.zeros(nDof)
    dU[nodeDof + 1] = 0.01 * coords[:, 1]  # far beyond yield
    _pass(asm, dU, dU)
    asm.acceptLastState()
    s0 = asm.group_state(0, "ref")
    assert (s0[..., 12] > 0).all()
    P, F, K = _pass(asm, dU, np.zeros(nDof))  # zero increment: |d eps| < 1e-14 shortcut
    assert np.array_equal(asm.group_state(0, "temp"), s0)
    _, _, Kel = _pass(el, dU, np.zeros(nDof))
    assert np.abs(K - Kel).max() <= 1e-12 * np.abs(Kel).max()


def test_non_finite_input_is_flagged_not_trapped():
    from edelweissfe_gb300 import ElementGroup, GPUAssembler, meshes
    from edelweissfe_gb300 import _lib as L

    coords, conn, nodeDof, nDof = meshes.box(2, 1, 1, nNodes=8)
    asm = GPUAssembler(coords, nodeDof, nDof, [ElementGroup("C3D8", "vonmises", VM, conn)])
    dU = np.zeros(nDof)
    dU[5] = np.nan
    P, F, K = asm.constructDofVector(), asm.constructDofVector(), asm.constructSystemMatrix()
    asm.status.zero_()
    asm.launch(torch.tensor(dU, device=asm.device), torch.tensor(dU, device=asm.device), P, K, F)
    st = asm.status.cpu().numpy()
    assert st[0] & L.EFE_STATUS_NONFINITE
    # the context is still usable
    _pass(asm, np.zeros(nDof), np.zeros(nDof))


def test_plane_stress_hyperelastic_is_rejected_like_the_reference():
    from edelweissfe_gb300 import ElementGroup, GPUAssembler, meshes

    coords, conn, nodeDof, nDof = meshes.rect(2, 1, nNodes=8)
    with pytest.raises(NotImplementedError, match="Plane stress for hyperelastic materials is currently not possible"):
        GPUAssembler(coords, nodeDof, nDof, [ElementGroup("CPS8RTL", "neohookewa", [400.0, 4000.0], conn, 1.0)])
