"""GPU parity: the CUDA path (through the C ABI) replays every reference fixture.

FP64 mode: P, F, K and the quadrature-point state agree with the reference to 1e-12 relative
(to the largest entry of each output); the CSR pattern is bit-exact.
Mixed modes (FP32 tangent; "mixed-ff" also forms the small-strain strain increment and element
residual in float-float arithmetic): P, F and state keep the 1e-12 bar; K agrees to 2e-6 relative.
Failing material points raise CutbackRequest from the same element as the reference.
"""

import numpy as np
import pytest

import golden_cases as gc

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

RTOL = 1e-12
RTOL_K_MIXED = 2e-6

# Stresses of ~1.5e4 make one ulp (1.8e-12) larger than the von Mises return map's absolute 1e-12
# tolerance (vonmises.py:56,229): whether the scalar Newton meets it, or runs into its 15-iteration
# CutbackRequest, depends on the last bit of the strain increment.  The reference converged on this
# case; a mode with different rounding of the strain (mixed-ff) may legitimately ask for a cutback.
ROUNDING_CRITICAL = {"cutback_c3d20_vm"}


def _assembler(case, precision):
    from edelweissfe_gb300 import ElementGroup, GPUAssembler

    g = ElementGroup(str(case["elType"]), str(case["kind"]), case["props"], case["conn"], case["thickness"])
    return GPUAssembler(case["coords"], case["node_dof"], int(case["nDof"]), [g], precision=precision)


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed-ff"])
@pytest.mark.parametrize("name", gc.case_names())
def test_gpu_matches_reference(name, precision):
    from edelweissfe_gb300 import CutbackRequest

    case = gc.load(name)
    asm = _assembler(case, precision)
    if "indptr" in case:
        assert np.array_equal(asm.indptr_host, case["indptr"])
        assert np.array_equal(asm.indices_host, case["indices"])
    for call in gc.calls(case):
        if call["accept_before"]:
            asm.acceptLastState()
        P, F, K = asm.constructDofVector(), asm.constructDofVector(), asm.constructSystemMatrix()
        U = torch.tensor(call["U"], device=asm.device)
        dU = torch.tensor(call["dU"], device=asm.device)
        if call["raised"] >= 0:
            with pytest.raises(CutbackRequest) as ei:
                asm.computeElements(None, U, dU, P, K, F)
            assert f"element {call['raised']} " in str(ei.value)
            assert ei.value.cutbackSize == 0.5
            return
        if name in ROUNDING_CRITICAL and precision != "fp64":
            try:
                asm.computeElements(None, U, dU, P, K, F)
            except CutbackRequest:
                return  # an allowed outcome, see ROUNDING_CRITICAL
        else:
            asm.computeElements(None, U, dU, P, K, F)
        assert _rel(P.cpu().numpy(), call["P"]) <= RTOL, f"call {call['index']} P"
        assert _rel(F.cpu().numpy(), call["F"]) <= RTOL, f"call {call['index']} F"
        if call["Kdata"] is not None:
            tol = RTOL if precision == "fp64" else RTOL_K_MIXED
            err = _rel(K.double().cpu().numpy(), call["Kdata"])
            assert err <= tol, f"call {call['index']} K rel err {err:.3e}"
        err = _rel(asm.group_state(0), call["state"])
        assert err <= RTOL, f"call {call['index']} state rel err {err:.3e}"


def test_csr_output_matches_scipy_layout():
    case = gc.load("cfg1_cpe4_le_40x8")
    asm = _assembler(case, "fp64")
    call = next(gc.calls(case))
    P, F, K = asm.constructDofVector(), asm.constructDofVector(), asm.constructSystemMatrix()
    U = torch.tensor(call["U"], device=asm.device)
    asm.computeElements(None, U, U, P, K, F)
    A = asm.assembleStiffnessCSR(K, host=True)
    assert A.indptr.dtype == np.int32 and A.indices.dtype == np.int32 and A.has_canonical_format
    assert _rel(A.data, call["Kdata"]) <= RTOL
    At = asm.assembleStiffnessCSR(K)
    assert At.layout == torch.sparse_csr
    y = (At @ U.unsqueeze(1)).squeeze(1).cpu().numpy()
    assert _rel(y, A @ call["U"]) <= 1e-12


def test_shared_properties_many_elements():
    """One property vector shared by all elements (a section without fields) on a multi-CTA mesh."""
    case = gc.load("cfg2_c3d8_vm_3cube")
    assert np.all(case["props"] == case["props"][0])
    case = dict(case)
    case["props"] = case["props"][0]
    asm = _assembler(case, "fp64")
    for call in gc.calls(case):
        if call["accept_before"]:
            asm.acceptLastState()
        P, F, K = asm.constructDofVector(), asm.constructDofVector(), asm.constructSystemMatrix()
        asm.computeElements(None, torch.tensor(call["U"], device=asm.device),
                            torch.tensor(call["dU"], device=asm.device), P, K, F)  # fmt: skip
        assert _rel(P.cpu().numpy(), call["P"]) <= RTOL
        assert _rel(asm.group_state(0), call["state"]) <= RTOL
