"""GPU parity on a mesh of hundreds of CTA tiles: the headline workload's element pass (boxGen C3D8,
interior nodes jittered +-5 %, von Mises J2 [210000, 0.3, 250, 1000], increment 1 of uniaxial strain
accepted, then a plastic increment 2 with seeded noise) on an 18^3 mesh (5,832 elements: 365 tiles
of 16 elements, 183 of 32, the last ragged) against the oracle's pass over the whole mesh, in every
precision and every CTA tile variant, and with the autotuner's choice.

Tolerances (max |gpu - oracle| / max |oracle|): R, F and state 1e-12 (state also per field: stress,
strain and kappa each against its own largest entry); K 1e-12 in FP64, 2e-6 with the FP32 tangent;
CSR pattern bit-exact.  The oracle is the FP64 NumPy restatement pinned to the reference's own
outputs (tests/test_oracle_golden.py); the element algorithm follows vonmises.py:186-254 and
displacementelement/element.py:290-346, the assembly nonlinearimplicitstatic.py:794-849 and
csrgenerator.pyx:100-115.
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

N = 18
RTOL = 1e-12
RTOL_K_MIXED = 2e-6


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.fixture(scope="module")
def case():
    import bench

    coords, conn, nodeDof, nDof, dU1, dU2 = bench.workload(N)
    model = bench._oracle_model(coords, conn, nodeDof, nDof, np.arange(len(conn)))
    st = model.accept_state(model.compute_elements(dU1, dU1, model.initial_state())["stateTemp"])
    ref = model.compute_elements(dU1 + dU2, dU2, st)
    assert ref["first_failed_element"] is None
    assert (ref["stateTemp"][0]["state"][..., 12] > st[0]["state"][..., 12]).mean() > 0.9  # plastic increment
    return dict(coords=coords, conn=conn, nodeDof=nodeDof, nDof=nDof, dU1=dU1, dU2=dU2, model=model, ref=ref)


def _pass(case, precision, variant=None, tune=False, tmp_path=None):
    import bench
    from edelweissfe_gb300 import ElementGroup, GPUAssembler

    asm = GPUAssembler(case["coords"], case["nodeDof"], case["nDof"],
                       [ElementGroup("C3D8", "vonmises", bench.VM, case["conn"])], precision=precision)  # fmt: skip
    if variant is not None:
        asm._groups_c[0].tileVariant = variant
    dev = asm.device
    P, F, K = asm.constructDofVector(), asm.constructDofVector(), asm.constructSystemMatrix()
    d1 = torch.tensor(case["dU1"], device=dev)
    asm.computeElements(None, d1, d1, P, K, F)
    asm.acceptLastState()
    U = torch.tensor(case["dU1"] + case["dU2"], device=dev)
    dU = torch.tensor(case["dU2"], device=dev)
    if tune:
        from edelweissfe_gb300.autotune import VARIANTS, Autotuner

        Autotuner(cache=str(tmp_path / "tune.json")).tune_assembler(asm, U, dU, P, K, F)
        assert asm._groups_c[0].tileVariant in VARIANTS
    for t in (P, F, K):
        t.zero_()
    asm.computeElements(None, U, dU, P, K, F)
    return asm, P.cpu().numpy(), F.cpu().numpy(), K.double().cpu().numpy()


def _check(case, precision, asm, P, F, K):
    ref, model = case["ref"], case["model"]
    assert np.array_equal(asm.indptr_host, model.indptr) and np.array_equal(asm.indices_host, model.indices)
    assert _rel(P, ref["P"]) <= RTOL
    assert _rel(F, ref["F"]) <= RTOL
    tol_k = RTOL if precision == "fp64" else RTOL_K_MIXED
    assert _rel(K, ref["Kdata"]) <= tol_k
    st, so = asm.group_state(0), ref["stateTemp"][0]["state"]
    assert _rel(st, so) <= RTOL
    for name, s in (("stress", slice(0, 6)), ("strain", slice(6, 12)), ("kappa", slice(12, 13))):
        err = _rel(st[..., s], so[..., s])
        assert err <= RTOL, f"{name} rel err {err:.3e}"


@pytest.mark.parametrize("variant", [0, 1, 2])
@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed-ff"])
def test_tile_variants_match_the_oracle(case, precision, variant):
    asm, P, F, K = _pass(case, precision, variant)
    _check(case, precision, asm, P, F, K)


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed-ff"])
def test_autotuned_pass_matches_the_oracle(case, precision, tmp_path):
    asm, P, F, K = _pass(case, precision, tune=True, tmp_path=tmp_path)
    _check(case, precision, asm, P, F, K)
