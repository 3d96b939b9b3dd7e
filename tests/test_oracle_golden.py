"""Pin the oracle to the reference: every golden fixture is replayed through the oracle.

Tolerances: the oracle restates the reference algorithm in FP64 with the same
operation order per material point, so outputs agree to round-off; the bar is
1e-12 relative to the largest entry of each output.
"""

import numpy as np
import pytest

import golden_cases as gc
from oracle import library, shapes

RTOL = 1e-12


def _close(a, b, rtol=RTOL):
    scale = max(np.abs(b).max(), 1e-300)
    err = np.abs(a - b).max() / scale
    return err, err <= rtol


@pytest.mark.parametrize("name", gc.case_names())
def test_oracle_matches_reference(name):
    case = gc.load(name)
    model = gc.oracle_model(case)
    if "indptr" in case:
        assert np.array_equal(model.indptr, case["indptr"]), "CSR indptr differs"
        assert np.array_equal(model.indices, case["indices"]), "CSR indices differ"
    el_dofs = np.array(model.dofs)
    assert np.array_equal(el_dofs, case["el_dofs"]), "element DOF map differs"
    state = model.initial_state()
    last_temp = None
    for call in gc.calls(case):
        if call["accept_before"]:
            state = model.accept_state(last_temp)
        r = model.compute_elements(call["U"], call["dU"], state)
        if call["raised"] >= 0:
            assert r["first_failed_element"] == call["raised"], (r["first_failed_element"], call["raised"])
            return
        assert r["first_failed_element"] is None
        for key, ours in (("P", r["P"]), ("F", r["F"]), ("Kdata", r["Kdata"])):
            if call[key] is None:
                continue
            err, ok = _close(ours, call[key])
            assert ok, f"call {call['index']} {key} rel err {err:.3e}"
        st = r["stateTemp"][0]["state"]
        err, ok = _close(st, call["state"])
        assert ok, f"call {call['index']} state rel err {err:.3e}"
        last_temp = r["stateTemp"]


def test_library_table_matches_reference():
    d = np.load(gc.GOLDEN + "/library.npz")
    names = sorted({k.split("__")[0] for k in d.files})
    assert sorted(library.elLibrary) == names
    for n in names:
        e = library.get(n)
        meta = d[f"{n}__meta"]
        pe = {1: True, 0: False, -1: None}[int(meta[4])]
        assert [e["nNodes"], e["nDof"], e["nSpatialDimensions"], e["nInt"]] == list(meta[:4])
        assert e["plStrain"] == pe
        assert e["elClass"] == str(d[f"{n}__class"])
        for f in ("xi", "eta", "w"):
            assert np.array_equal(np.asarray(e[f], float), d[f"{n}__{f}"]), (n, f)
        if f"{n}__zeta" in d.files:
            assert np.array_equal(np.asarray(e["zeta"], float), d[f"{n}__zeta"])


def test_geometry_matches_reference():
    d = np.load(gc.GOLDEN + "/geometry.npz")
    for et in sorted({k.split("__")[0] for k in d.files}):
        e = library.get(et)
        X = d[f"{et}__X"]
        dim = e["nSpatialDimensions"]
        J = np.einsum("qra,ac->qrc", shapes.jacobian_table(e), X)
        G = np.linalg.solve(J, shapes.derivative_table(e))
        assert np.abs(J - d[f"{et}__J"]).max() < 1e-13
        assert np.abs(G - d[f"{et}__nablaN"]).max() < 1e-12
        B = d[f"{et}__B"]
        assert np.abs(B[:, 0, 0::dim] - G[:, 0]).max() < 1e-12
        assert np.abs(B[:, 1, 1::dim] - G[:, 1]).max() < 1e-12
        assert np.abs(shapes.shape_table(e) - d[f"{et}__N"]).max() < 1e-15


def test_fixtures_exercise_plasticity():
    """The J2 fixtures must contain plastic points (kappa > 0), else they pin nothing of the return map."""
    n_plastic = 0
    for name in gc.case_names():
        case = gc.load(name)
        if str(case["kind"]) != "vonmises":
            continue
        for call in gc.calls(case):
            if call["state"] is not None:
                n_plastic += int((call["state"][..., 12] > 0).sum())
    assert n_plastic > 1000
