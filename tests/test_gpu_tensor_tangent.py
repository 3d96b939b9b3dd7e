"""The Hexa20 3x3x3 element tangent on the tensor cores (tile variant 3: tcgen05 TF32 MMAs with a hi/lo
split, FP32 accumulation in TMEM), total-Lagrangian Neo-Hooke and small strain, against the reference
and the oracle.

* The reference's own fixtures of C3D20TL with Neo-Hooke a, b, c (tests/golden, recorded from
  displacementtlelement/element.py:346-427 and neohookepencegouformulation{a,b,c}.py): P, F and
  state within 1e-12, K within the FP32-tangent tolerance 2e-6 (max-norm ratios), in both FP32
  tangent modes (mixed, mixed-ff).
* A jittered 8 x 8 x 6 C3D20TL block (384 elements: more tiles than resident CTAs, so each CTA
  strides over several elements and reuses its TMEM) under F = I + 0.05 N(0,1) plus noise, Neo-Hooke b
  (all four tangent coefficients non-zero): against the oracle's pass (same tolerances, CSR pattern
  bit-exact) and against the SIMT tangent of tile variant 0 (K within 2e-6).
"""

import numpy as np
import pytest

import golden_cases as gc

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

RTOL = 1e-12
RTOL_K = 2e-6
TC = 3


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("precision", ["mixed", "mixed-ff"])
@pytest.mark.parametrize("name", ["tl_c3d20tl_wa", "tl_c3d20tl_wb", "tl_c3d20tl_wc"])
def test_tensor_tangent_matches_reference_fixtures(name, precision):
    from edelweissfe_gb300 import ElementGroup, GPUAssembler

    case = gc.load(name)
    g = ElementGroup(str(case["elType"]), str(case["kind"]), case["props"], case["conn"], case["thickness"])
    asm = GPUAssembler(case["coords"], case["node_dof"], int(case["nDof"]), [g], precision=precision)
    asm._groups_c[0].tileVariant = TC
    for call in gc.calls(case):
        if call["accept_before"]:
            asm.acceptLastState()
        assert call["raised"] < 0
        P, F, K = asm.constructDofVector(), asm.constructDofVector(), asm.constructSystemMatrix()
        asm.computeElements(None, torch.tensor(call["U"], device=asm.device),
                            torch.tensor(call["dU"], device=asm.device), P, K, F)  # fmt: skip
        assert _rel(P.cpu().numpy(), call["P"]) <= RTOL
        assert _rel(F.cpu().numpy(), call["F"]) <= RTOL
        if call["Kdata"] is not None:  # the fixtures record K on most calls
            err = _rel(K.double().cpu().numpy(), call["Kdata"])
            assert err <= RTOL_K, f"K rel err {err:.3e}"
        assert _rel(asm.group_state(0), call["state"]) <= RTOL


def _block():
    from edelweissfe_gb300 import meshes

    coords, conn, nodeDof, nDof = meshes.box(8, 8, 6, lX=1.0, lY=1.0, lZ=0.75, nNodes=20)
    coords = meshes.jitter(coords, 0.08, [1 / 8, 1 / 8, 0.75 / 6], 5, [0, 0, 0], [1, 1, 0.75])
    rng = np.random.default_rng(6)
    Fbar = np.eye(3) + 0.05 * rng.normal(size=(3, 3))
    disp = coords @ (Fbar - np.eye(3)).T + 0.002 * rng.normal(size=coords.shape) / 8
    U = np.zeros(nDof)
    for c in range(3):
        U[nodeDof + c] = disp[:, c]
    return coords, conn, nodeDof, nDof, U


@pytest.mark.parametrize("precision", ["mixed", "mixed-ff"])
def test_persistent_launch_with_tensor_core_hexa20(precision):
    """Uneven Hexa20 total-Lagrangian meshes (two batches, every group on tile variant 3) and a Quad8
    batch in ONE persistent launch: the Hexa20 tangents come from the tensor cores; results equal
    the per-batch launches with the SIMT tangent (K 2e-6) and the oracle mesh by mesh."""
    from edelweissfe_gb300 import meshes
    from edelweissfe_gb300.batch import BatchedPass, MeshBatch
    from oracle.assembly import Model

    rng = np.random.default_rng(11)
    ms3 = []
    for n in ((3, 2, 2), (2, 4, 3), (5, 3, 2)):
        coords, conn, nodeDof, nDof = meshes.box(*n, nNodes=20)
        Fbar = np.eye(3) + 0.05 * rng.normal(size=(3, 3))
        disp = coords @ (Fbar - np.eye(3)).T + 0.002 * rng.normal(size=coords.shape)
        U = np.zeros(nDof)
        for c in range(3):
            U[nodeDof + c] = disp[:, c]
        ms3.append(dict(coords=coords, conn=conn, nodeDof=nodeDof, nDof=nDof, props=[float(10 ** rng.uniform(2, 4)),
                        float(10 ** rng.uniform(3, 5))], U=U))  # fmt: skip
    coords, conn, nodeDof, nDof = meshes.rect(6, 4, nNodes=8)
    U = np.zeros(nDof)
    used = nodeDof >= 0
    disp = coords @ (0.05 * rng.normal(size=(2, 2))).T
    for c in range(2):
        U[nodeDof[used] + c] = disp[used, c]
    ms2 = [dict(coords=coords, conn=conn, nodeDof=nodeDof, nDof=nDof, props=[500.0, 5000.0], thickness=1.0, U=U)]
    spec = [(ms3[:2], "C3D20TL"), (ms3[2:], "C3D20TL"), (ms2, "CPE8RTL")]
    batches = []
    for ms, et in spec:
        b = MeshBatch(ms, et, "neohookewa", precision)
        b.U.copy_(torch.tensor(np.concatenate([m["U"] for m in ms])))
        batches.append(b)
    out = {}
    for mode in ("perbatch", "persistent"):
        for b, (ms, et) in zip(batches, spec):
            b.asm._groups_c[0].tileVariant = TC if (mode == "persistent" and et == "C3D20TL") else 0
        bp = BatchedPass(batches, persistent=(mode == "persistent"))
        assert bp.persistent == (mode == "persistent")
        bp.step()
        torch.cuda.synchronize()
        bp.check_status()
        out[mode] = [(b.P.cpu().numpy().copy(), b.K.double().cpu().numpy().copy()) for b in batches]
    for (P, K), (Pr, Kr) in zip(out["persistent"], out["perbatch"]):
        assert _rel(P, Pr) <= RTOL and _rel(K, Kr) <= RTOL_K
    for bi, (b, (ms, et)) in enumerate(zip(batches, spec)):
        for i, m in enumerate(ms):
            E = len(m["conn"])
            model = Model(m["coords"], m["nodeDof"], m["nDof"], [dict(
                elType=et, kind="neohookewa", props=np.tile(m["props"], (E, 1)), conn=np.asarray(m["conn"], np.int64),
                thickness=np.ones(E), order=np.arange(E))])  # fmt: skip
            r = model.compute_elements(m["U"], m["U"], model.initial_state())
            ds, ks = b.mesh_slice(i)
            P, K = out["persistent"][bi]
            assert _rel(P[ds], r["P"]) <= RTOL and _rel(K[ks], r["Kdata"]) <= RTOL_K


@pytest.mark.parametrize("precision", ["mixed", "mixed-ff"])
def test_tensor_tangent_on_a_block_against_oracle_and_simt(precision):
    from edelweissfe_gb300 import ElementGroup, GPUAssembler
    from oracle.assembly import Model

    coords, conn, nodeDof, nDof, U = _block()
    props = [300.0, 3000.0]
    E = len(conn)
    model = Model(coords, nodeDof, nDof, [dict(elType="C3D20TL", kind="neohookewb", props=np.tile(props, (E, 1)),
                                               conn=conn.astype(np.int64), thickness=np.ones(E), order=np.arange(E))])
    ref = model.compute_elements(U, U, model.initial_state())
    out = {}
    for variant in (TC, 0):
        asm = GPUAssembler(coords, nodeDof, nDof, [ElementGroup("C3D20TL", "neohookewb", props, conn)],
                           precision=precision)  # fmt: skip
        asm._groups_c[0].tileVariant = variant
        P, F, K = asm.constructDofVector(), asm.constructDofVector(), asm.constructSystemMatrix()
        Ud = torch.tensor(U, device=asm.device)
        asm.computeElements(None, Ud, Ud, P, K, F)
        out[variant] = (P.cpu().numpy(), F.cpu().numpy(), K.double().cpu().numpy(), asm.group_state(0))
        assert np.array_equal(asm.indptr_host, model.indptr) and np.array_equal(asm.indices_host, model.indices)
    P, F, K, S = out[TC]
    assert _rel(P, ref["P"]) <= RTOL and _rel(F, ref["F"]) <= RTOL
    assert _rel(S, ref["stateTemp"][0]["state"]) <= RTOL
    err = _rel(K, ref["Kdata"])
    assert err <= RTOL_K, f"K vs oracle rel err {err:.3e}"
    assert _rel(K, out[0][2]) <= RTOL_K
    assert _rel(P, out[0][0]) <= RTOL  # the residual does not depend on the tangent's form


@pytest.mark.parametrize("precision", ["mixed", "mixed-ff"])
@pytest.mark.parametrize("name", ["ss_c3d20_li", "ss_c3d20_vmn", "ss_c3d20_vo", "cutback_c3d20_vm"])
def test_small_strain_tensor_tangent_matches_reference_fixtures(name, precision):
    """The small-strain Hexa20 3x3x3 form on the tensor cores (lambda' G (x) G - a nG (x) nG plain,
    mu' G (x) G swapped, mu' G.G diagonal; displacementelement/element.py:318-346 with
    vonmises.py:186-254 / linearelastic.py): the reference's C3D20 fixtures, elastic and plastic
    increments with state acceptance, and the cutback request of the reference's own run."""
    from edelweissfe_gb300 import CutbackRequest, ElementGroup, GPUAssembler

    case = gc.load(name)
    g = ElementGroup(str(case["elType"]), str(case["kind"]), case["props"], case["conn"], case["thickness"])
    asm = GPUAssembler(case["coords"], case["node_dof"], int(case["nDof"]), [g], precision=precision)
    asm._groups_c[0].tileVariant = TC
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
            return
        if name == "cutback_c3d20_vm":
            # rounding-critical return map: with the FP32-tangent modes' faster return-map
            # arithmetic a cutback one call early is an allowed outcome (as in test_gpu_parity)
            try:
                asm.computeElements(None, U, dU, P, K, F)
            except CutbackRequest:
                return
        else:
            asm.computeElements(None, U, dU, P, K, F)
        assert _rel(P.cpu().numpy(), call["P"]) <= RTOL
        assert _rel(F.cpu().numpy(), call["F"]) <= RTOL
        if call["Kdata"] is not None:
            err = _rel(K.double().cpu().numpy(), call["Kdata"])
            assert err <= RTOL_K, f"K rel err {err:.3e}"
        assert _rel(asm.group_state(0), call["state"]) <= RTOL


@pytest.mark.parametrize("precision", ["mixed", "mixed-ff"])
def test_small_strain_tensor_tangent_plastic_block(precision):
    """A jittered 6 x 5 x 4 C3D20 von Mises block in a plastic increment (per-element yield stress):
    the tensor-core tangent against the oracle's pass and the SIMT tangent (K 2e-6; P, F, state
    1e-12, the residual independent of the tangent's form)."""
    from edelweissfe_gb300 import ElementGroup, GPUAssembler, meshes
    from oracle.assembly import Model

    coords, conn, nodeDof, nDof = meshes.box(6, 5, 4, lX=1.0, lY=1.0, lZ=0.8, nNodes=20)
    coords = meshes.jitter(coords, 0.08, [1 / 6, 1 / 5, 0.2], 7, [0, 0, 0], [1, 1, 0.8])
    rng = np.random.default_rng(13)
    E = len(conn)
    props = np.tile([210e3, 0.3, 250.0, 1000.0, 0.0, 0.0], (E, 1))
    props[:, 2] *= rng.uniform(0.8, 1.2, E)
    dU = np.zeros(nDof)
    for c in range(3):
        dU[nodeDof + c] = coords @ (0.004 * rng.normal(size=3)) + 0.0005 * rng.normal(size=len(coords))
    model = Model(coords, nodeDof, nDof, [dict(elType="C3D20", kind="vonmises", props=props, conn=conn.astype(np.int64),
                                               thickness=np.ones(E), order=np.arange(E))])  # fmt: skip
    ref = model.compute_elements(dU, dU, model.initial_state())
    assert ref["first_failed_element"] is None
    st = ref["stateTemp"][0]["state"]
    assert (st[..., 12] > 0).mean() > 0.2  # a plastic increment
    out = {}
    for variant in (TC, 0):
        asm = GPUAssembler(coords, nodeDof, nDof, [ElementGroup("C3D20", "vonmises", props, conn)], precision=precision)
        asm._groups_c[0].tileVariant = variant
        P, F, K = asm.constructDofVector(), asm.constructDofVector(), asm.constructSystemMatrix()
        d = torch.tensor(dU, device=asm.device)
        asm.computeElements(None, d, d, P, K, F)
        out[variant] = (P.cpu().numpy(), F.cpu().numpy(), K.double().cpu().numpy(), asm.group_state(0))
    P, F, K, S = out[TC]
    assert _rel(P, ref["P"]) <= RTOL and _rel(F, ref["F"]) <= RTOL
    assert _rel(S, st) <= RTOL
    err = _rel(K, ref["Kdata"])
    assert err <= RTOL_K, f"K vs oracle rel err {err:.3e}"
    assert _rel(K, out[0][2]) <= RTOL_K
    assert _rel(P, out[0][0]) <= RTOL
