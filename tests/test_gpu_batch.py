"""Batched uneven meshes: the persistent launch (mixed element types), the per-batch launches and a CUDA-graph
replay give the same P, F, K as evaluating every mesh on its own; the autotuner's tile variants
give the same results (FP64: 1e-12 relative; mixed: P, F 1e-12, K 2e-6)."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _meshes(seed):
    from edelweissfe_gb300 import meshes

    rng = np.random.default_rng(seed)
    out2, out3 = [], []
    for k, n in enumerate([3, 7, 5]):
        coords, conn, nodeDof, nDof = meshes.rect(n, 2 + k, lX=1.0, lY=0.8, nNodes=8)
        Fbar = np.eye(2) + 0.05 * rng.normal(size=(2, 2))
        U = np.zeros(nDof)
        used = nodeDof >= 0
        U.reshape(-1)[:] = 0
        disp = coords @ (Fbar - np.eye(2)).T + 0.002 * rng.normal(size=coords.shape)
        for c in range(2):
            U[nodeDof[used] + c] = disp[used, c]
        mu = 10 ** rng.uniform(2, 4)
        out2.append(dict(coords=coords, conn=conn, nodeDof=nodeDof, nDof=nDof, props=[mu, 10 * mu], thickness=1.0, U=U))
    for k, n in enumerate([2, 3]):
        coords, conn, nodeDof, nDof = meshes.box(n, 2, 1 + k, nNodes=20)
        Fbar = np.eye(3) + 0.05 * rng.normal(size=(3, 3))
        disp = coords @ (Fbar - np.eye(3)).T + 0.002 * rng.normal(size=coords.shape)
        U = np.zeros(nDof)
        for c in range(3):
            U[nodeDof + c] = disp[:, c]
        mu = 10 ** rng.uniform(2, 4)
        out3.append(dict(coords=coords, conn=conn, nodeDof=nodeDof, nDof=nDof, props=[mu, 10 * mu], U=U))
    return out2, out3


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_pass_matches_single_meshes(precision):
    from edelweissfe_gb300 import ElementGroup, GPUAssembler
    from edelweissfe_gb300.autotune import Autotuner
    from edelweissfe_gb300.batch import BatchedPass, MeshBatch

    m2, m3 = _meshes(3)
    b2 = MeshBatch(m2, "CPE8RTL", "neohookewa", precision)
    b3 = MeshBatch(m3, "C3D20TL", "neohookewa", precision)
    for b, ms in ((b2, m2), (b3, m3)):
        b.U.copy_(torch.tensor(np.concatenate([m["U"] for m in ms])))
    ktol = 1e-12 if precision == "fp64" else 2e-6
    results = {}
    for mode in ("persistent", "perbatch", "graph"):
        bp = BatchedPass([b3, b2], persistent=(mode != "perbatch"))
        if mode == "graph":
            bp.capture()
            bp.replay()
        else:
            bp.step()
        torch.cuda.synchronize()
        bp.check_status()
        results[mode] = [(b.P.cpu().numpy().copy(), b.F.cpu().numpy().copy(), b.K.double().cpu().numpy().copy())
                         for b in (b2, b3)]  # fmt: skip
    for b, ms, (et, k) in ((b2, m2, ("CPE8RTL", 0)), (b3, m3, ("C3D20TL", 1))):
        for i, m in enumerate(ms):
            a = GPUAssembler(m["coords"], m["nodeDof"], m["nDof"],
                             [ElementGroup(et, "neohookewa", m["props"], m["conn"], m.get("thickness", 1.0))],
                             precision=precision)  # fmt: skip
            P, F, K = a.constructDofVector(), a.constructDofVector(), a.constructSystemMatrix()
            U = torch.tensor(m["U"], device=a.device)
            a.computeElements(None, U, U, P, K, F)
            ds, ks = b.mesh_slice(i)
            for mode, res in results.items():
                Pb, Fb, Kb = res[k]
                assert _rel(Pb[ds], P.cpu().numpy()) <= 1e-12, (mode, et, i)
                assert _rel(Fb[ds], F.cpu().numpy()) <= 1e-12, (mode, et, i)
                assert _rel(Kb[ks], K.double().cpu().numpy()) <= ktol, (mode, et, i)
    # tile variants
    tuner = Autotuner(cache="/tmp/efe_autotune_test.json")
    bp = BatchedPass([b3, b2])
    tuner.tune_batched(bp)
    bp.step()
    torch.cuda.synchronize()
    for k, b in enumerate((b2, b3)):
        assert _rel(b.P.cpu().numpy(), results["persistent"][k][0]) <= 1e-12
        assert _rel(b.K.double().cpu().numpy(), results["persistent"][k][2]) <= ktol


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed-ff"])
def test_persistent_pass_over_many_batches(precision):
    """Five batches (three Hexa20, two Quad8) in ONE persistent launch give the per-batch results; a
    CUDA-graph replay of it too; a batch of another element type is refused."""
    from edelweissfe_gb300 import meshes
    from edelweissfe_gb300.batch import BatchedPass, MeshBatch, persistent_capable

    m2, m3 = _meshes(4)
    m3 = m3 + _meshes(5)[1]
    groups = [(m3[:1], "C3D20TL"), (m3[1:3], "C3D20TL"), (m3[3:], "C3D20TL"), (m2[:2], "CPE8RTL"),
              (m2[2:], "CPE8RTL")]  # fmt: skip
    batches = []
    for ms, et in groups:
        b = MeshBatch(ms, et, "neohookewa", precision)
        b.U.copy_(torch.tensor(np.concatenate([m["U"] for m in ms])))
        batches.append(b)
    ktol = 1e-12 if precision == "fp64" else 2e-6
    out = {}
    for mode in ("perbatch", "persistent", "graph"):
        bp = BatchedPass(batches, persistent=(mode != "perbatch"))
        assert bp.persistent == (mode != "perbatch")
        if mode == "graph":
            bp.capture()
            bp.replay()
        else:
            bp.step()
        torch.cuda.synchronize()
        bp.check_status()
        out[mode] = [(b.P.cpu().numpy().copy(), b.K.double().cpu().numpy().copy()) for b in batches]
    for mode in ("persistent", "graph"):
        for (P, K), (Pr, Kr) in zip(out[mode], out["perbatch"]):
            assert _rel(P, Pr) <= 1e-12 and _rel(K, Kr) <= ktol, mode
    coords, conn, nodeDof, nDof = meshes.box(2, 2, 1, nNodes=8)
    other = MeshBatch([dict(coords=coords, conn=conn, nodeDof=nodeDof, nDof=nDof, props=[210e3, 0.3])],
                      "C3D8R", "linearelastic", precision)  # fmt: skip
    assert not persistent_capable(batches + [other])
    assert BatchedPass(batches + [other], persistent=True).persistent is False


def _oracle(m, elType, kind, U, dU):
    """The oracle's pass over one mesh from a zero history: P, F, CSR data (its own pattern) and state."""
    from oracle.assembly import Model

    E = len(m["conn"])
    props = np.broadcast_to(np.asarray(m["props"], float), (E, len(m["props"])))
    g = dict(elType=elType, kind=kind, props=np.array(props), conn=np.asarray(m["conn"], np.int64),
             thickness=np.full(E, float(m.get("thickness", 1.0))), order=np.arange(E))  # fmt: skip
    model = Model(m["coords"], m["nodeDof"], m["nDof"], [g])
    r = model.compute_elements(U, dU, model.initial_state())
    assert r["first_failed_element"] is None
    return model, r


def _check_against_oracle(b, i, m, elType, kind, ktol, dU=None):
    """Mesh i of batch b (after its pass) against the oracle: P, F, the mesh's CSR slice (pattern and
    values) and its elements' state."""
    U = m["U"]
    model, r = _oracle(m, elType, kind, U, U if dU is None else dU)
    ds, ks = b.mesh_slice(i)
    P, F, K = b.P.cpu().numpy()[ds], b.F.cpu().numpy()[ds], b.K.double().cpu().numpy()[ks]
    assert _rel(P, r["P"]) <= 1e-12 and _rel(F, r["F"]) <= 1e-12
    ip = b.asm.indptr_host
    rows = ip[int(b.dof_offsets[i]): int(b.dof_offsets[i + 1]) + 1] - ip[int(b.dof_offsets[i])]
    assert np.array_equal(rows, model.indptr)
    if b.asm.indices_host is not None:
        cols = b.asm.indices_host[ks] - int(b.dof_offsets[i])
        assert np.array_equal(cols, model.indices)
    assert _rel(K, r["Kdata"]) <= ktol
    e0, e1 = int(b.element_offsets[i]), int(b.element_offsets[i + 1])
    st = b.asm.group_state(0)[e0:e1]
    assert _rel(st, r["stateTemp"][0]["state"]) <= 1e-12


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_meshes_match_the_oracle(precision):
    """Every Quad8 and Hexa20 mesh of a two-batch persistent pass against the oracle's own pass over
    that mesh (the reference algorithm: displacementtlelement/element.py:346-414 with
    neohookepencegouformulationa.py:107-141, assembled as nonlinearimplicitstatic.py:794-849 and
    csrgenerator.pyx:100-115): P, F, state 1e-12; K 1e-12 (FP64) / 2e-6 (FP32 tangent); CSR pattern
    of each mesh's block bit-exact."""
    from edelweissfe_gb300.batch import BatchedPass, MeshBatch

    m2, m3 = _meshes(6)
    b2 = MeshBatch(m2, "CPE8RTL", "neohookewa", precision)
    b3 = MeshBatch(m3, "C3D20TL", "neohookewa", precision)
    for b, ms in ((b2, m2), (b3, m3)):
        b.U.copy_(torch.tensor(np.concatenate([m["U"] for m in ms])))
    bp = BatchedPass([b3, b2], persistent=True)
    assert bp.persistent
    bp.step()
    torch.cuda.synchronize()
    bp.check_status()
    ktol = 1e-12 if precision == "fp64" else 2e-6
    for b, ms, et in ((b2, m2, "CPE8RTL"), (b3, m3, "C3D20TL")):
        for i, m in enumerate(ms):
            _check_against_oracle(b, i, m, et, "neohookewa", ktol)


def _small_strain_meshes(seed, nNodes, sizes):
    """Jittered blocks under a plastic uniaxial strain increment (0.4 %) with seeded noise, one
    von Mises material per mesh (yield stress and hardening varied per mesh: load cases)."""
    from edelweissfe_gb300 import meshes

    rng = np.random.default_rng(seed)
    out = []
    for nx, ny, nz in sizes:
        coords, conn, nodeDof, nDof = meshes.box(nx, ny, nz, nNodes=nNodes)
        coords = meshes.jitter(coords, 0.05, [1 / nx, 1 / ny, 1 / nz], int(rng.integers(1 << 30)), [0, 0, 0],
                               [1, 1, 1])  # fmt: skip
        dU = np.zeros(nDof)
        dU[nodeDof + 1] = 0.004 * coords[:, 1]
        dU += rng.uniform(-1, 1, nDof) * 2e-5
        props = [210e3, 0.3, float(rng.uniform(200, 300)), float(rng.uniform(800, 1200)), 0.0, 0.0]
        out.append(dict(coords=coords, conn=conn, nodeDof=nodeDof, nDof=nDof, props=props, U=dU))
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed-ff"])
def test_mixed_type_persistent_launch(precision):
    """ONE persistent launch over Hexa20 total-Lagrangian Neo-Hooke, Hexa20 and Hexa8 small-strain von
    Mises (plastic increment), Hexa8 total-Lagrangian Neo-Hooke and Quad8 total-Lagrangian Neo-Hooke
    batches (nonlinearimplicitstaticparallelmk2.pyx:111-198 evaluates such a mixed element set in one
    loop): the per-batch launches' results and the oracle's, mesh by mesh; then load cases of the
    Hexa8 J2 material alone (three batches, their own persistent kernel) the same way."""
    from edelweissfe_gb300 import meshes
    from edelweissfe_gb300.batch import BatchedPass, MeshBatch

    m2, m3 = _meshes(7)
    rng = np.random.default_rng(9)
    h8tl = []
    for n in (2, 3):
        coords, conn, nodeDof, nDof = meshes.box(n, 2, 2, nNodes=8)
        Fbar = np.eye(3) + 0.05 * rng.normal(size=(3, 3))
        U = (coords @ (Fbar - np.eye(3)).T + 0.002 * rng.normal(size=coords.shape)).ravel()
        h8tl.append(dict(coords=coords, conn=conn, nodeDof=nodeDof, nDof=nDof, props=[300.0, 3000.0], U=U))
    ss8 = _small_strain_meshes(10, 8, [(3, 3, 2), (2, 4, 3)])
    ss20 = _small_strain_meshes(11, 20, [(2, 2, 1), (3, 2, 2)])
    spec = [(m3, "C3D20TL", "neohookewa"), (ss20, "C3D20", "vonmises"), (h8tl, "C3D8TL", "neohookewa"),
            (ss8, "C3D8", "vonmises"), (m2, "CPE8RTL", "neohookewa")]  # fmt: skip
    ktol = 1e-12 if precision == "fp64" else 2e-6

    def batches_of(spec):
        out = []
        for ms, et, kind in spec:
            b = MeshBatch(ms, et, kind, precision)
            u = torch.tensor(np.concatenate([m["U"] for m in ms]))
            b.U.copy_(u)
            b.dU.copy_(u)  # small strain: the increment from the zero history
            out.append(b)
        return out

    for case in (spec, [(ss8[:1], "C3D8", "vonmises"), (ss8[1:], "C3D8", "vonmises"),
                        (_small_strain_meshes(12, 8, [(4, 2, 2)]), "C3D8", "vonmises")]):  # fmt: skip
        batches = batches_of(case)
        res = {}
        for mode in ("perbatch", "persistent"):
            bp = BatchedPass(batches, persistent=(mode == "persistent"))
            assert bp.persistent == (mode == "persistent")
            bp.step()
            torch.cuda.synchronize()
            bp.check_status()
            res[mode] = [(b.P.cpu().numpy().copy(), b.K.double().cpu().numpy().copy(), b.asm.group_state(0).copy())
                         for b in batches]  # fmt: skip
        for (P, K, S), (Pr, Kr, Sr) in zip(res["persistent"], res["perbatch"]):
            assert _rel(P, Pr) <= 1e-12 and _rel(K, Kr) <= ktol and _rel(S, Sr) <= 1e-12
        for b, (ms, et, kind) in zip(batches, case):
            for i, m in enumerate(ms):
                _check_against_oracle(b, i, m, et, kind, ktol)
