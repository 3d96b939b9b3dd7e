"""Batched uneven meshes: the persistent two-type launch, the per-batch launches and a CUDA-graph
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


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
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
    other = MeshBatch([dict(coords=coords, conn=conn, nodeDof=nodeDof, nDof=nDof, props=[100.0, 1000.0])],
                      "C3D8TL", "neohookewa", precision)  # fmt: skip
    assert not persistent_capable(batches + [other])
    assert BatchedPass(batches + [other], persistent=True).persistent is False
