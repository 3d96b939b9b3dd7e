"""efe_compute_elements_persistent_noalloc: the element pass for callers that cannot allocate device
memory (their device memory belongs to another runtime's pool, or a cudaMalloc would stall their
time step).  It runs the same persistent kernel as efe_compute_elements_persistent, with the work
counter in the library's static device scratch instead of a caller buffer.

The GPU test calls both entry points through the C ABI on the same two batches (Quad8 plane strain
and Hexa20, total-Lagrangian Neo-Hooke), and the allocation-free one twice in a row, so the second
call starts from the counter value the first one left in the shared scratch.  Every result must
match the caller-counter entry point within the parity tolerances of the batch tests (FP64:
1e-12 relative; mixed: P, F 1e-12, K 2e-6).  This file is collected last, so the test also runs
after the rest of the suite has used the library on the same device.
"""

import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _meshes(seed):
    from edelweissfe_gb300 import meshes

    rng = np.random.default_rng(seed)
    out2, out3 = [], []
    for k, n in enumerate([4, 6, 3]):
        coords, conn, nodeDof, nDof = meshes.rect(n, 2 + k, lX=1.0, lY=0.7, nNodes=8)
        Fbar = np.eye(2) + 0.05 * rng.normal(size=(2, 2))
        disp = coords @ (Fbar - np.eye(2)).T + 0.002 * rng.normal(size=coords.shape)
        U = np.zeros(nDof)
        used = nodeDof >= 0
        for c in range(2):
            U[nodeDof[used] + c] = disp[used, c]
        mu = 10 ** rng.uniform(2, 4)
        out2.append(dict(coords=coords, conn=conn, nodeDof=nodeDof, nDof=nDof, props=[mu, 10 * mu], thickness=1.0, U=U))
    for k, n in enumerate([3, 2]):
        coords, conn, nodeDof, nDof = meshes.box(n, 2, 2 - k, nNodes=20)
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


def test_noalloc_rejects_bad_arguments_without_a_gpu():
    """Argument checks return before any CUDA call."""
    from edelweissfe_gb300 import _lib as L

    try:
        lib = L.load()
    except (RuntimeError, OSError) as e:
        pytest.skip(f"library not built: {e}")
    assert lib.efe_compute_elements_persistent_noalloc(None, 2, L.EFE_K_FP64, None, None) == L.EFE_ERR_ARGUMENT
    assert b"work items" in lib.efe_last_error()
    items = (L.EfeWorkItem * 2)()
    status = (ctypes.c_int32 * 4)()
    rc = lib.efe_compute_elements_persistent_noalloc(items, 2, 7, ctypes.addressof(status), None)
    assert rc == L.EFE_ERR_ARGUMENT and b"precision" in lib.efe_last_error()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_noalloc_pass_matches_persistent_pass(precision):
    from edelweissfe_gb300 import _lib as L
    from edelweissfe_gb300.batch import MeshBatch

    lib = L.load()
    m2, m3 = _meshes(5)
    b2 = MeshBatch(m2, "CPE8RTL", "neohookewa", precision)
    b3 = MeshBatch(m3, "C3D20TL", "neohookewa", precision)
    for b, ms in ((b2, m2), (b3, m3)):
        b.U.copy_(torch.tensor(np.concatenate([m["U"] for m in ms])))
    batches = (b3, b2)
    items = (L.EfeWorkItem * 2)(*[
        L.EfeWorkItem(ctypes.addressof(b.asm.mesh), ctypes.addressof(b.asm._groups_c[0]), b.U.data_ptr(),
                      b.dU.data_ptr(), b.K.data_ptr(), b.P.data_ptr(), b.F.data_ptr())
        for b in batches
    ])  # fmt: skip
    kprec = {torch.float32: L.EFE_K_FP32, torch.float64: L.EFE_K_FP64}[b2.K.dtype]
    dev = b2.U.device
    status = torch.zeros(4, dtype=torch.int32, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def run(noalloc):
        for b in batches:  # outputs are accumulated into: the caller zeroes them
            b.P.zero_()
            b.F.zero_()
            b.K.zero_()
        status.zero_()
        if noalloc:
            rc = lib.efe_compute_elements_persistent_noalloc(items, 2, kprec, ctypes.c_void_p(status.data_ptr()), stream)
            L.check(rc, "efe_compute_elements_persistent_noalloc")
        else:
            counter = torch.zeros(1, dtype=torch.int64, device=dev)
            rc = lib.efe_compute_elements_persistent(items, 2, kprec, ctypes.c_void_p(counter.data_ptr()),
                                                     ctypes.c_void_p(status.data_ptr()), stream)  # fmt: skip
            L.check(rc, "efe_compute_elements_persistent")
        torch.cuda.synchronize()
        assert int(status[0]) == 0, status.cpu().numpy()
        return [(b.P.cpu().numpy().copy(), b.F.cpu().numpy().copy(), b.K.double().cpu().numpy().copy())
                for b in batches]  # fmt: skip

    expected = run(noalloc=False)
    ktol = 1e-12 if precision == "fp64" else 2e-6
    for call in range(2):
        got = run(noalloc=True)
        for (P, F, K), (Pe, Fe, Ke) in zip(got, expected):
            assert np.abs(Pe).max() > 0 and np.abs(Ke).max() > 0
            assert _rel(P, Pe) <= 1e-12, call
            assert _rel(F, Fe) <= 1e-12, call
            assert _rel(K, Ke) <= ktol, call
