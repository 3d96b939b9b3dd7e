"""Device linear solve (efe_csr_spmv, efe_pcg_start, efe_pcg_iterate; nodal block-Jacobi and point
Jacobi preconditioners) against SciPy's direct solve of the same system: the assembled tangent of a jittered Hexa8 / Hexa20 von Mises block (FP64 and FP32
CSR data), a random right-hand side and a set of prescribed DOFs whose values are carried by the
right-hand side (identity rows, as applyDirichletK).  PCG relative tolerance 1e-14: solutions
agree to 1e-9 relative; two runs are bitwise identical (fixed-order reductions)."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("preconditioner", ["block", "jacobi"])
@pytest.mark.parametrize("elType,precision", [("C3D8", "fp64"), ("C3D8", "mixed"), ("C3D20", "mixed")])
def test_pcg_matches_direct_solve(elType, precision, preconditioner):
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla

    from edelweissfe_gb300 import ElementGroup, GPUAssembler, meshes
    from edelweissfe_gb300.solver import NISTGPU

    coords, conn, nodeDof, nDof = meshes.box(4, 3, 2, nNodes=20 if "20" in elType else 8)
    coords = meshes.jitter(coords, 0.1, [0.25, 1 / 3, 0.5], 3, [0, 0, 0], [1, 1, 1])
    asm = GPUAssembler(coords, nodeDof, nDof, [ElementGroup(elType, "vonmises", [210e3, 0.3, 250, 1000, 0, 0], conn)],
                       precision=precision)  # fmt: skip
    solver = NISTGPU(asm, pcgTolerance=1e-14, pcgPreconditioner=preconditioner)
    rng = np.random.default_rng(1)
    U = torch.tensor(rng.normal(0, 1e-3, nDof), device=asm.device)
    K = solver.tangentAt(U)
    fixed = np.unique(np.concatenate([(nodeDof[coords[:, 1] < 1e-9][:, None] + np.arange(3)).ravel(),
                                      nodeDof[coords[:, 1] > 1 - 1e-9] + 1]))  # fmt: skip
    R = torch.tensor(rng.normal(0, 1, nDof), device=asm.device)
    dir_idx = torch.as_tensor(fixed, device=asm.device)
    x1 = solver._solve_pcg(K, R, dir_idx)
    x2 = solver._solve_pcg(K, R, dir_idx)
    assert torch.equal(x1, x2)
    assert 0 < solver.linearIterations[-1] < 2000
    assert solver.linearConverged[-1] and solver.linearResiduals[-1] is None
    # a solve cut off by pcgMaxIter says so, with its final relative residual
    short = NISTGPU(asm, pcgTolerance=1e-14, pcgPreconditioner=preconditioner, pcgMaxIter=10)
    short._solve_pcg(K, R, dir_idx)
    assert short.linearIterations == [10] and short.linearConverged == [False]
    assert 1e-14 < short.linearResiduals[0] < 1.0
    A = sp.csr_matrix((K.double().cpu().numpy(), asm.indices_host, asm.indptr_host), shape=(nDof, nDof))
    free = np.setdiff1d(np.arange(nDof), fixed)
    Rh = R.cpu().numpy()
    ref = np.zeros(nDof)
    ref[fixed] = Rh[fixed]
    ref[free] = sla.spsolve(A[free][:, free].tocsc(), Rh[free] - A[free][:, fixed] @ Rh[fixed])
    x = x1.cpu().numpy()
    assert np.abs(x - ref).max() <= 1e-9 * np.abs(ref).max()
    # the product on its own
    from edelweissfe_gb300 import _lib as L
    import ctypes

    v = torch.tensor(rng.normal(0, 1, nDof), device=asm.device)
    y = torch.empty_like(v)
    work = torch.zeros(L.EFE_PCG_WORK_DOUBLES, dtype=torch.float64, device=asm.device)
    kp = L.EFE_K_FP64 if K.dtype == torch.float64 else L.EFE_K_FP32
    s = L.EfePcg(nDof, asm.indptr.data_ptr(), asm.indices.data_ptr(), K.data_ptr(), kp, None, y.data_ptr(),
                 y.data_ptr(), y.data_ptr(), y.data_ptr(), y.data_ptr(), y.data_ptr(), work.data_ptr(), None, 1)  # fmt: skip
    L.check(L.load().efe_csr_spmv(ctypes.byref(s), ctypes.c_void_p(v.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                                  None), "efe_csr_spmv")  # fmt: skip
    torch.cuda.synchronize()
    yr = A @ v.cpu().numpy()
    assert np.abs(y.cpu().numpy() - yr).max() <= 1e-12 * np.abs(yr).max()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_pcg_graph_replay_matches_direct_launches(precision):
    """Long solves replay their iteration batches as a CUDA graph: same iterations, same bits as the
    directly launched batches."""
    from edelweissfe_gb300 import ElementGroup, GPUAssembler, meshes
    from edelweissfe_gb300.solver import NISTGPU

    coords, conn, nodeDof, nDof = meshes.box(6, 5, 4, nNodes=8)
    asm = GPUAssembler(coords, nodeDof, nDof, [ElementGroup("C3D8", "vonmises", [210e3, 0.3, 250, 1000, 0, 0], conn)],
                       precision=precision)  # fmt: skip
    graphs = NISTGPU(asm, pcgTolerance=1e-14)
    direct = NISTGPU(asm, pcgTolerance=1e-14, pcgGraphs=False)
    rng = np.random.default_rng(3)
    K = graphs.tangentAt(torch.tensor(rng.normal(0, 1e-3, nDof), device=asm.device))
    dir_idx = torch.as_tensor(nodeDof[coords[:, 2] < 1e-9][:, None] + np.arange(3), device=asm.device).ravel()
    R = torch.tensor(rng.normal(0, 1, nDof), device=asm.device)
    xg = graphs._solve_pcg(K, R, dir_idx)
    xd = direct._solve_pcg(K, R, dir_idx)
    assert graphs.linearIterations == direct.linearIterations
    assert graphs.linearIterations[-1] >= 40  # at least two graph replays
    assert torch.equal(xg, xd)
