"""Aggregation multigrid preconditioner on the device: the two kernels it is built from
(efe_csr_gemv, efe_chebyshev_step) against SciPy / torch, the level operators of
AggregationAMG.update against SciPy's P^T A P, and CG with the V-cycle against SciPy's direct
solve of the Dirichlet-reduced tangent (1e-9), bitwise repeatable, with fewer iterations than
point Jacobi; a Newton run with it reaches the same solution as with point Jacobi."""

import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


@pytest.mark.parametrize("vdtype", [torch.float64, torch.float32])
def test_gemv_matches_scipy(vdtype):
    import scipy.sparse as sp

    from edelweissfe_gb300 import _lib as L

    lib = L.load()
    rng = np.random.default_rng(2)
    dev = torch.device("cuda", 0)
    for nRows, nCols, density in [(1000, 37, 0.05), (37, 1000, 0.05), (4000, 300, 0.003), (513, 513, 0.05)]:
        A = sp.random(nRows, nCols, density=density, random_state=3, format="csr")
        A.sort_indices()
        v = A.data.astype(np.float32 if vdtype == torch.float32 else np.float64)
        ip = torch.tensor(A.indptr, dtype=torch.int32, device=dev)
        ix = torch.tensor(A.indices, dtype=torch.int32, device=dev)
        vals = torch.tensor(v, device=dev)
        x = torch.tensor(rng.normal(size=nCols), device=dev)
        y0 = rng.normal(size=nRows)
        kp = L.EFE_K_FP64 if vdtype == torch.float64 else L.EFE_K_FP32
        mask = None
        if nRows == nCols:
            mask = torch.tensor(rng.random(nRows) > 0.2, dtype=torch.uint8, device=dev)
        csr = L.EfeCsr(nRows, nCols, A.nnz, ip.data_ptr(), ix.data_ptr(), vals.data_ptr(), kp,
                       mask.data_ptr() if mask is not None else None)  # fmt: skip
        Ah = sp.csr_matrix((v.astype(np.float64), A.indices, A.indptr), shape=(nRows, nCols))
        ax = Ah @ x.cpu().numpy()
        if mask is not None:
            mh = mask.cpu().numpy() > 0
            ax = np.where(mh, ax, x.cpu().numpy())
        for alpha, beta in [(1.0, 0.0), (-1.0, 1.0), (0.5, -2.0)]:
            y = torch.tensor(y0, device=dev)
            L.check(lib.efe_csr_gemv(ctypes.byref(csr), ctypes.c_void_p(x.data_ptr()), alpha, beta,
                                     ctypes.c_void_p(y.data_ptr()), _stream()), "efe_csr_gemv")  # fmt: skip
            ref = alpha * ax + (beta * y0 if beta != 0.0 else 0.0)
            assert np.abs(y.cpu().numpy() - ref).max() <= 1e-13 * max(np.abs(ref).max(), 1.0)
    # argument errors
    bad = L.EfeCsr(3, 4, 1, ip.data_ptr(), ix.data_ptr(), vals.data_ptr(), L.EFE_K_FP64, mask.data_ptr())
    assert lib.efe_csr_gemv(ctypes.byref(bad), None, 1.0, 0.0, None, None) == L.EFE_ERR_ARGUMENT


def test_chebyshev_step_matches_formula():
    from edelweissfe_gb300 import _lib as L

    lib = L.load()
    dev = torch.device("cuda", 0)
    g = torch.Generator().manual_seed(4)
    n = 100003
    dinv, r, d0, z0 = (torch.rand(n, generator=g, dtype=torch.float64).to(dev) for _ in range(4))
    for c1, c2, acc in [(0.0, 0.7, 0), (0.3, -1.2, 1), (1.5, 0.25, 0)]:
        d, z = d0.clone(), z0.clone()
        dp = torch.empty((n, 2), dtype=torch.float32, device=dev)
        L.check(lib.efe_chebyshev_step(n, ctypes.c_void_p(dinv.data_ptr()), ctypes.c_void_p(r.data_ptr()), c1, c2, acc,
                                       ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(z.data_ptr()),
                                       ctypes.c_void_p(dp.data_ptr()), _stream()), "efe_chebyshev_step")  # fmt: skip
        assert bool(((dp[:, 0].double() + dp[:, 1].double() - d).abs() <= 2.0**-46 * d.abs()).all())
        dref = c1 * d0 + c2 * (dinv * r)
        zref = z0 + dref if acc else dref
        # the kernel fuses c1 d + s into one rounding: compare on the scale of the terms
        scale = (c1 * d0).abs() + (c2 * dinv * r).abs()
        assert bool(((d - dref).abs() <= 4e-16 * scale).all())
        assert bool(((z - zref).abs() <= 4e-16 * (scale + (z0.abs() if acc else 0.0))).all())


def test_pairs_product_and_split():
    """efe_split_pairs gives hi + lo = x to ~2^-48; efe_csr_gemv_pairs agrees with the FP64 product
    of the same float values to ~1e-13 of sum |A_ij x_j|."""
    import scipy.sparse as sp

    from edelweissfe_gb300 import _lib as L

    lib = L.load()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(5)
    n = 2000
    A = sp.random(n, n, density=0.02, random_state=6, format="csr")
    A.sort_indices()
    v = A.data.astype(np.float32)
    ip = torch.tensor(A.indptr, dtype=torch.int32, device=dev)
    ix = torch.tensor(A.indices, dtype=torch.int32, device=dev)
    vals = torch.tensor(v, device=dev)
    x = torch.tensor(rng.normal(size=n), device=dev)
    pairs = torch.empty((n, 2), dtype=torch.float32, device=dev)
    L.check(lib.efe_split_pairs(n, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(pairs.data_ptr()), _stream()),
            "efe_split_pairs")  # fmt: skip
    back = pairs[:, 0].double() + pairs[:, 1].double()
    assert bool(((back - x).abs() <= 2.0**-46 * x.abs()).all())
    mask = torch.tensor(rng.random(n) > 0.1, dtype=torch.uint8, device=dev)
    csr = L.EfeCsr(n, n, A.nnz, ip.data_ptr(), ix.data_ptr(), vals.data_ptr(), L.EFE_K_FP32, mask.data_ptr())
    Ah = sp.csr_matrix((v.astype(np.float64), A.indices, A.indptr), shape=(n, n))
    xh = back.cpu().numpy()
    ref = np.where(mask.cpu().numpy() > 0, Ah @ xh, xh)
    scale = np.where(mask.cpu().numpy() > 0, abs(Ah) @ np.abs(xh), np.abs(xh))
    for alpha, beta in [(1.0, 0.0), (-1.0, 1.0)]:
        y0 = rng.normal(size=n)
        y = torch.tensor(y0, device=dev)
        L.check(lib.efe_csr_gemv_pairs(ctypes.byref(csr), ctypes.c_void_p(pairs.data_ptr()), alpha, beta,
                                       ctypes.c_void_p(y.data_ptr()), _stream()), "efe_csr_gemv_pairs")  # fmt: skip
        want = alpha * ref + beta * y0
        assert np.all(np.abs(y.cpu().numpy() - want) <= 1e-13 * scale + 1e-15 * np.abs(want))
    # FP64 values are rejected: the pairs product is for float tangents
    csr64 = L.EfeCsr(n, n, A.nnz, ip.data_ptr(), ix.data_ptr(), vals.data_ptr(), L.EFE_K_FP64, None)
    assert lib.efe_csr_gemv_pairs(ctypes.byref(csr64), ctypes.c_void_p(pairs.data_ptr()), 1.0, 0.0,
                                  ctypes.c_void_p(y.data_ptr()), None) == L.EFE_ERR_ARGUMENT  # fmt: skip


@pytest.mark.parametrize("elType", ["C3D8", "C3D20", "CPE8"])
def test_row_group_products_match_row_products(elType):
    """The node-row-group forms of the float-float products (one column index per node row group)
    against the per-row forms on an assembled tangent: CG product and efe_csr_gemv_pairs."""
    from edelweissfe_gb300 import ElementGroup, GPUAssembler, _lib as L, meshes

    lib = L.load()
    if elType == "CPE8":
        coords, conn, nodeDof, nDof = meshes.rect(9, 7, lX=1.0, lY=0.7, nNodes=8)
        props = [210e3, 0.3]
        mat = "linearelastic"
    else:
        coords, conn, nodeDof, nDof = meshes.box(5, 4, 3, nNodes=20 if "20" in elType else 8)
        props = [210e3, 0.3, 250, 1000, 0, 0]
        mat = "vonmises"
    asm = GPUAssembler(coords, nodeDof, nDof, [ElementGroup(elType, mat, props, conn)], precision="mixed")
    assert asm.rowGroup == asm.dim
    P, F, K = asm.constructDofVector(), asm.constructDofVector(), asm.constructSystemMatrix()
    rng = np.random.default_rng(8)
    asm.launch(torch.tensor(rng.normal(0, 1e-3, nDof), device=asm.device), asm.constructDofVector(), P, K, F)
    torch.cuda.synchronize()
    dev = asm.device
    x = torch.tensor(rng.normal(size=nDof), device=dev)
    pairs = torch.empty((nDof, 2), dtype=torch.float32, device=dev)
    L.check(lib.efe_split_pairs(nDof, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(pairs.data_ptr()), _stream()),
            "efe_split_pairs")  # fmt: skip
    mask = torch.tensor(rng.random(nDof) > 0.1, dtype=torch.uint8, device=dev)
    out = []
    for rb in (0, asm.dim):
        csr = L.EfeCsr(nDof, nDof, asm.nnz, asm.indptr.data_ptr(), asm.indices.data_ptr(), K.data_ptr(), L.EFE_K_FP32,
                       mask.data_ptr(), rb)  # fmt: skip
        y = torch.empty(nDof, dtype=torch.float64, device=dev)
        L.check(lib.efe_csr_gemv_pairs(ctypes.byref(csr), ctypes.c_void_p(pairs.data_ptr()), 1.0, 0.0,
                                       ctypes.c_void_p(y.data_ptr()), _stream()), "efe_csr_gemv_pairs")  # fmt: skip
        out.append(y.cpu().numpy())
    import scipy.sparse as sp

    Ah = sp.csr_matrix((K.double().cpu().numpy(), asm.indices_host, asm.indptr_host), shape=(nDof, nDof))
    xh = (pairs[:, 0].double() + pairs[:, 1].double()).cpu().numpy()
    mh = mask.cpu().numpy() > 0
    ref = np.where(mh, Ah @ xh, xh)
    scale = np.where(mh, abs(Ah) @ np.abs(xh), np.abs(xh))
    for y in out:
        assert np.all(np.abs(y - ref) <= 1e-13 * scale)


def _system(elType, precision, n=(6, 5, 4), jitter=True):
    from edelweissfe_gb300 import ElementGroup, GPUAssembler, meshes
    from edelweissfe_gb300.solver import NISTGPU

    coords, conn, nodeDof, nDof = meshes.box(*n, nNodes=20 if "20" in elType else 8)
    if jitter:
        coords = meshes.jitter(coords, 0.1, [1 / n[0], 1 / n[1], 1 / n[2]], 3, [0, 0, 0], [1, 1, 1])
    asm = GPUAssembler(coords, nodeDof, nDof, [ElementGroup(elType, "vonmises", [210e3, 0.3, 250, 1000, 0, 0], conn)],
                       precision=precision)  # fmt: skip
    fixed = np.unique(np.concatenate([(nodeDof[coords[:, 1] < 1e-9][:, None] + np.arange(3)).ravel(),
                                      nodeDof[coords[:, 1] > 1 - 1e-9] + 1]))  # fmt: skip
    return asm, NISTGPU, fixed, nDof


@pytest.mark.parametrize("elType,precision", [("C3D8", "fp64"), ("C3D8", "mixed"), ("C3D20", "mixed")])
def test_amg_pcg_matches_direct_solve(elType, precision):
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla

    asm, NISTGPU, fixed, nDof = _system(elType, precision)
    amgSolver = NISTGPU(asm, pcgTolerance=1e-14, pcgPreconditioner="amg", amgOptions=dict(coarseSize=50))
    jacobi = NISTGPU(asm, pcgTolerance=1e-14)
    rng = np.random.default_rng(1)
    K = amgSolver.tangentAt(torch.tensor(rng.normal(0, 1e-3, nDof), device=asm.device))
    R = torch.tensor(rng.normal(0, 1, nDof), device=asm.device)
    dir_idx = torch.as_tensor(fixed, device=asm.device)
    x1 = amgSolver._solve_pcg(K, R, dir_idx)
    x2 = amgSolver._solve_pcg(K, R, dir_idx)
    xj = jacobi._solve_pcg(K, R, dir_idx)
    assert torch.equal(x1, x2)
    assert len(amgSolver._amg.levels) >= 3, amgSolver._amg.describe()
    assert amgSolver.linearIterations[-1] < jacobi.linearIterations[-1], (amgSolver.linearIterations,
                                                                           jacobi.linearIterations)  # fmt: skip
    A = sp.csr_matrix((K.double().cpu().numpy(), asm.indices_host, asm.indptr_host), shape=(nDof, nDof))
    free = np.setdiff1d(np.arange(nDof), fixed)
    Rh = R.cpu().numpy()
    ref = np.zeros(nDof)
    ref[fixed] = Rh[fixed]
    ref[free] = sla.spsolve(A[free][:, free].tocsc(), Rh[free] - A[free][:, fixed] @ Rh[fixed])
    for x in (x1, xj):
        assert np.abs(x.cpu().numpy() - ref).max() <= 1e-9 * np.abs(ref).max()


def test_amg_level_operators_are_galerkin_products():
    import scipy.sparse as sp

    asm, NISTGPU, fixed, nDof = _system("C3D8", "fp64")
    solver = NISTGPU(asm, pcgTolerance=1e-10, pcgPreconditioner="amg", amgOptions=dict(coarseSize=100))
    K = solver.tangentAt(torch.zeros(nDof, dtype=torch.float64, device=asm.device))
    solver._solve_pcg(K, torch.ones(nDof, dtype=torch.float64, device=asm.device), torch.as_tensor(fixed, device=asm.device))
    h = solver._amg
    m = np.ones(nDof)
    m[fixed] = 0.0
    A = sp.csr_matrix((K.cpu().numpy(), asm.indices_host, asm.indptr_host), shape=(nDof, nDof))
    A = (sp.diags(m) @ A @ sp.diags(m)).tocsr()
    for k in range(len(h.levels) - 1):
        lev, nxt = h.levels[k], h.levels[k + 1]
        Pp, Pi, Pv = (t.cpu().numpy() for t in lev.P)
        P = sp.csr_matrix((Pv, Pi, Pp), shape=(lev.n, nxt.n))
        ref = (P.T @ A @ P).toarray()
        empty = nxt.empty.cpu().numpy()
        ref[empty, empty] = 1.0
        got = sp.csr_matrix((nxt.values.cpu().numpy(), nxt.indices.cpu().numpy(), nxt.indptr.cpu().numpy()),
                            shape=(nxt.n, nxt.n)).toarray()  # fmt: skip
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
        A = sp.csr_matrix(got)


def test_newton_with_amg_matches_jacobi():
    """The 6^3 jittered von Mises cube, 4 increments of uniaxial displacement: the same Newton
    iterations and displacements with either preconditioner, fewer CG iterations with the V-cycle."""
    from edelweissfe_gb300 import ElementGroup, GPUAssembler, meshes
    from edelweissfe_gb300.solver import AdaptiveTimeStepper, Dirichlet, NISTGPU

    c, conn, nodeDof, nDof = meshes.box(6, 6, 6, nNodes=8)
    c = meshes.jitter(c, 0.1, [1 / 6, 1 / 6, 1 / 6], 3, [0, 0, 0], [1, 1, 1])
    bcs = [Dirichlet(nodeDof[c[:, 1] < 1e-9] + 1, 0.0), Dirichlet(nodeDof[c[:, 0] < 1e-9], 0.0),
           Dirichlet(nodeDof[c[:, 2] < 1e-9] + 2, 0.0), Dirichlet(nodeDof[c[:, 1] > 1 - 1e-9] + 1, 0.004)]  # fmt: skip
    out = {}
    for pre in ("jacobi", "amg"):
        asm = GPUAssembler(c, nodeDof, nDof, [ElementGroup("C3D8", "vonmises", [210e3, 0.3, 250, 1000, 0, 0], conn)],
                           precision="mixed")  # fmt: skip
        s = NISTGPU(asm, linsolver="pcg", extrapolation="linear", maxIter=15, fluxResidualTolerance=1e-10,
                    fieldCorrectionTolerance=1e-10, fluxResidualFloor=0.0, pcgTolerance=1e-12, pcgPreconditioner=pre,
                    amgOptions=dict(coarseSize=100))  # fmt: skip
        U = s.solveStep(AdaptiveTimeStepper(maxIncrement=0.25, startIncrement=0.25), bcs)
        out[pre] = (U.cpu().numpy().copy(), [h["iterations"] for h in s.history], sum(s.linearIterations))
    Uj, itj, pj = out["jacobi"]
    Ua, ita, pa = out["amg"]
    # the linear solves agree to the CG tolerance, not bitwise: an increment whose residual lands
    # at the Newton tolerance may take one iteration more or less
    assert len(ita) == len(itj) and all(abs(a - b) <= 1 for a, b in zip(ita, itj)), (ita, itj)
    assert np.abs(Ua - Uj).max() <= 1e-8 * np.abs(Uj).max()
    assert pa < pj, (pa, pj)
