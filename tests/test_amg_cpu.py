"""Set-up of the aggregation multigrid preconditioner on the CPU (the functions are device-agnostic
torch code; the cycle itself runs through the CUDA kernels and is tested in test_gpu_amg.py):
the point graph against the CSR pattern, the aggregation (an independent set of roots, every point
next to its root), the Galerkin map S against SciPy's P^T A P, and the Chebyshev smoother's
polynomial against the min-max bound 1 / T_k."""

import numpy as np
import pytest
import scipy.sparse as sp

torch = pytest.importorskip("torch")

from edelweissfe_gb300 import amg, meshes  # noqa: E402
from edelweissfe_gb300.pattern import build_pattern  # noqa: E402


def _box_pattern(nx, ny, nz, nNodes=8):
    coords, conn, nodeDof, nDof = meshes.box(nx, ny, nz, nNodes=nNodes)
    indptr, indices = build_pattern(3, len(coords), nodeDof, nDof, [conn])[:2]
    return coords, np.asarray(indptr), np.asarray(indices), nDof


def test_point_graph_matches_pattern():
    _, ip, ix, n = _box_pattern(3, 2, 2)
    src, dst = amg.point_graph(torch.from_numpy(ip), torch.from_numpy(ix), 3)
    got = set(zip(src.tolist(), dst.tolist()))
    want = {(p, int(c) // 3) for p in range(n // 3) for c in ix[ip[3 * p] : ip[3 * p + 1]]}
    assert got == want
    assert all((p, p) in got for p in range(n // 3))


@pytest.mark.parametrize("nNodes", [8, 20])
def test_aggregation_is_a_maximal_independent_set(nNodes):
    _, ip, ix, n = _box_pattern(5, 4, 3, nNodes)
    src, dst = amg.point_graph(torch.from_numpy(ip), torch.from_numpy(ix), 3)
    points = n // 3
    agg, nAgg, roots = amg.mis_aggregate(src, dst, points, seed=3)
    agg2, nAgg2, _ = amg.mis_aggregate(src, dst, points, seed=3)
    assert torch.equal(agg, agg2) and nAgg == nAgg2
    s, d = src.numpy(), dst.numpy()
    r = roots.numpy()
    off = s != d
    assert not np.any(r[s[off]] & r[d[off]])  # no two roots adjacent
    a = agg.numpy()
    assert sorted(set(a.tolist())) == list(range(nAgg))
    rootOfAgg = np.empty(nAgg, np.int64)
    rootOfAgg[a[r]] = np.nonzero(r)[0]
    adj = set(zip(s.tolist(), d.tolist()))
    for p in range(points):  # every point is its aggregate's root or next to it
        q = rootOfAgg[a[p]]
        assert p == q or (p, q) in adj
    assert 1.5 < points / nAgg < 40


def _rect_pattern(nx, ny, nNodes=8):
    coords, conn, nodeDof, nDof = meshes.rect(nx, ny, lX=1.0, lY=0.7, nNodes=nNodes)
    indptr, indices = build_pattern(2, len(coords), nodeDof, nDof, [conn])[:2]
    return coords, np.asarray(indptr), np.asarray(indices), nDof


@pytest.mark.parametrize("dim", [3, 2])
def test_galerkin_map_and_transfer_match_scipy(dim):
    coords, ip, ix, n = _box_pattern(4, 3, 3) if dim == 3 else _rect_pattern(6, 4)
    rng = np.random.default_rng(0)
    vals = rng.normal(size=len(ix))
    A = sp.csr_matrix((vals, ix, ip), shape=(n, n))
    A = (A + A.T).tocsr()  # symmetric values on the same pattern
    A.sort_indices()
    ipT, ixT = torch.from_numpy(A.indptr.astype(np.int32)), torch.from_numpy(A.indices.astype(np.int32))
    src, dst = amg.point_graph(ipT, ixT, dim)
    agg, nAgg, _ = amg.mis_aggregate(src, dst, n // dim, seed=1)
    nc = nAgg * dim
    mask = torch.ones(n, dtype=torch.float64)
    mask[torch.from_numpy(np.arange(0, n, 7))] = 0.0  # some prescribed DOFs
    coarseOfDof = torch.repeat_interleave(agg, dim) * dim + torch.arange(n) % dim
    cnt = torch.zeros(nc, dtype=torch.float64).index_add_(0, coarseOfDof, mask)
    w = mask / torch.sqrt(torch.clamp(cnt, min=1.0))[coarseOfDof]
    (Pp, Pi, Pv), (Rp, Ri, Rv) = amg.transfer(coarseOfDof, w, nc)
    P = sp.csr_matrix((Pv.numpy(), Pi.numpy(), Pp.numpy()), shape=(n, nc))
    R = sp.csr_matrix((Rv.numpy(), Ri.numpy(), Rp.numpy()), shape=(nc, n))
    assert abs(R - P.T).max() == 0.0
    # columns of P are orthonormal on the aggregates that hold a free DOF
    G = (P.T @ P).toarray()
    assert np.allclose(G, np.diag((cnt.numpy() > 0).astype(float)), atol=1e-15)
    (cp, ci), (Sp, Si, Sv), diag = amg.galerkin_map(ipT, ixT, coarseOfDof, w, nc)
    S = sp.csr_matrix((Sv.numpy(), Si.numpy(), Sp.numpy()), shape=(len(Sp) - 1, A.nnz))
    Ac = sp.csr_matrix((S @ A.data, ci.numpy(), cp.numpy()), shape=(nc, nc))
    ref = (P.T @ A @ P).tocsr()
    assert abs(Ac - ref).max() <= 1e-13 * abs(ref).max()
    assert np.all(ci.numpy()[diag.numpy()] == np.arange(nc))


@pytest.mark.parametrize("degree", [1, 2, 3, 4])
def test_chebyshev_polynomial_meets_the_minmax_bound(degree):
    lmax = 3.7
    coeffs = amg.chebyshev_coefficients(lmax, degree)
    a, b = lmax / 30.0, 1.1 * lmax
    theta, delta = 0.5 * (a + b), 0.5 * (b - a)
    bound = 1.0 / np.cosh(degree * np.arccosh(theta / delta))
    lam = np.linspace(a, b, 2001)
    # scalar run of the smoother from z = 0 on A = lam, D = 1, r = 1 (as the kernels do it)
    res, d, z = np.ones_like(lam), np.zeros_like(lam), np.zeros_like(lam)
    for k, (c1, c2) in enumerate(coeffs):
        if k > 0:
            res = res - lam * d
        d = c1 * d + c2 * res
        z = z + d
    err = 1.0 - lam * z
    assert np.max(np.abs(err)) <= bound * (1 + 1e-12)
    assert np.max(np.abs(err)) >= bound * (1 - 1e-9)  # equioscillation: the bound is attained


class _CpuOps:
    """The five product/smoother entry points of AggregationAMG in torch CPU arithmetic, so the
    cycle's orchestration runs here (the product routes them to the CUDA kernels)."""

    def _csr(self, nRows, nCols, indptr, indices, values, kp, mask=None, rowBlock=0):
        ip = indptr.to(torch.int64)
        rows = torch.repeat_interleave(torch.arange(nRows), ip[1:] - ip[:-1])
        return dict(rows=rows, cols=indices.to(torch.int64), vals=values.to(torch.float64), n=nRows, mask=mask)

    def _gemv(self, A, x, alpha, beta, y):
        ax = torch.zeros(A["n"], dtype=torch.float64).index_add_(0, A["rows"], A["vals"] * x[A["cols"]])
        if A["mask"] is not None:
            ax = torch.where(A["mask"] > 0, ax, x)
        y.copy_(alpha * ax if beta == 0.0 else alpha * ax + beta * y)

    def _gemv_pairs(self, A, pairs, alpha, beta, y):
        self._gemv(A, pairs[:, 0].double() + pairs[:, 1].double(), alpha, beta, y)

    def _split(self, x, pairs):
        pairs[:, 0] = x.float()
        pairs[:, 1] = (x - pairs[:, 0].double()).float()

    def _cheb(self, lev, c1, c2, accumulate):
        s = c2 * (lev.dinv * lev.res)
        lev.d.copy_(s if c1 == 0.0 else c1 * lev.d + s)
        lev.z.copy_(lev.z + lev.d if accumulate else lev.d)
        if lev.ff:
            self._split(lev.d, lev.dFF)


def _elastic_system(precision=torch.float64):
    """Linear-elastic C3D8 block (10x8x6, oracle assembly): CSR pattern, K values, free mask
    (bottom face fixed), diagonal positions."""
    from oracle.assembly import Model

    coords, conn, nodeDof, nDof = meshes.box(10, 8, 6, nNodes=8)
    om = Model(coords, nodeDof, nDof, [dict(elType="C3D8", kind="linearelastic", props=np.tile([210e3, 0.3], (len(conn), 1)),
                                            conn=conn, thickness=np.ones(len(conn)), order=np.arange(len(conn)))])  # fmt: skip
    K = om.compute_elements(np.zeros(nDof), np.zeros(nDof), om.initial_state())["Kdata"]
    mask = np.ones(nDof, np.uint8)
    mask[(nodeDof[coords[:, 2] < 1e-9][:, None] + np.arange(3)).ravel()] = 0
    ip, ix = om.indptr.astype(np.int32), om.indices.astype(np.int32)
    rows = np.repeat(np.arange(nDof), np.diff(ip))
    diag = np.nonzero(ix == rows)[0]
    return (torch.from_numpy(ip), torch.from_numpy(ix), torch.from_numpy(K).to(precision), torch.from_numpy(mask),
            torch.from_numpy(diag), nDof)  # fmt: skip


@pytest.mark.parametrize("precision,degree", [(torch.float64, 1), (torch.float64, 2), (torch.float32, 1)])
def test_vcycle_is_a_symmetric_positive_definite_preconditioner(precision, degree):
    """M^-1 = one V-cycle (three levels here): x.M^-1 y = y.M^-1 x and x.M^-1 x > 0 on the free DOFs,
    zero output on the prescribed DOFs; CG with it solves the masked system (against SciPy) in fewer
    iterations than point-Jacobi CG."""
    import scipy.sparse.linalg as sla

    class CpuAMG(_CpuOps, amg.AggregationAMG):
        pass

    ip, ix, K, mask, diag, n = _elastic_system(precision)
    h = CpuAMG(ip, ix, mask, 3, coarseSize=30, degree=degree)
    assert len(h.levels) >= 3, h.describe()
    h.update(K, diag)
    m = mask.double()
    rng = np.random.default_rng(0)

    def M(v):
        z = torch.empty(n, dtype=torch.float64)
        h.apply(v * m, z)
        return z

    x, y = (torch.from_numpy(rng.normal(size=n)) * m for _ in range(2))
    Mx, My = M(x), M(y)
    assert float((Mx * (1 - m)).abs().max()) == 0.0
    tol = 1e-12 if precision == torch.float64 else 1e-7  # float-float level 0 rounds at ~2^-48 per product
    assert abs(float(x @ My) - float(y @ Mx)) <= tol * float(x.abs().sum() * My.abs().sum())
    for _ in range(5):
        v = torch.from_numpy(rng.normal(size=n)) * m
        assert float(v @ M(v)) > 0
    # CG on the free DOFs with M against point Jacobi and SciPy
    Kd = K.double().numpy()
    A = sp.csr_matrix((Kd, ix.numpy(), ip.numpy()), shape=(n, n))
    mm = m.numpy()
    Am = sp.diags(mm) @ A @ sp.diags(mm) + sp.diags(1 - mm)
    b = rng.normal(size=n) * mm
    ref = sla.spsolve(Am.tocsc(), b)

    def cg(prec):
        x = np.zeros(n)
        r = b.copy()
        z = prec(r)
        p = z.copy()
        rz = r @ z
        for it in range(1, 2000):
            Ap = Am @ p
            a = rz / (p @ Ap)
            x += a * p
            r -= a * Ap
            if np.linalg.norm(r) <= 1e-10 * np.linalg.norm(b):
                return x, it
            z = prec(r)
            rzn = r @ z
            p = z + rzn / rz * p
            rz = rzn
        return x, 2000

    xa, ia = cg(lambda r: M(torch.from_numpy(r)).numpy())
    dj = np.where(mm > 0, 1.0 / Am.diagonal(), 1.0)
    xj, ij = cg(lambda r: dj * r)
    assert np.abs(xa - ref).max() <= 1e-8 * np.abs(ref).max()
    assert ia < ij / 2, (ia, ij)
