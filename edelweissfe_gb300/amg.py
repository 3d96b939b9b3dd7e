"""Aggregation multigrid preconditioner for the conjugate-gradient solves of the Newton corrections
and adjoint systems on the device.

The reference solves the Newton correction directly (`linearSolve`,
`solvers/nonlinearimplicitstatic.py:727-751`: PARDISO, or SciPy's SuperLU on the row-modified
system of `applyDirichletK`, :559-593) and reaches multilevel methods only through external
libraries.  On the device, point-Jacobi CG needs O(1/h) iterations (about 10^4 per system on a
96 x 96 x 48 Hexa20 block); a V-cycle of plain (unsmoothed) aggregation multigrid brings that to a
few hundred at a few products per iteration.

Hierarchy.  Level 0 is the tangent as assembled (double or float CSR data, int32 pattern) with
identity rows on the prescribed DOFs.  A point is a block of `bs` consecutive DOFs (a node's
displacement components, the DofManager's node-major numbering).  Points are aggregated around
the roots of a maximal independent set of the point graph (random priorities, one neighbour-max
per sweep, every other point joins its highest-priority root neighbour); the coarse space holds
the translations of every aggregate: coarse DOF I = aggregate * bs + component, prolongation
P[i, I] = 1 / sqrt(number of free fine DOFs in I) on free DOFs, 0 on prescribed ones.  The
coarse operator is the Galerkin product P^T A P, summed in a fixed order through a precomputed
sparse map S (one row per coarse entry, one column per fine entry, weight w_i w_j), so a new
tangent costs one CSR product per level.  Coarse DOFs without a free fine DOF get an identity
row.  Coarsening stops at `coarseSize` DOFs, where the operator is inverted densely (Cholesky).

Cycle.  Symmetric V-cycle: Chebyshev smoothing of degree `degree` (default 1: one product per
smoothing pass, fewest level-0 products per solve on the meshes measured) in the point-Jacobi-scaled
operator on the interval [lambda_max / 30, 1.1 lambda_max] (lambda_max from power iterations),
restriction by P^T, the cycle on the next level, prolongation by P, the same smoothing after.
Pre- and post-smoothing are the same polynomial in D^-1 A, so the cycle is a symmetric positive
definite preconditioner.  Every product runs through `efe_csr_gemv` and every smoother step
through `efe_chebyshev_step`; the reductions are cuBLAS dot products (fixed order), so a solve is
bitwise repeatable.  With an FP32 tangent the level-0 products take their vector as float-float
pairs (`efe_csr_gemv_pairs`, FP32 pipe; the smoother writes the pairs of its step as it goes), as
the point-Jacobi CG products do; coarse levels hold FP64 values.
"""

import ctypes

import torch

from . import _lib as L

_ROOT, _UNDECIDED, _OUT = 2, 1, 0
_PRIO_BITS = 40


def point_graph(indptr, indices, bs):
    """Edges (src, dst) of the point graph: point p is adjacent to point q when row p*bs of the
    CSR pattern has a column in q's block (the diagonal gives the self edge).  int64 tensors."""
    n = indptr.numel() - 1
    points = n // bs
    ip = indptr.to(torch.int64)
    start = ip[0:n:bs][:points]
    lens = ip[1 : n + 1 : bs][:points] - start
    src = torch.repeat_interleave(torch.arange(points, device=indptr.device), lens)
    first = torch.cumsum(lens, 0) - lens
    pos = start[src] + (torch.arange(src.numel(), device=indptr.device) - first[src])
    dst = indices.to(torch.int64)[pos] // bs
    return src, dst


def mis_aggregate(src, dst, points, seed=0, maxSweeps=200):
    """Aggregates around the roots of a maximal independent set of the point graph.  Returns
    (agg [points] int64, nAgg, roots [points] bool).  Deterministic for a given seed."""
    dev = src.device
    g = torch.Generator().manual_seed(seed)
    prio = torch.randperm(points, generator=g).to(dev)
    state = torch.full((points,), _UNDECIDED, dtype=torch.int64, device=dev)
    for _ in range(maxSweeps):
        und = state == _UNDECIDED
        if not bool(und.any()):
            break
        key = (state << _PRIO_BITS) | prio
        mx = key.clone()
        mx.scatter_reduce_(0, src, key[dst], reduce="amax")
        newRoot = und & (mx == key)
        out = und & ((mx >> _PRIO_BITS) == _ROOT)
        state[newRoot] = _ROOT
        state[out] = _OUT
    state[state == _UNDECIDED] = _ROOT  # after maxSweeps: the rest are roots of their own (each sweep adds >= 1)
    roots = state == _ROOT
    aggOfRoot = torch.cumsum(roots.to(torch.int64), 0) - 1
    nAgg = int(roots.sum())
    # every other point joins the root neighbour of highest priority
    val = torch.where(roots[dst], prio[dst], torch.full_like(prio[dst], -1))
    best = torch.full((points,), -1, dtype=torch.int64, device=dev)
    best.scatter_reduce_(0, src, val, reduce="amax")
    pointOfPrio = torch.empty_like(prio)
    pointOfPrio[prio] = torch.arange(points, device=dev)
    agg = torch.where(roots, aggOfRoot, aggOfRoot[pointOfPrio[best.clamp(min=0)]])
    if bool((~roots & (best < 0)).any()):
        raise RuntimeError("aggregation left a point without a root neighbour")
    return agg, nAgg, roots


def transfer(coarseOfDof, w, nc):
    """Prolongation P (n x nc, one entry per row) and restriction R = P^T (nc x n) as CSR
    (indptr int32, indices int32, values float64)."""
    n = coarseOfDof.numel()
    dev = coarseOfDof.device
    Pp = torch.arange(n + 1, dtype=torch.int32, device=dev)
    Pi = coarseOfDof.to(torch.int32)
    order = torch.sort(coarseOfDof, stable=True).indices
    counts = torch.bincount(coarseOfDof, minlength=nc)
    Rp = torch.zeros(nc + 1, dtype=torch.int64, device=dev)
    Rp[1:] = torch.cumsum(counts, 0)
    return (Pp, Pi, w.clone()), (Rp.to(torch.int32), order.to(torch.int32), w[order].contiguous())


def galerkin_map(indptr, indices, coarseOfDof, w, nc):
    """Pattern of P^T A P and the map S that sums it: coarse CSR (indptr, indices int32), S as CSR
    (nnz_c x nnz_f: indptr, indices int32, values w_i w_j in fine-entry order per coarse entry),
    and the position of every coarse diagonal entry.  Transient memory: a few int64 arrays of the
    fine entry count and one sort of them (tens of GB at 10^9 entries); S keeps 12 bytes per fine
    entry."""
    n = indptr.numel() - 1
    dev = indices.device
    ip = indptr.to(torch.int64)
    rows = torch.repeat_interleave(torch.arange(n, device=dev), ip[1:] - ip[:-1])
    cols = indices.to(torch.int64)
    I = coarseOfDof[rows]
    J = coarseOfDof[cols]
    key = I * nc + J
    skey, perm = torch.sort(key, stable=True)
    del key, I, J
    ukey, counts = torch.unique_consecutive(skey, return_counts=True)
    del skey
    cRows = ukey // nc
    cCols = ukey % nc
    cIndptr = torch.zeros(nc + 1, dtype=torch.int64, device=dev)
    cIndptr[1:] = torch.cumsum(torch.bincount(cRows, minlength=nc), 0)
    Sp = torch.zeros(ukey.numel() + 1, dtype=torch.int64, device=dev)
    Sp[1:] = torch.cumsum(counts, 0)
    Sv = w[rows[perm]] * w[cols[perm]]
    diag = torch.nonzero(cRows == cCols).flatten()
    if diag.numel() != nc:
        raise RuntimeError("coarse operator without a full diagonal")
    return ((cIndptr.to(torch.int32), cCols.to(torch.int32)),
            (Sp.to(torch.int32), perm.to(torch.int32), Sv), diag)  # fmt: skip


def chebyshev_coefficients(lmax, degree, lo=1.0 / 30.0, hi=1.1):
    """(c1, c2) of each smoother step d_k = c1 d_{k-1} + c2 D^-1 r_k for the Chebyshev polynomial
    on [lo, hi] * lmax (three-term recurrence of the shifted Chebyshev iteration)."""
    a, b = lo * lmax, hi * lmax
    theta, delta = 0.5 * (b + a), 0.5 * (b - a)
    sigma = theta / delta
    rho = 1.0 / sigma
    out = [(0.0, 1.0 / theta)]
    for _ in range(1, degree):
        rhoNew = 1.0 / (2.0 * sigma - rho)
        out.append((rhoNew * rho, 2.0 * rhoNew / delta))
        rho = rhoNew
    return out


class _Level:
    pass


class AggregationAMG:
    """V-cycle preconditioner for A = K on free DOFs, identity on prescribed ones.

    indptr, indices: the tangent's int32 CSR pattern (device); freeMask: uint8 [n] (1 = free);
    bs: DOFs per point.  `update(K)` takes a new tangent's values (same pattern); `apply(r, z)`
    writes z = M^-1 r."""

    def __init__(self, indptr, indices, freeMask, bs, coarseSize=2000, degree=1, maxLevels=12, seed=0,
                 powerIterations=12, rowGroup=1):  # fmt: skip
        self.dev = indices.device
        self.bs = bs
        self.degree = degree
        self.powerIterations = powerIterations
        self.seed = seed
        self.rowGroup = rowGroup  # level-0 rows share column lists in groups of this size
        self.lib = L.load()
        n = indptr.numel() - 1
        if n % bs:
            raise ValueError("the system size is not a multiple of the point size")
        lev = _Level()
        lev.n, lev.indptr, lev.indices, lev.mask = n, indptr, indices, freeMask
        lev.values, lev.kp = None, None
        self.levels = [lev]
        mask = freeMask.to(torch.float64)
        while True:
            lev = self.levels[-1]
            if lev.n <= coarseSize or len(self.levels) >= maxLevels:
                break
            src, dst = point_graph(lev.indptr, lev.indices, bs)
            agg, nAgg, _ = mis_aggregate(src, dst, lev.n // bs, seed=seed + len(self.levels))
            del src, dst
            nc = nAgg * bs
            if nc > 0.8 * lev.n:  # coarsening stalled
                break
            comp = torch.arange(lev.n, device=self.dev) % bs
            coarseOfDof = torch.repeat_interleave(agg, bs) * bs + comp
            cnt = torch.zeros(nc, dtype=torch.float64, device=self.dev)
            cnt.index_add_(0, coarseOfDof, mask)  # integer-valued counts: exact in any order
            w = mask / torch.sqrt(torch.clamp(cnt, min=1.0))[coarseOfDof]
            (lev.P, lev.R) = transfer(coarseOfDof, w, nc)
            (cpat, lev.S, diag) = galerkin_map(lev.indptr, lev.indices, coarseOfDof, w, nc)
            nxt = _Level()
            nxt.n, nxt.indptr, nxt.indices = nc, cpat[0], cpat[1]
            nxt.diag = diag
            nxt.empty = cnt == 0
            nxt.values = torch.zeros(nxt.indices.numel(), dtype=torch.float64, device=self.dev)
            nxt.kp = L.EFE_K_FP64
            nxt.mask = None
            mask = (~nxt.empty).to(torch.float64)
            self.levels.append(nxt)
        for k, lev in enumerate(self.levels):
            lev.r = torch.zeros(lev.n, dtype=torch.float64, device=self.dev)
            lev.z = torch.zeros_like(lev.r)
            lev.res = torch.zeros_like(lev.r)
            lev.d = torch.zeros_like(lev.r)
            lev.dinv = torch.ones_like(lev.r)
            lev.ff = False
        lev0 = self.levels[0]
        lev0.dFF = torch.zeros((lev0.n, 2), dtype=torch.float32, device=self.dev)
        lev0.zFF = torch.zeros_like(lev0.dFF)
        self.dense = None
        self._vals0 = None

    # ---------------------------------------------------------------- products
    def _csr(self, nRows, nCols, indptr, indices, values, kp, mask=None, rowBlock=0):
        return L.EfeCsr(nRows, nCols, indices.numel(), indptr.data_ptr(), indices.data_ptr(), values.data_ptr(), kp,
                        mask.data_ptr() if mask is not None else None, rowBlock)  # fmt: skip

    def _gemv(self, A, x, alpha, beta, y):
        st = ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)
        L.check(self.lib.efe_csr_gemv(ctypes.byref(A), ctypes.c_void_p(x.data_ptr()), alpha, beta,
                                      ctypes.c_void_p(y.data_ptr()), st), "efe_csr_gemv")  # fmt: skip

    def _gemv_pairs(self, A, xPairs, alpha, beta, y):
        st = ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)
        L.check(self.lib.efe_csr_gemv_pairs(ctypes.byref(A), ctypes.c_void_p(xPairs.data_ptr()), alpha, beta,
                                            ctypes.c_void_p(y.data_ptr()), st), "efe_csr_gemv_pairs")  # fmt: skip

    def _split(self, x, pairs):
        st = ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)
        L.check(self.lib.efe_split_pairs(x.numel(), ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(pairs.data_ptr()),
                                         st), "efe_split_pairs")  # fmt: skip

    def _cheb(self, lev, c1, c2, accumulate):
        st = ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)
        L.check(self.lib.efe_chebyshev_step(lev.n, ctypes.c_void_p(lev.dinv.data_ptr()),
                                            ctypes.c_void_p(lev.res.data_ptr()), c1, c2, int(accumulate),
                                            ctypes.c_void_p(lev.d.data_ptr()), ctypes.c_void_p(lev.z.data_ptr()),
                                            ctypes.c_void_p(lev.dFF.data_ptr()) if lev.ff else None,
                                            st), "efe_chebyshev_step")  # fmt: skip

    def product(self, x, y, pairs):
        """y = A x on level 0 (the masked tangent); pairs: [n][2] float32 scratch for the
        float-float form of x when the tangent is FP32."""
        lev0 = self.levels[0]
        if lev0.ff:
            self._split(x, pairs)
            self._gemv_pairs(lev0.A, pairs, 1.0, 0.0, y)
        else:
            self._gemv(lev0.A, x, 1.0, 0.0, y)

    # ---------------------------------------------------------------- new tangent
    def update(self, K, diagPos):
        """Level operators for the tangent values K (float or double, the pattern's order);
        diagPos: positions of the diagonal entries of the level-0 rows."""
        lev0 = self.levels[0]
        lev0.values = K
        lev0.kp = L.EFE_K_FP64 if K.dtype == torch.float64 else L.EFE_K_FP32
        m0 = lev0.mask.to(torch.float64)
        lev0.dinv = torch.where(lev0.mask > 0, 1.0 / K[diagPos].to(torch.float64), torch.ones_like(m0))
        lev0.A = self._csr(lev0.n, lev0.n, lev0.indptr, lev0.indices, K, lev0.kp, lev0.mask, self.rowGroup)
        lev0.ff = K.dtype == torch.float32
        vals = K if K.dtype == torch.float64 else K.to(torch.float64)
        for k in range(len(self.levels) - 1):
            lev, nxt = self.levels[k], self.levels[k + 1]
            Sp, Si, Sv = lev.S
            S = self._csr(Sp.numel() - 1, vals.numel(), Sp, Si, Sv, L.EFE_K_FP64)
            self._gemv(S, vals, 1.0, 0.0, nxt.values)
            if bool(nxt.empty.any()):
                nxt.values[nxt.diag[nxt.empty]] = 1.0
            nxt.dinv = 1.0 / nxt.values[nxt.diag]
            nxt.A = self._csr(nxt.n, nxt.n, nxt.indptr, nxt.indices, nxt.values, L.EFE_K_FP64)
            Pp, Pi, Pv = lev.P
            lev.Pop = self._csr(lev.n, nxt.n, Pp, Pi, Pv, L.EFE_K_FP64)
            Rp, Ri, Rv = lev.R
            lev.Rop = self._csr(nxt.n, lev.n, Rp, Ri, Rv, L.EFE_K_FP64)
            vals = nxt.values
        del vals
        last = self.levels[-1]
        if last.n <= 8192:
            A = torch.zeros((last.n, last.n), dtype=torch.float64, device=self.dev)
            ip = last.indptr.to(torch.int64)
            rows = torch.repeat_interleave(torch.arange(last.n, device=self.dev), ip[1:] - ip[:-1])
            if len(self.levels) == 1:  # a single level: the masked tangent itself
                v = last.values.to(torch.float64)
                keep = (last.mask[rows] > 0) & (last.mask[last.indices.to(torch.int64)] > 0)
                A[rows[keep], last.indices.to(torch.int64)[keep]] = v[keep]
                A[torch.arange(last.n, device=self.dev)[last.mask == 0]] = 0.0
                A += torch.diag((last.mask == 0).to(torch.float64))
            else:
                A[rows, last.indices.to(torch.int64)] = last.values
            A = 0.5 * (A + A.T)
            self.dense = torch.cholesky_inverse(torch.linalg.cholesky(A))
        else:
            self.dense = None
        # smoother intervals
        g = torch.Generator().manual_seed(self.seed)
        for k, lev in enumerate(self.levels):
            if k == len(self.levels) - 1 and self.dense is not None:
                continue
            v = torch.rand(lev.n, generator=g, dtype=torch.float64).to(self.dev) - 0.5
            if lev.mask is not None and k == 0:
                v *= lev.mask.to(torch.float64)
            v /= torch.linalg.vector_norm(v)
            lam = torch.zeros((), dtype=torch.float64, device=self.dev)
            w = torch.empty_like(v)
            for _ in range(self.powerIterations):
                self._gemv(lev.A, v, 1.0, 0.0, w)
                w *= lev.dinv
                lam = torch.linalg.vector_norm(w)
                v = w / lam
            lev.cheb = chebyshev_coefficients(float(lam), self.degree)

    # ---------------------------------------------------------------- cycle
    def _smooth(self, lev, first):
        """Chebyshev steps on lev.res (the residual of lev.z); first: z starts from zero, and
        lev.res leaves as the residual after smoothing."""
        for k, (c1, c2) in enumerate(lev.cheb):
            if k > 0:
                self._residual_step(lev, lev.d, lev.dFF if lev.ff else None)
            self._cheb(lev, c1, c2, accumulate=(k > 0 or not first))
        if first:
            self._residual_step(lev, lev.d, lev.dFF if lev.ff else None)

    def _residual_step(self, lev, x, pairs):
        """lev.res -= A x (x also given as pairs on a float-float level)."""
        if lev.ff:
            self._gemv_pairs(lev.A, pairs, -1.0, 1.0, lev.res)
        else:
            self._gemv(lev.A, x, -1.0, 1.0, lev.res)

    def _cycle(self, k):
        lev = self.levels[k]
        if k == len(self.levels) - 1:
            if self.dense is not None:
                torch.mv(self.dense, lev.r, out=lev.z)
            else:
                lev.res.copy_(lev.r)
                self._smooth(lev, first=True)
            return
        nxt = self.levels[k + 1]
        lev.res.copy_(lev.r)
        self._smooth(lev, first=True)
        self._gemv(lev.Rop, lev.res, 1.0, 0.0, nxt.r)
        self._cycle(k + 1)
        self._gemv(lev.Pop, nxt.z, 1.0, 1.0, lev.z)
        lev.res.copy_(lev.r)
        if lev.ff:
            self._split(lev.z, lev.zFF)
        self._residual_step(lev, lev.z, lev.zFF if lev.ff else None)
        self._smooth(lev, first=False)

    def apply(self, r, z):
        """z = M^-1 r (r zero on the prescribed DOFs; z comes out zero there)."""
        lev0 = self.levels[0]
        lev0.r.copy_(r)
        self._cycle(0)
        z.copy_(lev0.z)

    def describe(self):
        """Sizes per level: [(DOFs, stored entries)]."""
        return [(lev.n, int(lev.indices.numel())) for lev in self.levels]
