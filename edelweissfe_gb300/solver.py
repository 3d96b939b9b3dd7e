"""Newton-Raphson driver around the GPU element pass (the reference's NIST, restated for the device).

`NISTGPU.solveStep` / `solveIncrement` follow `NIST.solveStep` / `NIST.solveIncrement`
(`edelweissfe/solvers/nonlinearimplicitstatic.py:134-332, 334-458`): the same increment loop and
cutback handling, Dirichlet treatment (prescribed increment in the first iteration, zeroed
residual rows afterwards, identity rows in K, `:559-623`), Abaqus-like convergence test
(`:625-725`: flux residual <= max(tol * spatially averaged flux, 1e-7) and correction < tol),
growing-residual and maximum-iteration checks, and linear extrapolation of the last increment
(`:947-986`).  `AdaptiveTimeStepper` restates `edelweissfe/timesteppers/adaptivetimestepper.py:38-183`.

The element pass, the residual, the tangent and the loads stay on the GPU.  The linear solve is
either SciPy's SuperLU on the host on the reference's row-modified CSR matrix (``"superlu"``, the
reference's fallback solver, for parity runs) or a Jacobi-preconditioned conjugate-gradient solve on
the device (``"pcg"``) on the equivalent symmetric system with the Dirichlet columns eliminated.
"""

from collections import namedtuple

import numpy as np
import torch

from .exceptions import CutbackRequest

TimeStep = namedtuple("TimeStep", "number stepProgressIncrement stepProgress timeIncrement stepTime totalTime")


class ReachedMaxIterations(Exception):
    pass


class DivergingSolution(Exception):
    pass


class ReachedMinIncrementSize(Exception):
    pass


class ReachedMaxIncrements(Exception):
    pass


class StepFailed(Exception):
    pass


class AdaptiveTimeStepper:
    """Increment generator of `timesteppers/adaptivetimestepper.py:38-183` (first increment is a zero
    increment; the increment grows by `increaseFactor` after three good increments)."""

    def __init__(self, currentTime=0.0, stepLength=1.0, startIncrement=1.0, maxIncrement=1.0, minIncrement=1e-4,
                 maxNumberIncrements=1000, increaseFactor=1.1):  # fmt: skip
        self.nPassedGoodIncrements = 0
        self.incrementCounter = 0
        self.maxIncrement = maxIncrement
        self.minIncrement = minIncrement
        self.maxNumberIncrements = maxNumberIncrements
        self.finishedStepProgress = 0.0
        self.increment = min(startIncrement, maxIncrement)
        self.allowedToIncreasedNext = True
        self.currentTime = currentTime
        self.stepLength = stepLength
        self.increaseFactor = increaseFactor

    def generateTimeStep(self):
        while self.finishedStepProgress < (1.0 - 1e-15):
            remainder = 1.0 - self.finishedStepProgress
            if remainder < self.increment:
                self.increment = remainder
            theIncrement = self.increment if self.incrementCounter > 0 else 0.0
            dT = self.stepLength * theIncrement
            self.finishedStepProgress += theIncrement
            endInStep = self.stepLength * self.finishedStepProgress
            yield TimeStep(self.incrementCounter, theIncrement, self.finishedStepProgress, dT, endInStep,
                           self.currentTime + endInStep)  # fmt: skip
            if self.incrementCounter > self.maxNumberIncrements:
                raise ReachedMaxIncrements()
            if self.nPassedGoodIncrements >= 3 and self.allowedToIncreasedNext:
                self.increment *= self.increaseFactor
                if self.increment > self.maxIncrement:
                    self.increment = self.maxIncrement
            self.allowedToIncreasedNext = True
            self.incrementCounter += 1
            self.nPassedGoodIncrements += 1

    def preventIncrementIncrease(self):
        self.allowedToIncreasedNext = False

    def reduceNextIncrement(self, scaleFactor):
        if self.increment == self.minIncrement:
            raise ReachedMinIncrementSize()
        new = self.increment * scaleFactor
        self.increment = min(self.maxIncrement, max(self.minIncrement, new))

    def discardAndChangeIncrement(self, scaleFactor):
        if self.incrementCounter == 0:
            raise ReachedMinIncrementSize()
        self.finishedStepProgress -= self.increment
        self.incrementCounter -= 1
        self.nPassedGoodIncrements = 0
        self.reduceNextIncrement(scaleFactor)


def _linear(x):
    return x


class Dirichlet:
    """Prescribed displacements: `values` are reached at the end of the step (stepactions/dirichlet.py:105-112)."""

    def __init__(self, dofs, values, amplitude=_linear):
        self.dofs = np.asarray(dofs, np.int64)
        self.values = np.broadcast_to(np.asarray(values, float), self.dofs.shape).copy()
        self.amplitude = amplitude

    def getDelta(self, ts):
        return self.values * (self.amplitude(ts.stepProgress) - self.amplitude(ts.stepProgress - ts.stepProgressIncrement))


class NodeForces:
    """Concentrated loads ramped over the step (stepactions/nodeforces.py:136-145)."""

    def __init__(self, dofs, values, amplitude=_linear):
        self.dofs = np.asarray(dofs, np.int64)
        self.values = np.broadcast_to(np.asarray(values, float), self.dofs.shape).copy()
        self.amplitude = amplitude

    def getCurrentLoad(self, ts):
        return self.values * self.amplitude(ts.stepProgress)


class BodyForce:
    """Body force per unit volume on a set of elements (global indices), ramped over the step
    (stepactions/bodyforce.py:95-101)."""

    def __init__(self, elements, force, amplitude=_linear):
        self.elements = None if elements is None else np.asarray(elements, np.int64)
        self.force = np.asarray(force, float)
        self.amplitude = amplitude

    def getCurrentLoad(self, ts):
        return self.force * self.amplitude(ts.stepProgress)


class NISTGPU:
    """Nonlinear implicit static solver with the element pass, loads and (optionally) the linear
    solve on the GPU.  `assembler` is a GPUAssembler."""

    def __init__(self, assembler, linsolver="pcg", extrapolation="linear", maxIter=10, criticalIter=5,
                 maxGrowingIter=10, fluxResidualTolerance=1e-8, fluxResidualToleranceAlternative=5e-3,
                 fieldCorrectionTolerance=1e-8, pcgTolerance=1e-12, pcgMaxIter=20000, fluxResidualFloor=1e-7,
                 pcgPreconditioner="jacobi", pcgGraphs=True, amgOptions=None):  # fmt: skip
        self.asm = assembler
        self.linsolver = linsolver
        self.extrapolation = extrapolation
        self.maxIter = maxIter
        self.criticalIter = criticalIter
        self.maxGrowingIter = maxGrowingIter
        self.fluxTol = fluxResidualTolerance
        self.fluxTolAlt = fluxResidualToleranceAlternative
        self.corrTol = fieldCorrectionTolerance
        self.pcgTolerance = pcgTolerance
        self.pcgMaxIter = pcgMaxIter
        self.fluxFloor = fluxResidualFloor
        # "jacobi": inverse of the diagonal; "block": inverses of the nodal diagonal blocks (the node's
        # displacement components) -- on near-regular hexahedral meshes of isotropic material the
        # same-node couplings nearly cancel and both need the same iterations
        self.pcgPreconditioner = pcgPreconditioner
        # replay the PCG iteration batches of long solves as one CUDA graph (same kernels and
        # arguments as the direct launches, so the same results bit for bit)
        self.pcgGraphs = pcgGraphs
        # "amg": aggregation multigrid V-cycles (amg.AggregationAMG, built once per set of
        # prescribed DOFs, its level operators once per tangent)
        self.amgOptions = dict(amgOptions or {})
        self._amg = None
        self.nAccumulatedFluxes = sum(len(g.conn) * len(g.conn[0]) * assembler.dim for g in assembler.groups if len(g.conn))
        dev = assembler.device
        ip, ix = assembler.indptr_host, assembler.indices_host
        rows = np.repeat(np.arange(assembler.nDof), np.diff(ip))
        self._diag_pos = torch.from_numpy(np.nonzero(ix == rows)[0]).to(dev)
        self.history = []  # one record per attempted increment
        self.linearIterations = []
        self.linearConverged = []  # per device CG solve: met pcgTolerance (False: stopped at pcgMaxIter)
        self.linearResiduals = []  # per device CG solve: final |r| / |b| when it stopped at pcgMaxIter
        self.lastK = self.lastU = self.lastP = None
        # called as onAccept(timeStep, U_old, U_new, dU) before each accepted increment's state is
        # committed (the state of the assembler is still the one before the increment)
        self.onAccept = None

    # ------------------------------------------------------------------ step
    def solveStep(self, stepper, dirichlets=(), nodeforces=(), bodyforces=(), cutbackFactor=0.25, U=None):
        asm = self.asm
        U = asm.constructDofVector() if U is None else U
        dU = asm.constructDofVector()
        prev = None
        try:
            for ts in stepper.generateTimeStep():
                try:
                    U_new, dU, P, iters, res = self.solveIncrement(U, dU, dirichlets, nodeforces, bodyforces, ts, prev)
                except CutbackRequest as e:
                    stepper.discardAndChangeIncrement(max(e.cutbackSize, cutbackFactor))
                    prev = None
                    self.history.append(dict(timeStep=ts, iterations=None, error="CutbackRequest"))
                except (ReachedMaxIterations, DivergingSolution) as e:
                    stepper.discardAndChangeIncrement(cutbackFactor)
                    prev = None
                    self.history.append(dict(timeStep=ts, iterations=None, error=type(e).__name__))
                else:
                    prev = ts
                    if iters >= self.criticalIter:
                        stepper.preventIncrementIncrease()
                    self.lastP = P
                    # the final tangent, assembled at exactly the accepted U (reused by adjoints)
                    self.lastK, self.lastU = self._incrementK, U_new
                    if self.onAccept is not None:
                        self.onAccept(ts, U, U_new, dU)
                    U = U_new
                    asm.acceptLastState()  # FEModel.advanceToTime (models/femodel.py:245-258)
                    self.history.append(dict(timeStep=ts, iterations=iters, error="", residuals=res))
        except (ReachedMaxIncrements, ReachedMinIncrementSize):
            raise StepFailed()
        return U

    # ------------------------------------------------------------------ increment
    def _dirichlet_rhs(self, vec, dirichlets, ts):
        for d in dirichlets:
            vec[torch.from_numpy(d.dofs).to(vec.device)] = torch.from_numpy(d.getDelta(ts)).to(vec)
        return vec

    def solveIncrement(self, U_n, dU, dirichlets, nodeforces, bodyforces, ts, prevTimeStep):
        asm = self.asm
        dev = asm.device
        dir_idx = (
            torch.from_numpy(np.unique(np.concatenate([d.dofs for d in dirichlets]))).to(dev) if dirichlets else None
        )
        # extrapolateLastIncrement (:947-986)
        if self.extrapolation == "linear" and prevTimeStep is not None and prevTimeStep.timeIncrement:
            dU = dU * (ts.stepProgressIncrement / prevTimeStep.stepProgressIncrement)
            dU = self._dirichlet_rhs(dU, dirichlets, ts)
            extrapolated = True
        else:
            dU = torch.zeros_like(dU)
            extrapolated = False
        it = 0
        ddU = None
        prevFlux, nGrew = 0.0, 0
        residuals = []
        time = (ts.stepTime, ts.totalTime)
        P, F, K = asm.constructDofVector(), asm.constructDofVector(), asm.constructSystemMatrix()
        while True:
            U_np = U_n + dU
            P.zero_()
            F.zero_()
            K.zero_()
            asm.status.zero_()
            asm.launch(U_np, dU, P, K, F, time, ts.timeIncrement)
            asm.check_status()
            PExt = asm.constructDofVector()
            for nf in nodeforces:
                PExt.index_add_(0, torch.from_numpy(nf.dofs).to(dev), torch.from_numpy(nf.getCurrentLoad(ts)).to(PExt))
            for bf in bodyforces:
                asm.computeBodyForce(PExt, bf.getCurrentLoad(ts), bf.elements)
            R = P + PExt
            if it == 0 and not extrapolated and dirichlets:
                R = self._dirichlet_rhs(R, dirichlets, ts)
            else:
                if dir_idx is not None:
                    R[dir_idx] = 0.0
                # checkConvergence (:625-725), one field
                flux = float(R.abs().max())
                avgFlux = max(1e-10, float(F.abs().sum()) / self.nAccumulatedFluxes)
                corr = float(ddU.abs().max()) if ddU is not None else 0.0
                tol = self.fluxTol if it < 15 else self.fluxTolAlt
                converged = corr < self.corrTol and flux <= max(tol * avgFlux, self.fluxFloor)
                if flux > prevFlux:
                    nGrew += 1
                prevFlux = flux
                residuals.append((flux, avgFlux, corr))
                if converged:
                    break
                if nGrew > self.maxGrowingIter:
                    raise DivergingSolution("Residual grew {:} times, cutting back".format(self.maxGrowingIter))
                if it == self.maxIter:
                    raise ReachedMaxIterations("Reached max. iterations in current increment, cutting back")
            ddU = self.linearSolve(K, R, dir_idx)
            if torch.isnan(ddU).any():
                raise DivergingSolution("Obtained NaN in linear solve")
            dU = dU + ddU
            it += 1
        self._incrementK = K  # the tangent of the last element pass, at the converged U_np
        return U_np, dU, P, it, residuals

    def tangentAt(self, U):
        """The tangent K (CSR data) at total displacement U with a zero increment (no state change)."""
        asm = self.asm
        P, F, K = asm.constructDofVector(), asm.constructDofVector(), asm.constructSystemMatrix()
        asm.status.zero_()
        asm.launch(U, torch.zeros_like(U), P, K, F)
        asm.check_status()
        return K

    def tangentAt_increment(self, U, dU):
        """The tangent K (CSR data) of the increment dU from the assembler's current stateRef
        (the state is not committed)."""
        asm = self.asm
        P, F, K = asm.constructDofVector(), asm.constructDofVector(), asm.constructSystemMatrix()
        asm.status.zero_()
        asm.launch(U, dU, P, K, F)
        asm.check_status()
        return K

    # ------------------------------------------------------------------ linear solve
    def linearSolve(self, K, R, dir_idx):
        if self.linsolver == "superlu":
            return self._solve_superlu(K, R, dir_idx)
        return self._solve_pcg(K, R, dir_idx)

    def _solve_superlu(self, K, R, dir_idx):
        """assembleStiffnessCSR + applyDirichletK (:559-593) + SciPy SuperLU, on the host."""
        import scipy.sparse.linalg as sla

        A = self.asm.assembleStiffnessCSR(K, host=True)
        if dir_idx is not None:
            rows = dir_idx.cpu().numpy()
            for r in rows:
                A.data[A.indptr[r] : A.indptr[r + 1]] = 0.0
            diag = A.diagonal()
            diag[rows] = 1.0
            A.setdiag(diag)
            A.eliminate_zeros()
        x = sla.spsolve(A, R.cpu().numpy(), use_umfpack=False)
        return torch.from_numpy(np.asarray(x, np.float64)).to(self.asm.device)

    def _solve_pcg(self, K, R, dir_idx):
        """Preconditioned CG on the device (efe_pcg_start / efe_pcg_iterate), nodal block-Jacobi or
        Jacobi (pcgPreconditioner).  The reference's
        system has identity rows for the Dirichlet DOFs; moving the known values to the right-hand
        side gives the same solution from the symmetric positive-definite system on the free DOFs:
        x = x_d + y with x_d = R on the prescribed DOFs and K_ff y_f = R_f - K_fd x_d.  K is used as
        assembled (FP32 or FP64 values).  Converged when |r| <= pcgTolerance |b| (checked every
        10 iterations, as b's norm includes the prescribed values).  The check of a batch is read
        while the next batch already runs (its r.r copied to pinned memory behind the batch), so the
        device never waits for the host; a converged solve therefore runs one batch past the batch
        that met the tolerance (the kernels stop moving x when p.Ap or r.z reach zero).  With pcgGraphs, a solve still
        running after its first 20 iterations captures one batch of 10 iterations (30 launches) as a
        CUDA graph and replays it: the kernels read the iteration number only for its parity, which
        is even at the start of every batch."""
        import ctypes

        from . import _lib as L

        if self.pcgPreconditioner == "amg":
            return self._solve_pcg_amg(K, R, dir_idx)
        asm = self.asm
        dev = asm.device
        n = asm.nDof
        lib = L.load()
        m = torch.ones(n, dtype=torch.uint8, device=dev)
        if dir_idx is not None:
            m[dir_idx] = 0
        mf = m.to(torch.float64)
        bs = asm.dim if self.pcgPreconditioner == "block" and n % asm.dim == 0 else 1
        if bs > 1:
            # a node's DOFs are consecutive and its own columns are contiguous in every one of its
            # rows, ending with column = row at the diagonal position: block (i, j) of node k is at
            # diag_pos[k*bs + i] - i + j
            ij = torch.arange(bs, device=dev)
            pos = self._diag_pos.view(-1, bs)[:, :, None] - ij[None, :, None] + ij[None, None, :]
            mb = mf.view(-1, bs)
            B = K[pos].to(torch.float64) * mb[:, :, None] * mb[:, None, :] + torch.diag_embed(1.0 - mb)
            dinv = torch.linalg.inv(B).contiguous()
        else:
            d = K[self._diag_pos].to(torch.float64)
            dinv = torch.where(m > 0, 1.0 / d, torch.ones_like(d))
        vec = torch.empty((5, n), dtype=torch.float64, device=dev)
        work = torch.zeros(L.EFE_PCG_WORK_DOUBLES, dtype=torch.float64, device=dev)
        kp = L.EFE_K_FP64 if K.dtype == torch.float64 else L.EFE_K_FP32
        split = torch.empty((n, 2), dtype=torch.float32, device=dev) if kp == L.EFE_K_FP32 else None
        s = L.EfePcg(n, asm.indptr.data_ptr(), asm.indices.data_ptr(), K.data_ptr(), kp, m.data_ptr(), dinv.data_ptr(),
                     *[vec[i].data_ptr() for i in range(5)], work.data_ptr(),
                     split.data_ptr() if split is not None else None, bs, asm.rowGroup)  # fmt: skip
        stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        xd = (1.0 - mf) * R
        Kxd = torch.empty_like(R)
        L.check(lib.efe_csr_spmv(ctypes.byref(s), ctypes.c_void_p(xd.data_ptr()), ctypes.c_void_p(Kxd.data_ptr()),
                                 stream), "efe_csr_spmv")  # fmt: skip
        b = mf * (R - Kxd)
        bnorm = float(torch.linalg.vector_norm(b + xd))
        L.check(lib.efe_pcg_start(ctypes.byref(s), ctypes.c_void_p(b.data_ptr()), stream), "efe_pcg_start")
        tol2 = (self.pcgTolerance * bnorm) ** 2
        k = 0
        graph = None
        if bnorm > 0.0 and float(work[2]) > tol2:
            seen = torch.empty((2, 2), dtype=torch.float64, pin_memory=True)  # r.r, p.Ap of two batches
            done = [torch.cuda.Event(), torch.cuda.Event()]
            batch = 0
            while k < self.pcgMaxIter:
                step = min(10, self.pcgMaxIter - k)
                if self.pcgGraphs and step == 10 and k >= 20:
                    if graph is None:
                        graph = self._capture_pcg_batch(lib, s, k, step)
                    graph.replay()
                else:
                    L.check(lib.efe_pcg_iterate(ctypes.byref(s), k, step, stream), "efe_pcg_iterate")
                k += step
                seen[batch % 2].copy_(work[2:4], non_blocking=True)
                done[batch % 2].record()
                batch += 1
                if batch < 2:
                    continue
                done[batch % 2].synchronize()  # the previous batch (the one just queued still runs)
                rr, pAp = seen[batch % 2].tolist()
                if not rr <= tol2 and rr == rr and pAp != 0.0:  # not converged, no NaN, no breakdown
                    continue
                break
        self._record_linear(k, bnorm, tol2, lambda: float(work[2]))
        return vec[0] + xd

    def _record_linear(self, k, bnorm, tol2, final_rr):
        """Iterations of one device CG solve, and whether it met its tolerance: a solve that ran into
        pcgMaxIter gives Newton an inexact correction (the Newton convergence test still decides),
        so it is recorded in linearConverged / linearResiduals (final |r| / |b|) instead of passing
        unseen.  final_rr reads the last r.r (one device read, only for solves that hit the limit)."""
        self.linearIterations.append(k)
        if k >= self.pcgMaxIter and bnorm > 0.0:
            rr = final_rr()
            self.linearConverged.append(bool(rr <= tol2))
            self.linearResiduals.append(float(np.sqrt(max(rr, 0.0)) / bnorm) if rr == rr else float("nan"))
        else:
            self.linearConverged.append(True)
            self.linearResiduals.append(None)

    def _solve_pcg_amg(self, K, R, dir_idx):
        """CG on the same system as _solve_pcg, preconditioned by one aggregation-multigrid V-cycle
        per iteration (amg.AggregationAMG).  Same convergence test, checked once per batch of 10
        iterations one batch behind; with pcgGraphs, from the third batch on a batch (its products,
        V-cycles and reductions: ~50 launches per iteration) is replayed as one CUDA graph."""
        from .amg import AggregationAMG

        asm = self.asm
        dev = asm.device
        n = asm.nDof
        m = torch.ones(n, dtype=torch.uint8, device=dev)
        if dir_idx is not None:
            m[dir_idx] = 0
        h = self._amg
        if h is None or not torch.equal(h.levels[0].mask, m):
            self._amg = h = None  # release the previous hierarchy before building the next
            h = AggregationAMG(asm.indptr, asm.indices, m, asm.dim, rowGroup=asm.rowGroup, **self.amgOptions)
            self._amg = h
        h.update(K, self._diag_pos)
        A = h.levels[0].A
        mf = m.to(torch.float64)
        xd = (1.0 - mf) * R
        Kxd = torch.empty_like(R)
        h._gemv(A, xd, 1.0, 0.0, Kxd)
        r = mf * (R - Kxd)
        bnorm = float(torch.linalg.vector_norm(r + xd))
        tol2 = (self.pcgTolerance * bnorm) ** 2
        x = torch.zeros_like(R)
        k = 0
        if bnorm > 0.0 and float(torch.dot(r, r)) > tol2:
            z = torch.empty_like(R)
            Ap = torch.empty_like(R)
            pairs = torch.empty((n, 2), dtype=torch.float32, device=dev)
            h.apply(r, z)
            p = z.clone()
            rz = torch.dot(r, z)  # the scalars live on the device and are updated in place
            pApLast = torch.zeros((), dtype=torch.float64, device=dev)
            rrLast = torch.zeros((), dtype=torch.float64, device=dev)
            zero = torch.zeros((), dtype=torch.float64, device=dev)

            def iterate(count):
                for _ in range(count):
                    h.product(p, Ap, pairs)
                    pAp = torch.dot(p, Ap)
                    alpha = torch.where(pAp != 0.0, rz / pAp, zero)
                    x.addcmul_(alpha, p)
                    r.addcmul_(alpha, Ap, value=-1.0)
                    h.apply(r, z)
                    rzNew = torch.dot(r, z)
                    beta = torch.where(rz != 0.0, rzNew / rz, zero)
                    p.mul_(beta).add_(z)
                    rz.copy_(rzNew)
                pApLast.copy_(pAp)
                rrLast.copy_(torch.dot(r, r))

            seen = torch.empty((2, 2), dtype=torch.float64, pin_memory=True)  # r.r, p.Ap of two batches
            done = [torch.cuda.Event(), torch.cuda.Event()]
            graph = None
            batch = 0
            while k < self.pcgMaxIter:
                step = min(10, self.pcgMaxIter - k)
                if self.pcgGraphs and step == 10 and k >= 20:
                    if graph is None:
                        graph = self._capture(lambda: iterate(10))
                    graph.replay()
                else:
                    iterate(step)
                k += step
                seen[batch % 2, 0].copy_(rrLast, non_blocking=True)
                seen[batch % 2, 1].copy_(pApLast, non_blocking=True)
                done[batch % 2].record()
                batch += 1
                if batch < 2:
                    continue
                done[batch % 2].synchronize()  # the previous batch (the one just queued still runs)
                rr, pApSeen = seen[batch % 2].tolist()
                if not rr <= tol2 and rr == rr and pApSeen != 0.0:  # not converged, no NaN, no breakdown
                    continue
                break
            self._record_linear(k, bnorm, tol2, lambda: float(rrLast))
        else:
            self._record_linear(k, bnorm, tol2, lambda: 0.0)
        return x + xd

    def _capture_pcg_batch(self, lib, s, k, step):
        """One batch of `step` PCG iterations starting at iteration k (even) as a CUDA graph."""
        import ctypes

        from . import _lib as L

        dev = self.asm.device
        return self._capture(lambda: L.check(lib.efe_pcg_iterate(ctypes.byref(s), k, step, ctypes.c_void_p(
            torch.cuda.current_stream(dev).cuda_stream)), "efe_pcg_iterate (graph capture)"))  # fmt: skip

    def _capture(self, fn):
        """The launches of fn() as a CUDA graph, captured on a side stream (fn launches on the
        current stream); replay() runs them on the current stream."""
        dev = self.asm.device
        graph = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):
            graph.capture_begin()
            try:
                fn()
            finally:
                graph.capture_end()
        torch.cuda.current_stream(dev).wait_stream(side)
        return graph
