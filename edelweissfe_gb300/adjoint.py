"""Adjoint gradients of an objective J(U) at equilibrium of a total-Lagrangian Neo-Hooke model.

The reference has no derivative capability; this is new.  At equilibrium the free-DOF residual
R_f(U, p) = P_f(U, p) + PExt_f vanishes, and dR_f/dU_f = -K_ff, so for any parameter p
(nodal reference coordinates X, per-element mu and K, or E with nu fixed):

    dJ/dp = lambda^T dP/dp,   K_ff lambda_f = dJ/dU_f,   lambda = 0 on prescribed DOFs.

The adjoint system is solved with the same device CG as the Newton steps (K is symmetric for
hyperelastic materials); lambda^T dP/dp is the hand-written reverse-mode kernel `efe_adjoint_tl`.
The hyperelastic state does not depend on the load path, so no history is needed.

`TLEquilibrium` puts the solve and its adjoint behind torch.autograd: U = TLEquilibrium.apply(
params, coords, problem) is differentiable in params ([E, 2] = (mu, K) per element) and coords
([nNodes, dim]), so any torch objective of U back-propagates through the Newton solution.
"""

import torch


def young_to_lame_chain(gP, nu):
    """dJ/dE per element from dJ/d(mu, K) for mu = E / (2(1+nu)), K = E / (3(1-2nu))."""
    return gP[:, 0] / (2.0 * (1.0 + nu)) + gP[:, 1] / (3.0 * (1.0 - 2.0 * nu))


def young_to_lame(E, nu):
    """(mu, K) per element from Young's modulus E (a torch tensor; differentiable)."""
    return torch.stack([E / (2.0 * (1.0 + nu)), E / (3.0 * (1.0 - 2.0 * nu))], 1)


class TLAdjoint:
    """solver: NISTGPU around an FP64 GPUAssembler whose groups are total-Lagrangian Neo-Hooke."""

    def __init__(self, solver):
        self.solver = solver
        self.asm = solver.asm
        self.lastLinearIterations = None

    def solve_adjoint(self, U, dJdU, dirichletDofs, K=None):
        """lambda with K_ff lambda_f = dJ/dU_f and lambda = 0 on the prescribed DOFs."""
        asm = self.asm
        g = dJdU.to(asm.device, torch.float64).clone()
        dir_idx = None
        if dirichletDofs is not None and len(dirichletDofs):
            dir_idx = torch.as_tensor(dirichletDofs, dtype=torch.int64, device=asm.device)
            g[dir_idx] = 0.0
        if K is None:
            # the forward solve's last element pass assembled K at exactly this U (hyperelastic: the
            # tangent depends on U only); otherwise assemble it
            if getattr(self.solver, "lastU", None) is U and self.solver.lastK is not None:
                K = self.solver.lastK
            else:
                K = self.solver.tangentAt(U.to(asm.device, torch.float64))
        n0 = len(self.solver.linearIterations)
        lam = self.solver._solve_pcg(K, g, dir_idx)
        self.lastLinearIterations = self.solver.linearIterations[n0:]
        if dir_idx is not None:
            lam[dir_idx] = 0.0
        return lam

    def gradient(self, U, dJdU, dirichletDofs):
        """(dJ/dX [nNodes, dim], [dJ/d(mu, K) per group [E, 2]]) at the equilibrium U."""
        lam = self.solve_adjoint(U, dJdU, dirichletDofs)
        U = U.to(self.asm.device, torch.float64)
        return self.asm.adjointTL(U, lam)


class TLProblem:
    """A quasi-static total-Lagrangian Neo-Hooke problem on one GPUAssembler (one group) with fixed
    Dirichlet conditions: solve(params, coords) resets the model, sets the per-element (mu, K) and
    the nodal coordinates, and runs the Newton step (NISTGPU.solveStep) to the final load."""

    def __init__(self, asm, dirichlets, stepper_factory, **solver_options):
        import numpy as np

        from .solver import NISTGPU

        self.asm = asm
        self.dirichlets = list(dirichlets)
        self.stepper_factory = stepper_factory
        self.solver = NISTGPU(asm, **solver_options)
        self.dirichletDofs = np.unique(np.concatenate([d.dofs for d in self.dirichlets])) if self.dirichlets else None

    def solve(self, params, coords):
        self.asm.setProperties(0, params.detach())
        self.asm.setCoordinates(coords.detach())
        self.asm.resetState()
        self.solver.history = []
        return self.solver.solveStep(self.stepper_factory(), self.dirichlets)


class TLEquilibrium(torch.autograd.Function):
    """U(params, coords) at equilibrium; backward: one adjoint solve + efe_adjoint_tl."""

    @staticmethod
    def forward(ctx, params, coords, problem):
        U = problem.solve(params, coords)
        ctx.problem = problem
        ctx.save_for_backward(U)
        return U.clone()

    @staticmethod
    def backward(ctx, gU):
        (U,) = ctx.saved_tensors
        problem = ctx.problem
        gX, gP = TLAdjoint(problem.solver).gradient(U, gU, problem.dirichletDofs)
        return gP[0], gX, None


class PathAdjoint:
    """Gradients of a function of the final increment of a plastic (path-dependent) small-strain
    solution with respect to the material properties of every element.

    The reference has no derivatives; this is new.  Attach it to a NISTGPU before solveStep: every
    accepted increment n checkpoints the quadrature-point history before it (s_{n-1}), its total
    displacement u_n and its increment du_n (host-side checkpoint list, device tensors).  The
    discrete adjoint then runs backward over the increments, recomputing each increment from its
    checkpoint:

      K_n          the consistent tangent of increment n (element pass from s_{n-1} with du_n),
      a            = (ds_n/du_n)^T sbar_n + (dP_n/du_n)^T cP_n        (efe_adjoint_small_strain)
      K_n lam_n    = a + ubar_n  on the free DOFs, lam_n = 0 on the prescribed ones
      b            = (dP_n/du_n)^T lam_n;   ubar_{n-1} = -(a + b);   sbar_{n-1}, dJ/dprops from both
                     passes,

    for J = cP . P_N + cU . u_N (cP: weights of the final residual, e.g. -1 on the DOFs whose
    reaction is wanted; cU: weights of the final displacement).  With an FP32 tangent the adjoint
    systems are refined against the exact FP64 operator (K v = -(dP/du)^T v from the reverse
    kernel), so the gradient is that of the FP64 path.

    Checkpoints hold one state array per group and increment (13 doubles per point for von Mises),
    i.e. history memory grows with the number of increments; nothing else is stored."""

    def __init__(self, solver, refine_steps=2, refine_tolerance=1e-4):
        self.solver = solver
        self.asm = solver.asm
        self.refine_steps = refine_steps
        # each refinement only has to shrink the error left by the FP32 tangent (~1e-7 relative)
        self.refine_tolerance = refine_tolerance
        self.checkpoints = []
        solver.onAccept = self._record

    def _record(self, ts, U_old, U_new, dU):
        states = [g._dev["stateRef"].clone() for g in self.asm.groups]
        self.checkpoints.append(dict(ts=ts, U=U_new.clone(), dU=dU.clone(), states=states))

    def _exact_Kv(self, ck, v):
        """K v with the FP64 consistent tangent of checkpointed increment ck, matrix-free."""
        asm = self.asm
        out = asm.constructDofVector()
        for gi in range(len(asm.groups)):
            asm.adjointSmallStrain(gi, ck["states"][gi], ck["dU"], out, Pbar=v)
        return -out

    def gradient(self, dirichletDofs, cP=None, cU=None, timing=None, coordinates=False):
        """dJ/dprops per group ([E, nProps] tensors) for J = cP . P_N + cU . u_N; with
        coordinates=True, (that list, dJ/dX) with dJ/dX [nNodes, dim] in the node order of the
        assembler's coordinates (the prescribed displacements and the nodal loads held fixed).
        With a dict as `timing`, the device time of the element work (tangent recomputation and the
        two reverse passes per increment) and of the adjoint solves is added to timing["kernel_ms"]
        and timing["solve_ms"] (CUDA events on the current stream)."""

        def event():
            if timing is None:
                return None
            ev = torch.cuda.Event(enable_timing=True)
            ev.record()
            return ev

        marks = []
        asm = self.asm
        solver = self.solver
        dev = asm.device
        dir_idx = None
        if dirichletDofs is not None and len(dirichletDofs):
            dir_idx = torch.as_tensor(dirichletDofs, dtype=torch.int64, device=dev)
        saved = [g._dev["stateRef"].clone() for g in asm.groups]
        sbar = [torch.zeros_like(g._dev["stateRef"]) for g in asm.groups]
        gP = [torch.zeros((len(g.conn), g._dev["props"].shape[1]), dtype=torch.float64, device=dev)
              for g in asm.groups]  # fmt: skip
        carry = asm.constructDofVector()
        gX = torch.zeros((asm.nNodes, asm.dim), dtype=torch.float64, device=dev) if coordinates else None
        self.linearIterations = []
        N = len(self.checkpoints)
        for n in reversed(range(N)):
            ck = self.checkpoints[n]
            last = n == N - 1
            # recompute increment n from its checkpoint: the tangent K_n
            for gi, g in enumerate(asm.groups):
                g._dev["stateRef"].copy_(ck["states"][gi])
            e0 = event()
            K = solver.tangentAt_increment(ck["U"], ck["dU"])
            a = asm.constructDofVector()
            sprev = [torch.zeros_like(s) for s in sbar]
            for gi in range(len(asm.groups)):
                asm.adjointSmallStrain(gi, ck["states"][gi], ck["dU"], a, Pbar=cP if last else None,
                                       stateBarIn=sbar[gi], stateBarOut=sprev[gi], gProps=gP[gi], gX=gX)  # fmt: skip
            e1 = event()
            rhs = a + carry
            if last and cU is not None:
                rhs = rhs + cU
            if dir_idx is not None:
                rhs[dir_idx] = 0.0
            n0 = len(solver.linearIterations)
            lam = solver.linearSolve(K, rhs, dir_idx)
            if K.dtype != torch.float64:
                tol = solver.pcgTolerance
                solver.pcgTolerance = max(tol, self.refine_tolerance)
                try:
                    for _ in range(self.refine_steps):
                        r = rhs - self._exact_Kv(ck, lam)
                        if dir_idx is not None:
                            r[dir_idx] = 0.0
                        lam = lam + solver.linearSolve(K, r, dir_idx)
                finally:
                    solver.pcgTolerance = tol
            if dir_idx is not None:
                lam[dir_idx] = 0.0
            self.linearIterations.append(solver.linearIterations[n0:])
            e2 = event()
            b = asm.constructDofVector()
            for gi in range(len(asm.groups)):
                asm.adjointSmallStrain(gi, ck["states"][gi], ck["dU"], b, Pbar=lam, stateBarOut=sprev[gi],
                                       gProps=gP[gi], gX=gX)  # fmt: skip
            e3 = event()
            marks.append((e0, e1, e2, e3))
            carry = -(a + b)
            sbar = sprev
        for gi, g in enumerate(asm.groups):
            g._dev["stateRef"].copy_(saved[gi])
        if timing is not None:
            torch.cuda.synchronize(dev)
            timing["kernel_ms"] = timing.get("kernel_ms", 0.0) + sum(
                a.elapsed_time(b) + c.elapsed_time(d) for a, b, c, d in marks)
            timing["solve_ms"] = timing.get("solve_ms", 0.0) + sum(b.elapsed_time(c) for a, b, c, d in marks)
        return (gP, gX) if coordinates else gP
