"""Adjoint gradients of an objective J(U) at equilibrium of a total-Lagrangian Neo-Hooke model.

The reference has no derivative capability; this is new.  At equilibrium the free-DOF residual
R_f(U, p) = P_f(U, p) + PExt_f vanishes, and dR_f/dU_f = -K_ff, so for any parameter p
(nodal reference coordinates X, per-element mu and K, or E with nu fixed):

    dJ/dp = lambda^T dP/dp,   K_ff lambda_f = dJ/dU_f,   lambda = 0 on prescribed DOFs.

The adjoint system is solved with the same device CG as the Newton steps (K is symmetric for
hyperelastic materials); lambda^T dP/dp is the hand-written reverse-mode kernel `efe_adjoint_tl`.
The hyperelastic state does not depend on the load path, so no history is needed.
"""

import torch


def young_to_lame_chain(gP, nu):
    """dJ/dE per element from dJ/d(mu, K) for mu = E / (2(1+nu)), K = E / (3(1-2nu))."""
    return gP[:, 0] / (2.0 * (1.0 + nu)) + gP[:, 1] / (3.0 * (1.0 - 2.0 * nu))


class TLAdjoint:
    """solver: NISTGPU around an FP64 GPUAssembler whose groups are total-Lagrangian Neo-Hooke."""

    def __init__(self, solver):
        self.solver = solver
        self.asm = solver.asm
        self.lastLinearIterations = None

    def gradient(self, U, dJdU, dirichletDofs):
        """(dJ/dX [nNodes, dim], [dJ/d(mu, K) per group [E, 2]]) at the equilibrium U."""
        asm = self.asm
        U = U.to(asm.device, torch.float64)
        g = dJdU.to(asm.device, torch.float64).clone()
        dir_idx = None
        if dirichletDofs is not None and len(dirichletDofs):
            dir_idx = torch.as_tensor(dirichletDofs, dtype=torch.int64, device=asm.device)
            g[dir_idx] = 0.0
        K = self.solver.tangentAt(U)
        n0 = len(self.solver.linearIterations)
        lam = self.solver._solve_pcg(K, g, dir_idx)
        self.lastLinearIterations = self.solver.linearIterations[n0:]
        if dir_idx is not None:
            lam[dir_idx] = 0.0
        return asm.adjointTL(U, lam)
