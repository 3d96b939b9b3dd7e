"""Adjoint gradients against gradients of the reference CPU path.

The reference has no derivatives, so its gradient is taken by central differences (h = 1e-6) of
J(U(E)) where U(E) comes from a small FP64 Newton loop on the host around the oracle's restatement
of the reference's computeElements + updateCSR (the oracle is pinned to the reference by the golden
fixtures).  Problem: a jittered 2x2x1 C3D8TL Neo-Hooke (a) block, per-element E, nu = 0.3; bottom
fixed, top pressed by 0.02; J = 1/2 |U_s - U*|^2 over 6 DOFs.  The GPU gradient comes from
TLEquilibrium (device Newton + adjoint kernel).  Agreement: U to 1e-10, dJ/dE to 1e-6 relative on
three random directions."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _problem():
    from edelweissfe_gb300 import meshes

    coords, conn, nodeDof, nDof = meshes.box(2, 2, 1, nNodes=8)
    coords = meshes.jitter(coords, 0.1, [0.5, 0.5, 1.0], 5, [0, 0, 0], [1, 1, 1])
    y = coords[:, 1]
    fixed = np.concatenate([(nodeDof[y < 1e-9][:, None] + np.arange(3)).ravel(), nodeDof[y > 1 - 1e-9] + 1])
    values = np.zeros(nDof)
    values[nodeDof[y > 1 - 1e-9] + 1] = -0.02
    rng = np.random.default_rng(6)
    E0 = 1000.0 * np.exp(0.3 * rng.normal(size=len(conn)))
    free = np.setdiff1d(np.arange(nDof), fixed)
    sdofs = rng.choice(free, 6, replace=False)
    target = rng.normal(0, 2e-3, 6)
    return coords, conn, nodeDof, nDof, fixed, values, E0, sdofs, target


def _lame(E, nu=0.3):
    return np.stack([E / (2 * (1 + nu)), E / (3 * (1 - 2 * nu))], 1)


def _oracle_solve(coords, conn, nodeDof, nDof, fixed, values, E):
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla

    from oracle.assembly import Model

    g = dict(elType="C3D8TL", kind="neohookewa", props=_lame(E), conn=conn.astype(np.int64),
             thickness=np.ones(len(conn)), order=np.arange(len(conn)))  # fmt: skip
    m = Model(coords, nodeDof, nDof, [g])
    free = np.setdiff1d(np.arange(nDof), fixed)
    U = values.copy()
    st = m.initial_state()
    for _ in range(30):
        r = m.compute_elements(U, U, st)
        R = r["P"]
        K = sp.csr_matrix((r["Kdata"], m.indices, m.indptr), shape=(nDof, nDof))
        if np.abs(R[free]).max() <= 1e-13 * np.abs(r["F"]).max():
            return U
        U[free] += sla.spsolve(K[free][:, free].tocsc(), R[free])  # K dU = R (R = P, K = -dP/dU)
    raise AssertionError("oracle Newton did not converge")


def test_adjoint_matches_finite_differences_of_the_reference_path():
    from edelweissfe_gb300 import ElementGroup, GPUAssembler
    from edelweissfe_gb300.adjoint import TLEquilibrium, TLProblem, young_to_lame
    from edelweissfe_gb300.solver import AdaptiveTimeStepper, Dirichlet

    coords, conn, nodeDof, nDof, fixed, values, E0, sdofs, target = _problem()

    def J_ref(E):
        U = _oracle_solve(coords, conn, nodeDof, nDof, fixed, values, E)
        return 0.5 * float(np.sum((U[sdofs] - target) ** 2)), U

    asm = GPUAssembler(coords, nodeDof, nDof, [ElementGroup("C3D8TL", "neohookewa", _lame(E0), conn)])
    top = fixed[values[fixed] != 0.0]
    problem = TLProblem(asm, [Dirichlet(np.setdiff1d(fixed, top), 0.0), Dirichlet(top, -0.02)],
                        lambda: AdaptiveTimeStepper(maxIncrement=1.0), linsolver="superlu", extrapolation="off",
                        maxIter=30, fluxResidualTolerance=1e-13, fieldCorrectionTolerance=1e-14,
                        fluxResidualFloor=0.0)  # fmt: skip
    E = torch.tensor(E0, device=asm.device, requires_grad=True)
    U = TLEquilibrium.apply(young_to_lame(E, 0.3), torch.tensor(coords, device=asm.device), problem)
    s = torch.as_tensor(sdofs, device=asm.device)
    Jg = 0.5 * ((U[s] - torch.as_tensor(target, device=asm.device)) ** 2).sum()
    Jg.backward()
    J0, Uref = J_ref(E0)
    assert np.abs(U.detach().cpu().numpy() - Uref).max() <= 1e-10 * np.abs(Uref).max()
    assert abs(float(Jg) - J0) <= 1e-10 * abs(J0)
    g = E.grad.cpu().numpy()
    rng = np.random.default_rng(7)
    h = 1e-6
    for _ in range(3):
        dE = rng.normal(0, 1, len(E0)) * E0
        fd = (J_ref(E0 + h * dE)[0] - J_ref(E0 - h * dE)[0]) / (2 * h)
        ad = float(np.sum(g * dE))
        assert abs(ad - fd) <= 1e-6 * abs(fd), (ad, fd)
