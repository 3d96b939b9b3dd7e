"""Adjoint gradients (efe_adjoint_tl) against central finite differences, in FP64.

1. Element level: L = lambda^T P(X, U, mu, K) on small jittered total-Lagrangian Neo-Hooke meshes
   (Hexa8 a/b/c, Hexa20, Quad8 plane strain); directional derivatives along random directions in
   the nodal coordinates and in (mu, K), central differences with h = 1e-6; relative error <= 1e-6.
2. Objective level (the shape of the adjoint configuration): a jittered 3x3x3 C3D8TL Neo-Hooke (a)
   cube with a lognormal Young's modulus field (median 1000, sigma 0.3, nu = 0.3), bottom fixed, top
   pressed by 0.01 in 5 increments; J = 1/2 sum over 10 sensor nodes of |u - u*|^2 with u* the
   solution for a perturbed modulus field.  dJ/dE and dJ/dX by the adjoint vs central differences
   of J through full Newton solves (h = 1e-6), on random directions; relative error <= 1e-6.
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

H = 1e-6
RTOL = 1e-6


def _mesh(shape, seed):
    from edelweissfe_gb300 import meshes

    if shape in ("C3D8TL", "C3D20TL"):
        coords, conn, nodeDof, nDof = meshes.box(2, 2, 1, nNodes=20 if "20" in shape else 8)
        coords = meshes.jitter(coords, 0.1, [0.5, 0.5, 1.0], seed, [0, 0, 0], [1, 1, 1])
    else:
        coords, conn, nodeDof, nDof = meshes.rect(3, 2, nNodes=8)
        coords = meshes.jitter(coords, 0.1, [1 / 3, 0.5], seed, [0, 0], [1, 1])
    return coords, conn, nodeDof, nDof


def _L(coords, conn, nodeDof, nDof, elType, kind, props, U, lam):
    from edelweissfe_gb300 import ElementGroup, GPUAssembler

    asm = GPUAssembler(coords, nodeDof, nDof, [ElementGroup(elType, kind, props, conn, 0.9)])
    P, F, K = asm.constructDofVector(), asm.constructDofVector(), asm.constructSystemMatrix()
    asm.computeElements(None, U, U, P, K, F)
    return float(torch.dot(P, lam)), asm


@pytest.mark.parametrize(
    "elType,kind",
    [("C3D8TL", "neohookewa"), ("C3D8TL", "neohookewb"), ("C3D8TL", "neohookewc"), ("C3D20TL", "neohookewa"),
     ("CPE8RTL", "neohookewa")],
)  # fmt: skip
def test_element_adjoint_matches_finite_differences(elType, kind):
    coords, conn, nodeDof, nDof = _mesh(elType, 3)
    rng = np.random.default_rng(4)
    E = len(conn)
    props = np.stack([rng.uniform(500, 1500, E), rng.uniform(5000, 15000, E)], 1)
    U = torch.tensor(rng.normal(0, 0.02, nDof), device="cuda")
    lam = torch.tensor(rng.normal(0, 1, nDof), device="cuda")
    L0, asm = _L(coords, conn, nodeDof, nDof, elType, kind, props, U, lam)
    gX, gP = asm.adjointTL(U, lam)
    gX = gX.cpu().numpy()
    gP = gP[0].cpu().numpy()
    for k in range(3):
        d = rng.normal(0, 1, coords.shape)
        fd = (_L(coords + H * d, conn, nodeDof, nDof, elType, kind, props, U, lam)[0]
              - _L(coords - H * d, conn, nodeDof, nDof, elType, kind, props, U, lam)[0]) / (2 * H)  # fmt: skip
        ad = float(np.sum(gX * d))
        assert abs(ad - fd) <= RTOL * max(abs(fd), 1e-3 * abs(L0)), (k, ad, fd)
        dp = rng.normal(0, 1, props.shape) * props
        fd = (_L(coords, conn, nodeDof, nDof, elType, kind, props + H * dp, U, lam)[0]
              - _L(coords, conn, nodeDof, nDof, elType, kind, props - H * dp, U, lam)[0]) / (2 * H)  # fmt: skip
        ad = float(np.sum(gP * dp))
        assert abs(ad - fd) <= RTOL * max(abs(fd), 1e-3 * abs(L0)), (k, ad, fd)


def _boundary_dofs(coords, nodeDof):
    y = coords[:, 1]
    bottom = np.nonzero(y < 1e-9)[0]
    top = np.nonzero(y > 1 - 1e-9)[0]
    return (nodeDof[bottom][:, None] + np.arange(3)).ravel(), nodeDof[top] + 1


def _cube_problem(Efield, coords, conn, nodeDof, nDof, bc, nu=0.3):
    from edelweissfe_gb300 import ElementGroup, GPUAssembler
    from edelweissfe_gb300.solver import AdaptiveTimeStepper, Dirichlet, NISTGPU

    props = np.stack([Efield / (2 * (1 + nu)), Efield / (3 * (1 - 2 * nu))], 1)
    asm = GPUAssembler(coords, nodeDof, nDof, [ElementGroup("C3D8TL", "neohookewa", props, conn)])
    bdofs, tdofs = bc  # fixed node sets: perturbed coordinates must not change the boundary conditions
    dirichlets = [Dirichlet(bdofs, 0.0), Dirichlet(tdofs, -0.01)]
    solver = NISTGPU(asm, linsolver="pcg", extrapolation="off", maxIter=25, fluxResidualTolerance=1e-12,
                     fieldCorrectionTolerance=1e-13, fluxResidualFloor=0.0, pcgTolerance=1e-14)  # fmt: skip
    U = solver.solveStep(AdaptiveTimeStepper(maxIncrement=0.2), dirichlets)
    return U, solver, np.concatenate([bdofs, tdofs])


def test_objective_gradient_matches_finite_differences():
    from edelweissfe_gb300 import meshes
    from edelweissfe_gb300.adjoint import TLAdjoint, young_to_lame_chain

    coords, conn, nodeDof, nDof = meshes.box(3, 3, 3, nNodes=8)
    coords = meshes.jitter(coords, 0.1, [1 / 3] * 3, 11, [0, 0, 0], [1, 1, 1])
    rng = np.random.default_rng(12)
    Efield = 1000.0 * np.exp(0.3 * rng.normal(size=len(conn)))
    sensors = rng.choice(np.nonzero((coords[:, 1] > 1e-9) & (coords[:, 1] < 1 - 1e-9))[0], 10, replace=False)
    sdofs = (nodeDof[sensors][:, None] + np.arange(3)).ravel()
    bc = _boundary_dofs(coords, nodeDof)
    target, _, _ = _cube_problem(Efield * (1 + 0.1 * rng.normal(size=len(conn))), coords, conn, nodeDof, nDof, bc)
    target = target.cpu().numpy()[sdofs]

    def J(Ef, X):
        U, solver, ddofs = _cube_problem(Ef, X, conn, nodeDof, nDof, bc)
        u = U.cpu().numpy()[sdofs]
        return 0.5 * float(np.sum((u - target) ** 2)), U, solver, ddofs

    J0, U, solver, ddofs = J(Efield, coords)
    dJdU = torch.zeros(nDof, dtype=torch.float64, device=U.device)
    dJdU[torch.as_tensor(sdofs, device=U.device)] = U[torch.as_tensor(sdofs, device=U.device)] - torch.as_tensor(
        target, device=U.device
    )
    gX, gP = TLAdjoint(solver).gradient(U, dJdU, ddofs)
    gE = young_to_lame_chain(gP[0], 0.3).cpu().numpy()
    gX = gX.cpu().numpy()
    for k in range(2):
        dE = rng.normal(0, 1, len(conn)) * Efield
        fd = (J(Efield + H * dE, coords)[0] - J(Efield - H * dE, coords)[0]) / (2 * H)
        assert abs(float(np.sum(gE * dE)) - fd) <= RTOL * abs(fd), ("E", k, float(np.sum(gE * dE)), fd)
        dX = rng.normal(0, 1, coords.shape)
        fd = (J(Efield, coords + H * dX)[0] - J(Efield, coords - H * dX)[0]) / (2 * H)
        assert abs(float(np.sum(gX * dX)) - fd) <= RTOL * abs(fd), ("X", k, float(np.sum(gX * dX)), fd)


def test_autograd_function_matches_finite_differences():
    """TLEquilibrium behind torch.autograd: J(U(E, X)) backpropagates to E and X; checked against
    central differences of the same objective along one random direction each (h = 1e-5: a step
    of 1e-6 moves J by ~1e-9 of itself here, the order of the Newton solution's own accuracy)."""
    h = 1e-5
    from edelweissfe_gb300 import ElementGroup, GPUAssembler, meshes
    from edelweissfe_gb300.adjoint import TLEquilibrium, TLProblem, young_to_lame
    from edelweissfe_gb300.solver import AdaptiveTimeStepper, Dirichlet

    coords, conn, nodeDof, nDof = meshes.box(3, 2, 2, nNodes=8)
    coords = meshes.jitter(coords, 0.1, [1 / 3, 0.5, 0.5], 21, [0, 0, 0], [1, 1, 1])
    rng = np.random.default_rng(22)
    E0 = 1000.0 * np.exp(0.3 * rng.normal(size=len(conn)))
    asm = GPUAssembler(coords, nodeDof, nDof, [ElementGroup("C3D8TL", "neohookewa", young_to_lame(
        torch.tensor(E0), 0.3).numpy(), conn)])  # fmt: skip
    bdofs, tdofs = _boundary_dofs(coords, nodeDof)
    problem = TLProblem(asm, [Dirichlet(bdofs, 0.0), Dirichlet(tdofs, -0.01)],
                        lambda: AdaptiveTimeStepper(maxIncrement=0.25), linsolver="pcg", extrapolation="off",
                        maxIter=25, fluxResidualTolerance=1e-12, fieldCorrectionTolerance=1e-13,
                        fluxResidualFloor=0.0, pcgTolerance=1e-14)  # fmt: skip
    sdofs = torch.as_tensor(rng.choice(np.setdiff1d(np.arange(nDof), np.concatenate([bdofs, tdofs])), 12,
                                       replace=False), device=asm.device)  # fmt: skip
    target = torch.as_tensor(rng.normal(0, 1e-3, 12), device=asm.device)

    def J(E, X):
        U = TLEquilibrium.apply(young_to_lame(E, 0.3), X, problem)
        return 0.5 * ((U[sdofs] - target) ** 2).sum()

    E = torch.tensor(E0, device=asm.device, requires_grad=True)
    X = torch.tensor(coords, device=asm.device, requires_grad=True)
    J(E, X).backward()
    with torch.no_grad():
        dE = torch.as_tensor(rng.normal(0, 1, len(conn)) * E0, device=asm.device)
        fd = (float(J(E + h * dE, X)) - float(J(E - h * dE, X))) / (2 * h)
        ad = float((E.grad * dE).sum())
        assert abs(ad - fd) <= RTOL * abs(fd), ("E", ad, fd)
        dX = torch.as_tensor(rng.normal(0, 1, coords.shape), device=asm.device)
        fd = (float(J(E, X + h * dX)) - float(J(E, X - h * dX))) / (2 * h)
        ad = float((X.grad * dX).sum())
        assert abs(ad - fd) <= RTOL * abs(fd), ("X", ad, fd)
