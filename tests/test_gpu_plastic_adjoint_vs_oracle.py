"""Plastic path adjoint against gradients of the reference CPU path.

The reference has no derivatives: its gradient is taken by central differences (h = 1e-6) of the
total top reaction after a plastic load path, computed by a small FP64 incremental Newton loop on
the host around the oracle's restatement of the reference's computeElements + updateCSR (state
accepted per increment, as NIST does).  Problem: a 2x1x1 C3D8 von Mises block with per-element
yield stress and hardening, bottom u_y = 0, left u_x = 0, back u_z = 0, top u_y -> 0.5 % in four
increments.  The GPU side runs the same path with NISTGPU (FP64, SuperLU) and PathAdjoint.
Agreement: final U to 1e-10, dJ/d(fy0, H) to 1e-6 relative on three random directions."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

N_INC = 4


def _problem():
    from edelweissfe_gb300 import meshes

    coords, conn, nodeDof, nDof = meshes.box(2, 1, 1, nNodes=8)
    x, y, z = coords[:, 0], coords[:, 1], coords[:, 2]
    top = nodeDof[y > 1 - 1e-9] + 1
    bcs = [(nodeDof[y < 1e-9] + 1, 0.0), (nodeDof[x < 1e-9], 0.0), (nodeDof[z < 1e-9] + 2, 0.0), (top, 0.005)]
    rng = np.random.default_rng(3)
    fy0 = rng.uniform(200, 300, len(conn))
    H = rng.uniform(800, 1200, len(conn))
    return coords, conn, nodeDof, nDof, bcs, top, fy0, H


def _props(fy0, H):
    E = len(fy0)
    return np.stack([np.full(E, 210e3), np.full(E, 0.3), fy0, H, np.zeros(E), np.zeros(E)], 1)


def _oracle_path(coords, conn, nodeDof, nDof, bcs, top, fy0, H):
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla

    from oracle.assembly import Model

    g = dict(elType="C3D8", kind="vonmises", props=_props(fy0, H), conn=conn.astype(np.int64),
             thickness=np.ones(len(conn)), order=np.arange(len(conn)))  # fmt: skip
    m = Model(coords, nodeDof, nDof, [g])
    fixed = np.unique(np.concatenate([d for d, _ in bcs]))
    free = np.setdiff1d(np.arange(nDof), fixed)
    target = np.zeros(nDof)
    for d, v in bcs:
        target[d] = v
    st = m.initial_state()
    U = np.zeros(nDof)
    for n in range(1, N_INC + 1):
        dU = np.zeros(nDof)
        dU[fixed] = target[fixed] / N_INC
        for _ in range(30):
            r = m.compute_elements(U + dU, dU, st)
            R = r["P"]
            if np.abs(R[free]).max() <= 1e-12 * np.abs(r["F"]).max():
                break
            K = sp.csr_matrix((r["Kdata"], m.indices, m.indptr), shape=(nDof, nDof))
            dU[free] += sla.spsolve(K[free][:, free].tocsc(), R[free])
        else:
            raise AssertionError("oracle Newton did not converge")
        st = m.accept_state(r["stateTemp"])
        U = U + dU
    return -float(r["P"][top].sum()), U


def test_path_adjoint_matches_finite_differences_of_the_reference_path():
    from edelweissfe_gb300 import ElementGroup, GPUAssembler
    from edelweissfe_gb300.adjoint import PathAdjoint
    from edelweissfe_gb300.solver import AdaptiveTimeStepper, Dirichlet, NISTGPU

    coords, conn, nodeDof, nDof, bcs, top, fy0, H = _problem()
    asm = GPUAssembler(coords, nodeDof, nDof, [ElementGroup("C3D8", "vonmises", _props(fy0, H), conn)])
    solver = NISTGPU(asm, linsolver="superlu", extrapolation="off", maxIter=30, fluxResidualTolerance=1e-13,
                     fieldCorrectionTolerance=1e-15, fluxResidualFloor=0.0)  # fmt: skip
    adj = PathAdjoint(solver)
    U = solver.solveStep(AdaptiveTimeStepper(maxIncrement=1.0 / N_INC, startIncrement=1.0 / N_INC),
                         [Dirichlet(d, v) for d, v in bcs])  # fmt: skip
    J0, Uref = _oracle_path(coords, conn, nodeDof, nDof, bcs, top, fy0, H)
    assert np.abs(U.cpu().numpy() - Uref).max() <= 1e-10 * np.abs(Uref).max()
    assert float((asm.groups[0]._dev["stateRef"][12] > 0).double().mean()) > 0.5
    cP = asm.constructDofVector()
    cP[torch.as_tensor(top, device=asm.device)] = -1.0
    ddofs = np.unique(np.concatenate([d for d, _ in bcs]))
    g = adj.gradient(ddofs, cP=cP)[0].cpu().numpy()
    rng = np.random.default_rng(4)
    h = 1e-6
    for _ in range(3):
        dfy, dH = rng.normal(0, 1, len(conn)) * fy0, rng.normal(0, 1, len(conn)) * H
        fd = (_oracle_path(coords, conn, nodeDof, nDof, bcs, top, fy0 + h * dfy, H + h * dH)[0]
              - _oracle_path(coords, conn, nodeDof, nDof, bcs, top, fy0 - h * dfy, H - h * dH)[0]) / (2 * h)  # fmt: skip
        ad = float(np.sum(g[:, 2] * dfy) + np.sum(g[:, 3] * dH))
        assert abs(ad - fd) <= 1e-6 * abs(fd), (ad, fd)
