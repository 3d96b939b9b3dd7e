"""Reverse mode of the small-strain element pass (efe_adjoint_small_strain) and the path adjoint
over plastic load increments (PathAdjoint), in FP64, against central differences.

1. One increment: L = sum(sbar * s_new) + pbar . P of one element pass from a plastic state s0
   with increment dU (von Mises with saturation hardening, and linear elasticity); directional
   derivatives of L in dU, in the state s0 and in the six material properties, h = 1e-7 relative;
   agreement to 1e-6 relative.  Both forms of the reverse pass: FP64 B-products (FP64 assembler)
   and float-float B-products (mixed assembler, which carries the float-float geometry).
   The nodal coordinates too (dN/dX and det J, the Hexa20 Jacobian term included), against central
   differences of L over moved nodes (geometry set up again).  Plane stress (CPS4, CPS8) through the
   reference's local Newton on eps33 (basehypoelasticmaterial.py:71-130), whose von Mises form
   restarts every local iteration from a zero stress and carries kappa from one local iteration to
   the next: both increments are sized just past yield, where that local Newton converges.
2. The plastic path: C3D20 (3x3x3 Gauss) von Mises cube, 2x2x2 elements with per-element yield
   stress U[200, 300] and hardening U[800, 1200]; bottom u_y = 0, left u_x = 0, back u_z = 0, top
   u_y -> 0.5 % in 4 increments; J = the total top reaction.  dJ/d(fy0, H) and dJ/dX by the path
   adjoint vs central differences of J through full Newton solves (h = 1e-6 relative), and the
   mixed (FP32-tangent, device PCG with refinement) adjoint vs the FP64 one.
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _model(elType, material, seed, precision="fp64"):
    from edelweissfe_gb300 import ElementGroup, GPUAssembler, meshes

    rng = np.random.default_rng(seed)
    if elType.startswith("C3D"):
        nn = 20 if "20" in elType else 8
        coords, conn, nodeDof, nDof = meshes.box(2, 2, 1, nNodes=nn)
        coords = meshes.jitter(coords, 0.1, [0.5, 0.5, 1.0], seed, [0, 0, 0], [1, 1, 1])
    else:
        coords, conn, nodeDof, nDof = meshes.rect(3, 2, nNodes=8 if "8" in elType else 4)
        coords = meshes.jitter(coords, 0.1, [1 / 3, 0.5], seed, [0, 0], [1, 1])
    E = len(conn)
    if material == "vonmises" and elType.startswith("CPS"):
        # the reference's plane-stress return converges only slightly past yield: a narrow spread of
        # yield strains keeps every element inside that window under one uniform strain
        props = np.stack([rng.uniform(205e3, 215e3, E), rng.uniform(0.28, 0.32, E), rng.uniform(240, 260, E),
                          rng.uniform(800, 1200, E), rng.uniform(20, 80, E), rng.uniform(5, 20, E)], 1)  # fmt: skip
    elif material == "vonmises":
        props = np.stack([rng.uniform(190e3, 230e3, E), rng.uniform(0.25, 0.35, E), rng.uniform(200, 300, E),
                          rng.uniform(800, 1200, E), rng.uniform(20, 80, E), rng.uniform(5, 20, E)], 1)  # fmt: skip
    else:
        props = np.stack([rng.uniform(190e3, 230e3, E), rng.uniform(0.25, 0.35, E)], 1)
    asm = GPUAssembler(coords, nodeDof, nDof, [ElementGroup(elType, material, props, conn, 1.0)], precision=precision)
    return asm, coords, nodeDof, nDof, props


def _uniaxial(coords, nodeDof, nDof, strain):
    dim = coords.shape[1]
    U = np.zeros(nDof)
    has = nodeDof >= 0  # Quad8 meshes carry unused centre nodes (nodeDof -1)
    d, c = nodeDof[has], coords[has]
    U[d + 1] = strain * c[:, 1]
    U[d + 0] = -0.3 * strain * c[:, 0]
    if dim == 3:
        U[d + 2] = -0.3 * strain * c[:, 2]
    return U


@pytest.mark.parametrize("precision", ["fp64", "mixed"])  # mixed: B-products in float-float arithmetic
@pytest.mark.parametrize("elType,material", [("C3D8", "vonmises"), ("C3D20", "vonmises"), ("C3D20R", "vonmises"),
                                             ("CPE8", "vonmises"), ("CPE4", "vonmises"), ("C3D8", "linearelastic"),
                                             ("CPS8", "vonmises"), ("CPS4", "vonmises"), ("CPS8", "linearelastic")])
def test_increment_reverse_matches_finite_differences(elType, material, precision):
    asm, coords, nodeDof, nDof, props = _model(elType, material, 5, precision)
    dev = asm.device
    rng = np.random.default_rng(6)
    g = asm.groups[0]._dev
    planeStress = elType.startswith("CPS")
    # plane stress: 1.1e-3 per increment, just past yield, where the reference's local Newton
    # converges; its first local iteration flows plastically, the later ones carry kappa over
    e1, e2, n1, n2 = (0.0011, 0.0011, 2e-6, 2e-6) if planeStress else (0.003, 0.001, 1e-4, 2e-4)
    dU1 = torch.tensor(_uniaxial(coords, nodeDof, nDof, e1) + rng.normal(0, n1, nDof), device=dev)
    P, F, K = asm.constructDofVector(), asm.constructDofVector(), asm.constructSystemMatrix()
    asm.computeElements(None, dU1, dU1, P, K, F)
    asm.acceptLastState()
    s0 = g["stateRef"].clone()
    if material == "vonmises":
        assert float((s0[12] > 0).double().mean()) > 0.5  # a plastic state
    dU = torch.tensor(_uniaxial(coords, nodeDof, nDof, e2) + rng.normal(0, n2, nDof), device=dev)
    sbar = torch.tensor(rng.normal(0, 1, tuple(s0.shape)), device=dev)
    pbar = torch.tensor(rng.normal(0, 1, nDof), device=dev)
    props_t = g["props"].clone()

    def L(dUx, s0x, px):
        g["stateRef"].copy_(s0x)
        asm.setProperties(0, px)
        P, F, K = asm.constructDofVector(), asm.constructDofVector(), asm.constructSystemMatrix()
        asm.computeElements(None, dUx, dUx, P, K, F)
        return float((sbar * g["stateTemp"]).sum() + (pbar * P).sum())

    L0 = L(dU, s0, props_t)
    if material == "vonmises":
        assert float((g["stateTemp"][12] > s0[12]).double().mean()) > 0.5  # the increment flows plastically
    dUbar = asm.constructDofVector()
    s0bar = torch.zeros_like(s0)
    gp = torch.zeros_like(props_t)
    gx = torch.zeros((asm.nNodes, asm.dim), dtype=torch.float64, device=dev)
    asm.adjointSmallStrain(0, s0, dU, dUbar, Pbar=pbar, stateBarIn=sbar, stateBarOut=s0bar, gProps=gp, gX=gx)
    # the coordinate adjoint changes nothing else: the other adjoints equal those of a pass without
    # gX (to the rounding of the atomic sums' order)
    dUbar2, gp2 = asm.constructDofVector(), torch.zeros_like(props_t)
    asm.adjointSmallStrain(0, s0, dU, dUbar2, Pbar=pbar, stateBarIn=sbar, gProps=gp2)
    for x, y in ((dUbar, dUbar2), (gp, gp2)):
        assert float((x - y).abs().max()) <= 1e-13 * float(y.abs().max())

    def LX(X):
        asm.setCoordinates(X)
        try:
            return L(dU, s0, props_t)
        finally:
            asm.setCoordinates(coords)

    h = 1e-7
    for what in ("dU", "state", "props", "coords"):
        for k in range(2):
            if what == "dU":
                d = torch.tensor(rng.normal(0, 1, nDof), device=dev) * 1e-3
                fd = (L(dU + h * d, s0, props_t) - L(dU - h * d, s0, props_t)) / (2 * h)
                ad = float((dUbar * d).sum())
            elif what == "state":
                d = torch.tensor(rng.normal(0, 1, tuple(s0.shape)), device=dev) * s0.abs().amax(1, keepdim=True)
                fd = (L(dU, s0 + h * d, props_t) - L(dU, s0 - h * d, props_t)) / (2 * h)
                ad = float((s0bar * d).sum())
            elif what == "props":
                d = torch.tensor(rng.normal(0, 1, tuple(props_t.shape)), device=dev) * props_t
                fd = (L(dU, s0, props_t + h * d) - L(dU, s0, props_t - h * d)) / (2 * h)
                ad = float((gp * d).sum())
            else:  # node coordinates (element size ~0.3-0.5): dN/dX and det J
                d = rng.normal(0, 0.05, coords.shape)
                fd = (LX(coords + h * d) - LX(coords - h * d)) / (2 * h)
                ad = float((gx.cpu().numpy() * d).sum())
            assert abs(ad - fd) <= 1e-6 * max(abs(fd), 1e-3 * abs(L0)), (what, k, ad, fd)


def test_reverse_pass_refuses_wrong_buffers():
    """Buffers of the wrong shape, dtype or device are refused on the host, before any launch."""
    asm, coords, nodeDof, nDof, props = _model("C3D8", "vonmises", 5)
    dev = asm.device
    g = asm.groups[0]._dev
    s0 = g["stateRef"].clone()
    dU = asm.constructDofVector()
    ok = dict(dUbar=asm.constructDofVector())
    bad = {
        "gX": torch.zeros((asm.nNodes - 1, asm.dim), dtype=torch.float64, device=dev),
        "gProps": torch.zeros((1, 6), dtype=torch.float64, device=dev),
        "stateBarOut": torch.zeros_like(s0)[:, :-1],
        "Pbar": torch.zeros(nDof, dtype=torch.float32, device=dev),
        "stateBarIn": torch.zeros_like(s0).cpu(),
    }
    for name, t in bad.items():
        with pytest.raises(ValueError, match=name):
            asm.adjointSmallStrain(0, s0, dU, **ok, **{name: t})
    with pytest.raises(ValueError, match="dUbar"):
        asm.adjointSmallStrain(0, s0, dU, asm.constructDofVector()[:-1])


def _path_problem(fy0, H, precision="fp64", linsolver="superlu", coords=None):
    from edelweissfe_gb300 import ElementGroup, GPUAssembler, meshes
    from edelweissfe_gb300.adjoint import PathAdjoint
    from edelweissfe_gb300.solver import AdaptiveTimeStepper, Dirichlet, NISTGPU

    c0, conn, nodeDof, nDof = meshes.box(2, 2, 2, nNodes=20)
    coords = c0 if coords is None else coords
    E = len(conn)
    props = np.stack([np.full(E, 210e3), np.full(E, 0.3), fy0, H, np.zeros(E), np.zeros(E)], 1)
    asm = GPUAssembler(coords, nodeDof, nDof, [ElementGroup("C3D20", "vonmises", props, conn)], precision=precision)
    x, y, z = c0[:, 0], c0[:, 1], c0[:, 2]  # the boundary sets of the unmoved box
    top = nodeDof[y > 1 - 1e-9] + 1
    dirichlets = [Dirichlet(nodeDof[y < 1e-9] + 1, 0.0), Dirichlet(nodeDof[x < 1e-9], 0.0),
                  Dirichlet(nodeDof[z < 1e-9] + 2, 0.0), Dirichlet(top, 0.005)]  # fmt: skip
    solver = NISTGPU(asm, linsolver=linsolver, extrapolation="off", maxIter=25, fluxResidualTolerance=1e-12,
                     fieldCorrectionTolerance=1e-14, fluxResidualFloor=0.0, pcgTolerance=1e-14)  # fmt: skip
    adj = PathAdjoint(solver)
    solver.solveStep(AdaptiveTimeStepper(maxIncrement=0.25, startIncrement=0.25), dirichlets)
    J = -float(solver.lastP[torch.as_tensor(top, device=asm.device)].sum())
    ddofs = np.unique(np.concatenate([d.dofs for d in dirichlets]))
    return J, adj, ddofs, top, asm


def _path_gradient(adj, ddofs, top, asm):
    cP = asm.constructDofVector()
    cP[torch.as_tensor(top, device=asm.device)] = -1.0
    return adj.gradient(ddofs, cP=cP)[0].cpu().numpy()


def test_path_adjoint_matches_finite_differences():
    rng = np.random.default_rng(8)
    fy0 = rng.uniform(200, 300, 8)
    H = rng.uniform(800, 1200, 8)
    J0, adj, ddofs, top, asm = _path_problem(fy0, H)
    assert len(adj.checkpoints) >= 5
    assert float((asm.groups[0]._dev["stateRef"][12] > 0).double().mean()) > 0.5
    g = _path_gradient(adj, ddofs, top, asm)
    h = 1e-6
    for k in range(3):
        dfy, dH = rng.normal(0, 1, 8) * fy0, rng.normal(0, 1, 8) * H
        fd = (_path_problem(fy0 + h * dfy, H + h * dH)[0] - _path_problem(fy0 - h * dfy, H - h * dH)[0]) / (2 * h)
        ad = float(np.sum(g[:, 2] * dfy) + np.sum(g[:, 3] * dH))
        assert abs(ad - fd) <= 1e-6 * abs(fd), (k, ad, fd)


def test_path_adjoint_coordinates_match_finite_differences():
    """dJ/dX of the plastic path (the total top reaction after the C3D20 von Mises increments) by
    the path adjoint against central differences of J through full Newton solves on moved nodes
    (h = 1e-6 in units of a 0.05 node displacement; the prescribed values held)."""
    rng = np.random.default_rng(10)
    fy0 = rng.uniform(200, 300, 8)
    H = rng.uniform(800, 1200, 8)
    J0, adj, ddofs, top, asm = _path_problem(fy0, H)
    cP = asm.constructDofVector()
    cP[torch.as_tensor(top, device=asm.device)] = -1.0
    gX = adj.gradient(ddofs, cP=cP, coordinates=True)[1].cpu().numpy()
    coords = asm.coords.cpu().numpy().copy()
    h = 1e-6
    for k in range(2):
        d = rng.normal(0, 0.05, coords.shape)
        fd = (_path_problem(fy0, H, coords=coords + h * d)[0] - _path_problem(fy0, H, coords=coords - h * d)[0]) / (2 * h)
        ad = float(np.sum(gX * d))
        assert abs(ad - fd) <= 1e-6 * max(abs(fd), 1e-3 * abs(J0)), (k, ad, fd)


def test_path_adjoint_mixed_matches_fp64():
    rng = np.random.default_rng(9)
    fy0 = rng.uniform(200, 300, 8)
    H = rng.uniform(800, 1200, 8)
    J64, adj64, ddofs, top, asm64 = _path_problem(fy0, H)
    g64 = _path_gradient(adj64, ddofs, top, asm64)
    J32, adj32, _, _, asm32 = _path_problem(fy0, H, precision="mixed", linsolver="pcg")
    g32 = _path_gradient(adj32, ddofs, top, asm32)
    assert abs(J32 - J64) <= 1e-9 * abs(J64)
    for k in (2, 3):
        assert np.abs(g32[:, k] - g64[:, k]).max() <= 1e-8 * np.abs(g64[:, k]).max(), k
