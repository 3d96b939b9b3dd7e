"""efe_body_force (GPUAssembler.computeBodyForce) against the oracle's restatement of the reference's
computeBodyForce (pinned to the reference in test_integration_cpu.py): all elements and a subset (an
element set), 2D with per-element section thickness and 3D, small-strain and total-Lagrangian types,
the Hexa20 geometry fit included.  Atomics accumulate the nodal sums, so the bound is relative
(1e-13 of the largest entry), not bitwise."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CASES = [("CPE4", 4, 2), ("CPS8R", 8, 2), ("CPE8RTL", 8, 2), ("C3D8", 8, 3), ("C3D20", 20, 3), ("C3D20TL", 20, 3)]


def _mesh(nn, dim):
    from edelweissfe_gb300 import meshes

    if dim == 2:
        coords, conn, nodeDof, nDof = meshes.rect(5, 3, lX=1.0, lY=0.6, nNodes=nn)
        coords = meshes.jitter(coords, 0.1, [0.2, 0.2], 2, [0, 0], [1.0, 0.6])
        thickness = np.linspace(0.5, 1.5, len(conn))
    else:
        coords, conn, nodeDof, nDof = meshes.box(3, 2, 2, nNodes=nn)
        coords = meshes.jitter(coords, 0.1, [1 / 3, 1 / 2, 1 / 2], 2, [0, 0, 0], [1, 1, 1])
        thickness = np.ones(len(conn))
    return coords, conn, nodeDof, nDof, thickness


def oracle_body_force(elType, kind, props, coords, conn, nodeDof, nDof, thickness, load, elements):
    from oracle.assembly import Model

    om = Model(coords, nodeDof, nDof, [dict(elType=elType, kind=kind, props=np.tile(props, (len(conn), 1)), conn=conn,
                                            thickness=thickness, order=np.arange(len(conn)))])  # fmt: skip
    return om.body_force(load, elements)


@pytest.mark.parametrize("elType,nn,dim", CASES)
def test_body_force_matches_oracle(elType, nn, dim):
    from edelweissfe_gb300 import ElementGroup, GPUAssembler

    coords, conn, nodeDof, nDof, thickness = _mesh(nn, dim)
    kind, props = ("neohookewa", [400.0, 4000.0]) if elType.endswith("TL") else ("linearelastic", [210e3, 0.3])
    asm = GPUAssembler(coords, nodeDof, nDof, [ElementGroup(elType, kind, np.array(props), conn, thickness)],
                       precision="fp64")  # fmt: skip
    load = np.array([1.5, -2.0, 0.7][:dim])
    scale = np.abs(oracle_body_force(elType, kind, props, coords, conn, nodeDof, nDof, thickness, load, None)).max()
    for elements in (None, np.arange(0, len(conn), 2)):
        P = asm.constructDofVector()
        asm.computeBodyForce(P, load, elements)
        want = oracle_body_force(elType, kind, props, coords, conn, nodeDof, nDof, thickness, load, elements)
        assert np.abs(P.cpu().numpy() - want).max() <= 1e-13 * scale
