"""Field output from the device state (ElementResultCollector) against the per-point accessor
getResultArray (the reference's element interface) after a plastic increment on two groups."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_collector_matches_per_point_results():
    from edelweissfe_gb300 import ElementGroup, GPUAssembler, meshes
    from edelweissfe_gb300.results import ElementResultCollector

    coords, conn, nodeDof, nDof = meshes.box(4, 2, 2, nNodes=8)
    half = len(conn) // 2
    asm = GPUAssembler(coords, nodeDof, nDof, [ElementGroup("C3D8", "vonmises", [210e3, 0.3, 250, 1000, 0, 0], conn[:half]),
                                                ElementGroup("C3D8R", "vonmises", [200e3, 0.3, 200, 500, 0, 0], conn[half:])])  # fmt: skip
    rng = np.random.default_rng(2)
    dU = torch.tensor(rng.normal(0, 2e-3, nDof), device=asm.device)
    P, F, K = asm.constructDofVector(), asm.constructDofVector(), asm.constructSystemMatrix()
    asm.computeElements(None, dU, dU, P, K, F)
    asm.acceptLastState()
    elements = rng.permutation(len(conn))[:10]
    for result, size in (("stress", 6), ("strain", 6), ("kappa", 1)):
        # the reduced-integration group has one point: ask both groups for point 0
        c = ElementResultCollector(asm, elements, range(1), result)
        table = c.getCurrentResults()
        assert table.shape == (10, size)
        for i, e in enumerate(elements):
            assert np.array_equal(table[i], asm.getResultArray(result, int(e), 0))
    c = ElementResultCollector(asm, [e for e in elements if e < half], range(8), "stress")
    t = c.getCurrentResults()
    for i, e in enumerate([e for e in elements if e < half]):
        for q in range(8):
            assert np.array_equal(t[i, q], asm.getResultArray("stress", int(e), q))
    with pytest.raises(KeyError):
        ElementResultCollector(asm, elements, range(1), "nothing")
