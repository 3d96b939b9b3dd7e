"""Host logic of batching: chunk_meshes keeps every batch's CSR pattern within int32 indexing."""

import numpy as np
import pytest


def _mesh(nEl, nn):
    return {"conn": np.zeros((nEl, nn), np.int32)}


def test_persistent_types():
    """The element types the persistent kernel takes, in its hand-out order; plane-stress Neo-Hooke
    (refused by the reference) and other rules / materials are not among them."""
    from edelweissfe_gb300.batch import persistent_type

    assert persistent_type("C3D20TL", "neohookewa") == 0
    assert persistent_type("C3D20", "vonmises") == 1 and persistent_type("C3D20", "linearelastic") == 1
    assert persistent_type("C3D8TL", "neohookewb") == 2
    assert persistent_type("C3D8", "vonmises") == 3
    assert persistent_type("CPE8RTL", "neohookewa") == 4
    assert persistent_type("CPS8RTL", "neohookewa") is None
    assert persistent_type("C3D8R", "vonmises") is None and persistent_type("C3D8TL", "vonmises") is None
    assert persistent_type("CPE4", "linearelastic") is None


def test_chunks_respect_the_entry_bound():
    from edelweissfe_gb300.batch import chunk_meshes

    per = (20 * 3) ** 2
    limit = 10 * per  # ten Hexa20 elements per chunk at most
    ms = [_mesh(n, 20) for n in (4, 5, 3, 7, 1, 10, 2)]
    chunks = chunk_meshes(ms, "C3D20TL", limit=limit)
    assert [m for c in chunks for m in c] == ms  # order kept, nothing lost
    assert all(sum(len(m["conn"]) for m in c) * per <= limit for c in chunks)
    assert [sum(len(m["conn"]) for m in c) for c in chunks] == [9, 10, 1, 10, 2]
    assert len(chunk_meshes(ms, "C3D20TL")) == 1
    with pytest.raises(ValueError):
        chunk_meshes([_mesh(11, 20)], "C3D20TL", limit=limit)
