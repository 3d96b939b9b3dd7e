"""Host logic of batching: chunk_meshes keeps every batch's CSR pattern within int32 indexing."""

import numpy as np
import pytest


def _mesh(nEl, nn):
    return {"conn": np.zeros((nEl, nn), np.int32)}


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
