"""C-ABI library checks that need no GPU: it loads, exports every declared symbol, and its host-side
CSR pattern / slot-map builder reproduces the reference's CSR pattern bit for bit."""

import re

import numpy as np
import pytest

import golden_cases as gc
from edelweissfe_gb300 import _build, _lib, library
from edelweissfe_gb300.pattern import build_pattern

HEADER = _build.INCLUDE + "/efe_gb300.h"


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return _lib.load()


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int32_t|int64_t|const char\*)\s+(efe_\w+)\s*\(", text, re.M)))


def test_header_declares_exports():
    assert declared_functions() == sorted(_lib.EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert lib.efe_abi_version() == _lib.EFE_ABI_VERSION
    assert lib.efe_state_size(_lib.EFE_MAT_LINEAR_ELASTIC) == 12
    assert lib.efe_state_size(_lib.EFE_MAT_VON_MISES) == 13
    assert [lib.efe_rule_points(r) for r in range(6)] == [1, 4, 9, 1, 8, 27]
    assert [lib.efe_shape_nodes(s) for s in range(4)] == [4, 8, 8, 20]


def test_element_table_matches_reference():
    d = np.load(gc.GOLDEN + "/library.npz")
    names = sorted({k.split("__")[0] for k in d.files})
    assert sorted(library.ELEMENT_TYPES) == names
    for n in names:
        et = library.element_type(n)
        meta = d[f"{n}__meta"]
        assert [et.nNodes, et.nDof, et.dim, et.nInt] == list(meta[:4])
        pe = {1: _lib.EFE_PLANE_STRAIN, 0: _lib.EFE_PLANE_STRESS, -1: _lib.EFE_SOLID}[int(meta[4])]
        assert et.plane == pe
        assert et.totalLagrangian == (str(d[f"{n}__class"]) == "DisplacementTLElement")


@pytest.mark.parametrize("name", [n for n in gc.case_names() if "indptr" in gc.load(n)])
def test_pattern_matches_reference(lib, name):
    case = gc.load(name)
    et = library.element_type(str(case["elType"]))
    indptr, indices, rowlen, slots = build_pattern(
        et.dim, len(case["coords"]), case["node_dof"], int(case["nDof"]), [case["conn"]]
    )
    assert np.array_equal(indptr, case["indptr"])
    assert np.array_equal(indices, case["indices"])
    # every element node pair's slot points at (row = dof(b), col = dof(a)) and entry (j, k) follows
    conn = case["conn"]
    nd = case["node_dof"]
    for e in range(len(conn)):
        for a in range(conn.shape[1]):
            for b in range(conn.shape[1]):
                s = slots[0][e, a, b]
                rb = nd[conn[e, b]]
                for k in range(et.dim):
                    for j in range(et.dim):
                        pos = s + k * rowlen[conn[e, b]] + j
                        assert indptr[rb + k] <= pos < indptr[rb + k + 1]
                        assert indices[pos] == nd[conn[e, a]] + j


def test_pattern_rejects_bad_dof(lib):
    with pytest.raises(RuntimeError):
        build_pattern(2, 4, np.array([0, 2, 4, 100]), 8, [np.array([[0, 1, 2, 3]])])
