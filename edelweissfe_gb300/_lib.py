"""ctypes binding of libefe_gb300.so (include/efe_gb300.h).

The library is the product path: if it is missing or fails to load, every call raises.
There is no CPU fallback.
"""

import ctypes
import os

from . import _build

# constants of include/efe_gb300.h
EFE_ABI_VERSION = 3
EFE_QUAD4, EFE_QUAD8, EFE_HEXA8, EFE_HEXA20 = 0, 1, 2, 3
EFE_RULE_2D_1, EFE_RULE_2D_2X2, EFE_RULE_2D_3X3 = 0, 1, 2
EFE_RULE_3D_1, EFE_RULE_3D_2X2X2, EFE_RULE_3D_3X3X3 = 3, 4, 5
EFE_SMALL_STRAIN, EFE_TOTAL_LAGRANGIAN = 0, 1
EFE_SOLID, EFE_PLANE_STRAIN, EFE_PLANE_STRESS = 0, 1, 2
EFE_MAT_LINEAR_ELASTIC, EFE_MAT_VON_MISES = 0, 1
EFE_MAT_NEOHOOKE_WA, EFE_MAT_NEOHOOKE_WB, EFE_MAT_NEOHOOKE_WC = 2, 3, 4
EFE_K_FP64, EFE_K_FP32, EFE_K_FP32_FF = 0, 1, 2
EFE_STATUS_CUTBACK, EFE_STATUS_BAD_JACOBIAN, EFE_STATUS_NONFINITE, EFE_STATUS_TC_TIMEOUT, EFE_STATUS_BOUNDS = 1, 2, 4, 8, 16
EFE_OK, EFE_ERR_ARGUMENT, EFE_ERR_UNSUPPORTED, EFE_ERR_CUDA, EFE_ERR_PATTERN = 0, 1, 2, 3, 4

# every symbol the header declares
EXPORTS = [
    "efe_abi_version",
    "efe_last_error",
    "efe_state_size",
    "efe_rule_points",
    "efe_shape_nodes",
    "efe_setup_geometry",
    "efe_compute_elements",
    "efe_compute_elements_persistent",
    "efe_compute_elements_persistent_noalloc",
    "efe_accept_state",
    "efe_fma_probe",
    "efe_csr_spmv",
    "efe_pcg_start",
    "efe_pcg_iterate",
    "efe_csr_gemv",
    "efe_csr_gemv_pairs",
    "efe_chebyshev_step",
    "efe_split_pairs",
    "efe_body_force",
    "efe_adjoint_tl",
    "efe_adjoint_small_strain",
    "efe_pattern_count",
    "efe_pattern_fill",
]


class EfeMesh(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int32),
        ("nNodes", ctypes.c_int32),
        ("nDof", ctypes.c_int64),
        ("nnz", ctypes.c_int64),
        ("coords", ctypes.c_void_p),
        ("nodeDof", ctypes.c_void_p),
        ("nodeRowLen", ctypes.c_void_p),
    ]


class EfeGroup(ctypes.Structure):
    _fields_ = [
        ("shape", ctypes.c_int32),
        ("rule", ctypes.c_int32),
        ("kinematics", ctypes.c_int32),
        ("plane", ctypes.c_int32),
        ("material", ctypes.c_int32),
        ("nProps", ctypes.c_int32),
        ("nElements", ctypes.c_int64),
        ("elementOffset", ctypes.c_int64),
        ("conn", ctypes.c_void_p),
        ("pairSlot", ctypes.c_void_p),
        ("props", ctypes.c_void_p),
        ("thickness", ctypes.c_void_p),
        ("geomG", ctypes.c_void_p),
        ("geomG32", ctypes.c_void_p),
        ("geomGlo", ctypes.c_void_p),
        ("geomS", ctypes.c_void_p),
        ("stateRef", ctypes.c_void_p),
        ("stateTemp", ctypes.c_void_p),
        ("auxRef", ctypes.c_void_p),
        ("auxTemp", ctypes.c_void_p),
        ("tileVariant", ctypes.c_int32),
    ]


EFE_PCG_WORK_DOUBLES = 6152


class EfePcg(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int64),
        ("indptr", ctypes.c_void_p),
        ("indices", ctypes.c_void_p),
        ("Kdata", ctypes.c_void_p),
        ("kPrecision", ctypes.c_int32),
        ("freeMask", ctypes.c_void_p),
        ("dinv", ctypes.c_void_p),
        ("x", ctypes.c_void_p),
        ("r", ctypes.c_void_p),
        ("z", ctypes.c_void_p),
        ("p", ctypes.c_void_p),
        ("Ap", ctypes.c_void_p),
        ("work", ctypes.c_void_p),
        ("pFF", ctypes.c_void_p),
        ("blockSize", ctypes.c_int32),
        ("patternBlock", ctypes.c_int32),
    ]


class EfeCsr(ctypes.Structure):
    _fields_ = [
        ("nRows", ctypes.c_int64),
        ("nCols", ctypes.c_int64),
        ("nnz", ctypes.c_int64),
        ("indptr", ctypes.c_void_p),
        ("indices", ctypes.c_void_p),
        ("values", ctypes.c_void_p),
        ("kPrecision", ctypes.c_int32),
        ("freeMask", ctypes.c_void_p),
        ("rowBlock", ctypes.c_int32),
    ]


class EfeWorkItem(ctypes.Structure):
    _fields_ = [
        ("mesh", ctypes.c_void_p),
        ("group", ctypes.c_void_p),
        ("U", ctypes.c_void_p),
        ("dU", ctypes.c_void_p),
        ("Kdata", ctypes.c_void_p),
        ("P", ctypes.c_void_p),
        ("F", ctypes.c_void_p),
    ]


_lib = None


def library_path():
    return _build.LIB


def load(build_if_missing=False):
    """Load libefe_gb300.so (building it first if asked).  Raises if it cannot be loaded."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise RuntimeError(
                f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                "(the CUDA path has no CPU fallback)"
            )
    lib = ctypes.CDLL(path)
    P = ctypes.c_void_p
    i32, i64, f64 = ctypes.c_int32, ctypes.c_int64, ctypes.c_double
    lib.efe_abi_version.restype = i32
    lib.efe_last_error.restype = ctypes.c_char_p
    lib.efe_state_size.restype = i32
    lib.efe_state_size.argtypes = [i32]
    lib.efe_rule_points.restype = i32
    lib.efe_rule_points.argtypes = [i32]
    lib.efe_shape_nodes.restype = i32
    lib.efe_shape_nodes.argtypes = [i32]
    lib.efe_setup_geometry.restype = i32
    lib.efe_setup_geometry.argtypes = [ctypes.POINTER(EfeMesh), ctypes.POINTER(EfeGroup), P, P]
    lib.efe_compute_elements.restype = i32
    lib.efe_compute_elements.argtypes = [
        ctypes.POINTER(EfeMesh),
        ctypes.POINTER(EfeGroup),
        i32,
        P,
        P,
        P,
        f64,
        i32,
        P,
        P,
        P,
        P,
        P,
    ]
    lib.efe_body_force.restype = i32
    lib.efe_body_force.argtypes = [ctypes.POINTER(EfeMesh), ctypes.POINTER(EfeGroup), P, i64, P, P, P]
    lib.efe_adjoint_tl.restype = i32
    lib.efe_adjoint_tl.argtypes = [ctypes.POINTER(EfeMesh), ctypes.POINTER(EfeGroup), P, P, P, P, P]
    lib.efe_adjoint_small_strain.restype = i32
    lib.efe_adjoint_small_strain.argtypes = [ctypes.POINTER(EfeMesh), ctypes.POINTER(EfeGroup), P, P, P, P, P, P, P, P, P]
    lib.efe_compute_elements_persistent.restype = i32
    lib.efe_compute_elements_persistent.argtypes = [ctypes.POINTER(EfeWorkItem), i32, i32, P, P, P]
    lib.efe_compute_elements_persistent_noalloc.restype = i32
    lib.efe_compute_elements_persistent_noalloc.argtypes = [ctypes.POINTER(EfeWorkItem), i32, i32, P, P]
    lib.efe_csr_spmv.restype = i32
    lib.efe_csr_spmv.argtypes = [ctypes.POINTER(EfePcg), P, P, P]
    lib.efe_pcg_start.restype = i32
    lib.efe_pcg_start.argtypes = [ctypes.POINTER(EfePcg), P, P]
    lib.efe_pcg_iterate.restype = i32
    lib.efe_pcg_iterate.argtypes = [ctypes.POINTER(EfePcg), i64, i32, P]
    lib.efe_csr_gemv.restype = i32
    lib.efe_csr_gemv.argtypes = [ctypes.POINTER(EfeCsr), P, f64, f64, P, P]
    lib.efe_csr_gemv_pairs.restype = i32
    lib.efe_csr_gemv_pairs.argtypes = [ctypes.POINTER(EfeCsr), P, f64, f64, P, P]
    lib.efe_chebyshev_step.restype = i32
    lib.efe_chebyshev_step.argtypes = [i64, P, P, f64, f64, i32, P, P, P, P]
    lib.efe_split_pairs.restype = i32
    lib.efe_split_pairs.argtypes = [i64, P, P, P]
    lib.efe_accept_state.restype = i32
    lib.efe_accept_state.argtypes = [ctypes.POINTER(EfeGroup), i32, P]
    lib.efe_fma_probe.restype = i32
    lib.efe_fma_probe.argtypes = [i32, i32, i64, P, P, P]
    lib.efe_pattern_count.restype = i64
    lib.efe_pattern_count.argtypes = [i32, i32, P, i32, P, P, P, i64, P, P]
    lib.efe_pattern_fill.restype = i32
    lib.efe_pattern_fill.argtypes = [i32, i32, P, i32, P, P, P, i64, P, P, P]
    if lib.efe_abi_version() != EFE_ABI_VERSION:
        raise RuntimeError("libefe_gb300 ABI version mismatch")
    _lib = lib
    return lib


def check(rc, what):
    if rc != EFE_OK:
        msg = load().efe_last_error().decode()
        if rc == EFE_ERR_UNSUPPORTED:
            raise NotImplementedError(msg)
        raise RuntimeError(f"{what} failed ({rc}): {msg}")
