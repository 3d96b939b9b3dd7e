"""GB300-native element evaluation and CSR assembly for EdelweissFE's Newton solver.

The CUDA kernels live in libefe_gb300.so (sources in csrc/, C ABI in include/efe_gb300.h);
`GPUAssembler` is the host-side drop-in for NIST.computeElements + CSRGenerator.updateCSR.
"""

from .exceptions import CutbackRequest  # noqa: F401
from .library import ELEMENT_TYPES, MATERIALS, element_type, material  # noqa: F401


def __getattr__(name):
    # torch-dependent parts are imported lazily so that the C ABI and the tables load without it
    if name in ("GPUAssembler", "ElementGroup"):
        from . import assembly

        return getattr(assembly, name)
    raise AttributeError(name)
