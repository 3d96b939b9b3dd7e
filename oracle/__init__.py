"""CPU oracle for EdelweissFE's element evaluation + CSR assembly path.

TEST INFRASTRUCTURE ONLY.  This package restates, in vectorised NumPy, the
algorithm of the reference's "edelweiss" element provider (small-strain and
total-Lagrangian displacement elements, linear-elastic / von Mises / Neo-Hooke
materials) and of its COO->CSR assembly.  It exists so that the tests, the
`smoke()` check and the CPU-baseline leg of `bench.py` can check the CUDA
product path against an independent statement of the reference algorithm.
The product (`edelweissfe_gb300`) never imports it.

Every function cites the reference file:line it follows (paths relative to the
EdelweissFE project root).  The restatement is pinned against fixtures that
were produced by running the reference itself (`tests/golden/make_golden.py`).
"""


from .exceptions import CutbackRequest  # noqa: F401
