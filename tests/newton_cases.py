"""Newton-run fixtures (tests/golden/make_newton_golden.py): load a case and build the GPU solver for it."""

import glob
import os

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GOLDEN = os.path.join(HERE, "newton")


def names(subdir="newton"):
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(HERE, subdir, "*.npz")))


def load(name, subdir="newton"):
    with np.load(os.path.join(HERE, subdir, name + ".npz")) as d:
        return {k: d[k] for k in d.files}


def groups(case):
    """Consecutive runs of elements with the same (type, material, properties) -> ElementGroup list."""
    from edelweissfe_gb300 import ElementGroup

    out = []
    key = None
    start = 0
    n = len(case["conn"])
    for e in range(n + 1):
        k = None if e == n else (str(case["elTypes"][e]), str(case["kinds"][e]))
        if k != key:
            if key is not None:
                et, kind = key
                out.append(ElementGroup(et, kind, case["props"][start:e], case["conn"][start:e],
                                        case["thickness"][start:e]))  # fmt: skip
            key, start = k, e
    return out


def step_inputs(case):
    from edelweissfe_gb300.solver import AdaptiveTimeStepper, BodyForce, Dirichlet, NodeForces

    c = case["step_controls"]
    stepper = AdaptiveTimeStepper(0.0, c[8], c[0], c[1], c[2], int(c[3]), c[9])
    dirichlets = [Dirichlet(case[f"dirichlet{k}_dofs"], case[f"dirichlet{k}_values"])
                  for k in range(10) if f"dirichlet{k}_dofs" in case]  # fmt: skip
    nodeforces = [NodeForces(case[f"nodeforce{k}_dofs"], case[f"nodeforce{k}_values"])
                  for k in range(10) if f"nodeforce{k}_dofs" in case]  # fmt: skip
    bodyforces = [BodyForce(case[f"bodyforce{k}_elements"], case[f"bodyforce{k}_values"])
                  for k in range(10) if f"bodyforce{k}_elements" in case]  # fmt: skip
    controls = dict(maxIter=int(c[4]), criticalIter=int(c[5]), maxGrowingIter=int(c[6]), cutbackFactor=float(c[7]))
    return stepper, dirichlets, nodeforces, bodyforces, controls
