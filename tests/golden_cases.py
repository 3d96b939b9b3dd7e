"""Loading and replaying the golden fixtures written by tests/golden/make_golden.py.

Each fixture holds one mesh (coordinates, connectivity, DOF map), one element
type and material, and a sequence of computeElements calls recorded from the
reference: inputs (U_np, dU, increment number) and outputs (P, F, CSR data,
per-element state after the call, or the element that raised CutbackRequest).
"""

import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def case_names():
    skip = {"library", "geometry"}
    return sorted(
        os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")) if os.path.basename(p)[:-4] not in skip
    )


def load(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as d:
        return {k: d[k] for k in d.files}


def calls(case):
    """Yield dicts per recorded call, with a flag telling whether an increment was accepted before it."""
    n = int(case["n_calls"])
    prev_inc = 0
    for c in range(n):
        inc = int(case[f"c{c}_inc"])
        rec = dict(
            index=c,
            U=case[f"c{c}_U"],
            dU=case[f"c{c}_dU"],
            inc=inc,
            accept_before=inc != prev_inc,
            raised=int(case[f"c{c}_raised"]),
            cutback=float(case[f"c{c}_cutback"]),
        )
        for k in ("P", "F", "Kdata", "state"):
            key = f"c{c}_{k}"
            rec[k] = case[key] if key in case else None
        prev_inc = inc
        yield rec


def oracle_model(case):
    """An oracle.assembly.Model for a fixture (single element group in element order)."""
    from oracle.assembly import Model

    E = len(case["conn"])
    g = dict(
        elType=str(case["elType"]),
        kind=str(case["kind"]),
        props=np.asarray(case["props"], float),
        conn=np.asarray(case["conn"]),
        thickness=np.asarray(case["thickness"], float),
        order=np.arange(E),
    )
    return Model(case["coords"], case["node_dof"], int(case["nDof"]), [g])
