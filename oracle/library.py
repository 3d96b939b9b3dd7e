"""Element-type table of the reference's "edelweiss" displacement elements.

Restates `edelweissfe/elements/library.py:33-551` (elLibrary): for every element
type the node count, spatial dimension, quadrature points (xi, eta, zeta),
weights, plane-strain flag and element class (small strain or total
Lagrangian).  The numbers are generated with the same floating-point
expressions as the reference table so that they agree bit for bit.
"""

import numpy as np

# Gauss constants, reference library.py:33-47
_g = 1 / np.sqrt(3)
_s = np.sqrt(0.6)
_w1 = (5 / 9) ** 2
_w2 = (5 / 9) * (8 / 9)
_w3 = (8 / 9) ** 2
_w1H = (5 / 9) ** 3
_w2H = (5 / 9) ** 2 * (8 / 9)
_w3H = (5 / 9) * (8 / 9) ** 2
_w4H = (8 / 9) ** 3
_wI = np.array([_w1H, _w2H, _w1H])
_wII = np.array([_w2H, _w3H, _w2H])
_s8 = 1 / np.sqrt(3) * np.array([-1, 1, 1, -1])
_t8 = 1 / np.sqrt(3) * np.array([-1, -1, 1, 1])
_s20 = np.array([-1, 0, 1])
_t20 = np.array([-1, -1, -1, 0, 0, 0, 1, 1, 1])


def _rule(name):
    """Quadrature rules used by the table (library.py:52-533)."""
    if name == "2d_2x2":  # e.g. CPE4 library.py:52-67
        return (_g * np.array([1, 1, -1, -1]), _g * np.array([1, -1, -1, 1]), None, np.ones(4))
    if name == "2d_1":  # e.g. CPE4R library.py:68-83
        return (np.array([0]), np.array([0]), None, np.array([4]))
    if name == "2d_3x3":  # e.g. CPE4E / CPE8 library.py:84-115
        return (
            _s * np.array([0, -1, -1, 1, 1, -1, 0, 1, 0]),
            _s * np.array([0, -1, 1, 1, -1, 0, 1, 0, -1]),
            None,
            np.array([_w3, _w1, _w1, _w1, _w1, _w2, _w2, _w2, _w2]),
        )
    if name == "3d_2x2x2":  # e.g. C3D8 library.py:212-227, C3D20R :276-291
        return (
            1 / np.sqrt(3) * np.hstack([-np.ones(4), np.ones(4)]),
            np.hstack([_t8, _t8]),
            np.hstack([_s8, _s8]),
            np.ones(8),
        )
    if name == "3d_1":  # C3D8R library.py:228-243
        return (np.array([0]), np.array([0]), np.array([0]), np.array([8]))
    if name == "3d_3x3x3":  # C3D8E / C3D20 library.py:244-275
        return (
            _s * np.hstack([-np.ones(9), np.zeros(9), np.ones(9)]),
            _s * np.hstack([_t20, _t20, _t20]),
            _s * np.hstack([_s20 for _ in range(9)]),
            np.hstack([_wI, _wII, _wI, _wII, np.array([_w3H, _w4H, _w3H]), _wII, _wI, _wII, _wI]),
        )
    raise KeyError(name)


# base name -> (nNodes, dim, plane strain flag, rule regular, rule reduced, rule extended)
_BASES = {
    "CPE4": (4, 2, True, "2d_2x2", "2d_1", "2d_3x3"),
    "CPS4": (4, 2, False, "2d_2x2", "2d_1", "2d_3x3"),
    "CPE8": (8, 2, True, "2d_3x3", "2d_2x2", None),
    "CPS8": (8, 2, False, "2d_3x3", "2d_2x2", None),
    "C3D8": (8, 3, None, "3d_2x2x2", "3d_1", "3d_3x3x3"),
    "C3D20": (20, 3, None, "3d_3x3x3", "3d_2x2x2", None),
}


def _build():
    lib = {}
    for tl in (False, True):
        for base, (nn, dim, pe, reg, red, ext) in _BASES.items():
            for suffix, rule in (("", reg), ("R", red), ("E", ext), ("N", reg)):
                if rule is None:
                    continue
                if suffix == "E" and tl is False and base in ("CPE8", "CPS8", "C3D20"):
                    continue
                name = base + suffix + ("TL" if tl else "")
                xi, eta, zeta, w = _rule(rule)
                lib[name] = dict(
                    elClass="DisplacementTLElement" if tl else "DisplacementElement",
                    nNodes=nn,
                    nDof=nn * dim,
                    nSpatialDimensions=dim,
                    nInt=len(w),
                    xi=xi,
                    eta=eta,
                    zeta=zeta,
                    w=w,
                    plStrain=pe,
                    index=np.array([0, 1, 3]) if dim == 2 else np.arange(6),
                    matSize=3 if dim == 2 else 6,
                )
    return lib


elLibrary = _build()


def get(elType: str) -> dict:
    """Case-insensitive lookup, like the reference's CaseInsensitiveDict (library.py:50)."""
    return elLibrary[elType.upper()]
