"""Element and material names of the reference's "edelweiss" provider, mapped to library codes.

Element types follow `edelweissfe/elements/library.py:50-551` (30 types plus the 12 "N"
aliases): CPE4/CPS4 (regular 2x2, R 1-point, E 3x3), CPE8/CPS8 (3x3, R 2x2), C3D8 (2x2x2,
R 1-point, E 3x3x3), C3D20 (3x3x3, R 2x2x2); a "TL" suffix selects the total-Lagrangian
element (`elements/displacementtlelement`).  Material names follow
`edelweissfe/config/materiallibrary.py:32-123` (provider "edelweiss").
"""

from dataclasses import dataclass

from . import _lib as L


@dataclass(frozen=True)
class ElementType:
    name: str
    shape: int
    rule: int
    kinematics: int
    plane: int
    nNodes: int
    dim: int
    nInt: int

    @property
    def nDof(self):
        return self.nNodes * self.dim

    @property
    def totalLagrangian(self):
        return self.kinematics == L.EFE_TOTAL_LAGRANGIAN


_NQ = {L.EFE_RULE_2D_1: 1, L.EFE_RULE_2D_2X2: 4, L.EFE_RULE_2D_3X3: 9, L.EFE_RULE_3D_1: 1,
       L.EFE_RULE_3D_2X2X2: 8, L.EFE_RULE_3D_3X3X3: 27}  # fmt: skip
# base -> (shape, nodes, dim, plane, regular, reduced, extended)
_BASES = {
    "CPE4": (L.EFE_QUAD4, 4, 2, L.EFE_PLANE_STRAIN, L.EFE_RULE_2D_2X2, L.EFE_RULE_2D_1, L.EFE_RULE_2D_3X3),
    "CPS4": (L.EFE_QUAD4, 4, 2, L.EFE_PLANE_STRESS, L.EFE_RULE_2D_2X2, L.EFE_RULE_2D_1, L.EFE_RULE_2D_3X3),
    "CPE8": (L.EFE_QUAD8, 8, 2, L.EFE_PLANE_STRAIN, L.EFE_RULE_2D_3X3, L.EFE_RULE_2D_2X2, None),
    "CPS8": (L.EFE_QUAD8, 8, 2, L.EFE_PLANE_STRESS, L.EFE_RULE_2D_3X3, L.EFE_RULE_2D_2X2, None),
    "C3D8": (L.EFE_HEXA8, 8, 3, L.EFE_SOLID, L.EFE_RULE_3D_2X2X2, L.EFE_RULE_3D_1, L.EFE_RULE_3D_3X3X3),
    "C3D20": (L.EFE_HEXA20, 20, 3, L.EFE_SOLID, L.EFE_RULE_3D_3X3X3, L.EFE_RULE_3D_2X2X2, None),
}


def _table():
    t = {}
    for base, (shape, nn, dim, plane, reg, red, ext) in _BASES.items():
        for tl in (False, True):
            for suffix, rule in (("", reg), ("R", red), ("E", ext), ("N", reg)):
                if rule is None:
                    continue
                name = base + suffix + ("TL" if tl else "")
                kin = L.EFE_TOTAL_LAGRANGIAN if tl else L.EFE_SMALL_STRAIN
                t[name] = ElementType(name, shape, rule, kin, plane, nn, dim, _NQ[rule])
    return t


ELEMENT_TYPES = _table()

MATERIALS = {
    "linearelastic": (L.EFE_MAT_LINEAR_ELASTIC, 2, 0),
    "vonmises": (L.EFE_MAT_VON_MISES, 6, 1),
    "neohookewa": (L.EFE_MAT_NEOHOOKE_WA, 2, 1),
    "neohookewb": (L.EFE_MAT_NEOHOOKE_WB, 2, 1),
    "neohookewc": (L.EFE_MAT_NEOHOOKE_WC, 2, 1),
}
HYPERELASTIC = ("neohookewa", "neohookewb", "neohookewc")


def element_type(name: str) -> ElementType:
    try:
        return ELEMENT_TYPES[name.upper()]
    except KeyError:
        raise KeyError(f"element type {name!r} is not an edelweiss displacement element") from None


def material(name: str):
    """(code, number of properties, number of material state variables) of a material name."""
    try:
        return MATERIALS[name.lower()]
    except KeyError:
        raise KeyError(f"material {name!r} is not supported by the GPU element path") from None
