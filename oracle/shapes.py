"""Shape functions and their natural-coordinate derivatives.

The reference writes the shape functions explicitly in
`edelweissfe/elements/displacementelement/_elementcomputationmatrices.py:106-212`
(computeNOperator) and obtains the Jacobian by a polynomial fit of the nodal
coordinates (`_J2D4:215`, `_J2D8:252`, `_J3D8:306`, `_J3D20:369`) and the
derivative tables `_Ndiff2D`/`_Ndiff3D`
(`displacementtlelement/_elementcomputationmatrices.py:309-498`).  Both evaluate
the derivatives at quadrature point i at the natural coordinates
(eta_i, xi_i, zeta_i), i.e. with the first two library coordinates swapped.
This module restates the standard serendipity/Lagrange shape functions with
the reference's node numbering and evaluates them at that swapped point.
"""

import numpy as np

# natural coordinates of the nodes, in the reference's node order
# (computeNOperator, _elementcomputationmatrices.py:127-210)
NODES = {
    (2, 4): np.array([[-1, -1], [1, -1], [1, 1], [-1, 1]], float),
    (2, 8): np.array([[-1, -1], [1, -1], [1, 1], [-1, 1], [0, -1], [1, 0], [0, 1], [-1, 0]], float),
    (3, 8): np.array(
        [[-1, -1, -1], [-1, -1, 1], [1, -1, 1], [1, -1, -1], [-1, 1, -1], [-1, 1, 1], [1, 1, 1], [1, 1, -1]],
        float,
    ),
    (3, 20): np.array(
        [
            [-1, -1, -1], [-1, -1, 1], [1, -1, 1], [1, -1, -1],
            [-1, 1, -1], [-1, 1, 1], [1, 1, 1], [1, 1, -1],
            [-1, -1, 0], [0, -1, 1], [1, -1, 0], [0, -1, -1],
            [-1, 1, 0], [0, 1, 1], [1, 1, 0], [0, 1, -1],
            [-1, 0, -1], [-1, 0, 1], [1, 0, 1], [1, 0, -1],
        ],
        float,
    ),
}  # fmt: skip


def shape_and_derivatives(dim: int, nNodes: int, p: np.ndarray):
    """N [nNodes] and dN/dxi [dim, nNodes] at natural point p [dim]."""
    c = NODES[(dim, nNodes)]
    p = np.asarray(p, float)
    N = np.zeros(nNodes)
    dN = np.zeros((dim, nNodes))
    quadratic = nNodes > 2**dim
    for a in range(nNodes):
        ca = c[a]
        if not quadratic or np.all(np.abs(ca) == 1):
            lin = 1 + ca * p  # [dim]
            base = np.prod(lin) / 2**dim
            dbase = np.array([ca[k] * np.prod(np.delete(lin, k)) / 2**dim for k in range(dim)])
            if quadratic:
                s = np.dot(ca, p) - (dim - 1)
                N[a] = base * s
                dN[:, a] = dbase * s + base * ca
            else:
                N[a] = base
                dN[:, a] = dbase
        else:
            m = int(np.nonzero(ca == 0)[0][0])
            others = [k for k in range(dim) if k != m]
            lin = {k: 1 + ca[k] * p[k] for k in others}
            q = 1 - p[m] ** 2
            N[a] = q * np.prod([lin[k] for k in others]) / 2 ** (dim - 1)
            dN[m, a] = -2 * p[m] * np.prod([lin[k] for k in others]) / 2 ** (dim - 1)
            for k in others:
                dN[k, a] = q * ca[k] * np.prod([lin[j] for j in others if j != k]) / 2 ** (dim - 1)
    return N, dN


def derivative_table(lib_entry: dict) -> np.ndarray:
    """dN/dxi at every quadrature point, evaluated at the swapped point (eta_i, xi_i, zeta_i).

    Returns [nInt, dim, nNodes].  Equivalent to the reference's `_Ndiff2D`/`_Ndiff3D`
    (displacementtlelement/_elementcomputationmatrices.py:309,370) and to the
    derivatives implied by the polynomial-fit Jacobians (`_J2D4` etc.).
    """
    dim = lib_entry["nSpatialDimensions"]
    nn = lib_entry["nNodes"]
    nInt = lib_entry["nInt"]
    out = np.zeros((nInt, dim, nn))
    for i in range(nInt):
        if dim == 2:
            p = np.array([lib_entry["eta"][i], lib_entry["xi"][i]], float)
        else:
            p = np.array([lib_entry["eta"][i], lib_entry["xi"][i], lib_entry["zeta"][i]], float)
        out[i] = shape_and_derivatives(dim, nn, p)[1]
    return out


def shape_table(lib_entry: dict) -> np.ndarray:
    """N at every quadrature point at the UNswapped library point (computeNOperator, :106-212)."""
    dim = lib_entry["nSpatialDimensions"]
    nn = lib_entry["nNodes"]
    out = np.zeros((lib_entry["nInt"], nn))
    for i in range(lib_entry["nInt"]):
        p = [lib_entry["xi"][i], lib_entry["eta"][i]] + ([lib_entry["zeta"][i]] if dim == 3 else [])
        out[i] = shape_and_derivatives(dim, nn, np.array(p, float))[0]
    return out


# Monomial basis of the reference's Hexa20 polynomial geometry fit, in the column order of the
# matrix A in `_J3D20` (displacementelement/_elementcomputationmatrices.py:392-415); exponents of
# the three natural coordinates (s, t, u) = node coordinates of NODES[(3, 20)].
_H20_BASIS = [
    (0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 0), (0, 1, 1), (1, 0, 1), (2, 0, 0), (0, 2, 0),
    (0, 0, 2), (2, 1, 0), (1, 2, 0), (0, 2, 1), (0, 1, 2), (1, 0, 2), (2, 0, 1), (1, 1, 1), (2, 1, 1),
    (1, 2, 1), (1, 1, 2),
]  # fmt: skip


def _h20_coefficient_rows():
    """inv(A) of the Hexa20 fit: row k maps nodal values to the coefficient of monomial k."""
    c = NODES[(3, 20)]
    A = np.array([[np.prod(c[a] ** np.array(e)) for e in _H20_BASIS] for a in range(20)], float)
    return np.linalg.inv(A)


def jacobian_table(lib_entry: dict) -> np.ndarray:
    """M [nInt, dim, nNodes] with J_i = M_i @ X (X [nNodes, dim]) exactly as the reference forms J.

    For Quad4, Quad8 and Hexa8 the reference's polynomial-fit Jacobians equal the isoparametric
    Jacobian at the swapped point, so M = derivative_table.  For Hexa20, `_J3D20`
    (displacementelement/_elementcomputationmatrices.py:369-540, identical copy in
    displacementtlelement/_elementcomputationmatrices.py:655-826) differentiates the t*u monomial
    with respect to u as ``a5 * zeta`` instead of ``a5 * xi`` (third row, term ``ax[5] * z[i]``), so
    its third row carries the extra term (zeta_i - xi_i) * a5.  That is restated here.
    """
    M = derivative_table(lib_entry).copy()
    if lib_entry["nSpatialDimensions"] == 3 and lib_entry["nNodes"] == 20:
        invA = _h20_coefficient_rows()
        for i in range(lib_entry["nInt"]):
            M[i, 2, :] += (lib_entry["zeta"][i] - lib_entry["xi"][i]) * invA[5, :]
    return M
