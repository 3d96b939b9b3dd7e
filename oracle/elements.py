"""Element evaluation (K_e, P_e, state update), vectorised over the elements of one type.

Restates `DisplacementElement.computeYourself`
(`edelweissfe/elements/displacementelement/element.py:290-346`) and
`DisplacementTLElement.computeYourself`
(`edelweissfe/elements/displacementtlelement/element.py:346-427`) for a batch of
elements of the same type and material kind.  The quadrature-point loop runs in
the reference's order; arithmetic inside one point follows the reference's
operation order.

State layout per element and quadrature point follows the reference
(`element.py:222-235`): ``[stress(6), strain(6), materialstate(m)]``.  The
total-Lagrangian element additionally keeps ``E_old`` (Green-Lagrange strain of
the last accepted state, `displacementtlelement/element.py:214-216,454-461`).
"""

import numpy as np

from . import library, materials, shapes


def _geometry(lib, X):
    """J, det J and dN/dX of every element and quadrature point.

    X [E, nN, d].  J follows computeJacobian (displacementelement/_elementcomputationmatrices.py:32-66);
    dN/dX follows computeBOperator's inv(J) (:69-103) / computeNablaN (displacementtlelement/
    _elementcomputationmatrices.py:247-281)."""
    M = shapes.jacobian_table(lib)  # [q, d, nN]
    D = shapes.derivative_table(lib)  # [q, d, nN]
    J = np.einsum("qra,eac->eqrc", M, X)
    detJ = np.linalg.det(J)
    invJ = np.linalg.inv(J)
    G = np.einsum("eqrs,qsa->eqra", invJ, D)  # dN/dX [E,q,d,nN]
    return J, detJ, G


def body_force(elType, X, load, thickness):
    """P_e [E, nDof] of a body force `load` [dim] for a batch of elements of one type
    (computeBodyForce, `displacementelement/element.py:348-371`, identical in
    `displacementtlelement/element.py:429-452`): at every quadrature point, in the reference's
    order, P_e += outer(N_i, load).flatten() * det J_i * t * w_i, with N at the library point
    (computeNOperator, `_elementcomputationmatrices.py:106-212`) and J as computeJacobian forms it
    (including the Hexa20 fit)."""
    lib = library.get(elType)
    dim = lib["nSpatialDimensions"]
    X = np.asarray(X, float)
    E = X.shape[0]
    N = shapes.shape_table(lib)  # [q, nN]
    _, detJ, _ = _geometry(lib, X)
    t = np.ones(E) if dim == 3 else np.asarray(thickness, float)
    load = np.asarray(load, float)[:dim]
    P = np.zeros((E, lib["nNodes"] * dim))
    for i in range(lib["nInt"]):
        P += ((np.outer(N[i], load).reshape(-1)[None, :] * detJ[:, i][:, None]) * t[:, None]) * lib["w"][i]
    return P


def small_strain_B(G, dim):
    """Small-strain B operator [E, nV, nDof] for one quadrature point (e.g. _B3D8, :679-817).

    Rows 2D: [eps11, eps22, gamma12]; 3D: [eps11, eps22, eps33, gamma12, gamma13, gamma23]
    (the matrix `a` at _elementcomputationmatrices.py:702-711)."""
    E, d, nN = G.shape
    nV = 3 if dim == 2 else 6
    B = np.zeros((E, nV, nN * dim))
    if dim == 2:
        B[:, 0, 0::2] = G[:, 0]
        B[:, 1, 1::2] = G[:, 1]
        B[:, 2, 0::2] = G[:, 1]
        B[:, 2, 1::2] = G[:, 0]
    else:
        B[:, 0, 0::3] = G[:, 0]
        B[:, 1, 1::3] = G[:, 1]
        B[:, 2, 2::3] = G[:, 2]
        B[:, 3, 0::3] = G[:, 1]
        B[:, 3, 1::3] = G[:, 0]
        B[:, 4, 0::3] = G[:, 2]
        B[:, 4, 2::3] = G[:, 0]
        B[:, 5, 1::3] = G[:, 2]
        B[:, 5, 2::3] = G[:, 1]
    return B


def tl_B0(F, G, dim):
    """Total-Lagrangian B0(F) [E, nV, nDof] (_B02D :830-864, _B03D :867-916).

    Rows 3D: [11, 22, 33, 12, 23, 13] of the Green-Lagrange strain (engineering shear)."""
    E, d, nN = G.shape
    if dim == 2:
        B = np.zeros((E, 3, 2 * nN))
        for c in range(2):
            B[:, 0, c::2] = G[:, 0] * F[:, c, 0, None]
            B[:, 1, c::2] = G[:, 1] * F[:, c, 1, None]
            B[:, 2, c::2] = G[:, 0] * F[:, c, 1, None] + G[:, 1] * F[:, c, 0, None]
        return B
    B = np.zeros((E, 6, 3 * nN))
    for c in range(3):
        B[:, 0, c::3] = G[:, 0] * F[:, c, 0, None]
        B[:, 1, c::3] = G[:, 1] * F[:, c, 1, None]
        B[:, 2, c::3] = G[:, 2] * F[:, c, 2, None]
        B[:, 3, c::3] = G[:, 0] * F[:, c, 1, None] + G[:, 1] * F[:, c, 0, None]
        B[:, 4, c::3] = G[:, 1] * F[:, c, 2, None] + G[:, 2] * F[:, c, 1, None]
        B[:, 5, c::3] = G[:, 0] * F[:, c, 2, None] + G[:, 2] * F[:, c, 0, None]
    return B


def _voigt_strain(dim, e):
    """doVoigtStrain (utils/voigtnotation.py:32-50), batched e [E,d,d]."""
    if dim == 2:
        return np.stack([e[:, 0, 0], e[:, 1, 1], e[:, 0, 1] * 2], axis=1)
    return np.stack([e[:, 0, 0], e[:, 1, 1], e[:, 2, 2], e[:, 0, 1] * 2, e[:, 1, 2] * 2, e[:, 0, 2] * 2], axis=1)


def _unvoigt_stress(dim, s):
    """undoVoigtStress (utils/voigtnotation.py:95-113), batched s [E,>=3]."""
    if dim == 2:
        return np.stack([np.stack([s[:, 0], s[:, 2]], 1), np.stack([s[:, 2], s[:, 1]], 1)], 1)
    return np.stack(
        [
            np.stack([s[:, 0], s[:, 3], s[:, 5]], 1),
            np.stack([s[:, 3], s[:, 1], s[:, 4]], 1),
            np.stack([s[:, 5], s[:, 4], s[:, 2]], 1),
        ],
        1,
    )


def _hypo_update(kind, plane_stress, props, stress, dstrain, kappa):
    """Dispatch of the hypoelastic material call (element.py:327-332; TL element.py:418-421)."""
    if kind == "linearelastic":
        if plane_stress:
            s, C, dstrain, fail = materials.linear_elastic_plane_stress(props, stress, dstrain)
        else:
            s, C, fail = materials.linear_elastic_3d(props, stress, dstrain)
        return s, C, dstrain, kappa, fail
    if kind == "vonmises":
        if plane_stress:
            return materials.von_mises_plane_stress(props, stress, dstrain, kappa)
        s, C, k, fail = materials.von_mises_3d(props, stress, dstrain, kappa)
        return s, C, dstrain, k, fail
    raise ValueError(f"material {kind!r} is not hypoelastic")


def compute_small_strain(elType, kind, props, X, dU, stateRef, thickness):
    """DisplacementElement.computeYourself (element.py:290-346) for E elements at once.

    elType: library name; kind: material kind; props [E, nP]; X [E, nN, d];
    dU [E, nDof]; stateRef [E, nQ, S]; thickness [E].
    Returns (Ke [E,nDof,nDof] row-major as the element fills it, Pe [E,nDof],
    stateTemp [E,nQ,S], fail [E])."""
    lib = library.get(elType)
    if lib["elClass"] != "DisplacementElement":
        raise ValueError(elType)
    if kind in materials.HYPERELASTIC:
        # element.py:333-334
        raise ValueError("Please use the nonlinear element (displacementtlelement) for hyperelastic materials.")
    dim = lib["nSpatialDimensions"]
    nDof = lib["nDof"]
    E = X.shape[0]
    plane_stress = dim == 2 and not lib["plStrain"]
    t = np.ones(E) if dim == 3 else np.asarray(thickness, float)
    idx = lib["index"]
    # C is taken from a 6x6 tangent for plane strain (element.py:217-219), 3x3 for plane stress
    cidx = np.array([0, 1, 3]) if (dim == 2 and not plane_stress) else np.arange(3 if dim == 2 else 6)
    J, detJ, G = _geometry(lib, X)
    K = np.zeros((E, nDof, nDof))
    P = np.zeros((E, nDof))
    stateTemp = stateRef.copy()  # :320
    fail = np.zeros(E, bool)
    w = lib["w"]
    for i in range(lib["nInt"]):
        B = small_strain_B(G[:, i], dim)
        dstrain = np.zeros((E, 6))
        dstrain[:, idx] = np.einsum("evk,ek->ev", B, dU)  # :322
        stress = stateTemp[:, i, 0:6]
        kappa = stateTemp[:, i, 12] if kind == "vonmises" else np.zeros(E)
        stress, Cfull, dstrain, kappa, f = _hypo_update(kind, plane_stress, props, stress, dstrain, kappa)
        fail |= f
        stateTemp[:, i, 0:6] = stress
        if kind == "vonmises":
            stateTemp[:, i, 12] = kappa
        C = Cfull[:, cidx][:, :, cidx]  # :336
        scale = detJ[:, i] * t * w[i]
        K += np.einsum("evk,evu,eul->ekl", B, C, B) * scale[:, None, None]  # :342
        P -= np.einsum("evk,ev->ek", B, stress[:, idx]) * (detJ[:, i] * w[i] * t)[:, None]  # :344
        stateTemp[:, i, 6:12] += dstrain  # :346
    return K, P, stateTemp, fail


def compute_total_lagrangian(elType, kind, props, X, U, stateRef, Eold, thickness):
    """DisplacementTLElement.computeYourself (displacementtlelement/element.py:346-427), batched.

    U is the TOTAL displacement (element.py:379).  Eold [E, nQ, d, d] is the Green-Lagrange
    strain of the last accepted state (used by hypoelastic materials only).
    Returns (Ke, Pe, stateTemp, Enew [E,nQ,d,d], fail)."""
    lib = library.get(elType)
    if lib["elClass"] != "DisplacementTLElement":
        raise ValueError(elType)
    dim = lib["nSpatialDimensions"]
    nDof = lib["nDof"]
    nN = lib["nNodes"]
    E = X.shape[0]
    plane_stress = dim == 2 and not lib["plStrain"]
    hyper = kind in materials.HYPERELASTIC
    if hyper and plane_stress:
        # basehyperelasticmaterial.py:72-95
        raise NotImplementedError("Plane stress for hyperelastic materials is currently not possible.")
    t = np.ones(E) if dim == 3 else np.asarray(thickness, float)
    idx = lib["index"]
    mvi = np.array([0, 1, 3]) if (dim == 2 and not plane_stress) else np.arange(3 if dim == 2 else 6)  # :278-281
    J, detJ, G = _geometry(lib, X)
    Ua = U.reshape(E, nN, dim)
    K = np.zeros((E, nDof, nDof))
    P = np.zeros((E, nDof))
    stateTemp = stateRef.copy()
    Enew = np.zeros((E, lib["nInt"], dim, dim))
    fail = np.zeros(E, bool)
    w = lib["w"]
    I = np.eye(dim)  # noqa: E741
    for i in range(lib["nInt"]):
        Gi = G[:, i]  # [E,d,nN]
        F = I + np.einsum("eaj,eka->ejk", Ua, Gi)  # computeDeformationGradient :70-106
        H = F - I
        Egl = 1 / 2 * (H + H.transpose(0, 2, 1) + H.transpose(0, 2, 1) @ H)  # :386
        Enew[:, i] = Egl
        invF = np.linalg.inv(F)
        scale = detJ[:, i] * t * w[i]
        if hyper:
            NAi = np.zeros((E, nN, 3))
            nab = np.zeros((E, 3, nN))
            NAi[:, :, :dim] = Gi.transpose(0, 2, 1) @ invF  # :391
            nab[:, :dim] = Gi
            strain = np.zeros((E, 6))
            strain[:, idx] = _voigt_strain(dim, Egl)  # :393
            F3 = np.zeros((E, 3, 3))
            F3[:, :dim, :dim] = F
            invF3 = np.zeros((E, 3, 3))
            invF3[:, :dim, :dim] = invF
            if dim == 2:
                F3[:, 2, 2] = 1
                invF3[:, 2, 2] = 1
            tau, D, energy = materials.neo_hooke(kind, props, F3)  # :398-400
            stateTemp[:, i, 0:6] = tau
            stateTemp[:, i, 12] = energy
            T = _unvoigt_stress(3, tau)
            PK1 = invF3 @ T  # :402
            stateTemp[:, i, 6:12] = strain  # :404
            Hk4 = np.einsum("eai,eijkl,ebl->eajbk", NAi, D, nab.transpose(0, 2, 1)) - np.einsum(
                "eak,ebi,eij->eajbk", NAi, NAi, T
            )  # :405-411
            Hk = Hk4[:, :, :dim, :, :dim].reshape(E, nDof, nDof)  # makeH2D :284-306
            P -= (Gi.transpose(0, 2, 1) @ PK1[:, :dim, :dim]).reshape(E, nDof) * scale[:, None]  # :414
        else:
            B = tl_B0(F, Gi, dim)
            dstrain = np.zeros((E, 6))
            dstrain[:, idx] = _voigt_strain(dim, Egl - Eold[:, i])  # :416
            stress = stateTemp[:, i, 0:6]
            kappa = stateTemp[:, i, 12] if kind == "vonmises" else np.zeros(E)
            stress, Cfull, dstrain, kappa, f = _hypo_update(kind, plane_stress, props, stress, dstrain, kappa)
            fail |= f
            stateTemp[:, i, 0:6] = stress
            if kind == "vonmises":
                stateTemp[:, i, 12] = kappa
            stateTemp[:, i, 6:12] += dstrain  # :422
            Cm = Cfull[:, mvi][:, :, mvi]  # :423
            # Hgeo (element.py:48-73); for 2D undoVoigtStress(2, .) reads stress[0], stress[1], stress[2]
            S = _unvoigt_stress(dim, stress)
            Hsub = Gi.transpose(0, 2, 1) @ S @ Gi  # [E,nN,nN]
            Hg = np.einsum("eab,ij->eaibj", Hsub, I).reshape(E, nDof, nDof)
            Hk = np.einsum("evk,evu,eul->ekl", B, Cm, B) + Hg  # :424
            P -= np.einsum("evk,ev->ek", B, stress[:, mvi]) * (detJ[:, i] * w[i] * t)[:, None]  # :426
        K += Hk * scale[:, None, None]  # :427
    return K, P, stateTemp, Enew, fail
