"""Material point updates, vectorised over material points.

Restates the reference's "edelweiss" materials:

* LinearElasticMaterial  `edelweissfe/materials/linearelastic/linearelastic.py:34-250`
* VonMisesMaterial       `edelweissfe/materials/vonmises/vonmises.py:67-299`
* plane stress for hypoelastic materials
                         `edelweissfe/materials/base/basehypoelasticmaterial.py:71-130`
* Neo-Hooke (Pence-Gou formulations a, b, c)
                         `edelweissfe/materials/neohooke/neohookepencegouformulation{a,b,c}.py`

Every function works on arrays with a leading "points" axis P.  The per-point
arithmetic follows the reference's operation order; iterations that the
reference runs per point (von Mises return map, plane-stress Newton) are run
with per-point activity masks, so each point performs exactly the iteration
sequence the reference would.

Each returns, besides its results, a boolean ``fail`` array marking points for
which the reference raises ``CutbackRequest(..., 0.5)``.
"""

import numpy as np

# vonmises.py:35-56
IDEV = np.array(
    [
        [2 / 3, -1 / 3, -1 / 3, 0, 0, 0],
        [-1 / 3, 2 / 3, -1 / 3, 0, 0, 0],
        [-1 / 3, -1 / 3, 2 / 3, 0, 0, 0],
        [0, 0, 0, 1, 0, 0],
        [0, 0, 0, 0, 1, 0],
        [0, 0, 0, 0, 0, 1],
    ]
)
IDEV_HALF_SHEAR = np.array(
    [
        [2 / 3, -1 / 3, -1 / 3, 0, 0, 0],
        [-1 / 3, 2 / 3, -1 / 3, 0, 0, 0],
        [-1 / 3, -1 / 3, 2 / 3, 0, 0, 0],
        [0, 0, 0, 0.5, 0, 0],
        [0, 0, 0, 0, 0.5, 0],
        [0, 0, 0, 0, 0, 0.5],
    ]
)
VM_MAX_ITER = 15  # vonmises.py:55
VM_TOL = 1e-12  # vonmises.py:56

# material kinds and the number of material state variables per point
STATE_VARS = {"linearelastic": 0, "vonmises": 1, "neohookewa": 1, "neohookewb": 1, "neohookewc": 1}
HYPERELASTIC = ("neohookewa", "neohookewb", "neohookewc")


def elasticity_3d(E, v):
    """3D isotropic elasticity matrix [P,6,6] (linearelastic.py:95-117, vonmises.py:126-149)."""
    E = np.asarray(E, float)[:, None, None]
    v = np.asarray(v, float)[:, None, None]
    z = np.zeros_like(v)
    o = np.ones_like(v)
    g = (1 - 2 * v) / 2
    m = np.concatenate(
        [
            np.concatenate([1 - v, v, v, z, z, z], axis=2),
            np.concatenate([v, 1 - v, v, z, z, z], axis=2),
            np.concatenate([v, v, 1 - v, z, z, z], axis=2),
            np.concatenate([z, z, z, g, z, z], axis=2),
            np.concatenate([z, z, z, z, g, z], axis=2),
            np.concatenate([z, z, z, z, z, g], axis=2),
        ],
        axis=1,
    )
    del o
    return E / ((1 + v) * (1 - 2 * v)) * m


def elasticity_plane_stress(E, v):
    """Plane-stress elasticity [P,3,3] in [11,22,12] order (linearelastic.py:63-72)."""
    E = np.asarray(E, float)[:, None, None]
    v = np.asarray(v, float)[:, None, None]
    z = np.zeros_like(v)
    o = np.ones_like(v)
    m = np.concatenate(
        [
            np.concatenate([o, v, z], axis=2),
            np.concatenate([v, o, z], axis=2),
            np.concatenate([z, z, (1 - v) / 2], axis=2),
        ],
        axis=1,
    )
    return E / (1 - v**2) * m


# ---------------------------------------------------------------- linear elastic
def linear_elastic_3d(props, stress, dstrain):
    """LinearElasticMaterial.computeStress (linearelastic.py:185-210): stress += C @ dStrain."""
    C = elasticity_3d(props[:, 0], props[:, 1])
    stress = stress + np.einsum("pij,pj->pi", C, dstrain)
    return stress, C, np.zeros(len(stress), bool)


def linear_elastic_plane_stress(props, stress, dstrain):
    """LinearElasticMaterial.computePlaneStress (linearelastic.py:127-154).

    Returns (stress, C[P,3,3], dstrain with eps33 overwritten, fail)."""
    C = elasticity_plane_stress(props[:, 0], props[:, 1])
    idx = [0, 1, 3]
    stress = stress.copy()
    stress[:, idx] += np.einsum("pij,pj->pi", C, dstrain[:, idx])
    dstrain = dstrain.copy()
    v = props[:, 1]
    dstrain[:, 2] = -v / (1 - v) * (dstrain[:, 0] + dstrain[:, 1])
    return stress, C, dstrain, np.zeros(len(stress), bool)


# ---------------------------------------------------------------- von Mises
def _fy(props, k):
    """Hardening law fy(kappa) (vonmises.py:113-117)."""
    return props[:, 2] + props[:, 3] * k + props[:, 4] * (1.0 - np.exp(-props[:, 5] * k))


def _dfy(props, k):
    """d fy / d kappa (vonmises.py:121)."""
    return props[:, 3] + props[:, 4] * props[:, 5] * np.exp(-props[:, 5] * k)


def von_mises_3d(props, stress, dstrain, kappa):
    """VonMisesMaterial.computeStress (vonmises.py:186-254), vectorised.

    props [P,6] = (E, nu, fy0, HLin, dfy, delta); stress [P,6]; dstrain [P,6]; kappa [P].
    Returns (stress, C[P,6,6], kappa, fail)."""
    P = len(stress)
    Ei = elasticity_3d(props[:, 0], props[:, 1])
    G = props[:, 0] / (2 * (1.0 + props[:, 1]))
    stress = stress.copy()
    kappa = kappa.copy()
    C = Ei.copy()
    fail = np.zeros(P, bool)

    zero = np.linalg.norm(dstrain, axis=1) < 10**-14  # :211-213
    live = ~zero
    trial = stress + np.einsum("pj,pji->pi", dstrain, Ei)  # dStrain @ Ei  (:215)
    dev = trial @ IDEV.T  # IDev @ trialStress (:59-60)
    devNorm = np.sqrt(np.sum(np.square(dev[:, 0:3]), axis=1) + 2 * np.sum(np.square(dev[:, 3:6]), axis=1))  # :63-64
    f = devNorm - np.sqrt(2 / 3) * _fy(props, kappa)
    plastic = live & (f > 0.0)
    elastic = live & ~plastic
    stress[elastic] = trial[elastic]

    if plastic.any():
        pp = props[plastic]
        dn = devNorm[plastic]
        k0 = kappa[plastic]
        Gp = G[plastic]
        n = dev[plastic] / dn[:, None]

        def R(dk):
            return dn - np.sqrt(6) * Gp * dk - np.sqrt(2 / 3) * _fy(pp, k0 + dk)

        dK = np.zeros(len(dn))
        counter = 0
        active = np.abs(R(dK)) > VM_TOL
        failp = np.zeros(len(dn), bool)
        while active.any():  # :229-236
            if counter == VM_MAX_ITER:
                failp |= active
                break
            a = active
            dR = -np.sqrt(6) * Gp[a] - np.sqrt(2 / 3) * _dfy(pp[a], k0[a] + dK[a])
            dK[a] -= R(dK)[a] / dR
            counter += 1
            active = active & (np.abs(R(dK)) > VM_TOL)
        dLambda = np.sqrt(3 / 2) * dK
        kNew = k0 + dK
        sNew = trial[plastic] - (2.0 * Gp * dLambda)[:, None] * n
        fac = 1.0 / (1.0 + _dfy(pp, kNew) / (3.0 * Gp)) - 2.0 * Gp * dLambda / dn
        Cp = (
            Ei[plastic]
            - (2.0 * Gp * fac)[:, None, None] * np.einsum("pi,pj->pij", n, n)
            - (4.0 * Gp**2 * dLambda / dn)[:, None, None] * IDEV_HALF_SHEAR[None]
        )
        kappa[plastic] = kNew
        stress[plastic] = sNew
        C[plastic] = Cp
        fail[plastic] = failp
    return stress, C, kappa, fail


def von_mises_plane_stress(props, stress, dstrain, kappa):
    """BaseHypoElasticMaterial.computePlaneStress (basehypoelasticmaterial.py:71-130) on von Mises.

    Faithful to the reference: each local Newton step calls the 3D update with a
    zero stress vector (:98-99) and with the material state view, so kappa
    accumulates the plastic increment of every local iteration; the converged
    3D stress is then added to the incoming stress (:111).
    Returns (stress, C[P,3,3], dstrain, kappa, fail)."""
    P = len(stress)
    dstrain = dstrain.copy()
    kappa = kappa.copy()
    dstrain[:, 2] = -dstrain[:, 0] - dstrain[:, 1]  # :95
    s3 = np.zeros((P, 6))
    C3 = np.zeros((P, 6, 6))
    fail = np.zeros(P, bool)
    active = np.ones(P, bool)
    counter = 1
    while active.any():
        a = active
        s_a, C_a, k_a, f_a = von_mises_3d(props[a], np.zeros((a.sum(), 6)), dstrain[a], kappa[a])
        s3[a] = s_a
        C3[a] = C_a
        kappa[a] = k_a
        fail[a] |= f_a
        residual = np.abs(s3[:, 2])
        done = (residual < 1e-11) | ((counter > 7) & (residual < 1e-8))
        done |= fail
        active = active & ~done
        if not active.any():
            break
        a = active
        with np.errstate(divide="ignore", invalid="ignore"):
            rev = 1.0 / C3[a, 2, 2]
        bad = np.isnan(rev) | (np.abs(rev) > 1e10)
        rev = np.where(bad, 1e10 * np.sign(rev), rev)
        dstrain[a, 2] -= rev * s3[a, 2]
        counter += 1
        if counter > 13:
            fail |= active
            break
    stress = stress + s3  # :111
    C = C3
    Cc = np.empty((P, 3, 3))
    rows = [0, 1, 3]
    for r, i in enumerate(rows):  # :113-130
        for c, j in enumerate(rows):
            Cc[:, r, c] = C[:, i, j] - C[:, 2, j] * C[:, i, 2] / C[:, 2, 2]
    return stress, Cc, dstrain, kappa, fail


# ---------------------------------------------------------------- Neo-Hooke
def _voigt_stress_3d(T):
    """doVoigtStress(3, .) (utils/voigtnotation.py:74-92): [11,22,33,12,23,13]."""
    return np.stack([T[:, 0, 0], T[:, 1, 1], T[:, 2, 2], T[:, 0, 1], T[:, 1, 2], T[:, 0, 2]], axis=1)


def neo_hooke(kind, props, F):
    """Kirchhoff stress, d tau / dF and energy for the Pence-Gou Neo-Hooke variants.

    kind 'neohookewa' follows neohookepencegouformulationa.py:107-141,
    'neohookewb' neohookepencegouformulationb.py:107-145,
    'neohookewc' neohookepencegouformulationc.py:107-143 (including its use of
    trace(F) as I1 in the energy).  props [P,2] = (mu, K); F [P,3,3].
    Returns (tau voigt [P,6], dtau_dF [P,3,3,3,3], energy [P])."""
    mu = props[:, 0]
    K = props[:, 1]
    I3 = np.eye(3)
    invF = np.linalg.inv(F)
    B = F @ F.transpose(0, 2, 1)
    J = np.linalg.det(F)
    d_ik_Fjl = np.einsum("ik,pjl->pijkl", I3, F)
    Fil_d_jk = np.einsum("pil,jk->pijkl", F, I3)
    d_ij_invFlk = np.einsum("ij,plk->pijkl", I3, invF)
    if kind == "neohookewa":
        I1 = np.trace(B, axis1=1, axis2=2)
        lambdaBar = (K - 2 / 3 * mu) * (J**2 - J) - mu
        muBar = (K - 2 / 3 * mu) * (2 * J**2 - J)
        tau = mu[:, None, None] * B + lambdaBar[:, None, None] * I3
        D = mu[:, None, None, None, None] * (d_ik_Fjl + Fil_d_jk) + muBar[:, None, None, None, None] * d_ij_invFlk
        energy = mu / 2 * (I1 - 3) + (K / 2 - mu / 3) * (J - 1) ** 2 - mu * np.log(J)
    elif kind == "neohookewb":
        I1 = np.trace(B, axis1=1, axis2=2)
        lambdaHat = K / 2 * (J**2 + 1 / J**2)
        muBar = mu / (3 * J ** (2 / 3))
        lambdaBar = K / 4 * (J**2 - 1 / J**2) - muBar * I1
        tau = (mu / J ** (2 / 3))[:, None, None] * B + lambdaBar[:, None, None] * I3
        x = lambda a: a[:, None, None, None, None]  # noqa: E731
        D = (
            x(3 * muBar) * (d_ik_Fjl + Fil_d_jk)
            - x(2 * muBar) * np.einsum("pij,plk->pijkl", B, invF)
            + x(lambdaHat + 2 / 3 * I1 * muBar) * d_ij_invFlk
            - x(2 * muBar) * np.einsum("ij,pkl->pijkl", I3, F)
        )
        energy = mu / 2 * (I1 / J ** (2 / 3) - 3) + K / 8 * (J**2 + 1 / J**2 - 2)
    elif kind == "neohookewc":
        I1 = np.trace(F, axis1=1, axis2=2)
        muBar = mu * J ** (2 / 3 - K / mu)
        lambdaBar = (K / mu - 2 / 3) * muBar
        tau = mu[:, None, None] * B - muBar[:, None, None] * I3
        D = mu[:, None, None, None, None] * (d_ik_Fjl + Fil_d_jk) + lambdaBar[:, None, None, None, None] * d_ij_invFlk
        energy = mu / 2 * (I1 - 3) + 3 * mu**2 / (3 * K - 2 * mu) * (J ** (2 / 3 - K / mu) - 1)
    else:
        raise KeyError(kind)
    return _voigt_stress_3d(tau), D, energy
