// efe_adjoint_ss.cuh -- reverse mode of one small-strain element pass (linear elastic, von Mises).
//
// Forward, per quadrature point (displacementelement/element.py:318-346, vonmises.py:186-254):
//   de = B dU_e,  (sig, kappa) = update(sig0, kappa0, de; props),  eps = eps0 + de,
//   P_e -= s B^T sig   (s = det J w t).
// Given adjoint seeds of the outputs -- sigBar, epsBar, kappaBar of the new state and PBar of the
// element residual -- the kernel accumulates the adjoints of the inputs: dUBar (DOF vector),
// sig0Bar, eps0Bar, kappa0Bar (state before the increment) and the material properties
// (E, nu, fy0, H, dfy, delta).  The return map is differentiated through its converged scalar
// equation R(dK) = q - sqrt(6) G dK - sqrt(2/3) fy(kappa0 + dK) = 0 (implicit function theorem),
// so the derivatives are those of the exact return map, consistent with the reference's
// consistent tangent (vonmises.py:241-251).
//
// With gX, also the adjoint of the nodal coordinates: per point, G = dN/dX enters de = B dU and
// the residual, s = det J w t the residual; Gbar_a = sym(deBar) u_a - s sigma PBar_a and
// sBar = -sigma : (B PBar), and through G = J^-1 D (D = J G, J = D' X with the Hexa20 quirk row in
// D'): Xbar_a = -M^T G_a + s sBar G_a (+ the quirk row's term), M = sum_a Gbar_a (x) G_a.
//
// Plane stress (2D): the reverse of the reference's local Newton on eps33, iteration by iteration.
//
// Tile: EPB elements per CTA.  Phase 0 gathers dU_e and PBar_e, stages the tile's dN/dX rows in
// shared memory (cp.async) and forms the elements' constants once; phase A runs one thread per
// point (B dU, B PBar, the reverse update, the point's strain adjoint); phase C forms B^T deBar per
// element DOF over the points (one atomic per element DOF) and sums the property adjoints (plain
// stores: one thread owns an element's property).
#pragma once
#include "efe_launch.cuh"

namespace efe {

// Per-element constants of the reverse pass: the forward update's (VMConst) and the reciprocals and
// derivatives the property adjoints need, formed once per element (the pass is FP64-bound, and an
// FP64 division costs several FP64 instructions).
struct SSRevConst {
  VMConst c;
  double E, nu;
  double rE, r1nu;  // 1 / E, 1 / (1 + nu)
  double f, df;     // f = E / ((1 + nu)(1 - 2 nu)) and df/dnu = E (1 + 4 nu) / ((1 + nu)(1 - 2 nu))^2
  double rDR;       // 1 / (sqrt(6) G + sqrt(2/3) H): minus the return map's Newton factor (linear hardening)
  double r3G;       // 1 / (3 G)
};
__device__ inline SSRevConst ss_rev_const(const double* props, bool vonMises) {
  SSRevConst r;
  r.c = vm_const(props, vonMises);
  r.E = props[0];
  r.nu = props[1];
  r.rE = 1.0 / r.E;
  r.r1nu = 1.0 / (1.0 + r.nu);
  const double rden = 1.0 / ((1.0 + r.nu) * (1.0 - 2.0 * r.nu));
  r.f = r.E * rden;
  r.df = r.E * (1.0 + 4.0 * r.nu) * rden * rden;
  r.rDR = -r.c.invdR;
  r.r3G = 1.0 / (3.0 * r.c.G);
  return r;
}

// Adjoint of the hypoelastic 3D update.  Accumulates into sig0Bar, k0Bar, deBar, pBar[6].  c22Bar:
// adjoint of the tangent's entry C_33,33 (the plane-stress Newton divides by it), 0 otherwise.
// Divisions are taken as products with reciprocals (per point: 1 / |dev|; per element: SSRevConst),
// which changes the recomputed state only by rounding.
__device__ inline void hypo3d_reverse(const SSRevConst& rc, bool vonMises, const double sig0[6], double k0,
                                      const double de[6], const double sBar[6], double kBar, double sig0Bar[6],
                                      double& k0Bar, double deBar[6], double pBar[6], double c22Bar = 0.0) {
  const VMConst& c = rc.c;
  const Iso& Ei = c.Ei;
  const double G = c.G;
  double trBar[6];
  for (int i = 0; i < 6; ++i) trBar[i] = sBar[i];
  double Gbar = 0.0;
  k0Bar += kBar;  // kappa = kappa0 (+ dK)
  double nrm = 0.0;
  for (int i = 0; i < 6; ++i) nrm += de[i] * de[i];
  if (vonMises && !(nrm < 1e-28)) {
    double tr[6], ds[6];
    iso_apply(Ei, de, ds);
    for (int i = 0; i < 6; ++i) tr[i] = sig0[i] + ds[i];
    double dev[6];
    const double mean = (tr[0] + tr[1] + tr[2]) * (1.0 / 3.0);
    dev[0] = tr[0] - mean;
    dev[1] = tr[1] - mean;
    dev[2] = tr[2] - mean;
    dev[3] = tr[3];
    dev[4] = tr[4];
    dev[5] = tr[5];
    // |dev| and 1 / |dev| from one reciprocal square root (as the forward pass with an FP32 tangent)
    double q, iq;
    vm_dev_norm(dev, q, iq);
    const double sq23 = sqrt(2.0 / 3.0), sq6 = sqrt(6.0);
    const double fy_k0 = c.fy0 + c.H * k0 + vm_sat(c, k0);
    if (q - sq23 * fy_k0 > 0.0) {
      // the scalar Newton of the forward return map (converged dK; with linear hardening its factor
      // is the per-element constant, as in the forward pass with an FP32 tangent)
      const bool lin = c.dfy == 0.0;
      double dK = 0.0;
      for (int counter = 0;; ++counter) {
        const double k = k0 + dK;
        const double R = q - sq6 * G * dK - sq23 * (c.fy0 + c.H * k + vm_sat(c, k));
        if (!(fabs(R) > 1e-12) || counter == 15) break;
        if (lin)
          dK += R * rc.rDR;
        else
          dK -= R / (-sq6 * G - sq23 * (c.H + vm_dsat(c, k)));
      }
      const double k = k0 + dK;
      const double g2 = 2.0 * G * (sqrt(1.5) * dK);  // sig = tr - g2 n, n = dev / q
      double g2Bar = 0.0, nd = 0.0, devBar[6];
      for (int i = 0; i < 6; ++i) g2Bar -= sBar[i] * (dev[i] * iq);
      for (int i = 0; i < 6; ++i) {
        const double nBar = -g2 * sBar[i];
        devBar[i] = nBar * iq;
        nd += nBar * dev[i];
      }
      double qBar = -nd * iq * iq;
      double kTBar = 0.0;  // adjoint of the final kappa through the tangent
      if (c22Bar != 0.0) {
        // C22 = Ei.c11 - 2/3 beta - a n2^2, beta = 2G g2 / q, a = 2G (tfac - g2 / q), n2 = dev2 / q,
        // tfac = 1 / (1 + z), z = (H + dsat(kappa)) / 3G  (vonmises.py:241-251); the Ei.c11 term is
        // taken with the trial's elasticity below
        const double n2 = dev[2] * iq;
        const double z = (c.H + vm_dsat(c, k)) * rc.r3G, tfac = lin ? c.tfac : 1.0 / (1.0 + z);
        const double aT = 2.0 * G * (tfac - g2 * iq);
        const double betaBar = -(2.0 / 3.0) * c22Bar, aBar = -c22Bar * n2 * n2, n2Bar = -c22Bar * 2.0 * aT * n2;
        Gbar += aBar * 2.0 * (tfac - g2 * iq) + betaBar * 2.0 * g2 * iq;
        g2Bar += (betaBar - aBar) * 2.0 * G * iq;
        const double invBar = (betaBar - aBar) * 2.0 * G * g2 + n2Bar * dev[2];
        devBar[2] += n2Bar * iq;
        qBar -= invBar * iq * iq;
        const double zBar = -tfac * tfac * aBar * 2.0 * G;
        Gbar -= zBar * z * 3.0 * rc.r3G;  // dz/dG = -z / G
        pBar[3] += zBar * rc.r3G;
        // dsat(kappa) = dfy delta exp(-delta kappa)
        const double dsBar = zBar * rc.r3G, ek = exp(-c.delta * k);
        pBar[4] += dsBar * c.delta * ek;
        pBar[5] += dsBar * c.dfy * ek * (1.0 - c.delta * k);
        kTBar = -dsBar * c.dfy * c.delta * c.delta * ek;
      }
      k0Bar += kTBar;
      const double dKBar = kBar + kTBar + g2Bar * 2.0 * G * sqrt(1.5);
      Gbar += g2Bar * 2.0 * sqrt(1.5) * dK;
      // dK(q, kappa0, G, fy0, H, dfy, delta) from R = 0: x_bar += dK_bar * (dR/dx) / D
      const double dfyk = c.H + vm_dsat(c, k);
      const double w = lin ? dKBar * rc.rDR : dKBar / (sq6 * G + sq23 * dfyk);
      qBar += w;
      k0Bar += -sq23 * dfyk * w;
      Gbar += -sq6 * dK * w;
      pBar[2] += -sq23 * w;
      pBar[3] += -sq23 * k * w;
      {
        // sat = dfy (1 - exp(-delta kappa)) is linear in dfy: its derivative holds at dfy = 0 too
        const double ek = c.delta == 0.0 ? 1.0 : exp(-c.delta * k);
        pBar[4] += -sq23 * (1.0 - ek) * w;
        pBar[5] += -sq23 * c.dfy * k * ek * w;
      }
      // q = |dev| with doubled shear terms, dev = deviatoric part of tr
      const double qi = qBar * iq;
      for (int i = 0; i < 6; ++i) devBar[i] += qi * (i < 3 ? 1.0 : 2.0) * dev[i];
      const double mb = (devBar[0] + devBar[1] + devBar[2]) * (1.0 / 3.0);
      for (int i = 0; i < 6; ++i) trBar[i] += devBar[i] - (i < 3 ? mb : 0.0);
    }
  }
  // trial stress tr = sig0 + Ei de (the elastic branch and the zero-increment shortcut included)
  double dd[6];
  iso_apply(Ei, trBar, dd);
  for (int i = 0; i < 6; ++i) {
    sig0Bar[i] += trBar[i];
    deBar[i] += dd[i];
  }
  // properties through C11, C12, C44 and G
  const double c11Bar = trBar[0] * de[0] + trBar[1] * de[1] + trBar[2] * de[2] + c22Bar;
  const double c12Bar = trBar[0] * (de[1] + de[2]) + trBar[1] * (de[0] + de[2]) + trBar[2] * (de[0] + de[1]);
  const double c44Bar = trBar[3] * de[3] + trBar[4] * de[4] + trBar[5] * de[5];
  const double nu = rc.nu, f = rc.f, df = rc.df;
  pBar[0] += (c11Bar * Ei.c11 + c12Bar * Ei.c12 + c44Bar * Ei.c44 + Gbar * G) * rc.rE;
  pBar[1] += c11Bar * (df * (1.0 - nu) - f) + c12Bar * (df * nu + f) + c44Bar * (df * (1.0 - 2.0 * nu) / 2.0 - f) -
             Gbar * G * rc.r1nu;
}

// Adjoint of the plane-stress von Mises update (von_mises_plane_stress; basehypoelasticmaterial.py:71-130).
// Forward: d_1 = -de0 - de1; iteration i evaluates the 3D update from a zero stress with the kappa the
// previous iteration left, s3_i, kappa_i = VM3D(0, kappa_{i-1}, de(d_i)), and steps
// d_{i+1} = d_i - rev_i s3_i[2], rev_i = 1 / C22_i (clamped to +-1e10), until |s3_n[2]| is small;
// sig = sig0 + s3_n, kappa = kappa_n, eps33 += d_n.  Because kappa carries over between the local
// iterations, the result depends on the iterates, so the reverse sweep runs through every iteration
// (with the derivative of rev_i) rather than through the converged equation alone.  e2Bar: adjoint of
// the strain increment d_n stored in eps33.
__device__ inline void von_mises_plane_stress_reverse(const SSRevConst& rc, const double sig0[6], double k0,
                                                      const double de[6], const double sBar[6], double kBar,
                                                      double e2Bar, double sig0Bar[6], double& k0Bar, double deBar[6],
                                                      double pBar[6]) {
  constexpr int MAXIT = 13;
  double D2[MAXIT], K0[MAXIT], R2[MAXIT], RV[MAXIT];
  double dd[6];
  for (int f = 0; f < 6; ++f) dd[f] = de[f];
  dd[2] = -de[0] - de[1];
  double kap = k0;
  int n = 0;                // index of the last evaluated iteration
  uint32_t clampMask = 0;   // bit i: step i's rev was clamped (no derivative through it)
  for (int counter = 1;; ++counter) {
    D2[n] = dd[2];
    K0[n] = kap;
    double s3[6] = {0, 0, 0, 0, 0, 0};
    Tangent3 T;
    if (!von_mises_3d<false>(rc.c, s3, dd, kap, T)) break;
    const double residual = fabs(s3[2]);
    if (residual < 1e-11 || (counter > 7 && residual < 1e-8) || counter == MAXIT) break;
    double rev = 1.0 / tangent3_entry(T, 2, 2);
    if (isnan(rev) || fabs(rev) > 1e10) {
      rev = 1e10 * (rev > 0 ? 1.0 : (rev < 0 ? -1.0 : rev));
      clampMask |= 1u << n;
    }
    RV[n] = rev;
    R2[n] = s3[2];
    dd[2] -= rev * s3[2];
    ++n;
  }
  for (int f = 0; f < 6; ++f) sig0Bar[f] += sBar[f];  // sig = sig0 + s3_n
  const double zero[6] = {0, 0, 0, 0, 0, 0};
  double scratch[6] = {0, 0, 0, 0, 0, 0};
  double inBar[6] = {0, 0, 0, 0, 0, 0};  // adjoints of the in-plane increments over all iterations
  double dBar = e2Bar, kCarry = 0.0;
  for (int i = n; i >= 0; --i) {
    double sSeed[6] = {0, 0, 0, 0, 0, 0}, kSeed, c22Bar = 0.0;
    if (i == n) {
      for (int f = 0; f < 6; ++f) sSeed[f] = sBar[f];
      kSeed = kBar;
    } else {
      // d_{i+1} = d_i - rev_i r_i: dBar carries to d_i unchanged
      const double rev = RV[i];
      sSeed[2] = -rev * dBar;
      if (!(clampMask >> i & 1u)) c22Bar = rev * rev * R2[i] * dBar;  // revBar = -r_i dBar, rev = 1 / C22
      kSeed = kCarry;
    }
    double ddi[6], ddBar[6] = {0, 0, 0, 0, 0, 0}, kinBar = 0.0;
    for (int f = 0; f < 6; ++f) ddi[f] = de[f];
    ddi[2] = D2[i];
    hypo3d_reverse(rc, true, zero, K0[i], ddi, sSeed, kSeed, scratch, kinBar, ddBar, pBar, c22Bar);
    dBar += ddBar[2];
    for (int f = 0; f < 6; ++f)
      if (f != 2) inBar[f] += ddBar[f];
    kCarry = kinBar;
  }
  k0Bar += kCarry;
  // d_1 = -de0 - de1
  deBar[0] += inBar[0] - dBar;
  deBar[1] += inBar[1] - dBar;
  deBar[3] += inBar[3];
  deBar[4] += inBar[4];
  deBar[5] += inBar[5];
}

// Adjoint of the plane-stress linear-elastic update (linear_elastic_plane_stress; linearelastic.py:127-154):
// sig += C(E, nu) de over 11, 22, 12 and eps33 += -nu / (1 - nu) (de0 + de1).
__device__ inline void linear_elastic_plane_stress_reverse(double E, double nu, const double de[6],
                                                           const double sBar[6], double e2Bar, double sig0Bar[6],
                                                           double deBar[6], double pBar[6]) {
  const double f = E / (1.0 - nu * nu), c11 = f, c12 = f * nu, c33 = f * ((1.0 - nu) / 2.0);
  const double r = nu / (1.0 - nu);
  for (int i = 0; i < 6; ++i) sig0Bar[i] += sBar[i];
  deBar[0] += c11 * sBar[0] + c12 * sBar[1] - r * e2Bar;
  deBar[1] += c12 * sBar[0] + c11 * sBar[1] - r * e2Bar;
  deBar[3] += c33 * sBar[3];
  const double c11Bar = sBar[0] * de[0] + sBar[1] * de[1], c12Bar = sBar[0] * de[1] + sBar[1] * de[0],
               c33Bar = sBar[3] * de[3], rBar = -e2Bar * (de[0] + de[1]);
  const double dfdnu = 2.0 * nu * f / (1.0 - nu * nu);
  pBar[0] += (c11Bar * c11 + c12Bar * c12 + c33Bar * c33) / E;
  pBar[1] += c11Bar * dfdnu + c12Bar * (dfdnu * nu + f) + c33Bar * (dfdnu * (1.0 - nu) / 2.0 - f / 2.0) +
             rBar / ((1.0 - nu) * (1.0 - nu));
}

// Coordinate adjoint of one point (see the head comment), accumulated into a.gX.  u and pb: the
// element's dU and PBar as staged by phase 0 (float-float relative to node 0 in the FF form, which
// leaves M unchanged: sum_a G_a = 0).
template <int SHAPE, int RULE, bool FF>
__device__ __forceinline__ void coordinate_adjoint(const SSAdjointArgs& a, int64_t e, int q, int64_t pt, int64_t stride,
                                                   double s, const VMConst& mc, bool vm, bool planeStress,
                                                   const double sig0[6], double k0, const double de[6],
                                                   const double deBar[6], const double bp[6], const double* u,
                                                   const double* pb) {
  constexpr int DIM = ShapeInfo<SHAPE>::DIM, NN = ShapeInfo<SHAPE>::NN;
  // the new stress (the FP64 form of the forward update)
  double sn[6], kn = k0, dp[6];
  for (int f = 0; f < 6; ++f) {
    sn[f] = sig0[f];
    dp[f] = de[f];
  }
  if (planeStress) {
    Tangent2 C2;
    if (vm)
      von_mises_plane_stress<false>(mc, sn, dp, kn, C2);
    else
      linear_elastic_plane_stress(a.props + e * a.nProps, sn, dp, C2);
  } else {
    Tangent3 Tt;
    if (vm)
      von_mises_3d<false>(mc, sn, de, kn, Tt);
    else
      linear_elastic_3d(mc, sn, de, Tt);
  }
  // Voigt 11, 22, 33, 12, 13, 23 (engineering shears in de, bp) as symmetric matrices
  const double S[3][3] = {{sn[0], sn[3], sn[4]}, {sn[3], sn[1], sn[5]}, {sn[4], sn[5], sn[2]}};
  const double Db[3][3] = {{deBar[0], deBar[3], deBar[4]}, {deBar[3], deBar[1], deBar[5]},
                           {deBar[4], deBar[5], deBar[2]}};
  double sBar = 0.0;
  if constexpr (DIM == 3) {
    for (int f = 0; f < 6; ++f) sBar -= sn[f] * bp[f];
  } else {
    sBar = -(sn[0] * bp[0] + sn[1] * bp[1] + sn[3] * bp[3]);
  }
  auto val = [&](const double* arr, int k) {
    if constexpr (FF)
      return ff_to_double(reinterpret_cast<const ff*>(arr)[k]);
    else
      return arr[k];
  };
  double M[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int n = 0; n < NN; ++n) {
    double G[3], ua[3], pa[3], Gb[3];
    for (int c = 0; c < DIM; ++c) {
      G[c] = a.geomG[(int64_t)(c * NN + n) * stride + pt];
      ua[c] = val(u, n * DIM + c);
      pa[c] = val(pb, n * DIM + c);
    }
    for (int k = 0; k < DIM; ++k) {
      double v = 0.0;
      for (int l = 0; l < DIM; ++l) v += Db[k][l] * ua[l] - s * S[k][l] * pa[l];
      Gb[k] = v;
    }
    for (int k = 0; k < DIM; ++k)
      for (int c = 0; c < DIM; ++c) M[k][c] += Gb[k] * G[c];
  }
  // the Hexa20 quirk row of J (J[2][c] += (zeta - xi) sum_a r_a X_a[c]): Jbar[2][c] feeds it
  double Jb2[3] = {0, 0, 0}, qk = 0.0;
  if constexpr (SHAPE == EFE_HEXA20) {
    double xi, eta, zeta, w;
    quadrature_point(RULE, q, xi, eta, zeta, w);
    qk = zeta - xi;
    const double p[3] = {eta, xi, zeta};
    double D[3][NN];
    shape_derivatives<SHAPE>(p, D);
    double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int n = 0; n < NN; ++n) {
      const int32_t node = a.conn[e * NN + n];
      for (int c = 0; c < 3; ++c) {
        const double x = a.coords[(int64_t)node * 3 + c];
        for (int r = 0; r < 3; ++r) J[r][c] += (D[r][n] + (r == 2 ? qk * a.fix.r[n] : 0.0)) * x;
      }
    }
    double iJ[3][3];
    inv3(J, det3(J), iJ);
    for (int c = 0; c < 3; ++c) {
      double v = s * sBar * iJ[c][2];
      for (int k = 0; k < 3; ++k) v -= iJ[k][2] * M[k][c];
      Jb2[c] = v;
    }
  }
  for (int n = 0; n < NN; ++n) {
    const int32_t node = a.conn[e * NN + n];
    for (int c = 0; c < DIM; ++c) {
      double v = s * sBar * a.geomG[(int64_t)(c * NN + n) * stride + pt];
      for (int k = 0; k < DIM; ++k) v -= M[k][c] * a.geomG[(int64_t)(k * NN + n) * stride + pt];
      if constexpr (SHAPE == EFE_HEXA20) v += qk * a.fix.r[n] * Jb2[c];
      atomicAdd(a.gX + (int64_t)node * DIM + c, v);
    }
  }
}

template <int SHAPE, int RULE>
struct SSAdjointTile {
  static constexpr int DIM = ShapeInfo<SHAPE>::DIM, NN = ShapeInfo<SHAPE>::NN, NQ = RuleInfo<RULE>::NQ;
  static constexpr int NDOF = NN * DIM, NT = 128;
  // per element: dU_e and PBar_e; its points' dN/dX (NDOF x NQ, 8 bytes each: doubles, or float-float
  // hi and lo floats), property adjoints (6) and strain adjoints (6)
  static constexpr size_t per_el = sizeof(double) * (2 * NDOF + NQ * NDOF + NQ * 12);
  static constexpr int EPB0 = NT / NQ > 0 ? NT / NQ : 1;
  static constexpr int EPB = (size_t)EPB0 * per_el <= 96 * 1024 ? EPB0 : (int)((96 * 1024) / per_el);
  static_assert(EPB >= 1, "one element must fit in shared memory");
  // the staged dN/dX: row r = l NN + a (component l of dN_a/dX) over the tile's points, an odd row
  // stride so that the per-DOF reads of phase C (different rows, one point) spread over the banks
  static constexpr int NP = EPB * NQ, NPS = NP | 1;
  static constexpr size_t u_off = 0, p_off = u_off + sizeof(double) * EPB * NDOF,
                          g_off = p_off + sizeof(double) * EPB * NDOF,
                          q_off = g_off + sizeof(double) * NDOF * NPS,  // double [NP][6]: property adjoints
                          d_off = q_off + sizeof(double) * NP * 6,      // double or ff [NP][6]: strain adjoints
                          c_off = d_off + sizeof(double) * NP * 6,      // SSRevConst [EPB]
                          bytes = c_off + sizeof(SSRevConst) * EPB;
};

// FF: the three B-products (B dU, B PBar, B^T deBar) in float-float arithmetic on the FP32 pipe from the
// float-float geometry (geomG32 + geomGlo), with nodal values taken relative to the element's first
// node (sum_a dN_a/dX = 0); the reverse return map stays FP64.  ~2^-48 relative accuracy.
// Phase 0 stages the tile's dN/dX rows in shared memory (cp.async), so that phase A (one thread per
// point: B dU, B PBar, the reverse update) and phase C (one thread per element DOF: B^T deBar summed
// over the points) read it there rather than twice from global memory.
template <int SHAPE, int RULE, bool FF, bool GX>
__global__ void __launch_bounds__(SSAdjointTile<SHAPE, RULE>::NT) adjoint_ss_kernel(SSAdjointArgs a) {
  using T = SSAdjointTile<SHAPE, RULE>;
  constexpr int DIM = T::DIM, NN = T::NN, NQ = T::NQ, NDOF = T::NDOF, EPB = T::EPB, NT = T::NT, NPS = T::NPS;
  extern __shared__ __align__(128) unsigned char smem[];
  double* su = reinterpret_cast<double*>(smem + T::u_off);
  double* sp = reinterpret_cast<double*>(smem + T::p_off);
  float* sGh = reinterpret_cast<float*>(smem + T::g_off);  // FF: hi floats, then lo floats
  float* sGl = sGh + NDOF * NPS;
  double* sGd = reinterpret_cast<double*>(smem + T::g_off);  // FP64 dN/dX
  double* sg = reinterpret_cast<double*>(smem + T::q_off);
  double* sd = reinterpret_cast<double*>(smem + T::d_off);
  SSRevConst* src = reinterpret_cast<SSRevConst*>(smem + T::c_off);
  const int64_t e0 = (int64_t)blockIdx.x * EPB;
  const int64_t nEl = a.nEl, stride = nEl * NQ;
  const bool vm = a.material == EFE_MAT_VON_MISES;
  const int nLoc = nEl - e0 < EPB ? (int)(nEl - e0) : EPB;  // elements of this tile

  // ---- phase 0: dN/dX rows (cp.async), dU_e and PBar_e, the elements' constants
  for (int t = threadIdx.x; t < NDOF * nLoc * NQ; t += NT) {
    const int r = t / (nLoc * NQ), j = t - r * (nLoc * NQ);
    const int64_t gi = (int64_t)r * stride + e0 * NQ + j;
    if constexpr (FF) {
      tc::cp_async4(sGh + r * NPS + j, a.geomG32 + gi);
      tc::cp_async4(sGl + r * NPS + j, a.geomGlo + gi);
    } else {
      tc::cp_async8(sGd + r * NPS + j, a.geomG + gi);
    }
  }
  if (threadIdx.x < nLoc) src[threadIdx.x] = ss_rev_const(a.props + (e0 + threadIdx.x) * a.nProps, vm);
  for (int t = threadIdx.x; t < EPB * NN; t += NT) {
    const int le = t / NN, n = t % NN;
    const int64_t e = e0 + le;
    if (e >= nEl) continue;
    const int32_t dof = a.nodeDof[a.conn[e * NN + n]];
    if constexpr (FF) {
      const int32_t dof0 = a.nodeDof[a.conn[e * NN]];
      ff* uf = reinterpret_cast<ff*>(su);
      ff* pf = reinterpret_cast<ff*>(sp);
      for (int c = 0; c < DIM; ++c) {
        uf[le * NDOF + n * DIM + c] = ff_split(a.dU[dof + c] - a.dU[dof0 + c]);
        pf[le * NDOF + n * DIM + c] = ff_split(a.Pbar ? a.Pbar[dof + c] - a.Pbar[dof0 + c] : 0.0);
      }
    } else {
      for (int c = 0; c < DIM; ++c) {
        su[le * NDOF + n * DIM + c] = a.dU[dof + c];
        sp[le * NDOF + n * DIM + c] = a.Pbar ? a.Pbar[dof + c] : 0.0;
      }
    }
  }
  tc::cp_async_wait_all();
  __syncthreads();

  // ---- phase A: one thread per point
  for (int t = threadIdx.x; t < EPB * NQ; t += NT) {
    const int le = t / NQ, q = t % NQ;
    const int64_t e = e0 + le;
    if (e >= nEl) continue;
    const int64_t pt = e * NQ + q;
    const int pl = le * NQ + q;  // the point in the tile
    const double s = a.geomS[pt];
    // B u and B PBar (small-strain Voigt 11,22,33,12,13,23, engineering shear)
    double de[6] = {0, 0, 0, 0, 0, 0}, bp[6] = {0, 0, 0, 0, 0, 0};
    if constexpr (FF) {
      const ff* uf = reinterpret_cast<const ff*>(su) + le * NDOF;
      const ff* pf = reinterpret_cast<const ff*>(sp) + le * NDOF;
      ff ad[6] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}}, ab[6] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}};
      for (int n = 0; n < NN; ++n) {
        const ff gx = ff{sGh[n * NPS + pl], sGl[n * NPS + pl]};
        const ff gy = ff{sGh[(NN + n) * NPS + pl], sGl[(NN + n) * NPS + pl]};
        if constexpr (DIM == 3) {
          const ff gz = ff{sGh[(2 * NN + n) * NPS + pl], sGl[(2 * NN + n) * NPS + pl]};
          const ff ux = uf[n * 3], uy = uf[n * 3 + 1], uz = uf[n * 3 + 2];
          const ff px = pf[n * 3], py = pf[n * 3 + 1], pz = pf[n * 3 + 2];
          ff_fma(ad[0], gx, ux);
          ff_fma(ad[1], gy, uy);
          ff_fma(ad[2], gz, uz);
          ff_fma(ad[3], gy, ux);
          ff_fma(ad[3], gx, uy);
          ff_fma(ad[4], gz, ux);
          ff_fma(ad[4], gx, uz);
          ff_fma(ad[5], gz, uy);
          ff_fma(ad[5], gy, uz);
          ff_fma(ab[0], gx, px);
          ff_fma(ab[1], gy, py);
          ff_fma(ab[2], gz, pz);
          ff_fma(ab[3], gy, px);
          ff_fma(ab[3], gx, py);
          ff_fma(ab[4], gz, px);
          ff_fma(ab[4], gx, pz);
          ff_fma(ab[5], gz, py);
          ff_fma(ab[5], gy, pz);
        } else {
          const ff ux = uf[n * 2], uy = uf[n * 2 + 1];
          const ff px = pf[n * 2], py = pf[n * 2 + 1];
          ff_fma(ad[0], gx, ux);
          ff_fma(ad[1], gy, uy);
          ff_fma(ad[3], gy, ux);
          ff_fma(ad[3], gx, uy);
          ff_fma(ab[0], gx, px);
          ff_fma(ab[1], gy, py);
          ff_fma(ab[3], gy, px);
          ff_fma(ab[3], gx, py);
        }
      }
      for (int f = 0; f < 6; ++f) {
        de[f] = ff_to_double(ad[f]);
        bp[f] = ff_to_double(ab[f]);
      }
    } else {
      const double* u = su + le * NDOF;
      const double* pb = sp + le * NDOF;
      for (int n = 0; n < NN; ++n) {
        const double gx = sGd[n * NPS + pl], gy = sGd[(NN + n) * NPS + pl];
        if constexpr (DIM == 3) {
          const double gz = sGd[(2 * NN + n) * NPS + pl];
          const double ux = u[n * 3], uy = u[n * 3 + 1], uz = u[n * 3 + 2];
          const double px = pb[n * 3], py = pb[n * 3 + 1], pz = pb[n * 3 + 2];
          de[0] = fma(gx, ux, de[0]);
          de[1] = fma(gy, uy, de[1]);
          de[2] = fma(gz, uz, de[2]);
          de[3] = fma(gx, uy, fma(gy, ux, de[3]));
          de[4] = fma(gx, uz, fma(gz, ux, de[4]));
          de[5] = fma(gy, uz, fma(gz, uy, de[5]));
          bp[0] += gx * px;
          bp[1] += gy * py;
          bp[2] += gz * pz;
          bp[3] += gy * px + gx * py;
          bp[4] += gz * px + gx * pz;
          bp[5] += gz * py + gy * pz;
        } else {
          const double ux = u[n * 2], uy = u[n * 2 + 1];
          const double px = pb[n * 2], py = pb[n * 2 + 1];
          de[0] += gx * ux;
          de[1] += gy * uy;
          de[3] += gy * ux + gx * uy;
          bp[0] += gx * px;
          bp[1] += gy * py;
          bp[3] += gy * px + gx * py;
        }
      }
    }
    // seeds: the new state's adjoint, plus P_e = -sum_q s B^T sig  =>  sigBar -= s B PBar
    double sBar[6], eBar[6], kBar = 0.0;
    for (int f = 0; f < 6; ++f) {
      sBar[f] = (a.barIn ? a.barIn[(int64_t)f * stride + pt] : 0.0) - s * bp[f];
      eBar[f] = a.barIn ? a.barIn[(int64_t)(6 + f) * stride + pt] : 0.0;
    }
    if (vm && a.barIn) kBar = a.barIn[(int64_t)12 * stride + pt];
    double sig0[6], k0 = 0.0;
    for (int f = 0; f < 6; ++f) sig0[f] = a.stateBefore[(int64_t)f * stride + pt];
    if (vm) k0 = a.stateBefore[(int64_t)12 * stride + pt];
    const double* props = a.props + e * a.nProps;
    const SSRevConst& rc = src[le];
    const VMConst& mc = rc.c;
    double sig0Bar[6] = {0, 0, 0, 0, 0, 0}, k0Bar = 0.0, pBar[6] = {0, 0, 0, 0, 0, 0};
    double deBar[6];
    for (int f = 0; f < 6; ++f) deBar[f] = eBar[f];  // eps = eps0 + de
    bool planeStress = false;
    if constexpr (DIM == 2) planeStress = a.planeStress;
    if (planeStress) {
      // eps33 receives the plane-stress solution's increment, not a B-product: its seed enters the
      // local Newton
      deBar[2] = 0.0;
      if (vm)
        von_mises_plane_stress_reverse(rc, sig0, k0, de, sBar, kBar, eBar[2], sig0Bar, k0Bar, deBar, pBar);
      else
        linear_elastic_plane_stress_reverse(props[0], props[1], de, sBar, eBar[2], sig0Bar, deBar, pBar);
    } else {
      hypo3d_reverse(rc, vm, sig0, k0, de, sBar, kBar, sig0Bar, k0Bar, deBar, pBar);
    }
    if (a.barOut) {
      for (int f = 0; f < 6; ++f) {
        a.barOut[(int64_t)f * stride + pt] += sig0Bar[f];
        a.barOut[(int64_t)(6 + f) * stride + pt] += eBar[f];
      }
      if (vm) a.barOut[(int64_t)12 * stride + pt] += k0Bar;
    }
    double* gq = sg + pl * 6;
    for (int k = 0; k < 6; ++k) gq[k] = pBar[k];
    if constexpr (GX) coordinate_adjoint<SHAPE, RULE, FF>(a, e, q, pt, stride, s, mc, vm, planeStress, sig0, k0, de,
                                                 deBar, bp, su + le * NDOF, sp + le * NDOF);
    // the strain adjoint, for B^T deBar in phase C
    if constexpr (FF) {
      ff* df = reinterpret_cast<ff*>(sd) + pl * 6;
      for (int f = 0; f < 6; ++f) df[f] = ff_split(deBar[f]);
    } else {
      for (int f = 0; f < 6; ++f) sd[pl * 6 + f] = deBar[f];
    }
  }
  __syncthreads();

  // ---- phase C: per element DOF (node n, component c): sum over the points of (B^T deBar)_(n,c) =
  // row c of the symmetric strain adjoint (Voigt, engineering shear) times dN_n/dX; one atomic per
  // element DOF.  Per element property: plain stores (one thread owns an element's property).
  for (int t = threadIdx.x; t < EPB * NDOF; t += NT) {
    const int le = t / NDOF, k = t % NDOF, n = k / DIM, c = k % DIM;
    const int64_t e = e0 + le;
    if (e >= nEl) continue;
    // row c: 3D (11 12 13 | 12 22 23 | 13 23 33) = Voigt (0 3 4 | 3 1 5 | 4 5 2); 2D (0 3 | 3 1)
    const int v0 = c == 0 ? 0 : (c == 1 ? 3 : 4), v1 = c == 0 ? 3 : (c == 1 ? 1 : 5), v2 = c == 0 ? 4 : (c == 1 ? 5 : 2);
    double v;
    if constexpr (FF) {
      const ff* df = reinterpret_cast<const ff*>(sd);
      ff acc{0, 0};
      for (int q = 0; q < NQ; ++q) {
        const int pl = le * NQ + q;
        ff_fma(acc, df[pl * 6 + v0], ff{sGh[n * NPS + pl], sGl[n * NPS + pl]});
        ff_fma(acc, df[pl * 6 + v1], ff{sGh[(NN + n) * NPS + pl], sGl[(NN + n) * NPS + pl]});
        if constexpr (DIM == 3) ff_fma(acc, df[pl * 6 + v2], ff{sGh[(2 * NN + n) * NPS + pl], sGl[(2 * NN + n) * NPS + pl]});
      }
      v = ff_to_double(acc);
    } else {
      v = 0.0;
      for (int q = 0; q < NQ; ++q) {
        const int pl = le * NQ + q;
        double r = sd[pl * 6 + v0] * sGd[n * NPS + pl] + sd[pl * 6 + v1] * sGd[(NN + n) * NPS + pl];
        if constexpr (DIM == 3) r += sd[pl * 6 + v2] * sGd[(2 * NN + n) * NPS + pl];
        v += r;
      }
    }
    const int32_t dof = a.nodeDof[a.conn[e * NN + n]] + c;
    atomicAdd(a.dUbar + dof, v);
  }
  if (a.gProps) {
    const int np = a.nProps < 6 ? a.nProps : 6;
    for (int t = threadIdx.x; t < EPB * np; t += NT) {
      const int le = t / np, k = t % np;
      const int64_t e = e0 + le;
      if (e >= nEl) continue;
      double v = 0.0;
      for (int q = 0; q < NQ; ++q) v += sg[(le * NQ + q) * 6 + k];
      a.gProps[e * a.nProps + k] += v;
    }
  }
}

template <int SHAPE, int RULE>
cudaError_t launch_adjoint_ss(const SSAdjointArgs& a, cudaStream_t st) {
  using T = SSAdjointTile<SHAPE, RULE>;
  if (a.nEl == 0) return cudaSuccess;
  const bool ff = a.geomG32 && a.geomGlo;
  auto kern = a.gX ? (ff ? adjoint_ss_kernel<SHAPE, RULE, true, true> : adjoint_ss_kernel<SHAPE, RULE, false, true>)
                   : (ff ? adjoint_ss_kernel<SHAPE, RULE, true, false> : adjoint_ss_kernel<SHAPE, RULE, false, false>);
  cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::bytes);
  if (err != cudaSuccess) return err;
  const int64_t blocks = (a.nEl + T::EPB - 1) / T::EPB;
  kern<<<(unsigned)blocks, T::NT, T::bytes, st>>>(a);
  return cudaGetLastError();
}

}  // namespace efe
