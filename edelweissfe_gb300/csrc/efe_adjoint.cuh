// efe_adjoint.cuh -- adjoint of the total-Lagrangian hyperelastic element residual.
//
// For L = lambda^T P(X, U, mu, K), with P the element residual of DisplacementTLElement with a
// Neo-Hooke material (displacementtlelement/element.py:389-414: P_a -= s tau h_a, s = det J w t,
// h_a = F^-T dN_a/dX, tau the Kirchhoff stress), the kernel returns dL/dX (nodal reference
// coordinates) and dL/dmu, dL/dK per element, by reverse-mode differentiation written out by hand:
//
//   L = -s phi,  phi = tau : M,  M = Lambda F^-1,  Lambda = sum_a lambda_a (x) dN_a/dX
//   dphi/dF  = c1 (M F + M^T F) + (c2 tr M + c3 M:B) F^-T + c4 tr(M) F - F^-T Lambda^T tau F^-T
//   dphi/dLambda = tau F^-T
//   then through F = I + sum_a U_a (x) G_a and Lambda to G = dN/dX = J^-1 dN/dxi, and through
//   J = dN/dxi . X (with the Hexa20 third-row term of the reference) and s = det J w t to X.
// Parameter derivatives use dtau/dmu, dtau/dK of each variant.
#pragma once
#include "efe_launch.cuh"

namespace efe {

// d tau / d mu and d tau / d K of the three Neo-Hooke variants (same formulas as neo_hooke()).
__device__ inline void neo_hooke_param_derivatives(int material, double mu, double K, const double F[3][3],
                                                   double dmu[3][3], double dK[3][3]) {
  double B[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) B[i][j] = F[i][0] * F[j][0] + F[i][1] * F[j][1] + F[i][2] * F[j][2];
  const double J = det3(F);
  const double I1 = B[0][0] + B[1][1] + B[2][2];
  double aB = 0.0, aI = 0.0, bI = 0.0;  // dtau/dmu = aB B + aI I, dtau/dK = bI I
  if (material == EFE_MAT_NEOHOOKE_WA) {
    aB = 1.0;
    aI = -(2.0 / 3.0) * (J * J - J) - 1.0;
    bI = J * J - J;
  } else if (material == EFE_MAT_NEOHOOKE_WB) {
    const double J23 = pow(J, 2.0 / 3.0);
    aB = 1.0 / J23;
    aI = -I1 / (3.0 * J23);
    bI = (J * J - 1.0 / (J * J)) / 4.0;
  } else {
    const double p = pow(J, 2.0 / 3.0 - K / mu);
    const double lnJ = log(J);
    aB = 1.0;
    aI = -p * (1.0 + (K / mu) * lnJ);
    bI = p * lnJ;
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      dmu[i][j] = aB * B[i][j] + (i == j ? aI : 0.0);
      dK[i][j] = (i == j ? bI : 0.0);
    }
}

// One thread per (element, quadrature point).  gX is [nNodes][dim], gP is [nElements][2] (mu, K);
// both are accumulated into (the caller zeroes them).
template <int SHAPE, int RULE>
__global__ void adjoint_tl_kernel(int64_t nEl, const int32_t* __restrict__ conn, const int32_t* __restrict__ nodeDof,
                                  const double* __restrict__ coords, const double* __restrict__ U,
                                  const double* __restrict__ lam, const double* __restrict__ props, int nProps,
                                  int material, const double* __restrict__ thickness, Hexa20Fix fix, double* gX,
                                  double* gP) {
  constexpr int DIM = ShapeInfo<SHAPE>::DIM, NN = ShapeInfo<SHAPE>::NN, NQ = RuleInfo<RULE>::NQ;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nEl * NQ) return;
  const int64_t e = t / NQ;
  const int q = (int)(t % NQ);
  double xi, eta, zeta, w;
  quadrature_point(RULE, q, xi, eta, zeta, w);
  const double p[3] = {eta, xi, zeta};
  double D[DIM][NN];
  shape_derivatives<SHAPE>(p, D);
  // nodal coordinates, U and lambda are read where they are used (L1-resident) rather than held
  // in registers across the whole point: fewer registers, no spills.  The nodal sums (J, dN/dX, F,
  // Lambda, and in reverse Gbar and iJbar) run in float-float arithmetic on the FP32 pipe with the
  // nodal values taken relative to node 0 (sum_a dN_a = 0); the material part stays FP64.
  const int32_t* en = conn + e * NN;
  const int32_t n0 = en[0];
  const int32_t dof0 = nodeDof[n0];
  // Jacobian table row 2 of Hexa20 carries (zeta - xi) * inv(A)[5] (the reference's _J3D20); that
  // row does not sum to zero over the nodes, so its sum times X_0 is added back in FP64
  const double quirk = (SHAPE == EFE_HEXA20) ? (zeta - xi) : 0.0;
  ff Dff[DIM][NN];
#pragma unroll
  for (int r = 0; r < DIM; ++r)
#pragma unroll 1
    for (int a = 0; a < NN; ++a) {
      double d = D[r][a];
      if constexpr (SHAPE == EFE_HEXA20) {
        if (r == 2) d += quirk * fix.r[a % 20];
      }
      Dff[r][a] = ff_split_bits(d);
    }
  ff Jff[3][3] = {{{0, 0}, {0, 0}, {0, 0}}, {{0, 0}, {0, 0}, {0, 0}}, {{0, 0}, {0, 0}, {0, 0}}};
#pragma unroll 1
  for (int a = 1; a < NN; ++a)
#pragma unroll
    for (int c = 0; c < DIM; ++c) {
      const ff xr = ff_split_bits(coords[(int64_t)en[a] * DIM + c] - coords[(int64_t)n0 * DIM + c]);
#pragma unroll
      for (int r = 0; r < DIM; ++r) ff_fma(Jff[r][c], Dff[r][a], xr);
    }
  double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 1}};
#pragma unroll
  for (int r = 0; r < DIM; ++r)
#pragma unroll
    for (int c = 0; c < DIM; ++c) J[r][c] = ff_to_double_bits(Jff[r][c]);
  if constexpr (SHAPE == EFE_HEXA20) {
    double rs = 0.0;
#pragma unroll 1
    for (int a = 0; a < NN; ++a) rs += fix.r[a % 20];
#pragma unroll
    for (int c = 0; c < DIM; ++c) J[2][c] += quirk * rs * coords[(int64_t)n0 * DIM + c];
  }
  double detJ, iJ[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 1}};
  if constexpr (DIM == 2) {
    detJ = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    const double rd = 1.0 / detJ;
    iJ[0][0] = J[1][1] * rd;
    iJ[0][1] = -J[0][1] * rd;
    iJ[1][0] = -J[1][0] * rd;
    iJ[1][1] = J[0][0] * rd;
  } else {
    detJ = det3(J);
    inv3(J, detJ, iJ);
  }
  // G = J^-1 dN/dxi (the plain table, without the Hexa20 row term: G uses the reference's
  // shape-function derivatives)
  ff G[DIM][NN];
  {
    ff iJf[DIM][DIM];
#pragma unroll
    for (int c = 0; c < DIM; ++c)
#pragma unroll
      for (int r = 0; r < DIM; ++r) iJf[c][r] = ff_split_bits(iJ[c][r]);
#pragma unroll
    for (int c = 0; c < DIM; ++c)
#pragma unroll 1
      for (int a = 0; a < NN; ++a) {
        ff g{0, 0};
#pragma unroll
        for (int r = 0; r < DIM; ++r) ff_fma(g, iJf[c][r], ff_split_bits(D[r][a]));
        G[c][a] = g;
      }
  }
  const double th = (DIM == 2 && thickness) ? thickness[e] : 1.0;
  const double s = detJ * w * th;
  double F[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  double Lam[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  {
    ff Ff[DIM][DIM], Lf[DIM][DIM];
#pragma unroll
    for (int i = 0; i < DIM; ++i)
#pragma unroll
      for (int j = 0; j < DIM; ++j) Ff[i][j] = Lf[i][j] = ff{0, 0};
#pragma unroll 1
    for (int a = 1; a < NN; ++a) {
      const int32_t dof = nodeDof[en[a]];
#pragma unroll
      for (int i = 0; i < DIM; ++i) {
        const ff ur = ff_split_bits(U[dof + i] - U[dof0 + i]);
        const ff lr = ff_split_bits(lam[dof + i] - lam[dof0 + i]);
#pragma unroll
        for (int j = 0; j < DIM; ++j) {
          ff_fma(Ff[i][j], ur, G[j][a]);
          ff_fma(Lf[i][j], lr, G[j][a]);
        }
      }
    }
#pragma unroll
    for (int i = 0; i < DIM; ++i)
#pragma unroll
      for (int j = 0; j < DIM; ++j) {
        F[i][j] += ff_to_double_bits(Ff[i][j]);
        Lam[i][j] = ff_to_double_bits(Lf[i][j]);
      }
  }
  const double Jf = det3(F);
  double iF[3][3];
  inv3(F, Jf, iF);
  const double mu = props[e * nProps + 0], Kb = props[e * nProps + 1];
  NeoHookeOut o;
  neo_hooke(material, mu, Kb, F, o);
  double M[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) M[i][j] = Lam[i][0] * iF[0][j] + Lam[i][1] * iF[1][j] + Lam[i][2] * iF[2][j];
  double phi = 0.0, trM = M[0][0] + M[1][1] + M[2][2], MB = 0.0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      phi += o.tau[i][j] * M[i][j];
      MB += M[i][j] * o.Bm[i][j];
    }
  // parameter derivatives
  {
    double dmu[3][3], dK[3][3];
    neo_hooke_param_derivatives(material, mu, Kb, F, dmu, dK);
    double gm = 0.0, gk = 0.0;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        gm += dmu[i][j] * M[i][j];
        gk += dK[i][j] * M[i][j];
      }
    atomicAdd(gP + 2 * e + 0, -s * gm);
    atomicAdd(gP + 2 * e + 1, -s * gk);
  }
  // dphi/dF and dphi/dLambda, scaled by dL/dphi = -s
  double MF[3][3], MtF[3][3], T1[3][3], Fbar[3][3], Lbar[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      MF[i][j] = M[i][0] * F[0][j] + M[i][1] * F[1][j] + M[i][2] * F[2][j];
      MtF[i][j] = M[0][i] * F[0][j] + M[1][i] * F[1][j] + M[2][i] * F[2][j];
    }
  // T1 = Lambda^T tau ; Fbar -= iF^T T1 iF^T
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) T1[i][j] = Lam[0][i] * o.tau[0][j] + Lam[1][i] * o.tau[1][j] + Lam[2][i] * o.tau[2][j];
  double T2[3][3];  // T1 iF^T
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) T2[i][j] = T1[i][0] * iF[j][0] + T1[i][1] * iF[j][1] + T1[i][2] * iF[j][2];
  const double cI = o.c2 * trM + o.c3 * MB;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      const double iFt_T2 = iF[0][i] * T2[0][j] + iF[1][i] * T2[1][j] + iF[2][i] * T2[2][j];
      const double v = o.c1 * (MF[i][j] + MtF[i][j]) + cI * iF[j][i] + o.c4 * trM * F[i][j] - iFt_T2;
      Fbar[i][j] = -s * v;
      Lbar[i][j] = -s * (o.tau[i][0] * iF[j][0] + o.tau[i][1] * iF[j][1] + o.tau[i][2] * iF[j][2]);
    }
  const double sbar = -phi;
  // Gbar[k][a] = sum_i Fbar[i][k] U[a][i] + Lbar[i][k] lambda[a][i], and G = iJ D:
  // iJbar[c][r] = sum_a Gbar[c][a] D[r][a] (U and lambda relative to node 0: sum_a D[r][a] = 0)
  double iJbar[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  {
    ff Fb[DIM][DIM], Lb[DIM][DIM], ib[DIM][DIM];
#pragma unroll
    for (int i = 0; i < DIM; ++i)
#pragma unroll
      for (int k = 0; k < DIM; ++k) {
        Fb[i][k] = ff_split_bits(Fbar[i][k]);
        Lb[i][k] = ff_split_bits(Lbar[i][k]);
        ib[i][k] = ff{0, 0};
      }
#pragma unroll 1
    for (int a = 1; a < NN; ++a) {
      const int32_t dof = nodeDof[en[a]];
      ff ur[DIM], lr[DIM];
#pragma unroll
      for (int i = 0; i < DIM; ++i) {
        ur[i] = ff_split_bits(U[dof + i] - U[dof0 + i]);
        lr[i] = ff_split_bits(lam[dof + i] - lam[dof0 + i]);
      }
#pragma unroll
      for (int k = 0; k < DIM; ++k) {
        ff gb{0, 0};
#pragma unroll
        for (int i = 0; i < DIM; ++i) {
          ff_fma(gb, Fb[i][k], ur[i]);
          ff_fma(gb, Lb[i][k], lr[i]);
        }
#pragma unroll
        for (int r = 0; r < DIM; ++r) ff_fma(ib[k][r], gb, ff_split_bits(D[r][a]));
      }
    }
#pragma unroll
    for (int c = 0; c < DIM; ++c)
#pragma unroll
      for (int r = 0; r < DIM; ++r) iJbar[c][r] = ff_to_double_bits(ib[c][r]);
  }
  // Jbar = -iJ^T iJbar iJ^T + sbar * w * t * detJ * iJ^T, as two 3x3 products (A = iJ^T iJbar first)
  double A[3][3];
  for (int r = 0; r < DIM; ++r)
    for (int l = 0; l < DIM; ++l) {
      double v = 0.0;
      for (int k = 0; k < DIM; ++k) v += iJ[k][r] * iJbar[k][l];
      A[r][l] = v;
    }
  const double sdet = sbar * w * th * detJ;
  double Jbar[3][3];
  for (int r = 0; r < DIM; ++r)
    for (int c = 0; c < DIM; ++c) {
      double v = 0.0;
      for (int l = 0; l < DIM; ++l) v += A[r][l] * iJ[c][l];
      Jbar[r][c] = -v + sdet * iJ[c][r];
    }
  for (int a = 0; a < NN; ++a) {
    const int32_t n = en[a];
    for (int c = 0; c < DIM; ++c) {
      double v = 0.0;
      for (int r = 0; r < DIM; ++r) {
        double d = D[r][a];
        if constexpr (SHAPE == EFE_HEXA20) {
          if (r == 2) d += quirk * fix.r[a % 20];
        }
        v += Jbar[r][c] * d;
      }
      atomicAdd(gX + (int64_t)n * DIM + c, v);
    }
  }
}

template <int SHAPE, int RULE>
cudaError_t launch_adjoint_tl(const AdjointArgs& a, cudaStream_t st) {
  const int64_t n = a.nEl * RuleInfo<RULE>::NQ;
  if (n == 0) return cudaSuccess;
  const int nt = 64;
  adjoint_tl_kernel<SHAPE, RULE><<<(unsigned)((n + nt - 1) / nt), nt, 0, st>>>(
      a.nEl, a.conn, a.nodeDof, a.coords, a.U, a.lam, a.props, a.nProps, a.material, a.thickness, a.fix, a.gX, a.gP);
  return cudaGetLastError();
}

}  // namespace efe
