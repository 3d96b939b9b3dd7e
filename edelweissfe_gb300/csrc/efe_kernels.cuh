// efe_kernels.cuh -- geometry set-up kernel and the fused element-evaluation + CSR-assembly kernel.
//
// One CTA evaluates a tile of EPB elements of one group in four phases:
//   0. gather the element nodes' displacements (dU for small strain, U for total Lagrangian)
//      and the CSR row lengths of the element nodes into shared memory;
//   A. one thread per (element, quadrature point): kinematics, material update (FP64, state read
//      from stateRef and written to stateTemp, structure-of-arrays, coalesced), residual
//      contribution and the per-point factors of the tangent, staged in shared memory;
//   C. one thread per (element, DOF): P_e = -sum_q r_q in quadrature-point order, atomically added
//      to P and |P_e| to F (NIST.computeElements, nonlinearimplicitstatic.py:837-844);
//   B. one thread per (element, node pair a, b): the 2x2 / 3x3 block of K_e for all quadrature
//      points, scattered with atomics into the CSR data through the pair slot map
//      (CSRGenerator.updateCSR, csrgenerator.pyx:100-115, without the VIJ vector).
// KT is the type of the tangent (double, or float in the mixed mode).
#pragma once
#include <type_traits>

#include "efe_device.cuh"
#include "efe_tc.cuh"

namespace efe {

struct GroupArgs {
  int64_t nElements, elementOffset;
  const int32_t* conn;
  const int32_t* pairSlot;
  const double* props;
  const double* thickness;
  const double* geomG;
  const float* geomG32;  // optional FP32 copy of geomG, used for the FP32 tangent
  const float* geomGlo;  // optional fl32(G - geomG32): with geomG32 the float-float form of G
  const double* geomS;
  const double* stateRef;
  double* stateTemp;
  const double* auxRef;
  double* auxTemp;
  int32_t nProps, material, plane, tileVariant;
  // mesh
  const int32_t* nodeDof;
  const int32_t* nodeRowLen;
  const double* U;
  const double* dU;
  void* Kdata;
  double* P;
  double* F;
  int32_t* status;
  // sizes for the device-side bounds checks (checks != 0: EFE_DEVICE_CHECKS=1 in the environment)
  int64_t nnz, nDof;
  int32_t nNodes, checks;
};

// Device-side bounds check (debug): false, with EFE_STATUS_BOUNDS and the element recorded, when an
// index read from the caller's arrays would leave its target array; the caller then skips the access.
__device__ __forceinline__ bool in_bounds(const GroupArgs& g, int64_t idx, int64_t size, int64_t e);

struct Hexa20Fix {
  double r[20];  // row 5 of the inverse of the Hexa20 polynomial-fit matrix (coefficient of t*u)
};

__device__ __forceinline__ void report(int32_t* status, int bits, int64_t globalElement, int npts) {
  atomicOr(status + 0, bits);
  atomicMax(status + 1, (int32_t)(0x7fffffff - globalElement));  // = INT32_MAX - first failing element
  atomicAdd(status + 2, npts);
}

__device__ __forceinline__ bool in_bounds(const GroupArgs& g, int64_t idx, int64_t size, int64_t e) {
  if (!g.checks || (idx >= 0 && idx < size)) return true;
  report(g.status, EFE_STATUS_BOUNDS, g.elementOffset + e, 0);
  return false;
}

// ------------------------------------------------------------------ geometry (once per mesh)
// J_i = dN/dxi (eta_i, xi_i, zeta_i) . X, with the reference's Hexa20 third-row term
// (displacementelement/_elementcomputationmatrices.py:369-540 uses a5*zeta where d(a5 t u)/du = a5 xi).
template <int SHAPE, int RULE>
__global__ void geometry_kernel(int64_t nEl, int64_t elOffset, const int32_t* __restrict__ conn,
                                const double* __restrict__ coords, const double* __restrict__ thickness,
                                double* __restrict__ G, float* __restrict__ G32, float* __restrict__ Glo,
                                double* __restrict__ S, int32_t* status, Hexa20Fix fix) {
  constexpr int DIM = ShapeInfo<SHAPE>::DIM, NN = ShapeInfo<SHAPE>::NN, NQ = RuleInfo<RULE>::NQ;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nEl * NQ) return;
  const int64_t e = t / NQ;
  const int q = (int)(t % NQ);
  double xi, eta, zeta, w;
  quadrature_point(RULE, q, xi, eta, zeta, w);
  const double p[3] = {eta, xi, zeta};  // swapped evaluation point
  double dN[DIM][NN];
  shape_derivatives<SHAPE>(p, dN);
  double X[NN][DIM];
  for (int a = 0; a < NN; ++a) {
    const int32_t n = conn[e * NN + a];
    for (int c = 0; c < DIM; ++c) X[a][c] = coords[(int64_t)n * DIM + c];
  }
  double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 1}};
  for (int r = 0; r < DIM; ++r)
    for (int c = 0; c < DIM; ++c) {
      double s = 0.0;
      for (int a = 0; a < NN; ++a) s += dN[r][a] * X[a][c];
      J[r][c] = s;
    }
  if constexpr (SHAPE == EFE_HEXA20) {
    for (int c = 0; c < DIM; ++c) {
      double a5 = 0.0;
      for (int a = 0; a < NN; ++a) a5 += fix.r[a] * X[a][c];
      J[2][c] += (zeta - xi) * a5;
    }
  }
  double detJ, iJ[3][3];
  if constexpr (DIM == 2) {
    detJ = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    iJ[0][0] = J[1][1] / detJ;
    iJ[0][1] = -J[0][1] / detJ;
    iJ[1][0] = -J[1][0] / detJ;
    iJ[1][1] = J[0][0] / detJ;
  } else {
    detJ = det3(J);
    inv3(J, detJ, iJ);
  }
  if (!(detJ > 0.0) || !isfinite(detJ)) report(status, EFE_STATUS_BAD_JACOBIAN, elOffset + e, 1);
  const int64_t stride = nEl * NQ;
  // dN/dX_c = sum_r invJ[c][r] dN/dxi_r   (B = a . blockdiag(invJ) . dN, _B3D8 :679-817)
  for (int c = 0; c < DIM; ++c)
    for (int a = 0; a < NN; ++a) {
      double s = 0.0;
      for (int r = 0; r < DIM; ++r) s += iJ[c][r] * dN[r][a];
      G[(int64_t)(c * NN + a) * stride + t] = s;
      if (G32) G32[(int64_t)(c * NN + a) * stride + t] = (float)s;
      if (Glo) Glo[(int64_t)(c * NN + a) * stride + t] = (float)(s - (double)(float)s);
    }
  const double th = (DIM == 2 && thickness) ? thickness[e] : 1.0;
  S[t] = detJ * w * th;
}

// ------------------------------------------------------------------ body force
// P_e[(a,c)] += sum_q N_a(xi_q, eta_q, zeta_q) * f_c * detJ_q * t * w_q with N at the library point and
// det J at the point the Jacobian is formed (DisplacementElement.computeBodyForce, element.py:348-371).
template <int SHAPE, int RULE>
__global__ void body_force_kernel(int64_t nSel, const int32_t* __restrict__ elems, const int32_t* __restrict__ conn,
                                  const int32_t* __restrict__ nodeDof, const double* __restrict__ S, double f0,
                                  double f1, double f2, double* P) {
  constexpr int DIM = ShapeInfo<SHAPE>::DIM, NN = ShapeInfo<SHAPE>::NN, NQ = RuleInfo<RULE>::NQ;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nSel * NN) return;
  const int64_t sel = t / NN;
  const int a = (int)(t % NN);
  const int64_t e = elems ? elems[sel] : sel;
  double acc = 0.0;
  for (int q = 0; q < NQ; ++q) {
    double xi, eta, zeta, w, N[NN];
    quadrature_point(RULE, q, xi, eta, zeta, w);
    const double p[3] = {xi, eta, zeta};
    shape_values<SHAPE>(p, N);
    acc += N[a] * S[e * NQ + q];
  }
  const int32_t dof = nodeDof[conn[e * NN + a]];
  const double f[3] = {f0, f1, f2};
  for (int c = 0; c < DIM; ++c) atomicAdd(P + dof + c, acc * f[c]);
}

// ------------------------------------------------------------------ assembly
enum Form { SS3 = 0, SS2 = 1, TLH = 2, TLV3 = 3, TLV2 = 4 };
template <int FORM, int DIM> struct FormInfo;
template <int DIM> struct FormInfo<SS3, DIM> { static constexpr int NVEC = 2, NSCAL = 3; };
template <int DIM> struct FormInfo<SS2, DIM> { static constexpr int NVEC = 1, NSCAL = 6; };
template <int DIM> struct FormInfo<TLH, DIM> { static constexpr int NVEC = 5, NSCAL = 2; };
template <int DIM> struct FormInfo<TLV3, DIM> { static constexpr int NVEC = 4, NSCAL = 9; };
template <int DIM> struct FormInfo<TLV2, DIM> { static constexpr int NVEC = 2, NSCAL = 10; };

template <int SHAPE, int RULE, int FORM, typename KT, int EPB>
struct Layout {
  static constexpr int DIM = ShapeInfo<SHAPE>::DIM, NN = ShapeInfo<SHAPE>::NN, NQ = RuleInfo<RULE>::NQ;
  static constexpr int NVEC = FormInfo<FORM, DIM>::NVEC, NSCAL = FormInfo<FORM, DIM>::NSCAL;
  static constexpr int NDOF = NN * DIM;
  // total-Lagrangian Neo-Hooke: per-point record between its sub-phases (F, F^-1, tau, B, c1-c3, s)
  // in FP64 and a copy of F, B, c1 s, c2 s, c3 s in the tangent's precision
  // Per-point strides of the shared arrays are odd (in their element size): consecutive threads
  // handle consecutive points, so an even stride would put several of them on one memory bank.
  static constexpr int NX = FORM == TLH ? 41 : 0, NXK = FORM == TLH ? 25 : 0;
  static constexpr int SR = (NN * DIM) | 1;                                           // doubles per point of r
  static constexpr int SC = FormInfo<FORM, DIM>::NSCAL | 1;                           // KT per point of sc
  static constexpr int SV = (NN * NVEC * DIM) | 1;                                    // KT per point of v
  // offsets in bytes; doubles first for alignment
  static constexpr size_t u_off = 0;                                              // double [EPB][NN][DIM]
  static constexpr size_t x_off = u_off + sizeof(double) * EPB * NDOF;            // double [EPB][NQ][NX]
  static constexpr size_t r_off = x_off + sizeof(double) * EPB * NQ * NX;         // double [EPB][NQ][SR]
  static constexpr size_t sc_off = r_off + sizeof(double) * EPB * NQ * SR;        // KT [EPB][NQ][SC]
  static constexpr size_t v_off = sc_off + sizeof(KT) * EPB * NQ * SC;            // KT [EPB][NQ][SV: NN][NVEC][DIM]
  static constexpr size_t xk_off = v_off + sizeof(KT) * EPB * NQ * SV;            // KT [EPB][NQ][NXK]
  static constexpr size_t mc_off = (xk_off + sizeof(KT) * EPB * NQ * NXK + 15) / 16 * 16;  // VMConst [EPB]
  static constexpr size_t rl_off = mc_off + sizeof(VMConst) * EPB;                                     // int [EPB][NN]
  static constexpr size_t bytes = rl_off + sizeof(int) * EPB * NN;
};

template <typename KT>
__device__ __forceinline__ void kadd(KT* p, KT v) {
  atomicAdd(p, v);
}

// State of the tensor-core tangent across the tiles of one CTA: the base of its TMEM columns and
// the parity of the MMA-completion mbarrier's next phase.
struct TCState {
  uint32_t tmem;
  uint32_t phase;
  bool failed;
  uint64_t* mbar;  // static shared memory of the kernel (never inside a tile's dynamic layout)
};

// Wait limit of the tensor-core completion (polls of mbarrier.try_wait); far beyond the ~1 us an
// MMA chunk takes.  On expiry the CTA records EFE_STATUS_TC_TIMEOUT and stops issuing MMAs.
constexpr int TC_WAIT_LIMIT = 1 << 22;

// FF: the strain increment and the residual of the small-strain 3D form are formed in float-float
// arithmetic from the float-float geometry (geomG32 + geomGlo); the return map stays FP64.
// One tile: the EPB elements starting at e0, processed by the NT threads of the calling CTA
// (every thread of the CTA must call it: it synchronises the CTA).
template <int SHAPE, int RULE, int FORM, typename KT, int EPB, int NT, bool FF>
__device__ __forceinline__ void assemble_tile(const GroupArgs& g, const int64_t e0, unsigned char* smem) {
  using L = Layout<SHAPE, RULE, FORM, KT, EPB>;
  constexpr int DIM = L::DIM, NN = L::NN, NQ = L::NQ, NVEC = L::NVEC, NDOF = L::NDOF;
  // the faster return-map arithmetic goes with the FP32 tangent (mixed modes)
  constexpr bool FASTRM = std::is_same<KT, float>::value;
  double* su = reinterpret_cast<double*>(smem + L::u_off);
  double* sr = reinterpret_cast<double*>(smem + L::r_off);
  KT* ssc = reinterpret_cast<KT*>(smem + L::sc_off);
  KT* sv = reinterpret_cast<KT*>(smem + L::v_off);
  int* srl = reinterpret_cast<int*>(smem + L::rl_off);
  VMConst* smc = reinterpret_cast<VMConst*>(smem + L::mc_off);

  const int64_t nEl = g.nElements;
  const bool tl = (FORM == TLH || FORM == TLV3 || FORM == TLV2);
  const double* Ux = tl ? g.U : g.dU;

  // ---- phase 0: nodal displacements and row lengths
  for (int t = threadIdx.x; t < EPB * NN; t += NT) {
    const int le = t / NN, a = t % NN;
    const int64_t e = e0 + le;
    if (e < nEl) {
      const int32_t node = g.conn[e * NN + a];
      if (!in_bounds(g, node, g.nNodes, e)) continue;
      const int32_t dof = g.nodeDof[node];
      if (!in_bounds(g, dof, g.nDof - DIM + 1, e)) continue;
      if constexpr (FF) {
        // displacement relative to node 0 (sum_a dN_a/dX = 0): no cancellation in the strain sum
        const int32_t node0 = g.conn[e * NN];
        if (!in_bounds(g, node0, g.nNodes, e)) continue;
        const int32_t dof0 = g.nodeDof[node0];
        if (!in_bounds(g, dof0, g.nDof - DIM + 1, e)) continue;
        ff* sf = reinterpret_cast<ff*>(su);
        for (int c = 0; c < DIM; ++c) sf[(le * NN + a) * DIM + c] = ff_split_bits(Ux[dof + c] - Ux[dof0 + c]);
      } else {
        for (int c = 0; c < DIM; ++c) su[(le * NN + a) * DIM + c] = Ux[dof + c];
      }
      srl[le * NN + a] = g.nodeRowLen[node];
    }
  }
  // per-element material constants, formed once per element instead of once per point
  if constexpr (FORM != TLH) {
    for (int le = threadIdx.x; le < EPB; le += NT) {
      const int64_t e = e0 + le;
      if (e < nEl) smc[le] = vm_const(g.props + e * g.nProps, g.material == EFE_MAT_VON_MISES);
    }
  }
  __syncthreads();

  // ---- phase A: material points
  const int64_t stride = nEl * NQ;
  if constexpr (FORM == TLH) {
    // Total Lagrangian Neo-Hooke (displacementtlelement/element.py:346-414) in three sub-phases, so
    // the per-node work of a point (the heavy part for 20-node elements) runs one thread per
    // (point, node) instead of one thread per point.
    double* sx = reinterpret_cast<double*>(smem + L::x_off);
    KT* sxk = reinterpret_cast<KT*>(smem + L::xk_off);
    // A0: F = I + sum_a U_a (x) dN_a/dX, one thread per (point, component)
    for (int t = threadIdx.x; t < EPB * NQ * DIM * DIM; t += NT) {
      const int c = t / (EPB * NQ), r = t % (EPB * NQ);
      const int le = r / NQ, q = r % NQ;
      const int64_t e = e0 + le;
      if (e >= nEl) continue;
      const int i = c / DIM, j = c % DIM;
      const int64_t pt = e * NQ + q;
      double f = (i == j) ? 1.0 : 0.0;
      if constexpr (FF) {
        // displacements relative to node 0 (sum_a dN_a/dX = 0) times the float-float geometry
        const ff* uf = reinterpret_cast<const ff*>(su) + le * NN * DIM;
        ff acc{0, 0};
        for (int a = 0; a < NN; ++a)
          ff_fma(acc, uf[a * DIM + i],
                 ff{g.geomG32[(int64_t)(j * NN + a) * stride + pt], g.geomGlo[(int64_t)(j * NN + a) * stride + pt]});
        f += ff_to_double_bits(acc);
      } else {
        const double* u = su + le * NN * DIM;
        double h = 0.0;
        for (int a = 0; a < NN; ++a) h += u[a * DIM + i] * g.geomG[(int64_t)(j * NN + a) * stride + pt];
        f += h;
      }
      sx[(le * NQ + q) * L::NX + i * 3 + j] = f;
    }
    __syncthreads();
    // A1: one thread per point: E, F^-1, Kirchhoff stress and its tangent scalars, state
    for (int t = threadIdx.x; t < EPB * NQ; t += NT) {
      const int le = t / NQ, q = t % NQ;
      const int64_t e = e0 + le;
      if (e >= nEl) continue;
      const int64_t pt = e * NQ + q;
      double* rec = sx + (le * NQ + q) * L::NX;
      KT* reck = sxk + (le * NQ + q) * L::NXK;
      const double* props = g.props + e * g.nProps;
      double F[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
      for (int i = 0; i < DIM; ++i)
        for (int j = 0; j < DIM; ++j) F[i][j] = rec[i * 3 + j];
      // Green-Lagrange E = 1/2 (H + H^T + H^T H), H = F - I  (:386)
      double Eg[3][3];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double hh = 0.0;
          for (int k = 0; k < DIM; ++k) hh += (F[k][i] - (k == i)) * (F[k][j] - (k == j));
          Eg[i][j] = (i < DIM && j < DIM) ? 0.5 * ((F[i][j] - (i == j)) + (F[j][i] - (i == j)) + hh) : 0.0;
        }
      const double Ev[6] = {Eg[0][0], Eg[1][1], Eg[2][2], Eg[0][1], Eg[1][2], Eg[0][2]};
      for (int f = 0; f < 6; ++f) g.auxTemp[(int64_t)f * stride + pt] = Ev[f];
      double detF, iF[3][3];
      if constexpr (DIM == 2) {
        detF = F[0][0] * F[1][1] - F[0][1] * F[1][0];
        iF[0][0] = F[1][1] / detF;
        iF[0][1] = -F[0][1] / detF;
        iF[1][0] = -F[1][0] / detF;
        iF[1][1] = F[0][0] / detF;
        iF[0][2] = iF[1][2] = iF[2][0] = iF[2][1] = 0.0;
        iF[2][2] = 1.0;
      } else {
        detF = det3(F);
        inv3(F, detF, iF);
      }
      NeoHookeOut o;
      neo_hooke(g.material, props[0], props[1], F, o);
      const double sig[6] = {o.tau[0][0], o.tau[1][1], o.tau[2][2], o.tau[0][1], o.tau[1][2], o.tau[0][2]};
      // strain slot = Voigt(E) at the active indices, zero elsewhere (:393, :404)
      double eps[6] = {Eg[0][0], Eg[1][1], 0.0, 2.0 * Eg[0][1], 0.0, 0.0};
      if constexpr (DIM == 3) {
        eps[2] = Eg[2][2];
        eps[4] = 2.0 * Eg[1][2];
        eps[5] = 2.0 * Eg[0][2];
      }
      const double s = g.geomS[pt];
      KT* sc = ssc + (le * NQ + q) * L::SC;
      const KT c1s = to_kt<KT>(o.c1 * s);
      sc[0] = c1s;
      sc[1] = to_kt<KT>(o.c4 * s);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          rec[i * 3 + j] = F[i][j];
          rec[9 + i * 3 + j] = iF[i][j];
          rec[18 + i * 3 + j] = o.tau[i][j];
          rec[27 + i * 3 + j] = o.Bm[i][j];
          reck[i * 3 + j] = to_kt<KT>(F[i][j]);
          reck[9 + i * 3 + j] = to_kt<KT>(o.Bm[i][j]);
        }
      rec[36] = o.c1;
      rec[37] = o.c2;
      rec[38] = o.c3;
      rec[39] = s;
      if constexpr (FF) {
        // the float-float sub-phase A2 reads F^-1, tau and s as (hi, lo) pairs from the same slots
        ff* recf = reinterpret_cast<ff*>(rec);
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) {
            recf[9 + i * 3 + j] = ff_split_bits(iF[i][j]);
            recf[18 + i * 3 + j] = ff_split_bits(o.tau[i][j]);
          }
        recf[39] = ff_split_bits(s);
      }
      reck[18] = c1s;
      reck[19] = to_kt<KT>(o.c2 * s);
      reck[20] = to_kt<KT>(o.c3 * s);
      // state write (stateTemp = updated copy of stateRef)
      for (int f = 0; f < 6; ++f) {
        g.stateTemp[(int64_t)f * stride + pt] = sig[f];
        g.stateTemp[(int64_t)(6 + f) * stride + pt] = eps[f];
      }
      g.stateTemp[(int64_t)12 * stride + pt] = o.energy;
      bool finite = true;
      for (int f = 0; f < 6; ++f) finite = finite && finite_bits(sig[f]);
      if (!finite) atomicOr(g.status, EFE_STATUS_NONFINITE);
    }
    __syncthreads();
    // A2: one thread per (point, node): h_a = F^-T dN_a/dX and the residual s tau h_a in FP64
    // (P_e -= s dN/dX^T F^-1 tau, :402, :414); the tangent's vectors in its own precision
    for (int t = threadIdx.x; t < EPB * NQ * NN; t += NT) {
      const int a = t / (EPB * NQ), r = t % (EPB * NQ);
      const int le = r / NQ, q = r % NQ;
      const int64_t e = e0 + le;
      if (e >= nEl) continue;
      const int64_t pt = e * NQ + q;
      const double* rec = sx + (le * NQ + q) * L::NX;
      const KT* reck = sxk + (le * NQ + q) * L::NXK;
      KT Gk[3], hk[3], gg[3], bh[3], thk[3];
      if constexpr (FF) {
        // h_a = F^-T G_a, tau h_a and s tau h_a in float-float arithmetic (FP32 pipe)
        const ff* recf = reinterpret_cast<const ff*>(rec);
        ff Gf[3] = {{0, 0}, {0, 0}, {0, 0}}, h[3] = {{0, 0}, {0, 0}, {0, 0}};
        for (int j = 0; j < DIM; ++j)
          Gf[j] = ff{g.geomG32[(int64_t)(j * NN + a) * stride + pt], g.geomGlo[(int64_t)(j * NN + a) * stride + pt]};
        for (int i = 0; i < DIM; ++i)
          for (int I = 0; I < DIM; ++I) ff_fma(h[i], Gf[I], recf[9 + I * 3 + i]);
        ff* rf = reinterpret_cast<ff*>(sr + (le * NQ + q) * L::SR);
        for (int j = 0; j < DIM; ++j) {
          ff th{0, 0}, ths{0, 0};
          for (int i = 0; i < DIM; ++i) ff_fma(th, recf[18 + j * 3 + i], h[i]);
          ff_fma(ths, th, recf[39]);
          rf[a * DIM + j] = ths;
          Gk[j] = Gf[j].h;
          hk[j] = h[j].h;
          thk[j] = ths.h;
        }
      } else {
        double G[3] = {0, 0, 0};
        for (int j = 0; j < DIM; ++j) G[j] = g.geomG[(int64_t)(j * NN + a) * stride + pt];
        double h[3] = {0, 0, 0};
        for (int i = 0; i < DIM; ++i)
          for (int I = 0; I < DIM; ++I) h[i] += G[I] * rec[9 + I * 3 + i];
        const double s = rec[39];
        double* rq = sr + (le * NQ + q) * L::SR;
        for (int j = 0; j < DIM; ++j) {
          double th = 0.0;
          for (int i = 0; i < DIM; ++i) th += rec[18 + j * 3 + i] * h[i];
          const double ths = th * s;
          rq[a * DIM + j] = ths;
          thk[j] = to_kt<KT>(ths);
        }
        for (int j = 0; j < DIM; ++j) {
          if constexpr (std::is_same<KT, float>::value)
            Gk[j] = g.geomG32 ? g.geomG32[(int64_t)(j * NN + a) * stride + pt] : to_kt<KT>(G[j]);
          else
            Gk[j] = G[j];
          hk[j] = to_kt<KT>(h[j]);
        }
      }
      for (int i = 0; i < DIM; ++i) {
        KT v1 = KT(0), v2 = KT(0);
        for (int I = 0; I < DIM; ++I) {
          v1 += reck[i * 3 + I] * Gk[I];      // g_a = F dN_a/dX
          v2 += reck[9 + i * 3 + I] * hk[I];  // B h_a
        }
        gg[i] = v1;
        bh[i] = v2;
      }
      const KT c1s = reck[18], c2s = reck[19], c3s = reck[20];
      KT* v = sv + (size_t)(le * NQ + q) * L::SV + a * NVEC * DIM;
      for (int j = 0; j < DIM; ++j) {
        v[0 * DIM + j] = Gk[j];
        v[1 * DIM + j] = hk[j];
        v[2 * DIM + j] = gg[j];
        v[3 * DIM + j] = c1s * gg[j] - thk[j];
        v[4 * DIM + j] = c2s * hk[j] + c3s * bh[j];
      }
    }
  } else {
  for (int t = threadIdx.x; t < EPB * NQ; t += NT) {
    const int le = t / NQ, q = t % NQ;
    const int64_t e = e0 + le;
    if (e >= nEl) continue;
    const int64_t pt = e * NQ + q;
    double Gm[DIM][NN];
    if constexpr (!FF) {
#pragma unroll
      for (int c = 0; c < DIM; ++c)
#pragma unroll
        for (int a = 0; a < NN; ++a) Gm[c][a] = g.geomG[(int64_t)(c * NN + a) * stride + pt];
    }
    const double s = g.geomS[pt];
    const double* u = su + le * NN * DIM;
    const double* props = g.props + e * g.nProps;
    double* rq = sr + (le * NQ + q) * L::SR;
    KT* sc = ssc + (le * NQ + q) * L::SC;
    KT* vq = sv + (size_t)(le * NQ + q) * L::SV;
    bool ok = true;
    double sig[6], eps[6], kappa = 0.0;
    for (int f = 0; f < 6; ++f) {
      sig[f] = g.stateRef[(int64_t)f * stride + pt];
      eps[f] = g.stateRef[(int64_t)(6 + f) * stride + pt];
    }
    const bool hasM = g.material != EFE_MAT_LINEAR_ELASTIC;
    if (hasM) kappa = g.stateRef[(int64_t)12 * stride + pt];

    if constexpr (FORM == SS3 || FORM == SS2) {
      // ------------------------------------------------ small strain (element.py:318-346)
      double de[6] = {0, 0, 0, 0, 0, 0};
      ff Gf[DIM][NN];
      if constexpr (FF) {
        const ff* uf = reinterpret_cast<const ff*>(su) + le * NN * DIM;
        ff acc[6] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}};
        for (int a = 0; a < NN; ++a) {
          for (int c = 0; c < DIM; ++c)
            Gf[c][a] = ff{g.geomG32[(int64_t)(c * NN + a) * stride + pt], g.geomGlo[(int64_t)(c * NN + a) * stride + pt]};
          const ff ux = uf[a * 3 + 0], uy = uf[a * 3 + 1], uz = uf[a * 3 + 2 % DIM];
          ff_fma(acc[0], Gf[0][a], ux);
          ff_fma(acc[1], Gf[1][a], uy);
          ff_fma(acc[2], Gf[2 % DIM][a], uz);
          ff_fma(acc[3], Gf[1][a], ux);
          ff_fma(acc[3], Gf[0][a], uy);
          ff_fma(acc[4], Gf[2 % DIM][a], ux);
          ff_fma(acc[4], Gf[0][a], uz);
          ff_fma(acc[5], Gf[2 % DIM][a], uy);
          ff_fma(acc[5], Gf[1][a], uz);
        }
        for (int f = 0; f < 6; ++f) de[f] = ff_to_double_bits(acc[f]);
      } else if constexpr (DIM == 3) {
        for (int a = 0; a < NN; ++a) {
          const double ux = u[a * 3 + 0], uy = u[a * 3 + 1], uz = u[a * 3 + 2];
          const double gx = Gm[0][a], gy = Gm[1][a], gz = Gm[2][a];
          // one FMA per product (B . dU, element.py:322)
          de[0] = fma(gx, ux, de[0]);
          de[1] = fma(gy, uy, de[1]);
          de[2] = fma(gz, uz, de[2]);
          de[3] = fma(gx, uy, fma(gy, ux, de[3]));
          de[4] = fma(gx, uz, fma(gz, ux, de[4]));
          de[5] = fma(gy, uz, fma(gz, uy, de[5]));
        }
      } else {
        for (int a = 0; a < NN; ++a) {
          const double ux = u[a * DIM + 0], uy = u[a * DIM + 1];
          const double gx = Gm[0][a], gy = Gm[1][DIM == 2 ? a : a];
          de[0] += gx * ux;
          de[1] += gy * uy;
          de[3] += gy * ux + gx * uy;
        }
      }
      if constexpr (FORM == SS3) {
        Tangent3 T;
        if (g.material == EFE_MAT_VON_MISES)
          ok = von_mises_3d<FASTRM>(smc[le], sig, de, kappa, T);
        else
          linear_elastic_3d(smc[le], sig, de, T);
        // residual r_a = s * sigma . G_a   (small-strain Voigt order 11,22,33,12,13,23)
        if constexpr (FF) {
          ff sf[6];
          const ff s_ff = ff_split_bits(s);
          for (int f = 0; f < 6; ++f) sf[f] = ff_mul(ff_split_bits(sig[f]), s_ff);
          ff* rf = reinterpret_cast<ff*>(rq);
          for (int a = 0; a < NN; ++a) {
            ff r0{0, 0}, r1{0, 0}, r2{0, 0};
            ff_fma(r0, sf[0], Gf[0][a]);
            ff_fma(r0, sf[3], Gf[1][a]);
            ff_fma(r0, sf[4], Gf[2 % DIM][a]);
            ff_fma(r1, sf[3], Gf[0][a]);
            ff_fma(r1, sf[1], Gf[1][a]);
            ff_fma(r1, sf[5], Gf[2 % DIM][a]);
            ff_fma(r2, sf[4], Gf[0][a]);
            ff_fma(r2, sf[5], Gf[1][a]);
            ff_fma(r2, sf[2], Gf[2 % DIM][a]);
            rf[a * DIM + 0] = r0;
            rf[a * DIM + 1] = r1;
            rf[a * DIM + 2 % DIM] = r2;
          }
        } else {
          double ss[6];
          for (int f = 0; f < 6; ++f) ss[f] = sig[f] * s;
          for (int a = 0; a < NN; ++a) {
            const double gx = Gm[0][a], gy = Gm[1][a], gz = Gm[2 % DIM][a];
            rq[a * DIM + 0] = ss[0] * gx + ss[3] * gy + ss[4] * gz;
            rq[a * DIM + 1] = ss[3] * gx + ss[1] * gy + ss[5] * gz;
            rq[a * DIM + 2 % DIM] = ss[4] * gx + ss[5] * gy + ss[2] * gz;
          }
        }
        sc[0] = to_kt<KT>(T.c12 * s);
        sc[1] = to_kt<KT>(T.c44 * s);
        sc[2] = to_kt<KT>(T.a * s);
        // tangent vectors G_a and n.G_a in the tangent's precision (FP32 copy of G when present)
        KT n[6];
        for (int f = 0; f < 6; ++f) n[f] = to_kt<KT>(T.n[f]);
        for (int a = 0; a < NN; ++a) {
          KT gx, gy, gz;
          if constexpr (FF) {
            gx = Gf[0][a].h;
            gy = Gf[1][a].h;
            gz = Gf[2 % DIM][a].h;
          } else if (std::is_same<KT, float>::value && g.geomG32) {
            gx = (KT)g.geomG32[(int64_t)(0 * NN + a) * stride + pt];
            gy = (KT)g.geomG32[(int64_t)(1 * NN + a) * stride + pt];
            gz = (KT)g.geomG32[(int64_t)(2 * NN + a) * stride + pt];
          } else {
            gx = (KT)Gm[0][a];
            gy = (KT)Gm[1][a];
            gz = (KT)Gm[2 % DIM][a];
          }
          KT* v = vq + a * NVEC * DIM;
          v[0] = gx;
          v[1] = gy;
          v[2 % DIM] = gz;
          v[DIM + 0] = n[0] * gx + n[3] * gy + n[4] * gz;
          v[DIM + 1] = n[3] * gx + n[1] * gy + n[5] * gz;
          v[DIM + 2 % DIM] = n[4] * gx + n[5] * gy + n[2] * gz;
        }
      } else {
        Tangent2 C;
        if (g.plane == EFE_PLANE_STRESS) {
          if (g.material == EFE_MAT_VON_MISES)
            ok = von_mises_plane_stress<FASTRM>(smc[le], sig, de, kappa, C);
          else
            linear_elastic_plane_stress(props, sig, de, C);
        } else {
          Tangent3 T;
          if (g.material == EFE_MAT_VON_MISES)
            ok = von_mises_3d<FASTRM>(smc[le], sig, de, kappa, T);
          else
            linear_elastic_3d(smc[le], sig, de, T);
          tangent2_from3(T, C);
        }
        for (int a = 0; a < NN; ++a) {
          const double gx = Gm[0][a], gy = Gm[1 % DIM][a];
          rq[a * DIM + 0] = (sig[0] * gx + sig[3] * gy) * s;
          rq[a * DIM + 1 % DIM] = (sig[3] * gx + sig[1] * gy) * s;
          KT* v = vq + a * NVEC * DIM;
          v[0] = (KT)gx;
          v[1 % DIM] = (KT)gy;
        }
        for (int k = 0; k < 6; ++k) sc[k] = (KT)(C.c[k] * s);
      }
      for (int f = 0; f < 6; ++f) eps[f] += de[f];
    } else {
      // ------------------------------------------------ total Lagrangian (displacementtlelement/element.py:346-427)
      double F[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
      for (int i = 0; i < DIM; ++i)
        for (int j = 0; j < DIM; ++j) {
          double h = 0.0;
          for (int a = 0; a < NN; ++a) h += u[a * DIM + i] * Gm[j][a];
          F[i][j] += h;
        }
      // Green-Lagrange E = 1/2 (H + H^T + H^T H), H = F - I  (:386)
      double Eg[3][3];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double hh = 0.0;
          for (int k = 0; k < DIM; ++k) hh += (F[k][i] - (k == i)) * (F[k][j] - (k == j));
          Eg[i][j] = (i < DIM && j < DIM) ? 0.5 * ((F[i][j] - (i == j)) + (F[j][i] - (i == j)) + hh) : 0.0;
        }
      const double Ev[6] = {Eg[0][0], Eg[1][1], Eg[2][2], Eg[0][1], Eg[1][2], Eg[0][2]};
      for (int f = 0; f < 6; ++f) g.auxTemp[(int64_t)f * stride + pt] = Ev[f];
      double detF, iF[3][3];
      if constexpr (DIM == 2) {
        detF = F[0][0] * F[1][1] - F[0][1] * F[1][0];
        iF[0][0] = F[1][1] / detF;
        iF[0][1] = -F[0][1] / detF;
        iF[1][0] = -F[1][0] / detF;
        iF[1][1] = F[0][0] / detF;
        iF[0][2] = iF[1][2] = iF[2][0] = iF[2][1] = 0.0;
        iF[2][2] = 1.0;
      } else {
        detF = det3(F);
        inv3(F, detF, iF);
      }
      {
        // hypoelastic material on the Green-Lagrange strain increment (:416-426)
        double de[6] = {0, 0, 0, 0, 0, 0};
        const double* Eo = g.auxRef;
        double Eold[6];
        for (int f = 0; f < 6; ++f) Eold[f] = Eo ? Eo[(int64_t)f * stride + pt] : 0.0;
        if constexpr (DIM == 3) {
          de[0] = Ev[0] - Eold[0];
          de[1] = Ev[1] - Eold[1];
          de[2] = Ev[2] - Eold[2];
          de[3] = (Ev[3] - Eold[3]) * 2.0;
          de[4] = (Ev[4] - Eold[4]) * 2.0;
          de[5] = (Ev[5] - Eold[5]) * 2.0;
        } else {
          de[0] = Ev[0] - Eold[0];
          de[1] = Ev[1] - Eold[1];
          de[3] = (Ev[3] - Eold[3]) * 2.0;
        }
        if constexpr (FORM == TLV3) {
          Tangent3 T;
          if (g.material == EFE_MAT_VON_MISES)
            ok = von_mises_3d<FASTRM>(smc[le], sig, de, kappa, T);
          else
            linear_elastic_3d(smc[le], sig, de, T);
          // TL Voigt order 11,22,33,12,23,13
          const double Sm[3][3] = {{sig[0], sig[3], sig[5]}, {sig[3], sig[1], sig[4]}, {sig[5], sig[4], sig[2]}};
          const double Nm[3][3] = {{T.n[0], T.n[3], T.n[5]}, {T.n[3], T.n[1], T.n[4]}, {T.n[5], T.n[4], T.n[2]}};
          sc[0] = (KT)(T.c12 * s);
          sc[1] = (KT)(T.c44 * s);
          sc[2] = (KT)(T.a * s);
          int k = 3;
          for (int i = 0; i < 3; ++i)
            for (int j = i; j < 3; ++j) sc[k++] = (KT)(F[i][0] * F[j][0] + F[i][1] * F[j][1] + F[i][2] * F[j][2]);
          for (int a = 0; a < NN; ++a) {
            double SG[3], NG[3];
            for (int i = 0; i < 3; ++i) {
              SG[i] = Sm[i][0] * Gm[0][a] + Sm[i][1] * Gm[1][a] + Sm[i][2] * Gm[2 % DIM][a];
              NG[i] = Nm[i][0] * Gm[0][a] + Nm[i][1] * Gm[1][a] + Nm[i][2] * Gm[2 % DIM][a];
            }
            KT* v = vq + a * NVEC * DIM;
            for (int c = 0; c < 3; ++c) {
              const double fsg = F[c][0] * SG[0] + F[c][1] * SG[1] + F[c][2] * SG[2];
              rq[a * DIM + c % DIM] = fsg * s;  // B0^T sigma = F sigma dN/dX
              v[0 * DIM + c % DIM] = (KT)Gm[c % DIM][a];
              v[1 * DIM + c % DIM] = (KT)(F[c][0] * Gm[0][a] + F[c][1] * Gm[1][a] + F[c][2] * Gm[2 % DIM][a]);
              v[2 * DIM + c % DIM] = (KT)(F[c][0] * NG[0] + F[c][1] * NG[1] + F[c][2] * NG[2]);
              v[3 * DIM + c % DIM] = (KT)(SG[c] * s);
            }
          }
        } else {  // TLV2
          Tangent2 C;
          if (g.plane == EFE_PLANE_STRESS) {
            if (g.material == EFE_MAT_VON_MISES)
              ok = von_mises_plane_stress<FASTRM>(smc[le], sig, de, kappa, C);
            else
              linear_elastic_plane_stress(props, sig, de, C);
          } else {
            Tangent3 T;
            if (g.material == EFE_MAT_VON_MISES)
              ok = von_mises_3d<FASTRM>(smc[le], sig, de, kappa, T);
            else
              linear_elastic_3d(smc[le], sig, de, T);
            tangent2_from3(T, C);
          }
          // stress entering P: indices [0,1,3] (plane strain) or [0,1,2] (plane stress, :278-281);
          // Hgeo always reads undoVoigtStress(2, stress) = [[s0, s2], [s2, s1]] (element.py:48-73)
          const double s12p = (g.plane == EFE_PLANE_STRESS) ? sig[2] : sig[3];
          const double Sp[2][2] = {{sig[0], s12p}, {s12p, sig[1]}};
          const double Sg[2][2] = {{sig[0], sig[2]}, {sig[2], sig[1]}};
          for (int k = 0; k < 6; ++k) sc[k] = (KT)(C.c[k] * s);
          sc[6] = (KT)F[0][0];
          sc[7] = (KT)F[0][1];
          sc[8] = (KT)F[1][0];
          sc[9] = (KT)F[1][1];
          for (int a = 0; a < NN; ++a) {
            const double gx = Gm[0][a], gy = Gm[1 % DIM][a];
            const double spx = Sp[0][0] * gx + Sp[0][1] * gy, spy = Sp[1][0] * gx + Sp[1][1] * gy;
            rq[a * DIM + 0] = (F[0][0] * spx + F[0][1] * spy) * s;
            rq[a * DIM + 1 % DIM] = (F[1][0] * spx + F[1][1] * spy) * s;
            KT* v = vq + a * NVEC * DIM;
            v[0] = (KT)gx;
            v[1 % DIM] = (KT)gy;
            v[DIM + 0] = (KT)((Sg[0][0] * gx + Sg[0][1] * gy) * s);
            v[DIM + 1 % DIM] = (KT)((Sg[1][0] * gx + Sg[1][1] * gy) * s);
          }
        }
        for (int f = 0; f < 6; ++f) eps[f] += de[f];
      }
    }
    // ---- state write (stateTemp = updated copy of stateRef)
    for (int f = 0; f < 6; ++f) {
      g.stateTemp[(int64_t)f * stride + pt] = sig[f];
      g.stateTemp[(int64_t)(6 + f) * stride + pt] = eps[f];
    }
    if (hasM) g.stateTemp[(int64_t)12 * stride + pt] = kappa;
    bool finite = true;
    for (int f = 0; f < 6; ++f) finite = finite && finite_bits(sig[f]);
    if (!ok) report(g.status, EFE_STATUS_CUTBACK, g.elementOffset + e, 1);
    if (!finite) atomicOr(g.status, EFE_STATUS_NONFINITE);
  }
  }
  __syncthreads();

  // ---- phase C: residual and flux
  for (int t = threadIdx.x; t < EPB * NDOF; t += NT) {
    const int le = t / NDOF, k = t % NDOF;
    const int64_t e = e0 + le;
    if (e >= nEl) continue;
    double pe = 0.0;
    if constexpr (FF) {
      const ff* rf = reinterpret_cast<const ff*>(sr);
      ff acc{0, 0};
      for (int q = 0; q < NQ; ++q) ff_add(acc, rf[(le * NQ + q) * L::SR + k]);
      pe = -ff_to_double_bits(acc);
    } else {
      for (int q = 0; q < NQ; ++q) pe -= sr[(le * NQ + q) * L::SR + k];
    }
    const int a = k / DIM, c = k % DIM;
    const int32_t node = g.conn[e * NN + a];
    if (!in_bounds(g, node, g.nNodes, e)) continue;
    const int32_t dof = g.nodeDof[node] + c;
    if (!in_bounds(g, dof, g.nDof, e)) continue;
    atomicAdd(g.P + dof, pe);
    atomicAdd(g.F + dof, fabs(pe));
  }

  // ---- phase B: tangent blocks
  KT* K = reinterpret_cast<KT*>(g.Kdata);
  // the element tangents are symmetric (K_ab[j][k] = K_ba[k][j]): evaluate the pairs a <= b and
  // scatter each block twice
  constexpr int NPAIR = NN * (NN + 1) / 2;
  for (int t = threadIdx.x; t < EPB * NPAIR; t += NT) {
    const int le = t / NPAIR;
    int r = t % NPAIR, a = 0;
    while (r >= NN - a) {
      r -= NN - a;
      ++a;
    }
    const int b = a + r;
    const int64_t e = e0 + le;
    if (e >= nEl) continue;
    KT acc[DIM][DIM];
#pragma unroll
    for (int j = 0; j < DIM; ++j)
#pragma unroll
      for (int k = 0; k < DIM; ++k) acc[j][k] = KT(0);
    for (int q = 0; q < NQ; ++q) {
      const KT* sc = ssc + (le * NQ + q) * L::SC;
      const KT* va = sv + (size_t)(le * NQ + q) * L::SV + a * NVEC * DIM;
      const KT* vb = sv + (size_t)(le * NQ + q) * L::SV + b * NVEC * DIM;
      if constexpr (FORM == SS3) {
        const KT Lq = sc[0], Mq = sc[1], Aq = sc[2];
        const KT dot = va[0] * vb[0] + va[1] * vb[1] + va[2 % DIM] * vb[2 % DIM];
#pragma unroll
        for (int j = 0; j < DIM; ++j)
#pragma unroll
          for (int k = 0; k < DIM; ++k)
            acc[j][k] += Lq * va[j] * vb[k] + Mq * ((j == k ? dot : KT(0)) + va[k] * vb[j]) -
                         Aq * va[DIM + j] * vb[DIM + k];
      } else if constexpr (FORM == SS2) {
        // B columns (11,22,12): (a,0) = [gx, 0, gy], (a,1) = [0, gy, gx]
        const KT c00 = sc[0], c01 = sc[1], c02 = sc[2], c11 = sc[3], c12 = sc[4], c22 = sc[5];
        const KT ax = va[0], ay = va[1 % DIM], bx = vb[0], by = vb[1 % DIM];
        // C * Bcol_b0 = C[:,0] bx + C[:,2] by ; C * Bcol_b1 = C[:,1] by + C[:,2] bx
        const KT cb0[3] = {c00 * bx + c02 * by, c01 * bx + c12 * by, c02 * bx + c22 * by};
        const KT cb1[3] = {c01 * by + c02 * bx, c11 * by + c12 * bx, c12 * by + c22 * bx};
        acc[0][0] += ax * cb0[0] + ay * cb0[2];
        acc[0][1 % DIM] += ax * cb1[0] + ay * cb1[2];
        acc[1 % DIM][0] += ay * cb0[1] + ax * cb0[2];
        acc[1 % DIM][1 % DIM] += ay * cb1[1] + ax * cb1[2];
      } else if constexpr (FORM == TLH) {
        const KT c1s = sc[0], c4s = sc[1];
        const KT* Ga = va;
        const KT* Gb = vb;
        const KT* ha = va + DIM;
        const KT* hb = vb + DIM;
        const KT* gb = vb + 2 * DIM;
        const KT* pb = vb + 3 * DIM;
        const KT* qa = va + 4 * DIM;
        KT dot = KT(0);
#pragma unroll
        for (int i = 0; i < DIM; ++i) dot += Ga[i] * Gb[i];
#pragma unroll
        for (int j = 0; j < DIM; ++j)
#pragma unroll
          for (int k = 0; k < DIM; ++k)
            acc[j][k] += pb[j] * ha[k] + qa[j] * hb[k] + c4s * ha[j] * gb[k] + (j == k ? c1s * dot : KT(0));
      } else if constexpr (FORM == TLV3) {
        const KT Lq = sc[0], Mq = sc[1], Aq = sc[2];
        const KT Fm[3][3] = {{sc[3], sc[4], sc[5]}, {sc[4], sc[6], sc[7]}, {sc[5], sc[7], sc[8]}};
        const KT* Ga = va;
        const KT* Gb = vb;
        const KT* ga = va + DIM;
        const KT* gb = vb + DIM;
        const KT* wa = va + 2 * DIM;
        const KT* wb = vb + 2 * DIM;
        const KT* ta = va + 3 * DIM;
        KT dot = KT(0), geo = KT(0);
#pragma unroll
        for (int i = 0; i < DIM; ++i) {
          dot += Ga[i] * Gb[i];
          geo += ta[i] * Gb[i];
        }
#pragma unroll
        for (int c = 0; c < DIM; ++c)
#pragma unroll
          for (int d = 0; d < DIM; ++d)
            acc[c][d] += Lq * ga[c] * gb[d] + Mq * (Fm[c][d] * dot + gb[c] * ga[d]) - Aq * wa[c] * wb[d] +
                         (c == d ? geo : KT(0));
      } else {  // TLV2
        const KT* C = sc;
        const KT F00 = sc[6], F01 = sc[7], F10 = sc[8], F11 = sc[9];
        const KT ax = va[0], ay = va[1 % DIM], bx = vb[0], by = vb[1 % DIM];
        const KT geo = va[DIM + 0] * bx + va[DIM + 1 % DIM] * by;
        // B0 columns: (a,c) = [ax F_c0, ay F_c1, ax F_c1 + ay F_c0]
        KT Ba[2][3], Bb[2][3];
        const KT Fr[2][2] = {{F00, F01}, {F10, F11}};
        for (int c = 0; c < 2; ++c) {
          Ba[c][0] = ax * Fr[c][0];
          Ba[c][1] = ay * Fr[c][1];
          Ba[c][2] = ax * Fr[c][1] + ay * Fr[c][0];
          Bb[c][0] = bx * Fr[c][0];
          Bb[c][1] = by * Fr[c][1];
          Bb[c][2] = bx * Fr[c][1] + by * Fr[c][0];
        }
        const KT Cm[3][3] = {{C[0], C[1], C[2]}, {C[1], C[3], C[4]}, {C[2], C[4], C[5]}};
        for (int d = 0; d < 2; ++d) {
          KT cb[3];
          for (int i = 0; i < 3; ++i) cb[i] = Cm[i][0] * Bb[d][0] + Cm[i][1] * Bb[d][1] + Cm[i][2] * Bb[d][2];
          for (int c = 0; c < 2; ++c)
            acc[c % DIM][d % DIM] += Ba[c][0] * cb[0] + Ba[c][1] * cb[1] + Ba[c][2] * cb[2] + (c == d ? geo : KT(0));
        }
      }
    }
    // Ke[(a,j),(b,k)] -> CSR (row = dof(b,k), col = dof(a,j)) = slot(a,b) + k*rowLen(b) + j
    const int32_t slot = g.pairSlot[(e * NN + a) * NN + b];
    const int rl = srl[le * NN + b];
    // the block's entries are slot + k rl + j, j, k < DIM
    if (!in_bounds(g, slot, g.nnz, e) || !in_bounds(g, slot + (int64_t)(DIM - 1) * (rl + 1), g.nnz, e)) continue;
#pragma unroll
    for (int j = 0; j < DIM; ++j)
#pragma unroll
      for (int k = 0; k < DIM; ++k) kadd(K + slot + (int64_t)k * rl + j, acc[j][k]);
    if (a != b) {  // Ke[(b,k),(a,j)] = Ke[(a,j),(b,k)] -> (row = dof(a,j), col = dof(b,k))
      const int32_t slot2 = g.pairSlot[(e * NN + b) * NN + a];
      const int rl2 = srl[le * NN + a];
      if (!in_bounds(g, slot2, g.nnz, e) || !in_bounds(g, slot2 + (int64_t)(DIM - 1) * (rl2 + 1), g.nnz, e))
        continue;
#pragma unroll
      for (int j = 0; j < DIM; ++j)
#pragma unroll
        for (int k = 0; k < DIM; ++k) kadd(K + slot2 + (int64_t)j * rl2 + k, acc[j][k]);
    }
  }
}

template <int SHAPE, int RULE, int FORM, typename KT, int EPB, int NT, int MINB, bool FF = false>
__global__ void __launch_bounds__(NT, MINB) assemble_kernel(GroupArgs g) {
  extern __shared__ __align__(128) unsigned char smem[];
  assemble_tile<SHAPE, RULE, FORM, KT, EPB, NT, FF>(g, (int64_t)blockIdx.x * EPB, smem);
}

// Set-up and tear-down of the tensor-core state of a CTA (every thread calls both): the mbarrier
// of MMA completion, 64 TMEM columns (two 128 x 32 FP32 accumulators) allocated by warp 0; at the
// end, after a bounded wait for MMAs still in flight if a wait expired, warp 0 frees the columns.
}  // namespace efe

#include "efe_hexa20_tc.cuh"

namespace efe {

// Set-up and tear-down of the tensor-core state of a CTA (every thread calls both): the mbarrier
// of MMA completion and H20TC::TMEM_COLS TMEM columns allocated by warp 0; at the end, after a
// bounded wait for MMAs still in flight if a wait expired, warp 0 frees the columns.
__device__ __forceinline__ TCState tc_begin(uint64_t* mbar, uint32_t* slot) {
  if (threadIdx.x == 0) tc::mbar_init(mbar, 1);
  if (threadIdx.x < 32) tc::tmem_alloc(slot, H20TC::TMEM_COLS);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  return TCState{*slot, 0u, false, mbar};
}
__device__ __forceinline__ void tc_end(TCState& tcs) {
  if (tcs.failed) tc::mbar_wait(tcs.mbar, tcs.phase, TC_WAIT_LIMIT);
  tc::fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32) tc::tmem_dealloc(tcs.tmem, H20TC::TMEM_COLS);
}

// Tile variant 3, the Hexa20 3x3x3 pass (total-Lagrangian Neo-Hooke or small strain) with the
// tensor-core tangent (efe_hexa20_tc.cuh): a grid of resident CTAs (sms per wave), one element per tile, tiles strided by
// the grid; each CTA allocates its TMEM columns once and frees them at the end.  The CTAs of one
// wave share no SM, so the wave index picks the warp of the per-point update.  Each element's
// K_e scatter runs during the next element's material update (the last one after the loop).
template <bool FF, int FORM>
__global__ void __launch_bounds__(128, 3) assemble_kernel_tc(GroupArgs g, int sms) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t slot;
  TCState tcs = tc_begin(&mbar, &slot);
  int rot = (int)(blockIdx.x / (unsigned)sms), par = 0;
  int64_t prev = H20TC_DEFER_NONE;  // the element whose K_e is pending in shared memory
  for (int64_t e = blockIdx.x; e < g.nElements; e += gridDim.x, ++rot, par ^= 1) {
    const int64_t next = e + gridDim.x < g.nElements ? e + gridDim.x : -1;
    assemble_tile_h20tc<FF, FORM>(g, e, smem, tcs, rot, prev, next, prev >= 0, par);
    prev = e;
    __syncthreads();
  }
  if (prev >= 0 && !tcs.failed) {
    using L = H20TCLayout<FF>;
    h20tc_scatter(g, prev, smem + L::tc_off, reinterpret_cast<const int*>(smem + L::ps_off) + (par ^ 1) * H20TC::NN * H20TC::NN,
                 reinterpret_cast<const int*>(smem + L::rl_off) + (par ^ 1) * H20TC::NN, threadIdx.x, 128);
  }
  tc_end(tcs);
}

// Groups of one element type for the persistent pass: group k owns the tiles
// [tileStart[k], tileStart[k+1]) of its type.  Passed by value (kernel parameters).
constexpr int MAX_PERSISTENT_GROUPS = EFE_PERSISTENT_MAX_GROUPS;
// The element types of the persistent pass, heaviest first: index of (shape, rule, form) or -1.
constexpr int PERSISTENT_NTYPES = 5;
__host__ __device__ inline int persistent_type_index(int shape, int rule, int form) {
  if (shape == EFE_HEXA20 && rule == EFE_RULE_3D_3X3X3 && form == TLH) return 0;
  if (shape == EFE_HEXA20 && rule == EFE_RULE_3D_3X3X3 && form == SS3) return 1;
  if (shape == EFE_HEXA8 && rule == EFE_RULE_3D_2X2X2 && form == TLH) return 2;
  if (shape == EFE_HEXA8 && rule == EFE_RULE_3D_2X2X2 && form == SS3) return 3;
  if (shape == EFE_QUAD8 && rule == EFE_RULE_2D_2X2 && form == TLH) return 4;
  return -1;
}
struct GroupTable {
  GroupArgs g[MAX_PERSISTENT_GROUPS];
  int64_t tileStart[MAX_PERSISTENT_GROUPS + 1];
  int n;
};

// One element type of the persistent pass: shape, quadrature rule, form, elements per tile and
// whether its tangent runs on the tensor cores.
template <int SHAPE_, int RULE_, int FORM_, int EPB_, bool TC_ = false>
struct PersistentType {
  static constexpr int SHAPE = SHAPE_, RULE = RULE_, FORM = FORM_, EPB = EPB_;
  static constexpr bool TC = TC_;
};

// The group tables of every type of one persistent launch (kernel parameters).
template <int N>
struct GroupTables {
  GroupTable t[N];
};

// Run tile t of the concatenated tile ranges of types I, I+1, ... (in the order of the type list) and
// return true, or return false when t lies past the last type's tiles.
template <typename KT, int NT, bool FF, int N, int I, typename T0, typename... Rest>
__device__ __forceinline__ bool persistent_tile(const GroupTables<N>& tabs, long long t, unsigned char* smem,
                                                TCState* tcs, int rot) {
  const GroupTable& tb = tabs.t[I];
  const long long tiles = tb.tileStart[tb.n];
  if (t < tiles) {
    int k = 0;
    while (t >= tb.tileStart[k + 1]) ++k;
    if constexpr (T0::TC)
      assemble_tile_h20tc<FF, T0::FORM>(tb.g[k], (int64_t)(t - tb.tileStart[k]), smem, *tcs, rot, H20TC_NOW, -1, false,
                                          0);
    else
      assemble_tile<T0::SHAPE, T0::RULE, T0::FORM, KT, T0::EPB, NT, FF>(tb.g[k], (int64_t)(t - tb.tileStart[k]) * T0::EPB,
                                                                        smem);
    return true;
  }
  if constexpr (sizeof...(Rest) > 0)
    return persistent_tile<KT, NT, FF, N, I + 1, Rest...>(tabs, t - tiles, smem, tcs, rot);
  else
    return false;
}

// Persistent form: a grid sized to the resident CTAs pulls tiles from one work counter (scratch,
// zeroed before the launch) over up to MAX_PERSISTENT_GROUPS groups of each element type of the
// list, the types in list order (the heaviest first), until all are done.  MINB: resident CTAs per SM
// the register budget is held to.  FF: the float-float forms (mixed-ff) of the types that have one.
template <typename KT, int NT, int MINB, bool FF, typename CT, typename... Types>
__global__ void __launch_bounds__(NT, MINB)
    assemble_persistent_kernel(GroupTables<sizeof...(Types)> tabs, CT* counter, int sms) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ long long tile;
  constexpr bool anyTC = (Types::TC || ...);
  __shared__ uint64_t mbar;
  __shared__ uint32_t slot;
  TCState tcs{};
  if constexpr (anyTC) tcs = tc_begin(&mbar, &slot);
  while (true) {
    if (threadIdx.x == 0) tile = (long long)atomicAdd(counter, (CT)1);
    __syncthreads();
    const long long t = tile;
    __syncthreads();
    if (!persistent_tile<KT, NT, FF, (int)sizeof...(Types), 0, Types...>(tabs, t, smem, &tcs,
                                                                         (int)(blockIdx.x / (unsigned)sms + t)))
      break;
    __syncthreads();
  }
  if constexpr (anyTC) tc_end(tcs);
}

}  // namespace efe
