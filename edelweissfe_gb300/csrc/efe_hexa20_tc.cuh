// efe_hexa20_tc.cuh -- the Hexa20 3x3x3 element pass, total-Lagrangian Neo-Hooke or small strain
// (von Mises, linear elastic), with its element tangent on the tensor cores (tile variant 3): one
// element per 128-thread CTA tile.
//
// The small-strain tangent (displacementelement/element.py:342) has the same three kinds of terms
// as the one below, with G for h and g: lambda' G_a[j] G_b[k] - a (nG_a)[j] (nG_b)[k] plain,
// mu' G_b[j] G_a[k] swapped, mu' G_a . G_b on the node-pair diagonal.
// The tangent of the TL Neo-Hooke form (displacementtlelement/element.py:408-412 in closed form) is,
// with per-point scalars c1s..c4s and per-node vectors G = dN/dX, h = F^-T G, g = F G,
// p = c1s g - s tau h, q = c2s h + c3s B h,
//   K[(a,j),(b,k)] = sum_q  q_a[j] h_b[k] + c4s h_a[j] g_b[k]        (plain: j with a, k with b)
//                         + p_b[j] h_a[k]                            (swapped: j with b, k with a)
//                         + delta_jk c1s G_a . G_b                   (node-pair diagonal)
// Each of the three kinds is a plain matrix product over K = (point, factor) of per-node vectors:
//   P[(a,j),(b,k)] = sum_q [q_a[j], c4s h_a[j]] . [h_b[k], g_b[k]]       (60 x 60, K = 2 per point)
//   X[(b,j),(a,k)] = sum_q p_b[j] h_a[k]                                 (60 x 60, K = 1 per point)
//   D[a,b]         = sum_q sum_l (c1s G_a[l]) G_b[l]                     (20 x 20, K = 3 per point)
// and K[(a,j),(b,k)] = P[(a,j),(b,k)] + X[(b,j),(a,k)] + delta_jk D[a,b].
// P and X share their B operand [h | g] and run as ONE M = 128 MMA (rows 0-59 plain, rows 64-123
// swapped; the swapped rows' g-slots are zero), D as a second one.  The per-node vectors are the
// operands themselves: phase A2 writes them (TF32 hi/lo split, ~2^-22 per product with the
// hi*hi + hi*lo + lo*hi MMAs, FP32 accumulation in TMEM) straight into the operand tiles, in three
// chunks of 9 points; no element stiffness block is formed on the SIMT pipes.
//
// The element residual uses the first Piola-Kirchhoff form P_e[a][j] = -sum_q (s tau F^-T)_q[j] . G_qa
// (:402, :414), one thread per (node, component), in FP64 (mixed) or float-float (mixed-ff); F is
// formed as in the SIMT pass.  In the mixed-ff pass the kinematics of a point (E, F^-1, B, tau,
// s tau F^-T) are float-float on the FP32 pipe, spread over all threads, and only the Neo-Hooke
// scalars (logarithms, powers) stay FP64 on one warp: on this GPU the FP64 pipe costs the same per
// warp instruction whatever the number of active lanes, so that warp's instruction count sets the
// phase's length.
// Across the elements of a CTA: an element's dN/dX, pair slots and U are staged (cp.async and
// register loads) while the previous element's last MMAs and material update run, and its K_e
// scatter runs during the next element's material update.
#pragma once

namespace efe {

struct H20TC {
  static constexpr int NN = 20, NQ = 27, NDOF = 60, QC = 9, NCH = 3;
  static constexpr int RK = 44;  // floats per point of the FP32 record (16-byte rows)
  // FP32 record offsets: F, F^-1 (row-major, F^-1[l][m] at 3l+m), B = F F^T, Pq = s tau F^-T,
  // c1 s .. c4 s
  static constexpr int R_F = 0, R_FI = 9, R_B = 18, R_PQ = 27, R_C = 36;
  // operand tiles (K-major, no swizzle; element (r, k) at (r/8) SBO + (k/4) 128 + (r%8) 16 + (k%4) 4)
  static constexpr int KPS = 24;  // P/X operands: K = 2 per point, 18 used per chunk
  static constexpr int KD = 32;   // D operands: K = 3 per point, 27 used per chunk
  static constexpr int SBO_PS = KPS / 4 * 128, SBO_D = KD / 4 * 128;
  // tile byte offsets inside the tensor-core region: the M = 128 read of the D operand covers
  // 16 row groups (rows 24-127: the following tiles, results never read), its N = 32 read 4
  static constexpr size_t dA_hi = 0, dA_lo = dA_hi + 3 * SBO_D, dB_hi = dA_lo + 3 * SBO_D,
                          dB_lo = dB_hi + 3 * SBO_D, a_hi = dB_lo + 3 * SBO_D, a_lo = a_hi + 16 * SBO_PS,
                          b_hi = a_lo + 16 * SBO_PS, b_lo = b_hi + 8 * SBO_PS, tc_bytes = b_lo + 8 * SBO_PS;
  static_assert(dA_lo + 16 * SBO_D <= tc_bytes && dB_lo + 4 * SBO_D <= tc_bytes, "D reads stay in the region");
  // epilogue: the accumulators copied to shared memory over the (then idle) operand tiles
  static constexpr int SS = NDOF + 1;  // odd row stride
  static constexpr size_t sP = 0, sX = sP + sizeof(float) * NDOF * SS, sD = sX + sizeof(float) * NDOF * SS;
  static_assert(sD + sizeof(float) * NN * (NN + 1) <= tc_bytes, "epilogue copy fits the operand tiles");
  // float-float material phase (mixed-ff): per point E (6), cofactors (9) and B (6) as float-float
  // (A1a), then the point's scalars (A1b), in the operand region behind the epilogue copy (free
  // until the operand tiles are zeroed; the pending epilogue copy stays intact)
  static constexpr int NA1 = 21;
  struct A1Scalars {
    ff sB, sI, aF, aI, rJ;
    double energy;
    float c[4];
  };
  static constexpr size_t a1_off = 32768, a1s_off = a1_off + 8 * NQ * NA1;
  static_assert(a1_off >= sD + sizeof(float) * NN * (NN + 1) && a1s_off + sizeof(A1Scalars) * NQ <= tc_bytes,
                "material scratch between the epilogue copy and the end of the operand region");
  // TMEM columns: P/X accumulator at 0 (64 columns), D at 64 (32 columns)
  static constexpr uint32_t TMEM_COLS = 128, D_COL = 64;
};

template <bool FF>
struct H20TCLayout {
  using T = H20TC;
  static constexpr size_t u_off = 0;                                          // ff or double [NN][3]
  static constexpr size_t f_off = u_off + 8 * T::NN * 3;                      // double [NQ][9]: F
  static constexpr size_t pq_off = f_off + 8 * T::NQ * 9;                     // ff or double [NQ][9]: s tau F^-T
  static constexpr size_t rk_off = pq_off + 8 * T::NQ * 9;                    // float [NQ][RK]
  static_assert(rk_off % 16 == 0 && T::RK % 4 == 0, "16-byte record rows");
  // the element's dN/dX, [(l NN + a) NQ + q]: float-float hi and lo arrays (mixed-ff) or double
  // (mixed), staged by cp.async
  static constexpr size_t g_off = rk_off + sizeof(float) * T::NQ * T::RK;
  static constexpr size_t glo_off = g_off + sizeof(float) * T::NQ * T::NDOF;
  // pair slots and row lengths of two consecutive elements (the pending K_e and the current one)
  static constexpr size_t ps_off = g_off + 8 * T::NQ * T::NDOF;         // int [2][NN][NN]
  static constexpr size_t rl_off = ps_off + sizeof(int) * 2 * T::NN * T::NN;  // int [2][NN]
  static constexpr size_t mc_off = (rl_off + sizeof(int) * 2 * T::NN + 15) / 16 * 16;  // VMConst (small strain)
  // staged with dN/dX (cp.async): det J w t per point and the element's properties (at most 8)
  static constexpr size_t s_off = (mc_off + sizeof(VMConst) + 15) / 16 * 16;  // double [NQ]
  static constexpr size_t pr_off = s_off + 8 * T::NQ;                        // double [8]
  static constexpr int NPR = 8;
  // first DOF of each node of two consecutive elements (-1 where a bounds check failed), for the
  // element residual's atomics
  static constexpr size_t dof_off = pr_off + 8 * NPR;  // int [2][NN]
  static constexpr size_t tc_off = (dof_off + sizeof(int) * 2 * T::NN + 127) / 128 * 128;
  static constexpr size_t bytes = tc_off + T::tc_bytes;
};

// round to TF32 (10 fraction bits, to nearest with ties away from zero) for a finite FP32 value
__device__ __forceinline__ float tf32_rna(float x) { return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u); }

// byte offset of element (r, k) in an operand tile with row-group stride SBO
template <int SBO>
__device__ __forceinline__ uint32_t tc_off(int r, int k) {
  return (uint32_t)((r >> 3) * SBO + (k >> 2) * 128 + (r & 7) * 16 + (k & 3) * 4);
}
// x at (r, k) of the hi and lo tiles (lo = the TF32 rounding of x - hi)
template <int SBO>
__device__ __forceinline__ void tc_put(unsigned char* hi, unsigned char* lo, int r, int k, float x) {
  const float h = tf32_rna(x);
  const uint32_t o = tc_off<SBO>(r, k);
  *reinterpret_cast<float*>(hi + o) = h;
  *reinterpret_cast<float*>(lo + o) = tf32_rna(__fsub_rn(x, h));
}
// x at (r, k) and y at (r, k + 1), k even (one 8-byte store per tile)
template <int SBO>
__device__ __forceinline__ void tc_put2(unsigned char* hi, unsigned char* lo, int r, int k, float x, float y) {
  const float hx = tf32_rna(x), hy = tf32_rna(y);
  const uint32_t o = tc_off<SBO>(r, k);
  *reinterpret_cast<float2*>(hi + o) = make_float2(hx, hy);
  *reinterpret_cast<float2*>(lo + o) = make_float2(tf32_rna(__fsub_rn(x, hx)), tf32_rna(__fsub_rn(y, hy)));
}

// K_e of element e (the accumulators copied to the tile's shared memory by its epilogue) into the
// CSR data: Ke[(a,j),(b,k)] at row dof(b,k), column dof(a,j) = slot(a,b) + k rowLen(b) + j, with the
// element's staged pair slots sps and row lengths srl, by threads ti = 0 .. nth - 1.
__device__ __forceinline__ void h20tc_scatter(const GroupArgs& g, int64_t e, const unsigned char* tb, const int* sps,
                                             const int* srl, int ti, int nth) {
  using T = H20TC;
  constexpr int NN = T::NN;
  const float* sP = reinterpret_cast<const float*>(tb + T::sP);
  const float* sX = reinterpret_cast<const float*>(tb + T::sX);
  const float* sD = reinterpret_cast<const float*>(tb + T::sD);
  float* K = reinterpret_cast<float*>(g.Kdata);
  // one thread per (b, k, a): the three contiguous columns j = 0, 1, 2 of node a in CSR row (b, k)
  for (int t = ti; t < T::NDOF * NN; t += nth) {
    const int bk = t / NN, a = t - bk * NN, b = bk / 3, k = bk - 3 * b;
    const int64_t pos = (int64_t)sps[a * NN + b] + (int64_t)k * srl[b];
    if (!in_bounds(g, pos, g.nnz - 2, e)) continue;
    const float d = sD[a * (NN + 1) + b];  // on the column j = k
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const float v = sP[(3 * a + j) * T::SS + 3 * b + k] + sX[(3 * b + j) * T::SS + 3 * a + k];
      atomicAdd(K + pos + j, j == k ? v + d : v);
    }
  }
}

// Stage element e into shared memory, in two parts that complete after tc::cp_async_wait_all:
// h20tc_stage_g (every thread): dN/dX, det J w t and the properties by cp.async; h20tc_stage_small
// (threads li = 0 .. nth - 1, nth >= NN): the pair slots by cp.async into buffer par, U, the row
// lengths and the node DOFs by plain loads.
template <bool FF>
__device__ __forceinline__ void h20tc_stage_g(const GroupArgs& g, int64_t e, unsigned char* smem) {
  using T = H20TC;
  using L = H20TCLayout<FF>;
  constexpr int NT = 128, NQ = T::NQ;
  const int64_t stride = g.nElements * NQ;
  for (int t = threadIdx.x; t < T::NDOF * NQ; t += NT) {
    const int la = t / NQ, q = t - la * NQ;
    const int64_t gi = (int64_t)la * stride + e * NQ + q;
    if constexpr (FF) {
      tc::cp_async4(reinterpret_cast<float*>(smem + L::g_off) + t, g.geomG32 + gi);
      tc::cp_async4(reinterpret_cast<float*>(smem + L::glo_off) + t, g.geomGlo + gi);
    } else {
      tc::cp_async8(reinterpret_cast<double*>(smem + L::g_off) + t, g.geomG + gi);
    }
  }
  if (threadIdx.x < NQ) tc::cp_async8(reinterpret_cast<double*>(smem + L::s_off) + threadIdx.x, g.geomS + e * NQ + threadIdx.x);
  if (threadIdx.x < g.nProps && threadIdx.x < L::NPR)
    tc::cp_async8(reinterpret_cast<double*>(smem + L::pr_off) + threadIdx.x, g.props + e * g.nProps + threadIdx.x);
}
// The small per-element data of h20tc_stage_small, loaded into registers first (so that the
// latency of the dependent loads can overlap other work) and stored later.
struct H20TCSmall {
  int32_t rowLen, dof;
  double u[3];
  bool valid;
};
template <bool FF, int FORM>
__device__ __forceinline__ H20TCSmall h20tc_load_small(const GroupArgs& g, int64_t e, int a) {
  constexpr int NN = H20TC::NN, DIM = 3;
  const double* Ux = FORM == SS3 ? g.dU : g.U;  // small strain: the increment; TL: the total
  H20TCSmall r{0, -1, {0.0, 0.0, 0.0}, false};
  const int32_t node = g.conn[e * NN + a];
  if (!in_bounds(g, node, g.nNodes, e)) return r;
  r.rowLen = g.nodeRowLen[node];
  const int32_t dof = g.nodeDof[node];
  if (!in_bounds(g, dof, g.nDof - DIM + 1, e)) return r;
  r.valid = true;
  r.dof = dof;
  if constexpr (FF) {
    // displacement relative to node 0 (sum_a dN_a/dX = 0): no cancellation in F
    const int32_t node0 = g.conn[e * NN];
    const int32_t dof0 = in_bounds(g, node0, g.nNodes, e) ? g.nodeDof[node0] : dof;
    const int32_t d0 = in_bounds(g, dof0, g.nDof - DIM + 1, e) ? dof0 : dof;
    for (int c = 0; c < DIM; ++c) r.u[c] = Ux[dof + c] - Ux[d0 + c];
  } else {
    for (int c = 0; c < DIM; ++c) r.u[c] = Ux[dof + c];
  }
  return r;
}
template <bool FF>
__device__ __forceinline__ void h20tc_store_small(const H20TCSmall& r, unsigned char* smem, int par, int a) {
  using L = H20TCLayout<FF>;
  constexpr int NN = H20TC::NN, DIM = 3;
  reinterpret_cast<int*>(smem + L::rl_off)[par * NN + a] = r.rowLen;
  reinterpret_cast<int*>(smem + L::dof_off)[par * NN + a] = r.valid ? r.dof : -1;
  if (!r.valid) return;
  for (int c = 0; c < DIM; ++c) {
    if constexpr (FF)
      reinterpret_cast<ff*>(smem + L::u_off)[a * DIM + c] = ff_split_bits(r.u[c]);
    else
      reinterpret_cast<double*>(smem + L::u_off)[a * DIM + c] = r.u[c];
  }
}
template <bool FF, int FORM>
__device__ __forceinline__ void h20tc_stage_small(const GroupArgs& g, int64_t e, unsigned char* smem, int par, int li,
                                                 int nth) {
  using L = H20TCLayout<FF>;
  constexpr int NN = H20TC::NN;
  int* sps = reinterpret_cast<int*>(smem + L::ps_off) + par * NN * NN;
  for (int t = li; t < NN * NN; t += nth) tc::cp_async4(sps + t, g.pairSlot + e * NN * NN + t);
  if (li < NN) h20tc_store_small<FF>(h20tc_load_small<FF, FORM>(g, e, li), smem, par, li);
}

// the float-float forms used by the per-point update of the mixed-ff pass
__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.h, -a.l}; }
__device__ __forceinline__ ff ff_sum(ff a, ff b) {
  ff r = a;
  ff_add(r, b);
  return r;
}
// a * b - c * d
__device__ __forceinline__ ff ff_det2(ff a, ff b, ff c, ff d) {
  ff r = ff_mul(a, b);
  ff_fma(r, ff_neg(c), d);
  return r;
}

// The three warps beside the material warp in phase A1 (li = 0 .. 95): load the next element's
// U and row lengths into registers, scatter the pending K_e of element prev (its pair slots and
// row lengths in buffer par ^ 1, U of this element already consumed), then -- once all three
// warps are past the scatter -- store the next element's small data into buffer par ^ 1.
template <bool FF, int FORM>
__device__ __forceinline__ void h20tc_pending_and_next(const GroupArgs& g, int64_t prev, int64_t next, unsigned char* smem,
                                                      const unsigned char* tb, const int* sps, const int* srl, int par,
                                                      int li, bool failed) {
  using L = H20TCLayout<FF>;
  constexpr int NN = H20TC::NN, NTH = 96;
  H20TCSmall nx{0, -1, {0.0, 0.0, 0.0}, false};
  if (next >= 0 && li < NN) nx = h20tc_load_small<FF, FORM>(g, next, li);
  if (prev >= 0 && !failed) h20tc_scatter(g, prev, tb, sps + (par ^ 1) * NN * NN, srl + (par ^ 1) * NN, li, NTH);
  if (next >= 0) {
    asm volatile("bar.sync 1, %0;" ::"n"(NTH) : "memory");
    int* nps = reinterpret_cast<int*>(smem + L::ps_off) + (par ^ 1) * NN * NN;
    for (int t = li; t < NN * NN; t += NTH) tc::cp_async4(nps + t, g.pairSlot + next * NN * NN + t);
    if (li < NN) h20tc_store_small<FF>(nx, smem, par ^ 1, li);
  }
}

// how a tile call scatters K_e (the prev argument of assemble_tile_h20tc)
constexpr int64_t H20TC_DEFER_NONE = -1;  // defer this element's K_e; nothing pending from before
constexpr int64_t H20TC_NOW = -2;         // scatter this element's K_e at the end of the call

// One element e of group g; every thread of the CTA (NT = 128) calls it.  tcs: the CTA's TMEM
// columns (H20TC::TMEM_COLS) and MMA-completion mbarrier.  rot (0-3): the warp that runs the
// per-point material update; warp w of every CTA sits on the same SM sub-partition, so the caller
// varies rot between the CTAs that share an SM.  par: the pair-slot buffer of this element
// (alternate between consecutive calls).
// prev == H20TC_NOW: K_e is scattered at the end of the call.  Otherwise K_e stays pending in shared
// memory, and prev >= 0 is the previous call's pending element (same group), scattered by the
// three other warps while one warp runs this element's material update; after the last call the
// caller scatters the pending one (h20tc_scatter).  next >= 0: the element of the next call, staged
// while this element's last MMAs run; staged: this element was staged that way by the previous call.
template <bool FF, int FORM>
__device__ __forceinline__ void assemble_tile_h20tc(const GroupArgs& g, const int64_t e, unsigned char* smem,
                                                      TCState& tcs, int rot, int64_t prev, int64_t next, bool staged,
                                                      int par) {
  using T = H20TC;
  using L = H20TCLayout<FF>;
  constexpr int NT = 128, NN = T::NN, NQ = T::NQ, DIM = 3;
  const int tid = threadIdx.x;
  const int rt = (tid - 32 * (rot & 3)) & (NT - 1);  // thread index with warp rot first
  double* sF = reinterpret_cast<double*>(smem + L::f_off);
  float* rk = reinterpret_cast<float*>(smem + L::rk_off);
  // staged dN/dX: FF hi / lo floats, else doubles
  float* sGh = reinterpret_cast<float*>(smem + L::g_off);
  float* sGl = reinterpret_cast<float*>(smem + L::glo_off);
  double* sGd = reinterpret_cast<double*>(smem + L::g_off);
  int* sps = reinterpret_cast<int*>(smem + L::ps_off);
  int* srl = reinterpret_cast<int*>(smem + L::rl_off);
  unsigned char* tb = smem + L::tc_off;
  const int64_t stride = g.nElements * NQ;

  // ---- phase 0: this element's dN/dX, pair slots, U and row lengths in shared memory
  if (!staged) {
    h20tc_stage_g<FF>(g, e, smem);
    h20tc_stage_small<FF, FORM>(g, e, smem, par, rt, NT);
  }
  tc::cp_async_wait_all();
  __syncthreads();
  const double* sS = reinterpret_cast<const double*>(smem + L::s_off);    // det J w t per point
  const double* sPr = reinterpret_cast<const double*>(smem + L::pr_off);  // the element's properties
  // small strain: the element's von Mises / elasticity constants, once per element (read in A1)
  if (FORM == SS3 && tid == NT - 1)
    *reinterpret_cast<VMConst*>(smem + L::mc_off) = vm_const(sPr, g.material == EFE_MAT_VON_MISES);

  // ---- A0: H = sum_a U_a (x) dN_a/dX (U: the increment dU for small strain), one thread per
  // (point, component); the mixed TL pass keeps F = I + H, the others H
  for (int t = tid; t < NQ * 9; t += NT) {
    const int c = t / NQ, q = t - c * NQ, i = c / 3, j = c - 3 * i;
    const int g0 = j * NN * NQ + q;
    if constexpr (FF) {
      const ff* uf = reinterpret_cast<const ff*>(smem + L::u_off);
      ff acc{0, 0};
      for (int a = 0; a < NN; ++a) ff_fma(acc, uf[a * DIM + i], ff{sGh[g0 + a * NQ], sGl[g0 + a * NQ]});
      reinterpret_cast<ff*>(sF)[q * 9 + i * 3 + j] = acc;
    } else {
      const double* u = reinterpret_cast<const double*>(smem + L::u_off);
      double h = 0.0;
      for (int a = 0; a < NN; ++a) h += u[a * DIM + i] * sGd[g0 + a * NQ];
      sF[q * 9 + i * 3 + j] = ((FORM == TLH && i == j) ? 1.0 : 0.0) + h;
    }
  }
  __syncthreads();

  // ---- A1: the material points.  Warp rot runs the per-point FP64 part (all of it for small strain
  // and in the mixed TL pass; in the mixed-ff TL pass only the Neo-Hooke scalars, between two
  // float-float sub-phases that use every thread); meanwhile the other warps scatter the pending
  // K_e of the previous element.
  if constexpr (FORM == SS3) {
    // small strain (displacementelement/element.py:318-346): strain increment, von Mises return
    // map or elasticity (FP64), state, s sigma for the residual, the FP32 tangent record
    if (rt < 32) {
      if (rt < NQ) {
        const int q = rt;
        const int64_t pt = e * NQ + q;
        const VMConst& mc = *reinterpret_cast<const VMConst*>(smem + L::mc_off);
        // de = sym(H), Voigt 11, 22, 33, 12, 13, 23 with engineering shears (element.py:322)
        double de[6];
        if constexpr (FF) {
          const ff* H = reinterpret_cast<const ff*>(sF) + q * 9;
          de[0] = ff_to_double_bits(H[0]);
          de[1] = ff_to_double_bits(H[4]);
          de[2] = ff_to_double_bits(H[8]);
          de[3] = ff_to_double_bits(ff_sum(H[1], H[3]));
          de[4] = ff_to_double_bits(ff_sum(H[2], H[6]));
          de[5] = ff_to_double_bits(ff_sum(H[5], H[7]));
        } else {
          const double* H = sF + q * 9;
          de[0] = H[0];
          de[1] = H[4];
          de[2] = H[8];
          de[3] = H[1] + H[3];
          de[4] = H[2] + H[6];
          de[5] = H[5] + H[7];
        }
        double sig[6], eps[6], kappa = 0.0;
        for (int f = 0; f < 6; ++f) {
          sig[f] = g.stateRef[(int64_t)f * stride + pt];
          eps[f] = g.stateRef[(int64_t)(6 + f) * stride + pt];
        }
        const bool hasM = g.material != EFE_MAT_LINEAR_ELASTIC;
        if (hasM) kappa = g.stateRef[(int64_t)12 * stride + pt];
        Tangent3 Tg;
        bool ok = true;
        if (g.material == EFE_MAT_VON_MISES)
          ok = von_mises_3d<true>(mc, sig, de, kappa, Tg);
        else
          linear_elastic_3d(mc, sig, de, Tg);
        for (int f = 0; f < 6; ++f) {
          g.stateTemp[(int64_t)f * stride + pt] = sig[f];
          g.stateTemp[(int64_t)(6 + f) * stride + pt] = eps[f] + de[f];
        }
        if (hasM) g.stateTemp[(int64_t)12 * stride + pt] = kappa;
        bool finite = true;
        for (int f = 0; f < 6; ++f) finite = finite && finite_bits(sig[f]);
        if (!ok) report(g.status, EFE_STATUS_CUTBACK, g.elementOffset + e, 1);
        if (!finite) atomicOr(g.status, EFE_STATUS_NONFINITE);
        const double s = sS[q];
        // s sigma (rows 11 12 13 / 12 22 23 / 13 23 33) for the residual r_a = s sigma . G_a
        const double S3[9] = {sig[0], sig[3], sig[4], sig[3], sig[1], sig[5], sig[4], sig[5], sig[2]};
        const double N3[9] = {Tg.n[0], Tg.n[3], Tg.n[4], Tg.n[3], Tg.n[1], Tg.n[5], Tg.n[4], Tg.n[5], Tg.n[2]};
        float* r = rk + q * T::RK;
        for (int c = 0; c < 9; ++c) {
          const double pq = s * S3[c];
          if constexpr (FF)
            reinterpret_cast<ff*>(smem + L::pq_off)[q * 9 + c] = ff_split_bits(pq);
          else
            reinterpret_cast<double*>(smem + L::pq_off)[q * 9 + c] = pq;
          r[T::R_F + c] = d2f_trunc(N3[c]);
        }
        // tangent lambda' G (x) G + mu' (delta G.G + G (x) G swapped) - a (nG) (x) (nG), times s
        r[T::R_C + 0] = d2f_trunc(Tg.c12 * s);
        r[T::R_C + 1] = d2f_trunc(Tg.c44 * s);
        r[T::R_C + 2] = d2f_trunc(Tg.a * s);
      }
    } else {
      h20tc_pending_and_next<FF, FORM>(g, prev, next, smem, tb, sps, srl, par, rt - 32, tcs.failed);
    }
  } else if constexpr (FF) {
    const ff* sH = reinterpret_cast<const ff*>(sF);
    ff* sA1 = reinterpret_cast<ff*>(tb + T::a1_off);  // [q][E 0-5 | C 6-14 | B 15-20]
    T::A1Scalars* sSc = reinterpret_cast<T::A1Scalars*>(tb + T::a1s_off);
    // Voigt entry v (11, 22, 33, 12, 23, 13) -> (i, j)
    auto vi = [](int v) { return v < 3 ? v : (v == 4 ? 1 : 0); };
    auto vj = [](int v) { return v < 3 ? v : (v == 3 ? 1 : 2); };
    // A1a: one thread per (point, entry): E = 1/2 (H + H^T + H^T H) (:386), the cofactors of F
    // (C = adj F: F^-1 = C / J) and B = F F^T, in float-float from H = F - I
    for (int t = tid; t < NQ * T::NA1; t += NT) {
      const int k = t / NQ, q = t - k * NQ;
      const ff* H = sH + q * 9;
      auto Fv = [&](int i, int j) { return i == j ? ff_sum(H[i * 3 + j], ff{1.0f, 0.0f}) : H[i * 3 + j]; };
      ff r;
      if (k < 6) {
        const int i = vi(k), j = vj(k);
        r = ff_sum(H[i * 3 + j], H[j * 3 + i]);
        ff_fma(r, H[0 * 3 + i], H[0 * 3 + j]);
        ff_fma(r, H[1 * 3 + i], H[1 * 3 + j]);
        ff_fma(r, H[2 * 3 + i], H[2 * 3 + j]);
        r = ff{0.5f * r.h, 0.5f * r.l};
      } else if (k < 15) {
        // C[i][j] = F[i1][j1] F[i2][j2] - F[i1][j2] F[i2][j1] with the rows of the transposed minor
        const int i = (k - 6) / 3, j = (k - 6) - 3 * i;
        const int r1 = (j + 1) % 3, r2 = (j + 2) % 3, c1 = (i + 1) % 3, c2 = (i + 2) % 3;
        r = ff_det2(Fv(r1, c1), Fv(r2, c2), Fv(r1, c2), Fv(r2, c1));
      } else {
        const int i = vi(k - 15), j = vj(k - 15);
        r = ff_mul(Fv(i, 0), Fv(j, 0));
        ff_fma(r, Fv(i, 1), Fv(j, 1));
        ff_fma(r, Fv(i, 2), Fv(j, 2));
      }
      sA1[q * T::NA1 + k] = r;
    }
    __syncthreads();
    // A1b: one thread per point of warp rot: J, I1, tr F, 1/J, the Neo-Hooke scalars (FP64)
    if (rt < 32) {
      if (rt < NQ) {
        const int q = rt;
        const int64_t pt = e * NQ + q;
        const double* props = sPr;
        const ff* H = sH + q * 9;
        const ff* A = sA1 + q * T::NA1;
        ff Jf = ff_mul(ff_sum(H[0], ff{1.0f, 0.0f}), A[6 + 0]);  // F00 C00 + F01 C10 + F02 C20
        ff_fma(Jf, H[1], A[6 + 3]);
        ff_fma(Jf, H[2], A[6 + 6]);
        const ff I1 = ff_sum(ff_sum(A[15], A[16]), A[17]);
        const ff trF = ff_sum(ff_sum(ff_sum(H[0], H[4]), H[8]), ff{3.0f, 0.0f});
        const NeoHookeScalars o = neo_hooke_scalars(g.material, props[0], props[1], ff_to_double_bits(Jf),
                                                    ff_to_double_bits(I1), ff_to_double_bits(trF));
        // 1/J: FP32 reciprocal and one Newton step in float-float
        const float r0 = __frcp_rn(Jf.h);
        ff rJ = ff_mul(Jf, ff{-r0, 0.0f});
        ff_add(rJ, ff{1.0f, 0.0f});
        rJ = ff_mul(rJ, ff{r0, 0.0f});
        ff_add(rJ, ff{r0, 0.0f});
        const double s = sS[q];
        T::A1Scalars sc;
        sc.sB = ff_split_bits(o.sB);
        sc.sI = ff_split_bits(o.sI);
        sc.aF = ff_split_bits(s * o.sB);  // s tau F^-T = (s sB) F + (s sI) F^-T
        sc.aI = ff_split_bits(s * o.sI);
        sc.rJ = rJ;
        sc.energy = o.energy;
        sc.c[0] = d2f_trunc(o.c1 * s);
        sc.c[1] = d2f_trunc(o.c2 * s);
        sc.c[2] = d2f_trunc(o.c3 * s);
        sc.c[3] = d2f_trunc(o.c4 * s);
        sSc[q] = sc;
      }
    } else {
      h20tc_pending_and_next<FF, FORM>(g, prev, next, smem, tb, sps, srl, par, rt - 32, tcs.failed);
    }
    __syncthreads();
    // A1c: one thread per (point, entry (i, j)): F^-1, s tau F^-T, the FP32 record, state
    for (int t = tid; t < NQ * 9; t += NT) {
      const int c = t / NQ, q = t - c * NQ, i = c / 3, j = c - 3 * i;
      const int64_t pt = e * NQ + q;
      const ff* H = sH + q * 9;
      const ff* A = sA1 + q * T::NA1;
      const T::A1Scalars& sc = sSc[q];
      const ff Fij = i == j ? ff_sum(H[c], ff{1.0f, 0.0f}) : H[c];
      const ff iFij = ff_mul(A[6 + c], sc.rJ), iFji = ff_mul(A[6 + j * 3 + i], sc.rJ);
      // B is stored in Voigt order 11, 22, 33, 12, 23, 13
      const ff Bij = A[15 + (i == j ? i : (i + j == 1 ? 3 : (i + j == 3 ? 4 : 5)))];
      ff pq = ff_mul(sc.aF, Fij);
      ff_fma(pq, sc.aI, iFji);
      float* r = rk + q * T::RK;
      r[T::R_F + c] = Fij.h;
      r[T::R_FI + c] = iFij.h;
      r[T::R_B + c] = Bij.h;
      r[T::R_PQ + c] = pq.h;
      reinterpret_cast<ff*>(smem + L::pq_off)[q * 9 + c] = pq;
      if (c < 4) r[T::R_C + c] = sc.c[c];
      if (c < 6) {
        // Voigt entry c: Kirchhoff stress tau = sB B + sI I, strain (E with doubled shears), E
        ff tv = ff_mul(sc.sB, A[15 + c]);
        if (c < 3) ff_add(tv, sc.sI);
        const double sig = ff_to_double_bits(tv), Ev = ff_to_double_bits(A[c]);
        g.stateTemp[(int64_t)c * stride + pt] = sig;
        g.stateTemp[(int64_t)(6 + c) * stride + pt] = c < 3 ? Ev : 2.0 * Ev;
        g.auxTemp[(int64_t)c * stride + pt] = Ev;
        if (!finite_bits(sig)) atomicOr(g.status, EFE_STATUS_NONFINITE);
      } else if (c == 6) {
        g.stateTemp[(int64_t)12 * stride + pt] = sc.energy;
      }
    }
  } else {
    if (rt < 32) {
      if (rt < NQ) {
        const int q = rt;
        const int64_t pt = e * NQ + q;
        const double* props = sPr;
        double F[3][3];
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) F[i][j] = sF[q * 9 + i * 3 + j];
        // Green-Lagrange E = 1/2 (H + H^T + H^T H), H = F - I  (:386), symmetric
        const double H[3][3] = {{F[0][0] - 1.0, F[0][1], F[0][2]}, {F[1][0], F[1][1] - 1.0, F[1][2]},
                                {F[2][0], F[2][1], F[2][2] - 1.0}};
        double Eg[3][3];
        for (int i = 0; i < 3; ++i)
          for (int j = i; j < 3; ++j)
            Eg[i][j] = Eg[j][i] = 0.5 * ((H[i][j] + H[j][i]) + (H[0][i] * H[0][j] + H[1][i] * H[1][j] + H[2][i] * H[2][j]));
        const double Ev[6] = {Eg[0][0], Eg[1][1], Eg[2][2], Eg[0][1], Eg[1][2], Eg[0][2]};
        for (int f = 0; f < 6; ++f) g.auxTemp[(int64_t)f * stride + pt] = Ev[f];
        // F^-1 from the cofactors, det F from the same cofactors
        double iF[3][3];
        iF[0][0] = F[1][1] * F[2][2] - F[1][2] * F[2][1];
        iF[1][0] = F[1][2] * F[2][0] - F[1][0] * F[2][2];
        iF[2][0] = F[1][0] * F[2][1] - F[1][1] * F[2][0];
        const double J = F[0][0] * iF[0][0] + F[0][1] * iF[1][0] + F[0][2] * iF[2][0];
        iF[0][1] = F[0][2] * F[2][1] - F[0][1] * F[2][2];
        iF[0][2] = F[0][1] * F[1][2] - F[0][2] * F[1][1];
        iF[1][1] = F[0][0] * F[2][2] - F[0][2] * F[2][0];
        iF[1][2] = F[0][2] * F[1][0] - F[0][0] * F[1][2];
        iF[2][1] = F[0][1] * F[2][0] - F[0][0] * F[2][1];
        iF[2][2] = F[0][0] * F[1][1] - F[0][1] * F[1][0];
        const double rJ = 1.0 / J;
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) iF[i][j] *= rJ;
        double B[3][3];
        for (int i = 0; i < 3; ++i)
          for (int j = i; j < 3; ++j) B[i][j] = B[j][i] = F[i][0] * F[j][0] + F[i][1] * F[j][1] + F[i][2] * F[j][2];
        const NeoHookeScalars o = neo_hooke_scalars(g.material, props[0], props[1], J, B[0][0] + B[1][1] + B[2][2],
                                                    F[0][0] + F[1][1] + F[2][2]);
        // Kirchhoff stress tau = sB B + sI I (Voigt 11, 22, 33, 12, 23, 13)
        const double sig[6] = {o.sB * B[0][0] + o.sI, o.sB * B[1][1] + o.sI, o.sB * B[2][2] + o.sI,
                               o.sB * B[0][1],        o.sB * B[1][2],        o.sB * B[0][2]};
        const double eps[6] = {Eg[0][0], Eg[1][1], Eg[2][2], 2.0 * Eg[0][1], 2.0 * Eg[1][2], 2.0 * Eg[0][2]};
        const double s = sS[q];
        // s tau F^-T = (s sB) F + (s sI) F^-T
        const double aF = s * o.sB, aI = s * o.sI;
        float* r = rk + q * T::RK;
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) {
            r[T::R_F + i * 3 + j] = d2f_trunc(F[i][j]);
            r[T::R_FI + i * 3 + j] = d2f_trunc(iF[i][j]);
            r[T::R_B + i * 3 + j] = d2f_trunc(B[i][j]);
            const double pq = aF * F[i][j] + aI * iF[j][i];
            r[T::R_PQ + i * 3 + j] = d2f_trunc(pq);
            reinterpret_cast<double*>(smem + L::pq_off)[q * 9 + i * 3 + j] = pq;
          }
        r[T::R_C + 0] = d2f_trunc(o.c1 * s);
        r[T::R_C + 1] = d2f_trunc(o.c2 * s);
        r[T::R_C + 2] = d2f_trunc(o.c3 * s);
        r[T::R_C + 3] = d2f_trunc(o.c4 * s);
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
    } else {
      h20tc_pending_and_next<FF, FORM>(g, prev, next, smem, tb, sps, srl, par, rt - 32, tcs.failed);
    }
  }
  __syncthreads();
  // zero the operand tiles (padding rows and slots must read as zero)
  for (int i = tid; i < (int)(T::tc_bytes / 16); i += NT) reinterpret_cast<float4*>(tb)[i] = make_float4(0, 0, 0, 0);
  __syncthreads();

  // ---- per chunk of 9 points: operands (A2) and the residual of the chunk's points, MMAs
  // residual threads: warps 2 and 3 (they have one A2 task each, warps 0 and 1 two); node ra,
  // component rj, one accumulator per component of dN/dX
  const int ri = tid - 64, ra = ri / 3, rj = ri - 3 * ra;
  double pe[3] = {0.0, 0.0, 0.0};
  ff pef[3] = {{0, 0}, {0, 0}, {0, 0}};
  const uint32_t base = tc::smem_addr(tb);
  for (int ch = 0; ch < T::NCH; ++ch) {
    // A2: one thread per (point, node)
    for (int t = tid; t < T::QC * NN; t += NT) {
      const int ql = t / NN, a = t - ql * NN, q = ch * T::QC + ql;
      // the point's record, 40 floats in ten 16-byte loads (the rows are 16-byte aligned)
      float r[40];
#pragma unroll
      for (int i = 0; i < 10; ++i) {
        const float4 v = reinterpret_cast<const float4*>(rk + q * T::RK)[i];
        r[4 * i] = v.x;
        r[4 * i + 1] = v.y;
        r[4 * i + 2] = v.z;
        r[4 * i + 3] = v.w;
      }
      float G[3];
      for (int l = 0; l < 3; ++l) {
        if constexpr (FF)
          G[l] = sGh[(l * NN + a) * NQ + q];
        else
          G[l] = d2f_trunc(sGd[(l * NN + a) * NQ + q]);
      }
      if constexpr (FORM == SS3) {
        // plain [lambda' G_a, -a nG_a] . [G_b, nG_b], swapped mu' G_b[j] G_a[k], diagonal mu' G_a . G_b
        float nG[3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
          nG[i] = r[T::R_F + i * 3 + 0] * G[0] + r[T::R_F + i * 3 + 1] * G[1] + r[T::R_F + i * 3 + 2] * G[2];
        const float Lq = r[T::R_C + 0], Mq = r[T::R_C + 1], Aq = r[T::R_C + 2];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const int row = 3 * a + j;
          tc_put2<T::SBO_PS>(tb + T::a_hi, tb + T::a_lo, row, 2 * ql, Lq * G[j], -Aq * nG[j]);
          tc_put<T::SBO_PS>(tb + T::a_hi, tb + T::a_lo, 64 + row, 2 * ql, Mq * G[j]);
          tc_put2<T::SBO_PS>(tb + T::b_hi, tb + T::b_lo, row, 2 * ql, G[j], nG[j]);
          tc_put<T::SBO_D>(tb + T::dA_hi, tb + T::dA_lo, a, 3 * ql + j, Mq * G[j]);
          tc_put<T::SBO_D>(tb + T::dB_hi, tb + T::dB_lo, a, 3 * ql + j, G[j]);
        }
      } else {
        float h[3], gg[3], th[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          h[i] = r[T::R_FI + 0 * 3 + i] * G[0] + r[T::R_FI + 1 * 3 + i] * G[1] + r[T::R_FI + 2 * 3 + i] * G[2];
          gg[i] = r[T::R_F + i * 3 + 0] * G[0] + r[T::R_F + i * 3 + 1] * G[1] + r[T::R_F + i * 3 + 2] * G[2];
          th[i] = r[T::R_PQ + i * 3 + 0] * G[0] + r[T::R_PQ + i * 3 + 1] * G[1] + r[T::R_PQ + i * 3 + 2] * G[2];
        }
        const float c1s = r[T::R_C + 0], c2s = r[T::R_C + 1], c3s = r[T::R_C + 2], c4s = r[T::R_C + 3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const float bh = r[T::R_B + j * 3 + 0] * h[0] + r[T::R_B + j * 3 + 1] * h[1] + r[T::R_B + j * 3 + 2] * h[2];
          const int row = 3 * a + j;
          tc_put2<T::SBO_PS>(tb + T::a_hi, tb + T::a_lo, row, 2 * ql, c2s * h[j] + c3s * bh, c4s * h[j]);
          tc_put<T::SBO_PS>(tb + T::a_hi, tb + T::a_lo, 64 + row, 2 * ql, c1s * gg[j] - th[j]);
          tc_put2<T::SBO_PS>(tb + T::b_hi, tb + T::b_lo, row, 2 * ql, h[j], gg[j]);
          tc_put<T::SBO_D>(tb + T::dA_hi, tb + T::dA_lo, a, 3 * ql + j, c1s * G[j]);
          tc_put<T::SBO_D>(tb + T::dB_hi, tb + T::dB_lo, a, 3 * ql + j, G[j]);
        }
      }
    }
    // residual of the chunk's points: P_e[a][j] -= sum_q sum_l Pq[j][l] G_qa[l]
    if (ri >= 0 && ri < T::NDOF) {
      for (int ql = 0; ql < T::QC; ++ql) {
        const int q = ch * T::QC + ql;
#pragma unroll
        for (int l = 0; l < 3; ++l) {
          const int gi = (l * NN + ra) * NQ + q;
          if constexpr (FF)
            ff_fma(pef[l], reinterpret_cast<const ff*>(smem + L::pq_off)[q * 9 + rj * 3 + l], ff{sGh[gi], sGl[gi]});
          else
            pe[l] -= reinterpret_cast<const double*>(smem + L::pq_off)[q * 9 + rj * 3 + l] * sGd[gi];
        }
      }
    }
    tc::fence_proxy_async();
    __syncthreads();
    // after the last chunk's operands and residual the staged dN/dX is dead: stage the next
    // element's while the MMAs run
    if (ch == T::NCH - 1 && next >= 0) h20tc_stage_g<FF>(g, next, smem);
    if (tid == 0 && !tcs.failed) {
      tc::fence_after_sync();
      constexpr uint32_t idPS = tc::idesc_tf32(128, 64), idD = tc::idesc_tf32(128, 32);
      for (int s = 0; s < T::KPS / 8; ++s) {
        const uint64_t ah = tc::smem_desc(base + T::a_hi + s * 256, 128, T::SBO_PS);
        const uint64_t al = tc::smem_desc(base + T::a_lo + s * 256, 128, T::SBO_PS);
        const uint64_t bh = tc::smem_desc(base + T::b_hi + s * 256, 128, T::SBO_PS);
        const uint64_t bl = tc::smem_desc(base + T::b_lo + s * 256, 128, T::SBO_PS);
        tc::mma_tf32(tcs.tmem, ah, bh, idPS, ch > 0 || s > 0);
        tc::mma_tf32(tcs.tmem, ah, bl, idPS, true);
        tc::mma_tf32(tcs.tmem, al, bh, idPS, true);
      }
      for (int s = 0; s < T::KD / 8; ++s) {
        const uint64_t ah = tc::smem_desc(base + T::dA_hi + s * 256, 128, T::SBO_D);
        const uint64_t al = tc::smem_desc(base + T::dA_lo + s * 256, 128, T::SBO_D);
        const uint64_t bh = tc::smem_desc(base + T::dB_hi + s * 256, 128, T::SBO_D);
        const uint64_t bl = tc::smem_desc(base + T::dB_lo + s * 256, 128, T::SBO_D);
        tc::mma_tf32(tcs.tmem + T::D_COL, ah, bh, idD, ch > 0 || s > 0);
        tc::mma_tf32(tcs.tmem + T::D_COL, ah, bl, idD, true);
        tc::mma_tf32(tcs.tmem + T::D_COL, al, bh, idD, true);
      }
      tc::mma_commit(tcs.mbar);
    }
    // the operand tiles are rewritten by the next chunk: wait for the MMAs that read them (the
    // phase parity advances only with a completed phase, so after a time-out tcs.phase is the one
    // still outstanding)
    if (!tcs.failed) {
      if (tc::mbar_wait(tcs.mbar, tcs.phase, TC_WAIT_LIMIT)) {
        tcs.phase ^= 1u;
      } else {
        tcs.failed = true;
        atomicOr(g.status, EFE_STATUS_TC_TIMEOUT);
      }
    }
    tcs.failed = __syncthreads_or(tcs.failed);
  }
  tc::fence_after_sync();

  // ---- epilogue: accumulators -> shared memory (over the operand tiles)
  {
    float* sP = reinterpret_cast<float*>(tb + T::sP);
    float* sX = reinterpret_cast<float*>(tb + T::sX);
    float* sD = reinterpret_cast<float*>(tb + T::sD);
    const int w = tid >> 5, lane = tid & 31, row = tid;  // warp w reads TMEM lanes 32w .. 32w+31
    const uint32_t ta = tcs.tmem + ((uint32_t)(w * 32) << 16);
    float v[16];
    for (int c0 = 0; c0 < 64; c0 += 16) {
      tc::tmem_ld16(ta + c0, v);
      if (row < T::NDOF) {
        for (int c = 0; c < 16; ++c)
          if (c0 + c < T::NDOF) sP[row * T::SS + c0 + c] = v[c];
      } else if (row >= 64 && row < 64 + T::NDOF) {
        for (int c = 0; c < 16; ++c)
          if (c0 + c < T::NDOF) sX[(row - 64) * T::SS + c0 + c] = v[c];
      }
    }
    if (w == 0) {
      for (int c0 = 0; c0 < 32; c0 += 16) {
        tc::tmem_ld16(ta + T::D_COL + c0, v);
        if (lane < NN)
          for (int c = 0; c < 16; ++c)
            if (c0 + c < NN) sD[lane * (NN + 1) + c0 + c] = v[c];
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();

  // ---- residual and flux (NIST.computeElements, nonlinearimplicitstatic.py:837-844)
  if (ri >= 0 && ri < T::NDOF) {
    double p;
    if constexpr (FF) {
      ff acc = pef[0];
      ff_add(acc, pef[1]);
      ff_add(acc, pef[2]);
      p = -ff_to_double_bits(acc);
    } else {
      p = (pe[0] + pe[1]) + pe[2];
    }
    // the node's first DOF as staged (-1: its bounds check failed and was reported)
    const int32_t d0 = reinterpret_cast<const int*>(smem + L::dof_off)[par * NN + ra];
    if (d0 >= 0) {
      atomicAdd(g.P + d0 + rj, p);
      atomicAdd(g.F + d0 + rj, fabs(p));
    }
  }
  if (prev == H20TC_NOW && !tcs.failed) h20tc_scatter(g, e, tb, sps + par * NN * NN, srl + par * NN, tid, NT);
}

}  // namespace efe
