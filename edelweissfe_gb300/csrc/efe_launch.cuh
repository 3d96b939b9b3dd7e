// efe_launch.cuh -- tile sizing and launch of the kernels of one element shape.
#pragma once
#include <algorithm>

#include "efe_kernels.cuh"

namespace efe {

// Tile shapes of the element pass.  Variant 0: about 128 material points per CTA (one per
// thread in phase A), 128 threads, at most 72 KB of shared memory so that three CTAs share an SM.
// Variant 1: about 256 points and 256 threads per CTA, up to 110 KB (one or two CTAs per SM).
// The autotuner (edelweissfe_gb300/autotune.py) picks one per group by timing both.
template <int SHAPE, int RULE, int FORM, typename KT, int VARIANT = 0>
struct Tile {
  // variant 0: 128 threads, ~128 points, 3 CTAs/SM where they fit; 1: 256 threads, ~256 points;
  // 2: variant 0's tile with 4 CTAs/SM where shared memory allows (the compiler then holds the
  // kernel to 128 registers per thread)
  static constexpr int NQ = RuleInfo<RULE>::NQ;
  static constexpr size_t per_element = Layout<SHAPE, RULE, FORM, KT, 1>::bytes;
  static constexpr size_t budget = VARIANT == 1 ? 110 * 1024 : 72 * 1024;
  static constexpr int points = VARIANT == 1 ? 256 : 128;
  static constexpr int fit = (int)(budget / per_element);
  static constexpr int want = (points + NQ - 1) / NQ;
  static constexpr int e0 = fit < want ? fit : want;
  static constexpr int EPB = e0 < 1 ? 1 : (e0 > 32 ? 32 : e0);
  static constexpr int NT = VARIANT == 1 ? 256 : 128;
  static constexpr size_t bytes = Layout<SHAPE, RULE, FORM, KT, EPB>::bytes;
  static constexpr int MINB = VARIANT == 1 ? 1
                              : (VARIANT == 2 && bytes <= 56 * 1024) ? 4
                              : (bytes <= 72 * 1024 ? 3 : 1);
};

template <int SHAPE, int RULE, int FORM, typename KT, bool FF, int VARIANT>
cudaError_t launch_assemble_variant(const GroupArgs& g, cudaStream_t st) {
  using T = Tile<SHAPE, RULE, FORM, KT, VARIANT>;
  static_assert(T::bytes <= 200 * 1024, "tile does not fit in shared memory");
  auto kern = assemble_kernel<SHAPE, RULE, FORM, KT, T::EPB, T::NT, T::MINB, FF>;
  cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::bytes);
  if (err != cudaSuccess) return err;
  const int64_t grid = (g.nElements + T::EPB - 1) / T::EPB;
  if (grid == 0) return cudaSuccess;
  kern<<<(unsigned)grid, T::NT, T::bytes, st>>>(g);
  return cudaGetLastError();
}

// the tensor-core tangent (tile variant 3) exists for the Hexa20 3x3x3 total-Lagrangian Neo-Hooke
// and small-strain (von Mises, linear elastic) forms with an FP32 tangent
template <int SHAPE, int RULE, int FORM, typename KT>
constexpr bool has_tc_variant() {
  return SHAPE == EFE_HEXA20 && RULE == EFE_RULE_3D_3X3X3 && (FORM == TLH || FORM == SS3) &&
         std::is_same<KT, float>::value;
}

// Resident CTAs per SM of a kernel that allocates tmemCols TMEM columns per CTA, from its registers
// (allocated per thread in units of 8), its shared memory (plus the per-CTA reservation), its threads
// and the SM's 512 TMEM columns.  The runtime's occupancy query answers 1 for kernels that allocate
// TMEM whatever their size; the CTAs beyond what actually fits only wait for an SM (none waits on
// another, and tcgen05.alloc waits for free columns), so an estimate that is too high costs nothing.
template <typename K>
cudaError_t resident_ctas_tmem(K kern, int nt, size_t dynBytes, int tmemCols, int* perSM) {
  cudaFuncAttributes fa;
  cudaError_t err = cudaFuncGetAttributes(&fa, kern);
  if (err != cudaSuccess) return err;
  int dev = 0, regsSM = 0, smemSM = 0, reserved = 0, threadsSM = 0;
  if ((err = cudaGetDevice(&dev)) != cudaSuccess) return err;
  if ((err = cudaDeviceGetAttribute(&regsSM, cudaDevAttrMaxRegistersPerMultiprocessor, dev)) != cudaSuccess) return err;
  if ((err = cudaDeviceGetAttribute(&smemSM, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev)) != cudaSuccess) return err;
  if ((err = cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev)) != cudaSuccess) return err;
  if ((err = cudaDeviceGetAttribute(&threadsSM, cudaDevAttrMaxThreadsPerMultiProcessor, dev)) != cudaSuccess) return err;
  const int regs = (fa.numRegs + 7) / 8 * 8;
  int n = regsSM / (regs * nt);
  const long long perCta = (long long)dynBytes + (long long)fa.sharedSizeBytes + reserved;
  n = std::min<long long>(n, smemSM / perCta);
  n = std::min(n, threadsSM / nt);
  n = std::min(n, 512 / tmemCols);
  *perSM = n;
  return n >= 1 ? cudaSuccess : cudaErrorInvalidConfiguration;
}

template <bool FF, int FORM>
cudaError_t launch_assemble_tc(const GroupArgs& g, cudaStream_t st) {
  constexpr int NT = 128;
  constexpr size_t bytes = H20TCLayout<FF>::bytes;
  static_assert(bytes <= 74 * 1024, "three tensor-core tiles must fit in one SM");
  auto kern = assemble_kernel_tc<FF, FORM>;
  cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (err != cudaSuccess) return err;
  // the largest shared-memory partition: without it the occupancy query (and the launch) assume the
  // default split and fit one CTA per SM
  err = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
  if (err != cudaSuccess) return err;
  int dev = 0, sms = 0, perSM = 0;
  if ((err = cudaGetDevice(&dev)) != cudaSuccess) return err;
  if ((err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return err;
  if ((err = resident_ctas_tmem(kern, NT, bytes, (int)H20TC::TMEM_COLS, &perSM)) != cudaSuccess) return err;
  int64_t grid = (int64_t)sms * perSM;
  if (grid > g.nElements) grid = g.nElements;
  if (grid == 0) return cudaSuccess;
  kern<<<(unsigned)grid, NT, bytes, st>>>(g, sms);
  return cudaGetLastError();
}

template <int SHAPE, int RULE, int FORM, typename KT, bool FF = false>
cudaError_t launch_assemble(const GroupArgs& g, cudaStream_t st) {
  if constexpr (has_tc_variant<SHAPE, RULE, FORM, KT>()) {
    if (g.tileVariant == 3) return launch_assemble_tc<FF, FORM>(g, st);
  }
  if (g.tileVariant == 1) return launch_assemble_variant<SHAPE, RULE, FORM, KT, FF, 1>(g, st);
  if constexpr (Tile<SHAPE, RULE, FORM, KT, 2>::MINB != Tile<SHAPE, RULE, FORM, KT, 0>::MINB) {
    if (g.tileVariant == 2) return launch_assemble_variant<SHAPE, RULE, FORM, KT, FF, 2>(g, st);
  }
  return launch_assemble_variant<SHAPE, RULE, FORM, KT, FF, 0>(g, st);
}

template <int SHAPE, int RULE>
cudaError_t launch_geometry(int64_t nEl, int64_t elOffset, const int32_t* conn, const double* coords,
                            const double* thickness, double* G, float* G32, float* Glo, double* S,
                            int32_t* status, const Hexa20Fix& fix, cudaStream_t st) {
  const int64_t n = nEl * RuleInfo<RULE>::NQ;
  if (n == 0) return cudaSuccess;
  const int nt = 128;
  geometry_kernel<SHAPE, RULE><<<(unsigned)((n + nt - 1) / nt), nt, 0, st>>>(nEl, elOffset, conn, coords, thickness,
                                                                             G, G32, Glo, S, status, fix);
  return cudaGetLastError();
}

template <int SHAPE, int RULE>
cudaError_t launch_body_force(int64_t nSel, const int32_t* elems, const int32_t* conn, const int32_t* nodeDof,
                              const double* S, const double* f, double* P, cudaStream_t st) {
  const int64_t n = nSel * ShapeInfo<SHAPE>::NN;
  if (n == 0) return cudaSuccess;
  const int nt = 128;
  body_force_kernel<SHAPE, RULE><<<(unsigned)((n + nt - 1) / nt), nt, 0, st>>>(nSel, elems, conn, nodeDof, S, f[0], f[1],
                                                                               ShapeInfo<SHAPE>::DIM == 3 ? f[2] : 0.0, P);
  return cudaGetLastError();
}

struct AdjointArgs {
  int64_t nEl;
  const int32_t* conn;
  const int32_t* nodeDof;
  const double* coords;
  const double* U;
  const double* lam;
  const double* props;
  int nProps, material;
  const double* thickness;
  Hexa20Fix fix;
  double* gX;
  double* gP;
};

template <int SHAPE, int RULE>
cudaError_t launch_adjoint_tl(const AdjointArgs& a, cudaStream_t st);

// reverse mode of one small-strain element pass (efe_adjoint_ss.cuh)
struct SSAdjointArgs {
  int64_t nEl;
  int32_t nProps, material;
  int32_t planeStress;  // 2D groups: 1 for plane stress (local Newton on eps33), 0 for plane strain
  const int32_t* conn;
  const int32_t* nodeDof;
  const double* props;
  const double* geomG;
  const float* geomG32;       // optional: with geomGlo the float-float geometry (B-products on the FP32 pipe)
  const float* geomGlo;
  const double* geomS;
  const double* stateBefore;  // [S][nPts]
  const double* dU;           // [nDof]
  const double* Pbar;         // [nDof] or null
  const double* barIn;        // [S][nPts] or null
  double* barOut;             // [S][nPts] or null (accumulated)
  double* dUbar;              // [nDof] (accumulated)
  double* gProps;             // [nEl][nProps] or null (accumulated)
  // nodal coordinate adjoints [nNodes][dim] (accumulated) or null; coords and the Hexa20 table for
  // the Jacobian of the Hexa20 quirk
  double* gX;
  const double* coords;
  Hexa20Fix fix;
};

template <int SHAPE, int RULE>
cudaError_t launch_adjoint_ss(const SSAdjointArgs& a, cudaStream_t st);

// form selector: small strain 3D/2D, total Lagrangian hyperelastic, total Lagrangian hypoelastic 3D/2D
template <int SHAPE, int RULE, typename KT, bool FF = false>
cudaError_t launch_form(int form, const GroupArgs& g, cudaStream_t st) {
  constexpr int DIM = ShapeInfo<SHAPE>::DIM;
  if constexpr (DIM == 3) {
    switch (form) {
      case SS3: return launch_assemble<SHAPE, RULE, SS3, KT, FF>(g, st);
      case TLH: return launch_assemble<SHAPE, RULE, TLH, KT, FF>(g, st);
      case TLV3: return launch_assemble<SHAPE, RULE, TLV3, KT>(g, st);
    }
  } else {
    switch (form) {
      case SS2: return launch_assemble<SHAPE, RULE, SS2, KT>(g, st);
      case TLH: return launch_assemble<SHAPE, RULE, TLH, KT, FF>(g, st);
      case TLV2: return launch_assemble<SHAPE, RULE, TLV2, KT>(g, st);
    }
  }
  return cudaErrorInvalidValue;
}

template <int SHAPE, int RULE>
cudaError_t launch_rule(int form, int kprec, const GroupArgs& g, cudaStream_t st) {
  if (kprec == EFE_K_FP32_FF) return launch_form<SHAPE, RULE, float, true>(form, g, st);
  return kprec == EFE_K_FP32 ? launch_form<SHAPE, RULE, float>(form, g, st)
                             : launch_form<SHAPE, RULE, double>(form, g, st);
}

// per-shape entry points (one translation unit each, compiled in parallel)
cudaError_t assemble_quad4(int rule, int form, int kprec, const GroupArgs& g, cudaStream_t st);
cudaError_t assemble_quad8(int rule, int form, int kprec, const GroupArgs& g, cudaStream_t st);
cudaError_t assemble_hexa8(int rule, int form, int kprec, const GroupArgs& g, cudaStream_t st);
cudaError_t assemble_hexa20(int rule, int form, int kprec, const GroupArgs& g, cudaStream_t st);
#define EFE_BODY_DECL(name)                                                                                \
  cudaError_t body_force_##name(int rule, int64_t nSel, const int32_t* elems, const int32_t* conn,            \
                                const int32_t* nodeDof, const double* S, const double* f, double* P, cudaStream_t st);
EFE_BODY_DECL(quad4)
EFE_BODY_DECL(quad8)
EFE_BODY_DECL(hexa8)
EFE_BODY_DECL(hexa20)
#undef EFE_BODY_DECL
// the persistent pass over up to MAX_PERSISTENT_GROUPS groups of each of its element types
// (groups[k][0 .. nGroups[k]) for type k of persistent_type_index)
cudaError_t persistent_groups(int kprec, const GroupArgs (*groups)[MAX_PERSISTENT_GROUPS], const int* nGroups,
                              unsigned long long* counter, cudaStream_t st);
// same pass with the work counter in the library's static scratch array; *needed = tile indices
// the counter runs through (written before the range check)
cudaError_t persistent_groups_noalloc(int kprec, const GroupArgs (*groups)[MAX_PERSISTENT_GROUPS], const int* nGroups,
                                      int64_t* needed, cudaStream_t st);
// FMA-chain probe of the FP64 / FP32 pipe (efe_probe.cu)
cudaError_t fma_probe(int fp64, int blocks, int64_t iterations, void* sink, cudaStream_t st);
int64_t fma_probe_flops(int blocks, int64_t iterations);
// device linear solve (efe_solve.cu)
cudaError_t csr_spmv(const EfePcg& s, const double* x, double* y, cudaStream_t st);
cudaError_t csr_gemv(const EfeCsr& a, const double* x, double alpha, double beta, double* y, cudaStream_t st);
cudaError_t csr_gemv_pairs(const EfeCsr& a, const float2* xf, double alpha, double beta, double* y,
                           cudaStream_t st);
cudaError_t chebyshev_step(int64_t n, const double* dinv, const double* r, double c1, double c2, int accumulate,
                           double* d, double* z, float2* dff, cudaStream_t st);
cudaError_t split_pairs(int64_t n, const double* x, float2* xf, cudaStream_t st);
cudaError_t pcg_start(const EfePcg& s, const double* b, cudaStream_t st);
cudaError_t pcg_iterate(const EfePcg& s, int64_t k0, int nIter, cudaStream_t st);
cudaError_t adjoint_ss_quad4(int rule, const SSAdjointArgs& a, cudaStream_t st);
cudaError_t adjoint_ss_quad8(int rule, const SSAdjointArgs& a, cudaStream_t st);
cudaError_t adjoint_ss_hexa8(int rule, const SSAdjointArgs& a, cudaStream_t st);
cudaError_t adjoint_ss_hexa20(int rule, const SSAdjointArgs& a, cudaStream_t st);
cudaError_t adjoint_tl_quad4(int rule, const AdjointArgs& a, cudaStream_t st);
cudaError_t adjoint_tl_quad8(int rule, const AdjointArgs& a, cudaStream_t st);
cudaError_t adjoint_tl_hexa8(int rule, const AdjointArgs& a, cudaStream_t st);
cudaError_t adjoint_tl_hexa20(int rule, const AdjointArgs& a, cudaStream_t st);
#define EFE_GEOMETRY_DECL(name)                                                                          \
  cudaError_t geometry_##name(int rule, int64_t nEl, int64_t off, const int32_t* conn, const double* coords, \
                              const double* th, double* G, float* G32, float* Glo, double* S,                 \
                              int32_t* status, const Hexa20Fix& fix, cudaStream_t st);
EFE_GEOMETRY_DECL(quad4)
EFE_GEOMETRY_DECL(quad8)
EFE_GEOMETRY_DECL(hexa8)
EFE_GEOMETRY_DECL(hexa20)
#undef EFE_GEOMETRY_DECL

}  // namespace efe
