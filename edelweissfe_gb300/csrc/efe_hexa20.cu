// efe_hexa20.cu -- kernel instantiations for the hexa20 element shape (one translation unit per shape).
#include "efe_adjoint.cuh"
#include "efe_adjoint_ss.cuh"

namespace efe {

cudaError_t assemble_hexa20(int rule, int form, int kprec, const GroupArgs& g, cudaStream_t st) {
  switch (rule) {
    case EFE_RULE_3D_2X2X2: return launch_rule<EFE_HEXA20, EFE_RULE_3D_2X2X2>(form, kprec, g, st);
    case EFE_RULE_3D_3X3X3: return launch_rule<EFE_HEXA20, EFE_RULE_3D_3X3X3>(form, kprec, g, st);
  }
  return cudaErrorInvalidValue;
}

cudaError_t geometry_hexa20(int rule, int64_t nEl, int64_t off, const int32_t* conn, const double* coords,
                             const double* th, double* G, float* G32, float* Glo, double* S,
                             int32_t* status, const Hexa20Fix& fix, cudaStream_t st) {
  switch (rule) {
    case EFE_RULE_3D_2X2X2: return launch_geometry<EFE_HEXA20, EFE_RULE_3D_2X2X2>(nEl, off, conn, coords, th, G, G32, Glo, S, status, fix, st);
    case EFE_RULE_3D_3X3X3: return launch_geometry<EFE_HEXA20, EFE_RULE_3D_3X3X3>(nEl, off, conn, coords, th, G, G32, Glo, S, status, fix, st);
  }
  return cudaErrorInvalidValue;
}

cudaError_t body_force_hexa20(int rule, int64_t nSel, const int32_t* elems, const int32_t* conn, const int32_t* nodeDof,
                              const double* S, const double* f, double* P, cudaStream_t st) {
  switch (rule) {
    case EFE_RULE_3D_2X2X2: return launch_body_force<EFE_HEXA20, EFE_RULE_3D_2X2X2>(nSel, elems, conn, nodeDof, S, f, P, st);
    case EFE_RULE_3D_3X3X3: return launch_body_force<EFE_HEXA20, EFE_RULE_3D_3X3X3>(nSel, elems, conn, nodeDof, S, f, P, st);
  }
  return cudaErrorInvalidValue;
}

cudaError_t adjoint_tl_hexa20(int rule, const AdjointArgs& a, cudaStream_t st) {
  switch (rule) {
    case EFE_RULE_3D_2X2X2: return launch_adjoint_tl<EFE_HEXA20, EFE_RULE_3D_2X2X2>(a, st);
    case EFE_RULE_3D_3X3X3: return launch_adjoint_tl<EFE_HEXA20, EFE_RULE_3D_3X3X3>(a, st);
  }
  return cudaErrorInvalidValue;
}

cudaError_t adjoint_ss_hexa20(int rule, const SSAdjointArgs& a, cudaStream_t st) {
  switch (rule) {
    case EFE_RULE_3D_2X2X2: return launch_adjoint_ss<EFE_HEXA20, EFE_RULE_3D_2X2X2>(a, st);
    case EFE_RULE_3D_3X3X3: return launch_adjoint_ss<EFE_HEXA20, EFE_RULE_3D_3X3X3>(a, st);
  }
  return cudaErrorInvalidValue;
}

}  // namespace efe
