// efe_batch.cu -- persistent launch over two element groups (uneven batches of meshes).
#include "efe_launch.cuh"

namespace efe {

namespace {

template <int SA, int RA, int FA, int SB, int RB, int FB, typename KT>
cudaError_t run_pair(const GroupArgs& a, const GroupArgs& b, unsigned long long* counter, cudaStream_t st) {
  using TA = Tile<SA, RA, FA, KT>;
  using TB = Tile<SB, RB, FB, KT>;
  static_assert(TA::NT == TB::NT, "both tile types must use the same CTA size");
  constexpr int NT = TA::NT;
  constexpr size_t bytes = TA::bytes > TB::bytes ? TA::bytes : TB::bytes;
  auto kern = assemble_persistent_kernel<SA, RA, FA, TA::EPB, SB, RB, FB, TB::EPB, KT, NT>;
  cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (err != cudaSuccess) return err;
  int dev = 0, sms = 0, perSM = 0;
  if ((err = cudaGetDevice(&dev)) != cudaSuccess) return err;
  if ((err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return err;
  if ((err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kern, NT, bytes)) != cudaSuccess) return err;
  if (perSM < 1) return cudaErrorInvalidConfiguration;
  const int64_t tilesA = (a.nElements + TA::EPB - 1) / TA::EPB;
  const int64_t tilesB = (b.nElements + TB::EPB - 1) / TB::EPB;
  if ((err = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st)) != cudaSuccess) return err;
  int64_t grid = (int64_t)sms * perSM;
  if (grid > tilesA + tilesB) grid = tilesA + tilesB;
  if (grid == 0) return cudaSuccess;
  kern<<<(unsigned)grid, NT, bytes, st>>>(a, b, tilesA, tilesB, counter);
  return cudaGetLastError();
}

template <typename KT>
cudaError_t dispatch(int shapeA, int ruleA, int formA, int shapeB, int ruleB, int formB, const GroupArgs& a,
                     const GroupArgs& b, unsigned long long* counter, cudaStream_t st) {
  const bool aH20 = shapeA == EFE_HEXA20 && ruleA == EFE_RULE_3D_3X3X3 && formA == TLH;
  const bool bQ8 = shapeB == EFE_QUAD8 && ruleB == EFE_RULE_2D_2X2 && formB == TLH;
  const bool aQ8 = shapeA == EFE_QUAD8 && ruleA == EFE_RULE_2D_2X2 && formA == TLH;
  const bool bH20 = shapeB == EFE_HEXA20 && ruleB == EFE_RULE_3D_3X3X3 && formB == TLH;
  // the heavier Hexa20 tiles are handed out first
  if (aH20 && bQ8)
    return run_pair<EFE_HEXA20, EFE_RULE_3D_3X3X3, TLH, EFE_QUAD8, EFE_RULE_2D_2X2, TLH, KT>(a, b, counter, st);
  if (aQ8 && bH20)
    return run_pair<EFE_HEXA20, EFE_RULE_3D_3X3X3, TLH, EFE_QUAD8, EFE_RULE_2D_2X2, TLH, KT>(b, a, counter, st);
  return cudaErrorNotSupported;
}

}  // namespace

cudaError_t persistent_pair(int shapeA, int ruleA, int formA, int shapeB, int ruleB, int formB, int kprec,
                            const GroupArgs& a, const GroupArgs& b, unsigned long long* counter, cudaStream_t st) {
  if (kprec == EFE_K_FP32) return dispatch<float>(shapeA, ruleA, formA, shapeB, ruleB, formB, a, b, counter, st);
  return dispatch<double>(shapeA, ruleA, formA, shapeB, ruleB, formB, a, b, counter, st);
}

}  // namespace efe
