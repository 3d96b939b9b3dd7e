// efe_batch.cu -- persistent launch over two element groups (uneven batches of meshes), and its
// variant for callers that cannot allocate device memory.
#include <mutex>

#include "efe_launch.cuh"

namespace efe {

namespace {

template <int SA, int RA, int FA, int SB, int RB, int FB, typename KT, typename CT>
cudaError_t run_pair(const GroupArgs& a, const GroupArgs& b, CT* counter, int64_t maxTiles, int64_t* needed,
                     cudaStream_t st) {
  using TA = Tile<SA, RA, FA, KT>;
  using TB = Tile<SB, RB, FB, KT>;
  static_assert(TA::NT == TB::NT, "both tile types must use the same CTA size");
  constexpr int NT = TA::NT;
  constexpr size_t bytes = TA::bytes > TB::bytes ? TA::bytes : TB::bytes;
  auto kern = assemble_persistent_kernel<SA, RA, FA, TA::EPB, SB, RB, FB, TB::EPB, KT, NT, CT>;
  cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (err != cudaSuccess) return err;
  int dev = 0, sms = 0, perSM = 0;
  if ((err = cudaGetDevice(&dev)) != cudaSuccess) return err;
  if ((err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return err;
  if ((err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kern, NT, bytes)) != cudaSuccess) return err;
  if (perSM < 1) return cudaErrorInvalidConfiguration;
  const int64_t tilesA = (a.nElements + TA::EPB - 1) / TA::EPB;
  const int64_t tilesB = (b.nElements + TB::EPB - 1) / TB::EPB;
  int64_t grid = (int64_t)sms * perSM;
  if (grid > tilesA + tilesB) grid = tilesA + tilesB;
  // the counter ends at tilesA + tilesB + grid (every CTA takes one tile index past the end)
  if (needed) *needed = tilesA + tilesB + grid;
  if (tilesA + tilesB + grid > maxTiles) return cudaErrorInvalidValue;
  if ((err = cudaMemsetAsync(counter, 0, sizeof(CT), st)) != cudaSuccess) return err;
  if (grid == 0) return cudaSuccess;
  kern<<<(unsigned)grid, NT, bytes, st>>>(a, b, tilesA, tilesB, counter);
  return cudaGetLastError();
}

template <typename KT, typename CT>
cudaError_t dispatch(int shapeA, int ruleA, int formA, int shapeB, int ruleB, int formB, const GroupArgs& a,
                     const GroupArgs& b, CT* counter, int64_t maxTiles, int64_t* needed, cudaStream_t st) {
  const bool aH20 = shapeA == EFE_HEXA20 && ruleA == EFE_RULE_3D_3X3X3 && formA == TLH;
  const bool bQ8 = shapeB == EFE_QUAD8 && ruleB == EFE_RULE_2D_2X2 && formB == TLH;
  const bool aQ8 = shapeA == EFE_QUAD8 && ruleA == EFE_RULE_2D_2X2 && formA == TLH;
  const bool bH20 = shapeB == EFE_HEXA20 && ruleB == EFE_RULE_3D_3X3X3 && formB == TLH;
  // the heavier Hexa20 tiles are handed out first
  if (aH20 && bQ8)
    return run_pair<EFE_HEXA20, EFE_RULE_3D_3X3X3, TLH, EFE_QUAD8, EFE_RULE_2D_2X2, TLH, KT>(a, b, counter, maxTiles,
                                                                                             needed, st);
  if (aQ8 && bH20)
    return run_pair<EFE_HEXA20, EFE_RULE_3D_3X3X3, TLH, EFE_QUAD8, EFE_RULE_2D_2X2, TLH, KT>(b, a, counter, maxTiles,
                                                                                             needed, st);
  return cudaErrorNotSupported;
}

template <typename CT>
cudaError_t persistent_pair_t(int shapeA, int ruleA, int formA, int shapeB, int ruleB, int formB, int kprec,
                              const GroupArgs& a, const GroupArgs& b, CT* counter, int64_t maxTiles, int64_t* needed,
                              cudaStream_t st) {
  if (kprec == EFE_K_FP32)
    return dispatch<float>(shapeA, ruleA, formA, shapeB, ruleB, formB, a, b, counter, maxTiles, needed, st);
  return dispatch<double>(shapeA, ruleA, formA, shapeB, ruleB, formB, a, b, counter, maxTiles, needed, st);
}

}  // namespace

cudaError_t persistent_pair(int shapeA, int ruleA, int formA, int shapeB, int ruleB, int formB, int kprec,
                            const GroupArgs& a, const GroupArgs& b, unsigned long long* counter, cudaStream_t st) {
  return persistent_pair_t(shapeA, ruleA, formA, shapeB, ruleB, formB, kprec, a, b, counter, INT64_MAX, nullptr, st);
}

// ---------------------------------------------------------------------------------------------
// Allocation-free variant (efe_compute_elements_persistent_noalloc).  Its one piece of scratch, the
// work counter, is word 0 of this fixed device array instead of caller-provided memory, so the
// call needs no device allocation at all.  Every GPU that loads the library holds these
// EFE_NOALLOC_SCRATCH_BYTES until the process exits.  In host code `noalloc_scratch` only names
// the array; its device address on a given device comes from cudaGetSymbolAddress, looked up
// once per device (noalloc_scratch_address).  All calls on a device share the array: the counter
// is zeroed by every call on the caller's stream before the launch, and calls whose launches
// overlap on the GPU race on it.
// ---------------------------------------------------------------------------------------------
static __device__ __align__(256) unsigned int noalloc_scratch[EFE_NOALLOC_SCRATCH_BYTES / sizeof(unsigned int)];

namespace {

constexpr int kNoallocMaxDevices = 64;
std::mutex noalloc_mutex;
void* noalloc_address[kNoallocMaxDevices] = {};

// Device address of noalloc_scratch on the current device.  The first call on a device looks it
// up (with that device current) and keeps it; later calls only read the table.
cudaError_t noalloc_scratch_address(unsigned int** out) {
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return err;
  if (dev < 0 || dev >= kNoallocMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(noalloc_mutex);
  if (!noalloc_address[dev]) {
    void* ptr = nullptr;
    err = cudaGetSymbolAddress(&ptr, noalloc_scratch);
    if (err != cudaSuccess) return err;
    if (!ptr) return cudaErrorInvalidSymbol;
    noalloc_address[dev] = ptr;
  }
  *out = static_cast<unsigned int*>(noalloc_address[dev]);
  return cudaSuccess;
}

}  // namespace

cudaError_t persistent_pair_noalloc(int shapeA, int ruleA, int formA, int shapeB, int ruleB, int formB, int kprec,
                                    const GroupArgs& a, const GroupArgs& b, int64_t* needed, cudaStream_t st) {
  unsigned int* counter = nullptr;
  cudaError_t err = noalloc_scratch_address(&counter);
  if (err != cudaSuccess) return err;
  return persistent_pair_t(shapeA, ruleA, formA, shapeB, ruleB, formB, kprec, a, b, counter,
                           (int64_t)EFE_NOALLOC_MAX_TILES, needed, st);
}

}  // namespace efe
