// efe_batch.cu -- persistent launch over several element groups of two types (uneven batches of
// meshes), and its variant for callers that cannot allocate device memory.
#include <mutex>

#include "efe_launch.cuh"

namespace efe {

namespace {

// Fill a group table: group k owns ceil(nElements / EPB) tiles.
template <int EPB>
void fill_table(GroupTable& t, const GroupArgs* g, int n) {
  t = GroupTable{};
  t.n = n;
  t.tileStart[0] = 0;
  for (int k = 0; k < MAX_PERSISTENT_GROUPS; ++k) {
    if (k < n) t.g[k] = g[k];
    t.tileStart[k + 1] = t.tileStart[k] + (k < n ? (g[k].nElements + EPB - 1) / EPB : 0);
  }
}

// heavy: Hexa20 3x3x3 total-Lagrangian Neo-Hooke groups, light: Quad8 2x2 total-Lagrangian
// Neo-Hooke groups; the heavier tiles are handed out first
template <typename KT, typename CT>
cudaError_t run_groups(const GroupArgs* heavy, int nHeavy, const GroupArgs* light, int nLight, CT* counter,
                       int64_t maxTiles, int64_t* needed, cudaStream_t st) {
  constexpr int SA = EFE_HEXA20, RA = EFE_RULE_3D_3X3X3, SB = EFE_QUAD8, RB = EFE_RULE_2D_2X2;
  using TA = Tile<SA, RA, TLH, KT>;
  using TB = Tile<SB, RB, TLH, KT>;
  static_assert(TA::NT == TB::NT, "both tile types must use the same CTA size");
  constexpr int NT = TA::NT;
  constexpr size_t bytes = TA::bytes > TB::bytes ? TA::bytes : TB::bytes;
  if (nHeavy < 0 || nLight < 0 || nHeavy > MAX_PERSISTENT_GROUPS || nLight > MAX_PERSISTENT_GROUPS)
    return cudaErrorInvalidValue;
  auto kern = assemble_persistent_kernel<SA, RA, TLH, TA::EPB, SB, RB, TLH, TB::EPB, KT, NT, CT>;
  cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (err != cudaSuccess) return err;
  int dev = 0, sms = 0, perSM = 0;
  if ((err = cudaGetDevice(&dev)) != cudaSuccess) return err;
  if ((err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return err;
  if ((err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kern, NT, bytes)) != cudaSuccess) return err;
  if (perSM < 1) return cudaErrorInvalidConfiguration;
  GroupTable ta, tb;
  fill_table<TA::EPB>(ta, heavy, nHeavy);
  fill_table<TB::EPB>(tb, light, nLight);
  const int64_t tilesA = ta.tileStart[nHeavy], tilesB = tb.tileStart[nLight];
  int64_t grid = (int64_t)sms * perSM;
  if (grid > tilesA + tilesB) grid = tilesA + tilesB;
  // the counter ends at tilesA + tilesB + grid (every CTA takes one tile index past the end)
  if (needed) *needed = tilesA + tilesB + grid;
  if (tilesA + tilesB + grid > maxTiles) return cudaErrorInvalidValue;
  if ((err = cudaMemsetAsync(counter, 0, sizeof(CT), st)) != cudaSuccess) return err;
  if (grid == 0) return cudaSuccess;
  kern<<<(unsigned)grid, NT, bytes, st>>>(ta, tb, counter);
  return cudaGetLastError();
}

template <typename CT>
cudaError_t persistent_groups_t(int kprec, const GroupArgs* heavy, int nHeavy, const GroupArgs* light, int nLight,
                                CT* counter, int64_t maxTiles, int64_t* needed, cudaStream_t st) {
  if (kprec == EFE_K_FP32)
    return run_groups<float>(heavy, nHeavy, light, nLight, counter, maxTiles, needed, st);
  return run_groups<double>(heavy, nHeavy, light, nLight, counter, maxTiles, needed, st);
}

}  // namespace

cudaError_t persistent_groups(int kprec, const GroupArgs* heavy, int nHeavy, const GroupArgs* light, int nLight,
                              unsigned long long* counter, cudaStream_t st) {
  return persistent_groups_t(kprec, heavy, nHeavy, light, nLight, counter, INT64_MAX, nullptr, st);
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

cudaError_t persistent_groups_noalloc(int kprec, const GroupArgs* heavy, int nHeavy, const GroupArgs* light,
                                      int nLight, int64_t* needed, cudaStream_t st) {
  unsigned int* counter = nullptr;
  cudaError_t err = noalloc_scratch_address(&counter);
  if (err != cudaSuccess) return err;
  return persistent_groups_t(kprec, heavy, nHeavy, light, nLight, counter, (int64_t)EFE_NOALLOC_MAX_TILES, needed, st);
}

}  // namespace efe
