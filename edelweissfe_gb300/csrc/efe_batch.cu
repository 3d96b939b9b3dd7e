// efe_batch.cu -- persistent launch over several element groups of mixed types (uneven batches of
// meshes and load cases), and its variant for callers that cannot allocate device memory.
#include <initializer_list>
#include <type_traits>
#include <mutex>

#include "efe_launch.cuh"

namespace efe {

namespace {

// Fill a group table: group k owns ceil(nElements / EPB) tiles.
void fill_table(GroupTable& t, const GroupArgs* g, int n, int EPB) {
  t = GroupTable{};
  t.n = n;
  t.tileStart[0] = 0;
  for (int k = 0; k < MAX_PERSISTENT_GROUPS; ++k) {
    if (k < n) t.g[k] = g[k];
    t.tileStart[k + 1] = t.tileStart[k] + (k < n ? (g[k].nElements + EPB - 1) / EPB : 0);
  }
}

// The element types of the persistent pass by persistent_type_index, each with its variant-0 tile
// (128 threads): the (shape, rule, form, elements per tile) and the tile's shared memory.
// SRC: the persistent_type_index whose groups the type runs.
template <int IDX, typename KT> struct TypeOf;
template <int S, int R, int F, typename KT, int SRC_>
struct TypeOfBase {
  using T = PersistentType<S, R, F, Tile<S, R, F, KT>::EPB>;
  static constexpr size_t bytes = Tile<S, R, F, KT>::bytes;
  static constexpr int NT = Tile<S, R, F, KT>::NT, SRC = SRC_;
};
template <typename KT> struct TypeOf<0, KT> : TypeOfBase<EFE_HEXA20, EFE_RULE_3D_3X3X3, TLH, KT, 0> {};
template <typename KT> struct TypeOf<1, KT> : TypeOfBase<EFE_HEXA20, EFE_RULE_3D_3X3X3, SS3, KT, 1> {};
template <typename KT> struct TypeOf<2, KT> : TypeOfBase<EFE_HEXA8, EFE_RULE_3D_2X2X2, TLH, KT, 2> {};
template <typename KT> struct TypeOf<3, KT> : TypeOfBase<EFE_HEXA8, EFE_RULE_3D_2X2X2, SS3, KT, 3> {};
template <typename KT> struct TypeOf<4, KT> : TypeOfBase<EFE_QUAD8, EFE_RULE_2D_2X2, TLH, KT, 4> {};
// type 0 with its tangent on the tensor cores (tile variant 3, efe_hexa20_tc.cuh; FP32 tangent only)
template <> struct TypeOf<5, float> {
  using T = PersistentType<EFE_HEXA20, EFE_RULE_3D_3X3X3, TLH, 1, true>;
  static constexpr size_t bytes = H20TCLayout<false>::bytes;
  static_assert(H20TCLayout<false>::bytes == H20TCLayout<true>::bytes, "one tile size for both forms");
  static constexpr int NT = 128, SRC = 0;
};

constexpr size_t max_of(std::initializer_list<size_t> v) {
  size_t m = 0;
  for (size_t x : v) m = x > m ? x : m;
  return m;
}

// One persistent kernel over the types IDX... (in that order; every other type must have no groups),
// with registers held to MINB resident CTAs per SM.
template <typename KT, bool FF, typename CT, int MINB, int... IDX>
cudaError_t run_list(const GroupArgs (*groups)[MAX_PERSISTENT_GROUPS], const int* nGroups, CT* counter,
                     int64_t maxTiles, int64_t* needed, cudaStream_t st) {
  constexpr int N = sizeof...(IDX);
  constexpr int idx[N] = {TypeOf<IDX, KT>::SRC...};
  constexpr int epb[N] = {TypeOf<IDX, KT>::T::EPB...};
  constexpr int NT = 128;
  static_assert(((TypeOf<IDX, KT>::NT == NT) && ...), "all tiles of a persistent kernel use 128 threads");
  constexpr size_t bytes = max_of({TypeOf<IDX, KT>::bytes...});
  static_assert(bytes <= 200 * 1024, "persistent tile does not fit in shared memory");
  auto kern = assemble_persistent_kernel<KT, NT, MINB, FF, CT, typename TypeOf<IDX, KT>::T...>;
  cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (err != cudaSuccess) return err;
  // the largest shared-memory partition, so that the grid is sized to every CTA that fits an SM
  err = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
  if (err != cudaSuccess) return err;
  int dev = 0, sms = 0, perSM = 0;
  if ((err = cudaGetDevice(&dev)) != cudaSuccess) return err;
  if ((err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return err;
  // a list with a tensor-core type allocates TMEM (the runtime's occupancy query then answers 1)
  if constexpr ((TypeOf<IDX, KT>::T::TC || ...)) {
    if ((err = resident_ctas_tmem(kern, NT, bytes, (int)H20TC::TMEM_COLS, &perSM)) != cudaSuccess) return err;
  } else {
    if ((err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kern, NT, bytes)) != cudaSuccess) return err;
  }
  if (perSM < 1) return cudaErrorInvalidConfiguration;
  GroupTables<N> tabs;
  int64_t tiles = 0;
  for (int j = 0; j < N; ++j) {
    fill_table(tabs.t[j], groups[idx[j]], nGroups[idx[j]], epb[j]);
    tiles += tabs.t[j].tileStart[nGroups[idx[j]]];
  }
  int64_t grid = (int64_t)sms * perSM;
  if (grid > tiles) grid = tiles;
  // the counter ends at tiles + grid (every CTA takes one tile index past the end)
  if (needed) *needed = tiles + grid;
  if (tiles + grid > maxTiles) return cudaErrorInvalidValue;
  if ((err = cudaMemsetAsync(counter, 0, sizeof(CT), st)) != cudaSuccess) return err;
  if (grid == 0) return cudaSuccess;
  kern<<<(unsigned)grid, NT, bytes, st>>>(tabs, counter, sms);
  return cudaGetLastError();
}

// The smallest instantiated type list covering the types present: total-Lagrangian Neo-Hooke Hexa20
// + Quad8 (batches of uneven 2D/3D meshes; with the FP32 tangent and every Hexa20 group on tile
// variant 3, the Hexa20 tangent on the tensor cores), Hexa8 small strain alone (load cases of one
// material, four CTAs per SM as tile variant 2), or all five types.
template <typename KT, bool FF, typename CT>
cudaError_t run_groups(const GroupArgs (*groups)[MAX_PERSISTENT_GROUPS], const int* nGroups, CT* counter,
                       int64_t maxTiles, int64_t* needed, cudaStream_t st) {
  unsigned present = 0;
  for (int k = 0; k < PERSISTENT_NTYPES; ++k) {
    if (nGroups[k] < 0 || nGroups[k] > MAX_PERSISTENT_GROUPS) return cudaErrorInvalidValue;
    if (nGroups[k] > 0) present |= 1u << k;
  }
  if ((present & ~((1u << 0) | (1u << 4))) == 0) {
    if constexpr (std::is_same<KT, float>::value) {
      // the Hexa20 groups' tangent on the tensor cores when the tile choice says so for all of them
      bool tc = nGroups[0] > 0;
      for (int k = 0; k < nGroups[0]; ++k) tc = tc && groups[0][k].tileVariant == 3;
      if (tc) return run_list<KT, FF, CT, 3, 5, 4>(groups, nGroups, counter, maxTiles, needed, st);
    }
    return run_list<KT, FF, CT, 1, 0, 4>(groups, nGroups, counter, maxTiles, needed, st);
  }
  if ((present & ~(1u << 3)) == 0) return run_list<KT, FF, CT, 4, 3>(groups, nGroups, counter, maxTiles, needed, st);
  return run_list<KT, FF, CT, 2, 0, 1, 2, 3, 4>(groups, nGroups, counter, maxTiles, needed, st);
}

template <typename CT>
cudaError_t persistent_groups_t(int kprec, const GroupArgs (*groups)[MAX_PERSISTENT_GROUPS], const int* nGroups,
                                CT* counter, int64_t maxTiles, int64_t* needed, cudaStream_t st) {
  if (kprec == EFE_K_FP32) return run_groups<float, false>(groups, nGroups, counter, maxTiles, needed, st);
  if (kprec == EFE_K_FP32_FF) return run_groups<float, true>(groups, nGroups, counter, maxTiles, needed, st);
  return run_groups<double, false>(groups, nGroups, counter, maxTiles, needed, st);
}

}  // namespace

cudaError_t persistent_groups(int kprec, const GroupArgs (*groups)[MAX_PERSISTENT_GROUPS], const int* nGroups,
                              unsigned long long* counter, cudaStream_t st) {
  return persistent_groups_t(kprec, groups, nGroups, counter, INT64_MAX, nullptr, st);
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

cudaError_t persistent_groups_noalloc(int kprec, const GroupArgs (*groups)[MAX_PERSISTENT_GROUPS], const int* nGroups,
                                      int64_t* needed, cudaStream_t st) {
  unsigned int* counter = nullptr;
  cudaError_t err = noalloc_scratch_address(&counter);
  if (err != cudaSuccess) return err;
  return persistent_groups_t(kprec, groups, nGroups, counter, (int64_t)EFE_NOALLOC_MAX_TILES, needed, st);
}

}  // namespace efe
