// efe_solve.cu -- CSR matrix-vector products and Jacobi-preconditioned conjugate gradients on the
// free DOFs of the assembled tangent, for the Newton correction (the reference's linearSolve,
// solvers/nonlinearimplicitstatic.py:727-751) and the adjoint systems.
//
// The matrix is the CSR data the element pass assembled (FP32 or FP64 values, int32 pattern); it is
// never converted.  Products accumulate in FP64; vectors are FP64.  The operator is K restricted
// to the free rows (prescribed rows are the identity): CG starts from x = 0 with a right-hand side
// that is zero on the prescribed DOFs, so every search direction is zero there and the column
// restriction comes for free.
//
// One iteration is three kernels: (1) Ap = A p with the partial sums of p.Ap per block, (2) alpha,
// x += alpha p, r -= alpha Ap, z = D^-1 r with the partial sums of r.z and r.r, (3) beta,
// p = z + beta p.  The scalars stay on the device: every block sums the previous kernel's partials
// in the same fixed order, so the iteration is deterministic, and rz is double-buffered by the
// parity of the iteration number so no kernel overwrites a scalar another block is reading.
#include "efe_launch.cuh"

namespace efe {

namespace {

constexpr int NT = 256;                 // threads per block of every kernel here
constexpr int WARPS = NT / 32;
constexpr int MAX_BLOCKS = 2048;        // partial-sum slots per reduction
// work layout (doubles): [0..1] rz (by parity), [2] r.r, [3] p.Ap, [8 ..) three partial arrays
constexpr int PART0 = 8, PART1 = PART0 + MAX_BLOCKS, PART2 = PART1 + MAX_BLOCKS;

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Block sum of v (fixed order); the result is valid in thread 0.
__device__ __forceinline__ double block_sum(double v, double* sh) {
  v = warp_sum(v);
  const int w = threadIdx.x / 32, l = threadIdx.x % 32;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int k = 0; k < WARPS; ++k) s += sh[k];
  return s;
}

// Sum of n partials, the same value in every thread of the block (fixed order).
__device__ __forceinline__ double sum_partials(const double* part, int n, double* sh) {
  double v = 0.0;
  for (int i = threadIdx.x; i < n; i += NT) v += part[i];
  v = block_sum(v, sh);
  __syncthreads();
  if (threadIdx.x == 0) sh[WARPS] = v;
  __syncthreads();
  return sh[WARPS];
}

template <typename KT>
__device__ __forceinline__ double row_product(int64_t r, const int32_t* __restrict__ indptr,
                                              const int32_t* __restrict__ indices, const KT* __restrict__ K,
                                              const double* __restrict__ x, int lane) {
  const int32_t b = indptr[r], e = indptr[r + 1];
  double s = 0.0;
  for (int32_t j = b + lane; j < e; j += 32) s = fma((double)K[j], x[indices[j]], s);
  return warp_sum(s);
}

// y_i = free_i ? (K x)_i : x_i; with part != null also the block partials of x.y.
template <typename KT>
__global__ void __launch_bounds__(NT) spmv_kernel(int64_t n, const int32_t* __restrict__ indptr,
                                                  const int32_t* __restrict__ indices, const KT* __restrict__ K,
                                                  const uint8_t* __restrict__ freeMask, const double* __restrict__ x,
                                                  double* __restrict__ y, double* part) {
  __shared__ double sh[WARPS + 1];
  const int lane = threadIdx.x % 32;
  const int64_t warp = ((int64_t)blockIdx.x * NT + threadIdx.x) / 32;
  const int64_t nw = (int64_t)gridDim.x * WARPS;
  double acc = 0.0;
  for (int64_t r = warp; r < n; r += nw) {
    const double v = row_product(r, indptr, indices, K, x, lane);
    if (lane == 0) {
      const double yr = (!freeMask || freeMask[r]) ? v : x[r];
      y[r] = yr;
      acc = fma(x[r], yr, acc);
    }
  }
  if (part) {
    const double s = block_sum(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
  }
}

// r = b, z = dinv r, p = z (x = 0); partials of r.z and r.r
__global__ void __launch_bounds__(NT) pcg_start_kernel(int64_t n, const double* __restrict__ b,
                                                       const double* __restrict__ dinv, double* __restrict__ x,
                                                       double* __restrict__ r, double* __restrict__ z,
                                                       double* __restrict__ p, double* work) {
  __shared__ double sh[WARPS + 1];
  double rz = 0.0, rr = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT) {
    const double ri = b[i], zi = dinv[i] * ri;
    x[i] = 0.0;
    r[i] = ri;
    z[i] = zi;
    p[i] = zi;
    rz = fma(ri, zi, rz);
    rr = fma(ri, ri, rr);
  }
  const double s1 = block_sum(rz, sh);
  if (threadIdx.x == 0) work[PART1 + blockIdx.x] = s1;
  const double s2 = block_sum(rr, sh);
  if (threadIdx.x == 0) work[PART2 + blockIdx.x] = s2;
}

__global__ void __launch_bounds__(NT) pcg_start_finish(double* work, int nb) {
  __shared__ double sh[WARPS + 1];
  const double rz = sum_partials(work + PART1, nb, sh);
  const double rr = sum_partials(work + PART2, nb, sh);
  if (threadIdx.x == 0) {
    work[0] = rz;
    work[1] = 0.0;
    work[2] = rr;
    work[3] = 0.0;
  }
}

// alpha = rz[cur] / p.Ap; x += alpha p; r -= alpha Ap; z = dinv r; partials of r.z (PART1), r.r (PART2)
__global__ void __launch_bounds__(NT) pcg_update_kernel(int64_t n, int cur, int nbSpmv, const double* __restrict__ p,
                                                        const double* __restrict__ Ap, const double* __restrict__ dinv,
                                                        double* __restrict__ x, double* __restrict__ r,
                                                        double* __restrict__ z, double* work) {
  __shared__ double sh[WARPS + 1];
  const double pAp = sum_partials(work + PART0, nbSpmv, sh);
  const double alpha = pAp != 0.0 ? work[cur] / pAp : 0.0;
  double rz = 0.0, rr = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT) {
    x[i] = fma(alpha, p[i], x[i]);
    const double ri = fma(-alpha, Ap[i], r[i]);
    const double zi = dinv[i] * ri;
    r[i] = ri;
    z[i] = zi;
    rz = fma(ri, zi, rz);
    rr = fma(ri, ri, rr);
  }
  const double s1 = block_sum(rz, sh);
  if (threadIdx.x == 0) work[PART1 + blockIdx.x] = s1;
  const double s2 = block_sum(rr, sh);
  if (threadIdx.x == 0) {
    work[PART2 + blockIdx.x] = s2;
    if (blockIdx.x == 0) work[3] = pAp;
  }
}

// beta = rz_new / rz[cur]; p = z + beta p; block 0 stores rz_new in rz[cur ^ 1] and r.r in work[2]
__global__ void __launch_bounds__(NT) pcg_direction_kernel(int64_t n, int cur, int nbVec, const double* __restrict__ z,
                                                           double* __restrict__ p, double* work) {
  __shared__ double sh[WARPS + 1];
  const double rzNew = sum_partials(work + PART1, nbVec, sh);
  const double rzOld = work[cur];
  const double beta = rzOld != 0.0 ? rzNew / rzOld : 0.0;
  for (int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT)
    p[i] = fma(beta, p[i], z[i]);
  if (blockIdx.x == 0) {
    const double rr = sum_partials(work + PART2, nbVec, sh);
    if (threadIdx.x == 0) {
      work[cur ^ 1] = rzNew;
      work[2] = rr;
    }
  }
}

int vec_blocks(int64_t n, int sms) {
  int64_t b = (n + NT - 1) / NT;
  const int64_t cap = (int64_t)sms * 4;
  if (b > cap) b = cap;
  if (b > MAX_BLOCKS) b = MAX_BLOCKS;
  return (int)(b < 1 ? 1 : b);
}

int spmv_blocks(int64_t n, int sms) {
  int64_t b = (n + WARPS - 1) / WARPS;
  const int64_t cap = (int64_t)sms * 8;
  if (b > cap) b = cap;
  if (b > MAX_BLOCKS) b = MAX_BLOCKS;
  return (int)(b < 1 ? 1 : b);
}

int sm_count() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      sms = 152;
  }
  return sms;
}

template <typename KT>
cudaError_t spmv_t(const EfePcg& s, const double* x, double* y, double* part, int nb, cudaStream_t st) {
  spmv_kernel<KT><<<nb, NT, 0, st>>>(s.n, s.indptr, s.indices, static_cast<const KT*>(s.Kdata), s.freeMask, x, y,
                                      part);
  return cudaGetLastError();
}

cudaError_t spmv(const EfePcg& s, const double* x, double* y, double* part, int nb, cudaStream_t st) {
  return s.kPrecision == EFE_K_FP64 ? spmv_t<double>(s, x, y, part, nb, st) : spmv_t<float>(s, x, y, part, nb, st);
}

}  // namespace

cudaError_t csr_spmv(const EfePcg& s, const double* x, double* y, cudaStream_t st) {
  if (s.n == 0) return cudaSuccess;
  return spmv(s, x, y, nullptr, spmv_blocks(s.n, sm_count()), st);
}

cudaError_t pcg_start(const EfePcg& s, const double* b, cudaStream_t st) {
  const int nb = vec_blocks(s.n, sm_count());
  pcg_start_kernel<<<nb, NT, 0, st>>>(s.n, b, s.dinv, s.x, s.r, s.z, s.p, s.work);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  pcg_start_finish<<<1, NT, 0, st>>>(s.work, nb);
  return cudaGetLastError();
}

cudaError_t pcg_iterate(const EfePcg& s, int64_t k0, int nIter, cudaStream_t st) {
  const int sms = sm_count();
  const int nbS = spmv_blocks(s.n, sms), nbV = vec_blocks(s.n, sms);
  for (int k = 0; k < nIter; ++k) {
    const int cur = (int)((k0 + k) & 1);
    cudaError_t e = spmv(s, s.p, s.Ap, s.work + PART0, nbS, st);
    if (e != cudaSuccess) return e;
    pcg_update_kernel<<<nbV, NT, 0, st>>>(s.n, cur, nbS, s.p, s.Ap, s.dinv, s.x, s.r, s.z, s.work);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    pcg_direction_kernel<<<nbV, NT, 0, st>>>(s.n, cur, nbV, s.z, s.p, s.work);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace efe
