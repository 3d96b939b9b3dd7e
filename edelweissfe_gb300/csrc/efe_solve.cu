// efe_solve.cu -- CSR matrix-vector products and Jacobi-preconditioned conjugate gradients on the
// free DOFs of the assembled tangent, for the Newton correction (the reference's linearSolve,
// solvers/nonlinearimplicitstatic.py:727-751) and the adjoint systems.
//
// The matrix is the CSR data the element pass assembled (FP32 or FP64 values, int32 pattern); it is
// never converted.  Vectors and scalars are FP64.  The operator is K restricted
// to the free rows (prescribed rows are the identity): CG starts from x = 0 with a right-hand side
// that is zero on the prescribed DOFs, so every search direction is zero there and the column
// restriction comes for free.
//
// Precision of the product.  This part issues FP64 at ~1/60 of its FP32 rate, so a product that
// spends even two FP64 operations per stored entry (a float->double conversion and a DFMA) is
// bound by the FP64 pipe, not by memory.  For FP32 tangents the CG iterations therefore keep the
// search direction also as float-float pairs (pFF[i] = (hi, lo), ~48-bit significand, written once per DOF
// by the vector kernels) and form every product and partial sum in float-float arithmetic on the
// FP32 pipe: k * (xh + xl) = fl(k xh) + [fma(k, xh, -fl(k xh)) + k xl], accumulated with
// error-free sums; one conversion to double per row.  The result carries ~2^-48 relative error of
// sum |K_ij x_j| -- below the attainable accuracy of a CG residual at any tolerance used here, and
// the Newton and adjoint drivers check their solutions with FP64 residuals.  FP64 tangents use
// DFMA.  Eight lanes per row (four rows per warp) keep the cross-lane reduction short.
//
// Preconditioner: the inverse of the diagonal (blockSize 1) or of the nodal diagonal blocks
// (blockSize = 2 or 3 consecutive DOFs, the node's displacement components), built by the caller.
// The building blocks of a multilevel preconditioner are here too: a general CSR product
// y = alpha A x + beta y (rectangular for the transfer operators, masked for the tangent) and the
// vector step of a Chebyshev smoother; the host composes them into V-cycles.
//
// One iteration is three kernels: (1) Ap = A p with the partial sums of p.Ap per block, (2) alpha,
// x += alpha p, r -= alpha Ap, z = M^-1 r with the partial sums of r.z and r.r, (3) beta,
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

constexpr int G = 8;  // lanes per row

__device__ __forceinline__ double group_sum(double v) {
  v += __shfl_xor_sync(0xffffffffu, v, 4);
  v += __shfl_xor_sync(0xffffffffu, v, 2);
  v += __shfl_xor_sync(0xffffffffu, v, 1);
  return v;
}

// (h, l) += (a, b): error-free sum of the high parts, low parts added
__device__ __forceinline__ void ff_acc(float& h, float& l, float a, float b) {
  const float s = __fadd_rn(h, a);
  const float bb = __fsub_rn(s, h);
  const float err = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(a, bb));
  l = __fadd_rn(l, __fadd_rn(err, b));
  h = s;
}
// (h, l) += k * (xh + xl)
__device__ __forceinline__ void ff_madd(float& h, float& l, float k, float xh, float xl) {
  const float p = __fmul_rn(k, xh);
  float e = __fmaf_rn(k, xh, -p);
  e = __fmaf_rn(k, xl, e);
  ff_acc(h, l, p, e);
}

// (K x)_r with FP64 arithmetic (double or float values); every lane of the row's group gets it
template <typename KT>
__device__ __forceinline__ double row_product(int32_t b, int32_t e, const int32_t* __restrict__ indices,
                                              const KT* __restrict__ K, const double* __restrict__ x, int sl) {
  // four independent loads per lane per step: the rows of solid tangents hold 81-243 entries
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
  for (int32_t j = b + sl; j < e; j += 4 * G) {
    const bool p1 = j + G < e, p2 = j + 2 * G < e, p3 = j + 3 * G < e;
    const int32_t c0 = indices[j];
    const int32_t c1 = p1 ? indices[j + G] : c0, c2 = p2 ? indices[j + 2 * G] : c0, c3 = p3 ? indices[j + 3 * G] : c0;
    const double k0 = (double)K[j], k1 = p1 ? (double)K[j + G] : 0.0, k2 = p2 ? (double)K[j + 2 * G] : 0.0,
                 k3 = p3 ? (double)K[j + 3 * G] : 0.0;
    s0 = fma(k0, x[c0], s0);
    s1 = fma(k1, x[c1], s1);
    s2 = fma(k2, x[c2], s2);
    s3 = fma(k3, x[c3], s3);
  }
  return group_sum((s0 + s1) + (s2 + s3));
}

// (K x)_r with float values and x = xh + xl in float-float arithmetic (FP32 pipe only); four
// independent entries per lane and step keep enough gathers in flight to approach DRAM speed
__device__ __forceinline__ double row_product_ff(int32_t b, int32_t e, const int32_t* __restrict__ indices,
                                                 const float* __restrict__ K, const float2* __restrict__ xf, int sl) {
  float h0 = 0.f, l0 = 0.f, h1 = 0.f, l1 = 0.f, h2 = 0.f, l2 = 0.f, h3 = 0.f, l3 = 0.f;
  for (int32_t j = b + sl; j < e; j += 4 * G) {
    const bool p1 = j + G < e, p2 = j + 2 * G < e, p3 = j + 3 * G < e;
    const int32_t c0 = indices[j];
    const int32_t c1 = p1 ? indices[j + G] : c0, c2 = p2 ? indices[j + 2 * G] : c0, c3 = p3 ? indices[j + 3 * G] : c0;
    const float k0 = K[j], k1 = p1 ? K[j + G] : 0.f, k2 = p2 ? K[j + 2 * G] : 0.f, k3 = p3 ? K[j + 3 * G] : 0.f;
    const float2 x0 = xf[c0], x1 = xf[c1], x2 = xf[c2], x3 = xf[c3];
    ff_madd(h0, l0, k0, x0.x, x0.y);
    ff_madd(h1, l1, k1, x1.x, x1.y);
    ff_madd(h2, l2, k2, x2.x, x2.y);
    ff_madd(h3, l3, k3, x3.x, x3.y);
  }
  ff_acc(h0, l0, h1, l1);
  ff_acc(h2, l2, h3, l3);
  ff_acc(h0, l0, h2, l2);
  for (int o = 4; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, h0, o), ol = __shfl_xor_sync(0xffffffffu, l0, o);
    ff_acc(h0, l0, oh, ol);
  }
  return (double)h0 + (double)l0;
}

// (K x) for the PB rows r0 .. r0+PB-1 of one node, which share one column list (the nodal DOF
// rows of an assembled tangent): each column index and x pair is read once for the PB rows, so a
// stored entry costs 4 + 4/PB bytes instead of 8.  Float values, x as float-float pairs, sums in
// float-float arithmetic.  Values of a row are read only within that row's own length, so a
// pattern without the shared-column property still reads inside the arrays.
template <int PB>
__device__ __forceinline__ void group_product_ff(const int32_t* __restrict__ indptr, int64_t r0, bool live,
                                                 const int32_t* __restrict__ indices, const float* __restrict__ K,
                                                 const float2* __restrict__ xf, int sl, double out[PB]) {
  int32_t bc[PB], lc[PB];
#pragma unroll
  for (int c = 0; c < PB; ++c) {
    bc[c] = live ? indptr[r0 + c] : 0;
    lc[c] = live ? indptr[r0 + c + 1] - bc[c] : 0;
  }
  float h0[PB], l0[PB], h1[PB], l1[PB];
#pragma unroll
  for (int c = 0; c < PB; ++c) h0[c] = l0[c] = h1[c] = l1[c] = 0.f;
  const int32_t len = lc[0];
  for (int32_t t = sl; t < len; t += 2 * G) {
    const bool p1 = t + G < len;
    const int32_t c0 = indices[bc[0] + t];
    const int32_t c1 = p1 ? indices[bc[0] + t + G] : c0;
    const float2 x0 = xf[c0], x1 = xf[c1];
#pragma unroll
    for (int c = 0; c < PB; ++c) {
      const float k0 = t < lc[c] ? K[bc[c] + t] : 0.f;
      const float k1 = (p1 && t + G < lc[c]) ? K[bc[c] + t + G] : 0.f;
      ff_madd(h0[c], l0[c], k0, x0.x, x0.y);
      ff_madd(h1[c], l1[c], k1, x1.x, x1.y);
    }
  }
#pragma unroll
  for (int c = 0; c < PB; ++c) {
    float h = h0[c], l = l0[c];
    ff_acc(h, l, h1[c], l1[c]);
    for (int o = 4; o > 0; o >>= 1) {
      const float oh = __shfl_xor_sync(0xffffffffu, h, o), ol = __shfl_xor_sync(0xffffffffu, l, o);
      ff_acc(h, l, oh, ol);
    }
    out[c] = (double)h + (double)l;
  }
}

// The float-float CG product over node row groups of PB rows (spmv_kernel<float, true> otherwise).
template <int PB>
__global__ void __launch_bounds__(NT) spmv_group_ff_kernel(int64_t n, const int32_t* __restrict__ indptr,
                                                           const int32_t* __restrict__ indices,
                                                           const float* __restrict__ K,
                                                           const uint8_t* __restrict__ freeMask,
                                                           const double* __restrict__ x, const float2* __restrict__ xf,
                                                           double* __restrict__ y, double* part) {
  __shared__ double sh[WARPS + 1];
  const int lane = threadIdx.x % 32, g = lane / G, sl = lane % G;
  constexpr int GPW = 32 / G;  // row groups per warp and step
  const int64_t warp = ((int64_t)blockIdx.x * NT + threadIdx.x) / 32;
  const int64_t nw = (int64_t)gridDim.x * WARPS;
  const int64_t nGroups = n / PB;
  double acc = 0.0;
  // the loop condition depends on the warp only: all 32 lanes reach every shuffle
  for (int64_t gb = warp * GPW; gb < nGroups; gb += nw * GPW) {
    const int64_t gi = gb + g;
    const bool live = gi < nGroups;
    double v[PB];
    group_product_ff<PB>(indptr, gi * PB, live, indices, K, xf, sl, v);
    if (live && sl == 0) {
#pragma unroll
      for (int c = 0; c < PB; ++c) {
        const int64_t r = gi * PB + c;
        const double yr = (!freeMask || freeMask[r]) ? v[c] : x[r];
        y[r] = yr;
        acc = fma(x[r], yr, acc);
      }
    }
  }
  if (part) {
    const double s = block_sum(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
  }
}

// y_r = free_r ? (K x)_r : x_r for rows r; with part != null also the block partials of x.y.
// FF: x is also given as the float-float pairs xf and K is float (the CG iterations of FP32 tangents).
template <typename KT, bool FF>
__global__ void __launch_bounds__(NT) spmv_kernel(int64_t n, const int32_t* __restrict__ indptr,
                                                  const int32_t* __restrict__ indices, const KT* __restrict__ K,
                                                  const uint8_t* __restrict__ freeMask, const double* __restrict__ x,
                                                  const float2* __restrict__ xf, double* __restrict__ y,
                                                  double* part) {
  __shared__ double sh[WARPS + 1];
  const int lane = threadIdx.x % 32, g = lane / G, sl = lane % G;
  constexpr int RPW = 32 / G;  // rows per warp and step
  const int64_t warp = ((int64_t)blockIdx.x * NT + threadIdx.x) / 32;
  const int64_t nw = (int64_t)gridDim.x * WARPS;
  double acc = 0.0;
  // the loop condition depends on the warp only: all 32 lanes reach every shuffle
  for (int64_t rb = warp * RPW; rb < n; rb += nw * RPW) {
    const int64_t r = rb + g;
    const bool live = r < n;
    const int32_t b = live ? indptr[r] : 0, e = live ? indptr[r + 1] : 0;
    double v;
    if constexpr (FF)
      v = row_product_ff(b, e, indices, reinterpret_cast<const float*>(K), xf, sl);
    else
      v = row_product(b, e, indices, K, x, sl);
    if (live && sl == 0) {
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

// z = M^-1 r on one block of BS consecutive DOFs (BS = 1: point Jacobi; 2, 3: the inverse of the
// node's diagonal block, [BS][BS] row-major per block)
template <int BS>
__device__ __forceinline__ void precondition(const double* __restrict__ dinv, int64_t blk, const double r[BS],
                                             double z[BS]) {
  const double* D = dinv + blk * BS * BS;
#pragma unroll
  for (int i = 0; i < BS; ++i) {
    double v = 0.0;
#pragma unroll
    for (int j = 0; j < BS; ++j) v = fma(D[i * BS + j], r[j], v);
    z[i] = v;
  }
}

__device__ __forceinline__ void split_ff(double v, float2* pf, int64_t i) {
  const float h = __double2float_rn(v);
  pf[i] = make_float2(h, __double2float_rn(v - (double)h));
}

// r = b, z = M^-1 r, p = z (x = 0); partials of r.z and r.r; one thread per block of BS DOFs
template <int BS>
__global__ void __launch_bounds__(NT) pcg_start_kernel(int64_t n, const double* __restrict__ b,
                                                       const double* __restrict__ dinv, double* __restrict__ x,
                                                       double* __restrict__ r, double* __restrict__ z,
                                                       double* __restrict__ p, float2* __restrict__ pf,
                                                       double* work) {
  __shared__ double sh[WARPS + 1];
  double rz = 0.0, rr = 0.0;
  const int64_t nb = n / BS;
  for (int64_t k = (int64_t)blockIdx.x * NT + threadIdx.x; k < nb; k += (int64_t)gridDim.x * NT) {
    double rv[BS], zv[BS];
#pragma unroll
    for (int c = 0; c < BS; ++c) rv[c] = b[k * BS + c];
    precondition<BS>(dinv, k, rv, zv);
#pragma unroll
    for (int c = 0; c < BS; ++c) {
      const int64_t i = k * BS + c;
      x[i] = 0.0;
      r[i] = rv[c];
      z[i] = zv[c];
      p[i] = zv[c];
      if (pf) split_ff(zv[c], pf, i);
      rz = fma(rv[c], zv[c], rz);
      rr = fma(rv[c], rv[c], rr);
    }
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

// alpha = rz[cur] / p.Ap; x += alpha p; r -= alpha Ap; z = M^-1 r; partials of r.z (PART1), r.r (PART2)
template <int BS>
__global__ void __launch_bounds__(NT) pcg_update_kernel(int64_t n, int cur, int nbSpmv, const double* __restrict__ p,
                                                        const double* __restrict__ Ap, const double* __restrict__ dinv,
                                                        double* __restrict__ x, double* __restrict__ r,
                                                        double* __restrict__ z, double* work) {
  __shared__ double sh[WARPS + 1];
  const double pAp = sum_partials(work + PART0, nbSpmv, sh);
  const double alpha = pAp != 0.0 ? work[cur] / pAp : 0.0;
  double rz = 0.0, rr = 0.0;
  const int64_t nb = n / BS;
  for (int64_t k = (int64_t)blockIdx.x * NT + threadIdx.x; k < nb; k += (int64_t)gridDim.x * NT) {
    double rv[BS], zv[BS];
#pragma unroll
    for (int c = 0; c < BS; ++c) {
      const int64_t i = k * BS + c;
      x[i] = fma(alpha, p[i], x[i]);
      rv[c] = fma(-alpha, Ap[i], r[i]);
      r[i] = rv[c];
    }
    precondition<BS>(dinv, k, rv, zv);
#pragma unroll
    for (int c = 0; c < BS; ++c) {
      z[k * BS + c] = zv[c];
      rz = fma(rv[c], zv[c], rz);
      rr = fma(rv[c], rv[c], rr);
    }
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
                                                           double* __restrict__ p, float2* __restrict__ pf,
                                                           double* work) {
  __shared__ double sh[WARPS + 1];
  const double rzNew = sum_partials(work + PART1, nbVec, sh);
  const double rzOld = work[cur];
  const double beta = rzOld != 0.0 ? rzNew / rzOld : 0.0;
  for (int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT) {
    const double pi = fma(beta, p[i], z[i]);
    p[i] = pi;
    if (pf) {  // float-float copy for the FP32 product: pi = h + l to ~48 bits
      const float h = __double2float_rn(pi);
      pf[i] = make_float2(h, __double2float_rn(pi - (double)h));
    }
  }
  if (blockIdx.x == 0) {
    const double rr = sum_partials(work + PART2, nbVec, sh);
    if (threadIdx.x == 0) {
      work[cur ^ 1] = rzNew;
      work[2] = rr;
    }
  }
}

// y = alpha A x + beta y over the rows of a CSR matrix with FP64 arithmetic (rectangular allowed);
// with freeMask, row r is the identity where freeMask[r] == 0 (then A is square).  beta == 0: y is
// not read.
template <typename KT>
__global__ void __launch_bounds__(NT) gemv_kernel(int64_t nRows, const int32_t* __restrict__ indptr,
                                                  const int32_t* __restrict__ indices, const KT* __restrict__ A,
                                                  const uint8_t* __restrict__ freeMask, const double* __restrict__ x,
                                                  double alpha, double beta, double* __restrict__ y) {
  const int lane = threadIdx.x % 32, g = lane / G, sl = lane % G;
  constexpr int RPW = 32 / G;
  const int64_t warp = ((int64_t)blockIdx.x * NT + threadIdx.x) / 32;
  const int64_t nw = (int64_t)gridDim.x * WARPS;
  // the loop condition depends on the warp only: all 32 lanes reach every shuffle
  for (int64_t rb = warp * RPW; rb < nRows; rb += nw * RPW) {
    const int64_t r = rb + g;
    const bool live = r < nRows;
    const int32_t b = live ? indptr[r] : 0, e = live ? indptr[r + 1] : 0;
    const double v = row_product(b, e, indices, A, x, sl);
    if (live && sl == 0) {
      const double ax = (!freeMask || freeMask[r]) ? v : x[r];
      y[r] = beta == 0.0 ? alpha * ax : fma(alpha, ax, beta * y[r]);
    }
  }
}

// y = alpha A x + beta y with float values and x given as float-float pairs xf[i] = (hi, lo):
// products and row sums in float-float arithmetic on the FP32 pipe (as the CG products of FP32
// tangents), one conversion to double per row.  Masked rows are the identity (x_r = hi + lo).
__global__ void __launch_bounds__(NT) gemv_pairs_kernel(int64_t nRows, const int32_t* __restrict__ indptr,
                                                        const int32_t* __restrict__ indices,
                                                        const float* __restrict__ A,
                                                        const uint8_t* __restrict__ freeMask,
                                                        const float2* __restrict__ xf, double alpha, double beta,
                                                        double* __restrict__ y) {
  const int lane = threadIdx.x % 32, g = lane / G, sl = lane % G;
  constexpr int RPW = 32 / G;
  const int64_t warp = ((int64_t)blockIdx.x * NT + threadIdx.x) / 32;
  const int64_t nw = (int64_t)gridDim.x * WARPS;
  for (int64_t rb = warp * RPW; rb < nRows; rb += nw * RPW) {
    const int64_t r = rb + g;
    const bool live = r < nRows;
    const int32_t b = live ? indptr[r] : 0, e = live ? indptr[r + 1] : 0;
    const double v = row_product_ff(b, e, indices, A, xf, sl);
    if (live && sl == 0) {
      double ax = v;
      if (freeMask && !freeMask[r]) {
        const float2 xr = xf[r];
        ax = (double)xr.x + (double)xr.y;
      }
      y[r] = beta == 0.0 ? alpha * ax : fma(alpha, ax, beta * y[r]);
    }
  }
}

// The same product with one thread per row, for matrices whose rows hold a few entries (the
// prolongation between levels: one entry per row), where eight lanes per row would mostly idle.
template <typename KT>
__global__ void __launch_bounds__(NT) gemv_rows_kernel(int64_t nRows, const int32_t* __restrict__ indptr,
                                                       const int32_t* __restrict__ indices, const KT* __restrict__ A,
                                                       const uint8_t* __restrict__ freeMask,
                                                       const double* __restrict__ x, double alpha, double beta,
                                                       double* __restrict__ y) {
  for (int64_t r = (int64_t)blockIdx.x * NT + threadIdx.x; r < nRows; r += (int64_t)gridDim.x * NT) {
    double v = 0.0;
    const int32_t e = indptr[r + 1];
    for (int32_t j = indptr[r]; j < e; ++j) v = fma((double)A[j], x[indices[j]], v);
    const double ax = (!freeMask || freeMask[r]) ? v : x[r];
    y[r] = beta == 0.0 ? alpha * ax : fma(alpha, ax, beta * y[r]);
  }
}

// gemv_pairs_kernel over node row groups of PB rows sharing one column list.
template <int PB>
__global__ void __launch_bounds__(NT) gemv_pairs_group_kernel(int64_t nRows, const int32_t* __restrict__ indptr,
                                                              const int32_t* __restrict__ indices,
                                                              const float* __restrict__ A,
                                                              const uint8_t* __restrict__ freeMask,
                                                              const float2* __restrict__ xf, double alpha, double beta,
                                                              double* __restrict__ y) {
  const int lane = threadIdx.x % 32, g = lane / G, sl = lane % G;
  constexpr int GPW = 32 / G;
  const int64_t warp = ((int64_t)blockIdx.x * NT + threadIdx.x) / 32;
  const int64_t nw = (int64_t)gridDim.x * WARPS;
  const int64_t nGroups = nRows / PB;
  for (int64_t gb = warp * GPW; gb < nGroups; gb += nw * GPW) {
    const int64_t gi = gb + g;
    const bool live = gi < nGroups;
    double v[PB];
    group_product_ff<PB>(indptr, gi * PB, live, indices, A, xf, sl, v);
    if (live && sl == 0) {
#pragma unroll
      for (int c = 0; c < PB; ++c) {
        const int64_t r = gi * PB + c;
        double ax = v[c];
        if (freeMask && !freeMask[r]) {
          const float2 xr = xf[r];
          ax = (double)xr.x + (double)xr.y;
        }
        y[r] = beta == 0.0 ? alpha * ax : fma(alpha, ax, beta * y[r]);
      }
    }
  }
}

// One Chebyshev smoother step on point-Jacobi-scaled residuals: d = c1 d + c2 dinv r (d not read
// when c1 == 0), then z += d (accumulate) or z = d; with dff, also d as float-float pairs.
__global__ void __launch_bounds__(NT) chebyshev_kernel(int64_t n, const double* __restrict__ dinv,
                                                       const double* __restrict__ r, double c1, double c2,
                                                       int accumulate, double* __restrict__ d,
                                                       double* __restrict__ z, float2* __restrict__ dff) {
  for (int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT) {
    const double s = c2 * (dinv[i] * r[i]);
    const double di = c1 == 0.0 ? s : fma(c1, d[i], s);
    d[i] = di;
    z[i] = accumulate ? z[i] + di : di;
    if (dff) split_ff(di, dff, i);
  }
}

// xf[i] = (hi, lo) with hi = fl32(x_i), lo = fl32(x_i - hi)
__global__ void __launch_bounds__(NT) split_kernel(int64_t n, const double* __restrict__ x, float2* __restrict__ xf) {
  for (int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT) split_ff(x[i], xf, i);
}

int vec_blocks(int64_t n, int sms) {
  int64_t b = (n + NT - 1) / NT;
  const int64_t cap = (int64_t)sms * 4;
  if (b > cap) b = cap;
  if (b > MAX_BLOCKS) b = MAX_BLOCKS;
  return (int)(b < 1 ? 1 : b);
}

int spmv_blocks(int64_t n, int sms) {
  int64_t b = (n + WARPS * (32 / G) - 1) / (WARPS * (32 / G));
  const int64_t cap = (int64_t)sms * 6;  // resident blocks at <= 40 registers per thread
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

bool use_ff(const EfePcg& s) { return s.kPrecision != EFE_K_FP64 && s.pFF; }
float2* pff(const EfePcg& s) { return use_ff(s) ? reinterpret_cast<float2*>(s.pFF) : nullptr; }

template <typename KT, bool FF>
cudaError_t spmv_t(const EfePcg& s, const double* x, const float2* xf, double* y, double* part, int nb,
                   cudaStream_t st) {
  spmv_kernel<KT, FF><<<nb, NT, 0, st>>>(s.n, s.indptr, s.indices, static_cast<const KT*>(s.Kdata), s.freeMask, x, xf,
                                          y, part);
  return cudaGetLastError();
}

// float-float product of an FP32 tangent, over node row groups where the pattern has them
cudaError_t spmv_pairs(const EfePcg& s, const double* x, const float2* xf, double* y, double* part, int nb,
                       cudaStream_t st) {
  const float* K = static_cast<const float*>(s.Kdata);
  if (s.patternBlock == 3 && s.n % 3 == 0)
    spmv_group_ff_kernel<3><<<nb, NT, 0, st>>>(s.n, s.indptr, s.indices, K, s.freeMask, x, xf, y, part);
  else if (s.patternBlock == 2 && s.n % 2 == 0)
    spmv_group_ff_kernel<2><<<nb, NT, 0, st>>>(s.n, s.indptr, s.indices, K, s.freeMask, x, xf, y, part);
  else
    return spmv_t<float, true>(s, x, xf, y, part, nb, st);
  return cudaGetLastError();
}

// FP64 arithmetic product (any x)
cudaError_t spmv(const EfePcg& s, const double* x, double* y, double* part, int nb, cudaStream_t st) {
  return s.kPrecision == EFE_K_FP64 ? spmv_t<double, false>(s, x, nullptr, y, part, nb, st)
                                    : spmv_t<float, false>(s, x, nullptr, y, part, nb, st);
}

}  // namespace

cudaError_t csr_gemv(const EfeCsr& a, const double* x, double alpha, double beta, double* y, cudaStream_t st) {
  if (a.nRows == 0) return cudaSuccess;
  if (a.nnz <= 2 * a.nRows) {  // short rows: one thread per row
    const int nv = vec_blocks(a.nRows, sm_count());
    if (a.kPrecision == EFE_K_FP64)
      gemv_rows_kernel<double><<<nv, NT, 0, st>>>(a.nRows, a.indptr, a.indices, static_cast<const double*>(a.values),
                                                  a.freeMask, x, alpha, beta, y);
    else
      gemv_rows_kernel<float><<<nv, NT, 0, st>>>(a.nRows, a.indptr, a.indices, static_cast<const float*>(a.values),
                                                 a.freeMask, x, alpha, beta, y);
    return cudaGetLastError();
  }
  const int nb = spmv_blocks(a.nRows, sm_count());
  if (a.kPrecision == EFE_K_FP64)
    gemv_kernel<double><<<nb, NT, 0, st>>>(a.nRows, a.indptr, a.indices, static_cast<const double*>(a.values),
                                           a.freeMask, x, alpha, beta, y);
  else
    gemv_kernel<float><<<nb, NT, 0, st>>>(a.nRows, a.indptr, a.indices, static_cast<const float*>(a.values),
                                          a.freeMask, x, alpha, beta, y);
  return cudaGetLastError();
}

cudaError_t csr_gemv_pairs(const EfeCsr& a, const float2* xf, double alpha, double beta, double* y,
                           cudaStream_t st) {
  if (a.nRows == 0) return cudaSuccess;
  const int nb = spmv_blocks(a.nRows, sm_count());
  const float* A = static_cast<const float*>(a.values);
  if (a.rowBlock == 3 && a.nRows % 3 == 0 && a.nRows == a.nCols)
    gemv_pairs_group_kernel<3><<<nb, NT, 0, st>>>(a.nRows, a.indptr, a.indices, A, a.freeMask, xf, alpha, beta, y);
  else if (a.rowBlock == 2 && a.nRows % 2 == 0 && a.nRows == a.nCols)
    gemv_pairs_group_kernel<2><<<nb, NT, 0, st>>>(a.nRows, a.indptr, a.indices, A, a.freeMask, xf, alpha, beta, y);
  else
    gemv_pairs_kernel<<<nb, NT, 0, st>>>(a.nRows, a.indptr, a.indices, A, a.freeMask, xf, alpha, beta, y);
  return cudaGetLastError();
}

cudaError_t chebyshev_step(int64_t n, const double* dinv, const double* r, double c1, double c2, int accumulate,
                           double* d, double* z, float2* dff, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  chebyshev_kernel<<<vec_blocks(n, sm_count()), NT, 0, st>>>(n, dinv, r, c1, c2, accumulate, d, z, dff);
  return cudaGetLastError();
}

cudaError_t split_pairs(int64_t n, const double* x, float2* xf, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  split_kernel<<<vec_blocks(n, sm_count()), NT, 0, st>>>(n, x, xf);
  return cudaGetLastError();
}

cudaError_t csr_spmv(const EfePcg& s, const double* x, double* y, cudaStream_t st) {
  if (s.n == 0) return cudaSuccess;
  return spmv(s, x, y, nullptr, spmv_blocks(s.n, sm_count()), st);
}

cudaError_t pcg_start(const EfePcg& s, const double* b, cudaStream_t st) {
  const int nb = vec_blocks(s.n, sm_count());
  switch (s.blockSize) {
    case 1: pcg_start_kernel<1><<<nb, NT, 0, st>>>(s.n, b, s.dinv, s.x, s.r, s.z, s.p, pff(s), s.work); break;
    case 2: pcg_start_kernel<2><<<nb, NT, 0, st>>>(s.n, b, s.dinv, s.x, s.r, s.z, s.p, pff(s), s.work); break;
    default: pcg_start_kernel<3><<<nb, NT, 0, st>>>(s.n, b, s.dinv, s.x, s.r, s.z, s.p, pff(s), s.work); break;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  pcg_start_finish<<<1, NT, 0, st>>>(s.work, nb);
  return cudaGetLastError();
}

cudaError_t pcg_iterate(const EfePcg& s, int64_t k0, int nIter, cudaStream_t st) {
  const int sms = sm_count();
  const int nbS = spmv_blocks(s.n, sms), nbV = vec_blocks(s.n, sms);
  float2* pf = pff(s);
  for (int k = 0; k < nIter; ++k) {
    const int cur = (int)((k0 + k) & 1);
    cudaError_t e = pf ? spmv_pairs(s, s.p, pf, s.Ap, s.work + PART0, nbS, st)
                       : spmv(s, s.p, s.Ap, s.work + PART0, nbS, st);
    if (e != cudaSuccess) return e;
    switch (s.blockSize) {
      case 1: pcg_update_kernel<1><<<nbV, NT, 0, st>>>(s.n, cur, nbS, s.p, s.Ap, s.dinv, s.x, s.r, s.z, s.work); break;
      case 2: pcg_update_kernel<2><<<nbV, NT, 0, st>>>(s.n, cur, nbS, s.p, s.Ap, s.dinv, s.x, s.r, s.z, s.work); break;
      default: pcg_update_kernel<3><<<nbV, NT, 0, st>>>(s.n, cur, nbS, s.p, s.Ap, s.dinv, s.x, s.r, s.z, s.work); break;
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    pcg_direction_kernel<<<nbV, NT, 0, st>>>(s.n, cur, nbV, s.z, s.p, pf, s.work);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace efe
