// efe_device.cuh -- device-side building blocks: element shapes, quadrature rules and the
// material point updates of the reference's "edelweiss" materials, all in FP64.
//
// Reference algorithms (paths relative to the EdelweissFE project root):
//   shape functions      elements/displacementelement/_elementcomputationmatrices.py:106-212
//   Jacobian / dN/dX     _elementcomputationmatrices.py:32-103, 215-540, displacementtlelement/
//                        _elementcomputationmatrices.py:247-281 (derivatives evaluated at the
//                        natural point (eta_i, xi_i, zeta_i) of quadrature point i)
//   quadrature rules     elements/library.py:33-533
//   linear elastic       materials/linearelastic/linearelastic.py:63-210
//   von Mises            materials/vonmises/vonmises.py:35-254
//   plane stress (hypo)  materials/base/basehypoelasticmaterial.py:71-130
//   Neo-Hooke a/b/c      materials/neohooke/neohookepencegouformulation{a,b,c}.py:107-145
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/efe_gb300.h"

namespace efe {

// ------------------------------------------------------------------ shapes and rules
template <int SHAPE> struct ShapeInfo;
template <> struct ShapeInfo<EFE_QUAD4> { static constexpr int DIM = 2, NN = 4; };
template <> struct ShapeInfo<EFE_QUAD8> { static constexpr int DIM = 2, NN = 8; };
template <> struct ShapeInfo<EFE_HEXA8> { static constexpr int DIM = 3, NN = 8; };
template <> struct ShapeInfo<EFE_HEXA20> { static constexpr int DIM = 3, NN = 20; };

template <int RULE> struct RuleInfo;
template <> struct RuleInfo<EFE_RULE_2D_1> { static constexpr int NQ = 1; };
template <> struct RuleInfo<EFE_RULE_2D_2X2> { static constexpr int NQ = 4; };
template <> struct RuleInfo<EFE_RULE_2D_3X3> { static constexpr int NQ = 9; };
template <> struct RuleInfo<EFE_RULE_3D_1> { static constexpr int NQ = 1; };
template <> struct RuleInfo<EFE_RULE_3D_2X2X2> { static constexpr int NQ = 8; };
template <> struct RuleInfo<EFE_RULE_3D_3X3X3> { static constexpr int NQ = 27; };

// natural coordinates of the nodes in the reference's node order (computeNOperator)
__device__ __forceinline__ void node_natural(int shape, int a, int c[3]) {
  // quad4 / corners of quad8: (-1,-1) (1,-1) (1,1) (-1,1); quad8 mids: (0,-1) (1,0) (0,1) (-1,0)
  const signed char q8[8][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}, {0, -1}, {1, 0}, {0, 1}, {-1, 0}};
  const signed char h20[20][3] = {{-1, -1, -1}, {-1, -1, 1}, {1, -1, 1}, {1, -1, -1}, {-1, 1, -1}, {-1, 1, 1},
                                  {1, 1, 1},    {1, 1, -1},  {-1, -1, 0}, {0, -1, 1}, {1, -1, 0}, {0, -1, -1},
                                  {-1, 1, 0},   {0, 1, 1},   {1, 1, 0},   {0, 1, -1}, {-1, 0, -1}, {-1, 0, 1},
                                  {1, 0, 1},    {1, 0, -1}};
  if (shape == EFE_QUAD4 || shape == EFE_QUAD8) {
    c[0] = q8[a][0];
    c[1] = q8[a][1];
    c[2] = 0;
  } else {
    c[0] = h20[a][0];
    c[1] = h20[a][1];
    c[2] = h20[a][2];
  }
}

// dN_a/dxi_r at natural point p (serendipity / Lagrange shape functions)
template <int SHAPE>
__device__ void shape_derivatives(const double p[3], double dN[ShapeInfo<SHAPE>::DIM][ShapeInfo<SHAPE>::NN]) {
  constexpr int DIM = ShapeInfo<SHAPE>::DIM, NN = ShapeInfo<SHAPE>::NN;
  constexpr bool quadratic = NN > (1 << DIM);
  for (int a = 0; a < NN; ++a) {
    int c[3];
    node_natural(SHAPE, a, c);
    bool corner = true;
    int mid = -1;
    for (int k = 0; k < DIM; ++k)
      if (c[k] == 0) {
        corner = false;
        mid = k;
      }
    if (!quadratic || corner) {
      double lin[3];
      for (int k = 0; k < DIM; ++k) lin[k] = 1.0 + c[k] * p[k];
      double base = 1.0;
      for (int k = 0; k < DIM; ++k) base *= lin[k];
      const double inv = 1.0 / (1 << DIM);
      double s = 0.0;
      if (quadratic) {
        for (int k = 0; k < DIM; ++k) s += c[k] * p[k];
        s -= (DIM - 1);
      }
      for (int r = 0; r < DIM; ++r) {
        double db = c[r];
        for (int k = 0; k < DIM; ++k)
          if (k != r) db *= lin[k];
        if (quadratic)
          dN[r][a] = (db * s + base * c[r]) * inv;
        else
          dN[r][a] = db * inv;
      }
    } else {
      const double inv = 1.0 / (1 << (DIM - 1));
      double prod = 1.0;
      for (int k = 0; k < DIM; ++k)
        if (k != mid) prod *= (1.0 + c[k] * p[k]);
      const double q = 1.0 - p[mid] * p[mid];
      for (int r = 0; r < DIM; ++r) {
        if (r == mid) {
          dN[r][a] = -2.0 * p[mid] * prod * inv;
        } else {
          double t = q * c[r];
          for (int k = 0; k < DIM; ++k)
            if (k != mid && k != r) t *= (1.0 + c[k] * p[k]);
          dN[r][a] = t * inv;
        }
      }
    }
  }
}

// N_a at natural point p (computeNOperator, _elementcomputationmatrices.py:106-212)
template <int SHAPE>
__device__ void shape_values(const double p[3], double N[ShapeInfo<SHAPE>::NN]) {
  constexpr int DIM = ShapeInfo<SHAPE>::DIM, NN = ShapeInfo<SHAPE>::NN;
  constexpr bool quadratic = NN > (1 << DIM);
  for (int a = 0; a < NN; ++a) {
    int c[3];
    node_natural(SHAPE, a, c);
    int mid = -1;
    for (int k = 0; k < DIM; ++k)
      if (c[k] == 0) mid = k;
    if (!quadratic || mid < 0) {
      double base = 1.0, s = -(DIM - 1);
      for (int k = 0; k < DIM; ++k) {
        base *= 1.0 + c[k] * p[k];
        s += c[k] * p[k];
      }
      N[a] = base / (1 << DIM) * (quadratic ? s : 1.0);
    } else {
      double prod = 1.0 - p[mid] * p[mid];
      for (int k = 0; k < DIM; ++k)
        if (k != mid) prod *= 1.0 + c[k] * p[k];
      N[a] = prod / (1 << (DIM - 1));
    }
  }
}

// quadrature point q of a rule: library coordinates (xi, eta, zeta) and weight
__device__ __forceinline__ void quadrature_point(int rule, int q, double& xi, double& eta, double& zeta, double& w) {
  const double g = 1.0 / sqrt(3.0);
  const double s = sqrt(0.6);
  zeta = 0.0;
  switch (rule) {
    case EFE_RULE_2D_1:
      xi = 0.0;
      eta = 0.0;
      w = 4.0;
      return;
    case EFE_RULE_2D_2X2: {
      const signed char X[4] = {1, 1, -1, -1}, Y[4] = {1, -1, -1, 1};
      xi = g * X[q];
      eta = g * Y[q];
      w = 1.0;
      return;
    }
    case EFE_RULE_2D_3X3: {
      const signed char X[9] = {0, -1, -1, 1, 1, -1, 0, 1, 0}, Y[9] = {0, -1, 1, 1, -1, 0, 1, 0, -1};
      const double w1 = (5.0 / 9.0) * (5.0 / 9.0), w2 = (5.0 / 9.0) * (8.0 / 9.0), w3 = (8.0 / 9.0) * (8.0 / 9.0);
      xi = s * X[q];
      eta = s * Y[q];
      w = (q == 0) ? w3 : (q < 5 ? w1 : w2);
      return;
    }
    case EFE_RULE_3D_1:
      xi = eta = zeta = 0.0;
      w = 8.0;
      return;
    case EFE_RULE_3D_2X2X2: {
      const signed char Y[4] = {-1, -1, 1, 1}, Z[4] = {-1, 1, 1, -1};
      xi = g * (q < 4 ? -1.0 : 1.0);
      eta = g * Y[q & 3];
      zeta = g * Z[q & 3];
      w = 1.0;
      return;
    }
    default: {  // EFE_RULE_3D_3X3X3
      const double W[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
      const int i = q / 9, j = (q / 3) % 3, k = q % 3;
      xi = s * (i - 1);
      eta = s * (j - 1);
      zeta = s * (k - 1);
      w = W[i] * W[j] * W[k];
      return;
    }
  }
}

// ------------------------------------------------------------------ small dense helpers
__device__ __forceinline__ double det3(const double A[3][3]) {
  return A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) - A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
         A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
}
__device__ __forceinline__ void inv3(const double A[3][3], double d, double B[3][3]) {
  const double id = 1.0 / d;
  B[0][0] = (A[1][1] * A[2][2] - A[1][2] * A[2][1]) * id;
  B[0][1] = (A[0][2] * A[2][1] - A[0][1] * A[2][2]) * id;
  B[0][2] = (A[0][1] * A[1][2] - A[0][2] * A[1][1]) * id;
  B[1][0] = (A[1][2] * A[2][0] - A[1][0] * A[2][2]) * id;
  B[1][1] = (A[0][0] * A[2][2] - A[0][2] * A[2][0]) * id;
  B[1][2] = (A[0][2] * A[1][0] - A[0][0] * A[1][2]) * id;
  B[2][0] = (A[1][0] * A[2][1] - A[1][1] * A[2][0]) * id;
  B[2][1] = (A[0][1] * A[2][0] - A[0][0] * A[2][1]) * id;
  B[2][2] = (A[0][0] * A[1][1] - A[0][1] * A[1][0]) * id;
}

// ------------------------------------------------------------------ float-float arithmetic
// A value x is carried as hi + lo with hi = fl32(x), lo = fl32(x - hi) (~48 significant bits).
// Error-free product (FMA) and sum (Knuth's two-sum) use the _rn intrinsics so that the compiler
// cannot contract or reorder them.
struct ff {
  float h, l;
};
__device__ __forceinline__ ff ff_split(double x) {
  const float h = __double2float_rn(x);
  return ff{h, __double2float_rn(x - (double)h)};
}
__device__ __forceinline__ double ff_to_double(ff a) { return (double)a.h + (double)a.l; }
// acc += a * b
__device__ __forceinline__ void ff_fma(ff& acc, ff a, ff b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  const float s = __fadd_rn(acc.h, p);
  const float bb = __fsub_rn(s, acc.h);
  const float err = __fadd_rn(__fsub_rn(acc.h, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  acc.l = __fadd_rn(acc.l, __fadd_rn(err, e));
  acc.h = s;
}
// ------------------------------------------------------------------ conversions off the FP64 pipe
// On this GPU the conversions between double and float (F2F) issue on the FP64 pipe, which binds
// the element pass; a float-float pass spends about a third of that pipe on them.  The forms below
// give the same values (or an equally accurate split) with integer and FP32 instructions, from the
// IEEE-754 bit layouts: float = sign | exponent (8, bias 127) | fraction (23); double = sign |
// exponent (11, bias 1023) | fraction (52).  Arguments outside the ranges they handle (zero is
// handled; subnormals, infinities, NaN and magnitudes beyond the float range) take the hardware
// conversions.

// float -> double, exact
__device__ __forceinline__ double f2d_bits(float f) {
  const uint32_t b = __float_as_uint(f);
  const uint32_t e = (b >> 23) & 0xffu;
  if (e - 1u < 254u) {  // normal: exponent + (1023 - 127), fraction shifted to the top of 52 bits
    const uint64_t mag = ((uint64_t)(b & 0x7fffffffu) << 29) + (896ull << 52);
    return __longlong_as_double((long long)(((uint64_t)(b & 0x80000000u) << 32) | mag));
  }
  if ((b & 0x7fffffffu) == 0u) return __longlong_as_double((long long)((uint64_t)b << 32));  // +-0
  return (double)f;
}

// double -> float, rounded toward zero (the 23 leading fraction bits)
__device__ __forceinline__ float d2f_trunc(double x) {
  const uint64_t X = (uint64_t)__double_as_longlong(x);
  const uint32_t hi = (uint32_t)(X >> 32), lo = (uint32_t)X;
  const uint32_t E = (hi >> 20) & 0x7ffu;
  if (E - 897u < 254u)  // the float exponent E - 896 is in [1, 254]; the exponent bits wrap mod 2^32
    return __uint_as_float((hi & 0x80000000u) | ((((hi & 0x7fffffffu) << 3) | (lo >> 29)) - (896u << 23)));
  if (((hi & 0x7fffffffu) | lo) == 0u) return __uint_as_float(hi & 0x80000000u);
  return __double2float_rn(x);
}

// double -> (hi, lo): hi = x rounded toward zero to 24 bits, lo = fl32(x - hi) (x - hi is the low 29
// fraction bits times 2^(E - 1075); fl32 of that integer from its exact 13- and 16-bit halves and
// one rounding FMA).  hi + lo agrees with x to ~2^-47 relative, like ff_split's.
__device__ __forceinline__ ff ff_split_bits(double x) {
  const uint64_t X = (uint64_t)__double_as_longlong(x);
  const uint32_t hi = (uint32_t)(X >> 32), lo = (uint32_t)X;
  const uint32_t E = (hi >> 20) & 0x7ffu;
  if (E - 949u < 202u) {  // E in [949, 1150]: hi normal, and 2^(E - 1075) a normal float
    const uint32_t sign = hi & 0x80000000u;
    const float h = __uint_as_float(sign | ((((hi & 0x7fffffffu) << 3) | (lo >> 29)) - (896u << 23)));
    const uint32_t R = lo & 0x1fffffffu;
    const float r1 = __fsub_rn(__uint_as_float(0x4B000000u | (R >> 16)), 8388608.0f);      // exact
    const float r0 = __fsub_rn(__uint_as_float(0x4B000000u | (R & 0xffffu)), 8388608.0f);  // exact
    const float l = __fmul_rn(__fmaf_rn(r1, 65536.0f, r0), __uint_as_float((E - 948u) << 23));
    return ff{h, sign ? -l : l};
  }
  if (((hi & 0x7fffffffu) | lo) == 0u) return ff{__uint_as_float(hi & 0x80000000u), 0.0f};
  return ff_split(x);
}

// hi + lo as a double: exact conversions, one rounding add
__device__ __forceinline__ double ff_to_double_bits(ff a) { return f2d_bits(a.h) + f2d_bits(a.l); }

// not infinite and not NaN, from the exponent bits
__device__ __forceinline__ bool finite_bits(double x) {
  return ((uint32_t)((uint64_t)__double_as_longlong(x) >> 32) & 0x7ff00000u) != 0x7ff00000u;
}

// the tangent's precision: doubles pass through, floats are truncated off the FP64 pipe
template <typename KT>
__device__ __forceinline__ KT to_kt(double x) {
  if constexpr (sizeof(KT) == 4)
    return d2f_trunc(x);
  else
    return x;
}

// a * b (both float-float), renormalised
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  const float s = __fadd_rn(p, e);
  return ff{s, __fsub_rn(e, __fsub_rn(s, p))};
}

// acc += a
__device__ __forceinline__ void ff_add(ff& acc, ff a) {
  const float s = __fadd_rn(acc.h, a.h);
  const float bb = __fsub_rn(s, acc.h);
  const float err = __fadd_rn(__fsub_rn(acc.h, __fsub_rn(s, bb)), __fsub_rn(a.h, bb));
  acc.l = __fadd_rn(acc.l, __fadd_rn(err, a.l));
  acc.h = s;
}

// ------------------------------------------------------------------ materials
// Isotropic elasticity matrix entries, formed like the reference: f = E/((1+v)(1-2v)),
// C11 = f(1-v), C12 = f v, C44 = f (1-2v)/2   (linearelastic.py:95-117, vonmises.py:126-149)
struct Iso {
  double c11, c12, c44;
};
__device__ __forceinline__ Iso iso3d(double E, double v) {
  const double f = E / ((1.0 + v) * (1.0 - 2.0 * v));
  return Iso{f * (1.0 - v), f * v, f * ((1.0 - 2.0 * v) / 2.0)};
}
__device__ __forceinline__ void iso_apply(const Iso& C, const double e[6], double s[6]) {
  s[0] = C.c11 * e[0] + C.c12 * e[1] + C.c12 * e[2];
  s[1] = C.c12 * e[0] + C.c11 * e[1] + C.c12 * e[2];
  s[2] = C.c12 * e[0] + C.c12 * e[1] + C.c11 * e[2];
  s[3] = C.c44 * e[3];
  s[4] = C.c44 * e[4];
  s[5] = C.c44 * e[5];
}

// Tangent of a hypoelastic 3D update in the form C = C_iso(c11, c12, c44) - a n (x) n,
// which covers linear elasticity (a = 0) and the consistent J2 tangent (vonmises.py:241-251).
struct Tangent3 {
  double c11, c12, c44, a;
  double n[6];
};
__device__ __forceinline__ double tangent3_entry(const Tangent3& T, int i, int j) {
  double v;
  if (i < 3 && j < 3)
    v = (i == j) ? T.c11 : T.c12;
  else
    v = (i == j) ? T.c44 : 0.0;
  return v - T.a * T.n[i] * T.n[j];
}

// Per-element constants of the von Mises / linear-elastic 3D update, formed once per element.
struct VMConst {
  Iso Ei;
  double G, fy0, H, dfy, delta;
  double tfac;  // 1 / (1 + H / (3G)): the tangent factor of vonmises.py:247 when dfy == 0
  double invdR; // 1 / (dR/d dK) of the return-map residual, constant per element when dfy == 0
};
__device__ __forceinline__ VMConst vm_const(const double* props, bool vonMises) {
  VMConst c;
  c.Ei = iso3d(props[0], props[1]);
  c.G = props[0] / (2.0 * (1.0 + props[1]));
  c.fy0 = vonMises ? props[2] : 0.0;
  c.H = vonMises ? props[3] : 0.0;
  c.dfy = vonMises ? props[4] : 0.0;
  c.delta = vonMises ? props[5] : 0.0;
  c.tfac = 1.0 / (1.0 + c.H / (3.0 * c.G));
  c.invdR = 1.0 / (-sqrt(6.0) * c.G - sqrt(2.0 / 3.0) * c.H);
  return c;
}

// dfy * (1 - exp(-delta k)); identical to the reference's expression, and exactly 0 when dfy == 0
__device__ __forceinline__ double vm_sat(const VMConst& c, double k) {
  return c.dfy == 0.0 ? 0.0 : c.dfy * (1.0 - exp(-c.delta * k));
}
__device__ __forceinline__ double vm_dsat(const VMConst& c, double k) {
  return c.dfy == 0.0 ? 0.0 : c.dfy * c.delta * exp(-c.delta * k);
}

// |dev| with the shear terms doubled (vonmises.py:63-64) and its reciprocal from one reciprocal
// square root (0 and inf for a zero deviator)
__device__ __forceinline__ void vm_dev_norm(const double dev[6], double& norm, double& inv) {
  const double q2 =
      dev[0] * dev[0] + dev[1] * dev[1] + dev[2] * dev[2] + 2.0 * (dev[3] * dev[3] + dev[4] * dev[4] + dev[5] * dev[5]);
  inv = rsqrt(q2);
  norm = q2 > 0.0 ? q2 * inv : 0.0;
}
// Newton step of the return map: R / dR (the derivative is constant per element for linear hardening)
__device__ __forceinline__ double vm_newton_step(const VMConst& c, double R, double k) {
  if (c.dfy == 0.0) return R * c.invdR;
  const double dR = -sqrt(6.0) * c.G - sqrt(2.0 / 3.0) * (c.H + vm_dsat(c, k));
  return R / dR;
}

// von Mises radial return (vonmises.py:186-254).  Updates sig and kappa in place.
// Returns false when the scalar Newton does not converge in 15 iterations (CutbackRequest).
// FAST (used with an FP32 tangent): |dev| and 1/|dev| from one rsqrt and the Newton step as a product
// with the per-element 1/dR; otherwise the reference's sqrt and divisions, whose rounding the FP64
// mode keeps so that rounding-critical return maps fail (cut back) exactly where the reference's do.
template <bool FAST = false>
__device__ inline bool von_mises_3d(const VMConst& c, double sig[6], const double de[6], double& kappa, Tangent3& T) {
  const Iso& Ei = c.Ei;
  T.c11 = Ei.c11;
  T.c12 = Ei.c12;
  T.c44 = Ei.c44;
  T.a = 0.0;
  for (int i = 0; i < 6; ++i) T.n[i] = 0.0;
  double nrm = 0.0;
  for (int i = 0; i < 6; ++i) nrm += de[i] * de[i];
  if (nrm < 1e-28) return true;  // zero increment, |dStrain| < 1e-14: C = Ei (:211-213)
  const double G = c.G;
  double tr[6], ds[6];
  iso_apply(Ei, de, ds);
  for (int i = 0; i < 6; ++i) tr[i] = sig[i] + ds[i];
  double dev[6];
  const double mean = (tr[0] + tr[1] + tr[2]) * (1.0 / 3.0);
  dev[0] = tr[0] - mean;
  dev[1] = tr[1] - mean;
  dev[2] = tr[2] - mean;
  dev[3] = tr[3];
  dev[4] = tr[4];
  dev[5] = tr[5];
  double devNorm, inv;
  if constexpr (FAST) {
    vm_dev_norm(dev, devNorm, inv);
  } else {
    devNorm = sqrt(dev[0] * dev[0] + dev[1] * dev[1] + dev[2] * dev[2] +
                   2.0 * (dev[3] * dev[3] + dev[4] * dev[4] + dev[5] * dev[5]));
    inv = 1.0 / devNorm;
  }
  const double k0 = kappa;
  const double sq23 = sqrt(2.0 / 3.0), sq6 = sqrt(6.0);
  const double fy_k0 = c.fy0 + c.H * k0 + vm_sat(c, k0);
  if (devNorm - sq23 * fy_k0 > 0.0) {
    double dK = 0.0;
    int counter = 0;
    bool ok = true;
    while (true) {
      const double k = k0 + dK;
      const double R = devNorm - sq6 * G * dK - sq23 * (c.fy0 + c.H * k + vm_sat(c, k));
      if (!(fabs(R) > 1e-12)) break;
      if (counter == 15) {
        ok = false;
        break;
      }
      if constexpr (FAST) {
        dK -= vm_newton_step(c, R, k);
      } else {
        const double dR = -sq6 * G - sq23 * (c.H + vm_dsat(c, k));
        dK -= R / dR;
      }
      ++counter;
    }
    const double dLambda = sqrt(1.5) * dK;
    kappa = k0 + dK;
    const double g2 = 2.0 * G * dLambda;
    for (int i = 0; i < 6; ++i) {
      T.n[i] = dev[i] * inv;
      sig[i] = tr[i] - g2 * T.n[i];
    }
    const double tfac = c.dfy == 0.0 ? c.tfac : 1.0 / (1.0 + (c.H + vm_dsat(c, kappa)) / (3.0 * G));
    const double beta = 2.0 * G * g2 * inv;  // 4 G^2 dLambda / devNorm, coefficient of IDevHalfShear
    T.a = 2.0 * G * (tfac - g2 * inv);
    T.c11 = Ei.c11 - beta * (2.0 / 3.0);
    T.c12 = Ei.c12 + beta * (1.0 / 3.0);
    T.c44 = Ei.c44 - beta * 0.5;
    return ok;
  }
  for (int i = 0; i < 6; ++i) sig[i] = tr[i];
  return true;
}

__device__ __forceinline__ void linear_elastic_3d(const VMConst& c, double sig[6], const double de[6], Tangent3& T) {
  double ds[6];
  iso_apply(c.Ei, de, ds);
  for (int i = 0; i < 6; ++i) sig[i] += ds[i];
  T.c11 = c.Ei.c11;
  T.c12 = c.Ei.c12;
  T.c44 = c.Ei.c44;
  T.a = 0.0;
  for (int i = 0; i < 6; ++i) T.n[i] = 0.0;
}

// symmetric 3x3 in-plane tangent (rows/cols 11, 22, 12): C00 C01 C02 C11 C12 C22
struct Tangent2 {
  double c[6];
};
__device__ __forceinline__ void tangent2_from3(const Tangent3& T, Tangent2& C) {
  // plane strain: rows/cols [0,1,3] of the 6x6 tangent (element.py:217-219,336)
  const int id[3] = {0, 1, 3};
  int k = 0;
  for (int i = 0; i < 3; ++i)
    for (int j = i; j < 3; ++j) C.c[k++] = tangent3_entry(T, id[i], id[j]);
}

// LinearElasticMaterial.computePlaneStress (linearelastic.py:127-154); de[2] is overwritten
__device__ __forceinline__ void linear_elastic_plane_stress(const double* props, double sig[6], double de[6],
                                                            Tangent2& C) {
  const double E = props[0], v = props[1];
  const double f = E / (1.0 - v * v);
  const double c11 = f * 1.0, c12 = f * v, c33 = f * ((1.0 - v) / 2.0);
  sig[0] += c11 * de[0] + c12 * de[1];
  sig[1] += c12 * de[0] + c11 * de[1];
  sig[3] += c33 * de[3];
  de[2] = -v / (1.0 - v) * (de[0] + de[1]);
  C.c[0] = c11;
  C.c[1] = c12;
  C.c[2] = 0.0;
  C.c[3] = c11;
  C.c[4] = 0.0;
  C.c[5] = c33;
}

// BaseHypoElasticMaterial.computePlaneStress applied to von Mises (basehypoelasticmaterial.py:71-130):
// local Newton on de[2]; every local step calls the 3D update with a zero stress vector and the
// material state, so kappa accumulates the plastic increments of all local steps; the converged
// 3D stress is added to sig.  Returns false on a cutback request.
template <bool FAST = false>
__device__ inline bool von_mises_plane_stress(const VMConst& vc, double sig[6], double de[6], double& kappa, Tangent2& C) {
  Tangent3 T;
  double s3[6];
  de[2] = -de[0] - de[1];
  int counter = 1;
  bool ok = true;
  while (true) {
    for (int i = 0; i < 6; ++i) s3[i] = 0.0;
    if (!von_mises_3d<FAST>(vc, s3, de, kappa, T)) {
      ok = false;
      break;
    }
    const double residual = fabs(s3[2]);
    if (residual < 1e-11 || (counter > 7 && residual < 1e-8)) break;
    const double C22 = tangent3_entry(T, 2, 2);
    double rev = 1.0 / C22;
    if (isnan(rev) || fabs(rev) > 1e10) rev = 1e10 * (rev > 0 ? 1.0 : (rev < 0 ? -1.0 : rev));
    de[2] -= rev * s3[2];
    ++counter;
    if (counter > 13) {
      ok = false;
      break;
    }
  }
  for (int i = 0; i < 6; ++i) sig[i] += s3[i];
  const int id[3] = {0, 1, 3};
  const double C22 = tangent3_entry(T, 2, 2);
  int k = 0;
  for (int i = 0; i < 3; ++i)
    for (int j = i; j < 3; ++j)
      C.c[k++] = tangent3_entry(T, id[i], id[j]) - tangent3_entry(T, 2, id[j]) * tangent3_entry(T, id[i], 2) / C22;
  return ok;
}

// Neo-Hooke (Pence-Gou a/b/c): Kirchhoff stress tau (3x3), energy, and the coefficients of
//   dtau_ij/dF_kl = c1 (d_ik F_jl + F_il d_jk) + c2 d_ij Finv_lk + c3 B_ij Finv_lk + c4 d_ij F_kl
// (neohookepencegouformulationa.py:128-141, b.py:128-145, c.py:128-143).
struct NeoHookeOut {
  double tau[3][3];
  double Bm[3][3];
  double c1, c2, c3, c4, energy;
};
// The scalar part of the three variants: tau = sB B + sI I, the tangent coefficients c1-c4 and the
// energy, from J = det F, I1 = tr B and tr F (the energy of c uses tr F as I1, c.py:141).  The
// first Piola-Kirchhoff stress follows without a 3x3 product: tau F^-T = sB F + sI F^-T, since
// B F^-T = F.  Variant b forms J^(-2/3) as rcbrt(J)^2 and 1/J^2 once (one reciprocal instead of
// pow and four divisions).
struct NeoHookeScalars {
  double sB, sI, c1, c2, c3, c4, energy;
};
__device__ inline NeoHookeScalars neo_hooke_scalars(int material, double mu, double K, double J, double I1,
                                                    double trF) {
  NeoHookeScalars o;
  if (material == EFE_MAT_NEOHOOKE_WA) {
    const double lambdaBar = (K - 2.0 / 3.0 * mu) * (J * J - J) - mu;
    const double muBar = (K - 2.0 / 3.0 * mu) * (2.0 * J * J - J);
    o.sB = mu;
    o.sI = lambdaBar;
    o.c1 = mu;
    o.c2 = muBar;
    o.c3 = 0.0;
    o.c4 = 0.0;
    o.energy = mu / 2.0 * (I1 - 3.0) + (K / 2.0 - mu / 3.0) * (J - 1.0) * (J - 1.0) - mu * log(J);
  } else if (material == EFE_MAT_NEOHOOKE_WB) {
    const double r = rcbrt(J);
    // J^(-2/3); NaN for an inverted point, like pow(J, 2/3) of a negative J
    const double rJ23 = J < 0.0 ? __longlong_as_double(0x7ff8000000000000ll) : r * r;
    const double J2 = J * J, rJ2 = 1.0 / J2;  // J^2, J^-2
    const double lambdaHat = K / 2.0 * (J2 + rJ2);
    const double muBar = mu * rJ23 / 3.0;
    const double lambdaBar = K / 4.0 * (J2 - rJ2) - muBar * I1;
    o.sB = mu * rJ23;
    o.sI = lambdaBar;
    o.c1 = 3.0 * muBar;
    o.c2 = lambdaHat + 2.0 / 3.0 * I1 * muBar;
    o.c3 = -2.0 * muBar;
    o.c4 = -2.0 * muBar;
    o.energy = mu / 2.0 * (I1 * rJ23 - 3.0) + K / 8.0 * (J2 + rJ2 - 2.0);
  } else {  // EFE_MAT_NEOHOOKE_WC
    const double p = pow(J, 2.0 / 3.0 - K / mu);
    const double muBar = mu * p;
    const double lambdaBar = (K / mu - 2.0 / 3.0) * muBar;
    o.sB = mu;
    o.sI = -muBar;
    o.c1 = mu;
    o.c2 = lambdaBar;
    o.c3 = 0.0;
    o.c4 = 0.0;
    o.energy = mu / 2.0 * (trF - 3.0) + 3.0 * mu * mu / (3.0 * K - 2.0 * mu) * (p - 1.0);
  }
  return o;
}
__device__ inline void neo_hooke(int material, double mu, double K, const double F[3][3], NeoHookeOut& o) {
  double B[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = i; j < 3; ++j) B[i][j] = B[j][i] = F[i][0] * F[j][0] + F[i][1] * F[j][1] + F[i][2] * F[j][2];
  const NeoHookeScalars n =
      neo_hooke_scalars(material, mu, K, det3(F), B[0][0] + B[1][1] + B[2][2], F[0][0] + F[1][1] + F[2][2]);
  o.c1 = n.c1;
  o.c2 = n.c2;
  o.c3 = n.c3;
  o.c4 = n.c4;
  o.energy = n.energy;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      o.tau[i][j] = n.sB * B[i][j] + (i == j ? n.sI : 0.0);
      o.Bm[i][j] = B[i][j];
    }
}

}  // namespace efe
