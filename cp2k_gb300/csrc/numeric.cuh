// Arithmetic types of the grid kernels.
//
//   double   plain FP64                        (GRID_GB300_FP64)
//   float    plain FP32                        (GRID_GB300_FP32)
//   dfloat   unevaluated sum of two floats      (GRID_GB300_MIXED)
//
// dfloat ("double-float") carries ~48 significant bits on the FP32 pipes:
// products are split exactly with an FMA (TwoProduct) and sums with Knuth's
// TwoSum (D. E. Knuth, TAOCP vol. 2, 4.2.2; T. J. Dekker, Numer. Math. 18
// (1971) 224-242).  On GB300 the FP64 pipe runs at about 1/56 of the FP32
// rate, so a dfloat FMA (about 12 FP32 operations) is several times cheaper
// than an FP64 FMA while keeping the per-point evaluation accurate to
// ~1e-14 relative.
#pragma once

#include <cuda_runtime.h>

namespace gb300 {

struct dfloat {
  float h, l;
  dfloat() = default;
  __host__ __device__ constexpr dfloat(float hi, float lo) : h(hi), l(lo) {}
  __host__ __device__ constexpr dfloat(float x) : h(x), l(0.f) {}
  __host__ __device__ constexpr dfloat(int x) : h((float)x), l(0.f) {}
  __device__ explicit dfloat(double x);
};

__device__ __forceinline__ dfloat df_make(double x) {
  const float h = (float)x;
  return dfloat{h, (float)(x - (double)h)};
}
__device__ __forceinline__ dfloat::dfloat(double x) : h((float)x), l((float)(x - (double)(float)x)) {}

// acc + a*b
__device__ __forceinline__ dfloat df_fma(dfloat acc, dfloat a, dfloat b) {
  const float p = a.h * b.h;
  float e = fmaf(a.h, b.h, -p);     // exact error of the leading product
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  const float s = acc.h + p;        // TwoSum(acc.h, p)
  const float bb = s - acc.h;
  const float err = (acc.h - (s - bb)) + (p - bb);
  const float t = err + (acc.l + e);
  const float h = s + t;            // renormalise
  return dfloat{h, t - (h - s)};
}

// acc + a*b without the final renormalisation: the pair (h, l) still sums to
// the compensated result, only |l| may grow to a few ulps of h.  Long
// accumulations (dot products, row sums) use this form and renormalise once
// at the end (the compensated dot product "Dot2" of Ogita, Rump and Oishi,
// SIAM J. Sci. Comput. 26 (2005) 1955-1988), saving 3 of 15 operations per
// term.  Multiplicands should be normalised (df_norm) pairs.
__device__ __forceinline__ dfloat df_fma_acc(dfloat acc, dfloat a, dfloat b) {
  const float p = a.h * b.h;
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  const float s = acc.h + p;
  const float bb = s - acc.h;
  const float err = (acc.h - (s - bb)) + (p - bb);
  return dfloat{s, err + (acc.l + e)};
}

__device__ __forceinline__ dfloat df_norm(dfloat a) {
  const float h = a.h + a.l;
  return dfloat{h, a.l - (h - a.h)};
}

// acc + a*b with b a plain float (exactly representable factor)
__device__ __forceinline__ dfloat df_fma1(dfloat acc, dfloat a, float b) {
  const float p = a.h * b;
  float e = fmaf(a.h, b, -p);
  e = fmaf(a.l, b, e);
  const float s = acc.h + p;
  const float bb = s - acc.h;
  const float err = (acc.h - (s - bb)) + (p - bb);
  const float t = err + (acc.l + e);
  const float h = s + t;
  return dfloat{h, t - (h - s)};
}

__device__ __forceinline__ dfloat df_mul(dfloat a, dfloat b) {
  return df_fma(dfloat{0.f, 0.f}, a, b);
}

// a*b with b a plain float that is exactly representable (a small integer):
// the exact leading product and its error term, not renormalised (|l| stays
// within a few ulps of h), for power chains
__device__ __forceinline__ dfloat df_mul1(dfloat a, float b) {
  const float p = a.h * b;
  float e = fmaf(a.h, b, -p);
  e = fmaf(a.l, b, e);
  return dfloat{p, e};
}

__device__ __forceinline__ dfloat df_add(dfloat a, dfloat b) {
  const float s = a.h + b.h;
  const float bb = s - a.h;
  const float err = (a.h - (s - bb)) + (b.h - bb);
  const float t = err + (a.l + b.l);
  const float h = s + t;
  return dfloat{h, t - (h - s)};
}

__device__ __forceinline__ dfloat operator+(dfloat a, dfloat b) { return df_add(a, b); }
__device__ __forceinline__ dfloat operator-(dfloat a) { return dfloat{-a.h, -a.l}; }
__device__ __forceinline__ dfloat operator-(dfloat a, dfloat b) { return df_add(a, -b); }
__device__ __forceinline__ dfloat operator*(dfloat a, dfloat b) { return df_mul(a, b); }
__device__ __forceinline__ dfloat &operator+=(dfloat &a, dfloat b) { return a = df_add(a, b); }
__device__ __forceinline__ dfloat &operator-=(dfloat &a, dfloat b) { return a = df_add(a, -b); }
__device__ __forceinline__ dfloat &operator*=(dfloat &a, dfloat b) { return a = df_mul(a, b); }
__device__ __forceinline__ bool operator!=(dfloat a, dfloat b) { return a.h != b.h || a.l != b.l; }
__device__ __forceinline__ double to_double(dfloat a) { return (double)a.h + (double)a.l; }
__device__ __forceinline__ double to_double(double a) { return a; }
__device__ __forceinline__ double to_double(float a) { return (double)a; }

// a + b for plain floats, exact (Knuth's TwoSum)
__device__ __forceinline__ dfloat df_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return dfloat{s, (a - (s - bb)) + (b - bb)};
}

// a + b with b a plain float
__device__ __forceinline__ dfloat df_add1(dfloat a, float b) {
  const dfloat s = df_two_sum(a.h, b);
  const float t = s.l + a.l;
  const float h = s.h + t;
  return dfloat{h, t - (h - s.h)};
}

// exp(-x) for a dfloat x >= 0, to ~1e-14 relative for x <= 40, following
// Tang's table-driven method (P. T. P. Tang, ACM TOMS 15 (1989) 144-157):
//   x = k ln2/64 + t, |t| <= ln2/128,  exp(-x) = 2^(-k/64) exp(-t),
// with k = 64 m + j, 2^(-j/64) from a 64-entry dfloat table (tab[j]) and
// exp(-t) from its Taylor polynomial to degree 5 (remainder below 4e-17).
// ln2/64 is split Cody-Waite style into L0 (11 significant bits, so k L0 is
// exact for k < 2^13) and two smaller parts.  Results below 2^-126 are
// returned as zero.
namespace dfexp {
constexpr double kL = 0.69314718055994530942 / 64.0;
constexpr float kL0 = (float)((double)(long long)(kL * 131072.0 + 0.5) / 131072.0);
constexpr float kL1 = (float)(kL - (double)kL0);
constexpr float kL2 = (float)(kL - (double)kL0 - (double)kL1);
constexpr float kInvL = (float)(64.0 / 0.69314718055994530942);
} // namespace dfexp

__device__ __forceinline__ dfloat df_exp_neg(dfloat x, const float2 *tab) {
  if (!(x.h < 87.0f))
    return dfloat{0.f, 0.f};
  const float kf = rintf(x.h * dfexp::kInvL);
  const int k = (int)kf;
  // t = x - k ln2/64
  const float th = fmaf(-kf, dfexp::kL0, x.h); // exact (Sterbenz)
  dfloat t = df_two_sum(th, x.l);
  const float p = kf * dfexp::kL1;
  const float pe = fmaf(kf, dfexp::kL1, -p) + kf * dfexp::kL2;
  t = df_add(t, dfloat{-p, -pe});
  // exp(s), s = -t: 1 + s + s^2 (1/2 + s (1/6 + s (1/24 + s/120)))
  const dfloat s{-t.h, -t.l};
  const float c = fmaf(s.h, fmaf(s.h, 1.0f / 120.0f, 1.0f / 24.0f), 1.0f / 6.0f);
  const dfloat u = df_two_sum(0.5f, s.h * c);
  dfloat r = df_add(s, df_mul(df_mul(s, s), u));
  r = df_add(dfloat{1.f, 0.f}, r);
  const float2 tj = tab[k & 63];
  r = df_mul(r, dfloat{tj.x, tj.y});
  const int m = k >> 6;
  const float sc = __int_as_float((127 - m) << 23); // 2^-m, m <= 125
  return dfloat{r.h * sc, r.l * sc};
}

__device__ __forceinline__ dfloat df_shfl_xor(dfloat v, int o) {
  return dfloat{__shfl_xor_sync(0xffffffffu, v.h, o), __shfl_xor_sync(0xffffffffu, v.l, o)};
}

// Exact FP32 -> FP64 conversion on the integer pipes (the FP64 pipe, which
// would otherwise do it, is the scarce unit on GB300).  Subnormal inputs
// (|x| < 1.2e-38) flush to signed zero.
__device__ __forceinline__ double f2d_exact(float x) {
  const unsigned u = __float_as_uint(x);
  const unsigned mag = u & 0x7fffffffu;
  const unsigned sign = u & 0x80000000u;
  unsigned hi = sign | ((mag >> 3) + 0x38000000u);
  unsigned lo = mag << 29;
  if (mag < 0x00800000u) {
    hi = sign;
    lo = 0u;
  }
  return __hiloint2double((int)hi, (int)lo);
}

// FP32 -> FP64 for the grid atomics: exact for every normal float, in four
// integer operations (the exponent rebias of f2d_exact without its zero and
// subnormal branch).  Zero and subnormal inputs (|x| < 1.2e-38) become
// doubles of magnitude below 1.2e-38, far under any value the grids resolve.
__device__ __forceinline__ double f2d_grid(float x) {
  const unsigned u = __float_as_uint(x);
  const unsigned hi = (((u >> 3) & 0x0fffffffu) + 0x38000000u) | (u & 0x80000000u);
  return __hiloint2double((int)hi, (int)(u << 29));
}

// ---------------------------------------------------------------------------
// uniform interface over double / float / dfloat
// ---------------------------------------------------------------------------
template <typename N> struct Num;

template <> struct Num<double> {
  using T = double;
  static __device__ __forceinline__ T zero() { return 0.0; }
  static __device__ __forceinline__ T from(double x) { return x; }
  static __device__ __forceinline__ T fma(T acc, T a, T b) { return fma_rn(acc, a, b); }
  static __device__ __forceinline__ T fma_rn(T acc, T a, T b) { return ::fma(a, b, acc); }
  static __device__ __forceinline__ T fma_acc(T acc, T a, T b) { return ::fma(a, b, acc); }
  static __device__ __forceinline__ T norm(T a) { return a; }
  static __device__ __forceinline__ T mul(T a, T b) { return a * b; }
  static __device__ __forceinline__ T add(T a, T b) { return a + b; }
  static __device__ __forceinline__ double to_double(T a) { return a; }
  static __device__ __forceinline__ T shfl_xor(T v, int o) {
    return __shfl_xor_sync(0xffffffffu, v, o);
  }
};

template <> struct Num<float> {
  using T = float;
  static __device__ __forceinline__ T zero() { return 0.f; }
  static __device__ __forceinline__ T from(double x) { return (float)x; }
  static __device__ __forceinline__ T fma(T acc, T a, T b) { return fmaf(a, b, acc); }
  static __device__ __forceinline__ T fma_acc(T acc, T a, T b) { return fmaf(a, b, acc); }
  static __device__ __forceinline__ T norm(T a) { return a; }
  static __device__ __forceinline__ T mul(T a, T b) { return a * b; }
  static __device__ __forceinline__ T add(T a, T b) { return a + b; }
  static __device__ __forceinline__ double to_double(T a) { return f2d_exact(a); }
  static __device__ __forceinline__ T shfl_xor(T v, int o) {
    return __shfl_xor_sync(0xffffffffu, v, o);
  }
};

template <> struct Num<dfloat> {
  using T = dfloat;
  static __device__ __forceinline__ T zero() { return dfloat{0.f, 0.f}; }
  static __device__ __forceinline__ T from(double x) { return df_make(x); }
  static __device__ __forceinline__ T fma(T acc, T a, T b) { return df_fma(acc, a, b); }
  static __device__ __forceinline__ T fma_acc(T acc, T a, T b) { return df_fma_acc(acc, a, b); }
  static __device__ __forceinline__ T norm(T a) { return df_norm(a); }
  static __device__ __forceinline__ T mul(T a, T b) { return df_mul(a, b); }
  static __device__ __forceinline__ T add(T a, T b) { return df_add(a, b); }
  static __device__ __forceinline__ double to_double(T a) {
    return f2d_exact(a.h) + f2d_exact(a.l);
  }
  static __device__ __forceinline__ T shfl_xor(T v, int o) { return df_shfl_xor(v, o); }
};

} // namespace gb300
