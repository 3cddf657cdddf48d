// Double-float ("df64") arithmetic on the FP32 pipe for complex128 passes.
//
// GB300 runs FP64 FMA at about 1/60 of its FP32 rate (measured 1.2 vs 70
// TFLOP/s), so a complex128 dense gate done in IEEE FP64 is bound by the
// FP64 pipe at about a third of HBM bandwidth.  Inside a shared-memory pass
// the tile is converted once to pairs of floats x = hi + lo (|lo| <= ulp(hi)/2,
// about 48 significant bits) and every gate of the pass is computed with
// error-free transformations on the FP32 pipe:
//   TwoProd(a, b): p = a*b, e = fma(a, b, -p)          (a*b = p + e exactly)
//   TwoSum(a, b):  s = a+b, e = (a-(s-bb)) + (b-bb)    (a+b = s + e exactly)
// (Dekker 1971; Knuth, TAOCP vol. 2, 4.2.2).  A row of a gate is summed with
// its leading products added exactly and the small terms in FP32, then
// renormalised, so each gate adds a relative error of a few 2^-48.  The tile
// is converted back to IEEE doubles when it is written (hi + lo is exact in
// FP64).  Storage in HBM stays complex128 throughout.
#pragma once

#include "qgb_common.cuh"

struct df {
  float hi, lo;
};
struct __align__(16) cdf {
  df re, im;
};

__host__ __device__ __forceinline__ df df_split(double x) {
  const float hi = (float)x;
  return {hi, (float)(x - (double)hi)};
}

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ df df_renorm(float s, float e) {
  const float hi = s + e;
  return {hi, e - (hi - s)};
}

// sum_k sx[k] * x[k] * y[k] over NT terms (sx = +1/-1), leading products exact
template <int NT>
__device__ __forceinline__ df df_dot(const df* x, const df* y, const float* sx) {
  float s = 0.f, e = 0.f;
#pragma unroll
  for (int k = 0; k < NT; ++k) {
    const float xh = sx[k] * x[k].hi, xl = sx[k] * x[k].lo;
    const float p = xh * y[k].hi;
    e += fmaf(xh, y[k].hi, -p);
    e += fmaf(xh, y[k].lo, xl * y[k].hi);
    if (k == 0) {
      s = p;
    } else {
      float t;
      two_sum(s, p, s, t);
      e += t;
    }
  }
  return df_renorm(s, e);
}

// sum_c u[c] * a[c] (complex), one output of a D-column gate row
template <int D>
__device__ __forceinline__ cdf cdf_row(const cdf* u, const cdf* a) {
  df xr[2 * D], yr[2 * D], xi[2 * D], yi[2 * D];
  float sr[2 * D], si[2 * D];
#pragma unroll
  for (int c = 0; c < D; ++c) {
    xr[2 * c] = u[c].re; yr[2 * c] = a[c].re; sr[2 * c] = 1.f;
    xr[2 * c + 1] = u[c].im; yr[2 * c + 1] = a[c].im; sr[2 * c + 1] = -1.f;
    xi[2 * c] = u[c].re; yi[2 * c] = a[c].im; si[2 * c] = 1.f;
    xi[2 * c + 1] = u[c].im; yi[2 * c + 1] = a[c].re; si[2 * c + 1] = 1.f;
  }
  cdf r;
  r.re = df_dot<2 * D>(xr, yr, sr);
  r.im = df_dot<2 * D>(xi, yi, si);
  return r;
}

__device__ __forceinline__ cdf cdf_mul(cdf x, cdf y) { return cdf_row<1>(&x, &y); }

// ---------------------------------------------------------------------------
// Per-gate complex128 kernels in double-float.  A gate pass reads and writes
// every IEEE double once, so the conversions cannot be amortised over many
// gates as in a shared-memory pass; they avoid the FP64 pipe instead.
//
// Split: hi = x with its mantissa truncated to 24 bits; the 29 remaining
// mantissa bits r give lo = RN(r) * 2^(e - 1075), |lo| < ulp(hi), so
// x - (hi + lo) is below 2^-47 |x| (for |x| >= 2^-100; below, lo is a
// subnormal float and the error below 2^-149).  df_split_exact covers the
// exponent fields E < 950 and E > 1150 with integer operations, one integer
// to float conversion and two multiplications by powers of two: |x| <
// 2^-126 becomes 0, |x| >= 2^128 an infinity, NaN a NaN.
__device__ __forceinline__ df df_split_exact(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const uint32_t h = (uint32_t)(u >> 32), l = (uint32_t)u;
  const uint32_t sign = h & 0x80000000u;
  const int E = (int)((h >> 20) & 0x7FF);
  const int fe = E - 896;  // float exponent field of hi
  const uint32_t mant = ((h & 0xFFFFFu) << 3) | (l >> 29);
  const bool nan = E == 0x7FF && ((h & 0xFFFFFu) | l) != 0;
  uint32_t hib = sign | ((uint32_t)fe << 23) | mant;
  hib = fe <= 0 ? sign : fe >= 255 ? (sign | 0x7F800000u | (nan ? 0x400000u : 0u)) : hib;
  // 2^(E - 1075) as 2^(E - 1011) * 2^-64: the first factor is a normal float
  // whenever hi is, and the second rounds lo into the subnormals gradually
  const float p2 = (fe > 0 && fe < 255) ? __uint_as_float((uint32_t)(E - 884) << 23) : 0.f;
  const float lo = __uint_as_float(__float_as_uint((__uint2float_rn(l & 0x1FFFFFFFu) * p2) * 5.42101086242752217e-20f) | sign);
  return {__uint_as_float(hib), lo};
}

// The rare cases of the two conversions below, out of line: a call is a
// branch the compiler cannot turn into predicated code on the common path.
static __device__ __noinline__ df df_split_rare(double x) { return df_split_exact(x); }
static __device__ __noinline__ double df_join_rare(float hi, float lo) { return (double)hi + (double)lo; }

// The same split, shorter for 2^-73 <= |x| < 2^128 (the exponent field E
// in [950, 1150]): hi's bits are bits 60..29 of x shifted left by 3 (the
// top 23 fraction bits under the low 9 exponent bits), re-biased by
// subtracting 0x180 from that 9-bit field modulo 2^9 (E - 896 = E mod 2^9 -
// 384 modulo 2^9, sign restored); lo is the low 29 fraction bits as a
// float times 2^(E - 1075), a normal float in this range.
__device__ __forceinline__ df df_split_int(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const uint32_t h = (uint32_t)(u >> 32), l = (uint32_t)u;
  const uint32_t E = (h >> 20) & 0x7FFu;
  if (__builtin_expect(E - 950u > 200u, 0)) return df_split_rare(x);
  const uint32_t w = __funnelshift_l(l, h, 3);
  const uint32_t sign = h & 0x80000000u;
  const uint32_t hib = ((w - 0xC0000000u) & 0x7FFFFFFFu) | sign;
  const float lo = __uint2float_rn(l & 0x1FFFFFFFu) * __uint_as_float((E - 948u) << 23);
  return {__uint_as_float(hib), __uint_as_float(__float_as_uint(lo) | sign)};
}

// hi + lo rounded once to an IEEE double (RN(hi + lo), as an FP64 addition
// of the widened floats gives), without the FP64 pipe when hi is normal and
// at least 2^-75, and the sum stays in hi's binade: hi widens by integer
// operations, and lo, in units of the double's last place at hi's exponent
// (one FP32 multiplication by 2^(179 - e) with hi's sign, exact), is rounded
// to an integer (ties to even) and added to the widened bits.  The binade is
// kept when that integer is below 2^29 in magnitude and, for hi a power of
// two, not negative.  Other pairs (zeros, subnormals, |hi| < 2^-75,
// infinities, NaNs, a lo at least as large as ulp(hi) after a cancellation)
// take one FP64 addition.
__device__ __forceinline__ double df_join(df a) {
  const uint32_t uh = __float_as_uint(a.hi);
  const uint32_t ex = uh & 0x7F800000u;
  const float scale = __uint_as_float(((306u << 23) - ex) | (uh & 0x80000000u));
  const float rf = a.lo * scale;
  const bool fast = (ex - (52u << 23)) < (203u << 23) && fabsf(rf) < 536870912.0f &&
                    ((uh & 0x7FFFFFu) != 0u || rf >= 0.f);
  if (__builtin_expect(!fast, 0)) return df_join_rare(a.hi, a.lo);
  const int64_t mag = ((int64_t)(uh & 0x7FFFFFFFu) << 29) + (int64_t)__float2int_rn(rf) + ((int64_t)896 << 52);
  return __longlong_as_double((long long)((uint64_t)mag | ((uint64_t)(uh & 0x80000000u) << 32)));
}

// hi + lo rounded once to an IEEE double by one FP64 addition, the two
// floats widened with integer operations (hi and lo come out of df_renorm,
// so each is a zero or a normal float, except a lo below 2^-126, which read
// as normal errs by less than 2^-125; infinities and NaNs keep exponent
// 2047).  Shared-memory passes use this form: their FP64 pipe is idle.
__device__ __forceinline__ double f2d_join(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xFFu;
  const uint64_t sign = (uint64_t)(u & 0x80000000u) << 32;
  const uint64_t de = e == 0xFFu ? 0x7FFull : (uint64_t)(e + 896u);
  const uint64_t bits = (u << 1) == 0 ? 0ull : (de << 52) | ((uint64_t)(u & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)(sign | bits));
}
__device__ __forceinline__ double df_join_fp64(df a) { return f2d_join(a.hi) + f2d_join(a.lo); }

__device__ __forceinline__ df df_add(df a, df b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e += a.lo + b.lo;
  return df_renorm(s, e);
}

// Per-gate traits: double2 in HBM, cdf in registers (k_1q_pairs, k_1q_shfl).
struct DF128 {
  typedef double2 S;
  typedef cdf V;
  static constexpr int kind = QGB_C128;
  static V coef(double re, double im) {
    cdf c;
    c.re = df_split(re);
    c.im = df_split(im);
    return c;
  }
  __device__ static V load(const S* p, i64 i) {
    const double2 v = p[i];
    cdf c;
    c.re = df_split_int(v.x);
    c.im = df_split_int(v.y);
    return c;
  }
  __device__ static void store(S* p, i64 i, V v) { p[i] = make_double2(df_join(v.re), df_join(v.im)); }
  __device__ static V mul(V a, V b) { return cdf_mul(a, b); }
  // u0 a0 + u1 a1 as one error-free dot product per real output
  __device__ static V row2(V u0, V a0, V u1, V a1) {
    const cdf u[2] = {u0, u1}, a[2] = {a0, a1};
    return cdf_row<2>(u, a);
  }
  __device__ static V fma(V a, V b, V acc) {
    const cdf m = cdf_mul(a, b);
    cdf r;
    r.re = df_add(acc.re, m.re);
    r.im = df_add(acc.im, m.im);
    return r;
  }
};

// Shared-memory pass traits: double2 in HBM, cdf in shared memory.
struct TC128F {
  typedef double2 G;
  typedef cdf S;
  typedef cdf V;
  static constexpr int kind = QGB_C128;
  __device__ static V one() { return cdf{{1.f, 0.f}, {0.f, 0.f}}; }
  static V coef(double re, double im) {
    cdf c;
    c.re = df_split(re);
    c.im = df_split(im);
    return c;
  }
  // tiles convert with integer operations (df_split_exact) and one FP64
  // addition per double on the way back (df_join_fp64): branch-free forms,
  // measured faster inside the passes than the per-gate kernels' fast paths
  __device__ static V from_global(double2 v) {
    cdf c;
    c.re = df_split_exact(v.x);
    c.im = df_split_exact(v.y);
    return c;
  }
  __device__ static double2 to_global(V v) { return make_double2(df_join_fp64(v.re), df_join_fp64(v.im)); }
  __device__ static V load(const S* p, int i) { return p[i]; }
  __device__ static void store(S* p, int i, V v) { p[i] = v; }
  __device__ static V mul(V a, V b) { return cdf_mul(a, b); }
  template <int D>
  __device__ static V row(const V* u, const V* a) { return cdf_row<D>(u, a); }
  template <int D>  // u real: one error-free dot product of D terms per part
  __device__ static V row_real(const V* u, const V* a) {
    df x[D], yr[D], yi[D];
    float sg[D];
#pragma unroll
    for (int c = 0; c < D; ++c) {
      x[c] = u[c].re;
      yr[c] = a[c].re;
      yi[c] = a[c].im;
      sg[c] = 1.f;
    }
    cdf r;
    r.re = df_dot<D>(x, yr, sg);
    r.im = df_dot<D>(x, yi, sg);
    return r;
  }
};
