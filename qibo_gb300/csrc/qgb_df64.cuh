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

__device__ __forceinline__ double df_to_double(df a) { return (double)a.hi + (double)a.lo; }

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

// Shared-memory pass traits: double2 in HBM, cdf in shared memory.
struct TC128F {
  typedef double2 G;
  typedef cdf S;
  typedef cdf V;
  static constexpr int kind = QGB_C128;
  static V coef(double re, double im) {
    cdf c;
    c.re = df_split(re);
    c.im = df_split(im);
    return c;
  }
  __device__ static V from_global(double2 v) {
    cdf c;
    c.re = df_split(v.x);
    c.im = df_split(v.y);
    return c;
  }
  __device__ static double2 to_global(V v) { return make_double2(df_to_double(v.re), df_to_double(v.im)); }
  __device__ static V load(const S* p, int i) { return p[i]; }
  __device__ static void store(S* p, int i, V v) { p[i] = v; }
  __device__ static V mul(V a, V b) { return cdf_mul(a, b); }
  template <int D>
  __device__ static V row(const V* u, const V* a) { return cdf_row<D>(u, a); }
};
