// Shared types and helpers of the GB300 state-vector engine.
//
// Amplitude "traits" separate how an amplitude is stored in HBM from how it
// is computed on:
//   TC64   complex64: float2 in HBM, FP32 arithmetic.
//   TC128  complex128: double2 in HBM, IEEE FP64 arithmetic.
// Kernels are templates over a traits type, so every kernel exists for every
// precision.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "../../include/qgb300.h"

typedef int64_t i64;
typedef uint64_t u64;

#define QGB_MAXQ 40          // largest supported qubit count (index math is 64-bit)
#define QGB_MAX_CTRL 8
#define QGB_MAX_K 5          // largest dense gate (2^5 x 2^5)

// ---------------------------------------------------------------- errors --
void qgb_set_error(const char* fmt, ...);
int qgb_cuda_status(cudaError_t e, const char* what);

#define QGB_TRY_CUDA(call)                                   \
  do {                                                       \
    cudaError_t _e = (call);                                 \
    if (_e != cudaSuccess) return qgb_cuda_status(_e, #call); \
  } while (0)

void qgb_count_launch();

// after every kernel launch: count it and turn a launch error into a status
#define QGB_LAUNCH_CHECK(what)                                       \
  do {                                                               \
    qgb_count_launch();                                              \
    cudaError_t _e = cudaGetLastError();                             \
    if (_e != cudaSuccess) return qgb_cuda_status(_e, what);         \
  } while (0)

int qgb_num_sms();

// Raise the dynamic shared-memory limit of kernel func to bytes on the
// current device, once per (kernel, device); thread-safe; a QGB status.
int qgb_func_smem(const void* func, int bytes);

// --------------------------------------------------------- complex math --
__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__host__ __device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
// acc + a*b
__host__ __device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 acc) {
  return make_float2(fmaf(-a.y, b.y, fmaf(a.x, b.x, acc.x)), fmaf(a.y, b.x, fmaf(a.x, b.y, acc.y)));
}
__host__ __device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 acc) {
  return make_double2(fma(-a.y, b.y, fma(a.x, b.x, acc.x)), fma(a.y, b.x, fma(a.x, b.y, acc.y)));
}

// Exact float -> double without the conversion instruction, which GB300
// issues on its slow FP64 pipe: integer operations only, on every path
// (a fallback to the instruction would be predicated, i.e. executed for
// every value).  Normal numbers rebias the exponent and widen the mantissa;
// subnormals are normalised (top bit p of the mantissa m: exponent p + 874);
// infinities and NaNs keep their payload.
__device__ __forceinline__ double f2d_exact(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xFFu;
  const uint32_t m = u & 0x7FFFFFu;
  const uint64_t sign = (uint64_t)(u & 0x80000000u) << 32;
  const uint64_t de = e == 0xFFu ? 0x7FFull : (uint64_t)(e + 896u);
  const uint64_t normal = (de << 52) | ((uint64_t)m << 29);
  const int p = 31 - __clz(m | 1u);
  const uint64_t sub = m == 0 ? 0ull
                              : ((uint64_t)(p + 874) << 52) | (((uint64_t)m << (52 - p)) & 0xFFFFFFFFFFFFFull);
  return __longlong_as_double((long long)(sign | (e != 0 ? normal : sub)));
}

// f^2 of a float as an exact double with integer operations only: the
// 24-bit mantissa squared is a 48-bit integer, placed under the exponent
// 2e - 300 (subnormals as exponent 1 without the implicit bit); infinities
// and NaNs give +inf / NaN.
__device__ __forceinline__ double sq_exact(float f) {
  const uint32_t u = __float_as_uint(f) & 0x7FFFFFFFu;
  const uint32_t e = u >> 23;
  const uint32_t m = (u & 0x7FFFFFu) | (e ? 0x800000u : 0u);
  const uint64_t q = (uint64_t)m * m;
  const int p = 63 - __clzll(q | 1ull);
  const uint64_t E = (uint64_t)(p + 2 * (int)(e ? e : 1u) - 300 + 1023);
  const uint64_t fin = q == 0 ? 0ull : (E << 52) | ((q << (52 - p)) & 0xFFFFFFFFFFFFFull);
  const uint64_t special = 0x7FF0000000000000ull | ((u & 0x7FFFFFu) ? (1ull << 51) : 0ull);
  return __longlong_as_double((long long)(e == 0xFFu ? special : fin));
}

// Double-float accumulator for sums of |a|^2 off the FP64 pipe (GB300 runs
// FP64 at about 1/64 of FP32): value hi + lo, every addition an error-free
// two-sum into hi with the rounding error carried in lo, renormalised after
// each step, so a partial keeps about 48 bits; partials are flushed to FP64.
struct DFAcc {
  float hi, lo;
};

__device__ __forceinline__ DFAcc df_add2(DFAcc s, float p, float e) {  // s + (p + e), |e| << |p|
  const float t = s.hi + p;
  const float bp = t - s.hi;
  const float err = (s.hi - (t - bp)) + (p - bp);
  const float lo = s.lo + (err + e);
  const float h = t + lo;
  DFAcc r;
  r.lo = lo - (h - t);
  r.hi = h;
  return r;
}

// a + b and a - b of double-float values (error-free sum of the heads, the
// tails added, renormalised)
__device__ __forceinline__ DFAcc df_plus(DFAcc a, DFAcc b) {
  const float t = a.hi + b.hi;
  const float bp = t - a.hi;
  const float err = (a.hi - (t - bp)) + (b.hi - bp);
  const float lo = (a.lo + b.lo) + err;
  const float h = t + lo;
  return DFAcc{h, lo - (h - t)};
}
__device__ __forceinline__ DFAcc df_minus(DFAcc a, DFAcc b) { return df_plus(a, DFAcc{-b.hi, -b.lo}); }

// x = hi + lo (+ a remainder below 2^-47 |x|) as floats, with integer
// operations and one integer-to-float conversion; valid for 2^-60 <= |x| <
// 2^60 (false otherwise)
__device__ __forceinline__ bool d_split(double x, float* hi, float* lo) {
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7FF) - 1023;
  if (e < -60 || e >= 60) return false;
  const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
  *hi = __uint_as_float(sign | ((uint32_t)(e + 127) << 23) | (uint32_t)((b >> 29) & 0x7FFFFFu));
  const float r = __uint2float_rn((uint32_t)(b & 0x1FFFFFFFu));  // the 29 bits below, rounded to 24
  *lo = __uint_as_float(__float_as_uint(r * __uint_as_float((uint32_t)(e - 52 + 127) << 23)) | sign);
  return true;
}

struct TC64 {
  typedef float2 S;   // storage
  typedef float2 V;   // value computed on
  typedef float R;
  static constexpr int kind = QGB_C64;
  __host__ __device__ static V coef(double re, double im) { return make_float2((float)re, (float)im); }
  __device__ static V zero() { return make_float2(0.f, 0.f); }
  __device__ static V load(const S* p, i64 i) { return p[i]; }
  __device__ static void store(S* p, i64 i, V v) { p[i] = v; }
  __device__ static V mul(V a, V b) { return cmul(a, b); }
  __device__ static V fma(V a, V b, V acc) { return cfma(a, b, acc); }
  __device__ static V row2(V u0, V a0, V u1, V a1) { return cfma(u1, a1, cmul(u0, a0)); }
  // x^2 and y^2 of floats are exact doubles (formed with integer
  // operations), so one FP64 addition gives the correctly rounded |a|^2,
  // the value of fma(x, x, y * y)
  __device__ static double abs2(V a) { return sq_exact(a.x) + sq_exact(a.y); }
  // sums of |a|^2: double-float partials (exact squares as float pairs),
  // flushed to FP64 by acc_value
  typedef DFAcc Acc;
  __device__ static Acc acc_zero() { return DFAcc{0.f, 0.f}; }
  __device__ static Acc acc_add(Acc s, V a, int) {
    const float px = a.x * a.x, py = a.y * a.y;
    s = df_add2(s, px, fmaf(a.x, a.x, -px));
    return df_add2(s, py, fmaf(a.y, a.y, -py));
  }
  __device__ static double acc_value(Acc s) { return f2d_exact(s.hi) + f2d_exact(s.lo); }
  // |a|^2 as a double-float (the squares split exactly)
  __device__ static DFAcc abs2_df(V a) {
    const float px = a.x * a.x, py = a.y * a.y;
    return df_add2(DFAcc{px, fmaf(a.x, a.x, -px)}, py, fmaf(a.y, a.y, -py));
  }
  // acc + |a|^2 as two FMAs (two FP64 operations instead of three)
  __device__ static double acc2(double acc, V a) {
    const double x = f2d_exact(a.x), y = f2d_exact(a.y);
    return ::fma(x, x, ::fma(y, y, acc));
  }
  // off the FP64 pipe: the FP64 factor split once into floats hi + lo (the
  // split is loop-invariant), each value rounded once by fma(x, hi, x lo), so
  // the factor keeps about 48 bits and an FP64 renormalisation stays one to
  // within the rounding of the stored floats
  __device__ static V scale(V a, double s) {
    const float hi = (float)s, lo = (float)(s - (double)hi);
    return make_float2(fmaf(a.x, hi, a.x * lo), fmaf(a.y, hi, a.y * lo));
  }
  __device__ static V neg(V a) { return make_float2(-a.x, -a.y); }
  __device__ static double re(V a) { return f2d_exact(a.x); }
  __device__ static double im(V a) { return f2d_exact(a.y); }
};

struct TC128 {
  typedef double2 S;
  typedef double2 V;
  typedef double R;
  static constexpr int kind = QGB_C128;
  __host__ __device__ static V coef(double re, double im) { return make_double2(re, im); }
  __device__ static V zero() { return make_double2(0., 0.); }
  __device__ static V load(const S* p, i64 i) { return p[i]; }
  __device__ static void store(S* p, i64 i, V v) { p[i] = v; }
  __device__ static V mul(V a, V b) { return cmul(a, b); }
  __device__ static V fma(V a, V b, V acc) { return cfma(a, b, acc); }
  __device__ static V row2(V u0, V a0, V u1, V a1) { return cfma(u1, a1, cmul(u0, a0)); }
  __device__ static double abs2(V a) { return fma_d(a.x, a.x, a.y * a.y); }
  __device__ static double acc2(double acc, V a) { return ::fma(a.x, a.x, ::fma(a.y, a.y, acc)); }
  // sums of |a|^2: amplitudes with ``alt`` set (every other loop step, the
  // same for a whole warp) go to a double-float partial through d_split,
  // the others to an FP64 partial, which halves the FP64 work; values
  // outside d_split's range take the FP64 partial
  struct Acc {
    double d;
    DFAcc f;
  };
  __device__ static Acc acc_zero() { return Acc{0.0, DFAcc{0.f, 0.f}}; }
  __device__ static Acc acc_add(Acc s, V a, int alt) {
    float xh, xl, yh, yl;
    if (alt && d_split(a.x, &xh, &xl) && d_split(a.y, &yh, &yl)) {
      const float px = xh * xh, py = yh * yh;
      // x^2 = xh^2 + (2 xh + xl) xl, the first product split exactly
      s.f = df_add2(s.f, px, fmaf(2.f * xh + xl, xl, fmaf(xh, xh, -px)));
      s.f = df_add2(s.f, py, fmaf(2.f * yh + yl, yl, fmaf(yh, yh, -py)));
    } else {
      s.d = acc2(s.d, a);
    }
    return s;
  }
  __device__ static double acc_value(Acc s) { return s.d + (f2d_exact(s.f.hi) + f2d_exact(s.f.lo)); }
  // |a|^2 as a double-float: split parts squared on the FP32 pipe; a part
  // of 2^60 or more goes through one FP64 square, one below 2^-60 adds
  // less than 2^-120
  __device__ static DFAcc abs2_df(V a) {
    float xh, xl, yh, yl;
    DFAcc r{0.f, 0.f};
    if (d_split(a.x, &xh, &xl)) {
      const float p = xh * xh;
      r = df_add2(r, p, fmaf(2.f * xh + xl, xl, fmaf(xh, xh, -p)));
    } else if (fabs(a.x) >= 0x1p60) {
      r = df_add2(r, (float)(a.x * a.x), 0.f);
    }
    if (d_split(a.y, &yh, &yl)) {
      const float p = yh * yh;
      r = df_add2(r, p, fmaf(2.f * yh + yl, yl, fmaf(yh, yh, -p)));
    } else if (fabs(a.y) >= 0x1p60) {
      r = df_add2(r, (float)(a.y * a.y), 0.f);
    }
    return r;
  }
  __device__ static double fma_d(double a, double b, double c) { return ::fma(a, b, c); }
  __device__ static V scale(V a, double s) { return make_double2(a.x * s, a.y * s); }
  __device__ static V neg(V a) { return make_double2(-a.x, -a.y); }
  __device__ static double re(V a) { return a.x; }
  __device__ static double im(V a) { return a.y; }
};

// ------------------------------------------------------- index helpers --
// Positions are amplitude-index bit positions (bit b has stride 2^b).
// qibo qubit q of an n-qubit state sits at bit n-1-q.
struct BitInsert {
  int n;          // number of inserted (fixed) bits
  int pos[QGB_MAX_K + QGB_MAX_CTRL + 2];  // ascending
};

// Insert a zero at every position of ``bi`` (ascending order) into t.
__device__ __forceinline__ i64 insert_zeros(i64 t, const BitInsert& bi) {
#pragma unroll 4
  for (int j = 0; j < bi.n; ++j) {
    const int p = bi.pos[j];
    t = ((t >> p) << (p + 1)) | (t & ((((i64)1) << p) - 1));
  }
  return t;
}

// Launch geometry: grid-stride loops with a grid that is a multiple of the
// SM count (152 on GB300), capped so each thread does several items.
inline void grid_for(i64 items, int threads, int* blocks) {
  const int sms = qgb_num_sms();
  i64 b = (items + threads - 1) / threads;
  i64 cap = (i64)sms * 16;  // 16 resident-ish CTAs of 256 threads per SM
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  *blocks = (int)b;
}

inline int dtype_bytes(int dtype) { return dtype == QGB_C128 ? 16 : 8; }
inline bool dtype_ok(int dtype) { return dtype == QGB_C64 || dtype == QGB_C128; }
