// Fused 5-qubit blocks in complex128 on the BF16 tensor cores (Ozaki scheme).
//
// The block acts on each group of 32 amplitudes as the realified 64x64 matrix
// B (see qgb_tc.cu), so 128 groups form D[128 x 64] = A[128 x 64] * B^T, here
// to FP64 accuracy.  GB300 runs FP64 at about 1/60 of FP32, and the BF16
// tensor cores at about 2 PFLOP/s; the product is therefore split into
// error-free integer pieces (Ozaki, Ogita, Oishi, Rump, "Error-free
// transformations of matrix multiplication by using fast routines of matrix
// multiplication and its applications", Numer. Algorithms 59 (2012)):
//
//  * every value of a tile (and every entry of a gate row) is written in
//    47-bit fixed point against the largest exponent sharing its scale (one
//    per tile of A, one per output row of B), and split into six balanced
//    base-256 digits d in [-128, 128] (exact as bf16);
//  * A_i * B_j^T over K = 64 then sums products of at most 2^14, so every
//    level l = i + j <= 6 accumulates exactly in its own FP32 accumulator
//    (|sum| <= 7 * 2^20 < 2^24);
//  * the seven level accumulators are combined with integer arithmetic into
//    sum_{l<=5} acc_l 256^(5-l) + round(acc_6 / 256) and rounded once to an
//    IEEE double.
//  With 2^E, 2^F the tile and gate-row scales (2^E <= 2 x the tile's largest
//  |value|), the fixed-point rounding of both operands over K = 64 and the
//  dropped levels (l >= 7) bound the error of an output by 2^(E + F - 41);
//  independent roundings give about 2^(E + F - 46).  Normalised states and
//  unitary blocks have 2^(E + F) <= 4, and far less for spread-out states.
//  The CPU replay tests/native/oz_check.cu checks the bound output by output.
//
// Tensor memory holds the seven level accumulators side by side (columns
// 64 l .. 64 l + 63, 448 of 512).  The six B slices are stacked along N (rows
// 64 j + n), so the MMA for A slice i with B slices 0..min(5, 6-i) written at
// TMEM column 64 i lands each product A_i B_j in level i + j: 9 instructions
// per K-step of 16 (N = 384 and 320 are split at 256; the first write of
// level 6 is its own instruction so that it starts the accumulation), 37
// per tile.
//
// A CTA (512 threads, one per SM: 223 KB of shared memory, 448 TMEM columns)
// owns 4096-amplitude tiles with the index geometry of qgb_tc.cu.  Warps 0-7
// convert (thread t moves amplitudes t + 256 r, r < 16, prefetched into
// registers while the previous MMAs run) and issue the MMAs; warps 8-15 read
// the levels from TMEM, combine and store, overlapping the conversion of the
// next tile.  The digit split runs on the FMA pipe (exact FP32 arithmetic
// on 16-bit chunks), the level combination as an integer multiply-add chain.
// Every wait on an mbarrier is bounded: on timeout the kernel records an
// error flag, both groups stop at their next check, the converter waits once
// more (bounded) for its in-flight MMAs, and tensor memory is freed.
//
// Runs of unitary blocks (qgb_run_oz_chain) keep the state in a 64-bit
// fixed-point format between blocks (k_fused5_oz<true>), converted from and
// back to IEEE doubles once per run.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "qgb_plan.h"
#include "qgb_tcgen05.cuh"

#define OZ_THREADS 512  // 8 converter warps + 8 epilogue warps
#define OZ_GROUP 256    // threads per group
#define OZ_STEPS 16     // amplitudes per group thread per tile
#define OZ_TILE 4096   // amplitudes per tile
#define OZ_NSLICE 6    // digits per value
#define OZ_NLEVEL 7    // digit-product levels kept (i + j <= 6)
#define OZ_TMEM_COLS 512
// A slices: 128 rows x 64 bf16, K-major no-swizzle core matrices (8 rows x
// 16 B); row groups 144 B apart, K chunks a_lbo = 2304 + 16 rot apart.
#define OZ_A_SBO 144
#define OZ_A_LBO0 2304
#define OZ_A_SLICE (8 * (OZ_A_LBO0 + 64))  // 18944
// B: 384 rows (6 slices x 64) x 64 bf16, dense core matrices
#define OZ_B_ROWS (OZ_NSLICE * 64)
#define OZ_B_SBO 128
#define OZ_B_LBO (OZ_B_ROWS / 8 * OZ_B_SBO)  // 6144
#define OZ_OFF_A 0
#define OZ_OFF_B (OZ_OFF_A + OZ_NSLICE * OZ_A_SLICE)  // 113664
#define OZ_SMEM (OZ_OFF_B + 8 * OZ_B_LBO)             // 162816

static_assert(OZ_OFF_B % 16 == 0, "operand regions 16-byte aligned");
static_assert(OZ_SMEM <= 227 * 1024, "one CTA per SM");
static_assert(OZ_GROUP * OZ_STEPS == OZ_TILE, "one amplitude per group thread and step");

// Tile geometry (the tile of the complex64 kernel).  Loads: tile index
// j = t + 256 r (t a converter thread) has global offset base + (t & 127) +
// t7 g7 + ghi[r] (t7 bit 7 of t); its (re, im) bf16 pair sits at byte
// aoff_lo[t] + aoff_hi[r] of every A slice.  Stores: output (group row,
// permuted block column c) goes to base + rowoff[row] + coloff[c], straight
// from the epilogue's registers (a warp's lanes are consecutive rows, i.e.
// the tile's lowest non-block index bits).
struct OzGeom {
  int nrest;
  int rest[32];
  uint32_t a_lbo;
  i64 g7;
  i64 ghi[OZ_STEPS];
  uint32_t aoff_lo[OZ_GROUP];
  uint32_t aoff_hi[OZ_STEPS];
  i64 rowoff[128];
  i64 coloff[32];
};

// The (permuted) block in FP64 and, per output row r, the biased exponent of
// its largest |entry| (the scale of that row's digits).
struct OzGate {
  double ur[32][32];
  double ui[32][32];
  int fexp[32];
};

__host__ __device__ __forceinline__ uint64_t oz_dbits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  memcpy(&u, &x, 8);
  return u;
#endif
}

__host__ __device__ __forceinline__ double oz_bitsd(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, 8);
  return x;
#endif
}

__host__ __device__ __forceinline__ uint32_t oz_fbits(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  uint32_t u;
  memcpy(&u, &x, 4);
  return u;
#endif
}

// 47-bit fixed-point value of x against exponent exm (the biased exponent
// of the largest |value| sharing the scale): X = round(x 2^(1069 - exm)),
// |X| <= 2^47, rounding error <= 2^(exm - 1070) in x; values below 2^-58 of
// the scale and subnormals become 0.
__host__ __device__ __forceinline__ int64_t oz_fix47(double x, int exm) {
  const uint64_t u = oz_dbits(x);
  const uint32_t hi = (uint32_t)(u >> 32);
  const int ex = (int)((hi >> 20) & 0x7FF);
  const int rs = 6 + exm - ex;
  if (ex == 0 || rs >= 60) return 0;
  const uint64_t M = ((uint64_t)((hi & 0xFFFFFu) | 0x100000u) << 32) | (uint32_t)u;
  const int64_t X = (int64_t)(((M >> (rs - 1)) + 1) >> 1);  // round half up
  return (int32_t)hi < 0 ? -X : X;
}

// exact float of an integer 0 <= c < 2^23, and of |c| < 2^22
__host__ __device__ __forceinline__ float oz_u2f(uint32_t c) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(0x4B000000u | c) - 8388608.0f;
#else
  return (float)c;
#endif
}
__host__ __device__ __forceinline__ float oz_i2f(int32_t c) {
#ifdef __CUDA_ARCH__
  return __int_as_float(0x4B400000 + c) - 12582912.0f;
#else
  return (float)c;
#endif
}

// nearest integer, ties to even, of |v| < 2^22, as a float (IEEE addition:
// neither compiler folds (v + C) - C without fast-math)
__host__ __device__ __forceinline__ float oz_rintf(float v) { return (v + 12582912.0f) - 12582912.0f; }

// Balanced base-256 digits of a 47-bit fixed-point value, as exact floats:
//   X = sum_{i<6} d[i] 256^(5-i),   |d[i]| <= 128.
// X splits into a signed top (bits 32..47) and two 16-bit chunks, each
// converted exactly to FP32; every digit is then w - 256 rint(w / 256) on
// the FMA pipe, carrying rint(.) upwards.
__host__ __device__ __forceinline__ void oz_digits_f(int64_t X, float d[OZ_NSLICE]) {
  const uint32_t lo = (uint32_t)X;
  const int32_t hi = (int32_t)(X >> 32);
  float w = oz_u2f(lo & 0xFFFFu);
  float q = oz_rintf(w * 0.00390625f);
  d[5] = w - 256.0f * q;
  float t = oz_rintf(q * 0.00390625f);
  d[4] = q - 256.0f * t;
  w = oz_u2f(lo >> 16) + t;
  q = oz_rintf(w * 0.00390625f);
  d[3] = w - 256.0f * q;
  t = oz_rintf(q * 0.00390625f);
  d[2] = q - 256.0f * t;
  w = oz_i2f(hi) + t;
  q = oz_rintf(w * 0.00390625f);
  d[1] = w - 256.0f * q;
  d[0] = q;
}

// the same digits as integers (host checks and the B slices)
__host__ __device__ __forceinline__ void oz_digits(double x, int exm, int d[OZ_NSLICE]) {
  float f[OZ_NSLICE];
  oz_digits_f(oz_fix47(x, exm), f);
#pragma unroll
  for (int i = 0; i < OZ_NSLICE; ++i) d[i] = (int)f[i];
}

// bf16 bit pattern of an integer |d| <= 256 (exact)
__host__ __device__ __forceinline__ uint32_t oz_bf16(int d) {
#ifdef __CUDA_ARCH__
  const float f = __int_as_float(0x4B400000 + d) - 12582912.0f;
#else
  const float f = (float)d;
#endif
  return oz_fbits(f) >> 16;
}

// (re, im) digit pair as packed bf16x2 (re in the low half); the digits are
// integers |d| <= 128, exact in bf16
__host__ __device__ __forceinline__ uint32_t oz_pack(float dre, float dim) {
#ifdef __CUDA_ARCH__
  return __byte_perm(__float_as_uint(dre), __float_as_uint(dim), 0x7632);
#else
  return (oz_fbits(dre) >> 16) | (oz_fbits(dim) & 0xFFFF0000u);
#endif
}

__host__ __device__ __forceinline__ int oz_clz64(uint64_t a) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)a);
#else
  return __builtin_clzll(a);
#endif
}

// T * 2^sc as an IEEE double (one rounding, to nearest even; 0 below the
// normal range)
__host__ __device__ __forceinline__ double oz_i64_to_double(int64_t T, int sc) {
  if (T == 0) return 0.0;
  const uint64_t s = (uint64_t)T & (1ull << 63);
  uint64_t a = T < 0 ? (uint64_t)(-T) : (uint64_t)T;
  const int lz = oz_clz64(a);
  a <<= lz;  // top bit at 63
  uint64_t mant = a >> 11;
  const uint32_t rb = (uint32_t)a & 0x7FFu;
  mant += (rb > 0x400u || (rb == 0x400u && (mant & 1))) ? 1 : 0;
  const int be = 63 - lz + sc + 1023;  // biased exponent of the result
  if (be <= 0) return oz_bitsd(s);
  return oz_bitsd(s | (((uint64_t)(be - 1) << 52) + mant));
}

// The level accumulators (integers in floats; levels 0..3 are below 2^22 and
// converted exactly, levels 4..6 only need their top bits) as
//   T = sum_{l<=3} acc[l] 256^(5-l) + 4 round(acc[4]/4) 256 + 4 round(acc[5]/4)
//       + round(acc[6]/256).
// Each level is rounded by a magic-constant addition on the FMA pipe; the
// integer then sits in the raw bits minus 0x4B400000, and that offset is
// folded into one constant of the multiply-add chain.
__host__ __device__ __forceinline__ int64_t oz_levels(const float acc[OZ_NLEVEL]) {
  const int32_t K = 0x4B400000;
  const float C = 12582912.0f;
  const int32_t b0 = (int32_t)oz_fbits(acc[0] + C), b1 = (int32_t)oz_fbits(acc[1] + C);
  const int32_t b2 = (int32_t)oz_fbits(acc[2] + C), b3 = (int32_t)oz_fbits(acc[3] + C);
  const int32_t b4 = (int32_t)oz_fbits(acc[4] * 0.25f + C), b5 = (int32_t)oz_fbits(acc[5] * 0.25f + C);
  const int32_t b6 = (int32_t)oz_fbits(acc[6] * 0.00390625f + C);
  const int32_t H = (b0 - K) * 256 + (b1 - K);
  const int64_t L = (int64_t)b2 * 16777216 + (int64_t)b3 * 65536 + (int64_t)b4 * 1024 + (int64_t)b5 * 4 +
                    (int64_t)b6 - (int64_t)K * (16777216 + 65536 + 1024 + 4 + 1);
  return L + (int64_t)H * ((int64_t)1 << 32);
}

// T * 2^sc as an IEEE double
__host__ __device__ __forceinline__ double oz_combine(const float acc[OZ_NLEVEL], int sc) {
  return oz_i64_to_double(oz_levels(acc), sc);
}

// Shift amounts of round(T 2^k) without branches (one pair per output
// column, shared by its real and imaginary parts): lsh = max(k, 0),
// rsh = min(max(-k, 0), 62) (a shift by 62 already rounds every |T| < 2^61
// to 0).
struct OzShift {
  int lsh, rsh;
};
__host__ __device__ __forceinline__ OzShift oz_shift(int k) {
  OzShift r;
  r.lsh = k > 0 ? k : 0;
  r.rsh = k < 0 ? (k > -62 ? -k : 62) : 0;
  return r;
}

// round(T * 2^k) as a 64-bit integer (fixed-point output; |result| < 2^62),
// straight-line code
__host__ __device__ __forceinline__ int64_t oz_combine_fix(const float acc[OZ_NLEVEL], OzShift sh) {
  const int64_t t = (int64_t)((uint64_t)oz_levels(acc) << sh.lsh);
  return (t + (((int64_t)1 << sh.rsh) >> 1)) >> sh.rsh;
}

// Fixed-point state format between consecutive tensor-core blocks: a real
// x is held as the integer X = round(x 2^(62 - e)), e a state-wide scale with
// 2^e > 2 ||psi|| (so |X| < 2^61, and unitary blocks keep it there).
__host__ __device__ __forceinline__ int64_t oz_to_fix(double x, int e) {
  const uint64_t u = oz_dbits(x);
  const uint32_t hi = (uint32_t)(u >> 32);
  const int ex = (int)((hi >> 20) & 0x7FF);
  if (ex == 0) return 0;
  const uint64_t M = ((uint64_t)((hi & 0xFFFFFu) | 0x100000u) << 32) | (uint32_t)u;
  const int sh = ex - 1013 - e;  // X = M 2^sh
  int64_t X;
  if (sh >= 0) X = (int64_t)(M << (sh < 8 ? sh : 8));  // sh <= 8 when |x| < 2^(e-1)
  else if (sh <= -60) X = 0;
  else X = (int64_t)(((M >> (-sh - 1)) + 1) >> 1);
  return (int32_t)hi < 0 ? -X : X;
}

__host__ __device__ __forceinline__ double oz_from_fix(int64_t X, int e) { return oz_i64_to_double(X, e - 62); }

// 47-bit value of a fixed-point X at tile shift sh (the tile's largest |X|
// is below 2^(47 + sh)), rounding half up
__host__ __device__ __forceinline__ int64_t oz_fix47_fix(int64_t X, int sh) {
  return (X + (((int64_t)1 << sh) >> 1)) >> sh;  // sh >= 0; no rounding term for sh = 0
}

// byte offset of element (row, k) of the stacked B slices (dense, K-major)
__host__ __device__ __forceinline__ uint32_t oz_boff(uint32_t row, uint32_t k) {
  return (k >> 3) * OZ_B_LBO + (row >> 3) * OZ_B_SBO + (row & 7) * 16 + (k & 7) * 2;
}

// kind::f16 instruction descriptor: D f32, A/B bf16, both K-major, N, M = 128
__host__ __device__ constexpr uint32_t oz_idesc(int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void oz_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void oz_bar(int id) { asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(OZ_GROUP) : "memory"); }

__device__ __forceinline__ void oz_arrive(uint32_t mbar) {
  asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];\n" ::"r"(mbar) : "memory");
}

// FIX: the state holds fixed-point integers (oz_to_fix) instead of IEEE
// doubles; the tile scale is then a shift and the output a rounding shift.
//
// Warps 0-7 convert: tile scale, digits into the A slices, and thread 0
// issues the tile's MMAs.  Warps 8-15 read the level accumulators from
// TMEM, combine them and store them straight to the state.  The converters of tile
// i + 1 run while the epilogue of tile i runs, and the epilogue's stores
// overlap the MMAs of tile i + 1.  Handoffs (each completes once per tile,
// and no waiter can fall two phases behind):
//   mb_full  (tcgen05.commit)       MMAs of tile i done: A free, TMEM ready
//   mb_tfree (epilogue thread 0)    TMEM of tile i read: MMAs of i + 1 may start
//   mb_scale (converter thread 0)   the scale of tile i is in tile_scale[i & 1]
template <bool FIX>
__global__ void __launch_bounds__(OZ_THREADS, 1)
    k_fused5_oz(double2* __restrict__ psi, i64 ntiles, const __grid_constant__ OzGeom geo,
                const __grid_constant__ OzGate G, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) uint64_t mb_full, mb_tfree, mb_scale;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;      // set by either group on a failed wait
  __shared__ int c_stop, e_stop;  // each group's decision, written by its thread 0 before its barrier
  __shared__ uint32_t red[OZ_GROUP / 32], red_hi[OZ_GROUP / 32];
  __shared__ int tile_scale[2];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t s_base = smem_u32(sm);
  const uint32_t mfull = smem_u32(&mb_full), mtfree = smem_u32(&mb_tfree), mscale = smem_u32(&mb_scale);

  // B slices: stacked row 64 j + n holds digit j of realified row n
  // (n = 2 r + re/im of output r), column k = 2 c + re/im of input c
  for (int e = tid; e < 64 * 64; e += OZ_THREADS) {
    const int n = e >> 6, k = e & 63, r = n >> 1, c = k >> 1;
    double v;
    if ((n & 1) == 0) v = (k & 1) == 0 ? G.ur[r][c] : -G.ui[r][c];
    else v = (k & 1) == 0 ? G.ui[r][c] : G.ur[r][c];
    int d[OZ_NSLICE];
    oz_digits(v, G.fexp[r], d);
#pragma unroll
    for (int j = 0; j < OZ_NSLICE; ++j) *(uint16_t*)(sm + OZ_OFF_B + oz_boff(64 * j + n, k)) = (uint16_t)oz_bf16(d[j]);
  }
  if (tid == 0) {
    abort_flag = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mfull));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mtfree));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mscale));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_base)),
                 "r"(OZ_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_base;
  const uint32_t a_lbo = geo.a_lbo;
  const int my_rest = lane < geo.nrest ? geo.rest[lane] : -1;
  const int g = tid & (OZ_GROUP - 1);  // thread within its group
  const i64 toff = (i64)(g & 127) + ((g >> 7) ? geo.g7 : 0);

  if (warp < OZ_GROUP / 32) {
    // ---------------------------------------------------------- converters
    const uint32_t aoff = geo.aoff_lo[g];
    double2 v[OZ_STEPS];
    i64 t = blockIdx.x;
    if (t < ntiles) {
      const double2* src = psi + tile_base(t, lane, my_rest) + toff;
#pragma unroll
      for (int r = 0; r < OZ_STEPS; ++r) v[r] = src[geo.ghi[r]];
    }
    int it = 0;
    bool pending = false;  // thread 0: MMAs issued whose completion it has not seen
    for (; t < ntiles; t += gridDim.x, ++it) {
      // tile scale: doubles -- the largest biased exponent among the tile's
      // 8192 values; fixed point -- the top bit of the OR of their magnitudes
      uint32_t m = 0, mh = 0;
      if (FIX) {
        uint64_t o = 0;
#pragma unroll
        for (int r = 0; r < OZ_STEPS; ++r) {
          const int64_t a = (int64_t)oz_dbits(v[r].x), b = (int64_t)oz_dbits(v[r].y);
          o |= (uint64_t)(a < 0 ? -a : a) | (uint64_t)(b < 0 ? -b : b);
        }
        m = __reduce_or_sync(0xffffffffu, (uint32_t)o);
        mh = __reduce_or_sync(0xffffffffu, (uint32_t)(o >> 32));
      } else {
#pragma unroll
        for (int r = 0; r < OZ_STEPS; ++r) {
          m = max(m, (uint32_t)(oz_dbits(v[r].x) >> 32) & 0x7FF00000u);
          m = max(m, (uint32_t)(oz_dbits(v[r].y) >> 32) & 0x7FF00000u);
        }
        m = __reduce_max_sync(0xffffffffu, m);
      }
      if (lane == 0) {
        red[warp] = m;
        red_hi[warp] = mh;
      }
      // the A slices are free once the MMAs of the previous tile are done
      if (g == 0) {
        bool bad = abort_flag != 0;
        if (!bad && pending) {
          if (mbar_wait(mfull, (uint32_t)(it - 1) & 1)) pending = false;
          else bad = true;
        }
        if (bad) abort_flag = 1;
        c_stop = bad;
      }
      oz_bar(1);
      if (c_stop) break;
      int scale;  // exm (doubles) or sh (fixed point)
      if (FIX) {
        uint64_t ot = 0;
#pragma unroll
        for (int w = 0; w < OZ_GROUP / 32; ++w) ot |= ((uint64_t)red_hi[w] << 32) | red[w];
        const int p = ot ? 63 - oz_clz64(ot) : -1;
        scale = p > 46 ? p - 46 : 0;
      } else {
        uint32_t mx = red[0];
#pragma unroll
        for (int w = 1; w < OZ_GROUP / 32; ++w) mx = max(mx, red[w]);
        scale = (int)(mx >> 20);
      }
      // digits -> A slices (one (re, im) bf16 pair per slice and amplitude)
#pragma unroll
      for (int r = 0; r < OZ_STEPS; ++r) {
        float dre[OZ_NSLICE], dim[OZ_NSLICE];
        if (FIX) {
          oz_digits_f(oz_fix47_fix((int64_t)oz_dbits(v[r].x), scale), dre);
          oz_digits_f(oz_fix47_fix((int64_t)oz_dbits(v[r].y), scale), dim);
        } else {
          oz_digits_f(oz_fix47(v[r].x, scale), dre);
          oz_digits_f(oz_fix47(v[r].y, scale), dim);
        }
        unsigned char* a = sm + OZ_OFF_A + aoff + geo.aoff_hi[r];
#pragma unroll
        for (int s = 0; s < OZ_NSLICE; ++s) *(uint32_t*)(a + s * OZ_A_SLICE) = oz_pack(dre[s], dim[s]);
      }
      asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
      oz_bar(1);
      // prefetch the next tile into registers (the digits are in shared
      // memory now); issued before the MMAs, whose issue blocks thread 0 and
      // with it the rest of warp 0, so that the loads run under the MMAs
      {
        const i64 tn = t + gridDim.x;
        if (tn < ntiles) {
          const double2* src = psi + tile_base(tn, lane, my_rest) + toff;
#pragma unroll
          for (int r = 0; r < OZ_STEPS; ++r) v[r] = src[geo.ghi[r]];
        }
      }
      if (g == 0) {
        // the MMAs overwrite TMEM: wait until the epilogue has read tile it - 1
        bool ok = it == 0 || mbar_wait(mtfree, (uint32_t)(it - 1) & 1);
        if (ok) {
          tile_scale[it & 1] = scale;
          oz_arrive(mscale);
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll
          for (int s = 0; s < 4; ++s) {  // K-steps of 16
            const uint32_t bs = s_base + OZ_OFF_B + s * 2 * OZ_B_LBO;
            const uint64_t b0 = smem_desc(bs, OZ_B_LBO, OZ_B_SBO);                    // B rows 0..
            const uint64_t b256 = smem_desc(bs + 32 * OZ_B_SBO, OZ_B_LBO, OZ_B_SBO);  // B rows 256..
            const uint64_t b320 = smem_desc(bs + 40 * OZ_B_SBO, OZ_B_LBO, OZ_B_SBO);  // B rows 320..
#pragma unroll
            for (int i = 0; i < OZ_NSLICE; ++i) {
              const uint64_t adesc = smem_desc(s_base + OZ_OFF_A + i * OZ_A_SLICE + s * 2 * a_lbo, a_lbo, OZ_A_SBO);
              const int nrows = 64 * (i <= 1 ? OZ_NSLICE : OZ_NLEVEL - i);  // B slices 0..min(5, 6 - i)
              const uint32_t acc = (i > 0 || s > 0) ? 1u : 0u;
              if (s == 0 && i == 1) {
                // levels 1..5 accumulate onto slice 0's products; level 6 starts here
                oz_mma(tmem + 64, adesc, b0, oz_idesc(256), 1u);
                oz_mma(tmem + 64 + 256, adesc, b256, oz_idesc(64), 1u);
                oz_mma(tmem + 64 + 320, adesc, b320, oz_idesc(64), 0u);
              } else {
                oz_mma(tmem + 64 * i, adesc, b0, oz_idesc(nrows < 256 ? nrows : 256), acc);
                if (nrows > 256) oz_mma(tmem + 64 * i + 256, adesc, b256, oz_idesc(nrows - 256), acc);
              }
            }
          }
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mfull)
                       : "memory");
          pending = true;
        } else {
          abort_flag = 1;
        }
      }
    }
    // on an abort, give the last issued MMAs one more bounded wait so that
    // tensor memory is not freed under them
    if (g == 0 && pending) mbar_wait(mfull, (uint32_t)(it - 1) & 1);
  } else {
    // ------------------------------------------------------------ epilogue
    const int ew = warp - OZ_GROUP / 32;  // TMEM sub-partition ew & 3, column half ew >> 2
    const int erow = 32 * (ew & 3) + lane;
    const int ehalf = ew >> 2;
    const uint32_t trow = tmem + ((uint32_t)(32 * (ew & 3)) << 16);
    const i64 myrow = geo.rowoff[erow];
    int it = 0;
    for (i64 t = blockIdx.x; t < ntiles; t += gridDim.x, ++it) {
      if (g == 0) {
        const uint32_t par = (uint32_t)it & 1;
        const bool bad = abort_flag || !mbar_wait(mscale, par) || !mbar_wait(mfull, par);
        if (bad) abort_flag = 1;
        e_stop = bad;
      }
      oz_bar(2);
      if (e_stop) break;
      const int scale = tile_scale[it & 1];
      double2* dst = psi + tile_base(t, lane, my_rest) + myrow;
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      // combine the seven levels of 8 reals (4 amplitudes) at a time
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        float acc[OZ_NLEVEL][8];
#pragma unroll
        for (int l = 0; l < OZ_NLEVEL; ++l) tmem_ld8(trow + 64 * l + 32 * ehalf + 8 * q, acc[l]);
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
        for (int e = 0; e < 8; e += 2) {
          const int c = 16 * ehalf + 4 * q + (e >> 1);  // output amplitude (permuted block index)
          float are[OZ_NLEVEL], aim[OZ_NLEVEL];
#pragma unroll
          for (int l = 0; l < OZ_NLEVEL; ++l) {
            are[l] = acc[l][e];
            aim[l] = acc[l][e + 1];
          }
          if (FIX) {
            const OzShift k = oz_shift(scale + G.fexp[c] - 1029);
            dst[geo.coloff[c]] = make_double2(oz_bitsd((uint64_t)oz_combine_fix(are, k)),
                                              oz_bitsd((uint64_t)oz_combine_fix(aim, k)));
          } else {
            const int sc = scale + G.fexp[c] - 2098;
            dst[geo.coloff[c]] = make_double2(oz_combine(are, sc), oz_combine(aim, sc));
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
      oz_bar(2);
      if (g == 0) oz_arrive(mtfree);  // TMEM of this tile read: the next MMAs may start
    }
  }
  __syncthreads();
  if (tid == 0 && abort_flag) atomicExch(err, 1);  // a wait gave up: reported by qgb_tc_status
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(OZ_TMEM_COLS));
}

namespace {

// Tile geometry of a block on target bits tbits (matrix order) of an
// n-qubit state (n >= 12).  Column bit cbit[jt] of the permuted block
// belongs to target jt (targets ranked by index position, lowest first).
//
// Banks: a warp writes one 4-byte (re, im) bf16 pair per lane and slice.
// The t5 block qubits on index bits 0..4 (the lanes) take column bits
// 0..t5-1, the other lanes group rows 0..4-t5.  Column bits 0-1 pick the
// word in a 16-byte core-matrix row, row bits 0-2 the 16-byte bank group
// (row groups 144 B = 9 groups apart), column bits 2+ the K chunk; a K-chunk
// stride rotating by rot = 4, 2, 1 bank groups for t5 = 3, 4, 5 then puts the
// 32 lanes on 32 distinct banks (t5 <= 1 leaves fewer distinct words: 2 or 4
// wavefronts).
void make_oz_geom(int n, const std::vector<int>& tbits, OzGeom* geo, int cbit[5]) {
  std::vector<int> sorted_t = tbits;
  std::sort(sorted_t.begin(), sorted_t.end());
  for (int jt = 0; jt < 5; ++jt)
    cbit[jt] = (int)(std::find(sorted_t.begin(), sorted_t.end(), tbits[jt]) - sorted_t.begin());
  std::vector<int> grp;
  for (int b = 0; b < n && (int)grp.size() < 7; ++b)
    if (std::find(tbits.begin(), tbits.end(), b) == tbits.end()) grp.push_back(b);
  std::vector<int> pos = tbits;
  pos.insert(pos.end(), grp.begin(), grp.end());
  std::sort(pos.begin(), pos.end());
  const int nb = (int)pos.size();  // 12
  std::vector<int> rowbit(nb, -1), colbit(nb, -1);
  for (int i = 0; i < nb; ++i) {
    auto g = std::find(grp.begin(), grp.end(), pos[i]);
    if (g != grp.end()) rowbit[i] = (int)(g - grp.begin());
    else colbit[i] = cbit[std::find(tbits.begin(), tbits.end(), pos[i]) - tbits.begin()];
  }
  int t5 = 0;
  for (int b : tbits) t5 += b < 5;
  const uint32_t rot = t5 == 3 ? 4 : t5 == 4 ? 2 : 1;
  geo->a_lbo = OZ_A_LBO0 + 16 * rot;
  auto aoff = [&](uint32_t row, uint32_t c) {
    return (c >> 2) * geo->a_lbo + (row >> 3) * OZ_A_SBO + (row & 7) * 16 + (c & 3) * 4;
  };
  auto split = [&](int bits, int first, int count, i64* dep, uint32_t* row, uint32_t* col) {
    *dep = 0;
    *row = 0;
    *col = 0;
    for (int i = 0; i < count; ++i) {
      const int b = first + i;
      if (b >= nb || !((bits >> i) & 1)) continue;
      *dep |= (i64)1 << pos[b];
      if (rowbit[b] >= 0) *row |= 1u << rowbit[b];
      else *col |= 1u << colbit[b];
    }
  };
  for (int v = 0; v < OZ_GROUP; ++v) {
    i64 dep;
    uint32_t row, col;
    split(v, 0, 8, &dep, &row, &col);
    geo->aoff_lo[v] = aoff(row, col);
  }
  geo->g7 = (i64)1 << pos[7];
  for (int r = 0; r < OZ_STEPS; ++r) {
    i64 dep;
    uint32_t row, col;
    split(r, 8, 4, &dep, &row, &col);
    geo->ghi[r] = dep;
    geo->aoff_hi[r] = aoff(row, col);
  }
  for (int r = 0; r < 128; ++r) {
    geo->rowoff[r] = 0;
    for (int b = 0; b < 7; ++b)
      if ((r >> b) & 1) geo->rowoff[r] |= (i64)1 << grp[b];
  }
  for (int c = 0; c < 32; ++c) {
    geo->coloff[c] = 0;
    for (int jt = 0; jt < 5; ++jt)
      if ((c >> cbit[jt]) & 1) geo->coloff[c] |= (i64)1 << tbits[jt];
  }
  geo->nrest = 0;
  for (int b = 0; b < n; ++b)
    if (std::find(pos.begin(), pos.end(), b) == pos.end()) geo->rest[geo->nrest++] = b;
}

// permuted block U'[r'][c'] = U[idx[r']][idx[c']] (see make_oz_geom) and the
// digit scale of each output row
void make_oz_gate(const GateOp& g, const int cbit[5], OzGate* G) {
  int idx[32];
  for (int c = 0; c < 32; ++c) {
    idx[c] = 0;
    for (int jt = 0; jt < 5; ++jt)
      if ((c >> cbit[jt]) & 1) idx[c] |= 1 << (4 - jt);
  }
  for (int r = 0; r < 32; ++r) {
    double mx = 0;
    for (int c = 0; c < 32; ++c) {
      const zd u = g.coef[idx[r] * 32 + idx[c]];
      G->ur[r][c] = u.real();
      G->ui[r][c] = u.imag();
      mx = std::max(mx, std::max(std::fabs(u.real()), std::fabs(u.imag())));
    }
    G->fexp[r] = (int)((oz_dbits(mx) >> 52) & 0x7FF);
  }
}

}  // namespace

int* qgb_tc_err_flag();  // qgb_tc.cu

// Uncontrolled 5-qubit dense block on a complex128 state of n >= 12 qubits;
// fix: the state is in the fixed-point format (oz_to_fix).
int qgb_launch_fused5_oz(void* state, int n, const GateOp& g, cudaStream_t s, bool fix) {
  if (g.tbits.size() != 5 || !g.cbits.empty() || n < 12) {
    qgb_set_error("qgb_apply_fused5_tc: complex128 needs an uncontrolled 5-qubit dense block on >= 12 qubits");
    return QGB_ERR_INVALID;
  }
  int* err = qgb_tc_err_flag();
  if (!err) return QGB_ERR_CUDA;
  OzGeom* geo = new OzGeom();
  OzGate* G = new OzGate();
  int cbit[5];
  make_oz_geom(n, g.tbits, geo, cbit);
  make_oz_gate(g, cbit, G);
  static bool attr[2] = {false, false};
  if (!attr[fix]) {
    cudaFuncSetAttribute(fix ? k_fused5_oz<true> : k_fused5_oz<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         OZ_SMEM);
    attr[fix] = true;
  }
  const i64 ntiles = (i64)1 << (n - 12);
  const int blocks = (int)std::min<i64>(ntiles, (i64)qgb_num_sms());
  if (fix) k_fused5_oz<true><<<blocks, OZ_THREADS, OZ_SMEM, s>>>((double2*)state, ntiles, *geo, *G, err);
  else k_fused5_oz<false><<<blocks, OZ_THREADS, OZ_SMEM, s>>>((double2*)state, ntiles, *geo, *G, err);
  delete G;
  delete geo;
  QGB_LAUNCH_CHECK("k_fused5_oz");
  return QGB_OK;
}

// ---- fixed-point chains of blocks -----------------------------------------

// e with 2^e > 2 ||psi|| from ||psi||^2 (no square root: ||psi|| < 2^ceil(x/2)
// when ||psi||^2 < 2^x); 0 for the zero state
__host__ __device__ __forceinline__ int oz_scale_exp(double norm2) {
  const int x = (int)((oz_dbits(norm2) >> 52) & 0x7FF) - 1022;  // norm2 < 2^x
  return norm2 > 0 ? ((x + 1) >> 1) + 1 : 0;
}

__global__ void k_oz_scale(const double* __restrict__ norm2, int* __restrict__ e) { *e = oz_scale_exp(*norm2); }

__global__ void k_oz_to_fix(double2* __restrict__ psi, i64 N, const int* __restrict__ e_ptr) {
  const int e = *e_ptr;
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < N; i += (i64)gridDim.x * blockDim.x) {
    const double2 v = psi[i];
    psi[i] = make_double2(oz_bitsd((uint64_t)oz_to_fix(v.x, e)), oz_bitsd((uint64_t)oz_to_fix(v.y, e)));
  }
}

__global__ void k_oz_from_fix(double2* __restrict__ psi, i64 N, const int* __restrict__ e_ptr) {
  const int e = *e_ptr;
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < N; i += (i64)gridDim.x * blockDim.x) {
    const double2 v = psi[i];
    psi[i] = make_double2(oz_from_fix((int64_t)oz_dbits(v.x), e), oz_from_fix((int64_t)oz_dbits(v.y), e));
  }
}

// A block keeps the fixed-point range only if it does not grow the norm:
// max |(U^dagger U - I)_ij| < 1e-9.
bool qgb_oz_unitary(const GateOp& g) {
  for (int i = 0; i < 32; ++i)
    for (int j = 0; j < 32; ++j) {
      zd acc = 0;
      for (int k = 0; k < 32; ++k) acc += std::conj(g.coef[k * 32 + i]) * g.coef[k * 32 + j];
      if (std::abs(acc - zd(i == j ? 1.0 : 0.0, 0.0)) > 1e-9) return false;
    }
  return true;
}

extern "C" int qgb_norm2(const void* state, int nqubits, int dtype, double* out, void* scratch, void* stream);
extern "C" size_t qgb_norm_scratch_bytes(void);

namespace {
// Chain scratch: ||psi||^2, the scale e and the norm reduction.  One set per
// stream, so that chains on different streams (the serving loop's slots) do
// not share it; the set of the default stream (and of any stream first seen
// while it is being captured) is made by qgb_tc_prepare.
struct OzChainScratch {
  double* norm = nullptr;
  int* e = nullptr;
  void* red = nullptr;
};
OzChainScratch g_oz_default;
std::mutex g_oz_mu;
std::unordered_map<cudaStream_t, OzChainScratch> g_oz_streams;

int oz_scratch_alloc(OzChainScratch* c) {
  QGB_TRY_CUDA(cudaMalloc(&c->norm, sizeof(double)));
  QGB_TRY_CUDA(cudaMalloc(&c->e, sizeof(int)));
  QGB_TRY_CUDA(cudaMalloc(&c->red, qgb_norm_scratch_bytes()));
  return QGB_OK;
}
}  // namespace

// Device buffers of the tensor-core paths (error flag, chain scratch),
// allocated once; called by qgb_device_init so that a stream capture of
// qgb_apply_circuit finds them in place.
int qgb_tc_prepare() {
  if (!qgb_tc_err_flag()) return QGB_ERR_CUDA;
  std::lock_guard<std::mutex> lk(g_oz_mu);
  if (!g_oz_default.norm) return oz_scratch_alloc(&g_oz_default);
  return QGB_OK;
}

// Chain scratch of stream s, allocated on its first use outside a capture
// (qgb_stream_create calls this so that the serving loop never allocates).
int qgb_oz_stream_scratch(cudaStream_t s, OzChainScratch** out) {
  int st = qgb_tc_prepare();
  if (st) return st;
  std::lock_guard<std::mutex> lk(g_oz_mu);
  *out = &g_oz_default;
  if (s == nullptr || s == cudaStreamLegacy || s == cudaStreamPerThread) return QGB_OK;
  auto it = g_oz_streams.find(s);
  if (it != g_oz_streams.end()) {
    *out = &it->second;
    return QGB_OK;
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  QGB_TRY_CUDA(cudaStreamIsCapturing(s, &cap));
  if (cap != cudaStreamCaptureStatusNone) return QGB_OK;
  OzChainScratch c;
  st = oz_scratch_alloc(&c);
  if (st) return st;
  *out = &(g_oz_streams[s] = c);
  return QGB_OK;
}

int qgb_oz_stream_prepare(cudaStream_t s) {
  OzChainScratch* c;
  return qgb_oz_stream_scratch(s, &c);
}

// Frees the chain scratch of a stream about to be destroyed (after the
// stream's work is done).
int qgb_oz_stream_release(cudaStream_t s) {
  std::lock_guard<std::mutex> lk(g_oz_mu);
  auto it = g_oz_streams.find(s);
  if (it == g_oz_streams.end()) return QGB_OK;
  QGB_TRY_CUDA(cudaStreamSynchronize(s));
  cudaFree(it->second.norm);
  cudaFree(it->second.e);
  cudaFree(it->second.red);
  g_oz_streams.erase(it);
  return QGB_OK;
}

// Consecutive unitary blocks on a complex128 state (n >= 12): the state is
// converted once to the fixed-point format (scale from its FP64 norm, all on
// the device), every block runs on it, and it is converted back.  Two extra
// state passes replace the double <-> digit conversions of every block.
int qgb_run_oz_chain(void* state, int n, const std::vector<const GateOp*>& blocks, cudaStream_t s) {
  OzChainScratch* cs;
  int st = qgb_oz_stream_scratch(s, &cs);
  if (st) return st;
  st = qgb_norm2(state, n, QGB_C128, cs->norm, cs->red, (void*)s);
  if (st) return st;
  k_oz_scale<<<1, 1, 0, s>>>(cs->norm, cs->e);
  QGB_LAUNCH_CHECK("k_oz_scale");
  const i64 N = (i64)1 << n;
  const int grid = (int)std::min<i64>((N + 255) / 256, (i64)qgb_num_sms() * 8);
  k_oz_to_fix<<<grid, 256, 0, s>>>((double2*)state, N, cs->e);
  QGB_LAUNCH_CHECK("k_oz_to_fix");
  for (const GateOp* g : blocks) {
    st = qgb_launch_fused5_oz(state, n, *g, s, true);
    if (st) return st;
  }
  k_oz_from_fix<<<grid, 256, 0, s>>>((double2*)state, N, cs->e);
  QGB_LAUNCH_CHECK("k_oz_from_fix");
  return QGB_OK;
}
