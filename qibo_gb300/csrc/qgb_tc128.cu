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
//    47-bit fixed point against a shared scale (IEEE doubles: the largest
//    exponent of the tile; the fixed-point chain format: one shift for the
//    whole launch, from the OR of the state's magnitudes; gate rows: their
//    largest entry, or the block's in the chain format) and split into six
//    balanced base-256 digits d in [-128, 128] (exact as bf16);
//  * A_i * B_j^T over K = 64 then sums products of at most 2^14, so every
//    level l = i + j <= 6 accumulates exactly in its own FP32 accumulator
//    (|sum| <= 7 * 2^20 < 2^24);
//  * the seven level accumulators are combined with integer arithmetic into
//    sum_{l<=5} acc_l 256^(5-l) + round(acc_6 / 256) and rounded once to an
//    IEEE double (the chain format keeps the lowest three levels to within
//    645 units of that sum, see oz_combine_fix).
//  With 2^E, 2^F the A and B scales (2^E <= 2 x the largest |value|
//  sharing it), the fixed-point rounding of both operands over K = 64 and
//  the dropped levels (l >= 7) bound the error of an output by
//  2^(E + F - 41); independent roundings give about 2^(E + F - 46).
//  Normalised states and unitary blocks have 2^(E + F) <= 4, and far less
//  for spread-out states.  The CPU replay tests/native/oz_check.cu checks
//  the bound output by output.
//
// Tensor memory holds the level accumulators of the two output halves
// (realified output rows 0-31 and 32-63) in two rings of seven levels:
// level l of half h at columns 256 h + 32 l .. + 31 (224 columns per half).
// The six B slices are stacked per half along N (row 192 h + 32 j + n'), so
// the MMA for A slice i with B slices 0..min(5, 6-i) written at TMEM column
// 256 h + 32 i lands each product A_i B_j in level i + j: one instruction
// per slice and K-step of 16 (N = 32 x slices <= 192; the first write of
// level 6 is its own instruction so that it starts the accumulation), 25
// per half and tile.
//
// A CTA (576 threads, one per SM: 224 KB of shared memory, 448 TMEM
// columns) owns 4096-amplitude tiles with the index geometry of qgb_tc.cu,
// in four roles that run as a pipeline:
//  * warp 17 copies the raw tiles into shared memory with the bulk-copy
//    engine, one tile ahead (32 runs of 128 contiguous amplitudes, a run per
//    lane), so the loads stay in flight without holding registers and the
//    converters never stop to issue them;
//  * warps 0-7 convert (thread t moves amplitudes t + 256 r, r < 16).  A
//    thread reads its amplitudes,
//    forms their digit words, frees the raw buffer for the next copy, and
//    writes digit slice s of A as soon as the previous tile's MMAs on slice
//    s are done;
//  * warp 16 (one thread) issues the MMAs: half 0 of tile i slice by slice
//    as the slices are written (once the epilogue has read half 0 of tile
//    i - 1), then half 1, committing "slice s free" after each of its
//    slices;
//  * warps 8-15 read each half's levels from TMEM (lane quarter = warp mod
//    4, 16 of the half's 32 output reals per warp), combine and store;
//    half 0 overlaps the MMAs of half 1, half 1 those of the next tile's
//    half 0.
// The digits are bytes: with Z = X + 0x8080808080 (X the 47-bit value),
// byte k of Z minus 128 is the digit of weight 256^k (k < 5) and Z >> 40
// the top one; a byte permutation puts each byte under the exponent of 2^23
// and one FP32 subtraction makes it an exact float.  The level combination
// is an integer multiply-add chain.  Every wait on an mbarrier is bounded
// and also ends when another role has recorded an abort; the MMA thread
// then waits once more (bounded) for its in-flight MMAs, the copy warp for
// an in-flight copy, and tensor memory is freed.
//
// Runs of blocks (qgb_run_oz_chain; non-unitary ones with headroom for
// their norm growth, qgb_oz_growth_bits) keep the state in a 64-bit
// fixed-point format between blocks (k_fused5_oz<true, *>), converted from and
// back to IEEE doubles once per run.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "qgb_plan.h"
#include "qgb_tcgen05.cuh"

#define OZ_CONV_WARPS 8                        // converter warps 0-7
#define OZ_EPI_WARPS 8                         // epilogue warps 8-15 (lane quarter = warp mod 4)
#define OZ_MMA_WARP (OZ_CONV_WARPS + OZ_EPI_WARPS)  // warp 16: MMA issue
#define OZ_COPY_WARP (OZ_MMA_WARP + 1)         // warp 17: bulk copies of the raw tiles
#define OZ_THREADS ((OZ_COPY_WARP + 1) * 32)   // 576
#define OZ_GROUP (OZ_CONV_WARPS * 32)          // converter threads
#define OZ_EPI (OZ_EPI_WARPS * 32)             // epilogue threads
#define OZ_STEPS 16     // amplitudes per converter thread per tile
#define OZ_TILE 4096    // amplitudes per tile
#define OZ_NSLICE 6     // digits per value
#define OZ_NLEVEL 7     // digit-product levels kept (i + j <= 6)
#define OZ_TMEM_COLS 512
#define OZ_HALF_COLS 256  // TMEM column of output half 1
#define OZ_C5 0x8080808080ull  // 128 in each of the five low digit bytes
// A slices: 128 rows x 64 bf16, K-major no-swizzle core matrices (8 rows x
// 16 B); row groups 144 B apart, K chunks a_lbo = 2304 + 16 rot apart.
#define OZ_A_SBO 144
#define OZ_A_LBO0 2304
#define OZ_A_SLICE (8 * (OZ_A_LBO0 + 64))  // 18944
// B: 384 rows ([half][slice][32 rows]) x 64 bf16, dense core matrices
#define OZ_B_ROWS (OZ_NSLICE * 64)
#define OZ_B_SBO 128
#define OZ_B_LBO (OZ_B_ROWS / 8 * OZ_B_SBO)  // 6144
// Raw tile: the 32 runs of 128 contiguous amplitudes of the next tile (2 KB
// each), copied in by the bulk-copy engine: run 2 r + (g >> 7) holds the
// amplitudes of converter thread g's step r.
#define OZ_RUN 2048
#define OZ_RAW_BYTES (32 * OZ_RUN)  // 65536
#define OZ_OFF_A 0
#define OZ_OFF_B (OZ_OFF_A + OZ_NSLICE * OZ_A_SLICE)  // 113664
#define OZ_OFF_RAW (OZ_OFF_B + 8 * OZ_B_LBO)          // 162816
#define OZ_SMEM (OZ_OFF_RAW + OZ_RAW_BYTES)           // 228352

static_assert(OZ_OFF_B % 16 == 0 && OZ_OFF_RAW % 128 == 0, "operand regions aligned");
static_assert(OZ_SMEM + 1024 <= 232448, "one CTA per SM");
static_assert(OZ_GROUP * OZ_STEPS == OZ_TILE, "one amplitude per converter thread and step");

// shared-memory offset of A slice s
__host__ __device__ __forceinline__ uint32_t oz_slot(int s) { return (uint32_t)(s * OZ_A_SLICE); }

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
  int pair;  // outputs 2 m and 2 m + 1 of a row are adjacent amplitudes at an even index
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

// exact float of an integer |c| < 2^22
__host__ __device__ __forceinline__ float oz_i2f(int32_t c) {
#ifdef __CUDA_ARCH__
  return __int_as_float(0x4B400000 + c) - 12582912.0f;
#else
  return (float)c;
#endif
}

// byte k (0..3) of w minus 128, as an exact float: the byte is placed under
// the exponent of 2^23 by one byte permutation and 2^23 + 128 subtracted
__host__ __device__ __forceinline__ float oz_bytef(uint32_t w, int k) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u | (uint32_t)k)) - 8388736.0f;
#else
  return (float)(int)((w >> (8 * k)) & 0xFFu) - 128.0f;
#endif
}

// Balanced base-256 digits of a 47-bit fixed-point value X (|X| <= 2^47),
// as exact floats, from Z = X + OZ_C5:
//   X = sum_{i<6} d[i] 256^(5-i),  d[0] = Z >> 40 in [-128, 128],
//   d[i] = byte 5 - i of Z minus 128 in [-128, 127] (i >= 1),
// since the five low bytes of OZ_C5 are 128 each.  The top digit: Z lies in
// [-2^47, 2^47 + 2^40), so Z >> 40 lies in [-128, 128].
__host__ __device__ __forceinline__ void oz_zdigits_top(uint64_t Z, float d[3]) {
  const uint32_t hi = (uint32_t)(Z >> 32);
  d[0] = oz_i2f((int32_t)hi >> 8);
  d[1] = oz_bytef(hi, 0);
  d[2] = oz_bytef((uint32_t)Z, 3);
}
// digits 3..5 from the low word of Z
__host__ __device__ __forceinline__ void oz_zdigits_low(uint32_t zlo, float d[3]) {
  d[0] = oz_bytef(zlo, 2);
  d[1] = oz_bytef(zlo, 1);
  d[2] = oz_bytef(zlo, 0);
}
__host__ __device__ __forceinline__ void oz_zdigits(uint64_t Z, float d[OZ_NSLICE]) {
  oz_zdigits_top(Z, d);
  oz_zdigits_low((uint32_t)Z, d + 3);
}

// digit s of Z alone (oz_zdigits)
__host__ __device__ __forceinline__ float oz_zdigit(uint64_t Z, int s) {
  const uint32_t hi = (uint32_t)(Z >> 32), lo = (uint32_t)Z;
  return s == 0 ? oz_i2f((int32_t)hi >> 8) : s == 1 ? oz_bytef(hi, 0) : oz_bytef(lo, 5 - s);
}

// the digits of oz_fix47(x, exm) as integers (host checks and the B slices)
__host__ __device__ __forceinline__ void oz_digits(double x, int exm, int d[OZ_NSLICE]) {
  float f[OZ_NSLICE];
  oz_zdigits((uint64_t)oz_fix47(x, exm) + OZ_C5, f);
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

// Shift amounts of round(T 2^k) without branches (one set per tile: the
// fixed-point kernel uses one gate-wide scale F): lsh = max(k, 0),
// rsh = min(max(-k, 0), 62) (a shift by 62 already rounds every |T| < 2^61
// to 0), rnd = 2^rsh / 2.
struct OzShift {
  int lsh, rsh;
  int64_t rnd;
};
__host__ __device__ __forceinline__ OzShift oz_shift(int k) {
  OzShift r;
  r.lsh = k > 0 ? k : 0;
  r.rsh = k < 0 ? (k > -62 ? -k : 62) : 0;
  r.rnd = ((int64_t)1 << r.rsh) >> 1;
  return r;
}

// round(T' * 2^k) as a 64-bit integer (fixed-point output; |result| < 2^62),
// where T' = H 2^32 + M 2^16 + Q 2^10 differs from T by the rounding of the
// three low levels only:
//   H = acc0 256 + acc1, M = acc2 256 + acc3 (exact: |acc_l| <= 2^22, each
//   read as an integer by one magic-constant addition; both fit in 31 bits),
//   Q = round(acc4 / 4 + (acc5 + acc6 / 256) / 1024) in FP32 (two FMA
//   roundings below 2^-3 and one to an integer: |Q 2^10 - exact| < 580).
// With the levels dropped (i + j >= 7: below 65) T' is within 645 of the
// exact product sum in units of T, far inside the digit rounding's 2^13.
__host__ __device__ __forceinline__ int64_t oz_combine_fix(const float acc[OZ_NLEVEL], const OzShift& sh) {
  const float C = 12582912.0f;
  const uint32_t K = 0x4B400000u;
  const uint32_t b0 = oz_fbits(acc[0] + C), b1 = oz_fbits(acc[1] + C);
  const uint32_t b2 = oz_fbits(acc[2] + C), b3 = oz_fbits(acc[3] + C);
  const int32_t H = (int32_t)(b0 * 256u + b1 - 257u * K);
  const int32_t M = (int32_t)(b2 * 256u + b3 - 257u * K);
  const float s = fmaf(acc[6], 0.00390625f, acc[5]);
  const int32_t Q = (int32_t)(oz_fbits(fmaf(acc[4], 0.25f, s * 0.0009765625f) + C) - K);
  const int64_t T = (int64_t)((uint64_t)(uint32_t)H << 32) + (int64_t)M * 65536 + (int64_t)Q * 1024;
  return ((int64_t)((uint64_t)T << sh.lsh) + sh.rnd) >> sh.rsh;
}

// Fixed-point state format between consecutive tensor-core blocks: a real
// x is held as the integer X = round(x 2^(62 - e)), e a state-wide scale with
// 2^e > 2 ||psi|| (so |X| < 2^61, and unitary blocks keep it there; a chain
// of blocks that can grow the norm by g bits in all starts g bits higher).
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

// Z of the digits (oz_zdigits) of a fixed-point X at tile shift sh (the
// tile's largest |X| is below 2^(47 + sh)): round(X / 2^sh), half up, plus
// OZ_C5, as (X + bias) >> sh with bias = oz_fix_bias(sh)
__host__ __device__ __forceinline__ int64_t oz_fix_bias(int sh) {
  return (int64_t)((((uint64_t)1 << sh) >> 1) + (OZ_C5 << sh));
}
__host__ __device__ __forceinline__ uint64_t oz_fix_z(int64_t X, int sh, int64_t bias) {
  return (uint64_t)((X + bias) >> sh);
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

// Bounded wait on an mbarrier phase that also gives up once another role
// has recorded an abort (checked every 64 polls).
__device__ __forceinline__ bool oz_wait(uint32_t mbar, uint32_t phase, const volatile int* abort_flag) {
  for (uint32_t it = 0; it < TC_SPIN_LIMIT; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(mbar), "r"(phase)
        : "memory");
    if (done) return true;
    if ((it & 63u) == 63u && *abort_flag) return false;
  }
  return false;
}

__device__ __forceinline__ void oz_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar) : "memory");
}

// One 2 KB run of the tile into shared memory by the bulk-copy engine,
// completing its bytes on mbarrier mbar (the caller set the expected count).
__device__ __forceinline__ void oz_copy_run(uint32_t dst, const void* src, uint32_t mbar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
               "l"(src), "r"((uint32_t)OZ_RUN), "r"(mbar)
               : "memory");
}

// The MMAs of A slices s0..s1-1 for output half h: B slices
// 0..min(5, 6 - s) of the half land in levels s.. at TMEM column 256 h + 32 s.
__device__ __forceinline__ void oz_issue(uint32_t s_base, uint32_t tmem, uint32_t a_lbo, int h, int s0, int s1) {
#pragma unroll 1
  for (int s = s0; s < s1; ++s) {
    const int cnt = s <= 1 ? OZ_NSLICE : OZ_NLEVEL - s;  // B slices used with A slice s
    const uint32_t a0 = s_base + OZ_OFF_A + oz_slot(s);
    const uint32_t d = tmem + OZ_HALF_COLS * h + 32 * s;
#pragma unroll
    for (int k = 0; k < 4; ++k) {  // K-steps of 16
      const uint64_t adesc = smem_desc(a0 + k * 2 * a_lbo, a_lbo, OZ_A_SBO);
      const uint32_t bs = s_base + OZ_OFF_B + k * 2 * OZ_B_LBO + 24 * h * OZ_B_SBO;  // B row 192 h
      const uint64_t bdesc = smem_desc(bs, OZ_B_LBO, OZ_B_SBO);
      if (k == 0 && s == 1) {
        // levels 1..5 accumulate onto slice 0's products; level 6 starts here
        oz_mma(d, adesc, bdesc, oz_idesc(160), 1u);
        oz_mma(d + 160, adesc, smem_desc(bs + 20 * OZ_B_SBO, OZ_B_LBO, OZ_B_SBO), oz_idesc(32), 0u);
      } else {
        oz_mma(d, adesc, bdesc, oz_idesc(32 * cnt), (s > 0 || k > 0) ? 1u : 0u);
      }
    }
  }
}

// The epilogue's stores skip L1 allocation (.L1::no_allocate): with the
// block on the lowest index bits a warp's 32 lanes write 32 lines 512 bytes
// apart, and the hint took such blocks from 7.65 to 7.26 ms at n=30 (other
// placements unchanged; an evict-first .cs store changed nothing).
__device__ __forceinline__ void oz_st16(double2* p, double2 a) {
  asm volatile("st.global.L1::no_allocate.v2.f64 [%0], {%1, %2};\n" ::"l"(p), "d"(a.x), "d"(a.y) : "memory");
}
// two adjacent amplitudes in one 32-byte store (p 32-byte aligned)
__device__ __forceinline__ void oz_st32(double2* p, double2 a, double2 b) {
  asm volatile("st.global.L1::no_allocate.v4.f64 [%0], {%1, %2, %3, %4};\n" ::"l"(p), "d"(a.x), "d"(a.y),
               "d"(b.x), "d"(b.y)
               : "memory");
}

// The epilogue's work on output half H of a tile for a warp of column
// group CG (reals 16 CG .. 16 CG + 15 of the half, i.e. outputs
// c = 16 H + 8 CG .. + 7): the seven levels of 8 reals (4 outputs) at a
// time from TMEM, combined and stored straight to the state; orm collects
// the OR of the fixed-point outputs' |high words|.  The loop over the two
// groups of 8 reals stays rolled: unrolled, the four instances of this
// function made the kernel's code large enough that its warps stalled on
// instruction fetch (n=30 chain block 9.2 ms unrolled, 7.3 ms rolled).
template <bool FIX, bool PAIR, int H, int CG>
__device__ __forceinline__ void oz_epi_half(double2* dst, uint32_t trow, const OzGeom& geo, const OzGate& G,
                                            const OzShift& fsh, int scale, uint32_t& orm) {
  const uint32_t th = trow + OZ_HALF_COLS * H;
#pragma unroll 1
  for (int q = 0; q < 2; ++q) {
    const int c4 = 2 * CG + q;
    float acc[OZ_NLEVEL][8];
#pragma unroll
    for (int l = 0; l < OZ_NLEVEL; ++l) tmem_ld8(th + 32 * l + 8 * c4, acc[l]);
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int ep = 0; ep < 8; ep += 4) {
      const int c = 16 * H + 4 * c4 + (ep >> 1);  // outputs c, c + 1 (permuted block index)
      double2 out[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int e = ep + 2 * h;
        float are[OZ_NLEVEL], aim[OZ_NLEVEL];
#pragma unroll
        for (int l = 0; l < OZ_NLEVEL; ++l) {
          are[l] = acc[l][e];
          aim[l] = acc[l][e + 1];
        }
        if (FIX) {
          const int64_t xr = oz_combine_fix(are, fsh), xi = oz_combine_fix(aim, fsh);
          orm |= (uint32_t)abs((int32_t)((uint64_t)xr >> 32)) | (uint32_t)abs((int32_t)((uint64_t)xi >> 32));
          out[h] = make_double2(oz_bitsd((uint64_t)xr), oz_bitsd((uint64_t)xi));
        } else {
          const int sc = scale + G.fexp[c + h] - 2098;
          out[h] = make_double2(oz_combine(are, sc), oz_combine(aim, sc));
        }
      }
      if (PAIR) {
        oz_st32(dst + geo.coloff[c], out[0], out[1]);
      } else {
        oz_st16(dst + geo.coloff[c], out[0]);
        oz_st16(dst + geo.coloff[c + 1], out[1]);
      }
    }
  }
}

// FIX: the state holds fixed-point integers (oz_to_fix) instead of IEEE
// doubles; the launch's scale is then one shift for all tiles, and each
// output a rounding shift.  PAIR (blocks on index bit 0, geo.pair): a lane's
// outputs c and c + 1 are adjacent amplitudes and go out as one 32-byte
// store, so a warp's stores stay whole sectors (lanes are 64 bytes or more
// apart on such blocks); a separate instance, because a runtime choice
// between the two store forms cost the other placements 2-3 %.
//
// Handoffs (each mbarrier phase completes once per tile, or once per two
// tiles for m_scale[b]; no waiter can fall two phases behind, because every
// completion of a phase needs the waiter's previous phase to have been
// consumed upstream):
//   m_raw    bulk copies -> converters    the raw tile is in shared memory
//   m_rawfree  converter -> copy warp     the raw tile has been read
//   m_ready[s]  converters -> MMA  (one arrival per converter warp)
//            A slice s of tile i written
//   m_free[s]   tcgen05.commit -> converter   the MMAs of tile i that read
//            slice s are done (the last ones, of half 1)
//   m_scale[i & 1]  converter -> epilogue  (doubles) scale of tile i in tile_scale[i & 1]
//   m_full[h]  tcgen05.commit -> epilogue   MMAs of half h of tile i done
//   m_tfree[h] epilogue (256 arrivals) -> MMA   half h of tile i read
template <bool FIX, bool PAIR>
__global__ void __maxnreg__(96)  // 18 warps: five share one SMSP's 16 K registers
    k_fused5_oz(double2* __restrict__ psi, i64 ntiles, const __grid_constant__ OzGeom geo,
                const __grid_constant__ OzGate G, int* __restrict__ err, const uint32_t* __restrict__ fix_in,
                uint32_t* __restrict__ fix_out, uint32_t* __restrict__ fix_zero) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) uint64_t m_raw, m_rawfree, m_ready[OZ_NSLICE], m_free[OZ_NSLICE], m_scale[2], m_full[2],
      m_tfree[2], m_drain;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;  // set by any role on a failed wait
  __shared__ int c_stop[2];   // the converters' decisions, written by their thread 0 before their barriers
  __shared__ uint32_t red[OZ_CONV_WARPS];
  __shared__ int tile_scale[2];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t s_base = smem_u32(sm);
  volatile int* abort_v = &abort_flag;

  // B slices: row 192 h + 32 j + n' holds digit j of realified output row
  // n = 32 h + n' (n = 2 r + re/im of output r), column k = 2 c + re/im of
  // input c
  for (int e = tid; e < 64 * 64; e += OZ_THREADS) {
    const int n = e >> 6, k = e & 63, r = n >> 1, c = k >> 1;
    double v;
    if ((n & 1) == 0) v = (k & 1) == 0 ? G.ur[r][c] : -G.ui[r][c];
    else v = (k & 1) == 0 ? G.ui[r][c] : G.ur[r][c];
    int d[OZ_NSLICE];
    oz_digits(v, G.fexp[r], d);
    const int hb = 192 * (n >> 5) + (n & 31);
#pragma unroll
    for (int j = 0; j < OZ_NSLICE; ++j)
      *(uint16_t*)(sm + OZ_OFF_B + oz_boff(hb + 32 * j, k)) = (uint16_t)oz_bf16(d[j]);
  }
  if (tid == 0) {
    abort_flag = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&m_raw)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&m_rawfree)));
    for (int k = 0; k < OZ_NSLICE; ++k) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(&m_ready[k])), "r"(OZ_CONV_WARPS));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&m_free[k])));
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&m_drain)));
    for (int h = 0; h < 2; ++h) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&m_scale[h])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&m_full[h])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(&m_tfree[h])), "r"(OZ_EPI));
    }
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_base)),
                 "r"(OZ_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // B slices -> tensor-core reads
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_base;
  const uint32_t a_lbo = geo.a_lbo;
  const int my_rest = lane < geo.nrest ? geo.rest[lane] : -1;
  // fixed point: the launch's shift from the OR of the state's |high words|
  // (largest |X| < 2^(33 + ph) <= 2^(47 + sh)); this launch ORs its outputs
  // into fix_out and clears fix_zero, the word the next launch ORs into
  int fix_sh = 0;
  if (FIX) {
    const uint32_t m = *fix_in;
    const int ph = m ? 31 - __clz((int)m) : -1;
    fix_sh = ph > 14 ? ph - 14 : 0;
    if (blockIdx.x == 0 && tid == 0) *fix_zero = 0;
  }

  if (warp < OZ_CONV_WARPS) {
    // ---------------------------------------------------------- converters
    // The raw tile arrives in shared memory by bulk copies issued one tile
    // ahead (the copy warp, one 2 KB run per lane), so the loads of the next
    // tile are in flight while this one converts, with no registers held.  A
    // thread reads its 16 amplitudes, turns them into their digit words Z
    // (oz_zdigits) in registers and frees the raw tile for the next copy;
    // then it writes digit slice s as soon as the previous tile's MMAs that
    // read slice s are done, so the slices follow the MMAs one by one.
    const int g = tid;  // 0..255
    const uint32_t aoff = geo.aoff_lo[g];
    const uint32_t mraw = smem_u32(&m_raw);
    i64 t = blockIdx.x;
    for (int it = 0; t < ntiles; t += gridDim.x, ++it) {
      // this tile's raw values -> registers
      const bool got = oz_wait(mraw, (uint32_t)it & 1, abort_v);
      uint64_t zr[OZ_STEPS], zi[OZ_STEPS];
#pragma unroll
      for (int r = 0; r < OZ_STEPS; ++r) {
        const double2 v = *(const double2*)(sm + OZ_OFF_RAW + (2 * r + (g >> 7)) * OZ_RUN + (g & 127) * 16);
        zr[r] = oz_dbits(v.x);
        zi[r] = oz_dbits(v.y);
      }
      if (!got) *abort_v = 1;
      int scale = 0;  // exm (doubles): the largest biased exponent of the tile
      if (!FIX) {
        uint32_t m = 0;
#pragma unroll
        for (int r = 0; r < OZ_STEPS; ++r) {
          m = max(m, (uint32_t)(zr[r] >> 32) & 0x7FF00000u);
          m = max(m, (uint32_t)(zi[r] >> 32) & 0x7FF00000u);
        }
        m = __reduce_max_sync(0xffffffffu, m);
        if (lane == 0) red[warp] = m;
      }
      if (g == 0) c_stop[0] = *abort_v;
      // generic reads of the raw tile before the copy engine rewrites it
      asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
      oz_bar(1);
      if (c_stop[0]) break;
      if (g == 0) oz_arrive(smem_u32(&m_rawfree));  // raw tile read: the next copy may land
      if (FIX) {
        const int64_t bias = oz_fix_bias(fix_sh);
#pragma unroll
        for (int r = 0; r < OZ_STEPS; ++r) {
          zr[r] = oz_fix_z((int64_t)zr[r], fix_sh, bias);
          zi[r] = oz_fix_z((int64_t)zi[r], fix_sh, bias);
        }
      } else {
        uint32_t mx = red[0];
#pragma unroll
        for (int w = 1; w < OZ_CONV_WARPS; ++w) mx = max(mx, red[w]);
        scale = (int)(mx >> 20);
#pragma unroll
        for (int r = 0; r < OZ_STEPS; ++r) {
          zr[r] = (uint64_t)oz_fix47(oz_bitsd(zr[r]), scale) + OZ_C5;
          zi[r] = (uint64_t)oz_fix47(oz_bitsd(zi[r]), scale) + OZ_C5;
        }
      }
      // slice by slice, each once the previous tile's MMAs on it are done
      bool ok = true;
#pragma unroll
      for (int s = 0; s < OZ_NSLICE; ++s) {
        ok = ok && (it == 0 || oz_wait(smem_u32(&m_free[s]), (uint32_t)(it - 1) & 1, abort_v));
        if (ok) {
#pragma unroll
          for (int r = 0; r < OZ_STEPS; ++r)
            *(uint32_t*)(sm + OZ_OFF_A + oz_slot(s) + aoff + geo.aoff_hi[r]) =
                oz_pack(oz_zdigit(zr[r], s), oz_zdigit(zi[r], s));
          asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        } else {
          *abort_v = 1;
        }
        // one arrival per warp once its lanes have written slice s (a
        // barrier of all converter threads per slice was 2-5 % slower)
        __syncwarp();
        if (lane == 0 && ok) oz_arrive(smem_u32(&m_ready[s]));
      }
      if (!FIX && g == 0 && ok) {
        tile_scale[it & 1] = scale;  // read by the epilogue of tile it - 2 long ago
        oz_arrive(smem_u32(&m_scale[it & 1]));
      }
      if (g == 0) c_stop[1] = *abort_v;
      oz_bar(1);
      if (c_stop[1]) break;
    }
  } else if (warp == OZ_COPY_WARP) {
    // ------------------------------------------------------------- copies
    // tile it's 32 runs of 128 amplitudes, one bulk copy per lane (run
    // 2 r + hi for lane 2 r + hi), once the converters have read tile it - 1
    const uint32_t mraw = smem_u32(&m_raw), mrawfree = smem_u32(&m_rawfree);
    const uint32_t raw = s_base + OZ_OFF_RAW;
    const i64 run_off = ((lane & 1) ? geo.g7 : 0) + geo.ghi[lane >> 1];
    int copies = 0;
    for (i64 t = blockIdx.x; t < ntiles; t += gridDim.x) {
      if (copies > 0 && !__all_sync(0xffffffffu, oz_wait(mrawfree, (uint32_t)(copies - 1) & 1, abort_v))) break;
      const i64 tb = tile_base(t, lane, my_rest);
      if (lane == 0)
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mraw), "r"((uint32_t)OZ_RAW_BYTES)
                     : "memory");
      __syncwarp();
      oz_copy_run(raw + lane * OZ_RUN, psi + tb + run_off, mraw);
      ++copies;
    }
    // after an abort the last copy may still be writing the raw tile: wait
    // for it (bounded) before the CTA's shared memory is released
    if (lane == 0 && copies > 0) mbar_wait(mraw, (uint32_t)(copies - 1) & 1);
  } else if (warp < OZ_MMA_WARP) {
    // ------------------------------------------------------------ epilogue
    const int q = warp & 3;                     // TMEM lane quarter (warp mod 4)
    const int cg = (warp - OZ_CONV_WARPS) >> 2;  // reals 16 cg .. 16 cg + 15 of each half
    const int erow = 32 * q + lane;
    const uint32_t trow = tmem + ((uint32_t)(32 * q) << 16);
    const i64 myrow = geo.rowoff[erow];
    const OzShift fsh = oz_shift(fix_sh + G.fexp[0] - 1029);  // fixed point: one shift per launch
    uint32_t orm = 0;  // fixed point: OR of the outputs' |high word| (the next launch's shift)
    int it = 0;
    bool failed = false;
    for (i64 t = blockIdx.x; t < ntiles; t += gridDim.x, ++it) {
      int scale = 0;
      if (!FIX) {
        if (!__all_sync(0xffffffffu, oz_wait(smem_u32(&m_scale[it & 1]), (uint32_t)(it >> 1) & 1, abort_v))) {
          failed = true;
          break;
        }
        scale = tile_scale[it & 1];
      }
      double2* dst = psi + tile_base(t, lane, my_rest) + myrow;
      if (!__all_sync(0xffffffffu, oz_wait(smem_u32(&m_full[0]), (uint32_t)it & 1, abort_v))) {
        failed = true;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      if (cg == 0) oz_epi_half<FIX, PAIR, 0, 0>(dst, trow, geo, G, fsh, scale, orm);
      else oz_epi_half<FIX, PAIR, 0, 1>(dst, trow, geo, G, fsh, scale, orm);
      asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
      oz_arrive(smem_u32(&m_tfree[0]));  // half 0 read: the next tile's MMAs may write it
      if (!__all_sync(0xffffffffu, oz_wait(smem_u32(&m_full[1]), (uint32_t)it & 1, abort_v))) {
        failed = true;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      if (cg == 0) oz_epi_half<FIX, PAIR, 1, 0>(dst, trow, geo, G, fsh, scale, orm);
      else oz_epi_half<FIX, PAIR, 1, 1>(dst, trow, geo, G, fsh, scale, orm);
      asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
      oz_arrive(smem_u32(&m_tfree[1]));
    }
    if (failed) *abort_v = 1;
    if (FIX) {
      orm = __reduce_or_sync(0xffffffffu, orm);
      if (lane == 0 && orm) atomicOr(fix_out, orm);
    }
  } else if (lane == 0) {
    // ---------------------------------------------------------------- MMAs
    bool issued = false, ok = true;
    int it = 0;
    for (i64 t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++it) {
      const uint32_t par = (uint32_t)it & 1, prev = (uint32_t)(it - 1) & 1;
      ok = it == 0 || oz_wait(smem_u32(&m_tfree[0]), prev, abort_v);
      for (int s = 0; s < OZ_NSLICE && ok; ++s) {
        ok = oz_wait(smem_u32(&m_ready[s]), par, abort_v);
        if (!ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        oz_issue(s_base, tmem, a_lbo, 0, s, s + 1);
        issued = true;
      }
      if (!ok) break;
      oz_commit(smem_u32(&m_full[0]));
      ok = it == 0 || oz_wait(smem_u32(&m_tfree[1]), prev, abort_v);
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      for (int s = 0; s < OZ_NSLICE; ++s) {
        oz_issue(s_base, tmem, a_lbo, 1, s, s + 1);
        oz_commit(smem_u32(&m_free[s]));  // slice s may be rewritten once these are done
      }
      oz_commit(smem_u32(&m_full[1]));
    }
    if (!ok) *abort_v = 1;
    // every issued MMA completes before tensor memory is freed (bounded)
    if (issued) {
      oz_commit(smem_u32(&m_drain));
      mbar_wait(smem_u32(&m_drain), 0);
    }
  }
  __syncthreads();
  if (tid == 0 && abort_flag) *(volatile int*)err = 1;  // a wait gave up: reported by qgb_tc_status
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
  // a block on index bit 0 puts output pairs next to each other: the
  // epilogue then stores 32 bytes per pair
  geo->pair = 1;
  for (int c = 0; c < 32; c += 2)
    if (geo->coloff[c + 1] != geo->coloff[c] + 1 || (geo->coloff[c] & 1)) geo->pair = 0;
  for (int r = 0; r < 128; ++r)
    if (geo->rowoff[r] & 1) geo->pair = 0;
  for (int j = 0; j < geo->nrest; ++j)
    if (geo->rest[j] == 0) geo->pair = 0;
}

// permuted block U'[r'][c'] = U[idx[r']][idx[c']] (see make_oz_geom) and the
// digit scale of each output row; uniform: every row takes the scale of the
// largest entry of the block (the fixed-point kernel's epilogue then shifts
// every output of a tile alike)
void make_oz_gate(const GateOp& g, const int cbit[5], OzGate* G, bool uniform) {
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
  if (uniform) {
    const int fm = *std::max_element(G->fexp, G->fexp + 32);
    for (int r = 0; r < 32; ++r) G->fexp[r] = fm;
  }
}

}  // namespace

int* qgb_tc_err_flag();  // qgb_tc.cu

// Uncontrolled 5-qubit dense block on a complex128 state of n >= 12 qubits;
// fix: the state is in the fixed-point format (oz_to_fix), and fix_words
// holds the three words of the launch shifts of a chain: the launch reads
// word b % 3 (the OR of the state's |high words|), ORs its outputs into
// word (b + 1) % 3 and clears word (b + 2) % 3 for the launch after.
int qgb_launch_fused5_oz(void* state, int n, const GateOp& g, cudaStream_t s, bool fix, uint32_t* fix_words,
                         int b) {
  if (fix && !fix_words) {
    qgb_set_error("qgb_launch_fused5_oz: the fixed-point format needs the chain's shift words");
    return QGB_ERR_INVALID;
  }
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
  if ((uintptr_t)state % 32 != 0) geo->pair = 0;  // 32-byte stores need a 32-byte aligned state
  make_oz_gate(g, cbit, G, fix);
  const bool pair = geo->pair != 0;
  const void* kfn = fix ? (pair ? (const void*)k_fused5_oz<true, true> : (const void*)k_fused5_oz<true, false>)
                        : (pair ? (const void*)k_fused5_oz<false, true> : (const void*)k_fused5_oz<false, false>);
  const int sa = qgb_func_smem(kfn, OZ_SMEM);
  if (sa) {
    delete G;
    delete geo;
    return sa;
  }
  const i64 ntiles = (i64)1 << (n - 12);
  const int blocks = (int)std::min<i64>(ntiles, (i64)qgb_num_sms());
  uint32_t* const f0 = fix ? fix_words + b % 3 : nullptr;
  uint32_t* const f1 = fix ? fix_words + (b + 1) % 3 : nullptr;
  uint32_t* const f2 = fix ? fix_words + (b + 2) % 3 : nullptr;
  if (fix && pair)
    k_fused5_oz<true, true><<<blocks, OZ_THREADS, OZ_SMEM, s>>>((double2*)state, ntiles, *geo, *G, err, f0, f1, f2);
  else if (fix)
    k_fused5_oz<true, false><<<blocks, OZ_THREADS, OZ_SMEM, s>>>((double2*)state, ntiles, *geo, *G, err, f0, f1, f2);
  else if (pair)
    k_fused5_oz<false, true><<<blocks, OZ_THREADS, OZ_SMEM, s>>>((double2*)state, ntiles, *geo, *G, err, f0, f1, f2);
  else
    k_fused5_oz<false, false><<<blocks, OZ_THREADS, OZ_SMEM, s>>>((double2*)state, ntiles, *geo, *G, err, f0, f1, f2);
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

// the scale e (plus the chain's headroom bits: the blocks may grow the
// norm by that many), and the chain's first two shift words cleared
__global__ void k_oz_scale(const double* __restrict__ norm2, int* __restrict__ e, uint32_t* __restrict__ fixw,
                           int headroom) {
  *e = oz_scale_exp(*norm2) + headroom;
  fixw[0] = 0;
  fixw[1] = 0;
}

// doubles -> fixed point; fixw[0] collects the OR of the values' |high
// words| (the first block's shift)
__global__ void k_oz_to_fix(double2* __restrict__ psi, i64 N, const int* __restrict__ e_ptr,
                            uint32_t* __restrict__ fixw) {
  const int e = *e_ptr;
  uint32_t m = 0;
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < N; i += (i64)gridDim.x * blockDim.x) {
    const double2 v = psi[i];
    const int64_t xr = oz_to_fix(v.x, e), xi = oz_to_fix(v.y, e);
    m |= (uint32_t)abs((int32_t)((uint64_t)xr >> 32)) | (uint32_t)abs((int32_t)((uint64_t)xi >> 32));
    psi[i] = make_double2(oz_bitsd((uint64_t)xr), oz_bitsd((uint64_t)xi));
  }
  m = __reduce_or_sync(0xffffffffu, m);
  if ((threadIdx.x & 31) == 0 && m) atomicOr(fixw, m);
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

// Bits by which a block can grow the 2-norm of a state: 0 for a unitary
// block, else ceil(log2 s) for a rigorous bound s on its largest singular
// value: s^2 = lambda_max(M), M = B^H B, is at most ||M^8||_inf^(1/8)
// (the largest absolute row sum of a matrix power bounds its spectral
// radius), tight for near-unitary and contractive blocks.
int qgb_oz_growth_bits(const GateOp& g) {
  if (qgb_oz_unitary(g)) return 0;
  std::vector<zd> M(1024, zd(0, 0)), T(1024);
  for (int i = 0; i < 32; ++i)
    for (int j = 0; j < 32; ++j) {
      zd acc = 0;
      for (int k = 0; k < 32; ++k) acc += std::conj(g.coef[k * 32 + i]) * g.coef[k * 32 + j];
      M[i * 32 + j] = acc;
    }
  for (int sq = 0; sq < 3; ++sq) {  // M <- M^2, three times: M^8
    for (int i = 0; i < 32; ++i)
      for (int j = 0; j < 32; ++j) {
        zd acc = 0;
        for (int k = 0; k < 32; ++k) acc += M[i * 32 + k] * M[k * 32 + j];
        T[i * 32 + j] = acc;
      }
    M.swap(T);
  }
  double row = 0;
  for (int i = 0; i < 32; ++i) {
    double r = 0;
    for (int j = 0; j < 32; ++j) r += std::abs(M[i * 32 + j]);
    row = std::max(row, r);
  }
  if (!(row > 0)) return 0;              // the zero block
  if (!std::isfinite(row)) return 1 << 20;  // too large to bound: never chained
  // s = row^(1/16); bits = ceil(log2 s), with a margin for the rounding of the bound
  const double bits = std::log2(row) / 16.0 + 1e-9;
  return bits <= 0 ? 0 : (int)std::ceil(bits);
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
  uint32_t* fixw = nullptr;  // the three shift words of the fixed-point launches
};
OzChainScratch g_oz_default;
std::mutex g_oz_mu;
std::unordered_map<cudaStream_t, OzChainScratch> g_oz_streams;

int oz_scratch_alloc(OzChainScratch* c) {
  QGB_TRY_CUDA(cudaMalloc(&c->norm, sizeof(double)));
  QGB_TRY_CUDA(cudaMalloc(&c->e, sizeof(int)));
  QGB_TRY_CUDA(cudaMalloc(&c->red, qgb_norm_scratch_bytes()));
  QGB_TRY_CUDA(cudaMalloc(&c->fixw, 3 * sizeof(uint32_t)));
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
// (qgb_stream_create calls this so that the serving loop never allocates);
// a stream seen for the first time while it is being captured is refused.
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
  if (cap != cudaStreamCaptureStatusNone) {
    // sharing the default set would let two graphs replayed at once on
    // different streams race on the chain's scale
    qgb_set_error(
        "complex128 block chains on a stream under capture need the stream's own scratch: create the stream with "
        "qgb_stream_create, or run one complex128 circuit on it before capturing");
    return QGB_ERR_INVALID;
  }
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
  cudaFree(it->second.fixw);
  g_oz_streams.erase(it);
  return QGB_OK;
}

// Consecutive blocks on a complex128 state (n >= 12): the state is
// converted once to the fixed-point format (scale from its FP64 norm, all on
// the device), every block runs on it, and it is converted back.  Two extra
// state passes replace the double <-> digit conversions of every block.
// ``headroom``: the blocks' growth bits together (qgb_oz_growth_bits; 0 for
// unitary blocks), added to the scale so that |X| < 2^61 holds throughout.
int qgb_run_oz_chain(void* state, int n, const std::vector<const GateOp*>& blocks, cudaStream_t s, int headroom) {
  OzChainScratch* cs;
  int st = qgb_oz_stream_scratch(s, &cs);
  if (st) return st;
  st = qgb_norm2(state, n, QGB_C128, cs->norm, cs->red, (void*)s);
  if (st) return st;
  k_oz_scale<<<1, 1, 0, s>>>(cs->norm, cs->e, cs->fixw, headroom);
  QGB_LAUNCH_CHECK("k_oz_scale");
  const i64 N = (i64)1 << n;
  const int grid = (int)std::min<i64>((N + 255) / 256, (i64)qgb_num_sms() * 8);
  k_oz_to_fix<<<grid, 256, 0, s>>>((double2*)state, N, cs->e, cs->fixw);
  QGB_LAUNCH_CHECK("k_oz_to_fix");
  for (size_t b = 0; b < blocks.size(); ++b) {
    st = qgb_launch_fused5_oz(state, n, *blocks[b], s, true, cs->fixw, (int)(b % 3));
    if (st) return st;
  }
  k_oz_from_fix<<<grid, 256, 0, s>>>((double2*)state, N, cs->e);
  QGB_LAUNCH_CHECK("k_oz_from_fix");
  return QGB_OK;
}
