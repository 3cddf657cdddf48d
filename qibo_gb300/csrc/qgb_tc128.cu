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
// A CTA (256 threads, one per SM: 223 KB of shared memory, 384 TMEM columns)
// owns 4096-amplitude tiles with the index geometry of qgb_tc.cu; the next
// tile is prefetched into registers while the MMAs run.  The wait on the
// mbarrier is bounded: on timeout the kernel records an error flag, waits
// once more (bounded) for the in-flight MMAs, frees its tensor memory and
// returns.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "qgb_plan.h"
#include "qgb_tcgen05.cuh"

#define OZ_THREADS 256
#define OZ_STEPS 16    // amplitudes per thread per tile
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
#define OZ_OFF_STAGE (OZ_OFF_B + 8 * OZ_B_LBO)        // 162816
#define OZ_SMEM (OZ_OFF_STAGE + OZ_TILE * 16)         // 228352

static_assert(OZ_OFF_B % 16 == 0 && OZ_OFF_STAGE % 16 == 0, "operand regions 16-byte aligned");
static_assert(OZ_SMEM <= 227 * 1024, "one CTA per SM");
static_assert(OZ_THREADS * OZ_STEPS == OZ_TILE, "one amplitude per thread and step");

// Tile geometry (same tile / thread mapping as the complex64 kernel): tile
// index j = t + 256 r has global offset base + (t & 127) + (t >> 7) g7 +
// ghi[r]; its (re, im) bf16 pair sits at byte aoff_lo[t] + aoff_hi[r] of
// every A slice; staging slot of (row, column c) is
//   (c << 7 | row) ^ ((c << g3) & 7),   g3 = 3 - (block qubits on bits 0..2),
// written as row ^ scol[c] and read as sread_lo[t] ^ sread_hi[r].
struct OzGeom {
  int nrest;
  int rest[32];
  uint32_t a_lbo;
  i64 g7;
  i64 ghi[OZ_STEPS];
  uint32_t aoff_lo[OZ_THREADS];
  uint32_t aoff_hi[OZ_STEPS];
  uint16_t sread_lo[OZ_THREADS];
  uint16_t sread_hi[OZ_STEPS];
  uint16_t scol[32];
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

// Balanced base-256 digits of x in 47-bit fixed point against exponent exm
// (the biased exponent of the largest |value| sharing the scale):
//   x ~= 2^(exm - 1069) * sum_{i<6} d[i] 256^(5-i),   |d[i]| <= 128,
// rounding error <= 2^(exm - 1070); values below 2^-58 of the scale and
// subnormals become 0.
__host__ __device__ __forceinline__ void oz_digits(double x, int exm, int d[OZ_NSLICE]) {
  const uint64_t u = oz_dbits(x);
  const int ex = (int)((u >> 52) & 0x7FF);
  const int rs = 6 + exm - ex;
  int64_t X = 0;
  if (ex != 0 && rs < 60) {
    const uint64_t M = (u & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    X = (int64_t)((M + (1ull << (rs - 1))) >> rs);
    if (u >> 63) X = -X;
  }
  // bottom-up: d = sign-extended low byte, X <- (X - d) / 256 (exact)
#pragma unroll
  for (int i = OZ_NSLICE - 1; i >= 1; --i) {
    const int di = (int)(int8_t)(uint8_t)(X & 0xFF);
    d[i] = di;
    X = (X - di) >> 8;
  }
  d[0] = (int)X;
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

// integer value of an integer-valued float: exact for |v| <= 2^22; for
// 2^22 < |v| < 2^24 rounded to a multiple of 4 (wide = true)
__host__ __device__ __forceinline__ int oz_f2i(float v, bool wide) {
#ifdef __CUDA_ARCH__
  return wide ? (__float_as_int(v + 50331648.0f) - 0x4C400000) * 4 : __float_as_int(v + 12582912.0f) - 0x4B400000;
#else
  return wide ? 4 * (int)std::nearbyint((double)v / 4.0) : (int)v;  // ties to even, as the FADD
#endif
}

__host__ __device__ __forceinline__ int oz_clz64(uint64_t a) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)a);
#else
  return __builtin_clzll(a);
#endif
}

// (sum_{l<=5} acc[l] 256^(5-l) + round(acc[6] / 256)) * 2^sc as an IEEE
// double (one rounding, to nearest even); acc[l] are the level accumulators
// (integers in floats)
__host__ __device__ __forceinline__ double oz_combine(const float acc[OZ_NLEVEL], int sc) {
  int64_t T = ((int64_t)oz_f2i(acc[6], true) + 128) >> 8;
#pragma unroll
  for (int l = 0; l < OZ_NSLICE; ++l) T += (int64_t)oz_f2i(acc[l], l >= 4) * ((int64_t)1 << (8 * (OZ_NSLICE - 1 - l)));
  if (T == 0) return 0.0;
  const uint64_t s = T < 0 ? (1ull << 63) : 0;
  const uint64_t a = T < 0 ? (uint64_t)(-T) : (uint64_t)T;
  const int p = 63 - oz_clz64(a);  // top bit
  const int be = p + sc + 1023;    // biased exponent of the result
  if (be <= 0) return oz_bitsd(s);  // below the normal range: 0
  uint64_t mant;
  if (p > 52) {
    const int r = p - 52;
    mant = a >> r;
    const uint64_t rem = a & ((1ull << r) - 1), half = 1ull << (r - 1);
    if (rem > half || (rem == half && (mant & 1))) mant += 1;
  } else {
    mant = a << (52 - p);
  }
  return oz_bitsd(s | (((uint64_t)(be - 1) << 52) + mant));
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

__global__ void __launch_bounds__(OZ_THREADS, 1)
    k_fused5_oz(double2* __restrict__ psi, i64 ntiles, const __grid_constant__ OzGeom geo,
                const __grid_constant__ OzGate G, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  __shared__ uint32_t red[OZ_THREADS / 32];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t s_base = smem_u32(sm);
  const uint32_t mb = smem_u32(&mbar);

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
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mb));
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
  uint32_t phase = 0;
  const uint32_t aoff = geo.aoff_lo[tid];
  const uint32_t srd = geo.sread_lo[tid];
  const uint32_t a_lbo = geo.a_lbo;
  const int my_rest = lane < geo.nrest ? geo.rest[lane] : -1;
  const i64 toff = (i64)(tid & 127) + ((tid >> 7) ? geo.g7 : 0);
  double2* stage = (double2*)(sm + OZ_OFF_STAGE);
  // epilogue: this warp's TMEM sub-partition (group rows) and column half
  const int erow = 32 * (warp & 3) + lane;
  const int ehalf = warp >> 2;
  const uint32_t trow = tmem + ((uint32_t)(32 * (warp & 3)) << 16);

  double2 v[OZ_STEPS];
  i64 t = blockIdx.x;
  i64 base = 0;
  if (t < ntiles) {
    base = tile_base(t, lane, my_rest);
    const double2* src = psi + base + toff;
#pragma unroll
    for (int r = 0; r < OZ_STEPS; ++r) v[r] = src[geo.ghi[r]];
  }
  for (; t < ntiles; t += gridDim.x) {
    // tile scale: the largest biased exponent among the tile's 8192 values
    uint32_t m = 0;
#pragma unroll
    for (int r = 0; r < OZ_STEPS; ++r) {
      m = max(m, (uint32_t)(oz_dbits(v[r].x) >> 32) & 0x7FF00000u);
      m = max(m, (uint32_t)(oz_dbits(v[r].y) >> 32) & 0x7FF00000u);
    }
    m = __reduce_max_sync(0xffffffffu, m);
    if (lane == 0) red[warp] = m;
    __syncthreads();
    uint32_t mx = red[0];
#pragma unroll
    for (int w = 1; w < OZ_THREADS / 32; ++w) mx = max(mx, red[w]);
    const int exm = (int)(mx >> 20);
    // digits -> A slices (one (re, im) bf16 pair per slice and amplitude)
#pragma unroll
    for (int r = 0; r < OZ_STEPS; ++r) {
      int dre[OZ_NSLICE], dim[OZ_NSLICE];
      oz_digits(v[r].x, exm, dre);
      oz_digits(v[r].y, exm, dim);
      unsigned char* a = sm + OZ_OFF_A + aoff + geo.aoff_hi[r];
#pragma unroll
      for (int s = 0; s < OZ_NSLICE; ++s) *(uint32_t*)(a + s * OZ_A_SLICE) = oz_bf16(dre[s]) | (oz_bf16(dim[s]) << 16);
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (tid == 0) {
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
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mb)
                   : "memory");
    }
    // prefetch the next tile into registers while the MMAs run
    const i64 tn = t + gridDim.x;
    i64 nbase = 0;
    if (tn < ntiles) {
      nbase = tile_base(tn, lane, my_rest);
      const double2* src = psi + nbase + toff;
#pragma unroll
      for (int r = 0; r < OZ_STEPS; ++r) v[r] = src[geo.ghi[r]];
    }
    // one thread waits for the MMAs; the rest park at the barrier
    if (tid == 0 && !mbar_wait(mb, phase)) abort_flag = 1;
    __syncthreads();
    if (abort_flag) {
      // record the failure, give the in-flight MMAs one more bounded wait so
      // tensor memory is not freed under them, then leave
      if (tid == 0) {
        atomicExch(err, 1);
        mbar_wait(mb, phase);
      }
      break;
    }
    phase ^= 1;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    // epilogue: combine the six levels of 8 reals at a time into doubles
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      float acc[OZ_NLEVEL][8];
#pragma unroll
      for (int l = 0; l < OZ_NLEVEL; ++l) tmem_ld8(trow + 64 * l + 32 * ehalf + 8 * q, acc[l]);
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
      for (int e = 0; e < 8; e += 2) {
        const int c = 16 * ehalf + 4 * q + (e >> 1);  // output amplitude (permuted block index)
        const int sc = exm + G.fexp[c] - 2098;
        float are[OZ_NLEVEL], aim[OZ_NLEVEL];
#pragma unroll
        for (int l = 0; l < OZ_NLEVEL; ++l) {
          are[l] = acc[l][e];
          aim[l] = acc[l][e + 1];
        }
        stage[erow ^ geo.scol[c]] = make_double2(oz_combine(are, sc), oz_combine(aim, sc));
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    double2* dst = psi + base + toff;
#pragma unroll
    for (int r = 0; r < OZ_STEPS; ++r) dst[geo.ghi[r]] = stage[srd ^ geo.sread_hi[r]];
    base = nbase;
  }
  __syncthreads();
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
// wavefronts).  The staging slots keep every quarter-warp of 16-byte
// accesses on 8 distinct bank groups, for the row-wise writes and for the
// tile-order reads.
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
  int t5 = 0, t3 = 0;
  for (int b : tbits) {
    t5 += b < 5;
    t3 += b < 3;
  }
  const uint32_t rot = t5 == 3 ? 4 : t5 == 4 ? 2 : 1;
  geo->a_lbo = OZ_A_LBO0 + 16 * rot;
  const int g3 = 3 - t3;
  auto scol = [&](uint32_t c) { return (uint32_t)((c << 7) ^ ((c << g3) & 7u)); };
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
  for (int v = 0; v < OZ_THREADS; ++v) {
    i64 dep;
    uint32_t row, col;
    split(v, 0, 8, &dep, &row, &col);
    geo->aoff_lo[v] = aoff(row, col);
    geo->sread_lo[v] = (uint16_t)(row ^ scol(col));
  }
  geo->g7 = (i64)1 << pos[7];
  for (int r = 0; r < OZ_STEPS; ++r) {
    i64 dep;
    uint32_t row, col;
    split(r, 8, 4, &dep, &row, &col);
    geo->ghi[r] = dep;
    geo->aoff_hi[r] = aoff(row, col);
    geo->sread_hi[r] = (uint16_t)(row ^ scol(col));
  }
  for (int c = 0; c < 32; ++c) geo->scol[c] = (uint16_t)scol((uint32_t)c);
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

// Uncontrolled 5-qubit dense block on a complex128 state of n >= 12 qubits.
int qgb_launch_fused5_oz(void* state, int n, const GateOp& g, cudaStream_t s) {
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
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_fused5_oz, cudaFuncAttributeMaxDynamicSharedMemorySize, OZ_SMEM);
    attr = true;
  }
  const i64 ntiles = (i64)1 << (n - 12);
  const int blocks = (int)std::min<i64>(ntiles, (i64)qgb_num_sms());
  k_fused5_oz<<<blocks, OZ_THREADS, OZ_SMEM, s>>>((double2*)state, ntiles, *geo, *G, err);
  delete G;
  delete geo;
  QGB_LAUNCH_CHECK("k_fused5_oz");
  return QGB_OK;
}
