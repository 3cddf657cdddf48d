// Fused 5-qubit blocks on the tensor cores (complex64, 3xTF32).
//
// A fused block (gates/special.py:28-153, matrix from Backend.matrix_fused,
// backends/abstract.py:2680-2717) is a dense 32x32 complex unitary U applied
// to every group of 32 amplitudes that differ only in the block's qubits.
// With amplitudes stored as interleaved (re, im) floats, U acts on a group as
// the 64x64 real matrix B with 2x2 blocks [[Ur, -Ui], [Ui, Ur]], so 128
// groups at a time form a GEMM  D[128 x 64] = A[128 x 64] * B^T.
//
// A CTA (256 threads, two per SM) owns a tile of 4096 amplitudes: the 5
// block bits plus the 7 lowest other index bits.  Tile index j has its 7 low
// bits equal to global index bits 0..6 (those bits are always in the tile),
// so thread t loads amplitudes j = t + 256 r, r = 0..15: every warp load is
// 256 contiguous bytes.  Each value is split into a TF32 head and a
// remainder (x = hi + lo) and written to A_hi / A_lo in shared memory in the
// K-major no-swizzle core-matrix layout (row = group, column = block index).
// One thread issues
//   D = A_hi*B_hi + A_hi*B_lo + A_lo*B_hi     (3xTF32, FP32 accumulation)
// as 24 tcgen05.mma.kind::tf32 instructions (M=128, N=64, K=8) into tensor
// memory, commits them to an mbarrier and waits on it; all threads have
// issued the loads of the next tile into registers just before, and the
// others park at the CTA barrier.
// Warps w and w+4 then read TMEM lanes 32(w%4).. (the groups) in two column
// halves with tcgen05.ld, stage the outputs in shared memory in tile order,
// and the CTA stores the tile back with the coalesced pattern of the load.
//
// Bank conflicts.  Core matrices are padded (row-group stride 144 B, K-chunk
// stride 2304 + 16*rot B) so that both strides rotate the 16-byte bank
// group; the block matrix is permuted (U -> P U P^T) so that the block
// qubits on the lowest index bits take the lowest column bits; and the
// staging buffer is XOR-swizzled in its low 4 index bits.  Every half-warp
// access then covers 16 distinct 8-byte slots (one wavefront), except the
// A write of a block with no qubit on index bits 0..3 (two).
//
// On full tiles most placements run k_fused5_tcm instead (below): A goes to
// tensor memory from registers, with no shared-memory staging, which takes
// a block from 0.69-0.74 to 0.79-0.96 of HBM bandwidth.
//
// The wait on the mbarrier is bounded: on timeout the kernel records an
// error flag, waits once more (bounded) for the in-flight MMAs, frees its
// tensor memory and returns.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "qgb_plan.h"
#include "qgb_tcgen05.cuh"

#define TC_M 128
#define TC_N 64
#define TC_K 64
#define TC_THREADS 256
#define TC_STEPS 16   // amplitudes per thread per tile
#define TC_TILE 4096  // amplitudes per tile (128 groups x 32)
// K-major, no swizzle: 8-row x 16-byte core matrices; core matrices adjacent
// along K are LBO bytes apart, along M/N SBO bytes apart.  A is padded by 16
// bytes per row group and by 16*rot bytes per K chunk, rot in {1, 2, 4}
// chosen per block (bank rotation); B is written once per CTA and stays
// dense.
#define TC_A_SBO 144
#define TC_A_LBO0 (TC_M / 8 * TC_A_SBO)  // 2304 = 0 mod 128
#define TC_A_LBO_MAX (TC_A_LBO0 + 64)
#define TC_B_SBO 128
#define TC_B_LBO (TC_N / 8 * TC_B_SBO)  // 1024
// shared memory layout (bytes)
#define TC_A_BYTES (TC_K / 4 * TC_A_LBO_MAX)  // 37888
#define TC_B_BYTES (TC_K / 4 * TC_B_LBO)      // 16384
#define TC_OFF_AHI 0
#define TC_OFF_ALO (TC_OFF_AHI + TC_A_BYTES)
#define TC_OFF_BHI (TC_OFF_ALO + TC_A_BYTES)
#define TC_OFF_BLO (TC_OFF_BHI + TC_B_BYTES)
#define TC_SMEM (TC_OFF_BLO + TC_B_BYTES)  // 108 544

static_assert(TC_TILE * 8 <= TC_A_BYTES, "staging buffer must fit in A_hi");
static_assert(TC_A_BYTES % 16 == 0 && TC_B_BYTES % 16 == 0, "operand regions 16-byte aligned");
static_assert(TC_THREADS * TC_STEPS == TC_TILE, "one amplitude per thread and step");
static_assert(QGB_MAXQ - 12 <= 32, "rest bits are spread over one warp's lanes");

struct TcGate {
  float ur[32][32];
  float ui[32][32];
};

// Tile geometry.  Tile index j = t + 256 r (thread t, step r); its global
// offset is base(tile) + (t & 127) + (t >> 7) * g7 + ghi[r] (tile bits 0..6
// are index bits 0..6; g7 is the offset of tile bit 7).  Shared-memory byte
// offset of j in A is aoff_lo[t] + aoff_hi[r] (the core-matrix offset is
// additive over disjoint row / column bits).  Staging slot of (group row,
// block column c) is
//   (c << 7 | row) ^ ((c << g) & 15),   g = 4 - (block qubits on bits 0..3),
// a bijection on [0, 4096) that is linear over disjoint bits: the epilogue
// writes row ^ scol[c], the store reads sread_lo[t] ^ sread_hi[r].
struct TcGeom {
  int nbits;         // bits in a tile (12, fewer for small states)
  int nrest;         // remaining index bits (at most 28)
  int rest[32];      // their global positions, ascending
  uint32_t a_lbo;    // K-chunk stride of A: TC_A_LBO0 + 16 * rot
  i64 g7;            // global offset of tile bit 7
  i64 ghi[TC_STEPS]; // global offsets of tile bits 8..11
  uint32_t aoff_lo[TC_THREADS];
  uint32_t aoff_hi[TC_STEPS];
  uint16_t sread_lo[TC_THREADS];
  uint16_t sread_hi[TC_STEPS];
  uint16_t scol[32];
};

__host__ __device__ __forceinline__ uint32_t core_off(uint32_t row, uint32_t k, uint32_t lbo, uint32_t sbo) {
  // byte offset of element (row, k) in a K-major no-swizzle operand
  return (k >> 2) * lbo + (row >> 3) * sbo + (row & 7) * 16 + (k & 3) * 4;
}

// kind::tf32 instruction descriptor: D f32, A/B tf32, both K-major, N, M
__host__ __device__ constexpr uint32_t tc_idesc(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ float tf32_head(float x) { return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u); }

// FULL: 4096-amplitude tiles (states of 12 qubits or more), no predicates.
template <bool FULL>
__global__ void __launch_bounds__(TC_THREADS, 2)
    k_fused5_tc(float2* __restrict__ psi, i64 ntiles, const __grid_constant__ TcGeom geo,
                const __grid_constant__ TcGate G, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t s_base = smem_u32(sm);
  const uint32_t mb = smem_u32(&mbar);

  // B = realified (permuted) U, split into TF32 head and remainder; row n =
  // output real, column k = input real
  for (int e = tid; e < TC_N * TC_K; e += TC_THREADS) {
    const int n = e / TC_K, k = e % TC_K;
    const int r = n >> 1, c = k >> 1;
    float v;
    if ((n & 1) == 0) v = (k & 1) == 0 ? G.ur[r][c] : -G.ui[r][c];
    else v = (k & 1) == 0 ? G.ui[r][c] : G.ur[r][c];
    const float h = tf32_head(v);
    const uint32_t o = core_off(n, k, TC_B_LBO, TC_B_SBO);
    *(float*)(sm + TC_OFF_BHI + o) = h;
    *(float*)(sm + TC_OFF_BLO + o) = v - h;
  }
  if (tid == 0) {
    abort_flag = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mb));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_base)),
                 "r"(TC_N));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_base;
  constexpr uint32_t IDESC = tc_idesc(TC_M, TC_N);
  uint32_t phase = 0;
  const int TN = FULL ? TC_TILE : (1 << geo.nbits);
  const int nr = FULL ? TC_STEPS : (TN >= TC_THREADS ? TN / TC_THREADS : 1);  // steps per thread
  const bool tval = FULL || tid < TN;                                        // this thread has elements
  const int nrows = TN >> 5;
  const uint32_t aoff = geo.aoff_lo[tid];
  const uint32_t srd = geo.sread_lo[tid];
  const uint32_t a_lbo = geo.a_lbo;
  const int my_rest = lane < geo.nrest ? geo.rest[lane] : -1;
  const i64 toff = (i64)(tid & 127) + ((tid >> 7) ? geo.g7 : 0);
  float2* stage = (float2*)(sm + TC_OFF_AHI);
  // epilogue: this warp's TMEM sub-partition (group rows) and column half
  const int erow = 32 * (warp & 3) + lane;
  const int ehalf = warp >> 2;

  float2 v[TC_STEPS];
  i64 t = blockIdx.x;
  i64 base = 0;
  if (t < ntiles) {
    base = tile_base(t, lane, my_rest);
    const float2* src = psi + base + toff;
#pragma unroll
    for (int r = 0; r < TC_STEPS; ++r)
      if (FULL || (tval && r < nr)) v[r] = src[geo.ghi[r]];
  }
  for (; t < ntiles; t += gridDim.x) {
    // registers -> A_hi / A_lo (row = group, columns 2c, 2c+1 = re, im of element c)
#pragma unroll
    for (int r = 0; r < TC_STEPS; ++r) {
      if (FULL || (tval && r < nr)) {
        const float2 x = v[r];
        const float2 h = make_float2(tf32_head(x.x), tf32_head(x.y));
        const uint32_t o = aoff + geo.aoff_hi[r];
        *(float2*)(sm + TC_OFF_AHI + o) = h;
        *(float2*)(sm + TC_OFF_ALO + o) = make_float2(x.x - h.x, x.y - h.y);
      }
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    // prefetch the next tile into registers while the MMAs run; issued
    // before the MMAs, whose issue blocks thread 0 and with it warp 0
    const i64 tn = t + gridDim.x;
    i64 nbase = 0;
    if (tn < ntiles) {
      nbase = tile_base(tn, lane, my_rest);
      const float2* src = psi + nbase + toff;
#pragma unroll
      for (int r = 0; r < TC_STEPS; ++r)
        if (FULL || (tval && r < nr)) v[r] = src[geo.ghi[r]];
    }
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      uint32_t acc = 0;
#pragma unroll
      for (int s = 0; s < TC_K / 8; ++s) {
        const uint64_t ahi = smem_desc(s_base + TC_OFF_AHI + s * 2 * a_lbo, a_lbo, TC_A_SBO);
        const uint64_t alo = smem_desc(s_base + TC_OFF_ALO + s * 2 * a_lbo, a_lbo, TC_A_SBO);
        const uint64_t bhi = smem_desc(s_base + TC_OFF_BHI + s * 2 * TC_B_LBO, TC_B_LBO, TC_B_SBO);
        const uint64_t blo = smem_desc(s_base + TC_OFF_BLO + s * 2 * TC_B_LBO, TC_B_LBO, TC_B_SBO);
        const uint64_t as[3] = {ahi, ahi, alo};
        const uint64_t bs[3] = {bhi, blo, bhi};
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          asm volatile(
              "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
              " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
              "l"(as[q]), "l"(bs[q]), "r"(IDESC), "r"(acc));
          acc = 1;
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mb)
                   : "memory");
    }
    // one thread waits for the MMAs; the rest park at the barrier
    if (tid == 0 && !mbar_wait(mb, phase)) abort_flag = 1;
    __syncthreads();
    if (abort_flag) {
      // record the failure, give the in-flight MMAs one more bounded wait so
      // tensor memory is not freed under them, then leave
      if (tid == 0) {
        *(volatile int*)err = 1;
        mbar_wait(mb, phase);
      }
      break;
    }
    phase ^= 1;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    float y[32];
    const uint32_t ta = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + 32 * ehalf;
    tmem_ld16(ta, y);
    tmem_ld16(ta + 16, y + 16);
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
    if (FULL || erow < nrows) {
#pragma unroll
      for (int c = 0; c < 16; ++c) stage[erow ^ geo.scol[16 * ehalf + c]] = make_float2(y[2 * c], y[2 * c + 1]);
    }
    __syncthreads();
    float2* dst = psi + base + toff;
#pragma unroll
    for (int r = 0; r < TC_STEPS; ++r)
      if (FULL || (tval && r < nr)) dst[geo.ghi[r]] = stage[srd ^ geo.sread_hi[r]];
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    base = nbase;
  }
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TC_N));
}

// The same product with A in tensor memory (states of 12 qubits or more,
// placements tcm_plan selects).  After the load, thread l of warp w holds
// group row 32 (w % 4) + l.  Two lane layouts get it there: strided lanes
// (the lanes are group rows; a warp access spans 2^(1 + b) lines, b = block
// qubits on index bits 0..3, and L1/L2 merge the sectors of a row's
// columns), or coalesced lanes (every warp access is one or two 128-byte
// lines, and up to four warp-shuffle exchanges of lane and register bits
// move rows onto lanes).  Each thread loads
// the 16 amplitudes of its row in one column half straight into registers,
// splits them and writes A_hi / A_lo to its own tensor-memory lane with
// tcgen05.st; the MMAs read A from tensor memory and only B from shared
// memory; the epilogue reads D back with tcgen05.ld and stores to the
// addresses it loaded from.  That removes the A writes, A operand reads and
// the staging buffer from shared memory, whose bandwidth bounds the kernel
// above.  Tensor memory per CTA: D in columns 0..63, A_hi 64..127, A_lo
// 128..191 (256 allocated, two CTAs per SM).
#define TCM_COLS 256
#define TCM_SMEM (2 * TC_B_BYTES)

// Tile geometry: a tile is the 5 block bits plus the 7 lowest other index
// bits.  Thread (warp w, lane l) loads and stores amplitude r at
// base(tile) + lanes[l] + rowhi[w % 4] + h * chi + clo[r], h = w / 4.
// With nswap = 0 (strided lanes) lanes[] are the group-row bits and clo[]
// the block columns, so thread l holds group row 32 (w % 4) + l, columns
// 16 h + r.  With nswap = k > 0 (coalesced lanes) lane bits 0..k-1 address
// block bits and register bits 0..k-1 group-row bits; exchanging lane bit i
// with register bit i (i < k, warp shuffles) after the load, and again
// before the store, gives the same row / column layout.
struct TcmGeom {
  int nrest;
  int rest[32];
  int nswap;      // lane bits exchanged with register bits (0-4)
  i64 lanes[32];  // offsets of the lane bits
  i64 rowhi[4];   // offsets of group-row bits 5, 6
  i64 chi;        // offset of block column bit 4
  i64 clo[16];    // offsets of the register bits
};

// Exchange lane bit I with register bit I of v: the value held for (lane
// bit a, register bit b) moves to (lane bit b, register bit a).  All lanes
// of the warp take part.
template <int I>
__device__ __forceinline__ void tcm_swap(float2 (&v)[16], int lane) {
  const bool up = (lane >> I) & 1;
#pragma unroll
  for (int r = 0; r < 16; ++r) {
    if (r & (1 << I)) continue;
    const int r1 = r | (1 << I);
    const float2 send = up ? v[r] : v[r1];
    float2 recv;
    recv.x = __shfl_xor_sync(0xffffffffu, send.x, 1 << I);
    recv.y = __shfl_xor_sync(0xffffffffu, send.y, 1 << I);
    if (up) v[r] = recv;
    else v[r1] = recv;
  }
}

// the exchanges commute and each is its own inverse: the same call maps
// the load layout to rows and the rows back to the store layout
__device__ __forceinline__ void tcm_transpose(float2 (&v)[16], int lane, int nswap) {
  if (nswap > 0) tcm_swap<0>(v, lane);
  if (nswap > 1) tcm_swap<1>(v, lane);
  if (nswap > 2) tcm_swap<2>(v, lane);
  if (nswap > 3) tcm_swap<3>(v, lane);
}

__global__ void __launch_bounds__(TC_THREADS, 2)
    k_fused5_tcm(float2* __restrict__ psi, i64 ntiles, const __grid_constant__ TcmGeom geo,
                 const __grid_constant__ TcGate G, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t s_base = smem_u32(sm);
  const uint32_t mb = smem_u32(&mbar);

  for (int e = tid; e < TC_N * TC_K; e += TC_THREADS) {
    const int n = e / TC_K, k = e % TC_K;
    const int r = n >> 1, c = k >> 1;
    float v;
    if ((n & 1) == 0) v = (k & 1) == 0 ? G.ur[r][c] : -G.ui[r][c];
    else v = (k & 1) == 0 ? G.ui[r][c] : G.ur[r][c];
    const float h = tf32_head(v);
    const uint32_t o = core_off(n, k, TC_B_LBO, TC_B_SBO);
    *(float*)(sm + o) = h;
    *(float*)(sm + TC_B_BYTES + o) = v - h;
  }
  if (tid == 0) {
    abort_flag = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mb));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_base)),
                 "r"(TCM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // B, written here, is read by the MMAs
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_base;
  constexpr uint32_t IDESC = tc_idesc(TC_M, TC_N);
  uint32_t phase = 0;
  const int h = warp >> 2;
  const uint32_t tlane = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + 32 * h;
  const int my_rest = lane < geo.nrest ? geo.rest[lane] : -1;
  const i64 toff = geo.lanes[lane] + geo.rowhi[warp & 3] + (h ? geo.chi : 0);

  float2 v[16];
  i64 t = blockIdx.x;
  i64 base = 0;
  if (t < ntiles) {
    base = tile_base(t, lane, my_rest);
    const float2* src = psi + base + toff;
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = src[geo.clo[j]];
  }
  for (; t < ntiles; t += gridDim.x) {
    // registers -> A_hi, A_lo (columns 2c, 2c + 1 = re, im of element c)
    tcm_transpose(v, lane, geo.nswap);
    {
      float a[32];
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        a[2 * j] = tf32_head(v[j].x);
        a[2 * j + 1] = tf32_head(v[j].y);
      }
      tmem_st16(tlane + 64, a);
      tmem_st16(tlane + 80, a + 16);
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        a[2 * j] = v[j].x - a[2 * j];
        a[2 * j + 1] = v[j].y - a[2 * j + 1];
      }
      tmem_st16(tlane + 128, a);
      tmem_st16(tlane + 144, a + 16);
      asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    // prefetch the next tile while the MMAs run
    const i64 tn = t + gridDim.x;
    i64 nbase = 0;
    if (tn < ntiles) {
      nbase = tile_base(tn, lane, my_rest);
      const float2* src = psi + nbase + toff;
#pragma unroll
      for (int j = 0; j < 16; ++j) v[j] = src[geo.clo[j]];
    }
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      uint32_t acc = 0;
#pragma unroll
      for (int s = 0; s < TC_K / 8; ++s) {
        const uint64_t bhi = smem_desc(s_base + s * 2 * TC_B_LBO, TC_B_LBO, TC_B_SBO);
        const uint64_t blo = smem_desc(s_base + TC_B_BYTES + s * 2 * TC_B_LBO, TC_B_LBO, TC_B_SBO);
        const uint32_t as[3] = {tmem + 64 + 8 * s, tmem + 64 + 8 * s, tmem + 128 + 8 * s};
        const uint64_t bs[3] = {bhi, blo, bhi};
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          asm volatile(
              "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
              " tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}\n" ::"r"(tmem),
              "r"(as[q]), "l"(bs[q]), "r"(IDESC), "r"(acc));
          acc = 1;
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mb)
                   : "memory");
    }
    if (tid == 0 && !mbar_wait(mb, phase)) abort_flag = 1;
    __syncthreads();
    if (abort_flag) {
      if (tid == 0) {
        *(volatile int*)err = 1;
        mbar_wait(mb, phase);
      }
      break;
    }
    phase ^= 1;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    float y[32];
    tmem_ld16(tlane, y);
    tmem_ld16(tlane + 16, y + 16);
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
    {
      float2 o[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) o[j] = make_float2(y[2 * j], y[2 * j + 1]);
      tcm_transpose(o, lane, geo.nswap);
      float2* dst = psi + base + toff;
#pragma unroll
      for (int j = 0; j < 16; ++j) dst[geo.clo[j]] = o[j];
    }
    // D and A are rewritten next: every thread's tensor-memory reads are done
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    base = nbase;
  }
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TCM_COLS));
}

namespace {
int* g_tc_err = nullptr;       // device address of the flag
int* g_tc_err_host = nullptr;  // the same word, page-locked host memory mapped into the device
}  // namespace

// Flag the tensor-core kernels set when a bounded mbarrier wait gives up:
// one word of mapped page-locked host memory, so the host reads it after a
// stream synchronisation without a copy.  Allocated and zeroed on first use,
// cleared by qgb_tc_status.
int* qgb_tc_err_flag() {
  if (!g_tc_err) {
    if (cudaHostAlloc((void**)&g_tc_err_host, sizeof(int), cudaHostAllocMapped) != cudaSuccess ||
        cudaHostGetDevicePointer((void**)&g_tc_err, g_tc_err_host, 0) != cudaSuccess) {
      qgb_set_error("tensor-core error flag: %s", cudaGetErrorString(cudaGetLastError()));
      g_tc_err = nullptr;
      return nullptr;
    }
    *(volatile int*)g_tc_err_host = 0;
  }
  return g_tc_err;
}

namespace {

// Tile geometry of a block on target bits tbits (matrix order: tbits[0] is
// the most significant bit of the block index) of an n-qubit state.  Column
// bit cbit[jt] of the permuted block matrix belongs to target jt: targets
// are ranked by index position, lowest first.
void make_geom(int n, const std::vector<int>& tbits, TcGeom* geo, int cbit[5]) {
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
  const int nb = (int)pos.size();
  geo->nbits = nb;
  // tile bit i -> group-row bit or block-column bit
  std::vector<int> rowbit(nb, -1), colbit(nb, -1);
  for (int i = 0; i < nb; ++i) {
    auto g = std::find(grp.begin(), grp.end(), pos[i]);
    if (g != grp.end()) rowbit[i] = (int)(g - grp.begin());
    else colbit[i] = cbit[std::find(tbits.begin(), tbits.end(), pos[i]) - tbits.begin()];
  }
  // t4 block qubits on index bits 0..3 (the lanes of a half-warp) take
  // column bits 0..t4-1, the rest of those lanes group rows 0..3-t4.  A
  // K-chunk stride that rotates the bank group by 2^(4-t4) (mod 8) then
  // makes every half-warp write of A hit 16 distinct 8-byte slots (t4 >= 1;
  // with t4 = 0 the column is fixed and 2 wavefronts are the minimum).
  int t4 = 0;
  for (int b : tbits) t4 += b < 4;
  const uint32_t rot = t4 == 3 ? 2 : t4 == 2 ? 4 : 1;
  geo->a_lbo = TC_A_LBO0 + 16 * rot;
  const int gsh = 4 - t4;
  auto scol = [&](uint32_t c) { return (uint32_t)((c << 7) ^ ((c << gsh) & 15u)); };
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
  for (int v = 0; v < TC_THREADS; ++v) {
    i64 dep;
    uint32_t row, col;
    split(v, 0, 8, &dep, &row, &col);
    geo->aoff_lo[v] = core_off(row, 2 * col, geo->a_lbo, TC_A_SBO);
    geo->sread_lo[v] = (uint16_t)(row ^ scol(col));
  }
  geo->g7 = nb > 7 ? (i64)1 << pos[7] : 0;
  for (int r = 0; r < TC_STEPS; ++r) {
    i64 dep;
    uint32_t row, col;
    split(r, 8, 4, &dep, &row, &col);
    geo->ghi[r] = dep;
    geo->aoff_hi[r] = core_off(row, 2 * col, geo->a_lbo, TC_A_SBO);
    geo->sread_hi[r] = (uint16_t)(row ^ scol(col));
  }
  for (int c = 0; c < 32; ++c) geo->scol[c] = (uint16_t)scol((uint32_t)c);
  geo->nrest = 0;
  for (int b = 0; b < n; ++b)
    if (std::find(pos.begin(), pos.end(), b) == pos.end()) geo->rest[geo->nrest++] = b;
}

// Permuted block matrix U'[r'][c'] = U[idx[r']][idx[c']]: idx[c'] is the
// block index whose bit (4 - jt) is bit cbit[jt] of c'.
void block_perm(const int cbit[5], int idx[32]) {
  for (int c = 0; c < 32; ++c) {
    idx[c] = 0;
    for (int jt = 0; jt < 5; ++jt)
      if ((c >> cbit[jt]) & 1) idx[c] |= 1 << (4 - jt);
  }
}

// Geometry of k_fused5_tcm for target bits tbits (index positions, matrix
// order) in a state of 12 qubits or more, and the column bit cbit[jt] of
// each target for block_perm.  Strided (shfl false): lanes are group rows
// 0..4, registers block columns 0..3, column bit i the i-th lowest target.
// Coalesced (shfl true): P = group-row bits 0..4 and the 4 lowest targets;
// lanes take the 5 lowest positions of P (index bits 0..4, or 0..3 and 5
// when the block is index bits 0..4), registers the other 4.  The k block
// bits among the lanes go first (lane bits 0..k-1), as do the k row bits
// among the registers, so exchanging lane and register bits 0..k-1 leaves
// rows on the lanes and block columns on the registers; block column bits
// 0..3 are then the exchanged block bits followed by the register ones.
void make_geom_m(int n, const std::vector<int>& tbits, bool shfl, TcmGeom* geo, int cbit[5]) {
  std::vector<int> st = tbits;
  std::sort(st.begin(), st.end());
  std::vector<int> grp;
  for (int b = 0; b < n && (int)grp.size() < 7; ++b)
    if (std::find(tbits.begin(), tbits.end(), b) == tbits.end()) grp.push_back(b);
  std::vector<int> lpos, rpos, colpos;
  if (!shfl) {
    lpos.assign(grp.begin(), grp.begin() + 5);
    rpos.assign(st.begin(), st.begin() + 4);
    colpos = rpos;
    geo->nswap = 0;
  } else {
    std::vector<int> P(grp.begin(), grp.begin() + 5);
    P.insert(P.end(), st.begin(), st.begin() + 4);
    std::sort(P.begin(), P.end());
    const std::vector<int> low5(P.begin(), P.begin() + 5), up4(P.begin() + 5, P.end());
    auto in = [](const std::vector<int>& v, int x) { return std::find(v.begin(), v.end(), x) != v.end(); };
    std::vector<int> blow, lrow, rup, ucol;
    for (int b : low5) (in(grp, b) ? lrow : blow).push_back(b);
    for (int b : up4) (in(grp, b) ? rup : ucol).push_back(b);
    lpos = blow;
    lpos.insert(lpos.end(), lrow.begin(), lrow.end());
    rpos = rup;
    rpos.insert(rpos.end(), ucol.begin(), ucol.end());
    colpos = blow;
    colpos.insert(colpos.end(), ucol.begin(), ucol.end());
    geo->nswap = (int)blow.size();
  }
  colpos.push_back(st[4]);
  for (int jt = 0; jt < 5; ++jt)
    cbit[jt] = (int)(std::find(colpos.begin(), colpos.end(), tbits[jt]) - colpos.begin());
  for (int l = 0; l < 32; ++l) {
    geo->lanes[l] = 0;
    for (int i = 0; i < 5; ++i)
      if ((l >> i) & 1) geo->lanes[l] += (i64)1 << lpos[i];
  }
  for (int k = 0; k < 4; ++k)
    geo->rowhi[k] = ((k & 1) ? (i64)1 << grp[5] : 0) + ((k & 2) ? (i64)1 << grp[6] : 0);
  for (int r = 0; r < 16; ++r) {
    geo->clo[r] = 0;
    for (int i = 0; i < 4; ++i)
      if ((r >> i) & 1) geo->clo[r] += (i64)1 << rpos[i];
  }
  geo->chi = (i64)1 << st[4];
  geo->nrest = 0;
  for (int b = 0; b < n; ++b)
    if (std::find(tbits.begin(), tbits.end(), b) == tbits.end() && std::find(grp.begin(), grp.end(), b) == grp.end())
      geo->rest[geo->nrest++] = b;
}

// The kernel and lane layout a full-tile block runs with: the larger of
// two estimates, each the fraction of HBM bandwidth measured at n=30 (8.6
// GB, 12 placements, `bench.py --workload tc5`), against 0.74 for
// k_fused5_tc.  Strided lanes, by 128-byte lines per warp access (2: 0.945,
// 4: 0.94, 8: 0.84; 32 sectors, when index bits 0 and 1 are both block
// bits, or more lines: 0.31-0.55).  Coalesced lanes, by lane / register
// exchanges (0-1: 0.955, 2: 0.895, 3: 0.78, 4: 0.72).
enum { TCM_OFF = 0, TCM_STRIDED = 1, TCM_SHFL = 2 };
int tcm_swaps(const std::vector<int>& tbits) {  // the nswap of make_geom_m's coalesced layout
  std::vector<int> st = tbits, P;
  std::sort(st.begin(), st.end());
  for (int b = 0; (int)P.size() < 5; ++b)
    if (std::find(tbits.begin(), tbits.end(), b) == tbits.end()) P.push_back(b);
  P.insert(P.end(), st.begin(), st.begin() + 4);
  std::sort(P.begin(), P.end());
  int k = 0;
  for (int i = 0; i < 5; ++i) k += std::find(st.begin(), st.begin() + 4, P[i]) != st.begin() + 4;
  return k;
}
int tcm_plan(const std::vector<int>& tbits) {
  int low4 = 0;
  bool b0 = false, b1 = false;
  for (int b : tbits) {
    low4 += b < 4;
    b0 |= b == 0;
    b1 |= b == 1;
  }
  const double strided = (b0 && b1) || low4 > 2 ? 0.45 : low4 == 0 ? 0.945 : low4 == 1 ? 0.94 : 0.84;
  const int k = tcm_swaps(tbits);
  const double shfl = k <= 1 ? 0.955 : k == 2 ? 0.895 : k == 3 ? 0.78 : 0.72;
  if (std::max(strided, shfl) <= 0.74) return TCM_OFF;
  return shfl > strided ? TCM_SHFL : TCM_STRIDED;
}

}  // namespace

int qgb_launch_fused5_tc(void* state, int n, const GateOp& g, cudaStream_t s) {
  if (g.tbits.size() != 5 || !g.cbits.empty() || n < 5) {
    qgb_set_error("qgb_apply_fused5_tc: needs an uncontrolled 5-qubit dense block");
    return QGB_ERR_INVALID;
  }
  int* err = qgb_tc_err_flag();
  if (!err) return QGB_ERR_CUDA;
  TcGeom* geo = new TcGeom();
  int cbit[5];
  make_geom(n, g.tbits, geo, cbit);
  const i64 ntiles = (i64)1 << (n - geo->nbits);
  const int blocks = (int)std::min<i64>(ntiles, (i64)qgb_num_sms() * 2);
  // QIBO_GB300_TC64_KERNEL=smem / tmem-strided / tmem-shfl picks the kernel
  // on full tiles (for comparisons); otherwise tcm_plan decides
  const char* pick = getenv("QIBO_GB300_TC64_KERNEL");
  const int plan = pick && !strcmp(pick, "smem")           ? TCM_OFF
                   : pick && !strcmp(pick, "tmem-strided") ? TCM_STRIDED
                   : pick && !strcmp(pick, "tmem-shfl")    ? TCM_SHFL
                                                           : tcm_plan(g.tbits);
  TcmGeom* gm = nullptr;
  if (geo->nbits == 12 && plan != TCM_OFF) {
    gm = new TcmGeom();
    make_geom_m(n, g.tbits, plan == TCM_SHFL, gm, cbit);
  }
  int idx[32];
  block_perm(cbit, idx);
  TcGate* G = new TcGate();
  for (int r = 0; r < 32; ++r)
    for (int c = 0; c < 32; ++c) {
      const zd u = g.coef[idx[r] * 32 + idx[c]];
      G->ur[r][c] = (float)u.real();
      G->ui[r][c] = (float)u.imag();
    }
  if (gm) {
    k_fused5_tcm<<<blocks, TC_THREADS, TCM_SMEM, s>>>((float2*)state, ntiles, *gm, *G, err);
    delete gm;
  } else {
    const bool full = geo->nbits == 12;
    const int sa = qgb_func_smem(full ? (const void*)k_fused5_tc<true> : (const void*)k_fused5_tc<false>, TC_SMEM);
    if (sa) {
      delete G;
      delete geo;
      return sa;
    }
    if (full) k_fused5_tc<true><<<blocks, TC_THREADS, TC_SMEM, s>>>((float2*)state, ntiles, *geo, *G, err);
    else k_fused5_tc<false><<<blocks, TC_THREADS, TC_SMEM, s>>>((float2*)state, ntiles, *geo, *G, err);
  }
  delete G;
  delete geo;
  QGB_LAUNCH_CHECK("k_fused5_tc");
  return QGB_OK;
}

extern "C" {

int qgb_apply_fused5_tc(void* state, int nqubits, int dtype, const int* qubits, const double* matrix,
                        void* stream) {
  const int nmin = dtype == QGB_C128 ? 12 : 5;
  if (!state || !qubits || !matrix || (dtype != QGB_C64 && dtype != QGB_C128) || nqubits > QGB_MAXQ) {
    qgb_set_error("qgb_apply_fused5_tc: bad arguments");
    return QGB_ERR_INVALID;
  }
  if (nqubits < nmin) {
    qgb_set_error("qgb_apply_fused5_tc: %s needs at least %d qubits (got %d)", dtype == QGB_C128 ? "complex128" : "complex64",
                  nmin, nqubits);
    return QGB_ERR_UNSUPPORTED;
  }
  GateOp g;
  int st = qgb_classify(nqubits, nullptr, 0, qubits, 5, nullptr, &g, "qgb_apply_fused5_tc");  // range/repeat checks
  if (st) return st;
  g = GateOp();
  g.kind = GK_DENSE;
  for (int j = 0; j < 5; ++j) g.tbits.push_back(nqubits - 1 - qubits[j]);
  g.coef.resize(1024);
  for (int i = 0; i < 1024; ++i) g.coef[i] = zd(matrix[2 * i], matrix[2 * i + 1]);
  return dtype == QGB_C128 ? qgb_launch_fused5_oz(state, nqubits, g, (cudaStream_t)stream, false)
                           : qgb_launch_fused5_tc(state, nqubits, g, (cudaStream_t)stream);
}

int qgb_tc_status(int* timed_out) {
  if (!timed_out) {
    qgb_set_error("qgb_tc_status: null");
    return QGB_ERR_INVALID;
  }
  *timed_out = 0;
  if (g_tc_err_host) {
    volatile int* f = g_tc_err_host;
    *timed_out = *f;
    if (*timed_out) *f = 0;
  }
  return QGB_OK;
}

}  // extern "C"
