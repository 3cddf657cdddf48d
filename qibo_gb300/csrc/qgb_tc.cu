// Fused 5-qubit blocks on the tensor cores (complex64, 3xTF32).
//
// A fused block (gates/special.py:28-153, matrix from Backend.matrix_fused,
// backends/abstract.py:2680-2717) is a dense 32x32 complex unitary U applied
// to every group of 32 amplitudes that differ only in the block's qubits.
// With amplitudes stored as interleaved (re, im) floats, U acts on a group as
// the 64x64 real matrix B with 2x2 blocks [[Ur, -Ui], [Ui, Ur]], so 128
// groups at a time form a GEMM  D[128 x 64] = A[128 x 64] * B^T.
//
// Each CTA (128 threads) gathers 128 groups, splits every value into a TF32
// head and a remainder (x = hi + lo), writes A_hi / A_lo to shared memory in
// the no-swizzle K-major core-matrix layout, and one thread issues
//   D = A_hi*B_hi + A_hi*B_lo + A_lo*B_hi     (3xTF32, FP32 accumulation)
// as 24 tcgen05.mma.kind::tf32 instructions (M=128, N=64, K=8) into tensor
// memory.  Completion is signalled through an mbarrier; thread t then reads
// TMEM lane t -- the output row of the very group it gathered -- with
// tcgen05.ld and scatters it back.  Every wait on the mbarrier is bounded:
// on timeout the kernel records an error flag, stops issuing work, frees its
// tensor memory and returns.
#include <algorithm>
#include <vector>

#include "qgb_plan.h"

#define TC_M 128
#define TC_N 64
#define TC_K 64
#define TC_THREADS 128
// shared memory layout (bytes); each operand region is padded so that the
// descriptor reads stay inside the allocation for either assignment of the
// leading/stride byte offsets
#define TC_A_BYTES (TC_M * TC_K * 4)          // 32 KB
#define TC_B_BYTES (TC_N * TC_K * 4)          // 16 KB
#define TC_OFF_AHI 0
#define TC_OFF_ALO (TC_OFF_AHI + TC_A_BYTES)  // 32 KB
#define TC_OFF_BHI (TC_OFF_ALO + TC_A_BYTES)  // 64 KB
#define TC_OFF_BLO (TC_OFF_BHI + TC_B_BYTES)  // 80 KB
// 96 KB of operands + 8 KB guard: with LBO/SBO exchanged the farthest read is
// B_lo + 7*2*128 + 7*1024 + 128 + 124 = 101.7 KB, still inside
#define TC_SMEM (TC_OFF_BLO + TC_B_BYTES + 8 * 1024)
#define TC_SPIN_LIMIT (1u << 26)

// K-major, no swizzle: 8-row x 16-byte core matrices; core matrices adjacent
// along K are LBO bytes apart, along M/N SBO bytes apart.
#define TC_A_SBO 128
#define TC_A_LBO (TC_M / 8 * 128)  // 2048: all 16 row-groups of one K-chunk
#define TC_B_SBO 128
#define TC_B_LBO (TC_N / 8 * 128)  // 1024

struct TcGate {
  float ur[32][32];
  float ui[32][32];
};

struct Offs32 {
  i64 o[32];
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for this architecture
  // base offset 0, absolute LBO mode 0, layout type 0 (no swizzle)
  return d;
}

// kind::tf32 instruction descriptor: D f32, A/B tf32, both K-major, N, M
__host__ __device__ constexpr uint32_t tc_idesc(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ uint32_t core_off(int row, int k, int lbo) {
  // byte offset of element (row, k) in a K-major no-swizzle operand
  return (uint32_t)((k >> 2) * lbo + (row >> 3) * 128 + (row & 7) * 16 + (k & 3) * 4);
}

__device__ __forceinline__ float tf32_head(float x) { return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u); }

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase) {
  for (uint32_t it = 0; it < TC_SPIN_LIMIT; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(mbar), "r"(phase)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__global__ void __launch_bounds__(TC_THREADS, 2)
    k_fused5_tc(float2* __restrict__ psi, i64 ngroups, BitInsert bi, Offs32 off, const __grid_constant__ TcGate G,
                int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t s_base = smem_u32(sm);
  const uint32_t mb = smem_u32(&mbar);

  // B = realified U, split into TF32 head and remainder; row n = output real,
  // column k = input real
  for (int e = tid; e < TC_N * TC_K; e += TC_THREADS) {
    const int n = e / TC_K, k = e % TC_K;
    const int r = n >> 1, c = k >> 1;
    float v;
    if ((n & 1) == 0) v = (k & 1) == 0 ? G.ur[r][c] : -G.ui[r][c];
    else v = (k & 1) == 0 ? G.ui[r][c] : G.ur[r][c];
    const float h = tf32_head(v);
    *(float*)(sm + TC_OFF_BHI + core_off(n, k, TC_B_LBO)) = h;
    *(float*)(sm + TC_OFF_BLO + core_off(n, k, TC_B_LBO)) = v - h;
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

  const i64 ntiles = (ngroups + TC_M - 1) / TC_M;
  for (i64 t = blockIdx.x; t < ntiles; t += gridDim.x) {
    // gather one group per thread and write A_hi / A_lo
    const i64 g = t * TC_M + tid;
    const bool valid = g < ngroups;
    const i64 base = valid ? insert_zeros(g, bi) : 0;
    float2 x[32];
#pragma unroll
    for (int c = 0; c < 32; ++c) x[c] = valid ? psi[base + off.o[c]] : make_float2(0.f, 0.f);
#pragma unroll
    for (int c = 0; c < 32; c += 2) {
      const float4 v = make_float4(x[c].x, x[c].y, x[c + 1].x, x[c + 1].y);
      const float4 h = make_float4(tf32_head(v.x), tf32_head(v.y), tf32_head(v.z), tf32_head(v.w));
      const uint32_t o = core_off(tid, 2 * c, TC_A_LBO);
      *(float4*)(sm + TC_OFF_AHI + o) = h;
      *(float4*)(sm + TC_OFF_ALO + o) = make_float4(v.x - h.x, v.y - h.y, v.z - h.z, v.w - h.w);
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      uint32_t acc = 0;
#pragma unroll
      for (int s = 0; s < TC_K / 8; ++s) {
        const uint64_t ahi = smem_desc(s_base + TC_OFF_AHI + s * 2 * TC_A_LBO, TC_A_LBO, TC_A_SBO);
        const uint64_t alo = smem_desc(s_base + TC_OFF_ALO + s * 2 * TC_A_LBO, TC_A_LBO, TC_A_SBO);
        const uint64_t bhi = smem_desc(s_base + TC_OFF_BHI + s * 2 * TC_B_LBO, TC_B_LBO, TC_B_SBO);
        const uint64_t blo = smem_desc(s_base + TC_OFF_BLO + s * 2 * TC_B_LBO, TC_B_LBO, TC_B_SBO);
        const uint64_t as[3] = {ahi, ahi, alo};
        const uint64_t bs[3] = {bhi, blo, bhi};
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          asm volatile(
              "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
              " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
              "l"(as[j]), "l"(bs[j]), "r"(IDESC), "r"(acc));
          acc = 1;
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mb)
                   : "memory");
    }
    const bool ok = mbar_wait(mb, phase);
    if (!ok) {
      if (lane == 0) atomicExch(&abort_flag, 1);
    }
    __syncthreads();
    if (abort_flag) {
      // record the failure, give the in-flight MMA one more bounded wait so
      // tensor memory is not freed under it, then leave
      if (tid == 0) atomicExch(err, 1);
      mbar_wait(mb, phase);
      break;
    }
    phase ^= 1;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    // TMEM lane (32*warp + lane) holds this thread's group
    float y[64];
    const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll
    for (int q = 0; q < 4; ++q) tmem_ld16(ta + q * 16, y + q * 16);
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
    if (valid) {
#pragma unroll
      for (int c = 0; c < 32; ++c) psi[base + off.o[c]] = make_float2(y[2 * c], y[2 * c + 1]);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
  }
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TC_N));
}

namespace {
int* g_tc_err = nullptr;
}

int qgb_launch_fused5_tc(void* state, int n, const GateOp& g, cudaStream_t s) {
  if (g.tbits.size() != 5 || !g.cbits.empty()) {
    qgb_set_error("qgb_apply_fused5_tc: needs an uncontrolled 5-qubit dense block");
    return QGB_ERR_INVALID;
  }
  if (!g_tc_err) QGB_TRY_CUDA(cudaMalloc(&g_tc_err, sizeof(int)));
  QGB_TRY_CUDA(cudaMemsetAsync(g_tc_err, 0, sizeof(int), s));
  BitInsert bi;
  std::vector<int> t = g.tbits;
  std::sort(t.begin(), t.end());
  bi.n = 5;
  for (int j = 0; j < 5; ++j) bi.pos[j] = t[j];
  Offs32 off;
  for (int m = 0; m < 32; ++m) {
    i64 o = 0;
    for (int j = 0; j < 5; ++j)
      if ((m >> (4 - j)) & 1) o |= (i64)1 << g.tbits[j];
    off.o[m] = o;
  }
  TcGate* G = new TcGate();
  for (int r = 0; r < 32; ++r)
    for (int c = 0; c < 32; ++c) {
      G->ur[r][c] = (float)g.coef[r * 32 + c].real();
      G->ui[r][c] = (float)g.coef[r * 32 + c].imag();
    }
  const i64 ngroups = (i64)1 << (n - 5);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_fused5_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM);
    attr = true;
  }
  const i64 ntiles = (ngroups + TC_M - 1) / TC_M;
  const int blocks = (int)std::min<i64>(ntiles, (i64)qgb_num_sms() * 2);
  k_fused5_tc<<<blocks, TC_THREADS, TC_SMEM, s>>>((float2*)state, ngroups, bi, off, *G, g_tc_err);
  delete G;
  QGB_LAUNCH_CHECK("k_fused5_tc");
  return QGB_OK;
}

extern "C" {

int qgb_apply_fused5_tc(void* state, int nqubits, const int* qubits, const double* matrix, void* stream) {
  if (!state || !qubits || !matrix || nqubits < 5 || nqubits > QGB_MAXQ) {
    qgb_set_error("qgb_apply_fused5_tc: bad arguments (complex64 state of at least 5 qubits)");
    return QGB_ERR_INVALID;
  }
  GateOp g;
  int st = qgb_classify(nqubits, nullptr, 0, qubits, 5, nullptr, &g, "qgb_apply_fused5_tc");  // range/repeat checks
  if (st) return st;
  g = GateOp();
  g.kind = GK_DENSE;
  for (int j = 0; j < 5; ++j) g.tbits.push_back(nqubits - 1 - qubits[j]);
  g.coef.resize(1024);
  for (int i = 0; i < 1024; ++i) g.coef[i] = zd(matrix[2 * i], matrix[2 * i + 1]);
  return qgb_launch_fused5_tc(state, nqubits, g, (cudaStream_t)stream);
}

int qgb_tc_status(int* timed_out) {
  if (!timed_out) { qgb_set_error("qgb_tc_status: null"); return QGB_ERR_INVALID; }
  *timed_out = 0;
  if (g_tc_err) QGB_TRY_CUDA(cudaMemcpy(timed_out, g_tc_err, sizeof(int), cudaMemcpyDeviceToHost));
  return QGB_OK;
}

}  // extern "C"
