// Measurement and observables on the device:
//  * marginal probabilities (Backend.calculate_probabilities,
//    backends/abstract.py:2734-2758, ordered as _order_probabilities
//    :3371-3381) with FP64 accumulation and a deterministic two-stage
//    reduction (no floating-point atomics: the same input gives the same
//    bits on every run);
//  * the squared norm;
//  * shot sampling (Backend.sample_shots / sample_frequencies,
//    :2760-2801): an FP64 two-level CDF (inclusive prefix over 64-entry
//    chunk sums, then an in-chunk running sum) searched by one thread per
//    shot with uniforms from a Philox4x32-10 counter-based stream (Salmon,
//    Moraes, Dror, Shaw, SC'11), so each shot's draw depends only on
//    (seed, shot index);
//  * Pauli-sum expectation values (Backend.exp_value_observable_symbolic,
//    :2946-3054): one pass per distinct X/Y flip mask covering all terms
//    that share it, instead of one einsum pass per term.
#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <type_traits>
#include <vector>

#include "qgb_common.cuh"
#include "qgb_df64.cuh"

// ------------------------------------------------------------ reductions --
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// deterministic block sum (256 threads): result valid in thread 0
__device__ double block_sum256(double v) {
  __shared__ double sh[8];
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x < 32) {
    r = (l < 8) ? sh[l] : 0.0;
    r = warp_sum(r);
  }
  __syncthreads();
  return r;
}

__host__ __device__ __forceinline__ i64 imin64(i64 a, i64 b) { return a < b ? a : b; }

// insert a zero at each of the ascending positions pos[0..n)
__device__ __forceinline__ i64 insert_zeros_n(i64 t, const int* pos, int n) {
  for (int j = 0; j < n; ++j) {
    const int p = pos[j];
    t = ((t >> p) << (p + 1)) | (t & ((((i64)1) << p) - 1));
  }
  return t;
}

// deposit the low bits of v into the (ascending) positions pos[0..n)
__device__ __forceinline__ i64 deposit(i64 v, const int* pos, int n) {
  i64 r = 0;
  for (int j = 0; j < n; ++j) r |= ((v >> j) & 1) << pos[j];
  return r;
}

struct ProbGeom {
  int n, nq, u;
  u64 umask;  // unmeasured positions
  int mpos[QGB_MAXQ];  // measured bit positions, output-bit order: mpos[j] <-> output bit j
  int msorted[QGB_MAXQ];  // measured positions ascending
  int upos[QGB_MAXQ];  // unmeasured positions ascending
};

// all qubits measured: out[j] = |psi[i]|^2 with j = gathered bits of i
template <typename T>
__global__ void __launch_bounds__(256) k_probs_all(const typename T::S* __restrict__ psi, i64 N, ProbGeom g,
                                                   int identity, double* __restrict__ out) {
  const i64 stride = (i64)gridDim.x * blockDim.x;
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < N; i += stride) {
    const double p = T::abs2(T::load(psi, i));
    i64 j = i;
    if (!identity) {
      j = 0;
      for (int b = 0; b < g.nq; ++b) j |= ((i >> g.mpos[b]) & 1) << b;
    }
    out[j] = p;
  }
}

// few unmeasured qubits: one thread per output sums its 2^u amplitudes
template <typename T>
__global__ void __launch_bounds__(256) k_probs_thread(const typename T::S* __restrict__ psi, i64 nout, ProbGeom g,
                                                      double* __restrict__ out) {
  const i64 stride = (i64)gridDim.x * blockDim.x;
  const i64 nr = (i64)1 << g.u;
  for (i64 j = blockIdx.x * (i64)blockDim.x + threadIdx.x; j < nout; j += stride) {
    i64 base = 0;
    for (int b = 0; b < g.nq; ++b) base |= ((j >> b) & 1) << g.mpos[b];
    typename T::Acc acc = T::acc_zero();
    // unmeasured offsets in order: a counter under the mask
    i64 off = 0;
    const i64 step = (i64)1 << g.upos[0];
    for (i64 r = 0; r < nr; ++r) {
      acc = T::acc_add(acc, T::load(psi, base | off), (int)(r & 1));
      off = (i64)(((u64)off | ~g.umask) + (u64)step) & (i64)g.umask;
    }
    out[j] = T::acc_value(acc);
  }
}

// many unmeasured qubits: block (j, p) sums part p of output j's amplitudes
template <typename T>
__global__ void __launch_bounds__(256) k_probs_block(const typename T::S* __restrict__ psi, int parts, i64 per_part,
                                                     ProbGeom g, double* __restrict__ dst) {
  const i64 j = blockIdx.x / parts;
  const int p = blockIdx.x % parts;
  i64 base = 0;
  for (int b = 0; b < g.nq; ++b) base |= ((j >> b) & 1) << g.mpos[b];
  typename T::Acc acc = T::acc_zero();
  const i64 r0 = (i64)p * per_part;
  // unmeasured index r -> amplitude index: zeros inserted at the measured
  // positions once, then a counter under the unmeasured mask advanced by
  // the deposited stride (carries skip the measured bits)
  i64 off = insert_zeros_n(r0 + threadIdx.x, g.msorted, g.nq);
  const u64 step = (u64)insert_zeros_n(blockDim.x, g.msorted, g.nq);
  int it = 0;
#pragma unroll 4
  for (i64 r = r0 + threadIdx.x; r < r0 + per_part; r += blockDim.x, ++it) {
    acc = T::acc_add(acc, T::load(psi, off | base), it & 1);
    off = (i64)(((u64)off | ~g.umask) + step) & (i64)g.umask;
  }
  const double sum = block_sum256(T::acc_value(acc));
  if (threadIdx.x == 0) dst[blockIdx.x] = sum;
}

// out[j] = sum_p src[j*parts + p], one warp per output, fixed order
__global__ void k_sum_parts(const double* __restrict__ src, i64 nout, int parts, double* __restrict__ out) {
  const i64 warp = (blockIdx.x * (i64)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= nout) return;
  double acc = 0.0;
  for (int p = lane; p < parts; p += 32) acc += src[warp * parts + p];
  acc = warp_sum(acc);
  if (lane == 0) out[warp] = acc;
}

namespace {

int prob_plan(int n, int nq, i64* parts, i64* per_part) {
  const int u = n - nq;
  if (u <= 10) { *parts = 0; *per_part = 0; return 0; }
  const i64 items = (i64)1 << u;
  i64 pp = std::max<i64>(8192, items / 1024);
  *per_part = pp;
  *parts = items / pp;
  return 0;
}

template <typename T>
int probs_impl(const void* state, int n, const int* qubits, int nq, double* out, void* scratch, cudaStream_t s) {
  ProbGeom g;
  g.n = n;
  g.nq = nq;
  g.u = n - nq;
  std::vector<int> mbits;
  u64 seen = 0;
  for (int j = 0; j < nq; ++j) {
    const int q = qubits[j];
    if (q < 0 || q >= n) { qgb_set_error("qgb_probabilities: qubit %d out of range", q); return QGB_ERR_INVALID; }
    if (seen & (1ull << q)) { qgb_set_error("qgb_probabilities: qubit %d repeated", q); return QGB_ERR_INVALID; }
    seen |= 1ull << q;
    // qubits[0] is the most significant output bit
    g.mpos[nq - 1 - j] = n - 1 - q;
    mbits.push_back(n - 1 - q);
  }
  int ui = 0;
  g.umask = 0;
  for (int b = 0; b < n; ++b)
    if (std::find(mbits.begin(), mbits.end(), b) == mbits.end()) {
      g.upos[ui++] = b;
      g.umask |= 1ull << b;
    }
  std::vector<int> sorted = mbits;
  std::sort(sorted.begin(), sorted.end());
  for (int j = 0; j < nq; ++j) g.msorted[j] = sorted[j];
  typedef typename T::S S;
  const i64 nout = (i64)1 << nq;
  if (g.u == 0) {
    bool identity = true;
    for (int b = 0; b < nq; ++b)
      if (g.mpos[b] != b) identity = false;
    int blocks;
    grid_for(nout, 256, &blocks);
    k_probs_all<T><<<blocks, 256, 0, s>>>((const S*)state, nout, g, identity ? 1 : 0, out);
    QGB_LAUNCH_CHECK("k_probs_all");
    return QGB_OK;
  }
  i64 parts, per_part;
  prob_plan(n, nq, &parts, &per_part);
  if (parts == 0) {
    int blocks;
    grid_for(nout, 256, &blocks);
    k_probs_thread<T><<<blocks, 256, 0, s>>>((const S*)state, nout, g, out);
    QGB_LAUNCH_CHECK("k_probs_thread");
    return QGB_OK;
  }
  const i64 nblocks = nout * parts;
  if (parts == 1) {
    k_probs_block<T><<<(unsigned)nblocks, 256, 0, s>>>((const S*)state, 1, per_part, g, out);
    QGB_LAUNCH_CHECK("k_probs_block");
    return QGB_OK;
  }
  if (!scratch) { qgb_set_error("qgb_probabilities: scratch buffer required"); return QGB_ERR_INVALID; }
  double* part = (double*)scratch;
  k_probs_block<T><<<(unsigned)nblocks, 256, 0, s>>>((const S*)state, (int)parts, per_part, g, part);
  QGB_LAUNCH_CHECK("k_probs_block");
  const i64 threads = nout * 32;
  k_sum_parts<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(part, nout, (int)parts, out);
  QGB_LAUNCH_CHECK("k_sum_parts");
  return QGB_OK;
}

}  // namespace

extern "C" {

size_t qgb_probs_scratch_bytes(int nqubits, int nq) {
  if (nq < 0 || nq > nqubits) return 0;
  i64 parts, per_part;
  prob_plan(nqubits, nq, &parts, &per_part);
  if (parts <= 1) return 0;
  return (size_t)(((i64)1 << nq) * parts * sizeof(double));
}

int qgb_probabilities(const void* state, int nqubits, int dtype, const int* qubits, int nq, double* out,
                      void* scratch, void* stream) {
  if (!state || !out) { qgb_set_error("qgb_probabilities: null pointer"); return QGB_ERR_INVALID; }
  if (nqubits < 1 || nqubits > QGB_MAXQ || nq < 0 || nq > nqubits) {
    qgb_set_error("qgb_probabilities: bad sizes n=%d nq=%d", nqubits, nq);
    return QGB_ERR_INVALID;
  }
  if (!dtype_ok(dtype)) { qgb_set_error("qgb_probabilities: bad dtype"); return QGB_ERR_INVALID; }
  cudaStream_t s = (cudaStream_t)stream;
  return dtype == QGB_C128 ? probs_impl<TC128>(state, nqubits, qubits, nq, out, scratch, s)
                           : probs_impl<TC64>(state, nqubits, qubits, nq, out, scratch, s);
}

}  // extern "C"

// ------------------------------------------------------------------ norm --
template <typename T>
__global__ void __launch_bounds__(256) k_norm_part(const typename T::S* __restrict__ psi, i64 N,
                                                   double* __restrict__ part) {
  typename T::Acc acc = T::acc_zero();
  const i64 stride = (i64)gridDim.x * blockDim.x;
  int it = 0;
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < N; i += stride, ++it)
    acc = T::acc_add(acc, T::load(psi, i), it & 1);
  const double sum = block_sum256(T::acc_value(acc));
  if (threadIdx.x == 0) part[blockIdx.x] = sum;
}

__global__ void k_final_sum(const double* __restrict__ part, int nparts, double* __restrict__ out) {
  double acc = 0.0;
  for (int p = threadIdx.x; p < nparts; p += blockDim.x) acc += part[p];
  acc = block_sum256(acc);
  if (threadIdx.x == 0) *out = acc;
}

static const int kNormBlocksCap = 16 * 160;

extern "C" size_t qgb_norm_scratch_bytes(void) { return (size_t)kNormBlocksCap * sizeof(double); }

extern "C" int qgb_norm2(const void* state, int nqubits, int dtype, double* out, void* scratch, void* stream) {
  if (!state || !out || !scratch || nqubits < 1 || nqubits > QGB_MAXQ || !dtype_ok(dtype)) {
    qgb_set_error("qgb_norm2: bad arguments");
    return QGB_ERR_INVALID;
  }
  const i64 N = (i64)1 << nqubits;
  int blocks;
  grid_for(N, 256, &blocks);
  if (blocks > kNormBlocksCap) blocks = kNormBlocksCap;
  double* part = (double*)scratch;
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == QGB_C128) k_norm_part<TC128><<<blocks, 256, 0, s>>>((const double2*)state, N, part);
  else k_norm_part<TC64><<<blocks, 256, 0, s>>>((const float2*)state, N, part);
  QGB_LAUNCH_CHECK("k_norm_part");
  k_final_sum<<<1, 256, 0, s>>>(part, blocks, out);
  QGB_LAUNCH_CHECK("k_final_sum");
  return QGB_OK;
}

// -------------------------------------------------------------- sampling --
// Philox4x32-10 (Salmon et al., SC'11): 10 rounds of two 32x32->64
// multiplications with the published multipliers and Weyl key increments.
struct Philox4 { uint32_t v[4]; };

__host__ __device__ __forceinline__ Philox4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                                          uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r > 0) { k0 += W0; k1 += W1; }
    const uint64_t p0 = (uint64_t)M0 * c0, p1 = (uint64_t)M1 * c2;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
  }
  Philox4 r;
  r.v[0] = c0; r.v[1] = c1; r.v[2] = c2; r.v[3] = c3;
  return r;
}

// uniform double in [0, 1) with 53 random bits
__device__ __forceinline__ double u01_53(uint32_t a, uint32_t b) {
  const uint64_t x = (((uint64_t)a << 32) | b) >> 11;
  return (double)x * (1.0 / 9007199254740992.0);
}

#define QGB_CHUNK 64

// chunk[c] = sequential sum of probs[c*64 .. c*64+64)
__global__ void k_chunk_sums(const double* __restrict__ probs, i64 nprobs, i64 nchunks, double* __restrict__ chunk) {
  const i64 stride = (i64)gridDim.x * blockDim.x;
  for (i64 c = blockIdx.x * (i64)blockDim.x + threadIdx.x; c < nchunks; c += stride) {
    double acc = 0.0;
    const i64 e = imin64(nprobs, (c + 1) * QGB_CHUNK);
    for (i64 i = c * QGB_CHUNK; i < e; ++i) acc += probs[i];
    chunk[c] = acc;
  }
}

// in-place inclusive scan of 1024-element tiles (256 threads x 4); tile totals to tot
__global__ void k_scan_tiles(double* __restrict__ a, i64 n, double* __restrict__ tot) {
  __shared__ double sh[256];
  const i64 base = (i64)blockIdx.x * 1024 + threadIdx.x * 4;
  double v[4];
  double run = 0.0;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    v[e] = (base + e < n) ? a[base + e] : 0.0;
    run += v[e];
    v[e] = run;
  }
  sh[threadIdx.x] = run;
  __syncthreads();
  // Hillis-Steele over the 256 thread totals
  for (int off = 1; off < 256; off <<= 1) {
    double add = (threadIdx.x >= off) ? sh[threadIdx.x - off] : 0.0;
    __syncthreads();
    sh[threadIdx.x] += add;
    __syncthreads();
  }
  const double prefix = threadIdx.x > 0 ? sh[threadIdx.x - 1] : 0.0;
#pragma unroll
  for (int e = 0; e < 4; ++e)
    if (base + e < n) a[base + e] = v[e] + prefix;
  if (threadIdx.x == 255 && tot) tot[blockIdx.x] = sh[255];
}

// add the exclusive prefix of tile totals (already scanned inclusively) to tiles 1..
__global__ void k_scan_add(double* __restrict__ a, i64 n, const double* __restrict__ tot_scanned) {
  const i64 t = blockIdx.x;
  if (t == 0) return;
  const double off = tot_scanned[t - 1];
  for (i64 i = t * 1024 + threadIdx.x; i < imin64(n, (t + 1) * 1024); i += blockDim.x) a[i] += off;
}

template <bool COUNTS>
__global__ void __launch_bounds__(256) k_draw(const double* __restrict__ probs, i64 nprobs,
                                              const double* __restrict__ cdf, i64 nchunks, i64 nshots,
                                              uint32_t k0, uint32_t k1, int64_t* __restrict__ dst) {
  const double total = cdf[nchunks - 1];
  const i64 stride = (i64)gridDim.x * blockDim.x;
  for (i64 s = blockIdx.x * (i64)blockDim.x + threadIdx.x; s < nshots; s += stride) {
    Philox4 r = philox4x32_10((uint32_t)s, (uint32_t)(s >> 32), 0u, 0u, k0, k1);
    const double target = u01_53(r.v[0], r.v[1]) * total;
    // first chunk whose inclusive prefix exceeds target
    i64 lo = 0, hi = nchunks - 1;
    while (lo < hi) {
      const i64 mid = (lo + hi) >> 1;
      if (cdf[mid] > target) hi = mid; else lo = mid + 1;
    }
    double run = lo > 0 ? cdf[lo - 1] : 0.0;
    const i64 b = lo * QGB_CHUNK, e = imin64(nprobs, b + QGB_CHUNK);
    i64 pick = -1, last_nz = -1;
    for (i64 i = b; i < e; ++i) {
      const double p = probs[i];
      if (p > 0.0) {
        last_nz = i;
        run += p;
        if (run > target) { pick = i; break; }
      }
    }
    if (pick < 0) pick = last_nz;  // rounding between the two CDF levels
    if (pick < 0) pick = b;        // all-zero distribution: caller error, stay in bounds
    if (COUNTS) atomicAdd((unsigned long long*)&dst[pick], 1ull);
    else dst[s] = pick;
  }
}

// Sampling every qubit straight from the state (no 2^n probability vector):
// chunk sums of |psi|^2 over 64 amplitudes, then an in-chunk recompute.  The
// in-chunk running sum accumulates the same terms in the same order, with
// the same partial (FP64 or double-float by position parity), as the chunk
// sum, so both CDF levels agree.
template <typename T>
__global__ void __launch_bounds__(256) k_state_chunk_sums(const typename T::S* __restrict__ psi, i64 N, i64 nchunks,
                                                          double* __restrict__ chunk) {
  const i64 stride = (i64)gridDim.x * blockDim.x;
  for (i64 c = blockIdx.x * (i64)blockDim.x + threadIdx.x; c < nchunks; c += stride) {
    typename T::Acc acc = T::acc_zero();
    const i64 b = c * QGB_CHUNK, e = imin64(N, b + QGB_CHUNK);
    for (i64 i = b; i < e; ++i) acc = T::acc_add(acc, T::load(psi, i), (int)((i - b) & 1));
    chunk[c] = T::acc_value(acc);
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_draw_state(const typename T::S* __restrict__ psi, i64 N,
                                                    const double* __restrict__ cdf, i64 nchunks, i64 nshots,
                                                    uint32_t k0, uint32_t k1, int64_t* __restrict__ dst) {
  const double total = cdf[nchunks - 1];
  const i64 stride = (i64)gridDim.x * blockDim.x;
  for (i64 s = blockIdx.x * (i64)blockDim.x + threadIdx.x; s < nshots; s += stride) {
    Philox4 r = philox4x32_10((uint32_t)s, (uint32_t)(s >> 32), 0u, 0u, k0, k1);
    const double target = u01_53(r.v[0], r.v[1]) * total;
    i64 lo = 0, hi = nchunks - 1;
    while (lo < hi) {
      const i64 mid = (lo + hi) >> 1;
      if (cdf[mid] > target) hi = mid; else lo = mid + 1;
    }
    const double before = lo > 0 ? cdf[lo - 1] : 0.0;
    typename T::Acc run = T::acc_zero();
    const i64 b = lo * QGB_CHUNK, e = imin64(N, b + QGB_CHUNK);
    i64 pick = -1, last_nz = -1;
    for (i64 i = b; i < e; ++i) {
      const typename T::V v = T::load(psi, i);
      run = T::acc_add(run, v, (int)((i - b) & 1));  // the chunk sums' operation
      if (T::re(v) != 0.0 || T::im(v) != 0.0) {
        last_nz = i;
        if (before + T::acc_value(run) > target) { pick = i; break; }
      }
    }
    if (pick < 0) pick = last_nz;
    if (pick < 0) pick = b;
    dst[s] = pick;
  }
}

__global__ void k_philox_fill(uint32_t* out, i64 nblocks4, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1) {
  const i64 stride = (i64)gridDim.x * blockDim.x;
  for (i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x; t < nblocks4; t += stride) {
    Philox4 r = philox4x32_10((uint32_t)t, (uint32_t)(t >> 32), c2, c3, k0, k1);
    for (int e = 0; e < 4; ++e) out[4 * t + e] = r.v[e];
  }
}

namespace {
i64 ceil_div(i64 a, i64 b) { return (a + b - 1) / b; }

// scan layout in scratch: chunk[nchunks], then one level of tile totals per
// recursion step (each 1/1024 of the one before)
size_t scan_bytes(i64 n) {
  size_t b = 0;
  while (n > 1) {
    n = ceil_div(n, 1024);
    b += (size_t)n * sizeof(double);
  }
  return b;
}

int scan_inplace(double* a, i64 n, double* tmp, cudaStream_t s) {
  if (n <= 1) return QGB_OK;
  const i64 tiles = ceil_div(n, 1024);
  k_scan_tiles<<<(unsigned)tiles, 256, 0, s>>>(a, n, tiles > 1 ? tmp : nullptr);
  QGB_LAUNCH_CHECK("k_scan_tiles");
  if (tiles > 1) {
    int st = scan_inplace(tmp, tiles, tmp + tiles, s);
    if (st) return st;
    k_scan_add<<<(unsigned)tiles, 256, 0, s>>>(a, n, tmp);
    QGB_LAUNCH_CHECK("k_scan_add");
  }
  return QGB_OK;
}
}  // namespace

extern "C" {

size_t qgb_sample_scratch_bytes(int m) {
  if (m < 0 || m > QGB_MAXQ) return 0;
  const i64 nchunks = ceil_div((i64)1 << m, QGB_CHUNK);
  return (size_t)nchunks * sizeof(double) + scan_bytes(nchunks) + 256;
}

int qgb_sample(const double* probs, int m, int64_t nshots, uint64_t seed, int64_t* samples, int64_t* counts,
               void* scratch, void* stream) {
  if (!probs || m < 0 || m > QGB_MAXQ || nshots < 0 || (!samples && !counts) || !scratch) {
    qgb_set_error("qgb_sample: bad arguments");
    return QGB_ERR_INVALID;
  }
  if (nshots == 0) return QGB_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const i64 nprobs = (i64)1 << m;
  const i64 nchunks = ceil_div(nprobs, QGB_CHUNK);
  double* cdf = (double*)scratch;
  double* tmp = cdf + nchunks;
  int blocks;
  grid_for(nchunks, 256, &blocks);
  k_chunk_sums<<<blocks, 256, 0, s>>>(probs, nprobs, nchunks, cdf);
  QGB_LAUNCH_CHECK("k_chunk_sums");
  int st = scan_inplace(cdf, nchunks, tmp, s);
  if (st) return st;
  grid_for(nshots, 256, &blocks);
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  if (counts) k_draw<true><<<blocks, 256, 0, s>>>(probs, nprobs, cdf, nchunks, nshots, k0, k1, counts);
  else k_draw<false><<<blocks, 256, 0, s>>>(probs, nprobs, cdf, nchunks, nshots, k0, k1, samples);
  QGB_LAUNCH_CHECK("k_draw");
  return QGB_OK;
}

size_t qgb_sample_state_scratch_bytes(int nqubits) { return qgb_sample_scratch_bytes(nqubits); }

int qgb_sample_state(const void* state, int nqubits, int dtype, int64_t nshots, uint64_t seed, int64_t* samples,
                     void* scratch, void* stream) {
  if (!state || nqubits < 1 || nqubits > QGB_MAXQ || !dtype_ok(dtype) || nshots < 0 || !samples || !scratch) {
    qgb_set_error("qgb_sample_state: bad arguments");
    return QGB_ERR_INVALID;
  }
  if (nshots == 0) return QGB_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const i64 N = (i64)1 << nqubits;
  const i64 nchunks = ceil_div(N, QGB_CHUNK);
  double* cdf = (double*)scratch;
  int blocks;
  grid_for(nchunks, 256, &blocks);
  if (dtype == QGB_C128) k_state_chunk_sums<TC128><<<blocks, 256, 0, s>>>((const double2*)state, N, nchunks, cdf);
  else k_state_chunk_sums<TC64><<<blocks, 256, 0, s>>>((const float2*)state, N, nchunks, cdf);
  QGB_LAUNCH_CHECK("k_state_chunk_sums");
  int st = scan_inplace(cdf, nchunks, cdf + nchunks, s);
  if (st) return st;
  grid_for(nshots, 256, &blocks);
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  if (dtype == QGB_C128)
    k_draw_state<TC128><<<blocks, 256, 0, s>>>((const double2*)state, N, cdf, nchunks, nshots, k0, k1, samples);
  else
    k_draw_state<TC64><<<blocks, 256, 0, s>>>((const float2*)state, N, cdf, nchunks, nshots, k0, k1, samples);
  QGB_LAUNCH_CHECK("k_draw_state");
  return QGB_OK;
}

// Raw Philox4x32-10 output: out[4*t + e] = word e of philox(ctr = (t_lo,
// t_hi, c2, c3), key = (k0, k1)) for t < n4 (device pointer; for tests).
int qgb_philox_fill(uint32_t* out, int64_t n4, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1, void* stream) {
  if (!out || n4 < 0) { qgb_set_error("qgb_philox_fill: bad arguments"); return QGB_ERR_INVALID; }
  int blocks;
  grid_for(n4, 256, &blocks);
  k_philox_fill<<<blocks, 256, 0, (cudaStream_t)stream>>>(out, n4, c2, c3, k0, k1);
  QGB_LAUNCH_CHECK("k_philox_fill");
  return QGB_OK;
}

}  // extern "C"

// ----------------------------------------------------------- expectation --
#define QGB_TERMS_PER_LAUNCH 64

struct TermSet {
  int nterms;
  u64 zmask[QGB_TERMS_PER_LAUNCH];   // amplitude-index bit masks
  double coef[QGB_TERMS_PER_LAUNCH]; // diagonal: c_t; flip: c_t f_t (see k_expect_flip)
  float chi[QGB_TERMS_PER_LAUNCH], clo[QGB_TERMS_PER_LAUNCH];  // coef as a double-float
  // diagonal terms on 2^(5 + WB) amplitudes or more (k_expect_diag_wht):
  // terms sorted by m = index bits 5..4+WB of their mask, [mstart[m],
  // mstart[m+1]) having that m
  uint32_t mused;
  int mstart[33];
  // flip terms: bit k set when term k uses Im(conj(psi_i) psi_j), else Re
  uint32_t use_im_lo, use_im_hi;
  int any_re, any_im;
};

// Terms with no X/Y factor: sum_i |psi_i|^2 * sum_t c_t (-1)^popc(i & z_t)
// (states of fewer than 2^(5 + WB) amplitudes, WB of k_expect_diag_wht).
template <typename T>
__global__ void __launch_bounds__(256) k_expect_diag(const typename T::S* __restrict__ psi, i64 N,
                                                     const __grid_constant__ TermSet ts, double* __restrict__ part) {
  double acc = 0.0;
  const i64 stride = (i64)gridDim.x * blockDim.x;
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < N; i += stride) {
    const double p = T::abs2(T::load(psi, i));
    double w = 0.0;
    for (int t = 0; t < ts.nterms; ++t) w += (__popcll((u64)i & ts.zmask[t]) & 1) ? -ts.coef[t] : ts.coef[t];
    acc = fma(p, w, acc);
  }
  acc = block_sum256(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

// The same on runs of 2^(5+WB) amplitudes, one per warp: lane l takes
// amplitudes base + l + 32 k, k < 2^WB (coalesced), so k spans index bits
// 5..4+WB.  With p_k = |psi|^2 and S the Walsh-Hadamard transform of p over
// k (S[m] = sum_k (-1)^popc(k & m) p_k, WB butterfly stages), term t adds
// c_t (-1)^popc(base & z_t) S[m_t] for the run, m_t = index bits 5..4+WB of
// z_t: a cost per amplitude independent of the number of terms, against one
// per term and amplitude.  Everything is double-float on the FP32 pipe
// (about 48 bits; GB300's FP64 pipe would bound the pass otherwise): the
// squares (split exactly), the butterflies, each run's signed coefficient
// sums and their products with S; each thread's partial becomes one double.
template <typename T, int WB>
__global__ void __launch_bounds__(256) k_expect_diag_wht(const typename T::S* __restrict__ psi, i64 nruns,
                                                         const __grid_constant__ TermSet ts,
                                                         double* __restrict__ part) {
  constexpr int K = 1 << WB;
  const int lane = threadIdx.x & 31;
  const i64 warp = (blockIdx.x * (i64)blockDim.x + threadIdx.x) >> 5;
  const i64 nwarps = ((i64)gridDim.x * blockDim.x) >> 5;
  DFAcc acc{0.f, 0.f};
  for (i64 w = warp; w < nruns; w += nwarps) {
    const i64 base = (w << (5 + WB)) | lane;
    DFAcc p[K];
#pragma unroll
    for (int k = 0; k < K; ++k) p[k] = T::abs2_df(T::load(psi, base | ((i64)k << 5)));
#pragma unroll
    for (int h = 1; h < K; h <<= 1) {
#pragma unroll
      for (int k = 0; k < K; ++k) {
        if ((k & h) == 0) {
          const DFAcc a = p[k], b = p[k | h];
          p[k] = df_plus(a, b);
          p[k | h] = df_minus(a, b);
        }
      }
    }
#pragma unroll
    for (int m = 0; m < K; ++m) {
      if (!((ts.mused >> m) & 1)) continue;
      // the run's signed coefficient sum, in four independent partial sums
      // (a single chain of double-float additions was latency-bound)
      DFAcc c4[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
      const int te = ts.mstart[m + 1];
      int t = ts.mstart[m];
      for (; t + 4 <= te; t += 4) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const bool odd = __popcll((u64)base & ts.zmask[t + j]) & 1;
          c4[j] = df_plus(c4[j], odd ? DFAcc{-ts.chi[t + j], -ts.clo[t + j]} : DFAcc{ts.chi[t + j], ts.clo[t + j]});
        }
      }
      for (; t < te; ++t) {
        const bool odd = __popcll((u64)base & ts.zmask[t]) & 1;
        c4[0] = df_plus(c4[0], odd ? DFAcc{-ts.chi[t], -ts.clo[t]} : DFAcc{ts.chi[t], ts.clo[t]});
      }
      const DFAcc cm = df_plus(df_plus(c4[0], c4[1]), df_plus(c4[2], c4[3]));
      // acc += cm * S[m]: the product of the heads split exactly, the cross terms added
      const float ph = cm.hi * p[m].hi;
      acc = df_add2(acc, ph, fmaf(cm.hi, p[m].hi, -ph) + fmaf(cm.hi, p[m].lo, cm.lo * p[m].hi));
    }
  }
  const double sum = block_sum256(f2d_exact(acc.hi) + f2d_exact(acc.lo));
  if (threadIdx.x == 0) part[blockIdx.x] = sum;
}

// Terms sharing flip mask x (highest set bit hb): for each pair (i, j = i^x)
// with bit hb of i clear, q = conj(psi_i) psi_j and the term adds
// c Re(i^ny (s_j q + s_i conj(q))), s_k = (-1)^popc(k & z).  Since
// s_j = s_i (-1)^ny (the bits of x & z are the term's Y factors), that is
// f s_i Re(q) for even ny and f s_i Im(q) for odd ny, f = +2 / -2 by ny mod
// 4: the host folds f into the coefficient and marks which part each term
// needs, so a pair costs the parts its terms need and one FMA each.
template <typename T>
__global__ void __launch_bounds__(256) k_expect_flip(const typename T::S* __restrict__ psi, i64 npairs, int hb,
                                                     u64 xmask, const __grid_constant__ TermSet ts,
                                                     double* __restrict__ part) {
  double acc = 0.0;
  const i64 stride = (i64)gridDim.x * blockDim.x;
  const i64 low = ((i64)1 << hb) - 1;
  if constexpr (T::kind == QGB_C64) {
    if (ts.nterms == 1) {
      // complex64, one term: the sign folded into a, the two products of
      // Re or Im of conj(a) b split exactly and summed in a double-float
      // partial (the FP32 pipe), times the coefficient once per thread
      DFAcc d{0.f, 0.f};
      for (i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x; t < npairs; t += stride) {
        const i64 i = ((t >> hb) << (hb + 1)) | (t & low);
        const float2 a = psi[i], b = psi[i ^ (i64)xmask];
        const bool odd = __popcll((u64)i & ts.zmask[0]) & 1;
        const float ax = odd ? -a.x : a.x, ay = odd ? -a.y : a.y;
        if (ts.any_im) {  // ax by - ay bx
          const float q1 = ax * b.y, q2 = ay * b.x;
          d = df_add2(d, q1, fmaf(ax, b.y, -q1));
          d = df_add2(d, -q2, -fmaf(ay, b.x, -q2));
        } else {  // ax bx + ay by
          const float q1 = ax * b.x, q2 = ay * b.y;
          d = df_add2(d, q1, fmaf(ax, b.x, -q1));
          d = df_add2(d, q2, fmaf(ay, b.y, -q2));
        }
      }
      const double sum = block_sum256(ts.coef[0] * (f2d_exact(d.hi) + f2d_exact(d.lo)));
      if (threadIdx.x == 0) part[blockIdx.x] = sum;
      return;
    }
  }
  for (i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x; t < npairs; t += stride) {
    const i64 i = ((t >> hb) << (hb + 1)) | (t & low);
    const i64 j = i ^ (i64)xmask;
    const typename T::V a = T::load(psi, i), b = T::load(psi, j);
    const double ar = T::re(a), ai = T::im(a), br = T::re(b), bi = T::im(b);
    if (ts.nterms == 1) {
      const double c = (__popcll((u64)i & ts.zmask[0]) & 1) ? -ts.coef[0] : ts.coef[0];
      acc = ts.any_im ? fma(c, fma(ar, bi, -(ai * br)), acc) : fma(c, fma(ar, br, ai * bi), acc);
      continue;
    }
    double cre = 0.0, cim = 0.0;
    for (int k = 0; k < ts.nterms; ++k) {
      const double c = (__popcll((u64)i & ts.zmask[k]) & 1) ? -ts.coef[k] : ts.coef[k];
      const uint32_t im = k < 32 ? (ts.use_im_lo >> k) & 1 : (ts.use_im_hi >> (k - 32)) & 1;
      if (im) cim += c;
      else cre += c;
    }
    if (ts.any_re) acc = fma(cre, fma(ar, br, ai * bi), acc);
    if (ts.any_im) acc = fma(cim, fma(ar, bi, -(ai * br)), acc);
  }
  acc = block_sum256(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

// Flip masks batched per tile: a CTA stages a tile of 2^L amplitudes in
// shared memory -- index bits 0..4 and the L - 5 index bits lpos[] above
// them, the other bits fixed by the tile -- and evaluates every term whose
// flip mask lies inside the tile from it, so terms on up to L - 5 distinct
// higher index bits share one read of the state instead of one pass per
// mask.  A term adds coef (-1)^popc(i & z) Re or Im of conj(psi_i)
// psi_{i^x} over the pairs with bit hb of i clear, as in k_expect_flip;
// the products are formed exactly in double-float on the FP32 pipe
// (complex128 tiles are split once on loading) and each term's tile sum is
// flushed to FP64.
#define FLIP_TILE_TERMS 16
struct FlipTileSet {
  int L;                         // a tile is 2^L amplitudes
  int nhi;                       // local bits 5..L-1 sit at index bits lpos[0..nhi)
  int lpos[16];
  int nrest;                     // the index bits the tile number spreads over, ascending
  int rest[64];
  int nterms;
  uint32_t xl[FLIP_TILE_TERMS];  // flip mask in local coordinates
  int hbl[FLIP_TILE_TERMS];      // its highest local bit
  uint32_t zl[FLIP_TILE_TERMS];  // z on the local bits, in local coordinates
  u64 zg[FLIP_TILE_TERMS];       // z on the index (the tile's own sign)
  double coef[FLIP_TILE_TERMS];  // c f, f = +-2 as for k_expect_flip
  uint32_t use_im;               // bit t: Im(conj(a) b), else Re
};

template <typename T>
__global__ void __launch_bounds__(256) k_expect_flip_tile(const typename T::S* __restrict__ psi, i64 ntiles,
                                                          const __grid_constant__ FlipTileSet fs,
                                                          double* __restrict__ part) {
  constexpr bool C128 = T::kind == QGB_C128;
  typedef typename std::conditional<C128, cdf, float2>::type E;
  extern __shared__ __align__(16) unsigned char flip_smem[];
  E* tile = reinterpret_cast<E*>(flip_smem);
  const int M = 1 << fs.L;
  double dsum = 0.0;
  for (i64 tt = blockIdx.x; tt < ntiles; tt += gridDim.x) {
    const i64 base = deposit(tt, fs.rest, fs.nrest);
    __syncthreads();  // the previous tile is no longer read
    for (int li = threadIdx.x; li < M; li += blockDim.x) {
      const i64 gi = base | (li & 31) | deposit(li >> 5, fs.lpos, fs.nhi);
      if constexpr (C128) {
        const double2 v = psi[gi];
        tile[li] = cdf{df_split_int(v.x), df_split_int(v.y)};
      } else {
        tile[li] = psi[gi];
      }
    }
    __syncthreads();
    for (int t = 0; t < fs.nterms; ++t) {
      const uint32_t xl = fs.xl[t], zl = fs.zl[t];
      const int hb = fs.hbl[t];
      const uint32_t low = (1u << hb) - 1u;
      const bool sb = __popcll((u64)base & fs.zg[t]) & 1;
      const bool im = (fs.use_im >> t) & 1;
      DFAcc acc{0.f, 0.f};
      for (int p = threadIdx.x; p < (M >> 1); p += blockDim.x) {
        const uint32_t li = (((uint32_t)p >> hb) << (hb + 1)) | ((uint32_t)p & low);
        const E a = tile[li], b = tile[li ^ xl];
        const bool odd = sb ^ (__popc(li & zl) & 1);
        if constexpr (C128) {
          // Re: a.re b.re + a.im b.im; Im: a.re b.im - a.im b.re
          const df x[2] = {a.re, a.im};
          const df y[2] = {im ? b.im : b.re, im ? b.re : b.im};
          const float sx[2] = {1.f, im ? -1.f : 1.f};
          const df r = df_dot<2>(x, y, sx);
          acc = odd ? df_add2(acc, -r.hi, -r.lo) : df_add2(acc, r.hi, r.lo);
        } else {
          const float ax = odd ? -a.x : a.x, ay = odd ? -a.y : a.y;
          const float b1 = im ? b.y : b.x, b2 = im ? b.x : b.y;
          const float q1 = ax * b1, q2 = ay * b2;
          acc = df_add2(acc, q1, fmaf(ax, b1, -q1));
          acc = im ? df_add2(acc, -q2, -fmaf(ay, b2, -q2)) : df_add2(acc, q2, fmaf(ay, b2, -q2));
        }
      }
      dsum += fs.coef[t] * (f2d_exact(acc.hi) + f2d_exact(acc.lo));
    }
  }
  const double sum = block_sum256(dsum);
  if (threadIdx.x == 0) part[blockIdx.x] = sum;
}

namespace {
const int kExpectBlocksCap = 16 * 160;

struct Group {
  u64 x;
  std::vector<int> terms;
};

std::vector<std::pair<Group, int>> expect_plan(int nterms, const uint64_t* xmask, int* nlaunch) {
  std::map<u64, Group> groups;
  for (int t = 0; t < nterms; ++t) {
    Group& g = groups[xmask[t]];
    g.x = xmask[t];
    g.terms.push_back(t);
  }
  std::vector<std::pair<Group, int>> out;
  int n = 0;
  for (auto& kv : groups) {
    const Group& g = kv.second;
    for (size_t s = 0; s < g.terms.size(); s += QGB_TERMS_PER_LAUNCH) {
      Group sub;
      sub.x = g.x;
      for (size_t e = s; e < std::min(g.terms.size(), s + QGB_TERMS_PER_LAUNCH); ++e) sub.terms.push_back(g.terms[e]);
      out.push_back({sub, n++});
    }
  }
  *nlaunch = n;
  return out;
}

// qibo qubit mask (bit q = qubit q) -> amplitude-index bit mask
u64 to_index_mask(u64 qmask, int n) {
  u64 r = 0;
  for (int q = 0; q < n; ++q)
    if ((qmask >> q) & 1) r |= 1ull << (n - 1 - q);
  return r;
}

template <typename T>
int expect_impl(const void* state, int n, const uint64_t* xmask, const uint64_t* zmask, const double* coef,
                int nterms, double* out, double* part, cudaStream_t s) {
  int nlaunch = 0;
  auto plan = expect_plan(nterms, xmask, &nlaunch);
  const i64 N = (i64)1 << n;
  typedef typename T::S S;
  int used = 0;
  // flip groups whose masks fit a tile (k_expect_flip_tile): batches of up
  // to FLIP_TILE_TERMS terms on at most L - 5 distinct index bits above bit
  // 4, one state read per batch; a batch of a single term keeps
  // k_expect_flip
  constexpr int L = T::kind == QGB_C128 ? 12 : 13;  // 64 KB tiles
  std::vector<char> tiled(plan.size(), 0);
  if (n >= L + 1) {
    std::vector<int> cand;
    for (size_t k = 0; k < plan.size(); ++k) {
      const u64 x = to_index_mask(plan[k].first.x, n);
      if (x != 0 && plan[k].first.terms.size() <= FLIP_TILE_TERMS && __builtin_popcountll(x & ~31ull) <= L - 5)
        cand.push_back((int)k);
    }
    std::stable_sort(cand.begin(), cand.end(), [&](int a, int b) {
      return to_index_mask(plan[a].first.x, n) < to_index_mask(plan[b].first.x, n);
    });
    std::vector<std::vector<int>> batches;
    u64 bits = 0;
    int bterms = 0;
    for (int k : cand) {
      const u64 hi = to_index_mask(plan[k].first.x, n) & ~31ull;
      const int nt = (int)plan[k].first.terms.size();
      if (batches.empty() || __builtin_popcountll(bits | hi) > L - 5 || bterms + nt > FLIP_TILE_TERMS) {
        batches.push_back({});
        bits = 0;
        bterms = 0;
      }
      batches.back().push_back(k);
      bits |= hi;
      bterms += nt;
    }
    for (const auto& batch : batches) {
      int bt = 0;
      u64 hib = 0;
      for (int k : batch) {
        bt += (int)plan[k].first.terms.size();
        hib |= to_index_mask(plan[k].first.x, n) & ~31ull;
      }
      if (bt < 2) continue;
      FlipTileSet* fs = new FlipTileSet();
      memset(fs, 0, sizeof(*fs));
      fs->L = L;
      for (int b = 5; b < n && __builtin_popcountll(hib) < L - 5; ++b) hib |= 1ull << b;  // fill the tile
      int local_of[64];
      for (int b = 0; b < 64; ++b) local_of[b] = b < 5 ? b : -1;
      for (int b = 5; b < n; ++b) {
        if ((hib >> b) & 1) {
          local_of[b] = 5 + fs->nhi;
          fs->lpos[fs->nhi++] = b;
        } else {
          fs->rest[fs->nrest++] = b;
        }
      }
      auto to_local = [&](u64 m) {
        uint32_t r = 0;
        for (int b = 0; b < n; ++b)
          if (((m >> b) & 1) && local_of[b] >= 0) r |= 1u << local_of[b];
        return r;
      };
      for (int k : batch) {
        const Group& g = plan[k].first;
        const u64 x = to_index_mask(g.x, n);
        for (int t : g.terms) {
          const int q = fs->nterms++;
          const u64 z = to_index_mask(zmask[t], n);
          const int ny = __builtin_popcountll(z & to_index_mask(xmask[t], n));
          fs->xl[q] = to_local(x);
          fs->hbl[q] = 31 - __builtin_clz(fs->xl[q]);
          fs->zl[q] = to_local(z);
          fs->zg[q] = z;
          fs->coef[q] = coef[t] * ((ny & 3) < 2 ? 2.0 : -2.0);
          if (ny & 1) fs->use_im |= 1u << q;
        }
      }
      const i64 ntiles = (i64)1 << (n - L);
      const int smem = (1 << L) * (T::kind == QGB_C128 ? 16 : 8);
      int st = qgb_func_smem((const void*)k_expect_flip_tile<T>, smem);
      if (st) {
        delete fs;
        return st;
      }
      const int blocks = (int)std::min<i64>(ntiles, std::min<i64>((i64)qgb_num_sms() * 3, kExpectBlocksCap));
      k_expect_flip_tile<T><<<blocks, 256, smem, s>>>((const S*)state, ntiles, *fs, part + used);
      delete fs;
      QGB_LAUNCH_CHECK("k_expect_flip_tile");
      used += blocks;
      for (int k : batch) tiled[k] = 1;
    }
  }
  for (size_t pk = 0; pk < plan.size(); ++pk) {
    if (tiled[pk]) continue;
    auto& pg = plan[pk];
    const Group& g = pg.first;
    TermSet ts;
    memset(&ts, 0, sizeof(ts));
    ts.nterms = (int)g.terms.size();
    const u64 x = to_index_mask(g.x, n);
    constexpr int WB = 4;  // transform bits of k_expect_diag_wht
    constexpr int WK = 1 << WB;
    const bool wht = x == 0 && n >= 5 + WB;
    std::vector<int> order(g.terms.begin(), g.terms.end());
    if (wht)  // diagonal terms by their index bits 5..4+WB
      std::stable_sort(order.begin(), order.end(), [&](int p, int q) {
        return ((to_index_mask(zmask[p], n) >> 5) & (WK - 1)) < ((to_index_mask(zmask[q], n) >> 5) & (WK - 1));
      });
    for (int k = 0; k < ts.nterms; ++k) {
      const int t = order[k];
      const u64 z = to_index_mask(zmask[t], n);
      const int ny = __builtin_popcountll(z & to_index_mask(xmask[t], n));
      ts.zmask[k] = z;
      ts.coef[k] = coef[t];
      ts.chi[k] = (float)coef[t];
      ts.clo[k] = (float)(coef[t] - (double)ts.chi[k]);
      if (x != 0) {  // f = +2 for ny mod 4 in {0, 1}, -2 for {2, 3}; odd ny uses Im
        ts.coef[k] = coef[t] * ((ny & 3) < 2 ? 2.0 : -2.0);
        if (ny & 1) {
          if (k < 32) ts.use_im_lo |= 1u << k;
          else ts.use_im_hi |= 1u << (k - 32);
          ts.any_im = 1;
        } else {
          ts.any_re = 1;
        }
      }
    }
    if (wht) {
      int k = 0;
      for (int m = 0; m < WK; ++m) {
        ts.mstart[m] = k;
        while (k < ts.nterms && (int)((ts.zmask[k] >> 5) & (WK - 1)) == m) ++k;
        if (k > ts.mstart[m]) ts.mused |= 1u << m;
      }
      ts.mstart[WK] = k;
    }
    int blocks;
    if (wht) {
      const i64 nruns = N >> (5 + WB);
      grid_for(nruns * 32, 256, &blocks);
      blocks = std::min(blocks, kExpectBlocksCap);
      k_expect_diag_wht<T, WB><<<blocks, 256, 0, s>>>((const S*)state, nruns, ts, part + used);
    } else if (x == 0) {
      grid_for(N, 256, &blocks);
      blocks = std::min(blocks, kExpectBlocksCap);
      k_expect_diag<T><<<blocks, 256, 0, s>>>((const S*)state, N, ts, part + used);
    } else {
      const int hb = 63 - __builtin_clzll(x);
      grid_for(N / 2, 256, &blocks);
      blocks = std::min(blocks, kExpectBlocksCap);
      k_expect_flip<T><<<blocks, 256, 0, s>>>((const S*)state, N / 2, hb, x, ts, part + used);
    }
    QGB_LAUNCH_CHECK("k_expect");
    used += blocks;
  }
  k_final_sum<<<1, 256, 0, s>>>(part, used, out);
  QGB_LAUNCH_CHECK("k_final_sum");
  return QGB_OK;
}
}  // namespace

// Dense observable: sum_i conj(psi_i) (H psi)_i, one warp per row of H
// (complex128, row-major, device).  Backend.expectation_value (:2807-2825).
template <typename T>
__global__ void __launch_bounds__(256) k_expect_dense(const typename T::S* __restrict__ psi, i64 N,
                                                      const double2* __restrict__ H, double* __restrict__ part) {
  const int lane = threadIdx.x & 31;
  const i64 warp = (blockIdx.x * (i64)blockDim.x + threadIdx.x) >> 5;
  const i64 nwarps = ((i64)gridDim.x * blockDim.x) >> 5;
  double acc = 0.0;
  for (i64 row = warp; row < N; row += nwarps) {
    double hr = 0.0, hi = 0.0;
    for (i64 j = lane; j < N; j += 32) {
      const double2 h = H[row * N + j];
      const typename T::V p = T::load(psi, j);
      hr += h.x * T::re(p) - h.y * T::im(p);
      hi += h.x * T::im(p) + h.y * T::re(p);
    }
    hr = warp_sum(hr);
    hi = warp_sum(hi);
    if (lane == 0) {
      const typename T::V a = T::load(psi, row);
      acc += T::re(a) * hr + T::im(a) * hi;  // Re(conj(a) * h)
    }
  }
  acc = block_sum256(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

extern "C" {

int qgb_expect_dense(const void* state, int nqubits, int dtype, const double* hamiltonian, double* out,
                     void* scratch, void* stream) {
  if (!state || !hamiltonian || !out || !scratch || nqubits < 1 || nqubits > 20 || !dtype_ok(dtype)) {
    qgb_set_error("qgb_expect_dense: bad arguments (dense observables up to 20 qubits)");
    return QGB_ERR_INVALID;
  }
  const i64 N = (i64)1 << nqubits;
  int blocks = (int)std::min<i64>((N + 7) / 8, kExpectBlocksCap);
  cudaStream_t s = (cudaStream_t)stream;
  double* part = (double*)scratch;
  if (dtype == QGB_C128) k_expect_dense<TC128><<<blocks, 256, 0, s>>>((const double2*)state, N, (const double2*)hamiltonian, part);
  else k_expect_dense<TC64><<<blocks, 256, 0, s>>>((const float2*)state, N, (const double2*)hamiltonian, part);
  QGB_LAUNCH_CHECK("k_expect_dense");
  k_final_sum<<<1, 256, 0, s>>>(part, blocks, out);
  QGB_LAUNCH_CHECK("k_final_sum");
  return QGB_OK;
}

size_t qgb_expect_scratch_bytes(int nqubits, int nterms) {
  (void)nqubits;
  // at most one launch per term plus one per distinct group
  return (size_t)(2 * std::max(nterms, 1)) * kExpectBlocksCap * sizeof(double);
}

int qgb_expect_pauli(const void* state, int nqubits, int dtype, const uint64_t* xmask, const uint64_t* zmask,
                     const double* coef, int nterms, double* out, void* scratch, void* stream) {
  if (!state || !out || !scratch || nterms < 0 || (nterms > 0 && (!xmask || !zmask || !coef)) || nqubits < 1 ||
      nqubits > 63 || !dtype_ok(dtype)) {
    qgb_set_error("qgb_expect_pauli: bad arguments");
    return QGB_ERR_INVALID;
  }
  for (int t = 0; t < nterms; ++t)
    if ((xmask[t] | zmask[t]) >> nqubits) {
      qgb_set_error("qgb_expect_pauli: term %d acts on a qubit >= %d", t, nqubits);
      return QGB_ERR_INVALID;
    }
  cudaStream_t s = (cudaStream_t)stream;
  if (nterms == 0) {
    QGB_TRY_CUDA(cudaMemsetAsync(out, 0, sizeof(double), s));
    return QGB_OK;
  }
  return dtype == QGB_C128 ? expect_impl<TC128>(state, nqubits, xmask, zmask, coef, nterms, out, (double*)scratch, s)
                           : expect_impl<TC64>(state, nqubits, xmask, zmask, coef, nterms, out, (double*)scratch, s);
}

}  // extern "C"

// ------------------------------------------------ sampling without allocation --
// Some callers cannot allocate device memory at the moment they need shots:
// a state vector sized to fill the GPU (33-34 qubits) leaves no room for a
// CDF buffer, and a serving loop that must not stall other requests cannot
// afford cudaMalloc/cudaFree, which may synchronise the whole device.  For
// them qgb_sample_noalloc keeps the CDF in a fixed device array that is part
// of this library's module: every GPU that loads the library holds it
// (QGB_NOALLOC_SAMPLE_MAX_M = 20, i.e. distributions of up to 2^20 outcomes,
// 2^14 chunk sums + 64 scan totals = 131 584 bytes) until the process exits.
#define QGB_NOALLOC_SAMPLE_MAX_M 20
#define QGB_NOALLOC_SAMPLE_DOUBLES ((1 << (QGB_NOALLOC_SAMPLE_MAX_M - 6)) + 64)

static __device__ __align__(256) double g_noalloc_sample_scratch[QGB_NOALLOC_SAMPLE_DOUBLES];

namespace {
std::mutex g_noalloc_mu;
double* g_noalloc_addr[64] = {};

// Device address of the built-in scratch for the current device, looked up
// once per device (host code must not use the array's name as an address).
int noalloc_scratch(double** out) {
  int dev = 0;
  QGB_TRY_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    qgb_set_error("qgb_sample_noalloc: device %d beyond the 64 devices supported", dev);
    return QGB_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_sample_scratch);
    if (e != cudaSuccess) return qgb_cuda_status(e, "cudaGetSymbolAddress(g_noalloc_sample_scratch)");
    g_noalloc_addr[dev] = (double*)p;
  }
  *out = g_noalloc_addr[dev];
  return QGB_OK;
}
}  // namespace

extern "C" int qgb_sample_noalloc(const double* probs, int m, int64_t nshots, uint64_t seed, int64_t* samples,
                                  int64_t* counts, void* stream) {
  if (m > QGB_NOALLOC_SAMPLE_MAX_M) {
    qgb_set_error("qgb_sample_noalloc: a distribution of 2^%d outcomes exceeds the built-in scratch "
                  "(at most 2^%d outcomes); use qgb_sample with a caller-provided scratch buffer",
                  m, QGB_NOALLOC_SAMPLE_MAX_M);
    return QGB_ERR_INVALID;
  }
  if (!probs || m < 0 || nshots < 0 || (!samples && !counts)) {
    qgb_set_error("qgb_sample_noalloc: bad arguments");
    return QGB_ERR_INVALID;
  }
  double* scratch = nullptr;
  int st = noalloc_scratch(&scratch);
  if (st) return st;
  // Every scratch word the sampler reads (chunk sums, scan totals) is written
  // earlier in the same call, so nothing has to be cleared between calls.
  return qgb_sample(probs, m, nshots, seed, samples, counts, scratch, stream);
}
