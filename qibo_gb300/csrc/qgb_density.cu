// Density matrices on the device.
//
// A density matrix rho of n qubits is kept as its (2^n x 2^n) matrix in
// row-major order, i.e. as the 2n-qubit vector v[i 2^n + j] = rho[i, j]:
// row qubit q is vector qubit q and column qubit q is vector qubit n + q,
// the layout of the reference's rho.ravel() (Backend.thermal_error_density_
// matrix, backends/abstract.py:2234-2241).  Gates and channels are then
// state-vector operations on 2n qubits (U on the row qubits and conj(U) on
// the column qubits; a channel as one superoperator on both), which
// qgb_apply_circuit runs with its shared-memory passes and tensor-core
// blocks.  This file holds what is specific to the matrix form:
//  * qgb_density_probabilities: marginals of the diagonal
//    (Backend.calculate_probabilities with density_matrix=True,
//    backends/abstract.py:2734-2758: "abab->a" then _order_probabilities),
//    in FP64 with a fixed reduction order;
//  * qgb_density_collapse: rows and columns projected onto a measured
//    outcome and divided by the kept block's trace
//    (Backend._collapse_density_matrix, :3249-3277), the outcome read from
//    device memory as qgb_collapse does;
//  * qgb_density_expect_pauli: sum_t c_t Re Tr(P_t rho)
//    (Backend.exp_value_observable_symbolic on a density matrix,
//    :2975-3054): with P|k> = i^ny (-1)^popc(k & z) |k ^ x>,
//    Tr(P rho) = sum_k i^ny (-1)^popc(k & z) rho[k, k ^ x];
//  * qgb_state_axpby: y = a x + b y, for channels whose superoperator is
//    wider than a 5-qubit gate (the weighted sum of Backend.apply_channel,
//    :2297-2312) and for the mean of repeated-execution states (:2603-2607).
#include <algorithm>
#include <cstring>
#include <vector>

#include "qgb_common.cuh"

#define QGB_DM_MAXQ (QGB_MAXQ / 2)  // 2n-qubit vectors
#define QGB_DM_TERMS 64             // Pauli terms per launch
#define QGB_DM_PARTS 4096           // partial sums in the scratch

namespace {

__device__ double dm_block_sum(double v) {  // 256 threads, fixed order; valid in thread 0
  __shared__ double sh[8];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < 8; ++w) r += sh[w];
  __syncthreads();
  return r;
}

// Row-index bit positions: qubit q of n sits at bit n - 1 - q.
struct DiagGeom {
  int n, nq, u;
  int mpos[QGB_DM_MAXQ];  // output bit b <-> row-index bit mpos[b]
  int upos[QGB_DM_MAXQ];  // unmeasured row-index bits, ascending
};

__device__ __forceinline__ i64 dm_deposit(i64 v, const int* pos, int k) {
  i64 r = 0;
  for (int j = 0; j < k; ++j) r |= ((v >> j) & 1) << pos[j];
  return r;
}

// Re rho[i, i]: vector index i (2^n + 1)
template <typename T>
__device__ __forceinline__ double dm_diag(const typename T::S* rho, int n, i64 i) {
  return T::re(T::load(rho, i * ((((i64)1) << n) + 1)));
}

// few unmeasured qubits: one thread per output sums its 2^u diagonal entries
template <typename T>
__global__ void __launch_bounds__(256) k_dm_probs_thread(const typename T::S* __restrict__ rho, i64 nout,
                                                         const __grid_constant__ DiagGeom g, double* __restrict__ out) {
  const i64 stride = (i64)gridDim.x * blockDim.x;
  for (i64 j = blockIdx.x * (i64)blockDim.x + threadIdx.x; j < nout; j += stride) {
    const i64 base = dm_deposit(j, g.mpos, g.nq);
    double acc = 0.0;
    for (i64 r = 0; r < ((i64)1 << g.u); ++r) acc += dm_diag<T>(rho, g.n, base | dm_deposit(r, g.upos, g.u));
    out[j] = acc;
  }
}

// many unmeasured qubits: one block per output
template <typename T>
__global__ void __launch_bounds__(256) k_dm_probs_block(const typename T::S* __restrict__ rho, i64 nout,
                                                        const __grid_constant__ DiagGeom g, double* __restrict__ out) {
  const i64 nr = (i64)1 << g.u;
  for (i64 j = blockIdx.x; j < nout; j += gridDim.x) {
    const i64 base = dm_deposit(j, g.mpos, g.nq);
    double acc = 0.0;
    for (i64 r = threadIdx.x; r < nr; r += blockDim.x) acc += dm_diag<T>(rho, g.n, base | dm_deposit(r, g.upos, g.u));
    acc = dm_block_sum(acc);
    if (threadIdx.x == 0) out[j] = acc;
  }
}

// Measured qubits of a collapse: row-index bits in the order of qubits[]
// (qubits[0] the most significant outcome bit) and ascending.
struct DmCollapse {
  int n, nq;
  int pos[QGB_DM_MAXQ];
  int sorted[QGB_DM_MAXQ];
};

__device__ __forceinline__ void dm_target(const DmCollapse& a, int64_t outcome, u64* mask, u64* value) {
  u64 m = 0, v = 0;
  for (int i = 0; i < a.nq; ++i) {
    const u64 bit = (u64)1 << a.pos[i];
    m |= bit;
    if (((u64)outcome >> (a.nq - 1 - i)) & 1) v |= bit;
  }
  *mask = m;
  *value = v;
}

// trace of the kept block: rows i with the outcome's bits, 2^(n - nq) of them
template <typename T>
__global__ void __launch_bounds__(256) k_dm_kept_trace(const typename T::S* __restrict__ rho, i64 nkept,
                                                       const __grid_constant__ DmCollapse a,
                                                       const int64_t* __restrict__ outcome, double* __restrict__ part) {
  u64 mask, value;
  dm_target(a, *outcome, &mask, &value);
  double acc = 0.0;
  const i64 stride = (i64)gridDim.x * blockDim.x;
  for (i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x; t < nkept; t += stride) {
    i64 i = t;
    for (int j = 0; j < a.nq; ++j) {
      const int p = a.sorted[j];
      i = ((i >> p) << (p + 1)) | (i & ((((i64)1) << p) - 1));
    }
    acc += dm_diag<T>(rho, a.n, i | (i64)value);
  }
  acc = dm_block_sum(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

// out = sum of part[0..nparts) (accumulate: out += that sum)
__global__ void k_dm_final(const double* __restrict__ part, int nparts, double* __restrict__ out, int accumulate) {
  double acc = 0.0;
  for (int p = threadIdx.x; p < nparts; p += blockDim.x) acc += part[p];
  acc = dm_block_sum(acc);
  if (threadIdx.x == 0) *out = accumulate ? *out + acc : acc;
}

// rho[i, j] kept (times 1 / trace) where both i and j carry the outcome, else 0;
// a kept block of trace 0 divides by 0, as in the reference
template <typename T>
__global__ void __launch_bounds__(256) k_dm_collapse_apply(typename T::S* __restrict__ rho, i64 total,
                                                           const __grid_constant__ DmCollapse a,
                                                           const int64_t* __restrict__ outcome,
                                                           const double* __restrict__ trace) {
  u64 mask, value;
  dm_target(a, *outcome, &mask, &value);
  const double inv = trace ? 1.0 / *trace : 1.0;
  const i64 low = (((i64)1) << a.n) - 1;
  const i64 stride = (i64)gridDim.x * blockDim.x;
  for (i64 v = blockIdx.x * (i64)blockDim.x + threadIdx.x; v < total; v += stride) {
    const u64 i = (u64)(v >> a.n), j = (u64)(v & low);
    const bool keep = (i & mask) == value && (j & mask) == value;
    T::store(rho, v, keep ? T::scale(T::load(rho, v), inv) : T::zero());
  }
}

struct DmTerms {
  int nterms;
  u64 x[QGB_DM_TERMS];      // row-index flip mask
  u64 z[QGB_DM_TERMS];      // row-index sign mask (Z and Y factors)
  int ph[QGB_DM_TERMS];     // number of Y factors mod 4
  double c[QGB_DM_TERMS];
};

template <typename T>
__global__ void __launch_bounds__(256) k_dm_expect(const typename T::S* __restrict__ rho, int n,
                                                   const __grid_constant__ DmTerms ts, double* __restrict__ part) {
  const i64 dim = (i64)1 << n;
  const i64 stride = (i64)gridDim.x * blockDim.x;
  double acc = 0.0;
  for (i64 k = blockIdx.x * (i64)blockDim.x + threadIdx.x; k < dim; k += stride) {
    for (int t = 0; t < ts.nterms; ++t) {
      const typename T::V v = T::load(rho, (k << n) | (k ^ (i64)ts.x[t]));
      // Re(i^ph v): ph 0 -> re, 1 -> -im, 2 -> -re, 3 -> im
      double w = (ts.ph[t] & 1) ? T::im(v) : T::re(v);
      if (ts.ph[t] == 1 || ts.ph[t] == 2) w = -w;
      if (__popcll((u64)k & ts.z[t]) & 1) w = -w;
      acc = fma(ts.c[t], w, acc);
    }
  }
  acc = dm_block_sum(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

template <typename S>
__global__ void __launch_bounds__(256) k_axpby(S* __restrict__ y, const S* __restrict__ x, i64 total, double a,
                                               double b) {
  const i64 stride = (i64)gridDim.x * blockDim.x;
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < total; i += stride) {
    const S xv = x[i];
    S out;
    if (b == 0.0) {  // y is not read: it may hold anything
      out.x = (decltype(out.x))(a * (double)xv.x);
      out.y = (decltype(out.y))(a * (double)xv.y);
    } else {
      const S yv = y[i];
      out.x = (decltype(out.x))fma(a, (double)xv.x, b * (double)yv.x);
      out.y = (decltype(out.y))fma(a, (double)xv.y, b * (double)yv.y);
    }
    y[i] = out;
  }
}

// qubit list of an n-qubit density matrix: in range and distinct
bool dm_qubits_ok(const int* qubits, int nq, int n, const char* who) {
  std::vector<int> seen;
  for (int i = 0; i < nq; ++i) {
    const int q = qubits[i];
    if (q < 0 || q >= n || std::find(seen.begin(), seen.end(), q) != seen.end()) {
      qgb_set_error("%s: qubit %d repeated or outside a %d-qubit density matrix", who, q, n);
      return false;
    }
    seen.push_back(q);
  }
  return true;
}

u64 dm_index_mask(u64 qmask, int n) {  // bit q = qubit q -> row-index bits
  u64 r = 0;
  for (int q = 0; q < n; ++q)
    if ((qmask >> q) & 1) r |= 1ull << (n - 1 - q);
  return r;
}

}  // namespace

extern "C" {

size_t qgb_density_scratch_bytes(void) { return (size_t)(QGB_DM_PARTS + 1) * sizeof(double); }

int qgb_density_probabilities(const void* rho, int nqubits, int dtype, const int* qubits, int nq, double* out,
                              void* scratch, void* stream) {
  (void)scratch;
  if (!rho || !out || nqubits < 1 || nqubits > QGB_DM_MAXQ || nq < 0 || nq > nqubits || (nq > 0 && !qubits) ||
      !dtype_ok(dtype)) {
    qgb_set_error("qgb_density_probabilities: bad arguments");
    return QGB_ERR_INVALID;
  }
  if (!dm_qubits_ok(qubits, nq, nqubits, "qgb_density_probabilities")) return QGB_ERR_INVALID;
  DiagGeom g;
  memset(&g, 0, sizeof(g));
  g.n = nqubits;
  g.nq = nq;
  g.u = nqubits - nq;
  for (int b = 0; b < nq; ++b) g.mpos[b] = nqubits - 1 - qubits[nq - 1 - b];
  int k = 0;
  for (int p = 0; p < nqubits; ++p) {
    bool measured = false;
    for (int b = 0; b < nq; ++b) measured = measured || g.mpos[b] == p;
    if (!measured) g.upos[k++] = p;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const i64 nout = (i64)1 << nq;
  if (g.u <= 6) {
    int blocks;
    grid_for(nout, 256, &blocks);
    if (dtype == QGB_C128) k_dm_probs_thread<TC128><<<blocks, 256, 0, s>>>((const double2*)rho, nout, g, out);
    else k_dm_probs_thread<TC64><<<blocks, 256, 0, s>>>((const float2*)rho, nout, g, out);
  } else {
    const int blocks = (int)std::min<i64>(nout, 65536);
    if (dtype == QGB_C128) k_dm_probs_block<TC128><<<blocks, 256, 0, s>>>((const double2*)rho, nout, g, out);
    else k_dm_probs_block<TC64><<<blocks, 256, 0, s>>>((const float2*)rho, nout, g, out);
  }
  QGB_LAUNCH_CHECK("k_dm_probs");
  return QGB_OK;
}

int qgb_density_collapse(void* rho, int nqubits, int dtype, const int* qubits, int nq, const int64_t* outcome,
                         int normalize, void* scratch, void* stream) {
  if (!rho || !outcome || nqubits < 1 || nqubits > QGB_DM_MAXQ || nq < 1 || nq > nqubits || !qubits ||
      !dtype_ok(dtype) || (normalize && !scratch)) {
    qgb_set_error("qgb_density_collapse: bad arguments");
    return QGB_ERR_INVALID;
  }
  if (!dm_qubits_ok(qubits, nq, nqubits, "qgb_density_collapse")) return QGB_ERR_INVALID;
  DmCollapse a;
  memset(&a, 0, sizeof(a));
  a.n = nqubits;
  a.nq = nq;
  for (int i = 0; i < nq; ++i) a.sorted[i] = a.pos[i] = nqubits - 1 - qubits[i];
  std::sort(a.sorted, a.sorted + nq);
  cudaStream_t s = (cudaStream_t)stream;
  double* trace = nullptr;
  if (normalize) {
    double* part = (double*)scratch;
    trace = part + QGB_DM_PARTS;
    const i64 nkept = (i64)1 << (nqubits - nq);
    int blocks;
    grid_for(nkept, 256, &blocks);
    blocks = std::min(blocks, QGB_DM_PARTS);
    if (dtype == QGB_C128) k_dm_kept_trace<TC128><<<blocks, 256, 0, s>>>((const double2*)rho, nkept, a, outcome, part);
    else k_dm_kept_trace<TC64><<<blocks, 256, 0, s>>>((const float2*)rho, nkept, a, outcome, part);
    QGB_LAUNCH_CHECK("k_dm_kept_trace");
    k_dm_final<<<1, 256, 0, s>>>(part, blocks, trace, 0);
    QGB_LAUNCH_CHECK("k_dm_final");
  }
  const i64 total = (i64)1 << (2 * nqubits);
  int blocks;
  grid_for(total, 256, &blocks);
  if (dtype == QGB_C128) k_dm_collapse_apply<TC128><<<blocks, 256, 0, s>>>((double2*)rho, total, a, outcome, trace);
  else k_dm_collapse_apply<TC64><<<blocks, 256, 0, s>>>((float2*)rho, total, a, outcome, trace);
  QGB_LAUNCH_CHECK("k_dm_collapse_apply");
  return QGB_OK;
}

int qgb_density_expect_pauli(const void* rho, int nqubits, int dtype, const uint64_t* xmask, const uint64_t* zmask,
                             const double* coef, int nterms, double* out, void* scratch, void* stream) {
  if (!rho || !out || !scratch || nqubits < 1 || nqubits > QGB_DM_MAXQ || nterms < 0 ||
      (nterms > 0 && (!xmask || !zmask || !coef)) || !dtype_ok(dtype)) {
    qgb_set_error("qgb_density_expect_pauli: bad arguments");
    return QGB_ERR_INVALID;
  }
  const u64 valid = nqubits >= 64 ? ~0ull : ((1ull << nqubits) - 1);
  for (int t = 0; t < nterms; ++t)
    if ((xmask[t] | zmask[t]) & ~valid) {
      qgb_set_error("qgb_density_expect_pauli: term %d acts outside a %d-qubit density matrix", t, nqubits);
      return QGB_ERR_INVALID;
    }
  cudaStream_t s = (cudaStream_t)stream;
  double* part = (double*)scratch;
  if (nterms == 0) {
    QGB_TRY_CUDA(cudaMemsetAsync(out, 0, sizeof(double), s));
    return QGB_OK;
  }
  const i64 dim = (i64)1 << nqubits;
  for (int t0 = 0; t0 < nterms; t0 += QGB_DM_TERMS) {
    DmTerms ts;
    memset(&ts, 0, sizeof(ts));
    ts.nterms = std::min(QGB_DM_TERMS, nterms - t0);
    for (int k = 0; k < ts.nterms; ++k) {
      const u64 x = dm_index_mask(xmask[t0 + k], nqubits), z = dm_index_mask(zmask[t0 + k], nqubits);
      ts.x[k] = x;
      ts.z[k] = z;
      ts.ph[k] = __builtin_popcountll(x & z) & 3;
      ts.c[k] = coef[t0 + k];
    }
    int blocks;
    grid_for(dim, 256, &blocks);
    blocks = std::min(blocks, QGB_DM_PARTS);
    if (dtype == QGB_C128) k_dm_expect<TC128><<<blocks, 256, 0, s>>>((const double2*)rho, nqubits, ts, part);
    else k_dm_expect<TC64><<<blocks, 256, 0, s>>>((const float2*)rho, nqubits, ts, part);
    QGB_LAUNCH_CHECK("k_dm_expect");
    k_dm_final<<<1, 256, 0, s>>>(part, blocks, out, t0 > 0);
    QGB_LAUNCH_CHECK("k_dm_final");
  }
  return QGB_OK;
}

int qgb_state_axpby(void* y, const void* x, int nqubits, int dtype, double a, double b, void* stream) {
  if (!y || !x || nqubits < 1 || nqubits > QGB_MAXQ || !dtype_ok(dtype)) {
    qgb_set_error("qgb_state_axpby: bad arguments");
    return QGB_ERR_INVALID;
  }
  const i64 total = (i64)1 << nqubits;
  int blocks;
  grid_for(total, 256, &blocks);
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == QGB_C128) k_axpby<double2><<<blocks, 256, 0, s>>>((double2*)y, (const double2*)x, total, a, b);
  else k_axpby<float2><<<blocks, 256, 0, s>>>((float2*)y, (const float2*)x, total, a, b);
  QGB_LAUNCH_CHECK("k_axpby");
  return QGB_OK;
}

}  // extern "C"
