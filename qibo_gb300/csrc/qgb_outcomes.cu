// Measurement outcomes on the device: expectation values from samples and
// state collapse.
//
// * qgb_parity_counts: the reference turns shots into an expectation value
//   of a diagonal Pauli sum by weighting every observed outcome with
//   (-1)^(number of 1 bits on each term's qubits) and its frequency
//   (Backend.exp_value_diagonal_observable_symbolic_from_samples,
//   backends/abstract.py:2873-2926).  Here the samples stay on the device
//   and a warp ballot counts, per term, the samples of odd parity; integer
//   counts make the result independent of the reduction order.
// * qgb_collapse: Backend.collapse_state / _collapse_statevector
//   (backends/abstract.py:2424-2440, :3279-3304) keeps the slice of the state
//   that agrees with a measured outcome, divides it by its norm and puts
//   zeros elsewhere.  Here the outcome is read from device memory (where
//   qgb_sample wrote it), so a mid-circuit measurement needs no host round
//   trip: one kernel accumulates the kept slice's norm in FP64 (a fixed
//   two-stage reduction), a second one projects and rescales in place.
#include <algorithm>
#include <vector>

#include "qgb_common.cuh"

namespace {

struct ParityMasks {
  int nterms;
  uint64_t m[QGB_PARITY_MAX_TERMS];
};

__global__ void __launch_bounds__(256) k_parity(const int64_t* __restrict__ samples, i64 nshots,
                                                const __grid_constant__ ParityMasks pm,
                                                unsigned long long* __restrict__ odd) {
  __shared__ unsigned long long cnt[QGB_PARITY_MAX_TERMS];
  for (int t = threadIdx.x; t < pm.nterms; t += blockDim.x) cnt[t] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const i64 stride = (i64)gridDim.x * blockDim.x;
  // base is the same for every thread of the block, so the ballots below
  // always see full warps
  for (i64 base = (i64)blockIdx.x * blockDim.x; base < nshots; base += stride) {
    const i64 i = base + threadIdx.x;
    const bool valid = i < nshots;
    const uint64_t v = valid ? (uint64_t)samples[i] : 0;
    for (int t = 0; t < pm.nterms; ++t) {
      const unsigned b = __ballot_sync(0xffffffffu, valid && (__popcll(v & pm.m[t]) & 1));
      if (lane == 0 && b) atomicAdd(&cnt[t], (unsigned long long)__popc(b));
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < pm.nterms; t += blockDim.x)
    if (cnt[t]) atomicAdd(&odd[t], cnt[t]);
}

// Index bit positions of the measured qubits, in the order of qubits[]
// (qubits[0] is the most significant outcome bit), and the same positions
// ascending for inserting fixed bits.
struct CollapseArgs {
  int nq;
  int pos[QGB_MAXQ];     // pos[i] = index bit of qubits[i]
  int sorted[QGB_MAXQ];  // ascending
};

__device__ __forceinline__ void collapse_target(const CollapseArgs& a, int64_t outcome, uint64_t* mask,
                                                uint64_t* value) {
  uint64_t m = 0, v = 0;
  for (int i = 0; i < a.nq; ++i) {
    const uint64_t bit = (uint64_t)1 << a.pos[i];
    m |= bit;
    if (((uint64_t)outcome >> (a.nq - 1 - i)) & 1) v |= bit;
  }
  *mask = m;
  *value = v;
}

__device__ double block_sum(double v) {
  __shared__ double warp_part[8];
  for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) warp_part[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r += warp_part[w];
  return r;
}

// FP64 |psi|^2 summed over the kept slice: its 2^(n - nq) indices are t with
// a zero inserted at every measured position, then the outcome's bits set.
template <typename T>
__global__ void __launch_bounds__(256) k_collapse_norm(const typename T::S* __restrict__ psi, i64 nkept,
                                                       const __grid_constant__ CollapseArgs a,
                                                       const int64_t* __restrict__ outcome,
                                                       double* __restrict__ part) {
  uint64_t mask, value;
  collapse_target(a, *outcome, &mask, &value);
  typename T::Acc acc = T::acc_zero();
  const i64 stride = (i64)gridDim.x * blockDim.x;
  // four kept amplitudes per step: their loads are in flight together
  constexpr int W = 4;
  int it = 0;
  for (i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x; t < nkept; t += W * stride) {
    typename T::V v[W];
#pragma unroll
    for (int w = 0; w < W; ++w) {
      i64 idx = t + w * stride;
      if (idx >= nkept) break;
      for (int j = 0; j < a.nq; ++j) {
        const int p = a.sorted[j];
        idx = ((idx >> p) << (p + 1)) | (idx & ((((i64)1) << p) - 1));
      }
      v[w] = T::load(psi, idx | (i64)value);
    }
#pragma unroll
    for (int w = 0; w < W; ++w, ++it)
      if (t + w * stride < nkept) acc = T::acc_add(acc, v[w], it & 1);
  }
  const double sum = block_sum(T::acc_value(acc));
  if (threadIdx.x == 0) part[blockIdx.x] = sum;
}

__global__ void k_collapse_final(const double* __restrict__ part, int nparts, double* __restrict__ out) {
  double acc = 0.0;
  for (int p = threadIdx.x; p < nparts; p += blockDim.x) acc += part[p];
  acc = block_sum(acc);
  if (threadIdx.x == 0) *out = acc;
}

// Kept amplitudes times 1/sqrt(norm^2) (1 without normalisation), others 0.
// As in the reference, a slice of norm 0 divides 0 by 0 (NaN).
template <typename T>
__global__ void __launch_bounds__(256) k_collapse_apply(typename T::S* __restrict__ psi, i64 N,
                                                        const __grid_constant__ CollapseArgs a,
                                                        const int64_t* __restrict__ outcome,
                                                        const double* __restrict__ norm2) {
  uint64_t mask, value;
  collapse_target(a, *outcome, &mask, &value);
  const double inv = norm2 ? 1.0 / sqrt(*norm2) : 1.0;
  const i64 stride = (i64)gridDim.x * blockDim.x;
  // four amplitudes per step: the loads of the kept ones are in flight
  // together before any store waits on them
  constexpr int W = 4;
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < N; i += W * stride) {
    typename T::V v[W];
#pragma unroll
    for (int w = 0; w < W; ++w) {
      const i64 j = i + w * stride;
      v[w] = j < N && ((uint64_t)j & mask) == value ? T::scale(T::load(psi, j), inv) : T::zero();
    }
#pragma unroll
    for (int w = 0; w < W; ++w)
      if (i + w * stride < N) T::store(psi, i + w * stride, v[w]);
  }
}

}  // namespace

extern "C" size_t qgb_norm_scratch_bytes(void);  // qgb_measure.cu: the collapse scratch is that size

extern "C" {

int qgb_parity_counts(const int64_t* samples, int64_t nshots, const uint64_t* masks, int nterms, int64_t* odd,
                      void* stream) {
  if (nshots < 0 || nterms < 0 || nterms > QGB_PARITY_MAX_TERMS || (nterms > 0 && (!masks || !odd)) ||
      (nshots > 0 && !samples)) {
    qgb_set_error("qgb_parity_counts: bad arguments (nterms %d, at most %d)", nterms, QGB_PARITY_MAX_TERMS);
    return QGB_ERR_INVALID;
  }
  if (nterms == 0) return QGB_OK;
  cudaStream_t s = (cudaStream_t)stream;
  QGB_TRY_CUDA(cudaMemsetAsync(odd, 0, sizeof(int64_t) * nterms, s));
  if (nshots == 0) return QGB_OK;
  ParityMasks pm;
  pm.nterms = nterms;
  for (int t = 0; t < nterms; ++t) pm.m[t] = masks[t];
  int blocks;
  grid_for(nshots, 256, &blocks);
  k_parity<<<blocks, 256, 0, s>>>(samples, nshots, pm, (unsigned long long*)odd);
  QGB_LAUNCH_CHECK("k_parity");
  return QGB_OK;
}

int qgb_collapse(void* state, int nqubits, int dtype, const int* qubits, int nq, const int64_t* outcome,
                 int normalize, void* scratch, void* stream) {
  if (!state || !outcome || nqubits < 1 || nqubits > QGB_MAXQ || nq < 1 || nq > nqubits || !qubits ||
      !dtype_ok(dtype) || (normalize && !scratch)) {
    qgb_set_error("qgb_collapse: bad arguments");
    return QGB_ERR_INVALID;
  }
  CollapseArgs a;
  a.nq = nq;
  std::vector<int> seen;
  for (int i = 0; i < nq; ++i) {
    const int q = qubits[i];
    if (q < 0 || q >= nqubits || std::find(seen.begin(), seen.end(), q) != seen.end()) {
      qgb_set_error("qgb_collapse: qubit %d repeated or outside a %d-qubit state", q, nqubits);
      return QGB_ERR_INVALID;
    }
    seen.push_back(q);
    a.pos[i] = nqubits - 1 - q;
    a.sorted[i] = a.pos[i];
  }
  std::sort(a.sorted, a.sorted + nq);
  cudaStream_t s = (cudaStream_t)stream;
  const i64 N = (i64)1 << nqubits;
  double* norm2 = nullptr;
  if (normalize) {
    const int cap = (int)(qgb_norm_scratch_bytes() / sizeof(double));  // partial sums, then the total
    const i64 nkept = N >> nq;
    int blocks;
    grid_for(nkept, 256, &blocks);
    if (blocks > cap - 1) blocks = cap - 1;
    double* part = (double*)scratch;
    norm2 = part + cap - 1;
    if (dtype == QGB_C128) k_collapse_norm<TC128><<<blocks, 256, 0, s>>>((const double2*)state, nkept, a, outcome, part);
    else k_collapse_norm<TC64><<<blocks, 256, 0, s>>>((const float2*)state, nkept, a, outcome, part);
    QGB_LAUNCH_CHECK("k_collapse_norm");
    k_collapse_final<<<1, 256, 0, s>>>(part, blocks, norm2);
    QGB_LAUNCH_CHECK("k_collapse_final");
  }
  int blocks;
  grid_for(N, 256, &blocks);
  if (dtype == QGB_C128) k_collapse_apply<TC128><<<blocks, 256, 0, s>>>((double2*)state, N, a, outcome, norm2);
  else k_collapse_apply<TC64><<<blocks, 256, 0, s>>>((float2*)state, N, a, outcome, norm2);
  QGB_LAUNCH_CHECK("k_collapse_apply");
  return QGB_OK;
}

}  // extern "C"
