// Adjoint-method gradients of <psi(theta)|H|psi(theta)> for a Pauli-sum H.
//
// The reference has no adjoint differentiation: its gradients are the
// parameter-shift rule (derivative.py:7-156, two full circuit runs per
// parameter) and finite differences (derivative.py:159-226); its backprop
// lives in an external package.  Here, with psi_L = U_L...U_1|psi_0> and
// lambda_L = H psi_L, one reverse sweep gives every parameter derivative:
//   for k = L..1:  psi_{k-1} = U_k^dagger psi_k
//                  dE/dtheta = 2 Re <lambda_k| (dU_k/dtheta) psi_{k-1}>
//                  lambda_{k-1} = U_k^dagger lambda_k
// (Jones & Gacon, arXiv:2009.02823).  Each parametrised gate is one fused
// pass that reads and writes both states and reduces its (up to 3)
// derivative inner products per CTA; partial sums are reduced in a fixed
// order, so results are deterministic.
#include <algorithm>
#include <cstdlib>
#include <map>
#include <vector>

#include <type_traits>

#include "qgb_df64.cuh"
#include "qgb_plan.h"

int qgb_launch_gateop(void* state, int n, int dtype, const GateOp& g, cudaStream_t s);  // qgb_gates.cu

namespace {
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// deterministic block sum (256 threads): result valid in thread 0
__device__ double block_sum_d(double v, double* sh) {
  v = warp_sum_d(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x < 32) {
    r = (l < 8) ? sh[l] : 0.0;
    r = warp_sum_d(r);
  }
  __syncthreads();
  return r;
}
}  // namespace

// ------------------------------------------------------ H|psi> for Pauli sums --
#define QGB_PS_MAX_GROUPS 64
#define QGB_PS_MAX_TERMS 256

struct PauliSum {
  int ngroups;
  int gstart[QGB_PS_MAX_GROUPS + 1];  // term range of each flip-mask group
  u64 gx[QGB_PS_MAX_GROUPS];          // index-space flip mask of the group
  u64 z[QGB_PS_MAX_TERMS];            // index-space phase masks
  double cre[QGB_PS_MAX_TERMS];       // coef * i^ny, real and imaginary parts
  double cim[QGB_PS_MAX_TERMS];
};

// dst_i = sum_t c_t i^ny_t (-1)^popc((i^x_t) & z_t) src_{i ^ x_t}
template <typename T>
__global__ void __launch_bounds__(256) k_pauli_sum(const typename T::S* __restrict__ src, typename T::S* __restrict__ dst,
                                                   i64 N, const __grid_constant__ PauliSum P) {
  const i64 stride = (i64)gridDim.x * blockDim.x;
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < N; i += stride) {
    double re = 0.0, im = 0.0;
    for (int g = 0; g < P.ngroups; ++g) {
      const i64 j = i ^ (i64)P.gx[g];
      const typename T::V a = T::load(src, j);
      double wr = 0.0, wi = 0.0;
      for (int t = P.gstart[g]; t < P.gstart[g + 1]; ++t) {
        const double s = (__popcll((u64)j & P.z[t]) & 1) ? -1.0 : 1.0;
        wr += s * P.cre[t];
        wi += s * P.cim[t];
      }
      re += wr * T::re(a) - wi * T::im(a);
      im += wr * T::im(a) + wi * T::re(a);
    }
    T::store(dst, i, T::coef(re, im));
  }
}

// <a|b> partial sums (re, im) per block
template <typename T>
__global__ void __launch_bounds__(256) k_inner(const typename T::S* __restrict__ a, const typename T::S* __restrict__ b,
                                               i64 N, double* __restrict__ part) {
  __shared__ double sh[8];
  double re = 0.0, im = 0.0;
  const i64 stride = (i64)gridDim.x * blockDim.x;
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < N; i += stride) {
    const typename T::V x = T::load(a, i), y = T::load(b, i);
    re += T::re(x) * T::re(y) + T::im(x) * T::im(y);
    im += T::re(x) * T::im(y) - T::im(x) * T::re(y);
  }
  re = block_sum_d(re, sh);
  im = block_sum_d(im, sh);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = re;
    part[2 * blockIdx.x + 1] = im;
  }
}

// <a|b> for states of different precision (complex128 vs complex64)
template <typename TA, typename TB>
__global__ void __launch_bounds__(256) k_inner2(const typename TA::S* __restrict__ a, const typename TB::S* __restrict__ b,
                                                i64 N, double* __restrict__ part) {
  __shared__ double sh[8];
  double re = 0.0, im = 0.0;
  const i64 stride = (i64)gridDim.x * blockDim.x;
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < N; i += stride) {
    const typename TA::V x = TA::load(a, i);
    const typename TB::V y = TB::load(b, i);
    re += TA::re(x) * TB::re(y) + TA::im(x) * TB::im(y);
    im += TA::re(x) * TB::im(y) - TA::im(x) * TB::re(y);
  }
  re = block_sum_d(re, sh);
  im = block_sum_d(im, sh);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = re;
    part[2 * blockIdx.x + 1] = im;
  }
}

// out[k] = sum_b part[b * stride + k] for k < nout, fixed order
__global__ void k_reduce_cols(const double* __restrict__ part, int nrows, int stride, int nout, double* __restrict__ out,
                              double scale) {
  __shared__ double sh[8];
  for (int k = 0; k < nout; ++k) {
    double acc = 0.0;
    for (int b = threadIdx.x; b < nrows; b += blockDim.x) acc += part[(i64)b * stride + k];
    acc = block_sum_d(acc, sh);
    if (threadIdx.x == 0) out[k] = scale * acc;
  }
}

// ------------------------------------------------------------ adjoint step --
struct Offs5 {
  i64 o[32];
};

template <typename T, int K>
struct AdjMats {
  typename T::V udag[1 << K][1 << K];
  typename T::V der[3][1 << K][1 << K];
};

// one parametrised gate of the reverse sweep (see the file comment)
template <typename T, int K>
__global__ void __launch_bounds__(256) k_adjoint_step(typename T::S* __restrict__ psi, typename T::S* __restrict__ lam,
                                                      i64 ngroups, const __grid_constant__ BitInsert bi, i64 cmask, Offs5 off, int nder,
                                                      const __grid_constant__ AdjMats<T, K> M, double* __restrict__ part,
                                                      int part_stride) {
  constexpr int D = 1 << K;
  __shared__ double sh[8];
  double acc[3] = {0.0, 0.0, 0.0};
  const i64 stride = (i64)gridDim.x * blockDim.x;
  for (i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x; t < ngroups; t += stride) {
    const i64 base = insert_zeros(t, bi) | cmask;
    typename T::V v[D], w[D], vp[D];
#pragma unroll
    for (int m = 0; m < D; ++m) {
      v[m] = T::load(psi, base + off.o[m]);
      w[m] = T::load(lam, base + off.o[m]);
    }
#pragma unroll
    for (int r = 0; r < D; ++r) {
      typename T::V a = T::mul(M.udag[r][0], v[0]);
#pragma unroll
      for (int c = 1; c < D; ++c) a = T::fma(M.udag[r][c], v[c], a);
      vp[r] = a;
    }
    for (int d = 0; d < nder; ++d) {
#pragma unroll
      for (int r = 0; r < D; ++r) {
        typename T::V mu = T::mul(M.der[d][r][0], vp[0]);
#pragma unroll
        for (int c = 1; c < D; ++c) mu = T::fma(M.der[d][r][c], vp[c], mu);
        acc[d] += T::re(w[r]) * T::re(mu) + T::im(w[r]) * T::im(mu);  // Re(conj(w) mu)
      }
    }
#pragma unroll
    for (int r = 0; r < D; ++r) {
      typename T::V a = T::mul(M.udag[r][0], w[0]);
#pragma unroll
      for (int c = 1; c < D; ++c) a = T::fma(M.udag[r][c], w[c], a);
      T::store(lam, base + off.o[r], a);
      T::store(psi, base + off.o[r], vp[r]);
    }
  }
  for (int d = 0; d < nder; ++d) {
    const double s = block_sum_d(acc[d], sh);
    if (threadIdx.x == 0) part[(i64)blockIdx.x * part_stride + d] = s;
  }
}

// Complex128 parametrised 1-qubit gates: the step's three complex 2x2
// products per amplitude pair (U^dagger psi, the derivatives, U^dagger
// lambda) bound an IEEE FP64 form by GB300's FP64 pipe, so the pairs are
// shared as in k_1q_pairs_mix: warps 0-3 (one per scheduler) of every other
// block compute in IEEE FP64, the others in double-float (error-free row
// products, the derivative inner products accumulated in double-float and
// flushed to FP64 per thread).  Which thread handles which pair, and the
// order of the partial sums, do not depend on the split.
template <typename T>
__device__ __forceinline__ void adj_pairs(typename T::S* __restrict__ psi, typename T::S* __restrict__ lam,
                                          i64 ngroups, const BitInsert& bi, i64 cmask, const Offs5& off, int nder,
                                          const AdjMats<T, 1>& M, double acc_out[3]) {
  constexpr bool kDF = std::is_same<T, DF128>::value;
  const i64 stride = (i64)gridDim.x * blockDim.x;
  double acc[3] = {0.0, 0.0, 0.0};
  DFAcc dacc[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
  for (i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x; t < ngroups; t += stride) {
    const i64 base = insert_zeros(t, bi) | cmask;
    const typename T::V v0 = T::load(psi, base + off.o[0]), v1 = T::load(psi, base + off.o[1]);
    const typename T::V w0 = T::load(lam, base + off.o[0]), w1 = T::load(lam, base + off.o[1]);
    const typename T::V p0 = T::row2(M.udag[0][0], v0, M.udag[0][1], v1);
    const typename T::V p1 = T::row2(M.udag[1][0], v0, M.udag[1][1], v1);
#pragma unroll
    for (int d = 0; d < 3; ++d) {  // unrolled: the accumulators stay in registers
      if (d >= nder) break;
      const typename T::V m0 = T::row2(M.der[d][0][0], p0, M.der[d][0][1], p1);
      const typename T::V m1 = T::row2(M.der[d][1][0], p0, M.der[d][1][1], p1);
      if constexpr (kDF) {  // Re(conj(w0) m0) + Re(conj(w1) m1), one error-free dot product
        const df x[4] = {w0.re, w0.im, w1.re, w1.im}, y[4] = {m0.re, m0.im, m1.re, m1.im};
        const float sx[4] = {1.f, 1.f, 1.f, 1.f};
        const df r = df_dot<4>(x, y, sx);
        dacc[d] = df_add2(dacc[d], r.hi, r.lo);
      } else {
        acc[d] += T::re(w0) * T::re(m0) + T::im(w0) * T::im(m0) + T::re(w1) * T::re(m1) + T::im(w1) * T::im(m1);
      }
    }
    T::store(lam, base + off.o[0], T::row2(M.udag[0][0], w0, M.udag[0][1], w1));
    T::store(lam, base + off.o[1], T::row2(M.udag[1][0], w0, M.udag[1][1], w1));
    T::store(psi, base + off.o[0], p0);
    T::store(psi, base + off.o[1], p1);
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) acc_out[d] = kDF ? f2d_exact(dacc[d].hi) + f2d_exact(dacc[d].lo) : acc[d];
}

__global__ void __launch_bounds__(256) k_adjoint_step_mix(double2* __restrict__ psi, double2* __restrict__ lam,
                                                          i64 ngroups, const __grid_constant__ BitInsert bi,
                                                          i64 cmask, Offs5 off, int nder,
                                                          const __grid_constant__ AdjMats<TC128, 1> Me,
                                                          const __grid_constant__ AdjMats<DF128, 1> Md,
                                                          double* __restrict__ part, int part_stride) {
  __shared__ double sh[8];
  double acc[3];
  if ((threadIdx.x >> 7) == 0 && (blockIdx.x & 1) == 0) adj_pairs<TC128>(psi, lam, ngroups, bi, cmask, off, nder, Me, acc);
  else adj_pairs<DF128>(psi, lam, ngroups, bi, cmask, off, nder, Md, acc);
  for (int d = 0; d < nder; ++d) {
    const double s = block_sum_d(acc[d], sh);
    if (threadIdx.x == 0) part[(i64)blockIdx.x * part_stride + d] = s;
  }
}

namespace {
const int kAdjBlocks = 4 * 152;

i64 mask_bits(const std::vector<int>& b) {
  i64 m = 0;
  for (int x : b) m |= (i64)1 << x;
  return m;
}

u64 idx_mask(u64 qmask, int n) {
  u64 r = 0;
  for (int q = 0; q < n; ++q)
    if ((qmask >> q) & 1) r |= 1ull << (n - 1 - q);
  return r;
}

template <typename T, int K>
int adjoint_step(void* psi, void* lam, int n, const GateOp& g, int nder, const double* const* ders, double* part,
                 int part_stride, cudaStream_t s) {
  constexpr int D = 1 << K;
  AdjMats<T, K>* M = new AdjMats<T, K>();
  for (int r = 0; r < D; ++r)
    for (int c = 0; c < D; ++c) {
      M->udag[r][c] = T::coef(g.coef[r * D + c].real(), g.coef[r * D + c].imag());
      for (int d = 0; d < 3; ++d)
        M->der[d][r][c] = d < nder ? T::coef(ders[d][2 * (r * D + c)], ders[d][2 * (r * D + c) + 1]) : T::coef(0, 0);
    }
  std::vector<int> fixed = g.tbits;
  fixed.insert(fixed.end(), g.cbits.begin(), g.cbits.end());
  BitInsert bi;
  std::sort(fixed.begin(), fixed.end());
  bi.n = (int)fixed.size();
  for (int j = 0; j < bi.n; ++j) bi.pos[j] = fixed[j];
  Offs5 off;
  for (int m = 0; m < 32; ++m) {
    i64 o = 0;
    if (m < D)
      for (int j = 0; j < K; ++j)
        if ((m >> (K - 1 - j)) & 1) o |= (i64)1 << g.tbits[j];
    off.o[m] = o;
  }
  const i64 ngroups = (i64)1 << (n - bi.n);
  int blocks;
  grid_for(ngroups, 256, &blocks);
  blocks = std::min(blocks, kAdjBlocks);
  typedef typename T::S S;
  if constexpr (std::is_same<T, TC128>::value && K == 1) {
    const char* strict = getenv("QIBO_GB300_STRICT_FP64");
    if (!(strict && strict[0] == '1' && strict[1] == 0)) {  // the FP64 / double-float warp split
      AdjMats<DF128, 1>* Md = new AdjMats<DF128, 1>();
      for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 2; ++c) {
          Md->udag[r][c] = DF128::coef(g.coef[r * 2 + c].real(), g.coef[r * 2 + c].imag());
          for (int d = 0; d < 3; ++d)
            Md->der[d][r][c] = d < nder ? DF128::coef(ders[d][2 * (r * 2 + c)], ders[d][2 * (r * 2 + c) + 1])
                                        : DF128::coef(0, 0);
        }
      k_adjoint_step_mix<<<blocks, 256, 0, s>>>((double2*)psi, (double2*)lam, ngroups, bi, mask_bits(g.cbits), off,
                                                nder, *M, *Md, part, part_stride);
      delete Md;
      delete M;
      QGB_LAUNCH_CHECK("k_adjoint_step_mix");
      return QGB_OK;
    }
  }
  k_adjoint_step<T, K><<<blocks, 256, 0, s>>>((S*)psi, (S*)lam, ngroups, bi, mask_bits(g.cbits), off, nder, *M,
                                             part, part_stride);
  delete M;
  QGB_LAUNCH_CHECK("k_adjoint_step");
  return QGB_OK;
}
}  // namespace

extern "C" {

int qgb_apply_pauli_sum(const void* src, void* dst, int nqubits, int dtype, const uint64_t* xmask,
                        const uint64_t* zmask, const double* coef, int nterms, void* stream) {
  if (!src || !dst || src == dst || nqubits < 1 || nqubits > 63 || !dtype_ok(dtype) || nterms < 0 ||
      nterms > QGB_PS_MAX_TERMS || (nterms && (!xmask || !zmask || !coef))) {
    qgb_set_error("qgb_apply_pauli_sum: bad arguments (distinct buffers, at most %d terms)", QGB_PS_MAX_TERMS);
    return QGB_ERR_INVALID;
  }
  std::map<u64, std::vector<int>> groups;
  for (int t = 0; t < nterms; ++t) {
    if ((xmask[t] | zmask[t]) >> nqubits) { qgb_set_error("qgb_apply_pauli_sum: term %d out of range", t); return QGB_ERR_INVALID; }
    groups[xmask[t]].push_back(t);
  }
  if ((int)groups.size() > QGB_PS_MAX_GROUPS) {
    qgb_set_error("qgb_apply_pauli_sum: %d distinct X/Y patterns (max %d)", (int)groups.size(), QGB_PS_MAX_GROUPS);
    return QGB_ERR_UNSUPPORTED;
  }
  PauliSum* P = new PauliSum();
  int k = 0, g = 0;
  for (auto& kv : groups) {
    P->gx[g] = idx_mask(kv.first, nqubits);
    P->gstart[g] = k;
    for (int t : kv.second) {
      const u64 z = idx_mask(zmask[t], nqubits), x = idx_mask(xmask[t], nqubits);
      const int ny = __builtin_popcountll(x & z) & 3;
      // i^ny
      const double pr[4] = {1, 0, -1, 0}, pi[4] = {0, 1, 0, -1};
      P->z[k] = z;
      P->cre[k] = coef[t] * pr[ny];
      P->cim[k] = coef[t] * pi[ny];
      ++k;
    }
    ++g;
  }
  P->gstart[g] = k;
  P->ngroups = g;
  const i64 N = (i64)1 << nqubits;
  int blocks;
  grid_for(N, 256, &blocks);
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == QGB_C128) k_pauli_sum<TC128><<<blocks, 256, 0, s>>>((const double2*)src, (double2*)dst, N, *P);
  else k_pauli_sum<TC64><<<blocks, 256, 0, s>>>((const float2*)src, (float2*)dst, N, *P);
  delete P;
  QGB_LAUNCH_CHECK("k_pauli_sum");
  return QGB_OK;
}

size_t qgb_inner_scratch_bytes(void) { return (size_t)2 * kAdjBlocks * sizeof(double); }

int qgb_inner(const void* a, const void* b, int nqubits, int dtype, double* out, void* scratch, void* stream) {
  if (!a || !b || !out || !scratch || nqubits < 1 || nqubits > QGB_MAXQ || !dtype_ok(dtype)) {
    qgb_set_error("qgb_inner: bad arguments");
    return QGB_ERR_INVALID;
  }
  const i64 N = (i64)1 << nqubits;
  int blocks;
  grid_for(N, 256, &blocks);
  blocks = std::min(blocks, kAdjBlocks);
  cudaStream_t s = (cudaStream_t)stream;
  double* part = (double*)scratch;
  if (dtype == QGB_C128) k_inner<TC128><<<blocks, 256, 0, s>>>((const double2*)a, (const double2*)b, N, part);
  else k_inner<TC64><<<blocks, 256, 0, s>>>((const float2*)a, (const float2*)b, N, part);
  QGB_LAUNCH_CHECK("k_inner");
  k_reduce_cols<<<1, 256, 0, s>>>(part, blocks, 2, 2, out, 1.0);
  QGB_LAUNCH_CHECK("k_reduce_cols");
  return QGB_OK;
}

int qgb_inner_mixed(const void* a, int dtype_a, const void* b, int dtype_b, int nqubits, double* out, void* scratch,
                    void* stream) {
  if (!a || !b || !out || !scratch || nqubits < 1 || nqubits > QGB_MAXQ || !dtype_ok(dtype_a) || !dtype_ok(dtype_b)) {
    qgb_set_error("qgb_inner_mixed: bad arguments");
    return QGB_ERR_INVALID;
  }
  if (dtype_a == dtype_b) return qgb_inner(a, b, nqubits, dtype_a, out, scratch, stream);
  const i64 N = (i64)1 << nqubits;
  int blocks;
  grid_for(N, 256, &blocks);
  blocks = std::min(blocks, kAdjBlocks);
  cudaStream_t s = (cudaStream_t)stream;
  double* part = (double*)scratch;
  if (dtype_a == QGB_C128)
    k_inner2<TC128, TC64><<<blocks, 256, 0, s>>>((const double2*)a, (const float2*)b, N, part);
  else
    k_inner2<TC64, TC128><<<blocks, 256, 0, s>>>((const float2*)a, (const double2*)b, N, part);
  QGB_LAUNCH_CHECK("k_inner2");
  k_reduce_cols<<<1, 256, 0, s>>>(part, blocks, 2, 2, out, 1.0);
  QGB_LAUNCH_CHECK("k_reduce_cols");
  return QGB_OK;
}

size_t qgb_adjoint_scratch_bytes(int nparams) { return (size_t)kAdjBlocks * std::max(nparams, 1) * sizeof(double); }

int qgb_adjoint_sweep(void* psi, void* lam, int nqubits, int dtype, const qgb_op* ops, int nops, const double* coefs,
                      const int* nder, const int64_t* der_offset, const int* grad_index, int nparams, double* grads,
                      void* scratch, void* stream) {
  if (!psi || !lam || psi == lam || nops < 0 || (nops && (!ops || !coefs || !nder || !der_offset || !grad_index)) ||
      !grads || !scratch || nparams < 0 || !dtype_ok(dtype)) {
    qgb_set_error("qgb_adjoint_sweep: bad arguments");
    return QGB_ERR_INVALID;
  }
  cudaStream_t s = (cudaStream_t)stream;
  double* part = (double*)scratch;
  QGB_TRY_CUDA(cudaMemsetAsync(part, 0, (size_t)kAdjBlocks * std::max(nparams, 1) * sizeof(double), s));
  for (int i = 0; i < nops; ++i) {
    GateOp g;
    int st = qgb_classify(nqubits, ops[i].qubits, ops[i].k, ops[i].controls, ops[i].ncontrols, coefs + ops[i].coef_offset,
                          &g, "qgb_adjoint_sweep");
    if (st) return st;
    if (nder[i] == 0) {
      st = qgb_launch_gateop(psi, nqubits, dtype, g, s);
      if (st) return st;
      st = qgb_launch_gateop(lam, nqubits, dtype, g, s);
      if (st) return st;
      continue;
    }
    if (nder[i] < 0 || nder[i] > 3 || grad_index[i] < 0 || grad_index[i] + nder[i] > nparams) {
      qgb_set_error("qgb_adjoint_sweep: op %d has a bad parameter slot", i);
      return QGB_ERR_INVALID;
    }
    // the derivative kernel works on the dense form over the given qubits
    GateOp d;
    d.kind = GK_DENSE;
    for (int j = 0; j < ops[i].k; ++j) d.tbits.push_back(nqubits - 1 - ops[i].qubits[j]);
    for (int j = 0; j < ops[i].ncontrols; ++j) d.cbits.push_back(nqubits - 1 - ops[i].controls[j]);
    const int D = 1 << ops[i].k;
    d.coef.resize(D * D);
    const double* u = coefs + ops[i].coef_offset;
    for (int e = 0; e < D * D; ++e) d.coef[e] = zd(u[2 * e], u[2 * e + 1]);
    const double* ders[3] = {nullptr, nullptr, nullptr};
    for (int j = 0; j < nder[i]; ++j) ders[j] = coefs + der_offset[i] + (i64)j * 2 * D * D;
    double* p = part + grad_index[i];
    if (ops[i].k == 1)
      st = dtype == QGB_C128 ? adjoint_step<TC128, 1>(psi, lam, nqubits, d, nder[i], ders, p, nparams, s)
                             : adjoint_step<TC64, 1>(psi, lam, nqubits, d, nder[i], ders, p, nparams, s);
    else if (ops[i].k == 2)
      st = dtype == QGB_C128 ? adjoint_step<TC128, 2>(psi, lam, nqubits, d, nder[i], ders, p, nparams, s)
                             : adjoint_step<TC64, 2>(psi, lam, nqubits, d, nder[i], ders, p, nparams, s);
    else {
      qgb_set_error("qgb_adjoint_sweep: parametrised gates on %d qubits are not supported (max 2)", ops[i].k);
      return QGB_ERR_UNSUPPORTED;
    }
    if (st) return st;
  }
  k_reduce_cols<<<1, 256, 0, s>>>(part, kAdjBlocks, nparams, nparams, grads, 2.0);
  QGB_LAUNCH_CHECK("k_reduce_cols");
  return QGB_OK;
}

}  // extern "C"
