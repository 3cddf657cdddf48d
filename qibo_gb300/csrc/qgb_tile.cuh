// Tile-level device code shared by the multi-gate pass kernel and the
// batched small-state serving kernel: pass traits (HBM type, tile type,
// arithmetic), the op record, and one op applied to a shared-memory tile.
#pragma once

#include "qgb_df64.cuh"
#include "qgb_plan.h"

// Pass traits: G = amplitude type in HBM, S = shared-memory tile element,
// V = value computed on.  complex64 and strict complex128 compute in their
// own precision; TC128F (qgb_df64.cuh) keeps complex128 tiles as double-float.
template <typename C, typename G_>
struct PlainPass {
  typedef G_ G;
  typedef G_ S;
  typedef G_ V;
  static V coef(double re, double im) { return C::coef(re, im); }
  __device__ static V one() { return C::coef(1.0, 0.0); }
  __device__ static V from_global(G v) { return v; }
  __device__ static G to_global(V v) { return v; }
  __device__ static V load(const S* p, int i) { return p[i]; }
  __device__ static void store(S* p, int i, V v) { p[i] = v; }
  __device__ static V mul(V a, V b) { return cmul(a, b); }
  template <int D>
  __device__ static V row(const V* u, const V* a) {
    V acc = cmul(u[0], a[0]);
#pragma unroll
    for (int c = 1; c < D; ++c) acc = cfma(u[c], a[c], acc);
    return acc;
  }
  template <int D>  // u real (imaginary parts zero)
  __device__ static V row_real(const V* u, const V* a) {
    V acc;
    acc.x = u[0].x * a[0].x;
    acc.y = u[0].x * a[0].y;
#pragma unroll
    for (int c = 1; c < D; ++c) {
      acc.x = fma(u[c].x, a[c].x, acc.x);
      acc.y = fma(u[c].x, a[c].y, acc.y);
    }
    return acc;
  }
};
typedef PlainPass<TC64, float2> P64;
typedef PlainPass<TC128, double2> P128;

// Device-only kinds set by the pass planner (qgb_blocked.cu), never by
// qgb_classify: a run of phase gates merged into one sweep, and a dense 1-
// or 2-qubit gate whose matrix is real (Hadamard, RY, ...), which needs half
// the multiplications of a complex one.
#define GK_PRUN 5
#define GK_REAL 6

struct POp {
  uint8_t kind, k;
  uint8_t tpos[5];   // tile-local target positions, most significant matrix bit first
  uint8_t pad;
  uint32_t lmask;    // tile-local bits that must be 1 (controls, phase mask)
  uint64_t gmask;    // non-local index bits that must be 1 (tested per tile)
  int32_t coef;      // offset into PassParams::coef
  int32_t pad2;
};


__device__ __forceinline__ int ins0(int j, int p) { return ((j >> p) << (p + 1)) | (j & ((1 << p) - 1)); }

template <typename T, int K, bool REAL = false>
__device__ __forceinline__ void apply_dense_tile(typename T::S* tile, int L, const POp& op,
                                                 const typename T::V* __restrict__ M) {
  constexpr int D = 1 << K;
  int sorted[K];
#pragma unroll
  for (int i = 0; i < K; ++i) sorted[i] = op.tpos[i];
#pragma unroll
  for (int a = 0; a < K; ++a)
#pragma unroll
    for (int b = a + 1; b < K; ++b)
      if (sorted[b] < sorted[a]) { int t = sorted[a]; sorted[a] = sorted[b]; sorted[b] = t; }
  int off[D];
#pragma unroll
  for (int mm = 0; mm < D; ++mm) {
    int o = 0;
#pragma unroll
    for (int i = 0; i < K; ++i)
      if ((mm >> (K - 1 - i)) & 1) o |= 1 << op.tpos[i];
    off[mm] = o;
  }
  const int groups = 1 << (L - K);
  if constexpr (K <= 2 && sizeof(typename T::V) == 8) {
    // complex64: two groups per step, so that their independent arithmetic
    // chains interleave (measured 7 % faster passes; the double-float
    // complex128 rows have too many live registers for it to pay)
    for (int g = threadIdx.x; g < groups; g += 2 * blockDim.x) {
      const int g1 = g + blockDim.x;
      const bool has1 = g1 < groups;
      int j0 = g, j1 = has1 ? g1 : g;
#pragma unroll
      for (int i = 0; i < K; ++i) {
        j0 = ins0(j0, sorted[i]);
        j1 = ins0(j1, sorted[i]);
      }
      const bool act0 = (j0 & op.lmask) == op.lmask, act1 = has1 && (j1 & op.lmask) == op.lmask;
      typename T::V v0[D], v1[D];
#pragma unroll
      for (int mm = 0; mm < D; ++mm) {
        v0[mm] = T::load(tile, j0 + off[mm]);
        v1[mm] = T::load(tile, j1 + off[mm]);
      }
#pragma unroll
      for (int r = 0; r < D; ++r) {
        typename T::V o0, o1;
        if constexpr (REAL) {
          o0 = T::template row_real<D>(M + r * D, v0);
          o1 = T::template row_real<D>(M + r * D, v1);
        } else {
          o0 = T::template row<D>(M + r * D, v0);
          o1 = T::template row<D>(M + r * D, v1);
        }
        if (act0) T::store(tile, j0 + off[r], o0);
        if (act1) T::store(tile, j1 + off[r], o1);
      }
    }
    return;
  }
  for (int g = threadIdx.x; g < groups; g += blockDim.x) {
    int j0 = g;
#pragma unroll
    for (int i = 0; i < K; ++i) j0 = ins0(j0, sorted[i]);
    if ((j0 & op.lmask) != op.lmask) continue;
    typename T::V v[D];
#pragma unroll
    for (int mm = 0; mm < D; ++mm) v[mm] = T::load(tile, j0 + off[mm]);
#pragma unroll
    for (int r = 0; r < D; ++r) {
      if constexpr (REAL) T::store(tile, j0 + off[r], T::template row_real<D>(M + r * D, v));
      else T::store(tile, j0 + off[r], T::template row<D>(M + r * D, v));
    }
  }
}

// Apply one op to a shared-memory tile of 2^L amplitudes (all threads of
// the CTA take part; the caller synchronises afterwards).
// MAXK: largest dense block the caller may pass (2 keeps the register count
// low enough for several CTAs per SM; 5 allows fused 5-qubit blocks).
template <typename T, int MAXK>
__device__ __forceinline__ void apply_tile_op(typename T::S* tile, int L, const POp& op,
                                              const typename T::V* __restrict__ M) {
  typedef typename T::S S;
  typedef typename T::V V;
  const int TN = 1 << L;
  switch (op.kind) {
    case GK_PHASE: {
      const V ph = M[0];
      for (int j = threadIdx.x; j < TN; j += blockDim.x)
        if ((j & op.lmask) == op.lmask) T::store(tile, j, T::mul(ph, T::load(tile, j)));
      break;
    }
    case GK_DIAG: {
      for (int j = threadIdx.x; j < TN; j += blockDim.x) {
        if ((j & op.lmask) != op.lmask) continue;
        int mm = 0;
        for (int i = 0; i < op.k; ++i) mm = (mm << 1) | ((j >> op.tpos[i]) & 1);
        T::store(tile, j, T::mul(M[mm], T::load(tile, j)));
      }
      break;
    }
    case GK_XLIKE: {
      const int p = op.tpos[0];
      for (int g = threadIdx.x; g < TN / 2; g += blockDim.x) {
        const int j0 = ins0(g, p), j1 = j0 | (1 << p);
        if ((j0 & op.lmask) != op.lmask) continue;
        const V a0 = T::load(tile, j0), a1 = T::load(tile, j1);
        T::store(tile, j0, T::mul(M[0], a1));
        T::store(tile, j1, T::mul(M[1], a0));
      }
      break;
    }
    case GK_SWAP: {
      const int p0 = min(op.tpos[0], op.tpos[1]), p1 = max(op.tpos[0], op.tpos[1]);
      for (int g = threadIdx.x; g < TN / 4; g += blockDim.x) {
        const int j = ins0(ins0(g, p0), p1);
        if ((j & op.lmask) != op.lmask) continue;
        const int ja = j | (1 << p0), jb = j | (1 << p1);
        const S va = tile[ja];
        tile[ja] = tile[jb];
        tile[jb] = va;
      }
      break;
    }
    case GK_REAL: {
      if (op.k == 1) apply_dense_tile<T, 1, true>(tile, L, op, M);
      else apply_dense_tile<T, 2, true>(tile, L, op, M);
      break;
    }
    default: {
      switch (op.k) {
        case 1: apply_dense_tile<T, 1>(tile, L, op, M); break;
        case 2: apply_dense_tile<T, 2>(tile, L, op, M); break;
        case 3: if constexpr (MAXK >= 3) apply_dense_tile<T, 3>(tile, L, op, M); break;
        case 4: if constexpr (MAXK >= 4) apply_dense_tile<T, 4>(tile, L, op, M); break;
        default: if constexpr (MAXK >= 5) apply_dense_tile<T, 5>(tile, L, op, M); break;
      }
    }
  }
}

