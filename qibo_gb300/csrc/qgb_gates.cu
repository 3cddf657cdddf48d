// Gate application: the GB300 replacement of Backend.apply_gate
// (backends/abstract.py:2322-2361) and Backend._apply_gate_controlled_by
// (backends/abstract.py:3176-3197).
//
// The reference moves the gate's qubit axes to the front with a transpose
// (a full copy), multiplies by the 2^k x 2^k matrix and transposes back.
// Here every gate is one in-place pass over only the amplitudes it changes:
//   * dense k-qubit gates gather the 2^k amplitudes of a group, multiply
//     and scatter back (k = 1 with a warp-shuffle variant for low bits);
//   * diagonal gates whose only non-unit entry sits on the all-ones corner
//     (CZ, CU1, CCZ, S, T, Z, U1 and controlled versions) multiply a phase
//     into 2^(n-c) amplitudes only;
//   * other diagonal gates (RZ, RZZ, CRZ) scale in place;
//   * X-like gates (X, Y, CNOT, CY, TOFFOLI) and SWAP move data only.
// The host-side classifier (``qgb_apply_gate``) finds "hidden" controls in
// a matrix (an axis on which the matrix is the identity when that qubit is
// 0), so CU1 / CNOT / TOFFOLI / CZ given as full matrices take the cheap
// kernels.
#include <algorithm>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <vector>

#include "qgb_df64.cuh"
#include "qgb_plan.h"

template <int K>
struct Offs { i64 o[1 << K]; };

template <typename T, int K>
struct DenseMat { typename T::V m[1 << K][1 << K]; };

// ---------------------------------------------------------------------------
// dense k-qubit gate with optional controls (generic)
template <typename T, int K>
__global__ void __launch_bounds__(256) k_dense(typename T::S* __restrict__ psi, i64 ngroups, BitInsert bi,
                                               i64 cmask, Offs<K> off, DenseMat<T, K> M) {
  constexpr int D = 1 << K;
  const i64 stride = (i64)gridDim.x * blockDim.x;
  for (i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x; t < ngroups; t += stride) {
    const i64 base = insert_zeros(t, bi) | cmask;
    typename T::V v[D];
#pragma unroll
    for (int m = 0; m < D; ++m) v[m] = T::load(psi, base + off.o[m]);
#pragma unroll
    for (int r = 0; r < D; ++r) {
      typename T::V acc = T::mul(M.m[r][0], v[0]);
#pragma unroll
      for (int c = 1; c < D; ++c) acc = T::fma(M.m[r][c], v[c], acc);
      T::store(psi, base + off.o[r], acc);
    }
  }
}

// dense 1-qubit gate, no controls, target bit >= 5: independent pairs,
// coalesced 16-byte (c128) / 8-byte (c64) accesses, two pairs per thread.
template <typename T>
__device__ __forceinline__ void pairs_body(typename T::S* __restrict__ psi, i64 npairs, int b, typename T::V u00,
                                           typename T::V u01, typename T::V u10, typename T::V u11) {
  const i64 stride = (i64)gridDim.x * blockDim.x;
  const i64 lowmask = ((i64)1 << b) - 1;
  const i64 step = (i64)1 << b;
  for (i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x; t < npairs; t += 2 * stride) {
    const i64 t2 = t + stride;
    const i64 i0 = ((t >> b) << (b + 1)) | (t & lowmask);
    const bool has2 = t2 < npairs;
    const i64 j0 = ((t2 >> b) << (b + 1)) | (t2 & lowmask);
    typename T::V a0 = T::load(psi, i0), a1 = T::load(psi, i0 + step);
    typename T::V c0, c1;
    if (has2) { c0 = T::load(psi, j0); c1 = T::load(psi, j0 + step); }
    T::store(psi, i0, T::row2(u00, a0, u01, a1));
    T::store(psi, i0 + step, T::row2(u10, a0, u11, a1));
    if (has2) {
      T::store(psi, j0, T::row2(u00, c0, u01, c1));
      T::store(psi, j0 + step, T::row2(u10, c0, u11, c1));
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_1q_pairs(typename T::S* __restrict__ psi, i64 npairs, int b,
                                                  typename T::V u00, typename T::V u01,
                                                  typename T::V u10, typename T::V u11) {
  pairs_body<T>(psi, npairs, b, u00, u01, u10, u11);
}

// complex128 gate by gate, the two arithmetic pipes at once: some warps
// compute their pairs in IEEE FP64 (the FP64 pipe, 16 DFMA per pair), the
// others in double-float (FP32 and integer pipes only).  Alone, the FP64
// form is bound by GB300's FP64 rate and the double-float form by
// instruction issue; sharing the pairs between them keeps both pipes busy.
// A block has 1024 threads, one per SM: warp w issues from scheduler w mod 4
// as the (w / 4)-th of that scheduler's eight warps, and the first nf64 of
// each scheduler's eight take the FP64 form, so all four schedulers (each
// with its own FP64 units) carry the same share.  Which warp computes which
// pair does not depend on nf64, and both forms are accurate to a few units
// in the last place of FP64.
//
// Loads go through a ring of MIX_STAGES slots per thread in shared memory,
// filled by cp.async (16 bytes per copy, no registers held), MIX_STAGES - 1
// steps ahead of the arithmetic: every thread reads back only its own
// slots, after cp.async.wait_group has seen its own copies land, so no
// barrier is needed.  A slot is refilled one step after it was read into
// registers, and stores go straight from registers to the state.
#define MIX_THREADS 1024
#define MIX_STAGES 4
struct Coef1q {
  cdf d[4];      // double-float u00, u01, u10, u11
  double2 e[4];  // the same in FP64
};

__device__ __forceinline__ bool mix_fp64_warp(int nf64) { return (int)(threadIdx.x >> 7) < nf64; }

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
               "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

extern __shared__ __align__(16) double2 mix_ring[];

// pairs_body through the ring: slot k of a thread holds its pair's two
// amplitudes at mix_ring[(2 k + h) MIX_THREADS + thread]
template <typename T>
__device__ __forceinline__ void pairs_ring_body(double2* __restrict__ psi, i64 npairs, int b, typename T::V u00,
                                                typename T::V u01, typename T::V u10, typename T::V u11) {
  const i64 stride = (i64)gridDim.x * MIX_THREADS;
  const i64 lowmask = ((i64)1 << b) - 1, step = (i64)1 << b;
  const i64 t0 = (i64)blockIdx.x * MIX_THREADS + threadIdx.x;
  double2* const slot = mix_ring + threadIdx.x;
  const auto fetch = [&](i64 t, int k) {
    if (t < npairs) {
      const i64 i0 = ((t >> b) << (b + 1)) | (t & lowmask);
      cp_async16(slot + (2 * k) * MIX_THREADS, psi + i0);
      cp_async16(slot + (2 * k + 1) * MIX_THREADS, psi + i0 + step);
    }
    cp_async_commit();
  };
#pragma unroll
  for (int k = 0; k < MIX_STAGES - 1; ++k) fetch(t0 + k * stride, k);
  int k = 0;
  for (i64 t = t0; t < npairs; t += stride) {
    cp_async_wait<MIX_STAGES - 2>();  // slot k has landed
    fetch(t + (MIX_STAGES - 1) * stride, k == 0 ? MIX_STAGES - 1 : k - 1);
    const typename T::V a0 = T::load(slot, (2 * k) * MIX_THREADS), a1 = T::load(slot, (2 * k + 1) * MIX_THREADS);
    const i64 i0 = ((t >> b) << (b + 1)) | (t & lowmask);
    T::store(psi, i0, T::row2(u00, a0, u01, a1));
    T::store(psi, i0 + step, T::row2(u10, a0, u11, a1));
    k = k == MIX_STAGES - 1 ? 0 : k + 1;
  }
  cp_async_wait<0>();
}

__global__ void __launch_bounds__(MIX_THREADS) k_1q_pairs_mix(double2* __restrict__ psi, i64 npairs, int b,
                                                              int nf64, const __grid_constant__ Coef1q u) {
  if (mix_fp64_warp(nf64)) pairs_ring_body<TC128>(psi, npairs, b, u.e[0], u.e[1], u.e[2], u.e[3]);
  else pairs_ring_body<DF128>(psi, npairs, b, u.d[0], u.d[1], u.d[2], u.d[3]);
}

// Dense complex128 gates of 1 qubit with controls or of 2 qubits, gate by
// gate, with the FP64 / double-float warp split and the load ring of
// k_1q_pairs_mix: a thread's group of D = 2^K amplitudes (base
// insert_zeros(t) | cmask, offsets off.o) sits in ring slots
// mix_ring[(k D + j) MIX_THREADS + thread], DENSE_STAGES(K) steps deep (the
// 2-qubit ring takes 192 KB).  An output row is a complex multiply-add chain
// in IEEE FP64, or one error-free dot product of 2 D terms per real output in
// double-float.
template <int K>
struct CoefDense {
  cdf d[1 << K][1 << K];      // double-float rows
  double2 e[1 << K][1 << K];  // the same in FP64
};
#define DENSE_STAGES(K) ((K) == 2 ? 3 : MIX_STAGES)

template <typename T, int D>
__device__ __forceinline__ typename T::V dense_row(const typename T::V* u, const typename T::V* a) {
  if constexpr (std::is_same<T, DF128>::value) {
    return cdf_row<D>(u, a);
  } else {
    typename T::V acc = T::mul(u[0], a[0]);
#pragma unroll
    for (int c = 1; c < D; ++c) acc = T::fma(u[c], a[c], acc);
    return acc;
  }
}

template <typename T, int K>
__device__ __forceinline__ void dense_ring_body(double2* __restrict__ psi, i64 ngroups, const BitInsert& bi,
                                                i64 cmask, const Offs<K>& off,
                                                const typename T::V (&m)[1 << K][1 << K]) {
  constexpr int D = 1 << K, S = DENSE_STAGES(K);
  const i64 stride = (i64)gridDim.x * MIX_THREADS;
  const i64 t0 = (i64)blockIdx.x * MIX_THREADS + threadIdx.x;
  double2* const slot = mix_ring + threadIdx.x;
  const auto fetch = [&](i64 t, int k) {
    if (t < ngroups) {
      const i64 base = insert_zeros(t, bi) | cmask;
#pragma unroll
      for (int j = 0; j < D; ++j) cp_async16(slot + (k * D + j) * MIX_THREADS, psi + base + off.o[j]);
    }
    cp_async_commit();
  };
#pragma unroll
  for (int k = 0; k < S - 1; ++k) fetch(t0 + k * stride, k);
  int k = 0;
  for (i64 t = t0; t < ngroups; t += stride) {
    cp_async_wait<S - 2>();  // slot k has landed
    fetch(t + (S - 1) * stride, k == 0 ? S - 1 : k - 1);
    typename T::V v[D];
#pragma unroll
    for (int j = 0; j < D; ++j) v[j] = T::load(slot, (k * D + j) * MIX_THREADS);
    const i64 base = insert_zeros(t, bi) | cmask;
#pragma unroll
    for (int r = 0; r < D; ++r) T::store(psi, base + off.o[r], dense_row<T, D>(m[r], v));
    k = k == S - 1 ? 0 : k + 1;
  }
  cp_async_wait<0>();
}

template <int K>
__global__ void __launch_bounds__(MIX_THREADS) k_dense_mix(double2* __restrict__ psi, i64 ngroups,
                                                           const __grid_constant__ BitInsert bi, i64 cmask,
                                                           const __grid_constant__ Offs<K> off, int nf64,
                                                           const __grid_constant__ CoefDense<K> u) {
  if (mix_fp64_warp(nf64)) dense_ring_body<TC128, K>(psi, ngroups, bi, cmask, off, u.e);
  else dense_ring_body<DF128, K>(psi, ngroups, bi, cmask, off, u.d);
}

template <typename V>
__device__ __forceinline__ V shfl_xor_v(V v, int mask);
template <>
__device__ __forceinline__ float2 shfl_xor_v(float2 v, int mask) {
  return make_float2(__shfl_xor_sync(0xffffffffu, v.x, mask), __shfl_xor_sync(0xffffffffu, v.y, mask));
}
template <>
__device__ __forceinline__ double2 shfl_xor_v(double2 v, int mask) {
  return make_double2(__shfl_xor_sync(0xffffffffu, v.x, mask), __shfl_xor_sync(0xffffffffu, v.y, mask));
}
template <>
__device__ __forceinline__ cdf shfl_xor_v(cdf v, int mask) {
  cdf r;
  r.re.hi = __shfl_xor_sync(0xffffffffu, v.re.hi, mask);
  r.re.lo = __shfl_xor_sync(0xffffffffu, v.re.lo, mask);
  r.im.hi = __shfl_xor_sync(0xffffffffu, v.im.hi, mask);
  r.im.lo = __shfl_xor_sync(0xffffffffu, v.im.lo, mask);
  return r;
}

// dense 1-qubit gate, no controls, target bit < 5: each lane owns one
// amplitude of a contiguous 32-amplitude window and fetches its partner
// (lane ^ 2^b) with a warp shuffle.  Requires N >= 32 and a whole number of
// warps per window (the grid covers N exactly in warps).
template <typename T>
__device__ __forceinline__ void shfl_body(typename T::S* __restrict__ psi, i64 N, int b, typename T::V u00,
                                          typename T::V u01, typename T::V u10, typename T::V u11) {
  const i64 stride = (i64)gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31;
  const bool hi = (lane >> b) & 1;
  const typename T::V cs = hi ? u11 : u00;  // coefficient of own amplitude
  const typename T::V cp = hi ? u10 : u01;  // coefficient of the partner
  // W windows per step (i, i + stride, ...) for W independent chains and W
  // loads in flight per thread (4 for 8-byte amplitudes, 2 for 16-byte);
  // N and stride are multiples of 32, so whole warps take the same branches
  // and every full-mask shuffle sees all 32 lanes
  constexpr int W = sizeof(typename T::S) == 8 ? 4 : 2;
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < N; i += W * stride) {
    typename T::V a[W];
#pragma unroll
    for (int w = 0; w < W; ++w)
      if (i + w * stride < N) a[w] = T::load(psi, i + w * stride);
#pragma unroll
    for (int w = 0; w < W; ++w) {
      if (i + w * stride < N) {
        const typename T::V p = shfl_xor_v(a[w], 1 << b);
        T::store(psi, i + w * stride, T::row2(cs, a[w], cp, p));
      }
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_1q_shfl(typename T::S* __restrict__ psi, i64 N, int b,
                                                 typename T::V u00, typename T::V u01,
                                                 typename T::V u10, typename T::V u11) {
  shfl_body<T>(psi, N, b, u00, u01, u10, u11);
}

// shfl_body through the ring (slot k of a thread: mix_ring[k MIX_THREADS +
// thread]).  N and the stride are multiples of 32, so whole warps run the
// same steps and every full-mask shuffle sees all 32 lanes.
template <typename T>
__device__ __forceinline__ void shfl_ring_body(double2* __restrict__ psi, i64 N, int b, typename T::V u00,
                                               typename T::V u01, typename T::V u10, typename T::V u11) {
  const i64 stride = (i64)gridDim.x * MIX_THREADS;
  const bool hi = ((threadIdx.x & 31) >> b) & 1;
  const typename T::V cs = hi ? u11 : u00;  // coefficient of own amplitude
  const typename T::V cp = hi ? u10 : u01;  // coefficient of the partner
  const i64 i0 = (i64)blockIdx.x * MIX_THREADS + threadIdx.x;
  double2* const slot = mix_ring + threadIdx.x;
  const auto fetch = [&](i64 i, int k) {
    if (i < N) cp_async16(slot + k * MIX_THREADS, psi + i);
    cp_async_commit();
  };
#pragma unroll
  for (int k = 0; k < MIX_STAGES - 1; ++k) fetch(i0 + k * stride, k);
  int k = 0;
  for (i64 i = i0; i < N; i += stride) {
    cp_async_wait<MIX_STAGES - 2>();
    fetch(i + (MIX_STAGES - 1) * stride, k == 0 ? MIX_STAGES - 1 : k - 1);
    const typename T::V a = T::load(slot, k * MIX_THREADS);
    const typename T::V p = shfl_xor_v(a, 1 << b);
    T::store(psi, i, T::row2(cs, a, cp, p));
    k = k == MIX_STAGES - 1 ? 0 : k + 1;
  }
  cp_async_wait<0>();
}

// k_1q_shfl with the pipes shared as in k_1q_pairs_mix (warp-uniform split,
// so every shuffle still sees a whole warp)
__global__ void __launch_bounds__(MIX_THREADS) k_1q_shfl_mix(double2* __restrict__ psi, i64 N, int b, int nf64,
                                                             const __grid_constant__ Coef1q u) {
  if (mix_fp64_warp(nf64)) shfl_ring_body<TC128>(psi, N, b, u.e[0], u.e[1], u.e[2], u.e[3]);
  else shfl_ring_body<DF128>(psi, N, b, u.d[0], u.d[1], u.d[2], u.d[3]);
}

// multiply ``phase`` into every amplitude whose ``mask`` bits are all 1
template <typename T>
__global__ void __launch_bounds__(256) k_phase(typename T::S* __restrict__ psi, i64 count, const __grid_constant__ BitInsert bi,
                                               i64 mask, typename T::V phase) {
  const i64 stride = (i64)gridDim.x * blockDim.x;
  for (i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x; t < count; t += stride) {
    const i64 i = insert_zeros(t, bi) | mask;
    T::store(psi, i, T::mul(phase, T::load(psi, i)));
  }
}

// The unit phases -1, i and -i (CZ, S, SDG and their controlled forms):
// sign flips and a swap of the real and imaginary parts, with integer
// operations, so the kernel never touches GB300's slow FP64 pipe.
__device__ __forceinline__ double flip_sign(double x) {
  return __longlong_as_double(__double_as_longlong(x) ^ (long long)0x8000000000000000ull);
}
__device__ __forceinline__ float flip_sign(float x) { return __int_as_float(__float_as_int(x) ^ (int)0x80000000u); }

template <typename S>
__global__ void __launch_bounds__(256) k_phase_unit(S* __restrict__ psi, i64 count, const __grid_constant__ BitInsert bi, i64 mask,
                                                    int mode) {
  const i64 stride = (i64)gridDim.x * blockDim.x;
  // W amplitudes per step for W loads in flight (4 of 8 bytes, 2 of 16)
  constexpr int W = sizeof(S) == 8 ? 4 : 2;
  for (i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x; t < count; t += W * stride) {
    i64 idx[W];
    S v[W];
#pragma unroll
    for (int w = 0; w < W; ++w) {
      idx[w] = t + w * stride < count ? insert_zeros(t + w * stride, bi) | mask : -1;
      if (idx[w] >= 0) v[w] = psi[idx[w]];
    }
#pragma unroll
    for (int w = 0; w < W; ++w) {
      if (idx[w] < 0) continue;
      if (mode == 1) {  // -1
        v[w].x = flip_sign(v[w].x);
        v[w].y = flip_sign(v[w].y);
      } else if (mode == 2) {  // i: (x, y) -> (-y, x)
        const auto x = v[w].x;
        v[w].x = flip_sign(v[w].y);
        v[w].y = x;
      } else {  // -i: (x, y) -> (y, -x)
        const auto x = v[w].x;
        v[w].x = v[w].y;
        v[w].y = flip_sign(x);
      }
      psi[idx[w]] = v[w];
    }
  }
}

// diagonal k-qubit gate with controls: amplitude *= d[target bits]
template <typename T>
struct DiagVec { typename T::V d[32]; };

template <typename T>
__global__ void __launch_bounds__(256) k_diagk(typename T::S* __restrict__ psi, i64 count, const __grid_constant__ BitInsert bi,
                                               i64 cmask, int k, Offs<QGB_MAX_K> tbit, DiagVec<T> D) {
  const i64 stride = (i64)gridDim.x * blockDim.x;
  for (i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x; t < count; t += stride) {
    const i64 i = insert_zeros(t, bi) | cmask;
    int m = 0;
    for (int j = 0; j < k; ++j) m = (m << 1) | (int)((i >> tbit.o[j]) & 1);
    T::store(psi, i, T::mul(D.d[m], T::load(psi, i)));
  }
}

// X-like 1-qubit gate [[0, a], [b, 0]] with controls: new0 = a*old1, new1 = b*old0
template <typename T>
__global__ void __launch_bounds__(256) k_xlike(typename T::S* __restrict__ psi, i64 count, const __grid_constant__ BitInsert bi,
                                               i64 cmask, i64 tstep, typename T::V a, typename T::V b,
                                               int plain) {
  const i64 stride = (i64)gridDim.x * blockDim.x;
  for (i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x; t < count; t += stride) {
    const i64 i0 = insert_zeros(t, bi) | cmask;
    typename T::V v0 = T::load(psi, i0), v1 = T::load(psi, i0 + tstep);
    if (plain) {
      T::store(psi, i0, v1);
      T::store(psi, i0 + tstep, v0);
    } else {
      T::store(psi, i0, T::mul(a, v1));
      T::store(psi, i0 + tstep, T::mul(b, v0));
    }
  }
}

// SWAP of bits (a, b) with controls: exchanges |..0..1..> and |..1..0..>
template <typename T>
__global__ void __launch_bounds__(256) k_swap(typename T::S* __restrict__ psi, i64 count, const __grid_constant__ BitInsert bi,
                                              i64 cmask, i64 sa, i64 sb) {
  const i64 stride = (i64)gridDim.x * blockDim.x;
  for (i64 t = blockIdx.x * (i64)blockDim.x + threadIdx.x; t < count; t += stride) {
    const i64 base = insert_zeros(t, bi) | cmask;
    typename T::V v01 = T::load(psi, base | sb), v10 = T::load(psi, base | sa);
    T::store(psi, base | sb, v10);
    T::store(psi, base | sa, v01);
  }
}

// ===========================================================================
// host side
namespace {

BitInsert make_insert(std::vector<int> bits) {
  BitInsert bi;
  std::sort(bits.begin(), bits.end());
  bi.n = (int)bits.size();
  for (int j = 0; j < bi.n; ++j) bi.pos[j] = bits[j];
  return bi;
}

i64 mask_of(const std::vector<int>& bits) {
  i64 m = 0;
  for (int b : bits) m |= (i64)1 << b;
  return m;
}

// Warps of every eight on a scheduler that compute dense 1-qubit complex128
// gates in IEEE FP64 while the rest use double-float (k_1q_pairs_mix); the
// QIBO_GB300_DF_FP64_WARPS variable (0-8) overrides it for comparisons.
// Measured at n=30 (one pass, 34.4 GB), target qubit 0 / n-1: 0 of 8
// 6.49 / 6.89 ms, 2 of 8 5.36 / 5.53 ms, 3 of 8 6.41 / 5.79 ms, 4 of 8
// 8.20 / 7.53 ms.
int df_fp64_warps() {
  const char* v = getenv("QIBO_GB300_DF_FP64_WARPS");
  if (v && *v) {
    const int w = atoi(v);
    return w < 0 ? 0 : w > 8 ? 8 : w;
  }
  return 2;
}

// widest dense gate a traits type runs (double-float per-gate gates: 2 qubits)
template <typename T>
constexpr int kMaxDenseK = QGB_MAX_K;
template <>
constexpr int kMaxDenseK<DF128> = 2;

template <typename T>
int launch_dense(void* state, int n, const GateOp& g, cudaStream_t s) {
  const int k = (int)g.tbits.size();
  std::vector<int> fixed = g.tbits;
  fixed.insert(fixed.end(), g.cbits.begin(), g.cbits.end());
  BitInsert bi = make_insert(fixed);
  const i64 cmask = mask_of(g.cbits);
  const i64 ngroups = (i64)1 << (n - (int)fixed.size());
  const int D = 1 << k;
  const std::vector<zd>& M = g.coef;
  typedef typename T::S S;
  // fast 1-qubit paths (no controls)
  if (k == 1 && g.cbits.empty()) {
    const int b = g.tbits[0];
    typename T::V u00 = T::coef(M[0].real(), M[0].imag()), u01 = T::coef(M[1].real(), M[1].imag());
    typename T::V u10 = T::coef(M[2].real(), M[2].imag()), u11 = T::coef(M[3].real(), M[3].imag());
    if constexpr (std::is_same<T, DF128>::value) {
      Coef1q cu;
      for (int m = 0; m < 4; ++m) {
        cu.d[m] = DF128::coef(M[m].real(), M[m].imag());
        cu.e[m] = TC128::coef(M[m].real(), M[m].imag());
      }
      const int nf64 = df_fp64_warps();
      // one block per SM, each looping over its share
      const auto mix_blocks = [](i64 items) {
        const i64 b = (items + MIX_THREADS - 1) / MIX_THREADS;
        return (int)std::max<i64>(1, std::min<i64>(b, qgb_num_sms()));
      };
      const int ring = MIX_STAGES * MIX_THREADS * (int)sizeof(double2);  // per amplitude of a step
      if (b < 5 && n >= 5) {
        const i64 N = (i64)1 << n;
        if (int st = qgb_func_smem((const void*)k_1q_shfl_mix, ring)) return st;
        k_1q_shfl_mix<<<mix_blocks(N), MIX_THREADS, ring, s>>>((double2*)state, N, b, nf64, cu);
        QGB_LAUNCH_CHECK("k_1q_shfl_mix");
        return QGB_OK;
      }
      if (b >= 5) {
        if (int st = qgb_func_smem((const void*)k_1q_pairs_mix, 2 * ring)) return st;
        k_1q_pairs_mix<<<mix_blocks(ngroups), MIX_THREADS, 2 * ring, s>>>((double2*)state, ngroups, b, nf64, cu);
        QGB_LAUNCH_CHECK("k_1q_pairs_mix");
        return QGB_OK;
      }
    }
    if (b < 5 && n >= 5) {
      const i64 N = (i64)1 << n;
      int blocks;
      grid_for(N, 256, &blocks);
      k_1q_shfl<T><<<blocks, 256, 0, s>>>((S*)state, N, b, u00, u01, u10, u11);
      QGB_LAUNCH_CHECK("k_1q_shfl");
      return QGB_OK;
    }
    if (b >= 5) {
      int blocks;
      grid_for((ngroups + 1) / 2, 256, &blocks);
      k_1q_pairs<T><<<blocks, 256, 0, s>>>((S*)state, ngroups, b, u00, u01, u10, u11);
      QGB_LAUNCH_CHECK("k_1q_pairs");
      return QGB_OK;
    }
  }
  if constexpr (std::is_same<T, DF128>::value) {
    // 1-qubit gates with controls and 2-qubit gates: k_dense_mix
    if (k == 1 || k == 2) {
      const int nf64 = df_fp64_warps();
      const int blocks = (int)std::max<i64>(1, std::min<i64>((ngroups + MIX_THREADS - 1) / MIX_THREADS,
                                                             qgb_num_sms()));
      const auto launch = [&](auto kk) -> int {
        constexpr int KK = decltype(kk)::value;
        Offs<KK> off;
        CoefDense<KK> cu;
        for (int m = 0; m < D; ++m) {
          i64 o = 0;
          for (int j = 0; j < k; ++j)
            if ((m >> (k - 1 - j)) & 1) o |= (i64)1 << g.tbits[j];
          off.o[m] = o;
          for (int c = 0; c < D; ++c) {
            cu.d[m][c] = DF128::coef(M[m * D + c].real(), M[m * D + c].imag());
            cu.e[m][c] = TC128::coef(M[m * D + c].real(), M[m * D + c].imag());
          }
        }
        const int bytes = DENSE_STAGES(KK) * D * MIX_THREADS * (int)sizeof(double2);
        if (int st = qgb_func_smem((const void*)k_dense_mix<KK>, bytes)) return st;
        k_dense_mix<KK><<<blocks, MIX_THREADS, bytes, s>>>((double2*)state, ngroups, bi, cmask, off, nf64, cu);
        QGB_LAUNCH_CHECK("k_dense_mix");
        return QGB_OK;
      };
      return k == 1 ? launch(std::integral_constant<int, 1>()) : launch(std::integral_constant<int, 2>());
    }
  }
  int blocks;
  grid_for(ngroups, 256, &blocks);
#define QGB_DENSE_CASE(KK)                                                                        \
  case KK: if constexpr (KK <= kMaxDenseK<T>) {                                                   \
    Offs<KK> off;                                                                                 \
    DenseMat<T, KK> dm;                                                                           \
    for (int m = 0; m < D; ++m) {                                                                 \
      i64 o = 0;                                                                                  \
      for (int j = 0; j < k; ++j)                                                                 \
        if ((m >> (k - 1 - j)) & 1) o |= (i64)1 << g.tbits[j];                                    \
      off.o[m] = o;                                                                               \
    }                                                                                             \
    for (int r = 0; r < D; ++r)                                                                   \
      for (int c = 0; c < D; ++c) dm.m[r][c] = T::coef(M[r * D + c].real(), M[r * D + c].imag()); \
    k_dense<T, KK><<<blocks, 256, 0, s>>>((S*)state, ngroups, bi, cmask, off, dm);                \
    QGB_LAUNCH_CHECK("k_dense");                                                                  \
    return QGB_OK;                                                                                \
  }
  switch (k) {
    QGB_DENSE_CASE(1)
    QGB_DENSE_CASE(2)
    QGB_DENSE_CASE(3)
    QGB_DENSE_CASE(4)
    QGB_DENSE_CASE(5)
    default:
      qgb_set_error("dense gate with %d qubits unsupported", k);
      return QGB_ERR_UNSUPPORTED;
  }
#undef QGB_DENSE_CASE
}

template <typename T>
int launch_phase(void* state, int n, const std::vector<int>& bits, zd ph, cudaStream_t s) {
  if (ph == zd(1.0, 0.0)) return QGB_OK;
  BitInsert bi = make_insert(bits);
  const i64 count = (i64)1 << (n - (int)bits.size());
  int blocks;
  grid_for(count, 256, &blocks);
  const int mode = ph == zd(-1.0, 0.0) ? 1 : ph == zd(0.0, 1.0) ? 2 : ph == zd(0.0, -1.0) ? 3 : 0;
  if (mode) {
    k_phase_unit<typename T::S><<<blocks, 256, 0, s>>>((typename T::S*)state, count, bi, mask_of(bits), mode);
    QGB_LAUNCH_CHECK("k_phase_unit");
    return QGB_OK;
  }
  k_phase<T><<<blocks, 256, 0, s>>>((typename T::S*)state, count, bi, mask_of(bits), T::coef(ph.real(), ph.imag()));
  QGB_LAUNCH_CHECK("k_phase");
  return QGB_OK;
}

template <typename T>
int launch_diag(void* state, int n, const GateOp& g, cudaStream_t s) {
  const int k = (int)g.tbits.size();
  BitInsert bi = make_insert(g.cbits);
  const i64 count = (i64)1 << (n - (int)g.cbits.size());
  Offs<QGB_MAX_K> tb;
  for (int j = 0; j < QGB_MAX_K; ++j) tb.o[j] = j < k ? g.tbits[j] : 0;
  DiagVec<T> D;
  for (int m = 0; m < 32; ++m) D.d[m] = m < (1 << k) ? T::coef(g.coef[m].real(), g.coef[m].imag()) : T::coef(1.0, 0.0);
  int blocks;
  grid_for(count, 256, &blocks);
  k_diagk<T><<<blocks, 256, 0, s>>>((typename T::S*)state, count, bi, mask_of(g.cbits), k, tb, D);
  QGB_LAUNCH_CHECK("k_diagk");
  return QGB_OK;
}

template <typename T>
int launch_xlike(void* state, int n, const GateOp& g, cudaStream_t s) {
  std::vector<int> fixed = g.cbits;
  fixed.push_back(g.tbits[0]);
  BitInsert bi = make_insert(fixed);
  const i64 count = (i64)1 << (n - (int)fixed.size());
  int blocks;
  grid_for(count, 256, &blocks);
  const zd a = g.coef[0], b = g.coef[1];
  const int plain = (a == zd(1, 0) && b == zd(1, 0)) ? 1 : 0;
  k_xlike<T><<<blocks, 256, 0, s>>>((typename T::S*)state, count, bi, mask_of(g.cbits), (i64)1 << g.tbits[0],
                                    T::coef(a.real(), a.imag()), T::coef(b.real(), b.imag()), plain);
  QGB_LAUNCH_CHECK("k_xlike");
  return QGB_OK;
}

template <typename T>
int launch_swap(void* state, int n, const GateOp& g, cudaStream_t s) {
  std::vector<int> fixed = g.cbits;
  fixed.push_back(g.tbits[0]);
  fixed.push_back(g.tbits[1]);
  BitInsert bi = make_insert(fixed);
  const i64 count = (i64)1 << (n - (int)fixed.size());
  int blocks;
  grid_for(count, 256, &blocks);
  k_swap<T><<<blocks, 256, 0, s>>>((typename T::S*)state, count, bi, mask_of(g.cbits), (i64)1 << g.tbits[0],
                                   (i64)1 << g.tbits[1]);
  QGB_LAUNCH_CHECK("k_swap");
  return QGB_OK;
}

template <typename T>
int launch_op(void* state, int n, const GateOp& g, cudaStream_t s) {
  if (g.identity) return QGB_OK;
  switch (g.kind) {
    case GK_PHASE: return launch_phase<T>(state, n, g.cbits, g.coef[0], s);
    case GK_DIAG: return launch_diag<T>(state, n, g, s);
    case GK_XLIKE: return launch_xlike<T>(state, n, g, s);
    case GK_SWAP: return launch_swap<T>(state, n, g, s);
    default: return launch_dense<T>(state, n, g, s);
  }
}

// Move a target into the controls when the matrix is the identity on the
// subspace where that qubit is 0 and does not couple it to the 1 subspace.
bool extract_control(GateOp& g) {
  const int k = (int)g.tbits.size();
  const int D = 1 << k;
  std::vector<zd>& M = g.coef;
  for (int j = 0; j < k; ++j) {
    const int bit = 1 << (k - 1 - j);
    bool ok = true;
    for (int r = 0; r < D && ok; ++r)
      for (int c = 0; c < D && ok; ++c) {
        if ((r & bit) && (c & bit)) continue;
        const zd want = (r == c) ? zd(1, 0) : zd(0, 0);
        if (M[r * D + c] != want) ok = false;
      }
    if (!ok) continue;
    std::vector<zd> R((D / 2) * (D / 2));
    int ri = 0;
    for (int r = 0; r < D; ++r) {
      if (!(r & bit)) continue;
      int ci = 0;
      for (int c = 0; c < D; ++c) {
        if (!(c & bit)) continue;
        R[ri * (D / 2) + ci] = M[r * D + c];
        ++ci;
      }
      ++ri;
    }
    g.cbits.push_back(g.tbits[j]);
    g.tbits.erase(g.tbits.begin() + j);
    M.swap(R);
    return true;
  }
  return false;
}

}  // namespace

int qgb_classify(int n, const int* qubits, int k, const int* controls, int nc, const double* matrix, GateOp* op,
                 const char* fn) {
  if (n < 1 || n > QGB_MAXQ) { qgb_set_error("%s: nqubits=%d out of range", fn, n); return QGB_ERR_INVALID; }
  if (k < 0 || k > QGB_MAX_K) { qgb_set_error("%s: %d target qubits (max %d)", fn, k, QGB_MAX_K); return QGB_ERR_UNSUPPORTED; }
  if (nc < 0 || nc > QGB_MAX_CTRL) { qgb_set_error("%s: %d controls (max %d)", fn, nc, QGB_MAX_CTRL); return QGB_ERR_UNSUPPORTED; }
  if (!matrix && k > 0) { qgb_set_error("%s: null matrix", fn); return QGB_ERR_INVALID; }
  u64 seen = 0;
  GateOp& g = *op;
  g = GateOp();
  for (int j = 0; j < k + nc; ++j) {
    const int q = j < k ? qubits[j] : controls[j - k];
    if (q < 0 || q >= n) { qgb_set_error("%s: qubit %d out of range for %d qubits", fn, q, n); return QGB_ERR_INVALID; }
    if (seen & (1ull << q)) { qgb_set_error("%s: qubit %d repeated", fn, q); return QGB_ERR_INVALID; }
    seen |= 1ull << q;
    (j < k ? g.tbits : g.cbits).push_back(n - 1 - q);
  }
  if (!matrix) {
    // validation only (qubit ranges and repeats): an identity phase
    g.kind = GK_PHASE;
    g.coef = {zd(1, 0)};
    g.identity = true;
    return QGB_OK;
  }
  const int D = 1 << k;
  g.coef.resize(D * D);
  for (int i = 0; i < D * D; ++i) g.coef[i] = zd(matrix[2 * i], matrix[2 * i + 1]);
  while (!g.tbits.empty() && extract_control(g)) {
  }
  const int kk = (int)g.tbits.size();
  const int DD = 1 << kk;
  if (kk == 0) {
    g.kind = GK_PHASE;
    g.identity = g.coef[0] == zd(1, 0);
    return QGB_OK;
  }
  bool diag = true, anti = (kk == 1);
  for (int r = 0; r < DD; ++r)
    for (int c = 0; c < DD; ++c) {
      if (r != c && g.coef[r * DD + c] != zd(0, 0)) diag = false;
      if (kk == 1 && r == c && g.coef[r * DD + c] != zd(0, 0)) anti = false;
    }
  if (diag) {
    if (kk == 1 && g.coef[0] == zd(1, 0)) {  // phase on the target's 1s
      const zd ph = g.coef[3];
      g.cbits.push_back(g.tbits[0]);
      g.tbits.clear();
      g.kind = GK_PHASE;
      g.coef = {ph};
      g.identity = ph == zd(1, 0);
      return QGB_OK;
    }
    std::vector<zd> d(DD);
    for (int m = 0; m < DD; ++m) d[m] = g.coef[m * DD + m];
    g.kind = GK_DIAG;
    g.coef = d;
    return QGB_OK;
  }
  if (anti) {
    g.kind = GK_XLIKE;
    g.coef = {g.coef[1], g.coef[2]};
    return QGB_OK;
  }
  if (kk == 2) {
    const zd one(1, 0), zero(0, 0);
    const zd sw[16] = {one, zero, zero, zero, zero, zero, one, zero, zero, one, zero, zero, zero, zero, zero, one};
    bool is_swap = true;
    for (int i = 0; i < 16; ++i)
      if (g.coef[i] != sw[i]) is_swap = false;
    if (is_swap) {
      g.kind = GK_SWAP;
      g.coef.clear();
      return QGB_OK;
    }
  }
  g.kind = GK_DENSE;
  return QGB_OK;
}

namespace {
int check_state_args(void* state, int dtype, const char* fn) {
  if (!state) { qgb_set_error("%s: null state", fn); return QGB_ERR_INVALID; }
  if (!dtype_ok(dtype)) { qgb_set_error("%s: unknown dtype %d", fn, dtype); return QGB_ERR_INVALID; }
  return QGB_OK;
}

int launch_any(void* state, int n, int dtype, const GateOp& g, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  return dtype == QGB_C128 ? launch_op<TC128>(state, n, g, s) : launch_op<TC64>(state, n, g, s);
}
}  // namespace

int qgb_launch_gateop(void* state, int n, int dtype, const GateOp& g, cudaStream_t s) {
  return launch_any(state, n, dtype, g, (void*)s);
}

// A complex128 dense gate of at most 2 qubits in double-float (DF128): the
// per-gate circuit path when IEEE FP64 is not asked for.  The FP64 pipe would
// bound these gates at about a third of HBM bandwidth.
namespace {
bool df_gate(const GateOp& g) { return g.kind == GK_DENSE && !g.identity && g.tbits.size() <= 2; }
}  // namespace

extern "C" {

int qgb_apply_gate(void* state, int nqubits, int dtype, const int* qubits, int k, const int* controls,
                   int ncontrols, const double* matrix, void* stream) {
  int st = check_state_args(state, dtype, "qgb_apply_gate");
  if (st) return st;
  GateOp g;
  st = qgb_classify(nqubits, qubits, k, controls, ncontrols, matrix, &g, "qgb_apply_gate");
  if (st) return st;
  return launch_any(state, nqubits, dtype, g, stream);
}

int qgb_apply_1q(void* state, int nqubits, int dtype, int target, const double* matrix, void* stream) {
  int st = check_state_args(state, dtype, "qgb_apply_1q");
  if (st) return st;
  GateOp g;
  st = qgb_classify(nqubits, &target, 0, nullptr, 0, nullptr, &g, "qgb_apply_1q");  // validation only
  if (st) return st;
  if (target < 0 || target >= nqubits || !matrix) { qgb_set_error("qgb_apply_1q: bad target or matrix"); return QGB_ERR_INVALID; }
  g = GateOp();
  g.kind = GK_DENSE;
  g.tbits = {nqubits - 1 - target};
  g.coef.resize(4);
  for (int i = 0; i < 4; ++i) g.coef[i] = zd(matrix[2 * i], matrix[2 * i + 1]);
  return launch_any(state, nqubits, dtype, g, stream);
}

int qgb_apply_2q(void* state, int nqubits, int dtype, int q0, int q1, const double* matrix, void* stream) {
  int st = check_state_args(state, dtype, "qgb_apply_2q");
  if (st) return st;
  const int qs[2] = {q0, q1};
  GateOp g;
  st = qgb_classify(nqubits, qs, 0, qs, 2, nullptr, &g, "qgb_apply_2q");  // range/duplicate checks
  if (st) return st;
  if (!matrix) { qgb_set_error("qgb_apply_2q: null matrix"); return QGB_ERR_INVALID; }
  g = GateOp();
  g.kind = GK_DENSE;
  g.tbits = {nqubits - 1 - q0, nqubits - 1 - q1};
  g.coef.resize(16);
  for (int i = 0; i < 16; ++i) g.coef[i] = zd(matrix[2 * i], matrix[2 * i + 1]);
  return launch_any(state, nqubits, dtype, g, stream);
}

int qgb_apply_phase(void* state, int nqubits, int dtype, const int* qubits, int nq, double phase_re,
                    double phase_im, void* stream) {
  int st = check_state_args(state, dtype, "qgb_apply_phase");
  if (st) return st;
  GateOp g;
  st = qgb_classify(nqubits, nullptr, 0, qubits, nq, nullptr, &g, "qgb_apply_phase");
  if (st) return st;
  g.kind = GK_PHASE;
  g.coef = {zd(phase_re, phase_im)};
  g.identity = g.coef[0] == zd(1, 0);
  return launch_any(state, nqubits, dtype, g, stream);
}

int qgb_apply_swap(void* state, int nqubits, int dtype, int q0, int q1, const int* controls, int ncontrols,
                   void* stream) {
  int st = check_state_args(state, dtype, "qgb_apply_swap");
  if (st) return st;
  const int qs[2] = {q0, q1};
  GateOp g;
  st = qgb_classify(nqubits, qs, 0, nullptr, 0, nullptr, &g, "qgb_apply_swap");
  if (st) return st;
  GateOp c;
  st = qgb_classify(nqubits, controls, 0, qs, 2, nullptr, &c, "qgb_apply_swap");  // overlap checks
  if (st) return st;
  std::vector<int> all(qs, qs + 2);
  for (int i = 0; i < ncontrols; ++i) all.push_back(controls[i]);
  st = qgb_classify(nqubits, nullptr, 0, all.data(), (int)all.size(), nullptr, &c, "qgb_apply_swap");
  if (st) return st;
  g = GateOp();
  g.kind = GK_SWAP;
  g.tbits = {nqubits - 1 - q0, nqubits - 1 - q1};
  for (int i = 0; i < ncontrols; ++i) g.cbits.push_back(nqubits - 1 - controls[i]);
  return launch_any(state, nqubits, dtype, g, stream);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// whole circuits
int qgb_run_blocked(void* state, int nqubits, int dtype, const qgb_op* ops, int nops, const double* coefs,
                    bool strict_fp64, bool use_tc, cudaStream_t s);  // qgb_blocked.cu

extern "C" int qgb_plan_passes(int nqubits, int dtype, const qgb_op* ops, int nops, const double* coefs,
                               int* npasses);  // qgb_blocked.cu

// QGB_PLAN_FUSE keeps the fused list when it has at most this many ops per
// pass of the unfused shared-memory plan (QIBO_GB300_FUSE_OPS_PER_PASS
// overrides it, for comparisons)
static const int kFuseOpsPerPass = 11;

static int fuse_ops_per_pass() {
  const char* v = getenv("QIBO_GB300_FUSE_OPS_PER_PASS");
  return v && *v ? atoi(v) : kFuseOpsPerPass;
}

extern "C" int qgb_apply_circuit(void* state, int nqubits, int dtype, const qgb_op* ops, int nops,
                                 const double* coefs, int flags, void* stream) {
  if (nops < 0 || (nops > 0 && (!ops || !coefs))) { qgb_set_error("qgb_apply_circuit: bad arguments"); return QGB_ERR_INVALID; }
  int st = check_state_args(state, dtype, "qgb_apply_circuit");
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  if ((flags & QGB_PLAN_BLOCKED) && (flags & QGB_PLAN_FUSE) && nops > 1) {
    for (int i = 0; i < nops; ++i) {  // validate every gate before fusion absorbs it
      GateOp g;
      st = qgb_classify(nqubits, ops[i].qubits, ops[i].k, ops[i].controls, ops[i].ncontrols,
                        coefs + ops[i].coef_offset, &g, "qgb_apply_circuit");
      if (st) return st;
    }
    std::vector<qgb_op> fops;
    std::vector<double> fcoefs;
    // where the tensor cores take 5-qubit blocks, every block is widened to
    // 5 qubits: one tensor-core pass beats a shared-memory pass with a dense
    // 3-4 qubit block (complex128 double-float is FP32-pipe-bound), and the
    // complex128 fixed-point chain stays unbroken
    const bool tc = (flags & QGB_PLAN_NO_TC) == 0 &&
                    (dtype == QGB_C64 || (dtype == QGB_C128 && nqubits >= 12 && !(flags & QGB_PLAN_STRICT_FP64)));
    qgb_fuse5(ops, nops, coefs, &fops, &fcoefs, tc && nqubits >= 12 ? nqubits : 0);
    // Fusion pays when the fused list has few ops per unfused shared-memory
    // pass.  Measured at 20-30 qubits: QFT alone (14 fused ops per pass) runs
    // faster in passes, QFT + brickwork (9 per pass) and brickwork (2.4) fused.
    int npasses = 0;
    st = qgb_plan_passes(nqubits, dtype, ops, nops, coefs, &npasses);
    if (st) return st;
    if ((long long)fops.size() <= fuse_ops_per_pass() * (long long)npasses)
      return qgb_run_blocked(state, nqubits, dtype, fops.data(), (int)fops.size(), fcoefs.data(),
                             (flags & QGB_PLAN_STRICT_FP64) != 0, (flags & QGB_PLAN_NO_TC) == 0, s);
    return qgb_run_blocked(state, nqubits, dtype, ops, nops, coefs, (flags & QGB_PLAN_STRICT_FP64) != 0,
                           (flags & QGB_PLAN_NO_TC) == 0, s);
  }
  if (flags & QGB_PLAN_BLOCKED)
    return qgb_run_blocked(state, nqubits, dtype, ops, nops, coefs, (flags & QGB_PLAN_STRICT_FP64) != 0,
                           (flags & QGB_PLAN_NO_TC) == 0, s);
  const bool df = dtype == QGB_C128 && !(flags & QGB_PLAN_STRICT_FP64);
  for (int i = 0; i < nops; ++i) {
    const qgb_op& op = ops[i];
    GateOp g;
    st = qgb_classify(nqubits, op.qubits, op.k, op.controls, op.ncontrols, coefs + op.coef_offset, &g,
                      "qgb_apply_circuit");
    if (st) return st;
    st = df && df_gate(g) ? launch_dense<DF128>(state, nqubits, g, s) : launch_any(state, nqubits, dtype, g, stream);
    if (st) return st;
  }
  return QGB_OK;
}
