// Multi-gate passes: many gates applied per read + write of the state.
//
// The reference applies every gate with a full transpose / matmul /
// transpose of the state (backends/abstract.py:2350-2355, gate loop
// :3321-3322), i.e. 2-3 state copies per gate.  Here a planner groups the
// circuit into passes.  A pass picks L "local" index bits (always including
// the lowest ones, so every tile is a set of contiguous 2^m-amplitude runs)
// and walks the state in tiles of 2^L amplitudes: a CTA loads a tile into
// shared memory, applies every gate of the pass to it, and writes it back.
// Only a gate's *target* bits have to be local: a control or a phase mask on
// a non-local bit is constant over a tile and is tested once per tile, so
// diagonal gates (CZ, CU1, ...) never force a new pass.
//
// Planner (host): a forward scan over the not-yet-placed gates in circuit
// order; a gate joins the current pass when no earlier unplaced gate shares
// a qubit with it and its targets fit in the L-bit local set; otherwise its
// qubits are blocked for the rest of the scan.  Gate order on every qubit is
// preserved, so the pass sequence equals the gate sequence.
#include <algorithm>
#include <set>
#include <vector>

#include "qgb_df64.cuh"
#include "qgb_plan.h"

#define QGB_PASS_MAX_OPS 96
#define QGB_PASS_MAX_COEF 1536

int qgb_launch_gateop(void* state, int n, int dtype, const GateOp& g, cudaStream_t s);  // qgb_gates.cu

// Pass traits: G = amplitude type in HBM, S = shared-memory tile element,
// V = value computed on.  complex64 and strict complex128 compute in their
// own precision; TC128F (qgb_df64.cuh) keeps complex128 tiles as double-float.
template <typename C, typename G_>
struct PlainPass {
  typedef G_ G;
  typedef G_ S;
  typedef G_ V;
  static V coef(double re, double im) { return C::coef(re, im); }
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
};
typedef PlainPass<TC64, float2> P64;
typedef PlainPass<TC128, double2> P128;

struct POp {
  uint8_t kind, k;
  uint8_t tpos[5];   // tile-local target positions, most significant matrix bit first
  uint8_t pad;
  uint32_t lmask;    // tile-local bits that must be 1 (controls, phase mask)
  uint64_t gmask;    // non-local index bits that must be 1 (tested per tile)
  int32_t coef;      // offset into PassParams::coef
  int32_t pad2;
};

template <typename T>
struct PassParams {
  int nops, L, m, n;
  int nonloc[QGB_MAXQ];  // ascending global positions of the non-local bits
  int hiloc[QGB_MAXQ];   // ascending global positions of local bits >= m
  POp ops[QGB_PASS_MAX_OPS];
  typename T::V coef[QGB_PASS_MAX_COEF];
};

__device__ __forceinline__ int ins0(int j, int p) { return ((j >> p) << (p + 1)) | (j & ((1 << p) - 1)); }

template <typename T, int K>
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
  for (int g = threadIdx.x; g < groups; g += blockDim.x) {
    int j0 = g;
#pragma unroll
    for (int i = 0; i < K; ++i) j0 = ins0(j0, sorted[i]);
    if ((j0 & op.lmask) != op.lmask) continue;
    typename T::V v[D];
#pragma unroll
    for (int mm = 0; mm < D; ++mm) v[mm] = T::load(tile, j0 + off[mm]);
#pragma unroll
    for (int r = 0; r < D; ++r) T::store(tile, j0 + off[r], T::template row<D>(M + r * D, v));
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_pass(typename T::G* __restrict__ psi, i64 ntiles,
                                              const __grid_constant__ PassParams<T> P) {
  typedef typename T::S S;
  typedef typename T::V V;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int L = P.L, m = P.m;
  const int TN = 1 << L;
  const int nhi = 1 << (L - m);
  S* tile = (S*)smem_raw;
  i64* dep = (i64*)(smem_raw + (size_t)TN * sizeof(S));  // local high part -> global offset
  for (int h = threadIdx.x; h < nhi; h += blockDim.x) {
    i64 o = 0;
    for (int b = 0; b < L - m; ++b) o |= (i64)((h >> b) & 1) << P.hiloc[b];
    dep[h] = o;
  }
  __syncthreads();
  const int nl = P.n - L;
  const int lowmask = (1 << m) - 1;
  for (i64 t = blockIdx.x; t < ntiles; t += gridDim.x) {
    i64 base = 0;
    for (int b = 0; b < nl; ++b) base |= ((t >> b) & 1) << P.nonloc[b];
    for (int j = threadIdx.x; j < TN; j += blockDim.x)
      T::store(tile, j, T::from_global(psi[base | dep[j >> m] | (j & lowmask)]));
    __syncthreads();
    for (int o = 0; o < P.nops; ++o) {
      const POp& op = P.ops[o];
      if ((base & (i64)op.gmask) != (i64)op.gmask) continue;  // uniform over the CTA
      const V* M = P.coef + op.coef;
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
        default: {
          switch (op.k) {
            case 1: apply_dense_tile<T, 1>(tile, L, op, M); break;
            case 2: apply_dense_tile<T, 2>(tile, L, op, M); break;
            case 3: apply_dense_tile<T, 3>(tile, L, op, M); break;
            case 4: apply_dense_tile<T, 4>(tile, L, op, M); break;
            default: apply_dense_tile<T, 5>(tile, L, op, M); break;
          }
        }
      }
      __syncthreads();
    }
    for (int j = threadIdx.x; j < TN; j += blockDim.x)
      psi[base | dep[j >> m] | (j & lowmask)] = T::to_global(T::load(tile, j));
    __syncthreads();
  }
}

// ===========================================================================
namespace {

struct Pass {
  std::vector<int> local;  // global positions (sorted, size L)
  std::vector<int> ops;    // indices into the op list
};

int coef_count(const GateOp& g) { return (int)g.coef.size(); }

std::vector<int> op_bits(const GateOp& g) {
  std::vector<int> b = g.tbits;
  b.insert(b.end(), g.cbits.begin(), g.cbits.end());
  return b;
}

std::vector<Pass> plan_passes(const std::vector<GateOp>& ops, int n, int L, int m) {
  std::vector<Pass> passes;
  std::vector<char> placed(ops.size(), 0);
  size_t first = 0;
  while (true) {
    while (first < ops.size() && (placed[first] || ops[first].identity)) {
      placed[first] = 1;
      ++first;
    }
    if (first >= ops.size()) break;
    std::set<int> S;
    for (int b = 0; b < m; ++b) S.insert(b);
    u64 blocked = 0;
    Pass p;
    int coef_used = 0;
    for (size_t i = first; i < ops.size(); ++i) {
      if (placed[i]) continue;
      const GateOp& g = ops[i];
      u64 bits = 0;
      for (int b : op_bits(g)) bits |= 1ull << b;
      if (bits & blocked) {
        blocked |= bits;
        continue;
      }
      std::set<int> need = S;
      if (g.kind != GK_PHASE)
        for (int b : g.tbits) need.insert(b);
      if ((int)need.size() <= L && coef_used + coef_count(g) <= QGB_PASS_MAX_COEF &&
          (int)p.ops.size() < QGB_PASS_MAX_OPS) {
        S.swap(need);
        p.ops.push_back((int)i);
        placed[i] = 1;
        coef_used += coef_count(g);
      } else {
        blocked |= bits;
      }
    }
    // fill the local set up to L bits with the lowest remaining positions
    for (int b = 0; b < n && (int)S.size() < L; ++b) S.insert(b);
    p.local.assign(S.begin(), S.end());
    passes.push_back(p);
  }
  return passes;
}

template <typename T>
int run_pass(void* state, int n, int L, int m, const Pass& pass, const std::vector<GateOp>& ops, cudaStream_t s) {
  PassParams<T>* P = new PassParams<T>();
  P->nops = (int)pass.ops.size();
  P->L = L;
  P->m = m;
  P->n = n;
  std::vector<int> pos_of(n, -1);
  for (int i = 0; i < L; ++i) pos_of[pass.local[i]] = i;
  for (int i = m; i < L; ++i) P->hiloc[i - m] = pass.local[i];
  int nl = 0;
  for (int b = 0; b < n; ++b)
    if (pos_of[b] < 0) P->nonloc[nl++] = b;
  int coef = 0;
  for (int o = 0; o < P->nops; ++o) {
    const GateOp& g = ops[pass.ops[o]];
    POp& po = P->ops[o];
    po = POp();
    po.kind = (uint8_t)g.kind;
    po.k = (uint8_t)g.tbits.size();
    for (size_t i = 0; i < g.tbits.size(); ++i) po.tpos[i] = (uint8_t)pos_of[g.tbits[i]];
    for (int b : g.cbits) {
      if (pos_of[b] >= 0) po.lmask |= 1u << pos_of[b];
      else po.gmask |= 1ull << b;
    }
    po.coef = coef;
    for (const zd& c : g.coef) P->coef[coef++] = T::coef(c.real(), c.imag());
  }
  const i64 ntiles = (i64)1 << (n - L);
  const size_t smem = ((size_t)sizeof(typename T::S) << L) + (sizeof(i64) << (L - m));
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(k_pass<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attr_set = true;
  }
  const int per_sm = (int)std::max<size_t>(1, std::min<size_t>(4, (220 * 1024) / (smem + 1024)));
  const i64 blocks = std::min<i64>(ntiles, (i64)qgb_num_sms() * per_sm);
  const int threads = std::min(256, std::max(32, 1 << L));
  k_pass<T><<<(unsigned)blocks, threads, smem, s>>>((typename T::G*)state, ntiles, *P);
  delete P;
  QGB_LAUNCH_CHECK("k_pass");
  return QGB_OK;
}

}  // namespace

int qgb_run_blocked(void* state, int nqubits, int dtype, const qgb_op* ops, int nops, const double* coefs,
                    bool strict_fp64, cudaStream_t s) {
  std::vector<GateOp> g(nops);
  for (int i = 0; i < nops; ++i) {
    int st = qgb_classify(nqubits, ops[i].qubits, ops[i].k, ops[i].controls, ops[i].ncontrols,
                          coefs + ops[i].coef_offset, &g[i], "qgb_apply_circuit");
    if (st) return st;
  }
  // tile: 2^L amplitudes = 64 KB of shared memory; runs of 2^m contiguous amplitudes (256 B)
  const int L = std::min(nqubits, dtype == QGB_C128 ? 12 : 13);
  const int m = std::min(L, dtype == QGB_C128 ? 4 : 5);
  std::vector<Pass> passes = plan_passes(g, nqubits, L, m);
  for (const Pass& p : passes) {
    int st;
    if (p.ops.size() == 1) {
      st = qgb_launch_gateop(state, nqubits, dtype, g[p.ops[0]], s);
    } else {
      if (dtype == QGB_C64) st = run_pass<P64>(state, nqubits, L, m, p, g, s);
      else if (strict_fp64) st = run_pass<P128>(state, nqubits, L, m, p, g, s);
      else st = run_pass<TC128F>(state, nqubits, L, m, p, g, s);
    }
    if (st) return st;
  }
  return QGB_OK;
}

extern "C" int qgb_plan_passes(int nqubits, int dtype, const qgb_op* ops, int nops, const double* coefs,
                               int* npasses) {
  std::vector<GateOp> g(nops);
  for (int i = 0; i < nops; ++i) {
    int st = qgb_classify(nqubits, ops[i].qubits, ops[i].k, ops[i].controls, ops[i].ncontrols,
                          coefs + ops[i].coef_offset, &g[i], "qgb_plan_passes");
    if (st) return st;
  }
  const int L = std::min(nqubits, dtype == QGB_C128 ? 12 : 13);
  const int m = std::min(L, dtype == QGB_C128 ? 4 : 5);
  *npasses = (int)plan_passes(g, nqubits, L, m).size();
  return QGB_OK;
}
