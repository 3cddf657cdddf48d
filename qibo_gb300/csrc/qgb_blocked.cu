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

#include "qgb_tile.cuh"

#define QGB_PASS_MAX_OPS 96
#define QGB_PASS_MAX_COEF 1536
#define QGB_PASS_MAX_RUNS 8
#define QGB_PASS_MAX_RUNOPS 256

int qgb_launch_gateop(void* state, int n, int dtype, const GateOp& g, cudaStream_t s);  // qgb_gates.cu

// Merged phase runs.  Consecutive phase gates of a pass (each multiplies
// the amplitudes whose index has all bits of its mask set) whose masks
// share a part P and have at most one bit c_o outside it act together as
// [P in j] * prod_o (c_o in j ? phi_o : 1).  With the tile index
// j = t + 2^tb r (t the thread, r the thread's step) and the tile's
// non-local bits, the product splits into FT[t] (ops whose c_o is a bit of
// t), FR[r] (a bit of r) and FG (a non-local bit, or no c_o): FT and FR are
// tabulated once per CTA, FG once per tile, so a run costs two complex
// multiplications per amplitude instead of one per gate.  QFT layers (the
// controlled phases after each Hadamard share its target) are such runs.
struct PRunOp {
  int16_t coef;  // offset of phi_o in PassParams::coef
  uint8_t dom;   // 0: bit of t, 1: bit of r, 2: non-local bit, 3: none
  uint8_t bit;   // position in t or r, or the global position
};
struct PRun {
  int16_t first, count;  // into PassParams::rops
};

template <typename T>
struct PassParams {
  int nops, L, m, n;
  int nruns, tb;         // merged phase runs; thread-index bits of the tile index
  int nonloc[QGB_MAXQ];  // ascending global positions of the non-local bits
  int hiloc[QGB_MAXQ];   // ascending global positions of local bits >= m
  POp ops[QGB_PASS_MAX_OPS];
  PRun runs[QGB_PASS_MAX_RUNS];
  PRunOp rops[QGB_PASS_MAX_RUNOPS];
  typename T::V coef[QGB_PASS_MAX_COEF];
};

// product of the run's phases whose c_o is in domain ``dom`` with its bit set in ``bits``
// (dom 2 also takes the ops without c_o)
template <typename T>
__device__ __forceinline__ typename T::V run_product(const PassParams<T>& P, const PRun& R, int dom, u64 bits) {
  typename T::V acc = T::one();
  for (int i = R.first; i < R.first + R.count; ++i) {
    const PRunOp& o = P.rops[i];
    const bool take = o.dom == dom ? ((bits >> o.bit) & 1) != 0 : (dom == 2 && o.dom == 3);
    if (take) acc = T::mul(acc, P.coef[o.coef]);
  }
  return acc;
}

__device__ __forceinline__ float2 shfl_down_v(float2 v, int o) {
  return make_float2(__shfl_down_sync(0xffffffffu, v.x, o), __shfl_down_sync(0xffffffffu, v.y, o));
}
__device__ __forceinline__ double2 shfl_down_v(double2 v, int o) {
  return make_double2(__shfl_down_sync(0xffffffffu, v.x, o), __shfl_down_sync(0xffffffffu, v.y, o));
}
__device__ __forceinline__ cdf shfl_down_v(cdf v, int o) {
  cdf r;
  r.re.hi = __shfl_down_sync(0xffffffffu, v.re.hi, o);
  r.re.lo = __shfl_down_sync(0xffffffffu, v.re.lo, o);
  r.im.hi = __shfl_down_sync(0xffffffffu, v.im.hi, o);
  r.im.lo = __shfl_down_sync(0xffffffffu, v.im.lo, o);
  return r;
}

// shared-memory bytes of the run tables: FT, FR and FG per run
template <typename T>
__host__ __device__ __forceinline__ size_t run_table_bytes(int nruns, int L, int tb) {
  return (size_t)nruns * (((size_t)1 << tb) + ((size_t)1 << (L - tb)) + 1) * sizeof(typename T::V);
}
__host__ __device__ __forceinline__ size_t align16(size_t b) { return (b + 15) & ~(size_t)15; }

// One pass over the state (see the file comment); P may live in kernel
// parameter space (k_pass) or in device memory (k_pass_dev, used by captured
// programs whose state pointer and coefficients change between replays).
template <typename T, int MAXK>
__device__ __forceinline__ void pass_body(typename T::G* __restrict__ psi, i64 ntiles, const PassParams<T>& P) {
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
  // run tables (see PRunOp): FT and FR once per CTA
  const int nT = 1 << P.tb, nR = 1 << (L - P.tb);
  V* FT = (V*)(smem_raw + align16((size_t)TN * sizeof(S) + ((size_t)nhi << 3)));
  V* FR = FT + P.nruns * nT;
  V* FG = FR + P.nruns * nR;
  for (int i = threadIdx.x; i < P.nruns * nT; i += blockDim.x) FT[i] = run_product(P, P.runs[i / nT], 0, i % nT);
  for (int i = threadIdx.x; i < P.nruns * nR; i += blockDim.x) FR[i] = run_product(P, P.runs[i / nR], 1, i % nR);
  __syncthreads();
  const int nl = P.n - L;
  const int lowmask = (1 << m) - 1;
  const int lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  for (i64 t = blockIdx.x; t < ntiles; t += gridDim.x) {
    i64 base = 0;
    for (int b = 0; b < nl; ++b) base |= ((t >> b) & 1) << P.nonloc[b];
    for (int j = threadIdx.x; j < TN; j += blockDim.x)
      T::store(tile, j, T::from_global(psi[base | dep[j >> m] | (j & lowmask)]));
    // FG of every run for this tile: one warp per run, lanes over its ops
    for (int r = threadIdx.x >> 5; r < P.nruns; r += nwarps) {
      const PRun& R = P.runs[r];
      V acc = T::one();
      for (int i = R.first + lane; i < R.first + R.count; i += 32) {
        const PRunOp& o = P.rops[i];
        if (o.dom == 3 || (o.dom == 2 && ((base >> o.bit) & 1))) acc = T::mul(acc, P.coef[o.coef]);
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) acc = T::mul(acc, shfl_down_v(acc, off));
      if (lane == 0) FG[r] = acc;
    }
    __syncthreads();
    for (int o = 0; o < P.nops; ++o) {
      const POp& op = P.ops[o];
      if ((base & (i64)op.gmask) != (i64)op.gmask) continue;  // uniform over the CTA
      if (op.kind == GK_PRUN) {
        const int r = op.coef;
        const V a = T::mul(FT[r * nT + (threadIdx.x & (nT - 1))], FG[r]);
        const V* fr = FR + r * nR;
        for (int j = threadIdx.x; j < TN; j += blockDim.x)
          if ((j & op.lmask) == op.lmask) T::store(tile, j, T::mul(T::load(tile, j), T::mul(a, fr[j >> P.tb])));
      } else {
        apply_tile_op<T, MAXK>(tile, L, op, P.coef + op.coef);
      }
      __syncthreads();
    }
    for (int j = threadIdx.x; j < TN; j += blockDim.x)
      psi[base | dep[j >> m] | (j & lowmask)] = T::to_global(T::load(tile, j));
    __syncthreads();
  }
}

// Passes whose dense blocks have at most 2 qubits (the common case) are
// compiled for three resident CTAs per SM (at most 85 registers a thread:
// the complex128 pass then fits three 64 KB tiles per SM instead of two,
// QFT(30) 283 -> 260 ms, a depth-10 brickwork 1576 -> 1341 ms); passes with
// 3-5-qubit fused blocks get the full register file.
// most norm-growth bits of one fixed-point chain of complex128 blocks (each
// bit of headroom is one bit less between the state's norm and 2^61 at the
// chain's start; the 47-bit digit windows follow the values, not the norm)
#define QGB_OZ_HEADROOM 8

#define QGB_PASS_MIN_CTAS(MAXK) ((MAXK) <= 2 ? 3 : 1)

template <typename T, int MAXK>
__global__ void __launch_bounds__(256, QGB_PASS_MIN_CTAS(MAXK))
    k_pass(typename T::G* __restrict__ psi, i64 ntiles, const __grid_constant__ PassParams<T> P) {
  pass_body<T, MAXK>(psi, ntiles, P);
}

template <typename T, int MAXK>
__global__ void __launch_bounds__(256, QGB_PASS_MIN_CTAS(MAXK))
    k_pass_dev(typename T::G* const* __restrict__ psi_slot, i64 ntiles, const PassParams<T>* __restrict__ P) {
  pass_body<T, MAXK>(*psi_slot, ntiles, *P);
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
void pack_params(PassParams<T>* P, int n, int L, int m, const Pass& pass, const std::vector<GateOp>& ops) {
  P->L = L;
  P->m = m;
  P->n = n;
  std::vector<int> pos_of(n, -1);
  for (int i = 0; i < L; ++i) pos_of[pass.local[i]] = i;
  for (int i = m; i < L; ++i) P->hiloc[i - m] = pass.local[i];
  int nl = 0;
  for (int b = 0; b < n; ++b)
    if (pos_of[b] < 0) P->nonloc[nl++] = b;
  P->tb = std::min(L, 8);  // the pass kernels run min(256, 2^L) threads (at least 32)
  P->nruns = 0;
  // coefficients of every op, in pass order
  const int nops = (int)pass.ops.size();
  std::vector<int> coef_at(nops);
  int coef = 0;
  for (int o = 0; o < nops; ++o) {
    coef_at[o] = coef;
    for (const zd& c : ops[pass.ops[o]].coef) P->coef[coef++] = T::coef(c.real(), c.imag());
  }
  auto mask_of = [&](int o) {
    u64 mk = 0;
    for (int b : ops[pass.ops[o]].cbits) mk |= 1ull << b;
    return mk;
  };
  auto is_phase = [&](int o) { return ops[pass.ops[o]].kind == GK_PHASE; };
  int npo = 0, nrops = 0;
  int o = 0;
  while (o < nops) {
    // the longest run of phase gates from o whose masks have at most one bit
    // outside their common part
    int e = o;
    u64 common = 0;
    if (is_phase(o) && P->nruns < QGB_PASS_MAX_RUNS) {
      common = mask_of(o);
      e = o + 1;
      while (e < nops && is_phase(e) && nrops + (e + 1 - o) <= QGB_PASS_MAX_RUNOPS) {
        const u64 c2 = common & mask_of(e);
        bool ok = true;
        for (int k = o; k <= e && ok; ++k) ok = __builtin_popcountll(mask_of(k) & ~c2) <= 1;
        if (!ok) break;
        common = c2;
        ++e;
      }
    }
    POp& po = P->ops[npo++];
    po = POp();
    if (e - o >= 2) {
      const int r = P->nruns++;
      P->runs[r].first = (int16_t)nrops;
      P->runs[r].count = (int16_t)(e - o);
      for (int k = o; k < e; ++k) {
        PRunOp& ro = P->rops[nrops++];
        ro.coef = (int16_t)coef_at[k];
        const u64 c = mask_of(k) & ~common;
        if (!c) {
          ro.dom = 3;
          ro.bit = 0;
        } else {
          const int b = __builtin_ctzll(c);
          const int lp = pos_of[b];
          if (lp < 0) { ro.dom = 2; ro.bit = (uint8_t)b; }
          else if (lp < P->tb) { ro.dom = 0; ro.bit = (uint8_t)lp; }
          else { ro.dom = 1; ro.bit = (uint8_t)(lp - P->tb); }
        }
      }
      po.kind = GK_PRUN;
      for (int b = 0; b < n; ++b)
        if ((common >> b) & 1) {
          if (pos_of[b] >= 0) po.lmask |= 1u << pos_of[b];
          else po.gmask |= 1ull << b;
        }
      po.coef = r;
      o = e;
      continue;
    }
    const GateOp& g = ops[pass.ops[o]];
    po.kind = (uint8_t)g.kind;
    po.k = (uint8_t)g.tbits.size();
    if (g.kind == GK_DENSE && po.k <= 2) {
      bool real = true;
      for (const zd& c : g.coef) real = real && c.imag() == 0.0;
      if (real) po.kind = GK_REAL;
    }
    for (size_t i = 0; i < g.tbits.size(); ++i) po.tpos[i] = (uint8_t)pos_of[g.tbits[i]];
    for (int b : g.cbits) {
      if (pos_of[b] >= 0) po.lmask |= 1u << pos_of[b];
      else po.gmask |= 1ull << b;
    }
    po.coef = coef_at[o];
    ++o;
  }
  P->nops = npo;
}

template <typename T>
struct PassLaunch {
  size_t smem;
  i64 ntiles, blocks;
  int threads;
  int status;  // QGB status of the shared-memory attribute
};

template <typename T>
PassLaunch<T> pass_launch(int n, int L, int m, int nruns) {
  PassLaunch<T> pl;
  pl.ntiles = (i64)1 << (n - L);
  pl.smem = align16(((size_t)sizeof(typename T::S) << L) + (sizeof(i64) << (L - m))) +
            run_table_bytes<T>(nruns, L, std::min(L, 8));
  pl.status = qgb_func_smem((const void*)k_pass<T, 2>, 200 * 1024);
  if (!pl.status) pl.status = qgb_func_smem((const void*)k_pass<T, 5>, 200 * 1024);
  if (!pl.status) pl.status = qgb_func_smem((const void*)k_pass_dev<T, 2>, 200 * 1024);
  if (!pl.status) pl.status = qgb_func_smem((const void*)k_pass_dev<T, 5>, 200 * 1024);
  const int per_sm = (int)std::max<size_t>(1, std::min<size_t>(4, (220 * 1024) / (pl.smem + 1024)));
  pl.blocks = std::min<i64>(pl.ntiles, (i64)qgb_num_sms() * per_sm);
  pl.threads = std::min(256, std::max(32, 1 << L));
  return pl;
}

// largest dense block of a pass (selects the kernel instantiation)
int pass_maxk(const Pass& pass, const std::vector<GateOp>& ops) {
  int k = 0;
  for (int i : pass.ops)
    if (ops[i].kind == GK_DENSE) k = std::max(k, (int)ops[i].tbits.size());
  return k;
}

template <typename T>
int run_pass(void* state, int n, int L, int m, const Pass& pass, const std::vector<GateOp>& ops, cudaStream_t s) {
  PassParams<T>* P = new PassParams<T>();
  pack_params<T>(P, n, L, m, pass, ops);
  const PassLaunch<T> pl = pass_launch<T>(n, L, m, P->nruns);
  if (pl.status) {
    delete P;
    return pl.status;
  }
  if (pass_maxk(pass, ops) <= 2)
    k_pass<T, 2><<<(unsigned)pl.blocks, pl.threads, pl.smem, s>>>((typename T::G*)state, pl.ntiles, *P);
  else
    k_pass<T, 5><<<(unsigned)pl.blocks, pl.threads, pl.smem, s>>>((typename T::G*)state, pl.ntiles, *P);
  delete P;
  QGB_LAUNCH_CHECK("k_pass");
  return QGB_OK;
}

}  // namespace


namespace {
bool is_tc_block(const GateOp& g) { return g.kind == GK_DENSE && g.tbits.size() == 5 && g.cbits.empty(); }

int run_segment(void* state, int nqubits, int dtype, const std::vector<GateOp>& g, bool strict_fp64, cudaStream_t s) {
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
}  // namespace

// Blocked execution.  Fused 5-qubit blocks (uncontrolled dense 32x32) run on
// the tensor cores, one pass each: complex64 in 3xTF32 (qgb_tc.cu), complex128
// from 12 qubits in the Ozaki scheme on BF16 (qgb_tc128.cu; not under
// strict FP64, which keeps IEEE arithmetic).  The gates between two such
// blocks are planned into shared-memory passes.
int qgb_run_blocked(void* state, int nqubits, int dtype, const qgb_op* ops, int nops, const double* coefs,
                    bool strict_fp64, bool use_tc, cudaStream_t s) {
  std::vector<GateOp> g(nops);
  for (int i = 0; i < nops; ++i) {
    int st = qgb_classify(nqubits, ops[i].qubits, ops[i].k, ops[i].controls, ops[i].ncontrols,
                          coefs + ops[i].coef_offset, &g[i], "qgb_apply_circuit");
    if (st) return st;
  }
  const bool tc_ok = use_tc && (dtype == QGB_C64 || (dtype == QGB_C128 && nqubits >= 12 && !strict_fp64));
  if (!tc_ok) return run_segment(state, nqubits, dtype, g, strict_fp64, s);
  // consecutive tensor-core blocks; in complex128, runs of two or more
  // blocks whose norm growth (qgb_oz_growth_bits: 0 for unitary blocks,
  // e.g. density-matrix channels otherwise) adds up to at most
  // QGB_OZ_HEADROOM bits run as fixed-point chains with that headroom; a
  // block left alone runs on IEEE doubles
  std::vector<const GateOp*> run;
  auto flush_run = [&]() -> int {
    if (run.empty()) return QGB_OK;
    int st = QGB_OK;
    if (dtype != QGB_C128) {
      for (const GateOp* b : run) {
        st = qgb_launch_fused5_tc(state, nqubits, *b, s);
        if (st) break;
      }
      run.clear();
      return st;
    }
    std::vector<const GateOp*> chain;
    int head = 0;
    auto flush_chain = [&]() -> int {
      int r = QGB_OK;
      if (chain.size() >= 2) r = qgb_run_oz_chain(state, nqubits, chain, s, head);
      else if (chain.size() == 1) r = qgb_launch_fused5_oz(state, nqubits, *chain[0], s, false);
      chain.clear();
      head = 0;
      return r;
    };
    for (const GateOp* b : run) {
      const int gb = qgb_oz_growth_bits(*b);
      if (gb > QGB_OZ_HEADROOM) {  // too expansive for any chain: alone, on IEEE doubles
        if ((st = flush_chain())) break;
        if ((st = qgb_launch_fused5_oz(state, nqubits, *b, s, false))) break;
        continue;
      }
      if (head + gb > QGB_OZ_HEADROOM && (st = flush_chain())) break;
      chain.push_back(b);
      head += gb;
    }
    if (!st) st = flush_chain();
    run.clear();
    return st;
  };
  std::vector<GateOp> seg;
  for (int i = 0; i <= nops; ++i) {
    const bool tc = i < nops && is_tc_block(g[i]);
    if (tc) {
      if (!seg.empty()) {
        int st = run_segment(state, nqubits, dtype, seg, strict_fp64, s);
        if (st) return st;
        seg.clear();
      }
      run.push_back(&g[i]);
    } else {
      int st = flush_run();
      if (st) return st;
      if (i == nops) {
        if (!seg.empty()) {
          st = run_segment(state, nqubits, dtype, seg, strict_fp64, s);
          if (st) return st;
        }
      } else {
        seg.push_back(g[i]);
      }
    }
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

// ===========================================================================
// Programs: a planned circuit whose pass parameters and state pointer live in
// device memory, so the launch sequence is captured once as a CUDA graph and
// replayed for every circuit of the same shape (same gates on the same
// qubits; matrices may change through qgb_program_update).
namespace {
struct Program {
  int n, dtype, L, m;
  bool strict;
  std::vector<GateOp> ops;
  std::vector<Pass> passes;
  size_t pbytes;             // bytes of one PassParams
  unsigned char* hparams;    // pinned host staging, passes * pbytes
  void* dparams;             // device copy
  void** dslot;              // device: the state pointer the kernels read
  void** hslot;              // pinned host copy of the state pointer
  cudaEvent_t staged;        // last host->device copy of hparams / hslot
  cudaGraphExec_t exec;
  bool captured;
  bool use_graph;
};

template <typename T>
void program_pack(Program* p) {
  for (size_t i = 0; i < p->passes.size(); ++i)
    pack_params<T>((PassParams<T>*)(p->hparams + i * p->pbytes), p->n, p->L, p->m, p->passes[i], p->ops);
}

template <typename T>
int program_launches(Program* p, cudaStream_t s) {
  int nruns = 0;  // tables sized for the pass with the most runs
  for (size_t i = 0; i < p->passes.size(); ++i)
    nruns = std::max(nruns, ((const PassParams<T>*)(p->hparams + i * p->pbytes))->nruns);
  const PassLaunch<T> pl = pass_launch<T>(p->n, p->L, p->m, nruns);
  if (pl.status) return pl.status;
  for (size_t i = 0; i < p->passes.size(); ++i) {
    const PassParams<T>* P = (const PassParams<T>*)((unsigned char*)p->dparams + i * p->pbytes);
    if (pass_maxk(p->passes[i], p->ops) <= 2)
      k_pass_dev<T, 2><<<(unsigned)pl.blocks, pl.threads, pl.smem, s>>>((typename T::G* const*)p->dslot, pl.ntiles, P);
    else
      k_pass_dev<T, 5><<<(unsigned)pl.blocks, pl.threads, pl.smem, s>>>((typename T::G* const*)p->dslot, pl.ntiles, P);
    QGB_LAUNCH_CHECK("k_pass_dev");
  }
  return QGB_OK;
}

int program_launch_any(Program* p, cudaStream_t s) {
  if (p->dtype == QGB_C64) return program_launches<P64>(p, s);
  if (p->strict) return program_launches<P128>(p, s);
  return program_launches<TC128F>(p, s);
}

void program_pack_any(Program* p) {
  if (p->dtype == QGB_C64) program_pack<P64>(p);
  else if (p->strict) program_pack<P128>(p);
  else program_pack<TC128F>(p);
}

size_t program_pbytes(int dtype, bool strict) {
  if (dtype == QGB_C64) return sizeof(PassParams<P64>);
  return strict ? sizeof(PassParams<P128>) : sizeof(PassParams<TC128F>);
}

int classify_all(int n, const qgb_op* ops, int nops, const double* coefs, std::vector<GateOp>* out) {
  out->resize(nops);
  for (int i = 0; i < nops; ++i) {
    int st = qgb_classify(n, ops[i].qubits, ops[i].k, ops[i].controls, ops[i].ncontrols, coefs + ops[i].coef_offset,
                          &(*out)[i], "qgb_program");
    if (st) return st;
  }
  return QGB_OK;
}

bool same_shape(const GateOp& a, const GateOp& b) {
  return a.kind == b.kind && a.tbits == b.tbits && a.cbits == b.cbits && a.coef.size() == b.coef.size() &&
         a.identity == b.identity;
}
}  // namespace

extern "C" {

int qgb_program_create(int nqubits, int dtype, const qgb_op* ops, int nops, const double* coefs, int flags,
                       void** prog) {
  if (!prog || nops <= 0 || !ops || !coefs || !dtype_ok(dtype) || nqubits < 1 || nqubits > QGB_MAXQ) {
    qgb_set_error("qgb_program_create: bad arguments");
    return QGB_ERR_INVALID;
  }
  *prog = nullptr;
  Program* p = new Program();
  p->n = nqubits;
  p->dtype = dtype;
  p->strict = (flags & QGB_PLAN_STRICT_FP64) != 0;
  p->use_graph = (flags & QGB_PROGRAM_NO_GRAPH) == 0;
  p->L = std::min(nqubits, dtype == QGB_C128 ? 12 : 13);
  p->m = std::min(p->L, dtype == QGB_C128 ? 4 : 5);
  int st = classify_all(nqubits, ops, nops, coefs, &p->ops);
  if (st) { delete p; return st; }
  p->passes = plan_passes(p->ops, nqubits, p->L, p->m);
  p->pbytes = (program_pbytes(dtype, p->strict) + 255) / 256 * 256;
  const size_t total = p->pbytes * p->passes.size();
  cudaError_t e = cudaMallocHost((void**)&p->hparams, total);
  if (e == cudaSuccess) e = cudaMalloc(&p->dparams, total);
  if (e == cudaSuccess) e = cudaMalloc((void**)&p->dslot, sizeof(void*));
  if (e == cudaSuccess) e = cudaMallocHost((void**)&p->hslot, sizeof(void*));
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->staged, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    qgb_program_destroy(p);
    return qgb_cuda_status(e, "qgb_program_create");
  }
  program_pack_any(p);
  e = cudaMemcpy(p->dparams, p->hparams, total, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    qgb_program_destroy(p);
    return qgb_cuda_status(e, "qgb_program_create");
  }
  *prog = p;
  return QGB_OK;
}

int qgb_program_passes(void* prog, int* npasses) {
  if (!prog || !npasses) { qgb_set_error("qgb_program_passes: bad arguments"); return QGB_ERR_INVALID; }
  *npasses = (int)((Program*)prog)->passes.size();
  return QGB_OK;
}

int qgb_program_update(void* prog, const qgb_op* ops, int nops, const double* coefs, void* stream) {
  Program* p = (Program*)prog;
  if (!p || !ops || !coefs || nops != (int)p->ops.size()) {
    qgb_set_error("qgb_program_update: bad arguments or a different gate count");
    return QGB_ERR_INVALID;
  }
  std::vector<GateOp> g;
  int st = classify_all(p->n, ops, nops, coefs, &g);
  if (st) return st;
  for (int i = 0; i < nops; ++i)
    if (!same_shape(g[i], p->ops[i])) {
      qgb_set_error("qgb_program_update: op %d has a different shape than the program", i);
      return QGB_ERR_INVALID;
    }
  QGB_TRY_CUDA(cudaEventSynchronize(p->staged));  // the previous copy has left hparams
  p->ops.swap(g);
  program_pack_any(p);
  cudaStream_t s = (cudaStream_t)stream;
  QGB_TRY_CUDA(cudaMemcpyAsync(p->dparams, p->hparams, p->pbytes * p->passes.size(), cudaMemcpyHostToDevice, s));
  QGB_TRY_CUDA(cudaEventRecord(p->staged, s));
  return QGB_OK;
}

int qgb_program_run(void* prog, void* state, void* stream) {
  Program* p = (Program*)prog;
  if (!p || !state) { qgb_set_error("qgb_program_run: bad arguments"); return QGB_ERR_INVALID; }
  cudaStream_t s = (cudaStream_t)stream;
  QGB_TRY_CUDA(cudaEventSynchronize(p->staged));
  *p->hslot = state;
  QGB_TRY_CUDA(cudaMemcpyAsync(p->dslot, p->hslot, sizeof(void*), cudaMemcpyHostToDevice, s));
  QGB_TRY_CUDA(cudaEventRecord(p->staged, s));
  // the legacy default stream cannot be captured: launch directly there
  if (!p->use_graph || s == nullptr) return program_launch_any(p, s);
  if (!p->captured) {
    cudaGraph_t graph;
    QGB_TRY_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    int st = program_launch_any(p, s);
    cudaError_t e = cudaStreamEndCapture(s, &graph);
    if (st) return st;
    if (e != cudaSuccess) return qgb_cuda_status(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&p->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return qgb_cuda_status(e, "cudaGraphInstantiate");
    p->captured = true;
  }
  QGB_TRY_CUDA(cudaGraphLaunch(p->exec, s));
  qgb_count_launch();
  return QGB_OK;
}

int qgb_program_destroy(void* prog) {
  Program* p = (Program*)prog;
  if (!p) return QGB_OK;
  if (p->staged) cudaEventSynchronize(p->staged);
  if (p->captured) cudaGraphExecDestroy(p->exec);
  if (p->staged) cudaEventDestroy(p->staged);
  if (p->dslot) cudaFree(p->dslot);
  if (p->dparams) cudaFree(p->dparams);
  if (p->hslot) cudaFreeHost(p->hslot);
  if (p->hparams) cudaFreeHost(p->hparams);
  delete p;
  return QGB_OK;
}

}  // extern "C"
