// Serving support: streams, event polling, and batched small circuits.
//
// The reference executes many circuits with joblib thread pools on the host
// (Backend.execute_circuits, backends/abstract.py:2514-2530;
// parallel_circuits_execution, parallel.py:60-121).  Here circuits small
// enough to live in one SM's shared memory (<= 13 qubits complex64, <= 12
// qubits complex128) are executed many at a time by one launch: each CTA
// takes a circuit, keeps its whole state in shared memory, applies the gate
// list and produces the requested output (state, shots or a Z-string
// expectation) before moving to the next circuit.  No CTA ever waits on
// another or on the host, so a launch always terminates.
#include <algorithm>
#include <cstring>
#include <vector>

#include "qgb_tile.cuh"

extern "C" {

int qgb_stream_create(void** stream) {
  if (!stream) { qgb_set_error("qgb_stream_create: null"); return QGB_ERR_INVALID; }
  QGB_TRY_CUDA(cudaStreamCreateWithFlags((cudaStream_t*)stream, cudaStreamNonBlocking));
  // the stream's own complex128 chain scratch, so that circuits run on it
  // later allocate nothing and share nothing with other streams
  return qgb_oz_stream_prepare((cudaStream_t)*stream);
}

int qgb_stream_destroy(void* stream) {
  if (!stream) return QGB_OK;
  int st = qgb_oz_stream_release((cudaStream_t)stream);
  if (st) return st;
  QGB_TRY_CUDA(cudaStreamDestroy((cudaStream_t)stream));
  return QGB_OK;
}

int qgb_event_query(void* ev) {
  cudaError_t e = cudaEventQuery((cudaEvent_t)ev);
  if (e == cudaSuccess) return QGB_OK;
  if (e == cudaErrorNotReady) return QGB_NOT_READY;
  return qgb_cuda_status(e, "cudaEventQuery");
}

}  // extern "C"

// Philox4x32-10 (Salmon et al., SC'11); same stream as qgb_sample.
__device__ __forceinline__ void philox10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r > 0) { k0 += W0; k1 += W1; }
    const uint64_t p0 = (uint64_t)M0 * c[0], p1 = (uint64_t)M1 * c[2];
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
    c[0] = n0; c[1] = (uint32_t)p1; c[2] = n2; c[3] = (uint32_t)p0;
  }
}

struct DevItem {
  void* state;
  const POp* ops;
  const void* coefs;
  int n, nops, init_zero, out_kind;
  i64 nshots;
  u64 seed;
  u64 zidx;  // index-space Z mask
  void* out;
};

template <typename T>
__device__ __forceinline__ double abs2_of(typename T::V v) {
  const typename T::G g = T::to_global(v);
  return (double)g.x * g.x + (double)g.y * g.y;
}

__device__ double block_sum_b(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x < 32) {
    r = (l < (int)(blockDim.x >> 5)) ? sh[l] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  __syncthreads();
  return r;
}

template <typename T>
__global__ void __launch_bounds__(256) k_batch(const DevItem* __restrict__ items, int nitems, int maxn) {
  typedef typename T::S S;
  typedef typename T::V V;
  typedef typename T::G G;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  S* tile = (S*)smem_raw;
  double* prob = (double*)(smem_raw + (sizeof(S) << maxn));
  __shared__ double red[32];
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const DevItem item = items[it];
    const int n = item.n, TN = 1 << n;
    G* psi = (G*)item.state;
    for (int j = threadIdx.x; j < TN; j += blockDim.x) {
      G g;
      if (item.init_zero) { g.x = (j == 0) ? 1 : 0; g.y = 0; }
      else g = psi[j];
      T::store(tile, j, T::from_global(g));
    }
    __syncthreads();
    const V* coefs = (const V*)item.coefs;
    for (int o = 0; o < item.nops; ++o) {
      const POp op = item.ops[o];
      apply_tile_op<T, 5>(tile, n, op, coefs + op.coef);
      __syncthreads();
    }
    if (item.out_kind == QGB_OUT_STATE) {
      for (int j = threadIdx.x; j < TN; j += blockDim.x) psi[j] = T::to_global(T::load(tile, j));
    } else if (item.out_kind == QGB_OUT_ZEXP) {
      double acc = 0.0;
      for (int j = threadIdx.x; j < TN; j += blockDim.x) {
        const double p = abs2_of<T>(T::load(tile, j));
        acc += (__popcll((u64)j & item.zidx) & 1) ? -p : p;
      }
      acc = block_sum_b(acc, red);
      if (threadIdx.x == 0) *(double*)item.out = acc;
    } else {
      // FP64 inclusive prefix of |psi|^2: serial within each thread's chunk,
      // then a scan of the chunk totals
      const int per = (TN + blockDim.x - 1) / blockDim.x;
      const int j0 = threadIdx.x * per, j1 = min(TN, j0 + per);
      double run = 0.0;
      for (int j = j0; j < j1; ++j) {
        run += abs2_of<T>(T::load(tile, j));
        prob[j] = run;
      }
      __syncthreads();
      // exclusive offsets of the chunk totals (blockDim <= 256)
      __shared__ double tot[256];
      tot[threadIdx.x] = run;
      __syncthreads();
      for (int off = 1; off < (int)blockDim.x; off <<= 1) {
        const double add = threadIdx.x >= off ? tot[threadIdx.x - off] : 0.0;
        __syncthreads();
        tot[threadIdx.x] += add;
        __syncthreads();
      }
      const double base = threadIdx.x > 0 ? tot[threadIdx.x - 1] : 0.0;
      for (int j = j0; j < j1; ++j) prob[j] += base;
      __syncthreads();
      const double total = prob[TN - 1];
      int64_t* out = (int64_t*)item.out;
      const uint32_t k0 = (uint32_t)item.seed, k1 = (uint32_t)(item.seed >> 32);
      for (i64 s = threadIdx.x; s < item.nshots; s += blockDim.x) {
        uint32_t c[4] = {(uint32_t)s, (uint32_t)(s >> 32), 0u, 0u};
        philox10(c, k0, k1);
        const u64 bits = (((u64)c[0] << 32) | c[1]) >> 11;
        const double target = (double)bits * (1.0 / 9007199254740992.0) * total;
        int lo = 0, hi = TN - 1;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (prob[mid] > target) hi = mid; else lo = mid + 1;
        }
        out[s] = lo;
      }
    }
    __syncthreads();
  }
}

namespace {
struct BatchCtx {
  size_t cap;
  unsigned char* host;   // pinned staging
  unsigned char* dev;    // device workspace
  cudaEvent_t staged;
};

size_t align256(size_t x) { return (x + 255) / 256 * 256; }

u64 idx_mask_q(u64 qmask, int n) {
  u64 r = 0;
  for (int q = 0; q < n; ++q)
    if ((qmask >> q) & 1) r |= 1ull << (n - 1 - q);
  return r;
}

template <typename T>
int batch_run(BatchCtx* c, const qgb_batch_item* items, int nitems, cudaStream_t s) {
  const int maxq = sizeof(typename T::G) == 16 ? QGB_BATCH_MAX_QUBITS_C128 : QGB_BATCH_MAX_QUBITS_C64;
  QGB_TRY_CUDA(cudaEventSynchronize(c->staged));  // staging is free again
  size_t off = align256(sizeof(DevItem) * nitems);
  if (off > c->cap) { qgb_set_error("qgb_batch_run: %d items exceed the batch capacity", nitems); return QGB_ERR_INVALID; }
  DevItem* di = (DevItem*)c->host;
  int maxn = 1;
  for (int i = 0; i < nitems; ++i) {
    const qgb_batch_item& it = items[i];
    if (it.nqubits < 1 || it.nqubits > maxq || !it.state || it.nops < 0 || (it.nops && (!it.ops || !it.coefs)) ||
        (it.out_kind != QGB_OUT_STATE && !it.out) || it.out_kind < 0 || it.out_kind > 2 || it.nshots < 0) {
      qgb_set_error("qgb_batch_run: bad item %d (at most %d qubits for this dtype)", i, maxq);
      return QGB_ERR_INVALID;
    }
    maxn = std::max(maxn, it.nqubits);
    std::vector<GateOp> g(it.nops);
    for (int o = 0; o < it.nops; ++o) {
      int st = qgb_classify(it.nqubits, it.ops[o].qubits, it.ops[o].k, it.ops[o].controls, it.ops[o].ncontrols,
                            it.coefs + it.ops[o].coef_offset, &g[o], "qgb_batch_run");
      if (st) return st;
    }
    size_t ncoef = 0;
    for (auto& x : g) ncoef += x.coef.size();
    const size_t ops_off = off, coef_off = align256(ops_off + sizeof(POp) * std::max(1, it.nops));
    const size_t end = align256(coef_off + sizeof(typename T::V) * std::max<size_t>(1, ncoef));
    if (end > c->cap) { qgb_set_error("qgb_batch_run: batch exceeds the context capacity"); return QGB_ERR_INVALID; }
    POp* po = (POp*)(c->host + ops_off);
    typename T::V* cv = (typename T::V*)(c->host + coef_off);
    int k = 0;
    for (int o = 0; o < it.nops; ++o) {
      POp p = POp();
      p.kind = (uint8_t)g[o].kind;
      p.k = (uint8_t)g[o].tbits.size();
      for (size_t t = 0; t < g[o].tbits.size(); ++t) p.tpos[t] = (uint8_t)g[o].tbits[t];
      for (int b : g[o].cbits) p.lmask |= 1u << b;
      p.coef = k;
      for (const zd& z : g[o].coef) cv[k++] = T::coef(z.real(), z.imag());
      po[o] = p;
    }
    DevItem d;
    d.state = it.state;
    d.ops = (const POp*)(c->dev + ops_off);
    d.coefs = c->dev + coef_off;
    d.n = it.nqubits;
    d.nops = it.nops;
    d.init_zero = it.init_zero;
    d.out_kind = it.out_kind;
    d.nshots = it.nshots;
    d.seed = it.seed;
    d.zidx = idx_mask_q(it.zmask, it.nqubits);
    d.out = it.out;
    di[i] = d;
    off = end;
  }
  QGB_TRY_CUDA(cudaMemcpyAsync(c->dev, c->host, off, cudaMemcpyHostToDevice, s));
  QGB_TRY_CUDA(cudaEventRecord(c->staged, s));
  const size_t smem = (sizeof(typename T::S) << maxn) + (sizeof(double) << maxn);
  const int sa = qgb_func_smem((const void*)k_batch<T>, 200 * 1024);
  if (sa) return sa;
  const int per_sm = (int)std::max<size_t>(1, std::min<size_t>(8, (220 * 1024) / (smem + 4096)));
  const int blocks = std::max(1, std::min(nitems, qgb_num_sms() * per_sm));
  k_batch<T><<<blocks, 256, smem, s>>>((const DevItem*)c->dev, nitems, maxn);
  QGB_LAUNCH_CHECK("k_batch");
  return QGB_OK;
}
}  // namespace

extern "C" {

int qgb_batch_create(size_t capacity, void** ctx) {
  if (!ctx || capacity < 4096) { qgb_set_error("qgb_batch_create: bad arguments"); return QGB_ERR_INVALID; }
  BatchCtx* c = new BatchCtx();
  c->cap = capacity;
  cudaError_t e = cudaMallocHost((void**)&c->host, capacity);
  if (e == cudaSuccess) e = cudaMalloc((void**)&c->dev, capacity);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->staged, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    if (c->host) cudaFreeHost(c->host);
    if (c->dev) cudaFree(c->dev);
    delete c;
    return qgb_cuda_status(e, "qgb_batch_create");
  }
  *ctx = c;
  return QGB_OK;
}

int qgb_batch_run(void* ctx, const qgb_batch_item* items, int nitems, int dtype, void* stream) {
  BatchCtx* c = (BatchCtx*)ctx;
  if (!c || nitems < 0 || (nitems && !items) || !dtype_ok(dtype)) {
    qgb_set_error("qgb_batch_run: bad arguments");
    return QGB_ERR_INVALID;
  }
  if (nitems == 0) return QGB_OK;
  cudaStream_t s = (cudaStream_t)stream;
  return dtype == QGB_C64 ? batch_run<P64>(c, items, nitems, s) : batch_run<TC128F>(c, items, nitems, s);
}

int qgb_batch_destroy(void* ctx) {
  BatchCtx* c = (BatchCtx*)ctx;
  if (!c) return QGB_OK;
  cudaEventSynchronize(c->staged);
  cudaEventDestroy(c->staged);
  cudaFreeHost(c->host);
  cudaFree(c->dev);
  delete c;
  return QGB_OK;
}

}  // extern "C"
