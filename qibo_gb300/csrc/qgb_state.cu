// Library plumbing (errors, device, memory, events) and state creation:
// zero state (Backend.zero_state, backends/abstract.py:2243-2273), basis
// states, dtype casts (NumpyBackend.cast, backends/numpy.py:38-64) and
// real scaling (renormalisation).
#include <cstdarg>
#include <cstdio>
#include <atomic>
#include <mutex>
#include <set>
#include <utility>

#include "qgb_common.cuh"

static thread_local char g_err[512] = "";
static int g_sms = 0;
static std::atomic<long long> g_launches(0);

void qgb_count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

void qgb_set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int qgb_cuda_status(cudaError_t e, const char* what) {
  qgb_set_error("%s: %s", what, cudaGetErrorString(e));
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();  // clear the sticky-free allocation error
    return QGB_ERR_OOM;
  }
  return QGB_ERR_CUDA;
}

int qgb_num_sms() {
  if (g_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_sms <= 0) g_sms = 152;
  }
  return g_sms;
}

int qgb_func_smem(const void* func, int bytes) {
  static std::mutex mu;
  static std::set<std::pair<const void*, int>> done;  // (kernel, device)
  int dev = 0;
  QGB_TRY_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  if (done.count({func, dev})) return QGB_OK;
  QGB_TRY_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  done.insert({func, dev});
  return QGB_OK;
}

int qgb_tc_prepare();  // qgb_tc128.cu: tensor-core device buffers

extern "C" {

const char* qgb_last_error(void) { return g_err; }
int64_t qgb_launch_count(void) { return g_launches.load(); }
int qgb_version(void) { return 100; }

int qgb_device_init(int device, int* sm_count) {
  QGB_TRY_CUDA(cudaSetDevice(device));
  QGB_TRY_CUDA(cudaFree(0));  // create the primary context
  g_sms = 0;
  int st = qgb_tc_prepare();
  if (st) return st;
  if (sm_count) *sm_count = qgb_num_sms();
  return QGB_OK;
}

int qgb_mem_info(size_t* free_bytes, size_t* total_bytes) {
  QGB_TRY_CUDA(cudaMemGetInfo(free_bytes, total_bytes));
  return QGB_OK;
}

int qgb_malloc(void** ptr, size_t bytes) {
  if (!ptr) { qgb_set_error("qgb_malloc: null ptr"); return QGB_ERR_INVALID; }
  *ptr = nullptr;
  if (bytes == 0) return QGB_OK;
  cudaError_t e = cudaMalloc(ptr, bytes);
  if (e != cudaSuccess) {
    *ptr = nullptr;
    return qgb_cuda_status(e, "cudaMalloc");
  }
  return QGB_OK;
}

int qgb_free(void* ptr) {
  if (ptr) QGB_TRY_CUDA(cudaFree(ptr));
  return QGB_OK;
}

int qgb_memcpy_h2d(void* dst, const void* src, size_t bytes, void* stream) {
  QGB_TRY_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, (cudaStream_t)stream));
  return QGB_OK;
}
int qgb_memcpy_d2h(void* dst, const void* src, size_t bytes, void* stream) {
  QGB_TRY_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  return QGB_OK;
}
int qgb_memcpy_d2d(void* dst, const void* src, size_t bytes, void* stream) {
  QGB_TRY_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
  return QGB_OK;
}
int qgb_host_alloc(void** ptr, size_t bytes) {
  if (!ptr) { qgb_set_error("qgb_host_alloc: null ptr"); return QGB_ERR_INVALID; }
  *ptr = nullptr;
  cudaError_t e = cudaMallocHost(ptr, bytes ? bytes : 1);
  if (e != cudaSuccess) return qgb_cuda_status(e, "cudaMallocHost");
  return QGB_OK;
}
int qgb_host_free(void* ptr) {
  if (ptr) QGB_TRY_CUDA(cudaFreeHost(ptr));
  return QGB_OK;
}
int qgb_memset_zero(void* ptr, size_t bytes, void* stream) {
  if (bytes) QGB_TRY_CUDA(cudaMemsetAsync(ptr, 0, bytes, (cudaStream_t)stream));
  return QGB_OK;
}
int qgb_stream_sync(void* stream) {
  QGB_TRY_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  return QGB_OK;
}

int qgb_event_create(void** ev) {
  QGB_TRY_CUDA(cudaEventCreate((cudaEvent_t*)ev));
  return QGB_OK;
}
int qgb_event_destroy(void* ev) {
  QGB_TRY_CUDA(cudaEventDestroy((cudaEvent_t)ev));
  return QGB_OK;
}
int qgb_event_record(void* ev, void* stream) {
  QGB_TRY_CUDA(cudaEventRecord((cudaEvent_t)ev, (cudaStream_t)stream));
  return QGB_OK;
}
int qgb_event_elapsed_ms(void* start, void* stop, float* ms) {
  QGB_TRY_CUDA(cudaEventSynchronize((cudaEvent_t)stop));
  QGB_TRY_CUDA(cudaEventElapsedTime(ms, (cudaEvent_t)start, (cudaEvent_t)stop));
  return QGB_OK;
}

}  // extern "C"

// ------------------------------------------------------------- kernels --
template <typename T>
__global__ void k_set_one(typename T::S* psi, i64 index) {
  T::store(psi, index, T::coef(1.0, 0.0));
}

template <typename T>
__global__ void k_scale(typename T::S* psi, i64 N, double s) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < N; i += (i64)gridDim.x * blockDim.x)
    T::store(psi, i, T::scale(T::load(psi, i), s));
}

__global__ void k_cast_128_to_64(const double2* __restrict__ a, float2* __restrict__ b, i64 N) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < N; i += (i64)gridDim.x * blockDim.x) {
    double2 v = a[i];
    b[i] = make_float2((float)v.x, (float)v.y);
  }
}
__global__ void k_cast_64_to_128(const float2* __restrict__ a, double2* __restrict__ b, i64 N) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < N; i += (i64)gridDim.x * blockDim.x) {
    float2 v = a[i];
    b[i] = make_double2((double)v.x, (double)v.y);
  }
}

static int check_state(const void* s, int n, int dtype, const char* fn) {
  if (!s) { qgb_set_error("%s: null state", fn); return QGB_ERR_INVALID; }
  if (n < 1 || n > QGB_MAXQ) { qgb_set_error("%s: nqubits=%d out of range [1,%d]", fn, n, QGB_MAXQ); return QGB_ERR_INVALID; }
  if (!dtype_ok(dtype)) { qgb_set_error("%s: unknown dtype %d", fn, dtype); return QGB_ERR_INVALID; }
  return QGB_OK;
}

extern "C" {

int qgb_state_basis(void* state, int nqubits, int dtype, int64_t index, void* stream) {
  int st = check_state(state, nqubits, dtype, "qgb_state_basis");
  if (st) return st;
  const i64 N = (i64)1 << nqubits;
  if (index < 0 || index >= N) { qgb_set_error("qgb_state_basis: index out of range"); return QGB_ERR_INVALID; }
  cudaStream_t s = (cudaStream_t)stream;
  QGB_TRY_CUDA(cudaMemsetAsync(state, 0, (size_t)N * dtype_bytes(dtype), s));
  if (dtype == QGB_C128) k_set_one<TC128><<<1, 1, 0, s>>>((double2*)state, index);
  else k_set_one<TC64><<<1, 1, 0, s>>>((float2*)state, index);
  QGB_LAUNCH_CHECK("k_set_one");
  return QGB_OK;
}

int qgb_state_zero(void* state, int nqubits, int dtype, void* stream) {
  return qgb_state_basis(state, nqubits, dtype, 0, stream);
}

int qgb_state_cast(const void* src, int src_dtype, void* dst, int dst_dtype, int nqubits, void* stream) {
  int st = check_state(src, nqubits, src_dtype, "qgb_state_cast");
  if (st) return st;
  st = check_state(dst, nqubits, dst_dtype, "qgb_state_cast");
  if (st) return st;
  const i64 N = (i64)1 << nqubits;
  cudaStream_t s = (cudaStream_t)stream;
  if (src_dtype == dst_dtype) {
    if (src != dst) QGB_TRY_CUDA(cudaMemcpyAsync(dst, src, (size_t)N * dtype_bytes(src_dtype), cudaMemcpyDeviceToDevice, s));
    return QGB_OK;
  }
  int blocks;
  grid_for(N, 256, &blocks);
  if (src_dtype == QGB_C128) k_cast_128_to_64<<<blocks, 256, 0, s>>>((const double2*)src, (float2*)dst, N);
  else k_cast_64_to_128<<<blocks, 256, 0, s>>>((const float2*)src, (double2*)dst, N);
  QGB_LAUNCH_CHECK("k_cast");
  return QGB_OK;
}

int qgb_state_scale(void* state, int nqubits, int dtype, double scale, void* stream) {
  int st = check_state(state, nqubits, dtype, "qgb_state_scale");
  if (st) return st;
  const i64 N = (i64)1 << nqubits;
  int blocks;
  grid_for(N, 256, &blocks);
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == QGB_C128) k_scale<TC128><<<blocks, 256, 0, s>>>((double2*)state, N, scale);
  else k_scale<TC64><<<blocks, 256, 0, s>>>((float2*)state, N, scale);
  QGB_LAUNCH_CHECK("k_scale");
  return QGB_OK;
}

}  // extern "C"
