// Device context, error reporting, caching pool and the runtime part of the
// C ABI.  One context per device holds everything the kernels share: the
// library stream, the exponential table, reduction scratch and a pool of
// device blocks so that solvers never call cudaMalloc once warmed up (the
// original allocates and frees several buffers inside every mpla_dgemv,
// mpla.cpp:716-751).
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <chrono>

#include "internal.h"

namespace mgb {

static thread_local char g_last_error[1024] = "";

int set_error(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return code;
}

int cuda_error(cudaError_t e, const char* expr, const char* file, int line) {
  int code = (e == cudaErrorMemoryAllocation) ? MGB_ERR_NOMEM
           : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? MGB_ERR_NODEV
           : MGB_ERR_CUDA;
  return set_error(code, "%s:%d: %s failed: %s", file, line, expr, cudaGetErrorString(e));
}

double wall_seconds() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

static std::atomic<long long> g_launches{0};
static thread_local bool tl_capturing = false;
static thread_local long long tl_capture_count = 0;

void count_launches(long long n) {
  if (tl_capturing) tl_capture_count += n;
  else g_launches += n;
}

void begin_capture_count() {
  tl_capturing = true;
  tl_capture_count = 0;
}

long long end_capture_count() {
  tl_capturing = false;
  return tl_capture_count;
}

static DeviceContext* g_contexts[64] = {nullptr};

static int create_context(int dev, DeviceContext** out) {
  DeviceContext* c = new DeviceContext();
  c->device = dev;
  cudaDeviceProp prop;
  MGB_CUDA(cudaGetDeviceProperties(&prop, dev));
  c->num_sms = prop.multiProcessorCount;
  // Blocking stream: work on it is ordered with the legacy default stream, so
  // user cores that call cuBLAS on stream 0 interleave correctly.
  MGB_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamDefault));
  std::vector<double> table(kExpTableSize);
  for (int j = 0; j < kExpTableSize; ++j) table[j] = std::exp2(-(double)j / (double)kExpTableSize);
  MGB_CUDA(cudaMalloc(&c->exp_table, sizeof(double) * kExpTableSize));
  MGB_CUDA(cudaMemcpy(c->exp_table, table.data(), sizeof(double) * kExpTableSize,
                      cudaMemcpyHostToDevice));
  MGB_CUDA(cudaMalloc(&c->partials, sizeof(double) * kMaxReduceBlocks * 4));
  MGB_CUDA(cudaMalloc(&c->dev_error, sizeof(unsigned int)));
  MGB_CUDA(cudaMemset(c->dev_error, 0, sizeof(unsigned int)));
  MGB_CUDA(cudaMallocHost(&c->state_host, sizeof(SolverState)));
  MGB_CUDA(cudaMallocHost(&c->state_ahead, 2 * sizeof(SolverState)));
  for (int i = 0; i < 2; ++i) MGB_CUDA(cudaEventCreateWithFlags(&c->state_ev[i], cudaEventDisableTiming));
  MGB_TRY(ensure_tickets(c, 4096));
  *out = c;
  return MGB_OK;
}

int context(DeviceContext** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice", __FILE__, __LINE__);
  if (dev < 0 || dev >= 64) return set_error(MGB_ERR_ARG, "device index %d out of range", dev);
  if (!g_contexts[dev]) {
    DeviceContext* c = nullptr;
    MGB_TRY(create_context(dev, &c));
    g_contexts[dev] = c;
  }
  *out = g_contexts[dev];
  return MGB_OK;
}

int ensure_tickets(DeviceContext* c, int count) {
  if (c->n_tickets >= count) return MGB_OK;
  if (c->tickets) {
    MGB_CUDA(cudaStreamSynchronize(c->stream));
    MGB_CUDA(cudaFree(c->tickets));
  }
  MGB_CUDA(cudaMalloc(&c->tickets, sizeof(unsigned int) * count));
  MGB_CUDA(cudaMemset(c->tickets, 0, sizeof(unsigned int) * count));
  c->n_tickets = count;
  return MGB_OK;
}

int ensure_split_partials(DeviceContext* c, size_t count) {
  if (c->split_partials_count >= count) return MGB_OK;
  if (c->split_partials) {
    MGB_CUDA(cudaDeviceSynchronize());
    MGB_CUDA(cudaFree(c->split_partials));
    c->split_partials = nullptr;
  }
  size_t want = count < (1u << 20) ? (1u << 20) : count;
  MGB_CUDA(cudaMalloc(&c->split_partials, sizeof(double) * want));
  c->split_partials_count = want;
  return MGB_OK;
}

int pool_alloc(DeviceContext* c, size_t bytes, void** out) {
  size_t sz = (bytes + 255) & ~size_t(255);
  if (sz == 0) sz = 256;
  auto it = c->free_blocks.find(sz);
  if (it != c->free_blocks.end() && !it->second.empty()) {
    *out = it->second.back();
    it->second.pop_back();
  } else {
    void* p = nullptr;
    MGB_CUDA(cudaMalloc(&p, sz));
    *out = p;
  }
  c->live_blocks[*out] = sz;
  return MGB_OK;
}

void pool_free(DeviceContext* c, void* p) {
  if (!p) return;
  auto it = c->live_blocks.find(p);
  if (it == c->live_blocks.end()) return;
  c->free_blocks[it->second].push_back(p);
  c->live_blocks.erase(it);
}

int check_device_error(DeviceContext* c, cudaStream_t s) {
  unsigned int word = 0;
  MGB_CUDA(cudaMemcpyAsync(&word, c->dev_error, sizeof(word), cudaMemcpyDeviceToHost, s));
  MGB_CUDA(cudaStreamSynchronize(s));
  if (word) {
    MGB_CUDA(cudaMemsetAsync(c->dev_error, 0, sizeof(unsigned int), s));
    if (word & DEV_ERR_WAIT_TIMEOUT)
      return set_error(MGB_ERR_TIMEOUT, "a bounded device-side wait gave up (error word 0x%x)", word);
    return set_error(MGB_ERR_CUDA, "device error word 0x%x", word);
  }
  return MGB_OK;
}

static void destroy_context(DeviceContext* c) {
  cudaStreamSynchronize(c->stream);
  for (auto& g : c->graph_cache) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    if (g.graph) cudaGraphDestroy(g.graph);
  }
  for (auto& kv : c->free_blocks)
    for (void* p : kv.second) cudaFree(p);
  for (auto& kv : c->live_blocks) cudaFree(kv.first);
  cudaFree(c->exp_table);
  cudaFree(c->partials);
  cudaFree(c->tickets);
  cudaFree(c->dev_error);
  cudaFree(c->split_partials);
  cudaFreeHost(c->state_host);
  cudaFreeHost(c->state_ahead);
  for (int i = 0; i < 2; ++i)
    if (c->state_ev[i]) cudaEventDestroy(c->state_ev[i]);
  cudaStreamDestroy(c->stream);
  delete c;
}

}  // namespace mgb

using namespace mgb;

extern "C" {

int mgb_version(void) { return 10000; }

long long mgb_kernel_launches(void) { return g_launches.load(); }

const char* mgb_last_error(void) { return g_last_error; }

int mgb_init(int device) {
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0)
    return set_error(MGB_ERR_NODEV, "no CUDA device available (%s)", cudaGetErrorString(e));
  if (device < 0 || device >= count)
    return set_error(MGB_ERR_ARG, "device %d out of range (have %d)", device, count);
  MGB_CUDA(cudaSetDevice(device));
  DeviceContext* c = nullptr;
  return context(&c);
}

int mgb_shutdown(void) {
  int dev = 0;
  MGB_CUDA(cudaGetDevice(&dev));
  if (dev >= 0 && dev < 64 && g_contexts[dev]) {
    destroy_context(g_contexts[dev]);
    g_contexts[dev] = nullptr;
  }
  return MGB_OK;
}

int mgb_device_sync(void) {
  MGB_CUDA(cudaDeviceSynchronize());
  return MGB_OK;
}

int mgb_malloc(void** ptr, size_t bytes) {
  if (!ptr) return set_error(MGB_ERR_ARG, "mgb_malloc: null output pointer");
  MGB_CUDA(cudaMalloc(ptr, bytes ? bytes : 1));
  return MGB_OK;
}

int mgb_free(void* ptr) {
  MGB_CUDA(cudaFree(ptr));
  return MGB_OK;
}

int mgb_memcpy_htod(void* dst, const void* src, size_t bytes) {
  MGB_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
  return MGB_OK;
}

int mgb_memcpy_dtoh(void* dst, const void* src, size_t bytes) {
  MGB_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
  return MGB_OK;
}

int mgb_memset(void* ptr, int value, size_t bytes) {
  MGB_CUDA(cudaMemset(ptr, value, bytes));
  return MGB_OK;
}

int mgb_host_alloc(void** ptr, size_t bytes) {
  if (!ptr) return set_error(MGB_ERR_ARG, "mgb_host_alloc: null output pointer");
  MGB_CUDA(cudaMallocHost(ptr, bytes ? bytes : 1));
  return MGB_OK;
}

int mgb_host_free(void* ptr) {
  MGB_CUDA(cudaFreeHost(ptr));
  return MGB_OK;
}

}  // extern "C"
