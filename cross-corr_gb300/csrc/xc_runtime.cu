// xc_runtime.cu -- host runtime pieces shared by every kernel family:
// thread-local error messages, the TMA descriptor encoder and the per-device
// flag word that bounded device waits report into.
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "xc_common.cuh"
#include "xc_internal.h"

namespace xc {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string& msg) { g_last_error = msg; }

xc_status fail(xc_status st, const std::string& msg) {
  set_error(msg);
  return st;
}

xc_status from_cuda(cudaError_t err, const char* what) {
  set_error(std::string(what) + ": " + cudaGetErrorName(err) + " (" + cudaGetErrorString(err) + ")");
  return XC_ERR_CUDA;
}

const char* last_error_cstr() { return g_last_error.c_str(); }

// ---------------------------------------------------------------------------
// TMA descriptor encoding through the runtime's driver entry point.
// ---------------------------------------------------------------------------
namespace {
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* ptr = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(ptr);
  });
  return fn;
}
}  // namespace

bool encode_tiled(CUtensorMap* map, CUtensorMapDataType dtype, int rank, const void* base, const uint64_t* dims,
                  const uint64_t* byte_strides, const uint32_t* box, CUtensorMapSwizzle swizzle) {
  EncodeTiledFn fn = encode_fn();
  if (fn == nullptr) {
    set_error("cuTensorMapEncodeTiled is not available from the driver");
    return false;
  }
  cuuint64_t d[5], s[4];
  cuuint32_t b[5], e[5];
  for (int i = 0; i < rank; ++i) {
    d[i] = dims[i];
    b[i] = box[i];
    e[i] = 1;
  }
  for (int i = 0; i < rank - 1; ++i) s[i] = byte_strides[i];
  CUresult r = fn(map, dtype, (cuuint32_t)rank, const_cast<void*>(base), d, s, b, e, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  swizzle, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed with CUresult " + std::to_string((int)r));
    return false;
  }
  return true;
}

// ---------------------------------------------------------------------------
// Identity of the calling thread's current CUDA context: cuCtxGetId's ID,
// unique for the life of the process, so a context that replaced an earlier
// one (after cudaDeviceReset) never shares it.  Taken through the runtime's
// driver entry points (no link to libcuda); 0 when unavailable or when no
// context is current yet.
// ---------------------------------------------------------------------------
namespace {
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);
template <typename F>
F driver_fn(const char* name, int version) {
  void* ptr = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion(name, &ptr, version, cudaEnableDefault, &q) == cudaSuccess &&
      q == cudaDriverEntryPointSuccess)
    return reinterpret_cast<F>(ptr);
  return nullptr;
}
}  // namespace

unsigned long long current_context_id() {
  static const CtxGetCurrentFn get_current = driver_fn<CtxGetCurrentFn>("cuCtxGetCurrent", 12000);
  static const CtxGetIdFn get_id = driver_fn<CtxGetIdFn>("cuCtxGetId", 12000);
  if (get_current == nullptr || get_id == nullptr) return 0;
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// ---------------------------------------------------------------------------
// Device flag word: a file-scope __device__ variable (no allocation).  Its
// device address is looked up with the device current, once per device and
// context (looked up again after a context reset; on every call when the
// context's identity is unavailable).
// ---------------------------------------------------------------------------
__device__ DeviceFlags g_device_flags;

namespace {
std::mutex g_flag_mutex;
DeviceFlags* g_flags[64] = {nullptr};
unsigned long long g_flags_ctx[64] = {0};
}  // namespace

DeviceFlags* device_flags() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  const unsigned long long ctx = current_context_id();
  std::lock_guard<std::mutex> lock(g_flag_mutex);
  if (g_flags[dev] == nullptr || ctx == 0 || g_flags_ctx[dev] != ctx) {
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_device_flags) != cudaSuccess) return nullptr;
    g_flags[dev] = static_cast<DeviceFlags*>(ptr);
    g_flags_ctx[dev] = ctx;
  }
  return g_flags[dev];
}

xc_status check_device_flags(cudaStream_t stream) {
  DeviceFlags* f = device_flags();
  if (f == nullptr) return XC_OK;
  DeviceFlags h;
  XC_CUDA_TRY(cudaMemcpyAsync(&h, f, sizeof(h), cudaMemcpyDeviceToHost, stream));
  XC_CUDA_TRY(cudaStreamSynchronize(stream));
  if (h.timeout != 0) {
    XC_CUDA_TRY(cudaMemsetAsync(f, 0, sizeof(DeviceFlags), stream));
    return fail(XC_ERR_TIMEOUT, "a bounded device wait expired (site " + std::to_string(h.where) + ")");
  }
  return XC_OK;
}

// ---------------------------------------------------------------------------
// Bounded-wait test hook: an mbarrier with one expected arrival that never
// comes; the wait gives up after `polls` polls and records site 99.
// ---------------------------------------------------------------------------
__global__ void expire_wait_kernel(DeviceFlags* flags, uint32_t polls) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0 && !mbar_wait_bounded(&bar, 0, polls)) record_timeout(flags, 99);
}

xc_status debug_expire_wait(uint32_t polls, cudaStream_t stream) {
  DeviceFlags* f = device_flags();
  if (f == nullptr) return fail(XC_ERR_CUDA, "device flag word unavailable");
  expire_wait_kernel<<<1, 32, 0, stream>>>(f, polls);
  XC_CUDA_TRY(cudaGetLastError());
  return XC_OK;
}

// ---------------------------------------------------------------------------
// Kernel timing: event pairs around each dense kernel launch while enabled.
// Events come from a pool that grows on demand and is reused after a read.
// ---------------------------------------------------------------------------
namespace {
struct KernelTimer {
  std::mutex mu;
  bool on = false;
  std::vector<cudaEvent_t> pool;  // 2 per slot
  size_t used = 0;                // slots recorded since the last enable
};
KernelTimer& ktimer() {
  static KernelTimer t;
  return t;
}
}  // namespace

int kernel_timer_begin(cudaStream_t stream) {
  KernelTimer& t = ktimer();
  std::lock_guard<std::mutex> lock(t.mu);
  if (!t.on) return -1;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return -1;
  while (t.pool.size() < 2 * (t.used + 1)) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return -1;
    t.pool.push_back(e);
  }
  const int slot = (int)t.used++;
  if (cudaEventRecord(t.pool[2 * slot], stream) != cudaSuccess) return -1;
  return slot;
}

void kernel_timer_end(int slot, cudaStream_t stream) {
  if (slot < 0) return;
  KernelTimer& t = ktimer();
  std::lock_guard<std::mutex> lock(t.mu);
  cudaEventRecord(t.pool[2 * slot + 1], stream);
}

xc_status kernel_timing(int enable) {
  KernelTimer& t = ktimer();
  std::lock_guard<std::mutex> lock(t.mu);
  t.on = enable != 0;
  t.used = 0;
  return XC_OK;
}

xc_status kernel_timing_read(double* total_ms, uint32_t* launches) {
  KernelTimer& t = ktimer();
  std::lock_guard<std::mutex> lock(t.mu);
  double sum = 0.0;
  for (size_t k = 0; k < t.used; ++k) {
    XC_CUDA_TRY(cudaEventSynchronize(t.pool[2 * k + 1]));
    float ms = 0.f;
    XC_CUDA_TRY(cudaEventElapsedTime(&ms, t.pool[2 * k], t.pool[2 * k + 1]));
    sum += ms;
  }
  *total_ms = sum;
  *launches = (uint32_t)t.used;
  return XC_OK;
}

// ---------------------------------------------------------------------------
// Mode -> pair map (src/validate.hpp:216-298).
// ---------------------------------------------------------------------------
bool make_pair_map(xc_mode mode, uint32_t n_left, uint32_t n_right, PairMap* pm, uint64_t* n_out) {
  if (n_left == 0 || n_right == 0) return false;
  PairMap m;
  m.n_left = (int)n_left;
  switch (mode) {
    case XC_ONE_TO_ONE:
      if (n_left != 1 || n_right != 1) return false;
      m.K = 1;
      m.o_l = 0; m.o_k = 1; m.r_l = 0; m.r_k = 1;
      *n_out = 1;
      break;
    case XC_ONE_TO_MANY:
      if (n_left != 1) return false;
      m.K = (int)n_right;
      m.o_l = 0; m.o_k = 1; m.r_l = 0; m.r_k = 1;
      *n_out = n_right;
      break;
    case XC_N_TO_MN:
      if (n_right % n_left != 0) return false;
      m.K = (int)(n_right / n_left);
      m.o_l = 1; m.o_k = n_left; m.r_l = 1; m.r_k = n_left;
      *n_out = n_right;
      break;
    case XC_N_TO_M:
      m.K = (int)n_right;
      m.o_l = n_right; m.o_k = 1; m.r_l = 0; m.r_k = 1;
      *n_out = (uint64_t)n_left * n_right;
      break;
    default:
      return false;
  }
  *pm = m;
  return true;
}

}  // namespace xc
