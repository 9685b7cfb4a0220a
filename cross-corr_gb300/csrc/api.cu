// api.cu -- the C ABI (include/xcorr.h): argument checks, method dispatch,
// per-thread caches of FFT plans and device buffers, and the drop-in
// launchers for the reference's run_* kernel-launch layer (src/kernels.cuh).
#include <cuda.h>
#include <cufft.h>

#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "xc_common.cuh"
#include "xc_internal.h"

namespace xc {
const char* last_error_cstr();
}  // namespace xc

using namespace xc;

namespace {

cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

xc_status check_sizes(xc_size2 left, xc_size2 right) {
  if (left.x == 0 || left.y == 0 || right.x == 0 || right.y == 0)
    return fail(XC_ERR_INVALID_ARGUMENT, "matrix sizes must be positive");
  if ((uint64_t)left.x + right.x - 1 > 0x7fffffffu || (uint64_t)left.y + right.y - 1 > 0x7fffffffu)
    return fail(XC_ERR_INVALID_ARGUMENT, "matrix sizes too large");
  return XC_OK;
}

size_t elem_size(xc_dtype d) { return d == XC_F32 ? sizeof(float) : sizeof(double); }

// Per-thread cache of FFT plans, keyed by the full problem description.
using PlanKey = std::tuple<int, int, uint32_t, uint32_t, uint32_t, uint32_t, uint32_t, uint32_t, int>;
struct PlanDeleter {
  void operator()(FftPlanImpl* p) const { fft_plan_destroy(p); }
};

// One slot of the host-buffer pipeline: the device copies of one call's
// inputs and output, its band counters, and the events that order its copies
// and its correlation.  Two slots let one call's copies overlap the
// neighbouring calls' kernels (xc_correlate_host_async).
struct HostSlot {
  void* d_left = nullptr;
  void* d_right = nullptr;
  void* d_out = nullptr;
  size_t left_bytes = 0, right_bytes = 0, out_bytes = 0;
  int* d_bands = nullptr;          // band completion counters of the split path (8 ints)
  cudaEvent_t ev_in = nullptr;     // inputs copied in
  cudaEvent_t ev_start = nullptr;  // band counters cleared
  cudaEvent_t ev_comp = nullptr;   // correlation done: inputs and workspace free
  cudaEvent_t ev_out = nullptr;    // output copied out: the call is complete
  uint64_t ticket = 0;             // the call that used the slot last
  bool pending = false;            // enqueued and not yet waited for

  xc_status create_events() {
    for (cudaEvent_t* e : {&ev_in, &ev_start, &ev_comp, &ev_out})
      XC_CUDA_TRY(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    return XC_OK;
  }
  void release() {
    cudaFree(d_left);
    cudaFree(d_right);
    cudaFree(d_out);
    cudaFree(d_bands);
    d_left = d_right = d_out = nullptr;
    d_bands = nullptr;
    left_bytes = right_bytes = out_bytes = 0;
    for (cudaEvent_t* e : {&ev_in, &ev_start, &ev_comp, &ev_out}) {
      if (*e != nullptr) cudaEventDestroy(*e);
      *e = nullptr;
    }
    pending = false;
  }
};

struct ThreadCache {
  std::map<PlanKey, std::unique_ptr<FftPlanImpl, PlanDeleter>> plans;
  // xc_correlate_host[_async] buffers (grow-only): two slots, and one
  // workspace that the calls' correlations share (they run one after another)
  HostSlot slots[2];
  void* d_ws = nullptr;
  size_t ws_bytes = 0;
  uint64_t next_ticket = 1;
  int device = -1;
  // copy-in and copy-out streams, a stream for reading the device flags, and
  // the per-chunk events of the chunked (large-output) pipeline
  cudaStream_t s_in = nullptr, s_out = nullptr, s_flag = nullptr;
  cudaEvent_t ev_start = nullptr, ev_in[4] = {}, ev_comp[4] = {};

  xc_status ensure_streams() {
    if (s_in != nullptr) return XC_OK;
    XC_CUDA_TRY(cudaStreamCreateWithFlags(&s_in, cudaStreamNonBlocking));
    XC_CUDA_TRY(cudaStreamCreateWithFlags(&s_out, cudaStreamNonBlocking));
    XC_CUDA_TRY(cudaStreamCreateWithFlags(&s_flag, cudaStreamNonBlocking));
    XC_CUDA_TRY(cudaEventCreateWithFlags(&ev_start, cudaEventDisableTiming));
    for (int i = 0; i < 4; ++i) {
      XC_CUDA_TRY(cudaEventCreateWithFlags(&ev_in[i], cudaEventDisableTiming));
      XC_CUDA_TRY(cudaEventCreateWithFlags(&ev_comp[i], cudaEventDisableTiming));
    }
    for (HostSlot& sl : slots) XC_TRY(sl.create_events());
    return XC_OK;
  }

  void release() {
    // calls still in flight finish before their buffers go
    for (HostSlot& sl : slots)
      if (sl.pending) cudaEventSynchronize(sl.ev_out);
    if (s_in != nullptr) {
      cudaStreamSynchronize(s_in);
      cudaStreamSynchronize(s_out);
    }
    plans.clear();
    for (HostSlot& sl : slots) sl.release();
    cudaFree(d_ws);
    d_ws = nullptr;
    ws_bytes = 0;
    if (s_in != nullptr) {
      cudaStreamDestroy(s_in);
      cudaStreamDestroy(s_out);
      cudaStreamDestroy(s_flag);
      cudaEventDestroy(ev_start);
      for (int i = 0; i < 4; ++i) {
        cudaEventDestroy(ev_in[i]);
        cudaEventDestroy(ev_comp[i]);
      }
      s_in = s_out = s_flag = nullptr;
    }
  }
  ~ThreadCache() {
    // Process teardown may already have destroyed the CUDA context; only the
    // host side is released here.
    for (auto& kv : plans) kv.second.release();
  }
};

ThreadCache& cache() {
  static thread_local ThreadCache c;
  int dev = 0;
  cudaGetDevice(&dev);
  if (c.device != dev) {
    if (c.device >= 0) {
      int cur = dev;
      cudaSetDevice(c.device);
      c.release();
      cudaSetDevice(cur);
    }
    c.device = dev;
  }
  return c;
}

// cuStreamWaitValue32 through the runtime's driver entry point (no link to
// libcuda); null when the driver has none.
using WaitValue32 = CUresult (*)(CUstream, CUdeviceptr, cuuint32_t, unsigned int);
WaitValue32 wait_value32() {
  static const WaitValue32 fn = []() -> WaitValue32 {
    void* ptr = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuStreamWaitValue32", &ptr, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return reinterpret_cast<WaitValue32>(ptr);
    return nullptr;
  }();
  return fn;
}

// Split tensor-core path with the output copied out in row bands while the
// kernel runs: the kernel counts each band's finished work items, and the
// copy stream waits on each count (stream memory wait) before a 2D copy of
// the band's rows of every output.  Inputs are already on the device.
xc_status host_banded_tc(ThreadCache& c, HostSlot& sl, xc_mode mode, bool tf32, xc_size2 left, uint32_t n_left,
                         xc_size2 right, uint32_t n_right, uint64_t n_out, void* h_out, int n_bands, cudaStream_t s) {
  const Geometry g = make_geometry(left, right);
  PairMap pm;
  uint64_t tmp = 0;
  if (!make_pair_map(mode, n_left, n_right, &pm, &tmp)) return fail(XC_ERR_INVALID_ARGUMENT, "bad pair map");
  XC_CUDA_TRY(cudaMemsetAsync(sl.d_bands, 0, 8 * sizeof(int), s));
  XC_CUDA_TRY(cudaEventRecord(sl.ev_start, s));
  XC_CUDA_TRY(cudaStreamWaitEvent(c.s_out, sl.ev_start, 0));
  TcBands bands;
  XC_TRY(tc_correlate_banded((const float*)sl.d_left, (const float*)sl.d_right, (float*)sl.d_out, g, pm, c.d_ws,
                             c.ws_bytes, s, tf32, n_bands, sl.d_bands, &bands));
  const size_t row = (size_t)g.Sx * sizeof(float), mat = row * g.Sy;
  // Once the kernel is queued, a failure to queue a band's wait or copy still
  // lets the copies already queued finish (the release after the kernel
  // frees every wait) before the call returns: none may write into h_out
  // after the caller has it back.
  const auto drain = [&](xc_status st, const char* what) {
    cudaStreamSynchronize(c.s_out);
    cudaStreamSynchronize(s);
    return fail(st, what);
  };
  for (int k = 0; k < bands.n; ++k) {
    const int b = bands.order[k];
    if (wait_value32()(reinterpret_cast<CUstream>(c.s_out), reinterpret_cast<CUdeviceptr>(sl.d_bands + b),
                       (cuuint32_t)bands.items[b], CU_STREAM_WAIT_VALUE_GEQ) != CUDA_SUCCESS)
      return drain(XC_ERR_CUDA, "stream wait on an output band failed");
    const size_t off = row * bands.row_lo[b];
    if (cudaMemcpy2DAsync(static_cast<char*>(h_out) + off, mat, static_cast<char*>(sl.d_out) + off, mat,
                          row * (bands.row_hi[b] - bands.row_lo[b]), n_out, cudaMemcpyDeviceToHost,
                          c.s_out) != cudaSuccess)
      return drain(XC_ERR_CUDA, "copy of an output band failed to queue");
  }
  return XC_OK;
}


xc_status cached_plan(xc_mode mode, xc_dtype dtype, xc_size2 left, uint32_t n_left, xc_size2 right,
                      uint32_t n_right, FftPlanImpl** plan) {
  ThreadCache& c = cache();
  PlanKey key{(int)mode, (int)dtype, left.x, left.y, n_left, right.x, right.y, n_right, 0};
  auto it = c.plans.find(key);
  if (it != c.plans.end()) {
    *plan = it->second.get();
    return XC_OK;
  }
  FftPlanImpl* p = nullptr;
  XC_TRY(fft_plan_create(&p, mode, dtype, left, n_left, right, n_right, xc_size2{0, 0}));
  c.plans.emplace(key, std::unique_ptr<FftPlanImpl, PlanDeleter>(p));
  *plan = p;
  return XC_OK;
}

size_t fft_workspace_bytes(xc_mode mode, xc_dtype dtype, xc_size2 left, uint32_t n_left, xc_size2 right,
                           uint32_t n_right) {
  PairMap pm;
  uint64_t n_out = 0;
  if (!make_pair_map(mode, n_left, n_right, &pm, &n_out)) return 0;
  long long py, px;
  if (left.x == right.x && left.y == right.y) {
    py = 2LL * left.y;
    px = 2LL * left.x;
  } else {
    // upper bound: the smooth size found at plan time is at most 2x the full size
    py = 2LL * (left.y + right.y);
    px = 2LL * (left.x + right.x);
  }
  const long long bins = py * (px / 2 + 1);
  const size_t ce = 2 * elem_size(dtype);
  return (size_t)(n_left + n_right) * bins * ce + (size_t)n_out * bins * ce + 256;
}

// ---------------------------------------------------------------------------
// Algorithm selection for XC_METHOD_AUTO: the MLP's prediction when weights
// are installed, else the last exhaustive-autotune result for the problem,
// else (in xc_correlate, which has the buffers) an exhaustive autotune.
// ---------------------------------------------------------------------------
// The selector's candidates, in the order of the network's outputs: the
// plain kernel's three tile shapes, the FFT path, the split-BF16 path with
// items of at most 32 or 64 left rows, the split-TF32 path.
const xc_algo kAlgos[XC_N_ALGOS] = {{XC_METHOD_DIRECT, 1}, {XC_METHOD_DIRECT, 2},    {XC_METHOD_DIRECT, 3},
                                    {XC_METHOD_FFT, 0},    {XC_METHOD_TC_BF16X3, 32}, {XC_METHOD_TC_BF16X3, 64},
                                    {XC_METHOD_TC_TF32X3, 0}};
std::mutex g_sel_mutex;
#if __has_include("selector_weights.inc")
#include "selector_weights.inc"
#endif
#ifdef XC_SELECTOR_BUILTIN
static_assert(sizeof(kSelectorBuiltin) / sizeof(float) == XC_MLP_PARAMS, "built-in selector size");
std::vector<float> g_sel_params(kSelectorBuiltin, kSelectorBuiltin + XC_MLP_PARAMS);
#else
std::vector<float> g_sel_params;  // empty: no network installed
#endif
using SelKey = std::tuple<int, int, uint32_t, uint32_t, uint32_t, uint32_t, uint32_t, uint32_t>;
std::map<SelKey, xc_algo> g_tuned;

bool method_supported(xc_method m, xc_dtype dtype, xc_size2 left, xc_size2 right) {
  if (m == XC_METHOD_TC_BF16X3 || m == XC_METHOD_TC_TF32X3)
    // FP32 only; sizes with Wl + Wr below 6400 (the mean-correction kernel's staging)
    return dtype == XC_F32 && (uint64_t)left.x + right.x + 2 <= 6400;
  return m == XC_METHOD_DIRECT || m == XC_METHOD_FFT;
}

// Tiles: plain kernel 0 (its default) to 3; FFT 0; split paths 0 (items of
// at most 64 left rows) or the item length cap, 4 to 1024.
bool tile_valid(xc_algo a) {
  switch (a.method) {
    case XC_METHOD_DIRECT: return a.tile >= 0 && a.tile <= 3;
    case XC_METHOD_FFT: return a.tile == 0;
    case XC_METHOD_TC_BF16X3:
    case XC_METHOD_TC_TF32X3: return a.tile == 0 || (a.tile >= 4 && a.tile <= 1024);
    default: return false;
  }
}

void selector_features(xc_mode mode, xc_size2 left, uint32_t n_left, xc_size2 right, uint32_t n_right,
                       uint64_t n_out, float* f) {
  const double la = std::log2((double)left.x * left.y), ra = std::log2((double)right.x * right.y);
  f[0] = (float)(la / 22.0);
  f[1] = (float)(ra / 22.0);
  f[2] = (float)(std::log2((double)n_out) / 8.0);
  for (int i = 0; i < 4; ++i) f[3 + i] = (int)mode == i ? 1.0f : 0.0f;
  f[7] = (float)((la + ra + std::log2((double)n_out)) / 64.0);
  (void)n_left;
  (void)n_right;
}

// Host copy of the network's forward pass (same arithmetic as mlp.cu).
void host_forward(const std::vector<float>& P, const float* x, float* y) {
  const int IN = XC_MLP_IN, H = XC_MLP_HIDDEN, OUT = XC_MLP_OUT;
  const float* W1 = P.data();
  const float* b1 = W1 + H * IN;
  const float* W2 = b1 + H;
  const float* b2 = W2 + H * H;
  const float* W3 = b2 + H;
  const float* b3 = W3 + OUT * H;
  float h1[XC_MLP_HIDDEN], h2[XC_MLP_HIDDEN];
  for (int j = 0; j < H; ++j) {
    float a = b1[j];
    for (int i = 0; i < IN; ++i) a = std::fma(W1[j * IN + i], x[i], a);
    h1[j] = std::max(a, 0.0f);
  }
  for (int j = 0; j < H; ++j) {
    float a = b2[j];
    for (int k = 0; k < H; ++k) a = std::fma(W2[j * H + k], h1[k], a);
    h2[j] = std::max(a, 0.0f);
  }
  for (int o = 0; o < OUT; ++o) {
    float a = b3[o];
    for (int k = 0; k < H; ++k) a = std::fma(W3[o * H + k], h2[k], a);
    y[o] = a;
  }
}

// The algorithm XC_METHOD_AUTO runs: the network's fastest prediction among
// the supported candidates, else the tuning record; false when neither
// exists.
bool select_algorithm(xc_mode mode, xc_dtype dtype, xc_size2 left, uint32_t n_left, xc_size2 right,
                      uint32_t n_right, xc_algo* algo) {
  std::lock_guard<std::mutex> lock(g_sel_mutex);
  PairMap pm;
  uint64_t n_out = 1;
  if (!make_pair_map(mode, n_left, n_right, &pm, &n_out)) return false;
  if (!g_sel_params.empty()) {
    float f[XC_MLP_IN], y[XC_MLP_OUT];
    selector_features(mode, left, n_left, right, n_right, n_out, f);
    host_forward(g_sel_params, f, y);
    int best = -1;
    for (int o = 0; o < XC_MLP_OUT; ++o)
      if (method_supported(kAlgos[o].method, dtype, left, right) && (best < 0 || y[o] < y[best])) best = o;
    if (best >= 0) {
      *algo = kAlgos[best];
      return true;
    }
  }
  auto it = g_tuned.find(SelKey{(int)mode, (int)dtype, left.x, left.y, n_left, right.x, right.y, n_right});
  if (it == g_tuned.end()) return false;
  *algo = it->second;
  return true;
}

size_t algo_workspace(xc_mode mode, xc_dtype dtype, xc_algo a, xc_size2 left, uint32_t n_left, xc_size2 right,
                      uint32_t n_right, const PairMap& pm) {
  switch (a.method) {
    case XC_METHOD_FFT: return fft_workspace_bytes(mode, dtype, left, n_left, right, n_right);
    case XC_METHOD_TC_BF16X3:
    case XC_METHOD_TC_TF32X3:
      return dtype == XC_F32 ? tc_workspace_size(make_geometry(left, right), pm, a.method == XC_METHOD_TC_TF32X3) : 0;
    default: return 0;
  }
}

// One correlation with a given algorithm (method and tile); arguments
// already checked.
xc_status run_algo(xc_mode mode, xc_dtype dtype, xc_algo a, const void* d_left, xc_size2 left, uint32_t n_left,
                   const void* d_right, xc_size2 right, uint32_t n_right, void* d_out, void* d_workspace,
                   size_t workspace_bytes, cudaStream_t stream) {
  if (!tile_valid(a)) return fail(XC_ERR_INVALID_ARGUMENT, "invalid tile for the method");
  PairMap pm;
  uint64_t n_out;
  make_pair_map(mode, n_left, n_right, &pm, &n_out);
  const Geometry g = make_geometry(left, right);
  switch (a.method) {
    case XC_METHOD_DIRECT:
      return direct_launch(dtype, d_left, d_right, d_out, g, pm, stream, -1, DirectAccumulate::kAuto, a.tile);
    case XC_METHOD_FFT: {
      FftPlanImpl* plan = nullptr;
      XC_TRY(cached_plan(mode, dtype, left, n_left, right, n_right, &plan));
      return fft_plan_execute(plan, d_left, d_right, d_out, 1, d_workspace, workspace_bytes, stream);
    }
    case XC_METHOD_TC_BF16X3:
    case XC_METHOD_TC_TF32X3:
      if (dtype != XC_F32) return fail(XC_ERR_UNSUPPORTED, "the split tensor-core paths are FP32 only");
      return tc_correlate((const float*)d_left, (const float*)d_right, (float*)d_out, g, pm, d_workspace,
                          workspace_bytes, stream, a.method == XC_METHOD_TC_TF32X3, a.tile == 0 ? 64 : a.tile);
    default: return fail(XC_ERR_INVALID_ARGUMENT, "unknown method");
  }
}

}  // namespace

extern "C" {

const char* xc_version(void) { return "xcorr-gb300 0.1.0 (sm_103a)"; }

const char* xc_status_string(xc_status s) {
  switch (s) {
    case XC_OK: return "ok";
    case XC_ERR_INVALID_ARGUMENT: return "invalid argument";
    case XC_ERR_CUDA: return "CUDA error";
    case XC_ERR_CUFFT: return "cuFFT error";
    case XC_ERR_UNSUPPORTED: return "unsupported";
    case XC_ERR_WORKSPACE: return "workspace too small";
    case XC_ERR_TIMEOUT: return "device wait timed out";
  }
  return "unknown status";
}

const char* xc_last_error(void) { return last_error_cstr(); }

xc_status xc_device_check(int device) {
  cudaDeviceProp prop;
  XC_CUDA_TRY(cudaGetDeviceProperties(&prop, device));
  if (prop.major != 10 || prop.minor != 3)
    return fail(XC_ERR_UNSUPPORTED, std::string("device ") + prop.name + " is sm_" + std::to_string(prop.major) +
                                        std::to_string(prop.minor) + "; this library is built for sm_103a");
  return XC_OK;
}

xc_status xc_check_device(void* stream) { return check_device_flags(as_stream(stream)); }

xc_status xc_debug_expire_wait(uint32_t polls, void* stream) {
  if (polls == 0 || polls > (1u << 24)) return fail(XC_ERR_INVALID_ARGUMENT, "polls must be in [1, 2^24]");
  return debug_expire_wait(polls, as_stream(stream));
}

xc_status xc_kernel_timing(int enable) { return kernel_timing(enable); }

xc_status xc_kernel_timing_read(double* total_ms, uint32_t* launches) {
  if (total_ms == nullptr || launches == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "NULL result pointer");
  return kernel_timing_read(total_ms, launches);
}

xc_status xc_output_count(xc_mode mode, uint32_t n_left, uint32_t n_right, uint64_t* n_out) {
  PairMap pm;
  if (n_out == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "n_out is NULL");
  if (!make_pair_map(mode, n_left, n_right, &pm, n_out))
    return fail(XC_ERR_INVALID_ARGUMENT, "invalid matrix counts " + std::to_string(n_left) + " x " +
                                             std::to_string(n_right) + " for mode " + std::to_string((int)mode));
  return XC_OK;
}

xc_status xc_output_size(xc_size2 left, xc_size2 right, xc_size2* out) {
  if (out == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "out is NULL");
  XC_TRY(check_sizes(left, right));
  out->x = left.x + right.x - 1;
  out->y = left.y + right.y - 1;
  return XC_OK;
}

xc_status xc_workspace_size(xc_mode mode, xc_dtype dtype, xc_method method, xc_size2 left, uint32_t n_left,
                            xc_size2 right, uint32_t n_right, size_t* bytes) {
  if (bytes == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "bytes is NULL");
  XC_TRY(check_sizes(left, right));
  PairMap pm;
  uint64_t n_out;
  if (!make_pair_map(mode, n_left, n_right, &pm, &n_out)) return fail(XC_ERR_INVALID_ARGUMENT, "invalid counts");
  if (method == XC_METHOD_AUTO) {
    xc_algo a;
    if (select_algorithm(mode, dtype, left, n_left, right, n_right, &a)) {
      *bytes = algo_workspace(mode, dtype, a, left, n_left, right, n_right, pm);
    } else {
      // undecided (the first call autotunes): enough for any candidate
      *bytes = 0;
      for (const xc_algo& c : kAlgos)
        if (method_supported(c.method, dtype, left, right))
          *bytes = std::max(*bytes, algo_workspace(mode, dtype, c, left, n_left, right, n_right, pm));
    }
    return XC_OK;
  }
  switch (method) {
    case XC_METHOD_DIRECT:
    case XC_METHOD_FFT:
      *bytes = algo_workspace(mode, dtype, xc_algo{method, 0}, left, n_left, right, n_right, pm);
      return XC_OK;
    case XC_METHOD_TC_BF16X3:
    case XC_METHOD_TC_TF32X3:
      if (dtype != XC_F32) return fail(XC_ERR_UNSUPPORTED, "the split tensor-core paths are FP32 only");
      *bytes = algo_workspace(mode, dtype, xc_algo{method, 0}, left, n_left, right, n_right, pm);
      return XC_OK;
    default: return fail(XC_ERR_INVALID_ARGUMENT, "unknown method");
  }
}

xc_status xc_correlate(xc_mode mode, xc_dtype dtype, xc_method method, const void* d_left, xc_size2 left,
                       uint32_t n_left, const void* d_right, xc_size2 right, uint32_t n_right, void* d_out,
                       void* d_workspace, size_t workspace_bytes, void* stream) {
  if (d_left == nullptr || d_right == nullptr || d_out == nullptr)
    return fail(XC_ERR_INVALID_ARGUMENT, "NULL device buffer");
  if (dtype != XC_F32 && dtype != XC_F64) return fail(XC_ERR_INVALID_ARGUMENT, "unknown dtype");
  XC_TRY(check_sizes(left, right));
  PairMap pm;
  uint64_t n_out;
  if (!make_pair_map(mode, n_left, n_right, &pm, &n_out))
    return fail(XC_ERR_INVALID_ARGUMENT, "invalid matrix counts for the mode");
  xc_algo a{method, 0};
  if (method == XC_METHOD_AUTO && !select_algorithm(mode, dtype, left, n_left, right, n_right, &a)) {
    // no network and no record for this problem: the exhaustive autotune on
    // these buffers decides (and is remembered)
    double ms = 0.0;
    XC_TRY(xc_autotune_algorithm(mode, dtype, d_left, left, n_left, d_right, right, n_right, d_out, stream, &a, &ms));
  }
  if (a.method != XC_METHOD_DIRECT && a.method != XC_METHOD_FFT && a.method != XC_METHOD_TC_BF16X3 &&
      a.method != XC_METHOD_TC_TF32X3)
    return fail(XC_ERR_INVALID_ARGUMENT, "unknown method");
  return run_algo(mode, dtype, a, d_left, left, n_left, d_right, right, n_right, d_out, d_workspace,
                  workspace_bytes, as_stream(stream));
}

xc_status xc_correlate_algo(xc_mode mode, xc_dtype dtype, xc_algo algo, const void* d_left, xc_size2 left,
                            uint32_t n_left, const void* d_right, xc_size2 right, uint32_t n_right, void* d_out,
                            void* d_workspace, size_t workspace_bytes, void* stream) {
  if (d_left == nullptr || d_right == nullptr || d_out == nullptr)
    return fail(XC_ERR_INVALID_ARGUMENT, "NULL device buffer");
  if (dtype != XC_F32 && dtype != XC_F64) return fail(XC_ERR_INVALID_ARGUMENT, "unknown dtype");
  XC_TRY(check_sizes(left, right));
  PairMap pm;
  uint64_t n_out;
  if (!make_pair_map(mode, n_left, n_right, &pm, &n_out))
    return fail(XC_ERR_INVALID_ARGUMENT, "invalid matrix counts for the mode");
  if (algo.method == XC_METHOD_AUTO) return xc_correlate(mode, dtype, XC_METHOD_AUTO, d_left, left, n_left, d_right,
                                                         right, n_right, d_out, d_workspace, workspace_bytes, stream);
  if (!method_supported(algo.method, dtype, left, right))
    return fail(XC_ERR_UNSUPPORTED, "the method does not support this problem");
  return run_algo(mode, dtype, algo, d_left, left, n_left, d_right, right, n_right, d_out, d_workspace,
                  workspace_bytes, as_stream(stream));
}

}  // extern "C"

namespace {

// Waits for the call in `sl`, if it has not been waited for: its output
// copied out and its correlation finished (its buffers and the workspace are
// then free); its status.
xc_status finish_slot(ThreadCache& c, HostSlot& sl) {
  if (!sl.pending) return XC_OK;
  sl.pending = false;
  XC_CUDA_TRY(cudaEventSynchronize(sl.ev_out));
  XC_CUDA_TRY(cudaEventSynchronize(sl.ev_comp));
  return check_device_flags(c.s_flag);
}

// Enqueues one host-buffer correlation in pipeline slot ticket % 2: copy-in
// on the copy-in stream, the correlation on the caller's stream, copy-out on
// the copy-out stream.  With `after_stream` the copies also wait for work
// already queued on the caller's stream.  Problems cut into chunks (192 MiB
// of output or more) run to completion here.
xc_status host_submit(xc_mode mode, xc_dtype dtype, xc_method method, const void* h_left, xc_size2 left,
                      uint32_t n_left, const void* h_right, xc_size2 right, uint32_t n_right, void* h_out,
                      void* stream, bool after_stream, uint64_t* ticket) {
  if (ticket == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "ticket is NULL");
  if (h_left == nullptr || h_right == nullptr || h_out == nullptr)
    return fail(XC_ERR_INVALID_ARGUMENT, "NULL host buffer");
  XC_TRY(check_sizes(left, right));
  uint64_t n_out;
  XC_TRY(xc_output_count(mode, n_left, n_right, &n_out));
  const size_t es = elem_size(dtype);
  const size_t lsz = (size_t)left.x * left.y * es, rsz = (size_t)right.x * right.y * es;
  const size_t osz = (size_t)(left.x + right.x - 1) * (left.y + right.y - 1) * es;
  const size_t lb = lsz * n_left, rb = rsz * n_right, ob = osz * n_out;

  // Pipelining: the problem is cut into chunks along one axis of the pair
  // map -- the partners (one_to_many, n_to_mn) or the left matrices (n_to_m)
  // -- each a problem of the same mode.  Chunk i's input copy, correlation
  // and output copy run on three streams, so copies overlap the correlation
  // of neighbouring chunks.  Each correlation call has a fixed cost (prep
  // kernels, a partly filled last wave): at 64 outputs of 511x511 FP32
  // (67 MB) one chunk measured 28.4k correlations/s, two 27.3k, four 21.0k,
  // so a chunk carries at least 192 MiB of output.  XC_HOST_CHUNKS fixes the
  // count (studies, tests).
  PairMap pm;
  uint64_t tmp = 0;
  make_pair_map(mode, n_left, n_right, &pm, &tmp);
  const bool by_left = mode == XC_N_TO_M;
  const int axis = mode == XC_ONE_TO_ONE ? 1 : (by_left ? (int)n_left : pm.K);
  int n_chunks = (int)std::min<size_t>(std::min<size_t>(4, (size_t)axis), ob / ((size_t)192 << 20));
  if (const char* e = std::getenv("XC_HOST_CHUNKS")) n_chunks = std::min(std::max(1, std::atoi(e)), std::min(4, axis));
  if (n_chunks < 1) n_chunks = 1;
  // The split tensor-core path instead copies the output out in row bands
  // while its kernel runs (one call, no per-chunk costs): eight bands from
  // 16 MiB of output (measured on 64 outputs of 511x511: 1, 2, 4 and 8 bands
  // took 1.91, 1.84, 1.88 and 1.78 ms).  A stream of calls
  // (xc_correlate_host_async) copies the output out after the kernel
  // instead: the next call's kernel hides that copy, and the kernel runs
  // with its own work list rather than a banded schedule (at 64 outputs of
  // 511x511 in a stream of calls: 1.149 ms per call against 1.221 with
  // bands; kernel 1.036 against 1.063 ms).  XC_HOST_BANDS fixes the count
  // (1 turns bands off).
  xc_algo sel{method, 0};
  if (method == XC_METHOD_AUTO && !select_algorithm(mode, dtype, left, n_left, right, n_right, &sel))
    sel = xc_algo{XC_METHOD_AUTO, 0};  // the first chunk's call autotunes
  const xc_method resolved = sel.method;
  int n_bands = after_stream && ob >= ((size_t)16 << 20) ? 8 : 1;
  if (const char* e = std::getenv("XC_HOST_BANDS")) n_bands = std::max(1, std::atoi(e));
  const bool banded = (resolved == XC_METHOD_TC_BF16X3 || resolved == XC_METHOD_TC_TF32X3) && dtype == XC_F32 &&
                      n_bands > 1 && std::getenv("XC_HOST_CHUNKS") == nullptr && wait_value32() != nullptr &&
                      method_supported(resolved, dtype, left, right);
  if (banded) n_chunks = 1;
  const int per = (axis + n_chunks - 1) / n_chunks;
  n_chunks = (axis + per - 1) / per;
  auto chunk_shape = [&](int i, uint32_t* nl, uint32_t* nr, size_t* l_off, size_t* r_off, size_t* o_off,
                         size_t* l_len, size_t* r_len, size_t* o_len) {
    const int a0 = i * per, a1 = std::min(axis, a0 + per), na = a1 - a0;
    if (n_chunks == 1) {
      *nl = n_left; *nr = n_right; *l_off = *r_off = *o_off = 0; *l_len = lb; *r_len = rb; *o_len = ob;
    } else if (by_left) {  // n_to_m: lefts [a0, a1), every right, outputs l*K + k
      *nl = (uint32_t)na; *nr = n_right;
      *l_off = lsz * a0; *l_len = lsz * na; *r_off = 0; *r_len = i == 0 ? rb : 0;
      *o_off = osz * (size_t)a0 * n_right; *o_len = osz * (size_t)na * n_right;
    } else {  // one_to_many / n_to_mn: partners [a0, a1) of every left
      const int n = pm.n_left;
      *nl = n_left; *nr = (uint32_t)(na * n);
      *l_off = 0; *l_len = i == 0 ? lb : 0;
      *r_off = rsz * (size_t)a0 * n; *r_len = rsz * (size_t)na * n;
      *o_off = osz * (size_t)a0 * n; *o_len = osz * (size_t)na * n;
    }
  };
  size_t wb = 0;
  for (int i = 0; i < n_chunks; ++i) {
    uint32_t nl, nr;
    size_t a, b, c2, d, e, f;
    chunk_shape(i, &nl, &nr, &a, &b, &c2, &d, &e, &f);
    size_t w = 0;
    XC_TRY(xc_workspace_size(mode, dtype, banded ? resolved : method, left, nl, right, nr, &w));
    wb = std::max(wb, w);
  }
  ThreadCache& c = cache();
  XC_TRY(c.ensure_streams());
  const uint64_t t = c.next_ticket;
  HostSlot& sl = c.slots[t % 2];
  HostSlot& other = c.slots[(t + 1) % 2];
  // the call two tickets back used this slot: it completes before the
  // slot's buffers are reused (a failure of it is reported here)
  XC_TRY(finish_slot(c, sl));
  ++c.next_ticket;
  *ticket = t;
  sl.ticket = t;
  // the shared workspace is regrown, and chunked problems run, only with
  // the other slot's call complete
  if (n_chunks > 1 || wb > c.ws_bytes) XC_TRY(finish_slot(c, other));
  auto grow = [](void** p, size_t* have, size_t need) -> xc_status {
    if (need <= *have) return XC_OK;
    cudaFree(*p);
    *p = nullptr;
    *have = 0;
    XC_CUDA_TRY(cudaMalloc(p, need));
    *have = need;
    return XC_OK;
  };
  XC_TRY(grow(&sl.d_left, &sl.left_bytes, lb));
  XC_TRY(grow(&sl.d_right, &sl.right_bytes, rb));
  XC_TRY(grow(&sl.d_out, &sl.out_bytes, ob));
  if (wb > 0) XC_TRY(grow(&c.d_ws, &c.ws_bytes, wb));
  if (banded && sl.d_bands == nullptr) XC_CUDA_TRY(cudaMalloc(&sl.d_bands, 8 * sizeof(int)));
  cudaStream_t s = as_stream(stream);
  // Once a copy is queued, a failure lets everything queued finish before
  // returning: no copy may touch the caller's buffers after the call.
  const auto enqueue = [&]() -> xc_status {
    if (after_stream || n_chunks > 1) {
      // the copy streams start after work already queued on the caller's stream
      XC_CUDA_TRY(cudaEventRecord(c.ev_start, s));
      XC_CUDA_TRY(cudaStreamWaitEvent(c.s_in, c.ev_start, 0));
      XC_CUDA_TRY(cudaStreamWaitEvent(c.s_out, c.ev_start, 0));
    }
    if (n_chunks > 1) {
      char* dl = static_cast<char*>(sl.d_left);
      char* dr = static_cast<char*>(sl.d_right);
      char* dout = static_cast<char*>(sl.d_out);
      for (int i = 0; i < n_chunks; ++i) {
        uint32_t nl, nr;
        size_t l_off, r_off, o_off, l_len, r_len, o_len;
        chunk_shape(i, &nl, &nr, &l_off, &r_off, &o_off, &l_len, &r_len, &o_len);
        if (l_len) XC_CUDA_TRY(cudaMemcpyAsync(dl + l_off, static_cast<const char*>(h_left) + l_off, l_len,
                                               cudaMemcpyHostToDevice, c.s_in));
        if (r_len) XC_CUDA_TRY(cudaMemcpyAsync(dr + r_off, static_cast<const char*>(h_right) + r_off, r_len,
                                               cudaMemcpyHostToDevice, c.s_in));
        XC_CUDA_TRY(cudaEventRecord(c.ev_in[i], c.s_in));
        XC_CUDA_TRY(cudaStreamWaitEvent(s, c.ev_in[i], 0));
        // a chunk reads every left (partner chunks) or every right (n_to_m):
        // those were copied with chunk 0, which this stream has already waited for
        const char* cl = by_left ? dl + l_off : dl;
        const char* cr = by_left ? dr : dr + r_off;
        XC_TRY(xc_correlate(mode, dtype, method, cl, left, nl, cr, right, nr, dout + o_off, c.d_ws, c.ws_bytes,
                            stream));
        XC_CUDA_TRY(cudaEventRecord(c.ev_comp[i], s));
        XC_CUDA_TRY(cudaStreamWaitEvent(c.s_out, c.ev_comp[i], 0));
        XC_CUDA_TRY(cudaMemcpyAsync(static_cast<char*>(h_out) + o_off, dout + o_off, o_len, cudaMemcpyDeviceToHost,
                                    c.s_out));
      }
      return XC_OK;
    }
    XC_CUDA_TRY(cudaMemcpyAsync(sl.d_left, h_left, lb, cudaMemcpyHostToDevice, c.s_in));
    XC_CUDA_TRY(cudaMemcpyAsync(sl.d_right, h_right, rb, cudaMemcpyHostToDevice, c.s_in));
    XC_CUDA_TRY(cudaEventRecord(sl.ev_in, c.s_in));
    XC_CUDA_TRY(cudaStreamWaitEvent(s, sl.ev_in, 0));
    // the workspace is free once the other slot's correlation is done
    XC_CUDA_TRY(cudaStreamWaitEvent(s, other.ev_comp, 0));
    if (banded) {
      XC_TRY(host_banded_tc(c, sl, mode, resolved == XC_METHOD_TC_TF32X3, left, n_left, right, n_right, n_out, h_out,
                            n_bands, s));
      XC_CUDA_TRY(cudaEventRecord(sl.ev_comp, s));
    } else {
      XC_TRY(xc_correlate(mode, dtype, method, sl.d_left, left, n_left, sl.d_right, right, n_right, sl.d_out, c.d_ws,
                          c.ws_bytes, stream));
      XC_CUDA_TRY(cudaEventRecord(sl.ev_comp, s));
      XC_CUDA_TRY(cudaStreamWaitEvent(c.s_out, sl.ev_comp, 0));
      XC_CUDA_TRY(cudaMemcpyAsync(h_out, sl.d_out, ob, cudaMemcpyDeviceToHost, c.s_out));
    }
    XC_CUDA_TRY(cudaEventRecord(sl.ev_out, c.s_out));
    return XC_OK;
  };
  const xc_status st = enqueue();
  if (st != XC_OK || n_chunks > 1) {
    cudaStreamSynchronize(c.s_in);
    cudaStreamSynchronize(c.s_out);
    cudaStreamSynchronize(s);
    XC_TRY(st);
    return check_device_flags(s);
  }
  sl.pending = true;
  return XC_OK;
}

}  // namespace

extern "C" {

xc_status xc_correlate_host(xc_mode mode, xc_dtype dtype, xc_method method, const void* h_left, xc_size2 left,
                            uint32_t n_left, const void* h_right, xc_size2 right, uint32_t n_right, void* h_out,
                            void* stream) {
  uint64_t t = 0;
  XC_TRY(host_submit(mode, dtype, method, h_left, left, n_left, h_right, right, n_right, h_out, stream, true, &t));
  XC_TRY(xc_host_wait(t));
  XC_CUDA_TRY(cudaStreamSynchronize(as_stream(stream)));
  return XC_OK;
}

xc_status xc_correlate_host_async(xc_mode mode, xc_dtype dtype, xc_method method, const void* h_left, xc_size2 left,
                                  uint32_t n_left, const void* h_right, xc_size2 right, uint32_t n_right, void* h_out,
                                  void* stream, uint64_t* ticket) {
  return host_submit(mode, dtype, method, h_left, left, n_left, h_right, right, n_right, h_out, stream, false,
                     ticket);
}

xc_status xc_host_wait(uint64_t ticket) {
  ThreadCache& c = cache();
  if (ticket == 0 || ticket >= c.next_ticket) return fail(XC_ERR_INVALID_ARGUMENT, "unknown ticket");
  HostSlot& sl = c.slots[ticket % 2];
  // a reused slot means the call completed (and was waited for) already
  if (sl.ticket != ticket) return XC_OK;
  return finish_slot(c, sl);
}

void xc_release_thread_cache(void) { cache().release(); }

// ---------------------------------------------------------------------------
// Explicit FFT plans
// ---------------------------------------------------------------------------
struct xc_fft_plan_s {
  FftPlanImpl* impl;
};

xc_status xc_fft_plan_create(xc_fft_plan* plan, xc_mode mode, xc_dtype dtype, xc_size2 left, uint32_t n_left,
                             xc_size2 right, uint32_t n_right, xc_size2 pad) {
  if (plan == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "plan is NULL");
  *plan = nullptr;
  XC_TRY(check_sizes(left, right));
  FftPlanImpl* impl = nullptr;
  XC_TRY(fft_plan_create(&impl, mode, dtype, left, n_left, right, n_right, pad));
  *plan = new xc_fft_plan_s{impl};
  return XC_OK;
}

xc_status xc_fft_plan_workspace_size(xc_fft_plan plan, size_t* bytes) {
  if (plan == nullptr || bytes == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "NULL argument");
  *bytes = fft_plan_workspace(plan->impl);
  return XC_OK;
}

xc_status xc_fft_plan_pad_size(xc_fft_plan plan, xc_size2* pad) {
  if (plan == nullptr || pad == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "NULL argument");
  *pad = fft_plan_pad(plan->impl);
  return XC_OK;
}

xc_status xc_fft_execute(xc_fft_plan plan, const void* d_left, const void* d_right, void* d_out, int normalize,
                         void* d_workspace, size_t workspace_bytes, void* stream) {
  if (plan == nullptr || d_left == nullptr || d_right == nullptr || d_out == nullptr)
    return fail(XC_ERR_INVALID_ARGUMENT, "NULL argument");
  return fft_plan_execute(plan->impl, d_left, d_right, d_out, normalize, d_workspace, workspace_bytes,
                          as_stream(stream));
}

xc_status xc_fft_forward(xc_fft_plan plan, const void* d_left, const void* d_right, void* d_workspace,
                         size_t workspace_bytes, void* stream) {
  if (plan == nullptr || d_left == nullptr || d_right == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "NULL argument");
  return fft_plan_forward(plan->impl, d_left, d_right, d_workspace, workspace_bytes, as_stream(stream));
}

xc_status xc_fft_multiply(xc_fft_plan plan, void* d_workspace, size_t workspace_bytes, void* stream) {
  if (plan == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "NULL plan");
  return fft_plan_multiply(plan->impl, d_workspace, workspace_bytes, as_stream(stream));
}

xc_status xc_fft_inverse(xc_fft_plan plan, void* d_out, int normalize, void* d_workspace, size_t workspace_bytes,
                         void* stream) {
  if (plan == nullptr || d_out == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "NULL argument");
  return fft_plan_inverse(plan->impl, d_out, normalize, d_workspace, workspace_bytes, as_stream(stream));
}

xc_status xc_fft_plan_destroy(xc_fft_plan plan) {
  if (plan == nullptr) return XC_OK;
  fft_plan_destroy(plan->impl);
  delete plan;
  return XC_OK;
}

// ---------------------------------------------------------------------------
// Method selector
// ---------------------------------------------------------------------------
xc_status xc_selector_features(xc_mode mode, xc_size2 left, uint32_t n_left, xc_size2 right, uint32_t n_right,
                               float* features) {
  if (features == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "features is NULL");
  XC_TRY(check_sizes(left, right));
  uint64_t n_out = 0;
  XC_TRY(xc_output_count(mode, n_left, n_right, &n_out));
  selector_features(mode, left, n_left, right, n_right, n_out, features);
  return XC_OK;
}

xc_status xc_mlp_forward(const float* d_params, const float* d_x, uint32_t n, float* d_y, void* stream) {
  if (d_params == nullptr || d_x == nullptr || d_y == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "NULL pointer");
  return mlp_forward(d_params, d_x, n, d_y, as_stream(stream));
}

xc_status xc_mlp_gradient(const float* d_params, const float* d_x, const float* d_target, const float* d_mask,
                          uint32_t n, float mask_count, float* d_grad, float* d_loss, void* stream) {
  if (d_params == nullptr || d_x == nullptr || d_target == nullptr || d_mask == nullptr || d_grad == nullptr ||
      d_loss == nullptr)
    return fail(XC_ERR_INVALID_ARGUMENT, "NULL pointer");
  return mlp_gradient(d_params, d_x, d_target, d_mask, n, mask_count, d_grad, d_loss, as_stream(stream));
}

xc_status xc_mlp_adam_step(float* d_params, const float* d_grad, float* d_m, float* d_v, uint32_t step, float lr,
                           void* stream) {
  if (d_params == nullptr || d_grad == nullptr || d_m == nullptr || d_v == nullptr)
    return fail(XC_ERR_INVALID_ARGUMENT, "NULL pointer");
  if (step == 0) return fail(XC_ERR_INVALID_ARGUMENT, "Adam steps count from 1");
  return mlp_adam(d_params, d_grad, d_m, d_v, step, lr, as_stream(stream));
}

xc_status xc_selector_load(const float* h_params) {
  std::lock_guard<std::mutex> lock(g_sel_mutex);
  if (h_params == nullptr) g_sel_params.clear();
  else g_sel_params.assign(h_params, h_params + XC_MLP_PARAMS);
  return XC_OK;
}

xc_status xc_selector_load_builtin(void) {
#ifdef XC_SELECTOR_BUILTIN
  return xc_selector_load(kSelectorBuiltin);
#else
  return fail(XC_ERR_UNSUPPORTED, "library built without a selector network");
#endif
}

xc_status xc_algorithm(uint32_t index, xc_algo* algo) {
  if (algo == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "algo is NULL");
  if (index >= XC_N_ALGOS) return fail(XC_ERR_INVALID_ARGUMENT, "candidate index out of range");
  *algo = kAlgos[index];
  return XC_OK;
}

xc_status xc_select_algorithm(xc_mode mode, xc_dtype dtype, xc_size2 left, uint32_t n_left, xc_size2 right,
                              uint32_t n_right, xc_algo* algo) {
  if (algo == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "algo is NULL");
  XC_TRY(check_sizes(left, right));
  uint64_t n_out = 0;
  XC_TRY(xc_output_count(mode, n_left, n_right, &n_out));
  if (!select_algorithm(mode, dtype, left, n_left, right, n_right, algo)) *algo = xc_algo{XC_METHOD_AUTO, 0};
  return XC_OK;
}

xc_status xc_select_method(xc_mode mode, xc_dtype dtype, xc_size2 left, uint32_t n_left, xc_size2 right,
                           uint32_t n_right, xc_method* method) {
  if (method == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "method is NULL");
  xc_algo a;
  XC_TRY(xc_select_algorithm(mode, dtype, left, n_left, right, n_right, &a));
  *method = a.method;
  return XC_OK;
}

xc_status xc_time_algorithm(xc_mode mode, xc_dtype dtype, xc_algo algo, const void* d_left, xc_size2 left,
                            uint32_t n_left, const void* d_right, xc_size2 right, uint32_t n_right, void* d_out,
                            void* d_workspace, size_t workspace_bytes, uint32_t reps, void* stream, double* ms) {
  if (ms == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "ms is NULL");
  if (reps == 0) return fail(XC_ERR_INVALID_ARGUMENT, "reps must be positive");
  if (algo.method == XC_METHOD_AUTO) return fail(XC_ERR_INVALID_ARGUMENT, "time a concrete algorithm");
  cudaStream_t s = as_stream(stream);
  // the warm-up call also creates plans and checks the arguments
  XC_TRY(xc_correlate_algo(mode, dtype, algo, d_left, left, n_left, d_right, right, n_right, d_out, d_workspace,
                           workspace_bytes, stream));
  cudaEvent_t e0, e1;
  XC_CUDA_TRY(cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return fail(XC_ERR_CUDA, "cudaEventCreate failed");
  }
  xc_status st = XC_OK;
  float t = 0.f;
  if (cudaEventRecord(e0, s) != cudaSuccess) st = fail(XC_ERR_CUDA, "cudaEventRecord failed");
  for (uint32_t r = 0; r < reps && st == XC_OK; ++r)
    st = run_algo(mode, dtype, algo, d_left, left, n_left, d_right, right, n_right, d_out, d_workspace,
                  workspace_bytes, s);
  if (st == XC_OK && (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                      cudaEventElapsedTime(&t, e0, e1) != cudaSuccess))
    st = fail(XC_ERR_CUDA, "event timing failed");
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  XC_TRY(st);
  *ms = t / reps;
  return XC_OK;
}

xc_status xc_autotune_algorithm(xc_mode mode, xc_dtype dtype, const void* d_left, xc_size2 left, uint32_t n_left,
                                const void* d_right, xc_size2 right, uint32_t n_right, void* d_out, void* stream,
                                xc_algo* best, double* best_ms) {
  if (best == nullptr || best_ms == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "NULL result pointer");
  XC_TRY(check_sizes(left, right));
  PairMap pm;
  uint64_t n_out;
  if (!make_pair_map(mode, n_left, n_right, &pm, &n_out))
    return fail(XC_ERR_INVALID_ARGUMENT, "invalid matrix counts for the mode");
  double bms = 1e300;
  xc_algo ba{XC_METHOD_DIRECT, 0};
  xc_status st = XC_OK;
  for (const xc_algo& c : kAlgos) {
    if (!method_supported(c.method, dtype, left, right)) continue;
    const size_t wb = algo_workspace(mode, dtype, c, left, n_left, right, n_right, pm);
    void* ws = nullptr;
    if (wb > 0 && cudaMalloc(&ws, wb) != cudaSuccess) {
      st = fail(XC_ERR_CUDA, "workspace allocation failed");
      break;
    }
    double ms = 0.0;
    st = xc_time_algorithm(mode, dtype, c, d_left, left, n_left, d_right, right, n_right, d_out, ws, wb, 3, stream,
                           &ms);
    cudaFree(ws);
    if (st != XC_OK) break;
    if (ms < bms) {
      bms = ms;
      ba = c;
    }
  }
  XC_TRY(st);
  {
    std::lock_guard<std::mutex> lock(g_sel_mutex);
    g_tuned[SelKey{(int)mode, (int)dtype, left.x, left.y, n_left, right.x, right.y, n_right}] = ba;
  }
  *best = ba;
  *best_ms = bms;
  return XC_OK;
}

xc_status xc_autotune_method(xc_mode mode, xc_dtype dtype, const void* d_left, xc_size2 left, uint32_t n_left,
                             const void* d_right, xc_size2 right, uint32_t n_right, void* d_out, void* stream,
                             xc_method* best, double* best_ms) {
  if (best == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "NULL result pointer");
  xc_algo a;
  XC_TRY(xc_autotune_algorithm(mode, dtype, d_left, left, n_left, d_right, right, n_right, d_out, stream, &a,
                               best_ms));
  *best = a.method;
  return XC_OK;
}

// ---------------------------------------------------------------------------
// Ragged batches
// ---------------------------------------------------------------------------
struct xc_ragged_plan_s {
  RaggedPlanImpl* impl;
};

xc_status xc_ragged_plan_create(xc_ragged_plan* plan, xc_dtype dtype, const void* d_left,
                                const xc_matrix_desc* lefts, uint32_t n_left, const void* d_right,
                                const xc_matrix_desc* rights, uint32_t n_right, const xc_pair_desc* pairs,
                                uint32_t n_pairs, void* d_out) {
  if (plan == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "plan is NULL");
  *plan = nullptr;
  RaggedPlanImpl* impl = nullptr;
  XC_TRY(ragged_plan_create(&impl, dtype, d_left, lefts, n_left, d_right, rights, n_right, pairs, n_pairs, d_out));
  *plan = new xc_ragged_plan_s{impl};
  return XC_OK;
}

xc_status xc_ragged_autotune(xc_ragged_plan plan, void* stream, int* chosen_shape, double* best_ms) {
  if (plan == nullptr || chosen_shape == nullptr || best_ms == nullptr)
    return fail(XC_ERR_INVALID_ARGUMENT, "NULL argument");
  return ragged_autotune(plan->impl, as_stream(stream), chosen_shape, best_ms);
}

xc_status xc_ragged_describe(xc_ragged_plan plan, int variant, xc_ragged_variant* out) {
  if (plan == nullptr || out == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "NULL argument");
  return ragged_describe(plan->impl, variant, out);
}

xc_status xc_ragged_select(xc_ragged_plan plan, int variant) {
  if (plan == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "plan is NULL");
  return ragged_select(plan->impl, variant);
}

xc_status xc_ragged_execute(xc_ragged_plan plan, void* stream) {
  if (plan == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "plan is NULL");
  return ragged_execute(plan->impl, as_stream(stream));
}

xc_status xc_ragged_plan_destroy(xc_ragged_plan plan) {
  if (plan == nullptr) return XC_OK;
  ragged_plan_destroy(plan->impl);
  delete plan;
  return XC_OK;
}

xc_status xc_correlate_pairs(xc_dtype dtype, const void* d_left, const xc_matrix_desc* lefts, uint32_t n_left,
                             const void* d_right, const xc_matrix_desc* rights, uint32_t n_right,
                             const xc_pair_desc* pairs, uint32_t n_pairs, void* d_out, void* stream) {
  if (d_left == nullptr || d_right == nullptr || d_out == nullptr || lefts == nullptr || rights == nullptr ||
      pairs == nullptr)
    return fail(XC_ERR_INVALID_ARGUMENT, "NULL argument");
  return correlate_pairs(dtype, d_left, lefts, n_left, d_right, rights, n_right, pairs, n_pairs, d_out,
                         as_stream(stream));
}

// ---------------------------------------------------------------------------
// Drop-ins for the reference's run_* launchers (src/kernels.cuh).
// ---------------------------------------------------------------------------
}  // extern "C"

namespace {

xc_status check_search(xc_size2 matrix_size, xc_size2 search_size) {
  if (search_size.x != 2 * matrix_size.x - 1 || search_size.y != 2 * matrix_size.y - 1)
    return fail(XC_ERR_INVALID_ARGUMENT, "search_size must be 2*matrix_size-1 for equal-size inputs");
  return check_sizes(matrix_size, matrix_size);
}

xc_status check_warps(uint32_t warps) {
  // src/naive_shuffle.cu:461-463
  if (warps == 0 || warps > 32)
    return fail(XC_ERR_INVALID_ARGUMENT, "Too many warps per thread block: " + std::to_string(warps) + " (max 32)");
  return XC_OK;
}

xc_status check_limit(uint32_t v, uint32_t lo, uint32_t hi, const char* what) {
  if (v < lo || v > hi)
    return fail(XC_ERR_INVALID_ARGUMENT, std::string("Invalid ") + what + ": " + std::to_string(v) + " [" +
                                             std::to_string(lo) + "-" + std::to_string(hi) + "]");
  return XC_OK;
}

// The reference's distributions (src/row_distribution.cpp:7-11).  The
// rectangle and triangle forms divide by max_rows_per_thread
// (src/row_distribution.cuh:34-253); none ignores it.
xc_status check_distribution(uint32_t dist, uint32_t max_rows_per_thread) {
  if (dist > XC_DIST_TRIANGLE) return fail(XC_ERR_INVALID_ARGUMENT, "Unknown distribution " + std::to_string(dist));
  if (dist != XC_DIST_NONE && max_rows_per_thread == 0)
    return fail(XC_ERR_INVALID_ARGUMENT, "max_rows_per_thread must be positive for the rectangle and triangle "
                                         "distributions");
  return XC_OK;
}

// One launch of the plain kernel for a launcher drop-in.  `acc`: kAuto for
// the launchers that write their output, kCaller for the work-distribution
// launchers, which add into an output the caller zeroed
// (src/one_to_one.hpp:276-277), as the reference's atomic kernels do.
template <typename T>
xc_status run_mode(xc_mode mode, const T* left, const T* right, T* out, xc_size2 ms, uint32_t nl, uint32_t nr,
                   void* stream, DirectAccumulate acc = DirectAccumulate::kAuto) {
  PairMap pm;
  uint64_t n_out;
  if (!make_pair_map(mode, nl, nr, &pm, &n_out)) return fail(XC_ERR_INVALID_ARGUMENT, "invalid matrix counts");
  if (left == nullptr || right == nullptr || out == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "NULL pointer");
  return direct_launch(sizeof(T) == 4 ? XC_F32 : XC_F64, left, right, out, make_geometry(ms, ms), pm,
                       as_stream(stream), -1, acc);
}

}  // namespace

extern "C" {

#define XC_DEFINE_SHUFFLE(SUFFIX, T)                                                                             \
  xc_status xc_run_ccn_shuffle_##SUFFIX(const T* left, const T* right, T* out, xc_size2 matrix_size,             \
                                        xc_size2 search_size, uint32_t warps_per_thread_block, void* stream) {   \
    XC_TRY(check_warps(warps_per_thread_block));                                                                 \
    XC_TRY(check_search(matrix_size, search_size));                                                              \
    return run_mode<T>(XC_ONE_TO_ONE, left, right, out, matrix_size, 1, 1, stream);                              \
  }                                                                                                              \
  xc_status xc_run_ccn_shuffle_multimat_right_##SUFFIX(                                                          \
      const T* left, const T* right, T* out, xc_size2 matrix_size, xc_size2 search_size,                         \
      uint32_t num_right_matrices, uint32_t warps_per_thread_block, uint32_t right_matrices_per_thread,           \
      void* stream) {                                                                                            \
    XC_TRY(check_warps(warps_per_thread_block));                                                                 \
    XC_TRY(check_limit(right_matrices_per_thread, 1, 8, "number of right matrices per thread"));                \
    XC_TRY(check_search(matrix_size, search_size));                                                              \
    return run_mode<T>(XC_ONE_TO_MANY, left, right, out, matrix_size, 1, num_right_matrices, stream);            \
  }                                                                                                              \
  xc_status xc_run_ccn_shuffle_one_to_many_multirow_both_multimat_right_##SUFFIX(                                \
      const T* left, const T* right, T* out, xc_size2 matrix_size, xc_size2 search_size,                         \
      uint32_t num_right_matrices, uint32_t warps_per_thread_block, uint32_t shifts_per_thread_right_matrix,      \
      uint32_t right_matrices_per_thread, uint32_t left_rows_per_iteration, void* stream) {                      \
    XC_TRY(check_warps(warps_per_thread_block));                                                                 \
    XC_TRY(check_limit(shifts_per_thread_right_matrix, 0, 4, "shifts per thread in each right matrix"));         \
    XC_TRY(check_limit(right_matrices_per_thread, 1, 4, "number of right matrices per thread"));                \
    XC_TRY(check_limit(left_rows_per_iteration, 0, 4, "left rows per iteration"));                               \
    XC_TRY(check_search(matrix_size, search_size));                                                              \
    return run_mode<T>(XC_ONE_TO_MANY, left, right, out, matrix_size, 1, num_right_matrices, stream);            \
  }                                                                                                              \
  xc_status xc_run_ccn_n_to_m_shuffle_multirow_both_multimat_both_##SUFFIX(                                      \
      const T* left, const T* right, T* out, xc_size2 matrix_size, xc_size2 search_size,                         \
      uint32_t num_left_matrices, uint32_t num_right_matrices, uint32_t warps_per_thread_block,                  \
      uint32_t shifts_per_thread_right_matrix, uint32_t left_matrices_per_thread,                                \
      uint32_t right_matrices_per_thread, uint32_t left_rows_per_iteration, void* stream) {                      \
    XC_TRY(check_warps(warps_per_thread_block));                                                                 \
    XC_TRY(check_limit(shifts_per_thread_right_matrix, 0, 4, "shifts per thread per right matrix"));             \
    XC_TRY(check_limit(left_matrices_per_thread, 1, 4, "left matrices per thread"));                             \
    XC_TRY(check_limit(right_matrices_per_thread, 1, 4, "right matrices per thread"));                           \
    XC_TRY(check_limit(left_rows_per_iteration, 0, 4, "left rows per iteration"));                              \
    XC_TRY(check_search(matrix_size, search_size));                                                              \
    return run_mode<T>(XC_N_TO_M, left, right, out, matrix_size, num_left_matrices, num_right_matrices, stream);  \
  }

XC_DEFINE_SHUFFLE(f32, float)
XC_DEFINE_SHUFFLE(f64, double)

// The work-distribution, multirow and multirow-multimat launchers (and the
// local_mem:: twins of two of them).  Limits are the reference's release
// build values (CMakeLists.txt:16-43).
#define XC_DEFINE_SHUFFLE_MORE(SUFFIX, T)                                                                        \
  xc_status xc_run_ccn_shuffle_work_distribution_##SUFFIX(                                                       \
      const T* left, const T* right, T* out, xc_size2 matrix_size, xc_size2 search_size,                         \
      uint32_t warps_per_thread_block, uint32_t max_rows_per_thread, xc_distribution distribution,               \
      void* stream) {                                                                                            \
    XC_TRY(check_warps(warps_per_thread_block));                                                                 \
    XC_TRY(check_distribution((uint32_t)distribution, max_rows_per_thread));                                    \
    XC_TRY(check_search(matrix_size, search_size));                                                              \
    return run_mode<T>(XC_ONE_TO_ONE, left, right, out, matrix_size, 1, 1, stream, DirectAccumulate::kCaller);   \
  }                                                                                                              \
  xc_status xc_run_ccn_shuffle_multimat_right_work_distribution_##SUFFIX(                                        \
      const T* left, const T* right, T* out, xc_size2 matrix_size, xc_size2 search_size,                         \
      uint32_t num_right_matrices, uint32_t warps_per_thread_block, uint32_t right_matrices_per_thread,           \
      uint32_t max_rows_per_thread, xc_distribution distribution, void* stream) {                                \
    XC_TRY(check_warps(warps_per_thread_block));                                                                 \
    XC_TRY(check_limit(right_matrices_per_thread, 1, 8, "number of right matrices per thread"));                \
    XC_TRY(check_distribution((uint32_t)distribution, max_rows_per_thread));                                    \
    XC_TRY(check_search(matrix_size, search_size));                                                              \
    return run_mode<T>(XC_ONE_TO_MANY, left, right, out, matrix_size, 1, num_right_matrices, stream,             \
                       DirectAccumulate::kCaller);                                                               \
  }                                                                                                              \
  xc_status xc_run_ccn_shuffle_n_to_m_multimat_both_work_distribution_##SUFFIX(                                  \
      const T* left, const T* right, T* out, xc_size2 matrix_size, xc_size2 search_size,                         \
      uint32_t num_left_matrices, uint32_t num_right_matrices, uint32_t warps_per_thread_block,                  \
      uint32_t left_matrices_per_thread, uint32_t right_matrices_per_thread, uint32_t max_rows_per_thread,       \
      xc_distribution distribution, void* stream) {                                                              \
    XC_TRY(check_warps(warps_per_thread_block));                                                                 \
    XC_TRY(check_limit(left_matrices_per_thread, 1, 4, "left matrices per thread"));                             \
    XC_TRY(check_limit(right_matrices_per_thread, 1, 4, "right matrices per thread"));                           \
    XC_TRY(check_distribution((uint32_t)distribution, max_rows_per_thread));                                    \
    XC_TRY(check_search(matrix_size, search_size));                                                              \
    return run_mode<T>(XC_N_TO_M, left, right, out, matrix_size, num_left_matrices, num_right_matrices, stream,  \
                       DirectAccumulate::kCaller);                                                               \
  }                                                                                                              \
  xc_status xc_run_ccn_shuffle_n_to_m_multimat_both_work_distribution_local_mem_##SUFFIX(                        \
      const T* left, const T* right, T* out, xc_size2 matrix_size, xc_size2 search_size,                         \
      uint32_t num_left_matrices, uint32_t num_right_matrices, uint32_t warps_per_thread_block,                  \
      uint32_t left_matrices_per_thread, uint32_t right_matrices_per_thread, uint32_t max_rows_per_thread,       \
      xc_distribution distribution, void* stream) {                                                              \
    return xc_run_ccn_shuffle_n_to_m_multimat_both_work_distribution_##SUFFIX(                                   \
        left, right, out, matrix_size, search_size, num_left_matrices, num_right_matrices, warps_per_thread_block, \
        left_matrices_per_thread, right_matrices_per_thread, max_rows_per_thread, distribution, stream);          \
  }                                                                                                              \
  xc_status xc_run_ccn_shuffle_multirow_right_##SUFFIX(const T* left, const T* right, T* out,                    \
                                                       xc_size2 matrix_size, xc_size2 search_size,               \
                                                       uint32_t warps_per_thread_block,                          \
                                                       uint32_t right_rows_per_thread, void* stream) {           \
    XC_TRY(check_warps(warps_per_thread_block));                                                                 \
    XC_TRY(check_limit(right_rows_per_thread, 1, 8, "number of right rows per thread"));                        \
    XC_TRY(check_search(matrix_size, search_size));                                                              \
    return run_mode<T>(XC_ONE_TO_ONE, left, right, out, matrix_size, 1, 1, stream);                              \
  }                                                                                                              \
  xc_status xc_run_ccn_shuffle_multirow_both_##SUFFIX(const T* left, const T* right, T* out,                     \
                                                      xc_size2 matrix_size, xc_size2 search_size,                \
                                                      uint32_t warps_per_thread_block,                           \
                                                      uint32_t max_shifts_per_thread, uint32_t max_left_rows,    \
                                                      void* stream) {                                            \
    XC_TRY(check_warps(warps_per_thread_block));                                                                 \
    XC_TRY(check_limit(max_shifts_per_thread, 1, 8, "shifts per thread"));                                      \
    XC_TRY(check_limit(max_left_rows, 1, 4, "left rows per iteration"));                                         \
    XC_TRY(check_search(matrix_size, search_size));                                                              \
    return run_mode<T>(XC_ONE_TO_ONE, left, right, out, matrix_size, 1, 1, stream);                              \
  }                                                                                                              \
  xc_status xc_run_ccn_shuffle_multirow_both_local_mem_##SUFFIX(const T* left, const T* right, T* out,           \
                                                                xc_size2 matrix_size, xc_size2 search_size,      \
                                                                uint32_t warps_per_thread_block,                 \
                                                                uint32_t max_shifts_per_thread,                  \
                                                                uint32_t max_left_rows, void* stream) {          \
    return xc_run_ccn_shuffle_multirow_both_##SUFFIX(left, right, out, matrix_size, search_size,                 \
                                                     warps_per_thread_block, max_shifts_per_thread,              \
                                                     max_left_rows, stream);                                     \
  }                                                                                                              \
  xc_status xc_run_ccn_shuffle_multirow_right_multimat_right_##SUFFIX(                                           \
      const T* left, const T* right, T* out, xc_size2 matrix_size, xc_size2 search_size,                         \
      uint32_t num_right_matrices, uint32_t warps_per_thread_block, uint32_t right_rows_per_thread,               \
      uint32_t right_matrices_per_thread, void* stream) {                                                        \
    XC_TRY(check_warps(warps_per_thread_block));                                                                 \
    XC_TRY(check_limit(right_rows_per_thread, 1, 4, "number of right rows per thread"));                        \
    XC_TRY(check_limit(right_matrices_per_thread, 1, 4, "number of right matrices per thread"));                \
    XC_TRY(check_search(matrix_size, search_size));                                                              \
    return run_mode<T>(XC_ONE_TO_MANY, left, right, out, matrix_size, 1, num_right_matrices, stream);            \
  }

XC_DEFINE_SHUFFLE_MORE(f32, float)
XC_DEFINE_SHUFFLE_MORE(f64, double)

#define XC_DEFINE_FFT_GLUE(CSUF, RSUF, DT, T)                                                                     \
  xc_status xc_run_hadamard_original_##CSUF(const void* ref, void* deformed, xc_size2 subregion_size,            \
                                            uint32_t subregions_per_pic, uint32_t batch_size,                    \
                                            uint32_t threads_per_block, void* stream) {                          \
    if (ref == nullptr || deformed == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "NULL pointer");             \
    const long long area = (long long)subregion_size.x * subregion_size.y * subregions_per_pic;                  \
    return glue_hadamard_original(DT, ref, deformed, area, batch_size, (int)threads_per_block,                   \
                                  as_stream(stream));                                                            \
  }                                                                                                              \
  xc_status xc_run_hadamard_n_to_m_over_output_##CSUF(const void* left, const void* right, void* out,            \
                                                      xc_size2 matrix_size, uint32_t left_num, uint32_t right_num, \
                                                      uint32_t threads_per_block, uint32_t min_items_per_thread,  \
                                                      void* stream) {                                            \
    (void)threads_per_block;                                                                                     \
    (void)min_items_per_thread;                                                                                  \
    if (left == nullptr || right == nullptr || out == nullptr)                                                   \
      return fail(XC_ERR_INVALID_ARGUMENT, "NULL pointer");                                                      \
    if (left_num == 0 || right_num == 0) return fail(XC_ERR_INVALID_ARGUMENT, "empty batch");                    \
    return glue_hadamard_n_to_m(DT, left, right, out, (long long)matrix_size.x * matrix_size.y, (int)left_num,   \
                                (int)right_num, as_stream(stream));                                              \
  }                                                                                                              \
  xc_status xc_run_scatter_##RSUF(const T* src, T* dst, xc_size2 src_matrix_size, uint32_t src_num_matrices,     \
                                  xc_size2 dst_matrix_size, xc_size2 dst_pos, uint32_t threads_per_block,        \
                                  uint32_t items_per_thread, void* stream) {                                     \
    (void)threads_per_block;                                                                                     \
    (void)items_per_thread;                                                                                      \
    if (src == nullptr || dst == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "NULL pointer");                   \
    if (dst_pos.x + src_matrix_size.x > dst_matrix_size.x || dst_pos.y + src_matrix_size.y > dst_matrix_size.y)  \
      return fail(XC_ERR_INVALID_ARGUMENT, "source does not fit into the destination at dst_pos");               \
    return glue_pad(DT, src, dst, (int)src_matrix_size.y, (int)src_matrix_size.x, (int)src_num_matrices,         \
                    (int)dst_matrix_size.y, (int)dst_matrix_size.x, (int)dst_pos.y, (int)dst_pos.x,               \
                    as_stream(stream));                                                                          \
  }                                                                                                              \
  xc_status xc_normalize_fft_results_##RSUF(const T* raw, T* norm, xc_size2 raw_size, uint32_t count,            \
                                            void* stream) {                                                      \
    if (raw == nullptr || norm == nullptr) return fail(XC_ERR_INVALID_ARGUMENT, "NULL pointer");                 \
    if (raw_size.x < 2 || raw_size.y < 2) return fail(XC_ERR_INVALID_ARGUMENT, "raw size must be at least 2x2"); \
    /* The reference puts raw index 0 (shift 0) at norm index (size-1)/2       */                            \
    /* (src/fft_helpers.hpp:222-226): the generic map with Hr-1 = (size-1)/2.  */                            \
    const int Sy = (int)raw_size.y - 1, Sx = (int)raw_size.x - 1;                                                \
    return glue_normalize(DT, raw, norm, (int)raw_size.y, (int)raw_size.x, (int)count, Sy / 2 + 1, Sx / 2 + 1,   \
                          Sy, Sx, as_stream(stream));                                                            \
  }

XC_DEFINE_FFT_GLUE(c64, f32, XC_F32, float)
XC_DEFINE_FFT_GLUE(c128, f64, XC_F64, double)

}  // extern "C"
