// algorithms.cpp -- the algorithm registry of `cross run` and the step runner.
//
// Every algorithm name of the reference (get_algorithms, src/main.cpp:361-411)
// is registered with its JSON arguments and defaults (the plug-in
// constructors, e.g. src/one_to_one.hpp:182-186).  Names map onto the GB300
// methods of the C ABI:
//   cpu_*                -> CPU definition (single thread, like the reference)
//   nai_*                -> XC_METHOD_DIRECT (plain FP32/FP64 kernel)
//   fft_*                -> XC_METHOD_FFT (cuFFT + fused glue)
//   tc_bf16x3_*          -> XC_METHOD_TC_BF16X3 (new: split-BF16 tensor cores)
//   tc_tf32x3_*          -> XC_METHOD_TC_TF32X3 (new: split-TF32 tensor cores)
// The reference's tile arguments are validated with its limits and reported
// in the measurement CSV, but the GB300 kernels choose their own tiling.
//
// The run loop reproduces run_measurement / run_computation_steps
// (src/main.cpp:123-326): load, then per outer loop prepare, transfer, run,
// finalize, free, optional timing output, store and validation.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <functional>
#include <fstream>
#include <iostream>
#include <memory>
#include <sstream>
#include <thread>

#include "cross.hpp"

namespace cross {

namespace {

enum class kind { cpu, direct, fft_orig, fft_reduced, fft_better, tc, tc32 };

struct arg_def {
  std::string key;
  std::string def;  // default value as text
  enum { integer, string, boolean } type;
};

struct alg_spec {
  std::string name;
  xc_mode mode;
  kind k;
  std::vector<arg_def> args;
};

xc_mode mode_of(const std::string& n) {
  auto ends = [&](const std::string& s) { return n.size() >= s.size() && n.compare(n.size() - s.size(), s.size(), s) == 0; };
  if (ends("_one_to_one")) return XC_ONE_TO_ONE;
  if (ends("_one_to_many")) return XC_ONE_TO_MANY;
  if (ends("_n_to_mn")) return XC_N_TO_MN;
  return XC_N_TO_M;
}

const std::vector<alg_spec>& registry() {
  static const std::vector<alg_spec> algs = [] {
    using A = std::vector<arg_def>;
    auto I = [](const char* k, const char* d) { return arg_def{k, d, arg_def::integer}; };
    auto S = [](const char* k, const char* d) { return arg_def{k, d, arg_def::string}; };
    auto B = [](const char* k, const char* d) { return arg_def{k, d, arg_def::boolean}; };
    const A none;
    const A warps{I("warps_per_thread_block", "8")};
    const A wd_rect{I("warps_per_thread_block", "8"), I("rows_per_thread", "10"), S("distribution_type", "rectangle")};
    const A mm2{I("warps_per_thread_block", "8"), I("right_matrices_per_thread", "2")};
    const A mm_wd{I("warps_per_thread_block", "8"), I("right_matrices_per_thread", "2"), I("rows_per_thread", "10"),
                  S("distribution_type", "rectangle")};
    const A mm_wd_s{I("warps_per_thread_block", "8"), I("right_matrices_per_thread", "2"), I("rows_per_thread", "10"),
                    S("distribution_type", "rectangle"), I("num_cuda_streams", "8")};
    const A both_wd{I("warps_per_thread_block", "8"), I("left_matrices_per_thread", "2"),
                    I("right_matrices_per_thread", "2"), I("rows_per_thread", "10"), S("distribution_type", "triangle")};
    const A mrbmb{I("warps_per_thread_block", "8"), I("shifts_per_thread_right_matrix", "2"),
                  I("left_matrices_per_thread", "2"), I("right_matrices_per_thread", "2"),
                  I("left_rows_per_iteration", "2")};
    const A mr{I("warps_per_thread_block", "8"), I("right_rows_per_thread", "4")};
    const A mb{I("warps_per_thread_block", "8"), I("shifts_per_thread", "4"), I("left_rows_per_iteration", "3")};
    const A mrmr{I("warps_per_thread_block", "8"), I("right_rows_per_thread", "4"), I("right_matrices_per_thread", "4")};
    const A mrmr_s{I("warps_per_thread_block", "8"), I("right_rows_per_thread", "4"),
                   I("right_matrices_per_thread", "4"), I("num_cuda_streams", "8")};
    const A mbmr{I("warps_per_thread_block", "8"), I("shifts_per_thread_right_matrix", "4"),
                 I("right_matrices_per_thread", "4"), I("left_rows_per_iteration", "4")};
    const A mbmr_s{I("warps_per_thread_block", "8"), I("shifts_per_thread_right_matrix", "4"),
                   I("right_matrices_per_thread", "4"), I("left_rows_per_iteration", "4"), I("num_cuda_streams", "8")};
    const A wps{I("shifts_per_thread_block", "8")};
    const A wps_wd{I("shifts_per_thread_block", "8"), I("rows_per_warp", "3"), S("distribution_type", "rectangle")};
    auto shm = [&](const char* spb, bool mats, bool streams) {
      A a{I("shifts_per_thread_block", spb), I("shared_mem_row_size", "32"), I("shared_mem_rows", spb),
          B("strided_load", "true"), B("column_group_per_block", "false")};
      if (mats) a.push_back(I("right_matrices_per_block", "8"));
      if (streams) a.push_back(I("num_cuda_streams", "8"));
      return a;
    };
    const A fft{I("hadamard_threads_per_block", "256")};
    const A fft_rt{I("scatter_threads_per_block", "256"), I("scatter_items_per_thread", "10"),
                   I("hadamard_threads_per_block", "256")};
    const A fft_b{I("hadamard_threads_per_block", "256"), I("hadamard_items_per_thread", "10")};
    const A streams{I("num_cuda_streams", "8")};

    std::vector<std::pair<std::string, std::pair<kind, A>>> list = {
        {"cpu_one_to_one", {kind::cpu, none}},
        {"cpu_one_to_many", {kind::cpu, none}},
        {"cpu_n_to_mn", {kind::cpu, none}},
        {"cpu_n_to_m", {kind::cpu, none}},
        {"nai_orig_one_to_one", {kind::direct, none}},
        {"nai_orig_one_to_many", {kind::direct, none}},
        {"nai_orig_n_to_mn", {kind::direct, none}},
        {"nai_orig_n_to_m", {kind::direct, streams}},
        {"nai_shuffle_one_to_one", {kind::direct, warps}},
        {"nai_shuffle_work_distribution_one_to_one", {kind::direct, wd_rect}},
        {"nai_shuffle_multimat_right_one_to_one", {kind::direct, warps}},
        {"nai_shuffle_multimat_right_one_to_many", {kind::direct, mm2}},
        {"nai_shuffle_multimat_right_work_distribution_one_to_one", {kind::direct, wd_rect}},
        {"nai_shuffle_multimat_right_work_distribution_one_to_many", {kind::direct, mm_wd}},
        {"nai_shuffle_multimat_right_work_distribution_n_to_mn", {kind::direct, mm_wd_s}},
        {"nai_shuffle_multimat_right_work_distribution_n_to_m", {kind::direct, mm_wd_s}},
        {"nai_shuffle_multimat_both_work_distribution_local_mem_n_to_m", {kind::direct, both_wd}},
        {"nai_shuffle_multimat_both_work_distribution_n_to_m", {kind::direct, both_wd}},
        {"nai_shuffle_multirow_both_multimat_both_n_to_m", {kind::direct, mrbmb}},
        {"nai_shuffle_multirow_right_one_to_one", {kind::direct, mr}},
        {"nai_shuffle_multirow_both_one_to_one", {kind::direct, mb}},
        {"nai_shuffle_multirow_both_local_mem_one_to_one", {kind::direct, mb}},
        {"nai_shuffle_multirow_right_multimat_right_one_to_one", {kind::direct, mr}},
        {"nai_shuffle_multirow_right_multimat_right_one_to_many", {kind::direct, mrmr}},
        {"nai_shuffle_multirow_right_multimat_right_n_to_mn", {kind::direct, mrmr_s}},
        {"nai_shuffle_multirow_both_multimat_right_one_to_many", {kind::direct, mbmr}},
        {"nai_shuffle_multirow_both_multimat_right_n_to_mn", {kind::direct, mbmr_s}},
        {"nai_warp_per_shift_one_to_one", {kind::direct, wps}},
        {"nai_warp_per_shift_simple_indexing_one_to_one", {kind::direct, wps}},
        {"nai_warp_per_shift_work_distribution_one_to_one", {kind::direct, wps_wd}},
        {"nai_warp_per_shift_shared_mem_one_to_one", {kind::direct, shm("32", false, false)}},
        {"nai_warp_per_shift_shared_mem_one_to_many", {kind::direct, shm("16", true, false)}},
        {"nai_warp_per_shift_shared_mem_n_to_mn", {kind::direct, shm("16", true, true)}},
        {"nai_warp_per_shift_shared_mem_n_to_m", {kind::direct, shm("16", true, true)}},
        {"nai_block_per_shift_one_to_one", {kind::direct, {I("block_size", "128")}}},
        {"fft_orig_one_to_one", {kind::fft_orig, fft}},
        {"fft_reduced_transfer_one_to_one", {kind::fft_reduced, fft_rt}},
        {"fft_orig_one_to_many", {kind::fft_orig, fft}},
        {"fft_reduced_transfer_one_to_many", {kind::fft_reduced, fft_rt}},
        {"fft_orig_n_to_mn", {kind::fft_orig, fft}},
        {"fft_reduced_transfer_n_to_mn", {kind::fft_reduced, fft_rt}},
        {"fft_better_n_to_m", {kind::fft_better, fft_b}},
        // New in this library: split-BF16 tensor-core correlation (FP32 data).
        {"tc_bf16x3_one_to_one", {kind::tc, none}},
        {"tc_bf16x3_one_to_many", {kind::tc, none}},
        {"tc_bf16x3_n_to_mn", {kind::tc, none}},
        {"tc_bf16x3_n_to_m", {kind::tc, none}},
        {"tc_tf32x3_one_to_one", {kind::tc32, none}},
        {"tc_tf32x3_one_to_many", {kind::tc32, none}},
        {"tc_tf32x3_n_to_mn", {kind::tc32, none}},
        {"tc_tf32x3_n_to_m", {kind::tc32, none}},
    };
    std::vector<alg_spec> out;
    for (auto& e : list) out.push_back(alg_spec{e.first, mode_of(e.first), e.second.first, e.second.second});
    return out;
  }();
  return algs;
}

const alg_spec* find_alg(const std::string& name) {
  for (const auto& a : registry())
    if (a.name == name) return &a;
  return nullptr;
}

// Reads the algorithm's JSON arguments, checks them against the reference's
// launcher limits and returns the (key, value) list reported in the
// measurement file (additional_properties).
std::vector<std::pair<std::string, std::string>> resolve_args(const alg_spec& spec, const json_args& j) {
  std::vector<std::pair<std::string, std::string>> props;
  for (const auto& a : spec.args) {
    std::string v;
    if (a.type == arg_def::integer) {
      long long x = j.get_int(a.key, std::stoll(a.def));
      if (x < 0) throw argument_error(a.key + " must not be negative");
      if (a.key == "warps_per_thread_block" && (x == 0 || x > 32))
        throw std::runtime_error("Too many warps per thread block: " + std::to_string(x) + " (max 32)");
      if ((a.key == "right_matrices_per_thread" || a.key == "left_matrices_per_thread") && x == 0)
        throw std::runtime_error("Invalid number of matrices per thread: 0");
      v = std::to_string(x);
    } else if (a.type == arg_def::string) {
      v = j.get_str(a.key, a.def);
      if (a.key == "distribution_type" && v != "none" && v != "rectangle" && v != "triangle")
        throw argument_error("Unknown distribution type " + v);
    } else {
      v = j.get_bool(a.key, a.def == "true") ? "1" : "0";
    }
    props.emplace_back(a.key, v);
  }
  return props;
}

struct logger {
  bool progress;
  void log(const std::string& m) const {
    if (progress) std::cout << m << std::endl;
  }
};

void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

void xc_check(xc_status s, const char* what) {
  if (s != XC_OK) throw std::runtime_error(std::string(what) + ": " + xc_status_string(s) + ": " + xc_last_error());
}

// A measured duration per iteration and the iteration count
// (measurement_result, src/stopwatch.hpp:13-50).
struct measurement {
  std::chrono::nanoseconds per_iter{0};
  size_t iterations = 0;
};

// Adaptive repetition of src/stopwatch.hpp:57-71: repeat until the total
// reaches min_time, growing the count by clamp(1.5 * ratio, 1.5, 100).
measurement adaptive(std::chrono::nanoseconds min_time, const std::function<void()>& body, bool gpu,
                     bool host_only = false) {
  size_t iters = 1;
  for (;;) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    std::chrono::nanoseconds total;
    if (gpu) {
      cuda_check(cudaEventCreate(&e0), "cudaEventCreate");
      cuda_check(cudaEventCreate(&e1), "cudaEventCreate");
      cuda_check(cudaEventRecord(e0), "cudaEventRecord");
      for (size_t i = 0; i < iters; ++i) body();
      cuda_check(cudaEventRecord(e1), "cudaEventRecord");
      cuda_check(cudaEventSynchronize(e1), "cudaEventSynchronize");
      float ms = 0;
      cuda_check(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      total = std::chrono::nanoseconds((long long)std::llround((double)ms * 1e6));
    } else {
      auto t0 = std::chrono::steady_clock::now();
      for (size_t i = 0; i < iters; ++i) body();
      if (!host_only) cuda_check(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
      total = std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0);
    }
    if (total >= min_time || min_time.count() <= 0) return measurement{total / (long long)iters, iters};
    double ratio = (double)min_time.count() / std::max<double>(1.0, (double)total.count());
    iters = (size_t)std::ceil(iters * std::max(std::min(ratio * 1.5, 100.0), 1.5));
  }
}

measurement once(const std::function<void()>& body) {
  auto t0 = std::chrono::steady_clock::now();
  body();
  return measurement{std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0), 1};
}

// Output of the measurement CSV (output_measurements, src/main.cpp:90-121).
void write_measurements(const std::string& path, const std::vector<std::string>& labels,
                        const std::vector<measurement>& ms,
                        const std::vector<std::pair<std::string, std::string>>& props, bool append) {
  std::ofstream f;
  if (append) {
    f.open(path, std::ios_base::app);
  } else {
    f.open(path);
    const char* sep = "";
    for (const auto& l : labels) {
      f << sep << l << "," << l << "_iterations";
      sep = ",";
    }
    for (const auto& p : props) {
      f << sep << p.first;
      sep = ",";
    }
    f << "\n";
  }
  const char* sep = "";
  for (const auto& m : ms) {
    f << sep << m.per_iter.count() << "," << m.iterations;
    sep = ",";
  }
  for (const auto& p : props) {
    f << sep << p.second;
    sep = ",";
  }
  f << "\n";
}

// ---------------------------------------------------------------------------
// One algorithm instance: the cross_corr_alg steps (src/cross_corr.hpp:21-189).
// ---------------------------------------------------------------------------
template <typename T>
class instance {
 public:
  instance(const alg_spec& spec, const run_args& ra) : spec_(spec), ra_(ra) {}
  ~instance() { release(); }

  const alg_spec& spec() const { return spec_; }
  bool is_fft() const { return spec_.k == kind::fft_orig || spec_.k == kind::fft_reduced || spec_.k == kind::fft_better; }
  bool store_raw() const { return is_fft() && ra_.out_path && !ra_.normalize; }

  std::vector<std::string> alg_labels() const {
    switch (spec_.k) {
      case kind::cpu: return {};
      case kind::fft_orig:
      case kind::fft_better: return {"Forward FFT", "Hadamard", "Inverse FFT", "Allocation", "Plan"};
      case kind::fft_reduced: return {"Forward FFT", "Hadamard", "Inverse FFT", "ToDevice", "Scatter", "Allocation", "Plan"};
      default: return {"Kernel"};
    }
  }

  void load() {
    left_ = load_csv<T>(ra_.ref_path);
    right_ = load_csv<T>(ra_.target_path);
    if (left_.count == 0 || right_.count == 0 || left_.rows == 0 || left_.cols == 0 || right_.rows == 0 ||
        right_.cols == 0)
      throw std::runtime_error("Empty input matrices");
    uint64_t n_out = 0;
    if (xc_output_count(spec_.mode, left_.count, right_.count, &n_out) != XC_OK)
      throw std::runtime_error(std::string("Invalid input data counts: ") + xc_last_error());
    n_out_ = (uint32_t)n_out;
  }

  void prepare() {
    const uint32_t Sy = left_.rows + right_.rows - 1, Sx = left_.cols + right_.cols - 1;
    if (spec_.k == kind::cpu) {
      result_ = data_array<T>(Sy, Sx, n_out_);
      return;
    }
    const xc_dtype dt = sizeof(T) == 4 ? XC_F32 : XC_F64;
    if ((spec_.k == kind::tc || spec_.k == kind::tc32) && dt != XC_F32)
      throw std::runtime_error("tc_bf16x3_* and tc_tf32x3_* algorithms take -d single data");
    auto alloc = [&]() {
      cuda_check(cudaMalloc(&d_left_, left_.size() * sizeof(T)), "cudaMalloc");
      cuda_check(cudaMalloc(&d_right_, right_.size() * sizeof(T)), "cudaMalloc");
    };
    if (is_fft()) {
      measure_alloc_ = once([&] {
        alloc();
      });
      measure_plan_ = once([&] {
        xc_check(xc_fft_plan_create(&plan_, spec_.mode, dt, left_.size2(), left_.count, right_.size2(), right_.count,
                                    xc_size2{0, 0}),
                 "xc_fft_plan_create");
      });
      xc_size2 pad;
      xc_check(xc_fft_plan_pad_size(plan_, &pad), "xc_fft_plan_pad_size");
      if (store_raw()) result_ = data_array<T>(pad.y, pad.x, n_out_);
      else result_ = data_array<T>(Sy, Sx, n_out_);
      auto t = once([&] {
        xc_check(xc_fft_plan_workspace_size(plan_, &ws_bytes_), "xc_fft_plan_workspace_size");
        cuda_check(cudaMalloc(&d_ws_, ws_bytes_), "cudaMalloc");
        cuda_check(cudaMalloc(&d_out_, result_.size() * sizeof(T)), "cudaMalloc");
      });
      measure_alloc_.per_iter += t.per_iter;
    } else {
      alloc();
      result_ = data_array<T>(Sy, Sx, n_out_);
      cuda_check(cudaMalloc(&d_out_, result_.size() * sizeof(T)), "cudaMalloc");
      xc_check(xc_workspace_size(spec_.mode, dt, method(), left_.size2(), left_.count, right_.size2(), right_.count,
                                 &ws_bytes_),
               "xc_workspace_size");
      if (ws_bytes_ > 0) cuda_check(cudaMalloc(&d_ws_, ws_bytes_), "cudaMalloc");
    }
  }

  void transfer() {
    if (spec_.k == kind::cpu) return;
    auto copy = [&] {
      cuda_check(cudaMemcpy(d_left_, left_.data.data(), left_.size() * sizeof(T), cudaMemcpyHostToDevice), "H2D");
      cuda_check(cudaMemcpy(d_right_, right_.data.data(), right_.size() * sizeof(T), cudaMemcpyHostToDevice), "H2D");
    };
    if (spec_.k == kind::fft_reduced && ra_.bench == benchmark_type::Algorithm)
      measure_todevice_ = once(copy);
    else
      copy();
  }

  void run(bool measure_alg, std::chrono::nanoseconds min_time) {
    const xc_dtype dt = sizeof(T) == 4 ? XC_F32 : XC_F64;
    if (spec_.k == kind::cpu) {
      result_ = cpu_correlate<T, T>(spec_.mode, left_, right_, 1);
      return;
    }
    if (!is_fft()) {
      auto body = [&] {
        xc_check(xc_correlate(spec_.mode, dt, method(), d_left_, left_.size2(), left_.count, d_right_, right_.size2(),
                              right_.count, d_out_, d_ws_, ws_bytes_, nullptr),
                 "xc_correlate");
      };
      if (measure_alg) kernel_ = adaptive(min_time, body, true);
      else body();
      return;
    }
    const int normalize = store_raw() ? 0 : 1;
    auto fwd = [&] { xc_check(xc_fft_forward(plan_, d_left_, d_right_, d_ws_, ws_bytes_, nullptr), "xc_fft_forward"); };
    auto mul = [&] { xc_check(xc_fft_multiply(plan_, d_ws_, ws_bytes_, nullptr), "xc_fft_multiply"); };
    auto inv = [&] { xc_check(xc_fft_inverse(plan_, d_out_, normalize, d_ws_, ws_bytes_, nullptr), "xc_fft_inverse"); };
    if (measure_alg) {
      fwd_ = adaptive(min_time, fwd, true);
      had_ = adaptive(min_time, [&] { mul(); }, true);
      inv_ = adaptive(min_time, [&] {
        // the inverse transform is in place, so each repetition re-multiplies
        mul();
        inv();
      }, true);
      inv_.per_iter -= had_.per_iter;
      if (inv_.per_iter.count() < 0) inv_.per_iter = std::chrono::nanoseconds(0);
    } else {
      fwd();
      mul();
      inv();
    }
  }

  void finalize() {
    if (spec_.k == kind::cpu) return;
    cuda_check(cudaMemcpy(result_.data.data(), d_out_, result_.size() * sizeof(T), cudaMemcpyDeviceToHost), "D2H");
  }

  void release() {
    if (plan_) xc_fft_plan_destroy(plan_);
    plan_ = nullptr;
    cudaFree(d_left_);
    cudaFree(d_right_);
    cudaFree(d_out_);
    cudaFree(d_ws_);
    d_left_ = d_right_ = d_out_ = d_ws_ = nullptr;
  }

  std::vector<measurement> alg_measurements() const {
    switch (spec_.k) {
      case kind::cpu: return {};
      case kind::fft_orig:
      case kind::fft_better: return {fwd_, had_, inv_, measure_alloc_, measure_plan_};
      // The device pad is part of the forward step here; "Scatter" reports 0.
      case kind::fft_reduced: return {fwd_, had_, inv_, measure_todevice_, measurement{}, measure_alloc_, measure_plan_};
      default: return {kernel_};
    }
  }

  void store(const std::string& path) const {
    store_csv(path, result_);
  }

  // Result normalised as the reference's validate() does (src/cross_corr.hpp:90-97).
  data_array<T> normalized_result() const { return store_raw() ? normalize_fft_host(result_) : result_; }

  data_array<double> compute_valid() const {
    const int threads = (int)std::max(1u, std::thread::hardware_concurrency());
    return cpu_correlate<T, double>(spec_.mode, left_, right_, threads);
  }

 private:
  xc_method method() const {
    switch (spec_.k) {
      case kind::tc: return XC_METHOD_TC_BF16X3;
      case kind::tc32: return XC_METHOD_TC_TF32X3;
      case kind::direct: return XC_METHOD_DIRECT;
      default: return XC_METHOD_FFT;
    }
  }

  const alg_spec& spec_;
  const run_args& ra_;
  data_array<T> left_, right_, result_;
  uint32_t n_out_ = 0;
  void *d_left_ = nullptr, *d_right_ = nullptr, *d_out_ = nullptr, *d_ws_ = nullptr;
  size_t ws_bytes_ = 0;
  xc_fft_plan plan_ = nullptr;
  measurement kernel_, fwd_, had_, inv_, measure_alloc_, measure_plan_, measure_todevice_;
};

template <typename T>
int run_typed(const alg_spec& spec, const run_args& ra) {
  logger log{ra.progress && ra.bench != benchmark_type::Compute};
  json_args j;
  if (ra.args_path) j = json_args::parse_file(*ra.args_path);
  const auto props = resolve_args(spec, j);

  instance<T> alg(spec, ra);
  std::vector<measurement> common(7);
  try {
    log.log("Loading inputs");
    common[0] = once([&] { alg.load(); });
  } catch (std::exception& e) {
    std::cerr << "Exception occured durign data loading step: " << e.what() << std::endl;
    return 3;
  }

  const bool measure_alg = ra.bench == benchmark_type::Algorithm;
  const bool measure_common = ra.bench == benchmark_type::CommonSteps;
  // cpu_* algorithms never touch the GPU (and run on hosts without one).
  const bool host_only = spec.k == kind::cpu;
  for (size_t loop = 0; loop < ra.outer_loops; ++loop) {
    int ret = 0;
    auto steps = [&]() {
      struct step {
        const char* msg;
        const char* err;
        int idx;
        std::function<void()> fn;
        bool adaptive_run;
      };
      const step seq[] = {
          {"Allocating", "allocation", 1, [&] { alg.prepare(); }, false},
          {"Transfering data", "data transfer", 2, [&] { alg.transfer(); }, false},
          {"Running test alg", "computation", 3, [&] { alg.run(measure_alg, ra.min_time); }, true},
          {"Copying output data to host", "finalization", 4, [&] { alg.finalize(); }, false},
          {"Free resources", "free", 5, [&] { alg.release(); }, false},
      };
      for (const auto& s : seq) {
        try {
          log.log(s.msg);
          if (measure_common) {
            common[s.idx] = s.adaptive_run ? adaptive(ra.min_time, s.fn, false, host_only) : once([&] {
              s.fn();
              if (!host_only) cuda_check(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
            });
          } else {
            s.fn();
          }
        } catch (std::exception& e) {
          std::cerr << "Exception occured durign " << s.err << " step: " << e.what() << std::endl;
          ret = 3;
          return;
        }
      }
    };
    std::vector<measurement> compute(1);
    if (ra.bench == benchmark_type::Compute) {
      compute[0] = adaptive(ra.min_time, [&] {
        if (ret == 0) steps();
      }, false, host_only);
    } else {
      steps();
    }
    if (ret != 0) return ret;
    cudaError_t e = host_only ? cudaSuccess : cudaDeviceSynchronize();
    if (e == cudaSuccess && !host_only) e = cudaGetLastError();
    if (e != cudaSuccess) {
      std::cerr << "Exception somewhere in CUDA code: " << cudaGetErrorString(e) << std::endl;
      return 3;
    }

    std::optional<std::string> out_path = ra.out_path;
    if (out_path && ra.outer_loops > 1) {
      // get_loop_out_path (src/run_args.cpp:142-152): stem_<loop>.ext
      std::string p = *out_path;
      size_t slash = p.find_last_of('/');
      size_t dot = p.find_last_of('.');
      if (dot == std::string::npos || (slash != std::string::npos && dot < slash)) dot = p.size();
      out_path = p.substr(0, dot) + "_" + std::to_string(loop) + p.substr(dot);
    }
    if (out_path) {
      log.log(alg.is_fft() ? "Normalizing and storing results" : "Storing results");
      if (measure_common)
        common[6] = once([&] { alg.store(*out_path); });
      else
        alg.store(*out_path);
    }

    if (ra.bench != benchmark_type::None) {
      std::vector<std::string> labels;
      std::vector<measurement> ms;
      if (ra.bench == benchmark_type::Compute) {
        labels = {"Computation"};
        ms = compute;
      } else if (measure_common) {
        labels = {"Load", "Prepare", "Transfer", "Run", "Finalize", "Free", "Store"};
        ms = common;
      } else {
        labels = alg.alg_labels();
        ms = alg.alg_measurements();
      }
      write_measurements(ra.measurements_path, labels, ms, props, ra.append || loop > 0);
    }

    if (!ra.validate) {
      log.log("No validation");
    } else {
      validation_results r;
      if (!ra.validate_path.empty()) {
        log.log("Validating results against " + ra.validate_path);
        auto valid = load_csv<T>(ra.validate_path);
        r = validate_result(alg.normalized_result(), valid);
      } else {
        log.log("Computing valid results and validating");
        auto valid = alg.compute_valid();
        r = validate_result(alg.normalized_result(), valid);
      }
      print_validation(r, log.progress, !ra.append && loop == 0);
    }
  }
  return 0;
}

}  // namespace

std::vector<std::string> algorithm_names() {
  std::vector<std::string> names;
  for (const auto& a : registry()) names.push_back(a.name);
  std::sort(names.begin(), names.end());
  return names;
}

bool algorithm_exists(const std::string& name) { return find_alg(name) != nullptr; }

int run_algorithm(const run_args& args) {
  const alg_spec* spec = find_alg(args.alg_name);
  if (spec == nullptr) throw std::runtime_error("Invalid algorithm specified \n" + args.alg_name + "\"");
  if (args.data_type == "single") return run_typed<float>(*spec, args);
  if (args.data_type == "double") return run_typed<double>(*spec, args);
  std::cerr << "Unknown data type " << args.data_type << "\n";
  return 1;
}

bool validate_input_size(const std::string& alg_type, uint32_t rows, uint32_t cols, uint32_t left, uint32_t right,
                         bool* known) {
  *known = true;
  const bool sizes = rows > 0 && cols > 0;
  if (alg_type == "one_to_one") return sizes && left == 1 && right == 1;
  if (alg_type == "one_to_many") return sizes && left == 1 && right > 0;
  if (alg_type == "n_to_mn") return sizes && left > 0 && right > 0 && right % left == 0;
  if (alg_type == "n_to_m") return sizes && left > 0 && right > 0;
  *known = false;
  return false;
}

}  // namespace cross
