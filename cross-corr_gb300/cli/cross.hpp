// cross.hpp -- internal interfaces of the `cross` command-line tool.
//
// The tool keeps the reference CLI's surface (src/main.cpp:465-683): commands
// help/run/list/validate/input, the same options, algorithm names, CSV files,
// measurement CSV and exit codes (1 argument errors, 2 other exceptions,
// 3 failures of a computation step).  All GPU work goes through the C ABI in
// include/xcorr.h.
#pragma once

#include <chrono>
#include <cstdint>
#include <map>
#include <optional>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "xcorr.h"

namespace cross {

// An invalid algorithm argument (exit code 1, src/argument_error.hpp).
struct argument_error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// ---------------------------------------------------------------------------
// Matrix arrays and the CSV format (src/matrix.hpp:94-185, 410-646):
// header "# rows,cols,count", then count row-major matrices stacked vertically.
// ---------------------------------------------------------------------------
template <typename T>
struct data_array {
  uint32_t rows = 0, cols = 0, count = 0;
  std::vector<T> data;

  data_array() = default;
  data_array(uint32_t r, uint32_t c, uint32_t n) : rows(r), cols(c), count(n), data((size_t)r * c * n) {}
  size_t area() const { return (size_t)rows * cols; }
  size_t size() const { return data.size(); }
  T* matrix(uint32_t i) { return data.data() + area() * i; }
  const T* matrix(uint32_t i) const { return data.data() + area() * i; }
  xc_size2 size2() const { return xc_size2{cols, rows}; }
};

template <typename T>
data_array<T> load_csv(const std::string& path);
template <typename T>
void store_csv(const std::string& path, const data_array<T>& a);

// normalize_fft_results (src/fft_helpers.hpp:193-261) on the host, for the
// `validate -n` command and for validating raw FFT output.
template <typename T>
data_array<T> normalize_fft_host(const data_array<T>& raw);

// validate_result (src/validate.hpp:134-188).
struct validation_results {
  bool empty = true;
  double max = 0, mean = 0, stddev = 0, at_result = 0, at_valid = 0;
};
template <typename A, typename B>
validation_results validate_result(const data_array<A>& result, const data_array<B>& valid);
void print_validation(const validation_results& r, bool human, bool header);

// CPU definition of the correlation used by the cpu_* algorithms and by `-v`
// without a file (the reference's cpu_cross_corr_*, src/validate.hpp:216-298).
// ACC is the accumulator type; threads split the (output, row) work items.
template <typename T, typename ACC>
data_array<ACC> cpu_correlate(xc_mode mode, const data_array<T>& left, const data_array<T>& right, int threads);

// ---------------------------------------------------------------------------
// JSON algorithm arguments (--args_path): a flat object of numbers, strings
// and booleans, read with defaults like nlohmann::json::value().
// ---------------------------------------------------------------------------
struct json_args {
  std::map<std::string, std::string> values;  // raw scalar text (strings unquoted)
  static json_args parse_file(const std::string& path);
  long long get_int(const std::string& key, long long def) const;
  std::string get_str(const std::string& key, const std::string& def) const;
  bool get_bool(const std::string& key, bool def) const;
};

// ---------------------------------------------------------------------------
// Run options and the algorithm registry.
// ---------------------------------------------------------------------------
enum class benchmark_type { None, Compute, CommonSteps, Algorithm };

struct run_args {
  benchmark_type bench = benchmark_type::None;
  std::string data_type = "single";
  std::string alg_name;
  std::optional<std::string> args_path;
  std::string ref_path, target_path;
  std::optional<std::string> out_path;
  std::string measurements_path = "measurements.csv";
  bool validate = false;
  std::string validate_path;  // empty: compute valid results on the CPU
  size_t outer_loops = 1;
  bool normalize = false;
  bool append = false;
  bool progress = true;
  std::chrono::nanoseconds min_time{1000000000};
};

std::vector<std::string> algorithm_names();
bool algorithm_exists(const std::string& name);
int run_algorithm(const run_args& args);  // returns the process exit code

// Input size predicates of the four modes (src/one_to_one.hpp:20-22, ...).
bool validate_input_size(const std::string& alg_type, uint32_t rows, uint32_t cols, uint32_t left, uint32_t right,
                         bool* known);

}  // namespace cross
