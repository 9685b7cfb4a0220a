// data_array.cpp -- CSV matrix files, host-side FFT normalisation, the
// validation statistics and the CPU definition used by cpu_* and `-v`.
#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <sstream>
#include <thread>

#include "cross.hpp"

namespace cross {

namespace {

// Splits a CSV line on commas (the reference reads with
// boost::escaped_list_separator; data files hold plain numbers).
void split_csv(const std::string& line, std::vector<std::string>& out) {
  out.clear();
  size_t start = 0;
  for (;;) {
    size_t pos = line.find(',', start);
    out.emplace_back(line.substr(start, pos == std::string::npos ? std::string::npos : pos - start));
    if (pos == std::string::npos) break;
    start = pos + 1;
  }
}

template <typename T>
T parse_value(const std::string& s, size_t row) {
  const char* b = s.c_str();
  while (*b == ' ' || *b == '\t') ++b;
  char* end = nullptr;
  errno = 0;
  double v = std::strtod(b, &end);
  if (end == b) throw std::runtime_error("Invalid value \"" + s + "\" on data line " + std::to_string(row));
  while (*end == ' ' || *end == '\t' || *end == '\r') ++end;
  if (*end != '\0') throw std::runtime_error("Invalid value \"" + s + "\" on data line " + std::to_string(row));
  return static_cast<T>(v);
}

}  // namespace

// read_header / read_data (src/matrix.hpp:94-159).
template <typename T>
data_array<T> load_csv(const std::string& path) {
  std::ifstream in(path);
  if (!in) throw std::runtime_error("Could not open file " + path);
  std::string line;
  if (!std::getline(in, line)) throw std::runtime_error("Could not read file header");
  if (line.compare(0, 2, "# ") != 0) throw std::runtime_error("Invalid file header format");
  std::vector<std::string> tok;
  split_csv(line.substr(2), tok);
  if (tok.empty() || tok[0].empty()) throw std::runtime_error("Missing matrix header");
  if (tok.size() < 2) throw std::runtime_error("Missing number of columns");
  if (tok.size() > 3) throw std::runtime_error("Invalid matrix header format, too many tokens");
  auto to_u32 = [](const std::string& s) {
    long long v = std::stoll(s);
    if (v < 0 || v > 0xffffffffLL) throw std::runtime_error("Invalid matrix header value " + s);
    return (uint32_t)v;
  };
  const uint32_t rows = to_u32(tok[0]), cols = to_u32(tok[1]);
  const uint32_t count = tok.size() == 3 ? to_u32(tok[2]) : 1;
  data_array<T> a(rows, cols, count);
  size_t total_rows = (size_t)rows * count;
  T* dst = a.data.data();
  for (size_t y = 0; y < total_rows; ++y) {
    if (!std::getline(in, line))
      throw std::runtime_error("Failed to read line " + std::to_string(y % rows) + " from csv file");
    if (!line.empty() && line.back() == '\r') line.pop_back();
    split_csv(line, tok);
    if (tok.size() > cols)
      throw std::runtime_error("Line " + std::to_string(y % rows) + " is too long, expected " + std::to_string(cols) +
                               "values");
    if (tok.size() < cols)
      throw std::runtime_error("Line" + std::to_string(y % rows) + " is too short, expected " + std::to_string(cols) +
                               ", got " + std::to_string(tok.size()) + " values");
    for (uint32_t x = 0; x < cols; ++x) dst[x] = parse_value<T>(tok[x], y);
    dst += cols;
  }
  return a;
}

// write_header / write_data (src/matrix.hpp:161-185), with the row stride
// fixed (the reference strides rows by matrix_size.y, src/matrix.hpp:180) and
// round-trip precision instead of 6 fixed decimals.
template <typename T>
void store_csv(const std::string& path, const data_array<T>& a) {
  FILE* f = std::fopen(path.c_str(), "w");
  if (f == nullptr) throw std::runtime_error("Could not open output file " + path);
  std::fprintf(f, "# %u,%u,%u\n", a.rows, a.cols, a.count);
  const char* fmt = sizeof(T) == 4 ? "%.9g" : "%.17g";
  std::string buf;
  char num[64];
  const size_t total_rows = (size_t)a.rows * a.count;
  for (size_t y = 0; y < total_rows; ++y) {
    buf.clear();
    const T* row = a.data.data() + y * a.cols;
    for (uint32_t x = 0; x < a.cols; ++x) {
      if (x) buf.push_back(',');
      int n = std::snprintf(num, sizeof(num), fmt, (double)row[x]);
      buf.append(num, (size_t)n);
    }
    buf.push_back('\n');
    std::fwrite(buf.data(), 1, buf.size(), f);
  }
  if (std::fclose(f) != 0) throw std::runtime_error("Failed to write " + path);
}

template <typename T>
data_array<T> normalize_fft_host(const data_array<T>& raw) {
  if (raw.rows < 2 || raw.cols < 2) throw std::runtime_error("FFT result too small to normalize");
  data_array<T> norm(raw.rows - 1, raw.cols - 1, raw.count);
  const uint32_t py = raw.rows, px = raw.cols;
  const uint32_t ny = norm.rows, nx = norm.cols;
  const uint32_t cy = ny / 2, cx = nx / 2;  // where shift 0 lands
  const T area = (T)((double)py * px);
  for (uint32_t m = 0; m < raw.count; ++m) {
    const T* r = raw.matrix(m);
    T* o = norm.matrix(m);
    for (uint32_t y = 0; y < ny; ++y) {
      uint32_t ry = y >= cy ? y - cy : y + py - cy;
      for (uint32_t x = 0; x < nx; ++x) {
        uint32_t rx = x >= cx ? x - cx : x + px - cx;
        o[(size_t)y * nx + x] = r[(size_t)ry * px + rx] / area;
      }
    }
  }
  return norm;
}

template <typename A, typename B>
validation_results validate_result(const data_array<A>& result, const data_array<B>& valid) {
  if (result.rows != valid.rows || result.cols != valid.cols || result.count != valid.count)
    throw std::runtime_error("Cannot validate matrices of different sizes");
  validation_results r;
  r.empty = false;
  const size_t n = result.size();
  double mx = 0, sum = 0, sumsq = 0;
  size_t arg = 0;
  bool have = false;
  for (size_t i = 0; i < n; ++i) {
    const double a = (double)result.data[i], b = (double)valid.data[i];
    double d = (std::fabs(a) <= 1e-5 && std::fabs(b) <= 1e-5) ? 0.0 : std::fabs(a - b) / std::max(std::fabs(a), std::fabs(b));
    if (!have || d > mx) {
      mx = d;
      arg = i;
      have = true;
    }
    sum += d;
    sumsq += d * d;
  }
  r.max = mx;
  r.mean = n ? sum / n : 0;
  double var = n ? sumsq / n - r.mean * r.mean : 0;
  r.stddev = std::sqrt(std::max(var, 0.0));
  r.at_result = n ? (double)result.data[arg] : std::numeric_limits<double>::quiet_NaN();
  r.at_valid = n ? (double)valid.data[arg] : std::numeric_limits<double>::quiet_NaN();
  return r;
}

// operator<< of validation_results / simple_logger::result_stats
// (src/validate.hpp:58-92, src/simple_logger.hpp:30-41).
void print_validation(const validation_results& r, bool human, bool header) {
  std::ostream& out = std::cout;
  if (human) {
    if (r.empty) {
      out << "No validation\n";
      return;
    }
    out << "Difference from valid values:\n";
    out << "Max: " << r.max << " (" << std::fixed << r.at_result << " instead of " << r.at_valid << ")\n";
    out.unsetf(std::ios_base::fixed);
    out << std::scientific;
    out << "Mean: " << r.mean << "\n";
    out << "Stddev: " << r.stddev << "\n";
    out.unsetf(std::ios_base::scientific);
  } else {
    if (header) out << "Max,Mean,Stddev\n";
    std::ostringstream ss;
    ss << std::scientific << r.max << "," << r.mean << "," << r.stddev;
    out << ss.str() << "\n";
  }
  out.flush();
}

template <typename T, typename ACC>
data_array<ACC> cpu_correlate(xc_mode mode, const data_array<T>& left, const data_array<T>& right, int threads) {
  uint64_t n_out = 0;
  if (xc_output_count(mode, left.count, right.count, &n_out) != XC_OK)
    throw std::runtime_error(std::string("Invalid ref and target data counts: ") + xc_last_error());
  const int Hl = (int)left.rows, Wl = (int)left.cols, Hr = (int)right.rows, Wr = (int)right.cols;
  const int Sy = Hl + Hr - 1, Sx = Wl + Wr - 1;
  data_array<ACC> out((uint32_t)Sy, (uint32_t)Sx, (uint32_t)n_out);
  const long long items = (long long)n_out * Sy;
  std::atomic<long long> next{0};
  auto worker = [&]() {
    for (;;) {
      long long it = next.fetch_add(1);
      if (it >= items) break;
      const long long o = it / Sy;
      const int sy_idx = (int)(it % Sy);
      long long l = 0, r = 0;
      switch (mode) {
        case XC_N_TO_MN: l = o % left.count; r = o; break;
        case XC_N_TO_M: l = o / right.count; r = o % right.count; break;
        case XC_ONE_TO_MANY: l = 0; r = o; break;
        default: l = 0; r = 0; break;
      }
      const T* L = left.matrix((uint32_t)l);
      const T* R = right.matrix((uint32_t)r);
      ACC* dst = out.matrix((uint32_t)o) + (size_t)sy_idx * Sx;
      const int sy = sy_idx - (Hr - 1);
      const int y0 = std::max(sy, 0), y1 = std::min(Hl, Hr + sy);
      for (int sx_idx = 0; sx_idx < Sx; ++sx_idx) {
        const int sx = sx_idx - (Wr - 1);
        const int x0 = std::max(sx, 0), x1 = std::min(Wl, Wr + sx);
        ACC sum = 0;
        for (int y = y0; y < y1; ++y) {
          const T* lrow = L + (size_t)y * Wl;
          const T* rrow = R + (size_t)(y - sy) * Wr - sx;
          for (int x = x0; x < x1; ++x) sum += (ACC)rrow[x] * (ACC)lrow[x];
        }
        dst[sx_idx] = sum;
      }
    }
  };
  threads = std::max(1, threads);
  std::vector<std::thread> pool;
  for (int t = 1; t < threads; ++t) pool.emplace_back(worker);
  worker();
  for (auto& th : pool) th.join();
  return out;
}

template data_array<float> load_csv<float>(const std::string&);
template data_array<double> load_csv<double>(const std::string&);
template void store_csv<float>(const std::string&, const data_array<float>&);
template void store_csv<double>(const std::string&, const data_array<double>&);
template data_array<float> normalize_fft_host<float>(const data_array<float>&);
template data_array<double> normalize_fft_host<double>(const data_array<double>&);
template validation_results validate_result<float, float>(const data_array<float>&, const data_array<float>&);
template validation_results validate_result<float, double>(const data_array<float>&, const data_array<double>&);
template validation_results validate_result<double, double>(const data_array<double>&, const data_array<double>&);
template data_array<float> cpu_correlate<float, float>(xc_mode, const data_array<float>&, const data_array<float>&,
                                                       int);
template data_array<double> cpu_correlate<float, double>(xc_mode, const data_array<float>&, const data_array<float>&,
                                                         int);
template data_array<double> cpu_correlate<double, double>(xc_mode, const data_array<double>&,
                                                          const data_array<double>&, int);

}  // namespace cross
