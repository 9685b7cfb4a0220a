// data_array.cpp -- CSV matrix files, host-side FFT normalisation, the
// validation statistics and the CPU definition used by cpu_* and `-v`.
#include <algorithm>
#include <atomic>
#include <cerrno>
#include <charconv>
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

// Worker threads for CSV parsing and formatting: the host's cores, at most
// 16, and at most one per 256 rows.
int csv_threads(size_t rows) {
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  return (int)std::max<size_t>(1, std::min<size_t>({(size_t)std::min(hw, 16u), rows / 256 + 1}));
}

// Runs fn(lo, hi) over [0, n) split into `threads` contiguous ranges.
template <typename F>
void parallel_rows(size_t n, int threads, F fn) {
  if (threads <= 1) {
    fn((size_t)0, n);
    return;
  }
  std::vector<std::thread> pool;
  const size_t per = (n + threads - 1) / threads;
  for (int t = 1; t < threads; ++t) {
    const size_t lo = std::min(n, per * t), hi = std::min(n, lo + per);
    pool.emplace_back([=, &fn] { fn(lo, hi); });
  }
  fn((size_t)0, std::min(n, per));
  for (auto& th : pool) th.join();
}

// One value of a data line: leading and trailing blanks and a leading '+'
// allowed, as strtod accepts them; correctly rounded to T.
template <typename T>
bool parse_token(const char* b, const char* e, T* v) {
  while (b < e && (*b == ' ' || *b == '\t')) ++b;
  while (e > b && (e[-1] == ' ' || e[-1] == '\t' || e[-1] == '\r')) --e;
  if (b < e && *b == '+' && e - b > 1 && b[1] != '-') ++b;
  if (b == e) return false;
  const auto r = std::from_chars(b, e, *v);
  return r.ec == std::errc() && r.ptr == e;
}

}  // namespace

// read_header / read_data (src/matrix.hpp:94-159): the same header rules and
// messages.  The file is read whole; its data lines are found with one memchr
// pass and parsed by several threads (std::from_chars), each over a range of
// lines.  A malformed line reports the same message the reference gives; the
// first such line in file order wins.
template <typename T>
data_array<T> load_csv(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (f == nullptr) throw std::runtime_error("Could not open file " + path);
  std::string buf;
  {
    char chunk[1 << 16];
    size_t n;
    while ((n = std::fread(chunk, 1, sizeof(chunk), f)) > 0) buf.append(chunk, n);
    std::fclose(f);
  }
  const char* base = buf.data();
  const size_t size = buf.size();
  size_t pos = 0;
  auto next_line = [&](size_t* b, size_t* e) {  // getline: false at end of input
    if (pos >= size) return false;
    const void* nl = std::memchr(base + pos, '\n', size - pos);
    *b = pos;
    *e = nl ? (size_t)((const char*)nl - base) : size;
    pos = *e + 1;
    return true;
  };
  size_t hb, he;
  if (!next_line(&hb, &he)) throw std::runtime_error("Could not read file header");
  std::string line(base + hb, he - hb);
  if (!line.empty() && line.back() == '\r') line.pop_back();
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
  const size_t total_rows = (size_t)rows * count;
  std::vector<size_t> lb(total_rows), le(total_rows);
  for (size_t y = 0; y < total_rows; ++y)
    if (!next_line(&lb[y], &le[y]))
      throw std::runtime_error("Failed to read line " + std::to_string(y % rows) + " from csv file");
  // per thread: the first bad line of its range and its message
  const int threads = csv_threads(total_rows);
  std::vector<size_t> bad_row(threads, (size_t)-1);
  std::vector<std::string> bad_msg(threads);
  T* out = a.data.data();
  const size_t per = (total_rows + threads - 1) / std::max(1, threads);
  parallel_rows(total_rows, threads, [&](size_t lo, size_t hi) {
    const int t = (int)(lo / std::max<size_t>(1, per));
    for (size_t y = lo; y < hi; ++y) {
      const char* b = base + lb[y];
      const char* e = base + le[y];
      if (e > b && e[-1] == '\r') --e;
      size_t n_tok = 1;
      for (const char* q = b; q < e; ++q) n_tok += *q == ',';
      std::string msg;
      if (n_tok > cols) {
        msg = "Line " + std::to_string(y % rows) + " is too long, expected " + std::to_string(cols) + "values";
      } else if (n_tok < cols) {
        msg = "Line" + std::to_string(y % rows) + " is too short, expected " + std::to_string(cols) + ", got " +
              std::to_string(n_tok) + " values";
      } else {
        T* dst = out + y * cols;
        const char* q = b;
        for (uint32_t x = 0; x < cols; ++x) {
          const char* c = x + 1 < cols ? static_cast<const char*>(std::memchr(q, ',', (size_t)(e - q))) : e;
          if (!parse_token<T>(q, c, dst + x)) {
            msg = "Invalid value \"" + std::string(q, c) + "\" on data line " + std::to_string(y);
            break;
          }
          q = c + 1;
        }
      }
      if (!msg.empty()) {
        bad_row[t] = y;
        bad_msg[t] = msg;
        return;
      }
    }
  });
  for (int t = 0; t < threads; ++t)
    if (bad_row[t] != (size_t)-1) throw std::runtime_error(bad_msg[t]);
  return a;
}

// write_header / write_data (src/matrix.hpp:161-185), with the row stride
// fixed (the reference strides rows by matrix_size.y, src/matrix.hpp:180) and
// the shortest round-trip representation (std::to_chars) instead of 6 fixed
// decimals.  Ranges of rows are formatted by several threads and written in
// order.
template <typename T>
void store_csv(const std::string& path, const data_array<T>& a) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (f == nullptr) throw std::runtime_error("Could not open output file " + path);
  std::fprintf(f, "# %u,%u,%u\n", a.rows, a.cols, a.count);
  const size_t total_rows = (size_t)a.rows * a.count;
  const int threads = csv_threads(total_rows);
  // blocks of rows: each formatted into its own buffer, written in order
  const size_t block = 4096;
  const size_t n_blocks = (total_rows + block - 1) / block;
  bool ok = true;
  for (size_t g0 = 0; g0 < n_blocks && ok; g0 += (size_t)threads) {
    const size_t g1 = std::min(n_blocks, g0 + (size_t)threads);
    std::vector<std::string> bufs(g1 - g0);
    parallel_rows(g1 - g0, (int)(g1 - g0), [&](size_t lo, size_t hi) {
      char num[64];
      for (size_t g = lo; g < hi; ++g) {
        std::string& out = bufs[g];
        const size_t y0 = (g0 + g) * block, y1 = std::min(total_rows, y0 + block);
        out.reserve((y1 - y0) * a.cols * 12);
        for (size_t y = y0; y < y1; ++y) {
          const T* row = a.data.data() + y * a.cols;
          for (uint32_t x = 0; x < a.cols; ++x) {
            if (x) out.push_back(',');
            const auto r = std::to_chars(num, num + sizeof(num), row[x]);
            out.append(num, (size_t)(r.ptr - num));
          }
          out.push_back('\n');
        }
      }
    });
    for (const auto& b : bufs)
      if (std::fwrite(b.data(), 1, b.size(), f) != b.size()) ok = false;
  }
  if (std::fclose(f) != 0 || !ok) throw std::runtime_error("Failed to write " + path);
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
