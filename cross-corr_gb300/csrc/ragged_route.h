// ragged_route.h -- host planning of a ragged plan's split-BF16 routes:
// which pairs a route sends to the split tensor-core path, and how those
// calls are dealt out to the side streams.  Header-only, shared by ragged.cu
// and a CPU test harness (tests/ragged_route_check.cpp).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <vector>

namespace xc {

// Routes of an FP32 plan: 0 keeps every pair on the plain kernel; 1-4 send
// the pairs with at least 2^32, 2^30, 2^28, 2^26 multiply-adds (that the
// split path takes) to the split path.
constexpr int kRaggedRoutes = 5;

inline double route_min_mac(int route) { return route <= 0 ? 0.0 : std::ldexp(1.0, 34 - 2 * route); }

inline bool in_route(double mac, bool split_ok, int route) {
  return route > 0 && split_ok && mac >= route_min_mac(route);
}

// The pairs of a route, most multiply-adds first (ties in pair order).
inline std::vector<size_t> route_pairs(const std::vector<double>& mac, const std::vector<char>& split_ok, int route) {
  std::vector<size_t> r;
  for (size_t i = 0; i < mac.size(); ++i)
    if (in_route(mac[i], split_ok[i] != 0, route)) r.push_back(i);
  std::stable_sort(r.begin(), r.end(), [&mac](size_t a, size_t b) { return mac[a] > mac[b]; });
  return r;
}

// Deals a route's pairs (in route_pairs order) to `n_streams` side streams:
// each to the stream with the least work so far, a call costing its
// multiply-adds plus about 2^26 of fixed work (its preparation launches).
// Returns each stream's pairs in issue order.
inline std::vector<std::vector<size_t>> deal_route(const std::vector<size_t>& pairs, const std::vector<double>& mac,
                                                   int n_streams) {
  std::vector<std::vector<size_t>> per(n_streams > 0 ? n_streams : 1);
  std::vector<double> load(per.size(), 0.0);
  for (size_t i : pairs) {
    const size_t k = (size_t)(std::min_element(load.begin(), load.end()) - load.begin());
    per[k].push_back(i);
    load[k] += mac[i] + std::ldexp(1.0, 26);
  }
  return per;
}

}  // namespace xc
