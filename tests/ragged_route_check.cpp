// Prints the split-BF16 routes of a ragged plan as the library plans them
// (ragged_route.h: route_min_mac, route_pairs, deal_route).  Reads one case
// per line:
//   route n_streams n_pairs mac_0 ok_0 mac_1 ok_1 ...
// and prints, per case, "<threshold> <streams>" followed by each stream's
// pair indices in issue order, streams separated by "|".
#include <cstdio>
#include <vector>

#include "ragged_route.h"

using namespace xc;

int main() {
  int route = 0, n_streams = 0, n = 0;
  while (std::scanf("%d %d %d", &route, &n_streams, &n) == 3) {
    std::vector<double> mac(n);
    std::vector<char> ok(n);
    for (int i = 0; i < n; ++i) {
      int o = 0;
      if (std::scanf("%lf %d", &mac[i], &o) != 2) return 1;
      ok[i] = (char)(o != 0);
    }
    const std::vector<size_t> pairs = route_pairs(mac, ok, route);
    const std::vector<std::vector<size_t>> per = deal_route(pairs, mac, n_streams);
    std::printf("%.0f %zu", route_min_mac(route), per.size());
    for (const auto& s : per) {
      std::printf(" |");
      for (size_t i : s) std::printf(" %zu", i);
    }
    std::printf("\n");
  }
  return 0;
}
