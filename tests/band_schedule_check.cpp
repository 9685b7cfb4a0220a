// Checks the banded schedule of the split tensor-core kernel on the CPU
// (tc_schedule.h: plan_bands, plan_band_schedule).  Reads one case per line:
//   Hl Hr DY Sy per_rank n_halves chunk_rows want G ks0 ks1
// and prints, per case, "ok <pieces> <rounds> <max_load> <mean_load>" or
// "FAIL <what>".
#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "tc_schedule.h"

using namespace xc;

static std::string check(int Hl, int Hr, int DY, int Sy, int per_rank, int n_halves, int chunk_rows, int want, int G,
                         int ks0, int ks1, long long* pieces, int* rounds_out, long long* max_load, double* mean) {
  const BandLayout L = plan_bands(Hl, Hr, DY, Sy, want);
  const int n_tiles = (Sy + DY - 1) / DY;
  // the layout: bands partition the tiles and the output rows; order and rank are inverse permutations
  if (L.n_bands < 1 || L.n_bands > kMaxBands || L.n_bands > want) return "band count";
  if (L.band_start[0] != 0 || L.band_start[L.n_bands] != n_tiles) return "band ends";
  for (int b = 0; b < L.n_bands; ++b) {
    if (L.band_start[b + 1] <= L.band_start[b]) return "empty band";
    if (L.row_lo[b] != (b == 0 ? 0 : L.row_hi[b - 1])) return "row ranges not contiguous";
    if (L.band_rank[L.order[b]] != b) return "order and rank disagree";
  }
  if (L.row_hi[L.n_bands - 1] != Sy) return "row ranges do not end at Sy";
  for (int r = 1; r < L.n_bands; ++r) {
    const int a = L.order[r - 1], c = L.order[r];
    if (L.row_hi[a] - L.row_lo[a] < L.row_hi[c] - L.row_lo[c]) return "bands not widest first";
  }

  BandPlanIn in;
  in.Hl = Hl;
  in.Hr = Hr;
  in.DY = DY;
  in.n_dytiles = n_tiles;
  in.per_rank = per_rank;
  in.n_halves = n_halves;
  in.chunk_rows = chunk_rows;
  in.n_bands = L.n_bands;
  for (int b = 0; b <= L.n_bands; ++b) in.band_start[b] = L.band_start[b];
  for (int b = 0; b < L.n_bands; ++b) in.band_rank[b] = L.band_rank[b];
  in.ks[0] = ks0;
  in.ks[1] = ks1;
  std::vector<BandPiece> sched;
  long long band_items[kMaxBands];
  const int rounds = plan_band_schedule(in, G, &sched, band_items, max_load, mean);
  *rounds_out = rounds;
  if (sched.size() != (size_t)rounds * G) return "entry count";

  // the unbanded item count bounds the pieces (workspace sizing)
  const int span = DY - 1 + std::min(Hl, Hr);
  const long long n_items = (long long)n_halves * ((span + chunk_rows - 1) / chunk_rows) * n_tiles * per_rank;
  const int tc = (Hr - 1) / DY;
  std::vector<int> rows_of(n_tiles), band_of(n_tiles);
  for (int rank = 0; rank < n_tiles; ++rank) {
    const int t = centre_out(rank, n_tiles, tc);
    if (t < 0 || t >= n_tiles) return "visiting order out of range";
    const int dy0 = -(Hr - 1) + t * DY;
    rows_of[rank] = std::max(0, std::min(Hl, dy0 + DY - 1 + Hr) - std::max(0, dy0));
    int b = 0;
    while (b + 1 < L.n_bands && t >= L.band_start[b + 1]) ++b;
    band_of[rank] = b;
  }

  // every tile key's rows are covered once, by pieces of 1..chunk_rows rows
  std::map<int, std::vector<std::pair<int, int>>> by_key;
  long long count[kMaxBands] = {0};
  long long n = 0;
  for (int c = 0; c < G; ++c) {
    bool ended = false;
    int last_rank = -1;
    for (int r = 0; r < rounds; ++r) {
      const BandPiece& e = sched[(size_t)r * G + c];
      if (e.key < 0) {
        ended = true;
        continue;
      }
      if (ended) return "a CTA's entries have a gap";
      if (e.key >= n_tiles * per_rank * n_halves) return "key out of range";
      if (e.rows < 1 || e.rows > chunk_rows) return "piece size";
      const int rank = e.key / n_halves / per_rank;
      const int band = band_of[rank];
      if (L.band_rank[band] < last_rank) return "a CTA's entries leave band order";
      last_rank = L.band_rank[band];
      by_key[e.key].push_back({e.row0, e.rows});
      ++count[band];
      ++n;
    }
  }
  if (n > 2 * n_items) return "more pieces than twice the unbanded items";
  if ((long long)rounds * G > 2 * n_items + 3LL * G) return "schedule larger than its workspace";
  for (int b = 0; b < L.n_bands; ++b)
    if (count[b] != band_items[b]) return "band piece counts";
  for (int rank = 0; rank < n_tiles; ++rank)
    for (int lp = 0; lp < per_rank; ++lp)
      for (int half = 0; half < n_halves; ++half) {
        const int key = (rank * per_rank + lp) * n_halves + half;
        auto it = by_key.find(key);
        if (rows_of[rank] == 0) {
          if (it != by_key.end()) return "piece of an empty tile";
          continue;
        }
        if (it == by_key.end()) return "tile key without pieces";
        auto v = it->second;
        std::sort(v.begin(), v.end());
        int next = 0;
        for (auto& pr : v) {
          if (pr.first != next) return "pieces overlap or leave a gap";
          next += pr.second;
        }
        if (next != rows_of[rank]) return "pieces do not cover the tile's rows";
      }
  *pieces = n;
  return "";
}

int main() {
  int Hl, Hr, DY, Sy, per_rank, n_halves, chunk_rows, want, G, ks0, ks1;
  while (std::scanf("%d %d %d %d %d %d %d %d %d %d %d", &Hl, &Hr, &DY, &Sy, &per_rank, &n_halves, &chunk_rows, &want,
                    &G, &ks0, &ks1) == 11) {
    long long pieces = 0, max_load = 0;
    int rounds = 0;
    double mean = 0.0;
    const std::string err = check(Hl, Hr, DY, Sy, per_rank, n_halves, chunk_rows, want, G, ks0, ks1, &pieces, &rounds,
                                  &max_load, &mean);
    if (err.empty())
      std::printf("ok %lld %d %lld %.3f\n", pieces, rounds, max_load, mean);
    else
      std::printf("FAIL %s\n", err.c_str());
  }
  return 0;
}
