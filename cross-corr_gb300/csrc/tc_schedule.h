// Work planning of the split tensor-core kernel that needs no device: the
// shift and column parts of an output and the MMA windows of their K-steps,
// the row-shift tile visiting order and the host-built schedule of a banded
// launch (output copied out band by band while the kernel runs).
// Header-only so that the CUDA source and plain C++ test harnesses compile
// the same code.
#pragma once

#include <algorithm>
#include <cstdint>
#include <cmath>
#include <functional>
#include <queue>
#include <utility>
#include <vector>

#ifdef __CUDACC__
#define XC_HD __host__ __device__ __forceinline__
#else
#define XC_HD inline
#endif

namespace xc {

// Shift and column parts of one output: x-parts of 512 shifts, each two
// halves of half_w shifts (tensor-memory columns [0, 256) and [256, 512)),
// and k-parts of 256 right columns; K-steps of 16 (BF16) or 8 (TF32)
// columns, in 128-byte chunks of 64 or 32 columns.
constexpr int kHalfCols = 256;                   // tensor-memory columns per shift half
constexpr int kTQBf16 = 98, kTQTf32 = 194;       // core matrices of the Toeplitz buffer
struct TcParts {
  int half_w, n_xparts, n_kparts, kstep, nkc;
};
inline TcParts tc_parts(int Sx, int Wr, bool tf32) {
  TcParts t;
  t.half_w = Sx > 512 ? 256 : ((Sx + 1) / 2 + 15) / 16 * 16;
  t.n_xparts = (Sx + 511) / 512;
  t.n_kparts = (Wr + 255) / 256;
  t.kstep = tf32 ? 8 : 16;
  const int chunk = tf32 ? 32 : 64;
  t.nkc = ((Wr < 256 ? Wr : 256) + chunk - 1) / chunk;
  return t;
}

// The MMA window of half h and the K-step whose first right column is k0,
// in the x-part starting at shift s0 and the k-part starting at column
// kbase: the shifts sx whose left columns sx + k - (Wr-1) meet the row for
// some column k of the K-step, clipped to the half and rounded out to 16.
// Packed: TMEM column (bits 0-8), N / 16 (9-13), active (14), and the core
// matrix of the Toeplitz buffer the MMA's B operand starts at (16-23): the
// item's staged row is X[i] = Lp[s0 + kbase + i], so B[n][k] = Lp[w0 + n +
// k0 + k] starts at X[w0 - s0 + k0 - kbase].  reset = true: the whole half
// from the part's first column (the first MMA of a window, which also
// starts every accumulator column afresh).
XC_HD uint32_t pack_window(int dcol, int n, bool active, int bq) {
  return (uint32_t)dcol | ((uint32_t)(n / 16) << 9) | ((active ? 1u : 0u) << 14) | ((uint32_t)bq << 16);
}
XC_HD uint32_t window_of(int Sx, int Wl, int Wr, int half_w, int kstep, int s0, int kbase, int h, int k0,
                         bool reset) {
  const int cm = kstep == 16 ? 8 : 4;
  const int H0 = s0 + h * half_w;
  const int H1 = Sx < H0 + half_w ? Sx : H0 + half_w;
  if (reset) return pack_window(h * kHalfCols, half_w, true, (H0 - s0) / cm);
  if (k0 >= Wr || H0 >= H1) return 0;
  const int k_hi = (k0 + kstep < Wr ? k0 + kstep : Wr) - 1;
  const int lo = H0 > Wr - 1 - k_hi ? H0 : Wr - 1 - k_hi;
  const int hi = H1 < Wr - 1 + Wl - k0 ? H1 : Wr - 1 + Wl - k0;
  if (lo >= hi) return 0;
  const int w0 = H0 + (lo - H0) / 16 * 16;
  const int n = (hi - w0 + 15) / 16 * 16;
  return pack_window(h * kHalfCols + (w0 - H0), n, true, (w0 - s0 + k0 - kbase) / cm);
}

// dy-tile visiting order: centre (heaviest overlap) first, then alternating
// outwards, so long tiles start early.
XC_HD int centre_out(int r, int n, int tc) {
  const int below = tc, above = n - tc - 1;
  const int m = below < above ? below : above;
  if (r == 0) return tc;
  if (r <= 2 * m) return (r & 1) ? tc + (r + 1) / 2 : tc - r / 2;
  const int extra = r - 2 * m;
  return above > below ? tc + m + extra : tc - m - extra;
}

constexpr int kMaxBands = 8;  // output row bands signalled as they complete

// Output row bands of a launch: contiguous runs of row-shift tiles with about
// equal numbers of left rows (the work); band b covers output rows
// [row_lo[b], row_hi[b]).
struct BandLayout {
  int n_bands;
  int band_start[kMaxBands + 1];  // band b: tiles [band_start[b], band_start[b+1])
  int band_rank[kMaxBands];       // place of band b in the work order
  int order[kMaxBands];           // the bands in work order
  int row_lo[kMaxBands], row_hi[kMaxBands];
};

// Up to `want` bands (at least one tile each; every tile has left rows).
// Boundaries fall where the running row count passes k / want of the total.
// Bands with the most output rows are worked first, so the copies still to
// run when the kernel ends are the shortest ones (equal work gives the edge
// bands far more rows, since the left rows per tile fall off towards both
// edges).
inline BandLayout plan_bands(int Hl, int Hr, int DY, int Sy, int want) {
  BandLayout L;
  const int n_tiles_y = (Sy + DY - 1) / DY;
  std::vector<long long> rows_of(n_tiles_y);
  long long total = 0;
  for (int ty = 0; ty < n_tiles_y; ++ty) {
    const int dy0 = -(Hr - 1) + ty * DY;
    rows_of[ty] = std::max(0, std::min(Hl, dy0 + DY - 1 + Hr) - std::max(0, dy0));
    total += rows_of[ty];
  }
  want = std::max(1, std::min(std::min(want, kMaxBands), n_tiles_y));
  L.band_start[0] = 0;
  long long acc = 0;
  int nb = 1;
  for (int ty = 0; ty + 1 < n_tiles_y && nb < want; ++ty) {
    acc += rows_of[ty];
    if (acc * want >= total * nb) L.band_start[nb++] = ty + 1;
  }
  L.band_start[nb] = n_tiles_y;
  L.n_bands = nb;
  for (int k = 0; k < nb; ++k) {
    L.order[k] = k;
    L.row_lo[k] = std::min(Sy, L.band_start[k] * DY);
    L.row_hi[k] = std::min(Sy, L.band_start[k + 1] * DY);
  }
  std::stable_sort(L.order, L.order + nb, [&](int a, int b) {
    return L.row_hi[a] - L.row_lo[a] > L.row_hi[b] - L.row_lo[b];
  });
  for (int r = 0; r < nb; ++r) L.band_rank[L.order[r]] = r;
  return L;
}

// What the banded schedule needs to know of a launch.
struct BandPlanIn {
  int Hl, Hr, DY;       // left/right rows, row shifts per tile
  int n_dytiles;        // row-shift tiles
  int per_rank;         // (left matrix, partner group) combinations
  int n_halves;         // halves of the shift columns (items per tile key)
  int chunk_rows;       // left rows per item of the unbanded list
  int n_bands;          // 1..kMaxBands
  int band_start[kMaxBands + 1];  // band b: tiles [band_start[b], band_start[b+1])
  int band_rank[kMaxBands];       // place of each band in the schedule
  int ks[2];            // active K-steps of an item of each half (its cost per left row)
};

// An entry of the schedule: tile key (rank * per_rank + lp) * n_halves + half
// (-1: nothing), first left row counted from the tile's first, left rows.
// Same layout as an int4.
struct BandPiece {
  int key, row0, rows, pad;
};

// Schedule of a banded launch on G CTAs.  Each band's left rows are cut into
// about G * m equal pieces, m = ceil(W / (G * chunk_rows)) for the band's work
// W (left rows over all tile keys); a piece has between half of chunk_rows and
// chunk_rows rows, and every tile key's rows are cut into near-equal pieces.
// The pieces then go, band by band (band_rank order) and longest first, each
// to the CTA with the least work so far (cost: (left rows + 3) x active
// K-steps, the 3 standing for an item's fixed drain), at most ceil(n / G) + 2
// per CTA.  CTA c finds its r-th entry at r * G + c.  Returns the number of
// rounds (entries = rounds * G); `band_items` receives the pieces per band
// and `max_load` / `mean_load` (when not null) the CTAs' modelled work.
// Pieces per tile key are at most 2 ceil(rows / chunk_rows), so n is at most
// twice the unbanded item count and the entries at most that plus 3 G.
inline int plan_band_schedule(const BandPlanIn& in, int G, std::vector<BandPiece>* sched, long long* band_items,
                              long long* max_load = nullptr, double* mean_load = nullptr) {
  struct Entry {
    int rank, rows, cost;
    BandPiece e;
  };
  const int tc = (in.Hr - 1) / in.DY;
  // left rows of each row-shift tile (by visiting rank) and each band's work
  std::vector<int> rows_of(in.n_dytiles), band_of(in.n_dytiles);
  std::vector<double> work(in.n_bands, 0.0);
  for (int rank = 0; rank < in.n_dytiles; ++rank) {
    const int t = centre_out(rank, in.n_dytiles, tc);
    const int dy0 = -(in.Hr - 1) + t * in.DY;
    rows_of[rank] = std::max(0, std::min(in.Hl, dy0 + in.DY - 1 + in.Hr) - std::max(0, dy0));
    int b = 0;
    while (b + 1 < in.n_bands && t >= in.band_start[b + 1]) ++b;
    band_of[rank] = b;
    work[b] += (double)rows_of[rank] * in.per_rank * in.n_halves;
  }
  std::vector<double> target(in.n_bands);
  for (int b = 0; b < in.n_bands; ++b) {
    const double m = std::max(1.0, std::ceil(work[b] / ((double)G * in.chunk_rows)));
    target[b] = std::max(0.5 * in.chunk_rows, work[b] / (G * m));
  }
  std::vector<Entry> es;
  for (int b = 0; b < in.n_bands; ++b) band_items[b] = 0;
  for (int rank = 0; rank < in.n_dytiles; ++rank) {
    const int rows = rows_of[rank], b = band_of[rank];
    if (rows <= 0) continue;
    const int np = std::max((rows + in.chunk_rows - 1) / in.chunk_rows,
                            std::max(1, (int)std::lround(rows / target[b])));
    for (int lp = 0; lp < in.per_rank; ++lp)
      for (int half = 0; half < in.n_halves; ++half) {
        const int key = (rank * in.per_rank + lp) * in.n_halves + half;
        int row0 = 0;
        for (int q = 0; q < np; ++q) {
          const int n = rows / np + (q < rows % np ? 1 : 0);
          es.push_back({in.band_rank[b], n, (n + 3) * in.ks[half], BandPiece{key, row0, n, 0}});
          row0 += n;
          ++band_items[b];
        }
      }
  }
  std::stable_sort(es.begin(), es.end(), [](const Entry& a, const Entry& b) {
    return a.rank != b.rank ? a.rank < b.rank : a.rows > b.rows;
  });
  const long long n = (long long)es.size();
  const int cap = (int)((n + G - 1) / G) + 2;
  using Slot = std::pair<long long, int>;  // (work so far, CTA): the smallest first
  std::priority_queue<Slot, std::vector<Slot>, std::greater<Slot>> heap;
  for (int c = 0; c < G; ++c) heap.push({0, c});
  std::vector<int> count(G, 0);
  std::vector<long long> load(G, 0);
  sched->assign((size_t)G * cap, BandPiece{-1, 0, 0, 0});
  int rounds = 0;
  for (const Entry& e : es) {
    const Slot s = heap.top();  // never empty: G * cap >= n + 2G
    heap.pop();
    (*sched)[(size_t)count[s.second] * G + s.second] = e.e;
    rounds = std::max(rounds, ++count[s.second]);
    load[s.second] = s.first + e.cost;
    if (count[s.second] < cap) heap.push({load[s.second], s.second});
  }
  sched->resize((size_t)rounds * G);
  if (max_load) *max_load = *std::max_element(load.begin(), load.end());
  if (mean_load) {
    double t = 0.0;
    for (long long v : load) t += (double)v;
    *mean_load = t / G;
  }
  return rounds;
}

}  // namespace xc
