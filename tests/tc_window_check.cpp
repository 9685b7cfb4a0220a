// Checks the MMA windows of the split tensor-core kernel on the CPU
// (tc_schedule.h: tc_parts, window_of).  Reads one case per line:
//   Wl Wr tf32
// and prints, per case, "ok <issued MACs> <algorithmic MACs>" (per left row
// and tensor-memory lane, the reset MMAs left out) or "FAIL <what>".
// Checked: every window lies inside its half's tensor-memory columns and its
// operand inside the Toeplitz buffer; the windows of a K-step cover every
// shift whose overlap with the K-step's columns is non-empty, in exactly one
// half of exactly one x-part, and no window starts outside its half.
#include <cstdio>
#include <string>
#include <vector>

#include "tc_schedule.h"

using namespace xc;

struct Win {
  int dcol, n, bq;
  bool active;
};

static Win unpack(uint32_t e) {
  return Win{(int)(e & 511u), (int)((e >> 9) & 31u) * 16, (int)(e >> 16), ((e >> 14) & 1u) != 0};
}

static std::string check(int Wl, int Wr, bool tf32, long long* issued, long long* algo) {
  const int Sx = Wl + Wr - 1;
  const TcParts t = tc_parts(Sx, Wr, tf32);
  const int cm = tf32 ? 4 : 8, kq = tf32 ? kTQTf32 : kTQBf16, step_q = tf32 ? 2 : 1;
  const int chunk_cols = tf32 ? 32 : 64;
  *issued = 0;
  *algo = (long long)Wl * Wr;
  for (int xp = 0; xp < t.n_xparts; ++xp)
    for (int kp = 0; kp < t.n_kparts; ++kp) {
      const int s0 = 512 * xp, kbase = 256 * kp;
      const int nkc = std::min(t.nkc, (Wr - kbase + chunk_cols - 1) / chunk_cols);
      for (int h = 0; h < 2; ++h) {
        const int H0 = s0 + h * t.half_w, H1 = std::min(Sx, H0 + t.half_w);
        const Win r = unpack(window_of(Sx, Wl, Wr, t.half_w, t.kstep, s0, kbase, h, kbase, true));
        if (H0 < H1) {
          if (r.dcol != h * kHalfCols || r.n != t.half_w) return "reset window";
          if (r.bq + (r.n / 8 - 1) * step_q + (t.kstep - 1) / cm >= kq) return "reset operand outside the buffer";
        }
        for (int j = 0; j < 4 * nkc; ++j) {
          const int k0 = kbase + j * t.kstep;
          const Win w = unpack(window_of(Sx, Wl, Wr, t.half_w, t.kstep, s0, kbase, h, k0, false));
          // shifts of this half whose overlap with columns [k0, k0 + kstep) is non-empty
          std::vector<char> need(std::max(0, H1 - H0), 0);
          for (int sx = H0; sx < H1; ++sx)
            for (int k = k0; k < std::min(k0 + t.kstep, Wr); ++k) {
              const int x = sx - (Wr - 1) + k;
              if (x >= 0 && x < Wl) need[sx - H0] = 1;
            }
          bool any = false;
          for (char c : need) any = any || c;
          if (!w.active) {
            if (any) return "a needed K-step has no window";
            continue;
          }
          if (w.n < 16 || w.n > 256 || w.n % 16 != 0) return "window width";
          if (w.dcol < h * kHalfCols || w.dcol + w.n > h * kHalfCols + kHalfCols) return "window outside its half";
          if (w.bq + (w.n / 8 - 1) * step_q + (t.kstep - 1) / cm >= kq) return "operand outside the buffer";
          const int w0 = H0 + (w.dcol - h * kHalfCols);
          for (int sx = H0; sx < H1; ++sx)
            if (need[sx - H0] && (sx < w0 || sx >= w0 + w.n)) return "needed shift outside its window";
          *issued += (long long)w.n * t.kstep;
        }
      }
    }
  return "";
}

int main() {
  int Wl, Wr, tf;
  while (std::scanf("%d %d %d", &Wl, &Wr, &tf) == 3) {
    long long issued = 0, algo = 0;
    const std::string err = check(Wl, Wr, tf != 0, &issued, &algo);
    if (err.empty())
      std::printf("ok %lld %lld\n", issued, algo);
    else
      std::printf("FAIL %s\n", err.c_str());
  }
  return 0;
}
