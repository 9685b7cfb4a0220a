/*
 * xcorr_oracle.c -- CPU oracle for the batched 2D cross-correlation path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C, the reference's
 * CPU algorithms (MK4H/cross-corr `cpu_*` family) so that tests, the smoke
 * check and the CPU-baseline leg of the benchmark can check the CUDA library
 * against it.  Nothing in the product library links, loads or calls this code;
 * the product fails loudly when its CUDA extension is missing.
 *
 * Parity pin: checked against every golden vector shipped with the reference
 * (`data/valid_*.csv` with `data/ina_*.csv`, copied to tests/golden/) and
 * against scipy.signal.correlate2d fixtures generated by the reference's own
 * Python implementation (existing/python/crosscorr.py); see tests/golden/.
 *
 * Restated functions (reference file:line):
 *   hadamard_and_sum          src/validate.hpp:94-114   -> xco_shift_sum_*
 *   naive_cpu_cross_corr      src/validate.hpp:117-132  -> xco_corr_*
 *   cpu_cross_corr_one_to_one src/validate.hpp:216-222
 *   cpu_cross_corr_one_to_many src/validate.hpp:231-240
 *   cpu_cross_corr_n_to_mn    src/validate.hpp:249-270  (pairing t*n + r)
 *   cpu_cross_corr_n_to_m     src/validate.hpp:279-290  (index r*M + t)
 *                                                       -> xco_run_mode
 *   validate_result           src/validate.hpp:134-188  -> xco_validate
 *   normalize_fft_results     src/fft_helpers.hpp:193-261 -> xco_normalize_fft
 *   get_interleaved_index     src/matrix.hpp:614-618    -> xco_interleaved_index
 *
 * Generalisation: the reference only accepts equal-size left/right matrices
 * (src/cross_corr.hpp:121-130).  Here the left matrix is Hl x Wl and the
 * right Hr x Wr; the output is (Hl+Hr-1) x (Wl+Wr-1) with
 *     out[sy + Hr-1][sx + Wr-1] = sum_{y,x} L[y+sy][x+sx] * R[y][x]
 * which is scipy's correlate2d(L, R, 'full') and equals the reference's
 * shift order (half = (S-1)/2) when the sizes are equal.
 *
 * Summation order follows hadamard_and_sum: left rows outer, left columns
 * inner, accumulator of type T (float or double) starting from zero.
 */
#include <math.h>
#include <pthread.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define XCO_ONE_TO_ONE 0
#define XCO_ONE_TO_MANY 1
#define XCO_N_TO_MN 2
#define XCO_N_TO_M 3

/* dtype codes: inputs / accumulator / output */
#define XCO_F32 0     /* float in, float accumulate, float out (reference T=float) */
#define XCO_F64 1     /* double in, double accumulate, double out (T=double)      */
#define XCO_F32_ACC64 2 /* float in, double accumulate, double out (FP64 oracle)  */

static inline int imax(int a, int b) { return a > b ? a : b; }
static inline int imin(int a, int b) { return a < b ? a : b; }

/* One output row (fixed sy) of naive_cpu_cross_corr for the three dtypes. */
#define XCO_DEFINE_ROW(NAME, TIN, TACC, TOUT)                                          \
  static void NAME(const TIN *L, int Hl, int Wl, const TIN *R, int Hr, int Wr,       \
                   TOUT *out, int sy_idx) {                                            \
    const int Sx = Wl + Wr - 1;                                                        \
    const int sy = sy_idx - (Hr - 1);                                                  \
    const int y0 = imax(sy, 0), y1 = imin(Hl, Hr + sy);                                \
    for (int sx_idx = 0; sx_idx < Sx; ++sx_idx) {                                      \
      const int sx = sx_idx - (Wr - 1);                                                \
      const int x0 = imax(sx, 0), x1 = imin(Wl, Wr + sx);                              \
      TACC sum = 0;                                                                    \
      for (int y = y0; y < y1; ++y) {                                                  \
        const TIN *lrow = L + (size_t)y * Wl;                                          \
        const TIN *rrow = R + (size_t)(y - sy) * Wr - sx;                              \
        for (int x = x0; x < x1; ++x) {                                                \
          sum += (TACC)rrow[x] * (TACC)lrow[x];                                        \
        }                                                                              \
      }                                                                                \
      out[(size_t)sy_idx * Sx + sx_idx] = (TOUT)sum;                                   \
    }                                                                                  \
  }

XCO_DEFINE_ROW(row_f32, float, float, float)
XCO_DEFINE_ROW(row_f64, double, double, double)
XCO_DEFINE_ROW(row_f32_acc64, float, double, double)

static size_t elem_in(int dtype) { return dtype == XCO_F32 ? sizeof(float) : (dtype == XCO_F64 ? sizeof(double) : sizeof(float)); }
static size_t elem_out(int dtype) { return dtype == XCO_F32 ? sizeof(float) : sizeof(double); }

static void do_row(int dtype, const void *L, int Hl, int Wl, const void *R, int Hr, int Wr, void *out, int sy_idx) {
  switch (dtype) {
    case XCO_F32: row_f32((const float *)L, Hl, Wl, (const float *)R, Hr, Wr, (float *)out, sy_idx); break;
    case XCO_F64: row_f64((const double *)L, Hl, Wl, (const double *)R, Hr, Wr, (double *)out, sy_idx); break;
    default: row_f32_acc64((const float *)L, Hl, Wl, (const float *)R, Hr, Wr, (double *)out, sy_idx); break;
  }
}

/* naive_cpu_cross_corr (src/validate.hpp:117-132) for one pair, single thread. */
void xco_corr(int dtype, const void *L, int Hl, int Wl, const void *R, int Hr, int Wr, void *out) {
  const int Sy = Hl + Hr - 1;
  for (int sy = 0; sy < Sy; ++sy) do_row(dtype, L, Hl, Wl, R, Hr, Wr, out, sy);
}

/* ------------------------------------------------------------------------ */
/* Pair lists for the four modes (src/validate.hpp:216-298).                */
/* ------------------------------------------------------------------------ */

/* Number of outputs for a mode; -1 when the counts are invalid.
 * one_to_one: 1x1 -> 1; one_to_many: 1xM -> M; n_to_mn: n x (m*n) -> m*n;
 * n_to_m: n x m -> n*m. */
long xco_num_outputs(int mode, int n_left, int n_right) {
  if (n_left <= 0 || n_right <= 0) return -1;
  switch (mode) {
    case XCO_ONE_TO_ONE: return (n_left == 1 && n_right == 1) ? 1 : -1;
    case XCO_ONE_TO_MANY: return n_left == 1 ? n_right : -1;
    case XCO_N_TO_MN: return (n_right % n_left == 0) ? n_right : -1;
    case XCO_N_TO_M: return (long)n_left * n_right;
    default: return -1;
  }
}

/* Left/right matrix indices of output `o`.
 * n_to_mn: output t*n + r is (left r, right t*n + r)  (src/validate.hpp:264-268)
 * n_to_m : output r*M + t is (left r, right t)        (src/validate.hpp:284-288) */
void xco_pair_of_output(int mode, int n_left, int n_right, long o, int *l, int *r) {
  switch (mode) {
    case XCO_N_TO_MN: *l = (int)(o % n_left); *r = (int)o; break;
    case XCO_N_TO_M: *l = (int)(o / n_right); *r = (int)(o % n_right); break;
    case XCO_ONE_TO_MANY: *l = 0; *r = (int)o; break;
    default: *l = 0; *r = 0; break;
  }
}

typedef struct {
  int dtype, mode, n_left, n_right, Hl, Wl, Hr, Wr;
  const char *L, *R;
  char *out;
  long n_items; /* outputs * Sy rows */
  long next;
  pthread_mutex_t lock;
} job_t;

static void *worker(void *arg) {
  job_t *j = (job_t *)arg;
  const int Sy = j->Hl + j->Hr - 1, Sx = j->Wl + j->Wr - 1;
  const size_t lsz = (size_t)j->Hl * j->Wl * elem_in(j->dtype);
  const size_t rsz = (size_t)j->Hr * j->Wr * elem_in(j->dtype);
  const size_t osz = (size_t)Sy * Sx * elem_out(j->dtype);
  for (;;) {
    long item;
    pthread_mutex_lock(&j->lock);
    item = j->next;
    j->next += 1;
    pthread_mutex_unlock(&j->lock);
    if (item >= j->n_items) break;
    long o = item / Sy;
    int sy = (int)(item % Sy);
    int l, r;
    xco_pair_of_output(j->mode, j->n_left, j->n_right, o, &l, &r);
    do_row(j->dtype, j->L + l * lsz, j->Hl, j->Wl, j->R + r * rsz, j->Hr, j->Wr, j->out + o * osz, sy);
  }
  return NULL;
}

/* cpu_cross_corr_{one_to_one,one_to_many,n_to_mn,n_to_m} over all outputs.
 * `threads` <= 1 runs on the calling thread (the reference is serial,
 * src/validate.hpp:237,263,284); more threads split the (output, row) items.
 * Returns 0, or -1 on invalid counts. */
int xco_run_mode(int mode, int dtype, const void *L, int n_left, int Hl, int Wl, const void *R, int n_right,
                 int Hr, int Wr, void *out, int threads) {
  long n_out = xco_num_outputs(mode, n_left, n_right);
  if (n_out < 0 || Hl <= 0 || Wl <= 0 || Hr <= 0 || Wr <= 0) return -1;
  job_t j;
  j.dtype = dtype; j.mode = mode; j.n_left = n_left; j.n_right = n_right;
  j.Hl = Hl; j.Wl = Wl; j.Hr = Hr; j.Wr = Wr;
  j.L = (const char *)L; j.R = (const char *)R; j.out = (char *)out;
  j.n_items = n_out * (long)(Hl + Hr - 1);
  j.next = 0;
  pthread_mutex_init(&j.lock, NULL);
  if (threads <= 1) {
    worker(&j);
  } else {
    if (threads > 256) threads = 256;
    pthread_t tid[256];
    int started = 0;
    for (int t = 0; t < threads; ++t) {
      if (pthread_create(&tid[t], NULL, worker, &j) == 0) started++;
      else break;
    }
    if (started == 0) worker(&j);
    for (int t = 0; t < started; ++t) pthread_join(tid[t], NULL);
  }
  pthread_mutex_destroy(&j.lock);
  return 0;
}

/* Ragged pair list: pair p correlates left p (Hl[p] x Wl[p], at left_off[p]
 * elements into L) with right p; output p starts at out_off[p] elements.
 * Used for the ragged n_to_m batches, which have no reference counterpart. */
typedef struct {
  int dtype, n_pairs;
  const int *Hl, *Wl, *Hr, *Wr;
  const long *loff, *roff, *ooff;
  const char *L, *R;
  char *out;
  long next;
  pthread_mutex_t lock;
} rjob_t;

static void *rworker(void *arg) {
  rjob_t *j = (rjob_t *)arg;
  const size_t ei = elem_in(j->dtype), eo = elem_out(j->dtype);
  for (;;) {
    long p;
    pthread_mutex_lock(&j->lock);
    p = j->next++;
    pthread_mutex_unlock(&j->lock);
    if (p >= j->n_pairs) break;
    xco_corr(j->dtype, j->L + j->loff[p] * ei, j->Hl[p], j->Wl[p], j->R + j->roff[p] * ei, j->Hr[p], j->Wr[p],
             j->out + j->ooff[p] * eo);
  }
  return NULL;
}

int xco_run_pairs(int dtype, int n_pairs, const int *Hl, const int *Wl, const int *Hr, const int *Wr,
                  const long *left_off, const long *right_off, const long *out_off, const void *L, const void *R,
                  void *out, int threads) {
  rjob_t j;
  j.dtype = dtype; j.n_pairs = n_pairs; j.Hl = Hl; j.Wl = Wl; j.Hr = Hr; j.Wr = Wr;
  j.loff = left_off; j.roff = right_off; j.ooff = out_off;
  j.L = (const char *)L; j.R = (const char *)R; j.out = (char *)out; j.next = 0;
  pthread_mutex_init(&j.lock, NULL);
  if (threads <= 1) {
    rworker(&j);
  } else {
    if (threads > 256) threads = 256;
    pthread_t tid[256];
    int started = 0;
    for (int t = 0; t < threads; ++t) {
      if (pthread_create(&tid[t], NULL, rworker, &j) == 0) started++;
      else break;
    }
    if (started == 0) rworker(&j);
    for (int t = 0; t < started; ++t) pthread_join(tid[t], NULL);
  }
  pthread_mutex_destroy(&j.lock);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* validate_result (src/validate.hpp:134-188)                               */
/* ------------------------------------------------------------------------ */
/* Element-wise relative difference |a-b| / max(|a|,|b|), forced to 0 when both
 * magnitudes are <= 1e-5; reports max, mean, population standard deviation
 * (boost accumulators' lazy variance) and the pair of values at the first
 * maximum. */
void xco_validate(const double *result, const double *valid, size_t n, double *out_max, double *out_mean,
                  double *out_std, double *at_result, double *at_valid) {
  double mx = 0.0, sum = 0.0, sumsq = 0.0;
  size_t arg = 0;
  int have = 0;
  for (size_t i = 0; i < n; ++i) {
    double a = result[i], b = valid[i], d;
    if (fabs(a) <= 1e-5 && fabs(b) <= 1e-5) d = 0.0;
    else d = fabs(a - b) / fmax(fabs(a), fabs(b));
    if (!have || d > mx) { mx = d; arg = i; have = 1; }
    sum += d;
    sumsq += d * d;
  }
  double mean = n ? sum / (double)n : 0.0;
  double var = n ? sumsq / (double)n - mean * mean : 0.0;
  if (var < 0) var = 0;
  *out_max = mx;
  *out_mean = mean;
  *out_std = sqrt(var);
  *at_result = n ? result[arg] : NAN;
  *at_valid = n ? valid[arg] : NAN;
}

/* ------------------------------------------------------------------------ */
/* normalize_fft_results (src/fft_helpers.hpp:193-261)                      */
/* ------------------------------------------------------------------------ */
/* `res` is one Py x Px circular correlation (unnormalised inverse FFT of
 * FFT(L) * conj(FFT(R))).  The reference swaps quadrants around the empty
 * row/column at Py/2, Px/2 and divides by Py*Px, producing (Py-1) x (Px-1),
 * with the same four quadrant copies as the reference. */
static void copy_quadrant(const double *src, int src_w, double *dst, int dst_w, int sx0, int sy0, int w, int h,
                          int tx0, int ty0, double area) {
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) dst[(size_t)(ty0 + y) * dst_w + tx0 + x] = src[(size_t)(sy0 + y) * src_w + sx0 + x] / area;
}

void xco_normalize_fft(const double *res, int Py, int Px, double *norm) {
  const int ny = Py - 1, nx = Px - 1;
  const int ex = Px / 2, ey = Py / 2;
  const double area = (double)Py * (double)Px;
  copy_quadrant(res, Px, norm, nx, 0, 0, ex, ey, nx / 2, ny / 2, area);
  copy_quadrant(res, Px, norm, nx, ex + 1, 0, Px - ex - 1, ey, 0, ny / 2, area);
  copy_quadrant(res, Px, norm, nx, 0, ey + 1, ex, Py - ey - 1, nx / 2, 0, area);
  copy_quadrant(res, Px, norm, nx, ex + 1, ey + 1, Px - ex - 1, Py - ey - 1, 0, 0, area);
}

/* get_interleaved_index (src/matrix.hpp:614-618). */
long xco_interleaved_index(long idx, long group_size, long num_groups) {
  long group = idx / group_size;
  long local = idx % group_size;
  return local * num_groups + group;
}
