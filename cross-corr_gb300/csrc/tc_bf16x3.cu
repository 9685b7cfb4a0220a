// tc_bf16x3.cu -- split-BF16 (and split-TF32) tensor-core correlation on
// tcgen05 (sm_103a).  The TF32x3 variant runs the same kernel with FP32
// operands rounded to TF32 (hi = tf32(x), lo = tf32(x - hi)), K = 8 per MMA
// (kind::tf32); it keeps ~21 bits per operand instead of ~16 at half the
// tensor rate.
//
// FP32 inputs, FP32 outputs, three BF16 products per FP32 product:
//   x = x_hi + x_lo, x_hi = bf16(x), x_lo = bf16(x - x_hi)
//   L*R ~= L_hi*R_hi + L_hi*R_lo + L_lo*R_hi      (Henry, Tang & Heinecke 2019)
//
// Formulation (implicit GEMM).  For a left row a and a right row b the
// contribution to output row sy = a - b + Hr - 1 is a 1D correlation, a
// Toeplitz matrix-vector product.  One tcgen05.mma computes
//     D[m][n] += sum_k A[m][k] * B[n][k]        (M=128, N<=256, K=16, BF16)
// with
//   m -> (partner matrix p, row shift dy): A[m][k] = R_p[a - dy][k0 + k]
//        (right rows, staged by TMA with 128-byte swizzle, K-major);
//   n -> column shift sx = w0 + n: B[n][k] = Lp_a[w0 + n + k0 + k],
//        Lp_a[j] = L[a][j - (Wr-1)] (zero outside the row).
// The shifts lie along N, i.e. along tensor-memory columns: the accumulator
// of a shift half is 128 lanes x 256 columns, and each K-step's MMA covers
// only the shifts whose overlap with the K-step's 16 right columns is not
// empty -- a window that slides along the diagonal of the (shift, column)
// plane, placed by the MMA's tensor-memory column offset and N.  A fixed
// 128-shift tile along M would multiply zeros over the triangles where that
// diagonal crosses it (half of every crossed tile: 1.5x the algorithmic work
// at Wl = Wr = 256); the windows waste only their rounding to 16 shifts.
// The first MMA of an accumulation window covers the whole half, which also
// starts every column of the accumulator afresh.
//
// The Toeplitz operand B is read from shared memory through an ordinary
// matrix descriptor.  In the K-major layout without swizzle an 8-row x
// 16-byte core matrix (r, t) sits at start + 16 r + e t (e = element bytes)
// and core matrices are LBO apart along K and SBO apart along N.  Element
// (n, k) lands at 128 (n/8 + k/8) + 16 (n%8) + 2 (k%8) for BF16 with
// LBO = SBO = 128 bytes, and its value Lp[c + n + k] depends only on
// 8 (n/8 + k/8) + n%8 + k%8, so one buffer T[q][r][t] = X[8 q + r + t] of
// 8-element core matrices serves every window and K-step as an offset of
// the start address: builder warps write T once per left row instead of a
// Toeplitz matrix per K-step.  TF32 (4-element core-matrix rows):
// T[q][r][t] = X[4 q + r + t], LBO = 128, SBO = 256.
//
// A work item is every shift of one (partner group, row-shift group, chunk
// of left rows); two issuer threads each issue one shift half's MMAs (one
// thread alone cannot issue the small windows fast enough: measured, about
// 79 cycles per MMA from one thread, at the pipe's rate from two).  The
// kernel is persistent (one CTA per SM) and walks a device-built list of the
// items.  Tensor memory holds the two halves' FP32 accumulators (all 512
// columns).  Every few left rows (the window, chosen per left matrix and
// partner group from the data's statistics) the epilogue warps read the
// accumulators and add them to the output with red.global.add, through a
// small shared-memory transpose so that each reduction instruction covers
// consecutive shifts.
//
// Right tiles come in stages of one plane (hi or lo) of one 128-byte column
// chunk (128 rows x 128 bytes).  Per chunk the MMAs that read the hi plane
// (R_hi L_hi and R_hi L_lo) run first, then those that read the lo plane
// (R_lo L_hi), so each stage is released as soon as its own MMAs finish.
//
// Accuracy.  Tensor-core FP32 accumulation drops low bits on every MMA with a
// consistent sign, so the error of a long chain grows linearly with its
// length and with the magnitude of the partial sums.  Each matrix is
// therefore shifted by its mean before the split (L' = L - mu_L,
// R' = R - mu_R): the tensor cores correlate the centred data, whose partial
// sums are small random walks, and the exact remainder
//   out = corr(L', R') + mu_R * S_L' + mu_L * S_R' + mu_L * mu_R * area
// (S = sum of the centred matrix over the overlap of a shift, four reads of
// a summed-area table of the centred matrix) is written first by a
// correction kernel, which the tensor-core results are then added to.
//
// Warp roles (736 threads, one CTA per SM):
//   warp 0      TMA producer of the right-row tiles
//   warp 1      TMEM allocation; one thread issues the MMAs of shift half 0
//   warp 22     one thread issues the MMAs of shift half 1
//   warps 2-5   builders of the Toeplitz core-matrix buffer (two row buffers)
//   warps 6-21  epilogue: four per TMEM lane quadrant, all draining each half
// Each half's accumulator is drained on its own schedule, the two offset by
// half a window: while the epilogue drains one half, the other half's issuer
// keeps the tensor pipe busy (as far as the shared right-tile stages allow).
// A stage's MMAs are one straight block under guard predicates, and the next
// stage's barrier is looked at before the current stage's MMAs are issued.
// All waits are bounded: an expired wait records a flag, the CTA winds down,
// waits (bounded) for its own copies and MMAs, frees TMEM and returns.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <queue>
#include <string>
#include <utility>
#include <vector>

#include "xc_common.cuh"
#include "tc_schedule.h"
#include "xc_internal.h"

namespace xc {

namespace {

constexpr int kLanes = 128;                // A rows per MMA: P partners x DY row shifts
constexpr int kStageBytes = kLanes * 128;  // one plane of one 128-byte column chunk
constexpr int kBuilderWarps = 4;
constexpr int kEpiWarps = 16;              // four per TMEM lane quadrant, all draining each half
// warp 0 producer, warps 1 and 22 MMA issuers (one per shift half), 2-5
// builders, 6-21 epilogue
constexpr int kThreads = 32 * (3 + kBuilderWarps + kEpiWarps);
constexpr int kIssuer1Warp = 2 + kBuilderWarps + kEpiWarps;
constexpr int kXLen = 792;                 // staged row elements: every shift plus a right row, padded
constexpr int kBarBytes = 256;             // 20 mbarriers at most, the abort flag, the TMEM address slot
constexpr int kMaxChunkRows = 1024;        // left rows per work item at most
constexpr int kMaxKSteps = 32;             // K-steps of a 256-column right row (16 BF16 or 32 TF32)

// Per operand type: right-tile stages and the Toeplitz buffer (hi or lo part
// of one left row): core matrices of 8 BF16 or 4 FP32 per 16-byte row,
// covering X[0, 776) (every shift of both halves plus a right row).
// An epilogue warp transposes 32 lane rows x kTransW shifts at a time
// through shared memory (rows padded by one float): 32 for BF16, so that one
// reduction instruction covers one output row's 32 shifts (a 128-byte line);
// 16 for TF32, whose larger Toeplitz buffer leaves less room.
template <bool TF>
struct TcCfg {
  static constexpr int kStages = TF ? 4 : 5;
  static constexpr int kCm = TF ? 4 : 8;            // elements per 16-byte core-matrix row
  static constexpr int kQ = TF ? kTQTf32 : kTQBf16;  // core matrices in T
  static constexpr int kTBytes = kQ * 128;          // one plane of T
  static constexpr int kTransW = TF ? 16 : 32;
  static constexpr int kTransBytes = kEpiWarps * 32 * (kTransW + 1) * 4;
  static constexpr int kOffBytes = kEpiWarps * 32 * 8;
  static constexpr int kTabBytes = 2 * (kMaxKSteps + 1) * 4 + 8;  // the issuers' K-step windows
  static constexpr int kSmem = 1024 + kStages * kStageBytes + 4 * kTBytes + 4 * kXLen * 4 + kTransBytes +
                               kOffBytes + kTabBytes + kBarBytes;
  static_assert(kCm * (kQ - 1) + 7 + kCm - 1 < kXLen, "T reads inside the staged row");
};

struct TcParams {
  const float* left;
  const float* mu_left;  // mean of every left matrix (the shift of the split)
  float* out;
  int Hl, Wl, Hr, Wr, Sy, Sx;
  PairMap pm;
  int P, DY;        // partners x row shifts per A tile, P*DY = 128
  int mats_mode;    // 1: one TMA box per row shift spans P partners; 0: one box per partner spans DY rows
  int n_pgroups;    // ceil(K / P)
  int n_dytiles;    // ceil(Sy / DY)
  // A work item covers one x-part (shifts [512 xp, 512 xp + 512), in two
  // halves) and one k-part (right columns [256 kp, 256 kp + 256)) of its
  // rows; parts of the same outputs add into them like row chunks do.
  int n_parts;      // work items per tile key: n_xparts * n_kparts
  int n_kparts;
  int half_w;       // shifts per half (a multiple of 16, at most 256): half h of x-part xp
                    // covers [512 xp + h half_w, 512 xp + (h+1) half_w)
  int nkc;          // 128-byte column chunks of a whole k-part (64 BF16 or 32 TF32 columns each)
  int kstep;        // columns per K-step: 16 (BF16) or 8 (TF32)
  const int* flush_tab;  // drain TMEM every this many left rows, per (left matrix, partner group)
  int chunk_rows;   // left rows per work item (a longer row range is split over items)
  const int* items;  // non-empty work items, most left rows first (tc_item encoding)
  // Output row bands: band b holds the items of row-shift tiles
  // [band_start[b], band_start[b+1]); the work list takes the bands one after
  // another in band_rank order, and with band_done set the
  // epilogue counts each band's finished items there (a host copy can wait
  // on the count and take the band's rows while the kernel runs on).
  int n_bands;
  int band_start[kMaxBands + 1];
  int band_rank[kMaxBands];  // place of each band in the work list (a permutation of 0..n_bands-1)
  int* band_done;
  // Host-built schedule (banded launches), or null: CTA c takes entry
  // r * gridDim.x + c in round r, *n_live entries in all.  An entry is
  // {tile key, first left row (from the tile's first), left rows, 0}, the
  // tile key rank * per_rank + lp as in tc_item; key -1: nothing.
  const int4* sched;
  const int* n_live; // entries of `items` (written on the device)
  int n_chunks;     // chunks per (dy tile): ceil(max rows / chunk_rows)
  DeviceFlags* flags;
};

// ---------------------------------------------------------------------------
// tcgen05 / descriptor helpers
// ---------------------------------------------------------------------------
// Shared-memory matrix descriptors are assembled from two 32-bit words:
// low word = start>>4 [0,14) | LBO>>4 [16,30); high word = SBO>>4 [0,14) |
// version 1 at bit 14 | layout type at bits [29,32) (2 = 128-byte swizzle).
// Instruction descriptor, kind::f16: D=F32 (bits 4-5 = 1), A=B=BF16 (bits 7-9,
// 10-12 = 1), both K-major, N>>3 at bit 17, M>>4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Instruction descriptor, kind::tf32: D=F32, A=B=TF32 (format 2), both
// K-major, N>>3 at bit 17, M>>4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_tf32_f32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D[tmem] (+)= A[smem] * B[smem]^T, both operands through descriptors, issued
// only when `exec` is non-zero (a guard predicate instead of a branch keeps a
// stage's MMAs one straight block of code).  No memory clobber: the MMA reads
// shared memory asynchronously, and volatile keeps it in order with the
// barrier waits and commits around it.
template <bool TF>
__device__ __forceinline__ void mma_ss_if(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate, uint32_t exec) {
  if constexpr (TF)
    asm volatile(
        "{\n\t.reg .pred p, e;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "setp.ne.b32 e, %5, 0;\n\t"
        "@e tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate), "r"(exec));
  else
    asm volatile(
        "{\n\t.reg .pred p, e;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "setp.ne.b32 e, %5, 0;\n\t"
        "@e tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate), "r"(exec));
}

// Round to TF32 (10 explicit mantissa bits), nearest with ties away.
__device__ __forceinline__ float tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ uint64_t make_desc(uint32_t lo, uint32_t hi) {
  return ((uint64_t)hi << 32) | (uint64_t)lo;
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive columns of this warp's 32 lanes: one register each.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// red.global.add under a predicate (no branch: a drain's adds stay one
// straight block the compiler can schedule; the address of a false one is
// not used).  No memory clobber: nothing in this thread reads the output, so
// the shared-memory loads that feed the adds may be scheduled ahead of
// earlier adds; the drain's closing fence and barrier arrival order the adds
// before the accumulator is released and before a band count moves.
__device__ __forceinline__ void red_add_if(float* addr, float v, uint32_t pred) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %2, 0;\n\t"
      "@p red.global.add.f32 [%0], %1;\n\t}" ::"l"(addr),
      "f"(v), "r"(pred));
}

// Non-blocking look at a phase: the MMA issuers ask for the next stage
// early and use the answer after the current stage's MMAs, so the barrier
// round trip overlaps them.
__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.test_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait that also gives up as soon as another role aborted.
__device__ __forceinline__ bool wait_or_abort(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                                              DeviceFlags* flags, unsigned where) {
  for (uint32_t i = 0; i < (1u << 22); ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort_flag) return false;
  }
  *abort_flag = 1;
  record_timeout(flags, where);
  return false;
}

// The same for roles that wait long and should not take issue slots from
// the MMA issuer: each poll sleeps up to 20 us (woken early when the phase
// completes); at most 2^17 polls.
__device__ __forceinline__ bool wait_or_abort_sleep(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                                                    DeviceFlags* flags, unsigned where) {
  for (uint32_t i = 0; i < (1u << 17); ++i) {
    if (mbar_try_wait_sleep(bar, parity, 20000u)) return true;
    if (*abort_flag) return false;
  }
  *abort_flag = 1;
  record_timeout(flags, where);
  return false;
}

// OR-reduction over the threads of named barrier `id` (also a barrier).
__device__ __forceinline__ bool bar_red_or(bool v, int id, int nthreads) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 q, %1, 0;\n\t"
      "bar.red.or.pred p, %2, %3, q;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(id), "r"(nthreads)
      : "memory");
  return r != 0;
}

// The MMA window of half h and the K-step whose first right column is k0
// (window_of in tc_schedule.h) for this launch's geometry.
__host__ __device__ __forceinline__ uint32_t kstep_window(const TcParams& p, int s0, int kbase, int h, int k0,
                                                          bool reset) {
  return window_of(p.Sx, p.Wl, p.Wr, p.half_w, p.kstep, s0, kbase, h, k0, reset);
}

// One work item: every shift of one (left matrix, partner group, row-shift
// group, chunk of left rows).
struct TcItem {
  int l, p0, dy0, a_lo, n_rows, rdim2;
  int s0, kbase, nkc;  // x-part's first shift, k-part's first right column, its 128-byte chunks
  int band;  // output row band of the item's row-shift tile
};

// The item of tile key (rank, lp, part) covering the tile's left rows
// [row0, row0 + n) (clipped to the tile); false when that is empty.
__host__ __device__ __forceinline__ bool tc_piece(const TcParams& p, int part, int lp, int rank, int row0, int n,
                                                  TcItem* w) {
  const int xp = part / p.n_kparts, kp = part % p.n_kparts;
  w->s0 = 512 * xp;
  w->kbase = 256 * kp;
  const int chunk_cols = 4 * p.kstep;
  w->nkc = min(p.nkc, (p.Wr - w->kbase + chunk_cols - 1) / chunk_cols);
  w->l = lp / p.n_pgroups;
  w->p0 = (lp % p.n_pgroups) * p.P;
  const int t = centre_out(rank, p.n_dytiles, (p.Hr - 1) / p.DY);
  w->dy0 = -(p.Hr - 1) + t * p.DY;
  const int tile_lo = max(0, w->dy0);
  const int tile_hi = min(p.Hl, w->dy0 + p.DY - 1 + p.Hr);
  w->a_lo = tile_lo + row0;
  const int a_hi = min(tile_hi, w->a_lo + n);
  w->n_rows = a_hi - w->a_lo;
  w->rdim2 = p.pm.r_l != 0 ? w->l : 0;
  int b = 0;
  while (b + 1 < p.n_bands && t >= p.band_start[b + 1]) ++b;
  w->band = b;
  return w->n_rows > 0;
}

// idx = ((chunk * n_dytiles + rank) * per_rank + lp) * n_parts + part; false
// when the item has no left rows.
__host__ __device__ __forceinline__ bool tc_item(const TcParams& p, long long idx, TcItem* w) {
  // 32-bit index arithmetic: launches hold fewer than 2^31 items
  const int i = (int)idx;
  const int per_rank = p.pm.n_left * p.n_pgroups;
  const int part = i % p.n_parts;
  const int key = i / p.n_parts;
  const int lp = key % per_rank;
  const int rank = (key / per_rank) % p.n_dytiles;
  const int chunk = key / (per_rank * p.n_dytiles);
  return tc_piece(p, part, lp, rank, chunk * p.chunk_rows, p.chunk_rows, w);
}

// An entry of the host-built schedule: tile key (rank * per_rank + lp) *
// n_parts + part.
__host__ __device__ __forceinline__ bool tc_entry(const TcParams& p, int4 e, TcItem* w) {
  if (e.x < 0) return false;
  const int per_rank = p.pm.n_left * p.n_pgroups;
  const int part = e.x % p.n_parts, key = e.x / p.n_parts;
  return tc_piece(p, part, key % per_rank, key / per_rank, e.y, e.z, w);
}

// Lists the non-empty work items by output row band (in the order
// band_rank gives), then most left rows first (a counting sort): one block,
// `cnt` a shared array of n_bands * (chunk_rows + 1) ints.  Every CTA of
// tc_kernel reads the same list.
__device__ __forceinline__ void worklist_block(const TcParams& p, int n, int* __restrict__ items,
                                               int* __restrict__ n_live, int* cnt) {
  // key = rank * (chunk_rows + 1) + (chunk_rows - rows): band first, then
  // the longest items
  const int stride = p.chunk_rows + 1, n_keys = p.n_bands * stride;
  for (int r = threadIdx.x; r < n_keys; r += blockDim.x) cnt[r] = 0;
  __syncthreads();
  for (int idx = threadIdx.x; idx < n; idx += blockDim.x) {
    TcItem w;
    if (tc_item(p, idx, &w)) atomicAdd(&cnt[p.band_rank[w.band] * stride + p.chunk_rows - w.n_rows], 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int k = 0; k < n_keys; ++k) {
      const int c = cnt[k];
      cnt[k] = run;  // first position of the items with key k
      run += c;
    }
    *n_live = run;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < n; idx += blockDim.x) {
    TcItem w;
    if (tc_item(p, idx, &w))
      items[atomicAdd(&cnt[p.band_rank[w.band] * stride + p.chunk_rows - w.n_rows], 1)] = idx;
  }
}

// After tc_kernel: every band counter to its largest value, so a host copy
// waiting on one is released even when the kernel gave up early (its
// device flag then reports the error).
__global__ void band_release_kernel(int* band_done, int n) {
  if ((int)threadIdx.x < n) band_done[threadIdx.x] = 0x7fffffff;
}

// The item a CTA takes in `round`: list entries are dealt to the CTAs in
// snake order, round r giving position r*G + c or r*G + G-1-c.
__device__ __forceinline__ bool round_item(const TcParams& p, long long n_live, long long round, TcItem* w) {
  if (p.sched != nullptr) {
    const long long pos = round * gridDim.x + blockIdx.x;
    return pos < n_live && tc_entry(p, p.sched[pos], w);
  }
  const long long G = gridDim.x, c = blockIdx.x;
  const long long pos = round * G + ((round & 1) ? G - 1 - c : c);
  if (pos >= n_live) return false;
  return tc_item(p, (long long)p.items[pos], w);
}

__device__ __forceinline__ long long n_rounds(long long n_live) { return (n_live + gridDim.x - 1) / gridDim.x; }

// Accumulator windows of an item: half 0 drains after every `flush` left
// rows, half 1 first after (flush + 1) / 2 rows and then every `flush`; both
// drain after the item's last row.  True when row ai (0-based) ends a window.
__device__ __forceinline__ bool window_end(int h, int ai, int n_rows, int flush) {
  if (ai == n_rows - 1) return true;
  const int off = h == 0 ? 0 : flush - (flush + 1) / 2;
  return (ai + 1 + off) % flush == 0;
}


// 23 warps: at most 6 on one SM sub-partition, whose 16K registers cap a
// thread at 80.  TF: TF32 operands (K = 8 per MMA) instead of BF16 (K = 16).
template <bool TF>
__global__ void __launch_bounds__(kThreads, 1)
    tc_kernel(const __grid_constant__ CUtensorMap map_hi, const __grid_constant__ CUtensorMap map_lo,
              const __grid_constant__ TcParams p) {
  using C = TcCfg<TF>;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* a_tiles = smem;                                       // kStages x (128 rows x 128 B)
  unsigned char* t_buf = a_tiles + C::kStages * kStageBytes;           // [row buffer][hi, lo] Toeplitz core matrices
  float* xs = reinterpret_cast<float*>(t_buf + 4 * C::kTBytes);        // [row buffer][hi, lo] x kXLen staged row
  float* trans = xs + 4 * kXLen;                                       // [epilogue warp] transpose tile
  long long* offs = reinterpret_cast<long long*>(trans + kEpiWarps * 32 * (C::kTransW + 1));  // [warp][lane row]
  uint32_t* ktab_all = reinterpret_cast<uint32_t*>(offs + kEpiWarps * 32);  // [half][K-step, then reset]
  uint64_t* bars = reinterpret_cast<uint64_t*>(ktab_all + 2 * (kMaxKSteps + 1) + 2);
  uint64_t* a_full = bars;                   // [kStages] right-row tile landed
  uint64_t* a_empty = bars + C::kStages;     // [kStages] tile consumed
  uint64_t* r_full = bars + 2 * C::kStages;  // [2] Toeplitz row buffer written
  uint64_t* r_empty = r_full + 2;            // [2] row buffer consumed
  uint64_t* t_full = r_empty + 2;            // [2] a half's accumulator ready to drain
  uint64_t* t_empty = t_full + 2;            // [2] a half's accumulator drained
  uint64_t* mma_done = t_empty + 2;          // [2] one per issuer
  volatile int* abort_flag = reinterpret_cast<volatile int*>(mma_done + 2);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mma_done + 3);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // Persistent: the work list is sorted by left rows (heaviest first) and
  // dealt out in a snake order (round r gives position r*G + c, or
  // r*G + G-1-c on odd rounds); every role walks the same items and keeps its
  // pipeline counters running across them, so the next item's loads and
  // MMAs overlap the previous item's final adds.
  const long long n_items = *p.n_live;
  const long long n_round = n_rounds(n_items);
  if (threadIdx.x == 0) {
    // consumed barriers take one commit from each issuer
    for (int s = 0; s < C::kStages; ++s) {
      mbar_init(&a_full[s], 1);
      mbar_init(&a_empty[s], 2);
    }
    for (int s = 0; s < 2; ++s) {
      mbar_init(&r_full[s], kBuilderWarps);
      mbar_init(&r_empty[s], 2);
      mbar_init(&t_full[s], 1);
      mbar_init(&t_empty[s], kEpiWarps);
      mbar_init(&mma_done[s], 1);
    }
    *abort_flag = 0;
    fence_mbar_init();
    prefetch_tensormap(&map_hi);
    prefetch_tensormap(&map_lo);
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(512)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    // per (row, column chunk): the hi plane, then the lo plane
    if (lane == 0) {
      int it = 0;
      bool ok = true;
      for (long long round = 0; round < n_round && ok; ++round) {
        TcItem w;
        if (!round_item(p, n_items, round, &w)) continue;
        for (int ai = 0; ai < w.n_rows && ok; ++ai) {
          const int a = w.a_lo + ai;
          for (int kc = 0; kc < w.nkc && ok; ++kc) {
            for (int pl = 0; pl < 2; ++pl, ++it) {
              const int s = it % C::kStages;
              if (!wait_or_abort_sleep(&a_empty[s], ((it / C::kStages) & 1) ^ 1, abort_flag, p.flags, 11)) {
                ok = false;
                break;
              }
              mbar_arrive_expect_tx(&a_full[s], kStageBytes);
              unsigned char* dst = a_tiles + s * kStageBytes;
              const CUtensorMap* map = pl == 0 ? &map_hi : &map_lo;
              const int x = w.kbase + kc * 4 * p.kstep;  // first column of the chunk
              if (p.mats_mode) {
                for (int d = 0; d < p.DY; ++d)
                  tma_load_4d(dst + d * p.P * 128, map, &a_full[s], x, a - (w.dy0 + d), w.rdim2, w.p0);
              } else {
                const int b0 = a - w.dy0 - (p.DY - 1);
                for (int q = 0; q < p.P; ++q)
                  tma_load_4d(dst + q * p.DY * 128, map, &a_full[s], x, b0, w.rdim2, w.p0 + q);
              }
            }
          }
        }
      }
      if (!ok) {
        for (int q = max(0, it - C::kStages); q < it; ++q)
          mbar_wait_bounded(&a_full[q % C::kStages], (q / C::kStages) & 1, 1u << 16);
      }
    }
  } else if (warp == 1 || warp == kIssuer1Warp) {
    // ------------------------------------------------------------ MMA issuers
    // Both walk the same items, rows and stages; issuer h issues the MMAs of
    // shift half h (its own accumulator, tensor-memory columns
    // [256 h, 256 h + 256)) and commits to the shared consumed barriers.
    const int h = warp == 1 ? 0 : 1;
    uint32_t* ktab = ktab_all + h * (kMaxKSteps + 1);
    {
      // A (right-row tile): SBO 1024 B (8 rows x 128 B), 128-byte swizzle.  B
      // (Toeplitz buffer): no swizzle, LBO 128 B along K, SBO 128 B (BF16) or
      // 256 B (TF32) along N.
      constexpr uint32_t kAHi = (1024u >> 4) | (1u << 14) | (2u << 29);
      constexpr uint32_t kBHi = ((TF ? 256u : 128u) >> 4) | (1u << 14);
      const uint32_t idesc0 = TF ? idesc_tf32_f32(128, 0) : idesc_bf16_f32(128, 0);
      const uint32_t a_word = ((smem_u32(a_tiles) >> 4) & 0x3FFFu) | (1u << 16);
      const uint32_t t_word = ((smem_u32(t_buf) >> 4) & 0x3FFFu) | ((128u >> 4) << 16);
      int s = 0, rb = 0;                      // stage, Toeplitz row buffer
      uint32_t s_phase = 0, r_phase = 0, t_phase = 1;
      bool s_ready = false;                   // stage s seen landed ahead of time
      bool ok = true;
      for (long long round = 0; round < n_round && ok; ++round) {
        TcItem w;
        if (!round_item(p, n_items, round, &w)) continue;
        // the item's windows, one K-step per lane (the whole warp), then lane
        // 0 issues
        __syncwarp();
        ktab[lane] = kstep_window(p, w.s0, w.kbase, h, w.kbase + lane * p.kstep, false);
        if (lane == 0) ktab[kMaxKSteps] = kstep_window(p, w.s0, w.kbase, h, w.kbase, true);
        __syncwarp();
        if (lane == 0) {
        const uint32_t kres = ktab[kMaxKSteps];
        const int n_rows = w.n_rows;
        const int flush = p.flush_tab[w.l * p.n_pgroups + w.p0 / p.P];
        int rows_in = 0;
        for (int ai = 0; ai < n_rows && ok; ++ai) {
          if (rows_in == 0) {
            // the epilogue must have drained the previous window
            if (!wait_or_abort(&t_empty[h], t_phase, abort_flag, p.flags, 14)) {
              ok = false;
              break;
            }
            t_phase ^= 1u;
          }
          if (!wait_or_abort(&r_full[rb], r_phase, abort_flag, p.flags, 12)) {
            ok = false;
            break;
          }
          // this row's Toeplitz buffers (hi, lo), 16-byte units
          const uint32_t th = t_word + (uint32_t)rb * (2 * C::kTBytes >> 4);
          const uint32_t tl = th + (C::kTBytes >> 4);
          for (int kc = 0; kc < w.nkc && ok; ++kc) {
            // the window's first MMA covers the whole half and starts the
            // accumulator afresh
            const uint32_t reset = (rows_in == 0 && kc == 0) ? 1u : 0u;
#pragma unroll
            for (int pl = 0; pl < 2; ++pl) {
              if (!s_ready && !wait_or_abort(&a_full[s], s_phase, abort_flag, p.flags, 13)) {
                ok = false;
                break;
              }
              tc_fence_after();
              {
                // ask for the following stage now, use the answer after this one's MMAs
                const int s2 = s + 1 == C::kStages ? 0 : s + 1;
                s_ready = mbar_test_wait(&a_full[s2], s2 == 0 ? s_phase ^ 1u : s_phase);
              }
              const uint32_t aw = a_word + (uint32_t)s * (kStageBytes >> 4);
#pragma unroll
              for (int ks = 0; ks < 4; ++ks) {
                const uint64_t ad = make_desc(aw + ks * 2, kAHi);
                const uint32_t e = ktab[4 * kc + ks];
                const uint32_t on = (e >> 14) & 1u;
                const uint32_t d = tmem_base + (e & 511u);
                const uint32_t id = idesc0 | ((((e >> 9) & 31u) * 2u) << 17);
                const uint32_t bq = (e >> 16) * (128u >> 4);  // core matrices -> 16-byte units
                if (pl == 0) {
                  // R_hi L_hi (the window's first one over the whole half), R_hi L_lo
                  const uint32_t r0 = (ks == 0) ? reset : 0u;
                  const uint32_t e0 = r0 ? kres : e;
                  mma_ss_if<TF>(tmem_base + (e0 & 511u), ad, make_desc(th + (e0 >> 16) * (128u >> 4), kBHi),
                                idesc0 | ((((e0 >> 9) & 31u) * 2u) << 17), r0 ? 0u : 1u, r0 | on);
                  mma_ss_if<TF>(d, ad, make_desc(tl + bq, kBHi), id, 1u, on);
                } else {
                  // R_lo L_hi
                  mma_ss_if<TF>(d, ad, make_desc(th + bq, kBHi), id, 1u, on);
                }
              }
              mma_commit(&a_empty[s]);
              // next stage, without a branch
              s = s + 1 == C::kStages ? 0 : s + 1;
              s_phase ^= s == 0 ? 1u : 0u;
            }
          }
          if (!ok) break;
          mma_commit(&r_empty[rb]);
          rb ^= 1;
          if (rb == 0) r_phase ^= 1u;
          ++rows_in;
          if (window_end(h, ai, n_rows, flush)) {
            mma_commit(&t_full[h]);
            rows_in = 0;
          }
        }
        }
        ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
      }
      // All MMAs issued by this thread must finish before TMEM is released.
      if (lane == 0) {
        mma_commit(&mma_done[h]);
        mbar_wait_bounded(&mma_done[h], 0, 1u << 22);
      }
    }
  } else if (warp < 2 + kBuilderWarps) {
    // ------------------------------------------------------------ Toeplitz builders
    // Per left row: stage the centred, split row X[i] = Lp[s0 + kbase + i]
    // (hi and lo parts; Lp[j] = L[a][j - (Wr-1)], zero outside the row), then write the
    // core-matrix buffer T[q][r][t] = X[kCm q + r + t] of both parts into the
    // free row buffer.
    const int bt = threadIdx.x - 64;  // 0..127
    constexpr int kChunks = 2 * C::kQ * 8;  // 16-byte rows of T, both parts
    int rows_done = 0;
    bool ok = true;
    for (long long round = 0; round < n_round; ++round) {
      TcItem w;
      if (!round_item(p, n_items, round, &w)) continue;
      const float* lrow_base = p.left + (long long)w.l * p.Hl * p.Wl;
      const float mu = __ldg(p.mu_left + w.l);
      const int x_off = w.s0 + w.kbase - (p.Wr - 1);  // left column of X[0]
      int ai = 0;
      for (; ai < w.n_rows; ++ai, ++rows_done) {
        const int rbuf = rows_done & 1;
        float* xh = xs + rbuf * (2 * kXLen);
        float* xl = xh + kXLen;
        const float* src = lrow_base + (long long)(w.a_lo + ai) * p.Wl;
        for (int i = bt; i < kXLen; i += 32 * kBuilderWarps) {
          const int x = x_off + i;
          const float v = (x >= 0 && x < p.Wl) ? __ldg(src + x) - mu : 0.0f;
          float hv, lv;
          if constexpr (TF) {
            hv = tf32_round(v);
            lv = tf32_round(v - hv);
          } else {
            hv = __bfloat162float(__float2bfloat16_rn(v));
            lv = v - hv;
          }
          xh[i] = hv;
          xl[i] = lv;
        }
        // the staged row is complete; the builder threads also leave together here
        if (bar_red_or(!ok, 1, 32 * kBuilderWarps)) {
          ok = false;
          break;
        }
        bool wt = wait_or_abort_sleep(&r_empty[rbuf], ((rows_done >> 1) & 1) ^ 1, abort_flag, p.flags, 15);
        ok = __all_sync(0xffffffffu, wt);
        if (ok) {
          unsigned char* tb = t_buf + rbuf * (2 * C::kTBytes);
          for (int c = bt; c < kChunks; c += 32 * kBuilderWarps) {
            const int part = c / (C::kQ * 8), q = (c >> 3) % C::kQ, r = c & 7;
            const float* x = (part ? xl : xh) + C::kCm * q + r;
            uint4 v;
            if constexpr (TF) {
              v.x = __float_as_uint(x[0]);
              v.y = __float_as_uint(x[1]);
              v.z = __float_as_uint(x[2]);
              v.w = __float_as_uint(x[3]);
            } else {
              auto pk = [](float lo_half, float hi_half) {
                const __nv_bfloat162 b = __floats2bfloat162_rn(lo_half, hi_half);
                return *reinterpret_cast<const uint32_t*>(&b);
              };
              v.x = pk(x[0], x[1]);
              v.y = pk(x[2], x[3]);
              v.z = pk(x[4], x[5]);
              v.w = pk(x[6], x[7]);
            }
            *reinterpret_cast<uint4*>(tb + part * C::kTBytes + q * 128 + r * 16) = v;
          }
          // generic-proxy writes become visible to the tensor core's reads
          fence_proxy_async_shared();
          __syncwarp();
          if (lane == 0) mbar_arrive(&r_full[rbuf]);  // one arrival per warp
        }
      }
      if (ai < w.n_rows) break;  // a failed wait: every builder left at the same barrier
    }
  } else if (warp < 2 + kBuilderWarps + kEpiWarps) {
    // ------------------------------------------------------------ epilogue
    // Every epilogue warp takes part in every drain, in the order the
    // windows end (by left row; half 0 first at the item's last row), and
    // releases the accumulator as soon as its columns are in registers: warp w
    // (index ew = w - 6) reads TMEM lane quadrant q = w % 4 (lane rows 32 q ..:
    // A rows, i.e. (partner, row shift)) and columns [64 cq, 64 cq + 64) of the
    // half, cq = ew / 4.  A 32-column load gives each thread one lane row's
    // 32 shifts; it goes through shared memory so that each reduction
    // instruction covers consecutive shifts of one output row.
    constexpr int TW = C::kTransW;
    const int ew = warp - (2 + kBuilderWarps);
    const int q = warp & 3;
    const int cq = ew >> 2;
    float* tb = trans + ew * (32 * (TW + 1));
    long long* my_off = offs + ew * 32;
    const int lgP = __ffs(p.P) - 1, lgDY = __ffs(p.DY) - 1;
    int drained0 = 0, drained1 = 0;  // drains of each half so far
    bool ok = true;
    for (long long round = 0; round < n_round && ok; ++round) {
      TcItem w;
      if (!round_item(p, n_items, round, &w)) continue;
      {
        // output offset of this thread's lane row m (or -1): partner-major
        // inside a row shift (P >= 8: m = d*P + pp, dy = dy0 + d) or
        // row-shift-major inside a partner (P < 8: m = pp*DY + d,
        // dy = dy0 + DY-1 - d)
        const int m = 32 * q + lane;
        int k, dy;
        if (p.mats_mode) {
          k = w.p0 + (m & (p.P - 1));
          dy = w.dy0 + (m >> lgP);
        } else {
          k = w.p0 + (m >> lgDY);
          dy = w.dy0 + (p.DY - 1) - (m & (p.DY - 1));
        }
        const int sy = dy + p.Hr - 1;
        long long o = -1;
        if (k < p.pm.K && sy >= 0 && sy < p.Sy)
          o = (((long long)w.l * p.pm.o_l + (long long)k * p.pm.o_k) * p.Sy + sy) * p.Sx;
        __syncwarp();  // the previous item's readers are done with the table
        my_off[lane] = o;
        __syncwarp();
      }
      const int flush = p.flush_tab[w.l * p.n_pgroups + w.p0 / p.P];
      for (int ai = 0; ai < w.n_rows && ok; ++ai) {
        for (int h = 0; h < 2; ++h) {
          if (!window_end(h, ai, w.n_rows, flush)) continue;
          bool wt = wait_or_abort_sleep(&t_full[h], (h ? drained1 : drained0) & 1, abort_flag, p.flags, 16);
          if (h) ++drained1;
          else ++drained0;
          wt = __all_sync(0xffffffffu, wt);  // tcgen05.ld below must stay warp-uniform
          if (!wt) {
            ok = false;
            break;
          }
          tc_fence_after();
          const int sx_end = min(p.Sx, w.s0 + (h + 1) * p.half_w);  // this half's shifts end here
          const int sx_base = w.s0 + h * p.half_w + 64 * cq;
          const bool live = sx_base < sx_end;
          const uint32_t col0 = tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(h * kHalfCols + 64 * cq);
          // reductions of lane rows x TW shifts from the transpose tile: shift
          // column cc, lane rows (lane / TW) + (32 / TW) i
          auto reduce_tile = [&](int sx0) {
            const int cc = lane & (TW - 1);
            const int sx = sx0 + cc;
            const uint32_t in_x = sx < sx_end ? 1u : 0u;
#pragma unroll
            for (int i = 0; i < TW; ++i) {
              const int r = (lane / TW) + (32 / TW) * i;
              const long long o = my_off[r];
              red_add_if(p.out + (o < 0 ? 0 : o) + sx, tb[r * (TW + 1) + cc], in_x & (o >= 0 ? 1u : 0u));
            }
          };
          float v[32];
          if constexpr (TW == 32) {
            // The first 32 columns go into the transpose tile and the next 32
            // into registers; then the accumulator is released, and the
            // issuer restarts the half while the adds below are issued.
            if (live) {
              tmem_ld32(col0, v);
              tmem_wait_ld();
#pragma unroll
              for (int c = 0; c < 32; ++c) tb[lane * (TW + 1) + c] = v[c];
              tmem_ld32(col0 + 32u, v);
              tmem_wait_ld();
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&t_empty[h]);  // one arrival per warp
            if (live) {
              reduce_tile(sx_base);
              __syncwarp();
#pragma unroll
              for (int c = 0; c < 32; ++c) tb[lane * (TW + 1) + c] = v[c];
              __syncwarp();
              reduce_tile(sx_base + 32);
              __syncwarp();
            }
          } else {
            // 16-wide tiles: the adds come first, then the release
            if (live) {
              for (int j = 0; j < 64; j += 32) {
                tmem_ld32(col0 + (uint32_t)j, v);
                tmem_wait_ld();
#pragma unroll
                for (int u = 0; u < 2; ++u) {
#pragma unroll
                  for (int c = 0; c < TW; ++c) tb[lane * (TW + 1) + c] = v[TW * u + c];
                  __syncwarp();
                  reduce_tile(sx_base + j + TW * u);
                  __syncwarp();
                }
              }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&t_empty[h]);  // one arrival per warp
          }
        }
      }
      if (p.band_done != nullptr) {
        // this thread's reductions become visible before the band count moves
        __threadfence();
        // the epilogue warps leave together (a failed wait reaches the others here)
        if (bar_red_or(!ok, 2, 32 * kEpiWarps)) {
          ok = false;
          break;
        }
        if (warp == 2 + kBuilderWarps && lane == 0) {
          __threadfence();
          atomicAdd(&p.band_done[w.band], 1);
        }
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(512) : "memory");
  }
}

// Matrices of one side (left or right) for the preparation kernels, which
// take both sides in one launch: blocks [0, a_blocks) work on side a, the
// rest on side b.
struct PrepSide {
  const float* src;  // the matrices, H x W each
  int H, W;
  long long area;    // H x W
  int slices;        // sum_kernel blocks per matrix
  double* sums;      // per-matrix sums and sums of squares
  double* sq;
  float* mu;         // per-matrix means (written by colsum_kernel)
  float* sat;        // (H+1) x (W+1) summed-area table per matrix
  long long sat_rows;  // matrices x (H+1)
  void* hi;          // split planes of the centred matrices (right side only;
  void* lo;          // nullptr: no split), rows of `pitch` elements
  int pitch;
  int split_tf32;    // 1: TF32-rounded FP32 planes, 0: BF16
};

// Matrix sums and sums of squares (means and spreads): blocks over (matrix,
// slice); FP64 partial sums of a slice, block-reduced, added into sums[m]
// and sq[m] (zeroed before the launch).
__device__ __forceinline__ void sum_block(const PrepSide& sd_, int b) {
  const float* __restrict__ src = sd_.src;
  const long long area = sd_.area;
  const int slices = sd_.slices;
  double* __restrict__ sums = sd_.sums;
  double* __restrict__ sq = sd_.sq;
  __shared__ double red[8], red2[8];
  const int m = b / slices, sl = b % slices;
  const long long per = (area + slices - 1) / slices;
  const long long lo = sl * per, hi = min(area, lo + per);
  const float* a = src + (long long)m * area;
  // FP32 within a thread (at most a few dozen terms; FP64 arithmetic is slow
  // on this GPU), FP64 across threads and blocks
  float part = 0.0f, part2 = 0.0f;
  if ((area & 3) == 0 && (per & 3) == 0 && (reinterpret_cast<uintptr_t>(src) & 15) == 0) {
    // float4 loads, eight in flight per thread (a slice is 8 per thread)
    const float4* a4 = reinterpret_cast<const float4*>(a);
    const long long lo4 = lo >> 2, hi4 = hi >> 2;
#pragma unroll 8
    for (long long i = lo4 + threadIdx.x; i < hi4; i += blockDim.x) {
      const float4 x = __ldg(a4 + i);
      part += (x.x + x.y) + (x.z + x.w);
      part2 = fmaf(x.x, x.x, fmaf(x.y, x.y, fmaf(x.z, x.z, fmaf(x.w, x.w, part2))));
    }
  } else {
    for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) {
      const float x = __ldg(a + i);
      part += x;
      part2 = fmaf(x, x, part2);
    }
  }
  double acc = (double)part, acc2 = (double)part2;
  for (int o = 16; o > 0; o >>= 1) {
    acc += __shfl_down_sync(0xffffffffu, acc, o);
    acc2 += __shfl_down_sync(0xffffffffu, acc2, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[threadIdx.x >> 5] = acc;
    red2[threadIdx.x >> 5] = acc2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0, t2 = 0.0;
    for (int j = 0; j < 8; ++j) {
      t += red[j];
      t2 += red2[j];
    }
    atomicAdd(&sums[m], t);
    atomicAdd(&sq[m], t2);
  }
}

__global__ void __launch_bounds__(256) sum_kernel(const PrepSide a, const PrepSide b, unsigned a_blocks) {
  if (blockIdx.x < a_blocks)
    sum_block(a, (int)blockIdx.x);
  else
    sum_block(b, (int)(blockIdx.x - a_blocks));
}

// Accumulation window (left rows between drains) per (left matrix, partner
// group).  The tensor-core accumulation error grows with the window and with
// the partial sums of the centred data relative to the result.  With
// rho = s_L s_R / (|m_L m_R| + s_L s_R) (means m, standard deviations s; at
// most 1, for zero-mean data), the centred partial sums are at most rho of
// the result's scale even when they add coherently, so the window may be
// 1/rho times the zero-mean one.  Largest rho over the group's partners.
// Mean and standard deviation of matrix m (FP64 from the sums; the variance
// is a difference of nearly equal terms for data far from zero).
struct MeanSd {
  float mu, sd;
};
__device__ __forceinline__ MeanSd mean_sd(const double* __restrict__ sums, const double* __restrict__ sq, int m,
                                          int n_left, double left_area, double right_area) {
  const double area = m < n_left ? left_area : right_area;
  const double mean = sums[m] / area;
  return {(float)mean, (float)sqrt(fmax(0.0, sq[m] / area - mean * mean))};
}

// Accumulation windows: one warp per (left matrix, partner group), lanes
// over the partners; from the same sums as the means, so the values agree
// bit for bit with the means the other kernels use.
struct WinArgs {
  const double* sums;
  const double* sq;
  int n_left;
  double left_area, right_area;
  PairMap pm;
  int n_pgroups, P, base_rows, max_rows, fixed;
  int* flush;
};
__device__ __forceinline__ void window_block(const WinArgs& wa, long long b) {
  const long long i = (b * (long long)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= (long long)wa.n_left * wa.n_pgroups) return;  // warp-uniform
  const int l = (int)(i / wa.n_pgroups), pg = (int)(i % wa.n_pgroups);
  const MeanSd vl = mean_sd(wa.sums, wa.sq, l, wa.n_left, wa.left_area, wa.right_area);
  const float ml = vl.mu, sl = vl.sd;
  float rho = 0.0f;
  for (int k = pg * wa.P + lane; k < min(wa.pm.K, pg * wa.P + wa.P); k += 32) {
    const long long r = (long long)l * wa.pm.r_l + (long long)k * wa.pm.r_k + wa.n_left;
    const MeanSd vr = mean_sd(wa.sums, wa.sq, (int)r, wa.n_left, wa.left_area, wa.right_area);
    const float den = fabsf(ml * vr.mu) + sl * vr.sd;
    if (den > 0.0f) rho = fmaxf(rho, sl * vr.sd / den);
  }
  for (int o = 16; o > 0; o >>= 1) rho = fmaxf(rho, __shfl_xor_sync(0xffffffffu, rho, o));
  int rows = wa.max_rows;
  if (wa.fixed > 0)
    rows = wa.fixed;
  else if (rho > 0.0f)
    rows = (int)fminf((float)wa.max_rows, fmaxf((float)wa.base_rows, wa.base_rows / rho));
  if (lane == 0) wa.flush[i] = max(1, rows);
}

// Summed-area tables of the centred matrices fl32(M - mu) (the values the
// split sees): S[m][y][x] = sum_{i<y, j<x} fl32(M[m][i][j] - mu_m),
// (H+1) x (W+1) per matrix, FP32, in two passes.  This one writes the column
// prefix sums C[y][x] = sum_{i<y} into S[y][x+1]; rowscan_kernel then scans
// each row.  Centred, these sums are random walks of modest size, so FP32
// holds them to ~1e-7; the summation is blocked (8-row segments, a carry per
// 64-row chunk), which keeps every FP32 chain short.  One block per (matrix,
// 32-column strip); each of its 8 warps loads 8 consecutive rows of a chunk
// (coalesced, independent loads).
// Split planes of the centred right matrices fl32(R - mu_R), hi/lo with a
// padded pitch: BF16 (T = __nv_bfloat16) or TF32-rounded FP32 (T = float).
// Block b covers 1/bpm of matrix b / bpm (its mean computed once, from the
// sums); a thread writes one 16-byte chunk of each plane (8 BF16 or 4 FP32
// values) and reads the row as float4 when it is 16-byte aligned; zeros in
// the pitch padding.
template <typename T>
__device__ __forceinline__ void split_block(const PrepSide& sd_, int b, int bpm) {
  constexpr int E = 16 / (int)sizeof(T);
  const int H = sd_.H, W = sd_.W, cpr = sd_.pitch / E;  // chunks per row
  const int m = b / bpm, part = b % bpm;
  const float mv = (float)(sd_.sums[m] / (double)sd_.area);
  const long long per = (long long)H * cpr;
  const long long lo = per * part / bpm, hi = per * (part + 1) / bpm;
  const float* src = sd_.src + (long long)m * H * W;
  const bool vec = (W % 4) == 0 && (reinterpret_cast<uintptr_t>(sd_.src) & 15) == 0;
  uint4* ph4 = reinterpret_cast<uint4*>(sd_.hi) + (long long)m * per;
  uint4* pl4 = reinterpret_cast<uint4*>(sd_.lo) + (long long)m * per;
  for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    const int r = (int)(i / cpr);
    const int c0 = (int)(i - (long long)r * cpr) * E;
    const float* row = src + (long long)r * W;
    float v[E];
    if (vec && c0 + E <= W) {
#pragma unroll
      for (int q = 0; q < E; q += 4) {
        const float4 f = __ldg(reinterpret_cast<const float4*>(row + c0 + q));
        v[q] = f.x;
        v[q + 1] = f.y;
        v[q + 2] = f.z;
        v[q + 3] = f.w;
      }
    } else {
#pragma unroll
      for (int q = 0; q < E; ++q) v[q] = c0 + q < W ? __ldg(row + c0 + q) : mv;
    }
    uint4 oh, ol;
    uint32_t* ph = reinterpret_cast<uint32_t*>(&oh);
    uint32_t* pl = reinterpret_cast<uint32_t*>(&ol);
#pragma unroll
    for (int q = 0; q < E; q += (sizeof(T) == 4 ? 1 : 2)) {
      if constexpr (sizeof(T) == 4) {
        const float x = c0 + q < W ? v[q] - mv : 0.0f;
        const float h = tf32_round(x);
        ph[q] = __float_as_uint(h);
        pl[q] = __float_as_uint(tf32_round(x - h));
      } else {
        const float x0 = c0 + q < W ? v[q] - mv : 0.0f, x1 = c0 + q + 1 < W ? v[q + 1] - mv : 0.0f;
        const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
        const __nv_bfloat162 l = __floats2bfloat162_rn(x0 - __low2float(h), x1 - __high2float(h));
        ph[q / 2] = *reinterpret_cast<const uint32_t*>(&h);
        pl[q / 2] = *reinterpret_cast<const uint32_t*>(&l);
      }
    }
    ph4[i] = oh;
    pl4[i] = ol;
  }
}

__device__ __forceinline__ void colsum_block(const PrepSide& sd_, int b) {
  const float* __restrict__ src = sd_.src;
  const int H = sd_.H, W = sd_.W;
  float* __restrict__ C = sd_.sat;
  __shared__ float seg[8][32];
  __shared__ float carry[32];
  const int strips = (W + 31) / 32;
  const int m = b / strips;
  const int lane = threadIdx.x & 31;
  const int x = (b % strips) * 32 + lane;
  const int w = threadIdx.x >> 5;
  const float* a = src + (long long)m * H * W;
  float* c = C + (long long)m * (H + 1) * (W + 1) + 1;  // column x of C is column x + 1 of S
  // the mean as the statistics of every other kernel see it: FP64 sum over
  // the area, rounded once
  const float mv = (float)(sd_.sums[m] / (double)sd_.area);
  if (b % strips == 0 && threadIdx.x == 0) sd_.mu[m] = mv;
  if (w == 0) {
    carry[lane] = 0.0f;
    if (x < W) c[x] = 0.0f;
  }
  for (int y0 = 0; y0 < H; y0 += 64) {
    const int yb = y0 + 8 * w;
    float run[8];
    float acc = 0.0f;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const float v = (x < W && yb + i < H) ? __ldg(a + (long long)(yb + i) * W + x) - mv : 0.0f;
      acc += v;
      run[i] = acc;
    }
    seg[w][lane] = acc;
    __syncthreads();
    float off = carry[lane];
    for (int j = 0; j < w; ++j) off += seg[j][lane];
    if (x < W) {
#pragma unroll
      for (int i = 0; i < 8; ++i)
        if (yb + i < H) c[(long long)(yb + i + 1) * (W + 1) + x] = off + run[i];
    }
    __syncthreads();
    if (w == 0) {
      float t = 0.0f;
      for (int j = 0; j < 8; ++j) t += seg[j][lane];
      carry[lane] += t;
    }
    __syncthreads();
  }
}

// The work list (block 0, unless the launch is banded: its schedule comes
// from the host), then one block per (matrix, 32-column strip) of either
// side (which also writes the means), then the blocks of the right side's
// split planes, then those of the accumulation windows: independent jobs in
// one launch, the split filling the SMs the latency-bound column sums leave
// idle and the work list's serial steps hidden under both.
__global__ void __launch_bounds__(256) colsum_kernel(const PrepSide a, const PrepSide b, unsigned a_blocks,
                                                     unsigned ab_blocks, unsigned split_end, int split_bpm,
                                                     const WinArgs wa, const TcParams p, int list, int n_items,
                                                     int* items, int* n_live) {
  extern __shared__ int wl_cnt[];  // the work list's counts (its block only)
  if (list) {
    if (blockIdx.x == 0) {
      worklist_block(p, n_items, items, n_live, wl_cnt);
      return;
    }
  }
  const unsigned bid = blockIdx.x - (list ? 1u : 0u);
  if (bid < a_blocks)
    colsum_block(a, (int)bid);
  else if (bid < ab_blocks)
    colsum_block(b, (int)(bid - a_blocks));
  else if (bid < split_end) {
    if (b.split_tf32)
      split_block<float>(b, (int)(bid - ab_blocks), split_bpm);
    else
      split_block<__nv_bfloat16>(b, (int)(bid - ab_blocks), split_bpm);
  } else {
    window_block(wa, bid - split_end);
  }
}

// Second pass of the summed-area tables: row y of matrix m (one warp per
// row, 8 rows per block) becomes its inclusive prefix sum over x, S[y][0] = 0.
// The warp scans 32 consecutive columns at a time (coalesced), carrying the
// running total (FP32 chains of at most W/32 + 5 terms).
__global__ void __launch_bounds__(256) rowscan_kernel(const PrepSide a, const PrepSide b, unsigned a_blocks) {
  const bool first = blockIdx.x < a_blocks;
  const PrepSide& sd_ = first ? a : b;
  float* __restrict__ S = sd_.sat;
  const long long n_rows = sd_.sat_rows;
  const int W = sd_.W;
  const int lane = threadIdx.x & 31;
  const long long row = (first ? blockIdx.x : blockIdx.x - a_blocks) * 8LL + (threadIdx.x >> 5);
  if (row >= n_rows) return;  // warp-uniform
  float* q = S + row * (W + 1) + 1;
  if (lane == 0) q[-1] = 0.0f;
  float carry = 0.0f;
  for (int c0 = 0; c0 < W; c0 += 256) {
    // eight 32-column chunks loaded together (the scan is latency-bound)
    float v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = c0 + 32 * u + lane < W ? q[c0 + 32 * u + lane] : 0.0f;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const float y = __shfl_up_sync(0xffffffffu, v[u], o);
        if (lane >= o) v[u] += y;
      }
      v[u] += carry;
      if (c0 + 32 * u + lane < W) q[c0 + 32 * u + lane] = v[u];
      carry = __shfl_sync(0xffffffffu, v[u], 31);
    }
  }
}

// out[o][sy][sx] = mu_R * S_L' + mu_L * S_R' + mu_L * mu_R * area over the
// overlap of shift (sy, sx), where S' are sums of the centred matrices over
// the overlap, read from the summed-area tables.  A block covers one row
// shift sy of up to 8 outputs that share a left matrix (partners k0..k0+7
// of left l).  Along a row the overlap's rows y0..y1 are fixed, so the block
// first stages the table-row differences D_L[x] = S_L[y1][x] - S_L[y0][x]
// once (the same for all its partners) and each warp stages its partner's
// D_R likewise, in shared memory (coalesced table rows, 8 loads in flight
// per lane).  Then each thread takes one shift column sx (the overlap's
// columns x0..x1 depend on sx alone): S'_L = D_L[x1] - D_L[x0] once, and
// per partner S'_R = D_R[x1 - dx] - D_R[x0 - dx].  The kernel writes every
// output once and is bound by instruction issue, hence the reuse of the
// left differences and of the index arithmetic across partners.  FP32 (the
// centred sums are small, and the result's rounding stays near 1e-7 of
// max|out|).
// Staged floats: D_L (Wl + 1) and D_R (Wr + 1), each padded to 4.
inline int corr_stage(int W) { return (W + 1 + 3) / 4 * 4; }
constexpr int kCorrPartners = 8;  // partners per block, one warp each
__global__ void __launch_bounds__(256) correction_kernel(float* __restrict__ out, const float* __restrict__ SL,
                                                         const float* __restrict__ SR,
                                                         const float* __restrict__ mu_l,
                                                         const float* __restrict__ mu_r, int Hl, int Wl, int Hr,
                                                         int Wr, int Sy, int Sx, PairMap pm, int n_kgroups,
                                                         int stage_l, int stage_r) {
  extern __shared__ float stage_all[];  // D_L, then one D_R per warp
  __shared__ float mr[kCorrPartners];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  long long bid = blockIdx.x;
  const int sy = (int)(bid % Sy);
  bid /= Sy;
  const int kg = (int)(bid % n_kgroups);
  const long long l = bid / n_kgroups;
  const int k0 = kg * kCorrPartners;
  const int n_here = min(kCorrPartners, pm.K - k0);
  const int dy = sy - (Hr - 1);
  const int y0 = max(0, dy), y1 = min(Hl, Hr + dy);
  {  // D_L, all threads
    const float* l0 = SL + (l * (Hl + 1) + y0) * (long long)(Wl + 1);
    const float* l1 = SL + (l * (Hl + 1) + y1) * (long long)(Wl + 1);
    for (int t = threadIdx.x; t < Wl + 1; t += blockDim.x) stage_all[t] = __ldg(l1 + t) - __ldg(l0 + t);
  }
  if (wid < n_here) {  // warp-uniform: D_R of partner k0 + wid
    const long long r = l * pm.r_l + (long long)(k0 + wid) * pm.r_k;
    const float* r0 = SR + (r * (Hr + 1) + (y0 - dy)) * (long long)(Wr + 1);
    const float* r1 = SR + (r * (Hr + 1) + (y1 - dy)) * (long long)(Wr + 1);
    float* st = stage_all + stage_l + wid * stage_r;
    for (int t0 = 0; t0 < Wr + 1; t0 += 256) {
      float a[8], b[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int t = t0 + 32 * u + lane;
        a[u] = t < Wr + 1 ? __ldg(r1 + t) : 0.0f;
        b[u] = t < Wr + 1 ? __ldg(r0 + t) : 0.0f;
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int t = t0 + 32 * u + lane;
        if (t < Wr + 1) st[t] = a[u] - b[u];
      }
    }
    if (lane == 0) mr[wid] = mu_r[r];
  }
  __syncthreads();
  const float cl = mu_l[l], cy = (float)(y1 - y0);
  float cr[kCorrPartners], clr[kCorrPartners];
#pragma unroll
  for (int w = 0; w < kCorrPartners; ++w) {
    cr[w] = w < n_here ? mr[w] : 0.0f;
    clr[w] = cl * cr[w];
  }
  const float* dl = stage_all;
  float* o0 = out + ((l * pm.o_l + (long long)k0 * pm.o_k) * Sy + sy) * (long long)Sx;
  const long long ostep = (long long)pm.o_k * Sy * Sx;  // next partner's output row
  for (int sx = threadIdx.x; sx < Sx; sx += blockDim.x) {
    const int dx = sx - (Wr - 1);
    const int x0 = max(0, dx), x1 = min(Wl, Wr + dx);
    const float area = cy * (float)(x1 - x0);
    const float sl = dl[x1] - dl[x0];
    const float* dr0 = stage_all + stage_l + (x0 - dx);  // D_R[j0] of partner 0
    const int span = x1 - x0;                             // j1 - j0
    float* o = o0 + sx;
#pragma unroll
    for (int w = 0; w < kCorrPartners; ++w) {
      if (w < n_here) *o = fmaf(cr[w], sl, fmaf(cl, dr0[span] - dr0[0], clr[w] * area));
      dr0 += stage_r;
      o += ostep;
    }
  }
}

struct TcPlan {
  int P, DY, mats_mode, half_w, nkc, kstep, es, pitch, n_chunks, chunk_rows, n_parts, n_kparts;
  long long n_items;
  long long n_items_ws;  // items at 32-row chunks: the work list and schedule space of either form of launch
  int smem_bytes;
};

int chunk_rows_fixed();
int sm_count();

bool tc_plan(const Geometry& g, const PairMap& pm, bool tf32, TcPlan* t, bool banded = false, int max_rows = 64,
             int min_rows = 4) {
  // sizes accepted: Wl + Wr below 6400 (the correction kernel stages
  // (Wl + 1) + 8 (Wr + 1) floats, well inside 200 KB there)
  if ((size_t)8 * ((g.Wl + g.Wr + 2 + 3) / 4 * 4) * sizeof(float) > 200 * 1024) return false;
  int P = 1;
  while (P < kLanes && P < pm.K) P *= 2;
  t->P = P;
  t->DY = kLanes / P;
  t->mats_mode = P >= 8 ? 1 : 0;
  // x-parts of 512 shifts (two halves), k-parts of 256 right columns
  const TcParts parts = tc_parts(g.Sx, g.Wr, tf32);
  t->half_w = parts.half_w;
  t->n_kparts = parts.n_kparts;
  t->n_parts = parts.n_xparts * parts.n_kparts;
  t->es = tf32 ? 4 : 2;                 // bytes per operand element
  t->kstep = parts.kstep;               // columns per MMA K-step (32 bytes)
  t->nkc = parts.nkc;                   // 128-byte column chunks of a k-part
  t->pitch = (g.Wr + 16 / t->es - 1) / (16 / t->es) * (16 / t->es);
  // left rows per item: at most max_rows (64), fewer when that leaves fewer
  // than two items per SM (small problems), at least min_rows (4; callers
  // that run several problems at once ask for longer items).  Longer items end fewer
  // accumulator windows early (at one_to_many 256x256 x 64: 1.071 ms with
  // 32-row items, 1.039 ms with 64).  A banded launch keeps at most 32: its
  // host plan cuts each band into pieces of half to one item, and 152 CTAs
  // need that many pieces per band.
  const long long span = t->DY - 1 + std::min(g.Hl, g.Hr);
  const long long per_tile_key = (long long)div_up(g.Sy, t->DY) * pm.n_left * div_up(pm.K, t->P) * t->n_parts;
  const long long rows_all = span * per_tile_key;
  const long long fair = rows_all / (2LL * sm_count());
  const int chunk32 = chunk_rows_fixed() > 0 ? chunk_rows_fixed() : (int)std::max(4LL, std::min(32LL, fair));
  const long long lo = std::max(1, std::min(min_rows, max_rows));
  t->chunk_rows = chunk_rows_fixed() > 0 || banded ? chunk32 : (int)std::max(lo, std::min((long long)max_rows, fair));
  t->n_chunks = (int)div_up(span, (long long)t->chunk_rows);
  t->n_items = (long long)t->n_chunks * per_tile_key;
  t->n_items_ws = std::max(t->n_items, div_up(span, (long long)chunk32) * per_tile_key);
  t->smem_bytes = tf32 ? TcCfg<true>::kSmem : TcCfg<false>::kSmem;
  return t->smem_bytes <= 227 * 1024;
}

long long n_right_of(const PairMap& pm) {
  // right matrices addressed by the pair map: r = l*r_l + k*r_k
  return (long long)(pm.n_left - 1) * pm.r_l + (long long)(pm.K - 1) * pm.r_k + 1;
}

int env_int(const char* name, int def) {
  const char* e = std::getenv(name);
  const int v = e ? std::atoi(e) : 0;
  return v > 0 ? v : def;
}

// The zero-mean window: left rows accumulated in tensor memory between two
// drains when the data has zero mean, at most 240 MMAs (12 per 128-byte
// chunk of a right row: 4 K-steps x 3 products) per accumulator.  Measured on
// zero-mean 256x256 data: windows of 5 rows (240 MMAs) 6.0e-6 of max|out|,
// 8 rows 8e-6, 12 rows 1.1e-5, 32 rows 3e-5 (the split alone gives ~6e-6).
// The window blocks of colsum_kernel widen it for data whose means dominate.  Every drain stalls
// the MMAs while the epilogue reads the accumulators.
// XC_TC_FLUSH_ROWS fixes the window, XC_TC_CHUNK_ROWS the item length (studies).
int flush_rows(int nkc) { return std::max(1, std::min(32, 240 / (12 * nkc))); }
int flush_fixed() {
  static const int v = env_int("XC_TC_FLUSH_ROWS", 0);
  return v;
}
int chunk_rows_fixed() {
  static int v = std::min(kMaxChunkRows, env_int("XC_TC_CHUNK_ROWS", 0));
  return v;
}
int sm_count() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      sms <= 0)
    return 152;
  return sms;
}

// Dynamic shared-memory limits raised so far, per kernel and context.  A
// limit is raised only when a launch needs more than the kernel has, so a
// plan that calls tc_prepare for its problems before it captures them into a
// graph makes no cudaFuncSetAttribute call inside the capture.
struct SmemLimit {
  const void* fn;
  unsigned long long ctx;
  int bytes;
};
std::mutex g_limit_mutex;
std::vector<SmemLimit> g_limits;

xc_status raise_smem_limit(const void* fn, int bytes) {
  const unsigned long long ctx = current_context_id();
  std::lock_guard<std::mutex> lock(g_limit_mutex);
  for (SmemLimit& l : g_limits)
    if (l.fn == fn && ctx != 0 && l.ctx == ctx) {
      if (l.bytes < bytes) {
        XC_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        l.bytes = bytes;
      }
      return XC_OK;
    }
  XC_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  if (ctx != 0) g_limits.push_back(SmemLimit{fn, ctx, bytes});
  return XC_OK;
}

// Shared memory of the correction kernel: a left table row and the rows of
// kCorrPartners right tables.
size_t corr_smem_bytes(const Geometry& g) {
  return (size_t)(corr_stage(g.Wl) + kCorrPartners * corr_stage(g.Wr)) * sizeof(float);
}

// Workspace layout (each part 256-byte aligned).
struct TcWs {
  float* mu;        // n_left + n_right means
  double* sums;     // n_left + n_right matrix sums
  double* sq;       // n_left + n_right sums of squares
  int* flush;       // n_left x n_pgroups accumulation windows
  int* sched;       // banded launches: entry count (16 bytes), then the schedule (3 n_items + 3 x SMs int4s)
  float* CL;        // n_left x (Hl+1) x (Wl+1) summed-area tables of the centred matrices
  float* CR;        // n_right x (Hr+1) x (Wr+1)
  void* hi;         // n_right x Hr x pitch, BF16 or TF32-rounded FP32
  void* lo;
  int* items;       // the kernel's work list
  size_t bytes;
};

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

TcWs ws_layout(void* base, const Geometry& g, const PairMap& pm, const TcPlan& t) {
  const long long nr = n_right_of(pm);
  const size_t plane = (size_t)nr * g.Hr * t.pitch;
  size_t off = 0;
  TcWs w;
  char* b = reinterpret_cast<char*>(base);
  auto take = [&](size_t bytes) {
    char* ptr = b ? b + off : nullptr;
    off += align256(bytes);
    return ptr;
  };
  w.mu = reinterpret_cast<float*>(take(sizeof(float) * (pm.n_left + nr)));
  w.sums = reinterpret_cast<double*>(take(2 * sizeof(double) * (pm.n_left + nr)));
  w.sq = w.sums ? w.sums + (pm.n_left + nr) : nullptr;  // zeroed together with the sums
  w.flush = reinterpret_cast<int*>(take(sizeof(int) * (size_t)pm.n_left * div_up(pm.K, t.P)));
  w.CL = reinterpret_cast<float*>(take(sizeof(float) * (size_t)pm.n_left * (g.Hl + 1) * (g.Wl + 1)));
  w.CR = reinterpret_cast<float*>(take(sizeof(float) * (size_t)nr * (g.Hr + 1) * (g.Wr + 1)));
  w.hi = take((size_t)t.es * plane);
  w.lo = take((size_t)t.es * plane);
  w.items = reinterpret_cast<int*>(take(sizeof(int) * ((size_t)t.n_items_ws + 1)));  // list + its length
  w.sched = reinterpret_cast<int*>(take(16 * (1 + 3 * (size_t)t.n_items_ws + 3 * (size_t)sm_count())));
  w.bytes = off + 256;
  return w;
}

// Pinned staging for the host-built schedule, reused once its last copy has
// run.
struct SchedStage {
  int4* host = nullptr;
  size_t cap = 0;
  cudaEvent_t copied = nullptr;
  ~SchedStage() {
    if (host) cudaFreeHost(host);
    if (copied) cudaEventDestroy(copied);
  }
};
thread_local SchedStage t_stage;

// Schedule of a banded launch (plan_band_schedule), copied to `region`: its
// entry count in the first 16 bytes, then the entries.  The device work list
// deals its entries out in a fixed snake order, which keeps the CTAs even only
// while neighbouring entries are about equally long; sorted band by band, each
// band's short last items sit beside the next band's long ones, and on 64
// outputs of 511x511 the busiest CTA then carries 7% (two bands) to 16% (four
// or eight) more than the mean.  With about 8 items per CTA, even assigning
// each item to the CTA with the least work so far leaves 6% (the last band's
// items are all alike, with nothing small left to fill the gaps); hence the
// plan's equal pieces per band.
xc_status upload_band_schedule(const TcParams& prm, int G, int* region, long long* band_items,
                               cudaStream_t stream) {
  BandPlanIn in;
  in.Hl = prm.Hl;
  in.Hr = prm.Hr;
  in.DY = prm.DY;
  in.n_dytiles = prm.n_dytiles;
  in.per_rank = prm.pm.n_left * prm.n_pgroups;
  in.n_halves = prm.n_parts;
  in.chunk_rows = prm.chunk_rows;
  in.n_bands = prm.n_bands;
  for (int b = 0; b <= prm.n_bands; ++b) in.band_start[b] = prm.band_start[b];
  for (int b = 0; b < prm.n_bands; ++b) in.band_rank[b] = prm.band_rank[b];
  // cost of a left row of a part: the MMA windows of both halves (of the
  // first part), in 16-shift units
  int units = 0;
  for (int h = 0; h < 2; ++h)
    for (int j = 0; j < 4 * prm.nkc; ++j) {
      const uint32_t e = kstep_window(prm, 0, 0, h, j * prm.kstep, false);
      if ((e >> 14) & 1u) units += (int)((e >> 9) & 31u);
    }
  in.ks[0] = in.ks[1] = std::max(1, units);
  std::vector<BandPiece> sched;
  plan_band_schedule(in, G, &sched, band_items);
  static_assert(sizeof(BandPiece) == sizeof(int4), "a schedule entry is an int4");
  const size_t n_ent = sched.size();
  if (t_stage.copied == nullptr) XC_CUDA_TRY(cudaEventCreateWithFlags(&t_stage.copied, cudaEventDisableTiming));
  XC_CUDA_TRY(cudaEventSynchronize(t_stage.copied));  // the previous copy has read the staging buffer
  if (t_stage.cap < n_ent + 1) {
    if (t_stage.host) XC_CUDA_TRY(cudaFreeHost(t_stage.host));
    t_stage.host = nullptr;
    t_stage.cap = 0;
    XC_CUDA_TRY(cudaMallocHost(&t_stage.host, (n_ent + 1) * sizeof(int4)));
    t_stage.cap = n_ent + 1;
  }
  t_stage.host[0] = make_int4((int)n_ent, 0, 0, 0);
  std::memcpy(t_stage.host + 1, sched.data(), n_ent * sizeof(int4));
  XC_CUDA_TRY(cudaMemcpyAsync(region, t_stage.host, (n_ent + 1) * sizeof(int4), cudaMemcpyHostToDevice, stream));
  XC_CUDA_TRY(cudaEventRecord(t_stage.copied, stream));
  return XC_OK;
}

}  // namespace

size_t tc_workspace_size(const Geometry& g, const PairMap& pm, bool tf32) {
  TcPlan t;
  if (!tc_plan(g, pm, tf32, &t)) return 0;
  return ws_layout(nullptr, g, pm, t).bytes;
}

xc_status tc_correlate_banded(const float* left, const float* right, float* out, const Geometry& g,
                              const PairMap& pm, void* workspace, size_t ws_bytes, cudaStream_t stream, bool tf32,
                              int want_bands, int* band_done, TcBands* bands, int max_rows, int min_rows) {
  TcPlan t;
  if (!tc_plan(g, pm, tf32, &t, band_done != nullptr, max_rows, min_rows))
    return fail(XC_ERR_UNSUPPORTED,
                "split tensor-core paths need Wl + Wr below 6400");
  const size_t need = ws_layout(nullptr, g, pm, t).bytes;
  if (workspace == nullptr || ws_bytes < need)
    return fail(XC_ERR_WORKSPACE, "split tensor-core path needs " + std::to_string(need) + " bytes of workspace");
  const TcWs w = ws_layout(reinterpret_cast<void*>(((uintptr_t)workspace + 255) & ~uintptr_t(255)), g, pm, t);
  const long long nr = n_right_of(pm);
  const int nl = pm.n_left;

  CUtensorMap mhi, mlo;
  {
    const uint64_t es = (uint64_t)t.es, mat = (uint64_t)t.pitch * g.Hr * es;
    const uint32_t box_x = 128u / (uint32_t)t.es;  // one 128-byte swizzle row
    const uint64_t d2 = pm.r_l != 0 ? (uint64_t)pm.n_left : 1;
    uint64_t dims[4] = {(uint64_t)t.pitch, (uint64_t)g.Hr, d2, (uint64_t)pm.K};
    uint64_t strides[3] = {(uint64_t)t.pitch * es, mat * (uint64_t)(pm.r_l != 0 ? pm.r_l : 1), mat * (uint64_t)pm.r_k};
    uint32_t box[4];
    if (t.mats_mode) {
      box[0] = box_x; box[1] = 1; box[2] = 1; box[3] = (uint32_t)t.P;
    } else {
      box[0] = box_x; box[1] = (uint32_t)t.DY; box[2] = 1; box[3] = 1;
    }
    const CUtensorMapDataType dt = tf32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
    if (!encode_tiled(&mhi, dt, 4, w.hi, dims, strides, box, CU_TENSOR_MAP_SWIZZLE_128B))
      return XC_ERR_INVALID_ARGUMENT;
    if (!encode_tiled(&mlo, dt, 4, w.lo, dims, strides, box, CU_TENSOR_MAP_SWIZZLE_128B))
      return XC_ERR_INVALID_ARGUMENT;
  }

  TcParams prm;
  prm.left = left;
  prm.mu_left = w.mu;
  prm.out = out;
  prm.Hl = g.Hl;
  prm.Wl = g.Wl;
  prm.Hr = g.Hr;
  prm.Wr = g.Wr;
  prm.Sy = g.Sy;
  prm.Sx = g.Sx;
  prm.pm = pm;
  prm.P = t.P;
  prm.DY = t.DY;
  prm.mats_mode = t.mats_mode;
  prm.n_pgroups = div_up(pm.K, t.P);
  prm.n_dytiles = div_up(g.Sy, t.DY);
  prm.n_parts = t.n_parts;
  prm.n_kparts = t.n_kparts;
  prm.half_w = t.half_w;
  prm.nkc = t.nkc;
  prm.kstep = t.kstep;
  prm.flush_tab = w.flush;
  prm.chunk_rows = t.chunk_rows;
  prm.n_chunks = t.n_chunks;
  prm.flags = device_flags();

  const long long n_list = t.n_items;
  if (n_list > 0x7fffffffLL) return fail(XC_ERR_INVALID_ARGUMENT, "problem too large for one launch");
  prm.items = w.items;
  prm.sched = nullptr;
  prm.n_live = w.items + t.n_items;  // written by the work list (unbanded)

  // Output row bands (one unless banded); a banded launch's pieces per band
  // come with its schedule below
  {
    const BandLayout L = plan_bands(g.Hl, g.Hr, t.DY, g.Sy, band_done ? want_bands : 1);
    prm.n_bands = L.n_bands;
    for (int k = 0; k <= L.n_bands; ++k) prm.band_start[k] = L.band_start[k];
    for (int k = 0; k < L.n_bands; ++k) prm.band_rank[k] = L.band_rank[k];
    prm.band_done = band_done;
    if (bands) {
      bands->n = L.n_bands;
      for (int k = 0; k < L.n_bands; ++k) {
        bands->order[k] = L.order[k];
        bands->items[k] = 0;
        bands->row_lo[k] = L.row_lo[k];
        bands->row_hi[k] = L.row_hi[k];
      }
    }
  }

  // 1. per-matrix sums; 2. means, column prefix sums of the centred
  // matrices, the split planes of the centred right matrices and the
  // accumulation windows (one launch); 3. row scans of the tables
  {
    const long long la = (long long)g.Hl * g.Wl, ra = (long long)g.Hr * g.Wr;
    // slices of at most 8192 elements: a thread adds at most 32 terms in FP32
    // (2048-element slices took 19 us instead of 10 at 64 x 256x256: the
    // blocks' FP64 atomics on one matrix's sum serialise)
    const int ls = (int)((la + 8191) / 8192), rs = (int)((ra + 8191) / 8192);
    const PrepSide sl{left,  g.Hl, g.Wl, la, ls, w.sums,      w.sq,      w.mu,      w.CL, (long long)nl * (g.Hl + 1),
                      nullptr, nullptr, 0, 0};
    const PrepSide sr{right, g.Hr, g.Wr, ra, rs, w.sums + nl, w.sq + nl, w.mu + nl, w.CR, (long long)nr * (g.Hr + 1),
                      w.hi, w.lo, t.pitch, tf32 ? 1 : 0};
    XC_CUDA_TRY(cudaMemsetAsync(w.sums, 0, 2 * sizeof(double) * (nl + nr), stream));
    sum_kernel<<<(unsigned)(nl * ls + nr * rs), 256, 0, stream>>>(sl, sr, (unsigned)(nl * ls));
    XC_CUDA_TRY(cudaGetLastError());
    const int npg = div_up(pm.K, t.P);
    const WinArgs wa{w.sums, w.sq, nl, (double)la, (double)ra, pm, npg, t.P, flush_rows(t.nkc), t.chunk_rows,
                     flush_fixed(), w.flush};
    const unsigned lc = (unsigned)(nl * ((g.Wl + 31) / 32));
    const unsigned lrc = lc + (unsigned)(nr * ((g.Wr + 31) / 32));
    // split: blocks of about 2048 chunks of 16 bytes, each within one matrix
    const long long chunks = (long long)g.Hr * (t.pitch / (16 / t.es));
    const int bpm = (int)std::max(1LL, std::min(64LL, chunks / 2048));
    const unsigned split_end = lrc + (unsigned)(nr * bpm);
    const unsigned wb = (unsigned)((32LL * nl * npg + 255) / 256);
    if ((long long)split_end + wb + 1 > 0x7fffffffLL)
      return fail(XC_ERR_INVALID_ARGUMENT, "problem too large for one launch");
    const int list = band_done == nullptr ? 1 : 0;
    const size_t list_smem = list ? sizeof(int) * (size_t)prm.n_bands * (t.chunk_rows + 1) : 0;
    colsum_kernel<<<split_end + wb + (unsigned)list, 256, list_smem, stream>>>(
        sl, sr, lc, lrc, split_end, bpm, wa, prm, list, (int)n_list, w.items, w.items + t.n_items);
    XC_CUDA_TRY(cudaGetLastError());
    // second pass: every row of the left and of the right tables
    const unsigned lb = (unsigned)((sl.sat_rows + 7) / 8);
    rowscan_kernel<<<(unsigned)(lb + (sr.sat_rows + 7) / 8), 256, 0, stream>>>(sl, sr, lb);
    XC_CUDA_TRY(cudaGetLastError());
  }
  // 4. the mean terms initialise the output
  {
    const int stage_l = corr_stage(g.Wl), stage_r = corr_stage(g.Wr);
    const size_t corr_smem = corr_smem_bytes(g);
    if (corr_smem > 200 * 1024) return fail(XC_ERR_UNSUPPORTED, "split tensor-core paths: right matrices too wide");
    if (corr_smem > 48 * 1024) XC_TRY(raise_smem_limit((const void*)correction_kernel, (int)corr_smem));
    const int n_kgroups = div_up(pm.K, kCorrPartners);
    const long long n_blocks = (long long)nl * n_kgroups * g.Sy;
    if (n_blocks > 0x7fffffffLL) return fail(XC_ERR_INVALID_ARGUMENT, "problem too large for one launch");
    correction_kernel<<<(unsigned)n_blocks, 256, corr_smem, stream>>>(out, w.CL, w.CR, w.mu, w.mu + nl, g.Hl, g.Wl,
                                                                      g.Hr, g.Wr, g.Sy, g.Sx, pm, n_kgroups, stage_l,
                                                                      stage_r);
  }
  XC_CUDA_TRY(cudaGetLastError());

  // persistent: one CTA per SM (about 205 KB of shared memory and all 512 TMEM
  // columns each), walking the list in snake order
  auto kern = tf32 ? tc_kernel<true> : tc_kernel<false>;
  XC_TRY(raise_smem_limit((const void*)kern, t.smem_bytes));
  const long long blocks = std::max(1LL, std::min<long long>(n_list, sm_count()));
  if (band_done) {
    // banded: the host deals the items out to the CTAs by least work
    if (blocks > sm_count()) return fail(XC_ERR_WORKSPACE, "banded launch wider than its schedule space");
    long long band_items[kMaxBands];
    XC_TRY(upload_band_schedule(prm, (int)blocks, w.sched, band_items, stream));
    prm.n_live = w.sched;
    prm.sched = reinterpret_cast<const int4*>(w.sched) + 1;
    if (bands)
      for (int k = 0; k < prm.n_bands; ++k) bands->items[k] = band_items[k];
  }
  const int slot = kernel_timer_begin(stream);
  kern<<<(unsigned)blocks, kThreads, (size_t)t.smem_bytes, stream>>>(mhi, mlo, prm);
  kernel_timer_end(slot, stream);
  XC_CUDA_TRY(cudaGetLastError());
  if (band_done) {
    band_release_kernel<<<1, 32, 0, stream>>>(band_done, prm.n_bands);
    XC_CUDA_TRY(cudaGetLastError());
  }
  return XC_OK;
}

xc_status tc_prepare(const Geometry& g, const PairMap& pm, bool tf32) {
  TcPlan t;
  if (!tc_plan(g, pm, tf32, &t)) return fail(XC_ERR_UNSUPPORTED, "split tensor-core paths need Wl + Wr below 6400");
  const size_t corr_smem = corr_smem_bytes(g);
  if (corr_smem > 200 * 1024) return fail(XC_ERR_UNSUPPORTED, "split tensor-core paths: right matrices too wide");
  if (corr_smem > 48 * 1024) XC_TRY(raise_smem_limit((const void*)correction_kernel, (int)corr_smem));
  XC_TRY(raise_smem_limit(tf32 ? (const void*)tc_kernel<true> : (const void*)tc_kernel<false>, t.smem_bytes));
  return XC_OK;
}

xc_status tc_correlate(const float* left, const float* right, float* out, const Geometry& g, const PairMap& pm,
                       void* workspace, size_t ws_bytes, cudaStream_t stream, bool tf32, int max_rows, int min_rows) {
  return tc_correlate_banded(left, right, out, g, pm, workspace, ws_bytes, stream, tf32, 1, nullptr, nullptr,
                             max_rows, min_rows);
}

// ---------------------------------------------------------------------------
// Allocation-free variant of the split-BF16 path.
//
// Some callers cannot call cudaMalloc: hosts that hand a library a fixed
// device-memory budget or their own pool (and forbid raw allocations), and
// latency-critical loops where cudaMalloc/cudaFree may stall or synchronise
// the device.  xc_correlate_tc_noalloc serves them with the scratch of this
// path (sums, means, column prefix sums, BF16 planes) in the file-scope array below,
// of fixed size XC_TC_NOALLOC_SCRATCH_BYTES.  Every GPU that loads the library
// holds that array until the process exits.
// ---------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_tc_noalloc_scratch[XC_TC_NOALLOC_SCRATCH_BYTES];

namespace {
std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[64] = {nullptr};
unsigned long long g_noalloc_ctx[64] = {0};

// Device address of the scratch array for the current device.  In host code
// the array's name only stands in for it, so the address is looked up with
// the device current: once per device and context (again after a context
// reset, which gives the array a new address; on every call when the
// context's identity is unavailable).
xc_status noalloc_scratch(void** ptr) {
  int dev = 0;
  XC_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(XC_ERR_INVALID_ARGUMENT, "device index out of range");
  const unsigned long long ctx = current_context_id();
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (g_noalloc_ptr[dev] == nullptr || ctx == 0 || g_noalloc_ctx[dev] != ctx) {
    void* p = nullptr;
    XC_CUDA_TRY(cudaGetSymbolAddress(&p, g_tc_noalloc_scratch));
    g_noalloc_ptr[dev] = p;
    g_noalloc_ctx[dev] = ctx;
  }
  *ptr = g_noalloc_ptr[dev];
  return XC_OK;
}
}  // namespace

}  // namespace xc

extern "C" xc_status xc_correlate_tc_noalloc(xc_mode mode, const float* d_left, xc_size2 left, uint32_t n_left,
                                             const float* d_right, xc_size2 right, uint32_t n_right, float* d_out,
                                             void* stream) {
  using namespace xc;
  if (d_left == nullptr || d_right == nullptr || d_out == nullptr)
    return fail(XC_ERR_INVALID_ARGUMENT, "NULL device buffer");
  if (left.x == 0 || left.y == 0 || right.x == 0 || right.y == 0)
    return fail(XC_ERR_INVALID_ARGUMENT, "matrix sizes must be positive");
  PairMap pm;
  uint64_t n_out = 0;
  if (!make_pair_map(mode, n_left, n_right, &pm, &n_out))
    return fail(XC_ERR_INVALID_ARGUMENT, "invalid matrix counts for the mode");
  const Geometry g = make_geometry(left, right);
  TcPlan t;
  if (!tc_plan(g, pm, false, &t))
    return fail(XC_ERR_UNSUPPORTED,
                "split-BF16 tensor path needs Wl + Wr below 6400");
  const size_t need = ws_layout(nullptr, g, pm, t).bytes;
  if (need > (size_t)XC_TC_NOALLOC_SCRATCH_BYTES)
    return fail(XC_ERR_WORKSPACE, "xc_correlate_tc_noalloc: this problem needs " + std::to_string(need) +
                                      " bytes of scratch, more than the fixed " +
                                      std::to_string((size_t)XC_TC_NOALLOC_SCRATCH_BYTES) +
                                      " bytes; use xc_correlate with a caller-owned workspace");
  void* scratch = nullptr;
  XC_TRY(noalloc_scratch(&scratch));
  return tc_correlate(d_left, d_right, d_out, g, pm, scratch, (size_t)XC_TC_NOALLOC_SCRATCH_BYTES,
                      reinterpret_cast<cudaStream_t>(stream), false, 64);
}
