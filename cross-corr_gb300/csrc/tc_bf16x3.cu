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
//     D[m][n] += sum_k A[m][k] * B[n][k]        (M=128, N=128, K=16, BF16)
// with
//   m -> column shift sx = s0 + m of a 128-shift tile:
//        A[m][k] = Lp_a[s0 + m + k0 + k], Lp_a[j] = L[a][j - (Wr-1)] (zero
//        outside the row).  A is a Toeplitz matrix; builder warps write it
//        straight into tensor memory (tcgen05.st), one lane per shift, from
//        a staged copy of the left row.
//   n -> (partner matrix p, row shift dy): B[n][k] = R_p[a - dy][k0 + k]
//        (right rows, staged by TMA with 128-byte swizzle, K-major).
// N = 128 keeps each MMA at the tensor pipe's full rate (narrower MMAs are
// bound by a per-instruction cost of ~44 cycles on GB300, measured), and the
// shift axis lies along M, so K-steps whose 128 shifts see only zeros are
// skipped (a quarter of them at Wl = Wr).
//
// A work item is two shift tiles (256 shifts) of one (partner group,
// row-shift group, chunk of left rows); a second item covers the other two
// when Sx > 256.  The kernel is persistent (one CTA per SM) and walks a
// device-built list of the items.  Tensor memory holds the two FP32
// accumulator tiles (256 columns) and a two-slot ring of split Toeplitz
// operands (256 columns).
// Every `flush_rows` left rows the epilogue warps drain the accumulators into
// FP32 registers; at the end they add them to the output with coalesced
// red.global.add (consecutive lanes are consecutive shifts).
//
// Accuracy.  Tensor-core FP32 accumulation drops low bits on every MMA with a
// consistent sign, so the error of a long chain grows linearly with its
// length and with the magnitude of the partial sums (measured on GB300:
// ~1.2e-6 of max|out| per 48-MMA left row for uniform [0,1) data).  Each
// matrix is therefore shifted by its mean before the split
// (L' = L - mu_L, R' = R - mu_R): the tensor cores correlate the centred data,
// whose partial sums are small random walks, and the exact remainder
//   out = corr(L', R') + mu_R * S_L' + mu_L * S_R' + mu_L * mu_R * area
// (S = sum of the centred matrix over the overlap of a shift, from column
// prefix sums of the centred matrices, scanned along the row per output row)
// is written first by a correction kernel, which the tensor-core results are
// then added to.  The drains bound every accumulator's chain at
// 192 MMAs.
//
// Warp roles (736 threads, one CTA per SM):
//   warp 0      TMA producer of the right-row tiles (hi and lo planes)
//   warp 1      TMEM allocation; one thread issues the MMAs of shift tile 0
//   warp 22     one thread issues the MMAs of shift tile 1
//   warps 2-5   Toeplitz builders (one per TMEM lane quadrant)
//   warps 6-21  epilogue: 4 per lane quadrant, 64 accumulator columns each
// Two issuers: a single thread cannot issue a 128x128x16 MMA every 64
// cycles once it also waits on barriers and walks the loop (measured: ~85
// cycles per MMA from one thread against 64 for the pipe alone); the two
// tiles' accumulators are independent, so each issuer feeds one of them and
// the tensor pipe interleaves their instructions.
// All waits are bounded: an expired wait records a flag, the CTA winds down,
// waits (bounded) for its own copies and MMAs, frees TMEM and returns.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdlib>
#include <mutex>
#include <string>
#include <vector>

#include "xc_common.cuh"
#include "xc_internal.h"

namespace xc {

namespace {

constexpr int kStages = 6;             // right-row tile pipeline depth
constexpr int kTileBytes = 128 * 128;  // 128 rows x 64 bf16 (one plane)
constexpr int kStageBytes = 2 * kTileBytes;
constexpr int kBuilderWarps = 4;       // one per TMEM lane quadrant
constexpr int kEpiWarps = 16;          // four per TMEM lane quadrant
// warp 0 producer, warps 1 and 22 MMA issuers, 2-5 builders, 6-21 epilogue
constexpr int kThreads = 32 * (3 + kBuilderWarps + kEpiWarps);
constexpr int kMaxLp = 512 + 256;      // staged left row pairs: 128 * tiles + 64 * chunks
constexpr uint32_t kRingCol = 256;     // first TMEM column of the Toeplitz ring
constexpr int kBarBytes = 256;         // 20 mbarriers, the abort flag, the TMEM address slot
constexpr int kMaxChunkRows = 1024;    // left rows per work item at most

struct TcParams {
  const float* left;
  const float* mu_left;  // mean of every left matrix (the shift of the split)
  float* out;
  int Hl, Wl, Hr, Wr, Sy, Sx;
  PairMap pm;
  int P, DY;        // partners x row shifts per B tile, P*DY = 128
  int mats_mode;    // 1: one TMA box per row shift spans P partners; 0: one box per partner spans DY rows
  int n_pgroups;    // ceil(K / P)
  int n_dytiles;    // ceil(Sy / DY)
  int n_halves;     // CTAs per work item (two 128-shift tiles each)
  int nkc;          // 128-byte column chunks of a right row (64 BF16 or 32 TF32 columns)
  int kstep;        // columns per K-step: 16 (BF16) or 8 (TF32)
  int lp_len;       // staged left row length
  int flush_rows;   // drain TMEM every this many left rows
  int chunk_rows;   // left rows per work item (a longer row range is split over items)
  const int* items;  // non-empty work items, most left rows first (index encoding of tc_item)
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

// D[tmem] (+)= A[tmem] * B[smem]^T, TF32 operands (K = 8 per instruction).
__device__ __forceinline__ void mma_tf32_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
      "r"(a_tmem), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

// Round to TF32 (10 explicit mantissa bits), nearest with ties away.
__device__ __forceinline__ float tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// D[tmem] (+)= A[tmem] * B[smem]^T.  No memory clobber: the MMA reads
// shared and tensor memory asynchronously, and volatile keeps it in order with
// the barrier waits and commits around it.
__device__ __forceinline__ void mma_bf16_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
      "r"(a_tmem), "l"(bdesc), "r"(idesc), "r"(accumulate));
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

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void red_add(float* addr, float v) {
  asm volatile("red.global.add.f32 [%0], %1;" ::"l"(addr), "f"(v) : "memory");
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

// dy-tile visiting order: centre (heaviest overlap) first, then alternating
// outwards, so long tiles start early.
__host__ __device__ __forceinline__ int centre_out(int r, int n, int tc) {
  const int below = tc, above = n - tc - 1;
  const int m = below < above ? below : above;
  if (r == 0) return tc;
  if (r <= 2 * m) return (r & 1) ? tc + (r + 1) / 2 : tc - r / 2;
  const int extra = r - 2 * m;
  return above > below ? tc + m + extra : tc - m - extra;
}

// Active K-steps of a 128-shift tile starting at s0: bit j is set when
// A's K-step j (right columns kstep*j .. kstep*j + kstep - 1) meets a left
// column.
__device__ __forceinline__ uint32_t tile_mask(int s0, const TcParams& p) {
  uint32_t m = 0;
  if (s0 >= p.Sx) return 0;
  for (int j = 0; j < 4 * p.nkc; ++j) {
    const int k0 = p.kstep * j;
    if (k0 < p.Wr && s0 + k0 + 127 + p.kstep - 1 >= p.Wr - 1 && s0 + k0 <= p.Wr + p.Wl - 2) m |= 1u << j;
  }
  return m;
}

// One work item: two 128-shift tiles (one CTA half) of one (left matrix,
// partner group, row-shift group, chunk of left rows).
struct TcItem {
  int l, p0, dy0, a_lo, n_rows, rdim2, s0_0, s0_1;
  uint32_t mask0, mask1;
};

// idx = ((chunk * n_dytiles + rank) * per_rank + lp) * n_halves + half;
// false when the item has no left rows.
__device__ __forceinline__ bool tc_item(const TcParams& p, long long idx, TcItem* w) {
  const int half = (int)(idx % p.n_halves);
  const long long bid = idx / p.n_halves;
  const int per_rank = p.pm.n_left * p.n_pgroups;
  const int lp = (int)(bid % per_rank);
  const int rank = (int)((bid / per_rank) % p.n_dytiles);
  const int chunk = (int)(bid / ((long long)per_rank * p.n_dytiles));
  w->l = lp / p.n_pgroups;
  w->p0 = (lp % p.n_pgroups) * p.P;
  const int t = centre_out(rank, p.n_dytiles, (p.Hr - 1) / p.DY);
  w->dy0 = -(p.Hr - 1) + t * p.DY;
  const int tile_lo = max(0, w->dy0);
  const int tile_hi = min(p.Hl, w->dy0 + p.DY - 1 + p.Hr);
  w->a_lo = tile_lo + chunk * p.chunk_rows;
  const int a_hi = min(tile_hi, w->a_lo + p.chunk_rows);
  w->n_rows = a_hi - w->a_lo;
  w->rdim2 = p.pm.r_l != 0 ? w->l : 0;
  w->s0_0 = 256 * half;
  w->s0_1 = w->s0_0 + 128;
  w->mask0 = tile_mask(w->s0_0, p);
  w->mask1 = tile_mask(w->s0_1, p);
  return w->n_rows > 0;
}

// Lists the non-empty work items, most left rows first (a counting sort by
// row count): one block.  Every CTA of tc_kernel reads the same list.
__global__ void __launch_bounds__(1024) worklist_kernel(const TcParams p, long long n_total, int* __restrict__ items,
                                                        int* __restrict__ n_live) {
  __shared__ int cnt[kMaxChunkRows + 1];
  for (int r = threadIdx.x; r <= kMaxChunkRows; r += blockDim.x) cnt[r] = 0;
  __syncthreads();
  for (long long idx = threadIdx.x; idx < n_total; idx += blockDim.x) {
    TcItem w;
    if (tc_item(p, idx, &w)) atomicAdd(&cnt[w.n_rows], 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int r = p.chunk_rows; r >= 1; --r) {
      const int c = cnt[r];
      cnt[r] = run;  // first position of the items with r rows
      run += c;
    }
    *n_live = run;
  }
  __syncthreads();
  for (long long idx = threadIdx.x; idx < n_total; idx += blockDim.x) {
    TcItem w;
    if (tc_item(p, idx, &w)) items[atomicAdd(&cnt[w.n_rows], 1)] = (int)idx;
  }
}

__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t* r) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]),
      "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
      : "memory");
}

__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ uint32_t bf16x2_bits(__nv_bfloat162 v) { return *reinterpret_cast<uint32_t*>(&v); }

// 23 warps: at most 6 on one SM sub-partition, whose 16K registers cap a
// thread at 80.  TF: TF32 operands (K = 8 per MMA) instead of BF16 (K = 16).
template <bool TF>
__global__ void __launch_bounds__(kThreads, 1)
    tc_kernel(const __grid_constant__ CUtensorMap map_hi, const __grid_constant__ CUtensorMap map_lo,
              const TcParams p) {
  constexpr int kCols = 64;  // accumulator columns per epilogue warp
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* b_tiles = smem;                                                  // kStages x (hi, lo) x 16 KB
  // split left row as overlapping BF16 pairs, two rows: pairs[row][hi/lo][j] = (x_j, x_j+1)
  uint32_t* pairs = reinterpret_cast<uint32_t*>(smem + kStages * kStageBytes);    // 2 x 2 x kMaxLp
  long long* row_base = reinterpret_cast<long long*>(pairs + 4 * kMaxLp);         // 2 x 128 output row offsets
  uint64_t* bars = reinterpret_cast<uint64_t*>(row_base + 256);
  uint64_t* a_full = bars;              // [kStages] right-row tiles landed
  uint64_t* a_empty = bars + kStages;   // [kStages] tiles consumed
  uint64_t* s_full = bars + 2 * kStages;  // [2] Toeplitz ring slot written
  uint64_t* s_empty = s_full + 2;         // [2] ring slot consumed
  uint64_t* t_full = s_empty + 2;         // accumulators ready to drain
  uint64_t* t_empty = t_full + 1;         // accumulators drained
  uint64_t* mma_done = t_empty + 1;     // [2] one per issuer
  volatile int* abort_flag = reinterpret_cast<volatile int*>(mma_done + 2);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mma_done + 3);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // Persistent: the work list is sorted by left rows (heaviest first) and
  // dealt out in a snake order (round r gives position r*G + c, or
  // r*G + G-1-c on odd rounds); every role walks the same items and keeps its
  // pipeline counters running across them, so the next item's loads and
  // MMAs overlap the previous item's final adds.
  const long long n_items = *p.n_live;

  if (threadIdx.x == 0) {
    // consumed / accumulated barriers take one commit from each issuer
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&a_full[s], 1);
      mbar_init(&a_empty[s], 2);
    }
    for (int s = 0; s < 2; ++s) {
      mbar_init(&s_full[s], kBuilderWarps);
      mbar_init(&s_empty[s], 2);
    }
    mbar_init(t_full, 2);
    mbar_init(t_empty, kEpiWarps);
    mbar_init(&mma_done[0], 1);
    mbar_init(&mma_done[1], 1);
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
    if (lane == 0) {
      int it = 0;
      bool ok = true;
      for (long long round = 0; round * gridDim.x < n_items && ok; ++round) {
        const long long pos = round * gridDim.x + ((round & 1) ? gridDim.x - 1 - blockIdx.x : blockIdx.x);
        if (pos >= n_items) continue;
        TcItem w;
        if (!tc_item(p, p.items[pos], &w)) continue;
        for (int ai = 0; ai < w.n_rows && ok; ++ai) {
          const int a = w.a_lo + ai;
          for (int kc = 0; kc < p.nkc && ok; ++kc, ++it) {
            const int s = it % kStages;
            if (!wait_or_abort_sleep(&a_empty[s], ((it / kStages) & 1) ^ 1, abort_flag, p.flags, 11)) {
              ok = false;
              break;
            }
            mbar_arrive_expect_tx(&a_full[s], kStageBytes);
            unsigned char* hi = b_tiles + s * kStageBytes;
            unsigned char* lo = hi + kTileBytes;
            if (p.mats_mode) {
              for (int d = 0; d < p.DY; ++d) {
                const int b = a - (w.dy0 + d);
                tma_load_4d(hi + d * p.P * 128, &map_hi, &a_full[s], kc * 4 * p.kstep, b, w.rdim2, w.p0);
                tma_load_4d(lo + d * p.P * 128, &map_lo, &a_full[s], kc * 4 * p.kstep, b, w.rdim2, w.p0);
              }
            } else {
              const int b0 = a - w.dy0 - (p.DY - 1);
              for (int q = 0; q < p.P; ++q) {
                tma_load_4d(hi + q * p.DY * 128, &map_hi, &a_full[s], kc * 4 * p.kstep, b0, w.rdim2, w.p0 + q);
                tma_load_4d(lo + q * p.DY * 128, &map_lo, &a_full[s], kc * 4 * p.kstep, b0, w.rdim2, w.p0 + q);
              }
            }
          }
        }
      }
      if (!ok) {
        for (int q = max(0, it - kStages); q < it; ++q)
          mbar_wait_bounded(&a_full[q % kStages], (q / kStages) & 1, 1u << 16);
      }
    }
  } else if (warp == 1 || warp == 2 + kBuilderWarps + kEpiWarps) {
    // ------------------------------------------------------------ MMA issuers
    // Both walk the same items, rows and K-chunks and wait on the same
    // barriers; each issues the MMAs of its own shift tile and commits to
    // the shared consumed / accumulated barriers.
    const int my_tt = warp == 1 ? 0 : 1;
    if (lane == 0) {
      // The issue loop is on the critical path (a 128x128x16 MMA takes 64
      // cycles of tensor pipe): every per-item value lives in a scalar, the
      // stage / slot counters advance without divisions.
      constexpr uint32_t kDescHi = (1024u >> 4) | (1u << 14) | (2u << 29);  // SBO 1024 B, 128-byte swizzle
      const uint32_t idesc = TF ? idesc_tf32_f32(128, 128) : idesc_bf16_f32(128, 128);
      const uint32_t b_lo_word = ((smem_u32(b_tiles) >> 4) & 0x3FFFu) | (1u << 16);
      const uint32_t d_tmem = tmem_base + (uint32_t)my_tt * 128;
      const uint32_t a_base = tmem_base + kRingCol + (uint32_t)my_tt * 64;  // this tile's 4 K-steps of a slot
      int s = 0, slot = 0;                    // stage and ring slot of the next K-chunk
      uint32_t s_phase = 0, r_phase = 0, t_phase = 1;  // parities awaited on a_full, s_full, t_empty
      bool ok = true;
      for (long long round = 0; round * gridDim.x < n_items && ok; ++round) {
        const long long pos = round * gridDim.x + ((round & 1) ? gridDim.x - 1 - blockIdx.x : blockIdx.x);
        if (pos >= n_items) continue;
        TcItem w;
        if (!tc_item(p, p.items[pos], &w)) continue;
        const uint32_t my_mask = my_tt == 0 ? w.mask0 : w.mask1;
        const int first = my_mask ? __ffs(my_mask) - 1 : -1;
        const int n_rows = w.n_rows;
        int rows_in = 0;
        for (int ai = 0; ai < n_rows && ok; ++ai) {
          if (rows_in == 0) {
            // the epilogue must have drained the previous window
            if (!wait_or_abort(t_empty, t_phase, abort_flag, p.flags, 14)) {
              ok = false;
              break;
            }
            t_phase ^= 1u;
          }
          for (int kc = 0; kc < p.nkc; ++kc) {
            if (!wait_or_abort(&a_full[s], s_phase, abort_flag, p.flags, 13) ||
                !wait_or_abort(&s_full[slot], r_phase, abort_flag, p.flags, 12)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t pat = (my_mask >> (4 * kc)) & 0xFu;
            const int rk = (rows_in == 0 && (first >> 2) == kc) ? (first & 3) : -1;  // K-step that resets
            const uint32_t bw = b_lo_word + (uint32_t)s * (kStageBytes >> 4);
            const uint32_t ra = a_base + (uint32_t)slot * 128;
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
              if (!(pat & (1u << ks))) continue;
              const uint64_t bhi = make_desc(bw + ks * 2, kDescHi);
              const uint64_t blo = make_desc(bw + (kTileBytes >> 4) + ks * 2, kDescHi);
              const uint32_t ahi = ra + (uint32_t)ks * 16, alo = ahi + 8;
              const uint32_t acc0 = ks == rk ? 0u : 1u;
              if constexpr (TF) {
                mma_tf32_ts(d_tmem, ahi, bhi, idesc, acc0);
                mma_tf32_ts(d_tmem, ahi, blo, idesc, 1u);
                mma_tf32_ts(d_tmem, alo, bhi, idesc, 1u);
              } else {
                mma_bf16_ts(d_tmem, ahi, bhi, idesc, acc0);
                mma_bf16_ts(d_tmem, ahi, blo, idesc, 1u);
                mma_bf16_ts(d_tmem, alo, bhi, idesc, 1u);
              }
            }
            mma_commit(&a_empty[s]);
            mma_commit(&s_empty[slot]);
            if (++s == kStages) {
              s = 0;
              s_phase ^= 1u;
            }
            slot ^= 1;
            if (slot == 0) r_phase ^= 1u;
          }
          if (!ok) break;
          ++rows_in;
          if (rows_in == p.flush_rows || ai == n_rows - 1) {
            mma_commit(t_full);
            rows_in = 0;
          }
        }
      }
      // All MMAs issued by this thread must finish before TMEM is released.
      mma_commit(&mma_done[my_tt]);
      mbar_wait_bounded(&mma_done[my_tt], 0, 1u << 22);
    }
  } else if (warp < 2 + kBuilderWarps) {
    // ------------------------------------------------------------ Toeplitz builders
    // Lane m of TMEM quadrant q (m = 32 q + lane) is shift s0 + m; per K-step
    // it writes 8 columns of packed hi pairs and 8 of lo pairs, read from
    // the row's overlapping pair arrays (one 32-bit load per column).
    const int bt = threadIdx.x - 64;  // 0..127
    const int qd = warp & 3;
    const int m = 32 * qd + lane;
    const uint32_t lane_addr = tmem_base + ((uint32_t)(32 * qd) << 16) + kRingCol;
    int it = 0, rows_done = 0;
    bool ok = true;
    for (long long round = 0; round * gridDim.x < n_items && ok; ++round) {
      const long long pos = round * gridDim.x + ((round & 1) ? gridDim.x - 1 - blockIdx.x : blockIdx.x);
      if (pos >= n_items) continue;
      TcItem w;
      if (!tc_item(p, p.items[pos], &w)) continue;
      const float* lrow_base = p.left + (long long)w.l * p.Hl * p.Wl;
      const float mu = p.mu_left[w.l];
      for (int ai = 0; ai < w.n_rows; ++ai, ++rows_done) {
        // split the centred, zero-padded left row x_j = L[a][j - (Wr-1)] - mu
        // into pairs (x_j, x_j+1) of BF16 hi parts and of BF16 lo parts
        uint32_t* ph = pairs + (rows_done & 1) * (2 * kMaxLp);
        uint32_t* pl = ph + kMaxLp;
        const float* src = lrow_base + (long long)(w.a_lo + ai) * p.Wl;
        for (int j = bt; j < p.lp_len; j += 32 * kBuilderWarps) {
          const int x = j - (p.Wr - 1);
          const float x0 = (x >= 0 && x < p.Wl) ? __ldg(src + x) - mu : 0.0f;
          if constexpr (TF) {
            // TF32: one element per column, hi and lo parts
            const float h = tf32_round(x0);
            ph[j] = __float_as_uint(h);
            pl[j] = __float_as_uint(tf32_round(x0 - h));
          } else {
            const float x1 = (x + 1 >= 0 && x + 1 < p.Wl) ? __ldg(src + x + 1) - mu : 0.0f;
            const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
            ph[j] = bf16x2_bits(h);
            pl[j] = bf16x2_bits(__floats2bfloat162_rn(x0 - __low2float(h), x1 - __high2float(h)));
          }
        }
        // the builder threads leave together (they share a named barrier)
        if (bar_red_or(!ok, 1, 32 * kBuilderWarps)) {
          ok = false;
          break;
        }
        for (int kc = 0; kc < p.nkc; ++kc, ++it) {
          const int slot = it & 1;
          bool wt = wait_or_abort_sleep(&s_empty[slot], ((it >> 1) & 1) ^ 1, abort_flag, p.flags, 15);
          wt = __all_sync(0xffffffffu, wt);  // tcgen05.st below must stay warp-uniform
          if (!wt) {
            ok = false;
            break;
          }
          tc_fence_after();
#pragma unroll
          for (int tt = 0; tt < 2; ++tt) {
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
              const int j = kc * 4 + ks;
              if (!(((tt == 0 ? w.mask0 : w.mask1) >> j) & 1u)) continue;
              const int base = (tt == 0 ? w.s0_0 : w.s0_1) + m + p.kstep * j;
              uint32_t r[16];
#pragma unroll
              for (int e = 0; e < 8; ++e) {
                r[e] = ph[base + (TF ? 1 : 2) * e];
                r[8 + e] = pl[base + (TF ? 1 : 2) * e];
              }
              tmem_st16(lane_addr + (uint32_t)slot * 128 + (uint32_t)(tt * 4 + ks) * 16, r);
            }
          }
          tmem_wait_st();
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&s_full[slot]);  // one arrival per warp
        }
        // a failed wait reaches the other builders at the next row's barrier
      }
    }
  } else if (warp < 2 + kBuilderWarps + kEpiWarps) {
    // ------------------------------------------------------------ epilogue
    // Warp w (index ew = w - 6): lane quadrant q = w % 4, accumulator
    // columns [64 * (ew / 4), +64): tile tt = ew / 8, B rows nb.. of it.
    const int ew = warp - (2 + kBuilderWarps);
    const int q = warp & 3;
    const int tt = ew >> 3;
    const int nb = ((ew >> 2) & 1) * kCols;
    const int et = threadIdx.x - 32 * (2 + kBuilderWarps);  // 0..511
    int d_all = 0, n_done = 0;
    bool ok = true;
    for (long long round = 0; round * gridDim.x < n_items && ok; ++round) {
      const long long pos = round * gridDim.x + ((round & 1) ? gridDim.x - 1 - blockIdx.x : blockIdx.x);
      if (pos >= n_items) continue;
      TcItem w;
      if (!tc_item(p, p.items[pos], &w)) continue;
      long long* rbase = row_base + (n_done & 1) * 128;
      if (et < 128) {
        // output row offset of B row n (-1: outside the output)
        const int n = et;
        int pp, dy;
        if (p.mats_mode) {
          pp = n % p.P;
          dy = w.dy0 + n / p.P;
        } else {
          pp = n / p.DY;
          dy = w.dy0 + (p.DY - 1) - (n % p.DY);
        }
        const int k = w.p0 + pp, sy = dy + p.Hr - 1;
        rbase[n] = (k < p.pm.K && sy >= 0 && sy < p.Sy)
                       ? (((long long)w.l * p.pm.o_l + (long long)k * p.pm.o_k) * p.Sy + sy) * p.Sx
                       : -1LL;
      }
      // publishes the table; every epilogue thread has finished the item
      // that used this half of it two items ago
      asm volatile("bar.sync 2, %0;" ::"r"(32 * kEpiWarps) : "memory");
      float acc[kCols];
#pragma unroll
      for (int i = 0; i < kCols; ++i) acc[i] = 0.0f;
      const uint32_t tmask = tt == 0 ? w.mask0 : w.mask1;
      const bool live = tmask != 0u;
      const int n_drains = (w.n_rows + p.flush_rows - 1) / p.flush_rows;
      for (int d = 0; d < n_drains; ++d, ++d_all) {
        bool wt = wait_or_abort_sleep(t_full, d_all & 1, abort_flag, p.flags, 16);
        wt = __all_sync(0xffffffffu, wt);  // tcgen05.ld below must stay warp-uniform
        if (!wt) {
          ok = false;
          break;
        }
        tc_fence_after();
        if (live) {
          const uint32_t col0 = tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(tt * 128 + nb);
#pragma unroll
          for (int j = 0; j < kCols; j += 8) {
            float v[8];
            tmem_ld8(col0 + (uint32_t)j, v);
            tmem_wait_ld();
#pragma unroll
            for (int i = 0; i < 8; ++i) acc[j + i] += v[i];
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(t_empty);  // one arrival per warp
      }
      const int sx = (tt == 0 ? w.s0_0 : w.s0_1) + 32 * q + lane;
      if (ok && live && sx < p.Sx) {
#pragma unroll
        for (int i = 0; i < kCols; ++i) {
          const long long rb = rbase[nb + i];
          if (rb >= 0) red_add(p.out + rb + sx, acc[i]);
        }
      }
      ++n_done;
    }
  }

  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(512) : "memory");
  }
}

// Matrix sums for the means: grid (matrix, slice); FP64 partial sums of a
// slice, block-reduced, added into sums[m] (zeroed before the launch).
__global__ void __launch_bounds__(256) sum_kernel(const float* __restrict__ src, long long area, int slices,
                                                  double* __restrict__ sums) {
  __shared__ double red[8];
  const int m = blockIdx.x / slices, sl = blockIdx.x % slices;
  const long long per = (area + slices - 1) / slices;
  const long long lo = sl * per, hi = min(area, lo + per);
  const float* a = src + (long long)m * area;
  // FP32 within a thread (at most a few dozen terms; FP64 arithmetic is slow
  // on this GPU), FP64 across threads and blocks
  float part = 0.0f;
  for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) part += __ldg(a + i);
  double acc = (double)part;
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int j = 0; j < 8; ++j) t += red[j];
    atomicAdd(&sums[m], t);
  }
}

__global__ void mean_kernel(const double* __restrict__ sums, int n_left, double left_area, int n_total,
                            double right_area, float* __restrict__ mu) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m < n_total) mu[m] = (float)(sums[m] / (m < n_left ? left_area : right_area));
}

// Column prefix sums of the centred matrices fl32(M - mu) (the values the
// split sees): C[m][y][x] = sum_{i<y} fl32(M[m][i][x] - mu_m), (H+1) x W per
// matrix, FP32.  Centred, these sums are random walks of modest size, so FP32
// holds them to ~1e-7; the summation is blocked (8-row segments, a carry per
// 64-row chunk), which keeps every FP32 chain short.  One block per (matrix,
// 32-column strip); each of its 8 warps loads 8 consecutive rows of a chunk
// (coalesced, independent loads).
__global__ void __launch_bounds__(256) colsum_kernel(const float* __restrict__ src, int H, int W,
                                                     const float* __restrict__ mu, float* __restrict__ C) {
  __shared__ float seg[8][32];
  __shared__ float carry[32];
  const int strips = (W + 31) / 32;
  const int m = blockIdx.x / strips;
  const int lane = threadIdx.x & 31;
  const int x = (blockIdx.x % strips) * 32 + lane;
  const int w = threadIdx.x >> 5;
  const float* a = src + (long long)m * H * W;
  float* c = C + (long long)m * (H + 1) * W;
  const float mv = mu[m];
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
        if (yb + i < H) c[(long long)(yb + i + 1) * W + x] = off + run[i];
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

// Exclusive prefix of q[1..n] in place by one warp (q[0] = 0 on entry):
// afterwards q[x] = sum of the first x band values.  Each lane scans a
// contiguous segment, then a shuffle scan combines the segment totals.
__device__ __forceinline__ void warp_scan_inplace(float* q, int n, int lane) {
  const int per = (n + 31) / 32;
  const int lo = 1 + lane * per, hi = min(n + 1, lo + per);
  float acc = 0.0f;
  for (int i = lo; i < hi; ++i) {
    acc += q[i];
    q[i] = acc;
  }
  float v = acc;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const float u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += u;
  }
  const float off = v - acc;
  for (int i = lo; i < hi; ++i) q[i] += off;
  __syncwarp();
}

// Splits the centred right matrices fl32(R - mu_R) into hi/lo planes with a
// padded pitch: BF16 (T = __nv_bfloat16) or TF32-rounded FP32 (T = float).
template <typename T>
__global__ void split_kernel(const float* __restrict__ src, const float* __restrict__ mu, T* __restrict__ hi,
                             T* __restrict__ lo, long long rows, int rows_per_matrix, int cols, int pitch) {
  const long long total = rows * pitch;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long r = i / pitch;
    const int c = (int)(i % pitch);
    const float v = c < cols ? src[r * cols + c] - mu[r / rows_per_matrix] : 0.0f;
    if constexpr (sizeof(T) == 4) {
      const float h = tf32_round(v);
      hi[i] = h;
      lo[i] = tf32_round(v - h);
    } else {
      const __nv_bfloat16 h = __float2bfloat16_rn(v);
      hi[i] = h;
      lo[i] = __float2bfloat16_rn(v - __bfloat162float(h));
    }
  }
}

// out[o][sy][sx] = mu_R * S_L' + mu_L * S_R' + mu_L * mu_R * area over the
// overlap of shift (sy, sx), where S' are sums of the centred matrices; one
// warp per output row (8 rows per block, no block-wide barrier).  The band
// sums of the overlapping rows, b[x] = C[y1][x] - C[y0][x] (centred column
// prefix sums), are scanned along x in the warp's shared-memory slice;
// everything is FP32 (the centred sums are small, and the result's rounding
// stays near 1e-7 of max|out|).
__global__ void __launch_bounds__(256) correction_kernel(float* __restrict__ out, const float* __restrict__ CL,
                                                         const float* __restrict__ CR,
                                                         const float* __restrict__ mu_l,
                                                         const float* __restrict__ mu_r, int Hl, int Wl, int Hr,
                                                         int Wr, int Sy, int Sx, long long n_rows, PairMap pm) {
  extern __shared__ float qs[];  // 8 x ((Wl + 1) + (Wr + 1))
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const long long row = blockIdx.x * 8LL + wid;  // o * Sy + sy
  if (row >= n_rows) return;  // warp-uniform
  const long long o = row / Sy;
  const int sy = (int)(row % Sy);
  // invert o = l*o_l + k*o_k for the three pair-map forms
  long long l, k;
  if (pm.o_l == 0) {  // one_to_one / one_to_many: o = k
    l = 0;
    k = o;
  } else if (pm.o_k == 1 && pm.o_l == pm.K) {  // n_to_m: o = l*K + k
    l = o / pm.K;
    k = o % pm.K;
  } else {  // n_to_mn: o = l + k*n
    l = o % pm.n_left;
    k = o / pm.n_left;
  }
  const long long r = l * pm.r_l + k * pm.r_k;
  const int dy = sy - (Hr - 1);
  const int y0 = max(0, dy), y1 = min(Hl, Hr + dy);
  const float* cl0 = CL + (l * (Hl + 1) + y0) * (long long)Wl;
  const float* cl1 = CL + (l * (Hl + 1) + y1) * (long long)Wl;
  const float* cr0 = CR + (r * (Hr + 1) + (y0 - dy)) * (long long)Wr;
  const float* cr1 = CR + (r * (Hr + 1) + (y1 - dy)) * (long long)Wr;
  float* ql = qs + wid * (Wl + Wr + 2);
  float* qr = ql + (Wl + 1);
  for (int x = lane; x < Wl; x += 32) ql[x + 1] = cl1[x] - cl0[x];
  for (int x = lane; x < Wr; x += 32) qr[x + 1] = cr1[x] - cr0[x];
  if (lane == 0) {
    ql[0] = 0.0f;
    qr[0] = 0.0f;
  }
  __syncwarp();
  warp_scan_inplace(ql, Wl, lane);
  warp_scan_inplace(qr, Wr, lane);
  const float ml = mu_l[l], mr = mu_r[r];
  const float mlr = ml * mr;
  const float rows = (float)(y1 - y0);
  float* orow = out + row * Sx;
  for (int sx = lane; sx < Sx; sx += 32) {
    const int dx = sx - (Wr - 1);
    const int x0 = max(0, dx), x1 = min(Wl, Wr + dx);
    const float sl = ql[x1] - ql[x0];
    const float sr = qr[x1 - dx] - qr[x0 - dx];
    orow[sx] = fmaf(mr, sl, fmaf(ml, sr, mlr * (rows * (float)(x1 - x0))));
  }
}

struct TcPlan {
  int P, DY, mats_mode, n_tiles, n_halves, nkc, kstep, es, lp_len, pitch, n_chunks;
  long long n_items;
  int smem_bytes;
};

int chunk_rows();

bool tc_plan(const Geometry& g, const PairMap& pm, bool tf32, TcPlan* t) {
  if (g.Sx > 512 || g.Wr > 256) return false;  // four 128-shift tiles, 16 K-steps
  int P = 1;
  while (P < 128 && P < pm.K) P *= 2;
  t->P = P;
  t->DY = 128 / P;
  t->mats_mode = P >= 8 ? 1 : 0;
  t->n_tiles = (g.Sx + 127) / 128;
  t->n_halves = (t->n_tiles + 1) / 2;
  t->es = tf32 ? 4 : 2;                 // bytes per operand element
  t->kstep = tf32 ? 8 : 16;             // columns per MMA K-step (32 bytes)
  const int chunk = 128 / t->es;        // columns per 128-byte TMA box row
  t->nkc = (g.Wr + chunk - 1) / chunk;
  t->lp_len = 128 * t->n_tiles + 4 * t->kstep * t->nkc;
  t->pitch = (g.Wr + 16 / t->es - 1) / (16 / t->es) * (16 / t->es);
  t->n_chunks = div_up(t->DY - 1 + std::min(g.Hl, g.Hr), chunk_rows());
  t->n_items = (long long)t->n_halves * t->n_chunks * div_up(g.Sy, t->DY) * pm.n_left * div_up(pm.K, t->P);
  t->smem_bytes = 1024 + kStages * kStageBytes + 4 * kMaxLp * 4 + 2 * 128 * 8 + kBarBytes;
  return t->lp_len <= kMaxLp && t->smem_bytes <= 227 * 1024;
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

// Left rows accumulated in tensor memory between two drains: at most 192
// MMAs (12 per 64-column chunk of a right row: 4 K-steps x 3 products) feed
// one accumulator between drains, which keeps the truncation error of the
// tensor-core accumulation (about 5e-8 of the partial sum per MMA, measured)
// near 5e-8 x 192 ~ 1e-5 of the largest partial sum, even for zero-mean data
// whose partial sums are as large as the result.
// XC_TC_FLUSH_ROWS / XC_TC_CHUNK_ROWS override the defaults (studies).
int flush_rows(int nkc) {
  static const int v = env_int("XC_TC_FLUSH_ROWS", 0);
  if (v > 0) return v;
  return std::max(1, std::min(32, 192 / (12 * nkc)));
}
int chunk_rows() {
  static int v = std::min(kMaxChunkRows, env_int("XC_TC_CHUNK_ROWS", 32));
  return v;
}

// Workspace layout (each part 256-byte aligned).
struct TcWs {
  float* mu;        // n_left + n_right means
  double* sums;     // n_left + n_right matrix sums
  float* CL;        // n_left x (Hl+1) x Wl centred column prefix sums
  float* CR;        // n_right x (Hr+1) x Wr
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
  w.sums = reinterpret_cast<double*>(take(sizeof(double) * (pm.n_left + nr)));
  w.CL = reinterpret_cast<float*>(take(sizeof(float) * (size_t)pm.n_left * (g.Hl + 1) * g.Wl));
  w.CR = reinterpret_cast<float*>(take(sizeof(float) * (size_t)nr * (g.Hr + 1) * g.Wr));
  w.hi = take((size_t)t.es * plane);
  w.lo = take((size_t)t.es * plane);
  w.items = reinterpret_cast<int*>(take(sizeof(int) * ((size_t)t.n_items + 1)));  // list + its length
  w.bytes = off + 256;
  return w;
}

}  // namespace

size_t tc_workspace_size(const Geometry& g, const PairMap& pm, bool tf32) {
  TcPlan t;
  if (!tc_plan(g, pm, tf32, &t)) return 0;
  return ws_layout(nullptr, g, pm, t).bytes;
}

xc_status tc_correlate(const float* left, const float* right, float* out, const Geometry& g, const PairMap& pm,
                       void* workspace, size_t ws_bytes, cudaStream_t stream, bool tf32) {
  TcPlan t;
  if (!tc_plan(g, pm, tf32, &t))
    return fail(XC_ERR_UNSUPPORTED,
                "split tensor-core paths support outputs up to 512 columns and right widths up to 256");
  const size_t need = ws_layout(nullptr, g, pm, t).bytes;
  if (workspace == nullptr || ws_bytes < need)
    return fail(XC_ERR_WORKSPACE, "split tensor-core path needs " + std::to_string(need) + " bytes of workspace");
  const TcWs w = ws_layout(reinterpret_cast<void*>(((uintptr_t)workspace + 255) & ~uintptr_t(255)), g, pm, t);
  const long long nr = n_right_of(pm);
  const int nl = pm.n_left;
  const uint64_t n_out = (uint64_t)((long long)(nl - 1) * pm.o_l + (long long)(pm.K - 1) * pm.o_k + 1);

  // 1. per-matrix means, 2. column prefix sums of the centred matrices
  {
    const long long la = (long long)g.Hl * g.Wl, ra = (long long)g.Hr * g.Wr;
    // slices of at most 8192 elements: a thread adds at most 32 terms in FP32
    const int ls = (int)((la + 8191) / 8192), rs = (int)((ra + 8191) / 8192);
    XC_CUDA_TRY(cudaMemsetAsync(w.sums, 0, sizeof(double) * (nl + nr), stream));
    sum_kernel<<<(unsigned)(nl * ls), 256, 0, stream>>>(left, la, ls, w.sums);
    XC_CUDA_TRY(cudaGetLastError());
    sum_kernel<<<(unsigned)(nr * rs), 256, 0, stream>>>(right, ra, rs, w.sums + nl);
    XC_CUDA_TRY(cudaGetLastError());
    mean_kernel<<<(unsigned)((nl + nr + 255) / 256), 256, 0, stream>>>(w.sums, nl, (double)la, (int)(nl + nr),
                                                                        (double)ra, w.mu);
    XC_CUDA_TRY(cudaGetLastError());
  }
  colsum_kernel<<<(unsigned)(nl * ((g.Wl + 31) / 32)), 256, 0, stream>>>(left, g.Hl, g.Wl, w.mu, w.CL);
  XC_CUDA_TRY(cudaGetLastError());
  colsum_kernel<<<(unsigned)(nr * ((g.Wr + 31) / 32)), 256, 0, stream>>>(right, g.Hr, g.Wr, w.mu + nl, w.CR);
  XC_CUDA_TRY(cudaGetLastError());
  // 3. split of the centred right matrices
  {
    const long long rows = nr * g.Hr;
    long long blocks = (rows * t.pitch + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    if (tf32)
      split_kernel<float><<<(unsigned)blocks, 256, 0, stream>>>(right, w.mu + nl, (float*)w.hi, (float*)w.lo, rows,
                                                                 g.Hr, g.Wr, t.pitch);
    else
      split_kernel<__nv_bfloat16><<<(unsigned)blocks, 256, 0, stream>>>(
          right, w.mu + nl, (__nv_bfloat16*)w.hi, (__nv_bfloat16*)w.lo, rows, g.Hr, g.Wr, t.pitch);
    XC_CUDA_TRY(cudaGetLastError());
  }
  // 4. the mean terms initialise the output
  {
    const long long n_rows = (long long)n_out * g.Sy;
    const size_t smem = sizeof(float) * 8 * (g.Wl + g.Wr + 2);
    XC_CUDA_TRY(cudaFuncSetAttribute(correction_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    correction_kernel<<<(unsigned)((n_rows + 7) / 8), 256, smem, stream>>>(
        out, w.CL, w.CR, w.mu, w.mu + nl, g.Hl, g.Wl, g.Hr, g.Wr, g.Sy, g.Sx, n_rows, pm);
  }
  XC_CUDA_TRY(cudaGetLastError());

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
  prm.n_halves = t.n_halves;
  prm.nkc = t.nkc;
  prm.lp_len = t.lp_len;
  prm.kstep = t.kstep;
  prm.flush_rows = flush_rows(t.nkc);
  prm.chunk_rows = chunk_rows();
  prm.n_chunks = t.n_chunks;
  prm.flags = device_flags();

  // the work list: non-empty items, most left rows first, built on the device
  if (t.n_items > 0x7fffffffLL) return fail(XC_ERR_INVALID_ARGUMENT, "problem too large for one launch");
  prm.items = w.items;
  prm.n_live = w.items + t.n_items;
  worklist_kernel<<<1, 1024, 0, stream>>>(prm, t.n_items, w.items, w.items + t.n_items);
  XC_CUDA_TRY(cudaGetLastError());
  // persistent: one CTA per SM (211 KB of shared memory and all 512 TMEM
  // columns each), walking the items round-robin
  int dev = 0, sms = 0;
  XC_CUDA_TRY(cudaGetDevice(&dev));
  XC_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const long long blocks = std::max(1LL, std::min<long long>(t.n_items, sms));
  auto kern = tf32 ? tc_kernel<true> : tc_kernel<false>;
  XC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, t.smem_bytes));
  const int slot = kernel_timer_begin(stream);
  kern<<<(unsigned)blocks, kThreads, t.smem_bytes, stream>>>(mhi, mlo, prm);
  kernel_timer_end(slot, stream);
  XC_CUDA_TRY(cudaGetLastError());
  return XC_OK;
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

// Device address of the scratch array for the current device, looked up once
// per device (with that device current) and cached.
xc_status noalloc_scratch(void** ptr) {
  int dev = 0;
  XC_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(XC_ERR_INVALID_ARGUMENT, "device index out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (g_noalloc_ptr[dev] == nullptr) {
    void* p = nullptr;
    XC_CUDA_TRY(cudaGetSymbolAddress(&p, g_tc_noalloc_scratch));
    g_noalloc_ptr[dev] = p;
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
                "split-BF16 tensor path supports outputs up to 512 columns and right widths up to 256");
  const size_t need = ws_layout(nullptr, g, pm, t).bytes;
  if (need > (size_t)XC_TC_NOALLOC_SCRATCH_BYTES)
    return fail(XC_ERR_WORKSPACE, "xc_correlate_tc_noalloc: this problem needs " + std::to_string(need) +
                                      " bytes of scratch, more than the fixed " +
                                      std::to_string((size_t)XC_TC_NOALLOC_SCRATCH_BYTES) +
                                      " bytes; use xc_correlate with a caller-owned workspace");
  void* scratch = nullptr;
  XC_TRY(noalloc_scratch(&scratch));
  return tc_correlate(d_left, d_right, d_out, g, pm, scratch, (size_t)XC_TC_NOALLOC_SCRATCH_BYTES,
                      reinterpret_cast<cudaStream_t>(stream), false);
}
