// tc_bf16x3.cu -- split-BF16 tensor-core correlation on tcgen05 (sm_103a).
//
// FP32 inputs, FP32 outputs, three BF16 products per FP32 product:
//   x = x_hi + x_lo, x_hi = bf16(x), x_lo = bf16(x - x_hi)
//   L*R ~= L_hi*R_hi + L_hi*R_lo + L_lo*R_hi      (Henry, Tang & Heinecke 2019)
//
// Formulation (implicit GEMM).  For a left row a and a right row b the
// contribution to output row sy = a - b + Hr - 1 is a 1D correlation, a
// Toeplitz matrix-vector product.  One tcgen05.mma computes
//     D[m][n] += sum_k A[m][k] * B[n][k]        (M=128, N<=64, K=16, BF16)
// with
//   m -> (partner matrix p, row shift dy): A[m][k] = R_p[a - dy][k0 + k]
//        (right rows, staged by TMA with 128-byte swizzle, K-major);
//   n -> column shift sx = c + 8n for a phase c in 0..7:
//        B[n][k] = Lpad_a[c + 8n + k0 + k]
//        where Lpad_a[j] = L[a][j - (Wr-1)] (zero outside the row).
// B is a Toeplitz matrix.  It is read straight out of one shared-memory copy
// of the (split) left row per phase c: a no-swizzle K-major descriptor whose
// 8x16-byte core matrices overlap (leading byte offset 16 = 8 elements along
// K, stride byte offset 128 = 64 elements along N) addresses element
// 8n + k of the copy.  Nothing is materialised per shift; eight phase copies
// of each left row cover every column shift.
//
// The accumulator tile is 128 lanes x (8 phases x N) FP32 columns of tensor
// memory.  Every `flush_rows` left rows the epilogue warps drain it into the
// output with FP32 reductions (red.global.add), so long row ranges can also
// be split over several CTAs; the MMA warp waits during a drain.
//
// Accuracy.  Tensor-core FP32 accumulation drops low bits on every MMA with a
// consistent sign, so the error of a long chain grows linearly with its
// length and with the magnitude of the partial sums (measured on GB300:
// ~1.2e-6 of max|out| per 48-MMA left row for uniform [0,1) data).  Each
// matrix is therefore shifted by its mean before the split
// (L' = L - mu_L, R' = R - mu_R): the tensor cores correlate the centred data,
// whose partial sums are small random walks, and the exact remainder
//   out = corr(L', R') + mu_R * S_L' + mu_L * S_R' + mu_L * mu_R * area
// (S = sum of the centred matrix over the overlap of a shift, from FP64 2D
// prefix sums) is written first by a correction kernel, which the tensor-core
// drains then accumulate into.
//
// Warp roles (256 threads, one CTA per SM):
//   warp 0    TMA producer of the right-row tiles (hi and lo planes)
//   warp 1    TMEM allocation and the single-thread MMA issuer
//   warps 2-3 build the eight phase copies of each split left row
//   warps 4-7 epilogue (tcgen05.ld -> shared staging -> coalesced global)
// All waits are bounded: an expired wait records a flag, the CTA winds down,
// waits (bounded) for its own copies and MMAs, frees TMEM and returns.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdlib>
#include <mutex>
#include <string>

#include "xc_common.cuh"
#include "xc_internal.h"

namespace xc {

namespace {

constexpr int kStages = 4;          // right-row tile pipeline depth
constexpr int kTileBytes = 128 * 128;  // 128 rows x 64 bf16 (one plane)
constexpr int kStageBytes = 2 * kTileBytes;
constexpr int kEpiWarps = 8;        // epilogue warps (2 per TMEM lane quadrant)
constexpr int kThreads = 32 * (4 + kEpiWarps);
constexpr int kMaxLeftCols = 512;   // staged centred left row (Sx <= 512 on this path)
// 17 mbarriers (136 B), the abort flag and the TMEM address slot
constexpr int kBarBytes = 256;

struct TcParams {
  const float* left;
  const float* mu_left;  // mean of every left matrix (the shift of the split)
  float* out;
  int Hl, Wl, Hr, Wr, Sy, Sx;
  PairMap pm;
  int P, DY;        // partners x row shifts per tile, P*DY = 128
  int mats_mode;    // 1: one TMA box per row shift spans P partners; 0: one box per partner spans DY rows
  int n_pgroups;    // ceil(K / P)
  int n_dytiles;    // ceil(Sy / DY)
  int N;            // B rows per phase (multiple of 16, 8N >= Sx)
  int nkc;          // 64-column chunks of a right row
  int buf_len;      // elements of one phase copy (multiple of 8)
  int flush_rows;   // drain TMEM every this many left rows
  int chunk_rows;   // left rows per CTA (a longer row range is split over CTAs)
  int n_chunks;     // chunks per (dy tile): ceil(max rows / chunk_rows)
  DeviceFlags* flags;
};

// ---------------------------------------------------------------------------
// tcgen05 / descriptor helpers
// ---------------------------------------------------------------------------
// Shared-memory matrix descriptor (sm_100 family): start>>4 [0,14), LBO>>4
// [16,30), SBO>>4 [32,46), version 1 at bit 46, layout type [61,64)
// (0 = no swizzle, 2 = 128-byte swizzle).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo, uint32_t layout) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)(layout & 7u) << 61;
  return d;
}

// Instruction descriptor, kind::f16: D=F32 (bits 4-5 = 1), A=B=BF16 (bits 7-9,
// 10-12 = 1), both K-major, N>>3 at bit 17, M>>4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
      "[%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

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
__device__ __forceinline__ int centre_out(int r, int n, int tc) {
  const int below = tc, above = n - tc - 1;
  const int m = min(below, above);
  if (r == 0) return tc;
  if (r <= 2 * m) return (r & 1) ? tc + (r + 1) / 2 : tc - r / 2;
  const int extra = r - 2 * m;
  return above > below ? tc + m + extra : tc - m - extra;
}

template <int N>
__global__ void __launch_bounds__(kThreads, 1)
    tc_kernel(const __grid_constant__ CUtensorMap map_hi, const __grid_constant__ CUtensorMap map_lo,
              const TcParams p) {
  constexpr int kPhases = 4;            // column phases handled by this CTA
  constexpr int kDCols = kPhases * N;   // TMEM columns of one accumulator buffer
  constexpr int kAcc = 2 * N;           // accumulators per epilogue thread (4 phases x N/2)
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* a_tiles = smem;  // kStages x (hi, lo) x 16 KB
  __nv_bfloat16* b_bufs = reinterpret_cast<__nv_bfloat16*>(smem + kStages * kStageBytes);
  const int b_slot_elems = kPhases * 2 * p.buf_len;  // 4 phases x (hi, lo) per slot
  float* lrows = reinterpret_cast<float*>(b_bufs + 2 * b_slot_elems);  // 2 x kMaxLeftCols
  uint64_t* bars = reinterpret_cast<uint64_t*>(lrows + 2 * kMaxLeftCols);
  uint64_t* a_full = bars;
  uint64_t* a_empty = bars + kStages;
  uint64_t* b_full = bars + 2 * kStages;
  uint64_t* b_empty = b_full + 2;
  uint64_t* t_full = b_empty + 2;   // [2]
  uint64_t* t_empty = t_full + 2;   // [2]
  uint64_t* mma_done = t_empty + 2;
  volatile int* abort_flag = reinterpret_cast<volatile int*>(mma_done + 1);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mma_done + 2);

  // ---- work item of this CTA ---------------------------------------------
  // blockIdx = ((chunk * n_dytiles + rank) * per_rank + lp) * 2 + half
  const int half = blockIdx.x & 1;
  const int bid = blockIdx.x >> 1;
  const int per_rank = p.pm.n_left * p.n_pgroups;
  const int lp = bid % per_rank;
  const int rank = (bid / per_rank) % p.n_dytiles;
  const int chunk = bid / (per_rank * p.n_dytiles);
  const int l = lp / p.n_pgroups;
  const int p0 = (lp % p.n_pgroups) * p.P;
  const int t = centre_out(rank, p.n_dytiles, (p.Hr - 1) / p.DY);
  const int dy0 = -(p.Hr - 1) + t * p.DY;
  const int tile_lo = max(0, dy0);
  const int tile_hi = min(p.Hl, dy0 + p.DY - 1 + p.Hr);
  const int a_lo = tile_lo + chunk * p.chunk_rows;
  const int a_hi = min(tile_hi, a_lo + p.chunk_rows);
  const int n_rows = a_hi - a_lo;
  if (n_rows <= 0) return;  // uniform over the CTA
  const int n_drains = (n_rows + p.flush_rows - 1) / p.flush_rows;
  const int rdim2 = p.pm.r_l != 0 ? l : 0;
  constexpr uint32_t ncols = 2 * kDCols <= 32 ? 32u : (2 * kDCols <= 64 ? 64u : (2 * kDCols <= 128 ? 128u : (2 * kDCols <= 256 ? 256u : 512u)));

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&a_full[s], 1);
      mbar_init(&a_empty[s], 1);
    }
    for (int s = 0; s < 2; ++s) {
      mbar_init(&b_full[s], 64);
      mbar_init(&b_empty[s], 1);
      mbar_init(&t_full[s], 1);
      mbar_init(&t_empty[s], 32 * kEpiWarps);
    }
    mbar_init(mma_done, 1);
    *abort_flag = 0;
    fence_mbar_init();
    prefetch_tensormap(&map_hi);
    prefetch_tensormap(&map_lo);
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(ncols)
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
      for (int ai = 0; ai < n_rows && ok; ++ai) {
        const int a = a_lo + ai;
        for (int kc = 0; kc < p.nkc && ok; ++kc, ++it) {
          const int s = it % kStages;
          if (!wait_or_abort(&a_empty[s], ((it / kStages) & 1) ^ 1, abort_flag, p.flags, 11)) {
            ok = false;
            break;
          }
          mbar_arrive_expect_tx(&a_full[s], kStageBytes);
          unsigned char* hi = a_tiles + s * kStageBytes;
          unsigned char* lo = hi + kTileBytes;
          if (p.mats_mode) {
            for (int d = 0; d < p.DY; ++d) {
              const int b = a - (dy0 + d);
              tma_load_4d(hi + d * p.P * 128, &map_hi, &a_full[s], kc * 64, b, rdim2, p0);
              tma_load_4d(lo + d * p.P * 128, &map_lo, &a_full[s], kc * 64, b, rdim2, p0);
            }
          } else {
            const int b0 = a - dy0 - (p.DY - 1);
            for (int q = 0; q < p.P; ++q) {
              tma_load_4d(hi + q * p.DY * 128, &map_hi, &a_full[s], kc * 64, b0, rdim2, p0 + q);
              tma_load_4d(lo + q * p.DY * 128, &map_lo, &a_full[s], kc * 64, b0, rdim2, p0 + q);
            }
          }
        }
      }
      if (!ok) {
        for (int q = max(0, it - kStages); q < it; ++q)
          mbar_wait_bounded(&a_full[q % kStages], (q / kStages) & 1, 1u << 16);
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      const uint32_t idesc = idesc_bf16_f32(128, N);
      const uint32_t a_base = smem_u32(a_tiles);
      const uint32_t b_base = smem_u32(b_bufs);
      const uint32_t copy_bytes = (uint32_t)p.buf_len * 2;
      int it = 0, buf = 0, rows_in = 0;
      uint32_t uses[2] = {0u, 0u};
      bool ok = true;
      for (int ai = 0; ai < n_rows && ok; ++ai) {
        const int bs = ai & 1;
        if (!wait_or_abort(&b_full[bs], (ai >> 1) & 1, abort_flag, p.flags, 12)) {
          ok = false;
          break;
        }
        if (rows_in == 0) {
          // the epilogue must have drained this buffer's previous use
          if (!wait_or_abort(&t_empty[buf], (uses[buf] & 1) ^ 1, abort_flag, p.flags, 14)) {
            ok = false;
            break;
          }
        }
        tc_fence_after();
        const uint32_t bslot = b_base + (uint32_t)bs * (uint32_t)b_slot_elems * 2;
        const uint32_t dbase = tmem_base + (uint32_t)(buf * kDCols);
        for (int kc = 0; kc < p.nkc; ++kc, ++it) {
          const int s = it % kStages;
          if (!wait_or_abort(&a_full[s], (it / kStages) & 1, abort_flag, p.flags, 13)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t a_hi_addr = a_base + (uint32_t)s * kStageBytes;
          const uint32_t a_lo_addr = a_hi_addr + kTileBytes;
#pragma unroll 1
          for (int ks = 0; ks < 4; ++ks) {
            const uint64_t ahi = smem_desc(a_hi_addr + ks * 32, 16, 1024, 2);
            const uint64_t alo = smem_desc(a_lo_addr + ks * 32, 16, 1024, 2);
            const uint32_t koff = (uint32_t)(kc * 64 + ks * 16) * 2;
            const uint32_t acc0 = (rows_in == 0 && kc == 0 && ks == 0) ? 0u : 1u;
#pragma unroll
            for (int c = 0; c < kPhases; ++c) {
              const uint32_t bhi_addr = bslot + (uint32_t)c * 2 * copy_bytes + koff;
              const uint64_t bhi = smem_desc(bhi_addr, 16, 128, 0);
              const uint64_t blo = smem_desc(bhi_addr + copy_bytes, 16, 128, 0);
              const uint32_t d = dbase + (uint32_t)(c * N);
              mma_bf16(d, ahi, bhi, idesc, acc0);
              mma_bf16(d, ahi, blo, idesc, 1u);
              mma_bf16(d, alo, bhi, idesc, 1u);
            }
          }
          mma_commit(&a_empty[s]);
        }
        if (!ok) break;
        mma_commit(&b_empty[bs]);
        ++rows_in;
        if (rows_in == p.flush_rows || ai == n_rows - 1) {
          mma_commit(&t_full[buf]);
          ++uses[buf];
          buf ^= 1;
          rows_in = 0;
        }
      }
      // All MMAs issued by this thread must finish before TMEM is released.
      mma_commit(mma_done);
      mbar_wait_bounded(mma_done, 0, 1u << 22);
    }
  } else if (warp < 4) {
    // ------------------------------------------------------------ B builders
    const int bt = threadIdx.x - 64;  // 0..63
    const float* lrow_base = p.left + (long long)l * p.Hl * p.Wl;
    const float mu = p.mu_left[l];
    const int nvec = p.buf_len / 8;
    for (int ai = 0; ai < n_rows; ++ai) {
      const int bs = ai & 1;
      const bool ok = wait_or_abort(&b_empty[bs], ((ai >> 1) & 1) ^ 1, abort_flag, p.flags, 15);
      // the 64 builder threads leave together (they share a named barrier)
      if (bar_red_or(!ok, 1, 64)) break;
      // stage the centred left row (coalesced), then build the phase copies
      float* lr = lrows + bs * kMaxLeftCols;
      const float* src = lrow_base + (long long)(a_lo + ai) * p.Wl;
      for (int x = bt; x < p.Wl; x += 64) lr[x] = __ldg(src + x) - mu;
      asm volatile("bar.sync 1, 64;" ::: "memory");
      __nv_bfloat16* slot = b_bufs + bs * b_slot_elems;
      for (int item = bt; item < kPhases * nvec; item += 64) {
        const int cl = item / nvec, jv = item % nvec;
        const int c = half * kPhases + cl;
        const int j0 = jv * 8 + c - (p.Wr - 1);  // left column of element 0
        __align__(16) __nv_bfloat16 hi[8];
        __align__(16) __nv_bfloat16 lo[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          const int x = j0 + e;
          const float v = (x >= 0 && x < p.Wl) ? lr[x] : 0.0f;
          const __nv_bfloat16 h = __float2bfloat16_rn(v);
          hi[e] = h;
          lo[e] = __float2bfloat16_rn(v - __bfloat162float(h));
        }
        __nv_bfloat16* dst = slot + (cl * 2) * p.buf_len + jv * 8;
        *reinterpret_cast<uint4*>(dst) = *reinterpret_cast<const uint4*>(hi);
        *reinterpret_cast<uint4*>(dst + p.buf_len) = *reinterpret_cast<const uint4*>(lo);
      }
      fence_proxy_async_shared();
      mbar_arrive(&b_full[bs]);
    }
  } else {
    // ------------------------------------------------------------ epilogue
    // warps 4..11: lane quadrant q, B-row half e: phases 0..3, rows n in
    // [e*N/2, (e+1)*N/2) of each.  acc[c * N/2 + n'] is shift
    // sx = half*4 + c + 8 * (e*N/2 + n').
    constexpr int kHalfN = N / 2;
    const int q = warp & 3;
    const int e = (warp - 4) >> 2;
    float acc[kAcc];
#pragma unroll
    for (int i = 0; i < kAcc; ++i) acc[i] = 0.0f;
    bool ok = true;
    for (int d = 0; d < n_drains; ++d) {
      const int b = d & 1;
      if (!wait_or_abort(&t_full[b], (d >> 1) & 1, abort_flag, p.flags, 16)) {
        ok = false;
        break;
      }
      tc_fence_after();
      const uint32_t lane_base = tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * kDCols + e * kHalfN);
#pragma unroll
      for (int c = 0; c < kPhases; ++c) {
#pragma unroll
        for (int j = 0; j + 16 <= kHalfN; j += 16) {
          float v[16];
          tmem_ld16(lane_base + (uint32_t)(c * N + j), v);
          tmem_wait_ld();
#pragma unroll
          for (int i = 0; i < 16; ++i) acc[c * kHalfN + j + i] += v[i];
        }
        if constexpr (kHalfN % 16 != 0) {
          constexpr int j = kHalfN - 8;
          float v[8];
          tmem_ld8(lane_base + (uint32_t)(c * N + j), v);
          tmem_wait_ld();
#pragma unroll
          for (int i = 0; i < 8; ++i) acc[c * kHalfN + j + i] += v[i];
        }
      }
      tc_fence_before();
      mbar_arrive(&t_empty[b]);
    }
    if (ok) {
      // Coalesced reduction into the output: each warp stages 32 rows x 32
      // consecutive owned shifts at a time in shared memory (the right-row
      // stages are idle once the last buffer is drained), then adds row by
      // row, so one warp instruction covers 32 owned shifts of one row.
      fence_proxy_async_shared();
      float* stage = reinterpret_cast<float*>(a_tiles) + (warp - 4) * (32 * 33);
      // output row of this lane's accumulator row m (-1: outside the output)
      long long row_base = -1;
      {
        const int m = q * 32 + lane;
        int pp, dy;
        if (p.mats_mode) {
          pp = m % p.P;
          dy = dy0 + m / p.P;
        } else {
          pp = m / p.DY;
          dy = dy0 + (p.DY - 1) - (m % p.DY);
        }
        const int k = p0 + pp, sy = dy + p.Hr - 1;
        if (k < p.pm.K && sy >= 0 && sy < p.Sy)
          row_base = (((long long)l * p.pm.o_l + (long long)k * p.pm.o_k) * p.Sy + sy) * p.Sx;
      }
#pragma unroll
      for (int h = 0; h < kAcc / 32; ++h) {
        // owned shift index s' = 4 n' + c in [32h, 32h + 32)
#pragma unroll
        for (int i = 0; i < 32; ++i) stage[lane * 33 + i] = acc[(i & 3) * kHalfN + 8 * h + (i >> 2)];
        __syncwarp();
        const int sp = 32 * h + lane;
        const int sx = half * kPhases + (sp & 3) + 8 * (e * kHalfN + (sp >> 2));
        for (int r = 0; r < 32; ++r) {
          const long long rb = __shfl_sync(0xffffffffu, row_base, r);
          if (rb >= 0 && sx < p.Sx) red_add(p.out + rb + sx, stage[r * 33 + lane]);
        }
        __syncwarp();
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(ncols) : "memory");
  }
}

// Mean of every matrix (FP64 sum, FP32 result): one block per matrix.
__global__ void mean_kernel(const float* __restrict__ left, long long left_area, int n_left,
                            const float* __restrict__ right, long long right_area, float* __restrict__ mu) {
  const int m = blockIdx.x;
  const float* src = m < n_left ? left + (long long)m * left_area : right + (long long)(m - n_left) * right_area;
  const long long area = m < n_left ? left_area : right_area;
  double acc = 0.0;
  for (long long i = threadIdx.x; i < area; i += blockDim.x) acc += (double)src[i];
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (threadIdx.x == 0) mu[m] = (float)(acc / (double)area);
  }
}

// 2D prefix sums (FP64) of the centred matrices fl32(x - mu):
// P[y][x] = sum_{i<y, j<x}, (H+1) x (W+1) per matrix.  Pass 1: one warp per
// row scans it (warp shuffles); pass 2: one thread per column accumulates
// down the rows.
__global__ void prefix_rows_kernel(const float* __restrict__ src, int n_mats, int H, int W,
                                   const float* __restrict__ mu, double* __restrict__ P) {
  const long long gw = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;  // (matrix, y) with y in [0, H]
  const int lane = threadIdx.x & 31;
  if (gw >= (long long)n_mats * (H + 1)) return;
  const int m = (int)(gw / (H + 1));
  const int y = (int)(gw % (H + 1));
  double* row = P + ((long long)m * (H + 1) + y) * (W + 1);
  if (y == 0) {
    for (int x = lane; x <= W; x += 32) row[x] = 0.0;
    return;
  }
  const float* a = src + ((long long)m * H + (y - 1)) * W;
  const float mv = mu[m];
  if (lane == 0) row[0] = 0.0;
  double carry = 0.0;
  for (int x0 = 0; x0 < W; x0 += 32) {
    const int x = x0 + lane;
    double v = x < W ? (double)(a[x] - mv) : 0.0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double t = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += t;
    }
    if (x < W) row[x + 1] = carry + v;
    carry += __shfl_sync(0xffffffffu, v, 31);
  }
}

__global__ void prefix_cols_kernel(int n_mats, int H, int W, double* __restrict__ P) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)n_mats * (W + 1)) return;
  const int m = (int)(t / (W + 1));
  const int x = (int)(t % (W + 1));
  double* q = P + (long long)m * (H + 1) * (W + 1) + x;
  double acc = 0.0;
  for (int y = 1; y <= H; ++y) {
    acc += q[(long long)y * (W + 1)];
    q[(long long)y * (W + 1)] = acc;
  }
}

// Splits the centred right matrices fl32(R - mu_R) into BF16 hi/lo planes
// with a padded pitch.
__global__ void split_kernel(const float* __restrict__ src, const float* __restrict__ mu,
                             __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo, long long rows,
                             int rows_per_matrix, int cols, int pitch) {
  const long long total = rows * pitch;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long r = i / pitch;
    const int c = (int)(i % pitch);
    const float v = c < cols ? src[r * cols + c] - mu[r / rows_per_matrix] : 0.0f;
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    hi[i] = h;
    lo[i] = __float2bfloat16_rn(v - __bfloat162float(h));
  }
}

// out[o][sy][sx] = mu_R * S_L' + mu_L * S_R' + mu_L * mu_R * area over the
// overlap of shift (sy, sx); one block per output row.  The row band sums
// Q[x] = P[y1][x] - P[y0][x] of both matrices are formed once per row in
// shared memory (FP64); per element only the two band differences are FP64
// and the products are FP32 (their rounding is ~6e-8 of max|out|).
__global__ void correction_kernel(float* __restrict__ out, const double* __restrict__ PL,
                                  const double* __restrict__ PR, const float* __restrict__ mu_l,
                                  const float* __restrict__ mu_r, int Hl, int Wl, int Hr, int Wr, int Sy, int Sx,
                                  PairMap pm) {
  extern __shared__ double qs[];  // (Wl + 1) + (Wr + 1)
  const long long row = blockIdx.x;  // o * Sy + sy
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
  const double* pl0 = PL + (l * (Hl + 1) + y0) * (long long)(Wl + 1);
  const double* pl1 = PL + (l * (Hl + 1) + y1) * (long long)(Wl + 1);
  const double* pr0 = PR + (r * (Hr + 1) + (y0 - dy)) * (long long)(Wr + 1);
  const double* pr1 = PR + (r * (Hr + 1) + (y1 - dy)) * (long long)(Wr + 1);
  double* ql = qs;
  double* qr = qs + (Wl + 1);
  for (int x = threadIdx.x; x <= Wl; x += blockDim.x) ql[x] = pl1[x] - pl0[x];
  for (int x = threadIdx.x; x <= Wr; x += blockDim.x) qr[x] = pr1[x] - pr0[x];
  __syncthreads();
  const float ml = mu_l[l], mr = mu_r[r];
  const float mlr = ml * mr;
  const float rows = (float)(y1 - y0);
  float* orow = out + row * Sx;
  for (int sx = threadIdx.x; sx < Sx; sx += blockDim.x) {
    const int dx = sx - (Wr - 1);
    const int x0 = max(0, dx), x1 = min(Wl, Wr + dx);
    const float sl = (float)(ql[x1] - ql[x0]);
    const float sr = (float)(qr[x1 - dx] - qr[x0 - dx]);
    orow[sx] = fmaf(mr, sl, fmaf(ml, sr, mlr * (rows * (float)(x1 - x0))));
  }
}

struct TcPlan {
  int P, DY, mats_mode, N, nkc, buf_len, pitch;
  int smem_bytes;
};

bool tc_plan(const Geometry& g, const PairMap& pm, TcPlan* t) {
  if (g.Sx > 512 || g.Wr > 256) return false;  // 8 phases x N <= 512 TMEM columns
  int P = 1;
  while (P < 128 && P < pm.K) P *= 2;
  t->P = P;
  t->DY = 128 / P;
  t->mats_mode = P >= 8 ? 1 : 0;
  int N = (g.Sx + 7) / 8;
  N = (N + 15) / 16 * 16;
  if (N < 16) N = 16;
  t->N = N;
  t->nkc = (g.Wr + 63) / 64;
  t->buf_len = t->nkc * 64 + 8 * N;
  t->pitch = (g.Wr + 7) / 8 * 8;
  t->smem_bytes = 1024 + kStages * kStageBytes + 2 * 4 * 2 * t->buf_len * 2 + 2 * kMaxLeftCols * 4 + kBarBytes;
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
  static int v = env_int("XC_TC_CHUNK_ROWS", 32);
  return v;
}

// Workspace layout (each part 256-byte aligned).
struct TcWs {
  float* mu;        // n_left + n_right means
  double* PL;       // n_left x (Hl+1)(Wl+1)
  double* PR;       // n_right x (Hr+1)(Wr+1)
  __nv_bfloat16* hi;  // n_right x Hr x pitch
  __nv_bfloat16* lo;
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
  w.PL = reinterpret_cast<double*>(take(sizeof(double) * (size_t)pm.n_left * (g.Hl + 1) * (g.Wl + 1)));
  w.PR = reinterpret_cast<double*>(take(sizeof(double) * (size_t)nr * (g.Hr + 1) * (g.Wr + 1)));
  w.hi = reinterpret_cast<__nv_bfloat16*>(take(sizeof(__nv_bfloat16) * plane));
  w.lo = reinterpret_cast<__nv_bfloat16*>(take(sizeof(__nv_bfloat16) * plane));
  w.bytes = off + 256;
  return w;
}

}  // namespace

size_t tc_workspace_size(const Geometry& g, const PairMap& pm) {
  TcPlan t;
  if (!tc_plan(g, pm, &t)) return 0;
  return ws_layout(nullptr, g, pm, t).bytes;
}

xc_status tc_correlate(const float* left, const float* right, float* out, const Geometry& g, const PairMap& pm,
                       void* workspace, size_t ws_bytes, cudaStream_t stream) {
  TcPlan t;
  if (!tc_plan(g, pm, &t))
    return fail(XC_ERR_UNSUPPORTED,
                "split-BF16 tensor path supports outputs up to 512 columns and right widths up to 256");
  const size_t need = ws_layout(nullptr, g, pm, t).bytes;
  if (workspace == nullptr || ws_bytes < need)
    return fail(XC_ERR_WORKSPACE, "split-BF16 path needs " + std::to_string(need) + " bytes of workspace");
  const TcWs w = ws_layout(reinterpret_cast<void*>(((uintptr_t)workspace + 255) & ~uintptr_t(255)), g, pm, t);
  const long long nr = n_right_of(pm);
  const int nl = pm.n_left;
  const uint64_t n_out = (uint64_t)((long long)(nl - 1) * pm.o_l + (long long)(pm.K - 1) * pm.o_k + 1);

  // 1. per-matrix means, 2. FP64 prefix sums of the centred matrices
  mean_kernel<<<(unsigned)(nl + nr), 256, 0, stream>>>(left, (long long)g.Hl * g.Wl, nl, right,
                                                         (long long)g.Hr * g.Wr, w.mu);
  XC_CUDA_TRY(cudaGetLastError());
  {
    auto prefix = [&](const float* src, int n, int H, int W, const float* mu, double* P) -> xc_status {
      const long long warps = (long long)n * (H + 1);
      prefix_rows_kernel<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, stream>>>(src, n, H, W, mu, P);
      XC_CUDA_TRY(cudaGetLastError());
      const long long cols = (long long)n * (W + 1);
      prefix_cols_kernel<<<(unsigned)((cols + 255) / 256), 256, 0, stream>>>(n, H, W, P);
      XC_CUDA_TRY(cudaGetLastError());
      return XC_OK;
    };
    XC_TRY(prefix(left, nl, g.Hl, g.Wl, w.mu, w.PL));
    XC_TRY(prefix(right, (int)nr, g.Hr, g.Wr, w.mu + nl, w.PR));
  }
  // 3. split of the centred right matrices
  {
    const long long rows = nr * g.Hr;
    long long blocks = (rows * t.pitch + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    split_kernel<<<(unsigned)blocks, 256, 0, stream>>>(right, w.mu + nl, w.hi, w.lo, rows, g.Hr, g.Wr, t.pitch);
    XC_CUDA_TRY(cudaGetLastError());
  }
  // 4. the mean terms initialise the output
  correction_kernel<<<(unsigned)(n_out * g.Sy), 256, sizeof(double) * (g.Wl + g.Wr + 2), stream>>>(
      out, w.PL, w.PR, w.mu, w.mu + nl, g.Hl, g.Wl, g.Hr, g.Wr, g.Sy, g.Sx, pm);
  XC_CUDA_TRY(cudaGetLastError());

  CUtensorMap mhi, mlo;
  {
    const uint64_t es = 2, mat = (uint64_t)t.pitch * g.Hr * es;
    const uint64_t d2 = pm.r_l != 0 ? (uint64_t)pm.n_left : 1;
    uint64_t dims[4] = {(uint64_t)t.pitch, (uint64_t)g.Hr, d2, (uint64_t)pm.K};
    uint64_t strides[3] = {(uint64_t)t.pitch * es, mat * (uint64_t)(pm.r_l != 0 ? pm.r_l : 1), mat * (uint64_t)pm.r_k};
    uint32_t box[4];
    if (t.mats_mode) {
      box[0] = 64; box[1] = 1; box[2] = 1; box[3] = (uint32_t)t.P;
    } else {
      box[0] = 64; box[1] = (uint32_t)t.DY; box[2] = 1; box[3] = 1;
    }
    if (!encode_tiled(&mhi, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, w.hi, dims, strides, box, CU_TENSOR_MAP_SWIZZLE_128B))
      return XC_ERR_INVALID_ARGUMENT;
    if (!encode_tiled(&mlo, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, w.lo, dims, strides, box, CU_TENSOR_MAP_SWIZZLE_128B))
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
  prm.N = t.N;
  prm.nkc = t.nkc;
  prm.buf_len = t.buf_len;
  prm.flush_rows = flush_rows(t.nkc);
  prm.chunk_rows = chunk_rows();
  prm.n_chunks = div_up(t.DY - 1 + std::min(g.Hl, g.Hr), prm.chunk_rows);
  prm.flags = device_flags();

  const long long blocks = 2LL * prm.n_chunks * prm.n_dytiles * pm.n_left * prm.n_pgroups;
  if (blocks > 0x7fffffffLL) return fail(XC_ERR_INVALID_ARGUMENT, "problem too large for one launch");
  auto launch = [&](auto kern) -> xc_status {
    XC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, t.smem_bytes));
    const int slot = kernel_timer_begin(stream);
    kern<<<(unsigned)blocks, kThreads, t.smem_bytes, stream>>>(mhi, mlo, prm);
    kernel_timer_end(slot, stream);
    XC_CUDA_TRY(cudaGetLastError());
    return XC_OK;
  };
  switch (t.N) {
    case 16: return launch(tc_kernel<16>);
    case 32: return launch(tc_kernel<32>);
    case 48: return launch(tc_kernel<48>);
    default: return launch(tc_kernel<64>);
  }
}

// ---------------------------------------------------------------------------
// Allocation-free variant of the split-BF16 path.
//
// Some callers cannot call cudaMalloc: hosts that hand a library a fixed
// device-memory budget or their own pool (and forbid raw allocations), and
// latency-critical loops where cudaMalloc/cudaFree may stall or synchronise
// the device.  xc_correlate_tc_noalloc serves them with the scratch of this
// path (means, FP64 prefix sums, BF16 planes) in the file-scope array below,
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
  if (!tc_plan(g, pm, &t))
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
                      reinterpret_cast<cudaStream_t>(stream));
}
