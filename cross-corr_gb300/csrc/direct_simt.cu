// direct_simt.cu -- plain definition-based full 2D cross-correlation on the
// FP32/FP64 FMA pipes of GB300 (sm_103a).
//
// Replaces the reference's warp-shuffle kernel family (src/naive_shuffle*.cu,
// e.g. ccn_shuffle src/naive_shuffle.cu:86-267 and the best one_to_many kernel
// src/naive_shuffle_one_to_many_multirow_both_multimat_right.cu:91-535).
// Same result and shift order, different design:
//
//  * A CTA owns an output tile of BSY x BSX shifts for G right matrices that
//    share one left matrix (the reference's "multimat right" reuse).
//  * Work is streamed in stages (x-chunk of XC right columns) x (one right row
//    y).  Each stage's left window (BSY rows x XC+BSX columns) and right rows
//    (G matrices x XC columns) are staged in shared memory by TMA
//    (cp.async.bulk.tensor), whose out-of-bounds zero fill replaces every
//    bounds check of the reference (src/bound_checked_loads.cuh:22-39).  Row
//    pitches TMA cannot describe (not a multiple of 16 bytes) fall back to
//    cp.async with zero fill.
//  * Each thread accumulates TSY x TSX shifts x TG matrices in registers.  The
//    left values of its TSX consecutive shifts form a sliding window carried
//    in registers across x steps; every 4 columns it loads one new 128-bit
//    vector per left row and one broadcast 128-bit vector per right matrix,
//    so an x step issues TSY*TSX*TG*4 FMAs per (TSY+TG) vector loads.  The
//    register carry replaces the reference's per-FMA shuffle rotation
//    (src/naive_shuffle.cu:134-148), which made it shuffle-issue bound.
//  * FP32 partial sums are flushed into the output every FLUSH_STAGES stages
//    (store first, then add), so no FP32 accumulation chain exceeds
//    FLUSH_STAGES*XC products: serial FP32 sums over 256x256 overlaps would
//    otherwise drift past 1e-5 of max|out|.
//  * Bounded mbarrier waits: a wait that expires records a flag and the whole
//    CTA returns (no trap, no hang).
#include <algorithm>

#include "xc_common.cuh"
#include "xc_internal.h"

namespace xc {

namespace {

template <typename T>
struct V4 {
  T v[4];
};

template <typename T>
__device__ __forceinline__ V4<T> lds4(const T* p);

template <>
__device__ __forceinline__ V4<float> lds4<float>(const float* p) {
  float4 a = *reinterpret_cast<const float4*>(p);
  return V4<float>{{a.x, a.y, a.z, a.w}};
}

template <>
__device__ __forceinline__ V4<double> lds4<double>(const double* p) {
  double2 a = reinterpret_cast<const double2*>(p)[0];
  double2 b = reinterpret_cast<const double2*>(p)[1];
  return V4<double>{{a.x, a.y, b.x, b.y}};
}

template <typename T>
struct DirectParams {
  const T* left;
  const T* right;
  T* out;
  int Hl, Wl, Hr, Wr, Sy, Sx;
  PairMap pm;
  int tiles_sx, tiles_sy, kgroups;
  int sx_origin;  // first tile's sx (<= 0) so that every tile's left x origin is 16-byte aligned
  DeviceFlags* flags;
};

// Tile configuration.
//  lanes: 4 (sy) x 8 (sx) per warp; warps: WY x WX x WG per CTA.
template <typename T, int TSY_, int TSX_, int TG_, int WY_, int WX_, int WG_, int XC_, int STAGES_, int MINB_>
struct Cfg {
  using type = T;
  static constexpr int TSY = TSY_, TSX = TSX_, TG = TG_, WY = WY_, WX = WX_, WG = WG_;
  static constexpr int XC = XC_, STAGES = STAGES_, MINB = MINB_;
  static constexpr int LANES_Y = 4, LANES_X = 8;
  static constexpr int NWARPS = WY * WX * WG;
  static constexpr int NT = NWARPS * 32;
  static constexpr int WSY = LANES_Y * TSY;  // sy rows per warp
  static constexpr int WSX = LANES_X * TSX;  // sx columns per warp
  static constexpr int BSY = WY * WSY;
  static constexpr int BSX = WX * WSX;
  static constexpr int G = WG * TG;
  static constexpr int LW = XC + BSX;  // left window width (elements)
  static constexpr int VEC = 16 / (int)sizeof(T);
  static constexpr int L_ELEMS = BSY * LW;
  static constexpr int R_ELEMS = G * XC;
  static constexpr int STAGE_BYTES = ((L_ELEMS + R_ELEMS) * (int)sizeof(T) + 127) / 128 * 128;
  static constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 128;
  // FP32 chains are capped at 4096 products per flush; FP64 needs no flush.
  static constexpr int FLUSH_STAGES = sizeof(T) == 4 ? (4096 / XC) : (1 << 30);
  static_assert(TSX % 4 == 0, "TSX must be a multiple of 4");
  static_assert(LW <= 256 && BSY <= 256 && XC <= 256 && G <= 256, "TMA box dimensions are limited to 256");
  static_assert((LW * (int)sizeof(T)) % 16 == 0 && (XC * (int)sizeof(T)) % 16 == 0, "TMA inner box must be 16B");
};

template <typename C>
__global__ void __launch_bounds__(C::NT, C::MINB)
    direct_kernel(const __grid_constant__ CUtensorMap lmap, const __grid_constant__ CUtensorMap rmap,
                  const DirectParams<typename C::type> p, const bool use_tma) {
  using T = typename C::type;
  constexpr int TSY = C::TSY, TSX = C::TSX, TG = C::TG, XC = C::XC, S = C::STAGES;
  constexpr int BSY = C::BSY, BSX = C::BSX, G = C::G, LW = C::LW;

  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + S * C::STAGE_BYTES);

  // ---- decode the CTA's tile --------------------------------------------
  const int nlk = p.pm.n_left * p.kgroups;
  int bid = blockIdx.x;
  const int lk = bid % nlk;
  bid /= nlk;
  const int tx = bid % p.tiles_sx;
  const int ty = bid / p.tiles_sx;
  const int l = lk / p.kgroups;
  const int k0 = (lk % p.kgroups) * G;
  const int SY0 = ty * BSY;
  const int SX0 = p.sx_origin + tx * BSX;

  // Right rows / columns that meet any shift of the tile.
  const int y_lo = max(0, p.Hr - 1 - (SY0 + BSY - 1));
  const int y_hi = min(p.Hr, p.Hl + p.Hr - 1 - SY0);
  const int x_lo = max(0, p.Wr - 1 - (SX0 + BSX - 1)) & ~(C::VEC - 1);
  const int x_hi = min(p.Wr, p.Wl + p.Wr - 1 - SX0);
  if (y_lo >= y_hi || x_lo >= x_hi) return;  // uniform over the CTA
  const int ny = y_hi - y_lo;
  const int nxc = (x_hi - x_lo + XC - 1) / XC;
  const int nst = ny * nxc;

  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int wg = warp % C::WG;
  const int wx = (warp / C::WG) % C::WX;
  const int wy = warp / (C::WG * C::WX);
  const int lyy = lane >> 3, lxx = lane & 7;
  const int row0 = wy * C::WSY + lyy * TSY;  // first local sy row of this thread
  const int col0 = wx * C::WSX + lxx * TSX;  // first local sx column of this thread
  const int wsy0 = SY0 + wy * C::WSY, wsx0 = SX0 + wx * C::WSX;

  const int rdim2 = p.pm.r_l != 0 ? l : 0;

  if (use_tma && tid == 0) {
    prefetch_tensormap(&lmap);
    prefetch_tensormap(&rmap);
    for (int s = 0; s < S; ++s) mbar_init(&bars[s], 1);
    fence_mbar_init();
  }
  __syncthreads();

  auto stage_ptrL = [&](int slot) { return reinterpret_cast<T*>(smem + slot * C::STAGE_BYTES); };
  auto stage_ptrR = [&](int slot) { return reinterpret_cast<T*>(smem + slot * C::STAGE_BYTES) + C::L_ELEMS; };

  // Issue the loads of stage j into its slot.
  auto issue = [&](int j) {
    if (j >= nst) {
      if (!use_tma) cp_async_commit();
      return;
    }
    const int slot = j % S;
    const int xc_start = x_lo + (j / ny) * XC;
    const int y = y_lo + (j % ny);
    const int lx0 = xc_start + SX0 - (p.Wr - 1);
    const int ly0 = y + SY0 - (p.Hr - 1);
    T* sL = stage_ptrL(slot);
    T* sR = stage_ptrR(slot);
    if (use_tma) {
      if (tid == 0) {
        mbar_arrive_expect_tx(&bars[slot], (uint32_t)((C::L_ELEMS + C::R_ELEMS) * sizeof(T)));
        tma_load_3d(sL, &lmap, &bars[slot], lx0, ly0, l);
        tma_load_4d(sR, &rmap, &bars[slot], xc_start, y, rdim2, k0);
      }
    } else {
      const T* Lm = p.left + (long long)l * p.Hl * p.Wl;
      for (int e = tid; e < C::L_ELEMS; e += C::NT) {
        const int r = e / LW, c = e % LW;
        const int gy = ly0 + r, gx = lx0 + c;
        const bool ok = gy >= 0 && gy < p.Hl && gx >= 0 && gx < p.Wl;
        cp_async_zfill<sizeof(T)>(sL + e, ok ? Lm + (long long)gy * p.Wl + gx : p.left, ok);
      }
      for (int e = tid; e < C::R_ELEMS; e += C::NT) {
        const int g = e / XC, c = e % XC;
        const int k = k0 + g, gx = xc_start + c;
        const bool ok = k < p.pm.K && gx < p.Wr;
        const long long r = ok ? (long long)l * p.pm.r_l + (long long)k * p.pm.r_k : 0;
        cp_async_zfill<sizeof(T)>(sR + e, ok ? p.right + (r * p.Hr + y) * p.Wr + gx : p.right, ok);
      }
      cp_async_commit();
    }
  };

  T acc[TSY][TSX][TG];
#pragma unroll
  for (int t = 0; t < TSY; ++t)
#pragma unroll
    for (int j = 0; j < TSX; ++j)
#pragma unroll
      for (int i = 0; i < TG; ++i) acc[t][j][i] = T(0);
  bool flushed = false;

  // The empty asm keeps the compiler from hoisting the 4*TSY*TSX*TG output
  // addresses out of the stage loop (they would pin ~100 registers).
  auto flush = [&]() {
    int sy_base = SY0 + row0, sx_base = SX0 + col0, kb = k0 + wg * TG;
    asm volatile("" : "+r"(sy_base), "+r"(sx_base), "+r"(kb));
#pragma unroll
    for (int i = 0; i < TG; ++i) {
      const int k = kb + i;
      if (k >= p.pm.K) continue;
      T* o = p.out + ((long long)l * p.pm.o_l + (long long)k * p.pm.o_k) * p.Sy * p.Sx;
#pragma unroll
      for (int t = 0; t < TSY; ++t) {
        const int sy = sy_base + t;
        if (sy >= p.Sy) continue;
#pragma unroll
        for (int j = 0; j < TSX; ++j) {
          const int sx = sx_base + j;
          if (sx < 0 || sx >= p.Sx) continue;
          T* dst = o + (long long)sy * p.Sx + sx;
          *dst = flushed ? *dst + acc[t][j][i] : acc[t][j][i];
          acc[t][j][i] = T(0);
        }
      }
    }
    flushed = true;
  };

  for (int s = 0; s < S - 1; ++s) issue(s);

  for (int j = 0; j < nst; ++j) {
    issue(j + S - 1);
    const int slot = j % S;
    if (use_tma) {
      const bool ok = mbar_wait_bounded(&bars[slot], (uint32_t)((j / S) & 1));
      if (__syncthreads_or(!ok)) {
        if (tid == 0) {
          record_timeout(p.flags, 1);
          // Give copies still in flight a bounded chance to land before exit.
          for (int q = j; q < min(nst, j + S); ++q) mbar_wait_bounded(&bars[q % S], (uint32_t)((q / S) & 1), 1u << 16);
        }
        return;
      }
    } else {
      cp_async_wait<S - 1>();
      __syncthreads();
    }

    const int xc_start = x_lo + (j / ny) * XC;
    const int y = y_lo + (j % ny);
    // Does this warp's 16-row band of shifts meet right row y?
    const bool y_ok = (y >= p.Hr - 1 - (wsy0 + C::WSY - 1)) && (y < p.Hl + p.Hr - 1 - wsy0);
    // Columns of this chunk that meet the warp's shifts, in 4-column steps.
    int xs = max(0, p.Wr - 1 - (wsx0 + C::WSX - 1)) - xc_start;
    int xe = min(p.Wr, p.Wl + p.Wr - 1 - wsx0) - xc_start;
    xs = max(xs, 0) & ~3;
    xe = min(xe, XC);
    if (y_ok && xs < xe) {
      const T* sL = stage_ptrL(slot) + row0 * LW + col0;
      const T* sR = stage_ptrR(slot) + (wg * TG) * XC;
      T cur[TSY][TSX];
#pragma unroll
      for (int t = 0; t < TSY; ++t) {
#pragma unroll
        for (int q = 0; q < TSX / 4; ++q) {
          V4<T> v = lds4<T>(sL + t * LW + xs + 4 * q);
          cur[t][4 * q + 0] = v.v[0];
          cur[t][4 * q + 1] = v.v[1];
          cur[t][4 * q + 2] = v.v[2];
          cur[t][4 * q + 3] = v.v[3];
        }
      }
#pragma unroll 1
      for (int xo = xs; xo < xe; xo += 4) {
        V4<T> rv[TG];
#pragma unroll
        for (int i = 0; i < TG; ++i) rv[i] = lds4<T>(sR + i * XC + xo);
#pragma unroll
        for (int t = 0; t < TSY; ++t) {
          const V4<T> nw = lds4<T>(sL + t * LW + xo + TSX);
          T win[TSX + 4];
#pragma unroll
          for (int q = 0; q < TSX; ++q) win[q] = cur[t][q];
#pragma unroll
          for (int q = 0; q < 4; ++q) win[TSX + q] = nw.v[q];
#pragma unroll
          for (int xx = 0; xx < 4; ++xx)
#pragma unroll
            for (int jj = 0; jj < TSX; ++jj)
#pragma unroll
              for (int i = 0; i < TG; ++i) acc[t][jj][i] = fma(win[xx + jj], rv[i].v[xx], acc[t][jj][i]);
#pragma unroll
          for (int q = 0; q < TSX; ++q) cur[t][q] = win[q + 4];
        }
      }
    }
    if ((j + 1) % C::FLUSH_STAGES == 0) flush();
    __syncthreads();
  }
  flush();
}

using CfgF32Multi = Cfg<float, 4, 4, 4, 2, 2, 2, 128, 3, 2>;   // 32 sy x 64 sx x 8 mats, 256 threads
using CfgF32Single = Cfg<float, 4, 8, 1, 4, 1, 1, 128, 2, 2>;  // 64 sy x 64 sx x 1 mat, 128 threads
using CfgF64Multi = Cfg<double, 4, 4, 2, 2, 2, 2, 64, 3, 1>;   // 32 x 64 x 4 mats
using CfgF64Single = Cfg<double, 4, 4, 1, 2, 2, 1, 64, 3, 2>;  // 32 x 64 x 1 mat

template <typename C>
xc_status launch_cfg(const typename C::type* left, const typename C::type* right, typename C::type* out,
                     const Geometry& g, const PairMap& pm, cudaStream_t stream, int force_loader) {
  using T = typename C::type;
  DirectParams<T> p;
  p.left = left;
  p.right = right;
  p.out = out;
  p.Hl = g.Hl;
  p.Wl = g.Wl;
  p.Hr = g.Hr;
  p.Wr = g.Wr;
  p.Sy = g.Sy;
  p.Sx = g.Sx;
  p.pm = pm;
  const int rem = (g.Wr - 1) % C::VEC;
  p.sx_origin = rem == 0 ? 0 : rem - C::VEC;
  p.tiles_sx = div_up(g.Sx - p.sx_origin, C::BSX);
  p.tiles_sy = div_up(g.Sy, C::BSY);
  p.kgroups = div_up(pm.K, C::G);
  p.flags = device_flags();

  const long long blocks = (long long)p.tiles_sx * p.tiles_sy * pm.n_left * p.kgroups;
  if (blocks <= 0) return XC_OK;
  if (blocks > 0x7fffffffLL) return fail(XC_ERR_INVALID_ARGUMENT, "problem too large for one launch");

  // TMA needs 16-byte aligned bases and row/matrix pitches.
  const size_t es = sizeof(T);
  bool tma_ok = ((uintptr_t)left % 16 == 0) && ((uintptr_t)right % 16 == 0) && ((size_t)g.Wl * es % 16 == 0) &&
                ((size_t)g.Wr * es % 16 == 0);
  bool use_tma = force_loader < 0 ? tma_ok : (force_loader == 1);
  if (use_tma && !tma_ok) return fail(XC_ERR_INVALID_ARGUMENT, "TMA loader requested for unaligned pitches");

  CUtensorMap lmap, rmap;
  memset(&lmap, 0, sizeof(lmap));
  memset(&rmap, 0, sizeof(rmap));
  if (use_tma) {
    const CUtensorMapDataType dt = sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
    {
      uint64_t dims[3] = {(uint64_t)g.Wl, (uint64_t)g.Hl, (uint64_t)pm.n_left};
      uint64_t strides[2] = {(uint64_t)g.Wl * es, (uint64_t)g.Wl * g.Hl * es};
      uint32_t box[3] = {(uint32_t)C::LW, (uint32_t)C::BSY, 1};
      if (!encode_tiled(&lmap, dt, 3, left, dims, strides, box, CU_TENSOR_MAP_SWIZZLE_NONE))
        return XC_ERR_INVALID_ARGUMENT;
    }
    {
      const uint64_t mat = (uint64_t)g.Wr * g.Hr * es;
      uint64_t d2 = pm.r_l != 0 ? (uint64_t)pm.n_left : 1;
      uint64_t dims[4] = {(uint64_t)g.Wr, (uint64_t)g.Hr, d2, (uint64_t)pm.K};
      uint64_t strides[3] = {(uint64_t)g.Wr * es, mat * (uint64_t)(pm.r_l != 0 ? pm.r_l : 1),
                             mat * (uint64_t)pm.r_k};
      uint32_t box[4] = {(uint32_t)C::XC, 1, 1, (uint32_t)C::G};
      if (!encode_tiled(&rmap, dt, 4, right, dims, strides, box, CU_TENSOR_MAP_SWIZZLE_NONE))
        return XC_ERR_INVALID_ARGUMENT;
    }
  }

  static_assert(C::SMEM_BYTES <= 227 * 1024, "shared memory budget");
  auto kern = direct_kernel<C>;
  XC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM_BYTES));
  kern<<<(unsigned)blocks, C::NT, C::SMEM_BYTES, stream>>>(lmap, rmap, p, use_tma);
  XC_CUDA_TRY(cudaGetLastError());
  return XC_OK;
}

}  // namespace

xc_status direct_launch(xc_dtype dtype, const void* left, const void* right, void* out, const Geometry& g,
                        const PairMap& pm, cudaStream_t stream, int force_loader) {
  if (dtype == XC_F32) {
    if (pm.K >= 4)
      return launch_cfg<CfgF32Multi>((const float*)left, (const float*)right, (float*)out, g, pm, stream,
                                     force_loader);
    return launch_cfg<CfgF32Single>((const float*)left, (const float*)right, (float*)out, g, pm, stream,
                                    force_loader);
  }
  if (pm.K >= 3)
    return launch_cfg<CfgF64Multi>((const double*)left, (const double*)right, (double*)out, g, pm, stream,
                                   force_loader);
  return launch_cfg<CfgF64Single>((const double*)left, (const double*)right, (double*)out, g, pm, stream,
                                  force_loader);
}

}  // namespace xc
