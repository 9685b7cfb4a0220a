// direct_simt.cu -- plain definition-based full 2D cross-correlation on the
// FP32/FP64 FMA pipes of GB300 (sm_103a), for uniform batches (the four
// modes) and for ragged batches of pairs of any sizes.
//
// Replaces the reference's warp-shuffle kernel family (src/naive_shuffle*.cu,
// e.g. ccn_shuffle src/naive_shuffle.cu:86-267 and the best one_to_many kernel
// src/naive_shuffle_one_to_many_multirow_both_multimat_right.cu:91-535).
// Same result and shift order, different design:
//
//  * Work is cut into tiles: BSY x BSX shifts for up to G right matrices that
//    share one left matrix (the reference's "multimat right" reuse).  A tile
//    is streamed in stages of (XC right columns) x (one right row y); a
//    stage's left window (BSY rows x XC+BSX columns) and right rows (G x XC)
//    land in shared memory by TMA (cp.async.bulk.tensor).  TMA's zero fill
//    of out-of-bounds elements replaces every bounds check of the reference
//    (src/bound_checked_loads.cuh:22-39).  Row pitches TMA cannot describe
//    (not a multiple of 16 bytes) are loaded with cp.async + zero fill.
//  * One producer warp issues the loads into a ring of STAGES slots; the
//    consumer warps wait on per-slot "full" mbarriers and release slots with
//    per-slot "empty" mbarriers, so no CTA-wide barrier is taken per stage.
//    The producer also publishes each stage's tile geometry in shared memory,
//    which lets the same kernel run persistently over a queue of tiles.
//  * Each consumer thread accumulates TSY x TSX shifts x TG matrices in
//    registers.  The left values of its TSX consecutive shifts form a sliding
//    window held in three 4-element register buffers that rotate through a
//    3x unrolled column loop (no register moves); every 4 columns it loads
//    one 128-bit vector per left row and one broadcast vector per right
//    matrix.  This replaces the reference's per-FMA shuffle rotation
//    (src/naive_shuffle.cu:134-148), which made it shuffle-issue bound.
//  * FP32 partial sums are flushed into the output every FLUSH_STAGES stages
//    (store first, then add), so no FP32 accumulation chain exceeds
//    FLUSH_STAGES*XC products: serial FP32 sums over 256x256 overlaps would
//    otherwise drift past 1e-5 of max|out|.
//  * Row split (the reference's work distribution, src/naive_shuffle.cu:306-413
//    with src/row_distribution.cuh:34-284): when a launch's tiles would not
//    fill one wave of CTAs, each tile's right-row range is cut into slices of
//    `rows_per_slice` rows, one CTA per slice, and every flush adds into the
//    output with red.global.add (the output is zeroed first, or by the
//    caller for the work-distribution launchers, as in the reference).  The
//    reference splits the rows of one shift over warps; here a slice holds
//    the rows of a whole tile of shifts, so the left window and right rows a
//    stage stages in shared memory still serve all of the tile's shifts.
//  * Bounded mbarrier waits: an expired wait records a flag and the CTA
//    winds down (no trap, no hang).
#include <algorithm>
#include <cstdlib>
#include <cstring>

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

// Geometry of one tile as the producer publishes it with every stage.
struct TileInfo {
  int Hl, Wl, Hr, Wr, Sy, Sx;
  int SY0, SX0;
  int nmat;              // right matrices of the tile that exist (<= G)
  int lc;                // left TMA coordinate (matrix index within its map)
  int rc2, rc3;          // right TMA coordinates of dims 2 and 3
  long long out0;        // element offset of the first matrix's output
  long long ostride;     // element offset between consecutive matrices' outputs
  long long lsrc;        // element offset of the left matrix (cp.async loader)
  long long rsrc0;       // element offset of the first right matrix (cp.async loader)
  long long rstride;     // element offset between the tile's right matrices (cp.async loader)
  const void* lmap;      // tensor maps (TMA loader)
  const void* rmap;
};

struct StageMeta {
  TileInfo ti;
  int y, xc_start;
  int first, last, end;
};

// Uniform batches: the four modes over equal-size matrices.
template <typename T>
struct Uniform {
  int Hl, Wl, Hr, Wr, Sy, Sx;
  PairMap pm;
  int tiles_sx, tiles_sy, kgroups;
  int sx_origin;  // first tile's sx (<= 0) so that every tile's left x origin is 16-byte aligned
  int n_slices;        // CTAs per tile, each taking `rows_per_slice` of the tile's right rows
  int rows_per_slice;
  int accumulate;      // 1: every flush adds into the output (red.global.add), which starts zeroed
};

// Ragged batches: one tile queue over pairs of arbitrary sizes.
struct RaggedView {
  const RaggedTile* tiles;
  const RaggedPairDev* pairs;
  const CUtensorMap* lmaps;  // per left matrix (padded copies)
  const CUtensorMap* rmaps;  // per right matrix
  unsigned int* queue;       // next tile to hand out
  int n_tiles;
};

template <typename T>
struct DirectArgs {
  const T* left;
  const T* right;
  T* out;
  Uniform<T> u;
  RaggedView rg;  // rg.tiles == nullptr for uniform batches
  DeviceFlags* flags;
};

// Tile configuration.
//  lanes: 4 (sy) x 8 (sx) per warp; consumer warps: WY x WX x WG; one producer warp.
template <typename T, int TSY_, int TG_, int WY_, int WX_, int WG_, int XC_, int STAGES_, int MINB_>
struct Cfg {
  using type = T;
  static constexpr int TSY = TSY_, TSX = 8, TG = TG_, WY = WY_, WX = WX_, WG = WG_;
  static constexpr int XC = XC_, STAGES = STAGES_, MINB = MINB_;
  static constexpr int LANES_Y = 4, LANES_X = 8;
  static constexpr int NW = WY * WX * WG;  // consumer warps
  static constexpr int NT = (NW + 1) * 32;
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
  static constexpr int META_BYTES = (STAGES * (int)sizeof(StageMeta) + 127) / 128 * 128;
  static constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + META_BYTES + 2 * STAGES * 8 + 128;
  // FP32 chains are capped at 4096 products per flush; FP64 needs no flush.
  static constexpr int FLUSH_STAGES = sizeof(T) == 4 ? (4096 / XC) : (1 << 30);
  static_assert(LW <= 256 && BSY <= 256 && XC <= 256 && G <= 256, "TMA box dimensions are limited to 256");
  static_assert((LW * (int)sizeof(T)) % 16 == 0 && (XC * (int)sizeof(T)) % 16 == 0, "TMA inner box must be 16B");
  static_assert(XC % 4 == 0, "column chunks are walked 4 at a time");
};

// Stage count and column range of a tile.
struct TileSpan {
  int y_lo, ny, x_lo, nxc;
};

template <typename C>
__device__ __forceinline__ TileSpan tile_span(const TileInfo& ti) {
  TileSpan s;
  s.y_lo = max(0, ti.Hr - 1 - (ti.SY0 + C::BSY - 1));
  const int y_hi = min(ti.Hr, ti.Hl + ti.Hr - 1 - ti.SY0);
  s.x_lo = max(0, ti.Wr - 1 - (ti.SX0 + C::BSX - 1)) & ~(C::VEC - 1);
  const int x_hi = min(ti.Wr, ti.Wl + ti.Wr - 1 - ti.SX0);
  s.ny = max(0, y_hi - s.y_lo);
  s.nxc = x_hi > s.x_lo ? (x_hi - s.x_lo + C::XC - 1) / C::XC : 0;
  return s;
}

template <typename C>
__global__ void __launch_bounds__(C::NT, C::MINB)
    direct_kernel(const __grid_constant__ CUtensorMap lmap_u, const __grid_constant__ CUtensorMap rmap_u,
                  const DirectArgs<typename C::type> p, const bool use_tma) {
  using T = typename C::type;
  constexpr int TSY = C::TSY, TSX = C::TSX, TG = C::TG, XC = C::XC, S = C::STAGES;
  constexpr int BSY = C::BSY, BSX = C::BSX, G = C::G, LW = C::LW;

  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  StageMeta* meta = reinterpret_cast<StageMeta*>(smem + S * C::STAGE_BYTES);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + S * C::STAGE_BYTES + C::META_BYTES);
  uint64_t* empty = full + S;

  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const bool ragged = p.rg.tiles != nullptr;

  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      // TMA: the producer's arrive.expect_tx; cp.async: one asynchronous
      // arrival per producer lane plus lane 0's release arrival after it
      // wrote the stage's metadata
      mbar_init(&full[s], use_tma ? 1 : 33);
      mbar_init(&empty[s], C::NW);
    }
    fence_mbar_init();
    if (use_tma && !ragged) {
      prefetch_tensormap(&lmap_u);
      prefetch_tensormap(&rmap_u);
    }
  }
  __syncthreads();

  auto stage_L = [&](int slot) { return reinterpret_cast<T*>(smem + slot * C::STAGE_BYTES); };
  auto stage_R = [&](int slot) { return reinterpret_cast<T*>(smem + slot * C::STAGE_BYTES) + C::L_ELEMS; };

  if (warp == C::NW) {
    // ================================================================ producer
    int j = 0;
    bool ok = true;
    for (int iter = 0; ok; ++iter) {
      TileInfo ti;
      int slice = 0;
      if (!ragged) {
        if (iter > 0) break;
        const Uniform<T>& u = p.u;
        const int nlk = u.pm.n_left * u.kgroups;
        int bid = blockIdx.x;
        slice = bid % u.n_slices;  // the slices of a tile are neighbouring CTAs
        bid /= u.n_slices;
        const int lk = bid % nlk;
        bid /= nlk;
        const int tx = bid % u.tiles_sx;
        const int ty = bid / u.tiles_sx;
        const int l = lk / u.kgroups;
        const int k0 = (lk % u.kgroups) * G;
        ti.Hl = u.Hl; ti.Wl = u.Wl; ti.Hr = u.Hr; ti.Wr = u.Wr; ti.Sy = u.Sy; ti.Sx = u.Sx;
        ti.SY0 = ty * BSY;
        ti.SX0 = u.sx_origin + tx * BSX;
        ti.nmat = min(G, u.pm.K - k0);
        ti.lc = l;
        ti.rc2 = u.pm.r_l != 0 ? l : 0;
        ti.rc3 = k0;
        ti.out0 = ((long long)l * u.pm.o_l + (long long)k0 * u.pm.o_k) * u.Sy * u.Sx;
        ti.ostride = u.pm.o_k * (long long)u.Sy * u.Sx;
        ti.lsrc = (long long)l * u.Hl * u.Wl;
        ti.rsrc0 = ((long long)l * u.pm.r_l + (long long)k0 * u.pm.r_k) * u.Hr * u.Wr;
        ti.rstride = u.pm.r_k * (long long)u.Hr * u.Wr;
        ti.lmap = &lmap_u;
        ti.rmap = &rmap_u;
      } else {
        unsigned int t = 0;
        if (lane == 0) t = atomicAdd(p.rg.queue, 1u);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= (unsigned)p.rg.n_tiles) break;
        const RaggedTile rt = p.rg.tiles[t];
        const RaggedPairDev pr = p.rg.pairs[rt.pair];
        ti.Hl = pr.Hl; ti.Wl = pr.Wl; ti.Hr = pr.Hr; ti.Wr = pr.Wr;
        ti.Sy = pr.Hl + pr.Hr - 1;
        ti.Sx = pr.Wl + pr.Wr - 1;
        ti.SY0 = rt.sy0;
        ti.SX0 = rt.sx0;
        ti.nmat = 1;
        ti.lc = 0;
        ti.rc2 = 0;
        ti.rc3 = 0;
        ti.out0 = (long long)pr.out_off;
        ti.ostride = 0;
        ti.lsrc = 0;
        ti.rsrc0 = 0;
        ti.rstride = 0;
        ti.lmap = p.rg.lmaps + pr.left;
        ti.rmap = p.rg.rmaps + pr.right;
      }
      TileSpan sp = tile_span<C>(ti);
      if (!ragged && p.u.n_slices > 1) {
        // this CTA's slice of the tile's right rows (empty for the last
        // slices of tiles with fewer rows: no stages, just the sentinel)
        const int y0 = slice * p.u.rows_per_slice;
        sp.ny = max(0, min(p.u.rows_per_slice, sp.ny - y0));
        sp.y_lo += y0;
      }
      const int nst = sp.ny * sp.nxc;
      for (int st = 0; st < nst; ++st, ++j) {
        const int slot = j % S;
        bool w = true;
        if (lane == 0) w = mbar_wait_bounded(&empty[slot], ((j / S) & 1) ^ 1);
        if (!__shfl_sync(0xffffffffu, (int)w, 0)) {
          if (lane == 0) record_timeout(p.flags, 2);
          ok = false;
          break;
        }
        const int xc_start = sp.x_lo + (st / sp.ny) * XC;
        const int y = sp.y_lo + (st % sp.ny);
        if (lane == 0) {
          StageMeta& m = meta[slot];
          m.ti = ti;
          m.y = y;
          m.xc_start = xc_start;
          m.first = st == 0;
          m.last = st == nst - 1;
          m.end = 0;
        }
        const int lx0 = xc_start + ti.SX0 - (ti.Wr - 1);
        const int ly0 = y + ti.SY0 - (ti.Hr - 1);
        T* sL = stage_L(slot);
        T* sR = stage_R(slot);
        if (use_tma) {
          if (lane == 0) {
            mbar_arrive_expect_tx(&full[slot], (uint32_t)((C::L_ELEMS + C::R_ELEMS) * sizeof(T)));
            tma_load_3d(sL, reinterpret_cast<const CUtensorMap*>(ti.lmap), &full[slot], lx0, ly0, ti.lc);
            tma_load_4d(sR, reinterpret_cast<const CUtensorMap*>(ti.rmap), &full[slot], xc_start, y, ti.rc2,
                        ti.rc3);
          }
        } else {
          const T* Lm = p.left + ti.lsrc;
          for (int e = lane; e < C::L_ELEMS; e += 32) {
            const int r = e / LW, c = e % LW;
            const int gy = ly0 + r, gx = lx0 + c;
            const bool okk = gy >= 0 && gy < ti.Hl && gx >= 0 && gx < ti.Wl;
            cp_async_zfill<sizeof(T)>(sL + e, okk ? Lm + (long long)gy * ti.Wl + gx : p.left, okk);
          }
          for (int e = lane; e < C::R_ELEMS; e += 32) {
            const int g = e / XC, c = e % XC;
            const int gx = xc_start + c;
            const bool okk = g < ti.nmat && gx < ti.Wr;
            const T* src = p.right + ti.rsrc0 + (long long)g * ti.rstride + (long long)y * ti.Wr + gx;
            cp_async_zfill<sizeof(T)>(sR + e, okk ? src : p.right, okk);
          }
          cp_async_mbar_arrive(&full[slot]);
          if (lane == 0) mbar_arrive(&full[slot]);
        }
      }
    }
    if (ok) {
      // end-of-work sentinel
      const int slot = j % S;
      bool w = true;
      if (lane == 0) w = mbar_wait_bounded(&empty[slot], ((j / S) & 1) ^ 1);
      if (__shfl_sync(0xffffffffu, (int)w, 0)) {
        if (lane == 0) {
          meta[slot].end = 1;
          mbar_arrive_count(&full[slot], use_tma ? 1u : 33u);
        }
      } else if (lane == 0) {
        record_timeout(p.flags, 3);
      }
    }
    return;
  }

  // ================================================================== consumers
  const int wg = warp % C::WG;
  const int wx = (warp / C::WG) % C::WX;
  const int wy = warp / (C::WG * C::WX);
  const int lyy = lane >> 3, lxx = lane & 7;
  const int row0 = wy * C::WSY + lyy * TSY;  // first local sy row of this thread
  const int col0 = wx * C::WSX + lxx * TSX;  // first local sx column of this thread

  T acc[TSY][TSX][TG];
  bool flushed = false;
  int since = 0;
  // tile state kept across its stages
  int t_Sy = 0, t_Sx = 0, t_SY0 = 0, t_SX0 = 0, t_nmat = 0;
  long long t_out0 = 0, t_ostride = 0;
  int yw_lo = 0, yw_hi = 0, xw_lo = 0, xw_hi = 0;

  auto zero = [&]() {
#pragma unroll
    for (int t = 0; t < TSY; ++t)
#pragma unroll
      for (int q = 0; q < TSX; ++q)
#pragma unroll
        for (int i = 0; i < TG; ++i) acc[t][q][i] = T(0);
  };

  // The empty asm keeps the compiler from hoisting the output addresses out of
  // the stage loop (they would pin many registers).
  const bool accumulate = !ragged && p.u.accumulate;
  auto flush = [&]() {
    int sy_base = t_SY0 + row0, sx_base = t_SX0 + col0, gb = wg * TG;
    asm volatile("" : "+r"(sy_base), "+r"(sx_base), "+r"(gb));
#pragma unroll
    for (int i = 0; i < TG; ++i) {
      if (gb + i >= t_nmat) continue;
      T* o = p.out + t_out0 + (long long)(gb + i) * t_ostride;
#pragma unroll
      for (int t = 0; t < TSY; ++t) {
        const int sy = sy_base + t;
        if (sy >= t_Sy) continue;
#pragma unroll
        for (int q = 0; q < TSX; ++q) {
          const int sx = sx_base + q;
          if (sx < 0 || sx >= t_Sx) continue;
          T* dst = o + (long long)sy * t_Sx + sx;
          if (accumulate)
            atomicAdd(dst, acc[t][q][i]);  // result unused: a red.global.add
          else
            *dst = flushed ? *dst + acc[t][q][i] : acc[t][q][i];
          acc[t][q][i] = T(0);
        }
      }
    }
    flushed = true;
  };

  zero();
  for (int j = 0;; ++j) {
    const int slot = j % S;
    if (!mbar_wait_bounded(&full[slot], (j / S) & 1)) {
      if (lane == 0) record_timeout(p.flags, 1);
      break;
    }
    const StageMeta& m = meta[slot];
    if (m.end) break;
    const int y = m.y, xc_start = m.xc_start;
    const int last = m.last;
    if (m.first) {
      const TileInfo& ti = m.ti;
      t_Sy = ti.Sy;
      t_Sx = ti.Sx;
      t_SY0 = ti.SY0;
      t_SX0 = ti.SX0;
      t_nmat = ti.nmat;
      t_out0 = ti.out0;
      t_ostride = ti.ostride;
      const int wsy0 = ti.SY0 + wy * C::WSY, wsx0 = ti.SX0 + wx * C::WSX;
      // right rows / columns that meet this warp's band of shifts
      yw_lo = ti.Hr - 1 - (wsy0 + C::WSY - 1);
      yw_hi = ti.Hl + ti.Hr - 1 - wsy0;
      xw_lo = max(0, ti.Wr - 1 - (wsx0 + C::WSX - 1));
      xw_hi = min(ti.Wr, ti.Wl + ti.Wr - 1 - wsx0);
      flushed = false;
      since = 0;
    }
    int xs = max(xw_lo - xc_start, 0) & ~3;
    int xe = min(xw_hi - xc_start, XC);
    if (y >= yw_lo && y < yw_hi && xs < xe) {
      const T* sL = stage_L(slot) + row0 * LW + col0;
      const T* sR = stage_R(slot) + (wg * TG) * XC;
      // three rotating 4-column buffers per left row: window = 12 columns
      V4<T> P[TSY], Q[TSY], R[TSY];
#pragma unroll
      for (int t = 0; t < TSY; ++t) {
        P[t] = lds4<T>(sL + t * LW + xs);
        Q[t] = lds4<T>(sL + t * LW + xs + 4);
      }
      // one 4-column step over the window (A | B | C), C freshly loaded
      auto step = [&](V4<T>* A, V4<T>* B, V4<T>* Cn, int x) {
        V4<T> rv[TG];
#pragma unroll
        for (int i = 0; i < TG; ++i) rv[i] = lds4<T>(sR + i * XC + x);
#pragma unroll
        for (int t = 0; t < TSY; ++t) {
          Cn[t] = lds4<T>(sL + t * LW + x + 8);
#pragma unroll
          for (int xx = 0; xx < 4; ++xx)
#pragma unroll
            for (int q = 0; q < TSX; ++q) {
              const int w = xx + q;
              const T lv = w < 4 ? A[t].v[w] : (w < 8 ? B[t].v[w - 4] : Cn[t].v[w - 8]);
#pragma unroll
              for (int i = 0; i < TG; ++i) acc[t][q][i] = fma(lv, rv[i].v[xx], acc[t][q][i]);
            }
        }
      };
#pragma unroll 1
      for (int xo = xs; xo < xe; xo += 12) {
        step(P, Q, R, xo);
        if (xo + 4 >= xe) break;
        step(Q, R, P, xo + 4);
        if (xo + 8 >= xe) break;
        step(R, P, Q, xo + 8);
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[slot]);
    if (++since == C::FLUSH_STAGES || last) {
      flush();
      since = 0;
    }
  }
}

// Tile shapes.  Cfg<T, TSY, TG, WY, WX, WG, XC, STAGES, MINB>.
using CfgF32Multi = Cfg<float, 2, 4, 4, 1, 2, 128, 4, 1>;   // 32 sy x 64 sx x 8 mats, 8+1 warps
using CfgF32Single = Cfg<float, 4, 1, 4, 1, 1, 128, 2, 2>;  // 64 sy x 64 sx x 1 mat, 4+1 warps
using CfgF32Small = Cfg<float, 2, 1, 4, 1, 1, 128, 3, 3>;   // 32 sy x 64 sx x 1 mat, 4+1 warps
using CfgF64Multi = Cfg<double, 2, 2, 4, 1, 2, 64, 3, 1>;   // 32 x 64 x 4 mats
using CfgF64Single = Cfg<double, 2, 1, 4, 1, 1, 64, 3, 2>;  // 32 x 64 x 1 mat

// Right rows of the tiles in tile row ty (the y range of tile_span).
template <typename C>
int tile_rows(const Geometry& g, int ty) {
  const int sy0 = ty * C::BSY;
  const int lo = std::max(0, g.Hr - 1 - (sy0 + C::BSY - 1));
  const int hi = std::min(g.Hr, g.Hl + g.Hr - 1 - sy0);
  return std::max(0, hi - lo);
}

int sm_count_cached() {
  static const int n = [] {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
      return 152;
    return sms;
  }();
  return n;
}

// Rows per slice for a launch of `blocks` tiles: none (0) while the tiles
// fill a wave of CTAs (`wave` resident at once); else the longest slices (a
// power of two, at least 4 rows) that give two waves of non-empty slices,
// or 4-row slices when even those give fewer.  XC_DIRECT_SLICE_ROWS fixes
// the slice length (studies, tests).
template <typename C>
int pick_slice_rows(const Geometry& g, long long blocks, int tiles_sy, long long per_tile_row, int wave) {
  static const int fixed = [] {
    const char* e = std::getenv("XC_DIRECT_SLICE_ROWS");
    return e ? std::max(0, std::atoi(e)) : 0;
  }();
  if (fixed > 0) return fixed;
  if (blocks >= wave) return 0;
  int max_rows = 0;
  for (int ty = 0; ty < tiles_sy; ++ty) max_rows = std::max(max_rows, tile_rows<C>(g, ty));
  int rows = 4;
  while (rows < max_rows) rows *= 2;
  for (; rows > 4; rows /= 2) {
    long long live = 0;
    for (int ty = 0; ty < tiles_sy; ++ty) live += (long long)div_up(tile_rows<C>(g, ty), rows) * per_tile_row;
    if (live >= 2LL * wave) break;
  }
  return rows >= max_rows ? 0 : rows;
}

template <typename C>
xc_status launch_uniform(const typename C::type* left, const typename C::type* right, typename C::type* out,
                         const Geometry& g, const PairMap& pm, cudaStream_t stream, int force_loader,
                         DirectAccumulate acc_mode) {
  using T = typename C::type;
  DirectArgs<T> p;
  std::memset(&p, 0, sizeof(p));
  p.left = left;
  p.right = right;
  p.out = out;
  Uniform<T>& u = p.u;
  u.Hl = g.Hl;
  u.Wl = g.Wl;
  u.Hr = g.Hr;
  u.Wr = g.Wr;
  u.Sy = g.Sy;
  u.Sx = g.Sx;
  u.pm = pm;
  const int rem = (g.Wr - 1) % C::VEC;
  u.sx_origin = rem == 0 ? 0 : rem - C::VEC;
  u.tiles_sx = div_up(g.Sx - u.sx_origin, C::BSX);
  u.tiles_sy = div_up(g.Sy, C::BSY);
  u.kgroups = div_up(pm.K, C::G);
  p.flags = device_flags();

  const long long tiles = (long long)u.tiles_sx * u.tiles_sy * pm.n_left * u.kgroups;
  if (tiles <= 0) return XC_OK;
  auto kern = direct_kernel<C>;
  int per_sm = 0;
  XC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM_BYTES));
  XC_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, C::NT, C::SMEM_BYTES));
  const int slice_rows = acc_mode == DirectAccumulate::kNever
                             ? 0
                             : pick_slice_rows<C>(g, tiles, u.tiles_sy, (long long)u.tiles_sx * pm.n_left * u.kgroups,
                                                  std::max(1, per_sm) * sm_count_cached());
  u.n_slices = 1;
  u.rows_per_slice = 1 << 30;
  if (slice_rows > 0) {
    int max_rows = 0;
    for (int ty = 0; ty < u.tiles_sy; ++ty) max_rows = std::max(max_rows, tile_rows<C>(g, ty));
    u.n_slices = std::max(1, div_up(max_rows, slice_rows));
    u.rows_per_slice = slice_rows;
  }
  // the caller's output is added into (work-distribution launchers), or is
  // zeroed here when slices of a tile add into the same outputs
  u.accumulate = (acc_mode == DirectAccumulate::kCaller || u.n_slices > 1) ? 1 : 0;
  const long long blocks = tiles * u.n_slices;
  if (blocks > 0x7fffffffLL) return fail(XC_ERR_INVALID_ARGUMENT, "problem too large for one launch");
  if (u.accumulate && acc_mode != DirectAccumulate::kCaller) {
    const long long n_out = (long long)(pm.n_left - 1) * pm.o_l + (long long)(pm.K - 1) * pm.o_k + 1;
    XC_CUDA_TRY(cudaMemsetAsync(out, 0, (size_t)n_out * g.Sy * g.Sx * sizeof(T), stream));
  }

  // TMA needs 16-byte aligned bases and row/matrix pitches.
  const size_t es = sizeof(T);
  const bool tma_ok = ((uintptr_t)left % 16 == 0) && ((uintptr_t)right % 16 == 0) && ((size_t)g.Wl * es % 16 == 0) &&
                      ((size_t)g.Wr * es % 16 == 0);
  const bool use_tma = force_loader < 0 ? tma_ok : (force_loader == 1);
  if (use_tma && !tma_ok) return fail(XC_ERR_INVALID_ARGUMENT, "TMA loader requested for unaligned pitches");

  CUtensorMap lmap, rmap;
  std::memset(&lmap, 0, sizeof(lmap));
  std::memset(&rmap, 0, sizeof(rmap));
  if (use_tma) {
    const CUtensorMapDataType dt = sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
    uint64_t ldims[3] = {(uint64_t)g.Wl, (uint64_t)g.Hl, (uint64_t)pm.n_left};
    uint64_t lstr[2] = {(uint64_t)g.Wl * es, (uint64_t)g.Wl * g.Hl * es};
    uint32_t lbox[3] = {(uint32_t)C::LW, (uint32_t)C::BSY, 1};
    if (!encode_tiled(&lmap, dt, 3, left, ldims, lstr, lbox, CU_TENSOR_MAP_SWIZZLE_NONE)) return XC_ERR_INVALID_ARGUMENT;
    const uint64_t mat = (uint64_t)g.Wr * g.Hr * es;
    uint64_t rdims[4] = {(uint64_t)g.Wr, (uint64_t)g.Hr, pm.r_l != 0 ? (uint64_t)pm.n_left : 1, (uint64_t)pm.K};
    uint64_t rstr[3] = {(uint64_t)g.Wr * es, mat * (uint64_t)(pm.r_l != 0 ? pm.r_l : 1), mat * (uint64_t)pm.r_k};
    uint32_t rbox[4] = {(uint32_t)C::XC, 1, 1, (uint32_t)C::G};
    if (!encode_tiled(&rmap, dt, 4, right, rdims, rstr, rbox, CU_TENSOR_MAP_SWIZZLE_NONE)) return XC_ERR_INVALID_ARGUMENT;
  }

  static_assert(C::SMEM_BYTES <= 227 * 1024, "shared memory budget");
  const int slot = kernel_timer_begin(stream);
  kern<<<(unsigned)blocks, C::NT, C::SMEM_BYTES, stream>>>(lmap, rmap, p, use_tma);
  kernel_timer_end(slot, stream);
  XC_CUDA_TRY(cudaGetLastError());
  return XC_OK;
}

template <typename C>
xc_status launch_ragged(const RaggedLaunch& rl, cudaStream_t stream) {
  using T = typename C::type;
  DirectArgs<T> p;
  std::memset(&p, 0, sizeof(p));
  p.left = reinterpret_cast<const T*>(rl.left);
  p.right = reinterpret_cast<const T*>(rl.right);
  p.out = reinterpret_cast<T*>(rl.out);
  p.rg.tiles = rl.tiles;
  p.rg.pairs = rl.pairs;
  p.rg.lmaps = rl.lmaps;
  p.rg.rmaps = rl.rmaps;
  p.rg.queue = rl.queue;
  p.rg.n_tiles = rl.n_tiles;
  p.flags = device_flags();
  CUtensorMap dummy;
  std::memset(&dummy, 0, sizeof(dummy));
  // (the caller raised the kernel's shared-memory limit before any capture)
  direct_kernel<C><<<(unsigned)rl.grid, C::NT, C::SMEM_BYTES, stream>>>(dummy, dummy, p, true);
  XC_CUDA_TRY(cudaGetLastError());
  return XC_OK;
}

template <typename C>
RaggedShape shape_of() {
  RaggedShape s;
  s.bsy = C::BSY;
  s.bsx = C::BSX;
  s.lw = C::LW;
  s.xc = C::XC;
  s.vec = C::VEC;
  s.threads = C::NT;
  s.smem = C::SMEM_BYTES;
  s.kernel = reinterpret_cast<const void*>(&direct_kernel<C>);
  return s;
}

}  // namespace

xc_status direct_launch(xc_dtype dtype, const void* left, const void* right, void* out, const Geometry& g,
                        const PairMap& pm, cudaStream_t stream, int force_loader, DirectAccumulate acc, int tile) {
  // tile 0: 8 partners per CTA when there are 4 or more (3 for FP64), else
  // one; 1: 8 (FP64: 4) partners, 32 x 64 shifts; 2: one partner, 64 x 64
  // shifts (FP64: 32 x 64); 3: one partner, 32 x 64 shifts
  if (tile < 0 || tile > 3) return fail(XC_ERR_INVALID_ARGUMENT, "plain kernel tiles are 0-3");
  if (dtype == XC_F32) {
    const int t = tile != 0 ? tile : (pm.K >= 4 ? 1 : 2);
    const float* l = (const float*)left;
    const float* r = (const float*)right;
    float* o = (float*)out;
    if (t == 1) return launch_uniform<CfgF32Multi>(l, r, o, g, pm, stream, force_loader, acc);
    if (t == 2) return launch_uniform<CfgF32Single>(l, r, o, g, pm, stream, force_loader, acc);
    return launch_uniform<CfgF32Small>(l, r, o, g, pm, stream, force_loader, acc);
  }
  const int t = tile != 0 ? tile : (pm.K >= 3 ? 1 : 2);
  const double* l = (const double*)left;
  const double* r = (const double*)right;
  double* o = (double*)out;
  if (t == 1) return launch_uniform<CfgF64Multi>(l, r, o, g, pm, stream, force_loader, acc);
  return launch_uniform<CfgF64Single>(l, r, o, g, pm, stream, force_loader, acc);
}

// Tile shapes a ragged plan may pick from (the autotuner's candidates).
int ragged_shape_count(xc_dtype dtype) { return dtype == XC_F32 ? 2 : 1; }

RaggedShape ragged_shape(xc_dtype dtype, int index) {
  if (dtype == XC_F32) return index == 0 ? shape_of<CfgF32Single>() : shape_of<CfgF32Small>();
  return shape_of<CfgF64Single>();
}

xc_status ragged_launch(xc_dtype dtype, int index, const RaggedLaunch& rl, cudaStream_t stream) {
  if (dtype == XC_F32)
    return index == 0 ? launch_ragged<CfgF32Single>(rl, stream) : launch_ragged<CfgF32Small>(rl, stream);
  return launch_ragged<CfgF64Single>(rl, stream);
}

}  // namespace xc
