// fft_glue.cu -- HBM-bound glue of the FFT path, as fused and coalesced
// kernels (sm_103a).
//
//  pad_kernel            replaces the host-side relative_zero_padding<2>
//                        (src/matrix.hpp:33-46) and the memset + scatter pair
//                        (src/scatter.cu:16-102, src/one_to_many.hpp:705-725):
//                        one pass writes every element of the padded buffer
//                        (data or zero), a warp per row, in 8- or 16-byte
//                        units.
//  conj_multiply_kernel  replaces hadamard_original (src/hadamard.cu:33-58) and
//                        hadamard_n_to_m_over_output (src/hadamard.cu:116-149):
//                        out[o] = L[l] * conj(R[r]) for every output of the
//                        mode's pair map; each left bin is loaded once and
//                        reused for all its partners.
//  normalize_kernel      replaces the host loop normalize_fft_results
//                        (src/fft_helpers.hpp:193-261): quadrant swap, division
//                        by the transform size and crop in one coalesced pass.
#include <algorithm>
#include <cstring>
#include <type_traits>

#include "xc_common.cuh"
#include "xc_internal.h"

namespace xc {

namespace {

template <typename T>
struct Cplx;
template <>
struct Cplx<float> {
  using type = float2;
};
template <>
struct Cplx<double> {
  using type = double2;
};

// multiply_conjugate (src/hadamard.cu:18-24): left * conj(right).
template <typename C>
__device__ __forceinline__ C mul_conj(C a, C b) {
  C r;
  r.x = a.x * b.x + a.y * b.y;
  r.y = -a.x * b.y + a.y * b.x;
  return r;
}

constexpr int kGlueRows = 8;  // rows per block in the row-walking glue kernels

// dst[m][y][x] = src[m][y - dst_y][x - dst_x] inside the source, 0 elsewhere;
// dst rows have pitch `dst_pitch` elements (>= pad_cols; the tail of a row
// beyond pad_cols is left untouched).  One warp per destination row (the
// (matrix, row) pair costs one division per warp).  The row moves in units
// U of E = sizeof(U) / sizeof(T) elements: E = 2 (8-byte floats, 16-byte
// doubles) when the row starts, the pitch, the source width and the offset
// dst_x allow it -- rows of the in-place R2C layout, pitch 2 (px/2 + 1),
// start 8-byte aligned, so 16-byte units would not do for FP32 -- else
// E = 1.  A lane loads its units of eight 32-unit strips before it stores
// any, so eight loads per lane are in flight; rows outside the source are
// zeros and read nothing.
template <typename T, typename U>
__global__ void __launch_bounds__(256) pad_kernel(const T* __restrict__ src, T* __restrict__ dst, int rows, int cols,
                                                  long long n_rows, int pad_rows, int pad_cols, int dst_pitch,
                                                  int dst_y, int dst_x) {
  constexpr int E = (int)(sizeof(U) / sizeof(T));
  constexpr int kStrips = 8;
  const int lane = threadIdx.x & 31;
  const long long row = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (row >= n_rows) return;  // warp-uniform
  const long long m = row / pad_rows;
  const int sy = (int)(row - m * pad_rows) - dst_y;
  const bool row_in = sy >= 0 && sy < rows;
  const U* __restrict__ su = reinterpret_cast<const U*>(src + (m * rows + (row_in ? sy : 0)) * (long long)cols);
  U* __restrict__ du = reinterpret_cast<U*>(dst + row * (long long)dst_pitch);
  const int units = pad_cols / E, src_units = cols / E, dxu = dst_x / E;
  U zero;
  memset(&zero, 0, sizeof(zero));
  for (int u0 = 0; u0 < units; u0 += 32 * kStrips) {
    U v[kStrips];
#pragma unroll
    for (int j = 0; j < kStrips; ++j) {
      const int u = u0 + 32 * j + lane, x = u - dxu;
      v[j] = (row_in && u < units && x >= 0 && x < src_units) ? __ldg(su + x) : zero;
    }
#pragma unroll
    for (int j = 0; j < kStrips; ++j) {
      const int u = u0 + 32 * j + lane;
      if (u < units) du[u] = v[j];
    }
  }
}

// out[l*o_l + k*o_k] = lspec[l] * conj(rspec[l*r_l + k*r_k]) bin by bin:
// grid.y = left index l, each thread owns one bin and walks the K partners
// of l eight at a time, with the eight right loads issued together.
template <typename C>
__global__ void conj_multiply_kernel(const C* __restrict__ lspec, const C* __restrict__ rspec, C* __restrict__ out,
                                     long long bins, PairMap pm, long long n_out) {
  (void)n_out;
  const int l = blockIdx.y;
  const C* lrow = lspec + (long long)l * bins;
  const C* rbase = rspec + (long long)l * pm.r_l * bins;
  C* obase = out + (long long)l * pm.o_l * bins;
  const long long rstep = (long long)pm.r_k * bins, ostep = (long long)pm.o_k * bins;
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < bins;
       b += (long long)gridDim.x * blockDim.x) {
    const C lv = __ldg(lrow + b);
    int k = 0;
    for (; k + 8 <= pm.K; k += 8) {
      C rv[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) rv[u] = __ldg(rbase + (k + u) * rstep + b);
#pragma unroll
      for (int u = 0; u < 8; ++u) obase[(k + u) * ostep + b] = mul_conj(lv, rv[u]);
    }
    for (; k < pm.K; ++k) obase[k * ostep + b] = mul_conj(lv, __ldg(rbase + k * rstep + b));
  }
}

// out[m][sy][sx] = raw[m][(sy - (Hr-1)) mod py][(sx - (Wr-1)) mod px] * scale;
// with raw=true it instead copies raw[m][y][x] (dense py x px output).  A
// block takes kGlueRows output rows (one division per block) and resolves
// their row pointers first; each thread then steps along the rows with the
// kGlueRows loads of a column issued together.
template <typename T, bool F64SCALE>
__global__ void normalize_kernel(const T* __restrict__ raw, T* __restrict__ out, int py, int px, int raw_pitch,
                                 int count, int Hr, int Wr, int Sy, int Sx, double scale, bool rawcopy) {
  const int oy = rawcopy ? py : Sy, ox = rawcopy ? px : Sx;
  const long long n_rows = (long long)count * oy;
  const T fscale = (T)scale;
  const long long r0 = (long long)blockIdx.x * kGlueRows;
  long long m = r0 / oy;
  int sy = (int)(r0 - m * oy);
  const T* rrow[kGlueRows];
  const int nr = (int)min((long long)kGlueRows, n_rows - r0);
#pragma unroll
  for (int i = 0; i < kGlueRows; ++i) {
    int ry = sy;
    if (!rawcopy) {
      ry = sy - (Hr - 1);
      if (ry < 0) ry += py;
    }
    rrow[i] = raw + (m * py + ry) * (long long)raw_pitch;
    if (++sy == oy) {
      sy = 0;
      ++m;
    }
  }
  T* orow = out + r0 * (long long)ox;
  const int xoff = rawcopy ? 0 : Wr - 1;
  for (int sx = threadIdx.x; sx < ox; sx += blockDim.x) {
    int rx = sx - xoff;
    if (rx < 0) rx += px;
    T v[kGlueRows];
#pragma unroll
    for (int i = 0; i < kGlueRows; ++i) v[i] = i < nr ? __ldg(rrow[i] + rx) : T(0);
#pragma unroll
    for (int i = 0; i < kGlueRows; ++i) {
      if (i < nr) {
        T w;
        if (rawcopy) w = v[i];
        else if (F64SCALE) w = (T)((double)v[i] * scale);
        else w = v[i] * fscale;
        orow[(long long)i * ox + sx] = w;
      }
    }
  }
}

// hadamard_original (src/hadamard.cu:33-58): deformed[i] = ref[i mod A] *
// conj(deformed[i]) over `batch` consecutive blocks of A bins.
template <typename C>
__global__ void hadamard_original_kernel(const C* __restrict__ ref, C* __restrict__ deformed, long long A,
                                         long long batch) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < A; i += (long long)gridDim.x * blockDim.x) {
    const C rv = ref[i];
    for (long long b = 0; b < batch; ++b) deformed[b * A + i] = mul_conj(rv, deformed[b * A + i]);
  }
}

int grid_for(long long work, int threads) {
  long long b = (work + threads - 1) / threads;
  if (b > 152LL * 64) b = 152LL * 64;
  if (b < 1) b = 1;
  return (int)b;
}

}  // namespace

xc_status glue_pad(xc_dtype dtype, const void* src, void* dst, int rows, int cols, int count, int pad_rows,
                   int pad_cols, int dst_y, int dst_x, cudaStream_t stream) {
  return glue_pad_pitched(dtype, src, dst, rows, cols, count, pad_rows, pad_cols, pad_cols, dst_y, dst_x, stream);
}

xc_status glue_pad_pitched(xc_dtype dtype, const void* src, void* dst, int rows, int cols, int count, int pad_rows,
                           int pad_cols, int dst_pitch, int dst_y, int dst_x, cudaStream_t stream) {
  if (count <= 0) return XC_OK;
  const long long n_rows = (long long)count * pad_rows;
  const long long blocks = (n_rows + 7) / 8;  // 8 warps, one row each
  if (blocks > 0x7fffffffLL) return fail(XC_ERR_INVALID_ARGUMENT, "too many rows for one launch");
  const size_t es = dtype == XC_F32 ? 4 : 8;
  // two-element units: every row start, source and destination, and the
  // placement of the source on a two-element boundary
  const bool pairs = dst_x % 2 == 0 && cols % 2 == 0 && pad_cols % 2 == 0 && dst_pitch % 2 == 0 &&
                     (uintptr_t)src % (2 * es) == 0 && (uintptr_t)dst % (2 * es) == 0;
  const long long nr = n_rows;
  if (dtype == XC_F32) {
    if (pairs)
      pad_kernel<float, float2><<<(unsigned)blocks, 256, 0, stream>>>((const float*)src, (float*)dst, rows, cols, nr,
                                                                     pad_rows, pad_cols, dst_pitch, dst_y, dst_x);
    else
      pad_kernel<float, float><<<(unsigned)blocks, 256, 0, stream>>>((const float*)src, (float*)dst, rows, cols, nr,
                                                                    pad_rows, pad_cols, dst_pitch, dst_y, dst_x);
  } else {
    if (pairs)
      pad_kernel<double, double2><<<(unsigned)blocks, 256, 0, stream>>>((const double*)src, (double*)dst, rows, cols,
                                                                       nr, pad_rows, pad_cols, dst_pitch, dst_y, dst_x);
    else
      pad_kernel<double, double><<<(unsigned)blocks, 256, 0, stream>>>((const double*)src, (double*)dst, rows, cols,
                                                                      nr, pad_rows, pad_cols, dst_pitch, dst_y, dst_x);
  }
  XC_CUDA_TRY(cudaGetLastError());
  return XC_OK;
}

xc_status glue_conj_multiply_pairs(xc_dtype dtype, const void* lspec, const void* rspec, void* out, long long bins,
                                   const PairMap& pm, long long n_out, cudaStream_t stream) {
  if (n_out <= 0 || bins <= 0) return XC_OK;
  const int threads = 256;
  long long bx = (bins + threads - 1) / threads;
  const long long cap = (152LL * 64 + pm.n_left - 1) / pm.n_left;
  if (bx > cap) bx = cap;
  if (pm.n_left > 65535) return fail(XC_ERR_INVALID_ARGUMENT, "too many left matrices for one launch");
  dim3 grid((unsigned)bx, (unsigned)pm.n_left);
  if (dtype == XC_F32)
    conj_multiply_kernel<float2><<<grid, threads, 0, stream>>>((const float2*)lspec, (const float2*)rspec,
                                                               (float2*)out, bins, pm, n_out);
  else
    conj_multiply_kernel<double2><<<grid, threads, 0, stream>>>((const double2*)lspec, (const double2*)rspec,
                                                                (double2*)out, bins, pm, n_out);
  XC_CUDA_TRY(cudaGetLastError());
  return XC_OK;
}

xc_status glue_normalize_pitched(xc_dtype dtype, const void* raw, void* out, int py, int px, int raw_pitch, int count,
                                 int Hr, int Wr, int Sy, int Sx, bool rawcopy, cudaStream_t stream) {
  if (count <= 0) return XC_OK;
  const int ox = rawcopy ? px : Sx;
  const int threads = ox >= 512 ? 128 : 64;
  const long long n_rows = (long long)count * (rawcopy ? py : Sy);
  const long long nb = (n_rows + kGlueRows - 1) / kGlueRows;
  if (nb > 0x7fffffffLL) return fail(XC_ERR_INVALID_ARGUMENT, "too many rows for one launch");
  const unsigned blocks = (unsigned)nb;
  const double scale = 1.0 / ((double)py * (double)px);
  // FP64 scaling for transform sides of 1024 or more.
  const bool f64scale = py >= 1024 || px >= 1024;
  if (dtype == XC_F32) {
    if (f64scale)
      normalize_kernel<float, true><<<blocks, threads, 0, stream>>>((const float*)raw, (float*)out, py, px, raw_pitch,
                                                                     count, Hr, Wr, Sy, Sx, scale, rawcopy);
    else
      normalize_kernel<float, false><<<blocks, threads, 0, stream>>>((const float*)raw, (float*)out, py, px,
                                                                      raw_pitch, count, Hr, Wr, Sy, Sx, scale, rawcopy);
  } else {
    normalize_kernel<double, true><<<blocks, threads, 0, stream>>>((const double*)raw, (double*)out, py, px,
                                                                    raw_pitch, count, Hr, Wr, Sy, Sx, scale, rawcopy);
  }
  XC_CUDA_TRY(cudaGetLastError());
  return XC_OK;
}

xc_status glue_normalize(xc_dtype dtype, const void* raw, void* out, int py, int px, int count, int Hr, int Wr, int Sy,
                         int Sx, cudaStream_t stream) {
  return glue_normalize_pitched(dtype, raw, out, py, px, px, count, Hr, Wr, Sy, Sx, false, stream);
}

xc_status glue_hadamard_original(xc_dtype dtype, const void* ref, void* deformed, long long area_per_pic,
                                 long long batch, int threads, cudaStream_t stream) {
  if (threads <= 0 || threads > 1024) return fail(XC_ERR_INVALID_ARGUMENT, "threads_per_block must be in [1, 1024]");
  const int blocks = grid_for(area_per_pic, threads);
  if (dtype == XC_F32)
    hadamard_original_kernel<float2><<<blocks, threads, 0, stream>>>((const float2*)ref, (float2*)deformed,
                                                                     area_per_pic, batch);
  else
    hadamard_original_kernel<double2><<<blocks, threads, 0, stream>>>((const double2*)ref, (double2*)deformed,
                                                                      area_per_pic, batch);
  XC_CUDA_TRY(cudaGetLastError());
  return XC_OK;
}

xc_status glue_hadamard_n_to_m(xc_dtype dtype, const void* left, const void* right, void* out, long long area,
                               int n_left, int n_right, cudaStream_t stream) {
  PairMap pm;
  pm.n_left = n_left;
  pm.K = n_right;
  pm.o_l = n_right;
  pm.o_k = 1;
  pm.r_l = 0;
  pm.r_k = 1;
  return glue_conj_multiply_pairs(dtype, left, right, out, area, pm, (long long)n_left * n_right, stream);
}

}  // namespace xc
