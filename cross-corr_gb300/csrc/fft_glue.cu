// fft_glue.cu -- HBM-bound glue of the FFT path, as fused and coalesced
// kernels (sm_103a).
//
//  pad_kernel            replaces the host-side relative_zero_padding<2>
//                        (src/matrix.hpp:33-46) and the memset + scatter pair
//                        (src/scatter.cu:16-102, src/one_to_many.hpp:705-725):
//                        one pass writes every element of the padded buffer
//                        (data or zero) with 16-byte stores.
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
// beyond pad_cols is left untouched).  A block walks `rows_per_block`
// consecutive (matrix, row) pairs, so the row indices cost one division per
// block.  Each row is written as a scalar head up to its first 16-byte
// boundary (rows of the in-place R2C layout, pitch 2 (px/2 + 1), start only
// 8-byte aligned every other row), a body of 16-byte stores and a scalar
// tail; rows outside the source are zeros and read nothing.  A thread loads
// its 16-byte chunk of every one of the block's rows before it stores any,
// so up to kGlueRows loads per thread are in flight; a chunk whose source is
// 8-byte but not 16-byte aligned (the odd rows' bodies) is read as two
// 8-byte loads.
template <typename T>
__device__ __forceinline__ T pad_value(const T* srow, bool row_in, int sx, int cols) {
  return (row_in && sx >= 0 && sx < cols) ? __ldg(srow + sx) : T(0);
}

template <typename T, typename Vec>
__device__ __forceinline__ Vec pad_chunk(const T* srow, bool row_in, int sx0, int cols) {
  constexpr int V = 16 / (int)sizeof(T);
  T v[V];
  if (!row_in || sx0 >= cols || sx0 + V <= 0) {
#pragma unroll
    for (int e = 0; e < V; ++e) v[e] = T(0);
  } else if (sx0 >= 0 && sx0 + V <= cols && (((uintptr_t)(srow + sx0)) & 15) == 0) {
    const Vec f = __ldg(reinterpret_cast<const Vec*>(srow + sx0));
    memcpy(v, &f, sizeof(f));
  } else if (sizeof(T) == 4 && sx0 >= 0 && sx0 + V <= cols && (((uintptr_t)(srow + sx0)) & 7) == 0) {
    const float2 a = __ldg(reinterpret_cast<const float2*>(srow + sx0));
    const float2 b = __ldg(reinterpret_cast<const float2*>(srow + sx0 + 2));
    memcpy(v, &a, 8);
    memcpy(reinterpret_cast<char*>(v) + 8, &b, 8);
  } else {
#pragma unroll
    for (int e = 0; e < V; ++e) v[e] = pad_value(srow, true, sx0 + e, cols);
  }
  Vec o;
  memcpy(&o, v, sizeof(o));
  return o;
}

template <typename T>
__global__ void pad_kernel(const T* __restrict__ src, T* __restrict__ dst, int rows, int cols, int count, int pad_rows,
                           int pad_cols, int dst_pitch, int dst_y, int dst_x, int rows_per_block) {
  constexpr int V = 16 / (int)sizeof(T);  // elements per 16-byte store
  constexpr int R = kGlueRows;
  using Vec = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
  const long long n_rows = (long long)count * pad_rows;
  const long long r0 = (long long)blockIdx.x * rows_per_block;
  const int nr = (int)min((long long)min(rows_per_block, R), n_rows - r0);
  long long m = r0 / pad_rows;
  int y = (int)(r0 - m * pad_rows);
  const T* srow[R];
  T* drow[R];
  bool row_in[R];
  int lead[R], n_body[R];
  int nb_max = 0;
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int sy = y - dst_y;
    row_in[i] = i < nr && sy >= 0 && sy < rows;
    srow[i] = src + (m * rows + (row_in[i] ? sy : 0)) * (long long)cols;
    drow[i] = dst + (r0 + min(i, nr - 1)) * (long long)dst_pitch;
    lead[i] = min(pad_cols, (int)(((16u - ((uint32_t)(uintptr_t)drow[i] & 15u)) & 15u) / sizeof(T)));
    n_body[i] = i < nr ? (pad_cols - lead[i]) / V : 0;
    nb_max = max(nb_max, n_body[i]);
    if (i < nr) {
      const int tail0 = lead[i] + n_body[i] * V;
      if ((int)threadIdx.x < lead[i])
        drow[i][threadIdx.x] = pad_value(srow[i], row_in[i], (int)threadIdx.x - dst_x, cols);
      if ((int)threadIdx.x < pad_cols - tail0)
        drow[i][tail0 + threadIdx.x] = pad_value(srow[i], row_in[i], tail0 + (int)threadIdx.x - dst_x, cols);
    }
    if (++y == pad_rows) {
      y = 0;
      ++m;
    }
  }
  for (int k = threadIdx.x; k < nb_max; k += blockDim.x) {
    Vec v[R];
#pragma unroll
    for (int i = 0; i < R; ++i)
      if (k < n_body[i]) v[i] = pad_chunk<T, Vec>(srow[i], row_in[i], lead[i] + k * V - dst_x, cols);
#pragma unroll
    for (int i = 0; i < R; ++i)
      if (k < n_body[i]) reinterpret_cast<Vec*>(drow[i] + lead[i])[k] = v[i];
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
  // a few rows per block when there are many (fewer index divisions), one
  // when there are few (enough blocks to fill the GPU)
  const int rpb = (int)std::max(1LL, std::min((long long)kGlueRows, n_rows / (152LL * 16)));
  const long long blocks = (n_rows + rpb - 1) / rpb;
  if (blocks > 0x7fffffffLL) return fail(XC_ERR_INVALID_ARGUMENT, "too many rows for one launch");
  const int threads = pad_cols >= 512 ? 128 : 64;
  if (dtype == XC_F32)
    pad_kernel<float><<<(unsigned)blocks, threads, 0, stream>>>((const float*)src, (float*)dst, rows, cols, count,
                                                                pad_rows, pad_cols, dst_pitch, dst_y, dst_x, rpb);
  else
    pad_kernel<double><<<(unsigned)blocks, threads, 0, stream>>>((const double*)src, (double*)dst, rows, cols, count,
                                                                 pad_rows, pad_cols, dst_pitch, dst_y, dst_x, rpb);
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
