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

// dst[m][y][x] = src[m][y - dst_y][x - dst_x] inside the source, 0 elsewhere;
// dst rows have pitch `dst_pitch` elements (>= pad_cols; the tail of a row
// beyond pad_cols is left untouched).  grid.y walks the (matrix, row) pairs,
// so a row's indices are computed once per block; each thread writes 4
// consecutive elements of the row.
template <typename T>
__global__ void pad_kernel(const T* __restrict__ src, T* __restrict__ dst, int rows, int cols, int count, int pad_rows,
                           int pad_cols, int dst_pitch, int dst_y, int dst_x) {
  const long long n_rows = (long long)count * pad_rows;
  const int x0 = (blockIdx.x * blockDim.x + threadIdx.x) * 4;
  if (x0 >= pad_cols) return;
  for (long long rowid = blockIdx.y; rowid < n_rows; rowid += gridDim.y) {
    const int y = (int)(rowid % pad_rows);
    const long long m = rowid / pad_rows;
    const int sy = y - dst_y;
    const bool row_in = sy >= 0 && sy < rows;
    const T* srow = src + (m * rows + sy) * (long long)cols;
    T* drow = dst + rowid * (long long)dst_pitch;
    T v[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int sx = x0 + e - dst_x;
      v[e] = (row_in && sx >= 0 && sx < cols) ? __ldg(srow + sx) : T(0);
    }
    bool done = false;
    if constexpr (sizeof(T) == 4) {
      if (x0 + 4 <= pad_cols && (((uintptr_t)(drow + x0)) & 15) == 0) {
        *reinterpret_cast<float4*>(drow + x0) = make_float4(v[0], v[1], v[2], v[3]);
        done = true;
      }
    }
    if (!done) {
#pragma unroll
      for (int e = 0; e < 4; ++e)
        if (x0 + e < pad_cols) drow[x0 + e] = v[e];
    }
  }
}

// out[o] = lspec[l] * conj(rspec[r]) bin by bin; grid.y walks the outputs o
// of the pair map (o -> (l, k) decoded once per block), threads the bins, so
// every thread issues independent loads.
template <typename C>
__global__ void conj_multiply_kernel(const C* __restrict__ lspec, const C* __restrict__ rspec, C* __restrict__ out,
                                     long long bins, PairMap pm, long long n_out) {
  const long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (b >= bins) return;
  for (long long o = blockIdx.y; o < n_out; o += gridDim.y) {
    // invert o = l*o_l + k*o_k for the three pair-map forms
    long long l, k;
    if (pm.o_l == 0) {
      l = 0;
      k = o;
    } else if (pm.o_k == 1 && pm.o_l == pm.K) {
      l = o / pm.K;
      k = o % pm.K;
    } else {
      l = o % pm.n_left;
      k = o / pm.n_left;
    }
    const long long r = l * pm.r_l + k * pm.r_k;
    out[o * bins + b] = mul_conj(__ldg(lspec + l * bins + b), __ldg(rspec + r * bins + b));
  }
}

// out[m][sy][sx] = raw[m][(sy - (Hr-1)) mod py][(sx - (Wr-1)) mod px] * scale;
// with raw=true it instead copies raw[m][y][x] (dense py x px output).
// grid.y walks the output rows (indices once per block), threads the columns.
template <typename T, bool F64SCALE>
__global__ void normalize_kernel(const T* __restrict__ raw, T* __restrict__ out, int py, int px, int raw_pitch,
                                 int count, int Hr, int Wr, int Sy, int Sx, double scale, bool rawcopy) {
  const int oy = rawcopy ? py : Sy, ox = rawcopy ? px : Sx;
  const int sx = blockIdx.x * blockDim.x + threadIdx.x;
  if (sx >= ox) return;
  const long long n_rows = (long long)count * oy;
  const T fscale = (T)scale;
  int rx = sx;
  if (!rawcopy) {
    rx = sx - (Wr - 1);
    if (rx < 0) rx += px;
  }
  for (long long row = blockIdx.y; row < n_rows; row += gridDim.y) {
    const int sy = (int)(row % oy);
    const long long m = row / oy;
    int ry = sy;
    if (!rawcopy) {
      ry = sy - (Hr - 1);
      if (ry < 0) ry += py;
    }
    const T v = __ldg(raw + (m * py + ry) * (long long)raw_pitch + rx);
    T* o = out + row * (long long)ox + sx;
    if (rawcopy) *o = v;
    else if (F64SCALE) *o = (T)((double)v * scale);
    else *o = v * fscale;
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
  const int threads = 128;
  const long long n_rows = (long long)count * pad_rows;
  dim3 grid((unsigned)((pad_cols + 4 * threads - 1) / (4 * threads)), (unsigned)std::min<long long>(n_rows, 65535));
  if (dtype == XC_F32)
    pad_kernel<float><<<grid, threads, 0, stream>>>((const float*)src, (float*)dst, rows, cols, count, pad_rows,
                                                    pad_cols, dst_pitch, dst_y, dst_x);
  else
    pad_kernel<double><<<grid, threads, 0, stream>>>((const double*)src, (double*)dst, rows, cols, count, pad_rows,
                                                     pad_cols, dst_pitch, dst_y, dst_x);
  XC_CUDA_TRY(cudaGetLastError());
  return XC_OK;
}

xc_status glue_conj_multiply_pairs(xc_dtype dtype, const void* lspec, const void* rspec, void* out, long long bins,
                                   const PairMap& pm, long long n_out, cudaStream_t stream) {
  if (n_out <= 0 || bins <= 0) return XC_OK;
  const int threads = 256;
  const long long bx = (bins + threads - 1) / threads;
  if (bx > 0x7fffffffLL) return fail(XC_ERR_INVALID_ARGUMENT, "spectrum too large for one launch");
  dim3 grid((unsigned)bx, (unsigned)std::min<long long>(n_out, 65535));
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
  const int threads = 128;
  const int ox = rawcopy ? px : Sx;
  const long long n_rows = (long long)count * (rawcopy ? py : Sy);
  dim3 blocks((unsigned)((ox + threads - 1) / threads), (unsigned)std::min<long long>(n_rows, 65535));
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
