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
// beyond pad_cols is left untouched).  Each thread writes 4 consecutive
// elements of one dst row.
template <typename T>
__global__ void pad_kernel(const T* __restrict__ src, T* __restrict__ dst, int rows, int cols, int count, int pad_rows,
                           int pad_cols, int dst_pitch, int dst_y, int dst_x) {
  const int quads = (pad_cols + 3) / 4;
  const long long total = (long long)count * pad_rows * quads;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(i % quads);
    const long long rowid = i / quads;
    const int y = (int)(rowid % pad_rows);
    const long long m = rowid / pad_rows;
    const int sy = y - dst_y;
    const T* srow = src + (m * rows + sy) * (long long)cols;
    T* drow = dst + (m * pad_rows + y) * (long long)dst_pitch;
    const int x0 = q * 4;
    T v[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int sx = x0 + e - dst_x;
      v[e] = (sy >= 0 && sy < rows && sx >= 0 && sx < cols) ? srow[sx] : T(0);
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

// grid.y = left index l; each thread owns one spectral bin and walks the K
// partners of l.
template <typename C>
__global__ void conj_multiply_kernel(const C* __restrict__ lspec, const C* __restrict__ rspec, C* __restrict__ out,
                                     long long bins, PairMap pm) {
  const int l = blockIdx.y;
  const C* lrow = lspec + (long long)l * bins;
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < bins;
       b += (long long)gridDim.x * blockDim.x) {
    const C lv = lrow[b];
    for (int k = 0; k < pm.K; ++k) {
      const long long r = (long long)l * pm.r_l + (long long)k * pm.r_k;
      const long long o = (long long)l * pm.o_l + (long long)k * pm.o_k;
      out[o * bins + b] = mul_conj(lv, __ldg(rspec + r * bins + b));
    }
  }
}

// out[m][sy][sx] = raw[m][(sy - (Hr-1)) mod py][(sx - (Wr-1)) mod px] * scale;
// with raw=true it instead copies raw[m][y][x] (dense py x px output).
template <typename T, bool F64SCALE>
__global__ void normalize_kernel(const T* __restrict__ raw, T* __restrict__ out, int py, int px, int raw_pitch,
                                 int count, int Hr, int Wr, int Sy, int Sx, double scale, bool rawcopy) {
  const int oy = rawcopy ? py : Sy, ox = rawcopy ? px : Sx;
  const long long total = (long long)count * oy * ox;
  const T fscale = (T)scale;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int sx = (int)(i % ox);
    const long long t = i / ox;
    const int sy = (int)(t % oy);
    const long long m = t / oy;
    int ry = sy, rx = sx;
    if (!rawcopy) {
      ry = sy - (Hr - 1);
      rx = sx - (Wr - 1);
      if (ry < 0) ry += py;
      if (rx < 0) rx += px;
    }
    const T v = raw[(m * py + ry) * (long long)raw_pitch + rx];
    if (rawcopy) out[i] = v;
    else if (F64SCALE) out[i] = (T)((double)v * scale);
    else out[i] = v * fscale;
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
  const long long work = (long long)count * pad_rows * ((pad_cols + 3) / 4);
  const int threads = 256;
  const int blocks = grid_for(work, threads);
  if (dtype == XC_F32)
    pad_kernel<float><<<blocks, threads, 0, stream>>>((const float*)src, (float*)dst, rows, cols, count, pad_rows,
                                                      pad_cols, dst_pitch, dst_y, dst_x);
  else
    pad_kernel<double><<<blocks, threads, 0, stream>>>((const double*)src, (double*)dst, rows, cols, count, pad_rows,
                                                       pad_cols, dst_pitch, dst_y, dst_x);
  XC_CUDA_TRY(cudaGetLastError());
  return XC_OK;
}

xc_status glue_conj_multiply_pairs(xc_dtype dtype, const void* lspec, const void* rspec, void* out, long long bins,
                                   const PairMap& pm, long long n_out, cudaStream_t stream) {
  (void)n_out;
  const int threads = 256;
  long long bx = (bins + threads - 1) / threads;
  const long long cap = (152LL * 32 + pm.n_left - 1) / pm.n_left;
  if (bx > cap) bx = cap;
  if (bx < 1) bx = 1;
  if (pm.n_left > 65535) return fail(XC_ERR_INVALID_ARGUMENT, "too many left matrices for one launch");
  dim3 grid((unsigned)bx, (unsigned)pm.n_left);
  if (dtype == XC_F32)
    conj_multiply_kernel<float2><<<grid, threads, 0, stream>>>((const float2*)lspec, (const float2*)rspec,
                                                               (float2*)out, bins, pm);
  else
    conj_multiply_kernel<double2><<<grid, threads, 0, stream>>>((const double2*)lspec, (const double2*)rspec,
                                                                (double2*)out, bins, pm);
  XC_CUDA_TRY(cudaGetLastError());
  return XC_OK;
}

xc_status glue_normalize_pitched(xc_dtype dtype, const void* raw, void* out, int py, int px, int raw_pitch, int count,
                                 int Hr, int Wr, int Sy, int Sx, bool rawcopy, cudaStream_t stream) {
  if (count <= 0) return XC_OK;
  const long long work = (long long)count * (rawcopy ? (long long)py * px : (long long)Sy * Sx);
  const int threads = 256;
  const int blocks = grid_for(work, threads);
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
