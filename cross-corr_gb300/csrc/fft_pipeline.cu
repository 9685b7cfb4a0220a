// fft_pipeline.cu -- FFT-based correlation of a whole batch:
//   pad (device) -> batched in-place R2C of every left and right matrix ->
//   fused conj-multiply over the mode's pair map -> batched in-place C2R ->
//   device normalisation (or the raw circular result).
//
// Replaces the fft_orig_* / fft_reduced_transfer_* / fft_better_n_to_m
// plug-ins (src/one_to_one.hpp:887-1180, src/one_to_many.hpp:501-801,
// src/n_to_mn.hpp:720-1023, src/n_to_m.hpp:646-787).  cuFFT stays for the
// transforms.  Differences by design:
//  * one R2C plan covers left and right matrices together (the reference
//    plans and runs them separately for n_to_m), in place in the padded
//    layout cuFFT expects (rows of 2*(px/2+1) reals), so the pad kernel writes
//    straight into the transform buffer;
//  * plans are created once per shape and reused (the reference re-plans in
//    every prepare step, which dominates its small-size timings);
//  * normalisation runs on the device instead of the host.
#include <cufft.h>

#include <new>
#include <string>

#include "xc_common.cuh"
#include "xc_internal.h"

namespace xc {

struct FftPlanImpl {
  xc_mode mode;
  xc_dtype dtype;
  Geometry g;
  PairMap pm;
  uint64_t n_out;
  int n_left, n_right;
  int py, px;         // transform size
  int cols_c;         // px/2 + 1 complex columns
  long long bins;     // py * cols_c
  cufftHandle r2c = 0, c2r = 0;
  bool have_r2c = false, have_c2r = false;
  size_t ws_inputs, ws_products;  // bytes
};

namespace {

xc_status cufft_fail(cufftResult r, const char* what) {
  return fail(XC_ERR_CUFFT, std::string(what) + " failed with cufftResult " + std::to_string((int)r));
}

bool smooth(long long n) {
  for (int p : {2, 3, 5, 7})
    while (n % p == 0) n /= p;
  return n == 1;
}

int next_smooth(long long n) {
  while (!smooth(n)) ++n;
  return (int)n;
}

}  // namespace

xc_status fft_plan_create(FftPlanImpl** out, xc_mode mode, xc_dtype dtype, xc_size2 left, uint32_t n_left,
                          xc_size2 right, uint32_t n_right, xc_size2 pad) {
  *out = nullptr;
  FftPlanImpl* p = new (std::nothrow) FftPlanImpl();
  if (p == nullptr) return fail(XC_ERR_CUDA, "host allocation failed");
  p->mode = mode;
  p->dtype = dtype;
  p->g = make_geometry(left, right);
  p->n_left = (int)n_left;
  p->n_right = (int)n_right;
  if (!make_pair_map(mode, n_left, n_right, &p->pm, &p->n_out)) {
    delete p;
    return fail(XC_ERR_INVALID_ARGUMENT, "invalid matrix counts for the mode");
  }
  if (pad.x == 0 && pad.y == 0) {
    if (left.x == right.x && left.y == right.y) {
      // The reference's relative_zero_padding<2> (src/matrix.hpp:33-46).
      p->py = 2 * (int)left.y;
      p->px = 2 * (int)left.x;
    } else {
      p->py = next_smooth(p->g.Sy);
      p->px = next_smooth(p->g.Sx);
    }
  } else {
    p->py = (int)pad.y;
    p->px = (int)pad.x;
  }
  if (p->py < p->g.Sy || p->px < p->g.Sx) {
    delete p;
    return fail(XC_ERR_INVALID_ARGUMENT, "FFT size smaller than the full correlation size");
  }
  p->cols_c = p->px / 2 + 1;
  p->bins = (long long)p->py * p->cols_c;
  const size_t ce = dtype == XC_F32 ? sizeof(float2) : sizeof(double2);
  p->ws_inputs = (size_t)(n_left + n_right) * (size_t)p->bins * ce;
  p->ws_products = (size_t)p->n_out * (size_t)p->bins * ce;

  int n[2] = {p->py, p->px};
  int rembed[2] = {p->py, 2 * p->cols_c};
  int cembed[2] = {p->py, p->cols_c};
  const int rdist = p->py * 2 * p->cols_c, cdist = p->py * p->cols_c;
  cufftResult r = cufftPlanMany(&p->r2c, 2, n, rembed, 1, rdist, cembed, 1, cdist,
                                dtype == XC_F32 ? CUFFT_R2C : CUFFT_D2Z, (int)(n_left + n_right));
  if (r != CUFFT_SUCCESS) {
    delete p;
    return cufft_fail(r, "cufftPlanMany(R2C)");
  }
  p->have_r2c = true;
  r = cufftPlanMany(&p->c2r, 2, n, cembed, 1, cdist, rembed, 1, rdist, dtype == XC_F32 ? CUFFT_C2R : CUFFT_Z2D,
                    (int)p->n_out);
  if (r != CUFFT_SUCCESS) {
    cufftDestroy(p->r2c);
    delete p;
    return cufft_fail(r, "cufftPlanMany(C2R)");
  }
  p->have_c2r = true;
  *out = p;
  return XC_OK;
}

size_t fft_plan_workspace(const FftPlanImpl* p) { return p->ws_inputs + p->ws_products + 256; }

xc_size2 fft_plan_pad(const FftPlanImpl* p) { return xc_size2{(uint32_t)p->px, (uint32_t)p->py}; }

namespace {
struct WsView {
  char* inputs;
  char* products;
};

xc_status ws_view(const FftPlanImpl* p, void* workspace, size_t ws_bytes, WsView* v) {
  if (workspace == nullptr || ws_bytes < fft_plan_workspace(p))
    return fail(XC_ERR_WORKSPACE, "FFT workspace missing or smaller than xc_fft_plan_workspace_size");
  char* ws = reinterpret_cast<char*>(((uintptr_t)workspace + 255) & ~uintptr_t(255));
  v->inputs = ws;
  v->products = ws + p->ws_inputs;
  return XC_OK;
}

size_t input_stride(const FftPlanImpl* p) { return (size_t)p->bins * 2 * (p->dtype == XC_F32 ? 4 : 8); }
}  // namespace

// Stage 1: zero-pad every input straight into the transform layout, then one
// batched forward transform of all inputs.
xc_status fft_plan_forward(FftPlanImpl* p, const void* left, const void* right, void* workspace, size_t ws_bytes,
                           cudaStream_t stream) {
  WsView v;
  XC_TRY(ws_view(p, workspace, ws_bytes, &v));
  const int pitch = 2 * p->cols_c;  // reals per padded row
  XC_TRY(glue_pad_pitched(p->dtype, left, v.inputs, p->g.Hl, p->g.Wl, p->n_left, p->py, p->px, pitch, 0, 0, stream));
  XC_TRY(glue_pad_pitched(p->dtype, right, v.inputs + p->n_left * input_stride(p), p->g.Hr, p->g.Wr, p->n_right,
                          p->py, p->px, pitch, 0, 0, stream));
  cufftResult r = cufftSetStream(p->r2c, stream);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftSetStream");
  if (p->dtype == XC_F32)
    r = cufftExecR2C(p->r2c, (cufftReal*)v.inputs, (cufftComplex*)v.inputs);
  else
    r = cufftExecD2Z(p->r2c, (cufftDoubleReal*)v.inputs, (cufftDoubleComplex*)v.inputs);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftExecR2C");
  return XC_OK;
}

// Stage 2: conj-multiply every output pair.
xc_status fft_plan_multiply(FftPlanImpl* p, void* workspace, size_t ws_bytes, cudaStream_t stream) {
  WsView v;
  XC_TRY(ws_view(p, workspace, ws_bytes, &v));
  return glue_conj_multiply_pairs(p->dtype, v.inputs, v.inputs + p->n_left * input_stride(p), v.products, p->bins,
                                  p->pm, (long long)p->n_out, stream);
}

// Stage 3: batched in-place inverse transform, then normalise (quadrant swap +
// scale + crop) or copy out the raw circular result.
xc_status fft_plan_inverse(FftPlanImpl* p, void* out, int normalize, void* workspace, size_t ws_bytes,
                           cudaStream_t stream) {
  WsView v;
  XC_TRY(ws_view(p, workspace, ws_bytes, &v));
  cufftResult r = cufftSetStream(p->c2r, stream);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftSetStream");
  if (p->dtype == XC_F32)
    r = cufftExecC2R(p->c2r, (cufftComplex*)v.products, (cufftReal*)v.products);
  else
    r = cufftExecZ2D(p->c2r, (cufftDoubleComplex*)v.products, (cufftDoubleReal*)v.products);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftExecC2R");
  return glue_normalize_pitched(p->dtype, v.products, out, p->py, p->px, 2 * p->cols_c, (int)p->n_out, p->g.Hr,
                                p->g.Wr, p->g.Sy, p->g.Sx, normalize == 0, stream);
}

xc_status fft_plan_execute(FftPlanImpl* p, const void* left, const void* right, void* out, int normalize,
                           void* workspace, size_t ws_bytes, cudaStream_t stream) {
  XC_TRY(fft_plan_forward(p, left, right, workspace, ws_bytes, stream));
  XC_TRY(fft_plan_multiply(p, workspace, ws_bytes, stream));
  return fft_plan_inverse(p, out, normalize, workspace, ws_bytes, stream);
}

void fft_plan_destroy(FftPlanImpl* p) {
  if (p == nullptr) return;
  if (p->have_r2c) cufftDestroy(p->r2c);
  if (p->have_c2r) cufftDestroy(p->c2r);
  delete p;
}

}  // namespace xc
