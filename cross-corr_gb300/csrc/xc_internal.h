// xc_internal.h -- C++ interfaces shared between the library's translation
// units (not part of the public C ABI).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "xcorr.h"

namespace xc {

// Mapping of (left l, k-th partner of l) to output and right indices:
//   output o(l,k) = l*o_l + k*o_k,  right r(l,k) = l*r_l + k*r_k,  k < K.
// one_to_one/one_to_many: (0,1,0,1); n_to_mn: (1,n,1,n); n_to_m: (M,1,0,1)
// (src/validate.hpp:216-298).
struct PairMap {
  int n_left;
  int K;
  long long o_l, o_k, r_l, r_k;
};

bool make_pair_map(xc_mode mode, uint32_t n_left, uint32_t n_right, PairMap* pm, uint64_t* n_out);

struct Geometry {
  int Hl, Wl, Hr, Wr;  // left and right matrix sizes
  int Sy, Sx;          // output size
};

inline Geometry make_geometry(xc_size2 left, xc_size2 right) {
  Geometry g;
  g.Hl = (int)left.y;
  g.Wl = (int)left.x;
  g.Hr = (int)right.y;
  g.Wr = (int)right.x;
  g.Sy = g.Hl + g.Hr - 1;
  g.Sx = g.Wl + g.Wr - 1;
  return g;
}

xc_status debug_expire_wait(uint32_t polls, cudaStream_t stream);

// Optional CUDA-event timing of the dense kernels (xc_kernel_timing).
// kernel_timer_begin returns a slot (or -1 when timing is off) that
// kernel_timer_end closes after the launch on the same stream.
int kernel_timer_begin(cudaStream_t stream);
void kernel_timer_end(int slot, cudaStream_t stream);
xc_status kernel_timing(int enable);
xc_status kernel_timing_read(double* total_ms, uint32_t* launches);

// Plain definition-based correlation (direct_simt.cu).  How results reach
// the output:
//  kAuto   - the output is written; under-filled launches split each tile's
//            rows over several CTAs, which zero the output first and add;
//  kCaller - always added into the output, which the caller zeroed (the
//            reference's work-distribution launchers, src/one_to_one.hpp:276-277);
//  kNever  - written, never split (studies and tests of the unsplit kernel).
enum class DirectAccumulate { kAuto = 0, kCaller = 1, kNever = 2 };
xc_status direct_launch(xc_dtype dtype, const void* left, const void* right, void* out, const Geometry& g,
                        const PairMap& pm, cudaStream_t stream, int force_loader /* -1 auto, 0 cp.async, 1 TMA */,
                        DirectAccumulate acc = DirectAccumulate::kAuto, int tile = 0);

// Ragged batches (ragged.cu drives direct_simt.cu's persistent mode).
struct RaggedTile {     // one tile of shifts of one pair
  int pair;
  int sy0, sx0;
};
struct RaggedPairDev {  // a pair, with offsets into the padded copies
  int left, right;
  int Hl, Wl, Hr, Wr;
  long long out_off;    // element offset of the output in the caller's buffer
};
struct RaggedLaunch {
  const void* left;     // unused by the TMA path; kept for symmetry
  const void* right;
  void* out;
  const RaggedTile* tiles;
  const RaggedPairDev* pairs;
  const CUtensorMap* lmaps;
  const CUtensorMap* rmaps;
  unsigned int* queue;
  int n_tiles;
  int grid;
};
struct RaggedShape {    // a tile shape the ragged kernel can run with
  int bsy, bsx, lw, xc, vec, threads, smem;
  const void* kernel;
};
int ragged_shape_count(xc_dtype dtype);
RaggedShape ragged_shape(xc_dtype dtype, int index);
xc_status ragged_launch(xc_dtype dtype, int index, const RaggedLaunch& rl, cudaStream_t stream);
struct RaggedPlanImpl;
xc_status ragged_plan_create(RaggedPlanImpl** plan, xc_dtype dtype, const void* d_left, const xc_matrix_desc* lefts,
                             uint32_t n_left, const void* d_right, const xc_matrix_desc* rights, uint32_t n_right,
                             const xc_pair_desc* pairs, uint32_t n_pairs, void* d_out);
xc_status ragged_execute(RaggedPlanImpl* plan, cudaStream_t stream);
xc_status ragged_autotune(RaggedPlanImpl* plan, cudaStream_t stream, int* chosen, double* best_ms);
xc_status ragged_describe(RaggedPlanImpl* plan, int variant, xc_ragged_variant* out);
xc_status ragged_select(RaggedPlanImpl* plan, int variant);
void ragged_plan_destroy(RaggedPlanImpl* plan);
xc_status correlate_pairs(xc_dtype dtype, const void* d_left, const xc_matrix_desc* lefts, uint32_t n_left,
                          const void* d_right, const xc_matrix_desc* rights, uint32_t n_right,
                          const xc_pair_desc* pairs, uint32_t n_pairs, void* d_out, cudaStream_t stream);

// Selector network (mlp.cu).
xc_status mlp_forward(const float* params, const float* x, uint32_t n, float* y, cudaStream_t stream);
xc_status mlp_gradient(const float* params, const float* x, const float* target, const float* mask, uint32_t n,
                       float mask_count, float* grad, float* loss, cudaStream_t stream);
xc_status mlp_adam(float* params, const float* grad, float* m, float* v, uint32_t step, float lr,
                   cudaStream_t stream);

// FFT pipeline (fft_pipeline.cu).
struct FftPlanImpl;
xc_status fft_plan_create(FftPlanImpl** plan, xc_mode mode, xc_dtype dtype, xc_size2 left, uint32_t n_left,
                          xc_size2 right, uint32_t n_right, xc_size2 pad);
size_t fft_plan_workspace(const FftPlanImpl* plan);
xc_size2 fft_plan_pad(const FftPlanImpl* plan);
xc_status fft_plan_execute(FftPlanImpl* plan, const void* left, const void* right, void* out, int normalize,
                           void* workspace, size_t ws_bytes, cudaStream_t stream);
xc_status fft_plan_forward(FftPlanImpl* plan, const void* left, const void* right, void* workspace, size_t ws_bytes,
                           cudaStream_t stream);
xc_status fft_plan_multiply(FftPlanImpl* plan, void* workspace, size_t ws_bytes, cudaStream_t stream);
xc_status fft_plan_inverse(FftPlanImpl* plan, void* out, int normalize, void* workspace, size_t ws_bytes,
                           cudaStream_t stream);
void fft_plan_destroy(FftPlanImpl* plan);

// FFT glue kernels (fft_glue.cu).
xc_status glue_pad(xc_dtype dtype, const void* src, void* dst, int rows, int cols, int count, int pad_rows,
                   int pad_cols, int dst_y, int dst_x, cudaStream_t stream);
xc_status glue_pad_pitched(xc_dtype dtype, const void* src, void* dst, int rows, int cols, int count, int pad_rows,
                           int pad_cols, int dst_pitch, int dst_y, int dst_x, cudaStream_t stream);
xc_status glue_normalize_pitched(xc_dtype dtype, const void* raw, void* out, int py, int px, int raw_pitch, int count,
                                 int Hr, int Wr, int Sy, int Sx, bool rawcopy, cudaStream_t stream);
xc_status glue_conj_multiply_pairs(xc_dtype dtype, const void* lspec, const void* rspec, void* out, long long bins,
                                   const PairMap& pm, long long n_out, cudaStream_t stream);
xc_status glue_normalize(xc_dtype dtype, const void* raw, void* out, int py, int px, int count, int Hr, int Wr,
                         int Sy, int Sx, cudaStream_t stream);
xc_status glue_hadamard_original(xc_dtype dtype, const void* ref, void* deformed, long long area_per_pic,
                                 long long batch, int threads, cudaStream_t stream);
xc_status glue_hadamard_n_to_m(xc_dtype dtype, const void* left, const void* right, void* out, long long area,
                               int n_left, int n_right, cudaStream_t stream);

// Output row bands of the split tensor-core path.  With `band_done` (device,
// one int per band) the kernel counts each band's finished work items there;
// `bands` receives the bands' expected counts and output row ranges, so a
// copy can wait for a band and take its rows while the kernel runs on.
struct TcBands {
  int n;
  long long items[8];
  int row_lo[8], row_hi[8];
  int order[8];  // bands in the order the kernel works (and completes) them
};
xc_status tc_correlate_banded(const float* left, const float* right, float* out, const Geometry& g,
                              const PairMap& pm, void* workspace, size_t ws_bytes, cudaStream_t stream, bool tf32,
                              int want_bands, int* band_done, TcBands* bands, int max_rows = 64,
                              int min_rows = 4);

// Split tensor-core paths (tc_bf16x3.cu): one launch sequence per problem on
// `stream` (no host synchronisation, so it can be captured into a graph).
// Work items take between min_rows and max_rows left rows: as few as give two
// items per SM, within those bounds.
xc_status tc_correlate(const float* left, const float* right, float* out, const Geometry& g, const PairMap& pm,
                       void* workspace, size_t ws_bytes, cudaStream_t stream, bool tf32, int max_rows = 64,
                       int min_rows = 4);
// Workspace bytes of a problem; 0 when the split paths do not take it.
size_t tc_workspace_size(const Geometry& g, const PairMap& pm, bool tf32);
// Raises the kernels' shared-memory limits for a problem (what tc_correlate
// would otherwise do on its first call): call it before capturing
// tc_correlate into a graph.
xc_status tc_prepare(const Geometry& g, const PairMap& pm, bool tf32);

}  // namespace xc
