/*
 * xcorr.h -- C ABI of the GB300 (sm_103a) batched 2D cross-correlation library.
 *
 * Drop-in boundary for the hot path of MK4H/cross-corr: the definition-based
 * warp-shuffle algorithms (`nai_shuffle_*`) and the FFT algorithms (`fft_*`).
 * The reference has no FFI; its embeddable interface is the C++ kernel-launch
 * layer in src/kernels.cuh (what its sample_app calls) plus the per-algorithm
 * plug-in classes (src/cross_corr.hpp).  Every function below names the
 * reference interface it replaces.
 *
 * Conventions
 *  - Plain pointers and sizes only; no C++ or torch types cross this ABI.
 *  - Device buffers are owned by the caller (as in the reference's
 *    prepare_impl, src/one_to_one.hpp:112-118).  Launch-level calls allocate
 *    nothing and never synchronise; they enqueue on `stream` (a cudaStream_t,
 *    NULL = legacy default stream).
 *  - Matrices are row-major, stacked contiguously ("# rows,cols,count" CSV
 *    order, src/matrix.hpp:94-185).  A size2 is {x = columns, y = rows}, the
 *    reference's dsize2_t (src/types.cuh:12-156).
 *  - Output of one pair: (Hl+Hr-1) x (Wl+Wr-1), element
 *      out[sy + Hr-1][sx + Wr-1] = sum_{y,x} L[y+sy][x+sx] * R[y][x],
 *    the reference's shift order (src/validate.hpp:117-132) generalised to
 *    unequal left/right sizes.
 *  - Result order of the modes follows src/validate.hpp:216-298:
 *      one_to_one : 1 left, 1 right                 -> 1 output
 *      one_to_many: 1 left, M right                 -> output i = (left 0, right i)
 *      n_to_mn    : n left, m*n right               -> output i = (left i mod n, right i)
 *      n_to_m     : n left, M right                 -> output l*M + r = (left l, right r)
 *  - Errors never abort: a status is returned and xc_last_error() holds a
 *    message for the calling thread.
 */
#ifndef XCORR_GB300_H
#define XCORR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum xc_status {
  XC_OK = 0,
  XC_ERR_INVALID_ARGUMENT = 1, /* bad sizes/counts/pointers: the reference's argument_error (exit 1) */
  XC_ERR_CUDA = 2,             /* CUDA runtime error: the reference's exit-3 path (src/main.cpp:268-275) */
  XC_ERR_CUFFT = 3,            /* cuFFT error: the reference's FFTCH throw (src/fft_helpers.hpp:67-76) */
  XC_ERR_UNSUPPORTED = 4,      /* valid request this build does not implement (e.g. FP64 tensor path) */
  XC_ERR_WORKSPACE = 5,        /* workspace too small or missing */
  XC_ERR_TIMEOUT = 6           /* a bounded device-side wait expired; the context stays usable */
} xc_status;

typedef enum xc_mode { XC_ONE_TO_ONE = 0, XC_ONE_TO_MANY = 1, XC_N_TO_MN = 2, XC_N_TO_M = 3 } xc_mode;

typedef enum xc_dtype { XC_F32 = 0, XC_F64 = 1 } xc_dtype;

typedef enum xc_method {
  XC_METHOD_AUTO = 0,     /* library choice */
  XC_METHOD_DIRECT = 1,   /* plain definition-based kernel (FP32 or FP64 FMA, TMA-staged) */
  XC_METHOD_FFT = 2,      /* cuFFT transforms + fused pad / conj-multiply / normalise kernels */
  XC_METHOD_TC_BF16X3 = 3, /* split-BF16 (3 products) tcgen05 tensor-core implicit GEMM, FP32 only */
  XC_METHOD_TC_TF32X3 = 4  /* the same with split-TF32 operands (kind::tf32): more accurate, half the rate */
} xc_method;

/* An algorithm: a method and one of its tile configurations.  Tiles: the
 * plain kernel 0 (its default: 8 partners per CTA when there are 4 or more,
 * else one), 1 (8 partners, 32 x 64 shifts; FP64: 4), 2 (one partner,
 * 64 x 64 shifts; FP64: 32 x 64), 3 (one partner, 32 x 64 shifts); the FFT
 * path 0; the split tensor-core paths 0 (items of at most 64 left rows) or
 * the item length cap, 4 to 1024.  The reference names algorithm and tile
 * arguments by hand (src/main.cpp:361-411, the JSON tile arguments of each
 * plug-in). */
typedef struct xc_algo {
  xc_method method;
  int32_t tile;
} xc_algo;

typedef struct xc_size2 {
  uint32_t x; /* columns */
  uint32_t y; /* rows */
} xc_size2;

/* ------------------------------------------------------------------------ */
/* Library information                                                      */
/* ------------------------------------------------------------------------ */
const char* xc_version(void);
const char* xc_status_string(xc_status status);
/* Message of the last failed call on this thread ("" if none). */
const char* xc_last_error(void);
/* Device compute capability check: XC_OK only on an sm_103 device. */
xc_status xc_device_check(int device);
/* Synchronises `stream`, then reports XC_ERR_TIMEOUT if a bounded device-side
 * wait of an earlier launch on this device gave up (and clears that record).
 * The reference has no device-side waits; it surfaces asynchronous errors
 * the same way, after a synchronisation (src/main.cpp:268-275). */
xc_status xc_check_device(void* stream);
/* Test hook for the bounded waits (new, no reference counterpart): launches
 * one block that waits on a shared-memory mbarrier nothing completes, gives up
 * after `polls` polls, records the expiry and returns.  No fault, no hang. */
xc_status xc_debug_expire_wait(uint32_t polls, void* stream);
/* Kernel timing (new, no reference counterpart; the reference times whole
 * steps with its stopwatch, src/stopwatch.hpp:57-71).  While enabled, every
 * launch of a dense correlation kernel (the plain kernel and the split-BF16
 * tensor kernel; not the ragged plan, which runs as a captured graph) is
 * bracketed by CUDA events on its own stream.  xc_kernel_timing_read waits
 * for the recorded events and returns the summed kernel time and the launch
 * count since the last enable.  Enabling clears the record; the record is
 * process-wide. */
xc_status xc_kernel_timing(int enable);
xc_status xc_kernel_timing_read(double* total_ms, uint32_t* launches);

/* ------------------------------------------------------------------------ */
/* Geometry (src/validate.hpp:190-214 result_matrix_size / counts)          */
/* ------------------------------------------------------------------------ */
/* Number of result matrices of `mode`; replaces check_num_result_matrices and
 * the *_validate_input_size predicates (src/one_to_one.hpp:20-22,
 * src/one_to_many.hpp:15-17, src/n_to_mn.hpp:23-25, src/n_to_m.hpp:19-21). */
xc_status xc_output_count(xc_mode mode, uint32_t n_left, uint32_t n_right, uint64_t* n_out);
/* (Hl+Hr-1) x (Wl+Wr-1); replaces result_matrix_size (src/validate.hpp:190). */
xc_status xc_output_size(xc_size2 left, xc_size2 right, xc_size2* out);

/* ------------------------------------------------------------------------ */
/* Batched correlation on caller-owned device buffers.                      */
/* Replaces the run_impl step of every cross_corr_alg plug-in               */
/* (src/cross_corr.hpp:145, e.g. src/one_to_one.hpp:196-207,                */
/* src/one_to_many.hpp:571-587, src/n_to_m.hpp:198-212).                    */
/* ------------------------------------------------------------------------ */
/* Bytes of device workspace xc_correlate needs (0 for XC_METHOD_DIRECT). */
xc_status xc_workspace_size(xc_mode mode, xc_dtype dtype, xc_method method, xc_size2 left, uint32_t n_left,
                            xc_size2 right, uint32_t n_right, size_t* bytes);
/* Correlates all pairs of `mode`.  `d_left` holds n_left matrices of size
 * `left`, `d_right` n_right of size `right`, `d_out` receives the outputs in
 * the mode's order, normalised (FFT results are quadrant-swapped and divided
 * by the transform size on the device).  The FFT method keeps a per-thread
 * cache of cuFFT plans: its first call for a shape creates (allocates) plans;
 * create them explicitly with xc_fft_plan_create to keep allocation out of
 * timed or captured regions. */
xc_status xc_correlate(xc_mode mode, xc_dtype dtype, xc_method method, const void* d_left, xc_size2 left,
                       uint32_t n_left, const void* d_right, xc_size2 right, uint32_t n_right, void* d_out,
                       void* d_workspace, size_t workspace_bytes, void* stream);

/* Host buffers in and out: allocation, host->device copy, correlation,
 * device->host copy and free, i.e. the reference's whole
 * prepare/transfer/run/finalize/free sequence (src/main.cpp:123-174).
 * Synchronises `stream` before returning. Device buffers are cached per
 * thread between calls of the same size.  Host buffers should be pinned for
 * copies to overlap computation.
 *  - The split tensor-core methods (FP32, from 16 MiB of output) copy the
 *    output out in up to eight row bands while their one kernel runs: the
 *    kernel counts each band's finished work in device memory and the copy
 *    stream waits on the count.  Their pieces of work are cut per band, so
 *    the result may differ from xc_correlate's by a few FP32 roundings of
 *    the partial sums (both stay within 1e-5 of max|out| of the exact
 *    result).
 *  - Otherwise problems run in one chunk of partners (left matrices in
 *    n_to_m) per 192 MiB of output, up to four, each chunk's copy-in,
 *    correlation and copy-out on its own stream so that copies overlap the
 *    neighbouring chunks' correlations; with XC_METHOD_AUTO each chunk picks
 *    its own method. */
xc_status xc_correlate_host(xc_mode mode, xc_dtype dtype, xc_method method, const void* h_left, xc_size2 left,
                            uint32_t n_left, const void* h_right, xc_size2 right, uint32_t n_right, void* h_out,
                            void* stream);
/* xc_correlate_host for a stream of independent problems (new; the
 * reference runs one problem per process, src/main.cpp:123-174): enqueues
 * the call's copy-in, correlation (on `stream`) and copy-out, returns at
 * once and names the call in *ticket.  Two calls per thread are in flight:
 * the next call's copy-in runs while this one's kernel does, and this one's
 * copy-out (after its kernel, not in row bands) runs under the next one's
 * kernel.  A call first waits for
 * the call two tickets back (and returns its error, enqueueing nothing, if
 * that call failed unwaited).  Unlike xc_correlate_host, the copies do not
 * wait for work already queued on `stream`: the host inputs must be ready
 * when the call is made.  h_left, h_right and h_out must stay valid, and
 * h_out unread, until xc_host_wait(ticket) returns; pinned host buffers
 * let the copies run asynchronously.  Problems cut into chunks (192 MiB of
 * output or more) run to completion before the call returns.  Tickets
 * belong to the calling thread. */
xc_status xc_correlate_host_async(xc_mode mode, xc_dtype dtype, xc_method method, const void* h_left,
                                  xc_size2 left, uint32_t n_left, const void* h_right, xc_size2 right,
                                  uint32_t n_right, void* h_out, void* stream, uint64_t* ticket);
/* Blocks until the call `ticket` has its output in h_out; its status (a
 * bounded device wait that expired reports XC_ERR_TIMEOUT).  Waiting again,
 * or for a call whose slot a later call has reused, returns XC_OK. */
xc_status xc_host_wait(uint64_t ticket);
/* Releases the calling thread's cached buffers and plans (after the calls
 * in flight complete). */
void xc_release_thread_cache(void);

/* ------------------------------------------------------------------------ */
/* Allocation-free split-BF16 correlation.  No counterpart in the reference. */
/* ------------------------------------------------------------------------ */
/* Size of the fixed scratch array xc_correlate_tc_noalloc works in (64 MiB).
 * Every GPU that loads this library holds it until the process exits. */
#define XC_TC_NOALLOC_SCRATCH_BYTES (64u * 1024u * 1024u)
/* Same result as xc_correlate(mode, XC_F32, XC_METHOD_TC_BF16X3, ...), for
 * callers that must not allocate device memory: hosts that own the device
 * memory budget (a fixed arena or their own pool, no raw cudaMalloc) and
 * latency-critical loops where cudaMalloc/cudaFree may block or synchronise
 * the device.  Instead of a caller workspace it uses one file-scope device
 * array of XC_TC_NOALLOC_SCRATCH_BYTES per GPU; it calls no cudaMalloc,
 * cudaFree or allocating library routine.
 *  - The first call on a device looks up that array's device address (with
 *    the device current) and caches it for that device's context; make that
 *    first call before any stream capture.  After cudaDeviceReset the next
 *    call looks the address up again (the new context's array is new).
 *  - Problems whose scratch exceeds the array are rejected with
 *    XC_ERR_WORKSPACE and a message giving both sizes.  (The 256x256 x 64
 *    one_to_many problem needs about 51 MB.)
 *  - All calls on a device share the array and nothing in it needs to start
 *    at zero; calls whose work overlaps on the GPU (different streams, or
 *    different host threads on one device) race on it and must be ordered by
 *    the caller. */
xc_status xc_correlate_tc_noalloc(xc_mode mode, const float* d_left, xc_size2 left, uint32_t n_left,
                                  const float* d_right, xc_size2 right, uint32_t n_right, float* d_out,
                                  void* stream);

/* ------------------------------------------------------------------------ */
/* FFT pipeline with explicit plans (replaces the cufftPlanMany/exec calls  */
/* and the host-side normalisation of the fft_* plug-ins:                   */
/* src/one_to_one.hpp:925-990, src/one_to_many.hpp:538-587,                 */
/* src/n_to_m.hpp:700-745, src/fft_helpers.hpp:193-261).                    */
/* ------------------------------------------------------------------------ */
typedef struct xc_fft_plan_s* xc_fft_plan;
/* `pad` = transform size; {0,0} selects the reference's 2H x 2W for equal
 * sizes and the smallest 2^a3^b5^c7^d size >= H+Hr-1 otherwise. */
xc_status xc_fft_plan_create(xc_fft_plan* plan, xc_mode mode, xc_dtype dtype, xc_size2 left, uint32_t n_left,
                             xc_size2 right, uint32_t n_right, xc_size2 pad);
xc_status xc_fft_plan_workspace_size(xc_fft_plan plan, size_t* bytes);
xc_status xc_fft_plan_pad_size(xc_fft_plan plan, xc_size2* pad);
/* normalize != 0: normalised (Hl+Hr-1)x(Wl+Wr-1) outputs.  normalize == 0:
 * the raw, unnormalised pad.y x pad.x circular correlations the reference's
 * fft_* algorithms store without -n (src/fft_alg.hpp:13-20). */
xc_status xc_fft_execute(xc_fft_plan plan, const void* d_left, const void* d_right, void* d_out, int normalize,
                         void* d_workspace, size_t workspace_bytes, void* stream);
/* The three stages of xc_fft_execute, for per-step timing (the reference's
 * "Forward FFT" / "Hadamard" / "Inverse FFT" measurements,
 * src/one_to_one.hpp:967-990).  They communicate through the workspace. */
xc_status xc_fft_forward(xc_fft_plan plan, const void* d_left, const void* d_right, void* d_workspace,
                         size_t workspace_bytes, void* stream);
xc_status xc_fft_multiply(xc_fft_plan plan, void* d_workspace, size_t workspace_bytes, void* stream);
xc_status xc_fft_inverse(xc_fft_plan plan, void* d_out, int normalize, void* d_workspace, size_t workspace_bytes,
                         void* stream);
xc_status xc_fft_plan_destroy(xc_fft_plan plan);

/* ------------------------------------------------------------------------ */
/* Ragged batches: pairs of matrices of arbitrary, different sizes (new; the */
/* reference correlates equal sizes only, src/cross_corr.hpp:121-130).      */
/* ------------------------------------------------------------------------ */
typedef struct xc_matrix_desc {
  uint64_t offset; /* elements from the base pointer to the matrix */
  uint32_t rows;
  uint32_t cols;
} xc_matrix_desc;
typedef struct xc_pair_desc {
  uint32_t left;       /* index into the left descriptors */
  uint32_t right;      /* index into the right descriptors */
  uint64_t out_offset; /* elements from the output base to this pair's (Hl+Hr-1)x(Wl+Wr-1) result */
} xc_pair_desc;
typedef struct xc_ragged_plan_s* xc_ragged_plan;
/* Binds the buffers and prepares padded copies, per-matrix tensor maps and a
 * work-sorted tile queue, and captures the step (repack, queue reset, one
 * persistent launch of the plain kernel) into a CUDA graph.  Allocates. */
xc_status xc_ragged_plan_create(xc_ragged_plan* plan, xc_dtype dtype, const void* d_left,
                                const xc_matrix_desc* lefts, uint32_t n_left, const void* d_right,
                                const xc_matrix_desc* rights, uint32_t n_right, const xc_pair_desc* pairs,
                                uint32_t n_pairs, void* d_out);
/* A plan's variants: a tile shape of the plain kernel and, for FP32 plans, a
 * route.  Variant index = tile_shape + (tile shapes) x route.  Route 0 keeps
 * every pair on the plain kernel; routes 1-4 run the pairs with at least
 * 2^32, 2^30, 2^28, 2^26 multiply-adds (that the split path takes) as
 * one_to_one calls of the split-BF16 tensor-core path, on eight side streams
 * captured into the same graph beside the plain kernel's launch (those
 * pairs' outputs then carry the split path's error, up to about 1e-5 of
 * max|out| on zero-mean data).  XC_RAGGED_TC=0 in the environment leaves FP32
 * plans with route 0 only.  Variant 0 runs until another is chosen. */
typedef struct xc_ragged_variant {
  int32_t index;        /* the variant described */
  int32_t n_variants;   /* variants of this plan */
  int32_t tile_shape;   /* plain-kernel tile shape of the pairs left on the plain kernel */
  uint32_t tc_pairs;    /* pairs run on the split-BF16 path */
  uint64_t tc_min_macs; /* ... those with at least this many multiply-adds (0: none) */
} xc_ragged_variant;
/* Times every tile shape with route 0, then every route with the best shape,
 * on the plan's batch, and keeps the fastest variant (`chosen_shape` receives
 * its index); decisions are cached by batch signature in $XC_AUTOTUNE_CACHE
 * (default ~/.cache/xcorr_gb300_autotune.jsonl).  best_ms < 0 when taken from
 * the cache. */
xc_status xc_ragged_autotune(xc_ragged_plan plan, void* stream, int* chosen_shape, double* best_ms);
/* Describes variant `variant` (-1: the chosen one). */
xc_status xc_ragged_describe(xc_ragged_plan plan, int variant, xc_ragged_variant* out);
/* Chooses a variant (builds its graph now; allocates for the first split-path route). */
xc_status xc_ragged_select(xc_ragged_plan plan, int variant);
/* Replays the chosen variant's graph on `stream`. */
xc_status xc_ragged_execute(xc_ragged_plan plan, void* stream);
xc_status xc_ragged_plan_destroy(xc_ragged_plan plan);
/* The same batch as one launch of the plain kernel per pair (baseline). */
xc_status xc_correlate_pairs(xc_dtype dtype, const void* d_left, const xc_matrix_desc* lefts, uint32_t n_left,
                             const void* d_right, const xc_matrix_desc* rights, uint32_t n_right,
                             const xc_pair_desc* pairs, uint32_t n_pairs, void* d_out, void* stream);

/* ------------------------------------------------------------------------ */
/* Method selector (new; the reference picks algorithms and tiles by hand,  */
/* benchmarking/args_test/*.yml): a 3-layer 64-wide FP32 MLP predicting the */
/* log run time of each candidate algorithm (method and tile), trained on   */
/* timings measured on this GPU.                                            */
/* ------------------------------------------------------------------------ */
#define XC_MLP_IN 8
#define XC_MLP_HIDDEN 64
#define XC_MLP_OUT 7 /* one per selector candidate (xc_algorithm) */
#define XC_N_ALGOS 7
#define XC_MLP_PARAMS                                                                                       \
  (XC_MLP_HIDDEN * XC_MLP_IN + XC_MLP_HIDDEN + XC_MLP_HIDDEN * XC_MLP_HIDDEN + XC_MLP_HIDDEN +            \
   XC_MLP_OUT * XC_MLP_HIDDEN + XC_MLP_OUT)
/* The 8 selector features of a problem: log2 of the left area, right area,
 * output count and multiply-accumulate count (scaled to ~[0,1]) and the mode
 * one-hot. */
xc_status xc_selector_features(xc_mode mode, xc_size2 left, uint32_t n_left, xc_size2 right, uint32_t n_right,
                               float* features);
/* Batched inference: y[n][3] = MLP(x[n][8]) on the device. */
xc_status xc_mlp_forward(const float* d_params, const float* d_x, uint32_t n, float* d_y, void* stream);
/* Gradient of the masked mean-squared error
 *   loss = sum_{s,o} mask[s][o] (y[s][o] - target[s][o])^2 / mask_count
 * with respect to the parameters, into d_grad (XC_MLP_PARAMS floats), and the
 * loss into d_loss (1 float). */
xc_status xc_mlp_gradient(const float* d_params, const float* d_x, const float* d_target, const float* d_mask,
                          uint32_t n, float mask_count, float* d_grad, float* d_loss, void* stream);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8, bias-corrected; step >= 1). */
xc_status xc_mlp_adam_step(float* d_params, const float* d_grad, float* d_m, float* d_v, uint32_t step, float lr,
                           void* stream);
/* Installs trained weights (host copy of XC_MLP_PARAMS floats) for
 * XC_METHOD_AUTO; NULL uninstalls them.  The library starts with the
 * network trained on its own GB300 timings installed. */
xc_status xc_selector_load(const float* h_params);
/* Reinstalls that built-in network (XC_ERR_UNSUPPORTED if the library was
 * built without one). */
xc_status xc_selector_load_builtin(void);
/* The selector's candidates (the network's outputs, in order): index
 * 0-2 the plain kernel's tiles 1-3, 3 the FFT path, 4-5 split-BF16 with
 * items of at most 32 and 64 left rows, 6 split-TF32. */
xc_status xc_algorithm(uint32_t index, xc_algo* algo);
/* The algorithm XC_METHOD_AUTO runs for a problem: the network's fastest
 * prediction among the candidates that support it; without weights, the
 * candidate xc_autotune_algorithm last measured fastest for this problem;
 * with neither, {XC_METHOD_AUTO, 0}: xc_correlate's first call for the
 * problem then runs the exhaustive autotune on its own buffers (allocating
 * temporary workspaces and synchronising its stream) and remembers the
 * result. */
xc_status xc_select_algorithm(xc_mode mode, xc_dtype dtype, xc_size2 left, uint32_t n_left, xc_size2 right,
                              uint32_t n_right, xc_algo* algo);
/* The method of xc_select_algorithm's choice. */
xc_status xc_select_method(xc_mode mode, xc_dtype dtype, xc_size2 left, uint32_t n_left, xc_size2 right,
                           uint32_t n_right, xc_method* method);
/* xc_correlate with a given algorithm (method and tile); {XC_METHOD_AUTO, *}
 * is xc_correlate's automatic choice.  The workspace is the method's
 * (xc_workspace_size). */
xc_status xc_correlate_algo(xc_mode mode, xc_dtype dtype, xc_algo algo, const void* d_left, xc_size2 left,
                            uint32_t n_left, const void* d_right, xc_size2 right, uint32_t n_right, void* d_out,
                            void* d_workspace, size_t workspace_bytes, void* stream);
/* Time of one correlation with `algo`: one warm-up call, then `reps` calls
 * back to back between CUDA events on `stream` (synchronised); *ms is the
 * mean.  The timing the selector's dataset is measured with (no per-call
 * overhead of a binding inside the timed region). */
xc_status xc_time_algorithm(xc_mode mode, xc_dtype dtype, xc_algo algo, const void* d_left, xc_size2 left,
                            uint32_t n_left, const void* d_right, xc_size2 right, uint32_t n_right, void* d_out,
                            void* d_workspace, size_t workspace_bytes, uint32_t reps, void* stream, double* ms);
/* Exhaustive autotune (the selector's fallback and judge): times every
 * candidate that supports the problem on the given device buffers
 * (xc_time_algorithm, 3 calls each, workspaces allocated for the run),
 * remembers the fastest for this problem and returns it with its time. */
xc_status xc_autotune_algorithm(xc_mode mode, xc_dtype dtype, const void* d_left, xc_size2 left, uint32_t n_left,
                                const void* d_right, xc_size2 right, uint32_t n_right, void* d_out, void* stream,
                                xc_algo* best, double* best_ms);
/* The method of xc_autotune_algorithm's choice. */
xc_status xc_autotune_method(xc_mode mode, xc_dtype dtype, const void* d_left, xc_size2 left, uint32_t n_left,
                             const void* d_right, xc_size2 right, uint32_t n_right, void* d_out, void* stream,
                             xc_method* best, double* best_ms);

/* ------------------------------------------------------------------------ */
/* Kernel-launch layer: drop-ins for the reference's run_* launchers        */
/* (src/kernels.cuh), typed per element type like its explicit              */
/* instantiations (src/naive_shuffle.cu:527-651).  Tile arguments are       */
/* validated with the reference's limits and otherwise advisory: the GB300  */
/* kernels pick their own tiling.  Nothing is allocated.                    */
/* ------------------------------------------------------------------------ */
/* run_ccn_shuffle (src/kernels.cuh:65-73): one_to_one, matrix_size both inputs. */
xc_status xc_run_ccn_shuffle_f32(const float* left, const float* right, float* out, xc_size2 matrix_size,
                                 xc_size2 search_size, uint32_t warps_per_thread_block, void* stream);
xc_status xc_run_ccn_shuffle_f64(const double* left, const double* right, double* out, xc_size2 matrix_size,
                                 xc_size2 search_size, uint32_t warps_per_thread_block, void* stream);
/* run_ccn_shuffle_multimat_right (src/kernels.cuh:87-97): one left, many right. */
xc_status xc_run_ccn_shuffle_multimat_right_f32(const float* left, const float* right, float* out,
                                                xc_size2 matrix_size, xc_size2 search_size,
                                                uint32_t num_right_matrices, uint32_t warps_per_thread_block,
                                                uint32_t right_matrices_per_thread, void* stream);
xc_status xc_run_ccn_shuffle_multimat_right_f64(const double* left, const double* right, double* out,
                                                xc_size2 matrix_size, xc_size2 search_size,
                                                uint32_t num_right_matrices, uint32_t warps_per_thread_block,
                                                uint32_t right_matrices_per_thread, void* stream);
/* run_ccn_shuffle_one_to_many_multirow_both_multimat_right (src/kernels.cuh:223-236),
 * the launcher the reference's sample_app embeds (sample_app/src/main.cpp:48-59). */
xc_status xc_run_ccn_shuffle_one_to_many_multirow_both_multimat_right_f32(
    const float* left, const float* right, float* out, xc_size2 matrix_size, xc_size2 search_size,
    uint32_t num_right_matrices, uint32_t warps_per_thread_block, uint32_t shifts_per_thread_right_matrix,
    uint32_t right_matrices_per_thread, uint32_t left_rows_per_iteration, void* stream);
xc_status xc_run_ccn_shuffle_one_to_many_multirow_both_multimat_right_f64(
    const double* left, const double* right, double* out, xc_size2 matrix_size, xc_size2 search_size,
    uint32_t num_right_matrices, uint32_t warps_per_thread_block, uint32_t shifts_per_thread_right_matrix,
    uint32_t right_matrices_per_thread, uint32_t left_rows_per_iteration, void* stream);
/* run_ccn_n_to_m_shuffle_multirow_both_multimat_both (src/kernels.cuh:238-252):
 * output index l*num_right + r. */
xc_status xc_run_ccn_n_to_m_shuffle_multirow_both_multimat_both_f32(
    const float* left, const float* right, float* out, xc_size2 matrix_size, xc_size2 search_size,
    uint32_t num_left_matrices, uint32_t num_right_matrices, uint32_t warps_per_thread_block,
    uint32_t shifts_per_thread_right_matrix, uint32_t left_matrices_per_thread, uint32_t right_matrices_per_thread,
    uint32_t left_rows_per_iteration, void* stream);
xc_status xc_run_ccn_n_to_m_shuffle_multirow_both_multimat_both_f64(
    const double* left, const double* right, double* out, xc_size2 matrix_size, xc_size2 search_size,
    uint32_t num_left_matrices, uint32_t num_right_matrices, uint32_t warps_per_thread_block,
    uint32_t shifts_per_thread_right_matrix, uint32_t left_matrices_per_thread, uint32_t right_matrices_per_thread,
    uint32_t left_rows_per_iteration, void* stream);

/* Work distribution (src/row_distribution.cuh:9-13, the DIST template
 * argument of the *_work_distribution launchers): how the reference splits
 * the rows of a shift over workers.  Validated (rectangle and triangle need
 * max_rows_per_thread > 0) and otherwise advisory: the GB300 kernel splits
 * the right rows of a whole tile of shifts over CTAs when its tiles would
 * not fill the GPU. */
typedef enum xc_distribution { XC_DIST_NONE = 0, XC_DIST_RECTANGLE = 1, XC_DIST_TRIANGLE = 2 } xc_distribution;
/* The work-distribution launchers ADD their results into `out`, which the
 * caller zeroes first, like the reference's atomic kernels
 * (src/one_to_one.hpp:276-277 zeroes before run_ccn_shuffle_work_distribution). */
/* run_ccn_shuffle_work_distribution (src/kernels.cuh:75-85): one_to_one. */
xc_status xc_run_ccn_shuffle_work_distribution_f32(const float* left, const float* right, float* out,
                                                   xc_size2 matrix_size, xc_size2 search_size,
                                                   uint32_t warps_per_thread_block, uint32_t max_rows_per_thread,
                                                   xc_distribution distribution, void* stream);
xc_status xc_run_ccn_shuffle_work_distribution_f64(const double* left, const double* right, double* out,
                                                   xc_size2 matrix_size, xc_size2 search_size,
                                                   uint32_t warps_per_thread_block, uint32_t max_rows_per_thread,
                                                   xc_distribution distribution, void* stream);
/* run_ccn_shuffle_multimat_right_work_distribution (src/kernels.cuh:130-142): one left, many right. */
xc_status xc_run_ccn_shuffle_multimat_right_work_distribution_f32(
    const float* left, const float* right, float* out, xc_size2 matrix_size, xc_size2 search_size,
    uint32_t num_right_matrices, uint32_t warps_per_thread_block, uint32_t right_matrices_per_thread,
    uint32_t max_rows_per_thread, xc_distribution distribution, void* stream);
xc_status xc_run_ccn_shuffle_multimat_right_work_distribution_f64(
    const double* left, const double* right, double* out, xc_size2 matrix_size, xc_size2 search_size,
    uint32_t num_right_matrices, uint32_t warps_per_thread_block, uint32_t right_matrices_per_thread,
    uint32_t max_rows_per_thread, xc_distribution distribution, void* stream);
/* run_ccn_shuffle_n_to_m_multimat_both_work_distribution (src/kernels.cuh:161-174)
 * and its local_mem:: twin (src/kernels.cuh:256-269): output l*num_right + r. */
xc_status xc_run_ccn_shuffle_n_to_m_multimat_both_work_distribution_f32(
    const float* left, const float* right, float* out, xc_size2 matrix_size, xc_size2 search_size,
    uint32_t num_left_matrices, uint32_t num_right_matrices, uint32_t warps_per_thread_block,
    uint32_t left_matrices_per_thread, uint32_t right_matrices_per_thread, uint32_t max_rows_per_thread,
    xc_distribution distribution, void* stream);
xc_status xc_run_ccn_shuffle_n_to_m_multimat_both_work_distribution_f64(
    const double* left, const double* right, double* out, xc_size2 matrix_size, xc_size2 search_size,
    uint32_t num_left_matrices, uint32_t num_right_matrices, uint32_t warps_per_thread_block,
    uint32_t left_matrices_per_thread, uint32_t right_matrices_per_thread, uint32_t max_rows_per_thread,
    xc_distribution distribution, void* stream);
xc_status xc_run_ccn_shuffle_n_to_m_multimat_both_work_distribution_local_mem_f32(
    const float* left, const float* right, float* out, xc_size2 matrix_size, xc_size2 search_size,
    uint32_t num_left_matrices, uint32_t num_right_matrices, uint32_t warps_per_thread_block,
    uint32_t left_matrices_per_thread, uint32_t right_matrices_per_thread, uint32_t max_rows_per_thread,
    xc_distribution distribution, void* stream);
xc_status xc_run_ccn_shuffle_n_to_m_multimat_both_work_distribution_local_mem_f64(
    const double* left, const double* right, double* out, xc_size2 matrix_size, xc_size2 search_size,
    uint32_t num_left_matrices, uint32_t num_right_matrices, uint32_t warps_per_thread_block,
    uint32_t left_matrices_per_thread, uint32_t right_matrices_per_thread, uint32_t max_rows_per_thread,
    xc_distribution distribution, void* stream);
/* run_ccn_shuffle_multirow_right (src/kernels.cuh:176-185): one_to_one. */
xc_status xc_run_ccn_shuffle_multirow_right_f32(const float* left, const float* right, float* out,
                                                xc_size2 matrix_size, xc_size2 search_size,
                                                uint32_t warps_per_thread_block, uint32_t right_rows_per_thread,
                                                void* stream);
xc_status xc_run_ccn_shuffle_multirow_right_f64(const double* left, const double* right, double* out,
                                                xc_size2 matrix_size, xc_size2 search_size,
                                                uint32_t warps_per_thread_block, uint32_t right_rows_per_thread,
                                                void* stream);
/* run_ccn_shuffle_multirow_both (src/kernels.cuh:187-197) and its local_mem::
 * twin (src/kernels.cuh:271-281): one_to_one. */
xc_status xc_run_ccn_shuffle_multirow_both_f32(const float* left, const float* right, float* out,
                                               xc_size2 matrix_size, xc_size2 search_size,
                                               uint32_t warps_per_thread_block, uint32_t max_shifts_per_thread,
                                               uint32_t max_left_rows, void* stream);
xc_status xc_run_ccn_shuffle_multirow_both_f64(const double* left, const double* right, double* out,
                                               xc_size2 matrix_size, xc_size2 search_size,
                                               uint32_t warps_per_thread_block, uint32_t max_shifts_per_thread,
                                               uint32_t max_left_rows, void* stream);
xc_status xc_run_ccn_shuffle_multirow_both_local_mem_f32(const float* left, const float* right, float* out,
                                                         xc_size2 matrix_size, xc_size2 search_size,
                                                         uint32_t warps_per_thread_block,
                                                         uint32_t max_shifts_per_thread, uint32_t max_left_rows,
                                                         void* stream);
xc_status xc_run_ccn_shuffle_multirow_both_local_mem_f64(const double* left, const double* right, double* out,
                                                         xc_size2 matrix_size, xc_size2 search_size,
                                                         uint32_t warps_per_thread_block,
                                                         uint32_t max_shifts_per_thread, uint32_t max_left_rows,
                                                         void* stream);
/* run_ccn_shuffle_multirow_right_multimat_right (src/kernels.cuh:209-221): one left, many right. */
xc_status xc_run_ccn_shuffle_multirow_right_multimat_right_f32(
    const float* left, const float* right, float* out, xc_size2 matrix_size, xc_size2 search_size,
    uint32_t num_right_matrices, uint32_t warps_per_thread_block, uint32_t right_rows_per_thread,
    uint32_t right_matrices_per_thread, void* stream);
xc_status xc_run_ccn_shuffle_multirow_right_multimat_right_f64(
    const double* left, const double* right, double* out, xc_size2 matrix_size, xc_size2 search_size,
    uint32_t num_right_matrices, uint32_t warps_per_thread_block, uint32_t right_rows_per_thread,
    uint32_t right_matrices_per_thread, void* stream);

/* run_hadamard_original (src/kernels.cuh:7-15, src/hadamard.cu:33-58,176-192):
 * in place, deformed[i] = ref[i mod (area*subregions)] * conj(deformed[i]);
 * complex values as interleaved (re, im) pairs. */
xc_status xc_run_hadamard_original_c64(const void* ref, void* deformed, xc_size2 subregion_size,
                                       uint32_t subregions_per_pic, uint32_t batch_size, uint32_t threads_per_block,
                                       void* stream);
xc_status xc_run_hadamard_original_c128(const void* ref, void* deformed, xc_size2 subregion_size,
                                        uint32_t subregions_per_pic, uint32_t batch_size, uint32_t threads_per_block,
                                        void* stream);
/* run_hadamard_n_to_m_over_output (src/kernels.cuh:29-38, src/hadamard.cu:116-149):
 * out[l*R*A + r*A + k] = left[l*A + k] * conj(right[r*A + k]), A = area. */
xc_status xc_run_hadamard_n_to_m_over_output_c64(const void* left, const void* right, void* out, xc_size2 matrix_size,
                                                 uint32_t left_num, uint32_t right_num, uint32_t threads_per_block,
                                                 uint32_t min_items_per_thread, void* stream);
xc_status xc_run_hadamard_n_to_m_over_output_c128(const void* left, const void* right, void* out,
                                                  xc_size2 matrix_size, uint32_t left_num, uint32_t right_num,
                                                  uint32_t threads_per_block, uint32_t min_items_per_thread,
                                                  void* stream);
/* run_scatter (src/kernels.cuh:54-63, src/scatter.cu:16-102): copies each src
 * matrix into dst at dst_pos.  Fixes the reference's non-square column index
 * (src/scatter.cu:39).  Unlike the reference, also zero-fills the rest of dst,
 * so no separate cudaMemset pass is needed. */
xc_status xc_run_scatter_f32(const float* src, float* dst, xc_size2 src_matrix_size, uint32_t src_num_matrices,
                             xc_size2 dst_matrix_size, xc_size2 dst_pos, uint32_t threads_per_block,
                             uint32_t items_per_thread, void* stream);
xc_status xc_run_scatter_f64(const double* src, double* dst, xc_size2 src_matrix_size, uint32_t src_num_matrices,
                             xc_size2 dst_matrix_size, xc_size2 dst_pos, uint32_t threads_per_block,
                             uint32_t items_per_thread, void* stream);
/* normalize_fft_results (src/fft_helpers.hpp:193-261) on the device: `raw` holds
 * `count` raw circular correlations of size raw_size, `norm` receives
 * (raw_size.y-1) x (raw_size.x-1) each, quadrant-swapped and divided by the area. */
xc_status xc_normalize_fft_results_f32(const float* raw, float* norm, xc_size2 raw_size, uint32_t count,
                                       void* stream);
xc_status xc_normalize_fft_results_f64(const double* raw, double* norm, xc_size2 raw_size, uint32_t count,
                                       void* stream);

#ifdef __cplusplus
}
#endif

#endif /* XCORR_GB300_H */
