// ragged.cu -- ragged batches: pairs of matrices of arbitrary, different sizes
// (new in this library; the reference only correlates equal sizes,
// src/cross_corr.hpp:121-130).
//
// A plan binds the caller's input and output buffers and prepares, once:
//  * padded copies of every matrix with a 16-byte row pitch, so that TMA can
//    describe each of them (packed ragged matrices rarely have one), and one
//    tensor map per matrix;
//  * the list of output tiles of every pair, sorted by estimated work
//    (heaviest first), for each candidate tile shape;
//  * a CUDA graph per variant holding the whole step: repack the inputs
//    into the padded copies, reset the tile queue, one persistent launch of
//    the plain kernel whose CTAs pull tiles from the queue until it is empty.
// A variant is a tile shape of the plain kernel and, for FP32 batches, a
// route: the pairs with at least the route's multiply-add count run instead
// as one_to_one calls of the split-BF16 tensor-core path, dealt out over
// up to kMaxTcStreams side streams (longest first, each to the least loaded stream)
// and captured into the same graph, beside the plain kernel's branch.  Route
// 0 keeps every pair on the plain kernel.
// Executing the plan replays the chosen variant's graph.  The autotuner times
// every tile shape with route 0, then the routes with the best shape, keeps
// the fastest and remembers the choice in a small JSON-lines cache keyed by
// the batch's signature.
#include <cuda_runtime.h>
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "ragged_route.h"
#include "xc_common.cuh"
#include "xc_internal.h"

namespace xc {

namespace {

constexpr int kMaxTcStreams = 8;  // side streams of the split-BF16 route (XC_RAGGED_TC_STREAMS, default 8)
// Left rows per work item of a routed pair.  A lone call shortens its items
// until they give two per SM; with eight calls in flight longer items pay
// (512-pair batch, 448 pairs routed: 33.3 ms with the lone-call rule, 31.1 /
// 30.6 / 30.8 / 32.0 ms with items of 24 / 32 / 48 / 64 rows).
constexpr int kTcItemRows = 32;

struct CopyJob {  // one matrix into its padded copy
  long long src, dst;
  int rows, cols, pitch;
};

// One block per (job, row); copies a row and zero-fills the pitch tail.
template <typename T>
__global__ void repack_kernel(const T* __restrict__ src, T* __restrict__ dst, const CopyJob* __restrict__ jobs,
                              int max_rows) {
  const CopyJob jb = jobs[blockIdx.x / max_rows];
  const int r = blockIdx.x % max_rows;
  if (r >= jb.rows) return;
  const T* s = src + jb.src + (long long)r * jb.cols;
  T* d = dst + jb.dst + (long long)r * jb.pitch;
  for (int c = threadIdx.x; c < jb.pitch; c += blockDim.x) d[c] = c < jb.cols ? s[c] : T(0);
}

}  // namespace

struct RaggedPlanImpl {
  xc_dtype dtype;
  size_t es;
  const void* left;
  const void* right;
  void* out;
  std::vector<xc_matrix_desc> lefts, rights;
  std::vector<xc_pair_desc> pairs;
  // device state
  void* lpad = nullptr;
  void* rpad = nullptr;
  CopyJob* jobs = nullptr;
  int n_jobs = 0, max_rows = 0;
  RaggedPairDev* dpairs = nullptr;
  unsigned int* queue = nullptr;
  cudaStream_t capture_stream = nullptr;
  struct Variant {
    bool built = false;
    RaggedTile* tiles = nullptr;
    int n_tiles = 0;
    int tc_pairs = 0;  // pairs of the variant's route (split-BF16 calls)
    int grid = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
  };
  std::vector<Variant> variants;         // index = shape + n_shapes * route
  std::vector<void*> maps_for_shape;     // per-shape tensor-map arrays (the box depends on the tile shape)
  int n_shapes = 1, n_routes = 1;
  int chosen = 0;
  double tuned_ms = -1.0;
  // split-BF16 routes (FP32)
  std::vector<double> pair_mac;          // multiply-adds of each pair
  std::vector<char> tc_ok;               // the split path takes the pair
  int n_streams = kMaxTcStreams;
  cudaStream_t tc_streams[kMaxTcStreams] = {};
  cudaEvent_t fork = nullptr;
  cudaEvent_t joins[kMaxTcStreams] = {};
  void* tc_ws[kMaxTcStreams] = {};
  size_t tc_ws_bytes = 0;
};

namespace {

size_t pitch_of(int cols, size_t es) {
  const size_t per16 = 16 / es;
  return (cols + per16 - 1) / per16 * per16;
}

// Work estimate of a tile: right rows x right columns it streams, times its shifts.
double tile_cost(const RaggedPairDev& p, int sy0, int sx0, const RaggedShape& sh) {
  const int y_lo = std::max(0, p.Hr - 1 - (sy0 + sh.bsy - 1));
  const int y_hi = std::min(p.Hr, p.Hl + p.Hr - 1 - sy0);
  const int x_lo = std::max(0, p.Wr - 1 - (sx0 + sh.bsx - 1));
  const int x_hi = std::min(p.Wr, p.Wl + p.Wr - 1 - sx0);
  return (double)std::max(0, y_hi - y_lo) * std::max(0, x_hi - x_lo);
}

bool pair_in_route(const RaggedPlanImpl* P, size_t pair, int route) {
  return in_route(P->pair_mac[pair], P->tc_ok[pair] != 0, route);
}

RaggedPairDev pair_dev(const RaggedPlanImpl* P, size_t i) {
  const xc_pair_desc& pd = P->pairs[i];
  const xc_matrix_desc& L = P->lefts[pd.left];
  const xc_matrix_desc& R = P->rights[pd.right];
  RaggedPairDev d;
  d.left = (int)pd.left;
  d.right = (int)pd.right;
  d.Hl = (int)L.rows;
  d.Wl = (int)L.cols;
  d.Hr = (int)R.rows;
  d.Wr = (int)R.cols;
  d.out_off = (long long)pd.out_offset;
  return d;
}

// Tensor maps of the padded copies for one tile shape's boxes (built once per shape).
xc_status shape_maps(RaggedPlanImpl* P, int shape, const RaggedShape& sh) {
  if (P->maps_for_shape[2 * shape] != nullptr) return XC_OK;
  const CUtensorMapDataType dt = P->es == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
  std::vector<CUtensorMap> lm(P->lefts.size()), rm(P->rights.size());
  long long off = 0;
  for (size_t i = 0; i < P->lefts.size(); ++i) {
    const xc_matrix_desc& m = P->lefts[i];
    const uint64_t pitch = pitch_of((int)m.cols, P->es);
    uint64_t dims[3] = {m.cols, m.rows, 1};
    uint64_t str[2] = {pitch * P->es, pitch * m.rows * P->es};
    uint32_t box[3] = {(uint32_t)sh.lw, (uint32_t)sh.bsy, 1};
    if (!encode_tiled(&lm[i], dt, 3, (const char*)P->lpad + off * P->es, dims, str, box, CU_TENSOR_MAP_SWIZZLE_NONE))
      return XC_ERR_INVALID_ARGUMENT;
    off += (long long)pitch * m.rows;
  }
  off = 0;
  for (size_t i = 0; i < P->rights.size(); ++i) {
    const xc_matrix_desc& m = P->rights[i];
    const uint64_t pitch = pitch_of((int)m.cols, P->es);
    uint64_t dims[4] = {m.cols, m.rows, 1, 1};
    uint64_t str[3] = {pitch * P->es, pitch * m.rows * P->es, pitch * m.rows * P->es};
    uint32_t box[4] = {(uint32_t)sh.xc, 1, 1, 1};
    if (!encode_tiled(&rm[i], dt, 4, (const char*)P->rpad + off * P->es, dims, str, box, CU_TENSOR_MAP_SWIZZLE_NONE))
      return XC_ERR_INVALID_ARGUMENT;
    off += (long long)pitch * m.rows;
  }
  CUtensorMap *dl = nullptr, *dr = nullptr;
  XC_CUDA_TRY(cudaMalloc(&dl, sizeof(CUtensorMap) * lm.size()));
  P->maps_for_shape[2 * shape] = dl;
  XC_CUDA_TRY(cudaMalloc(&dr, sizeof(CUtensorMap) * rm.size()));
  P->maps_for_shape[2 * shape + 1] = dr;
  XC_CUDA_TRY(cudaMemcpy(dl, lm.data(), sizeof(CUtensorMap) * lm.size(), cudaMemcpyHostToDevice));
  XC_CUDA_TRY(cudaMemcpy(dr, rm.data(), sizeof(CUtensorMap) * rm.size(), cudaMemcpyHostToDevice));
  return XC_OK;
}

// Side streams, fork/join events and one workspace per side stream (sized
// for the largest pair the split path takes), made on the first route that
// needs them.
xc_status tc_resources(RaggedPlanImpl* P) {
  if (P->fork != nullptr) return XC_OK;
  PairMap pm;
  uint64_t n_out = 0;
  make_pair_map(XC_ONE_TO_ONE, 1, 1, &pm, &n_out);
  size_t ws = 0;
  for (size_t i = 0; i < P->pairs.size(); ++i)
    if (P->tc_ok[i]) {
      const RaggedPairDev d = pair_dev(P, i);
      ws = std::max(ws, tc_workspace_size(Geometry{d.Hl, d.Wl, d.Hr, d.Wr, d.Hl + d.Hr - 1, d.Wl + d.Wr - 1}, pm,
                                          false));
    }
  // (what an earlier, failed attempt made is kept and reused)
  for (int k = 0; k < P->n_streams; ++k) {
    if (P->tc_streams[k] == nullptr)
      XC_CUDA_TRY(cudaStreamCreateWithFlags(&P->tc_streams[k], cudaStreamNonBlocking));
    if (P->joins[k] == nullptr) XC_CUDA_TRY(cudaEventCreateWithFlags(&P->joins[k], cudaEventDisableTiming));
    if (P->tc_ws[k] == nullptr) XC_CUDA_TRY(cudaMalloc(&P->tc_ws[k], std::max<size_t>(ws, 256)));
  }
  P->tc_ws_bytes = std::max<size_t>(ws, 256);
  XC_CUDA_TRY(cudaEventCreateWithFlags(&P->fork, cudaEventDisableTiming));
  return XC_OK;
}

xc_status build_variant(RaggedPlanImpl* P, int index) {
  RaggedPlanImpl::Variant& v = P->variants[index];
  if (v.built) return XC_OK;
  const int shape = index % P->n_shapes, route = index / P->n_shapes;
  const RaggedShape sh = ragged_shape(P->dtype, shape);
  // tiles of every pair the plain kernel keeps, heaviest first; the pairs of
  // the route, longest first
  std::vector<RaggedPairDev> hp(P->pairs.size());
  std::vector<std::pair<double, RaggedTile>> tiles;
  const std::vector<size_t> tc_pairs = route_pairs(P->pair_mac, P->tc_ok, route);
  for (size_t i = 0; i < P->pairs.size(); ++i) {
    const RaggedPairDev d = pair_dev(P, i);
    hp[i] = d;
    if (pair_in_route(P, i, route)) continue;
    const int Sy = d.Hl + d.Hr - 1, Sx = d.Wl + d.Wr - 1;
    const int rem = (d.Wr - 1) % sh.vec;
    const int origin = rem == 0 ? 0 : rem - sh.vec;
    for (int sy0 = 0; sy0 < Sy; sy0 += sh.bsy)
      for (int sx0 = origin; sx0 < Sx; sx0 += sh.bsx) {
        RaggedTile t;
        t.pair = (int)i;
        t.sy0 = sy0;
        t.sx0 = sx0;
        tiles.emplace_back(tile_cost(d, sy0, sx0, sh), t);
      }
  }
  std::stable_sort(tiles.begin(), tiles.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
  std::vector<RaggedTile> ht(tiles.size());
  for (size_t i = 0; i < tiles.size(); ++i) ht[i] = tiles[i].second;
  if (P->dpairs == nullptr) {
    XC_CUDA_TRY(cudaMalloc(&P->dpairs, sizeof(RaggedPairDev) * hp.size()));
    XC_CUDA_TRY(cudaMemcpy(P->dpairs, hp.data(), sizeof(RaggedPairDev) * hp.size(), cudaMemcpyHostToDevice));
  }
  v.n_tiles = (int)ht.size();
  v.tc_pairs = (int)tc_pairs.size();
  if (v.tiles != nullptr) {  // left by an earlier, failed build of this variant
    cudaFree(v.tiles);
    v.tiles = nullptr;
  }
  if (v.n_tiles > 0) {
    XC_CUDA_TRY(cudaMalloc(&v.tiles, sizeof(RaggedTile) * ht.size()));
    XC_CUDA_TRY(cudaMemcpy(v.tiles, ht.data(), sizeof(RaggedTile) * ht.size(), cudaMemcpyHostToDevice));
    XC_TRY(shape_maps(P, shape, sh));
    // persistent grid: every SM filled to the kernel's occupancy
    int dev = 0, sms = 0, per_sm = 0;
    XC_CUDA_TRY(cudaGetDevice(&dev));
    XC_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    XC_CUDA_TRY(cudaFuncSetAttribute(sh.kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, sh.smem));
    XC_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sh.kernel, sh.threads, sh.smem));
    v.grid = std::max(1, std::min(v.n_tiles, sms * std::max(1, per_sm)));
  }

  // the route's pairs: each to the side stream with the least work so far
  PairMap pm1;
  uint64_t n_out1 = 0;
  make_pair_map(XC_ONE_TO_ONE, 1, 1, &pm1, &n_out1);
  const std::vector<std::vector<size_t>> per_stream = deal_route(tc_pairs, P->pair_mac, P->n_streams);
  if (!tc_pairs.empty()) {
    XC_TRY(tc_resources(P));
    for (size_t i : tc_pairs) {
      const RaggedPairDev& d = hp[i];
      XC_TRY(tc_prepare(Geometry{d.Hl, d.Wl, d.Hr, d.Wr, d.Hl + d.Hr - 1, d.Wl + d.Wr - 1}, pm1, false));
    }
  }

  // capture the step into a graph: the split-path branches fork from the
  // capture stream first, so they depend on nothing; the plain branch runs
  // beside them; the branches join before the capture ends
  cudaStream_t s = P->capture_stream;
  XC_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  xc_status st = XC_OK;
  const bool forked = !tc_pairs.empty();
  if (forked && cudaEventRecord(P->fork, s) != cudaSuccess) st = fail(XC_ERR_CUDA, "ragged capture: fork failed");
  for (int k = 0; k < P->n_streams && forked; ++k)
    if (st == XC_OK && !per_stream[k].empty() && cudaStreamWaitEvent(P->tc_streams[k], P->fork, 0) != cudaSuccess)
      st = fail(XC_ERR_CUDA, "ragged capture: a side stream could not join");
  if (st == XC_OK && v.n_tiles > 0) {
    RaggedLaunch rl;
    rl.left = P->lpad;
    rl.right = P->rpad;
    rl.out = P->out;
    rl.tiles = v.tiles;
    rl.pairs = P->dpairs;
    rl.lmaps = static_cast<const CUtensorMap*>(P->maps_for_shape[2 * shape]);
    rl.rmaps = static_cast<const CUtensorMap*>(P->maps_for_shape[2 * shape + 1]);
    rl.queue = P->queue;
    rl.n_tiles = v.n_tiles;
    rl.grid = v.grid;
    const unsigned nb_l = (unsigned)P->lefts.size() * (unsigned)P->max_rows;  // left jobs only
    if (P->es == 4) {
      repack_kernel<float><<<nb_l, 128, 0, s>>>((const float*)P->left, (float*)P->lpad, P->jobs, P->max_rows);
    } else {
      repack_kernel<double><<<nb_l, 128, 0, s>>>((const double*)P->left, (double*)P->lpad, P->jobs, P->max_rows);
    }
    // rights: jobs after the lefts in the same table, different source / destination
    const int nl = (int)P->lefts.size();
    const unsigned nb_r = (unsigned)(P->n_jobs - nl) * (unsigned)P->max_rows;
    if (nb_r > 0) {
      if (P->es == 4)
        repack_kernel<float><<<nb_r, 128, 0, s>>>((const float*)P->right, (float*)P->rpad, P->jobs + nl,
                                                  P->max_rows);
      else
        repack_kernel<double><<<nb_r, 128, 0, s>>>((const double*)P->right, (double*)P->rpad, P->jobs + nl,
                                                   P->max_rows);
    }
    if (cudaMemsetAsync(P->queue, 0, sizeof(unsigned int), s) != cudaSuccess)
      st = fail(XC_ERR_CUDA, "ragged capture: queue reset failed");
    if (st == XC_OK) st = ragged_launch(P->dtype, shape, rl, s);
  }
  for (int k = 0; k < P->n_streams && forked; ++k) {
    if (per_stream[k].empty()) continue;
    const cudaStream_t sk = P->tc_streams[k];
    for (size_t i : per_stream[k]) {
      if (st != XC_OK) break;
      const RaggedPairDev& d = hp[i];
      const xc_matrix_desc& L = P->lefts[d.left];
      const xc_matrix_desc& R = P->rights[d.right];
      st = tc_correlate((const float*)P->left + L.offset, (const float*)P->right + R.offset,
                        (float*)P->out + d.out_off, Geometry{d.Hl, d.Wl, d.Hr, d.Wr, d.Hl + d.Hr - 1, d.Wl + d.Wr - 1},
                        pm1, P->tc_ws[k], P->tc_ws_bytes, sk, false, kTcItemRows, kTcItemRows);
    }
    // every forked stream joins, also after an error, so that the capture can end
    cudaEventRecord(P->joins[k], sk);
    cudaStreamWaitEvent(s, P->joins[k], 0);
  }
  cudaGraph_t graph = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(s, &graph);
  if (st != XC_OK) {
    if (graph) cudaGraphDestroy(graph);
    return st;
  }
  XC_CUDA_TRY(ce);
  v.graph = graph;
  XC_CUDA_TRY(cudaGraphInstantiate(&v.exec, graph, 0));
  v.built = true;
  return XC_OK;
}

std::string cache_path() {
  const char* e = std::getenv("XC_AUTOTUNE_CACHE");
  if (e && *e) return e;
  const char* home = std::getenv("HOME");
  return std::string(home ? home : "/tmp") + "/.cache/xcorr_gb300_autotune.jsonl";
}

// Side streams of the split-BF16 routes: XC_RAGGED_TC_STREAMS (1-8), default
// 8 (512-pair batch, 448 pairs routed, 32-row items: 31.8 ms on 6 streams,
// 30.6 ms on 8; with the lone-call item rule 40.9 / 34.2 / 33.3 ms on 2 / 4 / 8).
int tc_stream_count() {
  static const int n = [] {
    const char* e = std::getenv("XC_RAGGED_TC_STREAMS");
    const int v = e ? std::atoi(e) : 0;
    return v >= 1 && v <= kMaxTcStreams ? v : kMaxTcStreams;
  }();
  return n;
}

// XC_RAGGED_TC=0 keeps every pair of FP32 plans on the plain kernel.
bool tc_routes_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("XC_RAGGED_TC");
    return !(e && std::strcmp(e, "0") == 0);
  }();
  return on;
}

std::string signature(const RaggedPlanImpl* P) {
  cudaDeviceProp prop;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaGetDeviceProperties(&prop, dev);
  double mac = 0.0;
  for (const auto& pd : P->pairs) {
    const auto& L = P->lefts[pd.left];
    const auto& R = P->rights[pd.right];
    mac += (double)L.rows * L.cols * R.rows * R.cols;
  }
  std::ostringstream ss;
  ss << prop.name << "|dtype=" << (int)P->dtype << "|pairs=" << P->pairs.size() << "|mac_log2="
     << (int)std::floor(std::log2(std::max(1.0, mac / std::max<size_t>(1, P->pairs.size())))) << "|variants="
     << P->n_shapes << "x" << P->n_routes;
  return ss.str();
}

}  // namespace

xc_status ragged_plan_create(RaggedPlanImpl** out, xc_dtype dtype, const void* d_left, const xc_matrix_desc* lefts,
                             uint32_t n_left, const void* d_right, const xc_matrix_desc* rights, uint32_t n_right,
                             const xc_pair_desc* pairs, uint32_t n_pairs, void* d_out) {
  *out = nullptr;
  if (d_left == nullptr || d_right == nullptr || d_out == nullptr || lefts == nullptr || rights == nullptr ||
      pairs == nullptr)
    return fail(XC_ERR_INVALID_ARGUMENT, "NULL argument");
  if (n_left == 0 || n_right == 0 || n_pairs == 0) return fail(XC_ERR_INVALID_ARGUMENT, "empty ragged batch");
  if (dtype != XC_F32 && dtype != XC_F64) return fail(XC_ERR_INVALID_ARGUMENT, "unknown dtype");
  for (uint32_t i = 0; i < n_left; ++i)
    if (lefts[i].rows == 0 || lefts[i].cols == 0) return fail(XC_ERR_INVALID_ARGUMENT, "empty left matrix");
  for (uint32_t i = 0; i < n_right; ++i)
    if (rights[i].rows == 0 || rights[i].cols == 0) return fail(XC_ERR_INVALID_ARGUMENT, "empty right matrix");
  for (uint32_t i = 0; i < n_pairs; ++i)
    if (pairs[i].left >= n_left || pairs[i].right >= n_right)
      return fail(XC_ERR_INVALID_ARGUMENT, "pair " + std::to_string(i) + " names a matrix out of range");

  auto P = new RaggedPlanImpl();
  P->dtype = dtype;
  P->es = dtype == XC_F32 ? 4 : 8;
  P->left = d_left;
  P->right = d_right;
  P->out = d_out;
  P->lefts.assign(lefts, lefts + n_left);
  P->rights.assign(rights, rights + n_right);
  P->pairs.assign(pairs, pairs + n_pairs);
  P->n_shapes = ragged_shape_count(dtype);
  P->n_routes = dtype == XC_F32 && tc_routes_enabled() ? kRaggedRoutes : 1;
  P->n_streams = tc_stream_count();
  P->variants.resize((size_t)P->n_shapes * P->n_routes);
  P->maps_for_shape.assign(2 * (size_t)P->n_shapes, nullptr);
  // multiply-adds of every pair, and whether the split path takes it
  {
    PairMap pm1;
    uint64_t n_out1 = 0;
    make_pair_map(XC_ONE_TO_ONE, 1, 1, &pm1, &n_out1);
    for (uint32_t i = 0; i < n_pairs; ++i) {
      const xc_matrix_desc& L = lefts[pairs[i].left];
      const xc_matrix_desc& R = rights[pairs[i].right];
      P->pair_mac.push_back((double)L.rows * L.cols * R.rows * R.cols);
      const Geometry g = make_geometry(xc_size2{L.cols, L.rows}, xc_size2{R.cols, R.rows});
      P->tc_ok.push_back(dtype == XC_F32 && tc_workspace_size(g, pm1, false) > 0 ? 1 : 0);
    }
  }
  auto cleanup = [&](xc_status s) {
    ragged_plan_destroy(P);
    return s;
  };

  // padded copies and the repack jobs (lefts first, then rights)
  std::vector<CopyJob> jobs;
  long long off = 0;
  for (const auto& m : P->lefts) {
    const int pitch = (int)pitch_of((int)m.cols, P->es);
    jobs.push_back(CopyJob{(long long)m.offset, off, (int)m.rows, (int)m.cols, pitch});
    off += (long long)pitch * m.rows;
    P->max_rows = std::max(P->max_rows, (int)m.rows);
  }
  const long long lbytes = off * (long long)P->es;
  off = 0;
  for (const auto& m : P->rights) {
    const int pitch = (int)pitch_of((int)m.cols, P->es);
    jobs.push_back(CopyJob{(long long)m.offset, off, (int)m.rows, (int)m.cols, pitch});
    off += (long long)pitch * m.rows;
    P->max_rows = std::max(P->max_rows, (int)m.rows);
  }
  const long long rbytes = off * (long long)P->es;
  P->n_jobs = (int)jobs.size();
  if (cudaMalloc(&P->lpad, lbytes) != cudaSuccess || cudaMalloc(&P->rpad, rbytes) != cudaSuccess ||
      cudaMalloc(&P->jobs, sizeof(CopyJob) * jobs.size()) != cudaSuccess ||
      cudaMalloc(&P->queue, sizeof(unsigned int)) != cudaSuccess)
    return cleanup(fail(XC_ERR_CUDA, "device allocation for the ragged plan failed"));
  if (cudaMemcpy(P->jobs, jobs.data(), sizeof(CopyJob) * jobs.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return cleanup(fail(XC_ERR_CUDA, "upload of the repack table failed"));
  if (cudaStreamCreateWithFlags(&P->capture_stream, cudaStreamNonBlocking) != cudaSuccess)
    return cleanup(fail(XC_ERR_CUDA, "stream creation failed"));
  device_flags();  // resolve the flag word's address outside any stream capture
  const xc_status st = build_variant(P, 0);
  if (st != XC_OK) return cleanup(st);
  *out = P;
  return XC_OK;
}

xc_status ragged_execute(RaggedPlanImpl* P, cudaStream_t stream) {
  XC_TRY(build_variant(P, P->chosen));
  XC_CUDA_TRY(cudaGraphLaunch(P->variants[P->chosen].exec, stream));
  return XC_OK;
}

xc_status ragged_autotune(RaggedPlanImpl* P, cudaStream_t stream, int* chosen, double* best_ms) {
  const std::string sig = signature(P);
  // cached decision?
  {
    std::ifstream in(cache_path());
    std::string line, hit;
    while (std::getline(in, line))
      if (line.find("\"sig\": \"" + sig + "\"") != std::string::npos) hit = line;
    const size_t pos = hit.find("\"variant\": ");
    if (pos != std::string::npos) {
      const int idx = std::atoi(hit.c_str() + pos + 11);
      if (idx >= 0 && idx < (int)P->variants.size()) {
        P->chosen = idx;
        *chosen = idx;
        *best_ms = -1.0;
        return XC_OK;
      }
    }
  }
  cudaEvent_t e0, e1;
  XC_CUDA_TRY(cudaEventCreate(&e0));
  XC_CUDA_TRY(cudaEventCreate(&e1));
  double best = 1e30;
  int arg = 0;
  auto time_variant = [&](int i) -> xc_status {
    XC_TRY(build_variant(P, i));
    for (int w = 0; w < 2; ++w) XC_CUDA_TRY(cudaGraphLaunch(P->variants[i].exec, stream));
    float ms = 0.f;
    XC_CUDA_TRY(cudaEventRecord(e0, stream));
    for (int r = 0; r < 5; ++r) XC_CUDA_TRY(cudaGraphLaunch(P->variants[i].exec, stream));
    XC_CUDA_TRY(cudaEventRecord(e1, stream));
    XC_CUDA_TRY(cudaEventSynchronize(e1));
    XC_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    if (ms / 5.0 < best) {
      best = ms / 5.0;
      arg = i;
    }
    return XC_OK;
  };
  xc_status st = XC_OK;
  // every tile shape with all pairs on the plain kernel, then the routes
  // with the best shape (a route whose pairs are those of the previous one,
  // or none, is not timed again)
  for (int sh = 0; sh < P->n_shapes && st == XC_OK; ++sh) st = time_variant(sh);
  const int best_shape = arg;
  size_t prev = 0;
  for (int r = 1; r < P->n_routes && st == XC_OK; ++r) {
    size_t n = 0;
    for (size_t i = 0; i < P->pairs.size(); ++i) n += pair_in_route(P, i, r) ? 1 : 0;
    if (n == 0 || n == prev) continue;
    prev = n;
    st = time_variant(best_shape + P->n_shapes * r);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  XC_TRY(st);
  P->chosen = arg;
  P->tuned_ms = best;
  *chosen = arg;
  *best_ms = best;
  // remember the decision (best effort; a missing cache directory is created)
  const std::string path = cache_path();
  FILE* f = std::fopen(path.c_str(), "a");
  if (f == nullptr) {
    const size_t slash = path.find_last_of('/');
    if (slash != std::string::npos) mkdir(path.substr(0, slash).c_str(), 0755);
    f = std::fopen(path.c_str(), "a");
  }
  if (f != nullptr) {
    std::fprintf(f, "{\"sig\": \"%s\", \"variant\": %d, \"ms\": %.6f}\n", sig.c_str(), arg, best);
    std::fclose(f);
  }
  return XC_OK;
}

xc_status ragged_describe(RaggedPlanImpl* P, int variant, xc_ragged_variant* out) {
  if (variant == -1) variant = P->chosen;
  if (variant < 0 || variant >= (int)P->variants.size())
    return fail(XC_ERR_INVALID_ARGUMENT, "variant " + std::to_string(variant) + " out of range");
  const int route = variant / P->n_shapes;
  out->index = variant;
  out->n_variants = (int32_t)P->variants.size();
  out->tile_shape = variant % P->n_shapes;
  uint32_t n = 0;
  for (size_t i = 0; i < P->pairs.size(); ++i) n += pair_in_route(P, i, route) ? 1 : 0;
  out->tc_pairs = n;
  out->tc_min_macs = (uint64_t)route_min_mac(route);
  return XC_OK;
}

xc_status ragged_select(RaggedPlanImpl* P, int variant) {
  if (variant < 0 || variant >= (int)P->variants.size())
    return fail(XC_ERR_INVALID_ARGUMENT, "variant " + std::to_string(variant) + " out of range");
  XC_TRY(build_variant(P, variant));
  P->chosen = variant;
  return XC_OK;
}

void ragged_plan_destroy(RaggedPlanImpl* P) {
  if (P == nullptr) return;
  for (auto& v : P->variants) {
    if (v.exec) cudaGraphExecDestroy(v.exec);
    if (v.graph) cudaGraphDestroy(v.graph);
    cudaFree(v.tiles);
  }
  for (void* m : P->maps_for_shape) cudaFree(m);
  for (int k = 0; k < kMaxTcStreams; ++k) {
    cudaFree(P->tc_ws[k]);
    if (P->joins[k]) cudaEventDestroy(P->joins[k]);
    if (P->tc_streams[k]) cudaStreamDestroy(P->tc_streams[k]);
  }
  if (P->fork) cudaEventDestroy(P->fork);
  cudaFree(P->dpairs);
  cudaFree(P->lpad);
  cudaFree(P->rpad);
  cudaFree(P->jobs);
  cudaFree(P->queue);
  if (P->capture_stream) cudaStreamDestroy(P->capture_stream);
  delete P;
}

// Baseline: one launch of the plain kernel per pair, on the caller's buffers.
xc_status correlate_pairs(xc_dtype dtype, const void* d_left, const xc_matrix_desc* lefts, uint32_t n_left,
                          const void* d_right, const xc_matrix_desc* rights, uint32_t n_right,
                          const xc_pair_desc* pairs, uint32_t n_pairs, void* d_out, cudaStream_t stream) {
  const size_t es = dtype == XC_F32 ? 4 : 8;
  PairMap pm;
  uint64_t n_out = 0;
  make_pair_map(XC_ONE_TO_ONE, 1, 1, &pm, &n_out);
  for (uint32_t i = 0; i < n_pairs; ++i) {
    const xc_pair_desc& pd = pairs[i];
    if (pd.left >= n_left || pd.right >= n_right) return fail(XC_ERR_INVALID_ARGUMENT, "pair out of range");
    const xc_matrix_desc& L = lefts[pd.left];
    const xc_matrix_desc& R = rights[pd.right];
    const Geometry g = make_geometry(xc_size2{L.cols, L.rows}, xc_size2{R.cols, R.rows});
    XC_TRY(direct_launch(dtype, (const char*)d_left + L.offset * es, (const char*)d_right + R.offset * es,
                         (char*)d_out + pd.out_offset * es, g, pm, stream, -1));
  }
  return XC_OK;
}

}  // namespace xc
