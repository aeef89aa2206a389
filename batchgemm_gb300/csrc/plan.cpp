// plan.cpp -- host side of the C ABI: argument checks, the per-matrix tiling
// heuristic, the largest-first tile queue, descriptor upload and launch.
//
// Rewrites of the reference's host driver (CUDA/framework/gemm.cu):
//   - per-matrix tile choice (gemm.cu:107-118: largest tile dividing M and N)
//     becomes a cost-model choice over tiles that handle ragged edges;
//   - the "wavefront" demotion loop (gemm.cu:121-169: demote every matrix of
//     the largest strategy while total parallelism is below a threshold)
//     becomes a rebalance that splits the longest tiles until none exceeds
//     the average load of one persistent CTA;
//   - the dense (max tiles M, max tiles N, batch) grid (gemm.cu:181-196)
//     becomes a queue of only the real tiles, ordered largest-first, pulled
//     by one wave of persistent CTAs;
//   - the six synchronous cudaMemcpy uploads (gemm.cu:57-77, 172-174) become
//     one asynchronous copy of a packed descriptor block from pinned memory.
#include <algorithm>
#include <array>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <list>
#include <mutex>
#include <queue>
#include <string>
#include <unordered_map>
#include <vector>

#include "bgemm.h"
#include "bgemm_debug.h"
#include "bgemm_internal.h"
#include "plan_internal.h"
#include "tile_table.h"

namespace bgemm {

// ------------------------------------------------------------- errors ----
static thread_local int t_err_arg = 0;
static thread_local int t_err_mat = -1;
static thread_local char t_err_msg[512] = "";

bgemm_status_t set_error(bgemm_status_t st, int arg, int mat, const char* fmt, ...) {
  t_err_arg = arg;
  t_err_mat = mat;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(t_err_msg, sizeof(t_err_msg), fmt, ap);
  va_end(ap);
  return st;
}
void clear_error() {
  t_err_arg = 0;
  t_err_mat = -1;
  t_err_msg[0] = 0;
}
bgemm_status_t cuda_error(cudaError_t e, const char* what) {
  return set_error(BGEMM_ERROR_CUDA, 0, -1, "%s: %s", what, cudaGetErrorString(e));
}

// -------------------------------------------------------- device facts ----
bgemm_status_t device_facts(DeviceFacts* out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
  static std::mutex mu;
  static std::unordered_map<int, DeviceFacts> cache;
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find(dev);
  if (it != cache.end()) {
    *out = it->second;
    return BGEMM_SUCCESS;
  }
  DeviceFacts f{};
  f.device = dev;
  int major = 0, minor = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  cudaDeviceGetAttribute(&f.num_sms, cudaDevAttrMultiProcessorCount, dev);
  f.cc = major * 10 + minor;
  if (f.cc != 103)
    return set_error(BGEMM_ERROR_NOT_SUPPORTED, 0, -1,
                     "device %d has compute capability %d.%d; this library is built for "
                     "sm_103a (GB300) only",
                     dev, major, minor);
  f.simt_ctas_per_sm = simt_ctas_per_sm();
  f.tc_ctas_per_sm = 1;
  cache[dev] = f;
  *out = f;
  return BGEMM_SUCCESS;
}

// ------------------------------------------------------------ planning ----
static inline long long ceil_div(long long a, long long b) { return (a + b - 1) / b; }

// Candidate (cost, tiles) of configuration c for matrix (M, N, K).
static bool simt_eval(int c, int M, int N, int K, long long* tiles, double* t_tile) {
  const SimtCfg& g = kSimtCfgs[c];
  if (ceil_div(M, g.bm) > 65535 || ceil_div(N, g.bn) > 65535) return false;
  *tiles = ceil_div(M, g.bm) * ceil_div(N, g.bn);
  *t_tile = kSimtCost[c].a_ns + kSimtCost[c].b_ns * (double)K;
  return true;
}

static bgemm_status_t choose_simt(const int* M, const int* N, const int* K, int batch, int slots,
                                  const bgemm_plan_options_t* opt, std::vector<MatPlan>& mp) {
  return choose_tiles(kSimtNumCfgs, simt_eval, M, N, K, batch, slots, opt, mp);
}

bgemm_status_t choose_tiles(int ncfg, TileEval eval, const int* M, const int* N, const int* K,
                            int batch, int slots, const bgemm_plan_options_t* opt,
                            std::vector<MatPlan>& mp) {
  mp.assign(batch, MatPlan{-1, 0, 0.0});
  double total = 0.0;
  for (int i = 0; i < batch; ++i) {
    if (M[i] == 0 || N[i] == 0) continue;
    int best = -1;
    long long bt = 0;
    double bw = 0, btt = 0;
    for (int c = ncfg - 1; c >= 0; --c) {
      if (opt && opt->force_tile_config >= 0 && c != opt->force_tile_config) continue;
      long long t;
      double tt;
      if (!eval(c, M[i], N[i], K[i], &t, &tt)) continue;
      const double w = (double)t * tt;
      if (best < 0 || w < bw * 0.999) {
        best = c; bt = t; bw = w; btt = tt;
      }
    }
    if (best < 0 || bt > (1LL << 31))
      return set_error(BGEMM_ERROR_NOT_SUPPORTED, 1, i, "matrix %d: no tile configuration fits",
                       i);
    mp[i] = MatPlan{best, bt, btt};
    total += bw;
  }
  if (opt && (opt->disable_rebalance || opt->force_tile_config >= 0)) return BGEMM_SUCCESS;
  // Rebalance: while the longest tile is longer than the average load of a
  // persistent CTA, move the matrix owning it to the configuration with the
  // shortest tile among those that do not raise its total time by more than
  // the parallelism gained.
  using Entry = std::pair<double, int>;
  std::priority_queue<Entry> heap;
  for (int i = 0; i < batch; ++i)
    if (mp[i].cfg >= 0) heap.push({mp[i].t_tile, i});
  int guard = 8 * batch + 64;
  while (!heap.empty() && guard-- > 0) {
    const auto [tt, i] = heap.top();
    if (tt != mp[i].t_tile) { heap.pop(); continue; }
    if (tt <= total / slots) break;
    // best alternative with a shorter tile
    int best = -1;
    long long bt = 0;
    double btt = 0, bw = 0;
    for (int c = 0; c < ncfg; ++c) {
      long long t;
      double t2;
      if (!eval(c, M[i], N[i], K[i], &t, &t2)) continue;
      if (t2 >= tt || t <= mp[i].tiles) continue;
      const double w = (double)t * t2;
      if (best < 0 || w < bw) { best = c; bt = t; btt = t2; bw = w; }
    }
    heap.pop();
    if (best < 0) continue;
    const double old_w = (double)mp[i].tiles * mp[i].t_tile;
    const double new_total = total - old_w + bw;
    // accept if the makespan bound improves
    const double before = std::max(total / slots, tt);
    const double after = std::max(new_total / slots, btt);
    if (after >= before) continue;
    total = new_total;
    mp[i] = MatPlan{best, bt, btt};
    heap.push({btt, i});
  }
  return BGEMM_SUCCESS;
}

static bgemm_status_t check_args(const int* M, const int* N, const int* K, const int* lda,
                                 const int* ldb, const int* ldc, int batch, int mode,
                                 int arg_M, int arg_N, int arg_K, int arg_lda, int arg_ldb,
                                 int arg_ldc, int arg_batch, int arg_mode, bool row_major = false,
                                 bool ta = false, bool tb = false) {
  if (batch < 0) return set_error(BGEMM_ERROR_INVALID_VALUE, arg_batch, -1, "batch < 0");
  if (mode < BGEMM_MODE_SIMT_FP32 || mode > BGEMM_MODE_BF16X3)
    return set_error(BGEMM_ERROR_INVALID_VALUE, arg_mode, -1, "unknown mode %d", mode);
  if (batch == 0) return BGEMM_SUCCESS;
  if (!M) return set_error(BGEMM_ERROR_INVALID_VALUE, arg_M, -1, "M is NULL");
  if (!N) return set_error(BGEMM_ERROR_INVALID_VALUE, arg_N, -1, "N is NULL");
  if (!K) return set_error(BGEMM_ERROR_INVALID_VALUE, arg_K, -1, "K is NULL");
  if (!lda) return set_error(BGEMM_ERROR_INVALID_VALUE, arg_lda, -1, "lda is NULL");
  if (!ldb) return set_error(BGEMM_ERROR_INVALID_VALUE, arg_ldb, -1, "ldb is NULL");
  if (!ldc) return set_error(BGEMM_ERROR_INVALID_VALUE, arg_ldc, -1, "ldc is NULL");
  for (int i = 0; i < batch; ++i) {
    if (M[i] < 0) return set_error(BGEMM_ERROR_INVALID_VALUE, arg_M, i, "M[%d] = %d < 0", i, M[i]);
    if (N[i] < 0) return set_error(BGEMM_ERROR_INVALID_VALUE, arg_N, i, "N[%d] = %d < 0", i, N[i]);
    if (K[i] < 0) return set_error(BGEMM_ERROR_INVALID_VALUE, arg_K, i, "K[%d] = %d < 0", i, K[i]);
    // the extent each leading dimension spans (rows of a column-major
    // matrix, columns of a row-major one)
    const char* na = row_major ? (ta ? "M" : "K") : (ta ? "K" : "M");
    const char* nb = row_major ? (tb ? "K" : "N") : (tb ? "N" : "K");
    const char* nc = row_major ? "N" : "M";
    auto dim = [&](const char* n) { return n[0] == 'M' ? M[i] : n[0] == 'N' ? N[i] : K[i]; };
    if (lda[i] < std::max(1, dim(na)))
      return set_error(BGEMM_ERROR_INVALID_VALUE, arg_lda, i, "lda[%d] = %d < max(1, %s = %d)", i,
                       lda[i], na, dim(na));
    if (ldb[i] < std::max(1, dim(nb)))
      return set_error(BGEMM_ERROR_INVALID_VALUE, arg_ldb, i, "ldb[%d] = %d < max(1, %s = %d)", i,
                       ldb[i], nb, dim(nb));
    if (ldc[i] < std::max(1, dim(nc)))
      return set_error(BGEMM_ERROR_INVALID_VALUE, arg_ldc, i, "ldc[%d] = %d < max(1, %s = %d)", i,
                       ldc[i], nc, dim(nc));
  }
  return BGEMM_SUCCESS;
}

// Queue order: matrices by modelled tile time, longest first (the
// longest-processing-time rule over one wave of persistent CTAs).  Returns
// the number of work items.
static long long order_matrices(const std::vector<MatPlan>& mp, std::vector<int>& order) {
  order.clear();
  long long n_items = 0;
  for (int i = 0; i < (int)mp.size(); ++i)
    if (mp[i].cfg >= 0) {
      order.push_back(i);
      n_items += mp[i].tiles;
    }
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return mp[a].t_tile > mp[b].t_tile; });
  return n_items;
}

// Writes the work items; each matrix's tiles stay together (n outer, m
// inner) so consecutive items share operand panels in L2.
static void expand_items(int mode, bgemm_plan_s* p, const int* M, const int* N,
                         const std::vector<MatPlan>& mp, const std::vector<int>& order,
                         MatDesc* hd, TileItem* hi) {
  size_t w = 0;
  for (int i : order) {
    int bm, bn;
    if (mode == BGEMM_MODE_SIMT_FP32) {
      bm = kSimtCfgs[mp[i].cfg].bm;
      bn = kSimtCfgs[mp[i].cfg].bn;
    } else {
      tc_tile_dims(p, i, M[i], N[i], mp[i].cfg, &bm, &bn, &hd[i]);
    }
    const bool swap = (hd[i].aux & kTcSwapFlag) != 0;
    const int tmx = (int)ceil_div(swap ? N[i] : M[i], bm);
    const int tnx = (int)ceil_div(swap ? M[i] : N[i], bn);
    for (int tn = 0; tn < tnx; ++tn)
      for (int tm = 0; tm < tmx; ++tm) hi[w++] = TileItem{i, (uint16_t)tm, (uint16_t)tn};
  }
}

// Host-only replay of the SIMT planner (tests and the autotuner use it; no
// GPU needed).  Returns the number of items, or -1 on error / overflow.
int debug_simt_queue(const int* M, const int* N, const int* K, int batch, int slots,
                     int force_cfg, int rebalance, int* cfg_out, int* items_out,
                     int max_items) {
  bgemm_plan_options_t opt{};
  opt.force_tile_config = force_cfg;
  opt.disable_rebalance = rebalance ? 0 : 1;
  std::vector<MatPlan> mp;
  if (choose_simt(M, N, K, batch, std::max(slots, 1), &opt, mp) != BGEMM_SUCCESS) return -1;
  std::vector<int> order;
  const long long n = order_matrices(mp, order);
  if (cfg_out)
    for (int i = 0; i < batch; ++i) cfg_out[i] = mp[i].cfg;
  if (!items_out) return (int)n;
  if (n > max_items) return -1;
  std::vector<MatDesc> hd(batch);
  for (int i = 0; i < batch; ++i) hd[i] = MatDesc{M[i], N[i], K[i], 0, 0, 0, mp[i].cfg, 0};
  std::vector<TileItem> it((size_t)n);
  expand_items(BGEMM_MODE_SIMT_FP32, nullptr, M, N, mp, order, hd.data(), it.data());
  for (long long t = 0; t < n; ++t) {
    items_out[3 * t] = it[t].mat;
    items_out[3 * t + 1] = it[t].tm;
    items_out[3 * t + 2] = it[t].tn;
  }
  return (int)n;
}

static bgemm_status_t plan_batch(bgemm_plan_s* p, const int* M, const int* N, const int* K,
                                 const int* lda, const int* ldb, const int* ldc, int batch,
                                 bool first, BatchPlan& bp);
static bgemm_plan_options_t default_options();

// Host-only replay of the tensor-core planner with a given number of one-SM
// slots and CTA pairs (tests; no GPU needed).  Returns the number of items,
// or -1 on error / overflow.
int debug_tc_plan(const int* M, const int* N, const int* K, int batch, int mode, int family,
                  int slots, int clusters, int* cfg_out, int* items_out, int max_items,
                  long long* ws_out, int* jobs_out, int max_jobs, int* n_jobs,
                  long long* ws_bytes, int* pair) {
  if (mode < BGEMM_MODE_TF32 || mode > BGEMM_MODE_BF16X3 || slots < 1 || clusters < 0) return -1;
  std::vector<int> ld(batch);
  for (int i = 0; i < batch; ++i) ld[i] = std::max(1, std::max(M[i], K[i]));
  bgemm_plan_s p;
  p.mode = mode;
  p.facts = DeviceFacts{0, 103, slots, 2, 1};
  p.opt = default_options();
  p.opt.kernel_family = family;
  BatchPlan bp;
  bgemm_status_t st = tc_init(&p, &p.opt, clusters);
  if (st == BGEMM_SUCCESS)
    st = plan_batch(&p, M, N, K, ld.data(), ld.data(), ld.data(), batch, true, bp);
  int n = -1;
  if (st == BGEMM_SUCCESS) {
    n = bp.req.tiles;
    for (int i = 0; cfg_out && i < batch; ++i)
      cfg_out[i] = (M[i] && N[i]) ? bp.descs[i].cfg | (bp.descs[i].aux & kTcSwapFlag ? 1 << 8 : 0)
                                  : -1;
    if (items_out) {
      if (n > max_items) {
        n = -1;
      } else {
        for (int t = 0; t < n; ++t) {
          items_out[3 * t] = bp.items[t].mat;
          items_out[3 * t + 1] = bp.items[t].tm;
          items_out[3 * t + 2] = bp.items[t].tn;
        }
      }
    }
    tc_debug_layout(&p, ws_out, jobs_out, max_jobs, n_jobs, pair);
    *ws_bytes = (long long)bp.req.workspace_bytes;
  }
  if (p.tc) tc_plan_release(&p);
  return n;
}

static void free_plan_memory(bgemm_plan_s* p) {
  if (p->d_mem) cudaFree(p->d_mem);
  for (int s = 0; s < kStageBufs; ++s) {
    if (p->h_stage[s]) cudaFreeHost(p->h_stage[s]);
    if (p->ev_stage[s]) cudaEventDestroy(p->ev_stage[s]);
    p->h_stage[s] = nullptr;
    p->ev_stage[s] = nullptr;
  }
  if (p->tc) tc_plan_release(p);
  p->d_mem = nullptr;
}

static bgemm_plan_options_t default_options() {
  bgemm_plan_options_t o{};
  o.force_tile_config = -1;
  return o;
}

// Host planning of one batch: tile choice, largest-first queue, descriptors
// and (tensor-core modes) the pre-pass layout.  Touches no device memory.
static bgemm_status_t plan_batch(bgemm_plan_s* p, const int* M, const int* N, const int* K,
                                 const int* lda, const int* ldb, const int* ldc, int batch,
                                 bool first, BatchPlan& bp) {
  std::vector<MatPlan> mp;
  bgemm_status_t st;
  if (p->mode == BGEMM_MODE_SIMT_FP32)
    st = choose_simt(M, N, K, batch, p->facts.num_sms * p->facts.simt_ctas_per_sm, &p->opt, mp);
  else
    st = tc_choose(p, M, N, K, batch, first, mp);
  if (st != BGEMM_SUCCESS) return st;
  std::vector<int> order;
  const long long n_items = order_matrices(mp, order);
  if (n_items > (1LL << 31) - 1024)
    return set_error(BGEMM_ERROR_NOT_SUPPORTED, 0, -1, "batch has %lld tiles", n_items);
  bp.batch = batch;
  bp.descs.resize(batch);
  bp.items.resize((size_t)n_items);
  std::memset(bp.hist, 0, sizeof(bp.hist));
  bp.flops = bp.bytes = 0;
  for (int i = 0; i < batch; ++i) {
    bp.descs[i] = MatDesc{M[i], N[i], K[i], lda[i], ldb[i], ldc[i], mp[i].cfg < 0 ? 0 : mp[i].cfg,
                          p->aux_trans};
    bp.flops += 2.0 * M[i] * (double)N[i] * K[i];
    bp.bytes += 4.0 * ((double)M[i] * K[i] + (double)K[i] * N[i] + (double)M[i] * N[i]);
    if (mp[i].cfg >= 0 && mp[i].cfg < 16) bp.hist[mp[i].cfg]++;
  }
  expand_items(p->mode, p, M, N, mp, order, bp.descs.data(), bp.items.data());
  bp.req = bgemm_plan_requirements_t{};
  bp.req.batch = batch;
  bp.req.tiles = (int)n_items;
  if (p->mode != BGEMM_MODE_SIMT_FP32) tc_layout(p, bp.descs, &bp.req);
  return BGEMM_SUCCESS;
}

// Device buffers for the plan's capacity, pinned staging, launch shapes.
static bgemm_status_t plan_alloc(bgemm_plan_s* p) {
  p->off_descs = kHdrBytes;
  p->off_items = p->off_descs + ((sizeof(MatDesc) * (size_t)p->cap.batch + 255) & ~size_t(255));
  p->mem_bytes = p->off_items + ((sizeof(TileItem) * (size_t)p->cap.tiles + 255) & ~size_t(255));
  cudaError_t e = cudaMalloc(&p->d_mem, p->mem_bytes);
  if (e != cudaSuccess)
    return set_error(BGEMM_ERROR_ALLOC, 0, -1, "device plan memory of %zu bytes: %s", p->mem_bytes,
                     cudaGetErrorString(e));
  for (int s = 0; s < kStageBufs; ++s) {
    e = cudaMallocHost(&p->h_stage[s], p->mem_bytes);
    if (e != cudaSuccess)
      return set_error(BGEMM_ERROR_ALLOC, 0, -1, "pinned staging of %zu bytes: %s", p->mem_bytes,
                       cudaGetErrorString(e));
    e = cudaEventCreateWithFlags(&p->ev_stage[s], cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_error(e, "staging event");
  }
  char* d = static_cast<char*>(p->d_mem);
  p->d_counters = reinterpret_cast<int*>(d);
  p->d_descs = reinterpret_cast<MatDesc*>(d + p->off_descs);
  p->d_items = reinterpret_cast<TileItem*>(d + p->off_items);
  const DeviceFacts& df = p->facts;
  const int ctas_per_sm =
      (p->mode == BGEMM_MODE_SIMT_FP32) ? df.simt_ctas_per_sm : df.tc_ctas_per_sm;
  long long grid = (long long)df.num_sms * ctas_per_sm;
  if (p->opt.max_ctas > 0) grid = std::min<long long>(grid, p->opt.max_ctas);
  grid = std::min<long long>(grid, std::max(p->cap.tiles, 1));
  p->grid = (int)grid;
  p->info.grid = p->grid;
  p->info.device_bytes = p->mem_bytes;
  p->info.kernels_per_execute = (p->mode == BGEMM_MODE_SIMT_FP32) ? 1 : 2;
  if (p->mode != BGEMM_MODE_SIMT_FP32) return tc_alloc(p);
  return BGEMM_SUCCESS;
}

// Stages a planned batch in the next pinned buffer and uploads it on
// `stream`.  The buffer's previous upload (two commits ago) must have been
// consumed before it is rewritten.
static bgemm_status_t plan_commit(bgemm_plan_s* p, BatchPlan& bp, bool first,
                                  cudaStream_t stream) {
  const int s = p->stage;
  cudaError_t e = cudaSuccess;
  if (p->stage_used[s]) {
    e = cudaEventSynchronize(p->ev_stage[s]);
    if (e != cudaSuccess) return cuda_error(e, "waiting for the staging buffer");
  }
  char* h = static_cast<char*>(p->h_stage[s]);
  char* d = static_cast<char*>(p->d_mem);
  std::memset(h, 0, kHdrBytes);
  int* hdr = reinterpret_cast<int*>(h);
  hdr[kHdrItems] = bp.req.tiles;
  hdr[kHdrJobs] = bp.req.pack_jobs;
  if (bp.batch) std::memcpy(h + p->off_descs, bp.descs.data(), sizeof(MatDesc) * bp.descs.size());
  if (!bp.items.empty())
    std::memcpy(h + p->off_items, bp.items.data(), sizeof(TileItem) * bp.items.size());
  auto copy = [&](size_t off, size_t bytes) {
    return bytes ? cudaMemcpyAsync(d + off, h + off, bytes, cudaMemcpyHostToDevice, stream)
                 : cudaSuccess;
  };
  e = copy(0, kHdrBytes);
  if (e == cudaSuccess) e = copy(p->off_descs, sizeof(MatDesc) * bp.descs.size());
  if (e == cudaSuccess) e = copy(p->off_items, sizeof(TileItem) * bp.items.size());
  if (e != cudaSuccess) return cuda_error(e, "descriptor upload");
  p->batch = bp.batch;
  p->n_items = bp.req.tiles;
  p->host_descs.swap(bp.descs);
  if (p->mode != BGEMM_MODE_SIMT_FP32) {
    bgemm_status_t st = tc_commit(p, s, p->batch, first, stream);
    if (st != BGEMM_SUCCESS) return st;
  }
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(stream, &cs);
  if (cs != cudaStreamCaptureStatusNone) {
    // created inside a capture: the graph's copies read this staging buffer
    // whenever it runs, so it may never be rewritten (updates are refused)
    p->staged_in_capture = true;
  } else {
    e = cudaEventRecord(p->ev_stage[s], stream);
    if (e != cudaSuccess) return cuda_error(e, "staging event record");
    p->stage_used[s] = true;
  }
  p->stage = (p->stage + 1) % kStageBufs;
  p->info.batch = p->batch;
  p->info.num_tiles = p->n_items;
  std::memcpy(p->info.tile_config_hist, bp.hist, sizeof(bp.hist));
  p->info.useful_flops = bp.flops;
  p->info.min_bytes = bp.bytes;
  return BGEMM_SUCCESS;
}

static bgemm_status_t check_capacity_option(const bgemm_plan_requirements_t& c) {
  if (c.batch < 0 || c.tiles < 0 || c.pack_jobs < 0)
    return set_error(BGEMM_ERROR_INVALID_VALUE, 11, -1, "negative capacity");
  return BGEMM_SUCCESS;
}

static bgemm_status_t stream_not_capturing(cudaStream_t stream, int arg) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(stream, &cs);
  if (e != cudaSuccess) return cuda_error(e, "cudaStreamIsCapturing");
  if (cs != cudaStreamCaptureStatusNone)
    return set_error(BGEMM_ERROR_INVALID_VALUE, arg, -1,
                     "the stream is capturing: re-planning writes host staging buffers "
                     "that a captured copy would read later");
  return BGEMM_SUCCESS;
}

// Storage order and transposition of the options -> the planned column-major
// product.  Row-major plans compute C^T = op(B)^T op(A)^T: the B array is the
// planned A side (with B's flag) and the A array the planned B side.
static bgemm_status_t set_orientation(bgemm_plan_s* p, int arg) {
  const bgemm_plan_options_t& o = p->opt;
  if ((o.layout != 0 && o.layout != 1) || (o.trans_a != 0 && o.trans_a != 1) ||
      (o.trans_b != 0 && o.trans_b != 1))
    return set_error(BGEMM_ERROR_INVALID_VALUE, arg, -1,
                     "layout, trans_a and trans_b must each be 0 or 1");
  p->row_major = o.layout == BGEMM_ROW_MAJOR;
  const bool pa = p->row_major ? o.trans_b : o.trans_a;
  const bool pb = p->row_major ? o.trans_a : o.trans_b;
  p->aux_trans = (pa ? kTransAFlag : 0) | (pb ? kTransBFlag : 0);
  return BGEMM_SUCCESS;
}

// plan_batch on the planned product's shapes (row-major: swapped operands).
static bgemm_status_t plan_batch_oriented(bgemm_plan_s* p, const int* M, const int* N,
                                          const int* K, const int* lda, const int* ldb,
                                          const int* ldc, int batch, bool first, BatchPlan& bp) {
  if (p->row_major) return plan_batch(p, N, M, K, ldb, lda, ldc, batch, first, bp);
  return plan_batch(p, M, N, K, lda, ldb, ldc, batch, first, bp);
}

// ------------------------------------------------------------ mixed plans --
bgemm_status_t plan_create(bgemm_plan_t* out, const int* M, const int* N, const int* K,
                           const int* lda, const int* ldb, const int* ldc, int batch, int mode,
                           cudaStream_t stream, const bgemm_plan_options_t* opt);
bgemm_status_t plan_update(bgemm_plan_t p, const int* M, const int* N, const int* K,
                           const int* lda, const int* ldb, const int* ldc, int batch,
                           cudaStream_t stream);
bgemm_status_t plan_requirements(const int* M, const int* N, const int* K, const int* lda,
                                 const int* ldb, const int* ldc, int batch, int mode,
                                 const bgemm_plan_options_t* opt,
                                 bgemm_plan_requirements_t* out);
bgemm_status_t plan_destroy(bgemm_plan_t p);

// M of the matrices that run on the SIMT kernel (simt = true) or on the
// tensor cores (simt = false); the others get M = 0, which both planners
// treat as an empty matrix (no tiles, no pre-pass jobs, pointers not read).
static std::vector<int> mixed_mask(const int* M, const int* N, const int* K, int batch,
                                   int below, bool simt) {
  std::vector<int> m((size_t)std::max(batch, 1), 0);
  for (int i = 0; i < batch; ++i) {
    const bool small = std::min(M[i], std::min(N[i], K[i])) < below;
    m[i] = (small == simt) ? M[i] : 0;
  }
  return m;
}

static void mixed_info(bgemm_plan_s* p) {
  const bgemm_plan_info_t& a = p->mix_simt->info;
  const bgemm_plan_info_t& b = p->mix_tc->info;
  p->info = b;
  p->info.batch = p->batch;
  p->info.num_tiles = p->mix_simt->n_items + p->mix_tc->n_items;
  p->info.useful_flops = a.useful_flops + b.useful_flops;
  p->info.min_bytes = a.min_bytes + b.min_bytes;
  p->info.device_bytes = a.device_bytes + b.device_bytes;
  p->info.kernels_per_execute = a.kernels_per_execute + b.kernels_per_execute;
}

static bgemm_status_t plan_create_mixed(bgemm_plan_t* out, const int* M, const int* N,
                                        const int* K, const int* lda, const int* ldb,
                                        const int* ldc, int batch, int mode, cudaStream_t stream,
                                        const bgemm_plan_options_t* opt) {
  bgemm_plan_options_t o = *opt;
  o.simt_below = 0;
  bgemm_plan_options_t os = o;
  os.capacity = bgemm_plan_requirements_t{};
  os.capacity.batch = opt->capacity.batch;
  os.capacity.tiles = opt->capacity.simt_tiles;
  bgemm_plan_options_t ot = o;
  ot.capacity.simt_tiles = 0;
  const std::vector<int> ms = mixed_mask(M, N, K, batch, opt->simt_below, true);
  const std::vector<int> mt = mixed_mask(M, N, K, batch, opt->simt_below, false);
  bgemm_plan_t ps = nullptr, pt = nullptr;
  bgemm_status_t st = plan_create(&ps, ms.data(), N, K, lda, ldb, ldc, batch,
                                  BGEMM_MODE_SIMT_FP32, stream, &os);
  if (st == BGEMM_SUCCESS)
    st = plan_create(&pt, mt.data(), N, K, lda, ldb, ldc, batch, mode, stream, &ot);
  if (st != BGEMM_SUCCESS) {
    plan_destroy(ps);
    return st;
  }
  auto* p = new bgemm_plan_s();
  p->mode = mode;
  p->batch = batch;
  p->facts = pt->facts;
  p->opt = *opt;
  p->mix_simt = ps;
  p->mix_tc = pt;
  p->cap = pt->cap;
  p->cap.simt_tiles = ps->cap.tiles;
  p->grid = pt->grid;
  mixed_info(p);
  *out = p;
  return BGEMM_SUCCESS;
}

bgemm_status_t plan_create(bgemm_plan_t* out, const int* M, const int* N, const int* K,
                           const int* lda, const int* ldb, const int* ldc, int batch, int mode,
                           cudaStream_t stream, const bgemm_plan_options_t* opt) {
  if (!out) return set_error(BGEMM_ERROR_INVALID_VALUE, 1, -1, "plan is NULL");
  *out = nullptr;
  if (opt && opt->simt_below < 0)
    return set_error(BGEMM_ERROR_INVALID_VALUE, 11, -1, "simt_below %d < 0", opt->simt_below);
  if (opt && opt->simt_below > 0 && mode != BGEMM_MODE_SIMT_FP32) {
    bgemm_status_t st = check_args(M, N, K, lda, ldb, ldc, batch, mode, 2, 3, 4, 5, 6, 7, 8, 9,
                                   opt->layout == 1, opt->trans_a != 0, opt->trans_b != 0);
    if (st != BGEMM_SUCCESS) return st;
    return plan_create_mixed(out, M, N, K, lda, ldb, ldc, batch, mode, stream, opt);
  }
  bgemm_plan_s probe;
  probe.opt = opt ? *opt : default_options();
  bgemm_status_t st = set_orientation(&probe, 11);
  if (st != BGEMM_SUCCESS) return st;
  st = check_args(M, N, K, lda, ldb, ldc, batch, mode, 2, 3, 4, 5, 6, 7, 8, 9, probe.row_major,
                  probe.opt.trans_a != 0, probe.opt.trans_b != 0);
  if (st != BGEMM_SUCCESS) return st;
  if (opt && (st = check_capacity_option(opt->capacity)) != BGEMM_SUCCESS) return st;
  DeviceFacts df;
  st = device_facts(&df);
  if (st != BGEMM_SUCCESS) return st;

  auto* p = new bgemm_plan_s();
  p->mode = mode;
  p->facts = df;
  p->opt = probe.opt;
  p->row_major = probe.row_major;
  p->aux_trans = probe.aux_trans;
  p->info.mode = mode;
  BatchPlan bp;
  if (mode != BGEMM_MODE_SIMT_FP32) st = tc_init(p, &p->opt);
  if (st == BGEMM_SUCCESS) st = plan_batch_oriented(p, M, N, K, lda, ldb, ldc, batch, true, bp);
  if (st == BGEMM_SUCCESS) {
    const bgemm_plan_requirements_t& c = p->opt.capacity;
    p->cap = bp.req;
    p->cap.batch = std::max(p->cap.batch, c.batch);
    p->cap.tiles = std::max(p->cap.tiles, c.tiles);
    p->cap.pack_jobs = std::max(p->cap.pack_jobs, c.pack_jobs);
    p->cap.workspace_bytes = std::max(p->cap.workspace_bytes, c.workspace_bytes);
    st = plan_alloc(p);
  }
  if (st == BGEMM_SUCCESS) st = plan_commit(p, bp, true, stream);
  if (st != BGEMM_SUCCESS) {
    free_plan_memory(p);
    delete p;
    return st;
  }
  *out = p;
  return BGEMM_SUCCESS;
}

bgemm_status_t plan_update(bgemm_plan_t p, const int* M, const int* N, const int* K,
                           const int* lda, const int* ldb, const int* ldc, int batch,
                           cudaStream_t stream) {
  if (!p) return set_error(BGEMM_ERROR_INVALID_VALUE, 1, -1, "plan is NULL");
  if (p->mix_tc) {
    bgemm_status_t st = check_args(M, N, K, lda, ldb, ldc, batch, p->mode, 2, 3, 4, 5, 6, 7, 8,
                                   8, p->opt.layout == 1, p->opt.trans_a != 0,
                                   p->opt.trans_b != 0);
    if (st != BGEMM_SUCCESS) return st;
    const std::vector<int> ms = mixed_mask(M, N, K, batch, p->opt.simt_below, true);
    const std::vector<int> mt = mixed_mask(M, N, K, batch, p->opt.simt_below, false);
    // both children check their capacity before they change anything
    bgemm_plan_requirements_t rs{}, rt{};
    bgemm_plan_options_t o = p->opt;
    o.simt_below = 0;
    st = plan_requirements(ms.data(), N, K, lda, ldb, ldc, batch, BGEMM_MODE_SIMT_FP32, &o, &rs);
    if (st == BGEMM_SUCCESS)
      st = plan_requirements(mt.data(), N, K, lda, ldb, ldc, batch, p->mode, &o, &rt);
    if (st != BGEMM_SUCCESS) return st;
    if (batch > p->cap.batch || rs.tiles > p->mix_simt->cap.tiles ||
        rt.tiles > p->mix_tc->cap.tiles || rt.pack_jobs > p->mix_tc->cap.pack_jobs ||
        rt.workspace_bytes > p->mix_tc->cap.workspace_bytes)
      return set_error(BGEMM_ERROR_NOT_SUPPORTED, 0, -1,
                       "batch needs %d SIMT tiles, %d tensor-core tiles, %d pack jobs, %zu "
                       "workspace bytes; the mixed plan holds %d, %d, %d, %zu",
                       rs.tiles, rt.tiles, rt.pack_jobs, rt.workspace_bytes,
                       p->mix_simt->cap.tiles, p->mix_tc->cap.tiles, p->mix_tc->cap.pack_jobs,
                       p->mix_tc->cap.workspace_bytes);
    st = plan_update(p->mix_simt, ms.data(), N, K, lda, ldb, ldc, batch, stream);
    if (st == BGEMM_SUCCESS)
      st = plan_update(p->mix_tc, mt.data(), N, K, lda, ldb, ldc, batch, stream);
    if (st != BGEMM_SUCCESS) return st;
    p->batch = batch;
    mixed_info(p);
    return BGEMM_SUCCESS;
  }
  bgemm_status_t st =
      check_args(M, N, K, lda, ldb, ldc, batch, p->mode, 2, 3, 4, 5, 6, 7, 8, 8, p->row_major,
                 p->opt.trans_a != 0, p->opt.trans_b != 0);
  if (st != BGEMM_SUCCESS) return st;
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != p->facts.device)
    return set_error(BGEMM_ERROR_INVALID_VALUE, 1, -1, "plan belongs to device %d, current is %d",
                     p->facts.device, dev);
  if ((st = stream_not_capturing(stream, 9)) != BGEMM_SUCCESS) return st;
  if (p->staged_in_capture)
    return set_error(BGEMM_ERROR_NOT_SUPPORTED, 1, -1,
                     "the plan was created during a stream capture; the captured upload reads "
                     "its staging, so it cannot be updated");
  if (batch > p->cap.batch)
    return set_error(BGEMM_ERROR_NOT_SUPPORTED, 8, -1, "batch %d exceeds the plan's capacity %d",
                     batch, p->cap.batch);
  BatchPlan bp;
  st = plan_batch_oriented(p, M, N, K, lda, ldb, ldc, batch, false, bp);
  if (st != BGEMM_SUCCESS) return st;
  const bgemm_plan_requirements_t& r = bp.req;
  if (r.tiles > p->cap.tiles || r.pack_jobs > p->cap.pack_jobs ||
      r.workspace_bytes > p->cap.workspace_bytes)
    return set_error(BGEMM_ERROR_NOT_SUPPORTED, 0, -1,
                     "batch needs %d tiles, %d pack jobs, %zu workspace bytes; the plan holds "
                     "%d, %d, %zu",
                     r.tiles, r.pack_jobs, r.workspace_bytes, p->cap.tiles, p->cap.pack_jobs,
                     p->cap.workspace_bytes);
  return plan_commit(p, bp, false, stream);
}

bgemm_status_t plan_requirements(const int* M, const int* N, const int* K, const int* lda,
                                 const int* ldb, const int* ldc, int batch, int mode,
                                 const bgemm_plan_options_t* opt,
                                 bgemm_plan_requirements_t* out) {
  if (opt && opt->simt_below > 0 && mode != BGEMM_MODE_SIMT_FP32) {
    if (!out) return set_error(BGEMM_ERROR_INVALID_VALUE, 10, -1, "out is NULL");
    bgemm_status_t st = check_args(M, N, K, lda, ldb, ldc, batch, mode, 1, 2, 3, 4, 5, 6, 7, 8,
                                   opt->layout == 1, opt->trans_a != 0, opt->trans_b != 0);
    if (st != BGEMM_SUCCESS) return st;
    bgemm_plan_options_t o = *opt;
    o.simt_below = 0;
    const std::vector<int> ms = mixed_mask(M, N, K, batch, opt->simt_below, true);
    const std::vector<int> mt = mixed_mask(M, N, K, batch, opt->simt_below, false);
    bgemm_plan_requirements_t rs{}, rt{};
    st = plan_requirements(ms.data(), N, K, lda, ldb, ldc, batch, BGEMM_MODE_SIMT_FP32, &o, &rs);
    if (st == BGEMM_SUCCESS) st = plan_requirements(mt.data(), N, K, lda, ldb, ldc, batch, mode,
                                                    &o, &rt);
    if (st != BGEMM_SUCCESS) return st;
    *out = rt;
    out->simt_tiles = rs.tiles;
    return BGEMM_SUCCESS;
  }
  bgemm_plan_s p;
  p.opt = opt ? *opt : default_options();
  bgemm_status_t st = set_orientation(&p, 9);
  if (st != BGEMM_SUCCESS) return st;
  st = check_args(M, N, K, lda, ldb, ldc, batch, mode, 1, 2, 3, 4, 5, 6, 7, 8, p.row_major,
                  p.opt.trans_a != 0, p.opt.trans_b != 0);
  if (st != BGEMM_SUCCESS) return st;
  if (!out) return set_error(BGEMM_ERROR_INVALID_VALUE, 10, -1, "out is NULL");
  DeviceFacts df;
  st = device_facts(&df);
  if (st != BGEMM_SUCCESS) return st;
  p.mode = mode;
  p.facts = df;
  BatchPlan bp;
  if (mode != BGEMM_MODE_SIMT_FP32) st = tc_init(&p, &p.opt);
  if (st == BGEMM_SUCCESS) st = plan_batch_oriented(&p, M, N, K, lda, ldb, ldc, batch, true, bp);
  if (p.tc) tc_plan_release(&p);
  if (st == BGEMM_SUCCESS) *out = bp.req;
  return st;
}

bgemm_status_t plan_execute(bgemm_plan_t p, float alpha, const float* const* dA,
                            const float* const* dB, float beta, float* const* dC,
                            cudaStream_t stream) {
  if (!p) return set_error(BGEMM_ERROR_INVALID_VALUE, 1, -1, "plan is NULL");
  if (p->mix_tc) {
    // the matrices of the two children are disjoint: SIMT first, then the
    // tensor-core pre-pass and GEMM, in stream order
    bgemm_status_t st = plan_execute(p->mix_simt, alpha, dA, dB, beta, dC, stream);
    if (st != BGEMM_SUCCESS) return st;
    return plan_execute(p->mix_tc, alpha, dA, dB, beta, dC, stream);
  }
  if (p->cap.tiles == 0) return BGEMM_SUCCESS;
  if (!dA) return set_error(BGEMM_ERROR_INVALID_VALUE, 3, -1, "dA is NULL");
  if (!dB) return set_error(BGEMM_ERROR_INVALID_VALUE, 4, -1, "dB is NULL");
  if (!dC) return set_error(BGEMM_ERROR_INVALID_VALUE, 6, -1, "dC is NULL");
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != p->facts.device)
    return set_error(BGEMM_ERROR_INVALID_VALUE, 1, -1, "plan belongs to device %d, current is %d",
                     p->facts.device, dev);
  if (p->row_major) std::swap(dA, dB);
  if (p->mode == BGEMM_MODE_SIMT_FP32) {
    SimtParams sp{p->d_descs, p->d_items,  p->n_items, p->d_counters + kHdrItems,
                  p->d_counters, alpha,    beta,       dA, dB, dC};
    if (p->ev_start) cudaEventRecord(p->ev_start, stream);
    cudaError_t e = simt_launch(sp, p->grid, stream, p->aux_trans != 0);
    if (p->ev_stop) cudaEventRecord(p->ev_stop, stream);
    if (e != cudaSuccess) return cuda_error(e, "SIMT launch");
    return BGEMM_SUCCESS;
  }
  return tc_execute(p, alpha, dA, dB, beta, dC, stream);
}

bgemm_status_t plan_destroy(bgemm_plan_t p) {
  if (!p) return BGEMM_SUCCESS;
  if (p->mix_tc) {
    plan_destroy(p->mix_simt);
    plan_destroy(p->mix_tc);
    delete p;
    return BGEMM_SUCCESS;
  }
  free_plan_memory(p);
  delete p;
  return BGEMM_SUCCESS;
}

// ---------------------------------------------------------- plan cache ----
// Plans of the one-shot entries, keyed by the batch's shape MULTISET: the
// (M, N, K, lda, ldb, ldc) tuples sorted, plus device, mode and orientation.
// The reference sorts its shape file offline by K and tile class before a
// run (ROCm/data/sort.cpp:17-60) so that its dense grid meets similar tiles
// together; here the planner orders the tile queue itself, so a batch's
// order never matters for speed, and the cache makes it not matter for
// planning either: the same shapes in another order reuse the plan through
// plan_update (host planning + one upload; the device buffers, the
// workspace and the kernels stay), and the result is bit-identical because
// each matrix's tile choice depends only on its shape and on the multiset.
//
// The stream is not part of the key: an entry remembers the stream of its
// last execute and an event recorded after it, and a call on another stream
// first makes that stream wait for the event.  Entries are evicted least
// recently used first when the cached device bytes would exceed the budget
// (bgemm_plan_cache_set_limit; default a third of the device's memory), and
// an allocation failure evicts every other entry of the device and retries
// once.  An entry that was created or used while a stream was capturing is
// pinned: a captured graph may replay it at any time, so it is never freed
// or re-planned.
namespace {
struct CacheEntry {
  bgemm_plan_t plan = nullptr;
  int dev = 0;
  std::string canon;          // device | mode | orientation | sorted tuples
  std::vector<int> order;     // the committed batch's arrays M|N|K|lda|ldb|ldc
  cudaStream_t stream = nullptr;  // stream of the last execute
  cudaEvent_t done = nullptr;     // recorded after the last execute (outside capture)
  bool done_valid = false;
  bool pinned = false;        // used inside a stream capture
  size_t bytes = 0;           // device bytes the plan owns
};
struct PlanCache {
  std::mutex mu;
  std::list<CacheEntry> lru;  // front = most recent
  size_t limit = 0;           // 0: default of the device, set at first use
  bool limit_set = false;
  long long hits = 0, reorders = 0, misses = 0, evictions = 0;
  ~PlanCache() {
    // plans are intentionally leaked at process exit: the CUDA context may
    // already be gone, and freeing into it would fail.
  }
};
PlanCache& cache() {
  static PlanCache* c = new PlanCache();
  return *c;
}

size_t cache_bytes(const PlanCache& c, int dev) {
  size_t b = 0;
  for (const CacheEntry& e : c.lru)
    if (e.dev == dev) b += e.bytes;
  return b;
}

size_t cache_limit(PlanCache& c) {
  if (!c.limit_set) {
    size_t free_b = 0, total_b = 0;
    c.limit = cudaMemGetInfo(&free_b, &total_b) == cudaSuccess ? total_b / 3 : (size_t)8 << 30;
    c.limit_set = true;
  }
  return c.limit;
}

void drop_entry(PlanCache& c, std::list<CacheEntry>::iterator it) {
  plan_destroy(it->plan);  // cudaFree waits for work still using it
  if (it->done) cudaEventDestroy(it->done);
  c.lru.erase(it);
  ++c.evictions;
}

// Evicts unpinned entries of `dev`, least recently used first, until `need`
// more bytes fit under the limit (or nothing evictable is left).
void make_room(PlanCache& c, int dev, size_t need, bool all) {
  const size_t lim = cache_limit(c);
  while (all || cache_bytes(c, dev) + need > lim) {
    auto victim = c.lru.end();
    for (auto it = c.lru.begin(); it != c.lru.end(); ++it)
      if (it->dev == dev && !it->pinned) victim = it;  // the last match is the oldest
    if (victim == c.lru.end()) return;
    drop_entry(c, victim);
  }
}

std::string canonical_key(const int* M, const int* N, const int* K, const int* lda,
                          const int* ldb, const int* ldc, int batch, int dev, int mode,
                          int orient) {
  std::vector<std::array<int, 6>> t((size_t)batch);
  for (int i = 0; i < batch; ++i) t[i] = {M[i], N[i], K[i], lda[i], ldb[i], ldc[i]};
  std::sort(t.begin(), t.end());
  std::string key(sizeof(int) * (3 + 6 * (size_t)batch), '\0');
  int hdr[3] = {dev, mode, orient};
  std::memcpy(&key[0], hdr, sizeof(hdr));
  if (batch) std::memcpy(&key[sizeof(hdr)], t.data(), sizeof(int) * 6 * (size_t)batch);
  return key;
}
}  // namespace

// Looks up (or builds) the plan of this batch and runs it on `stream`.
bgemm_status_t cached_execute(const int* M, const int* N, const int* K, const int* lda,
                              const int* ldb, const int* ldc, int batch, int mode,
                              cudaStream_t stream, int layout, int ta, int tb, float alpha,
                              const float* const* dA, const float* const* dB, float beta,
                              float* const* dC) {
  int dev = 0;
  cudaGetDevice(&dev);
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(stream, &cs);
  const bool capturing = cs != cudaStreamCaptureStatusNone;
  const int orient = layout | (ta << 1) | (tb << 2);
  std::string canon = canonical_key(M, N, K, lda, ldb, ldc, batch, dev, mode, orient);
  std::vector<int> order(6 * (size_t)batch);
  {
    int* o = order.data();
    for (const int* a : {M, N, K, lda, ldb, ldc}) {
      if (batch) std::memcpy(o, a, sizeof(int) * (size_t)batch);
      o += batch;
    }
  }
  PlanCache& c = cache();
  std::lock_guard<std::mutex> lk(c.mu);
  // 1. an entry holding this exact order; 2. one holding another order that
  // may be re-planned (outside a capture, not pinned)
  auto exact = c.lru.end(), other = c.lru.end();
  for (auto it = c.lru.begin(); it != c.lru.end(); ++it) {
    if (it->dev != dev || it->canon != canon) continue;
    const bool stream_ok = it->stream == stream || !capturing;
    if (it->order == order && stream_ok) {
      exact = it;
      break;
    }
    if (other == c.lru.end() && !capturing && !it->pinned) other = it;
  }
  auto ent = exact != c.lru.end() ? exact : other;
  bgemm_status_t st = BGEMM_SUCCESS;
  if (ent != c.lru.end()) {
    if (ent->stream != stream && ent->done_valid) {
      cudaError_t e = cudaStreamWaitEvent(stream, ent->done, 0);
      if (e != cudaSuccess) return cuda_error(e, "ordering a cached plan across streams");
    }
    if (ent == other) {
      st = plan_update(ent->plan, M, N, K, lda, ldb, ldc, batch, stream);
      if (st == BGEMM_SUCCESS) {
        ent->order.swap(order);
        ++c.reorders;
      } else {
        clear_error();
        ent = c.lru.end();  // not re-plannable: build a plan of its own below
      }
    } else {
      ++c.hits;
    }
    if (ent != c.lru.end()) c.lru.splice(c.lru.begin(), c.lru, ent);
  }
  if (ent == c.lru.end()) {
    ++c.misses;
    bgemm_plan_options_t opt = default_options();
    opt.layout = layout;
    opt.trans_a = ta;
    opt.trans_b = tb;
    if (!capturing) {
      // room for the new plan before it allocates
      bgemm_plan_requirements_t req{};
      if (plan_requirements(M, N, K, lda, ldb, ldc, batch, mode, &opt, &req) == BGEMM_SUCCESS)
        make_room(c, dev,
                  req.workspace_bytes + 32 * (size_t)req.batch + 8 * (size_t)req.tiles + 65536,
                  false);
    }
    bgemm_plan_t p = nullptr;
    st = plan_create(&p, M, N, K, lda, ldb, ldc, batch, mode, stream, &opt);
    if (st == BGEMM_ERROR_ALLOC && !capturing) {
      make_room(c, dev, 0, true);
      st = plan_create(&p, M, N, K, lda, ldb, ldc, batch, mode, stream, &opt);
    }
    if (st != BGEMM_SUCCESS) return st;
    CacheEntry e;
    e.plan = p;
    e.dev = dev;
    e.canon.swap(canon);
    e.order.swap(order);
    e.bytes = p->info.device_bytes;
    cudaEventCreateWithFlags(&e.done, cudaEventDisableTiming);
    c.lru.push_front(std::move(e));
    ent = c.lru.begin();
  }
  st = plan_execute(ent->plan, alpha, dA, dB, beta, dC, stream);
  ent->stream = stream;
  if (capturing) {
    ent->pinned = true;
    ent->done_valid = false;
  } else if (ent->done) {
    ent->done_valid = cudaEventRecord(ent->done, stream) == cudaSuccess;
  }
  return st;
}

}  // namespace bgemm

// ================================================================ C ABI ====
using namespace bgemm;

namespace bgemm {
// Shared body of the one-shot entries; arg[] holds the caller's argument
// numbers of M, N, K, dA, lda, dB, ldb, dC, ldc, batch, mode.
static bgemm_status_t vbatched(int layout, int ta, int tb, const int* M, const int* N,
                               const int* K, float alpha, const float* const* dA, const int* lda,
                               const float* const* dB, const int* ldb, float beta,
                               float* const* dC, const int* ldc, int batch, int mode,
                               cudaStream_t stream, const int (&arg)[11]) {
  bgemm_status_t st = check_args(M, N, K, lda, ldb, ldc, batch, mode, arg[0], arg[1], arg[2],
                                 arg[4], arg[6], arg[8], arg[9], arg[10], layout == 1, ta, tb);
  if (st != BGEMM_SUCCESS || batch == 0) return st;
  bool any = false;
  for (int i = 0; i < batch && !any; ++i) any = M[i] > 0 && N[i] > 0;
  if (!any) return BGEMM_SUCCESS;
  if (!dA) return set_error(BGEMM_ERROR_INVALID_VALUE, arg[3], -1, "dA is NULL");
  if (!dB) return set_error(BGEMM_ERROR_INVALID_VALUE, arg[5], -1, "dB is NULL");
  if (!dC) return set_error(BGEMM_ERROR_INVALID_VALUE, arg[7], -1, "dC is NULL");
  st = cached_execute(M, N, K, lda, ldb, ldc, batch, mode, stream, layout, ta, tb, alpha, dA,
                      dB, beta, dC);
  if (st == BGEMM_ERROR_INVALID_VALUE && t_err_arg > 0) {
    // plan_execute numbers its own arguments; map them to this entry point
    const int map[7] = {0, 0, 0, arg[3], arg[5], 0, arg[7]};
    if (t_err_arg < 7 && map[t_err_arg]) t_err_arg = map[t_err_arg];
  }
  return st;
}
}  // namespace bgemm

extern "C" {

bgemm_status_t bgemm_sgemm_vbatched(const int* M, const int* N, const int* K, float alpha,
                                    const float* const* dA, const int* lda,
                                    const float* const* dB, const int* ldb, float beta,
                                    float* const* dC, const int* ldc, int batch,
                                    bgemm_mode_t mode, bgemm_stream_t stream) {
  clear_error();
  static const int arg[11] = {1, 2, 3, 5, 6, 7, 8, 10, 11, 12, 13};
  return vbatched(0, 0, 0, M, N, K, alpha, dA, lda, dB, ldb, beta, dC, ldc, batch, (int)mode,
                  stream, arg);
}

bgemm_status_t bgemm_sgemm_vbatched_ex(bgemm_layout_t layout, bgemm_op_t transA,
                                       bgemm_op_t transB, const int* M, const int* N,
                                       const int* K, float alpha, const float* const* dA,
                                       const int* lda, const float* const* dB, const int* ldb,
                                       float beta, float* const* dC, const int* ldc, int batch,
                                       bgemm_mode_t mode, bgemm_stream_t stream) {
  clear_error();
  if (layout != BGEMM_COL_MAJOR && layout != BGEMM_ROW_MAJOR)
    return set_error(BGEMM_ERROR_INVALID_VALUE, 1, -1, "unknown layout %d", (int)layout);
  if (transA != BGEMM_OP_N && transA != BGEMM_OP_T)
    return set_error(BGEMM_ERROR_INVALID_VALUE, 2, -1, "unknown transA %d", (int)transA);
  if (transB != BGEMM_OP_N && transB != BGEMM_OP_T)
    return set_error(BGEMM_ERROR_INVALID_VALUE, 3, -1, "unknown transB %d", (int)transB);
  static const int arg[11] = {4, 5, 6, 8, 9, 10, 11, 13, 14, 15, 16};
  return vbatched((int)layout, (int)transA, (int)transB, M, N, K, alpha, dA, lda, dB, ldb, beta,
                  dC, ldc, batch, (int)mode, stream, arg);
}

bgemm_status_t bgemm_plan_create(bgemm_plan_t* plan, const int* M, const int* N, const int* K,
                                 const int* lda, const int* ldb, const int* ldc, int batch,
                                 bgemm_mode_t mode, bgemm_stream_t stream) {
  clear_error();
  return plan_create(plan, M, N, K, lda, ldb, ldc, batch, (int)mode, stream, nullptr);
}

bgemm_status_t bgemm_plan_create_ex(bgemm_plan_t* plan, const int* M, const int* N,
                                    const int* K, const int* lda, const int* ldb,
                                    const int* ldc, int batch, bgemm_mode_t mode,
                                    bgemm_stream_t stream, const bgemm_plan_options_t* options) {
  clear_error();
  if (options && options->force_tile_config >= 0) {
    const int ncfg = (mode == BGEMM_MODE_SIMT_FP32) ? kSimtNumCfgs : kTcNumCfgs;
    if (options->force_tile_config >= ncfg)
      return set_error(BGEMM_ERROR_INVALID_VALUE, 11, -1, "force_tile_config %d >= %d",
                       options->force_tile_config, ncfg);
  }
  return plan_create(plan, M, N, K, lda, ldb, ldc, batch, (int)mode, stream, options);
}

bgemm_status_t bgemm_plan_execute(bgemm_plan_t plan, float alpha, const float* const* dA,
                                  const float* const* dB, float beta, float* const* dC,
                                  bgemm_stream_t stream) {
  clear_error();
  return plan_execute(plan, alpha, dA, dB, beta, dC, stream);
}

bgemm_status_t bgemm_plan_info(bgemm_plan_t plan, bgemm_plan_info_t* info) {
  clear_error();
  if (!plan) return set_error(BGEMM_ERROR_INVALID_VALUE, 1, -1, "plan is NULL");
  if (!info) return set_error(BGEMM_ERROR_INVALID_VALUE, 2, -1, "info is NULL");
  *info = plan->info;
  return BGEMM_SUCCESS;
}

bgemm_status_t bgemm_plan_requirements(const int* M, const int* N, const int* K,
                                       const int* lda, const int* ldb, const int* ldc, int batch,
                                       bgemm_mode_t mode, const bgemm_plan_options_t* options,
                                       bgemm_plan_requirements_t* out) {
  clear_error();
  if (options && options->force_tile_config >= 0) {
    const int ncfg = (mode == BGEMM_MODE_SIMT_FP32) ? kSimtNumCfgs : kTcNumCfgs;
    if (options->force_tile_config >= ncfg)
      return set_error(BGEMM_ERROR_INVALID_VALUE, 9, -1, "force_tile_config %d >= %d",
                       options->force_tile_config, ncfg);
  }
  return plan_requirements(M, N, K, lda, ldb, ldc, batch, (int)mode, options, out);
}

bgemm_status_t bgemm_plan_update(bgemm_plan_t plan, const int* M, const int* N, const int* K,
                                 const int* lda, const int* ldb, const int* ldc, int batch,
                                 bgemm_stream_t stream) {
  clear_error();
  return plan_update(plan, M, N, K, lda, ldb, ldc, batch, stream);
}

bgemm_status_t bgemm_plan_capacity(bgemm_plan_t plan, bgemm_plan_requirements_t* out) {
  clear_error();
  if (!plan) return set_error(BGEMM_ERROR_INVALID_VALUE, 1, -1, "plan is NULL");
  if (!out) return set_error(BGEMM_ERROR_INVALID_VALUE, 2, -1, "out is NULL");
  *out = plan->cap;
  return BGEMM_SUCCESS;
}

bgemm_status_t bgemm_plan_set_cta_timer(bgemm_plan_t plan, void* d_times) {
  clear_error();
  if (!plan) return set_error(BGEMM_ERROR_INVALID_VALUE, 1, -1, "plan is NULL");
  if (plan->mode == BGEMM_MODE_SIMT_FP32)
    return set_error(BGEMM_ERROR_NOT_SUPPORTED, 1, -1,
                     "per-CTA timing is a hook of the tensor-core GEMM kernels");
  if (plan->mix_tc) plan = plan->mix_tc;
  plan->d_cta_times = static_cast<unsigned long long*>(d_times);
  return BGEMM_SUCCESS;
}

bgemm_status_t bgemm_plan_set_kernel_events(bgemm_plan_t plan, void* ev_start, void* ev_stop) {
  clear_error();
  if (!plan) return set_error(BGEMM_ERROR_INVALID_VALUE, 1, -1, "plan is NULL");
  if (plan->mix_tc) plan = plan->mix_tc;  // the tensor-core GEMM, the dominant kernel
  plan->ev_start = static_cast<cudaEvent_t>(ev_start);
  plan->ev_stop = static_cast<cudaEvent_t>(ev_stop);
  return BGEMM_SUCCESS;
}

bgemm_status_t bgemm_plan_check_device(bgemm_plan_t plan, bgemm_stream_t stream) {
  clear_error();
  if (!plan) return set_error(BGEMM_ERROR_INVALID_VALUE, 1, -1, "plan is NULL");
  cudaError_t e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return cuda_error(e, "cudaStreamSynchronize");
  if (plan->mix_tc) plan = plan->mix_tc;
  if (plan->mode == BGEMM_MODE_SIMT_FP32) return BGEMM_SUCCESS;
  return tc_check_device(plan, stream);
}

bgemm_status_t bgemm_plan_destroy(bgemm_plan_t plan) {
  clear_error();
  return plan_destroy(plan);
}

int bgemm_last_error_arg(int* matrix) {
  if (matrix) *matrix = t_err_mat;
  return t_err_arg;
}

const char* bgemm_last_error_message(void) { return t_err_msg; }

const char* bgemm_status_string(bgemm_status_t s) {
  switch (s) {
    case BGEMM_SUCCESS: return "BGEMM_SUCCESS";
    case BGEMM_ERROR_INVALID_VALUE: return "BGEMM_ERROR_INVALID_VALUE";
    case BGEMM_ERROR_NOT_SUPPORTED: return "BGEMM_ERROR_NOT_SUPPORTED";
    case BGEMM_ERROR_ALLOC: return "BGEMM_ERROR_ALLOC";
    case BGEMM_ERROR_CUDA: return "BGEMM_ERROR_CUDA";
    case BGEMM_ERROR_DEVICE_TIMEOUT: return "BGEMM_ERROR_DEVICE_TIMEOUT";
    case BGEMM_ERROR_INTERNAL: return "BGEMM_ERROR_INTERNAL";
  }
  return "BGEMM_STATUS_UNKNOWN";
}

bgemm_status_t bgemm_device_info(int* num_sms, int* simt_ctas_per_sm, int* tc_ctas_per_sm) {
  clear_error();
  DeviceFacts f;
  bgemm_status_t st = device_facts(&f);
  if (st != BGEMM_SUCCESS) return st;
  if (num_sms) *num_sms = f.num_sms;
  if (simt_ctas_per_sm) *simt_ctas_per_sm = f.simt_ctas_per_sm;
  if (tc_ctas_per_sm) *tc_ctas_per_sm = f.tc_ctas_per_sm;
  return BGEMM_SUCCESS;
}

int bgemm_version(void) { return 100; }

bgemm_status_t bgemm_plan_cache_set_limit(size_t bytes) {
  clear_error();
  PlanCache& c = cache();
  std::lock_guard<std::mutex> lk(c.mu);
  if (bytes == 0) {
    c.limit_set = false;  // back to the default, taken at the next use
  } else {
    c.limit = bytes;
    c.limit_set = true;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess) make_room(c, dev, 0, false);
  return BGEMM_SUCCESS;
}

bgemm_status_t bgemm_plan_cache_clear(void) {
  clear_error();
  PlanCache& c = cache();
  std::lock_guard<std::mutex> lk(c.mu);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
  make_room(c, dev, 0, true);
  return BGEMM_SUCCESS;
}

int bgemm_debug_plan_cache_stats(long long* entries, long long* bytes, long long* hits,
                                 long long* reorders, long long* misses, long long* evictions,
                                 long long* limit) {
  PlanCache& c = cache();
  std::lock_guard<std::mutex> lk(c.mu);
  int dev = 0;
  cudaGetDevice(&dev);
  long long n = 0;
  for (const CacheEntry& e : c.lru) n += e.dev == dev;
  if (entries) *entries = n;
  if (bytes) *bytes = (long long)cache_bytes(c, dev);
  if (hits) *hits = c.hits;
  if (reorders) *reorders = c.reorders;
  if (misses) *misses = c.misses;
  if (evictions) *evictions = c.evictions;
  if (limit) *limit = c.limit_set ? (long long)c.limit : 0;
  return 0;
}

int bgemm_debug_compare_tensor_maps(void* plan, void* stream, int* n_maps, int* n_diff,
                                    int* first_byte) {
  clear_error();
  if (!plan || !n_maps || !n_diff || !first_byte) return -1;
  return tc_debug_compare_tmaps(static_cast<bgemm_plan_s*>(plan),
                                static_cast<cudaStream_t>(stream), n_maps, n_diff, first_byte);
}

int bgemm_debug_tc_plan(const int* M, const int* N, const int* K, int batch, int mode,
                        int family, int slots, int clusters, int* cfg_out, int* items_out,
                        int max_items, long long* ws_out, int* jobs_out, int max_jobs,
                        int* n_jobs, long long* ws_bytes, int* kernel_family) {
  clear_error();
  if (batch < 0 || (batch > 0 && (!M || !N || !K)) || !n_jobs || !ws_bytes || !kernel_family)
    return -1;
  for (int i = 0; i < batch; ++i)
    if (M[i] < 0 || N[i] < 0 || K[i] < 0) return -1;
  return debug_tc_plan(M, N, K, batch, mode, family, slots, clusters, cfg_out, items_out,
                       max_items, ws_out, jobs_out, max_jobs, n_jobs, ws_bytes, kernel_family);
}

int bgemm_debug_simt_queue(const int* M, const int* N, const int* K, int batch, int slots,
                           int force_cfg, int rebalance, int* cfg_out, int* items_out,
                           int max_items) {
  clear_error();
  if (batch < 0 || (batch > 0 && (!M || !N || !K))) return -1;
  for (int i = 0; i < batch; ++i)
    if (M[i] < 0 || N[i] < 0 || K[i] < 0) return -1;
  return debug_simt_queue(M, N, K, batch, slots, force_cfg, rebalance, cfg_out, items_out,
                          max_items);
}

}  // extern "C"
