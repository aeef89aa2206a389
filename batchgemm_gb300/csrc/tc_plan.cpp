// tc_plan.cpp -- planner of the tensor-core modes: per-matrix tile
// configuration (orientation and MMA width), split-operand workspace layout,
// pack jobs, per-matrix TMA tensor maps, and the two launches of an execute.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include <cudaTypedefs.h>

#include "bgemm_debug.h"
#include "plan_internal.h"
#include "tc_common.h"
#include "tile_table.h"

namespace bgemm {

struct TcPlan {
  int kind = kKindTF32;
  int split = 1;             // the kernels read hi/lo pairs (kind TF32/BF16 split modes)
  bool split_mode = true;    // the plan's mode is TF32X3 or BF16X3
  int want_family = 0;       // 0: cost model, 1: one-SM, 2: CTA pair
  bool pair = false;         // CTA-pair kernel (tc2_kernel.cu)
  int clusters = 0;          // CTA pairs resident at once
  bool host_tmaps = false;   // encode every tensor map on the host (comparison path)
  // capacity and device memory
  int cap_batch = 0, cap_jobs = 0;
  size_t cap_ws = 0;
  void* d_ws = nullptr;      // split operands
  void* d_mem = nullptr;     // templates | tensor maps | pack descs | jobs | error word
  void* h_stage[kStageBufs] = {};  // pinned staging ring, same layout as d_mem
  size_t off_tm = 0, off_pd = 0, off_jobs = 0, off_err = 0, mem_bytes = 0;
  CUtensorMap* d_templ = nullptr;
  CUtensorMap* d_tmaps = nullptr;
  PackDesc* d_pdescs = nullptr;
  PackJob* d_jobs = nullptr;
  int* d_err = nullptr;
  int n_jobs = 0;
  int pack_grid = 1;
  // layout of the last planned batch, uploaded by tc_commit
  std::vector<PackDesc> pd;
  std::vector<PackJob> jobs;
};

static inline long long cdiv(long long a, long long b) { return (a + b - 1) / b; }

// ------------------------------------------------------ promotion schedule --
static std::mutex g_sched_mu;
static bool g_sched_override[3] = {false, false, false};
static TcSchedule g_sched[3];

TcSchedule tc_schedule(int mode) {
  TcSchedule s{};
  const int m = (mode >= BGEMM_MODE_TF32 && mode <= BGEMM_MODE_BF16X3) ? mode - 1 : 1;
  std::lock_guard<std::mutex> lk(g_sched_mu);
  if (g_sched_override[m]) return g_sched[m];
  for (int b = 0; b < kTcSchedBuckets; ++b) s.set(b, kTcGroupTable[m][b]);
  return s;
}
static inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

static int g_mode = BGEMM_MODE_TF32X3;
static bool g_pair = false;

// Tile time from the (autotuned) cost table of the mode.  Only the
// configurations of the plan's kernel (one-SM or CTA-pair) are offered.
static bool tc_eval(int c, int M, int N, int K, long long* tiles, double* t_tile) {
  if (tc_cfg_pair(c) != g_pair) return false;
  if (g_pair && !tc2_cfg_valid(c)) return false;
  TileCost tc = kTcCost[g_mode - 1][c];
  if (tc.b_ns <= 0.0f) {
    // not in the table (not yet tuned): the 3xTF32 cost of the same tile,
    // halved per unit of K for a mode that loads and multiplies one part
    const TileCost& t3 = kTcCost[BGEMM_MODE_TF32X3 - 1][c];
    if (t3.b_ns <= 0.0f) return false;
    tc = TileCost{t3.a_ns, g_mode == BGEMM_MODE_TF32X3 ? t3.b_ns : 0.5f * t3.b_ns};
  }
  const bool swap = tc_cfg_swap(c);
  const int bm = g_pair ? 256 : kTcBM;
  const int bn = g_pair ? tc2_cfg_bn(c) : tc_cfg_bn(c);
  const long long ra = swap ? N : M, rb = swap ? M : N;
  if (cdiv(ra, bm) > 65535 || cdiv(rb, bn) > 65535) return false;
  *tiles = cdiv(ra, bm) * cdiv(rb, bn);
  *t_tile = tc.a_ns + tc.b_ns * (double)K;
  return true;
}

bgemm_status_t tc_init(bgemm_plan_s* p, const bgemm_plan_options_t* opt, int clusters) {
  auto* t = new TcPlan();
  p->tc = t;
  t->kind = (p->mode == BGEMM_MODE_BF16X3) ? kKindBF16 : kKindTF32;
  t->split_mode = p->mode != BGEMM_MODE_TF32;
  t->split = t->split_mode ? 1 : 0;
  t->host_tmaps = opt->host_tensor_maps != 0;
  int fam = opt->kernel_family;
  if (fam < 0 || fam > 2)
    return set_error(BGEMM_ERROR_INVALID_VALUE, 11, -1, "kernel_family %d is not 0, 1 or 2", fam);
  if (opt->force_tile_config >= 0) {
    const int forced = tc_cfg_pair(opt->force_tile_config) ? 2 : 1;
    if (fam != 0 && fam != forced)
      return set_error(BGEMM_ERROR_INVALID_VALUE, 11, -1,
                       "force_tile_config %d belongs to kernel family %d, not %d",
                       opt->force_tile_config, forced, fam);
    fam = forced;
  }
  t->clusters = clusters >= 0 ? clusters : tc2_max_clusters();
  if (fam == 2 && t->clusters < 1)
    return set_error(BGEMM_ERROR_NOT_SUPPORTED, 11, -1, "no CTA pair fits on this device");
  t->want_family = fam;
  return BGEMM_SUCCESS;
}

bgemm_status_t tc_choose(bgemm_plan_s* p, const int* M, const int* N, const int* K, int batch,
                         bool first, std::vector<MatPlan>& mp) {
  TcPlan* t = p->tc;
  const bgemm_plan_options_t* opt = &p->opt;
  static std::mutex mu;
  std::lock_guard<std::mutex> lk(mu);
  g_mode = p->mode;
  const int single_slots = p->facts.num_sms * p->facts.tc_ctas_per_sm;
  if (!first) {
    g_pair = t->pair;
    return choose_tiles(kTcNumCfgs, tc_eval, M, N, K, batch, t->pair ? t->clusters : single_slots,
                        opt, mp);
  }
  int fam = t->want_family;
  if (fam == 0 && t->clusters < 1) fam = 1;
  bgemm_status_t st = BGEMM_SUCCESS;
  if (fam == 0) {
    // plan both kernels with the cost table and keep the shorter makespan
    auto makespan = [&](const std::vector<MatPlan>& v, int slots) {
      double total = 0, longest = 0;
      for (const MatPlan& m : v)
        if (m.cfg >= 0) {
          total += (double)m.tiles * m.t_tile;
          longest = std::max(longest, m.t_tile);
        }
      return std::max(total / slots, longest);
    };
    std::vector<MatPlan> one, two;
    g_pair = false;
    bgemm_status_t s1 = choose_tiles(kTcNumCfgs, tc_eval, M, N, K, batch, single_slots, opt, one);
    g_pair = true;
    bgemm_status_t s2 = choose_tiles(kTcNumCfgs, tc_eval, M, N, K, batch, t->clusters, opt, two);
    if (s1 != BGEMM_SUCCESS && s2 != BGEMM_SUCCESS) return s1;
    t->pair = s2 == BGEMM_SUCCESS &&
              (s1 != BGEMM_SUCCESS || makespan(two, t->clusters) < makespan(one, single_slots));
    mp = t->pair ? two : one;
  } else {
    t->pair = fam == 2;
    g_pair = t->pair;
    st = choose_tiles(kTcNumCfgs, tc_eval, M, N, K, batch, t->pair ? t->clusters : single_slots,
                      opt, mp);
  }
  return st;
}

void tc_tile_dims(bgemm_plan_s* p, int, int, int, int cfg, int* bm, int* bn, MatDesc* d) {
  const bool pair = p->tc->pair;
  *bm = pair ? 256 : kTcBM;
  *bn = pair ? tc2_cfg_bn(cfg) : tc_cfg_bn(cfg);
  d->aux = (d->aux & ~kTcSwapFlag) | (tc_cfg_swap(cfg) ? kTcSwapFlag : 0);
}

// Workspace: per matrix [A hi][A lo][B hi][B lo], rows of kpad elements;
// pack jobs: strips of 32 rows, matrices with the longest K first.
void tc_layout(bgemm_plan_s* p, const std::vector<MatDesc>& hd, bgemm_plan_requirements_t* req) {
  TcPlan* t = p->tc;
  const int batch = (int)hd.size();
  const int esz = (t->kind == kKindBF16) ? 2 : 4;
  t->pd.assign(batch, PackDesc{});
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off += align256(bytes);
    return (long long)o;
  };
  for (int i = 0; i < batch; ++i) {
    const MatDesc& d = hd[i];
    PackDesc& q = t->pd[i];
    q.kpad = (int)((d.K + (16 / esz) - 1) / (16 / esz) * (16 / esz));
    if (d.M == 0 || d.N == 0 || d.K == 0) continue;
    const size_t a = (size_t)d.M * q.kpad * esz, b = (size_t)d.N * q.kpad * esz;
    q.a_hi = take(a);
    q.a_lo = t->split ? take(a) : q.a_hi;
    q.b_hi = take(b);
    q.b_lo = t->split ? take(b) : q.b_hi;
  }
  std::vector<int> order;
  for (int i = 0; i < batch; ++i)
    if (hd[i].M > 0 && hd[i].N > 0 && hd[i].K > 0) order.push_back(i);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return hd[a].K > hd[b].K; });
  t->jobs.clear();
  for (int i : order) {
    for (int r = 0; r < hd[i].M; r += 32) t->jobs.push_back(PackJob{i, 0, r, 0});
    for (int r = 0; r < hd[i].N; r += 32) t->jobs.push_back(PackJob{i, 1, r, 0});
  }
  req->pack_jobs = (int)std::min<size_t>(t->jobs.size(), (size_t)1 << 30);
  req->workspace_bytes = std::max<size_t>(off, 256);
  req->kernel_family = t->pair ? 2 : 1;
}

// ----------------------------------------------------------- tensor maps --
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  });
  return fn;
}

// 2-D K-major panel: dim 0 = K (elements, contiguous), dim 1 = rows.
static bool encode_panel(CUtensorMap* out, int kind, void* base, int K, int rows, int kpad,
                         int box_rows) {
  auto fn = encode_fn();
  if (!fn) return false;
  const int esz = (kind == kKindBF16) ? 2 : 4;  // TF32 halves and raw FP32: 4 bytes
  cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)kpad * esz};
  cuuint32_t box[2] = {(cuuint32_t)(128 / esz), (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(out, kind == kKindBF16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16
                                         : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                  2, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// The four maps of matrix i (A-side hi/lo, B-side hi/lo) encoded on the host.
static bool encode_matrix_maps(const TcPlan* t, const MatDesc& d, const PackDesc& q, char* ws,
                               CUtensorMap* out) {
  const bool swap = tc_cfg_swap(d.cfg);
  // one SM: A-side boxes of 128 rows, B-side boxes of bn rows; a CTA pair
  // loads per CTA 128 A-side rows and half of the bn B-side rows
  const int bbox = t->pair ? tc2_cfg_bn(d.cfg) / 2 : tc_cfg_bn(d.cfg);
  const long long off[4] = {swap ? q.b_hi : q.a_hi, swap ? q.b_lo : q.a_lo,
                            swap ? q.a_hi : q.b_hi, swap ? q.a_lo : q.b_lo};
  const int rows[4] = {swap ? d.N : d.M, swap ? d.N : d.M, swap ? d.M : d.N, swap ? d.M : d.N};
  for (int part = 0; part < 4; ++part)
    if (!encode_panel(&out[part], t->kind, ws + off[part], d.K, rows[part], q.kpad,
                      part < 2 ? kTcBM : bbox))
      return false;
  return true;
}

// Templates per (box height, extent class); the device patches one copy per
// operand panel (address, dims, row stride).
bool tc_encode_templates(int kind, void* base, CUtensorMap* tpl) {
  const int esz = (kind == kKindBF16) ? 2 : 4;
  const int ke = 128 / esz;
  for (int b = 16; b <= 128; b *= 2) {
    if (!encode_panel(&tpl[tmap_template_index(b, false)], kind, base, ke, kTcBM, ke,
                      b) ||  // 128 rows x 128 B = 16 KiB
        !encode_panel(&tpl[tmap_template_index(b, true)], kind, base, ke, 1 << 20, ke,
                      b))  // 2^20 rows x 128 B = 128 MiB
      return false;
  }
  return true;
}

bgemm_status_t tc_alloc(bgemm_plan_s* p) {
  TcPlan* t = p->tc;
  t->cap_batch = p->cap.batch;
  t->cap_jobs = p->cap.pack_jobs;
  t->cap_ws = std::max<size_t>(p->cap.workspace_bytes, 256);
  t->off_tm = sizeof(CUtensorMap) * 2 * kTmapBoxClasses;  // templates first
  t->off_pd = t->off_tm + sizeof(CUtensorMap) * 4 * (size_t)t->cap_batch;
  t->off_jobs = t->off_pd + align256(sizeof(PackDesc) * (size_t)t->cap_batch);
  t->off_err = t->off_jobs + align256(sizeof(PackJob) * (size_t)t->cap_jobs);
  t->mem_bytes = t->off_err + 256;

  cudaError_t e = cudaMalloc(&t->d_ws, t->cap_ws);
  if (e != cudaSuccess)
    return set_error(BGEMM_ERROR_ALLOC, 0, -1, "split-operand workspace of %zu bytes: %s",
                     t->cap_ws, cudaGetErrorString(e));
  e = cudaMalloc(&t->d_mem, t->mem_bytes);
  for (int s = 0; s < kStageBufs && e == cudaSuccess; ++s)
    e = cudaMallocHost(&t->h_stage[s], t->mem_bytes);
  if (e != cudaSuccess)
    return set_error(BGEMM_ERROR_ALLOC, 0, -1, "tensor-core plan memory: %s",
                     cudaGetErrorString(e));
  for (int s = 0; s < kStageBufs; ++s) std::memset(t->h_stage[s], 0, t->mem_bytes);
  if (!tc_encode_templates(t->kind, t->d_ws, static_cast<CUtensorMap*>(t->h_stage[0])))
    return set_error(BGEMM_ERROR_INTERNAL, 0, -1, "template tensor map encoding failed");
  char* dm = static_cast<char*>(t->d_mem);
  t->d_templ = reinterpret_cast<CUtensorMap*>(dm);
  t->d_tmaps = reinterpret_cast<CUtensorMap*>(dm + t->off_tm);
  t->d_pdescs = reinterpret_cast<PackDesc*>(dm + t->off_pd);
  t->d_jobs = reinterpret_cast<PackJob*>(dm + t->off_jobs);
  t->d_err = reinterpret_cast<int*>(dm + t->off_err);
  // 16 CTAs per SM, ~5 waves of the 3 that fit: a shorter last wave than 8 per
  // SM (measured: the skewed pre-pass 3.03 -> 2.98 ms; 4 per SM, 1.3 waves, 3.63)
  t->pack_grid = (int)std::max<long long>(
      1, std::min<long long>(t->cap_jobs, (long long)p->facts.num_sms * kPackCtasPerSm));
  p->info.workspace_bytes = t->cap_ws;
  p->info.device_bytes += t->cap_ws + t->mem_bytes;
  p->info.kernels_per_execute = 2;
  if (t->pair) {
    // one CTA pair per cluster slot, never more pairs than tiles
    int pairs = std::max(1, std::min(t->clusters, std::max(p->cap.tiles, 1)));
    if (p->opt.max_ctas > 0) pairs = std::max(1, std::min(pairs, p->opt.max_ctas / 2));
    p->grid = 2 * pairs;
    p->info.grid = p->grid;
  }
  return BGEMM_SUCCESS;
}

bgemm_status_t tc_commit(bgemm_plan_s* p, int stage, int batch, bool first, cudaStream_t stream) {
  TcPlan* t = p->tc;
  char* h = static_cast<char*>(t->h_stage[stage]);
  char* dm = static_cast<char*>(t->d_mem);
  char* ws = static_cast<char*>(t->d_ws);
  if (batch > 0) std::memcpy(h + t->off_pd, t->pd.data(), sizeof(PackDesc) * (size_t)batch);
  if (!t->jobs.empty())
    std::memcpy(h + t->off_jobs, t->jobs.data(), sizeof(PackJob) * t->jobs.size());
  if (t->host_tmaps) {
    auto* tm = reinterpret_cast<CUtensorMap*>(h + t->off_tm);
    for (int i = 0; i < batch; ++i) {
      const MatDesc& d = p->host_descs[i];
      if (d.M == 0 || d.N == 0 || d.K == 0) continue;
      if (!encode_matrix_maps(t, d, t->pd[i], ws, &tm[4 * i]))
        return set_error(BGEMM_ERROR_INTERNAL, 0, i, "tensor map encoding failed for matrix %d", i);
    }
  }
  auto copy = [&](size_t off, size_t bytes) {
    return bytes ? cudaMemcpyAsync(dm + off, h + off, bytes, cudaMemcpyHostToDevice, stream)
                 : cudaSuccess;
  };
  cudaError_t e = cudaSuccess;
  if (first) {
    e = copy(0, t->off_tm);  // templates
    if (e == cudaSuccess) e = copy(t->off_err, 256);  // zero error word
  }
  if (e == cudaSuccess && t->host_tmaps) e = copy(t->off_tm, sizeof(CUtensorMap) * 4 * (size_t)batch);
  if (e == cudaSuccess) e = copy(t->off_pd, sizeof(PackDesc) * (size_t)batch);
  if (e == cudaSuccess) e = copy(t->off_jobs, sizeof(PackJob) * t->jobs.size());
  if (e != cudaSuccess) return cuda_error(e, "tensor-core descriptor upload");
  t->n_jobs = (int)t->jobs.size();
  if (!t->host_tmaps && batch > 0) {
    // per-matrix tensor maps built on the device, once per batch
    TcTmapParams tp{p->d_descs, t->d_pdescs, t->d_templ, t->d_tmaps, ws, batch, t->kind,
                    t->pair ? 1 : 0};
    e = tc_tmap_launch(tp, stream);
    if (e != cudaSuccess) return cuda_error(e, "tensor-map build launch");
  }
  return BGEMM_SUCCESS;
}

// Host re-encoding of every map the device built, for a byte comparison.
int tc_debug_compare_tmaps(bgemm_plan_s* p, cudaStream_t stream, int* n_maps, int* n_diff,
                           int* first_byte) {
  TcPlan* t = p->tc;
  if (!t) return -1;
  if (cudaStreamSynchronize(stream) != cudaSuccess) return -1;
  const int batch = p->batch;
  std::vector<CUtensorMap> dev(4 * (size_t)batch), host(4 * (size_t)batch);
  if (batch > 0 && cudaMemcpy(dev.data(), t->d_tmaps, sizeof(CUtensorMap) * 4 * (size_t)batch,
                              cudaMemcpyDeviceToHost) != cudaSuccess)
    return -1;
  std::vector<PackDesc> pd(batch);
  if (batch > 0 && cudaMemcpy(pd.data(), t->d_pdescs, sizeof(PackDesc) * (size_t)batch,
                              cudaMemcpyDeviceToHost) != cudaSuccess)
    return -1;
  char* ws = static_cast<char*>(t->d_ws);
  int maps = 0, diff = 0, first = -1;
  for (int i = 0; i < batch; ++i) {
    const MatDesc& d = p->host_descs[i];
    if (d.M == 0 || d.N == 0 || d.K == 0) continue;
    if (!encode_matrix_maps(t, d, pd[i], ws, &host[4 * i])) return -1;
    for (int part = 0; part < 4; ++part) {
      ++maps;
      const unsigned char* a = reinterpret_cast<const unsigned char*>(&host[4 * i + part]);
      const unsigned char* b = reinterpret_cast<const unsigned char*>(&dev[4 * i + part]);
      for (int k = 0; k < (int)sizeof(CUtensorMap); ++k)
        if (a[k] != b[k]) {
          if (first < 0) first = k;
          ++diff;
          break;
        }
    }
  }
  *n_maps = maps;
  *n_diff = diff;
  *first_byte = first;
  return 0;
}

bgemm_status_t tc_execute(bgemm_plan_s* p, float alpha, const float* const* dA,
                          const float* const* dB, float beta, float* const* dC,
                          cudaStream_t stream) {
  TcPlan* t = p->tc;
  TcPackParams pp{p->d_descs, t->d_pdescs,  t->d_jobs, t->n_jobs, p->d_counters + kHdrJobs,
                  t->kind,       t->split,      static_cast<char*>(t->d_ws), dA, dB};
  cudaError_t e = tc_pack_launch(pp, t->pack_grid, stream);
  if (e != cudaSuccess) return cuda_error(e, "split/pack launch");
  TcGemmParams gp{p->d_descs, p->d_items,  p->n_items, p->d_counters + kHdrItems,
                  p->d_counters, t->d_tmaps, alpha,      beta,
                  dC,            t->d_err,   2000000000ull, p->d_cta_times,
                  tc_schedule(p->mode)};
  if (p->ev_start) cudaEventRecord(p->ev_start, stream);
  e = t->pair ? tc2_gemm_launch(t->kind, t->split, gp, p->grid, stream)
              : tc_gemm_launch(t->kind, t->split, gp, p->grid, stream);
  if (p->ev_stop) cudaEventRecord(p->ev_stop, stream);
  if (e != cudaSuccess) return cuda_error(e, "tcgen05 GEMM launch");
  return BGEMM_SUCCESS;
}

bgemm_status_t tc_check_device(bgemm_plan_s* p, cudaStream_t) {
  TcPlan* t = p->tc;
  int err = 0;
  cudaError_t e = cudaMemcpy(&err, t->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_error(e, "device error word");
  if (err) {
    cudaMemset(t->d_err, 0, sizeof(int));
    // an aborted launch may have left the tile queue's counters mid-walk
    cudaMemset(p->d_counters, 0, 2 * sizeof(int));
    return set_error(BGEMM_ERROR_DEVICE_TIMEOUT, 0, -1,
                     "a bounded wait in the tensor-core kernel expired; results are invalid");
  }
  return BGEMM_SUCCESS;
}

void tc_plan_release(bgemm_plan_s* p) {
  TcPlan* t = p->tc;
  if (!t) return;
  if (t->d_ws) cudaFree(t->d_ws);
  if (t->d_mem) cudaFree(t->d_mem);
  for (void* h : t->h_stage)
    if (h) cudaFreeHost(h);
  delete t;
  p->tc = nullptr;
}

}  // namespace bgemm

namespace bgemm {
// The pre-pass layout of the last planned batch (host-only debug replay).
void tc_debug_layout(bgemm_plan_s* p, long long* ws_out, int* jobs_out, int max_jobs,
                     int* n_jobs, int* pair) {
  TcPlan* t = p->tc;
  for (size_t i = 0; ws_out && i < t->pd.size(); ++i) {
    const PackDesc& q = t->pd[i];
    const long long v[5] = {q.a_hi, q.a_lo, q.b_hi, q.b_lo, q.kpad};
    for (int k = 0; k < 5; ++k) ws_out[5 * i + k] = v[k];
  }
  *n_jobs = (int)t->jobs.size();
  for (int j = 0; jobs_out && j < *n_jobs && j < max_jobs; ++j) {
    jobs_out[3 * j] = t->jobs[j].mat;
    jobs_out[3 * j + 1] = t->jobs[j].op;
    jobs_out[3 * j + 2] = t->jobs[j].r0;
  }
  *pair = t->pair ? 2 : 1;
}
}  // namespace bgemm

extern "C" int bgemm_debug_bounded_wait_selftest(unsigned long long limit_ns, int* error,
                                                 int* returned, int* wait_ok) {
  using namespace bgemm;
  int* d = nullptr;
  if (cudaMalloc(&d, 4 * sizeof(int)) != cudaSuccess) return -1;
  int h[4] = {0, 0, 0, 0};
  cudaError_t e = cudaMemset(d, 0, 4 * sizeof(int));
  if (e == cudaSuccess) e = tc_wait_selftest_launch(d, d + 1, limit_ns, nullptr);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return -1;
  if (error) *error = h[0];
  if (returned) *returned = h[1];
  if (wait_ok) *wait_ok = h[2];
  return 0;
}

extern "C" int bgemm_debug_set_tc_schedule(int mode, const int* group) {
  using namespace bgemm;
  if (mode < BGEMM_MODE_TF32 || mode > BGEMM_MODE_BF16X3) return -1;
  std::lock_guard<std::mutex> lk(g_sched_mu);
  if (!group) {
    g_sched_override[mode - 1] = false;
    return 0;
  }
  for (int b = 0; b < kTcSchedBuckets; ++b)
    if (group[b] < 0 || group[b] > 64) return -1;
  for (int b = 0; b < kTcSchedBuckets; ++b) g_sched[mode - 1].set(b, group[b]);
  g_sched_override[mode - 1] = true;
  return 0;
}

extern "C" int bgemm_debug_get_tc_schedule(int mode, int* group) {
  using namespace bgemm;
  if (mode < BGEMM_MODE_TF32 || mode > BGEMM_MODE_BF16X3 || !group) return -1;
  const TcSchedule s = tc_schedule(mode);
  for (int b = 0; b < kTcSchedBuckets; ++b) group[b] = s.group(b);
  return 0;
}
