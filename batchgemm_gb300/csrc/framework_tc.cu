// framework_tc.cu -- the device-resident-size entry (the reference framework
// kernel's argument list: device arrays of sizes and pointers, C_i += A_i*B_i
// column-major, lda = M_i, ldb = K_i, ldc = M_i) in the tensor-core modes.
//
// Everything a tensor-core execute needs is built on the device, from sizes
// that never leave it, so a captured sequence of these launches replays with
// whatever the size arrays hold:
//   1. fwtc_plan_kernel (one CTA) picks each matrix's CTA-pair tile
//      configuration with the same cost table as the host planner (no
//      rebalance), buckets matrices by modelled tile time (quarter-octave
//      bins, longest first) and reserves each matrix its queue range, its
//      split-operand panels in the workspace and its pre-pass strips;
//   2. fwtc_expand_kernel writes the work items and strips (one warp per
//      matrix);
//   3. the tensor maps (tc_tmap_kernel), the split/pack pre-pass and the
//      CTA-pair GEMM run as for a plan, reading item and strip counts from
//      the device.
// Scratch (descriptors, queue, maps, workspace) is owned by the library, one
// buffer per device and mode, sized from batch, max_dim, max_k and the bound
// on the batch's operand elements, and grown when a call needs more.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "bgemm.h"
#include "plan_internal.h"
#include "tc_common.h"
#include "tile_table.h"

namespace bgemm {

bool tc_encode_templates(int kind, void* base, CUtensorMap* out);

namespace {

constexpr int kBins = 64;
// the six CTA-pair configurations: BN 64 / 128 / 256, unswapped (8..10) and
// swapped (12..14)
__host__ __device__ constexpr int pair_cfg(int q) { return 8 + q % 3 + (q / 3) * 4; }

__constant__ TileCost c_tc_cost[3][16];

struct FwTcScratch {
  int* err;          // bit 0: a size was negative or above max_dim / max_k;
                     // bit 1: the workspace could not hold the batch (nothing ran);
                     // bit 2: no costed tile configuration (matrix skipped)
  int* gemm_err;     // bit 0: a bounded device wait of the GEMM expired
  int* counts;       // [0] work items, [1] pre-pass strips
  int* counters;     // GEMM queue counters (reset by the kernel)
  MatDesc* descs;    // [cap_batch]
  PackDesc* pdescs;  // [cap_batch]
  int* bins;         // [cap_batch] tile-time bin | K bin << 8
  int* mat_start;    // [cap_batch] first queue slot (-1: none)
  int* job_start;    // [cap_batch] first pre-pass strip (-1: none)
  TileItem* items;   // [cap_items]
  PackJob* jobs;     // [cap_jobs]
  CUtensorMap* tmaps;  // [4 * cap_batch]
  CUtensorMap* templ;  // [2 * kTmapBoxClasses]
  char* ws;
  unsigned long long cap_ws;
};

__host__ __device__ __forceinline__ int cdiv(int a, int b) { return (a + b - 1) / b; }

// What the planner decides for one matrix, independently of the others; the
// kernel then reserves queue slots, strips and workspace with atomics, and a
// host replay (bgemm_debug_framework_tc_plan) with plain sums.
struct FwTcMat {
  MatDesc desc;
  int kpad;        // packed row length (elements)
  int bad;         // size negative or above max_dim / max_k: skipped
  int nocfg;       // no costed CTA-pair configuration: skipped
  int tiles;       // work items (0: none)
  int bin;         // quarter-octave bin of the modelled tile time
  int kbin;        // quarter-octave bin of K (strips of the longest K first)
  int strips;      // pre-pass strips (0: nothing to pack)
  unsigned long long a_bytes, b_bytes;  // one part of each operand, 256-byte aligned
};

__host__ __device__ inline FwTcMat fwtc_plan_matrix(int M, int N, int K, int max_dim, int max_k,
                                                    int mode, const TileCost* cost) {
  FwTcMat r{};
  const int esz = (mode == BGEMM_MODE_BF16X3) ? 2 : 4;
  r.bad = M < 0 || N < 0 || K < 0 || M > max_dim || N > max_dim || K > max_k;
  int best = -1;
  if (!r.bad && M > 0 && N > 0) {
    float bw = 0.f, btt = 0.f;
    int bt = 0;
    for (int q = 5; q >= 0; --q) {
      const int c = pair_cfg(q);
      const TileCost tc = cost[c];
      if (tc.b_ns <= 0.f) continue;
      const bool swap = tc_cfg_swap(c);
      const int ra = swap ? N : M, rb = swap ? M : N;
      const int t = cdiv(ra, 256) * cdiv(rb, tc2_cfg_bn(c));
      const float tt = tc.a_ns + tc.b_ns * (float)K;
      const float w = (float)t * tt;
      if (best < 0 || w < bw * 0.999f) { best = c; bt = t; bw = w; btt = tt; }
    }
    if (best >= 0) {
      r.tiles = bt;
      r.bin = min(kBins - 1, max(0, quarter_octave(btt) - 24));
    } else {
      r.nocfg = 1;
    }
  }
  // a skipped matrix keeps an empty descriptor (no maps, strips or tiles)
  r.desc = r.bad ? MatDesc{0, 0, 0, 1, 1, 1, pair_cfg(0), 0}
                 : MatDesc{M, N, K, max(M, 1), max(K, 1), max(M, 1),
                           best < 0 ? pair_cfg(0) : best, 0};
  r.kpad = r.bad ? 0 : (K * esz + 15) / 16 * 16 / esz;
  if (best >= 0 && K > 0) {
    r.a_bytes = ((unsigned long long)M * r.kpad * esz + 255) & ~255ull;
    r.b_bytes = ((unsigned long long)N * r.kpad * esz + 255) & ~255ull;
    r.kbin = min(kBins - 1, quarter_octave((float)K));
    r.strips = cdiv(M, 32) + cdiv(N, 32);
  }
  return r;
}

__global__ void fwtc_plan_kernel(const int* __restrict__ dM, const int* __restrict__ dN,
                                 const int* __restrict__ dK, int batch, int max_dim, int max_k,
                                 int mode, FwTcScratch s) {
  __shared__ int bin_tiles[kBins];
  __shared__ int bin_start[kBins];
  __shared__ int kbin_jobs[kBins];  // pre-pass strips per quarter-octave of K
  __shared__ int kbin_start[kBins];
  __shared__ unsigned long long ws_total;
  __shared__ int jobs_total;
  for (int b = threadIdx.x; b < kBins; b += blockDim.x) bin_tiles[b] = kbin_jobs[b] = 0;
  if (threadIdx.x == 0) {
    ws_total = 0;
    jobs_total = 0;
  }
  __syncthreads();
  const int parts = (mode == BGEMM_MODE_TF32) ? 1 : 2;
  for (int i = threadIdx.x; i < batch; i += blockDim.x) {
    const FwTcMat r = fwtc_plan_matrix(dM[i], dN[i], dK[i], max_dim, max_k, mode,
                                       c_tc_cost[mode - 1]);
    if (r.bad) atomicOr(s.err, 1);
    if (r.nocfg) atomicOr(s.err, 4);
    s.descs[i] = r.desc;
    s.mat_start[i] = r.tiles ? atomicAdd(&bin_tiles[r.bin], r.tiles) : -1;
    // split-operand panels and pre-pass strips of a matrix with work
    PackDesc pd{};
    pd.kpad = r.kpad;
    int js = -1;
    if (r.strips) {
      const unsigned long long off = atomicAdd(&ws_total, parts * (r.a_bytes + r.b_bytes));
      pd.a_hi = (long long)off;
      pd.a_lo = parts == 2 ? (long long)(off + r.a_bytes) : pd.a_hi;
      pd.b_hi = (long long)(off + parts * r.a_bytes);
      pd.b_lo = parts == 2 ? (long long)(off + parts * r.a_bytes + r.b_bytes) : pd.b_hi;
      js = atomicAdd(&kbin_jobs[r.kbin], r.strips);
    }
    s.pdescs[i] = pd;
    s.job_start[i] = js;
    s.bins[i] = r.bin | (r.kbin << 8);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int b = kBins - 1; b >= 0; --b) {  // longest tiles first
      bin_start[b] = run;
      run += bin_tiles[b];
    }
    for (int b = kBins - 1; b >= 0; --b) {  // strips of the longest K first
      kbin_start[b] = jobs_total;
      jobs_total += kbin_jobs[b];
    }
    if (ws_total > s.cap_ws) {
      atomicOr(s.err, 2);
      run = 0;
      jobs_total = 0;
    }
    s.counts[0] = run;
    s.counts[1] = jobs_total;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < batch; i += blockDim.x) {
    const int off = s.mat_start[i];
    if (off >= 0) s.mat_start[i] = bin_start[s.bins[i] & 0xff] + off;
    const int js = s.job_start[i];
    if (js >= 0) s.job_start[i] = kbin_start[s.bins[i] >> 8] + js;
  }
}

__global__ void fwtc_expand_kernel(int batch, FwTcScratch s) {
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= batch || s.counts[0] == 0) return;
  const int start = s.mat_start[i];
  if (start < 0) return;
  const MatDesc d = s.descs[i];
  const bool swap = tc_cfg_swap(d.cfg);
  const int tmx = cdiv(swap ? d.N : d.M, 256);
  const int tnx = cdiv(swap ? d.M : d.N, tc2_cfg_bn(d.cfg));
  for (int t = lane; t < tmx * tnx; t += 32)
    s.items[start + t] = TileItem{i, (uint16_t)(t % tmx), (uint16_t)(t / tmx)};
  const int js = s.job_start[i];
  if (js < 0) return;
  const int sa = cdiv(d.M, 32), sb = cdiv(d.N, 32);
  for (int j = lane; j < sa + sb; j += 32)
    s.jobs[js + j] = j < sa ? PackJob{i, 0, 32 * j, 0} : PackJob{i, 1, 32 * (j - sa), 0};
}

struct FwTcContext {
  void* mem = nullptr;
  size_t cap_batch = 0, cap_items = 0, cap_jobs = 0, cap_ws = 0;
  FwTcScratch s{};
  bool templ = false;
  int clusters = 0;  // co-resident CTA pairs of the GEMM kernel
};

std::mutex g_mu;
std::unordered_map<long long, FwTcContext> g_ctx;  // key: device * 4 + mode
bool g_consts[64] = {};

size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

// The cost table with the host planner's rule for untuned entries: the
// 3xTF32 cost of the same tile, halved per unit of K for one-part modes.
void fwtc_cost_table(TileCost (&cost)[3][16]) {
  for (int m = 0; m < 3; ++m)
    for (int c = 0; c < 16; ++c) {
      cost[m][c] = kTcCost[m][c];
      const TileCost& t3 = kTcCost[BGEMM_MODE_TF32X3 - 1][c];
      if (cost[m][c].b_ns <= 0.0f && t3.b_ns > 0.0f)
        cost[m][c] = TileCost{t3.a_ns, m == BGEMM_MODE_TF32X3 - 1 ? t3.b_ns : 0.5f * t3.b_ns};
    }
}

// Scratch a call needs: queue items, pre-pass strips, split-operand bytes.
void fwtc_capacity(int batch, int max_dim, int max_k, long long max_operand_elems, int mode,
                   size_t* items, size_t* jobs, size_t* ws) {
  const size_t esz = (mode == BGEMM_MODE_BF16X3) ? 2 : 4;
  const size_t parts = (mode == BGEMM_MODE_TF32) ? 1 : 2;
  *items = (size_t)batch * ((max_dim + 255) / 256) * ((max_dim + 63) / 64);
  *jobs = (size_t)batch * 2 * ((max_dim + 31) / 32);
  // operand elements, plus each row's padding to 16 bytes and each panel's
  // 256-byte alignment
  const size_t elems = max_operand_elems > 0 ? (size_t)max_operand_elems
                                             : (size_t)batch * 2 * max_dim * (size_t)max_k;
  const size_t pad_elems = (size_t)batch * 2 * max_dim * (16 / esz - 1);
  *ws = parts * (esz * (elems + pad_elems) + (size_t)batch * 2 * 256);
}

}  // namespace

// Errors of the device-resident tensor-core path on `dev` (cleared once
// reported); called by bgemm_framework_check_device.
bgemm_status_t fwtc_check_device(int dev) {
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto& kv : g_ctx) {
    if (kv.first / 4 != dev || !kv.second.mem) continue;
    int err[2] = {0, 0};
    cudaError_t e = cudaMemcpy(&err[0], kv.second.s.err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
      e = cudaMemcpy(&err[1], kv.second.s.gemm_err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_error(e, "framework error words");
    if (err[0] || err[1]) {
      cudaMemset(kv.second.s.err, 0, sizeof(int));
      cudaMemset(kv.second.s.gemm_err, 0, sizeof(int));
      // an aborted launch may have left the tile queue's counters mid-walk
      if (err[1]) cudaMemset(kv.second.s.counters, 0, 2 * sizeof(int));
      if (err[1])
        return set_error(BGEMM_ERROR_DEVICE_TIMEOUT, 0, -1,
                         "a bounded wait in the tensor-core kernel expired; results are invalid");
      if (err[0] & 4)
        return set_error(BGEMM_ERROR_INTERNAL, 0, -1, "no CTA-pair tile configuration is costed");
      if (err[0] & 2)
        return set_error(BGEMM_ERROR_NOT_SUPPORTED, 0, -1,
                         "the batch's split operands exceed the workspace sized from "
                         "max_operand_elems (or max_dim and max_k); nothing was computed");
      return set_error(BGEMM_ERROR_INVALID_VALUE, 1, -1,
                       "a matrix size was negative or above max_dim / max_k; such matrices were "
                       "skipped");
    }
  }
  return BGEMM_SUCCESS;
}

// Frees the tensor-core scratch of every mode on `dev`.
bgemm_status_t fwtc_release(int dev) {
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto& kv : g_ctx) {
    if (kv.first / 4 != dev || !kv.second.mem) continue;
    const cudaError_t e = cudaFree(kv.second.mem);  // waits for kernels still using it
    kv.second = FwTcContext{};
    if (e != cudaSuccess) return cuda_error(e, "framework scratch release");
  }
  return BGEMM_SUCCESS;
}

}  // namespace bgemm

using namespace bgemm;

extern "C" bgemm_status_t bgemm_framework_gemm_mode(const int* dM, const int* dN, const int* dK,
                                                    float* const* dA, float* const* dB,
                                                    float* const* dC, int batch, int max_dim,
                                                    int max_k, long long max_operand_elems,
                                                    bgemm_mode_t mode, bgemm_stream_t stream) {
  if (mode == BGEMM_MODE_SIMT_FP32)
    return bgemm_framework_gemm(dM, dN, dK, dA, dB, dC, nullptr, batch, max_dim, stream);
  if (mode < BGEMM_MODE_TF32 || mode > BGEMM_MODE_BF16X3)
    return set_error(BGEMM_ERROR_INVALID_VALUE, 11, -1, "unknown mode %d", (int)mode);
  if (batch < 0) return set_error(BGEMM_ERROR_INVALID_VALUE, 7, -1, "batch < 0");
  if (batch == 0) return BGEMM_SUCCESS;
  if (!dM) return set_error(BGEMM_ERROR_INVALID_VALUE, 1, -1, "M is NULL");
  if (!dN) return set_error(BGEMM_ERROR_INVALID_VALUE, 2, -1, "N is NULL");
  if (!dK) return set_error(BGEMM_ERROR_INVALID_VALUE, 3, -1, "K is NULL");
  if (!dA) return set_error(BGEMM_ERROR_INVALID_VALUE, 4, -1, "A is NULL");
  if (!dB) return set_error(BGEMM_ERROR_INVALID_VALUE, 5, -1, "B is NULL");
  if (!dC) return set_error(BGEMM_ERROR_INVALID_VALUE, 6, -1, "C is NULL");
  if (max_dim < 1 || max_dim > (1 << 20))
    return set_error(BGEMM_ERROR_INVALID_VALUE, 8, -1, "max_dim = %d not in [1, 2^20]", max_dim);
  if (max_k < 1 || max_k > (1 << 24))
    return set_error(BGEMM_ERROR_INVALID_VALUE, 9, -1, "max_k = %d not in [1, 2^24]", max_k);
  if (max_operand_elems < 0)
    return set_error(BGEMM_ERROR_INVALID_VALUE, 10, -1, "max_operand_elems < 0");
  size_t need_items, need_jobs, need_ws;
  fwtc_capacity(batch, max_dim, max_k, max_operand_elems, mode, &need_items, &need_jobs, &need_ws);
  if (need_items > (size_t)INT32_MAX || need_jobs > (size_t)INT32_MAX)
    return set_error(BGEMM_ERROR_NOT_SUPPORTED, 8, -1,
                     "batch %d with max_dim %d can hold more than 2^31 tiles", batch, max_dim);
  DeviceFacts df;
  bgemm_status_t st = device_facts(&df);
  if (st != BGEMM_SUCCESS) return st;

  const int kind = (mode == BGEMM_MODE_BF16X3) ? kKindBF16 : kKindTF32;
  const int split = (mode == BGEMM_MODE_TF32) ? 0 : 1;

  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_consts[df.device & 63]) {
    TileCost cost[3][16];
    fwtc_cost_table(cost);
    cudaError_t e = cudaMemcpyToSymbol(c_tc_cost, cost, sizeof(cost));
    if (e != cudaSuccess) return cuda_error(e, "framework constants");
    g_consts[df.device & 63] = true;
  }
  FwTcContext& ctx = g_ctx[(long long)df.device * 4 + mode];
  if (ctx.clusters == 0) ctx.clusters = tc2_max_clusters();
  const int clusters = ctx.clusters;
  if (clusters < 1) return set_error(BGEMM_ERROR_NOT_SUPPORTED, 0, -1, "no CTA pair fits");
  if ((size_t)batch > ctx.cap_batch || need_items > ctx.cap_items || need_jobs > ctx.cap_jobs ||
      need_ws > ctx.cap_ws) {
    const size_t cb = std::max((size_t)batch, ctx.cap_batch);
    const size_t ci = std::max(need_items, ctx.cap_items);
    const size_t cj = std::max(need_jobs, ctx.cap_jobs);
    const size_t cw = std::max(need_ws, ctx.cap_ws);
    size_t off = 256;
    auto take = [&](size_t bytes) {
      const size_t o = off;
      off += a256(bytes);
      return o;
    };
    const size_t o_descs = take(sizeof(MatDesc) * cb), o_pd = take(sizeof(PackDesc) * cb);
    const size_t o_bins = take(sizeof(int) * cb), o_ms = take(sizeof(int) * cb);
    const size_t o_js = take(sizeof(int) * cb), o_items = take(sizeof(TileItem) * ci);
    const size_t o_jobs = take(sizeof(PackJob) * cj);
    const size_t o_tm = take(sizeof(CUtensorMap) * 4 * cb);
    const size_t o_tpl = take(sizeof(CUtensorMap) * 2 * kTmapBoxClasses);
    const size_t o_ws = take(cw);
    if (ctx.mem) cudaFree(ctx.mem);  // waits for kernels still using it
    ctx = FwTcContext{};
    ctx.clusters = clusters;
    cudaError_t e = cudaMalloc(&ctx.mem, off);
    if (e != cudaSuccess)
      return set_error(BGEMM_ERROR_ALLOC, 0, -1, "framework scratch of %zu bytes: %s", off,
                       cudaGetErrorString(e));
    e = cudaMemset(ctx.mem, 0, 256);
    if (e != cudaSuccess) return cuda_error(e, "framework scratch init");
    char* b = static_cast<char*>(ctx.mem);
    FwTcScratch& s = ctx.s;
    s.err = reinterpret_cast<int*>(b);
    s.gemm_err = reinterpret_cast<int*>(b + 4);
    s.counts = reinterpret_cast<int*>(b + 64);
    s.counters = reinterpret_cast<int*>(b + 128);
    s.descs = reinterpret_cast<MatDesc*>(b + o_descs);
    s.pdescs = reinterpret_cast<PackDesc*>(b + o_pd);
    s.bins = reinterpret_cast<int*>(b + o_bins);
    s.mat_start = reinterpret_cast<int*>(b + o_ms);
    s.job_start = reinterpret_cast<int*>(b + o_js);
    s.items = reinterpret_cast<TileItem*>(b + o_items);
    s.jobs = reinterpret_cast<PackJob*>(b + o_jobs);
    s.tmaps = reinterpret_cast<CUtensorMap*>(b + o_tm);
    s.templ = reinterpret_cast<CUtensorMap*>(b + o_tpl);
    s.ws = b + o_ws;
    s.cap_ws = cw;
    ctx.cap_batch = cb;
    ctx.cap_items = ci;
    ctx.cap_jobs = cj;
    ctx.cap_ws = cw;
  }
  if (!ctx.templ) {
    CUtensorMap tpl[2 * kTmapBoxClasses];
    if (!tc_encode_templates(kind, ctx.s.ws, tpl))
      return set_error(BGEMM_ERROR_INTERNAL, 0, -1, "template tensor map encoding failed");
    cudaError_t e = cudaMemcpy(ctx.s.templ, tpl, sizeof(tpl), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_error(e, "template upload");
    ctx.templ = true;
  }
  const FwTcScratch s = ctx.s;
  fwtc_plan_kernel<<<1, 1024, 0, stream>>>(dM, dN, dK, batch, max_dim, max_k, (int)mode, s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "framework plan kernel");
  fwtc_expand_kernel<<<(batch + 7) / 8, 256, 0, stream>>>(batch, s);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "framework expand kernel");
  TcTmapParams tp{s.descs, s.pdescs, s.templ, s.tmaps, s.ws, batch, kind, 1};
  e = tc_tmap_launch(tp, stream);
  if (e != cudaSuccess) return cuda_error(e, "tensor-map build launch");
  TcPackParams pp{s.descs, s.pdescs, s.jobs, 0, s.counts + 1, kind, split, s.ws,
                  const_cast<const float* const*>(dA), const_cast<const float* const*>(dB)};
  e = tc_pack_launch(pp, df.num_sms * kPackCtasPerSm, stream);
  if (e != cudaSuccess) return cuda_error(e, "split/pack launch");
  TcGemmParams gp{s.descs, s.items, 0, s.counts, s.counters, s.tmaps, 1.0f, 1.0f, dC,
                  s.gemm_err, 2000000000ull, nullptr, tc_schedule(mode)};
  e = tc2_gemm_launch(kind, split, gp, 2 * clusters, stream);
  if (e != cudaSuccess) return cuda_error(e, "tcgen05 GEMM launch");
  return BGEMM_SUCCESS;
}

// Host replay of the device planner (fwtc_plan_kernel + fwtc_expand_kernel)
// for tests without a GPU: the same per-matrix decisions, the reservations
// made in matrix order instead of by atomics.
extern "C" int bgemm_debug_framework_tc_plan(const int* M, const int* N, const int* K, int batch,
                                             int max_dim, int max_k, long long max_operand_elems,
                                             int mode, int* items_out, int max_items,
                                             int* jobs_out, int max_jobs, long long* ws_out,
                                             int* n_jobs, long long* ws_used,
                                             long long* ws_capacity, int* err, int* cfg_out) {
  if (batch < 0 || mode < BGEMM_MODE_TF32 || mode > BGEMM_MODE_BF16X3 || !n_jobs || !ws_used ||
      !ws_capacity || !err || (batch > 0 && (!M || !N || !K)))
    return -1;
  TileCost cost[3][16];
  fwtc_cost_table(cost);
  size_t cap_items, cap_jobs, cap_ws;
  fwtc_capacity(batch, max_dim, max_k, max_operand_elems, mode, &cap_items, &cap_jobs, &cap_ws);
  const unsigned long long parts = (mode == BGEMM_MODE_TF32) ? 1 : 2;
  std::vector<FwTcMat> r(batch);
  std::vector<int> mat_start(batch, -1), job_start(batch, -1);
  int bin_tiles[kBins] = {}, kbin_jobs[kBins] = {};
  unsigned long long ws_total = 0;
  *err = 0;
  for (int i = 0; i < batch; ++i) {
    r[i] = fwtc_plan_matrix(M[i], N[i], K[i], max_dim, max_k, mode, cost[mode - 1]);
    if (r[i].bad) *err |= 1;
    if (r[i].nocfg) *err |= 4;
    if (cfg_out) cfg_out[i] = r[i].tiles ? r[i].desc.cfg : -1;
    if (r[i].tiles) {
      mat_start[i] = bin_tiles[r[i].bin];
      bin_tiles[r[i].bin] += r[i].tiles;
    }
    long long off[4] = {0, 0, 0, 0};
    if (r[i].strips) {
      const unsigned long long o = ws_total;
      ws_total += parts * (r[i].a_bytes + r[i].b_bytes);
      off[0] = (long long)o;
      off[1] = parts == 2 ? (long long)(o + r[i].a_bytes) : off[0];
      off[2] = (long long)(o + parts * r[i].a_bytes);
      off[3] = parts == 2 ? (long long)(o + parts * r[i].a_bytes + r[i].b_bytes) : off[2];
      job_start[i] = kbin_jobs[r[i].kbin];
      kbin_jobs[r[i].kbin] += r[i].strips;
    }
    if (ws_out) {
      for (int q = 0; q < 4; ++q) ws_out[5 * i + q] = off[q];
      ws_out[5 * i + 4] = r[i].kpad;
    }
  }
  int bin_start[kBins], kbin_start[kBins], n_items = 0, nj = 0;
  for (int b = kBins - 1; b >= 0; --b) {
    bin_start[b] = n_items;
    n_items += bin_tiles[b];
    kbin_start[b] = nj;
    nj += kbin_jobs[b];
  }
  *ws_used = (long long)ws_total;
  *ws_capacity = (long long)cap_ws;
  if (ws_total > cap_ws) {
    *err |= 2;
    n_items = 0;
    nj = 0;
  }
  *n_jobs = nj;
  if ((items_out && n_items > max_items) || (jobs_out && nj > max_jobs)) return -1;
  for (int i = 0; i < batch && n_items > 0; ++i) {
    if (mat_start[i] < 0) continue;
    const MatDesc& d = r[i].desc;
    const bool swap = tc_cfg_swap(d.cfg);
    const int tmx = cdiv(swap ? d.N : d.M, 256), tnx = cdiv(swap ? d.M : d.N, tc2_cfg_bn(d.cfg));
    const int start = bin_start[r[i].bin] + mat_start[i];
    for (int t = 0; items_out && t < tmx * tnx; ++t) {
      items_out[3 * (start + t)] = i;
      items_out[3 * (start + t) + 1] = t % tmx;
      items_out[3 * (start + t) + 2] = t / tmx;
    }
    if (job_start[i] < 0) continue;
    const int js = kbin_start[r[i].kbin] + job_start[i];
    const int sa = cdiv(d.M, 32), sb = cdiv(d.N, 32);
    for (int j = 0; jobs_out && j < sa + sb; ++j) {
      jobs_out[3 * (js + j)] = i;
      jobs_out[3 * (js + j) + 1] = j < sa ? 0 : 1;
      jobs_out[3 * (js + j) + 2] = 32 * (j < sa ? j : j - sa);
    }
  }
  return n_items;
}

// The compile-time schedule parameters of tile_table.h as built.
extern "C" int bgemm_debug_build_params(int* simt_ring_cap, int* c_prefetch_lead) {
  if (!simt_ring_cap || !c_prefetch_lead) return -1;
  *simt_ring_cap = kSimtRingCap;
  *c_prefetch_lead = kTcCPrefetchLead;
  return 0;
}

// The cost-model entry (a + b*K ns per tile) the planners use for a mode's
// configuration: the SIMT table (mode 0) or the tensor-core table as the
// device planner completes it.
extern "C" int bgemm_debug_tile_cost(int mode, int cfg, float* a_ns, float* b_ns) {
  if (!a_ns || !b_ns || mode < BGEMM_MODE_SIMT_FP32 || mode > BGEMM_MODE_BF16X3) return -1;
  if (mode == BGEMM_MODE_SIMT_FP32) {
    if (cfg < 0 || cfg >= kSimtNumCfgs) return -1;
    *a_ns = kSimtCost[cfg].a_ns;
    *b_ns = kSimtCost[cfg].b_ns;
    return 0;
  }
  if (cfg < 0 || cfg >= 16) return -1;
  TileCost cost[3][16];
  fwtc_cost_table(cost);
  *a_ns = cost[mode - 1][cfg].a_ns;
  *b_ns = cost[mode - 1][cfg].b_ns;
  return 0;
}
