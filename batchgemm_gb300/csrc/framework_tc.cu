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
  int* bins;         // [cap_batch]
  int* mat_start;    // [cap_batch] first queue slot (-1: none)
  int* job_start;    // [cap_batch] first pre-pass strip (-1: none)
  TileItem* items;   // [cap_items]
  PackJob* jobs;     // [cap_jobs]
  CUtensorMap* tmaps;  // [4 * cap_batch]
  CUtensorMap* templ;  // [2 * kTmapBoxClasses]
  char* ws;
  unsigned long long cap_ws;
};

__device__ __forceinline__ int cdiv(int a, int b) { return (a + b - 1) / b; }

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
  const int esz = (mode == BGEMM_MODE_BF16X3) ? 2 : 4;
  const int parts = (mode == BGEMM_MODE_TF32) ? 1 : 2;
  for (int i = threadIdx.x; i < batch; i += blockDim.x) {
    const int M = dM[i], N = dN[i], K = dK[i];
    const bool bad = M < 0 || N < 0 || K < 0 || M > max_dim || N > max_dim || K > max_k;
    if (bad) atomicOr(s.err, 1);
    int best = -1, bin = 0;
    int bt = 0;
    if (!bad && M > 0 && N > 0) {
      float bw = 0.f, btt = 0.f;
      for (int q = 5; q >= 0; --q) {
        const int c = pair_cfg(q);
        const TileCost tc = c_tc_cost[mode - 1][c];
        if (tc.b_ns <= 0.f) continue;
        const bool swap = tc_cfg_swap(c);
        const int ra = swap ? N : M, rb = swap ? M : N;
        const int t = cdiv(ra, 256) * cdiv(rb, tc2_cfg_bn(c));
        const float tt = tc.a_ns + tc.b_ns * (float)K;
        const float w = (float)t * tt;
        if (best < 0 || w < bw * 0.999f) { best = c; bt = t; bw = w; btt = tt; }
      }
      if (best >= 0)
        bin = min(kBins - 1, max(0, (int)(4.0f * __log2f(fmaxf(btt, 1.0f)) - 24.0f)));
      else
        atomicOr(s.err, 4);  // no CTA-pair configuration in the cost table
    }
    // a skipped matrix keeps an empty descriptor (no maps, strips or tiles)
    s.descs[i] = bad ? MatDesc{0, 0, 0, 1, 1, 1, pair_cfg(0), 0}
                     : MatDesc{M, N, K, max(M, 1), max(K, 1), max(M, 1),
                               best < 0 ? pair_cfg(0) : best, 0};
    s.mat_start[i] = best < 0 ? -1 : atomicAdd(&bin_tiles[bin], bt);
    // split-operand panels and pre-pass strips of a matrix with work
    PackDesc pd{};
    pd.kpad = bad ? 0 : (K * esz + 15) / 16 * 16 / esz;
    int js = -1, kbin = 0;
    if (best >= 0 && K > 0) {
      const unsigned long long a =
          ((unsigned long long)M * pd.kpad * esz + 255) & ~255ull;
      const unsigned long long b =
          ((unsigned long long)N * pd.kpad * esz + 255) & ~255ull;
      const unsigned long long off = atomicAdd(&ws_total, parts * (a + b));
      pd.a_hi = (long long)off;
      pd.a_lo = parts == 2 ? (long long)(off + a) : pd.a_hi;
      pd.b_hi = (long long)(off + parts * a);
      pd.b_lo = parts == 2 ? (long long)(off + parts * a + b) : pd.b_hi;
      kbin = min(kBins - 1, (int)(4.0f * __log2f((float)K)));
      js = atomicAdd(&kbin_jobs[kbin], cdiv(M, 32) + cdiv(N, 32));
    }
    s.pdescs[i] = pd;
    s.job_start[i] = js;
    s.bins[i] = bin | (kbin << 8);
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
  DeviceFacts df;
  bgemm_status_t st = device_facts(&df);
  if (st != BGEMM_SUCCESS) return st;

  const int kind = (mode == BGEMM_MODE_BF16X3) ? kKindBF16 : kKindTF32;
  const int split = (mode == BGEMM_MODE_TF32) ? 0 : 1;
  const size_t esz = kind == kKindBF16 ? 2 : 4;
  const size_t tiles_per = (size_t)((max_dim + 255) / 256) * ((max_dim + 63) / 64);
  const size_t need_items = (size_t)batch * tiles_per;
  const size_t need_jobs = (size_t)batch * 2 * ((max_dim + 31) / 32);
  if (need_items > (size_t)INT32_MAX || need_jobs > (size_t)INT32_MAX)
    return set_error(BGEMM_ERROR_NOT_SUPPORTED, 8, -1,
                     "batch %d with max_dim %d can hold more than 2^31 tiles", batch, max_dim);
  // operand elements, plus each row's padding to 16 bytes and each panel's
  // 256-byte alignment
  const size_t elems = max_operand_elems > 0 ? (size_t)max_operand_elems
                                             : (size_t)batch * 2 * max_dim * (size_t)max_k;
  const size_t pad_elems = (size_t)batch * 2 * max_dim * (16 / esz - 1);
  const size_t need_ws =
      (size_t)(1 + split) * (esz * (elems + pad_elems) + (size_t)batch * 2 * 256);

  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_consts[df.device & 63]) {
    // the cost table with the host planner's rule for untuned entries: the
    // 3xTF32 cost of the same tile, halved per unit of K for one-part modes
    TileCost cost[3][16];
    for (int m = 0; m < 3; ++m)
      for (int c = 0; c < 16; ++c) {
        cost[m][c] = kTcCost[m][c];
        const TileCost& t3 = kTcCost[BGEMM_MODE_TF32X3 - 1][c];
        if (cost[m][c].b_ns <= 0.0f && t3.b_ns > 0.0f)
          cost[m][c] = TileCost{t3.a_ns, m == BGEMM_MODE_TF32X3 - 1 ? t3.b_ns : 0.5f * t3.b_ns};
      }
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
  e = tc_pack_launch(pp, df.num_sms * 8, stream);
  if (e != cudaSuccess) return cuda_error(e, "split/pack launch");
  TcGemmParams gp{s.descs, s.items, 0, s.counts, s.counters, s.tmaps, 1.0f, 1.0f, dC,
                  s.gemm_err, 2000000000ull};
  e = tc2_gemm_launch(kind, split, gp, 2 * clusters, stream);
  if (e != cudaSuccess) return cuda_error(e, "tcgen05 GEMM launch");
  return BGEMM_SUCCESS;
}
