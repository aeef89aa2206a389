// framework.cu -- drop-in for the reference framework's kernel entry
//   gemm<<<grid, 256, 16 KB>>>(M, N, K, A, B, C, T_strategy)
// (CUDA/framework/kernel.h:11, launched at CUDA/framework/gemm.cu:200): the
// sizes are device arrays, C_i += A_i * B_i column-major with lda = M_i,
// ldb = K_i, ldc = M_i.
//
// Because the sizes live on the device, the tile queue is built there too:
//   1. fw_plan_kernel (one CTA) picks each matrix's SIMT tile configuration
//      with the same cost model as the host planner, rebalances for
//      parallelism (the host planner's rule, in rounds: a matrix whose tile
//      is longer than the average load of a persistent CTA moves to smaller
//      tiles when that lowers the makespan bound), buckets matrices by
//      modelled tile time (quarter-octave bins) and reserves each matrix a
//      contiguous range of the queue, longest tiles first;
//   2. fw_expand_kernel writes the work items (one warp per matrix);
//   3. the persistent SIMT kernel reads the item count from the device.
// The three launches allocate nothing and can be captured in a CUDA graph;
// the queue scratch is owned by the library (one buffer per device, grown
// when a call needs more).
#include <mutex>
#include <unordered_map>
#include <vector>

#include "bgemm.h"
#include "bgemm_internal.h"
#include "plan_internal.h"
#include "tile_table.h"

namespace bgemm {
namespace {

constexpr int kBins = 64;

__constant__ SimtCfg c_cfgs[kSimtNumCfgs];
__constant__ TileCost c_cost[kSimtNumCfgs];

struct FwScratch {
  int* err;         // bit 0: a size was negative or above max_dim
  int* n_items;
  int* counters;    // 2 ints: queue head, CTAs finished
  MatDesc* descs;   // [cap_batch]
  int* mat_start;   // [cap_batch] first queue slot of each matrix (-1: none)
  TileItem* items;  // [cap_items]
};

// One matrix's tile configuration and bin (the same cost model as the host
// planner); shared by fw_plan_kernel and its host replay.  Tile times are
// formed with one fmaf and work is summed as 64-bit integer nanoseconds, so
// the device and the host replay (on any CPU) make the same decisions.
struct FwMat {
  int bad;    // size negative or above max_dim: skipped
  int cfg;    // -1: no output (M or N is 0, or skipped)
  int tiles;
  int bin;    // quarter-octave bin of the modelled tile time
};

__host__ __device__ inline long long fw_tiles(int M, int N, const SimtCfg& g) {
  return (long long)((M + g.bm - 1) / g.bm) * ((N + g.bn - 1) / g.bn);
}
__host__ __device__ inline float fw_tile_ns(int K, const TileCost& c) {
  return fmaf(c.b_ns, (float)K, c.a_ns);
}
// TileItem holds 16-bit tile coordinates: a configuration with more than
// 65535 tiles along M or N is not a candidate (the host planner's rule).
__host__ __device__ inline bool fw_fits(int M, int N, const SimtCfg& g) {
  return (M + g.bm - 1) / g.bm <= 65535 && (N + g.bn - 1) / g.bn <= 65535;
}
__host__ __device__ inline long long fw_work(int M, int N, int K, int cfg, const SimtCfg* cfgs,
                                             const TileCost* cost) {
  return fw_tiles(M, N, cfgs[cfg]) * (long long)fw_tile_ns(K, cost[cfg]);
}

__host__ __device__ inline FwMat fw_plan_matrix(int M, int N, int K, int max_dim,
                                                const SimtCfg* cfgs, const TileCost* cost) {
  FwMat r{};
  r.bad = M < 0 || N < 0 || K < 0 || M > max_dim || N > max_dim;
  r.cfg = -1;
  if (!r.bad && M > 0 && N > 0) {
    double bw = 0.0;
    for (int c = kSimtNumCfgs - 1; c >= 0; --c) {
      if (!fw_fits(M, N, cfgs[c])) continue;
      const long long t = fw_tiles(M, N, cfgs[c]);
      const double w = (double)t * fw_tile_ns(K, cost[c]);
      if (r.cfg < 0 || w < bw * 0.999) {
        r.cfg = c;
        r.tiles = (int)t;
        bw = w;
      }
    }
  }
  return r;
}

// Rebalance step of one matrix on configuration `cfg` (the host planner's
// rule, plan.cpp choose_tiles): if its tile is longer than the average load
// W / slots of a persistent CTA, the configuration with shorter and more
// tiles of least total work, if that lowers the makespan bound
// max(W / slots, longest tile) by at least a quarter; else -1.  (Measured on
// the reference's shape file: the model overstates what splitting gains --
// 4.8x predicted, 1.46x measured at 8 matrices -- and a 6 % predicted gain at
// 256 matrices was a 7 % loss, hence the margin.)
__host__ __device__ inline int fw_rebalance(int M, int N, int K, int cfg, long long W,
                                            long long slots, const SimtCfg* cfgs,
                                            const TileCost* cost) {
  const long long tt = (long long)fw_tile_ns(K, cost[cfg]);
  if (tt * slots <= W) return -1;
  const long long tiles = fw_tiles(M, N, cfgs[cfg]);
  const long long w_old = tiles * tt;
  int best = -1;
  long long bw = 0, btt = 0;
  for (int c = 0; c < kSimtNumCfgs; ++c) {
    if (!fw_fits(M, N, cfgs[c])) continue;
    const long long t2 = (long long)fw_tile_ns(K, cost[c]);
    const long long n2 = fw_tiles(M, N, cfgs[c]);
    if (t2 >= tt || n2 <= tiles) continue;
    const long long w = n2 * t2;
    if (best < 0 || w < bw) {
      best = c;
      bw = w;
      btt = t2;
    }
  }
  if (best < 0) return -1;
  const long long w_new = W - w_old + bw;
  const long long before = W > tt * slots ? W : tt * slots;
  const long long after = w_new > btt * slots ? w_new : btt * slots;
  return after < before - before / 4 ? best : -1;
}
constexpr int kRebalanceRounds = 8;

__global__ void fw_plan_kernel(const int* __restrict__ dM, const int* __restrict__ dN,
                               const int* __restrict__ dK, int batch, int max_dim, int slots,
                               FwScratch s) {
  __shared__ int bin_tiles[kBins];
  __shared__ int bin_start[kBins];
  __shared__ unsigned long long work, dwork;
  __shared__ int changed;
  for (int b = threadIdx.x; b < kBins; b += blockDim.x) bin_tiles[b] = 0;
  if (threadIdx.x == 0) work = 0;
  __syncthreads();
  // per-matrix choice (mat_start: -1 no output, 0 has tiles, until the end)
  for (int i = threadIdx.x; i < batch; i += blockDim.x) {
    const int M = dM[i], N = dN[i], K = dK[i];
    const FwMat r = fw_plan_matrix(M, N, K, max_dim, c_cfgs, c_cost);
    if (r.bad) atomicOr(s.err, 1);
    s.descs[i] = MatDesc{M, N, K, max(M, 1), max(K, 1), max(M, 1), r.cfg < 0 ? 0 : r.cfg, 0};
    s.mat_start[i] = r.cfg < 0 ? -1 : 0;
    if (r.cfg >= 0) atomicAdd(&work, (unsigned long long)fw_work(M, N, K, r.cfg, c_cfgs, c_cost));
  }
  // parallelism rebalance in rounds, each against the round's starting total
  for (int round = 0; round < kRebalanceRounds; ++round) {
    __syncthreads();
    const long long W = (long long)work;
    if (threadIdx.x == 0) {
      dwork = 0;
      changed = 0;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < batch; i += blockDim.x) {
      if (s.mat_start[i] < 0) continue;
      const MatDesc d = s.descs[i];
      const int c2 = fw_rebalance(d.M, d.N, d.K, d.cfg, W, slots, c_cfgs, c_cost);
      if (c2 < 0) continue;
      atomicAdd(&dwork, (unsigned long long)(fw_work(d.M, d.N, d.K, c2, c_cfgs, c_cost) -
                                            fw_work(d.M, d.N, d.K, d.cfg, c_cfgs, c_cost)));
      s.descs[i].cfg = c2;
      changed = 1;
    }
    __syncthreads();
    if (!changed) break;
    if (threadIdx.x == 0) work = (unsigned long long)W + dwork;
  }
  __syncthreads();
  // bins of the final tile times; each matrix reserves its tiles in its bin
  for (int i = threadIdx.x; i < batch; i += blockDim.x) {
    if (s.mat_start[i] < 0) continue;
    const MatDesc d = s.descs[i];
    const int bin = min(kBins - 1, max(0, quarter_octave(fw_tile_ns(d.K, c_cost[d.cfg])) - 24));
    s.descs[i].aux = bin;
    s.mat_start[i] = atomicAdd(&bin_tiles[bin], (int)fw_tiles(d.M, d.N, c_cfgs[d.cfg]));
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int b = kBins - 1; b >= 0; --b) {  // longest tiles first
      bin_start[b] = run;
      run += bin_tiles[b];
    }
    *s.n_items = run;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < batch; i += blockDim.x) {
    const int off = s.mat_start[i];
    if (off >= 0) s.mat_start[i] = bin_start[s.descs[i].aux] + off;
  }
}

__global__ void fw_expand_kernel(int batch, FwScratch s) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= batch) return;
  const int start = s.mat_start[warp];
  if (start < 0) return;
  const MatDesc d = s.descs[warp];
  const int tmx = (d.M + c_cfgs[d.cfg].bm - 1) / c_cfgs[d.cfg].bm;
  const int tnx = (d.N + c_cfgs[d.cfg].bn - 1) / c_cfgs[d.cfg].bn;
  const int tiles = tmx * tnx;
  for (int t = lane; t < tiles; t += 32)
    s.items[start + t] = TileItem{warp, (uint16_t)(t % tmx), (uint16_t)(t / tmx)};
}

struct FwContext {
  void* mem = nullptr;
  size_t cap_batch = 0;
  size_t cap_items = 0;
  FwScratch s{};
  bool consts = false;
};

std::mutex g_fw_mu;
std::unordered_map<int, FwContext> g_fw;

}  // namespace
}  // namespace bgemm

using namespace bgemm;

extern "C" bgemm_status_t bgemm_framework_gemm(const int* dM, const int* dN, const int* dK,
                                               float* const* dA, float* const* dB,
                                               float* const* dC, const int* dT, int batch,
                                               int max_dim, bgemm_stream_t stream) {
  (void)dT;  // tile choice is this library's own
  if (batch < 0) return set_error(BGEMM_ERROR_INVALID_VALUE, 8, -1, "batch < 0");
  if (batch == 0) return BGEMM_SUCCESS;
  if (!dM) return set_error(BGEMM_ERROR_INVALID_VALUE, 1, -1, "M is NULL");
  if (!dN) return set_error(BGEMM_ERROR_INVALID_VALUE, 2, -1, "N is NULL");
  if (!dK) return set_error(BGEMM_ERROR_INVALID_VALUE, 3, -1, "K is NULL");
  if (!dA) return set_error(BGEMM_ERROR_INVALID_VALUE, 4, -1, "A is NULL");
  if (!dB) return set_error(BGEMM_ERROR_INVALID_VALUE, 5, -1, "B is NULL");
  if (!dC) return set_error(BGEMM_ERROR_INVALID_VALUE, 6, -1, "C is NULL");
  if (max_dim < 1 || max_dim > (1 << 20))
    return set_error(BGEMM_ERROR_INVALID_VALUE, 9, -1, "max_dim = %d not in [1, 2^20]",
                     max_dim);
  DeviceFacts df;
  bgemm_status_t st = device_facts(&df);
  if (st != BGEMM_SUCCESS) return st;

  // worst-case queue: every matrix max_dim x max_dim in 16 x 16 tiles, 8
  // bytes per item (batch = 1024, max_dim = 65536 would be 128 GB)
  const size_t per = (size_t)((max_dim + 15) / 16);
  const size_t need_items = (size_t)batch * per * per;
  if (need_items > (size_t)INT32_MAX)
    return set_error(BGEMM_ERROR_NOT_SUPPORTED, 9, -1,
                     "batch * ceil(max_dim/16)^2 = %zu queue items exceeds 2^31 - 1; pass a "
                     "tighter max_dim",
                     need_items);
  std::lock_guard<std::mutex> lk(g_fw_mu);
  FwContext& ctx = g_fw[df.device];
  if (!ctx.consts) {
    cudaError_t e = cudaMemcpyToSymbol(c_cfgs, kSimtCfgs, sizeof(kSimtCfgs));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_cost, kSimtCost, sizeof(kSimtCost));
    if (e != cudaSuccess) return cuda_error(e, "framework constants");
    ctx.consts = true;
  }
  if ((size_t)batch > ctx.cap_batch || need_items > ctx.cap_items) {
    const size_t cb = std::max((size_t)batch, ctx.cap_batch);
    const size_t ci = std::max(need_items, ctx.cap_items);
    const size_t off_descs = 256;
    const size_t off_start = off_descs + ((sizeof(MatDesc) * cb + 255) & ~size_t(255));
    const size_t off_items = off_start + ((sizeof(int) * cb + 255) & ~size_t(255));
    const size_t total = off_items + sizeof(TileItem) * ci;
    if (ctx.mem) cudaFree(ctx.mem);  // waits for kernels still using it
    ctx.mem = nullptr;
    ctx.cap_batch = ctx.cap_items = 0;
    cudaError_t e = cudaMalloc(&ctx.mem, total);
    if (e != cudaSuccess)
      return set_error(BGEMM_ERROR_ALLOC, 0, -1, "framework queue of %zu bytes: %s", total,
                       cudaGetErrorString(e));
    e = cudaMemset(ctx.mem, 0, 256);
    if (e != cudaSuccess) return cuda_error(e, "framework queue init");
    char* b = static_cast<char*>(ctx.mem);
    ctx.s.err = reinterpret_cast<int*>(b);
    ctx.s.n_items = reinterpret_cast<int*>(b + 4);
    ctx.s.counters = reinterpret_cast<int*>(b + 128);
    ctx.s.descs = reinterpret_cast<MatDesc*>(b + off_descs);
    ctx.s.mat_start = reinterpret_cast<int*>(b + off_start);
    ctx.s.items = reinterpret_cast<TileItem*>(b + off_items);
    ctx.cap_batch = cb;
    ctx.cap_items = ci;
  }
  const int grid = df.num_sms * df.simt_ctas_per_sm;
  fw_plan_kernel<<<1, 1024, 0, stream>>>(dM, dN, dK, batch, max_dim, grid, ctx.s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "framework plan kernel");
  fw_expand_kernel<<<(batch + 7) / 8, 256, 0, stream>>>(batch, ctx.s);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "framework expand kernel");
  SimtParams sp{ctx.s.descs, ctx.s.items, 0, ctx.s.n_items, ctx.s.counters, 1.0f, 1.0f,
                const_cast<const float* const*>(dA), const_cast<const float* const*>(dB), dC};
  e = simt_launch(sp, grid, stream);
  if (e != cudaSuccess) return cuda_error(e, "framework SIMT launch");
  return BGEMM_SUCCESS;
}

namespace bgemm {

// Runs the three launches of the device-queue path on scratch the caller
// provides: `base` holds counters, descriptors, per-matrix queue offsets and
// up to `cap_items` work items for up to `cap_batch` matrices (layout below,
// fw_scratch_bytes gives its size); `err` receives bit 0 for a size that is
// negative or above max_dim.  Allocates nothing.
size_t fw_scratch_bytes(size_t cap_batch, size_t cap_items) {
  const size_t off_descs = 256;
  const size_t off_start = off_descs + ((sizeof(MatDesc) * cap_batch + 255) & ~size_t(255));
  const size_t off_items = off_start + ((sizeof(int) * cap_batch + 255) & ~size_t(255));
  return off_items + sizeof(TileItem) * cap_items;
}

cudaError_t fw_launch_on_scratch(const int* dM, const int* dN, const int* dK, float* const* dA,
                                 float* const* dB, float* const* dC, int batch, int max_dim,
                                 void* base, size_t cap_batch, int* err, int grid,
                                 cudaStream_t stream) {
  const size_t off_descs = 256;
  const size_t off_start = off_descs + ((sizeof(MatDesc) * cap_batch + 255) & ~size_t(255));
  const size_t off_items = off_start + ((sizeof(int) * cap_batch + 255) & ~size_t(255));
  char* b = static_cast<char*>(base);
  FwScratch s;
  s.err = err;
  s.n_items = reinterpret_cast<int*>(b + 4);
  s.counters = reinterpret_cast<int*>(b + 128);
  s.descs = reinterpret_cast<MatDesc*>(b + off_descs);
  s.mat_start = reinterpret_cast<int*>(b + off_start);
  s.items = reinterpret_cast<TileItem*>(b + off_items);
  {
    std::lock_guard<std::mutex> lk(g_fw_mu);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    FwContext& ctx = g_fw[dev];
    if (!ctx.consts) {
      e = cudaMemcpyToSymbol(c_cfgs, kSimtCfgs, sizeof(kSimtCfgs));
      if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_cost, kSimtCost, sizeof(kSimtCost));
      if (e != cudaSuccess) return e;
      ctx.consts = true;
    }
  }
  fw_plan_kernel<<<1, 1024, 0, stream>>>(dM, dN, dK, batch, max_dim, grid, s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  fw_expand_kernel<<<(batch + 7) / 8, 256, 0, stream>>>(batch, s);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  SimtParams sp{s.descs, s.items, 0, s.n_items, s.counters, 1.0f, 1.0f,
                const_cast<const float* const*>(dA), const_cast<const float* const*>(dB), dC};
  return simt_launch(sp, grid, stream);
}

}  // namespace bgemm

extern "C" bgemm_status_t bgemm_framework_release(void) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
  {
    std::lock_guard<std::mutex> lk(g_fw_mu);
    auto it = g_fw.find(dev);
    if (it != g_fw.end() && it->second.mem) {
      e = cudaFree(it->second.mem);  // waits for kernels still using it
      it->second.mem = nullptr;
      it->second.cap_batch = it->second.cap_items = 0;
      if (e != cudaSuccess) return cuda_error(e, "framework scratch release");
    }
  }
  return fwtc_release(dev);
}

extern "C" bgemm_status_t bgemm_framework_check_device(bgemm_stream_t stream) {
  int dev = 0;
  cudaGetDevice(&dev);
  cudaError_t e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return cuda_error(e, "cudaStreamSynchronize");
  bgemm_status_t st = fwtc_check_device(dev);
  if (st != BGEMM_SUCCESS) return st;
  std::lock_guard<std::mutex> lk(g_fw_mu);
  auto it = g_fw.find(dev);
  if (it == g_fw.end() || !it->second.mem) return BGEMM_SUCCESS;
  int err = 0;
  e = cudaMemcpy(&err, it->second.s.err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_error(e, "framework error word");
  if (err) {
    cudaMemset(it->second.s.err, 0, sizeof(int));
    return set_error(BGEMM_ERROR_INVALID_VALUE, 1, -1,
                     "a matrix size was negative or above max_dim; such matrices were skipped");
  }
  return BGEMM_SUCCESS;
}

// Host replay of fw_plan_kernel + fw_expand_kernel (tests without a GPU): the
// same per-matrix choices and rebalance rounds, reserved in matrix order
// instead of by atomics; `slots` is the persistent SIMT grid the entry uses.
extern "C" int bgemm_debug_framework_plan(const int* M, const int* N, const int* K, int batch,
                                          int max_dim, int slots, int* cfg_out, int* items_out,
                                          int max_items, int* err) {
  if (batch < 0 || !err || slots < 1 || (batch > 0 && (!M || !N || !K))) return -1;
  std::vector<int> cfg(batch, -1);
  std::vector<int> start(batch, -1);
  int bin_tiles[kBins] = {};
  *err = 0;
  long long W = 0;
  for (int i = 0; i < batch; ++i) {
    const FwMat r = fw_plan_matrix(M[i], N[i], K[i], max_dim, kSimtCfgs, kSimtCost);
    if (r.bad) *err |= 1;
    cfg[i] = r.cfg;
    if (r.cfg >= 0) W += fw_work(M[i], N[i], K[i], r.cfg, kSimtCfgs, kSimtCost);
  }
  for (int round = 0; round < kRebalanceRounds; ++round) {
    long long dW = 0;
    bool changed = false;
    for (int i = 0; i < batch; ++i) {
      if (cfg[i] < 0) continue;
      const int c2 = fw_rebalance(M[i], N[i], K[i], cfg[i], W, slots, kSimtCfgs, kSimtCost);
      if (c2 < 0) continue;
      dW += fw_work(M[i], N[i], K[i], c2, kSimtCfgs, kSimtCost) -
            fw_work(M[i], N[i], K[i], cfg[i], kSimtCfgs, kSimtCost);
      cfg[i] = c2;
      changed = true;
    }
    if (!changed) break;
    W += dW;
  }
  std::vector<int> bin(batch, 0);
  for (int i = 0; i < batch; ++i) {
    if (cfg_out) cfg_out[i] = cfg[i];
    if (cfg[i] < 0) continue;
    bin[i] = std::min(kBins - 1,
                      std::max(0, quarter_octave(fw_tile_ns(K[i], kSimtCost[cfg[i]])) - 24));
    start[i] = bin_tiles[bin[i]];
    bin_tiles[bin[i]] += (int)fw_tiles(M[i], N[i], kSimtCfgs[cfg[i]]);
  }
  int bin_start[kBins], n = 0;
  for (int b = kBins - 1; b >= 0; --b) {
    bin_start[b] = n;
    n += bin_tiles[b];
  }
  if (items_out && n > max_items) return -1;
  for (int i = 0; items_out && i < batch; ++i) {
    if (start[i] < 0) continue;
    const int tmx = (M[i] + kSimtCfgs[cfg[i]].bm - 1) / kSimtCfgs[cfg[i]].bm;
    const int tnx = (N[i] + kSimtCfgs[cfg[i]].bn - 1) / kSimtCfgs[cfg[i]].bn;
    const int s0 = bin_start[bin[i]] + start[i];
    for (int t = 0; t < tmx * tnx; ++t) {
      items_out[3 * (s0 + t)] = i;
      items_out[3 * (s0 + t) + 1] = t % tmx;
      items_out[3 * (s0 + t) + 2] = t / tmx;
    }
  }
  return n;
}
