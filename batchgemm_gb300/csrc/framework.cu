// framework.cu -- drop-in for the reference framework's kernel entry
//   gemm<<<grid, 256, 16 KB>>>(M, N, K, A, B, C, T_strategy)
// (CUDA/framework/kernel.h:11, launched at CUDA/framework/gemm.cu:200): the
// sizes are device arrays, C_i += A_i * B_i column-major with lda = M_i,
// ldb = K_i, ldc = M_i.
//
// Because the sizes live on the device, the tile queue is built there too:
//   1. fw_plan_kernel (one CTA) picks each matrix's SIMT tile configuration
//      with the same cost model as the host planner, buckets matrices by
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
// planner); shared by fw_plan_kernel and its host replay.
struct FwMat {
  int bad;    // size negative or above max_dim: skipped
  int cfg;    // -1: no output (M or N is 0, or skipped)
  int tiles;
  int bin;    // quarter-octave bin of the modelled tile time
};

__host__ __device__ inline FwMat fw_plan_matrix(int M, int N, int K, int max_dim,
                                                const SimtCfg* cfgs, const TileCost* cost) {
  FwMat r{};
  r.bad = M < 0 || N < 0 || K < 0 || M > max_dim || N > max_dim;
  r.cfg = -1;
  if (!r.bad && M > 0 && N > 0) {
    double bw = 0.0;
    float btt = 0.f;
    for (int c = kSimtNumCfgs - 1; c >= 0; --c) {
      const long long t = (long long)((M + cfgs[c].bm - 1) / cfgs[c].bm) *
                          ((N + cfgs[c].bn - 1) / cfgs[c].bn);
      const float tt = cost[c].a_ns + cost[c].b_ns * (float)K;
      const double w = (double)t * tt;
      if (r.cfg < 0 || w < bw * 0.999) {
        r.cfg = c;
        r.tiles = (int)t;
        bw = w;
        btt = tt;
      }
    }
    r.bin = min(kBins - 1, max(0, quarter_octave(btt) - 24));
  }
  return r;
}

__global__ void fw_plan_kernel(const int* __restrict__ dM, const int* __restrict__ dN,
                               const int* __restrict__ dK, int batch, int max_dim,
                               FwScratch s) {
  __shared__ int bin_tiles[kBins];
  __shared__ int bin_start[kBins];
  for (int b = threadIdx.x; b < kBins; b += blockDim.x) bin_tiles[b] = 0;
  __syncthreads();
  // per-matrix choice; the bin and offset are parked in mat_start for now
  for (int i = threadIdx.x; i < batch; i += blockDim.x) {
    const int M = dM[i], N = dN[i], K = dK[i];
    const FwMat r = fw_plan_matrix(M, N, K, max_dim, c_cfgs, c_cost);
    if (r.bad) atomicOr(s.err, 1);
    s.descs[i] = MatDesc{M, N, K, max(M, 1), max(K, 1), max(M, 1), r.cfg < 0 ? 0 : r.cfg,
                         r.cfg < 0 ? 0 : r.bin};
    s.mat_start[i] = r.cfg < 0 ? -1 : atomicAdd(&bin_tiles[r.bin], r.tiles);
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
  fw_plan_kernel<<<1, 1024, 0, stream>>>(dM, dN, dK, batch, max_dim, ctx.s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "framework plan kernel");
  fw_expand_kernel<<<(batch + 7) / 8, 256, 0, stream>>>(batch, ctx.s);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "framework expand kernel");
  SimtParams sp{ctx.s.descs, ctx.s.items, 0, ctx.s.n_items, ctx.s.counters, 1.0f, 1.0f,
                const_cast<const float* const*>(dA), const_cast<const float* const*>(dB), dC};
  e = simt_launch(sp, df.num_sms * df.simt_ctas_per_sm, stream);
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
  fw_plan_kernel<<<1, 1024, 0, stream>>>(dM, dN, dK, batch, max_dim, s);
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
// same per-matrix choices, reserved in matrix order instead of by atomics.
extern "C" int bgemm_debug_framework_plan(const int* M, const int* N, const int* K, int batch,
                                          int max_dim, int* cfg_out, int* items_out,
                                          int max_items, int* err) {
  if (batch < 0 || !err || (batch > 0 && (!M || !N || !K))) return -1;
  std::vector<FwMat> r(batch);
  std::vector<int> start(batch, -1);
  int bin_tiles[kBins] = {};
  *err = 0;
  for (int i = 0; i < batch; ++i) {
    r[i] = fw_plan_matrix(M[i], N[i], K[i], max_dim, kSimtCfgs, kSimtCost);
    if (r[i].bad) *err |= 1;
    if (cfg_out) cfg_out[i] = r[i].cfg;
    if (r[i].cfg >= 0) {
      start[i] = bin_tiles[r[i].bin];
      bin_tiles[r[i].bin] += r[i].tiles;
    }
  }
  int bin_start[kBins], n = 0;
  for (int b = kBins - 1; b >= 0; --b) {
    bin_start[b] = n;
    n += bin_tiles[b];
  }
  if (items_out && n > max_items) return -1;
  for (int i = 0; items_out && i < batch; ++i) {
    if (start[i] < 0) continue;
    const int tmx = (M[i] + kSimtCfgs[r[i].cfg].bm - 1) / kSimtCfgs[r[i].cfg].bm;
    const int tnx = (N[i] + kSimtCfgs[r[i].cfg].bn - 1) / kSimtCfgs[r[i].cfg].bn;
    const int s0 = bin_start[r[i].bin] + start[i];
    for (int t = 0; t < tmx * tnx; ++t) {
      items_out[3 * (s0 + t)] = i;
      items_out[3 * (s0 + t) + 1] = t % tmx;
      items_out[3 * (s0 + t) + 2] = t / tmx;
    }
  }
  return n;
}
