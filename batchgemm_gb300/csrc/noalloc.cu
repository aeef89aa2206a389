// noalloc.cu -- bgemm_framework_gemm_noalloc: the device-queue FP32 path of
// bgemm_framework_gemm for callers that cannot allocate device memory.
//
// Who needs it: code that must not call cudaMalloc/cudaFree once it is
// running -- a real-time or latency-bound loop where an allocation (which can
// synchronise the whole device) is not allowed, or a plug-in hosted by an
// application that owns the device memory budget through its own pool and
// forbids allocations behind its back.
//
// The tile queue that the regular entry keeps in library-allocated memory
// lives here in one file-scope __device__ array of fixed size, so no call
// allocates anything.  Limits: at most kNoAllocMaxBatch matrices and a worst
// case of kNoAllocMaxTiles 16 x 16 tiles (batch * ceil(max_dim/16)^2);
// anything larger is rejected with BGEMM_ERROR_NOT_SUPPORTED before any work.
// Every device that loads the library holds the array (about 2.2 MB) until
// the process exits.
//
// Set-up: the first call on a device looks up the array's device address
// (cudaGetSymbolAddress, return code checked) with that device current, and
// the shared device planner uploads its cost tables to the device once
// (cudaMemcpyToSymbol, a synchronous copy); make that first call before any
// stream capture begins.  All calls share the one array and it keeps the last
// call's contents, so calls whose work overlaps on the GPU (different
// streams, or different host threads without ordering) race on it and must be
// serialised by the caller.  Each call clears the queue counters and the
// error word it needs before its kernels run.  With d_info == NULL the error
// word is the array's own first int, which the next call clears and nothing
// reads: out-of-range matrices are then skipped silently.
#include <mutex>
#include <unordered_map>

#include "bgemm.h"
#include "bgemm_internal.h"
#include "plan_internal.h"

namespace bgemm {

size_t fw_scratch_bytes(size_t cap_batch, size_t cap_items);
cudaError_t fw_launch_on_scratch(const int* dM, const int* dN, const int* dK, float* const* dA,
                                 float* const* dB, float* const* dC, int batch, int max_dim,
                                 void* base, size_t cap_batch, int* err, int grid,
                                 cudaStream_t stream);

namespace {

constexpr size_t kNoAllocMaxBatch = 4096;
constexpr size_t kNoAllocMaxTiles = size_t(1) << 18;
// 256 B of counters + 32 B descriptors + 4 B offsets per matrix + 8 B per tile
constexpr size_t kNoAllocBytes = 256 + 32 * kNoAllocMaxBatch + 4 * kNoAllocMaxBatch +
                                 8 * kNoAllocMaxTiles + 1024;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_mu;
std::unordered_map<int, void*> g_addr;  // device -> device address of the array

}  // namespace
}  // namespace bgemm

using namespace bgemm;

extern "C" bgemm_status_t bgemm_framework_gemm_noalloc(const int* dM, const int* dN,
                                                       const int* dK, float* const* dA,
                                                       float* const* dB, float* const* dC,
                                                       int batch, int max_dim, int* d_info,
                                                       bgemm_stream_t stream) {
  if (batch < 0) return set_error(BGEMM_ERROR_INVALID_VALUE, 7, -1, "batch < 0");
  if (batch == 0) return BGEMM_SUCCESS;
  if (!dM) return set_error(BGEMM_ERROR_INVALID_VALUE, 1, -1, "M is NULL");
  if (!dN) return set_error(BGEMM_ERROR_INVALID_VALUE, 2, -1, "N is NULL");
  if (!dK) return set_error(BGEMM_ERROR_INVALID_VALUE, 3, -1, "K is NULL");
  if (!dA) return set_error(BGEMM_ERROR_INVALID_VALUE, 4, -1, "A is NULL");
  if (!dB) return set_error(BGEMM_ERROR_INVALID_VALUE, 5, -1, "B is NULL");
  if (!dC) return set_error(BGEMM_ERROR_INVALID_VALUE, 6, -1, "C is NULL");
  if (max_dim < 1 || max_dim > (1 << 20))
    return set_error(BGEMM_ERROR_INVALID_VALUE, 8, -1, "max_dim = %d not in [1, 2^20]",
                     max_dim);
  if ((size_t)batch > kNoAllocMaxBatch)
    return set_error(BGEMM_ERROR_NOT_SUPPORTED, 7, -1,
                     "batch = %d exceeds the %zu matrices the allocation-free queue holds",
                     batch, kNoAllocMaxBatch);
  const size_t per = (size_t)((max_dim + 15) / 16);
  const size_t worst = (size_t)batch * per * per;
  if (worst > kNoAllocMaxTiles)
    return set_error(BGEMM_ERROR_NOT_SUPPORTED, 8, -1,
                     "batch * ceil(max_dim/16)^2 = %zu tiles exceeds the %zu tiles the "
                     "allocation-free queue holds",
                     worst, kNoAllocMaxTiles);
  static_assert(kNoAllocBytes >= 256 + 32 * kNoAllocMaxBatch + 256 + 4 * kNoAllocMaxBatch + 256 +
                                     8 * kNoAllocMaxTiles,
                "scratch layout");
  DeviceFacts df;
  bgemm_status_t st = device_facts(&df);
  if (st != BGEMM_SUCCESS) return st;

  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_addr.find(df.device);
    if (it == g_addr.end()) {
      // once per device, with that device current (device_facts read it)
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(no-alloc scratch)");
      it = g_addr.emplace(df.device, p).first;
    }
    base = it->second;
  }
  if (fw_scratch_bytes(kNoAllocMaxBatch, kNoAllocMaxTiles) > kNoAllocBytes)
    return set_error(BGEMM_ERROR_INTERNAL, 0, -1, "no-alloc scratch layout too small");
  // counters, item count and the error word start from zero on every call
  cudaError_t e = cudaMemsetAsync(base, 0, 256, stream);
  if (e != cudaSuccess) return cuda_error(e, "clearing the no-alloc queue counters");
  int* err = d_info ? d_info : static_cast<int*>(base);
  e = fw_launch_on_scratch(dM, dN, dK, dA, dB, dC, batch, max_dim, base, kNoAllocMaxBatch, err,
                           df.num_sms * df.simt_ctas_per_sm, stream);
  if (e != cudaSuccess) return cuda_error(e, "no-alloc framework launch");
  return BGEMM_SUCCESS;
}
