// hbm_probe.cu -- streaming kernels that measure the HBM ceiling of a given
// read:write mix, the denominator of the split pre-pass's roofline.
//
// The pre-pass (tc_pack_kernel) reads each operand element once and writes
// its hi and lo halves: one read for two writes.  A plain device copy (one
// read, one write) is a different mix, and HBM turns writes around more
// slowly than reads, so the probe times that exact mix.  Each kernel walks
// float4 words grid-stride; the host entry picks the grid.
#include <cuda_runtime.h>

#include "bgemm_internal.h"

namespace bgemm {
namespace {

__global__ void probe_r1w2(const float4* __restrict__ x, float4* __restrict__ y1,
                           float4* __restrict__ y2, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float4 v = x[i];
    y1[i] = v;
    y2[i] = make_float4(v.x * 0.5f, v.y * 0.5f, v.z * 0.5f, v.w * 0.5f);
  }
}

__global__ void probe_r1w1(const float4* __restrict__ x, float4* __restrict__ y, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = x[i];
}

__global__ void probe_w1(float4* __restrict__ y, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = make_float4(1.0f, 2.0f, 3.0f, 4.0f);
}

// Reads only; the sum is stored only under a condition the data never meets,
// which keeps the loads alive.
__global__ void probe_r1(const float4* __restrict__ x, float* __restrict__ sink, long long n) {
  float s = 0.0f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float4 v = x[i];
    s += v.x + v.y + v.z + v.w;
  }
  if (s == -1.2345e38f) sink[0] = s;
}

}  // namespace
}  // namespace bgemm

// kind 0: read x, write y1 and y2 (the pre-pass's mix); 1: copy x -> y1;
// 2: write y1; 3: read x.  n4 float4 words per buffer; 256 threads per CTA.
extern "C" int bgemm_debug_hbm_probe(int kind, const float* x, float* y1, float* y2, long long n4,
                                     int grid, void* stream) {
  using namespace bgemm;
  if (kind < 0 || kind > 3 || n4 <= 0 || grid < 1) return -1;
  if (!y1 || (kind != 2 && !x) || (kind == 0 && !y2)) return -1;
  const uintptr_t mis = reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y1) |
                        reinterpret_cast<uintptr_t>(y2);
  if (mis & 15u) return -1;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const float4* xv = reinterpret_cast<const float4*>(x);
  float4* y1v = reinterpret_cast<float4*>(y1);
  float4* y2v = reinterpret_cast<float4*>(y2);
  switch (kind) {
    case 0: probe_r1w2<<<grid, 256, 0, s>>>(xv, y1v, y2v, n4); break;
    case 1: probe_r1w1<<<grid, 256, 0, s>>>(xv, y1v, n4); break;
    case 2: probe_w1<<<grid, 256, 0, s>>>(y1v, n4); break;
    default: probe_r1<<<grid, 256, 0, s>>>(xv, y1, n4); break;
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}
