// ref_shim.h -- lets the reference's CUDA tile bodies compile as host C++ so
// that their outputs can be produced on a CPU (test infrastructure only).
//
// Each CUDA thread of a block becomes one std::thread; __syncthreads() becomes
// a std::barrier wait over the block's threads; threadIdx/blockIdx are
// thread-local.  Blocks run one after another.  Nothing here changes the
// arithmetic of the included tile bodies: fma(float, float, float) maps to the
// correctly rounded single-precision fused multiply-add, as on the GPU.
#pragma once
#include <barrier>
#include <cstddef>

#define __device__
#define __global__
#define __shared__
#define __forceinline__ inline

struct alignas(8) float2 { float x, y; };
struct alignas(16) float4 { float x, y, z, w; };
struct dim3 { unsigned x = 0, y = 0, z = 0; };

extern thread_local dim3 threadIdx;
extern thread_local dim3 blockIdx;
extern thread_local std::barrier<>* g_block_barrier;

inline void __syncthreads() { g_block_barrier->arrive_and_wait(); }
