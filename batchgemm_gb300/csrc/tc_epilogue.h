// tc_epilogue.h -- the C read/write of the tensor-core kernels' epilogue warps.
//
// A warp of an epilogue holds, per lane, one accumulator row of a tile (TMEM
// lane row0 + lane, the "A side") and COLS consecutive accumulator columns
// (the "B side", starting at col_base).  Unswapped tiles map the A side to
// C's rows m, so lane-consecutive elements are contiguous in column-major C
// and every access is a coalesced 128-byte line.  Swapped tiles (C^T =
// B^T A^T) map the A side to C's columns n: there each 32 x 32 block is first
// transposed across the warp with shuffles, after which lanes again walk
// consecutive m.
//
// With beta != 0 the old C is read.  In the one-SM kernel c_prefetch pulls
// those lines into L2 when a tile starts, so the final reads (issued in
// groups before the stores of their group) hit L2 instead of waiting on HBM
// per element.  The CTA-pair kernel prefetches only if its autotuned lead is
// nonzero (measured: none is fastest -- the prefetched lines displace operand
// lines the MMA still needs) and pipelines its reads one group ahead of the
// stores (c_store_pipe).
#pragma once
#include <stdint.h>

namespace bgemm {

__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(reinterpret_cast<uint64_t>(p)));
}

// x[off .. off+31] of every lane form a 32 x 32 block X (lane t holds row t);
// afterwards lane t holds column t (x[off + j] = X[j][t]).  Recursive block
// transpose: at step s, lanes with bit s clear hand their columns with bit s
// set to the partner lane t ^ s and take the partner's columns with bit s
// clear.
template <int COLS>
__device__ __forceinline__ void warp_transpose32(float (&x)[COLS], int off, int lane) {
#pragma unroll
  for (int s = 16; s >= 1; s >>= 1) {
    const bool upper = (lane & s) != 0;
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      if (j & s) continue;
      const float send = upper ? x[off + j] : x[off + (j | s)];
      const float recv = __shfl_xor_sync(0xffffffffu, send, s);
      if (upper)
        x[off + j] = recv;
      else
        x[off + (j | s)] = recv;
    }
  }
}

// L2 prefetch of the C elements this warp reads in c_store (beta != 0).
template <int COLS>
__device__ __forceinline__ void c_prefetch(const float* C, long long ldc, int M, int N, bool swap,
                                           int row0, int col_base, int ncols, int lane) {
  if (!swap) {
    const int m = row0 + lane;
    if (m >= M) return;
#pragma unroll 8
    for (int j = 0; j < COLS; ++j) {
      const int n = col_base + j;
      if (j < ncols && n < N) prefetch_l2(C + m + (long long)n * ldc);
    }
  } else {
#pragma unroll
    for (int c0 = 0; c0 < COLS; c0 += 32) {
      if (c0 >= ncols) break;
      const int m = col_base + c0 + lane;
      if (c0 + lane < ncols && m < M) {
#pragma unroll 8
        for (int j = 0; j < 32; ++j) {
          const int n = row0 + j;
          if (n < N) prefetch_l2(C + m + (long long)n * ldc);
        }
      }
    }
  }
}

// C <- alpha * r + beta * C over the warp's block (C is not read when beta is
// 0).  Swapped tiles transpose r in place.  Reads go kCRead at a time, all
// before the stores of their elements (a store may alias a later load as far
// as the compiler knows, so interleaving them would serialise every read).
constexpr int kCRead = 8;  // C reads in flight per lane (default)

template <int COLS, int NRD = kCRead>
__device__ __forceinline__ void c_store(float (&r)[COLS], float* C, long long ldc, int M, int N,
                                        bool swap, int row0, int col_base, int ncols, float alpha,
                                        float beta, int lane) {
  const bool rd = beta != 0.0f;
#pragma unroll
  for (int c0 = 0; c0 < COLS; c0 += 32) {
    if (c0 >= ncols) break;  // warp-uniform
    int m, n0, nlim;
    bool ok;
    long long step;
    if (!swap) {
      // lane: row m; element j: column col_base + c0 + j
      m = row0 + lane;
      n0 = col_base + c0;
      nlim = min(N - n0, ncols - c0);
      ok = m < M;
    } else {
      warp_transpose32(r, c0, lane);
      // lane: row col_base + c0 + lane; element j: column row0 + j
      m = col_base + c0 + lane;
      n0 = row0;
      nlim = N - n0;
      ok = (c0 + lane < ncols) && m < M;
    }
    step = ldc;
    float* base = C + m + (long long)n0 * ldc;
#pragma unroll
    for (int h = 0; h < 32; h += NRD) {
      float cv[NRD];
#pragma unroll
      for (int j = 0; j < NRD; ++j)
        cv[j] = (rd && ok && h + j < nlim) ? base[(h + j) * step] : 0.0f;
#pragma unroll
      for (int j = 0; j < NRD; ++j)
        if (ok && h + j < nlim)
          base[(h + j) * step] =
              rd ? fmaf(alpha, r[c0 + h + j], beta * cv[j]) : alpha * r[c0 + h + j];
    }
  }
}

// beta != 0 in the CTA-pair kernel: the same read-modify-write, software
// pipelined -- the reads of the next NRD elements are issued before the
// stores of the current NRD (two register buffers), so reads stay in flight
// without a gap at each store (measured: 1 % off the beta = 1 GEMM against
// c_store with 16 reads at a time; 16 pipelined would spill).
template <int COLS, int NRD>
__device__ __forceinline__ void c_store_pipe(float (&r)[COLS], float* C, long long ldc, int M,
                                             int N, bool swap, int row0, int col_base, int ncols,
                                             float alpha, float beta, int lane) {
#pragma unroll
  for (int c0 = 0; c0 < COLS; c0 += 32) {
    if (c0 >= ncols) break;
    int m, n0, nlim;
    bool ok;
    if (!swap) {
      m = row0 + lane;
      n0 = col_base + c0;
      nlim = min(N - n0, ncols - c0);
      ok = m < M;
    } else {
      warp_transpose32(r, c0, lane);
      m = col_base + c0 + lane;
      n0 = row0;
      nlim = N - n0;
      ok = (c0 + lane < ncols) && m < M;
    }
    float* base = C + m + (long long)n0 * ldc;
    float cv[2][NRD];
#pragma unroll
    for (int j = 0; j < NRD; ++j) cv[0][j] = (ok && j < nlim) ? base[(long long)j * ldc] : 0.0f;
#pragma unroll
    for (int h = 0; h < 32; h += NRD) {
      const int cur = (h / NRD) & 1;
      if (h + NRD < 32) {
#pragma unroll
        for (int j = 0; j < NRD; ++j)
          cv[cur ^ 1][j] = (ok && h + NRD + j < nlim) ? base[(long long)(h + NRD + j) * ldc] : 0.0f;
      }
#pragma unroll
      for (int j = 0; j < NRD; ++j)
        if (ok && h + j < nlim)
          base[(long long)(h + j) * ldc] = fmaf(alpha, r[c0 + h + j], beta * cv[cur][j]);
    }
  }
}

}  // namespace bgemm
