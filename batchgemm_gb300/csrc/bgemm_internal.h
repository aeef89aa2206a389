// bgemm_internal.h -- structures shared by the host planner and the kernels.
#pragma once
#include <stdint.h>

#include <cuda_runtime.h>

namespace bgemm {

// Per-matrix descriptor, uploaded once per plan (32 bytes).
struct MatDesc {
  int M, N, K;
  int lda, ldb, ldc;
  int cfg;    // tile configuration id of the plan's mode
  int aux;    // flag bits below (plan paths); size bin (device-built framework path)
};
// MatDesc::aux flags: op(A) = A^T (A stored K x M), op(B) = B^T (B stored
// N x K); bit 30 is the tensor-core modes' operand swap.
constexpr int kTransAFlag = 1 << 28;
constexpr int kTransBFlag = 1 << 29;

// floor(4 * log2(x)) for x >= 1 (0 for smaller x), from the float's exponent
// and mantissa bits with fixed quarter-octave edges, so that the host
// replays of the device planners bin exactly as the device does (log2f of
// the host C library and of CUDA may differ in the last bit).
__host__ __device__ inline int quarter_octave(float x) {
  if (!(x >= 1.0f)) return 0;
  union {
    float f;
    uint32_t u;
  } v;
  v.f = x;
  const int e = (int)((v.u >> 23) & 0xffu) - 127;
  v.u = (v.u & 0x007fffffu) | 0x3f800000u;  // mantissa in [1, 2)
  const int q = (v.f >= 1.18920712f) + (v.f >= 1.41421356f) + (v.f >= 1.68179283f);
  return 4 * e + q;
}

// One work item of the largest-first tile queue (8 bytes).
struct TileItem {
  int mat;
  uint16_t tm, tn;  // tile coordinates along M and N (tensor-core swapped
                    // orientation: along the MMA's M and N)
};

// ---------------------------------------------------------------- SIMT ----
// Tile configurations of the FP32 SIMT kernel: 256 threads arranged 16 x 16,
// each owning a TM x TN register tile.
struct SimtCfg {
  int bm, bn, tm, tn;
};
// Ids 8 and 9 are the thin tiles: 8 x 128 for M <= 8 (each thread four rows
// of one column) and 128 x 8 for N <= 8 (one row of four columns), where the
// 16-wide tiles would compute mostly padding.
constexpr int kSimtNumCfgs = 10;
constexpr SimtCfg kSimtCfgs[kSimtNumCfgs] = {
    {16, 16, 1, 1},  {32, 32, 2, 2},  {64, 32, 4, 2},  {32, 64, 2, 4},
    {64, 64, 4, 4},  {128, 64, 8, 4}, {64, 128, 4, 8}, {128, 128, 8, 8},
    {8, 128, 4, 1},  {128, 8, 1, 4},
};

struct SimtParams {
  const MatDesc* descs;
  const TileItem* items;
  int n_items;
  const int* n_items_dev;  // if set, the item count is read from the device
  int* counters;  // [0]: next work item, [1]: CTAs finished (self-reset)
  float alpha, beta;
  const float* const* A;
  const float* const* B;
  float* const* C;
};

// transposed: the plan's matrices carry kTransAFlag / kTransBFlag
cudaError_t simt_launch(const SimtParams& p, int grid, cudaStream_t stream,
                        bool transposed = false);
int simt_ctas_per_sm();

}  // namespace bgemm
