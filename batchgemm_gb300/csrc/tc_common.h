// tc_common.h -- structures of the tensor-core (tcgen05) path shared by the
// planner and the kernels.
#pragma once
#include <stdint.h>

#include <cuda.h>
#include <cuda_runtime.h>

#include "bgemm_internal.h"

namespace bgemm {

// Element kinds of the packed operands.
enum TcKind : int { kKindTF32 = 0, kKindBF16 = 1 };
// Split pre-pass grid: CTAs per SM (about five waves of the three resident).
constexpr int kPackCtasPerSm = 16;

// Tile configurations: UMMA M = 128 rows of the "A side" operand, UMMA N =
// BN rows of the "B side".  Ids 0..3 keep A on the A side (BN 16/32/64/128);
// ids 4..7 swap the operands (C^T = B^T A^T, the A side walks N) for
// matrices whose M is small.
constexpr int kTcBM = 128;
constexpr int kTcMaxBN = 128;
__host__ __device__ constexpr int tc_cfg_bn(int cfg) { return 16 << (cfg & 3); }
__host__ __device__ constexpr bool tc_cfg_swap(int cfg) { return (cfg & 4) != 0; }
// CTA-pair configurations (ids 8..15): a 256 x BN tile on two SMs,
// BN = 64, 128, 256 (ids with (cfg & 3) == 3 are unused); bit 2 swaps.
// Every mode can run them (tc2_kernel.cu).
constexpr int kTcPairCfg0 = 8;
__host__ __device__ constexpr bool tc_cfg_pair(int cfg) { return cfg >= kTcPairCfg0; }
__host__ __device__ constexpr int tc2_cfg_bn(int cfg) { return 64 << (cfg & 3); }
__host__ __device__ constexpr bool tc2_cfg_valid(int cfg) { return (cfg & 3) != 3; }

// Promotion schedule of the split modes on CTA pairs, per bucket of K:
// bucket 0 is K <= 64, then one bucket per octave ((64, 128], (128, 256],
// ..., (2048, 4096], above 4096).  group[b] = the number of 128-byte K
// slices whose MMAs accumulate into one TMEM buffer before the epilogue adds
// it into FP32 registers; 0 = promote after every MMA of K and keep the
// lo*lo product too (the small-K path, where the split error dominates).
constexpr int kTcSchedBuckets = 8;
struct TcSchedule {
  unsigned long long packed;  // byte b = group of bucket b (shifts, no indexing)
  __host__ __device__ int group(int b) const { return (int)((packed >> (8 * b)) & 0xffu); }
  __host__ __device__ void set(int b, int g) {
    packed = (packed & ~(0xffull << (8 * b))) | ((unsigned long long)(g & 0xff) << (8 * b));
  }
};
__host__ __device__ inline int tc_sched_bucket(int K) {
  if (K <= 64) return 0;
  int b = 0;
  for (unsigned v = (unsigned)(K - 1) >> 6; v > 1u; v >>= 1) ++b;  // floor(log2(K-1)) - 6
  return b + 1 < kTcSchedBuckets ? b + 1 : kTcSchedBuckets - 1;
}

// One pre-pass job: split/pack a strip of 32 rows of one operand.
struct PackJob {
  int mat;
  int op;  // 0: A (M x K, transposed to rows of K), 1: B (N x K rows)
  int r0;  // first row of the strip
  int pad;
};

// Where the packed operands of a matrix live (byte offsets into the workspace).
struct PackDesc {
  long long a_hi, a_lo, b_hi, b_lo;
  int kpad;  // row length in elements (K rounded up to 16 bytes)
  int pad[3];
};

struct TcPackParams {
  const MatDesc* descs;
  const PackDesc* pdescs;
  const PackJob* jobs;
  int n_jobs;
  const int* n_jobs_dev;  // if set, the job count is read from the device
  int kind;
  int split;
  char* ws;
  const float* const* A;
  const float* const* B;
};

struct TcGemmParams {
  const MatDesc* descs;
  const TileItem* items;
  int n_items;
  const int* n_items_dev;      // if set, the item count is read from the device
  int* counters;               // [0] queue head, [1] CTAs finished
  const CUtensorMap* tmaps;    // 4 per matrix: A-side hi, A-side lo, B-side hi, B-side lo
  float alpha, beta;
  float* const* C;
  int* error;                  // bit 0: a bounded device wait expired
  unsigned long long timeout_ns;
  unsigned long long* cta_times;  // if set: [2 * blockIdx] start, [+1] end (global timer, ns)
  TcSchedule sched;               // promotion groups of the split modes (pair kernel)
};
// The schedule the kernels use for a mode: the autotuned table, or a process-
// wide override set through bgemm_debug_set_tc_schedule (the autotuner's sweep).
TcSchedule tc_schedule(int mode);

// Device-side construction of the per-matrix tensor maps: one warp per map
// copies a host-encoded template, patches address, dims and row stride with
// tensormap.replace, and publishes it with a release fence.  The driver's
// encoding also holds fields derived from the box height and from the
// tensor's total extent (measured on GB300: two classes, below and at or
// above 128 KiB), which the replace instruction does not recompute; so there
// is one template per (box height 16/32/64/128, extent class), and the
// result is byte-identical to encoding the map on the host.
constexpr int kTmapBoxClasses = 4;
constexpr long long kTmapLargeExtent = 131072;
__host__ __device__ constexpr int tmap_template_index(int box_rows, bool large) {
  return (box_rows <= 16 ? 0 : box_rows <= 32 ? 1 : box_rows <= 64 ? 2 : 3) * 2 + (large ? 1 : 0);
}
struct TcTmapParams {
  const MatDesc* descs;
  const PackDesc* pdescs;
  const CUtensorMap* templ;  // 2 * kTmapBoxClasses templates of the plan's element kind
  CUtensorMap* out;          // 4 per matrix
  const char* ws;
  int batch;
  int kind;
  int pair;
};

cudaError_t tc_pack_launch(const TcPackParams& p, int grid, cudaStream_t s);
// one CTA waiting on a barrier that never completes (bounded-wait self-test)
cudaError_t tc_wait_selftest_launch(int* err, int* out, unsigned long long limit_ns,
                                    cudaStream_t s);
cudaError_t tc_tmap_launch(const TcTmapParams& p, cudaStream_t s);
cudaError_t tc_gemm_launch(int kind, int split, const TcGemmParams& p, int grid, cudaStream_t s);
int tc_smem_bytes(int kind, int split);
// CTA-pair kernel; grid = 2 x clusters
cudaError_t tc2_gemm_launch(int kind, int split, const TcGemmParams& p, int grid,
                            cudaStream_t s);
int tc2_max_clusters();

}  // namespace bgemm
