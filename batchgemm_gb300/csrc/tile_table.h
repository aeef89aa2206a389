// tile_table.h -- per-tile cost model consumed by the planners.
//
// Time of one work item of configuration c on a matrix with inner dimension
// K is modelled as  t = a_c + b_c * K  (nanoseconds for the CTA -- or CTA
// pair -- that runs it, with every other persistent CTA busy too).  The
// planner picks, per matrix, the configuration with the least total time and
// then splits the largest tiles until no single tile is longer than the
// average load of one persistent CTA (the parallelism rebalance).
//
// tile_table_tuned.inc, written by batchgemm_gb300/autotune.py from
// measurements on the GPU, replaces the defaults below when present.
#pragma once

namespace bgemm {

struct TileCost {
  float a_ns;  // fixed cost per tile (prologue, epilogue, latency)
  float b_ns;  // cost per unit of K
};

// Tensor-core cost tables are indexed [mode - 1][cfg]: TF32, TF32X3, BF16X3;
// cfg 0..7 one-SM tiles, 8..15 CTA-pair tiles.  b = 0 marks a configuration
// the mode does not run.
#if defined(BGEMM_HAVE_TUNED_TABLE)
#include "tile_table_tuned.inc"
#else
// Defaults from a first-principles model.  SIMT: 2 CTAs per SM share 128
// FP32 lanes at ~1.9 GHz, b = BM*BN / (64 lanes * 1.9 GHz) / efficiency.
constexpr TileCost kSimtCost[10] = {
    {1500.f, 16 * 16 / 64 / 1.9f / 0.20f},    {1600.f, 32 * 32 / 64 / 1.9f / 0.45f},
    {1700.f, 64 * 32 / 64 / 1.9f / 0.60f},    {1700.f, 32 * 64 / 64 / 1.9f / 0.60f},
    {1800.f, 64 * 64 / 64 / 1.9f / 0.70f},    {2000.f, 128 * 64 / 64 / 1.9f / 0.80f},
    {2000.f, 64 * 128 / 64 / 1.9f / 0.80f},   {2200.f, 128 * 128 / 64 / 1.9f / 0.85f},
    {1600.f, 8 * 128 / 64 / 1.9f / 0.45f},    {1600.f, 128 * 8 / 64 / 1.9f / 0.45f},
};
// Tensor cores: per 128-byte K slice a tile streams its operands from L2,
// which bounds the narrow tiles, so a tile costs at least what a 128-wide
// (one SM) or 256-wide (pair) tile costs for the same K.  TF32 runs 4096
// flops/clk/SM (BF16 8192) at ~1.9 GHz.
#define BGEMM_TC1(bn, prod, rate) {1500.f, 2.f * 128 * ((bn) > 128 ? (bn) : 128) * (prod) / (rate)}
#define BGEMM_TC2(bn, prod, rate) {2500.f, 2.f * 256 * (0.6f * 256 + 0.4f * (bn)) * (prod) / (2 * (rate))}
#define BGEMM_TC_ROW(prod, rate, pairs)                                                          \
  {BGEMM_TC1(16, prod, rate), BGEMM_TC1(32, prod, rate), BGEMM_TC1(64, prod, rate),             \
   BGEMM_TC1(128, prod, rate), BGEMM_TC1(16, prod, rate), BGEMM_TC1(32, prod, rate),            \
   BGEMM_TC1(64, prod, rate), BGEMM_TC1(128, prod, rate),                                        \
   pairs ? TileCost BGEMM_TC2(64, prod, rate) : TileCost{0.f, 0.f},                              \
   pairs ? TileCost BGEMM_TC2(128, prod, rate) : TileCost{0.f, 0.f},                             \
   pairs ? TileCost BGEMM_TC2(256, prod, rate) : TileCost{0.f, 0.f}, TileCost{0.f, 0.f},         \
   pairs ? TileCost BGEMM_TC2(64, prod, rate) : TileCost{0.f, 0.f},                              \
   pairs ? TileCost BGEMM_TC2(128, prod, rate) : TileCost{0.f, 0.f},                             \
   pairs ? TileCost BGEMM_TC2(256, prod, rate) : TileCost{0.f, 0.f}, TileCost{0.f, 0.f}}
constexpr TileCost kTcCost[3][16] = {
    BGEMM_TC_ROW(1, 7782.f, false),
    BGEMM_TC_ROW(3, 7782.f, true),
    BGEMM_TC_ROW(3, 15564.f, true),
};
#undef BGEMM_TC_ROW
#undef BGEMM_TC2
#undef BGEMM_TC1
#endif

// Promotion schedule of the split tensor-core modes on CTA pairs, indexed
// [mode - 1][bucket of K] (see TcSchedule in tc_common.h): 128-byte K slices
// per promotion group, 0 = promote every MMA of K and keep lo*lo.  The
// single-product TF32 row is unused.  Defaults: the small-K path up to
// K = 64, groups of two slices above; the autotuner replaces them with the
// fastest groups whose error against FP64 stays within the FP32 SIMT path's.
#if !defined(BGEMM_TUNED_HAS_SCHEDULE)
constexpr unsigned char kTcGroupTable[3][8] = {
    {0, 2, 2, 2, 2, 2, 2, 2}, {0, 2, 2, 2, 2, 2, 2, 2}, {0, 2, 2, 2, 2, 2, 2, 2}};
#endif

// Compile-time schedule parameters, swept by the autotuner with a rebuild per
// candidate:
//   kSimtRingCap      cp.async ring stages of a SIMT tile: a tile takes as
//                     many 16-k stages as the CTA's shared memory holds, up
//                     to this cap (the 128 x 128 tile always has 4);
//   kTcCPrefetchLead  beta != 0: promotion groups before the end of a pair
//                     tile at which its C lines are prefetched into L2 (0:
//                     none; the epilogue's pipelined reads then go to HBM).
#if !defined(BGEMM_TUNED_HAS_BUILD_PARAMS)
constexpr int kSimtRingCap = 4;
constexpr int kTcCPrefetchLead = 0;
#endif

}  // namespace bgemm
