// tile_table.h -- per-tile cost model consumed by the planner.
//
// Time of one work item of configuration c on a matrix with inner dimension
// K is modelled as  t = a_c + b_c * K  (nanoseconds, one CTA, with the CTAs
// that share its SM busy too).  The planner picks, per matrix, the
// configuration with the least total time and then splits the largest tiles
// until no single tile is longer than the average load of one persistent
// CTA (the parallelism rebalance).  tile_table_tuned.inc, written by
// batchgemm_gb300/autotune.py from measurements on the GPU, overrides the
// defaults below when present.
#pragma once

namespace bgemm {

struct TileCost {
  float a_ns;  // fixed cost per tile (prologue, epilogue, latency)
  float b_ns;  // cost per unit of K
};

#if defined(BGEMM_HAVE_TUNED_TABLE)
#include "tile_table_tuned.inc"
#else
// Defaults from a first-principles model: 2 CTAs per SM share 128 FP32
// lanes at ~1.9 GHz, b = BM*BN / (64 lanes * 1.9 GHz) / efficiency.
constexpr TileCost kSimtCost[8] = {
    {1500.f, 16 * 16 / 64 / 1.9f / 0.20f},    {1600.f, 32 * 32 / 64 / 1.9f / 0.45f},
    {1700.f, 64 * 32 / 64 / 1.9f / 0.60f},    {1700.f, 32 * 64 / 64 / 1.9f / 0.60f},
    {1800.f, 64 * 64 / 64 / 1.9f / 0.70f},    {2000.f, 128 * 64 / 64 / 1.9f / 0.80f},
    {2000.f, 64 * 128 / 64 / 1.9f / 0.80f},   {2200.f, 128 * 128 / 64 / 1.9f / 0.85f},
};
#endif

}  // namespace bgemm
