/*
 * bgemm_debug.h -- host-only introspection of libbgemm_gb300.so's planner,
 * for tests and the autotuner.  Needs no GPU.
 *
 * Replaces the reference's host tile-strategy pass (CUDA/framework/gemm.cu:
 * 107-169, the per-matrix T_strategy choice and the wavefront demotion loop)
 * as an observable function: given the sizes and the number of persistent
 * CTA slots, it returns each matrix's tile configuration and the ordered
 * tile queue the SIMT kernel would pull.
 */
#ifndef BGEMM_GB300_DEBUG_H
#define BGEMM_GB300_DEBUG_H

#ifdef __cplusplus
extern "C" {
#endif

/* cfg_out [batch] receives the SIMT tile configuration of each matrix (-1 for
 * empty matrices); items_out [3*max_items] receives (matrix, tile_m, tile_n)
 * per queue slot in pull order (may be NULL to only count).  force_cfg < 0
 * lets the heuristic choose; rebalance != 0 enables the parallelism
 * rebalance for `slots` persistent CTAs.  Returns the number of work items,
 * or -1 on invalid sizes or when max_items is too small. */
int bgemm_debug_simt_queue(const int* M, const int* N, const int* K, int batch, int slots,
                           int force_cfg, int rebalance, int* cfg_out, int* items_out,
                           int max_items);

/* Host-only replay of the tensor-core planner for `mode` (1 TF32, 2 TF32X3,
 * 3 BF16X3) as it would plan on a device with `slots` one-SM persistent CTAs
 * and `clusters` CTA pairs (family: 0 cost model, 1 one-SM tiles, 2 CTA
 * pairs).  Every output may be NULL.  cfg_out[batch]: tile configuration
 * (bit 8 set when the operands are swapped, -1 for empty matrices);
 * items_out[3*max_items]: (matrix, tile along the MMA's M side, tile along
 * its N side) in queue order; ws_out[5*batch]: byte offsets of the packed
 * A hi, A lo, B hi, B lo panels and the padded row length kpad (elements);
 * jobs_out[3*max_jobs]: pre-pass strips (matrix, operand 0 A / 1 B, first
 * row).  *n_jobs, *ws_bytes and *kernel_family (1 one-SM, 2 pairs) are
 * always written.  Returns the number of work items, or -1 on invalid sizes,
 * planner errors, or max_items too small. */
int bgemm_debug_tc_plan(const int* M, const int* N, const int* K, int batch, int mode,
                        int family, int slots, int clusters, int* cfg_out, int* items_out,
                        int max_items, long long* ws_out, int* jobs_out, int max_jobs,
                        int* n_jobs, long long* ws_bytes, int* kernel_family);

/* Host replay of the planner that bgemm_framework_gemm runs on the device
 * (same per-matrix SIMT tile choice, parallelism rebalance rounds for
 * `slots` persistent CTAs, and bins, reserved in matrix order).
 * cfg_out[batch]: tile configuration (-1: no output); items_out
 * [3*max_items]: (matrix, tile along M, tile along N) in queue order; *err:
 * bit 0 when a size is negative or above max_dim.  Returns the number of work
 * items, or -1 on invalid arguments or too small output arrays. */
int bgemm_debug_framework_plan(const int* M, const int* N, const int* K, int batch, int max_dim,
                               int slots, int* cfg_out, int* items_out, int max_items, int* err);

/* Host replay of the planner that bgemm_framework_gemm_mode runs on the
 * device (same per-matrix tile choice, bins and reservations, made in matrix
 * order instead of by atomics).  items_out[3*max_items]: (matrix, tile along
 * the MMA's M side, tile along its N side) in queue order; jobs_out
 * [3*max_jobs]: pre-pass strips (matrix, operand, first row); ws_out[5*batch]:
 * A hi, A lo, B hi, B lo byte offsets and kpad.  *n_jobs, *ws_used (bytes of
 * split operands), *ws_capacity (the scratch the entry sizes from its bounds)
 * and *err (the device error bits: 1 size out of bounds, 2 workspace too
 * small, 4 no costed configuration) are always written; cfg_out[batch] (may
 * be NULL) receives each matrix's CTA-pair configuration (-1: no tiles).
 * Returns the number of work items, or -1 on invalid arguments or too small
 * output arrays. */
int bgemm_debug_framework_tc_plan(const int* M, const int* N, const int* K, int batch,
                                  int max_dim, int max_k, long long max_operand_elems, int mode,
                                  int* items_out, int max_items, int* jobs_out, int max_jobs,
                                  long long* ws_out, int* n_jobs, long long* ws_used,
                                  long long* ws_capacity, int* err, int* cfg_out);

/* Cost-model entry of configuration `cfg` of `mode` (0 SIMT, 1 TF32,
 * 2 TF32X3, 3 BF16X3): modelled time of one tile = *a_ns + *b_ns * K
 * nanoseconds, as the device planners read it.  Returns 0, or -1 for an
 * invalid mode or configuration. */
int bgemm_debug_tile_cost(int mode, int cfg, float* a_ns, float* b_ns);

/* The compile-time schedule parameters the library was built with (from the
 * autotuned table): *simt_ring_cap = the most cp.async ring stages of a SIMT
 * tile, *c_prefetch_lead = promotion groups before the end of a CTA-pair
 * tile at which its C is prefetched when beta != 0.  Returns 0, or -1 for a
 * NULL argument. */
int bgemm_debug_build_params(int* simt_ring_cap, int* c_prefetch_lead);

/* HBM streaming probe (no counterpart in the reference): launches one
 * grid-stride float4 kernel of `grid` CTAs x 256 threads on `stream` over n4
 * float4 words per buffer.  kind 0 reads x and writes y1 and y2 (one read,
 * two writes: the split pre-pass's mix), 1 copies x to y1, 2 writes y1,
 * 3 reads x (y1 is a sink).  The caller times it; batchgemm_gb300.peaks
 * reports the ceilings.  Returns 0, or -1 for invalid arguments (a NULL or
 * non-16-byte-aligned buffer the kind needs) or a failed launch. */
int bgemm_debug_hbm_probe(int kind, const float* x, float* y1, float* y2, long long n4, int grid,
                          void* stream);

/* Tensor-core plans: waits for `stream`, encodes on the host the tensor maps
 * that the device built for the plan, and compares them byte by byte.
 * *n_maps receives the number of maps compared, *n_diff how many differ,
 * *first_byte the first differing byte of the first differing map (-1 if
 * none).  Returns 0, or -1 for a non-tensor-core plan. */
int bgemm_debug_compare_tensor_maps(void* plan, void* stream, int* n_maps, int* n_diff,
                                    int* first_byte);

/* Self-test of the bounded device-side wait used by every tensor-core
 * kernel (no counterpart in the reference, whose kernels have no device
 * waits): one CTA waits on an mbarrier that nothing arrives on.  The wait
 * must expire after limit_ns, set the error flag and let the kernel return,
 * leaving the context usable.  *error receives the device error word (1
 * expected), *returned 1 if the waiting thread got past the wait, *wait_ok
 * the wait's result (0 expected).  Synchronises the device; returns 0, or -1
 * if a CUDA call failed. */
int bgemm_debug_bounded_wait_selftest(unsigned long long limit_ns, int* error, int* returned,
                                      int* wait_ok);

/* Promotion schedule of the split tensor-core modes on CTA pairs (mode 2
 * TF32X3, 3 BF16X3; 1 is accepted and unused): group[b] for the 8 buckets
 * of K (K <= 64, then (64,128], (128,256], ..., (2048,4096], > 4096) is the
 * number of 128-byte K slices accumulated in tensor memory before the
 * epilogue promotes them into FP32 registers, 0 = promote every MMA and keep
 * the lo*lo product.  bgemm_debug_set_tc_schedule overrides the autotuned
 * table for every later launch in the process (NULL restores it; values
 * above 64 are rejected); bgemm_debug_get_tc_schedule reads the schedule in
 * use.  For the autotuner.  Return 0, or -1 on invalid arguments. */
int bgemm_debug_set_tc_schedule(int mode, const int* group);
int bgemm_debug_get_tc_schedule(int mode, int* group);

/* Counters of the one-shot entries' plan cache on the current device:
 * entries and device bytes held, and since the process started: calls that
 * found their exact batch (hits), calls that re-planned a cached plan for
 * the same shapes in another order (reorders), plans built (misses), plans
 * freed to make room (evictions); *limit is the byte limit (0 until first
 * set or used).  Every pointer may be NULL.  Returns 0. */
int bgemm_debug_plan_cache_stats(long long* entries, long long* bytes, long long* hits,
                                 long long* reorders, long long* misses, long long* evictions,
                                 long long* limit);

#ifdef __cplusplus
}
#endif
#endif
