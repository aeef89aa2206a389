/*
 * bgemm.h -- variable-size batched SGEMM for NVIDIA GB300 (sm_103a).
 *
 * C ABI of libbgemm_gb300.so.  Every matrix is column-major:
 *     C_i <- alpha * A_i * B_i + beta * C_i,   i = 0 .. batch-1
 * A_i is M_i x K_i (element (m,k) at A_i[m + k*lda_i]), B_i is K_i x N_i
 * ((k,n) at B_i[k + n*ldb_i]), C_i is M_i x N_i ((m,n) at C_i[m + n*ldc_i]).
 *
 * Reference interface replaced (paths inside the BatchGEMM project):
 *   - the framework kernel entry
 *       __global__ void gemm(int M[], int N[], int K[], float *A[], float *B[],
 *                            float *C[], int T_strategy[])
 *     (CUDA/framework/kernel.h:11), which computes C_i += A_i*B_i over device
 *     arrays of sizes and pointers, and
 *   - the host driver that reads the per-matrix sizes, picks a tile strategy
 *     per matrix, uploads the descriptors and launches one kernel for the
 *     whole batch (CUDA/framework/gemm.cu:31-77, 88-174, 181-209).
 * Generalised to the magma-style "vbatched" contract: per-matrix leading
 * dimensions, alpha/beta, a stream, and status codes instead of exit().
 *
 * Numerics of BGEMM_MODE_SIMT_FP32 (bit-exact contract): every output element
 * is one FP32 fma chain over k = 0..K-1 in order.  When alpha == 1 and
 * beta == 1 the chain starts from the old C value, exactly like the
 * reference's tile bodies (C += A*B); otherwise it starts from 0 and the
 * result is alpha*acc (beta == 0, C is then never read) or
 * fmaf(alpha, acc, beta*C).
 *
 * The tensor-core modes run on tcgen05 with FP32 accumulation in tensor
 * memory: TF32 (one product of TF32-rounded operands), TF32X3 (hi*hi +
 * hi*lo + lo*hi of a TF32 hi/lo split) and BF16X3 (the same with a bfloat16
 * split).  They are checked against an FP64 oracle with a sqrt(K)-scaled
 * relative tolerance.
 *
 * Ownership: the caller owns every A/B/C buffer and the device arrays of
 * device pointers dA/dB/dC; the library owns its plans, their device
 * descriptors and workspace.  All device work is asynchronous on `stream`.
 * A plan may be executed on one stream at a time (its tile queue counter is
 * reset by the kernel itself at the end of each launch).
 */
#ifndef BGEMM_GB300_H
#define BGEMM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same type as cudaStream_t; NULL is the legacy default stream. */
typedef struct CUstream_st* bgemm_stream_t;

typedef enum bgemm_status {
  BGEMM_SUCCESS = 0,
  BGEMM_ERROR_INVALID_VALUE = 1,  /* bgemm_last_error_arg() gives the argument */
  BGEMM_ERROR_NOT_SUPPORTED = 2,  /* no sm_103 device, or a size beyond a limit */
  BGEMM_ERROR_ALLOC = 3,          /* device or pinned host allocation failed */
  BGEMM_ERROR_CUDA = 4,           /* a CUDA runtime call failed */
  BGEMM_ERROR_DEVICE_TIMEOUT = 5, /* a bounded device-side wait expired; the
                                     kernel returned early, results invalid */
  BGEMM_ERROR_INTERNAL = 6
} bgemm_status_t;

typedef enum bgemm_mode {
  BGEMM_MODE_SIMT_FP32 = 0, /* FP32 SIMT fma, bit-exact with the reference chain */
  BGEMM_MODE_TF32 = 1,      /* tcgen05 kind::tf32, one product            */
  BGEMM_MODE_TF32X3 = 2,    /* tcgen05 kind::tf32, 3-product split (hi/lo) */
  BGEMM_MODE_BF16X3 = 3     /* tcgen05 kind::f16 (bf16), 3-product split    */
} bgemm_mode_t;

/* Storage order of every matrix of a call and per-operand transposition
 * (BLAS / magma vbatched convention: C = alpha * op(A) * op(B) + beta * C,
 * op(A) is M x K, op(B) is K x N).  Column-major: A (N) is M x K with
 * lda >= M, A (T) is stored K x M with lda >= K; B (N) is K x N with
 * ldb >= K, B (T) is stored N x K with ldb >= N; ldc >= M.  Row-major: the
 * same matrices stored by rows, so lda >= K (A N) or M (A T), ldb >= N (B N)
 * or K (B T), ldc >= N. */
typedef enum bgemm_layout { BGEMM_COL_MAJOR = 0, BGEMM_ROW_MAJOR = 1 } bgemm_layout_t;
typedef enum bgemm_op { BGEMM_OP_N = 0, BGEMM_OP_T = 1 } bgemm_op_t;

typedef struct bgemm_plan_s* bgemm_plan_t;

/* Per-plan facts (for benchmarks and tests). */
typedef struct bgemm_plan_info {
  int batch;
  int mode;
  int num_tiles;            /* work items in the largest-first tile queue   */
  int grid;                 /* persistent CTAs launched per execute          */
  int tile_config_hist[16]; /* matrices per tile configuration               */
  double useful_flops;      /* sum 2*M*N*K                                    */
  double min_bytes;         /* compulsory HBM bytes: 4*(MK + KN + MN(1 + [beta!=0])) at beta=0 */
  size_t device_bytes;      /* descriptors + queue + workspace owned by the plan */
  size_t workspace_bytes;   /* split-operand workspace (tensor-core modes)   */
  int kernels_per_execute;  /* kernel launches one bgemm_plan_execute makes  */
  int reserved[7];
} bgemm_plan_info_t;

/* Device sizes a batch needs inside a plan; bgemm_plan_requirements computes
 * them, and bgemm_plan_options_t.capacity reserves them so that the plan can
 * later take other batches through bgemm_plan_update. */
typedef struct bgemm_plan_requirements {
  int batch;               /* matrices                                       */
  int tiles;               /* work items of the largest-first tile queue     */
  int pack_jobs;           /* split/pack pre-pass jobs (tensor-core modes)   */
  int kernel_family;       /* 0 SIMT, 1 one-SM tcgen05 tiles, 2 CTA-pair tiles */
  size_t workspace_bytes;  /* split-operand workspace (tensor-core modes)    */
  int simt_tiles;          /* mixed plans (options.simt_below): tiles of the
                              matrices that run on the FP32 SIMT kernel      */
  int reserved[3];
} bgemm_plan_requirements_t;

/* Options for bgemm_plan_create_ex (zero-initialise, then set fields). */
typedef struct bgemm_plan_options {
  int force_tile_config;    /* -1: heuristic; otherwise a config id of the mode */
  int max_ctas;             /* 0: one wave of persistent CTAs; otherwise a cap  */
  int disable_rebalance;    /* 1: skip the parallelism (wavefront) rebalance    */
  int host_tensor_maps;     /* 1: encode the TMA tensor maps on the host instead
                               of building them on the device (for comparison) */
  int kernel_family;        /* split tensor-core modes: 0 chosen by the cost
                               model, 1 one-SM tiles, 2 CTA-pair tiles        */
  int layout;               /* bgemm_layout_t of every matrix (0: column-major) */
  int trans_a;              /* bgemm_op_t applied to every A (0: N)          */
  int trans_b;              /* bgemm_op_t applied to every B (0: N)          */
  int simt_below;           /* tensor-core modes: matrices with min(M, N, K)
                               below this run on the FP32 SIMT kernel in the
                               same execute, the rest on the tensor cores
                               (0: all on the tensor cores).  Thin and short
                               matrices are memory-bound, and the SIMT kernel
                               reads 4 B per operand element where the split
                               path moves ~20 B; their results are the FP32
                               chain's, so the batch's error cannot exceed
                               the all-SIMT path's where the tensor-core
                               matrices beat it.  Two GEMM kernels per execute
                               instead of one. */
  int reserved[2];          /* must be zero                                  */
  /* Capacity for bgemm_plan_update: each field is raised to the creating
   * batch's own requirement, so all-zero means "this batch only".
   * kernel_family is ignored here (see the field above). */
  bgemm_plan_requirements_t capacity;
} bgemm_plan_options_t;

/* --- one-shot entry (host size arrays, like CUDA/framework/gemm.cu:39-41) ---
 * M, N, K, lda, ldb, ldc: HOST arrays [batch]; dA, dB, dC: DEVICE arrays
 * [batch] of device pointers.  Requirements: M,N,K >= 0, lda >= max(1,M),
 * ldb >= max(1,K), ldc >= max(1,M); pointers of empty matrices are not read.
 * Plans are cached per shape multiset (device, mode and orientation, and
 * the batch's (M, N, K, lda, ldb, ldc) tuples in any order -- the
 * counterpart of the reference's offline shape sort, ROCm/data/sort.cpp:
 * 17-60): the same shapes in another order re-plan into the cached plan
 * (host planning + one upload, no allocation) and give bit-identical
 * results per matrix.  A cached plan used on another stream first waits
 * for its previous use.  A cache miss builds and uploads a plan on `stream`
 * without blocking on the GPU; it first evicts least recently used plans
 * so that the cached device bytes stay under the limit of
 * bgemm_plan_cache_set_limit, and on an allocation failure it evicts every
 * other plan of the device and retries once.  Plans created or used while
 * `stream` is capturing are never evicted or re-planned (a graph may replay
 * them). */
bgemm_status_t bgemm_sgemm_vbatched(const int* M, const int* N, const int* K,
                                    float alpha, const float* const* dA,
                                    const int* lda, const float* const* dB,
                                    const int* ldb, float beta,
                                    float* const* dC, const int* ldc,
                                    int batch, bgemm_mode_t mode,
                                    bgemm_stream_t stream);

/* Same as bgemm_sgemm_vbatched with a storage order and op(A), op(B) (see
 * bgemm_layout_t).  The FP32 SIMT mode stays one fma chain per element over
 * k in order, so the result is bit-identical to the column-major NN call on
 * the materialised op(A), op(B).  Row-major calls run as the column-major
 * product C^T = op(B)^T op(A)^T on the same memory (no copies).  Argument
 * numbers: layout 1, transA 2, transB 3, M 4, N 5, K 6, alpha 7, dA 8,
 * lda 9, dB 10, ldb 11, beta 12, dC 13, ldc 14, batch 15, mode 16. */
bgemm_status_t bgemm_sgemm_vbatched_ex(bgemm_layout_t layout, bgemm_op_t transA,
                                       bgemm_op_t transB, const int* M,
                                       const int* N, const int* K, float alpha,
                                       const float* const* dA, const int* lda,
                                       const float* const* dB, const int* ldb,
                                       float beta, float* const* dC,
                                       const int* ldc, int batch,
                                       bgemm_mode_t mode, bgemm_stream_t stream);

/* --- plan / execute split (execute allocates nothing: capturable) --------- */
bgemm_status_t bgemm_plan_create(bgemm_plan_t* plan, const int* M,
                                 const int* N, const int* K, const int* lda,
                                 const int* ldb, const int* ldc, int batch,
                                 bgemm_mode_t mode, bgemm_stream_t stream);
bgemm_status_t bgemm_plan_create_ex(bgemm_plan_t* plan, const int* M,
                                    const int* N, const int* K,
                                    const int* lda, const int* ldb,
                                    const int* ldc, int batch,
                                    bgemm_mode_t mode, bgemm_stream_t stream,
                                    const bgemm_plan_options_t* options);
bgemm_status_t bgemm_plan_execute(bgemm_plan_t plan, float alpha,
                                  const float* const* dA,
                                  const float* const* dB, float beta,
                                  float* const* dC, bgemm_stream_t stream);
bgemm_status_t bgemm_plan_info(bgemm_plan_t plan, bgemm_plan_info_t* info);

/* --- batch streams: re-plan into an existing plan ------------------------
 * No counterpart in the reference, whose driver plans, uploads and launches
 * one batch per process run (CUDA/framework/gemm.cu:31-209).
 *
 * bgemm_plan_requirements: host-only planning of a batch (the same tile
 * choice, queue and pre-pass layout as bgemm_plan_create_ex with these
 * options) that reports the device sizes it needs; nothing is allocated and
 * no GPU work is issued.  The element-wise maximum over the batches of a
 * stream, passed as options->capacity, sizes a plan that can take each of
 * them.
 *
 * bgemm_plan_update: plans a new batch (same mode, kernel family and
 * options as at creation) into the plan's existing device buffers and
 * uploads its descriptors, tile queue, pre-pass jobs and tensor maps on
 * `stream`.  Device addresses, kernels and launch shapes stay the same, so a
 * CUDA graph that captured bgemm_plan_execute stays valid and computes the
 * new batch on its next launch (A/B/C pointer arrays are the caller's: put
 * the new batch's pointers where the graph reads them).  The update is
 * stream-ordered: executes enqueued on `stream` before it see the previous
 * batch, later ones the new batch; work on other streams must be ordered by
 * the caller.  Host staging is a ring of three pinned buffers, so the call
 * blocks only until the upload of the third update back has been consumed
 * by the GPU; it must not be called while `stream` is capturing.  A batch beyond the
 * plan's capacity fails with BGEMM_ERROR_NOT_SUPPORTED and leaves the plan
 * holding its previous batch. */
bgemm_status_t bgemm_plan_requirements(const int* M, const int* N, const int* K,
                                       const int* lda, const int* ldb,
                                       const int* ldc, int batch,
                                       bgemm_mode_t mode,
                                       const bgemm_plan_options_t* options,
                                       bgemm_plan_requirements_t* out);
bgemm_status_t bgemm_plan_update(bgemm_plan_t plan, const int* M, const int* N,
                                 const int* K, const int* lda, const int* ldb,
                                 const int* ldc, int batch,
                                 bgemm_stream_t stream);
/* Capacity the plan was created with (what bgemm_plan_update accepts). */
bgemm_status_t bgemm_plan_capacity(bgemm_plan_t plan,
                                   bgemm_plan_requirements_t* out);
/* Profiling hook (no counterpart in the reference, which brackets its whole
 * launch loop with events, CUDA/framework/gemm.cu:203-214): every following
 * bgemm_plan_execute records ev_start / ev_stop (cudaEvent_t; either may be
 * NULL) on its stream immediately before and after the plan's GEMM kernel,
 * so the kernel's own duration can be read with cudaEventElapsedTime.
 * Pass NULL, NULL to stop. */
bgemm_status_t bgemm_plan_set_kernel_events(bgemm_plan_t plan, void* ev_start,
                                            void* ev_stop);
/* Profiling hook of the tensor-core modes (no reference counterpart): every
 * following bgemm_plan_execute makes each persistent CTA of the GEMM kernel
 * write the device's global timer (ns) when it starts and when it finishes,
 * to d_times[2*cta] and d_times[2*cta + 1] (a device array of 2 x
 * bgemm_plan_info_t.grid unsigned 64-bit ints), so the spread of finish
 * times -- the load imbalance of the static tile schedule -- can be read.
 * Pass NULL to stop.  BGEMM_ERROR_NOT_SUPPORTED for FP32 SIMT plans. */
bgemm_status_t bgemm_plan_set_cta_timer(bgemm_plan_t plan, void* d_times);
/* Blocks until the plan's previous launches on `stream` finish and reports
 * BGEMM_ERROR_DEVICE_TIMEOUT if a device-side wait expired in any of them
 * (the flag is then cleared). */
bgemm_status_t bgemm_plan_check_device(bgemm_plan_t plan, bgemm_stream_t stream);
bgemm_status_t bgemm_plan_destroy(bgemm_plan_t plan);

/* --- reference drop-in: the framework kernel's own argument list ----------
 * Device arrays dM, dN, dK [batch] and dA, dB, dC [batch] exactly as the
 * reference passes them to gemm<<<...>>>(M, N, K, A, B, C, T_strategy)
 * (CUDA/framework/gemm.cu:200, kernel.h:11); computes C_i += A_i*B_i with
 * lda = M_i, ldb = K_i, ldc = M_i in FP32 SIMT (the reference's in-place
 * fma chain, bit-exact).  dT (the reference's per-matrix tile strategy) may
 * be NULL; it is ignored because this library picks tiles itself.  Sizes
 * never leave the device: a device-side pass builds the tile queue, so the
 * call needs no host copy of M/N/K.  max_dim bounds every M_i and N_i (the
 * queue capacity is sized from it); M_i or N_i above it is an error reported
 * by bgemm_framework_check_device(). */
bgemm_status_t bgemm_framework_gemm(const int* dM, const int* dN,
                                    const int* dK, float* const* dA,
                                    float* const* dB, float* const* dC,
                                    const int* dT, int batch, int max_dim,
                                    bgemm_stream_t stream);
bgemm_status_t bgemm_framework_check_device(bgemm_stream_t stream);

/* --- the same entry in any mode ------------------------------------------
 * No counterpart in the reference (its kernel is FP32 only).  Same arguments
 * and result as bgemm_framework_gemm (device arrays of sizes and pointers,
 * C_i += A_i*B_i, lda = M_i, ldb = K_i, ldc = M_i), in any bgemm_mode_t.  For
 * the tensor-core modes the tile choice (CTA-pair tiles, the autotuned cost
 * table), the tile queue, the split-operand layout, the pre-pass strips and
 * the tensor maps are all built on the device, so the sizes never leave it
 * and a captured sequence of calls replays with whatever the size arrays
 * hold.  max_dim bounds every M_i and N_i, max_k every K_i, and
 * max_operand_elems the batch's sum of (M_i + N_i) * K_i (0: batch * 2 *
 * max_dim * max_k); the library's scratch is sized from them (the split
 * operands take 8 bytes per operand element for TF32X3, 4 for TF32 and
 * BF16X3).  A matrix outside max_dim / max_k is skipped, a batch above
 * max_operand_elems is not computed; bgemm_framework_check_device reports
 * both, and an expired device wait (BGEMM_ERROR_DEVICE_TIMEOUT).  Calls in
 * one mode on one device share that scratch, so order them (one stream, or
 * events between streams); a call that grows it (the first, or larger
 * bounds) allocates and must not be inside a stream capture.
 * BGEMM_MODE_SIMT_FP32 is exactly bgemm_framework_gemm (max_k and
 * max_operand_elems unused).  Argument numbers: dM 1, dN 2, dK 3, dA 4,
 * dB 5, dC 6, batch 7, max_dim 8, max_k 9, max_operand_elems 10, mode 11. */
bgemm_status_t bgemm_framework_gemm_mode(const int* dM, const int* dN,
                                         const int* dK, float* const* dA,
                                         float* const* dB, float* const* dC,
                                         int batch, int max_dim, int max_k,
                                         long long max_operand_elems,
                                         bgemm_mode_t mode, bgemm_stream_t stream);

/* Frees the scratch that bgemm_framework_gemm and bgemm_framework_gemm_mode
 * keep on the current device (it is allocated again, at the size the next
 * call needs).  Waits for the device; errors not yet collected by
 * bgemm_framework_check_device are dropped.  No reference counterpart. */
bgemm_status_t bgemm_framework_release(void);

/* --- allocation-free variant of bgemm_framework_gemm ----------------------
 * No counterpart in the reference.  Same arguments and result as
 * bgemm_framework_gemm (device size arrays, C_i += A_i*B_i, FP32 SIMT,
 * bit-exact), for callers that cannot allocate device memory while they
 * run: a real-time or latency-bound loop where an allocation (which can
 * synchronise the whole device) is not allowed, or a plug-in whose host
 * application owns the device memory budget through its own pool and
 * forbids allocations behind its back.  The tile queue lives in a fixed
 * __device__ array inside the library (about 2.2 MB per device, held until
 * the process exits) instead of library-allocated memory, so the call never
 * calls cudaMalloc, cudaFree or any allocating routine.  Limits:
 * batch <= 4096 and batch * ceil(max_dim/16)^2 <= 262144; larger calls
 * return BGEMM_ERROR_NOT_SUPPORTED before any work is issued.  d_info
 * (device int, may be NULL) receives bit 0 when a matrix size was negative
 * or above max_dim (that matrix is skipped); the caller clears it.  With
 * d_info == NULL such a matrix is skipped silently: nothing reports it.
 * Set-up: the first call on a device looks up the array's device address
 * and uploads the planner's small cost tables to that device (a
 * synchronous copy); make that first call before any stream capture.
 * All calls share the array and it keeps the last call's contents (each
 * call clears the counters it needs): calls that overlap on the GPU race
 * and must be ordered by the caller. */
bgemm_status_t bgemm_framework_gemm_noalloc(const int* dM, const int* dN,
                                            const int* dK, float* const* dA,
                                            float* const* dB, float* const* dC,
                                            int batch, int max_dim, int* d_info,
                                            bgemm_stream_t stream);

/* --- the one-shot entries' plan cache -------------------------------------
 * No counterpart in the reference.  bgemm_plan_cache_set_limit sets the
 * device bytes (per device) the cached plans of bgemm_sgemm_vbatched[_ex]
 * may hold (0: the default, a third of the device's memory) and evicts down
 * to it; bgemm_plan_cache_clear frees every evictable cached plan of the
 * current device (waits for the device). */
bgemm_status_t bgemm_plan_cache_set_limit(size_t bytes);
bgemm_status_t bgemm_plan_cache_clear(void);

/* --- errors and device facts --------------------------------------------- */
/* 1-based position of the first invalid argument of the last failing call on
 * this host thread (BLAS convention), 0 if none; for per-matrix arrays the
 * offending matrix index is returned through *matrix (may be NULL). */
int bgemm_last_error_arg(int* matrix);
const char* bgemm_last_error_message(void);
const char* bgemm_status_string(bgemm_status_t status);
/* Number of SMs of the current device and persistent CTAs per SM per mode. */
bgemm_status_t bgemm_device_info(int* num_sms, int* simt_ctas_per_sm,
                                 int* tc_ctas_per_sm);
/* Library version, e.g. 100 for 0.1.0. */
int bgemm_version(void);

#ifdef __cplusplus
}
#endif
#endif /* BGEMM_GB300_H */
