// plan_internal.h -- the plan object and the hooks of the tensor-core modes.
#pragma once
#include <vector>

#include "bgemm.h"
#include "bgemm_internal.h"

namespace bgemm {

struct DeviceFacts {
  int device;
  int cc;
  int num_sms;
  int simt_ctas_per_sm;
  int tc_ctas_per_sm;
};

// Tile choice of one matrix.
struct MatPlan {
  int cfg;         // -1: matrix has no output (M or N is 0)
  long long tiles;
  double t_tile;   // modelled time of one tile, ns
};
struct TcPlan;

// MatDesc::aux bit of the tensor-core modes: the matrix runs with A and B
// swapped (C^T = B^T A^T), so the MMA's M dimension walks N.
constexpr int kTcSwapFlag = 1 << 30;
// ids 0..7: one-SM tiles; ids 8..15: CTA-pair tiles (split modes)
constexpr int kTcNumCfgs = 16;

// The plan's device header (256 bytes, ints): [0] queue head and [1] CTAs
// finished (reset by the kernels themselves), [kHdrItems] work items of the
// current batch, [kHdrJobs] pre-pass jobs of the current batch.  Kernels read
// the counts from here, so a captured launch serves every batch an update
// uploads.
constexpr int kHdrItems = 16;
constexpr int kHdrJobs = 17;
constexpr size_t kHdrBytes = 256;
// Pinned staging buffers of a plan's uploads, used in turn: an update waits
// only for the upload kStageBufs updates back to have been consumed.
constexpr int kStageBufs = 3;

// Host result of planning one batch, before anything is written to the
// plan's buffers (an update that does not fit leaves the plan untouched).
struct BatchPlan {
  int batch = 0;
  std::vector<MatDesc> descs;
  std::vector<TileItem> items;
  int hist[16] = {};
  double flops = 0, bytes = 0;
  bgemm_plan_requirements_t req{};
};

}  // namespace bgemm

struct bgemm_plan_s {
  int batch = 0;
  int mode = 0;
  int n_items = 0;
  int grid = 0;
  bgemm::DeviceFacts facts{};
  bgemm_plan_options_t opt{};      // options of creation, reused by updates
  bgemm_plan_requirements_t cap{}; // capacity of the device buffers
  // Row-major plans run the column-major product C^T = op(B)^T op(A)^T:
  // their shapes are planned as (N, M, K, ldb, lda, ldc) with the trans flags
  // of B and A, and execute passes dB as A and dA as B.
  bool row_major = false;
  int aux_trans = 0;               // kTransAFlag / kTransBFlag of the planned product
  void* d_mem = nullptr;           // header | descs[cap] | items[cap]
  void* h_stage[bgemm::kStageBufs] = {};      // ring of pinned staging, same layout
  cudaEvent_t ev_stage[bgemm::kStageBufs] = {};  // upload from h_stage[i] consumed
  bool stage_used[bgemm::kStageBufs] = {};
  int stage = 0;                   // staging buffer of the next upload
  bool staged_in_capture = false;  // created during a stream capture (no updates)
  size_t off_descs = 0, off_items = 0, mem_bytes = 0;
  int* d_counters = nullptr;       // the device header
  bgemm::MatDesc* d_descs = nullptr;
  bgemm::TileItem* d_items = nullptr;
  bgemm::TcPlan* tc = nullptr;
  std::vector<bgemm::MatDesc> host_descs;
  bgemm_plan_info_t info{};
  unsigned long long* d_cta_times = nullptr;  // profiling hook: per-CTA start/end times
  // Mixed plan (options.simt_below > 0): two child plans over masked sizes --
  // matrices with min(M, N, K) < simt_below on FP32 SIMT, the rest in the
  // plan's tensor-core mode; both take the caller's full pointer arrays.
  bgemm_plan_s* mix_simt = nullptr;
  bgemm_plan_s* mix_tc = nullptr;
  cudaEvent_t ev_start = nullptr;  // profiling hook around the GEMM launch
  cudaEvent_t ev_stop = nullptr;
};

namespace bgemm {

bgemm_status_t set_error(bgemm_status_t st, int arg, int mat, const char* fmt, ...);
bgemm_status_t cuda_error(cudaError_t e, const char* what);
bgemm_status_t device_facts(DeviceFacts* out);

// Tile count and modelled time of one tile of configuration c; false if the
// configuration cannot take the matrix.
using TileEval = bool (*)(int c, int M, int N, int K, long long* tiles, double* t_tile);
// Per-matrix least-total-time choice, then the parallelism rebalance over
// `slots` persistent CTAs (shared by the SIMT and tensor-core planners).
bgemm_status_t choose_tiles(int ncfg, TileEval eval, const int* M, const int* N, const int* K,
                            int batch, int slots, const bgemm_plan_options_t* opt,
                            std::vector<MatPlan>& mp);

// tensor-core hooks (tc_plan.cpp)
// tc_init: mode facts and option checks, once per plan.
// clusters >= 0 overrides the CTA pairs the device fits (host-only replays).
bgemm_status_t tc_init(bgemm_plan_s* p, const bgemm_plan_options_t* opt, int clusters = -1);
void tc_debug_layout(bgemm_plan_s* p, long long* ws_out, int* jobs_out, int max_jobs,
                     int* n_jobs, int* pair);
// tc_choose: tile configurations of a batch; the first call of a plan also
// fixes its kernel family (one-SM or CTA pair), later calls keep it.
bgemm_status_t tc_choose(bgemm_plan_s* p, const int* M, const int* N, const int* K, int batch,
                         bool first, std::vector<MatPlan>& mp);
void tc_tile_dims(bgemm_plan_s* p, int i, int M, int N, int cfg, int* bm, int* bn, MatDesc* d);
// tc_layout: split-operand workspace offsets and pre-pass jobs of a planned
// batch (kept in the TcPlan until tc_commit); fills the requirement fields.
void tc_layout(bgemm_plan_s* p, const std::vector<MatDesc>& hd, bgemm_plan_requirements_t* req);
// tc_alloc: device/pinned buffers for the plan's capacity, launch shapes.
bgemm_status_t tc_alloc(bgemm_plan_s* p);
// tc_commit: stage and upload the laid-out batch through staging buffer
// `stage`, build its tensor maps (first: also templates and error word).
bgemm_status_t tc_commit(bgemm_plan_s* p, int stage, int batch, bool first, cudaStream_t stream);
bgemm_status_t tc_execute(bgemm_plan_s* p, float alpha, const float* const* dA,
                          const float* const* dB, float beta, float* const* dC,
                          cudaStream_t stream);
bgemm_status_t tc_check_device(bgemm_plan_s* p, cudaStream_t stream);
int tc_debug_compare_tmaps(bgemm_plan_s* p, cudaStream_t stream, int* n_maps, int* n_diff,
                           int* first_byte);
void tc_plan_release(bgemm_plan_s* p);
// errors of the device-resident tensor-core path (framework_tc.cu)
bgemm_status_t fwtc_check_device(int dev);
bgemm_status_t fwtc_release(int dev);

}  // namespace bgemm
