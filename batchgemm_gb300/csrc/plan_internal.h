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

}  // namespace bgemm

struct bgemm_plan_s {
  int batch = 0;
  int mode = 0;
  int n_items = 0;
  int grid = 0;
  bgemm::DeviceFacts facts{};
  void* d_mem = nullptr;     // counters | descs | items | mode extras
  void* h_pinned = nullptr;  // staging of counters | descs | items
  int* d_counters = nullptr;
  bgemm::MatDesc* d_descs = nullptr;
  bgemm::TileItem* d_items = nullptr;
  char* d_extra = nullptr;
  bgemm::TcPlan* tc = nullptr;
  std::vector<bgemm::MatDesc> host_descs;
  bgemm_plan_info_t info{};
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
bgemm_status_t tc_choose(bgemm_plan_s* p, const int* M, const int* N, const int* K, int batch,
                         const bgemm_plan_options_t* opt, std::vector<MatPlan>& mp);
void tc_tile_dims(bgemm_plan_s* p, int i, int M, int N, int cfg, int* bm, int* bn, MatDesc* d);
size_t tc_extra_bytes(bgemm_plan_s* p, int batch);
bgemm_status_t tc_plan_finish(bgemm_plan_s* p, cudaStream_t stream);
bgemm_status_t tc_execute(bgemm_plan_s* p, float alpha, const float* const* dA,
                          const float* const* dB, float beta, float* const* dC,
                          cudaStream_t stream);
bgemm_status_t tc_check_device(bgemm_plan_s* p, cudaStream_t stream);
int tc_debug_compare_tmaps(bgemm_plan_s* p, cudaStream_t stream, int* n_maps, int* n_diff,
                           int* first_byte);
void tc_plan_release(bgemm_plan_s* p);

}  // namespace bgemm
