// tc_plan.cpp -- planner hooks of the tensor-core modes (placeholder until
// the tcgen05 kernel lands).
#include "plan_internal.h"

namespace bgemm {

bgemm_status_t tc_choose(bgemm_plan_s*, const int*, const int*, const int*, int,
                         const bgemm_plan_options_t*, std::vector<MatPlan>&) {
  return set_error(BGEMM_ERROR_NOT_SUPPORTED, 13, -1, "tensor-core modes are not built yet");
}
void tc_tile_dims(bgemm_plan_s*, int, int, int, int, int* bm, int* bn, MatDesc*) {
  *bm = 128;
  *bn = 128;
}
size_t tc_extra_bytes(bgemm_plan_s*, int) { return 0; }
bgemm_status_t tc_plan_finish(bgemm_plan_s*, cudaStream_t) { return BGEMM_ERROR_NOT_SUPPORTED; }
bgemm_status_t tc_execute(bgemm_plan_s*, float, const float* const*, const float* const*, float,
                          float* const*, cudaStream_t) {
  return BGEMM_ERROR_NOT_SUPPORTED;
}
bgemm_status_t tc_check_device(bgemm_plan_s*, cudaStream_t) { return BGEMM_SUCCESS; }
void tc_plan_release(bgemm_plan_s*) {}

}  // namespace bgemm
