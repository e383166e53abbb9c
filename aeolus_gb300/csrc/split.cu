// Contraction precision control.  The split-precision (bf16-sliced,
// tcgen05) Legendre contraction is selected per plan here.
#include "common.cuh"

namespace aeolus {

struct SplitTables {
  int slices = 0;
};

void free_split(aeolus_plan_impl* p) {
  delete p->split;
  p->split = nullptr;
}

}  // namespace aeolus

using namespace aeolus;

extern "C" int aeolus_plan_set_precision(aeolus_plan plan, int precision, int slices) {
  if (!plan) return fail(AEOLUS_ERR_ARG, "aeolus_plan_set_precision: plan is NULL");
  if (precision == AEOLUS_PREC_FP64) {
    plan->precision = precision;
    plan->slices = 0;
    return AEOLUS_OK;
  }
  (void)slices;
  return fail(AEOLUS_ERR_ARG, "aeolus_plan_set_precision: unsupported precision mode");
}
