// batch.cu — batched and served placement (many resident instances).
#include "../../include/texo_gp.h"

extern "C" {
int32_t texo_gp_batch_create(const texo_gp_params*, uint64_t, uint32_t, texo_gp_batch* out) {
  if (out) *out = nullptr;
  return TEXO_GP_ERR_UNSUPPORTED;
}
int32_t texo_gp_batch_destroy(texo_gp_batch) { return TEXO_GP_ERR_UNSUPPORTED; }
int32_t texo_gp_batch_admit(texo_gp_batch, const texo_gp_problem*, uint64_t, uint32_t*) { return TEXO_GP_ERR_UNSUPPORTED; }
int32_t texo_gp_batch_advance(texo_gp_batch, uint32_t) { return TEXO_GP_ERR_UNSUPPORTED; }
int32_t texo_gp_batch_retire(texo_gp_batch, uint64_t*, uint32_t*, uint64_t, texo_gp_stats*) { return TEXO_GP_ERR_UNSUPPORTED; }
int32_t texo_gp_batch_counts(texo_gp_batch, uint32_t*, uint32_t*, uint64_t*) { return TEXO_GP_ERR_UNSUPPORTED; }
}
