// Batched persistent path (under construction).
#include "../../include/ndfiltrs_gb300.h"

extern "C" {

int ndf_batch_create(const ndf_filter_desc*, int32_t, ndf_batch** batch) {
  if (batch) *batch = nullptr;
  return NDF_ERR_UNSUPPORTED;
}
int ndf_batch_destroy(ndf_batch*) { return NDF_OK; }
int ndf_batch_run(ndf_batch*, const void* const*, void* const*, void*) { return NDF_ERR_UNSUPPORTED; }
int32_t ndf_batch_launches(const ndf_batch*) { return 0; }

}  // extern "C"
