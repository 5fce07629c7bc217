// Variants not built yet report HD_ERR_UNSUPPORTED.
#include "hd_internal.h"
namespace hdg {
}
extern "C" {
hd_status hd_solve_batch(hd_ctx* c, const float*, uint64_t, const float*, uint64_t, int,
                         const hd_problem*, uint64_t, uint32_t, hd_batch_result*) {
  return hdg::fail(*c, HD_ERR_UNSUPPORTED, "batch not built");
}
hd_status hd_solve_batch_plain(hd_ctx* c, const float*, uint64_t, const float*, uint64_t, int,
                               const hd_problem*, uint64_t, uint32_t, hd_batch_result*) {
  return hdg::fail(*c, HD_ERR_UNSUPPORTED, "batch not built");
}
}
