// Variants not built yet report HD_ERR_UNSUPPORTED.
#include "hd_internal.h"
namespace hdg {
hd_status run_brute(Ctx& c, const DirInput&) { return fail(c, HD_ERR_UNSUPPORTED, "brute not built"); }
hd_status run_bf16(Ctx& c, const DirInput&, DirResult*) { return fail(c, HD_ERR_UNSUPPORTED, "bf16 not built"); }
hd_status select_variant(Ctx&, const DirInput& in, int* v) {
  *v = (in.dims == 2 || in.dims == 3) ? HD_VARIANT_LBVH : HD_VARIANT_EB;
  return HD_OK;
}
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
