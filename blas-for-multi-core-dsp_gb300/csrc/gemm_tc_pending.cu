// gemm_tc_pending.cu -- entry points of the tensor-core DGEMM form that this
// build does not contain yet; it reports GB_ERR_UNSUPPORTED.
#include "gb_common.cuh"

namespace gb {
gb_status launch_dgemm_ozaki(const GemmArgs &, int) {
    return set_status(GB_ERR_UNSUPPORTED, "gb_dgemm: OZAKI is not built in this library");
}
}  // namespace gb
