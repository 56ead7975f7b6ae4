// gb_internal.h -- interfaces shared between the library's host modules.
#pragma once

#include "gbblas.h"

namespace gb {

// grouped.cu: the grouped persistent kernel's launcher (slots of pinned
// staging + device work list + optional CUDA graph).
struct GroupRunner;
GroupRunner *group_runner_create(int nslots, int max_items);
void group_runner_destroy(GroupRunner *r);
gb_status group_runner_run(GroupRunner *r, const gb_gemm_desc *d, int n, void *stream, int use_graph);
gb_status check_desc(const gb_gemm_desc &q, int i);

}  // namespace gb
