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

// gemm_api.cu: the algorithm a GEMM runs with (algo as given, GB_ALGO_AUTO
// resolved), and an upper bound on the library workspace (bytes, per stream)
// that the call may need -- used by the server to reserve workspace before
// capturing a request into a CUDA graph.
int resolve_algo(int bits, int algo, bool ta, bool tb, int64_t M, int64_t N, int64_t K);
size_t gemm_workspace_bound(int bits, int algo, bool ta, bool tb, int64_t M, int64_t N, int64_t K, const void *A,
                            int64_t lda, const void *B, int64_t ldb, int slices, int split_k);

}  // namespace gb
