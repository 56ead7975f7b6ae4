/* The serving loop and the workspace query as a C caller uses them (the
 * calls of the serving example in the integration notes), on a dry-run
 * server: admission, routing, completion and statistics run on the host and
 * no device work is done, so this runs without a GPU.  Exit status 0 when
 * every check holds; the failing check's number otherwise. */
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "gbblas.h"

int main(void) {
    gb_server_config cfg;
    gb_server_config_init(&cfg);
    if (cfg.streams != 6 || cfg.short_streams != 2 || cfg.short_us != 200.0 || cfg.long_sm_percent != 100) return 1;
    cfg.dry_run = 1;
    cfg.use_grouped = 0;
    gb_server *srv = NULL;
    if (gb_server_create(&cfg, &srv) != GB_OK || srv == NULL) return 2;

    /* dummy, never dereferenced operand addresses */
    static double dA[4], dB[4], dC[4];
    for (int i = 0; i < 5; i++) {   /* long: a 2048^3 FP64 product */
        gb_request r;
        memset(&r, 0, sizeof r);
        r.op = GB_OP_GEMM; r.dtype_bits = 64; r.transA = 'N'; r.transB = 'T';
        r.algo = GB_ALGO_OZAKI; r.semantics = GB_SEM_BLAS;
        r.M = 2048; r.N = 2048; r.K = 2048; r.alpha = 1.0; r.beta = 0.0;
        r.A = dA; r.lda = 2048; r.B = dB; r.ldb = 2048; r.C = dC; r.ldc = 2048; r.tag = (uint64_t)i;
        if (gb_server_submit(srv, &r) != GB_OK) return 3;
    }
    for (int i = 0; i < 3; i++) {   /* short: a 256 x 256 FP32 transpose */
        gb_request r;
        memset(&r, 0, sizeof r);
        r.op = GB_OP_TRANSPOSE; r.dtype_bits = 32;
        r.M = 256; r.N = 256;
        r.A = dA; r.lda = 256; r.B = dB; r.ldb = 256; r.tag = 100 + (uint64_t)i;
        if (gb_server_submit(srv, &r) != GB_OK) return 4;
    }
    if (gb_server_drain(srv, 10.0) != GB_OK) return 5;
    uint64_t tags[64];
    double lat[64];
    int n = gb_server_poll(srv, tags, lat, 64);
    if (n != 8) return 6;
    uint64_t tag_sum = 0;
    for (int i = 0; i < n; i++) {
        tag_sum += tags[i];
        if (lat[i] < 0.0) return 7;
    }
    if (tag_sum != (0 + 1 + 2 + 3 + 4) + (100 + 101 + 102)) return 8;
    gb_server_stats st;
    if (gb_server_get_stats(srv, &st) != GB_OK) return 9;
    if (st.submitted != 8 || st.completed != 8 || st.launches != 8 || st.urgent_launches != 3) return 10;
    if (st.inflight != 0 || st.inflight_bytes != 0 || st.p99_s < st.p50_s) return 11;
    gb_server_destroy(srv);

    /* the two-pass forms' workspace bound needs no device */
    gb_gemm_opts o;
    gb_gemm_opts_init(&o);
    o.algo = GB_ALGO_FP16X3;
    size_t bytes = 0;
    if (gb_workspace_query(32, 'N', 'N', 1000, 700, 900, NULL, 900, NULL, 700, &o, &bytes) != GB_OK) return 12;
    const size_t kp = 960, lines = 1700;
    if (bytes != 2 * (3 * lines * kp * 2 + lines * 4 + 1024) + 4096) return 13;
    if (gb_workspace_query(16, 'N', 'N', 4, 4, 4, NULL, 4, NULL, 4, &o, &bytes) != GB_ERR_INVALID_ARG) return 14;
    if (gb_last_error_string() == NULL || gb_last_error_string()[0] == '\0') return 15;
    puts("server dry run ok");
    return 0;
}
