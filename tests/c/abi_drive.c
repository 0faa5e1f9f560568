/* abi_drive.c -- a plain C99 caller of libewpt (include/ewpt.h), the third
 * client of the boundary besides the Julia and Python bindings.
 *
 *   abi_drive host          argument checks only; no device work
 *   abi_drive gpu N steps   N^3 FP64 lattice: tanh-bubble IC on the device,
 *                           `steps` RK4 steps, then prints the snapshot row
 *                           and the B-field energy from ewpt_fields, one
 *                           "%.17g" number per line
 *
 * Exit status 0 on success, 1 on a failed check, 2 on a library error. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ewpt.h"

#define CHECK(cond, msg)                                \
    do {                                                \
        if (!(cond)) {                                  \
            fprintf(stderr, "check failed: %s\n", msg); \
            return 1;                                   \
        }                                               \
    } while (0)

#define CALL(expr)                                                                   \
    do {                                                                             \
        int rc_ = (expr);                                                            \
        if (rc_ != EWPT_OK) {                                                        \
            fprintf(stderr, "%s -> %d: %s\n", #expr, rc_, ewpt_last_error(ctx));     \
            return 2;                                                                \
        }                                                                            \
    } while (0)

static int host_checks(void) {
    ewpt_params p;
    ewpt_ctx* ctx = NULL;
    CHECK(ewpt_params_default(&p, 32) == EWPT_OK, "params_default");
    CHECK(p.nx == 32 && p.ny == 32 && p.nz == 32 && p.precision == EWPT_FP64, "default dims / form");
    CHECK(fabs(p.dt - p.dx / 10.0) < 1e-15 && p.stencil_order == 6, "default dt / order");
    CHECK(ewpt_create(NULL, &ctx) == EWPT_ERR_ARG, "create rejects NULL params");
    p.nx = 3;
    CHECK(ewpt_create(&p, &ctx) == EWPT_ERR_ARG && ctx == NULL, "create rejects nx < 7");
    CHECK(strlen(ewpt_last_error(NULL)) > 0, "error message");
    CHECK(ewpt_step(NULL, 1) == EWPT_ERR_ARG, "step rejects NULL ctx");
    CHECK(ewpt_step_host(NULL, NULL, NULL, 1) == EWPT_ERR_ARG, "step_host rejects NULL ctx");
    CHECK(ewpt_field_components(EWPT_FIELD_DENSITY) == 7 && ewpt_field_components(99) == -1, "field components");
    CHECK(ewpt_kc_bin_nums(4, 4, 4) > 0 && ewpt_kc_bin_nums(0, 4, 4) == -1, "kc_bin_nums");
    printf("host ok\n");
    return 0;
}

static int gpu_run(int n, int steps) {
    ewpt_params p;
    ewpt_ctx* ctx = NULL;
    double row[EWPT_NDIAG];
    /* 3 bubbles: centre (1-based), direction; tanh profile R = 2/sqrt(lambda), w = 1/(sqrt(lambda) vev) */
    const double bub[3][7] = {{4, 5, 6, 1, 0, 0, 0}, {n / 2.0, n / 2.0, n / 3.0, 0, 1, 0, 0}, {n - 3.0, 7, n / 2.0, 0, 0, 0.6, 0.8}};
    size_t S;
    double* f;
    double eb = 0.0;
    int q;
    size_t c;
    if (ewpt_params_default(&p, n) != EWPT_OK) return 2;
    CALL(ewpt_create(&p, &ctx));
    CALL(ewpt_init_bubbles(ctx, 3, &bub[0][0], EWPT_BUBBLE_TANH, 2.0 / sqrt(p.lambda), 1.0 / (sqrt(p.lambda) * p.vev)));
    CALL(ewpt_step(ctx, steps));
    CALL(ewpt_sync(ctx));
    CALL(ewpt_diagnostics(ctx, row));
    S = (size_t)n * n * n;
    f = (double*)malloc(3 * S * sizeof(double));
    if (!f) return 2;
    CALL(ewpt_fields(ctx, EWPT_FIELD_B, f, 0));
    for (c = 0; c < 3 * S; ++c) eb += f[c] * f[c];
    eb *= 0.5 * p.dx * p.dx * p.dx;
    free(f);
    CHECK(ewpt_iteration(ctx) == steps, "iteration counter");
    for (q = 0; q < EWPT_NDIAG; ++q) printf("%.17g\n", row[q]);
    printf("%.17g\n", eb);
    CALL(ewpt_destroy(ctx));
    return 0;
}

int main(int argc, char** argv) {
    if (argc >= 2 && strcmp(argv[1], "host") == 0) return host_checks();
    if (argc >= 4 && strcmp(argv[1], "gpu") == 0) return gpu_run(atoi(argv[2]), atoi(argv[3]));
    fprintf(stderr, "usage: abi_drive host | abi_drive gpu N steps\n");
    return 2;
}
