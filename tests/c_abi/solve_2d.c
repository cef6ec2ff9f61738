/* A C program on the engine's C ABI (include/dcrf.h) -- what a host that binds
 * the library directly (cgo, JNI, a C++ service) does for one DenseCRF2D solve.
 *
 *   solve_2d W H M T        solve a seeded W x H image with M labels, T iterations
 *
 * Prints the ABI version, then either "no device: <message>" (exit 0: the
 * library reports DCRF_ERR_NO_DEVICE explicitly, with no CPU fallback) or the
 * checks of the solve: every point's marginals sum to 1, the argmax labels
 * of dcrf_map agree with the marginals, and a second solve of the same handle
 * reproduces the first bit for bit. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "dcrf.h"

static uint32_t rng = 12345u;
static float uniform(void) {
    rng = rng * 1664525u + 1013904223u;
    return (float)(rng >> 8) / 16777216.0f;
}

static int fail(const char *what, int rc) {
    char msg[512];
    dcrf_last_error(msg, sizeof msg);
    fprintf(stderr, "%s failed (%d): %s\n", what, rc, msg);
    return 1;
}

int main(int argc, char **argv) {
    const int W = argc > 1 ? atoi(argv[1]) : 64, H = argc > 2 ? atoi(argv[2]) : 48;
    const int M = argc > 3 ? atoi(argv[3]) : 5, T = argc > 4 ? atoi(argv[4]) : 5;
    const int N = W * H;
    printf("abi %d\n", dcrf_abi_version());
    dcrf_crf *h = NULL;
    int rc = dcrf_create_2d(W, H, M, &h);
    if (rc == DCRF_ERR_NO_DEVICE) {
        char msg[512];
        dcrf_last_error(msg, sizeof msg);
        printf("no device: %s\n", msg);
        return 0;
    }
    if (rc) return fail("dcrf_create_2d", rc);

    float *U = malloc(sizeof(float) * (size_t)M * N), *Q = malloc(sizeof(float) * (size_t)M * N);
    float *Q2 = malloc(sizeof(float) * (size_t)M * N);
    uint8_t *img = malloc((size_t)3 * N);
    int16_t *map = malloc(sizeof(int16_t) * (size_t)N);
    for (size_t i = 0; i < (size_t)M * N; i++) U[i] = 0.05f + 3.0f * uniform();  /* label-major M x N */
    for (size_t i = 0; i < (size_t)3 * N; i++) img[i] = (uint8_t)(256.0f * uniform());
    const float w_gauss = 3.0f, w_bilat = 5.0f;
    if ((rc = dcrf_set_unary(h, U, DCRF_LAYOUT_LM, DCRF_HOST))) return fail("dcrf_set_unary", rc);
    if ((rc = dcrf_add_pairwise_gaussian(h, 3.0f, 3.0f, DCRF_COMPAT_POTTS, &w_gauss, DCRF_DIAG_KERNEL,
                                         DCRF_NORMALIZE_SYMMETRIC, NULL)))
        return fail("dcrf_add_pairwise_gaussian", rc);
    if ((rc = dcrf_add_pairwise_bilateral(h, 20.0f, 20.0f, 13.0f, 13.0f, 13.0f, img, DCRF_HOST, DCRF_COMPAT_POTTS,
                                          &w_bilat, DCRF_DIAG_KERNEL, DCRF_NORMALIZE_SYMMETRIC, NULL)))
        return fail("dcrf_add_pairwise_bilateral", rc);
    if ((rc = dcrf_inference(h, T, Q, DCRF_LAYOUT_PM, DCRF_HOST))) return fail("dcrf_inference", rc);
    if ((rc = dcrf_inference(h, T, Q2, DCRF_LAYOUT_PM, DCRF_HOST))) return fail("dcrf_inference (again)", rc);
    if ((rc = dcrf_map(h, T, map, DCRF_HOST))) return fail("dcrf_map", rc);

    double worst = 0.0;
    int map_ok = 1;
    for (int p = 0; p < N; p++) {
        double s = 0.0;
        int best = 0;
        for (int m = 0; m < M; m++) {
            s += Q[(size_t)p * M + m];
            if (Q[(size_t)p * M + m] > Q[(size_t)p * M + best]) best = m;
        }
        if (fabs(s - 1.0) > worst) worst = fabs(s - 1.0);
        if (map[p] != best) map_ok = 0;
    }
    const int same = memcmp(Q, Q2, sizeof(float) * (size_t)M * N) == 0;
    printf("solved %dx%d M=%d T=%d: max |sum Q - 1| = %.3g, map %s, repeat %s\n", W, H, M, T, worst,
           map_ok ? "ok" : "MISMATCH", same ? "identical" : "DIFFERENT");
    dcrf_destroy(h);
    free(U), free(Q), free(Q2), free(img), free(map);
    return (worst < 1e-5 && map_ok && same) ? 0 : 2;
}
