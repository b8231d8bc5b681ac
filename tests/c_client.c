/*
 * c_client.c -- a plain C99 caller of libenkfg, as EnKF-C's host code would
 * be: it includes only include/enkfg.h and links the shared library.  Used by
 * tests/test_capi.py.  Exercises the host-only entry points (status strings,
 * the NetCDF files) and context creation, which fails cleanly without a GPU.
 * Prints "ok" and returns 0 on success.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "enkfg.h"

#define CHECK(cond, msg)                                           \
    do {                                                           \
        if (!(cond)) {                                             \
            fprintf(stderr, "c_client: %s (%s)\n", msg, enkfg_nc_last_error()); \
            return 1;                                              \
        }                                                          \
    } while (0)

int main(int argc, char** argv)
{
    const int nj = 3, ni = 4, md = 2, m = 5;
    float T[3 * 4 * 2 * 5], w[3 * 4 * 5], back[3 * 4 * 5];
    long long start[3] = { 0, 0, 0 }, count[3] = { 3, 4, 5 }, dims[ENKFG_NC_MAXDIMS];
    int ndims = 0, type = 0, rec = -1, k;
    enkfg_ctx* ctx = NULL;
    enkfg_status st;

    if (argc < 2)
        return 2;
    for (k = 0; k < nj * ni * md * m; ++k)
        T[k] = (float) k * 0.25f;
    for (k = 0; k < nj * ni * m; ++k)
        w[k] = (float) k - 7.5f;

    CHECK(strcmp(enkfg_status_string(ENKFG_OK), "ok") == 0, "status string");
    CHECK(enkfg_version() >= 1, "version");
    st = enkfg_nc_write_transforms(argv[1], nj, ni, md, m, T, w, 3, "grid0");
    CHECK(st == ENKFG_OK, "write transforms");
    st = enkfg_nc_inq_var(argv[1], "w", &ndims, dims, &type, &rec);
    CHECK(st == ENKFG_OK && ndims == 3 && dims[0] == nj && dims[1] == ni && dims[2] == m && type == 5 && rec == 0,
          "inquire w");
    st = enkfg_nc_get_vara_float(argv[1], "w", start, count, back);
    CHECK(st == ENKFG_OK && memcmp(back, w, sizeof(w)) == 0, "read w back");
    st = enkfg_nc_inq_var(argv[1], "nope", NULL, NULL, NULL, NULL);
    CHECK(st == ENKFG_EINVAL && strstr(enkfg_nc_last_error(), "nope") != NULL, "missing variable is an error");

    /* the per-type search options and RANDOMISE: a NULL context is refused */
    CHECK(enkfg_set_obstype_nlobsmax(NULL, 1, NULL) == ENKFG_EINVAL, "nlobsmax without a context");
    CHECK(enkfg_set_obstype_visible(NULL, 1, NULL) == ENKFG_EINVAL, "visibility without a context");
    CHECK(enkfg_set_field_noise(NULL, 0, 0, NULL, NULL, NULL) == ENKFG_EINVAL, "noise without a context");

    /* a context: ENKFG_OK on a GPU machine, an error status (not an abort) without one */
    st = enkfg_create(0, &ctx);
    if (st == ENKFG_OK) {
        CHECK(enkfg_set_obs(ctx, 1, NULL, NULL, NULL, NULL, NULL, NULL) == ENKFG_ESTATE, "call order is checked");
        CHECK(enkfg_set_obstype_nlobsmax(ctx, 1, NULL) == ENKFG_ESTATE, "nlobsmax needs the obs types");
        enkfg_destroy(ctx);
    } else {
        CHECK(ctx == NULL || st != ENKFG_OK, "failed creation");
    }
    printf("ok\n");
    return 0;
}
