/* The C ABI used the way a foreign-function binding uses it (Julia ccall,
 * ctypes): plain structs and pointers, no headers beyond include/geosgs.h.
 *
 *   c_abi_smoke nogpu   argument and state errors (no device needed)
 *   c_abi_smoke gpu     a 2D plan end to end: create, prepare, simulate into a
 *                       host buffer, info, destroy; a datum on a cell centre
 *                       is reproduced within 1e-6 (nugget 0) and two seeded
 *                       calls agree bit for bit
 * Exit status 0 on success; the failing check is printed. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "geosgs.h"

#define CHECK(c)                                                   \
    do {                                                           \
        if (!(c)) {                                                \
            fprintf(stderr, "check failed line %d: %s\n", __LINE__, #c); \
            return 1;                                              \
        }                                                          \
    } while (0)

static void problem_2d(sgs_problem* p, const double* xy, const double* v, int64_t nd) {
    memset(p, 0, sizeof(*p));
    p->dim = 2;
    p->dims[0] = 64;
    p->dims[1] = 48;
    p->dims[2] = 1;
    p->spacing[0] = p->spacing[1] = p->spacing[2] = 1.0;
    p->ndata = nd;
    p->data_coords = xy;
    p->data_values = v;
    p->variogram.type = SGS_SPHERICAL;
    p->variogram.sill = 1.0;
    p->variogram.nugget = 0.0;
    for (int j = 0; j < 3; ++j) p->variogram.ranges[j] = 10.0;
    for (int j = 0; j < 3; ++j) p->variogram.rotation[4 * j] = 1.0;
    p->mean = 0.5;
    p->minneighbors = 1;
    p->maxneighbors = 12;
    p->search = SGS_SEARCH_RANGE;
    p->precision = SGS_PREC_FP32_REFINE;
    p->refine_steps = 2;
}

static int nogpu(void) {
    sgs_plan* plan = NULL;
    CHECK(sgs_plan_create(NULL, &plan) == SGS_ERR_ARG);
    CHECK(sgs_last_error(NULL) != NULL);
    sgs_problem p;
    problem_2d(&p, NULL, NULL, 0);
    p.dim = 4;
    CHECK(sgs_plan_create(&p, &plan) == SGS_ERR_ARG && plan == NULL);
    p.dim = 2;
    p.maxneighbors = 65;
    CHECK(sgs_plan_create(&p, &plan) == SGS_ERR_ARG);
    CHECK(sgs_plan_prepare(NULL) == SGS_ERR_ARG);
    sgs_plan_destroy(NULL); /* no-op */
    CHECK(strlen(sgs_version()) > 0);
    return 0;
}

static int gpu(void) {
    const double xy[2] = {20.5, 30.5}; /* the centre of cell (20, 30) */
    const double v[1] = {2.25};
    sgs_problem p;
    problem_2d(&p, xy, v, 1);
    sgs_plan* plan = NULL;
    CHECK(sgs_plan_create(&p, &plan) == SGS_OK && plan != NULL);
    const int R = 6;
    const int64_t N = 64 * 48;
    double* a = malloc(sizeof(double) * R * N);
    double* b = malloc(sizeof(double) * R * N);
    CHECK(a && b);
    CHECK(sgs_plan_simulate(plan, R, NULL, 7, a) == SGS_ERR_STATE); /* before prepare */
    CHECK(sgs_plan_prepare(plan) == SGS_OK);
    CHECK(sgs_plan_simulate(plan, R, NULL, 7, a) == SGS_OK);
    CHECK(sgs_plan_simulate(plan, R, NULL, 7, b) == SGS_OK);
    CHECK(memcmp(a, b, sizeof(double) * R * N) == 0);
    const int64_t cell = 20 + 64 * 30;
    for (int r = 0; r < R; ++r) {
        CHECK(fabs(a[r * N + cell] - 2.25) <= 1e-6);
        for (int64_t g = 0; g < N; ++g) CHECK(isfinite(a[r * N + g]));
    }
    sgs_info info;
    CHECK(sgs_plan_info(plan, &info) == SGS_OK);
    CHECK(info.nnodes == N && info.ndata == 1 && info.nlevels > 0 && info.launches > 0);
    sgs_plan_destroy(plan);
    free(a);
    free(b);
    return 0;
}

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    const int rc = strcmp(argv[1], "gpu") == 0 ? gpu() : nogpu();
    if (rc == 0) printf("c_abi_smoke %s ok\n", argv[1]);
    return rc;
}
