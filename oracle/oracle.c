/*
 * CPU oracle for the TMz FDTD step -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
 *
 * A plain-C restatement of the reference's per-step update equations
 * (FDTD_2D_Full/kernel.cu:127-805, step order :2073-2157), run either in FP64
 * (the parity oracle the CUDA path is checked against) or in FP32 (the timed
 * CPU baseline).  It consumes the same fdtd2d_setup the CUDA library does, so
 * both see identical coefficient tables, maps and source parameters.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this library, and only as the checker / the baseline.
 *
 * Parity status: pinned against the reference program itself, compiled from
 * its own sources for the CPU by oracle/ref_build.py into oracle/_ref/ (its
 * CUDA kernels run serially on the host through oracle/ref_shim/); the
 * committed vectors in tests/golden/ come from that build
 * (tests/golden/make_golden.py).
 */
#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/fdtd2d.h"

#define MAXP 128
#define ORACLE_PI 3.14159265358979323846

#define REAL double
#define NAME(x) o64_##x
#include "oracle_impl.h"
#undef REAL
#undef NAME

#define REAL float
#define NAME(x) o32_##x
#include "oracle_impl.h"
#undef REAL
#undef NAME

typedef struct oracle {
    int fp32;
    o64_state *d;
    o32_state *f;
} oracle;

/* The checks fdtd2d_create makes on the grid and the point lists, so that
   the oracle refuses what the library refuses instead of indexing outside
   its arrays: NULL for a grid below 8 cells or one that the CPML strips do
   not fit, or a source, detector or component detector outside the cells
   1..nx-2 x 1..ny-2. */
static int oracle_points_ok(const fdtd2d_point *pts, int n, const fdtd2d_setup *s) {
    int e;
    if (n < 0 || (n > 0 && !pts)) return 0;
    for (e = 0; e < n; ++e)
        if (pts[e].i < 1 || pts[e].i > s->nx - 2 || pts[e].j < 1 || pts[e].j > s->ny - 2) return 0;
    return 1;
}

oracle *oracle_create(const fdtd2d_setup *s, int fp32) {
    oracle *o;
    if (!s) return NULL;
    if (s->nx < 8 || s->ny < 8 || s->npml < 2 || 2 * s->npml + 2 > s->nx || 2 * s->npml + 2 > s->ny ||
        s->n_steps < 1)
        return NULL;
    if (!oracle_points_ok(s->src, s->n_src, s) || !oracle_points_ok(s->det, s->n_det, s) ||
        !oracle_points_ok(s->comp, s->n_comp, s))
        return NULL;
    o = (oracle *)calloc(1, sizeof(*o));
    if (!o) return NULL;
    o->fp32 = fp32;
    if (fp32) o->f = o32_create(s);
    else o->d = o64_create(s);
    if (!o->d && !o->f) {
        free(o);
        return NULL;
    }
    return o;
}

void oracle_destroy(oracle *o) {
    if (!o) return;
    o64_free_state(o->d);
    o32_free_state(o->f);
    free(o);
}

int oracle_current_step(const oracle *o) { return o ? (o->fp32 ? o->f->step : o->d->step) : -1; }

/* Steps n_first..n_last inclusive; n_first must follow the last step run. */
int oracle_run(oracle *o, int n_first, int n_last) {
    int n;
    const int cur = oracle_current_step(o);
    const int nmax = o ? (o->fp32 ? o->f->n_steps : o->d->n_steps) : 0;
    if (!o || n_first != cur + 1 || n_last > nmax) return FDTD2D_ERR_RANGE;
    for (n = n_first; n <= n_last; ++n) {
        if (o->fp32) o32_step(o->f, n);
        else o64_step(o->d, n);
    }
    return FDTD2D_OK;
}

int oracle_field_shape(oracle *o, int which, int *rows, int *cols) {
    void *p = o->fp32 ? (void *)o32_field(o->f, which, rows, cols) : (void *)o64_field(o->d, which, rows, cols);
    return p ? FDTD2D_OK : FDTD2D_ERR_INVALID;
}

int oracle_read_field(oracle *o, int which, double *out) {
    int rows, cols;
    size_t k, n;
    if (!o || !out) return FDTD2D_ERR_INVALID;
    if (o->fp32) {
        const float *p = o32_field(o->f, which, &rows, &cols);
        if (!p) return FDTD2D_ERR_INVALID;
        n = (size_t)rows * cols;
        for (k = 0; k < n; ++k) out[k] = p[k];
    } else {
        const double *p = o64_field(o->d, which, &rows, &cols);
        if (!p) return FDTD2D_ERR_INVALID;
        memcpy(out, p, (size_t)rows * cols * sizeof(double));
    }
    return FDTD2D_OK;
}

int oracle_write_field(oracle *o, int which, const double *in) {
    int rows, cols;
    size_t k, n;
    if (!o || !in) return FDTD2D_ERR_INVALID;
    if (o->fp32) {
        float *p = o32_field(o->f, which, &rows, &cols);
        if (!p) return FDTD2D_ERR_INVALID;
        n = (size_t)rows * cols;
        for (k = 0; k < n; ++k) p[k] = (float)in[k];
    } else {
        double *p = o64_field(o->d, which, &rows, &cols);
        if (!p) return FDTD2D_ERR_INVALID;
        memcpy(p, in, (size_t)rows * cols * sizeof(double));
    }
    return FDTD2D_OK;
}

int oracle_read_traces(oracle *o, int n0, int n1, float *det, float *cez, float *chx, float *chy) {
    int n, e, nd, nc, rec, nmax;
    const float *tr, *ct;
    if (!o) return FDTD2D_ERR_INVALID;
    nd = o->fp32 ? o->f->n_det : o->d->n_det;
    nc = o->fp32 ? o->f->n_comp : o->d->n_comp;
    rec = o->fp32 ? o->f->record : o->d->record;
    nmax = o->fp32 ? o->f->n_steps : o->d->n_steps;
    tr = o->fp32 ? o->f->trace : o->d->trace;
    ct = o->fp32 ? o->f->ctrace : o->d->ctrace;
    if (!rec) return FDTD2D_ERR_STATE;
    if (n0 < 1 || n1 < n0 || n1 > nmax) return FDTD2D_ERR_RANGE;
    for (n = n0; n <= n1; ++n) {
        for (e = 0; e < nd; ++e)
            if (det) det[(size_t)(n - n0) * nd + e] = tr[(size_t)(n - 1) * nd + e];
        for (e = 0; e < nc; ++e) {
            const float *src = ct + ((size_t)(n - 1) * nc + e) * 3;
            if (cez) cez[(size_t)(n - n0) * nc + e] = src[0];
            if (chx) chx[(size_t)(n - n0) * nc + e] = src[1];
            if (chy) chy[(size_t)(n - n0) * nc + e] = src[2];
        }
    }
    return FDTD2D_OK;
}

int oracle_read_dft(oracle *o, double *re, double *im) {
    int e, nd;
    if (!o || !re || !im) return FDTD2D_ERR_INVALID;
    nd = o->fp32 ? o->f->n_det : o->d->n_det;
    for (e = 0; e < nd; ++e) {
        re[e] = o->fp32 ? o->f->dft_re[e] : o->d->dft_re[e];
        im[e] = o->fp32 ? o->f->dft_im[e] : o->d->dft_im[e];
    }
    return FDTD2D_OK;
}

int oracle_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
