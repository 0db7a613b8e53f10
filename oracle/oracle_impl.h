/*
 * Body of the CPU oracle, included twice by oracle.c: once with REAL=double
 * (the FP64 parity oracle) and once with REAL=float (the FP32 restatement
 * timed as the CPU baseline).  TEST INFRASTRUCTURE ONLY: nothing in the
 * product links or calls this code.
 *
 * Every array is in the reference's own layout (FDTD_2D_Full/kernel.cu:1104-1220):
 *   Ez, Jz [ny][nx]   Hx [ny-1][nx]   Hy [ny][nx-1]
 *   psi_Ezx_{1,2} [ny][P]    psi_Hyx_{1,2} [ny][P-1]
 *   psi_Ezy_{1,2} [P][nx]    psi_Hxy_{1,2} [P-1][nx]
 * and each phase of a step is a separate loop over exactly the index range
 * of the reference kernel it restates, in the reference launch order
 * (FDTD_2D_Full/kernel.cu:2073-2157).
 */

typedef struct NAME(state) {
    int nx, ny, P, n_steps, step;
    int medium;
    REAL dt, dx, dy;
    REAL *ez, *hx, *hy, *jz;
    REAL *pezx1, *pezx2, *phyx1, *phyx2, *pezy1, *pezy2, *phxy1, *phxy2;
    REAL be_x_1[MAXP], ce_x_1[MAXP], be_x_2[MAXP], ce_x_2[MAXP];
    REAL bh_x_1[MAXP], ch_x_1[MAXP], bh_x_2[MAXP], ch_x_2[MAXP];
    REAL be_y_1[MAXP], ce_y_1[MAXP], be_y_2[MAXP], ce_y_2[MAXP];
    REAL bh_y_1[MAXP], ch_y_1[MAXP], bh_y_2[MAXP], ch_y_2[MAXP];
    REAL *den_ex, *den_hx, *den_ey, *den_hy;
    /* per-cell coefficients (uniform medium fills them from the scalars) */
    REAL *da1, *db1, *da2, *db2, *ca3, *cb3, *drive3;
    unsigned char *pec3;
    REAL jz_decay;
    /* source / detectors */
    int n_src, n_det, n_comp;
    int *src_i, *src_j, *det_i, *det_j, *comp_i, *comp_j;
    double *src_val;      /* [n_steps+1][n_src], FP64 */
    int record;
    float *trace, *ctrace;
    double *dft_re, *dft_im, dft_fdt;
    int dft;
    /* reference launch coverage (fdtd2d_setup.cover), material medium only */
    long long cov[8];
} NAME(state);

static void NAME(free_state)(NAME(state) *o) {
    if (!o) return;
    free(o->ez); free(o->hx); free(o->hy); free(o->jz);
    free(o->pezx1); free(o->pezx2); free(o->phyx1); free(o->phyx2);
    free(o->pezy1); free(o->pezy2); free(o->phxy1); free(o->phxy2);
    free(o->den_ex); free(o->den_hx); free(o->den_ey); free(o->den_hy);
    free(o->da1); free(o->db1); free(o->da2); free(o->db2);
    free(o->ca3); free(o->cb3); free(o->drive3); free(o->pec3);
    free(o->src_i); free(o->src_j); free(o->det_i); free(o->det_j);
    free(o->comp_i); free(o->comp_j); free(o->src_val);
    free(o->trace); free(o->ctrace); free(o->dft_re); free(o->dft_im);
    free(o);
}

static NAME(state) *NAME(create)(const fdtd2d_setup *s) {
    const int nx = s->nx, ny = s->ny, P = s->npml;
    const size_t cells = (size_t)nx * ny;
    NAME(state) *o;
    size_t c;
    int k, e, n;
    if (P < 2 || P > MAXP || nx < 2 * P + 2 || ny < 2 * P + 2) return NULL;
    o = (NAME(state) *)calloc(1, sizeof(*o));
    if (!o) return NULL;
    o->nx = nx; o->ny = ny; o->P = P; o->n_steps = s->n_steps; o->step = 0;
    for (k = 0; k < 8; ++k) {
        const long long v = s->cover[k];
        o->cov[k] = (s->medium != FDTD2D_MEDIUM_MATERIAL_ID || v == 0) ? LLONG_MAX : (v < 0 ? 0 : v);
    }
    o->medium = s->medium;
    o->dt = (REAL)s->dt;
    /* the psi kernels receive dx, dy as float arguments */
    o->dx = (REAL)(float)s->dx; o->dy = (REAL)(float)s->dy;
    o->ez = (REAL *)calloc(cells, sizeof(REAL));
    o->hx = (REAL *)calloc(cells, sizeof(REAL));
    o->hy = (REAL *)calloc(cells, sizeof(REAL));
    o->jz = (REAL *)calloc(cells, sizeof(REAL));
    o->pezx1 = (REAL *)calloc((size_t)ny * P, sizeof(REAL));
    o->pezx2 = (REAL *)calloc((size_t)ny * P, sizeof(REAL));
    o->phyx1 = (REAL *)calloc((size_t)ny * P, sizeof(REAL));
    o->phyx2 = (REAL *)calloc((size_t)ny * P, sizeof(REAL));
    o->pezy1 = (REAL *)calloc((size_t)nx * P, sizeof(REAL));
    o->pezy2 = (REAL *)calloc((size_t)nx * P, sizeof(REAL));
    o->phxy1 = (REAL *)calloc((size_t)nx * P, sizeof(REAL));
    o->phxy2 = (REAL *)calloc((size_t)nx * P, sizeof(REAL));
    o->den_ex = (REAL *)calloc(nx, sizeof(REAL));
    o->den_hx = (REAL *)calloc(nx, sizeof(REAL));
    o->den_ey = (REAL *)calloc(ny, sizeof(REAL));
    o->den_hy = (REAL *)calloc(ny, sizeof(REAL));
    o->da1 = (REAL *)calloc(cells, sizeof(REAL));
    o->db1 = (REAL *)calloc(cells, sizeof(REAL));
    o->da2 = (REAL *)calloc(cells, sizeof(REAL));
    o->db2 = (REAL *)calloc(cells, sizeof(REAL));
    o->ca3 = (REAL *)calloc(cells, sizeof(REAL));
    o->cb3 = (REAL *)calloc(cells, sizeof(REAL));
    o->drive3 = (REAL *)calloc(cells, sizeof(REAL));
    o->pec3 = (unsigned char *)calloc(cells, 1);
    if (!o->ez || !o->hx || !o->hy || !o->jz || !o->pezx1 || !o->pezx2 || !o->phyx1 || !o->phyx2 ||
        !o->pezy1 || !o->pezy2 || !o->phxy1 || !o->phxy2 || !o->den_ex || !o->den_hx ||
        !o->den_ey || !o->den_hy || !o->da1 || !o->db1 || !o->da2 || !o->db2 || !o->ca3 ||
        !o->cb3 || !o->drive3 || !o->pec3) {
        NAME(free_state)(o);
        return NULL;
    }
    for (k = 0; k < P; ++k) {
        o->be_x_1[k] = s->be_x_1[k]; o->ce_x_1[k] = s->ce_x_1[k];
        o->be_x_2[k] = s->be_x_2[k]; o->ce_x_2[k] = s->ce_x_2[k];
        o->be_y_1[k] = s->be_y_1[k]; o->ce_y_1[k] = s->ce_y_1[k];
        o->be_y_2[k] = s->be_y_2[k]; o->ce_y_2[k] = s->ce_y_2[k];
    }
    for (k = 0; k < P - 1; ++k) {
        o->bh_x_1[k] = s->bh_x_1[k]; o->ch_x_1[k] = s->ch_x_1[k];
        o->bh_x_2[k] = s->bh_x_2[k]; o->ch_x_2[k] = s->ch_x_2[k];
        o->bh_y_1[k] = s->bh_y_1[k]; o->ch_y_1[k] = s->ch_y_1[k];
        o->bh_y_2[k] = s->bh_y_2[k]; o->ch_y_2[k] = s->ch_y_2[k];
    }
    for (k = 0; k < nx - 1; ++k) { o->den_ex[k] = s->den_ex[k]; o->den_hx[k] = s->den_hx[k]; }
    for (k = 0; k < ny - 1; ++k) { o->den_ey[k] = s->den_ey[k]; o->den_hy[k] = s->den_hy[k]; }

    /* Jz update: Jz = a Jz + b ne Ez with a = (1 - nu dt/2)/(1 + nu dt/2),
       b = (e^2/m_e) dt / (1 + nu dt/2); at nu = 0 this is the reference's
       Jz += D_CJ Ez NE dt (FDTD_2D_Full/kernel.cu:156-157), applied only where
       NE > 0. */
    {
        const double half = 0.5 * s->nu * s->dt;
        const double beta = s->jz_coef * s->dt / (1.0 + half);
        o->jz_decay = (REAL)((1.0 - half) / (1.0 + half));
        for (c = 0; c < cells; ++c) {
            double ne;
            if (s->medium == FDTD2D_MEDIUM_MATERIAL_ID) {
                const int a = s->id1[c], b = s->id2[c], d = s->id3[c];
                if (a < 0 || b < 0 || d < 0 || a >= s->n_materials || b >= s->n_materials ||
                    d >= s->n_materials) {
                    NAME(free_state)(o);
                    return NULL;
                }
                o->da1[c] = s->mat_da[a]; o->db1[c] = s->mat_db[a];
                o->da2[c] = s->mat_da[b]; o->db2[c] = s->mat_db[b];
                o->ca3[c] = s->mat_ca[d]; o->cb3[c] = s->mat_cb[d];
                o->pec3[c] = (unsigned char)(d == 1);
                ne = s->mat_ne[d];
            } else {
                o->da1[c] = o->da2[c] = s->da;
                o->db1[c] = o->db2[c] = s->db;
                o->ca3[c] = s->ca; o->cb3[c] = s->cb;
                o->pec3[c] = 0;
                ne = s->ne ? s->ne[c] : 0.0;
            }
            o->drive3[c] = (REAL)(ne > 0 ? beta * ne : 0.0);
        }
    }

    o->n_src = s->n_src; o->n_det = s->n_det; o->n_comp = s->n_comp;
    o->src_i = (int *)calloc(s->n_src + 1, sizeof(int));
    o->src_j = (int *)calloc(s->n_src + 1, sizeof(int));
    o->det_i = (int *)calloc(s->n_det + 1, sizeof(int));
    o->det_j = (int *)calloc(s->n_det + 1, sizeof(int));
    o->comp_i = (int *)calloc(s->n_comp + 1, sizeof(int));
    o->comp_j = (int *)calloc(s->n_comp + 1, sizeof(int));
    for (e = 0; e < s->n_src; ++e) { o->src_i[e] = s->src[e].i; o->src_j[e] = s->src[e].j; }
    for (e = 0; e < s->n_det; ++e) { o->det_i[e] = s->det[e].i; o->det_j[e] = s->det[e].j; }
    for (e = 0; e < s->n_comp; ++e) { o->comp_i[e] = s->comp[e].i; o->comp_j[e] = s->comp[e].j; }

    /* Source waveform, FP64: s_e(n) = scale*env[n]*cos(2*pi_c*(beta/2 t^2 +
       f0 t + phase_e/360)), t = n dt (FDTD_2D_Full/kernel.cu:653, 694-698). */
    o->src_val = (double *)calloc((size_t)(s->n_steps + 1) * (s->n_src + 1), sizeof(double));
    if (s->n_src > 0) {
        const double pic = s->src_pi > 0 ? s->src_pi : ORACLE_PI;
        const double bh = (s->f1 != s->f0) ? 0.5 * (s->f1 - s->f0) / s->t1 : 0.0;
        for (n = 0; n <= s->n_steps; ++n) {
            const double t = (double)n * s->dt;
            for (e = 0; e < s->n_src; ++e) {
                double x = bh * t * t + s->f0 * t + s->src_phase_deg[e] / 360.0;
                double cs;
                if (pic == ORACLE_PI) {
                    x -= floor(x);
                    cs = cos(2.0 * ORACLE_PI * x);
                } else {
                    cs = cos(2.0 * pic * x);
                }
                o->src_val[(size_t)n * s->n_src + e] = s->src_scale * (double)s->envelope[n] * cs;
            }
        }
    }
    o->record = s->record_traces ? 1 : 0;
    if (o->record) {
        o->trace = (float *)calloc((size_t)s->n_steps * (s->n_det + 1), sizeof(float));
        o->ctrace = (float *)calloc((size_t)s->n_steps * (s->n_comp + 1) * 3, sizeof(float));
    }
    o->dft = (s->dft_freq > 0 && s->n_det > 0);
    o->dft_fdt = s->dft_freq * s->dt;
    o->dft_re = (double *)calloc(s->n_det + 1, sizeof(double));
    o->dft_im = (double *)calloc(s->n_det + 1, sizeof(double));
    return o;
}

/* One full step n (1-based). */
static void NAME(step)(NAME(state) *o, int n) {
    const int nx = o->nx, ny = o->ny, P = o->P;
    const int hyp = nx - 1;        /* Hy row pitch */
    REAL *ez = o->ez, *hx = o->hx, *hy = o->hy, *jz = o->jz;
    int i, j, e;

    /* Dev_HxCalc (kernel.cu:167-196): i in [0,nx-2], j in [0,ny-2] */
#pragma omp parallel for private(i) schedule(static)
    for (j = 0; j <= ny - 2; ++j)
        for (i = 0; i <= nx - 2; ++i) {
            const size_t c = (size_t)j * nx + i;
            if ((long long)j * (nx - 1) + i >= o->cov[0]) continue;
            hx[c] = o->da1[c] * hx[c] + o->db1[c] * ((ez[c] - ez[c + nx]) * o->den_hy[j]);
        }
    /* Dev_HxPML_Jdir_Calc (kernel.cu:198-240): j in [0,P-2], mirror jj = ny-2-j */
#pragma omp parallel for private(i) schedule(static)
    for (j = 0; j <= P - 2; ++j)
        for (i = 0; i <= nx - 2; ++i) {
            const int jj = ny - 2 - j;
            const size_t c1 = (size_t)j * nx + i, c2 = (size_t)jj * nx + i, p = (size_t)j * nx + i;
            if ((long long)j * (nx - 1) + i >= o->cov[1]) continue;
            o->phxy1[p] = o->bh_y_1[j] * o->phxy1[p] + o->ch_y_1[j] * (ez[c1] - ez[c1 + nx]) / o->dy;
            hx[c1] = hx[c1] + o->db1[c1] * o->phxy1[p];
            o->phxy2[p] = o->bh_y_2[j] * o->phxy2[p] + o->ch_y_2[j] * (ez[c2] - ez[c2 + nx]) / o->dy;
            hx[c2] = hx[c2] + o->db1[c2] * o->phxy2[p];
        }
    /* Dev_HyCalc (kernel.cu:288-318) */
#pragma omp parallel for private(i) schedule(static)
    for (j = 0; j <= ny - 2; ++j)
        for (i = 0; i <= nx - 2; ++i) {
            const size_t c = (size_t)j * nx + i, h = (size_t)j * hyp + i;
            if ((long long)j * (nx - 1) + i >= o->cov[2]) continue;
            hy[h] = o->da2[c] * hy[h] + o->db2[c] * ((ez[c + 1] - ez[c]) * o->den_hx[i]);
        }
    /* Dev_HyPML_Idir_Calc (kernel.cu:321-362): i in [0,P-2], mirror ii = nx-2-i */
#pragma omp parallel for private(i) schedule(static)
    for (j = 0; j <= ny - 2; ++j)
        for (i = 0; i <= P - 2; ++i) {
            const int ii = nx - 2 - i;
            const size_t c1 = (size_t)j * nx + i, c2 = (size_t)j * nx + ii;
            const size_t p = (size_t)j * (P - 1) + i;
            if ((long long)j * (P - 1) + i >= o->cov[3]) continue;
            o->phyx1[p] = o->bh_x_1[i] * o->phyx1[p] + o->ch_x_1[i] * (ez[c1 + 1] - ez[c1]) / o->dx;
            hy[(size_t)j * hyp + i] = hy[(size_t)j * hyp + i] + o->db2[c1] * o->phyx1[p];
            o->phyx2[p] = o->bh_x_2[i] * o->phyx2[p] + o->ch_x_2[i] * (ez[c2 + 1] - ez[c2]) / o->dx;
            hy[(size_t)j * hyp + ii] = hy[(size_t)j * hyp + ii] + o->db2[c2] * o->phyx2[p];
        }
    /* Dev_JzCalc (kernel.cu:127-163), Drude form */
#pragma omp parallel for private(i) schedule(static)
    for (j = 1; j <= ny - 2; ++j)
        for (i = 1; i <= nx - 2; ++i) {
            const size_t c = (size_t)j * nx + i;
            if ((long long)(j - 1) * (nx - 2) + (i - 1) >= o->cov[4]) continue;
            if (o->drive3[c] > 0) jz[c] = o->jz_decay * jz[c] + o->drive3[c] * ez[c];
        }
    /* Dev_EzCalc (kernel.cu:413-451) */
#pragma omp parallel for private(i) schedule(static)
    for (j = 1; j <= ny - 2; ++j)
        for (i = 1; i <= nx - 2; ++i) {
            const size_t c = (size_t)j * nx + i, h = (size_t)j * hyp + i;
            if ((long long)(j - 1) * (nx - 2) + (i - 1) >= o->cov[5]) continue;
            if (o->pec3[c]) {
                ez[c] = 0;
            } else {
                ez[c] = o->ca3[c] * ez[c] +
                        o->cb3[c] * ((hy[h] - hy[h - 1]) * o->den_ex[i] +
                                     (hx[c - nx] - hx[c]) * o->den_ey[j] - jz[c]);
            }
        }
    /* Dev_EzPML_Idir_Calc (kernel.cu:453-494): i in [1,P-1], mirror ii = nx-1-i */
#pragma omp parallel for private(i) schedule(static)
    for (j = 1; j <= ny - 2; ++j)
        for (i = 1; i <= P - 1; ++i) {
            const int ii = nx - 1 - i;
            const size_t c1 = (size_t)j * nx + i, c2 = (size_t)j * nx + ii, p = (size_t)j * P + i;
            const size_t h1 = (size_t)j * hyp + i, h2 = (size_t)j * hyp + ii;
            if ((long long)(j - 1) * (P - 1) + (i - 1) >= o->cov[6]) continue;
            o->pezx1[p] = o->be_x_1[i] * o->pezx1[p] + o->ce_x_1[i] * (hy[h1] - hy[h1 - 1]) / o->dx;
            ez[c1] = ez[c1] + o->cb3[c1] * o->pezx1[p];
            o->pezx2[p] = o->be_x_2[i] * o->pezx2[p] + o->ce_x_2[i] * (hy[h2] - hy[h2 - 1]) / o->dx;
            ez[c2] = ez[c2] + o->cb3[c2] * o->pezx2[p];
        }
    /* Dev_EzPML_Jdir_Calc (kernel.cu:496-537): j in [1,P-1], mirror jj = ny-1-j */
#pragma omp parallel for private(i) schedule(static)
    for (j = 1; j <= P - 1; ++j)
        for (i = 1; i <= nx - 2; ++i) {
            const int jj = ny - 1 - j;
            const size_t c1 = (size_t)j * nx + i, c2 = (size_t)jj * nx + i, p = (size_t)j * nx + i;
            if ((long long)(j - 1) * (nx - 2) + (i - 1) >= o->cov[7]) continue;
            o->pezy1[p] = o->be_y_1[j] * o->pezy1[p] + o->ce_y_1[j] * (hx[c1 - nx] - hx[c1]) / o->dy;
            ez[c1] = ez[c1] + o->cb3[c1] * o->pezy1[p];
            o->pezy2[p] = o->be_y_2[j] * o->pezy2[p] + o->ce_y_2[j] * (hx[c2 - nx] - hx[c2]) / o->dy;
            ez[c2] = ez[c2] + o->cb3[c2] * o->pezy2[p];
        }
    /* Dev_AESASourceCalc (kernel.cu:621-659): soft source after the E update */
    for (e = 0; e < o->n_src; ++e) {
        const size_t c = (size_t)o->src_j[e] * nx + o->src_i[e];
        ez[c] = ez[c] - (REAL)o->src_val[(size_t)n * o->n_src + e];
    }
    /* Dev_AESADetectorSim / Dev_AESAComponentDetector (kernel.cu:719-805) */
    for (e = 0; e < o->n_det; ++e) {
        const REAL v = ez[(size_t)o->det_j[e] * nx + o->det_i[e]];
        if (o->record) o->trace[(size_t)(n - 1) * o->n_det + e] = (float)v;
        if (o->dft) {
            double ph = o->dft_fdt * (double)n;
            ph -= floor(ph);
            o->dft_re[e] += (double)v * cos(2.0 * ORACLE_PI * ph);
            o->dft_im[e] -= (double)v * sin(2.0 * ORACLE_PI * ph);
        }
    }
    if (o->record) {
        for (e = 0; e < o->n_comp; ++e) {
            const size_t c = (size_t)o->comp_j[e] * nx + o->comp_i[e];
            float *dst = o->ctrace + ((size_t)(n - 1) * o->n_comp + e) * 3;
            dst[0] = (float)ez[c];
            dst[1] = (float)hx[c];
            dst[2] = (float)hy[(size_t)o->comp_j[e] * hyp + o->comp_i[e]];
        }
    }
    o->step = n;
}

/* Field access in the reference layout (fdtd2d.h FDTD2D_FIELD_*). */
static REAL *NAME(field)(NAME(state) *o, int which, int *rows, int *cols) {
    const int nx = o->nx, ny = o->ny, P = o->P;
    switch (which) {
    case FDTD2D_FIELD_EZ: *rows = ny; *cols = nx; return o->ez;
    case FDTD2D_FIELD_JZ: *rows = ny; *cols = nx; return o->jz;
    case FDTD2D_FIELD_HX: *rows = ny - 1; *cols = nx; return o->hx;
    case FDTD2D_FIELD_HY: *rows = ny; *cols = nx - 1; return o->hy;
    case FDTD2D_FIELD_PSI_EZX_1: *rows = ny; *cols = P; return o->pezx1;
    case FDTD2D_FIELD_PSI_EZX_2: *rows = ny; *cols = P; return o->pezx2;
    case FDTD2D_FIELD_PSI_HYX_1: *rows = ny; *cols = P - 1; return o->phyx1;
    case FDTD2D_FIELD_PSI_HYX_2: *rows = ny; *cols = P - 1; return o->phyx2;
    case FDTD2D_FIELD_PSI_EZY_1: *rows = P; *cols = nx; return o->pezy1;
    case FDTD2D_FIELD_PSI_EZY_2: *rows = P; *cols = nx; return o->pezy2;
    case FDTD2D_FIELD_PSI_HXY_1: *rows = P - 1; *cols = nx; return o->phxy1;
    case FDTD2D_FIELD_PSI_HXY_2: *rows = P - 1; *cols = nx; return o->phxy2;
    default: return NULL;
    }
}
