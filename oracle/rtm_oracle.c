/*
 * rtm_oracle.c -- CPU restatement of rtmUq2D's migration path (TEST INFRASTRUCTURE).
 *
 * This file is the oracle: what the CUDA engine's results are compared with, and the timed CPU
 * baseline.  It is never part of the product library.  See rtm_oracle.h for the
 * routine-by-routine map to the reference sources.
 */
#include <math.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "rtm_oracle.h"

/* 8th-order second-derivative weights -- SRC/stencilDFM.h:8-12 */
#define ORC_AC0 (-2.97399944f)
#define ORC_AC1 (+1.70507669f)
#define ORC_AC2 (-0.25861812f)
#define ORC_AC3 (+0.04577745f)
#define ORC_AC4 (-0.00523630f)
/* 8th-order first-derivative weights -- SRC/absorbingBoundaryCondition.h:21-24 */
#define ORC_B1 (+0.8f)
#define ORC_B2 (-0.2f)
#define ORC_B3 (+0.025396825f)
#define ORC_B4 (-0.001785714f)

#define ORC_MAX_THICK 512

int orc_dim_x(const orc_params *p) { return p->th_left + p->nx + p->th_right; }
int orc_dim_z(const orc_params *p) { return p->th_up + p->nz + p->th_down; }

void orc_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int orc_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/*
 * Edge replication of the Nx x Nz model into the CPML -- SRC/generic_functions.c:5-48.
 * Order and bounds are the reference's, including the right-pad loop whose z bound is
 * Nz + th_down (:27), which only covers the model rows when th_up == th_down.
 * ext is zeroed first (the reference's caller callocs it).
 */
void orc_extend_matrix(const orc_params *p, float *ext, const float *model)
{
    const int dimx = orc_dim_x(p), dimz = orc_dim_z(p);
    const int nx = p->nx, nz = p->nz, thl = p->th_left, thr = p->th_right;
    const int thu = p->th_up, thd = p->th_down;
    memset(ext, 0, (size_t)dimx * dimz * sizeof(float));
    for (int i = 0; i < nx; i++)
        for (int k = 0; k < nz; k++)
            ext[(size_t)(i + thl) * dimz + (k + thu)] = model[(size_t)i * nz + k];
    for (int i = 0; i < thl; i++)
        for (int k = thu; k < nz + thu; k++)
            ext[(size_t)i * dimz + k] = ext[(size_t)thl * dimz + k];
    for (int i = nx + thl; i < nx + thl + thr; i++)
        for (int k = thu; k < nz + thd; k++)
            ext[(size_t)i * dimz + k] = ext[(size_t)(nx + thl - 1) * dimz + k];
    for (int i = 0; i < dimx; i++)
        for (int k = 0; k < thu; k++)
            ext[(size_t)i * dimz + k] = ext[(size_t)i * dimz + thu];
    for (int i = 0; i < dimx; i++)
        for (int k = nz + thu; k < dimz; k++)
            ext[(size_t)i * dimz + k] = ext[(size_t)i * dimz + (nz + thu - 1)];
}

/*
 * CPML damping profiles -- SRC/absorbingBoundaryCondition.c:11-148, float arithmetic as
 * there: sigma = sigma_max * d^2 with sigma_max from the LEFT thickness for every side
 * (:65), alpha = alpha_max*(1-d) + 0.1*alpha_max, b = e^{-(sigma+alpha) dt},
 * a = sigma (b-1)/(sigma+alpha).  Left/top run d from 1 at cell 4 down to 1/(th-8);
 * right/bottom are indexed from the inner edge, d = (1+j)/(th-8) at cell 4+j (:93-100).
 * Entries outside [4, th-4) stay 0.
 */
void orc_cpml_profile(const orc_params *p, float *a_l, float *a_r, float *a_t, float *a_b,
                      float *b_l, float *b_r, float *b_t, float *b_b)
{
    const float pi = (float)M_PI;
    const float att = 3.0f * pi;
    const float vmax = 4000.0f;
    const float fcut = 60.0f;
    const float e = (float)M_E;
    const float dx = p->dx, dt = p->dt;
    const float f0 = (float)(fcut / (3.0f * sqrt(pi)));
    const float len_l = (float)(p->th_left - 8) * dx;
    const float len_r = (float)(p->th_right - 8) * dx;
    const float len_t = (float)(p->th_up - 8) * dx;
    const float len_b = (float)(p->th_down - 8) * dx;
    const float smax = att * (((2.0f + 1.0f) * vmax) / len_l);
    const float amax = pi * f0;

    memset(a_l, 0, p->th_left * sizeof(float));  memset(b_l, 0, p->th_left * sizeof(float));
    memset(a_r, 0, p->th_right * sizeof(float)); memset(b_r, 0, p->th_right * sizeof(float));
    memset(a_t, 0, p->th_up * sizeof(float));    memset(b_t, 0, p->th_up * sizeof(float));
    memset(a_b, 0, p->th_down * sizeof(float));  memset(b_b, 0, p->th_down * sizeof(float));

    for (int i = 4; i < p->th_left - 4; i++) {
        const float d = (len_l - dx * (float)(i - 4)) / len_l;
        const float sg = smax * powf(d, 2.0f);
        const float al = amax * (1.0f - d) + 0.1f * amax;
        b_l[i] = powf(e, -(sg + al) * dt);
        a_l[i] = sg * (b_l[i] - 1.0f) / (sg + al);
    }
    for (int j = 0; j < p->th_right - 8; j++) {
        const float d = (dx + dx * (float)j) / len_r;
        const float sg = smax * powf(d, 2.0f);
        const float al = amax * (1.0f - d) + 0.1f * amax;
        b_r[j + 4] = powf(e, -(sg + al) * dt);
        a_r[j + 4] = sg * (b_r[j + 4] - 1.0f) / (sg + al);
    }
    for (int k = 4; k < p->th_up - 4; k++) {
        const float d = (len_t - dx * (float)(k - 4)) / len_t;
        const float sg = smax * powf(d, 2.0f);
        const float al = amax * (1.0f - d) + 0.1f * amax;
        b_t[k] = powf(e, -(sg + al) * dt);
        a_t[k] = sg * (b_t[k] - 1.0f) / (sg + al);
    }
    for (int j = 0; j < p->th_down - 8; j++) {
        const float d = (dx + dx * (float)j) / len_b;
        const float sg = smax * powf(d, 2.0f);
        const float al = amax * (1.0f - d) + 0.1f * amax;
        b_b[j + 4] = powf(e, -(sg + al) * dt);
        a_b[j + 4] = sg * (b_b[j + 4] - 1.0f) / (sg + al);
    }
}

/* 8th-order Laplacian of an Nx x Nz image, no 1/dx^2, 4-cell border untouched --
 * SRC/math_functions.c:9-27 */
void orc_laplacian(const orc_params *p, float *lp, const float *in)
{
    const int nx = p->nx, nz = p->nz;
    const float c0 = 2.0f * ORC_AC0;
    int i;
#pragma omp parallel for schedule(static)
    for (i = 4; i < nx - 4; i++) {
        const float *c = in + (size_t)i * nz;
        for (int k = 4; k < nz - 4; k++)
            lp[(size_t)i * nz + k] = c0 * c[k]
                + ORC_AC1 * (c[k - nz] + c[k + nz] + c[k - 1] + c[k + 1])
                + ORC_AC2 * (c[k - 2 * nz] + c[k + 2 * nz] + c[k - 2] + c[k + 2])
                + ORC_AC3 * (c[k - 3 * nz] + c[k + 3 * nz] + c[k - 3] + c[k + 3])
                + ORC_AC4 * (c[k - 4 * nz] + c[k + 4 * nz] + c[k - 4] + c[k + 4]);
    }
}

#define REAL float
#define SFX(name) name##_f
#include "rtm_oracle_core.inc"
#undef REAL
#undef SFX

#define REAL double
#define SFX(name) name##_d
#include "rtm_oracle_core.inc"
#undef REAL
#undef SFX
