/*
 * rtm_host.c -- host-side set-up of the RTM engine (plain C, built with gcc).
 *
 *   rtm_attenuation_profile_cpml   SRC/absorbingBoundaryCondition.c:11-148
 *   rtm_extend_matrix              SRC/generic_functions.c:5-48
 *
 * Both run once per migration on the host, in float, with the reference's formulas and
 * evaluation order, so the damping profiles the GPU uses equal the reference's bit for
 * bit on the same machine (built with -ffp-contract=off).
 */
#include <math.h>
#include <string.h>

#include "rtm_gpu.h"

/*
 * CPML profiles.  d is the normalised distance into the layer; sigma = sigma_max d^2
 * (NPOWER = 2, absorbingBoundaryCondition.h:5) with sigma_max = 3 pi * 3 v_max / L_left
 * for all four sides (:65), alpha = alpha_max (1 - d) + 0.1 alpha_max with
 * alpha_max = pi f0, f0 = 60 / (3 sqrt(pi)) (:43,56,67), b = e^{-(sigma+alpha) dt},
 * a = sigma (b - 1) / (sigma + alpha).  L = (thickness - 8) dx (:59-62).  Left/top count
 * d down from 1 at cell 4; right/bottom count it up from 1/(th-8) at cell 4 (:90-103).
 */
void rtm_attenuation_profile_cpml(const rtm_params *p, float *a_l, float *a_r, float *a_t,
                                  float *a_b, float *b_l, float *b_r, float *b_t, float *b_b)
{
    const float pi = (float)M_PI;
    const float kappa = 3.0f * pi;      /* attenuationCoef */
    const float vmax = 4000.0f;
    const float fcut = 60.0f;
    const float euler = (float)M_E;
    const float h = p->dx, dt = p->dt;
    const float f0 = (float)(fcut / (3.0f * sqrt(pi)));
    const float len_l = (float)(p->th_left - 8) * h;
    const float len_r = (float)(p->th_right - 8) * h;
    const float len_t = (float)(p->th_up - 8) * h;
    const float len_b = (float)(p->th_down - 8) * h;
    const float sig_max = kappa * (((2.0f + 1.0f) * vmax) / len_l);
    const float alf_max = pi * f0;
    int n;

    memset(a_l, 0, (size_t)p->th_left * sizeof(float));
    memset(b_l, 0, (size_t)p->th_left * sizeof(float));
    memset(a_r, 0, (size_t)p->th_right * sizeof(float));
    memset(b_r, 0, (size_t)p->th_right * sizeof(float));
    memset(a_t, 0, (size_t)p->th_up * sizeof(float));
    memset(b_t, 0, (size_t)p->th_up * sizeof(float));
    memset(a_b, 0, (size_t)p->th_down * sizeof(float));
    memset(b_b, 0, (size_t)p->th_down * sizeof(float));

    for (n = 4; n < p->th_left - 4; n++) {
        const float d = (len_l - h * (float)(n - 4)) / len_l;
        const float sg = sig_max * powf(d, 2.0f);
        const float al = alf_max * (1.0f - d) + 0.1f * alf_max;
        b_l[n] = powf(euler, -(sg + al) * dt);
        a_l[n] = sg * (b_l[n] - 1.0f) / (sg + al);
    }
    for (n = 0; n < p->th_right - 8; n++) {
        const float d = (h + h * (float)n) / len_r;
        const float sg = sig_max * powf(d, 2.0f);
        const float al = alf_max * (1.0f - d) + 0.1f * alf_max;
        b_r[n + 4] = powf(euler, -(sg + al) * dt);
        a_r[n + 4] = sg * (b_r[n + 4] - 1.0f) / (sg + al);
    }
    for (n = 4; n < p->th_up - 4; n++) {
        const float d = (len_t - h * (float)(n - 4)) / len_t;
        const float sg = sig_max * powf(d, 2.0f);
        const float al = alf_max * (1.0f - d) + 0.1f * alf_max;
        b_t[n] = powf(euler, -(sg + al) * dt);
        a_t[n] = sg * (b_t[n] - 1.0f) / (sg + al);
    }
    for (n = 0; n < p->th_down - 8; n++) {
        const float d = (h + h * (float)n) / len_b;
        const float sg = sig_max * powf(d, 2.0f);
        const float al = alf_max * (1.0f - d) + 0.1f * alf_max;
        b_b[n + 4] = powf(euler, -(sg + al) * dt);
        a_b[n + 4] = sg * (b_b[n + 4] - 1.0f) / (sg + al);
    }
}

/*
 * Pads an nx x nz model with the CPML by edge replication: interior copy, left, right,
 * top, bottom, in that order.  The right pad's z bound is nz + th_down as in the
 * reference (:27), which equals the model rows only when th_up == th_down; the same
 * cells are produced for any thicknesses.  `ext` is zeroed first.
 */
void rtm_extend_matrix(const rtm_params *p, float *ext, const float *model)
{
    const int nx = p->nx, nz = p->nz;
    const int l = p->th_left, r = p->th_right, u = p->th_up, d = p->th_down;
    const int dz = u + nz + d, dxx = l + nx + r;
    int i, k;
    memset(ext, 0, (size_t)dxx * dz * sizeof(float));
    for (i = 0; i < nx; i++)
        memcpy(ext + (size_t)(i + l) * dz + u, model + (size_t)i * nz, (size_t)nz * sizeof(float));
    for (i = 0; i < l; i++)
        for (k = u; k < nz + u; k++) ext[(size_t)i * dz + k] = ext[(size_t)l * dz + k];
    for (i = nx + l; i < dxx; i++)
        for (k = u; k < nz + d; k++) ext[(size_t)i * dz + k] = ext[(size_t)(nx + l - 1) * dz + k];
    for (i = 0; i < dxx; i++)
        for (k = 0; k < u; k++) ext[(size_t)i * dz + k] = ext[(size_t)i * dz + u];
    for (i = 0; i < dxx; i++)
        for (k = nz + u; k < dz; k++) ext[(size_t)i * dz + k] = ext[(size_t)i * dz + nz + u - 1];
}
