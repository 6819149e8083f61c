/* Host geometry routines of csrc/rtm_host.c (extend_matrix, the CPML profiles) over
 * minimum-size and asymmetric geometries, built with AddressSanitizer and UBSan by
 * tests/test_capi_host.py; exit status 0 when they stay in bounds. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "rtm_gpu.h"

int main(void)
{
    const int th[][4] = {{12, 12, 12, 12}, {12, 30, 17, 50}, {50, 50, 50, 50}, {40, 13, 64, 12}};
    const int dims[][2] = {{1, 1}, {5, 3}, {37, 29}, {400, 200}};
    for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b) {
            rtm_params p;
            memset(&p, 0, sizeof p);
            p.nx = dims[b][0]; p.nz = dims[b][1];
            p.th_left = th[a][0]; p.th_right = th[a][1]; p.th_up = th[a][2]; p.th_down = th[a][3];
            p.dx = 10.0f; p.dt = 1e-3f; p.nt = 20; p.n_wavelet = 10; p.time_slices = 20;
            p.rec_count = 1; p.rec_spacing = 2;
            const int dx = p.th_left + p.nx + p.th_right, dz = p.th_up + p.nz + p.th_down;
            float *model = malloc(sizeof(float) * p.nx * p.nz), *ext = malloc(sizeof(float) * dx * dz);
            for (int i = 0; i < p.nx * p.nz; ++i) model[i] = (float)i;
            rtm_extend_matrix(&p, ext, model);
            float *pr[8];
            const int len[8] = {p.th_left, p.th_right, p.th_up, p.th_down, p.th_left, p.th_right, p.th_up, p.th_down};
            for (int k = 0; k < 8; ++k) pr[k] = malloc(sizeof(float) * len[k]);
            rtm_attenuation_profile_cpml(&p, pr[0], pr[1], pr[2], pr[3], pr[4], pr[5], pr[6], pr[7]);
            for (int k = 0; k < 8; ++k) free(pr[k]);
            free(model); free(ext);
        }
    return 0;
}
