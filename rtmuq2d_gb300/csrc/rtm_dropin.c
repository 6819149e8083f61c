/*
 * rtm_dropin.c -- the reference's entry points (include/rtm_dropin.h) over the engine's C
 * ABI.  Built into librtm_dropin.so, which links librtmgpu.so; kept out of librtmgpu so the
 * reference's generic names (extend_matrix, reading_file, ...) enter a process only when a
 * program asks for them.
 *
 * Every entry point uses the configuration set by rtm_dropin_configure; calling one before
 * that is a usage error and exits like the reference's failures do.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "rtm_dropin.h"

#define DROPIN_PATH_LEN 4096

static rtm_params g_p;
static rtm_survey g_s;
static char g_paths[6][DROPIN_PATH_LEN];
static int g_configured = 0;

static void die(const char *what)
{
    fprintf(stderr, "\nrtm drop-in: %s: %s\n", what, rtm_last_error());
    exit(1);
}

static const rtm_params *cfg(void)
{
    if (!g_configured) {
        fprintf(stderr, "\nrtm drop-in: rtm_dropin_configure() was not called\n");
        exit(1);
    }
    return &g_p;
}

static const char *keep(int k, const char *s)
{
    if (!s) return NULL;
    snprintf(g_paths[k], DROPIN_PATH_LEN, "%s", s);
    return g_paths[k];
}

int rtm_dropin_configure(const rtm_params *p, const rtm_survey *survey)
{
    if (!p || !survey) return RTM_ERR_INVALID;
    g_p = *p;
    g_s = *survey;
    g_s.velocity_file = keep(0, survey->velocity_file);
    g_s.wavelet_file = keep(1, survey->wavelet_file);
    g_s.seismogram_file = keep(2, survey->seismogram_file);
    g_s.stacked_file = keep(3, survey->stacked_file);
    g_s.laplacian_file = keep(4, survey->laplacian_file);
    g_s.checkpoint_file = keep(5, survey->checkpoint_file);
    g_configured = 1;
    return RTM_OK;
}

/* rtm_iso2d.c:15 */
void rtm_routine(int simulationId)
{
    if (rtm_routine_run(cfg(), &g_s, simulationId) != RTM_OK) die("rtm_routine");
}

/* forward_modeling.c:12 */
void isotropicAcousticModeling(int simId, int *shot, float *velocity, float *wavelet)
{
    rtm_params p = *cfg();
    p.shot_x = shot[0];
    p.shot_z = shot[1];
    if (rtm_forward_modeling(&p, simId, shot, velocity, wavelet) != RTM_OK)
        die("isotropicAcousticModeling");
}

/* backward_modeling.c:12; returns 1 like the reference */
int adjointModeling(int simId, int *shot, float *velocity, float *wavelet, float *seismogram,
                    float *imageCondition, float *selfImageCondition)
{
    rtm_params p = *cfg();
    p.shot_x = shot[0];
    p.shot_z = shot[1];
    if (rtm_adjoint_modeling(&p, simId, shot, velocity, wavelet, seismogram, imageCondition,
                             selfImageCondition) != RTM_OK)
        die("adjointModeling");
    return 1;
}

/* compression_tools.c:78: 0 on success, 1 on a failed decode */
int zfp2d_lossyDecompression(char *zfp_data_02, float *array, int dimension1, int dimension2,
                             float tolerance)
{
    const int st = rtm_zfp_decode_file(zfp_data_02, array, dimension1, dimension2, tolerance);
    if (st == RTM_ERR_IO) die("zfp2d_lossyDecompression: cannot read the stream");
    if (st != RTM_OK) {
        fprintf(stderr, "Decompression Failed\n");
        return 1;
    }
    return 0;
}

/* compression_tools.c:10-71: the stream zfp_compress writes for the field (dimension1 fastest)
 * at this accuracy, in a malloc'ed buffer of the library's maximum size */
int zfp2d_lossyCompression(void **compression, float *array, int dimension1, int dimension2, float tolerance)
{
    *compression = NULL;
    const size_t cap = rtm_zfp_encode_bound(dimension1, dimension2);
    void *buf = malloc(cap > 0 ? cap : 1);
    if (!buf) return 0;
    size_t used = 0;
    if (rtm_zfp_encode_float2d(array, dimension1, dimension2, tolerance, buf, cap, &used) != RTM_OK) {
        free(buf);
        return 0;
    }
    *compression = buf;
    return (int)used;
}

/* image_conditions.c:8: the image only (the self image goes to a scratch buffer) */
void cross_correlation(float *imageCondition, float *sourceWavefield, float *receiverWavefield)
{
    const rtm_params *p = cfg();
    float *scratch = (float *)calloc((size_t)p->nx * (size_t)p->nz, sizeof(float));
    if (!scratch) die("cross_correlation: out of host memory");
    const int st = rtm_normalized_cross_correlation(p, imageCondition, scratch, sourceWavefield,
                                                    receiverWavefield);
    free(scratch);
    if (st != RTM_OK) die("cross_correlation");
}

/* image_conditions.c:20 */
void normalized_cross_correlation(float *imageCondition, float *selfImageCondition,
                                  float *sourceWavefield, float *receiverWavefield)
{
    if (rtm_normalized_cross_correlation(cfg(), imageCondition, selfImageCondition, sourceWavefield,
                                         receiverWavefield) != RTM_OK)
        die("normalized_cross_correlation");
}

/* stencilDFM.c:7 */
void iso_acoustic_wave_equation(float *pond, float *waveField2, float *waveField3)
{
    if (rtm_iso_acoustic_wave_equation(cfg(), pond, waveField2, waveField3) != RTM_OK)
        die("iso_acoustic_wave_equation");
}

/* absorbingBoundaryCondition.c:11 */
void attenuation_profile_cpml(float *a_Left, float *a_Right, float *a_Top, float *a_Bottom,
                              float *b_Left, float *b_Right, float *b_Top, float *b_Bottom)
{
    rtm_attenuation_profile_cpml(cfg(), a_Left, a_Right, a_Top, a_Bottom, b_Left, b_Right, b_Top,
                                 b_Bottom);
}

/* absorbingBoundaryCondition.c:150 */
void aiso_attenuation_cpml(float *waveField1, float *waveField2, float *Coef, float *a_left,
                           float *b_left, float *a_right, float *b_right, float *a_top,
                           float *b_top, float *a_bottom, float *b_bottom, float *psi_borderLeft,
                           float *psi_borderRight, float *psi_borderTop, float *psi_borderBottom,
                           float *csi_borderLeft, float *csi_borderRight, float *csi_borderTop,
                           float *csi_borderBottom)
{
    if (rtm_aiso_attenuation_cpml(cfg(), waveField1, waveField2, Coef, a_left, b_left, a_right, b_right,
                                  a_top, b_top, a_bottom, b_bottom, psi_borderLeft, psi_borderRight,
                                  psi_borderTop, psi_borderBottom, csi_borderLeft, csi_borderRight,
                                  csi_borderTop, csi_borderBottom) != RTM_OK)
        die("aiso_attenuation_cpml");
}

/* generic_functions.c:5 */
void extend_matrix(float *extendedModel, float *model)
{
    rtm_extend_matrix(cfg(), extendedModel, model);
}

/* math_functions.c:9 */
void laplacian_filter2D(float *lp, float *inputMatrix)
{
    if (rtm_laplacian_filter2D(cfg(), lp, inputMatrix) != RTM_OK) die("laplacian_filter2D");
}

/* pi_file.c:11: exits on a missing file or a short read, like the reference */
int reading_file(char *path, float *matrix, int dim1, int dim2)
{
    FILE *f = fopen(path, "rb");
    if (!f) {
        printf("\nError oppening file (fopen in reading_file function)\n");
        exit(1);
    }
    const size_t n = (size_t)dim1 * (size_t)dim2;
    const size_t got = fread(matrix, sizeof(float), n, f);
    fclose(f);
    if (got != n) {
        printf("\nError reading file (fread in reading_file function)\n");
        exit(1);
    }
    return 0;
}

/* pi_file.c:37 */
int recording_file(char *path, float *matrix, int dim1, int dim2)
{
    FILE *f = fopen(path, "wb");
    if (!f) {
        printf("\nError oppening file (fopen in recording_file function)\n");
        exit(1);
    }
    const size_t n = (size_t)dim1 * (size_t)dim2;
    const size_t put = fwrite(matrix, sizeof(float), n, f);
    fclose(f);
    if (put != n) {
        printf("\nError reading file (fread in recording_file function)\n");
        exit(1);
    }
    return 0;
}
