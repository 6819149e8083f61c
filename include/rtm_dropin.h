/*
 * rtm_dropin.h -- the reference's own entry points of the migration path, with the
 * reference's names and signatures, served by the GB300 engine (librtm_dropin.so, which
 * links librtmgpu.so).  A program written against rtmUq2D's SRC/ headers links this
 * library instead of the reference's forward_modeling.c, backward_modeling.c,
 * image_conditions.c, stencilDFM.c, absorbingBoundaryCondition.c, generic_functions.c,
 * math_functions.c, compression_tools.c (decode) and rtm_iso2d.c.
 *
 * The reference takes its sizes from SRC/fixed_parameters.h at compile time; the library
 * takes them once at run time through rtm_dropin_configure().  A translation unit that
 * includes the reference's fixed_parameters.h (and forward_modeling.h for TIME_SLICES)
 * before this header gets rtm_dropin_configure_from_fixed_parameters(), which fills both
 * structures from those constants: call it once at the top of main().
 *
 * Observable behaviour kept: the same argument meaning and order, images accumulated into
 * caller buffers, adjointModeling returns 1, and the process exits with status 1 where
 * the reference exits (unreadable inputs, failed propagation); the message comes from the
 * engine (rtm_last_error).
 */
#ifndef RTM_DROPIN_H
#define RTM_DROPIN_H

#include "rtm_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Sizes and file contracts for every entry point below (copied; strings too). */
int rtm_dropin_configure(const rtm_params *p, const rtm_survey *survey);

void rtm_routine(int simulationId);                                              /* rtm_iso2d.h:11 */
void isotropicAcousticModeling(int simId, int *shot, float *velocity, float *wavelet);
int adjointModeling(int simId, int *shot, float *velocity, float *wavelet, float *seismogram,
                    float *imageCondition, float *selfImageCondition);
int zfp2d_lossyDecompression(char *zfp_data_02, float *array, int dimension1, int dimension2,
                             float tolerance);                                   /* compression_tools.h:9 */
/* compression_tools.h:5: *compression = a malloc'ed buffer holding the stream (the caller
 * frees it), the stream's byte length returned (0 on failure, as zfp_compress). */
int zfp2d_lossyCompression(void **compression, float *array, int dimension1, int dimension2,
                           float tolerance);
void cross_correlation(float *imageCondition, float *sourceWavefield, float *receiverWavefield);
void normalized_cross_correlation(float *imageCondition, float *selfImageCondition,
                                  float *sourceWavefield, float *receiverWavefield);
void iso_acoustic_wave_equation(float *pond, float *waveField2, float *waveField3);
void attenuation_profile_cpml(float *a_Left, float *a_Right, float *a_Top, float *a_Bottom,
                              float *b_Left, float *b_Right, float *b_Top, float *b_Bottom);
void aiso_attenuation_cpml(float *waveField1, float *waveField2, float *Coef, float *a_left,
                           float *b_left, float *a_right, float *b_right, float *a_top,
                           float *b_top, float *a_bottom, float *b_bottom, float *psi_borderLeft,
                           float *psi_borderRight, float *psi_borderTop, float *psi_borderBottom,
                           float *csi_borderLeft, float *csi_borderRight, float *csi_borderTop,
                           float *csi_borderBottom);
void extend_matrix(float *extendedModel, float *model);                          /* generic_functions.h:5 */
void laplacian_filter2D(float *lp, float *inputMatrix);                          /* math_functions.h:15 */
int reading_file(char *path, float *matrix, int dim1, int dim2);                 /* pi_file.h:5 */
int recording_file(char *path, float *matrix, int dim1, int dim2);               /* pi_file.h:6 */

#ifdef FIXED_PARAMETERS_H
/* Run-time copy of the reference's compile-time configuration. */
static inline int rtm_dropin_configure_from_fixed_parameters(void)
{
    rtm_params p;
    rtm_survey s;
    p.nx = Nx; p.nz = Nz;
    p.th_left = thicknessLeft; p.th_right = thicknessRight;
    p.th_up = thicknessUp; p.th_down = thicknessDown;
    p.dx = spacingGrid; p.dt = sampling;
    p.nt = numberOfTimeStep; p.n_wavelet = sampligWavelet;
    p.shot_x = firstLocationShot; p.shot_z = depthShot;
    p.rec_first = firstLocationReceiver; p.rec_spacing = spacingReceiver;
    p.rec_count = numberOfReceivers; p.rec_depth = depthReceiver;
#ifdef TIME_SLICES
    p.time_slices = TIME_SLICES;
#else
    p.time_slices = 20;
#endif
    rtm_params_defaults(&p);
    s.velocity_file = velocityFile; s.wavelet_file = waveletFile;
    s.seismogram_file = seismogramFile; s.stacked_file = stackedFile;
    s.laplacian_file = stackedLaplacianFile;
    s.first_shot = firstLocationShot; s.shot_depth = depthShot;
    s.shot_spacing = spacingShot; s.n_shots = numberOfShots;
    s.zfp_tolerance = zfp_tolerance;
    s.normalize_by_self = 0;            /* rtm_iso2d.c:152 is commented out */
    s.checkpoint_file = NULL;
    return rtm_dropin_configure(&p, &s);
}
#endif

#ifdef __cplusplus
}
#endif
#endif
