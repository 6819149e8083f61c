/*
 * ref_runtime_params.c -- storage and setter for the run-time configuration of the
 * reference build (test infrastructure, oracle/_ref only).  See ref_runtime_params.h.
 */
#include <stdio.h>
#include "ref_runtime_params.h"

#define REF_PATH_LEN 4096
char velocityFile[REF_PATH_LEN] = "./INPUTS/vp_%05d.bin";
char waveletFile[REF_PATH_LEN] = "./INPUTS/wavelet.bin";
char seismogramFile[REF_PATH_LEN] = "./INPUTS/seismogram_%05d.zfp";
char stackedFile[REF_PATH_LEN] = "./OUTPUTS/stackedBrute_%05d.bin";
char stackedLaplacianFile[REF_PATH_LEN] = "./OUTPUTS/stackedLaplacian_%05d.bin";
float zfp_tolerance = 0.0f;
float spacingGrid = 10.0f;
float sampling = 0.001f;
int numberOfSimulations = 1;
int Nx = 0, Nz = 0;
int firstLocationShot = 0, depthShot = 0, spacingShot = 0, numberOfShots = 1;
int firstLocationReceiver = 0, depthReceiver = 0, spacingReceiver = 2, numberOfReceivers = 0;
int numberOfTimeStep = 0;
int sampligWavelet = 800;
float cutFrequency = 50.0f;
int thicknessUp = 0, thicknessDown = 0, thicknessLeft = 0, thicknessRight = 0;

/* Integer settings in the order of struct ref_int_params in oracle/oracle.py. */
void ref_set_params(const int *iv, const float *fv)
{
    Nx = iv[0]; Nz = iv[1];
    thicknessLeft = iv[2]; thicknessRight = iv[3]; thicknessUp = iv[4]; thicknessDown = iv[5];
    numberOfTimeStep = iv[6]; sampligWavelet = iv[7];
    firstLocationShot = iv[8]; depthShot = iv[9]; spacingShot = iv[10]; numberOfShots = iv[11];
    firstLocationReceiver = iv[12]; spacingReceiver = iv[13]; numberOfReceivers = iv[14];
    depthReceiver = iv[15]; numberOfSimulations = iv[16];
    spacingGrid = fv[0]; sampling = fv[1]; zfp_tolerance = fv[2];
}

void ref_set_paths(const char *vel, const char *wav, const char *seis, const char *stacked,
                   const char *laplacian)
{
    if (vel) snprintf(velocityFile, REF_PATH_LEN, "%s", vel);
    if (wav) snprintf(waveletFile, REF_PATH_LEN, "%s", wav);
    if (seis) snprintf(seismogramFile, REF_PATH_LEN, "%s", seis);
    if (stacked) snprintf(stackedFile, REF_PATH_LEN, "%s", stacked);
    if (laplacian) snprintf(stackedLaplacianFile, REF_PATH_LEN, "%s", laplacian);
}
