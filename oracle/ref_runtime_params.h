/*
 * ref_runtime_params.h -- forced-include header for building the reference's own C
 * sources (test infrastructure, oracle/_ref only).
 *
 * The reference takes every size from SRC/fixed_parameters.h as `static const`
 * values.  This header is passed with `-include` ahead of each reference source: it
 * defines the include guard FIXED_PARAMETERS_H (so the reference's copy is skipped) and
 * declares the same names as run-time globals, defined and set by ref_runtime_params.c.
 * The reference's code is compiled unchanged; only its configuration becomes settable.
 */
#ifndef FIXED_PARAMETERS_H
#define FIXED_PARAMETERS_H

extern char velocityFile[];
extern char waveletFile[];
extern char seismogramFile[];
extern char stackedFile[];
extern char stackedLaplacianFile[];
extern float zfp_tolerance;
extern float spacingGrid;
extern float sampling;
extern int numberOfSimulations;
extern int Nx, Nz;
extern int firstLocationShot, depthShot, spacingShot, numberOfShots;
extern int firstLocationReceiver, depthReceiver, spacingReceiver, numberOfReceivers;
extern int numberOfTimeStep;
extern int sampligWavelet;
extern float cutFrequency;
extern int thicknessUp, thicknessDown, thicknessLeft, thicknessRight;

#endif
