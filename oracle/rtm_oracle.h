/*
 * rtm_oracle.h -- CPU restatement of rtmUq2D's migration path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the CUDA engine is compared
 * against, and the timed CPU baseline ("port").  The product library never
 * links, loads or calls it; only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg do.
 *
 * Every routine restates one routine of the reference (paths relative to the
 * reference project root):
 *   orc_extend_matrix      SRC/generic_functions.c:5-48
 *   orc_cpml_profile       SRC/absorbingBoundaryCondition.c:11-148
 *   orc_coef_*             SRC/forward_modeling.c:71-81 (backward_modeling.c:243-250)
 *   orc_stencil_*          SRC/stencilDFM.c:7-31
 *   orc_cpml_*             SRC/absorbingBoundaryCondition.c:150-361
 *   orc_forward_*          SRC/forward_modeling.c:12-159 (+ optional trace recording,
 *                          which the reference does not have)
 *   orc_adjoint_*          SRC/backward_modeling.c:12-165
 *   orc_xcorr_*            SRC/image_conditions.c:20-33
 *   orc_laplacian          SRC/math_functions.c:9-27
 *
 * Unlike the reference, sizes are run-time values (struct orc_params) instead of
 * compile-time constants from SRC/fixed_parameters.h, and the forward->adjoint
 * snapshot side channel is a caller-owned array instead of a temporary file.
 * The arithmetic (operation order, float constants) is the reference's; built
 * with -ffp-contract=off it reproduces the reference build bit for bit.
 *
 * Each REAL-typed routine exists twice: suffix _f (float, the reference's
 * precision) and _d (double: the same scheme in FP64, used to state errors).
 */
#ifndef RTM_ORACLE_H
#define RTM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_params {
    int nx, nz;                       /* Nx, Nz: model size without CPML        */
    int th_left, th_right, th_up, th_down; /* CPML thickness (cells)           */
    float dx;                         /* spacingGrid (m)                        */
    float dt;                         /* sampling (s)                           */
    int nt;                           /* numberOfTimeStep                       */
    int n_wavelet;                    /* sampligWavelet                         */
    int shot_x, shot_z;               /* shot[0], shot[1] (model coordinates)   */
    int rec_first, rec_spacing, rec_count, rec_depth; /* receiver line        */
    int time_slices;                  /* TIME_SLICES (imaging interval)         */
} orc_params;

int orc_dim_x(const orc_params *p);
int orc_dim_z(const orc_params *p);

/* setup (float only, like the reference) */
void orc_extend_matrix(const orc_params *p, float *ext, const float *model);
void orc_cpml_profile(const orc_params *p, float *a_l, float *a_r, float *a_t, float *a_b,
                      float *b_l, float *b_r, float *b_t, float *b_b);
void orc_laplacian(const orc_params *p, float *lp, const float *in);

/* per-step kernels and drivers, float */
void orc_coef_f(const orc_params *p, float *coef, const float *vel_ext);
void orc_stencil_f(const orc_params *p, const float *coef, const float *u_cur, float *u_prev_next);
void orc_cpml_f(const orc_params *p, const float *u_cur, float *u_next, const float *coef,
                const float *a_l, const float *b_l, const float *a_r, const float *b_r,
                const float *a_t, const float *b_t, const float *a_b, const float *b_b,
                float *psi_l, float *psi_r, float *psi_t, float *psi_b,
                float *xi_l, float *xi_r, float *xi_t, float *xi_b);
void orc_xcorr_f(const orc_params *p, float *img, float *self_img, const float *src, const float *rcv);
/* snapshots: (nt/time_slices + (nt%time_slices!=0)) x dimX*dimZ, may be NULL.
 * seis_out: rec_count x nt, [irec][t], may be NULL.  u_last/u_prev: dimX*dimZ,
 * may be NULL; receive the two final wavefields (u_nt, u_nt-1). */
void orc_forward_f(const orc_params *p, const float *vel_ext, const float *wavelet,
                   float *snapshots, float *seis_out, float *u_last, float *u_prev);
void orc_adjoint_f(const orc_params *p, const float *vel_ext, const float *seis,
                   const float *snapshots, float *img, float *self_img);

/* the same scheme in double precision */
void orc_coef_d(const orc_params *p, double *coef, const float *vel_ext);
void orc_stencil_d(const orc_params *p, const double *coef, const double *u_cur, double *u_prev_next);
void orc_cpml_d(const orc_params *p, const double *u_cur, double *u_next, const double *coef,
                const float *a_l, const float *b_l, const float *a_r, const float *b_r,
                const float *a_t, const float *b_t, const float *a_b, const float *b_b,
                double *psi_l, double *psi_r, double *psi_t, double *psi_b,
                double *xi_l, double *xi_r, double *xi_t, double *xi_b);
void orc_xcorr_d(const orc_params *p, double *img, double *self_img, const double *src, const double *rcv);
void orc_forward_d(const orc_params *p, const float *vel_ext, const float *wavelet,
                   double *snapshots, double *seis_out, double *u_last, double *u_prev);
void orc_adjoint_d(const orc_params *p, const float *vel_ext, const double *seis,
                   const double *snapshots, double *img, double *self_img);

/* thread control for the OpenMP loops (<=0: leave the runtime default) */
void orc_set_threads(int n);
int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
