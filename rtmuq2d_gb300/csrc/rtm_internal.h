// rtm_internal.h -- types shared by the sm_103a kernels (rtm_kernels.cu) and the host
// engine (rtm_engine.cu).  Not part of the public C ABI.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace rtm {

// ---- tile shape of the fused step kernel ------------------------------------------------
// A CTA owns TX x TZ cells: lanes run along z (4 consecutive cells each, one 16-byte
// vector for fp32), warps along x (RX columns per thread).  The current wavefield tile is
// brought into shared memory by one TMA 2-D load with a 4-cell halo on every side.
constexpr int TZ = 128;               // z cells per tile  (32 lanes x 4)
constexpr int HALO = 4;               // half stencil width (8th order)
constexpr int SZ = TZ + 2 * HALO;     // shared-memory row length (z)
constexpr int kMaxWarps = 8;

// Step flags (bit set in StepArgs::flags)
enum : int {
    F_SRC = 1 << 0,          // add wavelet[t]*coef at the shot cell (forward)
    F_RECORD = 1 << 1,       // record u at receiver cells (forward)
    F_RING_SAVE = 1 << 2,    // save the boundary ring of u_next (forward, ring storage)
    F_SNAP_SAVE = 1 << 3,    // save the interior of u_next (forward, snapshot storage)
    F_OVERWRITE = 1 << 4,    // overwrite receiver cells with the seismogram (backward)
    F_RECON = 1 << 5,        // reconstruct the source field one step back (backward)
    F_RECON_SRC = 1 << 6,    // ...including the source term
    F_IMAGE = 1 << 7,        // cross-correlate this step (backward)
    F_IMAGE_SNAP = 1 << 8,   // ...with S read from a snapshot
    F_IMAGE_FIXED = 1 << 9,  // ...with S read from a resident buffer (first two steps)
    F_NO_STENCIL = 1 << 10,  // keep u_next as given (CPML-only drop-in step)
    F_NO_CPML = 1 << 11,     // skip the CPML corrections (stencil-only drop-in step)
};

// Device-side error bits (StepArgs::status)
enum : unsigned {
    ST_TMA_TIMEOUT = 1u << 0,
};

struct Geom {
    int nx, nz, thl, thr, thu, thd;
    int dimx, dimz, pitch;      // padded grid; pitch = z stride of every field (elements)
    int st, sb;                 // z stride of the top / bottom CPML strip arrays
    int xs, zs;                 // shot cell (padded coordinates)
    int zrec;                   // receiver row (padded)
    int rx0, rx1, rz0, rz1;     // reconstruction region [rx0,rx1) x [rz0,rz1)
    int ring_w, ring_h;         // rx1-rx0+8, rz1-rz0
    int ring_cells;             // 8*ring_w + 8*ring_h
    int nt, nwav, slices, nrec;
    int tx;                     // x columns per tile
    int tiles_x, tiles_z;
};

template <typename T>
struct StepArgs {
    Geom g;
    T h1, h2, h3;               // 1/dx, dx^2, 1/dx^2 (absorbingBoundaryCondition.c:159-161)
    const T *coef;
    T *u_next;                  // in: u_prev, out: u_next (in place, like the reference)
    const T *psi_l, *psi_r, *psi_t, *psi_b;
    T *xi_l, *xi_r, *xi_t, *xi_b;
    const float *a_l, *b_l, *a_r, *b_r, *a_t, *b_t, *a_b, *b_b;
    int t;                      // forward: time; backward: time (tau = nt-1-time)
    int flags;
    const float *wavelet;       // n_wavelet values
    const int *rec_last;        // per column: last receiver index there, or -1
    const int *rec_first;       // per column: first receiver index there, or -1
    const int *rec_cnt;         // per column: receivers there
    const float *seis_row;      // backward: seismogram row tau ([t][irec] copy)
    T *rec_out;                 // forward: recorded seismogram, [irec][nt]
    void *store;                // ring slot / snapshot slot for this step
    int store_prec;             // rtm_precision
    float *store_scale;         // per-tile scales of this step (16-bit storage)
    T *s_next;                  // backward: source field, in: u_{tau+3}, out: u_{tau+1}
    const T *s_snap;            // backward: snapshot slot for imaging
    const T *s_fixed;           // backward: resident S for the first two steps
    double *img, *slf;          // FP64 image accumulators, [x-thl][pitch]
    unsigned *status;
};

template <typename T>
struct PsiArgs {
    Geom g;
    T h1;
    const T *u;                 // current wavefield
    T *psi_l, *psi_r, *psi_t, *psi_b;
    const float *a_l, *b_l, *a_r, *b_r, *a_t, *b_t, *a_b, *b_b;
};

// ---- launchers (rtm_kernels.cu) --------------------------------------------------------
template <typename T>
cudaError_t launch_step(int backward, const CUtensorMap *tm_u, const CUtensorMap *tm_s,
                        const StepArgs<T> &a, cudaStream_t s);
template <typename T>
cudaError_t launch_psi(const PsiArgs<T> &a, cudaStream_t s);
template <typename T>
cudaError_t launch_coef(const Geom &g, const float *vel, int vel_pitch, T *coef, float dx,
                        float dt, cudaStream_t s);
cudaError_t launch_transpose(const float *in, float *out, int rows, int cols, cudaStream_t s);
template <typename T>
cudaError_t launch_image_out(const Geom &g, const double *img, T *out, int accumulate,
                             cudaStream_t s);
template <typename T>
cudaError_t launch_field_out(const Geom &g, const T *field, T *out, cudaStream_t s);
template <typename T>
cudaError_t launch_field_in(const Geom &g, const T *in, T *field, cudaStream_t s);
cudaError_t launch_laplacian(int nx, int nz, const float *in, float *out, cudaStream_t s);
template <typename T>
cudaError_t launch_xcorr(const Geom &g, const T *src, const T *rcv, double *img, double *slf,
                         cudaStream_t s);
size_t step_smem_bytes(int backward, int elem_size, int tx);

}  // namespace rtm
