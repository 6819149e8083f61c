// rtm_internal.h -- types shared by the sm_103a kernels (rtm_kernels.cu, rtm_step.cuh) and
// the host engine (rtm_engine.cu).  Not part of the public C ABI.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace rtm {

// ---- tile shape of the fused step kernel ------------------------------------------------
// A tile is TX x TZ cells: lanes run along z (4 consecutive cells each, one 16-byte vector
// for fp32), warps along x (2 columns per thread).  The current-field tile is staged in
// shared memory by a TMA 2-D copy with a 4-cell halo on every side; u_prev and coef tiles
// by TMA copies without halo.
constexpr int TZ = 128;               // z cells per tile  (32 lanes x 4)
constexpr int HALO = 4;               // half stencil width (8th order)
constexpr int SZ = TZ + 2 * HALO;     // shared-memory row length of a halo tile (z)
constexpr int RXC = 2;                // x columns per thread

// Step flags (bit set in StepArgs::flags)
enum : int {
    F_SRC = 1 << 0,          // add wavelet[t]*coef at the shot cell (forward)
    F_RECORD = 1 << 1,       // record u at receiver cells (forward)
    F_RING_SAVE = 1 << 2,    // save the boundary ring (forward, ring storage): of u_cur at full
                             // precision, of u_next in 16 bits
    F_SNAP_SAVE = 1 << 3,    // save the interior of u_next (forward, snapshot storage)
    F_OVERWRITE = 1 << 4,    // overwrite receiver cells with the seismogram (backward)
    F_RECON = 1 << 5,        // reconstruct the source field one step back (backward)
    F_RECON_SRC = 1 << 6,    // ...including the source term
    F_IMAGE = 1 << 7,        // cross-correlate this step (backward)
    F_IMAGE_SNAP = 1 << 8,   // ...with S read from a snapshot
    F_IMAGE_FIXED = 1 << 9,  // ...with S read from a resident buffer (first two steps)
    F_NO_STENCIL = 1 << 10,  // keep u_next as given (CPML-only drop-in step)
    F_NO_CPML = 1 << 11,     // skip the CPML corrections (stencil-only drop-in step)
    F_STRIPS_FRESH = 1 << 12,  // first step of a pass: psi/xi start from zero (batched members)
};

// Device-side error bits (StepArgs::status)
enum : unsigned {
    ST_TMA_TIMEOUT = 1u << 0,
};

struct Geom {
    int nx, nz, thl, thr, thu, thd;
    int dimx, dimz, pitch;      // padded grid; pitch = z stride of every field (elements)
    int st;                     // z stride of the top strip arrays (>= round4(thu) + 4)
    int zb0;                    // first z of the bottom strip arrays (4-aligned, <= dimz-thd)
    int sb;                     // z stride of the bottom strip arrays (>= round4(dimz-zb0) + 4)
    int xs, zs;                 // shot cell (padded coordinates)
    int zrec;                   // receiver row (padded)
    int rx0, rx1, rz0, rz1;     // reconstruction region [rx0,rx1) x [rz0,rz1)
    int ring_w, ring_h;         // rx1-rx0+8, rz1-rz0
    int ring_cells;             // 8*ring_w + 8*ring_h
    int nt, nwav, slices, nrec;
    int tx;                     // x columns per tile
    int ztop;                   // height of z-tile 0 (4-aligned, <= TZ): the top CPML band;
                                // z-tile k >= 1 starts at ztop + (k-1)*TZ
    int zbot;                   // > 0: the last z-tile is [zbot, dimz) (4-aligned, holds the
                                // bottom CPML band), the ones before it end at zbot at most
    int tiles_x, tiles_z, tiles;
    int nxl, xr0;               // left CPML x-tiles [0,nxl), right ones [xr0,tiles_x)
};

// Scheduling order of the tiles of one step: the slow ones first -- the top and bottom
// z-tiles (CPML strips, ring bands, receiver row), then the left/right CPML x-tiles of the
// other z-tiles, then the plain interior.  x-tiles [0, nxl) and [xr0, tiles_x) are the
// left/right CPML columns (nxl <= xr0).
__host__ __device__ __forceinline__ void tile_coords(const Geom &g, int t, int &xt, int &zt)
{
    const int nzb = g.tiles_z > 1 ? 2 : 1;
    const int n1 = g.tiles_x * nzb;
    if (t < n1) {
        xt = t / nzb;
        zt = (t % nzb == 0) ? 0 : g.tiles_z - 1;
        return;
    }
    t -= n1;
    const int nzi = g.tiles_z - nzb;
    const int nxb = g.nxl + (g.tiles_x - g.xr0);
    if (t < nxb * nzi) {
        const int xi = t / nzi;
        xt = xi < g.nxl ? xi : g.xr0 + (xi - g.nxl);
        zt = 1 + t % nzi;
        return;
    }
    t -= nxb * nzi;
    xt = g.nxl + t / nzi;
    zt = 1 + t % nzi;
}

// Tiles of the top and bottom z-tile rows and of the left/right CPML x-tiles of the other
// rows: the first boundary_tiles(g) tiles of tile_coords' order.
__host__ __device__ __forceinline__ int boundary_tiles(const Geom &g)
{
    const int nzb = g.tiles_z > 1 ? 2 : 1;
    return g.tiles_x * nzb + (g.nxl + (g.tiles_x - g.xr0)) * (g.tiles_z - nzb);
}

// Number of psi quads of each strip (the batched psi kernel k_bpsi's enumeration: left, top,
// right, bottom).
__host__ __device__ __forceinline__ void psi_counts(const Geom &g, int (&n)[4])
{
    const int nlr = (g.dimz - 8 + 3) / 4;
    n[0] = (g.thl - 8) * nlr;
    n[1] = (g.dimx - 8) * ((g.thu - 8 + 3) / 4);
    n[2] = (g.thr - 8) * nlr;
    const int q0 = (g.dimz - g.thd + 4) & ~3;
    n[3] = (g.dimx - 8) * ((g.dimz - 4 - q0 + 3) / 4);
}

__host__ __device__ __forceinline__ int ztile_origin(const Geom &g, int zt)
{
    if (zt == 0) return 0;
    if (g.zbot > 0 && zt == g.tiles_z - 1) return g.zbot;
    return g.ztop + (zt - 1) * TZ;
}
__host__ __device__ __forceinline__ int ztile_end(const Geom &g, int zt)
{
    if (g.zbot > 0) {
        if (zt == g.tiles_z - 1) return g.dimz;
        const int e = zt == 0 ? g.ztop : g.ztop + zt * TZ;
        return e < g.zbot ? e : g.zbot;
    }
    return zt == 0 ? g.ztop : g.ztop + zt * TZ;
}

// Offsets (floats) of the eight damping profiles in the packed, 16-byte aligned profile
// array: a_l b_l a_r b_r (by column), a_t b_t (by z, length st), a_b b_b (by z - zb0,
// length sb).
struct ProfLayout {
    int off[8];
    int total;
};

template <typename T>
struct StepArgs {
    Geom g;
    T h1, h2, h3;               // 1/dx, dx^2, 1/dx^2 (absorbingBoundaryCondition.c:159-161)
    T *u_next;                  // in: u_prev, out: u_next (in place, like the reference)
    const T *psi_l, *psi_r, *psi_t, *psi_b;   // psi of the previous step (read)
    T *psn_l, *psn_r, *psn_t, *psn_b;         // psi of this step (written; the other buffer)
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

// Tensor maps of one step: halo maps box {SZ, tx+8}, plain maps box {TZ, tx}.
struct StepMaps {
    CUtensorMap cur;            // current propagated field (halo)
    CUtensorMap cur8;           // ...with an 8-column x halo, box {SZ, tx+16} (side CPML tiles)
    CUtensorMap prev;           // previous propagated field = output buffer (plain)
    CUtensorMap coef;           // (v dt/dx)^2 (plain)
    CUtensorMap scur;           // backward reconstruction: current source field (halo)
    CUtensorMap sprev;          // backward reconstruction: previous source field (plain)
};

// One member of a batch (a resident migration): descriptor read by k_bpsi / k_bstep.
template <typename T>
struct BMember {                 // aligned like its leading tensor maps
    CUtensorMap tm_u[2], tm_up[2], tm_r[2], tm_rp[2], tm_c;   // halo / plain maps
    Geom g;
    T h1, h2, h3;
    T *u[2], *r[2];
    const T *coef;
    T *psi[4], *xi[4];          // left, right, top, bottom
    T *rec_out;                 // recorded seismogram [irec][nt] (forward; NULL: none)
    const float *prof[8];       // a_l b_l a_r b_r a_t b_t a_b b_b (packed, see ProfLayout)
    const int *rec_last, *rec_first, *rec_cnt;
    const float *wav, *seis_t;
    double *img, *slf;
    void *store;
    size_t slot_elems;
    float *scales;
    int scales_per_slot;        // 16-bit storage: scales of one slot (tiles / strip blocks)
    int store_prec, storage;
    unsigned *status;
};

constexpr int kMaxMembers = 1024;  // members of one batch (the kernels read their tables from global memory)
constexpr int kBatchTileX = 32;    // widest tile of the batched step kernel (MTX); members use it or half

// Work lists of one batch.  The tile work of a step runs in two phases: first every
// member's interior field tiles and source-reconstruction tiles, then every member's field
// tiles touching a CPML strip.  Member i owns items [base1[i], base1[i+1]) of phase 1 and
// [base2[i], base2[i+1]) of phase 2, psi quads [psi_base[i], ...) and strip items
// [corr_base[i], ...) of k_bstrip.
struct BatchIndex {
    int nmem;
    int base1[kMaxMembers + 1];         // phase 1: interior field tiles + source-field tiles
    int base2[kMaxMembers + 1];         // phase 2: field tiles touching a CPML strip
    int psi_base[kMaxMembers + 1];      // k_bpsi quads
    int corr_base[kMaxMembers + 1];     // k_bstrip items
    int tiles[kMaxMembers];             // field tiles of member i (forward / receiver)
    int nb[kMaxMembers];                // ...of which touch a strip (tile_coords order first)
    int nt[kMaxMembers];                // time steps of member i
};

// ---- batched steps (rtm_batch.cuh) -------------------------------------------------------
// state[m] = (pass, step): pass 0 idle, 1 forward (nt steps), 2 backward (nt + 1 steps,
// the last one images only), 3 finished.
// done[0]: CTA counter of the step in flight (zero between launches); done[1]: error bits;
// done[2]: chunk counter of k_mstep (cleared by k_bstrip's last CTA).
constexpr int kBatchDoneWords = 3;
template <typename T>
cudaError_t launch_bpsi(const BatchIndex *ix, const BMember<T> *mem, const int2 *state, int grid,
                        int pdl, cudaStream_t s);
template <typename T>
cudaError_t launch_bstrip(const BatchIndex *ix, const BMember<T> *mem, int2 *state, unsigned *done, int grid,
                          int pdl, cudaStream_t s);
template <typename T>
cudaError_t launch_bstep(const BatchIndex *ix, const BMember<T> *mem, int2 *state, unsigned *done,
                         int grid, int pdl, cudaStream_t s);
template <typename T>
int bstep_grid();                                 // persistent CTAs of k_mstep
void psi_counts_host(const Geom &g, int (&n)[4]);
int strip_items_host(const Geom &g, int ring);     // k_bstrip items of one member
int strip_blocks_host(const Geom &g);              // its strip-quad blocks (16-bit ring scales)
int boundary_tiles_host(const Geom &g);            // field tiles touching a CPML strip

// ---- launchers (rtm_kernels.cu) --------------------------------------------------------
// pdl: launch with programmatic stream serialization (overlaps the preceding kernel's tail)
template <typename T>
cudaError_t launch_step(int backward, const StepMaps &maps, const StepArgs<T> &a, int grid,
                        int pdl, cudaStream_t s);
template <typename T>
int step_grid(int backward, const Geom &g);      // persistent CTAs for one step
size_t step_smem_bytes(int backward, int elem_size, int tx);
constexpr int kMaxStripThickness = 120;   // top / bottom CPML: each band inside one z-tile
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
cudaError_t launch_stack_add(const Geom &g, const double *img, const double *slf, float *acc_img,
                             float *acc_slf, unsigned *plan_status, unsigned *stack_status, cudaStream_t s);
cudaError_t launch_stack_finish(int n, const float *acc_img, const float *acc_slf, int normalize, float *out,
                                cudaStream_t s);

}  // namespace rtm
