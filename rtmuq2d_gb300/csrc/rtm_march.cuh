// rtm_march.cuh -- tile step of the batched engine (included by rtm_kernels.cu after
// rtm_step.cuh, whose stencil helpers it shares).
//
// A tile is TX = 8 x CW columns (CW = 4 or 2 columns per warp: 32 or 16, a member's tile
// width, chosen per grid shape by rtm_autotune_batched) x TZ = 128 z cells of ONE field of one
// migration.  Its inputs -- the field with a 4-cell halo (TX+8 rows of SZ), the previous field
// and coef (TX rows of TZ) -- arrive in one shared-memory stage by TMA.  Warp w owns columns
// CW w .. CW w + CW - 1 and marches along x through them with a 9-column register window
// (1 new row per column); lane l owns the 4 z cells 4l..4l+3 of every column (16-byte
// vectors).  Each thread thus updates 4 CW cells per tile, and everything that is decided per
// tile is decided once for those cells.  A tile reads nothing from global memory: the per-cell work that needs
// other data -- the CPML corrections of the strips, the boundary ring's storage and
// restoration -- is done afterwards by the strip kernel k_bstrip (rtm_batch.cuh), over
// the strip cells only.
//
// Roles (one tile = one role):
//   ROLE_FWD  forward propagation: 8th-order leapfrog (SRC/stencilDFM.c:17-29), source
//             injection (forward_modeling.c:105-109), trace recording, snapshot storage
//             (FP32 or 16-bit with a per-step, per-tile max-abs scale).
//   ROLE_RCV  backward receiver propagation: leapfrog + receiver overwrite
//             (backward_modeling.c:106-110), and the cross-correlation image
//             (image_conditions.c:20-33) of the PREVIOUS step: this step's input field is
//             the previous step's receiver field, and the previous step's source field
//             sits in a buffer nobody writes during this step, so imaging costs no extra
//             pass (the last step's image is taken by one extra image-only step).
//   ROLE_SRC  reverse-time reconstruction of the source field: leapfrog on the
//             reconstruction region, the previous value elsewhere (k_bstrip then restores
//             the ring cells), the source term undone at the shot.
// Receiver and source fields of a backward step are separate tiles of equal stage size,
// so every tile's stage holds 3 arrays (54.5 KB for FP32) and two CTAs per SM keep two
// tile loads in flight while two are computed.  Source, receivers, snapshots and the image
// never touch a CPML strip, so the strip kernel's later updates do not reorder any of the
// reference's operations on a cell.

constexpr int MWARPS = 8;                 // warps per CTA
constexpr int MCW = 4;                    // columns per warp of the widest tile
constexpr int MTX = MWARPS * MCW;         // 32 columns per tile (the stage is sized for it)
constexpr int MTHREADS = MWARPS * 32;

// CTA barriers of the tile code (named barrier 1 over the MWARPS warps).
__device__ __forceinline__ void group_sync()
{
    asm volatile("bar.sync 1, %0;" ::"n"(MWARPS * 32) : "memory");
}
__device__ __forceinline__ float group_max(float v, float *red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    group_sync();
    float m = red[0];
#pragma unroll
    for (int w = 1; w < MWARPS; ++w) m = fmaxf(m, red[w]);
    group_sync();
    return m;
}

enum : int { ROLE_FWD = 0, ROLE_RCV = 1, ROLE_SRC = 2 };
enum : int { F_NO_STEP = 1 << 13 };       // image-only step (no propagation)

template <typename T>
struct MCfg {
    static constexpr int UT = (MTX + 2 * HALO) * SZ;      // halo tile, elements
    static constexpr int PT = MTX * TZ;                    // plain tile, elements
    static constexpr int STAGE = UT + 2 * PT;
    static constexpr int NS = 2;                           // stages per CTA
    static constexpr size_t SMEM = (size_t)NS * STAGE * sizeof(T);
};
// Stage layout of a tile TX columns wide (TX <= MTX): halo tile, previous field, coef.
__host__ __device__ __forceinline__ int mstage_ut(int tx) { return (tx + 2 * HALO) * SZ; }
__host__ __device__ __forceinline__ int mstage_elems(int tx) { return mstage_ut(tx) + 2 * tx * TZ; }

// Per (member, role) arguments of a step, built by the issuing thread in shared memory.
template <typename T>
struct MArgs {
    Geom g;
    T *out;                       // next field, written in place over the previous one
    const float *wavelet;
    const int *rec_last, *rec_first, *rec_cnt;
    const float *seis_row;        // RCV: seismogram row tau ([t][irec] copy)
    T *rec_out;                   // FWD: recorded seismogram [irec][nt] (optional)
    void *store;                  // FWD: snapshot slot saved; RCV: snapshot slot read
    float *store_scale;           // per-tile scales of that slot (16-bit storage)
    const T *s_img;               // RCV, ring storage: source field of the previous step
    double *img, *slf;            // FP64 image accumulators, [x-thl][pitch]
    int t;                        // step of the pass
    int tsrc;                     // SRC: forward step whose source term is undone
    int flags;
    int store_prec;
};

// The 16-bit storage scale of a block: max |v| over the cells it stores, mapped to target.
__host__ __device__ __forceinline__ float store_scale_of(float mx, int prec)
{
    const float target = prec == 2 ? kFp16Target : kBf16Target;
    // A block ahead of the wavefront can hold only denormal-size values: clamping keeps the
    // inverse finite (an infinite inverse would turn 0 into NaN).
    return fmaxf(mx, 1e-30f) / target;
}

// The arguments live in shared memory and the tile stores through generic pointers: the
// __restrict__ qualifiers tell the compiler that those stores never modify the arguments
// or the stage, so it keeps argument values in registers across them instead of reloading.
template <typename T, int ROLE, int CW>
__device__ __forceinline__ void march_tile(const MArgs<T> *__restrict__ ap, const T *__restrict__ stage,
                                           int lt, float *red)
{
    const MArgs<T> &a = *ap;
    constexpr int TXW = MWARPS * CW;                 // columns of this tile width
    constexpr int UT = (TXW + 2 * HALO) * SZ, PT = TXW * TZ;
    const Geom &g = a.g;
    const int flags = a.flags;
    const T *su = stage;                   // field + halo   [TXW+8][SZ]
    const T *sprv = stage + UT;            // previous field [TXW][TZ]
    const T *scf = stage + UT + PT;        // coef           [TXW][TZ]

    int xt, zt;
    tile_coords(g, lt, xt, zt);
    const int x0 = xt * TXW, z0 = ztile_origin(g, zt);
    const int x1 = x0 + TXW, z1 = min(ztile_end(g, zt), z0 + TZ);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int zq = z0 + 4 * lane;
    const int xw = x0 + CW * warp;         // first column of this warp
    const int rw = CW * warp;              // halo-tile row of column xw - 4
    const int zi = 4 * lane + HALO;
    const bool zok = zq < min(z1, g.dimz);
    const size_t P = (size_t)g.pitch;

    // ---- tile classification (uniform over the CTA)
    const bool step = !(flags & F_NO_STEP);
    const bool in_domain = x0 >= 4 && x1 <= g.dimx - 4 && z0 >= 4 && z1 <= g.dimz - 4;
    const bool src_t = ((ROLE == ROLE_FWD && (flags & F_SRC)) || (ROLE == ROLE_SRC && (flags & F_RECON_SRC))) &&
                       g.xs >= x0 && g.xs < x1 && g.zs >= z0 && g.zs < z1;
    const bool rec_t = ((ROLE == ROLE_FWD && (flags & F_RECORD)) || (ROLE == ROLE_RCV && (flags & F_OVERWRITE))) &&
                       step && g.zrec >= z0 && g.zrec < z1;
    const bool in_region = x0 >= g.rx0 && x1 <= g.rx1 && z0 >= g.rz0 && z1 <= g.rz1;
    const bool int_full = x0 >= g.thl && x1 <= g.thl + g.nx && z0 >= g.thu && z1 <= g.thu + g.nz;
    const bool int_any = x0 < g.thl + g.nx && x1 > g.thl && z0 < g.thu + g.nz && z1 > g.thu;
    const bool snap_t = ROLE == ROLE_FWD && (flags & F_SNAP_SAVE) && int_any;
    const bool scaled = snap_t && a.store_prec != 0;
    const bool snap_fast = snap_t && int_full && !scaled && !src_t;
    const bool image_t = ROLE == ROLE_RCV && (flags & F_IMAGE) && int_any;
    const bool image_fast = image_t && int_full;
    const bool fast = step && in_domain && !src_t && !rec_t && (!snap_t || snap_fast) &&
                      (!image_t || image_fast) && (ROLE != ROLE_SRC || in_region);
    if (!step && !image_t) return;                       // image-only step off the interior

    // source field of the imaged step (RCV): the ring-storage buffer, or the snapshot slot
    const bool img_snap = (flags & F_IMAGE_SNAP) != 0;
    const float img_scale = (image_t && img_snap && a.store_prec != 0) ? a.store_scale[lt] : 1.0f;

    T W[9][4];
#pragma unroll
    for (int m = 0; m < 8; ++m) ld4(su + (rw + m) * SZ + zi, W[m]);

    if (fast) {
        // ================= no per-cell decisions =================
#pragma unroll
        for (int c = 0; c < CW; ++c) {
            const int x = xw + c;
            ld4(su + (rw + c + 8) * SZ + zi, W[8]);
            T zz[12];
            z_line<T>(su, rw + c + 4, zi, W[4], zz);
            T prv[4], cf[4], s[4];
            ld4(sprv + (rw + c) * TZ + 4 * lane, prv);
            ld4(scf + (rw + c) * TZ + 4 * lane, cf);
#pragma unroll
            for (int j = 0; j < 4; ++j) s[j] = cf[j] * lap8<T>(W, zz, j) + (T)2.0f * W[4][j] - prv[j];
            if (zok) {
                st4(a.out + (size_t)x * P + zq, s);
                if (snap_fast)
                    st4(reinterpret_cast<T *>(a.store) + (size_t)(x - g.thl) * P + zq, s);
                if (image_fast) {
                    const size_t o = (size_t)(x - g.thl) * P + zq;
                    T sv[4];
                    if (img_snap) {
#pragma unroll
                        for (int j = 0; j < 4; ++j) sv[j] = store_get<T>(a.store, a.store_prec, o + j, img_scale);
                    } else {
                        ld4(a.s_img + (size_t)x * P + zq, sv);
                    }
                    image_quad<T>(a.img + o, a.slf + o, sv, W[4]);
                }
            }
#pragma unroll
            for (int m = 0; m < 8; ++m)
#pragma unroll
                for (int j = 0; j < 4; ++j) W[m][j] = W[m + 1][j];
        }
        return;
    }

    // ================= tiles with per-cell decisions =================
    float mx = 0.0f;                       // 16-bit snapshots: max |v| over the stored cells
    T keep[CW][4];                         // ...and the tile's values until the scale is known
#pragma unroll
    for (int c = 0; c < CW; ++c) {
        const int x = xw + c;
        ld4(su + (rw + c + 8) * SZ + zi, W[8]);
        T zz[12];
        z_line<T>(su, rw + c + 4, zi, W[4], zz);
        T prv[4], cf[4], v[4];
        ld4(sprv + (rw + c) * TZ + 4 * lane, prv);
        ld4(scf + (rw + c) * TZ + 4 * lane, cf);
        const bool col_ok = zok && x < g.dimx;
        if (step) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const T s = cf[j] * lap8<T>(W, zz, j) + (T)2.0f * W[4][j] - prv[j];
                const int z = zq + j;
                bool upd;
                if (ROLE == ROLE_SRC) upd = x >= g.rx0 && x < g.rx1 && z >= g.rz0 && z < g.rz1;
                else upd = x >= 4 && x < g.dimx - 4 && z >= 4 && z < g.dimz - 4;
                v[j] = upd ? s : prv[j];
            }
            if (col_ok && src_t && x == g.xs) {
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (zq + j == g.zs)
                        v[j] = add_source<T>(a.wavelet, ROLE == ROLE_SRC ? a.tsrc : a.t, v[j], cf[j]);
            }
            if (col_ok && rec_t && g.zrec >= zq && g.zrec < zq + 4) {
                const int jr = g.zrec - zq;
                if (ROLE == ROLE_FWD) {
                    const int n = a.rec_cnt[x], f = a.rec_first[x];
                    for (int q = 0; q < n; ++q) a.rec_out[(size_t)(f + q) * g.nt + a.t] = v[jr];
                } else {
                    const int q = a.rec_last[x];
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        if (j == jr && q >= 0) v[j] = (T)a.seis_row[q];
                }
            }
            if (col_ok) st4(a.out + (size_t)x * P + zq, v);
            if (snap_t && col_ok) {
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int z = zq + j;
                    if (z < g.dimz && in_interior(g, x, z)) {
                        if (!scaled) reinterpret_cast<T *>(a.store)[(size_t)(x - g.thl) * P + z] = v[j];
                        else mx = fmaxf(mx, fabsf((float)v[j]));
                    }
                }
            }
            if (scaled) {
#pragma unroll
                for (int j = 0; j < 4; ++j) keep[c][j] = v[j];
            }
        }
        // ---- image of the previous step (its receiver field is this step's input)
        if (image_t && col_ok) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int z = zq + j;
                if (z < g.dimz && in_interior(g, x, z)) {
                    const size_t o = (size_t)(x - g.thl) * P + z;
                    const T sv = img_snap ? store_get<T>(a.store, a.store_prec, o, img_scale)
                                          : a.s_img[(size_t)x * P + z];
                    a.img[o] += (double)sv * (double)W[4][j];
                    a.slf[o] += (double)sv * (double)sv;
                }
            }
        }
#pragma unroll
        for (int m = 0; m < 8; ++m)
#pragma unroll
            for (int j = 0; j < 4; ++j) W[m][j] = W[m + 1][j];
    }
    if (scaled) {   // 16-bit snapshots: per-step, per-tile max-abs scale, then quantise
        mx = group_max(mx, red);
        const float scale = store_scale_of(mx, a.store_prec);
        const float inv = 1.0f / scale;
        if (threadIdx.x == 0) a.store_scale[lt] = scale;
#pragma unroll
        for (int c = 0; c < CW; ++c)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int x = xw + c, z = zq + j;
                if (!zok || x >= g.dimx || z >= g.dimz) continue;
                if (in_interior(g, x, z))
                    store_put<T>(a.store, a.store_prec, (size_t)(x - g.thl) * P + z, keep[c][j], inv);
            }
    }
}
