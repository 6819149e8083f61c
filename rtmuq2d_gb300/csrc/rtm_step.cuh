// rtm_step.cuh -- the persistent, TMA-pipelined time-step kernel k_step (included by
// rtm_kernels.cu).
//
// Grid: a fixed number of CTAs (filling the SMs); CTA b processes tiles b, b+G, b+2G, ...
// of the TX x 128 tiling (z-tile index fastest, so boundary and interior tiles interleave).
// Each tile's inputs -- the current field with a 4-cell halo, u_prev and coef (backward
// reconstruction: also the source field with halo and its predecessor) -- arrive by TMA 2-D
// copies into one of NS shared-memory stages; thread 0 refills a stage as soon as its tile
// is done, so NS-1 tiles are in flight while one is computed.
//
// Per tile, every thread owns RXC = 2 columns x 4 consecutive z cells, keeps a 9-column
// register window along x and reads z neighbours as aligned 16-byte vectors:
//   * 8th-order leapfrog (SRC/stencilDFM.c:17-29);
//   * on tiles touching the CPML, the corrections of the four strips in the reference's
//     order left, top, right, bottom (SRC/absorbingBoundaryCondition.c:191-357), vectorised
//     per 4-cell quad (psi and xi moved as 16-byte vectors);
//   * source injection (SRC/forward_modeling.c:105-109) or receiver overwrite
//     (backward_modeling.c:277-281), trace recording, boundary-ring or snapshot storage
//     (FP32, or BF16/FP16 with a per-step, per-tile max-abs scale);
//   * backward: reverse-time source reconstruction on the stencil-only region and the FP64
//     cross-correlation image (SRC/image_conditions.c:20-33).
// Chaining with k_psi uses programmatic dependent launch: psi is read only after
// griddepcontrol.wait, and only by tiles that need it.

__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void griddep_launch() { asm volatile("griddepcontrol.launch_dependents;" :::); }

template <typename T, int WARPS, int BWD>
struct StepCfg {
    static constexpr int TXC = WARPS * RXC;                       // x columns per tile
    static constexpr int UT = (TXC + 2 * HALO) * SZ;              // halo tile, elements
    static constexpr int PT = TXC * TZ;                           // plain tile, elements
    static constexpr int STAGE = BWD ? 2 * UT + 3 * PT : UT + 2 * PT;
    static constexpr int NS = (sizeof(T) == 4 && !BWD) ? 3 : 2;   // pipeline stages
    static constexpr size_t SMEM = (size_t)NS * STAGE * sizeof(T);
};

template <typename T>
__device__ __forceinline__ T add_source(const float *wavelet, int t, T v, T cf)
{
    if (sizeof(T) == sizeof(float)) return v + (T)(wavelet[t] * (float)cf);   // float product, as the reference
    return v + (T)wavelet[t] * cf;
}

template <typename T>
__device__ __forceinline__ void image_quad(double *img, double *slf, const T (&s)[4], const T (&r)[4])
{
    double2 i0 = reinterpret_cast<double2 *>(img)[0], i1 = reinterpret_cast<double2 *>(img)[1];
    double2 s0 = reinterpret_cast<double2 *>(slf)[0], s1 = reinterpret_cast<double2 *>(slf)[1];
    i0.x += (double)s[0] * (double)r[0]; i0.y += (double)s[1] * (double)r[1];
    i1.x += (double)s[2] * (double)r[2]; i1.y += (double)s[3] * (double)r[3];
    s0.x += (double)s[0] * (double)s[0]; s0.y += (double)s[1] * (double)s[1];
    s1.x += (double)s[2] * (double)s[2]; s1.y += (double)s[3] * (double)s[3];
    reinterpret_cast<double2 *>(img)[0] = i0; reinterpret_cast<double2 *>(img)[1] = i1;
    reinterpret_cast<double2 *>(slf)[0] = s0; reinterpret_cast<double2 *>(slf)[1] = s1;
}

// dpsi of 4 cells from psi along a strided line: rows p[0..3] = f[-4..-1], p[4..7] = f[1..4].
template <typename T>
__device__ __forceinline__ T dpsi_x(const T (&m)[4][4], const T (&p)[4][4], int j)
{
    return (T)RTM_B4 * (p[3][j] - m[0][j]) + (T)RTM_B3 * (p[2][j] - m[1][j])
         + (T)RTM_B2 * (p[1][j] - m[2][j]) + (T)RTM_B1 * (p[0][j] - m[3][j]);
}
// dpsi of 4 cells along z from a 12-value line q (q[4+j] is cell j).
template <typename T>
__device__ __forceinline__ T dpsi_z(const T (&q)[12], int j)
{
    return (T)RTM_B4 * (q[8 + j] - q[j]) + (T)RTM_B3 * (q[7 + j] - q[1 + j])
         + (T)RTM_B2 * (q[6 + j] - q[2 + j]) + (T)RTM_B1 * (q[5 + j] - q[3 + j]);
}
template <typename T>
__device__ __forceinline__ T d2x_w(const T (&W)[9][4], int j)
{
    return (T)RTM_AC4 * (W[8][j] + W[0][j]) + (T)RTM_AC3 * (W[7][j] + W[1][j])
         + (T)RTM_AC2 * (W[6][j] + W[2][j]) + (T)RTM_AC1 * (W[5][j] + W[3][j])
         + (T)RTM_AC0 * W[4][j];
}
template <typename T>
__device__ __forceinline__ T d2z_q(const T (&zz)[12], int j)
{
    return (T)RTM_AC4 * (zz[8 + j] + zz[j]) + (T)RTM_AC3 * (zz[7 + j] + zz[1 + j])
         + (T)RTM_AC2 * (zz[6 + j] + zz[2 + j]) + (T)RTM_AC1 * (zz[5 + j] + zz[3 + j])
         + (T)RTM_AC0 * zz[4 + j];
}

// Left/right strip (x-derivative) correction of one quad.  psi, xi: strip arrays with row
// stride P addressed at the quad; ab, bb: the column's profile values.
template <typename T>
__device__ __forceinline__ void cpml_x_quad(const T *psi, T *xi, size_t P, T ab, T bb, const T (&W)[9][4],
                                            const T (&cf)[4], T (&v)[4], int zq, int zlo, int zhi,
                                            T h1, T h2, T h3, bool fresh)
{
    // dpsi = B4 (f+4 - f-4) + B3 (f+3 - f-3) + B2 (f+2 - f-2) + B1 (f+1 - f-1), one row pair
    // at a time (same operand order as absorbingBoundaryCondition.c:198-203)
    T acc[4];
    {
        const T bk[4] = {(T)RTM_B4, (T)RTM_B3, (T)RTM_B2, (T)RTM_B1};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            T mk[4], pk[4];
            ld4(psi - (ptrdiff_t)(4 - k) * (ptrdiff_t)P, mk);
            ld4(psi + (ptrdiff_t)(4 - k) * (ptrdiff_t)P, pk);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const T term = bk[k] * (pk[j] - mk[j]);
                acc[j] = k == 0 ? term : acc[j] + term;
            }
        }
    }
    T x4[4];
    if (fresh) {                          // first step of a pass: xi starts from zero
#pragma unroll
        for (int j = 0; j < 4; ++j) x4[j] = (T)0;
    } else {
        ld4(xi, x4);
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int z = zq + j;
        if (z >= zlo && z < zhi) {
            const T dp = acc[j] * h1;
            const T xn = bb * x4[j] + ab * (d2x_w<T>(W, j) * h3 + dp);
            x4[j] = xn;
            v[j] = v[j] + (cf[j] * h2) * (dp + xn);
        }
    }
    st4(xi, x4);
}

// Top/bottom strip (z-derivative) correction of one quad.  psi, xi, ab, bb addressed at the
// quad's first cell in 4-aligned strip arrays (psi readable at -4..+7).
template <typename T>
__device__ __forceinline__ void cpml_z_quad(const T *psi, T *xi, const float *ab, const float *bb,
                                            const T (&zz)[12], const T (&cf)[4], T (&v)[4], int zq,
                                            int zlo, int zhi, T h1, T h2, T h3, bool fresh)
{
    T q[12];
    {
        T a0[4], a1[4], a2[4];
        ld4(psi - 4, a0);
        ld4(psi, a1);
        ld4(psi + 4, a2);
#pragma unroll
        for (int j = 0; j < 4; ++j) { q[j] = a0[j]; q[4 + j] = a1[j]; q[8 + j] = a2[j]; }
    }
    T x4[4];
    if (fresh) {                          // first step of a pass: xi starts from zero
#pragma unroll
        for (int j = 0; j < 4; ++j) x4[j] = (T)0;
    } else {
        ld4(xi, x4);
    }
    const float4 av = *reinterpret_cast<const float4 *>(ab);
    const float4 bv = *reinterpret_cast<const float4 *>(bb);
    const float aa[4] = {av.x, av.y, av.z, av.w}, bbv[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int z = zq + j;
        if (z >= zlo && z < zhi) {
            const T dp = dpsi_z<T>(q, j) * h1;
            const T xn = (T)bbv[j] * x4[j] + (T)aa[j] * (d2z_q<T>(zz, j) * h3 + dp);
            x4[j] = xn;
            v[j] = v[j] + (cf[j] * h2) * (dp + xn);
        }
    }
    st4(xi, x4);
}

// Loads the 12-value z line (zm | centre | zp) of column row `row` of a halo tile.
template <typename T>
__device__ __forceinline__ void z_line(const T *tile, int row, int zi, const T (&c)[4], T (&zz)[12])
{
    T zm[4], zp[4];
    ld4(tile + row * SZ + zi - 4, zm);
    ld4(tile + row * SZ + zi + 4, zp);
#pragma unroll
    for (int j = 0; j < 4; ++j) { zz[j] = zm[j]; zz[4 + j] = c[j]; zz[8 + j] = zp[j]; }
}

// All CPML corrections of one quad (column c, quad qi) of a boundary tile, in the
// reference's strip order left, top, right, bottom, on the stencil result in O.
template <typename T>
__device__ __forceinline__ void cpml_quad_all(const StepArgs<T> &a, const T *su, const T *scf, T *O,
                                              int x0, int z0, int c, int qi)
{
    const Geom &g = a.g;
    const size_t P = (size_t)g.pitch;
    const int x = x0 + c, zq = z0 + 4 * qi;
    const bool zx = zq + 4 > 4 && zq < g.dimz - 4;              // quad meets [4, dimZ-4)
    const bool inL = zx && x >= 4 && x < g.thl - 4;
    const bool inR = zx && x >= g.dimx - g.thr + 4 && x < g.dimx - 4;
    const bool inT = zq + 4 > 4 && zq < g.thu - 4;               // every column (the quirk)
    const bool inB = x >= 4 && x < g.dimx - 4 && zq + 4 > g.dimz - g.thd + 4 && zq < g.dimz - 4;
    if (!(inL || inR || inT || inB)) return;
    const bool fresh = (a.flags & F_STRIPS_FRESH) != 0;
    T v[4], cf[4];
    ld4(O + c * TZ + 4 * qi, v);
    ld4(scf + c * TZ + 4 * qi, cf);
    const T *col = su + (c + HALO) * SZ + 4 * qi + HALO;         // centre quad in the halo tile
    if (inL || inR) {
        T W[9][4];
#pragma unroll
        for (int m = 0; m < 9; ++m) ld4(col + (m - 4) * SZ, W[m]);
        if (inL)
            cpml_x_quad<T>(a.psi_l + (size_t)x * P + zq, a.xi_l + (size_t)x * P + zq, P, (T)a.a_l[x],
                           (T)a.b_l[x], W, cf, v, zq, 4, g.dimz - 4, a.h1, a.h2, a.h3, fresh);
        if (inT) {
            T zz[12];
            z_line<T>(su, c + HALO, 4 * qi + HALO, W[4], zz);
            cpml_z_quad<T>(a.psi_t + (size_t)x * g.st + zq, a.xi_t + (size_t)x * g.st + zq, a.a_t + zq,
                           a.b_t + zq, zz, cf, v, zq, 4, g.thu - 4, a.h1, a.h2, a.h3, fresh);
        }
        if (inR) {
            const int li = x - (g.dimx - g.thr);
            cpml_x_quad<T>(a.psi_r + (size_t)li * P + zq, a.xi_r + (size_t)li * P + zq, P, (T)a.a_r[li],
                           (T)a.b_r[li], W, cf, v, zq, 4, g.dimz - 4, a.h1, a.h2, a.h3, fresh);
        }
        if (inB) {
            T zz[12];
            z_line<T>(su, c + HALO, 4 * qi + HALO, W[4], zz);
            const int lq = zq - g.zb0;
            cpml_z_quad<T>(a.psi_b + (size_t)x * g.sb + lq, a.xi_b + (size_t)x * g.sb + lq, a.a_b + lq,
                           a.b_b + lq, zz, cf, v, zq, g.dimz - g.thd + 4, g.dimz - 4, a.h1, a.h2, a.h3, fresh);
        }
    } else {
        T c4[4], zz[12];
        ld4(col, c4);
        z_line<T>(su, c + HALO, 4 * qi + HALO, c4, zz);
        if (inT)
            cpml_z_quad<T>(a.psi_t + (size_t)x * g.st + zq, a.xi_t + (size_t)x * g.st + zq, a.a_t + zq,
                           a.b_t + zq, zz, cf, v, zq, 4, g.thu - 4, a.h1, a.h2, a.h3, fresh);
        if (inB) {
            const int lq = zq - g.zb0;
            cpml_z_quad<T>(a.psi_b + (size_t)x * g.sb + lq, a.xi_b + (size_t)x * g.sb + lq, a.a_b + lq,
                           a.b_b + lq, zz, cf, v, zq, g.dimz - g.thd + 4, g.dimz - 4, a.h1, a.h2, a.h3, fresh);
        }
    }
    st4(O + c * TZ + 4 * qi, v);
}

// One pass over every quad of a boundary tile (threads take quads from a compact list).
template <typename T, int TXC>
__device__ __forceinline__ void cpml_pass(const StepArgs<T> &a, const T *su, const T *scf, T *O,
                                          int x0, int z0, int z1)
{
    const Geom &g = a.g;
    const int ncol = min(TXC, g.dimx - x0);
    const int nq = (min(z1, g.dimz) - z0 + 3) >> 2;
    const int n = ncol * nq;
    for (int item = threadIdx.x; item < n; item += blockDim.x)
        cpml_quad_all<T>(a, su, scf, O, x0, z0, item / nq, item % nq);
}

template <typename T, int BWD, int WARPS>
__device__ __forceinline__ void step_tile(const StepArgs<T> &a, const T *stage, int t, bool &psi_ready,
                                          float *red)
{
    using Cfg = StepCfg<T, WARPS, BWD>;
    constexpr int TXC = Cfg::TXC, UT = Cfg::UT, PT = Cfg::PT;
    const Geom &g = a.g;
    const int flags = a.flags;
    const bool recon = BWD && (flags & F_RECON);
    const T *su = stage;                 // current field + halo   [TXC+8][SZ]
    T *sprv = const_cast<T *>(stage) + UT;   // previous field [TXC][TZ]; boundary tiles reuse
                                             // it as the output tile once it has been read
    const T *scf = stage + UT + PT;      // coef                    [TXC][TZ]
    const T *ss = stage + UT + 2 * PT;   // source field + halo     (backward reconstruction)
    const T *ssp = stage + 2 * UT + 2 * PT;

    int xt, zt;
    tile_coords(g, t, xt, zt);
    const int x0 = xt * TXC, z0 = ztile_origin(g, zt), zend = ztile_end(g, zt);
    const int x1 = x0 + TXC, z1 = min(zend, z0 + TZ);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int zq = z0 + 4 * lane;        // first z of this thread's quad
    const int xb = x0 + warp * RXC;      // first column of this thread
    const int row0 = warp * RXC;         // halo-tile row of column xb - 4
    const int zi = 4 * lane + HALO;      // halo-tile index of the quad's first cell
    const bool zok = zq < min(z1, g.dimz);
    const size_t P = (size_t)g.pitch;

    // ---- tile classification (uniform over the CTA)
    const bool in_domain = x0 >= 4 && x1 <= g.dimx - 4 && z0 >= 4 && z1 <= g.dimz - 4;
    const bool cpml_t = !(flags & F_NO_CPML) &&
                        (x0 < g.thl - 4 || x1 > g.dimx - g.thr + 4 || z0 < g.thu - 4 ||
                         z1 > g.dimz - g.thd + 4);
    const bool src_t = (flags & (BWD ? F_RECON_SRC : F_SRC)) && g.xs >= x0 && g.xs < x1 &&
                       g.zs >= z0 && g.zs < z1;
    const bool rec_t = (flags & (F_RECORD | F_OVERWRITE)) && g.zrec >= z0 && g.zrec < z1;
    const bool in_region = x0 >= g.rx0 && x1 <= g.rx1 && z0 >= g.rz0 && z1 <= g.rz1;
    const bool near_ring = x0 < g.rx1 + 4 && x1 > g.rx0 - 4 && z0 < g.rz1 + 4 && z1 > g.rz0 - 4;
    const bool ring_t = (flags & (BWD ? F_RECON : F_RING_SAVE)) && near_ring && !in_region;
    const bool int_full = x0 >= g.thl && x1 <= g.thl + g.nx && z0 >= g.thu && z1 <= g.thu + g.nz;
    const bool int_any = x0 < g.thl + g.nx && x1 > g.thl && z0 < g.thu + g.nz && z1 > g.thu;
    const bool snap_t = !BWD && (flags & F_SNAP_SAVE) && int_any;
    const bool snap_fast = snap_t && int_full && a.store_prec == 0 && !src_t;
    const bool scaled = !BWD && a.store_prec != 0 && (ring_t || snap_t);
    const bool image_t = BWD && (flags & F_IMAGE) && int_any;
    const bool image_fast = image_t && int_full && !rec_t && !src_t;
    const bool boundary = !in_domain || cpml_t || src_t || rec_t || ring_t || (snap_t && !snap_fast) ||
                          (image_t && !image_fast) || (flags & F_NO_STENCIL);

    // ================= the propagated field: leapfrog =================
    T v[RXC][4];
    {
        T W[9][4];
#pragma unroll
        for (int m = 0; m < 8; ++m) ld4(su + (row0 + m) * SZ + zi, W[m]);
#pragma unroll
        for (int r = 0; r < RXC; ++r) {
            ld4(su + (row0 + r + 8) * SZ + zi, W[8]);
            T zz[12];
            z_line<T>(su, row0 + r + 4, zi, W[4], zz);
            T prv[4], cf[4];
            ld4(sprv + (row0 + r) * TZ + 4 * lane, prv);
            ld4(scf + (row0 + r) * TZ + 4 * lane, cf);
            const int x = xb + r;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const T s = cf[j] * lap8<T>(W, zz, j) + (T)2.0f * W[4][j] - prv[j];
                if (!boundary) v[r][j] = s;
                else {
                    const int z = zq + j;
                    v[r][j] = (!(flags & F_NO_STENCIL) && x >= 4 && x < g.dimx - 4 && z >= 4 &&
                               z < g.dimz - 4) ? s : prv[j];
                }
            }
            if (!boundary) {
                if (zok && x < g.dimx) st4(a.u_next + (size_t)x * P + zq, v[r]);
                if (snap_fast) st4(reinterpret_cast<T *>(a.store) + (size_t)(x - g.thl) * P + zq, v[r]);
            }
#pragma unroll
            for (int m = 0; m < 8; ++m)
#pragma unroll
                for (int j = 0; j < 4; ++j) W[m][j] = W[m + 1][j];
        }
    }

    if (boundary) {
        // ---- CPML: stencil results to the output tile, four compact strip passes
        if (cpml_t) {
            if (!psi_ready) {            // psi of this step comes from the preceding k_psi
                griddep_wait();
                psi_ready = true;
            }
#pragma unroll
            for (int r = 0; r < RXC; ++r) st4(sprv + (row0 + r) * TZ + 4 * lane, v[r]);
            __syncthreads();
            cpml_pass<T, TXC>(a, su, scf, sprv, x0, z0, z1);
            __syncthreads();
#pragma unroll
            for (int r = 0; r < RXC; ++r) ld4(sprv + (row0 + r) * TZ + 4 * lane, v[r]);
        }
        // ---- the thread's own cells: source, receivers, stores, storage
        float mx = 0.0f;
#pragma unroll
        for (int r = 0; r < RXC; ++r) {
            const int x = xb + r;
            if (!(zok && x < g.dimx)) continue;
            if (!BWD && src_t && x == g.xs) {
                T cf[4];
                ld4(scf + (row0 + r) * TZ + 4 * lane, cf);
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (zq + j == g.zs) v[r][j] = add_source<T>(a.wavelet, a.t, v[r][j], cf[j]);
            }
            if (rec_t && g.zrec >= zq && g.zrec < zq + 4) {
                const int jr = g.zrec - zq;
                if (!BWD && (flags & F_RECORD)) {
                    const int n = a.rec_cnt[x], f = a.rec_first[x];
                    for (int q = 0; q < n; ++q) a.rec_out[(size_t)(f + q) * g.nt + a.t] = v[r][jr];
                }
                if (BWD && (flags & F_OVERWRITE)) {
                    const int q = a.rec_last[x];
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        if (j == jr && q >= 0) v[r][j] = (T)a.seis_row[q];
                }
            }
            st4(a.u_next + (size_t)x * P + zq, v[r]);
            const bool ring_q = ring_t && ring_quad(g, x, zq);
            if (!BWD && (ring_q || snap_t)) {
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int z = zq + j;
                    if (z >= g.dimz) continue;
                    size_t o = (size_t)-1;
                    if (ring_q) {
                        const int idx = ring_index(g, x, z);
                        if (idx >= 0) o = (size_t)idx;
                    }
                    if (snap_t && in_interior(g, x, z)) o = (size_t)(x - g.thl) * P + z;
                    if (o != (size_t)-1) {
                        if (a.store_prec == 0) reinterpret_cast<T *>(a.store)[o] = v[r][j];
                        else mx = fmaxf(mx, fabsf((float)v[r][j]));
                    }
                }
            }
        }
        if (scaled) {   // 16-bit storage: per-step, per-tile max-abs scale, then quantise
            mx = block_max<WARPS>(mx, red);
            const float target = a.store_prec == 2 ? kFp16Target : kBf16Target;
            // Ahead of the wavefront a tile can hold only denormal-size values; clamping the
            // maximum keeps target/max finite (an unclamped inverse overflows to inf and
            // 0 * inf would store NaN).
            const float scale = fmaxf(mx, 1e-30f) / target;
            const float inv = 1.0f / scale;
            if (threadIdx.x == 0) a.store_scale[t] = scale;
#pragma unroll
            for (int r = 0; r < RXC; ++r)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int x = xb + r, z = zq + j;
                    if (!zok || x >= g.dimx || z >= g.dimz) continue;
                    if (ring_t && ring_quad(g, x, zq)) {
                        const int idx = ring_index(g, x, z);
                        if (idx >= 0) store_put<T>(a.store, a.store_prec, (size_t)idx, v[r][j], inv);
                    }
                    if (snap_t && in_interior(g, x, z))
                        store_put<T>(a.store, a.store_prec, (size_t)(x - g.thl) * P + z, v[r][j], inv);
                }
        }
    }
    if (!BWD) return;

    // ================= backward: source reconstruction and imaging =================
    if (!recon && !image_t) return;
    const float tile_scale = (a.store_prec != 0 && a.store_scale) ? a.store_scale[t] : 1.0f;
    const int tsrc = g.nt + 1 - a.t;     // forward step whose source term is undone
    T W[9][4];
    if (recon) {
#pragma unroll
        for (int m = 0; m < 8; ++m) ld4(ss + (row0 + m) * SZ + zi, W[m]);
    }
#pragma unroll
    for (int r = 0; r < RXC; ++r) {
        const int x = xb + r;
        const bool col_ok = zok && x < g.dimx;
        T s[4];
        if (recon) {
            ld4(ss + (row0 + r + 8) * SZ + zi, W[8]);
            T zz[12];
            z_line<T>(ss, row0 + r + 4, zi, W[4], zz);
            T sp[4], cf[4];
            ld4(ssp + (row0 + r) * TZ + 4 * lane, sp);
            ld4(scf + (row0 + r) * TZ + 4 * lane, cf);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const T sv = cf[j] * lap8<T>(W, zz, j) + (T)2.0f * W[4][j] - sp[j];
                if (in_region) s[j] = sv;
                else {
                    const int z = zq + j;
                    s[j] = (x >= g.rx0 && x < g.rx1 && z >= g.rz0 && z < g.rz1) ? sv : sp[j];
                }
            }
            if (col_ok && src_t && x == g.xs) {
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (zq + j == g.zs) s[j] = add_source<T>(a.wavelet, tsrc, s[j], cf[j]);
            }
            if (col_ok && ring_t && ring_quad(g, x, zq)) {
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int z = zq + j;
                    const int idx = z < g.dimz ? ring_index(g, x, z) : -1;
                    if (idx >= 0) s[j] = store_get<T>(a.store, a.store_prec, (size_t)idx, tile_scale);
                }
            }
            if (col_ok) st4(a.s_next + (size_t)x * P + zq, s);
#pragma unroll
            for (int m = 0; m < 8; ++m)
#pragma unroll
                for (int j = 0; j < 4; ++j) W[m][j] = W[m + 1][j];
        }
        if (image_t && col_ok) {
            if (!recon) {
                if (flags & F_IMAGE_SNAP) {
                    const size_t o = (size_t)(x - g.thl) * P + zq;
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        s[j] = (x >= g.thl && x < g.thl + g.nx)
                                   ? store_get<T>(a.s_snap, a.store_prec, o + j, tile_scale) : (T)0;
                } else {
                    ld4(a.s_fixed + (size_t)x * P + zq, s);
                }
            }
            // the receiver quad this thread stored above (reloaded rather than kept live
            // through the reconstruction, which keeps the kernel at two CTAs per SM)
            T rv[4];
            ld4(a.u_next + (size_t)x * P + zq, rv);
            if (image_fast) {
                const size_t o = (size_t)(x - g.thl) * P + zq;
                image_quad<T>(a.img + o, a.slf + o, s, rv);
            } else {
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int z = zq + j;
                    if (z < g.dimz && in_interior(g, x, z)) {
                        const size_t o = (size_t)(x - g.thl) * P + z;
                        a.img[o] += (double)s[j] * (double)rv[j];
                        a.slf[o] += (double)s[j] * (double)s[j];
                    }
                }
            }
        }
    }
}

template <typename T, int BWD, int WARPS>
__global__ void __launch_bounds__(WARPS * 32, (sizeof(T) == 4 && WARPS <= 8) ? 2 : 1)
    k_step(const __grid_constant__ StepMaps m, const __grid_constant__ StepArgs<T> a)
{
    using Cfg = StepCfg<T, WARPS, BWD>;
    constexpr int UT = Cfg::UT, PT = Cfg::PT, STAGE = Cfg::STAGE, NS = Cfg::NS, TXC = Cfg::TXC;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T *stage0 = reinterpret_cast<T *>(smem_raw);
    __shared__ __align__(8) uint64_t full[NS];
    __shared__ int tile_of[NS];          // tile held by each stage (>= tiles: none)
    __shared__ float red[WARPS];
    const Geom &g = a.g;
    const bool recon = BWD && (a.flags & F_RECON);
    const uint32_t tile_bytes = (uint32_t)(sizeof(T) * (recon ? 2 * UT + 3 * PT : UT + 2 * PT));

    if (threadIdx.x == 0) {
#pragma unroll
        for (int s = 0; s < NS; ++s) mbar_init(&full[s], 1);
        fence_barrier_init();
    }
    __syncthreads();
    // Static balanced schedule over the boundary-first order (tile_coords): CTA b takes the
    // boundary tiles b, b + G, ... (the slow ones: CPML, ring, source, receivers), then its
    // share of the interior tiles.  The r = nb mod G CTAs that carry one boundary tile more
    // take kBalance interior tiles fewer, a boundary tile counting as 1 + kBalance interior
    // ones.  The interior goes out in rounds -- round j gives one tile to every CTA with more
    // than j interior tiles, in CTA order -- so that all CTAs sweep the grid together (their
    // halos and, backward, the image and source rows stay in L2).  Measured on 3400 x 700
    // against plain round-robin: forward 24.5 -> 22.6 us, backward 38.2 -> 30.9 us per step.
    // Every tile is taken exactly once.  A stage with no tile left still completes its
    // barrier phase.
    constexpr int kBalance = BWD ? 2 : 3;
    const int G = gridDim.x, b = blockIdx.x;
    const int nb = boundary_tiles(g), ni = g.tiles - nb;
    const int r = nb % G;
    const int kb = nb / G + (b < r ? 1 : 0);                 // boundary tiles of this CTA
    int xlo = (ni + r * kBalance) / G, xhi = xlo - kBalance;  // interior tiles for b >= r, b < r
    if (xhi < 0) { xhi = 0; xlo = ni / (G - r); }
    const int rem = ni - r * xhi - (G - r) * xlo;            // one more each: b >= r first
    const int ex = max(0, rem - (G - r)), nc = min(rem, G - r);
    // CTA groups by interior count: [0,ex) xhi+1, [ex,r) xhi, [r,r+nc) xlo+1, [r+nc,G) xlo
    const int cnt = b < r ? xhi + (b < ex ? 1 : 0) : xlo + (b - r < nc ? 1 : 0);
    auto interior = [&](int j) {          // position of this CTA's j-th interior tile
        const int lo[4] = {0, ex, r, r + nc}, hi[4] = {ex, r, r + nc, G};
        const int c[4] = {xhi + 1, xhi, xlo + 1, xlo};
        int p = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            p += min(j, c[k]) * (hi[k] - lo[k]);               // rounds before j
            if (c[k] > j) p += max(0, min(b, hi[k]) - lo[k]);  // CTAs before b in round j
        }
        return p;
    };
    auto issue = [&](int i, int s) {
        const int t = i < kb ? b + i * G : (i - kb < cnt ? nb + interior(i - kb) : g.tiles);
        tile_of[s] = t;
        if (t >= g.tiles) {
            mbar_arrive(&full[s]);
            return;
        }
        int xt, zt;
        tile_coords(g, t, xt, zt);
        const int x0 = xt * TXC, z0 = ztile_origin(g, zt);
        T *st = stage0 + (size_t)s * STAGE;
        mbar_arrive_expect_tx(&full[s], tile_bytes);
        tma_load_2d(st, &m.cur, z0 - HALO, x0 - HALO, &full[s]);
        tma_load_2d(st + UT, &m.prev, z0, x0, &full[s]);
        tma_load_2d(st + UT + PT, &m.coef, z0, x0, &full[s]);
        if (recon) {
            tma_load_2d(st + UT + 2 * PT, &m.scur, z0 - HALO, x0 - HALO, &full[s]);
            tma_load_2d(st + 2 * UT + 2 * PT, &m.sprev, z0, x0, &full[s]);
        }
    };
    if (threadIdx.x == 0) {
        for (int s = 0; s < NS; ++s) issue(s, s);
    }
    // The next kernel in the stream may be scheduled now; it waits for this grid's
    // completion (griddepcontrol.wait) before it touches anything this grid writes.
    griddep_launch();
    bool psi_ready = false;
    for (int i = 0;; ++i) {
        const int s = i % NS;
        const uint32_t par = (uint32_t)((i / NS) & 1);
        const bool ok = mbar_wait_bounded(&full[s], par, 2000000000ull);
        if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0) {
                atomicOr(a.status, ST_TMA_TIMEOUT);
                for (int k = 0; k < NS; ++k) {   // let the copies in flight land
                    const int ii = i + k;
                    mbar_wait_bounded(&full[ii % NS], (uint32_t)((ii / NS) & 1), 1000000000ull);
                }
            }
            __syncthreads();
            return;
        }
        const int t = *reinterpret_cast<volatile int *>(&tile_of[s]);
        if (t >= g.tiles) break;                 // tiles are consumed in issue order
        step_tile<T, BWD, WARPS>(a, stage0 + (size_t)s * STAGE, t, psi_ready, red);
        __syncthreads();                         // stage s is free again
        if (threadIdx.x == 0) issue(i + NS, s);
    }
}
