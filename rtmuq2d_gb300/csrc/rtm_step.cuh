// rtm_step.cuh -- the persistent, TMA-pipelined time-step kernel k_step (included by
// rtm_kernels.cu).
//
// Grid: a fixed number of CTAs (filling the SMs); each CTA takes a static, balanced share of
// the TX x 128 tiles of the step (boundary tiles first).  Each tile's inputs -- the current
// field with a 4-cell halo (8 columns in x on the side CPML tiles), u_prev and coef
// (backward reconstruction: also the source field with halo and its predecessor) -- arrive by
// TMA 2-D copies into one of NS shared-memory stages; thread 0 refills a stage as soon as its
// tile is done, so NS-1 tiles are in flight while one is computed.
//
// Per tile, every thread owns RXC = 2 columns x 4 consecutive z cells, keeps a 9-column
// register window along x and reads z neighbours as aligned 16-byte vectors:
//   * 8th-order leapfrog (SRC/stencilDFM.c:17-29);
//   * on tiles touching the CPML, the whole CPML update of the step
//     (SRC/absorbingBoundaryCondition.c:150-361): psi of the step computed in the tile from
//     the halo of the current field (the reference's psi loops, :171-189, 219-235, 265-281,
//     312-328), then the corrections of the four strips in the reference's order left, top,
//     right, bottom (:191-357).  psi is double-buffered (read: the previous step's, written:
//     this step's), so that a tile can rebuild the psi cells of its neighbours that its own
//     corrections read while those neighbours write theirs;
//   * source injection (SRC/forward_modeling.c:105-109) or receiver overwrite
//     (backward_modeling.c:277-281), trace recording, boundary-ring or snapshot storage
//     (FP32, or BF16/FP16 with a per-step, per-tile max-abs scale);
//   * backward: reverse-time source reconstruction on the stencil-only region and the FP64
//     cross-correlation image (SRC/image_conditions.c:20-33).
// Consecutive steps chain by programmatic dependent launch: a step's CTAs start while the
// previous step's last CTAs finish and issue their first tile loads after griddepcontrol.wait.

__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void griddep_launch() { asm volatile("griddepcontrol.launch_dependents;" :::); }

template <typename T, int WARPS, int BWD>
struct StepCfg {
    static constexpr int TXC = WARPS * RXC;                       // x columns per tile
    static constexpr int UT8 = (TXC + 4 * HALO) * SZ;             // current field, 8-column x halo
    static constexpr int UT = (TXC + 2 * HALO) * SZ;              // halo tile, elements
    static constexpr int PT = TXC * TZ;                           // plain tile, elements
    static constexpr int STAGE = BWD ? UT8 + UT + 3 * PT : UT8 + 2 * PT;
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

// First derivative (times dx) of 4 cells along x from a 9-column window W[k] = f(x-4+k):
// B4 (f+4 - f-4) + B3 (f+3 - f-3) + B2 (f+2 - f-2) + B1 (f+1 - f-1), the operand order of
// absorbingBoundaryCondition.c:177-181 (psi) and :198-203 (dpsi).
template <typename T>
__device__ __forceinline__ T d1x_w(const T (&W)[9][4], int j)
{
    return (T)RTM_B4 * (W[8][j] - W[0][j]) + (T)RTM_B3 * (W[7][j] - W[1][j])
         + (T)RTM_B2 * (W[6][j] - W[2][j]) + (T)RTM_B1 * (W[5][j] - W[3][j]);
}
// The same along z from a 12-value line q (q[4+j] is cell j).
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

// The x-strip (left or right) whose psi array holds column x, if any: the left array covers
// [0, th_left), the right one [dimX-th_right, dimX).  Sets the column's arrays (old psi, new
// psi, xi; row stride pitch) and profile values; *upd: x is one of the strip's psi /
// correction columns, [4, th_left-4) or [dimX-th_right+4, dimX-4)
// (absorbingBoundaryCondition.c:174, 266).  The other columns of an array keep their psi,
// which the corrections next to them read.
template <typename T>
__device__ __forceinline__ bool x_strip(const StepArgs<T> &a, int x, const T *&po, T *&pn, T *&xi, T &ab,
                                        T &bb, bool &upd)
{
    const Geom &g = a.g;
    const size_t P = (size_t)g.pitch;
    if (x >= 0 && x < g.thl) {
        po = a.psi_l + (size_t)x * P; pn = a.psn_l + (size_t)x * P; xi = a.xi_l + (size_t)x * P;
        ab = (T)a.a_l[x]; bb = (T)a.b_l[x];
        upd = x >= 4 && x < g.thl - 4;
        return true;
    }
    if (x >= g.dimx - g.thr && x < g.dimx) {
        const int li = x - (g.dimx - g.thr);
        po = a.psi_r + (size_t)li * P; pn = a.psn_r + (size_t)li * P; xi = a.xi_r + (size_t)li * P;
        ab = (T)a.a_r[li]; bb = (T)a.b_r[li];
        upd = li >= 4 && x < g.dimx - 4;
        return true;
    }
    return false;
}

// psi of this step on 4 cells of an x-strip column from the 9-column window of u and the
// previous psi (absorbingBoundaryCondition.c:177-181, 269-273): psi = b psi + a D1x(u) / dx on
// z in [4, dimZ-4); the other cells keep their psi.
template <typename T>
__device__ __forceinline__ void psi_x_new(const T (&W)[9][4], T (&ps)[4], T ab, T bb, T h1, int zq, int dimz)
{
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if (zq + j >= 4 && zq + j < dimz - 4) ps[j] = bb * ps[j] + ab * d1x_w<T>(W, j) * h1;
}

// z-strips of a top or bottom tile that touches no x-strip, one column per thread: the band's
// nq <= 16 quads of a column go to a half-warp (lanes 0-15: the warp's first column, 16-31:
// its second), rather than both columns to the lanes that own the quads, which on a tile
// holding a 13-quad band left 19 of 32 lanes idle through the whole correction.  The same
// arithmetic as cpml_fused's z-strip part (absorbingBoundaryCondition.c:219-263, 312-357): psi
// of the quad from the tile's z line, the neighbours' psi by shuffles within the half-warp,
// then xi and the correction term, which goes back by shuffle to the lane that owns the quad
// and is added to v there.  qb: the band's first quad in the tile; top: the top band.
template <typename T, int WARPS>
__device__ __forceinline__ void cpml_z_half(const StepArgs<T> &a, const T *su, const T *scf, T (&dzo)[RXC][4],
                                            bool (&czo)[RXC], int x0, int z0, int qb, int nq, bool top)
{
    static_assert(RXC == 2, "one column per half-warp");
    const Geom &g = a.g;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int k = lane & 15, c = warp * RXC + (lane >> 4), x = x0 + c;
    const bool act = k < nq && x < g.dimx;               // (column, quad) in the band's array
    const int qi = qb + min(k, nq - 1), zq = z0 + 4 * qi;
    const T h1 = a.h1, h2 = a.h2, h3 = a.h3;
    const int zlo = top ? 4 : g.dimz - g.thd + 4, zhi = top ? g.thu - 4 : g.dimz - 4;
    const bool qC = zq + 4 > zlo && zq < zhi;            // the quad holds correction rows
    const size_t o = top ? (size_t)x * g.st + zq : (size_t)x * g.sb + (zq - g.zb0);
    T ps[4] = {(T)0, (T)0, (T)0, (T)0}, xz[4] = {(T)0, (T)0, (T)0, (T)0};
    float aa[4] = {0.f, 0.f, 0.f, 0.f}, bz[4] = {0.f, 0.f, 0.f, 0.f};
    if (act) {
        ld4((top ? a.psi_t : a.psi_b) + o, ps);
        if (qC) ld4((top ? a.xi_t : a.xi_b) + o, xz);
        const float4 av = *reinterpret_cast<const float4 *>(top ? a.a_t + zq : a.a_b + (zq - g.zb0));
        const float4 bv = *reinterpret_cast<const float4 *>(top ? a.b_t + zq : a.b_b + (zq - g.zb0));
        aa[0] = av.x; aa[1] = av.y; aa[2] = av.z; aa[3] = av.w;
        bz[0] = bv.x; bz[1] = bv.y; bz[2] = bv.z; bz[3] = bv.w;
    }
    T zz[12];
    {
        const int zi = 4 * qi + HALO;
        T c4[4];
        ld4(su + (c + HALO) * SZ + zi, c4);
        z_line<T>(su, c + HALO, zi, c4, zz);
    }
    if (act) {
        if (x >= 4 && x < g.dimx - 4) {                   // psi cells: x in [4, dimX-4)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int z = zq + j;
                if (z >= zlo && z < zhi) ps[j] = (T)bz[j] * ps[j] + (T)aa[j] * dpsi_z<T>(zz, j) * h1;
            }
        }
        st4((top ? a.psn_t : a.psn_b) + o, ps);
    }
    T q[12];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const T up = __shfl_up_sync(0xffffffffu, ps[j], 1, 16);
        const T dn = __shfl_down_sync(0xffffffffu, ps[j], 1, 16);
        q[j] = k > 0 ? up : (T)0;
        q[4 + j] = ps[j];
        q[8 + j] = k < 15 ? dn : (T)0;
    }
    T dZ[4] = {(T)0, (T)0, (T)0, (T)0};
    if (act && qC && (top || (x >= 4 && x < g.dimx - 4))) {   // the top rows cover every column
        T cf[4];
        ld4(scf + c * TZ + 4 * qi, cf);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int z = zq + j;
            if (z >= zlo && z < zhi) {
                const T dp = dpsi_z<T>(q, j) * h1;
                const T xn = (T)bz[j] * xz[j] + (T)aa[j] * (d2z_q<T>(zz, j) * h3 + dp);
                xz[j] = xn;
                dZ[j] = (cf[j] * h2) * (dp + xn);
            }
        }
        st4((top ? a.xi_t : a.xi_b) + o, xz);
    }
    // the correction terms back to the lanes owning the quads (lane = quad of the tile);
    // czo: the owner's column gets a z correction on this quad
    const int kk = lane - qb;
    const bool mine = kk >= 0 && kk < nq;
    const int src = mine ? kk : 0;
    const int zo = z0 + 4 * lane;
    const bool qCo = zo + 4 > zlo && zo < zhi;
#pragma unroll
    for (int r = 0; r < RXC; ++r) {
#pragma unroll
        for (int j = 0; j < 4; ++j) dzo[r][j] = __shfl_sync(0xffffffffu, dZ[j], 16 * r + src);
        const int xo = x0 + warp * RXC + r;
        czo[r] = mine && qCo && xo < g.dimx && (top || (xo >= 4 && xo < g.dimx - 4));
    }
}

// The CPML update of a tile touching a strip, on the stencil results v of the thread's own
// cells (RXC columns x one 4-cell quad), in registers.  Per strip cell, in the reference's
// order left, top, right, bottom: dpsi = D1(psi)/dx, xi = b xi + a (D2(u)/dx^2 + dpsi),
// u_next += coef dx^2 (dpsi + xi) (absorbingBoundaryCondition.c:191-217, 237-263, 283-310,
// 330-357), with the psi of this step computed here:
//   * x-strips (left, right; only the side tiles): a thread computes the psi of its own cells
//     (from the 9-column window of u) into the stage's u_prev tile, which only it has read;
//     the tile computes the psi of the 4 columns on either side (from the 8-column halo) into
//     the u rows of the outermost halo columns, which nothing reads after that; the
//     corrections read both;
//   * z-strips (top, bottom): every tile row holds a whole band plus 4 rows, so a lane
//     computes the psi of a quad from the tile's z line and takes its neighbours' from the
//     lanes above and below (warp shuffles).  When the band has at most 16 quads (a CPML of
//     up to 64 cells) it goes to half-warps, one column per thread (cpml_z_half), and the
//     correction terms come back to the quads' owners; otherwise each lane does its own quad
//     of both its columns.
// u8: the stage's current-field area (tile column c at row c + 8; 4-halo tiles fill rows
// 4 .. TXC + 12); sprv: the stage's u_prev tile.  The previous psi, xi and the profiles come
// from global memory, each thread's loads issued before the work that needs them.
template <typename T, int WARPS>
__device__ __forceinline__ void cpml_fused(const StepArgs<T> &a, T *u8, T *sprv, const T *scf, T (&v)[RXC][4],
                                           int x0, int z0, int z1)
{
    constexpr int TXC = WARPS * RXC;
    constexpr int NTHR = WARPS * 32;
    constexpr int RING_ITEMS = 8 * 32;                      // 4 columns either side x 32 quads
    constexpr int RPT = (RING_ITEMS + NTHR - 1) / NTHR;    // ring items per thread
    const Geom &g = a.g;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int zq = z0 + 4 * lane;
    const int zi = 4 * lane + HALO;                 // the quad's first cell within a halo column
    const T *su = u8 + HALO * SZ;                   // 4-halo view: tile column c at row c + HALO
    const int zend = min(z1, g.dimz);
    const bool own = zq < zend;                     // the quad belongs to this tile
    const bool qT = zq + 4 > 4 && zq < g.thu - 4;                        // top correction rows
    const bool qB = zq + 4 > g.dimz - g.thd + 4 && zq < g.dimz - 4;      // bottom ones
    const bool tX = x0 < g.thl - 4 || x0 + TXC > g.dimx - g.thr + 4;     // tile-uniform
    const bool tZ = z0 < g.thu - 4 || zend > g.dimz - g.thd + 4;
    // the quad in the top psi array (rows [0, th_up)) or the bottom one (rows [zb0, dimZ))
    const bool inTa = own && zq < g.thu;
    const bool inBa = own && !inTa && zq >= g.zb0;
    const T h1 = a.h1, h2 = a.h2, h3 = a.h3;

    // ---- x-strips
    T dX[RXC][4];
    bool cX[RXC];
#pragma unroll
    for (int r = 0; r < RXC; ++r) {
        cX[r] = false;
#pragma unroll
        for (int j = 0; j < 4; ++j) dX[r][j] = (T)0;
    }
    if (tX) {
        const bool zin = zq + 4 > 4 && zq < g.dimz - 4;
        T xX[RXC][4];
        // psi of the 4 columns either side (read the whole 8-column halo)
        T psR[RPT][4];
#pragma unroll
        for (int k = 0; k < RPT; ++k) {
            const int item = threadIdx.x + k * NTHR;
            const int rc = item >> 5, l = item & 31;
            const int c = rc < 4 ? rc - 4 : TXC + rc - 4;
            const int zr = z0 + 4 * l;
            const T *po; T *pn, *xi; T ab, bb;
            bool upd = false, arr = false;
            if (item < RING_ITEMS && zr < zend) arr = x_strip<T>(a, x0 + c, po, pn, xi, ab, bb, upd);
#pragma unroll
            for (int j = 0; j < 4; ++j) psR[k][j] = (T)0;
            if (arr) {
                ld4(po + zr, psR[k]);
                if (upd && zr + 4 > 4 && zr < g.dimz - 4) {
                    T W[9][4];
#pragma unroll
                    for (int m = 0; m < 9; ++m) ld4(u8 + (c + 4 + m) * SZ + 4 * l + HALO, W[m]);
                    psi_x_new<T>(W, psR[k], ab, bb, h1, zr, g.dimz);
                }
            }
        }
        // psi of the own cells, into the u_prev tile (each thread overwrites only what it read)
#pragma unroll
        for (int r = 0; r < RXC; ++r) {
            const int c = warp * RXC + r, x = x0 + c;
            T ps[4] = {(T)0, (T)0, (T)0, (T)0};
#pragma unroll
            for (int j = 0; j < 4; ++j) xX[r][j] = (T)0;
            const T *po; T *pn, *xi; T ab, bb;
            bool upd;
            if (own && x_strip<T>(a, x, po, pn, xi, ab, bb, upd)) {
                ld4(po + zq, ps);
                if (upd && zin) {
                    cX[r] = true;
                    ld4(xi + zq, xX[r]);
                    T W[9][4];
#pragma unroll
                    for (int m = 0; m < 9; ++m) ld4(su + (c + m) * SZ + zi, W[m]);
                    psi_x_new<T>(W, ps, ab, bb, h1, zq, g.dimz);
                }
                st4(pn + zq, ps);
            }
            st4(sprv + c * TZ + 4 * lane, ps);
        }
        __syncthreads();                              // the outermost halo columns are read
#pragma unroll
        for (int k = 0; k < RPT; ++k) {
            const int item = threadIdx.x + k * NTHR;
            if (item < RING_ITEMS) {
                const int rc = item >> 5, l = item & 31;
                st4(u8 + (rc < 4 ? rc : TXC + 8 + rc) * SZ + 4 * l, psR[k]);
            }
        }
        __syncthreads();
        // psi of tile column cc (-4 <= cc < TXC + 4) at this thread's quad
        auto psi_at = [&](int cc, T (&out)[4]) {
            if (cc < 0) ld4(u8 + (cc + 4) * SZ + 4 * lane, out);
            else if (cc >= TXC) ld4(u8 + (cc + 12) * SZ + 4 * lane, out);
            else ld4(sprv + cc * TZ + 4 * lane, out);
        };
#pragma unroll
        for (int r = 0; r < RXC; ++r) {
            if (!cX[r]) continue;
            const int c = warp * RXC + r, x = x0 + c;
            const T *po; T *pn, *xi; T ab, bb;
            bool upd;
            x_strip<T>(a, x, po, pn, xi, ab, bb, upd);
            const T bk[4] = {(T)RTM_B4, (T)RTM_B3, (T)RTM_B2, (T)RTM_B1};
            T acc[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                T mk[4], pk[4];
                psi_at(c - (4 - k), mk);
                psi_at(c + (4 - k), pk);
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const T term = bk[k] * (pk[j] - mk[j]);
                    acc[j] = k == 0 ? term : acc[j] + term;
                }
            }
            T W[9][4], cf[4];
#pragma unroll
            for (int m = 0; m < 9; ++m) ld4(su + (c + m) * SZ + zi, W[m]);
            ld4(scf + c * TZ + 4 * lane, cf);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int z = zq + j;
                if (z >= 4 && z < g.dimz - 4) {
                    const T dp = acc[j] * h1;
                    const T xn = bb * xX[r][j] + ab * (d2x_w<T>(W, j) * h3 + dp);
                    xX[r][j] = xn;
                    dX[r][j] = (cf[j] * h2) * (dp + xn);
                }
            }
            st4(xi + zq, xX[r]);
        }
    }

    // ---- z-strips of a tile whose band fits a half-warp (top and bottom tiles, corners
    // included): the correction terms of the thread's own quads, applied below in strip order
    T dZh[RXC][4];
    bool cZh[RXC] = {false, false};
    bool zhalf = false;
    if (tZ) {
        const bool hasT = z0 < g.thu, hasB = zend > g.zb0;
        if (hasT != hasB) {
            const int qb = hasT ? 0 : (max(g.zb0, z0) - z0) >> 2;
            const int qe = ((hasT ? min(g.thu, zend) : zend) - z0 + 3) >> 2;
            if (qe - qb <= 16) {
                cpml_z_half<T, WARPS>(a, su, scf, dZh, cZh, x0, z0, qb, qe - qb, hasT);
                zhalf = true;
                if (!tX) {
#pragma unroll
                    for (int r = 0; r < RXC; ++r)
                        if (cZh[r]) {
#pragma unroll
                            for (int j = 0; j < 4; ++j) v[r][j] = v[r][j] + dZh[r][j];
                        }
                    return;
                }
            }
        }
    }

    // ---- z-strip loads (previous psi, xi) of both columns.  On the top and bottom tiles they
    // are the pass's first loads; on the corner tiles they follow the x-strips, whose
    // registers they would otherwise share (loaded before them, they pushed the backward
    // kernel into spilling: 27.0 -> 29.4 us per backward step on 3400 x 700)
    T psZ[RXC][4], xZ[RXC][4];
#pragma unroll
    for (int r = 0; r < RXC; ++r) {
        const int x = x0 + warp * RXC + r;
#pragma unroll
        for (int j = 0; j < 4; ++j) { psZ[r][j] = (T)0; xZ[r][j] = (T)0; }
        if (tZ && !zhalf && (inTa || inBa) && x < g.dimx) {
            const size_t o = inTa ? (size_t)x * g.st + zq : (size_t)x * g.sb + (zq - g.zb0);
            ld4((inTa ? a.psi_t : a.psi_b) + o, psZ[r]);
            if (qT || qB) ld4((inTa ? a.xi_t : a.xi_b) + o, xZ[r]);
        }
    }

    // ---- z-strips: psi of the own quad (absorbingBoundaryCondition.c:225-229, 318-322), the
    // neighbours' by shuffle, the correction term; the corrections applied in strip order
    float aa[4] = {0.f, 0.f, 0.f, 0.f}, bz[4] = {0.f, 0.f, 0.f, 0.f};
    const int zlo = inTa ? 4 : g.dimz - g.thd + 4, zhi = inTa ? g.thu - 4 : g.dimz - 4;
    if (tZ && !zhalf && (inTa || inBa)) {
        const float *pa = inTa ? a.a_t + zq : a.a_b + (zq - g.zb0);
        const float *pb = inTa ? a.b_t + zq : a.b_b + (zq - g.zb0);
        const float4 av = *reinterpret_cast<const float4 *>(pa);
        const float4 bv = *reinterpret_cast<const float4 *>(pb);
        aa[0] = av.x; aa[1] = av.y; aa[2] = av.z; aa[3] = av.w;
        bz[0] = bv.x; bz[1] = bv.y; bz[2] = bv.z; bz[3] = bv.w;
    }
#pragma unroll
    for (int r = 0; r < RXC; ++r) {
        const int c = warp * RXC + r, x = x0 + c;
        const bool left = cX[r] && x < g.thl;
        T dZ[4] = {(T)0, (T)0, (T)0, (T)0};
        bool cZ = false;
        if (zhalf) {
            cZ = cZh[r];
#pragma unroll
            for (int j = 0; j < 4; ++j) dZ[j] = dZh[r][j];
        } else if (tZ) {
            const bool arr = (inTa || inBa) && x < g.dimx;
            cZ = arr && (qT || (qB && x >= 4 && x < g.dimx - 4));   // the top rows cover every column
            T zz[12];
            {
                T c4[4];
                ld4(su + (c + HALO) * SZ + zi, c4);
                z_line<T>(su, c + HALO, zi, c4, zz);
            }
            if (arr) {
                if (x >= 4 && x < g.dimx - 4) {       // psi cells: x in [4, dimX-4)
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const int z = zq + j;
                        if (z >= zlo && z < zhi)
                            psZ[r][j] = (T)bz[j] * psZ[r][j] + (T)aa[j] * dpsi_z<T>(zz, j) * h1;
                    }
                }
                const size_t o = inTa ? (size_t)x * g.st + zq : (size_t)x * g.sb + (zq - g.zb0);
                st4((inTa ? a.psn_t : a.psn_b) + o, psZ[r]);
            }
            T q[12];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const T up = __shfl_up_sync(0xffffffffu, psZ[r][j], 1);
                const T dn = __shfl_down_sync(0xffffffffu, psZ[r][j], 1);
                q[j] = lane > 0 ? up : (T)0;
                q[4 + j] = psZ[r][j];
                q[8 + j] = lane < 31 ? dn : (T)0;
            }
            if (cZ) {
                T cf[4];
                ld4(scf + c * TZ + 4 * lane, cf);
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int z = zq + j;
                    if (z >= zlo && z < zhi) {
                        const T dp = dpsi_z<T>(q, j) * h1;
                        const T xn = (T)bz[j] * xZ[r][j] + (T)aa[j] * (d2z_q<T>(zz, j) * h3 + dp);
                        xZ[r][j] = xn;
                        dZ[j] = (cf[j] * h2) * (dp + xn);
                    }
                }
                const size_t o = inTa ? (size_t)x * g.st + zq : (size_t)x * g.sb + (zq - g.zb0);
                st4((inTa ? a.xi_t : a.xi_b) + o, xZ[r]);
            }
        }
        // order: left, top, right, bottom
        const bool xfirst = cX[r] && (left || !qT);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (xfirst) v[r][j] = v[r][j] + dX[r][j];
            if (cZ) v[r][j] = v[r][j] + dZ[j];
            if (cX[r] && !xfirst) v[r][j] = v[r][j] + dX[r][j];
        }
    }
}

// Full-precision ring save of the thread's quad of one column of the current field u_t
// (forward, ring storage): slot t holds the ring of u_t.  The region's z bounds are
// quad-aligned, so a quad is either wholly in a ring band or not: one 16-byte store.  Saving
// u_t from the halo tile before the CPML pass, rather than u_{t+1} from registers after it
// with per-cell index arithmetic, took the forward step on 3400 x 700 from 20.0 to 17.9 us.
// Ring offset of the quad [zq, zq+4) of column x (ring_index of its first cell), or -1 when
// the quad holds no ring cell.  With quad-aligned region bounds a quad is either wholly in the
// ring or not, and its 4 cells are consecutive there (ring_save_quad writes the same offsets).
__device__ __forceinline__ long long ring_quad_offset(const Geom &g, int x, int zq)
{
    if (x < g.rx0 - 4 || x >= g.rx1 + 4 || zq < g.rz0 - 4 || zq >= g.rz1 + 4) return -1;
    if (zq < g.rz0) return (long long)(x - (g.rx0 - 4)) * 4;                              // top band
    if (zq >= g.rz1) return (long long)4 * g.ring_w + (long long)(x - (g.rx0 - 4)) * 4;   // bottom
    if (x < g.rx0) return (long long)8 * g.ring_w + (long long)(x - (g.rx0 - 4)) * g.ring_h + (zq - g.rz0);
    if (x >= g.rx1)
        return (long long)8 * g.ring_w + (long long)4 * g.ring_h + (long long)(x - g.rx1) * g.ring_h +
               (zq - g.rz0);
    return -1;
}

template <typename T>
__device__ __forceinline__ void ring_save_quad(const StepArgs<T> &a, const T (&q)[4], int x, int zq)
{
    const Geom &g = a.g;
    if (x < g.rx0 - 4 || x >= g.rx1 + 4 || zq < g.rz0 - 4 || zq >= g.rz1 + 4) return;
    T *ring = reinterpret_cast<T *>(a.store);
    size_t o;
    if (zq < g.rz0) o = (size_t)(x - (g.rx0 - 4)) * 4;                                 // top band
    else if (zq >= g.rz1) o = (size_t)4 * g.ring_w + (size_t)(x - (g.rx0 - 4)) * 4;    // bottom
    else if (x < g.rx0) o = (size_t)8 * g.ring_w + (size_t)(x - (g.rx0 - 4)) * g.ring_h + (zq - g.rz0);
    else if (x >= g.rx1)
        o = (size_t)8 * g.ring_w + (size_t)4 * g.ring_h + (size_t)(x - g.rx1) * g.ring_h + (zq - g.rz0);
    else return;
    st4(ring + o, q);
}

template <typename T, int BWD, int WARPS>
__device__ __forceinline__ void step_tile(const StepArgs<T> &a, T *stage, int t, float *red)
{
    using Cfg = StepCfg<T, WARPS, BWD>;
    constexpr int TXC = Cfg::TXC, UT8 = Cfg::UT8, UT = Cfg::UT, PT = Cfg::PT;
    const Geom &g = a.g;
    const int flags = a.flags;
    const bool recon = BWD && (flags & F_RECON);
    T *su8 = stage;                      // current field, 8-column x halo area [TXC+16][SZ]
    const T *su = stage + HALO * SZ;     // ...its 4-halo view               [TXC+8][SZ]
    const T *sprv = stage + UT8;         // previous field                    [TXC][TZ]
    const T *scf = stage + UT8 + PT;     // coef                              [TXC][TZ]
    const T *ss = stage + UT8 + 2 * PT;  // source field + halo   (backward reconstruction)
    const T *ssp = stage + UT8 + UT + 2 * PT;

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
    // Two copies of the column loop, chosen once per tile, so that the plain interior tiles
    // carry none of the boundary tiles' per-cell range tests (the compiler would otherwise
    // predicate them into every tile).
    T v[RXC][4];
    {
        T W[9][4];
#pragma unroll
        for (int m = 0; m < 8; ++m) ld4(su + (row0 + m) * SZ + zi, W[m]);
        if (!boundary) {
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
                for (int j = 0; j < 4; ++j) v[r][j] = cf[j] * lap8<T>(W, zz, j) + (T)2.0f * W[4][j] - prv[j];
                if (zok && x < g.dimx) st4(a.u_next + (size_t)x * P + zq, v[r]);
                if (snap_fast) st4(reinterpret_cast<T *>(a.store) + (size_t)(x - g.thl) * P + zq, v[r]);
#pragma unroll
                for (int m = 0; m < 8; ++m)
#pragma unroll
                    for (int j = 0; j < 4; ++j) W[m][j] = W[m + 1][j];
            }
        } else {
            const bool stencil = !(flags & F_NO_STENCIL);
#pragma unroll
            for (int r = 0; r < RXC; ++r) {
                ld4(su + (row0 + r + 8) * SZ + zi, W[8]);
                T zz[12];
                z_line<T>(su, row0 + r + 4, zi, W[4], zz);
                T prv[4], cf[4];
                ld4(sprv + (row0 + r) * TZ + 4 * lane, prv);
                ld4(scf + (row0 + r) * TZ + 4 * lane, cf);
                const int x = xb + r;
                const bool xs = stencil && x >= 4 && x < g.dimx - 4;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const T sv = cf[j] * lap8<T>(W, zz, j) + (T)2.0f * W[4][j] - prv[j];
                    const int z = zq + j;
                    v[r][j] = (xs && z >= 4 && z < g.dimz - 4) ? sv : prv[j];
                }
#pragma unroll
                for (int m = 0; m < 8; ++m)
#pragma unroll
                    for (int j = 0; j < 4; ++j) W[m][j] = W[m + 1][j];
            }
        }
    }

    if (boundary) {
        // ---- ring of u_t (full precision), from the thread's own quads of the halo tile.  Ring
        // tiles are CPML tiles, so the plain interior tiles carry no ring code at all (in the
        // stencil loop it cost every tile ~60 instructions per warp: forward step 18.5 us
        // against 16.2 us without ring storage on 3400 x 700)
        if (!BWD && ring_t && a.store_prec == 0 && zok) {
#pragma unroll
            for (int r = 0; r < RXC; ++r) {
                T q[4];
                ld4(su + (row0 + r + HALO) * SZ + zi, q);
                ring_save_quad<T>(a, q, xb + r, zq);
            }
        }
        // ---- CPML: psi of this step and the four strips' corrections, on v in registers
        if (cpml_t) cpml_fused<T, WARPS>(a, su8, const_cast<T *>(sprv), scf, v, x0, z0, z1);
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
            const bool ring_q = ring_t && a.store_prec != 0 && ring_quad(g, x, zq);
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
    // Plain reconstruction tiles (inside the region, no source cell, imaged without per-cell
    // tests if at all): their own copy of the column loop, free of the per-cell range tests
    // of the general one below.
    if (recon && in_region && !src_t && (!image_t || image_fast)) {
#pragma unroll
        for (int r = 0; r < RXC; ++r) {
            const int x = xb + r;
            ld4(ss + (row0 + r + 8) * SZ + zi, W[8]);
            T zz[12];
            z_line<T>(ss, row0 + r + 4, zi, W[4], zz);
            T sp[4], cf[4], s[4];
            ld4(ssp + (row0 + r) * TZ + 4 * lane, sp);
            ld4(scf + (row0 + r) * TZ + 4 * lane, cf);
#pragma unroll
            for (int j = 0; j < 4; ++j) s[j] = cf[j] * lap8<T>(W, zz, j) + (T)2.0f * W[4][j] - sp[j];
            if (zok) {
                st4(a.s_next + (size_t)x * P + zq, s);
                if (image_t) {
                    T rv[4];
                    ld4(a.u_next + (size_t)x * P + zq, rv);
                    const size_t o = (size_t)(x - g.thl) * P + zq;
                    image_quad<T>(a.img + o, a.slf + o, s, rv);
                }
            }
#pragma unroll
            for (int m = 0; m < 8; ++m)
#pragma unroll
                for (int j = 0; j < 4; ++j) W[m][j] = W[m + 1][j];
        }
        return;
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
            if (col_ok && ring_t) {
                const long long o = ring_quad_offset(g, x, zq);
                if (o >= 0) {
                    if (a.store_prec == 0) {
                        ld4(reinterpret_cast<const T *>(a.store) + o, s);
                    } else {
#pragma unroll
                        for (int j = 0; j < 4; ++j)
                            s[j] = store_get<T>(a.store, a.store_prec, (size_t)o + j, tile_scale);
                    }
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
    constexpr int UT8 = Cfg::UT8, UT = Cfg::UT, PT = Cfg::PT, STAGE = Cfg::STAGE, NS = Cfg::NS, TXC = Cfg::TXC;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T *stage0 = reinterpret_cast<T *>(smem_raw);
    __shared__ __align__(8) uint64_t full[NS];
    __shared__ int tile_of[NS];          // tile held by each stage (>= tiles: none)
    __shared__ float red[WARPS];
    const Geom &g = a.g;
    const bool recon = BWD && (a.flags & F_RECON);
    const bool cpml_on = !(a.flags & F_NO_CPML);
    // bytes of one tile's loads; the side CPML tiles load the current field with 8 halo
    // columns on either side (their psi needs D1x(u) 4 columns beyond the tile)
    const uint32_t tile_bytes = (uint32_t)(sizeof(T) * (recon ? UT + UT + 3 * PT : UT + 2 * PT));
    const uint32_t side_bytes = tile_bytes + (uint32_t)(sizeof(T) * (UT8 - UT));

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
    // ones (measured per class with clock64 on 3400 x 700: a boundary tile costs 4.1-5.8
    // interior ones forward, 2.7-4.4 backward; 5 and 3 were the fastest weights).  The interior goes out in rounds -- round j gives one tile to every CTA with more
    // than j interior tiles, in CTA order -- so that all CTAs sweep the grid together (their
    // halos and, backward, the image and source rows stay in L2).  Measured on 3400 x 700
    // against plain round-robin: forward 24.5 -> 22.6 us, backward 38.2 -> 30.9 us per step.
    // Every tile is taken exactly once.  A stage with no tile left still completes its
    // barrier phase.
    constexpr int kBalance = BWD ? 2 : 4;
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
        const bool side = cpml_on && (x0 < g.thl - 4 || x0 + TXC > g.dimx - g.thr + 4);
        T *st = stage0 + (size_t)s * STAGE;
        mbar_arrive_expect_tx(&full[s], side ? side_bytes : tile_bytes);
        if (side) tma_load_2d(st, &m.cur8, z0 - HALO, x0 - 2 * HALO, &full[s]);
        else tma_load_2d(st + HALO * SZ, &m.cur, z0 - HALO, x0 - HALO, &full[s]);
        tma_load_2d(st + UT8, &m.prev, z0, x0, &full[s]);
        tma_load_2d(st + UT8 + PT, &m.coef, z0, x0, &full[s]);
        if (recon) {
            tma_load_2d(st + UT8 + 2 * PT, &m.scur, z0 - HALO, x0 - HALO, &full[s]);
            tma_load_2d(st + UT8 + UT + 2 * PT, &m.sprev, z0, x0, &full[s]);
        }
    };
    if (threadIdx.x == 0) {
        // the previous step (same stream, programmatic dependent launch) wrote this step's
        // inputs: wait for its completion before the first load
        griddep_wait();
        for (int s = 0; s < NS; ++s) issue(s, s);
    }
    // The next kernel in the stream may be scheduled now; it waits for this grid's
    // completion (griddepcontrol.wait) before it touches anything this grid writes.
    griddep_launch();
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
        step_tile<T, BWD, WARPS>(a, stage0 + (size_t)s * STAGE, t, red);
        __syncthreads();                         // stage s is free again
        if (threadIdx.x == 0) issue(i + NS, s);
    }
}
