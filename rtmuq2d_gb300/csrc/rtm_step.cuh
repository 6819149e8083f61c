// rtm_step.cuh -- the fused time-step kernel k_step (included by rtm_kernels.cu).
//
// Per CTA: one TX x TZ tile.  Thread 0 loads the current-field tile (+4-cell halo) with a
// TMA 2-D copy; meanwhile every thread loads its u_prev and coef quads.  Then:
//
//   phase 1 (all tiles, fully unrolled, no per-cell branches on interior tiles)
//     8th-order leapfrog (SRC/stencilDFM.c:17-29) for RXC columns x 4 z cells per thread,
//     store of u_next; backward: reverse-time source reconstruction on the stencil-only
//     region and, on tiles that need nothing else, the FP64 cross-correlation
//     (SRC/image_conditions.c:20-33); forward: FP32 interior snapshots.
//   phase 2 (boundary / special tiles only, one compact loop over the thread's cells)
//     CPML corrections in the reference's strip order left, top, right, bottom
//     (SRC/absorbingBoundaryCondition.c:191-357), source injection
//     (SRC/forward_modeling.c:105-109) or receiver overwrite (backward_modeling.c:277-281),
//     trace recording, boundary-ring save/load, 16-bit scaled storage, imaging.
//
// The split keeps the hot path short (no CPML code in the instruction stream of interior
// tiles) and the boundary code small (one copy of the loop body instead of an unrolled one).

template <typename T>
__device__ __forceinline__ T d2s(const T *c, int s)   // 1-D second derivative, stride s (smem)
{
    return (T)RTM_AC4 * (c[4 * s] + c[-4 * s]) + (T)RTM_AC3 * (c[3 * s] + c[-3 * s])
         + (T)RTM_AC2 * (c[2 * s] + c[-2 * s]) + (T)RTM_AC1 * (c[s] + c[-s])
         + (T)RTM_AC0 * c[0];
}

// CPML correction of one cell (reference strip order), u_cur neighbours from the tile.
template <typename T>
__device__ __forceinline__ T cpml_cell(const StepArgs<T> &a, const T *sc, int x, int z, T cf, T v)
{
    const Geom &g = a.g;
    const size_t P = (size_t)g.pitch;
    const T ch2 = cf * a.h2;
    if (x >= 4 && x < g.thl - 4 && z >= 4 && z < g.dimz - 4) {
        const size_t at = (size_t)x * P + z;
        const T dpsi = d1<T>(a.psi_l + at, (ptrdiff_t)P) * a.h1;
        const T xi = (T)a.b_l[x] * a.xi_l[at] + (T)a.a_l[x] * (d2s<T>(sc, SZ) * a.h3 + dpsi);
        a.xi_l[at] = xi;
        v = v + ch2 * (dpsi + xi);
    }
    if (z >= 4 && z < g.thu - 4) {
        const size_t at = (size_t)x * g.st + z;
        const T dpsi = d1<T>(a.psi_t + at, 1) * a.h1;
        const T xi = (T)a.b_t[z] * a.xi_t[at] + (T)a.a_t[z] * (d2s<T>(sc, 1) * a.h3 + dpsi);
        a.xi_t[at] = xi;
        v = v + ch2 * (dpsi + xi);
    }
    if (x >= g.dimx - g.thr + 4 && x < g.dimx - 4 && z >= 4 && z < g.dimz - 4) {
        const int li = x - (g.dimx - g.thr);
        const size_t at = (size_t)li * P + z;
        const T dpsi = d1<T>(a.psi_r + at, (ptrdiff_t)P) * a.h1;
        const T xi = (T)a.b_r[li] * a.xi_r[at] + (T)a.a_r[li] * (d2s<T>(sc, SZ) * a.h3 + dpsi);
        a.xi_r[at] = xi;
        v = v + ch2 * (dpsi + xi);
    }
    if (x >= 4 && x < g.dimx - 4 && z >= g.dimz - g.thd + 4 && z < g.dimz - 4) {
        const int lz = z - (g.dimz - g.thd);
        const size_t at = (size_t)x * g.sb + lz;
        const T dpsi = d1<T>(a.psi_b + at, 1) * a.h1;
        const T xi = (T)a.b_b[lz] * a.xi_b[at] + (T)a.a_b[lz] * (d2s<T>(sc, 1) * a.h3 + dpsi);
        a.xi_b[at] = xi;
        v = v + ch2 * (dpsi + xi);
    }
    return v;
}

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

// RXC columns x 4 cells of leapfrog from the tile `t` (centre quad at row r0+4, index zi).
// dom: apply the stencil-domain predicate per cell (tiles touching the outer frame).
template <typename T, int RXC>
__device__ __forceinline__ void stencil_cols(const T *tile, int row0, int zi, const T (&prv)[RXC][4],
                                             const T (&cf)[RXC][4], T (&out)[RXC][4], bool per_cell,
                                             int xb, int zq, int xlo, int xhi, int zlo, int zhi)
{
    T W[9][4];
#pragma unroll
    for (int m = 0; m < 8; ++m) ld4(tile + (row0 + m) * SZ + zi, W[m]);
#pragma unroll
    for (int r = 0; r < RXC; ++r) {
        ld4(tile + (row0 + r + 8) * SZ + zi, W[8]);
        T zz[12];
        {
            T zm[4], zp[4];
            ld4(tile + (row0 + r + 4) * SZ + zi - 4, zm);
            ld4(tile + (row0 + r + 4) * SZ + zi + 4, zp);
#pragma unroll
            for (int j = 0; j < 4; ++j) { zz[j] = zm[j]; zz[4 + j] = W[4][j]; zz[8 + j] = zp[j]; }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const T v = cf[r][j] * lap8<T>(W, zz, j) + (T)2.0f * W[4][j] - prv[r][j];
            if (per_cell) {
                const int x = xb + r, z = zq + j;
                out[r][j] = (x >= xlo && x < xhi && z >= zlo && z < zhi) ? v : prv[r][j];
            } else {
                out[r][j] = v;
            }
        }
#pragma unroll
        for (int m = 0; m < 8; ++m)
#pragma unroll
            for (int j = 0; j < 4; ++j) W[m][j] = W[m + 1][j];
    }
}

template <typename T, int WARPS>
struct StepCfg {
    static constexpr int RXC = 2;                      // x columns per thread
    static constexpr int TXC = WARPS * RXC;            // x columns per tile
    static constexpr int TILE = (TXC + 2 * HALO) * SZ; // smem elements per field tile
    static constexpr int MINB = sizeof(T) == 4 ? (768 / (WARPS * 32) > 0 ? 768 / (WARPS * 32) : 1) : 1;
};

template <typename T, int BWD, int WARPS>
__global__ void __launch_bounds__(WARPS * 32, (StepCfg<T, WARPS>::MINB))
    k_step(const __grid_constant__ CUtensorMap tm_u, const __grid_constant__ CUtensorMap tm_s,
           const __grid_constant__ StepArgs<T> a)
{
    constexpr int RXC = StepCfg<T, WARPS>::RXC;
    constexpr int TXC = StepCfg<T, WARPS>::TXC;
    constexpr int TILE = StepCfg<T, WARPS>::TILE;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T *su = reinterpret_cast<T *>(smem_raw);
    T *ss = su + TILE;
    __shared__ __align__(8) uint64_t bar;
    __shared__ float red[WARPS];

    const Geom &g = a.g;
    const int flags = a.flags;
    const int x0 = blockIdx.x * TXC;
    const int z0 = blockIdx.y * TZ;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const bool recon = BWD && (flags & F_RECON);

    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_barrier_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t bytes = (uint32_t)(TILE * sizeof(T)) * (recon ? 2u : 1u);
        mbar_arrive_expect_tx(&bar, bytes);
        tma_load_2d(su, &tm_u, z0 - HALO, x0 - HALO, &bar);
        if (recon) tma_load_2d(ss, &tm_s, z0 - HALO, x0 - HALO, &bar);
    }

    const int zq = z0 + 4 * lane;          // first z of this thread's quad
    const int xb = x0 + warp * RXC;        // first x column of this thread
    const bool zok = zq < g.dimz;
    const size_t P = (size_t)g.pitch;

    // ---- tile classification (uniform over the CTA)
    const int x1 = x0 + TXC, z1 = z0 + TZ;
    const bool in_domain = x0 >= 4 && x1 <= g.dimx - 4 && z0 >= 4 && z1 <= g.dimz - 4;
    const bool cpml_t = !(flags & F_NO_CPML) &&
                        (x0 < g.thl - 4 || x1 > g.dimx - g.thr + 4 || z0 < g.thu - 4 ||
                         z1 > g.dimz - g.thd + 4);
    const int src_flag = BWD ? F_RECON_SRC : F_SRC;
    const bool src_t = (flags & src_flag) && g.xs >= x0 && g.xs < x1 && g.zs >= z0 && g.zs < z1;
    const bool rec_t = (flags & (F_RECORD | F_OVERWRITE)) && g.zrec >= z0 && g.zrec < z1;
    const bool in_region = x0 >= g.rx0 && x1 <= g.rx1 && z0 >= g.rz0 && z1 <= g.rz1;
    const bool near_ring = x0 < g.rx1 + 4 && x1 > g.rx0 - 4 && z0 < g.rz1 + 4 && z1 > g.rz0 - 4;
    const bool ring_t = (flags & (BWD ? F_RECON : F_RING_SAVE)) && near_ring && !in_region;
    const bool int_full = x0 >= g.thl && x1 <= g.thl + g.nx && z0 >= g.thu && z1 <= g.thu + g.nz;
    const bool int_any = x0 < g.thl + g.nx && x1 > g.thl && z0 < g.thu + g.nz && z1 > g.thu;
    const bool snap_t = !BWD && (flags & F_SNAP_SAVE) && int_any;
    // the snapshot holds u after source injection: the shot's tile saves it in phase 2
    const bool snap_fast = snap_t && int_full && a.store_prec == 0 && !src_t;
    const bool image_t = BWD && (flags & F_IMAGE) && int_any;
    const bool image_fast = image_t && int_full && !rec_t && !src_t;
    const bool phase2 = cpml_t || src_t || rec_t || ring_t || (snap_t && !snap_fast) ||
                        (image_t && !image_fast);

    // Per-cell inputs with no reuse go straight to registers while the TMA is in flight.
    T prv[RXC][4], cf[RXC][4];
#pragma unroll
    for (int r = 0; r < RXC; ++r) {
        const int x = xb + r;
        if (zok && x < g.dimx) {
            ld4(a.u_next + (size_t)x * P + zq, prv[r]);
            ldg4(a.coef + (size_t)x * P + zq, cf[r]);
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) { prv[r][j] = (T)0; cf[r][j] = (T)0; }
        }
    }

    const bool ok = mbar_wait_bounded(&bar, 0, 2000000000ull);
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) atomicOr(a.status, ST_TMA_TIMEOUT);
        mbar_wait_bounded(&bar, 0, 2000000000ull);   // let copies in flight land
        return;
    }

    const int row0 = warp * RXC;            // tile row of column xb-4
    const int zi = 4 * lane + HALO;         // tile index of the quad's first cell

    // ================= phase 1: leapfrog of the propagated field ========================
    T un[RXC][4];
    if (flags & F_NO_STENCIL) {
#pragma unroll
        for (int r = 0; r < RXC; ++r)
#pragma unroll
            for (int j = 0; j < 4; ++j) un[r][j] = prv[r][j];
    } else {
        stencil_cols<T, RXC>(su, row0, zi, prv, cf, un, !in_domain, xb, zq, 4, g.dimx - 4, 4,
                             g.dimz - 4);
    }
#pragma unroll
    for (int r = 0; r < RXC; ++r) {
        const int x = xb + r;
        if (zok && x < g.dimx) st4(a.u_next + (size_t)x * P + zq, un[r]);
    }
    if (snap_fast) {   // FP32 interior snapshot of a tile inside the interior
#pragma unroll
        for (int r = 0; r < RXC; ++r)
            st4(reinterpret_cast<T *>(a.store) + (size_t)(xb + r - g.thl) * P + zq, un[r]);
    }

    // ================= phase 1 (backward): source reconstruction and imaging ============
    T s[RXC][4];
    if (BWD && recon) {
        T sp[RXC][4];
#pragma unroll
        for (int r = 0; r < RXC; ++r) {
            const int x = xb + r;
            if (zok && x < g.dimx) ld4(a.s_next + (size_t)x * P + zq, sp[r]);
            else {
#pragma unroll
                for (int j = 0; j < 4; ++j) sp[r][j] = (T)0;
            }
        }
        stencil_cols<T, RXC>(ss, row0, zi, sp, cf, s, !in_region, xb, zq, g.rx0, g.rx1, g.rz0, g.rz1);
#pragma unroll
        for (int r = 0; r < RXC; ++r) {
            const int x = xb + r;
            if (zok && x < g.dimx) st4(a.s_next + (size_t)x * P + zq, s[r]);
        }
    }
    if (BWD && image_fast) {
#pragma unroll
        for (int r = 0; r < RXC; ++r) {
            const int x = xb + r;
            const size_t o = (size_t)(x - g.thl) * P + zq;
            T sv[4];
            if (recon) {
#pragma unroll
                for (int j = 0; j < 4; ++j) sv[j] = s[r][j];
            } else if (flags & F_IMAGE_SNAP) {
                if (a.store_prec == 0) ld4(a.s_snap + o, sv);
                else {
                    const float sc = a.store_scale[blockIdx.y * gridDim.x + blockIdx.x];
#pragma unroll
                    for (int j = 0; j < 4; ++j) sv[j] = store_get<T>(a.s_snap, a.store_prec, o + j, sc);
                }
            } else {
                ld4(a.s_fixed + (size_t)x * P + zq, sv);
            }
            image_quad<T>(a.img + o, a.slf + o, sv, un[r]);
        }
    }
    if (!phase2) return;

    // ================= phase 2: boundary and special cells (compact loop) ==============
    const float tile_scale = (a.store_prec != 0 && a.store_scale &&
                              ((BWD && recon) || (BWD && (flags & F_IMAGE_SNAP))))
                                 ? a.store_scale[blockIdx.y * gridDim.x + blockIdx.x] : 1.0f;
    const int tsrc = BWD ? g.nt + 1 - a.t : a.t;     // backward: step whose source term is undone
    const bool scaled_store = !BWD && a.store_prec != 0 && (ring_t || snap_t);
    float mx = 0.0f;
#pragma unroll 1
    for (int c = 0; c < RXC * 4; ++c) {
        const int x = xb + (c >> 2), z = zq + (c & 3);
        if (x >= g.dimx || z >= g.dimz) continue;
        const size_t at = (size_t)x * P + z;
        T v = a.u_next[at];
        const T cfc = a.coef[at];
        bool dirty = false;
        if (cpml_t) {
            const T *sc = su + (row0 + (c >> 2) + HALO) * SZ + zi + (c & 3);
            const T w = cpml_cell<T>(a, sc, x, z, cfc, v);
            dirty = dirty || (w != v);
            v = w;
        }
        if (!BWD) {
            if (src_t && x == g.xs && z == g.zs) { v = add_source<T>(a.wavelet, tsrc, v, cfc); dirty = true; }
            if (rec_t && (flags & F_RECORD) && z == g.zrec) {
                const int n = a.rec_cnt[x], f = a.rec_first[x];
                for (int q = 0; q < n; ++q) a.rec_out[(size_t)(f + q) * g.nt + a.t] = v;
            }
        } else if (rec_t && (flags & F_OVERWRITE) && z == g.zrec) {
            const int q = a.rec_last[x];
            if (q >= 0) { v = (T)a.seis_row[q]; dirty = true; }
        }
        if (dirty) a.u_next[at] = v;
        if (!BWD) {
            if (ring_t) {
                const int idx = ring_index(g, x, z);
                if (idx >= 0) {
                    if (a.store_prec == 0) reinterpret_cast<T *>(a.store)[idx] = v;
                    else mx = fmaxf(mx, fabsf((float)v));
                }
            }
            if (snap_t && !snap_fast && in_interior(g, x, z)) {
                const size_t o = (size_t)(x - g.thl) * P + z;
                if (a.store_prec == 0) reinterpret_cast<T *>(a.store)[o] = v;
                else mx = fmaxf(mx, fabsf((float)v));
            }
        } else {
            T sv = (T)0;
            bool have_s = false;
            if (recon) {
                const int idx = ring_t ? ring_index(g, x, z) : -1;
                if (idx >= 0) {
                    a.s_next[at] = store_get<T>(a.store, a.store_prec, (size_t)idx, tile_scale);
                } else if (src_t && x == g.xs && z == g.zs) {
                    a.s_next[at] = add_source<T>(a.wavelet, tsrc, a.s_next[at], cfc);
                }
            }
            if (image_t && !image_fast && in_interior(g, x, z)) {
                const size_t o = (size_t)(x - g.thl) * P + z;
                if (recon) sv = a.s_next[at];
                else if (flags & F_IMAGE_SNAP) sv = store_get<T>(a.s_snap, a.store_prec, o, tile_scale);
                else sv = a.s_fixed[at];
                have_s = true;
                a.img[o] += (double)sv * (double)v;
                a.slf[o] += (double)sv * (double)sv;
            }
            (void)have_s;
        }
    }
    if (scaled_store) {   // 16-bit storage: per-step, per-tile max-abs scale, then quantise
        mx = block_max<WARPS>(mx, red);
        const float target = a.store_prec == 2 ? kFp16Target : kBf16Target;
        const float inv = mx > 0.0f ? target / mx : 1.0f;
        if (threadIdx.x == 0) a.store_scale[blockIdx.y * gridDim.x + blockIdx.x] = mx > 0.0f ? mx / target : 1.0f;
#pragma unroll 1
        for (int c = 0; c < RXC * 4; ++c) {
            const int x = xb + (c >> 2), z = zq + (c & 3);
            if (x >= g.dimx || z >= g.dimz) continue;
            const T v = a.u_next[(size_t)x * P + z];
            if (ring_t) {
                const int idx = ring_index(g, x, z);
                if (idx >= 0) store_put<T>(a.store, a.store_prec, (size_t)idx, v, inv);
            }
            if (snap_t && in_interior(g, x, z))
                store_put<T>(a.store, a.store_prec, (size_t)(x - g.thl) * P + z, v, inv);
        }
    }
}
