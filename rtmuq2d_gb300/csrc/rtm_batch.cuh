// rtm_batch.cuh -- batched time steps over many resident migrations (included by
// rtm_kernels.cu).
//
// Each batch member is one migration (one shot of one velocity realization) whose buffers
// are laid out like a single-migration plan.  Its descriptor (geometry, pointers, tensor
// maps) lives in device memory, its progress (pass, step) too.  One k_bpsi + one k_bstep
// launch advance every active member by one time step; the members may have different
// grids, time axes and storage precisions, and may be in different passes (forward,
// backward) -- the per-member flags of the step are derived here on the device from
// (pass, step), mirroring the single-plan drivers in rtm_engine.cu (run_forward /
// run_adjoint).  The last CTA of k_bstep advances every member's state, so a CUDA graph of a
// few steps can be replayed while the host admits new members and retires finished ones.

static_assert(alignof(BMember<float>) >= 64 && sizeof(BMember<float>) % 64 == 0,
              "tensor maps of consecutive members must stay 64-byte aligned");

// Orders the host's earlier writes of a tensor map in global memory before its use by TMA.
__device__ __forceinline__ void prefetch_l2(const void *p)
{
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

__device__ __forceinline__ void tensormap_acquire(const CUtensorMap *m)
{
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(m) : "memory");
}


// Slot k of a member's source-wavefield store and its scales (16-bit storage).
template <typename T>
__device__ __forceinline__ void *member_slot(const BMember<T> &M, int k)
{
    const size_t se = M.store_prec == 0 ? sizeof(T) : 2;
    return static_cast<unsigned char *>(M.store) + (size_t)k * M.slot_elems * se;
}
template <typename T>
__device__ __forceinline__ float *member_scales(const BMember<T> &M, int k)
{
    return M.scales ? M.scales + (size_t)k * M.scales_per_slot : nullptr;
}

// ctrl of the reference's imaging loop at tau (backward_modeling.c:267): it starts at
// nt/slices - 1 at the first tau % slices == 0 and counts down, so it lags tau/slices by one
// when slices does not divide nt.
__host__ __device__ __forceinline__ int image_ctrl(const Geom &g, int tau)
{
    return g.nt / g.slices - 1 - ((g.nt - 1) / g.slices - tau / g.slices);
}

// Arguments of member M's tiles of role `role` at step t of its pass, and the tensor maps
// they load (mu: field with halo, mp: previous field; u maps for FWD/SRC, r maps for RCV).
// Mirrors the single-migration drivers run_forward / run_adjoint (forward_modeling.c:98-128,
// backward_modeling.c:268-297), with the imaging moved one step later (rtm_march.cuh).
template <typename T>
__device__ __forceinline__ void margs(const BMember<T> &M, int t, int role, MArgs<T> &a, int &mu, int &mp)
{
    const Geom &g = M.g;
    a.g = g;
    a.wavelet = M.wav;
    a.rec_last = M.rec_last; a.rec_first = M.rec_first; a.rec_cnt = M.rec_cnt;
    a.seis_row = nullptr;
    a.rec_out = nullptr;
    a.store = nullptr; a.store_scale = nullptr;
    a.s_img = nullptr;
    a.img = M.img; a.slf = M.slf;
    a.t = t;
    a.tsrc = 0;
    a.store_prec = M.store_prec;
    const bool ring = M.storage == 1;
    const int cur = t & 1;
    const int ua = g.nt & 1, ub = 1 - ua;          // u buffers holding u_nt, u_{nt-1}
    int f = 0;
    if (role == ROLE_FWD) {
        mu = cur; mp = 1 - cur;
        a.out = M.u[1 - cur];
        if (t < g.nwav) f |= F_SRC;
        if (M.rec_out) { f |= F_RECORD; a.rec_out = M.rec_out; }
        if (!ring && t % g.slices == 0) {
            f |= F_SNAP_SAVE;
            a.store = member_slot(M, t / g.slices);
            a.store_scale = member_scales(M, t / g.slices);
        }
    } else if (role == ROLE_RCV) {
        mu = cur; mp = 1 - cur;
        a.out = M.r[1 - cur];
        if (t == g.nt) f |= F_NO_STEP;             // image-only step after the last one
        else if (g.nrec > 0) {
            f |= F_OVERWRITE;
            a.seis_row = M.seis_t + (size_t)(g.nt - 1 - t) * g.nrec;
        }
        if (t >= 1) {                              // image of step t-1
            const int taup = g.nt - t;
            const int ctrl = image_ctrl(g, taup);
            if (taup % g.slices == 0 && ctrl >= 0) {
                f |= F_IMAGE;
                if (ring) {
                    a.s_img = M.u[((t - 1) & 1) ? ub : ua];   // S(j) lives in u[ua] for even j
                } else {
                    f |= F_IMAGE_SNAP;
                    a.store = member_slot(M, ctrl);
                    a.store_scale = member_scales(M, ctrl);
                }
            }
        }
    } else {                                       // ROLE_SRC, 2 <= t < nt
        const int tau = g.nt - 1 - t;
        const int sc = ((t - 2) & 1) ? ua : ub, sp = 1 - sc;
        mu = sc; mp = sp;
        a.out = M.u[sp];
        if (tau + 2 < g.nwav) { f |= F_RECON_SRC; a.tsrc = tau + 2; }
    }
    a.flags = f;
}

// ---- strip kernel (k_bstrip) ------------------------------------------------------------
// For one quad of a strip: xi_n = b xi_{n-1} + a (D2(u_n) / dx^2 + D1(psi_n) / dx) and the
// correction coef dx^2 (D1(psi_n)/dx + xi_n) that the reference adds to u_{n+1}
// (absorbingBoundaryCondition.c:191-217 left, 237-263 top, 283-310 right, 330-357 bottom);
// the same arithmetic, in the same operand order, as the single-migration step kernel's CPML
// pass (cpml_fused / cpml_z_half, rtm_step.cuh).  c4 gets the correction.
template <typename T>
__device__ __forceinline__ void strip_x_quad(const T *psi, T *xi, const T *ucol, size_t P, T ab, T bb,
                                             const T (&cf)[4], int zq, int zlo, int zhi, T h1, T h2, T h3,
                                             bool fresh, T (&c4)[4])
{
    // dpsi (B coefficients) and D2 along x (AC coefficients) accumulated one row pair at a
    // time, +-4 first, in the operand order of d1x_w / d2x_w (rtm_step.cuh), so that only two rows of
    // each field are live at once
    T acc[4], d2[4];
    {
        const T bk[4] = {(T)RTM_B4, (T)RTM_B3, (T)RTM_B2, (T)RTM_B1};
        const T ak[4] = {(T)RTM_AC4, (T)RTM_AC3, (T)RTM_AC2, (T)RTM_AC1};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const ptrdiff_t off = (ptrdiff_t)(4 - k) * (ptrdiff_t)P;
            T mk[4], pk[4], um[4], up[4];
            ld4(psi - off, mk);
            ld4(psi + off, pk);
            ld4(ucol - off, um);
            ld4(ucol + off, up);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const T term = bk[k] * (pk[j] - mk[j]);
                acc[j] = k == 0 ? term : acc[j] + term;
                const T dterm = ak[k] * (up[j] + um[j]);
                d2[j] = k == 0 ? dterm : d2[j] + dterm;
            }
        }
        T uc[4];
        ld4(ucol, uc);
#pragma unroll
        for (int j = 0; j < 4; ++j) d2[j] = d2[j] + (T)RTM_AC0 * uc[j];
    }
    T x4[4];
    if (fresh) {
#pragma unroll
        for (int j = 0; j < 4; ++j) x4[j] = (T)0;
    } else {
        ld4(xi, x4);
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int z = zq + j;
        c4[j] = (T)0;
        if (z >= zlo && z < zhi) {
            const T dp = acc[j] * h1;
            const T xn = bb * x4[j] + ab * (d2[j] * h3 + dp);
            x4[j] = xn;
            c4[j] = (cf[j] * h2) * (dp + xn);
        }
    }
    st4(xi, x4);
}

template <typename T>
__device__ __forceinline__ void strip_z_quad(const T *psi, T *xi, const float *ab, const float *bb,
                                             const T (&zz)[12], const T (&cf)[4], int zq, int zlo, int zhi,
                                             T h1, T h2, T h3, bool fresh, T (&c4)[4])
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
    if (fresh) {
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
        c4[j] = (T)0;
        if (z >= zlo && z < zhi) {
            const T dp = dpsi_z<T>(q, j) * h1;
            const T xn = (T)bbv[j] * x4[j] + (T)aa[j] * (d2z_q<T>(zz, j) * h3 + dp);
            x4[j] = xn;
            c4[j] = (cf[j] * h2) * (dp + xn);
        }
    }
    st4(xi, x4);
}

// Strip quads of one member: every strip column x in [4, thl-4) or [dimx-thr+4, dimx-4)
// with all its z quads in [4, dimz-4) (nA items), then every column x in [0, dimx) with its
// top quads (z in [4, thu-4)) and bottom quads (z in [dimz-thd+4, dimz-4)) -- items of strip
// columns (already covered) or bottom quads outside [4, dimx-4) are skipped (nB items).
struct CorrShape {
    int nql, nA, ntq, q0, nbq, nB;
};
__host__ __device__ __forceinline__ CorrShape corr_shape(const Geom &g)
{
    CorrShape c;
    c.nql = (g.dimz - 8 + 3) / 4;
    c.nA = (g.thl - 8 + g.thr - 8) * c.nql;
    c.ntq = (g.thu - 8 + 3) / 4;
    c.q0 = (g.dimz - g.thd + 4) & ~3;
    c.nbq = (g.dimz - 4 - c.q0 + 3) / 4;
    c.nB = g.dimx * (c.ntq + c.nbq);
    return c;
}
constexpr int kStripBlock = 256;          // strip items per block (and per 16-bit ring scale)
// Members whose per-member tables (work-list bases, tile counts, nt, state) the batched
// kernels stage in shared memory; members beyond it (up to kMaxMembers) are read from the
// index in global memory, which cost the 64-member ensemble 4% when every member went that way.
constexpr int kSmemMembers = 128;

__host__ __device__ __forceinline__ int round_block(int n)
{
    return (n + kStripBlock - 1) / kStripBlock * kStripBlock;
}

// Item index of quad (x, zq) in the list above (the quad holding a ring cell).
__device__ __forceinline__ int strip_item(const Geom &g, const CorrShape &cs, int x, int zq)
{
    if (x >= 4 && x < g.thl - 4) return (x - 4) * cs.nql + (zq - 4) / 4;
    if (x >= g.dimx - g.thr + 4 && x < g.dimx - 4)
        return (g.thl - 8 + x - (g.dimx - g.thr + 4)) * cs.nql + (zq - 4) / 4;
    const int k = zq < g.thu - 4 ? (zq - 4) / 4 : cs.ntq + (zq - cs.q0) / 4;
    return cs.nA + x * (cs.ntq + cs.nbq) + k;
}

// Cell of ring index r (inverse of ring_index).
__device__ __forceinline__ void ring_cell(const Geom &g, int r, int &x, int &z)
{
    const int w4 = g.ring_w * 4;
    if (r < w4) { x = g.rx0 - 4 + r / 4; z = g.rz0 - 4 + r % 4; return; }
    r -= w4;
    if (r < w4) { x = g.rx0 - 4 + r / 4; z = g.rz1 + r % 4; return; }
    r -= w4;
    const int h4 = 4 * g.ring_h;
    if (r < h4) { x = g.rx0 - 4 + r / g.ring_h; z = g.rz0 + r % g.ring_h; return; }
    r -= h4;
    x = g.rx1 + r / g.ring_h;
    z = g.rz0 + r % g.ring_h;
}

// One strip quad: the corrections of every strip covering it added to the stencil value
// that k_mstep stored in u_next, in the reference's order left, top, right, bottom; fv gets
// the final values.  Returns false for skipped items.
template <typename T>
__device__ __forceinline__ bool strip_quad(const BMember<T> &M, const CorrShape &cs, const T *u, T *un,
                                           int idx, bool fresh, int &x, int &zq, T (&fv)[4])
{
    const Geom &g = M.g;
    const size_t P = (size_t)g.pitch;
    if (idx < cs.nA) {
        const int i = idx / cs.nql;
        x = i < g.thl - 8 ? 4 + i : g.dimx - g.thr + 4 + (i - (g.thl - 8));
        zq = 4 + 4 * (idx % cs.nql);
    } else {
        idx -= cs.nA;
        const int nq = cs.ntq + cs.nbq;
        x = idx / nq;
        const int k = idx % nq;
        if ((x >= 4 && x < g.thl - 4) || (x >= g.dimx - g.thr + 4 && x < g.dimx - 4)) return false;
        if (k < cs.ntq) zq = 4 + 4 * k;
        else {
            if (x < 4 || x >= g.dimx - 4) return false;
            zq = cs.q0 + 4 * (k - cs.ntq);
        }
    }
    const bool zx = zq + 4 > 4 && zq < g.dimz - 4;
    const bool inL = zx && x >= 4 && x < g.thl - 4;
    const bool inR = zx && x >= g.dimx - g.thr + 4 && x < g.dimx - 4;
    const bool inT = zq + 4 > 4 && zq < g.thu - 4;                 // every column (the quirk)
    const bool inB = x >= 4 && x < g.dimx - 4 && zq + 4 > g.dimz - g.thd + 4 && zq < g.dimz - 4;
    if (!(inL || inR || inT || inB)) return false;
    // Request every line of the item at once (no registers held); the loads below, which
    // the register budget issues a few at a time, then mostly find them in L2.
    {
        const T *col = u + (size_t)x * P + zq;
        prefetch_l2(M.coef + (size_t)x * P + zq);
        prefetch_l2(un + (size_t)x * P + zq);
        prefetch_l2(col - 4);
        prefetch_l2(col + 4);
        if (inL || inR) {
            const T *ps = inL ? M.psi[0] + (size_t)x * P + zq
                              : M.psi[1] + (size_t)(x - (g.dimx - g.thr)) * P + zq;
#pragma unroll
            for (int k = 1; k <= 4; ++k) {
                prefetch_l2(ps - (ptrdiff_t)k * (ptrdiff_t)P);
                prefetch_l2(ps + (ptrdiff_t)k * (ptrdiff_t)P);
                prefetch_l2(col - (ptrdiff_t)k * (ptrdiff_t)P);
                prefetch_l2(col + (ptrdiff_t)k * (ptrdiff_t)P);
            }
            prefetch_l2((inL ? M.xi[0] + (size_t)x * P : M.xi[1] + (size_t)(x - (g.dimx - g.thr)) * P) + zq);
        }
        if (inT) {
            prefetch_l2(M.psi[2] + (size_t)x * g.st + zq - 4);
            prefetch_l2(M.psi[2] + (size_t)x * g.st + zq + 4);
            prefetch_l2(M.xi[2] + (size_t)x * g.st + zq);
        } else if (inB) {
            const int lq = zq - g.zb0;
            prefetch_l2(M.psi[3] + (size_t)x * g.sb + lq - 4);
            prefetch_l2(M.psi[3] + (size_t)x * g.sb + lq + 4);
            prefetch_l2(M.xi[3] + (size_t)x * g.sb + lq);
        }
    }
    T cf[4], cx[4], cz[4];
    ld4(M.coef + (size_t)x * P + zq, cf);
    ld4(un + (size_t)x * P + zq, fv);
    const T *col = u + (size_t)x * P + zq;
    if (inL)
        strip_x_quad<T>(M.psi[0] + (size_t)x * P + zq, M.xi[0] + (size_t)x * P + zq, col, P, (T)M.prof[0][x],
                        (T)M.prof[1][x], cf, zq, 4, g.dimz - 4, M.h1, M.h2, M.h3, fresh, cx);
    else if (inR) {
        const int li = x - (g.dimx - g.thr);
        strip_x_quad<T>(M.psi[1] + (size_t)li * P + zq, M.xi[1] + (size_t)li * P + zq, col, P,
                        (T)M.prof[2][li], (T)M.prof[3][li], cf, zq, 4, g.dimz - 4, M.h1, M.h2, M.h3,
                        fresh, cx);
    }
    if (inT || inB) {
        T c4[4], zz[12];
        ld4(col, c4);
        {
            T zm[4], zp[4];
            ld4(col - 4, zm);
            ld4(col + 4, zp);
#pragma unroll
            for (int j = 0; j < 4; ++j) { zz[j] = zm[j]; zz[4 + j] = c4[j]; zz[8 + j] = zp[j]; }
        }
        if (inT)
            strip_z_quad<T>(M.psi[2] + (size_t)x * g.st + zq, M.xi[2] + (size_t)x * g.st + zq, M.prof[4] + zq,
                            M.prof[5] + zq, zz, cf, zq, 4, g.thu - 4, M.h1, M.h2, M.h3, fresh, cz);
        else {
            const int lq = zq - g.zb0;
            strip_z_quad<T>(M.psi[3] + (size_t)x * g.sb + lq, M.xi[3] + (size_t)x * g.sb + lq, M.prof[6] + lq,
                            M.prof[7] + lq, zz, cf, zq, g.dimz - g.thd + 4, g.dimz - 4, M.h1, M.h2, M.h3,
                            fresh, cz);
        }
    }
    // cells outside a strip's z range are left untouched, so that the stored value stays
    // bit for bit the stencil's
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int z = zq + j;
        if (inL && z >= 4 && z < g.dimz - 4) fv[j] = fv[j] + cx[j];
        if (inT && z >= 4 && z < g.thu - 4) fv[j] = fv[j] + cz[j];
        if (inR && z >= 4 && z < g.dimz - 4) fv[j] = fv[j] + cx[j];
        if (inB && z >= g.dimz - g.thd + 4 && z < g.dimz - 4) fv[j] = fv[j] + cz[j];
    }
    st4(un + (size_t)x * P + zq, fv);
    return true;
}

// After a step's tiles: the CPML corrections of every active field (forward, backward
// receiver) with the ring storage of the forward field, and the ring restoration of the
// reconstructed source field.  Member m's items: round_block(strip quads), then
// round_block(ring cells) -- a block of kStripBlock items never mixes members, so one
// block's ring cells share one 16-bit scale.  The last CTA advances every member's state.
template <typename T>
__global__ void __launch_bounds__(kStripBlock, 4) k_bstrip(const BatchIndex *__restrict__ ix,
                                                        const BMember<T> *__restrict__ mem,
                                                        int2 *__restrict__ state, unsigned *__restrict__ done)
{
    __shared__ int s_base[kSmemMembers + 1];
    __shared__ int2 s_state[kSmemMembers];
    __shared__ float red[kStripBlock / 32];
    // The block's member descriptor (all but its tensor maps) in shared memory, so that an
    // item's addresses come from there and its data loads all issue at once.  Consecutive
    // blocks of a CTA are a grid apart, mostly in other members: the next block's descriptor
    // is copied (cp.async) into the other buffer while this block's items run.
    constexpr int kMapBytes = (int)offsetof(BMember<T>, g);
    static_assert(kMapBytes % 16 == 0 && sizeof(BMember<T>) % 16 == 0, "16-byte copy of the descriptor");
    __shared__ __align__(64) int4 s_desc[2][sizeof(BMember<T>) / 16];
    auto stage_desc = [&](int mm, int buf) {
        const int4 *src = reinterpret_cast<const int4 *>(mem + mm);
        for (int k = kMapBytes / 16 + threadIdx.x; k < (int)(sizeof(BMember<T>) / 16); k += blockDim.x)
            cp_async16(&s_desc[buf][k], &src[k]);
        cp_async_commit();
    };
    // the next step's k_bpsi may launch; it waits for this grid to complete
    griddep_launch();
    // The per-member tables: item bases and the members' (pass, step), staged for the first
    // kSmemMembers members, read from global memory beyond (state[] is final for this step:
    // only this grid's last CTA rewrites it, after every CTA is done).
    const int nmem = ix->nmem, nsm = min(nmem, kSmemMembers);
    for (int k = threadIdx.x; k <= nsm; k += blockDim.x) s_base[k] = ix->corr_base[k];
    for (int k = threadIdx.x; k < nsm; k += blockDim.x) s_state[k] = state[k];
    __syncthreads();
    auto cbase = [&](int k) { return k <= kSmemMembers ? s_base[k] : __ldg(&ix->corr_base[k]); };
    const int n = cbase(nmem);
    const int stride = gridDim.x * kStripBlock;
    int m = 0, buf = 0;
    if (blockIdx.x * kStripBlock < n) {
        while (cbase(m + 1) <= blockIdx.x * kStripBlock) ++m;
        stage_desc(m, 0);                              // descriptors do not change in a replay
    }
    griddep_wait();                                    // this step's tiles (and psi)
    for (int base = blockIdx.x * kStripBlock; base < n; base += stride) {
        int next_m = m;                                // member of the CTA's next block
        if (base + stride < n)
            while (cbase(next_m + 1) <= base + stride) ++next_m;
        cp_async_wait_all();
        __syncthreads();          // descriptor `buf` visible; the previous block is done with the other
        if (base + stride < n) stage_desc(next_m, buf ^ 1);
        const int2 st = m < kSmemMembers ? s_state[m] : state[m];
        const BMember<T> &M = *reinterpret_cast<const BMember<T> *>(s_desc[buf]);
        const Geom &g = M.g;
        const bool live = (st.x == 1 || st.x == 2) && st.y < g.nt;
        const CorrShape cs = corr_shape(g);
        const int nstrip = round_block(cs.nA + cs.nB);
        const int local = base - cbase(m);
        const bool ring = M.storage == 1;
        if (local < nstrip) {
            // ---- corrections (+ ring storage of the forward field)
            const bool save = live && ring && st.x == 1;
            const int cur = st.y & 1;
            const T *u = st.x == 1 ? M.u[cur] : M.r[cur];
            T *un = st.x == 1 ? M.u[1 - cur] : M.r[1 - cur];
            const int idx = local + threadIdx.x;
            int x = 0, zq = 0;
            T fv[4];
            bool have = false;
            if (live && idx < cs.nA + cs.nB) have = strip_quad<T>(M, cs, u, un, idx, st.y == 0, x, zq, fv);
            if (save) {
                void *slot = member_slot(M, st.y + 1);
                int ri[4];
                const bool rq = have && ring_quad(g, x, zq);
#pragma unroll
                for (int j = 0; j < 4; ++j) ri[j] = (rq && zq + j < g.dimz) ? ring_index(g, x, zq + j) : -1;
                if (M.store_prec == 0) {
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        if (ri[j] >= 0) reinterpret_cast<T *>(slot)[ri[j]] = fv[j];
                } else {                               // block-uniform branch
                    float mx = 0.0f;
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        if (ri[j] >= 0) mx = fmaxf(mx, fabsf((float)fv[j]));
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
                    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
                    __syncthreads();
                    mx = red[0];
#pragma unroll
                    for (int w = 1; w < kStripBlock / 32; ++w) mx = fmaxf(mx, red[w]);
                    __syncthreads();
                    const float scale = store_scale_of(mx, M.store_prec);
                    const float inv = 1.0f / scale;
                    if (threadIdx.x == 0) member_scales(M, st.y + 1)[local / kStripBlock] = scale;
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        if (ri[j] >= 0) store_put<T>(slot, M.store_prec, (size_t)ri[j], fv[j], inv);
                }
            }
        } else if (live && ring && st.x == 2 && st.y >= 2) {
            // ---- ring cells of the reconstructed source field, from storage slot tau + 1
            const int r = local - nstrip + threadIdx.x;
            if (r < g.ring_cells) {
                const int tau = g.nt - 1 - st.y;
                const int ua = g.nt & 1, ub = 1 - ua;
                const int sc = ((st.y - 2) & 1) ? ua : ub, sp = 1 - sc;
                int x, z;
                ring_cell(g, r, x, z);
                float scale = 1.0f;
                if (M.store_prec != 0)
                    scale = member_scales(M, tau + 1)[strip_item(g, cs, x, z & ~3) / kStripBlock];
                M.u[sp][(size_t)x * g.pitch + z] =
                    store_get<T>(member_slot(M, tau + 1), M.store_prec, (size_t)r, scale);
            }
        }
        m = next_m;
        buf ^= 1;
    }
    // The last CTA to finish advances every active member by one step (a forward pass has
    // nt steps, a backward pass nt + 1, the last one images only), one member per thread.
    __shared__ int s_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (s_last) {
        __threadfence();
        for (int k = threadIdx.x; k < nmem; k += blockDim.x) {
            int2 st = state[k];                        // the state this step ran with
            if (st.x != 1 && st.x != 2) continue;
            const int nt = ix->nt[k];
            ++st.y;
            if (st.x == 1 && st.y == nt) { st.x = 2; st.y = 0; }
            else if (st.x == 2 && st.y > nt) { st.x = 3; st.y = 0; }
            state[k] = st;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            done[2] = 0u;                              // k_mstep's chunk counter
            atomicExch(done, 0u);
            __threadfence();
        }
    }
}

// psi update of every active member (one thread per quad of the flattened work list).
template <typename T>
__global__ void __launch_bounds__(256) k_bpsi(const BatchIndex *__restrict__ ix,
                                              const BMember<T> *__restrict__ mem,
                                              const int2 *__restrict__ state)
{
    // This grid follows the step's k_mstep, which triggers it only after the previous step's
    // k_bstrip has completed: the fields and state read here are final.  k_bstrip may launch.
    griddep_launch();
    __shared__ int s_base[kSmemMembers + 1];
    __shared__ int2 s_state[kSmemMembers];
    const int nmem = ix->nmem, nsm = min(nmem, kSmemMembers);
    for (int k = threadIdx.x; k <= nsm; k += blockDim.x) s_base[k] = ix->psi_base[k];
    for (int k = threadIdx.x; k < nsm; k += blockDim.x) s_state[k] = state[k];
    __syncthreads();
    auto pbase = [&](int k) { return k <= kSmemMembers ? s_base[k] : __ldg(&ix->psi_base[k]); };
    const int n = pbase(nmem);
    int m = 0;                                         // member of q (monotone in q)
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        while (pbase(m + 1) <= q) ++m;
        const int2 st = m < kSmemMembers ? s_state[m] : state[m];   // (pass, t)
        if (st.x != 1 && st.x != 2) continue;
        const BMember<T> &M = mem[m];
        const Geom &g = M.g;
        if (st.x == 2 && st.y >= g.nt) continue;          // image-only step: no propagation
        int cnt[4];
        psi_counts(g, cnt);
        int lq = q - pbase(m), strip = 0;
        while (strip < 3 && lq >= cnt[strip]) lq -= cnt[strip++];
        const T *u = st.x == 1 ? M.u[st.y & 1] : M.r[st.y & 1];
        const bool fresh = st.y == 0;
        psi_quad<T>(g, M.h1, u, M.psi, M.prof, strip, lq, fresh);
    }
    // Every CTA waits for this step's k_mstep before it completes, so k_bstrip's wait on this
    // grid also covers the tiles' u_next.
    __syncthreads();
    if (threadIdx.x == 0) griddep_wait();
}

// One batched step: every tile of every active member, in two phases (BatchIndex): phase 1
// = each member's interior field tiles (tile_coords order nb..tiles-1) and, backward with
// ring storage, its source-field tiles; phase 2 = each member's field tiles touching a CPML
// strip (tile_coords order 0..nb-1).  Items go to CTAs in chunks of kChunk consecutive items,
// so that consecutive items of a CTA mostly share their member and role; a CTA's first chunk
// is its index, the later ones come from a step-wide counter (dynamic balance, single items
// in the tail).  An NS-stage TMA pipeline is refilled by thread 0.  Tiles read no CPML data:
// the step's k_bpsi follows (it fills the SMs this grid's tail frees), and k_bstrip completes
// the strip cells afterwards.
constexpr int kChunk = 4;
constexpr int kTail = 2;                  // single-item grabs for the last kTail * G items

template <typename T>
__global__ void __launch_bounds__(MTHREADS, sizeof(T) == 4 ? 2 : 1)
    k_mstep(const BatchIndex *__restrict__ ix, const BMember<T> *__restrict__ mem,
            int2 *__restrict__ state, unsigned *__restrict__ done)
{
    using Cfg = MCfg<T>;
    constexpr int UT = Cfg::UT, PT = Cfg::PT, STAGE = Cfg::STAGE, NS = Cfg::NS;
    static_assert(NS == 2, "two argument slots serve two stages");
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T *stage0 = reinterpret_cast<T *>(smem_raw);
    __shared__ __align__(8) uint64_t full[NS];
    __shared__ int tile_of[NS], role_of[NS], args_of[NS];
    __shared__ MArgs<T> sargs[2];
    __shared__ float red[MWARPS];
    // The work lists and the members' (pass, step) of this launch, staged once for the first
    // kSmemMembers members (read from global memory beyond).  state[] is final here: this
    // grid launches after the previous step's k_bstrip completed, whose last CTA rewrote it.
    const BatchIndex &X = *ix;
    __shared__ int s_base1[kSmemMembers + 1], s_base2[kSmemMembers + 1];
    __shared__ short s_tiles[kSmemMembers], s_nb[kSmemMembers];
    __shared__ int s_nt[kSmemMembers];
    __shared__ int2 s_state[kSmemMembers];
    const int nmem = X.nmem, nsm = min(nmem, kSmemMembers);
    for (int k = threadIdx.x; k <= nsm; k += blockDim.x) {
        s_base1[k] = X.base1[k];
        s_base2[k] = X.base2[k];
    }
    for (int k = threadIdx.x; k < nsm; k += blockDim.x) {
        s_tiles[k] = (short)X.tiles[k];
        s_nb[k] = (short)X.nb[k];
        s_nt[k] = X.nt[k];
    }
    auto base1 = [&](int k) { return k <= kSmemMembers ? s_base1[k] : __ldg(&X.base1[k]); };
    auto base2 = [&](int k) { return k <= kSmemMembers ? s_base2[k] : __ldg(&X.base2[k]); };
    auto m_tiles = [&](int k) { return k < kSmemMembers ? (int)s_tiles[k] : __ldg(&X.tiles[k]); };
    auto m_nb = [&](int k) { return k < kSmemMembers ? (int)s_nb[k] : __ldg(&X.nb[k]); };
    auto m_nt = [&](int k) { return k < kSmemMembers ? s_nt[k] : __ldg(&X.nt[k]); };
    auto m_state = [&](int k) { return k < kSmemMembers ? s_state[k] : state[k]; };
    if (threadIdx.x == 0) {
#pragma unroll
        for (int s = 0; s < NS; ++s) mbar_init(&full[s], 1);
        fence_barrier_init();
    }
    // the previous step (its k_bstrip wrote the strip cells and the state) has completed;
    // only then may this step's k_bpsi launch
    griddep_wait();
    griddep_launch();
    for (int k = threadIdx.x; k < nsm; k += blockDim.x) s_state[k] = state[k];
    __syncthreads();
    const int total1 = base1(nmem), total = total1 + base2(nmem);
    // Thread 0 maps the i-th work item of this CTA to (member, role, tile), builds the
    // arguments of (member, role) when they differ from the last item's (in the argument
    // slot the other stage is not using) and starts the stage's TMA loads.
    // Items [pos, end) of this CTA: kChunk items at blockIdx.x * kChunk first, then grabs
    // from the step's counter (done[2], items past the G * kChunk static ones): kChunk items
    // while more than kTail * G remain, single items in the tail, so that CTAs finish
    // together.  The next grab is fetched one grab ahead so that the atomic's latency hides
    // behind the items; a CTA's grabs only grow, so its items stay in work-list order.
    int cur1 = 0, cur2 = 0;              // member of the latest item of each phase (monotone)
    int last_key = -1, last_args = 0;
    int l_mu = 0, l_mp = 0;
    const int base = (int)gridDim.x * kChunk;
    int pos = blockIdx.x * kChunk, end = pos + kChunk;
    int ahead = 0x0fffffff, ahead_n = 1;  // (past every work list)
    auto grab = [&](int seen) {           // seen: the latest position this CTA knows of
        ahead_n = seen < total - kTail * (int)gridDim.x ? kChunk : 1;
        ahead = base + (int)atomicAdd(done + 2, (unsigned)ahead_n);
    };
    auto issue = [&](int i, int s) {
        if (i == 0) {
            if (pos < total) grab(pos);
        } else if (pos >= end) {
            pos = ahead;
            end = ahead + ahead_n;
            if (pos < total) grab(pos);
        }
        const int tg = pos++;
        if (tg >= total) {
            // past the end: the chunk index only grows, so every later item is too
            tile_of[s] = -1;
            mbar_arrive(&full[s]);
            return;
        }
        int m, lt, role;
        bool skip;
        if (tg < total1) {
            while (base1(cur1 + 1) <= tg) ++cur1;
            m = cur1;
            const int2 st = m_state(m);
            const int nbm = m_nb(m);
            const int k = tg - base1(m), ni = m_tiles(m) - nbm;
            skip = st.x != 1 && st.x != 2;               // idle or finished member
            if (k < ni) {
                role = st.x == 1 ? ROLE_FWD : ROLE_RCV;
                lt = nbm + k;
            } else {
                role = ROLE_SRC;
                lt = k - ni;
                skip = skip || st.x != 2 || st.y < 2 || st.y >= m_nt(m);
            }
        } else {
            const int t2 = tg - total1;
            while (base2(cur2 + 1) <= t2) ++cur2;
            m = cur2;
            const int2 st = m_state(m);
            role = st.x == 1 ? ROLE_FWD : ROLE_RCV;
            lt = t2 - base2(m);
            skip = st.x != 1 && st.x != 2;
        }
        if (skip) {
            tile_of[s] = -2;
            mbar_arrive(&full[s]);
            return;
        }
        const int2 st = m_state(m);
        const BMember<T> &M = mem[m];
        const int key = m * 4 + role;
        if (key != last_key) {
            if (st.x == 1 && st.y == 0) {
                // first step after admission: the host has just written this member's tensor
                // maps; order those writes before their first use by TMA
                tensormap_acquire(&M.tm_u[0]); tensormap_acquire(&M.tm_u[1]);
                tensormap_acquire(&M.tm_up[0]); tensormap_acquire(&M.tm_up[1]);
                tensormap_acquire(&M.tm_r[0]); tensormap_acquire(&M.tm_r[1]);
                tensormap_acquire(&M.tm_rp[0]); tensormap_acquire(&M.tm_rp[1]);
                tensormap_acquire(&M.tm_c);
            }
            last_args = 1 - args_of[1 - s];          // the slot the other stage is not using
            margs<T>(M, st.y, role, sargs[last_args], l_mu, l_mp);
            last_key = key;
        }
        args_of[s] = last_args;
        tile_of[s] = lt;
        role_of[s] = role;
        int xt, zt;
        tile_coords(sargs[last_args].g, lt, xt, zt);
        const int tx = sargs[last_args].g.tx;           // the member's tile width (16 or 32)
        const int x0 = xt * tx, z0 = ztile_origin(sargs[last_args].g, zt);
        const bool rfield = role == ROLE_RCV;
        const CUtensorMap *mc = rfield ? &M.tm_r[l_mu] : &M.tm_u[l_mu];
        const CUtensorMap *mp = rfield ? &M.tm_rp[l_mp] : &M.tm_up[l_mp];
        T *stg = stage0 + (size_t)s * STAGE;
        const int ut = mstage_ut(tx), pt = tx * TZ;
        mbar_arrive_expect_tx(&full[s], (uint32_t)(sizeof(T) * mstage_elems(tx)));
        tma_load_2d(stg, mc, z0 - HALO, x0 - HALO, &full[s]);
        tma_load_2d(stg + ut, mp, z0, x0, &full[s]);
        tma_load_2d(stg + ut + pt, &M.tm_c, z0, x0, &full[s]);
    };
    if (threadIdx.x == 0) {
        args_of[0] = args_of[1] = 0;
    }
    if (threadIdx.x == 0) {
        for (int s = 0; s < NS; ++s) issue(s, s);
    }
    for (int i = 0;; ++i) {
        const int s = i % NS;
        const uint32_t par = (uint32_t)((i / NS) & 1);
        const bool ok = mbar_wait_bounded(&full[s], par, 2000000000ull);
        if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0) {
                atomicOr(done + 1, ST_TMA_TIMEOUT);
                for (int k = 0; k < NS; ++k) {
                    const int ii = i + k;
                    mbar_wait_bounded(&full[ii % NS], (uint32_t)((ii / NS) & 1), 1000000000ull);
                }
            }
            __syncthreads();
            return;
        }
        const int lt = *reinterpret_cast<volatile int *>(&tile_of[s]);
        if (lt == -1) break;
        if (lt >= 0) {
            const T *stg = stage0 + (size_t)s * STAGE;
            const int role = role_of[s];
            const MArgs<T> *ap = &sargs[args_of[s]];
            if (ap->g.tx == MTX) {
                if (role == ROLE_FWD) march_tile<T, ROLE_FWD, MCW>(ap, stg, lt, red);
                else if (role == ROLE_RCV) march_tile<T, ROLE_RCV, MCW>(ap, stg, lt, red);
                else march_tile<T, ROLE_SRC, MCW>(ap, stg, lt, red);
            } else {
                if (role == ROLE_FWD) march_tile<T, ROLE_FWD, MCW / 2>(ap, stg, lt, red);
                else if (role == ROLE_RCV) march_tile<T, ROLE_RCV, MCW / 2>(ap, stg, lt, red);
                else march_tile<T, ROLE_SRC, MCW / 2>(ap, stg, lt, red);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) issue(i + NS, s);
    }
}
