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
__device__ __forceinline__ void tensormap_acquire(const CUtensorMap *m)
{
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(m) : "memory");
}

// Number of psi quads of a member (the four strips of k_psi).
__host__ __device__ __forceinline__ void psi_counts(const Geom &g, int (&n)[4])
{
    const int nlr = (g.dimz - 8 + 3) / 4;
    n[0] = (g.thl - 8) * nlr;
    n[1] = (g.dimx - 8) * ((g.thu - 8 + 3) / 4);
    n[2] = (g.thr - 8) * nlr;
    const int q0 = (g.dimz - g.thd + 4) & ~3;
    n[3] = (g.dimx - 8) * ((g.dimz - 4 - q0 + 3) / 4);
}

// Step arguments of member M at (pass, t), as run_forward / run_adjoint set them.
template <typename T>
__device__ __forceinline__ void member_args(const BMember<T> &M, int pass, int t, StepArgs<T> &a,
                                            int &cur, int &sc, int &sp)
{
    const Geom &g = M.g;
    a.g = g;
    a.h1 = M.h1; a.h2 = M.h2; a.h3 = M.h3;
    a.psi_l = M.psi[0]; a.psi_r = M.psi[1]; a.psi_t = M.psi[2]; a.psi_b = M.psi[3];
    a.xi_l = M.xi[0]; a.xi_r = M.xi[1]; a.xi_t = M.xi[2]; a.xi_b = M.xi[3];
    a.a_l = M.prof[0]; a.b_l = M.prof[1]; a.a_r = M.prof[2]; a.b_r = M.prof[3];
    a.a_t = M.prof[4]; a.b_t = M.prof[5]; a.a_b = M.prof[6]; a.b_b = M.prof[7];
    a.rec_last = M.rec_last; a.rec_first = M.rec_first; a.rec_cnt = M.rec_cnt;
    a.store_prec = M.store_prec;
    a.img = M.img; a.slf = M.slf;
    a.status = M.status;
    a.wavelet = M.wav;
    a.rec_out = nullptr;
    a.t = t;
    a.s_next = nullptr; a.s_snap = nullptr; a.s_fixed = nullptr;
    a.store = nullptr; a.store_scale = nullptr;
    a.seis_row = nullptr;
    const bool ring = M.storage == 1;
    const size_t se = M.store_prec == 0 ? sizeof(T) : 2;
    auto slot = [&](int k) { return static_cast<void *>(static_cast<unsigned char *>(M.store) + (size_t)k * M.slot_elems * se); };
    auto scl = [&](int k) { return M.scales ? M.scales + (size_t)k * g.tiles : (float *)nullptr; };
    int f = (t == 0) ? F_STRIPS_FRESH : 0;   // psi/xi of this pass start from zero
    cur = t & 1;
    sc = sp = 0;
    if (pass == 1) {                      // forward: forward_modeling.c:98-128
        a.u_next = M.u[1 - cur];
        if (t < g.nwav) f |= F_SRC;
        if (ring) {
            f |= F_RING_SAVE;
            a.store = slot(t + 1);
            a.store_scale = scl(t + 1);
        } else if (t % g.slices == 0) {
            f |= F_SNAP_SAVE;
            a.store = slot(t / g.slices);
            a.store_scale = scl(t / g.slices);
        }
    } else {                              // backward: backward_modeling.c:268-297
        const int tau = g.nt - t - 1;
        a.u_next = M.r[1 - cur];
        if (g.nrec > 0) {
            f |= F_OVERWRITE;
            a.seis_row = M.seis_t + (size_t)tau * g.nrec;
        }
        const int ua = g.nt & 1, ub = 1 - ua;     // buffers holding u_nt, u_{nt-1}
        const bool recon = ring && t >= 2;
        if (recon) {
            f |= F_RECON;
            if (tau + 2 < g.nwav) f |= F_RECON_SRC;
            sc = ((t - 2) & 1) ? ua : ub;
            sp = 1 - sc;
            a.s_next = M.u[sp];
            a.store = slot(tau + 1);
            a.store_scale = scl(tau + 1);
        }
        // imaging at tau % slices == 0 with the reference's snapshot counter
        // (backward_modeling.c:267): ctrl starts at nt/slices - 1 at the first such tau and
        // counts down, so it lags tau/slices by one when slices does not divide nt
        const int ctrl = g.nt / g.slices - 1 - ((g.nt - 1) / g.slices - tau / g.slices);
        if (tau % g.slices == 0 && ctrl >= 0) {
            f |= F_IMAGE;
            if (!ring) {
                f |= F_IMAGE_SNAP;
                a.s_snap = static_cast<const T *>(slot(ctrl));
                a.store = slot(ctrl);
                a.store_scale = scl(ctrl);
            } else if (!recon) {
                f |= F_IMAGE_FIXED;
                a.s_fixed = t == 0 ? M.u[ua] : M.u[ub];
            }
        }
    }
    a.flags = f;
}

// psi update of every active member (one thread per quad of the flattened work list).
template <typename T>
__global__ void __launch_bounds__(256) k_bpsi(const BatchIndex *__restrict__ ix,
                                              const BMember<T> *__restrict__ mem,
                                              const int2 *__restrict__ state)
{
    __shared__ int s_base[kMaxMembers + 1];
    __shared__ int2 s_state[kMaxMembers];
    griddep_wait();
    griddep_launch();
    const int nmem = ix->nmem;
    for (int k = threadIdx.x; k <= nmem; k += blockDim.x) s_base[k] = ix->psi_base[k];
    for (int k = threadIdx.x; k < nmem; k += blockDim.x) s_state[k] = state[k];
    __syncthreads();
    const int n = s_base[nmem];
    int m = 0;                                         // member of q (monotone in q)
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        while (s_base[m + 1] <= q) ++m;
        const int2 st = s_state[m];                    // (pass, t)
        if (st.x != 1 && st.x != 2) continue;
        const BMember<T> &M = mem[m];
        const Geom &g = M.g;
        int cnt[4];
        psi_counts(g, cnt);
        int lq = q - s_base[m], strip = 0;
        while (strip < 3 && lq >= cnt[strip]) lq -= cnt[strip++];
        const T *u = st.x == 1 ? M.u[st.y & 1] : M.r[st.y & 1];
        const bool fresh = st.y == 0;
        psi_quad<T>(g, M.h1, u, M.psi, M.prof, strip, lq, fresh);
    }
}

template <typename T, int WARPS>
__global__ void __launch_bounds__(WARPS * 32, (sizeof(T) == 4 && WARPS <= 8) ? 2 : 1)
    k_bstep(const BatchIndex *__restrict__ ix, const BMember<T> *__restrict__ mem,
            int2 *__restrict__ state, unsigned *__restrict__ done)
{
    using Cfg = StepCfg<T, WARPS, 1>;
    constexpr int UT = Cfg::UT, PT = Cfg::PT, STAGE = Cfg::STAGE, NS = Cfg::NS, TXC = Cfg::TXC;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T *stage0 = reinterpret_cast<T *>(smem_raw);
    __shared__ __align__(8) uint64_t full[NS];
    __shared__ int tile_of[NS], pass_of[NS];
    __shared__ StepArgs<T> sargs[NS];
    __shared__ float red[WARPS];
    // The work list and the members' (pass, step) of this launch, staged once: the tile ->
    // member lookups of the issuing thread then stay in shared memory.  state[] is final
    // here: k_bpsi of this step waited for the previous k_bstep before letting this grid
    // launch, and the last CTA of this grid rewrites state[] only after every CTA is done.
    __shared__ int s_base[kMaxMembers + 1];
    __shared__ int2 s_state[kMaxMembers];
    const int nmem = ix->nmem;
    for (int k = threadIdx.x; k <= nmem; k += blockDim.x) s_base[k] = ix->tile_base[k];
    for (int k = threadIdx.x; k < nmem; k += blockDim.x) s_state[k] = state[k];

    if (threadIdx.x == 0) {
#pragma unroll
        for (int s = 0; s < NS; ++s) mbar_init(&full[s], 1);
        fence_barrier_init();
    }
    __syncthreads();
    const int total = s_base[nmem];
    // Thread 0 maps the i-th tile of this CTA to (member, local tile), builds the member's
    // step arguments in shared memory and starts the stage's TMA loads.  The tiles of a CTA
    // visit the members in increasing order; all tiles of a member share its arguments, so
    // they are built once per member and copied between stage slots.
    int cur_m = 0;          // member of the latest tile (monotone)
    int last_m = -1;        // member whose arguments sit in slot last_slot
    int last_slot = 0;
    int l_cur = 0, l_sc = 0, l_sp = 0;
    auto issue = [&](int i, int s) {
        const int tg = blockIdx.x + i * gridDim.x;
        if (tg >= total) {
            tile_of[s] = -1;
            mbar_arrive(&full[s]);
            return;
        }
        while (s_base[cur_m + 1] <= tg) ++cur_m;
        const int m = cur_m;
        const int2 st = s_state[m];
        if (st.x != 1 && st.x != 2) {     // idle or finished member: nothing to do
            tile_of[s] = -2;
            mbar_arrive(&full[s]);
            return;
        }
        const BMember<T> &M = mem[m];
        if (m != last_m) {
            // the descriptors were rewritten by the host when the slot was (re)admitted
            tensormap_acquire(&M.tm_u[0]); tensormap_acquire(&M.tm_u[1]);
            tensormap_acquire(&M.tm_up[0]); tensormap_acquire(&M.tm_up[1]);
            tensormap_acquire(&M.tm_r[0]); tensormap_acquire(&M.tm_r[1]);
            tensormap_acquire(&M.tm_rp[0]); tensormap_acquire(&M.tm_rp[1]);
            tensormap_acquire(&M.tm_c);
            member_args<T>(M, st.x, st.y, sargs[s], l_cur, l_sc, l_sp);
            last_m = m;
        } else if (last_slot != s) {
            const int *src = reinterpret_cast<const int *>(&sargs[last_slot]);
            int *dst = reinterpret_cast<int *>(&sargs[s]);
#pragma unroll 8
            for (int k = 0; k < (int)(sizeof(StepArgs<T>) / sizeof(int)); ++k) dst[k] = src[k];
        }
        last_slot = s;
        const int lt = tg - s_base[m];
        tile_of[s] = lt;
        pass_of[s] = st.x;
        const Geom &g = sargs[s].g;
        int xt, zt;
        tile_coords(g, lt, xt, zt);
        const int x0 = xt * TXC, z0 = ztile_origin(g, zt);
        const bool recon = st.x == 2 && (sargs[s].flags & F_RECON);
        const CUtensorMap *mc = st.x == 1 ? &M.tm_u[l_cur] : &M.tm_r[l_cur];
        const CUtensorMap *mp = st.x == 1 ? &M.tm_up[1 - l_cur] : &M.tm_rp[1 - l_cur];
        T *stg = stage0 + (size_t)s * STAGE;
        mbar_arrive_expect_tx(&full[s], (uint32_t)(sizeof(T) * (recon ? 2 * UT + 3 * PT : UT + 2 * PT)));
        tma_load_2d(stg, mc, z0 - HALO, x0 - HALO, &full[s]);
        tma_load_2d(stg + UT, mp, z0, x0, &full[s]);
        tma_load_2d(stg + UT + PT, &M.tm_c, z0, x0, &full[s]);
        if (recon) {
            tma_load_2d(stg + UT + 2 * PT, &M.tm_u[l_sc], z0 - HALO, x0 - HALO, &full[s]);
            tma_load_2d(stg + 2 * UT + 2 * PT, &M.tm_up[l_sp], z0, x0, &full[s]);
        }
    };
    if (threadIdx.x == 0) {
        for (int s = 0; s < NS; ++s) issue(s, s);
    }
    griddep_launch();
    bool psi_ready = false;
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
            if (pass_of[s] == 1) step_tile<T, 0, WARPS>(sargs[s], stg, lt, psi_ready, red);
            else step_tile<T, 1, WARPS>(sargs[s], stg, lt, psi_ready, red);
        }
        __syncthreads();
        if (threadIdx.x == 0) issue(i + NS, s);
    }
    // The last CTA to finish advances every active member by one step.
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned ticket = atomicAdd(done, 1u);
        if (ticket == gridDim.x - 1) {
            griddep_wait();               // k_bpsi of this step has finished reading state[]
            __threadfence();
            for (int m = 0; m < ix->nmem; ++m) {
                int2 st = state[m];
                if (st.x != 1 && st.x != 2) continue;
                const int nt = mem[m].g.nt;
                if (++st.y == nt) {
                    st.y = 0;
                    st.x = st.x == 1 ? 2 : 3;
                }
                state[m] = st;
            }
            atomicExch(done, 0u);
            __threadfence();
        }
    }
}
