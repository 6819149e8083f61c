// rtm_engine.cu -- host side of the RTM engine: plans (device state of one migration),
// the forward / adjoint time loops, and the C ABI declared in include/rtm_gpu.h.
//
// The time loops replace SRC/forward_modeling.c:98-130 and SRC/backward_modeling.c:268-297.
// One step = one k_step launch (stencil, CPML psi and corrections, source, receivers, storage,
// reconstruction and imaging, fused).  The forward
// pass leaves u_nt, u_{nt-1} and the stored source wavefield (rings or snapshots) in HBM;
// the adjoint pass consumes them in place of ./TEMPORARY_FILES.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "rtm_gpu.h"
#include "rtm_internal.h"

namespace rtm {

// ---- tracing -----------------------------------------------------------------------------
// An NVTX range over a host phase (forward / adjoint pass, autotuning, a server step and its
// admissions and harvests), shown by Nsight Systems and usable as an ncu --nvtx filter; a
// push and a pop when no tool is attached.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// ---- errors ------------------------------------------------------------------------------
static thread_local std::string t_err;

static int fail(int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    t_err = buf;
    return code;
}

#define RTM_CUDA(call)                                                                          \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess)                                                                  \
            return fail(e_ == cudaErrorMemoryAllocation ? RTM_ERR_NOMEM : RTM_ERR_CUDA,        \
                        "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);   \
    } while (0)

#define RTM_TRY(expr)                                                                           \
    do {                                                                                        \
        int s_ = (expr);                                                                        \
        if (s_ != RTM_OK) return s_;                                                            \
    } while (0)

// ---- tensor maps (driver entry point, no libcuda link) ----------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn tensor_map_encoder()
{
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

// 2-D map over a pitched field: dims {pitch (z), dimx (x)}, box {SZ, tx + 2 xhalo}, zero fill.
static int make_field_map(CUtensorMap *m, void *base, const Geom &g, size_t es, int xhalo = HALO)
{
    EncodeTiledFn enc = tensor_map_encoder();
    if (!enc) return fail(RTM_ERR_CUDA, "cuTensorMapEncodeTiled entry point unavailable");
    cuuint64_t dims[2] = {(cuuint64_t)g.pitch, (cuuint64_t)g.dimx};
    cuuint64_t strides[1] = {(cuuint64_t)g.pitch * es};
    cuuint32_t box[2] = {(cuuint32_t)SZ, (cuuint32_t)(g.tx + 2 * xhalo)};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(m, es == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                     2, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(RTM_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return RTM_OK;
}

// ---- geometry and validation ----------------------------------------------------------------
static inline int round_up(int v, int m) { return (v + m - 1) / m * m; }

// ---- tile-width autotuning (rtm_autotune) ---------------------------------------------------
// Best tile width per grid shape, measured by rtm_autotune and used by every plan of that
// shape created afterwards with tile_x = 0.
struct TuneKey {
    int dimx, dimz, thl, thr, thu, thd, storage, precision, compute;
    bool operator<(const TuneKey &o) const
    {
        return std::tie(dimx, dimz, thl, thr, thu, thd, storage, precision, compute) <
               std::tie(o.dimx, o.dimz, o.thl, o.thr, o.thu, o.thd, o.storage, o.precision, o.compute);
    }
};
static std::mutex g_tune_mutex;
static std::map<TuneKey, int> g_tuned;

static TuneKey tune_key(const rtm_params &p)
{
    return {p.th_left + p.nx + p.th_right, p.th_up + p.nz + p.th_down, p.th_left, p.th_right, p.th_up,
            p.th_down, p.storage, p.precision, p.compute};
}

static int default_tile_x(const rtm_params &p)
{
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    auto it = g_tuned.find(tune_key(p));
    return it != g_tuned.end() ? it->second : 16;
}

// batched: a member of the batched step kernels, whose tiles carry no CPML work: z-tiles
// are uniform (TZ rows from z = 0), so that no tile's TMA boxes load rows it does not use.
static Geom make_geom(const rtm_params &p, bool batched = false)
{
    Geom g;
    memset(&g, 0, sizeof g);
    g.nx = p.nx; g.nz = p.nz;
    g.thl = p.th_left; g.thr = p.th_right; g.thu = p.th_up; g.thd = p.th_down;
    g.dimx = g.thl + g.nx + g.thr;
    g.dimz = g.thu + g.nz + g.thd;
    g.pitch = round_up(g.dimz, 32);
    // top/bottom strip arrays: z-aligned rows with 4 spare cells so that a quad's
    // 12-value line (-4..+7) never leaves its row
    g.st = round_up(g.thu, 4) + 4;
    g.zb0 = (g.dimz - g.thd) & ~3;
    g.sb = round_up(g.dimz - g.zb0, 4) + 4;
    g.xs = p.shot_x + g.thl;
    g.zs = p.shot_z + g.thu;
    g.zrec = g.thu + p.rec_depth;
    g.rx0 = g.thl - 4; g.rx1 = g.dimx - g.thr + 4;
    // z bounds of the reconstruction region on quad boundaries (inside the stencil-only rows
    // [th_up - 4, dimZ - th_down + 4), still covering the model rows): every ring band is
    // whole 4-cell quads
    g.rz0 = round_up(g.thu - 4, 4); g.rz1 = (g.dimz - g.thd + 4) & ~3;
    g.ring_w = g.rx1 - g.rx0 + 8;
    g.ring_h = g.rz1 - g.rz0;
    g.ring_cells = 8 * g.ring_w + 8 * g.ring_h;
    g.nt = p.nt; g.nwav = p.n_wavelet; g.slices = p.time_slices; g.nrec = p.rec_count;
    g.tx = p.tile_x > 0 ? p.tile_x : default_tile_x(p);
    if (p.compute == RTM_COMPUTE_FP64 && g.tx > 16) g.tx = 16;   // FP64 stages must fit in smem
    g.tiles_x = (g.dimx + g.tx - 1) / g.tx;
    // z-tile 0 holds the top CPML band (corrections, ring) and, when they sit just below
    // it, the receiver row and the shot, so that every other top tile is plain interior
    if (batched) {
        g.ztop = TZ;
        g.zbot = 0;
        g.tiles_z = g.dimz <= g.ztop ? 1 : 1 + (g.dimz - g.ztop + TZ - 1) / TZ;
    } else {
        // the last z-tile starts at the 4-aligned row at or above the bottom CPML band, so
        // that each band (plus 4 rows inward) lies inside one z-tile: the fused CPML update
        // rebuilds psi in the tile from the tile's own rows
        if (g.dimz <= TZ) {
            g.ztop = round_up(g.dimz, 4);
            g.zbot = 0;
            g.tiles_z = 1;
        } else {
            int top = g.thu - 4;
            if (g.zrec < g.thu + 16) top = std::max(top, g.zrec + 1);
            if (g.zs < g.thu + 16) top = std::max(top, g.zs + 1);
            g.ztop = std::min(TZ, std::max(4, round_up(top, 4)));
            // uniform TZ-row tiles below the top one, when the last of them holds the bottom
            // band; otherwise the last tile starts at the band and the one above it is short
            const int last = g.ztop + (g.dimz - g.ztop - 1) / TZ * TZ;
            g.zbot = last <= ((g.dimz - g.thd) & ~3) ? last : std::max(g.ztop, (g.dimz - g.thd) & ~3);
            g.tiles_z = 2 + (g.zbot - g.ztop + TZ - 1) / TZ;
        }
    }
    g.tiles = g.tiles_x * g.tiles_z;
    g.nxl = std::min(g.tiles_x, (g.thl - 4 + g.tx - 1) / g.tx);
    g.xr0 = std::max(g.nxl, std::min(g.tiles_x, (g.dimx - g.thr + 4) / g.tx));
    return g;
}

static int check_params(const rtm_params &p)
{
    if (p.nx < 1 || p.nz < 4) return fail(RTM_ERR_INVALID, "nx must be >= 1 and nz >= 4");
    if (p.th_left < 12 || p.th_right < 12 || p.th_up < 12 || p.th_down < 12)
        return fail(RTM_ERR_INVALID, "every CPML thickness must be >= 12 cells");
    if (p.th_up > kMaxStripThickness || p.th_down > kMaxStripThickness)
        return fail(RTM_ERR_INVALID, "top and bottom CPML thickness must be <= %d cells", kMaxStripThickness);
    if (!(p.dx > 0.0f) || !(p.dt > 0.0f)) return fail(RTM_ERR_INVALID, "dx and dt must be > 0");
    if (p.nt < 1) return fail(RTM_ERR_INVALID, "nt must be >= 1");
    if (p.n_wavelet < 0) return fail(RTM_ERR_INVALID, "n_wavelet must be >= 0");
    if (p.time_slices < 1) return fail(RTM_ERR_INVALID, "time_slices must be >= 1");
    if (p.nt % p.time_slices != 0)
        return fail(RTM_ERR_INVALID, "nt (%d) must be a multiple of time_slices (%d)", p.nt,
                    p.time_slices);
    if (p.rec_count < 0) return fail(RTM_ERR_INVALID, "rec_count must be >= 0");
    if (p.storage != RTM_STORE_SNAPSHOT && p.storage != RTM_STORE_RING)
        return fail(RTM_ERR_INVALID, "unknown storage %d", p.storage);
    if (p.precision < RTM_PREC_FP32 || p.precision > RTM_PREC_FP16)
        return fail(RTM_ERR_INVALID, "unknown precision %d", p.precision);
    if (p.compute != RTM_COMPUTE_FP32 && p.compute != RTM_COMPUTE_FP64)
        return fail(RTM_ERR_INVALID, "unknown compute type %d", p.compute);
    if (p.compute == RTM_COMPUTE_FP64 && p.precision != RTM_PREC_FP32)
        return fail(RTM_ERR_INVALID, "16-bit storage needs FP32 compute");
    if (p.tile_x != 0 && p.tile_x != 8 && p.tile_x != 16 && p.tile_x != 32)
        return fail(RTM_ERR_INVALID, "tile_x must be 0, 8, 16 or 32");
    const long long dimx = (long long)p.th_left + p.nx + p.th_right;
    const long long dimz = (long long)p.th_up + p.nz + p.th_down;
    if (dimx * (long long)round_up((int)dimz, 32) > (1ll << 31) - 1)
        return fail(RTM_ERR_INVALID, "grid too large");
    const Geom g = make_geom(p);
    if (g.xs < 0 || g.xs >= g.dimx || g.zs < 0 || g.zs >= g.dimz)
        return fail(RTM_ERR_INVALID, "shot cell (%d,%d) outside the padded grid", g.xs, g.zs);
    if (p.storage == RTM_STORE_RING &&
        !(g.xs >= g.rx0 && g.xs < g.rx1 && g.zs >= g.rz0 && g.zs < g.rz1))
        return fail(RTM_ERR_INVALID, "ring storage needs the shot inside the stencil-only region");
    if (p.rec_count > 0) {
        if (g.zrec < 0 || g.zrec >= g.dimz) return fail(RTM_ERR_INVALID, "receiver depth outside the grid");
        const long long c0 = (long long)p.th_left + p.rec_first;
        const long long c1 = c0 + (long long)(p.rec_spacing - 1) * (p.rec_count - 1);
        if (std::min(c0, c1) < 0 || std::max(c0, c1) >= g.dimx)
            return fail(RTM_ERR_INVALID, "receiver line outside the grid");
        if ((long long)p.rec_count * p.nt > (1ll << 31) - 1)
            return fail(RTM_ERR_INVALID, "seismogram too large");
    }
    return RTM_OK;
}

// ---- device memory layout of one plan ----------------------------------------------------
struct Layout {
    size_t u[2], r[2], coef, strips, strip_bytes, prof, rec, wav, seis_t, img, slf, store,
        store_bytes, scales, staging, status, total;
    size_t psi[4], xi[4];
    size_t psn[4];       // the second psi buffer (a step reads one psi buffer, writes the other)
    int nslots;
    size_t slot_elems;   // elements per storage slot
    size_t n_scales_per_slot;
};

static size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Packed damping profiles, every array starting on a 16-byte boundary (see ProfLayout).
static ProfLayout prof_layout(const Geom &g)
{
    ProfLayout pl;
    const int len[8] = {g.thl, g.thl, g.thr, g.thr, g.st, g.st, g.sb, g.sb};
    int off = 0;
    for (int i = 0; i < 8; ++i) { pl.off[i] = off; off += round_up(len[i], 4); }
    pl.total = off;
    return pl;
}

// Packs reference-layout profiles (attenuation_profile_cpml's eight arrays) into `out`
// (prof_layout(g).total floats): the bottom arrays move from index z-(dimZ-th_down) to
// z - zb0; padding is zero.
static void pack_profiles(const Geom &g, const float *a_l, const float *b_l, const float *a_r,
                          const float *b_r, const float *a_t, const float *b_t, const float *a_b,
                          const float *b_b, float *out)
{
    const ProfLayout pl = prof_layout(g);
    memset(out, 0, sizeof(float) * (size_t)pl.total);
    memcpy(out + pl.off[0], a_l, sizeof(float) * g.thl);
    memcpy(out + pl.off[1], b_l, sizeof(float) * g.thl);
    memcpy(out + pl.off[2], a_r, sizeof(float) * g.thr);
    memcpy(out + pl.off[3], b_r, sizeof(float) * g.thr);
    memcpy(out + pl.off[4], a_t, sizeof(float) * g.thu);
    memcpy(out + pl.off[5], b_t, sizeof(float) * g.thu);
    const int shift = (g.dimz - g.thd) - g.zb0;
    memcpy(out + pl.off[6] + shift, a_b, sizeof(float) * g.thd);
    memcpy(out + pl.off[7] + shift, b_b, sizeof(float) * g.thd);
}

// The reference's profiles for *p, packed.
static void make_profiles(const rtm_params &p, const Geom &g, float *out)
{
    std::vector<float> ref(2 * (size_t)(g.thl + g.thr + g.thu + g.thd));
    float *a_l = ref.data(), *b_l = a_l + g.thl, *a_r = b_l + g.thl, *b_r = a_r + g.thr;
    float *a_t = b_r + g.thr, *b_t = a_t + g.thu, *a_b = b_t + g.thu, *b_b = a_b + g.thd;
    rtm_attenuation_profile_cpml(&p, a_l, a_r, a_t, a_b, b_l, b_r, b_t, b_b);
    pack_profiles(g, a_l, b_l, a_r, b_r, a_t, b_t, a_b, b_b, out);
}

static Layout make_layout(const rtm_params &p, const Geom &g)
{
    Layout L;
    memset(&L, 0, sizeof L);
    const size_t es = p.compute == RTM_COMPUTE_FP64 ? 8 : 4;
    const size_t se = p.precision == RTM_PREC_FP32 ? es : 2;
    const size_t field = (size_t)g.dimx * g.pitch * es;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = align_up(off + bytes, 256); return o; };
    L.u[0] = take(field); L.u[1] = take(field);
    L.r[0] = take(field); L.r[1] = take(field);
    L.coef = take(field);
    const size_t n_l = (size_t)g.thl * g.pitch, n_r = (size_t)g.thr * g.pitch;
    const size_t n_t = (size_t)g.dimx * g.st, n_b = (size_t)g.dimx * g.sb;
    L.strips = off;
    L.psi[0] = take(n_l * es); L.psi[1] = take(n_r * es); L.psi[2] = take(n_t * es); L.psi[3] = take(n_b * es);
    L.xi[0] = take(n_l * es); L.xi[1] = take(n_r * es); L.xi[2] = take(n_t * es); L.xi[3] = take(n_b * es);
    L.psn[0] = take(n_l * es); L.psn[1] = take(n_r * es); L.psn[2] = take(n_t * es); L.psn[3] = take(n_b * es);
    L.strip_bytes = off - L.strips;
    L.prof = take(sizeof(float) * (size_t)prof_layout(g).total);
    L.rec = take(sizeof(int) * 3 * (size_t)g.dimx);
    L.wav = take(sizeof(float) * (size_t)std::max(p.n_wavelet, 1));
    L.seis_t = take(sizeof(float) * (size_t)std::max(1, p.rec_count) * p.nt);
    L.img = take(sizeof(double) * (size_t)g.nx * g.pitch);
    L.slf = take(sizeof(double) * (size_t)g.nx * g.pitch);
    if (p.storage == RTM_STORE_RING) {
        L.nslots = p.nt + 1;
        L.slot_elems = (size_t)g.ring_cells;
    } else {
        L.nslots = (p.nt + p.time_slices - 1) / p.time_slices;
        L.slot_elems = (size_t)g.nx * g.pitch;
    }
    L.store_bytes = (size_t)L.nslots * L.slot_elems * se;
    L.store = take(L.store_bytes);
    // 16-bit storage scales of one slot: per tile (snapshots) or per strip block (rings)
    L.n_scales_per_slot = std::max((size_t)g.tiles_x * g.tiles_z, (size_t)strip_blocks_host(g));
    L.scales = take(p.precision == RTM_PREC_FP32 ? 0 : sizeof(float) * L.nslots * L.n_scales_per_slot);
    const size_t stage = std::max({(size_t)g.dimx * g.dimz, (size_t)std::max(1, p.rec_count) * p.nt,
                                   (size_t)2 * g.nx * g.nz});
    L.staging = take(stage * sizeof(float) * (es / 4));
    L.status = take(256);
    L.total = off;
    return L;
}

// A profiled block of consecutive step-kernel launches: its events and launch count.
struct ProfBlock {
    cudaEvent_t e0, e1;
    int launches;
};

// ---- plan ---------------------------------------------------------------------------------
}  // namespace rtm

struct rtm_plan {
    rtm_params p;
    rtm::Geom g;
    rtm::Layout L;
    size_t es = 4;
    unsigned char *base = nullptr;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    CUtensorMap tm_u[2], tm_r[2];      // halo maps (box tx+8 x 136) of u[], r[]
    CUtensorMap tm_u8[2], tm_r8[2];    // 8-column x halo maps (box tx+16 x 136): side CPML tiles
    CUtensorMap tm_up[2], tm_rp[2];    // plain maps (box tx x 128) of u[], r[]
    CUtensorMap tm_c;                  // plain map of coef
    int cur_u = 0;        // u buffer holding u_nt after the forward pass
    int cur_r = 0;        // r buffer holding the last receiver field
    bool forward_done = false;
    bool image_valid = false;
    long long launches = 0;
    std::vector<float> h_prof;
    float *h_pinned = nullptr;   // pinned staging for host-buffer entry points
    size_t h_pinned_bytes = 0;
    // sampled timing of k_step: blocks of consecutive launches bracketed by CUDA events on
    // the plan's stream
    int prof_every = 0;
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_used = 0;
    std::vector<rtm::ProfBlock> prof_launch[2];   // [forward, backward]
    cudaEvent_t prof_e0 = nullptr;     // the open block's start event
    int prof_n = 0;                    // launches in the open block
    // CUDA graphs of the two time loops, captured on first use and replayed afterwards
    bool use_graphs = true;
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    int graph_key[2] = {-1, -1};
    long long graph_launches[2] = {0, 0};
    int capture_pass = -1;       // pass being captured (0 forward, 1 backward), or -1
    std::vector<rtm::ProfBlock> graph_events[2];
    // source-field captures of the next adjoint pass (rtm_plan_capture_source)
    std::vector<int> cap_times;
    void *cap_out = nullptr;

    template <typename T> T *at(size_t off) { return reinterpret_cast<T *>(base + off); }

    cudaEvent_t next_event()
    {
        if (ev_used == ev_pool.size()) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
            ev_pool.push_back(e);
        }
        return ev_pool[ev_used++];
    }
};

namespace rtm {

// Plain 2-D map over a pitched field: box {TZ, tx} (no halo), zero fill out of range.
static int make_plain_map(CUtensorMap *m, void *base, const Geom &g, size_t es)
{
    EncodeTiledFn enc = tensor_map_encoder();
    if (!enc) return fail(RTM_ERR_CUDA, "cuTensorMapEncodeTiled entry point unavailable");
    cuuint64_t dims[2] = {(cuuint64_t)g.pitch, (cuuint64_t)g.dimx};
    cuuint64_t strides[1] = {(cuuint64_t)g.pitch * es};
    cuuint32_t box[2] = {(cuuint32_t)TZ, (cuuint32_t)g.tx};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(m, es == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                     2, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(RTM_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return RTM_OK;
}

static int make_maps(rtm_plan *P)
{
    for (int i = 0; i < 2; ++i) {
        RTM_TRY(make_field_map(&P->tm_u[i], P->base + P->L.u[i], P->g, P->es));
        RTM_TRY(make_field_map(&P->tm_r[i], P->base + P->L.r[i], P->g, P->es));
        RTM_TRY(make_field_map(&P->tm_u8[i], P->base + P->L.u[i], P->g, P->es, 2 * HALO));
        RTM_TRY(make_field_map(&P->tm_r8[i], P->base + P->L.r[i], P->g, P->es, 2 * HALO));
        RTM_TRY(make_plain_map(&P->tm_up[i], P->base + P->L.u[i], P->g, P->es));
        RTM_TRY(make_plain_map(&P->tm_rp[i], P->base + P->L.r[i], P->g, P->es));
    }
    return make_plain_map(&P->tm_c, P->base + P->L.coef, P->g, P->es);
}

static int plan_alloc(const rtm_params &p, rtm_plan **out, bool batched = false)
{
    RTM_TRY(check_params(p));
    std::unique_ptr<rtm_plan> P(new rtm_plan());
    P->p = p;
    P->g = make_geom(p, batched);
    P->L = make_layout(p, P->g);
    P->es = p.compute == RTM_COMPUTE_FP64 ? 8 : 4;
    cudaError_t e = cudaMalloc(&P->base, P->L.total);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(RTM_ERR_NOMEM, "cudaMalloc(%zu bytes) failed: %s", P->L.total, cudaGetErrorString(e));
    }
    RTM_TRY(make_maps(P.get()));
    RTM_CUDA(cudaStreamCreateWithFlags(&P->stream, cudaStreamNonBlocking));
    P->own_stream = true;
    // CPML profiles (host, reference arithmetic) and receiver maps
    const Geom &g = P->g;
    std::vector<float> prof((size_t)prof_layout(g).total);
    make_profiles(p, g, prof.data());
    P->h_prof = prof;
    std::vector<int> rec(3 * (size_t)g.dimx, 0);
    int *last = rec.data(), *first = last + g.dimx, *cnt = first + g.dimx;
    for (int x = 0; x < g.dimx; ++x) { last[x] = -1; first[x] = -1; }
    for (int i = 0; i < p.rec_count; ++i) {
        const int x = g.thl + p.rec_first + (p.rec_spacing - 1) * i;  // backward_modeling.c:279
        last[x] = i;
        if (cnt[x] == 0) first[x] = i;
        cnt[x]++;
    }
    RTM_CUDA(cudaMemcpyAsync(P->base + P->L.prof, prof.data(), prof.size() * sizeof(float),
                             cudaMemcpyHostToDevice, P->stream));
    RTM_CUDA(cudaMemcpyAsync(P->base + P->L.rec, rec.data(), rec.size() * sizeof(int),
                             cudaMemcpyHostToDevice, P->stream));
    RTM_CUDA(cudaMemsetAsync(P->base + P->L.status, 0, 256, P->stream));
    RTM_CUDA(cudaStreamSynchronize(P->stream));
    *out = P.release();
    return RTM_OK;
}

static void plan_free(rtm_plan *P)
{
    if (!P) return;
    if (P->stream) cudaStreamSynchronize(P->stream);
    if (P->base) cudaFree(P->base);
    if (P->h_pinned) cudaFreeHost(P->h_pinned);
    for (cudaEvent_t e : P->ev_pool) cudaEventDestroy(e);
    for (int k = 0; k < 2; ++k) {
        if (P->gexec[k]) cudaGraphExecDestroy(P->gexec[k]);
        for (auto &pb : P->graph_events[k]) { cudaEventDestroy(pb.e0); cudaEventDestroy(pb.e1); }
    }
    if (P->own_stream && P->stream) cudaStreamDestroy(P->stream);
    delete P;
}

static int pinned(rtm_plan *P, size_t bytes, float **out)
{
    if (P->h_pinned_bytes < bytes) {
        if (P->h_pinned) cudaFreeHost(P->h_pinned);
        P->h_pinned = nullptr;
        P->h_pinned_bytes = 0;
        RTM_CUDA(cudaMallocHost(&P->h_pinned, bytes));
        P->h_pinned_bytes = bytes;
    }
    *out = P->h_pinned;
    return RTM_OK;
}

// psi buffers of step t: it reads set (t+1) & 1 (the previous step's psi) and writes set t & 1,
// set 0 = L.psi, set 1 = L.psn.
template <typename T>
static void set_psi_parity(rtm_plan *P, StepArgs<T> &a, int t)
{
    const size_t *rd = (t & 1) ? P->L.psi : P->L.psn;
    const size_t *wr = (t & 1) ? P->L.psn : P->L.psi;
    a.psi_l = P->at<T>(rd[0]); a.psi_r = P->at<T>(rd[1]); a.psi_t = P->at<T>(rd[2]); a.psi_b = P->at<T>(rd[3]);
    a.psn_l = P->at<T>(wr[0]); a.psn_r = P->at<T>(wr[1]); a.psn_t = P->at<T>(wr[2]); a.psn_b = P->at<T>(wr[3]);
}

template <typename T>
static void fill_common(rtm_plan *P, StepArgs<T> &a)
{
    memset(&a, 0, sizeof a);
    const Geom &g = P->g;
    a.g = g;
    const T dx = (T)P->p.dx;
    a.h1 = (T)1.0f / dx;
    a.h2 = dx * dx;
    a.h3 = (T)1.0f / (dx * dx);
    set_psi_parity<T>(P, a, 0);
    a.xi_l = P->at<T>(P->L.xi[0]); a.xi_r = P->at<T>(P->L.xi[1]);
    a.xi_t = P->at<T>(P->L.xi[2]); a.xi_b = P->at<T>(P->L.xi[3]);
    const float *prof = P->at<float>(P->L.prof);
    const ProfLayout pl = prof_layout(g);
    a.a_l = prof + pl.off[0]; a.b_l = prof + pl.off[1]; a.a_r = prof + pl.off[2]; a.b_r = prof + pl.off[3];
    a.a_t = prof + pl.off[4]; a.b_t = prof + pl.off[5]; a.a_b = prof + pl.off[6]; a.b_b = prof + pl.off[7];
    const int *rec = P->at<int>(P->L.rec);
    a.rec_last = rec; a.rec_first = rec + g.dimx; a.rec_cnt = rec + 2 * g.dimx;
    a.store_prec = P->p.precision;
    a.img = P->at<double>(P->L.img);
    a.slf = P->at<double>(P->L.slf);
    a.status = P->at<unsigned>(P->L.status);
}

static void *slot_ptr(rtm_plan *P, int slot)
{
    const size_t se = P->p.precision == RTM_PREC_FP32 ? P->es : 2;
    return P->base + P->L.store + (size_t)slot * P->L.slot_elems * se;
}

static float *scale_ptr(rtm_plan *P, int slot)
{
    if (P->p.precision == RTM_PREC_FP32) return nullptr;
    return P->at<float>(P->L.scales) + (size_t)slot * P->L.n_scales_per_slot;
}

// Launches per profiled block: with profiling on (prof_every > 0), the step kernels of steps
// [k every, k every + kProfBlock) are bracketed together by one pair of CUDA events, so that
// the launches inside a block keep their programmatic overlap; the block's time over its
// launches is their average launch duration.
constexpr int kProfBlock = 8;

static cudaEvent_t prof_event(rtm_plan *P)
{
    cudaEvent_t e = nullptr;
    if (P->capture_pass >= 0) {          // events owned by the graph being captured
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        return e;
    }
    return P->next_event();
}

// One k_step launch of a pass of `steps` steps, inside a profiled block when profiling is on.
// Consecutive step kernels chain by programmatic dependent launch, except right after an
// event record.
template <typename T>
static int timed_step(rtm_plan *P, int backward, int step, int steps, const StepMaps &maps,
                      const StepArgs<T> &a)
{
    const int every = P->prof_every;
    const int block = every > 0 ? std::min(kProfBlock, every) : 0;
    const bool opens = every > 0 && step % every == 0;
    const bool closes = every > 0 && step % every < block && (step % every == block - 1 || step == steps - 1);
    const unsigned rec_flags = P->capture_pass >= 0 ? cudaEventRecordExternal : 0;
    bool after_event = step == 0;
    if (opens) {
        P->prof_e0 = prof_event(P);
        if (!P->prof_e0) return fail(RTM_ERR_CUDA, "event pool");
        // inside a capture, an external event-record node keeps the event timeable
        RTM_CUDA(cudaEventRecordWithFlags(P->prof_e0, P->stream, rec_flags));
        P->prof_n = 0;
        after_event = true;
    }
    if (every > 0 && step > 0 && (step - 1) % every == block - 1) after_event = true;   // a block closed
    const int grid = step_grid<T>(backward, P->g);
    if (grid < 1) return fail(RTM_ERR_CUDA, "step kernel cannot be configured (tile_x %d)", P->g.tx);
    RTM_CUDA(launch_step<T>(backward, maps, a, grid, after_event ? 0 : 1, P->stream));
    P->prof_n++;
    if (closes) {
        cudaEvent_t e1 = prof_event(P);
        if (!e1) return fail(RTM_ERR_CUDA, "event pool");
        RTM_CUDA(cudaEventRecordWithFlags(e1, P->stream, rec_flags));
        const ProfBlock pb{P->prof_e0, e1, P->prof_n};
        if (P->capture_pass >= 0) P->graph_events[P->capture_pass].push_back(pb);
        else P->prof_launch[backward ? 1 : 0].push_back(pb);
    }
    return RTM_OK;
}

// Issues one pass's time loop (`issue` launches it on P->stream) directly, or through a
// CUDA graph captured on first use and replayed afterwards.  The kernels' arguments only
// name plan-owned buffers, so one capture serves every later migration of the plan.
template <typename F>
static int run_loop(rtm_plan *P, int which, bool graphable, F issue)
{
    if (!graphable || !P->use_graphs) return issue();
    const int key = P->prof_every;
    if (!P->gexec[which] || P->graph_key[which] != key) {
        if (P->gexec[which]) cudaGraphExecDestroy(P->gexec[which]);
        P->gexec[which] = nullptr;
        for (auto &pb : P->graph_events[which]) { cudaEventDestroy(pb.e0); cudaEventDestroy(pb.e1); }
        P->graph_events[which].clear();
        const long long before = P->launches;
        RTM_CUDA(cudaStreamBeginCapture(P->stream, cudaStreamCaptureModeThreadLocal));
        P->capture_pass = which;
        const int st = issue();
        P->capture_pass = -1;
        cudaGraph_t graph = nullptr;
        const cudaError_t e = cudaStreamEndCapture(P->stream, &graph);
        if (st != RTM_OK) {
            if (graph) cudaGraphDestroy(graph);
            return st;
        }
        if (e != cudaSuccess) return fail(RTM_ERR_CUDA, "stream capture: %s", cudaGetErrorString(e));
        const cudaError_t ei = cudaGraphInstantiate(&P->gexec[which], graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess) {
            P->gexec[which] = nullptr;
            return fail(RTM_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ei));
        }
        P->graph_launches[which] = P->launches - before;
        P->launches = before;
        P->graph_key[which] = key;
    }
    RTM_CUDA(cudaGraphLaunch(P->gexec[which], P->stream));
    P->launches += P->graph_launches[which];
    for (auto &pr : P->graph_events[which]) P->prof_launch[which].push_back(pr);
    return RTM_OK;
}

// Forward pass: SRC/forward_modeling.c:12-159 on the device.
template <typename T>
static int run_forward(rtm_plan *P, const float *d_vel, int vel_pitch, const float *d_wav,
                       T *d_seis_out)
{
    NvtxRange range("rtm forward pass");
    const Geom &g = P->g;
    cudaStream_t s = P->stream;
    T *u[2] = {P->at<T>(P->L.u[0]), P->at<T>(P->L.u[1])};
    RTM_CUDA(launch_coef<T>(g, d_vel, vel_pitch, P->at<T>(P->L.coef), P->p.dx, P->p.dt, s));
    P->launches++;
    RTM_CUDA(cudaMemsetAsync(u[0], 0, (size_t)g.dimx * g.pitch * sizeof(T), s));
    RTM_CUDA(cudaMemsetAsync(u[1], 0, (size_t)g.dimx * g.pitch * sizeof(T), s));
    RTM_CUDA(cudaMemsetAsync(P->base + P->L.strips, 0, P->L.strip_bytes, s));
    StepArgs<T> a;
    fill_common<T>(P, a);
    a.wavelet = d_wav;
    a.rec_out = d_seis_out;
    const bool ring = P->p.storage == RTM_STORE_RING;
    (void)step_grid<T>(0, g);            // configure the kernels before any capture
    auto loop = [&]() -> int {
        int c = 0;
        StepMaps maps;
        for (int t = 0; t < g.nt; ++t) {
            a.u_next = u[1 - c];
            a.t = t;
            set_psi_parity<T>(P, a, t);
            int f = 0;
            if (t < g.nwav) f |= F_SRC;
            if (d_seis_out && g.nrec > 0) f |= F_RECORD;
            a.store = nullptr;
            a.store_scale = nullptr;
            if (ring) {                  // slot k holds the ring of u_k: full-precision rings
                f |= F_RING_SAVE;        // are saved from u_t (step t), 16-bit ones from u_{t+1}
                const int slot = P->p.precision == RTM_PREC_FP32 ? t : t + 1;
                a.store = slot_ptr(P, slot);
                a.store_scale = scale_ptr(P, slot);
            } else if (t % g.slices == 0) {
                f |= F_SNAP_SAVE;
                a.store = slot_ptr(P, t / g.slices);
                a.store_scale = scale_ptr(P, t / g.slices);
            }
            a.flags = f;
            maps.cur = P->tm_u[c];
            maps.cur8 = P->tm_u8[c];
            maps.prev = P->tm_up[1 - c];
            maps.coef = P->tm_c;
            maps.scur = P->tm_u[c];
            maps.sprev = P->tm_up[1 - c];
            RTM_TRY(timed_step<T>(P, 0, t, g.nt, maps, a));
            P->launches += 1;
            c ^= 1;
        }
        return RTM_OK;
    };
    RTM_TRY(run_loop(P, 0, d_seis_out == nullptr, loop));
    const int c = g.nt & 1;             // u buffer holding u_nt
    P->cur_u = c;
    P->forward_done = true;
    P->image_valid = false;
    return RTM_OK;
}

static int check_status(rtm_plan *P)
{
    unsigned st = 0;
    RTM_CUDA(cudaMemcpyAsync(&st, P->base + P->L.status, sizeof st, cudaMemcpyDeviceToHost, P->stream));
    RTM_CUDA(cudaStreamSynchronize(P->stream));
    if (st & ST_TMA_TIMEOUT) {
        cudaMemsetAsync(P->base + P->L.status, 0, sizeof st, P->stream);
        return fail(RTM_ERR_TIMEOUT, "a tile load did not complete within its time limit");
    }
    return RTM_OK;
}

// Adjoint pass: SRC/backward_modeling.c:12-165 on the device.  d_seis: [irec][nt].
template <typename T>
static int run_adjoint(rtm_plan *P, const float *d_seis)
{
    NvtxRange range("rtm adjoint pass");
    if (!P->forward_done) return fail(RTM_ERR_STATE, "adjoint pass without a forward pass");
    const Geom &g = P->g;
    cudaStream_t s = P->stream;
    T *u[2] = {P->at<T>(P->L.u[0]), P->at<T>(P->L.u[1])};
    T *r[2] = {P->at<T>(P->L.r[0]), P->at<T>(P->L.r[1])};
    float *seis_t = P->at<float>(P->L.seis_t);
    if (g.nrec > 0) {
        RTM_CUDA(launch_transpose(d_seis, seis_t, g.nrec, g.nt, s));
        P->launches++;
    }
    RTM_CUDA(cudaMemsetAsync(r[0], 0, (size_t)g.dimx * g.pitch * sizeof(T), s));
    RTM_CUDA(cudaMemsetAsync(r[1], 0, (size_t)g.dimx * g.pitch * sizeof(T), s));
    RTM_CUDA(cudaMemsetAsync(P->base + P->L.strips, 0, P->L.strip_bytes, s));
    RTM_CUDA(cudaMemsetAsync(P->base + P->L.img, 0, sizeof(double) * (size_t)g.nx * g.pitch, s));
    RTM_CUDA(cudaMemsetAsync(P->base + P->L.slf, 0, sizeof(double) * (size_t)g.nx * g.pitch, s));
    StepArgs<T> a;
    fill_common<T>(P, a);
    a.wavelet = P->at<float>(P->L.wav);
    const bool ring = P->p.storage == RTM_STORE_RING;
    const int ua = P->cur_u, ub = 1 - P->cur_u;   // u_nt, u_{nt-1}
    (void)step_grid<T>(1, g);            // configure the kernels before any capture
    // source-field captures: u_nt and u_{nt-1} are the forward pass's last fields; u_t for
    // t <= nt - 2 is the reconstruction output of backward step nt - t
    const size_t cap_n = (size_t)g.dimx * g.dimz;
    auto capture = [&](int t, const T *field) -> int {
        for (size_t k = 0; k < P->cap_times.size(); ++k)
            if (P->cap_times[k] == t) {
                RTM_CUDA(launch_field_out<T>(g, field, static_cast<T *>(P->cap_out) + k * cap_n, s));
                P->launches++;
            }
        return RTM_OK;
    };
    if (!P->cap_times.empty()) {
        RTM_TRY(capture(g.nt, u[ua]));
        RTM_TRY(capture(g.nt - 1, u[ub]));
    }
    auto loop = [&]() -> int {
        int sc = ub, sp = ua;                          // reconstruction: current / previous
        int c = 0;
        int ctrl = g.nt / g.slices - 1;                // backward_modeling.c:267
        for (int time = 0; time < g.nt; ++time) {
            const int tau = g.nt - time - 1;
            int f = F_OVERWRITE;
            a.seis_row = seis_t + (size_t)tau * std::max(g.nrec, 1);
            if (g.nrec == 0) f &= ~F_OVERWRITE;
            a.t = time;
            a.store = nullptr;
            a.store_scale = nullptr;
            a.s_next = nullptr;
            a.s_snap = nullptr;
            a.s_fixed = nullptr;
            const bool recon = ring && time >= 2;
            if (recon) {
                f |= F_RECON;
                if (tau + 2 < g.nwav) f |= F_RECON_SRC;
                a.s_next = u[sp];
                a.store = slot_ptr(P, tau + 1);
                a.store_scale = scale_ptr(P, tau + 1);
            }
            if (tau % g.slices == 0) {
                if (ctrl >= 0) {
                    f |= F_IMAGE;
                    if (!ring) {
                        f |= F_IMAGE_SNAP;
                        a.s_snap = reinterpret_cast<const T *>(slot_ptr(P, ctrl));
                        a.store = slot_ptr(P, ctrl);
                        a.store_scale = scale_ptr(P, ctrl);
                    } else if (!recon) {
                        f |= F_IMAGE_FIXED;
                        a.s_fixed = time == 0 ? u[ua] : u[ub];
                    }
                }
                ctrl--;
            }
            a.flags = f;
            a.u_next = r[1 - c];
            set_psi_parity<T>(P, a, time);
            StepMaps maps;
            maps.cur = P->tm_r[c];
            maps.cur8 = P->tm_r8[c];
            maps.prev = P->tm_rp[1 - c];
            maps.coef = P->tm_c;
            maps.scur = P->tm_u[sc];
            maps.sprev = P->tm_up[sp];
            RTM_TRY(timed_step<T>(P, 1, time, g.nt, maps, a));
            P->launches += 1;
            c ^= 1;
            if (recon && !P->cap_times.empty()) RTM_TRY(capture(g.nt - time, u[sp]));
            if (recon) std::swap(sc, sp);
        }
        return RTM_OK;
    };
    RTM_TRY(run_loop(P, 1, P->cap_times.empty(), loop));
    const int c = g.nt & 1;             // r buffer holding the last receiver field
    P->cur_r = c;
    P->forward_done = false;   // the stored source wavefield has been consumed
    P->image_valid = true;
    return RTM_OK;
}

template <typename T>
static int plan_forward(rtm_plan *P, const float *d_vel, int vel_pitch, const float *d_wav,
                        void *d_seis_out)
{
    // The adjoint pass undoes the source term during reconstruction: keep the wavelet.
    float *wav = P->at<float>(P->L.wav);
    if (P->g.nwav > 0 && d_wav != wav)
        RTM_CUDA(cudaMemcpyAsync(wav, d_wav, sizeof(float) * P->g.nwav, cudaMemcpyDeviceToDevice,
                                 P->stream));
    return run_forward<T>(P, d_vel, vel_pitch, wav, reinterpret_cast<T *>(d_seis_out));
}

static int dispatch_forward(rtm_plan *P, const float *d_vel, int vel_pitch, const float *d_wav,
                            void *d_seis_out)
{
    if (P->es == 8) return plan_forward<double>(P, d_vel, vel_pitch, d_wav, d_seis_out);
    return plan_forward<float>(P, d_vel, vel_pitch, d_wav, d_seis_out);
}

static int dispatch_adjoint(rtm_plan *P, const float *d_seis)
{
    if (P->es == 8) return run_adjoint<double>(P, d_seis);
    return run_adjoint<float>(P, d_seis);
}

// Image (float, nx x nz) from the FP64 accumulators.
static int image_to(rtm_plan *P, int which, void *d_out, int as_double, int accumulate)
{
    if (!P->image_valid) return fail(RTM_ERR_STATE, "no image: run the adjoint pass first");
    const double *src = P->at<double>(which ? P->L.slf : P->L.img);
    if (as_double) RTM_CUDA(launch_image_out<double>(P->g, src, (double *)d_out, accumulate, P->stream));
    else RTM_CUDA(launch_image_out<float>(P->g, src, (float *)d_out, accumulate, P->stream));
    P->launches++;
    return RTM_OK;
}

// ---- plan cache for the host-buffer entry points -------------------------------------
static std::mutex g_mu;
static std::map<int, rtm_plan *> g_sim;           // sim_id -> plan holding a forward state
static std::vector<rtm_plan *> g_idle;            // finished plans kept for reuse

static bool same_params(const rtm_params &a, const rtm_params &b)
{
    return memcmp(&a, &b, sizeof a) == 0;
}

static int acquire_plan(const rtm_params &p, rtm_plan **out)
{
    {
        std::lock_guard<std::mutex> lk(g_mu);
        for (size_t i = 0; i < g_idle.size(); ++i)
            if (same_params(g_idle[i]->p, p)) {
                *out = g_idle[i];
                g_idle.erase(g_idle.begin() + i);
                return RTM_OK;
            }
    }
    return plan_alloc(p, out);
}

static void release_plan(rtm_plan *P)
{
    std::lock_guard<std::mutex> lk(g_mu);
    g_idle.push_back(P);
    while (g_idle.size() > 2) {
        plan_free(g_idle.front());
        g_idle.erase(g_idle.begin());
    }
}

static int upload_host(rtm_plan *P, void *dst, const void *src, size_t bytes)
{
    float *h;
    RTM_TRY(pinned(P, bytes, &h));
    RTM_CUDA(cudaStreamSynchronize(P->stream));   // pinned staging is free again
    memcpy(h, src, bytes);
    RTM_CUDA(cudaMemcpyAsync(dst, h, bytes, cudaMemcpyHostToDevice, P->stream));
    return RTM_OK;
}

static int forward_host(rtm_plan *P, const float *velocity, const float *wavelet, void *d_seis)
{
    const Geom &g = P->g;
    float *stage = P->at<float>(P->L.staging);
    RTM_TRY(upload_host(P, stage, velocity, sizeof(float) * (size_t)g.dimx * g.dimz));
    float *wav = P->at<float>(P->L.wav);
    if (g.nwav > 0) {
        RTM_CUDA(cudaStreamSynchronize(P->stream));
        RTM_CUDA(cudaMemcpyAsync(wav, wavelet, sizeof(float) * g.nwav, cudaMemcpyHostToDevice, P->stream));
    }
    return dispatch_forward(P, stage, g.dimz, wav, d_seis);
}

static int adjoint_host(rtm_plan *P, const float *seismogram, float *image, float *self_image)
{
    const Geom &g = P->g;
    float *stage = P->at<float>(P->L.staging);
    if (g.nrec > 0) RTM_TRY(upload_host(P, stage, seismogram, sizeof(float) * (size_t)g.nrec * g.nt));
    RTM_TRY(dispatch_adjoint(P, stage));
    const size_t n = (size_t)g.nx * g.nz;
    RTM_TRY(image_to(P, 0, stage, 0, 0));
    RTM_TRY(image_to(P, 1, stage + n, 0, 0));
    float *h;
    RTM_TRY(pinned(P, 2 * n * sizeof(float), &h));
    RTM_CUDA(cudaMemcpyAsync(h, stage, 2 * n * sizeof(float), cudaMemcpyDeviceToHost, P->stream));
    RTM_TRY(check_status(P));
    // imageCondition[i] += ..., selfImageCondition[i] += ... (image_conditions.c:28-30)
    for (size_t i = 0; i < n; ++i) image[i] = image[i] + h[i];
    for (size_t i = 0; i < n; ++i) self_image[i] = self_image[i] + h[n + i];
    return RTM_OK;
}

}  // namespace rtm

using namespace rtm;

// ================================ C ABI ======================================================
extern "C" {

void rtm_params_defaults(rtm_params *p)
{
    p->storage = RTM_STORE_RING;
    p->precision = RTM_PREC_FP32;
    p->compute = RTM_COMPUTE_FP32;
    p->tile_x = 0;
    p->reserved[0] = p->reserved[1] = p->reserved[2] = 0;
}

int rtm_params_check(const rtm_params *p)
{
    if (!p) return fail(RTM_ERR_INVALID, "null params");
    return check_params(*p);
}

long long rtm_footprint_bytes(const rtm_params *p)
{
    if (!p || check_params(*p) != RTM_OK) return -1;
    const Geom g = make_geom(*p);
    return (long long)make_layout(*p, g).total;
}

const char *rtm_status_string(int status)
{
    switch (status) {
    case RTM_OK: return "ok";
    case RTM_ERR_INVALID: return "invalid argument";
    case RTM_ERR_CUDA: return "CUDA error";
    case RTM_ERR_NOMEM: return "out of device memory";
    case RTM_ERR_STATE: return "call out of order";
    case RTM_ERR_TIMEOUT: return "device wait timed out";
    case RTM_ERR_IO: return "I/O error";
    case RTM_ERR_DECODE: return "decode error";
    case RTM_ERR_BUSY: return "busy";
    default: return "unknown status";
    }
}

const char *rtm_last_error(void) { return t_err.c_str(); }

int rtm_device_info(char *name, int name_len, int *sm_count, long long *hbm_bytes)
{
    int dev = 0;
    RTM_CUDA(cudaGetDevice(&dev));
    cudaDeviceProp prop;
    RTM_CUDA(cudaGetDeviceProperties(&prop, dev));
    if (name && name_len > 0) snprintf(name, name_len, "%s", prop.name);
    if (sm_count) *sm_count = prop.multiProcessorCount;
    if (hbm_bytes) *hbm_bytes = (long long)prop.totalGlobalMem;
    return RTM_OK;
}

// Times `steps` forward steps of *p's grid (constant 2000 m/s medium, the configured source)
// for each tile width the step kernel supports and keeps the fastest for this grid shape.
int rtm_autotune(const rtm_params *p, int steps, int *best_tile_x, float *best_ms_per_step)
{
    NvtxRange range("rtm autotune");
    if (!p) return fail(RTM_ERR_INVALID, "null argument");
    RTM_TRY(check_params(*p));
    if (steps < 1) return fail(RTM_ERR_INVALID, "steps must be >= 1");
    rtm_params q = *p;
    q.nt = (steps + q.time_slices - 1) / q.time_slices * q.time_slices;
    const int cands[3] = {8, 16, 32};
    int best = -1;
    float best_ms = 0.0f;
    for (int tx : cands) {
        if (q.compute == RTM_COMPUTE_FP64 && tx > 16) continue;
        q.tile_x = tx;
        rtm_plan *P = nullptr;
        int st = plan_alloc(q, &P);
        if (st != RTM_OK) return st;
        const size_t nv = (size_t)P->g.dimx * P->g.dimz;
        float *d_vel = nullptr, *d_wav = nullptr;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        float ms = 0.0f;
        std::vector<float> hv(nv, 2000.0f), hw((size_t)std::max(q.n_wavelet, 1), 0.0f);
        for (size_t k = 0; k < hw.size(); ++k) hw[k] = (k % 7) * 0.1f;
        cudaError_t e = cudaMalloc(&d_vel, nv * sizeof(float));
        if (e == cudaSuccess) e = cudaMalloc(&d_wav, hw.size() * sizeof(float));
        if (e == cudaSuccess) e = cudaMemcpy(d_vel, hv.data(), nv * sizeof(float), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(d_wav, hw.data(), hw.size() * sizeof(float), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaEventCreate(&e0);
        if (e == cudaSuccess) e = cudaEventCreate(&e1);
        for (int rep = 0; rep < 2 && e == cudaSuccess && st == RTM_OK; ++rep) {
            e = cudaEventRecord(e0, P->stream);
            if (e == cudaSuccess) st = dispatch_forward(P, d_vel, P->g.dimz, d_wav, nullptr);
            if (e == cudaSuccess && st == RTM_OK) e = cudaEventRecord(e1, P->stream);
            if (e == cudaSuccess && st == RTM_OK) e = cudaEventSynchronize(e1);
            if (e == cudaSuccess && st == RTM_OK) e = cudaEventElapsedTime(&ms, e0, e1);
        }
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        cudaFree(d_vel);
        cudaFree(d_wav);
        plan_free(P);
        if (st != RTM_OK) return st;
        if (e != cudaSuccess) return fail(RTM_ERR_CUDA, "autotune: %s", cudaGetErrorString(e));
        const float per = ms / (float)q.nt;
        if (best < 0 || per < best_ms) { best = tx; best_ms = per; }
    }
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        g_tuned[tune_key(*p)] = best;
    }
    if (best_tile_x) *best_tile_x = best;
    if (best_ms_per_step) *best_ms_per_step = best_ms;
    return RTM_OK;
}

int rtm_plan_create(const rtm_params *p, rtm_plan **plan)
{
    if (!p || !plan) return fail(RTM_ERR_INVALID, "null argument");
    return plan_alloc(*p, plan);
}

int rtm_plan_destroy(rtm_plan *plan)
{
    plan_free(plan);
    return RTM_OK;
}

int rtm_plan_set_stream(rtm_plan *plan, void *stream)
{
    if (!plan) return fail(RTM_ERR_INVALID, "null plan");
    RTM_CUDA(cudaStreamSynchronize(plan->stream));
    if (plan->own_stream) cudaStreamDestroy(plan->stream);
    plan->stream = (cudaStream_t)stream;
    plan->own_stream = false;
    return RTM_OK;
}

int rtm_plan_forward(rtm_plan *plan, const void *d_velocity, const void *d_wavelet,
                     void *d_seismogram_out)
{
    if (!plan || !d_velocity || (!d_wavelet && plan->g.nwav > 0))
        return fail(RTM_ERR_INVALID, "null argument");
    return dispatch_forward(plan, (const float *)d_velocity, plan->g.dimz, (const float *)d_wavelet,
                            d_seismogram_out);
}

int rtm_plan_adjoint(rtm_plan *plan, const void *d_seismogram, void *d_image, void *d_self_image)
{
    if (!plan || (!d_seismogram && plan->g.nrec > 0)) return fail(RTM_ERR_INVALID, "null argument");
    if (!plan->forward_done) return fail(RTM_ERR_STATE, "adjoint pass without a forward pass");
    // the wavelet of the forward pass is needed for the source term of the reconstruction
    RTM_TRY(dispatch_adjoint(plan, (const float *)d_seismogram));
    if (d_image) RTM_TRY(image_to(plan, 0, d_image, 0, 0));
    if (d_self_image) RTM_TRY(image_to(plan, 1, d_self_image, 0, 0));
    return check_status(plan);
}

int rtm_plan_read_image(rtm_plan *plan, int which, int as_double, void *d_out)
{
    if (!plan || !d_out) return fail(RTM_ERR_INVALID, "null argument");
    return image_to(plan, which, d_out, as_double, 0);
}

int rtm_plan_read_field(rtm_plan *plan, int which, void *d_out)
{
    if (!plan || !d_out) return fail(RTM_ERR_INVALID, "null argument");
    const size_t off = which == 0 ? plan->L.u[plan->cur_u]
                     : which == 1 ? plan->L.u[1 - plan->cur_u]
                                  : plan->L.r[1 - plan->cur_r];
    if (plan->es == 8) RTM_CUDA(launch_field_out<double>(plan->g, plan->at<double>(off), (double *)d_out, plan->stream));
    else RTM_CUDA(launch_field_out<float>(plan->g, plan->at<float>(off), (float *)d_out, plan->stream));
    plan->launches++;
    RTM_CUDA(cudaStreamSynchronize(plan->stream));
    return RTM_OK;
}

int rtm_plan_capture_source(rtm_plan *P, int count, const int *times, void *d_out)
{
    if (!P) return fail(RTM_ERR_INVALID, "null plan");
    if (count < 0 || (count > 0 && (!times || !d_out))) return fail(RTM_ERR_INVALID, "bad capture list");
    if (count > 0 && P->p.storage != RTM_STORE_RING)
        return fail(RTM_ERR_INVALID, "source-field capture needs ring storage (the reconstructed field)");
    for (int k = 0; k < count; ++k)
        if (times[k] < 0 || times[k] > P->p.nt) return fail(RTM_ERR_INVALID, "capture time %d outside [0, nt]", times[k]);
    P->cap_times.assign(times, times + count);
    P->cap_out = count > 0 ? d_out : nullptr;
    return RTM_OK;
}

int rtm_plan_sync(rtm_plan *plan)
{
    if (!plan) return fail(RTM_ERR_INVALID, "null plan");
    return check_status(plan);
}

long long rtm_plan_launch_count(const rtm_plan *plan) { return plan ? plan->launches : -1; }

int rtm_plan_profile(rtm_plan *plan, int every)
{
    if (!plan || every < 0) return fail(RTM_ERR_INVALID, "bad argument");
    RTM_CUDA(cudaStreamSynchronize(plan->stream));
    plan->prof_every = every;
    plan->ev_used = 0;
    plan->prof_launch[0].clear();
    plan->prof_launch[1].clear();
    return RTM_OK;
}

int rtm_plan_profile_read(rtm_plan *plan, double *fwd_ms, int *fwd_n, double *bwd_ms, int *bwd_n)
{
    if (!plan) return fail(RTM_ERR_INVALID, "null plan");
    RTM_CUDA(cudaStreamSynchronize(plan->stream));
    double ms[2] = {0.0, 0.0};
    int n[2] = {0, 0};
    for (int k = 0; k < 2; ++k)
        for (auto &pb : plan->prof_launch[k]) {
            float v = 0.0f;
            RTM_CUDA(cudaEventElapsedTime(&v, pb.e0, pb.e1));
            ms[k] += v;
            n[k] += pb.launches;
        }
    if (fwd_ms) *fwd_ms = ms[0];
    if (fwd_n) *fwd_n = n[0];
    if (bwd_ms) *bwd_ms = ms[1];
    if (bwd_n) *bwd_n = n[1];
    plan->ev_used = 0;
    plan->prof_launch[0].clear();
    plan->prof_launch[1].clear();
    return RTM_OK;
}

long long rtm_plan_bytes(const rtm_plan *plan) { return plan ? (long long)plan->L.total : -1; }

// ---- reference-shaped host-buffer entry points ------------------------------------------
static rtm_params with_shot(const rtm_params *p, const int *shot)
{
    rtm_params q = *p;
    if (shot) { q.shot_x = shot[0]; q.shot_z = shot[1]; }
    return q;
}

int rtm_forward_modeling(const rtm_params *p, int sim_id, const int *shot, const float *velocity,
                         const float *wavelet)
{
    if (!p || !velocity || (!wavelet && p->n_wavelet > 0)) return fail(RTM_ERR_INVALID, "null argument");
    const rtm_params q = with_shot(p, shot);
    rtm_plan *P = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        auto it = g_sim.find(sim_id);
        if (it != g_sim.end()) {          // a forward state nobody consumed: replace it
            P = it->second;
            g_sim.erase(it);
        }
    }
    if (P && !same_params(P->p, q)) { plan_free(P); P = nullptr; }
    if (!P) RTM_TRY(acquire_plan(q, &P));
    int st = forward_host(P, velocity, wavelet, nullptr);
    if (st != RTM_OK) { release_plan(P); return st; }
    std::lock_guard<std::mutex> lk(g_mu);
    g_sim[sim_id] = P;
    return RTM_OK;
}

int rtm_adjoint_modeling(const rtm_params *p, int sim_id, const int *shot, const float *velocity,
                         const float *wavelet, const float *seismogram, float *image,
                         float *self_image)
{
    (void)velocity; (void)wavelet;   // the forward pass already holds coef and the wavelet
    if (!p || !image || !self_image || (!seismogram && p->rec_count > 0))
        return fail(RTM_ERR_INVALID, "null argument");
    rtm_plan *P = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        auto it = g_sim.find(sim_id);
        if (it == g_sim.end()) return fail(RTM_ERR_STATE, "no forward state for simulation %d", sim_id);
        P = it->second;
        g_sim.erase(it);
    }
    if (!same_params(P->p, with_shot(p, shot))) {
        release_plan(P);
        return fail(RTM_ERR_INVALID, "parameters differ from the forward pass of simulation %d", sim_id);
    }
    const int st = adjoint_host(P, seismogram, image, self_image);
    release_plan(P);
    return st;
}

int rtm_migrate_shot(const rtm_params *p, const float *velocity, const float *wavelet,
                     const float *seismogram, float *image, float *self_image)
{
    if (!p || !velocity || !image || !self_image) return fail(RTM_ERR_INVALID, "null argument");
    if (p->n_wavelet > 0 && !wavelet) return fail(RTM_ERR_INVALID, "null wavelet");
    if (p->rec_count > 0 && !seismogram) return fail(RTM_ERR_INVALID, "null seismogram");
    rtm_plan *P = nullptr;
    RTM_TRY(acquire_plan(*p, &P));
    int st = forward_host(P, velocity, wavelet, nullptr);
    if (st == RTM_OK) st = adjoint_host(P, seismogram, image, self_image);
    release_plan(P);
    return st;
}

int rtm_migrate_shot_zfp(const rtm_params *p, const float *velocity, const float *wavelet,
                         const void *zfp_stream, size_t zfp_bytes, float tol, float *image,
                         float *self_image)
{
    if (!p || !velocity || !image || !self_image) return fail(RTM_ERR_INVALID, "null argument");
    if (p->n_wavelet > 0 && !wavelet) return fail(RTM_ERR_INVALID, "null wavelet");
    if (p->rec_count > 0 && !zfp_stream) return fail(RTM_ERR_INVALID, "null seismogram stream");
    rtm_plan *P = nullptr;
    RTM_TRY(acquire_plan(*p, &P));
    // the host decodes the seismogram on a thread of its own while the forward pass runs
    const size_t n = (size_t)std::max(p->rec_count, 0) * (size_t)p->nt;
    std::vector<float> seis(std::max<size_t>(n, 1));
    int dec_st = RTM_OK;
    std::thread decoder([&] {
        if (n) dec_st = rtm_zfp_decode_float2d(zfp_stream, zfp_bytes, tol, p->rec_count, p->nt, seis.data());
    });
    int st = forward_host(P, velocity, wavelet, nullptr);
    decoder.join();
    if (st == RTM_OK && dec_st != RTM_OK) st = fail(dec_st, "seismogram stream: %s", rtm_status_string(dec_st));
    if (st == RTM_OK) st = adjoint_host(P, seis.data(), image, self_image);
    if (st != RTM_OK) cudaStreamSynchronize(P->stream);
    release_plan(P);
    return st;
}

int rtm_model_seismogram(const rtm_params *p, const float *velocity, const float *wavelet,
                         float *seismogram)
{
    if (!p || !velocity || !seismogram) return fail(RTM_ERR_INVALID, "null argument");
    if (p->n_wavelet > 0 && !wavelet) return fail(RTM_ERR_INVALID, "null wavelet");
    if (p->compute != RTM_COMPUTE_FP32) return fail(RTM_ERR_INVALID, "host recording is FP32");
    rtm_plan *P = nullptr;
    RTM_TRY(acquire_plan(*p, &P));
    const size_t n = (size_t)p->rec_count * p->nt;
    float *d_seis = nullptr;
    int st = RTM_OK;
    if (cudaMalloc(&d_seis, std::max<size_t>(n, 1) * sizeof(float)) != cudaSuccess) {
        cudaGetLastError();
        release_plan(P);
        return fail(RTM_ERR_NOMEM, "seismogram buffer");
    }
    st = forward_host(P, velocity, wavelet, n ? d_seis : nullptr);
    if (st == RTM_OK && n) {
        if (cudaMemcpyAsync(seismogram, d_seis, n * sizeof(float), cudaMemcpyDeviceToHost, P->stream) != cudaSuccess)
            st = fail(RTM_ERR_CUDA, "seismogram download");
    }
    if (st == RTM_OK) st = check_status(P);
    P->forward_done = false;
    cudaFree(d_seis);
    release_plan(P);
    return st;
}

}  // extern "C"

// ---- shot stack on the device ----------------------------------------------------------
// One allocation: acc = [image stack | self-image stack] (float32, nx x nz each, [x][z]),
// out = [stacked image | its Laplacian], then the status word, so that the final result and
// the status come back in one copy.
struct rtm_stack {
    rtm_params p;
    Geom g;
    size_t n = 0;
    unsigned char *base = nullptr;
    float *acc_img = nullptr, *acc_slf = nullptr, *out = nullptr;
    unsigned *status = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t last_add = nullptr;    // the latest shot's accumulation (shot order)
    bool added = false;
    float *h_pinned = nullptr;         // 2n floats + the status word
    long long d2h_copies = 0, d2h_bytes = 0;
};

namespace rtm {

static void stack_free(rtm_stack *S)
{
    if (!S) return;
    if (S->stream) cudaStreamSynchronize(S->stream);
    if (S->last_add) cudaEventDestroy(S->last_add);
    if (S->base) cudaFree(S->base);
    if (S->h_pinned) cudaFreeHost(S->h_pinned);
    if (S->stream) cudaStreamDestroy(S->stream);
    delete S;
}

// Makes the stack's stream wait for the latest accumulation.
static int stack_order(rtm_stack *S, cudaStream_t s)
{
    if (S->added) RTM_CUDA(cudaStreamWaitEvent(s, S->last_add, 0));
    return RTM_OK;
}

}  // namespace rtm

extern "C" {

int rtm_stack_create(const rtm_params *p, rtm_stack **out)
{
    if (!p || !out) return fail(RTM_ERR_INVALID, "null argument");
    *out = nullptr;
    RTM_TRY(check_params(*p));
    std::unique_ptr<rtm_stack> S(new rtm_stack());
    S->p = *p;
    S->g = make_geom(*p);
    S->n = (size_t)p->nx * p->nz;
    const size_t bytes = 4 * S->n * sizeof(float) + 256;
    cudaError_t e = cudaMalloc(&S->base, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        S->base = nullptr;
        return fail(RTM_ERR_NOMEM, "cudaMalloc(%zu bytes) for the shot stack: %s", bytes, cudaGetErrorString(e));
    }
    float *f = reinterpret_cast<float *>(S->base);
    S->acc_img = f;
    S->acc_slf = f + S->n;
    S->out = f + 2 * S->n;
    S->status = reinterpret_cast<unsigned *>(f + 4 * S->n);
    rtm_stack *raw = S.release();
    auto bail = [&](int st) { stack_free(raw); return st; };
    if (cudaStreamCreateWithFlags(&raw->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&raw->last_add, cudaEventDisableTiming) != cudaSuccess ||
        cudaMallocHost(&raw->h_pinned, 2 * raw->n * sizeof(float) + sizeof(unsigned)) != cudaSuccess) {
        cudaGetLastError();
        return bail(fail(RTM_ERR_CUDA, "shot stack: stream, event or pinned buffer"));
    }
    if (cudaMemsetAsync(raw->base, 0, bytes, raw->stream) != cudaSuccess ||
        cudaStreamSynchronize(raw->stream) != cudaSuccess)
        return bail(fail(RTM_ERR_CUDA, "shot stack: clear"));
    *out = raw;
    return RTM_OK;
}

int rtm_stack_destroy(rtm_stack *stack)
{
    stack_free(stack);
    return RTM_OK;
}

int rtm_stack_load(rtm_stack *S, const float *image_stack, const float *self_stack)
{
    if (!S) return fail(RTM_ERR_INVALID, "null stack");
    RTM_TRY(stack_order(S, S->stream));
    const size_t b = S->n * sizeof(float);
    RTM_CUDA(cudaStreamSynchronize(S->stream));    // the pinned buffer is free
    if (image_stack) memcpy(S->h_pinned, image_stack, b);
    else memset(S->h_pinned, 0, b);
    if (self_stack) memcpy(S->h_pinned + S->n, self_stack, b);
    else memset(S->h_pinned + S->n, 0, b);
    RTM_CUDA(cudaMemcpyAsync(S->acc_img, S->h_pinned, 2 * b, cudaMemcpyHostToDevice, S->stream));
    RTM_CUDA(cudaEventRecord(S->last_add, S->stream));
    S->added = true;
    RTM_CUDA(cudaStreamSynchronize(S->stream));
    return RTM_OK;
}

int rtm_adjoint_modeling_stacked(const rtm_params *p, int sim_id, const int *shot, const float *seismogram,
                                 rtm_stack *S)
{
    if (!p || !S || (!seismogram && p->rec_count > 0)) return fail(RTM_ERR_INVALID, "null argument");
    if (p->nx != S->p.nx || p->nz != S->p.nz) return fail(RTM_ERR_INVALID, "stack of another image size");
    rtm_plan *P = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        auto it = g_sim.find(sim_id);
        if (it == g_sim.end()) return fail(RTM_ERR_STATE, "no forward state for simulation %d", sim_id);
        P = it->second;
        g_sim.erase(it);
    }
    if (!same_params(P->p, with_shot(p, shot))) {
        release_plan(P);
        return fail(RTM_ERR_INVALID, "parameters differ from the forward pass of simulation %d", sim_id);
    }
    auto run = [&]() -> int {
        const Geom &g = P->g;
        float *stage = P->at<float>(P->L.staging);
        if (g.nrec > 0) RTM_TRY(upload_host(P, stage, seismogram, sizeof(float) * (size_t)g.nrec * g.nt));
        RTM_TRY(dispatch_adjoint(P, stage));
        if (!P->image_valid) return fail(RTM_ERR_STATE, "no image after the adjoint pass");
        RTM_TRY(stack_order(S, P->stream));           // the shots' sums in shot order
        RTM_CUDA(launch_stack_add(g, P->at<double>(P->L.img), P->at<double>(P->L.slf), S->acc_img, S->acc_slf,
                                  P->at<unsigned>(P->L.status), S->status, P->stream));
        P->launches++;
        RTM_CUDA(cudaEventRecord(S->last_add, P->stream));
        S->added = true;
        return RTM_OK;
    };
    const int st = run();
    release_plan(P);
    return st;
}

int rtm_stack_read_raw(rtm_stack *S, float *image_stack, float *self_stack)
{
    if (!S || !image_stack || !self_stack) return fail(RTM_ERR_INVALID, "null argument");
    RTM_TRY(stack_order(S, S->stream));
    const size_t b = 2 * S->n * sizeof(float);
    RTM_CUDA(cudaMemcpyAsync(S->h_pinned, S->acc_img, b, cudaMemcpyDeviceToHost, S->stream));
    RTM_CUDA(cudaStreamSynchronize(S->stream));
    S->d2h_copies++;
    S->d2h_bytes += (long long)b;
    memcpy(image_stack, S->h_pinned, S->n * sizeof(float));
    memcpy(self_stack, S->h_pinned + S->n, S->n * sizeof(float));
    return RTM_OK;
}

int rtm_stack_finish(rtm_stack *S, int normalize_by_self, float *stacked, float *laplacian)
{
    if (!S || !stacked || !laplacian) return fail(RTM_ERR_INVALID, "null argument");
    const int nx = S->p.nx, nz = S->p.nz;
    const size_t n = S->n;
    float *out = S->out, *lap = S->out + n;
    RTM_TRY(stack_order(S, S->stream));
    RTM_CUDA(launch_stack_finish((int)n, S->acc_img, S->acc_slf, normalize_by_self, out, S->stream));
    RTM_CUDA(cudaMemsetAsync(lap, 0, n * sizeof(float), S->stream));
    RTM_CUDA(launch_laplacian(nx, nz, out, lap, S->stream));
    // stacked image, Laplacian and status word: one copy
    const size_t b = 2 * n * sizeof(float) + sizeof(unsigned);
    RTM_CUDA(cudaMemcpyAsync(S->h_pinned, out, b, cudaMemcpyDeviceToHost, S->stream));
    RTM_CUDA(cudaStreamSynchronize(S->stream));
    S->d2h_copies++;
    S->d2h_bytes += (long long)b;
    unsigned st;
    memcpy(&st, S->h_pinned + 2 * n, sizeof st);
    if (st & ST_TMA_TIMEOUT) return fail(RTM_ERR_TIMEOUT, "a tile load of a stacked shot did not complete within its time limit");
    memcpy(stacked, S->h_pinned, n * sizeof(float));
    memcpy(laplacian, S->h_pinned + n, n * sizeof(float));
    return RTM_OK;
}

int rtm_stack_transfers(const rtm_stack *S, long long *d2h_copies, long long *d2h_bytes)
{
    if (!S) return fail(RTM_ERR_INVALID, "null stack");
    if (d2h_copies) *d2h_copies = S->d2h_copies;
    if (d2h_bytes) *d2h_bytes = S->d2h_bytes;
    return RTM_OK;
}

void rtm_release_cached(void)
{
    std::lock_guard<std::mutex> lk(g_mu);
    for (rtm_plan *P : g_idle) plan_free(P);
    g_idle.clear();
    for (auto &kv : g_sim) plan_free(kv.second);
    g_sim.clear();
}

}  // extern "C"

// ---- per-step drop-ins on host buffers (parity and unit testing of single steps) -------
namespace rtm {

// A plan sized for one step of *p: no receivers, one storage slot.
static int step_plan(const rtm_params *p, rtm_plan **out)
{
    rtm_params q = *p;
    q.nt = 1; q.time_slices = 1; q.n_wavelet = 0; q.rec_count = 0;
    q.shot_x = 0; q.shot_z = 0;
    q.storage = RTM_STORE_SNAPSHOT; q.precision = RTM_PREC_FP32; q.compute = RTM_COMPUTE_FP32;
    return acquire_plan(q, out);
}

// host [dimx][dimz] -> pitched device field
static int field_from_host(rtm_plan *P, float *dst, const float *src)
{
    float *stage = P->at<float>(P->L.staging);
    RTM_TRY(upload_host(P, stage, src, sizeof(float) * (size_t)P->g.dimx * P->g.dimz));
    RTM_CUDA(launch_field_in<float>(P->g, stage, dst, P->stream));
    P->launches++;
    return RTM_OK;
}

static int field_to_host(rtm_plan *P, float *dst, const float *src)
{
    float *stage = P->at<float>(P->L.staging);
    RTM_CUDA(launch_field_out<float>(P->g, src, stage, P->stream));
    P->launches++;
    RTM_CUDA(cudaMemcpyAsync(dst, stage, sizeof(float) * (size_t)P->g.dimx * P->g.dimz,
                             cudaMemcpyDeviceToHost, P->stream));
    RTM_CUDA(cudaStreamSynchronize(P->stream));
    return RTM_OK;
}

// strip arrays between the reference layouts and the pitched device layouts.  A one-step
// plan's step (t = 0) reads psi from the second buffer (L.psn) and writes it to the first
// (L.psi): psi goes up to L.psn and comes back from L.psi.
static int strips_io(rtm_plan *P, int to_device, float *const host[8])
{
    const Geom &g = P->g;
    // the bottom strip's reference rows start at z = dimZ - th_down, the device rows at zb0
    const size_t bsh = (size_t)((g.dimz - g.thd) - g.zb0);
    const size_t *psi = to_device ? P->L.psn : P->L.psi;
    struct { size_t off; int rows, host_w, dev_w; size_t shift; } s[8] = {
        {psi[0], g.thl, g.dimz, g.pitch, 0}, {psi[1], g.thr, g.dimz, g.pitch, 0},
        {psi[2], g.dimx, g.thu, g.st, 0},    {psi[3], g.dimx, g.thd, g.sb, bsh},
        {P->L.xi[0], g.thl, g.dimz, g.pitch, 0},  {P->L.xi[1], g.thr, g.dimz, g.pitch, 0},
        {P->L.xi[2], g.dimx, g.thu, g.st, 0},     {P->L.xi[3], g.dimx, g.thd, g.sb, bsh}};
    for (int i = 0; i < 8; ++i) {
        unsigned char *row0 = P->base + s[i].off;
        float *dev = reinterpret_cast<float *>(row0) + s[i].shift;
        if (to_device) {
            RTM_CUDA(cudaMemsetAsync(row0, 0, (size_t)s[i].rows * s[i].dev_w * sizeof(float), P->stream));
            RTM_CUDA(cudaMemcpy2DAsync(dev, s[i].dev_w * sizeof(float), host[i], s[i].host_w * sizeof(float),
                                       s[i].host_w * sizeof(float), s[i].rows, cudaMemcpyHostToDevice, P->stream));
            if (i < 4) {                  // psi: the written buffer starts as the input, so that
                                          // the cells the step does not update come back as given
                unsigned char *w0 = P->base + P->L.psi[i];
                RTM_CUDA(cudaMemcpyAsync(w0, row0, (size_t)s[i].rows * s[i].dev_w * sizeof(float),
                                         cudaMemcpyDeviceToDevice, P->stream));
            }
        } else {
            RTM_CUDA(cudaMemcpy2DAsync(host[i], s[i].host_w * sizeof(float), dev, s[i].dev_w * sizeof(float),
                                       s[i].host_w * sizeof(float), s[i].rows, cudaMemcpyDeviceToHost, P->stream));
        }
    }
    RTM_CUDA(cudaStreamSynchronize(P->stream));
    return RTM_OK;
}

// One step of u[0] into u[1] (t = 0: psi read from L.psn, written to L.psi; see strips_io).
static int one_step(rtm_plan *P, int flags)
{
    StepArgs<float> a;
    fill_common<float>(P, a);
    a.u_next = P->at<float>(P->L.u[1]);
    a.flags = flags;
    StepMaps maps;
    maps.cur = P->tm_u[0];
    maps.cur8 = P->tm_u8[0];
    maps.prev = P->tm_up[1];
    maps.coef = P->tm_c;
    maps.scur = P->tm_u[0];
    maps.sprev = P->tm_up[1];
    RTM_CUDA(launch_step<float>(0, maps, a, step_grid<float>(0, P->g), 0, P->stream));
    P->launches++;
    return check_status(P);
}

}  // namespace rtm

extern "C" {

int rtm_iso_acoustic_wave_equation(const rtm_params *p, const float *pond, const float *wave2,
                                   float *wave3)
{
    if (!p || !pond || !wave2 || !wave3) return fail(RTM_ERR_INVALID, "null argument");
    rtm_plan *P = nullptr;
    RTM_TRY(step_plan(p, &P));
    int st = field_from_host(P, P->at<float>(P->L.coef), pond);
    if (st == RTM_OK) st = field_from_host(P, P->at<float>(P->L.u[0]), wave2);
    if (st == RTM_OK) st = field_from_host(P, P->at<float>(P->L.u[1]), wave3);
    if (st == RTM_OK) st = one_step(P, F_NO_CPML);
    if (st == RTM_OK) st = field_to_host(P, wave3, P->at<float>(P->L.u[1]));
    release_plan(P);
    return st;
}

int rtm_aiso_attenuation_cpml(const rtm_params *p, const float *wave1, float *wave2,
                              const float *coef, const float *a_left, const float *b_left,
                              const float *a_right, const float *b_right, const float *a_top,
                              const float *b_top, const float *a_bottom, const float *b_bottom,
                              float *psi_left, float *psi_right, float *psi_top,
                              float *psi_bottom, float *xi_left, float *xi_right, float *xi_top,
                              float *xi_bottom)
{
    if (!p || !wave1 || !wave2 || !coef) return fail(RTM_ERR_INVALID, "null argument");
    rtm_plan *P = nullptr;
    RTM_TRY(step_plan(p, &P));
    const Geom &g = P->g;
    int st = field_from_host(P, P->at<float>(P->L.coef), coef);
    if (st == RTM_OK) st = field_from_host(P, P->at<float>(P->L.u[0]), wave1);
    if (st == RTM_OK) st = field_from_host(P, P->at<float>(P->L.u[1]), wave2);
    float *strips[8] = {psi_left, psi_right, psi_top, psi_bottom, xi_left, xi_right, xi_top, xi_bottom};
    if (st == RTM_OK) st = strips_io(P, 1, strips);
    // caller-supplied profiles for this call; the plan's own are restored afterwards
    std::vector<float> prof(P->h_prof.size());
    pack_profiles(g, a_left, b_left, a_right, b_right, a_top, b_top, a_bottom, b_bottom, prof.data());
    if (st == RTM_OK && cudaMemcpy(P->base + P->L.prof, prof.data(), prof.size() * sizeof(float),
                                   cudaMemcpyHostToDevice) != cudaSuccess)
        st = fail(RTM_ERR_CUDA, "profile upload");
    if (st == RTM_OK) st = one_step(P, F_NO_STENCIL);
    if (st == RTM_OK) st = field_to_host(P, wave2, P->at<float>(P->L.u[1]));
    if (st == RTM_OK) st = strips_io(P, 0, strips);
    cudaMemcpy(P->base + P->L.prof, P->h_prof.data(), P->h_prof.size() * sizeof(float),
               cudaMemcpyHostToDevice);
    release_plan(P);
    return st;
}

int rtm_normalized_cross_correlation(const rtm_params *p, float *image, float *self_image,
                                     const float *source, const float *receiver)
{
    if (!p || !image || !self_image || !source || !receiver) return fail(RTM_ERR_INVALID, "null argument");
    rtm_plan *P = nullptr;
    RTM_TRY(step_plan(p, &P));
    const Geom &g = P->g;
    const size_t n = (size_t)g.nx * g.nz;
    int st = field_from_host(P, P->at<float>(P->L.u[0]), source);
    if (st == RTM_OK) st = field_from_host(P, P->at<float>(P->L.r[0]), receiver);
    float *stage = P->at<float>(P->L.staging);
    if (st == RTM_OK) {
        cudaMemsetAsync(P->base + P->L.img, 0, sizeof(double) * (size_t)g.nx * g.pitch, P->stream);
        cudaMemsetAsync(P->base + P->L.slf, 0, sizeof(double) * (size_t)g.nx * g.pitch, P->stream);
        if (launch_xcorr<float>(g, P->at<float>(P->L.u[0]), P->at<float>(P->L.r[0]),
                                P->at<double>(P->L.img), P->at<double>(P->L.slf), P->stream) != cudaSuccess)
            st = fail(RTM_ERR_CUDA, "xcorr launch");
        P->image_valid = true;
        P->launches++;
    }
    if (st == RTM_OK) st = upload_host(P, stage, image, n * sizeof(float));
    if (st == RTM_OK) st = image_to(P, 0, stage, 0, 1);
    if (st == RTM_OK && cudaMemcpyAsync(image, stage, n * sizeof(float), cudaMemcpyDeviceToHost, P->stream) != cudaSuccess)
        st = fail(RTM_ERR_CUDA, "image download");
    if (st == RTM_OK) st = upload_host(P, stage, self_image, n * sizeof(float));
    if (st == RTM_OK) st = image_to(P, 1, stage, 0, 1);
    if (st == RTM_OK && cudaMemcpyAsync(self_image, stage, n * sizeof(float), cudaMemcpyDeviceToHost, P->stream) != cudaSuccess)
        st = fail(RTM_ERR_CUDA, "image download");
    if (st == RTM_OK) st = check_status(P);
    P->image_valid = false;
    release_plan(P);
    return st;
}

int rtm_laplacian_filter2D(const rtm_params *p, float *lp, const float *image)
{
    if (!p || !lp || !image) return fail(RTM_ERR_INVALID, "null argument");
    if (p->nx < 1 || p->nz < 1) return fail(RTM_ERR_INVALID, "empty image");
    const size_t n = (size_t)p->nx * p->nz;
    float *d = nullptr;
    if (cudaMalloc(&d, 2 * n * sizeof(float)) != cudaSuccess) {
        cudaGetLastError();
        return fail(RTM_ERR_NOMEM, "laplacian buffers");
    }
    int st = RTM_OK;
    if (cudaMemcpy(d, image, n * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
        launch_laplacian(p->nx, p->nz, d, d + n, 0) != cudaSuccess)
        st = fail(RTM_ERR_CUDA, "laplacian");
    // only the cells the reference writes: [4, nx-4) x [4, nz-4) (math_functions.c:11-14)
    if (st == RTM_OK && p->nx > 8 && p->nz > 8 &&
        cudaMemcpy2D(lp + 4 * (size_t)p->nz + 4, p->nz * sizeof(float), d + n + 4 * (size_t)p->nz + 4,
                     p->nz * sizeof(float), (p->nz - 8) * sizeof(float), p->nx - 8,
                     cudaMemcpyDeviceToHost) != cudaSuccess)
        st = fail(RTM_ERR_CUDA, "laplacian download");
    cudaFree(d);
    return st;
}

}  // extern "C"

// ---- single-shot migration without device allocation --------------------------------------
// Scratch of rtm_migrate_shot_static: the wavefields, CPML strips, source-wavefield store,
// transposed seismogram and FP64 image accumulators of one migration live in this
// file-scope array instead of a cudaMalloc'd plan.  Every GPU that loads the library holds
// these 64 MiB until the process exits.  All calls on a device share it.
#define RTM_STATIC_SCRATCH_BYTES (64ull << 20)
#define RTM_STATIC_MAX_THICK 512
static __device__ __align__(256) unsigned char g_static_scratch[RTM_STATIC_SCRATCH_BYTES];

namespace rtm {

// Receiver column maps on the device (same maps plan_alloc builds on the host).
__global__ void k_rec_maps(Geom g, int rec_first, int rec_spacing, int rec_count, int *last,
                           int *first, int *cnt)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= g.dimx) return;
    const int c0 = g.thl + rec_first;                    // column of receiver 0
    const int step = rec_spacing - 1;                    // backward_modeling.c:279
    int l = -1, f = -1, n = 0;
    if (rec_count > 0) {
        if (step == 0) {
            if (x == c0) { l = rec_count - 1; f = 0; n = rec_count; }
        } else if ((x - c0) % step == 0) {
            const int i = (x - c0) / step;
            if (i >= 0 && i < rec_count) { l = i; f = i; n = 1; }
        }
    }
    last[x] = l;
    first[x] = f;
    cnt[x] = n;
}

static std::mutex g_static_mu;
static void *g_static_ptr[256];

// Device address of the static scratch on device `dev` (looked up once per device, with
// that device current).
static int static_scratch(int dev, void **out)
{
    std::lock_guard<std::mutex> lk(g_static_mu);
    if (dev < 0 || dev >= 256) return fail(RTM_ERR_INVALID, "device ordinal %d out of range", dev);
    if (!g_static_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p)
            return fail(RTM_ERR_CUDA, "cudaGetSymbolAddress(static scratch): %s", cudaGetErrorString(e));
        g_static_ptr[dev] = p;
    }
    *out = g_static_ptr[dev];
    return RTM_OK;
}

}  // namespace rtm

extern "C" int rtm_migrate_shot_static(const rtm_params *p, const void *d_velocity,
                                       const void *d_wavelet, const void *d_seismogram,
                                       void *d_image, void *d_self_image, void *stream)
{
    if (!p || !d_velocity || !d_image || !d_self_image) return fail(RTM_ERR_INVALID, "null argument");
    if (p->n_wavelet > 0 && !d_wavelet) return fail(RTM_ERR_INVALID, "null wavelet");
    if (p->rec_count > 0 && !d_seismogram) return fail(RTM_ERR_INVALID, "null seismogram");
    RTM_TRY(check_params(*p));
    if (p->th_left > RTM_STATIC_MAX_THICK || p->th_right > RTM_STATIC_MAX_THICK ||
        p->th_up > RTM_STATIC_MAX_THICK || p->th_down > RTM_STATIC_MAX_THICK)
        return fail(RTM_ERR_INVALID, "CPML thicker than %d cells", RTM_STATIC_MAX_THICK);
    const Geom g = make_geom(*p);
    const Layout L = make_layout(*p, g);
    if (L.total > RTM_STATIC_SCRATCH_BYTES)
        return fail(RTM_ERR_INVALID,
                    "this migration needs %zu bytes of scratch; the static array holds %llu bytes",
                    L.total, (unsigned long long)RTM_STATIC_SCRATCH_BYTES);
    int dev = 0;
    RTM_CUDA(cudaGetDevice(&dev));
    void *base = nullptr;
    RTM_TRY(static_scratch(dev, &base));

    rtm_plan P;                                   // host-side view over the static scratch
    P.p = *p;
    P.g = g;
    P.L = L;
    P.es = p->compute == RTM_COMPUTE_FP64 ? 8 : 4;
    P.base = static_cast<unsigned char *>(base);
    P.stream = static_cast<cudaStream_t>(stream);
    P.own_stream = false;
    P.use_graphs = false;                         // nothing outlives the call
    RTM_TRY(make_maps(&P));
    // what the previous call left in the array: status word and receiver maps are rebuilt;
    // fields, strips and accumulators are zeroed by the forward / adjoint drivers
    if (cudaMemsetAsync(P.base + L.status, 0, 256, P.stream) != cudaSuccess) {
        cudaGetLastError();
        cudaStreamSynchronize(P.stream);
        return fail(RTM_ERR_CUDA, "clearing the status word of the static scratch");
    }
    float ref[8 * RTM_STATIC_MAX_THICK], prof[8 * (RTM_STATIC_MAX_THICK + 16)];
    float *a_l = ref, *b_l = a_l + g.thl, *a_r = b_l + g.thl, *b_r = a_r + g.thr;
    float *a_t = b_r + g.thr, *b_t = a_t + g.thu, *a_b = b_t + g.thu, *b_b = a_b + g.thd;
    rtm_attenuation_profile_cpml(p, a_l, a_r, a_t, a_b, b_l, b_r, b_t, b_b);
    pack_profiles(g, a_l, b_l, a_r, b_r, a_t, b_t, a_b, b_b, prof);
    if (cudaMemcpyAsync(P.base + L.prof, prof, sizeof(float) * (size_t)prof_layout(g).total,
                        cudaMemcpyHostToDevice, P.stream) != cudaSuccess) {
        cudaGetLastError();
        cudaStreamSynchronize(P.stream);
        return fail(RTM_ERR_CUDA, "uploading the CPML profiles to the static scratch");
    }
    // From the first enqueued operation on, a failure waits for what is already queued on the
    // stream before it returns, so that nothing of this call still writes the shared array
    // when the next call starts.
    auto run = [&]() -> int {
        int *rec = P.at<int>(L.rec);
        k_rec_maps<<<(g.dimx + 127) / 128, 128, 0, P.stream>>>(g, p->rec_first, p->rec_spacing, p->rec_count,
                                                                rec, rec + g.dimx, rec + 2 * g.dimx);
        RTM_CUDA(cudaGetLastError());
        RTM_TRY(dispatch_forward(&P, static_cast<const float *>(d_velocity), g.dimz,
                                 static_cast<const float *>(d_wavelet), nullptr));
        RTM_TRY(dispatch_adjoint(&P, static_cast<const float *>(d_seismogram)));
        RTM_TRY(image_to(&P, 0, d_image, 0, 0));
        RTM_TRY(image_to(&P, 1, d_self_image, 0, 0));
        return check_status(&P);
    };
    const int st = run();
    if (st != RTM_OK) cudaStreamSynchronize(P.stream);
    return st;
}

#include "rtm_serve.cuh"
