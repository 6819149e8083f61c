// rtm_serve.cuh -- serving and batching engine (host side; included at the end of
// rtm_engine.cu, whose plan helpers it uses).
//
// A server holds up to kMaxMembers resident migrations ("members").  Requests are admitted
// in arrival order while a member slot is free and their device footprint fits the HBM
// budget; admission uploads the inputs and sets the member up (coef, seismogram transpose,
// zeroed wavefields and image accumulators).  rtm_server_step replays a CUDA graph of
// `steps_per_launch` batched time steps (k_mstep + k_bpsi + k_bstrip per step, chained by
// programmatic dependent launch): every active member advances one step per batched step,
// whatever its grid, time axis or pass.  Members that finished their backward pass are harvested (image
// and self image copied to host buffers) and their slots freed for the next admissions --
// continuous batching.  One thread drives a server; each server has its own stream.

namespace rtm {

struct ServeRequest {
    long long id;
    rtm_params p;
    std::vector<float> vel, wav, seis;     // host copies of the inputs
    std::vector<unsigned char> zfp;        // ZFP seismogram still to decode (or empty)
    float zfp_tol = 0.0f;
    std::atomic<int> ready{1};             // 0 while a decoder thread works on it, -1 failed
    double t_submit, t_admit, t_done;
    std::vector<float> img, slf;
    long long bytes;
};

}  // namespace rtm

struct rtm_server {
    long long budget = 0, in_use = 0;
    int max_members = rtm::kMaxMembers;
    int steps_per_launch = 16;
    cudaStream_t stream = nullptr;
    // admission uploads run on their own stream while the graph replays on `stream`; the
    // admitted members are activated (descriptor, state) on `stream` after both
    cudaStream_t up = nullptr;
    cudaEvent_t up_ev = nullptr;
    std::vector<int> pending;              // slots uploaded, not yet activated
    std::vector<int> finished;             // slots whose member finished, not yet harvested
    double last_replay_ms = 0.0;
    // device side
    rtm::BatchIndex *d_ix = nullptr;
    rtm::BMember<float> *d_mem = nullptr;
    int2 *d_state = nullptr;
    unsigned *d_done = nullptr;
    // host mirrors
    std::vector<rtm::BMember<float>> mem;
    rtm::BatchIndex ix;
    int2 *h_state = nullptr;               // pinned
    std::vector<rtm_plan *> slot_plan;     // plan backing each slot (nullptr: free)
    std::vector<rtm::ServeRequest *> slot_req;
    std::vector<rtm_plan *> idle;          // finished plans kept for reuse
    std::deque<rtm::ServeRequest *> queue;
    std::map<long long, rtm::ServeRequest *> done;
    long long next_id = 1;
    cudaGraphExec_t gexec = nullptr;
    long long cell_updates_done = 0;
    long long launches = 0;
    double busy_ms = 0.0;                  // GPU time of the replays (events)
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // the tile kernel of the second step of each replay, timed alone (no overlap with the
    // kernels around it): events recorded by the graph, read after each replay
    cudaEvent_t kev0 = nullptr, kev1 = nullptr;
    bool kernel_sampled = false;
    double kernel_ms_last = 0.0;
    // host threads decoding ZFP seismograms of submitted requests (rtm_server_submit_zfp)
    std::vector<std::thread> decoders;
    std::deque<rtm::ServeRequest *> to_decode;
    std::mutex dmu;
    std::condition_variable dcv;
    bool stopping = false;
};

namespace rtm {

static double now_s()
{
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

static void member_from_plan(rtm_plan *P, BMember<float> &M)
{
    memset(&M, 0, sizeof M);
    M.tm_u[0] = P->tm_u[0]; M.tm_u[1] = P->tm_u[1];
    M.tm_up[0] = P->tm_up[0]; M.tm_up[1] = P->tm_up[1];
    M.tm_r[0] = P->tm_r[0]; M.tm_r[1] = P->tm_r[1];
    M.tm_rp[0] = P->tm_rp[0]; M.tm_rp[1] = P->tm_rp[1];
    M.tm_c = P->tm_c;
    M.g = P->g;
    const float dx = P->p.dx;
    M.h1 = 1.0f / dx;
    M.h2 = dx * dx;
    M.h3 = 1.0f / (dx * dx);
    M.u[0] = P->at<float>(P->L.u[0]); M.u[1] = P->at<float>(P->L.u[1]);
    M.r[0] = P->at<float>(P->L.r[0]); M.r[1] = P->at<float>(P->L.r[1]);
    M.coef = P->at<float>(P->L.coef);
    for (int k = 0; k < 4; ++k) {
        M.psi[k] = P->at<float>(P->L.psi[k]);
        M.xi[k] = P->at<float>(P->L.xi[k]);
    }
    const float *prof = P->at<float>(P->L.prof);
    const ProfLayout pl = prof_layout(P->g);
    for (int k = 0; k < 8; ++k) M.prof[k] = prof + pl.off[k];
    const int *rec = P->at<int>(P->L.rec);
    M.rec_last = rec; M.rec_first = rec + P->g.dimx; M.rec_cnt = rec + 2 * P->g.dimx;
    M.wav = P->at<float>(P->L.wav);
    M.seis_t = P->at<float>(P->L.seis_t);
    M.img = P->at<double>(P->L.img);
    M.slf = P->at<double>(P->L.slf);
    M.store = P->base + P->L.store;
    M.slot_elems = P->L.slot_elems;
    M.scales = P->p.precision == RTM_PREC_FP32 ? nullptr : P->at<float>(P->L.scales);
    M.scales_per_slot = (int)P->L.n_scales_per_slot;
    M.store_prec = P->p.precision;
    M.storage = P->p.storage;
    M.status = P->at<unsigned>(P->L.status);
}

// Work lists of the current membership (inactive slots own no work).
static void rebuild_index(rtm_server *S)
{
    S->ix.nmem = S->max_members;
    int b1 = 0, b2 = 0, pb = 0, cb = 0;
    for (int m = 0; m < S->max_members; ++m) {
        S->ix.base1[m] = b1;
        S->ix.base2[m] = b2;
        S->ix.psi_base[m] = pb;
        S->ix.corr_base[m] = cb;
        S->ix.tiles[m] = 0;
        S->ix.nb[m] = 0;
        S->ix.nt[m] = 0;
        if (S->slot_plan[m]) {
            const rtm_plan *P = S->slot_plan[m];
            const Geom &g = P->g;
            int n[4];
            psi_counts_host(g, n);
            const int nb = boundary_tiles_host(g);
            b1 += (g.tiles - nb) + (P->p.storage == RTM_STORE_RING ? g.tiles : 0);
            b2 += nb;
            pb += n[0] + n[1] + n[2] + n[3];
            cb += strip_items_host(g, P->p.storage == RTM_STORE_RING);
            S->ix.tiles[m] = g.tiles;
            S->ix.nb[m] = nb;
            S->ix.nt[m] = g.nt;
        }
    }
    S->ix.base1[S->max_members] = b1;
    S->ix.base2[S->max_members] = b2;
    S->ix.psi_base[S->max_members] = pb;
    S->ix.corr_base[S->max_members] = cb;
}

// Uploads one admitted request into slot m on the upload stream: the graph replaying on the
// server's stream touches only active members, and this one becomes active (activate) after
// the replay and these uploads.  The sources are the request's pageable host copies: each
// copy returns once its data is staged, so they are released right after.
static int admit(rtm_server *S, int m, ServeRequest *R)
{
    NvtxRange range("rtm server admit");
    rtm_plan *P = nullptr;
    for (size_t i = 0; i < S->idle.size(); ++i)
        if (same_params(S->idle[i]->p, R->p)) {
            P = S->idle[i];
            S->idle.erase(S->idle.begin() + i);
            break;
        }
    if (!P) {
        // make room: drop reusable plans that do not match
        while (!S->idle.empty() && S->in_use + R->bytes > S->budget) {
            S->in_use -= (long long)S->idle.back()->L.total;
            plan_free(S->idle.back());
            S->idle.pop_back();
        }
        RTM_TRY(plan_alloc(R->p, &P, true));
        S->in_use += (long long)P->L.total;
        RTM_CUDA(cudaStreamSynchronize(P->stream));
        if (P->own_stream) cudaStreamDestroy(P->stream);
        P->stream = S->stream;
        P->own_stream = false;
    }
    const Geom &g = P->g;
    if (g.tx != kBatchTileX && g.tx != kBatchTileX / 2) {   // tensor-map boxes must match the kernel's tiles
        S->idle.push_back(P);
        return fail(RTM_ERR_INVALID, "batched member with tile width %d (needs %d or %d)", g.tx, kBatchTileX, kBatchTileX / 2);
    }
    cudaStream_t s = S->up;
    float *stage = P->at<float>(P->L.staging);
    RTM_CUDA(cudaMemcpyAsync(stage, R->vel.data(), R->vel.size() * sizeof(float), cudaMemcpyHostToDevice, s));
    RTM_CUDA(launch_coef<float>(g, stage, g.dimz, P->at<float>(P->L.coef), P->p.dx, P->p.dt, s));
    if (g.nwav > 0)
        RTM_CUDA(cudaMemcpyAsync(P->at<float>(P->L.wav), R->wav.data(), sizeof(float) * g.nwav,
                                 cudaMemcpyHostToDevice, s));
    if (g.nrec > 0) {                     // staging is reused after the coef kernel (stream order)
        RTM_CUDA(cudaMemcpyAsync(stage, R->seis.data(), R->seis.size() * sizeof(float), cudaMemcpyHostToDevice, s));
        RTM_CUDA(launch_transpose(stage, P->at<float>(P->L.seis_t), g.nrec, g.nt, s));
    }
    const size_t field = (size_t)g.dimx * g.pitch * sizeof(float);
    for (int k = 0; k < 2; ++k) {
        RTM_CUDA(cudaMemsetAsync(P->base + P->L.u[k], 0, field, s));
        RTM_CUDA(cudaMemsetAsync(P->base + P->L.r[k], 0, field, s));
    }
    // psi/xi cells outside the updated ranges are read by the stencils as zero; the updated
    // ones restart from zero at each pass (F_STRIPS_FRESH)
    RTM_CUDA(cudaMemsetAsync(P->base + P->L.strips, 0, P->L.strip_bytes, s));
    RTM_CUDA(cudaMemsetAsync(P->base + P->L.img, 0, sizeof(double) * (size_t)g.nx * g.pitch, s));
    RTM_CUDA(cudaMemsetAsync(P->base + P->L.slf, 0, sizeof(double) * (size_t)g.nx * g.pitch, s));
    RTM_CUDA(cudaMemsetAsync(P->base + P->L.status, 0, 256, s));
    std::vector<float>().swap(R->vel);
    std::vector<float>().swap(R->seis);
    member_from_plan(P, S->mem[m]);
    S->pending.push_back(m);
    S->slot_plan[m] = P;
    S->slot_req[m] = R;
    R->t_admit = now_s();
    return RTM_OK;
}

// Activates the members uploaded by admit: after the graph replay enqueued before them and
// after their uploads, their descriptors and initial state (1, 0) are written and the work
// lists rebuilt, all on the server's stream.
static int activate(rtm_server *S)
{
    if (S->pending.empty()) return RTM_OK;
    static const int2 kFirstStep = {1, 0};
    RTM_CUDA(cudaEventRecord(S->up_ev, S->up));
    RTM_CUDA(cudaStreamWaitEvent(S->stream, S->up_ev, 0));
    for (int m : S->pending) {
        RTM_CUDA(cudaMemcpyAsync(S->d_mem + m, &S->mem[m], sizeof(BMember<float>), cudaMemcpyHostToDevice,
                                 S->stream));
        RTM_CUDA(cudaMemcpyAsync(S->d_state + m, &kFirstStep, sizeof kFirstStep, cudaMemcpyHostToDevice,
                                 S->stream));
    }
    S->pending.clear();
    rebuild_index(S);
    RTM_CUDA(cudaMemcpyAsync(S->d_ix, &S->ix, sizeof S->ix, cudaMemcpyHostToDevice, S->stream));
    return RTM_OK;
}

// A finished member's image and self image to its request, on the upload stream: the graph
// replaying meanwhile skips the member (its state is past its backward pass), so the copies
// overlap the replay.  The slot is free afterwards.
static int harvest(rtm_server *S, int m)
{
    NvtxRange range("rtm server harvest");
    rtm_plan *P = S->slot_plan[m];
    ServeRequest *R = S->slot_req[m];
    const Geom &g = P->g;
    const size_t n = (size_t)g.nx * g.nz;
    float *stage = P->at<float>(P->L.staging);
    cudaStream_t s = S->up;
    RTM_CUDA(launch_image_out<float>(g, P->at<double>(P->L.img), stage, 0, s));
    RTM_CUDA(launch_image_out<float>(g, P->at<double>(P->L.slf), stage + n, 0, s));
    R->img.resize(n);
    R->slf.resize(n);
    RTM_CUDA(cudaMemcpyAsync(R->img.data(), stage, n * sizeof(float), cudaMemcpyDeviceToHost, s));
    RTM_CUDA(cudaMemcpyAsync(R->slf.data(), stage + n, n * sizeof(float), cudaMemcpyDeviceToHost, s));
    unsigned st = 0;
    RTM_CUDA(cudaMemcpyAsync(&st, P->base + P->L.status, sizeof st, cudaMemcpyDeviceToHost, s));
    static const int2 kIdle = {0, 0};
    RTM_CUDA(cudaMemcpyAsync(S->d_state + m, &kIdle, sizeof kIdle, cudaMemcpyHostToDevice, s));
    RTM_CUDA(cudaStreamSynchronize(s));
    R->t_done = now_s();
    S->cell_updates_done += 2LL * g.dimx * g.dimz * g.nt;
    S->done[R->id] = R;
    S->slot_plan[m] = nullptr;
    S->slot_req[m] = nullptr;
    S->idle.push_back(P);
    if (st) return fail(RTM_ERR_TIMEOUT, "a tile load of request %lld timed out", R->id);
    return RTM_OK;
}

static int capture_graph(rtm_server *S)
{
    const int grid = bstep_grid<float>();
    if (grid < 1) return fail(RTM_ERR_CUDA, "batched step kernel cannot be configured");
    int dev = 0, sms = 0;
    RTM_CUDA(cudaGetDevice(&dev));
    RTM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int pgrid = 4 * sms;
    RTM_CUDA(cudaStreamBeginCapture(S->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    S->kernel_sampled = S->steps_per_launch >= 2;
    for (int k = 0; k < S->steps_per_launch && e == cudaSuccess; ++k) {
        const bool sample = S->kernel_sampled && k == 1;
        if (sample) e = cudaEventRecordWithFlags(S->kev0, S->stream, cudaEventRecordExternal);
        if (e == cudaSuccess)
            e = launch_bstep<float>(S->d_ix, S->d_mem, S->d_state, S->d_done, grid, k > 0 && !sample, S->stream);
        if (e == cudaSuccess && sample) e = cudaEventRecordWithFlags(S->kev1, S->stream, cudaEventRecordExternal);
        if (e == cudaSuccess) e = launch_bpsi<float>(S->d_ix, S->d_mem, S->d_state, pgrid, !sample, S->stream);
        if (e == cudaSuccess)
            e = launch_bstrip<float>(S->d_ix, S->d_mem, S->d_state, S->d_done, pgrid, 1, S->stream);
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(S->stream, &graph);
    if (e != cudaSuccess || ec != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return fail(RTM_ERR_CUDA, "batch graph capture: %s",
                    cudaGetErrorString(e != cudaSuccess ? e : ec));
    }
    const cudaError_t ei = cudaGraphInstantiate(&S->gexec, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) {
        S->gexec = nullptr;
        return fail(RTM_ERR_CUDA, "batch graph instantiate: %s", cudaGetErrorString(ei));
    }
    return RTM_OK;
}

static void decoder_loop(rtm_server *S)
{
    for (;;) {
        ServeRequest *R = nullptr;
        {
            std::unique_lock<std::mutex> lock(S->dmu);
            S->dcv.wait(lock, [&] { return S->stopping || !S->to_decode.empty(); });
            if (S->stopping && S->to_decode.empty()) return;
            R = S->to_decode.front();
            S->to_decode.pop_front();
        }
        R->seis.resize((size_t)R->p.rec_count * R->p.nt);
        const int st = rtm_zfp_decode_float2d(R->zfp.data(), R->zfp.size(), (double)R->zfp_tol, R->p.rec_count,
                                              R->p.nt, R->seis.data());
        std::vector<unsigned char>().swap(R->zfp);
        R->ready.store(st == RTM_OK ? 1 : -1);
    }
}

// Hands a finished request to the caller and frees it.
static int take_done(rtm_server *S, std::map<long long, ServeRequest *>::iterator it,
                     long long *request_id, float *image, float *self_image, double *times)
{
    ServeRequest *R = it->second;
    if (request_id) *request_id = R->id;
    if (image) memcpy(image, R->img.data(), R->img.size() * sizeof(float));
    if (self_image) memcpy(self_image, R->slf.data(), R->slf.size() * sizeof(float));
    if (times) { times[0] = R->t_submit; times[1] = R->t_admit; times[2] = R->t_done; }
    S->done.erase(it);
    delete R;
    return RTM_OK;
}

// Device resources, graph and decoder threads of a new server (rtm_server_create).
static int server_init(rtm_server *S, long long hbm_budget_bytes)
{
    if (hbm_budget_bytes <= 0) {
        size_t fr = 0, tot = 0;
        RTM_CUDA(cudaMemGetInfo(&fr, &tot));
        hbm_budget_bytes = (long long)(0.8 * (double)fr);
    }
    S->budget = hbm_budget_bytes;
    RTM_CUDA(cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking));
    RTM_CUDA(cudaStreamCreateWithFlags(&S->up, cudaStreamNonBlocking));
    RTM_CUDA(cudaEventCreateWithFlags(&S->up_ev, cudaEventDisableTiming));
    RTM_CUDA(cudaMalloc(&S->d_ix, sizeof(BatchIndex)));
    RTM_CUDA(cudaMalloc(&S->d_mem, sizeof(BMember<float>) * kMaxMembers));
    RTM_CUDA(cudaMalloc(&S->d_state, sizeof(int2) * kMaxMembers));
    RTM_CUDA(cudaMalloc(&S->d_done, kBatchDoneWords * sizeof(unsigned)));
    RTM_CUDA(cudaMallocHost(&S->h_state, sizeof(int2) * kMaxMembers));
    RTM_CUDA(cudaMemsetAsync(S->d_state, 0, sizeof(int2) * kMaxMembers, S->stream));
    RTM_CUDA(cudaMemsetAsync(S->d_done, 0, kBatchDoneWords * sizeof(unsigned), S->stream));
    RTM_CUDA(cudaEventCreate(&S->ev0));
    RTM_CUDA(cudaEventCreate(&S->ev1));
    RTM_CUDA(cudaEventCreate(&S->kev0));
    RTM_CUDA(cudaEventCreate(&S->kev1));
    S->mem.resize(kMaxMembers);
    S->slot_plan.assign(S->max_members, nullptr);
    S->slot_req.assign(S->max_members, nullptr);
    memset(&S->ix, 0, sizeof S->ix);
    rebuild_index(S);
    RTM_CUDA(cudaMemcpyAsync(S->d_ix, &S->ix, sizeof S->ix, cudaMemcpyHostToDevice, S->stream));
    RTM_TRY(capture_graph(S));
    RTM_CUDA(cudaStreamSynchronize(S->stream));
    const unsigned hw = std::max(2u, std::thread::hardware_concurrency());
    const int nthreads = (int)std::min(8u, hw / 2);
    for (int k = 0; k < nthreads; ++k) S->decoders.emplace_back(decoder_loop, S);
    return RTM_OK;
}

// ---- batched tile width per grid shape ---------------------------------------------------
// rtm_autotune_batched's choices (16 or 32 columns), keyed like the single-migration tuner's.
static std::map<TuneKey, int> g_tuned_batch;   // guarded by g_tune_mutex

// Tile width of a batched member: the request's tile_x when it is one the batched kernel has
// (16, 32), else the tuned width of its grid shape, else 32.
static int batched_tile_x(const rtm_params &p)
{
    if (p.tile_x == kBatchTileX || p.tile_x == kBatchTileX / 2) return p.tile_x;
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    auto it = g_tuned_batch.find(tune_key(p));
    return it != g_tuned_batch.end() ? it->second : kBatchTileX;
}

// rtm_server_submit; with `zfp`, the seismogram comes later from a decoder thread.
static int submit_request(rtm_server *S, const rtm_params *p, const float *velocity, const float *wavelet,
                          const float *seismogram, bool zfp, long long *request_id)
{
    if (!S || !p || !velocity) return fail(RTM_ERR_INVALID, "null argument");
    RTM_TRY(check_params(*p));
    if (p->compute != RTM_COMPUTE_FP32) return fail(RTM_ERR_INVALID, "the server runs FP32 migrations");
    if (p->n_wavelet > 0 && !wavelet) return fail(RTM_ERR_INVALID, "null wavelet");
    if (p->rec_count > 0 && !seismogram && !zfp) return fail(RTM_ERR_INVALID, "null seismogram");
    rtm_params q = *p;
    q.tile_x = batched_tile_x(*p);
    const long long bytes = (long long)make_layout(q, make_geom(q, true)).total;
    if (bytes > S->budget) return fail(RTM_ERR_NOMEM, "request needs %lld bytes, budget %lld", bytes, S->budget);
    auto *R = new ServeRequest();
    R->id = S->next_id++;
    R->p = *p;
    R->p.tile_x = q.tile_x;              // the member's tile width in the batched kernel
    const size_t nv = (size_t)(p->th_left + p->nx + p->th_right) * (p->th_up + p->nz + p->th_down);
    R->vel.assign(velocity, velocity + nv);
    if (p->n_wavelet > 0) R->wav.assign(wavelet, wavelet + p->n_wavelet);
    if (p->rec_count > 0 && seismogram) R->seis.assign(seismogram, seismogram + (size_t)p->rec_count * p->nt);
    R->bytes = bytes;
    R->t_submit = now_s();
    S->queue.push_back(R);
    if (request_id) *request_id = R->id;
    return RTM_OK;
}

}  // namespace rtm

extern "C" {

int rtm_server_create(long long hbm_budget_bytes, int max_members, int steps_per_launch,
                      rtm_server **out)
{
    if (!out) return fail(RTM_ERR_INVALID, "null argument");
    if (max_members < 1 || max_members > kMaxMembers)
        return fail(RTM_ERR_INVALID, "max_members must be in [1, %d]", kMaxMembers);
    if (steps_per_launch < 1 || steps_per_launch > 256)
        return fail(RTM_ERR_INVALID, "steps_per_launch must be in [1, 256]");
    rtm_server *S = new rtm_server();
    S->max_members = max_members;
    S->steps_per_launch = steps_per_launch;
    const int st = server_init(S, hbm_budget_bytes);
    if (st != RTM_OK) {
        rtm_server_destroy(S);            // releases what was created before the failure
        return st;
    }
    *out = S;
    return RTM_OK;
}

int rtm_server_destroy(rtm_server *S)
{
    if (!S) return RTM_OK;
    {
        std::lock_guard<std::mutex> lock(S->dmu);
        S->stopping = true;
    }
    S->dcv.notify_all();
    for (auto &t : S->decoders) t.join();
    if (S->up) cudaStreamSynchronize(S->up);
    if (S->stream) cudaStreamSynchronize(S->stream);
    for (rtm_plan *P : S->slot_plan) if (P) plan_free(P);
    for (rtm_plan *P : S->idle) plan_free(P);
    for (auto *R : S->slot_req) delete R;
    for (auto *R : S->queue) delete R;
    for (auto &kv : S->done) delete kv.second;
    if (S->gexec) cudaGraphExecDestroy(S->gexec);
    cudaFree(S->d_ix); cudaFree(S->d_mem); cudaFree(S->d_state); cudaFree(S->d_done);
    if (S->h_state) cudaFreeHost(S->h_state);
    for (cudaEvent_t e : {S->ev0, S->ev1, S->kev0, S->kev1, S->up_ev})
        if (e) cudaEventDestroy(e);
    if (S->up) cudaStreamDestroy(S->up);
    if (S->stream) cudaStreamDestroy(S->stream);
    delete S;
    return RTM_OK;
}

int rtm_server_submit(rtm_server *S, const rtm_params *p, const float *velocity, const float *wavelet,
                      const float *seismogram, long long *request_id)
{
    return submit_request(S, p, velocity, wavelet, seismogram, false, request_id);
}

// As rtm_server_submit, with the seismogram as a ZFP fixed-accuracy stream (what
// zfp2d_lossyCompression writes, tolerance `tol`): a host decoder thread decodes it while
// the GPU steps; the request is admitted once decoded.
int rtm_server_submit_zfp(rtm_server *S, const rtm_params *p, const float *velocity, const float *wavelet,
                          const void *zfp_stream, size_t zfp_bytes, float tol, long long *request_id)
{
    if (!S || !p || !velocity || (!zfp_stream && zfp_bytes)) return fail(RTM_ERR_INVALID, "null argument");
    long long id = 0;
    RTM_TRY(submit_request(S, p, velocity, wavelet, nullptr, true, &id));
    ServeRequest *R = S->queue.back();
    R->zfp.assign(static_cast<const unsigned char *>(zfp_stream),
                  static_cast<const unsigned char *>(zfp_stream) + zfp_bytes);
    R->zfp_tol = tol;
    R->ready.store(0);
    {
        std::lock_guard<std::mutex> lock(S->dmu);
        S->to_decode.push_back(R);
    }
    S->dcv.notify_one();
    if (request_id) *request_id = id;
    return RTM_OK;
}

// Replays steps_per_launch batched steps of the active members, admits what fits while the
// replay runs (uploads overlap it), activates the admitted members after it, and harvests
// finished members.
int rtm_server_step(rtm_server *S, int *n_active, int *n_queued)
{
    NvtxRange range("rtm server step");
    if (!S) return fail(RTM_ERR_INVALID, "null server");
    int active = 0;
    for (int m = 0; m < S->max_members; ++m) active += S->slot_plan[m] != nullptr;
    active -= (int)S->finished.size();           // members still stepping
    if (active > 0) {
        RTM_CUDA(cudaEventRecord(S->ev0, S->stream));
        RTM_CUDA(cudaGraphLaunch(S->gexec, S->stream));
        RTM_CUDA(cudaEventRecord(S->ev1, S->stream));
        S->launches += 3LL * S->steps_per_launch;
    }
    // the members that finished in the previous replay, harvested while this one runs
    const bool freed = !S->finished.empty();
    for (int m : S->finished) RTM_TRY(harvest(S, m));
    S->finished.clear();
    // admission in arrival order among the requests whose inputs are ready (a request whose
    // seismogram is still being decoded is passed over; one that does not fit blocks the
    // rest), for as long as the replay runs: one request at least, then while the host time
    // spent here stays below the previous replay's duration
    const double t0 = now_s();
    int admitted = 0;
    for (auto it = S->queue.begin(); it != S->queue.end();) {
        if (admitted > 0 && (now_s() - t0) * 1e3 > S->last_replay_ms) break;
        ServeRequest *R = *it;
        const int ready = R->ready.load();
        if (ready == 0) { ++it; continue; }
        if (ready < 0) {
            const long long rid = R->id;
            S->queue.erase(it);
            delete R;
            return fail(RTM_ERR_DECODE, "request %lld: the ZFP seismogram could not be decoded", rid);
        }
        int slot = -1;
        for (int m = 0; m < S->max_members; ++m)
            if (!S->slot_plan[m]) { slot = m; break; }
        if (slot < 0) break;
        bool reusable = false;
        for (rtm_plan *P : S->idle) if (same_params(P->p, R->p)) reusable = true;
        long long idle_bytes = 0;
        for (rtm_plan *P : S->idle) idle_bytes += (long long)P->L.total;
        if (!reusable && S->in_use - idle_bytes + R->bytes > S->budget) break;
        const int st = admit(S, slot, R);
        if (st != RTM_OK) return st;
        it = S->queue.erase(it);
        ++admitted;
    }
    RTM_TRY(activate(S));
    if (active > 0) {
        RTM_CUDA(cudaMemcpyAsync(S->h_state, S->d_state, sizeof(int2) * S->max_members,
                                 cudaMemcpyDeviceToHost, S->stream));
        RTM_CUDA(cudaStreamSynchronize(S->stream));
        float ms = 0.0f;
        RTM_CUDA(cudaEventElapsedTime(&ms, S->ev0, S->ev1));
        S->busy_ms += ms;
        S->last_replay_ms = ms;
        if (S->kernel_sampled) {
            float kms = 0.0f;
            RTM_CUDA(cudaEventElapsedTime(&kms, S->kev0, S->kev1));
            S->kernel_ms_last = kms;
        }
        unsigned flags[2] = {0, 0};
        RTM_CUDA(cudaMemcpy(flags, S->d_done, sizeof flags, cudaMemcpyDeviceToHost));
        if (flags[1]) return fail(RTM_ERR_TIMEOUT, "a batched tile load timed out");
        for (int m = 0; m < S->max_members; ++m)
            if (S->slot_plan[m] && S->h_state[m].x == 3) S->finished.push_back(m);
    }
    // slots freed by this call's harvests leave the work lists before the next replay (an
    // activation above has already rebuilt them)
    if (freed && !admitted) {
        rebuild_index(S);
        RTM_CUDA(cudaMemcpyAsync(S->d_ix, &S->ix, sizeof S->ix, cudaMemcpyHostToDevice, S->stream));
    }
    if (n_active) {
        int a = 0;
        for (int m = 0; m < S->max_members; ++m) a += S->slot_plan[m] != nullptr;
        *n_active = a;
    }
    if (n_queued) *n_queued = (int)S->queue.size();
    return RTM_OK;
}

// Takes one finished request, if any: RTM_BUSY when none is ready.  image / self_image
// (nx x nz, may be NULL) receive the result; times (may be NULL) get the submit, admit and
// finish times in seconds on a monotonic clock.
int rtm_server_poll(rtm_server *S, long long *request_id, float *image, float *self_image,
                    double *times)
{
    if (!S) return fail(RTM_ERR_INVALID, "null server");
    if (S->done.empty()) return RTM_ERR_BUSY;
    return take_done(S, S->done.begin(), request_id, image, self_image, times);
}

// Steps the server until request `request_id` has finished and returns it as
// rtm_server_poll does; requests that finish meanwhile stay queued for rtm_server_poll.
int rtm_server_wait(rtm_server *S, long long request_id, float *image, float *self_image,
                    double *times)
{
    if (!S) return fail(RTM_ERR_INVALID, "null server");
    if (request_id < 1 || request_id >= S->next_id)
        return fail(RTM_ERR_INVALID, "unknown request %lld", request_id);
    for (;;) {
        auto it = S->done.find(request_id);
        if (it != S->done.end()) return take_done(S, it, nullptr, image, self_image, times);
        bool live = false;
        for (const ServeRequest *R : S->queue) live |= R->id == request_id;
        for (const ServeRequest *R : S->slot_req) live |= R && R->id == request_id;
        if (!live) return fail(RTM_ERR_INVALID, "request %lld was already returned", request_id);
        int active = 0;
        RTM_TRY(rtm_server_step(S, &active, nullptr));
        // nothing resident: the request's seismogram is still being decoded
        if (active == 0) std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
}

// Totals since creation: credited cell-updates of finished requests, GPU milliseconds of
// the batched steps, kernel launches, device bytes held.
int rtm_server_stats(const rtm_server *S, long long *cell_updates, double *gpu_ms, long long *launches,
                     long long *bytes_in_use)
{
    if (!S) return fail(RTM_ERR_INVALID, "null server");
    if (cell_updates) *cell_updates = S->cell_updates_done;
    if (gpu_ms) *gpu_ms = S->busy_ms;
    if (launches) *launches = S->launches;
    if (bytes_in_use) *bytes_in_use = S->in_use;
    return RTM_OK;
}

int rtm_server_kernel_ms(const rtm_server *S, double *tile_kernel_ms)
{
    if (!S || !tile_kernel_ms) return fail(RTM_ERR_INVALID, "null argument");
    *tile_kernel_ms = S->kernel_sampled ? S->kernel_ms_last : 0.0;
    return RTM_OK;
}

// Batched tile width for p's grid shape: `members` copies of p (a constant 2000 m/s model,
// zero seismogram; nt rounded to `steps`) migrated through a server with each tile width the
// batched kernel has, timed by the server's CUDA events over the batched steps; the faster
// width is kept for later submissions of that shape (tile_x = 0).
int rtm_autotune_batched(const rtm_params *p, int members, int steps, int *best_tile_x,
                         float *best_ms_per_step)
{
    NvtxRange range("rtm autotune batched");
    if (!p) return fail(RTM_ERR_INVALID, "null argument");
    RTM_TRY(check_params(*p));
    if (p->compute != RTM_COMPUTE_FP32) return fail(RTM_ERR_INVALID, "the server runs FP32 migrations");
    if (members < 1 || members > kMaxMembers) return fail(RTM_ERR_INVALID, "members must be in [1, %d]", kMaxMembers);
    if (steps < 1) return fail(RTM_ERR_INVALID, "steps must be >= 1");
    rtm_params q = *p;
    q.nt = (steps + q.time_slices - 1) / q.time_slices * q.time_slices;
    const size_t nv = (size_t)(q.th_left + q.nx + q.th_right) * (q.th_up + q.nz + q.th_down);
    std::vector<float> vel(nv, 2000.0f), wav((size_t)std::max(q.n_wavelet, 1), 0.0f);
    for (size_t k = 0; k < wav.size(); ++k) wav[k] = (float)(k % 7) * 0.1f;
    std::vector<float> seis((size_t)std::max(q.rec_count, 1) * q.nt, 0.0f);
    const int cands[2] = {kBatchTileX, kBatchTileX / 2};
    int best = -1;
    float best_ms = 0.0f;
    for (int tx : cands) {
        q.tile_x = tx;
        rtm_server *S = nullptr;
        RTM_TRY(rtm_server_create(0, members, 16, &S));
        int st = RTM_OK;
        for (int m = 0; m < members && st == RTM_OK; ++m) {
            long long id = 0;
            st = rtm_server_submit(S, &q, vel.data(), wav.data(), seis.data(), &id);
        }
        long long polled = 0;
        while (st == RTM_OK && polled < members) {
            int active = 0, queued = 0;
            st = rtm_server_step(S, &active, &queued);
            long long id = 0;
            while (st == RTM_OK && rtm_server_poll(S, &id, nullptr, nullptr, nullptr) == RTM_OK) ++polled;
            if (st == RTM_OK && active == 0 && queued == 0 && polled < members)
                st = fail(RTM_ERR_STATE, "batched autotune: requests neither resident nor queued");
        }
        double ms = 0.0;
        if (st == RTM_OK) st = rtm_server_stats(S, nullptr, &ms, nullptr, nullptr);
        rtm_server_destroy(S);
        if (st != RTM_OK) return st;
        const float per = (float)(ms / (2.0 * q.nt + 1.0));      // per batched step of the batch
        if (best < 0 || per < best_ms) { best = tx; best_ms = per; }
    }
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        g_tuned_batch[tune_key(*p)] = best;
    }
    if (best_tile_x) *best_tile_x = best;
    if (best_ms_per_step) *best_ms_per_step = best_ms;
    return RTM_OK;
}

}  // extern "C"
