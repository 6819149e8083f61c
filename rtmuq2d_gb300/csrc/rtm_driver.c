/*
 * rtm_driver.c -- the migration driver of one simulation, SRC/rtm_iso2d.c:15-177
 * (rtm_routine), over the engine's C ABI.
 *
 * Same inputs, outputs and arithmetic of the stack as the reference: velocity and wavelet
 * read raw (pi_file.c:11-32), edge-replicated into the CPML (extend_matrix), per shot a
 * forward propagation, the shot's ZFP seismogram decoded, an adjoint propagation; images and
 * self images summed over shots in float32 in shot order (rtm_iso2d.c:115-129), optionally
 * the image stack divided by the self-image stack (the whole-survey branch the reference
 * leaves commented out, rtm_iso2d.c:150-156; a pixel with a zero self-image stack is 0), the
 * stack written, its Laplacian (laplacian_filter2D) written.
 * Differences: the stacks stay in device memory (rtm_stack: each shot's image is added where
 * the adjoint pass leaves it, and only the final stack and its Laplacian come back, in one
 * copy) instead of TEMPORARY_FILES round trips (rtm_iso2d.c:95-103, 108-140), the seismograms
 * are decoded ahead on host threads while the GPU migrates earlier shots, errors are returned
 * (RTM_ERR_IO) where the reference exits, and, with a checkpoint file, the stacks are saved
 * after each shot so that a run stopped by a failure resumes after its last finished shot.
 */
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "rtm_gpu.h"

#define RTM_PATH_LEN 4096

static int read_raw(const char *path, float *dst, size_t n)
{
    FILE *f = fopen(path, "rb");
    if (!f) return RTM_ERR_IO;
    const size_t got = fread(dst, sizeof(float), n, f);
    fclose(f);
    return got == n ? RTM_OK : RTM_ERR_IO;
}

static int write_raw(const char *path, const float *src, size_t n)
{
    FILE *f = fopen(path, "wb");
    if (!f) return RTM_ERR_IO;
    const size_t put = fwrite(src, sizeof(float), n, f);
    const int closed = fclose(f);
    return (put == n && closed == 0) ? RTM_OK : RTM_ERR_IO;
}

/* Checkpoint of a simulation's shot stack: "RTMCKPT2", int32 simulation id, nx, nz, n_shots,
 * shots done, a 64-bit key of the run, then the image stack and the self-image stack (float32,
 * nx * nz each).  Written to `path`.tmp and renamed over `path`, so a reader sees a whole file
 * or the previous one.  The key (FNV-1a over the migration parameters, the survey's shot
 * geometry, ZFP tolerance and normalisation, and the input file names of this simulation)
 * keeps a checkpoint of another survey of the same shape from being resumed. */
static const char kCkptMagic[8] = {'R', 'T', 'M', 'C', 'K', 'P', 'T', '2'};

static unsigned long long fnv1a(unsigned long long h, const void *data, size_t n)
{
    const unsigned char *b = (const unsigned char *)data;
    for (size_t i = 0; i < n; ++i) {
        h ^= b[i];
        h *= 1099511628211ull;
    }
    return h;
}

static unsigned long long run_key(const rtm_params *p, const rtm_survey *s, int sim)
{
    rtm_params q = *p;
    q.shot_x = q.shot_z = 0;             /* per shot; the survey's geometry is keyed below */
    unsigned long long h = 14695981039346656037ull;
    h = fnv1a(h, &q, sizeof q);
    const int geo[5] = {s->first_shot, s->shot_depth, s->shot_spacing, s->n_shots, s->normalize_by_self};
    h = fnv1a(h, geo, sizeof geo);
    h = fnv1a(h, &s->zfp_tolerance, sizeof s->zfp_tolerance);
    char path[RTM_PATH_LEN];
    const char *pats[3] = {s->velocity_file, s->wavelet_file, s->seismogram_file};
    for (int k = 0; k < 3; ++k) {
        const int n = snprintf(path, sizeof path, pats[k], sim);
        if (n > 0) h = fnv1a(h, path, (size_t)(n < RTM_PATH_LEN ? n : RTM_PATH_LEN - 1));
        h = fnv1a(h, "|", 1);
    }
    return h;
}

static int ckpt_write(const char *path, int sim, int nx, int nz, int n_shots, int done,
                      unsigned long long key, const float *stack, const float *sstack, size_t n)
{
    char tmp[RTM_PATH_LEN + 8];
    const int len = snprintf(tmp, sizeof tmp, "%s.tmp", path);
    if (len < 0 || len >= (int)sizeof tmp) return RTM_ERR_INVALID;
    FILE *f = fopen(tmp, "wb");
    if (!f) return RTM_ERR_IO;
    const int hdr[5] = {sim, nx, nz, n_shots, done};
    int ok = fwrite(kCkptMagic, 1, 8, f) == 8 && fwrite(hdr, sizeof(int), 5, f) == 5 &&
             fwrite(&key, sizeof key, 1, f) == 1 &&
             fwrite(stack, sizeof(float), n, f) == n && fwrite(sstack, sizeof(float), n, f) == n;
    ok = (fclose(f) == 0) && ok;
    if (!ok || rename(tmp, path) != 0) {
        remove(tmp);
        return RTM_ERR_IO;
    }
    return RTM_OK;
}

/* Shots already stacked by a matching checkpoint (0: none, or one of another run). */
static int ckpt_read(const char *path, int sim, int nx, int nz, int n_shots, unsigned long long key,
                     float *stack, float *sstack, size_t n)
{
    FILE *f = fopen(path, "rb");
    if (!f) return 0;
    char magic[8];
    int hdr[5];
    unsigned long long k = 0;
    int done = 0;
    if (fread(magic, 1, 8, f) == 8 && memcmp(magic, kCkptMagic, 8) == 0 &&
        fread(hdr, sizeof(int), 5, f) == 5 && hdr[0] == sim && hdr[1] == nx && hdr[2] == nz &&
        hdr[3] == n_shots && hdr[4] > 0 && hdr[4] <= n_shots && fread(&k, sizeof k, 1, f) == 1 &&
        k == key && fread(stack, sizeof(float), n, f) == n && fread(sstack, sizeof(float), n, f) == n)
        done = hdr[4];
    fclose(f);
    if (!done) {                          /* not ours: start from zero stacks */
        memset(stack, 0, n * sizeof(float));
        memset(sstack, 0, n * sizeof(float));
    }
    return done;
}

/* rtm_iso2d.c:148-156: the whole-survey branch divides the stack by the self-image stack
 * (commented out in the reference, which keeps the plain stack).  A pixel whose self-image
 * stack is 0 -- no source energy reached it -- is set to 0, where the reference's division
 * would write 0/0 (NaN) or x/0 (inf); rtm_stack_finish applies the same rule on the device. */
static void normalize_stack(float *stack, const float *self_stack, size_t n)
{
    for (size_t i = 0; i < n; ++i) stack[i] = self_stack[i] != 0.0f ? stack[i] / self_stack[i] : 0.0f;
}

/* Device-to-host copies of the last rtm_routine_run on this thread (see rtm_routine_last_transfers). */
static __thread long long t_last_d2h_copies = -1, t_last_d2h_bytes = -1;

int rtm_routine_last_transfers(long long *d2h_copies, long long *d2h_bytes)
{
    if (d2h_copies) *d2h_copies = t_last_d2h_copies;
    if (d2h_bytes) *d2h_bytes = t_last_d2h_bytes;
    return t_last_d2h_copies < 0 ? RTM_ERR_STATE : RTM_OK;
}

static int format_path(char *out, const char *pattern, int id)
{
    if (!pattern) return RTM_ERR_INVALID;
    const int n = snprintf(out, RTM_PATH_LEN, pattern, id);
    return (n < 0 || n >= RTM_PATH_LEN) ? RTM_ERR_INVALID : RTM_OK;
}

/* ---- seismogram decode ahead of the migrations ------------------------------------------
 * A ZFP fixed-accuracy stream decodes serially (no block offsets), at about a hundred MB/s
 * on one host core: longer than a full-size shot takes on the GPU.  A few threads decode
 * the next shots' streams (at most `ahead` beyond the one being migrated) while the GPU
 * migrates the current one; the driver takes them in shot order. */
typedef struct {
    const rtm_params *p;
    const rtm_survey *s;
    int last;               /* last shot id */
    int ahead;              /* shots decoded beyond the one consumed */
    size_t nseis;
    float **buf;            /* per shot id: decoded seismogram (owned until taken) */
    int *st;                /* per shot id: 0 pending, else RTM status + 1 */
    int next;               /* next shot id to decode */
    int consumed;           /* shots taken by the driver */
    int stop;
    pthread_mutex_t mu;
    pthread_cond_t cv;
} decode_ahead;

static void *decode_worker(void *arg)
{
    decode_ahead *d = (decode_ahead *)arg;
    char path[RTM_PATH_LEN];
    pthread_mutex_lock(&d->mu);
    for (;;) {
        while (!d->stop && d->next <= d->last && d->next > d->consumed + d->ahead)
            pthread_cond_wait(&d->cv, &d->mu);
        if (d->stop || d->next > d->last) break;
        const int shot = d->next++;
        pthread_mutex_unlock(&d->mu);
        float *b = (float *)malloc((d->nseis > 0 ? d->nseis : 1) * sizeof(float));
        int st = b ? format_path(path, d->s->seismogram_file, shot) : RTM_ERR_NOMEM;
        if (st == RTM_OK && d->nseis > 0)
            st = rtm_zfp_decode_file(path, b, d->p->rec_count, d->p->nt, d->s->zfp_tolerance);
        pthread_mutex_lock(&d->mu);
        d->buf[shot] = b;
        d->st[shot] = st + 1;
        pthread_cond_broadcast(&d->cv);
    }
    pthread_mutex_unlock(&d->mu);
    return NULL;
}

/* The decoded seismogram of `shot` (the caller frees it), or NULL with *status set. */
static float *decode_take(decode_ahead *d, int shot, int *status)
{
    pthread_mutex_lock(&d->mu);
    while (d->st[shot] == 0) pthread_cond_wait(&d->cv, &d->mu);
    float *b = d->buf[shot];
    d->buf[shot] = NULL;
    *status = d->st[shot] - 1;
    d->consumed = shot;
    pthread_cond_broadcast(&d->cv);
    pthread_mutex_unlock(&d->mu);
    if (*status != RTM_OK) {
        free(b);
        return NULL;
    }
    return b;
}

int rtm_routine_run(const rtm_params *params, const rtm_survey *s, int simulation_id)
{
    if (!params || !s || !s->velocity_file || !s->wavelet_file || !s->seismogram_file ||
        !s->stacked_file || !s->laplacian_file || s->n_shots < 0)
        return RTM_ERR_INVALID;
    rtm_params p = *params;
    p.shot_x = s->first_shot;
    p.shot_z = s->shot_depth;
    int st = rtm_params_check(&p);
    if (st != RTM_OK) return st;

    const size_t nimg = (size_t)p.nx * (size_t)p.nz;
    const size_t next = (size_t)(p.th_left + p.nx + p.th_right) * (size_t)(p.th_up + p.nz + p.th_down);
    const size_t nseis = (size_t)p.rec_count * (size_t)p.nt;
    const size_t nwav = p.n_wavelet > 0 ? (size_t)p.n_wavelet : 1;
    float *model = (float *)calloc(nimg, sizeof(float));
    float *ext = (float *)calloc(next, sizeof(float));
    float *wav = (float *)calloc(nwav, sizeof(float));
    float *seis = NULL;
    float *stack = (float *)calloc(nimg, sizeof(float));
    float *sstack = (float *)calloc(nimg, sizeof(float));
    float *lap = (float *)calloc(nimg, sizeof(float));
    char path[RTM_PATH_LEN], ckpt[RTM_PATH_LEN];
    int first_shot = 1;
    rtm_stack *dstack = NULL;
    unsigned long long ckey = 0;
    decode_ahead dec;
    pthread_t workers[4];
    int nworkers = 0;
    memset(&dec, 0, sizeof dec);
    pthread_mutex_init(&dec.mu, NULL);
    pthread_cond_init(&dec.cv, NULL);
    dec.buf = (float **)calloc((size_t)s->n_shots + 1, sizeof(float *));
    dec.st = (int *)calloc((size_t)s->n_shots + 1, sizeof(int));
    t_last_d2h_copies = t_last_d2h_bytes = -1;
    if (!model || !ext || !wav || !stack || !sstack || !lap || !dec.buf || !dec.st) {
        st = RTM_ERR_NOMEM;
        goto done;
    }
    if ((st = rtm_stack_create(&p, &dstack)) != RTM_OK) goto done;
    if (s->checkpoint_file) {             /* resume after the shots a checkpoint holds */
        if ((st = format_path(ckpt, s->checkpoint_file, simulation_id)) != RTM_OK) goto done;
        ckey = run_key(&p, s, simulation_id);
        first_shot = 1 + ckpt_read(ckpt, simulation_id, p.nx, p.nz, s->n_shots, ckey, stack, sstack, nimg);
        if (first_shot > 1 && (st = rtm_stack_load(dstack, stack, sstack)) != RTM_OK) goto done;
    }
    /* the shots' seismograms decode ahead on up to four host threads */
    dec.p = &p;
    dec.s = s;
    dec.last = s->n_shots;
    dec.nseis = nseis;
    dec.next = first_shot;
    dec.consumed = first_shot - 1;
    dec.ahead = s->n_shots - first_shot + 1 < 4 ? s->n_shots - first_shot + 1 : 4;
    for (int k = 0; k < dec.ahead; ++k)
        if (pthread_create(&workers[nworkers], NULL, decode_worker, &dec) == 0) ++nworkers;
    if (dec.ahead > 0 && nworkers == 0) {
        st = RTM_ERR_NOMEM;
        goto done;
    }
    /* rtm_iso2d.c:70-75 */
    if ((st = format_path(path, s->velocity_file, simulation_id)) != RTM_OK) goto done;
    if ((st = read_raw(path, model, nimg)) != RTM_OK) goto done;
    if (p.n_wavelet > 0 && (st = read_raw(s->wavelet_file, wav, (size_t)p.n_wavelet)) != RTM_OK) goto done;
    rtm_extend_matrix(&p, ext, model);

    /* rtm_iso2d.c:77-104: shots in an arithmetic progression */
    for (int shot_id = first_shot; shot_id <= s->n_shots; ++shot_id) {
        int shot[2];
        shot[0] = s->first_shot + (shot_id - 1) * s->shot_spacing;
        shot[1] = s->shot_depth;
        p.shot_x = shot[0];
        p.shot_z = shot[1];
        if ((st = rtm_forward_modeling(&p, simulation_id, shot, ext, wav)) != RTM_OK) goto done;
        /* decoded meanwhile (or before) by the decode-ahead threads */
        free(seis);
        if (!(seis = decode_take(&dec, shot_id, &st))) goto done;
        /* rtm_iso2d.c:121-126: float sums in shot order, on the device */
        if ((st = rtm_adjoint_modeling_stacked(&p, simulation_id, shot, seis, dstack)) != RTM_OK) goto done;
        if (s->checkpoint_file) {
            if ((st = rtm_stack_read_raw(dstack, stack, sstack)) != RTM_OK) goto done;
            if ((st = ckpt_write(ckpt, simulation_id, p.nx, p.nz, s->n_shots, shot_id, ckey, stack, sstack,
                                 nimg)) != RTM_OK)
                goto done;
        }
    }
    /* the stack (normalised if asked) and its Laplacian, computed on the device: one copy back */
    if ((st = rtm_stack_finish(dstack, s->normalize_by_self, stack, lap)) != RTM_OK) goto done;
    rtm_stack_transfers(dstack, &t_last_d2h_copies, &t_last_d2h_bytes);
    if ((st = format_path(path, s->stacked_file, simulation_id)) != RTM_OK) goto done;
    if ((st = write_raw(path, stack, nimg)) != RTM_OK) goto done;
    if ((st = format_path(path, s->laplacian_file, simulation_id)) != RTM_OK) goto done;
    st = write_raw(path, lap, nimg);
    if (st == RTM_OK && s->checkpoint_file) remove(ckpt);   /* the outputs hold the result */
done:
    if (dstack) rtm_stack_destroy(dstack);
    pthread_mutex_lock(&dec.mu);
    dec.stop = 1;
    pthread_cond_broadcast(&dec.cv);
    pthread_mutex_unlock(&dec.mu);
    for (int k = 0; k < nworkers; ++k) pthread_join(workers[k], NULL);
    if (dec.buf)
        for (int k = 0; k <= s->n_shots; ++k) free(dec.buf[k]);
    free(dec.buf); free(dec.st);
    pthread_cond_destroy(&dec.cv);
    pthread_mutex_destroy(&dec.mu);
    free(model); free(ext); free(wav); free(seis);
    free(stack); free(sstack); free(lap);
    return st;
}

/* Whole file as bytes (a ZFP stream). */
static int read_bytes(const char *path, unsigned char **out, size_t *n)
{
    *out = NULL;
    *n = 0;
    FILE *f = fopen(path, "rb");
    if (!f) return RTM_ERR_IO;
    int st = RTM_ERR_IO;
    if (fseek(f, 0, SEEK_END) == 0) {
        const long len = ftell(f);
        if (len >= 0 && fseek(f, 0, SEEK_SET) == 0) {
            unsigned char *b = (unsigned char *)malloc(len > 0 ? (size_t)len : 1);
            if (!b) st = RTM_ERR_NOMEM;
            else if (fread(b, 1, (size_t)len, f) == (size_t)len) {
                *out = b;
                *n = (size_t)len;
                st = RTM_OK;
            } else {
                free(b);
            }
        }
    }
    fclose(f);
    return st;
}

/*
 * Several simulations' migrations through one batched server: the reference fans
 * rtm_routine(simulation) out over MPI ranks (mpi_rtm_iso2d.c:39-51); here every (simulation,
 * shot) migration is a request of one rtm_server on this GPU, so the UQ realizations and
 * their shots run resident together.  Per simulation the same files and outputs as
 * rtm_routine_run: the shots' images and self images summed in float32 in shot order (an
 * image that finishes early waits for its predecessors), the stack (normalised as
 * rtm_routine_run does it) and its Laplacian written.  Each shot's ZFP
 * stream (keyed by shot id, as the reference keys it) is read once and decoded per request
 * by the server's host threads while the GPU steps.
 */
int rtm_routine_batch(const rtm_params *params, const rtm_survey *s, const int *simulation_ids,
                      int n_simulations, long long hbm_budget_bytes, int max_members)
{
    if (!params || !s || !simulation_ids || n_simulations < 1 || !s->velocity_file || !s->wavelet_file ||
        !s->seismogram_file || !s->stacked_file || !s->laplacian_file || s->n_shots < 0)
        return RTM_ERR_INVALID;
    rtm_params p = *params;
    p.shot_x = s->first_shot;
    p.shot_z = s->shot_depth;
    int st = rtm_params_check(&p);
    if (st != RTM_OK) return st;
    if (max_members < 1 || max_members > 128) max_members = 128;
    const int n_shots = s->n_shots;
    const size_t nimg = (size_t)p.nx * (size_t)p.nz;
    const size_t next = (size_t)(p.th_left + p.nx + p.th_right) * (size_t)(p.th_up + p.nz + p.th_down);
    const size_t nwav = p.n_wavelet > 0 ? (size_t)p.n_wavelet : 1;
    const size_t n_req = (size_t)n_simulations * (size_t)n_shots;
    float *model = (float *)calloc(nimg, sizeof(float));
    float *ext = (float *)calloc(next, sizeof(float));
    float *wav = (float *)calloc(nwav, sizeof(float));
    float *img = (float *)calloc(nimg, sizeof(float));
    float *slf = (float *)calloc(nimg, sizeof(float));
    float *lap = (float *)calloc(nimg, sizeof(float));
    float *stack = (float *)calloc(nimg * (size_t)n_simulations, sizeof(float));
    float *sstack = (float *)calloc(nimg * (size_t)n_simulations, sizeof(float));
    unsigned char **zs = (unsigned char **)calloc(n_shots > 0 ? (size_t)n_shots : 1, sizeof(*zs));
    size_t *zb = (size_t *)calloc(n_shots > 0 ? (size_t)n_shots : 1, sizeof(*zb));
    long long *ids = (long long *)calloc(n_req > 0 ? n_req : 1, sizeof(*ids));
    /* finished, not yet summed: image then self image */
    float **held = (float **)calloc(n_req > 0 ? n_req : 1, sizeof(*held));
    int *next_shot = (int *)calloc((size_t)n_simulations, sizeof(int));
    rtm_server *srv = NULL;
    char path[RTM_PATH_LEN];
    if (!model || !ext || !wav || !img || !slf || !lap || !stack || !sstack || !zs || !zb || !ids || !held ||
        !next_shot) {
        st = RTM_ERR_NOMEM;
        goto done;
    }
    if (p.n_wavelet > 0 && (st = read_raw(s->wavelet_file, wav, (size_t)p.n_wavelet)) != RTM_OK) goto done;
    for (int k = 0; k < n_shots; ++k) {
        if ((st = format_path(path, s->seismogram_file, k + 1)) != RTM_OK) goto done;
        if ((st = read_bytes(path, &zs[k], &zb[k])) != RTM_OK) goto done;
    }
    if ((st = rtm_server_create(hbm_budget_bytes, max_members, 16, &srv)) != RTM_OK) goto done;
    for (int i = 0; i < n_simulations; ++i) {
        if ((st = format_path(path, s->velocity_file, simulation_ids[i])) != RTM_OK) goto done;
        if ((st = read_raw(path, model, nimg)) != RTM_OK) goto done;
        rtm_extend_matrix(&p, ext, model);
        for (int k = 0; k < n_shots; ++k) {
            p.shot_x = s->first_shot + k * s->shot_spacing;
            p.shot_z = s->shot_depth;
            st = rtm_server_submit_zfp(srv, &p, ext, wav, zs[k], zb[k], s->zfp_tolerance,
                                       &ids[(size_t)i * n_shots + k]);
            if (st != RTM_OK) goto done;
        }
    }
    for (size_t finished = 0; finished < n_req;) {
        int active = 0, queued = 0;
        if ((st = rtm_server_step(srv, &active, &queued)) != RTM_OK) goto done;
        for (;;) {
            long long rid = 0;
            st = rtm_server_poll(srv, &rid, img, slf, NULL);
            if (st == RTM_ERR_BUSY) { st = RTM_OK; break; }
            if (st != RTM_OK) goto done;
            size_t r = 0;
            while (r < n_req && ids[r] != rid) ++r;
            if (r == n_req) { st = RTM_ERR_INVALID; goto done; }
            held[r] = (float *)malloc(2 * nimg * sizeof(float));
            if (!held[r]) { st = RTM_ERR_NOMEM; goto done; }
            memcpy(held[r], img, nimg * sizeof(float));
            memcpy(held[r] + nimg, slf, nimg * sizeof(float));
            ++finished;
            /* rtm_iso2d.c:121-126: float sums in shot order */
            const int i = (int)(r / (size_t)n_shots);
            float *stk = stack + (size_t)i * nimg;
            float *sstk = sstack + (size_t)i * nimg;
            while (next_shot[i] < n_shots && held[(size_t)i * n_shots + next_shot[i]]) {
                float *im = held[(size_t)i * n_shots + next_shot[i]];
                for (size_t q = 0; q < nimg; ++q) {
                    stk[q] = stk[q] + im[q];
                    sstk[q] = sstk[q] + im[nimg + q];
                }
                free(im);
                held[(size_t)i * n_shots + next_shot[i]] = NULL;
                ++next_shot[i];
            }
        }
        if (finished < n_req && active == 0 && queued == 0) { st = RTM_ERR_INVALID; goto done; }
    }
    for (int i = 0; i < n_simulations; ++i) {
        float *stk = stack + (size_t)i * nimg;
        if (s->normalize_by_self) normalize_stack(stk, sstack + (size_t)i * nimg, nimg);
        if ((st = format_path(path, s->stacked_file, simulation_ids[i])) != RTM_OK) goto done;
        if ((st = write_raw(path, stk, nimg)) != RTM_OK) goto done;
        if ((st = rtm_laplacian_filter2D(&p, lap, stk)) != RTM_OK) goto done;
        if ((st = format_path(path, s->laplacian_file, simulation_ids[i])) != RTM_OK) goto done;
        if ((st = write_raw(path, lap, nimg)) != RTM_OK) goto done;
    }
done:
    if (srv) rtm_server_destroy(srv);
    if (held) for (size_t r = 0; r < n_req; ++r) free(held[r]);
    if (zs) for (int k = 0; k < n_shots; ++k) free(zs[k]);
    free(model); free(ext); free(wav); free(img); free(slf); free(lap); free(stack); free(sstack);
    free(zs); free(zb); free(ids); free(held); free(next_shot);
    return st;
}
