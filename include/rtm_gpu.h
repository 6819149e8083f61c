/*
 * rtm_gpu.h -- C ABI of the GB300 (sm_103a) engine for 2-D isotropic acoustic
 * reverse-time migration.  Drop-in for the migration path of rtmUq2D.
 *
 * Plain C types only: sizes as ints, host arrays as float*, device arrays as void*
 * (CUDA device pointers), streams as void* (cudaStream_t).  Every entry point returns an
 * rtm_status code; none calls exit().
 *
 * Layout convention shared with the reference: 2-D arrays are x-major with z
 * contiguous, element (x, z) at x*dimZ + z, where dimX = th_left + nx + th_right and
 * dimZ = th_up + nz + th_down (SRC/stencilDFM.c:23).  Images are nx x nz, (x, z) at
 * x*nz + z (SRC/image_conditions.c:28).  Seismograms are rec_count x nt, (irec, t) at
 * irec*nt + t (SRC/backward_modeling.c:280).
 */
#ifndef RTM_GPU_H
#define RTM_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------ */
typedef enum rtm_status {
    RTM_OK = 0,
    RTM_ERR_INVALID = 1,      /* bad argument or unsupported configuration            */
    RTM_ERR_CUDA = 2,         /* a CUDA runtime/driver call failed                    */
    RTM_ERR_NOMEM = 3,        /* device allocation failed or admission refused        */
    RTM_ERR_STATE = 4,        /* call out of order (e.g. adjoint before forward)      */
    RTM_ERR_TIMEOUT = 5,      /* a bounded device-side wait gave up (kernel flag);
                                 the results and the device state of the plan, server or
                                 static array are then undefined: destroy and recreate it */
    RTM_ERR_IO = 6,           /* file missing, short read or write                    */
    RTM_ERR_DECODE = 7,       /* ZFP stream could not be decoded                      */
    RTM_ERR_BUSY = 8          /* serving queue full / result not ready                */
} rtm_status;

/* ---- configuration ------------------------------------------------------------------ */
enum rtm_storage {            /* how the backward pass gets the source wavefield      */
    RTM_STORE_SNAPSHOT = 0,   /* interior snapshot every time_slices steps (the        */
                              /* reference's TEMPORARY_FILES contents, kept in HBM)    */
    RTM_STORE_RING = 1        /* 4-cell boundary ring every step + reverse-time        */
                              /* reconstruction of the source field                    */
};
enum rtm_precision {          /* element type of stored rings / snapshots             */
    RTM_PREC_FP32 = 0,
    RTM_PREC_BF16 = 1,        /* with a per-step, per-tile max-abs scale               */
    RTM_PREC_FP16 = 2
};
enum rtm_compute {            /* wavefield arithmetic                                  */
    RTM_COMPUTE_FP32 = 0,     /* the reference's precision                             */
    RTM_COMPUTE_FP64 = 1      /* same scheme in double: the error yardstick            */
};

/*
 * Run-time form of SRC/fixed_parameters.h (plus TIME_SLICES from forward_modeling.h:4).
 * The first 17 fields mirror the reference's constants one for one:
 *   nx, nz            Nx, Nz
 *   th_*              thicknessLeft/Right/Up/Down
 *   dx, dt            spacingGrid, sampling
 *   nt                numberOfTimeStep
 *   n_wavelet         sampligWavelet
 *   shot_x, shot_z    shot[0], shot[1] as passed to isotropicAcousticModeling
 *   rec_*             firstLocationReceiver, spacingReceiver, numberOfReceivers,
 *                     depthReceiver
 *   time_slices       TIME_SLICES (imaging / snapshot interval)
 */
typedef struct rtm_params {
    int nx, nz;
    int th_left, th_right, th_up, th_down;
    float dx, dt;
    int nt, n_wavelet;
    int shot_x, shot_z;
    int rec_first, rec_spacing, rec_count, rec_depth;
    int time_slices;
    int storage;               /* enum rtm_storage                                    */
    int precision;             /* enum rtm_precision (stored source wavefield)        */
    int compute;               /* enum rtm_compute                                    */
    int tile_x;                /* x columns per CTA tile: 0 = autotuned default        */
    int reserved[3];
} rtm_params;

/* Fills *p with the engine's defaults for the fields after time_slices. */
void rtm_params_defaults(rtm_params *p);
/* RTM_OK if the engine supports *p (checks sizes, CPML >= 12 cells, positions inside
 * the grid, nt multiple of time_slices, shot inside the reconstruction region for
 * RTM_STORE_RING). */
int rtm_params_check(const rtm_params *p);
/* Device bytes one migration of *p holds (admission by HBM footprint). */
long long rtm_footprint_bytes(const rtm_params *p);

const char *rtm_status_string(int status);
const char *rtm_last_error(void);     /* detail of the last failure on this thread */
int rtm_device_info(char *name, int name_len, int *sm_count, long long *hbm_bytes);

/* ---- reference-shaped entry points (host buffers) ------------------------------------ */

/* Replaces isotropicAcousticModeling(int simId, int *shot, float *velocity,
 * float *wavelet) -- SRC/forward_modeling.h:11, forward_modeling.c:12-159.
 * velocity: padded dimX x dimZ model (what rtm_iso2d.c:85 passes).  The source
 * wavefield (rings or snapshots) stays in device memory keyed by sim_id, instead of
 * ./TEMPORARY_FILES/sourceWavefield_<simId>.bin, until rtm_adjoint_modeling consumes it. */
int rtm_forward_modeling(const rtm_params *p, int sim_id, const int *shot,
                         const float *velocity, const float *wavelet);

/* Replaces int adjointModeling(int simId, int *shot, float *velocity, float *wavelet,
 * float *seismogram, float *imageCondition, float *selfImageCondition) --
 * SRC/backward_modeling.h:11, backward_modeling.c:12-165.  Accumulates into image and
 * self_image (nx x nz).  Frees the sim_id state.  Returns RTM_OK (the reference
 * returns 1 whatever happens; rtm_dropin.c keeps that). */
int rtm_adjoint_modeling(const rtm_params *p, int sim_id, const int *shot,
                         const float *velocity, const float *wavelet,
                         const float *seismogram, float *image, float *self_image);

/* ---- shot stack on the device ---------------------------------------------------------------
 * The stacking of SRC/rtm_iso2d.c:108-165 without its host round trips: each shot's image and
 * self image are added to float32 stacks (nx x nz) in device memory where the adjoint pass
 * leaves them, in shot order and in the reference's arithmetic (the shot's image rounded to
 * float, then a float sum: rtm_iso2d.c:121-126), and the final stack and its Laplacian
 * (laplacian_filter2D, math_functions.c:9-27) are computed on the device and come back to the
 * host in one copy.  The reference sums per-shot temporary files on the host instead. */
typedef struct rtm_stack rtm_stack;
int rtm_stack_create(const rtm_params *p, rtm_stack **stack);   /* zeroed stacks of p's nx x nz */
int rtm_stack_destroy(rtm_stack *stack);
/* Sets both stacks from host arrays (NULL: zeros), e.g. when resuming from a checkpoint. */
int rtm_stack_load(rtm_stack *stack, const float *image_stack, const float *self_stack);
/* rtm_adjoint_modeling with the shot's image and self image added to the device stacks
 * instead of to host arrays; consumes the sim_id state of rtm_forward_modeling. */
int rtm_adjoint_modeling_stacked(const rtm_params *p, int sim_id, const int *shot,
                                 const float *seismogram, rtm_stack *stack);
/* The running image and self-image stacks to the host (one copy), e.g. for a checkpoint. */
int rtm_stack_read_raw(rtm_stack *stack, float *image_stack, float *self_stack);
/* The stacked image -- the image stack, or with normalize_by_self the image stack divided by
 * the self-image stack (the branch rtm_iso2d.c:150-156 leaves commented out), where a pixel
 * whose self-image stack is 0 (no source energy reached it) is 0 rather than the reference's
 * 0/0 or x/0 -- and its Laplacian, computed on the device, to the host in one copy.
 * RTM_ERR_TIMEOUT if a stacked shot's kernels reported a timed-out wait. */
int rtm_stack_finish(rtm_stack *stack, int normalize_by_self, float *stacked, float *laplacian);
/* Device-to-host copies (and bytes) the stack has made since its creation. */
int rtm_stack_transfers(const rtm_stack *stack, long long *d2h_copies, long long *d2h_bytes);

/* Forward + adjoint of one shot in one call (rtm_iso2d.c:85-93 without the decode). */
int rtm_migrate_shot(const rtm_params *p, const float *velocity, const float *wavelet,
                     const float *seismogram, float *image, float *self_image);
/* The same with the seismogram as the ZFP fixed-accuracy stream the reference reads
 * (rtm_iso2d.c:85-93 with its zfp2d_lossyDecompression, compression_tools.c:78-135): a host
 * thread decodes it (rtm_zfp_decode_float2d) while the forward pass runs on the GPU; the
 * adjoint pass starts once both are done.  RTM_ERR_DECODE for a stream that ends early. */
int rtm_migrate_shot_zfp(const rtm_params *p, const float *velocity, const float *wavelet,
                         const void *zfp_stream, size_t zfp_bytes, float tol, float *image,
                         float *self_image);

/* Forward modelling with trace recording: seismogram[irec*nt + t] = u at the receiver
 * cells after step t's source injection.  (Not in the reference, whose
 * forward_modeling.c:92 computes z_receiver but never records; used to make the
 * observed data that the adjoint pass consumes.) */
int rtm_model_seismogram(const rtm_params *p, const float *velocity, const float *wavelet,
                         float *seismogram);

/* One leapfrog step on host buffers -- replaces iso_acoustic_wave_equation(float *pond,
 * float *waveField2, float *waveField3), SRC/stencilDFM.h:15.  wave3 is overwritten. */
int rtm_iso_acoustic_wave_equation(const rtm_params *p, const float *pond, const float *wave2,
                                   float *wave3);

/* One CPML update on host buffers -- replaces aiso_attenuation_cpml(...),
 * SRC/absorbingBoundaryCondition.h:29, argument order kept; psi/xi strips in the
 * reference's layouts and updated in place. */
int rtm_aiso_attenuation_cpml(const rtm_params *p, const float *wave1, float *wave2,
                              const float *coef,
                              const float *a_left, const float *b_left,
                              const float *a_right, const float *b_right,
                              const float *a_top, const float *b_top,
                              const float *a_bottom, const float *b_bottom,
                              float *psi_left, float *psi_right, float *psi_top,
                              float *psi_bottom, float *xi_left, float *xi_right,
                              float *xi_top, float *xi_bottom);

/* Host-side set-up, same arithmetic as the reference:
 *   attenuation_profile_cpml  SRC/absorbingBoundaryCondition.h:27
 *   extend_matrix             SRC/generic_functions.h:5
 * laplacian_filter2D (SRC/math_functions.h:15) runs on the GPU. */
void rtm_attenuation_profile_cpml(const rtm_params *p, float *a_left, float *a_right,
                                  float *a_top, float *a_bottom, float *b_left,
                                  float *b_right, float *b_top, float *b_bottom);
void rtm_extend_matrix(const rtm_params *p, float *extended, const float *model);
int rtm_laplacian_filter2D(const rtm_params *p, float *lp, const float *image);

/* normalized_cross_correlation(img, self, S, R) -- SRC/image_conditions.h:6: host
 * buffers, padded S and R, nx x nz images accumulated. */
int rtm_normalized_cross_correlation(const rtm_params *p, float *image, float *self_image,
                                     const float *source, const float *receiver);

/* ---- tile-width autotuning ---------------------------------------------------------------
 * Times `steps` forward steps of *p's grid shape for every tile width the step kernel
 * supports (8, 16, 32 columns: 4, 8, 16 warps per CTA; FP64 up to 16) and remembers the
 * fastest for that shape (grid, CPML, storage, precision, compute): every plan created
 * afterwards with tile_x = 0 for that shape uses it.  Returns the choice and its time per
 * step.  Process-wide, thread-safe.  No counterpart in the reference. */
int rtm_autotune(const rtm_params *p, int steps, int *best_tile_x, float *ms_per_step);

/* ---- device-resident plan (inputs already in HBM) ------------------------------------ */
typedef struct rtm_plan rtm_plan;

int rtm_plan_create(const rtm_params *p, rtm_plan **plan);
int rtm_plan_destroy(rtm_plan *plan);
int rtm_plan_set_stream(rtm_plan *plan, void *stream);
/* velocity/wavelet/seismogram/image pointers below are DEVICE pointers (float32,
 * reference layouts).  image/self_image receive (not accumulate) the nx x nz result. */
int rtm_plan_forward(rtm_plan *plan, const void *d_velocity, const void *d_wavelet,
                     void *d_seismogram_out);
int rtm_plan_adjoint(rtm_plan *plan, const void *d_seismogram, void *d_image,
                     void *d_self_image);
/* Device-side wavefield access for tests: which = 0 source field (u_nt after the
 * forward pass), 1 = its predecessor, 2 = receiver field.  Copies dimX x dimZ values of
 * the plan's compute type to a device buffer. */
int rtm_plan_read_field(rtm_plan *plan, int which, void *d_out);
/* image (which = 0) or self image (which = 1), nx x nz, float or double, to a device
 * buffer; valid after rtm_plan_adjoint. */
int rtm_plan_read_image(rtm_plan *plan, int which, int as_double, void *d_out);
/* Captures the source wavefield as the next rtm_plan_adjoint holds it at forward times
 * times[0..count) (0 <= t <= nt): u_nt and u_{nt-1} are the forward pass's last fields, u_t for
 * t <= nt-2 the boundary-ring reconstruction (RTM_STORE_RING only).  d_out: count dimX x dimZ
 * fields (x-major, compute type), written during the adjoint pass.  count = 0 clears.  No
 * counterpart in the reference; used to measure the reconstruction's error per storage
 * precision.  Time loops run without CUDA graphs while captures are set. */
int rtm_plan_capture_source(rtm_plan *plan, int count, const int *times, void *d_out);
/* Waits for the plan's stream and reports a device-side failure flag. */
int rtm_plan_sync(rtm_plan *plan);
/* Number of kernels the plan launched since creation (launch accounting). */
long long rtm_plan_launch_count(const rtm_plan *plan);
/* Device bytes the plan holds. */
long long rtm_plan_bytes(const rtm_plan *plan);
/* Sampled kernel timing: with every > 0, each step whose index is a multiple of `every`
 * brackets its fused step kernel with CUDA events on the plan's stream (0 = off).
 * _read returns the summed milliseconds and launch counts (forward, backward) since the
 * last call and resets them. */
int rtm_plan_profile(rtm_plan *plan, int every);
int rtm_plan_profile_read(rtm_plan *plan, double *fwd_ms, int *fwd_n, double *bwd_ms, int *bwd_n);

/* Frees the plans the host-buffer entry points keep for reuse. */
void rtm_release_cached(void);

/* ---- serving and batching ------------------------------------------------------------------
 * Replaces the reference's MPI fan-out over simulations (SRC/mpi_rtm_iso2d.c:39-51: ranks
 * run rtm_routine for disjoint simulation ranges, with no messages) by many migrations
 * resident on one GPU.  A server admits submitted migrations (any grid, time axis, storage
 * precision; FP32 compute) in arrival order while a member slot is free and their footprint
 * fits the HBM budget, and advances every resident migration one time step per batched step
 * -- one k_bpsi + one k_bstep launch over a (migration, tile) work list, replayed from a
 * CUDA graph.  Finished migrations free their slots for the next admissions (continuous
 * batching).  One thread drives a server. */
typedef struct rtm_server rtm_server;

/* hbm_budget_bytes <= 0: 80 % of the free device memory.  max_members <= 1024. */
int rtm_server_create(long long hbm_budget_bytes, int max_members, int steps_per_launch,
                      rtm_server **server);
int rtm_server_destroy(rtm_server *server);
/* Queues one migration; the host arrays are copied (velocity: padded dimX x dimZ,
 * wavelet: n_wavelet, seismogram: rec_count x nt). */
int rtm_server_submit(rtm_server *server, const rtm_params *p, const float *velocity,
                      const float *wavelet, const float *seismogram, long long *request_id);
/* Admits, runs steps_per_launch batched steps, harvests finished migrations. */
/* As rtm_server_submit, with the seismogram as a ZFP fixed-accuracy stream of rec_count x nt
 * (zfp2d_lossyCompression's output, tolerance tol): a host thread of the server decodes it
 * (rtm_zfp_decode_float2d) while the GPU steps, and the request is admitted once decoded;
 * a stream that fails to decode makes a later rtm_server_step return RTM_ERR_DECODE. */
int rtm_server_submit_zfp(rtm_server *server, const rtm_params *p, const float *velocity,
                          const float *wavelet, const void *zfp_stream, size_t zfp_bytes,
                          float tol, long long *request_id);
int rtm_server_step(rtm_server *server, int *n_active, int *n_queued);
/* One finished migration (RTM_ERR_BUSY if none): image and self image (nx x nz, each may be
 * NULL), times[3] = submit, admission, completion (seconds, monotonic clock; may be NULL). */
int rtm_server_poll(rtm_server *server, long long *request_id, float *image, float *self_image,
                    double *times);
/* Steps the server (rtm_server_step) until request_id has finished and returns it as
 * rtm_server_poll does; other requests finishing meanwhile stay for rtm_server_poll.
 * RTM_ERR_INVALID for an id never issued or already returned. */
int rtm_server_wait(rtm_server *server, long long request_id, float *image, float *self_image,
                    double *times);
int rtm_server_stats(const rtm_server *server, long long *cell_updates, double *gpu_ms,
                     long long *launches, long long *bytes_in_use);
/* CUDA-event time (ms) of the batched tile kernel on the second time step of the last
 * rtm_server_step's graph replay, launched without overlapping the kernels around it
 * (steps_per_launch >= 2; 0 otherwise).  For the kernel's roofline; the step itself
 * advances every active member as usual. */
int rtm_server_kernel_ms(const rtm_server *server, double *tile_kernel_ms);
/* Tile width of the batched kernel (32 or 16 columns) for p's grid shape, chosen by timing
 * `members` copies of p (nt shortened to `steps`) through a server with each width; later
 * submissions of that shape with tile_x = 0 use it (tile_x = 16 or 32 in a request forces a
 * width).  *best_ms_per_step: the batch's GPU time per batched step at that width.  No
 * counterpart in the reference. */
int rtm_autotune_batched(const rtm_params *p, int members, int steps, int *best_tile_x,
                         float *best_ms_per_step);

/* ---- migration without device allocation -------------------------------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc: a host whose
 * device memory is owned by another allocator or held to a fixed budget, or a serving loop
 * that cannot take the implicit device synchronisation of an allocation between requests.
 * Same work and results as rtm_plan_create + rtm_plan_forward + rtm_plan_adjoint (device
 * pointers, reference layouts, image and self image written, not accumulated), but every
 * scratch buffer (wavefields, CPML strips, source-wavefield store, transposed seismogram,
 * FP64 image accumulators) lives in one static 64 MiB device array inside the library; no
 * cudaMalloc, cudaFree or other allocating call is made.  Every GPU that loads the library
 * holds those 64 MiB until the process exits.
 * Limit: a configuration whose footprint (rtm_footprint_bytes) exceeds 64 MiB, or with a
 * CPML thicker than 512 cells, is rejected with RTM_ERR_INVALID and a message naming the
 * bytes needed -- e.g. a 400 x 200 model with nt = 2000 and ring storage fits (~52 MB).
 * The call cannot be made on a stream that is being captured into a CUDA graph: it copies
 * host data, reads its status word back and synchronises the stream.  The first call on each
 * device also looks up the array's device address (cudaGetSymbolAddress, with that device
 * current).
 * All calls on a device share the array and each call rebuilds what it needs, so calls run
 * one at a time: calls that overlap on the GPU (other streams, other host threads) race.
 * stream: cudaStream_t to run on (NULL = default stream).  Every call waits for its work on
 * `stream` to finish before it returns, whether it succeeds or fails. */
int rtm_migrate_shot_static(const rtm_params *p, const void *d_velocity, const void *d_wavelet,
                            const void *d_seismogram, void *d_image, void *d_self_image,
                            void *stream);

/* ---- seismogram decode (host) ---------------------------------------------------------------
 * ZFP 0.5.5 fixed-accuracy stream of a 2-D float field without header, as
 * SRC/compression_tools.c:78-135 (zfp2d_lossyDecompression) reads it: field nx (fastest) x ny
 * over `out` (the reference passes nx = numberOfReceivers, ny = numberOfTimeStep over the flat
 * [irec][t] seismogram), tolerance as given to zfp_stream_set_accuracy (0: lossless bound).
 * Bit-identical to the ZFP library's decode.  RTM_ERR_DECODE if the stream ends early. */
int rtm_zfp_decode_float2d(const void *stream, size_t bytes, double tolerance, int nx, int ny,
                           float *out);
/* The same from a file (the whole file is the stream).  RTM_ERR_IO if it cannot be read. */
int rtm_zfp_decode_file(const char *path, float *array, int nx, int ny, float tolerance);
/* The encoder side (zfp2d_lossyCompression, compression_tools.c:10-71: the seismogram
 * generator's output): the stream zfp_compress writes for the same field and tolerance,
 * byte for byte, flushed to whole 64-bit words.  *bytes = stream length; RTM_ERR_INVALID if
 * `capacity` is too small (rtm_zfp_encode_bound is always enough). */
size_t rtm_zfp_encode_bound(int nx, int ny);
int rtm_zfp_encode_float2d(const float *in, int nx, int ny, double tolerance, void *out,
                           size_t capacity, size_t *bytes);

/* ---- the migration driver (SRC/rtm_iso2d.c:15-177, rtm_routine) ----------------------------
 * File contracts of SRC/fixed_parameters.h: printf patterns with one %d (velocity, stacked,
 * laplacian: the simulation id; seismogram: the shot id, 1-based).  Velocity: raw float32
 * Nx*Nz, [x][z]; wavelet: raw float32, n_wavelet samples; seismogram: ZFP stream (above) of
 * rec_count x nt; outputs: raw float32 Nx*Nz [x][z] -- the stacked image and its 8th-order
 * Laplacian (laplacian_filter2D).  Shots: x = first_shot + (id - 1) * shot_spacing,
 * z = shot_depth, id = 1..n_shots (rtm_iso2d.c:81-83); p->shot_x / shot_z are ignored. */
typedef struct rtm_survey {
    const char *velocity_file;      /* velocityFile */
    const char *wavelet_file;       /* waveletFile */
    const char *seismogram_file;    /* seismogramFile */
    const char *stacked_file;       /* stackedFile */
    const char *laplacian_file;     /* stackedLaplacianFile */
    int first_shot;                 /* firstLocationShot */
    int shot_depth;                 /* depthShot */
    int shot_spacing;               /* spacingShot */
    int n_shots;                    /* numberOfShots */
    float zfp_tolerance;            /* zfp_tolerance */
    int normalize_by_self;          /* 1: stack / self-image stack, the whole-survey branch
                                       commented out at rtm_iso2d.c:152 (0: as the reference) */
    const char *checkpoint_file;    /* rtm_routine_run only, NULL = none: a file pattern (%d:
                                       simulation id) holding the stacks after each finished
                                       shot; a later run of the same simulation resumes after
                                       the last shot it holds; removed once the outputs are
                                       written */
} rtm_survey;
/* Runs the whole migration of one simulation: per shot a forward propagation on the GPU,
 * then the adjoint propagation with the shot's seismogram, which host threads decode ahead;
 * the per-shot images and self images stay in memory (no TEMPORARY_FILES) and are stacked in
 * shot order in float32 as the reference stacks them (the image stack divided by the self-image
 * stack when normalize_by_self is set); both output files are written.  RTM_ERR_IO when an
 * input cannot be read or an output written (the reference exits instead). */
int rtm_routine_run(const rtm_params *p, const rtm_survey *survey, int simulation_id);
/* Device-to-host copies (and bytes) the last rtm_routine_run on the calling thread made of its
 * stacks: 1 without a checkpoint file (the final stack with its Laplacian), plus one per shot
 * with one.  RTM_ERR_STATE (and -1s) if no run has finished on this thread. */
int rtm_routine_last_transfers(long long *d2h_copies, long long *d2h_bytes);
/* rtm_routine over several simulations on one GPU (replaces the MPI fan-out of
 * mpi_rtm_iso2d.c:39-51): every (simulation, shot) migration is a request of one batched
 * server (rtm_server_*; budget and member slots as rtm_server_create takes them, 0 = default),
 * so the simulations' shots run resident together; per simulation the same files and outputs
 * as rtm_routine_run, the images summed in shot order.  Each shot's seismogram file is read
 * once and decoded per request on the server's host threads. */
int rtm_routine_batch(const rtm_params *p, const rtm_survey *survey, const int *simulation_ids,
                      int n_simulations, long long hbm_budget_bytes, int max_members);

#ifdef __cplusplus
}
#endif
#endif
