/*
 * fivonagi.h -- C ABI of the GB300 (sm_103a) FiVoNAGI time-step hot path.
 *
 * One step of the 2-D nonlinear, dissipative acoustics solver:
 *   boundary forcing (app hook) -> y sweep -> x sweep -> CFL max-reduction
 *   -> (step accepted) fractional velocity diffusion, T += dt -> dt update.
 *
 * The reference composes this step out of ~34 kernels and 7 blocking
 * device-to-host copies per step (common/main.cu:310-635). Here one fused
 * kernel launch performs the whole step, the accept/reject decision and the
 * dt update happen on the device, and the host synchronises only when a
 * call returns.
 *
 * Plain C types only: no CUDA or torch types cross this boundary. All calls
 * return an fv_status; none of them exits the process (the reference calls
 * exit() on every error, common/main.cu:365-368, 600-609,
 * common/debug_tools.h:44-55).
 *
 * State layout: three FP32 fields u1 = rho-1, u2 = rho*vx, u3 = rho*vy,
 * each NX*NY, row-major with i (x, axial) fastest: offset = i + j*NX, the
 * reference's layout (apps/na/fv.h:15-17).
 */
#ifndef FIVONAGI_H
#define FIVONAGI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FV_ABI_VERSION 1

/* Status codes. 1, 2, 3, 4 are the reference's simError values
 * (common/data_definitions.h:78-83); the rest are the library's own. */
typedef enum fv_status {
  FV_OK = 0,
  FV_DT_TOO_LARGE = 1,        /* CFL >= CFLMAX on every retry of a step (max_retries) */
  FV_NEGATIVE_EIGENVALUE = 2, /* a Riemann solve met tmp3 < 0 (apps/na/fv.h:102, 290) */
  FV_TRANSONIC = 3,           /* declared by the reference, never raised; reserved */
  FV_COLLECT_OVERFLOW = 4,    /* the collection buffers filled before fv_collect_read (simError 4) */
  FV_TIMEOUT = 5,             /* a bounded device wait ran out */
  FV_CUDA_ERROR = 6,          /* a CUDA runtime call failed; see fv_last_error_string */
  FV_BAD_ARG = 7,             /* invalid argument; see fv_last_error_string */
  FV_NO_DEVICE = 8            /* no usable sm_103 device */
} fv_status;

/* Per-app plugins. The reference selects one app per build through
 * include-guard shadowing of parameters.h / init.h / boundary.h
 * (apps/hifu-beam/driver.cu:40-52); here the app is a runtime choice and
 * each app's boundary hook is a device functor fused into the step kernel. */
typedef enum fv_app {
  FV_APP_HIFU_BEAM = 0,       /* apps/hifu-beam: focused pulsed source, reflecting axis */
  FV_APP_TAYLOR_ANGLE_XY = 1, /* apps/taylor-angle-xy: analytic tanh (Taylor shock) ghosts */
  FV_APP_PLANE_WAVE = 2,      /* oblique sinusoidal plane wave, no-flux y walls */
  FV_APP_FOCUSED_BEAM = 3,    /* focused continuous-wave source, open boundaries */
  FV_APP_PHASED_ARRAY = 4     /* array of continuous-wave elements on the left edge, each
                                 with its own amplitude and phase (fv_set_array_weights),
                                 open boundaries; the adjoint's design variables */
} fv_app;

/* Run-time parameter block. Names follow the reference's parameters.h
 * constants (apps/hifu-beam/parameters.h:12-104,
 * apps/taylor-angle-xy/parameters.h:12-109). Values are double; the solver
 * rounds each to FP32 once, as the reference's `static const DATATYPEV`
 * definitions do at PRECISION=1. */
typedef struct fv_params {
  int32_t app;            /* fv_app */
  int32_t nx, ny;         /* NX, NY: grid cells (any size >= 8; the reference needs powers of 2) */
  int32_t cfl_even_only;  /* 1: CFL max over even flat offsets only, the reference's
                             pairwise reduction stopping at 2 (common/main.cu:503-519) */
  int32_t moving_domain;  /* 1: shift the window once T >= MDT (common/main.cu:109-177) */
  int32_t exact;          /* 1: no FMA contraction (bit-identical to the oracle);
                             0: contracted FMAs (within the FP32 tolerance) */
  int32_t max_retries;    /* consecutive rejected attempts before FV_DT_TOO_LARGE */
  int32_t array_elems;    /* phased array: number of elements (aperture / array_elems cells each) */
  double xmax, ymax;      /* XMAX, YMAX: dx = XMAX/(NX-1), dy = YMAX/(NY-1) (common/main.cu:790-791) */
  double beta;            /* BETA: nonlinearity coefficient */
  double diffdelta;       /* DIFFDELTA: dimensionless dissipation */
  double cflmax;          /* CFLMAX: steps with CFL >= CFLMAX are rejected */
  double cflwhish;        /* CFLWHISH: target CFL for the next dt */
  double dtini;           /* DTINI: dt of the first step */
  double tide;            /* TIDE: T starts at -TIDE */
  double mdvx, mdvy, mdt; /* MDVX, MDVY, MDT: moving-domain velocity and start time */
  /* app block */
  double ampl;            /* AMPL: source amplitude (Mach) */
  double frec;            /* FREC: source frequency (1/lambda) */
  double angle;           /* ISPTHETA (taylor) / propagation angle (plane wave), radians */
  double isp_a;           /* hifu ISPa: source aperture, lambda units */
  double isp_f;           /* hifu ISPF, focused-beam focal distance: in grid points */
  double isp_rhoa;        /* taylor ISPRHOA */
  double isp_c;           /* taylor ISPC */
  double aperture;        /* focused beam, phased array: aperture width, cells */
  double center;          /* focused beam, phased array: aperture centre, j index */
  double ramp_periods;    /* focused beam, phased array: linear amplitude ramp, periods */
} fv_params;

typedef struct fv_run_stats {
  int64_t accepted;       /* accepted steps in the call */
  int64_t rejected;       /* rejected attempts in the call */
  double dt;              /* dt for the next step */
  double T;               /* simulation time */
  double cfl;             /* CFL of the last attempted step */
  int32_t n;              /* total accepted steps since the state was set */
  int32_t status;         /* fv_status of the device run */
  int32_t mdx, mdy;       /* moving-domain offsets MDX, MDY */
} fv_run_stats;

/* Stages for fv_debug_step: the state after each phase of one step. */
typedef enum fv_stage {
  FV_STAGE_BOUNDARY = 0,  /* ghost cells rewritten (the app's boundary hook) */
  FV_STAGE_SWEEP_Y = 1,   /* after getWavesSpeedsCFL_y/step_y/calcLimiters_y/writeLimiters_y */
  FV_STAGE_SWEEP_X = 2,   /* after the x sweep */
  FV_STAGE_SOURCE = 3     /* after the diffusion step (source) */
} fv_stage;

typedef struct fv_handle fv_handle;

/* Library identification and the last error message of the calling thread. */
const char *fv_version(void);
const char *fv_last_error_string(void);

/* Fill *out with the app's reference parameter values.
 * Replaces the compile-time parameters.h of each app
 * (apps/hifu-beam/parameters.h:12-104, apps/taylor-angle-xy/parameters.h:12-109). */
fv_status fv_default_params(int32_t app, fv_params *out);

/* Allocate device state for one simulation on the current CUDA device.
 * Replaces gpu_init (common/data_definitions.h:523-871). */
fv_status fv_create(const fv_params *p, fv_handle **out);

/* Free everything fv_create allocated. Replaces clean_gpu
 * (common/data_definitions.h:415-517). */
fv_status fv_destroy(fv_handle *h);

/* Run the app's initial-value hook (host side, as the reference's init<TTT>,
 * apps/hifu-beam/init.h:16-25, apps/taylor-angle-xy/init.h:19-27), upload
 * it, and reset dt = DTINI, T = -TIDE, n = 0, MDX = MDY = 0
 * (common/main.cu:789-795, 807-815). */
fv_status fv_init_state(fv_handle *h);

/* Copy a state in or out. on_device = 0: host pointers; 1: device pointers
 * on the handle's device. Each pointer addresses NX*NY floats.
 * fv_set_state also resets dt, T, n, MDX, MDY as fv_init_state does. */
fv_status fv_set_state(fv_handle *h, const float *u1, const float *u2,
                       const float *u3, int32_t on_device);
fv_status fv_get_state(fv_handle *h, float *u1, float *u2, float *u3,
                       int32_t on_device);

/* Set or read the scalar time-stepping state (dt, T, n). */
fv_status fv_set_scalars(fv_handle *h, double dt, double T, int32_t n);
fv_status fv_get_stats(fv_handle *h, fv_run_stats *out);

/* Phased array (FV_APP_PHASED_ARRAY): element k drives the left ghost
 * cells of rows [j0 + k*w, j0 + (k+1)*w), w = aperture / array_elems and
 * j0 = center - aperture/2, with u1 = amp[k] * ramp(T) * sin(2 pi FREC T +
 * phase[k]), u2 = u1 (u1 + 1), u3 = 0 -- the focused beam's packet at normal
 * incidence. nelem must equal params.array_elems; host pointers. fv_create
 * starts every element at amplitude AMPL and phase 0. */
fv_status fv_set_array_weights(fv_handle *h, const float *amp, const float *phase, int32_t nelem);

/* ---------------------------------------------------------------- adjoint
 * Discrete adjoint of the step for the phased array's element weights. The
 * reference has none. The loss is the mean of u1^2 over a window of cells
 * and over the states after accepted steps step_first..step_last of an
 * nsteps-step run from rest (T0 = -TIDE); the dt schedule of the forward
 * run is held fixed in the derivative. fv_adjoint_forward runs the forward
 * (adaptive dt, recorded), storing a checkpoint every checkpoint_every
 * steps (0: ceil(sqrt(nsteps))); fv_adjoint_backward returns d loss / d
 * amplitude and d loss / d phase per element. fv_adjoint_replay runs the
 * forward again with other weights on the recorded schedule (for finite
 * differences); a backward pass needs a fv_adjoint_forward after it. Only
 * FV_APP_PHASED_ARRAY without the moving window. */
typedef struct fv_adjoint fv_adjoint;
typedef struct fv_loss_window {
  int32_t i0, j0;         /* first cell (i, j) of the window */
  int32_t ni, nj;         /* window size, cells */
  int64_t step_first;     /* first accepted step (1-based) whose state enters the loss */
  int64_t step_last;      /* last one */
} fv_loss_window;
fv_status fv_adjoint_create(const fv_params *p, const fv_loss_window *w, int64_t nsteps,
                            int32_t checkpoint_every, fv_adjoint **out);
fv_status fv_adjoint_destroy(fv_adjoint *a);
fv_status fv_adjoint_set_stream(fv_adjoint *a, void *cuda_stream);
fv_status fv_adjoint_forward(fv_adjoint *a, const float *amp, const float *phase, double *loss);
fv_status fv_adjoint_backward(fv_adjoint *a, double *grad_amp, double *grad_phase);
fv_status fv_adjoint_replay(fv_adjoint *a, const float *amp, const float *phase, double *loss);
/* The recorded schedule: dt and T (before the step) of each of the nsteps steps. */
fv_status fv_adjoint_schedule(fv_adjoint *a, double *dt, double *T);
/* The state after the last forward or replay (host buffers of NX*NY floats). */
fv_status fv_adjoint_get_state(fv_adjoint *a, float *u1, float *u2, float *u3);

/* Spectral low-pass of the current u1 (the filter the reference sketches in
 * common/filter.h:16-39 and main.cu:672-708 but never runs): a 2-D real FFT
 * (cuFFT, loaded at first use), every coefficient with wavenumber radius
 * sqrt(kx^2 + ky^2) > radius zeroed (kx, ky in index units, ky folded to
 * -NY/2..NY/2), the inverse FFT normalised by NX*NY. Writes NX*NY floats
 * to `out` (host, or device with on_device = 1); the state is unchanged. */
fv_status fv_filter_u1(fv_handle *h, double radius, float *out, int32_t on_device);

/* Headless display: the reference's draw kernel and colour map (apps/
 * hifu-beam/draw_float_cut.h:8-106), rendered into an RGBA8 buffer instead
 * of a GL window. A width x height map of u1 over the cells
 * (i0 + x*zoom, j0 + y*zoom) (NXWLB, NYWLB, NXW/ZOOM, NYW/ZOOM, ZOOM),
 * coloured from u1/(2 plot_scale AMPL) + 0.5, with the reference's guide
 * lines when overlays = 1; with jcut >= 0, a 128-pixel plot of u1 along
 * row jcut under it. Writes width * (height [+ 128]) pixels, row 0 first,
 * to `rgba` (host, or device with on_device = 1). */
typedef struct fv_render_spec {
  int32_t i0, j0;          /* first cell of the view */
  int32_t width, height;   /* map size, pixels */
  int32_t zoom;            /* cells per pixel */
  int32_t jcut;            /* row of the cut plot; -1: none */
  int32_t overlays;        /* 1: dashed cut row and focal column, centre and aperture lines */
  int32_t reserved;
  double plot_scale;       /* PLOTSCALE: full colour range is +-plot_scale*AMPL */
} fv_render_spec;
fv_status fv_render(fv_handle *h, const fv_render_spec *spec, uint8_t *rgba, int32_t on_device);

/* ------------------------------------------------------- data collection
 * On-device collection after every accepted step with T > 0, the
 * reference's dataCollect (apps/hifu-beam/data_collect.h:6-107,
 * apps/taylor-angle-xy/data_collect.h:6-98), read back between frames:
 *  - T and the step's CFL, one entry per step (measure1 rows 0, 1);
 *  - u1 at up to 8 probe cells ("microphones", rows 2-5), in lab
 *    coordinates (i + MDX, j + MDY); 0 while a probe is outside the window;
 *  - the running maximum of u1 along lab row envelope_row (u1max, row 6),
 *    over lab columns 0..envelope_len-1, only where |x_lab/ETA - T| <=
 *    envelope_halfwidth when that is > 0 (ETA = NX/XMAX; the hifu app's
 *    central-peak window is 0.5).
 * The per-step series hold `capacity` steps; a step beyond that stops the
 * run with FV_COLLECT_OVERFLOW, as simError 4 does. fv_collect_read copies
 * the series out (host buffers: T, cfl [capacity], probes [capacity][8],
 * envelope [envelope_len]; any may be NULL), returns the step count and
 * empties the series; the envelope keeps accumulating. A NULL spec turns
 * collection off. Setting the state clears everything. */
typedef struct fv_collect_spec {
  int32_t nprobes;             /* 0..8 */
  int32_t probe_i[8];          /* lab column of each probe */
  int32_t probe_j[8];          /* lab row of each probe */
  int32_t envelope_row;        /* lab row of the u1 envelope; -1: none */
  int32_t envelope_len;        /* lab columns of the envelope */
  int32_t capacity;            /* steps the series hold between reads (>= 1) */
  double envelope_halfwidth;   /* > 0: central-peak window, in units of x/ETA - T */
} fv_collect_spec;
fv_status fv_collect_enable(fv_handle *h, const fv_collect_spec *spec);
fv_status fv_collect_read(fv_handle *h, int32_t *nsteps, float *T, float *cfl, float *probes,
                          float *envelope);

/* Save the current state and time-stepping scalars (dt, T, n, window
 * offsets, retry state) in the handle's one snapshot slot, overwriting it;
 * fv_restore brings them back. Replaces the reference's texCpy/restore
 * pair (common/main.cu:72-107), which keeps the pre-step state to retry a
 * rejected step. fv_restore without a snapshot returns FV_BAD_ARG. */
fv_status fv_snapshot(fv_handle *h);
fv_status fv_restore(fv_handle *h);

/* Use a caller-provided cudaStream_t (passed as void*); NULL = the
 * library's own stream. */
fv_status fv_set_stream(fv_handle *h, void *cuda_stream);

/* Advance by exactly nsteps accepted steps (rejected attempts are retried
 * with the reduced dt and counted). The inner loop of calcFrame
 * (common/main.cu:310-635) without its per-step host synchronisation. */
fv_status fv_run(fv_handle *h, int64_t nsteps, fv_run_stats *out);

/* Advance until T >= t_stop, the calcFrame loop condition `while (T < Tprint)`
 * (common/main.cu:310). */
fv_status fv_run_until(fv_handle *h, double t_stop, fv_run_stats *out);

/* Enqueue nattempts step attempts on the handle's stream and return without
 * synchronising (accepted and rejected attempts both count). For timing
 * loops; pair with fv_sync. */
fv_status fv_launch_attempts(fv_handle *h, int64_t nattempts);
fv_status fv_sync(fv_handle *h, fv_run_stats *out);

/* Step attempts with every attempt's stats read back, pipelined: the
 * per-step host read of the calcFrame loop (common/main.cu:310-635 copies T
 * and n to the host every step) without stopping the GPU for it.
 * fv_steps_async enqueues nattempts attempts (in the same captured graphs
 * as fv_run) and returns without synchronising; at most 64 attempts may be
 * in flight (FV_BAD_ARG beyond). Each attempt's last launch writes its
 * control block to a slot of mapped pinned host memory. fv_step_wait waits
 * for the oldest attempt in flight and returns its stats (accepted 1 or 0,
 * rejected 0 or 1, dt, T, CFL, n) and status, as fv_run does. A run of
 * enqueued attempts has no step budget or stop time; consecutive
 * rejections carry over between its attempts, so max_retries ends a run of
 * rejections with FV_DT_TOO_LARGE, and an attempt enqueued after a failed
 * one does nothing and reports the same status. While attempts are in
 * flight, fv_run, fv_run_until, fv_launch_attempts, fv_time_* and
 * fv_debug_step return FV_BAD_ARG. A caller keeps a block of attempts
 * queued ahead of the one it reads (n a multiple of 32 here):
 *   fv_steps_async(h, 32);
 *   for (k = 0; k < n; ++k) {
 *     if (k % 32 == 0 && k + 32 < n) fv_steps_async(h, 32);
 *     fv_step_wait(h, &st);
 *   } */
fv_status fv_steps_async(fv_handle *h, int32_t nattempts);
fv_status fv_step_wait(fv_handle *h, fv_run_stats *out);

/* Runs nattempts attempts one at a time, without graph capture, with CUDA
 * events on the handle's stream between the attempt's launches, and returns
 * the step kernel's average duration and the whole attempt's, in ms.
 * Synchronises. For roofline measurements of the step kernel alone. No
 * reference counterpart: the reference times nothing on the device. */
fv_status fv_time_attempts(fv_handle *h, int32_t nattempts, float *step_kernel_ms,
                           float *attempt_ms);

/* Enqueues nattempts attempts as fv_launch_attempts does, between two
 * CUDA events on the handle's stream, synchronises, and returns the elapsed
 * device time in ms (the counters cover those attempts, as after
 * fv_launch_attempts; read them with fv_sync). For the autotuner. No
 * reference counterpart. */
fv_status fv_time_run(fv_handle *h, int64_t nattempts, float *ms);

/* Name of the current CUDA device (cudaGetDeviceProperties), NUL-terminated
 * within len bytes; the autotuner's cache key. No reference counterpart. */
fv_status fv_device_name(char *name, int32_t len);

/* Launch shape of the step kernel, for the autotuner: `blocks` persistent
 * CTAs of 4 warps, each warp streaming an even share of the grid's
 * (26-column window, row) work; 0 restores the default (one wave of
 * resident CTAs; at most 8 waves). fv_get_launch reports the current value and
 * how many CTAs fit on the device at once. No reference counterpart: the
 * reference launches one thread per cell (common/main.cu:252-253). */
fv_status fv_set_launch(fv_handle *h, int32_t blocks);
fv_status fv_get_launch(fv_handle *h, int32_t *blocks, int32_t *max_resident);

/* CTA shape of the step kernel, for the autotuner: 0 = 4 warps per CTA,
 * 4 CTAs per SM (the default); 1 = 2 warps, 8 per SM; 2 = 1 warp, 16 per
 * SM; 3 = 1 warp, 18 per SM (built for at most 112 registers a thread);
 * all loading input rows 2 ahead of the row in use; 4 and 5 = shape 0
 * loading 1 and 3 rows ahead (the sweep's prefetch depth).
 * Every warp streams its own share of the grid in every shape, so the
 * results are the same bit for bit; what changes is how many warps an SM
 * holds and how the launch groups them. Applies to the exact-division
 * kernel (FMA division runs shape 0). Setting it restores the default CTA
 * count for the shape (one wave); fv_get_launch then reports the shape's
 * resident CTAs. No reference counterpart. */
fv_status fv_set_cta_shape(fv_handle *h, int32_t shape);
fv_status fv_get_cta_shape(fv_handle *h, int32_t *shape, int32_t *warps_per_cta);

/* Division in the step kernel, for the autotuner. Both give the same
 * results bit for bit (IEEE-equal quotients everywhere):
 *   FV_DIVISION_FMA: FMA-based division, with a fix-up pass that recomputes
 *     the few rows where its operands leave its proven range (subnormal
 *     quotients) with exact division;
 *   FV_DIVISION_EXACT: exact division in the step kernel itself (the
 *     subnormal-proof form only for the quotients that can be subnormal),
 *     with no fix-up work in practice;
 *   FV_DIVISION_DEFAULT: EXACT (the faster at every size measured).
 * No reference counterpart: the reference uses the compiler's division. */
#define FV_DIVISION_DEFAULT (-1)
#define FV_DIVISION_FMA 0
#define FV_DIVISION_EXACT 1
fv_status fv_set_division(fv_handle *h, int32_t mode);
fv_status fv_get_division(fv_handle *h, int32_t *mode);

/* One step of the current state, stopped after `stage`; writes the stage's
 * full grid to u1/u2/u3 (host pointers) and leaves the handle's state,
 * dt, T and n unchanged. For per-phase parity tests. */
fv_status fv_debug_step(fv_handle *h, int32_t stage, float *u1, float *u2,
                        float *u3);

/* ------------------------------------------------------------- batches
 * n independent simulations, each with its own fv_params (app, grid size,
 * physics), dt, T and CFL, stepped together: every launch attempts one step
 * of each simulation that still has steps to take. No reference
 * counterpart: the reference runs one simulation per process and its sweep
 * scripts rebuild and rerun it per parameter point (apps/hifu-beam/run.sh:26-74). */
typedef struct fv_batch fv_batch;

/* All simulations of a batch share `exact`. */
fv_status fv_batch_create(int32_t n, const fv_params *params, fv_batch **out);
fv_status fv_batch_destroy(fv_batch *b);
fv_status fv_batch_set_stream(fv_batch *b, void *cuda_stream);
/* Every simulation's init hook; dt = DTINI, T = -TIDE, n = 0 for all. */
fv_status fv_batch_init_state(fv_batch *b);
/* State of simulation k (its own NX*NY floats per field); set_state also
 * resets that simulation's dt, T, n. */
fv_status fv_batch_set_state(fv_batch *b, int32_t k, const float *u1, const float *u2,
                             const float *u3, int32_t on_device);
fv_status fv_batch_get_state(fv_batch *b, int32_t k, float *u1, float *u2, float *u3,
                             int32_t on_device);
/* Every simulation takes exactly nsteps accepted steps; out[k] (n entries,
 * optional) receives each one's stats. */
fv_status fv_batch_run(fv_batch *b, int64_t nsteps, fv_run_stats *out);
/* Enqueue nattempts attempts of every simulation without synchronising;
 * fv_batch_sync waits and reports. */
fv_status fv_batch_launch_attempts(fv_batch *b, int64_t nattempts);
fv_status fv_batch_sync(fv_batch *b, fv_run_stats *out);
/* fv_batch_launch_attempts between two CUDA events on the batch's stream;
 * synchronises and returns the elapsed device time in ms. */
fv_status fv_batch_time_run(fv_batch *b, int64_t nattempts, float *ms);
/* CTAs of the batch launch, each warp streaming an even share of the
 * concatenated (simulation, window, row) work (0 = default: eight waves of
 * resident CTAs, at least 32 rows per warp). */
fv_status fv_batch_set_launch(fv_batch *b, int32_t blocks);
fv_status fv_batch_get_launch(fv_batch *b, int32_t *blocks, int32_t *max_resident);

/* ------------------------------------------------------ batched adjoint
 * D designs of one grid and one set of physical parameters (fv_params of
 * the phased array), each with its own element weights, loss window
 * (windows[d]) and adaptive dt schedule, stepped together: every attempt of
 * the recorded forward, every replayed step and every reverse step of the
 * backward is one launch sequence over all D designs. Each design's loss
 * and gradients equal what fv_adjoint_forward/backward give for it alone,
 * bit for bit. Memory: D times fv_adjoint's. amp, phase: D x array_elems,
 * design-major; loss: D; grad_amp, grad_phase: D x array_elems. No
 * reference counterpart (the reference has no adjoint). */
typedef struct fv_adjoint_batch fv_adjoint_batch;
fv_status fv_adjoint_batch_create(const fv_params *p, int32_t ndesigns, const fv_loss_window *windows,
                                  int64_t nsteps, int32_t checkpoint_every, fv_adjoint_batch **out);
fv_status fv_adjoint_batch_destroy(fv_adjoint_batch *b);
fv_status fv_adjoint_batch_set_stream(fv_adjoint_batch *b, void *cuda_stream);
fv_status fv_adjoint_batch_forward(fv_adjoint_batch *b, const float *amp, const float *phase, double *loss);
fv_status fv_adjoint_batch_backward(fv_adjoint_batch *b, double *grad_amp, double *grad_phase);
/* design's recorded dt and T (before each accepted step), nsteps each */
fv_status fv_adjoint_batch_schedule(fv_adjoint_batch *b, int32_t design, double *dt, double *T);

/* ------------------------------------------------- step without allocation
 * For callers that cannot let this library call cudaMalloc: programs whose
 * device memory belongs to one allocator of their own (a framework's
 * caching allocator, or an arena sized at start-up) would have a library
 * allocation bypass their accounting, or fail once the arena holds the
 * device. fv_step_noalloc attempts one step of `p`'s simulation from the
 * caller's input state into the caller's output state (NX*NY device floats
 * per field each) at time T with step dt and window offsets mdx, mdy, and
 * allocates nothing: the step kernel's scratch (control block, per-CTA CFL
 * maxima, ghost frame, fix-up scratch) is one fixed __device__ array of
 * FV_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until
 * the process exits. Limit: nx + ny <= FV_NOALLOC_MAX_PERIMETER; larger grids
 * are rejected with FV_BAD_ARG. All calls on a device share the array, so
 * calls that overlap on the GPU race: serialise them. The first call on
 * each device looks up the array's address, so make it before any stream
 * capture. The input and output buffers must be distinct (FV_BAD_ARG
 * otherwise). The attempt runs fv_create's launch shape and division.
 * Each call is one attempt: res->accepted = 0 means CFL >= CFLMAX, the
 * output holds no step, and res->dt_next is the retry's dt (update_dt's 0.9
 * rule); retry from the same input with it. The library keeps no count of
 * rejections across calls, so the caller bounds its own retries
 * (res->status is FV_DT_TOO_LARGE after a rejection only when
 * p->max_retries is 1). No reference counterpart. */
#define FV_NOALLOC_SCRATCH_BYTES (2104u * 1024u)
#define FV_NOALLOC_MAX_CTAS 2048
#define FV_NOALLOC_MAX_PERIMETER 16384

typedef struct fv_step_result {
  int32_t accepted;       /* 1: output holds the new state; 0: rejected (retry) */
  int32_t status;         /* fv_status of the attempt */
  double cfl;             /* CFL of the attempt */
  double dt_next;         /* dt for the next attempt (update_dt) */
  double T;               /* time after the attempt */
  int32_t mdx, mdy;       /* window offsets after the attempt */
} fv_step_result;

fv_status fv_step_noalloc(const fv_params *p, const float *in_u1, const float *in_u2,
                          const float *in_u3, float *out_u1, float *out_u2, float *out_u3,
                          double dt, double T, int32_t mdx, int32_t mdy, void *cuda_stream,
                          fv_step_result *res);

#ifdef __cplusplus
}
#endif

#endif /* FIVONAGI_H */
