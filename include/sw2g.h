/*
 * sw2g: GB300 (sm_103a) implementation of the SW2 shallow-water time step,
 * behind a plain C ABI (no CUDA or torch types in any signature).
 *
 * It replaces the reference's per-step hot path: the body of
 *   void loop(char *bname, char *output_folder, sw *SW)          (core.c:22, sw.h:223)
 * from core.c:134 to core.c:338, i.e. compute_Dt, solve_tracer, solve_cons_h,
 * do_AdamsBashforth, do_eta_geofactor, solve_adv_u/v, solve_pres_u/v,
 * dissipation_effect, laplacian_vels/laplacian_eta, solve_Coriolis_u/v,
 * halo_update and do_channel (sw.h:230-292; laplacian.c; sppde_hupdate.c),
 * together with the energy diagnostic calc_energy_balance (energy.c:25).
 *
 * Fields cross the boundary in the reference's own layout: padded
 * (nx+4) x (ny+4) arrays of doubles, halo width 2, x fastest, cell (i,j) at
 * (i+1) + (j+1)*(nx+4) for i in [-1,nx+2], j in [-1,ny+2] (sppde/sppde.h:131-142).
 *
 * Errors are returned, never raised: no call exits or aborts the process
 * (the reference calls MPI_Abort through CRASH, sppde_core.c:163-190).
 * A context is used by one host thread at a time; it owns its device memory
 * and its CUDA stream. Calls on one context are not reentrant.
 */
#ifndef SW2G_H
#define SW2G_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  SW2G_OK = 0,
  SW2G_ERR_BAD_ARG = 1,   /* invalid case or argument (the reference CRASHes in init.c) */
  SW2G_ERR_CFL = 2,       /* Dt > Dt_CFL at the start of a step (core.c:156-158) */
  SW2G_ERR_NONFINITE = 3, /* field range check failed after a step (core.c:309-312) */
  SW2G_ERR_TIMEOUT = 4,   /* a bounded device wait gave up (the FP32 form's TMA row loads;
                             the step's state is then not advanced consistently) */
  SW2G_ERR_CUDA = 5,      /* a CUDA runtime call failed */
  SW2G_ERR_NOMEM = 6,     /* device or host allocation failed */
  SW2G_ERR_STATE = 7,     /* call out of order (e.g. step before upload) */
  SW2G_ERR_FORCING = 8    /* a Gaussian evaluated on the device injected no volume, or the
                             rescaled volume missed its target (perturbs.c:310-326) */
} sw2g_status;

/* Arithmetic of the step. */
typedef enum {
  SW2G_FP64 = 0, /* plain FP64, bit-identical to the reference's single-rank run */
  SW2G_FP32 = 1  /* FP32 stencils on height perturbation, FP64 state accumulation */
} sw2g_precision;

/* Behaviour flags (sw2g_case.flags). Zero reproduces the reference exactly. */
#define SW2G_FLAG_VANLEER_SAFE 0x1u  /* Van Leer limiter gives 0 (its limit) at r = -1 instead of 0/0 */
/* Input conventions, for callers that fill sw2g_case from the reference's own
 * sw struct rather than from the .sw file: */
#define SW2G_FLAG_RADIANS 0x2u /* lon0..lat1 are in radians, as the sw struct holds them (init.c:56-58) */
#define SW2G_FLAG_SIGMA 0x4u   /* tau holds sigma_dis (0 = no damping), as the sw struct holds it (init.c:110-114) */
/* The hyperviscosity of eta takes eta as its source; the reference passes u
 * (calc.c:332), which stays the default. FP64 contexts only. */
#define SW2G_FLAG_LAPE_ETA 0x8u

/* The parsed case, as the reference's initialize() stores it in the sw struct
 * (init.c:48-161). Angles are in degrees, as in the .sw file. */
typedef struct {
  int nx, ny;                    /* interior cells; each >= 3 (sppde_core.c:431-459); nx = ny = n when polar */
  int sch;                       /* limiter 0..9 (calc.c:262-273) */
  double lon0, lon1, lat0, lat1; /* degrees (radians with SW2G_FLAG_RADIANS) */
  double Omega, rE, rP, gE, depth;
  double Dt;                     /* time step (s) */
  double courant;                /* CFL: Dt must not exceed courant / max(|u|/dx + |v|/dy) */
  double tau;                    /* Tau: sigma = 1/tau, 0 when tau > 1e10 (init.c:110-114);
                                    sigma itself with SW2G_FLAG_SIGMA */
  double tracer_dis;             /* TracerDis */
  double hypernu[3];             /* Hypernu as entered: nu2, nu4 (positive), nu6 */
  unsigned flags;                /* SW2G_FLAG_* */
  /* Polar caps (init.c:66-79, 154-162, 243-277): polar = 1 (north) or -1
   * (south) runs the square lon0..lon1 x lat0..lat1 = -angleSim..angleSim
   * around the pole on the sphere of radius rE^2/rP, with gravity and
   * Coriolis from each point's angular distance to the pole and a sponge of
   * rate sigma_sponge beyond beta_sponge from it (degrees, radians with
   * SW2G_FLAG_RADIANS); no walls. rE and rP are the case file's values.
   * Either form; an FP32 cap is batched alone. polar = 0: the band. */
  int polar;
  double beta_sponge, sigma_sponge;
} sw2g_case;

typedef struct sw2g_ctx sw2g_ctx;

/* Upload modes. */
#define SW2G_UPLOAD_RAW 0   /* every padded cell verbatim (state mid-run) */
#define SW2G_UPLOAD_FRAME 1 /* interiors of eta/u/v/tracer, halos refreshed by the single-rank
                               wrap (what load_binary_sw leaves, io.c:115-171); winds and hB verbatim */
#define SW2G_UPLOAD_CONTINUE 2 /* as RAW, but the Adams-Bashforth history and the step count are
                                  kept: a caller that holds the state on the host between steps */

/* Returns a static description of a status code. */
const char *sw2g_status_string(sw2g_status s);

/* Creates a context on CUDA device `device` and builds the per-row geometry
 * (coords.c:21-126, init.c:279-297). Replaces the allocation part of loop()
 * (core.c:55-81) and the geometry part of initialize(). */
sw2g_status sw2g_create(const sw2g_case *c, int precision, int device, sw2g_ctx **out);

/* Copies the state in. Any pointer among tracer/windx/windy/hB may be NULL
 * (read as zero). Resets the Adams-Bashforth start-up, as a reference restart
 * does (core.c:133-134). Replaces load_binary_sw (io.c:115) and the pre-loop
 * halo/channel set-up (core.c:88-101). */
sw2g_status sw2g_upload(sw2g_ctx *ctx, const double *eta, const double *u, const double *v,
                        const double *tracer, const double *windx, const double *windy,
                        const double *hB, int mode);

/* Advances nsteps time steps (the loop body, core.c:134-338). The
 * Adams-Bashforth history is kept across calls. On SW2G_ERR_CFL or
 * SW2G_ERR_NONFINITE, sw2g_error_step() gives the 0-based step (counted from
 * the last upload) where the reference would have aborted; the device state
 * is then unspecified. */
sw2g_status sw2g_step(sw2g_ctx *ctx, int nsteps);

/* One step in two halves, for callers that add the reference's forcing where
 * it adds it (core.c:292-294): sw2g_step_open runs the step through the
 * velocity halo update (core.c:134-290); the forcing calls below may then
 * change eta, u, v and the tracer; sw2g_step_close applies do_channel and the
 * range checks (core.c:303-312) and returns the step's status as sw2g_step
 * does. No other step call may come in between. In the FP32 form
 * sw2g_step_open runs the whole fused step with the plain halo update of u and
 * v, and sw2g_step_close also makes the halo update of a forced eta and
 * tracer (core.c:297-300) and refreshes the FP32 copies of what changed. */
sw2g_status sw2g_step_open(sw2g_ctx *ctx);
sw2g_status sw2g_step_close(sw2g_ctx *ctx);

/* The per-step call of a caller that keeps the state in its own padded host
 * arrays, as the reference's loop keeps SW->eta, SW->u and SW->v (core.c:134-338):
 * copies eta, u and v in (as sw2g_upload with SW2G_UPLOAD_CONTINUE), advances
 * nsteps steps (as sw2g_step) and copies the new state back into the same
 * arrays (as sw2g_download), also when a step fails. In the FP64 form most
 * of the copies overlap the step: v and eta go in while the step's first
 * kernels, which read only u (the eta Laplacians) or only u and v (the
 * advection of u and v), run; eta comes out while the step goes on with u
 * and v, and u while it computes v. Needs an earlier sw2g_upload (winds,
 * bottom, tracer, history). */
sw2g_status sw2g_step_host(sw2g_ctx *ctx, double *eta, double *u, double *v, int nsteps);

/* Step index of the last CFL/range failure, -1 if none. */
int sw2g_error_step(const sw2g_ctx *ctx);

/* Copies the padded state out; NULL pointers are skipped. */
sw2g_status sw2g_download(sw2g_ctx *ctx, double *eta, double *u, double *v, double *tracer);

/* Kinetic and available potential energy as calc_energy_balance (energy.c:25-55)
 * defines them, and mass = sum of H*DXC*DYC over the interior (same area element),
 * each summed with compensated FP64 arithmetic. */
sw2g_status sw2g_diag(sw2g_ctx *ctx, double *ke, double *ape, double *mass);

/* Restarts the Adams-Bashforth sequence with an Euler step (as after LoadFrom). */
sw2g_status sw2g_reset_ab(sw2g_ctx *ctx);

/* Test of the failure path of the FP32 form's bounded device waits: with
 * waits > 0 each warp of the following steps' kernels, once the first rows of
 * its first strip have arrived, also waits for a barrier phase that nothing
 * completes, gives up after `waits` tries, and the step returns
 * SW2G_ERR_TIMEOUT with the device still usable; waits = 0 restores normal
 * operation. FP32 contexts only. No counterpart in the reference. */
sw2g_status sw2g_test_tile_timeout(sw2g_ctx *ctx, int waits);

/* Exact restart of an FP64 context. The reference restarts from a frame
 * (interior only, halos rewrapped) with the Adams-Bashforth index reset
 * (core.c:115-134), so its restarted run departs from the uninterrupted one.
 * A checkpoint holds everything the next step reads: every padded cell of
 * eta, u, v, tracer, windx, windy and hB, the tendency histories D(n-1) and
 * D(n-2) of eta, u, v and tracer, the Adams-Bashforth index and whether the
 * tracer is advected. Loaded into a context created from the same case, the
 * run continues bit for bit as if it had not stopped.
 *   sw2g_checkpoint_doubles: length of the buffer (doubles); 0 for an FP32 context.
 *   sw2g_checkpoint_save / _load: buffer of that length; the first values are
 *   a header (format, nx, ny, Adams-Bashforth index, tracer flag). Loading a
 *   buffer of another grid or format gives SW2G_ERR_BAD_ARG. */
size_t sw2g_checkpoint_doubles(const sw2g_ctx *ctx);
sw2g_status sw2g_checkpoint_save(sw2g_ctx *ctx, double *buf, size_t n);
sw2g_status sw2g_checkpoint_load(sw2g_ctx *ctx, const double *buf, size_t n);

/* Steps taken since the last upload. */
long long sw2g_steps_done(const sw2g_ctx *ctx);

/* Forcing between steps, for the reference's time-dependent perturbations
 * (add_Gaussians and add_vortices, perturbs.c:22-477), which it applies after
 * a step's velocity update. `which` is 0 eta, 1 u, 2 v, 3 tracer; arrays are
 * padded host arrays of which the interior is read; each call ends with the
 * single-rank halo wrap of the field. Either form: an FP32 context changes its
 * FP64 state (heights given to the set calls are taken as eta) and starts
 * advecting a tracer that is forced.
 *   sw2g_add_field:       field(i,j) += scale * delta(i,j)   (perturbs.c:308, 474-481)
 *   sw2g_set_field_where: field(i,j) = value(i,j) where mask(i,j) != 0 (perturbs.c:356-358)
 *   sw2g_apply_channel:   do_channel on u, v, windx and windy (calc.c:600-649), for
 *                         the forcing at t0, which the reference follows with it
 *                         (core.c:96-101); nothing for a polar cap, which has no
 *                         walls.
 * During a run, apply the forcing between sw2g_step_open and sw2g_step_close:
 * the reference's halo update copies wall-row values into the x halos before
 * its do_channel, so the order is part of the result. */
sw2g_status sw2g_add_field(sw2g_ctx *ctx, int which, const double *delta, double scale);
sw2g_status sw2g_set_field_where(sw2g_ctx *ctx, int which, const double *value, const unsigned char *mask);
sw2g_status sw2g_apply_channel(sw2g_ctx *ctx);

/* The same forcing on a list of cells, for injections that touch few cells
 * (a Gaussian truncated at its radius, get_Gaussian_field, perturbs.c:333-364):
 * only the list crosses to the GPU. `cells` holds n padded indices
 * (i+1)+(j+1)*(nx+4) of interior cells, strictly increasing; `values` their n
 * values. Each call ends with the single-rank halo wrap of the field.
 *   sw2g_add_cells: field(i,j) += scale * value for listed cells and
 *                   field(i,j) += scale * 0.0 for every other interior cell,
 *                   exactly the reference's loop over the whole grid
 *                   (perturbs.c:305-309), so the result is that of
 *                   sw2g_add_field with a delta that is zero off the list;
 *   sw2g_set_cells: field(i,j) = value for listed cells (TRACER inside the
 *                   radius, perturbs.c:356), others unchanged.
 * The lists are copied before the call returns; the work is queued on the
 * context's stream without waiting for it. Either form. */
sw2g_status sw2g_add_cells(sw2g_ctx *ctx, int which, const int *cells, const double *values, int n,
                           double scale);
sw2g_status sw2g_set_cells(sw2g_ctx *ctx, int which, const int *cells, const double *values, int n);

/* A Gaussian injection evaluated on the device (add_Gaussian_core and
 * get_Gaussian_field, perturbs.c:199-364): the caller gives the values the
 * reference derives per step from its Gaussian table (the ramped flow rate,
 * the moved centre, the peak before rescaling, perturbs.c:56-241), the GPU
 * evaluates every cell's great-circle distance to the centre and to the
 * requested periodic images, sums the injected volume over the cells inside
 * the radius, rescales it to `volume` and adds it to eta, and sets the tracer
 * inside the radius. The distance, exp and volume sum use the GPU's FP64
 * arithmetic, so results are within rounding of the reference's (the
 * bit-identical path is the host evaluation with sw2g_add_cells and
 * sw2g_set_cells); a cell whose distance is within rounding of the radius can
 * fall on the other side of it. Either form; nothing crosses to the GPU but
 * these scalars, and the call does not wait for the GPU inside an opened step
 * (sw2g_step_open): a volume failure is then returned by sw2g_step_close as
 * SW2G_ERR_FORCING; outside one the call waits and returns it. */
typedef struct {
  double lon, lat;       /* centre, radians: planetographic latitude; lon within [lon0, lon1] */
  double amp;            /* peak height before the rescale (perturbs.c:241) */
  double sigma, radius;  /* metres */
  double inject;         /* tracer value at the centre (the tracer is set to inject*exp(-r^2/2sigma^2)) */
  double volume;         /* Dt times the ramped flow rate; |volume| <= 1e-7: no rescale and eta unchanged */
  int images;            /* bit 0: also the image at lon - (lon1 - lon0); bit 1: at lon + (lon1 - lon0)
                            (perturbs.c:250-258), evaluated after the centre in that order */
} sw2g_gaussian;
sw2g_status sw2g_add_gaussian(sw2g_ctx *ctx, const sw2g_gaussian *g);

/* Device pointer of a padded state field (0 eta, 1 u, 2 v, 3 tracer) for
 * callers that keep data on the GPU; NULL on a bad index. */
void *sw2g_device_field(sw2g_ctx *ctx, int which);

/* CUDA stream the context launches on (as void*; cudaStream_t underneath). */
void *sw2g_stream(sw2g_ctx *ctx);

/* Number of kernel launches issued by the last sw2g_step call. */
long long sw2g_last_launches(const sw2g_ctx *ctx);

/* Device time (ms, CUDA events on the context's stream) from the first to the
 * last launch of the last sw2g_step call. Replaces the reference's per-step
 * wall-clock channel (core.c:143,333-336). */
double sw2g_last_step_ms(const sw2g_ctx *ctx);

/* Named per-kernel device timers, the counterpart of the reference's
 * cr_start/cr_end channels (sppde/sppde_cr.c:38-217). While enabled, each
 * launch is bracketed by CUDA events; times accumulate per kernel name until
 * reset. Names are static strings owned by the library. */
sw2g_status sw2g_timers_enable(sw2g_ctx *ctx, int on);
void sw2g_timers_reset(sw2g_ctx *ctx);
int sw2g_timers_count(const sw2g_ctx *ctx);
sw2g_status sw2g_timer_read(const sw2g_ctx *ctx, int idx, const char **name, long long *launches,
                            double *total_ms);

void sw2g_destroy(sw2g_ctx *ctx);

/* ------------------------------------------------------------------ batches
 * Ensembles of independent runs (the reference runs one case per MPI job).
 * A batch steps several SW2G_FP32 contexts together: one launch per phase of
 * the step covers every strip of every member, grids may differ in size, and
 * the time loop replays a captured CUDA graph of one step. Members must be
 * uploaded FP32 contexts on one device with the same limiter; a polar cap
 * batches alone (n = 1; a cap among other members gives SW2G_ERR_BAD_ARG).
 * Each member's state stays readable through its own context (sw2g_download,
 * sw2g_diag). */
typedef struct sw2g_batch sw2g_batch;

/* Most members of one batch. */
#define SW2G_BATCH_MAX 96

sw2g_status sw2g_batch_create(sw2g_ctx *const *members, int n, sw2g_batch **out);
/* Advances every member nsteps steps. On SW2G_ERR_CFL / SW2G_ERR_NONFINITE
 * the first failing (step, member) is reported by the two calls below and
 * through that member's sw2g_error_step. */
sw2g_status sw2g_batch_step(sw2g_batch *b, int nsteps);
int sw2g_batch_error_member(const sw2g_batch *b);
int sw2g_batch_error_step(const sw2g_batch *b);
double sw2g_batch_last_step_ms(const sw2g_batch *b);
long long sw2g_batch_last_launches(const sw2g_batch *b);

/* Autotuner of the batch's launch shape. Neither the strip shape (128 cells
 * wide, 16, 32 or 64 rows high: SW2G_TILE_SHAPES shapes) nor the order in
 * which the strips of all members are taken by the kernels' warps
 * (SW2G_SCHEDULES orders: rows, columns, members interleaved, bands of 8
 * strip columns) changes any result, so the candidates are timed on the live
 * run: each of the SW2G_TILE_SHAPES x SW2G_SCHEDULES pairs advances the batch
 * steps_per_candidate steps (after one untimed step per shape, which captures
 * its graph); ms_per_step[shape * SW2G_SCHEDULES + schedule] receives its time
 * per step (may be NULL), and the fastest pair is kept.
 * sw2g_batch_set_schedule picks a pair by hand (tile_rows 16, 32 or 64). A
 * batch of one member sizes its strips itself, as a single context does. */
#define SW2G_SCHEDULES 4
#define SW2G_TILE_SHAPES 3
sw2g_status sw2g_batch_tune(sw2g_batch *b, int steps_per_candidate, double *ms_per_step);
sw2g_status sw2g_batch_set_schedule(sw2g_batch *b, int tile_rows, int schedule);
int sw2g_batch_schedule(const sw2g_batch *b);
int sw2g_batch_tile_rows(const sw2g_batch *b);
void sw2g_batch_destroy(sw2g_batch *b);

/* Self-check of the FP64 step's division by a row metric factor (one
 * multiplication and two fused multiply-adds with the metric's correctly
 * rounded reciprocal; results must equal IEEE division bit for bit). For each
 * of the n divisors (positive, normal) draws `samples` numerators, random and
 * near rounding midpoints, and also takes the 1024 numerators within 512 ulps
 * below +-2, on CUDA device `device`; returns in *mismatches how many
 * quotients differ from IEEE a/b. No counterpart in the reference. */
sw2g_status sw2g_selfcheck_division(const double *divisors, int n, long long samples, unsigned long long seed,
                                    int device, long long *mismatches);

/* Self-check of the FP64 step's additions done on the integer pipe (a + b and
 * a - b rounded to nearest even from the operands' bits; results must equal
 * the FP64 unit's bit for bit, NaNs as NaNs). Draws `samples` operand pairs,
 * random and at the adder's edge cases (cancellation, ties, carries, the
 * overflow and subnormal limits, zeros, inf, NaN), on CUDA device `device`,
 * and returns in *mismatches how many of the 2 * samples results differ.
 * No counterpart in the reference. */
sw2g_status sw2g_selfcheck_add(long long samples, unsigned long long seed, int device, long long *mismatches);

/* Largest ny accepted by sw2g_energy_noalloc. */
#define SW2G_NOALLOC_MAX_ROWS 8192

/* Energy diagnostic that allocates nothing. This entry point has no
 * counterpart in the reference.
 *
 * sw2g_diag needs a context, whose creation allocates device memory. Some
 * callers hold fields on the GPU but cannot let a library allocate: a host
 * loop whose device memory is already reserved by its own pool allocator, a
 * time loop in which a cudaMalloc/cudaFree would synchronise the device in
 * the middle of a step, or a post-processing tool that owns its field buffers
 * and never creates a context. This call gives them the same three sums as
 * sw2g_diag (kinetic and available potential energy as energy.c:25-55
 * defines them, and mass), without any cudaMalloc, cudaFree or other
 * allocating routine.
 *
 * All field pointers are device pointers on the current CUDA device, in the
 * padded layout; windx, windy and hB may be NULL (read as zero). out3 is a
 * device pointer to three doubles (ke, ape, mass). Work is queued on `stream`
 * (a cudaStream_t; NULL is the default stream); out3 is valid once it is done.
 *
 * Band cases only (a polar cap gives SW2G_ERR_BAD_ARG: its gravity is a 2-D
 * field; sw2g_diag covers caps).
 *
 * Limits and sharing: ny must not exceed SW2G_NOALLOC_MAX_ROWS (otherwise
 * SW2G_ERR_BAD_ARG and a message on stderr). The scratch is one fixed 320 KiB
 * array in device memory that every GPU loading the library holds until the
 * process exits, and that all calls share: each call rewrites the rows it
 * reads, but calls that overlap on the GPU (other streams, other host
 * threads) race on it and must be serialised by the caller. The first call on
 * a device looks up the array's device address (cudaGetSymbolAddress); make
 * that first call before any stream capture. */
sw2g_status sw2g_energy_noalloc(const sw2g_case *c, const double *eta, const double *u, const double *v,
                                const double *windx, const double *windy, const double *hB, double *out3,
                                void *stream);

#ifdef __cplusplus
}
#endif
#endif
