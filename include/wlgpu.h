/*
 * wlgpu.h -- C ABI of the GB300 Wilson-loop library (libwlgpu.so).
 *
 * Replaces the reference's kernel boundary (intEV.cu:111-148, intEVff.cu:96-131:
 * EV() launching ExpectValue and averaging with EVMean, Integrand.c:325-407)
 * with (1) the same legacy entry point EV() (declared in wl_legacy.h) and
 * (2) a status-returning batched API that evaluates many (centre of mass,
 * proper time, flux) instances of one field profile in one pass over a
 * device-resident loop ensemble.
 *
 * Conventions
 *  - Every function returns WL_OK (0) or a negative WL_ERR_* status; the
 *    message of the last failure is available from wl_last_error().
 *  - Pointers named host_* are host memory; the library copies them.  Device
 *    pointers are named dev_* .  Nothing is retained after a call returns
 *    unless stated (ensembles).
 *  - A context owns one CUDA stream on one device; calls on one context must
 *    not run concurrently from several host threads.
 *  - Loop ensembles are float32 [Nl][ppl][4] (x, y, z, w), the reference's
 *    float4 layout (EffAct.c:368-381); only x and y enter the Wilson loop.
 *    ppl must be a multiple of 4 (sub-loop structure, intEV.cu:461-506).
 */
#ifndef WLGPU_H
#define WLGPU_H

/* Legacy sources include intT.h first, whose profile names and constants
 * (step, smooth, ..., profile, tubedist, lmin, q1, q2, ...) are object-like
 * macros; they are set aside while this header is read and restored after. */
#pragma push_macro("step")
#undef step
#pragma push_macro("smooth")
#undef smooth
#pragma push_macro("quadratic")
#undef quadratic
#pragma push_macro("gaussian")
#undef gaussian
#pragma push_macro("periodic")
#undef periodic
#pragma push_macro("spline")
#undef spline
#pragma push_macro("fixflux")
#undef fixflux
#pragma push_macro("profile")
#undef profile
#pragma push_macro("pi")
#undef pi
#pragma push_macro("tubedist")
#undef tubedist
#pragma push_macro("lmin")
#undef lmin
#pragma push_macro("q1")
#undef q1
#pragma push_macro("q2")
#undef q2
#pragma push_macro("Nspline")
#undef Nspline
#pragma push_macro("verbosity")
#undef verbosity

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WL_OK 0
#define WL_ERR_INVALID (-1) /* an argument is out of range                 */
#define WL_ERR_CUDA (-2)    /* a CUDA runtime call failed                   */
#define WL_ERR_NOMEM (-3)   /* device or pinned host allocation failed      */
#define WL_ERR_TIMEOUT (-4) /* a bounded device-side wait gave up           */
#define WL_ERR_NOTFOUND (-5)/* unknown ensemble handle                      */
#define WL_ERR_ADMISSION (-6)/* request exceeds the admission budget        */

/* field profiles: the values of the reference's profile macros (intT.h) */
#define WL_PROFILE_STEP 0
#define WL_PROFILE_SMOOTH 1
#define WL_PROFILE_QUADRATIC 2
#define WL_PROFILE_GAUSSIAN 3
#define WL_PROFILE_PERIODIC 4
/* the tabulated profile of periodic.c:17-164: f(rho) integrates
 * (2/lambda^2) rho exp(-sin^2(pi rho/a)/lambda^2) from 0 on 1000 knots over
 * rho in (0, 20], interpolated by a clamped cubic spline in rho^2 (0 outside
 * the table, as interp, intEV.cu:64-107).  f' is the reference kernel's
 * exp(-sin^2(pi rho)/lambda^2)/lambda^2 (intEV.cu:389-397, which leaves a out)
 * in WL_MODE_REFCOMPAT and the derivative of the tabulated f (sin(pi rho/a))
 * in WL_MODE_EXACT.  The reference builds the table with GSL's ODE stepper,
 * which is not available here: this library integrates with Gauss-Legendre
 * quadrature per knot interval (the right-hand side does not depend on f). */
#define WL_PROFILE_SPLINE 5
#define WL_PROFILE_FIXFLUX 6
/* wl_legacy_configure only: the fixflux profile with intEVff.cu's phi / chi
 * fits (ff_variant 1), which the reference selects by linking intEVff.o
 * instead of intEV.o; wl_legacy_query then reports WL_PROFILE_FIXFLUX. */
#define WL_PROFILE_FIXFLUX_FF 7
/* Square lattice of identical Gaussian flux tubes at R = a(m, n), |R| <=
 * rimage (no counterpart in the reference, whose "periodic" profile is a
 * radial shell model, intEV.cu:201-232): every image contributes the
 * reference's single-tube Gaussian segment integral (intEV.cu:408-459,
 * 282-284) in coordinates relative to R.  Exact mode only: the reference's
 * b >= 1e-8 clamp would break the pure-gauge cancellation of distant images.
 * Images farther than sqrt(18) lambda from the loop's bounding box see
 * f = 1 - e^-18 along the whole loop, which is 1 in FP32 (pure gauge), and
 * lie outside it (winding 0): their continuum contribution is zero and they
 * are skipped. */
#define WL_PROFILE_LATTICE 8

/* clamp modes of the segment polynomial */
#define WL_MODE_REFCOMPAT 0 /* the reference's clamps (intEV.cu:418-422, 439) */
#define WL_MODE_EXACT 1     /* exact rho^2(t); 1e-30 floor where f/rho^2 divides */

/* flux-tube field and quadrature of one evaluation */
typedef struct {
  int profile;    /* WL_PROFILE_*                                             */
  int fermion;    /* 1: spinor QED (spin factor cosh), 0: scalar QED          */
  int nint;       /* Simpson intervals per segment, even, 2..64 (ref: 50)     */
  int mode;       /* WL_MODE_*                                                */
  int ff_variant; /* fixflux: 0 = intEV.cu phi/chi fits, 1 = intEVff.cu ones  */
  int reserved;
  double lambda2; /* lambda^2                                                 */
  double tubedist;/* lattice spacing a (periodic, fixflux)                    */
  double lmin;    /* fixflux minimum width (0.1 a in the reference)           */
  double rimage;  /* lattice: image tubes with |R| <= rimage (e.g. 12 a)      */
} wl_field;

typedef struct wl_ctx wl_ctx;

/* version and status text */
const char *wl_version(void);
const char *wl_status_string(int status);

/* context: one device, one stream */
int wl_ctx_create(int device, wl_ctx **out);
int wl_ctx_destroy(wl_ctx *ctx);
int wl_last_error(wl_ctx *ctx, char *buf, int buflen);
int wl_ctx_synchronize(wl_ctx *ctx);

/* ---- resident loop ensembles ------------------------------------------ */
/* copy a host ensemble to the device; *handle identifies it afterwards */
int wl_ensemble_upload(wl_ctx *ctx, const float *host_loops, int Nl, int ppl,
                       int *handle);
/* use caller-owned device memory (not freed by the library) */
int wl_ensemble_wrap(wl_ctx *ctx, const float *dev_loops, int Nl, int ppl,
                     int *handle);
/* generate seeded unit loops on the device: closed Brownian bridges of unit
 * proper time, per-component step variance 2/ppl, centre of mass at the
 * origin; loop l draws Philox4x32-10 numbers keyed by (seed, first + l). */
int wl_ensemble_generate(wl_ctx *ctx, uint64_t seed, int first, int Nl, int ppl,
                         int *handle);
int wl_ensemble_download(wl_ctx *ctx, int handle, float *host_loops);
int wl_ensemble_release(wl_ctx *ctx, int handle);
/* device pointer and sizes of an ensemble */
int wl_ensemble_info(wl_ctx *ctx, int handle, const float **dev_loops, int *Nl,
                     int *ppl);

/* ---- batched <W> -------------------------------------------------------- */
/* Evaluate ninst instances (host_cx[i], host_cy[i], host_T[i]) for each of the
 * nF flux values host_F[j] (nF <= 4) on ensemble `handle`, with loops split
 * into ng = Nl / group groups (Nl % group == 0; the reference uses 128).
 * Outputs (host, any may be NULL):
 *   out_group[(i*nF + j)*ng + g]  <W> of group g, Richardson-combined
 *                                 8/3 W_N - 2 W_N/2 + 1/3 W_N/4
 *                                 (Integrand.c:352-400)
 *   out_mean[i*nF + j]            mean over groups
 *   out_sem[i*nF + j]             standard error of that mean over groups
 * The per-loop phases are FP32 (compensated sums); the loop averages FP64.  */
int wl_eval(wl_ctx *ctx, int handle, const wl_field *field, int ninst,
            const double *host_cx, const double *host_cy, const double *host_T,
            int nF, const double *host_F, int group, double *out_group,
            double *out_mean, double *out_sem);

/* Effective action density per centre of mass: for nrho radii rho[r] (centre
 * of mass (rho, 0), as rhogrand sets it, EffAct.c:21-25) and a log-spaced
 * proper-time grid T[0..nT-1] (ascending, nT >= 3), evaluates <W> on all
 * nrho*nT instances, then in FP64 on the device: the integrand of Tfunc
 * (Integrand.c:195-316; small-T series, constant-field and large-T forms,
 * else e^{-m^2 T}/T^3 (<W> - 1 + (eTB)^2/6) scalar / (<W> - 1 - (eTB)^2/3)
 * spinor with m^2 = 1, e = 0.30282212), Simpson over ln T on the grid, and
 *   out_leff[r*nF + j] = <I>/(4 pi) (spinor) or <I>/(-2 pi) (scalar)
 * (Tint.c:69-72), with out_err the jackknife error over nbins bins of the
 * Nl/group loop groups (nbins must divide Nl/group).  out_igrand (may be
 * NULL) receives the integrand [r][j][k][group]. */
int wl_tint(wl_ctx *ctx, int handle, const wl_field *field, int nrho, const double *host_rho,
            int nT, const double *host_T, int nF, const double *host_F, int group, int nbins,
            double *out_leff, double *out_err, double *out_igrand);

/* proper-time rules of wl_effective_action */
#define WL_TRULE_LOG 0   /* host_T: a log-spaced grid of nT points, Simpson in ln T
                            (as wl_tint)                                          */
#define WL_TRULE_SUBST 1 /* integrateT's rule (Tint.c:100-175): T = (1 - t)/t, nT
                            Simpson panels in t (rhogrand uses 40, EffAct.c:22);
                            host_T is ignored                                    */

/* The effective action per unit length (EffAct.c:83-306): the radial
 * integral of rho I_g(rho), I_g the proper-time integral of group g (flux F,
 * rule t_rule), divided by 4 pi (spinor) or -2 pi (scalar).  Isolated
 * profiles integrate rho over [0, inf) through rho = (1 - t)/t with nrho
 * Simpson panels in t (EffAct.c:140-210); periodic, spline and fixflux over
 * [0, a/2] with 2 nrho intervals (EffAct.c:83-138).  In WL_MODE_REFCOMPAT the
 * [0, a/2] rule keeps the reference's weights (the end a/2 counted twice,
 * the weights 2 and 4 on the opposite points of Simpson's rule); in
 * WL_MODE_EXACT it is Simpson's rule.  (The reference's t-panel rules, which
 * evaluate each panel's right end twice, equal Simpson's rule here: the
 * panel ends t = 0 and t = 1 contribute 0.)  Outputs the mean over groups and
 * its standard error, optionally the profile's classical action
 * (EffAct.c:228-279; NaN for the lattice) and the per-group values [Nl/group].
 * No counterpart as one call in the reference, which runs it as its main(). */
int wl_effective_action(wl_ctx *ctx, int handle, const wl_field *field, double F, int t_rule,
                        int nT, const double *host_T, int group, int nrho, double *out_action,
                        double *out_err, double *out_classical, double *out_groups);

/* Asynchronous variant on the context's stream for device-resident inputs and
 * outputs: dev_cx, dev_cy, dev_T [ninst] and the outputs are device pointers
 * (FP64, same layouts as wl_eval; outputs may be NULL), host_F stays a host
 * array.  Nothing is synchronised; invalid instances (T <= 0 or not finite)
 * and device-side wait time-outs are reported by the next
 * wl_ctx_synchronize().  Three kernel launches: instance set-up, sweep,
 * reduction. */
int wl_eval_device(wl_ctx *ctx, int handle, const wl_field *field, int ninst,
                   const double *dev_cx, const double *dev_cy, const double *dev_T,
                   int nF, const double *host_F, int group, double *dev_out_group,
                   double *dev_out_mean, double *dev_out_sem);

/* Throughput probe of one SM pipe on the context's device, for roofline
 * denominators: kind 0 = FP32 FMA, 1 = MUFU reciprocal, 2 = packed FP32x2 FMA
 * (fma.rn.f32x2, two FMAs per instruction).  *ops_per_s receives
 * lane operations per second over the whole device (about 0.1 s of work). */
int wl_peak_probe(wl_ctx *ctx, int kind, double *ops_per_s);

/* Self-test of the device's bounded waits (every shared-memory stage copy
 * is awaited by a bounded mbarrier wait that, when it gives up, sets the
 * launch's status so that the call returns WL_ERR_TIMEOUT and the context
 * stays usable).  One CTA waits, max_tries polls (1 .. 2^22; the sweeps use
 * 2^22) at most, on an mbarrier that gets its arrival (arrive = 1: returns
 * WL_OK) or never does (arrive = 0: the wait gives up and the call returns
 * WL_ERR_TIMEOUT).  No copy is issued.  *device_ms (may be NULL) receives the
 * kernel's time, i.e. how long max_tries polls take. */
int wl_selftest_wait(wl_ctx *ctx, int arrive, int max_tries, double *device_ms);

/* The spline profile's table for lambda^2 and the tube spacing (host only, no
 * device needed): knots rho2[n] (rho_i^2 as float, rho_i = 20 i/n) and the
 * spline coefficients coef4[n][4] = (f, b, c, d) of f + b d + c d^2 + d d^3,
 * d = rho^2 - rho2[i] (periodic.c:46-164 builds the same table). */
int wl_spline_table(double lambda2, double tubedist, int n, float *rho2, float *coef4);

/* Allocation-free variant of wl_eval_device.  No counterpart in the
 * reference.  For callers that cannot let a library allocate device memory:
 * a framework whose caching allocator owns the whole device (a cudaMalloc
 * behind its back can fail or break its accounting), code where cudaMalloc is
 * not permitted, or latency-critical loops where cudaMalloc/cudaFree would
 * synchronise the device.  It needs no context and allocates nothing: the
 * ensemble (dev_loops, float32 [Nl][ppl][4]), the instances and the outputs
 * are the caller's device buffers (layouts as wl_eval), and the scratch --
 * instance constants and FP64 partial sums -- lives in one fixed 32 MiB
 * device array inside the library, which every GPU that loads the library
 * holds until the process exits.  Requests that need more scratch than that
 * (about n_chunks * nF * 3 * ninst * 8 bytes, n_chunks = Nl / 8 for 32 or more
 * instances, Nl otherwise) are rejected with WL_ERR_INVALID and a message on
 * stderr; split them into smaller batches.  The first call on a device looks
 * up the array's device address (cudaGetSymbolAddress), so make that first
 * call before any stream capture.  Runs on `stream` (a cudaStream_t, NULL for
 * the default stream) and returns when the outputs are written.  All calls
 * share the one array, which keeps the last call's contents: calls that
 * overlap on the GPU (other host threads, other streams) race.  The lattice
 * and spline profiles are refused (WL_ERR_INVALID): they need per-loop
 * bounding boxes or a profile table that the library would allocate. */
int wl_eval_noalloc(const float *dev_loops, int Nl, int ppl, const wl_field *field,
                    int ninst, const double *dev_cx, const double *dev_cy,
                    const double *dev_T, int nF, const double *host_F, int group,
                    double *dev_out_group, double *dev_out_mean, double *dev_out_sem,
                    void *stream);

/* the context's CUDA stream (a cudaStream_t), for timing and interop */
int wl_ctx_stream(wl_ctx *ctx, void **stream);

/* Per-loop outputs of one instance, the reference kernel's Wsscal/Wsferm
 * (intEV.cu:553-561): host_scal[l*4 + k], host_ferm[l*4 + k], k = 0 (N/2),
 * 1 (N/4, i = 2 mod 4), 2 (N/4, i = 0 mod 4), 3 unused (0). */
int wl_loops(wl_ctx *ctx, int handle, const wl_field *field, double cx, double cy,
             double T, double F, float *host_scal, float *host_ferm);

/* How the last wl_eval on this context was run: kernel launches issued and
 * which sweep kernel ("instance-parallel" or "loop-parallel"). */
int wl_last_launches(wl_ctx *ctx, int *launches, const char **sweep_kind);

/* ---- uneven batches in one persistent launch ---------------------------- */
/* One evaluation job of a batch: instances of one ensemble and field. */
typedef struct {
  int handle;            /* ensemble                                         */
  wl_field field;        /* any profile (see wl_batch_eval)                  */
  int ninst;             /* instances (host arrays of ninst doubles)         */
  const double *cx, *cy, *T;
  int nF;                /* flux values (<= 4)                               */
  double F[4];
  int group;             /* loops per group (divides the ensemble's Nl)      */
  double *out_group;     /* host outputs as wl_eval (any may be NULL)        */
  double *out_mean, *out_sem;
} wl_job;

#define WL_BATCH_GRAPH 1 /* capture the device work as a CUDA graph and launch it */

/* Evaluate njobs jobs of uneven size in one persistent launch: every CTA takes
 * (job, instance tile, loop chunk) tiles from a device queue ordered by
 * decreasing cost; a job's results are identical to those it gets alone in a
 * batch (the tile shape depends only on the job and the tuned parameters).
 * The loops per tile come from the context's tuned points-per-tile target
 * (wl_batch_autotune; default 16384), the persistent grid from its tuned CTAs
 * per SM (default: the occupancy limit).  Jobs of the periodic, spline and
 * fixflux profiles are not tiles of the persistent kernel: each runs as one
 * launch of its profile's sweep kernel after it, with the same loops per
 * tile and partial-sum layout, before the common reduction. */
int wl_batch_eval(wl_ctx *ctx, int njobs, const wl_job *jobs, int flags);

/* Autotuner: times the batch for every candidate (points per tile in
 * {4096, 8192, 16384, 32768, 65536} x persistent CTAs per SM in
 * {occupancy - 1, occupancy}) and keeps the fastest in the context.  The
 * chosen values are returned (pointers may be NULL). */
int wl_batch_autotune(wl_ctx *ctx, int njobs, const wl_job *jobs, int *points_per_tile,
                      int *ctas_per_sm);

/* Statistics of the last wl_batch_eval: device time (ms, CUDA events around
 * the persistent kernel and the reduction), tiles, persistent CTAs, points per
 * tile. */
int wl_batch_stats(wl_ctx *ctx, double *device_ms, int *ntiles, int *grid,
                   int *points_per_tile);

/* The plain per-instance kernel, the baseline of the batched path: one
 * launch per instance with one thread per loop walking its points from
 * global memory (the reference kernel's structure, intEV.cu:573-582), same
 * arithmetic and outputs as wl_eval; the step, smooth, quadratic, gaussian
 * and lattice profiles.  *device_ms receives the summed time. */
int wl_eval_plain(wl_ctx *ctx, int handle, const wl_field *field, int ninst,
                  const double *host_cx, const double *host_cy, const double *host_T,
                  int nF, const double *host_F, int group, double *out_group,
                  double *out_mean, double *out_sem, double *device_ms);

/* ---- serving: continuously batched requests ----------------------------- */
#define WL_REQ_W 0    /* <W> per group of every (cx, cy, T) instance            */
#define WL_REQ_LEFF 1 /* effective action density L_eff(rho) as wl_tint        */

/* One request.  The ensemble is named by (seed, Nl, ppl) and generated on the
 * device the first time it is needed; it then stays resident.  Input arrays
 * are copied at submit; output arrays must stay valid until the request
 * completes. */
typedef struct {
  uint64_t seed;
  int Nl, ppl;
  wl_field field;
  int kind;                         /* WL_REQ_W or WL_REQ_LEFF                  */
  int ninst;                        /* WL_REQ_W: instances                      */
  const double *cx, *cy, *T;
  int nrho, nT, nbins;              /* WL_REQ_LEFF: rho x log-spaced T grid     */
  const double *rho, *Tgrid;
  int nF;
  double F[4];
  int group;
  double *out_group, *out_mean, *out_sem;  /* WL_REQ_W (layouts as wl_eval)  */
  double *out_leff, *out_err;              /* WL_REQ_LEFF: [nrho][nF]        */
} wl_request;

typedef struct {
  long long submitted, completed, rejected, failed;
  double p50_ms, p99_ms, p999_ms, mean_ms, max_ms;  /* submit -> complete      */
  double wall_s;            /* first submit -> last completion                */
  double segments;          /* loop-segments of the completed requests        */
  long long launches;       /* persistent-kernel launches                     */
  int resident_ensembles;
  double hbm_bytes_in_use;  /* ensembles + admitted requests' buffers         */
  double device_busy_s;     /* union of the launches' device intervals (the
                               persistent kernel and the heavy-profile sweeps,
                               event to event) since the statistics were reset */
  double device_span_s;     /* first launch start -> last launch end, same clock */
} wl_server_stats;

typedef struct wl_server wl_server;

typedef struct {
  int device;
  double hbm_budget_bytes;  /* ensembles + admitted requests; 0: 80% of the
                               device memory free at creation                 */
  double quantum_ms;        /* target device time of one launch; 0: 20 ms     */
  int points_per_tile;      /* loop points per tile; 0: 16384 (the batch
                               default, so results equal wl_batch_eval's)     */
  int ctas_per_sm;          /* persistent CTAs per SM; 0: occupancy limit     */
  int max_requests;         /* requests admitted at once; 0: 1024             */
} wl_server_config;

/* A request server: a worker thread admits requests in arrival order while
 * their HBM footprint (buffers, plus the ensemble if it is not resident) fits
 * the budget, least recently used idle ensembles being evicted when needed;
 * a request that can never fit completes with WL_ERR_ADMISSION.  Every
 * admitted request is cut into (instance tile, loop chunk) tiles; each launch
 * of the persistent kernel takes about quantum_ms of tiles from all admitted
 * requests, oldest first, and two launches are kept in flight on two streams
 * so that new requests' work overlaps the tail of the running one (periodic,
 * spline and fixflux requests take whole loop chunks per quantum, launched
 * as their profile's sweep over that chunk range).  Results
 * of a WL_REQ_W request are bit-identical to wl_batch_eval of the request
 * alone with the same points_per_tile; a WL_REQ_LEFF request integrates
 * those <W> values over proper time as wl_tint does. */
int wl_server_create(const wl_server_config *cfg, wl_server **out);
/* thread-safe; checks and copies the inputs; *ticket names the request */
int wl_server_submit(wl_server *srv, const wl_request *req, long long *ticket);
#define WL_PENDING 1 /* wl_server_wait: the request is not done yet        */
/* waits for a request (timeout_ms < 0: forever): WL_PENDING if it is not done
 * within timeout_ms, else the request's own status (the ticket is then
 * forgotten) */
int wl_server_wait(wl_server *srv, long long ticket, double timeout_ms);
int wl_server_get_stats(wl_server *srv, wl_server_stats *stats);
/* clears the statistics (latencies, counters, clocks); resident ensembles stay */
int wl_server_reset_stats(wl_server *srv);
/* the last error message of a submit or of the worker */
int wl_server_last_error(wl_server *srv, char *buf, int buflen);
/* finishes the admitted and queued requests, stops the worker, frees all */
int wl_server_destroy(wl_server *srv);

/* ---- legacy EV() configuration ----------------------------------------- */
/* The reference selects the profile at compile time (intT.h "profile"); the
 * library's EV() uses the profile, lattice spacing, Simpson intervals and
 * clamp mode set here (default: smooth, a = 1, 50 intervals, ref-compat).   */
int wl_legacy_configure(int profile, double tubedist, double lmin, int nint,
                        int mode);
/* the configuration EV() uses (any pointer may be NULL) */
int wl_legacy_query(int *profile, double *tubedist, double *lmin, int *nint, int *mode);
/* EV() keeps the per-loop W factors of its last (T, x_cm, F, lambda^2,
 * fermion, configuration, ensemble pointer and shape) so that the ng group
 * calls of one Tfunc (Integrand.c:249-305) cost one sweep.  A call for the
 * first group of 128 consecutive loops, or for any other index list, also
 * compares a 64-bit fingerprint of the ensemble's coordinates with the one
 * the cached sweep read, and recomputes if the loops were rewritten in
 * place.  Calls for the other consecutive groups at an unchanged key trust
 * the cache; a caller that rewrites the ensemble between those calls calls
 * wl_legacy_invalidate() (the next EV() call recomputes).  No counterpart in
 * the reference, whose EV() relaunches its kernel on every call
 * (intEV.cu:123). */
int wl_legacy_invalidate(void);

#ifdef __cplusplus
}
#endif

#pragma pop_macro("step")
#pragma pop_macro("smooth")
#pragma pop_macro("quadratic")
#pragma pop_macro("gaussian")
#pragma pop_macro("periodic")
#pragma pop_macro("spline")
#pragma pop_macro("fixflux")
#pragma pop_macro("profile")
#pragma pop_macro("pi")
#pragma pop_macro("tubedist")
#pragma pop_macro("lmin")
#pragma pop_macro("q1")
#pragma pop_macro("q2")
#pragma pop_macro("Nspline")
#pragma pop_macro("verbosity")

#endif /* WLGPU_H */
