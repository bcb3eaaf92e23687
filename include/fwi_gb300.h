/*
 * fwi_gb300.h -- C ABI of the GB300 (sm_103a) engine for the FWI gradient
 * hot path of FWI2DAcoustic-MPI-LBFGS.
 *
 * The reference's boundary is one collective call per MPI rank and shot,
 *     void grad4_1shot(fwi_plan *plan, int iter);          header.h:283
 * (called at MBotOpt.c:55 and MBotOpt.c:99, never defined in the reference),
 * which reads the velocity model plan->model->md (fwi_2d.c:179, the L-BFGS x
 * of MBotOpt.c:52), the observed traces plan->msf->obs0 (fwi_2d.c:196), the
 * geometry plan->sou->{xyz_sr, wav0} (fwi_2d.c:217-220) and writes the
 * gradient plan->grad->body (fwi_2d.c:380) and the misfit plan->msf->val
 * (fwi_2d.c:207).  This header splits that call into a context holding the
 * device state and a forward/backward pair, and batches all shots of an
 * iteration on one GPU instead of one shot per MPI rank.
 *
 * Conventions: every function returns an FWI_* status (0 = success) and never
 * exits; buffers are caller-owned host memory unless a name says _device;
 * every call is ordered on the context's CUDA stream and has completed when
 * it returns; a context is not thread safe.
 *
 * Discrete problem (identical to the CPU oracle):
 *   p^{it+1} = 2 p^it - p^{it-1} + K (L p^it) + s^it,  K = v^2 dt^2,
 *   L = the staggered 4th-order operator with CPML of a_lap_opt_2d_pml
 *       (fwi_2d.c:761-864; all-sides CPML when free_surface == 0),
 *   s^it = K(src) * wavelet[it] / (dx dz) at the source cell (fwi_2d.c:216),
 *   syn[r][k] = p^{k*jump+1}(receiver r),  k = 0 .. nt0-1, nt0 = (nt-1)/jump+1,
 *   J = 1/2 sum (syn - obs)^2,   gradient = dJ/dv on the physical grid
 *       (exact discrete adjoint; CPML cells are not imaged).
 */
#ifndef FWI_GB300_H
#define FWI_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define FWI_OK              0
#define FWI_ERR_ARG        -1   /* bad argument or configuration            */
#define FWI_ERR_GEOMETRY   -2   /* source/receiver outside the model        */
#define FWI_ERR_NOMEM      -3   /* device or host allocation failed         */
#define FWI_ERR_CUDA       -4   /* CUDA runtime error (see fwi_last_error)  */
#define FWI_ERR_STATE      -5   /* call order (e.g. backward before forward) */
#define FWI_ERR_CFL        -6   /* model violates the stability limit       */
#define FWI_ERR_NONFINITE  -7   /* NaN/Inf in an input                      */
#define FWI_ERR_NODEVICE   -8   /* no usable sm_103 device                  */

/* ---- configuration ------------------------------------------------------ */
typedef struct fwi_config {
    int   nx, nz;          /* physical grid, model is [nz][nx], x fastest (fwi_2d.c:148) */
    float dx, dz, dt;      /* metres, seconds (fwi_base, header.h:25) */
    int   nt_max;          /* largest per-shot nt that fwi_set_shots may pass */
    int   npml;            /* CPML cells (NPML, Mpar.h:16) */
    int   free_surface;    /* 1: CPML left/right/bottom, top is a free surface
                              (fwi_2d.c:154-157); 0: CPML on all four sides */
    int   jump;            /* receiver sampling interval in steps (DAT_JUMP;
                              (nt0-1)*jump == nt-1, fwi_2d.c:195) */
    float pml_max_f;       /* MAX_F  (fwi_sys.h:2), e.g. 15 */
    float pml_max_v;       /* MAX_V  (fwi_sys.h:3), e.g. 6000 */
    float pml_coef_r;      /* COEF_R (fwi_sys.h:4), e.g. 0.001 */
    int   device;          /* CUDA device ordinal */
    int   use_graph;       /* 1: capture the whole gradient (both time loops)
                              once and replay it as one CUDA graph */
    int   plain_per_shot;  /* 1: run shots one after another, one shot per
                              launch (the unbatched path, for comparison) */
    int   store;           /* how the backward half gets the forward field
                              (FWI_STORE_*; 0 = FWI_STORE_AUTO) */
    int   snapshots;       /* FWI_STORE_SNAPSHOTS: number of time segments,
                              i.e. checkpoints of the forward state; 0 picks
                              ceil(sqrt(nt)) */
    int   snap_precision;  /* FWI_SNAP_F32 (0), FWI_SNAP_F16, FWI_SNAP_BF16:
                              storage type of the checkpointed pressure fields */
    int   hbm_budget_mb;   /* FWI_STORE_AUTO: device memory (MiB) the shot state
                              may take; 0 = 90% of the free memory when
                              fwi_set_shots runs */
    int   fd_order;        /* 0 or 4: the reference's staggered 4th order
                              (fwi_sys.h:7, coefficients fwi_2d.c:304-314);
                              8: the 8th-order extension (see below) */
    int   reserved[1];     /* must be zero */
} fwi_config;

/* The 8th-order extension (fd_order 8; the reference has none).  A staggered
 * first difference uses the 8th-order stencil
 *     D+ at position j: sum_k w_k (a[j+k-1] - a[j-k]),   4 <= j <= n-4,
 *     D- at cell i:     sum_k w_k (b[i+k] - b[i-k+1]),   3 <= i <= n-4,
 * w = (1225/1024, -245/3072, 49/5120, -5/7168) / h, wherever its 8 points
 * lie inside the grid, and the reference's formulas of a_lap_opt_2d_pml
 * (the 4th-order pair, the edge and free-surface rows) elsewhere; the CPML
 * psi recursions are the reference's.  The rebuild keeps 2M-1 = 7 strips per
 * side.  The CFL check uses sum |w_k| = 1.2863. */

/* Forward-field storage for the backward half.
 *
 * FWI_STORE_STRIPS: the reference's boundary saving (write_bdr / read_bdr,
 *   fwi_2d.c:882-960): the 2M-1 = 3 outer rows and columns of the physical
 *   field of every step, an HBM ring of nt slots per shot in place of the
 *   reference's nt_mem-chunked temp files (header.h:24).  The backward rebuilds
 *   the source field in reverse time from them.
 * FWI_STORE_SNAPSHOTS: checkpointing.  The time axis is cut into `snapshots`
 *   segments of seg = ceil(nt/snapshots) steps; the forward pass keeps a
 *   checkpoint of the forward state (p at two time levels and the CPML psi
 *   memory) at every segment start and the strips of the last segment only.
 *   The backward takes the segments last to first: it restores the segment's
 *   checkpoint, recomputes the segment's forward steps into a strip ring of
 *   seg + 2 slots, and rebuilds and images the segment from it.  Device
 *   memory: (snapshots - 2) checkpoints plus seg + 2 strip slots per shot
 *   instead of nt strip slots; cost: one more forward pass.  FWI_SNAP_F32
 *   checkpoints are exact copies; the gradient then differs from
 *   FWI_STORE_STRIPS by FP32 rounding only, because the reverse-time rebuild
 *   restarts from recomputed fields at every segment instead of running
 *   through the whole record.  With FWI_SNAP_F16 / FWI_SNAP_BF16 a
 *   checkpoint holds p^{t_a} and the difference p^{t_a} - p^{t_a - 1}, each
 *   scaled by its own per-checkpoint, per-shot absmax factor (the psi memory
 *   stays FP32); the stencil arithmetic stays FP32.
 * FWI_STORE_AUTO: the strip ring when the shot state fits hbm_budget_mb,
 *   else snapshots with the segment count that needs the least memory (in
 *   the storage type snap_precision); FWI_ERR_NOMEM when neither fits. */
#define FWI_STORE_AUTO 0
#define FWI_STORE_STRIPS 1
#define FWI_STORE_SNAPSHOTS 2
#define FWI_SNAP_F32 0
#define FWI_SNAP_F16 1
#define FWI_SNAP_BF16 2

/* One shot.  Positions are metres, converted to cells as fwi_init does:
 * ix = round(x/dx), iz = round(z/dz - 0.5) (fwi_2d.c:363-371). */
typedef struct fwi_shot {
    int          nt;       /* time steps, 1 <= nt <= nt_max, (nt-1) % jump == 0 */
    int          nr;       /* receivers (may differ between shots) */
    float        src_x, src_z;
    const float *rec_xz;   /* [nr][2] receiver (x, z), like sr_location files (fwi_2d.c:343) */
    const float *wavelet;  /* [nt] source wavelet (sou->wav0, fwi_2d.c:352) */
} fwi_shot;

typedef struct fwi_stats {
    double ms_forward;     /* device time of the last forward loop */
    double ms_backward;    /* device time of the last backward loop */
    double ms_misfit;      /* device time of the misfit/residual kernel */
    double ms_total;       /* device time of the last public call, stream order */
    double cell_steps;     /* physical cell-steps of the last gradient (x3 for fwd+rebuild+adjoint) */
    long long launches;    /* kernels launched by the last gradient */
    long long device_bytes;/* device memory held by the context */
    int store;             /* storage in use: FWI_STORE_STRIPS or FWI_STORE_SNAPSHOTS */
    int segments;          /* FWI_STORE_SNAPSHOTS: time segments (1 with strips) */
    long long store_bytes; /* device memory of the forward-field storage
                              (strip ring, or checkpoints plus segment ring) */
} fwi_stats;

typedef struct fwi_ctx fwi_ctx;

/* Creates the device context (replaces fwi_init's allocations, fwi_2d.c:139-396;
 * the CPML profile follows cpml_coe, fwi_2d.c:110-137). */
fwi_ctx *fwi_create(const fwi_config *cfg, int *status);
void     fwi_destroy(fwi_ctx *ctx);

/* Velocity model [nz][nx] (plan->model->md, MBotOpt.c:52/98).  Checks finiteness
 * and the CFL limit; builds K = v^2 dt^2 on the padded grid (model_ext,
 * fwi_2d.c:29-107). */
int fwi_set_model(fwi_ctx *ctx, const float *vel);

/* All shots of an iteration (one fwi_init per MPI rank in the reference,
 * MBotOpt.c:51).  Allocates the per-shot device state.  FWI_ERR_ARG for
 * nshots outside 1 .. 65535 (the launches put the shot in the grid's z
 * dimension) or more than 2^31 - 1 wavelet samples in the batch. */
int fwi_set_shots(fwi_ctx *ctx, int nshots, const fwi_shot *shots);

/* Observed traces, all shots concatenated, shot s as [nr_s][nt0_s]
 * (msf->obs0, fwi_2d.c:196, read at fwi_2d.c:342). */
int fwi_set_observed(fwi_ctx *ctx, const float *obs);

/* Forward half: models every shot, keeps the boundary strips for the
 * backward half, and copies the traces to syn_out (layout of obs; NULL
 * leaves them on the device). */
int fwi_forward(fwi_ctx *ctx, float *syn_out);

/* Backward half: given the adjoint sources residual (layout of obs; for the
 * L2 misfit, syn - obs), back-propagates, images and reduces over shots in
 * FP64.  grad_out [nz][nx] = dJ/dv.  Requires a preceding fwi_forward on the
 * current model. */
int fwi_backward(fwi_ctx *ctx, const float *residual, double *grad_out);

/* Whole gradient on the device: forward, misfit + residual, backward, FP64
 * reduction.  With the default L2 misfit (the missing L2norm of
 * msf_pool.h:1 / Mpar.h:68) misfit[0] = misfit[1] = 1/2 sum (syn - obs)^2
 * (msf->val[0..1], MBotOpt.c:61,88); with FWI_MISFIT_XCORR (fwi_set_misfit)
 * they are XCORR1D's misfit[0..1] (xcorr_msf.c:56-131) and the residual is
 * d misfit[1] / d syn.  grad_out [nz][nx] host, or NULL to keep it on the
 * device (fwi_grad_device). */
int fwi_gradient(fwi_ctx *ctx, double *misfit, double *grad_out);

/* fwi_set_observed followed by fwi_gradient in one call, with the upload of
 * obs (layout of fwi_set_observed) running on a copy stream beside the
 * forward phase, which does not read it; the misfit phase waits for it.
 * From page-locked host memory the copy overlaps the forward modelling; from
 * pageable memory it is staged first, as fwi_set_observed's is.  The upload
 * has completed when the call returns, on success and on error alike, so obs
 * is the caller's again; afterwards the observed traces are set as if by
 * fwi_set_observed.  One call per iteration of the reference's loop with
 * fresh data (the per-shot msf->obs0 read at fwi_2d.c:342). */
int fwi_gradient_obs(fwi_ctx *ctx, const float *obs, double *misfit, double *grad_out);

/* Misfit of fwi_gradient (the misfit pool of the reference's fwi_init,
 * fwi_2d.c:194-213, par_xcorr1d header.h:309-315). */
#define FWI_MISFIT_L2 0
#define FWI_MISFIT_XCORR 1
#define FWI_XCORR_MIDDLE 0     /* conv_how_to_slice "middle" */
#define FWI_XCORR_LEADING 1    /* conv_how_to_slice "leading" */
typedef struct {
    int kind;                  /* FWI_MISFIT_L2 or FWI_MISFIT_XCORR */
    int slice;                 /* XCORR: FWI_XCORR_MIDDLE or FWI_XCORR_LEADING */
    float offset_min;          /* XCORR: traces whose source-receiver offset (metres, from */
    float offset_max;          /* the shot geometry) lies outside [min, max] are skipped */
    int reserved[4];           /* zero */
} fwi_misfit;
/* FWI_ERR_ARG for an unknown kind or slice, or XCORR traces longer than its
 * shared-memory limit (about 11,000 samples). */
int fwi_set_misfit(fwi_ctx *ctx, const fwi_misfit *misfit);

/* Same as fwi_gradient, float gradient (plan->grad->body is float). */
int fwi_gradient_f32(fwi_ctx *ctx, double *misfit, float *grad_out);

/* Device pointer of the FP64 gradient [nz][nx] of the last backward pass. */
const double *fwi_grad_device(const fwi_ctx *ctx);

/* Orders all later work of the context on the caller's CUDA stream
 * (a cudaStream_t of the context's device; NULL restores the context's own
 * stream).  Calls still complete before they return. */
int fwi_set_stream(fwi_ctx *ctx, void *stream);

int fwi_get_stats(const fwi_ctx *ctx, fwi_stats *out);

/* ---- launch tuning (no counterpart in the reference) -------------------- */
/* What the kernels allow to be chosen at run time.  The tile is 64 x 32
 * cells per 256 threads at compile time: the staging, the thread-to-cell
 * mapping and the register budgets of the kernels are built around it.  A
 * zero field keeps the default.
 *   x_first, z_first: first padded column / row of the interior tile
 *       rectangle (the tile grid is laid from there; default the first
 *       column / row whose stencils reach no edge, CPML or strip cell,
 *       round_up(max(8, npml + 5), 4), and row 8 with a free surface); a
 *       multiple of 4 no smaller than the default.  Changing them re-lays
 *       the fields: fwi_set_tuning then discards the shots and the model,
 *       which must be set again.
 *   fwd_gen_blocks, bwd_gen_blocks: resident blocks per SM the general-tile
 *       kernels are compiled for, 3 or 4 (default 4 forward, 3 backward);
 *       bwd_gen_blocks applies to the x-general and corner classes;
 *   bwd_zgen_blocks: the same for the z-general backward class, 3 or 4
 *       (default 4);
 *   fwd_int_blocks: the interior forward kernel, 4 or 6 (default 6);
 *   bwd_int_blocks: the interior backward kernel, 3 or 4 (default 4);
 *   class_order: 1 launches the z-general class first (default), 2 the
 *       x-general class first;
 *   serial: 1 runs the general classes and the receiver sampling on the
 *       context's stream, 2 (default) on their own streams, concurrently
 *       with the interior tiles;
 *   priority: 1 (default) gives the general classes' streams the same
 *       priority as the context's stream, 2 the device's highest, so that
 *       their (longer) blocks are scheduled first as SMs free up;
 *   gen_grid: 1 (default) launches one block per general tile and shot;
 *       k = 2 .. 5 launches k - 1 blocks per SM over the general classes,
 *       split by their work, each looping over its class's tiles, so that
 *       the general work shares the SMs with the interior tiles for the
 *       whole step instead of taking the device before them. */
typedef struct fwi_tuning {
    int x_first, z_first;
    int fwd_gen_blocks, bwd_gen_blocks;
    int fwd_int_blocks, bwd_int_blocks;
    int class_order;
    int serial;
    int priority;
    int gen_grid;
    int bwd_zgen_blocks;
    int reserved[5];       /* zero */
} fwi_tuning;
/* FWI_ERR_ARG for a value outside the lists above. */
int fwi_set_tuning(fwi_ctx *ctx, const fwi_tuning *tuning);
/* The tuning in use, every field resolved (no zeros). */
int fwi_get_tuning(const fwi_ctx *ctx, fwi_tuning *out);
/* Times `steps` forward and `steps` backward time steps of the current shot
 * batch (after fwi_set_shots and fwi_set_model), captured into CUDA graphs
 * and replayed as the gradient replays its phases, and returns the average
 * device time of one step of each; the fields they compute are discarded
 * (a following fwi_backward needs a new fwi_forward).  For sweeps over
 * fwi_tuning; the 8th-order path has nothing to tune but the serial flag and
 * the priority. */
int fwi_time_steps(fwi_ctx *ctx, int steps, double *ms_forward_step, double *ms_backward_step);
const char *fwi_status_string(int status);
const char *fwi_last_error(const fwi_ctx *ctx);   /* detail of the last failure */
int fwi_version(void);

/* ---- allocation-free entry point --------------------------------------- */
/* No counterpart in the reference: an addition for callers that must not
 * allocate device memory.  Some callers cannot call cudaMalloc: their
 * device memory belongs to another allocator (a framework's memory pool
 * that owns the whole budget), or they sit in a tight loop where
 * cudaMalloc/cudaFree would stall them by synchronising the device.
 *
 * The per-trace L2 misfit of traces already on the device, as the misfit
 * step of fwi_gradient computes it, using only caller-owned buffers:
 *   residual = syn - obs          (device, ntraces x nsamples, trace-major)
 *   misfit[0] = misfit[1] = 1/2 sum residual^2   (device, 2 doubles, FP64)
 * The per-trace FP64 partial sums live in a fixed scratch array inside the
 * library (FWI_NOALLOC_MAX_TRACES doubles = 512 KB per device, held from
 * when the library is loaded until the process exits); ntraces above that
 * limit returns FWI_ERR_ARG.  Work is queued on `stream` (a cudaStream_t of
 * the current device, NULL for the default stream) and the call returns
 * without waiting.  The first call on each device looks up the scratch
 * address (cudaGetSymbolAddress, with that device current) and keeps it;
 * make that first call before any stream capture.  Later calls look the
 * address up again whenever `stream` is not being captured, so a
 * cudaDeviceReset between calls is harmless.  If a CUDA error is already
 * pending on the calling thread, the call returns FWI_ERR_CUDA without
 * launching anything and leaves that error for the caller to read.  Every
 * call on a device uses the same scratch array, so calls whose work overlaps
 * on the GPU (different streams without ordering, or other threads) race
 * and must be serialised by the caller.  Each call overwrites the scratch
 * entries it reads, so nothing needs clearing. */
#define FWI_NOALLOC_MAX_TRACES 65536
int fwi_l2_misfit_noalloc(const float *syn, const float *obs, float *residual, int ntraces, int nsamples,
                          double *misfit, void *stream);

/* ---- routines around the gradient (standalone, host buffers) ---------- */
/* Each runs on the current device, allocates its device buffers for the call
 * and returns when the result is back in host memory. */

/* grad_precond_new5 (grad_prec.c:5-52) of body[mnz][mnx] in place: clip to
 * perc * (min, max) unless perc == 0, triangle2(rectx1, rectx1, repeat1)
 * (triangle_smooth.c:70-110), zero the cells above bottom[ix],
 * triangle2(rectx2, rectx2, repeat2), scale by alpha_grad.  Bit-identical to
 * the reference.  (fwi_grad's rectz1 / rectz2 are unused by the reference.) */
int fwi_grad_precond(float *body, int mnx, int mnz, float perc, int rectx1, int repeat1, int rectx2, int repeat2,
                     float alpha_grad, const int *bottom);

/* sfbandpass (butterworth_filter.c:127-200): Butterworth low-cut at flo and
 * high-cut at fhi (Hz) of nr traces of nt samples ([nr][nt]) with sample
 * interval dt; phase != 0 filters once (minimum phase), phase == 0 forward
 * and backward with half the orders (zero phase).  Bit-identical to the
 * reference.  FWI_ERR_ARG for flo < 0 (where the reference exits) or orders
 * above 32. */
int fwi_bandpass(const float *indat, int nt, int nr, float dt, int phase, int nphi, int nplo, float fhi, float flo,
                 float *outdat);

/* XCORR1D (xcorr_msf.c:4-181) of nr traces of nt samples ([nr][nt]);
 * sr_xyz = source x, z, then receiver x, z pairs (metres); slice
 * FWI_XCORR_MIDDLE or FWI_XCORR_LEADING.  misfit[2] and res[nr][nt] as the
 * reference; the correlations are exact sums (the reference's FFTs agree to
 * their rounding). */
int fwi_xcorr1d(const float *obs, const float *syn, int nr, int nt, const float *sr_xyz, float offset_min,
                float offset_max, int slice, float *misfit, float *res);

/* ---- L-BFGS optimizer (MBotOpt.c:55-214) on the device, FP64 ----------- */
/* The reference's driver with reverse communication: the caller evaluates
 * the objective f and gradient g at the point the optimizer returns in x,
 * then passes them to fwi_lbfgs_next, which takes MBotOpt's line-search
 * decision: Armijo (f > finit + step ftol dginit -> step *= 0.5), curvature
 * (g.d < wolfe dginit -> step *= 2.1), strong curvature (g.d > -wolfe dginit
 * -> step *= 0.5), at most max_linesearch trials; after an accepted step the
 * test |g| / |x| <= epsilon, the iteration limit, the correction pair and
 * the two-loop recursion over the last min(m, k) pairs; next first step 0.2
 * for k < 4, else the mean of the last two accepted steps.  x and the state
 * are FP64; g may be a device pointer (for example fwi_grad_device). */
typedef struct {
    int m;                     /* correction pairs kept (lbfgs.h:64) */
    double epsilon;            /* |g| / |x| convergence threshold */
    int max_iterations;        /* 0: no limit */
    int max_linesearch;        /* trials per line search */
    double ftol;               /* Armijo constant */
    double wolfe;              /* curvature constant */
} fwi_lbfgs_param;             /* NULL: the reference's defaults {12, 1e-9, 8, 6, 1e-7, 0.98} (lbfgs.h:77-79) */
#define FWI_LBFGS_SUCCESS 0            /* LBFGS_SUCCESS: converged, x is the solution */
#define FWI_LBFGS_MAXLINESEARCH 1      /* LBFGSERR_MAXIMUMLINESEARCH */
#define FWI_LBFGS_MAXITERATION 2       /* LBFGSERR_MAXIMUMITERATION */
#define FWI_LBFGS_EVALUATE 3           /* evaluate f and g at x, then call fwi_lbfgs_next */
typedef struct fwi_lbfgs fwi_lbfgs;
fwi_lbfgs *fwi_lbfgs_create(long long n, const fwi_lbfgs_param *param, int *status);
void fwi_lbfgs_destroy(fwi_lbfgs *opt);
/* x [n]: in, the start point (f, g evaluated there); out, the first trial point. */
int fwi_lbfgs_begin(fwi_lbfgs *opt, double *x, double f, const double *g, int g_on_device, int *state);
/* f, g at the last trial point; x out: the next trial point (state
 * FWI_LBFGS_EVALUATE) or the final point (the other states). */
int fwi_lbfgs_next(fwi_lbfgs *opt, double *x, double f, const double *g, int g_on_device, int *state);
/* iteration k (MBotOpt's k), the current step, objective evaluations so far */
int fwi_lbfgs_info(const fwi_lbfgs *opt, int *iteration, double *step, int *evaluations);

/* ---- host-only helpers (no device needed) ------------------------------ */
/* Validates a configuration without touching a device. */
int fwi_check_config(const fwi_config *cfg);
/* CPML profile a, b on 2*npml+1 half-cell nodes; replaces cpml_coe
 * (fwi_2d.c:110-137, header.h:227) with identical FP32 results. */
int fwi_cpml_profile(int npml, float d, float dt, float max_f, float max_v, float coef_r,
                     float *a, float *b);
/* {c0x, c1x, 1/dx, c0z, c1z, 1/dz, 1/(840 dz), 1/(24 dz)} as fwi_2d.c:304-314. */
int fwi_fd_coefficients(float dx, float dz, float *out8);
/* Cell of a position in metres, as fwi_2d.c:363-364. */
int fwi_cell_of(float x, float z, float dx, float dz, int *ix, int *iz);

#ifdef __cplusplus
}
#endif
#endif /* FWI_GB300_H */
