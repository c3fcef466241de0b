/*
 * bbpp.h -- C ABI of the GB300-native Bluebottle pressure-Poisson solver.
 *
 * The library (libbbpp.so) solves the reference's pressure system
 *     (-A) phi = rhs
 * (src/cuda_solver.cu:60-73): (-A) is the cell-centred 7-point Laplacian with
 * per-direction periodic or homogeneous-Neumann boundaries and the Physalis
 * phase mask, which turns each solid cell into a decoupled row
 * (src/solver_kernel.cu:684-707).  The method is the reference's Jacobi PCG
 * (src/cuda_solver.cu:192-268), with residual replacement every
 * `replace_every` iterations.
 *
 * All arrays are dense, x fastest: c = i + nx*(j + ny*k).  There is no ghost
 * layer: periodic neighbours wrap on the device and wall faces drop out of the
 * stencil.  `mask` holds one byte per cell, non-zero for solid (the reference's
 * `phase > -1`); NULL selects the particle-free operator
 * (cuda_PP_cg_noparts, src/cuda_solver.cu:573).
 *
 * Every pointer argument of bbpp_solve / bbpp_spmv is a device pointer.
 * bbpp_solve_host takes host pointers and does the copies itself.
 * No function here calls exit(); errors come back as a bbpp_status.
 *
 * The drop-in symbols the Bluebottle time loop calls (cuda_PP_cg,
 * cuda_PP_cg_noparts, cuda_PP_init_jacobi_preconditioner) live in
 * libbbpp_bluebottle.so and are declared in bbpp_bluebottle.h.
 */
#ifndef BBPP_H
#define BBPP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Pressure boundary type of a face, as the reference's bc.p{W,E,S,N,B,T}
 * (src/bluebottle.h:218,242). */
#define BBPP_PERIODIC 0
#define BBPP_NEUMANN 2

typedef struct bbpp_grid {
  int nx, ny, nz;   /* interior cells (dom[rank].Gcc.in, jn, kn) */
  double dx, dy, dz;
  int bc[6];        /* W, E, S, N, B, T; each direction periodic on both or Neumann on both */
} bbpp_grid;

typedef enum bbpp_status {
  BBPP_CONVERGED = 0,  /* stopping test met */
  BBPP_TINY_RHS = 1,   /* (rhs,rhs) < 1e-16; x = guess, as src/cuda_solver.cu:180-190 */
  BBPP_MAX_ITER = 2,   /* iteration limit reached (src/cuda_solver.cu:271-279) */
  BBPP_NAN = 3,        /* (r,z) became NaN (src/cuda_solver.cu:245-251) */
  BBPP_BAD_ARG = 4,
  BBPP_CUDA_ERROR = 5,
  BBPP_NO_DEVICE = 6,
  BBPP_WAIT_TIMEOUT = 7 /* a bounded device-side wait gave up */
} bbpp_status;

typedef enum bbpp_precision {
  BBPP_FP64 = 0,     /* plain FP64 PCG (the reference's arithmetic) */
  BBPP_FP32_IR = 1   /* FP32 inner PCG, FP64 residual / solution / dot accumulators */
} bbpp_precision;

typedef enum bbpp_guess {
  BBPP_GUESS_ZERO = 0,    /* x0 = 0 (src/solver_kernel.cu:280) */
  BBPP_GUESS_GIVEN = 1,   /* start from x on entry (warm start) */
  BBPP_GUESS_LEARNED = 2  /* x0 from the learned network (bbpp_net_*) */
} bbpp_guess;

typedef enum bbpp_ir_mode {
  BBPP_IR_RELIABLE = 0,  /* one FP32 PCG run; its residual replacements fold the FP32 correction into the
                            FP64 solution and recompute the residual in FP64 (no Krylov restart) */
  BBPP_IR_RESTART = 1    /* classic refinement: an FP32 PCG per outer FP64 residual, restarted each sweep */
} bbpp_ir_mode;

typedef enum bbpp_stop {
  BBPP_STOP_REF_RZ = 0,   /* (r,z) <= tol^2 (rhs,rhs): the reference rule (src/cuda_solver.cu:235) */
  BBPP_STOP_TRUE_REL = 1  /* ||rhs-(-A)x|| / ||rhs|| <= tol, confirmed with an explicit residual */
} bbpp_stop;

typedef struct bbpp_opts {
  int precision;      /* bbpp_precision */
  int guess;          /* bbpp_guess */
  int stop;           /* bbpp_stop */
  double tol;         /* pp_residual (REF_RZ) or relative residual (TRUE_REL) */
  int max_iter;       /* pp_max_iter; at most max_iter+1 iterations, as the reference */
  int replace_every;  /* explicit residual every n iterations (50 in the reference) */
  double inner_tol;   /* FP32_IR restart mode: relative residual reduction per sweep */
  int max_outer;      /* FP32_IR restart mode: refinement sweeps */
  void *net;          /* GUESS_LEARNED: a bbpp_net handle */
  const double *prev; /* GUESS_LEARNED: previous pressure (device), may be NULL */
  int ir_mode;        /* FP32_IR: bbpp_ir_mode */
  double ir_drop;     /* FP32_IR reliable mode: a checkpoint (every replace_every iterations) replaces the
                         residual once ||r|| has dropped by this factor since the last replacement (and at
                         least every 8 checkpoints); 0 = at every checkpoint.  Default 1e-2. */
  int net_coarsen;    /* GUESS_LEARNED: the network runs on the grid coarsened by this factor, 1 (the
                         grid itself), 2 or 4 (the means of FxFxF cells, every extent a multiple of
                         4F; the correction comes back by trilinear interpolation); 0 (default) = 2
                         when every extent is a multiple of 8 and at least 128, else 1 */
} bbpp_opts;

typedef struct bbpp_report {
  int status;         /* bbpp_status */
  int iters;          /* PCG iterations (all inner iterations for FP32_IR) */
  int outer;          /* FP32_IR refinement sweeps (0 for FP64) */
  int replacements;   /* explicit residual evaluations */
  double bb;          /* (rhs, rhs) */
  double rz;          /* final (r, z) */
  double rel_resid;   /* final recursive ||r|| / ||rhs|| */
  double true_rel;    /* ||rhs - (-A)x|| / ||rhs|| computed after the solve */
  double ms;          /* device time of the solve (CUDA events on the solver stream) */
  double guess_ms;    /* part of ms spent producing the learned guess */
  double bytes;       /* algorithmic HBM bytes moved (see the roofline notes) */
  int launches;       /* kernels launched by the solve (library kernels only) */
} bbpp_report;

typedef struct bbpp_ctx bbpp_ctx;

/* Context: owns the device workspace for one grid, one CUDA stream. */
int bbpp_create(const bbpp_grid *g, bbpp_ctx **out);
int bbpp_destroy(bbpp_ctx *ctx);
/* Use an external stream (cudaStream_t passed as void*); NULL = own stream. */
int bbpp_set_stream(bbpp_ctx *ctx, void *stream);
void bbpp_default_opts(bbpp_opts *o);
const char *bbpp_status_str(int status);
/* Last CUDA error text recorded by the context (or "" if none). */
const char *bbpp_last_error(const bbpp_ctx *ctx);

/* Solve (-A)x = rhs.  mask, rhs, x: device pointers (mask may be NULL). */
int bbpp_solve(bbpp_ctx *ctx, const uint8_t *mask, const double *rhs, double *x,
               const bbpp_opts *o, bbpp_report *rep);
/* Same with host pointers; the copies are inside the call. */
int bbpp_solve_host(bbpp_ctx *ctx, const uint8_t *mask, const double *rhs, double *x,
                    const bbpp_opts *o, bbpp_report *rep);

/* Kernel-level entry points (device pointers), used for parity checks. */
int bbpp_spmv(bbpp_ctx *ctx, const uint8_t *mask, const double *p, double *Ap);
int bbpp_invm(bbpp_ctx *ctx, double *invM);
/* The pressure right-hand side from the intermediate velocity, as PP_rhs (src/solver_kernel.cu:89-176):
 * rhs = -(rho_f/dt) div(u*, v*, w*) on every cell.  Dense device arrays: faces
 * u[i + (nx+1)(j + ny k)], v[i + nx(j + (ny+1) k)], w[i + nx(j + ny k)] (k = 0..nz); rhs as the cells. */
int bbpp_rhs_div(bbpp_ctx *ctx, double rho_f, double dt, const double *u, const double *v, const double *w,
                 double *rhs);
/* One launch of the PCG search kernel on caller vectors, on the scaled operator L = S(-A) with
 * S = 1 / (2/dx^2 + 2/dy^2 + 2/dz^2) (kernel-level checks; no counterpart in the reference, whose
 * PP_update_search + PP_spmv_shared_load + (p, Ap) in src/solver_kernel.cu:528-713,906-927 it fuses).
 * precision BBPP_FP64 (double vectors) or BBPP_FP32_IR (float vectors); kernel 0 = the solver's
 * choice, 1 = the z-marching tile kernel, 2 = the TMA-staged kernel (FP32 only; BBPP_BAD_ARG when the
 * grid does not suit it).  p_new = z + beta p_old (first: p_new = z), z = r / diag(L); Ap = L p_new
 * (0 on solid cells); x += alpha p_old when lag; *pAp = (p_new, Ap). */
int bbpp_search_step(bbpp_ctx *ctx, int precision, int kernel, const uint8_t *mask, const void *r, const void *pold,
                     void *pnew, void *Ap, void *x, double beta, double alpha, int first, int lag, double *pAp);
/* Residual: r = rhs - (-A)x; also returns (r,r) and (rhs,rhs). */
int bbpp_residual(bbpp_ctx *ctx, const uint8_t *mask, const double *rhs, const double *x,
                  double *r, double *rr, double *bb);

/* The residual of bbpp_residual without a context and without allocating:
 * for callers that cannot allocate device memory while they run (all buffers
 * sized at start-up, a fixed device-memory budget, or a loop that must not
 * call the allocator).  No counterpart in the reference.  Reduction scratch
 * is a static device array holding one state and BBPP_NOALLOC_MAX_CTAS x 3
 * partial sums (~200 KB per GPU, kept until exit); grids needing more than
 * BBPP_NOALLOC_MAX_CTAS column tiles of 32x8 cells are rejected
 * (BBPP_BAD_ARG).  Calls share that scratch: calls overlapping on the GPU
 * race.  Every call looks up the scratch's device address in the context
 * current at the time (so a cudaDeviceReset between calls is harmless); the
 * first call on a device also loads the library's device code and should
 * come before any stream capture.  The call waits for its stream before it
 * returns (the two norms are copied to the host).  mask/rhs/x/r are device
 * pointers; stream is a cudaStream_t or NULL.  rr, bb receive (r,r) and
 * (rhs,rhs). */
#define BBPP_NOALLOC_MAX_CTAS 8192
int bbpp_residual_noalloc(const bbpp_grid *g, const uint8_t *mask, const double *rhs,
                          const double *x, double *r, double *rr, double *bb, void *stream);

/* Phase mask of spheres, on the device (src/particle_kernel.cu:148-253):
 * cell (i,j,k) is solid when floor(d/r) < 1, d the distance of its centre
 * ((i+0.5)dx + xs, ...) from a sphere centre; periodic directions also test
 * the images at +-length.  Sphere arrays are host pointers. */
int bbpp_sphere_mask(bbpp_ctx *ctx, double xs, double ys, double zs, int nsph,
                     const double *cx, const double *cy, const double *cz,
                     const double *rad, uint8_t *mask);

/* Device memory helpers for callers without their own allocator. */
int bbpp_dev_alloc(size_t bytes, void **ptr);
int bbpp_dev_free(void *ptr);
int bbpp_h2d(void *dst, const void *src, size_t bytes);
int bbpp_d2h(void *dst, const void *src, size_t bytes);
int bbpp_memset(void *dst, int value, size_t bytes);
int bbpp_sync(void);
/* Fill a buffer larger than L2 to evict cached lines between timed runs. */
int bbpp_flush_l2(void);
/* FP64 fused multiply-adds per second this GPU issues (eight independent FMA
 * chains per thread, a full wave, best of three timed launches): the peak the
 * plain FP64 solve's roofline is reported against.  No counterpart in the
 * reference. */
int bbpp_fp64_fma_rate(double *fma_per_s);
/* Bytes per second a plain streaming kernel reaches with the fused FP32
 * iteration's per-cell traffic over `cells` cells (four FP32 reads, one mask
 * byte, four FP32 writes: 33 B/cell; L2 flushed before each of five timed
 * launches, the best kept).  Allocates its buffers (about 33 B per cell) for
 * the measurement.  No counterpart in the reference. */
int bbpp_stream_mix_rate(long long cells, double *bytes_per_s);
/* The z chunking the stencil kernels launch with (host arithmetic only): for
 * `units` CTA columns (tiles or slabs) per plane, nz planes and `slots` CTAs
 * resident at once, returns the number of z-chunks and sets *kz to the planes
 * per chunk (at least min_kz where nz allows).  One wave of slots / units
 * chunks when that fills at least 90% of the slots; otherwise the count that
 * minimises waves x (kz + 2).  Returns 0 on bad arguments. */
int bbpp_plan_z_chunks(long long units, int nz, long long slots, int min_kz, int *kz);
/* out[i] = the FP64 search kernel's neighbour sum of in[6i .. 6i+5] (host
 * buffers, n <= 2^26): the fixed-point sum, or FP64 adds where all six are
 * zero or tiny or one is not finite.  For tests of that arithmetic. */
int bbpp_neighbour_sums(const double *in, double *out, long long n);
/* The same arithmetic compiled for the host, on host buffers (no GPU). */
int bbpp_neighbour_sums_host(const double *in, double *out, long long n);
/* Page-locked host memory (for end-to-end timing from pinned buffers). */
int bbpp_host_alloc(size_t bytes, void **ptr);
int bbpp_host_free(void *ptr);

/* Per-kernel-kind device time accumulated since bbpp_set_profiling(ctx, 1):
 * launches that did work, their summed CUDA-event ms and algorithmic bytes.
 * Kinds: search_spmv, update, axpy_x, resid (and _f32 variants). */
typedef struct bbpp_kstat {
  char name[32];
  int launches;
  double ms;
  double bytes;
} bbpp_kstat;
int bbpp_kernel_stats(bbpp_ctx *ctx, bbpp_kstat *out, int max, int *n);
/* Enable (1) or disable (0) per-kernel CUDA-event timing and reset the
 * counters; events are captured between the kernels of the graphs. */
int bbpp_set_profiling(bbpp_ctx *ctx, int on);
/* The FP32 iteration of reliable-update solves: 1 = one fused kernel per
 * iteration (the default where the TMA kernels take the grid), 0 = a search
 * kernel and an update kernel. */
int bbpp_set_fused(bbpp_ctx *ctx, int on);
/* The outer residuals of the reliable updates (FP64 x into the FP32
 * residual): 0 = FP64 arithmetic (the default), 1 = float-float arithmetic on
 * the FP32 pipe (about 48 bits). */
int bbpp_set_ff_resid(bbpp_ctx *ctx, int on);
/* FP64 stencils on a grid with dx = dy = dz (the plain iteration's search
 * kernel and the FP64 residuals of both methods): 1 = each interior cell's
 * six-neighbour sum as an exact fixed-point sum on the integer pipe, rounded
 * once (the default; within 1/2 ulp plus ulp(max)/128 of the exact sum),
 * 0 = five FP64 adds.  No counterpart in the reference, whose stencil adds in
 * FP64 (src/solver_kernel.cu:691-707). */
int bbpp_set_xsum(bbpp_ctx *ctx, int on);
/* Record alpha_k and beta_k of the first n iterations of the following plain
 * FP64 solves (n = 0: stop; at most 2^20); bbpp_get_trace copies them out,
 * NaN where a solve ended earlier.  For comparing the iteration with the
 * reference's (src/cuda_solver.cu:205-243); no counterpart there. */
int bbpp_set_trace(bbpp_ctx *ctx, int n);
int bbpp_get_trace(bbpp_ctx *ctx, double *alpha, double *beta, int n);

/* ---- learned initial guess (no counterpart in the reference) ----
 * A 3-level 3D conv encoder-decoder (channels 16/32/64, 3x3x3 kernels, BF16
 * activations and tensor-core convolutions with FP32 accumulation, FP32
 * master weights, Adam) that maps (rhs, previous pressure, phase mask) to an
 * initial guess p0.  Volumes need sizes divisible by 4; padding is periodic in
 * x and y and zero in z.  All array arguments are device pointers. */
typedef struct bbpp_net bbpp_net;
int bbpp_net_create(unsigned long long seed, bbpp_net **out);
int bbpp_net_destroy(bbpp_net *net);
int bbpp_net_num_params(const bbpp_net *net);
int bbpp_net_get_params(const bbpp_net *net, float *host);
int bbpp_net_set_params(bbpp_net *net, const float *host);
/* The network predicts the correction to the previous pressure p_prev from
 * r = rhs - (-A) p_prev, p_prev and the mask: p0 = p_prev + h2 out / (1/s_r),
 * s_r the fluid RMS of r.  Loss: mean over fluid cells of
 * (out - target / (s_r h2))^2 with target = p* - p_prev; gradient to a host
 * array of num_params floats (may be NULL) for nb stacked volumes. */
int bbpp_net_loss_grad(bbpp_net *net, int nx, int ny, int nz, int nb, double h2, const float *r,
                       const float *prev, const float *target, const uint8_t *mask, double *loss,
                       float *grads_host);
/* Adam training on nsamples device-resident volumes (batches drawn by Ranq1). */
int bbpp_net_train(bbpp_net *net, int nx, int ny, int nz, int nsamples, double h2, const float *r,
                   const float *prev, const float *target, const uint8_t *mask, int steps, int batch,
                   float lr, unsigned long long seed, float *loss_hist_host);
/* p0 (FP64) from r and p_prev (FP64, p_prev may be NULL: then r = rhs). */
int bbpp_net_infer(bbpp_net *net, int nx, int ny, int nz, double h2, const double *r, const double *prev,
                   const uint8_t *mask, double *p0);
int bbpp_net_set_stream(bbpp_net *net, void *stream);
int bbpp_net_save(const bbpp_net *net, const char *path);
int bbpp_net_load(bbpp_net *net, const char *path);
/* One 3x3x3 convolution on BF16 channels-last volumes (w: [27][cout][cin]);
 * the weight gradient dW += sum_v g[v]^T in[v + tap] (FP32 [27][cout][cin]);
 * and the flipped transpose of w used for the input gradient. */
int bbpp_conv3(int cin, int cout, const void *in, int ldi, int ci_off, const void *w, const float *bias,
               void *out, int ldo, int co_off, int nx, int ny, int nz, int nb, int px, int py, int pz, int relu);
int bbpp_conv3_wgrad(int cin, int cout, const void *in, int ldi, int ci_off, const void *g, int ldg, float *dW,
                     int nx, int ny, int nz, int nb, int px, int py, int pz);
int bbpp_conv3_wflip(int cin, int cout, const void *w, void *wt);
/* Convolutions run so far on a tcgen05 (tensor-memory) kernel.  With the
 * default choice, forward layers with 16 or 32 outputs on rows of 128 voxels
 * (or 16 outputs on rows of 256) take it; the others take the mma.sync kernel. */
long long bbpp_conv3_tc_launches(void);
/* Choose the forward convolution kernel: 0 mma.sync; 1 tcgen05 with x-shifted
 * A tiles in tensor memory; 2 tcgen05 with the three x-taps stacked in N
 * (the default: rows of 128 voxels, or 256 with 16 output channels; other
 * widths take mma.sync); -1 leaves the choice to the environment
 * (BBPP_CONV_TC=0, 1 or 2; 2 when unset).
 * Caps the persistent grid at max_ctas CTAs (0: one per SM). */
int bbpp_conv3_tc_config(int enable, int max_ctas);

/* Ranq1 generator (src/rng.c:25-107), for reproducible synthetic inputs. */
void bbpp_rng_uniform(unsigned long long seed, long long n, double lo, double hi, double *out);
void bbpp_rng_gauss(unsigned long long seed, long long n, double *out);

/* Library version string. */
const char *bbpp_version(void);
/* Failure-detection test hook (no counterpart in the reference): set the bound of the solver's device-side
 * waits (wait_ns > 0; 0 restores one second) and, with inject, make the next FP32 solves' TMA search kernel
 * leave one plane's copies unissued in its first CTA, so that the wait for them runs out and the solve
 * returns BBPP_WAIT_TIMEOUT.  Nothing faults or hangs; the context stays usable. */
int bbpp_debug_wait(bbpp_ctx *ctx, long long wait_ns, int inject);
/* Select the GPU for this host thread's later contexts and buffers (one process per GPU; no counterpart in
 * the reference, whose ranks each own one GPU through cudaSetDevice in its start-up code). */
int bbpp_set_device(int device);

#ifdef __cplusplus
}
#endif
#endif /* BBPP_H */
