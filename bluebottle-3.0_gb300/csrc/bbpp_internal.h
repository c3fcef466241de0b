// bbpp_internal.h -- host-side context shared by the translation units.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <utility>
#include <vector>

#include "../../include/bbpp.h"
#include "bbpp_dev.cuh"
#include "bbpp_fast.cuh"

struct GraphKey {
  const void *mask = nullptr, *rhs = nullptr, *x = nullptr, *r = nullptr, *p0 = nullptr, *p1 = nullptr,
             *Ap = nullptr, *st = nullptr;
  int len = 0, replace_every = 0, elem = 0;
  bool rr = false;
  double bscale = 1.0;
  const void *xhi = nullptr, *rhs64 = nullptr;
  const void *r1 = nullptr, *Ap1 = nullptr;  // fused iterations: the second r and Ap buffers
  cudaStream_t stream = nullptr;
  bool operator==(const GraphKey &o) const {
    return mask == o.mask && rhs == o.rhs && x == o.x && r == o.r && p0 == o.p0 && p1 == o.p1 && Ap == o.Ap &&
           st == o.st && len == o.len && replace_every == o.replace_every && elem == o.elem && rr == o.rr &&
           bscale == o.bscale && xhi == o.xhi && rhs64 == o.rhs64 && r1 == o.r1 && Ap1 == o.Ap1 &&
           stream == o.stream;
  }
};

// One timed kernel launch: events around it, its kind and the iteration
// (1-based, within its graph or single launch) it belongs to.
struct KEv {
  cudaEvent_t a = nullptr, b = nullptr;
  int kind = 0;
  int iter = 0;
  double bytes = 0;  // algorithmic bytes of the launch
};

enum KernelKind { KK_SEARCH_SPMV = 0, KK_UPDATE, KK_AXPY, KK_RESID, KK_SEARCH_SPMV_F32, KK_UPDATE_F32,
                  KK_AXPY_F32, KK_RESID_F32, KK_FUSED_F32, KK_COUNT };

struct GraphCache {
  GraphKey key;
  cudaGraphExec_t exec = nullptr;
  int kernels = 0;          // kernel nodes per launch
  std::vector<KEv> evs;     // profiling events captured into the graph
};

struct IrBuffers;   // FP32 inner-sweep workspace (bbpp_ir.cu)
struct NetWork;     // learned-guess workspace (bbpp_net.cu)

struct bbpp_tma_state;
void *bbpp_tensor_map_encoder();  // cuTensorMapEncodeTiled, or null
bool bbpp_tma_chunks(const bbpp_ctx *ctx, int *kz, int *nzc);  // z chunking of the TMA search kernel

struct bbpp_ctx {
  bbpp_grid grid{};
  bbpp::Geo G{};       // unscaled operator (kernel-level entry points, checks)
  bbpp::GeoL GL{};     // scaled operator of the iteration kernels
  int sms = 1;
  int kz = 1;          // z planes per stencil CTA (unscaled kernels)
  dim3 sgrid;          // stencil grid (unscaled kernels)
  int fkz = 1;         // z planes per CTA of the residual kernel
  dim3 fgrid;          // grid of the residual kernel (32x16 tiles)
  int pkz[2] = {1, 1};  // z planes per CTA of the search kernel [FP32, FP64]
  dim3 pgrid[2];        // grid of the search kernel (64x16 tiles) [FP32, FP64]
  int egrid = 1;       // elementwise grid (1-D)
  size_t nparts = 0;   // capacity of partials (per sum)
  cudaStream_t own_stream = nullptr, stream = nullptr;
  bbpp::DevState *st = nullptr;  // [0]: solve, [1]: auxiliary (residual checks)
  bbpp::DevState *hst = nullptr; // pinned host mirror
  double *partials = nullptr;
  double *r = nullptr, *p[2] = {nullptr, nullptr}, *Ap = nullptr;
  double *hbuf_rhs = nullptr, *hbuf_x = nullptr;
  uint8_t *hbuf_mask = nullptr;
  cudaStream_t copy_stream = nullptr;  // the host-buffer solve's copy of x, beside its residual check
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev_copy = nullptr;
  std::vector<GraphCache> graphs;
  bool profiling = false;
  std::vector<KEv> *rec = nullptr;   // when set, launches record events here
  std::vector<KEv> free_ev;          // event pool
  int rec_iter = 0;                  // iteration tag for recorded launches
  double kms[KK_COUNT] = {0};        // accumulated device ms per kind (profiling)
  long long klaunch[KK_COUNT] = {0}; // launches per kind (profiling)
  double kbytes[KK_COUNT] = {0};     // algorithmic bytes per kind (profiling)
  long long launches = 0;            // kernels launched by the last solve
  std::string err;
  IrBuffers *ir = nullptr;
  NetWork *net = nullptr;
  bbpp_tma_state *tma = nullptr;  // launch shape and tensor maps of the TMA search kernel
  bool pdl = false;               // iteration kernels launch with a programmatic dependency
  bool rev_update = true;         // the update kernel walks the search kernel's planes in reverse
  bool l2hint = true;             // FP32 iteration: mask evict_last in L2, p / Ap / x evict_first
  bool fused = true;              // FP32 reliable-update solves: one fused kernel per iteration
  bool ff_resid = false;          // FP64 x -> FP32 r residuals in float-float arithmetic (else FP64)
  int inject = 0;                 // test hook of bbpp_debug_wait (see DevState::inject)
  long long wait_ns = 0;          // bound of device-side waits (0: one second)
  double *trace = nullptr;        // alpha / beta trace of the next solves (2 * trace_n doubles), or null
  int trace_n = 0;
};

// Launch an iteration kernel on ctx->stream; with ctx->pdl it may start while
// its predecessor drains (the kernel's pdl_sync orders it after that kernel).
template <typename... KArgs, typename... Args>
inline void bbpp_launch(const bbpp_ctx *ctx, void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem,
                        Args &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = ctx->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = ctx->pdl ? 1 : 0;
  cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

// z chunking of a kernel whose CTAs each own one of `units` columns (tiles or
// slabs) for one chunk of planes, `slots` CTAs resident at once: returns the
// number of chunks and sets *kz (planes per chunk, at least min_kz where nz
// allows).  One wave of slots / units chunks while that fills at least 90% of
// the resident CTAs.  Otherwise (at 512^3, 256 tile columns against 456 slots
// leave a single wave 56% full) the count that minimises waves x (kz + 2),
// the time of a latency-bound kernel whose CTAs take the same time per plane,
// two halo planes included.
inline int bbpp_z_chunks(long long units, int nz, long long slots, int min_kz, int *kz) {
  if (units < 1) units = 1;
  if (slots < 1) slots = 1;
  auto norm = [&](int nzc, int *k) {
    int kk = (nz + nzc - 1) / nzc;
    if (kk < min_kz && nz >= min_kz) kk = min_kz;
    *k = kk;
    return (nz + kk - 1) / kk;
  };
  long long c0 = slots / units;
  if (c0 < 1) c0 = 1;
  if (c0 > nz) c0 = nz;
  int best = norm((int)c0, kz);
  if ((double)units * best >= 0.9 * (double)slots) return best;
  double tbest = 1e300;
  for (int c = 1; c <= nz; c++) {
    int k = 0;
    const int cc = norm(c, &k);
    if (cc != c) continue;
    const long long waves = (units * cc + slots - 1) / slots;
    const double t = (double)waves * (k + 2);
    if (t < tbest) {
      tbest = t;
      best = cc;
      *kz = k;
    }
  }
  return best;
}

void bbpp_record_error(bbpp_ctx *ctx, cudaError_t e, const char *what, int line);
int bbpp_geo_init(const bbpp_grid *g, bbpp::Geo *G);
// profiling helpers (bbpp_solver.cu)
void bbpp_rec_begin(bbpp_ctx *ctx, int kind, double bytes_per_cell);
void bbpp_rec_end(bbpp_ctx *ctx);
void bbpp_rec_collect(bbpp_ctx *ctx, std::vector<KEv> &evs, int iters_done, bool release);

template <typename T>
int bbpp_pcg_loop(bbpp_ctx *ctx, const uint8_t *mask, const T *rhs, T *x, T *r, T *const p[2], T *Ap,
                  bbpp::DevState *st, bbpp::DevState *hst, int replace_every, bool confirm, bool rr, int *iters_out);
template <typename T>
int bbpp_pcg_init(bbpp_ctx *ctx, const uint8_t *mask, const T *rhs, T *x, T *r, bbpp::DevState *st,
                  bbpp::DevState *hst, double tol, int stop, int max_iter, bool zero_x, double bscale);
// r (TR) = bscale rhs - L x (scaled operator), state init mode (0) or confirm (2)
template <typename TXT, typename TR>
void bbpp_launch_resid_s(bbpp_ctx *ctx, const uint8_t *mask, TXT *x, const TXT *rhs, TR *r, bbpp::DevState *st,
                         int mode, double bscale);

// FP32-inner / FP64-refinement method (bbpp_ir.cu)
int bbpp_solve_ir(bbpp_ctx *ctx, const uint8_t *mask, const double *rhs, double *x, const bbpp_opts *o, bool zero_x,
                  bbpp_report *rep);
void bbpp_ir_free(bbpp_ctx *ctx);

void bbpp_set_reliable(double *xhi, const double *rhs);
// TMA-staged FP32 search kernel (bbpp_tma.cu)
void bbpp_tma_init(bbpp_ctx *ctx);
void bbpp_tma_free(bbpp_ctx *ctx);
size_t bbpp_tma_partials(const bbpp_ctx *ctx);
bool bbpp_tma_fused_ok(const bbpp_ctx *ctx);
bool bbpp_tma_fused_maps(bbpp_ctx *ctx, const float *const r[2], const float *const a[2], const float *const p[2]);
// FP32 PCG loop with one fused kernel per iteration (bbpp_solver.cu)
int bbpp_pcg_loop_fused(bbpp_ctx *ctx, const uint8_t *mask, const float *rhs, float *x, float *const r[2],
                        float *const p[2], float *const Ap[2], bbpp::DevState *st, bbpp::DevState *hst,
                        int replace_every, bool confirm, int *iters_out);
// the fused FP32 iteration kernel (update of the pending step + search step)
bool bbpp_tma_fused(bbpp_ctx *ctx, const uint8_t *mask, const float *rin, const float *apin, const float *pold,
                    float *rout, float *pnew, float *apout, float *x, bbpp::DevState *st);
bool bbpp_tma_search(bbpp_ctx *ctx, const uint8_t *mask, const float *r, const float *pold, float *pnew, float *Ap,
                     float *x, bbpp::DevState *st);
int bbpp_residual_async(bbpp_ctx *ctx, const uint8_t *mask, const double *rhs, const double *x, double *r);

// learned initial guess (bbpp_net.cu)
int bbpp_net_guess(bbpp_ctx *ctx, void *net, const uint8_t *mask, const double *rhs, const double *prev, double *x,
                   int coarsen, double *ms);
void bbpp_net_ctx_free(bbpp_ctx *ctx);
