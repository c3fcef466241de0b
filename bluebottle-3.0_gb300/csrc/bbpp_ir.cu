// bbpp_ir.cu -- FP32-inner / FP64 iterative-refinement PCG, in two forms:
// reliable updates (default, below) and restarted refinement.
//
// Restarted refinement: outer loop (FP64): r = rhs - (-A)x, stop when
// ||r|| <= tol ||rhs||.
// Inner sweep (FP32 vectors, FP64 dot accumulators across threads and CTAs):
// Jacobi PCG on (-A)d = r from d = 0 until ||r_d|| <= inner_tol ||r||, then
// x += d in FP64.  The inner sweeps reuse the FP64 method's kernels
// instantiated for float.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "bbpp_internal.h"
#include "bbpp_kernels.cuh"
#include "bbpp_fast.cuh"

using namespace bbpp;

#define CK(call)                                   \
  do {                                             \
    cudaError_t e_ = (call);                       \
    if (e_ != cudaSuccess) {                       \
      bbpp_record_error(ctx, e_, #call, __LINE__); \
      return BBPP_CUDA_ERROR;                      \
    }                                              \
  } while (0)

struct IrBuffers {
  float *r = nullptr, *d = nullptr, *rd = nullptr, *p[2] = {nullptr, nullptr}, *Ap = nullptr;
  float *rd2 = nullptr, *Ap2 = nullptr;  // second residual and Ap buffers of the fused iterations
};

void bbpp_ir_free(bbpp_ctx *ctx) {
  if (!ctx || !ctx->ir) return;
  IrBuffers *b = ctx->ir;
  cudaFree(b->r);
  cudaFree(b->d);
  cudaFree(b->rd);
  cudaFree(b->p[0]);
  cudaFree(b->p[1]);
  cudaFree(b->Ap);
  cudaFree(b->rd2);
  cudaFree(b->Ap2);
  delete b;
  ctx->ir = nullptr;
}

// x += d (FP64 accumulation of the FP32 correction, widened exactly with
// integer operations)
__global__ void k_add_correction(const Geo G, double *__restrict__ x, const float *__restrict__ d) {
  const unsigned int n = (unsigned int)G.n;
  for (unsigned int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x)
    x[c] += widen_f32(d[c]);
}

static int ensure_ir(bbpp_ctx *ctx);

// Reliable-update form: one FP32 PCG on L d = S rhs - L x; every residual
// replacement (and the confirmation of a recursive convergence) adds d into x
// in FP64, zeroes d and recomputes the residual from x in FP64.  The search
// direction is kept, so nothing of the Krylov space is lost to restarts.
static int solve_reliable(bbpp_ctx *ctx, const uint8_t *mask, const double *rhs, double *x, const bbpp_opts *o,
                          bool zero_x, bbpp_report *rep) {
  const size_t n = (size_t)ctx->G.n;
  int rc = ensure_ir(ctx);
  if (rc) return rc;
  IrBuffers *b = ctx->ir;
  DevState *st = ctx->st, *hst = ctx->hst;
  const double S = ctx->GL.S;
  if (zero_x) CK(cudaMemsetAsync(x, 0, sizeof(double) * n, ctx->stream));
  memset(hst, 0, sizeof(DevState));
  hst->tol2bb = o->tol * o->tol * (o->stop == 0 ? S : S * S);
  hst->tiny = 1e-16;
  hst->rep_d2 = o->ir_drop * o->ir_drop;
  hst->rep_maxgap = 8 * o->replace_every;
  hst->max_iter = o->max_iter;
  hst->inject = ctx->inject;
  hst->wait_ns = ctx->wait_ns;
  hst->stop = o->stop;
  hst->first = 1;
  CK(cudaMemcpyAsync(st, hst, sizeof(DevState), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemsetAsync(b->d, 0, sizeof(float) * n, ctx->stream));
  bbpp_launch_resid_s<double, float>(ctx, mask, x, rhs, b->rd, st, RES_INIT, S);
  ctx->launches += 1;
  CK(cudaGetLastError());
  bbpp_set_reliable(x, rhs);
  float *const p[2] = {b->p[0], b->p[1]};
  int it = 0;
  bool fused = ctx->fused && bbpp_tma_fused_ok(ctx);
  if (fused && !b->rd2) {
    CK(cudaMalloc(&b->rd2, sizeof(float) * n));
    CK(cudaMalloc(&b->Ap2, sizeof(float) * n));
  }
  float *const rs[2] = {b->rd, b->rd2}, *const as[2] = {b->Ap, b->Ap2};
  if (fused) fused = bbpp_tma_fused_maps(ctx, rs, as, p);
  if (fused)
    rc = bbpp_pcg_loop_fused(ctx, mask, b->r, b->d, rs, p, as, st, hst, o->replace_every,
                             o->stop == BBPP_STOP_TRUE_REL, &it);
  else
    rc = bbpp_pcg_loop<float>(ctx, mask, b->r, b->d, b->rd, p, b->Ap, st, hst, o->replace_every,
                              o->stop == BBPP_STOP_TRUE_REL, true, &it);
  bbpp_set_reliable(nullptr, nullptr);
  if (rc) return rc;  // the loop's last fold has brought x up to date
  rep->iters = it;
  rep->outer = hst->replacements;
  rep->replacements = hst->replacements;
  rep->bb = hst->bb;
  rep->rz = hst->rz_last / S;
  rep->rel_resid = hst->bb > 0 ? std::sqrt(std::max(0.0, hst->rr) / hst->bb) / S : 0.0;
  switch (hst->done) {
    case DONE_CONVERGED: rep->status = BBPP_CONVERGED; break;
    case DONE_TINY: rep->status = BBPP_TINY_RHS; break;
    case DONE_TIMEOUT: rep->status = BBPP_WAIT_TIMEOUT; break;
    case DONE_NAN: rep->status = BBPP_NAN; break;
    default: rep->status = BBPP_MAX_ITER;
  }
  // canonical bytes of the work (the reference formulation's traffic): 41
  // B/cell per FP32 iteration, 25 per FP64 residual and 12 per fold
  rep->bytes = (double)n * (41.0 * it + 37.0 * (hst->replacements + 1));
  return 0;
}

static int ensure_ir(bbpp_ctx *ctx) {
  const size_t n = (size_t)ctx->G.n;
  if (!ctx->ir) {
    IrBuffers *b = new IrBuffers();
    ctx->ir = b;
    CK(cudaMalloc(&b->r, sizeof(float) * n));
    CK(cudaMalloc(&b->d, sizeof(float) * n));
    CK(cudaMalloc(&b->rd, sizeof(float) * n));
    CK(cudaMalloc(&b->p[0], sizeof(float) * n));
    CK(cudaMalloc(&b->p[1], sizeof(float) * n));
    CK(cudaMalloc(&b->Ap, sizeof(float) * n));
  }
  return 0;
}

int bbpp_solve_ir(bbpp_ctx *ctx, const uint8_t *mask, const double *rhs, double *x, const bbpp_opts *o, bool zero_x,
                  bbpp_report *rep) {
  if (o->ir_mode == BBPP_IR_RELIABLE) return solve_reliable(ctx, mask, rhs, x, o, zero_x, rep);
  const size_t n = (size_t)ctx->G.n;
  if (!ctx->ir) {
    IrBuffers *b = new IrBuffers();
    ctx->ir = b;
    CK(cudaMalloc(&b->r, sizeof(float) * n));
    CK(cudaMalloc(&b->d, sizeof(float) * n));
    CK(cudaMalloc(&b->rd, sizeof(float) * n));
    CK(cudaMalloc(&b->p[0], sizeof(float) * n));
    CK(cudaMalloc(&b->p[1], sizeof(float) * n));
    CK(cudaMalloc(&b->Ap, sizeof(float) * n));
  }
  IrBuffers *b = ctx->ir;
  DevState *st = ctx->st, *hst = ctx->hst;          // outer state
  DevState *sti = ctx->st + 1, *hsti = ctx->hst + 1;  // inner state
  const double S = ctx->GL.S;
  if (zero_x) CK(cudaMemsetAsync(x, 0, sizeof(double) * n, ctx->stream));
  int inner_total = 0, outer = 0;
  double bb = 0, rr = 0, rz = 0;
  int status = BBPP_MAX_ITER;
  const double tol2 = o->tol * o->tol;
  for (;;) {
    // outer residual in FP64, rounded to FP32 for the inner right-hand side
    memset(hst, 0, sizeof(DevState));
    hst->stop = 1;
    hst->tiny = 1e-16;
    CK(cudaMemcpyAsync(st, hst, sizeof(DevState), cudaMemcpyHostToDevice, ctx->stream));
    // r = S rhs - L x: the inner system L d = r gives the correction in x units
    bbpp_launch_resid_s<double, float>(ctx, mask, x, rhs, b->r, st, RES_INIT, S);
    ctx->launches += 1;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(hst, st, sizeof(DevState), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    bb = hst->bb;
    rr = hst->rr / (S * S);  // unscaled (r, r) and (r, z)
    rz = hst->rz / S;
    if (bb < 1e-16) {
      status = BBPP_TINY_RHS;
      break;
    }
    const double rel2 = rr / bb;
    if (std::isnan(rel2)) {
      status = BBPP_NAN;
      break;
    }
    const bool conv = (o->stop == BBPP_STOP_REF_RZ) ? (rz <= tol2 * bb) : (rel2 <= tol2);
    if (conv) {
      status = BBPP_CONVERGED;
      break;
    }
    if (outer >= o->max_outer || inner_total > o->max_iter) {
      status = BBPP_MAX_ITER;
      break;
    }
    // inner target: reduce ||r|| by inner_tol, but never below what the outer
    // tolerance needs (plus a margin for FP32 round-off)
    double itol = o->inner_tol;
    const double need = o->tol / std::sqrt(rel2);
    if (need > itol) itol = std::min(0.5, need * 0.5);
    int rc = bbpp_pcg_init<float>(ctx, mask, b->r, b->d, b->rd, sti, hsti, itol, 1, o->max_iter, true, 1.0);
    if (rc) return rc;
    float *const p[2] = {b->p[0], b->p[1]};
    int it = 0;
    rc = bbpp_pcg_loop<float>(ctx, mask, b->r, b->d, b->rd, p, b->Ap, sti, hsti, o->replace_every, false, true, &it);
    if (rc) return rc;
    inner_total += it;
    outer++;
    k_add_correction<<<ctx->egrid, NT, 0, ctx->stream>>>(ctx->G, x, b->d);
    CK(cudaGetLastError());
    if (hsti->done == DONE_NAN) {
      status = BBPP_NAN;
      break;
    }
    if (hsti->done == DONE_TIMEOUT) {
      status = BBPP_WAIT_TIMEOUT;
      break;
    }
  }
  rep->iters = inner_total;
  rep->outer = outer;
  rep->bb = bb;
  rep->rz = rz;
  rep->rel_resid = bb > 0 ? std::sqrt(std::max(0.0, rr) / bb) : 0.0;
  rep->status = status;
  // canonical bytes of the work (the reference formulation's traffic): 41
  // B/cell per inner FP32 iteration, 25 per FP64 outer residual, 12 per
  // correction
  rep->bytes = (double)n * (41.0 * inner_total + 25.0 * (outer + 1) + 12.0 * outer);
  return 0;
}
