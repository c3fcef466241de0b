// bbpp_solver.cu -- host side of the C ABI (include/bbpp.h): context,
// launch shapes, CUDA-graph chunks of PCG iterations, and the solve loop.
//
// The iteration (src/cuda_solver.cu:192-268) runs as a captured graph of
// `chunk` iterations: [K1, K2] per iteration, with the replacement iteration
// (q % replace_every == 0) as [K1, x += alpha p, r = rhs - (-A)x].  Kernels
// return at once when the device state says the solve is done, so the host
// reads the state only once per chunk.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/bbpp.h"
#include "bbpp_internal.h"
#include "bbpp_kernels.cuh"
#include "bbpp_fast.cuh"

using namespace bbpp;

#define CK(call)                                                    \
  do {                                                              \
    cudaError_t e_ = (call);                                        \
    if (e_ != cudaSuccess) {                                        \
      bbpp_record_error(ctx, e_, #call, __LINE__);                  \
      return BBPP_CUDA_ERROR;                                       \
    }                                                               \
  } while (0)

static char g_err[512];

void bbpp_record_error(bbpp_ctx *ctx, cudaError_t e, const char *what, int line) {
  char buf[512];
  snprintf(buf, sizeof(buf), "%s (%s) at bbpp_solver.cu:%d: %s", cudaGetErrorName(e), cudaGetErrorString(e), line,
           what);
  if (ctx) ctx->err = buf;
  snprintf(g_err, sizeof(g_err), "%s", buf);
}

// --------------------------------------------------------------- geometry --
static unsigned long long div_magic(unsigned int d) {
  if (d <= 1) return 0ull;
  // ceil(2^64 / d) = floor((2^64 - 1) / d) + 1 for d > 1
  return (~0ull) / d + 1ull;
}

int bbpp_geo_init(const bbpp_grid *g, Geo *G) {
  if (!g || g->nx < 1 || g->ny < 1 || g->nz < 1) return BBPP_BAD_ARG;
  if (!(g->dx > 0) || !(g->dy > 0) || !(g->dz > 0)) return BBPP_BAD_ARG;
  for (int f = 0; f < 6; f++)
    if (g->bc[f] != BBPP_PERIODIC && g->bc[f] != BBPP_NEUMANN) return BBPP_BAD_ARG;
  if (g->bc[0] != g->bc[1] || g->bc[2] != g->bc[3] || g->bc[4] != g->bc[5]) return BBPP_BAD_ARG;
  const long long n = (long long)g->nx * g->ny * g->nz;
  if (n >= (1ll << 31)) return BBPP_BAD_ARG;
  memset(G, 0, sizeof(*G));
  G->nx = g->nx;
  G->ny = g->ny;
  G->nz = g->nz;
  G->px = g->bc[0] == BBPP_PERIODIC;
  G->py = g->bc[2] == BBPP_PERIODIC;
  G->pz = g->bc[4] == BBPP_PERIODIC;
  G->n = n;
  const double idx2 = 1. / (g->dx * g->dx), idy2 = 1. / (g->dy * g->dy), idz2 = 1. / (g->dz * g->dz);
  G->cx = idx2;
  G->cy = idy2;
  G->cz = idz2;
  const double pfx = -(g->dx * g->dx) / 6., pfy = -(g->dy * g->dy) / 6., pfz = -(g->dz * g->dz) / 6.;
  for (int wz = 0; wz < 3; wz++)
    for (int wy = 0; wy < 3; wy++)
      for (int wx = 0; wx < 3; wx++) {
        const int cls = wx + 3 * wy + 9 * wz;
        const int fx = 2 - wx, fy = 2 - wy, fz = 2 - wz;  // faces present
        // M as in PP_jacobi_init (src/solver_kernel.cu:72-80)
        const double M = -idx2 * fx - idy2 * fy - idz2 * fz;
        G->tab[cls] = -M;
        G->tab[27 + cls] = (M != 0.) ? -1. / M : 0.;
        // solid row: sum_d idd2 * pf_d * (faces), src/solver_kernel.cu:684-707
        G->tab[54 + cls] = idx2 * pfx * fx + idy2 * pfy * fy + idz2 * pfz * fz;
      }
  G->mx = div_magic((unsigned)g->nx);
  G->mxy = div_magic((unsigned)(g->nx * g->ny));
  return 0;
}

// Scaled operator L = S (-A), S = 1 / (fluid interior diagonal).
static void geol_init(const Geo &G, GeoL *L) {
  memset(L, 0, sizeof(*L));
  L->nx = G.nx;
  L->ny = G.ny;
  L->nz = G.nz;
  L->px = G.px;
  L->py = G.py;
  L->pz = G.pz;
  L->n = G.n;
  L->mx = G.mx;
  L->mxy = G.mxy;
  const double S = 1.0 / G.tab[0];
  L->S = S;
  L->ax = S * G.cx;
  L->ay = S * G.cy;
  L->az = S * G.cz;
  L->iso = (L->ax == L->ay && L->ay == L->az);
  for (int c = 0; c < 27; c++) {
    L->dL[c] = (c == 0) ? 1.0 : S * G.tab[c];
    L->invL[c] = (c == 0) ? 1.0 : (L->dL[c] != 0 ? 1.0 / L->dL[c] : 0.0);
    L->fdL[c] = (float)L->dL[c];
    L->finvL[c] = (float)L->invL[c];
  }
  L->fax = (float)L->ax;
  L->fay = (float)L->ay;
  L->faz = (float)L->az;
}

namespace bbpp {
struct Sphere {
  double x, y, z, w;
};

// invM per cell (PP_jacobi_init, src/solver_kernel.cu:26-87)
__global__ void k_invm(const Geo G, double *invM) {
  const unsigned int n = (unsigned int)G.n;
  for (unsigned int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    const unsigned int row = fdiv(c, G.mx);
    const unsigned int k = fdiv(c, G.mxy);
    const int i = (int)(c - row * (unsigned)G.nx);
    const int j = (int)(row - k * (unsigned)G.ny);
    invM[c] = G.tab[27 + wall_class(G, i, j, (int)k)];
  }
}

// Sphere phase mask (build_phase, src/particle_kernel.cu:148-253).  One CTA
// per (sphere, periodic image) walks the image's bounding box and marks the
// cells whose centre satisfies floor(d/r) < 1.  The mask must be zeroed first.
// Products and sums use round-to-nearest intrinsics (no FMA contraction) so
// the result is bit-identical to the host restatement.
__global__ void k_sphere_mask(const Geo G, double dx, double dy, double dz, double xs, double ys,
                              double zs, int nimg_x, int nimg_y, int nimg_z,
                              const Sphere *__restrict__ sph, uint8_t *mask) {
  const int nimg = nimg_x * nimg_y * nimg_z;
  const int s = blockIdx.x / nimg;
  int im = blockIdx.x - s * nimg;
  const int ox = (nimg_x == 3) ? (im % 3) - 1 : 0;
  im /= nimg_x;
  const int oy = (nimg_y == 3) ? (im % 3) - 1 : 0;
  im /= nimg_y;
  const int oz = (nimg_z == 3) ? im - 1 : 0;
  const Sphere S = sph[s];
  const double irad = 1.0 / S.w;
  const double X = __dadd_rn(S.x, __dmul_rn((double)ox, __dmul_rn((double)G.nx, dx)));
  const double Y = __dadd_rn(S.y, __dmul_rn((double)oy, __dmul_rn((double)G.ny, dy)));
  const double Z = __dadd_rn(S.z, __dmul_rn((double)oz, __dmul_rn((double)G.nz, dz)));
  int i0 = (int)floor(__ddiv_rn(__dsub_rn(__dsub_rn(X, xs), S.w), dx)) - 1;
  int i1 = (int)ceil(__ddiv_rn(__dadd_rn(__dsub_rn(X, xs), S.w), dx)) + 1;
  int j0 = (int)floor(__ddiv_rn(__dsub_rn(__dsub_rn(Y, ys), S.w), dy)) - 1;
  int j1 = (int)ceil(__ddiv_rn(__dadd_rn(__dsub_rn(Y, ys), S.w), dy)) + 1;
  int k0 = (int)floor(__ddiv_rn(__dsub_rn(__dsub_rn(Z, zs), S.w), dz)) - 1;
  int k1 = (int)ceil(__ddiv_rn(__dadd_rn(__dsub_rn(Z, zs), S.w), dz)) + 1;
  i0 = max(i0, 0); j0 = max(j0, 0); k0 = max(k0, 0);
  i1 = min(i1, G.nx - 1); j1 = min(j1, G.ny - 1); k1 = min(k1, G.nz - 1);
  if (i1 < i0 || j1 < j0 || k1 < k0) return;
  const int bx = i1 - i0 + 1, by = j1 - j0 + 1, bz = k1 - k0 + 1;
  const int nbox = bx * by * bz;
  const double Xs = __dsub_rn(X, xs), Ys = __dsub_rn(Y, ys), Zs = __dsub_rn(Z, zs);
  for (int e = threadIdx.x; e < nbox; e += blockDim.x) {
    const int li = e % bx, t = e / bx;
    const int lj = t % by, lk = t / by;
    const int i = i0 + li, j = j0 + lj, k = k0 + lk;
    const double xx = __dsub_rn(__dmul_rn((double)(i + 1) - 0.5, dx), Xs);
    const double yy = __dsub_rn(__dmul_rn((double)(j + 1) - 0.5, dy), Ys);
    const double zz = __dsub_rn(__dmul_rn((double)(k + 1) - 0.5, dz), Zs);
    const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(xx, xx), __dmul_rn(yy, yy)), __dmul_rn(zz, zz));
    const double d = __dsqrt_rn(d2);
    if (floor(__dmul_rn(d, irad)) < 1.0) mask[i + (long long)G.nx * (j + (long long)G.ny * k)] = 1;
  }
}

}  // namespace bbpp

// ---------------------------------------------------------------- context --
static int dev_sms() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 1;
}

static void stencil_shape(bbpp_ctx *ctx) {
  const Geo &G = ctx->G;
  const int gx = (G.nx + TX - 1) / TX, gy = (G.ny + TY - 1) / TY;
  // enough CTAs for one full wave of resident CTAs, each marching kz planes
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_resid<double, double, true>, NT, 0);
  if (per_sm < 1) per_sm = 1;
  // at least 4 planes per chunk keeps the halo-plane overhead small
  int kz = 0;
  const int nzc = bbpp_z_chunks((long long)gx * gy, G.nz, (long long)ctx->sms * per_sm, 4, &kz);
  ctx->kz = kz;
  ctx->sgrid = dim3(gx, gy, nzc);
  {
    const int fx = (G.nx + FX - 1) / FX, fy = (G.ny + FY - 1) / FY;
    int pf = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pf, k_resid_s<double, double, true, true>, FNT, 0);
    if (pf < 1) pf = 1;
    int kzf = 0;
    const int nzf = bbpp_z_chunks((long long)fx * fy, G.nz, (long long)ctx->sms * pf, 8, &kzf);
    ctx->fkz = kzf;
    ctx->fgrid = dim3(fx, fy, nzf);
  }
  for (int prec = 0; prec < 2; prec++) {
    // one full wave of resident CTAs of the search kernel of this precision
    const int fx = (G.nx + PX - 1) / PX, fy = (G.ny + PY - 1) / PY;
    int pf = 0;
    if (prec)
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pf, k1_search2<double, true, true>, FNT, 0);
    else
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pf, k1_search2<float, true, true>, FNT, 0);
    if (pf < 1) pf = 1;
    int kzf = 0;
    const int nzf = bbpp_z_chunks((long long)fx * fy, G.nz, (long long)ctx->sms * pf, 8, &kzf);
    ctx->pkz[prec] = kzf;
    ctx->pgrid[prec] = dim3(fx, fy, nzf);
  }
  int per_sm2 = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm2, k_settle<double>, FNT, 0);
  if (per_sm2 < 1) per_sm2 = 1;
  long long eb = std::min<long long>((G.n + NT - 1) / NT, (long long)ctx->sms * per_sm2);
  ctx->egrid = (int)std::max<long long>(1, eb);
}

extern "C" int bbpp_create(const bbpp_grid *g, bbpp_ctx **out) {
  if (!out) return BBPP_BAD_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    snprintf(g_err, sizeof(g_err), "no CUDA device");
    return BBPP_NO_DEVICE;
  }
  bbpp_ctx *ctx = new bbpp_ctx();
  int rc = bbpp_geo_init(g, &ctx->G);
  if (rc) {
    delete ctx;
    return rc;
  }
  ctx->grid = *g;
  geol_init(ctx->G, &ctx->GL);
  ctx->sms = dev_sms();
  stencil_shape(ctx);
  bbpp_tma_init(ctx);
  {
    // programmatic dependent launch of the iteration kernels: off unless
    // BBPP_PDL=1 (measured at 256^3: no gain, the kernels' own drain and fill
    // dominate the launch latency it hides)
    const char *e = getenv("BBPP_PDL");
    ctx->pdl = e && e[0] == '1';
    // the update kernel's reversed plane order (BBPP_REV_UPDATE=0: ascending)
    const char *ru = getenv("BBPP_REV_UPDATE");
    ctx->rev_update = !(ru && ru[0] == '0');
    // L2 eviction priorities of the FP32 iteration (BBPP_L2HINT=0: none).
    // Measured at 256^3: the mask kept (evict_last) and p, Ap, x streamed
    // (evict_first) save 1.3%; keeping r as well, with or without a
    // persisting-L2 set-aside, is slower
    const char *lh = getenv("BBPP_L2HINT");
    ctx->l2hint = !(lh && lh[0] == '0');
    // one fused kernel per FP32 iteration (BBPP_FUSED=0: search and update kernels)
    const char *fu = getenv("BBPP_FUSED");
    ctx->fused = !(fu && fu[0] == '0');
    // residuals of FP64 x into FP32 r: FP64 arithmetic, the outer residual of
    // the mixed-precision method; BBPP_FF_RESID=1 selects float-float
    // arithmetic on the FP32 pipe (~48 bits; measured 0.2 ms per C3 solve)
    const char *ff = getenv("BBPP_FF_RESID");
    ctx->ff_resid = ff && ff[0] == '1';
    // FP64 stencils on an isotropic grid (search kernel, residuals): interior
    // neighbour sums as exact fixed-point sums on the integer pipe
    // (BBPP_XSUM=0: FP64 adds)
    const char *xs = getenv("BBPP_XSUM");
    ctx->GL.xsum = !(xs && xs[0] == '0');
  }
  const size_t n = (size_t)ctx->G.n;
  const size_t nparts = std::max<size_t>(
      std::max<size_t>(std::max<size_t>((size_t)ctx->sgrid.x * ctx->sgrid.y * ctx->sgrid.z, (size_t)ctx->egrid),
                       (size_t)ctx->fgrid.x * ctx->fgrid.y * ctx->fgrid.z),
      std::max<size_t>(std::max<size_t>((size_t)ctx->pgrid[0].x * ctx->pgrid[0].y * ctx->pgrid[0].z,
                                        (size_t)ctx->pgrid[1].x * ctx->pgrid[1].y * ctx->pgrid[1].z),
                       bbpp_tma_partials(ctx)));
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
  ctx->stream = ctx->own_stream;
  if (e == cudaSuccess) e = cudaMalloc(&ctx->st, sizeof(DevState) * 2);
  if (e == cudaSuccess) e = cudaMalloc(&ctx->partials, sizeof(double) * 3 * nparts);
  if (e == cudaSuccess) e = cudaMalloc(&ctx->r, sizeof(double) * n);
  if (e == cudaSuccess) e = cudaMalloc(&ctx->p[0], sizeof(double) * n);
  if (e == cudaSuccess) e = cudaMalloc(&ctx->p[1], sizeof(double) * n);
  if (e == cudaSuccess) e = cudaMalloc(&ctx->Ap, sizeof(double) * n);
  if (e == cudaSuccess) e = cudaMallocHost(&ctx->hst, sizeof(DevState) * 2);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
  if (e == cudaSuccess) e = cudaMemsetAsync(ctx->st, 0, sizeof(DevState) * 2, ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(ctx->partials, 0, sizeof(double) * 3 * nparts, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    bbpp_record_error(ctx, e, "bbpp_create", __LINE__);
    bbpp_destroy(ctx);
    return BBPP_CUDA_ERROR;
  }
  ctx->nparts = nparts;
  *out = ctx;
  return BBPP_CONVERGED;
}

static void drop_graphs(bbpp_ctx *ctx) {
  for (auto &gc : ctx->graphs) {
    if (gc.exec) cudaGraphExecDestroy(gc.exec);
    bbpp_rec_collect(ctx, gc.evs, 0, true);
  }
  ctx->graphs.clear();
}

extern "C" int bbpp_destroy(bbpp_ctx *ctx) {
  if (!ctx) return BBPP_BAD_ARG;
  drop_graphs(ctx);
  bbpp_ir_free(ctx);
  bbpp_net_ctx_free(ctx);
  bbpp_tma_free(ctx);
  if (ctx->st) cudaFree(ctx->st);
  if (ctx->trace) cudaFree(ctx->trace);
  if (ctx->partials) cudaFree(ctx->partials);
  if (ctx->r) cudaFree(ctx->r);
  if (ctx->p[0]) cudaFree(ctx->p[0]);
  if (ctx->p[1]) cudaFree(ctx->p[1]);
  if (ctx->Ap) cudaFree(ctx->Ap);
  if (ctx->hst) cudaFreeHost(ctx->hst);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  for (auto &gc : ctx->graphs) bbpp_rec_collect(ctx, gc.evs, 0, true);
  for (auto &k : ctx->free_ev) {
    cudaEventDestroy(k.a);
    cudaEventDestroy(k.b);
  }
  if (ctx->hbuf_mask) cudaFree(ctx->hbuf_mask);
  if (ctx->hbuf_rhs) cudaFree(ctx->hbuf_rhs);
  if (ctx->hbuf_x) cudaFree(ctx->hbuf_x);
  if (ctx->ev_copy) cudaEventDestroy(ctx->ev_copy);
  if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
  return BBPP_CONVERGED;
}

extern "C" int bbpp_set_stream(bbpp_ctx *ctx, void *stream) {
  if (!ctx) return BBPP_BAD_ARG;
  drop_graphs(ctx);
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
  return BBPP_CONVERGED;
}

extern "C" void bbpp_default_opts(bbpp_opts *o) {
  if (!o) return;
  memset(o, 0, sizeof(*o));
  o->precision = BBPP_FP64;
  o->guess = BBPP_GUESS_ZERO;
  o->stop = BBPP_STOP_TRUE_REL;
  o->tol = 1e-8;
  o->max_iter = 20000;
  o->replace_every = 50;
  o->inner_tol = 1e-4;
  o->max_outer = 30;
  o->ir_mode = BBPP_IR_RELIABLE;
  o->ir_drop = 1e-2;
  o->net = nullptr;
  o->prev = nullptr;
  o->net_coarsen = 0;
}

extern "C" const char *bbpp_status_str(int s) {
  switch (s) {
    case BBPP_CONVERGED: return "converged";
    case BBPP_TINY_RHS: return "tiny rhs";
    case BBPP_MAX_ITER: return "max iterations";
    case BBPP_NAN: return "nan residual";
    case BBPP_BAD_ARG: return "bad argument";
    case BBPP_CUDA_ERROR: return "cuda error";
    case BBPP_NO_DEVICE: return "no device";
    case BBPP_WAIT_TIMEOUT: return "device wait timeout";
    default: return "unknown";
  }
}

extern "C" const char *bbpp_last_error(const bbpp_ctx *ctx) {
  if (ctx) return ctx->err.c_str();
  return g_err;
}

extern "C" const char *bbpp_version(void) { return "bbpp 0.1 (sm_103a)"; }

// The GPU this host thread's later contexts and buffers use (one process per
// GPU: the process's local rank).
extern "C" int bbpp_set_device(int device) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n < 1) return BBPP_NO_DEVICE;
  if (device < 0 || device >= n) return BBPP_BAD_ARG;
  return cudaSetDevice(device) == cudaSuccess ? 0 : BBPP_CUDA_ERROR;
}

// ---------------------------------------------------------------- launches --
// All launches go to ctx->stream.  Typed on the vector element.
template <typename T>
static void launch_search_spmv(bbpp_ctx *ctx, const uint8_t *mask, const T *r, const T *pold, T *pnew, T *Ap, T *x,
                               DevState *st) {
  // bytes/cell: read r, p_old (+ mask), write p_new, Ap; read and write x
  bbpp_rec_begin(ctx, sizeof(T) == 8 ? KK_SEARCH_SPMV : KK_SEARCH_SPMV_F32, 6.0 * sizeof(T) + (mask ? 1 : 0));
  const int prec = sizeof(T) == 8 ? 1 : 0;
  if (sizeof(T) == 4 && bbpp_tma_search(ctx, mask, (const float *)r, (const float *)pold, (float *)pnew,
                                        (float *)Ap, (float *)x, st)) {
    // FP32 on a TMA-eligible grid: launched by bbpp_tma_search
  } else {
    const dim3 g = ctx->pgrid[prec];
    const int kz = ctx->pkz[prec];
    const dim3 b(FNT);
    if (mask) {
      if (ctx->GL.iso)
        bbpp_launch(ctx, k1_search2<T, true, true>, g, b, 0, ctx->GL, r, pold, pnew, Ap, x, mask, st, ctx->partials, kz);
      else
        bbpp_launch(ctx, k1_search2<T, true, false>, g, b, 0, ctx->GL, r, pold, pnew, Ap, x, mask, st, ctx->partials,
                    kz);
    } else {
      if (ctx->GL.iso)
        bbpp_launch(ctx, k1_search2<T, false, true>, g, b, 0, ctx->GL, r, pold, pnew, Ap, x, mask, st, ctx->partials,
                    kz);
      else
        bbpp_launch(ctx, k1_search2<T, false, false>, g, b, 0, ctx->GL, r, pold, pnew, Ap, x, mask, st,
                    ctx->partials, kz);
    }
  }
  bbpp_rec_end(ctx);
}

// cond: a checkpoint, where the update runs only if the residual is not replaced
template <typename T>
static void launch_update(bbpp_ctx *ctx, T *r, const T *Ap, DevState *st, int cond) {
  // bytes/cell: read r, Ap, write r
  bbpp_rec_begin(ctx, sizeof(T) == 8 ? KK_UPDATE : KK_UPDATE_F32, 3.0 * sizeof(T));
  // walk the planes in the reverse of the search kernel's order (its z chunks
  // from the top down), so that both kernels start on the planes the other
  // one touched last, still in L2; needs a power-of-two count of vectors per plane
  int kz = 0, nzc = 0, shift = 0;
  const int prec = sizeof(T) == 8 ? 1 : 0;
  if (!(sizeof(T) == 4 && bbpp_tma_chunks(ctx, &kz, &nzc))) {
    kz = ctx->pkz[prec];
    nzc = (int)ctx->pgrid[prec].z;
  }
  const long long pv = (long long)ctx->GL.nx * ctx->GL.ny / (16 / (int)sizeof(T));
  while (shift < 31 && (1ll << shift) < pv) shift++;
  // FP64: the update is bound by the FP64 pipe, and the index arithmetic of the
  // reversed walk costs more than the L2 hits save (measured 282 -> 297 ms)
  if (sizeof(T) == 8 || (1ll << shift) != pv || (long long)kz * nzc * pv >= (1ll << 32) || ctx->rev_update == 0)
    kz = 0;
  bbpp_launch(ctx, k2_update<T>, dim3(ctx->egrid), dim3(FNT), 0, ctx->GL, r, Ap, st, ctx->partials, cond, kz, nzc,
              div_magic((unsigned)std::max(nzc, 1)), shift, (int)(sizeof(T) == 4 && ctx->l2hint));
  bbpp_rec_end(ctx);
}

// general-form residual / SpMV on the unscaled operator (checks, kernel ABI)
template <typename TXT, typename TR>
static void launch_resid(bbpp_ctx *ctx, const uint8_t *mask, const TXT *x, const TXT *rhs, TR *r, DevState *st,
                         int mode) {
  if (mask)
    k_resid<TXT, TR, true><<<ctx->sgrid, NT, 0, ctx->stream>>>(ctx->G, x, rhs, r, mask, st, ctx->partials, ctx->kz,
                                                               mode);
  else
    k_resid<TXT, TR, false><<<ctx->sgrid, NT, 0, ctx->stream>>>(ctx->G, x, rhs, r, mask, st, ctx->partials,
                                                                ctx->kz, mode);
}

template <typename TXT, typename TR>
void bbpp_launch_resid_s(bbpp_ctx *ctx, const uint8_t *mask, TXT *x, const TXT *rhs, TR *r, DevState *st, int mode,
                         double bscale) {
  // bytes/cell: read x, rhs (+ mask), write r
  bbpp_rec_begin(ctx, sizeof(TXT) == 8 ? KK_RESID : KK_RESID_F32, 2.0 * sizeof(TXT) + sizeof(TR) + (mask ? 1 : 0));
  const dim3 g = ctx->fgrid, b(FNT);
  if constexpr (std::is_same<TXT, double>::value && std::is_same<TR, float>::value) {
    // FP64 x into an FP32 residual: float-float arithmetic on the FP32 pipe
    if (ctx->ff_resid) {
      if (mask) {
        if (ctx->GL.iso)
          bbpp_launch(ctx, k_resid_ff<true, true>, g, b, 0, ctx->GL, x, rhs, r, mask, st, ctx->partials, ctx->fkz, mode,
                      bscale);
        else
          bbpp_launch(ctx, k_resid_ff<true, false>, g, b, 0, ctx->GL, x, rhs, r, mask, st, ctx->partials, ctx->fkz,
                      mode, bscale);
      } else {
        if (ctx->GL.iso)
          bbpp_launch(ctx, k_resid_ff<false, true>, g, b, 0, ctx->GL, x, rhs, r, mask, st, ctx->partials, ctx->fkz,
                      mode, bscale);
        else
          bbpp_launch(ctx, k_resid_ff<false, false>, g, b, 0, ctx->GL, x, rhs, r, mask, st, ctx->partials, ctx->fkz,
                      mode, bscale);
      }
      bbpp_rec_end(ctx);
      return;
    }
  }
  if (mask) {
    if (ctx->GL.iso)
      bbpp_launch(ctx, k_resid_s<TXT, TR, true, true>, g, b, 0, ctx->GL, x, rhs, r, mask, st, ctx->partials,
                  ctx->fkz, mode, bscale);
    else
      bbpp_launch(ctx, k_resid_s<TXT, TR, true, false>, g, b, 0, ctx->GL, x, rhs, r, mask, st, ctx->partials,
                  ctx->fkz, mode, bscale);
  } else {
    if (ctx->GL.iso)
      bbpp_launch(ctx, k_resid_s<TXT, TR, false, true>, g, b, 0, ctx->GL, x, rhs, r, mask, st, ctx->partials,
                  ctx->fkz, mode, bscale);
    else
      bbpp_launch(ctx, k_resid_s<TXT, TR, false, false>, g, b, 0, ctx->GL, x, rhs, r, mask, st, ctx->partials,
                  ctx->fkz, mode, bscale);
  }
  bbpp_rec_end(ctx);
}

template void bbpp_launch_resid_s<double, double>(bbpp_ctx *, const uint8_t *, double *, const double *, double *,
                                                  DevState *, int, double);
template void bbpp_launch_resid_s<double, float>(bbpp_ctx *, const uint8_t *, double *, const double *, float *,
                                                 DevState *, int, double);
template void bbpp_launch_resid_s<float, float>(bbpp_ctx *, const uint8_t *, float *, const float *, float *,
                                                DevState *, int, double);

// bscale of the right-hand side the current solve runs on (S for the user's
// rhs, 1 for an already scaled one)
static thread_local double t_bscale = 1.0;

// Reliable updates of the mixed-precision solve: when set, the FP32 loop's
// residual replacements and confirmations fold the FP32 correction into the
// FP64 solution and recompute the residual from it in FP64.
struct Reliable {
  double *xhi = nullptr;
  const double *rhs = nullptr;
};
static thread_local Reliable t_rel;

void bbpp_set_reliable(double *xhi, const double *rhs) {
  t_rel.xhi = xhi;
  t_rel.rhs = rhs;
}

// Reliable update of the mixed-precision solve: x_hi += d (+ alpha p when d
// lags), d = 0, all in FP64; d and p are widened with integer operations, so
// the FP64 pipe sees only the add and the FMA.  check as for k_settle.
__global__ void __launch_bounds__(FNT) k_fold(const GeoL G, double *__restrict__ xhi, float *__restrict__ d,
                                              const float *__restrict__ p, const DevState *st, int check) {
  pdl_sync();
  if (skip_step(st, check)) return;
  const bool lag = *(volatile const int *)&st->dlag;
  const double alpha = lag ? *(volatile const double *)&st->alpha : 0.0;
  const unsigned int n = (unsigned int)G.n;
  for (unsigned int c = blockIdx.x * FNT + threadIdx.x; c < n; c += gridDim.x * FNT) {
    double v = xhi[c] + widen_f32(d[c]);
    if (lag) v = fma(alpha, widen_f32(p[c]), v);
    xhi[c] = v;
    d[c] = 0.f;
  }
}

// x += alpha p if x lags (check: return at once in a finished solve)
template <typename T>
static void launch_settle(bbpp_ctx *ctx, T *x, const T *p, DevState *st, int check) {
  bbpp_rec_begin(ctx, sizeof(T) == 8 ? KK_AXPY : KK_AXPY_F32, 3.0 * sizeof(T));
  bbpp_launch(ctx, k_settle<T>, dim3(ctx->egrid), dim3(FNT), 0, ctx->GL, x, p, st, check);
  bbpp_rec_end(ctx);
}

// The residual step of an iteration or a confirmation, for vectors of type T:
// bring x up to date (p = the last search direction), then r from x.
template <typename T>
static void launch_replace(bbpp_ctx *ctx, const uint8_t *mask, T *x, const T *rhs, T *r, const T *p, DevState *st,
                           int mode) {
  const int check = mode == RES_ITER ? 2 : 0;
  if (sizeof(T) == 4 && t_rel.xhi) {
    bbpp_rec_begin(ctx, KK_AXPY_F32, 20.0);
    bbpp_launch(ctx, k_fold, dim3(ctx->egrid), dim3(FNT), 0, ctx->GL, t_rel.xhi, (float *)x, (const float *)p, st,
                check);
    bbpp_rec_end(ctx);
    bbpp_launch_resid_s<double, float>(ctx, mask, t_rel.xhi, t_rel.rhs, (float *)r, st, mode, ctx->GL.S);
  } else {
    launch_settle<T>(ctx, x, p, st, check);
    bbpp_launch_resid_s<T, T>(ctx, mask, x, rhs, r, st, mode, t_bscale);
  }
}

template <typename T>
static void launch_iteration(bbpp_ctx *ctx, const uint8_t *mask, const T *rhs, T *x, T *r, T *const p[2], T *Ap,
                             DevState *st, int q, int replace_every, bool rr) {
  (void)rr;
  // q = 1-based iteration number; K1 reads p[(q-1)%2] and writes p[q%2]
  T *pold = p[(q - 1) & 1], *pnew = p[q & 1];
  launch_search_spmv<T>(ctx, mask, r, pold, pnew, Ap, x, st);
  if (q % replace_every == 0) {
    // checkpoint: the search kernel has decided between the recursive update
    // and a residual replacement; the other kernels return at once
    launch_update<T>(ctx, r, Ap, st, 1);
    launch_replace<T>(ctx, mask, x, rhs, r, pnew, st, RES_ITER);
  } else {
    launch_update<T>(ctx, r, Ap, st, 0);
  }
}

// Capture (or reuse) the graph of iterations q0+1 .. q0+len for these buffers.
// Returns its index in ctx->graphs, or -1 after a CUDA error.
// Capture len iterations (launch(i), i = 1 .. len) into a cached graph.
template <typename F>
static int capture_chunk(bbpp_ctx *ctx, const GraphKey &key, int len, F launch, cudaGraphExec_t *out) {
  for (auto &gc : ctx->graphs)
    if (gc.key == key) {
      *out = gc.exec;
      return (int)(&gc - &ctx->graphs[0]);
    }
  cudaGraph_t graph = nullptr;
  bbpp_ctx *c = ctx;
  cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    bbpp_record_error(c, e, "cudaStreamBeginCapture", __LINE__);
    return -1;
  }
  GraphCache gc;
  gc.key = key;
  ctx->rec = nullptr;  // graphs carry no profiling events
  for (int i = 1; i <= len; i++) {
    ctx->rec_iter = i;
    launch(i);
  }
  ctx->rec = nullptr;
  e = cudaStreamEndCapture(ctx->stream, &graph);
  if (e != cudaSuccess) {
    bbpp_record_error(c, e, "cudaStreamEndCapture", __LINE__);
    return -1;
  }
  cudaGraphExec_t exec = nullptr;
  size_t nnodes = 0;
  cudaGraphGetNodes(graph, nullptr, &nnodes);
  e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    bbpp_record_error(c, e, "cudaGraphInstantiate", __LINE__);
    return -1;
  }
  if (ctx->graphs.size() >= 8) {
    cudaGraphExecDestroy(ctx->graphs.front().exec);
    bbpp_rec_collect(ctx, ctx->graphs.front().evs, 0, true);
    ctx->graphs.erase(ctx->graphs.begin());
  }
  gc.exec = exec;
  gc.kernels = (int)(nnodes - 2 * gc.evs.size());
  ctx->graphs.push_back(gc);
  *out = exec;
  return (int)ctx->graphs.size() - 1;
}

template <typename T>
static int get_chunk_graph(bbpp_ctx *ctx, const uint8_t *mask, const T *rhs, T *x, T *r, T *const p[2], T *Ap,
                           DevState *st, int len, int replace_every, bool rr, cudaGraphExec_t *out) {
  GraphKey key;
  key.mask = mask;
  key.rhs = rhs;
  key.x = x;
  key.r = r;
  key.p0 = p[0];
  key.p1 = p[1];
  key.Ap = Ap;
  key.st = st;
  key.len = len;
  key.replace_every = replace_every;
  key.rr = rr;
  key.elem = (int)sizeof(T);
  key.stream = ctx->stream;
  key.bscale = t_bscale;
  key.xhi = t_rel.xhi;
  key.rhs64 = t_rel.rhs;
  return capture_chunk(
      ctx, key, len, [&](int i) { launch_iteration<T>(ctx, mask, rhs, x, r, p, Ap, st, i, replace_every, rr); }, out);
}

static int status_of(int done) {
  switch (done) {
    case DONE_CONVERGED: return BBPP_CONVERGED;
    case DONE_MAX_ITER: return BBPP_MAX_ITER;
    case DONE_NAN: return BBPP_NAN;
    case DONE_TINY: return BBPP_TINY_RHS;
    case DONE_TIMEOUT: return BBPP_WAIT_TIMEOUT;
    default: return BBPP_MAX_ITER;
  }
}

// Core PCG loop for vectors of type T on a given device state.  Used by the
// FP64 method directly and by FP32_IR for its inner sweeps.  On entry the
// state has been initialised by a RES_INIT residual (r, rz, rr, bb set).
template <typename T>
int bbpp_pcg_loop(bbpp_ctx *ctx, const uint8_t *mask, const T *rhs, T *x, T *r, T *const p[2], T *Ap, DevState *st,
                  DevState *hst, int replace_every, bool confirm, bool rr, int *iters_out) {
  const int chunk = (replace_every % 2 == 0) ? replace_every : 2 * replace_every;
  // q = completed iterations, read back from the device
  CK(cudaMemcpyAsync(hst, st, sizeof(DevState), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  int q = hst->iter;
  // host-side bound: the device state stops the solve after max_iter + 1
  // iterations; this only guards against a state that never advances
  long long rounds = 0;
  const long long max_rounds = 4ll * (hst->max_iter / 1 + 2) + 64;
  while (hst->done == RUNNING) {
    if (++rounds > max_rounds) {
      bbpp_record_error(ctx, cudaErrorUnknown, "solve loop made no progress", __LINE__);
      return BBPP_CUDA_ERROR;
    }
    const int q0 = q;
    int gi = -1;
    std::vector<KEv> single;
    if (q % chunk == 0 && !ctx->profiling) {
      cudaGraphExec_t exec;
      gi = get_chunk_graph<T>(ctx, mask, rhs, x, r, p, Ap, st, chunk, replace_every, rr, &exec);
      if (gi < 0) return BBPP_CUDA_ERROR;
      CK(cudaGraphLaunch(exec, ctx->stream));
      ctx->launches += ctx->graphs[gi].kernels;
    } else if (q % chunk == 0) {
      // profiling: the same chunk as direct launches enqueued back to back,
      // with an event pair around every kernel (no host gap between kernels)
      ctx->rec = &single;
      for (int i = 1; i <= chunk; i++) {
        ctx->rec_iter = i;
        launch_iteration<T>(ctx, mask, rhs, x, r, p, Ap, st, q + i, replace_every, rr);
        ctx->launches += ((q + i) % replace_every == 0) ? 4 : 2;
      }
      ctx->rec = nullptr;
      CK(cudaGetLastError());
    } else {
      if (ctx->profiling) ctx->rec = &single;
      ctx->rec_iter = 1;
      launch_iteration<T>(ctx, mask, rhs, x, r, p, Ap, st, q + 1, replace_every, rr);
      ctx->rec = nullptr;
      ctx->launches += ((q + 1) % replace_every == 0) ? 4 : 2;
      CK(cudaGetLastError());
    }
    CK(cudaMemcpyAsync(hst, st, sizeof(DevState), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    q = hst->iter;
    if (ctx->profiling) {
      if (gi >= 0) bbpp_rec_collect(ctx, ctx->graphs[gi].evs, q - q0, false);
      else bbpp_rec_collect(ctx, single, q - q0, true);
    }
    if (hst->done == DONE_PENDING) {
      if (!confirm) {
        hst->done = DONE_CONVERGED;
        CK(cudaMemcpyAsync(&st->done, &hst->done, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
        break;
      }
      launch_replace<T>(ctx, mask, x, rhs, r, p[q & 1], st, RES_CONFIRM);
      ctx->launches += 2;
      CK(cudaGetLastError());
      CK(cudaMemcpyAsync(hst, st, sizeof(DevState), cudaMemcpyDeviceToHost, ctx->stream));
      CK(cudaStreamSynchronize(ctx->stream));
    }
  }
  // x (or d) still lacks alpha p of the last iteration unless a residual
  // replacement or confirmation came last
  if (sizeof(T) == 4 && t_rel.xhi) {
    k_fold<<<ctx->egrid, FNT, 0, ctx->stream>>>(ctx->GL, t_rel.xhi, (float *)x, (const float *)p[q & 1], st, 0);
  } else {
    k_settle<T><<<ctx->egrid, FNT, 0, ctx->stream>>>(ctx->GL, x, p[q & 1], st, 0);
  }
  ctx->launches += 1;
  CK(cudaGetLastError());
  if (iters_out) *iters_out = q;
  return 0;
}

// ---------------------------------------------------- fused iterations --
// Iteration q (1-based) is one kernel: it reads r[(q-1)&1], Ap[(q-1)&1] and
// p[(q-1)&1], writes r[q&1], Ap[q&1] and p[q&1], and leaves its own step
// (alpha_q p_q into x, alpha_q Ap_q out of r) pending for the next kernel or
// for the fold and residual kernels of a replacement or confirmation, which
// write r[q&1].  The host counts kernels (st->fq); an iteration ends (st->iter)
// in the kernel after it.
static void launch_fused(bbpp_ctx *ctx, const uint8_t *mask, const float *rhs, float *x, float *const r[2],
                         float *const p[2], float *const Ap[2], DevState *st, int q, int replace_every) {
  const int i = (q - 1) & 1, o = q & 1;
  // bytes/cell: read r, Ap, p_old, x (+ mask), write r, p, Ap, x
  bbpp_rec_begin(ctx, KK_FUSED_F32, 32.0 + (mask ? 1 : 0));
  bbpp_tma_fused(ctx, mask, r[i], Ap[i], p[i], r[o], p[o], Ap[o], x, st);
  bbpp_rec_end(ctx);
  // checkpoint: the kernel has decided between the recursive residual and a
  // replacement; the replacement kernels return at once without one
  if (q % replace_every == 0) launch_replace<float>(ctx, mask, x, rhs, r[o], p[o], st, RES_ITER);
}

int bbpp_pcg_loop_fused(bbpp_ctx *ctx, const uint8_t *mask, const float *rhs, float *x, float *const r[2],
                        float *const p[2], float *const Ap[2], DevState *st, DevState *hst, int replace_every,
                        bool confirm, int *iters_out) {
  const int chunk = (replace_every % 2 == 0) ? replace_every : 2 * replace_every;
  CK(cudaMemcpyAsync(hst, st, sizeof(DevState), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  int q = hst->fq;
  long long rounds = 0;
  const long long max_rounds = 4ll * (hst->max_iter / 1 + 2) + 64;
  auto per_launch = [&](int qq) { return (qq % replace_every == 0) ? 3 : 1; };
  while (hst->done == RUNNING) {
    if (++rounds > max_rounds) {
      bbpp_record_error(ctx, cudaErrorUnknown, "solve loop made no progress", __LINE__);
      return BBPP_CUDA_ERROR;
    }
    const int q0 = q;
    int gi = -1;
    std::vector<KEv> single;
    if (q % chunk == 0 && !ctx->profiling) {
      GraphKey key;
      key.mask = mask;
      key.rhs = rhs;
      key.x = x;
      key.r = r[0];
      key.r1 = r[1];
      key.p0 = p[0];
      key.p1 = p[1];
      key.Ap = Ap[0];
      key.Ap1 = Ap[1];
      key.st = st;
      key.len = chunk;
      key.replace_every = replace_every;
      key.elem = 4;
      key.stream = ctx->stream;
      key.bscale = t_bscale;
      key.xhi = t_rel.xhi;
      key.rhs64 = t_rel.rhs;
      cudaGraphExec_t exec;
      gi = capture_chunk(
          ctx, key, chunk, [&](int i) { launch_fused(ctx, mask, rhs, x, r, p, Ap, st, i, replace_every); }, &exec);
      if (gi < 0) return BBPP_CUDA_ERROR;
      CK(cudaGraphLaunch(exec, ctx->stream));
      ctx->launches += ctx->graphs[gi].kernels;
    } else if (q % chunk == 0) {
      ctx->rec = &single;
      for (int i = 1; i <= chunk; i++) {
        ctx->rec_iter = i;
        launch_fused(ctx, mask, rhs, x, r, p, Ap, st, q + i, replace_every);
        ctx->launches += per_launch(q + i);
      }
      ctx->rec = nullptr;
      CK(cudaGetLastError());
    } else {
      if (ctx->profiling) ctx->rec = &single;
      ctx->rec_iter = 1;
      launch_fused(ctx, mask, rhs, x, r, p, Ap, st, q + 1, replace_every);
      ctx->rec = nullptr;
      ctx->launches += per_launch(q + 1);
      CK(cudaGetLastError());
    }
    CK(cudaMemcpyAsync(hst, st, sizeof(DevState), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    q = hst->fq;
    if (ctx->profiling) {
      if (gi >= 0) bbpp_rec_collect(ctx, ctx->graphs[gi].evs, q - q0, false);
      else bbpp_rec_collect(ctx, single, q - q0, true);
    }
    if (hst->done == DONE_PENDING) {
      if (!confirm) {
        hst->done = DONE_CONVERGED;
        CK(cudaMemcpyAsync(&st->done, &hst->done, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
        break;
      }
      launch_replace<float>(ctx, mask, x, rhs, r[q & 1], p[q & 1], st, RES_CONFIRM);
      ctx->launches += 2;
      CK(cudaGetLastError());
      CK(cudaMemcpyAsync(hst, st, sizeof(DevState), cudaMemcpyDeviceToHost, ctx->stream));
      CK(cudaStreamSynchronize(ctx->stream));
    }
  }
  // x still lacks the pending step unless a replacement or confirmation came last
  k_fold<<<ctx->egrid, FNT, 0, ctx->stream>>>(ctx->GL, t_rel.xhi, x, p[q & 1], st, 0);
  ctx->launches += 1;
  CK(cudaGetLastError());
  if (iters_out) *iters_out = hst->iter;
  return 0;
}

template int bbpp_pcg_loop<double>(bbpp_ctx *, const uint8_t *, const double *, double *, double *, double *const[2],
                                   double *, DevState *, DevState *, int, bool, bool, int *);
template int bbpp_pcg_loop<float>(bbpp_ctx *, const uint8_t *, const float *, float *, float *, float *const[2],
                                  float *, DevState *, DevState *, int, bool, bool, int *);

// Initialise a device state and run r = rhs - (-A)x (RES_INIT) for type T.
template <typename T>
int bbpp_pcg_init(bbpp_ctx *ctx, const uint8_t *mask, const T *rhs, T *x, T *r, DevState *st, DevState *hst,
                  double tol, int stop, int max_iter, bool zero_x, double bscale) {
  memset(hst, 0, sizeof(DevState));
  // thresholds on the scaled quantities: (r,z) scales by bscale, (r,r) by
  // bscale^2; RES_INIT multiplies by the unscaled (rhs,rhs)
  hst->tol2bb = tol * tol * (stop == 0 ? bscale : bscale * bscale);
  // the reference's absolute exit (rhs,rhs) < 1e-16 applies to a user's
  // right-hand side; an inner correction system only stops on an exact zero
  hst->tiny = (bscale == 1.0) ? 2.2250738585072014e-308 : 1e-16;
  t_bscale = bscale;
  hst->max_iter = max_iter;
  hst->inject = ctx->inject;
  hst->wait_ns = ctx->wait_ns;
  hst->stop = stop;
  hst->first = 1;
  if (ctx->trace && sizeof(T) == 8) {
    // the plain FP64 method's alpha and beta; entries not reached stay NaN
    hst->trace_a = ctx->trace;
    hst->trace_b = ctx->trace + ctx->trace_n;
    hst->trace_n = ctx->trace_n;
    CK(cudaMemsetAsync(ctx->trace, 0xff, sizeof(double) * 2 * (size_t)ctx->trace_n, ctx->stream));
  }
  CK(cudaMemcpyAsync(st, hst, sizeof(DevState), cudaMemcpyHostToDevice, ctx->stream));
  if (zero_x) CK(cudaMemsetAsync(x, 0, sizeof(T) * (size_t)ctx->G.n, ctx->stream));
  bbpp_launch_resid_s<T, T>(ctx, mask, x, rhs, r, st, RES_INIT, bscale);
  ctx->launches += 1;
  CK(cudaGetLastError());
  return 0;
}

template int bbpp_pcg_init<double>(bbpp_ctx *, const uint8_t *, const double *, double *, double *, DevState *,
                                   DevState *, double, int, int, bool, double);
template int bbpp_pcg_init<float>(bbpp_ctx *, const uint8_t *, const float *, float *, float *, DevState *,
                                  DevState *, double, int, int, bool, double);

// ------------------------------------------------------------------ solve --
static int check_opts(const bbpp_opts *o) {
  if (!o) return BBPP_BAD_ARG;
  if (o->precision != BBPP_FP64 && o->precision != BBPP_FP32_IR) return BBPP_BAD_ARG;
  if (o->guess < BBPP_GUESS_ZERO || o->guess > BBPP_GUESS_LEARNED) return BBPP_BAD_ARG;
  if (o->stop != BBPP_STOP_REF_RZ && o->stop != BBPP_STOP_TRUE_REL) return BBPP_BAD_ARG;
  if (o->ir_mode != BBPP_IR_RELIABLE && o->ir_mode != BBPP_IR_RESTART) return BBPP_BAD_ARG;
  if (!(o->ir_drop >= 0.0 && o->ir_drop < 1.0)) return BBPP_BAD_ARG;
  if (!(o->tol >= 0) || o->max_iter < 0 || o->replace_every < 1) return BBPP_BAD_ARG;
  if (o->guess == BBPP_GUESS_LEARNED && !o->net) return BBPP_BAD_ARG;
  if (o->net_coarsen < 0 || o->net_coarsen > 4 || o->net_coarsen == 3) return BBPP_BAD_ARG;
  return 0;
}

static int solve_fp64(bbpp_ctx *ctx, const uint8_t *mask, const double *rhs, double *x, const bbpp_opts *o,
                      bool zero_x, bbpp_report *rep) {
  DevState *st = ctx->st, *hst = ctx->hst;
  const double S = ctx->GL.S;
  int rc = bbpp_pcg_init<double>(ctx, mask, rhs, x, ctx->r, st, hst, o->tol, o->stop, o->max_iter, zero_x, S);
  if (rc) return rc;
  double *const p[2] = {ctx->p[0], ctx->p[1]};
  int iters = 0;
  rc = bbpp_pcg_loop<double>(ctx, mask, rhs, x, ctx->r, p, ctx->Ap, st, hst, o->replace_every,
                             o->stop == BBPP_STOP_TRUE_REL, o->stop == BBPP_STOP_TRUE_REL, &iters);
  if (rc) return rc;
  rep->iters = iters;
  rep->replacements = hst->replacements;
  rep->bb = hst->bb;
  rep->rz = hst->rz_last / S;  // back to the unscaled (r, z)
  rep->rel_resid = hst->bb > 0 ? std::sqrt(std::max(0.0, hst->rr) / hst->bb) / S : 0.0;
  rep->status = status_of(hst->done);
  // canonical bytes of the work (the reference formulation's traffic): per
  // iteration 81 (mask) or 80 B/cell; per replacement x-update 24 + residual
  // 25; init residual 25
  const double n = (double)ctx->G.n;
  const double per_it = mask ? 81.0 : 80.0;
  rep->bytes = n * (per_it * iters + 49.0 * hst->replacements + 25.0);
  return 0;
}

// Explicit true relative residual of x (uses ctx->Ap as scratch).
static int true_rel(bbpp_ctx *ctx, const uint8_t *mask, const double *rhs, const double *x, double *out) {
  DevState *st = ctx->st + 1, *hst = ctx->hst + 1;
  memset(hst, 0, sizeof(DevState));
  hst->tol2bb = 0.0;
  hst->stop = 1;
  CK(cudaMemcpyAsync(st, hst, sizeof(DevState), cudaMemcpyHostToDevice, ctx->stream));
  launch_resid<double, double>(ctx, mask, x, rhs, ctx->Ap, st, RES_INIT);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(hst, st, sizeof(DevState), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  *out = hst->bb > 0 ? std::sqrt(hst->rr / hst->bb) : std::sqrt(hst->rr);
  return 0;
}

// The solve without the final residual check: guess, solver, the device time
// of both in rep->ms.  x is final when it returns (its stream has it in order).
static int solve_core(bbpp_ctx *ctx, const uint8_t *mask, const double *rhs, double *x, const bbpp_opts *o,
                      bbpp_report *rep) {
  memset(rep, 0, sizeof(*rep));
  if (!ctx || !rhs || !x) return rep->status = BBPP_BAD_ARG;
  int rc = check_opts(o);
  if (rc) return rep->status = rc;
  ctx->launches = 0;
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  bool zero_x = o->guess == BBPP_GUESS_ZERO;
  if (o->guess == BBPP_GUESS_LEARNED) {
    rc = bbpp_net_guess(ctx, o->net, mask, rhs, o->prev, x, o->net_coarsen, &rep->guess_ms);
    if (rc) return rep->status = rc;
    zero_x = false;
  }
  if (o->precision == BBPP_FP64)
    rc = solve_fp64(ctx, mask, rhs, x, o, zero_x, rep);
  else
    rc = bbpp_solve_ir(ctx, mask, rhs, x, o, zero_x, rep);
  if (rc) return rep->status = rc;
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  CK(cudaEventSynchronize(ctx->ev1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  rep->ms = ms;
  rep->launches = (int)ctx->launches;
  return 0;
}

extern "C" int bbpp_solve(bbpp_ctx *ctx, const uint8_t *mask, const double *rhs, double *x, const bbpp_opts *o,
                          bbpp_report *rep) {
  bbpp_report tmp;
  if (!rep) rep = &tmp;
  int rc = solve_core(ctx, mask, rhs, x, o, rep);
  if (rc) return rc;
  rc = true_rel(ctx, mask, rhs, x, &rep->true_rel);
  if (rc) return rep->status = rc;
  return rep->status;
}

extern "C" int bbpp_solve_host(bbpp_ctx *ctx, const uint8_t *mask, const double *rhs, double *x,
                               const bbpp_opts *o, bbpp_report *rep) {
  bbpp_report tmp;
  if (!rep) rep = &tmp;
  memset(rep, 0, sizeof(*rep));
  if (!ctx || !rhs || !x) return rep->status = BBPP_BAD_ARG;
  const size_t n = (size_t)ctx->G.n;
  if (!ctx->hbuf_rhs) {
    CK(cudaMalloc(&ctx->hbuf_rhs, sizeof(double) * n));
    CK(cudaMalloc(&ctx->hbuf_x, sizeof(double) * n));
    CK(cudaMalloc(&ctx->hbuf_mask, n));
    CK(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&ctx->ev_copy, cudaEventDisableTiming));
  }
  CK(cudaMemcpyAsync(ctx->hbuf_rhs, rhs, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  if (mask) CK(cudaMemcpyAsync(ctx->hbuf_mask, mask, n, cudaMemcpyHostToDevice, ctx->stream));
  if (o && o->guess == BBPP_GUESS_GIVEN)
    CK(cudaMemcpyAsync(ctx->hbuf_x, x, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  const uint8_t *dmask = mask ? ctx->hbuf_mask : nullptr;
  int rc = solve_core(ctx, dmask, ctx->hbuf_rhs, ctx->hbuf_x, o, rep);
  if (rc) return rc;
  rc = rep->status;
  if (rc != BBPP_CONVERGED && rc != BBPP_TINY_RHS && rc != BBPP_MAX_ITER && rc != BBPP_NAN) return rc;
  // x is final: its copy to the host (at the link's ~200 GB/s) runs beside the
  // residual check, which only reads it
  CK(cudaEventRecord(ctx->ev_copy, ctx->stream));
  CK(cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_copy, 0));
  CK(cudaMemcpyAsync(x, ctx->hbuf_x, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->copy_stream));
  const int rc_check = true_rel(ctx, dmask, ctx->hbuf_rhs, ctx->hbuf_x, &rep->true_rel);
  CK(cudaStreamSynchronize(ctx->copy_stream));
  if (rc_check) return rep->status = rc_check;
  return rc;
}

// ------------------------------------------------------- kernel-level ABI --
extern "C" int bbpp_spmv(bbpp_ctx *ctx, const uint8_t *mask, const double *p, double *Ap) {
  if (!ctx || !p || !Ap) return BBPP_BAD_ARG;
  launch_resid<double, double>(ctx, mask, p, nullptr, Ap, ctx->st + 1, RES_PLAIN);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return 0;
}

extern "C" int bbpp_invm(bbpp_ctx *ctx, double *invM) {
  if (!ctx || !invM) return BBPP_BAD_ARG;
  k_invm<<<ctx->egrid, NT, 0, ctx->stream>>>(ctx->G, invM);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return 0;
}

// PP_rhs (src/solver_kernel.cu:152-173) on dense face arrays: rhs = -(rho/dt)
// div u*, the reference's evaluation order without contraction.
__global__ void k_rhs_div(int nx, int ny, int nz, double idx, double idy, double idz, double rho_idt,
                          const double *__restrict__ u, const double *__restrict__ v, const double *__restrict__ w,
                          double *__restrict__ rhs) {
  const long long n = (long long)nx * ny * nz;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(c % nx);
    const long long r = c / nx;
    const int j = (int)(r % ny), k = (int)(r / ny);
    const long long uw = i + (long long)(nx + 1) * (j + (long long)ny * k);
    const long long vs = i + (long long)nx * (j + (long long)(ny + 1) * k);
    double s = __dmul_rn(__dsub_rn(u[uw + 1], u[uw]), idx);
    s = __dadd_rn(s, __dmul_rn(__dsub_rn(v[vs + nx], v[vs]), idy));
    s = __dadd_rn(s, __dmul_rn(__dsub_rn(w[c + (long long)nx * ny], w[c]), idz));
    rhs[c] = -__dmul_rn(s, rho_idt);
  }
}

extern "C" int bbpp_rhs_div(bbpp_ctx *ctx, double rho_f, double dt, const double *u, const double *v, const double *w,
                            double *rhs) {
  if (!ctx || !u || !v || !w || !rhs || !(dt != 0.0)) return BBPP_BAD_ARG;
  const Geo &G = ctx->G;
  k_rhs_div<<<ctx->egrid, NT, 0, ctx->stream>>>(G.nx, G.ny, G.nz, 1. / ctx->grid.dx, 1. / ctx->grid.dy,
                                                 1. / ctx->grid.dz, rho_f / dt, u, v, w, rhs);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return 0;
}

// Failure-detection test hook: the bound of device-side waits, and whether the
// next solves' TMA search kernel leaves one plane's copies unissued (its wait
// then runs out and the solve returns BBPP_WAIT_TIMEOUT; no fault, no hang).
extern "C" int bbpp_debug_wait(bbpp_ctx *ctx, long long wait_ns, int inject) {
  if (!ctx || wait_ns < 0) return BBPP_BAD_ARG;
  ctx->wait_ns = wait_ns;
  ctx->inject = inject ? 1 : 0;
  return 0;
}

// One search-kernel launch on caller vectors (kernel-level checks).
template <typename T>
static int search_once(bbpp_ctx *ctx, int kernel, const uint8_t *mask, const T *r, const T *pold, T *pnew, T *Ap,
                       T *x, DevState *st) {
  if (kernel == 2) {
    if (sizeof(T) != 4 || !bbpp_tma_search(ctx, mask, (const float *)r, (const float *)pold, (float *)pnew,
                                           (float *)Ap, (float *)x, st))
      return BBPP_BAD_ARG;
  } else if (kernel == 1) {
    const int prec = sizeof(T) == 8 ? 1 : 0;
    const dim3 g = ctx->pgrid[prec];
    const int kz = ctx->pkz[prec];
    cudaStream_t s = ctx->stream;
    if (mask) {
      if (ctx->GL.iso) k1_search2<T, true, true><<<g, FNT, 0, s>>>(ctx->GL, r, pold, pnew, Ap, x, mask, st, ctx->partials, kz);
      else k1_search2<T, true, false><<<g, FNT, 0, s>>>(ctx->GL, r, pold, pnew, Ap, x, mask, st, ctx->partials, kz);
    } else {
      if (ctx->GL.iso) k1_search2<T, false, true><<<g, FNT, 0, s>>>(ctx->GL, r, pold, pnew, Ap, x, mask, st, ctx->partials, kz);
      else k1_search2<T, false, false><<<g, FNT, 0, s>>>(ctx->GL, r, pold, pnew, Ap, x, mask, st, ctx->partials, kz);
    }
  } else {
    launch_search_spmv<T>(ctx, mask, r, pold, pnew, Ap, x, st);
  }
  return 0;
}

extern "C" int bbpp_search_step(bbpp_ctx *ctx, int precision, int kernel, const uint8_t *mask, const void *r,
                                const void *pold, void *pnew, void *Ap, void *x, double beta, double alpha, int first,
                                int lag, double *pAp) {
  if (!ctx || !r || !pnew || !Ap || !x || (!first && !pold)) return BBPP_BAD_ARG;
  if (precision != BBPP_FP64 && precision != BBPP_FP32_IR) return BBPP_BAD_ARG;
  if (kernel < 0 || kernel > 2) return BBPP_BAD_ARG;
  DevState *st = ctx->st + 1, *hst = ctx->hst + 1;
  memset(hst, 0, sizeof(DevState));
  hst->first = first ? 1 : 0;
  hst->beta = beta;
  hst->alpha = alpha;
  hst->dlag = lag ? 1 : 0;
  hst->rz = 1.0;  // the kernel leaves alpha = rz / (p, Ap)
  hst->inject = ctx->inject;
  hst->wait_ns = ctx->wait_ns;
  CK(cudaMemcpyAsync(st, hst, sizeof(DevState), cudaMemcpyHostToDevice, ctx->stream));
  int rc;
  if (precision == BBPP_FP64)
    rc = search_once<double>(ctx, kernel, mask, (const double *)r, (const double *)pold, (double *)pnew,
                             (double *)Ap, (double *)x, st);
  else
    rc = search_once<float>(ctx, kernel, mask, (const float *)r, (const float *)pold, (float *)pnew, (float *)Ap,
                            (float *)x, st);
  if (rc) return rc;
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(hst, st, sizeof(DevState), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (hst->done == DONE_TIMEOUT) return BBPP_WAIT_TIMEOUT;
  if (pAp) *pAp = hst->pAp;
  return 0;
}

extern "C" int bbpp_residual(bbpp_ctx *ctx, const uint8_t *mask, const double *rhs, const double *x, double *r,
                             double *rr, double *bb) {
  if (!ctx || !rhs || !x || !r) return BBPP_BAD_ARG;
  DevState *st = ctx->st + 1, *hst = ctx->hst + 1;
  memset(hst, 0, sizeof(DevState));
  hst->stop = 1;
  CK(cudaMemcpyAsync(st, hst, sizeof(DevState), cudaMemcpyHostToDevice, ctx->stream));
  launch_resid<double, double>(ctx, mask, x, rhs, r, st, RES_INIT);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(hst, st, sizeof(DevState), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (rr) *rr = hst->rr;
  if (bb) *bb = hst->bb;
  return 0;
}

// r = rhs - (-A) x on the context's stream, no synchronisation (internal)
int bbpp_residual_async(bbpp_ctx *ctx, const uint8_t *mask, const double *rhs, const double *x, double *r) {
  DevState *st = ctx->st + 1, *hst = ctx->hst + 1;
  memset(hst, 0, sizeof(DevState));
  hst->stop = 1;
  CK(cudaMemcpyAsync(st, hst, sizeof(DevState), cudaMemcpyHostToDevice, ctx->stream));
  launch_resid<double, double>(ctx, mask, x, rhs, r, st, RES_INIT);
  CK(cudaGetLastError());
  return 0;
}

extern "C" int bbpp_sphere_mask(bbpp_ctx *ctx, double xs, double ys, double zs, int nsph, const double *cx,
                                const double *cy, const double *cz, const double *rad, uint8_t *mask) {
  if (!ctx || !mask || nsph < 0 || (nsph > 0 && (!cx || !cy || !cz || !rad))) return BBPP_BAD_ARG;
  CK(cudaMemsetAsync(mask, 0, (size_t)ctx->G.n, ctx->stream));
  if (nsph == 0) {
    CK(cudaStreamSynchronize(ctx->stream));
    return 0;
  }
  std::vector<Sphere> h(nsph);
  for (int s = 0; s < nsph; s++) {
    if (!(rad[s] > 0)) return BBPP_BAD_ARG;
    h[s] = Sphere{cx[s], cy[s], cz[s], rad[s]};
  }
  Sphere *d = nullptr;
  CK(cudaMalloc(&d, sizeof(Sphere) * nsph));
  CK(cudaMemcpyAsync(d, h.data(), sizeof(Sphere) * nsph, cudaMemcpyHostToDevice, ctx->stream));
  const int ix = ctx->G.px ? 3 : 1, iy = ctx->G.py ? 3 : 1, iz = ctx->G.pz ? 3 : 1;
  k_sphere_mask<<<nsph * ix * iy * iz, NT, 0, ctx->stream>>>(ctx->G, ctx->grid.dx, ctx->grid.dy, ctx->grid.dz, xs,
                                                              ys, zs, ix, iy, iz, d, mask);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(d);
  CK(e);
  return 0;
}

// ---------------------------------------------------------- memory helpers --
extern "C" int bbpp_dev_alloc(size_t bytes, void **ptr) {
  bbpp_ctx *ctx = nullptr;
  if (!ptr) return BBPP_BAD_ARG;
  CK(cudaMalloc(ptr, bytes ? bytes : 1));
  return 0;
}
extern "C" int bbpp_dev_free(void *ptr) {
  bbpp_ctx *ctx = nullptr;
  CK(cudaFree(ptr));
  return 0;
}
extern "C" int bbpp_h2d(void *dst, const void *src, size_t bytes) {
  bbpp_ctx *ctx = nullptr;
  CK(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
  return 0;
}
extern "C" int bbpp_d2h(void *dst, const void *src, size_t bytes) {
  bbpp_ctx *ctx = nullptr;
  CK(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
  return 0;
}
extern "C" int bbpp_memset(void *dst, int value, size_t bytes) {
  bbpp_ctx *ctx = nullptr;
  CK(cudaMemset(dst, value, bytes));
  return 0;
}
extern "C" int bbpp_sync(void) {
  bbpp_ctx *ctx = nullptr;
  CK(cudaDeviceSynchronize());
  return 0;
}

__global__ void k_flush(uint4 *buf, size_t n, unsigned int v) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    buf[i] = make_uint4(v, v + 1, v + 2, (unsigned)i);
}

extern "C" int bbpp_flush_l2(void) {
  bbpp_ctx *ctx = nullptr;
  static uint4 *buf = nullptr;
  static unsigned int v = 0;
  const size_t bytes = 512ull << 20;  // 4x the 129 MB L2
  if (!buf) CK(cudaMalloc(&buf, bytes));
  k_flush<<<1024, 256>>>(buf, bytes / sizeof(uint4), ++v);
  CK(cudaGetLastError());
  CK(cudaDeviceSynchronize());
  return 0;
}

// FP64 FMA rate of this GPU: eight independent FMA chains per thread, one
// wave of 8 CTAs x 256 threads per SM, timed with CUDA events.  The plain
// FP64 solve is bound by this pipe on parts that issue FP64 at a small
// fraction of the FP32 rate; its roofline is reported against this number.
__global__ void __launch_bounds__(256) k_fp64_fma(double *out, int iters, double a, double b) {
  double v[8];
#pragma unroll
  for (int k = 0; k < 8; k++) v[k] = 1e-3 * (threadIdx.x + 1) + k;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 8; k++) v[k] = fma(v[k], a, b);
  }
  double t = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) t += v[k];
  if (t == -1.0) out[blockIdx.x] = t;  // never true; keeps the chains live
}

extern "C" int bbpp_fp64_fma_rate(double *fma_per_s) {
  bbpp_ctx *ctx = nullptr;
  if (!fma_per_s) return BBPP_BAD_ARG;
  const int sms = dev_sms();
  const int blocks = 8 * sms, threads = 256, iters = 4096;
  double *out = nullptr;
  cudaEvent_t e0, e1;
  CK(cudaMalloc(&out, sizeof(double) * blocks));
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  float best = 0.f;
  for (int rep = 0; rep < 5; rep++) {
    CK(cudaEventRecord(e0));
    k_fp64_fma<<<blocks, threads>>>(out, iters, 0.9999999, 1e-7);
    CK(cudaEventRecord(e1));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    if (rep >= 2 && (best == 0.f || ms < best)) best = ms;  // two warm-ups
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  *fma_per_s = (double)blocks * threads * iters * 8.0 / (best * 1e-3);
  return 0;
}

extern "C" int bbpp_plan_z_chunks(long long units, int nz, long long slots, int min_kz, int *kz) {
  if (units < 1 || nz < 1 || slots < 1 || min_kz < 1 || !kz) return 0;
  return bbpp_z_chunks(units, nz, slots, min_kz, kz);
}

// nb_sum6 over n six-tuples (the FP64 search kernel's interior neighbour sum)
__global__ void k_nb_sum6(const double *__restrict__ in, double *__restrict__ out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double *v = in + 6 * i;
    out[i] = nb_sum6(v[0], v[1], v[2], v[3], v[4], v[5], false);
  }
}

extern "C" int bbpp_neighbour_sums_host(const double *in, double *out, long long n) {
  if (n < 0 || (n > 0 && (!in || !out))) return BBPP_BAD_ARG;
  for (long long i = 0; i < n; i++) {
    const double *v = in + 6 * i;
    out[i] = nb_sum6(v[0], v[1], v[2], v[3], v[4], v[5], false);
  }
  return 0;
}

extern "C" int bbpp_neighbour_sums(const double *in, double *out, long long n) {
  bbpp_ctx *ctx = nullptr;
  if (n < 0 || (n > 0 && (!in || !out)) || n > (1ll << 26)) return BBPP_BAD_ARG;
  if (n == 0) return 0;
  double *d_in = nullptr, *d_out = nullptr;
  cudaError_t e = cudaMalloc(&d_in, sizeof(double) * 6 * n);
  if (e == cudaSuccess) e = cudaMalloc(&d_out, sizeof(double) * n);
  if (e == cudaSuccess) e = cudaMemcpy(d_in, in, sizeof(double) * 6 * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_nb_sum6<<<(unsigned)std::min<long long>((n + 255) / 256, 4096), 256>>>(d_in, d_out, n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out, d_out, sizeof(double) * n, cudaMemcpyDeviceToHost);
  cudaFree(d_in);
  cudaFree(d_out);
  CK(e);
  return 0;
}

// The bandwidth a plain streaming kernel reaches with the fused FP32
// iteration's per-cell traffic: four FP32 reads, one mask byte, four FP32
// writes (33 B/cell), elementwise, no stencil.  It separates what the traffic
// mix allows from what the stencil's pipeline costs.
__global__ void __launch_bounds__(256) k_stream_mix(const float4 *__restrict__ r, const float4 *__restrict__ a,
                                                    const float4 *__restrict__ p, const float4 *__restrict__ x,
                                                    const uchar4 *__restrict__ m, float4 *__restrict__ ro,
                                                    float4 *__restrict__ po, float4 *__restrict__ ao,
                                                    float4 *__restrict__ xo, long long n4) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4; i += (long long)gridDim.x * blockDim.x) {
    float4 rv = r[i], av = a[i], pv = p[i], xv = x[i];
    const uchar4 mv = m[i];
    const float s = mv.x | mv.y | mv.z | mv.w ? 0.f : 1.f;
    rv.x = fmaf(-0.5f, av.x, rv.x);
    rv.y = fmaf(-0.5f, av.y, rv.y);
    rv.z = fmaf(-0.5f, av.z, rv.z);
    rv.w = fmaf(-0.5f, av.w, rv.w);
    pv.x = fmaf(0.5f * s, pv.x, rv.x);
    pv.y = fmaf(0.5f, pv.y, rv.y);
    pv.z = fmaf(0.5f, pv.z, rv.z);
    pv.w = fmaf(0.5f, pv.w, rv.w);
    xv.x += pv.x;
    xv.y += pv.y;
    xv.z += pv.z;
    xv.w += pv.w;
    ro[i] = rv;
    po[i] = pv;
    ao[i] = av;
    xo[i] = xv;
  }
}

extern "C" int bbpp_stream_mix_rate(long long cells, double *bytes_per_s) {
  bbpp_ctx *ctx = nullptr;
  if (!bytes_per_s || cells < 1024 || cells % 4) return BBPP_BAD_ARG;
  float *buf = nullptr;
  unsigned char *m = nullptr;
  cudaEvent_t e0, e1;
  CK(cudaMalloc(&buf, sizeof(float) * 8 * (size_t)cells));
  CK(cudaMalloc(&m, (size_t)cells));
  CK(cudaMemset(buf, 0, sizeof(float) * 8 * (size_t)cells));
  CK(cudaMemset(m, 0, (size_t)cells));
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  const long long n = cells, n4 = cells / 4;
  const int blocks = 16 * dev_sms();
  float best = 0.f;
  for (int rep = 0; rep < 6; rep++) {
    const int rc = bbpp_flush_l2();
    if (rc) return rc;
    CK(cudaEventRecord(e0));
    k_stream_mix<<<blocks, 256>>>((const float4 *)buf, (const float4 *)(buf + n), (const float4 *)(buf + 2 * n),
                                  (const float4 *)(buf + 3 * n), (const uchar4 *)m, (float4 *)(buf + 4 * n),
                                  (float4 *)(buf + 5 * n), (float4 *)(buf + 6 * n), (float4 *)(buf + 7 * n), n4);
    CK(cudaEventRecord(e1));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    if (rep >= 1 && (best == 0.f || ms < best)) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  cudaFree(m);
  *bytes_per_s = 33.0 * (double)cells / (best * 1e-3);
  return 0;
}

// ----------------------------------------------------------- kernel stats --
static const char *kk_name[KK_COUNT] = {"search_spmv", "update", "axpy_x", "resid", "search_spmv_f32",
                                        "update_f32", "axpy_x_f32", "resid_f32", "fused_f32"};

void bbpp_rec_begin(bbpp_ctx *ctx, int kind, double bytes_per_cell) {
  if (!ctx->rec) return;
  KEv k;
  if (!ctx->free_ev.empty()) {
    k = ctx->free_ev.back();
    ctx->free_ev.pop_back();
  } else {
    cudaEventCreate(&k.a);
    cudaEventCreate(&k.b);
  }
  k.kind = kind;
  k.iter = ctx->rec_iter;
  k.bytes = bytes_per_cell * (double)ctx->G.n;
  cudaEventRecord(k.a, ctx->stream);
  ctx->rec->push_back(k);
}

void bbpp_rec_end(bbpp_ctx *ctx) {
  if (!ctx->rec || ctx->rec->empty()) return;
  cudaEventRecord(ctx->rec->back().b, ctx->stream);
}

// Add the device time of the launches that did work (iteration tag <=
// iters_done; the rest returned at once) and optionally release the events.
void bbpp_rec_collect(bbpp_ctx *ctx, std::vector<KEv> &evs, int iters_done, bool release) {
  for (auto &k : evs) {
    if (k.iter <= iters_done) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, k.a, k.b) == cudaSuccess) {
        ctx->kms[k.kind] += ms;
        ctx->klaunch[k.kind] += 1;
        ctx->kbytes[k.kind] += k.bytes;
      } else {
        (void)cudaGetLastError();  // timing is best effort; never leak its error
      }
    }
  }
  if (release) {
    for (auto &k : evs) ctx->free_ev.push_back(k);
    evs.clear();
  }
}

extern "C" int bbpp_set_fused(bbpp_ctx *ctx, int on) {
  if (!ctx || (on != 0 && on != 1)) return BBPP_BAD_ARG;
  ctx->fused = on == 1;
  return 0;
}

extern "C" int bbpp_set_ff_resid(bbpp_ctx *ctx, int on) {
  if (!ctx || (on != 0 && on != 1)) return BBPP_BAD_ARG;
  ctx->ff_resid = on == 1;
  drop_graphs(ctx);  // the replacement kernels are captured in the iteration graphs
  return 0;
}

extern "C" int bbpp_set_trace(bbpp_ctx *ctx, int n) {
  if (!ctx || n < 0 || n > (1 << 20)) return BBPP_BAD_ARG;
  CK(cudaStreamSynchronize(ctx->stream));
  if (ctx->trace) CK(cudaFree(ctx->trace));
  ctx->trace = nullptr;
  ctx->trace_n = 0;
  if (n > 0) {
    CK(cudaMalloc(&ctx->trace, sizeof(double) * 2 * (size_t)n));
    ctx->trace_n = n;
  }
  return 0;
}

extern "C" int bbpp_get_trace(bbpp_ctx *ctx, double *alpha, double *beta, int n) {
  if (!ctx || n < 0 || n > ctx->trace_n || (n > 0 && (!alpha || !beta))) return BBPP_BAD_ARG;
  if (n == 0) return 0;
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaMemcpy(alpha, ctx->trace, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(beta, ctx->trace + ctx->trace_n, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost));
  return 0;
}

extern "C" int bbpp_set_xsum(bbpp_ctx *ctx, int on) {
  if (!ctx || (on != 0 && on != 1)) return BBPP_BAD_ARG;
  ctx->GL.xsum = on;
  drop_graphs(ctx);  // the geometry is a parameter of the captured kernels
  return 0;
}

extern "C" int bbpp_set_profiling(bbpp_ctx *ctx, int on) {
  if (!ctx) return BBPP_BAD_ARG;
  if ((on != 0) != ctx->profiling) drop_graphs(ctx);
  ctx->profiling = on != 0;
  for (int k = 0; k < KK_COUNT; k++) {
    ctx->kms[k] = 0;
    ctx->klaunch[k] = 0;
    ctx->kbytes[k] = 0;
  }
  return 0;
}

extern "C" int bbpp_kernel_stats(bbpp_ctx *ctx, bbpp_kstat *out, int max, int *n) {
  if (!ctx || !n) return BBPP_BAD_ARG;
  int k = 0;
  for (int i = 0; i < KK_COUNT; i++) {
    if (!ctx->klaunch[i]) continue;
    if (out && k < max) {
      memset(&out[k], 0, sizeof(bbpp_kstat));
      snprintf(out[k].name, sizeof(out[k].name), "%s", kk_name[i]);
      out[k].launches = (int)ctx->klaunch[i];
      out[k].ms = ctx->kms[i];
      out[k].bytes = ctx->kbytes[i];
    }
    k++;
  }
  *n = k;
  return 0;
}

extern "C" int bbpp_host_alloc(size_t bytes, void **ptr) {
  bbpp_ctx *ctx = nullptr;
  if (!ptr) return BBPP_BAD_ARG;
  CK(cudaMallocHost(ptr, bytes ? bytes : 1));
  return 0;
}

extern "C" int bbpp_host_free(void *ptr) {
  bbpp_ctx *ctx = nullptr;
  CK(cudaFreeHost(ptr));
  return 0;
}

// ---------------------------------------------------------------- RNG -----
// Ranq1 (src/rng.c:28-51), uniform (src/rng.c:78-81), polar Gaussian
// (src/rng.c:85-107).
namespace {
struct Ranq1 {
  unsigned long long v;
  explicit Ranq1(unsigned long long seed) {
    v = 4101842887655102017ULL;
    v ^= seed;
    v = next();
  }
  unsigned long long next() {
    v ^= v >> 21;
    v ^= v << 35;
    v ^= v >> 4;
    return v * 2685821657736338717ULL;
  }
  double dbl() { return 5.42101086242752217e-20 * (double)next(); }
};
}  // namespace

extern "C" void bbpp_rng_uniform(unsigned long long seed, long long n, double lo, double hi, double *out) {
  Ranq1 g(seed);
  for (long long i = 0; i < n; i++) out[i] = lo + (hi - lo) * g.dbl();
}

extern "C" void bbpp_rng_gauss(unsigned long long seed, long long n, double *out) {
  Ranq1 g(seed);
  long long i = 0;
  while (i < n) {
    double v1, v2, s;
    do {
      const double u1 = g.dbl(), u2 = g.dbl();
      v1 = 2 * u1 - 1;
      v2 = 2 * u2 - 1;
      s = v1 * v1 + v2 * v2;
    } while (s >= 1 || s == 0);
    const double f = std::sqrt(-2 * std::log(s) / s);
    out[i++] = v1 * f;
    if (i < n) out[i++] = v2 * f;
  }
}
