// bbpp_noalloc.cu -- residual evaluation that allocates no memory.
//
// Some callers cannot allocate device memory once they are running: a host
// program that sizes and allocates every device buffer once at start-up and
// must not grow its footprint later (Bluebottle's cuda_dom_malloc_dev is such
// a plan), a process held to a fixed device-memory budget by whoever shares
// the GPU with it, or a time-stepping loop that must not call into the CUDA
// allocator because cudaMalloc and cudaFree can synchronise the device.  For
// them, bbpp_residual_noalloc computes r = rhs - (-A)x and the two norms with
// the same kernel as bbpp_residual, but takes no context and allocates
// nothing: its reduction scratch is the file-scope device array below.
//
// The scratch holds one solver state and BBPP_NOALLOC_MAX_CTAS x 3 partial
// sums (about 200 KB).  Every GPU that loads this library holds that array
// until the process exits.  Grids whose stencil launch would need more CTAs
// than that are rejected with BBPP_BAD_ARG and a message.
//
// All calls share the array and it keeps the contents of the last call; each
// call clears the part that must start at zero.  Calls whose work overlaps on
// the GPU (on different streams, or from different host threads) race on the
// array, so callers must order them.
//
// Host code cannot use the array's name as a device address: on the host it
// names a stand-in, not device memory.  So every call looks the device address
// up with cudaGetSymbolAddress while the caller's device is current (a table
// lookup in the CUDA runtime; it allocates nothing) and passes that address to
// the kernel.  Looking it up on every call, not once per device, keeps the
// address valid for the context that is current now, also after a
// cudaDeviceReset has replaced the one the previous call ran in.  The first
// call on a device also loads this library's device code there, so make that
// first call before any stream capture on that device.  Each call waits for
// its stream (it copies the two norms to the host) before it returns.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>

#include "../../include/bbpp.h"
#include "bbpp_internal.h"
#include "bbpp_kernels.cuh"

using namespace bbpp;

namespace {

struct NoallocScratch {
  DevState st;
  double partials[3 * BBPP_NOALLOC_MAX_CTAS];
};

__device__ __align__(256) unsigned char g_scratch[sizeof(NoallocScratch)];

int fail(int rc, const char *msg) {
  fprintf(stderr, "bbpp_residual_noalloc: %s\n", msg);
  return rc;
}

}  // namespace

extern "C" int bbpp_residual_noalloc(const bbpp_grid *g, const uint8_t *mask, const double *rhs, const double *x,
                                     double *r, double *rr, double *bb, void *stream) {
  if (!g || !rhs || !x || !r) return fail(BBPP_BAD_ARG, "null argument");
  Geo G;
  int rc = bbpp_geo_init(g, &G);
  if (rc) return fail(rc, "invalid grid (sizes, spacings or boundary types)");
  // launch shape of the stencil kernel within the scratch capacity
  const long long gx = (G.nx + TX - 1) / TX, gy = (G.ny + TY - 1) / TY;
  if (gx * gy > BBPP_NOALLOC_MAX_CTAS) {
    char m[200];
    snprintf(m, sizeof(m), "grid %dx%dx%d needs %lld column tiles, more than the %d the scratch holds", G.nx, G.ny,
             G.nz, gx * gy, BBPP_NOALLOC_MAX_CTAS);
    return fail(BBPP_BAD_ARG, m);
  }
  const long long nzc = std::max<long long>(1, std::min<long long>(G.nz, BBPP_NOALLOC_MAX_CTAS / (gx * gy)));
  const int kz = (int)((G.nz + nzc - 1) / nzc);
  const dim3 grid((unsigned)gx, (unsigned)gy, (unsigned)((G.nz + kz - 1) / kz));

  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return fail(BBPP_NO_DEVICE, "no current CUDA device");
  // the device address of the scratch in the context current now
  void *base = nullptr;
  const cudaError_t ea = cudaGetSymbolAddress(&base, g_scratch);
  if (ea != cudaSuccess || !base) {
    char m[200];
    snprintf(m, sizeof(m), "cudaGetSymbolAddress failed on device %d: %s", dev, cudaGetErrorString(ea));
    return fail(BBPP_CUDA_ERROR, m);
  }
  NoallocScratch *sc = reinterpret_cast<NoallocScratch *>(base);
  cudaStream_t s = (cudaStream_t)stream;
  // the solver state (ticket counter, thresholds) must start at zero
  cudaError_t e = cudaMemsetAsync(&sc->st, 0, sizeof(DevState), s);
  if (e == cudaSuccess) {
    if (mask)
      k_resid<double, double, true><<<grid, NT, 0, s>>>(G, x, rhs, r, mask, &sc->st, sc->partials, kz, RES_INIT);
    else
      k_resid<double, double, false><<<grid, NT, 0, s>>>(G, x, rhs, r, mask, &sc->st, sc->partials, kz, RES_INIT);
    e = cudaGetLastError();
  }
  DevState h;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, &sc->st, sizeof(DevState), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    char m[200];
    snprintf(m, sizeof(m), "CUDA error: %s", cudaGetErrorString(e));
    return fail(BBPP_CUDA_ERROR, m);
  }
  if (rr) *rr = h.rr;
  if (bb) *bb = h.bb;
  return BBPP_CONVERGED;
}
