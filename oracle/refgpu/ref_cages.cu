// ref_cages.cu -- host harness that runs the reference's own cage builder on
// the GPU (test and measurement infrastructure; never part of the product).
//
// The kernels (src/particle_kernel.cu, unmodified) come compiled in
// oracle/_ref/ref_cages.cubin.  This file restates the one-rank host side of
// cuda_build_cages (src/cuda_particle.cu:1516-1646) and launches them through
// the driver API: the flag and phase resets, then per particle in index order
// cage_setup, a device-to-host copy of the cage size and build_phase, the same
// loop with build_phase_shell, then cage_flag_u/v/w and flag_external_* on the
// walls of non-periodic directions.  The whole sequence is timed with CUDA
// events, host copies included, as the time loop pays it.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

namespace {

typedef CUresult (*PFN_load)(CUmodule *, const void *);
typedef CUresult (*PFN_getfn)(CUfunction *, CUmodule, const char *);
typedef CUresult (*PFN_getglobal)(CUdeviceptr *, size_t *, CUmodule, const char *);
typedef CUresult (*PFN_launch)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned,
                               CUstream, void **, void **);
typedef CUresult (*PFN_unload)(CUmodule);

struct CageRef {
  PFN_load load = nullptr;
  PFN_getfn getfn = nullptr;
  PFN_getglobal getglobal = nullptr;
  PFN_launch launch = nullptr;
  PFN_unload unload = nullptr;
  CUmodule mod = nullptr;
  CUfunction f_fill, f_layout, f_bc, f_rfu, f_rfv, f_rfw, f_rph, f_setup, f_phase, f_shell, f_cfu, f_cfv, f_cfw,
      f_efu, f_efv, f_efw;
  int nx = 0, ny = 0, nz = 0, bc[6] = {0, 0, 0, 0, 0, 0};
  long long info[16], layout[7];
  int *phase = nullptr, *shell = nullptr, *fu = nullptr, *fv = nullptr, *fw = nullptr, *cage_dim = nullptr;
  void *dom = nullptr, *bcs = nullptr;
  char err[256] = {0};
};

CageRef *g_cr = nullptr;
std::vector<unsigned char> g_cages_cubin;
constexpr int MAXT = 16;  // MAX_THREADS_DIM, src/bluebottle.h:205

int cdiv(int a, int b) { return (a + b - 1) / b; }
int thr(int n) { return n < MAXT ? n : MAXT; }

bool go(CageRef *R, CUfunction f, dim3 g, dim3 b, void **args) {
  if (R->launch(f, g.x, g.y, g.z, b.x, b.y, b.z, 0, 0, args, nullptr) != CUDA_SUCCESS) {
    snprintf(R->err, sizeof(R->err), "cuLaunchKernel failed");
    return false;
  }
  return true;
}

void release(CageRef *R) {
  for (void *q : {(void *)R->phase, (void *)R->shell, (void *)R->fu, (void *)R->fv, (void *)R->fw,
                  (void *)R->cage_dim, R->dom, R->bcs})
    if (q) cudaFree(q);
  if (R->mod) R->unload(R->mod);
  delete R;
}

}  // namespace

extern "C" {

int refgpu_cages_set_cubin(const void *data, size_t bytes) {
  g_cages_cubin.assign((const unsigned char *)data, (const unsigned char *)data + bytes);
  return 0;
}

const char *refgpu_cages_error(void) { return g_cr ? g_cr->err : "no setup"; }

void refgpu_cages_free(void) {
  if (g_cr) release(g_cr);
  g_cr = nullptr;
}

// One rank on [0, nx dx] x [0, ny dy] x [0, nz dz] with pressure BCs bcs[6]
// (W, E, S, N, B, T; 0 periodic).  Returns 0 or an error code.
int refgpu_cages_setup(int nx, int ny, int nz, double dx, double dy, double dz, const int *bcs) {
  refgpu_cages_free();
  if (g_cages_cubin.empty() || nx < 1 || ny < 1 || nz < 1) return 1;
  CageRef *R = new CageRef();
  g_cr = R;
  cudaFree(0);
  cudaDriverEntryPointQueryResult q;
  void *p;
#define GET(field, name)                                                                                   \
  if (cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||        \
      q != cudaDriverEntryPointSuccess)                                                                    \
    return 2;                                                                                              \
  R->field = reinterpret_cast<decltype(R->field)>(p);
  GET(load, "cuModuleLoadData")
  GET(getfn, "cuModuleGetFunction")
  GET(getglobal, "cuModuleGetGlobal")
  GET(launch, "cuLaunchKernel")
  GET(unload, "cuModuleUnload")
#undef GET
  if (R->load(&R->mod, g_cages_cubin.data()) != CUDA_SUCCESS) {
    snprintf(R->err, sizeof(R->err), "cuModuleLoadData failed");
    return 3;
  }
  struct {
    CUfunction *f;
    const char *name;
  } fns[] = {{&R->f_fill, "refgpu_fill_dom"},
             {&R->f_layout, "refgpu_part_layout"},
             {&R->f_bc, "refgpu_fill_bc"},
             {&R->f_rfu, "_Z12reset_flag_uPi"},
             {&R->f_rfv, "_Z12reset_flag_vPi"},
             {&R->f_rfw, "_Z12reset_flag_wPi"},
             {&R->f_rph, "_Z12reset_phasesPiS_"},
             {&R->f_setup, "_Z10cage_setupP11part_structiPi"},
             {&R->f_phase, "_Z11build_phaseP11part_structiPiS1_S1_P10dom_structP2BC"},
             {&R->f_shell, "_Z17build_phase_shellP11part_structiPiS1_S1_P10dom_structP2BC"},
             {&R->f_cfu, "_Z11cage_flag_uPiS_S_"},
             {&R->f_cfv, "_Z11cage_flag_vPiS_S_"},
             {&R->f_cfw, "_Z11cage_flag_wPiS_S_"},
             {&R->f_efu, "_Z15flag_external_uPii"},
             {&R->f_efv, "_Z15flag_external_vPii"},
             {&R->f_efw, "_Z15flag_external_wPii"}};
  for (auto &f : fns)
    if (R->getfn(f.f, R->mod, f.name) != CUDA_SUCCESS) {
      snprintf(R->err, sizeof(R->err), "kernel %s not in the image", f.name);
      return 4;
    }
  R->nx = nx;
  R->ny = ny;
  R->nz = nz;
  for (int k = 0; k < 6; k++) R->bc[k] = bcs[k];
  CUdeviceptr dom_sym;
  size_t dom_bytes = 0;
  if (R->getglobal(&dom_sym, &dom_bytes, R->mod, "_dom") != CUDA_SUCCESS) {
    snprintf(R->err, sizeof(R->err), "_dom not in the image");
    return 5;
  }
  long long *dinfo = nullptr;
  if (cudaMalloc(&R->dom, dom_bytes + 256) != cudaSuccess || cudaMalloc(&dinfo, sizeof(long long) * 16) != cudaSuccess)
    return 6;
  {
    void *args[] = {&R->dom, &dinfo, &nx, &ny, &nz, &dx, &dy, &dz};
    if (!go(R, R->f_fill, dim3(1), dim3(1), args)) return 6;
  }
  cudaMemcpy(R->info, dinfo, sizeof(long long) * 16, cudaMemcpyDeviceToHost);
  {
    void *args[] = {&dinfo};
    if (!go(R, R->f_layout, dim3(1), dim3(1), args)) return 6;
  }
  cudaMemcpy(R->layout, dinfo, sizeof(long long) * 7, cudaMemcpyDeviceToHost);
  cudaFree(dinfo);
  if (R->info[15] != (long long)dom_bytes) {
    snprintf(R->err, sizeof(R->err), "domain struct size mismatch");
    return 7;
  }
  // _dom (the constant the kernels read) and the DOM pointer build_phase takes: one rank, the same struct
  cudaMemcpy((void *)dom_sym, R->dom, dom_bytes, cudaMemcpyDeviceToDevice);
  if (cudaMalloc(&R->bcs, (size_t)R->layout[6] + 64) != cudaSuccess) return 6;
  {
    void *args[] = {&R->bcs, &R->bc[0], &R->bc[1], &R->bc[2], &R->bc[3], &R->bc[4], &R->bc[5]};
    if (!go(R, R->f_bc, dim3(1), dim3(1), args)) return 6;
  }
  const long long s3b = R->info[2];
  if (cudaMalloc(&R->phase, sizeof(int) * s3b) != cudaSuccess || cudaMalloc(&R->shell, sizeof(int) * s3b) != cudaSuccess ||
      cudaMalloc(&R->fu, sizeof(int) * R->info[8]) != cudaSuccess ||
      cudaMalloc(&R->fv, sizeof(int) * R->info[11]) != cudaSuccess ||
      cudaMalloc(&R->fw, sizeof(int) * R->info[14]) != cudaSuccess || cudaMalloc(&R->cage_dim, sizeof(int) * 4) != cudaSuccess)
    return 6;
  if (cudaDeviceSynchronize() != cudaSuccess) return 8;
  return 0;
}

// sizes of the outputs: Gcc s3b, Gfx s3b, Gfy s3b, Gfz s3b; sizeof(part_struct) and offsets of N, r, x, y, z
void refgpu_cages_sizes(long long *out) {
  out[0] = g_cr->info[2];
  out[1] = g_cr->info[8];
  out[2] = g_cr->info[11];
  out[3] = g_cr->info[14];
  for (int k = 0; k < 6; k++) out[4 + k] = g_cr->layout[k];
}

// parts: np part_structs in the reference's layout (host bytes); with_parts:
// NPARTS > 0.  Outputs to host arrays of the sizes above; *ms = the device
// time of the whole builder, host copies included.
int refgpu_build_cages(int with_parts, int np, const void *parts, int *phase, int *shell, int *fu, int *fv, int *fw,
                       double *ms) {
  CageRef *R = g_cr;
  if (!R) return 1;
  void *dparts = nullptr;
  const size_t pbytes = (size_t)R->layout[0] * (size_t)(np > 0 ? np : 1);
  if (cudaMalloc(&dparts, pbytes) != cudaSuccess) return 6;
  if (np > 0) cudaMemcpy(dparts, parts, pbytes, cudaMemcpyHostToDevice);
  const int jnb = R->ny + 2, knb = R->nz + 2, inb = R->nx + 2;
  // cuda_blocks_init's shapes for the face grids' inb / jnb / knb launches
  const dim3 fx_b(thr(jnb), thr(knb)), fx_g(cdiv(jnb, thr(jnb)), cdiv(knb, thr(knb)));
  const dim3 fy_b(thr(knb), thr(inb)), fy_g(cdiv(knb, thr(knb)), cdiv(inb, thr(inb)));
  const dim3 fz_b(thr(inb), thr(jnb)), fz_g(cdiv(inb, thr(inb)), cdiv(jnb, thr(jnb)));
  const dim3 cc_b(thr(inb), thr(jnb)), cc_g(cdiv(inb, thr(inb)), cdiv(jnb, thr(jnb)));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaDeviceSynchronize();
  cudaEventRecord(e0);
  bool ok = true;
  {
    void *a1[] = {&R->fu};
    void *a2[] = {&R->fv};
    void *a3[] = {&R->fw};
    ok = ok && go(R, R->f_rfu, fx_g, fx_b, a1) && go(R, R->f_rfv, fy_g, fy_b, a2) && go(R, R->f_rfw, fz_g, fz_b, a3);
  }
  if (ok && with_parts > 0) {
    void *ar[] = {&R->phase, &R->shell};
    ok = go(R, R->f_rph, cc_g, cc_b, ar);
    const int tx = (int)(0.5 * MAXT), ty = tx, tz = tx;
    const double itx = 1. / tx, ity = 1. / ty, itz = 1. / tz;
    int cd[4];
    for (int pass = 0; pass < 2 && ok; pass++)
      for (int n = 0; n < np && ok; n++) {
        void *as[] = {&dparts, &n, &R->cage_dim};
        ok = go(R, R->f_setup, dim3(1), dim3(1), as);
        cudaMemcpy(cd, R->cage_dim, 3 * sizeof(int), cudaMemcpyDeviceToHost);
        const int bx = (int)ceil((double)cd[0] * itx), by = (int)ceil((double)cd[1] * ity),
                  bz = (int)ceil((double)cd[2] * itz);
        if (ok && bx > 0 && by > 0 && bz > 0) {
          void *ab[] = {&dparts, &n, &R->cage_dim, &R->phase, &R->shell, &R->dom, &R->bcs};
          ok = go(R, pass == 0 ? R->f_phase : R->f_shell, dim3(bx, by, bz), dim3(tx, ty, tz), ab);
        }
      }
    void *c1[] = {&R->fu, &R->phase, &R->shell};
    void *c2[] = {&R->fv, &R->phase, &R->shell};
    void *c3[] = {&R->fw, &R->phase, &R->shell};
    ok = ok && go(R, R->f_cfu, fx_g, fx_b, c1) && go(R, R->f_cfv, fy_g, fy_b, c2) && go(R, R->f_cfw, fz_g, fz_b, c3);
  }
  // flag_external_* on both walls of a non-periodic direction (one rank: first and last subdomain)
  int lo = 1, hx = R->nx + 1, hy = R->ny + 1, hz = R->nz + 1;
  if (ok && R->bc[0] != 0 && R->bc[1] != 0) {
    void *a[] = {&R->fu, &lo};
    void *b[] = {&R->fu, &hx};
    ok = go(R, R->f_efu, fx_g, fx_b, a) && go(R, R->f_efu, fx_g, fx_b, b);
  }
  if (ok && R->bc[2] != 0 && R->bc[3] != 0) {
    void *a[] = {&R->fv, &lo};
    void *b[] = {&R->fv, &hy};
    ok = go(R, R->f_efv, fy_g, fy_b, a) && go(R, R->f_efv, fy_g, fy_b, b);
  }
  if (ok && R->bc[4] != 0 && R->bc[5] != 0) {
    void *a[] = {&R->fw, &lo};
    void *b[] = {&R->fw, &hz};
    ok = go(R, R->f_efw, fz_g, fz_b, a) && go(R, R->f_efw, fz_g, fz_b, b);
  }
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float t = 0.f;
  cudaEventElapsedTime(&t, e0, e1);
  *ms = t;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(dparts);
  if (!ok) return 9;
  cudaMemcpy(phase, R->phase, sizeof(int) * R->info[2], cudaMemcpyDeviceToHost);
  cudaMemcpy(shell, R->shell, sizeof(int) * R->info[2], cudaMemcpyDeviceToHost);
  cudaMemcpy(fu, R->fu, sizeof(int) * R->info[8], cudaMemcpyDeviceToHost);
  cudaMemcpy(fv, R->fv, sizeof(int) * R->info[11], cudaMemcpyDeviceToHost);
  cudaMemcpy(fw, R->fw, sizeof(int) * R->info[14], cudaMemcpyDeviceToHost);
  return cudaGetLastError() == cudaSuccess ? 0 : 10;
}

}  // extern "C"
