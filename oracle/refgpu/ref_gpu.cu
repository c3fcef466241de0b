// ref_gpu.cu -- host harness that runs the reference's own CUDA pressure solve
// on the GPU (test and measurement infrastructure; never part of the product).
//
// The reference's kernels (src/solver_kernel.cu, unmodified) come compiled in
// oracle/_ref/ref_solver.cubin (built from the reference tree by
// build_cubin.py).  This file restates the host side that Bluebottle wraps
// around them on one rank and launches those kernels through the driver API:
//   * the solver loops cuda_PP_cg / cuda_PP_cg_noparts
//     (src/cuda_solver.cu:38-300, :573-761): the same kernels, launch shapes,
//     thrust::inner_product dot products (the same library call, with its host
//     synchronisation), residual replacement every 50 iterations, stopping
//     test (r,z) <= pp_residual^2 (b,b), the (b,b) < 1e-16 exit;
//   * cuda_PP_init_jacobi_preconditioner (src/cuda_solver.cu:31-36);
//   * launch shapes of cuda_blocks_init (src/cuda_bluebottle.cu:511-581);
//   * the one-rank ghost exchange in place of mpi_cuda_exchange_Gcc
//     (src/mpi_comm.c:257-315): a periodic direction's ghost plane is the
//     opposite interior plane, a Neumann ghost is not written;
//   * part_BC_p's effect on the solve (src/particle_kernel.cu:1753): solid rhs
//     is zero; and the phase / face flags of a sphere mask (cage_flag_*,
//     flag_external_*: -1 across a fluid/solid face, 0 on a wall face).
// The right-hand side is injected into the interior of _rhs_p where the
// reference would call PP_rhs (the same substitution as the host pin).
#include <cuda.h>
#include <cuda_runtime.h>
#include <thrust/device_ptr.h>
#include <thrust/inner_product.h>

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

struct Drv {
  PFN_load load = nullptr;
  PFN_getfn getfn = nullptr;
  PFN_getglobal getglobal = nullptr;
  PFN_launch launch = nullptr;
  PFN_unload unload = nullptr;
};

bool get_drv(Drv &d) {
  cudaDriverEntryPointQueryResult q;
  void *p;
#define GET(field, name)                                                                                   \
  if (cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||        \
      q != cudaDriverEntryPointSuccess)                                                                    \
    return false;                                                                                          \
  d.field = reinterpret_cast<decltype(d.field)>(p);
  GET(load, "cuModuleLoadData")
  GET(getfn, "cuModuleGetFunction")
  GET(getglobal, "cuModuleGetGlobal")
  GET(launch, "cuLaunchKernel")
  GET(unload, "cuModuleUnload")
#undef GET
  return true;
}

constexpr int PERIODIC = 0;    // pressure BC codes of the reference (src/bluebottle.h)
constexpr int MAX_THREADS_DIM = 16;  // src/bluebottle.h:205
constexpr int SLACK = 4096;    // extra elements on every device array

struct Shape {
  dim3 num, dim;
};

struct Ref {
  Drv drv;
  CUmodule mod = nullptr;
  CUfunction f_jacobi, f_cg_init, f_spmv, f_spmv_np, f_soln_resid, f_solution, f_residual, f_search, f_refine,
      f_zero_i, f_zero_j, f_zero_k, f_fill;
  int nx = 0, ny = 0, nz = 0, bc[6] = {0, 0, 0, 0, 0, 0};
  bool parts = false;
  long long info[16];
  // Gcc strides, face-grid strides
  long long s1b, s2b, s3b, s3, fx1, fx2, fx3, fy1, fy2, fy3, fz1, fz2, fz3;
  double *phi = nullptr, *rhs = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *pb = nullptr, *Ap = nullptr,
         *invM = nullptr, *inj = nullptr;
  int *flag_u = nullptr, *flag_v = nullptr, *flag_w = nullptr, *phase = nullptr;
  Shape kn, kn_s, inb, jnb, knb;
  char err[256] = {0};
};

Ref *g_ref = nullptr;
std::vector<unsigned char> g_cubin;

int cdiv(int a, int b) { return (a + b - 1) / b; }
int threads_of(int n) { return n < MAX_THREADS_DIM ? n : MAX_THREADS_DIM; }

bool launch(Ref *R, CUfunction f, const Shape &s, void **args) {
  CUresult e = R->drv.launch(f, s.num.x, s.num.y, s.num.z, s.dim.x, s.dim.y, s.dim.z, 0, 0, args, nullptr);
  if (e != CUDA_SUCCESS) {
    snprintf(R->err, sizeof(R->err), "cuLaunchKernel failed (%d)", (int)e);
    return false;
  }
  return true;
}

// ---------------------------------------------------------------- helpers --
// one-rank ghost exchange of an s3b Gcc array: x, then y, then z, each over the
// full ghosted extent of the previous directions
template <typename T>
__global__ void ex_x(T *a, int inb, int jnb, int knb, long long s1, long long s2) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
  if (j >= jnb || k >= knb) return;
  const long long row = j * s1 + k * s2;
  a[row + 0] = a[row + (inb - 2)];
  a[row + (inb - 1)] = a[row + 1];
}
template <typename T>
__global__ void ex_y(T *a, int inb, int jnb, int knb, long long s1, long long s2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
  if (i >= inb || k >= knb) return;
  const long long b = i + k * s2;
  a[b + 0 * s1] = a[b + (jnb - 2) * s1];
  a[b + (jnb - 1) * s1] = a[b + 1 * s1];
}
template <typename T>
__global__ void ex_z(T *a, int inb, int jnb, int knb, long long s1, long long s2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i >= inb || j >= jnb) return;
  const long long b = i + j * s1;
  a[b + 0 * s2] = a[b + (knb - 2) * s2];
  a[b + (knb - 1) * s2] = a[b + 1 * s2];
}

template <typename T>
void exchange(Ref *R, T *a) {
  const int inb = R->nx + 2, jnb = R->ny + 2, knb = R->nz + 2;
  if (R->bc[0] == PERIODIC) ex_x<T><<<dim3(cdiv(jnb, 128), knb), 128>>>(a, inb, jnb, knb, R->s1b, R->s2b);
  if (R->bc[2] == PERIODIC) ex_y<T><<<dim3(cdiv(inb, 128), knb), 128>>>(a, inb, jnb, knb, R->s1b, R->s2b);
  if (R->bc[4] == PERIODIC) ex_z<T><<<dim3(cdiv(inb, 128), jnb), 128>>>(a, inb, jnb, knb, R->s1b, R->s2b);
}

// rhs interior (s3b) <- dense (nz, ny, nx)
__global__ void k_inject(double *rhs, const double *dense, int nx, int ny, int nz, long long s1b, long long s2b) {
  const long long n = (long long)nx * ny * nz;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(c % nx);
    const long long t = c / nx;
    const int j = (int)(t % ny), k = (int)(t / ny);
    rhs[(i + 1) + (j + 1) * s1b + (k + 1) * s2b] = dense[c];
  }
}

// dense (nz, ny, nx) <- phi interior
__global__ void k_extract(double *dense, const double *phi, int nx, int ny, int nz, long long s1b, long long s2b) {
  const long long n = (long long)nx * ny * nz;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(c % nx);
    const long long t = c / nx;
    const int j = (int)(t % ny), k = (int)(t / ny);
    dense[c] = phi[(i + 1) + (j + 1) * s1b + (k + 1) * s2b];
  }
}

// part_BC_p's effect: rhs of solid cells is zero (src/particle_kernel.cu:1753)
__global__ void k_part_bc(double *rhs, const int *phase, long long n) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
    if (phase[c] > -1) rhs[c] = 0.;
}

void release(Ref *R) {
  for (void *q : {(void *)R->phi, (void *)R->rhs, (void *)R->r, (void *)R->z, (void *)R->p, (void *)R->pb,
                  (void *)R->Ap, (void *)R->invM, (void *)R->inj, (void *)R->flag_u, (void *)R->flag_v,
                  (void *)R->flag_w, (void *)R->phase})
    if (q) cudaFree(q);
  if (R->mod) R->drv.unload(R->mod);
  delete R;
}

template <typename T>
T *dalloc(long long n) {
  T *q = nullptr;
  if (cudaMalloc(&q, sizeof(T) * (size_t)(n + SLACK)) != cudaSuccess) return nullptr;
  cudaMemset(q, 0, sizeof(T) * (size_t)(n + SLACK));
  return q;
}

double dot(const double *a, const double *b, long long n) {
  thrust::device_ptr<const double> ta(a), tb(b);
  return thrust::inner_product(ta, ta + n, tb, 0.);
}

}  // namespace

extern "C" {

// The reference kernels' image: the bytes of ref_solver.cubin.
int refgpu_set_cubin(const void *data, size_t bytes) {
  g_cubin.assign((const unsigned char *)data, (const unsigned char *)data + bytes);
  return 0;
}

const char *refgpu_error(void) { return g_ref ? g_ref->err : "no setup"; }

void refgpu_free(void) {
  if (g_ref) release(g_ref);
  g_ref = nullptr;
}

// Single-rank domain [0, nx dx] x ... with pressure BCs (W,E,S,N,B,T; 0 =
// periodic, otherwise Neumann) and an optional solid mask (dense (nz,ny,nx),
// 1 = solid; NULL runs cuda_PP_cg_noparts).  Builds flags and phase and runs
// the reference's Jacobi initialisation.
int refgpu_setup(int nx, int ny, int nz, double dx, double dy, double dz, const int *bcs, const uint8_t *mask) {
  refgpu_free();
  if (g_cubin.empty() || nx < 1 || ny < 1 || nz < 1) return 1;
  Ref *R = new Ref();
  g_ref = R;
  cudaFree(0);
  if (!get_drv(R->drv)) {
    snprintf(R->err, sizeof(R->err), "driver entry points unavailable");
    return 2;
  }
  if (R->drv.load(&R->mod, g_cubin.data()) != CUDA_SUCCESS) {
    snprintf(R->err, sizeof(R->err), "cuModuleLoadData failed");
    return 3;
  }
  struct {
    CUfunction *f;
    const char *name;
  } fns[] = {{&R->f_jacobi, "_Z14PP_jacobi_initPiS_S_Pd"},
             {&R->f_cg_init, "_Z10PP_cg_initPdS_S_S_S_S_S_"},
             {&R->f_spmv, "_Z19PP_spmv_shared_loadPiS_S_PdS0_S_"},
             {&R->f_spmv_np, "_Z27PP_spmv_shared_load_nopartsPiS_S_PdS0_"},
             {&R->f_soln_resid, "_Z20PP_update_soln_residPdS_S_S_S_dS_"},
             {&R->f_solution, "_Z18PP_update_solutionPdS_d"},
             {&R->f_residual, "_Z18PP_update_residualPdS_S_S_S_"},
             {&R->f_search, "_Z16PP_update_searchPdS_S_d"},
             {&R->f_refine, "_Z13coeffs_refinePdPiS0_S0_S0_"},
             {&R->f_zero_i, "_Z16zero_rhs_ghost_iPd"},
             {&R->f_zero_j, "_Z16zero_rhs_ghost_jPd"},
             {&R->f_zero_k, "_Z16zero_rhs_ghost_kPd"},
             {&R->f_fill, "refgpu_fill_dom"}};
  for (auto &f : fns)
    if (R->drv.getfn(f.f, R->mod, f.name) != CUDA_SUCCESS) {
      snprintf(R->err, sizeof(R->err), "kernel %s not in the image", f.name);
      return 4;
    }
  R->nx = nx;
  R->ny = ny;
  R->nz = nz;
  for (int q = 0; q < 6; q++) R->bc[q] = bcs ? bcs[q] : PERIODIC;
  R->parts = mask != nullptr;
  // the domain struct, built on the device in the reference's layout
  CUdeviceptr dom_sym;
  size_t dom_bytes = 0;
  if (R->drv.getglobal(&dom_sym, &dom_bytes, R->mod, "_dom") != CUDA_SUCCESS) {
    snprintf(R->err, sizeof(R->err), "_dom not in the image");
    return 5;
  }
  void *dbuf = nullptr;
  long long *dinfo = nullptr;
  cudaMalloc(&dbuf, dom_bytes + 256);
  cudaMalloc(&dinfo, sizeof(long long) * 16);
  {
    void *args[] = {&dbuf, &dinfo, &nx, &ny, &nz, &dx, &dy, &dz};
    Shape one{dim3(1), dim3(1)};
    if (!launch(R, R->f_fill, one, args)) return 6;
  }
  cudaMemcpy(R->info, dinfo, sizeof(long long) * 16, cudaMemcpyDeviceToHost);
  if (R->info[15] != (long long)dom_bytes) {
    snprintf(R->err, sizeof(R->err), "domain struct size mismatch (%lld vs %zu)", R->info[15], dom_bytes);
    cudaFree(dbuf);
    cudaFree(dinfo);
    return 7;
  }
  cudaMemcpy((void *)dom_sym, dbuf, dom_bytes, cudaMemcpyDeviceToDevice);
  cudaFree(dbuf);
  cudaFree(dinfo);
  R->s1b = R->info[0]; R->s2b = R->info[1]; R->s3b = R->info[2]; R->s3 = R->info[5];
  R->fx1 = R->info[6]; R->fx2 = R->info[7]; R->fx3 = R->info[8];
  R->fy1 = R->info[9]; R->fy2 = R->info[10]; R->fy3 = R->info[11];
  R->fz1 = R->info[12]; R->fz2 = R->info[13]; R->fz3 = R->info[14];
  // launch shapes (cuda_blocks_init for Gcc)
  {
    int tx = threads_of(nx), ty = threads_of(ny), tz;
    R->kn = {dim3(cdiv(nx, tx), cdiv(ny, ty)), dim3(tx, ty)};
    tx = threads_of(nx + 2);
    ty = threads_of(ny + 2);
    R->kn_s = {dim3(cdiv(nx, tx - 2), cdiv(ny, ty - 2)), dim3(tx, ty)};
    tx = threads_of(nx + 2);
    ty = threads_of(ny + 2);
    tz = threads_of(nz + 2);
    R->inb = {dim3(cdiv(ny + 2, ty), cdiv(nz + 2, tz)), dim3(ty, tz)};
    R->jnb = {dim3(cdiv(nz + 2, tz), cdiv(nx + 2, tx)), dim3(tz, tx)};
    R->knb = {dim3(cdiv(nx + 2, tx), cdiv(ny + 2, ty)), dim3(tx, ty)};
  }
  R->phi = dalloc<double>(R->s3b);
  R->rhs = dalloc<double>(R->s3b);
  R->pb = dalloc<double>(R->s3b);
  R->r = dalloc<double>(R->s3);
  R->z = dalloc<double>(R->s3);
  R->p = dalloc<double>(R->s3);
  R->Ap = dalloc<double>(R->s3);
  R->invM = dalloc<double>(R->s3);
  R->inj = dalloc<double>(R->s3);
  R->phase = dalloc<int>(R->s3b);
  R->flag_u = dalloc<int>(R->fx3);
  R->flag_v = dalloc<int>(R->fy3);
  R->flag_w = dalloc<int>(R->fz3);
  if (!R->phi || !R->rhs || !R->pb || !R->r || !R->z || !R->p || !R->Ap || !R->invM || !R->inj || !R->phase ||
      !R->flag_u || !R->flag_v || !R->flag_w) {
    snprintf(R->err, sizeof(R->err), "out of device memory");
    return 8;
  }
  // phase (-1 fluid, 0 solid) and face flags on the host, as the host pin does
  const int inb = nx + 2, jnb = ny + 2, knb = nz + 2;
  std::vector<int> ph((size_t)R->s3b, -1);
  auto ccb = [&](int i, int j, int k) { return (size_t)i + (size_t)j * R->s1b + (size_t)k * R->s2b; };
  if (mask)
    for (int k = 0; k < nz; k++)
      for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++)
          if (mask[(size_t)i + (size_t)nx * (j + (size_t)ny * k)]) ph[ccb(i + 1, j + 1, k + 1)] = 0;
  // periodic ghosts of the phase
  if (R->bc[0] == PERIODIC)
    for (int k = 0; k < knb; k++)
      for (int j = 0; j < jnb; j++) {
        ph[ccb(0, j, k)] = ph[ccb(inb - 2, j, k)];
        ph[ccb(inb - 1, j, k)] = ph[ccb(1, j, k)];
      }
  if (R->bc[2] == PERIODIC)
    for (int k = 0; k < knb; k++)
      for (int i = 0; i < inb; i++) {
        ph[ccb(i, 0, k)] = ph[ccb(i, jnb - 2, k)];
        ph[ccb(i, jnb - 1, k)] = ph[ccb(i, 1, k)];
      }
  if (R->bc[4] == PERIODIC)
    for (int j = 0; j < jnb; j++)
      for (int i = 0; i < inb; i++) {
        ph[ccb(i, j, 0)] = ph[ccb(i, j, knb - 2)];
        ph[ccb(i, j, knb - 1)] = ph[ccb(i, j, 1)];
      }
  // GFX_LOC = j + k s1b + i s2b; GFY_LOC = k + i s1b + j s2b; GFZ_LOC = i + j s1b + k s2b
  auto fx = [&](int i, int j, int k) { return (size_t)j + (size_t)k * R->fx1 + (size_t)i * R->fx2; };
  auto fy = [&](int i, int j, int k) { return (size_t)k + (size_t)i * R->fy1 + (size_t)j * R->fy2; };
  auto fz = [&](int i, int j, int k) { return (size_t)i + (size_t)j * R->fz1 + (size_t)k * R->fz2; };
  std::vector<int> fu((size_t)R->fx3, 1), fv((size_t)R->fy3, 1), fw((size_t)R->fz3, 1);
  for (int k = 0; k < knb; k++)
    for (int j = 0; j < jnb; j++)
      for (int i = 1; i < inb; i++)
        if ((ph[ccb(i - 1, j, k)] < 0) != (ph[ccb(i, j, k)] < 0)) fu[fx(i, j, k)] = -1;
  for (int k = 0; k < knb; k++)
    for (int j = 1; j < jnb; j++)
      for (int i = 0; i < inb; i++)
        if ((ph[ccb(i, j - 1, k)] < 0) != (ph[ccb(i, j, k)] < 0)) fv[fy(i, j, k)] = -1;
  for (int k = 1; k < knb; k++)
    for (int j = 0; j < jnb; j++)
      for (int i = 0; i < inb; i++)
        if ((ph[ccb(i, j, k - 1)] < 0) != (ph[ccb(i, j, k)] < 0)) fw[fz(i, j, k)] = -1;
  // wall faces of a non-periodic direction: index 1 and n+1 of the face grid
  if (R->bc[0] != PERIODIC && R->bc[1] != PERIODIC)
    for (int k = 0; k < knb; k++)
      for (int j = 0; j < jnb; j++) {
        fu[fx(1, j, k)] = 0;
        fu[fx(nx + 1, j, k)] = 0;
      }
  if (R->bc[2] != PERIODIC && R->bc[3] != PERIODIC)
    for (int k = 0; k < knb; k++)
      for (int i = 0; i < inb; i++) {
        fv[fy(i, 1, k)] = 0;
        fv[fy(i, ny + 1, k)] = 0;
      }
  if (R->bc[4] != PERIODIC && R->bc[5] != PERIODIC)
    for (int j = 0; j < jnb; j++)
      for (int i = 0; i < inb; i++) {
        fw[fz(i, j, 1)] = 0;
        fw[fz(i, j, nz + 1)] = 0;
      }
  cudaMemcpy(R->phase, ph.data(), sizeof(int) * ph.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(R->flag_u, fu.data(), sizeof(int) * fu.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(R->flag_v, fv.data(), sizeof(int) * fv.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(R->flag_w, fw.data(), sizeof(int) * fw.size(), cudaMemcpyHostToDevice);
  // cuda_PP_init_jacobi_preconditioner
  void *args[] = {&R->flag_u, &R->flag_v, &R->flag_w, &R->invM};
  if (!launch(R, R->f_jacobi, R->kn, args)) return 9;
  if (cudaDeviceSynchronize() != cudaSuccess) {
    snprintf(R->err, sizeof(R->err), "setup: %s", cudaGetErrorString(cudaGetLastError()));
    return 10;
  }
  return 0;
}

// One reference solve of rhs (dense (nz,ny,nx), the -b the reference's PP_rhs
// would produce) to (r,z) <= residual^2 (b,b).  phi: dense solution out (may be
// NULL); niter, resid (sqrt((r,z)/(b,b)) at exit) and ms (CUDA events around
// the whole solve, from the rhs reset to the last check) out.  Returns 0, or
// 11 on a NaN residual, 12 when max_iter is exceeded (the reference exits).
// alpha_k and beta_k of the next solves, iterations 1 .. n (host arrays; NULL: none)
static double *g_trace_a = nullptr, *g_trace_b = nullptr;
static int g_trace_n = 0;
void refgpu_set_trace(double *alpha, double *beta, int n) {
  g_trace_a = alpha;
  g_trace_b = beta;
  g_trace_n = (alpha && beta && n > 0) ? n : 0;
}

int refgpu_solve(const double *rhs, double residual, int max_iter, double *phi, int *niter, double *resid,
                 double *ms) {
  Ref *R = g_ref;
  if (!R || !R->mod) return 1;
  const int nx = R->nx, ny = R->ny, nz = R->nz;
  cudaMemcpy(R->inj, rhs, sizeof(double) * (size_t)R->s3, cudaMemcpyHostToDevice);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaDeviceSynchronize();
  cudaEventRecord(e0, 0);
  int status = 0;
  // cudaMemset(_rhs_p, 0, s3b); PP_rhs -> injected
  cudaMemset(R->rhs, 0, sizeof(double) * (size_t)R->s3b);
  k_inject<<<1024, 256>>>(R->rhs, R->inj, nx, ny, nz, R->s1b, R->s2b);
  if (R->parts) {
    k_part_bc<<<1024, 256>>>(R->rhs, R->phase, R->s3b);
    exchange<double>(R, R->rhs);
    void *a_ref[] = {&R->rhs, &R->phase, &R->flag_u, &R->flag_v, &R->flag_w};
    launch(R, R->f_refine, R->kn, a_ref);
    void *a_z[] = {&R->rhs};
    launch(R, R->f_zero_i, R->inb, a_z);
    launch(R, R->f_zero_j, R->jnb, a_z);
    launch(R, R->f_zero_k, R->knb, a_z);
  }
  const double sp_rhs = dot(R->rhs, R->rhs, R->s3b);
  exchange<double>(R, R->rhs);
  {
    void *a[] = {&R->r, &R->p, &R->pb, &R->phi, &R->rhs, &R->z, &R->invM};
    launch(R, R->f_cg_init, R->kn, a);
  }
  exchange<double>(R, R->pb);
  double sp_rq = dot(R->r, R->z, R->s3);
  int q = 0;
  double sp_rq1 = 0.0;
  const double RHS_TOL = 1.e-8;
  CUfunction spmv = R->parts ? R->f_spmv : R->f_spmv_np;
  double rz_exit = 0.0;
  if (sp_rhs < RHS_TOL * RHS_TOL) {
    rz_exit = 0.0;
  } else {
    while (q <= max_iter) {
      ++q;
      {
        void *a[] = {&R->flag_u, &R->flag_v, &R->flag_w, &R->pb, &R->Ap, &R->phase};
        launch(R, spmv, R->kn_s, a);
      }
      const double DENOM = dot(R->p, R->Ap, R->s3);
      double alpha = sp_rq / DENOM;
      if (q - 1 < g_trace_n) g_trace_a[q - 1] = alpha;
      if (q % 50 == 0) {
        void *a1[] = {&R->phi, &R->p, &alpha};
        launch(R, R->f_solution, R->kn, a1);
        exchange<double>(R, R->phi);
        void *a2[] = {&R->flag_u, &R->flag_v, &R->flag_w, &R->phi, &R->Ap, &R->phase};
        launch(R, spmv, R->kn_s, a2);
        void *a3[] = {&R->r, &R->rhs, &R->Ap, &R->z, &R->invM};
        launch(R, R->f_residual, R->kn, a3);
      } else {
        void *a[] = {&R->phi, &R->p, &R->r, &R->Ap, &R->z, &alpha, &R->invM};
        launch(R, R->f_soln_resid, R->kn, a);
      }
      sp_rq1 = dot(R->r, R->z, R->s3);
      if (sp_rq1 <= residual * residual * sp_rhs) {
        rz_exit = std::sqrt(sp_rq1) / std::sqrt(sp_rhs);
        break;
      } else if (std::isnan(sp_rq1)) {
        status = 11;
        break;
      } else {
        double beta = sp_rq1 / sp_rq;
        if (q - 1 < g_trace_n) g_trace_b[q - 1] = beta;
        void *a[] = {&R->p, &R->pb, &R->z, &beta};
        launch(R, R->f_search, R->kn, a);
        exchange<double>(R, R->pb);
        sp_rq = sp_rq1;
      }
    }
    if (status == 0 && q > max_iter) status = 12;
  }
  cudaEventRecord(e1, 0);
  cudaEventSynchronize(e1);
  float t = 0.f;
  cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (cudaGetLastError() != cudaSuccess) {
    snprintf(R->err, sizeof(R->err), "solve: CUDA error");
    return 13;
  }
  if (phi) {
    k_extract<<<1024, 256>>>(R->inj, R->phi, nx, ny, nz, R->s1b, R->s2b);
    cudaMemcpy(phi, R->inj, sizeof(double) * (size_t)R->s3, cudaMemcpyDeviceToHost);
  }
  if (niter) *niter = q;
  if (resid) *resid = rz_exit;
  if (ms) *ms = t;
  return status;
}

}  // extern "C"
