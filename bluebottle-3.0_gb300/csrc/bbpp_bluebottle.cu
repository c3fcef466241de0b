// bbpp_bluebottle.cu -- the drop-in entry points of include/bbpp_bluebottle.h.
//
// The reference solve (src/cuda_solver.cu:38-300) does, per call: zero
// _rhs_p; PP_rhs; [particles] cuda_part_BC_p, exchange, coeffs_refine, zero
// ghosts; (rhs,rhs); PP_cg_init; the PCG loop; recorder_PP.  Here the rhs
// build and coeffs_refine are two kernels that read the reference's s3b face
// and cell arrays directly, the PCG runs in libbbpp on dense workspaces, and
// the solution is written back into _phi's interior.
#include <cuda_runtime.h>
#include <sys/time.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#define BBPP_BLUEBOTTLE_IMPL
#include "../../include/bbpp.h"
#include "../../include/bbpp_bluebottle.h"

extern "C" bb_bc_pressure bc;  // leading members of the host program's BC

namespace {

struct DropIn {
  bbpp_ctx *ctx = nullptr;
  int nx = 0, ny = 0, nz = 0;
  double dx = 0, dy = 0, dz = 0;
  int bcs[6] = {0, 0, 0, 0, 0, 0};
  uint8_t *mask = nullptr;  // dense, one byte per cell
  double *b = nullptr, *x = nullptr;
  bool mask_valid = false;
};
DropIn g;

void fail(const char *what, int rc) {
  fprintf(stderr, "N%d >> bbpp pressure solver: %s failed (%s): %s\n", rank, what, bbpp_status_str(rc),
          bbpp_last_error(g.ctx));
  exit(EXIT_FAILURE);
}

void ensure_ctx() {
  if (nprocs != 1) {
    fprintf(stderr, "N%d >> bbpp pressure solver: one rank per GPU only (nprocs = %d)\n", rank, nprocs);
    exit(EXIT_FAILURE);
  }
  const bb_dom_struct &d = dom[rank];
  const int b6[6] = {bc.pW, bc.pE, bc.pS, bc.pN, bc.pB, bc.pT};
  bool same = g.ctx && g.nx == d.Gcc.in && g.ny == d.Gcc.jn && g.nz == d.Gcc.kn && g.dx == d.dx && g.dy == d.dy &&
              g.dz == d.dz && memcmp(g.bcs, b6, sizeof(b6)) == 0;
  if (same) return;
  bbpp_bluebottle_release();
  bbpp_grid gr;
  gr.nx = d.Gcc.in;
  gr.ny = d.Gcc.jn;
  gr.nz = d.Gcc.kn;
  gr.dx = d.dx;
  gr.dy = d.dy;
  gr.dz = d.dz;
  memcpy(gr.bc, b6, sizeof(b6));
  int rc = bbpp_create(&gr, &g.ctx);
  if (rc) fail("bbpp_create", rc);
  g.nx = gr.nx;
  g.ny = gr.ny;
  g.nz = gr.nz;
  g.dx = gr.dx;
  g.dy = gr.dy;
  g.dz = gr.dz;
  memcpy(g.bcs, b6, sizeof(b6));
  const size_t n = (size_t)gr.nx * gr.ny * gr.nz;
  if (cudaMalloc(&g.mask, n) != cudaSuccess || cudaMalloc(&g.b, n * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&g.x, n * sizeof(double)) != cudaSuccess)
    fail("workspace allocation", BBPP_CUDA_ERROR);
  g.mask_valid = false;
}

// Reference s3b index of interior cell (i, j, k) (0-based), GCC_LOC
// (src/bluebottle.h:70) with DOM_BUF = 1.
__device__ __forceinline__ long long gcc_b(int i, int j, int k, int s1b, int s2b) {
  return (long long)(i + 1) + (long long)(j + 1) * s1b + (long long)(k + 1) * s2b;
}

struct Shape {
  int nx, ny, nz;
  int s1b, s2b;                  // Gcc s1b, s2b
  int fx_s1b, fx_s2b;            // Gfx: GFX_LOC = j + k s1b + i s2b
  int fy_s1b, fy_s2b;            // Gfy: GFY_LOC = k + i s1b + j s2b
  int fz_s1b, fz_s2b;            // Gfz: GFZ_LOC = i + j s1b + k s2b
  int px, py, pz;
  double idx, idy, idz, idx2, idy2, idz2;
};

// mask = (_phase > -1) on the interior
__global__ void k_mask_from_phase(Shape S, const int *__restrict__ phase, uint8_t *__restrict__ mask) {
  const long long n = (long long)S.nx * S.ny * S.nz;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(c % S.nx);
    const long long r = c / S.nx;
    const int j = (int)(r % S.ny), k = (int)(r / S.ny);
    mask[c] = phase[gcc_b(i, j, k, S.s1b, S.s2b)] > -1;
  }
}

// PP_rhs (src/solver_kernel.cu:152-173): rhs = -(rho/dt) div u* on the
// interior of _rhs_p (ghosts left zero, as after the reference's memset).
__global__ void k_rhs_div_b(Shape S, double rho_idt, const double *__restrict__ u, const double *__restrict__ v,
                            const double *__restrict__ w, double *__restrict__ rhs_b) {
  const long long n = (long long)S.nx * S.ny * S.nz;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(c % S.nx);
    const long long r = c / S.nx;
    const int j = (int)(r % S.ny), k = (int)(r / S.ny);
    const int TI = i + 1, TJ = j + 1, TK = k + 1;
    const double uw = u[TJ + (long long)TK * S.fx_s1b + (long long)TI * S.fx_s2b];
    const double ue = u[TJ + (long long)TK * S.fx_s1b + (long long)(TI + 1) * S.fx_s2b];
    const double vs = v[TK + (long long)TI * S.fy_s1b + (long long)TJ * S.fy_s2b];
    const double vn = v[TK + (long long)TI * S.fy_s1b + (long long)(TJ + 1) * S.fy_s2b];
    const double wb = w[TI + (long long)TJ * S.fz_s1b + (long long)TK * S.fz_s2b];
    const double wt = w[TI + (long long)TJ * S.fz_s1b + (long long)(TK + 1) * S.fz_s2b];
    double s = __dmul_rn(__dsub_rn(ue, uw), S.idx);
    s = __dadd_rn(s, __dmul_rn(__dsub_rn(vn, vs), S.idy));
    s = __dadd_rn(s, __dmul_rn(__dsub_rn(wt, wb), S.idz));
    s = __dmul_rn(s, rho_idt);
    rhs_b[gcc_b(i, j, k, S.s1b, S.s2b)] = -s;
  }
}

// coeffs_refine (src/solver_kernel.cu:212-256) on the s3b rhs, then the dense
// copy the solver works on.  Periodic neighbours wrap (the reference
// exchanges rhs first); a wall neighbour adds nothing (its phase ghost is -1).
__global__ void k_refine_pack(Shape S, const double *__restrict__ rhs_b, const uint8_t *__restrict__ mask,
                              double *__restrict__ b) {
  const long long n = (long long)S.nx * S.ny * S.nz;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(c % S.nx);
    const long long r = c / S.nx;
    const int j = (int)(r % S.ny), k = (int)(r / S.ny);
    double acc = rhs_b[gcc_b(i, j, k, S.s1b, S.s2b)];
    if (mask && !mask[c]) {
      const int ie = (i + 1 < S.nx) ? i + 1 : (S.px ? 0 : -1);
      const int iw = (i > 0) ? i - 1 : (S.px ? S.nx - 1 : -1);
      const int jn = (j + 1 < S.ny) ? j + 1 : (S.py ? 0 : -1);
      const int js = (j > 0) ? j - 1 : (S.py ? S.ny - 1 : -1);
      const int kt = (k + 1 < S.nz) ? k + 1 : (S.pz ? 0 : -1);
      const int kb = (k > 0) ? k - 1 : (S.pz ? S.nz - 1 : -1);
      const long long sy = S.nx, sz = (long long)S.nx * S.ny;
      if (ie >= 0 && mask[ie + j * sy + k * sz]) acc = __dadd_rn(acc, __dmul_rn(S.idx2, -rhs_b[gcc_b(ie, j, k, S.s1b, S.s2b)]));
      if (iw >= 0 && mask[iw + j * sy + k * sz]) acc = __dadd_rn(acc, __dmul_rn(S.idx2, -rhs_b[gcc_b(iw, j, k, S.s1b, S.s2b)]));
      if (jn >= 0 && mask[i + jn * sy + k * sz]) acc = __dadd_rn(acc, __dmul_rn(S.idy2, -rhs_b[gcc_b(i, jn, k, S.s1b, S.s2b)]));
      if (js >= 0 && mask[i + js * sy + k * sz]) acc = __dadd_rn(acc, __dmul_rn(S.idy2, -rhs_b[gcc_b(i, js, k, S.s1b, S.s2b)]));
      if (kt >= 0 && mask[i + j * sy + kt * sz]) acc = __dadd_rn(acc, __dmul_rn(S.idz2, -rhs_b[gcc_b(i, j, kt, S.s1b, S.s2b)]));
      if (kb >= 0 && mask[i + j * sy + kb * sz]) acc = __dadd_rn(acc, __dmul_rn(S.idz2, -rhs_b[gcc_b(i, j, kb, S.s1b, S.s2b)]));
    }
    b[c] = acc;
  }
}

// _phi interior = x (ghosts are the caller's, src/bluebottle.c:233-234)
__global__ void k_unpack_phi(Shape S, const double *__restrict__ x, double *__restrict__ phi_b) {
  const long long n = (long long)S.nx * S.ny * S.nz;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(c % S.nx);
    const long long r = c / S.nx;
    const int j = (int)(r % S.ny), k = (int)(r / S.ny);
    phi_b[gcc_b(i, j, k, S.s1b, S.s2b)] = x[c];
  }
}

Shape shape_of(const bb_dom_struct &d) {
  Shape S;
  S.nx = d.Gcc.in;
  S.ny = d.Gcc.jn;
  S.nz = d.Gcc.kn;
  S.s1b = d.Gcc.s1b;
  S.s2b = d.Gcc.s2b;
  S.fx_s1b = d.Gfx.s1b;
  S.fx_s2b = d.Gfx.s2b;
  S.fy_s1b = d.Gfy.s1b;
  S.fy_s2b = d.Gfy.s2b;
  S.fz_s1b = d.Gfz.s1b;
  S.fz_s2b = d.Gfz.s2b;
  S.px = bc.pW == BBPP_PERIODIC;
  S.py = bc.pS == BBPP_PERIODIC;
  S.pz = bc.pB == BBPP_PERIODIC;
  S.idx = 1. / d.dx;
  S.idy = 1. / d.dy;
  S.idz = 1. / d.dz;
  S.idx2 = 1. / (d.dx * d.dx);
  S.idy2 = 1. / (d.dy * d.dy);
  S.idz2 = 1. / (d.dz * d.dz);
  return S;
}

int grid_blocks(long long n) {
  long long b = (n + 255) / 256;
  return (int)(b < 4096 ? (b > 0 ? b : 1) : 4096);
}

void check(cudaError_t e, const char *what) {
  if (e != cudaSuccess) {
    fprintf(stderr, "N%d >> bbpp pressure solver: %s: %s\n", rank, what, cudaGetErrorString(e));
    exit(EXIT_FAILURE);
  }
}

void solve(bool particles, bool timed) {
  const char *recname = timed ? "solver_expd_timed.rec" : "solver_expd.rec";
  struct timeval ts, te;
  gettimeofday(&ts, 0);
  ensure_ctx();
  const bb_dom_struct &d = dom[rank];
  const Shape S = shape_of(d);
  const long long n = (long long)S.nx * S.ny * S.nz;
  const int nb = grid_blocks(n);
  // rhs into _rhs_p (reference layout), as PP_rhs
  check(cudaMemset(_rhs_p, 0, sizeof(double) * (size_t)d.Gcc.s3b), "memset rhs");
  k_rhs_div_b<<<nb, 256>>>(S, rho_f / dt, _u_star, _v_star, _w_star, _rhs_p);
  check(cudaGetLastError(), "rhs kernel");
  // the particle solve needs the phase field; without one it is the
  // particle-free operator
  particles = particles && NPARTS > 0 && _phase != nullptr;
  if (particles) {
    if (nparts > 0) cuda_part_BC_p();
    if (!g.mask_valid) {
      k_mask_from_phase<<<nb, 256>>>(S, _phase, g.mask);
      check(cudaGetLastError(), "mask kernel");
      g.mask_valid = true;
    }
  }
  k_refine_pack<<<nb, 256>>>(S, _rhs_p, (particles && nparts > 0) ? g.mask : nullptr, g.b);
  check(cudaGetLastError(), "refine kernel");
  check(cudaDeviceSynchronize(), "rhs build");

  bbpp_opts o;
  bbpp_default_opts(&o);
  o.precision = BBPP_FP64;
  o.guess = BBPP_GUESS_ZERO;
  o.stop = BBPP_STOP_REF_RZ;
  o.tol = pp_residual;
  o.max_iter = pp_max_iter;
  o.replace_every = 50;
  bbpp_report rep;
  char rname[256];
  snprintf(rname, sizeof(rname), "%s", recname);
  if (timed) {
    if (stepnum == 1) recorder_PP_init_timed(rname);
    bbpp_set_profiling(g.ctx, 1);
  }
  const int rc = bbpp_solve(g.ctx, particles ? g.mask : nullptr, g.b, g.x, &o, &rep);
  double t_spmv = 0, t_up = 0;
  if (timed) {
    bbpp_kstat ks[16];
    int nk = 0;
    bbpp_kernel_stats(g.ctx, ks, 16, &nk);
    for (int q = 0; q < nk && q < 16; q++) {
      if (strncmp(ks[q].name, "search_spmv", 11) == 0) t_spmv += ks[q].ms * 1e-3;
      else t_up += ks[q].ms * 1e-3;
    }
    bbpp_set_profiling(g.ctx, 0);
  }
  auto record = [&](int niter, double resid, double etime) {
    if (timed) recorder_PP_timed(rname, niter, resid, etime, t_spmv, 0., 0., t_up, 0., 0., 0., 0.);
    else recorder_PP(rname, niter, resid, etime);
  };
  if (rc == BBPP_TINY_RHS) {
    gettimeofday(&te, 0);
    double etime = (te.tv_sec - ts.tv_sec) + (te.tv_usec - ts.tv_usec) * 1.e-6;
    record(0, 0., etime);
    if (rank == 0) printf("N%d >> Norm of the rhs is less than %.1e, exiting solver\n", rank, 1.e-8);
    return;  // phi untouched, as the reference
  }
  if (rc == BBPP_NAN) {
    if (rank == 0) {
      printf("N%d >> The PP equation did not converge.\n", rank);
      printf("N%d >> The residual at iteration %d is nan (%lf).\n", rank, rep.iters, sqrt(rep.rz));
    }
    exit(EXIT_FAILURE);
  }
  if (rc == BBPP_MAX_ITER) {
    printf("N%d >> The pressure-Poisson equation did not converge.\n", rank);
    printf("N%d >> (rhs, rhs) is %e\n", rank, rep.bb);
    printf("N%d >> Residual at iteration %d is %lf\n", rank, rep.iters, sqrt(rep.rz) / sqrt(rep.bb));
    exit(EXIT_FAILURE);
  }
  if (rc != BBPP_CONVERGED) fail("bbpp_solve", rc);
  k_unpack_phi<<<nb, 256>>>(S, g.x, _phi);
  check(cudaGetLastError(), "unpack kernel");
  check(cudaDeviceSynchronize(), "unpack");
  gettimeofday(&te, 0);
  double etime = (te.tv_sec - ts.tv_sec) + (te.tv_usec - ts.tv_usec) * 1.e-6;
  record(rep.iters, sqrt(rep.rz) / sqrt(rep.bb), etime);
}

// ------------------------------------------------------------ epilogue --
// The time loop's steps after the solve (src/bluebottle.c:233-252): ghosts of
// phi, the projection of u*, and the pressure update.  The arithmetic is the
// reference kernels' (src/bluebottle_kernel.cu) in their evaluation order with
// no contraction, so u, v, w and the ghosts equal the reference's bit for bit;
// the pressure mean is a deterministic block-ordered sum.

// cuda_dom_BC_p: on a Neumann face the ghost is the adjacent interior cell
// (BC_p_W_N .. BC_p_T_N, src/bluebottle_kernel.cu:26-102).  blockIdx.y = face.
__global__ void k_dom_bc_p(Shape S, int faces, double *__restrict__ a) {
  const int f = blockIdx.y;
  if (!((faces >> f) & 1)) return;
  const int nx = S.nx, ny = S.ny, nz = S.nz;
  const long long n = f < 2 ? (long long)ny * nz : (f < 4 ? (long long)nx * nz : (long long)nx * ny);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    long long dst, src;
    if (f < 2) {  // W, E: (j, k)
      const int j = 1 + (int)(t % ny), k = 1 + (int)(t / ny);
      const long long row = (long long)j * S.s1b + (long long)k * S.s2b;
      dst = row + (f == 0 ? 0 : nx + 1);
      src = row + (f == 0 ? 1 : nx);
    } else if (f < 4) {  // S, N: (i, k)
      const int i = 1 + (int)(t % nx), k = 1 + (int)(t / nx);
      const long long col = i + (long long)k * S.s2b;
      dst = col + (long long)(f == 2 ? 0 : ny + 1) * S.s1b;
      src = col + (long long)(f == 2 ? 1 : ny) * S.s1b;
    } else {  // B, T: (i, j)
      const int i = 1 + (int)(t % nx), j = 1 + (int)(t / nx);
      const long long col = i + (long long)j * S.s1b;
      dst = col + (long long)(f == 4 ? 0 : nz + 1) * S.s2b;
      src = col + (long long)(f == 4 ? 1 : nz) * S.s2b;
    }
    a[dst] = a[src];
  }
}

// u = u* - (dt/rho) |flag| ddx (phi_c - phi_w) on every x face
// (project_u, src/bluebottle_kernel.cu:2303-2319); threads follow the face
// array's own order (GFX_LOC = j + k s1b + i s2b: j fastest).
__global__ void k_project_x(Shape S, double dtr, double dd, const double *__restrict__ us,
                            const double *__restrict__ phi, const int *__restrict__ flag, double *__restrict__ u) {
  const int nx = S.nx, ny = S.ny, nz = S.nz;
  const long long n = (long long)(nx + 1) * ny * nz;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int j = 1 + (int)(t % ny);
    const long long r = t / ny;
    const int k = 1 + (int)(r % nz), i = 1 + (int)(r / nz);
    const long long f = j + (long long)k * S.fx_s1b + (long long)i * S.fx_s2b;
    const long long cc = i + (long long)j * S.s1b + (long long)k * S.s2b;
    const double grad = __dmul_rn(__dmul_rn((double)abs(flag[f]), dd), __dsub_rn(phi[cc], phi[cc - 1]));
    u[f] = __dsub_rn(us[f], __dmul_rn(dtr, grad));
  }
}

// v faces (project_v): GFY_LOC = k + i s1b + j s2b, k fastest
__global__ void k_project_y(Shape S, double dtr, double dd, const double *__restrict__ vs,
                            const double *__restrict__ phi, const int *__restrict__ flag, double *__restrict__ v) {
  const int nx = S.nx, ny = S.ny, nz = S.nz;
  const long long n = (long long)nx * (ny + 1) * nz;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int k = 1 + (int)(t % nz);
    const long long r = t / nz;
    const int i = 1 + (int)(r % nx), j = 1 + (int)(r / nx);
    const long long f = k + (long long)i * S.fy_s1b + (long long)j * S.fy_s2b;
    const long long cc = i + (long long)j * S.s1b + (long long)k * S.s2b;
    const double grad = __dmul_rn(__dmul_rn((double)abs(flag[f]), dd), __dsub_rn(phi[cc], phi[cc - S.s1b]));
    v[f] = __dsub_rn(vs[f], __dmul_rn(dtr, grad));
  }
}

// w faces (project_w): GFZ_LOC = i + j s1b + k s2b, i fastest
__global__ void k_project_z(Shape S, double dtr, double dd, const double *__restrict__ ws,
                            const double *__restrict__ phi, const int *__restrict__ flag, double *__restrict__ w) {
  const int nx = S.nx, ny = S.ny, nz = S.nz;
  const long long n = (long long)nx * ny * (nz + 1);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(t % nx);
    const long long r = t / nx;
    const int j = 1 + (int)(r % ny), k = 1 + (int)(r / ny);
    const long long f = i + (long long)j * S.fz_s1b + (long long)k * S.fz_s2b;
    const long long cc = i + (long long)j * S.s1b + (long long)k * S.s2b;
    const double grad = __dmul_rn(__dmul_rn((double)abs(flag[f]), dd), __dsub_rn(phi[cc], phi[cc - S.s2b]));
    w[f] = __dsub_rn(ws[f], __dmul_rn(dtr, grad));
  }
}

// p = (fluid) (p0 + phi) on the interior (update_p, src/bluebottle_kernel.cu:
// 2385-2402) with the block partial sums of p; the last block to finish
// leaves -mean in *neg_mean.
__global__ void __launch_bounds__(256) k_update_p(Shape S, const double *__restrict__ p0,
                                                  const double *__restrict__ phi, const int *__restrict__ phase,
                                                  double *__restrict__ p, double *partials, unsigned int *ticket,
                                                  double *neg_mean) {
  __shared__ double s_sum[8];
  __shared__ int s_last;
  const long long n = (long long)S.nx * S.ny * S.nz;
  double acc = 0.0;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(c % S.nx);
    const long long r = c / S.nx;
    const int j = (int)(r % S.ny), k = (int)(r / S.ny);
    const long long C = gcc_b(i, j, k, S.s1b, S.s2b);
    const double v = __dmul_rn((double)(phase[C] < 0), __dadd_rn(p0[C], phi[C]));
    p[C] = v;
    acc += v;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) s_sum[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += s_sum[w];
    partials[blockIdx.x] = t;
    __threadfence();
    s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (s_last && threadIdx.x == 0) {
    __threadfence();
    double t = 0.0;
    for (unsigned int b = 0; b < gridDim.x; b++) t += __ldcg(&partials[b]);
    *neg_mean = -(t / (double)n);
    *ticket = 0;
  }
}

// p += -mean on the interior (forcing_add_c_const, src/bluebottle_kernel.cu:1507)
__global__ void k_add_const(Shape S, const double *__restrict__ neg_mean, double *__restrict__ p) {
  const long long n = (long long)S.nx * S.ny * S.nz;
  const double v = *neg_mean;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(c % S.nx);
    const long long r = c / S.nx;
    const int j = (int)(r % S.ny), k = (int)(r / S.ny);
    const long long C = gcc_b(i, j, k, S.s1b, S.s2b);
    p[C] = __dadd_rn(p[C], v);
  }
}

// -------------------------------------------------------------- cages --
// cuda_build_cages (src/cuda_particle.cu:1516-1646) in six launches instead of
// 2 x nparts serial launches with a host copy each: reset of phase and
// phase_shell; one block per particle marking the cells of its cage inside it;
// one block per particle clearing phase_shell on its boundary cells; one pass
// over each face array writing every flag.  The geometry is the
// reference kernels' (cage_setup, build_phase, build_phase_shell,
// src/particle_kernel.cu:134-426) in their evaluation order with no
// contraction, so the cells marked are the same.  build_phase runs the
// particles in index order and the last one to contain a cell keeps it, which
// is the largest index: atomicMax gives that without the order.

struct CageAxis {
  int s, e, reach;  // first and last cell of the cage (ghosted index), cells the reference's launch reaches
};

// cage_setup and the clamp of build_phase on one axis: cells [s, e] of a cage
// of 2 ceil(r/h) + 2 - (n % 2) cells centred on the particle's cell, clamped
// to the ghosted range [0, n + 1] ([1, n] on a wall), of which the
// reference's blocks of 8 threads reach ceil(cage / 8) * 8 from s.
__device__ CageAxis cage_axis(double c, double origin, double h, double rad, int n, bool lo_wall, bool hi_wall) {
  CageAxis a;
  const int dim = (int)(2. * ceil(__ddiv_rn(rad, h))) + 2 - n % 2;
  const double ih = __ddiv_rn(1., h);
  int s = (int)__dadd_rn(__dsub_rn(round(__dmul_rn(__dsub_rn(c, origin), ih)), 0.5 * dim), 1.0);
  int e = s + dim;
  const int lo = lo_wall ? 1 : 0, hi = hi_wall ? n : n + 1;
  s = s < lo ? lo : (s > hi ? hi : s);
  e = e < lo ? lo : (e > hi ? hi : e);
  a.s = s;
  a.e = e;
  a.reach = (int)ceil((double)dim * 0.125) * 8;
  return a;
}

// floor(|(x, y, z)| / r) < 1 as build_phase evaluates it
__device__ __forceinline__ bool in_sphere(double x, double y, double z, double irad) {
  const double d = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z)));
  return floor(__dmul_rn(d, irad)) < 1.0;
}

// (cell index - 0.5) h - offset: the cell centre relative to the particle
__device__ __forceinline__ double centre_rel(int i, double h, double off) {
  return __dsub_rn(__dmul_rn((double)i - 0.5, h), off);
}

struct CageGeom {
  int nx, ny, nz;          // interior cells
  int cx, cy, cz;          // ghosted extents (n + 2)
  double dx, dy, dz;
  double xs, ys, zs;       // domain origin
  int wall[6];             // W, E, S, N, B, T face of a non-periodic direction
};

// Particle n's centre and radius from the host program's part_struct array
// (stride BB_PART_STRUCT_BYTES; r, x, y, z at bytes 8, 16, 24, 32).
__device__ __forceinline__ void part_of(const unsigned char *parts, int n, double &x, double &y, double &z,
                                        double &r) {
  const bb_part_head *p = reinterpret_cast<const bb_part_head *>(parts + (size_t)n * BB_PART_STRUCT_BYTES);
  x = p->x;
  y = p->y;
  z = p->z;
  r = p->r;
}

__global__ void k_cage_reset(long long ncc, int *__restrict__ phase, int *__restrict__ shell) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncc; c += (long long)gridDim.x * blockDim.x) {
    phase[c] = -1;
    shell[c] = 1;
  }
}

// pass 0 (build_phase): cells of particle n's cage inside it take n (the largest
// such n wins); pass 1 (build_phase_shell): cells of n with a face neighbour
// whose centre lies outside n get phase_shell 0.  blockIdx.x = particle.
template <int PASS>
__global__ void __launch_bounds__(256) k_cage(CageGeom G, const unsigned char *__restrict__ parts,
                                              int *__restrict__ phase, int *__restrict__ shell) {
  const int n = blockIdx.x;
  double px, py, pz, pr;
  part_of(parts, n, px, py, pz, pr);
  const CageAxis ax = cage_axis(px, G.xs, G.dx, pr, G.nx, G.wall[0], G.wall[1]);
  const CageAxis ay = cage_axis(py, G.ys, G.dy, pr, G.ny, G.wall[2], G.wall[3]);
  const CageAxis az = cage_axis(pz, G.zs, G.dz, pr, G.nz, G.wall[4], G.wall[5]);
  if (ax.s == ax.e || ay.s == ay.e || az.s == az.e) return;
  const int lx = min(ax.e, ax.s + ax.reach - 1) - ax.s + 1;
  const int ly = min(ay.e, ay.s + ay.reach - 1) - ay.s + 1;
  const int lz = min(az.e, az.s + az.reach - 1) - az.s + 1;
  const double rx = __dsub_rn(px, G.xs), ry = __dsub_rn(py, G.ys), rz = __dsub_rn(pz, G.zs);
  const double irad = __ddiv_rn(1., pr);
  const int cells = lx * ly * lz;
  for (int t = threadIdx.x; t < cells; t += blockDim.x) {
    const int i = ax.s + t % lx, j = ay.s + (t / lx) % ly, k = az.s + t / (lx * ly);
    const long long C = i + (long long)G.cx * (j + (long long)G.cy * k);
    const double xx = centre_rel(i, G.dx, rx), yy = centre_rel(j, G.dy, ry), zz = centre_rel(k, G.dz, rz);
    if (PASS == 0) {
      if (in_sphere(xx, yy, zz, irad)) atomicMax(&phase[C], n);
    } else if (phase[C] == n) {
      const bool edge = !in_sphere(centre_rel(i - 1, G.dx, rx), yy, zz, irad) ||
                        !in_sphere(centre_rel(i + 1, G.dx, rx), yy, zz, irad) ||
                        !in_sphere(xx, centre_rel(j - 1, G.dy, ry), zz, irad) ||
                        !in_sphere(xx, centre_rel(j + 1, G.dy, ry), zz, irad) ||
                        !in_sphere(xx, yy, centre_rel(k - 1, G.dz, rz), irad) ||
                        !in_sphere(xx, yy, centre_rel(k + 1, G.dz, rz), irad);
      if (edge) shell[C] = 0;
    }
  }
}

// The face flags (cage_flag_*, flag_external_*, src/particle_kernel.cu:428-576):
// on the interior face planes -1 across a phase change or between two shell
// cells, else 1; the ghost face planes 1; both wall planes of a non-periodic
// direction 0.  The cell arrays run x fastest, flag_u [i][k][j] (y fastest)
// and flag_v [j][i][k] (z fastest): their kernels read cells along x and go
// through a 32 x 32 shared tile to write the flags along their own fastest
// axis, so both sides are coalesced; flag_w [k][j][i] runs like the cells.
__device__ __forceinline__ int face_flag(int parts, const int *__restrict__ phase, const int *__restrict__ shell,
                                         long long lo, long long hi) {
  if (!parts) return 1;
  const bool flip = ((phase[lo] < 0) != (phase[hi] < 0)) || (shell[hi] < 1 && shell[lo] < 1);
  return flip ? -1 : 1;
}

// flag_u: faces (i, j, k), i = 0 .. nx + 2; tile (i, j) of one k; block 32 x 8
__global__ void __launch_bounds__(256) k_cage_flag_x(CageGeom G, int parts, const int *__restrict__ phase,
                                                     const int *__restrict__ shell, int *__restrict__ fu) {
  __shared__ int tile[32][33];
  const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32, k = blockIdx.z;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const bool walls = G.wall[0] && G.wall[1];
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + tx, j = j0 + r;
    int f = 1;
    if (i <= G.nx + 2 && j < G.cy) {
      if (i >= 1 && i <= G.nx + 1) {
        const long long hi = i + (long long)G.cx * (j + (long long)G.cy * k);
        f = face_flag(parts, phase, shell, hi - 1, hi);
      }
      if (walls && (i == 1 || i == G.nx + 1)) f = 0;
    }
    tile[r][tx] = f;
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + r, j = j0 + tx;
    if (i <= G.nx + 2 && j < G.cy) fu[j + (long long)G.cy * (k + (long long)G.cz * i)] = tile[tx][r];
  }
}

// flag_v: faces (i, j, k), j = 0 .. ny + 2; tile (i, k) of one j
__global__ void __launch_bounds__(256) k_cage_flag_y(CageGeom G, int parts, const int *__restrict__ phase,
                                                     const int *__restrict__ shell, int *__restrict__ fv) {
  __shared__ int tile[32][33];
  const int i0 = blockIdx.x * 32, k0 = blockIdx.y * 32, j = blockIdx.z;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const bool walls = G.wall[2] && G.wall[3];
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + tx, k = k0 + r;
    int f = 1;
    if (i < G.cx && k < G.cz) {
      if (j >= 1 && j <= G.ny + 1) {
        const long long hi = i + (long long)G.cx * (j + (long long)G.cy * k);
        f = face_flag(parts, phase, shell, hi - G.cx, hi);
      }
      if (walls && (j == 1 || j == G.ny + 1)) f = 0;
    }
    tile[r][tx] = f;
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + r, k = k0 + tx;
    if (i < G.cx && k < G.cz) fv[k + (long long)G.cz * (i + (long long)G.cx * j)] = tile[tx][r];
  }
}

// flag_w: faces (i, j, k), k = 0 .. nz + 2 (blockIdx.y), in the cells' own order
__global__ void k_cage_flag_z(CageGeom G, int parts, const int *__restrict__ phase, const int *__restrict__ shell,
                              int *__restrict__ fw) {
  const int plane = G.cx * G.cy, k = blockIdx.y;
  const bool wall = G.wall[4] && G.wall[5] && (k == 1 || k == G.nz + 1);
  const bool inner = k >= 1 && k <= G.nz + 1;
  const long long base = (long long)plane * k;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < plane; c += gridDim.x * blockDim.x) {
    int f = 1;
    if (inner) f = face_flag(parts, phase, shell, base + c - plane, base + c);
    fw[base + c] = wall ? 0 : f;
  }
}

struct Epi {
  double *partials = nullptr;  // one per block of k_update_p, then -mean
  unsigned int *ticket = nullptr;
};
Epi e_ws;
constexpr int kEpiBlocks = 1024;

}  // namespace

extern "C" void cuda_dom_BC_p(bb_real *array) {
  if (nprocs != 1) {
    fprintf(stderr, "N%d >> bbpp: one rank per GPU only (nprocs = %d)\n", rank, nprocs);
    exit(EXIT_FAILURE);
  }
  const Shape S = shape_of(dom[rank]);
  // one rank: a face is a domain boundary exactly when its direction is not periodic
  const int faces = (bc.pW == BBPP_NEUMANN) | (bc.pE == BBPP_NEUMANN) << 1 | (bc.pS == BBPP_NEUMANN) << 2 |
                    (bc.pN == BBPP_NEUMANN) << 3 | (bc.pB == BBPP_NEUMANN) << 4 | (bc.pT == BBPP_NEUMANN) << 5;
  if (!faces) return;
  const long long mx = std::max<long long>(std::max<long long>((long long)S.ny * S.nz, (long long)S.nx * S.nz),
                                           (long long)S.nx * S.ny);
  k_dom_bc_p<<<dim3(grid_blocks(mx), 6), 256>>>(S, faces, array);
  check(cudaGetLastError(), "dom_BC_p kernel");
}

extern "C" void cuda_project(void) {
  const bb_dom_struct &d = dom[rank];
  const Shape S = shape_of(d);
  const double dtr = dt / rho_f;
  k_project_x<<<grid_blocks((long long)(S.nx + 1) * S.ny * S.nz), 256>>>(S, dtr, 1. / d.dx, _u_star, _phi, _flag_u,
                                                                           _u);
  k_project_y<<<grid_blocks((long long)S.nx * (S.ny + 1) * S.nz), 256>>>(S, dtr, 1. / d.dy, _v_star, _phi, _flag_v,
                                                                           _v);
  k_project_z<<<grid_blocks((long long)S.nx * S.ny * (S.nz + 1)), 256>>>(S, dtr, 1. / d.dz, _w_star, _phi, _flag_w,
                                                                           _w);
  check(cudaGetLastError(), "project kernels");
}

extern "C" void cuda_update_p(void) {
  const Shape S = shape_of(dom[rank]);
  if (!e_ws.partials) {
    check(cudaMalloc(&e_ws.partials, sizeof(double) * (kEpiBlocks + 1)), "epilogue workspace");
    check(cudaMalloc(&e_ws.ticket, sizeof(unsigned int)), "epilogue workspace");
    check(cudaMemset(e_ws.ticket, 0, sizeof(unsigned int)), "epilogue workspace");
  }
  const long long n = (long long)S.nx * S.ny * S.nz;
  const int nb = std::min(kEpiBlocks, grid_blocks(n));
  k_update_p<<<nb, 256>>>(S, _p0, _phi, _phase, _p, e_ws.partials, e_ws.ticket, e_ws.partials + kEpiBlocks);
  k_add_const<<<grid_blocks(n), 256>>>(S, e_ws.partials + kEpiBlocks, _p);
  check(cudaGetLastError(), "update_p kernels");
}

extern "C" void bbpp_bluebottle_release(void) {
  if (g.ctx) bbpp_destroy(g.ctx);
  if (g.mask) cudaFree(g.mask);
  if (g.b) cudaFree(g.b);
  if (g.x) cudaFree(g.x);
  g = DropIn();
  if (e_ws.partials) cudaFree(e_ws.partials);
  if (e_ws.ticket) cudaFree(e_ws.ticket);
  e_ws = Epi();
}

extern "C" void cuda_PP_init_jacobi_preconditioner(void) {
  ensure_ctx();
  const bb_dom_struct &d = dom[rank];
  const Shape S = shape_of(d);
  const long long n = (long long)S.nx * S.ny * S.nz;
  if (NPARTS > 0 && _phase) {
    k_mask_from_phase<<<grid_blocks(n), 256>>>(S, _phase, g.mask);
    check(cudaGetLastError(), "mask kernel");
    g.mask_valid = true;
  }
  if (_invM) {
    int rc = bbpp_invm(g.ctx, _invM);
    if (rc) fail("bbpp_invm", rc);
  }
  check(cudaDeviceSynchronize(), "preconditioner init");
}

extern "C" void cuda_build_cages(void) {
  if (nprocs != 1) {
    fprintf(stderr, "N%d >> bbpp: one rank per GPU only (nprocs = %d)\n", rank, nprocs);
    exit(EXIT_FAILURE);
  }
  const bb_dom_struct &d = dom[rank];
  CageGeom G;
  G.nx = d.Gcc.in;
  G.ny = d.Gcc.jn;
  G.nz = d.Gcc.kn;
  G.cx = G.nx + 2;
  G.cy = G.ny + 2;
  G.cz = G.nz + 2;
  G.dx = d.dx;
  G.dy = d.dy;
  G.dz = d.dz;
  G.xs = d.xs;
  G.ys = d.ys;
  G.zs = d.zs;
  const int b6[6] = {bc.pW, bc.pE, bc.pS, bc.pN, bc.pB, bc.pT};
  for (int f = 0; f < 6; f++) G.wall[f] = b6[f] != BBPP_PERIODIC;
  const bool parts = NPARTS > 0;
  if (parts) {
    const long long ncc = (long long)G.cx * G.cy * G.cz;
    k_cage_reset<<<grid_blocks(ncc), 256>>>(ncc, _phase, _phase_shell);
    if (nparts > 0) {
      k_cage<0><<<nparts, 256>>>(G, reinterpret_cast<const unsigned char *>(_parts), _phase, _phase_shell);
      k_cage<1><<<nparts, 256>>>(G, reinterpret_cast<const unsigned char *>(_parts), _phase, _phase_shell);
    }
  }
  const int pp = parts ? 1 : 0;
  k_cage_flag_x<<<dim3((G.nx + 3 + 31) / 32, (G.cy + 31) / 32, G.cz), dim3(32, 8)>>>(G, pp, _phase, _phase_shell,
                                                                                     _flag_u);
  k_cage_flag_y<<<dim3((G.cx + 31) / 32, (G.cz + 31) / 32, G.ny + 3), dim3(32, 8)>>>(G, pp, _phase, _phase_shell,
                                                                                     _flag_v);
  k_cage_flag_z<<<dim3(std::min((G.cx * G.cy + 255) / 256, 128), G.nz + 3), 256>>>(G, pp, _phase, _phase_shell,
                                                                                  _flag_w);
  check(cudaGetLastError(), "cage kernels");
}

extern "C" void cuda_PP_cg(void) { solve(true, false); }

extern "C" void cuda_PP_cg_noparts(void) { solve(false, false); }

// The reference's timed variant is the particle solve (src/cuda_solver.cu:302-571).
extern "C" void cuda_PP_cg_timed(void) { solve(true, true); }
