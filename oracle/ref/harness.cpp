// harness.cpp -- single-rank host harness around the reference's unmodified
// pressure solver (src/cuda_solver.cu, src/solver_kernel.cu), compiled for the
// CPU with emu_cuda.h.  Test infrastructure: it provides what the rest of
// Bluebottle normally provides to the solver -- the globals of
// src/bluebottle.c and src/cuda_bluebottle.cu, a one-rank periodic ghost
// exchange in place of mpi_cuda_exchange_Gcc (src/mpi_comm.c:257-315), the
// masking effect of part_BC_p (src/particle_kernel.cu:1753), a recorder that
// keeps the iteration count, and an injected right-hand side.
#include <cstdint>
#include <cstring>
#include <vector>

extern "C" {
#include "bluebottle.h"
#include "bluebottle.cuh"
#include "recorder.h"
}
#include "cuda_solver.h"
#include "cuda_bluebottle.h"

// ------------------------------------------------------------- globals ----
dom_struct DOM;
dom_struct *dom = nullptr;
dom_struct _dom;
bin_struct _bins;  // read by particle kernels of src/bluebottle_kernel.cu, never by the ones used here
cuda_blocks_struct blocks;
BC bc;
int rank = 0;
int nprocs = 1;
int NPARTS = 0;
int nparts = 0;
real rho_f = 1.0, dt = 1.0, dt0 = 1.0, mu = 1.0, nu = 1.0, ttime = 0.0;
int stepnum = 0;
real pp_residual = 1e-8;
int pp_max_iter = 20000;
real *_phi, *_rhs_p, *_r_q, *_z_q, *_p_q, *_pb_q, *_Apb_q, *_invM, *_u_star, *_v_star, *_w_star;
real *_u, *_v, *_w, *_p, *_p0;  // the post-solve epilogue's fields
int *_flag_u, *_flag_v, *_flag_w, *_phase, *_phase_shell;

static std::vector<double> g_inject;  // dense rhs to inject (nz, ny, nx)
static int g_niter = 0;
static double g_resid = 0;

static inline long long ccb(int i, int j, int k) {  // s3b index of interior (i,j,k), 0-based
  return (long long)(i + 1) + (long long)(j + 1) * dom[0].Gcc.s1b + (long long)(k + 1) * dom[0].Gcc.s2b;
}

// ------------------------------------------------------------ callbacks ---
extern "C" void recorder_PP(char *name, int niter, real resid, real etime) {
  (void)name;
  (void)etime;
  g_niter = niter;
  g_resid = resid;
}

extern "C" void recorder_PP_timed(char *name, int niter, real resid, real etime, real t0, real t1, real t2,
                                  real t3, real t4, real t5, real t6, real t7) {
  (void)name; (void)etime; (void)t0; (void)t1; (void)t2; (void)t3; (void)t4; (void)t5; (void)t6; (void)t7;
  g_niter = niter;
  g_resid = resid;
}

extern "C" void recorder_PP_init_timed(char *name) { (void)name; }

// One rank: a periodic direction's ghost plane is the opposite interior plane
// (the self-neighbour MPI_Put, src/domain.c:1151-1209); a Neumann ghost is
// never written (MPI_PROC_NULL).  Directions in x, y, z order over the full
// ghosted extent of the previous directions, so edges and corners fill too.
template <typename T>
static void exchange(T *a) {
  const grid_info &G = dom[0].Gcc;
  const int s1 = G.s1b, s2 = G.s2b;
  if (bc.pW == PERIODIC) {
    for (int k = 0; k < G.knb; k++)
      for (int j = 0; j < G.jnb; j++) {
        a[0 + j * s1 + k * s2] = a[G._ie + j * s1 + k * s2];
        a[G._ieb + j * s1 + k * s2] = a[G._is + j * s1 + k * s2];
      }
  }
  if (bc.pS == PERIODIC) {
    for (int k = 0; k < G.knb; k++)
      for (int i = 0; i < G.inb; i++) {
        a[i + 0 * s1 + k * s2] = a[i + G._je * s1 + k * s2];
        a[i + G._jeb * s1 + k * s2] = a[i + G._js * s1 + k * s2];
      }
  }
  if (bc.pB == PERIODIC) {
    for (int j = 0; j < G.jnb; j++)
      for (int i = 0; i < G.inb; i++) {
        a[i + j * s1 + 0 * s2] = a[i + j * s1 + G._ke * s2];
        a[i + j * s1 + G._keb * s2] = a[i + j * s1 + G._ks * s2];
      }
  }
}

extern "C" void mpi_cuda_exchange_Gcc(real *array) { exchange<real>(array); }

// part_BC_p's effect on the solve: rhs of solid cells is zero
extern "C" void cuda_part_BC_p(void) {
  const grid_info &G = dom[0].Gcc;
  for (long long c = 0; c < G.s3b; c++)
    if (_phase[c] > -1) _rhs_p[c] = 0.;
}

// injected right-hand side: the solver is compiled with PP_rhs renamed to this
__global__ void PP_rhs_inject(real rho_f_, real *u, real *v, real *w, real *rhs, real dt_) {
  if (g_inject.empty()) {  // no injected rhs: run the reference's PP_rhs
    PP_rhs(rho_f_, u, v, w, rhs, dt_);
    return;
  }
  if (threadIdx.x || threadIdx.y || blockIdx.x || blockIdx.y) return;
  const grid_info &G = dom[0].Gcc;
  for (int k = 0; k < G.kn; k++)
    for (int j = 0; j < G.jn; j++)
      for (int i = 0; i < G.in; i++) rhs[ccb(i, j, k)] = g_inject[(size_t)i + (size_t)G.in * (j + (size_t)G.jn * k)];
}

// ---------------------------------------------------------------- setup ---
static void fill_grid(grid_info &g, int in, int jn, int kn) {
  memset(&g, 0, sizeof(g));
  g.is = g._is = DOM_BUF; g.isb = g._isb = 0; g.in = in; g.inb = in + 2; g.ie = g._ie = in; g.ieb = g._ieb = in + 1;
  g.js = g._js = DOM_BUF; g.jsb = g._jsb = 0; g.jn = jn; g.jnb = jn + 2; g.je = g._je = jn; g.jeb = g._jeb = jn + 1;
  g.ks = g._ks = DOM_BUF; g.ksb = g._ksb = 0; g.kn = kn; g.knb = kn + 2; g.ke = g._ke = kn; g.keb = g._keb = kn + 1;
}

static void strides_xfast(grid_info &g) {
  g.s1 = g.in; g.s2 = g.s1 * g.jn; g.s3 = g.s2 * g.kn;
  g.s1b = g.inb; g.s2b = g.s1b * g.jnb; g.s3b = g.s2b * g.knb;
}

static int threads_of(int n) { return n < MAX_THREADS_DIM ? n : MAX_THREADS_DIM; }
static int cdiv(int a, int b) { return (a + b - 1) / b; }

static void release() {
  for (void *p : {(void *)_phi, (void *)_rhs_p, (void *)_r_q, (void *)_z_q, (void *)_p_q, (void *)_pb_q,
                  (void *)_Apb_q, (void *)_invM, (void *)_u_star, (void *)_v_star, (void *)_w_star,
                  (void *)_flag_u, (void *)_flag_v, (void *)_flag_w, (void *)_phase, (void *)_phase_shell,
                  (void *)_u, (void *)_v, (void *)_w, (void *)_p, (void *)_p0})
    free(p);
  _phi = _rhs_p = _r_q = _z_q = _p_q = _pb_q = _Apb_q = _invM = _u_star = _v_star = _w_star = nullptr;
  _u = _v = _w = _p = _p0 = nullptr;
  _flag_u = _flag_v = _flag_w = _phase = _phase_shell = nullptr;
  delete[] dom;
  dom = nullptr;
}

extern "C" void ref_free(void) { release(); }

// Set up a single-rank domain [0, nx dx] x ... with pressure BCs bcs[6]
// (W,E,S,N,B,T) and an optional solid mask (dense (nz,ny,nx), 1 = solid).
extern "C" int ref_setup(int nx, int ny, int nz, double dx, double dy, double dz, const int *bcs,
                         const uint8_t *mask) {
  release();
  dom = new dom_struct[1];
  dom_struct &d = dom[0];
  memset(&d, 0, sizeof(d));
  d.xs = 0; d.xn = nx; d.dx = dx; d.xe = nx * dx; d.xl = d.xe;
  d.ys = 0; d.yn = ny; d.dy = dy; d.ye = ny * dy; d.yl = d.ye;
  d.zs = 0; d.zn = nz; d.dz = dz; d.ze = nz * dz; d.zl = d.ze;
  d.In = d.Jn = d.Kn = 1; d.S1 = d.S2 = d.S3 = 1;
  fill_grid(d.Gcc, nx, ny, nz);
  strides_xfast(d.Gcc);
  fill_grid(d.Gfx, nx + 1, ny, nz);   // Gfx: GFX_LOC = j + k s1b + i s2b
  d.Gfx.s1 = d.Gfx.jn; d.Gfx.s2 = d.Gfx.s1 * d.Gfx.kn; d.Gfx.s3 = d.Gfx.s2 * d.Gfx.in;
  d.Gfx.s1b = d.Gfx.jnb; d.Gfx.s2b = d.Gfx.s1b * d.Gfx.knb; d.Gfx.s3b = d.Gfx.s2b * d.Gfx.inb;
  fill_grid(d.Gfy, nx, ny + 1, nz);   // Gfy: GFY_LOC = k + i s1b + j s2b
  d.Gfy.s1 = d.Gfy.kn; d.Gfy.s2 = d.Gfy.s1 * d.Gfy.in; d.Gfy.s3 = d.Gfy.s2 * d.Gfy.jn;
  d.Gfy.s1b = d.Gfy.knb; d.Gfy.s2b = d.Gfy.s1b * d.Gfy.inb; d.Gfy.s3b = d.Gfy.s2b * d.Gfy.jnb;
  fill_grid(d.Gfz, nx, ny, nz + 1);   // Gfz: GFZ_LOC = i + j s1b + k s2b
  strides_xfast(d.Gfz);
  DOM = d;
  _dom = d;
  memset(&bc, 0, sizeof(bc));
  bc.pW = bcs[0]; bc.pE = bcs[1]; bc.pS = bcs[2]; bc.pN = bcs[3]; bc.pB = bcs[4]; bc.pT = bcs[5];
  NPARTS = nparts = mask ? 1 : 0;

  // launch shapes as cuda_blocks_init (src/cuda_bluebottle.cu:511-581,763-790)
  const grid_info &G = d.Gcc;
  int tx = threads_of(G.in), ty = threads_of(G.jn), tz = threads_of(G.kn);
  blocks.Gcc.dim_kn = dim3(tx, ty);
  blocks.Gcc.num_kn = dim3(cdiv(G.in, tx), cdiv(G.jn, ty));
  tx = threads_of(G.in + 2); ty = threads_of(G.jn + 2); tz = threads_of(G.kn + 2);
  blocks.Gcc.dim_kn_s = dim3(tx, ty);
  blocks.Gcc.num_kn_s = dim3(cdiv(G.in, tx - 2), cdiv(G.jn, ty - 2));
  tx = threads_of(G.inb); ty = threads_of(G.jnb); tz = threads_of(G.knb);
  blocks.Gcc.dim_inb = dim3(ty, tz); blocks.Gcc.num_inb = dim3(cdiv(G.jnb, ty), cdiv(G.knb, tz));
  blocks.Gcc.dim_jnb = dim3(tz, tx); blocks.Gcc.num_jnb = dim3(cdiv(G.knb, tz), cdiv(G.inb, tx));
  blocks.Gcc.dim_knb = dim3(tx, ty); blocks.Gcc.num_knb = dim3(cdiv(G.inb, tx), cdiv(G.jnb, ty));
  // in / jn / kn shapes of every grid (cuda_blocks_init, src/cuda_bluebottle.cu:511-790)
  auto faces = [](const grid_info &F, cuda_blocks_info &B) {
    const int fx = threads_of(F.in), fy = threads_of(F.jn), fz = threads_of(F.kn);
    const int bx = cdiv(F.in, fx), by = cdiv(F.jn, fy), bz = cdiv(F.kn, fz);
    B.dim_in = dim3(fy, fz); B.num_in = dim3(by, bz);
    B.dim_jn = dim3(fz, fx); B.num_jn = dim3(bz, bx);
    B.dim_kn = dim3(fx, fy); B.num_kn = dim3(bx, by);
  };
  faces(d.Gcc, blocks.Gcc);
  faces(d.Gfx, blocks.Gfx);
  faces(d.Gfy, blocks.Gfy);
  faces(d.Gfz, blocks.Gfz);

  _phi = (real *)calloc(G.s3b, sizeof(real));
  _rhs_p = (real *)calloc(G.s3b, sizeof(real));
  _pb_q = (real *)calloc(G.s3b, sizeof(real));
  _r_q = (real *)calloc(G.s3, sizeof(real));
  _z_q = (real *)calloc(G.s3, sizeof(real));
  _p_q = (real *)calloc(G.s3, sizeof(real));
  _Apb_q = (real *)calloc(G.s3, sizeof(real));
  _invM = (real *)calloc(G.s3, sizeof(real));
  _u_star = (real *)calloc(d.Gfx.s3b, sizeof(real));
  _v_star = (real *)calloc(d.Gfy.s3b, sizeof(real));
  _w_star = (real *)calloc(d.Gfz.s3b, sizeof(real));
  _u = (real *)calloc(d.Gfx.s3b, sizeof(real));
  _v = (real *)calloc(d.Gfy.s3b, sizeof(real));
  _w = (real *)calloc(d.Gfz.s3b, sizeof(real));
  _p = (real *)calloc(G.s3b, sizeof(real));
  _p0 = (real *)calloc(G.s3b, sizeof(real));
  _phase = (int *)malloc(sizeof(int) * G.s3b);
  _phase_shell = (int *)malloc(sizeof(int) * G.s3b);
  _flag_u = (int *)malloc(sizeof(int) * d.Gfx.s3b);
  _flag_v = (int *)malloc(sizeof(int) * d.Gfy.s3b);
  _flag_w = (int *)malloc(sizeof(int) * d.Gfz.s3b);

  // phase: -1 fluid, particle index (0) solid; ghosts by the periodic rule
  for (long long c = 0; c < G.s3b; c++) { _phase[c] = -1; _phase_shell[c] = 1; }
  if (mask)
    for (int k = 0; k < nz; k++)
      for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++)
          if (mask[(size_t)i + (size_t)nx * (j + (size_t)ny * k)]) _phase[ccb(i, j, k)] = 0;
  exchange<int>(_phase);
  // face flags: 1, -1 across a fluid/solid face (cage_flag_*), 0 on the walls
  // of a non-periodic direction (flag_external_*)
  for (long long c = 0; c < d.Gfx.s3b; c++) _flag_u[c] = 1;
  for (long long c = 0; c < d.Gfy.s3b; c++) _flag_v[c] = 1;
  for (long long c = 0; c < d.Gfz.s3b; c++) _flag_w[c] = 1;
  for (int k = 0; k < G.knb; k++)
    for (int j = 0; j < G.jnb; j++)
      for (int i = 1; i < G.inb; i++) {
        const int pw = _phase[(i - 1) + j * G.s1b + k * G.s2b], pe = _phase[i + j * G.s1b + k * G.s2b];
        if ((pw < 0) != (pe < 0)) _flag_u[GFX_LOC(i, j, k, d.Gfx.s1b, d.Gfx.s2b)] = -1;
      }
  for (int k = 0; k < G.knb; k++)
    for (int j = 1; j < G.jnb; j++)
      for (int i = 0; i < G.inb; i++) {
        const int ps = _phase[i + (j - 1) * G.s1b + k * G.s2b], pn = _phase[i + j * G.s1b + k * G.s2b];
        if ((ps < 0) != (pn < 0)) _flag_v[GFY_LOC(i, j, k, d.Gfy.s1b, d.Gfy.s2b)] = -1;
      }
  for (int k = 1; k < G.knb; k++)
    for (int j = 0; j < G.jnb; j++)
      for (int i = 0; i < G.inb; i++) {
        const int pb = _phase[i + j * G.s1b + (k - 1) * G.s2b], pt = _phase[i + j * G.s1b + k * G.s2b];
        if ((pb < 0) != (pt < 0)) _flag_w[GFZ_LOC(i, j, k, d.Gfz.s1b, d.Gfz.s2b)] = -1;
      }
  if (bc.pW != PERIODIC && bc.pE != PERIODIC)
    for (int k = 0; k < d.Gfx.knb; k++)
      for (int j = 0; j < d.Gfx.jnb; j++) {
        _flag_u[GFX_LOC(d.Gfx._is, j, k, d.Gfx.s1b, d.Gfx.s2b)] = 0;
        _flag_u[GFX_LOC(d.Gfx._ie, j, k, d.Gfx.s1b, d.Gfx.s2b)] = 0;
      }
  if (bc.pS != PERIODIC && bc.pN != PERIODIC)
    for (int k = 0; k < d.Gfy.knb; k++)
      for (int i = 0; i < d.Gfy.inb; i++) {
        _flag_v[GFY_LOC(i, d.Gfy._js, k, d.Gfy.s1b, d.Gfy.s2b)] = 0;
        _flag_v[GFY_LOC(i, d.Gfy._je, k, d.Gfy.s1b, d.Gfy.s2b)] = 0;
      }
  if (bc.pB != PERIODIC && bc.pT != PERIODIC)
    for (int j = 0; j < d.Gfz.jnb; j++)
      for (int i = 0; i < d.Gfz.inb; i++) {
        _flag_w[GFZ_LOC(i, j, d.Gfz._ks, d.Gfz.s1b, d.Gfz.s2b)] = 0;
        _flag_w[GFZ_LOC(i, j, d.Gfz._ke, d.Gfz.s1b, d.Gfz.s2b)] = 0;
      }
  cuda_PP_init_jacobi_preconditioner();
  return 0;
}

// Run the reference solve on rhs (dense, = the interior of _rhs_p).
extern "C" int ref_solve(const double *rhs, double residual, int max_iter, double *phi, int *niter, double *resid) {
  const grid_info &G = dom[0].Gcc;
  g_inject.assign(rhs, rhs + (size_t)G.s3);
  pp_residual = residual;
  pp_max_iter = max_iter;
  g_niter = -1;
  if (NPARTS > 0) cuda_PP_cg();
  else cuda_PP_cg_noparts();
  for (int k = 0; k < G.kn; k++)
    for (int j = 0; j < G.jn; j++)
      for (int i = 0; i < G.in; i++) phi[(size_t)i + (size_t)G.in * (j + (size_t)G.jn * k)] = _phi[ccb(i, j, k)];
  *niter = g_niter;
  *resid = g_resid;
  return 0;
}

static void load_faces(const double *u, const double *v, const double *w) {
  const dom_struct &d = dom[0];
  const int nx = d.Gcc.in, ny = d.Gcc.jn, nz = d.Gcc.kn;
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i <= nx; i++)
        _u_star[GFX_LOC(i + 1, j + 1, k + 1, d.Gfx.s1b, d.Gfx.s2b)] = u[i + (size_t)(nx + 1) * (j + (size_t)ny * k)];
  for (int k = 0; k < nz; k++)
    for (int j = 0; j <= ny; j++)
      for (int i = 0; i < nx; i++)
        _v_star[GFY_LOC(i + 1, j + 1, k + 1, d.Gfy.s1b, d.Gfy.s2b)] = v[i + (size_t)nx * (j + (size_t)(ny + 1) * k)];
  for (int k = 0; k <= nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++)
        _w_star[GFZ_LOC(i + 1, j + 1, k + 1, d.Gfz.s1b, d.Gfz.s2b)] = w[i + (size_t)nx * (j + (size_t)ny * k)];
}

// The whole reference solve including its rhs build from u*, v*, w*
// (dense face arrays as ref_rhs), as the time loop calls it.
extern "C" int ref_solve_u(double rho, double dtt, const double *u, const double *v, const double *w,
                           double residual, int max_iter, double *phi, int *niter, double *resid) {
  const grid_info &G = dom[0].Gcc;
  load_faces(u, v, w);
  g_inject.clear();
  rho_f = rho;
  dt = dtt;
  pp_residual = residual;
  pp_max_iter = max_iter;
  g_niter = -1;
  if (NPARTS > 0) cuda_PP_cg();
  else cuda_PP_cg_noparts();
  for (int k = 0; k < G.kn; k++)
    for (int j = 0; j < G.jn; j++)
      for (int i = 0; i < G.in; i++) phi[(size_t)i + (size_t)G.in * (j + (size_t)G.jn * k)] = _phi[ccb(i, j, k)];
  *niter = g_niter;
  *resid = g_resid;
  return 0;
}

// (-A)p with the reference SpMV kernels (src/solver_kernel.cu:528-836).
extern "C" int ref_spmv(const double *p, double *Ap) {
  const grid_info &G = dom[0].Gcc;
  memset(_pb_q, 0, sizeof(real) * G.s3b);
  for (int k = 0; k < G.kn; k++)
    for (int j = 0; j < G.jn; j++)
      for (int i = 0; i < G.in; i++) _pb_q[ccb(i, j, k)] = p[(size_t)i + (size_t)G.in * (j + (size_t)G.jn * k)];
  mpi_cuda_exchange_Gcc(_pb_q);
  if (NPARTS > 0)
    emu::launch(blocks.Gcc.num_kn_s, blocks.Gcc.dim_kn_s,
                [&] { PP_spmv_shared_load(_flag_u, _flag_v, _flag_w, _pb_q, _Apb_q, _phase); });
  else
    emu::launch(blocks.Gcc.num_kn_s, blocks.Gcc.dim_kn_s,
                [&] { PP_spmv_shared_load_noparts(_flag_u, _flag_v, _flag_w, _pb_q, _Apb_q); });
  memcpy(Ap, _Apb_q, sizeof(real) * G.s3);
  return 0;
}

extern "C" int ref_invm(double *invM) {
  memcpy(invM, _invM, sizeof(real) * dom[0].Gcc.s3);
  return 0;
}

// rhs = PP_rhs(u*, v*, w*) (src/solver_kernel.cu:89-176).  Dense face arrays:
// u[(i + (nx+1)(j + ny k))], v[i + nx(j + (ny+1) k)], w[i + nx(j + ny k)], k <= nz.
extern "C" int ref_rhs(double rho, double dtt, const double *u, const double *v, const double *w, double *rhs) {
  const dom_struct &d = dom[0];
  const int nx = d.Gcc.in, ny = d.Gcc.jn, nz = d.Gcc.kn;
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i <= nx; i++)
        _u_star[GFX_LOC(i + 1, j + 1, k + 1, d.Gfx.s1b, d.Gfx.s2b)] = u[i + (size_t)(nx + 1) * (j + (size_t)ny * k)];
  for (int k = 0; k < nz; k++)
    for (int j = 0; j <= ny; j++)
      for (int i = 0; i < nx; i++)
        _v_star[GFY_LOC(i + 1, j + 1, k + 1, d.Gfy.s1b, d.Gfy.s2b)] = v[i + (size_t)nx * (j + (size_t)(ny + 1) * k)];
  for (int k = 0; k <= nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++)
        _w_star[GFZ_LOC(i + 1, j + 1, k + 1, d.Gfz.s1b, d.Gfz.s2b)] = w[i + (size_t)nx * (j + (size_t)ny * k)];
  memset(_rhs_p, 0, sizeof(real) * d.Gcc.s3b);
  emu::launch(blocks.Gcc.num_kn_s, blocks.Gcc.dim_kn_s, [&] { PP_rhs(rho, _u_star, _v_star, _w_star, _rhs_p, dtt); });
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) rhs[(size_t)i + (size_t)nx * (j + (size_t)ny * k)] = _rhs_p[ccb(i, j, k)];
  return 0;
}

// ------------------------------------------------------------- epilogue --
// The time loop's steps after the solve (src/bluebottle.c:233-252, one rank):
// mpi_cuda_exchange_Gcc(_phi); cuda_dom_BC_p(_phi); cuda_project(); and
// cuda_update_p() (src/cuda_bluebottle.cu:2495-2589), with the reference's
// kernels BC_p_*_N, project_u/v/w, update_p_laplacian, update_p,
// copy_p_p_noghost and forcing_add_c_const (src/bluebottle_kernel.cu).
// The host sequencing of those three functions is restated here; thrust's
// reduce of the pressure mean is a plain sum.  Inputs: phi (dense interior),
// u*, v*, w* and p0 as ghosted s3b arrays of their grids; outputs: the
// ghost-filled phi (s3b), u, v, w (face s3b) and p (s3b).
extern "C" int ref_epilogue(double rho, double dtt, double nu_, const double *phi, const double *us,
                            const double *vs, const double *ws, const double *p0, double *phi_b, double *u, double *v,
                            double *w, double *p) {
  const dom_struct &d = dom[0];
  const grid_info &G = d.Gcc;
  rho_f = rho;
  dt = dtt;
  nu = nu_;
  memset(_phi, 0, sizeof(real) * G.s3b);
  for (int k = 0; k < G.kn; k++)
    for (int j = 0; j < G.jn; j++)
      for (int i = 0; i < G.in; i++) _phi[ccb(i, j, k)] = phi[(size_t)i + (size_t)G.in * (j + (size_t)G.jn * k)];
  memcpy(_u_star, us, sizeof(real) * d.Gfx.s3b);
  memcpy(_v_star, vs, sizeof(real) * d.Gfy.s3b);
  memcpy(_w_star, ws, sizeof(real) * d.Gfz.s3b);
  memcpy(_p0, p0, sizeof(real) * G.s3b);
  memset(_u, 0, sizeof(real) * d.Gfx.s3b);
  memset(_v, 0, sizeof(real) * d.Gfy.s3b);
  memset(_w, 0, sizeof(real) * d.Gfz.s3b);
  memset(_p, 0, sizeof(real) * G.s3b);
  // mpi_cuda_exchange_Gcc(_phi); cuda_dom_BC_p(_phi): Neumann faces of one rank
  mpi_cuda_exchange_Gcc(_phi);
  if (bc.pW == NEUMANN) emu::launch(blocks.Gcc.num_in, blocks.Gcc.dim_in, [&] { BC_p_W_N(_phi); });
  if (bc.pE == NEUMANN) emu::launch(blocks.Gcc.num_in, blocks.Gcc.dim_in, [&] { BC_p_E_N(_phi); });
  if (bc.pS == NEUMANN) emu::launch(blocks.Gcc.num_jn, blocks.Gcc.dim_jn, [&] { BC_p_S_N(_phi); });
  if (bc.pN == NEUMANN) emu::launch(blocks.Gcc.num_jn, blocks.Gcc.dim_jn, [&] { BC_p_N_N(_phi); });
  if (bc.pB == NEUMANN) emu::launch(blocks.Gcc.num_kn, blocks.Gcc.dim_kn, [&] { BC_p_B_N(_phi); });
  if (bc.pT == NEUMANN) emu::launch(blocks.Gcc.num_kn, blocks.Gcc.dim_kn, [&] { BC_p_T_N(_phi); });
  // cuda_project
  emu::launch(blocks.Gfx.num_in, blocks.Gfx.dim_in,
              [&] { project_u(_u_star, _phi, rho_f, dt, _u, 1. / d.dx, _flag_u); });
  emu::launch(blocks.Gfy.num_jn, blocks.Gfy.dim_jn,
              [&] { project_v(_v_star, _phi, rho_f, dt, _v, 1. / d.dy, _flag_v); });
  emu::launch(blocks.Gfz.num_kn, blocks.Gfz.dim_kn,
              [&] { project_w(_w_star, _phi, rho_f, dt, _w, 1. / d.dz, _flag_w); });
  // cuda_update_p
  std::vector<real> Lp((size_t)G.s3b, 0.), pm((size_t)G.s3, 0.);
  emu::launch(blocks.Gcc.num_kn, blocks.Gcc.dim_kn, [&] { update_p_laplacian(Lp.data(), _phi); });
  emu::launch(blocks.Gcc.num_kn, blocks.Gcc.dim_kn, [&] { update_p(Lp.data(), _p0, _p, _phi, nu, dt, _phase); });
  emu::launch(blocks.Gcc.num_kn, blocks.Gcc.dim_kn, [&] { copy_p_p_noghost(pm.data(), _p); });
  real pmean = 0.;
  for (long long c = 0; c < G.s3; c++) pmean += pm[c];
  pmean /= (real)G.s3;
  emu::launch(blocks.Gcc.num_kn, blocks.Gcc.dim_kn, [&] { forcing_add_c_const(-pmean, _p); });
  memcpy(phi_b, _phi, sizeof(real) * G.s3b);
  memcpy(u, _u, sizeof(real) * d.Gfx.s3b);
  memcpy(v, _v, sizeof(real) * d.Gfy.s3b);
  memcpy(w, _w, sizeof(real) * d.Gfz.s3b);
  memcpy(p, _p, sizeof(real) * G.s3b);
  return 0;
}

// sizes of the ghosted arrays: Gcc, Gfx, Gfy, Gfz s3b
extern "C" void ref_sizes(long long *out) {
  out[0] = dom[0].Gcc.s3b;
  out[1] = dom[0].Gfx.s3b;
  out[2] = dom[0].Gfy.s3b;
  out[3] = dom[0].Gfz.s3b;
}

// the face flags and phase the harness built (for the other implementations)
extern "C" void ref_flags(int *fu, int *fv, int *fw, int *phase) {
  memcpy(fu, _flag_u, sizeof(int) * dom[0].Gfx.s3b);
  memcpy(fv, _flag_v, sizeof(int) * dom[0].Gfy.s3b);
  memcpy(fw, _flag_w, sizeof(int) * dom[0].Gfz.s3b);
  memcpy(phase, _phase, sizeof(int) * dom[0].Gcc.s3b);
}
