/*
 * bbpp_oracle.h -- CPU oracle for the Bluebottle pressure-Poisson solve.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C FP64 restatement of the
 * reference algorithm.  It is used to check the CUDA path and to time the
 * CPU baseline.  The product library never links, loads or calls it.
 *
 * Parity of this restatement is pinned against the reference's own solver
 * sources (src/cuda_solver.cu, src/solver_kernel.cu), which are compiled
 * unmodified for the host by oracle/ref/build_ref.py and run on the same
 * inputs (tests/test_oracle_vs_ref.py, tests/golden/).
 *
 * Layout: dense cell-centred arrays, no ghost layer, index
 *   c = i + nx*(j + ny*k)   (x fastest; the reference GCC_LOC order,
 *   src/bluebottle.h:70, with the ghost layer stripped).
 * System: the reference solves (-A) phi = rhs with rhs = "_rhs_p"
 * (src/cuda_solver.cu:60-73), so every operator below is (-A), which is
 * symmetric positive (semi-)definite on the fluid cells.
 */
#ifndef BBPP_ORACLE_H
#define BBPP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Boundary type per face: 0 = PERIODIC, 2 = NEUMANN (src/bluebottle.h:218,242). */
typedef struct orc_grid {
  int nx, ny, nz;
  double dx, dy, dz;
  int bc[6]; /* W, E, S, N, B, T */
} orc_grid;

enum { ORC_STOP_REF_RZ = 0, ORC_STOP_TRUE_REL = 1 };
enum {
  ORC_CONVERGED = 0,
  ORC_TINY_RHS = 1,
  ORC_MAX_ITER = 2,
  ORC_NAN = 3,
  ORC_BAD_ARG = 4
};

typedef struct orc_pcg_opts {
  int stop;          /* ORC_STOP_REF_RZ (reference rule) or ORC_STOP_TRUE_REL */
  double tol;        /* pp_residual for REF_RZ; relative residual for TRUE_REL */
  int max_iter;      /* pp_max_iter */
  int replace_every; /* 50 in the reference */
  int nonzero_guess; /* 0: x0 = 0 (reference); 1: start from x on entry */
  int trace_len;     /* number of alpha/beta values to record (may be 0) */
  double *trace_alpha;
  double *trace_beta;
} orc_pcg_opts;

typedef struct orc_pcg_result {
  int status;
  int iters;
  double bb;        /* (rhs, rhs) */
  double rz;        /* last (r, z) */
  double rr;        /* last (r, r), recursive residual */
  double true_rel;  /* ||rhs - (-A)x|| / ||rhs|| evaluated after the solve */
} orc_pcg_result;

/* Ranq1 (Numerical Recipes 3rd ed.), as in src/rng.c:25-51,78-107. */
typedef struct orc_rng { unsigned long long v; int gphase; double g_v1, g_v2, g_s; } orc_rng;
void orc_rng_init(orc_rng *g, unsigned long long seed);
unsigned long long orc_rng_u64(orc_rng *g);
double orc_rng_dbl(orc_rng *g);
double orc_rng_gauss(orc_rng *g);
/* n draws of one stream seeded with seed: uniform on [lo, hi) as lo + (hi - lo)
 * rng_dbl(), or Gaussian by the polar method, in the order the reference's
 * generator returns them (src/rng.c:78-107).  Synthetic inputs. */
void orc_rng_fill_uniform(unsigned long long seed, long long n, double lo, double hi, double *out);
void orc_rng_fill_gauss(unsigned long long seed, long long n, double *out);

int orc_grid_check(const orc_grid *g);
void orc_invm(const orc_grid *g, double *invM);
void orc_spmv(const orc_grid *g, const uint8_t *solid, const double *p, double *Ap);
double orc_dot(long long n, const double *a, const double *b);
int orc_pcg(const orc_grid *g, const uint8_t *solid, const double *rhs, double *x,
            const orc_pcg_opts *o, orc_pcg_result *res);
double orc_true_rel(const orc_grid *g, const uint8_t *solid, const double *rhs, const double *x);

/* Phase mask of spheres (src/particle_kernel.cu:148-253): cell (i,j,k) is
 * solid when floor(d/r) < 1 for the distance d of its centre from a sphere
 * centre; periodic directions use the images at +-length.  Domain origin
 * (xs, ys, zs).  Writes 1 for solid, 0 for fluid. */
void orc_sphere_mask(const orc_grid *g, double xs, double ys, double zs, int nsph,
                     const double *cx, const double *cy, const double *cz,
                     const double *rad, uint8_t *solid);

/* rhs = -(rho/dt) div(u*) (src/solver_kernel.cu:89-176) from face arrays in
 * dense layouts u[(i + (nx+1)*(j + ny*k))] (x faces, i = 0..nx), v[i + nx*(j +
 * (ny+1)*k)] and w[i + nx*(j + ny*k)] with k = 0..nz. */
void orc_rhs_div(const orc_grid *g, double rho_f, double dt, const double *u,
                 const double *v, const double *w, double *rhs);
/* Particle masking of the rhs (src/particle_kernel.cu:1753) followed by
 * coeffs_refine (src/solver_kernel.cu:212-256). */
void orc_rhs_mask_refine(const orc_grid *g, const uint8_t *solid, double *rhs);

/* The time loop's steps after the solve on one rank (src/bluebottle.c:233-252):
 * phi's ghosts (periodic: opposite interior plane, mpi_cuda_exchange_Gcc;
 * Neumann: adjacent interior cell, BC_p_*_N, src/bluebottle_kernel.cu:26-102),
 * the projection u = u* - dt/rho |flag| dphi/dx on every face
 * (project_u/v/w, src/bluebottle_kernel.cu:2303-2355; |flag| = 0 only on a wall
 * face of a non-periodic direction), and the pressure update
 * p = (fluid) (p0 + phi) minus its mean over all cells (update_p,
 * copy_p_p_noghost, forcing_add_c_const, src/cuda_bluebottle.cu:2506-2536).
 * Dense arrays: cells as above; faces u[i + (nx+1)(j + ny k)], i = 0..nx,
 * v[i + nx(j + (ny+1) k)], w[i + nx(j + ny k)], k = 0..nz (as orc_rhs_div). */
void orc_epilogue(const orc_grid *g, const uint8_t *solid, double rho_f, double dt, const double *phi,
                  const double *us, const double *vs, const double *ws, const double *p0, double *u, double *v,
                  double *w, double *p);

/* cuda_build_cages (src/cuda_particle.cu:1516-1646) on one rank: flags reset to
 * 1 (reset_flag_*); with particles, phase = -1 and phase_shell = 1 (reset_phases),
 * then particle by particle in index order the cells of its cage whose centre
 * lies inside it take its index (cage_setup, build_phase), then the solid cells
 * of each particle with a face neighbour centre outside it get phase_shell = 0
 * (build_phase_shell), then the face flags -1 across a phase change or between
 * two shell cells, else 1 (cage_flag_*); finally 0 on both wall faces of a
 * non-periodic direction (flag_external_*).  src/particle_kernel.cu:79-576.
 * Ghosted layouts of the reference: phase, phase_shell (nx+2)(ny+2)(nz+2) x
 * fastest; flag_u [i][k][j] over (nx+3)(nz+2)(ny+2); flag_v [j][i][k] over
 * (ny+3)(nx+2)(nz+2); flag_w [k][j][i] over (nz+3)(ny+2)(nx+2).  Particle
 * centres in domain coordinates, domain origin (xs, ys, zs); with_parts is the
 * reference's NPARTS > 0. */
void orc_build_cages(const orc_grid *g, double xs, double ys, double zs, int with_parts, int nparts,
                     const double *px, const double *py, const double *pz, const double *pr, int *phase,
                     int *phase_shell, int *flag_u, int *flag_v, int *flag_w);

#ifdef __cplusplus
}
#endif
#endif
