/*
 * bbpp_oracle.c -- CPU oracle (test infrastructure; see bbpp_oracle.h).
 *
 * Plain C, FP64, OpenMP over z-planes.  Reductions are deterministic: fixed
 * chunks of cells are summed in parallel and the chunk sums are then added in
 * order, so the result does not depend on the thread count.
 * Compiled with -ffp-contract=off so x86 and Arm hosts give identical bits.
 */
#include "bbpp_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_CHUNK 4096

/* ---------------------------------------------------------------- RNG ---- */
/* Ranq1, src/rng.c:28-51; uniform double src/rng.c:78-81; Marsaglia polar
 * Gaussian src/rng.c:85-107 (state kept per generator instead of static). */
void orc_rng_init(orc_rng *g, unsigned long long seed)
{
  g->v = 4101842887655102017ULL;
  g->v ^= seed;
  g->v = orc_rng_u64(g);
  g->gphase = 0;
  g->g_v1 = g->g_v2 = g->g_s = 0.;
}

unsigned long long orc_rng_u64(orc_rng *g)
{
  g->v ^= g->v >> 21;
  g->v ^= g->v << 35;
  g->v ^= g->v >> 4;
  return g->v * 2685821657736338717ULL;
}

double orc_rng_dbl(orc_rng *g) { return 5.42101086242752217e-20 * (double)orc_rng_u64(g); }

double orc_rng_gauss(orc_rng *g)
{
  double X;
  if (g->gphase == 0) {
    do {
      double U1 = orc_rng_dbl(g);
      double U2 = orc_rng_dbl(g);
      g->g_v1 = 2 * U1 - 1;
      g->g_v2 = 2 * U2 - 1;
      g->g_s = g->g_v1 * g->g_v1 + g->g_v2 * g->g_v2;
    } while (g->g_s >= 1 || g->g_s == 0);
    X = g->g_v1 * sqrt(-2 * log(g->g_s) / g->g_s);
  } else {
    X = g->g_v2 * sqrt(-2 * log(g->g_s) / g->g_s);
  }
  g->gphase = 1 - g->gphase;
  return X;
}

void orc_rng_fill_uniform(unsigned long long seed, long long n, double lo, double hi, double *out)
{
  orc_rng g;
  orc_rng_init(&g, seed);
  for (long long i = 0; i < n; i++) out[i] = lo + (hi - lo) * orc_rng_dbl(&g);
}

void orc_rng_fill_gauss(unsigned long long seed, long long n, double *out)
{
  orc_rng g;
  orc_rng_init(&g, seed);
  for (long long i = 0; i < n; i++) out[i] = orc_rng_gauss(&g);
}

/* --------------------------------------------------------------- grid ---- */
int orc_grid_check(const orc_grid *g)
{
  if (!g || g->nx < 1 || g->ny < 1 || g->nz < 1) return ORC_BAD_ARG;
  if (!(g->dx > 0) || !(g->dy > 0) || !(g->dz > 0)) return ORC_BAD_ARG;
  for (int f = 0; f < 6; f++)
    if (g->bc[f] != 0 && g->bc[f] != 2) return ORC_BAD_ARG;
  /* a direction is either periodic on both faces or walled on both faces
   * (flag_external_* is applied only in that case, src/cuda_particle.cu:1606-1639) */
  if (g->bc[0] != g->bc[1] || g->bc[2] != g->bc[3] || g->bc[4] != g->bc[5]) return ORC_BAD_ARG;
  return 0;
}

/* Face flag squared (0 or 1): 0 only on the two walls of a non-periodic
 * direction (flag_external_*, src/particle_kernel.cu:542-576). */
static inline int face_lo(int i, int per) { return (i == 0 && !per) ? 0 : 1; }
static inline int face_hi(int i, int n, int per) { return (i == n - 1 && !per) ? 0 : 1; }

/* invM, src/solver_kernel.cu:72-80: M = -idx2(fE^2+fW^2) - idy2(..) - idz2(..),
 * invM = -1/M. */
void orc_invm(const orc_grid *g, double *invM)
{
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const int px = g->bc[0] == 0, py = g->bc[2] == 0, pz = g->bc[4] == 0;
  const double idx2 = 1. / (g->dx * g->dx);
  const double idy2 = 1. / (g->dy * g->dy);
  const double idz2 = 1. / (g->dz * g->dz);
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        double M = -idx2 * (face_hi(i, nx, px) + face_lo(i, px))
                   - idy2 * (face_hi(j, ny, py) + face_lo(j, py))
                   - idz2 * (face_hi(k, nz, pz) + face_lo(k, pz));
        invM[i + (long long)nx * (j + (long long)ny * k)] = -1. / M;
      }
}

/* (-A)p, src/solver_kernel.cu:684-707 (particles) and :824-829 (no particles).
 * solid == NULL selects the particle-free operator.  A neighbour across a
 * wall face is never read (its coefficient is a zero flag). */
void orc_spmv(const orc_grid *g, const uint8_t *solid, const double *p, double *Ap)
{
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const int px = g->bc[0] == 0, py = g->bc[2] == 0, pz = g->bc[4] == 0;
  const double idx2 = 1. / (g->dx * g->dx);
  const double idy2 = 1. / (g->dy * g->dy);
  const double idz2 = 1. / (g->dz * g->dz);
  const long long sx = 1, sy = nx, sz = (long long)nx * ny;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; k++) {
    for (int j = 0; j < ny; j++) {
      for (int i = 0; i < nx; i++) {
        const long long c = i + sy * j + sz * k;
        const int fe = face_hi(i, nx, px), fw = face_lo(i, px);
        const int fn = face_hi(j, ny, py), fs = face_lo(j, py);
        const int ft = face_hi(k, nz, pz), fb = face_lo(k, pz);
        const long long ce = fe ? c + (i == nx - 1 ? -(nx - 1) * sx : sx) : c;
        const long long cw = fw ? c + (i == 0 ? (nx - 1) * sx : -sx) : c;
        const long long cn = fn ? c + (j == ny - 1 ? -(ny - 1) * sy : sy) : c;
        const long long cs = fs ? c + (j == 0 ? (ny - 1) * sy : -sy) : c;
        const long long ct = ft ? c + (k == nz - 1 ? -(nz - 1) * sz : sz) : c;
        const long long cb = fb ? c + (k == 0 ? (nz - 1) * sz : -sz) : c;
        const double pc = p[c];
        const double pe = fe ? p[ce] : 0., pw = fw ? p[cw] : 0.;
        const double pn = fn ? p[cn] : 0., ps = fs ? p[cs] : 0.;
        const double pt = ft ? p[ct] : 0., pb = fb ? p[cb] : 0.;
        double a;
        if (!solid) {
          a = -idx2 * (fe * (pe - pc) - fw * (pc - pw))
              - idy2 * (fn * (pn - pc) - fs * (pc - ps))
              - idz2 * (ft * (pt - pc) - fb * (pc - pb));
        } else {
          const int sc = solid[c] != 0;
          const int fl = !sc;
          /* particle modification factors, src/solver_kernel.cu:684-696 */
          const double pfx = -(g->dx * g->dx) / 6. * sc + (double)fl;
          const double pfy = -(g->dy * g->dy) / 6. * sc + (double)fl;
          const double pfz = -(g->dz * g->dz) / 6. * sc + (double)fl;
          const int pfe = fl && !(fe && solid[ce]);
          const int pfw = fl && !(fw && solid[cw]);
          const int pfn = fl && !(fn && solid[cn]);
          const int pfs = fl && !(fs && solid[cs]);
          const int pft = fl && !(ft && solid[ct]);
          const int pfb = fl && !(fb && solid[cb]);
          a = -idx2 * (fe * (pe * pfe - pfx * pc) - fw * (pc * pfx - pfw * pw));
          a += -idy2 * (fn * (pn * pfn - pfy * pc) - fs * (pc * pfy - pfs * ps));
          a += -idz2 * (ft * (pt * pft - pfz * pc) - fb * (pc * pfz - pfb * pb));
        }
        Ap[c] = a;
      }
    }
  }
}

double orc_dot(long long n, const double *a, const double *b)
{
  const long long nch = (n + ORC_CHUNK - 1) / ORC_CHUNK;
  double *part = (double *)malloc(sizeof(double) * (size_t)(nch > 0 ? nch : 1));
#pragma omp parallel for schedule(static)
  for (long long ch = 0; ch < nch; ch++) {
    const long long lo = ch * ORC_CHUNK;
    const long long hi = lo + ORC_CHUNK < n ? lo + ORC_CHUNK : n;
    double s = 0.;
    for (long long c = lo; c < hi; c++) s += a[c] * b[c];
    part[ch] = s;
  }
  double s = 0.;
  for (long long ch = 0; ch < nch; ch++) s += part[ch];
  free(part);
  return s;
}

/* r.z with z = invM r, and r.r, both deterministic. */
static void dot_rz_rr(long long n, const double *r, const double *invM, double *rz, double *rr)
{
  const long long nch = (n + ORC_CHUNK - 1) / ORC_CHUNK;
  double *part = (double *)malloc(sizeof(double) * 2 * (size_t)(nch > 0 ? nch : 1));
#pragma omp parallel for schedule(static)
  for (long long ch = 0; ch < nch; ch++) {
    const long long lo = ch * ORC_CHUNK;
    const long long hi = lo + ORC_CHUNK < n ? lo + ORC_CHUNK : n;
    double s = 0., t = 0.;
    for (long long c = lo; c < hi; c++) {
      const double z = r[c] * invM[c];
      s += r[c] * z;
      t += r[c] * r[c];
    }
    part[2 * ch] = s;
    part[2 * ch + 1] = t;
  }
  double s = 0., t = 0.;
  for (long long ch = 0; ch < nch; ch++) { s += part[2 * ch]; t += part[2 * ch + 1]; }
  free(part);
  *rz = s;
  *rr = t;
}

double orc_true_rel(const orc_grid *g, const uint8_t *solid, const double *rhs, const double *x)
{
  const long long n = (long long)g->nx * g->ny * g->nz;
  double *Ax = (double *)malloc(sizeof(double) * (size_t)n);
  orc_spmv(g, solid, x, Ax);
#pragma omp parallel for schedule(static)
  for (long long c = 0; c < n; c++) Ax[c] = rhs[c] - Ax[c];
  const double rr = orc_dot(n, Ax, Ax);
  const double bb = orc_dot(n, rhs, rhs);
  free(Ax);
  return bb > 0 ? sqrt(rr / bb) : sqrt(rr);
}

/* Jacobi PCG, src/cuda_solver.cu:150-279 with the kernels
 * PP_cg_init (src/solver_kernel.cu:258-283), PP_update_soln_resid (:838-862),
 * PP_update_solution / PP_update_residual (:864-904) and PP_update_search
 * (:906-927).  Residual replacement when q % replace_every == 0
 * (src/cuda_solver.cu:209-224).  Tiny-RHS exit at (rhs,rhs) < 1e-16
 * (src/cuda_solver.cu:178-190).  TRUE_REL stops on the recursive ||r||, then
 * confirms with an explicit rhs - (-A)x and continues after a residual
 * replacement if the explicit residual is still too large. */
int orc_pcg(const orc_grid *g, const uint8_t *solid, const double *rhs, double *x,
            const orc_pcg_opts *o, orc_pcg_result *res)
{
  orc_pcg_result tmp;
  if (!res) res = &tmp;
  memset(res, 0, sizeof(*res));
  if (orc_grid_check(g) || !rhs || !x || !o || o->replace_every < 1 || o->max_iter < 0) {
    res->status = ORC_BAD_ARG;
    return ORC_BAD_ARG;
  }
  const long long n = (long long)g->nx * g->ny * g->nz;
  double *invM = (double *)malloc(sizeof(double) * (size_t)n);
  double *r = (double *)malloc(sizeof(double) * (size_t)n);
  double *p = (double *)malloc(sizeof(double) * (size_t)n);
  double *Ap = (double *)malloc(sizeof(double) * (size_t)n);
  orc_invm(g, invM);

  const double bb = orc_dot(n, rhs, rhs);
  res->bb = bb;
  if (o->nonzero_guess) {
    orc_spmv(g, solid, x, Ap);
#pragma omp parallel for schedule(static)
    for (long long c = 0; c < n; c++) r[c] = rhs[c] - Ap[c];
  } else {
#pragma omp parallel for schedule(static)
    for (long long c = 0; c < n; c++) { r[c] = rhs[c]; x[c] = 0.; }
  }
#pragma omp parallel for schedule(static)
  for (long long c = 0; c < n; c++) p[c] = r[c] * invM[c];
  double rz, rr;
  dot_rz_rr(n, r, invM, &rz, &rr);
  const double tol2bb = o->tol * o->tol * bb;

  int q = 0;
  int status = ORC_MAX_ITER;
  const double RHS_TOL = 1.e-8;
  if (bb < RHS_TOL * RHS_TOL) {
    status = ORC_TINY_RHS;
  } else if (o->stop == ORC_STOP_TRUE_REL && rr <= tol2bb) {
    status = ORC_CONVERGED; /* a guess already good enough */
  } else {
    double rz1 = rz, rr1 = rr;
    while (q <= o->max_iter) {
      ++q;
      orc_spmv(g, solid, p, Ap);
      const double denom = orc_dot(n, p, Ap);
      const double alpha = rz / denom;
      if (q - 1 < o->trace_len && o->trace_alpha) o->trace_alpha[q - 1] = alpha;
      if (q % o->replace_every == 0) {
#pragma omp parallel for schedule(static)
        for (long long c = 0; c < n; c++) x[c] += alpha * p[c];
        orc_spmv(g, solid, x, Ap);
#pragma omp parallel for schedule(static)
        for (long long c = 0; c < n; c++) r[c] = rhs[c] - Ap[c];
      } else {
#pragma omp parallel for schedule(static)
        for (long long c = 0; c < n; c++) {
          x[c] += alpha * p[c];
          r[c] -= alpha * Ap[c];
        }
      }
      dot_rz_rr(n, r, invM, &rz1, &rr1);
      int conv;
      if (o->stop == ORC_STOP_REF_RZ) {
        conv = rz1 <= tol2bb;
      } else {
        conv = rr1 <= tol2bb;
        if (conv) {
          /* confirm against the explicit residual */
          orc_spmv(g, solid, x, Ap);
#pragma omp parallel for schedule(static)
          for (long long c = 0; c < n; c++) r[c] = rhs[c] - Ap[c];
          dot_rz_rr(n, r, invM, &rz1, &rr1);
          conv = rr1 <= tol2bb;
        }
      }
      if (conv) {
        status = ORC_CONVERGED;
        break;
      } else if (isnan(rz1)) {
        status = ORC_NAN;
        break;
      }
      const double beta = rz1 / rz;
      if (q - 1 < o->trace_len && o->trace_beta) o->trace_beta[q - 1] = beta;
#pragma omp parallel for schedule(static)
      for (long long c = 0; c < n; c++) p[c] = r[c] * invM[c] + beta * p[c];
      rz = rz1;
      rr = rr1;
    }
    rz = rz1;
    rr = rr1;
    if (status == ORC_MAX_ITER) q = o->max_iter + 1;
  }
  res->status = status;
  res->iters = q;
  res->rz = rz;
  res->rr = rr;
  res->true_rel = orc_true_rel(g, solid, rhs, x);
  free(invM);
  free(r);
  free(p);
  free(Ap);
  return status;
}

/* --------------------------------------------------------------- mask ---- */
void orc_sphere_mask(const orc_grid *g, double xs, double ys, double zs, int nsph,
                     const double *cx, const double *cy, const double *cz,
                     const double *rad, uint8_t *solid)
{
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const int px = g->bc[0] == 0, py = g->bc[2] == 0, pz = g->bc[4] == 0;
  const double xl = nx * g->dx, yl = ny * g->dy, zl = nz * g->dz;
  memset(solid, 0, (size_t)nx * ny * nz);
  for (int s = 0; s < nsph; s++) {
    const double irad = 1. / rad[s];
    for (int ox = px ? -1 : 0; ox <= (px ? 1 : 0); ox++)
      for (int oy = py ? -1 : 0; oy <= (py ? 1 : 0); oy++)
        for (int oz = pz ? -1 : 0; oz <= (pz ? 1 : 0); oz++) {
          const double X = cx[s] + ox * xl, Y = cy[s] + oy * yl, Z = cz[s] + oz * zl;
          int i0 = (int)floor((X - xs - rad[s]) / g->dx) - 1, i1 = (int)ceil((X - xs + rad[s]) / g->dx) + 1;
          int j0 = (int)floor((Y - ys - rad[s]) / g->dy) - 1, j1 = (int)ceil((Y - ys + rad[s]) / g->dy) + 1;
          int k0 = (int)floor((Z - zs - rad[s]) / g->dz) - 1, k1 = (int)ceil((Z - zs + rad[s]) / g->dz) + 1;
          if (i0 < 0) i0 = 0;
          if (j0 < 0) j0 = 0;
          if (k0 < 0) k0 = 0;
          if (i1 > nx - 1) i1 = nx - 1;
          if (j1 > ny - 1) j1 = ny - 1;
          if (k1 > nz - 1) k1 = nz - 1;
          for (int k = k0; k <= k1; k++)
            for (int j = j0; j <= j1; j++)
              for (int i = i0; i <= i1; i++) {
                /* cell centre ((ti - 0.5) dx with ti = i + 1), src/particle_kernel.cu:236-245 */
                const double xx = ((double)(i + 1) - 0.5) * g->dx - (X - xs);
                const double yy = ((double)(j + 1) - 0.5) * g->dy - (Y - ys);
                const double zz = ((double)(k + 1) - 0.5) * g->dz - (Z - zs);
                const double d = sqrt(xx * xx + yy * yy + zz * zz);
                if (floor(d * irad) < 1) solid[i + (long long)nx * (j + (long long)ny * k)] = 1;
              }
        }
  }
}

/* ---------------------------------------------------------------- rhs ---- */
void orc_rhs_div(const orc_grid *g, double rho_f, double dt, const double *u,
                 const double *v, const double *w, double *rhs)
{
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const double idx = 1. / g->dx, idy = 1. / g->dy, idz = 1. / g->dz;
  const double rho_idt = rho_f / dt;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        const long long uw = i + (long long)(nx + 1) * (j + (long long)ny * k);
        const long long vs = i + (long long)nx * (j + (long long)(ny + 1) * k);
        const long long wb = i + (long long)nx * (j + (long long)ny * k);
        double s = (u[uw + 1] - u[uw]) * idx;
        s += (v[vs + nx] - v[vs]) * idy;
        s += (w[wb + (long long)nx * ny] - w[wb]) * idz;
        s *= rho_idt;
        rhs[i + (long long)nx * (j + (long long)ny * k)] = -s;
      }
}

void orc_rhs_mask_refine(const orc_grid *g, const uint8_t *solid, double *rhs)
{
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const long long n = (long long)nx * ny * nz;
  if (!solid) return;
  const int px = g->bc[0] == 0, py = g->bc[2] == 0, pz = g->bc[4] == 0;
  const double idx2 = 1. / (g->dx * g->dx);
  const double idy2 = 1. / (g->dy * g->dy);
  const double idz2 = 1. / (g->dz * g->dz);
  /* part_BC_p: rhs of a solid cell is zero (src/particle_kernel.cu:1753) */
  for (long long c = 0; c < n; c++)
    if (solid[c]) rhs[c] = 0.;
  /* coeffs_refine: rhs[fluid] += sum over solid neighbours of idd2*(-rhs[nbr]).
   * The ghost of a wall face holds zero rhs (zero_rhs_ghost_*), so walls add
   * nothing; periodic neighbours wrap. */
  double *out = (double *)malloc(sizeof(double) * (size_t)n);
  memcpy(out, rhs, sizeof(double) * (size_t)n);
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        const long long c = i + (long long)nx * (j + (long long)ny * k);
        if (solid[c]) continue;
        const long long sy = nx, sz = (long long)nx * ny;
        double acc = out[c];
        int ok;
        long long e;
        ok = (i < nx - 1) || px; e = c + (i == nx - 1 ? -(nx - 1) : 1);
        if (ok) acc += (solid[e] != 0) * idx2 * (-rhs[e]);
        ok = (i > 0) || px; e = c + (i == 0 ? (nx - 1) : -1);
        if (ok) acc += (solid[e] != 0) * idx2 * (-rhs[e]);
        ok = (j < ny - 1) || py; e = c + (j == ny - 1 ? -(ny - 1) * sy : sy);
        if (ok) acc += (solid[e] != 0) * idy2 * (-rhs[e]);
        ok = (j > 0) || py; e = c + (j == 0 ? (ny - 1) * sy : -sy);
        if (ok) acc += (solid[e] != 0) * idy2 * (-rhs[e]);
        ok = (k < nz - 1) || pz; e = c + (k == nz - 1 ? -(nz - 1) * sz : sz);
        if (ok) acc += (solid[e] != 0) * idz2 * (-rhs[e]);
        ok = (k > 0) || pz; e = c + (k == 0 ? (nz - 1) * sz : -sz);
        if (ok) acc += (solid[e] != 0) * idz2 * (-rhs[e]);
        out[c] = acc;
      }
  memcpy(rhs, out, sizeof(double) * (size_t)n);
  free(out);
}

/* ------------------------------------------------------------ epilogue --- */
/* phi at cell index g (may be -1 or n: a ghost): periodic wrap, or the
 * adjacent interior cell (Neumann ghost, BC_p_*_N) */
static inline int ghost_cell(int g, int n, int periodic)
{
  if (g < 0) return periodic ? n - 1 : 0;
  if (g >= n) return periodic ? 0 : n - 1;
  return g;
}

void orc_epilogue(const orc_grid *g, const uint8_t *solid, double rho_f, double dt, const double *phi,
                  const double *us, const double *vs, const double *ws, const double *p0, double *u, double *v,
                  double *w, double *p)
{
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const int px = g->bc[0] == 0, py = g->bc[2] == 0, pz = g->bc[4] == 0;
  const double ddx = 1. / g->dx, ddy = 1. / g->dy, ddz = 1. / g->dz;
#define PHI(i, j, k) phi[(long long)(i) + (long long)nx * ((j) + (long long)ny * (k))]
  /* project_u: faces i = 0..nx between cells i-1 and i */
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i <= nx; i++) {
        const int fl = px || (i > 0 && i < nx); /* |flag_u| */
        const double grad = (double)fl * ddx * (PHI(ghost_cell(i, nx, px), j, k) - PHI(ghost_cell(i - 1, nx, px), j, k));
        const long long f = i + (long long)(nx + 1) * (j + (long long)ny * k);
        u[f] = us[f] - dt / rho_f * grad;
      }
  for (int k = 0; k < nz; k++)
    for (int j = 0; j <= ny; j++)
      for (int i = 0; i < nx; i++) {
        const int fl = py || (j > 0 && j < ny);
        const double grad = (double)fl * ddy * (PHI(i, ghost_cell(j, ny, py), k) - PHI(i, ghost_cell(j - 1, ny, py), k));
        const long long f = i + (long long)nx * (j + (long long)(ny + 1) * k);
        v[f] = vs[f] - dt / rho_f * grad;
      }
  for (int k = 0; k <= nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        const int fl = pz || (k > 0 && k < nz);
        const double grad = (double)fl * ddz * (PHI(i, j, ghost_cell(k, nz, pz)) - PHI(i, j, ghost_cell(k - 1, nz, pz)));
        const long long f = i + (long long)nx * (j + (long long)ny * k);
        w[f] = ws[f] - dt / rho_f * grad;
      }
#undef PHI
  /* update_p and the mean removal: a sequential sum in cell order */
  const long long n = (long long)nx * ny * nz;
  double s = 0.;
  for (long long c = 0; c < n; c++) {
    p[c] = (double)(!solid || !solid[c]) * (p0[c] + phi[c]);
    s += p[c];
  }
  const double mean = s / (double)n;
  for (long long c = 0; c < n; c++) p[c] += -mean;
}

/* ------------------------------------------------------------- cages ---- */
/* The cage of particle n on one axis (cage_setup and the start/end clamp of
 * build_phase, src/particle_kernel.cu:134-146,158-224): first cell s, last
 * cell e (inclusive, ghosted index), and the number of cells the launch's
 * threads reach from s (blocks of 8 threads cover ceil(cage/8) * 8 cells). */
typedef struct cage_axis { int s, e, reach; } cage_axis;

static cage_axis cage_on_axis(double c, double origin, double h, double rad, int n, int lo_wall, int hi_wall)
{
  cage_axis a;
  const int dim = (int)(2. * ceil(rad / h)) + 2 - n % 2;
  const double ih = 1. / h;
  int s = (int)(round((c - origin) * ih) - 0.5 * dim + 1);
  int e = s + dim;
  const int lo = lo_wall ? 1 : 0, hi = hi_wall ? n : n + 1;
  s += (lo - s) * (s < lo) + (hi - s) * (s > hi);
  e += (lo - e) * (e < lo) + (hi - e) * (e > hi);
  a.s = s;
  a.e = e;
  a.reach = (int)ceil((double)dim * (1. / 8)) * 8;
  return a;
}

static int inside_sphere(double xx, double yy, double zz, double irad)
{
  const double d = sqrt(xx * xx + yy * yy + zz * zz);
  return floor(d * irad) < 1;
}

void orc_build_cages(const orc_grid *g, double xs, double ys, double zs, int with_parts, int nparts,
                     const double *px, const double *py, const double *pz, const double *pr, int *phase,
                     int *phase_shell, int *flag_u, int *flag_v, int *flag_w)
{
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const int cx = nx + 2, cy = ny + 2, cz = nz + 2;          /* ghosted cell extents */
  const long long ncc = (long long)cx * cy * cz;
  const long long nfx = (long long)(nx + 3) * cz * cy, nfy = (long long)(ny + 3) * cx * cz,
                  nfz = (long long)(nz + 3) * cy * cx;
  for (long long c = 0; c < nfx; c++) flag_u[c] = 1;
  for (long long c = 0; c < nfy; c++) flag_v[c] = 1;
  for (long long c = 0; c < nfz; c++) flag_w[c] = 1;
#define CC(i, j, k) ((i) + (long long)cx * ((j) + (long long)cy * (k)))
  if (with_parts) {
    for (long long c = 0; c < ncc; c++) { phase[c] = -1; phase_shell[c] = 1; }
    for (int pass = 0; pass < 2; pass++)
      for (int n = 0; n < nparts; n++) {
        const double rx = px[n] - xs, ry = py[n] - ys, rz = pz[n] - zs, irad = 1. / pr[n];
        const cage_axis ax = cage_on_axis(px[n], xs, g->dx, pr[n], nx, g->bc[0] != 0, g->bc[1] != 0);
        const cage_axis ay = cage_on_axis(py[n], ys, g->dy, pr[n], ny, g->bc[2] != 0, g->bc[3] != 0);
        const cage_axis az = cage_on_axis(pz[n], zs, g->dz, pr[n], nz, g->bc[4] != 0, g->bc[5] != 0);
        if (ax.s == ax.e || ay.s == ay.e || az.s == az.e || ax.reach <= 0 || ay.reach <= 0 || az.reach <= 0)
          continue;
        for (int k = az.s; k <= az.e && k < az.s + az.reach; k++)
          for (int j = ay.s; j <= ay.e && j < ay.s + ay.reach; j++)
            for (int i = ax.s; i <= ax.e && i < ax.s + ax.reach; i++) {
              const long long C = CC(i, j, k);
              const double xx = (i - 0.5) * g->dx - rx, yy = (j - 0.5) * g->dy - ry, zz = (k - 0.5) * g->dz - rz;
              if (pass == 0) {
                if (inside_sphere(xx, yy, zz, irad)) phase[C] = n;
              } else if (phase[C] == n) {
                const double xw = (i - 1 - 0.5) * g->dx - rx, xe = (i + 1 - 0.5) * g->dx - rx;
                const double ysn = (j - 1 - 0.5) * g->dy - ry, yn = (j + 1 - 0.5) * g->dy - ry;
                const double zb = (k - 1 - 0.5) * g->dz - rz, zt = (k + 1 - 0.5) * g->dz - rz;
                if (!inside_sphere(xw, yy, zz, irad) || !inside_sphere(xe, yy, zz, irad) ||
                    !inside_sphere(xx, ysn, zz, irad) || !inside_sphere(xx, yn, zz, irad) ||
                    !inside_sphere(xx, yy, zb, irad) || !inside_sphere(xx, yy, zt, irad))
                  phase_shell[C] = 0;
              }
            }
      }
    /* a face flips to -1 between a fluid and a solid cell, or between two shell cells */
#define FLIP(a, b) (((phase[a] < 0) != (phase[b] < 0)) || (phase_shell[a] < 1 && phase_shell[b] < 1))
    for (int k = 0; k < cz; k++)
      for (int j = 0; j < cy; j++)
        for (int i = 1; i <= nx + 1; i++)
          flag_u[j + (long long)cy * (k + (long long)cz * i)] = FLIP(CC(i - 1, j, k), CC(i, j, k)) ? -1 : 1;
    for (int k = 0; k < cz; k++)
      for (int j = 1; j <= ny + 1; j++)
        for (int i = 0; i < cx; i++)
          flag_v[k + (long long)cz * (i + (long long)cx * j)] = FLIP(CC(i, j - 1, k), CC(i, j, k)) ? -1 : 1;
    for (int k = 1; k <= nz + 1; k++)
      for (int j = 0; j < cy; j++)
        for (int i = 0; i < cx; i++)
          flag_w[i + (long long)cx * (j + (long long)cy * k)] = FLIP(CC(i, j, k - 1), CC(i, j, k)) ? -1 : 1;
#undef FLIP
  }
#undef CC
  /* walls of a non-periodic direction: flag 0 on both boundary faces */
  if (g->bc[0] != 0 && g->bc[1] != 0)
    for (int k = 0; k < cz; k++)
      for (int j = 0; j < cy; j++) {
        flag_u[j + (long long)cy * (k + (long long)cz * 1)] = 0;
        flag_u[j + (long long)cy * (k + (long long)cz * (nx + 1))] = 0;
      }
  if (g->bc[2] != 0 && g->bc[3] != 0)
    for (int k = 0; k < cz; k++)
      for (int i = 0; i < cx; i++) {
        flag_v[k + (long long)cz * (i + (long long)cx * 1)] = 0;
        flag_v[k + (long long)cz * (i + (long long)cx * (ny + 1))] = 0;
      }
  if (g->bc[4] != 0 && g->bc[5] != 0)
    for (int j = 0; j < cy; j++)
      for (int i = 0; i < cx; i++) {
        flag_w[i + (long long)cx * (j + (long long)cy * 1)] = 0;
        flag_w[i + (long long)cx * (j + (long long)cy * (nz + 1))] = 0;
      }
}
