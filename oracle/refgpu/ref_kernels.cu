// ref_kernels.cu -- device side of the GPU run of the reference solver.
//
// Test and measurement infrastructure.  Compiled here, by build_cubin.py, into
// oracle/_ref/ref_solver.cubin together with the reference's unmodified
// src/solver_kernel.cu (included below from the reference tree).  The host
// harness (ref_gpu.cu) loads the cubin with the driver API and launches the
// reference's kernels exactly as src/cuda_solver.cu:38-300 / :573-761 do.
//
// The reference kernels read the domain from __constant__ _dom
// (src/bluebottle.cuh:44).  refgpu_fill_dom builds that struct on the device
// with the reference's own layout (this file is compiled with the reference
// headers), so the host copies bytes it never interprets; it also returns the
// strides the host needs (one rank, grids filled as src/domain.c does for a
// single subdomain).
#include "solver_kernel.cu"

__constant__ dom_struct _dom;

static __device__ void fill_grid(grid_info &g, int in, int jn, int kn) {
  g.is = g._is = DOM_BUF; g.isb = g._isb = 0; g.in = in; g.inb = in + 2; g.ie = g._ie = in; g.ieb = g._ieb = in + 1;
  g.js = g._js = DOM_BUF; g.jsb = g._jsb = 0; g.jn = jn; g.jnb = jn + 2; g.je = g._je = jn; g.jeb = g._jeb = jn + 1;
  g.ks = g._ks = DOM_BUF; g.ksb = g._ksb = 0; g.kn = kn; g.knb = kn + 2; g.ke = g._ke = kn; g.keb = g._keb = kn + 1;
}

// out: a dom_struct in global memory; info[0..15]: Gcc s1b s2b s3b s1 s2 s3,
// Gfx s1b s2b s3b, Gfy s1b s2b s3b, Gfz s1b s2b s3b, sizeof(dom_struct)
extern "C" __global__ void refgpu_fill_dom(dom_struct *out, long long *info, int nx, int ny, int nz, double dx,
                                           double dy, double dz) {
  if (threadIdx.x || blockIdx.x) return;
  dom_struct d;
  memset(&d, 0, sizeof(d));
  d.xs = 0; d.xn = nx; d.dx = dx; d.xe = nx * dx; d.xl = d.xe;
  d.ys = 0; d.yn = ny; d.dy = dy; d.ye = ny * dy; d.yl = d.ye;
  d.zs = 0; d.zn = nz; d.dz = dz; d.ze = nz * dz; d.zl = d.ze;
  d.In = d.Jn = d.Kn = 1; d.S1 = d.S2 = d.S3 = 1;
  fill_grid(d.Gcc, nx, ny, nz);  // x fastest
  d.Gcc.s1 = d.Gcc.in; d.Gcc.s2 = d.Gcc.s1 * d.Gcc.jn; d.Gcc.s3 = d.Gcc.s2 * d.Gcc.kn;
  d.Gcc.s1b = d.Gcc.inb; d.Gcc.s2b = d.Gcc.s1b * d.Gcc.jnb; d.Gcc.s3b = d.Gcc.s2b * d.Gcc.knb;
  fill_grid(d.Gfx, nx + 1, ny, nz);  // GFX_LOC = j + k s1b + i s2b
  d.Gfx.s1 = d.Gfx.jn; d.Gfx.s2 = d.Gfx.s1 * d.Gfx.kn; d.Gfx.s3 = d.Gfx.s2 * d.Gfx.in;
  d.Gfx.s1b = d.Gfx.jnb; d.Gfx.s2b = d.Gfx.s1b * d.Gfx.knb; d.Gfx.s3b = d.Gfx.s2b * d.Gfx.inb;
  fill_grid(d.Gfy, nx, ny + 1, nz);  // GFY_LOC = k + i s1b + j s2b
  d.Gfy.s1 = d.Gfy.kn; d.Gfy.s2 = d.Gfy.s1 * d.Gfy.in; d.Gfy.s3 = d.Gfy.s2 * d.Gfy.jn;
  d.Gfy.s1b = d.Gfy.knb; d.Gfy.s2b = d.Gfy.s1b * d.Gfy.inb; d.Gfy.s3b = d.Gfy.s2b * d.Gfy.jnb;
  fill_grid(d.Gfz, nx, ny, nz + 1);  // GFZ_LOC = i + j s1b + k s2b
  d.Gfz.s1 = d.Gfz.in; d.Gfz.s2 = d.Gfz.s1 * d.Gfz.jn; d.Gfz.s3 = d.Gfz.s2 * d.Gfz.kn;
  d.Gfz.s1b = d.Gfz.inb; d.Gfz.s2b = d.Gfz.s1b * d.Gfz.jnb; d.Gfz.s3b = d.Gfz.s2b * d.Gfz.knb;
  *out = d;
  const grid_info *gs[4] = {&d.Gcc, &d.Gfx, &d.Gfy, &d.Gfz};
  info[0] = d.Gcc.s1b; info[1] = d.Gcc.s2b; info[2] = d.Gcc.s3b;
  info[3] = d.Gcc.s1; info[4] = d.Gcc.s2; info[5] = d.Gcc.s3;
  for (int g = 1; g < 4; g++) {
    info[3 + 3 * g] = gs[g]->s1b;
    info[4 + 3 * g] = gs[g]->s2b;
    info[5 + 3 * g] = gs[g]->s3b;
  }
  info[15] = sizeof(dom_struct);
}
