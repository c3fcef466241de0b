// bbpp_kernels.cuh -- general-form kernels on the unscaled operator (-A),
// templated on the vector type.  The PCG iteration itself runs on the scaled
// operator in bbpp_fast.cuh; these serve the kernel-level entry points
// (SpMV, residual, the context-free residual) and the checks.
//
//  k_axpy_x       x += alpha p (PP_update_solution, src/solver_kernel.cu:864-881).
//  k_resid        r = rhs - (-A) x with (r,z), (r,r), (rhs,rhs) partials
//                 (PP_update_residual after an SpMV of phi,
//                 src/solver_kernel.cu:883-904, src/cuda_solver.cu:209-224);
//                 with rhs == NULL it writes (-A) x (kernel-level SpMV).
//
// The last CTA of every reducing kernel finishes the global sum in block
// order and updates the device state (alpha; or beta and the stopping test),
// so no scalar crosses to the host inside an iteration.
#pragma once

#include "bbpp_dev.cuh"

namespace bbpp {

constexpr int TX = 32;  // tile width (x), one warp
constexpr int TY = 8;   // tile height (y)
constexpr int HX = TX + 2;
constexpr int HY = TY + 2;
constexpr int NT = TX * TY;  // 256 threads

enum ResidMode : int { RES_INIT = 0, RES_ITER = 1, RES_CONFIRM = 2, RES_PLAIN = 3 };

__device__ __forceinline__ void load_tab(const Geo &G, double *s_tab) {
  for (int e = threadIdx.x; e < 81; e += blockDim.x) s_tab[e] = G.tab[e];
}

template <typename T>
__global__ void __launch_bounds__(NT) k_axpy_x(const Geo G, T *__restrict__ x, const T *__restrict__ p,
                                               const DevState *st) {
  if (*(volatile const int *)&st->done) return;
  const T alpha = (T)(*(volatile const double *)&st->alpha);
  const unsigned int n = (unsigned int)G.n;
  for (unsigned int c = blockIdx.x * NT + threadIdx.x; c < n; c += gridDim.x * NT) x[c] = fma(alpha, p[c], x[c]);
}

// ------------------------------------------------------------ residual -----
// r = rhs - (-A) x   (rhs != NULL), or r = (-A) x  (rhs == NULL, RES_PLAIN).
// TX: type of x and rhs; TR: type of r.  Partials: (r,z), (r,r), (rhs,rhs).
template <typename TXT, typename TR, bool MASK>
__global__ void __launch_bounds__(NT) k_resid(const Geo G, const TXT *__restrict__ xin,
                                              const TXT *__restrict__ rhs, TR *__restrict__ rout,
                                              const uint8_t *__restrict__ mask, DevState *st,
                                              double *partials, int kz, int mode) {
  __shared__ double s_tab[81];
  __shared__ TXT sp[3][HY][HX];
  __shared__ uint8_t sm[3][HY][HX + 2];
  __shared__ double s_red[3 * NT / 32];
  if (mode == RES_ITER && *(volatile int *)&st->done) return;
  load_tab(G, s_tab);
  const int tid = threadIdx.x;
  const int tx = tid & (TX - 1), ty = tid / TX;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  const int z0 = blockIdx.z * kz;
  const int z1 = min(z0 + kz, G.nz);
  const int nx = G.nx, ny = G.ny, nz = G.nz;
  __syncthreads();

  auto load_plane = [&](int slot, int zr) {
    const int gz = halo_index(zr, nz, G.pz);
    for (int e = tid; e < HX * HY; e += NT) {
      const int ly = e / HX, lx = e - ly * HX;
      const int gx = halo_index(x0 + lx - 1, nx, G.px), gy = halo_index(y0 + ly - 1, ny, G.py);
      TXT val = TXT(0);
      uint8_t m = 0;
      if (gz >= 0 && gx >= 0 && gy >= 0) {
        const long long c = gx + (long long)nx * (gy + (long long)ny * gz);
        val = xin[c];
        if (MASK) m = mask[c];
      }
      sp[slot][ly][lx] = val;
      sm[slot][ly][lx] = m;
    }
  };

  double rz = 0, rr = 0, bb = 0;
  load_plane(0, z0 - 1);
  load_plane(1, z0);
  const TXT cx = (TXT)G.cx, cy = (TXT)G.cy, cz = (TXT)G.cz;
  const int gx = x0 + tx, gy = y0 + ty;
  const bool mine = gx < nx && gy < ny;
  const int cls_xy = mine ? (wall_count(gx, nx, G.px) + 3 * wall_count(gy, ny, G.py)) : 0;
  for (int z = z0; z < z1; z++) {
    const int sb = (z - z0) % 3, sc = (z - z0 + 1) % 3, st_ = (z - z0 + 2) % 3;
    load_plane(st_, z + 1);
    __syncthreads();
    if (mine) {
      TXT pc = sp[sc][ty + 1][tx + 1];
      TXT pe = sp[sc][ty + 1][tx + 2], pw = sp[sc][ty + 1][tx];
      TXT pn = sp[sc][ty + 2][tx + 1], ps = sp[sc][ty][tx + 1];
      TXT pt = sp[st_][ty + 1][tx + 1], pb = sp[sb][ty + 1][tx + 1];
      const int cls = cls_xy + 9 * wall_count(z, nz, G.pz);
      TXT d = (TXT)s_tab[cls];
      if (MASK) {
        const bool mc = sm[sc][ty + 1][tx + 1] != 0;
        pe = (mc || sm[sc][ty + 1][tx + 2]) ? TXT(0) : pe;
        pw = (mc || sm[sc][ty + 1][tx]) ? TXT(0) : pw;
        pn = (mc || sm[sc][ty + 2][tx + 1]) ? TXT(0) : pn;
        ps = (mc || sm[sc][ty][tx + 1]) ? TXT(0) : ps;
        pt = (mc || sm[st_][ty + 1][tx + 1]) ? TXT(0) : pt;
        pb = (mc || sm[sb][ty + 1][tx + 1]) ? TXT(0) : pb;
        d = mc ? (TXT)s_tab[54 + cls] : d;
      }
      TXT s = cx * (pe + pw);
      s = fma(cy, pn + ps, s);
      s = fma(cz, pt + pb, s);
      const TXT a = fma(d, pc, -s);
      const long long c = gx + (long long)nx * (gy + (long long)ny * z);
      if (rhs) {
        const TXT bv = rhs[c];
        const TXT rv = bv - a;
        const TR ro = (TR)rv;
        rout[c] = ro;
        const double rd = (double)rv;
        rz = fma(rd, s_tab[27 + cls] * rd, rz);
        rr = fma(rd, rd, rr);
        bb = fma((double)bv, (double)bv, bb);
      } else {
        rout[c] = (TR)a;
      }
    }
    __syncthreads();
  }
  if (mode == RES_PLAIN) return;
  double v[3] = {rz, rr, bb}, tot[3];
  const unsigned int nb = gridDim.x * gridDim.y * gridDim.z;
  const unsigned int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  if (last_cta_reduce<3>(v, partials, st, nb, bid, s_red, tot) && tid == 0) {
    const double rz1 = tot[0], rr1 = tot[1];
    if (mode == RES_INIT) {
      st->bb = tot[2];
      st->tol2bb = st->tol2bb * tot[2];  // host stores tol^2 here before the launch
      st->rz = rz1;
      st->rz_last = rz1;
      st->rr = rr1;
      st->iter = 0;
      st->first = 1;
      st->replacements = 0;
      if (tot[2] < 1e-16) st->done = DONE_TINY;
      else if (st->stop == 1 && rr1 <= st->tol2bb) st->done = DONE_CONVERGED;
      else st->done = RUNNING;
    } else if (mode == RES_ITER) {
      st->replacements += 1;
      finish_iteration(st, rz1, rr1, true);
    } else {  // RES_CONFIRM: explicit residual after a recursive convergence
      st->replacements += 1;
      st->rz_last = rz1;
      st->rr = rr1;
      if (rr1 <= st->tol2bb) {
        st->done = DONE_CONVERGED;
      } else if (isnan(rz1)) {
        st->done = DONE_NAN;
      } else {
        st->beta = rz1 / st->rz;
        st->rz = rz1;
        st->done = (st->iter > st->max_iter) ? DONE_MAX_ITER : RUNNING;
      }
    }
  }
}

}  // namespace bbpp
