// bbpp_tma.cu -- the FP32 iteration kernels with TMA-staged z-slabs: the
// search kernel of the two-kernel iteration (k1_tma), and the fused iteration
// kernel (k1_fused, described where it is defined), which adds the previous
// iteration's update to the same slab pipeline and L2 bulk prefetches.
//
// A CTA owns a slab of TY full x-rows (all nx cells of rows y0 .. y0+TY-1)
// and marches through its z range.  For every plane one thread issues tensor
// copies (cp.async.bulk.tensor) of r and p_old: the TY rows of the slab plus
// the two halo rows y0-1 and y0+TY (wrapped for periodic y; a row outside a
// wall reads the copy unit's zero fill).  Planes outside a Neumann wall are
// zero-filled the same way.  The copies land in a ring of NS stages, each
// completing on its own mbarrier, so several planes are in flight while the
// CTA computes.  Because a stage holds whole rows, the x neighbours of the
// periodic wrap are in shared memory already and no x halo is copied.
//
// Per plane: p_new = z + beta p_old over the stage (in place of r; z = r on
// fluid cells away from walls, r / dL on wall classes), then, one plane
// behind, Ap = L p_new on the slab's own cells with the (p, Ap) partial, the
// stores of p_new and Ap, and x += alpha p_old (x lags one iteration).  The
// arithmetic is the same as k1_search2's (apply_L), so both kernels give
// bit-identical p_new, Ap and x.  Replaces PP_update_search + halo exchange +
// PP_spmv_shared_load + thrust (p, Ap) (src/solver_kernel.cu:528-713,906-927,
// src/cuda_solver.cu:201-205,256-263), in FP32.
//
// Every mbarrier wait is bounded (one second of globaltimer, or the state's
// wait_ns); a wait that runs out marks the CTA, which keeps to the barrier
// schedule, drains its outstanding copies with bounded waits, and ends the
// solve with DONE_TIMEOUT for the host to report.  A test hook (inject) makes
// one CTA leave one plane's copies unissued, so that this path runs without
// any fault.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "bbpp_internal.h"
#include "bbpp_fast.cuh"

using namespace bbpp;

namespace {

constexpr int TNT = 256;  // threads per CTA

__device__ __forceinline__ unsigned int smem_addr(const void *p) {
  return (unsigned int)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned int bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned int parity) {
  unsigned int ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Wait for the phase with this parity; false after limit_ns without completion.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned int parity, unsigned long long limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = globaltimer();
  for (unsigned int k = 1;; k++) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((k & 255u) == 0 && globaltimer() - t0 > limit_ns) return false;
  }
}

// tensor copies with an L2 eviction policy (l2_policy)
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, unsigned long long *bar, int c0,
                                            int c1, int c2, unsigned long long pol) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1, "
      "{%3, %4, %5}], [%2], %6;" ::"r"(smem_addr(dst)),
      "l"(map), "r"(smem_addr(bar)), "r"(c0), "r"(c1), "r"(c2), "l"(pol)
      : "memory");
}

__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, unsigned long long *bar, int c0,
                                            int c1, int c2, int c3, unsigned long long pol) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1, "
      "{%3, %4, %5, %6}], [%2], %7;" ::"r"(smem_addr(dst)),
      "l"(map), "r"(smem_addr(bar)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "l"(pol)
      : "memory");
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// L2 prefetches (no shared memory, no completion): rows of a tensor map, and a
// contiguous range (16-byte aligned start, size a multiple of 16)
__device__ __forceinline__ void tma_prefetch_rows(const CUtensorMap *map, int y, int z, bool four_d) {
  if (four_d)
    asm volatile("cp.async.bulk.prefetch.tensor.4d.L2.global.tile [%0, {%1, %2, %3, %4}];" ::"l"(map), "r"(0), "r"(0),
                 "r"(y), "r"(z)
                 : "memory");
  else
    asm volatile("cp.async.bulk.prefetch.tensor.3d.L2.global.tile [%0, {%1, %2, %3}];" ::"l"(map), "r"(0), "r"(y),
                 "r"(z)
                 : "memory");
}

__device__ __forceinline__ void bulk_prefetch_l2(const void *p, unsigned int bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

struct TmaMaps {
  CUtensorMap r_rows, r_row, p_rows, p_row;  // TY-row and one-row boxes of r and p_old
};

// Load rows [y, y + nrow) of plane z of one array into dst (row-major, nx
// floats per row).  4-D maps split x into 256-wide pieces (nx > 256).
__device__ __forceinline__ void load_rows(float *dst, const CUtensorMap *map, unsigned long long *bar, int y, int z,
                                          bool four_d, unsigned long long pol) {
  if (four_d) tma_load_4d(dst, map, bar, 0, 0, y, z, pol);
  else tma_load_3d(dst, map, bar, 0, y, z, pol);
}

}  // namespace

// NPT: float4 elements per thread per plane (TY * nx / 1024)
template <int NPT, bool MASK, bool ISO>
__global__ void __launch_bounds__(TNT) k1_tma(const GeoL G, const __grid_constant__ TmaMaps M,
                                              float *__restrict__ pnew, float *__restrict__ Ap,
                                              float *__restrict__ x, const uint8_t *__restrict__ mask,
                                              DevState *st, double *partials, int ty, int kz, int ns, int four_d,
                                              int l2hint) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ float s_dL[27], s_inv[27];
  __shared__ double s_red[TNT / 32];
  __shared__ unsigned long long s_full[8];
  pdl_sync();
  if (*(volatile int *)&st->done) return;
  const bool first = *(volatile int *)&st->first;
  const float beta = first ? 0.f : (float)(*(volatile double *)&st->beta);
  const bool lag = !first && *(volatile int *)&st->dlag;
  const float alpha = lag ? (float)(*(volatile double *)&st->alpha) : 0.f;
  const long long wl = *(volatile long long *)&st->wait_ns;
  const unsigned long long limit = wl > 0 ? (unsigned long long)wl : 1000000000ull;
  // test hook: CTA (0,0) leaves one plane's copies unissued, so that its wait
  // for them runs out and the solve ends with DONE_TIMEOUT
  const bool skip_one = *(volatile int *)&st->inject && blockIdx.x == 0 && blockIdx.y == 0;
  load_tabs<float>(G, s_dL, s_inv);
  // L2 policies: the mask, read by every search kernel, stays (evict_last);
  // p, Ap and x stream through (evict_first); r keeps the normal priority
  const unsigned long long pol_r = l2_policy(0), pol_stream = l2_policy(l2hint ? 1 : 0);
  const unsigned long long pol_mask = l2_policy(l2hint ? 2 : 0);

  const int tid = threadIdx.x, lane = tid & 31;
  const int nx = G.nx, ny = G.ny, nz = G.nz;
  const int nxv = nx >> 2;                 // float4 per row
  const int rows = ty + 2;                 // stage rows with the halo
  const int arr = rows * nx;               // floats per array per stage
  float *stage = reinterpret_cast<float *>(smem_raw);  // [ns][2][rows][nx]
  const int y0 = blockIdx.x * ty;
  const int z0 = blockIdx.y * kz, z1 = min(z0 + kz, nz);
  const int np = z1 - z0 + 2;              // planes z0-1 .. z1
  const unsigned int plane = (unsigned int)nx * (unsigned int)ny;
  const unsigned int tx_bytes = (unsigned int)((first ? 1 : 2) * arr * 4);
  const int ys = G.py ? (y0 - 1 + ny) % ny : y0 - 1;  // south halo row (-1: zero fill)
  const int yn = G.py ? (y0 + ty) % ny : y0 + ty;     // north halo row (ny: zero fill)

  if (tid == 0) {
    for (int s = 0; s < ns; s++) mbar_init(&s_full[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  auto issue = [&](int j) {  // thread 0: copies of plane z0-1+j into its stage
    if (skip_one && j == 2) return;
    const int s = j % ns;
    int zr = z0 - 1 + j;
    if (G.pz) zr = (zr + nz) % nz;  // else -1 / nz read the zero fill
    float *rs = stage + (size_t)s * 2 * arr;
    unsigned long long *bar = &s_full[s];
    mbar_expect_tx(bar, tx_bytes);
    load_rows(rs + nx, &M.r_rows, bar, y0, zr, four_d, pol_r);
    load_rows(rs, &M.r_row, bar, ys, zr, four_d, pol_r);
    load_rows(rs + (ty + 1) * nx, &M.r_row, bar, yn, zr, four_d, pol_r);
    if (!first) {
      float *ps = rs + arr;
      load_rows(ps + nx, &M.p_rows, bar, y0, zr, four_d, pol_stream);
      load_rows(ps, &M.p_row, bar, ys, zr, four_d, pol_stream);
      load_rows(ps + (ty + 1) * nx, &M.p_row, bar, yn, zr, four_d, pol_stream);
    }
  };

  bool bad = false;
  // p_new over a stage, in place of r
  auto prep = [&](int j) {
    const int s = j % ns;
    // after a wait has run out this thread waits no more: the copy unit is
    // behind, and the drain at the end waits for what is in flight
    if (!bad && !mbar_wait(&s_full[s], (unsigned int)(j / ns) & 1u, limit)) bad = true;
    float4 *rs = reinterpret_cast<float4 *>(stage + (size_t)s * 2 * arr);
    const float4 *ps = reinterpret_cast<const float4 *>(stage + (size_t)s * 2 * arr + arr);
    int zr = z0 - 1 + j;
    const int gz = halo_index(zr, nz, G.pz);
    const int wz = gz >= 0 ? 9 * wall_count(gz, nz, G.pz) : 0;
    const int nel = rows * nxv;
    if (G.px && G.py && wz == 0) {
      for (int e = tid; e < nel; e += TNT) {
        float4 v = rs[e];
        if (!first) {
          const float4 q = ps[e];
          v.x = fmaf(beta, q.x, v.x);
          v.y = fmaf(beta, q.y, v.y);
          v.z = fmaf(beta, q.z, v.z);
          v.w = fmaf(beta, q.w, v.w);
        }
        rs[e] = v;
      }
    } else {
      for (int e = tid; e < nel; e += TNT) {
        const int row = e / nxv, c4 = e - row * nxv;
        const int gy = halo_index(y0 - 1 + row, ny, G.py);
        const int wy = gy >= 0 ? 3 * wall_count(gy, ny, G.py) : 0;
        const int xb = 4 * c4;
        float4 v = rs[e];
        float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
        if (!first) q = ps[e];
        float *vv = reinterpret_cast<float *>(&v);
        const float *qq = reinterpret_cast<const float *>(&q);
#pragma unroll
        for (int i = 0; i < 4; i++) {
          const int cls = wall_count(xb + i, nx, G.px) + wy + wz;
          const float zv = cls ? vv[i] * s_inv[cls] : vv[i];
          vv[i] = first ? zv : fmaf(beta, qq[i], zv);
        }
        rs[e] = v;
      }
    }
  };

  // own elements of this thread: float4 tid + k * TNT of the slab's TY x nxv
  int orow[NPT], oc4[NPT];
#pragma unroll
  for (int k = 0; k < NPT; k++) {
    const int e = tid + k * TNT;
    orow[k] = e / nxv;
    oc4[k] = e - orow[k] * nxv;
  }
  // own-cell mask and x of the next plane, loaded one plane ahead
  // two register sets, alternating by plane: the loads of plane j + 2 are in
  // flight while plane j is computed
  uchar4 mkA[NPT], mkB[NPT];
  float4 xvA[NPT], xvB[NPT];
  auto fetch = [&](int zc, uchar4 (&mk)[NPT], float4 (&xv)[NPT]) {
#pragma unroll
    for (int k = 0; k < NPT; k++) {
      const int row = orow[k], c4 = oc4[k];
      const unsigned int c = plane * (unsigned int)zc + (unsigned int)nx * (unsigned int)(y0 + row) + 4u * c4;
      if (MASK) {
        const unsigned int m = ld_u32_pol(mask + c, pol_mask);
        mk[k] = make_uchar4(m & 0xffu, (m >> 8) & 0xffu, (m >> 16) & 0xffu, m >> 24);
      }
      if (lag) xv[k] = ld4_pol(reinterpret_cast<const float4 *>(x + c), pol_stream);
    }
  };

  float acc = 0.f;
  auto stencil = [&](int j, const uchar4 (&mk)[NPT], const float4 (&xv)[NPT]) {
    const int zc = z0 - 1 + j;
    const float *cs = stage + (size_t)(j % ns) * 2 * arr;           // p_new, plane z
    const float *ts = stage + (size_t)((j + 1) % ns) * 2 * arr;     // plane z+1
    const float *bs = stage + (size_t)((j - 1 + ns) % ns) * 2 * arr;  // plane z-1
    const float *po = cs + arr;                                      // p_old, plane z
    const int wz = 9 * wall_count(zc, nz, G.pz);
    const bool interior = G.px && G.py && wz == 0;
#pragma unroll
    for (int k = 0; k < NPT; k++) {
      const int row = orow[k], c4 = oc4[k];
      const int off = (row + 1) * nx + 4 * c4;
      const float4 c = *reinterpret_cast<const float4 *>(cs + off);
      const float4 n = *reinterpret_cast<const float4 *>(cs + off + nx);
      const float4 s = *reinterpret_cast<const float4 *>(cs + off - nx);
      const float4 t = *reinterpret_cast<const float4 *>(ts + off);
      const float4 b = *reinterpret_cast<const float4 *>(bs + off);
      // x neighbours: the adjacent lanes hold the adjacent float4 of the row
      float w = __shfl_up_sync(0xffffffffu, c.w, 1);
      float ea = __shfl_down_sync(0xffffffffu, c.x, 1);
      if (lane == 0 || c4 == 0) {
        const int xw = 4 * c4 - 1;
        w = xw >= 0 ? cs[off - 1] : (G.px ? cs[(row + 1) * nx + nx - 1] : 0.f);
      }
      if (lane == 31 || c4 == nxv - 1) {
        const int xe = 4 * c4 + 4;
        ea = xe < nx ? cs[off + 4] : (G.px ? cs[(row + 1) * nx] : 0.f);
      }
      float a0, a1, a2, a3;
      if (interior) {
        a0 = apply_L<float, ISO>(G, s_dL, 0, c.x, c.y, w, n.x, s.x, t.x, b.x);
        a1 = apply_L<float, ISO>(G, s_dL, 0, c.y, c.z, c.x, n.y, s.y, t.y, b.y);
        a2 = apply_L<float, ISO>(G, s_dL, 0, c.z, c.w, c.y, n.z, s.z, t.z, b.z);
        a3 = apply_L<float, ISO>(G, s_dL, 0, c.w, ea, c.z, n.w, s.w, t.w, b.w);
      } else {
        const int wy = 3 * wall_count(y0 + row, ny, G.py) + wz;
        const int xb = 4 * c4;
        a0 = apply_L<float, ISO>(G, s_dL, wall_count(xb, nx, G.px) + wy, c.x, c.y, w, n.x, s.x, t.x, b.x);
        a1 = apply_L<float, ISO>(G, s_dL, wall_count(xb + 1, nx, G.px) + wy, c.y, c.z, c.x, n.y, s.y, t.y, b.y);
        a2 = apply_L<float, ISO>(G, s_dL, wall_count(xb + 2, nx, G.px) + wy, c.z, c.w, c.y, n.z, s.z, t.z, b.z);
        a3 = apply_L<float, ISO>(G, s_dL, wall_count(xb + 3, nx, G.px) + wy, c.w, ea, c.z, n.w, s.w, t.w, b.w);
      }
      if (MASK) {
        if (mk[k].x) a0 = 0.f;
        if (mk[k].y) a1 = 0.f;
        if (mk[k].z) a2 = 0.f;
        if (mk[k].w) a3 = 0.f;
      }
      acc = fmaf(c.x, a0, acc);
      acc = fmaf(c.y, a1, acc);
      acc = fmaf(c.z, a2, acc);
      acc = fmaf(c.w, a3, acc);
      const unsigned int g = plane * (unsigned int)zc + (unsigned int)nx * (unsigned int)(y0 + row) + 4u * c4;
      st4_pol(reinterpret_cast<float4 *>(Ap + g), make_float4(a0, a1, a2, a3), pol_stream);
      st4_pol(reinterpret_cast<float4 *>(pnew + g), c, pol_stream);
      if (lag) {
        const float4 q = *reinterpret_cast<const float4 *>(po + off);
        float4 xo = xv[k];
        xo.x = fmaf(alpha, q.x, xo.x);
        xo.y = fmaf(alpha, q.y, xo.y);
        xo.z = fmaf(alpha, q.z, xo.z);
        xo.w = fmaf(alpha, q.w, xo.w);
        st4_pol(reinterpret_cast<float4 *>(x + g), xo, pol_stream);
      }
    }
  };

  if (tid == 0) {
    const int pre = min(ns, np);
    for (int j = 0; j < pre; j++) issue(j);
  }
  const int nj = z1 - z0;  // planes of this CTA: j = 1 .. nj
  fetch(z0, mkA, xvA);
  if (nj >= 2) fetch(z0 + 1, mkB, xvB);
  prep(0);
  prep(1);
  auto step = [&](int j, uchar4 (&mk)[NPT], float4 (&xv)[NPT]) {
    prep(j + 1);
    fence_proxy_async();  // this thread's stage writes before later tensor copies
    __syncthreads();
    if (tid == 0 && j >= 2 && j - 2 + ns < np) issue(j - 2 + ns);
    // the mask / x registers of plane j are consumed here, then refilled with plane j + 2
    stencil(j, mk, xv);
    if (j + 2 <= nj) fetch(z0 + j + 1, mk, xv);
  };
  for (int j = 1; j <= nj; j += 2) {
    step(j, mkA, xvA);
    if (j + 1 <= nj) step(j + 1, mkB, xvB);
  }

  if (__syncthreads_or(bad)) {
    // drain: every stage's last issued copy, with bounded waits
    if (tid == 0) {
      // the last copy into every stage, with ten times the bound: the CTA must
      // not exit while a copy into its shared memory is still in flight
      for (int j = max(0, np - ns); j < np; j++)
        mbar_wait(&s_full[j % ns], (unsigned int)(j / ns) & 1u, 10ull * limit);
      atomicExch(&st->done, (int)DONE_TIMEOUT);
    }
    return;
  }
  double v[1] = {(double)acc}, tot[1];
  const unsigned int nb = gridDim.x * gridDim.y;
  const unsigned int bid = blockIdx.x + gridDim.x * blockIdx.y;
  if (last_cta_reduce<1>(v, partials, st, nb, bid, s_red, tot) && tid == 0) {
    st->pAp = tot[0];
    st->alpha = st->rz / tot[0];
    st->first = 0;
    st->dlag = 1;
    decide_replacement(st);
  }
}

// ------------------------------------------------------- fused iteration --
// One kernel per PCG iteration (FP32).  Iteration q's search kernel also does
// the update of iteration q - 1, which the two-kernel form leaves to a kernel
// of its own: on every staged row (the halo rows too)
//   r_{q-1} = r_{q-2} - alpha_{q-1} Ap_{q-1}      (when a step is pending)
//   p_q = z_{q-1} + beta_q p_{q-1},   z = r / dL on wall classes
// then, one plane behind, Ap_q = L p_q on the slab's own cells, the stores of
// r_{q-1}, p_q, Ap_q, x += alpha_{q-1} p_{q-1}, and five partial sums:
// (p_q, Ap_q), (r,z) and (r,r) of r_{q-1}, (Ap_q, z_{q-1}), (Ap_q, Ap_q / dL).
// beta_q cannot wait for (r_{q-1}, z_{q-1}), so it comes from the expansion
//   (r_{q-1}, z_{q-1}) = (r_{q-2}, z_{q-2}) - 2 alpha (Ap, z) + alpha^2 (Ap, Ap / dL)
// evaluated in FP64 at the end of the previous kernel; the exact value, summed
// here, restarts the expansion every iteration (alpha_q uses it), so no error
// accumulates.  The exact (r,z), (r,r) of r_{q-1} end iteration q - 1 (the
// convergence test runs one kernel late, on a settled x, r pair).  Traffic:
// r, Ap, p_old, x, mask in (17 B/cell) and r, p, Ap, x out (16 B/cell), in one
// kernel, against 37 B/cell in two.  r and Ap are double-buffered: a CTA's
// halo rows are another CTA's own cells.
struct FusedMaps {
  CUtensorMap r_rows, r_row, a_rows, a_row, p_rows, p_row;
};

template <int NPT, bool MASK, bool ISO>
__global__ void __launch_bounds__(TNT) k1_fused(const GeoL G, const __grid_constant__ FusedMaps M,
                                                float *__restrict__ rout, float *__restrict__ pnew,
                                                float *__restrict__ Apout, float *__restrict__ x,
                                                const uint8_t *__restrict__ mask, DevState *st, double *partials,
                                                int ty, int kz, int ns, int four_d, int l2hint, int pf) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ float s_dL[27], s_inv[27];
  __shared__ double s_red[5 * TNT / 32];
  __shared__ unsigned long long s_full[8];
  pdl_sync();
  if (*(volatile int *)&st->done) return;
  const bool first = *(volatile int *)&st->first;
  const float beta = first ? 0.f : (float)(*(volatile double *)&st->beta);
  const bool lag = !first && *(volatile int *)&st->dlag;  // a step is pending: r and x take alpha of it
  const float alpha = lag ? (float)(*(volatile double *)&st->alpha) : 0.f;
  const long long wl = *(volatile long long *)&st->wait_ns;
  const unsigned long long limit = wl > 0 ? (unsigned long long)wl : 1000000000ull;
  const bool skip_one = *(volatile int *)&st->inject && blockIdx.x == 0 && blockIdx.y == 0;
  load_tabs<float>(G, s_dL, s_inv);
  const unsigned long long pol_n = l2_policy(0), pol_stream = l2_policy(l2hint ? 1 : 0);
  const unsigned long long pol_mask = l2_policy(l2hint ? 2 : 0);

  const int tid = threadIdx.x, lane = tid & 31;
  const int nx = G.nx, ny = G.ny, nz = G.nz;
  const int nxv = nx >> 2;
  const int rows = ty + 2;
  const int arr = rows * nx;
  float *stage = reinterpret_cast<float *>(smem_raw);  // [ns][3][rows][nx]: r, Ap_old -> p_new, p_old
  const int y0 = blockIdx.x * ty;
  const int z0 = blockIdx.y * kz, z1 = min(z0 + kz, nz);
  const int np = z1 - z0 + 2;
  const unsigned int plane = (unsigned int)nx * (unsigned int)ny;
  const unsigned int tx_bytes = (unsigned int)((1 + (lag ? 1 : 0) + (first ? 0 : 1)) * arr * 4);
  const int ys = G.py ? (y0 - 1 + ny) % ny : y0 - 1;
  const int yn = G.py ? (y0 + ty) % ny : y0 + ty;

  if (tid == 0) {
    for (int s = 0; s < ns; s++) mbar_init(&s_full[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  auto issue = [&](int j) {
    if (skip_one && j == 2) return;
    const int s = j % ns;
    int zr = z0 - 1 + j;
    if (G.pz) zr = (zr + nz) % nz;
    float *rs = stage + (size_t)s * 3 * arr;
    unsigned long long *bar = &s_full[s];
    mbar_expect_tx(bar, tx_bytes);
    load_rows(rs + nx, &M.r_rows, bar, y0, zr, four_d, pol_n);
    load_rows(rs, &M.r_row, bar, ys, zr, four_d, pol_n);
    load_rows(rs + (ty + 1) * nx, &M.r_row, bar, yn, zr, four_d, pol_n);
    if (lag) {
      float *as = rs + arr;
      load_rows(as + nx, &M.a_rows, bar, y0, zr, four_d, pol_n);
      load_rows(as, &M.a_row, bar, ys, zr, four_d, pol_n);
      load_rows(as + (ty + 1) * nx, &M.a_row, bar, yn, zr, four_d, pol_n);
    }
    if (!first) {
      float *ps = rs + 2 * arr;
      load_rows(ps + nx, &M.p_rows, bar, y0, zr, four_d, pol_stream);
      load_rows(ps, &M.p_row, bar, ys, zr, four_d, pol_stream);
      load_rows(ps + (ty + 1) * nx, &M.p_row, bar, yn, zr, four_d, pol_stream);
    }
    // L2 prefetch pf planes further: the staged arrays' slab rows and the
    // own rows of x and the mask (contiguous: whole rows)
    const int zp = z0 - 1 + j + pf;
    if (pf > 0 && zp >= 0 && zp < nz && j + pf < np) {
      tma_prefetch_rows(&M.r_rows, y0, zp, four_d);
      if (lag) tma_prefetch_rows(&M.a_rows, y0, zp, four_d);
      if (!first) tma_prefetch_rows(&M.p_rows, y0, zp, four_d);
      const size_t c = (size_t)plane * zp + (size_t)nx * y0;
      if (lag) bulk_prefetch_l2(x + c, (unsigned int)(ty * nx * 4));
      if (MASK) bulk_prefetch_l2(mask + c, (unsigned int)(ty * nx));
    }
  };

  bool bad = false;
  // over a stage: r -= alpha Ap_old in place, p_new into the Ap_old slot
  auto prep = [&](int j) {
    const int s = j % ns;
    // after a wait has run out this thread waits no more: the copy unit is
    // behind, and the drain at the end waits for what is in flight
    if (!bad && !mbar_wait(&s_full[s], (unsigned int)(j / ns) & 1u, limit)) bad = true;
    float4 *rs = reinterpret_cast<float4 *>(stage + (size_t)s * 3 * arr);
    float4 *as = rs + arr / 4;
    const float4 *ps = rs + 2 * (arr / 4);
    const int zr = z0 - 1 + j;
    const int gz = halo_index(zr, nz, G.pz);
    const int wz = gz >= 0 ? 9 * wall_count(gz, nz, G.pz) : 0;
    const int nel = rows * nxv;
    if (G.px && G.py && wz == 0) {
      for (int e = tid; e < nel; e += TNT) {
        float4 r = rs[e];
        if (lag) {
          const float4 a = as[e];
          r.x = fmaf(-alpha, a.x, r.x);
          r.y = fmaf(-alpha, a.y, r.y);
          r.z = fmaf(-alpha, a.z, r.z);
          r.w = fmaf(-alpha, a.w, r.w);
          rs[e] = r;
        }
        float4 p = r;
        if (!first) {
          const float4 q = ps[e];
          p.x = fmaf(beta, q.x, r.x);
          p.y = fmaf(beta, q.y, r.y);
          p.z = fmaf(beta, q.z, r.z);
          p.w = fmaf(beta, q.w, r.w);
        }
        as[e] = p;
      }
    } else {
      for (int e = tid; e < nel; e += TNT) {
        const int row = e / nxv, c4 = e - row * nxv;
        const int gy = halo_index(y0 - 1 + row, ny, G.py);
        const int wy = gy >= 0 ? 3 * wall_count(gy, ny, G.py) : 0;
        const int xb = 4 * c4;
        float4 r = rs[e];
        if (lag) {
          const float4 a = as[e];
          r.x = fmaf(-alpha, a.x, r.x);
          r.y = fmaf(-alpha, a.y, r.y);
          r.z = fmaf(-alpha, a.z, r.z);
          r.w = fmaf(-alpha, a.w, r.w);
          rs[e] = r;
        }
        float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
        if (!first) q = ps[e];
        float4 p;
        const float *rr_ = reinterpret_cast<const float *>(&r);
        const float *qq = reinterpret_cast<const float *>(&q);
        float *pp = reinterpret_cast<float *>(&p);
#pragma unroll
        for (int i = 0; i < 4; i++) {
          const int cls = wall_count(xb + i, nx, G.px) + wy + wz;
          const float zv = cls ? rr_[i] * s_inv[cls] : rr_[i];
          pp[i] = first ? zv : fmaf(beta, qq[i], zv);
        }
        as[e] = p;
      }
    }
  };

  int orow[NPT], oc4[NPT];
#pragma unroll
  for (int k = 0; k < NPT; k++) {
    const int e = tid + k * TNT;
    orow[k] = e / nxv;
    oc4[k] = e - orow[k] * nxv;
  }
  uchar4 mkA[NPT], mkB[NPT];
  float4 xvA[NPT], xvB[NPT];
  auto fetch = [&](int zc, uchar4 (&mk)[NPT], float4 (&xv)[NPT]) {
#pragma unroll
    for (int k = 0; k < NPT; k++) {
      const unsigned int c = plane * (unsigned int)zc + (unsigned int)nx * (unsigned int)(y0 + orow[k]) + 4u * oc4[k];
      if (MASK) {
        const unsigned int m = ld_u32_pol(mask + c, pol_mask);
        mk[k] = make_uchar4(m & 0xffu, (m >> 8) & 0xffu, (m >> 16) & 0xffu, m >> 24);
      }
      if (lag) xv[k] = ld4_pol(reinterpret_cast<const float4 *>(x + c), pol_stream);
    }
  };

  // partial sums: (p,Ap), (r,r), wall part of (r,z) - (r,r), (Ap,z), (Ap,Ap/dL)
  float s_pap = 0.f, s_rr = 0.f, s_corr = 0.f, s_c1 = 0.f, s_c2 = 0.f;
  auto stencil = [&](int j, const uchar4 (&mk)[NPT], const float4 (&xv)[NPT]) {
    const int zc = z0 - 1 + j;
    const float *cr = stage + (size_t)(j % ns) * 3 * arr;      // r_new, plane z
    const float *cs = cr + arr;                                 // p_new, plane z
    const float *ts = stage + (size_t)((j + 1) % ns) * 3 * arr + arr;
    const float *bs = stage + (size_t)((j - 1 + ns) % ns) * 3 * arr + arr;
    const float *po = cr + 2 * arr;                             // p_old, plane z
    const int wz = 9 * wall_count(zc, nz, G.pz);
    const bool interior = G.px && G.py && wz == 0;
#pragma unroll
    for (int k = 0; k < NPT; k++) {
      const int row = orow[k], c4 = oc4[k];
      const int off = (row + 1) * nx + 4 * c4;
      const float4 c = *reinterpret_cast<const float4 *>(cs + off);
      const float4 n = *reinterpret_cast<const float4 *>(cs + off + nx);
      const float4 s = *reinterpret_cast<const float4 *>(cs + off - nx);
      const float4 t = *reinterpret_cast<const float4 *>(ts + off);
      const float4 b = *reinterpret_cast<const float4 *>(bs + off);
      float w = __shfl_up_sync(0xffffffffu, c.w, 1);
      float ea = __shfl_down_sync(0xffffffffu, c.x, 1);
      if (lane == 0 || c4 == 0) {
        const int xw = 4 * c4 - 1;
        w = xw >= 0 ? cs[off - 1] : (G.px ? cs[(row + 1) * nx + nx - 1] : 0.f);
      }
      if (lane == 31 || c4 == nxv - 1) {
        const int xe = 4 * c4 + 4;
        ea = xe < nx ? cs[off + 4] : (G.px ? cs[(row + 1) * nx] : 0.f);
      }
      float a[4];
      int cls[4] = {0, 0, 0, 0};
      if (interior) {
        a[0] = apply_L<float, ISO>(G, s_dL, 0, c.x, c.y, w, n.x, s.x, t.x, b.x);
        a[1] = apply_L<float, ISO>(G, s_dL, 0, c.y, c.z, c.x, n.y, s.y, t.y, b.y);
        a[2] = apply_L<float, ISO>(G, s_dL, 0, c.z, c.w, c.y, n.z, s.z, t.z, b.z);
        a[3] = apply_L<float, ISO>(G, s_dL, 0, c.w, ea, c.z, n.w, s.w, t.w, b.w);
      } else {
        const int wy = 3 * wall_count(y0 + row, ny, G.py) + wz;
        const int xb = 4 * c4;
#pragma unroll
        for (int i = 0; i < 4; i++) cls[i] = wall_count(xb + i, nx, G.px) + wy;
        a[0] = apply_L<float, ISO>(G, s_dL, cls[0], c.x, c.y, w, n.x, s.x, t.x, b.x);
        a[1] = apply_L<float, ISO>(G, s_dL, cls[1], c.y, c.z, c.x, n.y, s.y, t.y, b.y);
        a[2] = apply_L<float, ISO>(G, s_dL, cls[2], c.z, c.w, c.y, n.z, s.z, t.z, b.z);
        a[3] = apply_L<float, ISO>(G, s_dL, cls[3], c.w, ea, c.z, n.w, s.w, t.w, b.w);
      }
      if (MASK) {
        if (mk[k].x) a[0] = 0.f;
        if (mk[k].y) a[1] = 0.f;
        if (mk[k].z) a[2] = 0.f;
        if (mk[k].w) a[3] = 0.f;
      }
      const float4 r = *reinterpret_cast<const float4 *>(cr + off);
      const float rv[4] = {r.x, r.y, r.z, r.w};
      const float pv[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
      for (int i = 0; i < 4; i++) {
        s_pap = fmaf(pv[i], a[i], s_pap);
        s_rr = fmaf(rv[i], rv[i], s_rr);
        if (interior) {
          s_c1 = fmaf(a[i], rv[i], s_c1);
          s_c2 = fmaf(a[i], a[i], s_c2);
        } else {
          const float iv = cls[i] ? s_inv[cls[i]] : 1.f;
          s_corr = fmaf((iv - 1.f) * rv[i], rv[i], s_corr);
          s_c1 = fmaf(a[i], rv[i] * iv, s_c1);
          s_c2 = fmaf(a[i] * iv, a[i], s_c2);
        }
      }
      const unsigned int g = plane * (unsigned int)zc + (unsigned int)nx * (unsigned int)(y0 + row) + 4u * c4;
      st4_pol(reinterpret_cast<float4 *>(Apout + g), make_float4(a[0], a[1], a[2], a[3]), pol_n);
      st4_pol(reinterpret_cast<float4 *>(pnew + g), c, pol_stream);
      st4_pol(reinterpret_cast<float4 *>(rout + g), r, pol_n);
      if (lag) {
        const float4 q = *reinterpret_cast<const float4 *>(po + off);
        float4 xo = xv[k];
        xo.x = fmaf(alpha, q.x, xo.x);
        xo.y = fmaf(alpha, q.y, xo.y);
        xo.z = fmaf(alpha, q.z, xo.z);
        xo.w = fmaf(alpha, q.w, xo.w);
        st4_pol(reinterpret_cast<float4 *>(x + g), xo, pol_stream);
      }
    }
  };

  if (tid == 0) {
    const int pre = min(ns, np);
    for (int j = 0; j < pre; j++) issue(j);
  }
  const int nj = z1 - z0;
  fetch(z0, mkA, xvA);
  if (nj >= 2) fetch(z0 + 1, mkB, xvB);
  prep(0);
  prep(1);
  auto step = [&](int j, uchar4 (&mk)[NPT], float4 (&xv)[NPT]) {
    prep(j + 1);
    fence_proxy_async();
    __syncthreads();
    if (tid == 0 && j >= 2 && j - 2 + ns < np) issue(j - 2 + ns);
    stencil(j, mk, xv);
    if (j + 2 <= nj) fetch(z0 + j + 1, mk, xv);
  };
  for (int j = 1; j <= nj; j += 2) {
    step(j, mkA, xvA);
    if (j + 1 <= nj) step(j + 1, mkB, xvB);
  }

  if (__syncthreads_or(bad)) {
    if (tid == 0) {
      // the last copy into every stage, with ten times the bound: the CTA must
      // not exit while a copy into its shared memory is still in flight
      for (int j = max(0, np - ns); j < np; j++)
        mbar_wait(&s_full[j % ns], (unsigned int)(j / ns) & 1u, 10ull * limit);
      atomicExch(&st->done, (int)DONE_TIMEOUT);
    }
    return;
  }
  double v[5] = {(double)s_pap, (double)s_rr + (double)s_corr, (double)s_rr, (double)s_c1, (double)s_c2}, tot[5];
  const unsigned int nb = gridDim.x * gridDim.y;
  const unsigned int bid = blockIdx.x + gridDim.x * blockIdx.y;
  if (last_cta_reduce<5>(v, partials, st, nb, bid, s_red, tot) && tid == 0) {
    st->fq += 1;
    if (lag) finish_deferred(st, tot[1], tot[2]);  // r_{q-1} ends iteration q - 1
    st->dlag = 0;  // the pending step is in x and r now
    // the step of this kernel's direction stays pending (also when the
    // recursive residual has met TRUE_REL: the confirmation folds it in)
    if (st->done == RUNNING || st->done == DONE_PENDING) {
      const double rz = st->rz, pap = tot[0];
      const double a = rz / pap;
      st->pAp = pap;
      st->alpha = a;
      st->beta = (rz - 2.0 * a * tot[3] + a * a * tot[4]) / rz;
      st->first = 0;
      st->dlag = 1;
      decide_replacement(st);
    }
  }
}

// ------------------------------------------------ fused iteration, WS --
// The fused iteration with its copies issued by a warp of their own.  Warps
// 0-7 (256 threads) prep and stencil as k1_fused does; warp 8 is the producer:
// its first lane issues each plane's tensor copies as soon as the stage that
// plane goes to is released, instead of after the CTA barrier of a plane.
// Stages are handed back through empty mbarriers, one arrival per compute
// warp after its last read.  The stencil of plane j takes its lower z
// neighbour from the centre value the same thread read for plane j - 1 (a
// register), so a stage is free once the stencil of its own plane is done:
// with ns stages, plane j + ns is in flight from the end of plane j's stencil,
// ns - 2 planes ahead of the prep that waits for it.  The compute warps still
// meet at a barrier of their own once per plane, between the prep of plane
// j + 1 (rows other threads read) and the stencil of plane j.
// Arithmetic, order of the partial sums and the stored values are those of
// k1_fused, so the two kernels give identical results.
// A wait that runs out marks the CTA (s_bad); later waits then return at once,
// the producer stops issuing, and at the end the producer waits, with a bound
// of 10 x the wait limit, for the last copy into every stage before the CTA
// reports DONE_TIMEOUT and returns, so no copy is in flight when it exits.
constexpr int WS_WARPS = TNT / 32;       // compute warps
constexpr int WS_THREADS = TNT + 32;     // plus the producer warp

__device__ __forceinline__ void mbar_arrive(unsigned long long *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// barrier of the compute warps only (named barrier 1, 256 threads)
__device__ __forceinline__ void compute_sync() { asm volatile("bar.sync 1, %0;" ::"n"(TNT) : "memory"); }

template <int NPT, bool MASK, bool ISO>
__global__ void __launch_bounds__(WS_THREADS, 3) k1_fused_ws(const GeoL G, const __grid_constant__ FusedMaps M,
                                                          float *__restrict__ rout, float *__restrict__ pnew,
                                                          float *__restrict__ Apout, float *__restrict__ x,
                                                          const uint8_t *__restrict__ mask, DevState *st,
                                                          double *partials, int ty, int kz, int ns, int four_d,
                                                          int l2hint, int pf) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ float s_dL[27], s_inv[27];
  __shared__ double s_red[5 * WS_THREADS / 32];
  __shared__ unsigned long long s_full[8], s_empty[8];
  __shared__ int s_bad, s_issued, s_done;
  pdl_sync();
  // one read of the state for the whole CTA, so that it returns as a whole
  if (threadIdx.x == 0) s_done = *(volatile int *)&st->done;
  __syncthreads();
  if (s_done) return;
  const bool first = *(volatile int *)&st->first;
  const float beta = first ? 0.f : (float)(*(volatile double *)&st->beta);
  const bool lag = !first && *(volatile int *)&st->dlag;
  const float alpha = lag ? (float)(*(volatile double *)&st->alpha) : 0.f;
  const long long wl = *(volatile long long *)&st->wait_ns;
  const unsigned long long limit = wl > 0 ? (unsigned long long)wl : 1000000000ull;
  const bool skip_one = *(volatile int *)&st->inject && blockIdx.x == 0 && blockIdx.y == 0;
  load_tabs<float>(G, s_dL, s_inv);
  const unsigned long long pol_n = l2_policy(0), pol_stream = l2_policy(l2hint ? 1 : 0);
  const unsigned long long pol_mask = l2_policy(l2hint ? 2 : 0);

  const int tid = threadIdx.x, lane = tid & 31;
  const int nx = G.nx, ny = G.ny, nz = G.nz;
  const int nxv = nx >> 2;
  const int rows = ty + 2;
  const int arr = rows * nx;
  float *stage = reinterpret_cast<float *>(smem_raw);  // [ns][3][rows][nx]: r, Ap_old -> p_new, p_old
  const int y0 = blockIdx.x * ty;
  const int z0 = blockIdx.y * kz, z1 = min(z0 + kz, nz);
  const int np = z1 - z0 + 2;
  const int nj = z1 - z0;
  const unsigned int plane = (unsigned int)nx * (unsigned int)ny;
  const unsigned int tx_bytes = (unsigned int)((1 + (lag ? 1 : 0) + (first ? 0 : 1)) * arr * 4);
  const int ys = G.py ? (y0 - 1 + ny) % ny : y0 - 1;
  const int yn = G.py ? (y0 + ty) % ny : y0 + ty;

  if (tid == 0) {
    for (int q = 0; q < ns; q++) {
      mbar_init(&s_full[q], 1);
      mbar_init(&s_empty[q], WS_WARPS);
    }
    s_bad = 0;
    s_issued = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  // a bounded wait that gives up at once in a CTA already marked
  auto wait_phase = [&](unsigned long long *bar, unsigned int parity, unsigned long long lim) -> bool {
    if (*(volatile int *)&s_bad) return false;
    if (mbar_wait(bar, parity, lim)) return true;
    *(volatile int *)&s_bad = 1;
    return false;
  };

  bool bad = false;
  // partial sums: (p,Ap), (r,r), wall part of (r,z) - (r,r), (Ap,z), (Ap,Ap/dL);
  // zero in the producer warp
  float s_pap = 0.f, s_rr = 0.f, s_corr = 0.f, s_c1 = 0.f, s_c2 = 0.f;
  if (tid >= TNT) {
    // ---- producer warp: lane 0 issues, the warp moves through the planes together
    int issued = 0;
    for (int j = 0; j < np; j++) {
      const int q = j % ns;
      // lane 0 decides, the warp follows (its lanes stay converged)
      int ok = 1;
      if (lane == 0) {
        if (j >= ns) ok = wait_phase(&s_empty[q], (unsigned int)(j / ns - 1) & 1u, limit);
        ok = ok && !*(volatile int *)&s_bad;
      }
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) {
        bad = true;
        break;
      }
      if (lane == 0 && !(skip_one && j == 2)) {
        int zr = z0 - 1 + j;
        if (G.pz) zr = (zr + nz) % nz;
        float *rs = stage + (size_t)q * 3 * arr;
        unsigned long long *bar = &s_full[q];
        mbar_expect_tx(bar, tx_bytes);
        load_rows(rs + nx, &M.r_rows, bar, y0, zr, four_d, pol_n);
        load_rows(rs, &M.r_row, bar, ys, zr, four_d, pol_n);
        load_rows(rs + (ty + 1) * nx, &M.r_row, bar, yn, zr, four_d, pol_n);
        if (lag) {
          float *as = rs + arr;
          load_rows(as + nx, &M.a_rows, bar, y0, zr, four_d, pol_n);
          load_rows(as, &M.a_row, bar, ys, zr, four_d, pol_n);
          load_rows(as + (ty + 1) * nx, &M.a_row, bar, yn, zr, four_d, pol_n);
        }
        if (!first) {
          float *ps = rs + 2 * arr;
          load_rows(ps + nx, &M.p_rows, bar, y0, zr, four_d, pol_stream);
          load_rows(ps, &M.p_row, bar, ys, zr, four_d, pol_stream);
          load_rows(ps + (ty + 1) * nx, &M.p_row, bar, yn, zr, four_d, pol_stream);
        }
        const int zp = z0 - 1 + j + pf;
        if (pf > 0 && zp >= 0 && zp < nz && j + pf < np) {
          tma_prefetch_rows(&M.r_rows, y0, zp, four_d);
          if (lag) tma_prefetch_rows(&M.a_rows, y0, zp, four_d);
          if (!first) tma_prefetch_rows(&M.p_rows, y0, zp, four_d);
          const size_t c = (size_t)plane * zp + (size_t)nx * y0;
          if (lag) bulk_prefetch_l2(x + c, (unsigned int)(ty * nx * 4));
          if (MASK) bulk_prefetch_l2(mask + c, (unsigned int)(ty * nx));
        }
      }
      issued = j + 1;
      __syncwarp();
    }
    if (lane == 0) s_issued = issued;
  } else {
    // ---- compute warps
    auto prep = [&](int j) {
      const int q = j % ns;
      if (!wait_phase(&s_full[q], (unsigned int)(j / ns) & 1u, limit)) bad = true;
      float4 *rs = reinterpret_cast<float4 *>(stage + (size_t)q * 3 * arr);
      float4 *as = rs + arr / 4;
      const float4 *ps = rs + 2 * (arr / 4);
      const int zr = z0 - 1 + j;
      const int gz = halo_index(zr, nz, G.pz);
      const int wz = gz >= 0 ? 9 * wall_count(gz, nz, G.pz) : 0;
      const int nel = rows * nxv;
      if (G.px && G.py && wz == 0) {
        for (int e = tid; e < nel; e += TNT) {
          float4 r = rs[e];
          if (lag) {
            const float4 a = as[e];
            r.x = fmaf(-alpha, a.x, r.x);
            r.y = fmaf(-alpha, a.y, r.y);
            r.z = fmaf(-alpha, a.z, r.z);
            r.w = fmaf(-alpha, a.w, r.w);
            rs[e] = r;
          }
          float4 p = r;
          if (!first) {
            const float4 o = ps[e];
            p.x = fmaf(beta, o.x, r.x);
            p.y = fmaf(beta, o.y, r.y);
            p.z = fmaf(beta, o.z, r.z);
            p.w = fmaf(beta, o.w, r.w);
          }
          as[e] = p;
        }
      } else {
        for (int e = tid; e < nel; e += TNT) {
          const int row = e / nxv, c4 = e - row * nxv;
          const int gy = halo_index(y0 - 1 + row, ny, G.py);
          const int wy = gy >= 0 ? 3 * wall_count(gy, ny, G.py) : 0;
          const int xb = 4 * c4;
          float4 r = rs[e];
          if (lag) {
            const float4 a = as[e];
            r.x = fmaf(-alpha, a.x, r.x);
            r.y = fmaf(-alpha, a.y, r.y);
            r.z = fmaf(-alpha, a.z, r.z);
            r.w = fmaf(-alpha, a.w, r.w);
            rs[e] = r;
          }
          float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
          if (!first) o = ps[e];
          float4 p;
          const float *rr_ = reinterpret_cast<const float *>(&r);
          const float *oo = reinterpret_cast<const float *>(&o);
          float *pp = reinterpret_cast<float *>(&p);
#pragma unroll
          for (int i = 0; i < 4; i++) {
            const int cls = wall_count(xb + i, nx, G.px) + wy + wz;
            const float zv = cls ? rr_[i] * s_inv[cls] : rr_[i];
            pp[i] = first ? zv : fmaf(beta, oo[i], zv);
          }
          as[e] = p;
        }
      }
    };

    int orow[NPT], oc4[NPT];
#pragma unroll
    for (int k = 0; k < NPT; k++) {
      const int e = tid + k * TNT;
      orow[k] = e / nxv;
      oc4[k] = e - orow[k] * nxv;
    }
    uchar4 mkA[NPT], mkB[NPT];
    float4 xvA[NPT], xvB[NPT];
    float4 bv[NPT];  // p_new of the plane below, own cells
    auto fetch = [&](int zc, uchar4 (&mk)[NPT], float4 (&xv)[NPT]) {
#pragma unroll
      for (int k = 0; k < NPT; k++) {
        const unsigned int c =
            plane * (unsigned int)zc + (unsigned int)nx * (unsigned int)(y0 + orow[k]) + 4u * oc4[k];
        if (MASK) {
          const unsigned int m = ld_u32_pol(mask + c, pol_mask);
          mk[k] = make_uchar4(m & 0xffu, (m >> 8) & 0xffu, (m >> 16) & 0xffu, m >> 24);
        }
        if (lag) xv[k] = ld4_pol(reinterpret_cast<const float4 *>(x + c), pol_stream);
      }
    };

    auto stencil = [&](int j, const uchar4 (&mk)[NPT], const float4 (&xv)[NPT]) {
      const int zc = z0 - 1 + j;
      const float *cr = stage + (size_t)(j % ns) * 3 * arr;       // r_new, plane z
      const float *cs = cr + arr;                                  // p_new, plane z
      const float *ts = stage + (size_t)((j + 1) % ns) * 3 * arr + arr;
      const float *po = cr + 2 * arr;                              // p_old, plane z
      const int wz = 9 * wall_count(zc, nz, G.pz);
      const bool interior = G.px && G.py && wz == 0;
#pragma unroll
      for (int k = 0; k < NPT; k++) {
        const int row = orow[k], c4 = oc4[k];
        const int off = (row + 1) * nx + 4 * c4;
        const float4 c = *reinterpret_cast<const float4 *>(cs + off);
        const float4 n = *reinterpret_cast<const float4 *>(cs + off + nx);
        const float4 s = *reinterpret_cast<const float4 *>(cs + off - nx);
        const float4 t = *reinterpret_cast<const float4 *>(ts + off);
        const float4 b = j == 1 ? *reinterpret_cast<const float4 *>(stage + (size_t)((j - 1) % ns) * 3 * arr + arr +
                                                                     off)
                                : bv[k];
        bv[k] = c;
        float w = __shfl_up_sync(0xffffffffu, c.w, 1);
        float ea = __shfl_down_sync(0xffffffffu, c.x, 1);
        if (lane == 0 || c4 == 0) {
          const int xw = 4 * c4 - 1;
          w = xw >= 0 ? cs[off - 1] : (G.px ? cs[(row + 1) * nx + nx - 1] : 0.f);
        }
        if (lane == 31 || c4 == nxv - 1) {
          const int xe = 4 * c4 + 4;
          ea = xe < nx ? cs[off + 4] : (G.px ? cs[(row + 1) * nx] : 0.f);
        }
        float a[4];
        int cls[4] = {0, 0, 0, 0};
        if (interior) {
          a[0] = apply_L<float, ISO>(G, s_dL, 0, c.x, c.y, w, n.x, s.x, t.x, b.x);
          a[1] = apply_L<float, ISO>(G, s_dL, 0, c.y, c.z, c.x, n.y, s.y, t.y, b.y);
          a[2] = apply_L<float, ISO>(G, s_dL, 0, c.z, c.w, c.y, n.z, s.z, t.z, b.z);
          a[3] = apply_L<float, ISO>(G, s_dL, 0, c.w, ea, c.z, n.w, s.w, t.w, b.w);
        } else {
          const int wy = 3 * wall_count(y0 + row, ny, G.py) + wz;
          const int xb = 4 * c4;
#pragma unroll
          for (int i = 0; i < 4; i++) cls[i] = wall_count(xb + i, nx, G.px) + wy;
          a[0] = apply_L<float, ISO>(G, s_dL, cls[0], c.x, c.y, w, n.x, s.x, t.x, b.x);
          a[1] = apply_L<float, ISO>(G, s_dL, cls[1], c.y, c.z, c.x, n.y, s.y, t.y, b.y);
          a[2] = apply_L<float, ISO>(G, s_dL, cls[2], c.z, c.w, c.y, n.z, s.z, t.z, b.z);
          a[3] = apply_L<float, ISO>(G, s_dL, cls[3], c.w, ea, c.z, n.w, s.w, t.w, b.w);
        }
        if (MASK) {
          if (mk[k].x) a[0] = 0.f;
          if (mk[k].y) a[1] = 0.f;
          if (mk[k].z) a[2] = 0.f;
          if (mk[k].w) a[3] = 0.f;
        }
        const float4 r = *reinterpret_cast<const float4 *>(cr + off);
        const float rv[4] = {r.x, r.y, r.z, r.w};
        const float pv[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
        for (int i = 0; i < 4; i++) {
          s_pap = fmaf(pv[i], a[i], s_pap);
          s_rr = fmaf(rv[i], rv[i], s_rr);
          if (interior) {
            s_c1 = fmaf(a[i], rv[i], s_c1);
            s_c2 = fmaf(a[i], a[i], s_c2);
          } else {
            const float iv = cls[i] ? s_inv[cls[i]] : 1.f;
            s_corr = fmaf((iv - 1.f) * rv[i], rv[i], s_corr);
            s_c1 = fmaf(a[i], rv[i] * iv, s_c1);
            s_c2 = fmaf(a[i] * iv, a[i], s_c2);
          }
        }
        const unsigned int g = plane * (unsigned int)zc + (unsigned int)nx * (unsigned int)(y0 + row) + 4u * c4;
        st4_pol(reinterpret_cast<float4 *>(Apout + g), make_float4(a[0], a[1], a[2], a[3]), pol_n);
        st4_pol(reinterpret_cast<float4 *>(pnew + g), c, pol_stream);
        st4_pol(reinterpret_cast<float4 *>(rout + g), r, pol_n);
        if (lag) {
          const float4 q = *reinterpret_cast<const float4 *>(po + off);
          float4 xo = xv[k];
          xo.x = fmaf(alpha, q.x, xo.x);
          xo.y = fmaf(alpha, q.y, xo.y);
          xo.z = fmaf(alpha, q.z, xo.z);
          xo.w = fmaf(alpha, q.w, xo.w);
          st4_pol(reinterpret_cast<float4 *>(x + g), xo, pol_stream);
        }
      }
    };
    // hand a stage back to the producer: every lane's reads of it are done
    auto release = [&](int j) {
      __syncwarp();
      if (lane == 0) mbar_arrive(&s_empty[j % ns]);
    };

    fetch(z0, mkA, xvA);
    if (nj >= 2) fetch(z0 + 1, mkB, xvB);
    prep(0);
    prep(1);
    auto step = [&](int j, uchar4 (&mk)[NPT], float4 (&xv)[NPT]) {
      prep(j + 1);
      fence_proxy_async();  // this thread's stage writes before later tensor copies into the stage
      compute_sync();
      stencil(j, mk, xv);
      if (j == 1) release(0);
      release(j);
      if (j + 2 <= nj) fetch(z0 + j + 1, mk, xv);
    };
    for (int j = 1; j <= nj; j += 2) {
      step(j, mkA, xvA);
      if (j + 1 <= nj) step(j + 1, mkB, xvB);
    }
  }

  if (__syncthreads_or(bad)) {
    if (tid == TNT) {
      // copies issued and maybe still in flight: wait for the last one into every stage
      const int issued = s_issued;
      for (int j = max(0, issued - ns); j < issued; j++)
        if (!(skip_one && j == 2)) mbar_wait(&s_full[j % ns], (unsigned int)(j / ns) & 1u, 10ull * limit);
      atomicExch(&st->done, (int)DONE_TIMEOUT);
    }
    return;
  }
  double v[5] = {(double)s_pap, (double)s_rr + (double)s_corr, (double)s_rr, (double)s_c1, (double)s_c2}, tot[5];
  const unsigned int nb = gridDim.x * gridDim.y;
  const unsigned int bid = blockIdx.x + gridDim.x * blockIdx.y;
  if (last_cta_reduce<5>(v, partials, st, nb, bid, s_red, tot) && tid == 0) {
    st->fq += 1;
    if (lag) finish_deferred(st, tot[1], tot[2]);  // r_{q-1} ends iteration q - 1
    st->dlag = 0;
    if (st->done == RUNNING || st->done == DONE_PENDING) {
      const double rz = st->rz, pap = tot[0];
      const double a = rz / pap;
      st->pAp = pap;
      st->alpha = a;
      st->beta = (rz - 2.0 * a * tot[3] + a * a * tot[4]) / rz;
      st->first = 0;
      st->dlag = 1;
      decide_replacement(st);
    }
  }
}

// ------------------------------------------------------------------ host --
namespace {

typedef CUresult (*EncodeTiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
  static EncodeTiled fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiled>(p);
  }
  return fn;
}

// map of an nx x ny x nz float array with boxes of nrow full rows
bool make_map(CUtensorMap *m, const float *base, int nx, int ny, int nz, int nrow) {
  EncodeTiled fn = encode_fn();
  if (!fn) return false;
  CUresult r;
  const cuuint32_t es[4] = {1, 1, 1, 1};
  if (nx <= 256) {
    const cuuint64_t dim[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
    const cuuint64_t str[2] = {(cuuint64_t)nx * 4, (cuuint64_t)nx * ny * 4};
    const cuuint32_t box[3] = {(cuuint32_t)nx, (cuuint32_t)nrow, 1};
    r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(base), dim, str, box, es,
           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  } else {  // x split into 256-wide pieces so a box still lands as whole rows
    const cuuint64_t dim[4] = {256, (cuuint64_t)(nx / 256), (cuuint64_t)ny, (cuuint64_t)nz};
    const cuuint64_t str[3] = {1024, (cuuint64_t)nx * 4, (cuuint64_t)nx * ny * 4};
    const cuuint32_t box[4] = {256, (cuuint32_t)(nx / 256), (cuuint32_t)nrow, 1};
    r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float *>(base), dim, str, box, es,
           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  }
  return r == CUDA_SUCCESS;
}

struct MapPair {
  const float *ptr;
  CUtensorMap rows, row;
};

// Dynamic shared memory of one launch never exceeds this; the attribute is a
// per-function cap shared by all contexts, so it is set once to the maximum
// (a context of another grid must not lower it under this one).
constexpr int kMaxStageBytes = 200 * 1024;

template <int NPT, bool MASK, bool ISO>
void set_smem_attr() {
  cudaFuncSetAttribute(k1_tma<NPT, MASK, ISO>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxStageBytes);
  cudaFuncSetAttribute(k1_fused<NPT, MASK, ISO>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxStageBytes);
  cudaFuncSetAttribute(k1_fused_ws<NPT, MASK, ISO>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxStageBytes);
}

int env_int(const char *name, int dflt) {
  const char *e = getenv(name);
  return e ? atoi(e) : dflt;
}

}  // namespace

// cuTensorMapEncodeTiled of the driver (null when the driver has none)
void *bbpp_tensor_map_encoder() { return reinterpret_cast<void *>(encode_fn()); }

struct bbpp_tma_state {
  bool ok = false;
  int ty = 0, npt = 0, ns = 0, kz = 0, four_d = 0, smem = 0;
  dim3 grid;
  // the fused iteration kernel: three staged arrays, its own wave
  bool fok = false;
  int fkz = 0, fsmem = 0, pf = 0;
  dim3 fgrid;
  // its warp-specialised form (k1_fused_ws): own ring depth, smem and wave
  bool wok = false;
  int wns = 0, wkz = 0, wsmem = 0;
  dim3 wgrid;
  std::vector<MapPair> maps;
};

// Decide whether the grid suits the TMA kernel and pick its launch shape.
void bbpp_tma_init(bbpp_ctx *ctx) {
  bbpp_tma_state *t = new bbpp_tma_state();
  ctx->tma = t;
  const GeoL &G = ctx->GL;
  const int nx = G.nx, ny = G.ny, nz = G.nz;
  if (env_int("BBPP_TMA", 1) == 0) return;
  if (!encode_fn()) return;
  // slab height: one float4 per thread per plane (NPT = 1) unless BBPP_TMA_NPT asks for 2 or 4
  const int want = env_int("BBPP_TMA_NPT", 1);
  int ty;
  if (nx <= 256 && nx % 32 == 0) ty = (1024 / nx) * ((want == 2 || want == 4) ? want : 1);
  // wide rows (512 or 1024 floats): slabs of 2 rows, BBPP_TMA_TY=4 for 4.  At
  // 512^3 a 4-row fused stage ring takes 147 KB, one CTA per SM; 2 rows take
  // 98 KB, two per SM: 918 against 1005 us per fused launch
  else if (nx % 256 == 0 && nx <= 1024) ty = env_int("BBPP_TMA_TY", 2) == 4 ? 4 : 2;
  else return;
  if (ny % ty != 0 || ty > 256) return;
  const int npt = ty * nx / 1024;
  if ((npt != 1 && npt != 2 && npt != 4) || npt * 1024 != ty * nx) return;
  const int stage = 2 * (ty + 2) * nx * 4;
  // 4 stages: one plane in flight beyond the three in use; more stages cost
  // resident CTAs (measured at 256^3: 4 CTAs/SM with 4 stages beat deeper rings)
  int ns = env_int("BBPP_TMA_NS", 4);
  ns = std::max(4, std::min(8, ns));  // >= 4: the refilled stage is never one of the three in use
  while (ns > 4 && ns * stage > kMaxStageBytes) ns--;
  if (ns * stage > kMaxStageBytes) return;
  t->ty = ty;
  t->npt = npt;
  t->ns = ns;
  t->smem = ns * stage;
  t->four_d = nx > 256;
  // one wave of resident CTAs
  int per_sm = 0;
  static unsigned long long attr_set = 0;  // per device
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && !(attr_set & (1ull << dev))) {
    attr_set |= 1ull << dev;
    set_smem_attr<1, true, true>();
    set_smem_attr<1, true, false>();
    set_smem_attr<1, false, true>();
    set_smem_attr<1, false, false>();
    set_smem_attr<2, true, true>();
    set_smem_attr<2, true, false>();
    set_smem_attr<2, false, true>();
    set_smem_attr<2, false, false>();
    set_smem_attr<4, true, true>();
    set_smem_attr<4, true, false>();
    set_smem_attr<4, false, true>();
    set_smem_attr<4, false, false>();
  }
#define BBPP_TMA_ATTR(N) \
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k1_tma<N, true, true>, TNT, t->smem);
  if (npt == 1) { BBPP_TMA_ATTR(1) }
  else if (npt == 2) { BBPP_TMA_ATTR(2) }
  else { BBPP_TMA_ATTR(4) }
#undef BBPP_TMA_ATTR
  cudaGetLastError();
  if (per_sm < 1) return;
  const int slabs = ny / ty;
  auto chunking = [&](int per, int *kz_out, dim3 *grid_out) {
    const int nzc = bbpp_z_chunks(slabs, nz, (long long)ctx->sms * per, 1, kz_out);
    *grid_out = dim3(slabs, nzc, 1);
  };
  chunking(per_sm, &t->kz, &t->grid);
  t->ok = true;
  // fused kernel: r, Ap_old and p_old staged (three arrays per stage)
  const int fsmem = ns * 3 * (ty + 2) * nx * 4;
  int fper = 0;
  if (fsmem <= kMaxStageBytes) {
#define BBPP_FUSED_OCC(N) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fper, k1_fused<N, true, true>, TNT, fsmem);
    if (npt == 1) { BBPP_FUSED_OCC(1) }
    else if (npt == 2) { BBPP_FUSED_OCC(2) }
    else { BBPP_FUSED_OCC(4) }
#undef BBPP_FUSED_OCC
    cudaGetLastError();
  }
  if (fper >= 1) {
    // L2 prefetch distance in planes beyond the staged copies.  Measured at
    // 256^3 (ms per solve): 0 -> 72.6, 1 -> 69.8, 2 -> 71.8, 3 -> 75.4; the
    // staged arrays and x / mask both contribute
    t->pf = std::max(0, std::min(8, env_int("BBPP_L2PF", 1)));
    t->fsmem = fsmem;
    chunking(fper, &t->fkz, &t->fgrid);
    t->fok = true;
  }
  // the warp-specialised form: a stage is free once its own plane's stencil
  // is done, so 3 stages already keep one plane in flight (BBPP_WS_NS, 3..8)
  if (t->fok && env_int("BBPP_FUSED_WS", 0)) {
    int wns = std::max(3, std::min(8, env_int("BBPP_WS_NS", 4)));
    while (wns > 3 && wns * 3 * (ty + 2) * nx * 4 > kMaxStageBytes) wns--;
    const int wsmem = wns * 3 * (ty + 2) * nx * 4;
    int wper = 0;
    if (wsmem <= kMaxStageBytes) {
#define BBPP_WS_OCC(N) \
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&wper, k1_fused_ws<N, true, true>, WS_THREADS, wsmem);
      if (npt == 1) { BBPP_WS_OCC(1) }
      else if (npt == 2) { BBPP_WS_OCC(2) }
      else { BBPP_WS_OCC(4) }
#undef BBPP_WS_OCC
      cudaGetLastError();
    }
    if (wper >= 1) {
      t->wns = wns;
      t->wsmem = wsmem;
      chunking(wper, &t->wkz, &t->wgrid);
      t->wok = true;
    }
  }
}

void bbpp_tma_free(bbpp_ctx *ctx) {
  delete ctx->tma;
  ctx->tma = nullptr;
}

// z chunking of the TMA search kernel: kz planes per CTA, nzc chunks
bool bbpp_tma_chunks(const bbpp_ctx *ctx, int *kz, int *nzc) {
  if (!ctx->tma || !ctx->tma->ok) return false;
  *kz = ctx->tma->kz;
  *nzc = (int)ctx->tma->grid.y;
  return true;
}

size_t bbpp_tma_partials(const bbpp_ctx *ctx) {
  if (!ctx->tma || !ctx->tma->ok) return 0;
  size_t n = (size_t)ctx->tma->grid.x * ctx->tma->grid.y;
  // the fused kernel sums five products per CTA into room for three per CTA
  if (ctx->tma->fok) n = std::max(n, ((size_t)ctx->tma->fgrid.x * ctx->tma->fgrid.y * 5 + 2) / 3);
  if (ctx->tma->wok) n = std::max(n, ((size_t)ctx->tma->wgrid.x * ctx->tma->wgrid.y * 5 + 2) / 3);
  return n;
}

bool bbpp_tma_fused_ok(const bbpp_ctx *ctx) { return ctx->tma && ctx->tma->ok && ctx->tma->fok; }

// tensor maps of one vector (copied out: the cache may reallocate)
static bool get_maps(bbpp_tma_state *t, const float *p, const GeoL &G, MapPair *out) {
  for (const auto &m : t->maps)
    if (m.ptr == p) {
      *out = m;
      return true;
    }
  MapPair m;
  m.ptr = p;
  if (!make_map(&m.rows, p, G.nx, G.ny, G.nz, t->ty) || !make_map(&m.row, p, G.nx, G.ny, G.nz, 1)) return false;
  if (t->maps.size() >= 16) t->maps.erase(t->maps.begin());
  t->maps.push_back(m);
  *out = m;
  return true;
}

// tensor maps of the six buffers of a fused solve, built before its graphs
bool bbpp_tma_fused_maps(bbpp_ctx *ctx, const float *const r[2], const float *const a[2], const float *const p[2]) {
  bbpp_tma_state *t = ctx->tma;
  if (!t || !t->ok || !t->fok) return false;
  MapPair m;
  for (int i = 0; i < 2; i++)
    if (!get_maps(t, r[i], ctx->GL, &m) || !get_maps(t, a[i], ctx->GL, &m) || !get_maps(t, p[i], ctx->GL, &m))
      return false;
  return true;
}

bool bbpp_tma_fused(bbpp_ctx *ctx, const uint8_t *mask, const float *rin, const float *apin, const float *pold,
                    float *rout, float *pnew, float *apout, float *x, DevState *st) {
  bbpp_tma_state *t = ctx->tma;
  if (!t || !t->ok || !t->fok) return false;
  MapPair mr, ma, mp;
  if (!get_maps(t, rin, ctx->GL, &mr) || !get_maps(t, apin, ctx->GL, &ma) || !get_maps(t, pold, ctx->GL, &mp))
    return false;
  FusedMaps M;
  M.r_rows = mr.rows;
  M.r_row = mr.row;
  M.a_rows = ma.rows;
  M.a_row = ma.row;
  M.p_rows = mp.rows;
  M.p_row = mp.row;
#define BBPP_FUSED_LAUNCH(N, MK, IS)                                                                              \
  if (t->wok)                                                                                                     \
    bbpp_launch(ctx, k1_fused_ws<N, MK, IS>, t->wgrid, dim3(WS_THREADS), (size_t)t->wsmem, ctx->GL, M, rout, pnew, \
                apout, x, mask, st, ctx->partials, t->ty, t->wkz, t->wns, t->four_d, (int)ctx->l2hint, t->pf);     \
  else                                                                                                            \
    bbpp_launch(ctx, k1_fused<N, MK, IS>, t->fgrid, dim3(TNT), (size_t)t->fsmem, ctx->GL, M, rout, pnew, apout, x,  \
                mask, st, ctx->partials, t->ty, t->fkz, t->ns, t->four_d, (int)ctx->l2hint, t->pf)
#define BBPP_FUSED_NPT(N)                              \
  if (mask) {                                          \
    if (ctx->GL.iso) BBPP_FUSED_LAUNCH(N, true, true);   \
    else BBPP_FUSED_LAUNCH(N, true, false);              \
  } else {                                             \
    if (ctx->GL.iso) BBPP_FUSED_LAUNCH(N, false, true);  \
    else BBPP_FUSED_LAUNCH(N, false, false);             \
  }
  if (t->npt == 1) { BBPP_FUSED_NPT(1) }
  else if (t->npt == 2) { BBPP_FUSED_NPT(2) }
  else { BBPP_FUSED_NPT(4) }
#undef BBPP_FUSED_NPT
#undef BBPP_FUSED_LAUNCH
  return true;
}

bool bbpp_tma_search(bbpp_ctx *ctx, const uint8_t *mask, const float *r, const float *pold, float *pnew, float *Ap,
                     float *x, DevState *st) {
  bbpp_tma_state *t = ctx->tma;
  if (!t || !t->ok) return false;
  MapPair mr, mp;
  if (!get_maps(t, r, ctx->GL, &mr) || !get_maps(t, pold, ctx->GL, &mp)) return false;
  TmaMaps M;
  M.r_rows = mr.rows;
  M.r_row = mr.row;
  M.p_rows = mp.rows;
  M.p_row = mp.row;
#define BBPP_TMA_LAUNCH(N, MK, IS)                                                                          \
  bbpp_launch(ctx, k1_tma<N, MK, IS>, t->grid, dim3(TNT), (size_t)t->smem, ctx->GL, M, pnew, Ap, x, mask, st, \
              ctx->partials, t->ty, t->kz, t->ns, t->four_d, (int)ctx->l2hint)
#define BBPP_TMA_NPT(N)                            \
  if (mask) {                                      \
    if (ctx->GL.iso) BBPP_TMA_LAUNCH(N, true, true);   \
    else BBPP_TMA_LAUNCH(N, true, false);              \
  } else {                                         \
    if (ctx->GL.iso) BBPP_TMA_LAUNCH(N, false, true);  \
    else BBPP_TMA_LAUNCH(N, false, false);             \
  }
  if (t->npt == 1) { BBPP_TMA_NPT(1) }
  else if (t->npt == 2) { BBPP_TMA_NPT(2) }
  else { BBPP_TMA_NPT(4) }
#undef BBPP_TMA_NPT
#undef BBPP_TMA_LAUNCH
  return true;
}
