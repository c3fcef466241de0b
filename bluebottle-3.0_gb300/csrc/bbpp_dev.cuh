// bbpp_dev.cuh -- device-side building blocks shared by the solver kernels.
//
// Data layout (HBM): dense cell-centred arrays, x fastest,
// c = i + nx*(j + ny*k), no ghost layer.  One byte of mask per cell.
// Periodic neighbours wrap by index; a wall (Neumann) neighbour reads as 0 and
// the wall face is removed from the diagonal, which is the effect of
// flag_* == 0 in the reference stencil (src/solver_kernel.cu:699-707).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace bbpp {

// Programmatic dependent launch: wait until the preceding kernel of the stream
// has finished and its writes are visible (a no-op without a programmatic
// dependency), then let the next kernel start launching.  Every iteration
// kernel calls it before it reads anything a predecessor wrote.
__device__ __forceinline__ void pdl_sync() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Solve states written by the last CTA of a reduction kernel.
enum DoneCode : int {
  RUNNING = 0,
  DONE_CONVERGED = 1,
  DONE_MAX_ITER = 2,
  DONE_NAN = 3,
  DONE_PENDING = 4,  // recursive residual met TRUE_REL; explicit check pending
  DONE_TINY = 5,
  DONE_TIMEOUT = 6   // a bounded wait inside a kernel ran out
};

// Device-resident scalar state of one PCG solve.
struct DevState {
  double bb;       // (rhs, rhs)
  double tol2bb;   // tol^2 * (rhs, rhs)
  double rz;       // (r, z) of the current residual
  double rz_last;  // (r, z) of the most recent residual (also when stopping)
  double rr;       // (r, r) of the most recent residual
  double pAp;      // (p, Ap)
  double alpha;
  double beta;
  int iter;        // completed iterations
  int done;        // DoneCode
  int first;       // next search-direction update is p = z (beta = 0)
  int max_iter;
  int stop;        // 0 = (r,z) rule, 1 = recursive ||r|| rule + explicit confirm
  int replacements;
  unsigned int ticket;  // arrival counter of the last-CTA reductions
  int dlag;        // x lacks alpha * p of the last search direction (added by the next search kernel)
  double tiny;     // (rhs,rhs) below this ends the solve at once (DONE_TINY)
  // residual replacement at a checkpoint (every replace_every iterations)
  // happens when rep_now; the search kernel sets it from rep_d2 (0: always;
  // else once (r,r) <= rep_d2 * rr_ref, the (r,r) of the last replacement)
  // or when rep_maxgap iterations have passed since the last one
  double rr_ref;
  double rep_d2;
  int rep_maxgap;
  int last_rep;
  int rep_now;
  int inject;            // test hook: 1 = the first TMA search CTA skips the copies of one plane
  long long wait_ns;     // bound of a device-side wait (0: one second)
  int fq;                // fused iteration kernels completed in this solve
  // alpha_k and beta_k of iterations 1 .. trace_n (index k - 1), recorded by
  // the search kernel (k1_search2) and the end of an iteration; null: none
  double *trace_a;
  double *trace_b;
  int trace_n;
};

__device__ __forceinline__ void trace_put(double *buf, int n, int i, double v) {
  if (buf && i >= 0 && i < n) buf[i] = v;
}

// Set by the last CTA of a search kernel: does this iteration's checkpoint
// (if it is one) replace the residual?
__device__ __forceinline__ void decide_replacement(DevState *st) {
  st->rep_now = (st->rep_d2 <= 0.0) || (st->rr <= st->rep_d2 * st->rr_ref) ||
                (st->iter + 1 - st->last_rep >= st->rep_maxgap);
}

// Geometry and per-wall-class constants.  A cell's wall class is
// wx + 3 wy + 9 wz where w_d counts the wall faces of the cell in direction d
// (0 for periodic directions).  tab[0..26]: fluid diagonal of (-A);
// tab[27..53]: Jacobi invM; tab[54..80]: diagonal of a solid (identity) row.
struct Geo {
  int nx, ny, nz;
  int px, py, pz;   // 1 = periodic
  long long n;
  double cx, cy, cz;  // 1/dx^2, 1/dy^2, 1/dz^2
  double tab[81];
  // exact division by nx and nx*ny: q = umul64hi(n, ceil(2^64/d)) for 32-bit n
  // (Lemire, Kaser, Kurz 2019); d == 1 is stored as 0 and returns n.
  unsigned long long mx, mxy;
};

// L2 eviction priority of one access (createpolicy): 0 normal, 1 evict_first
// (streamed data), 2 evict_last (data the next kernel reads again)
__device__ __forceinline__ unsigned long long l2_policy(int kind) {
  unsigned long long p;
  if (kind == 2) asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  else if (kind == 1) asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  else asm volatile("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(p));
  return p;
}

__device__ __forceinline__ float4 ld4_pol(const float4 *a, unsigned long long pol) {
  float4 v;
  asm("ld.global.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
      : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
      : "l"(a), "l"(pol));
  return v;
}

__device__ __forceinline__ void st4_pol(float4 *a, const float4 v, unsigned long long pol) {
  asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(a), "f"(v.x), "f"(v.y), "f"(v.z),
               "f"(v.w), "l"(pol)
               : "memory");
}

__device__ __forceinline__ unsigned int ld_u32_pol(const void *a, unsigned long long pol) {
  unsigned int v;
  asm("ld.global.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(v) : "l"(a), "l"(pol));
  return v;
}

// FP32 -> FP64, exact, with integer operations: GB300 runs the conversion
// instruction on the FP64 pipe (1/64 of the FP32 rate).  Zero keeps its sign;
// subnormal inputs (never produced by the solver's vectors in practice) take
// the conversion instruction.
__device__ __forceinline__ double widen_f32(float f) {
  const unsigned int u = __float_as_uint(f);
  const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
  const unsigned int e32 = (u >> 23) & 0xffu;
  const unsigned long long frac = (unsigned long long)(u & 0x7fffffu) << 29;
  if (e32 == 0) return frac ? (double)f : __longlong_as_double((long long)sign);
  if (e32 == 0xffu) return __longlong_as_double((long long)(sign | 0x7ff0000000000000ull | frac));
  return __longlong_as_double((long long)(sign | ((unsigned long long)(e32 - 127u + 1023u) << 52) | frac));
}

__device__ __forceinline__ unsigned int fdiv(unsigned int n, unsigned long long m) {
  return m ? (unsigned int)__umul64hi((unsigned long long)n, m) : n;
}

__device__ __forceinline__ int wall_count(int g, int nmax, int periodic) {
  return periodic ? 0 : (int)(g == 0) + (int)(g == nmax - 1);
}

__device__ __forceinline__ int wall_class(const Geo &G, int gx, int gy, int gz) {
  return wall_count(gx, G.nx, G.px) + 3 * wall_count(gy, G.ny, G.py) + 9 * wall_count(gz, G.nz, G.pz);
}

// Map a halo coordinate g in [-1, n] (or beyond, for partial tiles) to a cell
// index; returns -1 when there is no cell (a wall, or outside the tile's use).
__device__ __forceinline__ int halo_index(int g, int n, int periodic) {
  if (g >= 0 && g < n) return g;
  if (periodic) {
    if (g == -1) return n - 1;
    if (g == n) return 0;
  }
  return -1;
}

template <typename T> struct Acc;  // per-thread partial-sum type
template <> struct Acc<double> { typedef double type; };
template <> struct Acc<float> { typedef float type; };

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum NV doubles over the CTA; result valid in thread 0.  s_buf holds
// NV * (blockDim/32) doubles.  Fixed order => deterministic.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double *s_buf) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
#pragma unroll
  for (int q = 0; q < NV; q++) v[q] = warp_sum(v[q]);
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < NV; q++) s_buf[q * nw + warp] = v[q];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int q = 0; q < NV; q++) {
      double t = lane < nw ? s_buf[q * nw + lane] : 0.0;
      v[q] = warp_sum(t);
    }
  }
  __syncthreads();
}

// Publish this CTA's NV partial sums and, in the CTA that arrives last,
// reduce all of them in block order.  Returns true in the last CTA, whose
// thread 0 then holds the totals in tot[].  1-D thread blocks only.
template <int NV>
__device__ __forceinline__ bool last_cta_reduce(double (&v)[NV], double *partials, DevState *st,
                                                unsigned int nblocks, unsigned int bid, double *s_buf,
                                                double (&tot)[NV]) {
  __shared__ int s_last;
  block_sum<NV>(v, s_buf);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < NV; q++) partials[(size_t)q * nblocks + bid] = v[q];
    __threadfence();
    unsigned int t = atomicAdd(&st->ticket, 1u);
    s_last = (t == nblocks - 1);
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  double acc[NV];
#pragma unroll
  for (int q = 0; q < NV; q++) acc[q] = 0.0;
  for (unsigned int b = threadIdx.x; b < nblocks; b += blockDim.x) {
#pragma unroll
    for (int q = 0; q < NV; q++) acc[q] += __ldcg(&partials[(size_t)q * nblocks + b]);
  }
  block_sum<NV>(acc, s_buf);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < NV; q++) tot[q] = acc[q];
    st->ticket = 0;
  }
  return true;
}

// End of an iteration: new residual products rz1, rr1 are known.
__device__ __forceinline__ void finish_iteration(DevState *st, double rz1, double rr1, bool count_iter) {
  int it = st->iter + (count_iter ? 1 : 0);
  st->iter = it;
  st->rz_last = rz1;
  st->rr = rr1;
  bool conv = (st->stop == 0) ? (rz1 <= st->tol2bb) : (rr1 <= st->tol2bb);
  if (conv) {
    if (it > st->max_iter) st->done = DONE_MAX_ITER;
    else st->done = (st->stop == 0) ? DONE_CONVERGED : DONE_PENDING;
  } else if (isnan(rz1)) {
    st->done = DONE_NAN;
  } else {
    st->beta = rz1 / st->rz;
    trace_put(st->trace_b, st->trace_n, it - 1, st->beta);
    st->rz = rz1;
    if (it > st->max_iter) st->done = DONE_MAX_ITER;
  }
}

// End of an iteration whose update a fused kernel deferred: its residual's
// products rz1, rr1 are known; the next beta comes from the fused kernel's
// expansion, so only rz is kept (the base of that expansion).
__device__ __forceinline__ void finish_deferred(DevState *st, double rz1, double rr1) {
  const int it = st->iter + 1;
  st->iter = it;
  st->rz_last = rz1;
  st->rr = rr1;
  const bool conv = (st->stop == 0) ? (rz1 <= st->tol2bb) : (rr1 <= st->tol2bb);
  if (isnan(rz1)) {
    st->done = DONE_NAN;
    return;
  }
  st->rz = rz1;
  if (conv) st->done = (it > st->max_iter) ? DONE_MAX_ITER : ((st->stop == 0) ? DONE_CONVERGED : DONE_PENDING);
  else if (it > st->max_iter) st->done = DONE_MAX_ITER;
}

}  // namespace bbpp
