// bbpp_fast.cuh -- the solver's iteration kernels on the scaled operator.
//
// The PCG runs on L = S (-A) with S = 1 / (2/dx^2 + 2/dy^2 + 2/dz^2), so a
// fluid cell away from walls has diagonal 1 and Jacobi weight 1, and the
// iteration needs no multiply for them.  With L x = S rhs the iterates are
// those of the reference's PCG on (-A) x = rhs (alpha and beta are unchanged;
// (r,z), (r,r) and (rhs,rhs) scale by S, S^2, S^2).  Scaling matters on GB300
// because FP64 issues at 1/64 of FP32: these kernels keep FP64 instructions
// per cell to one FMA per update, one per dot and one for the stencil, whose
// six-neighbour sum runs on the integer pipe (xsum6) on isotropic grids.
//
// Cells of a solid sphere hold r = p = Ap = x = 0 throughout (their rhs is
// taken as zero, as part_BC_p makes it, src/particle_kernel.cu:1753): the
// residual kernel writes r = 0 and x = 0 there, and the search kernel writes
// Ap = 0 there.  A fluid cell's solid neighbour then contributes p = 0, which
// is the reference's dropped off-diagonal (src/solver_kernel.cu:691-707).
//
//  k1_search2 p = invM r + beta p_old on a 64x16 tile plus halo (two cells per
//             thread), ring of three planes in shared memory while the CTA
//             marches in z; Ap = L p and the (p, Ap) partial.
//  k2_update  r -= alpha Ap, (r,r) and the wall correction of (r,z), 16-byte
//             vector loads; optionally in the reverse of the search kernel's
//             plane order.
//  k_resid_s  r = bscale rhs - L x (solid cells 0) with (r,z), (r,r), (rhs,rhs).
//  k_resid_ff the same for FP64 x into FP32 r in float-float arithmetic (an
//             option).
#pragma once

#include <cstring>
#include <type_traits>

#include "bbpp_dev.cuh"

namespace bbpp {

constexpr int FX = 32;       // tile width (x): one warp
constexpr int FY = 16;       // tile height (y): two rows per thread
constexpr int FHX = FX + 2;  // halo tile width
constexpr int FHY = FY + 2;
constexpr int FNT = 256;     // threads
constexpr int FHE = FHX * FHY;                    // halo elements per plane (612)
constexpr int FPER = (FHE + FNT - 1) / FNT;       // halo elements per thread (3)

// Scaled-operator constants.  Wall class as in Geo: wx + 3 wy + 9 wz.
struct GeoL {
  int nx, ny, nz;
  int px, py, pz;
  int iso;             // ax == ay == az
  int xsum;            // FP64 stencils, iso: interior neighbour sums on the integer pipe (xsum6)
  long long n;
  double S;            // scale of L = S (-A)
  double ax, ay, az;   // S/dx^2, S/dy^2, S/dz^2
  double dL[27];       // fluid diagonal of L per wall class (dL[0] = 1)
  double invL[27];     // Jacobi weight 1/dL (invL[0] = 1)
  float fax, fay, faz;
  float fdL[27], finvL[27];
  unsigned long long mx, mxy;  // exact division by nx, nx*ny
};

template <typename T> __device__ __forceinline__ T gl_ax(const GeoL &G);
template <> __device__ __forceinline__ double gl_ax<double>(const GeoL &G) { return G.ax; }
template <> __device__ __forceinline__ float gl_ax<float>(const GeoL &G) { return G.fax; }
template <typename T> __device__ __forceinline__ T gl_ay(const GeoL &G);
template <> __device__ __forceinline__ double gl_ay<double>(const GeoL &G) { return G.ay; }
template <> __device__ __forceinline__ float gl_ay<float>(const GeoL &G) { return G.fay; }
template <typename T> __device__ __forceinline__ T gl_az(const GeoL &G);
template <> __device__ __forceinline__ double gl_az<double>(const GeoL &G) { return G.az; }
template <> __device__ __forceinline__ float gl_az<float>(const GeoL &G) { return G.faz; }

template <typename T>
__device__ __forceinline__ void load_tabs(const GeoL &G, T *s_dL, T *s_inv) {
  for (int e = threadIdx.x; e < 27; e += blockDim.x) {
    if (sizeof(T) == 8) {
      s_dL[e] = (T)G.dL[e];
      s_inv[e] = (T)G.invL[e];
    } else {
      s_dL[e] = (T)G.fdL[e];
      s_inv[e] = (T)G.finvL[e];
    }
  }
}

// L p at one cell from its 7 values; cls = wall class; the masked variant has
// already zeroed the couplings of solid cells.
template <typename T, bool ISO>
__device__ __forceinline__ T apply_L(const GeoL &G, const T *s_dL, int cls, T pc, T pe, T pw, T pn, T ps, T pt,
                                     T pb) {
  // cls is a literal 0 on the interior path, so only one form is emitted there
  if (ISO) {
    const T s = ((pe + pw) + (pn + ps)) + (pt + pb);
    const T na = -gl_ax<T>(G);
    if (cls == 0) return fma(na, s, pc);
    return fma(s_dL[cls], pc, na * s);
  } else {
    T s = gl_ax<T>(G) * (pe + pw);
    s = fma(gl_ay<T>(G), pn + ps, s);
    s = fma(gl_az<T>(G), pt + pb, s);
    if (cls == 0) return pc - s;
    return fma(s_dL[cls], pc, -s);
  }
}

// ---------------------------------------------- exact neighbour sums ---
// bit-level helpers of xsum6 on either side (the host copy serves the tests)
__host__ __device__ __forceinline__ unsigned long long xs_bits(double d) {
#ifdef __CUDA_ARCH__
  return (unsigned long long)__double_as_longlong(d);
#else
  unsigned long long b;
  memcpy(&b, &d, sizeof b);
  return b;
#endif
}
__host__ __device__ __forceinline__ double xs_double(unsigned long long b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double d;
  memcpy(&d, &b, sizeof d);
  return d;
#endif
}
__host__ __device__ __forceinline__ int xs_clz64(unsigned long long m) {  // m != 0
#ifdef __CUDA_ARCH__
  return __clzll((long long)m);
#else
  return __builtin_clzll(m);
#endif
}

// The six-neighbour sum of the isotropic stencil in FP64 as one fixed-point
// sum on the integer pipe, rounded once to nearest even.  GB300 issues FP64 at
// 1/64 of its FP32 rate, and the five FP64 adds kept the FP64 search kernel on
// that pipe; the ~150 integer operations below run beside the remaining FP64
// work (at 256^3 the kernel went from 370 to 311 us per launch).
//
// Each 53-bit significand is aligned to the largest exponent of the six, the
// largest value's leading bit at bit 59 of a signed 64-bit accumulator; bits
// shifted below bit 0 are dropped, under one unit (2^-59 of the largest
// value's leading bit) per value.  Six aligned magnitudes stay below 6 * 2^60
// < 2^63, so the accumulator cannot overflow.  The result lies within 1/2 ulp
// of the exact sum plus six units (ulp(max)/128), against five roundings of up
// to 1/2 ulp each for the FP64 adds.  Returns false, with `out` unset, when
// the largest biased exponent lies outside [128, 2040] (all six zero or tiny,
// or an Inf or NaN).
__host__ __device__ __forceinline__ bool xsum6(const double (&v)[6], double &out) {
  // biased exponent << 20 of the largest magnitude
  unsigned int E = 0;
#pragma unroll
  for (int i = 0; i < 6; i++) {
    const unsigned int ei = (unsigned int)(xs_bits(v[i]) >> 32) & 0x7ff00000u;
    E = E > ei ? E : ei;
  }
  if (E < (128u << 20) || E > (2040u << 20)) return false;
  // A value of exponent field e shifts right by E - e + 4.  Zero and
  // subnormal values (e = 0) have no leading bit and lie below 2^-1022, under
  // 2^-68 of one unit (E >= 128), so any shift of 63 or more drops them.
  const unsigned int Ep = E + (4u << 20);
  long long acc = 0;
#pragma unroll
  for (int i = 0; i < 6; i++) {
    const unsigned long long bi = xs_bits(v[i]);
    const unsigned int hi = (unsigned int)(bi >> 32), lo = (unsigned int)bi;
    const unsigned int raw = hi & 0x7ff00000u;
    // significand left-aligned in 64 bits: fraction at bits 62..11, the
    // leading bit (set iff the exponent field is non-zero) at bit 63
    unsigned int whi = (hi << 11) | (lo >> 21);
    whi = (whi & 0x7fffffffu) | ((raw + 0x7fffffffu) & 0x80000000u);
    const unsigned int sh0 = (Ep - raw) >> 20, sh = sh0 < 63u ? sh0 : 63u;
    const long long w = (long long)((((unsigned long long)whi << 32) | (unsigned long long)(lo << 11)) >> sh);
    const long long sg = (long long)((int)hi >> 31);
    acc += (w ^ sg) - sg;
  }
  // value = acc * 2^(E - 1082), rounded once to nearest even in integer
  // arithmetic (a conversion instruction would run on the FP64 pipe)
  const long long sg = acc >> 63;
  unsigned long long m = (unsigned long long)((acc ^ sg) - sg);
  if (m == 0ull) {
    out = 0.0;
    return true;
  }
  const int lz = xs_clz64(m);  // >= 1: |acc| < 2^63
  m <<= lz;
  const unsigned long long mant = m >> 11;  // 53 bits, leading bit at 52
  const unsigned int rest = (unsigned int)m & 0x7ffu;
  const unsigned long long up = (rest > 0x400u || (rest == 0x400u && (mant & 1ull))) ? 1ull : 0ull;
  // biased exponent E + 4 - lz, of which the leading bit of mant adds one; a
  // carry out of the rounding adds another
  const unsigned long long bits = ((unsigned long long)((E >> 20) + 3u - (unsigned int)lz) << 52) + mant + up;
  out = xs_double(bits | ((unsigned long long)sg & 0x8000000000000000ull));
  return true;
}

// The isotropic neighbour sum of FP64 p: xsum6 where it applies, FP64 adds in
// the stencil's order otherwise.  A solid cell (`skip`) discards its result, so
// it never takes the FP64 branch.
__host__ __device__ __forceinline__ double nb_sum6(double pe, double pw, double pn, double ps, double pt, double pb,
                                          bool skip) {
  const double v[6] = {pe, pw, pn, ps, pt, pb};
  double s;
  if (!xsum6(v, s)) s = skip ? 0.0 : ((pe + pw) + (pn + ps)) + (pt + pb);
  return s;
}

// L p at an interior cell (class 0): apply_L, or for FP64 on an isotropic grid
// with G.xsum set, the centre minus ax times the exact neighbour sum.
template <typename T, bool ISO>
__device__ __forceinline__ T apply_L0(const GeoL &G, T pc, T pe, T pw, T pn, T ps, T pt, T pb, bool skip) {
  return apply_L<T, ISO>(G, nullptr, 0, pc, pe, pw, pn, ps, pt, pb);
}
template <>
__device__ __forceinline__ double apply_L0<double, true>(const GeoL &G, double pc, double pe, double pw, double pn,
                                                         double ps, double pt, double pb, bool skip) {
  if (!G.xsum) return apply_L<double, true>(G, nullptr, 0, pc, pe, pw, pn, ps, pt, pb);
  return fma(-G.ax, nb_sum6(pe, pw, pn, ps, pt, pb, skip), pc);
}

// ------------------------------------------------------------ K1, pairs ---
// K1, the search kernel: p_new = z + beta p_old (z = r on the scaled
// operator) on the CTA's tile plus a one-cell halo, kept in a 3-plane shared
// ring while the CTA marches in z; then Ap = L p_new and the (p, Ap) partial.
// Replaces PP_update_search + exchange + PP_spmv_shared_load + thrust (p,Ap)
// (src/solver_kernel.cu:528-713,906-927, src/cuda_solver.cu:201-205,256-263).
// Two x-adjacent cells per thread: a tile is 64 x 16 cells (32 x 8 threads, two rows each).  Halo rows are loaded as aligned
// pairs into shared rows padded so the pairs stay aligned (index 0 pad, 1 west
// halo, 2..65 tile, 66 east halo); the two edge columns are scalar loads.
// Only the thread's own cells need the mask (Ap = 0 in a solid cell), so it
// is read straight from global memory.  Pairs need an even nx; odd nx uses
// scalar loads.
constexpr int PX = 64;          // tile width
constexpr int PY = 16;          // tile height
constexpr int PW = PX + 4;      // padded shared row
constexpr int PHY = PY + 2;     // rows with halo
constexpr int PROWS = (PHY + 7) / 8;  // halo rows per thread (3)

template <typename T> struct V2of;
template <> struct V2of<double> { typedef double2 type; };
template <> struct V2of<float> { typedef float2 type; };

// Own cells of a committed plane: store p_new, and add the previous
// iteration's alpha p_old into x while p_old is at hand (x lags one step).
template <typename T, typename V2>
__device__ __forceinline__ void store_own(T *__restrict__ pnew, T *__restrict__ x, unsigned int c, const V2 v,
                                          const T (&po)[2], T alpha, bool lag, bool pair_full, int npair) {
  if (pair_full) {
    *reinterpret_cast<V2 *>(pnew + c) = v;
    if (lag) {
      V2 xv = *reinterpret_cast<const V2 *>(x + c);
      xv.x = fma(alpha, po[0], xv.x);
      xv.y = fma(alpha, po[1], xv.y);
      *reinterpret_cast<V2 *>(x + c) = xv;
    }
  } else {
    pnew[c] = v.x;
    if (lag) x[c] = fma(alpha, po[0], x[c]);
    if (npair == 2) {
      pnew[c + 1] = v.y;
      if (lag) x[c + 1] = fma(alpha, po[1], x[c + 1]);
    }
  }
}

template <typename T, bool MASK, bool ISO>
__global__ void __launch_bounds__(FNT, sizeof(T) == 8 ? 3 : 4) k1_search2(const GeoL G, const T *__restrict__ r, const T *__restrict__ pold,
                                                  T *__restrict__ pnew, T *__restrict__ Ap, T *__restrict__ x,
                                                  const uint8_t *__restrict__ mask, DevState *st, double *partials,
                                                  int kz) {
  typedef typename V2of<T>::type V2;
  __shared__ T s_dL[27], s_inv[27];
  __shared__ __align__(16) T sp[3][PHY][PW];
  __shared__ double s_red[FNT / 32];
  pdl_sync();
  if (*(volatile int *)&st->done) return;
  const bool first = *(volatile int *)&st->first;
  const T beta = first ? T(0) : (T)(*(volatile double *)&st->beta);
  // x += alpha p_old of the previous iteration, on the own cells as p_old passes
  const bool lag = !first && *(volatile int *)&st->dlag;
  const T alpha = lag ? (T)(*(volatile double *)&st->alpha) : T(0);
  load_tabs<T>(G, s_dL, s_inv);

  const int tid = threadIdx.x;
  const int tx = tid & 31, ty = tid >> 5;
  const int x0 = blockIdx.x * PX, y0 = blockIdx.y * PY;
  const int z0 = blockIdx.z * kz, z1 = min(z0 + kz, G.nz);
  const int nx = G.nx, ny = G.ny, nz = G.nz;
  const unsigned int plane = (unsigned int)nx * (unsigned int)ny;
  const bool vec = !(nx & 1);
  const bool xy_walls = !(G.px && G.py);

  // pair loads: rows ly = ty + 8k, columns x0 + 2tx, +1
  const int gxp = x0 + 2 * tx;
  const int npair = (gxp + 1 < nx) ? 2 : (gxp < nx ? 1 : 0);  // own cells of the pair
  // halo cells of the pair slot: in a partial tile the slot just past the
  // grid holds the periodic image (cell 0) of the east neighbour
  const int gxa = halo_index(gxp, nx, G.px), gxb = halo_index(gxp + 1, nx, G.px);
  const bool pair_full = vec && gxp + 1 < nx;
  const int wxp0 = gxa >= 0 ? wall_count(gxa, nx, G.px) : 0;
  const int wxp1 = gxb >= 0 ? wall_count(gxb, nx, G.px) : 0;
  int row_off[PROWS];  // nx * gy of the row, or -1
  int row_wy[PROWS];
#pragma unroll
  for (int k = 0; k < PROWS; k++) {
    const int ly = ty + 8 * k;
    row_off[k] = -1;
    row_wy[k] = 0;
    if (ly < PHY) {
      const int gy = halo_index(y0 + ly - 1, ny, G.py);
      if (gy >= 0) {
        row_off[k] = nx * gy;
        row_wy[k] = 3 * wall_count(gy, ny, G.py);
      }
    }
  }
  // edge column element: tid < 2*PHY -> side = tid / PHY, row = tid % PHY
  int edge_off = -1, edge_cls = 0, edge_ly = 0, edge_col = 0;
  if (tid < 2 * PHY) {
    const int side = tid / PHY;
    edge_ly = tid - side * PHY;
    edge_col = side ? PX + 2 : 1;
    const int gx = halo_index(side ? x0 + PX : x0 - 1, nx, G.px);
    const int gy = halo_index(y0 + edge_ly - 1, ny, G.py);
    if (gx >= 0 && gy >= 0) {
      edge_off = gx + nx * gy;
      edge_cls = wall_count(gx, nx, G.px) + 3 * wall_count(gy, ny, G.py);
    }
  }
  __syncthreads();

  T vr[PROWS][2], vp[PROWS][2], er = T(0), ep = T(0);
  int cur_gz = -1;
  auto issue = [&](int zr) {
    const int gz = halo_index(zr, nz, G.pz);
    cur_gz = gz;
    const unsigned int zoff = gz >= 0 ? plane * (unsigned int)gz : 0u;
#pragma unroll
    for (int k = 0; k < PROWS; k++) {
      vr[k][0] = vr[k][1] = vp[k][0] = vp[k][1] = T(0);
      if (gz >= 0 && row_off[k] >= 0) {
        const unsigned int rowz = zoff + (unsigned int)row_off[k];
        if (pair_full) {
          const unsigned int c = rowz + (unsigned int)gxp;
          const V2 a = *reinterpret_cast<const V2 *>(r + c);
          vr[k][0] = a.x;
          vr[k][1] = a.y;
          if (!first) {
            const V2 b = *reinterpret_cast<const V2 *>(pold + c);
            vp[k][0] = b.x;
            vp[k][1] = b.y;
          }
        } else {
          if (gxa >= 0) {
            vr[k][0] = r[rowz + gxa];
            if (!first) vp[k][0] = pold[rowz + gxa];
          }
          if (gxb >= 0) {
            vr[k][1] = r[rowz + gxb];
            if (!first) vp[k][1] = pold[rowz + gxb];
          }
        }
      }
    }
    er = ep = T(0);
    if (gz >= 0 && edge_off >= 0) {
      const unsigned int c = zoff + (unsigned int)edge_off;
      er = r[c];
      if (!first) ep = pold[c];
    }
  };
  auto commit = [&](int slot, int zr) {
    const int gz = cur_gz;
    const int wz = (gz >= 0) ? 9 * wall_count(gz, nz, G.pz) : 0;
    const bool ownz = (zr >= z0 && zr < z1) && gz >= 0;
    const unsigned int zoff = gz >= 0 ? plane * (unsigned int)gz : 0u;
    if (!xy_walls && wz == 0) {  // interior plane, periodic x/y: Jacobi weight 1
#pragma unroll
      for (int k = 0; k < PROWS; k++) {
        const int ly = ty + 8 * k;
        if (ly >= PHY) continue;
        V2 v;  // slots without a cell hold r = p_old = 0, so they stay 0
        v.x = first ? vr[k][0] : fma(beta, vp[k][0], vr[k][0]);
        v.y = first ? vr[k][1] : fma(beta, vp[k][1], vr[k][1]);
        *reinterpret_cast<V2 *>(&sp[slot][ly][2 + 2 * tx]) = v;
        if (ownz && ly >= 1 && ly <= PY && row_off[k] >= 0 && y0 + ly - 1 < ny && npair > 0) {
          const unsigned int c = zoff + (unsigned int)row_off[k] + (unsigned int)gxp;
          store_own<T, V2>(pnew, x, c, v, vp[k], alpha, lag, pair_full, npair);
        }
      }
    } else {
#pragma unroll
      for (int k = 0; k < PROWS; k++) {
        const int ly = ty + 8 * k;
        if (ly >= PHY) continue;
        V2 v;
        v.x = v.y = T(0);
        if (gz >= 0 && row_off[k] >= 0) {
          const T z0v = vr[k][0] * s_inv[wxp0 + row_wy[k] + wz];
          const T z1v = vr[k][1] * s_inv[wxp1 + row_wy[k] + wz];
          v.x = first ? z0v : fma(beta, vp[k][0], z0v);
          v.y = first ? z1v : fma(beta, vp[k][1], z1v);
        }
        *reinterpret_cast<V2 *>(&sp[slot][ly][2 + 2 * tx]) = v;
        if (ownz && ly >= 1 && ly <= PY && row_off[k] >= 0 && y0 + ly - 1 < ny && npair > 0) {
          const unsigned int c = zoff + (unsigned int)row_off[k] + (unsigned int)gxp;
          store_own<T, V2>(pnew, x, c, v, vp[k], alpha, lag, pair_full, npair);
        }
      }
    }
    if (tid < 2 * PHY) {
      T v = T(0);
      if (gz >= 0 && edge_off >= 0) {
        const int cls = edge_cls + wz;
        const T z = cls ? er * s_inv[cls] : er;
        v = first ? z : fma(beta, ep, z);
      }
      sp[slot][edge_ly][edge_col] = v;
    }
  };

  issue(z0 - 1);
  commit(0, z0 - 1);
  issue(z0);
  commit(1, z0);
  issue(z0 + 1);

  const int gy0 = y0 + ty, gy1 = y0 + ty + 8;
  const bool m0 = npair > 0 && gy0 < ny, m1 = npair > 0 && gy1 < ny;
  const int cy0 = m0 ? 3 * wall_count(gy0, ny, G.py) : 0;
  const int cy1 = m1 ? 3 * wall_count(gy1, ny, G.py) : 0;
  typename Acc<T>::type acc = 0;

  for (int z = z0; z < z1; z++) {
    const int sb = (z - z0) % 3, sc = (z - z0 + 1) % 3, st_ = (z - z0 + 2) % 3;
    commit(st_, z + 1);
    if (z + 2 <= z1) issue(z + 2);
    // own-cell mask of this plane (used after the barrier)
    uint8_t mk[2][2] = {{0, 0}, {0, 0}};
    if (MASK) {
#pragma unroll
      for (int h = 0; h < 2; h++) {
        if (!(h ? m1 : m0)) continue;
        const unsigned int c = plane * (unsigned int)z + (unsigned int)nx * (unsigned int)(h ? gy1 : gy0) + gxp;
        if (pair_full) {
          const uchar2 mm = *reinterpret_cast<const uchar2 *>(mask + c);
          mk[h][0] = mm.x;
          mk[h][1] = mm.y;
        } else {
          mk[h][0] = mask[c];
          if (npair == 2) mk[h][1] = mask[c + 1];
        }
      }
    }
    __syncthreads();
    const int wz = 9 * wall_count(z, nz, G.pz);
    const bool interior = !xy_walls && wz == 0;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      if (!(h ? m1 : m0)) continue;
      const int ly = ty + 1 + 8 * h;
      const int col = 2 + 2 * tx;
      const V2 c = *reinterpret_cast<const V2 *>(&sp[sc][ly][col]);
      const V2 n = *reinterpret_cast<const V2 *>(&sp[sc][ly + 1][col]);
      const V2 s = *reinterpret_cast<const V2 *>(&sp[sc][ly - 1][col]);
      const V2 t = *reinterpret_cast<const V2 *>(&sp[st_][ly][col]);
      const V2 b = *reinterpret_cast<const V2 *>(&sp[sb][ly][col]);
      const T w = sp[sc][ly][col - 1], e = sp[sc][ly][col + 2];
      T a0, a1;
      if (interior) {
        a0 = apply_L0<T, ISO>(G, c.x, c.y, w, n.x, s.x, t.x, b.x, MASK && mk[h][0]);
        a1 = apply_L0<T, ISO>(G, c.y, e, c.x, n.y, s.y, t.y, b.y, MASK && mk[h][1]);
      } else {
        const int cy = (h ? cy1 : cy0) + wz;
        a0 = apply_L<T, ISO>(G, s_dL, wxp0 + cy, c.x, c.y, w, n.x, s.x, t.x, b.x);
        a1 = apply_L<T, ISO>(G, s_dL, wxp1 + cy, c.y, e, c.x, n.y, s.y, t.y, b.y);
      }
      if (MASK) {
        if (mk[h][0]) a0 = T(0);
        if (mk[h][1]) a1 = T(0);
      }
      const unsigned int cc = plane * (unsigned int)z + (unsigned int)nx * (unsigned int)(h ? gy1 : gy0) + gxp;
      if (pair_full) {
        V2 o;
        o.x = a0;
        o.y = a1;
        *reinterpret_cast<V2 *>(Ap + cc) = o;
        acc = fma(c.x, a0, acc);
        acc = fma(c.y, a1, acc);
      } else {
        Ap[cc] = a0;
        acc = fma(c.x, a0, acc);
        if (npair == 2) {
          Ap[cc + 1] = a1;
          acc = fma(c.y, a1, acc);
        }
      }
    }
    __syncthreads();
  }
  double v[1] = {(double)acc}, tot[1];
  const unsigned int nb = gridDim.x * gridDim.y * gridDim.z;
  const unsigned int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  if (last_cta_reduce<1>(v, partials, st, nb, bid, s_red, tot) && tid == 0) {
    st->pAp = tot[0];
    st->alpha = st->rz / tot[0];
    trace_put(st->trace_a, st->trace_n, st->iter, st->alpha);
    st->first = 0;
    st->dlag = 1;
    decide_replacement(st);
  }
}


// ------------------------------------------------------------------ K2 ----

// Jacobi weight minus one of cell c (0 for interior cells)
__device__ __forceinline__ int cell_class(const GeoL &G, unsigned int c) {
  const unsigned int row = fdiv(c, G.mx);
  const unsigned int k = fdiv(c, G.mxy);
  const int i = (int)(c - row * (unsigned)G.nx);
  const int j = (int)(row - k * (unsigned)G.ny);
  return wall_count(i, G.nx, G.px) + 3 * wall_count(j, G.ny, G.py) + 9 * wall_count((int)k, G.nz, G.pz);
}

// 16-byte vectors of the update kernel
template <typename T> struct Vec16;
template <> struct Vec16<float> {
  typedef float4 type;
  static constexpr int E = 4;
};
template <> struct Vec16<double> {
  typedef double2 type;
  static constexpr int E = 2;
};

// vector loads and stores with an L2 policy (FP32); FP64 vectors plain
__device__ __forceinline__ float4 ldv(const float4 *a, unsigned long long pol) { return ld4_pol(a, pol); }
__device__ __forceinline__ double2 ldv(const double2 *a, unsigned long long) { return *a; }
__device__ __forceinline__ void stv(float4 *a, const float4 v, unsigned long long pol) { st4_pol(a, v, pol); }
__device__ __forceinline__ void stv(double2 *a, const double2 v, unsigned long long) { *a = v; }

// r -= alpha Ap on one vector; the new r^2 go into acc (one FMA per cell)
__device__ __forceinline__ void upd_vec(float4 &r, const float4 a, float alpha, float &acc) {
  r.x = fmaf(-alpha, a.x, r.x);
  r.y = fmaf(-alpha, a.y, r.y);
  r.z = fmaf(-alpha, a.z, r.z);
  r.w = fmaf(-alpha, a.w, r.w);
  acc = fmaf(r.x, r.x, acc);
  acc = fmaf(r.y, r.y, acc);
  acc = fmaf(r.z, r.z, acc);
  acc = fmaf(r.w, r.w, acc);
}
__device__ __forceinline__ void upd_vec(double2 &r, const double2 a, double alpha, double &acc) {
  r.x = fma(-alpha, a.x, r.x);
  r.y = fma(-alpha, a.y, r.y);
  acc = fma(r.x, r.x, acc);
  acc = fma(r.y, r.y, acc);
}

// r -= alpha Ap over the vectors [lo, hi) with the sum of r^2; two vectors
// per thread per trip, both loaded before either is used
template <typename T>
__device__ __forceinline__ T upd_range(typename Vec16<T>::type *__restrict__ r4,
                                       const typename Vec16<T>::type *__restrict__ a4, unsigned int lo,
                                       unsigned int hi, unsigned int t0, unsigned int stride, T alpha,
                                       unsigned long long pr, unsigned long long pa) {
  typedef typename Vec16<T>::type V;
  T acc = 0;
  for (unsigned int q = lo + t0; q < hi; q += 2 * stride) {
    const unsigned int q2 = q + stride;
    const bool two = q2 < hi;
    V rv0 = ldv(r4 + q, pr);
    const V av0 = ldv(a4 + q, pa);
    V rv1, av1;
    if (two) {
      rv1 = ldv(r4 + q2, pr);
      av1 = ldv(a4 + q2, pa);
    }
    upd_vec(rv0, av0, alpha, acc);
    stv(r4 + q, rv0, pr);
    if (two) {
      upd_vec(rv1, av1, alpha, acc);
      stv(r4 + q2, rv1, pr);
    }
  }
  return acc;
}

// r -= alpha Ap in the reverse of the search kernel's plane order: the search
// kernel gives each CTA a chunk of kz planes (nzc chunks) and all chunks
// ascend together, so its last planes are the top ones of every chunk.  Here
// virtual plane v = j * nzc + c is plane c kz + kz - 1 - j: the update starts
// on the planes still in L2 and ends on the bottom ones, where the next
// search kernel starts.  Plane vectors pv = 2^pv_shift.  Returns the sums of
// r^2 over interior planes and over the two z-wall planes (non-periodic z).
template <typename T>
__device__ __forceinline__ void upd_range_rev(typename Vec16<T>::type *__restrict__ r4,
                                              const typename Vec16<T>::type *__restrict__ a4, const GeoL &G,
                                              int kz, int nzc, unsigned long long mnzc, int pv_shift,
                                              unsigned int t0, unsigned int stride, T alpha, T &rr, T &wall,
                                              unsigned long long pr, unsigned long long pa) {
  typedef typename Vec16<T>::type V;
  const unsigned int pmask = (1u << pv_shift) - 1u;
  const unsigned int total = ((unsigned int)kz * (unsigned int)nzc) << pv_shift;
  const bool zw = !G.pz;
  // physical vector of virtual vector q (or ~0u past the last plane)
  auto phys = [&](unsigned int q, bool &w) {
    const unsigned int v = q >> pv_shift;
    const unsigned int j = fdiv(v, mnzc);
    const unsigned int c = v - j * (unsigned int)nzc;
    const unsigned int z = c * (unsigned int)kz + (unsigned int)kz - 1u - j;
    w = zw && (z == 0u || z == (unsigned int)G.nz - 1u);
    return z < (unsigned int)G.nz ? (z << pv_shift) | (q & pmask) : ~0u;
  };
  for (unsigned int q = t0; q < total; q += 2 * stride) {
    bool w0, w1 = false;
    const unsigned int p0 = phys(q, w0);
    const unsigned int p1 = q + stride < total ? phys(q + stride, w1) : ~0u;
    V rv0, av0, rv1, av1;
    if (p0 != ~0u) {
      rv0 = ldv(r4 + p0, pr);
      av0 = ldv(a4 + p0, pa);
    }
    if (p1 != ~0u) {
      rv1 = ldv(r4 + p1, pr);
      av1 = ldv(a4 + p1, pa);
    }
    if (p0 != ~0u) {
      T a = 0;
      upd_vec(rv0, av0, alpha, a);
      stv(r4 + p0, rv0, pr);
      if (w0) wall += a;
      else rr += a;
    }
    if (p1 != ~0u) {
      T a = 0;
      upd_vec(rv1, av1, alpha, a);
      stv(r4 + p1, rv1, pr);
      if (w1) wall += a;
      else rr += a;
    }
  }
}

// K2: r -= alpha Ap with (r,z) and (r,r); x += alpha p is left to the next
// search kernel (or the settle / fold kernels), which reads p anyway.
// (r,z) = (r,r) + sum over wall cells of (invL - 1) r^2.  Cells of interior
// planes carry no class arithmetic: with periodic x and y the vectors of the
// two z-wall planes run in loops of their own with one weight each.
template <typename T>
__global__ void __launch_bounds__(FNT) k2_update(const GeoL G, T *__restrict__ r, const T *__restrict__ Ap,
                                                 DevState *st, double *partials, int cond, int kz, int nzc,
                                                 unsigned long long mnzc, int pv_shift, int l2hint) {
  __shared__ T s_dL[27], s_inv[27];
  __shared__ double s_red[2 * FNT / 32];
  pdl_sync();
  if (*(volatile int *)&st->done) return;
  if (cond && *(volatile int *)&st->rep_now) return;  // a checkpoint that replaces the residual
  const T alpha = (T)(*(volatile double *)&st->alpha);
  load_tabs<T>(G, s_dL, s_inv);
  __syncthreads();
  typename Acc<T>::type rr = 0, corr = 0;
  typedef typename Vec16<T>::type V;
  constexpr int E = Vec16<T>::E;
  const unsigned int n = (unsigned int)G.n;
  const unsigned int stride = gridDim.x * FNT;
  const unsigned int t0 = blockIdx.x * FNT + threadIdx.x;
  const unsigned int plane = (unsigned int)G.nx * (unsigned int)G.ny;
  if (G.px && G.py && (plane % E) == 0) {
    // Ap is streamed (evict_first); r keeps the normal priority
    const unsigned long long pr = l2_policy(0), pa = l2_policy(l2hint ? 1 : 0);
    V *r4 = reinterpret_cast<V *>(r);
    const V *a4 = reinterpret_cast<const V *>(Ap);
    const unsigned int pv = plane / E, nv = n / E;
    // vectors [wall_lo, wall_hi) of the interior planes, then the wall planes
    const unsigned int wall_lo = G.pz ? 0u : pv;
    const unsigned int wall_hi = G.pz ? nv : nv - pv;
    if (kz > 0) {  // in the reverse of the search kernel's plane order
      T in = 0, wl = 0;
      upd_range_rev<T>(r4, a4, G, kz, nzc, mnzc, pv_shift, t0, stride, alpha, in, wl, pr, pa);
      const int wc = 9 * (G.nz == 1 ? 2 : 1);
      rr = in + wl;
      if (!G.pz) corr = (s_inv[wc] - T(1)) * wl;
    } else {
    rr = upd_range<T>(r4, a4, wall_lo, wall_hi, t0, stride, alpha, pr, pa);
    if (!G.pz) {
      const int wc = 9 * (G.nz == 1 ? 2 : 1);
      const T w = s_inv[wc] - T(1);
      T t = upd_range<T>(r4, a4, 0, wall_lo, t0, stride, alpha, pr, pa);
      if (G.nz > 1) t += upd_range<T>(r4, a4, wall_hi, nv, t0, stride, alpha, pr, pa);
      rr += t;
      corr = w * t;
    }
    }
  } else {
    // general walls: per-cell class
    for (unsigned int c = t0; c < n; c += stride) {
      const T rn = fma(-alpha, Ap[c], r[c]);
      r[c] = rn;
      rr = fma(rn, rn, rr);
      const int cl = cell_class(G, c);
      if (cl) corr = fma((s_inv[cl] - T(1)) * rn, rn, corr);
    }
  }
  double v[2] = {(double)rr + (double)corr, (double)rr}, tot[2];
  if (last_cta_reduce<2>(v, partials, st, gridDim.x, blockIdx.x, s_red, tot) && threadIdx.x == 0)
    finish_iteration(st, tot[0], tot[1], true);
}

// check: 0 always runs; 1 returns in a finished solve; 2 also returns at a
// checkpoint that keeps the recursive residual
__device__ __forceinline__ bool skip_step(const DevState *st, int check) {
  if (!check) return false;
  if (*(volatile const int *)&st->done) return true;
  return check == 2 && !*(volatile const int *)&st->rep_now;
}

// x += alpha p when x lags (before a residual replacement, a confirmation
// and at the end of a solve).
template <typename T>
__global__ void __launch_bounds__(FNT) k_settle(const GeoL G, T *__restrict__ x, const T *__restrict__ p,
                                                const DevState *st, int check) {
  pdl_sync();
  if (skip_step(st, check)) return;
  if (!*(volatile const int *)&st->dlag) return;
  const T alpha = (T)(*(volatile const double *)&st->alpha);
  const unsigned int n = (unsigned int)G.n;
  for (unsigned int c = blockIdx.x * FNT + threadIdx.x; c < n; c += gridDim.x * FNT) x[c] = fma(alpha, p[c], x[c]);
}

// --------------------------------------------------------------- residual --
__device__ __forceinline__ void resid_finish(DevState *st, const double (&tot)[3], int mode);

// r = bscale rhs - L x on fluid cells, r = 0 (and x = 0 with zero_solid_x) on
// solid cells.  TXT: type of x and rhs, TR: type of r.  Dots in FP64 of the
// stored r: (r,z), (r,r); and (rhs,rhs) of the unscaled rhs.
template <typename TXT, typename TR, bool MASK, bool ISO>
__global__ void __launch_bounds__(FNT, 3) k_resid_s(const GeoL G, TXT *__restrict__ xin, const TXT *__restrict__ rhs,
                                                 TR *__restrict__ rout, const uint8_t *__restrict__ mask,
                                                 DevState *st, double *partials, int kz, int mode, double bscale) {
  __shared__ TXT s_dL[27], s_inv[27];
  __shared__ TXT sp[3][FHY][FHX];
  __shared__ uint8_t sm[3][FHY][FHX + 2];
  __shared__ double s_red[3 * FNT / 32];
  pdl_sync();
  if (mode == 1 && skip_step(st, 2)) return;
  load_tabs<TXT>(G, s_dL, s_inv);
  const int tid = threadIdx.x;
  const int tx = tid & 31, ty = tid >> 5;
  const int x0 = blockIdx.x * FX, y0 = blockIdx.y * FY;
  const int z0 = blockIdx.z * kz, z1 = min(z0 + kz, G.nz);
  const int nx = G.nx, ny = G.ny, nz = G.nz;
  const long long sxy = (long long)nx * ny;
  __syncthreads();
  // The x tile of a plane plus halo is loaded into registers one plane ahead
  // (issue) and written to shared memory the next plane (commit), so the
  // loads are in flight while a plane is computed.  Per element: its offset in
  // a plane (-1 outside a wall) and its places in the two tiles.
  int eoff[FPER], epos[FPER], mpos[FPER];
#pragma unroll
  for (int k = 0; k < FPER; k++) {
    const int e = tid + k * FNT;
    eoff[k] = -1;
    epos[k] = -1;
    mpos[k] = 0;
    if (e < FHE) {
      const int ly = e / FHX, lx = e - ly * FHX;
      epos[k] = e;
      mpos[k] = ly * (FHX + 2) + lx;
      const int hx = halo_index(x0 + lx - 1, nx, G.px), hy = halo_index(y0 + ly - 1, ny, G.py);
      if (hx >= 0 && hy >= 0) eoff[k] = hx + nx * hy;
    }
  }
  TXT pv[FPER];
  uint8_t pm[FPER];
  auto issue = [&](int zr) {
    const int gz = halo_index(zr, nz, G.pz);
#pragma unroll
    for (int k = 0; k < FPER; k++) {
      pv[k] = TXT(0);
      pm[k] = 0;
      if (gz >= 0 && eoff[k] >= 0) {
        const long long c = eoff[k] + sxy * gz;
        if (MASK) pm[k] = mask[c];
        pv[k] = xin[c];
      }
    }
  };
  auto commit = [&](int slot) {
#pragma unroll
    for (int k = 0; k < FPER; k++) {
      if (epos[k] < 0) continue;
      (&sp[slot][0][0])[epos[k]] = pm[k] ? TXT(0) : pv[k];  // solid cells count as x = 0
      (&sm[slot][0][0])[mpos[k]] = pm[k];
    }
  };
  // (r,z) = (r,r) + sum over wall cells of (invL - 1) r^2; (rhs,rhs) only
  // when initialising.  Both are CTA-uniform choices, so the FP64 pipe sees
  // no predicated work on interior planes (FP64 issues at 1/64 of FP32).
  double corr = 0, rr = 0, bb = 0;
  const bool want_bb = mode == 0;
  issue(z0 - 1);
  commit(0);
  issue(z0);
  commit(1);
  issue(z0 + 1);
  const int gx = x0 + tx;
  // rhs of the thread's own cells of a plane, loaded one plane ahead
  auto load_b = [&](int z, TXT (&b)[2]) {
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int gy = y0 + ty + 8 * h;
      b[h] = (gx < nx && gy < ny) ? rhs[gx + (long long)nx * gy + sxy * z] : TXT(0);
    }
  };
  auto cell = [&](auto interior_tag, int sb, int sc, int st_, int z, const TXT (&bz)[2]) {
    constexpr bool INTERIOR = decltype(interior_tag)::value;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int gy = y0 + ty + 8 * h;
      if (gx >= nx || gy >= ny) continue;
      const int ly = ty + 1 + 8 * h, lx = tx + 1;
      const bool mc = MASK && sm[sc][ly][lx] != 0;
      const long long c = gx + (long long)nx * gy + sxy * z;
      const TXT bv = bz[h];
      if (want_bb) bb = fma((double)bv, (double)bv, bb);
      if (mc) {
        rout[c] = TR(0);
        if (mode == 0) xin[c] = TXT(0);
        continue;
      }
      TXT pc = sp[sc][ly][lx];
      TXT pe = sp[sc][ly][lx + 1], pw = sp[sc][ly][lx - 1];
      TXT pn = sp[sc][ly + 1][lx], ps = sp[sc][ly - 1][lx];
      TXT pt = sp[st_][ly][lx], pb = sp[sb][ly][lx];
      const int cls = INTERIOR ? 0 : wall_count(gx, nx, G.px) + 3 * wall_count(gy, ny, G.py) + 9 * wall_count(z, nz, G.pz);
      const TXT a = INTERIOR ? apply_L0<TXT, ISO>(G, pc, pe, pw, pn, ps, pt, pb, false)
                             : apply_L<TXT, ISO>(G, s_dL, cls, pc, pe, pw, pn, ps, pt, pb);
      const TXT rv = fma((TXT)bscale, bv, -a);
      const TR ro = (TR)rv;
      rout[c] = ro;
      const double rd = (double)rv;
      if (INTERIOR) {
        rr = fma(rd, rd, rr);
      } else {
        const double r2 = rd * rd;
        rr += r2;
        if (cls) corr = fma((double)s_inv[cls] - 1.0, r2, corr);
      }
    }
  };
  TXT bcur[2] = {TXT(0), TXT(0)}, bnext[2] = {TXT(0), TXT(0)};
  if (z0 < z1) load_b(z0, bcur);
  for (int z = z0; z < z1; z++) {
    const int sb = (z - z0) % 3, sc = (z - z0 + 1) % 3, st_ = (z - z0 + 2) % 3;
    commit(st_);  // plane z + 1, loaded during the previous plane
    if (z + 2 <= z1) issue(z + 2);
    if (z + 1 < z1) load_b(z + 1, bnext);
    __syncthreads();
    if (G.px && G.py && wall_count(z, nz, G.pz) == 0) cell(std::true_type(), sb, sc, st_, z, bcur);
    else cell(std::false_type(), sb, sc, st_, z, bcur);
    __syncthreads();
    bcur[0] = bnext[0];
    bcur[1] = bnext[1];
  }
  double v[3] = {rr + corr, rr, bb}, tot[3];
  const unsigned int nb = gridDim.x * gridDim.y * gridDim.z;
  const unsigned int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  if (last_cta_reduce<3>(v, partials, st, nb, bid, s_red, tot) && tid == 0) resid_finish(st, tot, mode);
}

// The device state after a residual: init (mode 0), replacement at a
// checkpoint (1) or confirmation of a recursive convergence (2).  tot: (r,z),
// (r,r), (rhs,rhs).
__device__ __forceinline__ void resid_finish(DevState *st, const double (&tot)[3], int mode) {
  {
    const double rz1 = tot[0], rr1 = tot[1];
    if (mode == 0) {  // init: thresholds from (rhs,rhs) of the unscaled rhs
      st->bb = tot[2];
      st->tol2bb = st->tol2bb * tot[2];  // host stores tol^2 * (S or S^2) here
      st->rz = rz1;
      st->rz_last = rz1;
      st->rr = rr1;
      st->iter = 0;
      st->fq = 0;
      st->first = 1;
      st->dlag = 0;
      st->replacements = 0;
      st->rr_ref = rr1;
      st->last_rep = 0;
      st->rep_now = 0;
      if (tot[2] < st->tiny) st->done = DONE_TINY;  // src/cuda_solver.cu:178-190
      else if (st->stop == 1 && rr1 <= st->tol2bb) st->done = DONE_CONVERGED;
      else st->done = RUNNING;
    } else if (mode == 1) {
      st->replacements += 1;
      st->dlag = 0;  // x was settled before this residual
      finish_iteration(st, rz1, rr1, true);
      st->rr_ref = rr1;
      st->last_rep = st->iter;
    } else {  // confirm
      st->replacements += 1;
      st->dlag = 0;
      st->rr_ref = rr1;
      st->last_rep = st->iter;
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

// ------------------------------------------------- float-float residual --
// r = bscale rhs - L x for FP64 x and rhs into an FP32 r, evaluated in
// float-float arithmetic on the FP32 pipe (GB300 issues FP64 at 1/64 of FP32);
// an option beside the FP64 residual kernel, not its default replacement.
// A value is an unevaluated sum hi + lo of two floats (about 48 bits); the
// error-free transformations are Knuth's two-sum and the FMA two-product
// (Dekker's product with a fused multiply-add), renormalised with
// Dekker's fast two-sum.  Each FP64 input is split once, when its tile is
// loaded (one FP64 subtraction).  The error of L x is ~2^-48 |x|, far below
// what the FP32 residual keeps.  Dots are summed in FP32 per thread and in
// FP64 across threads, as the iteration kernels do.  Same tiles, masking,
// wall classes and state updates as k_resid_s.
struct ff {
  float hi, lo;
};

__device__ __forceinline__ ff ff_split(double v) {
  const float h = __double2float_rn(v);
  return ff{h, __double2float_rn(v - (double)h)};
}

__device__ __forceinline__ ff ff_fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return ff{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ ff ff_add(ff a, ff b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  return ff_fast_two_sum(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.hi, -a.lo}; }

__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  const float p = __fmul_rn(a.hi, b.hi);
  const float e = __fmaf_rn(a.hi, b.hi, -p);
  return ff_fast_two_sum(p, __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e)));
}

template <bool MASK, bool ISO>
__global__ void __launch_bounds__(FNT) k_resid_ff(const GeoL G, double *__restrict__ xin,
                                                  const double *__restrict__ rhs, float *__restrict__ rout,
                                                  const uint8_t *__restrict__ mask, DevState *st, double *partials,
                                                  int kz, int mode, double bscale) {
  __shared__ ff s_dL[27];
  __shared__ float s_inv[27];
  __shared__ ff sp[3][FHY][FHX];
  __shared__ uint8_t sm[3][FHY][FHX + 2];
  __shared__ double s_red[3 * FNT / 32];
  pdl_sync();
  if (mode == 1 && skip_step(st, 2)) return;
  for (int e = threadIdx.x; e < 27; e += blockDim.x) {
    s_dL[e] = ff_split(G.dL[e]);
    s_inv[e] = G.finvL[e];
  }
  const ff ax = ff_split(G.ax), ay = ff_split(G.ay), az = ff_split(G.az), bs = ff_split(bscale);
  const int tid = threadIdx.x;
  const int tx = tid & 31, ty = tid >> 5;
  const int x0 = blockIdx.x * FX, y0 = blockIdx.y * FY;
  const int z0 = blockIdx.z * kz, z1 = min(z0 + kz, G.nz);
  const int nx = G.nx, ny = G.ny, nz = G.nz;
  const long long sxy = (long long)nx * ny;
  __syncthreads();
  auto load_plane = [&](int slot, int zr) {
    const int gz = halo_index(zr, nz, G.pz);
    for (int e = tid; e < FHE; e += FNT) {
      const int ly = e / FHX, lx = e - ly * FHX;
      const int gx = halo_index(x0 + lx - 1, nx, G.px), gy = halo_index(y0 + ly - 1, ny, G.py);
      ff val = ff{0.f, 0.f};
      uint8_t m = 0;
      if (gz >= 0 && gx >= 0 && gy >= 0) {
        const long long c = gx + (long long)nx * gy + sxy * gz;
        if (MASK) m = mask[c];
        if (!m) val = ff_split(xin[c]);  // solid cells count as x = 0
      }
      sp[slot][ly][lx] = val;
      sm[slot][ly][lx] = m;
    }
  };
  float corr = 0.f, rr = 0.f, bb = 0.f;
  const bool want_bb = mode == 0;
  load_plane(0, z0 - 1);
  load_plane(1, z0);
  const int gx = x0 + tx;
  auto cell = [&](auto interior_tag, int sb, int sc, int st_, int z) {
    constexpr bool INTERIOR = decltype(interior_tag)::value;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int gy = y0 + ty + 8 * h;
      if (gx >= nx || gy >= ny) continue;
      const int ly = ty + 1 + 8 * h, lx = tx + 1;
      const bool mc = MASK && sm[sc][ly][lx] != 0;
      const long long c = gx + (long long)nx * gy + sxy * z;
      const double bvd = rhs[c];
      const ff bv = ff_split(bvd);
      if (want_bb) bb = fmaf(bv.hi, bv.hi, bb);
      if (mc) {
        rout[c] = 0.f;
        if (mode == 0) xin[c] = 0.0;
        continue;
      }
      const ff pc = sp[sc][ly][lx];
      const ff pe = sp[sc][ly][lx + 1], pw = sp[sc][ly][lx - 1];
      const ff pn = sp[sc][ly + 1][lx], ps = sp[sc][ly - 1][lx];
      const ff pt = sp[st_][ly][lx], pb = sp[sb][ly][lx];
      const int cls = INTERIOR ? 0 : wall_count(gx, nx, G.px) + 3 * wall_count(gy, ny, G.py) + 9 * wall_count(z, nz, G.pz);
      // a = L x at the cell (apply_L's formula, in float-float)
      ff s;
      if (ISO) {
        s = ff_mul(ax, ff_add(ff_add(ff_add(pe, pw), ff_add(pn, ps)), ff_add(pt, pb)));
      } else {
        s = ff_add(ff_add(ff_mul(ax, ff_add(pe, pw)), ff_mul(ay, ff_add(pn, ps))), ff_mul(az, ff_add(pt, pb)));
      }
      const ff d = cls ? ff_mul(s_dL[cls], pc) : pc;
      const ff a = ff_add(d, ff_neg(s));
      const ff r = ff_add(ff_mul(bs, bv), ff_neg(a));
      const float rv = __fadd_rn(r.hi, r.lo);
      rout[c] = rv;
      const float r2 = rv * rv;
      rr += r2;
      if (!INTERIOR && cls) corr = fmaf(s_inv[cls] - 1.f, r2, corr);
    }
  };
  for (int z = z0; z < z1; z++) {
    const int sb = (z - z0) % 3, sc = (z - z0 + 1) % 3, st_ = (z - z0 + 2) % 3;
    load_plane(st_, z + 1);
    __syncthreads();
    if (G.px && G.py && wall_count(z, nz, G.pz) == 0) cell(std::true_type(), sb, sc, st_, z);
    else cell(std::false_type(), sb, sc, st_, z);
    __syncthreads();
  }
  double v[3] = {(double)rr + (double)corr, (double)rr, (double)bb}, tot[3];
  const unsigned int nb = gridDim.x * gridDim.y * gridDim.z;
  const unsigned int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  if (last_cta_reduce<3>(v, partials, st, nb, bid, s_red, tot) && tid == 0) resid_finish(st, tot, mode);
}

}  // namespace bbpp
