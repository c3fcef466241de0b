// bbpp_conv_tc.cuh -- forward 3x3x3 convolution on the 5th-generation tensor
// cores: tcgen05.mma with the A operand in tensor memory, FP32 accumulators in
// tensor memory, operands staged by TMA.  Selected by BBPP_CONV_TC=1 (or
// bbpp_conv3_tc_config(1, ...)); the default forward kernel is k_conv3_tx
// (bbpp_conv_tx.cuh), which needs a third of the MMAs.  The shared helpers
// (descriptors, bounded waits, TMA, tensor-memory loads) are used by both.
//
// Implicit GEMM, input-row stationary.  A CTA works on 128-voxel x blocks of
// TYR output rows and marches in z.  Per input plane and 16-channel chunk the
// producer warp stages, by TMA, the TYR + 2 input rows of the block (each row
// 144 voxels, x0-8 .. x0+135, as two 8-channel planes, so that eight
// consecutive voxels form one 8 x 16-byte core matrix) and the chunk's weights
// of all 27 taps.  For every staged row the MMA thread copies the three
// x-shifted 128 x 16 A tiles (first voxel x0-1, x0, x0+1) into tensor memory
// with tcgen05.cp -- a descriptor that starts one voxel later is the shift --
// and issues one M = 128, N = COUT, K = 16 MMA per (dx, dy, dz) tap that lands
// in the tile: input row (y, z) feeds output rows y - dy + 1 of output planes
// z - dz + 1.  Each A tile is read from shared memory once and serves up to
// nine taps, so the MMAs themselves read only the small weight tile.
//
// Accumulators: a ring of NACC output planes, TYR x COUT FP32 columns each.
// An output plane is complete after input plane z + 1; the MMA thread commits
// it to the epilogue warpgroup, which reads it with tcgen05.ld, adds the
// bias, applies the ReLU, stores BF16 channels-last and hands the slot back.
// CTAs are persistent: each takes a contiguous run of (volume, y block,
// x block, z) plane units and marches through it in segments.
//
// Roles (192 threads): warp 0 = TMA producer (lane 0 issues the copies; the
// lanes patch the periodic x wrap: voxels x0-1 and x0+128 of an edge block
// come from the far end of the row by plain loads, into slots the tensor
// copies leave alone), warp 1 = MMA issuer (one thread), warps 2-5 =
// epilogue (warp w reads tensor-memory lanes 32 (w mod 4) ..).
//
// Descriptors (shared-memory matrix descriptor, no swizzle, K-major): start
// >> 4, leading byte offset = the step between the two 8-channel core
// matrices, stride byte offset = 128 (the step between 8-voxel groups),
// version 1.  Instruction descriptor: FP32 accumulate, BF16 A and B, N >> 3,
// M >> 4.  A tcgen05.cp followed by MMAs of the same thread runs in issue
// order; an MMA followed by a tcgen05.cp into the columns it reads does not,
// so an A slot group is refilled only after a commit of the MMAs that read it.
//
// Every mbarrier wait is bounded (one second); a wait that runs out marks the
// CTA failed, every role leaves its loop, the producer and the MMA thread
// drain what they issued (again bounded), tensor memory is freed and the
// caller's error word is set.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include "bbpp_conv.cuh"

namespace bbnet {

constexpr int TM_THREADS = 192;
constexpr int TM_NACC = 4;           // output planes in flight in tensor memory
constexpr int TM_NAG = 4;            // A slot groups (three 8-column slots each)
constexpr int TM_NST = 4;            // shared-memory stages
constexpr int TM_RS = 144 * 16;      // bytes of one staged row in one 8-channel plane
constexpr int TM_TMEM_COLS = 512;

template <int COUT>
__host__ __device__ constexpr int tm_tyr() {
  return COUT <= 16 ? 4 : 3;
}
template <int COUT>
__host__ __device__ constexpr int tm_plane_bytes() {  // one 8-channel plane of a stage's rows
  return (tm_tyr<COUT>() + 2) * TM_RS;
}
template <int COUT>
__host__ __device__ constexpr int tm_wbytes() {  // weights of one 16-channel chunk
  return 27 * COUT * 32;
}
template <int CIN, int COUT>
__host__ __device__ constexpr int tm_stage_bytes() {
  return 2 * tm_plane_bytes<COUT>() + (CIN > 16 ? tm_wbytes<COUT>() : 0);
}
template <int CIN, int COUT>
__host__ __device__ constexpr int tm_smem() {
  return TM_NST * tm_stage_bytes<CIN, COUT>() + (CIN > 16 ? 0 : tm_wbytes<COUT>()) + 1024;
}

// Tensor maps of one launch.  Activations: 5-D (channel, x, y, z, volume)
// BF16, row boxes {8, W, 1, 1, 1} for W = 144 (no wrapped side), 136 (one
// side wrapped) and 128 (both sides), and one box {8, 144, TYR + 2, 1, 1} of
// all staged rows (its rows land 144 voxels apart, the staged pitch).
// Weights: 3-D (cin, cout, tap), box {8, COUT, 27}.
struct TmMaps {
  CUtensorMap rows, row[3];
  CUtensorMap w;
};

struct TmGeo {
  int nxb, nyb;     // x blocks (nx / 128), y blocks
  long long units;  // nb * nyb * nxb * nz plane units
};

__device__ __forceinline__ uint64_t tm_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

__device__ __forceinline__ bool tm_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred q;\n\tmbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n\tselp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}

// wait for the phase with this parity; false after one second
__device__ __forceinline__ bool tm_wait(uint32_t bar, uint32_t parity) {
  if (tm_try_wait(bar, parity)) return true;
  unsigned long long t0;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  for (uint32_t k = 1;; k++) {
    if (tm_try_wait(bar, parity)) return true;
    if ((k & 63u) == 0) {
      unsigned long long t;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
      if (t - t0 > 1000000000ull) return false;
    }
  }
}

__device__ __forceinline__ void tm_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tm_tma5(uint32_t dst, const CUtensorMap *map, uint32_t bar, int c0, int c1, int c2,
                                        int c3, int c4) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5, %6, "
      "%7}], [%2];" ::"r"(dst),
      "l"(map), "r"(bar), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4)
      : "memory");
}

__device__ __forceinline__ void tm_tma3(uint32_t dst, const CUtensorMap *map, uint32_t bar, int c0, int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], "
      "[%2];" ::"r"(dst),
      "l"(map), "r"(bar), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}

// One segment of a CTA's plane units: volume vb, block (xb, yb), output planes [zs, ze).
struct TmSeg {
  int vb, xb, yb, zs, ze;
};

__device__ __forceinline__ TmSeg tm_seg(long long u, long long u1, int nz, const TmGeo &g) {
  const long long t = u / nz;
  TmSeg s;
  s.zs = (int)(u - t * nz);
  s.ze = (int)min((long long)nz, s.zs + (u1 - u));
  s.xb = (int)(t % g.nxb);
  const long long t2 = t / g.nxb;
  s.yb = (int)(t2 % g.nyb);
  s.vb = (int)(t2 / g.nyb);
  return s;
}

template <int N>
__device__ __forceinline__ void tm_ld(uint32_t taddr, float (&v)[N]);

template <>
__device__ __forceinline__ void tm_ld<16>(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

template <>
__device__ __forceinline__ void tm_ld<32>(uint32_t taddr, float (&v)[32]) {
  float a[16], b[16];
  tm_ld<16>(taddr, a);
  tm_ld<16>(taddr + 16, b);
#pragma unroll
  for (int i = 0; i < 16; i++) {
    v[i] = a[i];
    v[16 + i] = b[i];
  }
}

// Requirements (checked by the launcher): nx % 128 == 0; ldi, ci_off, ldo,
// co_off multiples of 8; in, w and out 16-byte aligned.
template <int CIN, int COUT>
__global__ void __launch_bounds__(TM_THREADS, 1)
    k_conv3_tm(const ConvArgs a, const __grid_constant__ TmMaps M, const TmGeo g, int *err) {
  static_assert(CIN % 16 == 0 && (COUT == 16 || COUT == 32), "16-channel input chunks, 16 or 32 outputs");
  constexpr int NCH = CIN / 16;
  constexpr int TYR = tm_tyr<COUT>();
  constexpr int ROWS = TYR + 2;
  constexpr int PB = tm_plane_bytes<COUT>();
  constexpr int WB = tm_wbytes<COUT>();
  constexpr int WPB = WB / 2;  // one 8-channel plane of the weights
  constexpr int STAGE = tm_stage_bytes<CIN, COUT>();
  constexpr int ACC_COLS = TYR * COUT;  // one output plane
  constexpr int A_BASE = TM_NACC * ACC_COLS;
  static_assert(A_BASE + TM_NAG * 24 <= TM_TMEM_COLS, "tensor memory columns");
  static_assert(2 * ROWS <= 16, "one lane per wrapped voxel and side");
  constexpr uint32_t IDESC =
      (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(COUT >> 3) << 17) | ((128u >> 4) << 24);

  extern __shared__ unsigned char tm_raw[];
  __shared__ __align__(8) unsigned long long s_full[TM_NST], s_ready[TM_NST], s_empty[TM_NST];
  __shared__ __align__(8) unsigned long long s_abar[TM_NAG], s_accf[TM_NACC], s_acce[TM_NACC], s_wbar, s_fin;
  __shared__ uint32_t s_tmem;
  __shared__ int s_fail;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t raw = smem_u32(tm_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;  // stages, then the fixed weights
  unsigned char *const gbase = tm_raw + (base - raw);
  const uint32_t wfix = base + TM_NST * STAGE;
  const long long u0 = (long long)blockIdx.x * g.units / gridDim.x;
  const long long u1 = (long long)(blockIdx.x + 1) * g.units / gridDim.x;
  const int nx = a.nx, ny = a.ny, nz = a.nz;

  if (tid == 0) {
    s_fail = 0;
    for (int i = 0; i < TM_NST; i++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_full[i])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_ready[i])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_empty[i])));
    }
    for (int i = 0; i < TM_NAG; i++) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_abar[i])));
    for (int i = 0; i < TM_NACC; i++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_accf[i])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 128;" ::"r"(smem_u32(&s_acce[i])));
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_wbar)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_fin)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                 "r"(TM_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = s_tmem;

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    if (lane == 0 && NCH == 1) {
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&s_wbar)), "r"(WB)
                   : "memory");
      tm_tma3(wfix, &M.w, smem_u32(&s_wbar), 0, 0, 0);
      tm_tma3(wfix + WPB, &M.w, smem_u32(&s_wbar), 8, 0, 0);
    }
    // lane -> one wrapped voxel of an item: side (0 west, 1 east), staged row, channel plane
    const int side = lane / (2 * ROWS), rem = lane - side * 2 * ROWS;
    const int wr = rem >> 1, wkp = rem & 1;
    struct Wrap {
      uint4 v;
      uint32_t dst;
      bool on;
    };
    auto wrap_load = [&](const TmSeg &s, int zi, int c) {
      Wrap w;
      w.on = false;
      w.v = make_uint4(0u, 0u, 0u, 0u);
      w.dst = 0;
      const int x0 = s.xb * 128;
      if (!a.px || side > 1 || (side == 0 ? x0 != 0 : x0 + 128 != nx)) return w;
      w.on = true;
      w.dst = (uint32_t)(wkp * PB + wr * TM_RS + (side == 0 ? 7 : 136) * 16);
      int gy = s.yb * TYR - 1 + wr, gz = zi;
      const int gx = side == 0 ? nx - 1 : 0;
      if (pad_axis(gy, ny, a.py) && pad_axis(gz, nz, a.pz))
        w.v = *reinterpret_cast<const uint4 *>(a.in + ((((long long)s.vb * nz + gz) * ny + gy) * nx + gx) * a.ldi +
                                               a.ci_off + 16 * c + 8 * wkp);
      return w;
    };
    long long k = 0;  // items issued
    Wrap cur;
    cur.on = false;
    bool have = false, bad = false;
    for (long long u = u0; u < u1 && !bad;) {
      const TmSeg s = tm_seg(u, u1, nz, g);
      u += s.ze - s.zs;
      const int x0 = s.xb * 128, y0 = s.yb * TYR;
      const bool ww = a.px && x0 == 0, ew = a.px && x0 + 128 == nx;
      const int wi = (ww && ew) ? 2 : ((ww || ew) ? 1 : 0);
      const int wbox = wi == 2 ? 128 : (wi == 1 ? 136 : 144);
      const int xs = ww ? x0 : x0 - 8;             // first voxel copied
      const uint32_t xoff = ww ? 8u * 16u : 0u;    // its slot
      // one box for all rows lands them at a pitch of wbox voxels: only the
      // full 144-voxel box matches the staged row pitch
      const bool per_row = wbox != 144 || (a.py && (y0 == 0 || y0 + TYR >= ny));
      const uint32_t bytes = (uint32_t)(2 * ROWS * wbox * 16 + (NCH > 1 ? WB : 0));
      for (int zi = s.zs - 1; zi <= s.ze && !bad; zi++) {
        for (int c = 0; c < NCH; c++) {
          const int slot = (int)(k % TM_NST);
          const uint32_t sb = base + slot * STAGE;
          bool ok = k < TM_NST || tm_wait(smem_u32(&s_empty[slot]), (uint32_t)((k / TM_NST) - 1) & 1u);
          if (!__all_sync(0xffffffffu, ok)) {
            bad = true;
            break;
          }
          if (!have) cur = wrap_load(s, zi, c);
          if (lane == 0) {
            const uint32_t fb = smem_u32(&s_full[slot]);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fb), "r"(bytes) : "memory");
            const int gz = a.pz ? ((zi % nz) + nz) % nz : zi;  // else a plane outside reads the zero fill
            const int ch = a.ci_off + 16 * c;
            for (int kp = 0; kp < 2; kp++) {
              const uint32_t pb = sb + kp * PB + xoff;
              if (!per_row) {
                tm_tma5(pb, &M.rows, fb, ch + 8 * kp, xs, y0 - 1, gz, s.vb);
              } else {
                for (int r = 0; r < ROWS; r++) {
                  const int gy = ((y0 - 1 + r) % ny + ny) % ny;
                  tm_tma5(pb + r * TM_RS, &M.row[wi], fb, ch + 8 * kp, xs, gy, gz, s.vb);
                }
              }
            }
            if (NCH > 1) {
              tm_tma3(sb + 2 * PB, &M.w, fb, 16 * c, 0, 0);
              tm_tma3(sb + 2 * PB + WPB, &M.w, fb, 16 * c + 8, 0, 0);
            }
          }
          k++;
          // the next item's wrapped voxels are loaded before this item's are stored
          const bool more = zi < s.ze || c + 1 < NCH;
          Wrap nxt = cur;
          if (more) nxt = wrap_load(s, c + 1 < NCH ? zi : zi + 1, c + 1 < NCH ? c + 1 : 0);
          if (cur.on) *reinterpret_cast<uint4 *>(gbase + (sb - base) + cur.dst) = cur.v;
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          __syncwarp();
          if (lane == 0)
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&s_ready[slot])) : "memory");
          cur = nxt;
          have = more;
        }
      }
    }
    if (bad && lane == 0) atomicExch(&s_fail, 1);
    // drain: the copies of the last stages issued land before the CTA exits
    for (long long j = (k > TM_NST ? k - TM_NST : 0); j < k; j++)
      tm_wait(smem_u32(&s_full[(int)(j % TM_NST)]), (uint32_t)(j / TM_NST) & 1u);
    if (NCH == 1) tm_wait(smem_u32(&s_wbar), 0);
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      bool bad = NCH == 1 && !tm_wait(smem_u32(&s_wbar), 0);
      bool issued = false;
      long long k = 0, q0 = 0, arow = 0;  // items, output planes before this segment, staged rows used
      for (long long u = u0; u < u1 && !bad;) {
        const TmSeg s = tm_seg(u, u1, nz, g);
        u += s.ze - s.zs;
        for (int zi = s.zs - 1; zi <= s.ze && !bad; zi++) {
          // output plane zi + 1 starts here: its accumulator slot must have been drained
          if (zi + 1 < s.ze) {
            const long long q = q0 + (zi + 1 - s.zs);
            if (q >= TM_NACC &&
                !tm_wait(smem_u32(&s_acce[(int)(q % TM_NACC)]), (uint32_t)((q / TM_NACC) - 1) & 1u)) {
              bad = true;
              break;
            }
          }
          for (int c = 0; c < NCH && !bad; c++, k++) {
            const int slot = (int)(k % TM_NST);
            const uint32_t par = (uint32_t)(k / TM_NST) & 1u;
            if (!tm_wait(smem_u32(&s_full[slot]), par) || !tm_wait(smem_u32(&s_ready[slot]), par)) {
              bad = true;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sb = base + slot * STAGE;
            const uint64_t bd0 = tm_desc(NCH > 1 ? sb + 2 * PB : wfix, WPB, 128);
            for (int r = 0; r < ROWS; r++, arow++) {
              const int ag = (int)(arow % TM_NAG);
              if (arow >= TM_NAG && !tm_wait(smem_u32(&s_abar[ag]), (uint32_t)((arow / TM_NAG) - 1) & 1u)) {
                bad = true;
                break;
              }
              asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
              const uint32_t aslot = tmem + A_BASE + ag * 24;
              const uint64_t ad0 = tm_desc(sb + r * TM_RS + 7 * 16, PB, 128);
#pragma unroll
              for (int dx = 0; dx < 3; dx++)
                asm volatile("tcgen05.cp.cta_group::1.128x256b [%0], %1;" ::"r"(aslot + 8 * dx),
                             "l"(ad0 + (uint64_t)dx)
                             : "memory");
#pragma unroll
              for (int dz = 0; dz < 3; dz++) {
                const int zo = zi + 1 - dz;
                if (zo < s.zs || zo >= s.ze) continue;
                const uint32_t acc0 = tmem + (uint32_t)(((q0 + zo - s.zs) % TM_NACC) * ACC_COLS);
#pragma unroll
                for (int dy = 0; dy < 3; dy++) {
                  const int ty = r - dy;
                  if (ty < 0 || ty >= TYR) continue;
#pragma unroll
                  for (int dx = 0; dx < 3; dx++) {
                    const int tap = dz * 9 + dy * 3 + dx;
                    const uint32_t en = (c == 0 && dz == 0 && dy == 0 && dx == 0) ? 0u : 1u;
                    asm volatile(
                        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(acc0 + ty * COUT),
                        "r"(aslot + 8 * dx), "l"(bd0 + (uint64_t)((tap * COUT * 16) >> 4)), "r"(IDESC), "r"(en)
                        : "memory");
                  }
                }
              }
              tm_commit(smem_u32(&s_abar[ag]));
              issued = true;
            }
            if (bad) break;
            tm_commit(smem_u32(&s_empty[slot]));
          }
          if (bad) break;
          // output plane zi - 1 is complete
          if (zi - 1 >= s.zs) tm_commit(smem_u32(&s_accf[(int)((q0 + zi - 1 - s.zs) % TM_NACC)]));
        }
        q0 += s.ze - s.zs;
      }
      if (bad) atomicExch(&s_fail, 1);
      // drain: every MMA and copy issued has finished before tensor memory is freed
      if (issued) {
        tm_commit(smem_u32(&s_fin));
        tm_wait(smem_u32(&s_fin), 0);
      }
    }
  } else {
    // ------------------------------------------------------------ epilogue
    const int quarter = warp & 3;
    const uint32_t lrow = (uint32_t)(quarter * 32) << 16;
    float bias[COUT];
#pragma unroll
    for (int i = 0; i < COUT; i++) bias[i] = a.bias ? a.bias[i] : 0.f;
    long long q = 0;
    bool bad = false;
    for (long long u = u0; u < u1 && !bad;) {
      const TmSeg s = tm_seg(u, u1, nz, g);
      u += s.ze - s.zs;
      const int x = s.xb * 128 + quarter * 32 + lane;
      const int y0 = s.yb * TYR;
      for (int zo = s.zs; zo < s.ze; zo++, q++) {
        const int as = (int)(q % TM_NACC);
        const bool ok = tm_wait(smem_u32(&s_accf[as]), (uint32_t)(q / TM_NACC) & 1u);
        if (!__all_sync(0xffffffffu, ok)) {
          bad = true;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        bf16 *const oplane = a.out + ((long long)s.vb * nz + zo) * ny * (long long)nx * a.ldo + a.co_off;
#pragma unroll 1
        for (int ty = 0; ty < TYR; ty++) {
          float v[COUT];
          tm_ld<COUT>(tmem + lrow + (uint32_t)(as * ACC_COLS + ty * COUT), v);  // warp-collective
          const int y = y0 + ty;
          if (y >= ny) continue;
          bf16 *o = oplane + ((long long)y * nx + x) * a.ldo;
#pragma unroll
          for (int ch = 0; ch < COUT; ch += 8) {
            uint4 pk;
            __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(&pk);
#pragma unroll
            for (int i = 0; i < 4; i++) {
              float f0 = v[ch + 2 * i] + bias[ch + 2 * i], f1 = v[ch + 2 * i + 1] + bias[ch + 2 * i + 1];
              if (a.relu) {
                f0 = fmaxf(f0, 0.f);
                f1 = fmaxf(f1, 0.f);
              }
              h[i] = __floats2bfloat162_rn(f0, f1);
            }
            *reinterpret_cast<uint4 *>(o + ch) = pk;
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&s_acce[as])) : "memory");
      }
    }
    if (bad && lane == 0) atomicExch(&s_fail, 1);
  }

  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TM_TMEM_COLS));
  if (tid == 0 && s_fail) atomicExch(err, 1);
}

}  // namespace bbnet
