// bbpp_conv_tx.cuh -- forward 3x3x3 convolution on tcgen05 with the three
// x-taps stacked in N, for rows of 128 or 256 voxels.
//
// A tcgen05.mma of M = 128 and K = 16 costs about the same time for every N
// up to 256 on this part, so an implicit GEMM with N = COUT (16 or 32) output
// channels wastes most of each instruction.  Here one MMA serves the three
// x-taps of a (dy, dz) pair at once: A is an input row as it is (128 voxels x
// 16 channels, straight from shared memory), B is the three taps' weights
// stacked (N = 3 COUT: the layout the weights already have, taps dx = 0, 1, 2
// of one (dy, dz) being consecutive), so
//   D[v][dx COUT + c] = sum_k in[v][k] W[dz][dy][dx][c][k]
// holds the contribution of input voxel v through tap dx, which belongs to
// output voxel v + 1 - dx.  The epilogue completes the shift:
//   out[u] = D[u-1][0:COUT] + D[u][COUT:2COUT] + D[u+1][2COUT:3COUT]
// with warp shuffles and, across warps, 128-voxel blocks and the periodic
// wrap, a small exchange of edge values in shared memory.  A CTA spans whole
// x-rows (NXB blocks of 128 voxels), so no x halo is staged or patched.
//
// Otherwise as the tensor-memory layout of a persistent, input-row-stationary
// z-march: all weights stay in shared memory for the whole launch (one
// 16-channel chunk after the other); the producer warp stages, per input plane
// and 16-channel chunk, the TYR + 2 input rows of the tile (two 8-channel
// planes; eight consecutive voxels form one 8 x 16-byte core matrix); one thread
// issues, per staged row and block, one MMA per (dy, dz) that lands in the
// tile; a ring of NACC output planes of accumulators (TYR x NXB x 3 COUT FP32
// columns each) hands complete planes to the epilogue warpgroup.  Every
// mbarrier wait is bounded (one second); a wait that runs out marks the CTA
// failed, the roles leave their loops, what was issued is drained (bounded),
// tensor memory is freed and the caller's error word is set.
#pragma once

#include "bbpp_conv_tc.cuh"

namespace bbnet {

constexpr int TX_THREADS = 192;
constexpr int TX_NACC = 4;  // output planes in flight in tensor memory
constexpr int TX_NST = 4;   // shared-memory stages
constexpr int TX_TMEM_COLS = 512;

template <int COUT, int NXB>
__host__ __device__ constexpr int tx_tyr() {  // output rows per tile
  return NXB * COUT <= 16 ? 2 : 1;
}
template <int COUT>
__host__ __device__ constexpr int tx_accn() {  // columns of one accumulator (3 COUT, padded to a power of two)
  return 3 * COUT <= 64 ? 64 : 128;
}
template <int COUT, int NXB>
__host__ __device__ constexpr int tx_acc_cols() {  // tensor-memory columns of one output plane
  return tx_tyr<COUT, NXB>() * NXB * tx_accn<COUT>();
}
template <int COUT, int NXB>
__host__ __device__ constexpr int tx_plane_bytes() {  // one 8-channel plane of a stage's rows
  return (tx_tyr<COUT, NXB>() + 2) * NXB * 128 * 16;
}
template <int COUT, int NXB>
__host__ __device__ constexpr int tx_stage_bytes() {  // one 16-channel chunk of the staged rows
  return 2 * tx_plane_bytes<COUT, NXB>();
}
template <int CIN, int COUT, int NXB>
__host__ __device__ constexpr int tx_smem() {  // the stages, then all weights, resident
  return TX_NST * tx_stage_bytes<COUT, NXB>() + (CIN / 16) * tm_wbytes<COUT>() + 1024;
}

// Tensor maps of one launch: activations 5-D (channel, x, y, z, volume) BF16
// with boxes {8, nx, TYR + 2, 1, 1} (all rows) and {8, nx, 1, 1, 1} (one row,
// for a wrapped y halo); weights 3-D (cin, cout, tap), box {8, COUT, 27}.
struct TxMaps {
  CUtensorMap rows, row, w;
};

// first input channel of 8-channel plane kp of 16-channel chunk c in the weights
__device__ __forceinline__ int tx_wch(int c, int kp) { return 16 * c + 8 * kp; }

struct TxGeo {
  int nyb;          // y blocks
  long long units;  // nb * nyb * nz plane units
};

// One segment of a CTA's plane units: volume vb, y block yb, output planes [zs, ze).
struct TxSeg {
  int vb, yb, zs, ze;
};

__device__ __forceinline__ TxSeg tx_seg(long long u, long long u1, int nz, int nyb) {
  const long long t = u / nz;
  TxSeg s;
  s.zs = (int)(u - t * nz);
  s.ze = (int)min((long long)nz, s.zs + (u1 - u));
  s.yb = (int)(t % nyb);
  s.vb = (int)(t / nyb);
  return s;
}

// Requirements (checked by the launcher): nx == 128 NXB; ldi, ci_off, ldo,
// co_off multiples of 8; in, w and out 16-byte aligned.
template <int CIN, int COUT, int NXB>
__global__ void __launch_bounds__(TX_THREADS, 1)
    k_conv3_tx(const ConvArgs a, const __grid_constant__ TxMaps M, const TxGeo g, int *err) {
  static_assert(CIN % 16 == 0 && (COUT == 16 || COUT == 32) && (NXB == 1 || NXB == 2), "shapes");
  constexpr int NCH = CIN / 16;
  constexpr int TYR = tx_tyr<COUT, NXB>();
  constexpr int ROWS = TYR + 2;
  constexpr int NXV = NXB * 128;                 // voxels per row
  constexpr int RB = NXV * 16;                   // bytes of one staged row, one channel plane
  constexpr int PB = tx_plane_bytes<COUT, NXB>();
  constexpr int WB = tm_wbytes<COUT>();
  constexpr int WPB = WB / 2;
  constexpr int STAGE = tx_stage_bytes<COUT, NXB>();
  constexpr int N3 = 3 * COUT;                   // MMA N: three x-taps
  constexpr int AN = tx_accn<COUT>();            // accumulator stride in columns
  constexpr int ACC = tx_acc_cols<COUT, NXB>();
  static_assert(TX_NACC * ACC <= TX_TMEM_COLS, "tensor memory columns");
  static_assert(tx_smem<CIN, COUT, NXB>() <= 220 * 1024, "shared memory");
  static_assert(N3 % 16 == 0 && N3 <= 256, "MMA shape");
  constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N3 >> 3) << 17) | ((128u >> 4) << 24);

  extern __shared__ unsigned char tx_raw[];
  __shared__ __align__(8) unsigned long long s_full[TX_NST], s_empty[TX_NST];
  __shared__ __align__(8) unsigned long long s_accf[TX_NACC], s_acce[TX_NACC], s_wbar, s_fin;
  __shared__ float s_edge[2][NXB][4][2][COUT];  // [buffer][block][warp quarter][left, right][channel]
  __shared__ uint32_t s_tmem;
  __shared__ int s_fail;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t raw = smem_u32(tx_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  const uint32_t wfix = base + TX_NST * STAGE;
  const long long u0 = (long long)blockIdx.x * g.units / gridDim.x;
  const long long u1 = (long long)(blockIdx.x + 1) * g.units / gridDim.x;
  const int nx = a.nx, ny = a.ny, nz = a.nz;

  if (tid == 0) {
    s_fail = 0;
    for (int i = 0; i < TX_NST; i++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_full[i])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_empty[i])));
    }
    for (int i = 0; i < TX_NACC; i++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_accf[i])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 128;" ::"r"(smem_u32(&s_acce[i])));
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_wbar)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_fin)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                 "r"(TX_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = s_tmem;

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    if (lane == 0) {
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&s_wbar)), "r"(NCH * WB)
                   : "memory");
      for (int c = 0; c < NCH; c++) {
        tm_tma3(wfix + c * WB, &M.w, smem_u32(&s_wbar), tx_wch(c, 0), 0, 0);
        tm_tma3(wfix + c * WB + WPB, &M.w, smem_u32(&s_wbar), tx_wch(c, 1), 0, 0);
      }
      long long k = 0;
      bool bad = false;
      const uint32_t bytes = (uint32_t)(2 * ROWS * RB);
      for (long long u = u0; u < u1 && !bad;) {
        const TxSeg s = tx_seg(u, u1, nz, g.nyb);
        u += s.ze - s.zs;
        const int y0 = s.yb * TYR;
        const bool per_row = a.py && (y0 == 0 || y0 + TYR >= ny);  // a wrapped y halo row
        for (int zi = s.zs - 1; zi <= s.ze && !bad; zi++) {
          for (int c = 0; c < NCH; c++, k++) {
            const int slot = (int)(k % TX_NST);
            const uint32_t sb = base + slot * STAGE;
            if (k >= TX_NST && !tm_wait(smem_u32(&s_empty[slot]), (uint32_t)((k / TX_NST) - 1) & 1u)) {
              bad = true;
              break;
            }
            const uint32_t fb = smem_u32(&s_full[slot]);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fb), "r"(bytes) : "memory");
            const int gz = a.pz ? ((zi % nz) + nz) % nz : zi;  // else a plane outside reads the zero fill
            const int ch = a.ci_off + 16 * c;
            for (int kp = 0; kp < 2; kp++) {
              const uint32_t pb = sb + kp * PB;
              if (!per_row) {
                tm_tma5(pb, &M.rows, fb, ch + 8 * kp, 0, y0 - 1, gz, s.vb);
              } else {
                for (int r = 0; r < ROWS; r++)
                  tm_tma5(pb + r * RB, &M.row, fb, ch + 8 * kp, 0, ((y0 - 1 + r) % ny + ny) % ny, gz, s.vb);
              }
            }
          }
        }
      }
      if (bad) atomicExch(&s_fail, 1);
      // drain: the copies of the last stages issued land before the CTA exits
      for (long long j = (k > TX_NST ? k - TX_NST : 0); j < k; j++)
        tm_wait(smem_u32(&s_full[(int)(j % TX_NST)]), (uint32_t)(j / TX_NST) & 1u);
      tm_wait(smem_u32(&s_wbar), 0);
    }
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      bool bad = !tm_wait(smem_u32(&s_wbar), 0);
      bool issued = false;
      long long k = 0, q0 = 0;
      for (long long u = u0; u < u1 && !bad;) {
        const TxSeg s = tx_seg(u, u1, nz, g.nyb);
        u += s.ze - s.zs;
        for (int zi = s.zs - 1; zi <= s.ze && !bad; zi++) {
          if (zi + 1 < s.ze) {  // output plane zi + 1 starts here: its slot must be drained
            const long long q = q0 + (zi + 1 - s.zs);
            if (q >= TX_NACC &&
                !tm_wait(smem_u32(&s_acce[(int)(q % TX_NACC)]), (uint32_t)((q / TX_NACC) - 1) & 1u)) {
              bad = true;
              break;
            }
          }
          for (int c = 0; c < NCH && !bad; c++, k++) {
            const int slot = (int)(k % TX_NST);
            if (!tm_wait(smem_u32(&s_full[slot]), (uint32_t)(k / TX_NST) & 1u)) {
              bad = true;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sb = base + slot * STAGE;
            const uint64_t bd0 = tm_desc(wfix + c * WB, WPB, 128);
            for (int r = 0; r < ROWS; r++) {
#pragma unroll
              for (int b = 0; b < NXB; b++) {
                const uint64_t ad = tm_desc(sb + (r * NXB + b) * 2048, PB, 128);
#pragma unroll
                for (int dz = 0; dz < 3; dz++) {
                  const int zo = zi + 1 - dz;
                  if (zo < s.zs || zo >= s.ze) continue;
                  const int as = (int)((q0 + zo - s.zs) % TX_NACC);
#pragma unroll
                  for (int dy = 0; dy < 3; dy++) {
                    const int ty = r - dy;
                    if (ty < 0 || ty >= TYR) continue;
                    const uint32_t acc = tmem + (uint32_t)(((as * TYR + ty) * NXB + b) * AN);
                    const uint32_t en = (c == 0 && dz == 0 && dy == 0) ? 0u : 1u;
                    const uint64_t bd = bd0 + (uint64_t)(((dz * 9 + dy * 3) * COUT * 16) >> 4);
                    asm volatile(
                        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(acc),
                        "l"(ad), "l"(bd), "r"(IDESC), "r"(en)
                        : "memory");
                  }
                }
              }
            }
            tm_commit(smem_u32(&s_empty[slot]));
            issued = true;
          }
          if (bad) break;
          if (zi - 1 >= s.zs) tm_commit(smem_u32(&s_accf[(int)((q0 + zi - 1 - s.zs) % TX_NACC)]));
        }
        q0 += s.ze - s.zs;
      }
      if (bad) atomicExch(&s_fail, 1);
      if (issued) {  // drain: every MMA issued has finished before tensor memory is freed
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
    int eb = 0;  // edge buffer in use
    bool bad = false;
    for (long long u = u0; u < u1 && !bad;) {
      const TxSeg s = tx_seg(u, u1, nz, g.nyb);
      u += s.ze - s.zs;
      const int y0 = s.yb * TYR;
      for (int zo = s.zs; zo < s.ze; zo++, q++) {
        const int as = (int)(q % TX_NACC);
        const bool ok = tm_wait(smem_u32(&s_accf[as]), (uint32_t)(q / TX_NACC) & 1u);
        // one decision for the four epilogue warps (they meet at a named barrier below)
        uint32_t all_ok;
        asm volatile(
            "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 q, %1, 0;\n\tbar.red.and.pred p, 1, 128, q;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(all_ok)
            : "r"((uint32_t)ok)
            : "memory");
        if (!all_ok) {
          bad = true;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        bf16 *const oplane = a.out + ((long long)s.vb * nz + zo) * ny * (long long)nx * a.ldo + a.co_off;
#pragma unroll 1
        for (int ty = 0; ty < TYR; ty++) {
          float d0[NXB][COUT], d1[NXB][COUT], d2[NXB][COUT];
#pragma unroll
          for (int b = 0; b < NXB; b++) {
            const uint32_t col = tmem + lrow + (uint32_t)(((as * TYR + ty) * NXB + b) * AN);
            tm_ld<COUT>(col, d0[b]);  // warp-collective
            tm_ld<COUT>(col + COUT, d1[b]);
            tm_ld<COUT>(col + 2 * COUT, d2[b]);
            // the edge values the neighbouring warps need: tap 0 of the last
            // voxel, tap 2 of the first
            if (lane == 31)
#pragma unroll
              for (int i = 0; i < COUT; i++) s_edge[eb][b][quarter][0][i] = d0[b][i];
            if (lane == 0)
#pragma unroll
              for (int i = 0; i < COUT; i++) s_edge[eb][b][quarter][1][i] = d2[b][i];
          }
          asm volatile("bar.sync 1, 128;" ::: "memory");  // the epilogue warps only
          const int y = y0 + ty;
#pragma unroll
          for (int b = 0; b < NXB; b++) {
            // neighbours of this warp's first and last voxel across warps, blocks
            // and the periodic wrap (else the zero padding)
            int lb = b, lq = quarter - 1, rb = b, rq = quarter + 1;
            bool lok = true, rok = true;
            if (lq < 0) {
              lq = 3;
              lb = b - 1;
              if (lb < 0) {
                lb = NXB - 1;
                lok = a.px != 0;
              }
            }
            if (rq > 3) {
              rq = 0;
              rb = b + 1;
              if (rb >= NXB) {
                rb = 0;
                rok = a.px != 0;
              }
            }
            float o[COUT];
#pragma unroll
            for (int i = 0; i < COUT; i++) {
              float left = __shfl_up_sync(0xffffffffu, d0[b][i], 1);
              float right = __shfl_down_sync(0xffffffffu, d2[b][i], 1);
              if (lane == 0) left = lok ? s_edge[eb][lb][lq][0][i] : 0.f;
              if (lane == 31) right = rok ? s_edge[eb][rb][rq][1][i] : 0.f;
              o[i] = left + d1[b][i] + right;
            }
            if (y < ny) {
              const int x = b * 128 + quarter * 32 + lane;
              bf16 *op = oplane + ((long long)y * nx + x) * a.ldo;
#pragma unroll
              for (int ch = 0; ch < COUT; ch += 8) {
                uint4 pk;
                __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(&pk);
#pragma unroll
                for (int i = 0; i < 4; i++) {
                  float f0 = o[ch + 2 * i] + bias[ch + 2 * i], f1 = o[ch + 2 * i + 1] + bias[ch + 2 * i + 1];
                  if (a.relu) {
                    f0 = fmaxf(f0, 0.f);
                    f1 = fmaxf(f1, 0.f);
                  }
                  h[i] = __floats2bfloat162_rn(f0, f1);
                }
                *reinterpret_cast<uint4 *>(op + ch) = pk;
              }
            }
          }
          eb ^= 1;  // the next row writes the other edge buffer (one barrier per row suffices)
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&s_acce[as])) : "memory");
      }
    }
    if (bad && lane == 0) atomicExch(&s_fail, 1);
  }

  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TX_TMEM_COLS));
  if (tid == 0 && s_fail) atomicExch(err, 1);
}

}  // namespace bbnet
