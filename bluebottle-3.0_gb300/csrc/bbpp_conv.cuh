// bbpp_conv.cuh -- 3x3x3 convolutions of the learned initial guess as
// implicit GEMMs on BF16 tensor cores (mma.sync m16n8k16, FP32 accumulate).
//
// Activations are channels-last BF16 volumes, [volume][z][y][x][channel] with
// a channel stride `ld` and a channel offset, so a concatenation is two
// tensors writing disjoint channel ranges of one buffer.  Padding is periodic
// on the axes flagged periodic and zero otherwise.
//
//  k_conv3_fwd<CIN, COUT>   out = act(conv(in, W) + bias); a CTA computes a
//                           16x8xTZ tile of outputs (TZ = 8, 4, 2 for 16,
//                           32, 64 output channels) from a halo tile staged in
//                           shared memory 16 input channels at a time; the 27
//                           taps are 27 k16 steps whose A rows are shifted
//                           halo rows (ldmatrix gather).  dgrad uses the same
//                           kernel with the taps flipped and W transposed.
//  k_conv3_wgrad<CIN, COUT> dW[t] += sum_v g[v]^T in[v + t], one tap per CTA
//                           over a range of tiles, warps split the voxels.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace bbnet {

typedef __nv_bfloat16 bf16;

constexpr int CTX = 16, CTY = 8, CTZ = 2;                  // output tile of a CTA
constexpr int HTX = CTX + 2, HTY = CTY + 2, HTZ = CTZ + 2;  // with halo
constexpr int HVOX = HTX * HTY * HTZ;                      // 720 halo voxels
constexpr int RSB = 48;  // shared bytes per voxel row of a 16-channel chunk (32 + 16 pad)

struct ConvArgs {
  const bf16 *in;
  int ldi, ci_off;
  const bf16 *w;       // [27][COUT][CIN]
  const float *bias;   // [COUT] or null
  bf16 *out;
  int ldo, co_off;
  int nx, ny, nz, nb;  // volume, number of volumes
  int px, py, pz;      // periodic axes
  int relu;
};

struct WgradArgs {
  const bf16 *in;
  int ldi, ci_off;
  const bf16 *g;       // gradient of the conv output (after the activation gate)
  int ldg, cg_off;
  float *dW;           // [27][COUT][CIN], accumulated
  int nx, ny, nz, nb;
  int px, py, pz;
  int tiles_per_cta;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void ldsm_x4(uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3, const void *p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(smem_u32(p)));
}

__device__ __forceinline__ void ldsm_x4_t(uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3, const void *p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(smem_u32(p)));
}

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// index along one axis with periodic wrap or zero padding; false = padding
__device__ __forceinline__ bool pad_axis(int &g, int n, int periodic) {
  if (g >= 0 && g < n) return true;
  if (!periodic) return false;
  g = (g < 0) ? g + n : g - n;
  return g >= 0 && g < n;
}

// ------------------------------------------------------------- forward -----
// z planes of the forward kernel's output tile: deeper tiles reuse every
// weight fragment over more A fragments and cut the halo share, as long as
// the accumulators fit in registers
template <int COUT>
__host__ __device__ constexpr int fwd_tz() {
  return COUT <= 16 ? 8 : (COUT <= 32 ? 4 : 2);
}

template <int CIN, int COUT>
__global__ void __launch_bounds__(256) k_conv3_fwd(const ConvArgs a) {
  static_assert(CIN % 16 == 0 && COUT % 16 == 0, "channels in multiples of 16");
  constexpr int TZ = fwd_tz<COUT>();
  constexpr int HVZ = HTX * HTY * (TZ + 2);  // halo voxels
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned char *s_in = smem;              // HVZ rows of RSB bytes
  unsigned char *s_w = smem + HVZ * RSB;   // 27 * COUT rows of RSB bytes
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int x0 = blockIdx.x * CTX, y0 = blockIdx.y * CTY;
  const int nzt = (a.nz + TZ - 1) / TZ;
  const int vb = blockIdx.z / nzt;
  const int z0 = (blockIdx.z - vb * nzt) * TZ;
  const long long vol = (long long)a.nx * a.ny * a.nz;
  const bf16 *inb = a.in + (long long)vb * vol * a.ldi + a.ci_off;

  float acc[TZ][COUT / 8][4];
#pragma unroll
  for (int i = 0; i < TZ; i++)
#pragma unroll
    for (int j = 0; j < COUT / 8; j++)
#pragma unroll
      for (int q = 0; q < 4; q++) acc[i][j][q] = 0.f;

  for (int c0 = 0; c0 < CIN; c0 += 16) {
    for (int idx = tid; idx < HVZ * 2; idx += 256) {
      const int e = idx >> 1, half = idx & 1;
      const int hx = e % HTX, t = e / HTX;
      const int hy = t % HTY, hz = t / HTY;
      int gx = x0 + hx - 1, gy = y0 + hy - 1, gz = z0 + hz - 1;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (pad_axis(gx, a.nx, a.px) && pad_axis(gy, a.ny, a.py) && pad_axis(gz, a.nz, a.pz))
        v = *reinterpret_cast<const uint4 *>(inb + (((long long)gz * a.ny + gy) * a.nx + gx) * a.ldi + c0 + half * 8);
      *reinterpret_cast<uint4 *>(s_in + e * RSB + half * 16) = v;
    }
    for (int idx = tid; idx < 27 * COUT * 2; idx += 256) {
      const int row = idx >> 1, half = idx & 1;
      *reinterpret_cast<uint4 *>(s_w + row * RSB + half * 16) =
          *reinterpret_cast<const uint4 *>(a.w + (long long)row * CIN + c0 + half * 8);
    }
    __syncthreads();
#pragma unroll 1
    for (int tap = 0; tap < 27; tap++) {
      const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
      uint32_t bfr[COUT / 8][2];
#pragma unroll
      for (int j = 0; j < COUT / 8; j += 2) {
        const int n = tap * COUT + j * 8 + (lane & 7) + ((lane >> 4) << 3);
        ldsm_x4(bfr[j][0], bfr[j][1], bfr[j + 1][0], bfr[j + 1][1], s_w + n * RSB + ((lane >> 3) & 1) * 16);
      }
#pragma unroll
      for (int mi = 0; mi < TZ; mi++) {
        uint32_t afr[4];
        const int hv = ((mi + dz) * HTY + warp + dy) * HTX + (lane & 15) + dx;
        ldsm_x4(afr[0], afr[1], afr[2], afr[3], s_in + hv * RSB + (lane >> 4) * 16);
#pragma unroll
        for (int j = 0; j < COUT / 8; j++) mma16816(acc[mi][j], afr, bfr[j][0], bfr[j][1]);
      }
    }
    __syncthreads();
  }
  // epilogue: bias, activation, BF16 store
  const int y = y0 + warp;
  if (y >= a.ny) return;
  bf16 *outb = a.out + (long long)vb * vol * a.ldo + a.co_off;
#pragma unroll
  for (int mi = 0; mi < TZ; mi++) {
    const int z = z0 + mi;
    if (z >= a.nz) continue;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int x = x0 + (lane >> 2) + 8 * h;
      if (x >= a.nx) continue;
      bf16 *o = outb + (((long long)z * a.ny + y) * a.nx + x) * a.ldo;
#pragma unroll
      for (int j = 0; j < COUT / 8; j++) {
        const int ch = j * 8 + (lane & 3) * 2;
        float v0 = acc[mi][j][2 * h], v1 = acc[mi][j][2 * h + 1];
        if (a.bias) {
          v0 += a.bias[ch];
          v1 += a.bias[ch + 1];
        }
        if (a.relu) {
          v0 = fmaxf(v0, 0.f);
          v1 = fmaxf(v1, 0.f);
        }
        *reinterpret_cast<__nv_bfloat162 *>(o + ch) = __floats2bfloat162_rn(v0, v1);
      }
    }
  }
}

template <int CIN, int COUT>
__host__ __device__ constexpr int conv_fwd_smem() {
  return HTX * HTY * (fwd_tz<COUT>() + 2) * RSB + 27 * COUT * RSB;
}

// --------------------------------------------------------------- wgrad -----
// CTA (tap, slice of tiles); 8 warps take the 16 voxel rows (z, y) of a tile,
// two each.  A = g^T (COUT x voxels), B = in shifted by the tap (voxels x 16
// input channels), both staged in shared memory and read with ldmatrix.trans.
template <int CIN, int COUT>
__global__ void __launch_bounds__(256) k_conv3_wgrad(const WgradArgs a) {
  constexpr int GRS = COUT * 2 + 16;  // shared bytes per voxel row of g
  constexpr int MT = COUT / 16;       // m tiles (output channels)
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned char *s_g = smem;                             // 256 rows of GRS
  unsigned char *s_x = smem + 256 * GRS;                 // 256 rows of RSB (16 channels)
  float *s_red = reinterpret_cast<float *>(smem + 256 * GRS + 256 * RSB);  // 8 warps x COUT x 16
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int tap = blockIdx.y;
  const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
  const int tx_n = (a.nx + CTX - 1) / CTX, ty_n = (a.ny + CTY - 1) / CTY, tz_n = (a.nz + CTZ - 1) / CTZ;
  const long long ntiles = (long long)tx_n * ty_n * tz_n * a.nb;
  const long long vol = (long long)a.nx * a.ny * a.nz;
  for (int c0 = 0; c0 < CIN; c0 += 16) {
    float acc[MT][2][4];
#pragma unroll
    for (int m = 0; m < MT; m++)
#pragma unroll
      for (int n = 0; n < 2; n++)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[m][n][q] = 0.f;
    const long long t_begin = (long long)blockIdx.x * a.tiles_per_cta;
    const long long t_end = t_begin + a.tiles_per_cta < ntiles ? t_begin + a.tiles_per_cta : ntiles;
    for (long long tile = t_begin; tile < t_end; tile++) {
      long long tt = tile;
      const int bx = (int)(tt % tx_n);
      tt /= tx_n;
      const int by = (int)(tt % ty_n);
      tt /= ty_n;
      const int bz = (int)(tt % tz_n);
      const int vb = (int)(tt / tz_n);
      // stage g (zero outside the volume) and the shifted input
      for (int idx = tid; idx < 256 * (COUT / 8 + 2); idx += 256) {
        const int v = idx % 256, part = idx / 256;  // parts 0..COUT/8-1: g; then 2 parts of x
        const int lx = v % CTX, ly = (v / CTX) % CTY, lz = v / (CTX * CTY);
        const int ox = bx * CTX + lx, oy = by * CTY + ly, oz = bz * CTZ + lz;
        const bool inside = ox < a.nx && oy < a.ny && oz < a.nz;
        uint4 val = make_uint4(0u, 0u, 0u, 0u);
        if (part < COUT / 8) {
          if (inside)
            val = *reinterpret_cast<const uint4 *>(a.g + ((long long)vb * vol + ((long long)oz * a.ny + oy) * a.nx + ox) *
                                                            a.ldg + a.cg_off + part * 8);
          *reinterpret_cast<uint4 *>(s_g + v * GRS + part * 16) = val;
        } else {
          const int half = part - COUT / 8;
          int gx = ox + dx, gy = oy + dy, gz = oz + dz;
          if (inside && pad_axis(gx, a.nx, a.px) && pad_axis(gy, a.ny, a.py) && pad_axis(gz, a.nz, a.pz))
            val = *reinterpret_cast<const uint4 *>(a.in + ((long long)vb * vol + ((long long)gz * a.ny + gy) * a.nx + gx) *
                                                             a.ldi + a.ci_off + c0 + half * 8);
          *reinterpret_cast<uint4 *>(s_x + v * RSB + half * 16) = val;
        }
      }
      __syncthreads();
#pragma unroll
      for (int rr = 0; rr < 2; rr++) {
        const int row = warp + 8 * rr;  // voxel row (z, y) of the tile: voxels row*16 .. +15
        // B: two n tiles (input channels 0-7, 8-15), k = 16 voxels of the row
        uint32_t b00, b01, b10, b11;
        {
          const int mi = lane >> 3, i = lane & 7;
          const int v = row * 16 + i + (mi & 1) * 8;
          ldsm_x4_t(b00, b01, b10, b11, s_x + v * RSB + (mi >> 1) * 16);
        }
#pragma unroll
        for (int m = 0; m < MT; m++) {
          uint32_t af[4];
          const int mi = lane >> 3, i = lane & 7;
          const int v = row * 16 + i + (mi >> 1) * 8;
          ldsm_x4_t(af[0], af[1], af[2], af[3], s_g + v * GRS + (m * 16 + (mi & 1) * 8) * 2);
          mma16816(acc[m][0], af, b00, b01);
          mma16816(acc[m][1], af, b10, b11);
        }
      }
      __syncthreads();
    }
    // reduce the 8 warps' partial sums in shared memory, then add to dW
#pragma unroll
    for (int m = 0; m < MT; m++)
#pragma unroll
      for (int n = 0; n < 2; n++)
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const int co = m * 16 + (lane >> 2) + (q >> 1) * 8;
          const int ci = n * 8 + (lane & 3) * 2 + (q & 1);
          s_red[(warp * COUT + co) * 16 + ci] = acc[m][n][q];
        }
    __syncthreads();
    for (int e = tid; e < COUT * 16; e += 256) {
      float s = 0.f;
#pragma unroll
      for (int w = 0; w < 8; w++) s += s_red[w * COUT * 16 + e];
      const int co = e / 16, ci = e % 16;
      atomicAdd(&a.dW[((long long)tap * COUT + co) * CIN + c0 + ci], s);
    }
    __syncthreads();
  }
}

template <int CIN, int COUT>
constexpr int conv_wgrad_smem() {
  return 256 * (COUT * 2 + 16) + 256 * RSB + 8 * COUT * 16 * 4;
}

}  // namespace bbnet
