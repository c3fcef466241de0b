// ref_cages_kernels.cu -- device side of the GPU run of the reference's cage
// builder (test and measurement infrastructure; never part of the product).
//
// Compiled by build_cubin.py into oracle/_ref/ref_cages.cubin together with the
// reference's unmodified src/particle_kernel.cu (included from the reference
// tree) and the domain helper of ref_kernels.cu.  It is compiled without FMA
// contraction (-fmad=false), the arithmetic of the host pin the cage fixtures
// come from, so that the GPU run and the fixtures can be compared bit for bit.
// Two helpers give the host what it must not interpret itself: the layout of
// part_struct (size and the offsets of N, r, x, y, z) and a BC struct with the
// pressure boundary types set.
#include "ref_kernels.cu"
#include "particle_kernel.cu"

#include <cstddef>

// out[0] = sizeof(part_struct), out[1..5] = offsets of N, r, x, y, z, out[6] = sizeof(BC)
extern "C" __global__ void refgpu_part_layout(long long *out) {
  if (threadIdx.x || blockIdx.x) return;
  out[0] = sizeof(part_struct);
  out[1] = offsetof(part_struct, N);
  out[2] = offsetof(part_struct, r);
  out[3] = offsetof(part_struct, x);
  out[4] = offsetof(part_struct, y);
  out[5] = offsetof(part_struct, z);
  out[6] = sizeof(BC);
}

extern "C" __global__ void refgpu_fill_bc(BC *bc, int pW, int pE, int pS, int pN, int pB, int pT) {
  if (threadIdx.x || blockIdx.x) return;
  memset(bc, 0, sizeof(BC));
  bc->pW = pW;
  bc->pE = pE;
  bc->pS = pS;
  bc->pN = pN;
  bc->pB = pB;
  bc->pT = pT;
}
