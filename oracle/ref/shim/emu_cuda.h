/*
 * emu_cuda.h -- a small host emulation of the CUDA execution model, used only
 * to run the reference's unmodified solver sources on the CPU so that the
 * oracle can be checked against them (test infrastructure).
 *
 * Blocks run one after another; the threads of a block run as ucontext
 * fibers on the calling OS thread.  __syncthreads() yields to the block's
 * scheduler, which resumes every fiber round-robin, so each barrier is
 * passed only when all threads of the block reached it.  __shared__ arrays
 * become function statics, shared by the threads of the running block.
 */
#ifndef EMU_CUDA_H
#define EMU_CUDA_H

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef __cplusplus
#include <functional>

struct dim3 {
  unsigned int x, y, z;
  dim3(unsigned int x_ = 1, unsigned int y_ = 1, unsigned int z_ = 1) : x(x_), y(y_), z(z_) {}
};
struct uint3 {
  unsigned int x, y, z;
};

namespace emu {
extern uint3 cur_tid, cur_bid;
extern dim3 cur_bdim, cur_gdim;
void sync();
void launch(dim3 grid, dim3 block, const std::function<void()> &body);
}  // namespace emu

#define threadIdx (emu::cur_tid)
#define blockIdx (emu::cur_bid)
#define blockDim (emu::cur_bdim)
#define gridDim (emu::cur_gdim)
inline void __syncthreads() { emu::sync(); }
inline void __threadfence() {}

#define __global__
#define __device__
#define __host__
#define __shared__ static
#define __constant__
#define __forceinline__ inline

typedef int cudaError_t;
#define cudaSuccess 0
enum cudaMemcpyKind { cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost,
                      cudaMemcpyDeviceToDevice, cudaMemcpyDefault };
inline cudaError_t cudaMemset(void *p, int v, size_t n) { memset(p, v, n); return 0; }
inline cudaError_t cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind) { memmove(d, s, n); return 0; }
inline cudaError_t cudaMalloc(void **p, size_t n) { *p = calloc(1, n ? n : 1); return 0; }
inline cudaError_t cudaFree(void *p) { free(p); return 0; }
inline cudaError_t cudaDeviceSynchronize() { return 0; }
inline cudaError_t cudaGetLastError() { return 0; }
inline const char *cudaGetErrorString(cudaError_t) { return "no error"; }
#endif /* __cplusplus */

#endif
