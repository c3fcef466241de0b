/* Host-emulation stand-in for <cuda_runtime.h> (see emu_cuda.h). */
#include "emu_cuda.h"
