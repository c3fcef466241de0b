/* Host-emulation stand-in for <cuda.h> (see emu_cuda.h). */
#include "emu_cuda.h"
