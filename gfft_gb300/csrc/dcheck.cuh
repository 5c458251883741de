// Bounds checks of the debug build (compiled with -DGFFT_DEBUG, the library
// libgfft_gb300_debug.so): a failing check records GFFT_E_BOUNDS (16) and its
// source line in the launch's status words (status[0], status[1]; the first
// failure wins) and the access it guards is skipped, so a wrong index never
// reaches memory and never traps.  Release builds compile the checks away.
#pragma once
#include <cuda_runtime.h>

#ifdef GFFT_DEBUG
__device__ __forceinline__ bool gfft_dcheck(bool ok, int* status, int line) {
  if (!ok && status) {
    if (atomicCAS(status, 0, 16) == 0) atomicExch(status + 1, line);
  }
  return ok;
}
#define GFFT_DCHECK(ok, status) gfft_dcheck((ok), (status), __LINE__)
#else
#define GFFT_DCHECK(ok, status) true
#endif
