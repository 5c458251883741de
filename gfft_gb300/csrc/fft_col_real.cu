// The real-pair kernels of the tensor-copy column tiles (col.cuh, RF = 1:
// real forward post pass fused into the last global pass, RF = 2: real
// inverse pre pass fused into the first), in a translation unit of their own
// so that they compile beside the complex ones.
#include <cuda_runtime.h>

#include "col.cuh"

namespace {
template <typename T, int RF>
const void* real_fn(int L) {
  switch (L) {
    case 64: return (const void*)gfft::col_kernel<T, 64, RF>;
    case 128: return (const void*)gfft::col_kernel<T, 128, RF>;
    case 256: return (const void*)gfft::col_kernel<T, 256, RF>;
    case 512: return (const void*)gfft::col_kernel<T, 512, RF>;
    case 1024: return (const void*)gfft::col_kernel<T, 1024, RF>;
    case 2048: return (const void*)gfft::col_kernel<T, 2048, RF>;
    default: return nullptr;
  }
}
}  // namespace

extern "C" const void* gfft_col_real_fn(int dbl, int L, int rf) {
  if (rf == 1) return dbl ? real_fn<double, 1>(L) : real_fn<float, 1>(L);
  if (rf == 2) return dbl ? real_fn<double, 2>(L) : real_fn<float, 2>(L);
  return nullptr;
}
