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
template <typename T, int RF>
int real_smem(int L, int* tb, int* work) {
  switch (L) {
#define GFFT_COL_REAL_SMEM(LL)                             \
  case LL:                                                 \
    *tb = gfft::col::Geo<T, LL, RF>::TB;                   \
    *work = gfft::col::Geo<T, LL, RF>::WORK;               \
    return 0;
    GFFT_COL_REAL_SMEM(64)
    GFFT_COL_REAL_SMEM(128)
    GFFT_COL_REAL_SMEM(256)
    GFFT_COL_REAL_SMEM(512)
    GFFT_COL_REAL_SMEM(1024)
    GFFT_COL_REAL_SMEM(2048)
#undef GFFT_COL_REAL_SMEM
    default: return 1;
  }
}
}  // namespace

extern "C" const void* gfft_col_real_fn(int dbl, int L, int rf) {
  if (rf == 1) return dbl ? real_fn<double, 1>(L) : real_fn<float, 1>(L);
  if (rf == 2) return dbl ? real_fn<double, 2>(L) : real_fn<float, 2>(L);
  return nullptr;
}

extern "C" int gfft_col_real_smem(int dbl, int L, int rf, int* tb, int* work) {
  if (rf == 1) return dbl ? real_smem<double, 1>(L, tb, work) : real_smem<float, 1>(L, tb, work);
  if (rf == 2) return dbl ? real_smem<double, 2>(L, tb, work) : real_smem<float, 2>(L, tb, work);
  return 1;
}
