// Mixed-radix column tiles (variant 9 for the pass shapes of
// mixed_shapes.h), moved by 2-D tensor copies or, where the tiles do not fit
// a tensor map, gathered by cp.async: the kernels of colmix.cuh and their
// host side (tensor maps, launch).
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "colmix.cuh"
#include "mixed_shapes.h"

// fft_col.cu: a 2-D tensor map over rows x cols elements of esz bytes, boxes of w x br
extern "C" int gfft_tmap_2d(void* map, const void* base, long long rows, long long cols, int esz, int w, int br);

namespace {

#define GFFT_MIX_KERNEL(K, T)                                  \
  switch (idx) {                                               \
    case 0: return (const void*)gfft::K<T, 16, 16, 3, 1>;      \
    case 1: return (const void*)gfft::K<T, 5, 5, 5, 5>;        \
    case 2: return (const void*)gfft::K<T, 16, 12, 3, 1>;      \
    case 3: return (const void*)gfft::K<T, 16, 9, 3, 1>;       \
    case 4: return (const void*)gfft::K<T, 10, 10, 10, 1>;     \
    case 5: return (const void*)gfft::K<T, 9, 9, 9, 1>;        \
    case 6: return (const void*)gfft::K<T, 16, 15, 2, 1>;      \
    case 7: return (const void*)gfft::K<T, 15, 12, 2, 1>;      \
    default: return nullptr;                                   \
  }

// the kernel of shape `idx` (mixed_shapes.h order): tensor copies or gathers
template <typename T>
const void* mix_fn(int idx, int gather) {
  if (gather) {
    GFFT_MIX_KERNEL(colmix_gather_kernel, T)
  }
  GFFT_MIX_KERNEL(colmix_kernel, T)
}
#undef GFFT_MIX_KERNEL

const void* fn_for(int dbl, const EngineArgs* a, int gather) {
  int rs[4] = {1, 1, 1, 1};
  for (int i = 0; i < a->npass && i < 4; ++i) rs[i] = a->pass[i].R;
  const int idx = a->npass <= 4 ? mixed_shape_index(a->L, rs, a->npass) : -1;
  if (idx < 0 || (!gather && !gfft::colshape::mix_supported(dbl ? 16 : 8, a->L))) return nullptr;
  return dbl ? mix_fn<double>(idx, gather) : mix_fn<float>(idx, gather);
}

}  // namespace

extern "C" int gfft_colmix_setup(int dbl, size_t max_smem) {
  int e = 0;
  for (int gather = 0; gather < 2; ++gather)
    for (int i = 0; i < kNumMixedShapes; ++i) {
      const void* f = dbl ? mix_fn<double>(i, gather) : mix_fn<float>(i, gather);
      // the gather kernel's lane table takes 1 KB of static shared memory
      const int dyn = (int)max_smem - (gather ? 1024 : 0);
      if (f) e |= cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess;
    }
  return e;
}

extern "C" int gfft_colmix_occupancy(int dbl, const EngineArgs* a, int gather, int threads, size_t smem) {
  const void* f = fn_for(dbl, a, gather);
  if (!f) return 0;
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f, threads, smem);
  return n;
}

// One global pass: tensor maps of this launch's input and output, then the
// launch.  Requirements (checked by the planner): W divides N / L and Ns,
// row pitches of a multiple of 16 bytes, 16-byte aligned buffers.
extern "C" int gfft_colmix_launch(int dbl, const EngineArgs* a, int gather, unsigned grid, unsigned threads,
                                  size_t smem, cudaStream_t stream) {
  using namespace gfft::colshape;
  const void* f = fn_for(dbl, a, gather);
  if (!f) return (int)cudaErrorInvalidValue;
  const int esz = dbl ? 16 : 8;
  const int W = mix_lanes(esz, a->L), br = mix_rows(a->L);
  if ((int)threads != mix_threads()) return (int)cudaErrorInvalidValue;
  cudaGetLastError();  // clear a stale error of an earlier, unrelated call
  if (gather) {
    // element-aligned buffers (cp.async of one element), one or two stages
    if ((((uintptr_t)a->in) | ((uintptr_t)a->out)) & (uintptr_t)(esz - 1)) return (int)cudaErrorInvalidValue;
    if (a->stages < 1 || a->stages > 2) return (int)cudaErrorInvalidValue;
    void* gargs[] = {(void*)a};
    return (int)cudaLaunchKernel(f, dim3(grid), dim3(threads), gargs, smem, stream);
  }
  if ((((uintptr_t)a->in) | ((uintptr_t)a->out)) & 15) return (int)cudaErrorInvalidValue;
  if (a->stride % W || (a->gNs > 1 && a->gNs % W)) return (int)cudaErrorInvalidValue;
  if ((a->stride * esz) % 16 || (a->gNs > 1 && (a->gNs * esz) % 16)) return (int)cudaErrorInvalidValue;
  const long long batch = a->nunits / a->stride;
  gfft::col::ColMaps m;
  if (gfft_tmap_2d(&m.in[0], a->in, batch * a->L, a->stride, esz, W, br) != 0) return (int)cudaErrorInvalidValue;
  if (a->gNs > 1) {
    if (gfft_tmap_2d(&m.out[0], a->out, batch * (a->N / a->gNs), a->gNs, esz, W, br) != 0)
      return (int)cudaErrorInvalidValue;
  } else {
    m.out[0] = m.in[0];  // unused: the first pass stores from registers
  }
  m.in[1] = m.in[2] = m.in[0];
  m.out[1] = m.out[2] = m.out[0];
  void* args[] = {(void*)a, (void*)&m};
  return (int)cudaLaunchKernel(f, dim3(grid), dim3(threads), args, smem, stream);
}
