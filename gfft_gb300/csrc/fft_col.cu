// Column tiles of a multi-pass power-of-two length moved by 2-D tensor
// copies (variant 9): the kernels of col.cuh for complex passes, the host
// side (tensor maps, launch) for every variant-9 pass.  The real-pair
// kernels (fused real pre/post pass) are instantiated in fft_col_real.cu.
#include <cuda.h>  // CUtensorMap and the encoder's prototype (no driver symbols are linked)
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "col.cuh"

// fft_col_real.cu: the kernel of a real pass (rf 1: forward post, 2: inverse pre), null if not compiled
extern "C" const void* gfft_col_real_fn(int dbl, int L, int rf);

namespace {

typedef CUresult (*EncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiled g_encode = nullptr;
std::mutex g_encode_mu;

int get_encoder() {
  std::lock_guard<std::mutex> lk(g_encode_mu);
  if (g_encode) return 0;
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn)
    return 1;
  g_encode = (EncodeTiled)fn;
  return 0;
}

// rows x cols matrix of elements of `esz` bytes at `base` (row pitch = cols), boxes of w x br elements
int encode(CUtensorMap* m, const void* base, long long rows, long long cols, int esz, int w, int br) {
  const int xs = esz / 8;
  cuuint64_t dims[2] = {(cuuint64_t)(cols * xs), (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(cols * esz)};
  cuuint32_t box[2] = {(cuuint32_t)(w * xs), (cuuint32_t)br};
  cuuint32_t es[2] = {1, 1};
  return g_encode(m, CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, const_cast<void*>(base), dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS
             ? 0
             : 1;
}

template <typename T>
const void* col_fn(int L, int tk) {
  if (tk == 32) {  // half-size tiles: FP32 passes of 128 .. 1024
    if (sizeof(T) != 4) return nullptr;
    switch (L) {
      case 128: return (const void*)gfft::col_kernel<float, 128, 0, 32>;
      case 256: return (const void*)gfft::col_kernel<float, 256, 0, 32>;
      case 512: return (const void*)gfft::col_kernel<float, 512, 0, 32>;
      case 1024: return (const void*)gfft::col_kernel<float, 1024, 0, 32>;
      default: return nullptr;
    }
  }
  if (tk != 64) return nullptr;
  switch (L) {
    case 64: return (const void*)gfft::col_kernel<T, 64, 0>;
    case 128: return (const void*)gfft::col_kernel<T, 128, 0>;
    case 256: return (const void*)gfft::col_kernel<T, 256, 0>;
    case 512: return (const void*)gfft::col_kernel<T, 512, 0>;
    case 1024: return (const void*)gfft::col_kernel<T, 1024, 0>;
    case 2048: return (const void*)gfft::col_kernel<T, 2048, 0>;
    case 4096: return sizeof(T) == 4 ? (const void*)gfft::col_kernel<float, 4096, 0> : nullptr;
    default: return nullptr;
  }
}
const void* kernel_of(int dbl, int L, int rf, int tk) {
  if (rf) return tk == 64 ? gfft_col_real_fn(dbl, L, rf) : nullptr;
  return dbl ? col_fn<double>(L, tk) : col_fn<float>(L, tk);
}
}  // namespace

// a 2-D tensor map (fft_colmix.cu): rows x cols elements of esz bytes at
// base, boxes of w x br elements; 0 on success
extern "C" int gfft_tmap_2d(void* map, const void* base, long long rows, long long cols, int esz, int w, int br) {
  if (get_encoder() != 0) return 1;
  return encode(reinterpret_cast<CUtensorMap*>(map), base, rows, cols, esz, w, br);
}

extern "C" int gfft_col_setup(int dbl, size_t max_smem) {
  if (get_encoder() != 0) return 1;
  int e = 0;
  for (int tk : {64, 32})
    for (int rf = 0; rf < 3; ++rf)
      for (int L : {64, 128, 256, 512, 1024, 2048, 4096}) {
        const void* f = kernel_of(dbl, L, rf, tk);
        if (f) e |= cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem) != cudaSuccess;
      }
  return e;
}

extern "C" int gfft_col_occupancy(int dbl, int L, int rf, int tk, int threads, size_t smem) {
  const void* f = kernel_of(dbl, L, rf, tk);
  if (!f) return 0;
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f, threads, smem);
  return n;
}

// One global pass: tensor maps of this launch's input and output, then the
// launch.  Requirements (checked by the planner): N a power of two, the
// units per tile dividing N / L and Ns, 16-byte aligned buffers; a real pass
// (a->real) is the last (forward) or first (inverse) pass; tk the tile KB.
extern "C" int gfft_col_launch(int dbl, const EngineArgs* a, int tk, unsigned grid, unsigned threads, size_t smem,
                               cudaStream_t stream) {
  const int rf = a->real;
  const void* f = kernel_of(dbl, a->L, rf, tk);
  if (!f || !g_encode) return (int)cudaErrorInvalidValue;
  const int esz = dbl ? 16 : 8;
  const int W = gfft::colshape::lanes(esz, a->L, tk);
  if ((int)threads != gfft::colshape::threads(esz, a->L, tk)) return (int)cudaErrorInvalidValue;
  const long long batch = a->nunits / a->stride;
  const int br = a->L < 256 ? a->L : 256;
  if ((((uintptr_t)a->in) | ((uintptr_t)a->out)) & 15) return (int)cudaErrorInvalidValue;
  if (a->stride % W || (a->gNs > 1 && a->gNs % W)) return (int)cudaErrorInvalidValue;
  gfft::col::ColMaps m;
  EngineArgs a2 = *a;
  a2.ftw_box = 0;
  const long long rows_in = batch * a->L, rows_out = batch * (a->N / a->gNs);
  if (!rf) {
    if (encode(&m.in[0], a->in, rows_in, a->stride, esz, W, br) != 0) return (int)cudaErrorInvalidValue;
    m.in[1] = m.in[2] = m.in[0];
    if (a->gNs > 1) {
      if (encode(&m.out[0], a->out, rows_out, a->gNs, esz, W, br) != 0) return (int)cudaErrorInvalidValue;
      // the [16][Ns] four-step factors, one [16][W] box per tile, where the
      // table (16 Ns values) outgrows L1: measured at 2^28 points, 6-10 %
      // faster for Ns >= 1024 (2^20 .. 2^24), about 1 % slower for Ns <= 512
      // (else the kernel reads them from global memory)
      if (a->ftw && a->gNs >= 1024 && !(((uintptr_t)a->ftw) & 15) &&
          encode(&m.in[1], a->ftw, 16, a->gNs, esz, W, 16) == 0)
        a2.ftw_box = 1;
    } else {
      m.out[0] = m.in[0];  // unused: the first pass stores from registers
    }
    m.out[1] = m.out[2] = m.out[0];
  } else {
    // regions A (W/2 columns), B (the mirrors; FP32 two wider) and C (column S/2)
    const int h = W / 2, hb = dbl ? h : h + 2, hc = dbl ? 1 : 2;
    if (rf == 1 && a->gNs != a->stride) return (int)cudaErrorInvalidValue;  // forward: the last pass
    if (rf == 2 && a->gNs != 1) return (int)cudaErrorInvalidValue;          // inverse: the first pass
    if (encode(&m.in[0], a->in, rows_in, a->stride, esz, h, br) != 0 ||
        encode(&m.in[1], a->in, rows_in, a->stride, esz, hb, br) != 0 ||
        encode(&m.in[2], a->in, rows_in, a->stride, esz, hc, br) != 0)
      return (int)cudaErrorInvalidValue;
    if (rf == 1) {
      if (encode(&m.out[0], a->out, rows_out, a->gNs, esz, h, br) != 0 ||
          encode(&m.out[1], a->out, rows_out, a->gNs, esz, h, br) != 0)
        return (int)cudaErrorInvalidValue;
      m.out[2] = m.out[0];  // unused: column S/2 goes out by plain stores
    } else {
      m.out[0] = m.out[1] = m.out[2] = m.in[0];  // unused: the first pass stores from registers
    }
  }
  cudaGetLastError();  // clear a stale error of an earlier, unrelated call
  void* args[] = {(void*)&a2, (void*)&m};
  return (int)cudaLaunchKernel(f, dim3(grid), dim3(threads), args, smem, stream);
}
