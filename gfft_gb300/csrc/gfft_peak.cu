// Arithmetic peak of the CUDA cores, measured: a multiply-add loop in FP64
// or FP32 over every SM, timed with CUDA events.  It supplies the
// denominator of the FP64 configurations' roofline (GB300's FP64 rate is a
// small fraction of its FP32 rate, so FP64 transforms are bounded by the
// FP64 pipe, not by HBM).  No reference counterpart: the reference's harness
// reports time and 5 N log2 N / t only (test/gfft_performance.h:67-78).
#include <cuda_runtime.h>

#include "../../include/gfft_gb300.h"

namespace {

// eight independent dependency chains per thread; the result is written only
// when it equals a value it never takes, so the loop is not eliminated
template <typename T>
__global__ void __launch_bounds__(256) fma_loop(T* sink, int iters, T a, T b) {
  T x[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) x[c] = (T)(threadIdx.x + c) * (T)1e-3;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < 8; ++c) x[c] = fma(x[c], a, b);
  }
  T s = 0;
#pragma unroll
  for (int c = 0; c < 8; ++c) s += x[c];
  if (s == (T)-1.2345e30) sink[blockIdx.x] = s;
}

template <typename T>
int measure(int iters, double* gflops, double* ms_out) {
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return GFFT_E_CUDA;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fma_loop<T>, 256, 0);
  if (per < 1) per = 1;
  const int blocks = nsm * per;
  T* sink = nullptr;
  if (cudaMalloc(&sink, sizeof(T) * (size_t)blocks) != cudaSuccess) return GFFT_E_ALLOC;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int st = GFFT_OK;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) st = GFFT_E_CUDA;
  float best = 0.f;
  if (st == GFFT_OK) {
    fma_loop<T><<<blocks, 256>>>(sink, iters / 8 + 1, (T)0.999999, (T)1e-6);  // warm-up
    for (int rep = 0; rep < 5 && st == GFFT_OK; ++rep) {
      cudaEventRecord(e0);
      fma_loop<T><<<blocks, 256>>>(sink, iters, (T)0.999999, (T)1e-6);
      cudaEventRecord(e1);
      if (cudaEventSynchronize(e1) != cudaSuccess) {
        st = GFFT_E_CUDA;
        break;
      }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep == 0 || ms < best) best = ms;
    }
  }
  if (st == GFFT_OK) {
    const double flops = 2.0 * 8.0 * (double)iters * 256.0 * (double)blocks;
    *gflops = flops / ((double)best * 1e-3) / 1e9;
    if (ms_out) *ms_out = best;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(sink);
  return st;
}

}  // namespace

extern "C" int gfft_measure_fma_peak(int dbl, int iters, double* gflops, double* ms) {
  if (!gflops) return GFFT_E_NULL_POINTER;
  if (iters < 1) return GFFT_E_INVALID_PLAN;
  return dbl ? measure<double>(iters, gflops, ms) : measure<float>(iters, gflops, ms);
}
