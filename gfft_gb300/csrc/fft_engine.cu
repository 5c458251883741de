// Batched Stockham FFT engine for sm_103a.
//
// One launch = one global pass (see plan.h).  A thread block owns `W` units
// (whole short transforms, or W adjacent columns of a long one), stages them
// into shared memory with coalesced loads, runs the in-block radix passes
// between two padded shared buffers, and writes the result back with
// coalesced stores.  This replaces the reference's run-time path:
//   InTimeOOP / InTime recursion      src/gfftalg.h:383-507
//   DFTk_x_Im_T combine + recurrence  src/gfftalg.h:157-367, src/twiddles.h:212-339
//   GFFTswap2 digit reversal          src/gfftswap.h:74-227 (not needed: autosort)
//   Separate (real pre/post pass)     src/gfftswap.h:239-336, fused here
//   Backward 1/N scaling              src/gfftswap.h:355-374, fused into the store
//   OpenMP ParallLoop                 src/gfftomp.h:41-189 -> the block grid
#include <cuda_runtime.h>

#include "engine.cuh"

namespace gfft {

template <typename T>
__global__ void __launch_bounds__(512) engine_kernel(const __grid_constant__ EngineArgs a) {
  typedef typename Vec<T>::t V;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* b0 = reinterpret_cast<V*>(smem_raw);
  V* b1 = b0 + a.W * a.Lp;
  const long long u0 = (long long)blockIdx.x * a.W;
  const V* tw = (const V*)a.tw;
  load_tile<T>(a, b0, u0);
  __syncthreads();
  V* src = b0;
  V* dst = b1;
  if (a.dif) {
    // frequency decimation: the transposed passes in reverse order
    for (int p = a.npass - 1; p >= 0; --p) {
      const BlockPass bp = a.pass[p];
      switch (bp.R) {
        case 16: block_pass_dif<T, 16>(src, dst, a, bp, tw); break;
        case 8: block_pass_dif<T, 8>(src, dst, a, bp, tw); break;
        case 4: block_pass_dif<T, 4>(src, dst, a, bp, tw); break;
        case 2: block_pass_dif<T, 2>(src, dst, a, bp, tw); break;
        case 3: block_pass_dif<T, 3>(src, dst, a, bp, tw); break;
        case 5: block_pass_dif<T, 5>(src, dst, a, bp, tw); break;
        case 7: block_pass_dif<T, 7>(src, dst, a, bp, tw); break;
        case 6: block_pass_dif<T, 6>(src, dst, a, bp, tw); break;
        case 9: block_pass_dif<T, 9>(src, dst, a, bp, tw); break;
        case 10: block_pass_dif<T, 10>(src, dst, a, bp, tw); break;
        case 12: block_pass_dif<T, 12>(src, dst, a, bp, tw); break;
        case 15: block_pass_dif<T, 15>(src, dst, a, bp, tw); break;
        default: block_pass_generic_dif<T>(src, dst, a, bp, tw); break;
      }
      __syncthreads();
      V* t = src;
      src = dst;
      dst = t;
    }
    store_tile<T>(a, src, u0);
    return;
  }
  for (int p = 0; p < a.npass; ++p) {
    const BlockPass bp = a.pass[p];
    switch (bp.R) {
      case 16: block_pass<T, 16>(src, dst, a, bp, tw); break;
      case 8: block_pass<T, 8>(src, dst, a, bp, tw); break;
      case 4: block_pass<T, 4>(src, dst, a, bp, tw); break;
      case 2: block_pass<T, 2>(src, dst, a, bp, tw); break;
      case 3: block_pass<T, 3>(src, dst, a, bp, tw); break;
      case 5: block_pass<T, 5>(src, dst, a, bp, tw); break;
      case 7: block_pass<T, 7>(src, dst, a, bp, tw); break;
      case 6: block_pass<T, 6>(src, dst, a, bp, tw); break;
      case 9: block_pass<T, 9>(src, dst, a, bp, tw); break;
      case 10: block_pass<T, 10>(src, dst, a, bp, tw); break;
      case 12: block_pass<T, 12>(src, dst, a, bp, tw); break;
      case 15: block_pass<T, 15>(src, dst, a, bp, tw); break;
      default: block_pass_generic<T>(src, dst, a, bp, tw); break;
    }
    __syncthreads();
    V* t = src;
    src = dst;
    dst = t;
  }
  store_tile<T>(a, src, u0);
}

// Real pre/post pass for multi-pass lengths (not fused): in place on
// `batch` transforms of n complex slots.  dir=1 forward post (Z -> X),
// dir=2 inverse pre (X -> Z).
template <typename T>
__global__ void real_pass_kernel(typename Vec<T>::t* data, long long n, long long batch, int dir,
                                 const typename Vec<T>::t* __restrict__ rtw) {
  typedef typename Vec<T>::t V;
  const long long half = n / 2 + 1;
  const long long total = half * batch;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long t = i / half;
    const long long q = i - t * half;
    V* y = data + t * n;
    if (q == 0) {
      const V z0 = y[0];
      if (dir == 1) y[0] = mk<V>(z0.x + z0.y, z0.x - z0.y);
      else y[0] = mk<V>((T)0.5 * (z0.x + z0.y), (T)0.5 * (z0.x - z0.y));
      continue;
    }
    const long long qm = n - q;
    if (q > qm) continue;
    const V a = y[q], b = y[qm];
    if (dir == 1) {
      V F = mk<V>((T)0.5 * (a.x + b.x), (T)0.5 * (a.y - b.y));
      V G = mk<V>((T)0.5 * (a.y + b.y), (T)-0.5 * (a.x - b.x));
      V xq = cadd(F, cmul(__ldg(rtw + q), G));
      V F2 = mk<V>((T)0.5 * (b.x + a.x), (T)0.5 * (b.y - a.y));
      V G2 = mk<V>((T)0.5 * (b.y + a.y), (T)-0.5 * (b.x - a.x));
      V xm = cadd(F2, cmul(__ldg(rtw + qm), G2));
      y[q] = xq;
      if (qm != q) y[qm] = xm;
    } else {
      V F = mk<V>((T)0.5 * (a.x + b.x), (T)0.5 * (a.y - b.y));
      V D = mk<V>((T)0.5 * (a.x - b.x), (T)0.5 * (a.y + b.y));
      V G = cmul(D, cconj(__ldg(rtw + q)));
      V zq = mk<V>(F.x - G.y, F.y + G.x);
      V F2 = mk<V>((T)0.5 * (b.x + a.x), (T)0.5 * (b.y - a.y));
      V D2 = mk<V>((T)0.5 * (b.x - a.x), (T)0.5 * (b.y + a.y));
      V G2 = cmul(D2, cconj(__ldg(rtw + qm)));
      V zm = mk<V>(F2.x - G2.y, F2.y + G2.x);
      y[q] = zq;
      if (qm != q) y[qm] = zm;
    }
  }
}

}  // namespace gfft

// host-side launchers (called from gfft_capi.cpp)
extern "C" int gfft_engine_setup(int dbl, size_t max_smem) {
  cudaError_t e;
  if (dbl)
    e = cudaFuncSetAttribute(gfft::engine_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);
  else
    e = cudaFuncSetAttribute(gfft::engine_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);
  return e == cudaSuccess ? 0 : (int)e;
}

extern "C" int gfft_engine_launch(int dbl, const EngineArgs* a, unsigned grid, unsigned threads, size_t smem,
                                  cudaStream_t stream) {
  cudaGetLastError();  // clear a stale error of an earlier, unrelated call
  if (dbl) gfft::engine_kernel<double><<<grid, threads, smem, stream>>>(*a);
  else gfft::engine_kernel<float><<<grid, threads, smem, stream>>>(*a);
  return (int)cudaGetLastError();
}

extern "C" int gfft_real_pass_launch(int dbl, void* data, long long n, long long batch, int dir, const void* rtw,
                                     cudaStream_t stream) {
  cudaGetLastError();  // clear a stale error of an earlier, unrelated call
  long long total = (n / 2 + 1) * batch;
  unsigned threads = 256;
  long long blocks = (total + threads - 1) / threads;
  if (blocks > 152LL * 16) blocks = 152LL * 16;
  if (blocks < 1) blocks = 1;
  if (dbl)
    gfft::real_pass_kernel<double><<<(unsigned)blocks, threads, 0, stream>>>((double2*)data, n, batch, dir,
                                                                            (const double2*)rtw);
  else
    gfft::real_pass_kernel<float><<<(unsigned)blocks, threads, 0, stream>>>((float2*)data, n, batch, dir,
                                                                          (const float2*)rtw);
  return (int)cudaGetLastError();
}
