// Pipelined column-tile kernel for the passes of a multi-pass transform
// (variant 4).
//
// A global pass of super-radix L over a length-N transform is a batch of
// DFT_L over "lanes": lane b reads samples b, b + S, b + 2S, ... (S = N / L),
// multiplies them by the four-step twiddles W_N^{(b mod Ns) s N/(Ns L)} and
// writes its outputs with stride Ns (plan.h).  A tile is W adjacent lanes x L
// samples.  The engine kernel (fft_engine.cu) runs one tile per block and
// waits for its loads; here blocks are persistent and hide that wait:
//
//   - three padded [lane][sample] shared buffers: one receives the NEXT tile
//     through 8/16-byte cp.async copies (any stride works, unlike tensor-map
//     copies that need 16-byte-multiple row strides: 5^8 = 625 x 625 has
//     5000-byte FP32 rows) while the other two ping-pong the in-block
//     Stockham passes of the current tile (engine.cuh block_pass);
//   - each thread conjugates (inverse) and twiddles the elements it gathered
//     itself, in place, before the first pass;
//   - the result leaves through the engine's lane-mode store: consecutive
//     threads write adjacent lanes, so every output row is one coalesced
//     segment.
#include <cuda_runtime.h>
#include <stdint.h>

#include "engine.cuh"

namespace gfft {
namespace lane {

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

template <typename T> __device__ __forceinline__ void cp_async(uint32_t dst, const void* src);
template <> __device__ __forceinline__ void cp_async<float>(uint32_t dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst), "l"(src) : "memory");
}
template <> __device__ __forceinline__ void cp_async<double>(uint32_t dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// gather tile `tile` into `buf` ([lane][pad(s)]); thread -> (lane = tid % W,
// samples tid / W + k * blockDim / W)
template <typename T>
__device__ __forceinline__ void gather(const EngineArgs& a, typename Vec<T>::t* buf, long long tile) {
  typedef typename Vec<T>::t V;
  const V* in = (const V*)a.in;
  const int W = a.W, L = a.L;
  const int lane = threadIdx.x % W;
  const long long u = tile * W + lane;
  if (u >= a.nunits) return;  // lanes past the end are computed on stale data and never stored
  const long long t = u / a.stride;
  const long long b = u - t * a.stride;
  const V* src = in + t * a.N + b;
  V* bl = buf + lane * a.Lp;
  const int sstep = blockDim.x / W;
  for (int s = threadIdx.x / W; s < L; s += sstep) cp_async<T>(saddr(bl + pad<T>(s)), src + (long long)s * a.stride);
}

// conjugation and four-step twiddle on the elements this thread gathered
template <typename T>
__device__ __forceinline__ void twiddle_sweep(const EngineArgs& a, typename Vec<T>::t* buf, long long tile) {
  typedef typename Vec<T>::t V;
  const int W = a.W, L = a.L;
  const int lane = threadIdx.x % W;
  const long long u = tile * W + lane;
  const long long b = u % a.stride;
  const long long k = b % a.gNs;
  const long long kstep = a.notw ? 0 : k * (a.N / (a.gNs * L));
  if (!kstep && !a.conj) return;
  V* bl = buf + lane * a.Lp;
  const int sstep = blockDim.x / W;
  const int lgB = 63 - __clzll(a.gB);
  for (int s = threadIdx.x / W; s < L; s += sstep) {
    V x = bl[pad<T>(s)];
    if (a.conj) x = cconj(x);
    if (kstep) x = cmul(x, global_twiddle<T>(a, kstep * s, lgB));
    bl[pad<T>(s)] = x;
  }
}

}  // namespace lane

// launch bounds (threads, resident blocks per SM) the registers are sized
// for: FP32 launches 512-thread blocks and fits 64 registers (two blocks,
// 32 warps per SM); FP64 launches 256-thread blocks (planner.cpp)
template <typename T> struct LaneCfg;
template <> struct LaneCfg<float> {
  static constexpr int NT = 512, MINB = 2;
};
template <> struct LaneCfg<double> {
  static constexpr int NT = 512, MINB = 1;
};

template <typename T>
__global__ void __launch_bounds__(LaneCfg<T>::NT, LaneCfg<T>::MINB) lane_kernel(const __grid_constant__ EngineArgs a) {
  using namespace lane;
  typedef typename Vec<T>::t V;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* const in_buf = reinterpret_cast<V*>(smem_raw);  // receives the next tile
  V* const x0 = in_buf + a.W * a.Lp;
  V* const x1 = x0 + a.W * a.Lp;
  const V* tw = (const V*)a.tw;
  const long long G = gridDim.x;
  long long tile = blockIdx.x;
  if (tile >= a.ntiles) return;
  gather<T>(a, in_buf, tile);
  cp_commit();
  for (; tile < a.ntiles; tile += G) {
    cp_wait_all();  // this thread's copies of the current tile
    twiddle_sweep<T>(a, in_buf, tile);
    __syncthreads();
    // the first pass reads the gathered buffer; the next tile may then refill it
    V* src = in_buf;
    V* dst = x0;
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
      if (p == 0) {
        const long long next = tile + G;
        if (next < a.ntiles) gather<T>(a, in_buf, next);
        cp_commit();
        src = x0;
        dst = x1;
      } else {
        V* t = src;
        src = dst;
        dst = t;
      }
    }
    store_tile<T>(a, src, tile * a.W);
    __syncthreads();
  }
  cp_wait_all();
}

}  // namespace gfft

extern "C" int gfft_lane_setup(int dbl, size_t max_smem) {
  cudaError_t e;
  if (dbl)
    e = cudaFuncSetAttribute(gfft::lane_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);
  else
    e = cudaFuncSetAttribute(gfft::lane_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);
  return e == cudaSuccess ? 0 : (int)e;
}

extern "C" int gfft_lane_occupancy(int dbl, int threads, size_t smem) {
  int n = 0;
  if (dbl)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, gfft::lane_kernel<double>, threads, smem);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, gfft::lane_kernel<float>, threads, smem);
  return n;
}

extern "C" int gfft_lane_launch(int dbl, const EngineArgs* a, unsigned grid, unsigned threads, size_t smem,
                                cudaStream_t stream) {
  cudaGetLastError();  // clear a stale error of an earlier, unrelated call
  if (dbl) gfft::lane_kernel<double><<<grid, threads, smem, stream>>>(*a);
  else gfft::lane_kernel<float><<<grid, threads, smem, stream>>>(*a);
  return (int)cudaGetLastError();
}
