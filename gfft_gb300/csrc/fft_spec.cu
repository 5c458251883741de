// Length-specialised register-resident TMA-pipelined FFT (variant 3).
//
// The same pipeline as fft_fast.cu (persistent blocks, tiles of W whole
// transforms streamed into shared memory by 1-D bulk async copies, 16 values
// per thread, in-block Stockham passes in shared memory, the last pass
// stored straight to global memory), but with the power-of-two length L a
// template parameter: the pass radices, butterfly strides and twiddle strides
// are compile-time constants, so every shared-memory access is a register
// base plus an immediate offset and the index arithmetic per leg vanishes.
// The tile holds 4096 (FP32) or 2048 (FP64) complex values, W = tile / L;
// FP32 8192 runs one transform per tile with 512 threads.
//
// Pass order for L = 2^a: radix 16 while four bits remain, then 8 / 4 / 2,
// matching the planner's default (planner.cpp block_radices).
#include <cuda_runtime.h>
#include <stdint.h>

#include "butterflies.cuh"
#include "plan.h"
#include "spec.cuh"
#include "tma.cuh"

namespace gfft {

template <typename T, int L>
__global__ void __launch_bounds__(spec::tile_of<T>(L) / 16, 1) spec_kernel(const __grid_constant__ EngineArgs a) {
  using namespace spec;
  using namespace fast;
  typedef typename Vec<T>::t V;
  constexpr int TILE = tile_of<T>(L), W = TILE / L, NP = npass_of(L);
  constexpr int LP = L + (L >> Cfg<T>::PS) + 1;
  constexpr int TB = TILE * (int)sizeof(V);  // bytes of a full tile (multiple of 128)
  extern __shared__ __align__(128) unsigned char smem[];
  const int S = a.stages;
  unsigned char* stage0 = smem;
  V* work = reinterpret_cast<V*>(smem + (size_t)S * TB);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + (size_t)S * TB + (((size_t)W * LP * sizeof(V) + 7) & ~7));
  const V* in = (const V*)a.in;
  V* out = (V*)a.out;
  const V* tw = (const V*)a.tw;
  const bool conj = a.conj != 0;
  const T sc = (T)a.scale;
  const long long G = gridDim.x;

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) mbar_init(saddr(&bars[s]), 1);
    mbar_fence_init();
  }
  __syncthreads();

  auto issue = [&](long long tile, int s) {
    const long long u0 = tile * W;
    const long long left = a.nunits - u0;
    const int units = left < W ? (int)left : W;
    const uint32_t bytes = (uint32_t)units * (uint32_t)L * (uint32_t)sizeof(V);
    const uint32_t bar = saddr(&bars[s]);
    mbar_expect_tx(bar, bytes);
    bulk_load(saddr(stage0 + (size_t)s * TB), in + u0 * L, bytes, bar);
  };
  if (threadIdx.x == 0 && !a.debug_no_issue)
    for (int s = 0; s < S; ++s) {
      const long long tile = blockIdx.x + (long long)s * G;
      if (tile < a.ntiles) issue(tile, s);
    }

  int it = 0;
  V v[16];
  for (long long tile = blockIdx.x; tile < a.ntiles; tile += G, ++it) {
    const int s = it % S;
    const uint32_t ph = (uint32_t)((it / S) & 1);
    const bool ok = mbar_wait_bounded(saddr(&bars[s]), ph, a.spin_limit);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        atomicExch(a.status, 13 /* GFFT_E_TIMEOUT */);
        if (!a.debug_no_issue)
          for (int k = 1; k < S; ++k) {
            const long long t2 = tile + (long long)k * G;
            if (t2 >= a.ntiles) break;
            const int j = it + k;
            mbar_wait_bounded(saddr(&bars[j % S]), (uint32_t)((j / S) & 1), a.spin_limit);
          }
      }
      return;
    }
    const long long u0 = tile * W;
    const long long left = a.nunits - u0;
    const int units = left < W ? (int)left : W;
    const V* st = reinterpret_cast<const V*>(stage0 + (size_t)s * TB);
    V* o = out + u0 * L;

    sread<T, L, 0, true>(v, st);
    if (conj)
#pragma unroll
      for (int i = 0; i < 16; ++i) v[i] = cconj(v[i]);
    scompute<T, L, 0>(v, tw, a.pass[0].tw);
    __syncthreads();  // stage s read by every thread; the previous tile's reads of `work` are done
    if (threadIdx.x == 0 && !a.debug_no_issue) {
      const long long nt = tile + (long long)S * G;
      if (nt < a.ntiles) issue(nt, s);
    }
    if constexpr (NP == 1) {
      sstore<T, L, 0>(v, o, units, conj, sc);
    } else {
      swrite<T, L, 0>(v, work);
      __syncthreads();
      rest<T, L, 1>(v, work, tw, a.pass, o, units, conj, sc);
    }
  }
}


// One transform per block with no stage (stages = 0): the whole transform in
// the registers of L / 16 threads (16 values each); the first pass loads
// straight from global memory (consecutive threads read consecutive
// elements of each leg: coalesced), the middle passes go through the padded
// work buffer and the last pass stores straight to global memory; the next
// transform's loads are issued while other warps still finish the previous
// one's last pass.  FP32 16384 (one block of 1024 threads per SM: a stage
// and the work buffer would not both fit the shared memory), 8192 / 4096
// with MINB = 2 / 4 blocks per SM (64 registers; the blocks of an SM hide
// each other's load latency, no stage needed).
template <typename T, int L, int MINB>
__global__ void __launch_bounds__(L / 16, MINB) spec_direct_kernel(const __grid_constant__ EngineArgs a) {
  using namespace spec;
  typedef typename Vec<T>::t V;
  static_assert(L >= Cfg<T>::TILE, "one transform per block");
  constexpr int NP = npass_of(L);
  static_assert(NP > 1, "two or more passes");
  extern __shared__ __align__(128) unsigned char smem[];
  V* work = reinterpret_cast<V*>(smem);
  const V* in = (const V*)a.in;
  V* out = (V*)a.out;
  const V* tw = (const V*)a.tw;
  const bool conj = a.conj != 0;
  const T sc = (T)a.scale;
  V v[16];
  for (long long t = blockIdx.x; t < a.nunits; t += gridDim.x) {
    sread<T, L, 0, true>(v, in + t * L);  // global loads, 16 in flight per thread
    if (conj)
#pragma unroll
      for (int i = 0; i < 16; ++i) v[i] = cconj(v[i]);
    scompute<T, L, 0>(v, tw, a.pass[0].tw);
    __syncthreads();  // the previous transform's last pass has read the work buffer
    swrite<T, L, 0>(v, work);
    __syncthreads();
    rest<T, L, 1>(v, work, tw, a.pass, out + t * L, 1, conj, sc);
  }
}

// ---- power-of-two column tiles of a multi-pass length (variant 5) --------
// The passes of spec_kernel, for the W = tile / L adjacent lanes of a global
// pass (plan.h): the next tile is gathered with 8/16-byte cp.async copies
// into the second of two padded buffers while the current one is
// transformed; each thread conjugates / applies the four-step twiddle to the
// elements it gathered, the in-block passes run in place with their legs in
// registers, and the result is stored either straight from registers (first
// global pass: each lane's outputs are contiguous) or, through the buffer,
// lane-fastest with stride Ns (later passes).
namespace lanep2 {

template <typename T, int L, int P>
__device__ __forceinline__ void passes(typename Vec<T>::t (&v)[16], typename Vec<T>::t* buf,
                                       const typename Vec<T>::t* tw, const BlockPass* bp) {
  constexpr int NP = spec::npass_of(L);
  if constexpr (P < NP) {
    spec::sread<T, L, P, false>(v, buf);
    spec::scompute<T, L, P>(v, tw, bp[P].tw);
    if constexpr (P < NP - 1) {
      __syncthreads();
      spec::swrite<T, L, P>(v, buf);
      __syncthreads();
      passes<T, L, P + 1>(v, buf, tw, bp);
    }
  }
}

}  // namespace lanep2

template <typename T, int L>
__global__ void __launch_bounds__(spec::Cfg<T>::TILE / 16, 2) lanep2_kernel(const __grid_constant__ EngineArgs a) {
  typedef typename Vec<T>::t V;
  constexpr int TILE = spec::Cfg<T>::TILE, W = TILE / L, NP = spec::npass_of(L), NT = TILE / 16;
  constexpr int LP = L + (L >> spec::Cfg<T>::PS) + 1;
  constexpr int NB = L / spec::radix_of(L, NP - 1);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* const bufs0 = reinterpret_cast<V*>(smem_raw);
  V* const bufs1 = bufs0 + W * LP;
  const V* tw = (const V*)a.tw;
  const long long G = gridDim.x;
  const T sc = (T)a.scale;
  long long tile = blockIdx.x;
  if (tile >= a.ntiles) return;
  lanep2::gather<T, L>(a, bufs0, tile);
  asm volatile("cp.async.commit_group;" ::: "memory");
  V v[16];
  for (int it = 0; tile < a.ntiles; tile += G, ++it) {
    V* cur = (it & 1) ? bufs1 : bufs0;
    V* nxt = (it & 1) ? bufs0 : bufs1;
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    lanep2::sweep<T, L>(a, cur, tile);
    __syncthreads();
    if (tile + G < a.ntiles) lanep2::gather<T, L>(a, nxt, tile + G);
    asm volatile("cp.async.commit_group;" ::: "memory");
    lanep2::passes<T, L, 0>(v, cur, tw, a.pass);
    // v holds the last pass: thread's butterflies b = tid + q*NT, lane = b / NB, j = b % NB,
    // leg r is sample j + r*NB of that lane
    const long long u0 = tile * W;
    const long long t = u0 / a.stride;
    const long long b0 = u0 - t * a.stride;
    const int units = (int)((a.nunits - u0) < W ? (a.nunits - u0) : W);
    if (a.gNs == 1) {
      spec::sstore<T, L, NP - 1>(v, (V*)a.out + t * a.N + b0 * L, units, a.conj != 0, sc);
    } else {
      __syncthreads();
      spec::swrite<T, L, NP - 1>(v, cur);  // last pass: Ns*R == L, natural order
      __syncthreads();
      const int lane = threadIdx.x % W;
      const long long u = u0 + lane;
      if (u < a.nunits) {
        const long long tt = u / a.stride;
        const long long b = u - tt * a.stride;
        const long long k = b % a.gNs;
        V* dst = (V*)a.out + tt * a.N + (b - k) * L + k;
        const V* bl = cur + lane * LP;
        for (int s = threadIdx.x / W; s < L; s += NT / W) {
          V x = bl[spec::padi<T>(s)];
          if (a.conj) x = cconj(x);
          dst[(long long)s * a.gNs] = cscale(x, sc);
        }
      }
    }
    (void)NB;
    __syncthreads();
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
}

}  // namespace gfft

namespace {
template <typename T, int L>
int spec_setup_one(size_t max_smem) {
  return cudaFuncSetAttribute(gfft::spec_kernel<T, L>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem) ==
                 cudaSuccess
             ? 0
             : 1;
}
template <typename T>
int spec_setup_all(size_t m) {
  int e = 0;
  e |= spec_setup_one<T, 16>(m);
  e |= spec_setup_one<T, 32>(m);
  e |= spec_setup_one<T, 64>(m);
  e |= spec_setup_one<T, 128>(m);
  e |= spec_setup_one<T, 256>(m);
  e |= spec_setup_one<T, 512>(m);
  e |= spec_setup_one<T, 1024>(m);
  e |= spec_setup_one<T, 2048>(m);
  return e;
}
template <typename T>
const void* spec_fn(int L) {
  switch (L) {
    case 16: return (const void*)gfft::spec_kernel<T, 16>;
    case 32: return (const void*)gfft::spec_kernel<T, 32>;
    case 64: return (const void*)gfft::spec_kernel<T, 64>;
    case 128: return (const void*)gfft::spec_kernel<T, 128>;
    case 256: return (const void*)gfft::spec_kernel<T, 256>;
    case 512: return (const void*)gfft::spec_kernel<T, 512>;
    case 1024: return (const void*)gfft::spec_kernel<T, 1024>;
    case 2048: return (const void*)gfft::spec_kernel<T, 2048>;
    case 4096: return sizeof(T) == 4 ? (const void*)gfft::spec_kernel<float, 4096> : nullptr;
    case 8192: return sizeof(T) == 4 ? (const void*)gfft::spec_kernel<float, 8192> : nullptr;
    default: return nullptr;
  }
}
}  // namespace

namespace {
// the stage-free one-transform-per-block kernels (FP32)
const void* direct_fn(int dbl, int L) {
  if (dbl) return nullptr;
  switch (L) {
    case 4096: return (const void*)gfft::spec_direct_kernel<float, 4096, 4>;
    case 8192: return (const void*)gfft::spec_direct_kernel<float, 8192, 2>;
    case 16384: return (const void*)gfft::spec_direct_kernel<float, 16384, 1>;
    default: return nullptr;
  }
}
}  // namespace

// lengths with a specialised kernel: FP32 16..16384, FP64 16..2048
extern "C" int gfft_spec_supported(int dbl, int L) {
  return direct_fn(dbl, L) != nullptr || (dbl ? spec_fn<double>(L) : spec_fn<float>(L)) != nullptr;
}

extern "C" int gfft_spec_setup(int dbl, size_t max_smem) {
  if (dbl) return spec_setup_all<double>(max_smem);
  int e = spec_setup_all<float>(max_smem);
  e |= spec_setup_one<float, 4096>(max_smem);
  e |= spec_setup_one<float, 8192>(max_smem);
  for (int L : {4096, 8192, 16384})
    e |= cudaFuncSetAttribute(direct_fn(0, L), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem) !=
         cudaSuccess;
  return e;
}


extern "C" int gfft_spec_occupancy(int dbl, int L, int stages, int threads, size_t smem) {
  const void* f = stages == 0 ? direct_fn(dbl, L) : (dbl ? spec_fn<double>(L) : spec_fn<float>(L));
  if (!f) return 0;
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f, threads, smem);
  return n;
}

extern "C" int gfft_spec_launch(int dbl, const EngineArgs* a, unsigned grid, unsigned threads, size_t smem,
                                cudaStream_t stream) {
  const void* f = a->stages == 0 ? direct_fn(dbl, a->L) : (dbl ? spec_fn<double>(a->L) : spec_fn<float>(a->L));
  if (!f) return (int)cudaErrorInvalidValue;
  void* args[] = {(void*)a};
  return (int)cudaLaunchKernel(f, dim3(grid), dim3(threads), args, smem, stream);
}

namespace {
template <typename T>
const void* lanep2_fn(int L) {
  switch (L) {
    case 64: return (const void*)gfft::lanep2_kernel<T, 64>;
    case 128: return (const void*)gfft::lanep2_kernel<T, 128>;
    case 256: return (const void*)gfft::lanep2_kernel<T, 256>;
    case 512: return (const void*)gfft::lanep2_kernel<T, 512>;
    case 1024: return (const void*)gfft::lanep2_kernel<T, 1024>;
    default: return nullptr;
  }
}
}  // namespace

extern "C" int gfft_lanep2_setup(int dbl, size_t max_smem) {
  int e = 0;
  for (int L : {64, 128, 256, 512, 1024}) {
    const void* f = dbl ? lanep2_fn<double>(L) : lanep2_fn<float>(L);
    e |= cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem) != cudaSuccess;
  }
  return e;
}

extern "C" int gfft_lanep2_occupancy(int dbl, int L, int threads, size_t smem) {
  const void* f = dbl ? lanep2_fn<double>(L) : lanep2_fn<float>(L);
  if (!f) return 0;
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f, threads, smem);
  return n;
}

extern "C" int gfft_lanep2_launch(int dbl, const EngineArgs* a, unsigned grid, unsigned threads, size_t smem,
                                  cudaStream_t stream) {
  const void* f = dbl ? lanep2_fn<double>(a->L) : lanep2_fn<float>(a->L);
  if (!f) return (int)cudaErrorInvalidValue;
  cudaGetLastError();  // clear a stale error of an earlier, unrelated call
  void* args[] = {(void*)a};
  return (int)cudaLaunchKernel(f, dim3(grid), dim3(threads), args, smem, stream);
}
