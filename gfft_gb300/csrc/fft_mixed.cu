// Column tiles with compile-time mixed-radix passes (variant 7).
//
// The pipeline of the power-of-two column-tile kernel (fft_spec.cu, variant
// 5): persistent blocks, the next tile of W adjacent columns gathered with
// cp.async into a second padded buffer while the current one is
// transformed, the four-step twiddle applied by each thread to what it
// gathered, a coalesced store.  The in-block passes follow a radix sequence
// fixed at compile time (mixed_shapes.h), so butterfly counts, strides and
// padded offsets are constants.  The passes ping-pong between the current
// tile's buffer and a work buffer (three padded buffers in all, two blocks
// per SM), one butterfly live per thread at a time.
#include <cuda_runtime.h>
#include <stdint.h>

#include "butterflies.cuh"
#include "mixed_shapes.h"
#include "plan.h"
#include "spec.cuh"

namespace gfft {
namespace mixed {

constexpr int NT = 256;
template <typename T> struct Cfg;
template <> struct Cfg<float> {
  static constexpr int TILE = 4096, PS = 4;
};
template <> struct Cfg<double> {
  static constexpr int TILE = 2048, PS = 3;
};
constexpr int lanes(int L, int tile) { return (2 * L <= tile) ? 2 * lanes(2 * L, tile) : 1; }
// padded index: one slot per 2^PS values and one more per 2^(PS+4), so that
// strides of 2^(PS+4) values (which the first term alone turns into a
// multiple of the 128-byte bank window) land on different banks
template <typename T> __device__ __forceinline__ constexpr int padi(int s) {
  return s + (s >> Cfg<T>::PS) + (s >> (Cfg<T>::PS + 4));
}
// per-lane stride: odd (in elements), so that the lanes of a tile read at one
// sample index fall on different banks; equals engine_padded (plan.h)
template <typename T> constexpr int padded_len(int L) {
  return (L + (L >> Cfg<T>::PS) + (L >> (Cfg<T>::PS + 4)) + 1) | 1;
}

template <typename T, int L, int W>
__device__ __forceinline__ void gather(const EngineArgs& a, typename Vec<T>::t* buf, long long tile) {
  typedef typename Vec<T>::t V;
  constexpr int LP = padded_len<T>(L);
  const int lane = threadIdx.x % W;
  const long long u = tile * W + lane;
  if (u >= a.nunits) return;
  const long long t = u / a.stride;
  const long long b = u - t * a.stride;
  const V* src = (const V*)a.in + t * a.N + b;
  V* bl = buf + lane * LP;
  for (int s = threadIdx.x / W; s < L; s += NT / W)
    lanep2::cpa<T>(lanep2::sa(bl + padi<T>(s)), src + (long long)s * a.stride);
}

template <typename T, int L, int W>
__device__ __forceinline__ void sweep(const EngineArgs& a, typename Vec<T>::t* buf, long long tile) {
  typedef typename Vec<T>::t V;
  constexpr int LP = padded_len<T>(L);
  const int lane = threadIdx.x % W;
  const long long u = tile * W + lane;
  const unsigned b = (unsigned)(u % a.stride);
  const unsigned k = b % (unsigned)a.gNs;
  const unsigned kstep = a.notw ? 0u : k * (unsigned)(a.N / (a.gNs * L));
  if (!kstep && !a.conj) return;
  V* bl = buf + lane * LP;
  const V* lo = (const V*)a.gtw_lo;
  const V* hi = (const V*)a.gtw_hi;
  const unsigned mask = (unsigned)a.gB - 1;
  const int lgB = 31 - __clz((int)a.gB);
  for (int s = threadIdx.x / W; s < L; s += NT / W) {
    V x = bl[padi<T>(s)];
    if (a.conj) x = cconj(x);
    if (kstep) {
      const unsigned m = kstep * (unsigned)s;  // < N < 2^32
      x = cmul(x, cmul(__ldg(lo + (m & mask)), __ldg(hi + (m >> lgB))));
    }
    bl[padi<T>(s)] = x;
  }
}

// one radix-R pass (butterflies over W lanes x L / R): src -> dst
template <typename T, int L, int W, int R, int NS>
__device__ __forceinline__ void pass(const typename Vec<T>::t* __restrict__ src, typename Vec<T>::t* __restrict__ dst,
                                     const typename Vec<T>::t* __restrict__ tw, int twoff) {
  typedef typename Vec<T>::t V;
  constexpr int NB = L / R, TOT = W * NB;
  constexpr int LP = padded_len<T>(L);
  for (int i = threadIdx.x; i < TOT; i += NT) {
    const int lane = i / NB, j = i % NB, k = j % NS;
    const V* s = src + lane * LP;
    V v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = s[padi<T>(j + r * NB)];
    if constexpr (NS > 1) {
      const V* t = tw + twoff + k;
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = cmul(v[r], __ldg(t + (r - 1) * NS));
    }
    dft<T, V, R>(v);
    V* d = dst + lane * LP;
    const int base = (j - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) d[padi<T>(base + r * NS)] = v[r];
  }
  __syncthreads();
}

}  // namespace mixed

template <typename T, int R0, int R1, int R2, int R3>
__global__ void __launch_bounds__(mixed::NT, 2) mixed_kernel(const __grid_constant__ EngineArgs a) {
  using namespace mixed;
  typedef typename Vec<T>::t V;
  constexpr int L = R0 * R1 * R2 * R3;
  constexpr int W = lanes(L, Cfg<T>::TILE);
  constexpr int LP = padded_len<T>(L);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* const bufs0 = reinterpret_cast<V*>(smem_raw);  // gathered tiles (current / next)
  V* const bufs1 = bufs0 + W * LP;
  V* const work = bufs1 + W * LP;  // ping-pong partner of the current tile's buffer
  const V* tw = (const V*)a.tw;
  const long long G = gridDim.x;
  const T sc = (T)a.scale;
  long long tile = blockIdx.x;
  if (tile >= a.ntiles) return;
  gather<T, L, W>(a, bufs0, tile);
  asm volatile("cp.async.commit_group;" ::: "memory");
  for (int it = 0; tile < a.ntiles; tile += G, ++it) {
    V* cur = (it & 1) ? bufs1 : bufs0;
    V* nxt = (it & 1) ? bufs0 : bufs1;
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    sweep<T, L, W>(a, cur, tile);
    __syncthreads();
    if (tile + G < a.ntiles) gather<T, L, W>(a, nxt, tile + G);
    asm volatile("cp.async.commit_group;" ::: "memory");
    pass<T, L, W, R0, 1>(cur, work, tw, a.pass[0].tw);
    V* res = work;
    if constexpr (R1 > 1) {
      pass<T, L, W, R1, R0>(work, cur, tw, a.pass[1].tw);
      res = cur;
    }
    if constexpr (R2 > 1) {
      pass<T, L, W, R2, R0 * R1>(cur, work, tw, a.pass[2].tw);
      res = work;
    }
    if constexpr (R3 > 1) {
      pass<T, L, W, R3, R0 * R1 * R2>(work, cur, tw, a.pass[3].tw);
      res = cur;
    }
    const long long u0 = tile * W;
    if (a.gNs == 1) {
      // each lane's outputs are contiguous: lanes of the tile lie back to back
      const long long t = u0 / a.stride;
      const long long b0 = u0 - t * a.stride;
      V* dst = (V*)a.out + t * a.N + b0 * L;
      const int units = (int)((a.nunits - u0) < W ? (a.nunits - u0) : W);
      for (int i = threadIdx.x; i < units * L; i += NT) {
        const int lane = i / L, s = i - lane * L;
        V x = res[lane * LP + padi<T>(s)];
        if (a.conj) x = cconj(x);
        dst[i] = cscale(x, sc);
      }
    } else {
      const int lane = threadIdx.x % W;
      const long long u = u0 + lane;
      if (u < a.nunits) {
        const long long tt = u / a.stride;
        const long long b = u - tt * a.stride;
        const long long k = b % a.gNs;
        V* dst = (V*)a.out + tt * a.N + (b - k) * L + k;
        const V* bl = res + lane * LP;
        for (int s = threadIdx.x / W; s < L; s += NT / W) {
          V x = bl[padi<T>(s)];
          if (a.conj) x = cconj(x);
          dst[(long long)s * a.gNs] = cscale(x, sc);
        }
      }
    }
    __syncthreads();
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
}

}  // namespace gfft

namespace {
template <typename T>
const void* mixed_fn(int idx) {
  switch (idx) {
    case 0: return (const void*)gfft::mixed_kernel<T, 16, 16, 3, 1>;
    case 1: return (const void*)gfft::mixed_kernel<T, 5, 5, 5, 5>;
    case 2: return (const void*)gfft::mixed_kernel<T, 16, 12, 3, 1>;
    case 3: return (const void*)gfft::mixed_kernel<T, 16, 9, 3, 1>;
    case 4: return (const void*)gfft::mixed_kernel<T, 10, 10, 10, 1>;
    case 5: return (const void*)gfft::mixed_kernel<T, 9, 9, 9, 1>;
    case 6: return (const void*)gfft::mixed_kernel<T, 16, 15, 2, 1>;
    case 7: return (const void*)gfft::mixed_kernel<T, 15, 12, 2, 1>;
    default: return nullptr;
  }
}
const void* fn_for(int dbl, const EngineArgs* a) {
  int rs[4];
  for (int i = 0; i < a->npass && i < 4; ++i) rs[i] = a->pass[i].R;
  const int idx = a->npass <= 4 ? mixed_shape_index(a->L, rs, a->npass) : -1;
  return dbl ? mixed_fn<double>(idx) : mixed_fn<float>(idx);
}
}  // namespace

extern "C" int gfft_mixed_setup(int dbl, size_t max_smem) {
  int e = 0;
  for (int i = 0; i < kNumMixedShapes; ++i) {
    const void* f = dbl ? mixed_fn<double>(i) : mixed_fn<float>(i);
    e |= cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem) != cudaSuccess;
  }
  return e;
}

extern "C" int gfft_mixed_occupancy(int dbl, const EngineArgs* a, int threads, size_t smem) {
  const void* f = fn_for(dbl, a);
  if (!f) return 0;
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f, threads, smem);
  return n;
}

extern "C" int gfft_mixed_launch(int dbl, const EngineArgs* a, unsigned grid, unsigned threads, size_t smem,
                                 cudaStream_t stream) {
  const void* f = fn_for(dbl, a);
  if (!f) return (int)cudaErrorInvalidValue;
  cudaGetLastError();  // clear a stale error of an earlier, unrelated call
  void* args[] = {(void*)a};
  return (int)cudaLaunchKernel(f, dim3(grid), dim3(threads), args, smem, stream);
}
