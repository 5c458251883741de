// Register-resident, TMA-pipelined single-pass FFT for sm_103a (variant 2).
//
// For batched transforms of a power-of-two length L (16 <= L <= 8192 FP32,
// <= 4096 FP64) whose radices all divide 16.  A persistent block loops over
// tiles of W whole transforms (one contiguous chunk of memory each):
//
//   - one elected thread streams the next tiles into `stages` shared-memory
//     buffers with 1-D bulk async copies (cp.async.bulk ... mbarrier
//     complete_tx), so HBM reads run ahead of the arithmetic without holding
//     registers;
//   - every thread owns 16 complex values; each in-block Stockham pass reads
//     its butterflies' legs from shared memory, applies the twiddles and a
//     radix-16/8/4/2 butterfly in registers, and writes them back (in place:
//     all reads, a barrier, all writes);
//   - the first pass reads the bulk-copied tile, the last pass writes the
//     results straight to global memory (coalesced: consecutive threads,
//     consecutive addresses).
//
// Every mbarrier wait is bounded (EngineArgs::spin_limit); a wait that runs
// out sets the status word to GFFT_E_TIMEOUT, waits (bounded) for the copies
// this block still has in flight, and returns.
#include <cuda_runtime.h>
#include <stdint.h>

#include "butterflies.cuh"
#include "plan.h"
#include "tma.cuh"

namespace gfft {

namespace fast {

template <typename T> struct PadShift;
template <> struct PadShift<float> { static constexpr int v = 4; };
template <> struct PadShift<double> { static constexpr int v = 3; };
template <typename T> __device__ __forceinline__ int pad(int s) { return s + (s >> PadShift<T>::v); }

// Q = 16/R butterflies per thread; butterfly q of thread t is b = t + q*T
template <typename T, int R>
__device__ __forceinline__ void read_legs(typename Vec<T>::t (&v)[16], const typename Vec<T>::t* src, bool padded,
                                          int Lstride, int lgnb, int T_) {
  constexpr int Q = 16 / R;
  const int nb = 1 << lgnb;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int b = threadIdx.x + q * T_;
    const int lane = b >> lgnb;
    const int j = b & (nb - 1);
    const typename Vec<T>::t* s = src + lane * Lstride;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int e = j + r * nb;
      v[q * R + r] = s[padded ? pad<T>(e) : e];
    }
  }
}

template <typename T, int R>
__device__ __forceinline__ void twiddle_dft(typename Vec<T>::t (&v)[16], const typename Vec<T>::t* __restrict__ tw,
                                            int twoff, int lgnb, int lgNs, int T_) {
  typedef typename Vec<T>::t V;
  constexpr int Q = 16 / R;
  const int nb = 1 << lgnb;
  const int Ns = 1 << lgNs;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    if (Ns > 1) {
      const int b = threadIdx.x + q * T_;
      const int j = b & (nb - 1);
      const int k = j & (Ns - 1);
      const V* t = tw + twoff + k;
#pragma unroll
      for (int r = 1; r < R; ++r) v[q * R + r] = cmul(v[q * R + r], __ldg(t + (r - 1) * Ns));
    }
    dft<T, V, R>(&v[q * R]);
  }
}

template <typename T, int R>
__device__ __forceinline__ void write_legs_smem(const typename Vec<T>::t (&v)[16], typename Vec<T>::t* dst, int Lp,
                                                int lgnb, int lgNs, int T_) {
  constexpr int Q = 16 / R;
  const int nb = 1 << lgnb;
  const int Ns = 1 << lgNs;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int b = threadIdx.x + q * T_;
    const int lane = b >> lgnb;
    const int j = b & (nb - 1);
    const int k = j & (Ns - 1);
    const int base = (j - k) * R + k;
    typename Vec<T>::t* d = dst + lane * Lp;
#pragma unroll
    for (int r = 0; r < R; ++r) d[pad<T>(base + r * Ns)] = v[q * R + r];
  }
}

// last pass: Ns*R == L, so the output index of leg r is j + r*nb
template <typename T, int R>
__device__ __forceinline__ void write_legs_global(const typename Vec<T>::t (&v)[16], typename Vec<T>::t* out, int L,
                                                  int lgnb, int T_, int units, bool conj, T sc) {
  typedef typename Vec<T>::t V;
  constexpr int Q = 16 / R;
  const int nb = 1 << lgnb;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int b = threadIdx.x + q * T_;
    const int lane = b >> lgnb;
    const int j = b & (nb - 1);
    if (lane >= units) continue;
    V* d = out + (long long)lane * L;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      V x = v[q * R + r];
      if (conj) x = cconj(x);
      d[j + r * nb] = cscale(x, sc);
    }
  }
}

__device__ __forceinline__ int ilog2(int x) { return 31 - __clz(x); }

template <typename T>
__device__ __forceinline__ void do_read(int R, typename Vec<T>::t (&v)[16], const typename Vec<T>::t* src, bool padded,
                                        int Ls, int lgnb, int T_) {
  switch (R) {
    case 16: read_legs<T, 16>(v, src, padded, Ls, lgnb, T_); break;
    case 8: read_legs<T, 8>(v, src, padded, Ls, lgnb, T_); break;
    case 4: read_legs<T, 4>(v, src, padded, Ls, lgnb, T_); break;
    default: read_legs<T, 2>(v, src, padded, Ls, lgnb, T_); break;
  }
}
template <typename T>
__device__ __forceinline__ void do_compute(int R, typename Vec<T>::t (&v)[16], const typename Vec<T>::t* tw, int twoff,
                                           int lgnb, int lgNs, int T_) {
  switch (R) {
    case 16: twiddle_dft<T, 16>(v, tw, twoff, lgnb, lgNs, T_); break;
    case 8: twiddle_dft<T, 8>(v, tw, twoff, lgnb, lgNs, T_); break;
    case 4: twiddle_dft<T, 4>(v, tw, twoff, lgnb, lgNs, T_); break;
    default: twiddle_dft<T, 2>(v, tw, twoff, lgnb, lgNs, T_); break;
  }
}
template <typename T>
__device__ __forceinline__ void do_write_smem(int R, const typename Vec<T>::t (&v)[16], typename Vec<T>::t* dst, int Lp,
                                              int lgnb, int lgNs, int T_) {
  switch (R) {
    case 16: write_legs_smem<T, 16>(v, dst, Lp, lgnb, lgNs, T_); break;
    case 8: write_legs_smem<T, 8>(v, dst, Lp, lgnb, lgNs, T_); break;
    case 4: write_legs_smem<T, 4>(v, dst, Lp, lgnb, lgNs, T_); break;
    default: write_legs_smem<T, 2>(v, dst, Lp, lgnb, lgNs, T_); break;
  }
}
template <typename T>
__device__ __forceinline__ void do_write_global(int R, const typename Vec<T>::t (&v)[16], typename Vec<T>::t* out,
                                                int L, int lgnb, int T_, int units, bool conj, T sc) {
  switch (R) {
    case 16: write_legs_global<T, 16>(v, out, L, lgnb, T_, units, conj, sc); break;
    case 8: write_legs_global<T, 8>(v, out, L, lgnb, T_, units, conj, sc); break;
    case 4: write_legs_global<T, 4>(v, out, L, lgnb, T_, units, conj, sc); break;
    default: write_legs_global<T, 2>(v, out, L, lgnb, T_, units, conj, sc); break;
  }
}

}  // namespace fast

template <typename T>
__global__ void __launch_bounds__(512, 1) fast_kernel(const __grid_constant__ EngineArgs a) {
  using namespace fast;
  typedef typename Vec<T>::t V;
  extern __shared__ __align__(128) unsigned char smem[];
  const int S = a.stages;
  const int L = a.L;
  const int W = a.W;
  const int T_ = blockDim.x;
  const int tb_al = (a.tile_bytes + 127) & ~127;
  unsigned char* stage0 = smem;
  V* work = reinterpret_cast<V*>(smem + (size_t)S * tb_al);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + (size_t)S * tb_al + (((size_t)W * a.Lp * sizeof(V) + 7) & ~7));
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
    bulk_load(saddr(stage0 + (size_t)s * tb_al), in + u0 * L, bytes, bar);
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
        if (!a.debug_no_issue)  // drain the copies still in flight into this block
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
    const V* st = reinterpret_cast<const V*>(stage0 + (size_t)s * tb_al);

    // pass 0: the bulk-copied tile (unpadded) -> registers
    {
      const BlockPass& p = a.pass[0];
      const int lgnb = ilog2(L / p.R);
      do_read<T>(p.R, v, st, false, L, lgnb, T_);
      if (conj)
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] = cconj(v[i]);
      do_compute<T>(p.R, v, tw, p.tw, lgnb, 0, T_);
      __syncthreads();  // stage s fully read; previous tile's reads of `work` done
      if (threadIdx.x == 0 && !a.debug_no_issue) {
        const long long nt = tile + (long long)S * G;
        if (nt < a.ntiles) issue(nt, s);
      }
      if (a.npass == 1) {
        do_write_global<T>(p.R, v, out + u0 * L, L, lgnb, T_, units, conj, sc);
        continue;
      }
      do_write_smem<T>(p.R, v, work, a.Lp, lgnb, 0, T_);
      __syncthreads();
    }
    for (int pi = 1; pi < a.npass; ++pi) {
      const BlockPass& p = a.pass[pi];
      const int lgnb = ilog2(L / p.R);
      const int lgNs = ilog2(p.Ns);
      do_read<T>(p.R, v, work, true, a.Lp, lgnb, T_);
      do_compute<T>(p.R, v, tw, p.tw, lgnb, lgNs, T_);
      if (pi == a.npass - 1) {
        do_write_global<T>(p.R, v, out + u0 * L, L, lgnb, T_, units, conj, sc);
      } else {
        __syncthreads();
        do_write_smem<T>(p.R, v, work, a.Lp, lgnb, lgNs, T_);
        __syncthreads();
      }
    }
  }
}

}  // namespace gfft

extern "C" int gfft_fast_setup(int dbl, size_t max_smem) {
  cudaError_t e;
  if (dbl)
    e = cudaFuncSetAttribute(gfft::fast_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);
  else
    e = cudaFuncSetAttribute(gfft::fast_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);
  return e == cudaSuccess ? 0 : (int)e;
}

// blocks of `threads` threads and `smem` bytes that fit on one SM
extern "C" int gfft_fast_occupancy(int dbl, int threads, size_t smem) {
  int n = 0;
  if (dbl)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, gfft::fast_kernel<double>, threads, smem);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, gfft::fast_kernel<float>, threads, smem);
  return n;
}

extern "C" int gfft_fast_launch(int dbl, const EngineArgs* a, unsigned grid, unsigned threads, size_t smem,
                                cudaStream_t stream) {
  cudaGetLastError();  // clear a stale error of an earlier, unrelated call
  if (dbl) gfft::fast_kernel<double><<<grid, threads, smem, stream>>>(*a);
  else gfft::fast_kernel<float><<<grid, threads, smem, stream>>>(*a);
  return (int)cudaGetLastError();
}
