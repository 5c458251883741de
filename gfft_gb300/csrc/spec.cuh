// Compile-time Stockham passes shared by the length-specialised kernels
// (fft_spec.cu) and the tensor-core split-precision kernel (fft_tc.cu).
//
// A tile holds 4096 (FP32) or 2048 (FP64) complex values, or one transform
// of a longer L (tile_of): W = tile / L transforms (or column lanes) of a
// power-of-two length L, in a padded [lane][pad(s)] shared buffer.  Each of
// tile / 16 threads keeps 16 values in registers: 16 / R butterflies of
// radix R per pass.  Pass order for
// L = 2^a: radix 16 while four bits remain, then 8 / 4 / 2, matching the
// planner's default (planner.cpp block_radices).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "butterflies.cuh"
#include "plan.h"

namespace gfft {
namespace spec {

constexpr int lg2(int x) { return x <= 1 ? 0 : 1 + lg2(x / 2); }
constexpr int npass_of(int L) {
  return (lg2(L) % 4 == 0) ? lg2(L) / 4 : (lg2(L) % 4 == 1 ? (lg2(L) / 4 >= 1 ? lg2(L) / 4 + 1 : 1) : lg2(L) / 4 + 1);
}
constexpr int radix_of(int L, int p) {
  return (lg2(L) % 4 == 0)   ? 16
         : (lg2(L) % 4 == 1) ? (lg2(L) / 4 == 0 ? 2 : (p < lg2(L) / 4 - 1 ? 16 : (p == lg2(L) / 4 - 1 ? 8 : 4)))
         : (lg2(L) % 4 == 2) ? (p < lg2(L) / 4 ? 16 : 4)
                             : (p < lg2(L) / 4 ? 16 : 8);
}
constexpr int ns_of(int L, int p) { return p == 0 ? 1 : ns_of(L, p - 1) * radix_of(L, p - 1); }

template <typename T> struct Cfg;
template <> struct Cfg<float> {
  static constexpr int TILE = 4096;
  static constexpr int PS = 4;
};
template <> struct Cfg<double> {
  static constexpr int TILE = 2048;
  static constexpr int PS = 3;
};

// complex values per tile for length L: the type's tile, or one transform
template <typename T> constexpr int tile_of(int L) { return L > Cfg<T>::TILE ? L : Cfg<T>::TILE; }

template <typename T> __device__ __forceinline__ constexpr int padi(int s) { return s + (s >> Cfg<T>::PS); }

// pass P: read the legs of this thread's butterflies
template <typename T, int L, int P, bool FROM_STAGE>
__device__ __forceinline__ void sread(typename Vec<T>::t (&v)[16], const typename Vec<T>::t* src) {
  constexpr int R = radix_of(L, P), NB = L / R, Q = 16 / R, NT = tile_of<T>(L) / 16;
  constexpr int LP = L + (L >> Cfg<T>::PS) + 1;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int b = threadIdx.x + q * NT;
    const int lane = b / NB;
    const int j = b % NB;
    if (FROM_STAGE) {
      const typename Vec<T>::t* s = src + lane * L + j;
#pragma unroll
      for (int r = 0; r < R; ++r) v[q * R + r] = s[r * NB];
    } else {
      const typename Vec<T>::t* s = src + lane * LP;
#pragma unroll
      for (int r = 0; r < R; ++r) v[q * R + r] = s[padi<T>(j + r * NB)];
    }
  }
}

template <typename T, int L, int P>
__device__ __forceinline__ void scompute(typename Vec<T>::t (&v)[16], const typename Vec<T>::t* __restrict__ tw,
                                         int twoff) {
  typedef typename Vec<T>::t V;
  constexpr int R = radix_of(L, P), NB = L / R, Q = 16 / R, NS = ns_of(L, P), NT = tile_of<T>(L) / 16;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    if constexpr (NS > 1) {
      const int j = (threadIdx.x + q * NT) % NB;
      const V* t = tw + twoff + (j % NS);
#pragma unroll
      for (int r = 1; r < R; ++r) v[q * R + r] = cmul(v[q * R + r], __ldg(t + (r - 1) * NS));
    }
    dft<T, V, R>(&v[q * R]);
  }
}

template <typename T, int L, int P>
__device__ __forceinline__ void swrite(const typename Vec<T>::t (&v)[16], typename Vec<T>::t* work) {
  constexpr int R = radix_of(L, P), NB = L / R, Q = 16 / R, NS = ns_of(L, P), NT = tile_of<T>(L) / 16;
  constexpr int LP = L + (L >> Cfg<T>::PS) + 1;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int b = threadIdx.x + q * NT;
    const int lane = b / NB;
    const int j = b % NB;
    const int k = j % NS;
    const int base = (j - k) * R + k;
    typename Vec<T>::t* d = work + lane * LP;
#pragma unroll
    for (int r = 0; r < R; ++r) d[padi<T>(base + r * NS)] = v[q * R + r];
  }
}

template <typename T, int L, int P>
__device__ __forceinline__ void sstore(const typename Vec<T>::t (&v)[16], typename Vec<T>::t* out, int units,
                                       bool conj, T sc) {
  typedef typename Vec<T>::t V;
  constexpr int R = radix_of(L, P), NB = L / R, Q = 16 / R, NT = tile_of<T>(L) / 16;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int b = threadIdx.x + q * NT;
    const int lane = b / NB;
    const int j = b % NB;
    if (lane >= units) continue;
    V* d = out + lane * L + j;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      V x = v[q * R + r];
      if (conj) x = cconj(x);
      d[r * NB] = cscale(x, sc);
    }
  }
}

// middle passes 1 .. NP-2 (in place on `work`) and the last pass
template <typename T, int L, int P>
__device__ __forceinline__ void rest(typename Vec<T>::t (&v)[16], typename Vec<T>::t* work,
                                     const typename Vec<T>::t* tw, const BlockPass* passes, typename Vec<T>::t* out,
                                     int units, bool conj, T sc) {
  constexpr int NP = npass_of(L);
  if constexpr (P < NP) {
    sread<T, L, P, false>(v, work);
    scompute<T, L, P>(v, tw, passes[P].tw);
    if constexpr (P == NP - 1) {
      sstore<T, L, P>(v, out, units, conj, sc);
    } else {
      __syncthreads();
      swrite<T, L, P>(v, work);
      __syncthreads();
      rest<T, L, P + 1>(v, work, tw, passes, out, units, conj, sc);
    }
  }
}

}  // namespace spec

namespace lanep2 {

__device__ __forceinline__ uint32_t sa(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
template <typename T> __device__ __forceinline__ void cpa(uint32_t dst, const void* src);
template <> __device__ __forceinline__ void cpa<float>(uint32_t dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst), "l"(src) : "memory");
}
template <> __device__ __forceinline__ void cpa<double>(uint32_t dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}

template <typename T, int L>
__device__ __forceinline__ void gather(const EngineArgs& a, typename Vec<T>::t* buf, long long tile) {
  typedef typename Vec<T>::t V;
  constexpr int W = spec::Cfg<T>::TILE / L, NT = spec::Cfg<T>::TILE / 16, LP = L + (L >> spec::Cfg<T>::PS) + 1;
  const int lane = threadIdx.x % W;
  const long long u = tile * W + lane;
  if (u >= a.nunits) return;
  const long long t = u / a.stride;
  const long long b = u - t * a.stride;
  const V* src = (const V*)a.in + t * a.N + b;
  V* bl = buf + lane * LP;
  for (int s = threadIdx.x / W; s < L; s += NT / W)
    cpa<T>(sa(bl + spec::padi<T>(s)), src + (long long)s * a.stride);
}

template <typename T, int L>
__device__ __forceinline__ void sweep(const EngineArgs& a, typename Vec<T>::t* buf, long long tile) {
  typedef typename Vec<T>::t V;
  constexpr int W = spec::Cfg<T>::TILE / L, NT = spec::Cfg<T>::TILE / 16, LP = L + (L >> spec::Cfg<T>::PS) + 1;
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
    V x = bl[spec::padi<T>(s)];
    if (a.conj) x = cconj(x);
    if (kstep) {
      const unsigned m = kstep * (unsigned)s;  // < N < 2^32
      x = cmul(x, cmul(__ldg(lo + (m & mask)), __ldg(hi + (m >> lgB))));
    }
    bl[spec::padi<T>(s)] = x;
  }
}

}  // namespace lanep2

}  // namespace gfft
