// Device code of the Stockham engine (shared by the engine kernel in
// fft_engine.cu and the ragged persistent kernel in fft_ragged.cu).
#pragma once
#include <cuda_runtime.h>

#include "butterflies.cuh"
#include "dcheck.cuh"
#include "plan.h"

namespace gfft {

template <typename T> struct PadShift;
template <> struct PadShift<float> { static constexpr int v = 4; };   // 8-byte elements
template <> struct PadShift<double> { static constexpr int v = 3; };  // 16-byte elements

// padded index: one slot per 2^PS values, and one more per 2^(PS+4) so that
// strides of 2^(PS+4) values (a multiple of the 128-byte bank window after
// the first term) fall on different banks; engine_padded (plan.h) is the
// matching per-unit stride
template <typename T> __device__ __forceinline__ int pad(int s) {
  return s + (s >> PadShift<T>::v) + (s >> (PadShift<T>::v + 4));
}

// one in-block Stockham pass of compile-time radix R over all W units
template <typename T, int R>
__device__ __forceinline__ void block_pass(const typename Vec<T>::t* __restrict__ src,
                                           typename Vec<T>::t* __restrict__ dst, const EngineArgs& a,
                                           const BlockPass& p, const typename Vec<T>::t* __restrict__ tw) {
  typedef typename Vec<T>::t V;
  constexpr int PS = PadShift<T>::v;
  const int L = a.L;
  const int nb = L / R;
  const int total = a.W * nb;
  // when nb (resp. Ns) is a multiple of the longer padding period 2^(PS+4),
  // pad(x + r nb) = pad(x) + r pad'(nb) with pad'(nb) = nb + nb / 2^PS +
  // nb / 2^(PS+4): the legs sit at a constant padded stride
  const bool rd_lin = (nb & ((1 << (PS + 4)) - 1)) == 0;
  const bool wr_lin = (p.Ns & ((1 << (PS + 4)) - 1)) == 0;
  const int rd_st = nb + (nb >> PS) + (nb >> (PS + 4));
  const int wr_st = (int)p.Ns + ((int)p.Ns >> PS) + ((int)p.Ns >> (PS + 4));
  // the first pass (Ns = 1) writes each butterfly's R outputs R apart: with
  // lanes of a power-of-two count, consecutive threads take consecutive
  // lanes instead (the odd lane stride Lp spreads them over the banks)
  const bool lf = p.Ns == 1 && a.W >= 4 && (a.W & (a.W - 1)) == 0;
  const int lgw = __ffs(a.W) - 1;
  for (int i = threadIdx.x; i < total; i += blockDim.x) {
    const int lane = lf ? (i & (a.W - 1)) : (int)fdiv((unsigned)i, p.fd_nb);
    const int j = lf ? (i >> lgw) : i - lane * nb;
    const V* s = src + lane * a.Lp;
    V* d = dst + lane * a.Lp;
    V v[R];
    if (!GFFT_DCHECK(lane < a.W && pad<T>(j + (R - 1) * nb) < a.Lp, a.status)) continue;
    if (rd_lin) {
      const V* s0 = s + pad<T>(j);
#pragma unroll
      for (int r = 0; r < R; ++r) v[r] = s0[r * rd_st];
    } else {
#pragma unroll
      for (int r = 0; r < R; ++r) v[r] = s[pad<T>(j + r * nb)];
    }
    const int k = j - (int)fdiv((unsigned)j, p.fd_ns) * p.Ns;
    if (p.Ns > 1) {
      const V* t = tw + p.tw + k;
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = cmul(v[r], __ldg(t + (r - 1) * p.Ns));
    }
    dft<T, V, R>(v);
    const int base = (j - k) * R + k;
    if (!GFFT_DCHECK(pad<T>(base + (R - 1) * (int)p.Ns) < a.Lp, a.status)) continue;
    if (wr_lin) {
      V* d0 = d + pad<T>(base);
#pragma unroll
      for (int r = 0; r < R; ++r) d0[r * wr_st] = v[r];
    } else {
#pragma unroll
      for (int r = 0; r < R; ++r) d[pad<T>(base + r * p.Ns)] = v[r];
    }
  }
}

// The same pass transposed (decimation in frequency): gather the R legs
// from the positions the decimation-in-time pass writes, butterfly, then
// twiddle output r by W_(Ns R)^(k r) and scatter to the positions the
// decimation-in-time pass reads.  The DFT matrix is symmetric, so running
// the transposed passes in reverse order computes the same transform: the
// autosort (Stockham) form of the reference's frequency-decimation
// recursion InFreq / T_DFTk_x_Im (src/gfftalgfreq.h:106-432).
template <typename T, int R>
__device__ __forceinline__ void block_pass_dif(const typename Vec<T>::t* __restrict__ src,
                                               typename Vec<T>::t* __restrict__ dst, const EngineArgs& a,
                                               const BlockPass& p, const typename Vec<T>::t* __restrict__ tw) {
  typedef typename Vec<T>::t V;
  const int L = a.L;
  const int nb = L / R;
  const int total = a.W * nb;
  for (int i = threadIdx.x; i < total; i += blockDim.x) {
    const int lane = (int)fdiv((unsigned)i, p.fd_nb);
    const int j = i - lane * nb;
    const int k = j - (int)fdiv((unsigned)j, p.fd_ns) * p.Ns;
    const int base = (j - k) * R + k;
    if (!GFFT_DCHECK(lane < a.W && pad<T>(base + (R - 1) * (int)p.Ns) < a.Lp && pad<T>(j + (R - 1) * nb) < a.Lp,
                     a.status))
      continue;
    const V* s = src + lane * a.Lp;
    V* d = dst + lane * a.Lp;
    V v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = s[pad<T>(base + r * p.Ns)];
    dft<T, V, R>(v);
    if (p.Ns > 1) {
      const V* t = tw + p.tw + k;
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = cmul(v[r], __ldg(t + (r - 1) * p.Ns));
    }
#pragma unroll
    for (int r = 0; r < R; ++r) d[pad<T>(j + r * nb)] = v[r];
  }
}

// generic odd prime radix: every output sums R twiddled inputs (O(R^2))
template <typename T>
__device__ void block_pass_generic(const typename Vec<T>::t* __restrict__ src, typename Vec<T>::t* __restrict__ dst,
                                   const EngineArgs& a, const BlockPass& p, const typename Vec<T>::t* __restrict__ tw) {
  typedef typename Vec<T>::t V;
  const int L = a.L, R = p.R;
  const int nb = L / R;
  const int total = a.W * L;  // one output per iteration
  const V* wr = tw + p.gen;
  for (int i = threadIdx.x; i < total; i += blockDim.x) {
    const int lane = i / L;
    const int rem = i - lane * L;
    const int q = rem / nb;  // output leg
    const int j = rem - q * nb;
    const V* s = src + lane * a.Lp;
    V* d = dst + lane * a.Lp;
    const int k = j % p.Ns;
    V acc = mk<V>(0, 0);
    int m = 0;  // (r*q) mod R
    for (int r = 0; r < R; ++r) {
      V x = s[pad<T>(j + r * nb)];
      if (p.Ns > 1 && r > 0) x = cmul(x, __ldg(tw + p.tw + (r - 1) * p.Ns + k));
      acc = cadd(acc, cmul(x, __ldg(wr + m)));
      m += q;
      if (m >= R) m -= R;
    }
    d[pad<T>((j - k) * R + k + q * p.Ns)] = acc;
  }
}

// the generic prime pass transposed: output q = W_(Ns R)^(k q) * sum_r
// x[(j - k) R + k + r Ns] W_R^(r q), written to j + q nb
template <typename T>
__device__ void block_pass_generic_dif(const typename Vec<T>::t* __restrict__ src,
                                       typename Vec<T>::t* __restrict__ dst, const EngineArgs& a, const BlockPass& p,
                                       const typename Vec<T>::t* __restrict__ tw) {
  typedef typename Vec<T>::t V;
  const int L = a.L, R = p.R;
  const int nb = L / R;
  const int total = a.W * L;  // one output per iteration
  const V* wr = tw + p.gen;
  for (int i = threadIdx.x; i < total; i += blockDim.x) {
    const int lane = i / L;
    const int rem = i - lane * L;
    const int q = rem / nb;  // output leg
    const int j = rem - q * nb;
    const V* s = src + lane * a.Lp;
    V* d = dst + lane * a.Lp;
    const int k = j % p.Ns;
    const int base = (j - k) * R + k;
    V acc = mk<V>(0, 0);
    int m = 0;  // (r*q) mod R
    for (int r = 0; r < R; ++r) {
      acc = cadd(acc, cmul(s[pad<T>(base + r * p.Ns)], __ldg(wr + m)));
      m += q;
      if (m >= R) m -= R;
    }
    if (p.Ns > 1 && q > 0) acc = cmul(acc, __ldg(tw + p.tw + (q - 1) * p.Ns + k));
    d[pad<T>(j + q * nb)] = acc;
  }
}

// W_N^m = lo[m mod B] * hi[m / B], B a power of two
template <typename T>
__device__ __forceinline__ typename Vec<T>::t global_twiddle(const EngineArgs& a, long long m, int lgB) {
  typedef typename Vec<T>::t V;
  const V* lo = (const V*)a.gtw_lo;
  const V* hi = (const V*)a.gtw_hi;
  return cmul(__ldg(lo + (m & (a.gB - 1))), __ldg(hi + (m >> lgB)));
}

// global -> shared, with the conjugation of the inverse, the inter-pass
// twiddle of a multi-pass transform, or the real inverse pre-pass
template <typename T>
__device__ __forceinline__ void load_tile(const EngineArgs& a, typename Vec<T>::t* buf, long long u0) {
  typedef typename Vec<T>::t V;
  const V* in = (const V*)a.in;
  const int L = a.L;
  const int total = a.W * L;
  if (a.mode == 0 && a.real == 2) {
    // real inverse pre pass (the inverse of the reference's Separate with
    // S=-1, src/gfftswap.h:246-280): X packed -> Z = F + iG
    const V* rtw = (const V*)a.rtw;
    const int half = L / 2 + 1;
    for (int i = threadIdx.x; i < a.W * half; i += blockDim.x) {
      const int lane = (int)fdiv((unsigned)i, a.fd_half);
      const int q = i - lane * half;
      const long long u = u0 + lane;
      V* b = buf + lane * a.Lp;
      if (u >= a.nunits) continue;
      const V* x = in + u * L;
      if (q == 0) {
        const V x0 = x[0];  // (X_0, X_n)
        V z = mk<V>((T)0.5 * (x0.x + x0.y), (T)0.5 * (x0.x - x0.y));
        b[pad<T>(0)] = cconj(z);
        continue;
      }
      const int qm = L - q;
      if (q > qm) continue;
      const V xq = x[q], xm = x[qm];
      // Z_q = F + i G,  F = (X_q + conj X_m)/2,  G = (X_q - conj X_m) conj(w^q) / 2
      const V wq = __ldg(rtw + q);
      V F = mk<V>((T)0.5 * (xq.x + xm.x), (T)0.5 * (xq.y - xm.y));
      V D = mk<V>((T)0.5 * (xq.x - xm.x), (T)0.5 * (xq.y + xm.y));
      V G = cmul(D, cconj(wq));
      V zq = mk<V>(F.x - G.y, F.y + G.x);
      b[pad<T>(q)] = cconj(zq);
      if (qm != q) {
        const V wm = __ldg(rtw + qm);
        V F2 = mk<V>((T)0.5 * (xm.x + xq.x), (T)0.5 * (xm.y - xq.y));
        V D2 = mk<V>((T)0.5 * (xm.x - xq.x), (T)0.5 * (xm.y + xq.y));
        V G2 = cmul(D2, cconj(wm));
        V zm = mk<V>(F2.x - G2.y, F2.y + G2.x);
        b[pad<T>(qm)] = cconj(zm);
      }
    }
    return;
  }
  if (a.mode == 2) {
    // gathered lanes: lane l is a whole transform at in + lane_off[l]
    const int step = blockDim.x;
    const int lanes = (int)(a.nunits - u0);
    for (int i0 = threadIdx.x; i0 < total; i0 += 8 * step) {
      V v[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int i = i0 + q * step;
        const int lane = (int)fdiv((unsigned)i, a.fd_L);
        v[q] = (i < total && lane < lanes) ? in[a.lane_off[lane] + (i - lane * L)] : mk<V>(0, 0);
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int i = i0 + q * step;
        if (i >= total) break;
        const int lane = (int)fdiv((unsigned)i, a.fd_L);
        buf[lane * a.Lp + pad<T>(i - lane * L)] = a.conj ? cconj(v[q]) : v[q];
      }
    }
    return;
  }
  if (a.mode == 0) {
    const V* tile = in + u0 * L;
    const long long lim = (a.nunits - u0) * L;
    // eight loads in flight per thread before their shared-memory stores
    const int step = blockDim.x;
    for (int i0 = threadIdx.x; i0 < total; i0 += 8 * step) {
      V v[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int i = i0 + q * step;
        v[q] = (i < total && i < lim && GFFT_DCHECK(u0 * L + i < a.nunits * L, a.status)) ? tile[i] : mk<V>(0, 0);
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int i = i0 + q * step;
        if (i >= total) break;
        const int lane = (int)fdiv((unsigned)i, a.fd_L);
        const int s = i - lane * L;
        buf[lane * a.Lp + pad<T>(s)] = a.conj ? cconj(v[q]) : v[q];
      }
    }
  } else if (a.dif) {
    // lane units of a frequency-decimation pass: gather from the positions
    // the time-decimation pass writes (t N + (b - k) L + k + s Ns); the
    // twiddle comes after the butterflies (store_tile)
    const int W = a.W;
    const int lane = threadIdx.x % W;
    const int sstep = blockDim.x / W;
    const long long u = u0 + lane;
    V* bl = buf + lane * a.Lp;
    if (u >= a.nunits) {
      for (int s = threadIdx.x / W; s < L; s += sstep) bl[pad<T>(s)] = mk<V>(0, 0);
      return;
    }
    const long long t = u / a.stride;
    const long long b = u - t * a.stride;
    const long long k = b % a.gNs;
    const V* src = in + t * a.N + (b - k) * L + k;
    for (int s0 = threadIdx.x / W; s0 < L; s0 += 8 * sstep) {
      V v[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int s = s0 + q * sstep;
        if (s < L) v[q] = src[(long long)s * a.gNs];
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int s = s0 + q * sstep;
        if (s >= L) break;
        bl[pad<T>(s)] = a.conj ? cconj(v[q]) : v[q];
      }
    }
  } else {
    // lane units: the block's threads are a whole number of W-groups, so
    // each thread keeps one lane and walks its samples
    const int W = a.W;
    const int lane = threadIdx.x % W;
    const int sstep = blockDim.x / W;
    const long long u = u0 + lane;
    V* bl = buf + lane * a.Lp;
    if (u >= a.nunits) {
      for (int s = threadIdx.x / W; s < L; s += sstep) bl[pad<T>(s)] = mk<V>(0, 0);
      return;
    }
    const long long t = u / a.stride;
    const long long b = u - t * a.stride;
    const long long k = b % a.gNs;
    const long long kstep = a.notw ? 0 : k * (a.N / (a.gNs * L));  // twiddle exponent per sample
    const int lgB = 63 - __clzll(a.gB);
    const V* src = in + t * a.N + b;
    for (int s0 = threadIdx.x / W; s0 < L; s0 += 8 * sstep) {
      V v[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int s = s0 + q * sstep;
        if (s < L && GFFT_DCHECK(t * a.N + b + (long long)s * a.stride < a.nunits * L, a.status))
          v[q] = a.ldcg ? __ldcg(src + (long long)s * a.stride) : src[(long long)s * a.stride];
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int s = s0 + q * sstep;
        if (s >= L) break;
        V x = a.conj ? cconj(v[q]) : v[q];
        if (kstep) x = cmul(x, global_twiddle<T>(a, kstep * s, lgB));
        bl[pad<T>(s)] = x;
      }
    }
  }
}

template <typename T>
__device__ __forceinline__ void store_tile(const EngineArgs& a, const typename Vec<T>::t* buf, long long u0) {
  typedef typename Vec<T>::t V;
  V* out = (V*)a.out;
  const int L = a.L;
  const int total = a.W * L;
  const T sc = (T)a.scale;
  if (a.mode == 0 && a.real == 1) {
    // real forward post pass (the reference's Separate with S=+1,
    // src/gfftswap.h:246-280): Z -> X_0, X_n, X_1..X_{n-1}
    const V* rtw = (const V*)a.rtw;
    const int half = L / 2 + 1;
    for (int i = threadIdx.x; i < a.W * half; i += blockDim.x) {
      const int lane = (int)fdiv((unsigned)i, a.fd_half);
      const int q = i - lane * half;
      const long long u = u0 + lane;
      if (u >= a.nunits) continue;
      const V* b = buf + lane * a.Lp;
      V* y = out + u * L;
      if (q == 0) {
        const V z0 = b[pad<T>(0)];
        y[0] = mk<V>(z0.x + z0.y, z0.x - z0.y);
        continue;
      }
      const int qm = L - q;
      if (q > qm) continue;
      const V zq = b[pad<T>(q)], zm = b[pad<T>(qm)];
      {
        // X_q = F + w^q G, F = (Z_q + conj Z_m)/2, G = -i (Z_q - conj Z_m)/2
        V F = mk<V>((T)0.5 * (zq.x + zm.x), (T)0.5 * (zq.y - zm.y));
        V G = mk<V>((T)0.5 * (zq.y + zm.y), (T)-0.5 * (zq.x - zm.x));
        y[q] = cadd(F, cmul(__ldg(rtw + q), G));
      }
      if (qm != q) {
        V F = mk<V>((T)0.5 * (zm.x + zq.x), (T)0.5 * (zm.y - zq.y));
        V G = mk<V>((T)0.5 * (zm.y + zq.y), (T)-0.5 * (zm.x - zq.x));
        y[qm] = cadd(F, cmul(__ldg(rtw + qm), G));
      }
    }
    return;
  }
  if (a.mode == 2) {
    const int lanes = (int)(a.nunits - u0);
    for (int i = threadIdx.x; i < total; i += blockDim.x) {
      const int lane = (int)fdiv((unsigned)i, a.fd_L);
      if (lane >= lanes) break;
      const int s = i - lane * L;
      V v = buf[lane * a.Lp + pad<T>(s)];
      if (a.conj) v = cconj(v);
      out[a.lane_off[lane] + s] = cscale(v, sc);
    }
    return;
  }
  if (a.mode == 0) {
    V* tile = out + u0 * L;
    const long long lim = (a.nunits - u0) * L;
    for (int i = threadIdx.x; i < total; i += blockDim.x) {
      if (i >= lim) break;
      const int lane = (int)fdiv((unsigned)i, a.fd_L);
      const int s = i - lane * L;
      V v = buf[lane * a.Lp + pad<T>(s)];
      if (a.conj) v = cconj(v);
      if (GFFT_DCHECK(u0 * L + i < a.nunits * L, a.status)) tile[i] = cscale(v, sc);
    }
  } else if (a.dif) {
    // lane units of a frequency-decimation pass: the four-step twiddle of
    // sample s, then scatter to the positions the time-decimation pass
    // reads (t N + b + s N/L)
    const int W = a.W;
    const int lane = threadIdx.x % W;
    const int sstep = blockDim.x / W;
    const long long u = u0 + lane;
    if (u >= a.nunits) return;
    const long long t = u / a.stride;
    const long long b = u - t * a.stride;
    const long long k = b % a.gNs;
    const long long kstep = a.notw ? 0 : k * (a.N / (a.gNs * L));
    const int lgB = 63 - __clzll(a.gB);
    V* dstp = out + t * a.N + b;
    const V* bl = buf + lane * a.Lp;
    for (int s = threadIdx.x / W; s < L; s += sstep) {
      V v = bl[pad<T>(s)];
      if (kstep) v = cmul(v, global_twiddle<T>(a, kstep * s, lgB));
      if (a.conj) v = cconj(v);
      dstp[(long long)s * a.stride] = cscale(v, sc);
    }
  } else if (a.gNs == 1) {
    // first global pass: lane b's outputs are the L contiguous elements at
    // t*N + b*L, and adjacent lanes are adjacent rows, so the tile's output
    // is one contiguous run per transform: write it sample-fastest
    const int W = a.W;
    for (int i = threadIdx.x; i < W * L; i += blockDim.x) {
      const int lane = (int)fdiv((unsigned)i, a.fd_L);
      const int s = i - lane * L;
      const long long u = u0 + lane;
      if (u >= a.nunits) break;
      const long long t = u / a.stride;
      const long long b = u - t * a.stride;
      V v = buf[lane * a.Lp + pad<T>(s)];
      if (a.conj) v = cconj(v);
      out[t * a.N + b * L + s] = cscale(v, sc);
    }
  } else {
    const int W = a.W;
    const int lane = threadIdx.x % W;
    const int sstep = blockDim.x / W;
    const long long u = u0 + lane;
    if (u >= a.nunits) return;
    const long long t = u / a.stride;
    const long long b = u - t * a.stride;
    const long long k = b % a.gNs;
    V* dstp = out + t * a.N + (b - k) * L + k;
    const V* bl = buf + lane * a.Lp;
    for (int s = threadIdx.x / W; s < L; s += sstep) {
      V v = bl[pad<T>(s)];
      if (a.conj) v = cconj(v);
      if (GFFT_DCHECK(t * a.N + (b - k) * L + k + (long long)s * a.gNs < a.nunits * L, a.status))
        dstp[(long long)s * a.gNs] = cscale(v, sc);
    }
  }
}

}  // namespace gfft
