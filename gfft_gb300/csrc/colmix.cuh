// Mixed-radix column tiles moved by the tensor memory accelerator (variant 9
// for a pass length L that is not a power of two: the shapes of
// mixed_shapes.h, radices R0..R3 fixed at compile time).
//
// The data movement of col.cuh (the input of any global pass is a
// (batch L) x (N/L) matrix; a tile of W adjacent units is one W x L box,
// brought into a dense [L][W] stage by 2-D tensor copies on an mbarrier with
// bounded waits; a later pass's output is a W x L box of the matrix with rows
// of Ns elements, sent by 2-D tensor stores), with in-block passes whose
// radices need not divide 16:
//  - first pass (radix R0) from the dense stage, lane-fastest (a warp reads
//    consecutive words of a stage row), with the conjugation of the inverse
//    and the four-step twiddle W_N^(k s N/(Ns L)) applied on load (factored
//    as in col.cuh, with a [R0][Ns] table of W_(R0 Ns)^(k r)), written
//    to a padded [lane][Lp] work buffer; the stage is then free for the copy
//    of the tile S tiles ahead;
//  - the middle passes ping-pong between two padded work buffers, one
//    butterfly per thread at a time, twiddles from a shared-memory copy of
//    the pass's in-block table (L - 1 values, copied once per block);
//  - last pass: the first global pass stores straight to global memory
//    (each lane's L outputs are contiguous: consecutive threads write
//    consecutive addresses); a later pass writes a dense [L][W] tile into
//    the other work buffer and sends it by tensor stores, which the next
//    tile's first write waits for (cp.async.bulk.wait_group.read).
// Requirements (planner): W divides N / L and Ns (so a tile lies in one
// transform and maps to one output box), row pitches of a multiple of 16
// bytes, 16-byte aligned buffers, tensor boxes starting on 128-byte
// boundaries of the stage.  colmix_gather_kernel (below) has the same passes
// with per-element cp.async gathers for the passes that miss these.
//
// Replaces, for mixed radices, the same recursion levels as col.cuh:
// InTimeOOP (src/gfftalg.h:459-507) with DFTk_x_Im_T (src/gfftalg.h:169-267).
#pragma once
#include "col.cuh"

namespace gfft {
namespace colmix {

template <typename T> __device__ __forceinline__ constexpr int padi(int s) {
  return colshape::mix_pad(col::esz<T>(), s);
}

template <typename T, int R0, int R1, int R2, int R3> struct MixShape {
  static constexpr int ESZ = col::esz<T>();
  static constexpr int L = R0 * R1 * R2 * R3;
  static constexpr int NP = 1 + (R1 > 1) + (R2 > 1) + (R3 > 1);
  static constexpr int W = colshape::mix_lanes(ESZ, L);
  static constexpr int NT = colshape::mix_threads();
  static constexpr int LP = colshape::mix_stride(ESZ, L);
  static constexpr int BR = colshape::mix_rows(L);
  static constexpr int NBOX = L / BR;
  static constexpr int TB = colshape::mix_stage_bytes(ESZ, L);
  static constexpr int WB = colshape::mix_work_bytes(ESZ, L);
  static constexpr int XS = ESZ / 8;  // tensor-map elements (8 bytes) per complex element
};

// a middle pass of radix R (stride NS) over the W lanes: src -> dst (padded
// buffers), lane-major (consecutive threads walk one lane's butterflies)
template <typename T, int L, int W, int NT, int LP, int R, int NS>
__device__ __forceinline__ void mid(const typename Vec<T>::t* __restrict__ src, typename Vec<T>::t* __restrict__ dst,
                                    const typename Vec<T>::t* __restrict__ tw, int twoff, int* st) {
  typedef typename Vec<T>::t V;
  constexpr int NB = L / R, TOT = W * NB;
  (void)st;
  for (int i = threadIdx.x; i < TOT; i += NT) {
    const int lane = i / NB, j = i - lane * NB, k = j % NS;
    const V* s = src + lane * LP;
    V v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = s[padi<T>(j + r * NB)];
    if constexpr (NS > 1) {
      const V* t = tw + twoff + k;
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = cmul(v[r], t[(r - 1) * NS]);
    }
    dft<T, V, R>(v);
    V* d = dst + lane * LP;
    const int base = (j - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int e = lane * LP + padi<T>(base + r * NS);
      if (GFFT_DCHECK(e < W * LP, st)) d[padi<T>(base + r * NS)] = v[r];
    }
  }
}

}  // namespace colmix

template <typename T, int R0, int R1, int R2, int R3>
__global__ void __launch_bounds__(colshape::mix_threads(), 1)
    colmix_kernel(const __grid_constant__ EngineArgs a, const __grid_constant__ col::ColMaps maps) {
  using namespace colmix;
  typedef MixShape<T, R0, R1, R2, R3> Sh;
  typedef typename Vec<T>::t V;
  constexpr int L = Sh::L, W = Sh::W, NT = Sh::NT, LP = Sh::LP, NP = Sh::NP, TB = Sh::TB, BR = Sh::BR;
  constexpr int NBOX = Sh::NBOX, XS = Sh::XS, ESZ = Sh::ESZ;
  // the last pass's radix and stride
  constexpr int RL = NP == 4 ? R3 : (NP == 3 ? R2 : (NP == 2 ? R1 : R0));
  constexpr int NSL = L / RL;
  static_assert(NP >= 2, "a mixed shape has two or more in-block passes");
  extern __shared__ __align__(1024) unsigned char smem[];
  const int S = a.stages;
  V* const w0 = reinterpret_cast<V*>(smem + (size_t)S * TB);
  V* const w1 = reinterpret_cast<V*>(smem + (size_t)S * TB + Sh::WB);
  V* const stw = reinterpret_cast<V*>(smem + (size_t)S * TB + 2 * (size_t)Sh::WB);
  uint64_t* const bars =
      reinterpret_cast<uint64_t*>(smem + (size_t)S * TB + 2 * (size_t)Sh::WB + colshape::mix_tw_bytes(ESZ, L));
  const int tw0 = a.pass[0].tw;
  for (int e = threadIdx.x; e < L - 1; e += NT) stw[e] = __ldg((const V*)a.tw + tw0 + e);
  const T sc = (T)a.scale;
  const bool conj = a.conj != 0;
  const long long G = gridDim.x;
  const long long stride = a.stride;  // N / L: units per transform
  const long long tpt = stride / W;   // tiles per transform
  const long long gNs = a.gNs;
  const unsigned kfac = (unsigned)(a.N / (gNs * L));
  const V* lo = (const V*)a.gtw_lo;
  const V* hi = (const V*)a.gtw_hi;
  const unsigned mask = (unsigned)a.gB - 1;
  const int lgB = 31 - __clz((int)a.gB);

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) fast::mbar_init(fast::saddr(&bars[s]), 1);
    fast::mbar_fence_init();
  }
  __syncthreads();

  auto issue = [&](long long tile, int s) {
    const long long t = tile / tpt, p = tile - t * tpt;
    const uint32_t bar = fast::saddr(&bars[s]);
    unsigned char* st = smem + (size_t)s * TB;
    fast::mbar_expect_tx(bar, (uint32_t)(W * L * ESZ));
#pragma unroll 1
    for (int k = 0; k < NBOX; ++k)
      col::tma_load_2d(fast::saddr(st + (size_t)k * BR * W * ESZ), &maps.in[0], (int)(p * W * XS),
                       (int)(t * L + k * BR), bar);
  };
  if (threadIdx.x == 0 && !a.debug_no_issue)
    for (int s = 0; s < S; ++s) {
      const long long tile = blockIdx.x + (long long)s * G;
      if (tile < a.ntiles) issue(tile, s);
    }

  int it = 0;
  for (long long tile = blockIdx.x; tile < a.ntiles; tile += G, ++it) {
    const int s = it % S;
    const uint32_t ph = (uint32_t)((it / S) & 1);
    const bool ok = fast::mbar_wait_bounded(fast::saddr(&bars[s]), ph, a.spin_limit);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        atomicExch(a.status, 13 /* GFFT_E_TIMEOUT */);
        if (!a.debug_no_issue)
          for (int k = 1; k < S; ++k) {
            const long long t2 = tile + (long long)k * G;
            if (t2 >= a.ntiles) break;
            const int j = it + k;
            fast::mbar_wait_bounded(fast::saddr(&bars[j % S]), (uint32_t)((j / S) & 1), a.spin_limit);
          }
        asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
      }
      return;
    }
    const long long t = tile / tpt, p = tile - t * tpt;
    const V* const stg = reinterpret_cast<const V*>(smem + (size_t)s * TB);
    // the previous tile's tensor store has read its work buffer
    if (threadIdx.x == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
    __syncthreads();

    // first pass (radix R0, stride 1) from the dense stage, lane-fastest
    {
      constexpr int NB0 = L / R0;
      for (int i = threadIdx.x; i < W * NB0; i += NT) {
        const int lane = i % W, j = i / W;
        V v[R0];
#pragma unroll
        for (int r = 0; r < R0; ++r) {
          const int e = (j + r * NB0) * W + lane;
          if (GFFT_DCHECK(e < W * L, a.status)) v[r] = stg[e];
        }
        if (conj)
#pragma unroll
          for (int r = 0; r < R0; ++r) v[r] = cconj(v[r]);
        if (!a.notw) {
          const unsigned k = (unsigned)((p * W + lane) % gNs);
          const unsigned kstep = k * kfac;
          if (kstep && a.ftw) {
            // W_N^(kstep (j + r NB0)) = W_N^(kstep j) * W_(R0 Ns)^(k r): one
            // lookup of the first factor, the second from the [r][k] table
            const unsigned m0 = kstep * (unsigned)j;  // < N < 2^32
            const V t0 = cmul(__ldg(lo + (m0 & mask)), __ldg(hi + (m0 >> lgB)));
            const V* t2 = (const V*)a.ftw + k;
#pragma unroll
            for (int r = 0; r < R0; ++r) v[r] = cmul(v[r], cmul(t0, __ldg(t2 + (size_t)r * gNs)));
          } else if (kstep) {
#pragma unroll
            for (int r = 0; r < R0; ++r) {
              const unsigned m = kstep * (unsigned)(j + r * NB0);  // < N < 2^32
              v[r] = cmul(v[r], cmul(__ldg(lo + (m & mask)), __ldg(hi + (m >> lgB))));
            }
          }
        }
        dft<T, V, R0>(v);
        V* d = w0 + lane * LP;
#pragma unroll
        for (int r = 0; r < R0; ++r) d[padi<T>(j * R0 + r)] = v[r];
      }
    }
    __syncthreads();  // every thread has read stage s
    if (threadIdx.x == 0 && !a.debug_no_issue) {
      const long long nt = tile + (long long)S * G;
      if (nt < a.ntiles) issue(nt, s);
    }
    // middle passes: w0 -> w1 -> w0 ...; `src` holds the last pass's input
    const V* src = w0;
    V* oth = w1;
    if constexpr (NP >= 3) {
      mid<T, L, W, NT, LP, R1, R0>(w0, w1, stw, a.pass[1].tw - tw0, a.status);
      __syncthreads();
      src = w1;
      oth = w0;
    }
    if constexpr (NP >= 4) {
      mid<T, L, W, NT, LP, R2, R0 * R1>(w1, w0, stw, a.pass[2].tw - tw0, a.status);
      __syncthreads();
      src = w0;
      oth = w1;
    }
    const int twl = a.pass[NP - 1].tw - tw0;
    constexpr int NBL = L / RL;
    if (gNs == 1) {
      // first global pass: lane-major, straight to global memory
      for (int i = threadIdx.x; i < W * NBL; i += NT) {
        const int lane = i / NBL, j = i - lane * NBL;
        const V* sp = src + lane * LP;
        V v[RL];
#pragma unroll
        for (int r = 0; r < RL; ++r) v[r] = sp[padi<T>(j + r * NBL)];
#pragma unroll
        for (int r = 1; r < RL; ++r) v[r] = cmul(v[r], stw[twl + j + (r - 1) * NSL]);
        dft<T, V, RL>(v);
        const long long e0 = t * a.N + (p * W + lane) * L + j;
        V* d = (V*)a.out + e0;
#pragma unroll
        for (int r = 0; r < RL; ++r) {
          V x = v[r];
          if (conj) x = cconj(x);
          if (GFFT_DCHECK(e0 + r * NSL < a.nunits * L, a.status)) d[r * NSL] = cscale(x, sc);
        }
      }
    } else {
      // later global passes: lane-fastest, a dense [L][W] tile in `oth`, tensor stores
      for (int i = threadIdx.x; i < W * NBL; i += NT) {
        const int lane = i % W, j = i / W;
        const V* sp = src + lane * LP;
        V v[RL];
#pragma unroll
        for (int r = 0; r < RL; ++r) v[r] = sp[padi<T>(j + r * NBL)];
#pragma unroll
        for (int r = 1; r < RL; ++r) v[r] = cmul(v[r], stw[twl + j + (r - 1) * NSL]);
        dft<T, V, RL>(v);
#pragma unroll
        for (int r = 0; r < RL; ++r) {
          V x = v[r];
          if (conj) x = cconj(x);
          oth[(j + r * NSL) * W + lane] = cscale(x, sc);
        }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      if (threadIdx.x == 0) {
        const long long row0 = t * (a.N / gNs) + ((p * W) / gNs) * L;
        const long long k0 = (p * W) % gNs;
#pragma unroll 1
        for (int k = 0; k < NBOX; ++k)
          col::tma_store_2d(&maps.out[0], (int)(k0 * XS), (int)(row0 + k * BR),
                            fast::saddr(reinterpret_cast<const unsigned char*>(oth) + (size_t)k * BR * W * ESZ));
        asm volatile("cp.async.bulk.commit_group;" ::: "memory");
      }
    }
    // the next tile's barrier after its stage wait orders this tile's last
    // reads of the work buffers before its first writes
  }
  if (threadIdx.x == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}


// The same passes with the tile gathered by 8 / 16-byte cp.async copies (one
// per element) instead of tensor copies, and the outputs stored from
// registers: for passes whose tiles do not fit the tensor maps (W does not
// divide N / L or Ns, or a row pitch is not a multiple of 16 bytes, as for
// N = 5^8 = 625 x 625).  A tile's W lanes are units u = tile W + lane of the
// whole batch, each with its own transform and column, so a tile may span
// transforms and the last one may be partial.  S = 1 or 2 stages, each
// thread waiting on its own copies (cp.async.wait_group) before a barrier.
template <typename T, int R0, int R1, int R2, int R3>
__global__ void __launch_bounds__(colshape::mix_threads(), 1) colmix_gather_kernel(const __grid_constant__ EngineArgs a) {
  using namespace colmix;
  typedef MixShape<T, R0, R1, R2, R3> Sh;
  typedef typename Vec<T>::t V;
  constexpr int L = Sh::L, W = Sh::W, NT = Sh::NT, LP = Sh::LP, NP = Sh::NP, TB = Sh::TB;
  constexpr int RL = NP == 4 ? R3 : (NP == 3 ? R2 : (NP == 2 ? R1 : R0));
  constexpr int NSL = L / RL;
  static_assert(NP >= 2, "a mixed shape has two or more in-block passes");
  static_assert(NT % W == 0, "each thread keeps one lane");
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ long long lane_t[W], lane_b[W];  // transform and unit of each lane of the current tile
  const int S = a.stages;  // 1 or 2
  V* const w0 = reinterpret_cast<V*>(smem + (size_t)S * TB);
  V* const w1 = reinterpret_cast<V*>(smem + (size_t)S * TB + Sh::WB);
  V* const stw = reinterpret_cast<V*>(smem + (size_t)S * TB + 2 * (size_t)Sh::WB);
  const int tw0 = a.pass[0].tw;
  for (int e = threadIdx.x; e < L - 1; e += NT) stw[e] = __ldg((const V*)a.tw + tw0 + e);
  const T sc = (T)a.scale;
  const bool conj = a.conj != 0;
  const long long G = gridDim.x;
  const long long stride = a.stride;
  const long long gNs = a.gNs;
  const unsigned kfac = (unsigned)(a.N / (gNs * L));
  const V* lo = (const V*)a.gtw_lo;
  const V* hi = (const V*)a.gtw_hi;
  const unsigned mask = (unsigned)a.gB - 1;
  const int lgB = 31 - __clz((int)a.gB);
  const int my_lane = threadIdx.x % W;  // the lane this thread gathers, twiddles and stores

  // every thread copies its lane's rows of tile `tile` into stage s (zeros
  // past the last unit), then closes its copy group (empty past the end)
  auto gather = [&](long long tile, int s) {
    V* st = reinterpret_cast<V*>(smem + (size_t)s * TB);
    if (tile < a.ntiles) {
      const long long u = tile * W + my_lane;
      if (u < a.nunits) {
        const long long t = u / stride, b = u - t * stride;
        const V* src = (const V*)a.in + t * a.N + b;
        for (int row = threadIdx.x / W; row < L; row += NT / W)
          lanep2::cpa<T>(lanep2::sa(st + row * W + my_lane), src + (long long)row * stride);
      } else {
        for (int row = threadIdx.x / W; row < L; row += NT / W) st[row * W + my_lane] = mk<V>(0, 0);
      }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  for (int s = 0; s < S; ++s) gather(blockIdx.x + (long long)s * G, s);

  int it = 0;
  for (long long tile = blockIdx.x; tile < a.ntiles; tile += G, ++it) {
    const int s = it % S;
    if (S == 2)
      asm volatile("cp.async.wait_group 1;" ::: "memory");
    else
      asm volatile("cp.async.wait_group 0;" ::: "memory");
    if (threadIdx.x < W) {
      const long long u = tile * W + threadIdx.x;
      const long long t = u / stride;
      lane_t[threadIdx.x] = t;
      lane_b[threadIdx.x] = u - t * stride;
    }
    __syncthreads();  // stage s complete (every thread's copies), lane table written
    const V* const stg = reinterpret_cast<const V*>(smem + (size_t)s * TB);
    const long long my_u = tile * W + my_lane;
    const long long my_b = lane_b[my_lane], my_t = lane_t[my_lane];

    // first pass (radix R0) from the dense stage, lane-fastest
    {
      constexpr int NB0 = L / R0;
      const unsigned k = (unsigned)(my_b % gNs);
      const unsigned kstep = a.notw ? 0u : k * kfac;
      for (int i = threadIdx.x; i < W * NB0; i += NT) {
        const int j = i / W;
        V v[R0];
#pragma unroll
        for (int r = 0; r < R0; ++r) {
          const int e = (j + r * NB0) * W + my_lane;
          if (GFFT_DCHECK(e < W * L, a.status)) v[r] = stg[e];
        }
        if (conj)
#pragma unroll
          for (int r = 0; r < R0; ++r) v[r] = cconj(v[r]);
        if (kstep && a.ftw) {
          const unsigned m0 = kstep * (unsigned)j;  // < N < 2^32
          const V t0 = cmul(__ldg(lo + (m0 & mask)), __ldg(hi + (m0 >> lgB)));
          const V* t2 = (const V*)a.ftw + k;
#pragma unroll
          for (int r = 0; r < R0; ++r) v[r] = cmul(v[r], cmul(t0, __ldg(t2 + (size_t)r * gNs)));
        } else if (kstep) {
#pragma unroll
          for (int r = 0; r < R0; ++r) {
            const unsigned m = kstep * (unsigned)(j + r * NB0);  // < N < 2^32
            v[r] = cmul(v[r], cmul(__ldg(lo + (m & mask)), __ldg(hi + (m >> lgB))));
          }
        }
        dft<T, V, R0>(v);
        V* d = w0 + my_lane * LP;
#pragma unroll
        for (int r = 0; r < R0; ++r) d[padi<T>(j * R0 + r)] = v[r];
      }
    }
    __syncthreads();  // every thread has read stage s
    gather(tile + (long long)S * G, s);
    const V* src = w0;
    if constexpr (NP >= 3) {
      mid<T, L, W, NT, LP, R1, R0>(w0, w1, stw, a.pass[1].tw - tw0, a.status);
      __syncthreads();
      src = w1;
    }
    if constexpr (NP >= 4) {
      mid<T, L, W, NT, LP, R2, R0 * R1>(w1, w0, stw, a.pass[2].tw - tw0, a.status);
      __syncthreads();
      src = w0;
    }
    const int twl = a.pass[NP - 1].tw - tw0;
    constexpr int NBL = L / RL;
    if (gNs == 1) {
      // first global pass: lane-major, each lane's L outputs contiguous
      for (int i = threadIdx.x; i < W * NBL; i += NT) {
        const int lane = i / NBL, j = i - lane * NBL;
        if (tile * W + lane >= a.nunits) continue;
        const V* sp = src + lane * LP;
        V v[RL];
#pragma unroll
        for (int r = 0; r < RL; ++r) v[r] = sp[padi<T>(j + r * NBL)];
#pragma unroll
        for (int r = 1; r < RL; ++r) v[r] = cmul(v[r], stw[twl + j + (r - 1) * NSL]);
        dft<T, V, RL>(v);
        const long long e0 = lane_t[lane] * a.N + lane_b[lane] * L + j;
        V* d = (V*)a.out + e0;
#pragma unroll
        for (int r = 0; r < RL; ++r) {
          V x = v[r];
          if (conj) x = cconj(x);
          if (GFFT_DCHECK(e0 + r * NSL < a.nunits * L, a.status)) d[r * NSL] = cscale(x, sc);
        }
      }
    } else if (my_u < a.nunits) {
      // later global passes: lane-fastest, y[t N + (b - k) L + k + s Ns]
      const long long k = my_b % gNs;
      const long long e0 = my_t * a.N + (my_b - k) * L + k;
      V* d = (V*)a.out + e0;
      for (int i = threadIdx.x; i < W * NBL; i += NT) {
        const int j = i / W;
        const V* sp = src + my_lane * LP;
        V v[RL];
#pragma unroll
        for (int r = 0; r < RL; ++r) v[r] = sp[padi<T>(j + r * NBL)];
#pragma unroll
        for (int r = 1; r < RL; ++r) v[r] = cmul(v[r], stw[twl + j + (r - 1) * NSL]);
        dft<T, V, RL>(v);
#pragma unroll
        for (int r = 0; r < RL; ++r) {
          V x = v[r];
          if (conj) x = cconj(x);
          if (GFFT_DCHECK(e0 + (long long)(j + r * NSL) * gNs < a.nunits * L, a.status))
            d[(long long)(j + r * NSL) * gNs] = cscale(x, sc);
        }
      }
    }
    __syncthreads();  // the lane table and the work buffers are reused by the next tile
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
}

}  // namespace gfft
