// Column tiles of a multi-pass power-of-two length, moved by the tensor
// memory accelerator (variant 9).
//
// One launch runs one global pass (plan.h): for every unit b of every
// transform t, the L elements x[t*N + b + r*(N/L)] are transformed by the
// in-block Stockham passes of the length-specialised kernels.  Seen as a
// matrix with rows of N/L elements, the input of ANY global pass is
//   row = t*L + r, column = b,
// so the W adjacent units of a tile form one W x L box of that matrix.  The
// output of pass g (Ns = product of the earlier pass lengths) is
//   y[t*N + (b/Ns)*Ns*L + k + r*Ns],  k = b mod Ns,
// which is again a box of W columns x L rows of the matrix with rows of Ns
// elements (row = t*N/Ns + (b/Ns)*L + r, column = k), or, for the first pass
// (Ns = 1), W contiguous runs of L elements.
//
// Data flow per tile (persistent blocks, one per SM, S stages):
//  - 2-D tensor copies (cp.async.bulk.tensor, boxes of W x 256 rows) bring
//    the tile into a dense [L][W] stage, completing on an mbarrier (bounded
//    waits, GFFT_E_TIMEOUT on expiry).  The copies of tile i+S are issued as
//    soon as every thread has read tile i's stage.
//  - First in-block pass with the lane-fastest thread mapping (a warp reads
//    32 consecutive words of the dense stage: no bank conflict), conjugation
//    for the inverse and the four-step twiddle W_N^(k s N/(Ns L)) applied in
//    registers, radix-16 butterfly, written to a padded [lane][Lp] work
//    buffer whose lane stride Lp makes that write conflict-free as well.
//  - Later in-block passes with lane groups: a lane's butterflies stay with
//    the same consecutive threads in every pass, so these passes synchronise
//    only those threads (a warp, or a named barrier for lanes of 64 or more
//    threads) instead of the whole block.
//  - The four-step twiddle of a later global pass is factored as
//    W_N^(k kf (j + r L/16)) = W_N^(k kf j) * W_(16 Ns)^(k r): one two-level
//    lookup per thread and one load per element from a [16][Ns] table whose
//    rows are read by adjacent lanes (one wavefront), instead of two
//    scattered lookups per element.
//  - First global pass: the result is stored straight from registers
//    (coalesced: each lane's outputs are contiguous).  Later passes: the last
//    in-block pass is read lane-fastest, written dense [L][W] into the work
//    buffer and sent out by 2-D tensor stores, which the next tile's first
//    write into the work buffer waits for (cp.async.bulk.wait_group.read).
//  - Real transforms (RF = 1: forward post pass fused into the last global
//    pass; RF = 2: inverse pre pass fused into the first): the reference's
//    Separate step (src/gfftswap.h:239-287) pairs X_k with X_(n-k), and
//    element k = c + s S (S = N / L units) pairs with column S - c, row
//    L - 1 - s.  A real tile therefore holds W / 2 columns c = p W/2 + i
//    (region A) and their mirrors S - c (region B, one box of consecutive
//    columns), plus, in the transform's first tile, column S / 2 in place of
//    the mirror of column 0 (region C; columns 0 and S / 2 pair with
//    themselves).  The pairs are combined in shared memory between the
//    global load and the first butterflies (RF = 2) or between the last
//    butterflies and the store (RF = 1).  FP32 boxes must start on an even
//    column: region B is loaded two columns wider from the even column below
//    and, with region C, stored by plain stores.
//
// This replaces the deep levels of the reference's recursion, InTimeOOP
// (src/gfftalg.h:459-507) with its combine step DFTk_x_Im_T
// (src/gfftalg.h:169-267): one global pass is one level of DFT_L x I_M with
// the twiddles of that level, over the whole batch.
#pragma once
#include <cuda.h>  // CUtensorMap (type only: no driver symbols are linked)
#include <cuda_runtime.h>
#include <stdint.h>

#include "butterflies.cuh"
#include "colshape.h"
#include "dcheck.cuh"
#include "plan.h"
#include "spec.cuh"
#include "tma.cuh"

namespace gfft {
namespace col {

using spec::npass_of;
using spec::ns_of;
using spec::radix_of;

template <typename T> constexpr int esz() { return (int)sizeof(typename Vec<T>::t); }

// launch shape of a pass (colshape.h: the same arithmetic on the host)
template <typename T, int L, int TK = 64> struct Shape {
  typedef typename Vec<T>::t V;
  static constexpr int W = colshape::lanes(esz<T>(), L, TK);
  static constexpr int NT = W * L / 16;
  static constexpr int NP = npass_of(L);
  static constexpr int LP = colshape::lane_stride(esz<T>(), L, W);
  static constexpr int TB = W * L * esz<T>();       // bytes of one tile
  static constexpr int BR = L < 256 ? L : 256;      // rows per tensor box
  static constexpr int NBOX = L / BR;
  static constexpr int WORK = colshape::work_bytes(esz<T>(), L, TK);
};

// Tile geometry of a pass: RF = 0 one box of W columns; RF = 1, 2 (real
// pairs) regions A (H = W/2 columns), B (HB columns: the H mirrors, FP32 two
// wider) and C (HC columns: column S/2), each a dense [L][width] block.
template <typename T, int L, int RF, int TK = 64> struct Geo {
  static constexpr int W = Shape<T, L, TK>::W;
  static constexpr int H = W / 2;
  static constexpr bool F64 = esz<T>() == 16;
  static constexpr int WA = colshape::width_a(esz<T>(), L, RF);
  static constexpr int HB = colshape::width_b(esz<T>(), L, RF);
  static constexpr int BOFF = F64 ? 0 : 1;  // first needed column inside region B
  static constexpr int HC = colshape::width_c(esz<T>(), RF);
  static constexpr int OFF_B = WA * L, OFF_C = (WA + HB) * L;  // elements
  static constexpr int TB = colshape::stage_bytes(esz<T>(), L, RF, TK);
  static constexpr int FB = colshape::ftw_box_bytes(esz<T>(), L, RF, TK);  // four-step factor block
  static constexpr int TS = TB + FB;                                      // stage stride
  static constexpr int WORK = colshape::work_bytes_rf(esz<T>(), L, RF, TK);
};

// where lane `lane` of tile p finds its column: smem element offset of row s
// is base + s * width + col; `unit` is the column index within the
// transform (the unit b of the global pass)
struct LaneSrc {
  int base, width, col;
  long long unit;
};
template <typename T, int L, int RF, int TK = 64>
__device__ __forceinline__ LaneSrc lane_src(int lane, long long p, long long S) {
  typedef Geo<T, L, RF, TK> G;
  LaneSrc r;
  if (!RF) {
    r.base = 0;
    r.width = G::W;
    r.col = lane;
    r.unit = p * G::W + lane;
  } else if (lane < G::H) {
    r.base = 0;
    r.width = G::H;
    r.col = lane;
    r.unit = p * G::H + lane;
  } else if (p == 0 && lane == G::H) {
    r.base = G::OFF_C;
    r.width = G::HC;
    r.col = 0;
    r.unit = S / 2;
  } else {
    const int i = lane - G::H;
    r.base = G::OFF_B;
    r.width = G::HB;
    r.col = G::BOFF + G::H - 1 - i;
    r.unit = S - (p * G::H + i);
  }
  return r;
}

// The reference's Separate step on one pair (k, n - k) held in shared
// memory (src/gfftswap.h:239-287): forward (dir 1) turns the complex FFT Z
// of the packed reals into X_k = F + W_2n^k G, F = (Z_k + conj Z_(n-k)) / 2,
// G = -i (Z_k - conj Z_(n-k)) / 2 (and the mirror formula for X_(n-k));
// inverse (dir 2) recovers Z from the packed spectrum.  k = 0 packs / unpacks
// (X_0, X_n); a self pair (k = n/2) writes once.
template <typename T>
__device__ __forceinline__ void real_pair(typename Vec<T>::t* pa, typename Vec<T>::t* pb, long long q, long long qm,
                                          const typename Vec<T>::t* __restrict__ rtw, int dir) {
  typedef typename Vec<T>::t V;
  const V a = *pa, b = *pb;
  if (dir == 1) {
    V F = mk<V>((T)0.5 * (a.x + b.x), (T)0.5 * (a.y - b.y));
    V G = mk<V>((T)0.5 * (a.y + b.y), (T)-0.5 * (a.x - b.x));
    V xq = cadd(F, cmul(__ldg(rtw + q), G));
    V F2 = mk<V>((T)0.5 * (b.x + a.x), (T)0.5 * (b.y - a.y));
    V G2 = mk<V>((T)0.5 * (b.y + a.y), (T)-0.5 * (b.x - a.x));
    V xm = cadd(F2, cmul(__ldg(rtw + qm), G2));
    *pa = xq;
    if (qm != q) *pb = xm;
  } else {
    V F = mk<V>((T)0.5 * (a.x + b.x), (T)0.5 * (a.y - b.y));
    V D = mk<V>((T)0.5 * (a.x - b.x), (T)0.5 * (a.y + b.y));
    V G = cmul(D, cconj(__ldg(rtw + q)));
    V zq = mk<V>(F.x - G.y, F.y + G.x);
    V F2 = mk<V>((T)0.5 * (b.x + a.x), (T)0.5 * (b.y - a.y));
    V D2 = mk<V>((T)0.5 * (b.x - a.x), (T)0.5 * (b.y + a.y));
    V G2 = cmul(D2, cconj(__ldg(rtw + qm)));
    V zm = mk<V>(F2.x - G2.y, F2.y + G2.x);
    *pa = zq;
    if (qm != q) *pb = zm;
  }
}
template <typename T>
__device__ __forceinline__ void real_zero(typename Vec<T>::t* p0, int dir) {
  typedef typename Vec<T>::t V;
  const V z = *p0;
  *p0 = dir == 1 ? mk<V>(z.x + z.y, z.x - z.y) : mk<V>((T)0.5 * (z.x + z.y), (T)0.5 * (z.x - z.y));
}

// All pairs of a real tile, in place on a buffer laid out as the stage
// (regions A / B / C): H * L items over the block's threads.  Item (i, s):
// column c = p H + i row s with column S - c row L - 1 - s; in the first
// tile, column 0 pairs rows s and L - s (items s < L/2, item 0 also the
// self pair at row L/2 and the packed X_0 / X_n) and column S/2 pairs rows
// s and L - 1 - s (items L/2 .. L-1).
template <typename T, int L, int RF, int NT>
__device__ __forceinline__ void real_tile(typename Vec<T>::t* buf, long long p, long long S, long long n,
                                          const typename Vec<T>::t* __restrict__ rtw, int* status) {
  typedef Geo<T, L, RF> G;
  typedef typename Vec<T>::t V;
  for (int it = threadIdx.x; it < G::H * L; it += NT) {
    const int i = it % G::H, s = it / G::H;
    int la = i, sa = s, lb, sb;
    if (p == 0 && i == 0) {
      if (s == 0) {
        const LaneSrc z = lane_src<T, L, RF>(0, p, S);
        real_zero<T>(buf + z.base + z.col, RF);
        V* m = buf + z.base + (L / 2) * z.width + z.col;
        real_pair<T>(m, m, n / 2, n / 2, rtw, RF);
        continue;
      }
      if (s < L / 2) {
        lb = 0;
        sb = L - s;
      } else {
        la = G::H;
        sa = s - L / 2;
        lb = G::H;
        sb = L - 1 - sa;
      }
    } else {
      lb = G::H + i;
      sb = L - 1 - s;
    }
    const LaneSrc A = lane_src<T, L, RF>(la, p, S), B = lane_src<T, L, RF>(lb, p, S);
    const long long q = A.unit + (long long)sa * S;
    const int ea = A.base + sa * A.width + A.col, eb = B.base + sb * B.width + B.col;
    if (GFFT_DCHECK(ea >= 0 && eb >= 0 && ea < G::TB / (int)sizeof(V) && eb < G::TB / (int)sizeof(V) && q > 0 &&
                        q < n,
                    status))
      real_pair<T>(buf + ea, buf + eb, q, n - q, rtw, RF);
  }
}

// tensor maps of one launch: RF = 0 uses [0] (boxes of W units); a real pass
// [0] region A, [1] region B, [2] region C, each for its own box width
struct ColMaps {
  CUtensorMap in[3];
  CUtensorMap out[3];
};

// Butterfly q of this thread under the two mappings: lane-fastest (LF: lane
// = b mod W, j = b / W with b = tid + q NT) and lane groups (the NT / W
// threads of a lane are consecutive and keep that lane in every pass: j =
// tid mod TPL + q TPL), so the passes between the first and the last only
// synchronise a lane's own threads.
template <int W, int NT, bool LF> __device__ __forceinline__ int lane_of(int q) {
  return LF ? (int)((threadIdx.x + q * NT) % W) : (int)(threadIdx.x / (NT / W));
}
template <int W, int NT, bool LF> __device__ __forceinline__ int j_of(int q) {
  return LF ? (int)((threadIdx.x + q * NT) / W) : (int)(threadIdx.x % (NT / W) + q * (NT / W));
}

// synchronise the threads of this thread's lane group: a warp (or part of
// one) for lanes of at most 32 threads, else named barrier 1 + lane
template <int W, int NT> __device__ __forceinline__ void group_sync() {
  constexpr int TPL = NT / W;
  if constexpr (TPL <= 32) {
    __syncwarp();
  } else {
    asm volatile("bar.sync %0, %1;" ::"r"(1 + (int)(threadIdx.x / TPL)), "r"(TPL) : "memory");
  }
}

template <typename T, int L, int P, bool LF, int TK>
__device__ __forceinline__ void rd(typename Vec<T>::t (&v)[16], const typename Vec<T>::t* buf, int* st) {
  typedef Shape<T, L, TK> S;
  constexpr int R = radix_of(L, P), NB = L / R, Q = 16 / R;
  (void)st;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int lane = lane_of<S::W, S::NT, LF>(q), j = j_of<S::W, S::NT, LF>(q);
    const typename Vec<T>::t* s = buf + lane * S::LP;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int e = lane * S::LP + spec::padi<T>(j + r * NB);
      if (GFFT_DCHECK(e >= 0 && e < S::W * S::LP, st)) v[q * R + r] = s[spec::padi<T>(j + r * NB)];
    }
  }
}

template <typename T, int L, int P, bool LF, int TK>
__device__ __forceinline__ void cp(typename Vec<T>::t (&v)[16], const typename Vec<T>::t* tw, int twoff) {
  typedef Shape<T, L, TK> S;
  typedef typename Vec<T>::t V;
  constexpr int R = radix_of(L, P), Q = 16 / R, NS = ns_of(L, P);
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    if constexpr (NS > 1) {
      const int j = j_of<S::W, S::NT, LF>(q);
      const V* t = tw + twoff + (j % NS);  // shared memory
#pragma unroll
      for (int r = 1; r < R; ++r) v[q * R + r] = cmul(v[q * R + r], t[(r - 1) * NS]);
    }
    dft<T, V, R>(&v[q * R]);
  }
}

template <typename T, int L, int P, bool LF, int TK>
__device__ __forceinline__ void wr(const typename Vec<T>::t (&v)[16], typename Vec<T>::t* buf, int* st) {
  typedef Shape<T, L, TK> S;
  constexpr int R = radix_of(L, P), Q = 16 / R, NS = ns_of(L, P);
  (void)st;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int lane = lane_of<S::W, S::NT, LF>(q), j = j_of<S::W, S::NT, LF>(q);
    const int k = j % NS;
    const int base = (j - k) * R + k;
    typename Vec<T>::t* d = buf + lane * S::LP;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int e = lane * S::LP + spec::padi<T>(base + r * NS);
      if (GFFT_DCHECK(e >= 0 && e < S::W * S::LP, st)) d[spec::padi<T>(base + r * NS)] = v[q * R + r];
    }
  }
}

// in-block passes P .. NP-2 with lane groups, in place on the work buffer;
// the caller synchronises after the last write
template <typename T, int L, int P, int TK>
__device__ __forceinline__ void middle(typename Vec<T>::t (&v)[16], typename Vec<T>::t* work,
                                       const typename Vec<T>::t* tw, int tw0, const BlockPass* bp, int* st) {
  typedef Shape<T, L, TK> S;
  constexpr int NP = npass_of(L);
  if constexpr (P < NP - 1) {
    if constexpr (P > 1) group_sync<S::W, S::NT>();
    rd<T, L, P, false, TK>(v, work, st);
    cp<T, L, P, false, TK>(v, tw, bp[P].tw - tw0);
    group_sync<S::W, S::NT>();
    wr<T, L, P, false, TK>(v, work, st);
    middle<T, L, P + 1, TK>(v, work, tw, tw0, bp, st);
  }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(map), "r"(x), "r"(y), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, int x, int y, uint32_t src) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(map), "r"(x),
               "r"(y), "r"(src)
               : "memory");
}

}  // namespace col


template <typename T, int L, int RF, int TK = 64>
__global__ void __launch_bounds__(col::Shape<T, L, TK>::NT, 64 / TK)
    col_kernel(const __grid_constant__ EngineArgs a, const __grid_constant__ col::ColMaps maps) {
  using namespace col;
  typedef Shape<T, L, TK> Sh;
  typedef Geo<T, L, RF, TK> Gm;
  typedef typename Vec<T>::t V;
  constexpr int W = Sh::W, NT = Sh::NT, NP = Sh::NP, TB = Gm::TB, TS = Gm::TS, BR = Sh::BR, NBOX = Sh::NBOX;
  constexpr int NB0 = L / radix_of(L, 0);  // first pass: radix 16, one butterfly per thread
  constexpr int NBL = L / radix_of(L, NP - 1), QL = 16 / radix_of(L, NP - 1);
  constexpr int RL = radix_of(L, NP - 1);
  constexpr int XS = esz<T>() / 8;  // tensor-map elements (8 bytes) per complex element
  static_assert(radix_of(L, 0) == 16, "first pass radix 16");
  static_assert(NP > 1, "column tiles have two or more in-block passes");
  extern __shared__ __align__(1024) unsigned char smem[];
  const int S = a.stages;
  V* const work = reinterpret_cast<V*>(smem + (size_t)S * TS);
  // the pass's in-block twiddles (L - 1 entries from pass[0].tw on),
  // copied once per block: shared-memory loads instead of scattered L1 ones
  constexpr int TWN = colshape::tw_entries(L);
  V* const stw = reinterpret_cast<V*>(smem + (size_t)S * TS + Gm::WORK);
  uint64_t* const bars =
      reinterpret_cast<uint64_t*>(smem + (size_t)S * TS + Gm::WORK + colshape::tw_bytes(esz<T>(), L));
  const int tw0 = a.pass[0].tw;
  for (int e = threadIdx.x; e < TWN; e += NT) stw[e] = __ldg((const V*)a.tw + tw0 + e);
  const V* tw = stw;
  const V* rtw = (const V*)a.rtw;
  const T sc = (T)a.scale;
  const bool conj = a.conj != 0;
  const long long G = gridDim.x;
  const long long stride = a.stride;  // N / L: units per transform
  const long long tpt = stride / W;   // tiles per transform
  const long long gNs = a.gNs;
  const bool fbox = !RF && a.ftw_box && a.ftw && gNs > 1;  // factors staged with the tile
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
    const int y = (int)(t * L);
    const uint32_t bar = fast::saddr(&bars[s]);
    unsigned char* st = smem + (size_t)s * TS;
    if (!RF) {
      fast::mbar_expect_tx(bar, (uint32_t)(TB + (fbox ? Gm::FB : 0)));
#pragma unroll 1
      for (int k = 0; k < NBOX; ++k)
        tma_load_2d(fast::saddr(st + (size_t)k * BR * W * esz<T>()), &maps.in[0], (int)(p * W * XS), y + k * BR, bar);
      // the tile's units p W .. p W + W - 1 have k = (p W) mod Ns + lane
      if (fbox) tma_load_2d(fast::saddr(st + TB), &maps.in[1], (int)(((p * W) % gNs) * XS), 0, bar);
    } else {
      const int wc = p == 0 ? Gm::HC : 0;
      fast::mbar_expect_tx(bar, (uint32_t)(NBOX * BR * (Gm::H + Gm::HB + wc) * esz<T>()));
      const int xa = (int)(p * Gm::H * XS);
      const int xb = (int)((stride - p * Gm::H - Gm::H + 1 - Gm::BOFF) * XS);
      const int xc = (int)((stride / 2) * XS);
#pragma unroll 1
      for (int k = 0; k < NBOX; ++k) {
        tma_load_2d(fast::saddr(st + (size_t)k * BR * Gm::H * esz<T>()), &maps.in[0], xa, y + k * BR, bar);
        tma_load_2d(fast::saddr(st + ((size_t)Gm::OFF_B + (size_t)k * BR * Gm::HB) * esz<T>()), &maps.in[1], xb,
                    y + k * BR, bar);
        if (wc)
          tma_load_2d(fast::saddr(st + ((size_t)Gm::OFF_C + (size_t)k * BR * Gm::HC) * esz<T>()), &maps.in[2], xc,
                      y + k * BR, bar);
      }
    }
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
    V* const st = reinterpret_cast<V*>(smem + (size_t)s * TS);
    if constexpr (RF == 2) {
      // real inverse: recover Z from the packed spectrum before the butterflies
      real_tile<T, L, RF, NT>(st, p, stride, a.N, rtw, a.status);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // generic writes before the stage's next copy
      __syncthreads();
    }

    // first in-block pass, lane-fastest: lane = tid % W, j = tid / W
    {
      const int lane = threadIdx.x % W, j = threadIdx.x / W;
      const LaneSrc src = lane_src<T, L, RF, TK>(lane, p, stride);
      const V* sp = st + src.base + src.col;
#pragma unroll
      for (int r = 0; r < 16; ++r) {
        if (GFFT_DCHECK(src.base + src.col + (j + r * NB0) * src.width >= 0 &&
                            src.base + src.col + (j + r * NB0) * src.width < TB / (int)sizeof(V),
                        a.status))
          v[r] = sp[(j + r * NB0) * src.width];
      }
      if (conj)
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = cconj(v[r]);
      if (!a.notw) {
        const unsigned k = (unsigned)(src.unit % gNs);
        const unsigned kstep = k * kfac;
        if (kstep && a.ftw) {
          // W_N^(kstep (j + r NB0)) = W_N^(kstep j) * W_(16 Ns)^(k r): one lookup of
          // the first factor per thread, the second from the [r][k] table
          const unsigned m0 = kstep * (unsigned)j;  // < N < 2^32
          const V t0 = cmul(__ldg(lo + (m0 & mask)), __ldg(hi + (m0 >> lgB)));
          if (fbox) {
            // the tile's block of factors, staged with it: [r][lane]
            const V* t2 = reinterpret_cast<const V*>(reinterpret_cast<const unsigned char*>(st) + TB) + lane;
#pragma unroll
            for (int r = 0; r < 16; ++r) v[r] = cmul(v[r], cmul(t0, t2[r * W]));
          } else {
            const V* t2 = (const V*)a.ftw + k;
#pragma unroll
            for (int r = 0; r < 16; ++r) v[r] = cmul(v[r], cmul(t0, __ldg(t2 + (size_t)r * gNs)));
          }
        } else if (kstep) {
#pragma unroll
          for (int r = 0; r < 16; ++r) {
            const unsigned m = kstep * (unsigned)(j + r * NB0);  // < N < 2^32
            v[r] = cmul(v[r], cmul(__ldg(lo + (m & mask)), __ldg(hi + (m >> lgB))));
          }
        }
      }
      dft<T, V, 16>(v);
    }
    // the previous tile's tensor store has read the work buffer; every
    // thread has read stage s
    if (threadIdx.x == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0 && !a.debug_no_issue) {
      const long long nt = tile + (long long)S * G;
      if (nt < a.ntiles) issue(nt, s);
    }
    wr<T, L, 0, true, TK>(v, work, a.status);
    __syncthreads();
    middle<T, L, 1, TK>(v, work, tw, tw0, a.pass, a.status);
    if (gNs == 1) {
      // first global pass: lane groups, each lane's L outputs contiguous
      if constexpr (NP > 2) group_sync<W, NT>();
      rd<T, L, NP - 1, false, TK>(v, work, a.status);
      cp<T, L, NP - 1, false, TK>(v, tw, a.pass[NP - 1].tw - tw0);
      V* o = (V*)a.out + t * a.N;
#pragma unroll
      for (int q = 0; q < QL; ++q) {
        const int lane = lane_of<W, NT, false>(q), j = j_of<W, NT, false>(q);
        const long long e0 = t * a.N + lane_src<T, L, RF, TK>(lane, p, stride).unit * L + j;
        V* d = (V*)a.out + e0;
#pragma unroll
        for (int r = 0; r < RL; ++r) {
          V x = v[q * RL + r];
          if (conj) x = cconj(x);
          if (GFFT_DCHECK(e0 + r * NBL >= 0 && e0 + r * NBL < a.nunits * L, a.status)) d[r * NBL] = cscale(x, sc);
        }
      }
    } else {
      // later global passes: lane-fastest, dense tile in the work buffer, tensor stores
      if constexpr (NP > 2) __syncthreads();
      rd<T, L, NP - 1, true, TK>(v, work, a.status);
      cp<T, L, NP - 1, true, TK>(v, tw, a.pass[NP - 1].tw - tw0);
      __syncthreads();
#pragma unroll
      for (int q = 0; q < QL; ++q) {
        const int lane = lane_of<W, NT, true>(q), j = j_of<W, NT, true>(q);
        const LaneSrc dsrc = lane_src<T, L, RF, TK>(lane, p, stride);
#pragma unroll
        for (int r = 0; r < RL; ++r) {
          V x = v[q * RL + r];
          if (conj) x = cconj(x);
          const int e = dsrc.base + (j + r * NBL) * dsrc.width + dsrc.col;
          if (GFFT_DCHECK(e >= 0 && e < Gm::WORK / (int)sizeof(V), a.status)) work[e] = cscale(x, sc);
        }
      }
      if constexpr (RF == 1) {
        // real forward: the packed half spectrum from Z, in place
        __syncthreads();
        real_tile<T, L, RF, NT>(work, p, stride, a.N, rtw, a.status);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      const long long row0 = t * (a.N / gNs) + ((p * W) / gNs) * L;
      if (!RF) {
        if (threadIdx.x == 0) {
          const long long k0 = (p * W) % gNs;
#pragma unroll 1
          for (int k = 0; k < NBOX; ++k)
            tma_store_2d(&maps.out[0], (int)(k0 * XS), (int)(row0 + k * BR),
                         fast::saddr(smem + (size_t)S * TS + (size_t)k * BR * W * esz<T>()));
          asm volatile("cp.async.bulk.commit_group;" ::: "memory");
        }
      } else {
        // a real pass is the last one: Ns = S, row0 = t L.  Region A by tensor
        // stores; region B by tensor stores where its box starts on a 16-byte
        // boundary (FP64) and lies inside the tensor (not the first tile, whose
        // box reaches column S), else, with region C, by plain stores
        unsigned char* wb = smem + (size_t)S * TS;
        const bool tb_b = Gm::F64 && p != 0;
        if (threadIdx.x == 0) {
#pragma unroll 1
          for (int k = 0; k < NBOX; ++k) {
            tma_store_2d(&maps.out[0], (int)(p * Gm::H * XS), (int)(row0 + k * BR),
                         fast::saddr(wb + (size_t)k * BR * Gm::H * esz<T>()));
            if (tb_b)
              tma_store_2d(&maps.out[1], (int)((stride - p * Gm::H - Gm::H + 1) * XS), (int)(row0 + k * BR),
                           fast::saddr(wb + ((size_t)Gm::OFF_B + (size_t)k * BR * Gm::HB) * esz<T>()));
          }
          asm volatile("cp.async.bulk.commit_group;" ::: "memory");
        }
        V* o = (V*)a.out + t * a.N;
        for (int e = threadIdx.x; e < (Gm::H + 1) * L; e += NT) {
          const int m = e % (Gm::H + 1), srow = e / (Gm::H + 1);
          if (m < Gm::H) {
            const long long col = stride - p * Gm::H - Gm::H + 1 + m;
            if (!tb_b && col < stride && GFFT_DCHECK(col >= 0 && srow < L, a.status))
              o[srow * stride + col] = work[Gm::OFF_B + srow * Gm::HB + Gm::BOFF + m];
          } else if (p == 0) {
            o[srow * stride + stride / 2] = work[Gm::OFF_C + srow * Gm::HC];
          }
        }
      }
    }
  }
  if (threadIdx.x == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

}  // namespace gfft
