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
//  - Later in-block passes with the unit-major mapping (spec.cuh).
//  - First global pass: the result is stored straight from registers
//    (coalesced: each lane's outputs are contiguous).  Later passes: the last
//    in-block pass is read lane-fastest, written dense [L][W] into the work
//    buffer and sent out by 2-D tensor stores, which the next tile's first
//    write into the work buffer waits for (cp.async.bulk.wait_group.read).
//
// This replaces the deep levels of the reference's recursion, InTimeOOP
// (src/gfftalg.h:459-507) with its combine step DFTk_x_Im_T
// (src/gfftalg.h:169-267): one global pass is one level of DFT_L x I_M with
// the twiddles of that level, over the whole batch.
#include <cuda.h>  // CUtensorMap and the encoder's prototype (no driver symbols are linked)
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "butterflies.cuh"
#include "plan.h"
#include "spec.cuh"
#include "tma.cuh"

namespace gfft {
namespace col {

using spec::npass_of;
using spec::ns_of;
using spec::radix_of;

template <typename T> constexpr int esz() { return (int)sizeof(typename Vec<T>::t); }
// units per tile: tiles of about 64 KB, rows of at least 2 units
template <typename T, int L> constexpr int lanes() {
  return (65536 / esz<T>()) / L > 64 ? 64 : ((65536 / esz<T>()) / L < 2 ? 2 : (65536 / esz<T>()) / L);
}
// Lane stride of the padded work buffer (elements).  In-lane positions are
// padded by spec::padi (one slot per 2^PS).  The first pass writes with the
// lane-fastest mapping: a warp covers all W lanes and 32/W butterflies, whose
// 16 outputs are consecutive, so a write lands on slot (lane * Lp + j + r)
// mod 16 (8-byte elements, 16 slots per 128-byte wavefront) or on
// (lane * Lp + 2 j + r') mod 8 (16-byte elements, 8 slots): Lp = 32 / W mod
// 16 (FP32) and Lp odd (FP64) put exactly two (four) accesses on every slot.
template <typename T, int L, int W> constexpr int lane_stride() {
  constexpr int base = L + (L >> spec::Cfg<T>::PS);
  if (esz<T>() == 16 || W >= 32) return (base & 1) ? base : base + 1;
  constexpr int want = (32 / W) % 16;
  return base + ((want - base % 16) + 16) % 16;
}

template <typename T, int L> struct Shape {
  typedef typename Vec<T>::t V;
  static constexpr int W = lanes<T, L>();
  static constexpr int NT = W * L / 16;
  static constexpr int NP = npass_of(L);
  static constexpr int LP = lane_stride<T, L, W>();
  static constexpr int TB = W * L * esz<T>();       // bytes of one tile
  static constexpr int BR = L < 256 ? L : 256;      // rows per tensor box
  static constexpr int NBOX = L / BR;
  static constexpr int WORK = ((W * LP * esz<T>() + 1023) / 1024) * 1024;
};

// butterfly q of this thread: (lane, j) under the two mappings
template <int W, int NB, int NT, bool LF> __device__ __forceinline__ int lane_of(int q) {
  const int b = threadIdx.x + q * NT;
  return LF ? b % W : b / NB;
}
template <int W, int NB, int NT, bool LF> __device__ __forceinline__ int j_of(int q) {
  const int b = threadIdx.x + q * NT;
  return LF ? b / W : b % NB;
}

template <typename T, int L, int P, bool LF>
__device__ __forceinline__ void rd(typename Vec<T>::t (&v)[16], const typename Vec<T>::t* buf) {
  typedef Shape<T, L> S;
  constexpr int R = radix_of(L, P), NB = L / R, Q = 16 / R;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int lane = lane_of<S::W, NB, S::NT, LF>(q), j = j_of<S::W, NB, S::NT, LF>(q);
    const typename Vec<T>::t* s = buf + lane * S::LP;
#pragma unroll
    for (int r = 0; r < R; ++r) v[q * R + r] = s[spec::padi<T>(j + r * NB)];
  }
}

template <typename T, int L, int P, bool LF>
__device__ __forceinline__ void cp(typename Vec<T>::t (&v)[16], const typename Vec<T>::t* __restrict__ tw, int twoff) {
  typedef Shape<T, L> S;
  typedef typename Vec<T>::t V;
  constexpr int R = radix_of(L, P), NB = L / R, Q = 16 / R, NS = ns_of(L, P);
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    if constexpr (NS > 1) {
      const int j = j_of<S::W, NB, S::NT, LF>(q);
      const V* t = tw + twoff + (j % NS);
#pragma unroll
      for (int r = 1; r < R; ++r) v[q * R + r] = cmul(v[q * R + r], __ldg(t + (r - 1) * NS));
    }
    dft<T, V, R>(&v[q * R]);
  }
}

template <typename T, int L, int P, bool LF>
__device__ __forceinline__ void wr(const typename Vec<T>::t (&v)[16], typename Vec<T>::t* buf) {
  typedef Shape<T, L> S;
  constexpr int R = radix_of(L, P), NB = L / R, Q = 16 / R, NS = ns_of(L, P);
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int lane = lane_of<S::W, NB, S::NT, LF>(q), j = j_of<S::W, NB, S::NT, LF>(q);
    const int k = j % NS;
    const int base = (j - k) * R + k;
    typename Vec<T>::t* d = buf + lane * S::LP;
#pragma unroll
    for (int r = 0; r < R; ++r) d[spec::padi<T>(base + r * NS)] = v[q * R + r];
  }
}

// in-block passes P .. NP-2, unit-major, in place on the work buffer
template <typename T, int L, int P>
__device__ __forceinline__ void middle(typename Vec<T>::t (&v)[16], typename Vec<T>::t* work,
                                       const typename Vec<T>::t* tw, const BlockPass* bp) {
  constexpr int NP = npass_of(L);
  if constexpr (P < NP - 1) {
    rd<T, L, P, false>(v, work);
    cp<T, L, P, false>(v, tw, bp[P].tw);
    __syncthreads();
    wr<T, L, P, false>(v, work);
    __syncthreads();
    middle<T, L, P + 1>(v, work, tw, bp);
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

template <typename T, int L>
__global__ void __launch_bounds__(col::Shape<T, L>::NT, 1)
    col_kernel(const __grid_constant__ EngineArgs a, const __grid_constant__ CUtensorMap tin,
               const __grid_constant__ CUtensorMap tout) {
  using namespace col;
  typedef Shape<T, L> Sh;
  typedef typename Vec<T>::t V;
  constexpr int W = Sh::W, NT = Sh::NT, NP = Sh::NP, TB = Sh::TB, BR = Sh::BR, NBOX = Sh::NBOX;
  constexpr int NB0 = L / radix_of(L, 0);  // first pass: radix 16, one butterfly per thread
  constexpr int NBL = L / radix_of(L, NP - 1), QL = radix_of(L, NP - 1) == 16 ? 1 : 16 / radix_of(L, NP - 1);
  constexpr int RL = radix_of(L, NP - 1);
  constexpr int XS = esz<T>() / 8;  // tensor-map elements (8 bytes) per complex element
  static_assert(radix_of(L, 0) == 16, "first pass radix 16");
  extern __shared__ __align__(1024) unsigned char smem[];
  const int S = a.stages;
  V* const work = reinterpret_cast<V*>(smem + (size_t)S * TB);
  uint64_t* const bars = reinterpret_cast<uint64_t*>(smem + (size_t)S * TB + Sh::WORK);
  const V* tw = (const V*)a.tw;
  const T sc = (T)a.scale;
  const bool conj = a.conj != 0;
  const long long G = gridDim.x;
  const long long stride = a.stride;  // N / L: units per transform
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
    const long long u0 = tile * W;
    const long long t = u0 / stride;
    const int x = (int)((u0 - t * stride) * XS);
    const int y = (int)(t * L);
    const uint32_t bar = fast::saddr(&bars[s]);
    fast::mbar_expect_tx(bar, (uint32_t)TB);
#pragma unroll 1
    for (int k = 0; k < NBOX; ++k)
      tma_load_2d(fast::saddr(smem + (size_t)s * TB + (size_t)k * BR * W * esz<T>()), &tin, x, y + k * BR, bar);
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
    const long long u0 = tile * W;
    const long long t = u0 / stride;
    const long long b0 = u0 - t * stride;

    // first in-block pass, lane-fastest: lane = tid % W, j = tid / W
    {
      const V* st = reinterpret_cast<const V*>(smem + (size_t)s * TB);
      const int lane = threadIdx.x % W, j = threadIdx.x / W;
#pragma unroll
      for (int r = 0; r < 16; ++r) v[r] = st[(j + r * NB0) * W + lane];
      if (conj)
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = cconj(v[r]);
      if (kfac != 0u && !a.notw) {
        const unsigned k = (unsigned)((b0 + lane) % gNs);
        const unsigned kstep = k * kfac;
        if (kstep) {
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
    if constexpr (NP == 1) {
      static_assert(NP > 1, "column tiles have two or more in-block passes");
    } else {
      wr<T, L, 0, true>(v, work);
      __syncthreads();
      middle<T, L, 1>(v, work, tw, a.pass);
      if (gNs == 1) {
        // first global pass: unit-major, each lane's L outputs contiguous
        rd<T, L, NP - 1, false>(v, work);
        cp<T, L, NP - 1, false>(v, tw, a.pass[NP - 1].tw);
        V* o = (V*)a.out + t * a.N + b0 * L;
#pragma unroll
        for (int q = 0; q < QL; ++q) {
          const int lane = lane_of<W, NBL, NT, false>(q), j = j_of<W, NBL, NT, false>(q);
          V* d = o + lane * L + j;
#pragma unroll
          for (int r = 0; r < RL; ++r) {
            V x = v[q * RL + r];
            if (conj) x = cconj(x);
            d[r * NBL] = cscale(x, sc);
          }
        }
      } else {
        // later global passes: lane-fastest, dense [L][W] in the work buffer, tensor stores
        rd<T, L, NP - 1, true>(v, work);
        cp<T, L, NP - 1, true>(v, tw, a.pass[NP - 1].tw);
        __syncthreads();
#pragma unroll
        for (int q = 0; q < QL; ++q) {
          const int lane = lane_of<W, NBL, NT, true>(q), j = j_of<W, NBL, NT, true>(q);
#pragma unroll
          for (int r = 0; r < RL; ++r) {
            V x = v[q * RL + r];
            if (conj) x = cconj(x);
            work[(j + r * NBL) * W + lane] = cscale(x, sc);
          }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (threadIdx.x == 0) {
          const long long k0 = b0 % gNs;
          const long long row0 = t * (a.N / gNs) + (b0 / gNs) * L;
#pragma unroll 1
          for (int k = 0; k < NBOX; ++k)
            tma_store_2d(&tout, (int)(k0 * XS), (int)(row0 + k * BR),
                         fast::saddr(smem + (size_t)S * TB + (size_t)k * BR * W * esz<T>()));
          asm volatile("cp.async.bulk.commit_group;" ::: "memory");
        }
      }
    }
  }
  if (threadIdx.x == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

}  // namespace gfft

namespace {

typedef CUresult (*EncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiled g_encode = nullptr;
std::mutex g_encode_mu;

int get_encoder() {
  std::lock_guard<std::mutex> lk(g_encode_mu);
  if (g_encode) return 0;
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn)
    return 1;
  g_encode = (EncodeTiled)fn;
  return 0;
}

// rows x cols matrix of elements of `esz` bytes at `base` (row pitch = cols), boxes of w x br elements
int encode(CUtensorMap* m, const void* base, long long rows, long long cols, int esz, int w, int br) {
  const int xs = esz / 8;
  cuuint64_t dims[2] = {(cuuint64_t)(cols * xs), (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(cols * esz)};
  cuuint32_t box[2] = {(cuuint32_t)(w * xs), (cuuint32_t)br};
  cuuint32_t es[2] = {1, 1};
  return g_encode(m, CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, const_cast<void*>(base), dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS
             ? 0
             : 1;
}

template <typename T>
const void* col_fn(int L) {
  switch (L) {
    case 64: return (const void*)gfft::col_kernel<T, 64>;
    case 128: return (const void*)gfft::col_kernel<T, 128>;
    case 256: return (const void*)gfft::col_kernel<T, 256>;
    case 512: return (const void*)gfft::col_kernel<T, 512>;
    case 1024: return (const void*)gfft::col_kernel<T, 1024>;
    case 2048: return (const void*)gfft::col_kernel<T, 2048>;
    case 4096: return sizeof(T) == 4 ? (const void*)gfft::col_kernel<float, 4096> : nullptr;
    default: return nullptr;
  }
}
template <typename T>
void col_shape(int L, int* W, int* NT, int* work) {
  switch (L) {
#define GFFT_COL_SHAPE(LL)                                \
  case LL:                                                \
    *W = gfft::col::Shape<T, LL>::W;                      \
    *NT = gfft::col::Shape<T, LL>::NT;                    \
    *work = gfft::col::Shape<T, LL>::WORK;                \
    return;
    GFFT_COL_SHAPE(64)
    GFFT_COL_SHAPE(128)
    GFFT_COL_SHAPE(256)
    GFFT_COL_SHAPE(512)
    GFFT_COL_SHAPE(1024)
    GFFT_COL_SHAPE(2048)
    GFFT_COL_SHAPE(4096)
#undef GFFT_COL_SHAPE
    default: *W = *NT = *work = 0;
  }
}

}  // namespace

// Shape of the variant-9 pass of length L: units per tile, threads, and the
// shared memory of `stages` stages (0 if L has no such kernel).
extern "C" int gfft_col_shape(int dbl, int L, int stages, int* units, int* threads, size_t* smem) {
  int W = 0, NT = 0, work = 0;
  if (dbl) {
    if (L > 2048) return 1;
    col_shape<double>(L, &W, &NT, &work);
  } else {
    col_shape<float>(L, &W, &NT, &work);
  }
  if (!W) return 1;
  const size_t tb = (size_t)W * L * (dbl ? 16 : 8);
  *units = W;
  *threads = NT;
  *smem = (size_t)stages * tb + (size_t)work + 8 * (size_t)stages;
  return 0;
}

extern "C" int gfft_col_setup(int dbl, size_t max_smem) {
  if (get_encoder() != 0) return 1;
  int e = 0;
  for (int L : {64, 128, 256, 512, 1024, 2048, 4096}) {
    const void* f = dbl ? col_fn<double>(L) : col_fn<float>(L);
    if (f) e |= cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem) != cudaSuccess;
  }
  return e;
}

extern "C" int gfft_col_occupancy(int dbl, int L, int threads, size_t smem) {
  const void* f = dbl ? col_fn<double>(L) : col_fn<float>(L);
  if (!f) return 0;
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f, threads, smem);
  return n;
}

// One global pass: tensor maps of this launch's input and output, then the
// launch.  Requirements (checked by the planner): N a power of two, the
// units per tile dividing N / L and Ns, 16-byte aligned buffers.
extern "C" int gfft_col_launch(int dbl, const EngineArgs* a, unsigned grid, unsigned threads, size_t smem,
                               cudaStream_t stream) {
  const void* f = dbl ? col_fn<double>(a->L) : col_fn<float>(a->L);
  if (!f || !g_encode) return (int)cudaErrorInvalidValue;
  int W = 0, NT = 0, work = 0;
  if (dbl)
    col_shape<double>(a->L, &W, &NT, &work);
  else
    col_shape<float>(a->L, &W, &NT, &work);
  const int esz = dbl ? 16 : 8;
  const long long batch = a->nunits / a->stride;
  const int br = a->L < 256 ? a->L : 256;
  if ((((uintptr_t)a->in) | ((uintptr_t)a->out)) & 15) return (int)cudaErrorInvalidValue;
  if (a->stride % W || (a->gNs > 1 && a->gNs % W)) return (int)cudaErrorInvalidValue;
  CUtensorMap tin, tout;
  if (encode(&tin, a->in, batch * a->L, a->stride, esz, W, br) != 0) return (int)cudaErrorInvalidValue;
  if (a->gNs > 1) {
    if (encode(&tout, a->out, batch * (a->N / a->gNs), a->gNs, esz, W, br) != 0) return (int)cudaErrorInvalidValue;
  } else {
    tout = tin;  // unused: the first pass stores from registers
  }
  cudaGetLastError();  // clear a stale error of an earlier, unrelated call
  void* args[] = {(void*)a, (void*)&tin, (void*)&tout};
  return (int)cudaLaunchKernel(f, dim3(grid), dim3(threads), args, smem, stream);
}
