// One transform per thread-block cluster (variant 8): N = C x M complex
// points, M = 4096 (FP32) / 2048 (FP64), C = 2, 4 or 8 CTAs per cluster.
//
// With n = m + M c (CTA c holds the contiguous chunk c) and k = c' + C k2,
//   X[c' + C k2] = sum_m W_M^{m k2} [ W_N^{m c'} sum_c x[m + M c] W_C^{c c'} ],
// so the transform needs one HBM round trip:
//   1. CTA c loads its chunk x[M c .. M c + M) (coalesced) into shared memory;
//   2. cluster barrier (the chunks are visible across the cluster);
//   3. CTA c' forms, for every m, the c'-th output of the length-C DFT across
//      the chunks (reads of the other CTAs' shared memory through the
//      distributed shared-memory window) times W_N^{m c'};
//   4. cluster barrier (no CTA leaves or reuses memory another still reads);
//   5. the length-M transform of step 3's sequence with the compile-time
//      passes of the specialised kernels (spec.cuh);
//   6. output k2 of CTA c' goes to X[c' + C k2].
// Every CTA runs exactly two cluster barriers; all global reads of a
// transform precede the first and all its writes follow the second, so the
// transform may run in place.  The inverse conjugates on load and store and
// scales by 1/N.
#include <cuda_runtime.h>
#include <stdint.h>

#include "butterflies.cuh"
#include "plan.h"
#include "spec.cuh"

namespace gfft {
namespace cluster {

__device__ __forceinline__ uint32_t rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
  asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ uint32_t remote(uint32_t saddr, uint32_t r) {
  uint32_t ra;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(saddr), "r"(r));
  return ra;
}
template <typename V> __device__ __forceinline__ V ld_remote(uint32_t ra);
template <> __device__ __forceinline__ float2 ld_remote<float2>(uint32_t ra) {
  float2 v;
  asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(ra) : "memory");
  return v;
}
template <> __device__ __forceinline__ double2 ld_remote<double2>(uint32_t ra) {
  double2 v;
  asm volatile("ld.shared::cluster.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "r"(ra) : "memory");
  return v;
}

}  // namespace cluster

template <typename T, int C>
__global__ void __launch_bounds__(spec::Cfg<T>::TILE / 16) cluster_kernel(const __grid_constant__ EngineArgs a) {
  using namespace spec;
  typedef typename Vec<T>::t V;
  constexpr int M = Cfg<T>::TILE, NT = M / 16, NP = npass_of(M);
  constexpr int R = radix_of(M, NP - 1), NB = M / R, Q = 16 / R;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* const raw = reinterpret_cast<V*>(smem_raw);  // this CTA's chunk, unpadded
  V* const work = raw + M;                       // padded [pad(m)] sequence of step 3
  const uint32_t c = cluster::rank();
  const long long t = blockIdx.x / C;
  const long long N = (long long)M * C;
  const V* in = (const V*)a.in + t * N + (long long)c * M;
  const V* wN = (const V*)a.gtw_lo;  // W_N^j, j < N
  const bool conj = a.conj != 0;
  // 1. the chunk, sixteen loads in flight per thread
  {
    V v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = in[threadIdx.x + q * NT];
#pragma unroll
    for (int q = 0; q < 16; ++q) raw[threadIdx.x + q * NT] = conj ? cconj(v[q]) : v[q];
  }
  cluster::cluster_sync();
  // 3. output c of the length-C DFT across the chunks, times W_N^{m c}
  {
    const uint32_t base = (uint32_t)__cvta_generic_to_shared(raw);
#pragma unroll 4
    for (int q = 0; q < 16; ++q) {
      const int m = threadIdx.x + q * NT;
      V acc = mk<V>(0, 0);
#pragma unroll
      for (int r = 0; r < C; ++r) {  // chunk r lives in the CTA of rank r
        const V x = (r == (int)c) ? raw[m]
                                  : cluster::ld_remote<V>(cluster::remote(base + (uint32_t)(m * sizeof(V)), r));
        const int e = ((r * (int)c) % C) * M;  // W_C^{r c} = W_N^{(r c mod C) M}
        acc = cadd(acc, e == 0 ? x : cmul(x, __ldg(wN + e)));
      }
      work[padi<T>(m)] = c == 0 ? acc : cmul(acc, __ldg(wN + m * (int)c));
    }
  }
  cluster::cluster_sync();  // also orders the work buffer for the passes
  // 5. the length-M transform
  V v[16];
  const V* tw = (const V*)a.tw;
  if constexpr (NP == 1) {
    sread<T, M, 0, false>(v, work);
    scompute<T, M, 0>(v, tw, a.pass[0].tw);
  } else {
    sread<T, M, 0, false>(v, work);
    scompute<T, M, 0>(v, tw, a.pass[0].tw);
    __syncthreads();
    swrite<T, M, 0>(v, work);
    __syncthreads();
    if constexpr (NP > 2) {
      sread<T, M, 1, false>(v, work);
      scompute<T, M, 1>(v, tw, a.pass[1].tw);
      __syncthreads();
      swrite<T, M, 1>(v, work);
      __syncthreads();
    }
    if constexpr (NP > 3) {
      sread<T, M, 2, false>(v, work);
      scompute<T, M, 2>(v, tw, a.pass[2].tw);
      __syncthreads();
      swrite<T, M, 2>(v, work);
      __syncthreads();
    }
    sread<T, M, NP - 1, false>(v, work);
    scompute<T, M, NP - 1>(v, tw, a.pass[NP - 1].tw);
  }
  // 6. output k2 = j + r NB of the last pass goes to X[c + C k2]
  V* out = (V*)a.out + t * N + c;
  const T sc = (T)a.scale;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int j = threadIdx.x + q * NT;  // one lane: b = j
#pragma unroll
    for (int r = 0; r < R; ++r) {
      V x = v[q * R + r];
      if (conj) x = cconj(x);
      out[(long long)(j + r * NB) * C] = cscale(x, sc);
    }
  }
}

}  // namespace gfft

namespace {
template <typename T>
const void* cluster_fn(int C) {
  switch (C) {
    case 2: return (const void*)gfft::cluster_kernel<T, 2>;
    case 4: return (const void*)gfft::cluster_kernel<T, 4>;
    case 8: return (const void*)gfft::cluster_kernel<T, 8>;
    default: return nullptr;
  }
}
}  // namespace

extern "C" int gfft_cluster_setup(int dbl, size_t max_smem) {
  int e = 0;
  for (int C : {2, 4, 8}) {
    const void* f = dbl ? cluster_fn<double>(C) : cluster_fn<float>(C);
    e |= cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem) != cudaSuccess;
  }
  return e;
}

extern "C" int gfft_cluster_launch(int dbl, const EngineArgs* a, int C, long long batch, unsigned threads, size_t smem,
                                   cudaStream_t stream) {
  const void* f = dbl ? cluster_fn<double>(C) : cluster_fn<float>(C);
  if (!f || batch * C > 0x7FFFFFFFLL) return (int)cudaErrorInvalidValue;
  cudaGetLastError();  // clear a stale error of an earlier, unrelated call
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(batch * C));
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  void* args[] = {(void*)a};
  return (int)cudaLaunchKernelExC(&cfg, f, args);
}
