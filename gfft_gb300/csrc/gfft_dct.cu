// Cosine transforms (transform IDs 4-7): the reference declares DCT1 /
// IDCT1 / DCT2 / IDCT2 (src/gfftpolicy.h:302-365) with empty algorithms and
// defines them only by the direct sums of its test harness
// (src/direct.h:270-312):
//
//   DCT1: X_k = sum_{l<N} x_l cos(pi k l / (N - 1)),  N >= 2
//   DCT2: X_k = sum_{l<N} x_l cos(pi k l / N)
//
// and the inverse tags run the same sums under the Backward policy, which
// divides by N (src/gfftswap.h:355-361).  Both sums are real parts of one
// real DFT, so a cosine transform here is a pre pass, the library's real
// transform (out of place, any length) and a post pass:
//
//   DCT2: y = x padded with N zeros (2N reals); X_k = Re Y_k, k < N.
//   DCT1: M = N - 1, y = the even extension x_0 .. x_M, x_{M-1} .. x_1 (2M
//         reals); Re Y_k = x_0 + (-1)^k x_M + 2 sum_{0<l<M} x_l cos(pi k l/M),
//         so X_k = (Re Y_k + x_0 + (-1)^k x_M) / 2.
//
// The real transform writes Y packed as Y_0, Y_M, Y_1 .. Y_{M-1} (complex);
// the post pass reads Re Y_0 at 0, Re Y_M at 1, Re Y_k at 2k.  Both passes
// are grid-stride loops, coalesced in the output index.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>

#include "../../include/gfft_gb300.h"
#include "handle.h"

namespace {

template <typename T>
__global__ void dct_pre(int type, long long N, long long M, long long batch, const T* __restrict__ in,
                        T* __restrict__ ws) {
  const long long P = 2 * M;
  const long long total = batch * P;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long b = i / P, j = i - b * P;
    T v;
    if (type == 2) v = j < N ? in[b * N + j] : (T)0;
    else v = in[b * N + (j <= M ? j : P - j)];
    ws[i] = v;
  }
}

template <typename T>
__global__ void dct_post(int type, long long N, long long M, long long batch, const T* __restrict__ ext,
                         const T* __restrict__ spec, T* __restrict__ out, T scale) {
  const long long total = batch * N;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long b = i / N, k = i - b * N;
    const T* y = spec + b * 2 * M;
    const T re = k == 0 ? y[0] : (k == M ? y[1] : y[2 * k]);
    T v;
    if (type == 2) {
      v = re;
    } else {
      const T x0 = ext[b * 2 * M], xm = ext[b * 2 * M + M];
      v = (T)0.5 * (re + x0 + ((k & 1) ? -xm : xm));
    }
    out[i] = v * scale;
  }
}

unsigned grid_for(long long total) {
  long long g = (total + 255) / 256;
  return (unsigned)std::max<long long>(1, std::min<long long>(g, 152LL * 16));
}

}  // namespace

extern "C" {

int gfft_dct_create(gfft_plan** handle, uint64_t n, int vtype_id, int trans_id, int parall_id, int place_id,
                    uint64_t batch) {
  if (vtype_id != 0 && vtype_id != 1) return GFFT_E_INVALID_TYPE;  // real value types only
  const int type = (trans_id == 4 || trans_id == 5) ? 1 : 2;
  if (type == 1 && n < 2) return GFFT_E_INVALID_SIZE;
  const long long M = type == 1 ? (long long)n - 1 : (long long)n;
  gfft_plan* inner = nullptr;
  int st = gfft_create(&inner, (uint64_t)M, vtype_id, 2 /* RDFT */, 1, parall_id, 1 /* out of place */, batch);
  if (st != GFFT_OK) return st;
  gfft_plan* h = new (std::nothrow) gfft_plan();
  if (!h) {
    gfft_destroy(inner);
    return GFFT_E_ALLOC;
  }
  const int dbl = vtype_id == 0;
  h->hp.n = (long long)n;
  h->hp.batch = (long long)batch;
  h->hp.dbl = dbl;
  h->hp.trans = trans_id;
  h->hp.place = place_id;
  h->vtype = vtype_id;
  h->trans_id = trans_id;
  h->place_id = place_id;
  h->parall_id = parall_id;
  h->device = inner->device;
  h->dct_inner = inner;
  h->dct_type = type;
  h->dct_m = M;
  h->dct_bytes = (size_t)(2 * M) * (size_t)batch * (dbl ? 8 : 4);
  for (int i = 0; i < 2; ++i)
    if (cudaMalloc(&h->d_dct[i], h->dct_bytes) != cudaSuccess) {
      h->d_dct[i] = nullptr;
      gfft_destroy(h);
      return GFFT_E_ALLOC;
    }
  *handle = h;
  return GFFT_OK;
}

int gfft_dct_exec(gfft_plan* h, const void* src, void* dst, cudaStream_t stream) {
  const long long N = h->hp.n, M = h->dct_m, B = h->hp.batch;
  const bool inverse = (h->trans_id == 5 || h->trans_id == 7);
  cudaGetLastError();  // clear a stale error of an earlier, unrelated call
  if (h->hp.dbl) {
    dct_pre<double><<<grid_for(B * 2 * M), 256, 0, stream>>>(h->dct_type, N, M, B, (const double*)src,
                                                               (double*)h->d_dct[0]);
  } else {
    dct_pre<float><<<grid_for(B * 2 * M), 256, 0, stream>>>(h->dct_type, N, M, B, (const float*)src,
                                                              (float*)h->d_dct[0]);
  }
  if (cudaGetLastError() != cudaSuccess) return GFFT_E_CUDA;
  gfft_plan* in = h->dct_inner;
  int st = gfft_exec_ws(in, h->d_dct[0], h->d_dct[1], stream, in->d_ws[0], in->d_ws[1]);
  if (st != GFFT_OK) return st;
  if (h->hp.dbl) {
    dct_post<double><<<grid_for(B * N), 256, 0, stream>>>(h->dct_type, N, M, B, (const double*)h->d_dct[0],
                                                           (const double*)h->d_dct[1], (double*)dst,
                                                           inverse ? 1.0 / (double)N : 1.0);
  } else {
    dct_post<float><<<grid_for(B * N), 256, 0, stream>>>(h->dct_type, N, M, B, (const float*)h->d_dct[0],
                                                          (const float*)h->d_dct[1], (float*)dst,
                                                          inverse ? 1.0f / (float)N : 1.0f);
  }
  return cudaGetLastError() == cudaSuccess ? GFFT_OK : GFFT_E_CUDA;
}

}  // extern "C"
