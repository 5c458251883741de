// Multi-dimensional complex transforms (no reference counterpart: the
// reference carries a `Dim` parameter, src/gfftgen.h:49, 153-154, 200, but
// only Dim = 1 exists).
//
// An array of dims n_0 x ... x n_{r-1} (row-major, the last index fastest)
// is transformed axis by axis:
//   - the innermost axis is a batch of contiguous 1-D transforms (the whole
//     1-D machinery: any supported length);
//   - axis d < r-1, with inner stride s_d = n_{d+1} ... n_{r-1}, is a column
//     pass: every (outer block t, column b < s_d) holds the n_d samples
//     t n_d s_d + b + j s_d.  That is the last global pass of a 1-D four-step
//     transform of length n_d s_d without its inter-pass twiddle, so the
//     column-tile kernels run it (EngineArgs::notw = 1): tiles of W adjacent
//     columns, the next tile gathered while the current one is transformed,
//     output written back to the same columns (in place on the output).
// n_d of an outer axis is at most one tile (4096 FP32 / 2048 FP64 points).
// The inverse conjugates on load and store of every pass and divides by n_d
// in each axis, 1 / (n_0 ... n_{r-1}) in all.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/gfft_gb300.h"
#include "handle.h"

extern "C" int gfft_lane_occupancy(int dbl, int threads, size_t smem);
extern "C" int gfft_lane_launch(int dbl, const EngineArgs* a, unsigned grid, unsigned threads, size_t smem,
                                cudaStream_t stream);
extern "C" int gfft_lanep2_occupancy(int dbl, int L, int threads, size_t smem);
extern "C" int gfft_lanep2_launch(int dbl, const EngineArgs* a, unsigned grid, unsigned threads, size_t smem,
                                  cudaStream_t stream);

namespace {

long long padded(long long L, int dbl) { return L + (L >> (dbl ? 3 : 4)) + 1; }

// the column pass of one outer axis: radices from the single-pass plan of
// n_d, launch shape for the column-tile kernels
int build_axis(gfft_plan* h, int k, long long L, long long s, long long total, int dbl, int trans) {
  HostPlan hp;
  PlanOpts po;
  if (gfft_plan_build(hp, L, 1, dbl, trans, 1, po) != 0 || hp.nglobal != 1) return GFFT_E_INVALID_SIZE;
  GlobalPass gp = hp.gp[0];
  const long long TILE = dbl ? 2048 : 4096;
  const int esz = dbl ? 16 : 8;
  gp.mode = 1;
  gp.Ns = s;
  const bool pow2 = (L & (L - 1)) == 0;
  if (pow2 && L >= 64 && L <= 1024 && spec_radices(gp) && s % (TILE / L) == 0) {
    gp.variant = 5;
    gp.units = (int)(TILE / L);
    gp.threads = (int)(TILE / 16);
    gp.smem = (size_t)(2 * gp.units * padded(L, dbl) * esz);
  } else {
    long long W = 1;
    while (2 * W * L <= TILE && 2 * W <= s && 2 * W <= 8) W *= 2;
    gp.variant = 4;
    gp.units = (int)W;
    gp.threads = dbl ? 256 : 512;
    gp.smem = (size_t)(3 * W * engine_padded(L, dbl) * esz);
  }
  const long long nunits = total / L;
  gp.ntiles = (nunits + gp.units - 1) / gp.units;
  int maxopt = 0, nsm = 0;
  cudaDeviceGetAttribute(&maxopt, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, h->device);
  if (gp.smem > (size_t)maxopt) return GFFT_E_INVALID_SIZE;
  int per = gp.variant == 5 ? gfft_lanep2_occupancy(dbl, gp.L, gp.threads, gp.smem)
                            : gfft_lane_occupancy(dbl, gp.threads, gp.smem);
  if (per < 1) per = 1;
  h->nd_grid[k] = (unsigned)std::max<long long>(1, std::min<long long>((long long)nsm * per, gp.ntiles));
  h->nd_gp[k] = gp;
  h->nd_stride[k] = s;
  // in-block twiddles of the single-pass plan, rounded once
  const size_t cnt = std::max<size_t>(hp.table_count, 1);
  std::vector<double> tab(2 * cnt, 0.0);
  gfft_plan_tables(hp, tab.data());
  const size_t bytes = cnt * (size_t)esz;
  if (cudaMalloc(&h->nd_tab[k], bytes) != cudaSuccess) {
    h->nd_tab[k] = nullptr;
    return GFFT_E_ALLOC;
  }
  cudaError_t ce;
  if (dbl) {
    ce = cudaMemcpy(h->nd_tab[k], tab.data(), bytes, cudaMemcpyHostToDevice);
  } else {
    std::vector<float> f(tab.begin(), tab.end());
    ce = cudaMemcpy(h->nd_tab[k], f.data(), bytes, cudaMemcpyHostToDevice);
  }
  return ce == cudaSuccess ? GFFT_OK : GFFT_E_CUDA;
}

}  // namespace

extern "C" {

int gfft_create_nd(gfft_handle* handle, int rank, const uint64_t* dims, int vtype_id, int trans_id, int place_id,
                   uint64_t batch) {
  if (!handle || !dims) return GFFT_E_NULL_POINTER;
  *handle = nullptr;
  if (rank < 1 || rank > 3) return GFFT_E_INVALID_DIM;
  if (trans_id != 0 && trans_id != 1) return GFFT_E_INVALID_TRANSFORM;
  if (vtype_id < 0 || vtype_id > 3) return GFFT_E_INVALID_TYPE;
  if (place_id != 0 && place_id != 1) return GFFT_E_INVALID_PLACE;
  if (batch == 0) return GFFT_E_INVALID_SIZE;
  const int dbl = (vtype_id == 0 || vtype_id == 2) ? 1 : 0;
  long long total = (long long)batch;
  for (int d = 0; d < rank; ++d) {
    if (dims[d] == 0 || dims[d] > (1ULL << 30)) return GFFT_E_INVALID_SIZE;
    total *= (long long)dims[d];
    if (total > (1LL << 40)) return GFFT_E_INVALID_SIZE;
  }
  if (rank == 1)
    return gfft_create(handle, dims[0], vtype_id, trans_id, 1, 0, place_id, batch);
  const long long TILE = dbl ? 2048 : 4096;
  for (int d = 0; d < rank - 1; ++d)
    if ((long long)dims[d] > TILE) return GFFT_E_INVALID_SIZE;
  const long long inner_n = (long long)dims[rank - 1];
  gfft_plan* inner = nullptr;
  int st = gfft_create(&inner, (uint64_t)inner_n, vtype_id, trans_id, 1, 0, place_id,
                       (uint64_t)(total / inner_n));
  if (st != GFFT_OK) return st;
  gfft_plan* h = new (std::nothrow) gfft_plan();
  if (!h) {
    gfft_destroy(inner);
    return GFFT_E_ALLOC;
  }
  h->hp.n = total / (long long)batch;
  h->hp.batch = (long long)batch;
  h->hp.dbl = dbl;
  h->hp.trans = trans_id;
  h->hp.place = place_id;
  h->vtype = vtype_id;
  h->trans_id = trans_id;
  h->place_id = place_id;
  h->device = inner->device;
  h->nd_inner = inner;
  h->nd_rank = rank;
  for (int d = 0; d < rank; ++d) h->nd_dims[d] = (long long)dims[d];
  long long s = inner_n;
  for (int d = rank - 2; d >= 0; --d) {
    const long long L = (long long)dims[d];
    if (L > 1) {
      st = build_axis(h, d, L, s, total, dbl, trans_id);
      if (st != GFFT_OK) {
        gfft_destroy(h);
        return st;
      }
    }
    s *= L;
  }
  *handle = h;
  return GFFT_OK;
}

int gfft_nd_exec(gfft_plan* h, const void* src, void* dst, cudaStream_t stream) {
  gfft_plan* in = h->nd_inner;
  int st = gfft_exec_ws(in, src, dst, stream, in->d_ws[0], in->d_ws[1]);
  if (st != GFFT_OK) return st;
  const int dbl = h->hp.dbl;
  const bool inverse = h->trans_id == 1;
  long long total = h->hp.n * h->hp.batch;
  for (int d = h->nd_rank - 2; d >= 0; --d) {
    const GlobalPass& gp = h->nd_gp[d];
    const long long L = h->nd_dims[d];
    if (L <= 1) continue;
    EngineArgs a;
    std::memset(&a, 0, sizeof(a));
    a.in = dst;
    a.out = dst;
    a.L = (int)L;
    a.stride = h->nd_stride[d];
    a.N = L * a.stride;
    a.nunits = total / L;
    a.gNs = a.stride;
    a.gB = 1;
    a.tw = h->nd_tab[d];
    a.gtw_lo = h->nd_tab[d];
    a.gtw_hi = h->nd_tab[d];
    a.pad_shift = dbl ? 3 : 4;
    a.Lp = gp.variant == 4 ? (int)engine_padded(L, dbl) : (int)(L + (L >> a.pad_shift) + 1);
    a.W = gp.units;
    a.mode = 1;
    a.npass = gp.npass;
    for (int i = 0; i < gp.npass; ++i) {
      a.pass[i] = gp.pass[i];
      a.pass[i].fd_nb = make_fastdiv((unsigned)(L / gp.pass[i].R));
      a.pass[i].fd_ns = make_fastdiv((unsigned)gp.pass[i].Ns);
    }
    a.fd_L = make_fastdiv((unsigned)L);
    a.conj = inverse ? 1 : 0;
    a.scale = inverse ? 1.0 / (double)L : 1.0;
    a.status = in->d_status;
    a.ntiles = gp.ntiles;
    a.notw = 1;
    const int e = gp.variant == 5 ? gfft_lanep2_launch(dbl, &a, h->nd_grid[d], (unsigned)gp.threads, gp.smem, stream)
                                  : gfft_lane_launch(dbl, &a, h->nd_grid[d], (unsigned)gp.threads, gp.smem, stream);
    if (e != 0) return GFFT_E_CUDA;
  }
  return GFFT_OK;
}

}  // extern "C"
