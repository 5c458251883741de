// C ABI of the library (declared in include/gfft_gb300.h).
//
// A handle is the GPU counterpart of one reference transform object
// (GFFT::Transform<...>::Instance, src/gfftgen.h:46-87): it owns the plan,
// the device twiddle tables (the reference keeps "no additional data",
// release_notes.txt:55, and recomputes twiddles per call) and the workspace
// of a multi-pass transform.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>  // header-only: ranges cost a pointer test unless a profiler is attached

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/gfft_gb300.h"
#include "capi_host.h"
#include "dcheck.cuh"
#include "handle.h"
#include "plan.h"

extern "C" int gfft_engine_setup(int dbl, size_t max_smem);
extern "C" int gfft_engine_launch(int dbl, const EngineArgs* a, unsigned grid, unsigned threads, size_t smem,
                                  cudaStream_t stream);
extern "C" int gfft_fast_setup(int dbl, size_t max_smem);
extern "C" int gfft_fast_occupancy(int dbl, int threads, size_t smem);
extern "C" int gfft_fast_launch(int dbl, const EngineArgs* a, unsigned grid, unsigned threads, size_t smem,
                                cudaStream_t stream);
extern "C" int gfft_spec_setup(int dbl, size_t max_smem);
extern "C" int gfft_spec_occupancy(int dbl, int L, int stages, int threads, size_t smem);
extern "C" int gfft_spec_launch(int dbl, const EngineArgs* a, unsigned grid, unsigned threads, size_t smem,
                                cudaStream_t stream);
extern "C" int gfft_lane_setup(int dbl, size_t max_smem);
extern "C" int gfft_lane_occupancy(int dbl, int threads, size_t smem);
extern "C" int gfft_lane_launch(int dbl, const EngineArgs* a, unsigned grid, unsigned threads, size_t smem,
                                cudaStream_t stream);
extern "C" int gfft_lanep2_setup(int dbl, size_t max_smem);
extern "C" int gfft_lanep2_occupancy(int dbl, int L, int threads, size_t smem);
extern "C" int gfft_lanep2_launch(int dbl, const EngineArgs* a, unsigned grid, unsigned threads, size_t smem,
                                  cudaStream_t stream);
extern "C" int gfft_mixed_setup(int dbl, size_t max_smem);
extern "C" int gfft_mixed_occupancy(int dbl, const EngineArgs* a, int threads, size_t smem);
extern "C" int gfft_mixed_launch(int dbl, const EngineArgs* a, unsigned grid, unsigned threads, size_t smem,
                                 cudaStream_t stream);
extern "C" int gfft_tc_setup(size_t max_smem);
extern "C" int gfft_tc_occupancy(int L, int threads, size_t smem);
extern "C" int gfft_tc_launch(const EngineArgs* a, unsigned grid, unsigned threads, size_t smem, cudaStream_t stream);
extern "C" int gfft_col_setup(int dbl, size_t max_smem);
extern "C" int gfft_col_occupancy(int dbl, int L, int rf, int tk, int threads, size_t smem);
extern "C" int gfft_col_launch(int dbl, const EngineArgs* a, int tk, unsigned grid, unsigned threads, size_t smem,
                               cudaStream_t stream);
extern "C" int gfft_real_pass_launch(int dbl, void* data, long long n, long long batch, int dir, const void* rtw,
                                     cudaStream_t stream);
extern "C" int gfft_colmix_setup(int dbl, size_t max_smem);
extern "C" int gfft_colmix_occupancy(int dbl, const EngineArgs* a, int gather, int threads, size_t smem);
extern "C" int gfft_colmix_launch(int dbl, const EngineArgs* a, int gather, unsigned grid, unsigned threads,
                                  size_t smem, cudaStream_t stream);


namespace {

const unsigned kMagic = 0x6FF7B300u;

bool valid(gfft_handle h) { return h && h->magic == kMagic; }

int setup_device_once(int dbl) {
  static std::mutex mu;
  static bool done[2][64] = {{false}};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return GFFT_E_CUDA;
  std::lock_guard<std::mutex> lk(mu);
  if (dev < 64 && done[dbl][dev]) return GFFT_OK;
  int maxopt = 0;
  cudaDeviceGetAttribute(&maxopt, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (gfft_engine_setup(dbl, (size_t)maxopt) != 0) return GFFT_E_CUDA;
  if (gfft_fast_setup(dbl, (size_t)maxopt) != 0) return GFFT_E_CUDA;
  if (gfft_spec_setup(dbl, (size_t)maxopt) != 0) return GFFT_E_CUDA;
  if (gfft_lane_setup(dbl, (size_t)maxopt) != 0) return GFFT_E_CUDA;
  if (gfft_lanep2_setup(dbl, (size_t)maxopt) != 0) return GFFT_E_CUDA;
  if (!dbl && gfft_tc_setup((size_t)maxopt) != 0) return GFFT_E_CUDA;
  if (gfft_mixed_setup(dbl, (size_t)maxopt) != 0) return GFFT_E_CUDA;
  if (gfft_col_setup(dbl, (size_t)maxopt) != 0) return GFFT_E_CUDA;
  if (gfft_colmix_setup(dbl, (size_t)maxopt) != 0) return GFFT_E_CUDA;
  if (dev < 64) done[dbl][dev] = true;
  return GFFT_OK;
}

size_t elem_bytes(int dbl) { return dbl ? 16 : 8; }

// occupancy of the compile-time mixed-radix kernel of a pass (selected by
// its length and radices)
int mixed_occupancy(int dbl, const GlobalPass& gp) {
  EngineArgs a;
  std::memset(&a, 0, sizeof(a));
  a.L = gp.L;
  a.npass = gp.npass;
  for (int i = 0; i < gp.npass; ++i) a.pass[i] = gp.pass[i];
  return gfft_mixed_occupancy(dbl, &a, gp.threads, gp.smem);
}

// occupancy of a tensor-copy pass (power-of-two length, or a mixed shape)
int col_occupancy(int dbl, const GlobalPass& gp) {
  if ((gp.L & (gp.L - 1)) == 0) return gfft_col_occupancy(dbl, gp.L, gp.rf, gp.tk, gp.threads, gp.smem);
  EngineArgs a;
  std::memset(&a, 0, sizeof(a));
  a.L = gp.L;
  a.npass = gp.npass;
  for (int i = 0; i < gp.npass; ++i) a.pass[i] = gp.pass[i];
  return gfft_colmix_occupancy(dbl, &a, gp.gather, gp.threads, gp.smem);
}

}  // namespace

extern "C" {

int gfft_create_opts(gfft_handle* handle, uint64_t n, int vtype_id, int trans_id, int dim, int parall_id,
                     int place_id, uint64_t batch, const gfft_plan_opts* opts) {
  if (!handle) return GFFT_E_NULL_POINTER;
  *handle = nullptr;
  if ((dim == 2 || dim == 3) && trans_id <= 1 && parall_id >= 0 && !opts) {  // an n^dim array
    const uint64_t dims[3] = {n, n, n};
    return gfft_create_nd(handle, dim, dims, vtype_id, trans_id, place_id, batch);
  }
  int st0 = gfft::capi::check_ids(n, vtype_id, trans_id, dim, parall_id, place_id, batch);
  if (st0 != GFFT_OK) return st0;
  if (trans_id >= 4) return gfft_dct_create(handle, n, vtype_id, trans_id, parall_id, place_id, batch);
  PlanOpts po;
  st0 = gfft::capi::parse_opts(opts, po);
  if (st0 != GFFT_OK) return st0;
  const int dbl = (vtype_id == 0 || vtype_id == 2) ? 1 : 0;
  gfft_plan* h = new (std::nothrow) gfft_plan();
  if (!h) return GFFT_E_ALLOC;
  if (gfft_plan_build(h->hp, (long long)n, (long long)batch, dbl, trans_id, place_id, po) != 0) {
    delete h;
    return GFFT_E_INVALID_SIZE;
  }
  h->vtype = vtype_id;
  h->trans_id = trans_id;
  h->place_id = place_id;
  h->parall_id = parall_id;
  h->popts = po;
  h->has_opts = opts != nullptr;
  h->owns_ws = true;
  int st = setup_device_once(dbl);
  if (st != GFFT_OK) {
    delete h;
    return st;
  }
  cudaGetDevice(&h->device);
  int maxopt = 0;
  cudaDeviceGetAttribute(&maxopt, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
  for (int g = 0; g < h->hp.nglobal; ++g)
    if (h->hp.gp[g].smem > (size_t)maxopt) {
      delete h;
      return GFFT_E_INVALID_SIZE;
    }
  // tables: generated in extended precision, rounded once to the working type
  const size_t cnt = std::max<size_t>(h->hp.table_count, 1);
  std::vector<double> tab(2 * cnt, 0.0);
  gfft_plan_tables(h->hp, tab.data());
  h->tab_bytes = cnt * elem_bytes(dbl);
  if (cudaMalloc(&h->d_tab, h->tab_bytes) != cudaSuccess) {
    delete h;
    return GFFT_E_ALLOC;
  }
  cudaError_t ce;
  if (dbl) {
    ce = cudaMemcpy(h->d_tab, tab.data(), h->tab_bytes, cudaMemcpyHostToDevice);
  } else {
    std::vector<float> f(2 * cnt);
    for (size_t i = 0; i < 2 * cnt; ++i) f[i] = (float)tab[i];
    ce = cudaMemcpy(h->d_tab, f.data(), h->tab_bytes, cudaMemcpyHostToDevice);
  }
  if (ce != cudaSuccess) {
    cudaFree(h->d_tab);
    delete h;
    return GFFT_E_CUDA;
  }
  if (cudaMalloc((void**)&h->d_status, 256) != cudaSuccess || cudaMemset(h->d_status, 0, 256) != cudaSuccess) {
    cudaFree(h->d_tab);
    delete h;
    return GFFT_E_ALLOC;
  }
  {
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, h->device);
    for (int g = 0; g < h->hp.nglobal; ++g) {
      const GlobalPass& gp = h->hp.gp[g];
      if (gp.variant < 2) continue;
      int per = (opts && opts->blocks_per_sm)
                    ? opts->blocks_per_sm
                    : (gp.variant == 3   ? gfft_spec_occupancy(dbl, gp.L, gp.stages, gp.threads, gp.smem)
                       : gp.variant == 4 ? gfft_lane_occupancy(dbl, gp.threads, gp.smem)
                       : gp.variant == 5 ? gfft_lanep2_occupancy(dbl, gp.L, gp.threads, gp.smem)
                       : gp.variant == 6 ? gfft_tc_occupancy(gp.L, gp.threads, gp.smem)
                       : gp.variant == 7 ? mixed_occupancy(dbl, gp)
                       : gp.variant == 9 ? col_occupancy(dbl, gp)
                                         : gfft_fast_occupancy(dbl, gp.threads, gp.smem));
      if (gp.variant == 6 && !(opts && opts->blocks_per_sm)) {
        // two blocks fit by registers (launch bound) and shared memory whenever
        // two footprints plus the per-block reservation fit one SM
        int smem_sm = 0;
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, h->device);
        if (2 * (gp.smem + 1024) <= (size_t)smem_sm) per = std::max(per, 2);
      }
      if (per < 1) per = 1;
      long long grid = (long long)nsm * per;
      if (grid > gp.ntiles) grid = gp.ntiles;
      h->grid[g] = (unsigned)std::max<long long>(grid, 1);
    }
  }
  if (h->hp.n_ws > 0) {
    h->ws_bytes = h->hp.ws_elems * elem_bytes(dbl);
    for (int i = 0; i < h->hp.n_ws; ++i)
      if (cudaMalloc(&h->d_ws[i], h->ws_bytes) != cudaSuccess) {
        for (int j = 0; j < i; ++j) cudaFree(h->d_ws[j]);
        cudaFree(h->d_tab);
        delete h;
        return GFFT_E_ALLOC;
      }
  }
  *handle = h;
  return GFFT_OK;
}

int gfft_create(gfft_handle* handle, uint64_t n, int vtype_id, int trans_id, int dim, int parall_id, int place_id,
                uint64_t batch) {
  return gfft_create_opts(handle, n, vtype_id, trans_id, dim, parall_id, place_id, batch, nullptr);
}

int gfft_destroy(gfft_handle h) {
  if (!valid(h)) return GFFT_E_INVALID_HANDLE;
  h->magic = 0;
  if (h->unaligned) gfft_destroy(h->unaligned);
  if (h->dct_inner) gfft_destroy(h->dct_inner);
  if (h->nd_inner) gfft_destroy(h->nd_inner);
  for (int i = 0; i < 2; ++i)
    if (h->nd_tab[i]) cudaFree(h->nd_tab[i]);
  for (int i = 0; i < 2; ++i)
    if (h->d_dct[i]) cudaFree(h->d_dct[i]);
  cudaFree(h->d_tab);
  for (int i = 0; i < 2; ++i)
    if (h->d_ws[i]) cudaFree(h->d_ws[i]);
  if (h->d_stage) cudaFree(h->d_stage);
  if (h->d_status) cudaFree(h->d_status);
  for (int i = 0; i < 2; ++i)
    if (h->chunk_plan[i]) gfft_destroy(h->chunk_plan[i]);
  for (int i = 0; i < 3; ++i)
    if (h->hstream[i]) cudaStreamDestroy(h->hstream[i]);
  for (int i = 0; i < GFFT_MAX_CHUNKS; ++i) {
    if (h->ev_in[i]) cudaEventDestroy(h->ev_in[i]);
    if (h->ev_done[i]) cudaEventDestroy(h->ev_done[i]);
  }
  if (h->ev_user) cudaEventDestroy(h->ev_user);
  if (h->ev_end) cudaEventDestroy(h->ev_end);
  delete h;
  return GFFT_OK;
}

int gfft_get_info(gfft_handle h, gfft_plan_info* info) {
  if (!valid(h)) return GFFT_E_INVALID_HANDLE;
  if (!info) return GFFT_E_NULL_POINTER;
  if (h->nd_inner) {  // the innermost axis's plan plus one column pass per outer axis
    int st = gfft_get_info(h->nd_inner, info);
    if (st != GFFT_OK) return st;
    info->n = (uint64_t)h->hp.n;
    info->batch = (uint64_t)h->hp.batch;
    for (int d = 0; d < h->nd_rank - 1; ++d)
      if (h->nd_dims[d] > 1) ++info->kernels_per_exec;
    return GFFT_OK;
  }
  if (h->dct_inner) {  // the inner real transform's plan, under this handle's identity
    int st = gfft_get_info(h->dct_inner, info);
    if (st != GFFT_OK) return st;
    info->n = (uint64_t)h->hp.n;
    info->trans_id = h->trans_id;
    info->place_id = h->place_id;
    info->workspace_bytes += 2 * (uint64_t)h->dct_bytes;
    info->kernels_per_exec += 2;
    return GFFT_OK;
  }
  gfft::capi::fill_info(h->hp, h->vtype, h->tab_bytes, h->ws_bytes, info);
  return GFFT_OK;
}


namespace {
// an NVTX range around the launch of one global pass (closed on scope exit)
struct NvtxPass {
  NvtxPass(int g, int L, int variant) {
    char name[64];
    std::snprintf(name, sizeof(name), "gfft pass %d L=%d variant %d", g, L, variant);
    nvtxRangePushA(name);
  }
  ~NvtxPass() { nvtxRangePop(); }
};
}  // namespace

// shared by gfft_exec and the scratch-free entry point: runs the plan with
// the given workspace buffers
int gfft_exec_ws(gfft_handle h, const void* src, void* dst, cudaStream_t stream, void* ws0, void* ws1) {
  const HostPlan& p = h->hp;
  const int dbl = p.dbl;
  const size_t esz = elem_bytes(dbl);
  const char* tab = (const char*)h->d_tab;
  const bool inverse = (p.trans == 1 || p.trans == 3);
  const long long n = p.n, batch = p.batch;
  const void* cur_in = src;
  // real inverse with several passes: unfused pre pass in place on dst
  if (p.trans == 3 && !p.real_fused) {
    if (dst != src) {
      if (cudaMemcpyAsync(dst, src, (size_t)n * batch * esz, cudaMemcpyDeviceToDevice, stream) != cudaSuccess)
        return GFFT_E_CUDA;
    }
    if (gfft_real_pass_launch(dbl, dst, n, batch, 2, tab + p.rtw_off * esz, stream) != 0) return GFFT_E_CUDA;
    cur_in = dst;
  }
  // buffer sequence of the global passes (fixed arrays: the allocation-free
  // entry point runs through here too)
  const void* ins[GFFT_MAXG] = {};
  void* outs[GFFT_MAXG] = {};
  if (p.nglobal < 1 || p.nglobal > GFFT_MAXG) return GFFT_E_INVALID_PLAN;
  const bool inplace = (cur_in == dst);
  if (p.nglobal == 1) {
    ins[0] = cur_in;
    outs[0] = dst;
  } else if (p.nglobal % 2 == 0) {
    // in -> ws -> dst -> ws -> dst
    const void* a = cur_in;
    for (int g = 0; g < p.nglobal; ++g) {
      ins[g] = a;
      outs[g] = (g % 2 == 0) ? ws0 : dst;
      a = outs[g];
    }
  } else if (!inplace) {
    // in -> dst -> ws -> dst (-> ws -> dst)
    const void* a = cur_in;
    for (int g = 0; g < p.nglobal; ++g) {
      ins[g] = a;
      outs[g] = (g % 2 == 0) ? dst : ws0;
      a = outs[g];
    }
  } else {
    // in place, odd: in -> ws0 -> ws1 -> dst (the second buffer of an
    // out-of-place plan called in place is allocated on first need, only for
    // handles from gfft_create: any other caller gets GFFT_E_INVALID_PLAN)
    if (!ws1 && h->owns_ws && ws0 == h->d_ws[0]) {
      if (cudaMalloc(&h->d_ws[1], h->ws_bytes) != cudaSuccess) {
        h->d_ws[1] = nullptr;
        return GFFT_E_ALLOC;
      }
      ws1 = h->d_ws[1];
    }
    if (!ws1) return GFFT_E_INVALID_PLAN;
    ins[0] = cur_in;
    outs[0] = ws0;
    ins[1] = ws0;
    outs[1] = ws1;
    ins[2] = ws1;
    outs[2] = dst;
  }
  // step `step` runs global pass `step` (time decimation) or
  // nglobal - 1 - step (frequency decimation: the transposed passes, last
  // to first)
  for (int step = 0; step < p.nglobal; ++step) {
    const int g = p.dif ? p.nglobal - 1 - step : step;
    const GlobalPass& gp = p.gp[g];
    // one NVTX range per global pass, named by its length and kernel variant
    NvtxPass nvtx(g, gp.L, gp.variant);
    EngineArgs a;
    std::memset(&a, 0, sizeof(a));
    a.in = ins[step];
    a.out = outs[step];
    a.dif = p.dif;
    a.N = n;
    a.L = gp.L;
    a.stride = n / gp.L;
    a.nunits = batch * a.stride;
    a.gNs = gp.Ns;
    a.gB = (long long)p.gtw_B;
    a.gtw_lo = tab + p.gtw_lo_off * esz;
    a.gtw_hi = tab + p.gtw_hi_off * esz;
    a.tw = tab;
    a.rtw = tab + p.rtw_off * esz;
    a.pad_shift = dbl ? 3 : 4;
    // the run-time engine kernels (variants 1, 4) pad with engine_padded; the
    // others keep one slot per 2^pad_shift values
    a.Lp = (gp.variant == 1 || gp.variant == 4) ? (int)engine_padded(gp.L, dbl)
                                                : gp.L + (gp.L >> a.pad_shift) + 1;
    a.W = gp.units;
    a.mode = gp.mode;
    a.npass = gp.npass;
    for (int i = 0; i < gp.npass; ++i) {
      a.pass[i] = gp.pass[i];
      a.pass[i].fd_nb = make_fastdiv((unsigned)(gp.L / gp.pass[i].R));
      a.pass[i].fd_ns = make_fastdiv((unsigned)gp.pass[i].Ns);
    }
    a.fd_L = make_fastdiv((unsigned)gp.L);
    a.fd_half = make_fastdiv((unsigned)(gp.L / 2 + 1));
    const bool last = (step == p.nglobal - 1);
    a.real = p.real_fused ? ((p.trans == 2) ? 1 : 2) : 0;
    // The inverse runs as conj(FFT(conj x)) / N.  Every pass conjugates on
    // load and on store: the pairs cancel between passes, so the inter-pass
    // twiddles see forward-domain data.  The fused real inverse pre pass
    // conjugates inside its own load.
    a.conj = inverse ? 1 : 0;
    a.scale = (inverse && last) ? 1.0 / (double)n : 1.0;
    a.status = h->d_status;
    if (gp.variant == 6) {
      a.ntiles = gp.ntiles;
      a.spin_limit = 1LL << 26;
      if (gfft_tc_launch(&a, h->grid[g], (unsigned)gp.threads, gp.smem, stream) != 0) return GFFT_E_CUDA;
      continue;
    }
    if (gp.variant == 9) {
      a.real = gp.rf;
      a.ftw = p.ftw_off[g] ? (const void*)(tab + p.ftw_off[g] * esz) : nullptr;
      a.ntiles = gp.ntiles;
      a.stages = gp.stages;
      a.spin_limit = 1LL << 26;
      const int e = (gp.L & (gp.L - 1)) == 0
                        ? gfft_col_launch(dbl, &a, gp.tk, h->grid[g], (unsigned)gp.threads, gp.smem, stream)
                        : gfft_colmix_launch(dbl, &a, gp.gather, h->grid[g], (unsigned)gp.threads, gp.smem, stream);
      if (e != 0) return GFFT_E_CUDA;
      continue;
    }
    if (gp.variant == 7) {
      a.ntiles = gp.ntiles;
      if (gfft_mixed_launch(dbl, &a, h->grid[g], (unsigned)gp.threads, gp.smem, stream) != 0) return GFFT_E_CUDA;
      continue;
    }
    if (gp.variant == 4 || gp.variant == 5) {
      a.ntiles = gp.ntiles;
      const int e = gp.variant == 4 ? gfft_lane_launch(dbl, &a, h->grid[g], (unsigned)gp.threads, gp.smem, stream)
                                    : gfft_lanep2_launch(dbl, &a, h->grid[g], (unsigned)gp.threads, gp.smem, stream);
      if (e != 0) return GFFT_E_CUDA;
      continue;
    }
    if (gp.variant >= 2) {
      a.ntiles = gp.ntiles;
      a.stages = gp.stages;
      a.tile_bytes = gp.tile_bytes;
      a.spin_limit = 1LL << 26;
      a.debug_no_issue = 0;
      const int e = gp.variant == 3 ? gfft_spec_launch(dbl, &a, h->grid[g], (unsigned)gp.threads, gp.smem, stream)
                                    : gfft_fast_launch(dbl, &a, h->grid[g], (unsigned)gp.threads, gp.smem, stream);
      if (e != 0) return GFFT_E_CUDA;
      continue;
    }
    long long grid = (a.nunits + a.W - 1) / a.W;
    if (grid > 0x7FFFFFFFLL) return GFFT_E_INVALID_SIZE;
    if (gfft_engine_launch(dbl, &a, (unsigned)grid, (unsigned)gp.threads, gp.smem, stream) != 0)
      return GFFT_E_CUDA;
  }
  if (p.trans == 2 && !p.real_fused) {
    if (gfft_real_pass_launch(dbl, dst, n, batch, 1, tab + p.rtw_off * esz, stream) != 0) return GFFT_E_CUDA;
  }
  return GFFT_OK;
}

int gfft_get_device_status(gfft_handle h, int* status) {
  if (!valid(h)) return GFFT_E_INVALID_HANDLE;
  if (!status) return GFFT_E_NULL_POINTER;
  if (h->dct_inner) return gfft_get_device_status(h->dct_inner, status);
  if (h->nd_inner) return gfft_get_device_status(h->nd_inner, status);
  if (cudaDeviceSynchronize() != cudaSuccess) return GFFT_E_CUDA;
  if (cudaMemcpy(status, h->d_status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return GFFT_E_CUDA;
  if (cudaMemset(h->d_status, 0, sizeof(int)) != cudaSuccess) return GFFT_E_CUDA;
  return GFFT_OK;
}

int gfft_selftest_bounded_wait(long long spin_limit, int* status) {
  if (!status) return GFFT_E_NULL_POINTER;
  if (spin_limit < 1) return GFFT_E_INVALID_PLAN;
  gfft_handle h = nullptr;
  gfft_plan_opts o;
  std::memset(&o, 0, sizeof(o));
  o.kernel_variant = 2;
  int st = gfft_create_opts(&h, 4096, 1, 0, 1, 0, 1, 64, &o);
  if (st != GFFT_OK) return st;
  const GlobalPass& gp = h->hp.gp[0];
  if (gp.variant != 2) {
    gfft_destroy(h);
    return GFFT_E_INVALID_PLAN;
  }
  void* buf = nullptr;
  const size_t bytes = (size_t)4096 * 64 * 8;
  if (cudaMalloc(&buf, 2 * bytes) != cudaSuccess) {
    gfft_destroy(h);
    return GFFT_E_ALLOC;
  }
  EngineArgs a;
  std::memset(&a, 0, sizeof(a));
  a.in = buf;
  a.out = (char*)buf + bytes;
  a.N = 4096;
  a.L = 4096;
  a.stride = 1;
  a.nunits = 64;
  a.gNs = 1;
  a.tw = h->d_tab;
  a.pad_shift = 4;
  a.Lp = 4096 + 256 + 1;
  a.W = gp.units;
  a.mode = 0;
  a.npass = gp.npass;
  for (int i = 0; i < gp.npass; ++i) a.pass[i] = gp.pass[i];
  a.scale = 1.0;
  a.status = h->d_status;
  a.ntiles = gp.ntiles;
  a.stages = gp.stages;
  a.tile_bytes = gp.tile_bytes;
  a.spin_limit = spin_limit;
  a.debug_no_issue = 1;  // nothing ever arrives on the barriers
  st = gfft_fast_launch(h->hp.dbl, &a, 4, (unsigned)gp.threads, gp.smem, 0) != 0 ? GFFT_E_CUDA : GFFT_OK;
  if (st == GFFT_OK) st = gfft_get_device_status(h, status);
  cudaFree(buf);
  gfft_destroy(h);
  return st;
}

#ifdef GFFT_DEBUG
}  // extern "C"
namespace {
// one check that fails, with no access behind it
__global__ void dcheck_selftest(int* status) { (void)GFFT_DCHECK(threadIdx.x > 1000u, status); }
}  // namespace
extern "C" {
#endif

int gfft_selftest_bounds_check(int* status, int* line) {
  if (!status || !line) return GFFT_E_NULL_POINTER;
#ifdef GFFT_DEBUG
  int* d = nullptr;
  if (cudaMalloc(&d, 2 * sizeof(int)) != cudaSuccess) return GFFT_E_ALLOC;
  int st = GFFT_OK;
  int h[2] = {0, 0};
  if (cudaMemset(d, 0, 2 * sizeof(int)) != cudaSuccess) st = GFFT_E_CUDA;
  if (st == GFFT_OK) {
    dcheck_selftest<<<1, 1>>>(d);
    if (cudaGetLastError() != cudaSuccess || cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess)
      st = GFFT_E_CUDA;
  }
  cudaFree(d);
  *status = h[0];
  *line = h[1];
  return st;
#else
  *status = 0;
  *line = 0;
  return GFFT_E_INVALID_PLAN;
#endif
}

int gfft_exec(gfft_handle h, const void* src, void* dst, gfft_stream stream) {
  if (!valid(h)) return GFFT_E_INVALID_HANDLE;
  if (!src || !dst) return GFFT_E_NULL_POINTER;
  const size_t al = h->hp.dbl ? 16 : 8;
  if (((uintptr_t)src % al) || ((uintptr_t)dst % al)) return GFFT_E_MISALIGNED;
  if (h->hp.place == 0 && src != dst) return GFFT_E_INVALID_PLACE;
  if (h->dct_inner) return gfft_dct_exec(h, src, dst, (cudaStream_t)stream);
  if (h->nd_inner) return gfft_nd_exec(h, src, dst, (cudaStream_t)stream);
  if ((((uintptr_t)src) | ((uintptr_t)dst)) & 15) {
    bool col = false;
    for (int g = 0; g < h->hp.nglobal; ++g) col = col || (h->hp.gp[g].variant == 9 && !h->hp.gp[g].gather);
    if (col) {
      if (!h->unaligned) {
        gfft_plan_opts o;
        std::memset(&o, 0, sizeof(o));
        o.kernel_variant = 5;
        const int st = gfft_create_opts(&h->unaligned, (uint64_t)h->hp.n, h->vtype, h->trans_id, 1, h->parall_id,
                                        h->place_id, (uint64_t)h->hp.batch, &o);
        if (st != GFFT_OK) return st;
      }
      return gfft_exec(h->unaligned, src, dst, stream);
    }
  }
  return gfft_exec_ws(h, src, dst, (cudaStream_t)stream, h->d_ws[0], h->d_ws[1]);
}

// Pipelined host path: the batch is cut into up to GFFT_MAX_CHUNKS slices;
// slice i is uploaded on one stream, transformed on a second once its upload
// is done, and downloaded on a third once its transform is done, so the two
// copy directions and the kernels overlap.  Returns a status.
static int exec_host_chunked(gfft_handle h, const void* src, void* dst, cudaStream_t user) {
  const size_t esz = elem_bytes(h->hp.dbl);
  const long long n = h->hp.n, batch = h->hp.batch;
  if (h->n_chunks == 0) {
    const size_t bytes = (size_t)n * (size_t)batch * esz;
    long long K = (long long)(bytes / (128ull << 20));
    if (K < 4) K = 4;
    if (K > GFFT_MAX_CHUNKS) K = GFFT_MAX_CHUNKS;
    if (K > batch) K = batch;
    const long long cb = (batch + K - 1) / K;
    K = (batch + cb - 1) / cb;
    const long long last = batch - (K - 1) * cb;
    gfft_plan_opts o;
    std::memset(&o, 0, sizeof(o));
    o.radix_order = h->popts.radix_order;
    o.max_radix = h->popts.max_radix;
    o.threads_per_block = h->popts.threads;
    o.units_per_block = h->popts.units;
    o.max_pass_len = h->popts.max_pass_len;
    o.kernel_variant = h->popts.variant;
    o.stages = h->popts.stages;
    o.decimation = h->popts.dif;
    const gfft_plan_opts* op = h->has_opts ? &o : nullptr;
    int st = gfft_create_opts(&h->chunk_plan[0], (uint64_t)n, h->vtype, h->trans_id, 1, h->parall_id, h->place_id,
                              (uint64_t)cb, op);
    if (st != GFFT_OK) return st;
    if (last != cb) {
      st = gfft_create_opts(&h->chunk_plan[1], (uint64_t)n, h->vtype, h->trans_id, 1, h->parall_id, h->place_id,
                            (uint64_t)last, op);
      if (st != GFFT_OK) return st;
    }
    for (int i = 0; i < 3; ++i)
      if (cudaStreamCreateWithFlags(&h->hstream[i], cudaStreamNonBlocking) != cudaSuccess) return GFFT_E_CUDA;
    for (long long i = 0; i < K; ++i)
      if (cudaEventCreateWithFlags(&h->ev_in[i], cudaEventDisableTiming) != cudaSuccess ||
          cudaEventCreateWithFlags(&h->ev_done[i], cudaEventDisableTiming) != cudaSuccess)
        return GFFT_E_CUDA;
    if (cudaEventCreateWithFlags(&h->ev_user, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_end, cudaEventDisableTiming) != cudaSuccess)
      return GFFT_E_CUDA;
    h->chunk_batch = cb;
    h->n_chunks = (int)K;
  }
  cudaStream_t sin = h->hstream[0], scomp = h->hstream[1], sout = h->hstream[2];
  // order after earlier work on the caller's stream
  if (cudaEventRecord(h->ev_user, user) != cudaSuccess) return GFFT_E_CUDA;
  for (int i = 0; i < 3; ++i)
    if (cudaStreamWaitEvent(h->hstream[i], h->ev_user, 0) != cudaSuccess) return GFFT_E_CUDA;
  const long long cb = h->chunk_batch;
  for (int i = 0; i < h->n_chunks; ++i) {
    const long long b0 = (long long)i * cb;
    const long long nb = (b0 + cb <= batch) ? cb : batch - b0;
    gfft_plan* sub = (nb == cb) ? h->chunk_plan[0] : h->chunk_plan[1];
    const size_t off = (size_t)b0 * (size_t)n * esz, len = (size_t)nb * (size_t)n * esz;
    char* dev = (char*)h->d_stage + off;
    if (cudaMemcpyAsync(dev, (const char*)src + off, len, cudaMemcpyHostToDevice, sin) != cudaSuccess)
      return GFFT_E_CUDA;
    if (cudaEventRecord(h->ev_in[i], sin) != cudaSuccess) return GFFT_E_CUDA;
    if (cudaStreamWaitEvent(scomp, h->ev_in[i], 0) != cudaSuccess) return GFFT_E_CUDA;
    int st = gfft_exec_ws(sub, dev, dev, scomp, sub->d_ws[0], sub->d_ws[1]);
    if (st != GFFT_OK) return st;
    if (cudaEventRecord(h->ev_done[i], scomp) != cudaSuccess) return GFFT_E_CUDA;
    if (cudaStreamWaitEvent(sout, h->ev_done[i], 0) != cudaSuccess) return GFFT_E_CUDA;
    if (cudaMemcpyAsync((char*)dst + off, dev, len, cudaMemcpyDeviceToHost, sout) != cudaSuccess)
      return GFFT_E_CUDA;
  }
  if (cudaEventRecord(h->ev_end, sout) != cudaSuccess) return GFFT_E_CUDA;
  if (cudaStreamWaitEvent(user, h->ev_end, 0) != cudaSuccess) return GFFT_E_CUDA;
  if (cudaStreamSynchronize(sout) != cudaSuccess || cudaStreamSynchronize(scomp) != cudaSuccess ||
      cudaStreamSynchronize(sin) != cudaSuccess)
    return GFFT_E_CUDA;
  return GFFT_OK;
}

int gfft_exec_host(gfft_handle h, const void* src, void* dst, gfft_stream stream) {
  if (!valid(h)) return GFFT_E_INVALID_HANDLE;
  if (!src || !dst) return GFFT_E_NULL_POINTER;
  if (h->hp.place == 0 && src != dst) return GFFT_E_INVALID_PLACE;
  // complex elements, or reals for a cosine transform
  const size_t bytes =
      (size_t)h->hp.n * (size_t)h->hp.batch * elem_bytes(h->hp.dbl) / (h->dct_inner ? 2 : 1);
  if (!h->d_stage) {
    if (cudaMalloc(&h->d_stage, bytes) != cudaSuccess) {
      h->d_stage = nullptr;
      return GFFT_E_ALLOC;
    }
    h->stage_bytes = bytes;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (bytes >= (64ull << 20) && h->hp.batch >= 4 && !h->dct_inner && !h->nd_inner)
    return exec_host_chunked(h, src, dst, s);
  if (cudaMemcpyAsync(h->d_stage, src, bytes, cudaMemcpyHostToDevice, s) != cudaSuccess) return GFFT_E_CUDA;
  int st = h->dct_inner  ? gfft_dct_exec(h, h->d_stage, h->d_stage, s)
           : h->nd_inner ? gfft_nd_exec(h, h->d_stage, h->d_stage, s)
                         : gfft_exec_ws(h, h->d_stage, h->d_stage, s, h->d_ws[0], h->d_ws[1]);
  if (st != GFFT_OK) return st;
  if (cudaMemcpyAsync(dst, h->d_stage, bytes, cudaMemcpyDeviceToHost, s) != cudaSuccess) return GFFT_E_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return GFFT_E_CUDA;
  return GFFT_OK;
}

}  // extern "C"
