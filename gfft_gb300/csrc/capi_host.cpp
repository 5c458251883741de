// Host-only part of the C ABI (include/gfft_gb300.h): argument checks, plan
// options, plan descriptions, status texts and gfft_plan_query.  No CUDA:
// the sanitizer build of the CPU tests compiles this file with the planner.
#include <algorithm>
#include <cstring>

#include "../../include/gfft_gb300.h"
#include "capi_host.h"
#include "plan.h"

namespace gfft {
namespace capi {

int parse_opts(const gfft_plan_opts* opts, PlanOpts& po) {
  if (!opts) return GFFT_OK;
  if (opts->max_radix && opts->max_radix != 2 && opts->max_radix != 4 && opts->max_radix != 8 &&
      opts->max_radix != 16)
    return GFFT_E_INVALID_PLAN;
  if (opts->threads_per_block &&
      (opts->threads_per_block < 32 || opts->threads_per_block > 512 || opts->threads_per_block % 32))
    return GFFT_E_INVALID_PLAN;
  if (opts->units_per_block < 0 || opts->max_pass_len < 0 || opts->radix_order < 0 || opts->radix_order > 2)
    return GFFT_E_INVALID_PLAN;
  po.radix_order = opts->radix_order;
  po.max_radix = opts->max_radix ? opts->max_radix : 16;
  po.threads = opts->threads_per_block;
  po.units = opts->units_per_block;
  po.max_pass_len = opts->max_pass_len;
  po.variant = opts->kernel_variant;
  if (opts->stages < 0 || opts->stages > 8 || opts->blocks_per_sm < 0 || opts->blocks_per_sm > 32)
    return GFFT_E_INVALID_PLAN;
  po.stages = opts->stages;
  po.bps = opts->blocks_per_sm;
  if (opts->decimation < 0 || opts->decimation > 1) return GFFT_E_INVALID_PLAN;
  if (opts->decimation && opts->kernel_variant && opts->kernel_variant != 1) return GFFT_E_INVALID_PLAN;
  po.dif = opts->decimation;
  return GFFT_OK;
}

int check_ids(uint64_t n, int vtype_id, int trans_id, int dim, int parall_id, int place_id, uint64_t batch) {
  if (vtype_id < 0 || vtype_id > 3) return GFFT_E_INVALID_TYPE;
  if (trans_id < 0 || trans_id > 7) return GFFT_E_INVALID_TRANSFORM;
  if (place_id < 0 || place_id > 1) return GFFT_E_INVALID_PLACE;
  if (dim != 1) return GFFT_E_INVALID_DIM;
  if (parall_id < 0) return GFFT_E_INVALID_PARALL;
  if (n == 0 || batch == 0 || n > (1ULL << 40) || batch > (1ULL << 40)) return GFFT_E_INVALID_SIZE;
  return GFFT_OK;
}

void fill_info(const HostPlan& p, int vtype, size_t tab_bytes, size_t ws_bytes, gfft_plan_info* info) {
  std::memset(info, 0, sizeof(*info));
  info->n = (uint64_t)p.n;
  info->batch = (uint64_t)p.batch;
  info->vtype_id = vtype;
  info->trans_id = p.trans;
  info->place_id = p.place;
  info->n_global_passes = p.nglobal;
  for (int g = 0; g < p.nglobal && g < 4; ++g) {
    info->pass_len[g] = p.gp[g].L;
    for (int i = 0; i < p.gp[g].npass && i < 15; ++i) info->radices[g][i] = p.gp[g].pass[i].R;
    info->threads[g] = p.gp[g].threads;
    info->units[g] = p.gp[g].units;
    info->kernel_variant[g] = p.gp[g].variant;
  }
  info->workspace_bytes = (uint64_t)ws_bytes * (uint64_t)p.n_ws;
  info->table_bytes = (uint64_t)tab_bytes;
  info->real_fused = p.real_fused;
  info->kernels_per_exec = p.nglobal + ((p.trans >= 2 && !p.real_fused) ? 1 : 0);
}


}  // namespace capi
}  // namespace gfft

extern "C" {

const char* gfft_version(void) { return "gfft_gb300 0.2 (sm_103a)"; }

int gfft_debug_build(void) {
#ifdef GFFT_DEBUG
  return 1;
#else
  return 0;
#endif
}

const char* gfft_strerror(int status) {
  switch (status) {
    case GFFT_OK: return "success";
    case GFFT_E_INVALID_SIZE: return "invalid transform length or batch";
    case GFFT_E_INVALID_TYPE: return "invalid value type id";
    case GFFT_E_INVALID_TRANSFORM: return "invalid transform type id";
    case GFFT_E_INVALID_PLACE: return "invalid place id (in place requires src == dst)";
    case GFFT_E_INVALID_DIM: return "dimension not supported (1, 2 or 3; several dimensions for complex DFT/IDFT only)";
    case GFFT_E_INVALID_PARALL: return "invalid parallelization id";
    case GFFT_E_NULL_POINTER: return "null pointer";
    case GFFT_E_MISALIGNED: return "pointer not aligned to a complex element";
    case GFFT_E_ALLOC: return "memory allocation failed";
    case GFFT_E_CUDA: return "CUDA runtime error";
    case GFFT_E_INVALID_HANDLE: return "invalid handle";
    case GFFT_E_NOT_IN_LIST:
      return "Requested transform is not compiled! Check your instantiation of GenerateTransform class!";
    case GFFT_E_TIMEOUT: return "a bounded device wait timed out";
    case GFFT_E_INVALID_PLAN: return "inconsistent plan options";
    case GFFT_E_TOO_LARGE: return "request exceeds the fixed capacity of this entry point";
    case GFFT_E_BOUNDS: return "a device-side bounds check of the debug build failed (the access was skipped)";
    default: return "unknown status";
  }
}

int gfft_plan_query(uint64_t n, int vtype_id, int trans_id, int place_id, uint64_t batch, const gfft_plan_opts* opts,
                    gfft_plan_info* info) {
  if (!info) return GFFT_E_NULL_POINTER;
  int st = gfft::capi::check_ids(n, vtype_id, trans_id, 1, 0, place_id, batch);
  if (st != GFFT_OK) return st;
  PlanOpts po;
  st = gfft::capi::parse_opts(opts, po);
  if (st != GFFT_OK) return st;
  HostPlan hp;
  const int dbl = (vtype_id == 0 || vtype_id == 2) ? 1 : 0;
  if (trans_id >= 4) {  // cosine transform: the inner real transform's plan
    if (vtype_id > 1) return GFFT_E_INVALID_TYPE;
    const bool one = trans_id <= 5;
    if (one && n < 2) return GFFT_E_INVALID_SIZE;
    st = gfft_plan_query(one ? n - 1 : n, vtype_id, 2, 1, batch, opts, info);
    if (st != GFFT_OK) return st;
    info->n = n;
    info->trans_id = trans_id;
    info->place_id = place_id;
    info->kernels_per_exec += 2;
    return GFFT_OK;
  }
  if (gfft_plan_build(hp, (long long)n, (long long)batch, dbl, trans_id, place_id, po) != 0)
    return GFFT_E_INVALID_SIZE;
  const size_t esz = dbl ? 16 : 8;
  gfft::capi::fill_info(hp, vtype_id, std::max<size_t>(hp.table_count, 1) * esz, hp.ws_elems * esz, info);
  return GFFT_OK;
}

}  // extern "C"
