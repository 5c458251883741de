// Host-only helpers of the C ABI (capi_host.cpp), shared with gfft_capi.cu.
#pragma once
#include <cstddef>
#include <cstdint>

#include "../../include/gfft_gb300.h"
#include "plan.h"

namespace gfft {
namespace capi {

// plan options of the C ABI -> the planner's (GFFT_E_INVALID_PLAN if inconsistent)
int parse_opts(const gfft_plan_opts* opts, PlanOpts& po);
// transform identity and sizes (GFFT_E_* on the first invalid one)
int check_ids(uint64_t n, int vtype_id, int trans_id, int dim, int parall_id, int place_id, uint64_t batch);
// the plan description of gfft_get_info / gfft_plan_query
void fill_info(const HostPlan& p, int vtype, size_t tab_bytes, size_t ws_bytes, gfft_plan_info* info);

}  // namespace capi
}  // namespace gfft
