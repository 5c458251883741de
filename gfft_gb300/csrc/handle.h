// The handle behind gfft_handle (include/gfft_gb300.h), shared by the C ABI
// translation units.
#pragma once
#include <cstddef>

#include <cuda_runtime.h>

#include "plan.h"

#define GFFT_MAX_CHUNKS 16

struct gfft_plan {
  HostPlan hp;
  int vtype = 0;
  int device = 0;
  void* d_tab = nullptr;
  size_t tab_bytes = 0;
  void* d_ws[2] = {nullptr, nullptr};
  size_t ws_bytes = 0;
  // staging buffers for gfft_exec_host, allocated on first use
  void* d_stage = nullptr;
  size_t stage_bytes = 0;
  int* d_status = nullptr;     // device status word of this handle's kernels
  unsigned grid[GFFT_MAXG] = {0, 0, 0, 0};  // persistent grid of fast-path passes
  unsigned magic = 0x6FF7B300u;
  // creation arguments (the chunked host path re-plans slices of the batch)
  int trans_id = 0, place_id = 1, parall_id = 0;
  PlanOpts popts;
  bool has_opts = false;
  // chunked host path of gfft_exec_host: sub-plans over slices of the batch,
  // three streams (upload, transform, download) and per-chunk events
  gfft_plan* chunk_plan[2] = {nullptr, nullptr};
  long long chunk_batch = 0;
  int n_chunks = 0;
  cudaStream_t hstream[3] = {nullptr, nullptr, nullptr};
  cudaEvent_t ev_in[GFFT_MAX_CHUNKS] = {};
  cudaEvent_t ev_done[GFFT_MAX_CHUNKS] = {};
  cudaEvent_t ev_user = nullptr, ev_end = nullptr;
};

// Runs a plan with the given workspace buffers (defined in gfft_capi.cu).
extern "C" int gfft_exec_ws(gfft_plan* h, const void* src, void* dst, cudaStream_t stream, void* ws0, void* ws1);
