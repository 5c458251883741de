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
  // true for handles made by gfft_create: only those may allocate a missing
  // second workspace on first need (gfft_exec_ws)
  bool owns_ws = false;
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
  // plans with tensor-copy column tiles (variant 9) need 16-byte aligned
  // buffers: a pointer aligned only to its element runs through this
  // second handle (column tiles of variant 5), made on first need
  gfft_plan* unaligned = nullptr;
  // cosine transforms (transform IDs 4-7): pre pass, this inner real
  // transform of length dct_m (complex half-length), post pass
  gfft_plan* dct_inner = nullptr;
  int dct_type = 0;  // 1 or 2, 0 for every other transform
  long long dct_m = 0;
  void* d_dct[2] = {nullptr, nullptr};  // the extended input and the packed spectrum
  size_t dct_bytes = 0;
  // multi-dimensional transforms (gfft_create_nd): the innermost axis as
  // this inner batched plan, every outer axis as one column pass (no
  // four-step twiddle) in place on the output
  gfft_plan* nd_inner = nullptr;
  int nd_rank = 0;
  long long nd_dims[3] = {1, 1, 1};
  GlobalPass nd_gp[2];
  long long nd_stride[2] = {0, 0};
  void* nd_tab[2] = {nullptr, nullptr};
  unsigned nd_grid[2] = {0, 0};
};

// cosine transforms (defined in gfft_dct.cu)
extern "C" int gfft_dct_create(gfft_plan** handle, uint64_t n, int vtype_id, int trans_id, int parall_id,
                               int place_id, uint64_t batch);
extern "C" int gfft_dct_exec(gfft_plan* h, const void* src, void* dst, cudaStream_t stream);
// multi-dimensional transforms (defined in gfft_nd.cu)
extern "C" int gfft_nd_exec(gfft_plan* h, const void* src, void* dst, cudaStream_t stream);

// Runs a plan with the given workspace buffers (defined in gfft_capi.cu).
extern "C" int gfft_exec_ws(gfft_plan* h, const void* src, void* dst, cudaStream_t stream, void* ws0, void* ws1);
