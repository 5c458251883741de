// Ragged batches: transforms of many different lengths in ONE persistent
// launch driven by a device work queue, replayed from a CUDA graph.
//
// The reference's only batching is its OpenMP loop inside one transform
// (ParallLoop, src/gfftomp.h:41-189); a caller with many lengths builds one
// object per length (GenerateTransform over an NList, src/gfftgen.h:189-231)
// and runs them one after another.  Here every length gets a plan (the same
// planner as gfft_create, with a tighter shared-memory budget so that three
// blocks share an SM), and the whole set becomes a list of work items
// (plan, global pass, tile):
//
//   - a single-pass length contributes groups of up to W whole transforms
//     (lanes gathered from their own offsets);
//   - a multi-pass length contributes, per transform and per global pass,
//     tiles of W columns; the tiles of pass g+1 of a transform may start only
//     when all of its pass-g tiles are done (a per-(transform, pass) counter).
//
// Items are ordered largest first (the first passes of the long transforms,
// then the single-pass groups by length, then the later passes), and
// persistent blocks take them from a global queue head with atomicAdd.  A
// later-pass item is taken only after every earlier-pass item was taken by a
// running block, so its wait always ends; the wait is bounded anyway
// (RaggedArgs::spin_limit, then GFFT_E_TIMEOUT in the status word).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/gfft_gb300.h"
#include "engine.cuh"
#include "mixed_shapes.h"
#include "plan.h"

namespace gfft {

// One pass of compile-time radix R over the item's W lanes (run-time W and
// padded stride Lp, compile-time butterfly count per lane, strides and
// twiddle offsets): src -> dst.
template <typename T, int L, int R, int NS>
__device__ __forceinline__ void ct_pass(const typename Vec<T>::t* __restrict__ src,
                                        typename Vec<T>::t* __restrict__ dst, const EngineArgs& a,
                                        const typename Vec<T>::t* __restrict__ tw, int twoff) {
  typedef typename Vec<T>::t V;
  constexpr int NB = L / R;
  const int total = a.W * NB;
  // the first pass (NS = 1) writes each butterfly's R outputs R apart:
  // with lanes of a power-of-two count, consecutive threads take
  // consecutive lanes instead (odd lane stride Lp: distinct banks)
  const bool lf = NS == 1 && a.W >= 4 && (a.W & (a.W - 1)) == 0;
  const int lgw = __ffs(a.W) - 1;
  for (int i = threadIdx.x; i < total; i += blockDim.x) {
    const int lane = lf ? (i & (a.W - 1)) : i / NB;
    const int j = lf ? (i >> lgw) : i - lane * NB, k = j % NS;
    const V* s = src + lane * a.Lp;
    V v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = s[pad<T>(j + r * NB)];
    if constexpr (NS > 1) {
      const V* t = tw + twoff + k;
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = cmul(v[r], __ldg(t + (r - 1) * NS));
    }
    dft<T, V, R>(v);
    V* d = dst + lane * a.Lp;
    const int base = (j - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) d[pad<T>(base + r * NS)] = v[r];
  }
  __syncthreads();
}

// the in-block passes of one listed shape (mixed_shapes.h); returns the
// buffer that holds the result.  Not inlined: one function per shape keeps
// the kernel's own register frame small.
template <typename T, int R0, int R1, int R2, int R3>
__device__ __noinline__ typename Vec<T>::t* ct_passes(typename Vec<T>::t* b0, typename Vec<T>::t* b1,
                                                      const EngineArgs& a) {
  typedef typename Vec<T>::t V;
  constexpr int L = R0 * R1 * R2 * R3;
  const V* tw = (const V*)a.tw;
  ct_pass<T, L, R0, 1>(b0, b1, a, tw, a.pass[0].tw);
  if constexpr (R1 == 1) return b1;
  ct_pass<T, L, R1, R0>(b1, b0, a, tw, a.pass[1].tw);
  if constexpr (R2 == 1) return b0;
  ct_pass<T, L, R2, R0 * R1>(b0, b1, a, tw, a.pass[2].tw);
  if constexpr (R3 == 1) return b1;
  ct_pass<T, L, R3, R0 * R1 * R2>(b1, b0, a, tw, a.pass[3].tw);
  return b0;
}

// Warm L2 with the input tile of work item `it` (issued before the current
// item's passes, so that its load later hits L2 instead of waiting on
// DRAM): one prefetch per 128-byte line of each row segment of a column
// tile, or of each gathered transform of a single-pass group.  The lines
// are the ones load_tile reads; a later pass's input may still be in
// flight from its earlier pass, in which case the line is fetched again
// when written (L2 is the point of coherence), so the hint is only ever
// early, never stale data.
__device__ __forceinline__ void pf_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

template <typename T>
__device__ __forceinline__ void prefetch_item(const RaggedArgs& ra, long long it) {
  typedef typename Vec<T>::t V;
  const RaggedItem item = ra.items[it];
  const RaggedPlan& pl = ra.plans[item.plan];
  constexpr int ESZ = (int)sizeof(V);
  if (pl.nglobal == 1) {
    const long long L = pl.n;
    const int lines = (int)((L * ESZ + 127) / 128);
    for (int i = threadIdx.x; i < item.count * lines; i += blockDim.x) {
      const int l = i / lines, c = i - l * lines;
      pf_l2((const char*)ra.in + ra.lane_off[item.group + l] * ESZ + (long long)c * 128);
    }
  } else {
    const int g = item.pass;
    const V* base = g == 0 ? (const V*)ra.in : (const V*)ra.ws + (g == 2 ? ra.ws2_off : 0);
    base += ra.offset[item.transform] + item.unit0;
    const int L = pl.L[g];
    const long long stride = pl.n / L;
    const int seg = (item.count * ESZ + 127) / 128;  // lines per row segment
    for (int i = threadIdx.x; i < L * seg; i += blockDim.x) {
      const int s = i / seg, c = i - s * seg;
      pf_l2((const char*)(base + (long long)s * stride) + c * 128);
    }
  }
}

// resident blocks per SM the register budget is sized for (70 KB of shared
// memory per block)
template <typename T> struct RaggedOcc { static constexpr int v = sizeof(T) == 4 ? 3 : 2; };

template <typename T>
__global__ void __launch_bounds__(256, RaggedOcc<T>::v) ragged_kernel(const __grid_constant__ RaggedArgs ra) {
  typedef typename Vec<T>::t V;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ EngineArgs ea;
  __shared__ long long item_s, u0_s;
  __shared__ int abort_s, shape_s;
  V* b0 = reinterpret_cast<V*>(smem_raw);
  V* b1 = b0 + ra.lanes_max;
  int key = -1;  // (plan, pass) whose arguments `ea` holds
  if (threadIdx.x == 0) item_s = atomicAdd(ra.head, 1);
  while (true) {
    if (threadIdx.x == 0) abort_s = 0;
    __syncthreads();
    const long long it = item_s;
    if (it >= ra.nitems) return;
    const RaggedItem item = ra.items[it];
    const int k = item.plan * GFFT_MAXG + item.pass;
    if (k != key) {  // the engine arguments of this (plan, pass), copied by the whole block
      const int* src = reinterpret_cast<const int*>(ra.ea + k);
      int* dst = reinterpret_cast<int*>(&ea);
      for (int w = threadIdx.x; w < (int)(sizeof(EngineArgs) / sizeof(int)); w += blockDim.x) dst[w] = __ldg(src + w);
      key = k;
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      const RaggedPlan& pl = ra.plans[item.plan];
      const int g = item.pass;
      if (g > 0) {  // wait for every tile of the previous pass of this transform
        volatile int* d = ra.done + (long long)item.transform * GFFT_MAXG + (g - 1);
        const int need = pl.tiles[g - 1];
        long long i = 0;
        while (*d < need && i < ra.spin_limit) {
          __nanosleep(64);
          ++i;
        }
        if (*d < need) {
          atomicExch(ra.status, 13 /* GFFT_E_TIMEOUT */);
          abort_s = 1;
        }
        __threadfence();
      }
      shape_s = sizeof(T) == 8 ? -1 : pl.shape[g];
      if (pl.nglobal == 1) {
        ea.in = ra.in;
        ea.out = ra.out;
        ea.lane_off = ra.lane_off + item.group;
        ea.W = item.count;
        ea.nunits = item.count;
        u0_s = 0;
      } else {
        // buffer chain: 2 passes in -> ws -> out; 3 passes in -> ws -> ws2 -> out
        const long long off = ra.offset[item.transform];
        const bool last = (g == pl.nglobal - 1);
        const V* bufs_in[3] = {(const V*)ra.in, (const V*)ra.ws, (const V*)ra.ws + ra.ws2_off};
        V* bufs_out[3] = {(V*)ra.ws, (V*)ra.ws + ra.ws2_off, (V*)ra.out};
        ea.in = bufs_in[g] + off;
        ea.out = last ? (V*)ra.out + off : bufs_out[g] + off;
        u0_s = item.unit0;
      }
    }
    __syncthreads();
    if (abort_s) return;
    const long long u0 = u0_s;
    load_tile<T>(ea, b0, u0);
    // claim the next item now: the queue's round trip overlaps this item's
    // passes (the value is used only after them).  A block never holds a
    // claim on an item listed before the one it works on, so the dependency
    // waits still always end.
    __shared__ long long next_s;
    if (threadIdx.x == 0) next_s = atomicAdd(ra.head, 1);
    __syncthreads();
    const long long next_item = next_s;
    if (next_item < ra.nitems) prefetch_item<T>(ra, next_item);
    V* src = b0;
    V* dst = b1;
    const V* tw = (const V*)ea.tw;
    const int sh = shape_s;
    if constexpr (sizeof(T) == 4) {
      switch (sh) {
#define GFFT_RAGGED_CASE(i, a, b, c, d) \
  case i: src = ct_passes<T, a, b, c, d>(b0, b1, ea); break;
        GFFT_RAGGED_SHAPES(GFFT_RAGGED_CASE)
#undef GFFT_RAGGED_CASE
        default: break;
      }
    }
    for (int p = 0; p < ea.npass && !(sizeof(T) == 4 && sh >= 0); ++p) {
      const BlockPass bp = ea.pass[p];
      switch (bp.R) {
        case 16: block_pass<T, 16>(src, dst, ea, bp, tw); break;
        case 8: block_pass<T, 8>(src, dst, ea, bp, tw); break;
        case 4: block_pass<T, 4>(src, dst, ea, bp, tw); break;
        case 2: block_pass<T, 2>(src, dst, ea, bp, tw); break;
        case 3: block_pass<T, 3>(src, dst, ea, bp, tw); break;
        case 5: block_pass<T, 5>(src, dst, ea, bp, tw); break;
        case 7: block_pass<T, 7>(src, dst, ea, bp, tw); break;
        case 6: block_pass<T, 6>(src, dst, ea, bp, tw); break;
        case 9: block_pass<T, 9>(src, dst, ea, bp, tw); break;
        case 10: block_pass<T, 10>(src, dst, ea, bp, tw); break;
        case 12: block_pass<T, 12>(src, dst, ea, bp, tw); break;
        case 15: block_pass<T, 15>(src, dst, ea, bp, tw); break;
        default: block_pass_generic<T>(src, dst, ea, bp, tw); break;
      }
      __syncthreads();
      V* t = src;
      src = dst;
      dst = t;
    }
    store_tile<T>(ea, src, u0);
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
      if (ea.mode == 1 && item.pass < ra.plans[item.plan].nglobal - 1)
        atomicAdd(ra.done + (long long)item.transform * GFFT_MAXG + item.pass, 1);
      item_s = next_item;
    }
  }
}

}  // namespace gfft

struct gfft_ragged {
  int dbl = 0, inverse = 0;
  long long count = 0, total = 0;
  int nplans = 0;
  long long nitems = 0;
  void* d_tab = nullptr;
  RaggedPlan* d_plans = nullptr;
  RaggedItem* d_items = nullptr;
  EngineArgs* d_ea = nullptr;
  long long* d_lane_off = nullptr;
  long long* d_offset = nullptr;
  int* d_done = nullptr;
  int* d_head = nullptr;
  int* d_status = nullptr;
  void* d_ws = nullptr;
  long long ws2_off = 0;
  int lanes_max = 0;
  unsigned grid = 0, threads = 256;
  size_t smem = 0;
  size_t done_bytes = 0;
  // the captured launch sequence and the pointers it was captured with
  cudaStream_t cap_stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  const void* g_src = nullptr;
  void* g_dst = nullptr;
  int max_passes = 1;
  // host copy of the per-length plans (gfft_ragged_get_plan)
  std::vector<RaggedPlan> hplans;
  unsigned magic = 0x6A66ED00u;
};

namespace {

void free_ragged(gfft_ragged* r) {
  if (!r) return;
  if (r->gexec) cudaGraphExecDestroy(r->gexec);
  if (r->graph) cudaGraphDestroy(r->graph);
  if (r->cap_stream) cudaStreamDestroy(r->cap_stream);
  void* ps[] = {r->d_tab, r->d_plans, r->d_items, r->d_ea, r->d_lane_off, r->d_offset, r->d_done, r->d_head,
                r->d_status, r->d_ws};
  for (void* p : ps)
    if (p) cudaFree(p);
  delete r;
}

template <typename T>
int upload(void** dst, const std::vector<T>& v) {
  size_t bytes = std::max<size_t>(v.size(), 1) * sizeof(T);
  if (cudaMalloc(dst, bytes) != cudaSuccess) {
    *dst = nullptr;
    return GFFT_E_ALLOC;
  }
  if (!v.empty() && cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
    return GFFT_E_CUDA;
  return GFFT_OK;
}

}  // namespace

extern "C" {

int gfft_ragged_create(gfft_ragged** handle, uint64_t count, const uint64_t* sizes, int vtype_id, int trans_id) {
  return gfft_ragged_create_opts(handle, count, sizes, vtype_id, trans_id, 0, nullptr, nullptr);
}

int gfft_ragged_create_opts(gfft_ragged** handle, uint64_t count, const uint64_t* sizes, int vtype_id, int trans_id,
                            uint64_t n_opts, const uint64_t* opt_lengths, const gfft_plan_opts* opts) {
  if (!handle || !sizes) return GFFT_E_NULL_POINTER;
  *handle = nullptr;
  if (count == 0 || count > (1ULL << 31)) return GFFT_E_INVALID_SIZE;
  if (vtype_id < 0 || vtype_id > 3) return GFFT_E_INVALID_TYPE;
  if (trans_id != 0 && trans_id != 1) return GFFT_E_INVALID_TRANSFORM;
  if (n_opts && (!opt_lengths || !opts)) return GFFT_E_NULL_POINTER;
  for (uint64_t i = 0; i < n_opts; ++i) {
    const gfft_plan_opts& o = opts[i];
    if (o.radix_order < 0 || o.radix_order > 2 || o.units_per_block < 0 || o.units_per_block > 256 ||
        o.max_pass_len < 0 || (o.max_radix && o.max_radix != 2 && o.max_radix != 4 && o.max_radix != 8 &&
                               o.max_radix != 16))
      return GFFT_E_INVALID_PLAN;
  }
  gfft_ragged* r = new (std::nothrow) gfft_ragged();
  if (!r) return GFFT_E_ALLOC;
  r->dbl = (vtype_id == 0 || vtype_id == 2) ? 1 : 0;
  r->inverse = trans_id == 1;
  r->count = (long long)count;
  const int esz = r->dbl ? 16 : 8;
  const int ps = r->dbl ? 3 : 4;
  // distinct lengths, their plans and tables
  std::vector<long long> offs(count);
  std::vector<long long> distinct;
  long long total = 0;
  for (uint64_t i = 0; i < count; ++i) {
    if (sizes[i] == 0) {
      free_ragged(r);
      return GFFT_E_INVALID_SIZE;
    }
    offs[i] = total;
    total += (long long)sizes[i];
    distinct.push_back((long long)sizes[i]);
  }
  r->total = total;
  std::sort(distinct.begin(), distinct.end());
  distinct.erase(std::unique(distinct.begin(), distinct.end()), distinct.end());
  PlanOpts po;
  po.max_single = r->dbl ? 2048 : 4096;
  po.smem_budget = 72 * 1024;
  po.variant = 1;
  po.units = r->dbl ? 2 : 4;  // sizes the pass-length cap: passes up to 1024 within the budget
  const long long TILE = r->dbl ? 2048 : 4096;  // points per work item
  std::vector<RaggedPlan> plans(distinct.size());
  std::vector<double> tab;
  int lanes_max = 0;
  for (size_t d = 0; d < distinct.size(); ++d) {
    // this length's schedule: the caller's options (the autotuner's choice), else the defaults
    PlanOpts pod = po;
    int w_req = 0;
    for (uint64_t i = 0; i < n_opts; ++i)
      if ((long long)opt_lengths[i] == distinct[d]) {
        const gfft_plan_opts& o = opts[i];
        if (o.max_pass_len > 0) pod.max_pass_len = o.max_pass_len;
        pod.radix_order = o.radix_order;
        if (o.max_radix) pod.max_radix = o.max_radix;
        w_req = o.units_per_block;
        break;
      }
    HostPlan hp;
    if (gfft_plan_build(hp, distinct[d], 1, r->dbl, trans_id, 1, pod) != 0 || hp.nglobal > 3) {
      free_ragged(r);
      return GFFT_E_INVALID_SIZE;
    }
    RaggedPlan& rp = plans[d];
    std::memset(&rp, 0, sizeof(rp));
    rp.n = distinct[d];
    rp.nglobal = hp.nglobal;
    r->max_passes = std::max(r->max_passes, hp.nglobal);
    for (int g = 0; g < hp.nglobal; ++g) {
      const GlobalPass& gp = hp.gp[g];
      rp.L[g] = gp.L;
      rp.npass[g] = gp.npass;
      {
        int rs[GFFT_MAXP];
        for (int i = 0; i < gp.npass; ++i) rs[i] = gp.pass[i].R;
        rp.shape[g] = (!r->dbl && gp.npass <= 4) ? ragged_shape_index(rs, gp.npass) : -1;
      }
      rp.Ns[g] = gp.Ns;
      for (int i = 0; i < gp.npass; ++i) rp.pass[g][i] = gp.pass[i];
      if (hp.nglobal == 1) {
        // groups of whole transforms: about 4096 (FP32) / 2048 (FP64) points
        int W = w_req > 0 ? w_req : std::max<int>(1, (r->dbl ? 2048 : 4096) / gp.L);
        while (W > 1 && 2LL * W * engine_padded(gp.L, r->dbl) * esz > po.smem_budget) --W;
        rp.W[g] = W;
      } else {
        // columns per item: a power of two, about TILE points (or the
        // requested count), within the transform and the shared-memory budget
        const long long stride = distinct[d] / gp.L;
        long long W = 1;
        if (w_req > 0)
          while (2 * W <= w_req && 2 * W <= stride && 2 * 2 * W * engine_padded(gp.L, r->dbl) * esz <= po.smem_budget)
            W *= 2;
        else
          while (2 * W * gp.L <= TILE && 2 * W <= stride && 2 * W <= 256) W *= 2;
        rp.W[g] = (int)W;
        rp.tiles[g] = (int)((stride + W - 1) / W);
      }
      lanes_max = std::max<int>(lanes_max, (int)(rp.W[g] * engine_padded(gp.L, r->dbl)));
    }
    rp.tab = (long long)(tab.size() / 2);
    rp.gtw_lo = (long long)hp.gtw_lo_off;
    rp.gtw_hi = (long long)hp.gtw_hi_off;
    rp.gB = (long long)hp.gtw_B;
    std::vector<double> t(2 * std::max<size_t>(hp.table_count, 1), 0.0);
    gfft_plan_tables(hp, t.data());
    tab.insert(tab.end(), t.begin(), t.end());
  }
  r->nplans = (int)plans.size();
  r->lanes_max = lanes_max;
  r->hplans = plans;
  // work items, largest first
  std::vector<std::vector<long long>> members(distinct.size());
  for (uint64_t i = 0; i < count; ++i) {
    size_t d = std::lower_bound(distinct.begin(), distinct.end(), (long long)sizes[i]) - distinct.begin();
    members[d].push_back((long long)i);
  }
  std::vector<RaggedItem> items;
  std::vector<long long> lane_off;
  auto add_multi = [&](int g) {
    for (size_t dd = distinct.size(); dd-- > 0;) {
      const RaggedPlan& rp = plans[dd];
      if (rp.nglobal <= g || rp.nglobal == 1) continue;
      const long long stride = rp.n / rp.L[g];
      for (long long t : members[dd])
        for (int k = 0; k < rp.tiles[g]; ++k) {
          RaggedItem it;
          it.plan = (int)dd;
          it.pass = g;
          it.transform = (int)t;
          it.unit0 = (long long)k * rp.W[g];
          it.count = (int)std::min<long long>(rp.W[g], stride - it.unit0);
          it.group = 0;
          items.push_back(it);
        }
    }
  };
  add_multi(0);
  for (size_t dd = distinct.size(); dd-- > 0;) {
    const RaggedPlan& rp = plans[dd];
    if (rp.nglobal != 1) continue;
    const std::vector<long long>& m = members[dd];
    for (size_t k = 0; k < m.size(); k += rp.W[0]) {
      RaggedItem it;
      it.plan = (int)dd;
      it.pass = 0;
      it.transform = (int)m[k];
      it.unit0 = 0;
      it.count = (int)std::min<size_t>(rp.W[0], m.size() - k);
      it.group = (long long)lane_off.size();
      for (int j = 0; j < it.count; ++j) lane_off.push_back(offs[m[k + j]]);
      items.push_back(it);
    }
  }
  add_multi(1);
  add_multi(2);
  r->nitems = (long long)items.size();
  // device buffers
  int st = GFFT_OK;
  if (r->dbl) {
    st = upload(&r->d_tab, tab);
  } else {
    std::vector<float> f(tab.begin(), tab.end());
    st = upload(&r->d_tab, f);
  }
  if (st == GFFT_OK) st = upload((void**)&r->d_plans, plans);
  if (st == GFFT_OK) st = upload((void**)&r->d_items, items);
  if (st == GFFT_OK) {
    // engine arguments per (plan, global pass); the buffers are set per item
    std::vector<EngineArgs> eas((size_t)r->nplans * GFFT_MAXG);
    std::memset(eas.data(), 0, eas.size() * sizeof(EngineArgs));
    const char* tb = (const char*)r->d_tab;
    for (int d = 0; d < r->nplans; ++d) {
      const RaggedPlan& pl = plans[(size_t)d];
      for (int g = 0; g < pl.nglobal; ++g) {
        EngineArgs& e = eas[(size_t)d * GFFT_MAXG + g];
        const int L = pl.L[g];
        e.L = L;
        e.pad_shift = ps;
        e.Lp = (int)engine_padded(L, r->dbl);
        e.N = pl.n;
        e.npass = pl.npass[g];
        for (int i = 0; i < e.npass; ++i) {
          e.pass[i] = pl.pass[g][i];
          e.pass[i].fd_nb = make_fastdiv((unsigned)(L / e.pass[i].R));
          e.pass[i].fd_ns = make_fastdiv((unsigned)e.pass[i].Ns);
        }
        e.fd_L = make_fastdiv((unsigned)L);
        e.tw = tb + (size_t)pl.tab * esz;
        e.gtw_lo = tb + (size_t)(pl.tab + pl.gtw_lo) * esz;
        e.gtw_hi = tb + (size_t)(pl.tab + pl.gtw_hi) * esz;
        e.gB = pl.gB;
        e.conj = r->inverse;
        e.real = 0;
        e.scale = (r->inverse && g == pl.nglobal - 1) ? 1.0 / (double)pl.n : 1.0;
        e.ldcg = g > 0;
        if (pl.nglobal == 1) {
          e.mode = 2;
          e.stride = 1;
          e.gNs = 1;
        } else {
          e.mode = 1;
          e.W = pl.W[g];
          e.stride = pl.n / L;
          e.nunits = e.stride;
          e.gNs = pl.Ns[g];
        }
      }
    }
    st = upload((void**)&r->d_ea, eas);
  }
  if (st == GFFT_OK) st = upload((void**)&r->d_lane_off, lane_off);
  if (st == GFFT_OK) st = upload((void**)&r->d_offset, offs);
  r->done_bytes = (size_t)count * GFFT_MAXG * sizeof(int);
  if (st == GFFT_OK && cudaMalloc((void**)&r->d_done, r->done_bytes) != cudaSuccess) st = GFFT_E_ALLOC;
  if (st == GFFT_OK && cudaMalloc((void**)&r->d_head, 256) != cudaSuccess) st = GFFT_E_ALLOC;
  if (st == GFFT_OK && (cudaMalloc((void**)&r->d_status, 256) != cudaSuccess ||
                        cudaMemset(r->d_status, 0, 256) != cudaSuccess))
    st = GFFT_E_ALLOC;
  if (st == GFFT_OK && r->max_passes > 1) {
    r->ws2_off = r->max_passes > 2 ? total : 0;
    const size_t wsb = (size_t)total * esz * (r->max_passes > 2 ? 2 : 1);
    if (cudaMalloc(&r->d_ws, wsb) != cudaSuccess) st = GFFT_E_ALLOC;
  }
  if (st == GFFT_OK && cudaStreamCreateWithFlags(&r->cap_stream, cudaStreamNonBlocking) != cudaSuccess)
    st = GFFT_E_CUDA;
  if (st != GFFT_OK) {
    free_ragged(r);
    return st;
  }
  // persistent grid: every block resident
  r->smem = (size_t)2 * lanes_max * esz;
  int maxopt = 0, nsm = 0, dev = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maxopt, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (r->smem + 4096 > (size_t)maxopt) {  // dynamic buffers plus the kernel's static shared memory
    free_ragged(r);
    return GFFT_E_INVALID_SIZE;
  }
  cudaError_t ce = r->dbl ? cudaFuncSetAttribute(gfft::ragged_kernel<double>,
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)r->smem)
                          : cudaFuncSetAttribute(gfft::ragged_kernel<float>,
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)r->smem);
  if (ce != cudaSuccess) {
    cudaGetLastError();  // do not leave the failure for the next launch to report
    free_ragged(r);
    return GFFT_E_CUDA;
  }
  if (r->dbl)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, gfft::ragged_kernel<double>, r->threads, r->smem);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, gfft::ragged_kernel<float>, r->threads, r->smem);
  if (per < 1) {
    free_ragged(r);
    return GFFT_E_INVALID_SIZE;
  }
  r->grid = (unsigned)std::min<long long>((long long)nsm * per, r->nitems);
  *handle = r;
  return GFFT_OK;
}

static int ragged_launch(gfft_ragged* r, const void* src, void* dst, cudaStream_t s) {
  if (cudaMemsetAsync(r->d_done, 0, r->done_bytes, s) != cudaSuccess) return GFFT_E_CUDA;
  if (cudaMemsetAsync(r->d_head, 0, sizeof(int), s) != cudaSuccess) return GFFT_E_CUDA;
  RaggedArgs a;
  std::memset(&a, 0, sizeof(a));
  a.in = src;
  a.out = dst;
  a.ws = r->d_ws;
  a.ws2_off = r->ws2_off;
  a.tab = r->d_tab;
  a.plans = r->d_plans;
  a.items = r->d_items;
  a.ea = r->d_ea;
  a.lane_off = r->d_lane_off;
  a.offset = r->d_offset;
  a.done = r->d_done;
  a.head = r->d_head;
  a.status = r->d_status;
  a.nitems = r->nitems;
  a.spin_limit = 1LL << 24;
  a.conj = r->inverse;
  a.lanes_max = r->lanes_max;
  cudaGetLastError();  // clear a stale error of an earlier, unrelated call
  if (r->dbl)
    gfft::ragged_kernel<double><<<r->grid, r->threads, r->smem, s>>>(a);
  else
    gfft::ragged_kernel<float><<<r->grid, r->threads, r->smem, s>>>(a);
  return cudaGetLastError() == cudaSuccess ? GFFT_OK : GFFT_E_CUDA;
}

int gfft_ragged_exec(gfft_ragged* r, const void* src, void* dst, gfft_stream stream) {
  if (!r || r->magic != 0x6A66ED00u) return GFFT_E_INVALID_HANDLE;
  if (!src || !dst) return GFFT_E_NULL_POINTER;
  const size_t al = r->dbl ? 16 : 8;
  if (((uintptr_t)src % al) || ((uintptr_t)dst % al)) return GFFT_E_MISALIGNED;
  if (src == dst && r->max_passes > 1) {
    // a single-pass group reads and writes whole transforms, a multi-pass
    // transform goes through the workspace: both are safe in place except
    // the first pass of a multi-pass transform writing the workspace while
    // its input is also the output of the last pass -- also safe, since the
    // last pass runs after every first-pass tile of that transform.
  }
  if (!r->gexec || r->g_src != src || r->g_dst != dst) {
    if (r->gexec) {
      cudaGraphExecDestroy(r->gexec);
      r->gexec = nullptr;
    }
    if (r->graph) {
      cudaGraphDestroy(r->graph);
      r->graph = nullptr;
    }
    if (cudaStreamBeginCapture(r->cap_stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return GFFT_E_CUDA;
    int st = ragged_launch(r, src, dst, r->cap_stream);
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamEndCapture(r->cap_stream, &g);
    if (st != GFFT_OK || ce != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return GFFT_E_CUDA;
    }
    r->graph = g;
    if (cudaGraphInstantiate(&r->gexec, g, 0) != cudaSuccess) return GFFT_E_CUDA;
    r->g_src = src;
    r->g_dst = dst;
  }
  return cudaGraphLaunch(r->gexec, (cudaStream_t)stream) == cudaSuccess ? GFFT_OK : GFFT_E_CUDA;
}

int gfft_ragged_get_info(gfft_ragged* r, uint64_t* total_points, uint64_t* items, int* distinct_lengths,
                         int* max_passes, unsigned* grid) {
  if (!r || r->magic != 0x6A66ED00u) return GFFT_E_INVALID_HANDLE;
  if (total_points) *total_points = (uint64_t)r->total;
  if (items) *items = (uint64_t)r->nitems;
  if (distinct_lengths) *distinct_lengths = r->nplans;
  if (max_passes) *max_passes = r->max_passes;
  if (grid) *grid = r->grid;
  return GFFT_OK;
}

int gfft_ragged_get_plan(gfft_ragged* r, uint64_t n, gfft_plan_info* info) {
  if (!r || r->magic != 0x6A66ED00u) return GFFT_E_INVALID_HANDLE;
  if (!info) return GFFT_E_NULL_POINTER;
  for (const RaggedPlan& p : r->hplans) {
    if ((uint64_t)p.n != n) continue;
    std::memset(info, 0, sizeof(*info));
    info->n = n;
    info->batch = 0;
    info->vtype_id = r->dbl ? 0 : 1;
    info->trans_id = r->inverse ? 1 : 0;
    info->place_id = 1;
    info->n_global_passes = p.nglobal;
    for (int g = 0; g < p.nglobal && g < 4; ++g) {
      info->pass_len[g] = p.L[g];
      for (int i = 0; i < p.npass[g] && i < 15; ++i) info->radices[g][i] = p.pass[g][i].R;
      info->threads[g] = (int)r->threads;
      info->units[g] = p.W[g];
      info->kernel_variant[g] = 1;  // the run-time engine passes (or a compiled shape of them)
    }
    info->kernels_per_exec = 1;
    return GFFT_OK;
  }
  return GFFT_E_INVALID_SIZE;
}

int gfft_ragged_get_status(gfft_ragged* r, int* status) {
  if (!r || r->magic != 0x6A66ED00u) return GFFT_E_INVALID_HANDLE;
  if (!status) return GFFT_E_NULL_POINTER;
  if (cudaDeviceSynchronize() != cudaSuccess) return GFFT_E_CUDA;
  if (cudaMemcpy(status, r->d_status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return GFFT_E_CUDA;
  if (cudaMemset(r->d_status, 0, sizeof(int)) != cudaSuccess) return GFFT_E_CUDA;
  return GFFT_OK;
}

int gfft_ragged_destroy(gfft_ragged* r) {
  if (!r || r->magic != 0x6A66ED00u) return GFFT_E_INVALID_HANDLE;
  r->magic = 0;
  free_ragged(r);
  return GFFT_OK;
}

}  // extern "C"
