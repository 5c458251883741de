// Internal plan structures shared by the host planner (planner.cpp) and the
// CUDA kernels (fft_engine.cu).
//
// A transform of length N (complex points) runs as 1..4 "global passes".
// Global pass g is one Stockham step with super-radix L_g over the whole
// array (Stockham autosort: natural-order output, no digit-reversal pass,
// which replaces the reference's GFFTswap2, src/gfftswap.h:74-227):
//
//   for each unit (t, b), t < batch, b < N/L_g, k = b mod Ns_g:
//     v[r]  = x[t*N + b + r*(N/L_g)] * W_{Ns_g*L_g}^{k*r}      r < L_g
//     v     = DFT_{L_g}(v)                                       (in one block)
//     y[t*N + (b/Ns_g)*Ns_g*L_g + k + r*Ns_g] = v[r]
//
// with Ns_g = L_0*...*L_{g-1}.  One thread block computes DFT_{L_g} for
// `units` consecutive units in shared memory, as a sequence of in-block
// Stockham passes of radix R in {2,3,4,5,7,8,16} (or a generic odd prime).
#pragma once
#include <cstdint>

#define GFFT_MAXP 16     // in-block passes
#define GFFT_MAXG 4      // global passes

// Unsigned division by a run-time invariant d via multiply and shift
// (Granlund and Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994, round-up method): for d > 1 with
// l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1 and t = umulhi(x, m),
// x / d = (t + ((x - t) >> 1)) >> (l - 1) for every 32-bit x.
#ifdef __CUDACC__
#define GFFT_HD __host__ __device__
#else
#define GFFT_HD
#endif

struct FastDiv {
  unsigned d, m, l;
};
GFFT_HD inline FastDiv make_fastdiv(unsigned d) {
  FastDiv f;
  f.d = d;
  if (d <= 1) {
    f.m = 0;
    f.l = 0;
    return f;
  }
  unsigned l = 0;
  while ((1ull << l) < d) ++l;
  f.l = l;
  f.m = (unsigned)((((1ull << 32) * ((1ull << l) - d)) / d) + 1);
  return f;
}
#ifdef __CUDACC__
__device__ __forceinline__ unsigned fdiv(unsigned x, const FastDiv& f) {
  if (f.d <= 1) return x;
  const unsigned t = __umulhi(x, f.m);
  return (t + ((x - t) >> 1)) >> (f.l - 1);
}
#endif

struct BlockPass {
  int R;    // radix
  int Ns;   // product of the radices before this pass
  int tw;   // offset (complex elements) of this pass's twiddles in the table
  int gen;  // generic odd prime: offset of its W_R^m table (else -1)
  FastDiv fd_nb;  // L / R
  FastDiv fd_ns;  // Ns
};

// Arguments of one launch of the engine kernel (passed by value).
struct EngineArgs {
  const void* in;
  void* out;
  long long nunits;   // batch * (N / L)
  long long N;        // transform length
  long long stride;   // N / L
  long long gNs;      // Ns of this global pass
  long long gB;       // global twiddle split: W_N^m = lo[m % gB] * hi[m / gB]
  const void* gtw_lo;
  const void* gtw_hi;
  const void* tw;     // in-block pass twiddles (+ generic prime tables)
  const void* rtw;    // real pre/post twiddles W_{2n}^q, q < n
  int L;              // in-block length
  int Lp;             // padded per-unit stride in shared memory
  int W;              // units per block
  int mode;           // 0: units are whole contiguous transforms; 1: lane units
  int npass;
  int conj;           // inverse transform as conj(FFT(conj(x)))
  int real;           // 0 none, 1 real forward post pass, 2 real inverse pre pass
  int pad_shift;      // shared-memory padding: one slot per 2^pad_shift elements
  double scale;       // output scale
  // register-resident pipelined path (variant 2)
  int* status;        // device status word (0 ok, GFFT_E_TIMEOUT on a wait that ran out)
  long long ntiles;   // tiles of W contiguous transforms
  int stages;         // TMA stages per block
  int tile_bytes;     // bytes of one tile (multiple of 16)
  long long spin_limit;  // bound on every mbarrier wait (try_wait iterations)
  int debug_no_issue; // test hook: never issue the copies, so the first wait runs out
  FastDiv fd_L;       // L
  FastDiv fd_half;    // L/2 + 1 (real pre/post pass)
  const long long* lane_off;  // mode 2: element offset of each lane's transform
  int ldcg;           // read the input through L2 only (data written by other blocks of this launch)
  int notw;           // lane passes without the four-step twiddle (axis transforms of a multi-dimensional array)
  const void* ftw;    // variant 9, later global passes: W_(R0 Ns)^(k r) at [r * Ns + k] (null: two-level lookups)
  int dif;            // generic engine: frequency decimation (transposed passes, twiddles after the butterflies)
  int ftw_box;        // variant 9: a tile's [16][W] block of ftw arrives with it by tensor copy (ColMaps in[1])
  BlockPass pass[GFFT_MAXP];
};

struct GlobalPass {
  int L;
  long long Ns;
  int units;      // W
  int threads;
  int mode;
  int variant;    // 1 generic engine, 2 register-resident fast path
  int npass;
  BlockPass pass[GFFT_MAXP];
  size_t smem;
  int stages;     // variant 2: TMA pipeline depth
  int rf = 0;     // variant 9: real pre (2) / post (1) pass fused into this pass
  int tk = 64;    // variant 9: tile KB (64: one block per SM, 32: two)
  int gather = 0; // variant 9, mixed shape: tiles gathered by cp.async (no tensor maps)
  long long ntiles;
  int tile_bytes;
};

struct PlanOpts {
  int radix_order = 0;
  int max_radix = 16;
  int threads = 0;
  int units = 0;
  int max_pass_len = 0;
  int variant = 0;
  int stages = 0;
  // internal (ragged batches): largest single-pass length and shared-memory budget
  int max_single = 0;
  int smem_budget = 0;
  int dif = 0;  // frequency decimation (generic engine only)
  int bps = 0;  // requested blocks per SM (1: 64 KB column tiles for every pass)
};

// ---- ragged batches: one persistent launch over transforms of many sizes --
// Per distinct size: the global passes of its plan (in-block radices,
// twiddle offsets relative to the size's own table block).
struct RaggedPlan {
  long long n;
  int nglobal;
  int tiles[GFFT_MAXG];    // work items of each global pass (two-pass sizes)
  int shape[GFFT_MAXG];    // compile-time pass function of each global pass (mixed_shapes.h), -1: none
  int L[GFFT_MAXG], W[GFFT_MAXG], npass[GFFT_MAXG];
  long long Ns[GFFT_MAXG];
  long long tab;           // this size's tables, complex elements from the table base
  long long gtw_lo, gtw_hi, gB;  // relative to tab
  BlockPass pass[GFFT_MAXG][GFFT_MAXP];
};
// One unit of work: global pass `pass` of a plan, over `count` lanes starting
// at unit `unit0` of transform `transform` (multi-pass sizes), or over
// `count` whole transforms whose offsets are lane_off[group ..] (single-pass).
struct RaggedItem {
  int plan;
  int pass;
  int count;
  int transform;
  long long unit0;
  long long group;
};
struct RaggedArgs {
  const void* in;
  void* out;
  void* ws;
  long long ws2_off;          // second workspace (three-pass lengths), elements after ws
  const void* tab;
  const RaggedPlan* plans;
  const RaggedItem* items;
  const EngineArgs* ea;       // per (plan, global pass): the engine arguments but the buffers
  const long long* lane_off;  // single-pass groups
  const long long* offset;    // element offset of every transform
  int* done;                  // completed tiles per (transform, pass)
  int* head;                  // queue head
  int* status;
  long long nitems;
  long long spin_limit;
  int conj;
  int lanes_max;              // largest W*Lp of any item (shared buffer size)
};

struct HostPlan {
  long long n = 0;        // complex length of the transform
  long long batch = 1;
  int dbl = 0;            // 1 = FP64, 0 = FP32
  int trans = 0;          // 0 DFT, 1 IDFT, 2 RDFT, 3 IRDFT
  int place = 1;
  int nglobal = 0;
  GlobalPass gp[GFFT_MAXG];
  int real_fused = 0;     // real pre/post pass inside the single global pass
  int dif = 0;            // frequency decimation: global passes run last to first, transposed
  // host copy of the device tables (FP64 values; converted at upload)
  std::size_t tw_count = 0;      // in-block twiddles (complex)
  std::size_t gtw_lo_off = 0, gtw_hi_off = 0, gtw_B = 1;
  std::size_t rtw_off = 0;
  std::size_t ftw_off[GFFT_MAXG] = {0, 0, 0, 0};  // variant-9 four-step factor tables (0: none)
  std::size_t table_count = 0;   // total complex entries
  std::size_t ws_elems = 0;      // workspace, complex elements
  int n_ws = 0;                  // number of workspace buffers (0..2)
};

// planner.cpp
int gfft_plan_build(HostPlan& plan, long long n, long long batch, int dbl, int trans, int place,
                    const PlanOpts& opts);
// Fill `tab` (2*table_count doubles, interleaved) with every table the plan
// references, generated in extended precision and rounded once.
void gfft_plan_tables(const HostPlan& plan, double* tab);
// padded per-unit stride of the run-time engine's shared buffers (variants 1
// and 4, ragged batches): one slot per 2^ps values and one more per
// 2^(ps+4) (engine.cuh pad), ps = 4 for 8-byte and 3 for 16-byte elements
// The stride is odd (in elements) so that the units of a tile, read at one
// sample index, fall on different banks.
inline long long engine_padded(long long L, int dbl) {
  const int ps = dbl ? 3 : 4;
  const long long v = L + (L >> ps) + (L >> (ps + 4)) + 1;
  return v | 1;
}
// true when a power-of-two pass uses the length-specialised kernels' radices
bool spec_radices(const GlobalPass& gp);
