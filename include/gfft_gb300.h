/*
 * gfft_gb300 — C ABI of the GB300 (sm_103a) implementation of GFFT's
 * transform hot path.
 *
 * The reference (scpp/gfft) is a header-only C++ template library with no C
 * ABI: a transform object is made by GFFT::GenerateTransform<...> and looked
 * up by CreateTransformObject(n, vtype_id, trans_id, dim, parall_id,
 * place_id) (src/gfftgen.h:189-231); its fft(T*) / fft(const T*, T*)
 * virtual call (src/gfftpolicy.h:46-58) runs the transform.  The entry points
 * below are what a foreign-function binding of that path needs: plain
 * integers, sizes and pointers, a status code instead of a C++ exception.
 *
 * Conventions (identical to the reference):
 *   - data is interleaved (re, im), contiguous; a COMPLEX_* value type has
 *     the same bytes as the matching real one (std::complex<T>);
 *   - DFT  (trans_id 0) computes X_k = sum_n x_n e^{-2 pi i k n / N};
 *     IDFT (trans_id 1) uses e^{+2 pi i k n / N} and scales by 1/N
 *     (src/gfftspec.h:117-135, src/gfftswap.h:338-374);
 *   - RDFT (trans_id 2) of length n transforms 2n reals into the packed
 *     half spectrum X_0, X_n, X_1 .. X_{n-1}; IRDFT (3) inverts it,
 *     IRDFT(RDFT(x)) = x (src/gfftswap.h:239-287, src/gfftpolicy.h:262-297);
 *   - DCT1 (4) / DCT2 (6) of n reals (value types DOUBLE / FLOAT) compute the
 *     reference's direct sums X_k = sum_{l<n} x_l cos(pi k l / (n - 1)) and
 *     X_k = sum_{l<n} x_l cos(pi k l / n) (src/direct.h:270-312; the
 *     reference's DCT policies, src/gfftpolicy.h:302-365, have no algorithm);
 *     IDCT1 (5) / IDCT2 (7) are the same sums under the reference's Backward
 *     policy, divided by n (src/gfftswap.h:355-361); n >= 2 for types 1;
 *   - value type IDs DOUBLE=0, FLOAT=1, COMPLEX_DOUBLE=2, COMPLEX_FLOAT=3;
 *     place IDs IN_PLACE=0, OUT_OF_PLACE=1; parallel IDs Serial=0,
 *     OpenMP<NT>=NT-1 (src/gfftpolicy.h:78-453).  Every parallel ID maps to
 *     the same batched GPU grid.
 *
 * Beyond the reference: a batch count, in-place composite N, out-of-place and
 * non-power-of-two real transforms, and device-resident execution on a CUDA
 * stream.  Handles are immutable after creation and own their device
 * twiddle tables and workspace; calls on one handle must be serialised on one
 * stream (they share the workspace).
 */
#ifndef GFFT_GB300_H
#define GFFT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gfft_plan* gfft_handle;
typedef struct CUstream_st* gfft_stream; /* a cudaStream_t; NULL = legacy default stream */

/* status codes */
enum {
  GFFT_OK = 0,
  GFFT_E_INVALID_SIZE = 1,      /* n == 0, batch == 0, or a length this build cannot plan */
  GFFT_E_INVALID_TYPE = 2,      /* vtype_id not in {0,1,2,3} */
  GFFT_E_INVALID_TRANSFORM = 3, /* trans_id not in {0 .. 7} */
  GFFT_E_INVALID_PLACE = 4,     /* place_id not in {0,1}, or in place with src != dst */
  GFFT_E_INVALID_DIM = 5,       /* dim / rank not in 1..3 */
  GFFT_E_INVALID_PARALL = 6,    /* parall_id < 0 */
  GFFT_E_NULL_POINTER = 7,
  GFFT_E_MISALIGNED = 8,        /* pointer not aligned to one complex element */
  GFFT_E_ALLOC = 9,             /* device or host allocation failed */
  GFFT_E_CUDA = 10,             /* a CUDA runtime call or launch failed */
  GFFT_E_INVALID_HANDLE = 11,
  GFFT_E_NOT_IN_LIST = 12,      /* size/type not generated by the facade's typelist */
  GFFT_E_TIMEOUT = 13,          /* a bounded device wait ran out (persistent kernels) */
  GFFT_E_INVALID_PLAN = 14,     /* a caller-supplied plan option is inconsistent */
  GFFT_E_TOO_LARGE = 15,        /* request exceeds a fixed capacity of the entry point */
  GFFT_E_BOUNDS = 16            /* debug build: a device-side bounds check failed (the access was skipped) */
};

/* Replaces GenerateTransform<...>::CreateTransformObject(n, vtype_id,
 * trans_id, dim, parall_id, place_id) (src/gfftgen.h:222-231) plus the
 * Transform::Create() it ends in (src/gfftgen.h:81-83).  `n` is the transform
 * length (complex points; for RDFT/IRDFT the complex length of the packed
 * 2n reals; for the cosine transforms the number of reals).  `batch`
 * transforms lie back to back (stride 2n scalars, n for a cosine transform). */
int gfft_create(gfft_handle* handle, uint64_t n, int vtype_id, int trans_id, int dim, int parall_id,
                int place_id, uint64_t batch);

/* Plan options (the autotuner's knobs).  Zero means "planner default". */
typedef struct gfft_plan_opts {
  int radix_order;        /* 0 = default order, 1 = reversed, 2 = odd radices first */
  int max_radix;          /* largest in-block radix: 16, 8, 4 or 2 (0 = 16) */
  int threads_per_block;  /* 32..512, multiple of 32 */
  int units_per_block;    /* transforms (single-pass) or lanes (multi-pass) per block */
  int max_pass_len;       /* cap on one pass's in-block length (forces more passes) */
  int kernel_variant;     /* 0 = auto, 1 = generic engine, 2 = register-resident fast path,
                             3 = the fast path specialised for a power-of-two length,
                             4 = pipelined column tiles (passes of a multi-pass length),
                             5 = column tiles specialised for a power-of-two pass length,
                             6 = split-precision tensor-core form (FP32 complex, power-of-two
                                 passes of 64..4096: radix-16 sub-DFTs as FP16 hi/lo matrix
                                 products accumulated in FP32; used only when requested),
                             7 = column tiles specialised for a mixed-radix pass shape,
                             9 = column tiles moved by 2-D tensor copies (passes of 64..4096
                                 of a multi-pass power-of-two length; device buffers
                                 16-byte aligned, others run through variant 5) */
  int stages;             /* bulk-copy pipeline depth of the pipelined kernels (0 = the planner's
                             choice; FP32 single passes of 4096 / 8192 / 16384 then load straight
                             from global memory, one transform per block, and any explicit depth
                             selects the staged kernel instead) */
  int blocks_per_sm;      /* persistent blocks per SM of the fast path (0 = occupancy); for the
                             tensor-copy column tiles, 1 keeps 64 KB tiles on FP32 passes of
                             128..512 (default there: 32 KB tiles, one stage, two blocks per SM)
                             and 2 extends the 32 KB tiles to FP32 passes of 1024 */
  int decimation;         /* 0 = in time (DIT, default), 1 = in frequency (DIF: the transposed
                             Stockham passes in reverse order, twiddles after the butterflies;
                             the reference's InFreq / T_DFTk_x_Im, src/gfftalgfreq.h:106-432);
                             DIF runs on the generic engine (kernel variant 1) */
  int reserved[3];
} gfft_plan_opts;

int gfft_create_opts(gfft_handle* handle, uint64_t n, int vtype_id, int trans_id, int dim,
                     int parall_id, int place_id, uint64_t batch, const gfft_plan_opts* opts);

/* Multi-dimensional complex DFT / IDFT of `batch` row-major arrays of
 * dims[0] x ... x dims[rank-1] complex points (rank 1..3, the last index
 * fastest).  No reference counterpart: the reference carries a `Dim`
 * parameter (src/gfftgen.h:49, 153-154, 200) but implements only Dim = 1.
 * gfft_create with dim = 2 or 3 builds the n^dim case through this call.
 * Every axis but the last must be at most 4096 (FP32) / 2048 (FP64) points;
 * the last any supported 1-D length.  Execute with gfft_exec /
 * gfft_exec_host; the inverse divides by the product of the dims. */
int gfft_create_nd(gfft_handle* handle, int rank, const uint64_t* dims, int vtype_id, int trans_id, int place_id,
                   uint64_t batch);

/* Replaces AbstractFFT_inp<T>::fft(T*) and AbstractFFT_oop<T>::fft(const T*,
 * T*) (src/gfftpolicy.h:46-58) for DEVICE pointers: in place when
 * src == dst.  Asynchronous on `stream`. */
int gfft_exec(gfft_handle handle, const void* src, void* dst, gfft_stream stream);

/* The same call on HOST pointers (what the reference's fft() receives):
 * copies in, transforms, copies out on `stream` and waits for it. */
int gfft_exec_host(gfft_handle handle, const void* src, void* dst, gfft_stream stream);

/* Replaces `delete obj` of the object Create() returned (src/gfftgen.h:81-83). */
int gfft_destroy(gfft_handle handle);

/* Text of a status code (replaces TransformFactoryError::Exception::what(),
 * src/gfftgen.h:133-145, for GFFT_E_NOT_IN_LIST). */
const char* gfft_strerror(int status);

/* Plan description, for logs and the autotuner (no reference counterpart:
 * the reference's plan is its compile-time factor list, src/gfftfactor.h). */
typedef struct gfft_plan_info {
  uint64_t n, batch;
  int vtype_id, trans_id, place_id;
  int n_global_passes;         /* HBM round trips of the complex transform */
  int pass_len[4];             /* in-block length of each global pass */
  int radices[4][16];          /* in-block radix sequence of each pass (0-terminated) */
  int threads[4], units[4];    /* launch shape of each pass */
  int kernel_variant[4];       /* 1 generic engine, 2 register-resident fast path, 3 specialised,
                                  4 column tiles, 5 specialised column tiles, 6 tensor-core split,
                                  7 specialised mixed-radix column tiles,
                                  9 column tiles moved by 2-D tensor copies */
  uint64_t workspace_bytes;    /* device scratch owned by the handle */
  uint64_t table_bytes;        /* device twiddle tables owned by the handle */
  int real_fused;              /* real pre/post pass fused into the transform */
  int kernels_per_exec;        /* kernel launches of one gfft_exec */
} gfft_plan_info;

int gfft_get_info(gfft_handle handle, gfft_plan_info* info);

/* Plan a transform without creating it (no GPU needed): fills `info` as
 * gfft_get_info would for the same arguments.  No reference counterpart
 * (the reference plans at compile time). */
int gfft_plan_query(uint64_t n, int vtype_id, int trans_id, int place_id, uint64_t batch,
                    const gfft_plan_opts* opts, gfft_plan_info* info);

/* Status word the device code of this handle's kernels writes (a bounded
 * wait that ran out sets GFFT_E_TIMEOUT).  Synchronises the handle's device,
 * returns the word in *status and clears it. */
int gfft_get_device_status(gfft_handle handle, int* status);

/* Self-test of the bounded waits: launches the pipelined kernel with its
 * copies switched off, so that its first wait (limited to `spin_limit`
 * try-wait rounds) runs out; returns the status word it wrote (expected
 * GFFT_E_TIMEOUT) in *status.  No reference counterpart. */
int gfft_selftest_bounded_wait(long long spin_limit, int* status);

/* ---- autotuner and learned cost model -------------------------------------
 * No reference counterpart (the reference's plan is its compile-time factor
 * list, src/gfftfactor.h:160-169).  Candidates are the distinct plans reached
 * through gfft_plan_opts; gfft_tune_measure times each on caller-provided
 * device buffers (exhaustive measured search, `reps` launches each after one
 * warm-up); failed candidates get -1. */
#define GFFT_NFEAT 25
int gfft_tune_candidates(uint64_t n, int vtype_id, int trans_id, int place_id, uint64_t batch,
                         gfft_plan_opts* cands, int max_cands, int* ncands);
int gfft_tune_measure(uint64_t n, int vtype_id, int trans_id, int place_id, uint64_t batch,
                      const gfft_plan_opts* cands, int ncands, const void* d_src, void* d_dst, int reps,
                      float* ms_out);
/* Feature vector (GFFT_NFEAT floats) of the plan these options give:
 * [0] log2 N, [1-4] exponents of 2/3/5/7, [5] log2 batch, [6] FP64, [7]
 * global passes, [8-14] counts of in-block radices 16/8/4/2/3/5/7, [15] mean
 * log2 units per block, [16] log2 longest and [17] shortest pass length,
 * [18-21] passes run by the generic engine / the pipelined single-pass
 * kernels / the prefetching column tiles / the specialised column tiles
 * (variants 5-8), [22] pipeline stages requested, [23] first radix / 16,
 * [24] passes run by the tensor-copy column tiles (variant 9).  No GPU
 * needed. */
int gfft_plan_features(uint64_t n, int vtype_id, int trans_id, int place_id, uint64_t batch,
                       const gfft_plan_opts* opts, float* features);

/* A multi-layer perceptron cost model (FP32, `depth` hidden ReLU layers of
 * `width`, one linear output) trained on the GPU by the library's own
 * forward / backward / Adam kernels. */
typedef struct gfft_mlp gfft_mlp;
int gfft_mlp_create(gfft_mlp** m, int nin, int width, int depth, uint64_t seed);
int gfft_mlp_num_params(gfft_mlp* m);
int gfft_mlp_get_params(gfft_mlp* m, float* params);
int gfft_mlp_set_params(gfft_mlp* m, const float* params);
/* full-batch Adam on the mean squared error; X is n x nin row-major (host) */
int gfft_mlp_train(gfft_mlp* m, const float* X, const float* y, int n, int epochs, float lr, float* final_loss);
int gfft_mlp_predict(gfft_mlp* m, const float* X, int n, float* y_out);
/* gradient of the mean squared error w.r.t. every parameter (for checks) */
int gfft_mlp_gradients(gfft_mlp* m, const float* X, const float* y, int n, float* grad_out, float* loss_out);
int gfft_mlp_destroy(gfft_mlp* m);

/* ---- ragged batches -------------------------------------------------------
 * Transforms of many different lengths in ONE persistent launch driven by a
 * device work queue over (length, pass, tile), replayed from a CUDA graph.
 * Replaces running one reference object per length in turn (objects from
 * GenerateTransform over an NList, src/gfftgen.h:189-231, each fft() call
 * parallelised only inside one transform by the OpenMP policy,
 * src/gfftomp.h:41-189).  Data: the `count` transforms lie back to back in
 * the order of `sizes` (interleaved complex).  DFT (0) or IDFT (1). */
typedef struct gfft_ragged gfft_ragged;

int gfft_ragged_create(gfft_ragged** handle, uint64_t count, const uint64_t* sizes, int vtype_id, int trans_id);
/* The same with a schedule per length: for each of the n_opts lengths
 * opt_lengths[i], opts[i] sets its pass split (max_pass_len), in-block radix
 * order and largest radix, and units per work item (units_per_block: columns
 * of a multi-pass length, transforms of a single-pass group; a power of two
 * within the block's shared memory); other lengths keep the defaults.  The
 * project's autotuner (gfft_gb300.tuner.ragged_schedule) measures candidate
 * schedules of each length inside this kernel and passes the best here.  No
 * reference counterpart (the reference runs one object per length). */
int gfft_ragged_create_opts(gfft_ragged** handle, uint64_t count, const uint64_t* sizes, int vtype_id, int trans_id,
                            uint64_t n_opts, const uint64_t* opt_lengths, const gfft_plan_opts* opts);
/* The schedule a ragged handle uses for length n: passes, radices, units
 * per work item (GFFT_E_INVALID_SIZE when n is not in the batch). */
int gfft_ragged_get_plan(gfft_ragged* handle, uint64_t n, struct gfft_plan_info* info);
/* Device pointers; the launch sequence is captured into a CUDA graph on the
 * first call for a (src, dst) pair and replayed afterwards. */
int gfft_ragged_exec(gfft_ragged* handle, const void* src, void* dst, gfft_stream stream);
int gfft_ragged_get_info(gfft_ragged* handle, uint64_t* total_points, uint64_t* items, int* distinct_lengths,
                         int* max_passes, unsigned* grid);
/* Device status word of the persistent kernel (GFFT_E_TIMEOUT if a bounded
 * wait between passes ran out); synchronises, reads and clears it. */
int gfft_ragged_get_status(gfft_ragged* handle, int* status);
int gfft_ragged_destroy(gfft_ragged* handle);

/* A transform that allocates nothing.  No counterpart in the reference (its
 * transform objects never touch device memory).
 *
 * For callers that cannot call cudaMalloc when they transform: code whose
 * device memory is fixed at start-up (real-time and embedded pipelines), a
 * plugin inside a host application that owns every allocation, or a caller
 * for whom an allocation would synchronise the device at a bad moment.  A
 * handle from gfft_create allocates its twiddle tables and, for lengths that
 * need several passes through HBM, a workspace as large as the data; this
 * entry point keeps both in one fixed device array that the library reserves
 * on every GPU that loads it, held until the process exits, and plans on the
 * stack.
 *
 * Computes the complex DFT (trans_id 0) or IDFT (1) of `batch` transforms of
 * length n from src to dst (device pointers; in place when src == dst) on
 * `stream`.  Limits: n * batch * element size <= 64 MiB (32 MiB when an odd
 * number of passes runs in place: two workspaces), twiddle tables <= 1 MiB;
 * larger requests return GFFT_E_TOO_LARGE, real transforms
 * GFFT_E_INVALID_TRANSFORM.
 *
 * The first call on a device looks up the array's address with
 * cudaGetSymbolAddress (the device must be current).  Under CUDA's lazy
 * module loading that lookup is also what loads this code onto the device
 * and reserves the array (about 65 MiB), and it may synchronise the device:
 * make one warm-up call at start-up, before any stream capture.  All calls share the one array and leave their
 * data in it: nothing needs clearing (each call writes what it reads), but
 * calls that overlap on the GPU -- on two streams, or from two threads
 * without ordering -- race on it and must be serialised by the caller. */
int gfft_exec_noalloc(uint64_t n, int vtype_id, int trans_id, uint64_t batch, const void* src, void* dst,
                      gfft_stream stream);

/* Multiply-add throughput of the CUDA cores in GFLOP/s (2 flops per FMA),
 * FP64 (dbl = 1) or FP32: eight independent chains per thread over every
 * SM, best of five launches of `iters` iterations, CUDA events.  The FP64
 * figure bounds the FP64 transforms (FP64 is a small fraction of GB300's
 * FP32 rate).  No reference counterpart (its harness reports
 * 5 N log2 N / t only, test/gfft_performance.h:67-78). */
int gfft_measure_fma_peak(int dbl, int iters, double* gflops, double* ms);

/* 1 for the debug build of the library (compiled with -DGFFT_DEBUG: every
 * checked shared- and global-memory index of the column-tile and engine
 * kernels is tested before the access; a failing check skips the access and
 * leaves GFFT_E_BOUNDS, read by gfft_get_device_status), else 0.  No
 * reference counterpart (its only guards are an assert and a comment). */
int gfft_debug_build(void);
/* Debug build: runs one failing check in a one-thread kernel (no memory
 * access behind it) and returns the status words it left: GFFT_E_BOUNDS and
 * the source line.  Release build: GFFT_E_INVALID_PLAN. */
int gfft_selftest_bounds_check(int* status, int* line);

/* Library version string. */
const char* gfft_version(void);

#ifdef __cplusplus
}
#endif

#endif /* GFFT_GB300_H */
