// gfft_exec_noalloc: the multi-pass transform without any allocation.
//
// Who needs this: code that must not allocate device memory at the moment it
// transforms -- a real-time or embedded caller whose memory is fixed at
// start-up, a plugin that runs inside a host application that owns every
// allocation (and may forbid cudaMalloc on its threads), or a caller in the
// middle of an allocator-sensitive phase where a cudaMalloc would
// synchronise the device.  gfft_create/gfft_exec cannot serve them: a handle
// allocates its twiddle tables and, for lengths that take several passes
// through HBM, a workspace as large as the data.
//
// Here both live in one file-scope device array, sized once for the life of
// the process: every GPU that loads this library reserves it when the
// library's code is loaded on that device and keeps it until exit.  The
// entry point plans on the stack, computes the twiddles into the array with a
// small kernel, and runs the same Stockham engine kernel as gfft_exec with
// the array as its workspace.  It calls no cudaMalloc / cudaFree and no
// allocating library routine (no C++ containers, no torch).
//
// Limits: complex DFT / IDFT only; n * batch * element size must fit the
// workspace part of the array (64 MiB, or 32 MiB when an odd number of
// passes runs in place, which takes two workspaces), and the tables must fit
// 1 MiB.  Larger requests return GFFT_E_TOO_LARGE.
//
// Sharing: every call uses the same array and leaves its contents behind.
// Nothing in it has to start at zero -- each call writes every byte it reads
// before reading it -- but two calls that overlap on the GPU (different
// streams, or different host threads without ordering) race on it.
//
// Set-up: the first call on each device (with that device current) looks up
// the array's device address with cudaGetSymbolAddress and sets the engine
// kernel's shared-memory limit.  With CUDA's lazy module loading (the
// default), that lookup is what loads this translation unit's module on the
// device and reserves the array (about 65 MiB), and it may synchronise the
// device; callers make one warm-up call at start-up, before any stream
// capture on that device.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>

#include "../../include/gfft_gb300.h"
#include "handle.h"
#include "plan.h"

extern "C" int gfft_engine_setup(int dbl, size_t max_smem);

#define GFFT_NOALLOC_WS_BYTES (64ull << 20)
#define GFFT_NOALLOC_TAB_BYTES (1ull << 20)
#define GFFT_NOALLOC_MAX_DEVICES 64

// [0, TAB) twiddle tables | [TAB, TAB + 256) status word | then the workspace
static __device__ __align__(256) unsigned char g_noalloc_scratch[GFFT_NOALLOC_TAB_BYTES + 256 + GFFT_NOALLOC_WS_BYTES];

namespace {

std::mutex g_mu;
void* g_base[GFFT_NOALLOC_MAX_DEVICES];
bool g_ready[GFFT_NOALLOC_MAX_DEVICES];

// ---- planning on the stack (the planner's default rules, engine kernel) --
struct Factors {
  long long p[64];
  int n = 0;
};

bool factorize(long long n, Factors& f) {
  for (long long p = 2; p * p <= n; p += (p == 2 ? 1 : 2))
    while (n % p == 0) {
      if (f.n == 64) return false;
      f.p[f.n++] = p;
      n /= p;
    }
  if (n > 1) {
    if (f.n == 64) return false;
    f.p[f.n++] = n;
  }
  return true;
}

int block_radices(int L, int* out) {
  int a = 0, m = L, k = 0;
  while (m % 2 == 0) {
    m /= 2;
    ++a;
  }
  int q = a / 4, rem = a % 4;
  for (int i = 0; i < q; ++i) out[k++] = 16;
  if (rem == 1 && q >= 1) {
    out[k - 1] = 8;
    out[k++] = 4;
  } else if (rem) {
    out[k++] = 1 << rem;
  }
  for (int p : {7, 5, 3})
    while (m % p == 0) {
      if (k == GFFT_MAXP) return -1;
      m /= p;
      out[k++] = p;
    }
  Factors f;
  if (!factorize(m, f)) return -1;
  for (int i = 0; i < f.n; ++i) {
    if (k == GFFT_MAXP) return -1;
    out[k++] = (int)f.p[i];
  }
  return k;
}

bool split_passes(long long N, int P, long long cap, long long* g) {
  Factors f;
  if (!factorize(N, f)) return false;
  for (int i = 0; i < P; ++i) g[i] = 1;
  for (int i = f.n - 1; i >= 0; --i) {  // largest prime first
    int best = -1;
    for (int j = 0; j < P; ++j)
      if (g[j] * f.p[i] <= cap && (best < 0 || g[j] < g[best])) best = j;
    if (best < 0) return false;
    g[best] *= f.p[i];
  }
  for (int i = 0; i < P; ++i)  // descending
    for (int j = i + 1; j < P; ++j)
      if (g[j] > g[i]) {
        long long t = g[i];
        g[i] = g[j];
        g[j] = t;
      }
  return true;
}

int round32(long long x) { return (int)((x < 32 ? 32 : (x + 31) / 32 * 32)); }

// fills hp like gfft_plan_build for a complex transform on the engine kernel
bool plan(HostPlan& hp, long long n, long long batch, int dbl, int trans, int place) {
  hp.n = n;
  hp.batch = batch;
  hp.dbl = dbl;
  hp.trans = trans;
  hp.place = place;
  const long long esz = dbl ? 16 : 8;
  auto padded = [&](long long L) { return engine_padded(L, dbl); };  // the engine kernel's stride
  const long long budget = 160 * 1024;
  const long long cap1 = dbl ? 4096 : 8192;
  const int lane_w = dbl ? 4 : 8;
  long long capL = 1;
  while (2 * lane_w * padded(capL * 2) * esz <= budget) capL *= 2;
  long long Ls[GFFT_MAXG];
  int P = 0;
  if (n <= cap1) {
    Ls[0] = n;
    P = 1;
  } else {
    for (int q = 2; q <= GFFT_MAXG && !P; ++q)
      if (split_passes(n, q, capL, Ls)) P = q;
    if (!P) return false;
  }
  hp.nglobal = P;
  size_t tw = 0;
  long long Ns = 1;
  for (int g = 0; g < P; ++g) {
    GlobalPass& gp = hp.gp[g];
    gp.L = (int)Ls[g];
    gp.Ns = Ns;
    gp.mode = P == 1 ? 0 : 1;
    int rs[GFFT_MAXP];
    const int np = block_radices(gp.L, rs);
    if (np < 0) return false;
    gp.npass = np;
    int bNs = 1;
    for (int i = 0; i < np; ++i) {
      gp.pass[i].R = rs[i];
      gp.pass[i].Ns = bNs;
      gp.pass[i].tw = (int)tw;
      gp.pass[i].gen = -1;
      tw += (size_t)(rs[i] - 1) * bNs;
      bNs *= rs[i];
    }
    for (int i = 0; i < np; ++i) {
      const int R = rs[i];
      if (!(R == 2 || R == 3 || R == 4 || R == 5 || R == 7 || R == 8 || R == 16)) {
        gp.pass[i].gen = (int)tw;
        tw += R;
      }
    }
    if (gp.mode == 0) {
      long long W = (dbl ? 2048 : 4096) / gp.L;
      if (W < 1) W = 1;
      if (W > batch) W = batch;
      while (W > 1 && 2 * W * padded(gp.L) * esz > budget) --W;
      gp.units = (int)W;
    } else {
      const long long stride = n / gp.L;
      long long W = 1;
      while (W * 2 <= (stride < lane_w ? stride : lane_w)) W *= 2;
      gp.units = (int)W;
    }
    long long el = (long long)gp.units * gp.L / 16;
    gp.threads = round32(el < 64 ? 64 : (el > 512 ? 512 : el));
    gp.variant = 1;
    gp.smem = (size_t)(2LL * gp.units * padded(gp.L) * esz);
    Ns *= gp.L;
  }
  hp.tw_count = tw;
  size_t off = tw;
  if (P > 1) {
    long long B = 1;
    while (B * B < n) B *= 2;
    hp.gtw_B = (size_t)B;
    hp.gtw_lo_off = off;
    off += (size_t)B;
    hp.gtw_hi_off = off;
    off += (size_t)((n + B - 1) / B);
  }
  hp.table_count = off;
  if (P >= 2) {
    hp.ws_elems = (size_t)(n * batch);
    hp.n_ws = (P % 2 == 1 && place == 0) ? 2 : 1;
  }
  return true;
}

// ---- twiddles computed on the device into the array -------------------
struct Seg {
  long long off, M, mul, count;
  int kind, Ns;  // kind 0: in-block pass table, 1: W_M^(m*mul) for m < count
};
struct SegList {
  Seg s[96];
  int n;
  int dbl;
};

__global__ void fill_tables(const __grid_constant__ SegList L) {
  for (int si = 0; si < L.n; ++si) {
    const Seg g = L.s[si];
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < g.count;
         e += (long long)gridDim.x * blockDim.x) {
      long long j;
      if (g.kind == 0) {
        const long long r = e / g.Ns + 1, k = e % g.Ns;
        j = (k * r) % g.M;
      } else {
        j = (e * g.mul) % g.M;
      }
      double s, c;
      sincospi(-2.0 * (double)j / (double)g.M, &s, &c);
      if (L.dbl) {
        double2* t = reinterpret_cast<double2*>(g_noalloc_scratch) + g.off + e;
        *t = make_double2(c, s);
      } else {
        float2* t = reinterpret_cast<float2*>(g_noalloc_scratch) + g.off + e;
        *t = make_float2((float)c, (float)s);
      }
    }
  }
}

int setup_device(void** base) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return GFFT_E_CUDA;
  if (dev < 0 || dev >= GFFT_NOALLOC_MAX_DEVICES) return GFFT_E_CUDA;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_ready[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) return GFFT_E_CUDA;
    int maxopt = 0;
    if (cudaDeviceGetAttribute(&maxopt, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
      return GFFT_E_CUDA;
    if (gfft_engine_setup(0, (size_t)maxopt) != 0 || gfft_engine_setup(1, (size_t)maxopt) != 0) return GFFT_E_CUDA;
    g_base[dev] = p;
    g_ready[dev] = true;
  }
  *base = g_base[dev];
  return GFFT_OK;
}

}  // namespace

extern "C" int gfft_exec_noalloc(uint64_t n, int vtype_id, int trans_id, uint64_t batch, const void* src, void* dst,
                                 gfft_stream stream) {
  if (vtype_id < 0 || vtype_id > 3) return GFFT_E_INVALID_TYPE;
  if (trans_id != 0 && trans_id != 1) return GFFT_E_INVALID_TRANSFORM;
  if (n == 0 || batch == 0) return GFFT_E_INVALID_SIZE;
  if (!src || !dst) return GFFT_E_NULL_POINTER;
  const int dbl = (vtype_id == 0 || vtype_id == 2) ? 1 : 0;
  const uint64_t esz = dbl ? 16 : 8;
  if (((uintptr_t)src % esz) || ((uintptr_t)dst % esz)) return GFFT_E_MISALIGNED;
  if (n > (GFFT_NOALLOC_WS_BYTES / esz) || batch > (GFFT_NOALLOC_WS_BYTES / esz) / n) return GFFT_E_TOO_LARGE;
  const int place = (src == dst) ? 0 : 1;
  gfft_plan h;  // on the stack: no handle allocation
  if (!plan(h.hp, (long long)n, (long long)batch, dbl, trans_id, place)) return GFFT_E_INVALID_SIZE;
  const uint64_t ws_need = (uint64_t)h.hp.ws_elems * esz * (uint64_t)h.hp.n_ws;
  if (ws_need > GFFT_NOALLOC_WS_BYTES) return GFFT_E_TOO_LARGE;
  if ((uint64_t)h.hp.table_count * esz > GFFT_NOALLOC_TAB_BYTES) return GFFT_E_TOO_LARGE;
  void* base = nullptr;
  int st = setup_device(&base);
  if (st != GFFT_OK) return st;
  unsigned char* b = (unsigned char*)base;

  SegList sl;
  std::memset(&sl, 0, sizeof(sl));
  sl.dbl = dbl;
  for (int g = 0; g < h.hp.nglobal; ++g)
    for (int i = 0; i < h.hp.gp[g].npass; ++i) {
      const BlockPass& p = h.hp.gp[g].pass[i];
      if (sl.n + 4 > 96) return GFFT_E_TOO_LARGE;
      if (p.Ns > 1) sl.s[sl.n++] = Seg{p.tw, (long long)p.Ns * p.R, 1, (long long)(p.R - 1) * p.Ns, 0, p.Ns};
      if (p.gen >= 0) sl.s[sl.n++] = Seg{p.gen, p.R, 1, p.R, 1, 1};
    }
  if (h.hp.nglobal > 1) {
    const long long B = (long long)h.hp.gtw_B;
    sl.s[sl.n++] = Seg{(long long)h.hp.gtw_lo_off, (long long)n, 1, B, 1, 1};
    sl.s[sl.n++] = Seg{(long long)h.hp.gtw_hi_off, (long long)n, B, ((long long)n + B - 1) / B, 1, 1};
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (sl.n > 0) {
    cudaGetLastError();  // clear a stale error of an earlier, unrelated call
    fill_tables<<<64, 256, 0, s>>>(sl);
    if (cudaGetLastError() != cudaSuccess) return GFFT_E_CUDA;
  }
  h.vtype = vtype_id;
  h.d_tab = b;
  h.tab_bytes = GFFT_NOALLOC_TAB_BYTES;
  h.d_status = reinterpret_cast<int*>(b + GFFT_NOALLOC_TAB_BYTES);
  h.ws_bytes = (size_t)h.hp.ws_elems * esz;
  void* ws0 = b + GFFT_NOALLOC_TAB_BYTES + 256;
  void* ws1 = h.hp.n_ws > 1 ? (unsigned char*)ws0 + h.ws_bytes : nullptr;
  h.d_ws[0] = ws0;
  h.d_ws[1] = ws1;
  return gfft_exec_ws(&h, src, dst, s, ws0, ws1);
}
