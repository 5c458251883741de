// Host planner: the run-time replacement for the reference's compile-time
// factorisation and twiddle generation.
//
//  - The reference factorises N at compile time into ascending primes
//    (Factorize, src/gfftfactor.h:160-169) and recurses one prime per level
//    (InTimeOOP, src/gfftalg.h:459-507).  Here N is split into 1..4 global
//    passes ("super-radices" that fit one thread block) and each of those into
//    in-block Stockham radices {16, 8, 4, 2, 7, 5, 3} plus a generic odd
//    prime, so a power of two uses radix 16 instead of radix 2.
//  - The reference computes the first root of each level from compile-time
//    decimal series (GetFirstRoot, src/metaroot.h:104-120) and every other
//    twiddle by a run-time complex recurrence (ComputeRoots,
//    src/twiddles.h:234-339; radix 2 in the working type, src/gfftalg.h:
//    249-265).  Here every twiddle is computed directly in extended precision
//    with exact integer angle reduction and rounded once to the working type,
//    so there is no recurrence error.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <vector>

#include "mixed_shapes.h"
#include "colshape.h"
#include "plan.h"

bool spec_radices(const GlobalPass& gp);
// fft_col.cu: launch shape of the tensor-copy column tiles (variant 9)
extern "C" int gfft_col_shape(int dbl, int L, int stages, int rf, int tk, int* units, int* threads, size_t* smem);
extern "C" int gfft_colmix_shape(int dbl, int L, const int* rs, int np, int stages, int gather, int* units,
                                 int* threads, size_t* smem);

namespace {

struct PF {
  long long p;
  int k;
};

std::vector<PF> factorize(long long n) {
  std::vector<PF> f;
  for (long long p = 2; p * p <= n; p += (p == 2 ? 1 : 2)) {
    int k = 0;
    while (n % p == 0) {
      n /= p;
      ++k;
    }
    if (k) f.push_back({p, k});
  }
  if (n > 1) f.push_back({n, 1});
  return f;
}

// cos and sin of 2*pi*j/m in long double, j reduced exactly and folded into
// the first octant before the library call.
void root(long long j, long long m, long double* c, long double* s) {
  j %= m;
  if (j < 0) j += m;
  const long double PI4 = 0.785398163397448309615660845819875721L;
  // angle = 2*pi*j/m = (8j/m) * pi/4
  __int128 e = (__int128)8 * j;
  long long oct = (long long)(e / m);
  long long r = (long long)(e - (__int128)oct * m);
  bool flip = oct & 1;
  long double a = flip ? (long double)(m - r) / (long double)m * PI4 : (long double)r / (long double)m * PI4;
  long double ca = cosl(a), sa = sinl(a), cc, ss;
  switch (oct) {
    case 0: cc = ca; ss = sa; break;
    case 1: cc = sa; ss = ca; break;
    case 2: cc = -sa; ss = ca; break;
    case 3: cc = -ca; ss = sa; break;
    case 4: cc = -ca; ss = -sa; break;
    case 5: cc = -sa; ss = -ca; break;
    case 6: cc = sa; ss = -ca; break;
    default: cc = ca; ss = -sa; break;
  }
  *c = cc;
  *s = ss;
}

// forward root W_m^j = exp(-2 pi i j / m)
void wroot(long long j, long long m, double* re, double* im) {
  long double c, s;
  root(j, m, &c, &s);
  *re = (double)c;
  *im = (double)(-s);
}

// radices with a register butterfly (butterflies.cuh); any other prime runs
// the generic O(R^2) pass with its own root table
bool native_radix(int R) {
  switch (R) {
    case 2: case 3: case 4: case 5: case 6: case 7: case 8: case 9: case 10: case 12: case 15: case 16: return true;
    default: return false;
  }
}

// The fewest in-block passes for L = 2^a 3^b 5^c 7^d out of the register
// butterflies {16, 15, 12, 10, 9, 8, 7, 6, 5, 4, 3, 2}; among equally short
// sequences the one with the larger radices first (descending comparison).
// Returned largest first.
std::vector<int> group_radices(int a, int b, int c, int d) {
  static const int R[12] = {16, 15, 12, 10, 9, 8, 7, 6, 5, 4, 3, 2};
  static const int E[12][4] = {{4, 0, 0, 0}, {0, 1, 1, 0}, {2, 1, 0, 0}, {1, 0, 1, 0}, {0, 2, 0, 0}, {3, 0, 0, 0},
                               {0, 0, 0, 1}, {1, 1, 0, 0}, {0, 0, 1, 0}, {2, 0, 0, 0}, {0, 1, 0, 0}, {1, 0, 0, 0}};
  std::map<std::array<int, 4>, std::vector<int>> memo;
  std::function<std::vector<int>(std::array<int, 4>)> best = [&](std::array<int, 4> e) -> std::vector<int> {
    if (e[0] == 0 && e[1] == 0 && e[2] == 0 && e[3] == 0) return {};
    auto it = memo.find(e);
    if (it != memo.end()) return it->second;
    std::vector<int> out;
    bool have = false;
    for (int i = 0; i < 12; ++i) {
      std::array<int, 4> r = e;
      bool ok = true;
      for (int k = 0; k < 4; ++k) ok = ok && (r[k] -= E[i][k]) >= 0;
      if (!ok) continue;
      std::vector<int> cand = best(r);
      cand.push_back(R[i]);
      std::sort(cand.rbegin(), cand.rend());
      if (!have || cand.size() < out.size() || (cand.size() == out.size() && cand > out)) {
        out = cand;
        have = true;
      }
    }
    memo[e] = out;
    return out;
  };
  return best({a, b, c, d});
}

std::vector<int> block_radices(int L, const PlanOpts& o) {
  std::vector<int> pow2, odd, gen;
  int a = 0;
  int m = L;
  while (m % 2 == 0) {
    m /= 2;
    ++a;
  }
  if (m > 1 && o.max_radix >= 16) {
    // mixed radix with the default radix cap: composite butterflies
    int e[3] = {0, 0, 0};
    const int pr[3] = {3, 5, 7};
    int rest = m;
    for (int i = 0; i < 3; ++i)
      while (rest % pr[i] == 0) {
        rest /= pr[i];
        ++e[i];
      }
    std::vector<int> seq = group_radices(a, e[0], e[1], e[2]);
    for (const PF& f : factorize(rest))
      for (int i = 0; i < f.k; ++i) gen.push_back((int)f.p);
    if (o.radix_order == 2) {  // odd radices (and generic primes) first
      std::vector<int> oddf, evenf;
      for (int r : seq) (r % 2 ? oddf : evenf).push_back(r);
      seq = gen;
      seq.insert(seq.end(), oddf.begin(), oddf.end());
      seq.insert(seq.end(), evenf.begin(), evenf.end());
    } else {
      seq.insert(seq.end(), gen.begin(), gen.end());
      if (o.radix_order == 1) std::reverse(seq.begin(), seq.end());
    }
    return seq;
  }
  int mr = o.max_radix;
  int lg = mr >= 16 ? 4 : mr >= 8 ? 3 : mr >= 4 ? 2 : 1;
  int q = a / lg, rem = a % lg;
  for (int i = 0; i < q; ++i) pow2.push_back(1 << lg);
  if (rem) {
    if (lg == 4 && rem == 1 && q >= 1) {
      pow2.pop_back();
      pow2.push_back(8);
      pow2.push_back(4);
    } else {
      pow2.push_back(1 << rem);
    }
  }
  for (long long p : {7LL, 5LL, 3LL}) {
    while (m % p == 0) {
      m /= (int)p;
      odd.push_back((int)p);
    }
  }
  for (const PF& f : factorize(m))
    for (int i = 0; i < f.k; ++i) gen.push_back((int)f.p);
  std::vector<int> seq;
  if (o.radix_order == 2) {
    seq.insert(seq.end(), gen.begin(), gen.end());
    seq.insert(seq.end(), odd.begin(), odd.end());
    seq.insert(seq.end(), pow2.begin(), pow2.end());
  } else {
    seq.insert(seq.end(), pow2.begin(), pow2.end());
    seq.insert(seq.end(), odd.begin(), odd.end());
    seq.insert(seq.end(), gen.begin(), gen.end());
    if (o.radix_order == 1) std::reverse(seq.begin(), seq.end());
  }
  return seq;
}

// split N into `P` factors, each <= cap, balanced in log; false if impossible
bool split_passes(long long N, int P, long long cap, std::vector<long long>& out) {
  std::vector<long long> primes;
  for (const PF& f : factorize(N))
    for (int i = 0; i < f.k; ++i) primes.push_back(f.p);
  std::sort(primes.rbegin(), primes.rend());
  std::vector<long long> g(P, 1);
  for (long long p : primes) {
    int best = -1;
    for (int i = 0; i < P; ++i)
      if (g[i] * p <= cap && (best < 0 || g[i] < g[best])) best = i;
    if (best < 0) return false;
    g[best] *= p;
  }
  std::sort(g.rbegin(), g.rend());
  out = g;
  return true;
}

int round32(long long x) { return (int)std::max<long long>(32, (x + 31) / 32 * 32); }

}  // namespace

// The in-block radices of the length-specialised kernels for a power-of-two
// L: radix 16 while four bits remain, the remainder as 8 x 4 (one bit), 4 or
// 8 (fft_spec.cu, spec.cuh radix_of).
bool spec_radices(const GlobalPass& gp) {
  int lg = 0;
  while ((1LL << lg) < gp.L) ++lg;
  if ((1LL << lg) != gp.L || lg < 4) return false;
  std::vector<int> want((std::size_t)(lg / 4), 16);
  if (lg % 4 == 1) {
    want.back() = 8;
    want.push_back(4);
  } else if (lg % 4) {
    want.push_back(1 << (lg % 4));
  }
  bool ok = (int)want.size() == gp.npass;
  for (int i = 0; i < gp.npass && ok; ++i) ok = gp.pass[i].R == want[(std::size_t)i];
  return ok;
}


int gfft_plan_build(HostPlan& plan, long long n, long long batch, int dbl, int trans, int place,
                    const PlanOpts& opts) {
  if (n < 1 || batch < 1) return 1;
  plan = HostPlan();
  plan.n = n;
  plan.batch = batch;
  plan.dbl = dbl;
  plan.trans = trans;
  plan.place = place;
  PlanOpts o = opts;
  if (o.max_radix <= 0) o.max_radix = 16;
  // frequency decimation runs on the generic engine
  if (o.dif) o.variant = 1;
  plan.dif = o.dif ? 1 : 0;

  const int esz = dbl ? 16 : 8;
  const int pad_shift = dbl ? 3 : 4;
  const long long smem_budget = o.smem_budget > 0 ? o.smem_budget : 160 * 1024;
  auto padded = [&](long long L) { return L + (L >> pad_shift) + 1; };  // spec / fast kernels
  auto epadded = [&](long long L) { return engine_padded(L, dbl); };     // run-time engine kernels
  // largest single-pass length: two padded buffers of one transform
  long long cap1 = dbl ? 4096 : 8192;
  if (o.max_pass_len > 0) cap1 = std::min<long long>(cap1, o.max_pass_len);
  if (o.max_single > 0) cap1 = std::min<long long>(cap1, o.max_single);
  int lane_w = o.units > 0 ? o.units : (dbl ? 4 : 8);  // 64-byte rows
  if (lane_w > 32) lane_w = 32;
  long long capL = 1;
  while (2 * lane_w * epadded(capL * 2) * esz <= smem_budget) capL *= 2;
  if (o.max_pass_len > 0) capL = std::min<long long>(capL, o.max_pass_len);

  // tensor-copy column tiles (fft_col.cu, variant 9): multi-pass power-of-two
  // lengths with the default radices; passes of 64 .. 2048 (FP32 up to 4096
  // when max_pass_len asks for it: two passes for 2^23 / 2^24, whose
  // 4096-point pass has rows of only two units)
  // (power-of-two passes of other lengths too: 3 * 2^18 = 1024 x 768 runs
  // its 1024-point pass here and its 768-point pass on the mixed-radix tiles)
  const bool pow2n = (n & (n - 1)) == 0;
  const bool col_ok = n < (1LL << 32) && (o.variant == 0 || o.variant == 9) && o.threads == 0 && o.units == 0 &&
                      o.radix_order == 0 && o.max_radix == 16 && o.max_single == 0 && o.smem_budget == 0;
  const long long col_max = dbl ? 2048 : 4096;
  long long col_cap = 2048;
  if (o.max_pass_len > 0) col_cap = std::min<long long>(o.max_pass_len, col_max);

  // FP32 16384 in one pass (fft_spec.cu spec_direct_kernel: one transform
  // per 1024-thread block, loaded straight from global memory) with the
  // default radices and kernels
  const bool direct16k = !dbl && n == 16384 && trans < 2 && (o.variant == 0 || o.variant == 3) &&
                         o.radix_order == 0 && o.max_radix == 16 && o.units == 0 && o.threads == 0 &&
                         (o.max_pass_len == 0 || o.max_pass_len >= 16384) && o.max_single == 0 &&
                         o.smem_budget == 0 && o.stages == 0 && o.bps == 0 && !o.dif;
  if (direct16k) cap1 = 16384;
  std::vector<long long> Ls;
  if (n <= cap1) {
    Ls.push_back(n);
  } else {
    bool ok = false;
    if (col_ok && pow2n && col_cap >= 64) {
      for (int P = 2; P <= GFFT_MAXG && !ok; ++P) ok = split_passes(n, P, col_cap, Ls) && Ls.back() >= 64;
    }
    for (int P = 2; P <= GFFT_MAXG && !ok; ++P) ok = split_passes(n, P, capL, Ls);
    if (!ok) return 1;  // a prime factor larger than one block can hold
  }
  plan.nglobal = (int)Ls.size();
  std::size_t tw = 0;
  long long Ns = 1;
  for (int g = 0; g < plan.nglobal; ++g) {
    GlobalPass& gp = plan.gp[g];
    gp.L = (int)Ls[g];
    gp.Ns = Ns;
    gp.mode = plan.nglobal == 1 ? 0 : 1;
    std::vector<int> rs = block_radices(gp.L, o);
    if ((int)rs.size() > GFFT_MAXP) return 1;
    const std::size_t tw0 = tw;  // this pass's twiddles start here
    // the in-block passes of radix sequence `seq` and their twiddle offsets
    auto assign = [&](const std::vector<int>& seq) {
      tw = tw0;
      gp.npass = (int)seq.size();
      int bNs = 1;
      for (int i = 0; i < gp.npass; ++i) {
        BlockPass& bp = gp.pass[i];
        bp.R = seq[(std::size_t)i];
        bp.Ns = bNs;
        bp.tw = (int)tw;
        bp.gen = -1;
        tw += (std::size_t)(bp.R - 1) * bNs;
        bNs *= bp.R;
      }
      for (int i = 0; i < gp.npass; ++i) {
        BlockPass& bp = gp.pass[i];
        if (!native_radix(bp.R)) {
          bp.gen = (int)tw;
          tw += bp.R;
        }
      }
    };
    assign(rs);
    if (gp.mode == 0) {
      long long target = dbl ? 2048 : 4096;  // elements per block
      int W = o.units > 0 ? o.units : (int)std::max<long long>(1, target / gp.L);
      W = (int)std::min<long long>(W, batch);
      while (W > 1 && 2LL * W * epadded(gp.L) * esz > smem_budget) --W;
      gp.units = W;
    } else {
      // lane units: a power of two that divides the block (each thread keeps one lane)
      long long stride = n / gp.L;
      long long W = 1;
      while (W * 2 <= std::min<long long>(lane_w, stride)) W *= 2;
      gp.units = (int)W;
    }
    long long elems = (long long)gp.units * gp.L;
    int thr = o.threads > 0 ? o.threads : round32(std::min<long long>(512, std::max<long long>(64, elems / 16)));
    gp.threads = thr;
    gp.variant = 1;
    gp.smem = (size_t)(2LL * gp.units * epadded(gp.L) * esz);
    const int eng_units = gp.units, eng_threads = gp.threads;
    const size_t eng_smem = gp.smem;
    // register-resident TMA-pipelined path: power-of-two single pass whose
    // radices divide 16, 16 values per thread
    bool pow2ok = gp.mode == 0 && trans < 2 && gp.L >= 16 && (gp.L & (gp.L - 1)) == 0 && o.variant != 1;
    for (int i = 0; i < gp.npass && pow2ok; ++i) pow2ok = (16 % gp.pass[i].R) == 0;
    if (pow2ok) {
      long long target = 4096 * 8 / esz;  // ~32 KB tiles
      int W = o.units > 0 ? o.units : (int)std::max<long long>(1, target / gp.L);
      W = (int)std::min<long long>(W, batch);
      while (W > 1 && (long long)W * gp.L / 16 > 512) --W;
      // threads = W*L/16 must be a whole number of warps
      while (W > 1 && ((long long)W * gp.L / 16) % 32 != 0) --W;
      const long long T = (long long)W * gp.L / 16;
      const long long tile = (long long)W * gp.L * esz;
      if (T >= 32 && T % 32 == 0 && T <= 512 && tile % 16 == 0) {
        // one stage (FP32): the next tile's copy overlaps the passes after the
        // first; measured 1-3 % faster than two at L = 64 .. 4096
        int S = o.stages > 0 ? o.stages : (dbl ? 2 : 1);
        // keep the block within the opt-in shared memory of one SM
        while (S > 1 && S * ((tile + 127) & ~127LL) + W * padded(gp.L) * esz + 8 * S > 220 * 1024) --S;
        gp.variant = 2;
        gp.units = W;
        gp.threads = (int)T;
        gp.stages = S;
        gp.tile_bytes = (int)tile;
        gp.ntiles = (batch + W - 1) / W;
        const long long tb_al = (tile + 127) & ~127LL;
        gp.smem = (size_t)(S * tb_al + ((W * padded(gp.L) * esz + 7) & ~7LL) + 8 * S);
      }
    }
    // pipelined column tiles for the passes of a multi-pass length
    if (gp.mode == 1 && (o.variant == 0 || o.variant == 4) && o.threads == 0) {
      const long long TILE = dbl ? 2048 : 4096;
      const long long stride = n / gp.L;
      long long W = 1;
      if (o.units > 0) {  // requested lane width (a power of two), within 3 buffers of 64 KB
        while (W * 2 <= o.units && W * 2 <= stride && 3 * W * 2 * epadded(gp.L) * esz <= 200 * 1024) W *= 2;
      } else {
        while (W * 2 * gp.L <= TILE && W * 2 <= stride && W * 2 <= 8) W *= 2;
      }
      if (3 * W * epadded(gp.L) * esz <= 200 * 1024) {
        gp.variant = 4;
        gp.units = (int)W;
        gp.threads = dbl ? 256 : 512;  // fft_lane.cu LaneCfg
        gp.ntiles = (batch * stride + W - 1) / W;
        gp.smem = (size_t)(3 * W * epadded(gp.L) * esz);  // prefetch buffer + ping-pong pair
      }
    }
    // column tiles with the length-specialised passes: power-of-two L in
    // 64..1024 with the default radix order; every tile of W = tile / L lanes
    // lies inside one transform (n a multiple of the tile) and the twiddle
    // exponents fit 32 bits
    const long long TILE = dbl ? 2048 : 4096;
    if (gp.mode == 1 && (o.variant == 0 || o.variant == 5) && o.threads == 0 && o.units == 0 &&
        o.radix_order == 0 && o.max_radix == 16 && gp.L >= 64 && gp.L <= 1024 && (gp.L & (gp.L - 1)) == 0 &&
        n % TILE == 0 && n < (1LL << 31)) {
      if (spec_radices(gp)) {
        const long long W = TILE / gp.L;
        gp.variant = 5;
        gp.units = (int)W;
        gp.threads = (int)(TILE / 16);
        gp.ntiles = (batch * (n / gp.L)) / W;
        gp.smem = (size_t)(2 * W * padded(gp.L) * esz);  // current tile + the next one's gather
      }
    }
    // compile-time mixed-radix column tiles (fft_mixed.cu) for the shapes of
    // mixed_shapes.h: passes of a multi-pass length, or single-pass complex
    // lengths (stride 1); every lane finds its own transform and column, so
    // a tile may span transforms
    if ((o.variant == 0 || o.variant == 7) && o.threads == 0 && o.units == 0 && gp.variant != 5 &&
        gp.variant != 3 && gp.variant != 2 && (gp.mode == 1 || trans < 2) && n < (1LL << 31)) {
      int rs[GFFT_MAXP];
      for (int i = 0; i < gp.npass; ++i) rs[i] = gp.pass[i].R;
      const long long W = mixed_lanes(gp.L, dbl);
      const long long stride = n / gp.L;
      if (gp.npass <= 4 && mixed_shape_index(gp.L, rs, gp.npass) >= 0) {
        gp.variant = 7;
        gp.units = (int)W;
        gp.threads = 256;
        gp.ntiles = (batch * stride + W - 1) / W;
        // two gathered tiles and the work buffer, padded as fft_mixed.cu padded_len
        gp.smem = (size_t)(3 * W * epadded(gp.L) * esz);
        // the same shape as the column tiles of fft_colmix.cu (variant 9):
        // moved by 2-D tensor copies where every tile of W units lies in one
        // transform and one output box (W divides N / L and Ns) and the row
        // pitches are multiples of 16 bytes, else gathered by cp.async (a
        // tile may then span transforms); two stages where they fit the
        // shared memory (the gather kernel keeps 1 KB of static shared memory)
        int mW = 0, mT = 0;
        size_t msm = 0;
        const int tW = gfft::colshape::mix_lanes((int)esz, gp.L);
        const bool tma = gfft::colshape::mix_supported((int)esz, gp.L) && stride % tW == 0 &&
                         (g == 0 || Ns % tW == 0) && (stride * esz) % 16 == 0 && (g == 0 || (Ns * esz) % 16 == 0);
        // (gathers: FP32 only, one stage by default -- measured 1.1-1.4x two
        // stages at 2^27 points for 5^8, 3^12 and 360^2; FP64, FP64-pipe
        // bound, keeps the copy-free mixed tiles there)
        const int gather = tma ? 0 : 1;
        const size_t lim = (size_t)(227 * 1024 - (gather ? 1024 : 0));
        int S = o.stages > 0 ? o.stages : (gather ? 1 : 2);
        if (gather && S > 2) S = 2;
        if (col_ok && plan.nglobal > 1 && !(gather && dbl) &&
            gfft_colmix_shape(dbl, gp.L, rs, gp.npass, S, gather, &mW, &mT, &msm) == 0) {
          while (S > 1 && msm > lim) gfft_colmix_shape(dbl, gp.L, rs, gp.npass, --S, gather, &mW, &mT, &msm);
          if (msm <= lim) {
            gp.variant = 9;
            gp.units = mW;
            gp.threads = mT;
            gp.stages = S;
            gp.tk = 64;
            gp.gather = gather;
            gp.smem = msm;
            gp.ntiles = (batch * stride + mW - 1) / mW;
          }
        }
      }
    }
    // split-precision tensor-core form, on request: FP32 complex, power-of-two
    // L in 64..4096 with the specialised radices (the radix-16 passes on the
    // tensor cores); a multi-pass length must be a multiple of the tile
    if (o.variant == 6 && !dbl && trans < 2 && o.threads == 0 && o.units == 0 && o.radix_order == 0 &&
        o.max_radix == 16 && gp.L >= 64 && gp.L <= 4096 && (plan.nglobal == 1 || n % 4096 == 0) &&
        n < (1LL << 31) && spec_radices(gp)) {
      const long long W = 4096 / gp.L;
      gp.variant = 6;
      gp.units = (int)W;
      gp.threads = 256;
      gp.ntiles = (batch * (n / gp.L) + W - 1) / W;
      // aligned operands (1 KB slack, 32 KB A, 4 KB B), two padded buffers, mbarrier and TMEM slot
      gp.smem = (size_t)(1024 + 32768 + 4096 + 2 * W * padded(gp.L) * 8 + 16);
    }
    // tensor-copy column tiles: every tile of W units lies in one transform
    // (W divides N / L) and maps to W consecutive outputs (W divides Ns)
    if (col_ok && plan.nglobal > 1 && gp.L >= 64 && gp.L <= col_max && spec_radices(gp)) {
      int W = 0, T = 0;
      size_t sm = 0;
      // FP32 passes of 128 .. 512: half-size (32 KB) tiles, one stage, two
      // blocks per SM (measured on GB300 against 64 KB tiles with two
      // stages: 4-6 % faster for 2^17 .. 2^19 and 2^23 .. 2^24, within 2 %
      // for 2^14 .. 2^16); blocks_per_sm = 1 keeps the 64 KB tiles.  Other
      // passes: two stages where they fit the shared memory, else one (two
      // stages 2-12 % faster for passes of 128 .. 2048 with 64 KB tiles,
      // within 2 % for 1024 x 1024).
      int tk = 64;
      if (o.bps != 1 && (gp.L <= 512 || o.bps == 2) && gfft_col_shape(dbl, gp.L, 1, 0, 32, &W, &T, &sm) == 0)
        tk = 32;  // (FP32 passes of 1024: 32-byte rows, on request only)
      int S = o.stages > 0 ? o.stages : (tk == 32 ? 1 : 2);
      if (gfft_col_shape(dbl, gp.L, S, 0, tk, &W, &T, &sm) == 0 && (n / gp.L) % W == 0 && (g == 0 || Ns % W == 0)) {
        while (S > 1 && sm > 227 * 1024) gfft_col_shape(dbl, gp.L, --S, 0, tk, &W, &T, &sm);
        if (sm <= 227 * 1024) {
          gp.variant = 9;
          gp.units = W;
          gp.threads = T;
          gp.stages = S;
          gp.tk = tk;
          gp.smem = sm;
          gp.ntiles = batch * (n / gp.L) / W;
        }
      }
    }
    // FP32 passes left to the prefetching run-time column tiles (no compiled
    // shape): the generic engine with the radices in reverse order is
    // faster.  Measured over 150 lengths 256 .. 2^27 (the planner
    // evaluation): plans of such passes ran 1.25x (two passes) and 1.48x
    // (three) the best candidate, the engine in reverse order 1.05x / 1.02x.
    if (gp.variant == 4 && !dbl && o.variant == 0 && o.radix_order == 0 && o.max_radix == 16 && o.units == 0 &&
        o.threads == 0 && o.stages == 0 && o.max_single == 0) {
      assign(std::vector<int>(rs.rbegin(), rs.rend()));
      gp.variant = 1;
      gp.units = eng_units;
      gp.threads = eng_threads;
      gp.smem = eng_smem;
      gp.ntiles = 0;
    }
    // length-specialised variant: default radix order, L in the compiled set
    // (FP32 8192: one transform per tile, 512 threads)
    bool spec = gp.variant == 2 && (o.variant == 0 || o.variant == 3) && o.units == 0 && o.threads == 0 &&
                (gp.L <= TILE || (!dbl && gp.L == 8192)) && o.radix_order == 0 && o.max_radix == 16;
    if (spec) {
      const long long SPT = std::max<long long>(TILE, gp.L);
      const long long W = SPT / gp.L;
      gp.variant = 3;
      gp.units = (int)W;
      gp.threads = (int)(SPT / 16);
      gp.tile_bytes = (int)(SPT * esz);
      gp.ntiles = (batch + W - 1) / W;
      // 8192: one stage (measured 5 % faster than two; the copy of the next
      // tile overlaps the passes after the first)
      int S = gp.stages;
      while (S > 1 && S * SPT * esz + W * padded(gp.L) * esz + 8 * S > 220 * 1024) --S;
      gp.stages = S;
      gp.smem = (size_t)(S * SPT * esz + ((W * padded(gp.L) * esz + 7) & ~7LL) + 8 * S);
    }
    // one transform per block, no stage (spec_direct_kernel): FP32 4096 /
    // 8192 / 16384 with 4 / 2 / 1 blocks per SM by default (measured at 2^28
    // points: 86.4 -> 90.6 %, 68.0 -> 71.4 % of the copy bandwidth against
    // the staged single pass; 47.2 -> 57.1 % against two passes); an
    // explicit stage count keeps the staged kernel
    const bool direct_req = !dbl && trans < 2 && plan.nglobal == 1 && (o.variant == 0 || o.variant == 3) &&
                            o.radix_order == 0 && o.max_radix == 16 && o.units == 0 && o.threads == 0 &&
                            o.stages == 0 && o.bps == 0 && (gp.L == 4096 || gp.L == 8192);
    if (((direct16k && plan.nglobal == 1 && gp.L == 16384) || direct_req) && spec_radices(gp)) {
      gp.variant = 3;
      gp.units = 1;
      gp.threads = gp.L / 16;
      gp.stages = 0;
      gp.tile_bytes = (int)(gp.L * esz);
      gp.ntiles = batch;
      gp.smem = (size_t)(padded(gp.L) * esz);  // the work buffer only
    }
    Ns *= gp.L;
  }
  plan.tw_count = tw;
  // global four-step twiddles W_N^m = lo[m % B] * hi[m / B]
  std::size_t off = tw;
  if (plan.nglobal > 1) {
    long long B = 1;
    while (B * B < n) B *= 2;
    plan.gtw_B = (std::size_t)B;
    plan.gtw_lo_off = off;
    off += (std::size_t)B;
    plan.gtw_hi_off = off;
    off += (std::size_t)((n + B - 1) / B);
  }
  if (trans >= 2) {
    plan.rtw_off = off;
    off += (std::size_t)n;
    plan.real_fused = plan.nglobal == 1 ? 1 : 0;
    // several passes, all tensor-copy column tiles: the real post pass in the
    // last pass (forward), the pre pass in the first (inverse), where the
    // pass's real-pair tiles fit the shared memory
    bool all9 = plan.nglobal > 1;
    for (int g = 0; g < plan.nglobal; ++g) all9 = all9 && plan.gp[g].variant == 9;
    if (all9) {
      // real-pair tiles exist with 64 KB tiles only: the fused pass takes them
      GlobalPass& gp = plan.gp[trans == 2 ? plan.nglobal - 1 : 0];
      const int rf = trans == 2 ? 1 : 2;
      int W = 0, T = 0;
      size_t sm = 0;
      int S = gp.tk == 32 && o.stages == 0 ? 2 : gp.stages;
      int ok = gfft_col_shape(dbl, gp.L, S, rf, 64, &W, &T, &sm) == 0;
      while (ok && S > 1 && sm > 227 * 1024) ok = gfft_col_shape(dbl, gp.L, --S, rf, 64, &W, &T, &sm) == 0;
      if (ok && sm <= 227 * 1024 && W >= 2 && (n / gp.L) % W == 0) {
        gp.rf = rf;
        gp.tk = 64;
        gp.units = W;
        gp.threads = T;
        gp.ntiles = batch * (n / gp.L) / W;
        gp.stages = S;
        gp.smem = sm;
        plan.real_fused = 1;
      }
    }
  }
  // variant-9 later passes: W_(R0 Ns)^(k r), r < R0 (the first in-block
  // radix), k < Ns, when at most 2^20 entries
  for (int g = 1; g < plan.nglobal; ++g) {
    const GlobalPass& gp = plan.gp[g];
    if (gp.variant == 9 && gp.pass[0].R * gp.Ns <= (1LL << 20)) {
      off += off & 1;  // 16-byte aligned (FP32 complex: an even element offset) for tensor copies
      plan.ftw_off[g] = off;
      off += (std::size_t)(gp.pass[0].R * gp.Ns);
    }
  }
  plan.table_count = off;
  // workspace: odd pass counts in place need two buffers
  if (plan.nglobal >= 2) {
    plan.ws_elems = (std::size_t)(n * batch);
    plan.n_ws = (plan.nglobal % 2 == 1 && place == 0) ? 2 : 1;
  }
  return 0;
}

void gfft_plan_tables(const HostPlan& plan, double* tab) {
  // alignment gaps between the tables hold 1 (never read; every entry a root of unity)
  for (std::size_t i = 0; i < plan.table_count; ++i) {
    tab[2 * i] = 1.0;
    tab[2 * i + 1] = 0.0;
  }
  for (int g = 0; g < plan.nglobal; ++g) {
    const GlobalPass& gp = plan.gp[g];
    for (int i = 0; i < gp.npass; ++i) {
      const BlockPass& bp = gp.pass[i];
      const long long M = (long long)bp.Ns * bp.R;
      for (int r = 1; r < bp.R; ++r)
        for (int k = 0; k < bp.Ns; ++k) {
          std::size_t e = (std::size_t)bp.tw + (std::size_t)(r - 1) * bp.Ns + k;
          wroot((long long)k * r, M, &tab[2 * e], &tab[2 * e + 1]);
        }
      if (bp.gen >= 0)
        for (int m = 0; m < bp.R; ++m) wroot(m, bp.R, &tab[2 * (bp.gen + m)], &tab[2 * (bp.gen + m) + 1]);
    }
  }
  if (plan.nglobal > 1) {
    const long long B = (long long)plan.gtw_B;
    for (long long m = 0; m < B; ++m)
      wroot(m, plan.n, &tab[2 * (plan.gtw_lo_off + m)], &tab[2 * (plan.gtw_lo_off + m) + 1]);
    for (long long q = 0; q < (plan.n + B - 1) / B; ++q)
      wroot(q * B, plan.n, &tab[2 * (plan.gtw_hi_off + q)], &tab[2 * (plan.gtw_hi_off + q) + 1]);
  }
  if (plan.trans >= 2)
    for (long long q = 0; q < plan.n; ++q)
      wroot(q, 2 * plan.n, &tab[2 * (plan.rtw_off + q)], &tab[2 * (plan.rtw_off + q) + 1]);
  for (int g = 1; g < plan.nglobal; ++g) {
    if (!plan.ftw_off[g]) continue;
    const long long ns = plan.gp[g].Ns, r0 = plan.gp[g].pass[0].R;
    for (long long r = 0; r < r0; ++r)
      for (long long k = 0; k < ns; ++k) {
        const std::size_t e = plan.ftw_off[g] + (std::size_t)(r * ns + k);
        wroot(k * r, r0 * ns, &tab[2 * e], &tab[2 * e + 1]);
      }
  }
}
