// Host code under AddressSanitizer and UndefinedBehaviorSanitizer (built and
// run by tests/test_sanitizers.py): the planner (planner.cpp, colshape.cpp)
// and the host side of the C ABI (capi_host.cpp) over a sweep of lengths,
// types, transforms, places and plan options, with the invariants a plan
// must keep; and the oracle's C/C++ code (oracle_exact.c, gfft_restate.cpp)
// on small transforms checked against each other.  Exit status 0 when every
// check holds; the sanitizers abort on the first memory or UB error.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/gfft_gb300.h"
#include "plan.h"

extern "C" {
void orc_dft_q(int64_t n, const double* in, double* out_hi, double* out_lo, int sign);
void orc_fft_ld(int64_t n, int64_t batch, const double* in, double* out, int sign);
void orc_rdft_q(int64_t n, const double* in, double* out);
void orc_dct_q(int64_t n, int type, const double* in, double* out);
void orc_gen_uniform(uint64_t seed, int64_t count, double* out);
int orc_gfft_exec(int64_t n, int vtype, int trans, int place, const void* src, void* dst);
}

static int failures = 0;
#define CHECK(c, ...)                         \
  do {                                        \
    if (!(c)) {                               \
      std::fprintf(stderr, __VA_ARGS__);      \
      std::fprintf(stderr, "\n");             \
      ++failures;                             \
    }                                         \
  } while (0)

static void check_plan(uint64_t n, int vt, int tr, int pl, uint64_t batch, const gfft_plan_opts* o) {
  gfft_plan_info info;
  const int st = gfft_plan_query(n, vt, tr, pl, batch, o, &info);
  if (st != GFFT_OK) return;  // options this length cannot take are rejected, not planned
  CHECK(info.n_global_passes >= 1 && info.n_global_passes <= 4, "passes n=%llu", (unsigned long long)n);
  if (tr >= 4) return;  // cosine transforms report their inner real plan
  uint64_t prod = 1;
  for (int g = 0; g < info.n_global_passes; ++g) {
    uint64_t p = 1;
    for (int i = 0; i < 16 && info.radices[g][i]; ++i) p *= (uint64_t)info.radices[g][i];
    CHECK(p == (uint64_t)info.pass_len[g], "radices of pass %d n=%llu", g, (unsigned long long)n);
    CHECK(info.threads[g] > 0 && info.units[g] > 0, "launch shape n=%llu", (unsigned long long)n);
    prod *= (uint64_t)info.pass_len[g];
  }
  if (info.kernel_variant[0] != 8) CHECK(prod == n, "pass product n=%llu", (unsigned long long)n);
}

static void tables(uint64_t n, int dbl, int tr, const PlanOpts& po) {
  HostPlan hp;
  if (gfft_plan_build(hp, (long long)n, 3, dbl, tr, 1, po) != 0) return;
  std::vector<double> tab(2 * (hp.table_count ? hp.table_count : 1), 0.0);
  gfft_plan_tables(hp, tab.data());
  for (std::size_t i = 0; i < hp.table_count; ++i) {
    const double m = std::hypot(tab[2 * i], tab[2 * i + 1]);
    CHECK(std::fabs(m - 1.0) < 1e-12, "twiddle %zu of n=%llu has modulus %.17g", i, (unsigned long long)n, m);
  }
}

int main() {
  // the planner and the host side of the C ABI
  std::vector<uint64_t> lens;
  for (uint64_t n = 1; n <= 1100; ++n) lens.push_back(n);
  for (uint64_t n : {2048ull, 3000ull, 4096ull, 4099ull, 8192ull, 12288ull, 15625ull, 16384ull, 65536ull, 129600ull,
                     230400ull, 248832ull, 390625ull, 524288ull, 531441ull, 786432ull, 1000000ull, 1ull << 20,
                     1ull << 22, 1ull << 24, 1ull << 27, 2ull * 4099})
    lens.push_back(n);
  const int variants[] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9};
  for (uint64_t n : lens)
    for (int vt = 0; vt < 4; ++vt)
      for (int tr = 0; tr < 8; ++tr)
        for (int pl = 0; pl < 2; ++pl) {
          check_plan(n, vt, tr, pl, 1 + (n % 5), nullptr);
          if (n > 4096 || n % 7 == 0) {
            for (int v : variants) {
              gfft_plan_opts o;
              std::memset(&o, 0, sizeof(o));
              o.kernel_variant = v;
              o.max_pass_len = (int)(n % 3 == 0 ? 256 : 0);
              o.radix_order = (int)(n % 3);
              o.decimation = (v == 1 || v == 0) && (n % 2) ? 1 : 0;
              check_plan(n, vt, tr, pl, 4, &o);
              // tile-size and stage options of the column tiles and the single pass
              o.decimation = 0;
              o.max_pass_len = 0;
              o.radix_order = 0;
              o.blocks_per_sm = 1 + (int)(n % 2);
              o.stages = (int)(n % 3);
              check_plan(n, vt, tr, pl, 3, &o);
            }
          }
        }
  // invalid arguments come back as status codes
  gfft_plan_info info;
  CHECK(gfft_plan_query(0, 0, 0, 1, 1, nullptr, &info) == GFFT_E_INVALID_SIZE, "n = 0");
  CHECK(gfft_plan_query(16, 9, 0, 1, 1, nullptr, &info) == GFFT_E_INVALID_TYPE, "vtype");
  CHECK(gfft_plan_query(16, 0, 0, 1, 1, nullptr, nullptr) == GFFT_E_NULL_POINTER, "null info");
  for (int s = -2; s < 20; ++s) CHECK(gfft_strerror(s) != nullptr, "strerror %d", s);
  // every table entry a root of unity
  for (uint64_t n : {2ull, 60ull, 1000ull, 4096ull, 8192ull, 16384ull, 390625ull, 786432ull, 1ull << 20, 1ull << 24})
    for (int dbl = 0; dbl < 2; ++dbl)
      for (int tr : {0, 2}) {
        PlanOpts po;
        tables(n, dbl, tr, po);
        po.dif = 1;
        tables(n, dbl, tr, po);
      }
  // the oracle: binary128 direct DFT against the long-double FFT, the
  // restatement of the reference against both, real and cosine sums
  for (int64_t n : {1, 2, 3, 12, 60, 64, 97, 243, 256}) {
    std::vector<double> x(2 * n), hi(2 * n), lo(2 * n), f(2 * n), g(2 * n);
    orc_gen_uniform(7 + (uint64_t)n, 2 * n, x.data());
    orc_dft_q(n, x.data(), hi.data(), lo.data(), 1);
    orc_fft_ld(n, 1, x.data(), f.data(), 1);
    double e = 0, m = 0;
    for (int64_t i = 0; i < 2 * n; ++i) {
      e = std::fmax(e, std::fabs(hi[i] - f[i]));
      m = std::fmax(m, std::fabs(hi[i]));
    }
    CHECK(e <= 1e-13 * std::fmax(1.0, m), "oracle dft vs fft n=%lld err %g", (long long)n, e);
    if (orc_gfft_exec(n, 0, 0, 1, x.data(), g.data()) == 0) {
      double r = 0;
      for (int64_t i = 0; i < 2 * n; ++i) r = std::fmax(r, std::fabs(g[i] - hi[i]));
      CHECK(r <= 1e-12 * std::fmax(1.0, m), "restatement n=%lld err %g", (long long)n, r);
    }
    std::vector<double> rx(2 * n), ro(2 * n + 2), c(n);
    orc_gen_uniform(11, 2 * n, rx.data());
    orc_rdft_q(n, rx.data(), ro.data());
    if (n >= 2) orc_dct_q(n, 1, rx.data(), c.data());
    orc_dct_q(n, 2, rx.data(), c.data());
  }
  std::printf("sanitized host checks: %d failures\n", failures);
  return failures ? 1 : 0;
}
