/*
 * ORACLE (test infrastructure only; never part of the product path).
 *
 * Exact-arithmetic references for the GFFT transform definition:
 *
 *   X_k = sum_n x_n * exp(-2*pi*i*S*k*n/N),  S=+1 forward (DFT),
 *   S=-1 inverse (IDFT) followed by the 1/N scale,
 *
 * as defined by the reference's direct DFT (src/direct.h:153-173) and its
 * sign convention (DFT is Sign=+1 = e^{-2 pi i kn/N}: src/gfftpolicy.h:226-243,
 * radix-3 proof src/gfftspec.h:117-135; IDFT scales by 1/N:
 * src/gfftswap.h:355-374).
 *
 *  - orc_dft_q     : O(N^2) direct DFT in binary128 with exact integer angle
 *                    reduction (k*n mod N); result returned as a double-double
 *                    (hi + lo), so it is accurate far below FP64 rounding.
 *  - orc_fft_ld    : mixed-radix recursive DIT in long double with exactly
 *                    reduced twiddles (binary128 on aarch64, x87 80-bit on
 *                    x86-64: relative error ~1e-19*log2 N or better).
 *  - orc_rdft_q    : direct real-input DFT of 2N reals in binary128, packed
 *                    the way the reference's Separate packs it
 *                    (src/gfftswap.h:275-279): X_0, X_N, X_1 .. X_{N-1}.
 *  - orc_gen_*     : seeded input generators (splitmix64), shared with tests.
 *
 * binary128 is `_Float128` (x86-64: software quad; aarch64: long double).
 */
#define _GNU_SOURCE
#define __STDC_WANT_IEC_60559_TYPES_EXT__ 1
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef _Float128 q_t;

static const q_t Q_2PI = 6.283185307179586476925286766559005768F128;

/* cos/sin of 2*pi*m/n with m reduced into [0, n) and folded to an octant so
 * that the binary128 library call sees |angle| <= pi/4. */
static void q_root(int64_t m, int64_t n, q_t* c, q_t* s) {
  m %= n;
  if (m < 0) m += n;
  /* angle = 2 pi m / n ; use 8m relative to n to pick the octant */
  int64_t e = 8 * m; /* angle in units of (pi/4)/n */
  int oct = (int)(e / n);
  int64_t r = e - (int64_t)oct * n; /* remainder in [0,n): angle = oct*pi/4 + r*(pi/4)/n */
  q_t a;
  int flip = oct & 1;
  if (flip) a = (q_t)(n - r) / (q_t)n * (Q_2PI / 8); /* distance to next octant edge */
  else a = (q_t)r / (q_t)n * (Q_2PI / 8);
  q_t ca = cosf128(a), sa = sinf128(a);
  /* base values for angle = k*pi/4 + a (or (k+1)*pi/4 - a when flipped) */
  q_t cc, ss;
  switch (oct) {
    case 0: cc = ca; ss = sa; break;            /* a            */
    case 1: cc = sa; ss = ca; break;            /* pi/2 - a     */
    case 2: cc = -sa; ss = ca; break;           /* pi/2 + a     */
    case 3: cc = -ca; ss = sa; break;           /* pi - a       */
    case 4: cc = -ca; ss = -sa; break;          /* pi + a       */
    case 5: cc = -sa; ss = -ca; break;          /* 3pi/2 - a    */
    case 6: cc = sa; ss = -ca; break;           /* 3pi/2 + a    */
    default: cc = ca; ss = -sa; break;          /* 2pi - a      */
  }
  *c = cc;
  *s = ss;
}

static void split_q(q_t v, double* hi, double* lo) {
  double h = (double)v;
  *hi = h;
  if (lo) *lo = (double)(v - (q_t)h);
}

/* Direct complex DFT: in is interleaved (re,im) double, n points.
 * sign=+1 forward (e^{-}), sign=-1 inverse (e^{+}, scaled by 1/n). */
void orc_dft_q(int64_t n, const double* in, double* out_hi, double* out_lo, int sign) {
  q_t* wr = (q_t*)malloc(sizeof(q_t) * (size_t)n);
  q_t* wi = (q_t*)malloc(sizeof(q_t) * (size_t)n);
  for (int64_t m = 0; m < n; ++m) {
    q_t c, s;
    q_root(m, n, &c, &s);
    wr[m] = c;
    wi[m] = (sign > 0) ? -s : s;
  }
  for (int64_t k = 0; k < n; ++k) {
    q_t ar = 0, ai = 0;
    int64_t idx = 0;
    for (int64_t j = 0; j < n; ++j) {
      q_t xr = in[2 * j], xi = in[2 * j + 1];
      ar += xr * wr[idx] - xi * wi[idx];
      ai += xr * wi[idx] + xi * wr[idx];
      idx += k;
      if (idx >= n) idx -= n;
    }
    if (sign < 0) {
      ar /= (q_t)n;
      ai /= (q_t)n;
    }
    split_q(ar, &out_hi[2 * k], out_lo ? &out_lo[2 * k] : 0);
    split_q(ai, &out_hi[2 * k + 1], out_lo ? &out_lo[2 * k + 1] : 0);
  }
  free(wr);
  free(wi);
}

/* Sampled bins of the direct DFT (for large n): bins[] lists the k values. */
void orc_dft_bins_q(int64_t n, const double* in, int64_t nb, const int64_t* bins,
                    double* out_hi, int sign) {
  for (int64_t b = 0; b < nb; ++b) {
    int64_t k = bins[b] % n;
    q_t ar = 0, ai = 0;
    int64_t idx = 0;
    for (int64_t j = 0; j < n; ++j) {
      q_t c, s;
      q_root(idx, n, &c, &s);
      q_t w_i = (sign > 0) ? -s : s;
      q_t xr = in[2 * j], xi = in[2 * j + 1];
      ar += xr * c - xi * w_i;
      ai += xr * w_i + xi * c;
      idx += k;
      if (idx >= n) idx -= n;
    }
    if (sign < 0) {
      ar /= (q_t)n;
      ai /= (q_t)n;
    }
    out_hi[2 * b] = (double)ar;
    out_hi[2 * b + 1] = (double)ai;
  }
}

/* Direct real DFT of 2n reals, packed like the reference's RDFT output:
 * out[0] = X_0, out[1] = X_n (both real), out[2k], out[2k+1] = X_k, 1<=k<n. */
void orc_rdft_q(int64_t n, const double* in, double* out) {
  int64_t L = 2 * n;
  for (int64_t k = 0; k <= n; ++k) {
    q_t ar = 0, ai = 0;
    int64_t idx = 0;
    for (int64_t j = 0; j < L; ++j) {
      q_t c, s;
      q_root(idx, L, &c, &s);
      ar += (q_t)in[j] * c;
      ai -= (q_t)in[j] * s;
      idx += k;
      if (idx >= L) idx -= L;
    }
    if (k == 0) out[0] = (double)ar;
    else if (k == n) out[1] = (double)ar;
    else {
      out[2 * k] = (double)ar;
      out[2 * k + 1] = (double)ai;
    }
  }
}

/* Direct cosine transforms as the reference defines them (src/direct.h:270-312,
 * structs DCT1 and DCT2), summed in binary128 with the angle reduced exactly:
 *   type 1: X_k = sum_{l<n} x_l cos(pi k l / (n - 1)),  n >= 2
 *   type 2: X_k = sum_{l<n} x_l cos(pi k l / n)
 * (the reference's `inverse` flag only flips the sign of pi, which cos
 * ignores).  cos(pi m / M) = cos(2 pi m / (2M)), m = k l mod 2M. */
void orc_dct_q(int64_t n, int type, const double* in, double* out) {
  const int64_t M = type == 1 ? n - 1 : n;
  const int64_t P = 2 * M;
  for (int64_t k = 0; k < n; ++k) {
    q_t acc = 0;
    int64_t idx = 0;
    for (int64_t l = 0; l < n; ++l) {
      q_t c, sn;
      q_root(idx, P, &c, &sn);
      acc += (q_t)in[l] * c;
      idx += k % P;
      if (idx >= P) idx -= P;
    }
    out[k] = (double)acc;
  }
}

/* ------------------------------------------------------------------------ */
/* long double mixed-radix FFT with exactly reduced twiddles                */

typedef long double ld_t;

static void ld_root(int64_t m, int64_t n, int sign, ld_t* c, ld_t* s) {
  q_t qc, qs;
  q_root(m, n, &qc, &qs);
  *c = (ld_t)qc;
  *s = (sign > 0) ? -(ld_t)qs : (ld_t)qs;
}

static int64_t smallest_factor(int64_t n) {
  if (n % 4 == 0 && n > 4) return 4;
  for (int64_t p = 2; p * p <= n; ++p)
    if (n % p == 0) return p;
  return n;
}

/* out[k*os] for k<n  <- DFT of in[j*is] for j<n ; tw: table of n_top roots */
static void ld_fft_rec(int64_t n, const ld_t* in, int64_t is, ld_t* out, const ld_t* twr,
                       const ld_t* twi, int64_t tstride, ld_t* scratch) {
  if (n == 1) {
    out[0] = in[0];
    out[1] = in[1];
    return;
  }
  int64_t p = smallest_factor(n);
  int64_t m = n / p;
  /* sub-transforms: out[(r*m + k)] = DFT_m of in[(j*p + r)*is] */
  for (int64_t r = 0; r < p; ++r)
    ld_fft_rec(m, in + 2 * r * is, is * p, out + 2 * r * m, twr, twi, tstride * p, scratch);
  /* combine: X[k + q*m] = sum_r W_n^{r(k+q m)} Y_r[k] */
  ld_t* t = scratch; /* 2*p values */
  for (int64_t k = 0; k < m; ++k) {
    for (int64_t r = 0; r < p; ++r) {
      int64_t e = (r * k) % n * tstride;
      ld_t wr = twr[e], wi = twi[e];
      ld_t yr = out[2 * (r * m + k)], yi = out[2 * (r * m + k) + 1];
      t[2 * r] = yr * wr - yi * wi;
      t[2 * r + 1] = yr * wi + yi * wr;
    }
    for (int64_t q = 0; q < p; ++q) {
      ld_t ar = 0, ai = 0;
      for (int64_t r = 0; r < p; ++r) {
        int64_t e = ((r * q) % p) * m * tstride;
        ld_t wr = twr[e], wi = twi[e];
        ar += t[2 * r] * wr - t[2 * r + 1] * wi;
        ai += t[2 * r] * wi + t[2 * r + 1] * wr;
      }
      out[2 * (k + q * m)] = ar;
      out[2 * (k + q * m) + 1] = ai;
    }
  }
}

/* Complex FFT of `batch` transforms of length n: interleaved doubles in/out.
 * sign=+1 forward, -1 inverse with the 1/n scale. */
void orc_fft_ld(int64_t n, int64_t batch, const double* in, double* out, int sign) {
  ld_t* twr = (ld_t*)malloc(sizeof(ld_t) * (size_t)n);
  ld_t* twi = (ld_t*)malloc(sizeof(ld_t) * (size_t)n);
  ld_t* a = (ld_t*)malloc(sizeof(ld_t) * 2 * (size_t)n);
  ld_t* b = (ld_t*)malloc(sizeof(ld_t) * 2 * (size_t)n);
  ld_t* scratch = (ld_t*)malloc(sizeof(ld_t) * 2 * (size_t)n);
  for (int64_t m = 0; m < n; ++m) ld_root(m, n, sign, &twr[m], &twi[m]);
  for (int64_t bt = 0; bt < batch; ++bt) {
    const double* x = in + 2 * n * bt;
    for (int64_t j = 0; j < 2 * n; ++j) a[j] = x[j];
    ld_fft_rec(n, a, 1, b, twr, twi, 1, scratch);
    double* y = out + 2 * n * bt;
    for (int64_t j = 0; j < 2 * n; ++j) y[j] = (double)(sign < 0 ? b[j] / (ld_t)n : b[j]);
  }
  free(twr);
  free(twi);
  free(a);
  free(b);
  free(scratch);
}

/* ------------------------------------------------------------------------ */
/* seeded inputs                                                             */

static inline uint64_t splitmix64(uint64_t* s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

/* count doubles uniform in [-1, 1) from the top 53 bits of each draw */
void orc_gen_uniform(uint64_t seed, int64_t count, double* out) {
  uint64_t s = seed;
  for (int64_t i = 0; i < count; ++i) {
    uint64_t r = splitmix64(&s) >> 11;
    out[i] = (double)r * (1.0 / 4503599627370496.0) - 1.0; /* r/2^52 - 1 */
  }
}
