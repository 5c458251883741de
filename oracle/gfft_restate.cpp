/*
 * ORACLE (test infrastructure only; never part of the product path).
 *
 * CPU restatement of scpp/gfft's transform algorithm with a RUN-TIME length.
 * The reference resolves N, its factor list and its roots of unity at compile
 * time; this file performs the same arithmetic, in the same order and in the
 * same C++ types, with N as an ordinary argument.  It is used
 *   (1) as the parity checker for the CUDA path at sizes where no fixture
 *       from the compiled reference exists, and
 *   (2) as the timed CPU baseline ("port"), batched with OpenMP.
 *
 * Followed, function by function (paths inside scpp/gfft):
 *   factor list             Factorization / trial division, ascending primes
 *                           (src/gfftfactor.h:160-169; metafactor submodule)
 *   first root per level    GetFirstRoot (src/metaroot.h:104-120) evaluated to
 *                           Accuracy*9 decimals, turned into double by
 *                           Compute::value (src/metafunc.h:239-280,
 *                           src/sbigint.h:140-173); W^K for the next level
 *                           (IPowBig, src/gfftalg.h:475) is evaluated the same
 *                           way as the root of N/K
 *   out-of-place recursion  InTimeOOP (src/gfftalg.h:459-507)
 *   in-place recursion      GFFTswap2 + InTime (src/gfftswap.h:74-140,
 *                           src/gfftalg.h:383-442), prime powers only
 *   combine pass            DFTk_x_Im_T general (src/gfftalg.h:169-192),
 *                           radix 2 (src/gfftalg.h:228-267, 355-367)
 *   butterflies             DFTk (src/gfftspec.h:42-188),
 *                           DFTk_inp (src/gfftspec_inp.h:41-339)
 *   twiddle recurrences     ComputeRoots / RootsContainer (src/twiddles.h:212-339)
 *   odd-prime constants     ComputeTwiddles + Sin/Cos series
 *                           (src/twiddles.h:177-198, src/pseudometafunc.h:64-143)
 *   real transforms         Separate (src/gfftswap.h:239-287), stage order of
 *                           RDFT / IRDFT (src/gfftpolicy.h:262-297)
 *   scaling                 Forward / Backward (src/gfftswap.h:338-374)
 *   OpenMP loop             replaced by an OpenMP loop over the batch, i.e.
 *                           Serial objects in parallel (the reference's own
 *                           OpenMP<NT> policy, src/gfftomp.h, splits inside one
 *                           transform and is not restated here)
 *
 * Types follow the reference's value-type tags (src/gfftpolicy.h:78-127):
 *   DOUBLE: T=double, TempType=long double, 18 decimals (x86-64 Accuracy=2)
 *   FLOAT : T=float,  TempType=double,      9 decimals  (x86-64 Accuracy=1)
 * Build with -ffp-contract=off so that no multiply-add is fused; the golden
 * fixtures of the compiled reference are produced with the same flag.
 */
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

typedef long long_t;

/* M_PI exactly as the reference's series use it (a double constant). */
static const double kPi = 3.14159265358979323846;

/* ---- pseudo-meta Sin/Cos series (src/pseudometafunc.h:64-143) ---------- */
/* SinCosSeries<M,N,B,A>::value() = 1 - (A*pi/B)^2/M/(M+1) * next, all the
 * left factor in double, the product with the long double tail in long
 * double. */
static long double sincos_series(unsigned M, unsigned N, unsigned B, unsigned A) {
  if (M == N) return 1.0L;
  const double x = A * kPi / B;
  return 1 - x * x / M / (M + 1) * sincos_series(M + 2, N, B, A);
}
template <class T> struct Series;
template <> struct Series<float> {
  static float sin(unsigned B, unsigned A) { return (A * kPi / B) * sincos_series(2, 24, B, A); }
  static float cos(unsigned B, unsigned A) { return sincos_series(1, 23, B, A); }
};
template <> struct Series<double> {
  static double sin(unsigned B, unsigned A) { return (A * kPi / B) * sincos_series(2, 34, B, A); }
  static double cos(unsigned B, unsigned A) { return sincos_series(1, 33, B, A); }
};
template <> struct Series<long double> {
  static long double sin(unsigned B, unsigned A) { return (A * kPi / B) * sincos_series(2, 60, B, A); }
  static long double cos(unsigned B, unsigned A) { return sincos_series(1, 59, B, A); }
};

/* ---- compile-time decimal constants turned into double ----------------- */
/* A decimal value v with `words` base-1e9 fraction words is evaluated as the
 * reference's EvaluateToFloat does: w0 + 1e9*(w1 + 1e9*(w2 ...)), then
 * divided by 1e9^words (src/sbigint.h:140-173, src/metafunc.h:243-251). */
template <class R>
static R decimal_to(long double v, int words) {
  bool neg = v < 0;
  long double a = neg ? -v : v;
  /* scaled integer, rounded to nearest */
  long double scale = 1;
  for (int i = 0; i < words; ++i) scale *= 1e9L;
  long double q = std::floor(a * scale + 0.5L);
  /* split into base-1e9 words, least significant first */
  long double w[4] = {0, 0, 0, 0};
  for (int i = 0; i < 4; ++i) {
    long double hi = std::floor(q / 1e9L);
    w[i] = q - hi * 1e9L;
    q = hi;
  }
  R acc = static_cast<R>(w[3]);
  for (int i = 2; i >= 0; --i) acc = static_cast<R>(w[i]) + static_cast<R>(1000000000) * acc;
  R den = static_cast<R>(1);
  for (int i = 0; i < words; ++i) den = static_cast<R>(1000000000) * den;
  R r = acc / den;
  return neg ? -r : r;
}

/* cos(2 pi m / n) and sin(2 pi m / n) accurately (long double with exact
 * integer reduction). */
static void exact_root(long_t m, long_t n, long double* c, long double* s) {
  m %= n;
  const long double ang = 2.0L * 3.141592653589793238462643383279502884L * (long double)m / (long double)n;
  *c = std::cos(ang);
  *s = std::sin(ang);
}

template <class T> struct VType;
template <> struct VType<double> {
  typedef long double LT;
  static const int words = 2; /* Accuracy on x86-64 */
};
template <> struct VType<float> {
  typedef double LT;
  static const int words = 1;
};

/* First root of length L for sign S as Compute<...>::value() returns it (a
 * double): W = cos(2pi/L) - i*S*sin(2pi/L) (src/metaroot.h:104-120). */
template <class T>
struct Root {
  double re, im;
  Root(long_t L, int S) {
    long double c, s;
    exact_root(1, L, &c, &s);
    const int w = VType<T>::words;
    if (L == 1) { c = 1; s = 0; }
    re = decimal_to<double>(c, w);
    im = decimal_to<double>(S < 0 ? s : -s, w);
    if (L == 2) { re = -1; im = 0; }
    if (L == 4) { re = 0; im = S < 0 ? 1 : -1; }
  }
};

/* Optional per-level root constants (top-down), used to reproduce the
 * compiled reference bit for bit when its own constants are supplied. */
struct RootTable {
  int nlev;
  const double* re;
  const double* im;
};

template <class T>
static Root<T> level_root(long_t N, int S, int depth, const RootTable* rt) {
  Root<T> r(N, S);
  if (rt && depth < rt->nlev) {
    r.re = rt->re[depth];
    r.im = rt->im[depth];
  }
  return r;
}

/* sqrt(3)/2 with sign, as DFTk<3> computes m_coef (src/gfftspec.h:109-115) */
template <class T>
static T coef3(int S) {
  const T v = decimal_to<T>(std::sqrt(3.0L), VType<T>::words);
  return S * v * 0.5;
}

/* ---- butterflies ------------------------------------------------------- */

/* generic odd prime K: constants m_c[k]=cos(2(k+1)pi/K), m_s=S*sin(...) */
template <class T>
struct OddConsts {
  typedef typename VType<T>::LT LT;
  std::vector<LT> c, s;
  OddConsts(long_t K, int S) {
    long_t H = (K - 1) / 2;
    c.resize(H);
    s.resize(H);
    for (long_t k = 1; k <= H; ++k) {
      c[k - 1] = Series<LT>::cos((unsigned)K, (unsigned)(2 * k));
      s[k - 1] = S * Series<LT>::sin((unsigned)K, (unsigned)(2 * k));
    }
  }
};

/* _transform of DFTk_inp / the body of DFTk (src/gfftspec_inp.h:55-80,
 * src/gfftspec.h:76-102): writes legs 1..K-1 at dst[i*DI]; dst0 = x0 */
template <class T>
static void odd_core(long_t K, const OddConsts<T>& oc, T x0r, T x0i, const T* sr, const T* si,
                     const T* dr, const T* di, T* dst, long_t DI) {
  typedef typename VType<T>::LT LT;
  const long_t H = (K - 1) / 2;
  const long_t NDI = K * DI;
  for (long_t i = 1; i < H + 1; ++i) {
    T re1(0), re2(0), im1(0), im2(0);
    for (long_t j = 0; j < H; ++j) {
      const bool sign_change = (i * (j + 1) % K) > H;
      const long_t kk = (i + j * i) % K;
      const long_t k = (kk > H) ? K - kk - 1 : kk - 1;
      const T s1 = oc.s[k] * di[j];
      const T s2 = oc.s[k] * dr[j];
      re1 += oc.c[k] * sr[j];
      im1 += oc.c[k] * si[j];
      re2 += sign_change ? -s1 : s1;
      im2 -= sign_change ? -s2 : s2;
    }
    const long_t k = i * DI;
    dst[k] = x0r + re1 + re2;
    dst[k + 1] = x0i + im1 + im2;
    dst[NDI - k] = x0r + re1 - re2;
    dst[NDI - k + 1] = x0i + im1 - im2;
  }
  (void)sizeof(LT);
}

/* per-butterfly temporaries: on the stack for primes up to 129 */
template <class T>
struct Scratch {
  T fixed[4 * 64];
  std::vector<T> heap;
  T *sr, *si, *dr, *di;
  explicit Scratch(long_t H) {
    T* b = fixed;
    if (H > 64) {
      heap.resize(4 * H);
      b = heap.data();
    }
    sr = b;
    si = b + H;
    dr = b + 2 * H;
    di = b + 3 * H;
  }
};

/* In-place butterfly on legs data[0], data[M2], ..., data[(K-1)*M2]
 * (DFTk_inp<K,M2>), untwiddled. */
template <class T>
struct InpButterfly {
  typedef typename VType<T>::LT LT;
  long_t K;
  int S;
  T m_coef;
  OddConsts<T> oc;
  InpButterfly(long_t K_, int S_) : K(K_), S(S_), m_coef(K_ == 3 ? coef3<T>(S_) : T(0)), oc(K_ > 3 ? K_ : 3, S_) {}

  void apply(T* data, long_t M) const { /* M = leg stride in scalars */
    if (K == 2) {
      const T tr = data[M];
      const T ti = data[M + 1];
      data[M] = data[0] - tr;
      data[M + 1] = data[1] - ti;
      data[0] += tr;
      data[1] += ti;
    } else if (K == 3) {
      const long_t I10 = M, I11 = M + 1, I20 = M + M, I21 = I20 + 1;
      const T sum_r = data[I10] + data[I20];
      const T dif_r = m_coef * (data[I10] - data[I20]);
      const T sum_i = data[I11] + data[I21];
      const T dif_i = m_coef * (data[I11] - data[I21]);
      const T tr = data[0] - 0.5 * sum_r;
      const T ti = data[1] - 0.5 * sum_i;
      data[0] += sum_r;
      data[1] += sum_i;
      data[I10] = tr + dif_i;
      data[I11] = ti - dif_r;
      data[I20] = tr - dif_i;
      data[I21] = ti + dif_r;
    } else {
      const long_t H = (K - 1) / 2, NM = K * M;
      Scratch<T> sc(H);
      T *sr = sc.sr, *si = sc.si, *dr = sc.dr, *di = sc.di;
      for (long_t i = 0; i < H; ++i) {
        const long_t k = (i + 1) * M;
        sr[i] = data[k] + data[NM - k];
        si[i] = data[k + 1] + data[NM - k + 1];
        dr[i] = data[k] - data[NM - k];
        di[i] = data[k + 1] - data[NM - k + 1];
      }
      transform_odd(data, M, sr, si, dr, di);
    }
  }

  void transform_odd(T* data, long_t M, const T* sr, const T* si, const T* dr, const T* di) const {
    const long_t H = (K - 1) / 2;
    odd_core<T>(K, oc, data[0], data[1], sr, si, dr, di, data, M);
    for (long_t i = 0; i < H; ++i) {
      data[0] += sr[i];
      data[1] += si[i];
    }
  }

  /* twiddled, radix 2 with T twiddles (DFTk_inp<2>::apply(data,wr,wi)) */
  void apply2_tw(T* data, long_t M, const T* wr, const T* wi) const {
    const T tr = data[M] * (*wr) - data[M + 1] * (*wi);
    const T ti = data[M] * (*wi) + data[M + 1] * (*wr);
    data[M] = data[0] - tr;
    data[M + 1] = data[1] - ti;
    data[0] += tr;
    data[1] += ti;
  }
  /* radix 2 with twiddle -i*S (apply_1) */
  void apply2_1(T* data, long_t M) const {
    const T tr = (S < 0) ? -data[M + 1] : data[M + 1];
    const T ti = (S < 0) ? data[M] : -data[M];
    data[M] = data[0] - tr;
    data[M + 1] = data[1] - ti;
    data[0] += tr;
    data[1] += ti;
  }
  /* twiddled odd K with TempType twiddles wr[0..K-2] */
  void apply_tw(T* data, long_t M, const LT* wr, const LT* wi) const {
    if (K == 3) {
      const long_t I10 = M, I11 = M + 1, I20 = M + M, I21 = I20 + 1;
      const T tr1 = data[I10] * wr[0] - data[I11] * wi[0];
      const T ti1 = data[I10] * wi[0] + data[I11] * wr[0];
      const T tr2 = data[I20] * wr[1] - data[I21] * wi[1];
      const T ti2 = data[I20] * wi[1] + data[I21] * wr[1];
      const T sum_r = tr1 + tr2;
      const T dif_r = m_coef * (tr1 - tr2);
      const T sum_i = ti1 + ti2;
      const T dif_i = m_coef * (ti1 - ti2);
      const T tr = data[0] - 0.5 * sum_r;
      const T ti = data[1] - 0.5 * sum_i;
      data[0] += sum_r;
      data[1] += sum_i;
      data[I10] = tr + dif_i;
      data[I11] = ti - dif_r;
      data[I20] = tr - dif_i;
      data[I21] = ti + dif_r;
      return;
    }
    const long_t H = (K - 1) / 2, NM = K * M;
    Scratch<T> sc(H);
    T *sr = sc.sr, *si = sc.si, *dr = sc.dr, *di = sc.di;
    for (long_t i = 0; i < H; ++i) {
      const long_t k = (i + 1) * M;
      const T tr1 = data[k] * wr[i] - data[k + 1] * wi[i];
      const T ti1 = data[k] * wi[i] + data[k + 1] * wr[i];
      const T tr2 = data[NM - k] * wr[K - i - 2] - data[NM - k + 1] * wi[K - i - 2];
      const T ti2 = data[NM - k] * wi[K - i - 2] + data[NM - k + 1] * wr[K - i - 2];
      sr[i] = tr1 + tr2;
      si[i] = ti1 + ti2;
      dr[i] = tr1 - tr2;
      di[i] = ti1 - ti2;
    }
    transform_odd(data, M, sr, si, dr, di);
  }
};

/* Out-of-place leaf DFTk<K,SI,DI> (src/gfftspec.h:42-188) */
template <class T>
static void leaf_oop(long_t K, int S, const InpButterfly<T>& bf, const T* src, long_t SI, T* dst, long_t DI) {
  if (K == 2) {
    const T tr = src[0] - src[SI];
    const T ti = src[1] - src[SI + 1];
    dst[0] = src[0] + src[SI];
    dst[1] = src[1] + src[SI + 1];
    dst[DI] = tr;
    dst[DI + 1] = ti;
  } else if (K == 3) {
    const T m_coef = bf.m_coef;
    const long_t SI2 = SI + SI, DI2 = DI + DI;
    const T sr = src[SI] + src[SI2];
    const T dr = m_coef * (src[SI] - src[SI2]);
    const T si = src[SI + 1] + src[SI2 + 1];
    const T di = m_coef * (src[SI + 1] - src[SI2 + 1]);
    const T tr = src[0] - 0.5 * sr;
    const T ti = src[1] - 0.5 * si;
    dst[0] = src[0] + sr;
    dst[1] = src[1] + si;
    dst[DI] = tr + di;
    dst[DI + 1] = ti - dr;
    dst[DI2] = tr - di;
    dst[DI2 + 1] = ti + dr;
  } else {
    const OddConsts<T>& oc = bf.oc;
    const long_t H = (K - 1) / 2, NSI = K * SI;
    Scratch<T> sc(H);
    T *sr = sc.sr, *si = sc.si, *dr = sc.dr, *di = sc.di;
    for (long_t i = 0; i < H; ++i) {
      const long_t k = (i + 1) * SI;
      sr[i] = src[k] + src[NSI - k];
      si[i] = src[k + 1] + src[NSI - k + 1];
      dr[i] = src[k] - src[NSI - k];
      di[i] = src[k + 1] - src[NSI - k + 1];
    }
    odd_core<T>(K, oc, src[0], src[1], sr, si, dr, di, dst, DI);
    dst[0] = src[0];
    dst[1] = src[1];
    for (long_t i = 0; i < H; ++i) {
      dst[0] += sr[i];
      dst[1] += si[i];
    }
  }
}

/* Combine pass DFTk_x_Im_T<K, ., M, Step=1> on data of K*M complex values
 * with first root W1 of length K*M. */
template <class T>
static void combine(long_t K, long_t M, const InpButterfly<T>& bf, const Root<T>& W1, T* data) {
  typedef typename VType<T>::LT LT;
  const long_t M2 = 2 * M; /* leg stride in scalars */
  if (K == 2) {
    if (M == 2) { /* SimpleSpec == 2 (src/gfftalg.h:355-367) */
      bf.apply(data, M2);
      bf.apply2_1(data + 2, M2);
      return;
    }
    const long_t N = 2 * M; /* scalars in half the data */
    bf.apply(data, M2);
    if (M % 2 == 0) bf.apply2_1(data + M, M2);
    T wr, wi, t;
    const T wpr = W1.re;
    const T wpi = W1.im;
    wr = wpr;
    wi = wpi;
    bf.apply2_tw(data + 2, M2, &wr, &wi);
    t = -wr;
    bf.apply2_tw(data + N - 2, M2, &t, &wi);
    for (long_t i = 4; i < M; i += 2) {
      t = wr;
      wr = wr * wpr - wi * wpi;
      wi = wi * wpr + t * wpi;
      bf.apply2_tw(data + i, M2, &wr, &wi);
      t = -wr;
      bf.apply2_tw(data + N - i, M2, &t, &wi);
    }
    return;
  }
  /* general: ComputeRoots<K> in TempType (src/twiddles.h:291-339) */
  bf.apply(data, M2);
  LT fixed[4 * 32];
  std::vector<LT> heap;
  LT* b = fixed;
  if (K - 1 > 32) {
    heap.resize(4 * (K - 1));
    b = heap.data();
  }
  LT *wpr = b, *wpi = b + (K - 1), *wr = b + 2 * (K - 1), *wi = b + 3 * (K - 1);
  wpr[0] = W1.re;
  wpi[0] = W1.im;
  for (long_t i = 0; i < K - 2; ++i) {
    wpr[i + 1] = wpr[i] * wpr[0] - wpi[i] * wpi[0];
    wpi[i + 1] = wpr[i] * wpi[0] + wpr[0] * wpi[i];
  }
  for (long_t i = 0; i < K - 1; ++i) {
    wr[i] = wpr[i];
    wi[i] = wpi[i];
  }
  bf.apply_tw(data + 2, M2, wr, wi);
  for (long_t j = 4; j < M2; j += 2) {
    for (long_t i = 0; i < K - 1; ++i) { /* RootsContainer::step */
      LT tt = wr[i];
      wr[i] = tt * wpr[i] - wi[i] * wpi[i];
      wi[i] = wi[i] * wpr[i] + tt * wpi[i];
    }
    bf.apply_tw(data + j, M2, wr, wi);
  }
}

struct Factor {
  long_t p, k;
};

static std::vector<Factor> factorize(long_t n) {
  std::vector<Factor> f;
  for (long_t p = 2; p * p <= n; p += (p == 2 ? 1 : 2)) {
    long_t k = 0;
    while (n % p == 0) {
      n /= p;
      ++k;
    }
    if (k) f.push_back({p, k});
  }
  if (n > 1) f.push_back({n, 1});
  return f;
}

/* Everything a transform object holds constant between calls: the prime
 * peeled at each recursion depth, each depth's root, one butterfly object per
 * prime (the reference keeps these in its compile-time types and objects). */
template <class T>
struct Ctx {
  int S;
  std::vector<long_t> level;  /* prime peeled at depth d (ascending order) */
  std::vector<Root<T> > root; /* first root of the length at depth d */
  std::vector<InpButterfly<T>*> bf_of_depth;
  std::vector<InpButterfly<T>*> own;
  Ctx(long_t n, int S_, const RootTable* rt) : S(S_) {
    for (const Factor& f : factorize(n))
      for (long_t i = 0; i < f.k; ++i) level.push_back(f.p);
    long_t N = n;
    for (size_t d = 0; d < level.size(); ++d) {
      root.push_back(level_root<T>(N, S, (int)d, rt));
      InpButterfly<T>* b = nullptr;
      for (InpButterfly<T>* o : own)
        if (o->K == level[d]) b = o;
      if (!b) {
        b = new InpButterfly<T>(level[d], S);
        own.push_back(b);
      }
      bf_of_depth.push_back(b);
      N /= level[d];
    }
  }
  ~Ctx() {
    for (InpButterfly<T>* o : own) delete o;
  }
};

/* InTimeOOP (src/gfftalg.h:459-507) */
template <class T>
static void intime_oop(long_t N, const Ctx<T>& c, long_t LastK, const T* src, T* dst, int depth) {
  const long_t K = c.level[depth];
  if (N == K) { /* prime leaf */
    leaf_oop<T>(K, c.S, *c.bf_of_depth[depth], src, 2 * LastK, dst, 2);
    return;
  }
  const long_t M = N / K;
  for (long_t m = 0, lk = 0; m < 2 * N; m += 2 * M, lk += 2 * LastK)
    intime_oop<T>(M, c, K * LastK, src + lk, dst + m, depth + 1);
  combine<T>(K, M, *c.bf_of_depth[depth], c.root[depth], dst);
}

/* InTime (src/gfftalg.h:400-442), after the digit reversal; prime powers */
template <class T>
static void intime_inp(long_t N, const Ctx<T>& c, T* data, int depth) {
  const long_t p = c.level[depth];
  if (N == p) {
    c.bf_of_depth[depth]->apply(data, 2);
    return;
  }
  const long_t M = N / p;
  for (long_t m = 0; m < 2 * N; m += 2 * M) intime_inp<T>(M, c, data + m, depth + 1);
  combine<T>(p, M, *c.bf_of_depth[depth], c.root[depth], data);
}

/* base-p digit reversal of N = p^P complex values (GFFTswap2) */
template <class T>
static void digit_reverse(long_t N, long_t p, T* data) {
  long_t P = 0;
  for (long_t t = N; t > 1; t /= p) ++P;
  for (long_t n = 0; n < N; ++n) {
    long_t r = 0, t = n;
    for (long_t d = 0; d < P; ++d) {
      r = r * p + t % p;
      t /= p;
    }
    if (n > r) {
      std::swap(data[2 * n], data[2 * r]);
      std::swap(data[2 * n + 1], data[2 * r + 1]);
    }
  }
}

/* Separate<N,VType,S> (src/gfftswap.h:239-280) on 2N reals */
template <class T>
static void separate(long_t N, int S, T* data) {
  typedef typename VType<T>::LT LT;
  const int M = (S == 1) ? 2 : 1;
  long_t i, i1, i2, i3, i4;
  LT wtemp, wr, wi, wpr, wpi;
  LT h1r, h1i, h2r, h2i, h3r, h3i;
  wtemp = Series<LT>::sin((unsigned)(2 * N), 1);
  wpr = -2. * wtemp * wtemp;
  wpi = -S * Series<LT>::sin((unsigned)N, 1);
  wr = 1. + wpr;
  wi = wpi;
  for (i = 1; i < N / 2; ++i) {
    i1 = i + i;
    i2 = i1 + 1;
    i3 = 2 * N - i1;
    i4 = i3 + 1;
    h1r = 0.5 * (data[i1] + data[i3]);
    h1i = 0.5 * (data[i2] - data[i4]);
    h2r = S * 0.5 * (data[i2] + data[i4]);
    h2i = -S * 0.5 * (data[i1] - data[i3]);
    h3r = wr * h2r - wi * h2i;
    h3i = wr * h2i + wi * h2r;
    data[i1] = h1r + h3r;
    data[i2] = h1i + h3i;
    data[i3] = h1r - h3r;
    data[i4] = -h1i + h3i;
    wtemp = wr;
    wr += wr * wpr - wi * wpi;
    wi += wi * wpr + wtemp * wpi;
  }
  h1r = data[0];
  data[0] = M * 0.5 * (h1r + data[1]);
  data[1] = M * 0.5 * (h1r - data[1]);
  if (N > 1) data[N + 1] = -data[N + 1];
}

template <class T>
static void backward(long_t N, T* data) {
  for (T* i = data; i < data + 2 * N; ++i) *i /= N;
}

static bool is_prime_power(long_t n, long_t* p) {
  std::vector<Factor> f = factorize(n);
  if (f.size() != 1) return false;
  *p = f[0].p;
  return true;
}

/* status codes shared with the tests */
enum { OK = 0, E_SIZE = 1, E_PLACE = 2, E_TYPE = 3 };

/* One transform object of the reference: trans 0=DFT 1=IDFT 2=RDFT 3=IRDFT,
 * place 0=IN_PLACE 1=OUT_OF_PLACE.  Returns a status. */
template <class T>
static int exec_one(long_t n, int trans, int place, const T* src, T* dst, const RootTable* rt,
                    const Ctx<T>* cx = nullptr) {
  if (n < 1) return E_SIZE;
  const int S = (trans == 0 || trans == 2) ? 1 : -1;
  Ctx<T>* own = nullptr;
  if (!cx && n > 1) cx = own = new Ctx<T>(n, S, rt);
  struct Del {
    Ctx<T>* p;
    ~Del() { delete p; }
  } del_{own};
  if (trans >= 2) {
    /* real transforms: in place, N a power of two (src/gfftswap.h:282-286) */
    long_t p;
    if (place != 0) return E_PLACE;
    if (n > 1 && (!is_prime_power(n, &p) || p != 2)) return E_SIZE;
    T* d = dst;
    if (d != src) std::memcpy(d, src, sizeof(T) * 2 * n);
    if (trans == 3) separate<T>(n, S, d);
    if (n > 1) {
      digit_reverse<T>(n, 2, d);
      intime_inp<T>(n, *cx, d, 0);
    }
    if (trans == 3) backward<T>(n, d);
    if (trans == 2) separate<T>(n, S, d);
    return OK;
  }
  if (place == 0) {
    long_t p;
    if (n == 1) {
      if (dst != src) std::memcpy(dst, src, sizeof(T) * 2);
      return OK;
    }
    if (!is_prime_power(n, &p)) return E_PLACE;
    if (dst != src) std::memcpy(dst, src, sizeof(T) * 2 * n);
    digit_reverse<T>(n, p, dst);
    intime_inp<T>(n, *cx, dst, 0);
  } else {
    if (n == 1) {
      dst[0] = src[0];
      dst[1] = src[1];
    } else {
      intime_oop<T>(n, *cx, 1, src, dst, 0);
    }
  }
  if (trans == 1) backward<T>(n, dst);
  return OK;
}

template <class T>
static int exec_batch(int64_t n, int64_t batch, int trans, int place, const T* src, T* dst, int nthreads) {
  const int S = (trans == 0 || trans == 2) ? 1 : -1;
  Ctx<T> cx(n > 1 ? n : 2, S, nullptr);
  int err = 0;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads) reduction(max : err)
#endif
  for (int64_t b = 0; b < batch; ++b) {
    int e = exec_one<T>(n, trans, place, src + (size_t)b * 2 * n, dst + (size_t)b * 2 * n, nullptr,
                        n > 1 ? &cx : nullptr);
    if (e > err) err = e;
  }
  (void)nthreads;
  return err;
}

}  // namespace

extern "C" {

/* vtype: 0 = DOUBLE / COMPLEX_DOUBLE, 1 = FLOAT / COMPLEX_FLOAT */
int orc_gfft_exec(int64_t n, int vtype, int trans, int place, const void* src, void* dst) {
  if (vtype == 0) return exec_one<double>(n, trans, place, (const double*)src, (double*)dst, 0);
  if (vtype == 1) return exec_one<float>(n, trans, place, (const float*)src, (float*)dst, 0);
  return E_TYPE;
}

/* As orc_gfft_exec, with the per-level root constants given (top-down). */
int orc_gfft_exec_roots(int64_t n, int vtype, int trans, int place, const void* src, void* dst,
                        int nlev, const double* re, const double* im) {
  RootTable rt = {nlev, re, im};
  if (vtype == 0) return exec_one<double>(n, trans, place, (const double*)src, (double*)dst, &rt);
  if (vtype == 1) return exec_one<float>(n, trans, place, (const float*)src, (float*)dst, &rt);
  return E_TYPE;
}

/* Batched: transform b reads src + b*2n scalars and writes dst + b*2n;
 * one context (roots, butterfly constants) shared by the whole batch, an
 * OpenMP loop over the batch.  nthreads <= 0 uses every OpenMP thread. */
int orc_gfft_exec_batch(int64_t n, int64_t batch, int vtype, int trans, int place, const void* src,
                        void* dst, int nthreads) {
  if (vtype == 0) return exec_batch<double>(n, batch, trans, place, (const double*)src, (double*)dst, nthreads);
  if (vtype == 1) return exec_batch<float>(n, batch, trans, place, (const float*)src, (float*)dst, nthreads);
  return E_TYPE;
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
