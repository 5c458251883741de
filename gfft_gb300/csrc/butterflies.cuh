// Register-resident forward DFT butterflies of radix 2, 3, 4, 5, 7, 8, 16.
//
// They replace the reference's small-N kernels DFTk / DFTk_inp
// (src/gfftspec.h:42-188, src/gfftspec_inp.h:41-339), which exist only for
// radix 2, radix 3 and a generic O(p^2) odd prime; here radix 4/8/16 are
// built from radix 4 with internal twiddles by constants, and 5 and 7 use the
// symmetric odd-prime form (pairs x_j +- x_{R-j}) the reference's generic
// kernel also uses (src/gfftspec.h:61-102).  All are forward
// (e^{-2 pi i/R}); the inverse runs as conj(FFT(conj(x))).
#pragma once
#include <cuda_runtime.h>

namespace gfft {

template <typename T> struct Vec;
template <> struct Vec<float> { typedef float2 t; };
template <> struct Vec<double> { typedef double2 t; };

template <typename V> __device__ __forceinline__ V mk(decltype(V().x) x, decltype(V().x) y) {
  V r;
  r.x = x;
  r.y = y;
  return r;
}
template <typename V> __device__ __forceinline__ V cadd(V a, V b) { return mk<V>(a.x + b.x, a.y + b.y); }
template <typename V> __device__ __forceinline__ V csub(V a, V b) { return mk<V>(a.x - b.x, a.y - b.y); }
template <typename V> __device__ __forceinline__ V cmul(V a, V b) {
  return mk<V>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename V> __device__ __forceinline__ V cconj(V a) { return mk<V>(a.x, -a.y); }
template <typename V, typename T> __device__ __forceinline__ V cscale(V a, T s) { return mk<V>(a.x * s, a.y * s); }
// multiply by -i
template <typename V> __device__ __forceinline__ V cmi(V a) { return mk<V>(a.y, -a.x); }

template <typename V> __device__ __forceinline__ void dft2(V& a, V& b) {
  V t = a;
  a = cadd(t, b);
  b = csub(t, b);
}

template <typename V> __device__ __forceinline__ void dft4(V& a, V& b, V& c, V& d) {
  V t0 = cadd(a, c), t1 = csub(a, c), t2 = cadd(b, d), t3 = cmi(csub(b, d));
  a = cadd(t0, t2);
  c = csub(t0, t2);
  b = cadd(t1, t3);
  d = csub(t1, t3);
}

template <typename T, typename V> __device__ __forceinline__ void dft3(V* v) {
  const T h = (T)0.86602540378443864676372317075294;  // sin(2pi/3)
  V s = cadd(v[1], v[2]);
  V d = csub(v[1], v[2]);
  V m = mk<V>(v[0].x - (T)0.5 * s.x, v[0].y - (T)0.5 * s.y);
  v[0] = cadd(v[0], s);
  v[1] = mk<V>(m.x + h * d.y, m.y - h * d.x);
  v[2] = mk<V>(m.x - h * d.y, m.y + h * d.x);
}

// odd prime R, symmetric form: X_k = x0 + sum_j s_j cos(2 pi jk/R) - i sum_j d_j sin(2 pi jk/R)
template <typename T, typename V, int R> struct OddC;
template <typename T, typename V> struct OddC<T, V, 5> {
  __device__ static T c(int m) {
    const T t[5] = {(T)1, (T)0.30901699437494742410229341718282, (T)-0.80901699437494742410229341718282,
                    (T)-0.80901699437494742410229341718282, (T)0.30901699437494742410229341718282};
    return t[m];
  }
  __device__ static T s(int m) {
    const T t[5] = {(T)0, (T)0.95105651629515357211643933337938, (T)0.58778525229247312916870595463907,
                    (T)-0.58778525229247312916870595463907, (T)-0.95105651629515357211643933337938};
    return t[m];
  }
};
template <typename T, typename V> struct OddC<T, V, 7> {
  __device__ static T c(int m) {
    const T t[7] = {(T)1,
                    (T)0.62348980185873353052500488400424,
                    (T)-0.22252093395631440428890256449679,
                    (T)-0.90096886790241912623610231950745,
                    (T)-0.90096886790241912623610231950745,
                    (T)-0.22252093395631440428890256449679,
                    (T)0.62348980185873353052500488400424};
    return t[m];
  }
  __device__ static T s(int m) {
    const T t[7] = {(T)0,
                    (T)0.78183148246802980870844452667406,
                    (T)0.97492791218182360701813168299393,
                    (T)0.43388373911755812047576833284836,
                    (T)-0.43388373911755812047576833284836,
                    (T)-0.97492791218182360701813168299393,
                    (T)-0.78183148246802980870844452667406};
    return t[m];
  }
};

template <typename T, typename V, int R> __device__ __forceinline__ void dft_odd(V* v) {
  constexpr int H = (R - 1) / 2;
  V s[H], d[H];
#pragma unroll
  for (int j = 1; j <= H; ++j) {
    s[j - 1] = cadd(v[j], v[R - j]);
    d[j - 1] = csub(v[j], v[R - j]);
  }
  const V x0 = v[0];
  V sum = x0;
#pragma unroll
  for (int j = 0; j < H; ++j) sum = cadd(sum, s[j]);
#pragma unroll
  for (int k = 1; k <= H; ++k) {
    T re = x0.x, im = x0.y, ur = 0, ui = 0;
#pragma unroll
    for (int j = 1; j <= H; ++j) {
      const int m = (j * k) % R;
      const T c = OddC<T, V, R>::c(m), sn = OddC<T, V, R>::s(m);
      re += s[j - 1].x * c;
      im += s[j - 1].y * c;
      ur += d[j - 1].x * sn;
      ui += d[j - 1].y * sn;
    }
    v[k] = mk<V>(re + ui, im - ur);
    v[R - k] = mk<V>(re - ui, im + ur);
  }
  v[0] = sum;
}

template <typename T, typename V> __device__ __forceinline__ void dft8(V* v) {
  const T r = (T)0.70710678118654752440084436210485;
  // y0 = DFT4(x0,x2,x4,x6), y1 = DFT4(x1,x3,x5,x7)
  dft4(v[0], v[2], v[4], v[6]);
  dft4(v[1], v[3], v[5], v[7]);
  // y1[q] *= w8^q : slots y1[1]=v[3], y1[2]=v[5], y1[3]=v[7]
  V a = v[3];
  v[3] = mk<V>((a.x + a.y) * r, (a.y - a.x) * r);
  v[5] = cmi(v[5]);
  a = v[7];
  v[7] = mk<V>((a.y - a.x) * r, -(a.x + a.y) * r);
  // X_q = y0[q] + y1[q], X_{q+4} = y0[q] - y1[q]; y0[q] at v[2q], y1[q] at v[2q+1]
  V o[8];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    o[q] = cadd(v[2 * q], v[2 * q + 1]);
    o[q + 4] = csub(v[2 * q], v[2 * q + 1]);
  }
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = o[i];
}

template <typename T, typename V> __device__ __forceinline__ void dft16(V* v) {
  const T c1 = (T)0.92387953251128675612818318939679;  // cos(pi/8)
  const T s1 = (T)0.38268343236508977172845998403040;  // sin(pi/8)
  const T r = (T)0.70710678118654752440084436210485;
  // y_j[q] = DFT4_m(x_{j+4m}) for j=0..3, stored back in v[j+4q]
#pragma unroll
  for (int j = 0; j < 4; ++j) dft4(v[j], v[j + 4], v[j + 8], v[j + 12]);
  // twiddles w16^{jq} on v[j+4q]
  const V w1 = mk<V>(c1, -s1), w2 = mk<V>(r, -r), w3 = mk<V>(s1, -c1);
  const V w6 = mk<V>(-r, -r), w9 = mk<V>(-c1, s1);
  v[1 + 4] = cmul(v[5], w1);
  v[1 + 8] = cmul(v[9], w2);
  v[1 + 12] = cmul(v[13], w3);
  v[2 + 4] = cmul(v[6], w2);
  v[2 + 8] = cmi(v[10]);
  v[2 + 12] = cmul(v[14], w6);
  v[3 + 4] = cmul(v[7], w3);
  v[3 + 8] = cmul(v[11], w6);
  v[3 + 12] = cmul(v[15], w9);
  // X_{q+4p} = DFT4_j(y_j[q]) at p: for each q, legs v[4q+0..3]
  V o[16];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    V a = v[4 * q], b = v[4 * q + 1], c = v[4 * q + 2], d = v[4 * q + 3];
    dft4(a, b, c, d);
    o[q] = a;
    o[q + 4] = b;
    o[q + 8] = c;
    o[q + 12] = d;
  }
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = o[i];
}

template <typename T, typename V, int R> __device__ __forceinline__ void dft(V* v);

// Composite radix R = A * B with gcd(A, B) = 1 (6, 10, 12, 15): the
// prime-factor (Good-Thomas) split needs no twiddles.  Input n = (n1 B + n2 A)
// mod R, output k = (k1 B (B^-1 mod A) + k2 A (A^-1 mod B)) mod R; then
// W_R^{nk} = W_A^{n1 k1} W_B^{n2 k2}: B transforms of length A, A of length B.
constexpr int inv_mod(int x, int m) {
  int r = 1;
  while ((x * r) % m != 1) ++r;
  return r;
}
template <typename T, typename V, int A, int B> __device__ __forceinline__ void dft_pfa(V* v) {
  constexpr int R = A * B;
  constexpr int BI = inv_mod(B % A, A), AI = inv_mod(A % B, B);
  V t[R];
#pragma unroll
  for (int n2 = 0; n2 < B; ++n2) {
    V y[A];
#pragma unroll
    for (int n1 = 0; n1 < A; ++n1) y[n1] = v[(n1 * B + n2 * A) % R];
    dft<T, V, A>(y);
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) t[k1 * B + n2] = y[k1];
  }
#pragma unroll
  for (int k1 = 0; k1 < A; ++k1) {
    V z[B];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) z[n2] = t[k1 * B + n2];
    dft<T, V, B>(z);
#pragma unroll
    for (int k2 = 0; k2 < B; ++k2) v[(k1 * B * BI + k2 * A * AI) % R] = z[k2];
  }
}

// radix 9 = 3 x 3 (Cooley-Tukey): X[k1 + 3 k2] = sum_n2 W_3^{n2 k2} W_9^{n2 k1}
// sum_n1 x[3 n1 + n2] W_3^{n1 k1}
template <typename T, typename V> __device__ __forceinline__ void dft9(V* v) {
  // W_9^m = cos(2 pi m / 9) - i sin(2 pi m / 9), m = 1, 2, 4
  const V w1 = mk<V>((T)0.766044443118978035202392650555416674, (T)-0.642787609686539326322643409907263433);
  const V w2 = mk<V>((T)0.173648177666930348851716626769314796, (T)-0.984807753012208059366743024589523014);
  const V w4 = mk<V>((T)-0.93969262078590838405410927732473147, (T)-0.342020143325668733044099614682259581);
  V t[9];
#pragma unroll
  for (int n2 = 0; n2 < 3; ++n2) {
    V y[3] = {v[n2], v[3 + n2], v[6 + n2]};
    dft3<T, V>(y);
    t[n2] = y[0];
    t[3 + n2] = y[1];
    t[6 + n2] = y[2];
  }
  // twiddles W_9^{n2 k1} on t[3 k1 + n2]
  t[4] = cmul(t[4], w1);
  t[5] = cmul(t[5], w2);
  t[7] = cmul(t[7], w2);
  t[8] = cmul(t[8], w4);
#pragma unroll
  for (int k1 = 0; k1 < 3; ++k1) {
    V z[3] = {t[3 * k1], t[3 * k1 + 1], t[3 * k1 + 2]};
    dft3<T, V>(z);
    v[k1] = z[0];
    v[k1 + 3] = z[1];
    v[k1 + 6] = z[2];
  }
}

template <typename T, typename V, int R> __device__ __forceinline__ void dft(V* v) {
  if constexpr (R == 2) dft2(v[0], v[1]);
  else if constexpr (R == 3) dft3<T, V>(v);
  else if constexpr (R == 4) dft4(v[0], v[1], v[2], v[3]);
  else if constexpr (R == 5) dft_odd<T, V, 5>(v);
  else if constexpr (R == 7) dft_odd<T, V, 7>(v);
  else if constexpr (R == 8) dft8<T, V>(v);
  else if constexpr (R == 16) dft16<T, V>(v);
  else if constexpr (R == 6) dft_pfa<T, V, 2, 3>(v);
  else if constexpr (R == 10) dft_pfa<T, V, 2, 5>(v);
  else if constexpr (R == 12) dft_pfa<T, V, 4, 3>(v);
  else if constexpr (R == 15) dft_pfa<T, V, 3, 5>(v);
  else if constexpr (R == 9) dft9<T, V>(v);
}

}  // namespace gfft
