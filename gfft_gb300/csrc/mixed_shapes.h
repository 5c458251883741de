// Pass shapes (length and in-block radix sequence) that have a compile-time
// column-tile kernel (fft_mixed.cu, variant 7).  Shared by the planner and
// the kernel dispatch; a shape is used only when the planner's radices for
// that length are exactly these.
#pragma once

struct MixedShape {
  int L;
  int r[4];  // radices, 1 = unused
};

static const MixedShape kMixedShapes[] = {
    {768, {16, 16, 3, 1}},  {625, {5, 5, 5, 5}},  {576, {16, 12, 3, 1}}, {432, {16, 9, 3, 1}},
    {1000, {10, 10, 10, 1}}, {729, {9, 9, 9, 1}}, {480, {16, 15, 2, 1}}, {360, {15, 12, 2, 1}},
};
static const int kNumMixedShapes = (int)(sizeof(kMixedShapes) / sizeof(kMixedShapes[0]));

// index of the shape with length L and radices rs[0..np), or -1
inline int mixed_shape_index(int L, const int* rs, int np) {
  for (int i = 0; i < kNumMixedShapes; ++i) {
    const MixedShape& m = kMixedShapes[i];
    if (m.L != L) continue;
    int n = 0;
    while (n < 4 && m.r[n] > 1) ++n;
    if (n != np) continue;
    bool ok = true;
    for (int p = 0; p < n && ok; ++p) ok = m.r[p] == rs[p];
    if (ok) return i;
  }
  return -1;
}

// lanes per tile: the largest power of two W with W * L <= tile (4096 FP32,
// 2048 FP64 values)
inline int mixed_lanes(int L, int dbl) {
  const int tile = dbl ? 2048 : 4096;
  int W = 1;
  while (2 * W * L <= tile) W *= 2;
  return W;
}

// Pass shapes of the ragged kernel's compile-time pass functions (FP32): the
// most frequent (length, radices) of lengths 2^6..2^18 with 5-smooth sizes
// under the ragged planner, covering 99 % of the points of 10,000 such
// lengths drawn log-uniformly; X(index, R0, R1, R2, R3), 1 = unused.
#define GFFT_RAGGED_SHAPES(X) \
  X(0, 15, 12, 2, 1) \
  X(1, 15, 10, 2, 1) \
  X(2, 15, 15, 2, 1) \
  X(3, 16, 5, 5, 1) \
  X(4, 16, 15, 2, 1) \
  X(5, 12, 9, 3, 1) \
  X(6, 15, 5, 5, 1) \
  X(7, 10, 10, 5, 1) \
  X(8, 16, 10, 2, 1) \
  X(9, 16, 12, 2, 1) \
  X(10, 16, 9, 2, 1) \
  X(11, 16, 15, 1, 1) \
  X(12, 10, 5, 5, 1) \
  X(13, 15, 9, 2, 1) \
  X(14, 16, 9, 3, 1) \
  X(15, 15, 15, 1, 1) \
  X(16, 15, 9, 3, 1) \
  X(17, 15, 10, 4, 1) \
  X(18, 9, 9, 6, 1) \
  X(19, 16, 12, 3, 1) \
  X(20, 9, 9, 3, 1) \
  X(21, 10, 10, 2, 1) \
  X(22, 15, 12, 3, 1) \
  X(23, 16, 10, 4, 1) \
  X(24, 15, 12, 1, 1) \
  X(25, 15, 10, 1, 1) \
  X(26, 9, 9, 2, 1) \
  X(27, 16, 10, 1, 1) \
  X(28, 12, 9, 2, 1) \
  X(29, 16, 9, 1, 1) \
  X(30, 16, 12, 1, 1) \
  X(31, 15, 15, 3, 1) \
  X(32, 12, 9, 6, 1) \
  X(33, 5, 5, 5, 1) \
  X(34, 15, 8, 1, 1) \
  X(35, 16, 8, 4, 1) \
  X(36, 16, 16, 1, 1) \
  X(37, 15, 9, 1, 1) \
  X(38, 16, 15, 3, 1) \
  X(39, 10, 10, 1, 1) \
  X(40, 12, 9, 1, 1) \
  X(41, 5, 5, 5, 5) \
  X(42, 15, 6, 1, 1) \
  X(43, 9, 9, 9, 1) \
  X(44, 16, 8, 1, 1) \
  X(45, 16, 6, 1, 1) \
  X(46, 15, 5, 1, 1) \
  X(47, 12, 6, 1, 1) \
  X(48, 16, 5, 1, 1) \
  X(49, 9, 9, 1, 1) \
  X(50, 15, 4, 1, 1)

// index of the ragged pass shape with radices rs[0..np), or -1
inline int ragged_shape_index(const int* rs, int np) {
  static const int R[][4] = {
#define GFFT_RAGGED_ROW(i, a, b, c, d) {a, b, c, d},
      GFFT_RAGGED_SHAPES(GFFT_RAGGED_ROW)
#undef GFFT_RAGGED_ROW
  };
  const int ns = (int)(sizeof(R) / sizeof(R[0]));
  for (int i = 0; i < ns; ++i) {
    int n = 0;
    while (n < 4 && R[i][n] > 1) ++n;
    if (n != np) continue;
    bool ok = true;
    for (int p = 0; p < n && ok; ++p) ok = R[i][p] == rs[p];
    if (ok) return i;
  }
  return -1;
}
