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
