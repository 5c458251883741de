// Shape arithmetic of the tensor-copy column tiles (variant 9), shared by the
// kernels (col.cuh) and the host (planner.cpp, colshape.cpp).  Plain
// constexpr functions of the element size (8: FP32 complex, 16: FP64
// complex), the pass length L, the tile size tk in KB (64: one block per SM,
// 32: two) and, for the real-pair tiles, rf (0 complex, 1 forward post pass,
// 2 inverse pre pass): no CUDA types.
#pragma once

namespace gfft {
namespace colshape {

// in-lane padding of the work buffer: one slot per 2^ps elements
constexpr int ps(int esz) { return esz == 16 ? 3 : 4; }
// units per tile: tiles of about tk KB, rows of at least 2 units, at most 64
constexpr int lanes(int esz, int L, int tk = 64) {
  return (tk * 1024 / esz) / L > 64 ? 64 : ((tk * 1024 / esz) / L < 2 ? 2 : (tk * 1024 / esz) / L);
}
// Lane stride of the padded work buffer (elements).  Shared memory serves an
// 8-byte request per half-warp (16 threads, 16 slots of 8 bytes) and a
// 16-byte one per quarter-warp (8 slots).  The first pass writes with the
// lane-fastest mapping: a half-warp covers W lanes and 16 / W butterflies
// whose 16 outputs are consecutive, i.e. slots (lane * Lp + j + r) mod 16,
// so Lp = 16 / W mod 16 spreads them over all 16 slots (W <= 16); for
// W >= 16 and for 16-byte elements an odd Lp does the same.  The later
// passes keep a lane's butterflies in consecutive threads and do not depend
// on Lp.
constexpr int lane_stride(int esz, int L, int W) {
  return (esz == 16 || W >= 16) ? (((L + (L >> ps(esz))) & 1) ? L + (L >> ps(esz)) : L + (L >> ps(esz)) + 1)
                                : L + (L >> ps(esz)) + ((((16 / W) % 16) - (L + (L >> ps(esz))) % 16) + 16) % 16;
}
constexpr int round1k(int b) { return ((b + 1023) / 1024) * 1024; }
// threads: one radix-16 butterfly (16 values) each
constexpr int threads(int esz, int L, int tk = 64) { return lanes(esz, L, tk) * L / 16; }
// bytes of the padded work buffer of a complex pass
constexpr int work_bytes(int esz, int L, int tk = 64) {
  return round1k(lanes(esz, L, tk) * lane_stride(esz, L, lanes(esz, L, tk)) * esz);
}
// real-pair tiles: region widths (A: W/2 columns, B: the mirrors, FP32 two
// wider so that its box starts on an even column, C: column S/2)
constexpr int half(int esz, int L) { return lanes(esz, L) / 2; }
constexpr int width_b(int esz, int L, int rf) { return rf ? (esz == 16 ? half(esz, L) : half(esz, L) + 2) : 0; }
constexpr int width_c(int esz, int rf) { return rf ? (esz == 16 ? 1 : 2) : 0; }
constexpr int width_a(int esz, int L, int rf) { return rf ? half(esz, L) : lanes(esz, L); }
// bytes of one stage, and of the work buffer (it also holds a dense tile);
// real-pair tiles exist with 64 KB tiles only
constexpr int stage_bytes(int esz, int L, int rf, int tk = 64) {
  return rf ? (width_a(esz, L, rf) + width_b(esz, L, rf) + width_c(esz, rf)) * L * esz : lanes(esz, L, tk) * L * esz;
}
// a complex tile of a later pass brings its [16][W] block of four-step
// factors W_(16 Ns)^(k r) along (tensor copy into the stage, after the tile)
constexpr int ftw_box_bytes(int esz, int L, int rf, int tk = 64) { return rf ? 0 : 16 * lanes(esz, L, tk) * esz; }
constexpr int stage_stride(int esz, int L, int rf, int tk = 64) {
  return stage_bytes(esz, L, rf, tk) + ftw_box_bytes(esz, L, rf, tk);
}
constexpr int work_bytes_rf(int esz, int L, int rf, int tk = 64) {
  return work_bytes(esz, L, tk) > round1k(stage_bytes(esz, L, rf, tk)) ? work_bytes(esz, L, tk)
                                                                     : round1k(stage_bytes(esz, L, rf, tk));
}
// pass lengths with a kernel: powers of two 64 .. 4096 (FP32) / 2048 (FP64);
// real-pair tiles need two units of each kind (W >= 4 for FP32: an even first
// column of region A); 32 KB tiles for FP32 complex passes of 128 .. 1024
// (rows of 32 bytes or more)
constexpr bool supported(int esz, int L, int rf, int tk = 64) {
  return L >= 64 && (L & (L - 1)) == 0 && L <= (esz == 16 ? 2048 : 4096) &&
         (!rf || (L <= 2048 && (esz == 16 ? lanes(esz, L) >= 2 : lanes(esz, L) >= 4))) &&
         (tk == 64 || (tk == 32 && esz == 8 && !rf && L >= 128 && L <= 1024));
}
// in-block twiddles of a pass, sum over its in-block passes of (R - 1) Ns
// = L - 1 (the product telescopes): the contiguous block of the plan's table
// that the kernel copies to shared memory
constexpr int tw_entries(int L) { return L - 1; }
constexpr int tw_bytes(int esz, int L) { return ((tw_entries(L) * esz + 15) / 16) * 16; }
// shared memory of a launch with `stages` stages: the stages, the work
// buffer, the in-block twiddles and one mbarrier per stage
constexpr long long smem_bytes(int esz, int L, int rf, int stages, int tk = 64) {
  return (long long)stages * stage_stride(esz, L, rf, tk) + work_bytes_rf(esz, L, rf, tk) + tw_bytes(esz, L) +
         8LL * stages;
}

// ---- mixed-radix passes (L not a power of two, colmix.cuh) ----
// units per tile: the largest power of two W <= 64 with W L esz <= 64 KB
// (at least 2)
constexpr int mix_lanes(int esz, int L) {
  int w = 2;
  while (w < 64 && 2LL * w * L * esz <= 65536) w *= 2;
  return w;
}
// rows per tensor box: the largest divisor of L that is at most 256
constexpr int mix_rows(int L) {
  int b = L < 256 ? L : 256;
  while (L % b) --b;
  return b;
}
// padded element index and lane stride of the work buffers: one slot per
// 2^ps elements and one more per 2^(ps+4) (strides of 2^(ps+4) elements
// would otherwise fall on one bank), odd lane stride
constexpr int mix_pad(int esz, int s) { return s + (s >> ps(esz)) + (s >> (ps(esz) + 4)); }
constexpr int mix_stride(int esz, int L) { return (mix_pad(esz, L) + 1) | 1; }
constexpr int mix_threads() { return 512; }
constexpr int mix_stage_bytes(int esz, int L) { return round1k(mix_lanes(esz, L) * L * esz); }
constexpr int mix_work_bytes(int esz, int L) { return round1k(mix_lanes(esz, L) * mix_stride(esz, L) * esz); }
constexpr int mix_tw_bytes(int esz, int L) { return ((L - 1) * esz + 15) / 16 * 16; }
// tensor boxes start on 128-byte boundaries of the stage (and of the dense
// tile a later pass stores from)
constexpr bool mix_supported(int esz, int L) {
  return L >= 64 && (L & (L - 1)) != 0 && (mix_rows(L) * mix_lanes(esz, L) * esz) % 128 == 0;
}
// stages, two work buffers, the in-block twiddles, one mbarrier per stage
constexpr long long mix_smem_bytes(int esz, int L, int stages) {
  return (long long)stages * mix_stage_bytes(esz, L) + 2LL * mix_work_bytes(esz, L) + mix_tw_bytes(esz, L) +
         8LL * stages;
}

}  // namespace colshape
}  // namespace gfft
