// Host side of the column-tile shapes (colshape.h): what the planner asks
// of a variant-9 pass, without CUDA.
#include <cstddef>

#include "colshape.h"
#include "mixed_shapes.h"

// Shape of the variant-9 pass of length L (rf: 0 complex, 1 / 2 real
// forward post / inverse pre pass; tk: tile KB, 64 or 32): units per tile,
// threads, and the shared memory of `stages` stages; 1 if L (or the real
// pass, or the tile size) has no kernel.
extern "C" int gfft_col_shape(int dbl, int L, int stages, int rf, int tk, int* units, int* threads, size_t* smem) {
  using namespace gfft::colshape;
  const int esz = dbl ? 16 : 8;
  if (!supported(esz, L, rf, tk) || stages < 1 || !units || !threads || !smem) return 1;
  *units = lanes(esz, L, tk);
  *threads = gfft::colshape::threads(esz, L, tk);
  *smem = (size_t)smem_bytes(esz, L, rf, stages, tk);
  return 0;
}

// Shape of the mixed-radix pass (colmix.cuh) of length L with radices
// rs[0..np), moved by tensor copies (gather 0) or cp.async gathers (gather
// 1, at most two stages): units per tile, threads, and the dynamic shared
// memory of `stages` stages; 1 if the shape has no such kernel.
extern "C" int gfft_colmix_shape(int dbl, int L, const int* rs, int np, int stages, int gather, int* units,
                                 int* threads, size_t* smem) {
  using namespace gfft::colshape;
  const int esz = dbl ? 16 : 8;
  if (!rs || !units || !threads || !smem || stages < 1 || np > 4 || (gather && stages > 2)) return 1;
  if (mixed_shape_index(L, rs, np) < 0 || (!gather && !mix_supported(esz, L))) return 1;
  *units = mix_lanes(esz, L);
  *threads = mix_threads();
  *smem = (size_t)mix_smem_bytes(esz, L, stages);
  return 0;
}
