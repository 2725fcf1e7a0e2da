// Host-side TMA tensor maps for BF16 row-major matrices (K contiguous),
// loaded as 128B-swizzled tiles of 64 elements x `box_rows` rows.
#pragma once
#include <cuda.h>
#include <stdint.h>

namespace racer {

// rows x cols matrix with `ld` elements between rows (ld * 2 must be a multiple
// of 16; base 16-byte aligned). Out-of-range boxes read zeros.
int make_tmap_bf16(CUtensorMap* map, const void* base, uint64_t rows, uint64_t cols, uint64_t ld, uint32_t box_rows);

// FP32 rows x cols matrix (cols contiguous, `ld` elements between rows; ld * 4
// a multiple of 16, base 16-byte aligned) loaded unswizzled as boxes of
// box_cols x box_rows; out-of-range elements read zero.
int make_tmap_f32(CUtensorMap* map, const void* base, uint64_t rows, uint64_t cols, uint64_t ld, uint32_t box_cols,
                  uint32_t box_rows);

}  // namespace racer
