// tma_map.cuh - tensor-map encoding shared by the TMA-fed kernels.
#pragma once
#include <cuda.h>

#include <cstdint>

#include "gbblas.h"

namespace gbblas {

// 2-D tensor map over a float32 matrix: `inner` contiguous elements per row,
// `outer` rows `row_stride` elements apart; box of box_inner x box_outer
// elements; 128-byte swizzle (box_inner * 4 must then be 128) or none.
// Out-of-range elements of a box read as zero.  Fails (status, message set)
// when the driver rejects the layout: a base not 16-byte aligned or a row
// stride not a multiple of 16 bytes.
// 3-D tensor map over `planes` planes of rows x cols (cols contiguous) BF16
// (bytes = false) or 8-bit elements, planes one after another; box of
// box_rows x row_bytes (128 or 64 bytes of a row) x all planes, with the
// swizzle of that row width.
gbblas_status make_map(CUtensorMap* map, const void* base, uint64_t rows, uint64_t cols, uint64_t planes,
                       uint32_t box_rows, bool bytes, uint32_t row_bytes);

gbblas_status make_map_f32_2d(CUtensorMap* map, const float* base, uint64_t inner, uint64_t outer,
                              uint64_t row_stride, uint32_t box_inner, uint32_t box_outer, bool swizzle128);

}  // namespace gbblas
