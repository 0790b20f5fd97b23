// tmap.cuh — 2-D TMA tensor maps (cuTensorMapEncodeTiled, resolved through the
// runtime so that the library has no link-time dependency on the CUDA driver library).
#pragma once

#include <cuda.h>

#include "common.cuh"

namespace gn {

// rows x inner elements, row pitch row_bytes (a multiple of 16); boxes of
// box_inner x box_rows elements; elements outside the tensor read as zero.
int tmap_encode_2d(CUtensorMap *map, CUtensorMapDataType dtype, const void *base, uint64_t inner, uint64_t rows,
                   uint64_t row_bytes, uint32_t box_inner, uint32_t box_rows, CUtensorMapSwizzle swizzle);

}  // namespace gn
