// Internal constructors of the device table objects shared between translation units.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

struct GB300StencilTable;

namespace gb300 {

struct SellTable;

// The table's sliced evaluation layout (numSlices 0 when it has none).
const SellTable *stencil_table_sell(const GB300StencilTable *table);

// Wraps device buffers (sizes, offsets, indices, w, du, dv, duu, duv, dvv; unused = null, all
// allocated with cudaMalloc) in a table object that owns them, and builds its sliced
// evaluation layout on stream `s`.  numControl = largest control index + 1.  Returns null
// (buffers untouched, status recorded) when out of host memory or when the layout build
// fails.
GB300StencilTable *adopt_stencil_table(int numStencils, int64_t nnz, int numControl,
                                       void *const buf[9], cudaStream_t s, const char *who);

}  // namespace gb300
