// Internal constructors of the device table objects shared between translation units.
#pragma once

#include <cstdint>

struct GB300StencilTable;

namespace gb300 {

// Wraps device buffers (sizes, offsets, indices, w, du, dv, duu, duv, dvv; unused = null, all
// allocated with cudaMalloc / cudaMallocAsync) in a table object that owns them.  numControl =
// largest control index + 1.  Returns null (buffers untouched) when out of host memory.
GB300StencilTable *adopt_stencil_table(int numStencils, int64_t nnz, int numControl,
                                       void *const buf[9]);

}  // namespace gb300
