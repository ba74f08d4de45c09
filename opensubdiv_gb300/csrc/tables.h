// Internal constructors of the device table objects shared between translation units.
#pragma once

#include <cstdint>

struct GB300StencilTable;

namespace gb300 {

// Wraps device buffers (sizes, offsets, indices, w, du, dv, duu, duv, dvv; unused = null, all
// allocated with cudaMalloc) in a table object that owns them.  numControl = largest control
// index + 1.  Returns null (buffers untouched) when out of host memory.
GB300StencilTable *adopt_stencil_table(int numStencils, int64_t nnz, int numControl,
                                       void *const buf[9]);

// Also hands over an evaluation layout (the same stencils sorted by lowest control index:
// sizes, offsets, indices, weights..., as buf) and its outRow map (either may be null).
GB300StencilTable *adopt_stencil_table(int numStencils, int64_t nnz, int numControl,
                                       void *const buf[9], void *const ebuf[9], void *outRow);

}  // namespace gb300
