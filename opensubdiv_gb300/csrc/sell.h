// Sliced evaluation layout of a device stencil table (entry-major per 32 stencils), its
// construction on the device (sell_build.cu) and its EvalStencils launch (stencils_tma.cu).
//
// Positions: the table's stencils in locality order (sorted by lowest control index when
// consecutive stencils jump across the control points, else table order), then sorted by size
// (descending, stable) within windows of 256 positions so that the 32 stencils of a slice have
// similar sizes.  Slice s covers positions [32 s, 32 s + 32); its width is the largest size of
// its stencils, and entry j of the stencil at lane l sits in slot sliceSlot[s] + 32 j + l
// (slots past a stencil's size hold index 0 / weight 0 and are never read).
#pragma once

#include <cuda_runtime.h>

namespace gb300 {

struct SellTable {
    int numSlices = 0;
    const int *sz = nullptr;         // numSlices * 32: size of the stencil at each position
    const int *sliceSlot = nullptr;  // numSlices + 1 slot offsets (slice s: 32 * width slots)
    const int *idx = nullptr;        // slots
    const float *w[6] = {};          // slots, per weight array of the table
    const int *outRow = nullptr;     // numSlices * 32: destination stencil (-1: padding)
};

// Builds the layout of the device CSR table (sizes, offsets, indices, up to 6 weight arrays,
// entries sorted per stencil for the locality order to mean anything) on stream `s` and waits
// for it.  The 10 allocations (sz, sliceSlot, idx, w x 6, outRow) go to `owned` for the caller
// to free; `t` points into them.  GB300_ERR_UNSUPPORTED (nothing allocated): the layout would
// need more than 2^31 - 1 slots.
int build_sell(int numStencils, const int *sizes, const int *offsets, const int *indices,
               const float *const *w, cudaStream_t s, SellTable &t, void *owned[10],
               const char *who);

// Outputs / strides / weights in 6 slots (NULL = absent).
int eval_stencils_sell(const SellTable &t, const float *src, float *const *dst,
                       const int *strides, const float *const *w, int length, int srcStride,
                       cudaStream_t s, const char *who);

}  // namespace gb300
