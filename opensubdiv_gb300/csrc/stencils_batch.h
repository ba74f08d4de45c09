// Batched EvalStencils: the job descriptor and launch interface shared by GB300StencilBatch
// (stencils_batch.cu) and the serving loop (server.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/osd_gb300.h"

namespace gb300 {
namespace batch {

// One mesh's EvalStencils inside a batched launch.  The first fields are the argument view of
// tma::eval_one (one weight array, one output): src / dst include the descriptor offset.
struct Job {
    const float *src;
    float *dst[1];
    const float *w[1];
    int dstStride[1];
    int outOf[1];       // always 0
    int vecDst[1];      // 8: 32-byte aligned rows, 4: 16-byte aligned rows, 0: scalar stores
    const int *indices;
    const int *sizes, *offsets;
    int length, srcStride;
    int vw;             // source rows: 8 = 256-bit loads, 4 = 128-bit loads, 1 = scalar
    int mode;           // 0: one stencil per thread, 1: one stencil per warp, 2: sliced
    int numStencils;
    int tileStencils;   // stencils per tile of this job
    // the table's sliced layout (sell.h), null when absent: mode 2 tiles are kSliceTile slices
    // (one per consumer warp, one stencil per lane) read from it
    const int *slSz, *slSlot, *slIdx, *slRow;
    const float *slW;
    int numSlices;
};

constexpr int kSliceTile = 8;  // slices per tile of a sliced job

// Describes job k = (table, src, dst, length, strides); false (error recorded) on bad input.
// meanSize receives nnz / numStencils.
bool make_job(const GB300StencilTable *table, const float *src, float *dst, int length,
              int srcStride, int dstStride, Job &job, double &meanSize, const char *who);

// Chooses each job's mode and tile size and writes the tile prefix tileBase[0..n] (tileBase[n]
// = total tiles).  Jobs with a sliced layout take mode 2.  Jobs keep their order: tiles are
// handed out in job order.
int plan_tiles(Job *jobs, const double *meanSize, int n, int tileStencils, int warpThreshold,
               int *tileBase);

// One persistent launch over n jobs (device arrays dJobs[n], dTileBase[n + 1]).  dynamic: tiles
// are claimed from the work counter (reset on `s` first), else CTA b takes tiles b, b + grid,
// ...  dStatus receives GB300_ERR_DEVICE_TIMEOUT if a wait gave up.  cls: 0 any job; 1 every
// job is one output 9-12 floats wide over 16-byte aligned rows (the kernel's single 12-wide
// pass); 2 every job is at most 4 floats wide over 16-byte aligned rows (single 4-column pass,
// sliced launches only).  sliced: every job is mode 2 (plan_tiles of jobs that all carry a
// sliced layout).
int launch_jobs(const Job *dJobs, const int *dTileBase, int n, int numTiles, int *dCounter,
                int *dStatus, int ctasPerSm, cudaStream_t s, int dynamic = 1, int cls = 0,
                bool sliced = false);

// Padded copy of one source: rows [0, numRows) of `src` (length <= 16 floats, srcStride
// apart) written to `dst` with a stride of dstStride = 4, 8, 12 or 16 floats (elements >=
// length are 0), so the gathers of an unaligned layout become vector loads: one 128-bit load
// for up to 4 floats, one 256-bit load for 5-8, three 128-bit loads for 9-12 (only the bytes
// used), two 256-bit loads for 13-16.  Values are copied, so results do not change.
struct PadJob {
    const float *src;
    float *dst;
    int srcStride, length;
    long long numRows;
    int dstStride, pad;
};

// Row stride of the padded copy of a source `length` floats wide (0: not padded).
inline int padded_stride(int length) {
    return length <= 4 ? 4 : length <= 8 ? 8 : length <= 12 ? 12 : length <= 16 ? 16 : 0;
}

// One launch over `count` pad jobs (device arrays: jobs, rowBase[count + 1] = prefix of their
// numRows).  Nothing is launched when totalRows is 0.
int launch_pad(const PadJob *dJobs, const long long *dRowBase, int count, long long totalRows,
               cudaStream_t s);

// The same for one source, the job passed by value.
int launch_pad_one(const PadJob &job, cudaStream_t s);

// Rows a stencil table's indices address (its largest control index + 1).
int stencil_table_num_control(const GB300StencilTable *table);

}  // namespace batch
}  // namespace gb300
