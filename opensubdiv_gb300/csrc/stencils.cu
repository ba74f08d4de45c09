// EvalStencils for sm_103a: dst[i] = sum_j w[o_i + j] * src[idx[o_i + j]] over a
// Far::StencilTable (far/stencilTable.h:141-269), the value and all derivative outputs of a
// Far::LimitStencilTable in one pass.
//
// The work is a sparse weighted gather, bandwidth bound on the table stream (8 B per entry
// plus 4 B per extra derivative weight) and on the output stream; the source rows are small
// and stay L1/L2 resident.  Mapping: a group of G = nextpow2(min(length, 32)) lanes owns one
// stencil; lane l owns element l of the primvar, so every source-row fetch is one coalesced
// segment.  The group loads G table entries at a time with coalesced streaming loads and
// broadcasts them with shuffles; accumulation is in registers (the reference's generic
// kernel accumulates in global memory, osd/cudaKernel.cu:102-130).
#include "common.cuh"
#include "patchmap.h"

namespace gb300 {

int eval_stencils_staged(const float *src, float *const *dst, const int *strides,
                         const float *const *w, int length, int srcStride, const int *sizes,
                         const int *offsets, const int *indices, int start, int end,
                         cudaStream_t s);

struct StencilArgs {
    const float *src;
    float *dst[6];
    const float *w[6];
    int dstStride[6];
    const int *sizes;
    const int *offsets;
    const int *indices;
    int length;
    int srcStride;
    int active;  // bit k set: output k is written (its weights are read)
    int start;
    int end;
};

template <int G, int NOUT>
__global__ void __launch_bounds__(256) k_stencils_group(const StencilArgs a) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & (G - 1);
    const int group = tid / G;
    const int ngroups = (gridDim.x * blockDim.x) / G;
    const unsigned gmask =
        (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
    const uint64_t pol_stream = l2_evict_first(), pol_src = l2_evict_last();

    for (int i = a.start + group; i < a.end; i += ngroups) {
        const int n = __ldg(a.sizes + i);
        const int o = __ldg(a.offsets + i);
        for (int e0 = 0; e0 < a.length; e0 += G) {
            const int e = e0 + lane;
            const bool has_e = e < a.length;
            float acc[NOUT];
#pragma unroll
            for (int k = 0; k < NOUT; ++k) acc[k] = 0.0f;
            for (int j = 0; j < n; j += G) {
                const int jj = j + lane;
                int idx = 0;
                float w[NOUT];
#pragma unroll
                for (int k = 0; k < NOUT; ++k) w[k] = 0.0f;
                if (jj < n) {
                    idx = ld_stream(a.indices + o + jj, pol_stream);
#pragma unroll
                    for (int k = 0; k < NOUT; ++k)
                        if (a.active & (1 << k)) w[k] = ld_stream(a.w[k] + o + jj, pol_stream);
                }
                const int cnt = min(G, n - j);
                for (int t = 0; t < cnt; ++t) {
                    const int id = __shfl_sync(gmask, idx, t, G);
                    float wk[NOUT];
#pragma unroll
                    for (int k = 0; k < NOUT; ++k) wk[k] = __shfl_sync(gmask, w[k], t, G);
                    const float x = has_e ? ld_src(a.src + (size_t)id * a.srcStride + e, pol_src) : 0.0f;
#pragma unroll
                    for (int k = 0; k < NOUT; ++k) acc[k] = fmaf(wk[k], x, acc[k]);
                }
            }
            if (has_e) {
#pragma unroll
                for (int k = 0; k < NOUT; ++k)
                    if (a.active & (1 << k))
                        st_stream(a.dst[k] + (size_t)i * a.dstStride[k] + e, acc[k]);
            }
        }
    }
}

template <int NOUT>
static void launch_group(const StencilArgs &a, int G, cudaStream_t s) {
    const int threads = 256;
    long long groups = (long long)(a.end - a.start);
    long long blocks = (groups * G + threads - 1) / threads;
    long long cap = (long long)num_sms() * 16;
    int grid = (int)(blocks < cap ? blocks : cap);
    if (grid < 1) grid = 1;
    switch (G) {
        case 1: k_stencils_group<1, NOUT><<<grid, threads, 0, s>>>(a); break;
        case 2: k_stencils_group<2, NOUT><<<grid, threads, 0, s>>>(a); break;
        case 4: k_stencils_group<4, NOUT><<<grid, threads, 0, s>>>(a); break;
        case 8: k_stencils_group<8, NOUT><<<grid, threads, 0, s>>>(a); break;
        case 16: k_stencils_group<16, NOUT><<<grid, threads, 0, s>>>(a); break;
        default: k_stencils_group<32, NOUT><<<grid, threads, 0, s>>>(a); break;
    }
    count_launch();
}

static int group_width(int length) {
    int g = 1;
    while (g < length && g < 32) g <<= 1;
    return g;
}

// Validates and launches.  outputs/strides/weights hold 6 slots (NULL = absent).
int eval_stencils(const float *src, float *const *dst, const int *strides,
                  const float *const *w, int length, int srcStride, const int *sizes,
                  const int *offsets, const int *indices, int start, int end, cudaStream_t s,
                  const char *who) {
    if (end <= start) return ok();
    if (start < 0) return fail(GB300_ERR_INVALID_ARGUMENT, "%s: start < 0", who);
    if (!src || !sizes || !offsets || !indices)
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: null source or table pointer", who);
    if (length <= 0 || srcStride < length)
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: bad length %d / source stride %d", who,
                    length, srcStride);
    StencilArgs a{};
    a.src = src;
    a.sizes = sizes;
    a.offsets = offsets;
    a.indices = indices;
    a.length = length;
    a.srcStride = srcStride;
    a.start = start;
    a.end = end;
    int last = -1;
    for (int k = 0; k < 6; ++k) {
        if (!dst[k]) continue;
        if (!w[k]) return fail(GB300_ERR_INVALID_ARGUMENT, "%s: output %d has no weights", who, k);
        if (strides[k] < length)
            return fail(GB300_ERR_INVALID_ARGUMENT, "%s: output %d stride %d < length %d", who, k,
                        strides[k], length);
        a.dst[k] = dst[k];
        a.w[k] = w[k];
        a.dstStride[k] = strides[k];
        a.active |= 1 << k;
        last = k;
    }
    if (last < 0) return ok();
    // staged kernel first (16-byte aligned tables); the group kernel covers everything else
    const int staged = eval_stencils_staged(src, a.dst, a.dstStride, a.w, length, srcStride,
                                            sizes, offsets, indices, start, end, s);
    if (staged == GB300_OK) return check_launch(who);
    if (staged != GB300_ERR_UNSUPPORTED) return staged;
    const int G = group_width(length);
    if (last == 0)
        launch_group<1>(a, G, s);
    else if (last <= 2)
        launch_group<3>(a, G, s);
    else
        launch_group<6>(a, G, s);
    return check_launch(who);
}

}  // namespace gb300

using namespace gb300;

extern "C" {

int GB300EvalStencils(const float *src, float *dst, int length, int srcStride, int dstStride,
                      const int *sizes, const int *offsets, const int *indices,
                      const float *weights, int start, int end, void *stream) {
    if (!dst) return fail(GB300_ERR_INVALID_ARGUMENT, "GB300EvalStencils: null destination");
    float *d[6] = {dst, 0, 0, 0, 0, 0};
    int st[6] = {dstStride, 0, 0, 0, 0, 0};
    const float *w[6] = {weights, 0, 0, 0, 0, 0};
    return eval_stencils(src, d, st, w, length, srcStride, sizes, offsets, indices, start, end,
                         as_stream(stream), "GB300EvalStencils");
}

int GB300EvalStencilsWithDerivatives(
    const float *src, float *dst, float *du, float *dv, float *duu, float *duv, float *dvv,
    int length, int srcStride, int dstStride, int duStride, int dvStride, int duuStride,
    int duvStride, int dvvStride, const int *sizes, const int *offsets, const int *indices,
    const float *weights, const float *duWeights, const float *dvWeights,
    const float *duuWeights, const float *duvWeights, const float *dvvWeights, int start,
    int end, void *stream) {
    float *d[6] = {dst, du, dv, duu, duv, dvv};
    int st[6] = {dstStride, duStride, dvStride, duuStride, duvStride, dvvStride};
    const float *w[6] = {weights, duWeights, dvWeights, duuWeights, duvWeights, dvvWeights};
    return eval_stencils(src, d, st, w, length, srcStride, sizes, offsets, indices, start, end,
                         as_stream(stream), "GB300EvalStencilsWithDerivatives");
}

}  // extern "C"
