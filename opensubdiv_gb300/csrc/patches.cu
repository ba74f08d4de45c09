// EvalPatches for sm_103a: one thread per patch coordinate; PatchParam decode, basis and the
// gather of up to 20 control points are fused and kept in registers, and all requested
// outputs (P, dPdu, dPdv, dPduu, dPduv, dPdvv) come out of one pass.  Replaces
// computePatches (osd/cudaKernel.cu:244-328), which spills six float[20] weight arrays and
// accumulates each output in global memory.
#include "common.cuh"
#include "patch_basis.cuh"

namespace gb300 {

struct Coord {
    int arrayIndex, patchIndex, vertIndex;
    float s, t;
};
struct Array {
    int regDesc, desc, numPatches, indexBase, stride, primitiveIdBase;
};
struct ParamRec {
    int field0, field1;
    float sharpness;
};

// A query's patch coordinate (read once: evict-first) and its patch's param (evict-last).
__device__ __forceinline__ Coord load_coord(const Coord *p) {
    const int *q = reinterpret_cast<const int *>(p);
    const uint64_t pol = l2_evict_first();
    Coord c;
    c.arrayIndex = ld_stream(q, pol);
    c.patchIndex = ld_stream(q + 1, pol);
    c.vertIndex = ld_stream(q + 2, pol);
    c.s = __int_as_float(ld_stream(q + 3, pol));
    c.t = __int_as_float(ld_stream(q + 4, pol));
    return c;
}
__device__ __forceinline__ ParamRec load_param(const ParamRec *p) {
    const int *q = reinterpret_cast<const int *>(p);
    const uint64_t pol = l2_evict_last();
    return ParamRec{ld_keep(q, pol), ld_keep(q + 1, pol), __int_as_float(ld_keep(q + 2, pol))};
}

struct PatchArgs {
    const float *src;
    float *dst[6];
    int dstStride[6];
    int active;
    int length;
    int srcStride;
    int numCoords;
    const Coord *coords;
    const Array *arrays;
    const int *indices;
    const ParamRec *params;
};

// Highest output index a derivative order needs: 0 P only, 1 P + du + dv, 2 all six.  The
// kernels are instantiated per order so the unused accumulations compile away.
__host__ __device__ constexpr int last_output(int order) { return order == 0 ? 0 : order == 1 ? 2 : 5; }

// 5 resident blocks per SM where the registers allow it without spills (0.2847 vs 0.2908 ms
// for 4 M Loop points at LC = 3; LC = 4 would spill)
// QUAD: Catmull-Clark tables (REGULAR / GREGORY_BASIS / QUADS only): without the Loop and
// triangle bases the kernel fits 7 blocks per SM for orders 0 and 1 without spills.
template <int LC, int ORDER, bool QUAD = false>
__global__ void __launch_bounds__(128, LC == 4 ? 4 : (ORDER < 2 ? (QUAD ? 7 : 6) : 5))
    k_eval_patches(const PatchArgs a) {
    const int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.numCoords; i += stride) {
        const Coord c = load_coord(a.coords + i);
        for (int e0 = 0; e0 < a.length; e0 += LC) {
            Acc6<LC> acc;
            acc.zero();
            float d1 = 1.0f, d2 = 1.0f;
            if (c.arrayIndex >= 0) {
                const Array arr = a.arrays[c.arrayIndex];
                const ParamRec pr = load_param(a.params + c.patchIndex);
                const Param p{pr.field0, pr.field1};
                const int type = p.regular() ? arr.regDesc : arr.desc;
                const int *cvs =
                    a.indices + arr.indexBase + arr.stride * (c.patchIndex - arr.primitiveIdBase);
                if (!eval_patch_point<LC, QUAD>(type, p, c.s, c.t, cvs, a.src, a.srcStride, e0,
                                                a.length, acc, d1, d2))
                    acc.zero();
            }
            const float scale[6] = {1.0f, d1, d1, d2, d2, d2};
#pragma unroll
            for (int k = 0; k <= last_output(ORDER); ++k) {
                if (!(a.active & (1 << k))) continue;
                float *out = a.dst[k] + (size_t)i * a.dstStride[k] + e0;
#pragma unroll
                for (int m = 0; m < LC; ++m)
                    if (e0 + m < a.length) st_stream(out + m, acc.v[k][m] * scale[k]);
            }
        }
    }
}

// G lanes per point, lane l owning primvar elements l, l + G, ...: one source-row fetch is a
// single coalesced access for the whole group, the accumulators are per element (6 per
// lane) and no cross-lane reduction is needed.  The basis is evaluated by every lane of the
// group (cheap for the separable quad-family bases this kernel is used for).
template <int G, int ORDER>
__global__ void __launch_bounds__(256, 4) k_eval_patches_lanes(const PatchArgs a) {
    // G need not be a power of two: a warp holds floor(32 / G) groups (3 lanes per point
    // for xyz: 10 points per warp) and its remaining lanes stay idle
    constexpr int kPerWarp = 32 / G;
    const int wl = threadIdx.x & 31;
    const int slot = wl / G;
    if (slot >= kPerWarp) return;
    const int lane = wl - slot * G;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int group = warp * kPerWarp + slot;
    const int ngroups = nwarps * kPerWarp;
    for (int i = group; i < a.numCoords; i += ngroups) {
        const Coord c = load_coord(a.coords + i);
        for (int e0 = 0; e0 < a.length; e0 += G) {
            const int e = e0 + lane;
            Acc6<1> acc;
            acc.zero();
            float d1 = 1.0f, d2 = 1.0f;
            if (c.arrayIndex >= 0) {
                const Array arr = a.arrays[c.arrayIndex];
                const ParamRec pr = load_param(a.params + c.patchIndex);
                const Param p{pr.field0, pr.field1};
                const int type = p.regular() ? arr.regDesc : arr.desc;
                const int *cvs =
                    a.indices + arr.indexBase + arr.stride * (c.patchIndex - arr.primitiveIdBase);
                if (!eval_patch_point<1, true>(type, p, c.s, c.t, cvs, a.src, a.srcStride, e,
                                               a.length, acc, d1, d2))
                    acc.zero();
            }
            if (e < a.length) {
                const float scale[6] = {1.0f, d1, d1, d2, d2, d2};
#pragma unroll
                for (int k = 0; k <= last_output(ORDER); ++k)
                    if (a.active & (1 << k))
                        st_stream(a.dst[k] + (size_t)i * a.dstStride[k] + e, acc.v[k][0] * scale[k]);
            }
        }
    }
}

template <int ORDER>
void launch_lanes(int G, int grid, int threads, cudaStream_t s, const PatchArgs &a) {
    switch (G) {
        case 1: k_eval_patches_lanes<1, ORDER><<<grid, threads, 0, s>>>(a); break;
        case 2: k_eval_patches_lanes<2, ORDER><<<grid, threads, 0, s>>>(a); break;
        case 3: k_eval_patches_lanes<3, ORDER><<<grid, threads, 0, s>>>(a); break;
        case 4: k_eval_patches_lanes<4, ORDER><<<grid, threads, 0, s>>>(a); break;
        case 6: k_eval_patches_lanes<6, ORDER><<<grid, threads, 0, s>>>(a); break;
        case 8: k_eval_patches_lanes<8, ORDER><<<grid, threads, 0, s>>>(a); break;
        default: k_eval_patches_lanes<32, ORDER><<<grid, threads, 0, s>>>(a); break;
    }
}

template <int ORDER, bool QUAD>
void launch_points(int length, int grid, int threads, cudaStream_t s, const PatchArgs &a) {
    switch (length) {
        case 1: k_eval_patches<1, ORDER, QUAD><<<grid, threads, 0, s>>>(a); break;
        case 2: k_eval_patches<2, ORDER, QUAD><<<grid, threads, 0, s>>>(a); break;
        case 3: k_eval_patches<3, ORDER, QUAD><<<grid, threads, 0, s>>>(a); break;
        default: k_eval_patches<4, ORDER, QUAD><<<grid, threads, 0, s>>>(a); break;
    }
}

int eval_patches(const float *src, float *const *dst, const int *strides, int length,
                 int srcStride, int numCoords, const void *coords, const void *arrays,
                 const int *indices, const void *params, cudaStream_t s, const char *who,
                 int quadFamily, int grouped) {
    if (numCoords <= 0) return ok();
    if (!src || !coords || !arrays || !indices || !params)
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: null source, coord or table pointer", who);
    if (length <= 0 || srcStride < length)
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: bad length %d / source stride %d", who,
                    length, srcStride);
    PatchArgs a{};
    a.src = src;
    a.length = length;
    a.srcStride = srcStride;
    a.numCoords = numCoords;
    a.coords = (const Coord *)coords;
    a.arrays = (const Array *)arrays;
    a.indices = indices;
    a.params = (const ParamRec *)params;
    for (int k = 0; k < 6; ++k) {
        if (!dst[k]) continue;
        if (strides[k] < length)
            return fail(GB300_ERR_INVALID_ARGUMENT, "%s: output %d stride %d < length %d", who, k,
                        strides[k], length);
        a.dst[k] = dst[k];
        a.dstStride[k] = strides[k];
        a.active |= 1 << k;
    }
    if (!a.active) return ok();
    const int order = (a.active & 0x38) ? 2 : (a.active & 0x6) ? 1 : 0;
    if (quadFamily && !grouped) {
        // element-lane kernel: G = length lanes per point for the common widths, else 32
        // lanes looping over element chunks
        const int G = (length <= 4 || length == 6 || length == 8) ? length : 32;
        const int perWarp = 32 / G;
        const int threads = 256;
        long long warps = ((long long)numCoords + perWarp - 1) / perWarp;
        long long blocks = (warps * 32 + threads - 1) / threads;
        long long cap = (long long)num_sms() * 16;
        const int grid = (int)(blocks < cap ? blocks : cap);
        if (order == 0) launch_lanes<0>(G, grid, threads, s, a);
        else if (order == 1) launch_lanes<1>(G, grid, threads, s, a);
        else launch_lanes<2>(G, grid, threads, s, a);
        count_launch();
        return check_launch(who);
    }
    // one thread per point: tables with triangle patches, and points grouped by patch (a
    // tessellation's coords), whose row loads are shared by the warp and whose basis each
    // thread then computes once rather than once per element lane
    const int threads = 128;
    long long blocks = ((long long)numCoords + threads - 1) / threads;
    long long cap = (long long)num_sms() * 32;
    const int grid = (int)(blocks < cap ? blocks : cap);
    if (quadFamily) {
        if (order == 0) launch_points<0, true>(length, grid, threads, s, a);
        else if (order == 1) launch_points<1, true>(length, grid, threads, s, a);
        else launch_points<2, true>(length, grid, threads, s, a);
    } else {
        if (order == 0) launch_points<0, false>(length, grid, threads, s, a);
        else if (order == 1) launch_points<1, false>(length, grid, threads, s, a);
        else launch_points<2, false>(length, grid, threads, s, a);
    }
    count_launch();
    return check_launch(who);
}

}  // namespace gb300

using namespace gb300;

extern "C" {

int GB300EvalPatches(const float *src, float *dst, int length, int srcStride, int dstStride,
                     int numPatchCoords, const void *patchCoords, const void *patchArrays,
                     const int *patchIndices, const void *patchParams, void *stream) {
    if (!dst) return fail(GB300_ERR_INVALID_ARGUMENT, "GB300EvalPatches: null destination");
    float *d[6] = {dst, 0, 0, 0, 0, 0};
    int st[6] = {dstStride, 0, 0, 0, 0, 0};
    return eval_patches(src, d, st, length, srcStride, numPatchCoords, patchCoords, patchArrays,
                        patchIndices, patchParams, as_stream(stream), "GB300EvalPatches", 0, 0);
}

int GB300EvalPatchesWithDerivatives(
    const float *src, float *dst, float *du, float *dv, float *duu, float *duv, float *dvv,
    int length, int srcStride, int dstStride, int duStride, int dvStride, int duuStride,
    int duvStride, int dvvStride, int numPatchCoords, const void *patchCoords,
    const void *patchArrays, const int *patchIndices, const void *patchParams, void *stream) {
    float *d[6] = {dst, du, dv, duu, duv, dvv};
    int st[6] = {dstStride, duStride, dvStride, duuStride, duvStride, dvvStride};
    return eval_patches(src, d, st, length, srcStride, numPatchCoords, patchCoords, patchArrays,
                        patchIndices, patchParams, as_stream(stream),
                        "GB300EvalPatchesWithDerivatives", 0, 0);
}

}  // extern "C"
