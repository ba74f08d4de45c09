// Draw-time tessellation factors of OpenSubdiv's patch shaders, for every patch of a device
// table at once: the per-patch math of the tess-control stage (osd/glslPatchCommonTess.glsl:
// 92-550) and the transition-edge reparameterization of the tess-evaluation stage (:607-760).
//
// One thread per patch.  Uniform factors depend only on the patch's refinement level and
// transition mask (OsdGetTessLevelsUniform[Triangle]).  Screen-space factors project the
// bounding sphere of each boundary edge -- or of each half of a transition edge -- through the
// client's model-view and projection matrices (OsdComputeTessLevel); the edge end points are the
// patch's limit positions at its corners and, on transition edges, at the edge midpoints,
// which is what the shaders take from the patch's Bezier form (OsdEvalPatchBezierTessLevels,
// OsdEvalPatchBezierTriangleTessLevels: Bezier patches interpolate their corners and the
// boundary curve midpoints are limit points).  The patch is evaluated here with the same
// device bases as EvalPatches.  Outer and inner levels then follow the spacing mode
// (OsdComputeTessLevels[Triangle]).
#include "common.cuh"
#include "patch_basis.cuh"
#include "patchmap.h"

namespace gb300 {
namespace {

struct TfArray {
    int regDesc, desc, numPatches, indexBase, stride, primitiveIdBase;
};

struct TfArgs {
    const TfArray *arrays;
    int numArrays, numPatches;
    const int *indices;
    const int *params;  // 3 x 32 bits per patch
    const float *src;
    int srcStride;
    GB300PatchTessOptions o;
    float *outer, *inner, *lo, *hi;
};

// Limit position of patch (type, param) at patch-local (s, t).
__device__ __forceinline__ float3 limit_point(int type, Param p, float s, float t, const int *cvs,
                                              const float *src, int stride) {
    Acc6<3> acc;
    acc.zero();
    switch (type) {
        case 6: eval_bspline<3>(s, t, p.boundary(), cvs, src, stride, 0, 3, acc); break;
        case 9: eval_gregory<3>(s, t, cvs, src, stride, 0, 3, acc); break;
        case 5: eval_box_tri<3>(s, t, p.boundary(), cvs, src, stride, 0, 3, acc); break;
        case 10: eval_gregory_tri<3>(s, t, cvs, src, stride, 0, 3, acc); break;
        case 3: eval_linear_quad<3>(s, t, cvs, src, stride, 0, 3, acc); break;
        case 4: eval_linear_tri<3>(s, t, cvs, src, stride, 0, 3, acc); break;
        default: break;
    }
    return make_float3(acc.v[0][0], acc.v[0][1], acc.v[0][2]);
}

// m * (x, 1) for a column-major 4x4 matrix (GLSL mat4 layout)
__device__ __forceinline__ float4 xform(const float *m, float3 x) {
    return make_float4(m[0] * x.x + m[4] * x.y + m[8] * x.z + m[12],
                       m[1] * x.x + m[5] * x.y + m[9] * x.z + m[13],
                       m[2] * x.x + m[6] * x.y + m[10] * x.z + m[14],
                       m[3] * x.x + m[7] * x.y + m[11] * x.z + m[15]);
}

// OsdComputeTessLevel (glslPatchCommonTess.glsl:98-117): the projected diameter of the edge's
// bounding sphere times the tess level, at least 1 and at most half the device maximum.
__device__ float edge_level(const GB300PatchTessOptions &o, float3 p0, float3 p1) {
    const float4 a = xform(o.modelView, p0), b = xform(o.modelView, p1);
    const float3 c = make_float3((a.x + b.x) * 0.5f, (a.y + b.y) * 0.5f, (a.z + b.z) * 0.5f);
    const float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    const float diameter = sqrtf(dx * dx + dy * dy + dz * dz);
    const float4 q = xform(o.projection, c);
    const float proj = fabsf(diameter * o.projection[5] / q.w);
    return fminf(fmaxf(1.0f, o.tessLevel * proj), o.maxTessLevel * 0.5f);
}

__device__ __forceinline__ float round_up_even(float x) { return 2.0f * ceilf(x * 0.5f); }
__device__ __forceinline__ float round_up_odd(float x) { return 2.0f * ceilf((x + 1.0f) * 0.5f) - 1.0f; }

__global__ void __launch_bounds__(128) k_tess_factors(const TfArgs a) {
    const int stride = gridDim.x * blockDim.x;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.numPatches; p += stride) {
        int k = 0;
        while (k < a.numArrays && !(p >= a.arrays[k].primitiveIdBase &&
                                    p < a.arrays[k].primitiveIdBase + a.arrays[k].numPatches))
            ++k;
        float lo[4] = {0, 0, 0, 0}, hi[4] = {0, 0, 0, 0}, outer[4], inner[2];
        if (k == a.numArrays) {
            for (int e = 0; e < 4; ++e) outer[e] = 0.0f, lo[e] = hi[e] = 0.0f;
            inner[0] = inner[1] = 0.0f;
        } else {
            const TfArray arr = a.arrays[k];
            const Param prm{a.params[3 * p], a.params[3 * p + 1]};
            const int type = prm.regular() ? arr.regDesc : arr.desc;
            const bool tri = type == 4 || type == 5 || type == 10;
            const int transition = (prm.f0 >> 28) & 0xf;
            if (!a.o.screenSpace) {
                // OsdGetTessLevelsUniform[Triangle] (glslPatchCommonTess.glsl:119-163)
                const float level =
                    fminf(a.o.tessLevel, a.o.maxTessLevel) / ldexpf(1.0f, prm.depth() - 1);
                const int m[4] = {tri ? (transition >> 2) & 1 : (transition >> 3) & 1,
                                  transition & 1, (transition >> 1) & 1,
                                  tri ? 0 : (transition >> 2) & 1};
#pragma unroll
                for (int e = 0; e < 4; ++e) lo[e] = fmaxf(level, 1.0f + (float)m[e]);
            } else {
                const int *cvs = a.indices + arr.indexBase + arr.stride * (p - arr.primitiveIdBase);
                if (!tri) {
                    // Osd_GetTessLevelsFromPatchBoundaries4 (glslPatchCommonTess.glsl:231-264)
                    const float3 c0 = limit_point(type, prm, 0.0f, 0.0f, cvs, a.src, a.srcStride);
                    const float3 c1 = limit_point(type, prm, 1.0f, 0.0f, cvs, a.src, a.srcStride);
                    const float3 c2 = limit_point(type, prm, 1.0f, 1.0f, cvs, a.src, a.srcStride);
                    const float3 c3 = limit_point(type, prm, 0.0f, 1.0f, cvs, a.src, a.srcStride);
                    if (transition & 8) {
                        const float3 m = limit_point(type, prm, 0.0f, 0.5f, cvs, a.src, a.srcStride);
                        lo[0] = edge_level(a.o, c0, m);
                        hi[0] = edge_level(a.o, c3, m);
                    } else {
                        lo[0] = edge_level(a.o, c0, c3);
                    }
                    if (transition & 1) {
                        const float3 m = limit_point(type, prm, 0.5f, 0.0f, cvs, a.src, a.srcStride);
                        lo[1] = edge_level(a.o, c0, m);
                        hi[1] = edge_level(a.o, c1, m);
                    } else {
                        lo[1] = edge_level(a.o, c0, c1);
                    }
                    if (transition & 2) {
                        const float3 m = limit_point(type, prm, 1.0f, 0.5f, cvs, a.src, a.srcStride);
                        lo[2] = edge_level(a.o, c1, m);
                        hi[2] = edge_level(a.o, c2, m);
                    } else {
                        lo[2] = edge_level(a.o, c1, c2);
                    }
                    if (transition & 4) {
                        const float3 m = limit_point(type, prm, 0.5f, 1.0f, cvs, a.src, a.srcStride);
                        lo[3] = edge_level(a.o, c3, m);
                        hi[3] = edge_level(a.o, c2, m);
                    } else {
                        lo[3] = edge_level(a.o, c3, c2);
                    }
                } else {
                    // Osd_GetTessLevelsFromPatchBoundaries3 (glslPatchCommonTess.glsl:266-293)
                    const float3 c0 = limit_point(type, prm, 0.0f, 0.0f, cvs, a.src, a.srcStride);
                    const float3 c1 = limit_point(type, prm, 1.0f, 0.0f, cvs, a.src, a.srcStride);
                    const float3 c2 = limit_point(type, prm, 0.0f, 1.0f, cvs, a.src, a.srcStride);
                    if (transition & 4) {
                        const float3 m = limit_point(type, prm, 0.0f, 0.5f, cvs, a.src, a.srcStride);
                        lo[0] = edge_level(a.o, c0, m);
                        hi[0] = edge_level(a.o, c2, m);
                    } else {
                        lo[0] = edge_level(a.o, c0, c2);
                    }
                    if (transition & 1) {
                        const float3 m = limit_point(type, prm, 0.5f, 0.0f, cvs, a.src, a.srcStride);
                        lo[1] = edge_level(a.o, c0, m);
                        hi[1] = edge_level(a.o, c1, m);
                    } else {
                        lo[1] = edge_level(a.o, c0, c1);
                    }
                    if (transition & 2) {
                        const float3 m = limit_point(type, prm, 0.5f, 0.5f, cvs, a.src, a.srcStride);
                        lo[2] = edge_level(a.o, c2, m);
                        hi[2] = edge_level(a.o, c1, m);
                    } else {
                        lo[2] = edge_level(a.o, c1, c2);
                    }
                }
            }
            // OsdComputeTessLevels[Triangle] (glslPatchCommonTess.glsl:413-500)
            float comb[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) comb[e] = lo[e] + hi[e];
            if (a.o.spacing == 1) {
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    outer[e] = hi[e] > 0.0f ? round_up_even(lo[e]) + round_up_even(hi[e]) : comb[e];
            } else if (a.o.spacing == 2) {
                bool split = false;
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    outer[e] = hi[e] > 0.0f ? round_up_odd(lo[e]) + round_up_odd(hi[e]) : comb[e];
                    split = split || hi[e] > 0.0f;
                }
                if (split)
#pragma unroll
                    for (int e = 0; e < 4; ++e) comb[e] = fmaxf(3.0f, comb[e]);
            } else {
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    lo[e] = roundf(lo[e]);
                    hi[e] = roundf(hi[e]);
                    comb[e] = lo[e] + hi[e];
                    outer[e] = comb[e];
                }
            }
            inner[0] = (comb[1] + comb[3]) * 0.5f;
            inner[1] = (comb[0] + comb[2]) * 0.5f;
            if (tri) inner[0] = fmaxf(fmaxf(outer[0], outer[1]), outer[2]);
        }
        const size_t q = (size_t)p;
        reinterpret_cast<float4 *>(a.outer)[q] = make_float4(outer[0], outer[1], outer[2], outer[3]);
        reinterpret_cast<float2 *>(a.inner)[q] = make_float2(inner[0], inner[1]);
        if (a.lo) reinterpret_cast<float4 *>(a.lo)[q] = make_float4(lo[0], lo[1], lo[2], lo[3]);
        if (a.hi) reinterpret_cast<float4 *>(a.hi)[q] = make_float4(hi[0], hi[1], hi[2], hi[3]);
    }
}

// OsdGetTessFractionalSplit (glslPatchCommonTess.glsl:607-645)
__device__ float fractional_split(float t, float level, float levelUp, int spacing) {
    float offset;
    if (spacing == 1) {
        if (level <= 2.0f) return t;
        const float base = exp2f(floorf(log2f(levelUp)));
        offset = 1.0f / (float)(((int)(2.0f * base - levelUp) / 2) & (int)(base / 2.0f - 1.0f));
    } else {
        if (level <= 1.0f) return t;
        const float base = exp2f(floorf(log2f(levelUp)));
        offset = 1.0f / (float)((((int)(2.0f * base - levelUp) / 2 + 1) & (int)(base / 2.0f - 1.0f)) + 1);
    }
    const float dx0 = (1.0f - (levelUp - level) / 2.0f) / levelUp;
    const float dx1 = (1.0f - 2.0f * dx0) / (levelUp - 2.0f * ceilf(dx0));
    if (t < 0.5f) {
        const float x = levelUp / 2.0f - roundf(t * levelUp);
        return 0.5f - (x * dx1 + (float)(x * offset > 1.0f) * (dx0 - dx1));
    } else if (t > 0.5f) {
        const float x = roundf(t * levelUp) - levelUp / 2.0f;
        return 0.5f + (x * dx1 + (float)(x * offset > 1.0f) * (dx0 - dx1));
    }
    return t;
}

// OsdGetTessTransitionSplit (glslPatchCommonTess.glsl:647-690)
__device__ float transition_split(float t, float lo, float hi, int spacing) {
    if (spacing == 1) {
        const float loUp = round_up_even(lo), hiUp = round_up_even(hi);
        const float ti = roundf(t * (loUp + hiUp));
        if (ti <= loUp) return fractional_split(ti / loUp, lo, loUp, 1) * 0.5f;
        return fractional_split((ti - loUp) / hiUp, hi, hiUp, 1) * 0.5f + 0.5f;
    }
    if (spacing == 2) {
        const float loUp = round_up_odd(lo), hiUp = round_up_odd(hi);
        const float ti = roundf(t * (loUp + hiUp + 1.0f));
        if (ti <= loUp) return fractional_split(ti / loUp, lo, loUp, 2) * 0.5f;
        if (ti > loUp + 1.0f)
            return fractional_split((ti - (loUp + 1.0f)) / hiUp, hi, hiUp, 2) * 0.5f + 0.5f;
        return 0.5f;
    }
    const float ti = roundf(t * (lo + hi));
    if (ti <= lo) return (ti / lo) * 0.5f;
    return ((ti - lo) / hi) * 0.5f + 0.5f;
}

struct ParamArgs {
    int n, spacing, triangular;
    const float *domain;  // 3 floats per point (u, v, w; w unused for quads)
    const int *patch;
    const float *lo, *hi;
    float *uv;
};

// OsdGetTessParameterization[Triangle] (glslPatchCommonTess.glsl:692-730)
__global__ void __launch_bounds__(256) k_tess_parameterize(const ParamArgs a) {
    const int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
        const float px = a.domain[3 * i], py = a.domain[3 * i + 1], pz = a.domain[3 * i + 2];
        const int p = a.patch[i];
        const float4 lo = reinterpret_cast<const float4 *>(a.lo)[p];
        const float4 hi = reinterpret_cast<const float4 *>(a.hi)[p];
        float u = px, v = py;
        if (!a.triangular) {
            if (px == 0.0f && hi.x > 0.0f) v = transition_split(v, lo.x, hi.x, a.spacing);
            else if (py == 0.0f && hi.y > 0.0f) u = transition_split(u, lo.y, hi.y, a.spacing);
            else if (px == 1.0f && hi.z > 0.0f) v = transition_split(v, lo.z, hi.z, a.spacing);
            else if (py == 1.0f && hi.w > 0.0f) u = transition_split(u, lo.w, hi.w, a.spacing);
        } else {
            if (px == 0.0f && hi.x > 0.0f) v = transition_split(v, lo.x, hi.x, a.spacing);
            else if (py == 0.0f && hi.y > 0.0f) u = transition_split(u, lo.y, hi.y, a.spacing);
            else if (pz == 0.0f && hi.z > 0.0f) {
                u = transition_split(u, lo.z, hi.z, a.spacing);
                v = 1.0f - u;
            }
        }
        a.uv[2 * i] = u;
        a.uv[2 * i + 1] = v;
    }
}

int grid_of(long long n, int threads, int perSm) {
    long long b = (n + threads - 1) / threads;
    const long long cap = (long long)num_sms() * perSm;
    return (int)(b < 1 ? 1 : b < cap ? b : cap);
}

bool aligned16(const void *p) { return ((uintptr_t)p & 15) == 0; }

}  // namespace

int tess_factors(const void *arrays, int numArrays, const int *indices, const void *params,
                 int numPatches, const float *src, int srcStride,
                 const GB300PatchTessOptions *o, float *outer, float *inner, float *outerLo,
                 float *outerHi, cudaStream_t s) {
    const char *who = "GB300PatchTableTessFactors";
    if (!o || !outer || !inner) return fail(GB300_ERR_INVALID_ARGUMENT, "%s: null argument", who);
    if (o->screenSpace && (!src || srcStride < 3))
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: screen-space factors need xyz points", who);
    if (o->spacing < 0 || o->spacing > 2)
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: spacing must be 0, 1 or 2", who);
    if (!aligned16(outer) || ((uintptr_t)inner & 7) || (outerLo && !aligned16(outerLo)) ||
        (outerHi && !aligned16(outerHi)))
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: outputs must be 16-byte (inner 8-byte) "
                                                "aligned", who);
    if (numPatches <= 0) return ok();
    TfArgs a;
    a.arrays = (const TfArray *)arrays;
    a.numArrays = numArrays;
    a.numPatches = numPatches;
    a.indices = indices;
    a.params = (const int *)params;
    a.src = src;
    a.srcStride = srcStride;
    a.o = *o;
    a.outer = outer;
    a.inner = inner;
    a.lo = outerLo;
    a.hi = outerHi;
    k_tess_factors<<<grid_of(numPatches, 128, 16), 128, 0, s>>>(a);
    count_launch();
    return check_launch(who);
}

}  // namespace gb300

using namespace gb300;

extern "C" int GB300PatchTessParameterization(int n, const float *domain, const int *patchIndex,
                                              const float *outerLo, const float *outerHi,
                                              int spacing, int triangular, float *uv,
                                              void *stream) {
    const char *who = "GB300PatchTessParameterization";
    if (n <= 0) return ok();
    if (!domain || !patchIndex || !outerLo || !outerHi || !uv)
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: null argument", who);
    if (spacing < 0 || spacing > 2 || !aligned16(outerLo) || !aligned16(outerHi))
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: bad spacing or unaligned levels", who);
    ParamArgs a{n, spacing, triangular != 0, domain, patchIndex, outerLo, outerHi, uv};
    k_tess_parameterize<<<grid_of(n, 256, 16), 256, 0, as_stream(stream)>>>(a);
    count_launch();
    return check_launch(who);
}
