// Per-stencil evaluation shared by the staged EvalStencils kernel (stencils_tma.cu) and the
// batched kernel (stencils_batch.cu).  `A` is the launch's argument view: it provides src,
// srcStride, length, indices, w[k], dst[k], dstStride[k], outOf[k] and vecDst[k].
#pragma once

#include "common.cuh"

namespace gb300 {
namespace tma {

// Elements [c0, c0 + 8) of source row `id` (zeros past the primvar length): one 256-bit load
// for 32-byte aligned rows, two 128-bit loads for 16-byte aligned rows, else scalar loads.
// VW = 0 picks the width at run time from a.vw (one code path for jobs of mixed layouts).
template <int VW, class A>
__device__ __forceinline__ void gather_row(const A &a, int id, int c0, uint64_t pol_src,
                                           float (&x)[8]) {
    const float *row = a.src + (size_t)id * a.srcStride + c0;
    if constexpr (VW == 0) {
        if (a.vw == 8)
            gather_row<8>(a, id, c0, pol_src, x);
        else if (a.vw == 4)
            gather_row<4>(a, id, c0, pol_src, x);
        else
            gather_row<1>(a, id, c0, pol_src, x);
    } else if constexpr (VW == 8) {
        asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
            : "=f"(x[0]), "=f"(x[1]), "=f"(x[2]), "=f"(x[3]), "=f"(x[4]), "=f"(x[5]),
              "=f"(x[6]), "=f"(x[7])
            : "l"(row));
    } else if constexpr (VW == 4) {
        const float4 *r4 = reinterpret_cast<const float4 *>(row);
        const float4 v0 = __ldg(r4);
        x[0] = v0.x; x[1] = v0.y; x[2] = v0.z; x[3] = v0.w;
        if (c0 + 4 < a.length) {
            const float4 v1 = __ldg(r4 + 1);
            x[4] = v1.x; x[5] = v1.y; x[6] = v1.z; x[7] = v1.w;
        } else {
            x[4] = x[5] = x[6] = x[7] = 0.0f;
        }
    } else {
#pragma unroll
        for (int c = 0; c < 8; ++c) x[c] = (c0 + c < a.length) ? ld_src(row + c, pol_src) : 0.0f;
    }
}

template <int NW>
__device__ __forceinline__ void fma_row(const float (&wk)[NW], const float (&x)[8],
                                        float (&acc)[NW][8]) {
#pragma unroll
    for (int k = 0; k < NW; ++k)
#pragma unroll
        for (int c = 0; c < 8; ++c) acc[k][c] = fmaf(wk[k], x[c], acc[k][c]);
}

// One stencil, all requested outputs, elements [c0, c0 + 8) of the primvar; entries come from
// shared memory (lidx/lw at local offset o) or straight from global memory (when lidx null).
template <int NW, int VW, class A>
__device__ __forceinline__ void eval_one(const A &a, int i, int n, const int *lidx,
                                         const float *lw, int lstride, int o, uint64_t pol_src,
                                         uint64_t pol_stream) {
    for (int c0 = 0; c0 < a.length; c0 += 8) {
        float acc[NW][8];
#pragma unroll
        for (int k = 0; k < NW; ++k)
#pragma unroll
            for (int c = 0; c < 8; ++c) acc[k][c] = 0.0f;
        if (lidx) {
            // entries from shared memory in aligned chunks of 4 (one 128-bit shared load per
            // array and chunk); entries of the chunk outside [o, o + n) are skipped, so the
            // row gathers stay exact while every thread runs the same simple loop
            const int end = o + n;
            for (int q = o & ~3; q < end; q += 4) {
                const int4 id4 = *reinterpret_cast<const int4 *>(lidx + q);
                float4 w4[NW];
#pragma unroll
                for (int k = 0; k < NW; ++k)
                    w4[k] = *reinterpret_cast<const float4 *>(lw + k * lstride + q);
                const int ids[4] = {id4.x, id4.y, id4.z, id4.w};
                // rows gathered G at a time before they are accumulated: all 4 for one output,
                // 2 when the NW accumulators need the registers
                constexpr int G = NW == 1 ? 4 : 2;
                static_assert(4 % G == 0, "rows are gathered in groups that tile the chunk");
#pragma unroll
                for (int g = 0; g < 4; g += G) {
                    float x[G][8];
#pragma unroll
                    for (int m = 0; m < G; ++m)
                        if (q + g + m >= o && q + g + m < end)
                            gather_row<VW>(a, ids[g + m], c0, pol_src, x[m]);
#pragma unroll
                    for (int m = 0; m < G; ++m) {
                        const int e = g + m;
                        if (q + e < o || q + e >= end) continue;
                        float wk[NW];
#pragma unroll
                        for (int k = 0; k < NW; ++k)
                            wk[k] = e == 0 ? w4[k].x : e == 1 ? w4[k].y : e == 2 ? w4[k].z
                                                                         : w4[k].w;
                        fma_row<NW>(wk, x[m], acc);
                    }
                }
            }
        } else {
            for (int j = 0; j < n; ++j) {
                float wk[NW];
#pragma unroll
                for (int k = 0; k < NW; ++k) wk[k] = ld_stream(a.w[k] + o + j, pol_stream);
                float x[8];
                gather_row<VW>(a, ld_stream(a.indices + o + j, pol_stream), c0, pol_src, x);
                fma_row<NW>(wk, x, acc);
            }
        }
#pragma unroll
        for (int k = 0; k < NW; ++k) {
            float *d = a.dst[a.outOf[k]] + (size_t)i * a.dstStride[a.outOf[k]] + c0;
            const int rem = a.length - c0;
            if (a.vecDst[a.outOf[k]] == 8 && rem >= 8) {
                asm volatile("st.global.cs.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(d),
                             "f"(acc[k][0]), "f"(acc[k][1]), "f"(acc[k][2]), "f"(acc[k][3]),
                             "f"(acc[k][4]), "f"(acc[k][5]), "f"(acc[k][6]), "f"(acc[k][7])
                             : "memory");
            } else if (a.vecDst[a.outOf[k]] && rem >= 8) {
                asm volatile("st.global.cs.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(d),
                             "f"(acc[k][0]), "f"(acc[k][1]), "f"(acc[k][2]), "f"(acc[k][3])
                             : "memory");
                asm volatile("st.global.cs.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(d + 4),
                             "f"(acc[k][4]), "f"(acc[k][5]), "f"(acc[k][6]), "f"(acc[k][7])
                             : "memory");
            } else {
#pragma unroll
                for (int c = 0; c < 8; ++c)
                    if (c < rem) st_stream(d + c, acc[k][c]);
            }
        }
    }
}

// One stencil, one output, of a primvar 9-12 floats wide whose rows are 16-byte aligned with a
// stride of at least 12 floats: all elements in ONE pass over the shared-memory entries
// (12 accumulators, three 128-bit gathers per entry) instead of two 8-element passes, each
// element accumulated in entry order with the same fused multiply-adds (same results).
template <class A>
__device__ __forceinline__ void eval_one12(const A &a, int i, int n, const int *lidx,
                                           const float *lw, int o) {
    float acc[12];
#pragma unroll
    for (int c = 0; c < 12; ++c) acc[c] = 0.0f;
    const int end = o + n;
    for (int q = o & ~3; q < end; q += 4) {
        const int4 id4 = *reinterpret_cast<const int4 *>(lidx + q);
        const float4 w4 = *reinterpret_cast<const float4 *>(lw + q);
        const int ids[4] = {id4.x, id4.y, id4.z, id4.w};
        const float ws[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
        for (int g = 0; g < 4; g += 2) {
            float4 x[2][3];
#pragma unroll
            for (int m = 0; m < 2; ++m)
                if (q + g + m >= o && q + g + m < end) {
                    const float4 *r = reinterpret_cast<const float4 *>(
                        a.src + (size_t)ids[g + m] * a.srcStride);
                    x[m][0] = __ldg(r);
                    x[m][1] = __ldg(r + 1);
                    x[m][2] = __ldg(r + 2);
                }
#pragma unroll
            for (int m = 0; m < 2; ++m) {
                if (q + g + m < o || q + g + m >= end) continue;
                const float wk = ws[g + m];
#pragma unroll
                for (int v = 0; v < 3; ++v) {
                    acc[4 * v + 0] = fmaf(wk, x[m][v].x, acc[4 * v + 0]);
                    acc[4 * v + 1] = fmaf(wk, x[m][v].y, acc[4 * v + 1]);
                    acc[4 * v + 2] = fmaf(wk, x[m][v].z, acc[4 * v + 2]);
                    acc[4 * v + 3] = fmaf(wk, x[m][v].w, acc[4 * v + 3]);
                }
            }
        }
    }
    const int k = a.outOf[0];
    float *d = a.dst[k] + (size_t)i * a.dstStride[k];
    if (a.vecDst[k]) {
#pragma unroll
        for (int v = 0; v < 3; ++v) {
            if (4 * v + 4 <= a.length) {
                asm volatile("st.global.cs.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(d + 4 * v),
                             "f"(acc[4 * v]), "f"(acc[4 * v + 1]), "f"(acc[4 * v + 2]),
                             "f"(acc[4 * v + 3])
                             : "memory");
            } else {
#pragma unroll
                for (int c = 4 * v; c < 4 * v + 4; ++c)
                    if (c < a.length) st_stream(d + c, acc[c]);
            }
        }
    } else {
#pragma unroll
        for (int c = 0; c < 12; ++c)
            if (c < a.length) st_stream(d + c, acc[c]);
    }
}

}  // namespace tma
}  // namespace gb300
