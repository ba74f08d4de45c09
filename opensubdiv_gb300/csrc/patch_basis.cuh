// Limit-surface patch evaluation on the device, one point per thread, fused with the
// control-point gather.
//
// The bases are those of osd/patchBasis.h (OsdEvaluatePatchBasis, :1558-1610), evaluated in
// forms that keep everything in registers instead of the reference's six float[20] weight
// arrays (osd/cudaKernel.cu:270-326):
//   - REGULAR (bicubic B-spline, :206-245) and GREGORY_BASIS (:334-490) are tensor products,
//     evaluated separably: per row r, the s-weights (value, d/ds, d2/ds2) are applied to the
//     row's 4 points, then the t-weights combine rows.  Boundary phantom points
//     (:138-171) fold into the 1-D weights.  Gregory interior points are first blended by
//     their rational weights G into the 4 interior Bezier points (the approximate-derivative
//     form the reference uses by default, :421-440).
//   - GREGORY_TRIANGLE (:1115-1175) blends its 3 pairs of interior points into a 15-point
//     quartic Bezier triangle and applies the Bezier-triangle weights (:924-1044).
//   - LOOP (box spline, :892-917) evaluates the 12 quartic polynomials and folds phantom
//     boundary points (:666-850) in weight space.
//   - QUADS / TRIANGLES are the linear bases (:56-97, :496-525).
// Derivative scaling by +-2^depth and +-4^depth (:1587-1606) is applied to the sums (exact:
// powers of two).  Rows are gathered relative to a corner control point of the patch (see
// load_row below), which keeps the second-derivative sums accurate to well inside
// 1e-5 x the cage's size where the reference's absolute-coordinate sums are not.
#pragma once

#include <cuda_runtime.h>

namespace gb300 {

struct Param {
    int f0, f1;
    __device__ int u() const { return (f1 >> 22) & 0x3ff; }
    __device__ int v() const { return (f1 >> 12) & 0x3ff; }
    __device__ int boundary() const { return (f1 >> 7) & 0x1f; }
    __device__ int nonquad() const { return (f1 >> 4) & 1; }
    __device__ int depth() const { return f1 & 0xf; }
    __device__ bool regular() const { return ((f1 >> 5) & 1) != 0; }
};

// Accumulator for one point: 6 outputs (P, Ds, Dt, Dss, Dst, Dtt) x LC primvar elements.
template <int LC>
struct Acc6 {
    float v[6][LC];
    __device__ void zero() {
#pragma unroll
        for (int k = 0; k < 6; ++k)
#pragma unroll
            for (int c = 0; c < LC; ++c) v[k][c] = 0.0f;
    }
};

// Source points, patch index rows and params are gathered at random and re-read by every
// query that lands on the same patch: they are loaded with an evict-last L2 policy, so the
// streams read or written once (query coords, outputs) do not push them out of L2.

// Loads LC elements [e0, e0+LC) of control point `cv` (elements >= length read as 0).
template <int LC>
__device__ __forceinline__ void load_row(const float *__restrict__ src, int stride, int cv,
                                         int e0, int length, float (&x)[LC]) {
    const float *p = src + (size_t)cv * stride + e0;
    const uint64_t pol = l2_evict_last();
#pragma unroll
    for (int c = 0; c < LC; ++c) x[c] = (e0 + c < length) ? ld_src(p + c, pol) : 0.0f;
}

// Local origin.  Every basis is a partition of unity: its value weights sum to 1 and every
// derivative's weights sum to 0.  So  sum_j w_j x_j = xc + sum_j w_j (x_j - xc)  for the value
// and  sum_j w_j (x_j - xc)  for a derivative, for any point xc.  The bases below gather rows
// relative to one of the patch's own control points (a corner of the patch): the summands
// then scale with the patch's extent instead of the points' distance from the origin, and
// the float rounding of the cancelling derivative sums (which carry the 2^depth and 4^depth
// factors) shrinks by that ratio.  The value output adds xc back at the end.
template <int LC>
__device__ __forceinline__ void load_row(const float *__restrict__ src, int stride, int cv,
                                         int e0, int length, float (&x)[LC],
                                         const float (&xc)[LC]) {
    const float *p = src + (size_t)cv * stride + e0;
    const uint64_t pol = l2_evict_last();
#pragma unroll
    for (int c = 0; c < LC; ++c) x[c] = (e0 + c < length) ? ld_src(p + c, pol) - xc[c] : 0.0f;
}

template <int LC>
__device__ __forceinline__ void add_origin(const float (&xc)[LC], Acc6<LC> &acc) {
#pragma unroll
    for (int c = 0; c < LC; ++c) acc.v[0][c] += xc[c];
}

// N control-point indices of a patch: 128-bit loads when the index row is 16-byte aligned
// (REGULAR rows are 64 B, GREGORY_BASIS rows 80 B), scalar loads otherwise.
template <int N>
__device__ __forceinline__ void load_indices(const int *__restrict__ cvs, int (&idx)[N]) {
    const uint64_t pol = l2_evict_last();
    if ((N % 4) == 0 && (reinterpret_cast<uintptr_t>(cvs) & 15) == 0) {
#pragma unroll
        for (int j = 0; j < N / 4; ++j) {
            const int4 v = ld_keep4(cvs + 4 * j, pol);
            idx[4 * j] = v.x; idx[4 * j + 1] = v.y; idx[4 * j + 2] = v.z; idx[4 * j + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int j = 0; j < N; ++j) idx[j] = ld_keep(cvs + j, pol);
    }
}

__device__ __forceinline__ void bspline_curve(float t, float *p, float *d, float *dd) {
    const float sixth = 1.0f / 6.0f;
    float t2 = t * t, t3 = t * t2;
    p[0] = sixth * (1.0f - 3.0f * (t - t2) - t3);
    p[1] = sixth * (4.0f - 6.0f * t2 + 3.0f * t3);
    p[2] = sixth * (1.0f + 3.0f * (t + t2 - t3));
    p[3] = sixth * t3;
    d[0] = -0.5f * t2 + t - 0.5f;
    d[1] = 1.5f * t2 - 2.0f * t;
    d[2] = -1.5f * t2 + t + 0.5f;
    d[3] = 0.5f * t2;
    dd[0] = 1.0f - t;
    dd[1] = 3.0f * t - 2.0f;
    dd[2] = 1.0f - 3.0f * t;
    dd[3] = t;
}

__device__ __forceinline__ void bezier_curve(float t, float *p, float *d, float *dd) {
    float t2 = t * t, tc = 1.0f - t, tc2 = tc * tc;
    p[0] = tc2 * tc;
    p[1] = tc2 * t * 3.0f;
    p[2] = t2 * tc * 3.0f;
    p[3] = t2 * t;
    d[0] = -3.0f * tc2;
    d[1] = 9.0f * t2 - 12.0f * t + 3.0f;
    d[2] = -9.0f * t2 + 6.0f * t;
    d[3] = 3.0f * t2;
    dd[0] = 6.0f * tc;
    dd[1] = 18.0f * t - 12.0f;
    dd[2] = -18.0f * t + 6.0f;
    dd[3] = 6.0f * t;
}

// Phantom end point of a cubic B-spline curve: w[lo] folds into its neighbours
// (w[lo+1] += 2 w[lo], w[lo+2] -= w[lo]); `dir` = +1 folds the first point, -1 the last.
__device__ __forceinline__ void fold_first(float *w) { w[2] -= w[0]; w[1] += 2.0f * w[0]; w[0] = 0.0f; }
__device__ __forceinline__ void fold_last(float *w) { w[1] -= w[3]; w[2] += 2.0f * w[3]; w[3] = 0.0f; }

// Separable tensor-product evaluation over a 4x4 grid of points: sw = s weights (value,
// d, dd), tw = t weights; rows[r][c] = point at row r, column c.
template <int LC>
__device__ __forceinline__ void tensor_accumulate(const float (&sp)[4], const float (&sd)[4],
                                                  const float (&sdd)[4], float tp, float td,
                                                  float tdd, const float (&x)[4][LC],
                                                  Acc6<LC> &acc) {
#pragma unroll
    for (int c = 0; c < LC; ++c) {
        float ip = 0.0f, id = 0.0f, idd = 0.0f;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            ip = fmaf(sp[j], x[j][c], ip);
            id = fmaf(sd[j], x[j][c], id);
            idd = fmaf(sdd[j], x[j][c], idd);
        }
        acc.v[0][c] = fmaf(tp, ip, acc.v[0][c]);
        acc.v[1][c] = fmaf(tp, id, acc.v[1][c]);
        acc.v[2][c] = fmaf(td, ip, acc.v[2][c]);
        acc.v[3][c] = fmaf(tp, idd, acc.v[3][c]);
        acc.v[4][c] = fmaf(td, id, acc.v[4][c]);
        acc.v[5][c] = fmaf(tdd, ip, acc.v[5][c]);
    }
}

// REGULAR: 16 points in row-major (t rows, s columns) order.
template <int LC>
__device__ void eval_bspline(float s, float t, int boundary, const int *__restrict__ cvs,
                             const float *__restrict__ src, int stride, int e0, int length,
                             Acc6<LC> &acc) {
    float sp[4], sd[4], sdd[4], tp[4], td[4], tdd[4];
    bspline_curve(s, sp, sd, sdd);
    bspline_curve(t, tp, td, tdd);
    // boundary bits: 1 = first t row, 2 = last s column, 4 = last t row, 8 = first s column
    if (boundary & 1) { fold_first(tp); fold_first(td); fold_first(tdd); }
    if (boundary & 2) { fold_last(sp); fold_last(sd); fold_last(sdd); }
    if (boundary & 4) { fold_last(tp); fold_last(td); fold_last(tdd); }
    if (boundary & 8) { fold_first(sp); fold_first(sd); fold_first(sdd); }
    int idx[16];
    load_indices<16>(cvs, idx);
    float xc[LC];  // point 5: the patch's (0,0) corner, never a phantom
    load_row<LC>(src, stride, idx[5], e0, length, xc);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        float x[4][LC];
#pragma unroll
        for (int c = 0; c < 4; ++c)
            load_row<LC>(src, stride, idx[4 * r + c], e0, length, x[c], xc);
        tensor_accumulate<LC>(sp, sd, sdd, tp[r], td[r], tdd[r], x, acc);
    }
    add_origin<LC>(xc, acc);
}

// GREGORY_BASIS: 20 points; the Bezier grid is
//   row 0: 0 1 7 5 | row 1: 2 (3,4) (8,9) 6 | row 2: 16 (18,19) (13,14) 12 | row 3: 15 17 11 10
// where (a,b) is the pair of interior face points blended by G (patchBasis.h:346-378).
template <int LC>
__device__ void eval_gregory(float s, float t, const int *__restrict__ cvs,
                             const float *__restrict__ src, int stride, int e0, int length,
                             Acc6<LC> &acc) {
    float bs[4], bds[4], bdss[4], bt[4], bdt[4], bdtt[4];
    bezier_curve(s, bs, bds, bdss);
    bezier_curve(t, bt, bdt, bdtt);
    const float sc = 1.0f - s, tc = 1.0f - t;
    float d0 = s + t;   d0 = (d0 <= 0.0f) ? 1.0f : (1.0f / d0);
    float d1 = sc + t;  d1 = (d1 <= 0.0f) ? 1.0f : (1.0f / d1);
    float d2 = sc + tc; d2 = (d2 <= 0.0f) ? 1.0f : (1.0f / d2);
    float d3 = s + tc;  d3 = (d3 <= 0.0f) ? 1.0f : (1.0f / d3);
    const float g0 = s * d0, g2 = t * d1, g4 = sc * d2, g6 = tc * d3;
    int idx[20];
    load_indices<20>(cvs, idx);
    float xc[LC];  // point 0: the patch's (0,0) corner
    load_row<LC>(src, stride, idx[0], e0, length, xc);
    // rows of the Bezier grid; interior entries are blended pairs
    constexpr int kGrid[4][4] = {{0, 1, 7, 5}, {2, -1, -2, 6}, {16, -4, -3, 12}, {15, 17, 11, 10}};
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        float x[4][LC];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int g = kGrid[r][c];
            if (g >= 0) {
                load_row<LC>(src, stride, idx[g], e0, length, x[c], xc);
            } else {
                // -1: (3,4) by g0; -2: (8,9) by g2; -3: (13,14) by g4; -4: (18,19) by g6
                const int a = (g == -1) ? 3 : (g == -2) ? 8 : (g == -3) ? 13 : 18;
                const float ga = (g == -1) ? g0 : (g == -2) ? g2 : (g == -3) ? g4 : g6;
                float xa[LC], xb[LC];
                load_row<LC>(src, stride, idx[a], e0, length, xa, xc);
                load_row<LC>(src, stride, idx[a + 1], e0, length, xb, xc);
#pragma unroll
                for (int k = 0; k < LC; ++k) x[c][k] = ga * xa[k] + (1.0f - ga) * xb[k];
            }
        }
        tensor_accumulate<LC>(bs, bds, bdss, bt[r], bdt[r], bdtt[r], x, acc);
    }
    add_origin<LC>(xc, acc);
}

// Quartic Bezier triangle weights for derivative order (ds, dt) (patchBasis.h:924-1044).
__device__ __forceinline__ void bezier_tri_weights(float u, float v, int ds, int dt, float *b) {
    const float w = 1.0f - u - v;
    const float uu = u * u, vv = v * v, ww = w * w, uv = u * v, vw = v * w, uw = u * w;
    const int order = ds + dt;
    if (order == 0) {
        b[0] = ww * ww;        b[1] = 4 * uw * ww;   b[2] = 6 * uw * uw;   b[3] = 4 * uw * uu;
        b[4] = uu * uu;        b[5] = 4 * vw * ww;   b[6] = 12 * ww * uv;  b[7] = 12 * uu * vw;
        b[8] = 4 * uv * uu;    b[9] = 6 * vw * vw;   b[10] = 12 * vv * uw; b[11] = 6 * uv * uv;
        b[12] = 4 * vw * vv;   b[13] = 4 * uv * vv;  b[14] = vv * vv;
    } else if (order == 1 && ds == 1) {
        b[0] = -4 * ww * w;            b[1] = 4 * ww * (w - 3 * u);   b[2] = 12 * uw * (w - u);
        b[3] = 4 * uu * (3 * w - u);   b[4] = 4 * uu * u;             b[5] = -12 * vw * w;
        b[6] = 12 * vw * (w - 2 * u);  b[7] = 12 * uv * (2 * w - u);  b[8] = 12 * uv * u;
        b[9] = -12 * vv * w;           b[10] = 12 * vv * (w - u);     b[11] = 12 * vv * u;
        b[12] = -4 * vv * v;           b[13] = 4 * vv * v;            b[14] = 0;
    } else if (order == 1) {
        b[0] = -4 * ww * w;            b[1] = -12 * ww * u;           b[2] = -12 * uu * w;
        b[3] = -4 * uu * u;            b[4] = 0;                      b[5] = 4 * ww * (w - 3 * v);
        b[6] = 12 * uw * (w - 2 * v);  b[7] = 12 * uu * (w - v);      b[8] = 4 * uu * u;
        b[9] = 12 * vw * (w - v);      b[10] = 12 * uv * (2 * w - v); b[11] = 12 * uv * u;
        b[12] = 4 * vv * (3 * w - v);  b[13] = 12 * vv * u;           b[14] = 4 * vv * v;
    } else if (ds == 2) {
        b[0] = 12 * ww;                b[1] = 24 * (uw - ww);         b[2] = 12 * (uu - 4 * uw + ww);
        b[3] = 24 * (uw - uu);         b[4] = 12 * uu;                b[5] = 24 * vw;
        b[6] = 24 * (uv - 2 * vw);     b[7] = 24 * (vw - 2 * uv);     b[8] = 24 * uv;
        b[9] = 12 * vv;                b[10] = -24 * vv;              b[11] = 12 * vv;
        b[12] = 0; b[13] = 0; b[14] = 0;
    } else if (dt == 2) {
        b[0] = 12 * ww;                b[1] = 24 * uw;                b[2] = 12 * uu;
        b[3] = 0;                      b[4] = 0;                      b[5] = 24 * (vw - ww);
        b[6] = 24 * (uv - 2 * uw);     b[7] = -24 * uu;               b[8] = 0;
        b[9] = 12 * (vv - 4 * vw + ww); b[10] = 24 * (uw - 2 * uv);   b[11] = 12 * uu;
        b[12] = 24 * (vw - vv);        b[13] = 24 * uv;               b[14] = 12 * vv;
    } else {
        b[0] = 12 * ww;
        b[3] = -12 * uu;
        b[13] = 12 * vv;
        b[11] = 24 * uv;
        b[1] = 24 * uw - b[0];
        b[2] = -24 * uw - b[3];
        b[5] = 24 * vw - b[0];
        b[6] = -24 * vw + b[11] - b[1];
        b[8] = -b[3];
        b[7] = -(b[11] + b[2]);
        b[9] = b[13] - b[5] - b[0];
        b[10] = -(b[9] + b[11]);
        b[12] = -b[13];
        b[4] = 0;
        b[14] = 0;
    }
}

// GREGORY_TRIANGLE: 18 points mapped onto the 15 quartic Bezier points; interior Bezier
// points 6, 7 and 10 are blends of Gregory pairs (3,4), (8,9), (13,14) (patchBasis.h:1078-1106).
template <int LC>
__device__ void eval_gregory_tri(float s, float t, const int *__restrict__ cvs,
                                 const float *__restrict__ src, int stride, int e0, int length,
                                 Acc6<LC> &acc) {
    float g[6] = {1.0f, 0.0f, 1.0f, 0.0f, 1.0f, 0.0f};
    const float u = s, v = t, w = 1.0f - u - v;
    if ((u + v) > 0) { g[0] = u / (u + v); g[1] = v / (u + v); }
    if ((v + w) > 0) { g[2] = v / (v + w); g[3] = w / (v + w); }
    if ((w + u) > 0) { g[4] = w / (w + u); g[5] = u / (w + u); }
    // Bezier point m comes from Gregory point kBez[m] (or a blended pair for 6, 7, 10)
    constexpr int kBez[15] = {0, 1, 15, 7, 5, 2, -1, -2, 6, 17, -3, 16, 11, 12, 10};
    float xc[LC];  // point 0: the (0,0) corner
    load_row<LC>(src, stride, __ldg(cvs), e0, length, xc);
    float B[15][LC];
#pragma unroll
    for (int m = 0; m < 15; ++m) {
        const int gi = kBez[m];
        if (gi >= 0) {
            load_row<LC>(src, stride, __ldg(cvs + gi), e0, length, B[m], xc);
        } else {
            const int a = (gi == -1) ? 3 : (gi == -2) ? 8 : 13;
            const float ga = (gi == -1) ? g[0] : (gi == -2) ? g[2] : g[4];
            const float gb = (gi == -1) ? g[1] : (gi == -2) ? g[3] : g[5];
            float xa[LC], xb[LC];
            load_row<LC>(src, stride, __ldg(cvs + a), e0, length, xa, xc);
            load_row<LC>(src, stride, __ldg(cvs + a + 1), e0, length, xb, xc);
#pragma unroll
            for (int c = 0; c < LC; ++c) B[m][c] = ga * xa[c] + gb * xb[c];
        }
    }
    constexpr int kOrd[6][2] = {{0, 0}, {1, 0}, {0, 1}, {2, 0}, {1, 1}, {0, 2}};
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        float b[15];
        bezier_tri_weights(s, t, kOrd[k][0], kOrd[k][1], b);
#pragma unroll
        for (int m = 0; m < 15; ++m)
#pragma unroll
            for (int c = 0; c < LC; ++c) acc.v[k][c] = fmaf(b[m], B[m][c], acc.v[k][c]);
    }
    add_origin<LC>(xc, acc);
}

// Box-spline coefficient rows over the quartic monomials {1, s, t, s2, st, t2, s3, s2t, st2,
// t3, s4, s3t, s2t2, st3, t4} (patchBasis.h:557-669): value (x 1/12), d/ds and d/dt (x 1/6)
// over the first 10, second derivatives over the first 6 (d2/dsdt x 1/2).
__device__ __forceinline__ float box_row(const signed char *c, int n, const float *m) {
    float acc = 0.0f;
#pragma unroll
    for (int k = 0; k < n; ++k)
        if (c[k] != 0) acc = fmaf((float)c[k], m[k], acc);
    return acc;
}

__device__ __forceinline__ void box_fold(int mask, float *w) {
    if (mask == 0) return;
    const int upper = (mask >> 3) & 3, lower = mask & 7;
    int eb = lower, vb = 0;
    if (upper == 1) { vb = eb; eb = 0; }
    else if (upper == 2) { vb = ((eb & 1) << 2) | (eb >> 1); }
    const bool e0 = eb & 1, e1 = eb & 2, e2 = eb & 4;
    float a, b, c;
    if (e0) {
        a = w[0];
        if (e2) { w[4] += 2.0f * a; w[8] -= a; } else { w[4] += a; w[3] += a; w[7] -= a; }
        b = w[1]; w[4] += b; w[5] += b; w[8] -= b;
        c = w[2];
        if (e1) { w[5] += 2.0f * c; w[8] -= c; } else { w[5] += c; w[6] += c; w[9] -= c; }
        w[0] = w[1] = w[2] = 0.0f;
    }
    if (e1) {
        a = w[6];
        if (e0) { w[5] += 2.0f * a; w[4] -= a; } else { w[5] += a; w[2] += a; w[1] -= a; }
        b = w[9]; w[5] += b; w[8] += b; w[4] -= b;
        c = w[11];
        if (e2) { w[8] += 2.0f * c; w[4] -= c; } else { w[8] += c; w[10] += c; w[7] -= c; }
        w[6] = w[9] = w[11] = 0.0f;
    }
    if (e2) {
        a = w[10];
        if (e1) { w[8] += 2.0f * a; w[5] -= a; } else { w[8] += a; w[11] += a; w[9] -= a; }
        b = w[7]; w[8] += b; w[4] += b; w[5] -= b;
        c = w[3];
        if (e0) { w[4] += 2.0f * c; w[5] -= c; } else { w[4] += c; w[0] += c; w[1] -= c; }
        w[10] = w[7] = w[3] = 0.0f;
    }
    if (vb & 1) { a = w[3]; w[4] += a; w[7] += a; w[8] -= a; b = w[0]; w[4] += b; w[1] += b; w[5] -= b; w[3] = w[0] = 0.0f; }
    if (vb & 2) { a = w[2]; w[5] += a; w[1] += a; w[4] -= a; b = w[6]; w[5] += b; w[9] += b; w[8] -= b; w[2] = w[6] = 0.0f; }
    if (vb & 4) { a = w[11]; w[8] += a; w[9] += a; w[5] -= a; b = w[10]; w[8] += b; w[7] += b; w[4] -= b; w[11] = w[10] = 0.0f; }
}

// Box-spline weights of the 12 control points for derivative order k (0 value, 1 d/ds, 2 d/dt,
// 3 d2/ds2, 4 d2/dsdt, 5 d2/dt2) from the monomials m, before boundary folds.
__device__ __forceinline__ void box_weights(int k, const float *m, float (&w)[12]) {
    constexpr signed char kP[12][15] = {
        {1, -2, -4, 0, 6, 6, 2, 0, -6, -4, -1, -2, 0, 2, 1},
        {1, 2, -2, 0, -6, 0, -4, 0, 6, 2, 2, 4, 0, -2, -1},
        {0, 0, 0, 0, 0, 0, 2, 0, 0, 0, -1, -2, 0, 0, 0},
        {1, -4, -2, 6, 6, 0, -4, -6, 0, 2, 1, 2, 0, -2, -1},
        {6, 0, 0, -12, -12, -12, 8, 12, 12, 8, -1, -2, 0, -2, -1},
        {1, 4, 2, 6, 6, 0, -4, -6, -12, -4, -1, -2, 0, 4, 2},
        {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 2, 0, 0, 0},
        {1, -2, 2, 0, -6, 0, 2, 6, 0, -4, -1, -2, 0, 4, 2},
        {1, 2, 4, 0, 6, 6, -4, -12, -6, -4, 2, 4, 0, -2, -1},
        {0, 0, 0, 0, 0, 0, 2, 6, 6, 2, -1, -2, 0, -2, -1},
        {0, 0, 0, 0, 0, 0, 0, 0, 0, 2, 0, 0, 0, -2, -1},
        {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 2, 1}};
    constexpr signed char kDs[12][10] = {
        {-1, 0, 3, 3, 0, -3, -2, -3, 0, 1}, {1, 0, -3, -6, 0, 3, 4, 6, 0, -1},
        {0, 0, 0, 3, 0, 0, -2, -3, 0, 0},   {-2, 6, 3, -6, -6, 0, 2, 3, 0, -1},
        {0, -12, -6, 12, 12, 6, -2, -3, 0, -1}, {2, 6, 3, -6, -6, -6, -2, -3, 0, 2},
        {0, 0, 0, 0, 0, 0, 2, 3, 0, 0},     {-1, 0, -3, 3, 6, 0, -2, -3, 0, 2},
        {1, 0, 3, -6, -12, -3, 4, 6, 0, -1}, {0, 0, 0, 3, 6, 3, -2, -3, 0, -1},
        {0, 0, 0, 0, 0, 0, 0, 0, 0, -1},    {0, 0, 0, 0, 0, 0, 0, 0, 0, 1}};
    constexpr signed char kDt[12][10] = {
        {-2, 3, 6, 0, -6, -6, -1, 0, 3, 2},  {-1, -3, 0, 0, 6, 3, 2, 0, -3, -2},
        {0, 0, 0, 0, 0, 0, -1, 0, 0, 0},     {-1, 3, 0, -3, 0, 3, 1, 0, -3, -2},
        {0, -6, -12, 6, 12, 12, -1, 0, -3, -2}, {1, 3, 0, -3, -12, -6, -1, 0, 6, 4},
        {0, 0, 0, 0, 0, 0, 1, 0, 0, 0},      {1, -3, 0, 3, 0, -6, -1, 0, 6, 4},
        {2, 3, 6, -6, -6, -6, 2, 0, -3, -2}, {0, 0, 0, 3, 6, 3, -1, 0, -3, -2},
        {0, 0, 0, 0, 0, 3, 0, 0, -3, -2},    {0, 0, 0, 0, 0, 0, 0, 0, 3, 2}};
    constexpr signed char kDss[12][6] = {
        {0, 1, 0, -1, -1, 0}, {0, -2, 0, 2, 2, 0}, {0, 1, 0, -1, -1, 0}, {1, -2, -1, 1, 1, 0},
        {-2, 4, 2, -1, -1, 0}, {1, -2, -1, -1, -1, 0}, {0, 0, 0, 1, 1, 0}, {0, 1, 1, -1, -1, 0},
        {0, -2, -2, 2, 2, 0}, {0, 1, 1, -1, -1, 0}, {0, 0, 0, 0, 0, 0}, {0, 0, 0, 0, 0, 0}};
    constexpr signed char kDtt[12][6] = {
        {1, -1, -2, 0, 1, 1}, {0, 1, 1, 0, -1, -1}, {0, 0, 0, 0, 0, 0}, {0, 0, 1, 0, -1, -1},
        {-2, 2, 4, 0, -1, -1}, {0, -2, -2, 0, 2, 2}, {0, 0, 0, 0, 0, 0}, {0, 0, -2, 0, 2, 2},
        {1, -1, -2, 0, -1, -1}, {0, 1, 1, 0, -1, -1}, {0, 0, 1, 0, -1, -1}, {0, 0, 0, 0, 1, 1}};
    constexpr signed char kDst[12][6] = {
        {1, 0, -2, -1, 0, 1}, {-1, 0, 2, 2, 0, -1}, {0, 0, 0, -1, 0, 0}, {1, -2, 0, 1, 0, -1},
        {-2, 4, 4, -1, 0, -1}, {1, -2, -4, -1, 0, 2}, {0, 0, 0, 1, 0, 0}, {-1, 2, 0, -1, 0, 2},
        {1, -4, -2, 2, 0, -1}, {0, 2, 2, -1, 0, -1}, {0, 0, 0, 0, 0, -1}, {0, 0, 0, 0, 0, 1}};
    const float k12 = 1.0f / 12.0f, k6 = 1.0f / 6.0f;
#pragma unroll
    for (int j = 0; j < 12; ++j) {
        w[j] = (k == 0) ? k12 * box_row(kP[j], 15, m)
             : (k == 1) ? k6 * box_row(kDs[j], 10, m)
             : (k == 2) ? k6 * box_row(kDt[j], 10, m)
             : (k == 3) ? box_row(kDss[j], 6, m)
             : (k == 4) ? 0.5f * box_row(kDst[j], 6, m)
             : box_row(kDtt[j], 6, m);
    }
}

template <int LC>
__device__ void eval_box_tri(float s, float t, int boundary, const int *__restrict__ cvs,
                             const float *__restrict__ src, int stride, int e0, int length,
                             Acc6<LC> &acc) {
    float m[15];
    m[0] = 1.0f; m[1] = s; m[2] = t;
    m[3] = s * s; m[4] = s * t; m[5] = t * t;
    m[6] = m[3] * s; m[7] = m[4] * s; m[8] = m[4] * t; m[9] = m[5] * t;
    m[10] = m[6] * s; m[11] = m[7] * s; m[12] = m[3] * m[5]; m[13] = m[8] * t; m[14] = m[9] * t;
    // the 12 control points once (every index of a Loop patch is valid, phantom boundary
    // points included, as the reference's own gather of all 12 relies on), then one
    // derivative order at a time: 12 weights live instead of 72, no reloads
    float x[12][LC], xc[LC];
    {
        int idx[12];
        load_indices<12>(cvs, idx);
        load_row<LC>(src, stride, idx[4], e0, length, xc);  // point 4: the (0,0) corner
#pragma unroll
        for (int j = 0; j < 12; ++j) load_row<LC>(src, stride, idx[j], e0, length, x[j], xc);
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        float w[12];
        box_weights(k, m, w);
        box_fold(boundary, w);
#pragma unroll
        for (int j = 0; j < 12; ++j) {
            if (w[j] == 0.0f) continue;
#pragma unroll
            for (int c = 0; c < LC; ++c) acc.v[k][c] = fmaf(w[j], x[j][c], acc.v[k][c]);
        }
    }
    add_origin<LC>(xc, acc);
}

template <int LC>
__device__ void eval_linear_quad(float s, float t, const int *__restrict__ cvs,
                                 const float *__restrict__ src, int stride, int e0, int length,
                                 Acc6<LC> &acc) {
    const float sc = 1.0f - s, tc = 1.0f - t;
    const float wp[4] = {sc * tc, s * tc, s * t, sc * t};
    const float ws[4] = {-tc, tc, t, -t};
    const float wt[4] = {-sc, -s, s, sc};
    const float wst[4] = {1.0f, -1.0f, 1.0f, -1.0f};
    float xc[LC];
    load_row<LC>(src, stride, __ldg(cvs), e0, length, xc);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        float x[LC];
        load_row<LC>(src, stride, __ldg(cvs + j), e0, length, x, xc);
#pragma unroll
        for (int c = 0; c < LC; ++c) {
            acc.v[0][c] = fmaf(wp[j], x[c], acc.v[0][c]);
            acc.v[1][c] = fmaf(ws[j], x[c], acc.v[1][c]);
            acc.v[2][c] = fmaf(wt[j], x[c], acc.v[2][c]);
            acc.v[4][c] = fmaf(wst[j], x[c], acc.v[4][c]);
        }
    }
    add_origin<LC>(xc, acc);
}

template <int LC>
__device__ void eval_linear_tri(float s, float t, const int *__restrict__ cvs,
                                const float *__restrict__ src, int stride, int e0, int length,
                                Acc6<LC> &acc) {
    float x0[LC], x1[LC], x2[LC];
    load_row<LC>(src, stride, __ldg(cvs + 0), e0, length, x0);
    load_row<LC>(src, stride, __ldg(cvs + 1), e0, length, x1, x0);
    load_row<LC>(src, stride, __ldg(cvs + 2), e0, length, x2, x0);
    // relative to point 0: P = x0 + s (x1 - x0) + t (x2 - x0)
#pragma unroll
    for (int c = 0; c < LC; ++c) {
        acc.v[0][c] = x0[c] + (s * x1[c] + t * x2[c]);
        acc.v[1][c] = x1[c];
        acc.v[2][c] = x2[c];
    }
}

// OsdEvaluatePatchBasis + gather for one point: normalises (s,t) into the patch, evaluates
// the basis of `type`, accumulates into acc and returns the derivative scales d1, d2
// (patchBasis.h:1558-1610).  Returns false for an unknown type.
template <int LC, bool QUAD_ONLY = false>
__device__ bool eval_patch_point(int type, Param p, float s, float t,
                                 const int *__restrict__ cvs, const float *__restrict__ src,
                                 int stride, int e0, int length, Acc6<LC> &acc, float &d1,
                                 float &d2) {
    const int depth = p.depth();
    const float frac = 1.0f / (float)(1 << (depth - p.nonquad()));
    const float fracInv = 1.0f / frac;
    float sign = 1.0f;
    const bool tri = (type == 5 || type == 10 || type == 4);
    if (tri && (p.u() + p.v()) >= (1 << depth)) {
        const int df = 1 << depth;
        s = (float)(df - p.u()) - s * fracInv;
        t = (float)(df - p.v()) - t * fracInv;
        sign = -1.0f;
    } else {
        s = s * fracInv - (float)p.u();
        t = t * fracInv - (float)p.v();
    }
    if (QUAD_ONLY) {  // Catmull-Clark tables: REGULAR, GREGORY_BASIS, QUADS
        switch (type) {
            case 6: eval_bspline<LC>(s, t, p.boundary(), cvs, src, stride, e0, length, acc); break;
            case 9: eval_gregory<LC>(s, t, cvs, src, stride, e0, length, acc); break;
            case 3: eval_linear_quad<LC>(s, t, cvs, src, stride, e0, length, acc); break;
            default: return false;
        }
    } else {
        switch (type) {
            case 6: eval_bspline<LC>(s, t, p.boundary(), cvs, src, stride, e0, length, acc); break;
            case 9: eval_gregory<LC>(s, t, cvs, src, stride, e0, length, acc); break;
            case 5: eval_box_tri<LC>(s, t, p.boundary(), cvs, src, stride, e0, length, acc); break;
            case 10: eval_gregory_tri<LC>(s, t, cvs, src, stride, e0, length, acc); break;
            case 3: eval_linear_quad<LC>(s, t, cvs, src, stride, e0, length, acc); break;
            case 4: eval_linear_tri<LC>(s, t, cvs, src, stride, e0, length, acc); break;
            default: return false;
        }
    }
    d1 = sign * (float)(1 << depth);
    d2 = sign * d1 * d1;
    return true;
}

// ---- per-control-point weights ---------------------------------------------------------------
// The bases above written out per control point instead of applied to points: w[k][j] is the
// weight of control point j for output k (P, Ds, Dt, Dss, Dst, Dtt), k < NK, derivatives scaled
// by +-2^depth / +-4^depth as eval_patch_point scales its sums.  These are the per-location
// masks Far::LimitStencilTableFactory merges over its point stencils
// (far/stencilTableFactory.cpp:560-640) and the coefficients Bfr::Surface::EvaluateStencil
// returns (bfr/surface.h:244-265).  Returns the number of control points, 0 for an unknown type.
template <int NK>
__device__ __forceinline__ void put_tensor(float (&w)[NK][20], int j, float cell[6]) {
#pragma unroll
    for (int k = 0; k < NK; ++k) w[k][j] += cell[k];
}

template <int NK>
__device__ int patch_point_weights(int type, Param p, float s, float t, float (&w)[NK][20]) {
#pragma unroll
    for (int k = 0; k < NK; ++k)
#pragma unroll
        for (int j = 0; j < 20; ++j) w[k][j] = 0.0f;
    const int depth = p.depth();
    const float frac = 1.0f / (float)(1 << (depth - p.nonquad()));
    const float fracInv = 1.0f / frac;
    float sign = 1.0f;
    const bool tri = (type == 5 || type == 10 || type == 4);
    if (tri && (p.u() + p.v()) >= (1 << depth)) {
        const int df = 1 << depth;
        s = (float)(df - p.u()) - s * fracInv;
        t = (float)(df - p.v()) - t * fracInv;
        sign = -1.0f;
    } else {
        s = s * fracInv - (float)p.u();
        t = t * fracInv - (float)p.v();
    }
    int n = 0;
    if (type == 6 || type == 9) {
        // tensor products: cell (r, c) weights for the six outputs
        float sp[4], sd[4], sdd[4], tp[4], td[4], tdd[4];
        if (type == 6) {
            bspline_curve(s, sp, sd, sdd);
            bspline_curve(t, tp, td, tdd);
            const int b = p.boundary();
            if (b & 1) { fold_first(tp); fold_first(td); fold_first(tdd); }
            if (b & 2) { fold_last(sp); fold_last(sd); fold_last(sdd); }
            if (b & 4) { fold_last(tp); fold_last(td); fold_last(tdd); }
            if (b & 8) { fold_first(sp); fold_first(sd); fold_first(sdd); }
            n = 16;
        } else {
            bezier_curve(s, sp, sd, sdd);
            bezier_curve(t, tp, td, tdd);
            n = 20;
        }
        const float sc = 1.0f - s, tc = 1.0f - t;
        float d0 = s + t;   d0 = (d0 <= 0.0f) ? 1.0f : (1.0f / d0);
        float d1 = sc + t;  d1 = (d1 <= 0.0f) ? 1.0f : (1.0f / d1);
        float d2 = sc + tc; d2 = (d2 <= 0.0f) ? 1.0f : (1.0f / d2);
        float d3 = s + tc;  d3 = (d3 <= 0.0f) ? 1.0f : (1.0f / d3);
        const float g0 = s * d0, g2 = t * d1, g4 = sc * d2, g6 = tc * d3;
        constexpr int kGrid[4][4] = {{0, 1, 7, 5}, {2, -1, -2, 6}, {16, -4, -3, 12},
                                     {15, 17, 11, 10}};
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                float cell[6] = {sp[c] * tp[r], sd[c] * tp[r], sp[c] * td[r],
                                 sdd[c] * tp[r], sd[c] * td[r], sp[c] * tdd[r]};
                if (type == 6) {
                    put_tensor<NK>(w, 4 * r + c, cell);
                    continue;
                }
                const int g = kGrid[r][c];
                if (g >= 0) {
                    put_tensor<NK>(w, g, cell);
                } else {
                    // blended interior pair (a, a + 1) by ga (patchBasis.h:346-378)
                    const int a = (g == -1) ? 3 : (g == -2) ? 8 : (g == -3) ? 13 : 18;
                    const float ga = (g == -1) ? g0 : (g == -2) ? g2 : (g == -3) ? g4 : g6;
                    float ca[6], cb[6];
#pragma unroll
                    for (int k = 0; k < 6; ++k) ca[k] = ga * cell[k], cb[k] = (1.0f - ga) * cell[k];
                    put_tensor<NK>(w, a, ca);
                    put_tensor<NK>(w, a + 1, cb);
                }
            }
    } else if (type == 10) {
        float g[6] = {1.0f, 0.0f, 1.0f, 0.0f, 1.0f, 0.0f};
        const float u = s, v = t, ww = 1.0f - u - v;
        if ((u + v) > 0) { g[0] = u / (u + v); g[1] = v / (u + v); }
        if ((v + ww) > 0) { g[2] = v / (v + ww); g[3] = ww / (v + ww); }
        if ((ww + u) > 0) { g[4] = ww / (ww + u); g[5] = u / (ww + u); }
        constexpr int kBez[15] = {0, 1, 15, 7, 5, 2, -1, -2, 6, 17, -3, 16, 11, 12, 10};
        constexpr int kOrd[6][2] = {{0, 0}, {1, 0}, {0, 1}, {2, 0}, {1, 1}, {0, 2}};
#pragma unroll
        for (int k = 0; k < NK; ++k) {
            float b[15];
            bezier_tri_weights(s, t, kOrd[k][0], kOrd[k][1], b);
#pragma unroll
            for (int m = 0; m < 15; ++m) {
                const int gi = kBez[m];
                if (gi >= 0) {
                    w[k][gi] += b[m];
                } else {
                    const int a = (gi == -1) ? 3 : (gi == -2) ? 8 : 13;
                    const float ga = (gi == -1) ? g[0] : (gi == -2) ? g[2] : g[4];
                    const float gb = (gi == -1) ? g[1] : (gi == -2) ? g[3] : g[5];
                    w[k][a] += ga * b[m];
                    w[k][a + 1] += gb * b[m];
                }
            }
        }
        n = 18;
    } else if (type == 5) {
        // the box-spline rows of eval_box_tri, per derivative order, with the boundary folds
        float m[15];
        m[0] = 1.0f; m[1] = s; m[2] = t;
        m[3] = s * s; m[4] = s * t; m[5] = t * t;
        m[6] = m[3] * s; m[7] = m[4] * s; m[8] = m[4] * t; m[9] = m[5] * t;
        m[10] = m[6] * s; m[11] = m[7] * s; m[12] = m[3] * m[5]; m[13] = m[8] * t;
        m[14] = m[9] * t;
#pragma unroll
        for (int k = 0; k < NK; ++k) {
            float wk[12];
            box_weights(k, m, wk);
            box_fold(p.boundary(), wk);
#pragma unroll
            for (int j = 0; j < 12; ++j) w[k][j] = wk[j];
        }
        n = 12;
    } else if (type == 3) {
        const float sc = 1.0f - s, tc = 1.0f - t;
        const float wp[4] = {sc * tc, s * tc, s * t, sc * t};
        const float ws[4] = {-tc, tc, t, -t};
        const float wt[4] = {-sc, -s, s, sc};
        const float wst[4] = {1.0f, -1.0f, 1.0f, -1.0f};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            w[0][j] = wp[j];
            if constexpr (NK > 2) w[1][j] = ws[j], w[2][j] = wt[j];
            if constexpr (NK > 4) w[4][j] = wst[j];
        }
        n = 4;
    } else if (type == 4) {
        w[0][0] = 1.0f - s - t, w[0][1] = s, w[0][2] = t;
        if constexpr (NK > 2) {
            w[1][0] = -1.0f, w[1][1] = 1.0f;
            w[2][0] = -1.0f, w[2][2] = 1.0f;
        }
        n = 3;
    } else {
        return 0;
    }
    const float d1 = sign * (float)(1 << depth), d2 = sign * d1 * d1;
#pragma unroll
    for (int k = 1; k < NK; ++k) {
        const float sc = k < 3 ? d1 : d2;
#pragma unroll
        for (int j = 0; j < 20; ++j) w[k][j] *= sc;
    }
    return n;
}

}  // namespace gb300
