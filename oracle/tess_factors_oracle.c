/*
 * tess_factors_oracle.c -- CPU restatement of the draw-time tessellation factors of
 * OpenSubdiv's patch shaders (the checker).
 *
 * TEST INFRASTRUCTURE ONLY: loaded by tests/; never by the product.  The reference's version is
 * GLSL shader code (opensubdiv/osd/glslPatchCommonTess.glsl, with the same math in the HLSL and
 * Metal files), which cannot run without a graphics stack: this restatement follows the GLSL
 * line by line and is not pinned against an execution of the reference.  Limit positions at
 * the patch corners and edge midpoints come from the restated patch bases (osd_oracle.c).
 */
#include "osd_oracle.h"

#include <math.h>
#include <string.h>

typedef struct {
    float x, y, z;
} V3;

/* limit position at patch-local (s, t): the basis of the patch with its refinement level and
 * sub-face offset cleared, so that no normalization is applied */
static V3 limit_point(int type, int f0, int f1, float s, float t, const int *cvs, const float *src,
                      int stride) {
    float w[120];
    const int local = f1 & ((0x1f << 7) | (1 << 5));
    const int n = orc_patch_basis_f(type, f0, local, s, t, w);
    V3 p = {0.0f, 0.0f, 0.0f};
    for (int j = 0; j < n; ++j) {
        const float *r = src + (long)cvs[j] * stride;
        p.x += w[j] * r[0];
        p.y += w[j] * r[1];
        p.z += w[j] * r[2];
    }
    return p;
}

static void xform(const float *m, V3 x, float out[4]) {
    for (int r = 0; r < 4; ++r) out[r] = m[r] * x.x + m[4 + r] * x.y + m[8 + r] * x.z + m[12 + r];
}

/* OsdComputeTessLevel (glslPatchCommonTess.glsl:98-117) */
static float edge_level(float tessLevel, float maxLevel, const float *mv, const float *proj,
                        V3 p0, V3 p1) {
    float a[4], b[4], q[4];
    xform(mv, p0, a);
    xform(mv, p1, b);
    V3 c = {(a[0] + b[0]) / 2.0f, (a[1] + b[1]) / 2.0f, (a[2] + b[2]) / 2.0f};
    float dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    float diameter = sqrtf(dx * dx + dy * dy + dz * dz);
    xform(proj, c, q);
    float projLength = fabsf(diameter * proj[5] / q[3]);
    float level = fmaxf(1.0f, tessLevel * projLength);
    return fminf(level, maxLevel / 2.0f);
}

static float round_up_even(float x) { return 2.0f * ceilf(x / 2.0f); }
static float round_up_odd(float x) { return 2.0f * ceilf((x + 1.0f) / 2.0f) - 1.0f; }

int orc_tess_factors(const int *arrays, int numArrays, const int *indices, const int *params,
                     int numPatches, const float *src, int srcStride, float tessLevel,
                     float maxTessLevel, int screenSpace, int spacing, const float *mv,
                     const float *proj, float *outer, float *inner, float *outLo, float *outHi) {
    for (int p = 0; p < numPatches; ++p) {
        int k = 0;
        while (k < numArrays && !(p >= arrays[6 * k + 5] && p < arrays[6 * k + 5] + arrays[6 * k + 2]))
            ++k;
        float lo[4] = {0, 0, 0, 0}, hi[4] = {0, 0, 0, 0}, out[4] = {0, 0, 0, 0}, in[2] = {0, 0};
        if (k < numArrays) {
            const int *a = arrays + 6 * k;
            const int f0 = params[3 * p], f1 = params[3 * p + 1];
            const int regular = (f1 >> 5) & 1;
            const int type = regular ? a[0] : a[1];
            const int tri = type == 4 || type == 5 || type == 10;
            const int transition = (f0 >> 28) & 0xf;
            const int depth = f1 & 0xf;
            if (!screenSpace) {
                /* OsdGetTessLevelsUniform[Triangle] (glslPatchCommonTess.glsl:119-163) */
                float level = fminf(tessLevel, maxTessLevel) / powf(2.0f, (float)(depth - 1));
                float mn[4];
                if (tri) {
                    mn[0] = 1.0f + ((transition & 4) >> 2);
                    mn[1] = 1.0f + (transition & 1);
                    mn[2] = 1.0f + ((transition & 2) >> 1);
                    mn[3] = 1.0f;
                } else {
                    mn[0] = 1.0f + ((transition & 8) >> 3);
                    mn[1] = 1.0f + (transition & 1);
                    mn[2] = 1.0f + ((transition & 2) >> 1);
                    mn[3] = 1.0f + ((transition & 4) >> 2);
                }
                for (int e = 0; e < 4; ++e) lo[e] = fmaxf(level, mn[e]);
            } else {
                const int *cvs = indices + a[3] + a[4] * (p - a[5]);
#define LP(s, t) limit_point(type, f0, f1, s, t, cvs, src, srcStride)
#define EL(p0, p1) edge_level(tessLevel, maxTessLevel, mv, proj, p0, p1)
                if (!tri) {
                    /* Osd_GetTessLevelsFromPatchBoundaries4 (:231-264) */
                    V3 c0 = LP(0.0f, 0.0f), c1 = LP(1.0f, 0.0f), c2 = LP(1.0f, 1.0f),
                       c3 = LP(0.0f, 1.0f);
                    if (transition & 8) {
                        V3 m = LP(0.0f, 0.5f);
                        lo[0] = EL(c0, m), hi[0] = EL(c3, m);
                    } else {
                        lo[0] = EL(c0, c3);
                    }
                    if (transition & 1) {
                        V3 m = LP(0.5f, 0.0f);
                        lo[1] = EL(c0, m), hi[1] = EL(c1, m);
                    } else {
                        lo[1] = EL(c0, c1);
                    }
                    if (transition & 2) {
                        V3 m = LP(1.0f, 0.5f);
                        lo[2] = EL(c1, m), hi[2] = EL(c2, m);
                    } else {
                        lo[2] = EL(c1, c2);
                    }
                    if (transition & 4) {
                        V3 m = LP(0.5f, 1.0f);
                        lo[3] = EL(c3, m), hi[3] = EL(c2, m);
                    } else {
                        lo[3] = EL(c3, c2);
                    }
                } else {
                    /* Osd_GetTessLevelsFromPatchBoundaries3 (:266-293) */
                    V3 c0 = LP(0.0f, 0.0f), c1 = LP(1.0f, 0.0f), c2 = LP(0.0f, 1.0f);
                    if (transition & 4) {
                        V3 m = LP(0.0f, 0.5f);
                        lo[0] = EL(c0, m), hi[0] = EL(c2, m);
                    } else {
                        lo[0] = EL(c0, c2);
                    }
                    if (transition & 1) {
                        V3 m = LP(0.5f, 0.0f);
                        lo[1] = EL(c0, m), hi[1] = EL(c1, m);
                    } else {
                        lo[1] = EL(c0, c1);
                    }
                    if (transition & 2) {
                        V3 m = LP(0.5f, 0.5f);
                        lo[2] = EL(c2, m), hi[2] = EL(c1, m);
                    } else {
                        lo[2] = EL(c1, c2);
                    }
                }
#undef LP
#undef EL
            }
            /* OsdComputeTessLevels[Triangle] (:413-500) */
            float comb[4];
            for (int e = 0; e < 4; ++e) comb[e] = lo[e] + hi[e];
            if (spacing == 1) {
                for (int e = 0; e < 4; ++e) {
                    out[e] = comb[e];
                    if (hi[e] > 0) out[e] = round_up_even(lo[e]) + round_up_even(hi[e]);
                }
            } else if (spacing == 2) {
                for (int e = 0; e < 4; ++e) out[e] = comb[e];
                for (int e = 0; e < 4; ++e) {
                    if (hi[e] > 0) {
                        out[e] = round_up_odd(lo[e]) + round_up_odd(hi[e]);
                        for (int j = 0; j < 4; ++j) comb[j] = fmaxf(3.0f, comb[j]);
                    }
                }
            } else {
                for (int e = 0; e < 4; ++e) {
                    lo[e] = roundf(lo[e]);
                    hi[e] = roundf(hi[e]);
                    comb[e] = lo[e] + hi[e];
                    out[e] = comb[e];
                }
            }
            in[0] = (comb[1] + comb[3]) * 0.5f;
            in[1] = (comb[0] + comb[2]) * 0.5f;
            if (tri) in[0] = fmaxf(fmaxf(out[0], out[1]), out[2]);
        }
        memcpy(outer + 4 * (long)p, out, sizeof out);
        memcpy(inner + 2 * (long)p, in, sizeof in);
        if (outLo) memcpy(outLo + 4 * (long)p, lo, sizeof lo);
        if (outHi) memcpy(outHi + 4 * (long)p, hi, sizeof hi);
    }
    return 1;
}

/* OsdGetTessFractionalSplit (glslPatchCommonTess.glsl:607-645) */
static float fractional_split(float t, float level, float levelUp, int spacing) {
    float base, offset;
    if (spacing == 1) {
        if (level <= 2) return t;
        base = powf(2.0f, floorf(log2f(levelUp)));
        offset = 1.0f / (float)(((int)(2 * base - levelUp) / 2) & (int)(base / 2 - 1));
    } else {
        if (level <= 1) return t;
        base = powf(2.0f, floorf(log2f(levelUp)));
        offset = 1.0f / (float)((((int)(2 * base - levelUp) / 2 + 1) & (int)(base / 2 - 1)) + 1);
    }
    float dx0 = (1.0f - (levelUp - level) / 2) / levelUp;
    float dx1 = (1.0f - 2.0f * dx0) / (levelUp - 2.0f * ceilf(dx0));
    if (t < 0.5f) {
        float x = levelUp / 2 - roundf(t * levelUp);
        return 0.5f - (x * dx1 + (float)(x * offset > 1) * (dx0 - dx1));
    } else if (t > 0.5f) {
        float x = roundf(t * levelUp) - levelUp / 2;
        return 0.5f + (x * dx1 + (float)(x * offset > 1) * (dx0 - dx1));
    }
    return t;
}

/* OsdGetTessTransitionSplit (glslPatchCommonTess.glsl:647-690) */
static float transition_split(float t, float lo, float hi, int spacing) {
    if (spacing == 1) {
        float loUp = round_up_even(lo), hiUp = round_up_even(hi);
        float ti = roundf(t * (loUp + hiUp));
        if (ti <= loUp) return fractional_split(ti / loUp, lo, loUp, 1) * 0.5f;
        return fractional_split((ti - loUp) / hiUp, hi, hiUp, 1) * 0.5f + 0.5f;
    }
    if (spacing == 2) {
        float loUp = round_up_odd(lo), hiUp = round_up_odd(hi);
        float ti = roundf(t * (loUp + hiUp + 1));
        if (ti <= loUp) return fractional_split(ti / loUp, lo, loUp, 2) * 0.5f;
        if (ti > (loUp + 1)) return fractional_split((ti - (loUp + 1)) / hiUp, hi, hiUp, 2) * 0.5f + 0.5f;
        return 0.5f;
    }
    float ti = roundf(t * (lo + hi));
    if (ti <= lo) return (ti / lo) * 0.5f;
    return ((ti - lo) / hi) * 0.5f + 0.5f;
}

/* OsdGetTessParameterization[Triangle] (glslPatchCommonTess.glsl:692-730) */
int orc_tess_parameterization(int n, const float *domain, const int *patchIndex,
                              const float *outerLo, const float *outerHi, int spacing,
                              int triangular, float *uv) {
    for (int i = 0; i < n; ++i) {
        float px = domain[3 * i], py = domain[3 * i + 1], pz = domain[3 * i + 2];
        const float *lo = outerLo + 4 * (long)patchIndex[i], *hi = outerHi + 4 * (long)patchIndex[i];
        float u = px, v = py;
        if (!triangular) {
            if (px == 0 && hi[0] > 0) v = transition_split(v, lo[0], hi[0], spacing);
            else if (py == 0 && hi[1] > 0) u = transition_split(u, lo[1], hi[1], spacing);
            else if (px == 1 && hi[2] > 0) v = transition_split(v, lo[2], hi[2], spacing);
            else if (py == 1 && hi[3] > 0) u = transition_split(u, lo[3], hi[3], spacing);
        } else {
            if (px == 0 && hi[0] > 0) v = transition_split(v, lo[0], hi[0], spacing);
            else if (py == 0 && hi[1] > 0) u = transition_split(u, lo[1], hi[1], spacing);
            else if (pz == 0 && hi[2] > 0) {
                u = transition_split(u, lo[2], hi[2], spacing);
                v = 1.0f - u;
            }
        }
        uv[2 * i] = u;
        uv[2 * i + 1] = v;
    }
    return 1;
}
