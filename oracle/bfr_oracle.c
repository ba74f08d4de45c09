/*
 * bfr_oracle.c -- CPU restatement of Bfr::Parameterization and Bfr::Tessellation (the checker).
 *
 * TEST INFRASTRUCTURE ONLY: loaded by tests/ and bench.py's CPU baseline; never by the product.
 * Built with floating-point contraction disabled (oracle/Makefile) so that every coordinate
 * rounds exactly as the reference's float instantiation does.
 *
 * One face per call, sequential, following the reference's construction order: boundary
 * coords edge by edge, then interior rings from the outside in; facets ring by ring, each ring
 * strip by strip.  Citations are relative to the OpenSubdiv 3.6.0 source tree
 * (opensubdiv/bfr/tessellation.cpp unless named otherwise).
 */
#include "osd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

enum { K_QUAD = 0, K_TRI = 1, K_QSUB = 2 };

/* Far::VALENCE_LIMIT (far/types.h), the largest face Bfr::Parameterization accepts */
#define ORC_MAX_FACE_SIZE ((1 << 16) - 1)
#define ORC_MAX_RATE 32767

/* ---- Bfr::Parameterization (bfr/parameterization.cpp:40-66, 73-96) ------------------------ */

typedef struct {
    int kind, N, udim;
} Param;

static int param_init(Param *p, int regFaceSize, int N) {
    p->N = N;
    p->udim = 0;
    p->kind = (regFaceSize == 4) ? K_QUAD : K_TRI;
    if (N == regFaceSize) return 1;
    if (N < 3 || N > ORC_MAX_FACE_SIZE || regFaceSize == 3) return 0;
    p->kind = K_QSUB;
    p->udim = (N < 10) ? 2 + (N > 4) : 1 + (int)sqrtf((float)(N - 1));
    return 1;
}

static void param_vertex(const Param *p, int v, float uv[2]) {
    if (p->kind == K_QUAD) {
        uv[0] = (float)(v && v < 3);
        uv[1] = (float)(v > 1);
    } else if (p->kind == K_TRI) {
        uv[0] = (float)(v == 1);
        uv[1] = (float)(v == 2);
    } else {
        uv[0] = (float)(v % p->udim);
        uv[1] = (float)(v / p->udim);
    }
}

/* Parameterization::ConvertCoordToNormalizedSubFace (bfr/parameterization.cpp:135-162) */
int orc_param_to_subface(int regFaceSize, int N, int n, const float *uv, int *sub, float *st) {
    Param p;
    if (!param_init(&p, regFaceSize, N)) return 0;
    for (int i = 0; i < n; ++i) {
        float u = uv[2 * i], v = uv[2 * i + 1];
        if (p.kind != K_QSUB) {
            sub[i] = 0;
            st[2 * i] = u;
            st[2 * i + 1] = v;
            continue;
        }
        int ut = (int)u, vt = (int)v;
        float uf = u - (float)ut, vf = v - (float)vt;
        if (uf > 0.75f) {
            ut++;
            uf = uf - 1.0f;
        }
        if (vf > 0.75f) {
            vt++;
            vf = vf - 1.0f;
        }
        st[2 * i] = uf * 2.0f;
        st[2 * i + 1] = vf * 2.0f;
        sub[i] = p.udim * vt + ut;
    }
    return 1;
}

/* ---- output sinks ------------------------------------------------------------------------- */

typedef struct {
    float *c;
    int stride;
} Coords;

typedef struct {
    int *f;
    int size, stride;
} Facets;

static void put_uv(Coords o, int i, float u, float v) {
    o.c[(long)i * o.stride] = u;
    o.c[(long)i * o.stride + 1] = v;
}

/* appendVIsoLine / appendUIsoLine / appendUVLine (tessellation.cpp:160-188): the running
 * parameter is accumulated, not recomputed, so the roundings follow the reference's sums */
static int run_u(Coords o, int at, int n, float u, float v, float du) {
    for (int i = 0; i < n; ++i, u += du) put_uv(o, at + i, u, v);
    return n;
}
static int run_v(Coords o, int at, int n, float u, float v, float dv) {
    for (int i = 0; i < n; ++i, v += dv) put_uv(o, at + i, u, v);
    return n;
}
static int run_uv(Coords o, int at, int n, float u, float v, float du, float dv) {
    for (int i = 0; i < n; ++i, u += du, v += dv) put_uv(o, at + i, u, v);
    return n;
}

static int *facet_at(Facets o, int i) { return o.f + (long)i * o.stride; }

/* Facet::Set for three indices (tessellation.cpp:114-118): the last slot of a 4-tuple is -1 */
static int tri3(Facets o, int at, int a, int b, int c) {
    int *t = facet_at(o, at);
    t[o.size - 1] = -1;
    t[0] = a, t[1] = b, t[2] = c;
    return 1;
}

/* appendQuad (tessellation.cpp:200-219): sign 0 keeps the quad, > 0 splits along q0-q2,
 * < 0 along q1-q3 */
static int quad4(Facets o, int at, int a, int b, int c, int d, int sign) {
    if (sign == 0) {
        int *t = facet_at(o, at);
        t[0] = a, t[1] = b, t[2] = c, t[3] = d;
        return 1;
    }
    if (sign > 0) {
        tri3(o, at, a, b, c);
        tri3(o, at + 1, c, d, a);
    } else {
        tri3(o, at, c, d, b);
        tri3(o, at + 1, a, b, d);
    }
    return 2;
}

/* appendTriFan (tessellation.cpp:221-230) */
static int fan(Facets o, int at, int size, int start) {
    for (int i = 1; i <= size; ++i)
        tri3(o, at + i - 1, start + i - 1, start + ((i < size) ? i : 0), start + size);
    return size;
}

/* ---- FacetStrip (tessellation.cpp:233-617) ------------------------------------------------ */

typedef struct {
    int quads, triangulate, reversed;
    int exclFirst, splitFirst, splitLast, inclLast;
    int nOuter, nInner;
    int oFirst, oLast, oPrev, iFirst, iLast;
} Strip;

/* connectUniformQuads (tessellation.cpp:283-350) */
static int strip_quads(const Strip *s, Facets o, int at) {
    int n = 0;
    int tri = s->triangulate;
    if (s->splitFirst)
        n += tri3(o, at + n, s->oFirst, s->oFirst + 1, s->iFirst);
    else if (!s->exclFirst)
        n += quad4(o, at + n, s->oFirst, s->oFirst + 1, s->iFirst, s->oPrev, tri);

    int oi = s->oFirst + 1, ii = s->iFirst;
    int step = s->reversed ? -1 : 1;
    for (int i = 1; i <= s->nInner; ++i, ++oi, ii += step) {
        int sign = (i > s->nInner / 2) ? -tri : tri;
        int ij = (i < s->nInner) ? ii + step : s->iLast;
        n += quad4(o, at + n, oi, oi + 1, ij, ii, sign);
    }
    if (s->splitLast)
        n += tri3(o, at + n, oi, s->oLast, s->iLast);
    else if (s->inclLast)
        n += quad4(o, at + n, oi, s->oLast, s->oLast + 1, s->iLast, -tri);
    return n;
}

/* connectUniformTris (tessellation.cpp:352-420) */
static int strip_tris(const Strip *s, Facets o, int at) {
    int n = 0;
    int o0 = s->oFirst, i0 = s->iFirst;
    if (s->splitFirst) {
        n += tri3(o, at + n, o0, o0 + 1, i0);
    } else {
        n += tri3(o, at + n, o0, o0 + 1, s->oPrev);
        n += tri3(o, at + n, i0, s->oPrev, o0 + 1);
    }
    n += tri3(o, at + n, o0 + 1, o0 + 2, i0);
    int oi = o0 + 2, ii = i0;
    for (int i = 1; i <= s->nInner; ++i, ++ii, ++oi) {
        int ij = (i < s->nInner) ? ii + 1 : s->iLast;
        n += tri3(o, at + n, ij, ii, oi);
        n += tri3(o, at + n, oi, oi + 1, ij);
    }
    if (s->splitLast) n += tri3(o, at + n, oi, s->oLast, s->iLast);
    return n;
}

/* connectNonUniformFacets (tessellation.cpp:422-633): both rings are parameterised over
 * [0, M*N] and each facet takes the diagonal spanning the shorter interval, with a symmetric
 * middle facet; when quads are kept, a facet past the middle mirrors its counterpart's kind */
static int strip_general(const Strip *s, Facets o, int at) {
    int M = s->nInner + (s->quads ? 2 : 3);
    int N = s->nOuter;
    int dtO = M, dtI = N;
    int dtMin = dtI < dtO ? dtI : dtO, dtMax = dtI < dtO ? dtO : dtI;
    int slopeMax = ((dtMax / 2) < dtMin) ? (dtMin - 1) : (dtMax / 2);
    int tOLast = dtO * N, tOMid = tOLast / 2;
    int tIOff = 0, tILast = dtI * (M - 1);
    if (!s->quads) {
        tIOff = dtI / 2;
        tILast += tIOff - dtI;
    }
    int dI = s->reversed ? -1 : 1;

    int tO0 = 0, cO0 = s->oFirst;
    int tO1 = dtO, cO1 = (N == 1) ? s->oLast : s->oFirst + 1;
    int tI0 = tIOff + dtI, cI0 = s->iFirst;
    int tI1 = tI0 + (s->nInner ? dtI : 0);
    int cI1 = (s->nInner == 1) ? s->iLast : s->iFirst + dI;

    int keepQuads = s->quads && !s->triangulate;
    int total;
    if (keepQuads) {
        total = s->nInner > s->nOuter ? s->nInner : s->nOuter;
        if ((total & 1) == 0) total += (s->nInner & 1) || (s->nOuter & 1);
    } else {
        total = s->nInner + s->nOuter;
    }
    int lead = total / 2, mid = total & 1;
    int midFacet = mid ? lead : -1;
    int midQuad = keepQuads && (s->nOuter & 1) && (s->nInner & 1);

    for (int k = 0; k < total; ++k) {
        int triO = 0, triI = 0, q = 0;
        if (k == midFacet) {
            if (midQuad) q = 1;
            else if (s->nOuter & 1) triO = 1;
            else triI = 1;
        } else if (tI1 == tI0) {
            triO = 1;
        } else if (tO1 == tO0) {
            triI = 1;
        } else {
            if (keepQuads) {
                if (k >= lead) {
                    int mirror = lead - 1 - (k - lead - mid);
                    q = facet_at(o, at + mirror)[3] >= 0;
                } else if (tI1 > tOMid || tO1 > tOMid) {
                    q = 0;
                } else {
                    q = abs(tO1 - tI1) <= slopeMax;
                }
            }
            if (!q) {
                int toOuter = tO1 - tI0, toInner = tI1 - tO0;
                int useOuter = (toOuter == toInner) ? (tO1 > tOMid) : (toOuter < toInner);
                if (useOuter) triO = 1;
                else triI = 1;
            }
        }
        if (triO)
            tri3(o, at + k, cO0, cO1, cI0);
        else if (triI)
            tri3(o, at + k, cI1, cI0, cO0);
        else
            quad4(o, at + k, cO0, cO1, cI1, cI0, 0);

        if (triO || q) {
            tO0 = tO1, cO0 = cO1;
            tO1 += dtO, cO1 += 1;
            if (tO1 >= tOLast) tO1 = tOLast, cO1 = s->oLast;
        }
        if (triI || q) {
            tI0 = tI1, cI0 = cI1;
            tI1 += dtI, cI1 += dI;
            if (tI1 >= tILast) tI1 = tILast, cI1 = s->iLast;
        }
    }
    return total;
}

/* ---- quad parameterisation (tessellation.cpp:801-1285) ------------------------------------ */

static int quad_boundary_coords(const int *r, Coords o) {
    int n = 0;
    n += run_u(o, n, r[0], 0.0f, 0.0f, 1.0f / (float)r[0]);
    n += run_v(o, n, r[1], 1.0f, 0.0f, 1.0f / (float)r[1]);
    n += run_u(o, n, r[2], 1.0f, 1.0f, -1.0f / (float)r[2]);
    n += run_v(o, n, r[3], 0.0f, 1.0f, -1.0f / (float)r[3]);
    return n;
}

static int quad_interior_coords(const int uv[2], Coords o, int at) {
    int rings = (uv[0] / 2 < uv[1] / 2) ? uv[0] / 2 : uv[1] / 2;
    if (rings == 0) return 0;
    float du = 1.0f / (float)uv[0], dv = 1.0f / (float)uv[1];
    float u = du, v = dv;
    int ur = uv[0] - 2, vr = uv[1] - 2, n = 0;
    for (int i = 0; i < rings; ++i, ur -= 2, vr -= 2, u += du, v += dv) {
        if (ur > 0 && vr > 0) {
            float u1 = 1.0f - u, v1 = 1.0f - v;
            n += run_u(o, at + n, ur, u, v, du);
            n += run_v(o, at + n, vr, u1, v, dv);
            n += run_u(o, at + n, ur, u1, v1, -du);
            n += run_v(o, at + n, vr, u, v1, -dv);
        } else if (ur > 0) {
            n += run_u(o, at + n, ur + 1, u, v, du);
        } else if (vr > 0) {
            n += run_v(o, at + n, vr + 1, u, v, dv);
        } else {
            put_uv(o, at + n, 0.5f, 0.5f);
            n += 1;
        }
    }
    return n;
}

/* getSingleStripFacets (tessellation.cpp:998-1034) */
static int quad_single_strip(int ur, int vr, int c0, int tri, Facets o, int at) {
    Strip s;
    memset(&s, 0, sizeof s);
    s.quads = 1, s.triangulate = tri, s.reversed = 1, s.inclLast = 1;
    if (ur > 1) {
        s.nOuter = ur, s.nInner = ur - 2;
        s.oFirst = c0;
        s.oLast = c0 + ur;
        s.iLast = s.oLast + 2;
        s.iFirst = s.oLast + ur;
        s.oPrev = s.iFirst + 1;
    } else {
        s.nOuter = vr, s.nInner = vr - 2;
        s.oPrev = c0;
        s.oFirst = c0 + 1;
        s.oLast = s.oFirst + vr;
        s.iLast = s.oLast + 2;
        s.iFirst = s.oLast + vr;
    }
    return strip_quads(&s, o, at);
}

/* getInteriorRingFacets (tessellation.cpp:1037-1118) */
static int quad_ring(int ur, int vr, int c0, int tri, Facets o, int at) {
    int cells = ur * vr;
    if (cells == 0) return 0;
    if (cells == 1) return quad4(o, at, c0, c0 + 1, c0 + 2, c0 + 3, tri);
    if (ur == 1 || vr == 1) return quad_single_strip(ur, vr, c0, tri, o, at);

    int uIn = ur - 2, vIn = vr - 2;
    int outer0 = c0, inner0 = c0 + 2 * (ur + vr);
    int n = 0;
    Strip s;
    memset(&s, 0, sizeof s);
    s.quads = 1, s.triangulate = tri;

    s.nOuter = ur, s.oFirst = outer0, s.oPrev = inner0 - 1, s.oLast = outer0 + ur;
    s.nInner = uIn, s.reversed = 0, s.iFirst = inner0, s.iLast = inner0 + uIn;
    n += strip_quads(&s, o, at + n);

    s.nOuter = vr, s.oFirst += ur, s.oPrev = s.oFirst - 1, s.oLast = s.oFirst + vr;
    s.nInner = vIn, s.reversed = 0, s.iFirst = s.iLast, s.iLast += vIn;
    n += strip_quads(&s, o, at + n);

    s.nOuter = ur, s.oFirst += vr, s.oPrev = s.oFirst - 1, s.oLast = s.oFirst + ur;
    s.nInner = uIn, s.reversed = (vIn == 0), s.iFirst = s.iLast;
    s.iLast += uIn * (s.reversed ? -1 : 1);
    n += strip_quads(&s, o, at + n);

    s.nOuter = vr, s.oFirst += ur, s.oPrev = s.oFirst - 1, s.oLast = outer0;
    s.nInner = vIn, s.reversed = (uIn == 0), s.iFirst = s.iLast, s.iLast = inner0;
    n += strip_quads(&s, o, at + n);
    return n;
}

/* getBoundaryRingFacets (tessellation.cpp:1121-1225) */
static int quad_boundary_ring(const int *outer, int ur, int vr, int nB, int tri, Facets o,
                              int at) {
    int uni[4] = {outer[0] == ur, outer[1] == vr, outer[2] == ur, outer[3] == vr};
    int corner[4] = {uni[0] && uni[3], uni[1] && uni[0], uni[2] && uni[1], uni[3] && uni[2]};
    int uIn = ur - 2, vIn = vr - 2, n = 0;
    Strip s;
    memset(&s, 0, sizeof s);
    s.quads = 1, s.triangulate = tri;
    for (int e = 0; e < 4; ++e) {
        int inner = (e & 1) ? vIn : uIn;
        s.nOuter = outer[e];
        s.nInner = inner;
        if (e == 0) {
            s.oFirst = 0, s.oPrev = nB - 1, s.oLast = outer[0];
            s.reversed = 0, s.iFirst = nB, s.iLast = nB + uIn;
        } else {
            s.oFirst = s.oLast, s.oPrev = s.oFirst - 1;
            s.oLast = (e == 3) ? 0 : s.oLast + outer[e];
            s.reversed = (e == 2) ? (vIn == 0) : (e == 3) ? (uIn == 0) : 0;
            s.iFirst = s.iLast;
            s.iLast = (e == 3) ? nB : s.iLast + inner * (s.reversed ? -1 : 1);
        }
        if (uni[e]) {
            s.splitFirst = !corner[e];
            s.splitLast = !corner[(e + 1) & 3];
            n += strip_quads(&s, o, at + n);
        } else {
            s.splitFirst = s.splitLast = 1;
            n += strip_general(&s, o, at + n);
        }
    }
    return n;
}

/* ---- triangle parameterisation (tessellation.cpp:1301-1602) ------------------------------- */

static int tri_boundary_coords(const int *r, Coords o) {
    int n = 0;
    n += run_u(o, n, r[0], 0.0f, 0.0f, 1.0f / (float)r[0]);
    n += run_uv(o, n, r[1], 1.0f, 0.0f, -1.0f / (float)r[1], 1.0f / (float)r[1]);
    n += run_v(o, n, r[2], 0.0f, 1.0f, -1.0f / (float)r[2]);
    return n;
}

static int tri_interior_coords(int res, Coords o, int at) {
    int rings = res / 3;
    if (rings == 0) return 0;
    float dt = 1.0f / (float)res, u = dt, v = dt;
    int rr = res - 3, n = 0;
    for (int i = 0; i < rings; ++i, rr -= 3, u += dt, v += dt) {
        if (rr == 0) {
            put_uv(o, at + n, 1.0f / 3.0f, 1.0f / 3.0f);
            n += 1;
        } else {
            float u1 = 1.0f - u * 2.0f, v1 = 1.0f - v * 2.0f;
            n += run_u(o, at + n, rr, u, v, dt);
            n += run_uv(o, at + n, rr, u1, v, -dt, dt);
            n += run_v(o, at + n, rr, u, v1, -dt);
        }
    }
    return n;
}

/* tri::getInteriorRingFacets (tessellation.cpp:1425-1481) */
static int tri_ring(int res, int c0, Facets o, int at) {
    if (res < 1) return 0;
    if (res == 1) return tri3(o, at, c0, c0 + 1, c0 + 2);
    if (res == 2) {
        tri3(o, at + 0, c0 + 0, c0 + 1, c0 + 5);
        tri3(o, at + 1, c0 + 2, c0 + 3, c0 + 1);
        tri3(o, at + 2, c0 + 4, c0 + 5, c0 + 3);
        tri3(o, at + 3, c0 + 1, c0 + 3, c0 + 5);
        return 4;
    }
    int inner = res - 3, outer0 = c0, inner0 = c0 + 3 * res, n = 0;
    Strip s;
    memset(&s, 0, sizeof s);
    s.nInner = inner, s.nOuter = res;
    s.oFirst = outer0, s.oLast = outer0 + res, s.oPrev = inner0 - 1;
    s.iFirst = inner0, s.iLast = inner0 + inner;
    n += strip_tris(&s, o, at + n);
    s.oFirst += res, s.oLast += res, s.oPrev = s.oFirst - 1;
    s.iFirst += inner, s.iLast += inner;
    n += strip_tris(&s, o, at + n);
    s.oFirst += res, s.oLast = outer0, s.oPrev = s.oFirst - 1;
    s.iFirst += inner, s.iLast = inner0;
    n += strip_tris(&s, o, at + n);
    return n;
}

/* tri::getBoundaryRingFacets (tessellation.cpp:1484-1561) */
static int tri_boundary_ring(const int *outer, int res, int nB, Facets o, int at) {
    int uni[3] = {outer[0] == res, outer[1] == res, outer[2] == res};
    int corner[3] = {uni[0] && uni[2], uni[1] && uni[0], uni[2] && uni[1]};
    int inner = res - 3, n = 0;
    Strip s;
    memset(&s, 0, sizeof s);
    s.nInner = inner;
    for (int e = 0; e < 3; ++e) {
        s.nOuter = outer[e];
        if (e == 0) {
            s.oFirst = 0, s.oLast = outer[0], s.oPrev = nB - 1;
            s.iFirst = nB, s.iLast = nB + inner;
        } else {
            s.oFirst = s.oLast;
            s.oLast = (e == 2) ? 0 : s.oLast + outer[e];
            s.oPrev = s.oFirst - 1;
            s.iFirst = s.iLast;
            s.iLast = (e == 2) ? nB : s.iLast + inner;
        }
        if (uni[e]) {
            s.splitFirst = !corner[e];
            s.splitLast = !corner[(e + 1) % 3];
            n += strip_tris(&s, o, at + n);
        } else {
            s.splitFirst = s.splitLast = 1;
            n += strip_general(&s, o, at + n);
        }
    }
    return n;
}

/* ---- quad sub-faces of an N-gon (tessellation.cpp:1606-1983) ------------------------------ */

/* qsub::getRingEdgeCoords (tessellation.cpp:1689-1734): the first half of an edge runs along
 * u of sub-face `edge`, the second half down v of the next sub-face */
static int qsub_edge(const Param *p, int e, int res, int first, int last, float t0, float dt,
                     Coords o, int at) {
    int n0 = (res - 1) / 2, n1 = (res - 1) - n0, n = 0;
    if (first || n0) {
        float a[2];
        param_vertex(p, e, a);
        if (first) put_uv(o, at + n++, a[0] + t0, a[1] + t0);
        if (n0) n += run_u(o, at + n, n0, a[0] + t0 + dt, a[1] + t0, dt);
    }
    if (n1 || last) {
        float b[2];
        param_vertex(p, (e + 1) % p->N, b);
        if (n1) {
            float v = b[1] + ((res & 1) ? (0.5f - 0.5f * dt) : 0.5f);
            n += run_v(o, at + n, n1, b[0] + t0, v, -dt);
        }
        if (last) put_uv(o, at + n++, b[0] + t0, b[1] + t0);
    }
    return n;
}

static int qsub_boundary_coords(const Param *p, const int *r, Coords o) {
    int n = 0;
    for (int e = 0; e < p->N; ++e) n += qsub_edge(p, e, r[e], 1, 0, 0.0f, 1.0f / (float)r[e], o, n);
    return n;
}

static int qsub_interior_coords(const Param *p, int res, Coords o, int at) {
    int rings = res / 2;
    if (rings == 0) return 0;
    float dt = 1.0f / (float)res, t = dt;
    int rr = res - 2, n = 0;
    for (int i = 0; i < rings; ++i, rr -= 2, t += dt) {
        if (rr == 0) {
            put_uv(o, at + n++, 0.5f, 0.5f);
        } else if (rr == 1) {
            for (int e = 0; e < p->N; ++e) {
                float a[2];
                param_vertex(p, e, a);
                put_uv(o, at + n++, a[0] + t, a[1] + t);
            }
            if (p->N != 3) put_uv(o, at + n++, 0.5f, 0.5f);
        } else {
            for (int e = 0; e < p->N; ++e) n += qsub_edge(p, e, rr, 1, 0, t, dt, o, at + n);
        }
    }
    return n;
}

static int qsub_center(int N, int c0, Facets o, int at) {
    return (N == 3) ? tri3(o, at, c0, c0 + 1, c0 + 2) : fan(o, at, N, c0);
}

/* qsub::getInteriorRingFacets (tessellation.cpp:1831-1880) */
static int qsub_ring(int N, int res, int c0, int tri, Facets o, int at) {
    if (res < 1) return 0;
    if (res == 1) return qsub_center(N, c0, o, at);
    int inRes = res - 2, inner0 = c0 + N * res, n = 0;
    Strip s;
    memset(&s, 0, sizeof s);
    s.quads = 1, s.triangulate = tri, s.nOuter = res, s.nInner = inRes;
    for (int e = 0; e < N; ++e) {
        s.oFirst = c0 + e * res;
        s.iFirst = inner0 + e * inRes;
        s.oPrev = (e ? s.oFirst : inner0) - 1;
        if (e < N - 1) {
            s.oLast = s.oFirst + res;
            s.iLast = s.iFirst + inRes;
        } else {
            s.oLast = c0;
            s.iLast = inner0;
        }
        n += strip_quads(&s, o, at + n);
    }
    return n;
}

/* qsub::getBoundaryRingFacets (tessellation.cpp:1883-1938) */
static int qsub_boundary_ring(int N, const int *outer, int res, int nB, int tri, Facets o,
                              int at) {
    int n = 0;
    Strip s;
    memset(&s, 0, sizeof s);
    s.quads = 1, s.triangulate = tri, s.nInner = res - 2 > 0 ? res - 2 : 0;
    for (int e = 0; e < N; ++e) {
        s.nOuter = outer[e];
        if (e) {
            s.oFirst = s.oLast, s.oPrev = s.oFirst - 1, s.iFirst = s.iLast;
        } else {
            s.oFirst = 0, s.oPrev = nB - 1, s.iFirst = nB;
        }
        if (e < N - 1) {
            s.oLast = s.oFirst + s.nOuter;
            s.iLast = s.iFirst + s.nInner;
        } else {
            s.oLast = 0;
            s.iLast = nB;
        }
        if (outer[e] == res && res > 1) {
            s.splitFirst = outer[(e - 1 + N) % N] != res;
            s.splitLast = outer[(e + 1) % N] != res;
            n += strip_quads(&s, o, at + n);
        } else {
            s.splitFirst = s.splitLast = 1;
            n += strip_general(&s, o, at + n);
        }
    }
    return n;
}

/* ---- Tessellation (tessellation.cpp:1989-2427) -------------------------------------------- */

typedef struct {
    Param p;
    int *outer;
    int inner[2];
    int uniform, triangulate, facetSize;
    int nBoundary, nInterior, nFacets;
    int single, fanOnly, splitQuad, segmented;
} Tess;

/* quad::CountNonUniformFacets (tessellation.cpp:829-885) */
static int quad_nonuniform_count(const int *outer, const int *inner, int tri) {
    int ur = inner[0], vr = inner[1], uIn = ur - 2, vIn = vr - 2;
    int n = uIn * vIn;
    if (tri) return 2 * n + 2 * (uIn + vIn) + outer[0] + outer[1] + outer[2] + outer[3];
    int uni[4] = {outer[0] == ur, outer[1] == vr, outer[2] == ur, outer[3] == vr};
    for (int e = 0; e < 4; ++e) {
        int in = (e & 1) ? vIn : uIn;
        if (uni[e]) {
            int nextUniformCorner = uni[(e + 1) & 3] && uni[e];
            n += in + 1 + !nextUniformCorner;
        } else {
            int f = outer[e] > in ? outer[e] : in;
            if ((f & 1) == 0) f += (outer[e] & 1) || (in & 1);
            n += f;
        }
    }
    return n;
}

static int qsub_uniform_coords(int N, int res) {
    int H = res / 2;
    return (res & 1) ? (H + 1) * (H + 1) * N + ((N == 3) ? 0 : 1) : H * (H + 1) * N + 1;
}

static int qsub_uniform_facets(int N, int res, int tri) {
    int H = res / 2, odd = res & 1;
    int quads = (H + odd) * H * N;
    return (quads << tri) + (odd ? ((N == 3) ? 1 : N) : 0);
}

static int tess_init(Tess *t, int regFaceSize, int N, int numRates, const int *rates, int facetSize,
                     int preserveQuads) {
    memset(t, 0, sizeof *t);
    if (!param_init(&t->p, regFaceSize, N) || numRates < 1) return 0;
    for (int i = 0; i < numRates; ++i)
        if (rates[i] < 1) return 0;
    t->outer = (int *)malloc(sizeof(int) * (size_t)N);
    t->facetSize = (facetSize == 4) ? 4 : 3;
    t->triangulate = (t->facetSize == 3) || !preserveQuads;

    /* Tessellation::initializeRates (tessellation.cpp:2077-2145) */
    int quadFace = (N == 4), total = 0;
#define CLAMP(x) ((x) < ORC_MAX_RATE ? (x) : ORC_MAX_RATE)
    if (numRates < N) {
        if (numRates == 2 && quadFace) {
            t->inner[0] = CLAMP(rates[0]);
            t->inner[1] = CLAMP(rates[1]);
            t->outer[0] = t->outer[2] = t->inner[0];
            t->outer[1] = t->outer[3] = t->inner[1];
            t->uniform = t->inner[0] == t->inner[1];
            total = 2 * (t->inner[0] + t->inner[1]);
        } else {
            t->inner[0] = t->inner[1] = CLAMP(rates[0]);
            for (int i = 0; i < N; ++i) t->outer[i] = t->inner[0];
            t->uniform = 1;
            total = t->inner[0] * N;
        }
    } else {
        t->uniform = 1;
        for (int i = 0; i < N; ++i) {
            t->outer[i] = CLAMP(rates[i]);
            t->uniform = t->uniform && t->outer[i] == t->outer[0];
            total += t->outer[i];
        }
        if (numRates > N) {
            t->inner[0] = CLAMP(rates[N]);
            t->inner[1] = (numRates == 6 && quadFace) ? CLAMP(rates[5]) : t->inner[0];
            t->uniform = t->uniform && t->inner[0] == t->outer[0] && t->inner[1] == t->outer[0];
        } else if (quadFace) {
            t->inner[0] = (t->outer[0] + t->outer[2]) / 2;
            t->inner[1] = (t->outer[1] + t->outer[3]) / 2;
        } else {
            t->inner[0] = t->inner[1] = total / N;
        }
    }
#undef CLAMP

    const int *in = t->inner, *out = t->outer;
    int tri = t->triangulate;
    if (t->p.kind == K_QUAD) {
        /* initializeInventoryForParamQuad (tessellation.cpp:2165-2212) */
        if (t->uniform) {
            if (in[0] > 1) {
                t->nInterior = (in[0] - 1) * (in[0] - 1);
                t->nFacets = (in[0] * in[0]) << tri;
            } else if (tri) {
                t->nFacets = 2, t->splitQuad = 1;
            } else {
                t->nFacets = 1, t->single = 1;
            }
        } else if (in[0] > 1 && in[1] > 1) {
            t->nInterior = (in[0] - 1) * (in[1] - 1);
            t->nFacets = quad_nonuniform_count(out, in, tri);
        } else if (out[0] == in[0] && in[0] == out[2] && out[1] == in[1] && in[1] == out[3]) {
            t->nFacets = (in[0] * in[1]) << tri;
            t->segmented = 1;
        } else {
            t->nInterior = 1, t->nFacets = total, t->fanOnly = 1;
        }
    } else if (t->p.kind == K_TRI) {
        /* initializeInventoryForParamTri (tessellation.cpp:2215-2239) */
        int res = in[0];
        if (t->uniform) {
            if (res > 1) {
                t->nInterior = (res - 2) * (res - 1) / 2;
                t->nFacets = res * res;
            } else {
                t->nFacets = 1, t->single = 1;
            }
        } else if (res > 2) {
            int inner = res - 3;
            t->nInterior = (res - 2) * (res - 1) / 2;
            t->nFacets = inner * inner + 3 * inner + out[0] + out[1] + out[2];
        } else {
            t->nInterior = 1, t->nFacets = total, t->fanOnly = 1;
        }
    } else {
        /* initializeInventoryForParamQPoly (tessellation.cpp:2242-2272) */
        int res = in[0];
        if (t->uniform) {
            if (res > 1) {
                t->nInterior = qsub_uniform_coords(N, res - 2);
                t->nFacets = qsub_uniform_facets(N, res, tri);
            } else if (N == 3) {
                t->nFacets = 1, t->single = 1;
            } else {
                t->nInterior = 1, t->nFacets = N, t->fanOnly = 1;
            }
        } else if (res > 1) {
            /* qsub::CountNonUniformFacets (tessellation.cpp:1628-1662) */
            int inner = res - 2, n = inner ? qsub_uniform_facets(N, inner, tri) : 0;
            for (int i = 0; i < N; ++i) {
                if (tri) {
                    n += inner + out[i];
                } else if (out[i] == res) {
                    n += inner + 1 + (res != out[(i + 1) % N]);
                } else {
                    int f = inner > out[i] ? inner : out[i];
                    if ((f & 1) == 0) f += (inner & 1) || (out[i] & 1);
                    n += f;
                }
            }
            t->nInterior = qsub_uniform_coords(N, res - 2);
            t->nFacets = n;
        } else {
            t->nInterior = 1, t->nFacets = total, t->fanOnly = 1;
        }
    }
    t->nBoundary = total;
    return 1;
}

static int tess_coords(const Tess *t, Coords o) {
    int n;
    if (t->p.kind == K_QUAD) n = quad_boundary_coords(t->outer, o);
    else if (t->p.kind == K_TRI) n = tri_boundary_coords(t->outer, o);
    else n = qsub_boundary_coords(&t->p, t->outer, o);
    if (t->nInterior == 0) return n;
    if (t->nInterior == 1) {
        float c = (t->p.kind == K_TRI) ? 1.0f / 3.0f : 0.5f;
        put_uv(o, n, c, c);
        return n + 1;
    }
    if (t->p.kind == K_QUAD) return n + quad_interior_coords(t->inner, o, n);
    if (t->p.kind == K_TRI) return n + tri_interior_coords(t->inner[0], o, n);
    return n + qsub_interior_coords(&t->p, t->inner[0], o, n);
}

/* Tessellation::GetFacets (tessellation.cpp:2370-2426) */
static int tess_facets(const Tess *t, Facets o) {
    int N = t->p.N, tri = t->triangulate;
    if (t->single) return (N == 3) ? tri3(o, 0, 0, 1, 2) : quad4(o, 0, 0, 1, 2, 3, 0);
    if (t->fanOnly) return fan(o, 0, t->nFacets, 0);
    if (t->splitQuad) return quad4(o, 0, 0, 1, 2, 3, tri);

    int n = 0;
    if (t->p.kind == K_QUAD) {
        if (t->uniform) {
            int c0 = 0;
            for (int res = t->inner[0], ring = 0; ring < (t->inner[0] + 1) / 2; ++ring, res -= 2) {
                n += quad_ring(res, res, c0, tri, o, n);
                c0 += 4 * res;
            }
        } else if (t->segmented) {
            n = quad_single_strip(t->inner[0], t->inner[1], 0, tri, o, 0);
        } else {
            int ur = t->inner[0], vr = t->inner[1];
            n = quad_boundary_ring(t->outer, ur, vr, t->nBoundary, tri, o, 0);
            int rings = ((ur < vr ? ur : vr) + 1) / 2, c0 = t->nBoundary;
            for (int ring = 1; ring < rings; ++ring) {
                ur = ur - 2 > 0 ? ur - 2 : 0;
                vr = vr - 2 > 0 ? vr - 2 : 0;
                n += quad_ring(ur, vr, c0, tri, o, n);
                c0 += 2 * (ur + vr);
            }
        }
    } else if (t->p.kind == K_TRI) {
        int res = t->inner[0];
        if (t->uniform) {
            int c0 = 0, rings = 1 + res / 3;
            for (int ring = 0; ring < rings; ++ring, res -= 3) {
                n += tri_ring(res, c0, o, n);
                c0 += 3 * res;
            }
        } else {
            n = tri_boundary_ring(t->outer, res, t->nBoundary, o, 0);
            int rings = 1 + res / 3, c0 = t->nBoundary;
            for (int ring = 1; ring < rings; ++ring) {
                res -= 3;
                n += tri_ring(res, c0, o, n);
                c0 += 3 * res;
            }
        }
    } else {
        int res = t->inner[0];
        if (t->uniform) {
            if (res == 1) return qsub_center(N, 0, o, 0);
            int c0 = 0, rings = (res + 1) / 2;
            for (int ring = 0; ring < rings; ++ring, res -= 2) {
                n += qsub_ring(N, res, c0, tri, o, n);
                c0 += N * res;
            }
        } else {
            n = qsub_boundary_ring(N, t->outer, res, t->nBoundary, tri, o, 0);
            int rings = (res + 1) / 2, c0 = t->nBoundary;
            for (int ring = 1; ring < rings; ++ring) {
                res = res - 2 > 0 ? res - 2 : 0;
                n += qsub_ring(N, res, c0, tri, o, n);
                c0 += N * res;
            }
        }
    }
    return n;
}

int orc_tess_inventory(int regFaceSize, int N, int numRates, const int *rates, int facetSize,
                       int preserveQuads, int *counts) {
    Tess t;
    int ok = tess_init(&t, regFaceSize, N, numRates, rates, facetSize, preserveQuads);
    counts[0] = t.nBoundary + t.nInterior;
    counts[1] = t.nFacets;
    counts[2] = t.nBoundary;
    counts[3] = t.uniform;
    free(t.outer);
    return ok;
}

int orc_tess_generate(int regFaceSize, int N, int numRates, const int *rates, int facetSize,
                      int preserveQuads, float *coords, int coordStride, int *facets,
                      int facetStride) {
    Tess t;
    int ok = tess_init(&t, regFaceSize, N, numRates, rates, facetSize, preserveQuads);
    int nc = 0, nf = 0;
    if (ok) {
        Coords co = {coords, coordStride ? coordStride : 2};
        Facets fo = {facets, t.facetSize, facetStride ? facetStride : t.facetSize};
        nc = tess_coords(&t, co);
        nf = tess_facets(&t, fo);
    }
    free(t.outer);
    if (!ok) return 0;
    return (nc == t.nBoundary + t.nInterior && nf == t.nFacets) ? 1 : -1;
}

/* The batch form a mesh tessellation uses: face f gets faceSizes[f] vertices and the rates
 * rates[rateOffsets[f] .. rateOffsets[f+1]); its coords land at coordOffsets[f] and its facets
 * at facetOffsets[f], with facet indices offset by coordOffsets[f] as
 * Tessellation::TransformFacetCoordIndices(facets, commonOffset) does
 * (tessellation.cpp:2429-2447).  Offsets come from orc_tess_inventory. */
int orc_tess_mesh(int regFaceSize, int numFaces, const int *faceSizes, const int *rateOffsets,
                  const int *rates, int facetSize, int preserveQuads, const long *coordOffsets,
                  const long *facetOffsets, float *coords, int *facets, int threads) {
    int bad = 0;
    int fs = (facetSize == 4) ? 4 : 3;
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads) reduction(+ : bad)
    for (int f = 0; f < numFaces; ++f) {
        int nr = rateOffsets[f + 1] - rateOffsets[f];
        float *c = coords + 2 * coordOffsets[f];
        int *F = facets + (long)fs * facetOffsets[f];
        int r = orc_tess_generate(regFaceSize, faceSizes[f], nr, rates + rateOffsets[f], fs,
                                  preserveQuads, c, 2, F, fs);
        if (r < 0) {
            bad++;
            continue;
        }
        if (r == 0) continue;
        int nf = (int)(facetOffsets[f + 1] - facetOffsets[f]);
        int off = (int)coordOffsets[f];
        for (int i = 0; i < nf * fs; ++i)
            if (F[i] >= 0) F[i] += off;
    }
    return bad == 0;
}

/* Every coord of a mesh tessellation located for a patch table: the ptex face
 * (ptexOffsets[f] + the sub-face of Parameterization::ConvertCoordToNormalizedSubFace) and
 * its normalized (s, t), as the reference's Bfr regression locates tessellation coords
 * (regression/bfr_evaluate/farPatchEvaluator.cpp:190-207). */
int orc_tess_locate_mesh(int regFaceSize, int numFaces, const int *faceSizes,
                         const long *coordOffsets, const long *ptexOffsets, const float *coords,
                         int *ptexFaces, float *st, int threads) {
    int bad = 0;
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads) reduction(+ : bad)
    for (int f = 0; f < numFaces; ++f) {
        long c0 = coordOffsets[f];
        int n = (int)(coordOffsets[f + 1] - c0);
        if (n == 0) continue;
        if (!orc_param_to_subface(regFaceSize, faceSizes[f], n, coords + 2 * c0,
                                  ptexFaces + c0, st + 2 * c0)) {
            bad++;
            continue;
        }
        for (int i = 0; i < n; ++i) ptexFaces[c0 + i] += (int)ptexOffsets[f];
    }
    return bad == 0;
}

/* Shared (watertight) points of a mesh tessellation: the bookkeeping of the reference's
 * tessellation with shared vertex and edge points (tutorials/bfr/tutorial_2_2/
 * bfr_tutorial_2_2.cpp:244-430), with per-face rates.  Faces in order, faces without coords
 * skipped.  Walking the corners of a face, the first face to reach a mesh vertex makes its
 * vertex coord a new point; the first face to reach a mesh edge makes the rate - 1 coords
 * inside the edge new points, numbered in its own direction along the edge; later faces reuse
 * those points, reversed where they run the edge from its other end (the tutorial reverses
 * for every later face, which is the same on the manifold, consistently oriented meshes it
 * accepts).  All interior coords of a face are new.  Points are numbered in the order made.
 * Each facet index (a coord of its face: mesh-wide when meshIndices, else face-local) becomes
 * the index of its point, as Tessellation::TransformFacetCoordIndices(facets,
 * boundaryIndices, interiorOffset) maps it (tessellation.cpp:2449-2464); -1 stays -1.
 * pointOffsets[f] = the first point face f made (numFaces + 1 entries); pointSources[p] = the
 * mesh coord the point was made from.  Returns the number of points, -1 - f when face f runs
 * an edge at another rate than the face that made the edge's points, or -1 - numFaces for a
 * vertex or edge index out of range. */
long orc_tess_share(int regFaceSize, int numFaces, const int *faceSizes, const int *faceVerts,
                    const int *faceEdges, int numVertices, int numEdges, const int *rateOffsets,
                    const int *rates, int facetSize, int preserveQuads, const long *coordOffsets,
                    const long *facetOffsets, int facetStride, int meshIndices, int *facets,
                    long *pointOffsets, long *pointSources) {
    int fs = (facetSize == 4) ? 4 : 3;
    int fst = facetStride ? facetStride : fs;
    long *vpt = (long *)malloc(sizeof(long) * (size_t)(numVertices > 0 ? numVertices : 1));
    long *efirst = (long *)malloc(sizeof(long) * (size_t)(numEdges > 0 ? numEdges : 1));
    int *ecount = (int *)malloc(sizeof(int) * (size_t)(numEdges > 0 ? numEdges : 1));
    int *estart = (int *)malloc(sizeof(int) * (size_t)(numEdges > 0 ? numEdges : 1));
    for (int v = 0; v < numVertices; ++v) vpt[v] = -1;
    for (int e = 0; e < numEdges; ++e) efirst[e] = -1;
    long next = 0, corner = 0, result = 0;
    long *bidx = NULL;
    size_t bcap = 0;
    for (int f = 0; f < numFaces && result == 0; ++f) {
        int N = faceSizes[f];
        long c0 = coordOffsets[f], nc = coordOffsets[f + 1] - c0;
        pointOffsets[f] = next;
        const int *fv = faceVerts + corner, *fe = faceEdges + corner;
        corner += N;
        if (nc == 0) continue;
        Tess t;
        tess_init(&t, regFaceSize, N, rateOffsets[f + 1] - rateOffsets[f], rates + rateOffsets[f],
                  fs, preserveQuads);
        int nb = t.nBoundary;
        if ((size_t)nb > bcap) {
            bcap = (size_t)nb;
            bidx = (long *)realloc(bidx, sizeof(long) * bcap);
        }
        int k = 0;
        for (int i = 0; i < N && result == 0; ++i) {
            int v = fv[i], e = fe[i], n = t.outer[i] - 1;
            if (v < 0 || v >= numVertices || e < 0 || e >= numEdges) {
                result = -1 - (long)numFaces;
                break;
            }
            if (vpt[v] < 0) {
                vpt[v] = next;
                pointSources[next++] = c0 + k;
            }
            bidx[k++] = vpt[v];
            if (efirst[e] < 0) {
                efirst[e] = next, ecount[e] = n, estart[e] = v;
                for (int j = 0; j < n; ++j) {
                    pointSources[next] = c0 + k;
                    bidx[k++] = next++;
                }
            } else if (ecount[e] != n) {
                result = -1 - (long)f;
            } else {
                int rev = estart[e] != v;
                for (int j = 0; j < n; ++j) bidx[k++] = efirst[e] + (rev ? n - 1 - j : j);
            }
        }
        if (result == 0) {
            long interiorOffset = next - nb;
            for (long j = nb; j < nc; ++j) pointSources[next++] = c0 + j;
            long nfac = facetOffsets[f + 1] - facetOffsets[f];
            int *F = facets + (long)fst * facetOffsets[f];
            for (long q = 0; q < nfac; ++q)
                for (int j = 0; j < fs; ++j) {
                    int *x = F + q * fst + j;
                    if (*x < 0) continue;
                    long local = *x - (meshIndices ? c0 : 0);
                    *x = (int)(local < nb ? bidx[local] : local + interiorOffset);
                }
        }
        free(t.outer);
    }
    if (result == 0) {
        pointOffsets[numFaces] = next;
        result = next;
    }
    free(bidx);
    free(vpt);
    free(efirst);
    free(ecount);
    free(estart);
    return result;
}
