// Bfr::Tessellation patterns (bfr/tessellation.h, bfr/tessellation.cpp) for one face:
// inventory (how many coords and facets), the (u,v) coords and the facets.
//
// Functions are __host__ __device__: the host sizes the shared uniform-rate patterns, device
// threads generate patterns.  Every float operation is an explicitly rounded one (no fused
// multiply-add), so the coords round exactly as the reference's float instantiation does; the
// running parameter of each iso-line is accumulated, as the reference accumulates it.
//
// Construction order is the reference's: boundary coords edge by edge from vertex 0, then
// interior rings outside in; facets ring by ring, each ring strip by strip (one strip per
// edge between two concentric rings of coords).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace gb300 {
namespace tess {

enum { kQuad = 0, kTri = 1, kQsub = 2 };
enum { kGeneral = 0, kSingle = 1, kFan = 2, kSplitQuad = 3, kSegmented = 4 };

// Tessellation rates are clamped to a short (tessellation.cpp:2091); faces are at most
// Far::VALENCE_LIMIT vertices (bfr/limits.h:43).
constexpr int kMaxRate = 32767;
constexpr int kMaxFaceSize = 65535;

#define GB_HD __host__ __device__ __forceinline__

GB_HD float fadd(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
GB_HD float fsub(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
GB_HD float fmul(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
GB_HD float frcp(int r) {
#ifdef __CUDA_ARCH__
    return __fdiv_rn(1.0f, (float)r);
#else
    return 1.0f / (float)r;
#endif
}
GB_HD int imin(int a, int b) { return a < b ? a : b; }
GB_HD int imax(int a, int b) { return a > b ? a : b; }

// Where a face's coords and facets go: coords as (u,v) pairs `cs` floats apart, facets as
// `fsz` indices `fst` ints apart, each index offset by `base` (the face's first coord in a
// mesh-wide numbering, Tessellation::TransformFacetCoordIndices(facets, commonOffset),
// tessellation.cpp:2429-2447; -1 pads stay -1).
struct Sink {
    float *c;
    int cs;
    int *f;
    int fsz, fst;
    int base = 0;
    bool pairs = false;  // cs == 2 and c 8-byte aligned: a coord is one 8-byte store
    GB_HD void uv(int i, float u, float v) const {
#ifdef __CUDA_ARCH__
        if (pairs) {
            *reinterpret_cast<float2 *>(c + 2 * (int64_t)i) = make_float2(u, v);
            return;
        }
#endif
        c[(int64_t)i * cs] = u;
        c[(int64_t)i * cs + 1] = v;
    }
    GB_HD int *facet(int i) const { return f + (int64_t)i * fst; }
    // Facet::Set of three indices (tessellation.cpp:114-118): a 4-tuple's last slot is -1
    GB_HD int tri(int i, int a, int b, int c2) const {
        int *t = facet(i);
        if (fsz == 4) t[3] = -1;
        t[0] = a + base, t[1] = b + base, t[2] = c2 + base;
        return 1;
    }
    // appendQuad (tessellation.cpp:200-219): sign 0 keeps the quad, > 0 splits it along
    // a-c, < 0 along b-d
    GB_HD int quad(int i, int a, int b, int c2, int d, int sign) const {
        if (sign == 0) {
            int *t = facet(i);
            t[0] = a + base, t[1] = b + base, t[2] = c2 + base, t[3] = d + base;
            return 1;
        }
        if (sign > 0) {
            tri(i, a, b, c2);
            tri(i + 1, c2, d, a);
        } else {
            tri(i, c2, d, b);
            tri(i + 1, a, b, d);
        }
        return 2;
    }
    // appendTriFan (tessellation.cpp:221-230)
    GB_HD int fan(int i, int size, int start) const {
        for (int k = 1; k <= size; ++k)
            tri(i + k - 1, start + k - 1, start + ((k < size) ? k : 0), start + size);
        return size;
    }
    // iso-lines with an accumulated parameter (tessellation.cpp:160-188)
    GB_HD int run_u(int i, int n, float u, float v, float du) const {
        for (int k = 0; k < n; ++k, u = fadd(u, du)) uv(i + k, u, v);
        return n;
    }
    GB_HD int run_v(int i, int n, float u, float v, float dv) const {
        for (int k = 0; k < n; ++k, v = fadd(v, dv)) uv(i + k, u, v);
        return n;
    }
    GB_HD int run_uv(int i, int n, float u, float v, float du, float dv) const {
        for (int k = 0; k < n; ++k, u = fadd(u, du), v = fadd(v, dv)) uv(i + k, u, v);
        return n;
    }
};

// A strip of facets between an outer and an inner ring (FacetStrip, tessellation.cpp:233-268).
struct Strip {
    int quads = 0, triangulate = 0, reversed = 0;
    int exclFirst = 0, splitFirst = 0, splitLast = 0, inclLast = 0;
    int nOuter = 0, nInner = 0;
    int oFirst = 0, oLast = 0, oPrev = 0, iFirst = 0, iLast = 0;

    // connectUniformQuads (tessellation.cpp:283-350)
    GB_HD int quads_uniform(const Sink &o, int at) const {
        int n = 0;
        const int t = triangulate;
        if (splitFirst)
            n += o.tri(at + n, oFirst, oFirst + 1, iFirst);
        else if (!exclFirst)
            n += o.quad(at + n, oFirst, oFirst + 1, iFirst, oPrev, t);
        int oi = oFirst + 1, ii = iFirst;
        const int step = reversed ? -1 : 1;
        for (int k = 1; k <= nInner; ++k, ++oi, ii += step) {
            const int sign = (k > nInner / 2) ? -t : t;
            const int ij = (k < nInner) ? ii + step : iLast;
            n += o.quad(at + n, oi, oi + 1, ij, ii, sign);
        }
        if (splitLast)
            n += o.tri(at + n, oi, oLast, iLast);
        else if (inclLast)
            n += o.quad(at + n, oi, oLast, oLast + 1, iLast, -t);
        return n;
    }

    // connectUniformTris (tessellation.cpp:352-420)
    GB_HD int tris_uniform(const Sink &o, int at) const {
        int n = 0;
        const int o0 = oFirst, i0 = iFirst;
        if (splitFirst) {
            n += o.tri(at + n, o0, o0 + 1, i0);
        } else {
            n += o.tri(at + n, o0, o0 + 1, oPrev);
            n += o.tri(at + n, i0, oPrev, o0 + 1);
        }
        n += o.tri(at + n, o0 + 1, o0 + 2, i0);
        int oi = o0 + 2, ii = i0;
        for (int k = 1; k <= nInner; ++k, ++ii, ++oi) {
            const int ij = (k < nInner) ? ii + 1 : iLast;
            n += o.tri(at + n, ij, ii, oi);
            n += o.tri(at + n, oi, oi + 1, ij);
        }
        if (splitLast) n += o.tri(at + n, oi, oLast, iLast);
        return n;
    }

    // connectNonUniformFacets (tessellation.cpp:422-633): both rings are parameterised over
    // [0, M*N]; each facet takes the diagonal spanning the shorter interval around a symmetric
    // middle facet, and with quads kept a facet past the middle mirrors its counterpart's kind.
    GB_HD int general(const Sink &o, int at) const {
        const int M = nInner + (quads ? 2 : 3), N = nOuter;
        const int dtO = M, dtI = N;
        const int dtMin = imin(dtI, dtO), dtMax = imax(dtI, dtO);
        const int slopeMax = ((dtMax / 2) < dtMin) ? (dtMin - 1) : (dtMax / 2);
        const int tOLast = dtO * N, tOMid = tOLast / 2;
        int tIOff = 0, tILast = dtI * (M - 1);
        if (!quads) {
            tIOff = dtI / 2;
            tILast += tIOff - dtI;
        }
        const int dI = reversed ? -1 : 1;

        int tO0 = 0, cO0 = oFirst;
        int tO1 = dtO, cO1 = (N == 1) ? oLast : oFirst + 1;
        int tI0 = tIOff + dtI, cI0 = iFirst;
        int tI1 = tI0 + (nInner ? dtI : 0);
        int cI1 = (nInner == 1) ? iLast : iFirst + dI;

        const int keepQuads = quads && !triangulate;
        int total;
        if (keepQuads) {
            total = imax(nInner, nOuter);
            if ((total & 1) == 0) total += (nInner & 1) || (nOuter & 1);
        } else {
            total = nInner + nOuter;
        }
        const int lead = total / 2, mid = total & 1;
        const int midFacet = mid ? lead : -1;
        const int midQuad = keepQuads && (nOuter & 1) && (nInner & 1);

        for (int k = 0; k < total; ++k) {
            int triO = 0, triI = 0, q = 0;
            if (k == midFacet) {
                if (midQuad) q = 1;
                else if (nOuter & 1) triO = 1;
                else triI = 1;
            } else if (tI1 == tI0) {
                triO = 1;
            } else if (tO1 == tO0) {
                triI = 1;
            } else {
                if (keepQuads) {
                    if (k >= lead) {
                        const int mirror = lead - 1 - (k - lead - mid);
                        q = o.facet(at + mirror)[3] >= 0;
                    } else if (tI1 > tOMid || tO1 > tOMid) {
                        q = 0;
                    } else {
                        const int d = tO1 - tI1;
                        q = (d < 0 ? -d : d) <= slopeMax;
                    }
                }
                if (!q) {
                    const int toOuter = tO1 - tI0, toInner = tI1 - tO0;
                    const int useOuter = (toOuter == toInner) ? (tO1 > tOMid) : (toOuter < toInner);
                    if (useOuter) triO = 1;
                    else triI = 1;
                }
            }
            if (triO) o.tri(at + k, cO0, cO1, cI0);
            else if (triI) o.tri(at + k, cI1, cI0, cO0);
            else o.quad(at + k, cO0, cO1, cI1, cI0, 0);

            if (triO || q) {
                tO0 = tO1, cO0 = cO1;
                tO1 += dtO, cO1 += 1;
                if (tO1 >= tOLast) tO1 = tOLast, cO1 = oLast;
            }
            if (triI || q) {
                tI0 = tI1, cI0 = cI1;
                tI1 += dtI, cI1 += dI;
                if (tI1 >= tILast) tI1 = tILast, cI1 = iLast;
            }
        }
        return total;
    }
};

// Coords of a uniform quad-sub-face polygon at rate `res` (qsub::countUniformCoords,
// tessellation.cpp:1665-1670) and its facets (qsub::CountUniformFacets, :1615-1625).
GB_HD int qsub_uniform_coords(int N, int res) {
    const int H = res / 2;
    return (res & 1) ? (H + 1) * (H + 1) * N + ((N == 3) ? 0 : 1) : H * (H + 1) * N + 1;
}
GB_HD int qsub_uniform_facets(int N, int res, int tri) {
    const int H = res / 2, odd = res & 1;
    return (((H + odd) * H * N) << tri) + (odd ? ((N == 3) ? 1 : N) : 0);
}

// One face's tessellation: its parameterization (bfr/parameterization.cpp:40-66), rates
// (Tessellation::initializeRates, tessellation.cpp:2077-2145) and inventory
// (initializeInventoryForParam*, :2165-2272).  `rates` are the numRates rates given for the
// face, as Tessellation(param, numRates, rates, options) takes them.
struct Face {
    int kind = 0, N = 0, udim = 0;
    int nr = 0;
    const int *rates = nullptr;  // the given rates, or null for the one rate `single`
    int single = 0;
    int o0 = 0, o1 = 0, o2 = 0, o3 = 0;
    int in0 = 0, in1 = 0;
    int uniform = 0, triangulate = 1, fs = 3;
    int nBoundary = 0, nInterior = 0, nFacets = 0;
    int mode = kGeneral;
    int valid = 0;

    // rate of edge e (the edge from vertex e to e + 1); the edge rates of triangles and quads
    // are held in registers (o0..o3), larger faces read theirs from the given rates
    GB_HD int outer(int e) const {
        if (nr < N) return (nr == 2 && N == 4) ? ((e & 1) ? in1 : in0) : in0;
        if (N <= 4) return e == 0 ? o0 : e == 1 ? o1 : e == 2 ? o2 : o3;
        return imin(rates[e], kMaxRate);
    }
    GB_HD int given(int i) const { return rates ? rates[i] : single; }

    GB_HD void vertex(int v, float uv[2]) const {
        if (kind == kQuad) {
            uv[0] = (float)(v && v < 3);
            uv[1] = (float)(v > 1);
        } else if (kind == kTri) {
            uv[0] = (float)(v == 1);
            uv[1] = (float)(v == 2);
        } else {
            uv[0] = (float)(v % udim);
            uv[1] = (float)(v / udim);
        }
    }

    // One rate: givenRates may be null and the rate is singleRate (no pointer into the
    // caller's registers, which would put them in local memory on the device).
    GB_HD bool init(int regFaceSize, int faceSize, int numRates, const int *givenRates,
                    int facetSize, int preserveQuads, int singleRate = 0) {
        N = faceSize;
        valid = 0;
        nBoundary = nInterior = nFacets = 0;
        kind = (regFaceSize == 4) ? kQuad : kTri;
        udim = 0;
        if (N != regFaceSize) {
            if (N < 3 || N > kMaxFaceSize || regFaceSize == 3) return false;
            kind = kQsub;
            udim = (N < 10) ? 2 + (N > 4) : 1 + (int)sqrtf((float)(N - 1));
        }
        if (numRates < 1 || (!givenRates && numRates != 1)) return false;
        nr = numRates;
        rates = givenRates;
        single = singleRate;
        for (int i = 0; i < numRates; ++i)
            if (given(i) < 1) return false;
        fs = (facetSize == 4) ? 4 : 3;
        triangulate = (fs == 3) || !preserveQuads;

        const int quadFace = (N == 4);
        int total = 0;
        if (nr < N) {
            if (nr == 2 && quadFace) {
                in0 = imin(given(0), kMaxRate);
                in1 = imin(given(1), kMaxRate);
                uniform = in0 == in1;
                total = 2 * (in0 + in1);
            } else {
                in0 = in1 = imin(given(0), kMaxRate);
                uniform = 1;
                total = in0 * N;
            }
        } else {
            if (N <= 4) {
                o0 = imin(given(0), kMaxRate);
                o1 = imin(given(1), kMaxRate);
                o2 = imin(given(2), kMaxRate);
                o3 = N == 4 ? imin(given(3), kMaxRate) : 0;
            }
            uniform = 1;
            const int r0 = imin(given(0), kMaxRate);
            for (int i = 0; i < N; ++i) {
                const int oi = imin(given(i), kMaxRate);
                uniform = uniform && oi == r0;
                total += oi;
            }
            if (nr > N) {
                in0 = imin(given(N), kMaxRate);
                in1 = (nr == 6 && quadFace) ? imin(given(5), kMaxRate) : in0;
                uniform = uniform && in0 == r0 && in1 == r0;
            } else if (quadFace) {
                in0 = (outer(0) + outer(2)) / 2;
                in1 = (outer(1) + outer(3)) / 2;
            } else {
                in0 = in1 = total / N;
            }
        }
        nBoundary = total;
        mode = kGeneral;
        const int tri = triangulate;
        if (kind == kQuad) {
            if (uniform) {
                if (in0 > 1) {
                    nInterior = (in0 - 1) * (in0 - 1);
                    nFacets = (in0 * in0) << tri;
                } else if (tri) {
                    nFacets = 2, mode = kSplitQuad;
                } else {
                    nFacets = 1, mode = kSingle;
                }
            } else if (in0 > 1 && in1 > 1) {
                nInterior = (in0 - 1) * (in1 - 1);
                nFacets = quad_nonuniform_facets();
            } else if (outer(0) == in0 && in0 == outer(2) && outer(1) == in1 && in1 == outer(3)) {
                nFacets = (in0 * in1) << tri;
                mode = kSegmented;
            } else {
                nInterior = 1, nFacets = total, mode = kFan;
            }
        } else if (kind == kTri) {
            const int res = in0;
            if (uniform) {
                if (res > 1) {
                    nInterior = (res - 2) * (res - 1) / 2;
                    nFacets = res * res;
                } else {
                    nFacets = 1, mode = kSingle;
                }
            } else if (res > 2) {
                const int inner = res - 3;
                nInterior = (res - 2) * (res - 1) / 2;
                nFacets = inner * inner + 3 * inner + outer(0) + outer(1) + outer(2);
            } else {
                nInterior = 1, nFacets = total, mode = kFan;
            }
        } else {
            const int res = in0;
            if (uniform) {
                if (res > 1) {
                    nInterior = qsub_uniform_coords(N, res - 2);
                    nFacets = qsub_uniform_facets(N, res, tri);
                } else if (N == 3) {
                    nFacets = 1, mode = kSingle;
                } else {
                    nInterior = 1, nFacets = N, mode = kFan;
                }
            } else if (res > 1) {
                // qsub::CountNonUniformFacets (tessellation.cpp:1628-1662)
                const int inner = res - 2;
                int n = inner ? qsub_uniform_facets(N, inner, tri) : 0;
                for (int i = 0; i < N; ++i) {
                    const int oi = outer(i);
                    if (tri) {
                        n += inner + oi;
                    } else if (oi == res) {
                        n += inner + 1 + (res != outer((i + 1) % N));
                    } else {
                        int f = imax(inner, oi);
                        if ((f & 1) == 0) f += (inner & 1) || (oi & 1);
                        n += f;
                    }
                }
                nInterior = qsub_uniform_coords(N, res - 2);
                nFacets = n;
            } else {
                nInterior = 1, nFacets = total, mode = kFan;
            }
        }
        valid = 1;
        return true;
    }

    // an edge whose rate equals the inner rate along it keeps the uniform strip
    // (tessellation.cpp:1124-1135)
    GB_HD bool quad_uniform_edge(int e) const { return outer(e) == ((e & 1) ? in1 : in0); }

    // quad::CountNonUniformFacets (tessellation.cpp:829-885)
    GB_HD int quad_nonuniform_facets() const {
        const int uIn = in0 - 2, vIn = in1 - 2;
        int n = uIn * vIn;
        if (triangulate) return 2 * n + 2 * (uIn + vIn) + outer(0) + outer(1) + outer(2) + outer(3);
        for (int e = 0; e < 4; ++e) {
            const int in = (e & 1) ? vIn : uIn;
            if (quad_uniform_edge(e)) {
                n += in + 1 + !(quad_uniform_edge((e + 1) & 3) && quad_uniform_edge(e));
            } else {
                int f = imax(outer(e), in);
                if ((f & 1) == 0) f += (outer(e) & 1) || (in & 1);
                n += f;
            }
        }
        return n;
    }

    GB_HD int num_coords() const { return nBoundary + nInterior; }

    // ---- coords (Tessellation::GetCoords: boundary then interior) --------------------------

    // qsub::getRingEdgeCoords (tessellation.cpp:1689-1734): the first half of an edge runs
    // along u of sub-face `e`, the second half down v of sub-face e + 1
    GB_HD int qsub_edge(const Sink &o, int at, int e, int res, int first, float t0,
                        float dt) const {
        const int n0 = (res - 1) / 2, n1 = (res - 1) - n0;
        int n = 0;
        if (first || n0) {
            float a[2];
            vertex(e, a);
            if (first) o.uv(at + n++, fadd(a[0], t0), fadd(a[1], t0));
            if (n0) n += o.run_u(at + n, n0, fadd(fadd(a[0], t0), dt), fadd(a[1], t0), dt);
        }
        if (n1) {
            float b[2];
            vertex((e + 1) % N, b);
            const float v = fadd(b[1], (res & 1) ? fsub(0.5f, fmul(0.5f, dt)) : 0.5f);
            n += o.run_v(at + n, n1, fadd(b[0], t0), v, -dt);
        }
        return n;
    }

    template <int K>
    GB_HD int boundary_coords_k(const Sink &o) const {
        int n = 0;
        if constexpr (K == kQuad) {
            const int r0 = outer(0), r1 = outer(1), r2 = outer(2), r3 = outer(3);
            n += o.run_u(n, r0, 0.0f, 0.0f, frcp(r0));
            n += o.run_v(n, r1, 1.0f, 0.0f, frcp(r1));
            n += o.run_u(n, r2, 1.0f, 1.0f, -frcp(r2));
            n += o.run_v(n, r3, 0.0f, 1.0f, -frcp(r3));
        } else if constexpr (K == kTri) {
            const int r0 = outer(0), r1 = outer(1), r2 = outer(2);
            n += o.run_u(n, r0, 0.0f, 0.0f, frcp(r0));
            n += o.run_uv(n, r1, 1.0f, 0.0f, -frcp(r1), frcp(r1));
            n += o.run_v(n, r2, 0.0f, 1.0f, -frcp(r2));
        } else {
            for (int e = 0; e < N; ++e) {
                const int r = outer(e);
                n += qsub_edge(o, n, e, r, 1, 0.0f, frcp(r));
            }
        }
        return n;
    }

    template <int K>
    GB_HD int interior_coords_k(const Sink &o, int at) const {
        if (nInterior == 0) return 0;
        if (nInterior == 1) {
            const float c = (K == kTri) ? 1.0f / 3.0f : 0.5f;
            o.uv(at, c, c);
            return 1;
        }
        int n = 0;
        if constexpr (K == kQuad) {
            const int rings = imin(in0 / 2, in1 / 2);
            const float du = frcp(in0), dv = frcp(in1);
            float u = du, v = dv;
            int ur = in0 - 2, vr = in1 - 2;
            for (int i = 0; i < rings; ++i, ur -= 2, vr -= 2, u = fadd(u, du), v = fadd(v, dv)) {
                if (ur > 0 && vr > 0) {
                    const float u1 = fsub(1.0f, u), v1 = fsub(1.0f, v);
                    n += o.run_u(at + n, ur, u, v, du);
                    n += o.run_v(at + n, vr, u1, v, dv);
                    n += o.run_u(at + n, ur, u1, v1, -du);
                    n += o.run_v(at + n, vr, u, v1, -dv);
                } else if (ur > 0) {
                    n += o.run_u(at + n, ur + 1, u, v, du);
                } else if (vr > 0) {
                    n += o.run_v(at + n, vr + 1, u, v, dv);
                } else {
                    o.uv(at + n++, 0.5f, 0.5f);
                }
            }
        } else if constexpr (K == kTri) {
            const int rings = in0 / 3;
            const float dt = frcp(in0);
            float u = dt, v = dt;
            int rr = in0 - 3;
            for (int i = 0; i < rings; ++i, rr -= 3, u = fadd(u, dt), v = fadd(v, dt)) {
                if (rr == 0) {
                    o.uv(at + n++, 1.0f / 3.0f, 1.0f / 3.0f);
                } else {
                    const float u1 = fsub(1.0f, fmul(u, 2.0f)), v1 = fsub(1.0f, fmul(v, 2.0f));
                    n += o.run_u(at + n, rr, u, v, dt);
                    n += o.run_uv(at + n, rr, u1, v, -dt, dt);
                    n += o.run_v(at + n, rr, u, v1, -dt);
                }
            }
        } else {
            const int rings = in0 / 2;
            const float dt = frcp(in0);
            float t = dt;
            int rr = in0 - 2;
            for (int i = 0; i < rings; ++i, rr -= 2, t = fadd(t, dt)) {
                if (rr == 0) {
                    o.uv(at + n++, 0.5f, 0.5f);
                } else if (rr == 1) {
                    for (int e = 0; e < N; ++e) {
                        float a[2];
                        vertex(e, a);
                        o.uv(at + n++, fadd(a[0], t), fadd(a[1], t));
                    }
                    if (N != 3) o.uv(at + n++, 0.5f, 0.5f);
                } else {
                    for (int e = 0; e < N; ++e) n += qsub_edge(o, at + n, e, rr, 1, t, dt);
                }
            }
        }
        return n;
    }

    // Generation for a face of parameterization kind K (compiled per kind, so a kernel that
    // handles one kind carries only that kind's code); coords() / facets() dispatch on `kind`.
    template <int K>
    GB_HD int coords_k(const Sink &o) const {
        const int n = boundary_coords_k<K>(o);
        return n + interior_coords_k<K>(o, n);
    }
    GB_HD int coords(const Sink &o) const {
        return kind == kQuad ? coords_k<kQuad>(o) : kind == kTri ? coords_k<kTri>(o)
                                                                 : coords_k<kQsub>(o);
    }

    // ---- facets (Tessellation::GetFacets, tessellation.cpp:2370-2426) ----------------------

    // quad::getSingleStripFacets (tessellation.cpp:998-1034)
    GB_HD static int quad_single_strip(int ur, int vr, int c0, int tri, const Sink &o, int at) {
        Strip s;
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
        return s.quads_uniform(o, at);
    }

    // quad::getInteriorRingFacets (tessellation.cpp:1037-1118)
    GB_HD static int quad_ring(int ur, int vr, int c0, int tri, const Sink &o, int at) {
        const int cells = ur * vr;
        if (cells == 0) return 0;
        if (cells == 1) return o.quad(at, c0, c0 + 1, c0 + 2, c0 + 3, tri);
        if (ur == 1 || vr == 1) return quad_single_strip(ur, vr, c0, tri, o, at);
        const int uIn = ur - 2, vIn = vr - 2;
        const int outer0 = c0, inner0 = c0 + 2 * (ur + vr);
        int n = 0;
        Strip s;
        s.quads = 1, s.triangulate = tri;
        s.nOuter = ur, s.oFirst = outer0, s.oPrev = inner0 - 1, s.oLast = outer0 + ur;
        s.nInner = uIn, s.iFirst = inner0, s.iLast = inner0 + uIn;
        n += s.quads_uniform(o, at + n);
        s.nOuter = vr, s.oFirst += ur, s.oPrev = s.oFirst - 1, s.oLast = s.oFirst + vr;
        s.nInner = vIn, s.reversed = 0, s.iFirst = s.iLast, s.iLast += vIn;
        n += s.quads_uniform(o, at + n);
        s.nOuter = ur, s.oFirst += vr, s.oPrev = s.oFirst - 1, s.oLast = s.oFirst + ur;
        s.nInner = uIn, s.reversed = (vIn == 0), s.iFirst = s.iLast;
        s.iLast += uIn * (s.reversed ? -1 : 1);
        n += s.quads_uniform(o, at + n);
        s.nOuter = vr, s.oFirst += ur, s.oPrev = s.oFirst - 1, s.oLast = outer0;
        s.nInner = vIn, s.reversed = (uIn == 0), s.iFirst = s.iLast, s.iLast = inner0;
        n += s.quads_uniform(o, at + n);
        return n;
    }

    // quad::getBoundaryRingFacets (tessellation.cpp:1121-1225)
    GB_HD int quad_boundary_ring(const Sink &o) const {
        const int ur = in0, vr = in1, nB = nBoundary, tri = triangulate;
        const int uIn = ur - 2, vIn = vr - 2;
        int n = 0;
        Strip s;
        s.quads = 1, s.triangulate = tri;
        for (int e = 0; e < 4; ++e) {
            const int inner = (e & 1) ? vIn : uIn;
            s.nOuter = outer(e);
            s.nInner = inner;
            if (e == 0) {
                s.oFirst = 0, s.oPrev = nB - 1, s.oLast = outer(0);
                s.reversed = 0, s.iFirst = nB, s.iLast = nB + uIn;
            } else {
                s.oFirst = s.oLast, s.oPrev = s.oFirst - 1;
                s.oLast = (e == 3) ? 0 : s.oLast + outer(e);
                s.reversed = (e == 2) ? (vIn == 0) : (e == 3) ? (uIn == 0) : 0;
                s.iFirst = s.iLast;
                s.iLast = (e == 3) ? nB : s.iLast + inner * (s.reversed ? -1 : 1);
            }
            if (quad_uniform_edge(e)) {
                // a corner keeps its quad when both edges at it are uniform
                s.splitFirst = !quad_uniform_edge((e + 3) & 3);
                s.splitLast = !quad_uniform_edge((e + 1) & 3);
                n += s.quads_uniform(o, n);
            } else {
                s.splitFirst = s.splitLast = 1;
                n += s.general(o, n);
            }
        }
        return n;
    }

    // tri::getInteriorRingFacets (tessellation.cpp:1425-1481)
    GB_HD static int tri_ring(int res, int c0, const Sink &o, int at) {
        if (res < 1) return 0;
        if (res == 1) return o.tri(at, c0, c0 + 1, c0 + 2);
        if (res == 2) {
            o.tri(at + 0, c0 + 0, c0 + 1, c0 + 5);
            o.tri(at + 1, c0 + 2, c0 + 3, c0 + 1);
            o.tri(at + 2, c0 + 4, c0 + 5, c0 + 3);
            o.tri(at + 3, c0 + 1, c0 + 3, c0 + 5);
            return 4;
        }
        const int inner = res - 3, outer0 = c0, inner0 = c0 + 3 * res;
        int n = 0;
        Strip s;
        s.nInner = inner, s.nOuter = res;
        s.oFirst = outer0, s.oLast = outer0 + res, s.oPrev = inner0 - 1;
        s.iFirst = inner0, s.iLast = inner0 + inner;
        n += s.tris_uniform(o, at + n);
        s.oFirst += res, s.oLast += res, s.oPrev = s.oFirst - 1;
        s.iFirst += inner, s.iLast += inner;
        n += s.tris_uniform(o, at + n);
        s.oFirst += res, s.oLast = outer0, s.oPrev = s.oFirst - 1;
        s.iFirst += inner, s.iLast = inner0;
        n += s.tris_uniform(o, at + n);
        return n;
    }

    // tri::getBoundaryRingFacets (tessellation.cpp:1484-1561)
    GB_HD int tri_boundary_ring(const Sink &o) const {
        const int res = in0, nB = nBoundary;
        const int inner = res - 3;
        int n = 0;
        Strip s;
        s.nInner = inner;
        for (int e = 0; e < 3; ++e) {
            s.nOuter = outer(e);
            if (e == 0) {
                s.oFirst = 0, s.oLast = outer(0), s.oPrev = nB - 1;
                s.iFirst = nB, s.iLast = nB + inner;
            } else {
                s.oFirst = s.oLast;
                s.oLast = (e == 2) ? 0 : s.oLast + outer(e);
                s.oPrev = s.oFirst - 1;
                s.iFirst = s.iLast;
                s.iLast = (e == 2) ? nB : s.iLast + inner;
            }
            if (outer(e) == res) {
                s.splitFirst = outer((e + 2) % 3) != res;
                s.splitLast = outer((e + 1) % 3) != res;
                n += s.tris_uniform(o, n);
            } else {
                s.splitFirst = s.splitLast = 1;
                n += s.general(o, n);
            }
        }
        return n;
    }

    GB_HD int qsub_center(int c0, const Sink &o, int at) const {
        return (N == 3) ? o.tri(at, c0, c0 + 1, c0 + 2) : o.fan(at, N, c0);
    }

    // qsub::getInteriorRingFacets (tessellation.cpp:1831-1880)
    GB_HD int qsub_ring(int res, int c0, const Sink &o, int at) const {
        if (res < 1) return 0;
        if (res == 1) return qsub_center(c0, o, at);
        const int inRes = res - 2, inner0 = c0 + N * res;
        int n = 0;
        Strip s;
        s.quads = 1, s.triangulate = triangulate, s.nOuter = res, s.nInner = inRes;
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
            n += s.quads_uniform(o, at + n);
        }
        return n;
    }

    // qsub::getBoundaryRingFacets (tessellation.cpp:1883-1938)
    GB_HD int qsub_boundary_ring(const Sink &o) const {
        const int res = in0, nB = nBoundary;
        int n = 0;
        Strip s;
        s.quads = 1, s.triangulate = triangulate, s.nInner = imax(res - 2, 0);
        for (int e = 0; e < N; ++e) {
            s.nOuter = outer(e);
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
            if (outer(e) == res && res > 1) {
                s.splitFirst = outer((e - 1 + N) % N) != res;
                s.splitLast = outer((e + 1) % N) != res;
                n += s.quads_uniform(o, n);
            } else {
                s.splitFirst = s.splitLast = 1;
                n += s.general(o, n);
            }
        }
        return n;
    }

    template <int K>
    GB_HD int facets_k(const Sink &o) const {
        const int tri = triangulate;
        if (mode == kSingle) return (N == 3) ? o.tri(0, 0, 1, 2) : o.quad(0, 0, 1, 2, 3, 0);
        if (mode == kFan) return o.fan(0, nFacets, 0);
        if (mode == kSplitQuad) return o.quad(0, 0, 1, 2, 3, tri);
        int n = 0;
        if constexpr (K == kQuad) {
            if (uniform) {
                int c0 = 0, res = in0;
                for (int ring = 0; ring < (in0 + 1) / 2; ++ring, res -= 2) {
                    n += quad_ring(res, res, c0, tri, o, n);
                    c0 += 4 * res;
                }
            } else if (mode == kSegmented) {
                n = quad_single_strip(in0, in1, 0, tri, o, 0);
            } else {
                n = quad_boundary_ring(o);
                int ur = in0, vr = in1, c0 = nBoundary;
                const int rings = (imin(ur, vr) + 1) / 2;
                for (int ring = 1; ring < rings; ++ring) {
                    ur = imax(ur - 2, 0);
                    vr = imax(vr - 2, 0);
                    n += quad_ring(ur, vr, c0, tri, o, n);
                    c0 += 2 * (ur + vr);
                }
            }
        } else if constexpr (K == kTri) {
            int res = in0;
            if (uniform) {
                int c0 = 0;
                const int rings = 1 + res / 3;
                for (int ring = 0; ring < rings; ++ring, res -= 3) {
                    n += tri_ring(res, c0, o, n);
                    c0 += 3 * res;
                }
            } else {
                n = tri_boundary_ring(o);
                int c0 = nBoundary;
                const int rings = 1 + res / 3;
                for (int ring = 1; ring < rings; ++ring) {
                    res -= 3;
                    n += tri_ring(res, c0, o, n);
                    c0 += 3 * res;
                }
            }
        } else {
            int res = in0;
            if (uniform) {
                if (res == 1) return qsub_center(0, o, 0);
                int c0 = 0;
                const int rings = (res + 1) / 2;
                for (int ring = 0; ring < rings; ++ring, res -= 2) {
                    n += qsub_ring(res, c0, o, n);
                    c0 += N * res;
                }
            } else {
                n = qsub_boundary_ring(o);
                int c0 = nBoundary;
                const int rings = (res + 1) / 2;
                for (int ring = 1; ring < rings; ++ring) {
                    res = imax(res - 2, 0);
                    n += qsub_ring(res, c0, o, n);
                    c0 += N * res;
                }
            }
        }
        return n;
    }
    GB_HD int facets(const Sink &o) const {
        return kind == kQuad ? facets_k<kQuad>(o) : kind == kTri ? facets_k<kTri>(o)
                                                                 : facets_k<kQsub>(o);
    }
};

// Far::PtexIndices (far/ptexIndices.cpp:37-55): one ptex face for a face of the scheme's
// regular size, one per vertex otherwise.
GB_HD int ptex_count(int regFaceSize, int N) { return N == regFaceSize ? 1 : N; }

#undef GB_HD

}  // namespace tess
}  // namespace gb300
