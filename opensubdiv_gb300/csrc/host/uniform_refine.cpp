// Uniform subdivision and factorized stencil tables for closed (boundary-free) 2-manifold
// cages: the workload generator that produces Far::StencilTable-shaped inputs for the
// evaluator on hosts where the reference's Far factories are not available.
//
// It restates the subdivision rules that Far bakes into its tables, for the default
// Sdc::Options (uniform creasing, Catmark triangle subdivision, no boundaries):
//   - Catmull-Clark (sdc/catmarkScheme.h): face point = centroid; smooth edge point =
//     (v0 + v1 + F0 + F1) / 4 with F the adjacent face points; smooth vertex point =
//     (n-2)/n v + 1/n^2 (sum of edge neighbours + sum of face points);
//   - Loop (sdc/loopScheme.h:84-214): smooth edge point = 3/8 (v0 + v1) + 1/8 (opposite
//     vertices); vertex point with beta(n) = 1/4 cos(2 pi / n) + 3/8, edge weight
//     (5/8 - beta^2) / n;
//   - creases (sdc/scheme.h:390-598, sdc/crease.cpp): sharp edge point = midpoint; crease
//     vertex = 3/4 v + 1/8 (two sharp neighbours); corner vertex = v; semi-sharp transitions
//     blend parent and child rules by the fractional weight of the sharpness that decays to
//     zero; edge sharpness decreases by one per level.
// Child vertices are ordered vertices-from-vertices, then -from-faces, then -from-edges, the
// default order of Vtr refinement (vtr/refinement.cpp:253-270).  Stencils are factorized to
// the control vertices (StencilTableFactory's factorizeIntermediateLevels) and accumulated
// in double, then stored as float.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int kCatmark = 1, kLoop = 2;
constexpr float kInfinite = 10.0f;

struct Level {
    int nv = 0, nf = 0, ne = 0;
    std::vector<int> fOff, fv, fe;  // face -> verts / edges (edge i joins fv[i], fv[i+1])
    std::vector<int> ev;            // 2 per edge
    std::vector<int> ef;            // 2 faces per edge (closed manifold)
    std::vector<float> sharp;       // per edge
    std::vector<int> vOff, vEdge, vFace;  // vertex -> incident edges / faces (unordered)
};

// Sparse stencil rows over the control vertices, CSR.
struct Rows {
    std::vector<int64_t> off;
    std::vector<int> idx;
    std::vector<double> w;
};

struct Topology {
    int scheme = kCatmark;
    std::vector<Level> levels;
    std::vector<Rows> rows;  // rows[l] = stencils of level-l vertices (rows[0] identity)
    std::vector<int> ptexOff;
    // masks of one level, between GB300TopologyMaskCounts and GB300TopologyMaskCopy
    std::vector<int64_t> maskOff;
    std::vector<int> maskIdx;
    std::vector<float> maskW;
    // limit stencils produced by the last GB300TopologyLimitStencils call
    std::vector<int> lsizes, loffsets, lidx;
    std::vector<float> lw[3];
    std::string error;
};

thread_local std::string t_err;

inline int64_t edge_key(int a, int b) {
    if (a > b) std::swap(a, b);
    return ((int64_t)a << 32) | (uint32_t)b;
}

bool finish_level(Level &L, std::string &err) {
    // edge -> faces
    L.ef.assign(2 * (size_t)L.ne, -1);
    for (int f = 0; f < L.nf; ++f)
        for (int i = L.fOff[f]; i < L.fOff[f + 1]; ++i) {
            const int e = L.fe[i];
            if (L.ef[2 * (size_t)e] < 0) L.ef[2 * (size_t)e] = f;
            else if (L.ef[2 * (size_t)e + 1] < 0) L.ef[2 * (size_t)e + 1] = f;
            else { err = "non-manifold edge"; return false; }
        }
    for (int e = 0; e < L.ne; ++e)
        if (L.ef[2 * (size_t)e + 1] < 0) { err = "boundary edge (only closed cages are supported)"; return false; }
    // vertex -> edges, faces
    std::vector<int> ecount(L.nv + 1, 0), fcount(L.nv + 1, 0);
    for (int e = 0; e < L.ne; ++e) { ecount[L.ev[2 * e]]++; ecount[L.ev[2 * e + 1]]++; }
    for (size_t i = 0; i < L.fv.size(); ++i) fcount[L.fv[i]]++;
    L.vOff.assign(L.nv + 1, 0);
    for (int v = 0; v < L.nv; ++v) {
        if (ecount[v] != fcount[v]) { err = "non-manifold vertex"; return false; }
        L.vOff[v + 1] = L.vOff[v] + ecount[v];
    }
    L.vEdge.assign(L.vOff[L.nv], 0);
    L.vFace.assign(L.vOff[L.nv], 0);
    std::vector<int> pe(L.vOff.begin(), L.vOff.end() - 1), pf = pe;
    for (int e = 0; e < L.ne; ++e) {
        L.vEdge[pe[L.ev[2 * e]]++] = e;
        L.vEdge[pe[L.ev[2 * e + 1]]++] = e;
    }
    for (int f = 0; f < L.nf; ++f)
        for (int i = L.fOff[f]; i < L.fOff[f + 1]; ++i) L.vFace[pf[L.fv[i]]++] = f;
    return true;
}

bool make_base(Level &L, int nverts, int nfaces, const int *vpf, const int *fv, int ncreases,
               const int *cv, const float *cs, std::string &err) {
    L.nv = nverts;
    L.nf = nfaces;
    L.fOff.assign(nfaces + 1, 0);
    for (int f = 0; f < nfaces; ++f) L.fOff[f + 1] = L.fOff[f] + vpf[f];
    L.fv.assign(fv, fv + L.fOff[nfaces]);
    L.fe.assign(L.fv.size(), -1);
    std::unordered_map<int64_t, int> emap;
    emap.reserve(L.fv.size());
    for (int f = 0; f < nfaces; ++f) {
        const int b = L.fOff[f], n = vpf[f];
        for (int i = 0; i < n; ++i) {
            const int a = L.fv[b + i], c = L.fv[b + (i + 1) % n];
            auto it = emap.find(edge_key(a, c));
            int e;
            if (it == emap.end()) {
                e = (int)(L.ev.size() / 2);
                emap.emplace(edge_key(a, c), e);
                L.ev.push_back(a);
                L.ev.push_back(c);
            } else {
                e = it->second;
            }
            L.fe[b + i] = e;
        }
    }
    L.ne = (int)(L.ev.size() / 2);
    L.sharp.assign(L.ne, 0.0f);
    for (int k = 0; k < ncreases; ++k) {
        auto it = emap.find(edge_key(cv[2 * k], cv[2 * k + 1]));
        if (it == emap.end()) { err = "crease edge not in the mesh"; return false; }
        L.sharp[it->second] = std::max(L.sharp[it->second], cs[k]);
    }
    return finish_level(L, err);
}

inline float decrement(float s) {
    if (s <= 0.0f) return 0.0f;
    if (s >= kInfinite) return kInfinite;
    return s > 1.0f ? s - 1.0f : 0.0f;
}

// Child topology of a uniform refinement.  Catmark: every n-gon -> n quads; Loop: every
// triangle -> 4 triangles.
void refine_topology(int scheme, const Level &P, Level &C) {
    const bool cat = scheme == kCatmark;
    const int vFace = cat ? P.nv : -1;             // first child vertex from a face
    const int vEdge = cat ? P.nv + P.nf : P.nv;    // first child vertex from an edge
    C.nv = P.nv + (cat ? P.nf : 0) + P.ne;
    // child edges: from faces first, then 2 per parent edge
    int nFaceEdges = 0;
    if (cat) nFaceEdges = (int)P.fv.size();  // one per face corner
    else nFaceEdges = 3 * P.nf;              // interior triangle edges
    C.ne = nFaceEdges + 2 * P.ne;
    C.ev.assign(2 * (size_t)C.ne, 0);
    C.sharp.assign(C.ne, 0.0f);
    for (int e = 0; e < P.ne; ++e) {
        const int a = P.ev[2 * e], b = P.ev[2 * e + 1], m = vEdge + e;
        const int e0 = nFaceEdges + 2 * e, e1 = e0 + 1;
        C.ev[2 * (size_t)e0] = a; C.ev[2 * (size_t)e0 + 1] = m;
        C.ev[2 * (size_t)e1] = m; C.ev[2 * (size_t)e1 + 1] = b;
        C.sharp[e0] = C.sharp[e1] = decrement(P.sharp[e]);
    }
    // child edge of parent edge e incident to parent vertex v
    auto half = [&](int e, int v) { return nFaceEdges + 2 * e + (P.ev[2 * e] == v ? 0 : 1); };
    if (cat) {
        C.nf = (int)P.fv.size();
        C.fOff.resize(C.nf + 1);
        for (int i = 0; i <= C.nf; ++i) C.fOff[i] = 4 * i;
        C.fv.resize(4 * (size_t)C.nf);
        C.fe.resize(4 * (size_t)C.nf);
        for (int f = 0; f < P.nf; ++f) {
            const int b = P.fOff[f], n = P.fOff[f + 1] - b;
            for (int i = 0; i < n; ++i) {
                const int ip = (i + n - 1) % n;
                const int v = P.fv[b + i], ei = P.fe[b + i], ep = P.fe[b + ip];
                // interior edges of the face: corner i -> (face point, edge point of e_i)
                const int fe_i = b + i;
                C.ev[2 * (size_t)fe_i] = vFace + f;
                C.ev[2 * (size_t)fe_i + 1] = vEdge + ei;
                const int cf = b + i;  // child face index = parent face corner index
                int *cvp = &C.fv[4 * (size_t)cf];
                int *cep = &C.fe[4 * (size_t)cf];
                cvp[0] = v; cvp[1] = vEdge + ei; cvp[2] = vFace + f; cvp[3] = vEdge + ep;
                cep[0] = half(ei, v);
                cep[1] = b + i;
                cep[2] = b + ip;
                cep[3] = half(ep, v);
            }
        }
    } else {
        C.nf = 4 * P.nf;
        C.fOff.resize(C.nf + 1);
        for (int i = 0; i <= C.nf; ++i) C.fOff[i] = 3 * i;
        C.fv.resize(3 * (size_t)C.nf);
        C.fe.resize(3 * (size_t)C.nf);
        for (int f = 0; f < P.nf; ++f) {
            const int b = P.fOff[f];
            const int v[3] = {P.fv[b], P.fv[b + 1], P.fv[b + 2]};
            const int e[3] = {P.fe[b], P.fe[b + 1], P.fe[b + 2]};
            const int m[3] = {vEdge + e[0], vEdge + e[1], vEdge + e[2]};
            // interior edges: m0-m1, m1-m2, m2-m0
            for (int i = 0; i < 3; ++i) {
                const int ie = 3 * f + i;
                C.ev[2 * (size_t)ie] = m[i];
                C.ev[2 * (size_t)ie + 1] = m[(i + 1) % 3];
            }
            // corner triangles i: (v_i, m_i, m_{i-1}); center: (m0, m1, m2)
            for (int i = 0; i < 3; ++i) {
                const int ip = (i + 2) % 3, cf = 4 * f + i;
                int *cvp = &C.fv[3 * (size_t)cf];
                int *cep = &C.fe[3 * (size_t)cf];
                cvp[0] = v[i]; cvp[1] = m[i]; cvp[2] = m[ip];
                cep[0] = half(e[i], v[i]);
                cep[1] = 3 * f + ip;
                cep[2] = half(e[ip], v[i]);
            }
            int *cvp = &C.fv[3 * (size_t)(4 * f + 3)];
            int *cep = &C.fe[3 * (size_t)(4 * f + 3)];
            cvp[0] = m[0]; cvp[1] = m[1]; cvp[2] = m[2];
            cep[0] = 3 * f + 0; cep[1] = 3 * f + 1; cep[2] = 3 * f + 2;
        }
    }
}

// A child vertex as a small combination of parent vertices.
// At most 64 distinct parents (a Catmark vertex of valence up to 31 over quads); a mask that
// would need more sets `overflow` and the refinement reports an error.
struct Mask {
    int n = 0;
    bool overflow = false;
    int idx[64];
    double w[64];
    void add(int i, double x) {
        for (int k = 0; k < n; ++k)
            if (idx[k] == i) { w[k] += x; return; }
        if (n == 64) { overflow = true; return; }
        idx[n] = i; w[n] = x; ++n;
    }
};

inline int other_end(const Level &P, int e, int v) {
    return P.ev[2 * e] == v ? P.ev[2 * e + 1] : P.ev[2 * e];
}

void add_face_point(const Level &P, int f, double wt, Mask &m) {
    const int b = P.fOff[f], n = P.fOff[f + 1] - b;
    for (int i = 0; i < n; ++i) m.add(P.fv[b + i], wt / n);
}

// Loop: the vertex of face f opposite edge e
inline int opposite(const Level &P, int f, int e) {
    const int b = P.fOff[f];
    for (int i = 0; i < 3; ++i)
        if (P.fe[b + i] == e) return P.fv[b + (i + 2) % 3];
    return -1;
}

void edge_mask(int scheme, const Level &P, int e, Mask &m) {
    const int a = P.ev[2 * e], b = P.ev[2 * e + 1];
    const float s = P.sharp[e];
    if (s >= 1.0f) {  // crease (a full crease in the child as well)
        m.add(a, 0.5); m.add(b, 0.5);
        return;
    }
    const double pw = s > 0.0f ? (double)s : 0.0, cw = 1.0 - pw;
    const int f0 = P.ef[2 * (size_t)e], f1 = P.ef[2 * (size_t)e + 1];
    if (scheme == kCatmark) {
        m.add(a, pw * 0.5 + cw * 0.25); m.add(b, pw * 0.5 + cw * 0.25);
        add_face_point(P, f0, 0.25 * cw, m);
        add_face_point(P, f1, 0.25 * cw, m);
    } else {
        m.add(a, pw * 0.5 + cw * 0.375); m.add(b, pw * 0.5 + cw * 0.375);
        m.add(opposite(P, f0, e), 0.125 * cw);
        m.add(opposite(P, f1, e), 0.125 * cw);
    }
}

enum Rule { kSmooth, kCrease, kCorner };

// rule mask for vertex v given which incident edges are sharp
void rule_mask(int scheme, const Level &P, int v, Rule r, const std::vector<int> &sharpEnds,
               double scale, Mask &m) {
    const int b = P.vOff[v], n = P.vOff[v + 1] - b;
    if (r == kCorner) { m.add(v, scale); return; }
    if (r == kCrease) {
        m.add(v, 0.75 * scale);
        m.add(sharpEnds[0], 0.125 * scale);
        m.add(sharpEnds[1], 0.125 * scale);
        return;
    }
    if (scheme == kCatmark) {
        const double dn = n;
        m.add(v, scale * (dn - 2.0) / dn);
        for (int k = 0; k < n; ++k) {
            m.add(other_end(P, P.vEdge[b + k], v), scale / (dn * dn));
            add_face_point(P, P.vFace[b + k], scale / (dn * dn), m);
        }
    } else {
        double ew = 0.0625, vw = 0.625;
        if (n != 6) {
            const double inv = 1.0 / n;
            const double beta = 0.25 * std::cos(M_PI * 2.0 * inv) + 0.375;
            ew = (0.625 - beta * beta) * inv;
            vw = 1.0 - ew * n;
        }
        m.add(v, scale * vw);
        for (int k = 0; k < n; ++k) m.add(other_end(P, P.vEdge[b + k], v), scale * ew);
    }
}

void vertex_mask(int scheme, const Level &P, int v, Mask &m) {
    const int b = P.vOff[v], n = P.vOff[v + 1] - b;
    int psharp = 0, csharp = 0;
    double tsum = 0.0;
    int tcount = 0;
    std::vector<int> pEnds, cEnds;
    for (int k = 0; k < n; ++k) {
        const int e = P.vEdge[b + k];
        const float s = P.sharp[e];
        if (s > 0.0f) { ++psharp; pEnds.push_back(other_end(P, e, v)); }
        if (decrement(s) > 0.0f) { ++csharp; cEnds.push_back(other_end(P, e, v)); }
        if (s > 0.0f && s <= 1.0f) { tsum += s; ++tcount; }
    }
    auto rule = [](int c) { return c <= 1 ? kSmooth : c == 2 ? kCrease : kCorner; };
    const Rule pr = rule(psharp), cr = rule(csharp);
    if (pr == kSmooth || pr == cr) {
        rule_mask(scheme, P, v, pr, pEnds, 1.0, m);
        return;
    }
    double pw = tcount ? tsum / tcount : 0.0;
    if (pw > 1.0) pw = 1.0;
    rule_mask(scheme, P, v, pr, pEnds, pw, m);
    rule_mask(scheme, P, v, cr, cEnds, 1.0 - pw, m);
}

// Composes child masks with the parent's factorized rows; false when a mask overflowed.
bool compose(int scheme, const Level &P, const Rows &prow, int nControl, Rows &crow,
             int nChild) {
    const bool cat = scheme == kCatmark;
    const int vFace = cat ? P.nv : -1, vEdge = cat ? P.nv + P.nf : P.nv;
    std::vector<int> cnt(nChild, 0);
    std::vector<std::vector<int>> tidx;
    std::vector<std::vector<double>> tw;
    int nth = 1;
#ifdef _OPENMP
    nth = omp_get_max_threads();
#endif
    // two passes: sizes, then fill; each thread owns a dense accumulator
    crow.off.assign(nChild + 1, 0);
    std::vector<std::vector<int>> lidx(nth);
    std::vector<std::vector<double>> lw(nth);
    std::vector<int64_t> chunkStart(nth + 1, 0);
    const int chunk = (nChild + nth - 1) / nth;
    int overflow = 0;
#pragma omp parallel num_threads(nth) reduction(| : overflow)
    {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
        std::vector<double> acc(nControl, 0.0);
        std::vector<int> touched;
        touched.reserve(1024);
        std::vector<char> mark(nControl, 0);
        const int lo = t * chunk, hi = std::min(nChild, lo + chunk);
        auto &oi = lidx[t];
        auto &ow = lw[t];
        for (int c = lo; c < hi; ++c) {
            Mask m;
            if (c < P.nv) vertex_mask(scheme, P, c, m);
            else if (cat && c < vEdge) add_face_point(P, c - vFace, 1.0, m);
            else edge_mask(scheme, P, c - vEdge, m);
            overflow |= m.overflow ? 1 : 0;
            touched.clear();
            for (int k = 0; k < m.n; ++k) {
                const int p = m.idx[k];
                const double wk = m.w[k];
                for (int64_t j = prow.off[p]; j < prow.off[p + 1]; ++j) {
                    const int q = prow.idx[j];
                    if (!mark[q]) { mark[q] = 1; touched.push_back(q); }
                    acc[q] += wk * prow.w[j];
                }
            }
            cnt[c] = (int)touched.size();
            for (int q : touched) {
                oi.push_back(q);
                ow.push_back(acc[q]);
                acc[q] = 0.0;
                mark[q] = 0;
            }
        }
    }
    for (int c = 0; c < nChild; ++c) crow.off[c + 1] = crow.off[c] + cnt[c];
    crow.idx.resize(crow.off[nChild]);
    crow.w.resize(crow.off[nChild]);
    int64_t pos = 0;
    for (int t = 0; t < nth; ++t) {
        std::copy(lidx[t].begin(), lidx[t].end(), crow.idx.begin() + pos);
        std::copy(lw[t].begin(), lw[t].end(), crow.w.begin() + pos);
        pos += (int64_t)lidx[t].size();
    }
    return !overflow;
}

int fail(const char *msg) {
    t_err = msg;
    return 1;
}

}  // namespace

extern "C" {

const char *GB300TopologyGetLastError(void) { return t_err.c_str(); }

// Worker threads used by this calling thread's refinement and table copies (OpenMP
// nthreads-var of the calling thread); 1 when many meshes are generated concurrently.
void GB300TopologySetNumThreads(int n) { omp_set_num_threads(n > 0 ? n : 1); }

void *GB300TopologyCreate(int scheme, int nverts, int nfaces, const int *vertsPerFace,
                          const int *faceVerts, int ncreases, const int *creaseVerts,
                          const float *creaseSharpness) {
    if ((scheme != kCatmark && scheme != kLoop) || nverts <= 0 || nfaces <= 0) {
        t_err = "GB300TopologyCreate: unsupported scheme or empty cage";
        return nullptr;
    }
    if (scheme == kLoop)
        for (int f = 0; f < nfaces; ++f)
            if (vertsPerFace[f] != 3) { t_err = "Loop cages must be all triangles"; return nullptr; }
    std::unique_ptr<Topology> t(new Topology);
    t->scheme = scheme;
    t->levels.resize(1);
    if (!make_base(t->levels[0], nverts, nfaces, vertsPerFace, faceVerts, ncreases, creaseVerts,
                   creaseSharpness, t_err))
        return nullptr;
    Rows id;
    id.off.resize(nverts + 1);
    id.idx.resize(nverts);
    id.w.assign(nverts, 1.0);
    for (int v = 0; v <= nverts; ++v) id.off[v] = v;
    for (int v = 0; v < nverts; ++v) id.idx[v] = v;
    t->rows.push_back(std::move(id));
    const int reg = scheme == kLoop ? 3 : 4;
    t->ptexOff.assign(nfaces + 1, 0);
    for (int f = 0; f < nfaces; ++f)
        t->ptexOff[f + 1] = t->ptexOff[f] + (vertsPerFace[f] == reg ? 1 : vertsPerFace[f]);
    t_err.clear();
    return t.release();
}

void GB300TopologyDestroy(void *p) { delete (Topology *)p; }

// Refines uniformly up to `level` (1..10), building factorized rows for every level.
// Topology of levels 1..level (no stencils).
int GB300TopologyRefineTopology(void *p, int level) {
    Topology *t = (Topology *)p;
    if (!t || level < 1 || level > 10) return fail("GB300TopologyRefineTopology: bad level");
    while ((int)t->levels.size() <= level) {
        Level child;
        refine_topology(t->scheme, t->levels.back(), child);
        std::string err;
        if (!finish_level(child, err)) return fail(err.c_str());
        t->levels.push_back(std::move(child));
    }
    return 0;
}

// Topology and factorized stencils of levels 1..level.
int GB300TopologyRefineUniform(void *p, int level) {
    Topology *t = (Topology *)p;
    if (!t || level < 1 || level > 10) return fail("GB300TopologyRefineUniform: bad level");
    if (GB300TopologyRefineTopology(p, level)) return 1;
    while ((int)t->rows.size() <= level) {
        const size_t l = t->rows.size();  // compose level l from level l - 1
        Rows r;
        if (!compose(t->scheme, t->levels[l - 1], t->rows.back(), t->levels[0].nv, r,
                     t->levels[l].nv))
            return fail("GB300TopologyRefineUniform: a vertex valence or face size beyond "
                        "the generator's 64-parent masks");
        t->rows.push_back(std::move(r));
    }
    return 0;
}

// Subdivision masks of the level-`level` vertices in the form Far::PrimvarRefiner feeds a
// stencil builder (far/primvarRefiner.h:475-650): per child vertex, (source, float weight)
// pairs in call order -- face points: the face's vertices; edge points: both ends, then (Catmark)
// the adjacent face points of the same level or (Loop) the opposite vertices; vertex points:
// (Catmark) the incident face points, then the edge neighbours, then the vertex itself.  Zero
// weights are left out.  Sources are global indices (control vertices, then each level's
// vertices), so a level's masks name the previous level and its own face points.  These are
// the inputs of the GPU stencil-table factory (GB300StencilTableFactoryCreate).
struct FarMask {
    static constexpr int kMax = 160;
    int n = 0;
    bool overflow = false;
    int src[kMax];
    float w[kMax];
    void add(int s, double x) {
        const float f = (float)x;
        if (f == 0.0f) return;
        if (n == kMax) { overflow = true; return; }
        src[n] = s; w[n] = f; ++n;
    }
};

// per-slot weights of a vertex rule (incident faces / edges in vFace / vEdge order)
void vertex_slots(int scheme, const Level &P, int v, Rule r, const std::vector<int> &sharpEnds,
                  double scale, double *fw, double *ew, double &vw) {
    const int b = P.vOff[v], n = P.vOff[v + 1] - b;
    if (r == kCorner) { vw += scale; return; }
    if (r == kCrease) {
        vw += 0.75 * scale;
        for (int k = 0; k < n; ++k) {
            const int o = other_end(P, P.vEdge[b + k], v);
            if (o == sharpEnds[0] || o == sharpEnds[1]) ew[k] += 0.125 * scale;
        }
        return;
    }
    if (scheme == kCatmark) {
        const double dn = n;
        vw += scale * (dn - 2.0) / dn;
        for (int k = 0; k < n; ++k) {
            ew[k] += scale / (dn * dn);
            fw[k] += scale / (dn * dn);
        }
    } else {
        double e = 0.0625, c = 0.625;
        if (n != 6) {
            const double inv = 1.0 / n;
            const double beta = 0.25 * std::cos(M_PI * 2.0 * inv) + 0.375;
            e = (0.625 - beta * beta) * inv;
            c = 1.0 - e * n;
        }
        vw += scale * c;
        for (int k = 0; k < n; ++k) ew[k] += scale * e;
    }
}

void far_mask(int scheme, const Level &P, int c, int64_t parentBase, int64_t childBase,
              FarMask &m) {
    const bool cat = scheme == kCatmark;
    const int vFace = P.nv, vEdge = cat ? P.nv + P.nf : P.nv;
    auto faceChild = [&](int f) { return (int)(childBase + vFace + f); };
    if (c < P.nv) {  // vertex point
        const int v = c, b = P.vOff[v], n = P.vOff[v + 1] - b;
        if (2 * n + 1 > FarMask::kMax) { m.overflow = true; return; }
        double fw[FarMask::kMax] = {0}, ew[FarMask::kMax] = {0}, vw = 0.0;
        int psharp = 0, csharp = 0, tcount = 0;
        double tsum = 0.0;
        std::vector<int> pEnds, cEnds;
        for (int k = 0; k < n; ++k) {
            const int e = P.vEdge[b + k];
            const float s = P.sharp[e];
            if (s > 0.0f) { ++psharp; pEnds.push_back(other_end(P, e, v)); }
            if (decrement(s) > 0.0f) { ++csharp; cEnds.push_back(other_end(P, e, v)); }
            if (s > 0.0f && s <= 1.0f) { tsum += s; ++tcount; }
        }
        auto rule = [](int k) { return k <= 1 ? kSmooth : k == 2 ? kCrease : kCorner; };
        const Rule pr = rule(psharp), cr = rule(csharp);
        if (pr == kSmooth || pr == cr) {
            vertex_slots(scheme, P, v, pr, pEnds, 1.0, fw, ew, vw);
        } else {
            double pw = tcount ? tsum / tcount : 0.0;
            if (pw > 1.0) pw = 1.0;
            vertex_slots(scheme, P, v, pr, pEnds, pw, fw, ew, vw);
            vertex_slots(scheme, P, v, cr, cEnds, 1.0 - pw, fw, ew, vw);
        }
        if (cat)
            for (int k = 0; k < n; ++k) m.add(faceChild(P.vFace[b + k]), fw[k]);
        for (int k = 0; k < n; ++k) m.add((int)(parentBase + other_end(P, P.vEdge[b + k], v)), ew[k]);
        m.add((int)(parentBase + v), vw);
    } else if (cat && c < vEdge) {  // face point
        const int f = c - vFace, b = P.fOff[f], n = P.fOff[f + 1] - b;
        const float w = 1.0f / (float)n;
        for (int i = 0; i < n; ++i) m.add((int)(parentBase + P.fv[b + i]), w);
    } else {  // edge point
        const int e = c - vEdge;
        const int a = P.ev[2 * e], bb = P.ev[2 * e + 1];
        const float s = P.sharp[e];
        if (s >= 1.0f) {
            m.add((int)(parentBase + a), 0.5);
            m.add((int)(parentBase + bb), 0.5);
            return;
        }
        const double pw = s > 0.0f ? (double)s : 0.0, cw = 1.0 - pw;
        const int f0 = P.ef[2 * (size_t)e], f1 = P.ef[2 * (size_t)e + 1];
        const double vwt = pw * 0.5 + cw * (cat ? 0.25 : 0.375);
        m.add((int)(parentBase + a), vwt);
        m.add((int)(parentBase + bb), vwt);
        if (cat) {
            m.add(faceChild(f0), 0.25 * cw);
            m.add(faceChild(f1), 0.25 * cw);
        } else {
            m.add((int)(parentBase + opposite(P, f0, e)), 0.125 * cw);
            m.add((int)(parentBase + opposite(P, f1, e)), 0.125 * cw);
        }
    }
}

int GB300TopologyMaskCounts(void *p, int level, int *nChild, int64_t *nnz) {
    Topology *t = (Topology *)p;
    if (!t || level < 1 || level >= (int)t->levels.size())
        return fail("GB300TopologyMaskCounts: level not refined");
    const Level &P = t->levels[level - 1];
    const int nc = t->levels[level].nv;
    int64_t parentBase = 0;
    for (int l = 0; l < level - 1; ++l) parentBase += t->levels[l].nv;
    const int64_t childBase = parentBase + P.nv;
    // two passes (sizes, then the masks again into place): no per-child staging buffer
    t->maskOff.assign(nc + 1, 0);
    int overflow = 0;
#pragma omp parallel for schedule(static) reduction(| : overflow)
    for (int c = 0; c < nc; ++c) {
        FarMask m;
        far_mask(t->scheme, P, c, parentBase, childBase, m);
        t->maskOff[c + 1] = m.n;
        overflow |= m.overflow ? 1 : 0;
    }
    if (overflow) {
        std::vector<int64_t>().swap(t->maskOff);
        return fail("GB300TopologyMaskCounts: a vertex valence beyond the generator's masks");
    }
    for (int c = 0; c < nc; ++c) t->maskOff[c + 1] += t->maskOff[c];
    t->maskIdx.resize(t->maskOff[nc]);
    t->maskW.resize(t->maskOff[nc]);
#pragma omp parallel for schedule(static)
    for (int c = 0; c < nc; ++c) {
        FarMask m;
        far_mask(t->scheme, P, c, parentBase, childBase, m);
        std::copy(m.src, m.src + m.n, t->maskIdx.begin() + t->maskOff[c]);
        std::copy(m.w, m.w + m.n, t->maskW.begin() + t->maskOff[c]);
    }
    *nChild = nc;
    *nnz = t->maskOff[nc];
    return 0;
}

int GB300TopologyMaskCopy(void *p, int64_t *offsets, int *sources, float *weights) {
    Topology *t = (Topology *)p;
    if (!t || t->maskOff.empty()) return fail("GB300TopologyMaskCopy: no masks computed");
    std::copy(t->maskOff.begin(), t->maskOff.end(), offsets);
    std::copy(t->maskIdx.begin(), t->maskIdx.end(), sources);
    std::copy(t->maskW.begin(), t->maskW.end(), weights);
    std::vector<int64_t>().swap(t->maskOff);
    std::vector<int>().swap(t->maskIdx);
    std::vector<float>().swap(t->maskW);
    return 0;
}

int GB300TopologyGetNumVertices(void *p, int level) {
    Topology *t = (Topology *)p;
    return (t && level >= 0 && level < (int)t->levels.size()) ? t->levels[level].nv : -1;
}

int GB300TopologyGetNumPtexFaces(void *p) {
    Topology *t = (Topology *)p;
    return t ? t->ptexOff.back() : -1;
}

// Number of stencils and entries of levels [first, last] concatenated.
int GB300TopologyStencilCounts(void *p, int first, int last, int *numStencils, int64_t *nnz) {
    Topology *t = (Topology *)p;
    if (!t || first < 1 || last >= (int)t->rows.size() || first > last)
        return fail("GB300TopologyStencilCounts: bad level range");
    int64_t n = 0, z = 0;
    for (int l = first; l <= last; ++l) {
        n += t->levels[l].nv;
        z += t->rows[l].off.back();
    }
    if (n > 0x7fffffff || z > 0x7fffffff) return fail("stencil table exceeds 32-bit offsets");
    *numStencils = (int)n;
    *nnz = z;
    return 0;
}

int GB300TopologyStencilCopy(void *p, int first, int last, int *sizes, int *offsets,
                             int *indices, float *weights) {
    Topology *t = (Topology *)p;
    int ns;
    int64_t nz;
    if (GB300TopologyStencilCounts(p, first, last, &ns, &nz)) return 1;
    int64_t s = 0, z = 0;
    for (int l = first; l <= last; ++l) {
        const Rows &r = t->rows[l];
        const int nv = t->levels[l].nv;
#pragma omp parallel for schedule(static)
        for (int v = 0; v < nv; ++v) {
            sizes[s + v] = (int)(r.off[v + 1] - r.off[v]);
            offsets[s + v] = (int)(z + r.off[v]);
        }
#pragma omp parallel for schedule(static)
        for (int64_t j = 0; j < r.off[nv]; ++j) {
            indices[z + j] = r.idx[j];
            weights[z + j] = (float)r.w[j];
        }
        s += nv;
        z += r.off[nv];
    }
    return 0;
}

// Vertex indices (at the finest level L) of the corners of the level-L sub-square that
// contains (u, v) of ptex face `face`, in ptex frame order (0,0), (1,0), (1,1), (0,1), plus
// the local (s, t) in that sub-square.  Catmark only.
static bool locate(const Topology &t, int L, int face, float u, float v, int corner[4],
                   double &s, double &tt, std::vector<std::unordered_map<int64_t, int>> &emaps) {
    const Level &l0 = t.levels[0];
    int f = (int)(std::upper_bound(t.ptexOff.begin(), t.ptexOff.end(), face) - t.ptexOff.begin()) - 1;
    if (f < 0 || f >= l0.nf) return false;
    const int b = l0.fOff[f], n = l0.fOff[f + 1] - b;
    int c[4];
    int startLevel = 0;
    if (n == 4) {
        for (int i = 0; i < 4; ++i) c[i] = l0.fv[b + i];
    } else {
        // non-quad: ptex sub-face i is the level-1 child face at corner i
        const int i = face - t.ptexOff[f];
        const int ip = (i + n - 1) % n;
        const Level &p = l0;
        c[0] = p.fv[b + i];
        c[1] = p.nv + p.nf + p.fe[b + i];
        c[2] = p.nv + f;
        c[3] = p.nv + p.nf + p.fe[b + ip];
        startLevel = 1;
    }
    double uu = u, vv = v;
    for (int l = startLevel; l < L; ++l) {
        const Level &p = t.levels[l];
        auto edge_child = [&](int a, int bb) {
            auto it = emaps[l].find(edge_key(a, bb));
            return p.nv + p.nf + it->second;
        };
        // face point of the quad (c0..c3) at level l: find the face via the edge c0-c1
        auto it = emaps[l].find(edge_key(c[0], c[1]));
        const int e01 = it->second;
        int fq = p.ef[2 * (size_t)e01];
        {
            // pick the adjacent face that also contains c2
            const int bq = p.fOff[fq];
            bool has = false;
            for (int k = bq; k < p.fOff[fq + 1]; ++k) has |= p.fv[k] == c[2];
            if (!has) fq = p.ef[2 * (size_t)e01 + 1];
        }
        const int fp = p.nv + fq;
        const int m01 = edge_child(c[0], c[1]), m12 = edge_child(c[1], c[2]);
        const int m23 = edge_child(c[2], c[3]), m30 = edge_child(c[3], c[0]);
        const int hu = uu >= 0.5, hv = vv >= 0.5;
        if (hu) uu -= 0.5;
        if (hv) vv -= 0.5;
        uu *= 2.0;
        vv *= 2.0;
        int d[4];
        if (!hu && !hv) { d[0] = c[0]; d[1] = m01; d[2] = fp; d[3] = m30; }
        else if (hu && !hv) { d[0] = m01; d[1] = c[1]; d[2] = m12; d[3] = fp; }
        else if (hu && hv) { d[0] = fp; d[1] = m12; d[2] = c[2]; d[3] = m23; }
        else { d[0] = m30; d[1] = fp; d[2] = m23; d[3] = c[3]; }
        for (int k = 0; k < 4; ++k) c[k] = d[k];
    }
    for (int k = 0; k < 4; ++k) corner[k] = c[k];
    s = uu;
    tt = vv;
    return true;
}

// Limit stencils of a uniformly refined Catmark cage at n (ptex face, u, v) locations:
// bilinear over the finest-level faces (what LimitStencilTableFactory builds for a uniform
// refiner, far/stencilTableFactory.h:200-206), with du/dv weights.  Locations that do not
// resolve are dropped, as the reference drops them.  Returns the number of stencils.
int GB300TopologyLimitStencils(void *p, int n, const int *faces, const float *u, const float *v) {
    Topology *t = (Topology *)p;
    if (!t || t->scheme != kCatmark) return -fail("limit stencils: Catmark topology required");
    const int L = (int)t->levels.size() - 1;
    if (L < 1) return -fail("limit stencils: refine first");
    std::vector<std::unordered_map<int64_t, int>> emaps(L);
    for (int l = 0; l < L; ++l) {
        const Level &lv = t->levels[l];
        emaps[l].reserve(2 * (size_t)lv.ne);
        for (int e = 0; e < lv.ne; ++e) emaps[l].emplace(edge_key(lv.ev[2 * e], lv.ev[2 * e + 1]), e);
    }
    const Rows &R = t->rows[L];
    const int ncv = t->levels[0].nv;
    std::vector<int> cnt(n, -1);
    int nth = 1;
#ifdef _OPENMP
    nth = omp_get_max_threads();
#endif
    std::vector<std::vector<int>> li(nth);
    std::vector<std::vector<float>> lw0(nth), lw1(nth), lw2(nth);
    const int chunk = (n + nth - 1) / nth;
    const double scale = (double)(1 << L);
#pragma omp parallel num_threads(nth)
    {
        int th = 0;
#ifdef _OPENMP
        th = omp_get_thread_num();
#endif
        std::vector<double> a0(ncv, 0.0), a1(ncv, 0.0), a2(ncv, 0.0);
        std::vector<char> mark(ncv, 0);
        std::vector<int> touched;
        const int lo = th * chunk, hi = std::min(n, lo + chunk);
        for (int i = lo; i < hi; ++i) {
            int c[4];
            double s, tt;
            if (!locate(*t, L, faces[i], u[i], v[i], c, s, tt, emaps)) continue;
            // derivatives with respect to the ptex face's (u, v) scaled by 2^L on every face,
            // the sub-faces of non-quads included: Far's convention (its patch bases scale by
            // 2^depth whatever the non-quad root), so the table equals
            // LimitStencilTableFactory's
            const double ds = scale;
            const double wp[4] = {(1 - s) * (1 - tt), s * (1 - tt), s * tt, (1 - s) * tt};
            const double wu[4] = {-(1 - tt) * ds, (1 - tt) * ds, tt * ds, -tt * ds};
            const double wv[4] = {-(1 - s) * ds, -s * ds, s * ds, (1 - s) * ds};
            touched.clear();
            for (int k = 0; k < 4; ++k)
                for (int64_t j = R.off[c[k]]; j < R.off[c[k] + 1]; ++j) {
                    const int q = R.idx[j];
                    if (!mark[q]) { mark[q] = 1; touched.push_back(q); }
                    a0[q] += wp[k] * R.w[j];
                    a1[q] += wu[k] * R.w[j];
                    a2[q] += wv[k] * R.w[j];
                }
            cnt[i] = (int)touched.size();
            for (int q : touched) {
                li[th].push_back(q);
                lw0[th].push_back((float)a0[q]);
                lw1[th].push_back((float)a1[q]);
                lw2[th].push_back((float)a2[q]);
                a0[q] = a1[q] = a2[q] = 0.0;
                mark[q] = 0;
            }
        }
    }
    t->lsizes.clear();
    t->loffsets.clear();
    int64_t z = 0;
    for (int i = 0; i < n; ++i)
        if (cnt[i] >= 0) {
            t->lsizes.push_back(cnt[i]);
            t->loffsets.push_back((int)z);
            z += cnt[i];
        }
    t->lidx.clear();
    for (auto &w : t->lw) w.clear();
    t->lidx.reserve(z);
    for (int th = 0; th < nth; ++th) {
        t->lidx.insert(t->lidx.end(), li[th].begin(), li[th].end());
        t->lw[0].insert(t->lw[0].end(), lw0[th].begin(), lw0[th].end());
        t->lw[1].insert(t->lw[1].end(), lw1[th].begin(), lw1[th].end());
        t->lw[2].insert(t->lw[2].end(), lw2[th].begin(), lw2[th].end());
    }
    return (int)t->lsizes.size();
}

int64_t GB300TopologyLimitStencilNnz(void *p) {
    Topology *t = (Topology *)p;
    return t ? (int64_t)t->lidx.size() : -1;
}

int GB300TopologyLimitStencilCopy(void *p, int *sizes, int *offsets, int *indices, float *w,
                                  float *du, float *dv) {
    Topology *t = (Topology *)p;
    if (!t) return 1;
    std::memcpy(sizes, t->lsizes.data(), t->lsizes.size() * 4);
    std::memcpy(offsets, t->loffsets.data(), t->loffsets.size() * 4);
    std::memcpy(indices, t->lidx.data(), t->lidx.size() * 4);
    std::memcpy(w, t->lw[0].data(), t->lw[0].size() * 4);
    std::memcpy(du, t->lw[1].data(), t->lw[1].size() * 4);
    std::memcpy(dv, t->lw[2].data(), t->lw[2].size() * 4);
    return 0;
}

}  // extern "C"
