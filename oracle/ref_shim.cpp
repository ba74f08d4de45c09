// C entry points over the reference's own Far / Osd CPU code.
//
// TEST INFRASTRUCTURE ONLY.  This file is compiled together with the reference sources by
// oracle/Makefile into oracle/_ref/libosdref.so.  It is used to (a) generate the golden
// fixtures under tests/golden/, (b) pin the C restatement in osd_oracle.c against the
// reference itself, and (c) time the reference CpuEvaluator / OmpEvaluator where the
// reference is available.  Nothing in the product links or loads it.
//
// Every call below forwards to the public reference API named in its comment.

#include <opensubdiv/far/topologyDescriptor.h>
#include <opensubdiv/far/stencilTableFactory.h>
#include <opensubdiv/far/patchTableFactory.h>
#include <opensubdiv/far/patchMap.h>
#include <opensubdiv/far/ptexIndices.h>
#include <opensubdiv/osd/cpuEvaluator.h>
#include <opensubdiv/osd/ompEvaluator.h>
#include <opensubdiv/osd/cpuPatchTable.h>
#include <opensubdiv/osd/bufferDescriptor.h>
#include <opensubdiv/bfr/parameterization.h>
#include <opensubdiv/bfr/tessellation.h>
#include <opensubdiv/bfr/refinerSurfaceFactory.h>
#include <opensubdiv/bfr/surface.h>
#include <opensubdiv/bfr/surfaceFactoryCache.h>

#include <opensubdiv_gb300/far/gb300StencilTableFactory.h>

#include <cstring>
#include <mutex>
#include <shared_mutex>
#include <vector>

using namespace OpenSubdiv;

namespace {

struct Refiner {
    Far::TopologyRefiner *r = nullptr;
};

struct Stencils {
    int useDouble = 0;
    int limit = 0;
    Far::StencilTableReal<float> const *f = nullptr;
    Far::StencilTableReal<double> const *d = nullptr;
    Far::LimitStencilTableReal<float> const *lf = nullptr;
    Far::LimitStencilTableReal<double> const *ld = nullptr;
};

struct Patches {
    Far::PatchTable const *pt = nullptr;
    Osd::CpuPatchTable *cpu = nullptr;
    Far::PatchMap *map = nullptr;
    Far::StencilTable const *all = nullptr;   // refined + local point stencils (float)
};

template <class T>
void copyVec(std::vector<T> const &v, T *out) {
    if (out && !v.empty()) std::memcpy(out, v.data(), v.size() * sizeof(T));
}

// Weight vectors of a Far table may hold more entries than it has control indices; only the
// first nnz (= number of control indices) are meaningful.
template <class T>
void copyN(std::vector<T> const &v, T *out, size_t n) {
    if (out && !v.empty()) std::memcpy(out, v.data(), (v.size() < n ? v.size() : n) * sizeof(T));
}

}  // namespace

extern "C" {

// Far::TopologyRefinerFactory<TopologyDescriptor>::Create (far/topologyRefinerFactory.h)
// scheme: 0 bilinear, 1 catmark, 2 loop.  boundary: Sdc::Options::VtxBoundaryInterpolation.
void *ref_refiner_create(int scheme, int nverts, int nfaces, const int *vertsPerFace,
                         const int *faceVerts, int ncreases, const int *creaseVerts,
                         const float *creaseSharp, int ncorners, const int *cornerVerts,
                         const float *cornerSharp, int boundary) {
    Far::TopologyDescriptor desc;
    desc.numVertices = nverts;
    desc.numFaces = nfaces;
    desc.numVertsPerFace = vertsPerFace;
    desc.vertIndicesPerFace = faceVerts;
    desc.numCreases = ncreases;
    desc.creaseVertexIndexPairs = creaseVerts;
    desc.creaseWeights = creaseSharp;
    desc.numCorners = ncorners;
    desc.cornerVertexIndices = cornerVerts;
    desc.cornerWeights = cornerSharp;

    Sdc::SchemeType type = scheme == 0 ? Sdc::SCHEME_BILINEAR
                         : scheme == 1 ? Sdc::SCHEME_CATMARK : Sdc::SCHEME_LOOP;
    Sdc::Options opts;
    opts.SetVtxBoundaryInterpolation((Sdc::Options::VtxBoundaryInterpolation)boundary);
    Far::TopologyRefinerFactory<Far::TopologyDescriptor>::Options fo(type, opts);
    Refiner *h = new Refiner;
    h->r = Far::TopologyRefinerFactory<Far::TopologyDescriptor>::Create(desc, fo);
    if (!h->r) { delete h; return nullptr; }
    return h;
}

// As ref_refiner_create, plus one face-varying channel (Far::TopologyDescriptor::FVarChannel,
// far/topologyDescriptor.h:73-82): fvarIndices holds one value index per face-vertex.
void *ref_refiner_create_fvar(int scheme, int nverts, int nfaces, const int *vertsPerFace,
                              const int *faceVerts, int ncreases, const int *creaseVerts,
                              const float *creaseSharp, int boundary, int fvarNumValues,
                              const int *fvarIndices, int fvarLinear) {
    Far::TopologyDescriptor desc;
    desc.numVertices = nverts;
    desc.numFaces = nfaces;
    desc.numVertsPerFace = vertsPerFace;
    desc.vertIndicesPerFace = faceVerts;
    desc.numCreases = ncreases;
    desc.creaseVertexIndexPairs = creaseVerts;
    desc.creaseWeights = creaseSharp;
    Far::TopologyDescriptor::FVarChannel ch;
    ch.numValues = fvarNumValues;
    ch.valueIndices = fvarIndices;
    desc.numFVarChannels = 1;
    desc.fvarChannels = &ch;
    Sdc::SchemeType type = scheme == 0 ? Sdc::SCHEME_BILINEAR
                         : scheme == 1 ? Sdc::SCHEME_CATMARK : Sdc::SCHEME_LOOP;
    Sdc::Options opts;
    opts.SetVtxBoundaryInterpolation((Sdc::Options::VtxBoundaryInterpolation)boundary);
    opts.SetFVarLinearInterpolation(fvarLinear ? Sdc::Options::FVAR_LINEAR_ALL
                                               : Sdc::Options::FVAR_LINEAR_NONE);
    Far::TopologyRefinerFactory<Far::TopologyDescriptor>::Options fo(type, opts);
    Refiner *h = new Refiner;
    h->r = Far::TopologyRefinerFactory<Far::TopologyDescriptor>::Create(desc, fo);
    if (!h->r) { delete h; return nullptr; }
    return h;
}

void ref_refiner_destroy(void *p) {
    Refiner *h = (Refiner *)p;
    if (!h) return;
    delete h->r;
    delete h;
}

// Far::TopologyRefiner::RefineUniform (far/topologyRefiner.h:146)
void ref_refine_uniform(void *p, int level) {
    Far::TopologyRefiner::UniformOptions o(level);
    ((Refiner *)p)->r->RefineUniform(o);
}

// Far::TopologyRefiner::RefineAdaptive (far/topologyRefiner.h:192), options chosen the way
// PatchTableFactory::Options::GetRefineAdaptiveOptions derives them.
void ref_refine_adaptive(void *p, int isolation, int useSingleCrease, int useInfSharp) {
    Far::PatchTableFactory::Options po(isolation);
    po.useSingleCreasePatch = useSingleCrease;
    po.useInfSharpPatch = useInfSharp;
    if (((Refiner *)p)->r->GetNumFVarChannels() > 0) {
        // non-linear face-varying patches need isolation of the face-varying topology
        // (far/patchTableFactory.h:105-106)
        po.generateFVarTables = true;
        po.generateFVarLegacyLinearPatches = false;
    }
    ((Refiner *)p)->r->RefineAdaptive(po.GetRefineAdaptiveOptions());
}

// Adaptive refinement with a secondary (smooth feature) level, as the reference's Bfr
// regression builds the Far tables it compares Bfr::Surface against
// (regression/bfr_evaluate/farPatchEvaluator.cpp:52-78).
void ref_refine_adaptive_levels(void *p, int primary, int secondary, int useInfSharp) {
    Far::PatchTableFactory::Options po(primary);
    po.useInfSharpPatch = useInfSharp;
    if (((Refiner *)p)->r->GetNumFVarChannels() > 0) {
        // non-linear face-varying patches: isolate the face-varying topology too
        po.generateFVarTables = true;
        po.generateFVarLegacyLinearPatches = false;
    }
    Far::TopologyRefiner::AdaptiveOptions ro = po.GetRefineAdaptiveOptions();
    ro.SetIsolationLevel(primary);
    ro.SetSecondaryLevel(secondary);
    ((Refiner *)p)->r->RefineAdaptive(ro);
}

int ref_num_vertices_total(void *p) { return ((Refiner *)p)->r->GetNumVerticesTotal(); }
int ref_level_num_vertices(void *p, int level) {
    return ((Refiner *)p)->r->GetLevel(level).GetNumVertices();
}
int ref_max_level(void *p) { return ((Refiner *)p)->r->GetMaxLevel(); }
int ref_num_ptex_faces(void *p) {
    Far::PtexIndices pi(*((Refiner *)p)->r);
    return pi.GetNumFaces();
}
// Far::PtexIndices::GetFaceId (far/ptexIndices.cpp)
void ref_ptex_face_ids(void *p, int *out) {
    Far::TopologyRefiner *r = ((Refiner *)p)->r;
    Far::PtexIndices pi(*r);
    int n = r->GetLevel(0).GetNumFaces();
    for (int i = 0; i < n; ++i) out[i] = pi.GetFaceId(i);
}

// Far::StencilTableFactoryReal<REAL>::Create (far/stencilTableFactory.cpp:78-151)
void *ref_stencils_create(void *p, int useDouble, int genIntermediate, int factorize,
                          int genCtrl, int maxLevel) {
    Far::TopologyRefiner *r = ((Refiner *)p)->r;
    Stencils *s = new Stencils;
    s->useDouble = useDouble;
    if (useDouble) {
        Far::StencilTableFactoryReal<double>::Options o;
        o.generateIntermediateLevels = genIntermediate;
        o.factorizeIntermediateLevels = factorize;
        o.generateControlVerts = genCtrl;
        o.generateOffsets = true;
        o.maxLevel = maxLevel;
        s->d = Far::StencilTableFactoryReal<double>::Create(*r, o);
    } else {
        Far::StencilTableFactoryReal<float>::Options o;
        o.generateIntermediateLevels = genIntermediate;
        o.factorizeIntermediateLevels = factorize;
        o.generateControlVerts = genCtrl;
        o.generateOffsets = true;
        o.maxLevel = maxLevel;
        s->f = Far::StencilTableFactoryReal<float>::Create(*r, o);
    }
    return s;
}

// Far::LimitStencilTableFactoryReal<REAL>::Create (far/stencilTableFactory.cpp:411-662)
// Locations are given one per (ptex face, s, t) triple.
void *ref_limit_stencils_create(void *p, int useDouble, int n, const int *ptex,
                                const double *su, const double *tv, int d1, int d2) {
    Far::TopologyRefiner *r = ((Refiner *)p)->r;
    Stencils *s = new Stencils;
    s->useDouble = useDouble;
    s->limit = 1;
    if (useDouble) {
        typedef Far::LimitStencilTableFactoryReal<double> F;
        F::LocationArrayVec locs(n);
        for (int i = 0; i < n; ++i) {
            locs[i].ptexIdx = ptex[i];
            locs[i].numLocations = 1;
            locs[i].s = su + i;
            locs[i].t = tv + i;
        }
        F::Options o;
        o.generate1stDerivatives = d1;
        o.generate2ndDerivatives = d2;
        s->ld = F::Create(*r, locs, nullptr, nullptr, o);
    } else {
        typedef Far::LimitStencilTableFactoryReal<float> F;
        std::vector<float> sf(su, su + n), tf(tv, tv + n);
        F::LocationArrayVec locs(n);
        for (int i = 0; i < n; ++i) {
            locs[i].ptexIdx = ptex[i];
            locs[i].numLocations = 1;
            locs[i].s = sf.data() + i;
            locs[i].t = tf.data() + i;
        }
        F::Options o;
        o.generate1stDerivatives = d1;
        o.generate2ndDerivatives = d2;
        s->lf = F::Create(*r, locs, nullptr, nullptr, o);
    }
    return s;
}

// Far::StencilTableFactory::Create (float) in any interpolation mode.
void *ref_stencils_create_mode(void *p, int mode, int channel, int genIntermediate,
                               int genCtrl, int maxLevel) {
    Far::TopologyRefiner *r = ((Refiner *)p)->r;
    Stencils *s = new Stencils;
    Far::StencilTableFactory::Options o;
    o.interpolationMode = mode;
    o.fvarChannel = channel;
    o.generateIntermediateLevels = genIntermediate;
    o.generateControlVerts = genCtrl;
    o.generateOffsets = true;
    o.maxLevel = maxLevel;
    s->f = Far::StencilTableFactory::Create(*r, o);
    return s;
}

// The per-level masks the GPU factory consumes, recorded from Far::PrimvarRefiner by the
// product's own recorder (include/opensubdiv_gb300/far/gb300StencilTableFactory.h).
struct MaskSet {
    std::vector<Osd::GB300LevelMasks> levels;
    int numControl = 0;
};

void *ref_masks_record(void *p, int mode, int channel, int maxLevel) {
    Far::TopologyRefiner *r = ((Refiner *)p)->r;
    Far::StencilTableFactory::Options o;
    o.interpolationMode = mode;
    o.fvarChannel = channel;
    o.maxLevel = maxLevel;
    MaskSet *m = new MaskSet;
    if (!Osd::GB300StencilTableFactory::RecordMasks(*r, o, m->levels, &m->numControl)) {
        delete m;
        return nullptr;
    }
    return m;
}
int ref_masks_num_levels(void *p) { return (int)((MaskSet *)p)->levels.size(); }
int ref_masks_num_control(void *p) { return ((MaskSet *)p)->numControl; }
void ref_masks_level_counts(void *p, int level, int *numRows, long *nnz) {
    Osd::GB300LevelMasks const &L = ((MaskSet *)p)->levels[level];
    *numRows = L.numRows;
    *nnz = (long)L.sources.size();
}
void ref_masks_level_copy(void *p, int level, int64_t *offsets, int *sources, float *weights) {
    Osd::GB300LevelMasks const &L = ((MaskSet *)p)->levels[level];
    copyVec(L.offsets, offsets);
    copyVec(L.sources, sources);
    copyVec(L.weights, weights);
}
void ref_masks_destroy(void *p) { delete (MaskSet *)p; }

// Everything the GPU limit-stencil factory consumes and produces for one refiner and set of
// locations, recorded with the product's header (GB300LimitStencilTableFactory's helpers), plus
// the table Far::LimitStencilTableFactory builds itself.  Arrays are exported by key.
struct LimitRecord {
    std::vector<int> levelRows, levelSrc, locSrc, localSrc, farSizes, farOffsets, farIndices;
    std::vector<int64_t> levelOff, locOff, localOff;
    std::vector<float> levelW, localW, locW[6], farW[6];
    int numControl = 0, numChannels = 0, spliced = 0, cvIntermediate = 0;
};

void *ref_limit_record(void *p, int mode, int channel, int n, const int *ptex, const float *su,
                       const float *tv, int d1, int d2) {
    Far::TopologyRefiner *r = ((Refiner *)p)->r;
    typedef Osd::GB300LimitStencilTableFactory LF;
    LF::Options o;
    o.interpolationMode = mode;
    o.fvarChannel = channel;
    o.generate1stDerivatives = d1;
    o.generate2ndDerivatives = d2;
    LimitRecord *rec = new LimitRecord;
    LF::LocationArrayVec locs(n);
    for (int i = 0; i < n; ++i) {
        locs[i].ptexIdx = ptex[i];
        locs[i].numLocations = 1;
        locs[i].s = su + i;
        locs[i].t = tv + i;
    }
    // refined-vertex stencil masks
    Osd::GB300StencilTableFactory::Options co = LF::CvOptions(*r, o);
    rec->cvIntermediate = co.generateIntermediateLevels;
    std::vector<Osd::GB300LevelMasks> levels;
    if (!Osd::GB300StencilTableFactory::RecordMasks(*r, co, levels, &rec->numControl)) {
        delete rec;
        return nullptr;
    }
    for (auto const &L : levels) {
        rec->levelRows.push_back(L.numRows);
        rec->levelOff.insert(rec->levelOff.end(), L.offsets.begin(), L.offsets.end());
        rec->levelSrc.insert(rec->levelSrc.end(), L.sources.begin(), L.sources.end());
        rec->levelW.insert(rec->levelW.end(), L.weights.begin(), L.weights.end());
    }
    Far::PatchTable const *pt = LF::CreatePatchTable(*r, o);
    const bool fvar = mode == Far::LimitStencilTableFactory::INTERPOLATE_FACE_VARYING;
    const int nRefined = r->IsUniform()
        ? (fvar ? r->GetLevel(r->GetMaxLevel()).GetNumFVarValues(channel)
                : r->GetLevel(r->GetMaxLevel()).GetNumVertices())
        : (fvar ? r->GetNumFVarValuesTotal(channel) : r->GetNumVerticesTotal());
    int cvCount = rec->numControl;
    for (size_t l = co.generateIntermediateLevels ? 0 : (levels.empty() ? 0 : levels.size() - 1);
         l < levels.size(); ++l)
        cvCount += levels[l].numRows;
    rec->spliced = cvCount == nRefined &&
                   LF::LocalPointMasks(*pt, o, rec->localOff, rec->localSrc, rec->localW);
    rec->numChannels = LF::LocationMasks(*r, *pt, locs, o, rec->locOff, rec->locSrc, rec->locW);
    delete pt;
    // the reference's own table
    Far::LimitStencilTable const *far = Far::LimitStencilTableFactory::Create(*r, locs, nullptr,
                                                                             nullptr, o);
    if (far) {
        const size_t nnz = far->GetControlIndices().size();
        rec->farSizes = far->GetSizes();
        rec->farOffsets = far->GetOffsets();
        rec->farIndices = far->GetControlIndices();
        std::vector<float> const *fw[6] = {&far->GetWeights(), &far->GetDuWeights(),
                                           &far->GetDvWeights(), &far->GetDuuWeights(),
                                           &far->GetDuvWeights(), &far->GetDvvWeights()};
        for (int c = 0; c < rec->numChannels; ++c)
            rec->farW[c].assign(fw[c]->begin(), fw[c]->begin() + std::min(nnz, fw[c]->size()));
        delete far;
    }
    return rec;
}

// keys: 0 levelRows 1 levelOff 2 levelSrc 3 levelW 4 localOff 5 localSrc 6 localW 7 locOff
// 8 locSrc 9..14 locW[c] 15 farSizes 16 farOffsets 17 farIndices 18..23 farW[c]
static void limit_array(LimitRecord *r, int key, const void **ptr, long *n, int *esize) {
    *ptr = nullptr;
    *n = 0;
    *esize = 4;
    auto set = [&](auto const &v) {
        *ptr = v.data();
        *n = (long)v.size();
        *esize = (int)sizeof(v[0]);
    };
    if (key == 0) set(r->levelRows);
    else if (key == 1) set(r->levelOff);
    else if (key == 2) set(r->levelSrc);
    else if (key == 3) set(r->levelW);
    else if (key == 4) set(r->localOff);
    else if (key == 5) set(r->localSrc);
    else if (key == 6) set(r->localW);
    else if (key == 7) set(r->locOff);
    else if (key == 8) set(r->locSrc);
    else if (key >= 9 && key < 15) set(r->locW[key - 9]);
    else if (key == 15) set(r->farSizes);
    else if (key == 16) set(r->farOffsets);
    else if (key == 17) set(r->farIndices);
    else if (key >= 18 && key < 24) set(r->farW[key - 18]);
}
long ref_limit_array_size(void *p, int key) {
    const void *ptr;
    long n;
    int es;
    limit_array((LimitRecord *)p, key, &ptr, &n, &es);
    return n;
}
void ref_limit_array_copy(void *p, int key, void *dst) {
    const void *ptr;
    long n;
    int es;
    limit_array((LimitRecord *)p, key, &ptr, &n, &es);
    if (n) std::memcpy(dst, ptr, (size_t)n * es);
}
void ref_limit_info(void *p, int *info) {
    LimitRecord *r = (LimitRecord *)p;
    info[0] = r->numControl;
    info[1] = r->numChannels;
    info[2] = r->spliced;
    info[3] = r->cvIntermediate;
}
void ref_limit_destroy(void *p) { delete (LimitRecord *)p; }

void ref_stencils_destroy(void *p) {
    Stencils *s = (Stencils *)p;
    if (!s) return;
    delete s->f; delete s->d; delete s->lf; delete s->ld;
    delete s;
}

static Far::StencilTableReal<float> const *asF(Stencils *s) {
    return s->limit ? s->lf : s->f;
}
static Far::StencilTableReal<double> const *asD(Stencils *s) {
    return s->limit ? s->ld : s->d;
}

int ref_stencils_num(void *p) {
    Stencils *s = (Stencils *)p;
    if (s->useDouble) return asD(s) ? asD(s)->GetNumStencils() : 0;
    return asF(s) ? asF(s)->GetNumStencils() : 0;
}
long ref_stencils_nnz(void *p) {
    Stencils *s = (Stencils *)p;
    if (s->useDouble) return asD(s) ? (long)asD(s)->GetControlIndices().size() : 0;
    return asF(s) ? (long)asF(s)->GetControlIndices().size() : 0;
}
int ref_stencils_num_control(void *p) {
    Stencils *s = (Stencils *)p;
    if (s->useDouble) return asD(s) ? asD(s)->GetNumControlVertices() : 0;
    return asF(s) ? asF(s)->GetNumControlVertices() : 0;
}

// Copies sizes/offsets/indices and the weight arrays (float or double per the table).
// w[0..5] = weights, du, dv, duu, duv, dvv; entries may be NULL or absent (limit only).
void ref_stencils_copy(void *p, int *sizes, int *offsets, int *indices, void **w) {
    Stencils *s = (Stencils *)p;
    if (s->useDouble) {
        auto t = asD(s);
        size_t nnz = t->GetControlIndices().size();
        copyVec(t->GetSizes(), sizes);
        copyVec(t->GetOffsets(), offsets);
        copyVec(t->GetControlIndices(), indices);
        copyN(t->GetWeights(), (double *)w[0], nnz);
        if (s->limit) {
            copyN(s->ld->GetDuWeights(), (double *)w[1], nnz);
            copyN(s->ld->GetDvWeights(), (double *)w[2], nnz);
            copyN(s->ld->GetDuuWeights(), (double *)w[3], nnz);
            copyN(s->ld->GetDuvWeights(), (double *)w[4], nnz);
            copyN(s->ld->GetDvvWeights(), (double *)w[5], nnz);
        }
    } else {
        auto t = asF(s);
        size_t nnz = t->GetControlIndices().size();
        copyVec(t->GetSizes(), sizes);
        copyVec(t->GetOffsets(), offsets);
        copyVec(t->GetControlIndices(), indices);
        copyN(t->GetWeights(), (float *)w[0], nnz);
        if (s->limit) {
            copyN(s->lf->GetDuWeights(), (float *)w[1], nnz);
            copyN(s->lf->GetDvWeights(), (float *)w[2], nnz);
            copyN(s->lf->GetDuuWeights(), (float *)w[3], nnz);
            copyN(s->lf->GetDuvWeights(), (float *)w[4], nnz);
            copyN(s->lf->GetDvvWeights(), (float *)w[5], nnz);
        }
    }
}

// Osd::CpuEvaluator::EvalStencils, all three overloads (osd/cpuEvaluator.cpp:37-125).
// dsts/dstDescs/wts hold 1, 3 or 6 outputs.  Descriptors are (offset, length, stride).
int ref_cpu_eval_stencils(const float *src, const int *srcDesc, int nout, float **dsts,
                          const int *dstDescs, const int *sizes, const int *offsets,
                          const int *indices, const float **wts, int start, int end,
                          int useOmp) {
    Osd::BufferDescriptor sd(srcDesc[0], srcDesc[1], srcDesc[2]);
    Osd::BufferDescriptor d[6];
    for (int i = 0; i < nout; ++i)
        d[i] = Osd::BufferDescriptor(dstDescs[3 * i], dstDescs[3 * i + 1], dstDescs[3 * i + 2]);
    bool ok = false;
    if (nout == 1) {
        ok = useOmp ? Osd::OmpEvaluator::EvalStencils(src, sd, dsts[0], d[0], sizes, offsets,
                                                      indices, wts[0], start, end)
                    : Osd::CpuEvaluator::EvalStencils(src, sd, dsts[0], d[0], sizes, offsets,
                                                      indices, wts[0], start, end);
    } else if (nout == 3) {
        ok = useOmp ? Osd::OmpEvaluator::EvalStencils(src, sd, dsts[0], d[0], dsts[1], d[1],
                                                      dsts[2], d[2], sizes, offsets, indices,
                                                      wts[0], wts[1], wts[2], start, end)
                    : Osd::CpuEvaluator::EvalStencils(src, sd, dsts[0], d[0], dsts[1], d[1],
                                                      dsts[2], d[2], sizes, offsets, indices,
                                                      wts[0], wts[1], wts[2], start, end);
    } else if (nout == 6) {
        ok = useOmp ? Osd::OmpEvaluator::EvalStencils(
                          src, sd, dsts[0], d[0], dsts[1], d[1], dsts[2], d[2], dsts[3], d[3],
                          dsts[4], d[4], dsts[5], d[5], sizes, offsets, indices, wts[0], wts[1],
                          wts[2], wts[3], wts[4], wts[5], start, end)
                    : Osd::CpuEvaluator::EvalStencils(
                          src, sd, dsts[0], d[0], dsts[1], d[1], dsts[2], d[2], dsts[3], d[3],
                          dsts[4], d[4], dsts[5], d[5], sizes, offsets, indices, wts[0], wts[1],
                          wts[2], wts[3], wts[4], wts[5], start, end);
    }
    return ok ? 1 : 0;
}

void ref_omp_set_threads(int n) { Osd::OmpEvaluator::SetNumThreads(n); }

// Far::PatchTableFactory::Create (far/patchTableFactory.h:175) on an already refined
// refiner, then Osd::CpuPatchTable (osd/cpuPatchTable.cpp:35-158) to flatten it and
// Far::PatchMap (far/patchMap.cpp) for lookups.  A stencil table covering refined and
// local points is built the way examples/glEvalLimit does (StencilTableFactory with
// intermediate levels + AppendLocalPointStencilTable).
void *ref_patches_create_ex(void *p, int endcap, int maxIsolation, int useSingleCrease,
                            int useInfSharp, int shareEndCapPoints, int legacySharpCorners) {
    Far::TopologyRefiner *r = ((Refiner *)p)->r;
    Far::PatchTableFactory::Options po(maxIsolation);
    po.SetEndCapType((Far::PatchTableFactory::Options::EndCapType)endcap);
    po.useSingleCreasePatch = useSingleCrease;
    po.useInfSharpPatch = useInfSharp;
    po.shareEndCapPatchPoints = shareEndCapPoints;
    po.generateLegacySharpCornerPatches = legacySharpCorners;
    if (r->GetNumFVarChannels() > 0) {
        po.generateFVarTables = true;
        po.generateFVarLegacyLinearPatches = !r->IsUniform() ? false : true;
    }
    Patches *h = new Patches;
    h->pt = Far::PatchTableFactory::Create(*r, po);
    h->cpu = Osd::CpuPatchTable::Create(h->pt, nullptr);
    h->map = new Far::PatchMap(*h->pt);

    Far::StencilTableFactory::Options so;
    so.generateOffsets = true;
    // Patch indices count vertices of every level after the base (uniform tables offset the
    // last level by all earlier levels, far/patchTableFactory.cpp:813-814), so the source
    // buffer holds all levels.
    so.generateIntermediateLevels = true;
    Far::StencilTable const *st = Far::StencilTableFactory::Create(*r, so);
    Far::StencilTable const *local = h->pt->GetLocalPointStencilTable();
    if (local) {
        Far::StencilTable const *all =
            Far::StencilTableFactory::AppendLocalPointStencilTable(*r, st, local);
        delete st;
        st = all;
    }
    h->all = st;
    return h;
}

void *ref_patches_create(void *p, int endcap, int maxIsolation, int useSingleCrease,
                         int useInfSharp, int shareEndCapPoints) {
    return ref_patches_create_ex(p, endcap, maxIsolation, useSingleCrease, useInfSharp,
                                 shareEndCapPoints, 1);
}

void ref_patches_destroy(void *p) {
    Patches *h = (Patches *)p;
    if (!h) return;
    delete h->map;
    delete h->cpu;
    delete h->all;
    delete h->pt;
    delete h;
}

// counts[0..5] = numArrays, indexSize, paramSize, numLocalPoints, stencils(all), nnz(all)
void ref_patches_counts(void *p, long *counts) {
    Patches *h = (Patches *)p;
    counts[0] = h->pt->GetNumPatchArrays();
    counts[1] = (long)h->cpu->GetPatchIndexSize();
    counts[2] = (long)h->cpu->GetPatchParamSize();
    counts[3] = h->pt->GetNumLocalPoints();
    counts[4] = h->all ? h->all->GetNumStencils() : 0;
    counts[5] = h->all ? (long)h->all->GetControlIndices().size() : 0;
}

// arrays: 6 ints per array (Osd::PatchArray, osd/types.h:66-125);
// params: 3 x 32-bit per patch (Osd::PatchParam field0, field1, sharpness bits)
void ref_patches_copy(void *p, int *arrays, int *indices, int *params) {
    Patches *h = (Patches *)p;
    int na = h->pt->GetNumPatchArrays();
    std::memcpy(arrays, h->cpu->GetPatchArrayBuffer(), sizeof(Osd::PatchArray) * na);
    std::memcpy(indices, h->cpu->GetPatchIndexBuffer(), sizeof(int) * h->cpu->GetPatchIndexSize());
    std::memcpy(params, h->cpu->GetPatchParamBuffer(),
                sizeof(Osd::PatchParam) * h->cpu->GetPatchParamSize());
}

void ref_patches_copy_stencils(void *p, int *sizes, int *offsets, int *indices, float *w) {
    Patches *h = (Patches *)p;
    copyVec(h->all->GetSizes(), sizes);
    copyVec(h->all->GetOffsets(), offsets);
    copyVec(h->all->GetControlIndices(), indices);
    copyN(h->all->GetWeights(), w, h->all->GetControlIndices().size());
}

// Varying tables of Osd::CpuPatchTable (osd/cpuPatchTable.cpp:75-86): counts[0] = arrays,
// counts[1] = indices; arrays/indices may be NULL to query the counts.
void ref_patches_varying(void *p, long *counts, int *arrays, int *indices) {
    Patches *h = (Patches *)p;
    counts[0] = h->pt->GetNumPatchArrays();
    counts[1] = (long)h->cpu->GetVaryingPatchIndexSize();
    if (arrays)
        std::memcpy(arrays, h->cpu->GetVaryingPatchArrayBuffer(), counts[0] * 6 * sizeof(int));
    if (indices)
        std::memcpy(indices, h->cpu->GetVaryingPatchIndexBuffer(), counts[1] * sizeof(int));
}

// Face-varying tables of one channel (osd/cpuPatchTable.cpp:88-114): counts[0] = channels,
// counts[1] = arrays, counts[2] = indices, counts[3] = params (3 x 32-bit each).
void ref_patches_fvar(void *p, int channel, long *counts, int *arrays, int *indices,
                      int *params) {
    Patches *h = (Patches *)p;
    counts[0] = h->cpu->GetNumFVarChannels();
    if (channel >= counts[0]) { counts[1] = counts[2] = counts[3] = 0; return; }
    counts[1] = h->pt->GetNumPatchArrays();
    counts[2] = (long)h->cpu->GetFVarPatchIndexSize(channel);
    counts[3] = (long)h->cpu->GetFVarPatchParamSize(channel);
    if (arrays)
        std::memcpy(arrays, h->cpu->GetFVarPatchArrayBuffer(channel),
                    counts[1] * 6 * sizeof(int));
    if (indices)
        std::memcpy(indices, h->cpu->GetFVarPatchIndexBuffer(channel), counts[2] * sizeof(int));
    if (params)
        std::memcpy(params, h->cpu->GetFVarPatchParamBuffer(channel), counts[3] * 12);
}

// Face-varying values of channel `channel` for every refinement level and the channel's local
// points, as one stencil table over the channel's base values: Far::StencilTableFactory in
// INTERPOLATE_FACE_VARYING mode with intermediate levels, plus
// AppendLocalPointStencilTableFaceVarying (far/stencilTableFactory.h:334-346) with the patch
// table's face-varying local-point stencils.  counts[0] = stencils, counts[1] = entries; the
// arrays may be NULL to query the counts.
void ref_patches_fvar_stencils(void *refiner, void *p, int channel, long *counts, int *sizes,
                               int *offsets, int *indices, float *w) {
    Far::TopologyRefiner *r = ((Refiner *)refiner)->r;
    Patches *h = (Patches *)p;
    Far::StencilTableFactory::Options so;
    so.interpolationMode = Far::StencilTableFactory::INTERPOLATE_FACE_VARYING;
    so.fvarChannel = channel;
    so.generateOffsets = true;
    so.generateIntermediateLevels = true;
    Far::StencilTable const *st = Far::StencilTableFactory::Create(*r, so);
    Far::StencilTable const *local = h->pt->GetLocalPointFaceVaryingStencilTable(channel);
    if (local) {
        Far::StencilTable const *all = Far::StencilTableFactory::
            AppendLocalPointStencilTableFaceVarying(*r, st, local, channel);
        delete st;
        st = all;
    }
    counts[0] = st->GetNumStencils();
    counts[1] = (long)st->GetControlIndices().size();
    if (sizes) {
        copyVec(st->GetSizes(), sizes);
        copyVec(st->GetOffsets(), offsets);
        copyVec(st->GetControlIndices(), indices);
        copyN(st->GetWeights(), w, st->GetControlIndices().size());
    }
    delete st;
}

// Far::PatchMap::FindPatch (far/patchMap.h:192-231).  handles: 3 ints per query
// (arrayIndex, patchIndex, vertIndex); found[i] = 0 when FindPatch returns NULL.
void ref_find_patches(void *p, int n, const int *faces, const double *u, const double *v,
                      int *handles, int *found) {
    Patches *h = (Patches *)p;
    for (int i = 0; i < n; ++i) {
        Far::PatchMap::Handle const *hd = h->map->FindPatch(faces[i], u[i], v[i]);
        found[i] = hd ? 1 : 0;
        handles[3 * i + 0] = hd ? hd->arrayIndex : -1;
        handles[3 * i + 1] = hd ? hd->patchIndex : -1;
        handles[3 * i + 2] = hd ? hd->vertIndex : -1;
    }
}

// Osd::CpuEvaluator::EvalPatches, all three overloads (osd/cpuEvaluator.cpp:157-381).
// coords: 5 x 32-bit per point (Osd::PatchCoord).  nout = 1, 3 or 6.
int ref_cpu_eval_patches(const float *src, const int *srcDesc, int nout, float **dsts,
                         const int *dstDescs, int ncoords, const void *coords,
                         const void *arrays, const int *indices, const void *params) {
    Osd::BufferDescriptor sd(srcDesc[0], srcDesc[1], srcDesc[2]);
    Osd::BufferDescriptor d[6];
    for (int i = 0; i < nout; ++i)
        d[i] = Osd::BufferDescriptor(dstDescs[3 * i], dstDescs[3 * i + 1], dstDescs[3 * i + 2]);
    const Osd::PatchCoord *pc = (const Osd::PatchCoord *)coords;
    const Osd::PatchArray *pa = (const Osd::PatchArray *)arrays;
    const Osd::PatchParam *pp = (const Osd::PatchParam *)params;
    bool ok = false;
    if (nout == 1)
        ok = Osd::CpuEvaluator::EvalPatches(src, sd, dsts[0], d[0], ncoords, pc, pa, indices, pp);
    else if (nout == 3)
        ok = Osd::CpuEvaluator::EvalPatches(src, sd, dsts[0], d[0], dsts[1], d[1], dsts[2], d[2],
                                            ncoords, pc, pa, indices, pp);
    else if (nout == 6)
        ok = Osd::CpuEvaluator::EvalPatches(src, sd, dsts[0], d[0], dsts[1], d[1], dsts[2], d[2],
                                            dsts[3], d[3], dsts[4], d[4], dsts[5], d[5],
                                            ncoords, pc, pa, indices, pp);
    return ok ? 1 : 0;
}

// Far::PatchTable::EvaluateBasis<double> (far/patchTable.cpp:579-625) and a double
// accumulation of the same (float) source points: the FP64 oracle for EvalPatches.
// out: 6 outputs x length doubles per point (P, du, dv, duu, duv, dvv).
void ref_eval_patches_fp64(void *p, const float *src, int length, int srcStride, int n,
                           const int *handles, const double *s, const double *t, double *out) {
    Patches *h = (Patches *)p;
    double w[6][20];
    for (int i = 0; i < n; ++i) {
        Far::PatchTable::PatchHandle hd;
        hd.arrayIndex = handles[3 * i];
        hd.patchIndex = handles[3 * i + 1];
        hd.vertIndex = handles[3 * i + 2];
        h->pt->EvaluateBasis<double>(hd, s[i], t[i], w[0], w[1], w[2], w[3], w[4], w[5]);
        Far::ConstIndexArray cvs = h->pt->GetPatchVertices(hd);
        double *o = out + (size_t)i * 6 * length;
        for (int k = 0; k < 6 * length; ++k) o[k] = 0.0;
        for (int j = 0; j < cvs.size(); ++j) {
            const float *sv = src + (size_t)cvs[j] * srcStride;
            for (int k = 0; k < 6; ++k)
                for (int e = 0; e < length; ++e) o[k * length + e] += w[k][j] * (double)sv[e];
        }
    }
}

// ---- Bfr ------------------------------------------------------------------------------

static Sdc::SchemeType schemeOfRegularFaceSize(int regFaceSize) {
    return regFaceSize == 3 ? Sdc::SCHEME_LOOP : Sdc::SCHEME_CATMARK;
}

static Bfr::Tessellation::Options tessOptions(int facetSize, int preserveQuads) {
    Bfr::Tessellation::Options o;
    o.SetFacetSize(facetSize);
    o.PreserveQuads(preserveQuads != 0);
    return o;
}

// Bfr::Tessellation (bfr/tessellation.h:142-200): counts = {coords, facets, boundary coords,
// uniform}; returns IsValid().
int ref_bfr_tess_counts(int regFaceSize, int N, int numRates, const int *rates, int facetSize,
                        int preserveQuads, int *counts) {
    Bfr::Parameterization param(schemeOfRegularFaceSize(regFaceSize), N);
    Bfr::Tessellation t(param, numRates, rates, tessOptions(facetSize, preserveQuads));
    counts[0] = t.IsValid() ? t.GetNumCoords() : 0;
    counts[1] = t.IsValid() ? t.GetNumFacets() : 0;
    counts[2] = t.IsValid() ? t.GetNumBoundaryCoords() : 0;
    counts[3] = t.IsValid() ? (int)t.IsUniform() : 0;
    return t.IsValid() ? 1 : 0;
}

// Tessellation::GetCoords<float> and GetFacets (bfr/tessellation.h:221-262)
int ref_bfr_tess(int regFaceSize, int N, int numRates, const int *rates, int facetSize,
                 int preserveQuads, float *coords, int *facets) {
    Bfr::Parameterization param(schemeOfRegularFaceSize(regFaceSize), N);
    Bfr::Tessellation t(param, numRates, rates, tessOptions(facetSize, preserveQuads));
    if (!t.IsValid()) return 0;
    t.GetCoords(coords);
    t.GetFacets(facets);
    return 1;
}

// Parameterization::ConvertCoordToNormalizedSubFace (bfr/parameterization.h:166-170)
int ref_bfr_subface(int regFaceSize, int N, int n, const float *uv, int *sub, float *st) {
    Bfr::Parameterization param(schemeOfRegularFaceSize(regFaceSize), N);
    if (!param.IsValid()) return 0;
    for (int i = 0; i < n; ++i) {
        float in[2] = {uv[2 * i], uv[2 * i + 1]};
        if (param.HasSubFaces()) {
            sub[i] = param.ConvertCoordToNormalizedSubFace(in, st + 2 * i);
        } else {
            sub[i] = 0;
            st[2 * i] = in[0], st[2 * i + 1] = in[1];
        }
    }
    return 1;
}

}  // extern "C"

namespace {
struct BfrRecord {
    std::vector<long> coordOffsets, facetOffsets;
    std::vector<int> valid, regular, facets;
    std::vector<float> coords;
    std::vector<float> outF[6];
    std::vector<double> outD[6];
    std::vector<float> uv[3];  // face-varying channel 0 (2 values): UV, dUV/du, dUV/dv
};

template <class REAL>
void bfrEvalFace(Bfr::Surface<REAL> const &s, std::vector<REAL> &patch, const float *pos,
                 int nverts, std::vector<float> const &coords, size_t c0, size_t n,
                 std::vector<REAL> *out) {
    // mesh points in REAL: PreparePatchPoints reads the mesh array in the surface's precision
    static thread_local std::vector<REAL> mesh;
    if (mesh.size() != (size_t)nverts * 3) mesh.resize((size_t)nverts * 3);
    for (size_t i = 0; i < (size_t)nverts * 3; ++i) mesh[i] = (REAL)pos[i];
    patch.resize((size_t)s.GetNumPatchPoints() * 3);
    s.PreparePatchPoints(mesh.data(), 3, patch.data(), 3);
    for (size_t i = 0; i < n; ++i) {
        REAL uv[2] = {(REAL)coords[2 * (c0 + i)], (REAL)coords[2 * (c0 + i) + 1]};
        REAL r[6][3];
        s.Evaluate(uv, patch.data(), 3, r[0], r[1], r[2], r[3], r[4], r[5]);
        for (int k = 0; k < 6; ++k)
            for (int e = 0; e < 3; ++e) out[k][3 * (c0 + i) + e] = r[k][e];
    }
}
}  // namespace

extern "C" {

// The tessellate-and-evaluate loop of the reference's Bfr tutorials
// (tutorials/bfr/tutorial_1_2/bfr_tutorial_1_2.cpp:170-238) over every base face of a
// refiner: Bfr::RefinerSurfaceFactory with the given approximation levels, one
// Bfr::Tessellation per face from rates[rateOffsets[f] .. rateOffsets[f+1]), and
// Surface::Evaluate (P, Du, Dv, Duu, Duv, Dvv) at each coord in float and in double.
// Faces without a limit surface get no coords.  Facet indices are offset to the mesh-wide
// coord numbering (Tessellation::TransformFacetCoordIndices).
// uvs: optional values (2 floats each) of face-varying channel 0, evaluated per coord through
// SurfaceFactory::InitFaceVaryingSurface as the reference's tutorial 1.3 does
// (tutorials/bfr/tutorial_1_3/bfr_tutorial_1_3.cpp).
void *ref_bfr_mesh_record(void *refiner, int approxSharp, int approxSmooth, const float *pos,
                          const int *rateOffsets, const int *rates, int facetSize,
                          int preserveQuads, const float *uvs) {
    Far::TopologyRefiner const &mesh = *((Refiner *)refiner)->r;
    Bfr::SurfaceFactory::Options so;
    so.SetApproxLevelSharp(approxSharp);
    so.SetApproxLevelSmooth(approxSmooth);
    if (uvs) so.SetDefaultFVarID(0);
    Bfr::RefinerSurfaceFactory<> factory(mesh, so);
    int nf = factory.GetNumFaces();
    int nverts = mesh.GetLevel(0).GetNumVertices();
    BfrRecord *rec = new BfrRecord;
    rec->coordOffsets.assign(nf + 1, 0);
    rec->facetOffsets.assign(nf + 1, 0);
    rec->valid.assign(nf, 0);
    rec->regular.assign(nf, 0);
    int fs = facetSize == 4 ? 4 : 3;
    Bfr::Tessellation::Options to = tessOptions(fs, preserveQuads);
    Bfr::Surface<float> sf;
    Bfr::Surface<double> sd;
    std::vector<float> pf;
    std::vector<double> pd;
    for (int f = 0; f < nf; ++f) {
        rec->coordOffsets[f + 1] = rec->coordOffsets[f];
        rec->facetOffsets[f + 1] = rec->facetOffsets[f];
        if (!factory.InitVertexSurface(f, &sf)) continue;
        factory.InitVertexSurface(f, &sd);
        Bfr::Tessellation t(sf.GetParameterization(), rateOffsets[f + 1] - rateOffsets[f],
                            rates + rateOffsets[f], to);
        if (!t.IsValid()) continue;
        rec->valid[f] = 1;
        rec->regular[f] = sf.IsRegular() ? 1 : (sf.IsLinear() ? 2 : 0);
        size_t c0 = rec->coords.size() / 2, n = (size_t)t.GetNumCoords();
        rec->coords.resize(2 * (c0 + n));
        t.GetCoords(rec->coords.data() + 2 * c0);
        size_t f0 = rec->facets.size() / fs;
        rec->facets.resize(fs * (f0 + (size_t)t.GetNumFacets()));
        t.GetFacets(rec->facets.data() + fs * f0);
        t.TransformFacetCoordIndices(rec->facets.data() + fs * f0, (int)c0);
        for (int k = 0; k < 6; ++k) {
            rec->outF[k].resize(3 * (c0 + n));
            rec->outD[k].resize(3 * (c0 + n));
        }
        bfrEvalFace(sf, pf, pos, nverts, rec->coords, c0, n, rec->outF);
        bfrEvalFace(sd, pd, pos, nverts, rec->coords, c0, n, rec->outD);
        if (uvs) {
            Bfr::Surface<float> su;
            for (int k = 0; k < 3; ++k) rec->uv[k].resize(2 * (c0 + n));
            if (factory.InitFaceVaryingSurface(f, &su)) {
                std::vector<float> patch((size_t)su.GetNumPatchPoints() * 2);
                su.PreparePatchPoints(uvs, 2, patch.data(), 2);
                for (size_t i = 0; i < n; ++i) {
                    float r[3][2];
                    su.Evaluate(&rec->coords[2 * (c0 + i)], patch.data(), 2, r[0], r[1], r[2]);
                    for (int k = 0; k < 3; ++k)
                        for (int e = 0; e < 2; ++e) rec->uv[k][2 * (c0 + i) + e] = r[k][e];
                }
            }
        }
        rec->coordOffsets[f + 1] = (long)(c0 + n);
        rec->facetOffsets[f + 1] = (long)(f0 + t.GetNumFacets());
    }
    return rec;
}

// The same loop in float with P, Du and Dv only (the tutorial's outputs), keeping nothing:
// the reference's CPU Bfr path for timing.  Faces are split over `threads` OpenMP threads,
// each with its own Surface and buffers, sharing one factory with a thread-safe cache
// (Bfr::RefinerSurfaceFactory<Bfr::SurfaceFactoryCacheThreaded<...>>, as the reference's
// tutorial 2.2 recommends for threaded use).  Returns the number of points evaluated.
long ref_bfr_mesh_run(void *refiner, int approxSharp, int approxSmooth, const float *pos,
                      const int *rateOffsets, const int *rates, int facetSize, int threads) {
    Far::TopologyRefiner const &mesh = *((Refiner *)refiner)->r;
    Bfr::SurfaceFactory::Options so;
    so.SetApproxLevelSharp(approxSharp);
    so.SetApproxLevelSmooth(approxSmooth);
    typedef Bfr::RefinerSurfaceFactory<
        Bfr::SurfaceFactoryCacheThreaded<std::shared_mutex, std::shared_lock<std::shared_mutex>,
                                         std::unique_lock<std::shared_mutex>>>
        Factory;
    Factory factory(mesh, so);
    int nf = factory.GetNumFaces();
    Bfr::Tessellation::Options to = tessOptions(facetSize == 4 ? 4 : 3, 0);
    long total = 0;
#pragma omp parallel num_threads(threads) reduction(+ : total)
    {
        Bfr::Surface<float> sf;
        std::vector<float> patch, coords, P, Du, Dv;
        std::vector<int> facets;
#pragma omp for schedule(dynamic, 64)
        for (int f = 0; f < nf; ++f) {
            if (!factory.InitVertexSurface(f, &sf)) continue;
            Bfr::Tessellation t(sf.GetParameterization(), rateOffsets[f + 1] - rateOffsets[f],
                                rates + rateOffsets[f], to);
            if (!t.IsValid()) continue;
            int n = t.GetNumCoords();
            coords.resize(2 * (size_t)n);
            t.GetCoords(coords.data());
            patch.resize((size_t)sf.GetNumPatchPoints() * 3);
            sf.PreparePatchPoints(pos, 3, patch.data(), 3);
            P.resize(3 * (size_t)n);
            Du.resize(3 * (size_t)n);
            Dv.resize(3 * (size_t)n);
            for (int i = 0; i < n; ++i)
                sf.Evaluate(&coords[2 * i], patch.data(), 3, &P[3 * i], &Du[3 * i], &Dv[3 * i]);
            facets.resize((size_t)t.GetNumFacets() * t.GetFacetSize());
            t.GetFacets(facets.data());
            total += n;
        }
    }
    return total;
}

// sizes: {faces, coords, facets}
void ref_bfr_record_sizes(void *p, long *sizes) {
    BfrRecord *r = (BfrRecord *)p;
    sizes[0] = (long)r->valid.size();
    sizes[1] = (long)r->coords.size() / 2;
    sizes[2] = (long)r->facets.size();
}

// out6f / out6d: 6 arrays of 3 values per coord (P, Du, Dv, Duu, Duv, Dvv)
void ref_bfr_record_uv(void *p, float **uv3) {
    BfrRecord *r = (BfrRecord *)p;
    for (int k = 0; k < 3; ++k) copyVec(r->uv[k], uv3[k]);
}

void ref_bfr_record_copy(void *p, long *coordOffsets, long *facetOffsets, int *valid,
                         int *regular, float *coords, int *facets, float **out6f, double **out6d) {
    BfrRecord *r = (BfrRecord *)p;
    copyVec(r->coordOffsets, coordOffsets);
    copyVec(r->facetOffsets, facetOffsets);
    copyVec(r->valid, valid);
    copyVec(r->regular, regular);
    copyVec(r->coords, coords);
    copyVec(r->facets, facets);
    for (int k = 0; k < 6; ++k) {
        if (out6f) copyVec(r->outF[k], out6f[k]);
        if (out6d) copyVec(r->outD[k], out6d[k]);
    }
}

void ref_bfr_record_destroy(void *p) { delete (BfrRecord *)p; }

// Bfr::Surface::EvaluateStencil (bfr/surface.h:244-265) at every coord of the reference's
// tessellate loop (faces and coords in ref_bfr_mesh_record's order): each coord's limit
// stencils for P, Du and Dv over the surface's control points, mapped to mesh vertices through
// Surface::GetControlPointIndices (a vertex named twice sums its weights, at its first place).
// Writes stencil sizes (one per coord, capacity `maxCoords`) and returns the total number of
// entries, copying indices and the three weight arrays when `indices` is not null (capacity
// `maxEntries`); -1 when a capacity is too small.
long ref_bfr_stencils(void *refiner, int approxSharp, int approxSmooth, const int *rateOffsets,
                      const int *rates, int facetSize, int preserveQuads, long maxCoords,
                      int *sizes, long maxEntries, int *indices, float *wP, float *wDu,
                      float *wDv) {
    Far::TopologyRefiner const &mesh = *((Refiner *)refiner)->r;
    Bfr::SurfaceFactory::Options so;
    so.SetApproxLevelSharp(approxSharp);
    so.SetApproxLevelSmooth(approxSmooth);
    Bfr::RefinerSurfaceFactory<> factory(mesh, so);
    const int nf = factory.GetNumFaces();
    Bfr::Tessellation::Options to = tessOptions(facetSize == 4 ? 4 : 3, preserveQuads);
    Bfr::Surface<float> sf;
    std::vector<float> coords, sp, sdu, sdv;
    std::vector<Far::Index> cps;
    long nc = 0, ne = 0;
    for (int f = 0; f < nf; ++f) {
        if (!factory.InitVertexSurface(f, &sf)) continue;
        Bfr::Tessellation t(sf.GetParameterization(), rateOffsets[f + 1] - rateOffsets[f],
                            rates + rateOffsets[f], to);
        if (!t.IsValid()) continue;
        const int n = t.GetNumCoords(), ncp = sf.GetNumControlPoints();
        coords.resize(2 * (size_t)n);
        t.GetCoords(coords.data());
        cps.resize(ncp);
        sf.GetControlPointIndices(cps.data());
        sp.resize(ncp), sdu.resize(ncp), sdv.resize(ncp);
        for (int i = 0; i < n; ++i) {
            sf.EvaluateStencil(&coords[2 * i], sp.data(), sdu.data(), sdv.data());
            if (nc >= maxCoords) return -1;
            const long e0 = ne;
            for (int j = 0; j < ncp; ++j) {
                long at = -1;
                for (long k = e0; indices && k < ne; ++k)
                    if (indices[k] == cps[j]) at = k;
                if (!indices) {
                    // count distinct vertices only
                    bool seen = false;
                    for (int q = 0; q < j; ++q) seen = seen || cps[q] == cps[j];
                    if (!seen) ++ne;
                    continue;
                }
                if (at < 0) {
                    if (ne >= maxEntries) return -1;
                    at = ne++;
                    indices[at] = cps[j];
                    wP[at] = wDu[at] = wDv[at] = 0.0f;
                }
                wP[at] += sp[j];
                wDu[at] += sdu[j];
                wDv[at] += sdv[j];
            }
            sizes[nc++] = (int)(ne - e0);
        }
    }
    return ne;
}

// The per-edge rates of the reference's tutorial 2.1 with its limit option
// (tutorials/bfr/tutorial_2_1/bfr_tutorial_2_1.cpp:240-299): for each face with a limit
// surface, its limit positions at the face's corners (Parameterization::GetVertexCoord +
// Surface::Evaluate) and rate 1 + (int)(length / interval) capped at maxRate for the edge to
// the next corner.  One rate per face corner, faces in order; faces without a surface get 0.
void ref_bfr_limit_rates(void *refiner, int approxSharp, int approxSmooth, const float *pos,
                         float interval, int maxRate, int *rates, float *cornerPoints) {
    Far::TopologyRefiner const &mesh = *((Refiner *)refiner)->r;
    Bfr::SurfaceFactory::Options so;
    so.SetApproxLevelSharp(approxSharp);
    so.SetApproxLevelSmooth(approxSmooth);
    Bfr::RefinerSurfaceFactory<> factory(mesh, so);
    Bfr::Surface<float> sf;
    std::vector<float> patch, corner;
    long c = 0;
    for (int f = 0; f < factory.GetNumFaces(); ++f) {
        const int N = mesh.GetLevel(0).GetFaceVertices(f).size();
        if (!factory.InitVertexSurface(f, &sf)) {
            for (int i = 0; i < N; ++i) rates[c + i] = 0;
            c += N;
            continue;
        }
        patch.resize((size_t)sf.GetNumPatchPoints() * 3);
        sf.PreparePatchPoints(pos, 3, patch.data(), 3);
        corner.resize(3 * (size_t)N);
        Bfr::Parameterization param = sf.GetParameterization();
        for (int i = 0; i < N; ++i) {
            float uv[2];
            param.GetVertexCoord(i, uv);
            sf.Evaluate(uv, patch.data(), 3, &corner[3 * i]);
        }
        for (int i = 0; i < N; ++i) {
            const float *a = &corner[3 * i], *b = &corner[3 * ((i + 1) % N)];
            float d[3];
            for (int k = 0; k < 3; ++k) d[k] = std::abs(a[k] - b[k]);
            const float len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            rates[c + i] = std::min(1 + (int)(len / interval), maxRate);
            if (cornerPoints)
                for (int k = 0; k < 3; ++k) cornerPoints[3 * (c + i) + k] = a[k];
        }
        c += N;
    }
}

// Varying surfaces (Bfr::SurfaceFactory::InitVaryingSurface, bfr/surfaceFactory.h:252) at
// every coord of the reference's tessellate loop (faces and coords in ref_bfr_mesh_record's
// order): `values` holds `length` floats per mesh vertex; writes the evaluated value per coord.
// Returns the number of coords.
long ref_bfr_varying(void *refiner, int approxSharp, int approxSmooth, const int *rateOffsets,
                     const int *rates, int facetSize, int preserveQuads, const float *values,
                     int length, float *out) {
    Far::TopologyRefiner const &mesh = *((Refiner *)refiner)->r;
    Bfr::SurfaceFactory::Options so;
    so.SetApproxLevelSharp(approxSharp);
    so.SetApproxLevelSmooth(approxSmooth);
    Bfr::RefinerSurfaceFactory<> factory(mesh, so);
    const int nf = factory.GetNumFaces();
    Bfr::Tessellation::Options to = tessOptions(facetSize == 4 ? 4 : 3, preserveQuads);
    Bfr::Surface<float> sf, sv;
    std::vector<float> coords, patch;
    long nc = 0;
    for (int f = 0; f < nf; ++f) {
        if (!factory.InitVertexSurface(f, &sf)) continue;
        Bfr::Tessellation t(sf.GetParameterization(), rateOffsets[f + 1] - rateOffsets[f],
                            rates + rateOffsets[f], to);
        if (!t.IsValid()) continue;
        const int n = t.GetNumCoords();
        coords.resize(2 * (size_t)n);
        t.GetCoords(coords.data());
        if (!factory.InitVaryingSurface(f, &sv)) return -1;
        patch.resize((size_t)sv.GetNumPatchPoints() * length);
        sv.PreparePatchPoints(values, length, patch.data(), length);
        for (int i = 0; i < n; ++i)
            sv.Evaluate(&coords[2 * i], patch.data(), length, out + (size_t)(nc + i) * length);
        nc += n;
    }
    return nc;
}

// The tessellation with shared vertex and edge points of the reference's tutorial 2.2
// (tutorials/bfr/tutorial_2_2/bfr_tutorial_2_2.cpp:160-430), with per-face rates: faces in
// order through Bfr::RefinerSurfaceFactory (faces without a limit surface skipped), the
// boundary coords of each Bfr::Tessellation walked vertex by vertex and edge by edge against
// the base level's face vertices and edges; the point of a vertex, and the points inside an
// edge, are made by the first face to reach them and reused, edge points in reverse, by the
// later face; the facets are mapped through Tessellation::TransformFacetCoordIndices(facets,
// boundaryIndices, interiorOffset).  Writes the facets (point indices) in the order of
// ref_bfr_mesh_record, pointOffsets (faces + 1: the first point each face made) and, per
// point, the mesh coord (ref_bfr_mesh_record's numbering) it is evaluated at.  Returns the
// number of points; -1 for a shared edge that is non-manifold or has another rate.
long ref_bfr_share(void *refiner, int approxSharp, int approxSmooth, const int *rateOffsets,
                   const int *rates, int facetSize, int preserveQuads, int *facets,
                   long *pointOffsets, long *pointSources) {
    Far::TopologyRefiner const &mesh = *((Refiner *)refiner)->r;
    Far::TopologyLevel const &base = mesh.GetLevel(0);
    Bfr::SurfaceFactory::Options so;
    so.SetApproxLevelSharp(approxSharp);
    so.SetApproxLevelSmooth(approxSmooth);
    Bfr::RefinerSurfaceFactory<> factory(mesh, so);
    const int nf = factory.GetNumFaces();
    const int fs = facetSize == 4 ? 4 : 3;
    Bfr::Tessellation::Options to = tessOptions(fs, preserveQuads);
    std::vector<long> vertPoint(base.GetNumVertices(), -1), edgePoint(base.GetNumEdges(), -1);
    std::vector<int> edgeCount(base.GetNumEdges(), 0);
    std::vector<int> boundary, local;
    Bfr::Surface<float> sf;
    long points = 0, coords = 0, facetsDone = 0;
    for (int f = 0; f < nf; ++f) {
        pointOffsets[f] = points;
        if (!factory.InitVertexSurface(f, &sf)) continue;
        Bfr::Tessellation t(sf.GetParameterization(), rateOffsets[f + 1] - rateOffsets[f],
                            rates + rateOffsets[f], to);
        if (!t.IsValid()) continue;
        Far::ConstIndexArray fv = base.GetFaceVertices(f), fe = base.GetFaceEdges(f);
        boundary.resize(t.GetNumBoundaryCoords());
        int b = 0;
        for (int i = 0; i < fv.size(); ++i) {
            long &vp = vertPoint[fv[i]];
            if (vp < 0) {
                vp = points;
                pointSources[points++] = coords + b;
            }
            boundary[b++] = (int)vp;
            const int n = t.GetNumEdgeCoords(i);
            if (n < 1) continue;
            long &ep = edgePoint[fe[i]];
            if (ep < 0) {
                ep = points;
                edgeCount[fe[i]] = n;
                for (int j = 0; j < n; ++j) {
                    pointSources[points] = coords + b;
                    boundary[b++] = (int)points++;
                }
            } else {
                if (base.IsEdgeNonManifold(fe[i]) || edgeCount[fe[i]] != n) return -1;
                for (int j = 0; j < n; ++j) boundary[b++] = (int)(ep + n - 1 - j);
            }
        }
        const int nc = t.GetNumCoords(), ni = t.GetNumInteriorCoords();
        for (int j = 0; j < ni; ++j) pointSources[points++] = coords + b + j;
        local.resize((size_t)t.GetNumFacets() * fs);
        t.GetFacets(local.data());
        t.TransformFacetCoordIndices(local.data(), boundary.data(), (int)(points - nc));
        std::copy(local.begin(), local.end(), facets + facetsDone * fs);
        facetsDone += t.GetNumFacets();
        coords += nc;
    }
    pointOffsets[nf] = points;
    return points;
}

}  // extern "C"
