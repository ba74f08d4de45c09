//
// gb300StencilTableFactory.h -- Far::StencilTableFactory's factorized stencil tables built on
// the GPU (far/stencilTableFactory.cpp:78-151), returned as device tables ready for
// Osd::GB300Evaluator.
//
// Far builds a table by feeding the subdivision masks of every level, one child vertex at a
// time, to a StencilBuilder (far/primvarRefiner.h:475-650 -> far/stencilBuilder.cpp:164-198),
// which resolves each (source, weight) pair against the source's already-factorized row and
// merges the products into the child's row.  Here the same calls are RECORDED on the host
// (GB300MaskRecorder stands where StencilBuilder::Index stands) and the merging runs on the
// device (GB300StencilTableFactoryCreate): same first-touch entry order, same float products
// and sums, so the table equals Far's bit for bit.
//
// Build: -I<repo>/include; the Far-facing Create() overloads need OpenSubdiv's headers on the
// include path (and libosdCPU for the refiner); the recorder alone does not.
//
#ifndef OPENSUBDIV_GB300_FAR_GB300_STENCIL_TABLE_FACTORY_H
#define OPENSUBDIV_GB300_FAR_GB300_STENCIL_TABLE_FACTORY_H

#include <algorithm>
#include <cstdint>
#include <vector>

#include "../osd/gb300Evaluator.h"

#if defined(OSD_GB300_HAVE_OPENSUBDIV) && defined(__has_include)
#if __has_include(<opensubdiv/far/primvarRefiner.h>)
#define OSD_GB300_HAVE_FAR 1
#include <opensubdiv/far/patchMap.h>
#include <opensubdiv/far/patchTable.h>
#include <opensubdiv/far/patchTableFactory.h>
#include <opensubdiv/far/primvarRefiner.h>
#include <opensubdiv/far/stencilTableFactory.h>
#include <opensubdiv/far/topologyRefiner.h>
#endif
#endif

OSD_GB300_NAMESPACE_BEGIN

/// Records the (destination, source, weight) calls a PrimvarRefiner makes on its destination
/// primvar -- the calls a StencilBuilder::Index receives (far/stencilBuilder.h:75-104) --
/// for one refinement level, and hands them out as per-row masks (GB300StencilMasks).
class GB300MaskRecorder {
public:
    /// The primvar type given to PrimvarRefiner::Interpolate / InterpolateVarying /
    /// InterpolateFaceVarying: an index into the global vertex numbering (control vertices,
    /// then each level's vertices), like StencilBuilder::Index.
    class Index {
    public:
        Index(GB300MaskRecorder *owner, int index) : _owner(owner), _index(index) {}
        Index operator[](int i) const { return Index(_owner, _index + i); }
        void Clear() {}
        /// Zero weights are dropped, as StencilBuilder::Index::AddWithWeight does
        /// (far/stencilBuilder.cpp:509-518).
        void AddWithWeight(Index const &src, float weight) {
            if (weight != 0.0f) _owner->add(_index, src._index, weight);
        }
        int GetOffset() const { return _index; }

    private:
        GB300MaskRecorder *_owner;
        int _index;
    };

    void Reset() {
        _dst.clear();
        _src.clear();
        _w.clear();
    }

    /// Masks of rows [firstRow, firstRow + numRows) in row order (entries of a row in call
    /// order); `order` receives the rows in the order they were interpolated.
    bool GetMasks(int firstRow, int numRows, std::vector<int64_t> &offsets,
                  std::vector<int> &sources, std::vector<float> &weights,
                  std::vector<int> *order = nullptr) const {
        offsets.assign((size_t)numRows + 1, 0);
        for (int d : _dst) {
            const int r = d - firstRow;
            if (r < 0 || r >= numRows) return false;
            ++offsets[(size_t)r + 1];
        }
        for (int r = 0; r < numRows; ++r) offsets[(size_t)r + 1] += offsets[r];
        std::vector<int64_t> fill(offsets.begin(), offsets.end() - 1);
        sources.resize(_src.size());
        weights.resize(_w.size());
        if (order) order->clear();
        int last = -1;
        for (size_t e = 0; e < _dst.size(); ++e) {
            const int r = _dst[e] - firstRow;
            if (order && _dst[e] != last) order->push_back(r);
            last = _dst[e];
            sources[fill[r]] = _src[e];
            weights[fill[r]++] = _w[e];
        }
        return true;
    }

private:
    void add(int dst, int src, float w) {
        _dst.push_back(dst);
        _src.push_back(src);
        _w.push_back(w);
    }
    std::vector<int> _dst, _src;
    std::vector<float> _w;
};

/// Per-level masks held on the host (the arrays a GB300StencilMasks points at).
struct GB300LevelMasks {
    int numRows = 0;
    std::vector<int64_t> offsets;
    std::vector<int> sources;
    std::vector<float> weights;
    GB300StencilMasks view() const {
        GB300StencilMasks m;
        m.numRows = numRows;
        m.nnz = (int64_t)sources.size();
        m.offsets = offsets.data();
        m.sources = sources.empty() ? nullptr : sources.data();
        m.weights = weights.empty() ? nullptr : weights.data();
        return m;
    }
};

#ifdef OSD_GB300_HAVE_FAR
/// Far::StencilTableFactory::Create with the merging on the GPU.
class GB300StencilTableFactory {
public:
    typedef Far::StencilTableFactory::Options Options;

    /// Masks of levels 1..min(maxLevel, refiner's max level) in the interpolation mode of
    /// `options` (the calls far/stencilTableFactory.cpp:109-118 makes).
    static bool RecordMasks(Far::TopologyRefiner const &refiner, Options options,
                            std::vector<GB300LevelMasks> &levels, int *numControl) {
        const int mode = options.interpolationMode;
        const int ch = options.fvarChannel;
        const bool fvar = mode == Far::StencilTableFactory::INTERPOLATE_FACE_VARYING;
        auto count = [&](int level) {
            return fvar ? refiner.GetLevel(level).GetNumFVarValues(ch)
                        : refiner.GetLevel(level).GetNumVertices();
        };
        *numControl = count(0);
        const int maxLevel = std::min(int(options.maxLevel), refiner.GetMaxLevel());
        Far::PrimvarRefinerReal<float> primvar(refiner);
        GB300MaskRecorder rec;
        GB300MaskRecorder::Index src(&rec, 0), dst(&rec, *numControl);
        levels.assign(maxLevel, GB300LevelMasks());
        for (int level = 1; level <= maxLevel; ++level) {
            rec.Reset();
            if (mode == Far::StencilTableFactory::INTERPOLATE_VERTEX)
                primvar.Interpolate(level, src, dst);
            else if (mode == Far::StencilTableFactory::INTERPOLATE_VARYING)
                primvar.InterpolateVarying(level, src, dst);
            else
                primvar.InterpolateFaceVarying(level, src, dst, ch);
            GB300LevelMasks &L = levels[level - 1];
            L.numRows = count(level);
            if (!rec.GetMasks(dst.GetOffset(), L.numRows, L.offsets, L.sources, L.weights))
                return false;
            src = dst;
            dst = dst[L.numRows];
        }
        return true;
    }

    /// The factorized table (factorizeIntermediateLevels must be true) as a device table;
    /// `referenceEntryOrder` keeps each stencil's entries in Far's order (otherwise they are
    /// sorted by control index, the layout GB300StencilTable::Create gives).
    static GB300StencilTable *Create(Far::TopologyRefiner const &refiner,
                                     Options options = Options(), void *deviceContext = NULL,
                                     bool referenceEntryOrder = false) {
        if (!options.factorizeIntermediateLevels) return nullptr;
        std::vector<GB300LevelMasks> levels;
        int numControl = 0;
        if (!RecordMasks(refiner, options, levels, &numControl)) return nullptr;
        std::vector<GB300StencilMasks> views;
        for (auto const &L : levels) views.push_back(L.view());
        ::GB300StencilTable *h = GB300StencilTableFactoryCreate(
            numControl, (int)views.size(), views.empty() ? nullptr : views.data(),
            options.generateIntermediateLevels ? 1 : 0, options.generateControlVerts ? 1 : 0,
            referenceEntryOrder ? 0 : 1, gb300_detail::stream_of(deviceContext));
        return h ? GB300StencilTable::Adopt(h) : nullptr;
    }
};
/// Far::LimitStencilTableFactory::Create (far/stencilTableFactory.cpp:411-662) with the merging
/// on the GPU.  The host keeps Far's own PatchMap lookups and patch-basis evaluations; the
/// refined-vertex stencils (GB300StencilTableFactory), the local-point splice
/// (AppendLocalPointStencilTable, :255-407) and the per-location merges run on the device
/// (GB300StencilTableComposeRows), all in Far's merge order, so the table equals Far's.
class GB300LimitStencilTableFactory {
public:
    typedef Far::LimitStencilTableFactory::Options Options;
    typedef Far::LimitStencilTableFactory::LocationArray LocationArray;
    typedef Far::LimitStencilTableFactory::LocationArrayVec LocationArrayVec;

    /// The patch table LimitStencilTableFactory builds when it is given none
    /// (far/stencilTableFactory.cpp:481-505).
    static Far::PatchTable const *CreatePatchTable(Far::TopologyRefiner const &refiner,
                                                   Options options) {
        const bool uniform = refiner.IsUniform();
        const bool varying = options.interpolationMode == Far::LimitStencilTableFactory::INTERPOLATE_VARYING;
        const bool fvar =
            options.interpolationMode == Far::LimitStencilTableFactory::INTERPOLATE_FACE_VARYING;
        int channel = options.fvarChannel;
        Far::PatchTableFactory::Options po;
        po.SetPatchPrecision<float>();
        po.includeBaseLevelIndices = true;
        po.generateVaryingTables = varying;
        po.generateFVarTables = fvar;
        if (fvar) {
            po.includeFVarBaseLevelIndices = true;
            po.numFVarChannels = 1;
            po.fvarChannelIndices = &channel;
            po.generateFVarLegacyLinearPatches =
                uniform || !refiner.GetAdaptiveOptions().considerFVarChannels;
        }
        po.SetEndCapType(Far::PatchTableFactory::Options::ENDCAP_GREGORY_BASIS);
        po.useInfSharpPatch = !uniform && refiner.GetAdaptiveOptions().useInfSharpPatch;
        return Far::PatchTableFactory::Create(refiner, po);
    }

    /// Options of the refined-vertex stencils LimitStencilTableFactory builds
    /// (far/stencilTableFactory.cpp:462-476).
    static GB300StencilTableFactory::Options CvOptions(Far::TopologyRefiner const &refiner,
                                                       Options options) {
        GB300StencilTableFactory::Options o;
        o.generateIntermediateLevels = refiner.IsUniform() ? false : true;
        o.generateControlVerts = true;
        o.generateOffsets = true;
        o.interpolationMode = options.interpolationMode;
        o.fvarChannel = options.fvarChannel;
        return o;
    }

    /// The local-point stencils of the interpolation mode as masks over the refined-vertex
    /// table (entries of weight 0 dropped, as far/stencilTableFactory.cpp:355-371 does).
    static bool LocalPointMasks(Far::PatchTable const &patchTable, Options options,
                                std::vector<int64_t> &offsets, std::vector<int> &sources,
                                std::vector<float> &weights) {
        Far::StencilTableReal<float> const *local = nullptr;
        if (options.interpolationMode == Far::LimitStencilTableFactory::INTERPOLATE_VERTEX)
            local = patchTable.GetLocalPointStencilTable<float>();
        else if (options.interpolationMode ==
                 Far::LimitStencilTableFactory::INTERPOLATE_FACE_VARYING)
            local = patchTable.GetLocalPointFaceVaryingStencilTable<float>(options.fvarChannel);
        else
            local = patchTable.GetLocalPointVaryingStencilTable<float>();
        offsets.assign(1, 0);
        sources.clear();
        weights.clear();
        if (!local || local->GetNumStencils() == 0) return false;
        for (int i = 0; i < local->GetNumStencils(); ++i) {
            Far::StencilReal<float> st = local->GetStencil(i);
            for (int j = 0; j < st.GetSize(); ++j) {
                if (st.GetWeights()[j] == 0.0f) continue;
                sources.push_back(st.GetVertexIndices()[j]);
                weights.push_back(st.GetWeights()[j]);
            }
            offsets.push_back((int64_t)sources.size());
        }
        return true;
    }

    /// Per-location masks: for every location FindPatch resolves, the patch's points (rows of
    /// the refined + local-point table) with the basis weights EvaluateBasis[Varying /
    /// FaceVarying] returns (far/stencilTableFactory.cpp:545-633).  Returns the number of
    /// weight channels: 1 (P), 3 (+ du, dv) or 6 (+ duu, duv, dvv).
    static int LocationMasks(Far::TopologyRefiner const &refiner,
                             Far::PatchTable const &patchTable, LocationArrayVec const &locations,
                             Options options, std::vector<int64_t> &offsets,
                             std::vector<int> &sources, std::vector<float> (&weights)[6]) {
        const bool uniform = refiner.IsUniform();
        const int mode = options.interpolationMode;
        const bool vertexPatches =
            mode == Far::LimitStencilTableFactory::INTERPOLATE_VERTEX ||
            (mode == Far::LimitStencilTableFactory::INTERPOLATE_VARYING && uniform);
        const bool fvarPatches = mode == Far::LimitStencilTableFactory::INTERPOLATE_FACE_VARYING;
        const int ch = options.fvarChannel;
        const int nc = options.generate2ndDerivatives ? 6 : options.generate1stDerivatives ? 3 : 1;
        Far::PatchMap map(patchTable);
        offsets.assign(1, 0);
        sources.clear();
        for (auto &w : weights) w.clear();
        float w[6][20];
        for (auto const &array : locations) {
            for (int j = 0; j < array.numLocations; ++j) {
                const float s = array.s[j], t = array.t[j];
                Far::PatchMap::Handle const *h = map.FindPatch(array.ptexIdx, s, t);
                if (!h) continue;
                Far::ConstIndexArray cvs =
                    vertexPatches ? patchTable.GetPatchVertices(*h)
                    : fvarPatches ? patchTable.GetPatchFVarValues(*h, ch)
                                  : patchTable.GetPatchVaryingVertices(*h);
                float *p[6] = {w[0], nc > 1 ? w[1] : 0, nc > 1 ? w[2] : 0,
                               nc > 3 ? w[3] : 0, nc > 3 ? w[4] : 0, nc > 3 ? w[5] : 0};
                if (vertexPatches)
                    patchTable.EvaluateBasis<float>(*h, s, t, p[0], p[1], p[2], p[3], p[4], p[5]);
                else if (fvarPatches)
                    patchTable.EvaluateBasisFaceVarying<float>(*h, s, t, p[0], p[1], p[2], p[3],
                                                               p[4], p[5], ch);
                else
                    patchTable.EvaluateBasisVarying<float>(*h, s, t, p[0], p[1], p[2], p[3],
                                                           p[4], p[5]);
                for (int k = 0; k < cvs.size(); ++k) {
                    sources.push_back(cvs[k]);
                    for (int c = 0; c < nc; ++c) weights[c].push_back(w[c][k]);
                }
                offsets.push_back((int64_t)sources.size());
            }
        }
        return nc;
    }

    /// The limit stencil table on the device (`patchTable` may be NULL: one is built as
    /// LimitStencilTableFactory does).  `referenceEntryOrder` keeps Far's entry order.
    static GB300StencilTable *Create(Far::TopologyRefiner const &refiner,
                                     LocationArrayVec const &locations,
                                     Far::PatchTable const *patchTable = NULL,
                                     Options options = Options(), void *deviceContext = NULL,
                                     bool referenceEntryOrder = false) {
        void *s = gb300_detail::stream_of(deviceContext);
        Far::PatchTable const *pt = patchTable ? patchTable : CreatePatchTable(refiner, options);
        if (!pt) return nullptr;
        GB300StencilTable *cv =
            GB300StencilTableFactory::Create(refiner, CvOptions(refiner, options), deviceContext, true);
        GB300StencilTable *result = nullptr;
        if (cv) {
            const bool fvar =
                options.interpolationMode == Far::LimitStencilTableFactory::INTERPOLATE_FACE_VARYING;
            const int nRefined =
                refiner.IsUniform()
                    ? (fvar ? refiner.GetLevel(refiner.GetMaxLevel()).GetNumFVarValues(options.fvarChannel)
                            : refiner.GetLevel(refiner.GetMaxLevel()).GetNumVertices())
                    : (fvar ? refiner.GetNumFVarValuesTotal(options.fvarChannel)
                            : refiner.GetNumVerticesTotal());
            std::vector<int64_t> off;
            std::vector<int> src;
            std::vector<float> w[6];
            ::GB300StencilTable *all = cv->GetHandle();
            ::GB300StencilTable *spliced = nullptr;
            if (cv->GetNumStencils() == nRefined && LocalPointMasks(*pt, options, off, src, w[0])) {
                const float *w0 = w[0].data();
                spliced = splice(all, off, src, &w0, 1, 1, 0, s);
                all = spliced;
            }
            if (all) {
                const int nc = LocationMasks(refiner, *pt, locations, options, off, src, w);
                const float *wp[6] = {w[0].data(), w[1].data(), w[2].data(),
                                      w[3].data(), w[4].data(), w[5].data()};
                ::GB300StencilTable *h =
                    splice(all, off, src, wp, nc, 0, referenceEntryOrder ? 0 : 1, s);
                result = GB300StencilTable::Adopt(h);
            }
            if (spliced) GB300StencilTableDestroy(spliced);
            delete cv;
        }
        if (!patchTable) delete pt;
        return result;
    }

private:
    static ::GB300StencilTable *splice(::GB300StencilTable *base, std::vector<int64_t> const &off,
                                       std::vector<int> const &src, const float *const *w,
                                       int nc, int appendBase, int sortEntries, void *s) {
        return GB300StencilTableComposeRows(
            GB300StencilTableGetNumStencils(base), GB300StencilTableGetNumIndices(base),
            (const int *)GB300StencilTableGetBuffer(base, 0),
            (const int *)GB300StencilTableGetBuffer(base, 1),
            (const int *)GB300StencilTableGetBuffer(base, 2),
            (const float *)GB300StencilTableGetBuffer(base, 3), (int)off.size() - 1,
            (int64_t)src.size(), off.data(), src.empty() ? nullptr : src.data(), nc, w,
            appendBase, sortEntries, s);
    }
};
#endif  // OSD_GB300_HAVE_FAR

OSD_GB300_NAMESPACE_END

#endif  // OPENSUBDIV_GB300_FAR_GB300_STENCIL_TABLE_FACTORY_H
