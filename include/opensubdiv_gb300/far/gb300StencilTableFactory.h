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
#endif  // OSD_GB300_HAVE_FAR

OSD_GB300_NAMESPACE_END

#endif  // OPENSUBDIV_GB300_FAR_GB300_STENCIL_TABLE_FACTORY_H
