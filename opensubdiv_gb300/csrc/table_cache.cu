// On-disk table cache: one file per topology holding the arrays of a GB300TopologyDesc (refine
// stencils, patch-point stencils, flattened patch table), so a server can register topologies
// by path and re-read them from disk when it re-admits them, without keeping every topology's
// tables in host memory.
//
// Layout (little-endian, as both supported hosts are): a 256-byte header, then each array at a
// 64-byte aligned offset.  The header carries the counts, the byte offset of every array and an
// FNV-1a 64-bit checksum of everything after the header.  Files are written to a temporary name
// and renamed, so a reader never sees a partial file; opened files are mapped read-only.
#include "common.cuh"

#include <cstring>
#include <new>
#include <string>

#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

namespace gb300 {
namespace cache {

constexpr char kMagic[8] = {'G', 'B', '3', '0', '0', 'T', 'C', '1'};
constexpr uint32_t kVersion = 1;
constexpr int kSections = 11;

struct Header {
    char magic[8];
    uint32_t version, flags;  // flags: 1 = limit tables present, 2 = triangular
    int32_t numControl, length, numStencils, numPatchPoints;
    int32_t numPatchArrays, numPatches;
    int64_t nnz, patchPointNnz, numPatchIndices;
    uint64_t offset[kSections];  // sizes, offsets, indices, weights, pp x4, arrays, idx, params
    uint64_t payloadBytes;
    uint64_t checksum;
    uint8_t pad[256 - 8 - 8 - 24 - 24 - kSections * 8 - 16];
};
static_assert(sizeof(Header) == 256, "header size");

uint64_t fnv1a(const uint8_t *p, size_t n, uint64_t h = 1469598103934665603ull) {
    for (size_t i = 0; i < n; ++i) h = (h ^ p[i]) * 1099511628211ull;
    return h;
}

void section_sizes(const Header &h, uint64_t (&bytes)[kSections]) {
    const uint64_t ns = (uint64_t)h.numStencils, np = (uint64_t)h.numPatchPoints;
    const uint64_t v[kSections] = {ns * 4,
                                   ns * 4,
                                   (uint64_t)h.nnz * 4,
                                   (uint64_t)h.nnz * 4,
                                   np * 4,
                                   np * 4,
                                   (uint64_t)h.patchPointNnz * 4,
                                   (uint64_t)h.patchPointNnz * 4,
                                   (uint64_t)h.numPatchArrays * 24,
                                   (uint64_t)h.numPatchIndices * 4,
                                   (uint64_t)h.numPatches * 12};
    for (int k = 0; k < kSections; ++k) bytes[k] = v[k];
}

struct Mapping {
    void *base = nullptr;
    size_t size = 0;
};

}  // namespace cache
}  // namespace gb300

using namespace gb300;
using namespace gb300::cache;

extern "C" {

int GB300TableCacheWrite(const char *path, const GB300TopologyDesc *d) {
    const char *who = "GB300TableCacheWrite";
    if (!path || !d || d->numControl <= 0 || d->length <= 0 || d->numStencils < 0 ||
        d->nnz < 0 || d->numPatchArrays < 0)
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: bad arguments", who);
    Header h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, kMagic, 8);
    h.version = kVersion;
    const bool limit = d->numPatchArrays > 0;
    h.flags = (limit ? 1u : 0u) | (d->triangular ? 2u : 0u);
    h.numControl = d->numControl;
    h.length = d->length;
    h.numStencils = d->numStencils;
    h.nnz = d->nnz;
    if (limit) {
        h.numPatchPoints = d->numPatchPoints;
        h.patchPointNnz = d->patchPointNnz;
        h.numPatchArrays = d->numPatchArrays;
        h.numPatches = d->numPatches;
        h.numPatchIndices = d->numPatchIndices;
    }
    const void *src[kSections] = {d->sizes,     d->offsets,    d->indices,      d->weights,
                                  d->ppSizes,   d->ppOffsets,  d->ppIndices,    d->ppWeights,
                                  d->patchArrays, d->patchIndices, d->patchParams};
    uint64_t bytes[kSections];
    section_sizes(h, bytes);
    uint64_t off = sizeof(Header);
    for (int k = 0; k < kSections; ++k) {
        if (bytes[k] && !src[k]) return fail(GB300_ERR_INVALID_ARGUMENT, "%s: null array %d", who, k);
        off = (off + 63) & ~uint64_t(63);
        h.offset[k] = off;
        off += bytes[k];
    }
    h.payloadBytes = off - sizeof(Header);
    // checksum over the payload exactly as it is laid out in the file (zero padding included)
    uint64_t cs = 1469598103934665603ull;
    static const uint8_t zeros[64] = {0};
    uint64_t pos = sizeof(Header);
    for (int k = 0; k < kSections; ++k) {
        cs = fnv1a(zeros, h.offset[k] - pos, cs);
        cs = fnv1a((const uint8_t *)src[k], bytes[k], cs);
        pos = h.offset[k] + bytes[k];
    }
    h.checksum = cs;
    const std::string tmp = std::string(path) + ".tmp";
    FILE *f = std::fopen(tmp.c_str(), "wb");
    if (!f) return fail(GB300_ERR_INVALID_ARGUMENT, "%s: cannot create %s", who, tmp.c_str());
    bool good = std::fwrite(&h, sizeof(h), 1, f) == 1;
    pos = sizeof(Header);
    for (int k = 0; k < kSections && good; ++k) {
        const uint64_t gap = h.offset[k] - pos;
        if (gap) good = std::fwrite(zeros, 1, gap, f) == gap;
        if (good && bytes[k]) good = std::fwrite(src[k], 1, bytes[k], f) == bytes[k];
        pos = h.offset[k] + bytes[k];
    }
    good = (std::fclose(f) == 0) && good;
    if (!good || std::rename(tmp.c_str(), path) != 0) {
        std::remove(tmp.c_str());
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: writing %s failed", who, path);
    }
    return ok();
}

int GB300TableCacheOpen(const char *path, int verify, GB300TopologyDesc *out, void **handle) {
    const char *who = "GB300TableCacheOpen";
    if (!path || !out || !handle) return fail(GB300_ERR_INVALID_ARGUMENT, "%s: null argument", who);
    *handle = nullptr;
    const int fd = ::open(path, O_RDONLY);
    if (fd < 0) return fail(GB300_ERR_INVALID_ARGUMENT, "%s: cannot open %s", who, path);
    struct stat st;
    if (fstat(fd, &st) != 0 || (size_t)st.st_size < sizeof(Header)) {
        ::close(fd);
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: %s is not a table cache", who, path);
    }
    void *base = mmap(nullptr, (size_t)st.st_size, PROT_READ, MAP_SHARED, fd, 0);
    ::close(fd);
    if (base == MAP_FAILED) return fail(GB300_ERR_INVALID_ARGUMENT, "%s: cannot map %s", who, path);
    const Header &h = *(const Header *)base;
    auto bad = [&](const char *why) {
        munmap(base, (size_t)st.st_size);
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: %s: %s", who, path, why);
    };
    if (std::memcmp(h.magic, kMagic, 8) != 0 || h.version != kVersion)
        return bad("not a version-1 table cache");
    if (h.numControl <= 0 || h.length <= 0 || h.numStencils < 0 || h.nnz < 0 ||
        h.numPatchPoints < 0 || h.patchPointNnz < 0 || h.numPatchArrays < 0 || h.numPatches < 0 ||
        h.numPatchIndices < 0)
        return bad("negative counts");
    uint64_t bytes[kSections];
    section_sizes(h, bytes);
    for (int k = 0; k < kSections; ++k)
        if (h.offset[k] < sizeof(Header) || (h.offset[k] & 63) ||
            h.offset[k] + bytes[k] > (uint64_t)st.st_size)
            return bad("section outside the file");
    if (sizeof(Header) + h.payloadBytes > (uint64_t)st.st_size) return bad("truncated");
    if (verify) {
        const uint64_t cs =
            fnv1a((const uint8_t *)base + sizeof(Header), h.payloadBytes);
        if (cs != h.checksum) return bad("checksum mismatch");
    }
    auto *m = new (std::nothrow) Mapping;
    if (!m) return bad("host allocation");
    m->base = base;
    m->size = (size_t)st.st_size;
    const char *b = (const char *)base;
    GB300TopologyDesc d;
    std::memset(&d, 0, sizeof(d));
    d.numControl = h.numControl;
    d.length = h.length;
    d.numStencils = h.numStencils;
    d.nnz = h.nnz;
    d.sizes = (const int *)(b + h.offset[0]);
    d.offsets = (const int *)(b + h.offset[1]);
    d.indices = (const int *)(b + h.offset[2]);
    d.weights = (const float *)(b + h.offset[3]);
    if (h.flags & 1u) {
        d.numPatchPoints = h.numPatchPoints;
        d.patchPointNnz = h.patchPointNnz;
        d.ppSizes = (const int *)(b + h.offset[4]);
        d.ppOffsets = (const int *)(b + h.offset[5]);
        d.ppIndices = (const int *)(b + h.offset[6]);
        d.ppWeights = (const float *)(b + h.offset[7]);
        d.numPatchArrays = h.numPatchArrays;
        d.patchArrays = b + h.offset[8];
        d.numPatchIndices = h.numPatchIndices;
        d.patchIndices = (const int *)(b + h.offset[9]);
        d.numPatches = h.numPatches;
        d.patchParams = b + h.offset[10];
        d.triangular = (h.flags & 2u) ? 1 : 0;
    }
    *out = d;
    *handle = m;
    return ok();
}

void GB300TableCacheClose(void *handle) {
    Mapping *m = (Mapping *)handle;
    if (!m) return;
    munmap(m->base, m->size);
    delete m;
}

}  // extern "C"
