// Serving loop: resident topologies under a device-memory budget, continuous batching of
// refine / limit-evaluation requests, overlapped rounds on several streams.
//
// Memory: two device pools are allocated once at creation -- the table pool (the budget for
// resident topologies' stencil / patch tables and PatchMaps) and the request arena (inputs,
// outputs and scratch of requests in flight) -- and sub-allocated first-fit, so serving never
// calls cudaMalloc / cudaFree (which would synchronise the device).  A topology's tables are
// resident in two independent units -- its refine table, and its limit tables (patch-point
// stencils, patch table, PatchMap) -- so a request uploads only the unit it reads when that
// unit is not resident, evicting least-recently-used units that no in-flight request pins.
//
// Scheduling: one scheduler thread takes pending requests in arrival order into a round while
// a stream is free, the round's requests fit the arena and their topologies fit the pool, up
// to a per-round limit.  A round is: host->device copies of every request's control values
// (and query points), ONE batched stencil launch for every refine request and every limit
// request's patch-point stencils (stencils_batch.h), PatchMap lookup + EvalPatches per limit
// request, device->host copies of every result, and a host callback that timestamps
// completion.  Rounds on different streams overlap (copies of one with kernels of another),
// and requests arriving while rounds run join the next round as soon as a stream frees up.
// "plain" mode serves one request at a time through the plain entry points -- the reference
// behaviour this is compared with.
#include "common.cuh"
#include "patchmap.h"
#include "stencils_batch.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

namespace gb300 {
namespace serve {

using Clock = std::chrono::steady_clock;

inline double seconds_since(Clock::time_point t0) {
    return std::chrono::duration<double>(Clock::now() - t0).count();
}

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// First-fit sub-allocator over one device allocation (offsets, 256-byte granules).
class Pool {
  public:
    bool init(size_t bytes, const char *what) {
        cap_ = align256(bytes);
        if (cap_ == 0) return true;
        if (check_cuda(cudaMalloc((void **)&base_, cap_), what) != GB300_OK) {
            base_ = nullptr;
            return false;
        }
        free_[0] = cap_;
        return true;
    }
    ~Pool() {
        if (base_) cudaFree(base_);
    }
    bool alloc(size_t bytes, size_t &off) {
        bytes = align256(bytes ? bytes : 1);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            off = it->first;
            const size_t rest = it->second - bytes;
            free_.erase(it);
            if (rest) free_[off + bytes] = rest;
            used_ += bytes;
            return true;
        }
        return false;
    }
    void release(size_t off, size_t bytes) {
        bytes = align256(bytes ? bytes : 1);
        used_ -= bytes;
        auto next = free_.lower_bound(off);
        if (next != free_.end() && off + bytes == next->first) {
            bytes += next->second;
            next = free_.erase(next);
        }
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == off) {
                prev->second += bytes;
                return;
            }
        }
        free_[off] = bytes;
    }
    char *at(size_t off) const { return base_ + off; }
    size_t capacity() const { return cap_; }
    size_t used() const { return used_; }

  private:
    char *base_ = nullptr;
    size_t cap_ = 0, used_ = 0;
    std::map<size_t, size_t> free_;
};

// Byte layout of one allocation made of several 256-aligned pieces.
struct Layout {
    size_t total = 0;
    size_t add(size_t bytes) {
        const size_t off = total;
        total += align256(bytes);
        return off;
    }
};

struct Topology {
    int id = 0;
    GB300TopologyDesc d{};
    bool limit = false;
    int quadFamily = 0;
    PatchMapHost map;
    double refineMean = 0, ppMean = 0;
    // device footprint: unit 0 holds the refine table (oSizes .. oWeights, offsets inside
    // unit 0's pool range), unit 1 the limit tables (oPpSizes .. oHandles, inside unit 1's)
    size_t oSizes, oOffsets, oIndices, oWeights;
    size_t oPpSizes, oPpOffsets, oPpIndices, oPpWeights;
    size_t oArrays, oPIndices, oParams, oNodes, oHandles;
    struct Unit {
        Layout lay;
        bool resident = false;
        bool needsUpload = false;
        size_t poolOff = 0;
        int pins = 0;
        uint64_t lastUse = 0;
        cudaEvent_t ready = nullptr;  // recorded after the latest upload
    } unit[2];
};

// The unit a request reads: refine requests the refine table, limit requests the limit tables.
inline int unit_of(int kind) { return kind == GB300_REQUEST_LIMIT ? 1 : 0; }

struct Request {
    GB300Request r{};
    Topology *topo = nullptr;
    Clock::time_point tSubmit;
    double latency = -1.0;
    int status = -1;  // -1 pending, else a GB300 status
    // arena piece offsets (relative to arenaOff)
    Layout lay;
    size_t arenaOff = 0;
    size_t oCv = 0, oOut = 0, oFaces = 0, oU = 0, oV = 0, oCoords = 0, oPatchSrc = 0;
};

struct Round {
    GB300Server *srv = nullptr;
    std::vector<Request *> reqs;
    int stream = 0;
    std::vector<std::pair<Topology *, int>> uploads;  // (topology, unit) uploaded first
    std::vector<batch::Job> jobs;
    std::vector<int> tileBase;
    size_t metaOff = 0, metaBytes = 0;  // job table + tile prefix + counter/status in the arena
    std::atomic<bool> done{false};
    Clock::time_point tDone;
    cudaEvent_t start = nullptr, end = nullptr;  // device time of the round
    ~Round() {
        if (start) cudaEventDestroy(start);
        if (end) cudaEventDestroy(end);
    }
};

}  // namespace serve
}  // namespace gb300

using namespace gb300;
using namespace gb300::serve;

struct GB300Server {
    GB300ServerConfig cfg{};
    Pool tables, arena;
    std::vector<cudaStream_t> streams;
    std::vector<int> streamBusy;
    int device = 0;

    std::mutex m;
    std::condition_variable cv;       // scheduler wake-ups (submit, completion, stop)
    std::condition_variable doneCv;   // request completions (Wait)
    std::unordered_map<int, std::unique_ptr<Topology>> topos;
    std::deque<std::unique_ptr<Request>> all;  // every request, indexed by ticket - firstTicket
    uint64_t firstTicket = 1;
    std::deque<Request *> pending;
    std::vector<std::unique_ptr<Round>> inflight;
    uint64_t useClock = 0;
    GB300ServerStats stats{};
    bool stop = false;
    std::thread worker;
    std::vector<void *> registered;  // host ranges this server page-locked
    std::vector<void *> caches;      // table-cache mappings of topologies added from files
};

namespace gb300 {
namespace serve {

void on_round_done(void *p) {
    Round *r = (Round *)p;
    GB300Server *srv = r->srv;  // the scheduler may free r as soon as done is set
    r->tDone = Clock::now();
    {
        std::lock_guard<std::mutex> lock(srv->m);
        r->done.store(true);
    }
    srv->cv.notify_all();
}

// Arena bytes of one request (its device inputs, outputs and scratch).
void plan_request(Request &q) {
    const GB300TopologyDesc &d = q.topo->d;
    const size_t cv = (size_t)d.numControl * d.length * 4;
    q.lay = Layout{};
    q.oCv = q.lay.add(cv);
    if (q.r.kind == GB300_REQUEST_REFINE) {
        q.oOut = q.lay.add((size_t)d.numStencils * d.length * 4);
    } else {
        const size_t n = (size_t)q.r.numPoints;
        q.oFaces = q.lay.add(n * 4);
        q.oU = q.lay.add(n * 4);
        q.oV = q.lay.add(n * 4);
        q.oCoords = q.lay.add(n * 20);
        q.oPatchSrc = q.lay.add((size_t)d.numPatchPoints * 12);
        q.oOut = q.lay.add(n * 36);
    }
}

size_t out_bytes(const Request &q) {
    const GB300TopologyDesc &d = q.topo->d;
    return q.r.kind == GB300_REQUEST_REFINE ? (size_t)d.numStencils * d.length * 4
                                            : (size_t)q.r.numPoints * 36;
}

// Reserves table-pool space for unit k of `t`, evicting least-recently-used units that no
// in-flight request pins; false if it cannot fit now.  Called with the lock held; the upload
// itself happens outside the lock (upload_tables).
bool reserve(GB300Server *s, Topology *t, int k) {
    Topology::Unit &u = t->unit[k];
    if (u.resident) return true;
    size_t off = 0;
    while (!s->tables.alloc(u.lay.total, off)) {
        Topology::Unit *victim = nullptr;
        for (auto &kv : s->topos)
            for (Topology::Unit &c : kv.second->unit)
                if (c.resident && c.pins == 0 && (!victim || c.lastUse < victim->lastUse))
                    victim = &c;
        if (!victim) return false;
        s->tables.release(victim->poolOff, victim->lay.total);
        victim->resident = false;
        s->stats.evictions++;
        s->stats.residentBytes -= victim->lay.total;
    }
    u.resident = true;
    u.needsUpload = true;
    u.poolOff = off;
    s->stats.uploads++;
    s->stats.bytesUploaded += u.lay.total;
    s->stats.residentBytes += u.lay.total;
    s->stats.peakResidentBytes = std::max(s->stats.peakResidentBytes, s->stats.residentBytes);
    return true;
}

// Host -> device copies of unit k of a reserved topology on `st`, then the unit's ready event.
int upload_tables(GB300Server *s, Topology *t, int k, cudaStream_t st) {
    char *b = s->tables.at(t->unit[k].poolOff);
    const GB300TopologyDesc &d = t->d;
    int err = GB300_OK;
    auto h2d = [&](size_t o, const void *src, size_t bytes) {
        if (err == GB300_OK && bytes)
            err = check_cuda(cudaMemcpyAsync(b + o, src, bytes, cudaMemcpyHostToDevice, st),
                             "GB300Server table upload");
    };
    if (k == 0) {
        h2d(t->oSizes, d.sizes, (size_t)d.numStencils * 4);
        h2d(t->oOffsets, d.offsets, (size_t)d.numStencils * 4);
        h2d(t->oIndices, d.indices, (size_t)d.nnz * 4);
        h2d(t->oWeights, d.weights, (size_t)d.nnz * 4);
    } else {
        h2d(t->oPpSizes, d.ppSizes, (size_t)d.numPatchPoints * 4);
        h2d(t->oPpOffsets, d.ppOffsets, (size_t)d.numPatchPoints * 4);
        h2d(t->oPpIndices, d.ppIndices, (size_t)d.patchPointNnz * 4);
        h2d(t->oPpWeights, d.ppWeights, (size_t)d.patchPointNnz * 4);
        h2d(t->oArrays, d.patchArrays, (size_t)d.numPatchArrays * 24);
        h2d(t->oPIndices, d.patchIndices, (size_t)d.numPatchIndices * 4);
        h2d(t->oParams, d.patchParams, (size_t)d.numPatches * 12);
        h2d(t->oNodes, t->map.nodes.data(), t->map.nodes.size() * 4);
        h2d(t->oHandles, t->map.handles.data(), t->map.handles.size() * 4);
    }
    if (err == GB300_OK)
        err = check_cuda(cudaEventRecord(t->unit[k].ready, st), "GB300Server upload");
    return err;
}

PatchMapDevice device_map(GB300Server *s, Topology *t) {
    char *b = s->tables.at(t->unit[1].poolOff);
    PatchMapDevice pm;
    pm.nodes = b + t->oNodes;
    pm.handles = b + t->oHandles;
    pm.triangular = t->d.triangular;
    pm.minFace = t->map.minFace;
    pm.maxFace = t->map.maxFace;
    pm.maxDepth = t->map.maxDepth;
    pm.numPatches = t->d.numPatches;
    return pm;
}

batch::Job stencil_job(const int *sizes, const int *offsets, const int *indices,
                       const float *weights, int n, const float *src, float *dst, int length,
                       int srcStride, int dstStride) {
    auto al = [](const void *p, uintptr_t m) { return ((uintptr_t)p & (m - 1)) == 0; };
    batch::Job j{};
    j.src = src;
    j.dst[0] = dst;
    j.w[0] = weights;
    j.sizes = sizes;
    j.offsets = offsets;
    j.indices = indices;
    j.length = length;
    j.srcStride = srcStride;
    j.dstStride[0] = dstStride;
    j.vw = (al(src, 32) && srcStride % 8 == 0) ? 8 : (al(src, 16) && srcStride % 4 == 0) ? 4 : 1;
    j.vecDst[0] = (al(dst, 32) && dstStride % 8 == 0) ? 8
                  : (al(dst, 16) && dstStride % 4 == 0) ? 4 : 0;
    j.numStencils = n;
    return j;
}

// Queues one round on its stream.  Returns a status; on failure nothing was queued that still
// references the round's arena pieces after the stream drains.
int launch_round(GB300Server *s, Round *r) {
    cudaStream_t st = s->streams[r->stream];
    int err = GB300_OK;
    // after the first failure nothing more is queued (the scheduler then drains the stream)
#define chk(call, what)                                    \
    do {                                                   \
        if (err == GB300_OK) err = check_cuda((call), what); \
    } while (0)
    if (cudaEventCreate(&r->start) == cudaSuccess && cudaEventCreate(&r->end) == cudaSuccess)
        cudaEventRecord(r->start, st);
    else
        cudaGetLastError();
    uint64_t h2d = 0, d2h = 0;
    for (auto &up : r->uploads)
        if (err == GB300_OK) err = upload_tables(s, up.first, up.second, st);
    // tables uploaded by rounds on other streams
    std::vector<std::pair<Topology *, int>> seen;
    for (Request *q : r->reqs) {
        const std::pair<Topology *, int> key(q->topo, unit_of(q->r.kind));
        if (std::find(seen.begin(), seen.end(), key) == seen.end()) {
            seen.push_back(key);
            chk(cudaStreamWaitEvent(st, q->topo->unit[key.second].ready, 0),
                "GB300Server table wait");
        }
    }
    std::vector<double> mean;
    // inputs
    for (Request *q : r->reqs) {
        char *a = s->arena.at(q->arenaOff);
        const GB300TopologyDesc &d = q->topo->d;
        chk(cudaMemcpyAsync(a + q->oCv, q->r.controlValues, (size_t)d.numControl * d.length * 4,
                            cudaMemcpyHostToDevice, st), "GB300Server input copy");
        h2d += (size_t)d.numControl * d.length * 4;
        if (q->r.kind == GB300_REQUEST_LIMIT) {
            const size_t n = (size_t)q->r.numPoints * 4;
            h2d += 3 * n;
            chk(cudaMemcpyAsync(a + q->oFaces, q->r.faces, n, cudaMemcpyHostToDevice, st),
                "GB300Server input copy");
            chk(cudaMemcpyAsync(a + q->oU, q->r.u, n, cudaMemcpyHostToDevice, st),
                "GB300Server input copy");
            chk(cudaMemcpyAsync(a + q->oV, q->r.v, n, cudaMemcpyHostToDevice, st),
                "GB300Server input copy");
        }
    }
    // stencil work: refine tables, and the patch points of every limit request
    for (Request *q : r->reqs) {
        Topology *t = q->topo;
        char *a = s->arena.at(q->arenaOff);
        char *b = s->tables.at(t->unit[unit_of(q->r.kind)].poolOff);
        const GB300TopologyDesc &d = t->d;
        const float *cv = (const float *)(a + q->oCv);
        if (q->r.kind == GB300_REQUEST_REFINE) {
            if (d.numStencils == 0) continue;
            if (s->cfg.plain) {
                float *dsts[6] = {(float *)(a + q->oOut), 0, 0, 0, 0, 0};
                int strides[6] = {d.length, 0, 0, 0, 0, 0};
                const float *ws[6] = {(const float *)(b + t->oWeights), 0, 0, 0, 0, 0};
                if (err == GB300_OK)
                    err = eval_stencils(cv, dsts, strides, ws, d.length, d.length,
                                        (const int *)(b + t->oSizes),
                                        (const int *)(b + t->oOffsets),
                                        (const int *)(b + t->oIndices), 0, d.numStencils, st,
                                        "GB300Server refine");
                continue;
            }
            r->jobs.push_back(stencil_job((const int *)(b + t->oSizes),
                                          (const int *)(b + t->oOffsets),
                                          (const int *)(b + t->oIndices),
                                          (const float *)(b + t->oWeights), d.numStencils, cv,
                                          (float *)(a + q->oOut), d.length, d.length, d.length));
            mean.push_back(t->refineMean);
        } else {
            if (d.numPatchPoints == 0) continue;
            float *ps = (float *)(a + q->oPatchSrc);
            if (s->cfg.plain) {
                float *dsts[6] = {ps, 0, 0, 0, 0, 0};
                int strides[6] = {3, 0, 0, 0, 0, 0};
                const float *ws[6] = {(const float *)(b + t->oPpWeights), 0, 0, 0, 0, 0};
                if (err == GB300_OK)
                    err = eval_stencils(cv, dsts, strides, ws, 3, d.length,
                                        (const int *)(b + t->oPpSizes),
                                        (const int *)(b + t->oPpOffsets),
                                        (const int *)(b + t->oPpIndices), 0, d.numPatchPoints, st,
                                        "GB300Server patch points");
                continue;
            }
            r->jobs.push_back(stencil_job((const int *)(b + t->oPpSizes),
                                          (const int *)(b + t->oPpOffsets),
                                          (const int *)(b + t->oPpIndices),
                                          (const float *)(b + t->oPpWeights), d.numPatchPoints,
                                          cv, ps, 3, d.length, 3));
            mean.push_back(t->ppMean);
        }
    }
    if (!r->jobs.empty() && err == GB300_OK) {
        const int n = (int)r->jobs.size();
        r->tileBase.resize(n + 1);
        const int tiles =
            batch::plan_tiles(r->jobs.data(), mean.data(), n, 256, 64, r->tileBase.data());
        char *meta = s->arena.at(r->metaOff);
        const size_t jobBytes = align256((size_t)n * sizeof(batch::Job));
        const size_t baseBytes = align256((size_t)(n + 1) * sizeof(int));
        chk(cudaMemcpyAsync(meta, r->jobs.data(), n * sizeof(batch::Job),
                            cudaMemcpyHostToDevice, st), "GB300Server job table");
        chk(cudaMemcpyAsync(meta + jobBytes, r->tileBase.data(), (n + 1) * sizeof(int),
                            cudaMemcpyHostToDevice, st), "GB300Server job table");
        if (err == GB300_OK) {
            int *counter = (int *)(meta + jobBytes + baseBytes);
            err = batch::launch_jobs((const batch::Job *)meta, (const int *)(meta + jobBytes), n,
                                     tiles, counter, counter + 1, 2, st);
        }
    }
    // limit: PatchMap lookup and EvalPatches (P, dPdu, dPdv) per request
    for (Request *q : r->reqs) {
        if (q->r.kind != GB300_REQUEST_LIMIT || q->r.numPoints == 0 || err != GB300_OK) continue;
        Topology *t = q->topo;
        char *a = s->arena.at(q->arenaOff);
        char *b = s->tables.at(t->unit[1].poolOff);
        const int n = q->r.numPoints;
        err = find_patches(device_map(s, t), n, (const int *)(a + q->oFaces),
                           (const float *)(a + q->oU), (const float *)(a + q->oV),
                           a + q->oCoords, st);
        if (err != GB300_OK) break;
        float *out = (float *)(a + q->oOut);
        float *dsts[6] = {out, out + (size_t)n * 3, out + (size_t)n * 6, 0, 0, 0};
        int strides[6] = {3, 3, 3, 0, 0, 0};
        err = eval_patches((const float *)(a + q->oPatchSrc), dsts, strides, 3, 3, n,
                           a + q->oCoords, b + t->oArrays, (const int *)(b + t->oPIndices),
                           b + t->oParams, st, "GB300Server limit", t->quadFamily);
    }
    // results back to the host
    for (Request *q : r->reqs) {
        const size_t bytes = out_bytes(*q);
        d2h += bytes;
        if (bytes)
            chk(cudaMemcpyAsync(q->r.out, s->arena.at(q->arenaOff) + q->oOut, bytes,
                                cudaMemcpyDeviceToHost, st), "GB300Server output copy");
    }
    if (r->end) cudaEventRecord(r->end, st);
    chk(cudaLaunchHostFunc(st, on_round_done, r), "GB300Server completion callback");
    {
        std::lock_guard<std::mutex> lock(s->m);
        s->stats.h2dBytes += h2d;
        s->stats.d2hBytes += d2h;
    }
#undef chk
    return err;
}

void finish_request(GB300Server *s, Request *q, int status, Clock::time_point t) {
    q->status = status;
    q->latency = std::chrono::duration<double>(t - q->tSubmit).count();
    if (status == GB300_OK)
        s->stats.completed++;
    else
        s->stats.failed++;
}

// Reaps finished rounds; called with the lock held.
void reap(GB300Server *s) {
    for (size_t i = 0; i < s->inflight.size();) {
        Round *r = s->inflight[i].get();
        if (!r->done.load()) {
            ++i;
            continue;
        }
        for (Request *q : r->reqs) {
            s->arena.release(q->arenaOff, q->lay.total);
            q->topo->unit[unit_of(q->r.kind)].pins--;
            finish_request(s, q, GB300_OK, r->tDone);
        }
        if (r->metaBytes) s->arena.release(r->metaOff, r->metaBytes);
        float ms = 0.0f;
        if (r->start && r->end && cudaEventElapsedTime(&ms, r->start, r->end) == cudaSuccess)
            s->stats.roundDeviceNanos += (uint64_t)(ms * 1e6);
        else
            cudaGetLastError();
        s->streamBusy[r->stream] = 0;
        s->inflight.erase(s->inflight.begin() + i);
        s->doneCv.notify_all();
    }
}

void scheduler(GB300Server *s) {
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lock(s->m);
    const int maxPer = s->cfg.plain ? 1 : std::max(1, s->cfg.maxRequestsPerRound);
    for (;;) {
        reap(s);
        if (s->stop && s->pending.empty() && s->inflight.empty()) return;
        int free = -1;
        for (size_t k = 0; k < s->streams.size(); ++k)
            if (!s->streamBusy[k]) {
                free = (int)k;
                break;
            }
        if (free < 0 || s->pending.empty()) {
            const auto w0 = Clock::now();
            s->cv.wait_for(lock, std::chrono::microseconds(200));
            if (!s->pending.empty())
                s->stats.streamsBusyNanos += (uint64_t)(seconds_since(w0) * 1e9);
            continue;
        }
        auto round = std::make_unique<Round>();
        round->srv = s;
        round->stream = free;
        cudaStream_t st = s->streams[free];
        // round metadata (job table, tile prefix, counter/status): sized for maxPer jobs
        round->metaBytes = align256((size_t)maxPer * sizeof(batch::Job)) +
                           align256((size_t)(maxPer + 1) * sizeof(int)) + 256;
        if (!s->arena.alloc(round->metaBytes, round->metaOff)) {
            round->metaBytes = 0;
            const auto w0 = Clock::now();
            s->cv.wait_for(lock, std::chrono::microseconds(200));
            s->stats.memoryWaitNanos += (uint64_t)(seconds_since(w0) * 1e9);
            continue;
        }
        while (!s->pending.empty() && (int)round->reqs.size() < maxPer) {
            Request *q = s->pending.front();
            const int k = unit_of(q->r.kind);
            Topology::Unit &u = q->topo->unit[k];
            if (!s->arena.alloc(q->lay.total, q->arenaOff)) break;
            if (!reserve(s, q->topo, k)) {  // wait for in-flight rounds to unpin tables
                s->arena.release(q->arenaOff, q->lay.total);
                break;
            }
            if (u.needsUpload) {
                u.needsUpload = false;
                round->uploads.emplace_back(q->topo, k);
            }
            u.pins++;
            u.lastUse = ++s->useClock;
            s->pending.pop_front();
            round->reqs.push_back(q);
        }
        if (round->reqs.empty()) {
            s->arena.release(round->metaOff, round->metaBytes);
            const auto w0 = Clock::now();
            s->cv.wait_for(lock, std::chrono::microseconds(200));
            s->stats.memoryWaitNanos += (uint64_t)(seconds_since(w0) * 1e9);
            continue;
        }
        s->streamBusy[free] = 1;
        s->stats.rounds++;
        Round *r = round.get();
        s->inflight.push_back(std::move(round));
        // launch outside the lock (the completion callback takes it)
        lock.unlock();
        const auto l0 = Clock::now();
        const int err = launch_round(s, r);
        const uint64_t launchNs = (uint64_t)(seconds_since(l0) * 1e9);
        lock.lock();
        s->stats.launchNanos += launchNs;
        if (err != GB300_OK) {
            // the callback may still run if it was queued; wait for the stream to drain
            lock.unlock();
            cudaStreamSynchronize(st);
            lock.lock();
            for (Request *q : r->reqs) {
                s->arena.release(q->arenaOff, q->lay.total);
                q->topo->unit[unit_of(q->r.kind)].pins--;
                finish_request(s, q, err, Clock::now());
            }
            for (auto &up : r->uploads) {  // their tables may be incomplete: drop them
                Topology::Unit &u = up.first->unit[up.second];
                if (u.resident) {
                    s->tables.release(u.poolOff, u.lay.total);
                    u.resident = false;
                    s->stats.residentBytes -= u.lay.total;
                }
            }
            s->arena.release(r->metaOff, r->metaBytes);
            s->streamBusy[free] = 0;
            for (size_t i = 0; i < s->inflight.size(); ++i)
                if (s->inflight[i].get() == r) {
                    s->inflight.erase(s->inflight.begin() + i);
                    break;
                }
            s->doneCv.notify_all();
        }
    }
}

}  // namespace serve
}  // namespace gb300

extern "C" {

GB300Server *GB300ServerCreate(const GB300ServerConfig *cfg) {
    if (!cfg || cfg->streams < 1 || cfg->streams > 64 || cfg->maxRequestsPerRound < 1 ||
        cfg->tableBudgetBytes == 0 || cfg->arenaBytes == 0) {
        fail(GB300_ERR_INVALID_ARGUMENT, "GB300ServerCreate: bad configuration");
        return nullptr;
    }
    auto s = std::make_unique<GB300Server>();
    s->cfg = *cfg;
    if (s->cfg.plain) s->cfg.streams = 1;
    if (check_cuda(cudaGetDevice(&s->device), "GB300ServerCreate") != GB300_OK) return nullptr;
    if (!s->tables.init(cfg->tableBudgetBytes, "GB300ServerCreate table pool") ||
        !s->arena.init(cfg->arenaBytes, "GB300ServerCreate request arena"))
        return nullptr;
    for (int k = 0; k < s->cfg.streams; ++k) {
        cudaStream_t st;
        if (check_cuda(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking),
                       "GB300ServerCreate stream") != GB300_OK) {
            for (cudaStream_t x : s->streams) cudaStreamDestroy(x);
            return nullptr;
        }
        s->streams.push_back(st);
        s->streamBusy.push_back(0);
    }
    GB300Server *p = s.release();
    p->worker = std::thread(scheduler, p);
    ok();
    return p;
}

void GB300ServerDestroy(GB300Server *s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lock(s->m);
        s->stop = true;
    }
    s->cv.notify_all();
    if (s->worker.joinable()) s->worker.join();
    for (cudaStream_t st : s->streams) cudaStreamDestroy(st);
    for (auto &kv : s->topos)
        for (Topology::Unit &u : kv.second->unit)
            if (u.ready) cudaEventDestroy(u.ready);
    for (void *p : s->registered) cudaHostUnregister(p);
    for (void *c : s->caches) GB300TableCacheClose(c);
    delete s;
}

int GB300ServerAddTopology(GB300Server *s, int id, const GB300TopologyDesc *d) {
    const char *who = "GB300ServerAddTopology";
    if (!s || !d) return fail(GB300_ERR_INVALID_ARGUMENT, "%s: null argument", who);
    if (d->numControl <= 0 || d->length <= 0 || d->numStencils < 0 || d->nnz < 0 ||
        (d->numStencils > 0 && (!d->sizes || !d->offsets)) ||
        (d->nnz > 0 && (!d->indices || !d->weights)))
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: bad refine table", who);
    auto t = std::make_unique<Topology>();
    t->id = id;
    t->d = *d;
    t->limit = d->numPatchArrays > 0;
    if (t->limit) {
        if (d->length < 3 || d->numPatchPoints <= 0 || d->patchPointNnz <= 0 || !d->ppSizes ||
            !d->ppOffsets || !d->ppIndices || !d->ppWeights || !d->patchArrays ||
            !d->patchIndices || !d->patchParams || d->numPatches <= 0)
            return fail(GB300_ERR_INVALID_ARGUMENT, "%s: bad limit tables", who);
        if (build_patch_map(d->numPatchArrays, (const int *)d->patchArrays, d->numPatches,
                            (const int *)d->patchParams, d->triangular, t->map) != GB300_OK)
            return GB300_ERR_INVALID_ARGUMENT;
        const int *arr = (const int *)d->patchArrays;
        t->quadFamily = 1;
        for (int a = 0; a < d->numPatchArrays; ++a)
            for (int k = 0; k < 2; ++k) {
                const int type = arr[6 * a + k];
                if (type != GB300_PATCH_REGULAR && type != GB300_PATCH_GREGORY_BASIS &&
                    type != GB300_PATCH_QUADS)
                    t->quadFamily = 0;
            }
    }
    t->refineMean = d->numStencils ? (double)d->nnz / d->numStencils : 0;
    t->ppMean = d->numPatchPoints ? (double)d->patchPointNnz / d->numPatchPoints : 0;
    Layout &L0 = t->unit[0].lay;
    t->oSizes = L0.add((size_t)d->numStencils * 4);
    t->oOffsets = L0.add((size_t)d->numStencils * 4);
    t->oIndices = L0.add((size_t)d->nnz * 4);
    t->oWeights = L0.add((size_t)d->nnz * 4);
    Layout &L = t->unit[1].lay;
    if (t->limit) {
        t->oPpSizes = L.add((size_t)d->numPatchPoints * 4);
        t->oPpOffsets = L.add((size_t)d->numPatchPoints * 4);
        t->oPpIndices = L.add((size_t)d->patchPointNnz * 4);
        t->oPpWeights = L.add((size_t)d->patchPointNnz * 4);
        t->oArrays = L.add((size_t)d->numPatchArrays * 24);
        t->oPIndices = L.add((size_t)d->numPatchIndices * 4);
        t->oParams = L.add((size_t)d->numPatches * 12);
        t->oNodes = L.add(t->map.nodes.size() * 4);
        t->oHandles = L.add(t->map.handles.size() * 4);
    }
    if (std::max(L0.total, L.total) > s->tables.capacity())
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: topology %d needs %zu bytes, budget %zu",
                    who, id, std::max(L0.total, L.total), s->tables.capacity());
    for (Topology::Unit &u : t->unit) {
        const int st = check_cuda(cudaEventCreateWithFlags(&u.ready, cudaEventDisableTiming), who);
        if (st != GB300_OK) {
            for (Topology::Unit &v : t->unit)
                if (v.ready) cudaEventDestroy(v.ready);
            return st;
        }
    }
    std::vector<void *> pinned;  // CUDA calls stay outside the server lock
    uint64_t pinnedBytes = 0, pinFailures = 0;
    if (s->cfg.pinHostTables) {
        // page-lock the arrays uploads read from; ranges another topology already registered
        // (shared tables) are left as they are, and a range that cannot be registered stays
        // pageable (its uploads are then staged by the driver)
        auto pin = [&](const void *p, size_t bytes) {
            if (!p || !bytes) return;
            const cudaError_t e = cudaHostRegister(const_cast<void *>(p), bytes,
                                                   cudaHostRegisterDefault);
            if (e == cudaSuccess) {
                pinned.push_back(const_cast<void *>(p));
                pinnedBytes += bytes;
            } else {
                if (e != cudaErrorHostMemoryAlreadyRegistered) ++pinFailures;
                cudaGetLastError();
            }
        };
        pin(d->sizes, (size_t)d->numStencils * 4);
        pin(d->offsets, (size_t)d->numStencils * 4);
        pin(d->indices, (size_t)d->nnz * 4);
        pin(d->weights, (size_t)d->nnz * 4);
        if (t->limit) {
            pin(d->ppSizes, (size_t)d->numPatchPoints * 4);
            pin(d->ppOffsets, (size_t)d->numPatchPoints * 4);
            pin(d->ppIndices, (size_t)d->patchPointNnz * 4);
            pin(d->ppWeights, (size_t)d->patchPointNnz * 4);
            pin(d->patchIndices, (size_t)d->numPatchIndices * 4);
            pin(d->patchParams, (size_t)d->numPatches * 12);
            pin(t->map.nodes.data(), t->map.nodes.size() * 4);
            pin(t->map.handles.data(), t->map.handles.size() * 4);
        }
    }
    std::lock_guard<std::mutex> lock(s->m);
    s->registered.insert(s->registered.end(), pinned.begin(), pinned.end());
    s->stats.hostPinnedBytes += pinnedBytes;
    s->stats.hostPinFailures += pinFailures;
    auto it = s->topos.find(id);
    if (it != s->topos.end()) {
        for (Topology::Unit &u : t->unit) cudaEventDestroy(u.ready);
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: topology %d already registered", who, id);
    }
    s->topos[id] = std::move(t);
    return ok();
}

int GB300ServerAddTopologyFromCache(GB300Server *s, int id, const char *path) {
    if (!s) return fail(GB300_ERR_INVALID_ARGUMENT, "GB300ServerAddTopologyFromCache: null server");
    GB300TopologyDesc d;
    void *h = nullptr;
    int st = GB300TableCacheOpen(path, 1, &d, &h);
    if (st != GB300_OK) return st;
    st = GB300ServerAddTopology(s, id, &d);
    if (st != GB300_OK) {
        GB300TableCacheClose(h);
        return st;
    }
    std::lock_guard<std::mutex> lock(s->m);
    s->caches.push_back(h);
    return ok();
}

int GB300ServerSubmit(GB300Server *s, const GB300Request *r, uint64_t *ticket) {
    const char *who = "GB300ServerSubmit";
    if (!s || !r || !ticket) return fail(GB300_ERR_INVALID_ARGUMENT, "%s: null argument", who);
    auto q = std::make_unique<Request>();
    q->r = *r;
    q->tSubmit = Clock::now();
    std::lock_guard<std::mutex> lock(s->m);
    auto it = s->topos.find(r->topology);
    if (it == s->topos.end())
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: unknown topology %d", who, r->topology);
    q->topo = it->second.get();
    if (r->kind != GB300_REQUEST_REFINE && r->kind != GB300_REQUEST_LIMIT)
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: unknown request kind %d", who, r->kind);
    if (!r->controlValues || !r->out)
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: null control values or output", who);
    if (r->kind == GB300_REQUEST_LIMIT &&
        (!q->topo->limit || r->numPoints < 0 ||
         (r->numPoints > 0 && (!r->faces || !r->u || !r->v))))
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: bad limit request for topology %d", who,
                    r->topology);
    plan_request(*q);
    if (q->lay.total + 65536 > s->arena.capacity())
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: request needs %zu bytes, arena %zu", who,
                    q->lay.total, s->arena.capacity());
    *ticket = s->firstTicket + s->all.size();
    s->pending.push_back(q.get());
    s->all.push_back(std::move(q));
    s->stats.submitted++;
    s->cv.notify_all();
    return ok();
}

int GB300ServerWait(GB300Server *s, uint64_t ticket, double *latencySeconds) {
    if (!s) return fail(GB300_ERR_INVALID_ARGUMENT, "GB300ServerWait: null server");
    std::unique_lock<std::mutex> lock(s->m);
    if (ticket < s->firstTicket || ticket >= s->firstTicket + s->all.size())
        return fail(GB300_ERR_INVALID_ARGUMENT, "GB300ServerWait: unknown ticket");
    Request *q = s->all[ticket - s->firstTicket].get();
    s->doneCv.wait(lock, [&] { return q->status >= 0; });
    if (latencySeconds) *latencySeconds = q->latency;
    if (q->status != GB300_OK)
        return fail(q->status, "GB300ServerWait: request %llu failed",
                    (unsigned long long)ticket);
    return ok();
}

int GB300ServerReplay(GB300Server *s, int n, const GB300Request *reqs,
                      const double *arrivalSeconds, double *latencySeconds) {
    if (!s || n < 0 || (n > 0 && (!reqs || !arrivalSeconds)))
        return fail(GB300_ERR_INVALID_ARGUMENT, "GB300ServerReplay: bad arguments");
    std::vector<uint64_t> tickets(n);
    const Clock::time_point t0 = Clock::now();
    int first = GB300_OK;
    int submitted = 0;
    for (; submitted < n; ++submitted) {
        const int i = submitted;
        // open loop: submit at the trace's arrival time (spin for the last 50 us)
        for (;;) {
            const double wait = arrivalSeconds[i] - seconds_since(t0);
            if (wait <= 0) break;
            if (wait > 60e-6)
                std::this_thread::sleep_for(std::chrono::duration<double>(wait - 50e-6));
        }
        const int st = GB300ServerSubmit(s, &reqs[i], &tickets[i]);
        if (st != GB300_OK) {
            first = st;
            break;
        }
    }
    // wait for everything submitted, even after a rejected request: the requests' buffers
    // belong to the caller, who may free them once this returns
    for (int i = 0; i < n; ++i) {
        double lat = -1;
        if (i < submitted) {
            const int st = GB300ServerWait(s, tickets[i], &lat);
            if (st != GB300_OK && first == GB300_OK) first = st;
        }
        if (latencySeconds) latencySeconds[i] = lat;
    }
    return first == GB300_OK ? ok() : first;
}

int GB300ServerGetStats(GB300Server *s, GB300ServerStats *out) {
    if (!s || !out) return fail(GB300_ERR_INVALID_ARGUMENT, "GB300ServerGetStats: null argument");
    std::lock_guard<std::mutex> lock(s->m);
    *out = s->stats;
    return ok();
}

}  // extern "C"
