// GPU stencil-table factory: Far::StencilTableFactory's factorized tables
// (far/stencilTableFactory.cpp:78-151) and StencilBuilder compositions over a base table
// (LimitStencilTableFactory's per-location stencils, AppendLocalPointStencilTable;
// far/stencilTableFactory.cpp:255-407,560-640) built on the device from masks recorded on the
// host.
//
// Far's StencilBuilder builds a row by merging (index, weight) terms: a term whose index is
// already in the row is added to that entry, otherwise it is appended (WeightTable::merge /
// add, far/stencilBuilder.cpp:310-385).  A mask entry (source s, weight m) contributes m for a
// control vertex and w * m for each entry (i, w) of s's factorized row otherwise
// (WeightTable::AddWithWeight, :164-198); with a StencilReal source, entries with w == 0 are
// skipped and every weight channel is multiplied (:520-598).  Products and sums are single
// IEEE float operations, so the device rows equal Far's bit for bit.
//
// Device plan, per refinement level: rows are grouped into dependency waves (Catmark edge and
// vertex points read face points of their own level); per wave a COUNT pass sizes every row,
// a scan turns sizes into offsets in one arena of (index, weight) entries, and a FILL pass
// writes the rows.  One warp builds one row: each 32-entry chunk of a source row is merged at
// once -- lanes look their index up in the row built so far (shared memory, or the arena for
// long rows) and new indices are appended in lane order, which is the reference's sequential
// first-touch order because the indices of one source row are distinct.  Finally the wanted
// rows are copied into the output table (optionally with each stencil's entries sorted by
// control index).
#include "common.cuh"
#include "patch_basis.cuh"
#include "patchmap.h"
#include "tables.h"

#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <new>
#include <type_traits>
#include <vector>

namespace gb300 {
namespace factory {

constexpr int kCap = 256;  // entries of a row kept in shared memory
constexpr unsigned kFull = 0xffffffffu;

// status bits
constexpr int kNeedScratch = 1;  // a count pass ran out of scratch (rerun with more)
constexpr int kOverflow = 2;     // a fill pass produced more entries than counted
constexpr int kBadSource = 4;    // a mask names a source outside the allowed range
constexpr int kBadBase = 8;      // a base stencil's entry range lies outside its arrays

template <int NC>
constexpr int warps_of() { return NC == 6 ? 4 : 8; }

// Factorized source rows.  identity: sources below numControl are control vertices (one entry
// of weight 1); other sources s read meta row s - numControl.  Otherwise source s reads meta
// row s (a base table).
struct Rows {
    int numControl;
    int identity;
    const int *size;
    const long long *off;
    const int *idx;
    const float *w;
};

template <int NC>
struct Pass {
    Rows rows;
    const long long *moff;  // masks of the pass's rows (row-local)
    const int *msrc;
    const float *mw[NC];
    int numRows;
    const int *wave;  // per row (null: every row belongs to the pass)
    int waveId;
    int metaBase;  // meta index of row 0
    int *metaSize;
    const long long *metaOff;
    int *arenaIdx;
    float *arenaW[NC];
    int skipZero;     // skip zero entries of source rows (StencilReal sources)
    int rowsInArena;  // source rows live in the arena the pass appends to (factory levels)
    int *scratch;  // count-pass lists of rows whose term bound exceeds kCap
    long long scratchCap;
    unsigned long long *scratchUsed;
    int *status;
};

__device__ __forceinline__ void source_row(const Rows &r, int s, int &n, const int *&idx,
                                           const float *&w) {
    if (r.identity && s < r.numControl) {
        n = 1;
        idx = nullptr;
        w = nullptr;
        return;
    }
    const int g = r.identity ? s - r.numControl : s;
    n = r.size[g];
    const long long o = r.off[g];
    idx = r.idx + o;
    w = r.w + o;
}

template <int NC>
__device__ __forceinline__ bool mask_entry(const Pass<NC> &p, long long k, int &s, float (&m)[NC]) {
    s = p.msrc[k];
    bool any = false;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        m[c] = p.mw[c][k];
        any |= m[c] != 0.0f;
    }
    return any;
}

// Upper bound of a row's entry count: the number of terms its masks produce.
template <int NC>
__device__ long long term_bound(const Pass<NC> &p, int r, int lane) {
    long long t = 0;
    for (long long k = p.moff[r] + lane; k < p.moff[r + 1]; k += 32) {
        int s;
        float m[NC];
        if (!mask_entry(p, k, s, m)) continue;
        int n;
        const int *i;
        const float *w;
        source_row(p.rows, s, n, i, w);
        t += n;
    }
#pragma unroll
    for (int d = 16; d; d >>= 1) t += __shfl_xor_sync(kFull, t, d);
    return t;
}

// Builds row r into keys[0, n) (and v[c][0, n) when FILL); returns n.  keys / v may be shared
// or global memory; at most `cap` entries are written (more sets kOverflow).
template <int NC, bool FILL>
__device__ int merge_row(const Pass<NC> &p, int r, int *keys, float *const (&v)[NC], int cap,
                         int lane) {
    int n = 0;
    const unsigned lt = (1u << lane) - 1u;
    for (long long k = p.moff[r], k1 = p.moff[r + 1]; k < k1; ++k) {
        int s;
        float m[NC];
        if (!mask_entry(p, k, s, m)) continue;
        int rs;
        const int *ri;
        const float *rw;
        source_row(p.rows, s, rs, ri, rw);
        for (int e0 = 0; e0 < rs; e0 += 32) {
            const int e = e0 + lane;
            bool act = e < rs;
            int q = -1;
            float x = 0.0f;
            if (act) {
                q = ri ? ri[e] : s;
                x = ri ? rw[e] : 1.0f;
                if (p.skipZero && x == 0.0f) act = false;
            }
            int pos = -1;
            for (int i = 0; i < n; ++i)
                if (keys[i] == q) pos = i;
            const bool fresh = act && pos < 0;
            const unsigned fb = __ballot_sync(kFull, fresh);
            if (fresh) {
                pos = n + __popc(fb & lt);
                if (pos < cap) {
                    keys[pos] = q;
                    if (FILL) {
#pragma unroll
                        for (int c = 0; c < NC; ++c) v[c][pos] = __fmul_rn(m[c], x);
                    }
                } else {
                    atomicOr(p.status, kOverflow);
                }
            } else if (act && FILL) {
#pragma unroll
                for (int c = 0; c < NC; ++c)
                    v[c][pos] = __fadd_rn(v[c][pos], __fmul_rn(m[c], x));
            }
            n = min(n + __popc(fb), cap);
            __syncwarp();
        }
    }
    return n;
}

template <int NC>
__global__ void __launch_bounds__(warps_of<NC>() * 32) k_count(Pass<NC> p) {
    constexpr int W = warps_of<NC>();
    __shared__ int skeys[W][kCap];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    float *const none[NC] = {};
    for (int r = blockIdx.x * W + wib; r < p.numRows; r += gridDim.x * W) {
        if (p.wave && p.wave[r] != p.waveId) continue;
        const long long t = term_bound(p, r, lane);
        int *keys = skeys[wib];
        int cap = kCap;
        if (t > kCap) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(p.scratchUsed, (unsigned long long)t);
            base = __shfl_sync(kFull, base, 0);
            if ((long long)(base + t) > p.scratchCap) {
                if (lane == 0) atomicOr(p.status, kNeedScratch);
                continue;
            }
            keys = p.scratch + base;
            cap = (int)min(t, (long long)0x7fffffff);
        }
        const int n = merge_row<NC, false>(p, r, keys, none, cap, lane);
        if (lane == 0) p.metaSize[p.metaBase + r] = n;
        __syncwarp();
    }
}

template <int NC>
__global__ void __launch_bounds__(warps_of<NC>() * 32) k_fill(Pass<NC> p) {
    constexpr int W = warps_of<NC>();
    __shared__ int skeys[W][kCap];
    __shared__ float svals[W][NC][kCap];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    for (int r = blockIdx.x * W + wib; r < p.numRows; r += gridDim.x * W) {
        if (p.wave && p.wave[r] != p.waveId) continue;
        const int n = p.metaSize[p.metaBase + r];
        const long long o = p.metaOff[p.metaBase + r];
        if (n <= kCap) {
            float *v[NC];
#pragma unroll
            for (int c = 0; c < NC; ++c) v[c] = svals[wib][c];
            const int got = merge_row<NC, true>(p, r, skeys[wib], v, n, lane);
            for (int i = lane; i < got; i += 32) {
                p.arenaIdx[o + i] = skeys[wib][i];
#pragma unroll
                for (int c = 0; c < NC; ++c) p.arenaW[c][o + i] = svals[wib][c][i];
            }
        } else {
            float *v[NC];
#pragma unroll
            for (int c = 0; c < NC; ++c) v[c] = p.arenaW[c] + o;
            merge_row<NC, true>(p, r, p.arenaIdx + o, v, n, lane);
        }
        __syncwarp();
    }
}

// Term bounds of the pass's rows (0 for rows of other waves); element n is 0.
template <int NC>
__global__ void k_bounds(Pass<NC> p, long long *out) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r <= p.numRows;
         r += gridDim.x * blockDim.x) {
        long long t = 0;
        if (r < p.numRows && (!p.wave || p.wave[r] == p.waveId)) {
            for (long long k = p.moff[r]; k < p.moff[r + 1]; ++k) {
                int s;
                float m[NC];
                if (!mask_entry(p, k, s, m)) continue;
                int n;
                const int *i;
                const float *w;
                source_row(p.rows, s, n, i, w);
                t += n;
            }
        }
        out[r] = t;
    }
}

// Single merge pass: row r owns bound[r] entries of the arena from metaOff; it is built in
// shared memory when that bound fits (then copied out) and in place otherwise.  Writes the
// row's entry count.
template <int NC>
__global__ void __launch_bounds__(warps_of<NC>() * 32) k_merge1(Pass<NC> p,
                                                                const long long *bound) {
    constexpr int W = warps_of<NC>();
    __shared__ int skeys[W][kCap];
    __shared__ float svals[W][NC][kCap];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    for (int r = blockIdx.x * W + wib; r < p.numRows; r += gridDim.x * W) {
        if (p.wave && p.wave[r] != p.waveId) continue;
        const long long cap = bound[r];
        const long long o = p.metaOff[p.metaBase + r];
        int n;
        if (cap <= kCap) {
            float *v[NC];
#pragma unroll
            for (int c = 0; c < NC; ++c) v[c] = svals[wib][c];
            n = merge_row<NC, true>(p, r, skeys[wib], v, (int)cap, lane);
            for (int i = lane; i < n; i += 32) {
                p.arenaIdx[o + i] = skeys[wib][i];
#pragma unroll
                for (int c = 0; c < NC; ++c) p.arenaW[c][o + i] = svals[wib][c][i];
            }
        } else {
            float *v[NC];
#pragma unroll
            for (int c = 0; c < NC; ++c) v[c] = p.arenaW[c] + o;
            n = merge_row<NC, true>(p, r, p.arenaIdx + o, v,
                                    (int)min(cap, (long long)0x7fffffff), lane);
        }
        if (lane == 0) p.metaSize[p.metaBase + r] = n;
        __syncwarp();
    }
}

// Dependency waves of one level's rows: 0 when no source lies in the level itself, -1 (to be
// assigned) otherwise.  Also checks every source: a control vertex, a vertex of the previous
// level [prevFirst, levelFirst) or of this level.
__global__ void k_wave_init(const long long *moff, const int *msrc, int n, int numControl,
                            int prevFirst, int levelFirst, int *wave, int *pending, int *status) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        bool dep = false, bad = false;
        for (long long k = moff[r]; k < moff[r + 1]; ++k) {
            const int s = msrc[k];
            if (s < 0 || s >= levelFirst + n || (s >= numControl && s < prevFirst)) bad = true;
            dep |= s >= levelFirst;
        }
        if (bad) atomicOr(status, kBadSource);
        wave[r] = dep ? -1 : 0;
        if (dep) atomicAdd(pending, 1);
    }
}

// Rows still unassigned whose same-level sources all lie in waves [0, w) join wave w.
__global__ void k_wave_step(const long long *moff, const int *msrc, int n, int levelFirst, int w,
                            int *wave, int *assigned) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        if (wave[r] != -1) continue;
        bool ready = true;
        for (long long k = moff[r]; k < moff[r + 1] && ready; ++k) {
            const int s = msrc[k];
            if (s >= levelFirst) {
                const int ws = wave[s - levelFirst];
                ready = ws >= 0 && ws < w;
            }
        }
        if (ready) {
            wave[r] = w;
            atomicAdd(assigned, 1);
        }
    }
}

// sizes of the wave's rows (0 for the others), for the offset scan; element n is 0
__global__ void k_wave_sizes(const int *metaSize, int metaBase, const int *wave, int w, int n,
                             long long *out) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r <= n; r += gridDim.x * blockDim.x)
        out[r] = (r < n && (!wave || wave[r] == w)) ? metaSize[metaBase + r] : 0;
}

__global__ void k_wave_offsets(const long long *scan, const int *wave, int w, int n,
                               long long base, long long *metaOff, int metaBase) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
        if (!wave || wave[r] == w) metaOff[metaBase + r] = base + scan[r];
}

// Base table rows: 64-bit offsets plus a range check of every stencil.
__global__ void k_base_rows(const int *sizes, const int *offsets, int n, long long nnz,
                            long long *off64, int *status) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const long long o = offsets[r], s = sizes[r];
        if (s < 0 || o < 0 || o + s > nnz) atomicOr(status, kBadBase);
        off64[r] = o;
    }
}

__global__ void k_check_sources(const int *msrc, long long nnz, int limit, int *status) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nnz;
         k += (long long)gridDim.x * blockDim.x)
        if (msrc[k] < 0 || msrc[k] >= limit) atomicOr(status, kBadSource);
}

// The output table: nIdentity identity stencils, then nBase base stencils, then meta rows
// [metaFirst, metaFirst + nMeta).
struct Assemble {
    int nIdentity;
    int nBase;
    const int *bSize;
    const long long *bOff;
    const int *bIdx;
    const float *bW;
    int nMeta, metaFirst;
    const int *mSize;
    const long long *mOff;
    const int *aIdx;
    const float *aW[6];
    int nc;
    int sort;
};

__device__ __forceinline__ int out_row(const Assemble &a, int i, const int *&idx,
                                       const float *(&w)[6], int &self) {
    self = -1;
    if (i < a.nIdentity) {
        self = i;
        return 1;
    }
    i -= a.nIdentity;
    if (i < a.nBase) {
        const long long o = a.bOff[i];
        idx = a.bIdx + o;
        w[0] = a.bW + o;
        for (int c = 1; c < 6; ++c) w[c] = nullptr;
        return a.bSize[i];
    }
    i -= a.nBase;
    const long long o = a.mOff[a.metaFirst + i];
    idx = a.aIdx + o;
    for (int c = 0; c < 6; ++c) w[c] = c < a.nc ? a.aW[c] + o : nullptr;
    return a.mSize[a.metaFirst + i];
}

__global__ void k_out_sizes(Assemble a, int n, long long *out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += gridDim.x * blockDim.x) {
        if (i == n) {
            out[i] = 0;
            continue;
        }
        const int *idx;
        const float *w[6];
        int self;
        out[i] = out_row(a, i, idx, w, self);
    }
}

__global__ void k_out_copy(Assemble a, int n, const long long *off, int *outSize, int *outOff,
                           int *outIdx, float *outW0, float *outW1, float *outW2, float *outW3,
                           float *outW4, float *outW5, int *maxIdx) {
    const int lane = threadIdx.x & 31;
    const int warps = blockDim.x >> 5;
    float *outW[6] = {outW0, outW1, outW2, outW3, outW4, outW5};
    int mx = -1;
    for (int i = blockIdx.x * warps + (threadIdx.x >> 5); i < n; i += gridDim.x * warps) {
        const int *idx = nullptr;
        const float *w[6];
        int self;
        const int sz = out_row(a, i, idx, w, self);
        const long long o = off[i];
        if (lane == 0) {
            outSize[i] = sz;
            outOff[i] = (int)o;
        }
        for (int e = lane; e < sz; e += 32) {
            const int q = self >= 0 ? self : idx[e];
            long long d = e;
            if (a.sort && self < 0) {
                int rank = 0;
                for (int j = 0; j < sz; ++j) {
                    const int qj = idx[j];
                    rank += (qj < q) || (qj == q && j < e);
                }
                d = rank;
            }
            outIdx[o + d] = q;
            for (int c = 0; c < a.nc; ++c)
                outW[c][o + d] = self >= 0 ? (c == 0 ? 1.0f : 0.0f) : (w[c] ? w[c][e] : 0.0f);
            mx = max(mx, q);
        }
    }
#pragma unroll
    for (int d = 16; d; d >>= 1) mx = max(mx, __shfl_xor_sync(kFull, mx, d));
    if (lane == 0 && mx >= 0) atomicMax(maxIdx, mx);
}

// ---- host side --------------------------------------------------------------------------

int grid_for(long long items, int perBlock) {
    const long long b = (items + perBlock - 1) / perBlock;
    return (int)std::max<long long>(1, std::min<long long>(b, (long long)num_sms() * 16));
}

// Stream-ordered device allocations released together (on success or failure).
struct Scratch {
    cudaStream_t s;
    std::vector<void *> ptrs;
    explicit Scratch(cudaStream_t st) : s(st) {}
    ~Scratch() {
        for (void *p : ptrs) scratch_free(p, s);
    }
    template <class T>
    T *alloc(size_t n, const char *who) {
        void *p = nullptr;
        if (scratch_alloc(&p, std::max<size_t>(n, 1) * sizeof(T), s, who) != GB300_OK)
            return nullptr;
        ptrs.push_back(p);
        return (T *)p;
    }
    void release(void *p) {
        auto it = std::find(ptrs.begin(), ptrs.end(), p);
        if (it != ptrs.end()) {
            scratch_free(p, s);
            ptrs.erase(it);
        }
    }
};

template <class T>
bool d2h(T *host, const T *dev, size_t n, cudaStream_t s, const char *who) {
    return check_cuda(cudaMemcpyAsync(host, dev, n * sizeof(T), cudaMemcpyDeviceToHost, s),
                      who) == GB300_OK &&
           check_cuda(cudaStreamSynchronize(s), who) == GB300_OK;
}

template <class T>
bool h2d(T *dev, const T *host, size_t n, cudaStream_t s, const char *who) {
    return n == 0 ||
           check_cuda(cudaMemcpyAsync(dev, host, n * sizeof(T), cudaMemcpyHostToDevice, s),
                      who) == GB300_OK;
}

// The growing entry arena (indices + NC weight channels).
template <int NC>
struct Arena {
    int *idx = nullptr;
    float *w[NC] = {};
    long long cap = 0, fill = 0;
};

template <int NC>
bool arena_reserve(Arena<NC> &a, long long need, Scratch &sc, const char *who) {
    if (need <= a.cap) return true;
    const long long cap = std::max<long long>(need, a.cap + a.cap / 2);
    int *ni = sc.alloc<int>((size_t)cap, who);
    if (!ni) return false;
    float *nw[NC];
    for (int c = 0; c < NC; ++c)
        if (!(nw[c] = sc.alloc<float>((size_t)cap, who))) return false;
    if (a.fill) {
        if (check_cuda(cudaMemcpyAsync(ni, a.idx, a.fill * 4, cudaMemcpyDeviceToDevice, sc.s),
                       who) != GB300_OK)
            return false;
        for (int c = 0; c < NC; ++c)
            if (check_cuda(cudaMemcpyAsync(nw[c], a.w[c], a.fill * 4, cudaMemcpyDeviceToDevice,
                                           sc.s),
                           who) != GB300_OK)
                return false;
    }
    if (a.idx) sc.release(a.idx);
    for (int c = 0; c < NC; ++c)
        if (a.w[c]) sc.release(a.w[c]);
    a.idx = ni;
    for (int c = 0; c < NC; ++c) a.w[c] = nw[c];
    a.cap = cap;
    return true;
}

// Builds the rows of one pass (one wave); p.metaSize / metaOff / arena are updated.  When the
// rows' term bounds fit in half the free device memory every row gets room for its bound and
// ONE merge pass writes it (rows then leave gaps in the arena; the table assembly compacts);
// otherwise a COUNT pass sizes the rows exactly before the FILL pass.  Returns false with the
// status recorded on failure.
template <int NC>
bool run_pass(Pass<NC> p, Arena<NC> &arena, long long *sizesTmp, long long *scanTmp,
              void *cubTmp, size_t cubBytes, int *dStatus, unsigned long long *dUsed,
              Scratch &sc, const char *who) {
    cudaStream_t s = sc.s;
    constexpr int W = warps_of<NC>();
    const int grid = grid_for(p.numRows, W);
    p.status = dStatus;
    p.scratchUsed = dUsed;
    p.scratch = nullptr;
    p.scratchCap = 0;
    if (p.rowsInArena) {
        p.rows.idx = arena.idx;
        p.rows.w = arena.w[0];
    }
    {
        const int g1 = grid_for(p.numRows + 1, 256);
        k_bounds<NC><<<g1, 256, 0, s>>>(p, sizesTmp);
        count_launch();
        size_t bytes = 0;
        cub::DeviceScan::ExclusiveSum(nullptr, bytes, sizesTmp, scanTmp, p.numRows + 1, s);
        if (bytes > cubBytes && !(cubTmp = sc.alloc<char>(bytes, who))) return false;
        if (check_cuda(cub::DeviceScan::ExclusiveSum(cubTmp, bytes, sizesTmp, scanTmp,
                                                     p.numRows + 1, s),
                       who) != GB300_OK)
            return false;
        count_launch();
        long long bound = 0;
        if (!d2h(&bound, scanTmp + p.numRows, 1, s, who)) return false;
        size_t freeB = 0, totalB = 0;
        if (check_cuda(cudaMemGetInfo(&freeB, &totalB), who) != GB300_OK) return false;
        // a growing arena is reallocated (old copy alive until the move is done)
        const long long need = arena.fill + bound;
        const long long newCap = need > arena.cap ? std::max(need, arena.cap + arena.cap / 2) : 0;
        if ((double)newCap * 4.0 * (1 + NC) < 0.5 * (double)freeB) {
            if (!arena_reserve(arena, arena.fill + bound, sc, who)) return false;
            k_wave_offsets<<<g1, 256, 0, s>>>(scanTmp, p.wave, p.waveId, p.numRows, arena.fill,
                                              const_cast<long long *>(p.metaOff), p.metaBase);
            count_launch();
            if (p.rowsInArena) {
                p.rows.idx = arena.idx;
                p.rows.w = arena.w[0];
            }
            p.arenaIdx = arena.idx;
            for (int c = 0; c < NC; ++c) p.arenaW[c] = arena.w[c];
            // the bounds are needed by the merge: keep them apart from the scan's inputs
            k_merge1<NC><<<grid, W * 32, 0, s>>>(p, sizesTmp);
            count_launch();
            if (check_launch(who) != GB300_OK) return false;
            arena.fill += bound;
            return true;
        }
    }
    // count (rerun once with a larger scratch pool when long rows need it)
    for (int attempt = 0; attempt < 2; ++attempt) {
        if (check_cuda(cudaMemsetAsync(dStatus, 0, 4, s), who) != GB300_OK ||
            check_cuda(cudaMemsetAsync(dUsed, 0, 8, s), who) != GB300_OK)
            return false;
        k_count<NC><<<grid, W * 32, 0, s>>>(p);
        count_launch();
        if (check_launch(who) != GB300_OK) return false;
        int st = 0;
        unsigned long long used = 0;
        if (!d2h(&st, dStatus, 1, s, who) || !d2h(&used, dUsed, 1, s, who)) return false;
        if (st & ~kNeedScratch) {
            fail(GB300_ERR_CUDA, "%s: inconsistent row sizes (status %d)", who, st);
            return false;
        }
        if (!(st & kNeedScratch)) break;
        if (attempt == 1) {
            fail(GB300_ERR_CUDA, "%s: scratch for long rows not sufficient", who);
            return false;
        }
        int *scr = sc.alloc<int>((size_t)used, who);
        if (!scr) return false;
        p.scratch = scr;
        p.scratchCap = (long long)used;
    }
    // offsets
    const int g1 = grid_for(p.numRows + 1, 256);
    k_wave_sizes<<<g1, 256, 0, s>>>(p.metaSize, p.metaBase, p.wave, p.waveId, p.numRows,
                                    sizesTmp);
    count_launch();
    size_t bytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, bytes, sizesTmp, scanTmp, p.numRows + 1, s);
    if (bytes > cubBytes && !(cubTmp = sc.alloc<char>(bytes, who))) return false;
    if (check_cuda(cub::DeviceScan::ExclusiveSum(cubTmp, bytes, sizesTmp, scanTmp,
                                                 p.numRows + 1, s),
                   who) != GB300_OK)
        return false;
    count_launch();
    long long total = 0;
    if (!d2h(&total, scanTmp + p.numRows, 1, s, who)) return false;
    if (!arena_reserve(arena, arena.fill + total, sc, who)) return false;
    k_wave_offsets<<<g1, 256, 0, s>>>(scanTmp, p.wave, p.waveId, p.numRows, arena.fill,
                                      const_cast<long long *>(p.metaOff), p.metaBase);
    count_launch();
    // fill (the arena may have moved: source rows in it move along)
    if (p.rowsInArena) {
        p.rows.idx = arena.idx;
        p.rows.w = arena.w[0];
    }
    p.arenaIdx = arena.idx;
    for (int c = 0; c < NC; ++c) p.arenaW[c] = arena.w[c];
    if (check_cuda(cudaMemsetAsync(dStatus, 0, 4, s), who) != GB300_OK) return false;
    k_fill<NC><<<grid, W * 32, 0, s>>>(p);
    count_launch();
    if (check_launch(who) != GB300_OK) return false;
    int st = 0;
    if (!d2h(&st, dStatus, 1, s, who)) return false;
    if (st) {
        fail(GB300_ERR_CUDA, "%s: row fill overflow (status %d)", who, st);
        return false;
    }
    arena.fill += total;
    return true;
}

// Copies the assembled rows into a new table object.
GB300StencilTable *assemble(Assemble a, int n, Scratch &sc, void *cubTmp, size_t cubBytes,
                            const char *who) {
    cudaStream_t s = sc.s;
    long long *sz = sc.alloc<long long>((size_t)n + 1, who);
    long long *off = sc.alloc<long long>((size_t)n + 1, who);
    int *dMax = sc.alloc<int>(1, who);
    if (!sz || !off || !dMax) return nullptr;
    const int g1 = grid_for(n + 1, 256);
    k_out_sizes<<<g1, 256, 0, s>>>(a, n, sz);
    count_launch();
    size_t need = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, need, sz, off, n + 1, s);
    void *tmp = cubTmp;
    if (need > cubBytes && !(tmp = sc.alloc<char>(need, who))) return nullptr;
    if (check_cuda(cub::DeviceScan::ExclusiveSum(tmp, need, sz, off, n + 1, s), who) !=
        GB300_OK)
        return nullptr;
    count_launch();
    long long nnz = 0;
    if (!d2h(&nnz, off + n, 1, s, who)) return nullptr;
    if (nnz > 0x7fffffffLL) {
        fail(GB300_ERR_UNSUPPORTED, "%s: %lld entries exceed the int offsets of a stencil table",
             who, nnz);
        return nullptr;
    }
    void *buf[9] = {nullptr};
    auto cleanup = [&]() {
        for (void *&b : buf)
            if (b) cudaFree(b), b = nullptr;
    };
    const size_t bytes[9] = {(size_t)n * 4, (size_t)n * 4, (size_t)nnz * 4};
    for (int k = 0; k < 3 + a.nc; ++k) {
        const size_t b = k < 3 ? bytes[k] : (size_t)nnz * 4;
        if (check_cuda(cudaMalloc(&buf[k], (std::max<size_t>(b, 4) + 15) & ~size_t(15)), who) !=
            GB300_OK) {
            cleanup();
            return nullptr;
        }
    }
    if (check_cuda(cudaMemsetAsync(dMax, 0xff, 4, s), who) != GB300_OK) {
        cleanup();
        return nullptr;
    }
    k_out_copy<<<grid_for(n, 8), 256, 0, s>>>(a, n, off, (int *)buf[0], (int *)buf[1],
                                              (int *)buf[2], (float *)buf[3], (float *)buf[4],
                                              (float *)buf[5], (float *)buf[6], (float *)buf[7],
                                              (float *)buf[8], dMax);
    count_launch();
    int mx = -1;
    if (check_launch(who) != GB300_OK || !d2h(&mx, dMax, 1, s, who)) {
        cleanup();
        return nullptr;
    }
    GB300StencilTable *t = adopt_stencil_table(n, nnz, mx + 1, buf, s, who);
    if (!t) cleanup();
    return t;
}

bool masks_ok(const GB300StencilMasks &m) {
    if (m.numRows < 0 || m.nnz < 0 || !m.offsets) return false;
    if (m.nnz > 0 && (!m.sources || !m.weights)) return false;
    if (m.offsets[0] != 0 || m.offsets[m.numRows] != m.nnz) return false;
    for (int r = 0; r < m.numRows; ++r)
        if (m.offsets[r + 1] < m.offsets[r]) return false;
    return true;
}

}  // namespace factory
}  // namespace gb300

using namespace gb300;
using namespace gb300::factory;

extern "C" {

GB300StencilTable *GB300StencilTableFactoryCreate(int numControl, int numLevels,
                                                  const GB300StencilMasks *levels,
                                                  int generateIntermediateLevels,
                                                  int generateControlVerts, int sortEntries,
                                                  void *stream) {
    const char *who = "GB300StencilTableFactoryCreate";
    if (numControl < 0 || numLevels < 0 || (numLevels > 0 && !levels)) {
        fail(GB300_ERR_INVALID_ARGUMENT, "%s: bad arguments", who);
        return nullptr;
    }
    long long total = 0, maxRows = 0, maskNnz = 0;
    for (int l = 0; l < numLevels; ++l) {
        if (!masks_ok(levels[l])) {
            fail(GB300_ERR_INVALID_ARGUMENT, "%s: malformed masks of level %d", who, l + 1);
            return nullptr;
        }
        total += levels[l].numRows;
        maxRows = std::max<long long>(maxRows, levels[l].numRows);
        maskNnz += levels[l].nnz;
    }
    if ((long long)numControl + total > 0x7fffffffLL) {
        fail(GB300_ERR_UNSUPPORTED, "%s: more than 2^31 vertices", who);
        return nullptr;
    }
    cudaStream_t s = as_stream(stream);
    Scratch sc(s);
    int *metaSize = sc.alloc<int>((size_t)total, who);
    long long *metaOff = sc.alloc<long long>((size_t)total, who);
    int *wave = sc.alloc<int>((size_t)maxRows, who);
    long long *sizesTmp = sc.alloc<long long>((size_t)maxRows + 1, who);
    long long *scanTmp = sc.alloc<long long>((size_t)maxRows + 1, who);
    int *dStatus = sc.alloc<int>(4, who);
    unsigned long long *dUsed = sc.alloc<unsigned long long>(1, who);
    if (!metaSize || !metaOff || !wave || !sizesTmp || !scanTmp || !dStatus || !dUsed)
        return nullptr;
    size_t cubBytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, cubBytes, sizesTmp, scanTmp, (int)maxRows + 1, s);
    void *cubTmp = sc.alloc<char>(cubBytes, who);
    if (!cubTmp) return nullptr;
    Arena<1> arena;
    if (!arena_reserve(arena, std::max<long long>(2 * maskNnz, 1 << 16), sc, who)) return nullptr;
    long long first = numControl, prevFirst = 0;
    int metaBase = 0;
    for (int l = 0; l < numLevels; ++l) {
        const GB300StencilMasks &m = levels[l];
        const int n = m.numRows;
        long long *moff = sc.alloc<long long>((size_t)n + 1, who);
        int *msrc = sc.alloc<int>((size_t)m.nnz, who);
        float *mw = sc.alloc<float>((size_t)m.nnz, who);
        if (!moff || !msrc || !mw) return nullptr;
        if (!h2d(moff, (const long long *)m.offsets, (size_t)n + 1, s, who) ||
            !h2d(msrc, m.sources, (size_t)m.nnz, s, who) ||
            !h2d(mw, m.weights, (size_t)m.nnz, s, who))
            return nullptr;
        // dependency waves
        if (check_cuda(cudaMemsetAsync(dStatus, 0, 16, s), who) != GB300_OK) return nullptr;
        const int g = grid_for(n, 256);
        if (n > 0) {
            k_wave_init<<<g, 256, 0, s>>>(moff, msrc, n, numControl, (int)prevFirst, (int)first,
                                          wave, dStatus + 1, dStatus);
            count_launch();
        }
        int hs[4] = {0, 0, 0, 0};
        if (check_launch(who) != GB300_OK || !d2h(hs, dStatus, 4, s, who)) return nullptr;
        if (hs[0]) {
            fail(GB300_ERR_INVALID_ARGUMENT,
                 "%s: level %d masks name a source outside the previous level and this one", who,
                 l + 1);
            return nullptr;
        }
        int pending = hs[1], waves = 1;
        while (pending > 0) {
            if (check_cuda(cudaMemsetAsync(dStatus + 2, 0, 4, s), who) != GB300_OK) return nullptr;
            k_wave_step<<<g, 256, 0, s>>>(moff, msrc, n, (int)first, waves, wave, dStatus + 2);
            count_launch();
            int got = 0;
            if (check_launch(who) != GB300_OK || !d2h(&got, dStatus + 2, 1, s, who))
                return nullptr;
            if (got == 0) {
                fail(GB300_ERR_INVALID_ARGUMENT, "%s: level %d rows depend on each other", who,
                     l + 1);
                return nullptr;
            }
            pending -= got;
            ++waves;
        }
        Pass<1> p{};
        p.rows = Rows{numControl, 1, metaSize, metaOff, nullptr, nullptr};
        p.moff = moff;
        p.msrc = msrc;
        p.mw[0] = mw;
        p.numRows = n;
        p.wave = waves > 1 ? wave : nullptr;
        p.metaBase = metaBase;
        p.metaSize = metaSize;
        p.metaOff = metaOff;
        p.skipZero = 0;
        p.rowsInArena = 1;
        for (int w = 0; w < waves && n > 0; ++w) {
            p.waveId = w;
            if (!run_pass(p, arena, sizesTmp, scanTmp, cubTmp, cubBytes, dStatus, dUsed, sc, who))
                return nullptr;
        }
        sc.release(moff);
        sc.release(msrc);
        sc.release(mw);
        prevFirst = first;
        first += n;
        metaBase += n;
    }

    Assemble a{};
    a.nIdentity = generateControlVerts ? numControl : 0;
    long long firstRow = 0;
    const int firstLevel = generateIntermediateLevels ? 0 : std::max(0, numLevels - 1);
    for (int l = 0; l < firstLevel; ++l) firstRow += levels[l].numRows;
    a.nMeta = numLevels ? (int)(total - firstRow) : 0;
    a.metaFirst = (int)firstRow;
    a.mSize = metaSize;
    a.mOff = metaOff;
    a.aIdx = arena.idx;
    a.aW[0] = arena.w[0];
    a.nc = 1;
    a.sort = sortEntries ? 1 : 0;
    GB300StencilTable *t = assemble(a, a.nIdentity + a.nMeta, sc, cubTmp, cubBytes, who);
    if (t && check_cuda(cudaStreamSynchronize(s), who) != GB300_OK) {
        GB300StencilTableDestroy(t);
        return nullptr;
    }
    if (t) ok();
    return t;
}

}  // extern "C"

namespace gb300 {

// The composition of GB300StencilTableComposeRows with its masks already in device memory
// (moff: numRows + 1 offsets, msrc / mw[c]: nnz sources and weights); scratch from `sc`.
GB300StencilTable *compose_rows_device(int baseNumStencils, int64_t baseNumIndices,
                                       const int *baseSizes, const int *baseOffsets,
                                       const int *baseIndices, const float *baseWeights,
                                       int numRows, int64_t nnz, const long long *moff,
                                       const int *msrc, float *const *mw, int numChannels,
                                       int appendBase, int sortEntries, Scratch &sc,
                                       const char *who) {
    cudaStream_t s = sc.s;
    long long *baseOff = sc.alloc<long long>((size_t)baseNumStencils, who);
    int *metaSize = sc.alloc<int>((size_t)numRows, who);
    long long *metaOff = sc.alloc<long long>((size_t)numRows, who);
    long long *sizesTmp = sc.alloc<long long>((size_t)numRows + 1, who);
    long long *scanTmp = sc.alloc<long long>((size_t)numRows + 1, who);
    int *dStatus = sc.alloc<int>(4, who);
    unsigned long long *dUsed = sc.alloc<unsigned long long>(1, who);
    if (!baseOff || !metaSize || !metaOff || !sizesTmp || !scanTmp || !dStatus || !dUsed)
        return nullptr;
    if (check_cuda(cudaMemsetAsync(dStatus, 0, 16, s), who) != GB300_OK) return nullptr;
    if (baseNumStencils > 0) {
        k_base_rows<<<grid_for(baseNumStencils, 256), 256, 0, s>>>(
            baseSizes, baseOffsets, baseNumStencils, baseNumIndices, baseOff, dStatus);
        count_launch();
    }
    if (nnz > 0) {
        k_check_sources<<<grid_for(nnz, 256), 256, 0, s>>>(msrc, nnz, baseNumStencils, dStatus);
        count_launch();
    }
    int st = 0;
    if (check_launch(who) != GB300_OK || !d2h(&st, dStatus, 1, s, who)) return nullptr;
    if (st) {
        fail(GB300_ERR_INVALID_ARGUMENT, "%s: %s", who,
             (st & kBadBase) ? "a base stencil lies outside the base arrays"
                             : "a mask names a stencil outside the base table");
        return nullptr;
    }
    size_t cubBytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, cubBytes, sizesTmp, scanTmp, numRows + 1, s);
    void *cubTmp = sc.alloc<char>(cubBytes, who);
    if (!cubTmp) return nullptr;
    GB300StencilTable *t = nullptr;
    auto run = [&](auto nc_tag) -> GB300StencilTable * {
        constexpr int NC = decltype(nc_tag)::value;
        Arena<NC> arena;
        if (!arena_reserve(arena, std::max<long long>(4 * nnz, 1 << 16), sc, who)) return nullptr;
        Pass<NC> p{};
        p.rows = Rows{0, 0, baseSizes, baseOff, baseIndices, baseWeights};
        p.moff = moff;
        p.msrc = msrc;
        for (int c = 0; c < NC; ++c) p.mw[c] = mw[c];
        p.numRows = numRows;
        p.wave = nullptr;
        p.metaBase = 0;
        p.metaSize = metaSize;
        p.metaOff = metaOff;
        p.skipZero = 1;
        p.rowsInArena = 0;
        if (numRows > 0 &&
            !run_pass(p, arena, sizesTmp, scanTmp, cubTmp, cubBytes, dStatus, dUsed, sc, who))
            return nullptr;
        Assemble a{};
        a.nBase = appendBase ? baseNumStencils : 0;
        a.bSize = baseSizes;
        a.bOff = baseOff;
        a.bIdx = baseIndices;
        a.bW = baseWeights;
        a.nMeta = numRows;
        a.metaFirst = 0;
        a.mSize = metaSize;
        a.mOff = metaOff;
        a.aIdx = arena.idx;
        for (int c = 0; c < NC; ++c) a.aW[c] = arena.w[c];
        a.nc = NC;
        a.sort = sortEntries ? 1 : 0;
        return assemble(a, a.nBase + numRows, sc, cubTmp, cubBytes, who);
    };
    if (numChannels == 1)
        t = run(std::integral_constant<int, 1>());
    else if (numChannels == 3)
        t = run(std::integral_constant<int, 3>());
    else
        t = run(std::integral_constant<int, 6>());
    if (t && check_cuda(cudaStreamSynchronize(s), who) != GB300_OK) {
        GB300StencilTableDestroy(t);
        return nullptr;
    }
    if (t) ok();
    return t;
}


// Masks of a limit stencil per point at its PatchCoord (5 words: array, patch, vertex, s,
// t), at a fixed stride of 20 entries: the patch's control points and the per-control-point
// basis weights of P (and Ds, Dt; and Dss, Dst, Dtt), padded with the first control point at
// weight 0 (which adds no entries and changes no sums).  A point the PatchMap missed gets an
// all-zero mask over base stencil 0.
template <int NK>
__global__ void __launch_bounds__(128) k_point_masks(int numPoints, const int *coords,
                                                      const int *arrays, const int *indices,
                                                      const int *params, long long *moff,
                                                      int *msrc, float *mw0, float *mw1,
                                                      float *mw2, float *mw3, float *mw4,
                                                      float *mw5, int *status) {
    const int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= numPoints; i += stride) {
        moff[i] = 20LL * i;
        if (i == numPoints) continue;
        const int *c = coords + 5 * (size_t)i;
        const int ai = c[0], pi = c[1];
        float w[NK][20];
        int n = 0, cv[20];
        if (ai >= 0) {
            const int *arr = arrays + 6 * ai;
            const Param p{params[3 * pi], params[3 * pi + 1]};
            const int type = p.regular() ? arr[0] : arr[1];
            n = patch_point_weights<NK>(type, p, __int_as_float(c[3]), __int_as_float(c[4]), w);
            if (n == 0) atomicOr(status, 1);
            const int *row = indices + arr[3] + (size_t)arr[4] * (pi - arr[5]);
#pragma unroll
            for (int j = 0; j < 20; ++j) cv[j] = j < n ? row[j] : 0;
        }
        float *mw[6] = {mw0, mw1, mw2, mw3, mw4, mw5};
        const size_t o = 20 * (size_t)i;
#pragma unroll
        for (int j = 0; j < 20; ++j) {
            msrc[o + j] = j < n ? cv[j] : (n ? cv[0] : 0);
#pragma unroll
            for (int k = 0; k < NK; ++k) mw[k][o + j] = j < n ? w[k][j] : 0.0f;
        }
    }
}

// Limit stencils at numPoints device PatchCoords of a device patch table, composed over the
// stencils of the table's points (base table, Far's layout, one row per point the patch
// indices name: control vertices first, then refined and local points).
GB300StencilTable *tess_stencils(const void *arrays, const int *indices, const void *params,
                                 int numPoints, const void *patchCoords, int baseNumStencils,
                                 int64_t baseNumIndices, const int *baseSizes,
                                 const int *baseOffsets, const int *baseIndices,
                                 const float *baseWeights, int numChannels, int sortEntries,
                                 cudaStream_t s, const char *who) {
    Scratch sc(s);
    const int64_t nnz = 20LL * numPoints;
    long long *moff = sc.alloc<long long>((size_t)numPoints + 1, who);
    int *msrc = sc.alloc<int>((size_t)nnz, who);
    int *status = sc.alloc<int>(1, who);
    if (!moff || !msrc || !status) return nullptr;
    float *mw[6] = {};
    for (int c = 0; c < numChannels; ++c)
        if (!(mw[c] = sc.alloc<float>((size_t)nnz, who))) return nullptr;
    if (check_cuda(cudaMemsetAsync(status, 0, sizeof(int), s), who) != GB300_OK) return nullptr;
    const int grid = grid_for((long long)numPoints + 1, 128);
    const int *co = (const int *)patchCoords, *ar = (const int *)arrays,
              *pa = (const int *)params;
    if (numChannels == 1)
        k_point_masks<1><<<grid, 128, 0, s>>>(numPoints, co, ar, indices, pa, moff, msrc,
                                              mw[0], mw[0], mw[0], mw[0], mw[0], mw[0], status);
    else if (numChannels == 3)
        k_point_masks<3><<<grid, 128, 0, s>>>(numPoints, co, ar, indices, pa, moff, msrc,
                                              mw[0], mw[1], mw[2], mw[0], mw[0], mw[0], status);
    else
        k_point_masks<6><<<grid, 128, 0, s>>>(numPoints, co, ar, indices, pa, moff, msrc,
                                              mw[0], mw[1], mw[2], mw[3], mw[4], mw[5], status);
    count_launch();
    if (check_launch(who) != GB300_OK) return nullptr;
    int st = 0;
    if (!d2h(&st, status, 1, s, who)) return nullptr;
    if (st) {
        fail(GB300_ERR_INVALID_ARGUMENT, "%s: a patch of a type without a basis", who);
        return nullptr;
    }
    return compose_rows_device(baseNumStencils, baseNumIndices, baseSizes, baseOffsets,
                               baseIndices, baseWeights, numPoints, nnz, moff, msrc, mw,
                               numChannels, 0, sortEntries, sc, who);
}

}  // namespace gb300

extern "C" {

GB300StencilTable *GB300StencilTableComposeRows(
    int baseNumStencils, int64_t baseNumIndices, const int *baseSizes, const int *baseOffsets,
    const int *baseIndices, const float *baseWeights, int numRows, int64_t nnz,
    const int64_t *offsets, const int *sources, int numChannels, const float *const *weights,
    int appendBase, int sortEntries, void *stream) {
    const char *who = "GB300StencilTableComposeRows";
    GB300StencilMasks m{numRows, nnz, offsets, sources, weights ? weights[0] : nullptr};
    bool good = baseNumStencils >= 0 && baseNumIndices >= 0 &&
                (baseNumStencils == 0 || (baseSizes && baseOffsets)) &&
                (baseNumIndices == 0 || (baseIndices && baseWeights)) &&
                (numChannels == 1 || numChannels == 3 || numChannels == 6) && weights &&
                masks_ok(m) && !(appendBase && numChannels != 1);
    for (int c = 0; good && c < numChannels; ++c) good = nnz == 0 || weights[c];
    if (!good) {
        fail(GB300_ERR_INVALID_ARGUMENT, "%s: bad arguments", who);
        return nullptr;
    }
    cudaStream_t s = as_stream(stream);
    Scratch sc(s);
    long long *moff = sc.alloc<long long>((size_t)numRows + 1, who);
    int *msrc = sc.alloc<int>((size_t)nnz, who);
    if (!moff || !msrc) return nullptr;
    float *mw[6] = {};
    for (int c = 0; c < numChannels; ++c)
        if (!(mw[c] = sc.alloc<float>((size_t)nnz, who))) return nullptr;
    if (!h2d(moff, (const long long *)offsets, (size_t)numRows + 1, s, who) ||
        !h2d(msrc, sources, (size_t)nnz, s, who))
        return nullptr;
    for (int c = 0; c < numChannels; ++c)
        if (!h2d(mw[c], weights[c], (size_t)nnz, s, who)) return nullptr;
    return compose_rows_device(baseNumStencils, baseNumIndices, baseSizes, baseOffsets,
                               baseIndices, baseWeights, numRows, nnz, moff, msrc, mw,
                               numChannels, appendBase, sortEntries, sc, who);
}

}  // extern "C"
