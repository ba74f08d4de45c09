// Batched EvalStencils: many meshes of uneven sizes in ONE persistent launch.
//
// A launch is a device job table (one job per mesh: its stencil table arrays, source and
// destination with the descriptor offset applied, primvar length and strides) plus the prefix
// of the jobs' tile counts.  CTAs of 1 producer warp + 8 consumer warps claim global tile
// numbers from a device work counter (dynamic scheduling absorbs the uneven tile costs); the
// producer maps the tile to its job by a warp-wide forward scan of the prefix (claims only
// grow, so each CTA's scan position only moves forward), stages the tile's sizes / offsets /
// indices / weights with bulk copies into a 3-stage shared-memory ring, and the consumers
// evaluate it with the staged EvalStencils kernel's own per-stencil code (tma::eval_one: one
// stencil per thread, vector row gathers where the layout allows), or one stencil per warp
// with a shuffle reduction for jobs whose stencils are large (high-valence poles).  Tile size,
// CTAs per SM and the large-stencil threshold come from the autotuner
// (GB300StencilBatchTune), which times candidates on the batch itself and caches the winner by
// the batch's histogram of work.  The counter reset is a memset on the launch stream, so the
// pair is graph-capturable (GB300StencilBatchEvalGraph).
#include "common.cuh"
#include "sell.h"
#include "stencil_eval.cuh"
#include "stencils_batch.h"
#include "tables.h"

#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <new>
#include <vector>

namespace gb300 {
namespace batch {

constexpr int kStages = 3;
constexpr int kConsumers = 256;
constexpr int kThreads = kConsumers + 32;
constexpr int kCap = 4096;        // entries per stage
constexpr int kMaxTile = 256;     // stencils per tile (upper bound)
constexpr int kMeta = kMaxTile + 8;
constexpr size_t kStageBytes = (size_t)kCap * 8 + (size_t)kMeta * 8;

// Ring depth and CTAs per SM of an instantiation: the sliced kernels run a 2-stage ring at
// three CTAs per SM (72 registers; their gathers are latency-bound, so resident warps matter
// more than a third stage; the 12-wide one gathers 2 rows per step to fit: 3 spilled and ran
// 5% slower); the Far-layout ones 3 stages, two CTAs per SM.
template <int CLS, bool SLICED>
struct Ring {
    static constexpr bool kThin = SLICED;
    static constexpr int kDepth = kThin ? 2 : kStages;
    static constexpr int kMinBlocks = kThin ? 3 : 2;
    static constexpr size_t kSmem = kDepth * kStageBytes + 256;
};
constexpr unsigned long long kWaitNs = 4000000000ull;

struct Meta {
    int job, s0, s1, s0a, e0a, e1, staged, done;
};

__device__ __forceinline__ uint32_t su32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void bar_init(uint64_t *b, int n) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(n));
}
__device__ __forceinline__ void bar_arrive(uint64_t *b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(b)) : "memory");
}
__device__ __forceinline__ void bar_arrive_tx(uint64_t *b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(b)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool bar_try(uint64_t *b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(su32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ unsigned long long gtime() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}
// Bounded wait; sets *status to GB300_ERR_DEVICE_TIMEOUT and returns false on expiry.
__device__ __forceinline__ bool bar_wait(uint64_t *b, uint32_t parity, int *status) {
    if (bar_try(b, parity)) return true;
    const unsigned long long t0 = gtime();
    while (!bar_try(b, parity)) {
        if (gtime() - t0 > kWaitNs) {
            atomicExch(status, GB300_ERR_DEVICE_TIMEOUT);
            return false;
        }
    }
    return true;
}
__device__ __forceinline__ void bulk(void *dst, const void *src, uint32_t bytes, uint64_t *bar,
                                     uint64_t pol) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint"
        " [%0], [%1], %2, [%3], %4;" ::"r"(su32(dst)),
        "l"(src), "r"(bytes), "r"(su32(bar)), "l"(pol)
        : "memory");
}

// One (large) stencil by one warp: lanes split the entries, then a butterfly reduction.
__device__ __forceinline__ void stencil_warp(const Job &j, int i, int n, int o, const int *lidx,
                                             const float *lw, int lane, uint64_t pol_src) {
    for (int c0 = 0; c0 < j.length; c0 += 8) {
        float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int k = lane; k < n; k += 32) {
            const int id = lidx ? lidx[o + k] : __ldg(j.indices + o + k);
            const float w = lidx ? lw[o + k] : __ldg(j.w[0] + o + k);
            float x[8];
            tma::gather_row<0>(j, id, c0, pol_src, x);
#pragma unroll
            for (int c = 0; c < 8; ++c) acc[c] = fmaf(w, x[c], acc[c]);
        }
#pragma unroll
        for (int c = 0; c < 8; ++c)
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], d);
        if (lane == 0) {
            float *d = j.dst[0] + (size_t)i * j.dstStride[0] + c0;
#pragma unroll
            for (int c = 0; c < 8; ++c)
                if (c0 + c < j.length) st_stream(d + c, acc[c]);
        }
    }
}

// eval_one's view of a staged job: the fields every gather uses are held in registers, the
// ones used once per stencil (outputs, weights for the unstaged path) stay in the shared-memory
// copy of the descriptor and are reached through references.
struct JobView {
    const float *src;
    int srcStride, length, vw;
    const float *const (&w)[1];
    float *const (&dst)[1];
    const int (&dstStride)[1];
    const int (&outOf)[1];
    const int (&vecDst)[1];
    const int *const &indices;
    __device__ explicit JobView(const Job &j)
        : src(j.src), srcStride(j.srcStride), length(j.length), vw(j.vw), w(j.w), dst(j.dst),
          dstStride(j.dstStride), outOf(j.outOf), vecDst(j.vecDst), indices(j.indices) {}
};

// Consumers' work on one staged tile of a job 9-12 floats wide over 16-byte aligned rows
// (stride >= 12): the single 12-wide pass (the wide instantiation of the kernel only).
__device__ __forceinline__ void tile_threads12(const Job &j, const Meta &m, const int *sidx,
                                               const float *sw, const int *ssz, const int *sof,
                                               uint64_t pol_src, uint64_t pol_stream) {
    const JobView v(j);
    for (int i = m.s0 + (int)threadIdx.x; i < m.s1; i += kConsumers) {
        const int n = ssz[i - m.s0a], o = sof[i - m.s0a];
        if (m.staged && o >= m.e0a && o + n <= m.e1)
            tma::eval_one12(v, i, n, sidx, sw, o - m.e0a);
        else
            tma::eval_one<1, 4>(v, i, n, nullptr, nullptr, 0, o, pol_src, pol_stream);
    }
}

// Job classes of a launch: any width (run-time row width, 8 columns per pass), 9-12 floats
// wide over 16-byte aligned rows (one 12-column pass), at most 4 floats over 16-byte aligned
// rows (one 4-column pass; sliced batches only).
constexpr int kAny = 0, kWide = 1, kNarrow = 2;

// One slice of a sliced job by one warp (lane = stencil): entry j of the 32 stencils at a time,
// index and weight from the stage (slot base `slot0`) or, for a slice wider than the stage,
// from global memory; columns per pass by job class.
template <int CLS>
__device__ __forceinline__ void slice_warp(const Job &j, const Meta &m, int wl, const int *sidx,
                                           const float *sw, const int *ssz, const int *srow,
                                           int lane, uint64_t pol_src, uint64_t pol_stream) {
    constexpr bool WIDE = CLS == kWide;
    constexpr int CW = WIDE ? 12 : CLS == kNarrow ? 4 : 8;  // columns per pass
    constexpr int R = WIDE ? 2 : CLS == kNarrow ? 6 : 4;    // rows per step (72 registers)
    const JobView v(j);
    const int slice = m.s0 + wl;
    const int n = ssz[wl * 32 + lane], row = srow[wl * 32 + lane];
    const int b0 = __ldg(j.slSlot + slice);
    const int width = (__ldg(j.slSlot + slice + 1) - b0) >> 5;
    const int base = b0 - m.e0a + lane;
    for (int c0 = 0; c0 < j.length; c0 += CW) {
        float acc[CW];
#pragma unroll
        for (int c = 0; c < CW; ++c) acc[c] = 0.0f;
        for (int j0 = 0; j0 < width; j0 += R) {
            int ids[R];
            float wk[R];
#pragma unroll
            for (int q = 0; q < R; ++q) {
                const int e = j0 + q;
                if (e < n) {
                    if (m.staged) {
                        ids[q] = sidx[base + e * 32];
                        wk[q] = sw[base + e * 32];
                    } else {
                        ids[q] = ld_stream(j.slIdx + b0 + lane + (size_t)e * 32, pol_stream);
                        wk[q] = ld_stream(j.slW + b0 + lane + (size_t)e * 32, pol_stream);
                    }
                }
            }
            float x[R][CW];
#pragma unroll
            for (int q = 0; q < R; ++q) {
                if (j0 + q >= n) continue;
                if constexpr (CLS == kNarrow) {
                    const float4 f = __ldg(
                        reinterpret_cast<const float4 *>(v.src + (size_t)ids[q] * v.srcStride));
                    x[q][0] = f.x;
                    x[q][1] = f.y;
                    x[q][2] = f.z;
                    x[q][3] = f.w;
                } else if constexpr (WIDE) {
                    const float4 *r =
                        reinterpret_cast<const float4 *>(v.src + (size_t)ids[q] * v.srcStride);
#pragma unroll
                    for (int u = 0; u < 3; ++u) {
                        const float4 f = __ldg(r + u);
                        x[q][4 * u] = f.x;
                        x[q][4 * u + 1] = f.y;
                        x[q][4 * u + 2] = f.z;
                        x[q][4 * u + 3] = f.w;
                    }
                } else {
                    tma::gather_row<0>(v, ids[q], c0, pol_src, x[q]);
                }
            }
#pragma unroll
            for (int q = 0; q < R; ++q)
                if (j0 + q < n)
#pragma unroll
                    for (int c = 0; c < CW; ++c) acc[c] = fmaf(wk[q], x[q][c], acc[c]);
        }
        if (row < 0) continue;
        float *d = j.dst[0] + (size_t)row * j.dstStride[0] + c0;
        const int rem = j.length - c0;
        if (CW == 8 && j.vecDst[0] == 8 && rem >= 8) {
            asm volatile("st.global.cs.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(d),
                         "f"(acc[0]), "f"(acc[1]), "f"(acc[2]), "f"(acc[3]), "f"(acc[4]),
                         "f"(acc[5]), "f"(acc[6]), "f"(acc[7])
                         : "memory");
            continue;
        }
#pragma unroll
        for (int u = 0; u < CW / 4; ++u) {
            if (j.vecDst[0] && 4 * u + 4 <= rem) {
                asm volatile("st.global.cs.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(d + 4 * u),
                             "f"(acc[4 * u]), "f"(acc[4 * u + 1]), "f"(acc[4 * u + 2]),
                             "f"(acc[4 * u + 3])
                             : "memory");
            } else {
#pragma unroll
                for (int c = 4 * u; c < 4 * u + 4; ++c)
                    if (c < rem) st_stream(d + c, acc[c]);
            }
        }
    }
}

// Consumers' work on one staged tile (VW = 0: the job's row width chosen per gather).
template <int VW>
__device__ __forceinline__ void tile_threads(const Job &j, const Meta &m, const int *sidx,
                                             const float *sw, const int *ssz, const int *sof,
                                             uint64_t pol_src, uint64_t pol_stream) {
    const JobView v(j);
    for (int i = m.s0 + (int)threadIdx.x; i < m.s1; i += kConsumers) {
        const int n = ssz[i - m.s0a], o = sof[i - m.s0a];
        if (m.staged && o >= m.e0a && o + n <= m.e1)
            tma::eval_one<1, VW>(v, i, n, sidx, sw, kCap, o - m.e0a, pol_src, pol_stream);
        else
            tma::eval_one<1, VW>(v, i, n, nullptr, nullptr, 0, o, pol_src, pol_stream);
    }
}

struct Args {
    const Job *jobs;
    const int *tileBase;  // numJobs + 1 entries
    int numJobs, numTiles;
    int *counter;         // work counter, zeroed before the launch
    int *status;
    int dynamic;          // 1: tiles claimed from the counter, 0: CTA b takes b, b + grid, ...
};

// CLS: the class of every job of the launch (kAny, kWide: single 12-wide pass, kNarrow: single
// 4-column pass, sliced launches only).  SLICED: every job of the launch reads its table's
// sliced layout (mode 2; a separate instantiation: both tile paths in one kernel spill
// registers).
template <int CLS, bool SLICED>
__global__ void __launch_bounds__(kThreads, (Ring<CLS, SLICED>::kMinBlocks))
    k_stencils_batch(const Args a) {
    constexpr int S = Ring<CLS, SLICED>::kDepth;
    extern __shared__ __align__(128) char smem[];
    __shared__ __align__(8) uint64_t full[S], empty[S];
    __shared__ Meta meta[S];
    __shared__ __align__(16) Job sjob[S];  // the staged tile's job, read by consumers
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            bar_init(&full[s], 32);
            bar_init(&empty[s], kConsumers / 32);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const uint64_t pol_stream = l2_evict_first(), pol_src = l2_evict_last();
    auto stage_ptr = [&](int s, int **idx, float **w, int **sz, int **of) {
        char *p = smem + (size_t)s * kStageBytes;
        *idx = (int *)p;
        *w = (float *)(p + (size_t)kCap * 4);
        *sz = (int *)(p + (size_t)kCap * 8);
        *of = *sz + kMeta;
    };

    if (warp == kConsumers / 32) {
        // producer: claim tiles until the list is exhausted, then post one "done" stage
        int jc = 0;  // job of the last claimed tile (claims only grow)
        for (int it = 0;; ++it) {
            const int stage = it % S;
            const uint32_t use = (uint32_t)(it / S);
            if (use > 0 && !bar_wait(&empty[stage], (use - 1) & 1, a.status)) return;
            int t = (int)blockIdx.x + it * (int)gridDim.x;
            if (a.dynamic) {
                if (lane == 0) t = atomicAdd(a.counter, 1);
                t = __shfl_sync(0xffffffffu, t, 0);
            }
            int *sidx, *ssz, *sof;
            float *sw;
            stage_ptr(stage, &sidx, &sw, &ssz, &sof);
            if (t >= a.numTiles) {
                if (lane == 0) meta[stage] = Meta{0, 0, 0, 0, 0, 0, 0, 1};
                __syncwarp();
                bar_arrive(&full[stage]);  // all 32 lanes: completes the phase without tx
                return;
            }
            // advance jc to the last job whose first tile is <= t (tileBase is non-decreasing,
            // so the lanes that pass form a prefix)
            for (;;) {
                const int q = jc + 1 + lane;
                const bool pass = q < a.numJobs && __ldg(a.tileBase + q) <= t;
                const int cnt = __popc(__ballot_sync(0xffffffffu, pass));
                jc += cnt;
                if (cnt < 32) break;
            }
            const Job &j = a.jobs[jc];
            static_assert(sizeof(Job) % 4 == 0 && sizeof(Job) / 4 <= 64, "Job copy");
            for (int q = lane; q < (int)(sizeof(Job) / 4); q += 32)
                reinterpret_cast<int *>(&sjob[stage])[q] =
                    __ldg(reinterpret_cast<const int *>(&j) + q);
            if constexpr (SLICED) {
                // sliced: the tile's positions (sizes, destination rows: 128 B per slice) and
                // its contiguous slot range (128-byte multiples) when it fits the stage
                const int s0 = (t - __ldg(a.tileBase + jc)) * kSliceTile;
                const int s1 = min(s0 + kSliceTile, j.numSlices);
                const int slot0 = __ldg(j.slSlot + s0), slot1 = __ldg(j.slSlot + s1);
                const bool staged = slot1 - slot0 <= kCap;
                const uint32_t pb = (uint32_t)(s1 - s0) * 128;
                const uint32_t eb = staged ? (uint32_t)(slot1 - slot0) * 4 : 0;
                if (lane == 0) {
                    meta[stage] = Meta{jc, s0, s1, 0, slot0, 0, staged ? 1 : 0, 0};
                    bar_arrive_tx(&full[stage], 2 * pb + 2 * eb);
                    bulk(ssz, j.slSz + (size_t)s0 * 32, pb, &full[stage], pol_stream);
                    bulk(sof, j.slRow + (size_t)s0 * 32, pb, &full[stage], pol_stream);
                    if (eb) {
                        bulk(sidx, j.slIdx + slot0, eb, &full[stage], pol_stream);
                        bulk(sw, j.slW + slot0, eb, &full[stage], pol_stream);
                    }
                }
                __syncwarp();
                if (lane != 0) bar_arrive(&full[stage]);
                continue;
            }
            const int s0 = (t - __ldg(a.tileBase + jc)) * j.tileStencils;
            const int s1 = min(s0 + j.tileStencils, j.numStencils);
            int e0 = 0, e1 = 0;
            if (lane == 0) {
                e0 = __ldg(j.offsets + s0);
                e1 = __ldg(j.offsets + s1 - 1) + __ldg(j.sizes + s1 - 1);
            }
            e0 = __shfl_sync(0xffffffffu, e0, 0);
            e1 = __shfl_sync(0xffffffffu, e1, 0);
            const int s0a = s0 & ~3, s1t = s1 & ~3, e0a = e0 & ~3, e1t = e1 & ~3;
            const bool staged = e1 >= e0 && (e1 - e0a) <= kCap;
            if (lane == 0) meta[stage] = Meta{jc, s0, s1, s0a, e0a, e1, staged ? 1 : 0, 0};
            uint32_t bytes = 0;
            if (s1t > s0a) bytes += (uint32_t)(s1t - s0a) * 8;
            if (staged && e1t > e0a) bytes += (uint32_t)(e1t - e0a) * 8;
            if (lane == 0) {
                bar_arrive_tx(&full[stage], bytes);
                if (s1t > s0a) {
                    bulk(ssz, j.sizes + s0a, (uint32_t)(s1t - s0a) * 4, &full[stage], pol_stream);
                    bulk(sof, j.offsets + s0a, (uint32_t)(s1t - s0a) * 4, &full[stage],
                         pol_stream);
                }
                if (staged && e1t > e0a) {
                    bulk(sidx, j.indices + e0a, (uint32_t)(e1t - e0a) * 4, &full[stage],
                         pol_stream);
                    bulk(sw, j.w[0] + e0a, (uint32_t)(e1t - e0a) * 4, &full[stage], pol_stream);
                }
            }
            // the last partial 16-byte chunks with plain loads (nothing past the arrays' ends)
            const int st0 = max(s1t, s0a);
            if (lane < s1 - st0) {
                ssz[st0 - s0a + lane] = __ldg(j.sizes + st0 + lane);
                sof[st0 - s0a + lane] = __ldg(j.offsets + st0 + lane);
            }
            if (staged) {
                const int et0 = max(e1t, e0a);
                if (lane < e1 - et0) {
                    sidx[et0 - e0a + lane] = __ldg(j.indices + et0 + lane);
                    sw[et0 - e0a + lane] = __ldg(j.w[0] + et0 + lane);
                }
            }
            __syncwarp();
            if (lane != 0) bar_arrive(&full[stage]);
        }
    }

    // consumers
    for (int it = 0;; ++it) {
        const int stage = it % S;
        const uint32_t use = (uint32_t)(it / S);
        if (!bar_wait(&full[stage], use & 1, a.status)) return;
        const Meta m = meta[stage];
        if (m.done) return;
        int *sidx, *ssz, *sof;
        float *sw;
        stage_ptr(stage, &sidx, &sw, &ssz, &sof);
        const Job &j = sjob[stage];
        if constexpr (SLICED) {
            if (m.s0 + warp < m.s1)
                slice_warp<CLS>(j, m, warp, sidx, sw, ssz, sof, lane, pol_src, pol_stream);
        } else if (j.mode == 0) {
            // one code path for every row width (inlined width-specific paths spill registers)
            if constexpr (CLS == kWide)
                tile_threads12(j, m, sidx, sw, ssz, sof, pol_src, pol_stream);
            else
                tile_threads<0>(j, m, sidx, sw, ssz, sof, pol_src, pol_stream);
        } else {
            for (int i = m.s0 + warp; i < m.s1; i += kConsumers / 32) {
                const int n = ssz[i - m.s0a], o = sof[i - m.s0a];
                if (m.staged && o >= m.e0a && o + n <= m.e1)
                    stencil_warp(j, i, n, o - m.e0a, sidx, sw, lane, pol_src);
                else
                    stencil_warp(j, i, n, o, nullptr, nullptr, lane, pol_src);
            }
        }
        __syncwarp();
        if (lane == 0) bar_arrive(&empty[stage]);
    }
}

// Row i of a pad job: 4, 8, 12 or 16 floats, 128-bit stores.
__device__ __forceinline__ void pad_row(const PadJob &j, long long i) {
    const float *row = j.src + i * j.srcStride;
    float *d = j.dst + i * j.dstStride;
    for (int c0 = 0; c0 < j.dstStride; c0 += 4) {
        float x[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) x[c] = c0 + c < j.length ? __ldg(row + c0 + c) : 0.0f;
        *reinterpret_cast<float4 *>(d + c0) = make_float4(x[0], x[1], x[2], x[3]);
    }
}

__global__ void __launch_bounds__(256) k_pad_rows(const PadJob *jobs, const long long *rowBase,
                                                  int count, long long totalRows) {
    const long long step = (long long)gridDim.x * blockDim.x;
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < totalRows;
         r += step) {
        int lo = 0, hi = count - 1;  // last job whose first row is <= r
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(rowBase + mid) <= r)
                lo = mid;
            else
                hi = mid - 1;
        }
        const PadJob j = jobs[lo];
        pad_row(j, r - __ldg(rowBase + lo));
    }
}

__global__ void __launch_bounds__(256) k_pad_one(const PadJob j) {
    const long long step = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < j.numRows;
         i += step)
        pad_row(j, i);
}

int launch_pad_one(const PadJob &j, cudaStream_t s) {
    if (j.numRows <= 0) return GB300_OK;
    const long long blocks = (j.numRows + 255) / 256;
    const int grid = (int)std::min<long long>(blocks, (long long)num_sms() * 16);
    k_pad_one<<<grid, 256, 0, s>>>(j);
    count_launch();
    return check_launch("padded source copy");
}

int launch_pad(const PadJob *dJobs, const long long *dRowBase, int count, long long totalRows,
               cudaStream_t s) {
    if (count <= 0 || totalRows <= 0) return GB300_OK;
    const long long blocks = (totalRows + 255) / 256;
    const int grid = (int)std::min<long long>(blocks, (long long)num_sms() * 16);
    k_pad_rows<<<grid, 256, 0, s>>>(dJobs, dRowBase, count, totalRows);
    count_launch();
    return check_launch("padded source copy");
}

bool make_job(const GB300StencilTable *t, const float *src, float *dst, int length,
              int srcStride, int dstStride, Job &j, double &meanSize, const char *who) {
    auto al = [](const void *p, uintptr_t m) { return ((uintptr_t)p & (m - 1)) == 0; };
    if (!t || !src || !dst || length <= 0 || srcStride < length || dstStride < length) {
        fail(GB300_ERR_INVALID_ARGUMENT, "%s: bad table, buffer, length or stride", who);
        return false;
    }
    j = Job{};
    j.src = src;
    j.dst[0] = dst;
    j.sizes = (const int *)GB300StencilTableGetBuffer(t, 0);
    j.offsets = (const int *)GB300StencilTableGetBuffer(t, 1);
    j.indices = (const int *)GB300StencilTableGetBuffer(t, 2);
    j.w[0] = (const float *)GB300StencilTableGetBuffer(t, 3);
    j.length = length;
    j.srcStride = srcStride;
    j.dstStride[0] = dstStride;
    j.vw = (al(src, 32) && srcStride % 8 == 0) ? 8 : (al(src, 16) && srcStride % 4 == 0) ? 4 : 1;
    j.vecDst[0] = (al(dst, 32) && dstStride % 8 == 0) ? 8
                  : (al(dst, 16) && dstStride % 4 == 0) ? 4 : 0;
    j.numStencils = GB300StencilTableGetNumStencils(t);
    const SellTable *sl = stencil_table_sell(t);
    if (sl && sl->numSlices > 0 && sl->w[0]) {
        j.slSz = sl->sz;
        j.slSlot = sl->sliceSlot;
        j.slIdx = sl->idx;
        j.slRow = sl->outRow;
        j.slW = sl->w[0];
        j.numSlices = sl->numSlices;
    }
    const int64_t nnz = GB300StencilTableGetNumIndices(t);
    meanSize = j.numStencils ? (double)nnz / j.numStencils : 0.0;
    return true;
}

int plan_tiles(Job *jobs, const double *meanSize, int n, int tileStencils, int warpThreshold,
               int *tileBase) {
    long long total = 0;
    for (int k = 0; k < n; ++k) {
        Job &j = jobs[k];
        tileBase[k] = (int)total;
        if (j.slSz) {
            j.mode = 2;
            j.tileStencils = kSliceTile * 32;
            total += (j.numSlices + kSliceTile - 1) / kSliceTile;
            continue;
        }
        j.mode = meanSize[k] > warpThreshold ? 1 : 0;
        j.tileStencils = j.mode == 1 ? 32 : tileStencils;
        total += (j.numStencils + j.tileStencils - 1) / j.tileStencils;
    }
    tileBase[n] = (int)total;
    return (int)total;
}

int set_smem_attribute() {
    static std::atomic<uint64_t> attr{0};  // devices whose function attribute is set
    return once_per_device(attr, [] {
        void (*const kernels[5])(Args) = {
            k_stencils_batch<kAny, false>, k_stencils_batch<kWide, false>,
            k_stencils_batch<kAny, true>, k_stencils_batch<kWide, true>,
            k_stencils_batch<kNarrow, true>};
        const size_t bytes[5] = {Ring<kAny, false>::kSmem, Ring<kWide, false>::kSmem,
                                 Ring<kAny, true>::kSmem, Ring<kWide, true>::kSmem,
                                 Ring<kNarrow, true>::kSmem};
        int st = GB300_OK;
        for (int k = 0; k < 5 && st == GB300_OK; ++k)
            st = check_cuda(cudaFuncSetAttribute(kernels[k],
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)bytes[k]),
                            "batch smem attribute");
        return st;
    });
}

int launch_jobs(const Job *dJobs, const int *dTileBase, int n, int numTiles, int *dCounter,
                int *dStatus, int ctasPerSm, cudaStream_t s, int dynamic, int cls,
                bool sliced) {
    int st = set_smem_attribute();
    if (st != GB300_OK) return st;
    if (numTiles == 0) return ok();
    if (cls == kNarrow && !sliced)
        return fail(GB300_ERR_INVALID_ARGUMENT, "batched EvalStencils: narrow class unsliced");
    if (dynamic) {
        st = check_cuda(cudaMemsetAsync(dCounter, 0, sizeof(int), s), "batch counter");
        if (st != GB300_OK) return st;
    }
    Args a{dJobs, dTileBase, n, numTiles, dCounter, dStatus, dynamic};
    // at most the CTAs per SM the instantiation can keep resident
    const int perSm = std::min(ctasPerSm, sliced ? Ring<kAny, true>::kMinBlocks
                                                 : Ring<kAny, false>::kMinBlocks);
    const int grid = std::min(numTiles, num_sms() * std::max(1, perSm));
    if (sliced) {
        if (cls == kWide)
            k_stencils_batch<kWide, true><<<grid, kThreads, Ring<kWide, true>::kSmem, s>>>(a);
        else if (cls == kNarrow)
            k_stencils_batch<kNarrow, true><<<grid, kThreads, Ring<kNarrow, true>::kSmem, s>>>(a);
        else
            k_stencils_batch<kAny, true><<<grid, kThreads, Ring<kAny, true>::kSmem, s>>>(a);
    } else {
        if (cls == kWide)
            k_stencils_batch<kWide, false><<<grid, kThreads, Ring<kWide, false>::kSmem, s>>>(a);
        else
            k_stencils_batch<kAny, false><<<grid, kThreads, Ring<kAny, false>::kSmem, s>>>(a);
    }
    count_launch();
    return check_launch("batched EvalStencils");
}

struct Config {
    int tileStencils = 256;  // stencils per tile
    int ctasPerSm = 2;       // persistent CTAs per SM
    int warpThreshold = 64;  // mean stencil size above which a job uses warp-per-stencil
    int dynamic = 1;         // tiles claimed from a work counter (else round-robin)
};

// Tuner key: the batch's work (stencil entries x primvar width) as a histogram over classes
// of (log2 mean stencil size, log2 stencils per job, primvar width / 4), each bin's share
// quantized to 1/16, hashed.  Batches with the same shape of work share a tuned config.
uint64_t work_signature(const std::vector<Job> &jobs, const std::vector<double> &mean) {
    std::map<int, double> bins;
    double total = 0.0;
    for (size_t k = 0; k < jobs.size(); ++k) {
        const int sc = (int)std::log2(mean[k] + 1.0);
        const int jc = (int)std::log2((double)jobs[k].numStencils + 1.0);
        const int key = (sc << 16) | (jc << 8) | ((jobs[k].length + 3) / 4);
        const double w = mean[k] * jobs[k].numStencils * jobs[k].length;
        bins[key] += w;
        total += w;
    }
    uint64_t sig = 1469598103934665603ull;
    for (auto &kv : bins) {
        const uint64_t q = total > 0 ? (uint64_t)std::lround(16.0 * kv.second / total) : 0;
        if (!q) continue;
        sig = (sig ^ (((uint64_t)kv.first << 8) | q)) * 1099511628211ull;
    }
    return sig;
}

}  // namespace batch
}  // namespace gb300

using namespace gb300;
using namespace gb300::batch;

struct GB300StencilBatch {
    // in launch order, one launch per part: the general jobs, the jobs at most 4 floats wide
    // over 16-byte aligned rows (sliced batches: the 4-column instantiation), the jobs 9-12
    // floats wide over 16-byte aligned rows (the 12-wide instantiation); each part largest
    // first
    std::vector<Job> jobs;
    std::vector<double> mean;  // mean stencil size per job (same order)
    int part[3] = {0, 0, 0};   // jobs per part
    bool sliced = false;       // every job reads its table's sliced layout (mode 2)
    Config cfg;
    Job *dJobs = nullptr;      // jobs, then the tile prefixes of the parts (part[p] + 1 ints
    int *dTileBase = nullptr;  // each)
    int *dCounter = nullptr;   // [1] status word; [0], [2], [3] work counters of the parts
    int partTiles[3] = {0, 0, 0};
    int numTiles() const { return partTiles[0] + partTiles[1] + partTiles[2]; }
    uint64_t signature = 0;
    cudaGraphExec_t graph = nullptr;  // pad copy + counter reset + kernel, on first use
    cudaStream_t capture = nullptr;
    // padded copies of unaligned sources (rows of 8 floats), refreshed by every evaluation
    float *dPadded = nullptr;
    PadJob *dPad = nullptr;
    long long *dPadBase = nullptr;
    int numPad = 0;
    long long padRows = 0;
    void drop_graph() {
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
    }
    ~GB300StencilBatch() {
        drop_graph();
        if (capture) cudaStreamDestroy(capture);
        if (dJobs) cudaFree(dJobs);
        if (dCounter) cudaFree(dCounter);
        if (dPadded) cudaFree(dPadded);
        if (dPad) cudaFree(dPad);
    }
};

namespace {

std::mutex g_tuneLock;
std::map<uint64_t, Config> g_tuned;  // work signature -> best config

constexpr int kPartClass[3] = {kAny, kNarrow, kWide};
constexpr int kPartCounter[3] = {0, 3, 2};

// Applies b->cfg: job modes, tile sizes and the tile prefixes, uploaded to the device.
int upload_plan(GB300StencilBatch *b, cudaStream_t s) {
    const int n = (int)b->jobs.size();
    std::vector<int> base(n + 3);
    for (int p = 0, j0 = 0; p < 3; j0 += b->part[p], ++p)
        b->partTiles[p] = plan_tiles(b->jobs.data() + j0, b->mean.data() + j0, b->part[p],
                                     b->cfg.tileStencils, b->cfg.warpThreshold,
                                     base.data() + j0 + p);
    int st = check_cuda(cudaMemcpyAsync(b->dJobs, b->jobs.data(), n * sizeof(Job),
                                        cudaMemcpyHostToDevice, s), "batch jobs");
    if (st != GB300_OK) return st;
    st = check_cuda(cudaMemcpyAsync(b->dTileBase, base.data(), (n + 3) * sizeof(int),
                                    cudaMemcpyHostToDevice, s), "batch jobs");
    if (st != GB300_OK) return st;
    return check_cuda(cudaStreamSynchronize(s), "batch jobs");
}

int launch_batch(GB300StencilBatch *b, cudaStream_t s) {
    int st = launch_pad(b->dPad, b->dPadBase, b->numPad, b->padRows, s);
    if (st != GB300_OK) return st;
    for (int p = 0, j0 = 0; p < 3; j0 += b->part[p], ++p) {
        st = launch_jobs(b->dJobs + j0, b->dTileBase + j0 + p, b->part[p], b->partTiles[p],
                         b->dCounter + kPartCounter[p], b->dCounter + 1, b->cfg.ctasPerSm, s,
                         b->cfg.dynamic, kPartClass[p], b->sliced);
        if (st != GB300_OK) return st;
    }
    return GB300_OK;
}

// Jobs whose source rows are unaligned (scalar gathers) and at most 8 floats wide read a
// padded copy instead: one device buffer for all of them, rows of 8 floats.
int setup_padding(GB300StencilBatch *b, const std::vector<int> &tableRows, cudaStream_t s) {
    std::vector<PadJob> pads;
    std::vector<long long> base(1, 0);
    std::vector<int> which;
    for (size_t k = 0; k < b->jobs.size(); ++k) {
        const Job &j = b->jobs[k];
        // unaligned rows (scalar gathers), up to 16 floats wide
        if (j.vw != 1 || padded_stride(j.length) == 0 || tableRows[k] <= 0 ||
            j.numStencils == 0)
            continue;
        pads.push_back(PadJob{j.src, nullptr, j.srcStride, j.length, tableRows[k],
                              padded_stride(j.length), 0});
        which.push_back((int)k);
    }
    if (pads.empty()) return GB300_OK;
    // every job's region starts on a 64-byte boundary: rows of 8 / 16 floats are then 32-byte
    // aligned (256-bit gathers) and rows of 4 / 12 floats 16-byte aligned (128-bit gathers)
    long long floats = 0;
    std::vector<long long> at;
    for (const PadJob &p : pads) {
        floats = (floats + 15) & ~15LL;
        at.push_back(floats);
        floats += p.numRows * p.dstStride;
        base.push_back(base.back() + p.numRows);
    }
    const long long rows = base.back();
    int st = check_cuda(cudaMalloc((void **)&b->dPadded, (size_t)floats * 4), "batch padding");
    if (st != GB300_OK) {
        b->dPadded = nullptr;
        return st;
    }
    for (size_t p = 0; p < pads.size(); ++p) {
        pads[p].dst = b->dPadded + at[p];
        Job &j = b->jobs[which[p]];
        j.src = pads[p].dst;
        j.srcStride = pads[p].dstStride;
        j.vw = (pads[p].dstStride == 4 || pads[p].dstStride == 12) ? 4 : 8;
    }
    const size_t padBytes = ((pads.size() * sizeof(PadJob) + 255) / 256) * 256;
    st = check_cuda(cudaMalloc((void **)&b->dPad, padBytes + base.size() * sizeof(long long)),
                    "batch padding");
    if (st != GB300_OK) {
        b->dPad = nullptr;
        return st;
    }
    b->dPadBase = (long long *)((char *)b->dPad + padBytes);
    b->numPad = (int)pads.size();
    b->padRows = rows;
    st = check_cuda(cudaMemcpyAsync(b->dPad, pads.data(), pads.size() * sizeof(PadJob),
                                    cudaMemcpyHostToDevice, s), "batch padding");
    if (st == GB300_OK)
        st = check_cuda(cudaMemcpyAsync(b->dPadBase, base.data(), base.size() * sizeof(long long),
                                        cudaMemcpyHostToDevice, s), "batch padding");
    if (st == GB300_OK) st = check_cuda(cudaStreamSynchronize(s), "batch padding");
    return st;
}

}  // namespace


// ---- batched EvalStencils without allocation ------------------------------------------------
//
// The same kernel with all of its scratch -- work counter, job table and tile prefix -- in one
// fixed file-scope device array, so a call allocates no memory: the job table is built on the
// host stack and copied into the array, the counter is cleared by a memset, and the kernel runs
// every job one stencil per thread (jobs' mean stencil sizes are not known without reading the
// device tables).  An expired bounded wait is recorded in the library's status word (the one
// GB300GetDeviceStatus reads), which is only cleared by reading it.  One array per device means
// calls that overlap on the device (two streams, two host threads) race on it.
namespace {

constexpr int kNoAllocMaxJobs = 256;
constexpr size_t kNoAllocJobOffset = 256;  // [0] work counter
constexpr size_t kNoAllocBaseOffset =
    kNoAllocJobOffset + ((kNoAllocMaxJobs * sizeof(Job) + 255) / 256) * 256;
constexpr size_t kNoAllocScratchBytes =
    kNoAllocBaseOffset + (((kNoAllocMaxJobs + 1) * sizeof(int) + 255) / 256) * 256;
// the figure the header documents: 256 + 256 job descriptors of 136 bytes + 1,280
static_assert(sizeof(Job) == 136 && kNoAllocScratchBytes == 36352,
              "update the scratch size documented for GB300EvalStencilsBatchedNoAlloc");
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noallocLock;
unsigned char *g_noallocAddr[kNoAllocMaxDevices];  // scratch address per device
int *g_noallocStatus[kNoAllocMaxDevices];          // the library's status word per device
int g_noallocSms[kNoAllocMaxDevices];

}  // namespace

extern "C" {

GB300StencilBatch *GB300StencilBatchCreate(int numJobs, GB300StencilTable *const *tables,
                                           const float *const *src, float *const *dst,
                                           const int *length, const int *srcStride,
                                           const int *dstStride, void *stream) {
    if (numJobs <= 0 || !tables || !src || !dst || !length || !srcStride || !dstStride) {
        fail(GB300_ERR_INVALID_ARGUMENT, "GB300StencilBatchCreate: bad arguments");
        return nullptr;
    }
    GB300StencilBatch *b = new (std::nothrow) GB300StencilBatch;
    if (!b) {
        fail(GB300_ERR_OUT_OF_MEMORY, "GB300StencilBatchCreate: host allocation");
        return nullptr;
    }
    cudaStream_t s = as_stream(stream);
    std::vector<Job> jobs(numJobs);
    std::vector<double> mean(numJobs);
    for (int i = 0; i < numJobs; ++i) {
        if (!make_job(tables[i], src[i], dst[i], length[i], srcStride[i], dstStride[i], jobs[i],
                      mean[i], "GB300StencilBatchCreate")) {
            delete b;
            return nullptr;
        }
    }
    // launch order: largest jobs first, so the small ones fill the tail of the launch
    std::vector<int> order(numJobs);
    for (int i = 0; i < numJobs; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        return mean[x] * jobs[x].numStencils * jobs[x].length >
               mean[y] * jobs[y].numStencils * jobs[y].length;
    });
    std::vector<int> rows;
    for (int i : order) {
        b->jobs.push_back(jobs[i]);
        b->mean.push_back(mean[i]);
        rows.push_back(stencil_table_num_control(tables[i]));
    }
    // one tile path per launch: the sliced one when every table has its sliced layout
    b->sliced = true;
    for (const Job &j : b->jobs) b->sliced = b->sliced && j.slSz;
    if (!b->sliced)
        for (Job &j : b->jobs) j.slSz = nullptr;
    if (setup_padding(b, rows, s) != GB300_OK) {
        delete b;
        return nullptr;
    }
    // parts: jobs one output 9-12 floats wide over 16-byte aligned rows (stride >= 12) go to
    // the 12-wide launch, jobs at most 4 floats wide over 16-byte aligned rows of a sliced
    // batch to the 4-column launch, the rest to the general one (order within each part kept:
    // largest first)
    {
        const bool sliced = b->sliced;
        auto part_of = [sliced](const Job &j) {
            if (j.vw >= 4 && j.length > 8 && j.length <= 12) return 2;
            if (sliced && j.vw >= 4 && j.length <= 4) return 1;
            return 0;
        };
        std::vector<Job> pj[3];
        std::vector<double> pm[3];
        for (size_t k = 0; k < b->jobs.size(); ++k) {
            const int p = part_of(b->jobs[k]);
            pj[p].push_back(b->jobs[k]);
            pm[p].push_back(b->mean[k]);
        }
        b->jobs.clear();
        b->mean.clear();
        for (int p = 0; p < 3; ++p) {
            b->part[p] = (int)pj[p].size();
            b->jobs.insert(b->jobs.end(), pj[p].begin(), pj[p].end());
            b->mean.insert(b->mean.end(), pm[p].begin(), pm[p].end());
        }
    }
    // every job's vector width must match its rows' alignment (the gathers assume it)
    for (const Job &j : b->jobs) {
        const uintptr_t a = (uintptr_t)j.src;
        if ((j.vw == 8 && ((a & 31) || j.srcStride % 8)) ||
            (j.vw == 4 && ((a & 15) || j.srcStride % 4))) {
            fail(GB300_ERR_CUDA, "GB300StencilBatchCreate: internal error: job rows not "
                                 "aligned for %d-wide gathers", j.vw);
            delete b;
            return nullptr;
        }
    }
    b->signature = work_signature(b->jobs, b->mean);
    {
        std::lock_guard<std::mutex> lock(g_tuneLock);
        auto it = g_tuned.find(b->signature);
        if (it != g_tuned.end()) b->cfg = it->second;
    }
    const size_t jobBytes = ((numJobs * sizeof(Job) + 255) / 256) * 256;
    if (check_cuda(cudaMalloc((void **)&b->dJobs, jobBytes + (numJobs + 3) * sizeof(int)),
                   "batch jobs") != GB300_OK) {
        b->dJobs = nullptr;
        delete b;
        return nullptr;
    }
    b->dTileBase = (int *)((char *)b->dJobs + jobBytes);
    if (check_cuda(cudaMalloc((void **)&b->dCounter, 4 * sizeof(int)), "batch counter") !=
            GB300_OK ||
        check_cuda(cudaMemsetAsync(b->dCounter, 0, 4 * sizeof(int), s), "batch counter") !=
            GB300_OK ||
        upload_plan(b, s) != GB300_OK) {
        delete b;
        return nullptr;
    }
    ok();
    return b;
}

void GB300StencilBatchDestroy(GB300StencilBatch *b) { delete b; }

int GB300StencilBatchEval(GB300StencilBatch *b, void *stream) {
    if (!b) return fail(GB300_ERR_INVALID_ARGUMENT, "GB300StencilBatchEval: null batch");
    return launch_batch(b, as_stream(stream));
}

int GB300StencilBatchEvalGraph(GB300StencilBatch *b, void *stream) {
    if (!b) return fail(GB300_ERR_INVALID_ARGUMENT, "GB300StencilBatchEvalGraph: null batch");
    cudaStream_t s = as_stream(stream);
    if (!b->graph) {
        int st = set_smem_attribute();
        if (st != GB300_OK) return st;
        if (!b->capture &&
            (st = check_cuda(cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking),
                             "batch capture stream")) != GB300_OK)
            return st;
        cudaGraph_t g = nullptr;
        st = check_cuda(cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal),
                        "batch graph capture");
        if (st != GB300_OK) return st;
        const uint64_t before = g_launches.load();
        const int lst = launch_batch(b, b->capture);
        const cudaError_t ce = cudaStreamEndCapture(b->capture, &g);
        g_launches.store(before);  // captured, not launched
        if (lst != GB300_OK) {
            if (g) cudaGraphDestroy(g);
            return lst;
        }
        if ((st = check_cuda(ce, "batch graph capture")) != GB300_OK) return st;
        st = check_cuda(cudaGraphInstantiate(&b->graph, g, 0), "batch graph instantiate");
        cudaGraphDestroy(g);
        if (st != GB300_OK) {
            b->graph = nullptr;
            return st;
        }
    }
    int st = check_cuda(cudaGraphLaunch(b->graph, s), "GB300StencilBatchEvalGraph");
    if (st != GB300_OK) return st;
    for (int p = 0; p < 3; ++p)
        if (b->partTiles[p]) count_launch();
    return ok();
}

int GB300StencilBatchGetDeviceStatus(GB300StencilBatch *b, int *status) {
    if (!b || !status)
        return fail(GB300_ERR_INVALID_ARGUMENT, "GB300StencilBatchGetDeviceStatus: null argument");
    int st = check_cuda(cudaMemcpy(status, b->dCounter + 1, sizeof(int), cudaMemcpyDeviceToHost),
                        "batch status");
    if (st != GB300_OK) return st;
    if (*status) st = check_cuda(cudaMemset(b->dCounter + 1, 0, sizeof(int)), "batch status");
    return st != GB300_OK ? st : ok();
}

int GB300StencilBatchGetConfig(const GB300StencilBatch *b, int *tileStencils, int *ctasPerSm,
                               int *warpThreshold, int *numTiles, int *dynamicClaims) {
    if (!b) return fail(GB300_ERR_INVALID_ARGUMENT, "GB300StencilBatchGetConfig: null batch");
    if (tileStencils) *tileStencils = b->cfg.tileStencils;
    if (ctasPerSm) *ctasPerSm = b->cfg.ctasPerSm;
    if (warpThreshold) *warpThreshold = b->cfg.warpThreshold;
    if (numTiles) *numTiles = b->numTiles();
    if (dynamicClaims) *dynamicClaims = b->cfg.dynamic;
    return ok();
}

int GB300StencilBatchTune(GB300StencilBatch *b, int iterations, void *stream) {
    if (!b) return fail(GB300_ERR_INVALID_ARGUMENT, "GB300StencilBatchTune: null batch");
    cudaStream_t s = as_stream(stream);
    if (iterations < 1) iterations = 3;
    b->drop_graph();
    const int tiles[] = {64, 128, 256};
    const int ctas[] = {1, 2, 3};
    const int thresholds[] = {32, 96, 1 << 30};
    // a threshold only matters when some job's mean stencil size lies between candidates
    bool anyLarge = false;
    for (double m : b->mean) anyLarge |= m > 32;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    Config best = b->cfg;
    float bestMs = 1e30f;
    int st = GB300_OK;
    for (int ts : tiles)
        for (int c : ctas)
            for (int th : thresholds)
            for (int dyn = 0; dyn < 2; ++dyn) {
                if (!anyLarge && th != thresholds[0]) continue;
                // sliced jobs have fixed tiles and no warp-per-stencil mode
                if (b->sliced && (ts != tiles[0] || th != thresholds[0])) continue;
                b->cfg = Config{ts, c, th, dyn};
                if ((st = upload_plan(b, s)) != GB300_OK) goto done;
                if ((st = launch_batch(b, s)) != GB300_OK) goto done;  // warm-up
                cudaEventRecord(e0, s);
                for (int k = 0; k < iterations; ++k)
                    if ((st = launch_batch(b, s)) != GB300_OK) goto done;
                cudaEventRecord(e1, s);
                cudaEventSynchronize(e1);
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (ms < bestMs) {
                    bestMs = ms;
                    best = b->cfg;
                }
            }
done:
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->cfg = best;
    const int rb = upload_plan(b, s);
    if (st != GB300_OK) return st;
    if (rb != GB300_OK) return rb;
    {
        std::lock_guard<std::mutex> lock(g_tuneLock);
        g_tuned[b->signature] = best;
    }
    return ok();
}


int GB300EvalStencilsBatchedNoAlloc(int numJobs, const float *const *src, float *const *dst,
                                    const int *length, const int *srcStride,
                                    const int *dstStride, const int *numStencils,
                                    const int *const *sizes, const int *const *offsets,
                                    const int *const *indices, const float *const *weights,
                                    void *stream) {
    static const char *who = "GB300EvalStencilsBatchedNoAlloc";
    if (numJobs < 1 || numJobs > kNoAllocMaxJobs)
        return fail(GB300_ERR_INVALID_ARGUMENT,
                    "%s: %d jobs; between 1 and %d jobs fit its fixed %zu-byte device scratch",
                    who, numJobs, kNoAllocMaxJobs, kNoAllocScratchBytes);
    if (!src || !dst || !length || !srcStride || !dstStride || !numStencils || !sizes ||
        !offsets || !indices || !weights)
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: null argument array", who);
    // job table and tile prefix on the host stack (no heap allocation)
    Job jobs[kNoAllocMaxJobs];
    int base[kNoAllocMaxJobs + 1];
    auto al = [](const void *p, uintptr_t m) { return ((uintptr_t)p & (m - 1)) == 0; };
    long long tiles = 0;
    for (int k = 0; k < numJobs; ++k) {
        const int n = numStencils[k];
        if (n < 0 || length[k] <= 0 || srcStride[k] < length[k] || dstStride[k] < length[k] ||
            (n > 0 && (!src[k] || !dst[k] || !sizes[k] || !offsets[k] || !indices[k] ||
                       !weights[k])))
            return fail(GB300_ERR_INVALID_ARGUMENT,
                        "%s: job %d has a bad count, length, stride or null pointer", who, k);
        if (n > 0 && (!al(sizes[k], 16) || !al(offsets[k], 16) || !al(indices[k], 16) ||
                      !al(weights[k], 16)))
            return fail(GB300_ERR_INVALID_ARGUMENT,
                        "%s: job %d table arrays must be 16-byte aligned (bulk copies)", who, k);
        Job &j = jobs[k];
        j = Job{};
        j.src = src[k];
        j.dst[0] = dst[k];
        j.w[0] = weights[k];
        j.sizes = sizes[k];
        j.offsets = offsets[k];
        j.indices = indices[k];
        j.length = length[k];
        j.srcStride = srcStride[k];
        j.dstStride[0] = dstStride[k];
        j.vw = (al(src[k], 32) && srcStride[k] % 8 == 0)   ? 8
               : (al(src[k], 16) && srcStride[k] % 4 == 0) ? 4 : 1;
        j.vecDst[0] = (al(dst[k], 32) && dstStride[k] % 8 == 0)   ? 8
                      : (al(dst[k], 16) && dstStride[k] % 4 == 0) ? 4 : 0;
        j.numStencils = n;
        j.mode = 0;
        j.tileStencils = kMaxTile;
        base[k] = (int)tiles;
        tiles += (n + kMaxTile - 1) / kMaxTile;
        if (tiles > INT32_MAX)
            return fail(GB300_ERR_INVALID_ARGUMENT, "%s: more than 2^31 tiles", who);
    }
    base[numJobs] = (int)tiles;
    // scratch address and SM count, once per device (with that device current)
    int dev = 0;
    int st = check_cuda(cudaGetDevice(&dev), who);
    if (st != GB300_OK) return st;
    if (dev < 0 || dev >= kNoAllocMaxDevices)
        return fail(GB300_ERR_UNSUPPORTED, "%s: device %d beyond the first %d", who, dev,
                    kNoAllocMaxDevices);
    unsigned char *scratch = nullptr;
    int *status = nullptr;
    int sms = 0;
    {
        std::lock_guard<std::mutex> lock(g_noallocLock);
        if (!g_noallocAddr[dev]) {
            void *p = nullptr;
            st = check_cuda(cudaGetSymbolAddress(&p, g_noalloc_scratch), who);
            if (st != GB300_OK) return st;
            int *sw = nullptr;
            if ((st = status_word_address(&sw)) != GB300_OK) return st;
            int n = 0;
            st = check_cuda(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev), who);
            if (st != GB300_OK) return st;
            g_noallocSms[dev] = n > 0 ? n : 1;
            g_noallocStatus[dev] = sw;
            g_noallocAddr[dev] = (unsigned char *)p;
        }
        scratch = g_noallocAddr[dev];
        status = g_noallocStatus[dev];
        sms = g_noallocSms[dev];
    }
    if ((st = set_smem_attribute()) != GB300_OK) return st;
    if (tiles == 0) return ok();
    cudaStream_t s = as_stream(stream);
    int *counter = (int *)scratch;
    Job *dJobs = (Job *)(scratch + kNoAllocJobOffset);
    int *dBase = (int *)(scratch + kNoAllocBaseOffset);
    // pageable host -> device: the stack buffers are consumed before the calls return
    if ((st = check_cuda(cudaMemcpyAsync(dJobs, jobs, numJobs * sizeof(Job),
                                         cudaMemcpyHostToDevice, s), who)) != GB300_OK ||
        (st = check_cuda(cudaMemcpyAsync(dBase, base, (numJobs + 1) * sizeof(int),
                                         cudaMemcpyHostToDevice, s), who)) != GB300_OK ||
        (st = check_cuda(cudaMemsetAsync(counter, 0, sizeof(int), s), who)) != GB300_OK)
        return st;
    Args a{dJobs, dBase, numJobs, (int)tiles, counter, status, 1};
    const int grid = (int)std::min<long long>(tiles, 2LL * sms);
    k_stencils_batch<kAny, false><<<grid, kThreads, Ring<kAny, false>::kSmem, s>>>(a);
    count_launch();
    return check_launch(who);
}

}  // extern "C"
