// EvalStencils, staged kernel for sm_103a.
//
// A persistent CTA = 1 producer warp + 8 consumer warps.  The stencil range is cut into tiles
// of TS consecutive stencils.  For each tile the producer streams the tile's slice of every
// table array -- sizes, offsets, control indices and the 1, 3 or 6 weight arrays -- from HBM
// into one stage of a 3-deep shared-memory ring with bulk asynchronous copies
// (cp.async.bulk ... mbarrier::complete_tx), so the table stream runs at full memory-level
// parallelism independently of the consumers' dependent gathers.  Consumers take one stencil
// per thread, read its entries from shared memory, gather the source rows (float4 when the
// layout allows) from L1/L2 and accumulate every requested output in registers; outputs are
// written with streaming stores.
//
// Bulk copies need 16-byte aligned addresses and sizes: the copied window is the tile's range
// rounded down to 4 entries at the start and the last partial 16-byte chunk is loaded with
// plain loads by the producer lanes, so nothing outside [0, nnz) / [0, numStencils) is read.
// A tile whose entries do not fit the stage (or whose offsets are not monotone) is processed
// straight from global memory.  Every mbarrier wait is bounded by a %globaltimer deadline; on
// expiry the CTA records GB300_ERR_DEVICE_TIMEOUT in g_status and leaves.
//
// Table objects evaluate through their sliced layout (sell.h) with k_stencils_sell: the same
// producer / ring / consumer-group scheme, tiles of whole 32-stencil slices, one consumer warp
// per slice stepping through entry j of its 32 stencils together (one conflict-free 32-bit
// shared load per array per step).  The Far-layout kernel serves raw-pointer calls.
#include "common.cuh"
#include "sell.h"
#include "stencil_eval.cuh"

namespace gb300 {

__device__ int g_status = 0;

namespace tma {

constexpr int kStages = 3;
constexpr int kConsumers = 256;  // 8 warps
constexpr int kThreads = kConsumers + 32;
constexpr unsigned long long kWaitNs = 4000000000ull;  // 4 s per wait

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *b, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(uint64_t *b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ unsigned long long now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}
// Bounded wait: false (and g_status set) when the deadline passes.
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity) {
    if (mbar_try_wait(b, parity)) return true;
    const unsigned long long t0 = now_ns();
    while (!mbar_try_wait(b, parity)) {
        if (now_ns() - t0 > kWaitNs) {
            atomicExch(&g_status, GB300_ERR_DEVICE_TIMEOUT);
            return false;
        }
    }
    return true;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *bar, uint64_t policy) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint"
        " [%0], [%1], %2, [%3], %4;" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(policy)
        : "memory");
}

struct Meta {
    int s0, s1, s0a, e0a, e1, staged;
};

template <int NW>
struct Cfg {
    static constexpr int kCap = NW == 1 ? 4096 : NW <= 3 ? 2048 : 1024;  // entries per stage
    static constexpr int kTile = kCap / 16;                               // stencils per tile
    static constexpr int kMeta = kTile + 8;  // sizes/offsets slots (window starts 4-aligned)
    static constexpr size_t kStageBytes = (size_t)kCap * 4 * (1 + NW) + (size_t)kMeta * 8;
    // ring depth: 4 stages for 4-6 outputs (one CTA per SM, small stages), else 3
    static constexpr int kRing = NW >= 4 ? 4 : kStages;
    static constexpr size_t kSmem = kRing * kStageBytes + 256;
};

struct Args {
    const float *src;
    float *dst[6];
    const float *w[6];  // compacted: the NW weight arrays in output order
    int dstStride[6];
    int outOf[6];       // weight array k feeds output outOf[k]
    const int *sizes;
    const int *offsets;
    const int *indices;
    int length, srcStride, start, end, numTiles;
    int vecSrc, vecDst[6];
};

template <int NW>
__device__ __forceinline__ void stage_ptrs(char *base, int stage, int **idx, float **w,
                                           int **sz, int **of) {
    char *p = base + (size_t)stage * Cfg<NW>::kStageBytes;
    *idx = (int *)p;
    p += (size_t)Cfg<NW>::kCap * 4;
    *w = (float *)p;
    p += (size_t)Cfg<NW>::kCap * 4 * NW;
    *sz = (int *)p;
    p += (size_t)Cfg<NW>::kMeta * 4;
    *of = (int *)p;
}

template <int NW, int VW>
// two CTAs per SM up to 5 outputs (5: 16-32 B of spills, still faster: 0.141 vs 0.186 ms);
// 6 outputs keep one (a second 4-stage ring would not fit the shared memory)
__global__ void __launch_bounds__(kThreads, NW >= 6 ? 1 : 2) k_stencils_tma(const Args a) {
    extern __shared__ __align__(128) char smem[];
    using C = Cfg<NW>;
    constexpr int S = C::kRing;
    __shared__ __align__(8) uint64_t full[S], empty[S];
    __shared__ Meta meta[S];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // Consumer groups: a tile holds kTile stencils (one per thread), fewer than the consumers
    // when every stencil carries 3 or 6 weight arrays; the consumers then split into groups
    // of kTile threads that take turns on the tiles of the ring, so all of them have a
    // stencil to work on (2 groups for 3 outputs, 4 for 6 with a 4-stage ring).
    constexpr int G = kConsumers / C::kTile;
    static_assert(G >= 1 && G <= S && kConsumers % G == 0, "consumer groups");
    constexpr int GT = kConsumers / G;  // threads per group
    constexpr int GW = GT / 32;         // warps per group
    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(&full[s], 32);
            mbar_init(&empty[s], GW);  // one group consumes each tile
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const uint64_t pol_stream = l2_evict_first(), pol_src = l2_evict_last();

    if (warp == kConsumers / 32) {
        // ---------------- producer warp ----------------
        int it = 0;
        for (int t = blockIdx.x; t < a.numTiles; t += gridDim.x, ++it) {
            const int stage = it % S;
            const uint32_t use = (uint32_t)(it / S);
            if (use > 0 && !mbar_wait(&empty[stage], (use - 1) & 1)) return;
            int *sidx, *ssz, *sof;
            float *sw;
            stage_ptrs<NW>(smem, stage, &sidx, &sw, &ssz, &sof);
            const int s0 = a.start + t * C::kTile;
            const int s1 = min(s0 + C::kTile, a.end);
            int e0 = 0, e1 = 0;
            if (lane == 0) {
                e0 = __ldg(a.offsets + s0);
                e1 = __ldg(a.offsets + s1 - 1) + __ldg(a.sizes + s1 - 1);
            }
            e0 = __shfl_sync(0xffffffffu, e0, 0);
            e1 = __shfl_sync(0xffffffffu, e1, 0);
            const int s0a = s0 & ~3, s1t = s1 & ~3;
            const int e0a = e0 & ~3, e1t = e1 & ~3;
            const bool staged = e1 >= e0 && (e1 - e0a) <= C::kCap;
            if (lane == 0) meta[stage] = Meta{s0, s1, s0a, e0a, e1, staged ? 1 : 0};
            uint32_t bytes = 0;
            if (s1t > s0a) bytes += (uint32_t)(s1t - s0a) * 8;
            if (staged && e1t > e0a) bytes += (uint32_t)(e1t - e0a) * 4 * (1 + NW);
            if (lane == 0) {
                mbar_arrive_expect_tx(&full[stage], bytes);
                if (s1t > s0a) {
                    bulk_g2s(ssz, a.sizes + s0a, (uint32_t)(s1t - s0a) * 4, &full[stage], pol_stream);
                    bulk_g2s(sof, a.offsets + s0a, (uint32_t)(s1t - s0a) * 4, &full[stage], pol_stream);
                }
                if (staged && e1t > e0a) {
                    const uint32_t nb = (uint32_t)(e1t - e0a) * 4;
                    bulk_g2s(sidx, a.indices + e0a, nb, &full[stage], pol_stream);
#pragma unroll
                    for (int k = 0; k < NW; ++k)
                        bulk_g2s(sw + (size_t)k * C::kCap, a.w[k] + e0a, nb, &full[stage], pol_stream);
                }
            }
            // ragged tails (fewer than 4 entries each) with plain loads
            const int st0 = max(s1t, s0a);
            if (lane < s1 - st0) {
                ssz[st0 - s0a + lane] = __ldg(a.sizes + st0 + lane);
                sof[st0 - s0a + lane] = __ldg(a.offsets + st0 + lane);
            }
            if (staged) {
                const int et0 = max(e1t, e0a);
                if (lane < e1 - et0) {
                    sidx[et0 - e0a + lane] = __ldg(a.indices + et0 + lane);
#pragma unroll
                    for (int k = 0; k < NW; ++k)
                        sw[(size_t)k * C::kCap + et0 - e0a + lane] = __ldg(a.w[k] + et0 + lane);
                }
            }
            __syncwarp();
            if (lane != 0) mbar_arrive(&full[stage]);
        }
        return;
    }

    // ---------------- consumer warps ----------------
    // group g takes this CTA's tiles it = g, g + G, g + 2G, ... (tile t = blockIdx.x + it * grid)
    const int grp = warp / GW;
    const int gtid = (int)threadIdx.x - grp * GT;
    int it = grp;
    for (int t = blockIdx.x + grp * gridDim.x; t < a.numTiles; t += G * gridDim.x, it += G) {
        const int stage = it % S;
        const uint32_t use = (uint32_t)(it / S);
        if (!mbar_wait(&full[stage], use & 1)) return;
        int *sidx, *ssz, *sof;
        float *sw;
        stage_ptrs<NW>(smem, stage, &sidx, &sw, &ssz, &sof);
        const Meta m = meta[stage];
        for (int i = m.s0 + gtid; i < m.s1; i += GT) {
            const int n = ssz[i - m.s0a];
            const int o = sof[i - m.s0a];
            if constexpr (VW == 12) {  // one output, 9-12 floats: single 12-wide pass
                if (m.staged && o >= m.e0a && o + n <= m.e1)
                    eval_one12(a, i, n, sidx, sw, o - m.e0a);
                else
                    eval_one<NW, 4>(a, i, n, nullptr, nullptr, 0, o, pol_src, pol_stream);
            } else if (m.staged && o >= m.e0a && o + n <= m.e1) {
                eval_one<NW, VW>(a, i, n, sidx, sw, C::kCap, o - m.e0a, pol_src, pol_stream);
            } else {
                eval_one<NW, VW>(a, i, n, nullptr, nullptr, 0, o, pol_src, pol_stream);
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[stage]);
    }
}

template <int NW, int VW>
static int launch(const Args &a, cudaStream_t s) {
    using C = Cfg<NW>;
    auto kern = k_stencils_tma<NW, VW>;
    static std::atomic<uint64_t> attr{0};  // devices whose function attribute is set
    const int st = once_per_device(attr, [&] {
        return check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)C::kSmem),
                          "stencils (staged): smem attribute");
    });
    if (st != GB300_OK) return st;
    static int perSm = 0;
    if (perSm == 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kern, kThreads, C::kSmem) !=
                cudaSuccess || perSm < 1)
            perSm = 1;
    }
    Args b = a;
    b.numTiles = (a.end - a.start + C::kTile - 1) / C::kTile;
    const int grid = min(b.numTiles, num_sms() * perSm);
    kern<<<grid, kThreads, C::kSmem, s>>>(b);
    count_launch();
    return GB300_OK;
}

// ---- sliced layout (sell.h): the same producer / ring / consumer-group scheme ----------------
// A tile is SPT consecutive slices (one warp each, one stencil per lane); the producer copies
// the tile's positions (sizes, destination rows) and its contiguous slot range (indices and
// weights, 128-byte multiples) into a stage; a consumer warp steps through entry j of its 32
// stencils together, reading index and weights with one conflict-free shared load each.

// VW of the pass over rows of at most 4 floats at 16-byte aligned rows: one 128-bit load per
// entry and 4 columns per pass, so more rows fit in registers per entry step.
constexpr int kNarrow = 44;

// Ring of an instantiation.  One output over rows of at most 4 floats: 2 stages of 8-slice
// tiles (refine pass at L=4 0.196 -> 0.179 ms; the same ring measured 1-5% slower for 8- and
// 12-wide rows, which keep 3 stages of 4-slice tiles).
template <int NW, int VW>
struct SellCfg {
    static constexpr bool kTwo = NW == 1 && VW == kNarrow;
    static constexpr int kSlots = kTwo ? 4096 : NW <= 3 ? 2048 : 1024;  // slots per stage
    static constexpr int kSpt = kSlots / 512;  // slices per tile (staged up to width 16)
    static constexpr size_t kStageBytes = (size_t)kSpt * 32 * 8 + (size_t)kSlots * 4 * (1 + NW);
    static constexpr int kRing = kTwo ? 2 : NW >= 4 ? 4 : kStages;
    static constexpr size_t kSmem = kRing * kStageBytes + 256;
};

struct SellArgs {
    const float *src;
    int srcStride, length;
    const int *sz, *sliceSlot, *idx, *outRow;
    const float *w[6];  // compacted
    int numSlices, numTiles;
    float *dst[6];
    int dstStride[6];
    int outOf[6];
    int vecDst[6];
};

struct SellMeta {
    int s0, s1, slot0, staged;
};

// Columns [c0, c0 + 8) of source row `id`, all 12 columns of a 9-12 wide row (VW = 12: three
// 16-byte loads; the row stride is a multiple of 4 floats, at least 12), or the 4 columns of a
// row of at most 4 floats (VW = kNarrow: one 16-byte load, stride a multiple of 4).
template <int VW>
__device__ __forceinline__ void gather_cols(const SellArgs &a, int id, int c0, uint64_t pol_src,
                                            float (&x)[VW == 12 ? 12 : VW == kNarrow ? 4 : 8]) {
    if constexpr (VW == kNarrow) {
        const float4 q =
            __ldg(reinterpret_cast<const float4 *>(a.src + (size_t)id * a.srcStride + c0));
        x[0] = q.x;
        x[1] = q.y;
        x[2] = q.z;
        x[3] = q.w;
    } else if constexpr (VW == 12) {
        const float4 *r = reinterpret_cast<const float4 *>(a.src + (size_t)id * a.srcStride);
#pragma unroll
        for (int v = 0; v < 3; ++v) {
            const float4 q = __ldg(r + v);
            x[4 * v] = q.x;
            x[4 * v + 1] = q.y;
            x[4 * v + 2] = q.z;
            x[4 * v + 3] = q.w;
        }
    } else {
        gather_row<VW>(a, id, c0, pol_src, x);
    }
}

// Elements [c0, c0 + CW) (those below the primvar length) of output `o`'s row `row`:
// 256-bit or 128-bit streaming stores where the output layout allows, else scalar ones.
template <int CW>
__device__ __forceinline__ void store_cols(const SellArgs &a, int o, int row, int c0,
                                           const float (&acc)[CW]) {
    float *d = a.dst[o] + (size_t)row * a.dstStride[o] + c0;
    const int rem = a.length - c0;
    if (CW == 8 && a.vecDst[o] == 8 && rem >= 8) {
        asm volatile("st.global.cs.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(d),
                     "f"(acc[0]), "f"(acc[1]), "f"(acc[2]), "f"(acc[3]), "f"(acc[4]),
                     "f"(acc[5]), "f"(acc[6]), "f"(acc[7])
                     : "memory");
        return;
    }
#pragma unroll
    for (int v = 0; v < CW / 4; ++v) {
        if (a.vecDst[o] && 4 * v + 4 <= rem) {
            asm volatile("st.global.cs.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(d + 4 * v),
                         "f"(acc[4 * v]), "f"(acc[4 * v + 1]), "f"(acc[4 * v + 2]),
                         "f"(acc[4 * v + 3])
                         : "memory");
        } else {
#pragma unroll
            for (int c = 4 * v; c < 4 * v + 4; ++c)
                if (c < rem) st_stream(d + c, acc[c]);
        }
    }
}

// Three CTAs per SM for one output (72 registers, 53 KB of ring each: the gathers are
// latency-bound and the smaller carve-out leaves more L1 for source rows; 0.267 -> 0.238 ms on
// the refine pass, 12-wide rows 0.372 -> 0.356 ms), and for 3 outputs over rows of up to 4
// floats; two otherwise (more would spill), one for 6 outputs.
template <int NW, int VW>
__global__ void __launch_bounds__(kThreads, NW >= 6 ? 1 : (NW == 1 || VW == kNarrow) ? 3 : 2)
    k_stencils_sell(const SellArgs a) {
    extern __shared__ __align__(128) char smem[];
    using C = SellCfg<NW, VW>;
    constexpr int S = C::kRing, SPT = C::kSpt;
    constexpr int G = 8 / SPT;          // consumer groups (one warp per slice of a tile)
    constexpr int GT = kConsumers / G;  // threads per group
    constexpr int GW = GT / 32;         // warps per group (= SPT)
    static_assert(G >= 1 && G <= S && GW == SPT, "consumer groups");
    __shared__ __align__(8) uint64_t full[S], empty[S];
    __shared__ SellMeta meta[S];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int st = 0; st < S; ++st) {
            mbar_init(&full[st], 32);
            mbar_init(&empty[st], GW);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const uint64_t pol_stream = l2_evict_first(), pol_src = l2_evict_last();
    auto stage = [&](int st, int **sz, int **orow, int **idx, float **w) {
        char *p = smem + (size_t)st * C::kStageBytes;
        *sz = (int *)p;
        *orow = *sz + SPT * 32;
        *idx = *orow + SPT * 32;
        *w = (float *)(*idx + C::kSlots);
    };
    if (warp == kConsumers / 32) {
        // producer
        int it = 0;
        for (int t = blockIdx.x; t < a.numTiles; t += gridDim.x, ++it) {
            const int st = it % S;
            const uint32_t use = (uint32_t)(it / S);
            if (use > 0 && !mbar_wait(&empty[st], (use - 1) & 1)) return;
            int *ssz, *sor, *sidx;
            float *sw;
            stage(st, &ssz, &sor, &sidx, &sw);
            const int s0 = t * SPT, s1 = min(s0 + SPT, a.numSlices);
            const int slot0 = __ldg(a.sliceSlot + s0), slot1 = __ldg(a.sliceSlot + s1);
            const int nslots = slot1 - slot0;
            const bool staged = nslots <= C::kSlots;
            if (lane == 0) {
                meta[st] = SellMeta{s0, s1, slot0, staged ? 1 : 0};
                const uint32_t pb = (uint32_t)(s1 - s0) * 128;
                const uint32_t eb = staged ? (uint32_t)nslots * 4 : 0;
                mbar_arrive_expect_tx(&full[st], 2 * pb + eb * (1 + NW));
                bulk_g2s(ssz, a.sz + (size_t)s0 * 32, pb, &full[st], pol_stream);
                bulk_g2s(sor, a.outRow + (size_t)s0 * 32, pb, &full[st], pol_stream);
                if (eb) {
                    bulk_g2s(sidx, a.idx + slot0, eb, &full[st], pol_stream);
#pragma unroll
                    for (int k = 0; k < NW; ++k)
                        bulk_g2s(sw + (size_t)k * C::kSlots, a.w[k] + slot0, eb, &full[st],
                                 pol_stream);
                }
            }
            __syncwarp();
            if (lane != 0) mbar_arrive(&full[st]);
        }
        return;
    }
    // consumers: group g takes this CTA's tiles it = g, g + G, ...; warp wg of the group takes
    // slice wg of the tile
    const int grp = warp / GW, wg = warp - grp * GW;
    // entry steps gathered together, columns per pass
    constexpr int R = VW == kNarrow ? (NW == 1 ? 6 : 4) : VW == 12 ? 2 : NW <= 3 ? 4 : 2;
    constexpr int CW = VW == 12 ? 12 : VW == kNarrow ? 4 : 8;
    int it = grp;
    for (int t = blockIdx.x + grp * gridDim.x; t < a.numTiles; t += G * gridDim.x, it += G) {
        const int st = it % S;
        const uint32_t use = (uint32_t)(it / S);
        if (!mbar_wait(&full[st], use & 1)) return;
        int *ssz, *sor, *sidx;
        float *sw;
        stage(st, &ssz, &sor, &sidx, &sw);
        const SellMeta m = meta[st];
        const int slice = m.s0 + wg;
        if (slice < m.s1) {
            const int n = ssz[wg * 32 + lane];
            const int row = sor[wg * 32 + lane];
            const int b0 = __ldg(a.sliceSlot + slice);
            const int width = (__ldg(a.sliceSlot + slice + 1) - b0) >> 5;
            const int base = b0 - m.slot0 + lane;  // this lane's slot of entry 0 in the stage
            for (int c0 = 0; c0 < a.length; c0 += CW) {
                float acc[NW][CW];
#pragma unroll
                for (int k = 0; k < NW; ++k)
#pragma unroll
                    for (int c = 0; c < CW; ++c) acc[k][c] = 0.0f;
                for (int j0 = 0; j0 < width; j0 += R) {
                    int ids[R];
                    float wk[R][NW];
#pragma unroll
                    for (int q = 0; q < R; ++q) {
                        const int j = j0 + q;
                        if (j < n) {
                            if (m.staged) {
                                ids[q] = sidx[base + j * 32];
#pragma unroll
                                for (int k = 0; k < NW; ++k)
                                    wk[q][k] = sw[(size_t)k * C::kSlots + base + j * 32];
                            } else {
                                ids[q] = ld_stream(a.idx + b0 + lane + (size_t)j * 32, pol_stream);
#pragma unroll
                                for (int k = 0; k < NW; ++k)
                                    wk[q][k] = ld_stream(a.w[k] + b0 + lane + (size_t)j * 32,
                                                         pol_stream);
                            }
                        }
                    }
                    float x[R][CW];
#pragma unroll
                    for (int q = 0; q < R; ++q)
                        if (j0 + q < n) gather_cols<VW>(a, ids[q], c0, pol_src, x[q]);
#pragma unroll
                    for (int q = 0; q < R; ++q)
                        if (j0 + q < n)
#pragma unroll
                            for (int k = 0; k < NW; ++k)
#pragma unroll
                                for (int c = 0; c < CW; ++c)
                                    acc[k][c] = fmaf(wk[q][k], x[q][c], acc[k][c]);
                }
                if (row >= 0) {
#pragma unroll
                    for (int k = 0; k < NW; ++k) store_cols(a, a.outOf[k], row, c0, acc[k]);
                }
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[st]);
    }
}

template <int NW, int VW>
static int launch_sell(const SellArgs &a, cudaStream_t s) {
    using C = SellCfg<NW, VW>;
    auto kern = k_stencils_sell<NW, VW>;
    static std::atomic<uint64_t> attr{0};
    const int st = once_per_device(attr, [&] {
        return check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)C::kSmem),
                          "stencils (sliced): smem attribute");
    });
    if (st != GB300_OK) return st;
    static int perSm = 0;
    if (perSm == 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kern, kThreads, C::kSmem) !=
                cudaSuccess || perSm < 1)
            perSm = 1;
    }
    SellArgs b = a;
    b.numTiles = (a.numSlices + C::kSpt - 1) / C::kSpt;
    const int grid = min(b.numTiles, num_sms() * perSm);
    kern<<<grid, kThreads, C::kSmem, s>>>(b);
    count_launch();
    return GB300_OK;
}

}  // namespace tma

// Staged path; returns GB300_ERR_UNSUPPORTED when the arguments do not meet its alignment
// preconditions (the caller then uses the group kernel).
int eval_stencils_staged(const float *src, float *const *dst, const int *strides,
                         const float *const *w, int length, int srcStride, const int *sizes,
                         const int *offsets, const int *indices, int start, int end,
                         cudaStream_t s) {
    auto al16 = [](const void *p) { return ((uintptr_t)p & 15) == 0; };
    auto al32 = [](const void *p) { return ((uintptr_t)p & 31) == 0; };
    if (!al16(sizes) || !al16(offsets) || !al16(indices)) return GB300_ERR_UNSUPPORTED;
    tma::Args a{};
    a.src = src;
    a.sizes = sizes;
    a.offsets = offsets;
    a.indices = indices;
    a.length = length;
    a.srcStride = srcStride;
    a.start = start;
    a.end = end;
    int nw = 0;
    for (int k = 0; k < 6; ++k) {
        if (!dst[k]) continue;
        if (!al16(w[k])) return GB300_ERR_UNSUPPORTED;
        a.dst[k] = dst[k];
        a.dstStride[k] = strides[k];
        a.vecDst[k] = (al32(dst[k]) && strides[k] % 8 == 0) ? 8
                      : (al16(dst[k]) && strides[k] % 4 == 0) ? 4 : 0;
        a.w[nw] = w[k];
        a.outOf[nw] = k;
        ++nw;
    }
    // source row loads: 256-bit when rows are 32-byte aligned, 128-bit when 16-byte aligned
    a.vecSrc = (al32(src) && srcStride % 8 == 0) ? 8 : (al16(src) && srcStride % 4 == 0) ? 4 : 1;
    // one output 9-12 floats wide over 16-byte aligned rows (stride >= 12): single 12-wide pass
    if (nw == 1 && a.vecSrc >= 4 && length > 8 && length <= 12) return tma::launch<1, 12>(a, s);
    switch (nw * 10 + a.vecSrc) {
        case 18: return tma::launch<1, 8>(a, s);
        case 14: return tma::launch<1, 4>(a, s);
        case 11: return tma::launch<1, 1>(a, s);
        case 28: return tma::launch<2, 8>(a, s);
        case 24: return tma::launch<2, 4>(a, s);
        case 21: return tma::launch<2, 1>(a, s);
        case 38: return tma::launch<3, 8>(a, s);
        case 34: return tma::launch<3, 4>(a, s);
        case 31: return tma::launch<3, 1>(a, s);
        case 48: return tma::launch<4, 8>(a, s);
        case 44: return tma::launch<4, 4>(a, s);
        case 41: return tma::launch<4, 1>(a, s);
        case 58: return tma::launch<5, 8>(a, s);
        case 54: return tma::launch<5, 4>(a, s);
        case 51: return tma::launch<5, 1>(a, s);
        case 68: return tma::launch<6, 8>(a, s);
        case 64: return tma::launch<6, 4>(a, s);
        case 61: return tma::launch<6, 1>(a, s);
        default: return GB300_ERR_UNSUPPORTED;
    }
}

int eval_stencils_sell(const SellTable &t, const float *src, float *const *dst,
                       const int *strides, const float *const *w, int length, int srcStride,
                       cudaStream_t s, const char *who) {
    if (t.numSlices == 0) return ok();
    if (!src || length <= 0 || srcStride < length)
        return fail(GB300_ERR_INVALID_ARGUMENT, "%s: bad source", who);
    auto al16 = [](const void *p) { return ((uintptr_t)p & 15) == 0; };
    auto al32 = [](const void *p) { return ((uintptr_t)p & 31) == 0; };
    tma::SellArgs a{};
    a.src = src;
    a.srcStride = srcStride;
    a.length = length;
    a.sz = t.sz;
    a.sliceSlot = t.sliceSlot;
    a.idx = t.idx;
    a.outRow = t.outRow;
    a.numSlices = t.numSlices;
    int nw = 0;
    for (int k = 0; k < 6; ++k) {
        if (!dst[k]) continue;
        if (!w[k] || strides[k] < length)
            return fail(GB300_ERR_INVALID_ARGUMENT, "%s: output %d stride / weights", who, k);
        a.dst[k] = dst[k];
        a.dstStride[k] = strides[k];
        a.vecDst[k] = (al32(dst[k]) && strides[k] % 8 == 0) ? 8
                      : (al16(dst[k]) && strides[k] % 4 == 0) ? 4 : 0;
        a.w[nw] = w[k];
        a.outOf[nw] = k;
        ++nw;
    }
    if (nw == 0) return ok();
    const int vw = (al32(src) && srcStride % 8 == 0) ? 8 : (al16(src) && srcStride % 4 == 0) ? 4 : 1;
    int r;
    if ((nw == 1 || nw == 3) && vw >= 4 && length > 8 && length <= 12) {
        r = nw == 1 ? tma::launch_sell<1, 12>(a, s) : tma::launch_sell<3, 12>(a, s);
    } else if ((nw == 1 || nw == 3) && vw >= 4 && length <= 4) {
        r = nw == 1 ? tma::launch_sell<1, tma::kNarrow>(a, s) : tma::launch_sell<3, tma::kNarrow>(a, s);
    } else {
        switch (nw * 10 + vw) {
#define GB300_SELL_CASES(NW)                                   \
    case NW * 10 + 8: r = tma::launch_sell<NW, 8>(a, s); break; \
    case NW * 10 + 4: r = tma::launch_sell<NW, 4>(a, s); break; \
    case NW * 10 + 1: r = tma::launch_sell<NW, 1>(a, s); break;
            GB300_SELL_CASES(1)
            GB300_SELL_CASES(2)
            GB300_SELL_CASES(3)
            GB300_SELL_CASES(4)
            GB300_SELL_CASES(5)
            GB300_SELL_CASES(6)
#undef GB300_SELL_CASES
            default: return fail(GB300_ERR_INVALID_ARGUMENT, "%s: %d outputs", who, nw);
        }
    }
    return r != GB300_OK ? r : check_launch(who);
}

}  // namespace gb300

namespace gb300 {

int status_word_address(int **out) {
    void *p = nullptr;
    const int st = check_cuda(cudaGetSymbolAddress(&p, g_status), "status word address");
    *out = (int *)p;
    return st;
}

}  // namespace gb300

extern "C" int GB300GetDeviceStatus(void) {
    using namespace gb300;
    int v = 0;
    int st = check_cuda(cudaDeviceSynchronize(), "GB300GetDeviceStatus");
    if (st != GB300_OK) return st;
    st = check_cuda(cudaMemcpyFromSymbol(&v, g_status, sizeof(int)), "GB300GetDeviceStatus");
    if (st != GB300_OK) return st;
    if (v != 0) {
        const int zero = 0;
        cudaMemcpyToSymbol(g_status, &zero, sizeof(int));
        return fail(v, "a staged kernel's bounded wait expired");
    }
    return ok();
}
