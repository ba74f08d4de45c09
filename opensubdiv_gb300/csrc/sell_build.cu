// Device construction of the sliced evaluation layout (sell.h) of a stencil table: locality
// order (radix sort of the stencils by lowest control index, when consecutive stencils jump by
// more than 1% of the index range on average), stable size sort within windows of 256
// positions, slice widths and an exclusive scan of their slot counts, then one thread per
// position copying its stencil's entries into its lane of the slice.
#include <climits>

#include <cub/cub.cuh>

#include "common.cuh"
#include "sell.h"

namespace gb300 {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kWindow = 256;  // size-sort window (8 slices)

int grid_of(long long items, int perBlock) {
    const long long b = (items + perBlock - 1) / perBlock;
    return (int)std::max<long long>(1, std::min<long long>(b, (long long)num_sms() * 16));
}

// Per stencil its lowest control index (entries sorted: the first; -1 when empty), and the
// sum / max of the jumps between consecutive stencils' keys (empty stencils count as 0).
__global__ void k_keys(const int *sizes, const int *offsets, const int *idx, int n, int *keys,
                       int *iota, unsigned long long *jump, int *maxKey) {
    unsigned long long j = 0;
    int mx = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int k = sizes[i] > 0 ? idx[offsets[i]] : -1;
        keys[i] = k;
        iota[i] = i;
        const int a = max(k, 0);
        mx = max(mx, a);
        if (i > 0) {
            const int b = sizes[i - 1] > 0 ? idx[offsets[i - 1]] : 0;
            j += (unsigned long long)(a > b ? a - b : b - a);
        }
    }
    for (int d = 16; d; d >>= 1) {
        j += __shfl_xor_sync(kFull, j, d);
        mx = max(mx, __shfl_xor_sync(kFull, mx, d));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(jump, j);
        atomicMax(maxKey, mx);
    }
}

// One block of kWindow threads per window: stable descending sort of the window's stencils by
// size (rank = larger sizes + equal sizes earlier in the window).  Positions in [n, npos) get
// size 0 and row -1 and rank after every stencil of the (last) window.
__global__ void __launch_bounds__(kWindow) k_window(const int *sizes, const int *order, int n,
                                                    int npos, int *sz, int *row) {
    __shared__ int key[kWindow];
    const int i = threadIdx.x, p = blockIdx.x * kWindow + i;
    const int id = p < n ? (order ? order[p] : p) : -1;
    const int k = p < n ? sizes[id] : -1;
    key[i] = p < npos ? k : INT_MIN;
    __syncthreads();
    if (p >= npos) return;
    int r = 0;
    for (int j = 0; j < kWindow; ++j) {
        const int kj = key[j];
        r += (kj > k) || (kj == k && j < i);
    }
    const int q = blockIdx.x * kWindow + r;
    sz[q] = max(k, 0);
    row[q] = id;
}

// Warp per slice: slot count 32 * (largest size of its 32 stencils).
__global__ void k_width(const int *sz, int ns, long long *slots) {
    const int lane = threadIdx.x & 31, warps = blockDim.x >> 5;
    for (int sl = blockIdx.x * warps + (threadIdx.x >> 5); sl < ns; sl += gridDim.x * warps) {
        int m = sz[sl * 32 + lane];
        for (int d = 16; d; d >>= 1) m = max(m, __shfl_xor_sync(kFull, m, d));
        if (lane == 0) slots[sl] = 32LL * m;
    }
}

struct Weights {
    const float *in[6];
    float *out[6];
};

// Thread per position: its stencil's entries into slots start[s] + 32 j + lane (zeros past the
// stencil's size up to the slice width); lane 0 of each slice records the 32-bit slot offset.
__global__ void k_fill(const int *sz, const int *row, const long long *start, int ns,
                       const int *offsets, const int *indices, Weights w, int *sliceSlot,
                       int *idx) {
    const long long npos = (long long)ns * 32;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npos;
         p += (long long)gridDim.x * blockDim.x) {
        const int sl = (int)(p >> 5), lane = (int)(p & 31);
        const long long b = start[sl];
        const int width = (int)((start[sl + 1] - b) >> 5);
        if (lane == 0) sliceSlot[sl] = (int)b;
        if (p == 0) sliceSlot[ns] = (int)start[ns];
        const int n = sz[p], r = row[p];
        const long long o = r >= 0 ? offsets[r] : 0;
        for (int j = 0; j < width; ++j) {
            const long long slot = b + 32LL * j + lane;
            const bool on = j < n;
            idx[slot] = on ? indices[o + j] : 0;
#pragma unroll
            for (int k = 0; k < 6; ++k)
                if (w.in[k]) w.out[k][slot] = on ? w.in[k][o + j] : 0.0f;
        }
    }
}

// Stream-ordered temporaries released when the build returns.
struct Temps {
    cudaStream_t s;
    void *p[12] = {};
    int n = 0;
    template <class T>
    T *get(size_t count, const char *who) {
        void *q = nullptr;
        if (scratch_alloc(&q, std::max<size_t>(count * sizeof(T), 16), s, who) != GB300_OK)
            return nullptr;
        p[n++] = q;
        return (T *)q;
    }
    ~Temps() {
        for (int i = 0; i < n; ++i) scratch_free(p[i], s);
    }
};

}  // namespace

int build_sell(int n, const int *sizes, const int *offsets, const int *indices,
               const float *const *w, cudaStream_t s, SellTable &t, void *owned[10],
               const char *who) {
    t = SellTable{};
    for (int k = 0; k < 10; ++k) owned[k] = nullptr;
    if (n <= 0) return ok();
    auto fail_all = [&](int code) {
        for (int k = 0; k < 10; ++k)
            if (owned[k]) cudaFree(owned[k]), owned[k] = nullptr;
        t = SellTable{};
        return code;
    };
    Temps tmp{s};
    // locality order
    const int *order = nullptr;
    if (n >= 4096) {
        int *keys = tmp.get<int>(n, who), *keys2 = tmp.get<int>(n, who);
        int *iota = tmp.get<int>(n, who), *ord = tmp.get<int>(n, who);
        unsigned long long *jump = tmp.get<unsigned long long>(1, who);
        int *maxKey = tmp.get<int>(1, who);
        if (!keys || !keys2 || !iota || !ord || !jump || !maxKey) return GB300_ERR_OUT_OF_MEMORY;
        if (check_cuda(cudaMemsetAsync(jump, 0, 8, s), who) != GB300_OK ||
            check_cuda(cudaMemsetAsync(maxKey, 0, 4, s), who) != GB300_OK)
            return GB300_ERR_CUDA;
        k_keys<<<grid_of(n, 256), 256, 0, s>>>(sizes, offsets, indices, n, keys, iota, jump,
                                                maxKey);
        count_launch();
        unsigned long long hj = 0;
        int hm = 0;
        if (check_launch(who) != GB300_OK ||
            check_cuda(cudaMemcpyAsync(&hj, jump, 8, cudaMemcpyDeviceToHost, s), who) != GB300_OK ||
            check_cuda(cudaMemcpyAsync(&hm, maxKey, 4, cudaMemcpyDeviceToHost, s), who) !=
                GB300_OK ||
            check_cuda(cudaStreamSynchronize(s), who) != GB300_OK)
            return GB300_ERR_CUDA;
        if ((double)hj / (n - 1) >= 0.01 * std::max(1, hm)) {
            size_t bytes = 0;
            cub::DeviceRadixSort::SortPairs(nullptr, bytes, keys, keys2, iota, ord, n, 0, 32, s);
            void *cubTmp = tmp.get<char>(bytes, who);
            if (!cubTmp ||
                check_cuda(cub::DeviceRadixSort::SortPairs(cubTmp, bytes, keys, keys2, iota, ord,
                                                           n, 0, 32, s),
                           who) != GB300_OK)
                return GB300_ERR_CUDA;
            count_launch();
            order = ord;
        }
    }
    const int ns = (n + 31) / 32;
    const long long npos = (long long)ns * 32;
    // positions
    if (check_cuda(cudaMalloc(&owned[0], npos * 4), who) != GB300_OK ||
        check_cuda(cudaMalloc(&owned[9], npos * 4), who) != GB300_OK)
        return fail_all(GB300_ERR_OUT_OF_MEMORY);
    int *sz = (int *)owned[0], *row = (int *)owned[9];
    k_window<<<(int)((npos + kWindow - 1) / kWindow), kWindow, 0, s>>>(sizes, order, n, (int)npos,
                                                                      sz, row);
    count_launch();
    // slice widths and slot offsets
    long long *slots = tmp.get<long long>((size_t)ns + 1, who);
    long long *start = tmp.get<long long>((size_t)ns + 1, who);
    if (!slots || !start) return fail_all(GB300_ERR_OUT_OF_MEMORY);
    if (check_cuda(cudaMemsetAsync(slots + ns, 0, 8, s), who) != GB300_OK)
        return fail_all(GB300_ERR_CUDA);
    k_width<<<grid_of((long long)ns * 32, 256), 256, 0, s>>>(sz, ns, slots);
    count_launch();
    size_t bytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, bytes, slots, start, ns + 1, s);
    void *cubTmp = tmp.get<char>(bytes, who);
    if (!cubTmp || check_cuda(cub::DeviceScan::ExclusiveSum(cubTmp, bytes, slots, start, ns + 1, s),
                              who) != GB300_OK)
        return fail_all(GB300_ERR_CUDA);
    count_launch();
    long long total = 0;
    if (check_launch(who) != GB300_OK ||
        check_cuda(cudaMemcpyAsync(&total, start + ns, 8, cudaMemcpyDeviceToHost, s), who) !=
            GB300_OK ||
        check_cuda(cudaStreamSynchronize(s), who) != GB300_OK)
        return fail_all(GB300_ERR_CUDA);
    if (total > INT_MAX) return fail_all(GB300_ERR_UNSUPPORTED);
    // entries
    const size_t eb = std::max<size_t>((size_t)total * 4, 16);
    if (check_cuda(cudaMalloc(&owned[1], ((size_t)ns + 1) * 4), who) != GB300_OK ||
        check_cuda(cudaMalloc(&owned[2], eb), who) != GB300_OK)
        return fail_all(GB300_ERR_OUT_OF_MEMORY);
    Weights wt{};
    for (int k = 0; k < 6; ++k) {
        if (!w[k]) continue;
        if (check_cuda(cudaMalloc(&owned[3 + k], eb), who) != GB300_OK)
            return fail_all(GB300_ERR_OUT_OF_MEMORY);
        wt.in[k] = w[k];
        wt.out[k] = (float *)owned[3 + k];
    }
    k_fill<<<grid_of(npos, 256), 256, 0, s>>>(sz, row, start, ns, offsets, indices, wt,
                                              (int *)owned[1], (int *)owned[2]);
    count_launch();
    if (check_launch(who) != GB300_OK || check_cuda(cudaStreamSynchronize(s), who) != GB300_OK)
        return fail_all(GB300_ERR_CUDA);
    t.numSlices = ns;
    t.sz = sz;
    t.sliceSlot = (const int *)owned[1];
    t.idx = (const int *)owned[2];
    for (int k = 0; k < 6; ++k) t.w[k] = (const float *)owned[3 + k];
    t.outRow = row;
    return ok();
}

}  // namespace gb300
