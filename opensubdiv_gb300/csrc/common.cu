// Status reporting, launch accounting and device queries shared by every entry point.
#include "common.cuh"

#include <cstdarg>
#include <mutex>
#include <vector>

namespace gb300 {

std::atomic<uint64_t> g_launches{0};

static thread_local std::string t_last_error;

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    t_last_error = buf;
    return code;
}

int ok() {
    t_last_error.clear();
    return GB300_OK;
}

int check_cuda(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return GB300_OK;
    int code = (e == cudaErrorMemoryAllocation) ? GB300_ERR_OUT_OF_MEMORY : GB300_ERR_CUDA;
    return fail(code, "%s: %s", what, cudaGetErrorString(e));
}

int check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return check_cuda(e, what);
    return ok();
}

int scratch_alloc(void **p, size_t bytes, cudaStream_t s, const char *who) {
    static std::mutex m;
    static std::vector<cudaMemPool_t> pools;
    int dev = 0;
    int st = check_cuda(cudaGetDevice(&dev), who);
    if (st != GB300_OK) return st;
    cudaMemPool_t pool = nullptr;
    {
        std::lock_guard<std::mutex> lock(m);
        if ((int)pools.size() <= dev) pools.resize(dev + 1, nullptr);
        if (!pools[dev]) {
            cudaMemPoolProps props = {};
            props.allocType = cudaMemAllocationTypePinned;
            props.location.type = cudaMemLocationTypeDevice;
            props.location.id = dev;
            cudaMemPool_t created = nullptr;
            if ((st = check_cuda(cudaMemPoolCreate(&created, &props), who)) != GB300_OK)
                return st;
            uint64_t retain = kScratchRetainBytes;
            if ((st = check_cuda(cudaMemPoolSetAttribute(
                                     created, cudaMemPoolAttrReleaseThreshold, &retain),
                                 who)) != GB300_OK) {
                cudaMemPoolDestroy(created);
                return st;
            }
            pools[dev] = created;
        }
        pool = pools[dev];
    }
    return check_cuda(cudaMallocFromPoolAsync(p, bytes < 16 ? 16 : bytes, pool, s), who);
}

void scratch_free(void *p, cudaStream_t s) {
    if (p) cudaFreeAsync(p, s);
}

int num_sms() {
    static std::mutex m;
    static std::vector<int> cache;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    std::lock_guard<std::mutex> lock(m);
    if ((int)cache.size() <= dev) cache.resize(dev + 1, 0);
    if (cache[dev] == 0) {
        int n = 0;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        cache[dev] = n > 0 ? n : 1;
    }
    return cache[dev];
}

}  // namespace gb300

extern "C" {

const char *GB300GetLastErrorString(void) { return gb300::t_last_error.c_str(); }

int GB300GetVersion(void) { return 100; }

uint64_t GB300GetLaunchCount(void) { return gb300::g_launches.load(); }

int GB300Synchronize(void *stream) {
    return gb300::check_cuda(cudaStreamSynchronize(gb300::as_stream(stream)), "GB300Synchronize");
}

}  // extern "C"
