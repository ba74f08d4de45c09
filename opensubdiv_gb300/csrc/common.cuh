// Shared host/device helpers for libosd_gb300.so: status reporting, launch accounting and
// small PTX wrappers.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/osd_gb300.h"

namespace gb300 {

// ---- status -------------------------------------------------------------------------------

// Records `msg` as the calling thread's last error and returns `code`.
int fail(int code, const char *fmt, ...);
// Clears the calling thread's last error and returns GB300_OK.
int ok();
// Maps a CUDA error to a status (recording its message); GB300_OK for cudaSuccess.
int check_cuda(cudaError_t e, const char *what);
// Checks the launch that was just queued.
int check_launch(const char *what);

extern std::atomic<uint64_t> g_launches;
inline void count_launch(uint64_t n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// Number of SMs of the current device (cached per device).
int num_sms();

// Stream-ordered scratch from a memory pool the library keeps per device: allocations and
// frees are ordered on `s` like cudaMallocAsync / cudaFreeAsync, but up to kScratchRetainBytes
// of freed memory stay mapped in the pool between calls (the device's default pool returns
// freed memory at every synchronisation, so a per-call scratch paid a fresh mapping, ~0.1 ms,
// on every call).
constexpr size_t kScratchRetainBytes = size_t(512) << 20;
int scratch_alloc(void **p, size_t bytes, cudaStream_t s, const char *who);
void scratch_free(void *p, cudaStream_t s);

// Device address of the library's status word on the current device (the word
// GB300GetDeviceStatus reads and clears; staged kernels record an expired bounded wait there).
int status_word_address(int **out);

// Runs `fn` (returning a status) once per device for one call site: `done` is that call site's
// bitmask of devices it already succeeded on (devices >= 64 run it every time).
template <class F>
int once_per_device(std::atomic<uint64_t> &done, F fn) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return fn();
    const uint64_t bit = 1ull << dev;
    if (done.load(std::memory_order_acquire) & bit) return GB300_OK;
    const int st = fn();
    if (st == GB300_OK) done.fetch_or(bit, std::memory_order_release);
    return st;
}

// ---- device helpers -----------------------------------------------------------------------

// L2 eviction policies (createpolicy) for the cache-hinted loads below.
__device__ __forceinline__ uint64_t l2_evict_first() {
    uint64_t p;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ uint64_t l2_evict_last() {
    uint64_t p;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}

// Streaming (read-once) 32-bit loads for the stencil table: no L1 allocation and an
// evict-first L2 policy, so the table stream does not push the source rows out of L2.
__device__ __forceinline__ int ld_stream(const int *p, uint64_t pol) {
    int v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.b32 %0, [%1], %2;"
                 : "=r"(v) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ float ld_stream(const float *p, uint64_t pol) {
    float v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.f32 %0, [%1], %2;"
                 : "=f"(v) : "l"(p), "l"(pol));
    return v;
}

// Source-row loads: read-only path, kept in L1, evict-last in L2 (the control points are
// re-read by every stencil that touches them).
__device__ __forceinline__ float ld_src(const float *p, uint64_t pol) {
    float v;
    asm("ld.global.nc.L1::evict_last.L2::cache_hint.f32 %0, [%1], %2;"
                 : "=f"(v) : "l"(p), "l"(pol));
    return v;
}

__device__ __forceinline__ int ld_keep(const int *p, uint64_t pol) {
    int v;
    asm("ld.global.nc.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ int4 ld_keep4(const int *p, uint64_t pol) {
    int4 v;
    asm("ld.global.nc.L2::cache_hint.v4.b32 {%0, %1, %2, %3}, [%4], %5;"
        : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
        : "l"(p), "l"(pol));
    return v;
}

// Streaming stores for outputs (written once, not re-read by this launch).
__device__ __forceinline__ void st_stream(float *p, float v) {
    asm volatile("st.global.cs.f32 [%0], %1;" ::"l"(p), "f"(v) : "memory");
}

}  // namespace gb300
