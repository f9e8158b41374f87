// Internal helpers of libbubbledyn: context, error reporting, device buffers.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/bubbledyn.h"

namespace bd {

// Thread-local error text behind bd_last_error_string().
void set_error(const char* fmt, ...);
void clear_error();

struct Error {
    bd_status st;
};

// Throwing helpers used inside the library; every extern "C" entry point
// catches and converts to a bd_status.
[[noreturn]] void fail(bd_status st, const char* fmt, ...);

inline void cuda_check(cudaError_t e, const char* what, const char* file, int line) {
    if (e != cudaSuccess) {
        fail(e == cudaErrorMemoryAllocation ? BD_ERR_OOM : BD_ERR_CUDA, "%s: %s (%s:%d)", what,
             cudaGetErrorString(e), file, line);
    }
}
#define BD_CUDA(x) ::bd::cuda_check((x), #x, __FILE__, __LINE__)
#define BD_LAUNCHED(ctx) ::bd::after_launch((ctx), __FILE__, __LINE__)

template <class F>
bd_status guard(F&& f) {
    try {
        clear_error();
        f();
        return BD_OK;
    } catch (const Error& e) {
        return e.st;
    } catch (const std::bad_alloc&) {
        set_error("host allocation failed");
        return BD_ERR_OOM;
    } catch (...) {
        set_error("unknown exception");
        return BD_ERR_INVALID_ARG;
    }
}

// Device allocation owned by a context.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), bytes(o.bytes) { o.p = nullptr; o.bytes = 0; }
    DevBuf& operator=(DevBuf&& o) noexcept {
        if (this != &o) { release(); p = o.p; bytes = o.bytes; o.p = nullptr; o.bytes = 0; }
        return *this;
    }
    ~DevBuf() { release(); }
    void alloc(size_t n) {
        if (n == bytes && p) return;
        release();
        if (n == 0) return;
        BD_CUDA(cudaMalloc(&p, n));
        bytes = n;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
};

}  // namespace bd

#include <map>

struct bd_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int sm_count = 0;
    int64_t launches = 0;       // kernels of this library launched by the context
    // work counter of the persistent Gilmore launches made by bd_gilmore_run_device
    // (allocated with the context, freed with it)
    unsigned long long* gil_counter = nullptr;
    // device blocks released by finished solves, reused by the next one of the same size
    std::multimap<size_t, void*> pool;
    size_t pool_bytes = 0;
};

namespace bd {
// Device block from the context's pool (or cudaMalloc); returned by release().
struct PoolBuf {
    bd_context* ctx = nullptr;
    void* p = nullptr;
    size_t bytes = 0;
    PoolBuf() = default;
    PoolBuf(const PoolBuf&) = delete;
    PoolBuf& operator=(const PoolBuf&) = delete;
    PoolBuf(PoolBuf&& o) noexcept : ctx(o.ctx), p(o.p), bytes(o.bytes) { o.p = nullptr; o.bytes = 0; }
    PoolBuf& operator=(PoolBuf&& o) noexcept {
        if (this != &o) { release(); ctx = o.ctx; p = o.p; bytes = o.bytes; o.p = nullptr; o.bytes = 0; }
        return *this;
    }
    ~PoolBuf() { release(); }
    void alloc(bd_context* c, size_t n);
    void release();
    template <class T>
    T* as() const { return static_cast<T*>(p); }
};
void pool_trim(bd_context* ctx);
}  // namespace bd

namespace bd {
void after_launch(bd_context* ctx, const char* file, int line);
void ctx_check(bd_context* ctx);
// z-chunk for which tiles * ceil(nz / zb) CTAs fill whole waves of `slots`
// resident CTAs (at least `fill` of the last wave busy), the largest such
// chunk of at least 8 planes with the chunk count rounded up to cover w waves;
// failing that, the chunk count rounded down (just under w waves); 16 if
// neither qualifies.  down_first tries the rounded-down counts first (fewer,
// longer chunks, for kernels with a long per-chunk prologue).
inline int wave_fitted_zb(long long tiles, int nz, long long slots, double fill = 0.97, bool down_first = false) {
    for (int pass = 0; pass < 2; ++pass)
        for (int w = 1; w <= 16; ++w) {
            const bool down = (pass == 0) == down_first;
            const long long chunks = down ? (w * slots) / tiles : (w * slots + tiles - 1) / tiles;
            if (chunks > nz) break;
            if (chunks < 1) continue;
            const int zb = (int)((nz + chunks - 1) / chunks);
            if (zb < 8) break;
            const long long n = tiles * ((nz + zb - 1) / zb);
            const long long cap = ((n + slots - 1) / slots) * slots;
            if ((double)n >= fill * (double)cap) return zb;
        }
    return 16;
}

}  // namespace bd
