// Context lifetime, error text and small host helpers of the C ABI.
#include "bd_internal.h"

#include <cmath>
#include <cstring>

namespace bd {

static thread_local std::string g_err;

void set_error(const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
}

void clear_error() { g_err.clear(); }

void fail(bd_status st, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    throw Error{st};
}

void after_launch(bd_context* ctx, const char* file, int line) {
    cuda_check(cudaGetLastError(), "kernel launch", file, line);
    ctx->launches++;
}

void PoolBuf::alloc(bd_context* c, size_t n) {
    release();
    ctx = c;
    if (n == 0) return;
    auto it = ctx->pool.find(n);
    if (it != ctx->pool.end()) {
        p = it->second;
        ctx->pool.erase(it);
        ctx->pool_bytes -= n;
    } else {
        cudaError_t e = cudaMalloc(&p, n);
        if (e == cudaErrorMemoryAllocation) {
            cudaGetLastError();
            pool_trim(ctx);
            e = cudaMalloc(&p, n);
        }
        if (e != cudaSuccess) { p = nullptr; cuda_check(e, "cudaMalloc", __FILE__, __LINE__); }
    }
    bytes = n;
}

void PoolBuf::release() {
    if (p && ctx) {
        ctx->pool.emplace(bytes, p);
        ctx->pool_bytes += bytes;
    }
    p = nullptr;
    bytes = 0;
}

void pool_trim(bd_context* ctx) {
    cudaDeviceSynchronize();
    for (auto& kv : ctx->pool) cudaFree(kv.second);
    ctx->pool.clear();
    ctx->pool_bytes = 0;
}

void ctx_check(bd_context* ctx) {
    if (!ctx) fail(BD_ERR_INVALID_ARG, "null context");
    BD_CUDA(cudaSetDevice(ctx->device));
}

}  // namespace bd

using namespace bd;

extern "C" {

const char* bd_last_error_string(void) { return g_err.c_str(); }

int bd_abi_version(void) { return BD_ABI_VERSION; }

bd_status bd_context_create(int device, bd_context** out) {
    return guard([&] {
        if (!out) fail(BD_ERR_INVALID_ARG, "null output pointer");
        *out = nullptr;
        int n = 0;
        BD_CUDA(cudaGetDeviceCount(&n));
        if (device < 0 || device >= n) fail(BD_ERR_INVALID_ARG, "device %d out of range (%d devices)", device, n);
        BD_CUDA(cudaSetDevice(device));
        auto* c = new bd_context();
        c->device = device;
        cudaDeviceProp prop;
        BD_CUDA(cudaGetDeviceProperties(&prop, device));
        c->sm_count = prop.multiProcessorCount;
        BD_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        BD_CUDA(cudaEventCreate(&c->ev0));
        BD_CUDA(cudaEventCreate(&c->ev1));
        BD_CUDA(cudaMalloc(&c->gil_counter, 256));
        *out = c;
    });
}

bd_status bd_context_destroy(bd_context* ctx) {
    return guard([&] {
        if (!ctx) return;
        cudaSetDevice(ctx->device);
        if (ctx->stream) cudaStreamSynchronize(ctx->stream);
        pool_trim(ctx);
        if (ctx->gil_counter) cudaFree(ctx->gil_counter);
        if (ctx->ev0) cudaEventDestroy(ctx->ev0);
        if (ctx->ev1) cudaEventDestroy(ctx->ev1);
        if (ctx->stream) cudaStreamDestroy(ctx->stream);
        delete ctx;
    });
}

bd_status bd_context_kernel_launches(bd_context* ctx, int64_t* out) {
    return guard([&] {
        if (!ctx || !out) fail(BD_ERR_INVALID_ARG, "null argument");
        *out = ctx->launches;
    });
}

bd_status bd_unfold_quarter(const double* small, int32_t n_half, int32_t nz, double* full) {
    // T:280-302: full[iz][iy][ix] = small[iz][|iy - h|][|ix - h|]
    return guard([&] {
        if (!small || !full || n_half < 0 || nz <= 0) fail(BD_ERR_INVALID_ARG, "bad unfold arguments");
        const int64_t ns = (int64_t)n_half + 1, nf = 2 * (int64_t)n_half + 1;
        for (int64_t iz = 0; iz < nz; ++iz)
            for (int64_t iy = 0; iy < nf; ++iy) {
                const int64_t ys = iy < n_half ? n_half - iy : iy - n_half;
                for (int64_t ix = 0; ix < nf; ++ix) {
                    const int64_t xs = ix < n_half ? n_half - ix : ix - n_half;
                    full[(iz * nf + iy) * nf + ix] = small[(iz * ns + ys) * ns + xs];
                }
            }
    });
}

bd_status bd_gilmore_combo_tones(double A, const double f[3], const double* phi, bd_bubble* b) {
    // G:40-57: all equal -> single tone of amplitude A; f1 == f2 or f2 == f3 ->
    // tones f1 and f3 of amplitude A/sqrt(2); otherwise three tones of A/sqrt(3).
    return guard([&] {
        if (!f || !b) fail(BD_ERR_INVALID_ARG, "null argument");
        double R0 = b->R0;
        std::memset(b, 0, sizeof *b);
        b->R0 = R0;
        const double f1 = f[0], f2 = f[1], f3 = f[2];
        if (f1 == f2 && f1 == f3) {
            b->n_tones = 1; b->f[0] = f1; b->a[0] = A; b->phi[0] = phi ? phi[0] : 0.0;
        } else if (f1 == f2 || f2 == f3) {
            b->n_tones = 2; b->f[0] = f1; b->f[1] = f3;
            b->a[0] = b->a[1] = A / std::sqrt(2.0);
            b->phi[0] = phi ? phi[0] : 0.0; b->phi[1] = phi ? phi[2] : 0.0;
        } else {
            b->n_tones = 3;
            for (int k = 0; k < 3; ++k) { b->f[k] = f[k]; b->a[k] = A / std::sqrt(3.0); b->phi[k] = phi ? phi[k] : 0.0; }
        }
    });
}

bd_status bd_gilmore_combos(int32_t n_fr, double f_min, double f_max, double* out, int64_t cap,
                            int64_t* n_combo) {
    // G:498-520
    return guard([&] {
        if (n_fr < 2 || f_min <= 0 || f_max <= f_min || !n_combo) fail(BD_ERR_INVALID_ARG, "bad combo arguments");
        const double step_log = (std::log10(f_max) - std::log10(f_min)) / (n_fr - 1.0);
        int64_t k = 0;
        for (int i = 0; i < n_fr; i++) {
            bool first = true;
            for (int ii = i; ii < n_fr; ii++) {
                for (int iii = first ? ii : ii + 1; iii < n_fr; iii++) {
                    if (out && k < cap) {
                        out[3 * k] = std::pow(10.0, std::log10(f_min) + i * step_log);
                        out[3 * k + 1] = std::pow(10.0, std::log10(f_min) + ii * step_log);
                        out[3 * k + 2] = std::pow(10.0, std::log10(f_min) + iii * step_log);
                    }
                    k++;
                }
                first = false;
            }
        }
        *n_combo = k;
    });
}

}  // extern "C"
