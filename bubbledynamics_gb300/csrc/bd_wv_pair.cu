// Launches of the two-cells-per-thread Westervelt step (wv_tma_pair_kernel),
// kept in their own translation unit so they compile beside bd_westervelt.cu.
// FP32 fields with zero, one or two relaxation processes.
#include <algorithm>

#include "bd_internal.h"
#include "wv_tma_pair.h"
#include "wv_tma_pair.cuh"

namespace bd {

template <int TX, int TY, int NREL, int ZU, int FL, int NQ, int ACC>
static void pair_k(const PairCall& c) {
    using L = TmaLayout<float, TX, TY, (NREL >= 0 ? NREL : BD_MAX_RELAX), NQ>;
    auto kern = wv_tma_pair_kernel<float, TX, TY, NREL, ZU, FL, NQ, ACC>;
    static bool attr_done = false;
    static int per_sm = 0;
    if (!attr_done) {
        BD_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        BD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TX * TY / 2, L::SMEM));
        attr_done = true;
    }
    WvArgs<float> a = *c.a;
    const long long tiles = (long long)((a.nx + TX - 1) / TX) * ((a.ny + TY - 1) / TY);
    if (a.zb <= 0) a.zb = wave_fitted_zb(tiles, a.nz, (long long)c.ctx->sm_count * std::max(per_sm, 1));
    dim3 block(TX / 2, TY, 1);
    dim3 grid((a.nx + TX - 1) / TX, (a.ny + TY - 1) / TY, (a.nz + a.zb - 1) / a.zb);
    if (*c.pdl) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = grid;
        cfg.blockDim = block;
        cfg.dynamicSmemBytes = L::SMEM;
        cfg.stream = c.st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        const cudaError_t e = cudaLaunchKernelEx(&cfg, kern, a, c.K, c.koff, *c.maps, c.err);
        if (e == cudaSuccess) {
            BD_LAUNCHED(c.ctx);
            return;
        }
        (void)cudaGetLastError();
        *c.pdl = false;
    }
    kern<<<grid, block, L::SMEM, c.st>>>(a, c.K, c.koff, *c.maps, c.err);
    BD_LAUNCHED(c.ctx);
}

// material layout: 0 = no relaxation, 1 = one process, one material and a c
// map (compile-time), 2 = one process, 3 = two processes
template <int TX, int TY, int ZU, int NQ, int ACC>
static void pair_kind_acc(const PairCall& c) {
    switch (c.kind) {
        case 0: pair_k<TX, TY, 0, ZU, -1, NQ, ACC>(c); break;
        case 1: pair_k<TX, TY, 1, ZU, 3, NQ, ACC>(c); break;
        case 2: pair_k<TX, TY, 1, ZU, -1, NQ, ACC>(c); break;
        case 3: pair_k<TX, TY, 2, ZU, -1, NQ, ACC>(c); break;
        default: fail(BD_ERR_INVALID_ARG, "two-cell tile variants take at most two relaxation processes");
    }
}

// steps outside some accumulator windows take the kernel that skips those accumulators
template <int TX, int TY, int ZU, int NQ>
static void pair_kind(const PairCall& c) {
    switch (c.acc) {
        case ACC_NONE: pair_kind_acc<TX, TY, ZU, NQ, ACC_NONE>(c); break;
        case ACC_PEAK: pair_kind_acc<TX, TY, ZU, NQ, ACC_PEAK>(c); break;
        case ACC_PE: pair_kind_acc<TX, TY, ZU, NQ, ACC_PE>(c); break;
        default: pair_kind_acc<TX, TY, ZU, NQ, ACC_ALL>(c); break;
    }
}

void wv_pair_launch(const PairCall& c) {
    const int key = c.tx * 1000 + c.ty * 100 + c.zu * 10 + c.nq;   // tx <= 64, ty <= 16, zu and nq < 10
    switch (key) {
        case 32 * 1000 + 8 * 100 + 1 * 10 + 2: pair_kind<32, 8, 1, 2>(c); break;
        case 32 * 1000 + 8 * 100 + 2 * 10 + 2: pair_kind<32, 8, 2, 2>(c); break;
        case 64 * 1000 + 8 * 100 + 1 * 10 + 2: pair_kind<64, 8, 1, 2>(c); break;
        case 64 * 1000 + 8 * 100 + 2 * 10 + 2: pair_kind<64, 8, 2, 2>(c); break;
        case 32 * 1000 + 16 * 100 + 1 * 10 + 2: pair_kind<32, 16, 1, 2>(c); break;
        default: fail(BD_ERR_INVALID_ARG, "no two-cell kernel for tile %dx%d, %d planes per barrier, %d slots", c.tx,
                      c.ty, c.zu, c.nq);
    }
}

}  // namespace bd
