// Host-side call of the two-cells-per-thread Westervelt step (bd_wv_pair.cu).
#pragma once

#include "wv_tma.cuh"

namespace bd {

struct PairCall {
    bd_context* ctx;
    const WvArgs<float>* a;            // zb <= 0: fitted to whole waves
    const WvConst<float>* K;
    int koff;
    const TmaMaps* maps;
    unsigned* err;
    bool* pdl;                          // programmatic dependent launch (cleared if unavailable)
    cudaStream_t st;
    int tx, ty, zu, nq;                 // tile, planes per barrier, pointwise ring slots
    int kind;                           // 0: no relaxation, 1: one process + one material + c map, 2: one, 3: two
    int acc;                            // accumulators the step may touch (ACC_*): 0 all, 1 none, 2 the peak
                                        // map only, 3 peak and energy
};

void wv_pair_launch(const PairCall& c);

}  // namespace bd
