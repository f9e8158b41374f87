// TMA-pipelined Westervelt step for sm_103a.
//
// A CTA owns a TX x TY block of columns and marches through a z-chunk.  One
// elected thread streams, with cp.async.bulk.tensor, every z plane the CTA needs
// into shared memory ahead of use:
//   - the p^n plane tile with its stencil halo ((TX+8) x (TY+6); x starts 4 cells
//     left of the block so the TMA x coordinate stays 16-byte aligned; cells
//     outside the grid arrive as zeros, the OPEN-face ghost value), in a ring of
//     NP slots kept up to NP-4 planes ahead of the stencil;
//   - the pointwise tiles of that plane (p^{n-1..n-4}, R^{n-1}, R^{n-2}, c, peak,
//     energy), in a ring of NQ slots.
// Each slot has an mbarrier (expect-tx by the producer, completed by the TMA
// transaction bytes).  Every thread keeps p^n(iz-3..iz+3) of its own column in
// registers for the z stencil and reads x/y neighbours from the plane tile.
// The per-cell physics is cell_update() shared with the plain kernel, so both
// kernels give identical results.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include "wv_kernels.cuh"

namespace bd {

constexpr int TMA_NP = 8;   // p^n plane slots (>= 7)
constexpr int TMA_NQ = 3;   // pointwise slots

struct TmaMaps {
    CUtensorMap p0;                     // box (TX+8, TY+6, 1) on the p^n buffer
    CUtensorMap q[4];                   // box (TX, TY, 1) on p^{n-1..n-4}
    CUtensorMap rc[BD_MAX_RELAX];       // R^{n-1}
    CUtensorMap ro[BD_MAX_RELAX];       // R^{n-2}
    CUtensorMap cmap, peak, energy;
};

__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: gives up after a fixed number of polls, records the timeout in
// *err (bit 4) and returns false so the kernel can finish instead of hanging.
// Once any wait has timed out, later waits return at once, so a broken
// pipeline ends the kernel quickly.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, unsigned* err) {
    for (int i = 0; i < (1 << 22); ++i) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((i & 1023) == 1023 && (*reinterpret_cast<volatile unsigned*>(err) & 4u)) return false;
    }
    atomicOr(err, 4u);
    return false;
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

template <class real, int TX, int TY>
struct TmaLayout {
    static constexpr int PW = TX + 8, PH = TY + 6;
    static constexpr int PT = PW * PH;
    static constexpr int PSLOT = ((PT * (int)sizeof(real) + 127) / 128) * 128;   // bytes
    static constexpr int QT = TX * TY;
    static constexpr int QTB = QT * (int)sizeof(real);                            // bytes per real tile
    static constexpr int QTF = QT * 4;                                            // bytes of the float c tile
    __host__ __device__ static int qslot(int nrel, bool has_c) { return (4 + 2 * nrel + 2) * QTB + (has_c ? QTF : 0); }
    __host__ __device__ static int smem(int nrel, bool has_c) { return TMA_NP * PSLOT + TMA_NQ * qslot(nrel, has_c) + (TMA_NP + TMA_NQ) * 8; }
};

template <class real, int TX, int TY>
__global__ void __launch_bounds__(TX* TY) wv_tma_kernel(const WvArgs<real> a, const WvConst<real>* __restrict__ Kp,
                                                        int koff, const __grid_constant__ TmaMaps maps,
                                                        unsigned* __restrict__ err) {
    using L = TmaLayout<real, TX, TY>;
    extern __shared__ __align__(128) unsigned char smem[];
    const int nrel = a.max_relax;
    const bool has_c = a.cmap != nullptr;
    const int QS = L::qslot(nrel, has_c);
    real* Pring = reinterpret_cast<real*>(smem);
    unsigned char* Qring = smem + TMA_NP * L::PSLOT;
    uint64_t* barP = reinterpret_cast<uint64_t*>(Qring + TMA_NQ * QS);
    uint64_t* barQ = barP + TMA_NP;

    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * TX + tx;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const int ix = x0 + tx, iy = y0 + ty;
    const bool active = ix < a.nx && iy < a.ny;
    const int z0 = blockIdx.z * a.zb;
    const int z1 = min(a.nz, z0 + a.zb);
    const int zbn = z1 - z0;
    const long long step = *a.step_base + koff;
    const WvConst<real>& K = *Kp;

    auto pslot = [&](int q) { return reinterpret_cast<real*>(reinterpret_cast<unsigned char*>(Pring) + (q % TMA_NP) * L::PSLOT); };
    auto qtile = [&](int r, int k) { return reinterpret_cast<real*>(Qring + (r % TMA_NQ) * QS + k * L::QTB); };
    auto ctile = [&](int r) { return reinterpret_cast<float*>(Qring + (r % TMA_NQ) * QS + (4 + 2 * nrel + 2) * L::QTB); };

    // producer (thread 0): plane q = plane - (z0 - 3) of p^n, plane r = plane - z0 of the pointwise tiles
    auto issueP = [&](int q) {
        if (q > zbn + 5) return;
        const int plane = z0 - 3 + q;
        uint64_t* bar = &barP[q % TMA_NP];
        if (plane < 0 || plane >= a.nz) { mbar_arrive(bar); return; }   // read as zeros, nothing to copy
        mbar_expect_tx(bar, L::PW * L::PH * (unsigned)sizeof(real));
        tma_load_3d(pslot(q), &maps.p0, bar, x0 - 4, y0 - 3, plane);
    };
    auto issueQ = [&](int r) {
        if (r >= zbn) return;
        const int plane = z0 + r;
        uint64_t* bar = &barQ[r % TMA_NQ];
        mbar_expect_tx(bar, (unsigned)QS);
        for (int k = 0; k < 4; ++k) tma_load_3d(qtile(r, k), &maps.q[k], bar, x0, y0, plane);
        for (int v = 0; v < nrel; ++v) {
            tma_load_3d(qtile(r, 4 + v), &maps.rc[v], bar, x0, y0, plane);
            tma_load_3d(qtile(r, 4 + nrel + v), &maps.ro[v], bar, x0, y0, plane);
        }
        tma_load_3d(qtile(r, 4 + 2 * nrel), &maps.peak, bar, x0, y0, plane);
        tma_load_3d(qtile(r, 5 + 2 * nrel), &maps.energy, bar, x0, y0, plane);
        if (has_c) tma_load_3d(ctile(r), &maps.cmap, bar, x0, y0, plane);
    };

    if (tid == 0) {
        for (int s = 0; s < TMA_NP; ++s) mbar_init(&barP[s], 1);
        for (int s = 0; s < TMA_NQ; ++s) mbar_init(&barQ[s], 1);
        mbar_fence_init();
    }
    __syncthreads();
    if (tid == 0) {
        for (int q = 0; q < TMA_NP; ++q) issueP(q);
        for (int r = 0; r < TMA_NQ; ++r) issueQ(r);
    }
    auto waitP = [&](int q) { mbar_wait(&barP[q % TMA_NP], (unsigned)((q / TMA_NP) & 1), err); };
    auto waitQ = [&](int r) { mbar_wait(&barQ[r % TMA_NQ], (unsigned)((r / TMA_NQ) & 1), err); };

    const int own = (ty + 3) * L::PW + tx + 4;     // this column inside a plane tile
    real w[7];
    for (int k = 0; k < 6; ++k) {                  // planes z0-3 .. z0+2
        waitP(k);
        const int plane = z0 - 3 + k;
        w[k] = (plane >= 0 && plane < a.nz) ? pslot(k)[own] : real(0);
    }
    __syncthreads();                               // slots of planes z0-3..z0-1 are free again
    if (tid == 0)
        for (int q = TMA_NP; q < TMA_NP + 3; ++q) issueP(q);

    const bool col_in_box = ix <= a.xhi && iy <= a.yhi;
    const real sw_xy = (a.wx && active) ? a.wx[ix] * a.wy[iy] : real(1);
    const long long col = (long long)iy * a.nx + ix;
    const bool fix_x = a.mir_x && x0 == 0, fix_y = a.mir_y && y0 == 0;

    for (int iz = z0; iz < z1; ++iz) {
        const int qc = iz - z0 + 3;                // stencil plane
        const int r = iz - z0;
        waitP(qc + 3);
        w[6] = (iz + 3 < a.nz) ? pslot(qc + 3)[own] : real(0);
        real* T = pslot(qc);
        if (fix_x || fix_y) {                      // mirror planes x = 0 / y = 0 (W:176-200)
            if (fix_x)
                for (int e = tid; e < L::PH * 3; e += TX * TY) {
                    const int row = e / 3, k = e % 3 + 1;
                    T[row * L::PW + 4 - k] = T[row * L::PW + 4 + k];
                }
            __syncthreads();
            if (fix_y)
                for (int e = tid; e < L::PW * 3; e += TX * TY) {
                    const int c = e % L::PW, k = e / L::PW + 1;
                    T[(3 - k) * L::PW + c] = T[(3 + k) * L::PW + c];
                }
            __syncthreads();
        }
        waitQ(r);
        if (active) {
            const long long i = (long long)iz * a.plane + col;
            const int qi = ty * TX + tx;
            const real q1 = qtile(r, 0)[qi];
            const bool mur = is_mur_cell(a, ix, iy, iz);
            real pn;
            bool have = false;
            real ro[BD_MAX_RELAX];
            int m = 0;
            if (iz == a.src_iz) {
                pn = source_value<real>(a, step, (int)col);
                have = true;
            } else if (col_in_box && iz >= a.zlo && iz <= a.zhi) {
                const real* c0 = T + own;
                const real pc = w[3];
                const real sx1 = c0[1] + c0[-1], sx2 = c0[2] + c0[-2], sx3 = c0[3] + c0[-3];
                const int W = L::PW;
                const real sy1 = c0[W] + c0[-W], sy2 = c0[2 * W] + c0[-2 * W], sy3 = c0[3 * W] + c0[-3 * W];
                m = cell_mat(a, i, iz);
                const real c = has_c ? (real)ctile(r)[qi] : K.mat[m].c0;
                real rc[BD_MAX_RELAX];
                for (int v = 0; v < K.mat[m].n_relax; ++v) { rc[v] = qtile(r, 4 + v)[qi]; ro[v] = qtile(r, 4 + nrel + v)[qi]; }
                pn = cell_update(a, K.mat[m], c, pc, sx1, sx2, sx3, sy1, sy2, sy3, w, q1, qtile(r, 1)[qi],
                                 qtile(r, 2)[qi], qtile(r, 3)[qi], rc, ro);
                for (int v = 0; v < K.mat[m].n_relax; ++v) a.rold[v][i] = ro[v];
                if (a.wz) pn *= sw_xy * a.wz[iz];
                have = true;
            }
            if (have) {
                a.p4[i] = pn;
                if (!mur) {
                    if (step >= a.peak_start && step < a.peak_end) {
                        const real av = fabs(pn), pk = qtile(r, 4 + 2 * nrel)[qi];
                        a.peak[i] = av > pk ? av : pk;
                    }
                    if (step >= a.energy_start && step < a.energy_end) {
                        real e;
                        if (a.energy_mode == BD_ENERGY_DPDT2) {
                            const real dp = (pn - q1) / (real(2.0) * a.dt);
                            e = dp * dp * a.dt;
                        } else {
                            e = pn * pn * a.dt;
                        }
                        a.energy[i] = qtile(r, 5 + 2 * nrel)[qi] + e;
                    }
                    const long long ds = step - a.dft_start;
                    if (a.n_dft > 0 && ds >= 0 && ds < a.dft_len && iz >= a.dz_lo && iz < a.dz_hi) {
                        const long long pl = (long long)(iz - a.dz_lo) * a.plane + col;
                        const long long stride = (long long)(a.dz_hi - a.dz_lo) * a.plane;
                        const real* tw = a.tw + ds * a.n_dft * 2;
                        for (int j = 0; j < a.n_dft; ++j) {
                            a.dre[j * stride + pl] += pn * tw[2 * j];
                            a.dim[j * stride + pl] -= pn * tw[2 * j + 1];
                        }
                    }
                }
            }
        }
        __syncthreads();                           // everyone is done with plane iz and its tiles
        if (tid == 0) {
            issueP(qc + TMA_NP);
            issueQ(r + TMA_NQ);
        }
#pragma unroll
        for (int k = 0; k < 6; ++k) w[k] = w[k + 1];
    }
}

}  // namespace bd
