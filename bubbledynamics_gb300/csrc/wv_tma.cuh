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
// accumulator modes of the paired step kernel: all (peak, energy and the DFT),
// none, the peak map only, peak and energy without the DFT
constexpr int ACC_ALL = 0, ACC_NONE = 1, ACC_PEAK = 2, ACC_PE = 3;
constexpr int TMA_NQ = 3;   // pointwise slots

struct TmaMaps {
    CUtensorMap p0;                     // box (TX+8, TY+6, 1) on the p^n buffer
    CUtensorMap q[4];                   // box (TX, TY, 1) on p^{n-1..n-4}
    CUtensorMap rc[BD_MAX_RELAX];       // R^{n-1}
    CUtensorMap ro[BD_MAX_RELAX];       // R^{n-2}
    CUtensorMap cmap, peak, energy;
    CUtensorMap mat;                    // box (TX, TY, 1) on the per-cell material map (uint8), when staged
    CUtensorMap dre, dim;               // box (TX, TY, 1) on the DFT accumulators as (nx, ny, n_dft x planes)
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

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait: gives up after two seconds (mbar_wait_for: after limit_ns), records the timeout in *err
// (bit 4) and returns false so the kernel can finish instead of hanging.
// Once any wait has timed out, later waits return at once, so a broken
// pipeline ends the kernel quickly.
__device__ __forceinline__ bool mbar_wait_for(uint64_t* bar, unsigned parity, unsigned* err,
                                              unsigned long long limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    while (true) {
        if (mbar_try_wait(bar, parity)) return true;
        if (*reinterpret_cast<volatile unsigned*>(err) & 4u) return false;
        if (global_ns() - t0 > limit_ns) break;
    }
    atomicOr(err, 4u);
    return false;
}

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, unsigned* err) {
    return mbar_wait_for(bar, parity, err, 2000000000ull);
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

// Prefetch of one tile into L2 (no shared memory, no barrier): a hint for the
// loads that follow.
__device__ __forceinline__ void tma_prefetch_3d(const CUtensorMap* map, int x, int y, int z) {
    asm volatile("cp.async.bulk.prefetch.tensor.3d.L2.global.tile [%0, {%1, %2, %3}];"
                 ::"l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z)
                 : "memory");
}

// Shared-memory layout.  NRMAX is the number of relaxation processes the slot
// has room for (the compile-time count, or BD_MAX_RELAX for the generic kernel).
template <class real, int TX, int TY, int NRMAX, int NQ = TMA_NQ>
struct TmaLayout {
    static constexpr int PW = TX + 8, PH = TY + 6;
    static constexpr int PT = PW * PH;
    static constexpr int PSLOT = ((PT * (int)sizeof(real) + 127) / 128) * 128;   // bytes
    static constexpr int QT = TX * TY;
    static constexpr int QTB = QT * (int)sizeof(real);                            // bytes per real tile
    static constexpr int QTF = QT * 4;                                            // bytes of the float c tile
    static constexpr int QTM = ((QT + 127) / 128) * 128;                          // bytes of the uint8 material tile
    static constexpr int NQR = 4 + 2 * NRMAX + 2;                                 // real tiles per slot
    static constexpr int QS = NQR * QTB + QTF + QTM;                              // slot bytes
    static constexpr int K_PEAK = 4 + 2 * NRMAX, K_ENERGY = 5 + 2 * NRMAX;
    static constexpr int SMEM = TMA_NP * PSLOT + NQ * QS + (TMA_NP + NQ) * 8;
};

// One Westervelt step, TMA-pipelined.  Template parameters: tile TX x TY, CPT
// cells per thread along y (the CTA has TX x TY/CPT threads), NREL relaxation
// processes known at compile time (-1: read from the arguments, up to
// BD_MAX_RELAX), ZU planes per loop iteration (one CTA barrier and one round
// of TMA issues per ZU planes).  The cell update is cell_update(), so every variant gives the
// same bits as the plain kernel.
template <class real, int TX, int TY, int CPT, int NREL, int ZU, int FL = -1>
__global__ void __launch_bounds__(TX* TY / CPT) wv_tma_kernel(const WvArgs<real> a,
                                                              const WvConst<real>* __restrict__ Kp, int koff,
                                                              const __grid_constant__ TmaMaps maps,
                                                              unsigned* __restrict__ err) {
    constexpr int NRMAX = NREL >= 0 ? NREL : BD_MAX_RELAX;
    using L = TmaLayout<real, TX, TY, NRMAX>;
    constexpr int RPT = TY / CPT;                  // thread rows
    constexpr int NT = TX * RPT;                   // threads
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ MatConst<real> sK[BD_MAX_MATERIALS];
    const int nrel = NREL >= 0 ? NREL : a.max_relax;
    // FL >= 0: bit 0 = one material everywhere, bit 1 = per-cell c map (compile-time);
    // FL = -1: both read from the arguments
    const bool has_c = FL >= 0 ? (FL & 2) != 0 : a.cmap != nullptr;
    real* Pring = reinterpret_cast<real*>(smem);
    unsigned char* Qring = smem + TMA_NP * L::PSLOT;
    uint64_t* barP = reinterpret_cast<uint64_t*>(Qring + TMA_NQ * L::QS);
    uint64_t* barQ = barP + TMA_NP;

    const int tx = threadIdx.x, tyt = threadIdx.y;
    const int tid = tyt * TX + tx;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const int z0 = blockIdx.z * a.zb;
    const int z1 = min(a.nz, z0 + a.zb);
    const int zbn = z1 - z0;

    for (int e = tid; e < (int)(BD_MAX_MATERIALS * sizeof(MatConst<real>) / 4); e += NT)
        reinterpret_cast<unsigned*>(sK)[e] = reinterpret_cast<const unsigned*>(Kp)[e];

    auto pslot = [&](int q) {
        return reinterpret_cast<real*>(reinterpret_cast<unsigned char*>(Pring) + (q % TMA_NP) * L::PSLOT);
    };
    auto qslot = [&](int r) { return Qring + (r % TMA_NQ) * L::QS; };

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
        unsigned char* q = qslot(r);
        mbar_expect_tx(bar, (unsigned)((6 + 2 * nrel) * L::QTB + (has_c ? L::QTF : 0)));
        for (int k = 0; k < 4; ++k) tma_load_3d(q + k * L::QTB, &maps.q[k], bar, x0, y0, plane);
        for (int v = 0; v < nrel; ++v) {
            tma_load_3d(q + (4 + v) * L::QTB, &maps.rc[v], bar, x0, y0, plane);
            tma_load_3d(q + (4 + NRMAX + v) * L::QTB, &maps.ro[v], bar, x0, y0, plane);
        }
        tma_load_3d(q + L::K_PEAK * L::QTB, &maps.peak, bar, x0, y0, plane);
        tma_load_3d(q + L::K_ENERGY * L::QTB, &maps.energy, bar, x0, y0, plane);
        if (has_c) tma_load_3d(q + L::NQR * L::QTB, &maps.cmap, bar, x0, y0, plane);
    };

    if (tid == 0) {
        for (int s = 0; s < TMA_NP; ++s) mbar_init(&barP[s], 1);
        for (int s = 0; s < TMA_NQ; ++s) mbar_init(&barQ[s], 1);
        mbar_fence_init();
    }
    __syncthreads();
    // Programmatic dependent launch: with the attribute set by the host, the
    // prologue above (material constants, barrier set-up) overlaps the tail of
    // the previous step's grid; the fields and the step counter it wrote are
    // read only after this wait (a no-op for an ordinary launch).
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const long long step = *a.step_base + koff;
    if (tid == 0) {
        for (int q = 0; q < TMA_NP; ++q) issueP(q);
        for (int r = 0; r < TMA_NQ; ++r) issueQ(r);
    }
    auto waitP = [&](int q) { mbar_wait(&barP[q % TMA_NP], (unsigned)((q / TMA_NP) & 1), err); };
    auto waitQ = [&](int r) { mbar_wait(&barQ[r % TMA_NQ], (unsigned)((r / TMA_NQ) & 1), err); };

    // per-cell constants of this thread's CPT cells (rows tyt, tyt + RPT, ...)
    int own[CPT], qi[CPT];
    bool active[CPT], inbox[CPT], murxy[CPT];
    real swxy[CPT];
    int col[CPT];                                  // column index iy * nx + ix (a plane has < 2^31 cells)
#pragma unroll
    for (int c = 0; c < CPT; ++c) {
        const int ty = tyt + c * RPT;
        const int ix = x0 + tx, iy = y0 + ty;
        own[c] = (ty + 3) * L::PW + tx + 4;
        qi[c] = ty * TX + tx;
        active[c] = ix < a.nx && iy < a.ny;
        inbox[c] = ix <= a.xhi && iy <= a.yhi;
        murxy[c] = (a.mur_yp && iy >= a.ny - a.L) || (a.mur_xp && ix >= a.nx - a.L);
        swxy[c] = (a.wx && active[c]) ? mul_(a.wx[ix], a.wy[iy]) : real(1);
        col[c] = iy * a.nx + ix;
    }
    real w[CPT][7];
#pragma unroll
    for (int k = 0; k < 6; ++k) {                  // planes z0-3 .. z0+2
        waitP(k);
        const int plane = z0 - 3 + k;
        const bool in = plane >= 0 && plane < a.nz;
#pragma unroll
        for (int c = 0; c < CPT; ++c) w[c][k] = in ? pslot(k)[own[c]] : real(0);
    }
    __syncthreads();                               // slots of planes z0-3..z0-1 are free again
    if (tid == 0)
        for (int q = TMA_NP; q < TMA_NP + 3; ++q) issueP(q);

    const bool fix_x = a.mir_x && x0 == 0, fix_y = a.mir_y && y0 == 0;
    const bool do_peak = step >= a.peak_start && step < a.peak_end;
    const bool do_energy = step >= a.energy_start && step < a.energy_end;
    const long long ds = step - a.dft_start;
    const bool do_dft = a.n_dft > 0 && ds >= 0 && ds < a.dft_len;
    const bool single_mat = FL >= 0 ? (FL & 1) != 0 : (!a.matmap && !a.plane_mat);
    const bool dpdt = a.energy_mode == BD_ENERGY_DPDT2;
    // the material of single-material problems, in registers
    const MatConst<real> M0 = sK[0];

    for (int izg = z0; izg < z1; izg += ZU) {
        // the last planes of this CTA: the next step's grid may start its prologue
        if (izg + ZU >= z1) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#pragma unroll
    for (int u = 0; u < ZU; ++u) {
        const int iz = izg + u;
        if (iz >= z1) break;
        const int qc = iz - z0 + 3;                // stencil plane
        const int r = iz - z0;
        waitP(qc + 3);
        {
            const bool in = iz + 3 < a.nz;
            const real* T6 = pslot(qc + 3);
#pragma unroll
            for (int c = 0; c < CPT; ++c) w[c][6] = in ? T6[own[c]] : real(0);
        }
        real* T = pslot(qc);
        if (fix_x || fix_y) {                      // mirror planes x = 0 / y = 0 (W:176-200)
            if (fix_x)
                for (int e = tid; e < L::PH * 3; e += NT) {
                    const int row = e / 3, k = e % 3 + 1;
                    T[row * L::PW + 4 - k] = T[row * L::PW + 4 + k];
                }
            __syncthreads();
            if (fix_y)
                for (int e = tid; e < L::PW * 3; e += NT) {
                    const int cc = e % L::PW, k = e / L::PW + 1;
                    T[(3 - k) * L::PW + cc] = T[(3 + k) * L::PW + cc];
                }
            // TMA refills this slot later: order these ordinary stores before that copy
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncthreads();
        }
        waitQ(r);
        const unsigned char* Qs = qslot(r);
        const real* q1t = reinterpret_cast<const real*>(Qs);
        const real* q2t = q1t + L::QT;
        const real* q3t = q2t + L::QT;
        const real* q4t = q3t + L::QT;
        const real* pkt = reinterpret_cast<const real*>(Qs + L::K_PEAK * L::QTB);
        const real* ent = reinterpret_cast<const real*>(Qs + L::K_ENERGY * L::QTB);
        const float* ct = reinterpret_cast<const float*>(Qs + L::NQR * L::QTB);
        const bool src_plane = iz == a.src_iz;
        const bool zin = iz >= a.zlo && iz <= a.zhi && !src_plane;
        const bool murz = (a.mur_zp && iz >= a.nz - a.L) || (a.mur_zm && iz < a.Lzm);
        const real wzi = a.wz ? a.wz[iz] : real(1);
        const int mplane = single_mat ? 0 : (a.plane_mat ? __ldg(a.plane_mat + iz) : 0);
        const long long zoff = (long long)iz * a.plane;
        real* const p4z = a.p4 + zoff;
        real* const pkz = a.peak + zoff;
        real* const enz = a.energy + zoff;
        real* rolz[NRMAX > 0 ? NRMAX : 1];
#pragma unroll
        for (int v = 0; v < NRMAX; ++v) rolz[v] = a.rold[v] + zoff;
#pragma unroll
        for (int c = 0; c < CPT; ++c) {
            if (!active[c]) continue;
            const long long i = zoff + col[c];
            const int k = qi[c];
            const real q1 = q1t[k];
            real pn;
            bool have = false;
            if (src_plane) {
                pn = source_value<real>(a, step, (int)col[c]);
                have = true;
            } else if (zin && inbox[c]) {
                const real* c0 = T + own[c];
                const real pc = w[c][3];
                const real sx1 = c0[1] + c0[-1], sx2 = c0[2] + c0[-2], sx3 = c0[3] + c0[-3];
                constexpr int W = L::PW;
                const real sy1 = c0[W] + c0[-W], sy2 = c0[2 * W] + c0[-2 * W], sy3 = c0[3 * W] + c0[-3 * W];
                auto upd = [&](const MatConst<real>& M) -> real {
                    const real cs = has_c ? (real)ct[k] : M.c0;
                    real rc[NRMAX > 0 ? NRMAX : 1], ro[NRMAX > 0 ? NRMAX : 1];
#pragma unroll
                    for (int v = 0; v < NRMAX; ++v) {
                        if (v < M.n_relax) {
                            rc[v] = reinterpret_cast<const real*>(Qs + (4 + v) * L::QTB)[k];
                            ro[v] = reinterpret_cast<const real*>(Qs + (4 + NRMAX + v) * L::QTB)[k];
                        }
                    }
                    const real r = cell_update<real, NRMAX>(a, M, cs, pc, sx1, sx2, sx3, sy1, sy2, sy3, w[c], q1, q2t[k],
                                                            q3t[k], q4t[k], rc, ro);
#pragma unroll
                    for (int v = 0; v < NRMAX; ++v)
                        if (v < M.n_relax) rolz[v][col[c]] = ro[v];
                    return r;
                };
                if constexpr (FL >= 0 && (FL & 1)) {
                    pn = upd(M0);
                } else {
                    const int m = a.matmap ? (int)__ldg(a.matmap + i) : mplane;
                    pn = upd(sK[m]);
                }
                if (a.wz) pn = mul_(pn, mul_(swxy[c], wzi));
                have = true;
            }
            if (have) {
                p4z[col[c]] = pn;
                if (!(murz || murxy[c])) {
                    if (do_peak) {
                        const real av = fabs(pn), pk = pkt[k];
                        pkz[col[c]] = av > pk ? av : pk;
                    }
                    if (do_energy) {
                        real e;
                        if (dpdt) {
                            const real dp = div_(add_(pn, -q1), mul_(real(2.0), a.dt));
                            e = mul_(mul_(dp, dp), a.dt);
                        } else {
                            e = mul_(mul_(pn, pn), a.dt);
                        }
                        enz[col[c]] = add_(ent[k], e);
                    }
                    if (do_dft && iz >= a.dz_lo && iz < a.dz_hi) {
                        const long long pl = (long long)(iz - a.dz_lo) * a.plane + col[c];
                        const long long stride = (long long)(a.dz_hi - a.dz_lo) * a.plane;
                        const real* tw = a.tw + ds * a.n_dft * 2;
                        real* dr = a.dre + pl;
                        real* di = a.dim + pl;
                        int j = 0;
                        // four frequencies at a time: their eight loads are issued before any store
                        for (; j + 4 <= a.n_dft; j += 4) {
                            real r[4], m[4];
#pragma unroll
                            for (int u = 0; u < 4; ++u) { r[u] = dr[(j + u) * stride]; m[u] = di[(j + u) * stride]; }
#pragma unroll
                            for (int u = 0; u < 4; ++u) {
                                dr[(j + u) * stride] = fma_(pn, tw[2 * (j + u)], r[u]);
                                di[(j + u) * stride] = fma_(-pn, tw[2 * (j + u) + 1], m[u]);
                            }
                        }
                        for (; j < a.n_dft; ++j) {
                            dr[j * stride] = fma_(pn, tw[2 * j], dr[j * stride]);
                            di[j * stride] = fma_(-pn, tw[2 * j + 1], di[j * stride]);
                        }
                    }
                }
            }
        }
#pragma unroll
        for (int c = 0; c < CPT; ++c)
#pragma unroll
            for (int k = 0; k < 6; ++k) w[c][k] = w[c][k + 1];
    }
        __syncthreads();                           // everyone is done with planes izg..izg+ZU-1 and their tiles
        if (tid == 0) {
#pragma unroll
            for (int u = 0; u < ZU; ++u) {
                issueP(izg + u - z0 + 3 + TMA_NP);
                issueQ(izg + u - z0 + TMA_NQ);
            }
        }
    }
}

}  // namespace bd
