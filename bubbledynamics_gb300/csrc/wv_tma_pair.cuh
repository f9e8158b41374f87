// Two-cells-per-thread variant of the TMA-pipelined Westervelt step (sm_103a).
#pragma once

#include <type_traits>

#include "wv_tma.cuh"

namespace bd {

// CX consecutive values along x (CX = 1 or 2): one 8- or 16-byte access for a
// pair, whose first element sits at an even index of a buffer aligned to the
// pair's size.
template <class real> struct Pair;
template <> struct Pair<float> { using T = float2; };
template <> struct Pair<double> { using T = double2; };

template <int CX, class real>
__device__ __forceinline__ void ldx(const real* p, real* out) {
    if constexpr (CX == 2) {
        const typename Pair<real>::T v = *reinterpret_cast<const typename Pair<real>::T*>(p);
        out[0] = v.x;
        out[1] = v.y;
    } else {
        out[0] = *p;
    }
}

template <class real>
__device__ __forceinline__ void st2(real* p, real v0, real v1) {
    typename Pair<real>::T v;
    v.x = v0;
    v.y = v1;
    *reinterpret_cast<typename Pair<real>::T*>(p) = v;
}

// One Westervelt step, TMA-pipelined, two adjacent x cells per thread: the
// same pipeline as wv_tma_kernel (p^n plane ring with halo, pointwise ring,
// bounded mbarrier waits), with every tile and global access of a thread one
// 8- or 16-byte pair (nx must be even, which a 16-byte row pitch gives) and a
// pointwise ring of NQ slots (NQ >= ZU), so that a shallower ring leaves room
// for more CTAs per SM.  The CTA has TX/2 x TY threads; the launch bound asks
// for 24 resident warps per SM (at most 85 registers a thread).  The cell update is
// cell_update(), so the results are the plain kernel's bits.
//
// ACC: which accumulators the step may touch.  ACC_ALL: peak, energy and DFT
// (each still gated by its window); ACC_PE: peak and energy (a step outside the
// DFT window: no DFT code, so fewer registers); ACC_PEAK: only the peak map (a
// step outside the energy and DFT windows: the energy tile is not loaded, 4 B
// less per cell); ACC_NONE: none (outside every window, e.g. the recompute of
// the adjoint: neither tile is loaded, 8 B less per cell).  Planes on which
// every cell of the tile is updated take a copy of the cell code without the
// per-cell conditions, except in ACC_ALL, where the larger DFT code of that
// copy would cost registers (and spills) in the whole kernel.
template <class real, int TX, int TY, int NREL, int ZU, int FL, int NQ, int ACC = ACC_ALL>
__global__ void __launch_bounds__(TX* TY / 2, 1536 / (TX * TY)) wv_tma_pair_kernel(const WvArgs<real> a,
                                                                 const WvConst<real>* __restrict__ Kp, int koff,
                                                                 const __grid_constant__ TmaMaps maps,
                                                                 unsigned* __restrict__ err) {
    constexpr int CX = 2, CPT = 1;
    static_assert(NQ >= ZU, "the pointwise ring holds a whole group of planes");
    constexpr int NRMAX = NREL >= 0 ? NREL : BD_MAX_RELAX;
    using L = TmaLayout<real, TX, TY, NRMAX, NQ>;
    constexpr int TXT = TX / CX;                   // thread columns
    constexpr int RPT = TY / CPT;                  // thread rows
    constexpr int NT = TXT * RPT;                  // threads
    constexpr int NC = CPT * CX;                   // cells per thread
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ MatConst<real> sK[BD_MAX_MATERIALS];
    const int nrel = NREL >= 0 ? NREL : a.max_relax;
    // FL >= 0: bit 0 = one material everywhere, bit 1 = per-cell c map (compile-time);
    // FL = -1: both read from the arguments
    const bool has_c = FL >= 0 ? (FL & 2) != 0 : a.cmap != nullptr;
    real* Pring = reinterpret_cast<real*>(smem);
    unsigned char* Qring = smem + TMA_NP * L::PSLOT;
    uint64_t* barP = reinterpret_cast<uint64_t*>(Qring + NQ * L::QS);
    uint64_t* barQ = barP + TMA_NP;

    const int tx = threadIdx.x, tyt = threadIdx.y;
    const int tid = tyt * TXT + tx;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const int z0 = blockIdx.z * a.zb;
    const int z1 = min(a.nz, z0 + a.zb);
    const int zbn = z1 - z0;

    for (int e = tid; e < (int)(BD_MAX_MATERIALS * sizeof(MatConst<real>) / 4); e += NT)
        reinterpret_cast<unsigned*>(sK)[e] = reinterpret_cast<const unsigned*>(Kp)[e];

    auto pslot = [&](int q) {
        return reinterpret_cast<real*>(reinterpret_cast<unsigned char*>(Pring) + (q % TMA_NP) * L::PSLOT);
    };
    auto qslot = [&](int r) { return Qring + (r % NQ) * L::QS; };

    // producer (thread 0): plane q = plane - (z0 - 3) of p^n, plane r = plane - z0 of the pointwise tiles
    auto issueP = [&](int q) {
        if (q > zbn + 5) return;
        const int plane = z0 - 3 + q;
        uint64_t* bar = &barP[q % TMA_NP];
        if (plane < 0 || plane >= a.nz) { mbar_arrive(bar); return; }   // read as zeros, nothing to copy
        mbar_expect_tx(bar, L::PW * L::PH * (unsigned)sizeof(real));
        tma_load_3d(pslot(q), &maps.p0, bar, x0 - 4, y0 - 3, plane);
    };
    // steps inside the DFT window: the producer also asks L2 for the plane's
    // accumulator tiles when it issues the plane's pointwise tiles, so the
    // accumulators' read-modify-writes find them there (set once the step is known)
    bool pf_dft = false;
    auto issueQ = [&](int r) {
        if (r >= zbn) return;
        const int plane = z0 + r;
        if (pf_dft && plane >= a.dz_lo && plane < a.dz_hi) {
            const int ndz = a.dz_hi - a.dz_lo;
            for (int j = 0; j < a.n_dft; ++j) {
                tma_prefetch_3d(&maps.dre, x0, y0, j * ndz + plane - a.dz_lo);
                tma_prefetch_3d(&maps.dim, x0, y0, j * ndz + plane - a.dz_lo);
            }
        }
        uint64_t* bar = &barQ[r % NQ];
        unsigned char* q = qslot(r);
        constexpr int acc_tiles = ACC == ACC_ALL || ACC == ACC_PE ? 2 : ACC == ACC_PEAK ? 1 : 0;
        mbar_expect_tx(bar, (unsigned)((4 + acc_tiles + 2 * nrel) * L::QTB + (has_c ? L::QTF : 0) +
                                       (a.mat_tile ? L::QT : 0)));
        for (int k = 0; k < 4; ++k) tma_load_3d(q + k * L::QTB, &maps.q[k], bar, x0, y0, plane);
        for (int v = 0; v < nrel; ++v) {
            tma_load_3d(q + (4 + v) * L::QTB, &maps.rc[v], bar, x0, y0, plane);
            tma_load_3d(q + (4 + NRMAX + v) * L::QTB, &maps.ro[v], bar, x0, y0, plane);
        }
        if constexpr (ACC != ACC_NONE) tma_load_3d(q + L::K_PEAK * L::QTB, &maps.peak, bar, x0, y0, plane);
        if constexpr (ACC == ACC_ALL || ACC == ACC_PE)
            tma_load_3d(q + L::K_ENERGY * L::QTB, &maps.energy, bar, x0, y0, plane);
        if (has_c) tma_load_3d(q + L::NQR * L::QTB, &maps.cmap, bar, x0, y0, plane);
        if (a.mat_tile) tma_load_3d(q + L::NQR * L::QTB + L::QTF, &maps.mat, bar, x0, y0, plane);
    };

    if (tid == 0) {
        for (int s = 0; s < TMA_NP; ++s) mbar_init(&barP[s], 1);
        for (int s = 0; s < NQ; ++s) mbar_init(&barQ[s], 1);
        mbar_fence_init();
    }
    __syncthreads();
    // Programmatic dependent launch: with the attribute set by the host, the
    // prologue above (material constants, barrier set-up) overlaps the tail of
    // the previous step's grid; the fields and the step counter it wrote are
    // read only after this wait (a no-op for an ordinary launch).
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const long long step = *a.step_base + koff;
    if constexpr (ACC == ACC_ALL && sizeof(real) == 4)
        pf_dft = a.n_dft > 0 && step >= a.dft_start && step < a.dft_start + a.dft_len;
    if (tid == 0) {
        for (int q = 0; q < TMA_NP; ++q) issueP(q);
        for (int r = 0; r < NQ; ++r) issueQ(r);
    }
    auto waitP = [&](int q) { mbar_wait(&barP[q % TMA_NP], (unsigned)((q / TMA_NP) & 1), err); };
    auto waitQ = [&](int r) { mbar_wait(&barQ[r % NQ], (unsigned)((r / NQ) & 1), err); };

    // per-cell constants of this thread's cells: c = cy * CX + cx is the cell in
    // row tyt + cy * RPT and column CX * tx + cx of the tile
    int own[NC], qi[NC];
    bool active[NC], inbox[NC], murxy[NC];
    real swxy[NC];
    int col[NC];                                   // column index iy * nx + ix (a plane has < 2^31 cells)
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        const int ty = tyt + (c / CX) * RPT;
        const int lx = CX * tx + c % CX;
        const int ix = x0 + lx, iy = y0 + ty;
        own[c] = (ty + 3) * L::PW + lx + 4;
        qi[c] = ty * TX + lx;
        active[c] = ix < a.nx && iy < a.ny;
        inbox[c] = ix <= a.xhi && iy <= a.yhi;
        murxy[c] = (a.mur_yp && iy >= a.ny - a.L) || (a.mur_xp && ix >= a.nx - a.L);
        swxy[c] = (a.wx && active[c]) ? mul_(a.wx[ix], a.wy[iy]) : real(1);
        col[c] = iy * a.nx + ix;
    }
    real w[NC][7];
    // p^n of this thread's cells on one plane tile into w[.][k]
    auto load_w = [&](const real* tile, bool in, int k) {
#pragma unroll
        for (int cy = 0; cy < CPT; ++cy) {
            real v[CX];
            ldx<CX>(tile + own[cy * CX], v);
#pragma unroll
            for (int cx = 0; cx < CX; ++cx) w[cy * CX + cx][k] = in ? v[cx] : real(0);
        }
    };
#pragma unroll
    for (int k = 0; k < 6; ++k) {                  // planes z0-3 .. z0+2
        waitP(k);
        const int plane = z0 - 3 + k;
        load_w(pslot(k), plane >= 0 && plane < a.nz, k);
    }
    // every cell of the tile inside the grid and the update box and on no x / y
    // Mur layer: the planes of the tile inside the z range take the code without
    // per-cell conditions (the same operations on every cell, so the same bits)
    bool tile_fast = false;
    if constexpr (ACC != ACC_ALL) {
        bool mine = true;
#pragma unroll
        for (int c = 0; c < NC; ++c) mine = mine && active[c] && inbox[c] && !murxy[c];
        tile_fast = __syncthreads_and(mine) != 0;      // also: slots of planes z0-3..z0-1 are free again
    } else {
        __syncthreads();                               // slots of planes z0-3..z0-1 are free again
    }
    if (tid == 0)
        for (int q = TMA_NP; q < TMA_NP + 3; ++q) issueP(q);

    const bool fix_x = a.mir_x && x0 == 0, fix_y = a.mir_y && y0 == 0;
    const bool do_peak = ACC != ACC_NONE && step >= a.peak_start && step < a.peak_end;
    const bool do_energy = (ACC == ACC_ALL || ACC == ACC_PE) && step >= a.energy_start && step < a.energy_end;
    const long long ds = step - a.dft_start;
    const bool do_dft = ACC == ACC_ALL && a.n_dft > 0 && ds >= 0 && ds < a.dft_len;
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
        load_w(pslot(qc + 3), iz + 3 < a.nz, 6);
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
        const uint8_t* mtl = reinterpret_cast<const uint8_t*>(Qs + L::NQR * L::QTB + L::QTF);
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
        // FAST: every cell of the tile is updated and accumulates on this plane
        auto cells = [&](auto fast_tag) {
        constexpr bool FAST = decltype(fast_tag)::value;
#pragma unroll
        for (int cy = 0; cy < CPT; ++cy) {
            const int c0 = cy * CX;                // first cell of this row (the CX cells share `active`)
            if (!FAST && !active[c0]) continue;
            const int k = qi[c0];
            real q1[CX], pn[CX];
            bool have[CX];
            int nrx[CX];                           // relaxation processes of the cell's material
            real ro[CX][NRMAX > 0 ? NRMAX : 1];
            ldx<CX>(q1t + k, q1);
#pragma unroll
            for (int cx = 0; cx < CX; ++cx) { have[cx] = false; nrx[cx] = 0; }
            if (!FAST && src_plane) {
#pragma unroll
                for (int cx = 0; cx < CX; ++cx) {
                    pn[cx] = source_value<real>(a, step, (int)col[c0 + cx]);
                    have[cx] = true;
                }
            } else if (FAST || zin) {
                // x and y neighbours of the CX cells from the plane tile
                const real* cp = T + own[c0];
                constexpr int W = L::PW;
                real sx1[CX], sx2[CX], sx3[CX], sy1[CX], sy2[CX], sy3[CX];
                if constexpr (CX == 2) {
                    real xr[10];                   // x offsets -4 .. +5 from the first cell
#pragma unroll
                    for (int j = 0; j < 5; ++j) ldx<2>(cp - 4 + 2 * j, xr + 2 * j);
#pragma unroll
                    for (int cx = 0; cx < 2; ++cx) {
                        sx1[cx] = xr[5 + cx] + xr[3 + cx];
                        sx2[cx] = xr[6 + cx] + xr[2 + cx];
                        sx3[cx] = xr[7 + cx] + xr[1 + cx];
                    }
                    real ya[6][2];
#pragma unroll
                    for (int j = 0; j < 3; ++j) {
                        ldx<2>(cp + (j + 1) * W, ya[2 * j]);
                        ldx<2>(cp - (j + 1) * W, ya[2 * j + 1]);
                    }
#pragma unroll
                    for (int cx = 0; cx < 2; ++cx) {
                        sy1[cx] = ya[0][cx] + ya[1][cx];
                        sy2[cx] = ya[2][cx] + ya[3][cx];
                        sy3[cx] = ya[4][cx] + ya[5][cx];
                    }
                } else {
                    sx1[0] = cp[1] + cp[-1]; sx2[0] = cp[2] + cp[-2]; sx3[0] = cp[3] + cp[-3];
                    sy1[0] = cp[W] + cp[-W]; sy2[0] = cp[2 * W] + cp[-2 * W]; sy3[0] = cp[3 * W] + cp[-3 * W];
                }
                real q2[CX], q3[CX], q4[CX], cs[CX];
                ldx<CX>(q2t + k, q2);
                ldx<CX>(q3t + k, q3);
                ldx<CX>(q4t + k, q4);
                if (has_c) {
                    float cf[CX];
                    ldx<CX>(ct + k, cf);
#pragma unroll
                    for (int cx = 0; cx < CX; ++cx) cs[cx] = (real)cf[cx];
                }
                real rc[CX][NRMAX > 0 ? NRMAX : 1];
#pragma unroll
                for (int v = 0; v < NRMAX; ++v) {
                    if (v < nrel) {
                        real t[CX], u[CX];
                        ldx<CX>(reinterpret_cast<const real*>(Qs + (4 + v) * L::QTB) + k, t);
                        ldx<CX>(reinterpret_cast<const real*>(Qs + (4 + NRMAX + v) * L::QTB) + k, u);
#pragma unroll
                        for (int cx = 0; cx < CX; ++cx) { rc[cx][v] = t[cx]; ro[cx][v] = u[cx]; }
                    }
                }
#pragma unroll
                for (int cx = 0; cx < CX; ++cx) {
                    const int c = c0 + cx;
                    if (!FAST && !inbox[c]) continue;
                    auto upd = [&](const MatConst<real>& M) -> real {
                        const real r = cell_update<real, NRMAX>(a, M, has_c ? cs[cx] : M.c0, w[c][3], sx1[cx], sx2[cx],
                                                                sx3[cx], sy1[cx], sy2[cx], sy3[cx], w[c], q1[cx],
                                                                q2[cx], q3[cx], q4[cx], rc[cx], ro[cx]);
                        nrx[cx] = M.n_relax;
                        return r;
                    };
                    if constexpr (FL >= 0 && (FL & 1)) {
                        pn[cx] = upd(M0);
                    } else {
                        const int m = !a.matmap ? mplane
                                      : a.mat_tile ? (int)mtl[k + cx] : (int)__ldg(a.matmap + zoff + col[c]);
                        pn[cx] = upd(sK[m]);
                    }
                    if (a.wz) pn[cx] = mul_(pn[cx], mul_(swxy[c], wzi));
                    have[cx] = true;
                }
            }
            // stores: a pair access where both cells take part, else per cell
            const bool pair = CX == 2 && (FAST || (have[0] && have[CX - 1]));
            if (pair) st2(p4z + col[c0], pn[0], pn[CX - 1]);
            else
#pragma unroll
                for (int cx = 0; cx < CX; ++cx)
                    if (have[cx]) p4z[col[c0 + cx]] = pn[cx];
            // relaxation variables of the processes of each cell's material (as in cell_update)
#pragma unroll
            for (int v = 0; v < NRMAX; ++v) {
                if (CX == 2 && v < nrx[0] && v < nrx[CX - 1]) st2(rolz[v] + col[c0], ro[0][v], ro[CX - 1][v]);
                else
#pragma unroll
                    for (int cx = 0; cx < CX; ++cx)
                        if (v < nrx[cx]) rolz[v][col[c0 + cx]] = ro[cx][v];
            }
            bool acc[CX];
#pragma unroll
            for (int cx = 0; cx < CX; ++cx) acc[cx] = FAST || (have[cx] && !(murz || murxy[c0 + cx]));
            const bool acc_pair = CX == 2 && acc[0] && acc[CX - 1];
            if (do_peak) {
                real pk[CX], pv[CX];
                ldx<CX>(pkt + k, pk);
#pragma unroll
                for (int cx = 0; cx < CX; ++cx) {
                    const real av = fabs(pn[cx]);
                    pv[cx] = av > pk[cx] ? av : pk[cx];
                }
                if (acc_pair) st2(pkz + col[c0], pv[0], pv[CX - 1]);
                else
#pragma unroll
                    for (int cx = 0; cx < CX; ++cx)
                        if (acc[cx]) pkz[col[c0 + cx]] = pv[cx];
            }
            if (do_energy) {
                real en[CX], ev[CX];
                ldx<CX>(ent + k, en);
#pragma unroll
                for (int cx = 0; cx < CX; ++cx) {
                    real e;
                    if (dpdt) {
                        const real dp = div_(add_(pn[cx], -q1[cx]), mul_(real(2.0), a.dt));
                        e = mul_(mul_(dp, dp), a.dt);
                    } else {
                        e = mul_(mul_(pn[cx], pn[cx]), a.dt);
                    }
                    ev[cx] = add_(en[cx], e);
                }
                if (acc_pair) st2(enz + col[c0], ev[0], ev[CX - 1]);
                else
#pragma unroll
                    for (int cx = 0; cx < CX; ++cx)
                        if (acc[cx]) enz[col[c0 + cx]] = ev[cx];
            }
            if (do_dft && iz >= a.dz_lo && iz < a.dz_hi && acc_pair) {
                // both cells accumulate: one pair load and store per accumulator
                using P2 = typename Pair<real>::T;
                const long long pl = (long long)(iz - a.dz_lo) * a.plane + col[c0];
                const long long stride = (long long)(a.dz_hi - a.dz_lo) * a.plane;
                const real* tw = a.tw + ds * a.n_dft * 2;
                real* dr = a.dre + pl;
                real* di = a.dim + pl;
                int j = 0;
                for (; j + 4 <= a.n_dft; j += 4) {
                    P2 r[4], m[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        r[u] = *reinterpret_cast<const P2*>(dr + (j + u) * stride);
                        m[u] = *reinterpret_cast<const P2*>(di + (j + u) * stride);
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const real tr = tw[2 * (j + u)], ti = tw[2 * (j + u) + 1];
                        st2(dr + (j + u) * stride, fma_(pn[0], tr, r[u].x), fma_(pn[1], tr, r[u].y));
                        st2(di + (j + u) * stride, fma_(-pn[0], ti, m[u].x), fma_(-pn[1], ti, m[u].y));
                    }
                }
                for (; j < a.n_dft; ++j) {
                    const P2 r = *reinterpret_cast<const P2*>(dr + j * stride);
                    const P2 m = *reinterpret_cast<const P2*>(di + j * stride);
                    st2(dr + j * stride, fma_(pn[0], tw[2 * j], r.x), fma_(pn[1], tw[2 * j], r.y));
                    st2(di + j * stride, fma_(-pn[0], tw[2 * j + 1], m.x), fma_(-pn[1], tw[2 * j + 1], m.y));
                }
            } else if (do_dft && iz >= a.dz_lo && iz < a.dz_hi) {
#pragma unroll
                for (int cx = 0; cx < CX; ++cx) {
                    if (!acc[cx]) continue;
                    const real pv = pn[cx];
                    const long long pl = (long long)(iz - a.dz_lo) * a.plane + col[c0 + cx];
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
                            dr[(j + u) * stride] = fma_(pv, tw[2 * (j + u)], r[u]);
                            di[(j + u) * stride] = fma_(-pv, tw[2 * (j + u) + 1], m[u]);
                        }
                    }
                    for (; j < a.n_dft; ++j) {
                        dr[j * stride] = fma_(pv, tw[2 * j], dr[j * stride]);
                        di[j * stride] = fma_(-pv, tw[2 * j + 1], di[j * stride]);
                    }
                }
            }
        }
        };
        if constexpr (ACC != ACC_ALL) {
            if (tile_fast && zin && !murz) cells(std::true_type{});
            else cells(std::false_type{});
        } else {
            cells(std::false_type{});
        }
#pragma unroll
        for (int c = 0; c < NC; ++c)
#pragma unroll
            for (int k = 0; k < 6; ++k) w[c][k] = w[c][k + 1];
    }
        __syncthreads();                           // everyone is done with planes izg..izg+ZU-1 and their tiles
        if (tid == 0) {
#pragma unroll
            for (int u = 0; u < ZU; ++u) {
                issueP(izg + u - z0 + 3 + TMA_NP);
                issueQ(izg + u - z0 + NQ);
            }
        }
    }
}

}  // namespace bd
