// Device side of the Westervelt solver: one fused kernel per time step plus
// the Mur boundary passes, all templated on the storage/arithmetic type.
//
// Reference: W:139-236 (interior update), W:62-85 (source plane), W:88-135
// (Mur), W:242-265 (water power), W:268-345 (harmonic power via FFT; here an
// on-the-fly DFT), W:575-584 (time-level rotation; here a pointer ring).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/bubbledyn.h"

namespace bd {

#define BD_PI 3.14159265358979323846


// Per-material constants in a form that needs no division per cell, in the
// arithmetic type of the kernel.
template <class real>
struct MatConst {
    real c0;
    real delta_2dt;            // delta / (2 dt)            -> kd = delta_2dt / c^2   (W:216)
    real beta2_rho;            // 2 beta / rho              -> kn = beta2_rho / c^2   (W:217)
    real ra_num[BD_MAX_RELAX]; // 2dt*2*c_v*tau_v / (2dt^3 (2dt+3tau_v)) -> ra = ra_num / c^3 (W:226-227)
    real rb[BD_MAX_RELAX];     // tau_v / (2dt + 3 tau_v)                 (W:227)
    int n_relax;
    int pad;
};

template <class real>
struct WvConst {
    MatConst<real> mat[BD_MAX_MATERIALS];
};

template <class real>
struct WvArgs {
    int nx, ny, nz;
    int zb;                    // z-chunk per CTA
    long long plane;           // nx*ny
    // time levels: p^n (stencil), p^{n-1..n-3}, and the p^{n-4} buffer that receives p^{n+1}
    const real* __restrict__ p0;
    const real* __restrict__ p1;
    const real* __restrict__ p2;
    const real* __restrict__ p3;
    real* __restrict__ p4;
    // relaxation: R^{n-1} and the R^{n-2} buffer that receives R^n, per process
    const real* __restrict__ rcur[BD_MAX_RELAX];
    real* __restrict__ rold[BD_MAX_RELAX];
    int max_relax;
    // medium
    const float* __restrict__ cmap;
    const uint8_t* __restrict__ matmap;
    const int* __restrict__ plane_mat;
    // geometry of the update
    int xhi, yhi, zlo, zhi;    // box of the stencil update (inclusive)
    int src_iz;                // source plane or -1
    int mir_x, mir_y;
    int mur_xp, mur_yp, mur_zp, mur_zm, L, Lzm;
    const real* __restrict__ wx;    // sponge factors per axis (nullptr = none)
    const real* __restrict__ wy;
    const real* __restrict__ wz;
    real dt, kxy180, kz180, dt2;   // dt, dt^2/(180 dx^2), dt^2/(180 dz^2), dt^2
    real dtdx, dtdz;               // dt/dx, dt/dz (Mur)
    // source (W:62-85)
    const double* __restrict__ sA;      // p0*amp_e / var (FP32 path) or p0*amp_e (FP64 path)
    const double* __restrict__ sVar;    // var (FP64 path)
    const double* __restrict__ sTau;    // geometric delay
    const float* __restrict__ sAf;      // FP32 path amplitude p0*amp_e/var
    const float* __restrict__ sPsi;     // FP32 path per-tone phase offset [n_tones][plane]
    const float* __restrict__ sTauf;    // FP32 path delay (burst window)
    const double* __restrict__ sPhi;    // element phase (FP64 path)
    int n_tones;
    int burst;
    double freq[BD_MAX_TONES], tamp[BD_MAX_TONES], tphase[BD_MAX_TONES];
    float tampf[BD_MAX_TONES];
    double tau_max, burst_len;
    float burst_lenf;
    // step tables
    const long long* __restrict__ step_base;   // device step counter of the chunk start
    const double* __restrict__ t_src;          // per-step source time
    const float* __restrict__ theta;           // FP32 path: per step per tone 2 pi frac(f (t - shift))
    const float* __restrict__ tb0;             // FP32 path: per step t - tau_max
    // accumulators
    real* __restrict__ peak;
    real* __restrict__ energy;
    real* __restrict__ dre;
    real* __restrict__ dim;
    const real* __restrict__ tw;               // DFT twiddles [dft step][n_dft][2]
    long long peak_start, peak_end, energy_start, energy_end, dft_start, dft_len;
    int energy_mode, n_dft, dz_lo, dz_hi;
    int relax_scheme;
    int mat_tile;              // 1: the two-cell kernel receives the material map as a TMA tile per plane
};

// Explicitly rounded arithmetic: the compiler never re-contracts these, so
// every kernel variant that calls cell_update() produces the same bits.
__device__ __forceinline__ float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float mul_(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_(double a, double b) { return __dadd_rn(a, b); }
// FP32 divisions use the fast hardware path (max 2 ulp), FP64 ones are IEEE.
__device__ __forceinline__ float div_(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double div_(double a, double b) { return __ddiv_rn(a, b); }

template <class real>
__device__ __forceinline__ real ld(const real* p) { return __ldg(p); }

template <class real>
__device__ __forceinline__ real source_value(const WvArgs<real>& a, long long step, int j);

template <>
__device__ __forceinline__ double source_value<double>(const WvArgs<double>& a, long long step, int j) {
    // FP64 path: the arithmetic of W:78-82 (plus tones / bursts / elements).
    const double A = a.sA[j];
    if (A == 0.0) return 0.0;
    double tt = a.t_src[step] + a.sTau[j];
    if (a.burst) {
        const double tb = tt - a.tau_max;
        if (tb < 0.0 || tb >= a.burst_len) return 0.0;
        tt = tb;
    }
    double sum = 0.0;
    for (int k = 0; k < a.n_tones; ++k) sum += a.tamp[k] * sin(2 * BD_PI * a.freq[k] * tt + a.tphase[k] + a.sPhi[j]);
    return A * sum / a.sVar[j];
}

template <>
__device__ __forceinline__ float source_value<float>(const WvArgs<float>& a, long long step, int j) {
    // FP32 path: phases reduced on the host to [0, 2 pi) per step and per cell.
    const float A = a.sAf[j];
    if (A == 0.0f) return 0.0f;
    if (a.burst) {
        const float tb = a.tb0[step] + a.sTauf[j];
        if (tb < 0.0f || tb >= a.burst_lenf) return 0.0f;
    }
    float sum = 0.0f;
    for (int k = 0; k < a.n_tones; ++k)
        sum = fma_(a.tampf[k], sinf(add_(a.theta[step * BD_MAX_TONES + k], a.sPsi[(long long)k * a.plane + j])), sum);
    return mul_(A, sum);
}

template <class real>
__device__ __forceinline__ bool is_mur_cell(const WvArgs<real>& a, int ix, int iy, int iz) {
    return (a.mur_yp && iy >= a.ny - a.L) || (a.mur_xp && ix >= a.nx - a.L) ||
           (a.mur_zp && iz >= a.nz - a.L) || (a.mur_zm && iz < a.Lzm);
}

// Energy accumulator update: E + p^2 dt, or E + ((p^{n+1}-p^{n-1})/2dt)^2 dt (W:253-257).
template <class real>
__device__ __forceinline__ real energy_add(const WvArgs<real>& a, real old, real v, real vm1) {
    real e;
    if (a.energy_mode == BD_ENERGY_DPDT2) {
        const real dp = div_(add_(v, -vm1), mul_(real(2.0), a.dt));     // W:253
        e = mul_(mul_(dp, dp), a.dt);                                    // W:257
    } else {
        e = mul_(mul_(v, v), a.dt);
    }
    return add_(old, e);
}

// Peak / energy / DFT accumulation on the final p^{n+1} of a cell.
template <class real>
__device__ __forceinline__ void accumulate(const WvArgs<real>& a, long long step, long long i, int ix, int iy,
                                           int iz, real v, real vm1) {
    if (step >= a.peak_start && step < a.peak_end) {
        const real av = fabs(v);
        const real pk = a.peak[i];
        a.peak[i] = av > pk ? av : pk;
    }
    if (step >= a.energy_start && step < a.energy_end) a.energy[i] = energy_add(a, a.energy[i], v, vm1);
    const long long ds = step - a.dft_start;
    if (a.n_dft > 0 && ds >= 0 && ds < a.dft_len && iz >= a.dz_lo && iz < a.dz_hi) {
        const long long pl = (long long)(iz - a.dz_lo) * a.plane + (long long)iy * a.nx + ix;
        const long long stride = (long long)(a.dz_hi - a.dz_lo) * a.plane;
        const real* tw = a.tw + ds * a.n_dft * 2;
        for (int j = 0; j < a.n_dft; ++j) {
            a.dre[j * stride + pl] = fma_(v, tw[2 * j], a.dre[j * stride + pl]);
            a.dim[j * stride + pl] = fma_(-v, tw[2 * j + 1], a.dim[j * stride + pl]);
        }
    }
}

template <class real>
__device__ __forceinline__ real cell_c(const WvArgs<real>& a, const WvConst<real>& K, long long i, int m) {
    return a.cmap ? (real)__ldg(a.cmap + i) : K.mat[m].c0;
}

template <class real>
__device__ __forceinline__ int cell_mat(const WvArgs<real>& a, long long i, int iz) {
    if (a.matmap) return __ldg(a.matmap + i);
    if (a.plane_mat) return __ldg(a.plane_mat + iz);
    return 0;
}

// 6th-order second difference times 180 (W:203-205): -490 p + 270 s1 - 27 s2 + 2 s3
template <class real>
__device__ __forceinline__ real d2x180(real pc, real s1, real s2, real s3) {
    return fma_(real(2), s3, fma_(real(-27), s2, fma_(real(270), s1, mul_(real(-490), pc))));
}

// The update of one cell (W:203-234, or the semi-implicit relaxation coupling).
// sx1..sy3: sums of the +-1, +-2, +-3 neighbours along x / y; w[0..6]: p^n at
// iz-3..iz+3; q1..q4: p^{n-1..n-4}; rc / ro: R^{n-1} / R^{n-2} per process, ro
// returns R^n.  Returns p^{n+1} before the sponge factor.
template <class real, int NRMAX = BD_MAX_RELAX>
__device__ __forceinline__ real cell_update(const WvArgs<real>& a, const MatConst<real>& M, real c, real pc, real sx1,
                                            real sx2, real sx3, real sy1, real sy2, real sy3, const real* w, real q1,
                                            real q2, real q3, real q4, const real* rc, real* ro) {
    const real Dxx = d2x180(pc, sx1, sx2, sx3);
    const real Dyy = d2x180(pc, sy1, sy2, sy3);
    const real Dzz = d2x180(pc, add_(w[4], w[2]), add_(w[5], w[1]), add_(w[6], w[0]));
    // W:207: 5 p - 18 p1 + 24 p2 - 14 p3 + 3 p4
    const real Dttt = fma_(real(3), q4, fma_(real(-14), q3, fma_(real(24), q2, fma_(real(-18), q1, mul_(real(5), pc)))));
    const real s3 = fma_(real(3), pc, fma_(real(-4), q1, q2));
    const real D1 = mul_(mul_(s3, s3), real(0.25));                                                   // W:208
    const real D2 = mul_(pc, fma_(real(2), pc, fma_(real(-5), q1, fma_(real(4), q2, -q3))));          // W:209
    const real c2 = mul_(c, c);
    const real ic = div_(real(1), c);
    const real ic2 = mul_(ic, ic);
    const real kxy = mul_(c2, a.kxy180);
    const real kz = mul_(c2, a.kz180);
    const real kd = mul_(M.delta_2dt, ic2);
    const real kn = mul_(M.beta2_rho, ic2);
    // W:234 without the relaxation term, as an increment on p^n: Y = p + V with
    // V = (p - p1) + kxy (Dxx + Dyy) + kz Dzz + kd Dttt + kn (D1 + D2).  The terms are
    // summed at the size of the increment (about a quarter of p per step at 8
    // cells per wavelength) and p^{n+1} takes one final rounding: the FP32 field
    // error against FP64 after 3000 cfg1 steps drops from 1.04e-5 to 8.4e-6
    // (summing 2p - p1 + ... directly rounds at the size of p five times).
    real V = add_(pc, -q1);
    V = fma_(kxy, add_(Dxx, Dyy), V);
    V = fma_(kz, Dzz, V);
    V = fma_(kd, Dttt, V);
    V = fma_(kn, add_(D1, D2), V);
    real pn;
    if (M.n_relax > 0 && a.relax_scheme == BD_RELAX_SEMI_IMPLICIT) {
        // R_v = a_v (3 p^{n+1} + E) + b_v (4 R1 - R2) with the 2nd-order d3p/dt3 at t_n
        // through p^{n+1}..p^{n-3}; p^{n+1} = Y + (c dt)^2 sum_v R_v solved per cell
        const real E = fma_(real(-10), pc, fma_(real(12), q1, fma_(real(-6), q2, q3)));
        const real kr = mul_(c2, a.dt2);
        const real ic3 = mul_(ic2, ic);
        real sa = real(0), G = real(0);
        real av[NRMAX > 0 ? NRMAX : 1], bv[NRMAX > 0 ? NRMAX : 1];
#pragma unroll
        for (int v = 0; v < NRMAX; ++v) {
            if (v < M.n_relax) {
                av[v] = mul_(M.ra_num[v], ic3);
                bv[v] = mul_(M.rb[v], fma_(real(4), rc[v], -ro[v]));
                sa = add_(sa, av[v]);
                G = add_(G, fma_(av[v], E, bv[v]));
            }
        }
        // p = num / (1 - x) with x = 3 kr sum a small: written as num + num x / (1 - x) so
        // the (possibly approximate) division only touches the small correction
        const real x = mul_(mul_(real(3), kr), sa);
        const real Vn = fma_(kr, G, V);                          // num = p + Vn
        pn = add_(pc, fma_(add_(pc, Vn), div_(x, add_(real(1), -x)), Vn));
#pragma unroll
        for (int v = 0; v < NRMAX; ++v)
            if (v < M.n_relax) ro[v] = fma_(av[v], fma_(real(3), pn, E), bv[v]);
    } else {
        real sumR = real(0);
#pragma unroll
        for (int v = 0; v < NRMAX; ++v) {
            if (v < M.n_relax) {
                // W:227: R = 2dt 2 c_v tau Dttt/(2dt^3) / ((2dt+3tau) c^3) + tau (4 R1 - R2)/(2dt+3tau)
                const real rn = fma_(mul_(mul_(M.ra_num[v], ic2), ic), Dttt,
                                     mul_(M.rb[v], fma_(real(4), rc[v], -ro[v])));
                ro[v] = rn;
                sumR = add_(sumR, rn);
            }
        }
        pn = add_(pc, fma_(sumR, mul_(c2, a.dt2), V));                                       // W:234
    }
    return pn;
}

// One time step of the stencil update.  CTA = TX x TY columns; each thread
// marches along z over a chunk of a.zb planes keeping p^n(iz-3..iz+3) of its
// column in registers.  x/y neighbours come through the read-only cache.
template <class real, int TX, int TY>
__global__ void __launch_bounds__(TX* TY) wv_step_kernel(const WvArgs<real> a, const WvConst<real>* __restrict__ Kp,
                                                           int koff) {
    const int ix = blockIdx.x * TX + threadIdx.x;
    const int iy = blockIdx.y * TY + threadIdx.y;
    if (ix >= a.nx || iy >= a.ny) return;
    const WvConst<real>& K = *Kp;
    const long long step = *a.step_base + koff;
    const int z0 = blockIdx.z * a.zb;
    const int z1 = min(a.nz, z0 + a.zb);
    const int nx = a.nx;
    // neighbour offsets and weights along x and y (mirror at index 0, zero ghosts outside)
    int xo[6], yo[6];
    real xw[6], yw[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const int o = k < 3 ? k - 3 : k - 2;   // -3,-2,-1,1,2,3
        int jx = ix + o;
        real wxk = real(1);
        if (jx < 0) { if (a.mir_x) jx = -jx; else { jx = ix; wxk = real(0); } }
        if (jx >= nx) { jx = ix; wxk = real(0); }
        xo[k] = jx - ix; xw[k] = wxk;
        int jy = iy + o;
        real wyk = real(1);
        if (jy < 0) { if (a.mir_y) jy = -jy; else { jy = iy; wyk = real(0); } }
        if (jy >= a.ny) { jy = iy; wyk = real(0); }
        yo[k] = (jy - iy) * nx; yw[k] = wyk;
    }
    const bool col_in_box = ix <= a.xhi && iy <= a.yhi;
    const real sw_xy = a.wx ? mul_(a.wx[ix], a.wy[iy]) : real(1);
    const long long col = (long long)iy * nx + ix;
    // z window of p^n
    real w[7];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const int z = z0 - 3 + k;
        w[k] = (z >= 0 && z < a.nz) ? ld(a.p0 + (long long)z * a.plane + col) : real(0);
    }
    for (int iz = z0; iz < z1; ++iz) {
        {
            const int z = iz + 3;
            w[6] = (z < a.nz) ? ld(a.p0 + (long long)z * a.plane + col) : real(0);
        }
        const long long i = (long long)iz * a.plane + col;
        const bool mur = is_mur_cell(a, ix, iy, iz);
        real pn;
        bool have = false;
        if (iz == a.src_iz) {
            pn = source_value<real>(a, step, (int)col);
            have = true;
        } else if (col_in_box && iz >= a.zlo && iz <= a.zhi) {
            const real pc = w[3];
            const real* P = a.p0 + i;
            const real sx1 = xw[3] * ld(P + xo[3]) + xw[2] * ld(P + xo[2]);
            const real sx2 = xw[4] * ld(P + xo[4]) + xw[1] * ld(P + xo[1]);
            const real sx3 = xw[5] * ld(P + xo[5]) + xw[0] * ld(P + xo[0]);
            const real sy1 = yw[3] * ld(P + yo[3]) + yw[2] * ld(P + yo[2]);
            const real sy2 = yw[4] * ld(P + yo[4]) + yw[1] * ld(P + yo[1]);
            const real sy3 = yw[5] * ld(P + yo[5]) + yw[0] * ld(P + yo[0]);
            const real q1 = ld(a.p1 + i), q2 = ld(a.p2 + i), q3 = ld(a.p3 + i), q4 = a.p4[i];
            const int m = cell_mat(a, i, iz);
            const real c = cell_c(a, K, i, m);
            real rc[BD_MAX_RELAX], ro[BD_MAX_RELAX];
            for (int v = 0; v < K.mat[m].n_relax; ++v) { rc[v] = ld(a.rcur[v] + i); ro[v] = a.rold[v][i]; }
            pn = cell_update(a, K.mat[m], c, pc, sx1, sx2, sx3, sy1, sy2, sy3, w, q1, q2, q3, q4, rc, ro);
            for (int v = 0; v < K.mat[m].n_relax; ++v) a.rold[v][i] = ro[v];
            if (a.wz) pn = mul_(pn, mul_(sw_xy, a.wz[iz]));
            have = true;
        }
        if (have) {
            const real vm1 = (a.energy_mode == BD_ENERGY_DPDT2) ? ld(a.p1 + i) : real(0);
            a.p4[i] = pn;
            if (!mur) accumulate(a, step, i, ix, iy, iz, pn, vm1);
        }
#pragma unroll
        for (int k = 0; k < 6; ++k) w[k] = w[k + 1];
    }
}

template <class real>
__device__ __forceinline__ real mur_k(real c, real dth) {
    const real a = c * dth;
    return (a - real(1)) / (a + real(1));
}

// Mur on the z faces (W:101-113) for columns outside the x+/y+ layers.
template <class real>
__global__ void wv_mur_z_kernel(const WvArgs<real> a, const WvConst<real>* __restrict__ Kp, int koff) {
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    const int iy = blockIdx.y * blockDim.y + threadIdx.y;
    if (ix >= a.nx || iy >= a.ny) return;
    if ((a.mur_xp && ix >= a.nx - a.L) || (a.mur_yp && iy >= a.ny - a.L)) return;
    const WvConst<real>& K = *Kp;
    const long long step = *a.step_base + koff;
    const long long col = (long long)iy * a.nx + ix;
    const real* Pn = a.p0;
    real* F = a.p4;
    if (a.mur_zm) {
        for (int iz = 0; iz < a.Lzm; ++iz) {
            const long long i = (long long)iz * a.plane + col, j = i + a.plane;
            const real nb = (iz + 1 < a.Lzm) ? Pn[j] : F[j];   // pre-boundary value of P_next is p^n in W
            const real c = cell_c(a, K, i, cell_mat(a, i, iz));
            const real v = Pn[j] + (nb - Pn[i]) * mur_k(c, a.dtdz);
            F[i] = v;
            accumulate(a, step, i, ix, iy, iz, v, a.energy_mode == BD_ENERGY_DPDT2 ? a.p1[i] : real(0));
        }
    }
    if (a.mur_zp) {
        for (int iz = a.nz - a.L; iz < a.nz; ++iz) {
            const long long i = (long long)iz * a.plane + col, j = i - a.plane;
            const real c = cell_c(a, K, i, cell_mat(a, i, iz));
            const real v = Pn[j] + (F[j] - Pn[i]) * mur_k(c, a.dtdz);
            F[i] = v;
            accumulate(a, step, i, ix, iy, iz, v, a.energy_mode == BD_ENERGY_DPDT2 ? a.p1[i] : real(0));
        }
    }
}

// Mur on the x+ face (W:122-126), rows outside the y+ layers, inner layer first.
template <class real>
__global__ void wv_mur_x_kernel(const WvArgs<real> a, const WvConst<real>* __restrict__ Kp, int koff) {
    const int iy = blockIdx.x * blockDim.x + threadIdx.x;
    const int iz = blockIdx.y;
    if (iy >= a.ny || (a.mur_yp && iy >= a.ny - a.L)) return;
    const WvConst<real>& K = *Kp;
    const long long step = *a.step_base + koff;
    const real* Pn = a.p0;
    real* F = a.p4;
    for (int ix = a.nx - a.L; ix < a.nx; ++ix) {
        const long long i = (long long)iz * a.plane + (long long)iy * a.nx + ix, j = i - 1;
        const real c = cell_c(a, K, i, cell_mat(a, i, iz));
        const real v = Pn[j] + (F[j] - Pn[i]) * mur_k(c, a.dtdx);
        F[i] = v;
        accumulate(a, step, i, ix, iy, iz, v, a.energy_mode == BD_ENERGY_DPDT2 ? a.p1[i] : real(0));
    }
}

// Mur on the y+ face (W:129-133), all columns, inner layer first.
template <class real>
__global__ void wv_mur_y_kernel(const WvArgs<real> a, const WvConst<real>* __restrict__ Kp, int koff) {
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    const int iz = blockIdx.y;
    if (ix >= a.nx) return;
    const WvConst<real>& K = *Kp;
    const long long step = *a.step_base + koff;
    const real* Pn = a.p0;
    real* F = a.p4;
    for (int iy = a.ny - a.L; iy < a.ny; ++iy) {
        const long long i = (long long)iz * a.plane + (long long)iy * a.nx + ix, j = i - a.nx;
        const real c = cell_c(a, K, i, cell_mat(a, i, iz));
        const real v = Pn[j] + (F[j] - Pn[i]) * mur_k(c, a.dtdx);
        F[i] = v;
        accumulate(a, step, i, ix, iy, iz, v, a.energy_mode == BD_ENERGY_DPDT2 ? a.p1[i] : real(0));
    }
}

static __global__ void wv_advance_kernel(long long* step_base, int n) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *step_base += n;
}

// NaN / Inf / amplitude probe of a field: flag bit 1 = non-finite, bit 2 = above limit.
template <class real>
__global__ void wv_probe_kernel(const real* __restrict__ p, long long n, double limit, unsigned* flag) {
    unsigned f = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const real v = p[i];
        if (!isfinite(v)) f |= 1u;
        else if (limit > 0 && fabs((double)v) > limit) f |= 2u;
    }
    f = __reduce_or_sync(0xffffffffu, f);
    if (f && (threadIdx.x & 31) == 0) atomicOr(flag, f);
}

}  // namespace bd
