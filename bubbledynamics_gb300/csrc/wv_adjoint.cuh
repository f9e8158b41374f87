// Discrete adjoint of the Westervelt step (wv_kernels.cuh: cell_update and the
// source plane), for OPEN faces.  Forward step s maps the state
//   (p^s, p^{s-1}, p^{s-2}, p^{s-3}, p^{s-4}, R^{s-1}, R^{s-2})
// to (p^{s+1}, p^s, p^{s-1}, p^{s-2}, p^{s-3}, R^s, R^{s-1}).  Given the
// adjoints mu_0..mu_4, muR1, muR2 of the output state, one backward step gives
// the adjoints lambda of the input state:
//   lambda_k = mu_{k+1} + (d p^{s+1} / d p^{s-k})^T mu_0 + (d R^s / d p^{s-k})^T muR1
// The loss is sum_x w_L(x) sum_{s in window} p^{s+1}(x)^2 dt.
#pragma once

#include "wv_kernels.cuh"

namespace bd {

template <class real>
struct AdjArgs {
    int nx, ny, nz;
    long long plane;
    // adjoint ring of the output state: mu[k] = adjoint of p^{s+1-k}; lambda_k is written over mu[k+1]
    // (k = 0..3) and lambda_4 over mu[0], so the roles rotate by one per step
    real* mu[5];
    real* muR1[BD_MAX_RELAX];   // adjoint of R^s      (receives lambda of R^{s-2})
    real* muR2[BD_MAX_RELAX];   // adjoint of R^{s-1}  (receives lambda of R^{s-1})
    int max_relax;
    // forward fields: fp[0] = p^{s+1}, fp[1] = p^s, fp[2] = p^{s-1}, fp[3] = p^{s-2}, fp[4] = p^{s-3}
    const real* fp[5];
    real* H;                    // c^2 * (adjoint of Y), read with the stencil
    const float* cmap;
    const uint8_t* matmap;
    const int* plane_mat;
    const real* wx;
    const real* wy;
    const real* wz;
    real kxy180, kz180, dt2, dt;
    int relax_scheme;
    int src_iz;
    // source-plane gradients (per plane cell, FP64) and the pieces of S_j(t)
    double* gphi;
    double* gamp;
    const float* sAf;           // FP32: A_j a_e / var_j
    const float* sPsi;          // FP32: per-tone phase offsets
    const float* sTauf;
    const float* theta;         // FP32: per-step tone phases
    const float* tb0;
    const double* sA;           // FP64: A_j a_e
    const double* sVar;
    const double* sTau;
    const double* sPhi;
    const double* t_src;
    const double* e_amp;        // per plane cell: a_e of its element (1 for bowls)
    int n_tones, burst;
    double freq[BD_MAX_TONES], tamp[BD_MAX_TONES], tphase[BD_MAX_TONES];
    float tampf[BD_MAX_TONES];
    double tau_max, burst_len;
    float burst_lenf;
    // loss
    int fx, fy, fz, frad2, srad2;
    double side_w;
    int in_window;              // step s contributes p^{s+1} to the loss
    long long step;             // forward step index s
};

template <class real>
__device__ __forceinline__ int adj_mat(const AdjArgs<real>& a, long long i, int iz) {
    if (a.matmap) return __ldg(a.matmap + i);
    if (a.plane_mat) return __ldg(a.plane_mat + iz);
    return 0;
}

template <class real>
__device__ __forceinline__ real adj_c(const AdjArgs<real>& a, const MatConst<real>& M, long long i) {
    return a.cmap ? (real)__ldg(a.cmap + i) : M.c0;
}

template <class real>
__device__ __forceinline__ real loss_weight(const AdjArgs<real>& a, int ix, int iy, int iz) {
    const int dx = ix - a.fx, dy = iy - a.fy, dz = iz - a.fz;
    const int r2 = dx * dx + dy * dy + dz * dz;
    if (r2 <= a.frad2) return real(-1);
    if (iz == a.fz && r2 >= a.srad2) return (real)a.side_w;
    return real(0);
}

// d S_j / d phi_e and S_j (FP64 path, W:78-82 plus tones, bursts, elements)
__device__ __forceinline__ void src_derivs(const AdjArgs<double>& a, int j, double& S, double& dphi) {
    S = 0.0; dphi = 0.0;
    const double A = a.sA[j];
    if (A == 0.0) return;
    double tt = a.t_src[a.step] + a.sTau[j];
    if (a.burst) {
        const double tb = tt - a.tau_max;
        if (tb < 0.0 || tb >= a.burst_len) return;
        tt = tb;
    }
    double s = 0.0, c = 0.0;
    for (int k = 0; k < a.n_tones; ++k) {
        const double ang = 2 * BD_PI * a.freq[k] * tt + a.tphase[k] + a.sPhi[j];
        s += a.tamp[k] * sin(ang);
        c += a.tamp[k] * cos(ang);
    }
    S = A * s / a.sVar[j];
    dphi = A * c / a.sVar[j];
}

__device__ __forceinline__ void src_derivs(const AdjArgs<float>& a, int j, float& S, float& dphi) {
    S = 0.0f; dphi = 0.0f;
    const float A = a.sAf[j];
    if (A == 0.0f) return;
    if (a.burst) {
        const float tb = a.tb0[a.step] + a.sTauf[j];
        if (tb < 0.0f || tb >= a.burst_lenf) return;
    }
    float s = 0.0f, c = 0.0f;
    for (int k = 0; k < a.n_tones; ++k) {
        float sn, cs;
        sincosf(add_(a.theta[a.step * BD_MAX_TONES + k], a.sPsi[(long long)k * a.plane + j]), &sn, &cs);
        s = fma_(a.tampf[k], sn, s);
        c = fma_(a.tampf[k], cs, c);
    }
    S = mul_(A, s);
    dphi = mul_(A, c);
}

// Adjoint of p^{s+1} w.r.t. its update and of the relaxation coupling, shared by
// both passes: returns gY (adjoint of Y) and fills the relaxation pieces.
template <class real, int NRMAX>
struct AdjLocal {
    real gY, gD, gE;
    real lR1[NRMAX > 0 ? NRMAX : 1], lR2[NRMAX > 0 ? NRMAX : 1];
};

template <class real, int NRMAX>
__device__ __forceinline__ AdjLocal<real, NRMAX> adj_local(const AdjArgs<real>& a, const MatConst<real>& M, real c,
                                                          real m0, real w, long long i) {
    AdjLocal<real, NRMAX> L;
    const real g = m0 * w;                          // sponge: p^{s+1} = w * p_raw
    const real c2 = c * c;
    const real ic2 = real(1) / c2;
    const real ic3 = ic2 / c;
    const real kd = M.delta_2dt * ic2;
    const real kr = c2 * a.dt2;
    L.gE = real(0);
    if (M.n_relax > 0 && a.relax_scheme == BD_RELAX_SEMI_IMPLICIT) {
        // p_raw = (Y + kr G) den, den = 1/(1 - 3 kr sum a), G = sum (a E + b B), R = a (3 p_raw + E) + b B
        real sa = real(0), gP = g, sam = real(0);
        real mr[NRMAX > 0 ? NRMAX : 1];
#pragma unroll
        for (int v = 0; v < NRMAX; ++v)
            if (v < M.n_relax) {
                const real av = M.ra_num[v] * ic3;
                mr[v] = a.muR1[v][i];
                sa += av;
                gP += real(3) * av * mr[v];
                sam += av * mr[v];
            }
        const real den = real(1) / (real(1) - real(3) * kr * sa);
        L.gY = gP * den;
        const real gG = gP * kr * den;
        L.gE = gG * sa + sam;
#pragma unroll
        for (int v = 0; v < NRMAX; ++v)
            if (v < M.n_relax) {
                const real gB = M.rb[v] * (gG + mr[v]);
                L.lR1[v] = a.muR2[v][i] + real(4) * gB;
                L.lR2[v] = -gB;
            }
        L.gD = kd * L.gY;
    } else {
        // p_raw = Y + kr sum R, R = a Dttt + b (4 R1 - R2)
        L.gY = g;
        real gD = kd * g;
#pragma unroll
        for (int v = 0; v < NRMAX; ++v)
            if (v < M.n_relax) {
                const real gR = a.muR1[v][i] + kr * g;
                gD += M.ra_num[v] * ic3 * gR;
                L.lR1[v] = a.muR2[v][i] + real(4) * M.rb[v] * gR;
                L.lR2[v] = -M.rb[v] * gR;
            }
        L.gD = gD;
    }
    return L;
}

// Pass 1: loss term, source-plane gradients, H = c^2 gY.
template <class real, int NRMAX>
__global__ void adj_pass1_kernel(const AdjArgs<real> a, const WvConst<real>* __restrict__ Kp) {
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    const int iy = blockIdx.y * blockDim.y + threadIdx.y;
    const int iz = blockIdx.z;
    if (ix >= a.nx || iy >= a.ny) return;
    const long long col = (long long)iy * a.nx + ix;
    const long long i = (long long)iz * a.plane + col;
    real m0 = a.mu[0][i];
    if (a.in_window) {
        const real wl = loss_weight(a, ix, iy, iz);
        if (wl != real(0)) {
            m0 += real(2) * wl * a.fp[0][i] * a.dt;
            a.mu[0][i] = m0;
        }
    }
    if (iz == a.src_iz) {
        real S, dphi;
        src_derivs(a, (int)col, S, dphi);
        a.gphi[col] += (double)m0 * (double)dphi;
        const double ea = a.e_amp[col];
        if (ea != 0.0) a.gamp[col] += (double)m0 * (double)S / ea;
        a.H[i] = real(0);
        return;
    }
    const WvConst<real>& K = *Kp;
    const MatConst<real>& M = K.mat[adj_mat(a, i, iz)];
    const real c = adj_c(a, M, i);
    const real w = a.wx ? a.wx[ix] * a.wy[iy] * a.wz[iz] : real(1);
    const AdjLocal<real, NRMAX> L = adj_local<real, NRMAX>(a, M, c, m0, w, i);
    a.H[i] = c * c * L.gY;
}

template <class real>
__device__ __forceinline__ real hval(const AdjArgs<real>& a, int ix, int iy, int iz) {
    if (ix < 0 || iy < 0 || iz < 0 || ix >= a.nx || iy >= a.ny || iz >= a.nz) return real(0);
    return a.H[(long long)iz * a.plane + (long long)iy * a.nx + ix];
}

// Pass 2: the transposed stencil on H plus the pointwise Jacobian terms.
template <class real, int NRMAX>
__global__ void adj_pass2_kernel(const AdjArgs<real> a, const WvConst<real>* __restrict__ Kp) {
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    const int iy = blockIdx.y * blockDim.y + threadIdx.y;
    const int iz = blockIdx.z;
    if (ix >= a.nx || iy >= a.ny) return;
    const long long i = (long long)iz * a.plane + (long long)iy * a.nx + ix;
    // (d Lap / d p^s)^T H: the same symmetric 6th-order stencil applied to H
    const real h0 = a.H[i];
    auto ax = [&](int o) { return hval(a, ix + o, iy, iz) + hval(a, ix - o, iy, iz); };
    auto ay = [&](int o) { return hval(a, ix, iy + o, iz) + hval(a, ix, iy - o, iz); };
    auto az = [&](int o) { return hval(a, ix, iy, iz + o) + hval(a, ix, iy, iz - o); };
    const real sxy = real(-980) * h0 + real(270) * (ax(1) + ay(1)) - real(27) * (ax(2) + ay(2)) + real(2) * (ax(3) + ay(3));
    const real sz = real(-490) * h0 + real(270) * az(1) - real(27) * az(2) + real(2) * az(3);
    real lam0 = a.mu[1][i] + a.kxy180 * sxy + a.kz180 * sz;
    real lam1 = a.mu[2][i], lam2 = a.mu[3][i], lam3 = a.mu[4][i], lam4 = real(0);
    if (iz == a.src_iz) {
        // the source plane takes no input from the state; its relaxation values never feed p
        for (int v = 0; v < a.max_relax; ++v) { a.muR1[v][i] = real(0); a.muR2[v][i] = real(0); }
    } else {
        const WvConst<real>& K = *Kp;
        const MatConst<real>& M = K.mat[adj_mat(a, i, iz)];
        const real c = adj_c(a, M, i);
        const real w = a.wx ? a.wx[ix] * a.wy[iy] * a.wz[iz] : real(1);
        const real m0 = a.mu[0][i];
        const AdjLocal<real, NRMAX> L = adj_local<real, NRMAX>(a, M, c, m0, w, i);
        const real P0 = a.fp[1][i], P1 = a.fp[2][i], P2 = a.fp[3][i], P3 = a.fp[4][i];
        const real kn = M.beta2_rho / (c * c);
        const real s3 = real(3) * P0 - real(4) * P1 + P2;
        const real d2 = real(4) * P0 - real(5) * P1 + real(4) * P2 - P3;
        const real gY = L.gY, gD = L.gD, gE = L.gE;
        // Y = 2 P0 - P1 + Lap(P0) + kd Dttt + kn (s3^2/4 + P0 (2P0 - 5P1 + 4P2 - P3))
        lam0 += gY * (real(2) + kn * (real(1.5) * s3 + d2)) + real(5) * gD - real(10) * gE;
        lam1 += gY * (real(-1) + kn * (real(-2) * s3 - real(5) * P0)) - real(18) * gD + real(12) * gE;
        lam2 += gY * kn * (real(0.5) * s3 + real(4) * P0) + real(24) * gD - real(6) * gE;
        lam3 += gY * kn * (-P0) - real(14) * gD + gE;
        lam4 = real(3) * gD;
#pragma unroll
        for (int v = 0; v < NRMAX; ++v)
            if (v < M.n_relax) { a.muR2[v][i] = L.lR1[v]; a.muR1[v][i] = L.lR2[v]; }
    }
    a.mu[1][i] = lam0;
    a.mu[2][i] = lam1;
    a.mu[3][i] = lam2;
    a.mu[4][i] = lam3;
    a.mu[0][i] = lam4;
}

}  // namespace bd
