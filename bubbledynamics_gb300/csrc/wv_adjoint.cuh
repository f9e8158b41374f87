// Discrete adjoint of the Westervelt step (wv_kernels.cuh: cell_update and the
// source plane), for OPEN faces.  Forward step s maps the state
//   (p^s, p^{s-1}, p^{s-2}, p^{s-3}, p^{s-4}, R^{s-1}, R^{s-2})
// to (p^{s+1}, p^s, p^{s-1}, p^{s-2}, p^{s-3}, R^s, R^{s-1}).  Given the
// adjoints mu_0..mu_4, muR1, muR2 of the output state, one backward step gives
// the adjoints lambda of the input state:
//   lambda_k = mu_{k+1} + (d p^{s+1} / d p^{s-k})^T mu_0 + (d R^s / d p^{s-k})^T muR1
// The loss is sum_x w_L(x) sum_{s in window} p^{s+1}(x)^2 dt.
//
// The pointwise pass reads only its own cell (16-byte vector loads, several
// cells per thread): it adds the loss term, forms gY, gD, gE and the
// relaxation adjoints, writes lambda_1..lambda_4, the relaxation adjoints,
// lambda_0 without the stencil term, and H = c^2 gY.  The transposed 6th-order
// Laplacian of H still has to be added to lambda_0: FP32 grids with nx % 4 == 0
// do it in the next backward step's pointwise pass, as that pass loads lambda_0
// as its mu_0 (one kernel per step); the others run a stencil pass after the
// pointwise one (two kernels per step).  lambda_4 goes to a spare buffer (the
// adjoint ring has six) and the relaxation adjoints rotate through three
// buffers per process.
#pragma once

#include "wv_tma.cuh"

#include "wv_kernels.cuh"

namespace bd {

template <class real>
struct AdjArgs {
    int nx, ny, nz;
    long long plane;
    // adjoint ring of the output state: mu[k] = adjoint of p^{s+1-k}; lambda_k is written over mu[k+1]
    // (k = 0..3) and lambda_4 into mu5 (the spare), so the roles rotate by one per step
    real* mu[5];
    real* mu5;
    const real* muR1[BD_MAX_RELAX];   // adjoint of R^s
    real* muR2[BD_MAX_RELAX];         // adjoint of R^{s-1} (receives lambda of R^{s-1})
    real* muR3[BD_MAX_RELAX];         // spare (receives lambda of R^{s-2})
    int max_relax;
    // forward fields: fp[0] = p^{s+1}, fp[1] = p^s, fp[2] = p^{s-1}, fp[3] = p^{s-2}, fp[4] = p^{s-3}
    const real* fp[5];
    int zb;                     // z planes per CTA of the stencil pass
    real* H;                    // c^2 (adjoint of Y) of this backward step
    const real* Hin;            // H of the later backward step (fused pass: its stencil term completes mu_0)
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
    long long win0, win1;       // loss window: step s contributes p^{s+1} when win0 <= s < win1
    // forward step index s of this backward step = *bstep - koff: a device counter
    // that a small kernel moves after each chunk of backward steps, so one captured
    // CUDA graph of a chunk serves every segment of the sweep
    const long long* bstep;
    int koff;
};

template <class real>
__device__ __forceinline__ long long adj_step(const AdjArgs<real>& a) {
    return *a.bstep - a.koff;
}

__global__ void adj_advance_kernel(long long* bstep, int n) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *bstep -= n;
}

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
__device__ __forceinline__ void src_derivs(const AdjArgs<double>& a, long long step, int j, double& S, double& dphi) {
    S = 0.0; dphi = 0.0;
    const double A = a.sA[j];
    if (A == 0.0) return;
    double tt = a.t_src[step] + a.sTau[j];
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

__device__ __forceinline__ void src_derivs(const AdjArgs<float>& a, long long step, int j, float& S, float& dphi) {
    S = 0.0f; dphi = 0.0f;
    const float A = a.sAf[j];
    if (A == 0.0f) return;
    if (a.burst) {
        const float tb = a.tb0[step] + a.sTauf[j];
        if (tb < 0.0f || tb >= a.burst_lenf) return;
    }
    float s = 0.0f, c = 0.0f;
    for (int k = 0; k < a.n_tones; ++k) {
        float sn, cs;
        sincosf(add_(a.theta[step * BD_MAX_TONES + k], a.sPsi[(long long)k * a.plane + j]), &sn, &cs);
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
                                                          real m0, real w, const real* r1, const real* r2) {
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
                mr[v] = r1[v];
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
                L.lR1[v] = r2[v] + real(4) * gB;
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
                const real gR = r1[v] + kr * g;
                gD += M.ra_num[v] * ic3 * gR;
                L.lR1[v] = r2[v] + real(4) * M.rb[v] * gR;
                L.lR2[v] = -M.rb[v] * gR;
            }
        L.gD = gD;
    }
    return L;
}

// VEC consecutive values through one 16-byte access (VEC = 1: scalar).
template <class real, int VEC>
struct Vec {
    real v[VEC];
};

template <class real, int VEC>
__device__ __forceinline__ Vec<real, VEC> vload(const real* p) {
    Vec<real, VEC> r;
    if constexpr (VEC * sizeof(real) == 16) {
        const float4 q = __ldcs(reinterpret_cast<const float4*>(p));
        memcpy(&r, &q, 16);
    } else {
#pragma unroll
        for (int k = 0; k < VEC; ++k) r.v[k] = p[k];
    }
    return r;
}

template <class real, int VEC>
__device__ __forceinline__ void vstore(real* p, const Vec<real, VEC>& r) {
    if constexpr (VEC * sizeof(real) == 16) {
        float4 q;
        memcpy(&q, &r, 16);
        *reinterpret_cast<float4*>(p) = q;
    } else {
#pragma unroll
        for (int k = 0; k < VEC; ++k) p[k] = r.v[k];
    }
}

// The transposed 6th-order stencil of H (zero outside the grid) at four
// consecutive x cells (x0 % 4 == 0, nx % 4 == 0), added to lin:
// lin + kxy180 (Sxx + Syy) + kz180 Szz in the stencil pass's operation order.
__device__ __forceinline__ void add_stencil4(const AdjArgs<float>& a, const float* __restrict__ H, long long col,
                                             int x0, int iy, int iz, float* lin) {
    const long long nx = a.nx;
    auto row = [&](int z, int dy) -> float4 {
        const int y = iy + dy;
        if (z < 0 || z >= a.nz || y < 0 || y >= a.ny) return make_float4(0.f, 0.f, 0.f, 0.f);
        return __ldg(reinterpret_cast<const float4*>(H + (long long)z * a.plane + col + (long long)dy * nx));
    };
    const float* P = H + (long long)iz * a.plane + col;
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 c4 = row(iz, 0);
    const float4 Lq = x0 >= 4 ? __ldg(reinterpret_cast<const float4*>(P - 4)) : zero;
    const float4 Rq = x0 + 4 < a.nx ? __ldg(reinterpret_cast<const float4*>(P + 4)) : zero;
    const float4 yp1 = row(iz, 1), ym1 = row(iz, -1), yp2 = row(iz, 2), ym2 = row(iz, -2), yp3 = row(iz, 3),
                 ym3 = row(iz, -3);
    const float4 zp1 = row(iz + 1, 0), zm1 = row(iz - 1, 0), zp2 = row(iz + 2, 0), zm2 = row(iz - 2, 0),
                 zp3 = row(iz + 3, 0), zm3 = row(iz - 3, 0);
    const float xs[12] = {Lq.x, Lq.y, Lq.z, Lq.w, c4.x, c4.y, c4.z, c4.w, Rq.x, Rq.y, Rq.z, Rq.w};
    const float y1[4] = {yp1.x + ym1.x, yp1.y + ym1.y, yp1.z + ym1.z, yp1.w + ym1.w};
    const float y2[4] = {yp2.x + ym2.x, yp2.y + ym2.y, yp2.z + ym2.z, yp2.w + ym2.w};
    const float y3[4] = {yp3.x + ym3.x, yp3.y + ym3.y, yp3.z + ym3.z, yp3.w + ym3.w};
    const float z1[4] = {zp1.x + zm1.x, zp1.y + zm1.y, zp1.z + zm1.z, zp1.w + zm1.w};
    const float z2[4] = {zp2.x + zm2.x, zp2.y + zm2.y, zp2.z + zm2.z, zp2.w + zm2.w};
    const float z3[4] = {zp3.x + zm3.x, zp3.y + zm3.y, zp3.z + zm3.z, zp3.w + zm3.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float ax1 = xs[5 + k] + xs[3 + k], ax2 = xs[6 + k] + xs[2 + k], ax3 = xs[7 + k] + xs[1 + k];
        const float h0 = xs[4 + k];
        const float sxy = -980.f * h0 + 270.f * (ax1 + y1[k]) - 27.f * (ax2 + y2[k]) + 2.f * (ax3 + y3[k]);
        const float sz = -490.f * h0 + 270.f * z1[k] - 27.f * z2[k] + 2.f * z3[k];
        lin[k] = lin[k] + a.kxy180 * sxy + a.kz180 * sz;
    }
}

// Pointwise pass.  Thread = VEC consecutive cells along x (nx % VEC == 0).
// FUSE (FP32, VEC = 4): the stencil pass of the later step is folded in: mu_0
// arrives without its stencil term, which is added here from that step's H
// (a.Hin), and lambda_0 is left without its own, which the next step adds;
// one kernel per backward step and no lambda_0 round trip.
template <class real, int NRMAX, int VEC, bool FUSE = false>
__global__ void __launch_bounds__(256, FUSE ? 4 : 1) adj_point_kernel(const AdjArgs<real> a, const WvConst<real>* __restrict__ Kp) {
    static_assert(!FUSE || (VEC == 4 && sizeof(real) == 4), "the fused pass takes four FP32 cells per thread");
    __shared__ MatConst<real> sM[BD_MAX_MATERIALS];
    {
        const int n = (int)(sizeof(sM) / sizeof(int));
        const int* src = reinterpret_cast<const int*>(Kp->mat);
        int* dst = reinterpret_cast<int*>(sM);
        for (int t = threadIdx.x; t < n; t += blockDim.x) dst[t] = src[t];
    }
    __syncthreads();
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;   // vector index
    const long long i0 = q * VEC;
    if (i0 >= (long long)a.nz * a.plane) return;
    const int iz = (int)(i0 / a.plane);
    const long long col0 = i0 - (long long)iz * a.plane;
    const int iy = (int)(col0 / a.nx), ix0 = (int)(col0 - (long long)iy * a.nx);
    const long long step = adj_step(a);
    Vec<real, VEC> m0 = vload<real, VEC>(a.mu[0] + i0);
    if constexpr (FUSE) add_stencil4(a, a.Hin, col0, ix0, iy, iz, m0.v);
    Vec<real, VEC> l0 = vload<real, VEC>(a.mu[1] + i0);
    Vec<real, VEC> l1 = vload<real, VEC>(a.mu[2] + i0);
    Vec<real, VEC> l2 = vload<real, VEC>(a.mu[3] + i0);
    Vec<real, VEC> l3 = vload<real, VEC>(a.mu[4] + i0);
    Vec<real, VEC> l4, h;
    if (step >= a.win0 && step < a.win1) {
        const bool hit = abs(iz - a.fz) * abs(iz - a.fz) <= max(a.frad2, 0) || iz == a.fz;
        if (hit) {
#pragma unroll
            for (int k = 0; k < VEC; ++k) {
                const real wl = loss_weight(a, ix0 + k, iy, iz);
                if (wl != real(0)) m0.v[k] += real(2) * wl * a.fp[0][i0 + k] * a.dt;
            }
        }
    }
    if (iz == a.src_iz) {
#pragma unroll
        for (int k = 0; k < VEC; ++k) {
            const int col = (int)col0 + k;
            real S, dphi;
            src_derivs(a, step, col, S, dphi);
            a.gphi[col] += (double)m0.v[k] * (double)dphi;
            const double ea = a.e_amp[col];
            if (ea != 0.0) a.gamp[col] += (double)m0.v[k] * (double)S / ea;
            l4.v[k] = real(0);
            h.v[k] = real(0);
        }
        // the source plane takes no input from the state; its relaxation values never feed p
        for (int v = 0; v < a.max_relax; ++v) {
            Vec<real, VEC> z;
#pragma unroll
            for (int k = 0; k < VEC; ++k) z.v[k] = real(0);
            vstore<real, VEC>(a.muR2[v] + i0, z);
            vstore<real, VEC>(a.muR3[v] + i0, z);
        }
    } else {
        const Vec<real, VEC> P0 = vload<real, VEC>(a.fp[1] + i0);
        const Vec<real, VEC> P1 = vload<real, VEC>(a.fp[2] + i0);
        const Vec<real, VEC> P2 = vload<real, VEC>(a.fp[3] + i0);
        const Vec<real, VEC> P3 = vload<real, VEC>(a.fp[4] + i0);
        Vec<real, VEC> r1[NRMAX > 0 ? NRMAX : 1], r2[NRMAX > 0 ? NRMAX : 1], o2[NRMAX > 0 ? NRMAX : 1],
            o3[NRMAX > 0 ? NRMAX : 1];
#pragma unroll
        for (int v = 0; v < NRMAX; ++v) {
            r1[v] = vload<real, VEC>(a.muR1[v] + i0);
            r2[v] = vload<real, VEC>(a.muR2[v] + i0);
        }
        const real wyz = a.wx ? a.wy[iy] * a.wz[iz] : real(1);
#pragma unroll
        for (int k = 0; k < VEC; ++k) {
            const long long i = i0 + k;
            const MatConst<real>& M = sM[adj_mat(a, i, iz)];
            const real c = adj_c(a, M, i);
            const real w = a.wx ? a.wx[ix0 + k] * wyz : real(1);
            real rr1[NRMAX > 0 ? NRMAX : 1], rr2[NRMAX > 0 ? NRMAX : 1];
#pragma unroll
            for (int v = 0; v < NRMAX; ++v) { rr1[v] = r1[v].v[k]; rr2[v] = r2[v].v[k]; }
            const AdjLocal<real, NRMAX> L = adj_local<real, NRMAX>(a, M, c, m0.v[k], w, rr1, rr2);
            const real p0 = P0.v[k], p1 = P1.v[k], p2 = P2.v[k], p3 = P3.v[k];
            const real kn = M.beta2_rho / (c * c);
            const real s3 = real(3) * p0 - real(4) * p1 + p2;
            const real d2 = real(4) * p0 - real(5) * p1 + real(4) * p2 - p3;
            const real gY = L.gY, gD = L.gD, gE = L.gE;
            // Y = 2 P0 - P1 + Lap(P0) + kd Dttt + kn (s3^2/4 + P0 (2P0 - 5P1 + 4P2 - P3))
            l0.v[k] += gY * (real(2) + kn * (real(1.5) * s3 + d2)) + real(5) * gD - real(10) * gE;
            l1.v[k] += gY * (real(-1) + kn * (real(-2) * s3 - real(5) * p0)) - real(18) * gD + real(12) * gE;
            l2.v[k] += gY * kn * (real(0.5) * s3 + real(4) * p0) + real(24) * gD - real(6) * gE;
            l3.v[k] += gY * kn * (-p0) - real(14) * gD + gE;
            l4.v[k] = real(3) * gD;
            h.v[k] = c * c * gY;
#pragma unroll
            for (int v = 0; v < NRMAX; ++v) {
                const bool on = v < M.n_relax;
                o2[v].v[k] = on ? L.lR1[v] : real(0);
                o3[v].v[k] = on ? L.lR2[v] : real(0);
            }
        }
#pragma unroll
        for (int v = 0; v < NRMAX; ++v) {
            vstore<real, VEC>(a.muR2[v] + i0, o2[v]);
            vstore<real, VEC>(a.muR3[v] + i0, o3[v]);
        }
    }
    vstore<real, VEC>(a.mu[1] + i0, l0);
    vstore<real, VEC>(a.mu[2] + i0, l1);
    vstore<real, VEC>(a.mu[3] + i0, l2);
    vstore<real, VEC>(a.mu[4] + i0, l3);
    vstore<real, VEC>(a.mu5 + i0, l4);
    vstore<real, VEC>(a.H + i0, h);
}

// Stencil pass: lambda_0 += (d Lap / d p^s)^T H, the same symmetric
// 6th-order stencil applied to H with zero outside the grid.  Each thread
// marches along z over a.zb planes keeping H(iz-3..iz+4) of its column in
// registers and finishes two planes per iteration, with the x / y neighbour
// loads of both planes (through the cache) issued before either update.
template <class real>
__global__ void __launch_bounds__(256) adj_stencil_kernel(const AdjArgs<real> a) {
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    const int iy = blockIdx.y * blockDim.y + threadIdx.y;
    if (ix >= a.nx || iy >= a.ny) return;
    const int z0 = blockIdx.z * a.zb;
    const int z1 = min(a.nz, z0 + a.zb);
    const long long col = (long long)iy * a.nx + ix;
    const real* __restrict__ H = a.H;
    real* __restrict__ lam = a.mu[1];
    const long long nx = a.nx;
    const bool xin = ix >= 3 && ix + 3 < a.nx, yin = iy >= 3 && iy + 3 < a.ny;
    auto hz = [&](int z) { return (z >= 0 && z < a.nz) ? __ldg(H + (long long)z * a.plane + col) : real(0); };
    // sums of the +-1, +-2, +-3 neighbours along x and y on plane z
    auto sxy = [&](int z, real& s1, real& s2, real& s3) {
        const real* P = H + (long long)z * a.plane + col;
        real ax1, ax2, ax3, ay1, ay2, ay3;
        if (xin) {
            ax1 = __ldg(P + 1) + __ldg(P - 1); ax2 = __ldg(P + 2) + __ldg(P - 2); ax3 = __ldg(P + 3) + __ldg(P - 3);
        } else {
            auto hx = [&](int o) { const int jx = ix + o; return (jx >= 0 && jx < a.nx) ? __ldg(P + o) : real(0); };
            ax1 = hx(1) + hx(-1); ax2 = hx(2) + hx(-2); ax3 = hx(3) + hx(-3);
        }
        if (yin) {
            ay1 = __ldg(P + nx) + __ldg(P - nx); ay2 = __ldg(P + 2 * nx) + __ldg(P - 2 * nx);
            ay3 = __ldg(P + 3 * nx) + __ldg(P - 3 * nx);
        } else {
            auto hy = [&](int o) { const int jy = iy + o; return (jy >= 0 && jy < a.ny) ? __ldg(P + o * nx) : real(0); };
            ay1 = hy(1) + hy(-1); ay2 = hy(2) + hy(-2); ay3 = hy(3) + hy(-3);
        }
        s1 = ax1 + ay1; s2 = ax2 + ay2; s3 = ax3 + ay3;
    };
    auto upd = [&](int iz, const real* w, real s1, real s2, real s3, real l) {
        const real h0 = w[3];
        const real sxyv = real(-980) * h0 + real(270) * s1 - real(27) * s2 + real(2) * s3;
        const real sz = real(-490) * h0 + real(270) * (w[4] + w[2]) - real(27) * (w[5] + w[1]) + real(2) * (w[6] + w[0]);
        lam[(long long)iz * a.plane + col] = l + a.kxy180 * sxyv + a.kz180 * sz;
    };
    real w[8];
#pragma unroll
    for (int k = 0; k < 6; ++k) w[k] = hz(z0 - 3 + k);
    int iz = z0;
    for (; iz + 1 < z1; iz += 2) {
        w[6] = hz(iz + 3);
        w[7] = hz(iz + 4);
        real a1, a2, a3, b1, b2, b3;
        sxy(iz, a1, a2, a3);
        sxy(iz + 1, b1, b2, b3);
        const real l0 = lam[(long long)iz * a.plane + col];
        const real l1 = lam[(long long)(iz + 1) * a.plane + col];
        upd(iz, w, a1, a2, a3, l0);
        upd(iz + 1, w + 1, b1, b2, b3, l1);
#pragma unroll
        for (int k = 0; k < 6; ++k) w[k] = w[k + 2];
    }
    if (iz < z1) {
        w[6] = hz(iz + 3);
        real a1, a2, a3;
        sxy(iz, a1, a2, a3);
        upd(iz, w, a1, a2, a3, lam[(long long)iz * a.plane + col]);
    }
}

}  // namespace bd
