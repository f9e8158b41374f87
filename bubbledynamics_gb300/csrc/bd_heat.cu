// Bioheat + CEM43 dose along a scan trajectory: bd_spiral_heat_run (one
// domain, or z slabs of one device: bd_spiral_heat_run_slabs), one rank's z
// slab (bd_heat_slab_*) and bd_trajectory_shifts.  Replaces T:52-105 (kernel)
// and T:323-573 (host loop).
//
// BD_F64: temperature in double, dose increment pow(4|2, T-43) dt exactly as
//         T:99-102 (reference-faithful mode).
// BD_F32: theta = T - T_ref in float (the per-step change of about 1e-4 K would
//         be lost against 300 K in float), source Q in float, the dose rate
//         R^(T-43) in float and the dose itself accumulated in double (one
//         FP64 add per cell and step).  Traffic: theta read + write 8 B, Q 4 B,
//         dose RMW 16 B.
// The allocation-free entry point keeps its dose as a double-float pair (hi,
// lo) updated with error-free FP32 sums (its caller-owned buffer format).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <vector>

#include "bd_internal.h"

namespace bd {

template <class real>
struct HeatMat {
    real a0;        // 1 - 4 kxy - 2 kz - w dt
    real kxy, kz;   // dt k/(rho c dx^2), dt k/(rho c dz^2)  (T:212-215)
    real qc;        // dt/(rho c)                              (T:216-217)
    real wTa;       // w dt (T_art - T_ref)
};

template <class real>
struct HeatArgs {
    int nx, ny, nz, zb;
    long long plane;
    const real* __restrict__ Tin;
    real* __restrict__ Tout;
    const real* __restrict__ Q;
    double* __restrict__ TD;       // dose [s] in double
    float2* __restrict__ TDf;      // dose as (hi, lo) float pairs (allocation-free entry point; TD is then null)
    const int* __restrict__ plane_mat;
    const uint8_t* __restrict__ matmap;
    const int2* __restrict__ shifts;   // per step (sx, sy)
    const long long* __restrict__ step_base;
    HeatMat<real> mat[BD_MAX_MATERIALS];
    real dt;
    double T_ref;
    float T_refm43;                // T_ref - 273.15 - 43
};

// error-free a + b (Knuth TwoSum) on floats
__device__ __forceinline__ float2 two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    const float e = (a - (s - bb)) + (b - bb);
    return make_float2(s, e);
}

// double-float accumulate: (hi, lo) += x
__device__ __forceinline__ float2 df_add(float2 d, float x) {
    float2 s = two_sum(d.x, x);
    const float lo = s.y + d.y;
    const float hi = s.x + lo;
    return make_float2(hi, lo - (hi - s.x));
}

// A positive float widened to double with integer operations (exponent rebias,
// mantissa shift), so the conversion stays off the FP64 pipe, which the dose
// add already occupies; exact for normal floats, and values below the float
// normal range (dose rates under 1e-38) become zero.
__device__ __forceinline__ double widen_pos(float x) {
    const int b = __float_as_int(x);
    if (b < 0x00800000) return 0.0;                        // zero or subnormal
    return __longlong_as_double(((long long)b << 29) + (896LL << 52));
}

template <class real>
__global__ void heat_step_kernel(const HeatArgs<real> a, int koff) {
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    const int iy = blockIdx.y * blockDim.y + threadIdx.y;
    // interior only (T:65); faces keep their initial value
    if (ix < 1 || iy < 1 || ix >= a.nx - 1 || iy >= a.ny - 1) return;
    const long long step = *a.step_base + koff;
    const int2 sh = a.shifts[step];
    const int ixa = ix - sh.x, iya = iy - sh.y;                  // T:61-62
    const bool qin = ixa >= 0 && ixa < a.nx && iya >= 0 && iya < a.ny;
    const long long col = (long long)iy * a.nx + ix;
    const long long colq = (long long)iya * a.nx + ixa;
    const int z0 = max(1, blockIdx.z * a.zb);
    const int z1 = min(a.nz - 1, blockIdx.z * a.zb + a.zb);
    if (z0 >= z1) return;
    real tm = __ldg(a.Tin + (long long)(z0 - 1) * a.plane + col);
    real tc = __ldg(a.Tin + (long long)z0 * a.plane + col);
    // one cell: T:85-87 (plus the Pennes term -w dt (T - T_art), zero in the reference)
    auto cell = [&](int iz, real tmv, real tcv, real tpv, real sxy, real q) {
        const long long i = (long long)iz * a.plane + col;
        const int m = a.matmap ? a.matmap[i] : (a.plane_mat ? __ldg(a.plane_mat + iz) : 0);
        const HeatMat<real>& M = a.mat[m];
        const real tn = tcv * M.a0 + M.kxy * sxy + M.kz * (tpv + tmv) + M.qc * q + M.wTa;
        a.Tout[i] = tn;
        if (sizeof(real) == 8) {
            const double Tc = (double)tn - 273.15;                     // T:88
            // T:99-102
            a.TD[i] = a.TD[i] + (Tc < 43.0 ? pow(4.0, Tc - 43.0) : pow(2.0, Tc - 43.0)) * (double)a.dt;
        } else {
            const float x = (float)tn + a.T_refm43;                    // T_C - 43
            const float inc = exp2f(x < 0.0f ? 2.0f * x : x) * (float)a.dt;
            if (a.TD) a.TD[i] = a.TD[i] + widen_pos(inc);
            else a.TDf[i] = df_add(a.TDf[i], inc);
        }
    };
    auto sxy_at = [&](int iz) {
        const long long i = (long long)iz * a.plane + col;
        return __ldg(a.Tin + i - 1) + __ldg(a.Tin + i + 1) + __ldg(a.Tin + i + a.nx) + __ldg(a.Tin + i - a.nx);
    };
    auto q_at = [&](int iz) {                                           // T:76-77
        return qin ? __ldg(a.Q + (long long)iz * a.plane + colq) : real(0);
    };
    int iz = z0;
    // two planes per iteration: the loads of both are issued before either update
    // (four planes measured slower: fewer resident warps for the same bytes in flight)
    for (; iz + 1 < z1; iz += 2) {
        const long long i = (long long)iz * a.plane + col;
        const real tp0 = __ldg(a.Tin + i + a.plane);
        const real tp1 = __ldg(a.Tin + i + 2 * a.plane);
        const real s0 = sxy_at(iz), s1 = sxy_at(iz + 1);
        const real q0 = q_at(iz), q1 = q_at(iz + 1);
        cell(iz, tm, tc, tp0, s0, q0);
        cell(iz + 1, tc, tp0, tp1, s1, q1);
        tm = tp0;
        tc = tp1;
    }
    for (; iz < z1; ++iz) {
        const long long i = (long long)iz * a.plane + col;
        const real tp = __ldg(a.Tin + i + a.plane);
        cell(iz, tm, tc, tp, sxy_at(iz), q_at(iz));
        tm = tc;
        tc = tp;
    }
}

// FP32 step on four consecutive x cells per thread (nx % 4 == 0): theta, its
// neighbour rows and the dose pairs move as 16-byte vectors; the source Q,
// shifted by any whole number of cells, is read per cell.  Face cells keep
// their value (they are written back unchanged), like the scalar kernel.
__global__ void __launch_bounds__(128) heat_step4_kernel(const HeatArgs<float> a, int koff) {
    const int x0 = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
    const int iy = blockIdx.y * blockDim.y + threadIdx.y;
    if (x0 >= a.nx || iy < 1 || iy >= a.ny - 1) return;
    const long long step = *a.step_base + koff;
    const int2 sh = a.shifts[step];
    const int iya = iy - sh.y;                                   // T:61-62
    const bool qrow = iya >= 0 && iya < a.ny;
    const long long col = (long long)iy * a.nx + x0;
    const int z0 = max(1, blockIdx.z * a.zb);
    const int z1 = min(a.nz - 1, blockIdx.z * a.zb + a.zb);
    if (z0 >= z1) return;
    const long long P = a.plane, NX = a.nx;
    auto ld4 = [](const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); };
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 tm = ld4(a.Tin + (long long)(z0 - 1) * P + col);
    float4 tc = ld4(a.Tin + (long long)z0 * P + col);
    bool upd[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) upd[k] = x0 + k >= 1 && x0 + k < a.nx - 1;
    for (int iz = z0; iz < z1; ++iz) {
        const long long i = (long long)iz * P + col;
        const float4 tp = ld4(a.Tin + i + P);
        const float4 L = x0 >= 4 ? ld4(a.Tin + i - 4) : zero;
        const float4 R = x0 + 4 < a.nx ? ld4(a.Tin + i + 4) : zero;
        const float4 yu = ld4(a.Tin + i + NX), yd = ld4(a.Tin + i - NX);
        float q[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {                             // T:76-77
            const int ixa = x0 + k - sh.x;
            q[k] = (qrow && ixa >= 0 && ixa < a.nx) ? __ldg(a.Q + (long long)iz * P + (long long)iya * NX + ixa) : 0.f;
        }
        double2* dp = reinterpret_cast<double2*>(a.TD + i);
        double2 d01 = dp[0], d23 = dp[1];
        int mats[4];
        if (a.matmap) {
            const uchar4 mm = *reinterpret_cast<const uchar4*>(a.matmap + i);
            mats[0] = mm.x; mats[1] = mm.y; mats[2] = mm.z; mats[3] = mm.w;
        } else {
            const int m = a.plane_mat ? __ldg(a.plane_mat + iz) : 0;
            mats[0] = mats[1] = mats[2] = mats[3] = m;
        }
        const float cv[4] = {tc.x, tc.y, tc.z, tc.w};
        const float xl[4] = {L.w, tc.x, tc.y, tc.z}, xr[4] = {tc.y, tc.z, tc.w, R.x};
        const float su[4] = {yu.x, yu.y, yu.z, yu.w}, sd[4] = {yd.x, yd.y, yd.z, yd.w};
        const float zu[4] = {tp.x, tp.y, tp.z, tp.w}, zd[4] = {tm.x, tm.y, tm.z, tm.w};
        double dose[4] = {d01.x, d01.y, d23.x, d23.y};
        float tn[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const HeatMat<float>& M = a.mat[mats[k]];
            const float sxy = xl[k] + xr[k] + su[k] + sd[k];
            // T:85-87 (plus the Pennes term -w dt (T - T_art), zero in the reference)
            const float t = cv[k] * M.a0 + M.kxy * sxy + M.kz * (zu[k] + zd[k]) + M.qc * q[k] + M.wTa;
            tn[k] = upd[k] ? t : cv[k];
            if (upd[k]) {
                const float x = t + a.T_refm43;                   // T_C - 43
                const float inc = exp2f(x < 0.0f ? 2.0f * x : x) * a.dt;   // T:99-102
                dose[k] = dose[k] + widen_pos(inc);
            }
        }
        *reinterpret_cast<float4*>(a.Tout + i) = make_float4(tn[0], tn[1], tn[2], tn[3]);
        dp[0] = make_double2(dose[0], dose[1]);
        dp[1] = make_double2(dose[2], dose[3]);
        tm = tc;
        tc = tp;
    }
}

__global__ void heat_advance_kernel(long long* step_base, int n) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *step_base += n;
}

// Coefficients of T:212-217 (plus the Pennes term) for each material.
template <class real>
static void heat_materials(const bd_thermal* th, double T_ref, HeatMat<real>* out) {
    for (int k = 0; k < th->n_materials; ++k) {
        const bd_thermal_material& mt = th->mat[k];
        const double kk = mt.k_t / (mt.rho * mt.c_t);
        const double kxy = th->dt * kk / (th->dx * th->dx), kz = th->dt * kk / (th->dz * th->dz);
        const double w = mt.perfusion * th->dt;
        out[k] = HeatMat<real>{(real)(1.0 - 4.0 * kxy - 2.0 * kz - w), (real)kxy, (real)kz,
                               (real)(th->dt / (mt.rho * mt.c_t)), (real)(w * (mt.T_art - T_ref))};
    }
}

// ----------------------------------------------------------------------------
// Scratch of bd_heat_run_device_noalloc: one static device array, laid out as
// [step counter: 256 B][plane materials][per-step shifts][second theta buffer].
static __device__ __align__(256) unsigned char g_noalloc_scratch[BD_NOALLOC_SCRATCH_BYTES];

struct NoallocScratch {
    long long* step;
    int* planemat;
    int2* shifts;
    float* theta;
};

static std::mutex g_noalloc_mu;
static bool g_noalloc_ready[64];
static unsigned char* g_noalloc_base[64];

// Device address of the scratch array for the current device, looked up once
// per device with that device current.
static NoallocScratch noalloc_scratch(int dev) {
    if (dev < 0 || dev >= 64) fail(BD_ERR_INVALID_ARG, "device %d out of range for the scratch table", dev);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ready[dev]) {
        unsigned char* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) fail(BD_ERR_CUDA, "cudaGetSymbolAddress of the scratch array failed: %s", cudaGetErrorString(e));
        g_noalloc_base[dev] = p;
        g_noalloc_ready[dev] = true;
    }
    unsigned char* b = g_noalloc_base[dev];
    NoallocScratch s;
    s.step = reinterpret_cast<long long*>(b);
    s.planemat = reinterpret_cast<int*>(b + 256);
    s.shifts = reinterpret_cast<int2*>(b + 256 + 4 * BD_NOALLOC_MAX_PLANES);
    s.theta = reinterpret_cast<float*>(b + 256 + 4 * BD_NOALLOC_MAX_PLANES + 8 * BD_NOALLOC_MAX_STEPS);
    return s;
}

}  // namespace bd

using namespace bd;

// The heat + dose run (T:345-573) on z slabs: local slab k owns planes
// [zb_k, ze_k) and keeps one ghost plane beyond each internal face of the grid
// (the 7-point stencil reads iz +- 1, T:72-73).  The kernels see each slab as a
// grid of its local planes, whose first and last planes they never update (the
// grid's fixed faces, or the ghost planes), so one slab is the whole-grid run.
// Neighbouring local slabs refresh each other's ghost planes after every step;
// a rank-level slab (bd_heat_slab_*) leaves that to its caller.
struct HeatSlab {
    int zb = 0, ze = 0, lo = 0, hi = 0, nzl = 0, zbk = 32;
    long long nl = 0;                              // local cells
    PoolBuf Ta, Tb, Qd, TDd;
    dim3 grid, grid4;
};

struct HeatPlan {
    bd_context* ctx = nullptr;
    bool f64 = false, vec4 = false, use_graph = true, has_pm = false, has_mm = false;
    int nx = 0, ny = 0, nz = 0, n_legs = 0;
    long long plane = 0, n = 0;
    size_t esz = 4;
    double T_ref = 0.0, dt = 0.0;
    int64_t nsteps = 0;
    int64_t step = 0;                              // steps done
    static constexpr int leg_cap = 4096;
    std::vector<int64_t> leg_end;
    PoolBuf pm, mm, shd, sb;
    std::vector<HeatSlab> sl;
    HeatArgs<float> af{};
    HeatArgs<double> ad{};
    static constexpr int CH = 64;
    cudaGraphExec_t graphs[2] = {nullptr, nullptr};
    ~HeatPlan() {
        for (auto e : graphs)
            if (e) cudaGraphExecDestroy(e);
    }

    // checks, trajectory, initial fields (T:232-257) and the device buffers of
    // the slabs owning the given plane ranges
    void prepare(bd_context* c, const bd_thermal* th, const double* Q, const bd_trajectory* traj, int64_t max_steps,
                 const std::vector<std::pair<int, int>>& owned) {
        ctx = c;
        ctx_check(ctx);
        if (!th || !Q || !traj) fail(BD_ERR_INVALID_ARG, "null argument");
        nx = th->nx; ny = th->ny; nz = th->nz;
        if (nx < 3 || ny < 3 || nz < 3) fail(BD_ERR_INVALID_ARG, "grid too small");
        if (th->n_materials < 1 || th->n_materials > BD_MAX_MATERIALS)
            fail(BD_ERR_INVALID_ARG, "n_materials out of range");
        if (th->precision != BD_F32 && th->precision != BD_F64) fail(BD_ERR_INVALID_ARG, "bad precision");
        for (size_t k = 0; k < owned.size(); ++k) {
            const int zb = owned[k].first, ze = owned[k].second;
            if (!(0 <= zb && zb + 2 <= ze && ze <= nz)) fail(BD_ERR_INVALID_ARG, "slab [%d, %d) of %d planes", zb, ze, nz);
            if (k > 0 && owned[k - 1].second != zb) fail(BD_ERR_INVALID_ARG, "local slabs must be contiguous");
        }
        f64 = th->precision == BD_F64;
        plane = (long long)nx * ny;
        n = plane * nz;
        dt = th->dt;
        use_graph = th->plain_launches == 0;
        // trajectory
        leg_end.assign(leg_cap, 0);
        bd_status st = bd_trajectory_shifts(traj, nullptr, nullptr, 0, &nsteps, nullptr, 0);
        if (st != BD_OK) throw Error{st};
        std::vector<int32_t> sx(nsteps), sy(nsteps);
        st = bd_trajectory_shifts(traj, sx.data(), sy.data(), nsteps, &nsteps, leg_end.data(), leg_cap);
        if (st != BD_OK) throw Error{st};
        n_legs = traj->kind == BD_TRAJ_SPOTS ? traj->n_spots : traj->n_legs;
        if (max_steps > 0 && max_steps < nsteps) nsteps = max_steps;
        std::vector<int2> sh(std::max<int64_t>(nsteps, 1));
        for (int64_t s = 0; s < nsteps; ++s) sh[s] = make_int2(sx[s], sy[s]);
        // initial fields (T:232-257)
        auto mat_of = [&](long long i) -> int {
            int iz = (int)(i / plane);
            int m = th->material_map ? th->material_map[i] : (th->plane_material ? th->plane_material[iz] : 0);
            if (m < 0 || m >= th->n_materials) fail(BD_ERR_INVALID_ARG, "material index out of range");
            return m;
        };
        T_ref = f64 ? 0.0 : th->T_ref;
        std::vector<double> T0(n), TD0(n);
        for (long long i = 0; i < n; ++i) {
            const bd_thermal_material& mt = th->mat[mat_of(i)];
            T0[i] = th->T_start ? th->T_start[i] : mt.T_init;
            TD0[i] = th->dose_start ? th->dose_start[i]
                                    : (th->dose_init ? std::pow(4.0, mt.T_init - 273.15 - 43.0) * th->dt : 0.0);   // T:246, T:252
        }
        esz = f64 ? 8 : 4;
        std::vector<HeatSlab>(owned.size()).swap(sl);
        for (size_t k = 0; k < owned.size(); ++k) {
            HeatSlab& S = sl[k];
            S.zb = owned[k].first;
            S.ze = owned[k].second;
            S.lo = S.zb > 0 ? S.zb - 1 : 0;
            S.hi = S.ze < nz ? S.ze + 1 : nz;
            S.nzl = S.hi - S.lo;
            S.nl = plane * S.nzl;
        }
        shd.alloc(ctx, sh.size() * sizeof(int2));
        sb.alloc(ctx, 64);
        BD_CUDA(cudaMemcpy(shd.p, sh.data(), sh.size() * sizeof(int2), cudaMemcpyHostToDevice));
        for (HeatSlab& S : sl) {
            S.Ta.alloc(ctx, S.nl * esz); S.Tb.alloc(ctx, S.nl * esz); S.Qd.alloc(ctx, S.nl * esz);
            S.TDd.alloc(ctx, S.nl * 8);
            const long long o = plane * S.lo;
            if (f64) {
                BD_CUDA(cudaMemcpy(S.Ta.p, T0.data() + o, S.nl * 8, cudaMemcpyHostToDevice));
                BD_CUDA(cudaMemcpy(S.Tb.p, T0.data() + o, S.nl * 8, cudaMemcpyHostToDevice));
                BD_CUDA(cudaMemcpy(S.Qd.p, Q + o, S.nl * 8, cudaMemcpyHostToDevice));
            } else {
                std::vector<float> tf(S.nl), qf(S.nl);
                for (long long i = 0; i < S.nl; ++i) {
                    tf[i] = (float)(T0[o + i] - T_ref);
                    qf[i] = (float)Q[o + i];
                }
                BD_CUDA(cudaMemcpy(S.Ta.p, tf.data(), S.nl * 4, cudaMemcpyHostToDevice));
                BD_CUDA(cudaMemcpy(S.Tb.p, tf.data(), S.nl * 4, cudaMemcpyHostToDevice));
                BD_CUDA(cudaMemcpy(S.Qd.p, qf.data(), S.nl * 4, cudaMemcpyHostToDevice));
            }
            BD_CUDA(cudaMemcpy(S.TDd.p, TD0.data() + o, S.nl * 8, cudaMemcpyHostToDevice));
        }
        has_pm = th->plane_material != nullptr;
        has_mm = th->material_map != nullptr;
        if (has_pm) {
            pm.alloc(ctx, nz * 4);
            BD_CUDA(cudaMemcpy(pm.p, th->plane_material, nz * 4, cudaMemcpyHostToDevice));
        }
        if (has_mm) {
            mm.alloc(ctx, n);
            BD_CUDA(cudaMemcpy(mm.p, th->material_map, n, cudaMemcpyHostToDevice));
        }
        BD_CUDA(cudaMemset(sb.p, 0, 64));
        vec4 = !f64 && nx % 4 == 0;
        static int per_sm4 = 0;
        if (vec4 && !per_sm4) BD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm4, heat_step4_kernel, 128, 0));
        for (HeatSlab& S : sl) {
            S.zbk = 32;
            if (vec4) {
                // four-cell kernel: z-chunk fitted to whole waves of its resident CTAs
                const long long tiles = (long long)((nx / 4 + 15) / 16) * ((ny + 7) / 8);
                S.zbk = wave_fitted_zb(tiles, S.nzl, (long long)ctx->sm_count * std::max(per_sm4, 1), 0.9);
            }
            S.grid = dim3((nx + 31) / 32, (ny + 7) / 8, (S.nzl + S.zbk - 1) / S.zbk);
            S.grid4 = dim3((nx / 4 + 15) / 16, (ny + 7) / 8, (S.nzl + S.zbk - 1) / S.zbk);
        }
        // material constants (T:212-217, plus the Pennes term)
        std::memset(&af, 0, sizeof af);
        std::memset(&ad, 0, sizeof ad);
        for (int k = 0; k < th->n_materials; ++k) {
            const bd_thermal_material& mt = th->mat[k];
            const double kk = mt.k_t / (mt.rho * mt.c_t);
            const double kxy = th->dt * kk / (th->dx * th->dx), kz = th->dt * kk / (th->dz * th->dz);
            const double w = mt.perfusion * th->dt;
            const double a0 = 1.0 - 4.0 * kxy - 2.0 * kz - w;
            const double qc = th->dt / (mt.rho * mt.c_t);
            const double wTa = w * (mt.T_art - T_ref);
            af.mat[k] = HeatMat<float>{(float)a0, (float)kxy, (float)kz, (float)qc, (float)wTa};
            ad.mat[k] = HeatMat<double>{a0, kxy, kz, qc, wTa};
        }
        step = 0;
    }

    template <class A, class RR>
    void fill(A& a, const HeatSlab& S, bool a_to_b) const {
        a.nx = nx; a.ny = ny; a.nz = S.nzl; a.zb = S.zbk; a.plane = plane;
        a.Tin = (a_to_b ? S.Ta : S.Tb).template as<RR>();
        a.Tout = (a_to_b ? S.Tb : S.Ta).template as<RR>();
        a.Q = S.Qd.template as<RR>();
        a.TD = S.TDd.template as<double>();
        a.TDf = nullptr;
        a.plane_mat = has_pm ? pm.template as<int>() + S.lo : nullptr;
        a.matmap = has_mm ? mm.template as<uint8_t>() + plane * S.lo : nullptr;
        a.shifts = shd.template as<int2>();
        a.step_base = sb.template as<long long>();
        a.dt = (RR)dt;
        a.T_ref = T_ref;
        a.T_refm43 = (float)(T_ref - 273.15 - 43.0);
    }

    // the newest temperature of a slab after `steps` steps (the reference
    // toggles use_p each step, T:391; with Tin/Tout swapped per step the latest
    // field is Ta after an even number of steps)
    const PoolBuf& newest(const HeatSlab& S, int64_t steps) const { return (steps % 2 == 0) ? S.Ta : S.Tb; }

    // after a step, the ghost planes of neighbouring local slabs take each other's newest owned planes
    void exchange(cudaStream_t st, bool a_to_b) {
        const size_t pb = (size_t)plane * esz;
        for (size_t k = 0; k + 1 < sl.size(); ++k) {
            const HeatSlab& L = sl[k];
            const HeatSlab& U = sl[k + 1];
            unsigned char* lo_f = static_cast<unsigned char*>((a_to_b ? L.Tb : L.Ta).p);
            unsigned char* up_f = static_cast<unsigned char*>((a_to_b ? U.Tb : U.Ta).p);
            // L's last owned plane -> U's lower ghost; U's first owned plane -> L's upper ghost
            BD_CUDA(cudaMemcpyAsync(up_f, lo_f + (size_t)(L.ze - 1 - L.lo) * pb, pb, cudaMemcpyDeviceToDevice, st));
            BD_CUDA(cudaMemcpyAsync(lo_f + (size_t)(L.hi - 1 - L.lo) * pb, up_f + (size_t)(U.zb - U.lo) * pb, pb,
                                    cudaMemcpyDeviceToDevice, st));
        }
    }

    // steps s0 .. s0 + cnt - 1 of every local slab: the kernels read their step as
    // the device counter plus their offset, and one advance kernel moves the counter
    void issue(cudaStream_t st, int64_t s0, int cnt) {
        const dim3 block(32, 8), block4(16, 8);
        for (int k = 0; k < cnt; ++k) {
            const bool a_to_b = ((s0 + k) % 2) == 0;
            for (const HeatSlab& S : sl) {
                if (f64) {
                    HeatArgs<double> a = ad;
                    fill<HeatArgs<double>, double>(a, S, a_to_b);
                    heat_step_kernel<double><<<S.grid, block, 0, st>>>(a, k);
                } else {
                    HeatArgs<float> a = af;
                    fill<HeatArgs<float>, float>(a, S, a_to_b);
                    if (vec4) heat_step4_kernel<<<S.grid4, block4, 0, st>>>(a, k);
                    else heat_step_kernel<float><<<S.grid, block, 0, st>>>(a, k);
                }
                BD_LAUNCHED(ctx);
            }
            exchange(st, a_to_b);
        }
        heat_advance_kernel<<<1, 32, 0, st>>>(sb.as<long long>(), cnt);
        BD_LAUNCHED(ctx);
    }

    // a chunk depends only on the parity of its first step, so one captured
    // CUDA graph per parity serves every full chunk of CH steps
    cudaGraphExec_t chunk_graph(int parity) {
        if (graphs[parity]) return graphs[parity];
        cudaStream_t cs;
        BD_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        cudaGraph_t g = nullptr;
        const int64_t before = ctx->launches;
        BD_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
        try {
            issue(cs, parity, CH);
        } catch (...) {
            cudaStreamEndCapture(cs, &g);
            if (g) cudaGraphDestroy(g);
            cudaStreamDestroy(cs);
            throw;
        }
        BD_CUDA(cudaStreamEndCapture(cs, &g));
        ctx->launches = before;   // captured, not launched
        const cudaError_t e = cudaGraphInstantiate(&graphs[parity], g, 0);
        cudaGraphDestroy(g);
        cudaStreamDestroy(cs);
        BD_CUDA(e);
        return graphs[parity];
    }

    void run_steps(int64_t from, int64_t to) {
        for (int64_t s0 = from; s0 < to; s0 += CH) {
            const int cnt = (int)std::min<int64_t>(CH, to - s0);
            if (use_graph && cnt == CH) {
                BD_CUDA(cudaGraphLaunch(chunk_graph((int)(s0 % 2)), ctx->stream));
                ctx->launches += (int64_t)CH * sl.size() + 1;
            } else {
                issue(ctx->stream, s0, cnt);
            }
        }
        step = to;
    }

    // the owned planes of every local slab's temperature after `steps` steps, into the whole grid's T
    void copy_T(int64_t steps, double* dst) {
        cudaStream_t s = ctx->stream;
        for (const HeatSlab& S : sl) {
            const PoolBuf& src = newest(S, steps);
            const long long off = plane * (S.zb - S.lo), cnt = plane * (S.ze - S.zb);
            double* d = dst + plane * S.zb;
            if (f64) {
                BD_CUDA(cudaMemcpyAsync(d, static_cast<const double*>(src.p) + off, cnt * 8, cudaMemcpyDeviceToHost, s));
                BD_CUDA(cudaStreamSynchronize(s));
            } else {
                std::vector<float> tf(cnt);
                BD_CUDA(cudaMemcpyAsync(tf.data(), static_cast<const float*>(src.p) + off, cnt * 4,
                                        cudaMemcpyDeviceToHost, s));
                BD_CUDA(cudaStreamSynchronize(s));
                for (long long i = 0; i < cnt; ++i) d[i] = T_ref + (double)tf[i];
            }
        }
    }

    void copy_dose(double* dst) {
        for (const HeatSlab& S : sl)
            BD_CUDA(cudaMemcpy(dst + plane * S.zb, static_cast<const double*>(S.TDd.p) + plane * (S.zb - S.lo),
                               (size_t)plane * (S.ze - S.zb) * 8, cudaMemcpyDeviceToHost));
    }
};

static void heat_run(bd_context* ctx, const bd_thermal* th, const double* Q, const bd_trajectory* traj,
                     int64_t max_steps, int n_slabs, bd_heat_outputs* out) {
    ctx_check(ctx);
    if (!th || !out) fail(BD_ERR_INVALID_ARG, "null argument");
    if (n_slabs < 1 || n_slabs > th->nz / 2) fail(BD_ERR_INVALID_ARG, "n_slabs must be in [1, nz / 2]");
    std::vector<std::pair<int, int>> owned;
    for (int k = 0; k < n_slabs; ++k)
        owned.push_back({(int)((long long)th->nz * k / n_slabs), (int)((long long)th->nz * (k + 1) / n_slabs)});
    HeatPlan P;
    P.prepare(ctx, th, Q, traj, max_steps, owned);
    // snapshot schedule: after the listed legs (T:412-563)
    std::vector<std::pair<int64_t, int>> snaps;
    for (int k = 0; k < out->n_snap; ++k) {
        const int leg = out->snapshot_legs ? out->snapshot_legs[k] : 0;
        if (leg < 1 || leg > P.n_legs || leg > HeatPlan::leg_cap) fail(BD_ERR_INVALID_ARG, "snapshot leg %d out of range", leg);
        snaps.push_back({P.leg_end[leg - 1], k});
    }
    std::sort(snaps.begin(), snaps.end());
    cudaStream_t s = ctx->stream;
    BD_CUDA(cudaEventRecord(ctx->ev0, s));
    int64_t done = 0;
    size_t isnap = 0;
    while (true) {
        // snapshots due at this step (a leg of zero steps ends where it starts)
        while (isnap < snaps.size() && snaps[isnap].first <= done) {
            if (out->snapshots)
                P.copy_T(done, static_cast<double*>(out->snapshots) + (size_t)snaps[isnap].second * P.n);
            ++isnap;
        }
        if (done >= P.nsteps) break;
        int64_t next = P.nsteps;
        if (isnap < snaps.size()) next = std::min<int64_t>(next, snaps[isnap].first);
        P.run_steps(done, next);
        done = next;
    }
    BD_CUDA(cudaEventRecord(ctx->ev1, s));
    BD_CUDA(cudaEventSynchronize(ctx->ev1));
    float ms = 0;
    BD_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    if (out->T_final) P.copy_T(P.nsteps, static_cast<double*>(out->T_final));
    if (out->dose) P.copy_dose(static_cast<double*>(out->dose));
    out->elapsed_ms = ms;
    out->steps_done = P.nsteps;
}

// One rank's z slab of a heat run (bd_heat_slab_begin .. _end).
struct bd_heat_slab {
    HeatPlan P;
};

extern "C" {

bd_status bd_trajectory_shifts(const bd_trajectory* tr, int32_t* sx, int32_t* sy, int64_t cap, int64_t* n_steps,
                               int64_t* leg_end, int32_t leg_cap) {
    return guard([&] {
        if (!tr || !n_steps) fail(BD_ERR_INVALID_ARG, "null argument");
        int64_t k = 0;
        if (tr->kind == BD_TRAJ_SPOTS) {
            // discrete focal spots: hold shift (spot_sx, spot_sy) for spot_steps steps each
            if (tr->n_spots <= 0 || !tr->spot_sx || !tr->spot_sy || !tr->spot_steps) fail(BD_ERR_INVALID_ARG, "bad spot list");
            for (int s = 0; s < tr->n_spots; ++s) {
                if (tr->spot_steps[s] < 0) fail(BD_ERR_INVALID_ARG, "negative spot duration");
                for (int64_t n = 0; n < tr->spot_steps[s]; ++n) {
                    if (sx && k < cap) { sx[k] = tr->spot_sx[s]; sy[k] = tr->spot_sy[s]; }
                    ++k;
                }
                if (leg_end && s < leg_cap) leg_end[s] = k;
            }
            *n_steps = k;
            return;
        }
        if (tr->kind != BD_TRAJ_SQUARE_SPIRAL) fail(BD_ERR_INVALID_ARG, "unknown trajectory kind");
        if (!(tr->speed > 0 && tr->dt > 0 && tr->dxy > 0 && tr->t_acc > 0 && tr->scale > 0) || tr->n_legs < 0)
            fail(BD_ERR_INVALID_ARG, "bad spiral parameters");
        // T:141-173 and the loop T:345-410: trapezoidal speed, legs of increase*scale
        // alternating x / y, position snapped to the nearest grid node.
        const double dt = tr->dt, dxy = tr->dxy;
        const int Nt_scale = 1 + (int)(tr->scale / (tr->speed * dt));
        const int Nt_acc = 1 + (int)(tr->t_acc / dt);
        const double acc = (tr->speed - tr->speed_init) / tr->t_acc;
        std::vector<double> speed_acc(Nt_acc);
        for (int i = 0; i < Nt_acc; i++) speed_acc[i] = tr->speed_init + i * dt * acc;
        int lines = 0, increase = 1, sign_x = 1, sign_y = -1, shift_x = 0, shift_y = 0;
        bool right_left = true;
        double x_s = 0.0, y_s = 0.0, x_next = 0.0, x_prev = 0.0, y_next = 0.0, y_prev = 0.0;
        double v = tr->speed_init;
        while (lines < tr->n_legs) {
            int n = (lines == 0) ? 1 : 0;
            x_next = x_prev + sign_x * dxy;
            y_next = y_prev + sign_y * dxy;
            for (; n < increase * Nt_scale + 2 * Nt_acc; n++) {
                if (n < Nt_acc) v = speed_acc[n];
                if (n >= Nt_acc && n < increase * Nt_scale + Nt_acc) v = tr->speed;
                if (n >= increase * Nt_scale + Nt_acc) v = speed_acc[increase * Nt_scale + 2 * Nt_acc - n - 1];
                if (right_left) {
                    x_s = x_s + sign_x * v * dt;
                    if (std::fabs(x_next - x_s) / dxy < std::fabs(x_s - x_prev) / dxy) {
                        shift_x += sign_x; x_prev = x_next; x_next = x_next + sign_x * dxy;
                    }
                } else {
                    y_s = y_s + sign_y * v * dt;
                    if (std::fabs(y_next - y_s) / dxy < std::fabs(y_s - y_prev) / dxy) {
                        shift_y += sign_y; y_prev = y_next; y_next = y_next + sign_y * dxy;
                    }
                }
                if (sx && k < cap) { sx[k] = shift_x; sy[k] = shift_y; }
                ++k;
            }
            right_left = !right_left;
            if (right_left) { increase++; sign_x = -sign_x; x_next = x_prev; }
            else { sign_y = -sign_y; y_next = y_prev; }
            if (leg_end && lines < leg_cap) leg_end[lines] = k;
            lines++;
        }
        *n_steps = k;
    });
}

bd_status bd_spiral_heat_run(bd_context* ctx, const bd_thermal* th, const double* Q, const bd_trajectory* traj,
                             int64_t max_steps, bd_heat_outputs* out) {
    return guard([&] { heat_run(ctx, th, Q, traj, max_steps, 1, out); });
}

bd_status bd_spiral_heat_run_slabs(bd_context* ctx, const bd_thermal* th, const double* Q, const bd_trajectory* traj,
                                   int64_t max_steps, int32_t n_slabs, bd_heat_outputs* out) {
    return guard([&] { heat_run(ctx, th, Q, traj, max_steps, n_slabs, out); });
}

bd_status bd_heat_slab_begin(bd_context* ctx, const bd_thermal* th, const double* Q, const bd_trajectory* traj,
                             int64_t max_steps, int32_t z_begin, int32_t z_end, bd_heat_slab** out) {
    return guard([&] {
        if (!out) fail(BD_ERR_INVALID_ARG, "null output");
        *out = nullptr;
        std::unique_ptr<bd_heat_slab> h(new bd_heat_slab());
        h->P.prepare(ctx, th, Q, traj, max_steps, {{z_begin, z_end}});
        h->P.use_graph = false;                  // one step at a time between halo refreshes
        *out = h.release();
    });
}

bd_status bd_heat_slab_steps(bd_heat_slab* h, int64_t* total, int64_t* done) {
    return guard([&] {
        if (!h) fail(BD_ERR_INVALID_ARG, "null slab");
        if (total) *total = h->P.nsteps;
        if (done) *done = h->P.step;
    });
}

bd_status bd_heat_slab_advance(bd_heat_slab* h, int64_t n) {
    return guard([&] {
        if (!h) fail(BD_ERR_INVALID_ARG, "null slab");
        ctx_check(h->P.ctx);
        if (n < 0 || h->P.step + n > h->P.nsteps) fail(BD_ERR_INVALID_ARG, "advance past the end of the run");
        h->P.run_steps(h->P.step, h->P.step + n);
        BD_CUDA(cudaStreamSynchronize(h->P.ctx->stream));   // the steps are done when this returns
    });
}

bd_status bd_heat_slab_halo_bytes(bd_heat_slab* h, size_t* bytes) {
    return guard([&] {
        if (!h || !bytes) fail(BD_ERR_INVALID_ARG, "null argument");
        *bytes = (size_t)h->P.plane * h->P.esz;
    });
}

bd_status bd_heat_slab_halo_copy(bd_heat_slab* h, int32_t side, int32_t to_ghost, void* d_buf, void* stream) {
    return guard([&] {
        if (!h || !d_buf) fail(BD_ERR_INVALID_ARG, "null argument");
        ctx_check(h->P.ctx);
        const HeatSlab& S = h->P.sl[0];
        if (side != 0 && side != 1) fail(BD_ERR_INVALID_ARG, "side must be 0 or 1");
        if ((side == 0 && S.zb == 0) || (side == 1 && S.ze == h->P.nz))
            fail(BD_ERR_INVALID_ARG, "side %d of this slab is a face of the grid", side);
        const size_t pb = (size_t)h->P.plane * h->P.esz;
        // the newest temperature: the owned plane next to the face, or the ghost plane beyond it
        const int local = side == 0 ? (to_ghost ? 0 : 1) : (to_ghost ? S.nzl - 1 : S.nzl - 2);
        char* plane = static_cast<char*>(h->P.newest(S, h->P.step).p) + (size_t)local * pb;
        cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : h->P.ctx->stream;
        if (to_ghost) BD_CUDA(cudaMemcpyAsync(plane, d_buf, pb, cudaMemcpyDeviceToDevice, st));
        else BD_CUDA(cudaMemcpyAsync(d_buf, plane, pb, cudaMemcpyDeviceToDevice, st));
    });
}

bd_status bd_heat_slab_finish(bd_heat_slab* h, bd_heat_outputs* out) {
    return guard([&] {
        if (!h || !out) fail(BD_ERR_INVALID_ARG, "null argument");
        ctx_check(h->P.ctx);
        BD_CUDA(cudaStreamSynchronize(h->P.ctx->stream));
        if (out->T_final) h->P.copy_T(h->P.step, static_cast<double*>(out->T_final));
        if (out->dose) h->P.copy_dose(static_cast<double*>(out->dose));
        out->steps_done = h->P.step;
    });
}

bd_status bd_heat_slab_end(bd_heat_slab* h) {
    return guard([&] { delete h; });
}

bd_status bd_heat_run_device_noalloc(bd_context* ctx, const bd_thermal* th, float* d_theta, const float* d_Q,
                                     float* d_dose, const int32_t* shifts, int64_t n_steps, void* stream) {
    return guard([&] {
        ctx_check(ctx);
        if (!th || !d_theta || !d_Q || !d_dose || (n_steps > 0 && !shifts)) fail(BD_ERR_INVALID_ARG, "null argument");
        if (th->precision != BD_F32) fail(BD_ERR_INVALID_ARG, "the allocation-free heat run needs precision BD_F32");
        if (th->material_map) fail(BD_ERR_UNSUPPORTED, "the allocation-free heat run takes plane_material only");
        const int nx = th->nx, ny = th->ny, nz = th->nz;
        if (nx < 3 || ny < 3 || nz < 3) fail(BD_ERR_INVALID_ARG, "grid too small");
        const long long n = (long long)nx * ny * nz;
        if (n > BD_NOALLOC_MAX_CELLS)
            fail(BD_ERR_INVALID_ARG, "%lld cells exceed the allocation-free limit of %d", n, BD_NOALLOC_MAX_CELLS);
        if (nz > BD_NOALLOC_MAX_PLANES)
            fail(BD_ERR_INVALID_ARG, "%d planes exceed the allocation-free limit of %d", nz, BD_NOALLOC_MAX_PLANES);
        if (n_steps < 0 || n_steps > BD_NOALLOC_MAX_STEPS)
            fail(BD_ERR_INVALID_ARG, "%lld steps outside the allocation-free limit of %d", (long long)n_steps,
                 BD_NOALLOC_MAX_STEPS);
        if (th->n_materials < 1 || th->n_materials > BD_MAX_MATERIALS) fail(BD_ERR_INVALID_ARG, "n_materials out of range");
        if (th->plane_material)
            for (int iz = 0; iz < nz; ++iz)
                if (th->plane_material[iz] < 0 || th->plane_material[iz] >= th->n_materials)
                    fail(BD_ERR_INVALID_ARG, "plane_material entry out of range");
        if (n_steps == 0) return;
        const NoallocScratch sc = noalloc_scratch(ctx->device);
        cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
        // the array keeps the last call's contents: the step counter restarts at zero,
        // the partner buffer starts as a copy of the input field (faces are never written)
        BD_CUDA(cudaMemsetAsync(sc.step, 0, sizeof(long long), s));
        if (th->plane_material)
            BD_CUDA(cudaMemcpyAsync(sc.planemat, th->plane_material, nz * sizeof(int), cudaMemcpyHostToDevice, s));
        BD_CUDA(cudaMemcpyAsync(sc.shifts, shifts, (size_t)n_steps * sizeof(int2), cudaMemcpyHostToDevice, s));
        BD_CUDA(cudaMemcpyAsync(sc.theta, d_theta, (size_t)n * sizeof(float), cudaMemcpyDeviceToDevice, s));
        HeatArgs<float> a;
        std::memset(&a, 0, sizeof a);
        heat_materials<float>(th, th->T_ref, a.mat);
        a.nx = nx; a.ny = ny; a.nz = nz; a.zb = 32; a.plane = (long long)nx * ny;
        a.Q = d_Q;
        a.TD = nullptr;
        a.TDf = reinterpret_cast<float2*>(d_dose);
        a.plane_mat = th->plane_material ? sc.planemat : nullptr;
        a.matmap = nullptr;
        a.shifts = sc.shifts;
        a.step_base = sc.step;
        a.dt = (float)th->dt;
        a.T_ref = th->T_ref;
        a.T_refm43 = (float)(th->T_ref - 273.15 - 43.0);
        dim3 block(32, 8), grid((nx + 31) / 32, (ny + 7) / 8, (nz + a.zb - 1) / a.zb);
        const int CH = 64;
        for (int64_t s0 = 0; s0 < n_steps; s0 += CH) {
            const int cnt = (int)std::min<int64_t>(CH, n_steps - s0);
            for (int k = 0; k < cnt; ++k) {
                const bool even = ((s0 + k) % 2) == 0;   // even steps read the caller's field
                a.Tin = even ? d_theta : sc.theta;
                a.Tout = even ? sc.theta : d_theta;
                heat_step_kernel<float><<<grid, block, 0, s>>>(a, k);
                BD_LAUNCHED(ctx);
            }
            heat_advance_kernel<<<1, 32, 0, s>>>(sc.step, cnt);
            BD_LAUNCHED(ctx);
        }
        if (n_steps % 2 == 1)   // the latest field is in the partner buffer
            BD_CUDA(cudaMemcpyAsync(d_theta, sc.theta, (size_t)n * sizeof(float), cudaMemcpyDeviceToDevice, s));
    });
}

}  // extern "C"
