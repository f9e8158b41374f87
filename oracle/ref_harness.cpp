/*
 * ref_harness.cpp — runs the reference's own kernel code on the host.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/build.py extracts the kernel sections of
 * the three reference files (every line before `int main()`) into
 * oracle/_ref/src/ and compiles them here, each inside its own namespace, with
 * ref_stub.h turning the CUDA qualifiers into plain C++.  The drivers below
 * restate the reference's host loops (W:556-757, T:345-392, G:573) and emulate
 * each <<<blocks, threads>>> launch by calling the kernel body once per thread,
 * blocks in (z, y, x) order and threads in (z, y, x) order.  Kernels whose
 * threads are independent run with OpenMP over blocks; the Mur boundary kernel
 * (W:88-135), whose threads read each other's writes, always runs serially.
 */
#include "ref_stub.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

thread_local bdref_uint3 threadIdx;
thread_local bdref_uint3 blockIdx;
thread_local bdref_uint3 blockDim;

#define printf(...) ((void)0)
namespace refW {
#include "_ref/src/W_kernels.inc"
}
namespace refT {
#include "_ref/src/T_kernels.inc"
}
namespace refG {
#include "_ref/src/G_kernels.inc"
}

/* The spiral loop of T main, recording the shift passed to each launch. */
namespace refTtraj {
static std::vector<int>* g_rec = nullptr;
#define BDREF_RECORD(sx_, sy_, leg_) do { g_rec->push_back(sx_); g_rec->push_back(sy_); g_rec->push_back(leg_); } while (0)
static int run() {
#include "_ref/src/T_traj.inc"
    (void)use_p; (void)t; (void)x_next; (void)y_next;
    return 0;
}
#undef BDREF_RECORD
}
#undef printf

namespace {

struct Dim { unsigned x, y, z; };

template <class F>
void launch(Dim grid, Dim block, bool parallel, F&& body) {
    auto run_block = [&](unsigned bx, unsigned by, unsigned bz) {
        blockDim = {block.x, block.y, block.z};
        blockIdx = {bx, by, bz};
        for (unsigned tz = 0; tz < block.z; ++tz)
            for (unsigned ty = 0; ty < block.y; ++ty)
                for (unsigned tx = 0; tx < block.x; ++tx) {
                    threadIdx = {tx, ty, tz};
                    body();
                }
    };
    const long nblk = (long)grid.x * grid.y * grid.z;
    if (parallel) {
#pragma omp parallel for schedule(dynamic, 1)
        for (long b = 0; b < nblk; ++b) {
            unsigned bx = (unsigned)(b % grid.x);
            unsigned by = (unsigned)((b / grid.x) % grid.y);
            unsigned bz = (unsigned)(b / ((long)grid.x * grid.y));
            run_block(bx, by, bz);
        }
    } else {
        for (unsigned bz = 0; bz < grid.z; ++bz)
            for (unsigned by = 0; by < grid.y; ++by)
                for (unsigned bx = 0; bx < grid.x; ++bx) run_block(bx, by, bz);
    }
}

/* Forward C2C transform standing in for cufftExecC2C (W:743): only the bins
 * the reference reads afterwards (multiples of `periods` up to N_harm) are
 * formed; the other bins are zero.  Accumulated in double, stored as float
 * like cuFFT's single-precision output. */
void dft_bins(cufftComplex* C, long batch, int N, int periods, int N_harm) {
    std::vector<double> cs((size_t)N), sn((size_t)N);
    for (int j = 0; j < N; ++j) { cs[j] = std::cos(2.0 * M_PI * j / N); sn[j] = std::sin(2.0 * M_PI * j / N); }
#pragma omp parallel for schedule(static)
    for (long b = 0; b < batch; ++b) {
        cufftComplex* x = C + (size_t)b * N;
        std::vector<double> out_re(N, 0.0), out_im(N, 0.0);
        for (int h = 0; h <= N_harm; ++h) {
            int k = h * periods;
            if (k >= N) break;
            double re = 0.0, im = 0.0;
            for (int t = 0; t < N; ++t) {
                int j = (int)(((long)k * t) % N);
                re += x[t].x * cs[j] + x[t].y * sn[j];
                im += x[t].y * cs[j] - x[t].x * sn[j];
            }
            out_re[k] = re; out_im[k] = im;
        }
        for (int t = 0; t < N; ++t) { x[t].x = (float)out_re[t]; x[t].y = (float)out_im[t]; }
    }
}

}  // namespace

extern "C" {

/* Parameters of W:355-416 that the reference passes through __constant__. */
typedef struct bdref_w_cfg {
    int32_t Nxy, Nz;
    double rho, c_inf, delta, beta, abs_water;
    double rho_tissue, c_inf_tissue, beta_tissue, abs_tissue;
    double delta_tissue, c1, c2, tau1, tau2;
    double fr, d, alpha, alpha_hole, p0, water_tissue;
    double xy_min, dxy, z_min, dz, dt;
    double t_max;
    int32_t periods, iz_tissue, nx_slab, N_harm;
    int32_t do_power;
    int32_t pad0;
} bdref_w_cfg;

/* Restates W main (W:470-757) on caller-sized arrays.  P_snap receives d_P at
 * the end of the first loop (the 165-period snapshot of W:600-613), Q_out the
 * final acoustic power.  steps[0..2]: step counts of the three loops. */
int bdref_w_run(const bdref_w_cfg* c, double* P_snap, double* Q_out, int64_t* steps) {
    using namespace refW;
    rho = c->rho; c_inf = c->c_inf; delta = c->delta; beta = c->beta; abs_water = c->abs_water;
    rho_tissue = c->rho_tissue; c_inf_tissue = c->c_inf_tissue; beta_tissue = c->beta_tissue;
    abs_tissue = c->abs_tissue; delta_tissue = c->delta_tissue;
    c1 = c->c1; c2 = c->c2; tau1 = c->tau1; tau2 = c->tau2;
    fr = c->fr; d = c->d; alpha = c->alpha; alpha_hole = c->alpha_hole; p0 = c->p0;
    water_tissue = c->water_tissue;
    xy_min = c->xy_min; dxy = c->dxy; z_min = c->z_min; dz = c->dz; dt = c->dt;
    const int Nxy = c->Nxy, Nz = c->Nz;
    const size_t N = (size_t)Nxy * Nxy * Nz;
    std::vector<double> A[12];
    for (auto& a : A) a.assign(N, 0.0);
    double *P_next = A[0].data(), *P = A[1].data(), *P_m1 = A[2].data(), *P_m2 = A[3].data(),
           *P_m3 = A[4].data(), *P_m4 = A[5].data(), *R1 = A[6].data(), *R1m1 = A[7].data(),
           *R1m2 = A[8].data(), *R2 = A[9].data(), *R2m1 = A[10].data(), *R2m2 = A[11].data();
    Dim threads{8, 8, 8};
    Dim blocks{(unsigned)((Nxy + 7) / 8), (unsigned)((Nxy + 7) / 8), (unsigned)((Nz + 7) / 8)};
    auto rotate = [&]() {   /* W:575-584 */
        std::memcpy(P_m4, P_m3, N * 8); std::memcpy(P_m3, P_m2, N * 8); std::memcpy(P_m2, P_m1, N * 8);
        std::memcpy(P_m1, P, N * 8); std::memcpy(P, P_next, N * 8);
        std::memcpy(R1m2, R1m1, N * 8); std::memcpy(R1m1, R1, N * 8);
        std::memcpy(R2m2, R2m1, N * 8); std::memcpy(R2m1, R2, N * 8);
    };
    double t = 0.0;
    int64_t s1 = 0;
    while (t < c->t_max) {                                  /* W:558-585 */
        launch(blocks, threads, true, [&] { Westervelt_space6(P_next, P, P_m1, P_m2, P_m3, P_m4, R1, R1m1, R1m2, R2, R2m1, R2m2, Nxy, Nz); });
        s1++;
        t = t + c->dt;
        launch(blocks, threads, true, [&] { boundary_condition_source(P_next, t, Nxy, Nz); });
        launch(blocks, threads, false, [&] { boundary_condition_space6(P_next, P, t, Nxy, Nz); });
        rotate();
    }
    steps[0] = s1;
    if (P_snap) std::memcpy(P_snap, P, N * 8);
    if (!c->do_power) { steps[1] = steps[2] = 0; return 0; }
    std::vector<double> H[12];                               /* W:600-613 */
    for (int k = 0; k < 12; ++k) H[k] = A[k];
    const double time_165p = t;
    std::vector<double> Qv(N, 0.0);
    double* Q = Qv.data();
    int64_t s2 = 0;
    while (t < c->t_max + 1 / c->fr) {                      /* W:627-657 */
        launch(blocks, threads, true, [&] { Westervelt_space6(P_next, P, P_m1, P_m2, P_m3, P_m4, R1, R1m1, R1m2, R2, R2m1, R2m2, Nxy, Nz); });
        s2++;
        t = t + c->dt;
        launch(blocks, threads, true, [&] { boundary_condition_source(P_next, t, Nxy, Nz); });
        launch(blocks, threads, false, [&] { boundary_condition_space6(P_next, P, t, Nxy, Nz); });
        launch(blocks, threads, true, [&] { acoustic_power_water(Q, P_next, P_m1, Nxy, Nz, false); });
        rotate();
    }
    launch(blocks, threads, true, [&] { acoustic_power_water(Q, P_next, P_m1, Nxy, Nz, true); });   /* W:658 */
    steps[1] = s2;
    /* W:666-755: FFT path, slab by slab */
    const int periods = c->periods, N_time = periods * 100, N_harm = c->N_harm;
    const int iz_t = c->iz_tissue, Nz_tissue = Nz - iz_t, nx = c->nx_slab;
    const size_t Nxyz_tissue = (size_t)nx * Nxy * Nz_tissue;
    std::vector<double> Pt(Nxyz_tissue * N_time, 0.0);
    std::vector<cufftComplex> Pc(Nxyz_tissue * N_time);
    /* The reference launches the conversion kernels with the field grid, whose x
     * extent (>= Nxy) covers N_time at its own size; here the x extent is taken
     * large enough for N_time so that smaller boxes convert every sample. */
    Dim blocks_t{(unsigned)((std::max(Nxy, N_time) + 7) / 8), blocks.y, blocks.z};
    int64_t s3 = 0;
    for (int ixs = 0; ixs < Nxy / nx; ixs++) {
        t = time_165p;
        for (int k = 0; k < 12; ++k) A[k] = H[k];            /* W:690-703 */
        P_next = A[0].data(); P = A[1].data(); P_m1 = A[2].data(); P_m2 = A[3].data();
        P_m3 = A[4].data(); P_m4 = A[5].data(); R1 = A[6].data(); R1m1 = A[7].data();
        R1m2 = A[8].data(); R2 = A[9].data(); R2m1 = A[10].data(); R2m2 = A[11].data();
        for (int idx_time = 0; idx_time < N_time; idx_time++) {
            launch(blocks, threads, true, [&] { Westervelt_space6(P_next, P, P_m1, P_m2, P_m3, P_m4, R1, R1m1, R1m2, R2, R2m1, R2m2, Nxy, Nz); });
            t = t + c->dt;
            launch(blocks, threads, true, [&] { boundary_condition_source(P_next, t, Nxy, Nz); });
            launch(blocks, threads, false, [&] { boundary_condition_space6(P_next, P, t, Nxy, Nz); });
            launch(blocks, threads, true, [&] { copy_data(P_next, Pt.data(), ixs, nx, Nxy, Nz_tissue, iz_t, idx_time, N_time); });
            rotate();
            s3++;
        }
        launch(blocks_t, threads, true, [&] { Double_to_Complex(Pt.data(), Pc.data(), nx, Nxy, Nz_tissue, N_time); });
        dft_bins(Pc.data(), (long)Nxyz_tissue, N_time, periods, N_harm);
        launch(blocks_t, threads, true, [&] { Abs_Complex(Pc.data(), Pt.data(), nx, Nxy, Nz_tissue, N_time); });
        launch(blocks, threads, true, [&] { total_energy_Nharmonics_xyz(Q, Pt.data(), ixs, nx, Nxy, Nz_tissue, iz_t, N_time, periods, N_harm); });
    }
    steps[2] = s3;
    std::memcpy(Q_out, Q, N * 8);
    return 0;
}

/* Only the first loop of W (W:558-585) for n_steps steps; returns the 12
 * state arrays in `state` (order P_next, P, P_m1..P_m4, R1, R1m1, R1m2, R2,
 * R2m1, R2m2), each N doubles.  Used for the cost baseline and step parity. */
int bdref_w_steps(const bdref_w_cfg* c, int64_t n_steps, double* state) {
    using namespace refW;
    rho = c->rho; c_inf = c->c_inf; delta = c->delta; beta = c->beta; abs_water = c->abs_water;
    rho_tissue = c->rho_tissue; c_inf_tissue = c->c_inf_tissue; beta_tissue = c->beta_tissue;
    abs_tissue = c->abs_tissue; delta_tissue = c->delta_tissue;
    c1 = c->c1; c2 = c->c2; tau1 = c->tau1; tau2 = c->tau2;
    fr = c->fr; d = c->d; alpha = c->alpha; alpha_hole = c->alpha_hole; p0 = c->p0;
    water_tissue = c->water_tissue;
    xy_min = c->xy_min; dxy = c->dxy; z_min = c->z_min; dz = c->dz; dt = c->dt;
    const int Nxy = c->Nxy, Nz = c->Nz;
    const size_t N = (size_t)Nxy * Nxy * Nz;
    double* S[12];
    for (int k = 0; k < 12; ++k) S[k] = state + (size_t)k * N;
    double *P_next = S[0], *P = S[1], *P_m1 = S[2], *P_m2 = S[3], *P_m3 = S[4], *P_m4 = S[5];
    double *R1 = S[6], *R1m1 = S[7], *R1m2 = S[8], *R2 = S[9], *R2m1 = S[10], *R2m2 = S[11];
    Dim threads{8, 8, 8};
    Dim blocks{(unsigned)((Nxy + 7) / 8), (unsigned)((Nxy + 7) / 8), (unsigned)((Nz + 7) / 8)};
    double t = 0.0;
    for (int64_t s = 0; s < n_steps; ++s) {
        launch(blocks, threads, true, [&] { Westervelt_space6(P_next, P, P_m1, P_m2, P_m3, P_m4, R1, R1m1, R1m2, R2, R2m1, R2m2, Nxy, Nz); });
        t = t + c->dt;
        launch(blocks, threads, true, [&] { boundary_condition_source(P_next, t, Nxy, Nz); });
        launch(blocks, threads, false, [&] { boundary_condition_space6(P_next, P, t, Nxy, Nz); });
        std::memcpy(P_m4, P_m3, N * 8); std::memcpy(P_m3, P_m2, N * 8); std::memcpy(P_m2, P_m1, N * 8);
        std::memcpy(P_m1, P, N * 8); std::memcpy(P, P_next, N * 8);
        std::memcpy(R1m2, R1m1, N * 8); std::memcpy(R1m1, R1, N * 8);
        std::memcpy(R2m2, R2m1, N * 8); std::memcpy(R2m1, R2, N * 8);
    }
    return 0;
}

/* Per-step shifts of the reference's own spiral loop (T:323-410): rec holds
 * (shift_x, shift_y, leg) per heat step; returns the number of steps, or -1 if
 * cap is too small. */
int64_t bdref_t_trajectory(int32_t* rec, int64_t cap) {
    std::vector<int> v;
    refTtraj::g_rec = &v;
    refTtraj::run();
    const int64_t n = (int64_t)v.size() / 3;
    if (n > cap) return -1;
    for (size_t i = 0; i < v.size(); ++i) rec[i] = v[i];
    return n;
}

/* Constants of T:194-224. */
typedef struct bdref_t_cfg {
    int32_t Nxy, Nz;
    double dz, water_tissue, dt_T;
    double kdt_dxy, kdt_dz, kdt_dxy_water, kdt_dz_water, dt_rho_ct, dt_rho_ct_water;
} bdref_t_cfg;

/* Restates the launch loop of T:345-392 for given per-step shifts: one
 * Temperature_square per step, toggling use_p.  T_p, T_n, TD are updated in
 * place; *use_p_out gets the final flag (the latest field is T_n if it is 0). */
int bdref_t_run(const bdref_t_cfg* c, const double* Q, double* T_p, double* T_n, double* TD,
                const int32_t* sx, const int32_t* sy, int64_t n_steps, int32_t* use_p_out) {
    using namespace refT;
    dz = c->dz; water_tissue = c->water_tissue; dt_T = c->dt_T;
    kdt_dxy = c->kdt_dxy; kdt_dz = c->kdt_dz; kdt_dxy_water = c->kdt_dxy_water; kdt_dz_water = c->kdt_dz_water;
    dt_rho_ct = c->dt_rho_ct; dt_rho_ct_water = c->dt_rho_ct_water;
    const int Nxy = c->Nxy, Nz = c->Nz;
    Dim threads{8, 8, 8};
    Dim blocks{(unsigned)((Nxy + 7) / 8), (unsigned)((Nxy + 7) / 8), (unsigned)((Nz + 7) / 8)};
    bool use_p = true;
    double* Qm = const_cast<double*>(Q);
    for (int64_t s = 0; s < n_steps; ++s) {
        const int shx = sx[s], shy = sy[s];
        launch(blocks, threads, true, [&] { Temperature_square(T_n, T_p, Qm, TD, Nxy, Nz, use_p, shx, shy); });
        use_p = !use_p;
    }
    *use_p_out = use_p ? 1 : 0;
    return 0;
}

/* Constants of G:473-489. */
typedef struct bdref_g_cfg {
    double rho, P0, S2, mu4, G4_3, C_inf, lambda, n, B, gamma, gamma3;
    double minA, stepA, minR0, stepR0;
    int32_t triple_fr;
    int32_t pad0;
} bdref_g_cfg;

static void g_set(const bdref_g_cfg* c) {
    refG::rho = c->rho; refG::P0 = c->P0; refG::S2 = c->S2; refG::mu4 = c->mu4; refG::G4_3 = c->G4_3;
    refG::C_inf = c->C_inf; refG::lambda = c->lambda; refG::n = c->n; refG::B = c->B;
    refG::gamma1 = c->gamma; refG::gamma3 = c->gamma3; refG::triple_fr = c->triple_fr != 0;
    refG::minA = c->minA; refG::stepA = c->stepA; refG::minR0 = c->minR0; refG::stepR0 = c->stepR0;
}

/* One launch of DPRK_solver_threshold_fix_tissue (G:573) over n_combo*N_R0
 * threads, 128 per block. */
int bdref_g_threshold(const bdref_g_cfg* c, const double* fr_combo, int32_t n_combo, int32_t N_R0,
                      double* results) {
    g_set(c);
    const long N = (long)n_combo * N_R0;
    Dim threads{128, 1, 1};
    Dim blocks{(unsigned)((N + 127) / 128), 1, 1};
    double* fc = const_cast<double*>(fr_combo);
    launch(blocks, threads, true, [&] { refG::DPRK_solver_threshold_fix_tissue(results, fc, n_combo, N_R0, 0); });
    return 0;
}

/* Forward integration of bubbles with G's DPRK_step (G:212-318), the inner
 * loop of G:378-379 for a fixed amplitude: state[i*5..] = t, R, R', tau, q;
 * counts[i] = accepted steps; thr[i] = first time the threshold flag was set
 * (or -1).  max_steps bounds each bubble. */
int bdref_g_forward(const bdref_g_cfg* c, int64_t n, const double* R0, const double* A,
                    const double* f3, double endT, double h0, int64_t max_steps, int32_t stop_at_threshold,
                    double* state, int64_t* counts, double* thr) {
    g_set(c);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t i = 0; i < n; ++i) {
        double t = 0.0, R = R0[i], R1 = 0.0, Tau = 0.0, q = 0.0, h = h0;
        bool th = false;
        int64_t k = 0;
        double t_thr = -1.0;
        while (t < endT && k < max_steps) {
            refG::DPRK_step(t, R, R1, Tau, q, h, th, R0[i], A[i], f3[3 * i], f3[3 * i + 1], f3[3 * i + 2], endT);
            ++k;
            if (th && t_thr < 0) t_thr = t;
            if (th && stop_at_threshold) break;
        }
        state[5 * i] = t; state[5 * i + 1] = R; state[5 * i + 2] = R1; state[5 * i + 3] = Tau; state[5 * i + 4] = q;
        counts[i] = k;
        thr[i] = t_thr;
    }
    return 0;
}

}  // extern "C"
