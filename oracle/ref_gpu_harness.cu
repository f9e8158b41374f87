/*
 * ref_gpu_harness.cu — runs the reference's own CUDA kernels on the GPU.
 *
 * TEST / MEASUREMENT INFRASTRUCTURE ONLY (the reference-GPU baseline).
 * oracle/build.py extracts the kernel sections of the reference files (every
 * line before `int main()`) into oracle/_ref/src/; this file compiles them
 * unmodified with nvcc, each inside its own namespace, and restates the host
 * loops that drive them:
 *   - bdref_gpu_w_steps: the Westervelt time loop of W:558-585 —
 *     Westervelt_space6, boundary_condition_source, boundary_condition_space6
 *     on an (8, 8, 8)-thread grid (W:544-548) and the nine device-to-device
 *     copies of the level rotation — timed with CUDA events;
 *   - bdref_gpu_g_forward: one thread per bubble calling G's DPRK_step
 *     (G:212-318) until t reaches endT (the inner loop of G:378-379), with a
 *     per-bubble step cap.
 * Every access of those kernels stays inside the N = Nxy*Nxy*Nz arrays for
 * any Nxy, Nz >= 8: Westervelt_space6 updates iz in [3, Nz-4], ix, iy in
 * [0, Nxy-4] and mirrors indices below 0; the boundary kernels test ix, iy <
 * Nxy and iz < Nz (or the fixed planes 0..2, Nz-3..Nz-1) before every access.
 * boundary_condition_space6 reads Mur cells that other threads of the same
 * launch write, so the outer layers of W's own GPU result depend on thread
 * scheduling; the host build and this library use the serial order.
 */
#include <cuda_runtime.h>
#include <device_launch_parameters.h>
#include <cufft.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <stdint.h>
#include <fstream>
#include <iostream>

namespace refW {
#include "_ref/src/W_kernels.inc"
}
namespace refG {
#include "_ref/src/G_kernels.inc"
}

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

typedef struct bdref_g_cfg {
    double rho, P0, S2, mu4, G4_3, C_inf, lambda, n, B, gamma, gamma3;
    double minA, stepA, minR0, stepR0;
    int32_t triple_fr;
    int32_t pad0;
} bdref_g_cfg;

#define CK(x)                                                                          \
    do {                                                                               \
        cudaError_t e_ = (x);                                                          \
        if (e_ != cudaSuccess) {                                                       \
            fprintf(stderr, "ref_gpu_harness: %s: %s\n", #x, cudaGetErrorString(e_)); \
            return -1;                                                                 \
        }                                                                              \
    } while (0)

#define SETW(name, v) CK(cudaMemcpyToSymbol(refW::name, &(v), sizeof(double)))
#define SETG(name, v) CK(cudaMemcpyToSymbol(refG::name, &(v), sizeof(v)))

extern "C" {

/* Runs `warm` untimed then `n_steps` timed steps of W's loop; ms_out = timed
 * milliseconds.  state (optional, 12*N doubles on the host: P_next, P,
 * P_m1..P_m4, R1, R1m1, R1m2, R2, R2m1, R2m2) receives the final state; with
 * use_init it also supplies the initial state (else the state starts at 0). */
int bdref_gpu_w_steps(const bdref_w_cfg* c, int64_t warm, int64_t n_steps, double* ms_out, double* state,
                      int32_t use_init) {
    SETW(rho, c->rho); SETW(c_inf, c->c_inf); SETW(delta, c->delta); SETW(beta, c->beta);
    SETW(abs_water, c->abs_water); SETW(rho_tissue, c->rho_tissue); SETW(c_inf_tissue, c->c_inf_tissue);
    SETW(beta_tissue, c->beta_tissue); SETW(abs_tissue, c->abs_tissue); SETW(delta_tissue, c->delta_tissue);
    SETW(c1, c->c1); SETW(c2, c->c2); SETW(tau1, c->tau1); SETW(tau2, c->tau2);
    SETW(fr, c->fr); SETW(d, c->d); SETW(alpha, c->alpha); SETW(alpha_hole, c->alpha_hole); SETW(p0, c->p0);
    SETW(water_tissue, c->water_tissue); SETW(xy_min, c->xy_min); SETW(dxy, c->dxy); SETW(z_min, c->z_min);
    SETW(dz, c->dz); SETW(dt, c->dt);
    const int Nxy = c->Nxy, Nz = c->Nz;
    if (Nxy < 8 || Nz < 8) return -2;
    const size_t N = (size_t)Nxy * Nxy * Nz;
    double* S[12] = {};
    for (int k = 0; k < 12; ++k) {
        CK(cudaMalloc(&S[k], N * sizeof(double)));
        if (use_init && state) CK(cudaMemcpy(S[k], state + (size_t)k * N, N * sizeof(double), cudaMemcpyHostToDevice));
        else CK(cudaMemset(S[k], 0, N * sizeof(double)));
    }
    double *P_next = S[0], *P = S[1], *P_m1 = S[2], *P_m2 = S[3], *P_m3 = S[4], *P_m4 = S[5];
    double *R1 = S[6], *R1m1 = S[7], *R1m2 = S[8], *R2 = S[9], *R2m1 = S[10], *R2m2 = S[11];
    dim3 threads(8, 8, 8);
    dim3 blocks((Nxy + 7) / 8, (Nxy + 7) / 8, (Nz + 7) / 8);
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    double t = 0.0;
    const size_t B = N * sizeof(double);
    for (int64_t s = 0; s < warm + n_steps; ++s) {
        if (s == warm) CK(cudaEventRecord(e0));
        refW::Westervelt_space6<<<blocks, threads>>>(P_next, P, P_m1, P_m2, P_m3, P_m4, R1, R1m1, R1m2, R2, R2m1,
                                                     R2m2, Nxy, Nz);
        CK(cudaDeviceSynchronize());
        t = t + c->dt;
        refW::boundary_condition_source<<<blocks, threads>>>(P_next, t, Nxy, Nz);
        CK(cudaDeviceSynchronize());
        refW::boundary_condition_space6<<<blocks, threads>>>(P_next, P, t, Nxy, Nz);
        CK(cudaDeviceSynchronize());
        CK(cudaMemcpy(P_m4, P_m3, B, cudaMemcpyDeviceToDevice));
        CK(cudaMemcpy(P_m3, P_m2, B, cudaMemcpyDeviceToDevice));
        CK(cudaMemcpy(P_m2, P_m1, B, cudaMemcpyDeviceToDevice));
        CK(cudaMemcpy(P_m1, P, B, cudaMemcpyDeviceToDevice));
        CK(cudaMemcpy(P, P_next, B, cudaMemcpyDeviceToDevice));
        CK(cudaMemcpy(R1m2, R1m1, B, cudaMemcpyDeviceToDevice));
        CK(cudaMemcpy(R1m1, R1, B, cudaMemcpyDeviceToDevice));
        CK(cudaMemcpy(R2m2, R2m1, B, cudaMemcpyDeviceToDevice));
        CK(cudaMemcpy(R2m1, R2, B, cudaMemcpyDeviceToDevice));
    }
    CK(cudaEventRecord(e1));
    CK(cudaEventSynchronize(e1));
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    if (ms_out) *ms_out = ms;
    if (state)
        for (int k = 0; k < 12; ++k) CK(cudaMemcpy(state + (size_t)k * N, S[k], B, cudaMemcpyDeviceToHost));
    for (int k = 0; k < 12; ++k) cudaFree(S[k]);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return 0;
}

}  // extern "C"

__global__ void ref_g_forward_kernel(int64_t n, const double* R0, const double* A, const double* f3, double endT,
                                     double h0, int64_t max_steps, double* state, int64_t* counts) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double t = 0.0, R = R0[i], R1 = 0.0, Tau = 0.0, q = 0.0, h = h0;
    bool th = false;
    int64_t k = 0;
    while (t < endT && k < max_steps) {
        refG::DPRK_step(t, R, R1, Tau, q, h, th, R0[i], A[i], f3[3 * i], f3[3 * i + 1], f3[3 * i + 2], endT);
        ++k;
    }
    state[5 * i] = t; state[5 * i + 1] = R; state[5 * i + 2] = R1; state[5 * i + 3] = Tau; state[5 * i + 4] = q;
    counts[i] = k;
}

extern "C" {

/* One thread per bubble through G's DPRK_step from t = 0 to endT (at most
 * max_steps accepted steps each); state[5i..] = t, R, R', tau, q, counts[i] =
 * accepted steps; ms_out = kernel time. */
int bdref_gpu_g_forward(const bdref_g_cfg* c, int64_t n, const double* R0, const double* A, const double* f3,
                        double endT, double h0, int64_t max_steps, double* state, int64_t* counts, double* ms_out) {
    SETG(rho, c->rho); SETG(P0, c->P0); SETG(S2, c->S2); SETG(mu4, c->mu4); SETG(G4_3, c->G4_3);
    SETG(C_inf, c->C_inf); SETG(lambda, c->lambda); SETG(n, c->n); SETG(B, c->B);
    SETG(gamma1, c->gamma); SETG(gamma3, c->gamma3);
    const bool tf = c->triple_fr != 0;
    SETG(triple_fr, tf);
    SETG(minA, c->minA); SETG(stepA, c->stepA); SETG(minR0, c->minR0); SETG(stepR0, c->stepR0);
    if (n <= 0) return -2;
    double *dR0, *dA, *df, *ds;
    int64_t* dc;
    CK(cudaMalloc(&dR0, n * 8)); CK(cudaMalloc(&dA, n * 8)); CK(cudaMalloc(&df, 3 * n * 8));
    CK(cudaMalloc(&ds, 5 * n * 8)); CK(cudaMalloc(&dc, n * 8));
    CK(cudaMemcpy(dR0, R0, n * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dA, A, n * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(df, f3, 3 * n * 8, cudaMemcpyHostToDevice));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0));
    ref_g_forward_kernel<<<(unsigned)((n + 127) / 128), 128>>>(n, dR0, dA, df, endT, h0, max_steps, ds, dc);
    CK(cudaGetLastError());
    CK(cudaEventRecord(e1));
    CK(cudaEventSynchronize(e1));
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    if (ms_out) *ms_out = ms;
    CK(cudaMemcpy(state, ds, 5 * n * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(counts, dc, n * 8, cudaMemcpyDeviceToHost));
    cudaFree(dR0); cudaFree(dA); cudaFree(df); cudaFree(ds); cudaFree(dc);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return 0;
}

}  // extern "C"
