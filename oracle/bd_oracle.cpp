/*
 * bd_oracle.cpp — CPU restatement of the reference algorithms.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product links or calls this file;
 * it is imported by tests/, by __graft_entry__.smoke() and by the cpu_baseline
 * leg of bench.py, always as the reference answer or as the timed CPU baseline.
 *
 * It restates, in plain FP64 C++ (OpenMP over z planes / bubbles):
 *   - the Westervelt step of W:139-236 with the source of W:62-85, the Mur
 *     boundary of W:88-135 (applied in ascending cell order, the order a serial
 *     launch of that kernel gives), the water power of W:242-265 and the
 *     harmonic power of W:268-345 (the FFT replaced by the DFT at the bins the
 *     reference reads), generalised to per-cell c, N relaxation processes,
 *     sponge layers, bursts and phased arrays;
 *   - the bioheat + CEM43 step of T:52-105 (plus an optional Pennes term) and the
 *     square-spiral trajectory of T:141-173 / T:323-410;
 *   - the Gilmore-Zener right-hand side G:40-179, the Dormand-Prince step
 *     G:212-318 and the threshold search G:323-429.
 *
 * Its parity with the reference itself is pinned by tests that run the
 * reference's own kernel code compiled for the host (oracle/_ref).
 */
#include "../include/bubbledyn.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

inline size_t cidx(int ix, int iy, int iz, int nx, int ny) {
    return ((size_t)iz * ny + iy) * nx + ix;
}

/* ------------------------------------------------------------------------ */
/* Westervelt                                                                */
/* ------------------------------------------------------------------------ */

struct WvSetup {
    int nx, ny, nz;
    size_t ncell;
    std::vector<uint8_t> mat;
    std::vector<double> c;
    int xhi, yhi, zlo, zhi;
    int src_iz;
    bool mur_xp, mur_yp, mur_zp, mur_zm, mir_x, mir_y;
    int L, Lzm;
    std::vector<double> wx, wy, wz;
    std::vector<double> srcA, srcVar, srcTau;  /* per plane cell: p0*amp_e, var, delay */
    std::vector<double> srcPhi;                /* element phase */
    std::vector<int> srcOn;
    double tau_max;
    int max_relax;
};

bool wv_setup(const bd_grid* g, const bd_medium* m, const bd_source* s, WvSetup& S) {
    S.nx = g->nx; S.ny = g->ny; S.nz = g->nz;
    if (S.nx < 8 || S.ny < 8 || S.nz < 8) return false;
    S.ncell = (size_t)S.nx * S.ny * S.nz;
    S.mat.assign(S.ncell, 0);
    S.c.assign(S.ncell, 0.0);
    S.max_relax = 0;
    for (int k = 0; k < m->n_materials; ++k) S.max_relax = std::max(S.max_relax, (int)m->mat[k].n_relax);
    for (int iz = 0; iz < S.nz; ++iz)
        for (int iy = 0; iy < S.ny; ++iy)
            for (int ix = 0; ix < S.nx; ++ix) {
                size_t i = cidx(ix, iy, iz, S.nx, S.ny);
                int mm = 0;
                if (m->material_map) mm = m->material_map[i];
                else if (m->plane_material) mm = m->plane_material[iz];
                S.mat[i] = (uint8_t)mm;
                S.c[i] = m->c_map ? (double)m->c_map[i] : m->mat[mm].c0;
            }
    S.mir_x = g->face[0] == BD_FACE_MIRROR;
    S.mir_y = g->face[2] == BD_FACE_MIRROR;
    S.mur_xp = g->face[1] == BD_FACE_MUR;
    S.mur_yp = g->face[3] == BD_FACE_MUR;
    S.mur_zm = g->face[4] == BD_FACE_MUR;
    S.mur_zp = g->face[5] == BD_FACE_MUR;
    S.L = g->mur_layers;
    S.src_iz = (s && s->kind != BD_SRC_NONE) ? s->plane_iz : -1;
    S.Lzm = S.mur_zm ? (S.src_iz >= 0 ? S.src_iz : S.L) : 0;
    S.xhi = S.mur_xp ? S.nx - 1 - S.L : S.nx - 1;
    S.yhi = S.mur_yp ? S.ny - 1 - S.L : S.ny - 1;
    S.zlo = S.Lzm;
    S.zhi = S.mur_zp ? S.nz - 1 - S.L : S.nz - 1;
    auto sponge = [&](int n, int lo_face, int hi_face, std::vector<double>& w) {
        w.assign(n, 1.0);
        int W = g->sponge_cells;
        if (W <= 0) return;
        for (int i = 0; i < n; ++i) {
            double f = 1.0;
            if (lo_face == BD_FACE_OPEN && i < W) {
                double d = (double)(W - i) / W;
                f *= std::exp(-g->sponge_strength * d * d);
            }
            if (hi_face == BD_FACE_OPEN && i >= n - W) {
                double d = (double)(i - (n - W) + 1) / W;
                f *= std::exp(-g->sponge_strength * d * d);
            }
            w[i] = f;
        }
    };
    sponge(S.nx, g->face[0], g->face[1], S.wx);
    sponge(S.ny, g->face[2], g->face[3], S.wy);
    sponge(S.nz, g->face[4], g->face[5], S.wz);
    size_t np = (size_t)S.nx * S.ny;
    S.srcA.assign(np, 0.0); S.srcVar.assign(np, 1.0); S.srcTau.assign(np, 0.0);
    S.srcPhi.assign(np, 0.0); S.srcOn.assign(np, 0);
    S.tau_max = 0.0;
    if (s && s->kind != BD_SRC_NONE) {
        const double d = s->focal_length;
        for (int iy = 0; iy < S.ny; ++iy)
            for (int ix = 0; ix < S.nx; ++ix) {
                size_t j = (size_t)iy * S.nx + ix;
                double X = g->x0 + ix * g->dx - s->cx;   /* W:72 */
                double Y = g->y0 + iy * g->dx - s->cy;   /* W:73 */
                double r = std::sqrt(X * X + Y * Y);      /* W:74 */
                if (r <= d * std::tan(s->alpha) && r >= d * std::tan(s->alpha_hole)) {  /* W:78 */
                    double var = std::sqrt(1.0 + std::pow(r / d, 2));                    /* W:80 */
                    double amp = s->p0, phi = 0.0;
                    if (s->kind == BD_SRC_ARRAY) {
                        int e = s->element_of_cell ? s->element_of_cell[j] : -1;
                        if (e < 0 || e >= s->n_elements) continue;
                        amp *= s->element_amp ? s->element_amp[e] : 1.0;
                        phi = s->element_phase ? s->element_phase[e] : 0.0;
                    }
                    S.srcOn[j] = 1;
                    S.srcA[j] = amp;
                    S.srcVar[j] = var;
                    S.srcTau[j] = d * (var - 1.0) / s->c_delay;                            /* W:81 */
                    S.srcPhi[j] = phi;
                    S.tau_max = std::max(S.tau_max, S.srcTau[j]);
                }
            }
    }
    return true;
}

template <class T>
struct WvRun {
    const bd_grid* g;
    const bd_medium* m;
    const bd_source* s;
    const bd_westervelt_params* p;
    WvSetup S;
    std::vector<T> P[5];           /* ring: lvl(k) = p^{n-k} */
    int head = 0;                  /* buffer index of p^n */
    std::vector<T> R[BD_MAX_RELAX][2];
    int rhead = 0;                 /* buffer index of R^{n-1}; the other holds R^{n-2} */
    std::vector<T> peak, energy;
    std::vector<double> dre, dim;  /* DFT accumulators (double on the host) */
    size_t dplane = 0;
    int dz_lo = 0, dz_hi = 0;

    T& lvl(int k, size_t i) { return P[(head + k) % 5][i]; }

    double ghost_or(const std::vector<T>& f, int ix, int iy, int iz) const {
        if (ix < 0) { if (S.mir_x) ix = -ix; else return 0.0; }
        if (iy < 0) { if (S.mir_y) iy = -iy; else return 0.0; }
        if (iz < 0 || ix >= S.nx || iy >= S.ny || iz >= S.nz) return 0.0;
        return (double)f[cidx(ix, iy, iz, S.nx, S.ny)];
    }

    double source_value(size_t j, double t) const {
        if (!S.srcOn[j]) return 0.0;
        double tt = t + S.srcTau[j];                          /* W:81 */
        if (s->burst_cycles > 0.0) {
            double tb = tt - S.tau_max;
            if (tb < 0.0 || tb >= s->burst_cycles / s->freq[0]) return 0.0;
            tt = tb;
        }
        double sum = 0.0;
        for (int k = 0; k < s->n_tones; ++k)
            sum += s->amp[k] * std::sin(2 * M_PI * s->freq[k] * tt + s->phase[k] + S.srcPhi[j]);
        return S.srcA[j] * sum / S.srcVar[j];                 /* W:82 */
    }

    void init() {
        for (auto& v : P) v.assign(S.ncell, (T)0);
        for (int v = 0; v < S.max_relax; ++v)
            for (auto& r : R[v]) r.assign(S.ncell, (T)0);
        peak.assign(S.ncell, (T)0);
        energy.assign(S.ncell, (T)0);
        if (p->n_dft > 0) {
            dz_lo = std::max(0, p->dft_z_lo);
            dz_hi = std::min(S.nz, p->dft_z_hi);
            dplane = (size_t)S.nx * S.ny;
            size_t nd = (size_t)p->n_dft * dplane * std::max(0, dz_hi - dz_lo);
            dre.assign(nd, 0.0); dim.assign(nd, 0.0);
        }
    }

    /* One time step s (0-based) at source time t. */
    void step(int64_t s_idx, double t) {
        const int nx = S.nx, ny = S.ny, nz = S.nz;
        const double dt = g->dt;
        const int nb = (head + 4) % 5;  /* buffer receiving p^{n+1} (held p^{n-4}) */
        std::vector<T>& Pn = P[head];
        std::vector<T> Pnew(S.ncell);   /* written into P[nb] at the end */
        /* interior update W:139-236 */
#pragma omp parallel for schedule(static)
        for (int iz = 0; iz < nz; ++iz) {
            for (int iy = 0; iy < ny; ++iy)
                for (int ix = 0; ix < nx; ++ix) {
                    size_t i = cidx(ix, iy, iz, nx, ny);
                    if (iz == S.src_iz || iz < S.zlo || iz > S.zhi || ix > S.xhi || iy > S.yhi) {
                        Pnew[i] = Pn[i];   /* placeholder, overwritten by source / Mur */
                        continue;
                    }
                    /* W:203-234 in the reference's operation order, arithmetic in T */
                    const T pc = Pn[i];
                    auto gx = [&](int o) { return (T)ghost_or(Pn, ix + o, iy, iz); };
                    auto gy = [&](int o) { return (T)ghost_or(Pn, ix, iy + o, iz); };
                    auto gz = [&](int o) { return (T)ghost_or(Pn, ix, iy, iz + o); };
                    const T c490 = (T)-490.0, c270 = (T)270.0, c27 = (T)27.0, c2 = (T)2.0, c180 = (T)180.0;
                    T Dxx = (c490 * pc + c270 * (gx(1) + gx(-1)) - c27 * (gx(2) + gx(-2)) + c2 * (gx(3) + gx(-3))) / c180;
                    T Dyy = (c490 * pc + c270 * (gy(1) + gy(-1)) - c27 * (gy(2) + gy(-2)) + c2 * (gy(3) + gy(-3))) / c180;
                    T Dzz = (c490 * pc + c270 * (gz(1) + gz(-1)) - c27 * (gz(2) + gz(-2)) + c2 * (gz(3) + gz(-3))) / c180;
                    const T p1 = lvl(1, i), p2 = lvl(2, i), p3 = lvl(3, i), p4 = lvl(4, i);
                    T Dttt = (T)5.0 * pc - (T)18.0 * p1 + (T)24.0 * p2 - (T)14.0 * p3 + (T)3.0 * p4;   /* W:207 */
                    T D1 = (T)std::pow(3.0 * pc - 4.0 * p1 + p2, 2) / (T)4.0;                            /* W:208 */
                    if (sizeof(T) == 4) { T a = (T)3.0 * pc - (T)4.0 * p1 + p2; D1 = a * a / (T)4.0; }
                    T D2 = pc * ((T)2.0 * pc - (T)5.0 * p1 + (T)4.0 * p2 - p3);                          /* W:209 */
                    const bd_material& mt = m->mat[S.mat[i]];
                    const double c = S.c[i], dt_ = g->dt;
                    const T c2dt2_dxy2 = (T)std::pow(c * dt_ / g->dx, 2);                                 /* W:214 */
                    const T c2dt2_dz2 = (T)std::pow(c * dt_ / g->dz, 2);                                  /* W:215 */
                    const T delta_2dtc2 = (T)(mt.delta / (2.0 * dt_ * std::pow(c, 2)));                   /* W:216 */
                    const T beta2_rhoc2 = (T)(2.0 * mt.beta / (mt.rho * std::pow(c, 2)));                 /* W:217 */
                    T sum_R = (T)0.0;
                    T pn;
                    if (mt.n_relax > 0 && p->relax_scheme == BD_RELAX_SEMI_IMPLICIT) {
                        /* R_v = a_v (3 p^{n+1} + E) + b_v (4 R1 - R2), E = -10 p + 12 p1 - 6 p2 + p3
                         * (2nd-order d3p/dt3 at t_n times 2 dt^3), p^{n+1} = Y + (c dt)^2 sum R_v, solved */
                        const T E = (T)-10.0 * pc + (T)12.0 * p1 - (T)6.0 * p2 + p3;
                        const T kr = (T)std::pow(c * dt_, 2);
                        T sa = (T)0.0, G = (T)0.0;
                        T av[BD_MAX_RELAX], bv[BD_MAX_RELAX];
                        for (int v = 0; v < mt.n_relax; ++v) {
                            const double tau = mt.relax_tau[v], cv = mt.relax_c[v];
                            av[v] = (T)((2.0 * dt_ * 2.0 * cv * tau) / (2.0 * std::pow(dt_, 3)) / ((2.0 * dt_ + 3.0 * tau) * std::pow(c, 3)));
                            const T r1 = R[v][rhead][i], r2 = R[v][rhead ^ 1][i];
                            bv[v] = (T)(tau / (2.0 * dt_ + 3.0 * tau)) * ((T)4.0 * r1 - r2);
                            sa += av[v];
                            G += av[v] * E + bv[v];
                        }
                        const T Y = (T)2.0 * pc - p1 + c2dt2_dxy2 * (Dxx + Dyy) + c2dt2_dz2 * Dzz + delta_2dtc2 * Dttt
                                  + beta2_rhoc2 * (D1 + D2);
                        pn = (Y + kr * G) / ((T)1.0 - (T)3.0 * kr * sa);
                        for (int v = 0; v < mt.n_relax; ++v) R[v][rhead ^ 1][i] = av[v] * ((T)3.0 * pn + E) + bv[v];
                    } else {
                    if (mt.n_relax > 0) {
                        T Dttt_2dt = Dttt / (T)(2.0 * std::pow(dt_, 3));                                  /* W:226 */
                        T sR = (T)0.0;
                        for (int v = 0; v < mt.n_relax; ++v) {
                            const double tau = mt.relax_tau[v], cv = mt.relax_c[v];
                            T& Rn = R[v][rhead ^ 1][i];          /* the R^{n-2} buffer receives R^n */
                            const T r1 = R[v][rhead][i], r2 = Rn;
                            T rn = ((T)(2.0 * dt_ * 2.0 * cv * tau) * Dttt_2dt / (T)((2.0 * dt_ + 3.0 * tau) * std::pow(c, 3)))
                                 + (((T)tau * ((T)4.0 * r1 - r2)) / (T)(2.0 * dt_ + 3.0 * tau));             /* W:227-228 */
                            Rn = rn;
                            sR = (v == 0) ? Rn : sR + Rn;
                        }
                        sum_R = sR * (T)std::pow(c * dt_, 2);                                               /* W:230 */
                    }
                    pn = (T)2.0 * pc - p1 + c2dt2_dxy2 * (Dxx + Dyy) + c2dt2_dz2 * Dzz + delta_2dtc2 * Dttt
                         + beta2_rhoc2 * (D1 + D2) + sum_R;                                                 /* W:234 */
                    }
                    const double w = S.wx[ix] * S.wy[iy] * S.wz[iz];
                    if (w != 1.0) pn = pn * (T)w;
                    Pnew[i] = pn;
                }
        }
        /* source plane W:62-85 */
        if (S.src_iz >= 0) {
            for (int iy = 0; iy < ny; ++iy)
                for (int ix = 0; ix < nx; ++ix)
                    Pnew[cidx(ix, iy, S.src_iz, nx, ny)] = (T)source_value((size_t)iy * nx + ix, t);
        }
        /* Mur W:88-135, ascending linear order: the final value of a cell is set by the
         * last condition that applies (z-, z+, x+, y+); reads of the -1 neighbour see
         * final values, the z- read of the +1 neighbour sees its pre-boundary value,
         * which in W is p^n because of the copy rotation W:575-579. */
        auto kmur = [&](double c, double h) { double a = c * dt / h; return (a - 1.0) / (a + 1.0); };
        if (S.mur_zm || S.mur_zp || S.mur_xp || S.mur_yp) {
            for (int iz = 0; iz < nz; ++iz)
                for (int iy = 0; iy < ny; ++iy)
                    for (int ix = 0; ix < nx; ++ix) {
                        size_t i = cidx(ix, iy, iz, nx, ny);
                        const double pc = Pn[i];
                        if (S.mur_yp && iy >= ny - S.L) {
                            size_t jn = cidx(ix, iy - 1, iz, nx, ny);
                            Pnew[i] = (T)(Pn[jn] + ((double)Pnew[jn] - pc) * (S.c[i] * dt / g->dx - 1.0) / (S.c[i] * dt / g->dx + 1.0));
                        } else if (S.mur_xp && ix >= nx - S.L) {
                            size_t jn = cidx(ix - 1, iy, iz, nx, ny);
                            Pnew[i] = (T)(Pn[jn] + ((double)Pnew[jn] - pc) * (S.c[i] * dt / g->dx - 1.0) / (S.c[i] * dt / g->dx + 1.0));
                        } else if (S.mur_zp && iz >= nz - S.L) {
                            size_t jn = cidx(ix, iy, iz - 1, nx, ny);
                            Pnew[i] = (T)(Pn[jn] + ((double)Pnew[jn] - pc) * (S.c[i] * dt / g->dz - 1.0) / (S.c[i] * dt / g->dz + 1.0));
                        } else if (S.mur_zm && iz < S.Lzm) {
                            size_t jn = cidx(ix, iy, iz + 1, nx, ny);
                            double nbv = (iz + 1 < S.Lzm) ? (double)Pn[jn] : (double)Pnew[jn];
                            Pnew[i] = (T)(Pn[jn] + (nbv - pc) * (S.c[i] * dt / g->dz - 1.0) / (S.c[i] * dt / g->dz + 1.0));
                        }
                    }
        }
        (void)kmur;
        /* accumulators on the final p^{n+1} */
        const bool do_peak = s_idx >= p->peak_start && s_idx < p->peak_end;
        const bool do_en = s_idx >= p->energy_start && s_idx < p->energy_end;
        const int64_t ds = s_idx - p->dft_start;
        const bool do_dft = p->n_dft > 0 && ds >= 0 && ds < p->dft_len;
        std::vector<double> tc, ts;
        if (do_dft) {
            for (int j = 0; j < p->n_dft; ++j) {
                double th = 2.0 * M_PI * p->dft_freq[j] * ((double)ds * dt);
                tc.push_back(std::cos(th)); ts.push_back(std::sin(th));
            }
        }
        std::vector<T>& Pm1 = P[(head + 1) % 5];
#pragma omp parallel for schedule(static)
        for (int iz = 0; iz < nz; ++iz)
            for (int iy = 0; iy < ny; ++iy)
                for (int ix = 0; ix < nx; ++ix) {
                    size_t i = cidx(ix, iy, iz, nx, ny);
                    double v = Pnew[i];
                    if (do_peak) peak[i] = (T)std::max((double)peak[i], std::fabs(v));
                    if (do_en) {
                        if (p->energy_mode == BD_ENERGY_DPDT2) {
                            double dp = (v - (double)Pm1[i]) / (2.0 * dt);     /* W:253 */
                            energy[i] = (T)((double)energy[i] + std::pow(dp, 2) * dt);  /* W:257 */
                        } else {
                            energy[i] = (T)((double)energy[i] + v * v * dt);
                        }
                    }
                    if (do_dft && iz >= dz_lo && iz < dz_hi) {
                        size_t pl = (size_t)(iz - dz_lo) * dplane + (size_t)iy * nx + ix;
                        size_t stride = dplane * (dz_hi - dz_lo);
                        for (int j = 0; j < p->n_dft; ++j) {
                            dre[j * stride + pl] += v * tc[j];
                            dim[j * stride + pl] -= v * ts[j];
                        }
                    }
                }
        P[nb].swap(Pnew);
        head = nb;
        rhead ^= 1;
    }
};

template <class T>
bd_status wv_run(const bd_grid* g, const bd_medium* m, const bd_source* s,
                 const bd_westervelt_params* p, bd_westervelt_outputs* o) {
    WvRun<T> W;
    W.g = g; W.m = m; W.s = s; W.p = p;
    if (!wv_setup(g, m, s, W.S)) return BD_ERR_INVALID_ARG;
    W.init();
    for (int64_t st = 0; st < p->n_steps; ++st) {
        double t = p->t_src ? p->t_src[st] : p->t0 + (double)(st + 1) * g->dt;
        W.step(st, t);
    }
    const size_t n = W.S.ncell;
    if (o->p_final) for (size_t i = 0; i < n; ++i) ((T*)o->p_final)[i] = W.P[W.head][i];
    if (o->peak) for (size_t i = 0; i < n; ++i) ((T*)o->peak)[i] = W.peak[i];
    if (o->energy) for (size_t i = 0; i < n; ++i) ((T*)o->energy)[i] = W.energy[i];
    if (o->dft_re && p->n_dft > 0)
        for (size_t i = 0; i < W.dre.size(); ++i) { ((T*)o->dft_re)[i] = (T)W.dre[i]; ((T*)o->dft_im)[i] = (T)W.dim[i]; }
    if (o->Q && p->q_mode == BD_Q_REFERENCE) {
        const int nx = g->nx, ny = g->ny, nz = g->nz;
        const double f = p->q_freq;
        const size_t stride = W.dplane * (size_t)std::max(0, W.dz_hi - W.dz_lo);
        for (int iz = 0; iz < nz; ++iz)
            for (int iy = 0; iy < ny; ++iy)
                for (int ix = 0; ix < nx; ++ix) {
                    size_t i = cidx(ix, iy, iz, nx, ny);
                    const bd_material& mt = m->mat[W.S.mat[i]];
                    const double c = W.S.c[i];
                    double q = 0.0;
                    if (iz >= p->q_iz_split) {
                        if (iz >= W.dz_lo && iz < W.dz_hi) {
                            size_t pl = (size_t)(iz - W.dz_lo) * W.dplane + (size_t)iy * nx + ix;
                            for (int h = 1; h <= p->q_n_harm && h <= p->n_dft; ++h) {    /* W:339-343 */
                                double re = W.dre[(h - 1) * stride + pl], im = W.dim[(h - 1) * stride + pl];
                                double a = std::sqrt(re * re + im * im) / (double)p->dft_len;   /* W:299 */
                                double In = 2.0 * std::pow(a, 2) / (mt.rho * c);
                                q = q + (2.0 * (mt.harm_absorption * h * f / std::pow(10.0, 6)) * In);
                            }
                        }
                    } else {
                        q = 2.0 * mt.absorption * f * (double)W.energy[i] / (std::pow(2.0 * M_PI * f, 2) * mt.rho * c);  /* W:261 */
                    }
                    o->Q[i] = q;
                }
    }
    o->steps_done = p->n_steps;
    return BD_OK;
}

/* Discrete adjoint of wv_run<double> for OPEN faces (no reference
 * counterpart; the forward model is W:139-236 with the source of W:62-85).
 * Written in scatter form: every forward operation, visited in reverse,
 * pushes its output adjoint onto its inputs.  All forward time levels are
 * kept (small grids only), so no checkpointing is involved.  Loss:
 * L = sum_x w(x) E(x), E the p^2 dt energy over the loss window, w = -1 in the
 * focal ball, side_weight on the focal plane outside side_radius. */
bd_status wv_adjoint(const bd_grid* g, const bd_medium* m, const bd_source* s, const bd_westervelt_params* p0,
                     const bd_focal_loss* loss, double* loss_out, double* grad_phase, double* grad_amp) {
    for (int f = 0; f < 6; ++f)
        if (g->face[f] != BD_FACE_OPEN) return BD_ERR_UNSUPPORTED;
    if (!s || s->kind != BD_SRC_ARRAY) return BD_ERR_INVALID_ARG;
    bd_westervelt_params p = *p0;
    p.energy_mode = BD_ENERGY_P2;
    p.energy_start = loss->window_start;
    p.energy_end = loss->window_end;
    p.peak_start = p.peak_end = 0;
    p.n_dft = 0;
    WvRun<double> W;
    W.g = g; W.m = m; W.s = s; W.p = &p;
    if (!wv_setup(g, m, s, W.S)) return BD_ERR_INVALID_ARG;
    W.init();
    const WvSetup& S = W.S;
    const int nx = S.nx, ny = S.ny, nz = S.nz;
    const size_t n = S.ncell;
    const int64_t N = p.n_steps;
    const double dt = g->dt;
    std::vector<std::vector<double>> hist(N + 1);   /* hist[t] = p^t */
    std::vector<double> tsrc(N);
    hist[0].assign(n, 0.0);
    for (int64_t st = 0; st < N; ++st) {
        tsrc[st] = p.t_src ? p.t_src[st] : p.t0 + (double)(st + 1) * dt;
        W.step(st, tsrc[st]);
        hist[st + 1] = W.P[W.head];
    }
    auto wloss = [&](int ix, int iy, int iz) {
        const int dx = ix - loss->focus_ix, dy = iy - loss->focus_iy, dz = iz - loss->focus_iz;
        const int r2 = dx * dx + dy * dy + dz * dz;
        if (r2 <= loss->focal_radius * loss->focal_radius) return -1.0;
        if (iz == loss->focus_iz && r2 >= loss->side_radius * loss->side_radius) return loss->side_weight;
        return 0.0;
    };
    double L = 0.0;
    for (int iz = 0; iz < nz; ++iz)
        for (int iy = 0; iy < ny; ++iy)
            for (int ix = 0; ix < nx; ++ix) L += wloss(ix, iy, iz) * W.energy[cidx(ix, iy, iz, nx, ny)];
    if (loss_out) *loss_out = L;
    /* adjoints of every level: ap[t] for p^t (t = 0..N), ar[v][t + 2] for R^t (t = -2..N-1) */
    std::vector<std::vector<double>> ap(N + 1, std::vector<double>(n, 0.0));
    const int NR = S.max_relax;
    std::vector<std::vector<double>> ar[BD_MAX_RELAX];
    for (int v = 0; v < NR; ++v) ar[v].assign(N + 2, std::vector<double>(n, 0.0));
    const size_t np = (size_t)nx * ny;
    std::vector<double> gphi(np, 0.0), gamp(np, 0.0);
    const double coef[4] = {-490.0, 270.0, -27.0, 2.0};
    auto lev = [&](int64_t t, size_t i) { return t >= 0 ? hist[t][i] : 0.0; };
    for (int64_t st = N - 1; st >= 0; --st) {
        std::vector<double>& A = ap[st + 1];          /* complete: later steps were visited first */
        if (st >= loss->window_start && st < loss->window_end)
            for (int iz = 0; iz < nz; ++iz)
                for (int iy = 0; iy < ny; ++iy)
                    for (int ix = 0; ix < nx; ++ix) {
                        const size_t i = cidx(ix, iy, iz, nx, ny);
                        A[i] += 2.0 * wloss(ix, iy, iz) * hist[st + 1][i] * dt;
                    }
        auto push = [&](int64_t t, size_t i, double v) { if (t >= 0) ap[t][i] += v; };
        for (int iz = 0; iz < nz; ++iz)
            for (int iy = 0; iy < ny; ++iy)
                for (int ix = 0; ix < nx; ++ix) {
                    const size_t i = cidx(ix, iy, iz, nx, ny);
                    const double gout = A[i];
                    if (iz == S.src_iz) {
                        /* S_j(t) = A_j sum_k a_k sin(2 pi f_k tt + phi_k + phi_e) / var_j */
                        const size_t j = (size_t)iy * nx + ix;
                        if (!S.srcOn[j]) continue;
                        double tt = tsrc[st] + S.srcTau[j];
                        if (s->burst_cycles > 0.0) {
                            const double tb = tt - S.tau_max;
                            if (tb < 0.0 || tb >= s->burst_cycles / s->freq[0]) continue;
                            tt = tb;
                        }
                        double sn = 0.0, cs = 0.0;
                        for (int k = 0; k < s->n_tones; ++k) {
                            const double ang = 2 * M_PI * s->freq[k] * tt + s->phase[k] + S.srcPhi[j];
                            sn += s->amp[k] * std::sin(ang);
                            cs += s->amp[k] * std::cos(ang);
                        }
                        gphi[j] += gout * S.srcA[j] * cs / S.srcVar[j];
                        const int e = s->element_of_cell[j];
                        const double ae = s->element_amp ? s->element_amp[e] : 1.0;
                        if (ae != 0.0) gamp[j] += gout * S.srcA[j] * sn / S.srcVar[j] / ae;
                        continue;
                    }
                    const bd_material& mt = m->mat[S.mat[i]];
                    const double c = S.c[i];
                    const double w = S.wx[ix] * S.wy[iy] * S.wz[iz];
                    const double gpn = gout * w;                  /* p^{s+1} = w pn */
                    const double kxy = std::pow(c * dt / g->dx, 2) / 180.0, kz = std::pow(c * dt / g->dz, 2) / 180.0;
                    const double kd = mt.delta / (2.0 * dt * c * c), kn = 2.0 * mt.beta / (mt.rho * c * c);
                    const double kr = std::pow(c * dt, 2);
                    const double P0 = lev(st, i), P1 = lev(st - 1, i), P2 = lev(st - 2, i), P3 = lev(st - 3, i);
                    double gY = 0.0, gDttt = 0.0, gE = 0.0;
                    if (mt.n_relax > 0 && p.relax_scheme == BD_RELAX_SEMI_IMPLICIT) {
                        double av[BD_MAX_RELAX], bc[BD_MAX_RELAX], sa = 0.0, g_pn = gpn;
                        for (int v = 0; v < mt.n_relax; ++v) {
                            const double tau = mt.relax_tau[v], cv = mt.relax_c[v];
                            av[v] = (2.0 * dt * 2.0 * cv * tau) / (2.0 * dt * dt * dt) / ((2.0 * dt + 3.0 * tau) * c * c * c);
                            bc[v] = tau / (2.0 * dt + 3.0 * tau);
                            sa += av[v];
                            g_pn += 3.0 * av[v] * ar[v][st + 2][i];       /* R^s = a (3 pn + E) + b B */
                        }
                        const double den = 1.0 - 3.0 * kr * sa;      /* pn = (Y + kr G) / den */
                        gY = g_pn / den;
                        const double gG = g_pn * kr / den;
                        for (int v = 0; v < mt.n_relax; ++v) {
                            const double gR = ar[v][st + 2][i];
                            gE += av[v] * (gG + gR);
                            const double gB = bc[v] * (gG + gR);      /* B = 4 R^{s-1} - R^{s-2} */
                            ar[v][st + 1][i] += 4.0 * gB;
                            ar[v][st][i] -= gB;
                        }
                        gDttt = kd * gY;
                    } else {
                        gY = gpn;
                        gDttt = kd * gpn;
                        for (int v = 0; v < mt.n_relax; ++v) {
                            const double tau = mt.relax_tau[v], cv = mt.relax_c[v];
                            const double ra = (2.0 * dt * 2.0 * cv * tau) / (2.0 * dt * dt * dt) / ((2.0 * dt + 3.0 * tau) * c * c * c);
                            const double rb = tau / (2.0 * dt + 3.0 * tau);
                            const double gR = ar[v][st + 2][i] + kr * gpn;   /* pn = Y + kr sum R */
                            gDttt += ra * gR;
                            ar[v][st + 1][i] += 4.0 * rb * gR;
                            ar[v][st][i] -= rb * gR;
                        }
                    }
                    /* Y = 2 P0 - P1 + Lap(P0) + kd Dttt + kn (D1 + D2) */
                    push(st, i, 2.0 * gY);
                    push(st - 1, i, -gY);
                    for (int o = -3; o <= 3; ++o) {
                        const double cf = coef[o < 0 ? -o : o];
                        auto nb = [&](int jx, int jy, int jz, double k) {
                            if (jx < 0 || jy < 0 || jz < 0 || jx >= nx || jy >= ny || jz >= nz) return;
                            push(st, cidx(jx, jy, jz, nx, ny), k * cf * gY);
                        };
                        nb(ix + o, iy, iz, kxy);
                        nb(ix, iy + o, iz, kxy);
                        nb(ix, iy, iz + o, kz);
                    }
                    const double s3 = 3.0 * P0 - 4.0 * P1 + P2;
                    const double gN = kn * gY;                   /* D1 = s3^2 / 4, D2 = P0 (2P0 - 5P1 + 4P2 - P3) */
                    push(st, i, gN * (0.5 * s3 * 3.0 + (2.0 * P0 - 5.0 * P1 + 4.0 * P2 - P3) + 2.0 * P0));
                    push(st - 1, i, gN * (0.5 * s3 * -4.0 - 5.0 * P0));
                    push(st - 2, i, gN * (0.5 * s3 + 4.0 * P0));
                    push(st - 3, i, gN * -P0);
                    /* Dttt = 5 P0 - 18 P1 + 24 P2 - 14 P3 + 3 P4; E = -10 P0 + 12 P1 - 6 P2 + P3 */
                    push(st, i, 5.0 * gDttt - 10.0 * gE);
                    push(st - 1, i, -18.0 * gDttt + 12.0 * gE);
                    push(st - 2, i, 24.0 * gDttt - 6.0 * gE);
                    push(st - 3, i, -14.0 * gDttt + gE);
                    push(st - 4, i, 3.0 * gDttt);
                }
    }
    const int ne = s->n_elements;
    for (int e = 0; e < ne; ++e) {
        if (grad_phase) grad_phase[e] = 0.0;
        if (grad_amp) grad_amp[e] = 0.0;
    }
    for (size_t j = 0; j < np; ++j) {
        if (!S.srcOn[j]) continue;
        const int e = s->element_of_cell[j];
        if (grad_phase) grad_phase[e] += gphi[j];
        if (grad_amp) grad_amp[e] += gamp[j];
    }
    return BD_OK;
}

/* ------------------------------------------------------------------------ */
/* Heat + CEM43 (T:52-105)                                                   */
/* ------------------------------------------------------------------------ */

struct HeatCoef { double kxy, kz, q, w, Ta; };

}  // namespace

extern "C" {

int bdo_omp_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void bdo_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

bd_status bdo_westervelt_run(const bd_grid* g, const bd_medium* m, const bd_source* s,
                             const bd_westervelt_params* p, bd_westervelt_outputs* o) {
    if (p->precision == BD_F32) return wv_run<float>(g, m, s, p, o);
    return wv_run<double>(g, m, s, p, o);
}

bd_status bdo_westervelt_adjoint(const bd_grid* g, const bd_medium* m, const bd_source* s,
                                 const bd_westervelt_params* p, const bd_focal_loss* loss, double* loss_out,
                                 double* grad_phase, double* grad_amp) {
    return wv_adjoint(g, m, s, p, loss, loss_out, grad_phase, grad_amp);
}

/* Heat run: T:52-105 per step with the Q shift of each step; FP64 T and dose.
 * T_io holds the initial temperature on entry and the final one on exit; TD_io
 * likewise for the dose.  snap (optional) receives T after each step listed in
 * snap_steps (ascending).  Pennes term: -w dt (T - T_art). */
bd_status bdo_heat_run(const bd_thermal* th, const double* Q, const int32_t* sx, const int32_t* sy,
                       int64_t n_steps, double* T_io, double* TD_io,
                       const int64_t* snap_steps, int32_t n_snap, double* snap) {
    const int nx = th->nx, ny = th->ny, nz = th->nz;
    const size_t n = (size_t)nx * ny * nz;
    std::vector<double> Ta(T_io, T_io + n), Tb(T_io, T_io + n);
    std::vector<HeatCoef> hc(th->n_materials);
    for (int k = 0; k < th->n_materials; ++k) {
        const bd_thermal_material& mt = th->mat[k];
        double kk = mt.k_t / (mt.rho * mt.c_t);                  /* T:129, T:136 */
        hc[k].kxy = th->dt * kk / (th->dx * th->dx);              /* T:212 */
        hc[k].kz = th->dt * kk / (th->dz * th->dz);               /* T:213 */
        hc[k].q = th->dt / (mt.rho * mt.c_t);                     /* T:216 */
        hc[k].w = mt.perfusion * th->dt;
        hc[k].Ta = mt.T_art;
    }
    bool use_p = true;  /* T:323 */
    int isnap = 0;
    for (int64_t st = 0; st < n_steps; ++st) {
        std::vector<double>& src = use_p ? Ta : Tb;   /* T_p when use_p */
        std::vector<double>& dst = use_p ? Tb : Ta;   /* T_n when use_p */
        const int shx = sx[st], shy = sy[st];
#pragma omp parallel for schedule(static)
        for (int iz = 1; iz < nz - 1; ++iz)
            for (int iy = 1; iy < ny - 1; ++iy)
                for (int ix = 1; ix < nx - 1; ++ix) {
                    size_t i = cidx(ix, iy, iz, nx, ny);
                    int mm = th->material_map ? th->material_map[i] : (th->plane_material ? th->plane_material[iz] : 0);
                    const HeatCoef& k = hc[mm];
                    int ixa = ix - shx, iya = iy - shy;                              /* T:61-62 */
                    double q_ac = 0.0;
                    if (ixa >= 0 && ixa < nx && iya >= 0 && iya < ny) q_ac = Q[cidx(ixa, iya, iz, nx, ny)];  /* T:76-77 */
                    double Tn = src[i] * (1.0 - 4.0 * k.kxy - 2.0 * k.kz)
                              + k.kxy * (src[i - 1] + src[i + 1] + src[i + nx] + src[i - nx])
                              + k.kz * (src[i + (size_t)nx * ny] + src[i - (size_t)nx * ny]) + k.q * q_ac;   /* T:85-87 */
                    if (k.w != 0.0) Tn -= k.w * (src[i] - k.Ta);
                    dst[i] = Tn;
                    double Tc = Tn - 273.15;                                          /* T:88 */
                    if (Tc < 43.0) TD_io[i] = TD_io[i] + std::pow(4.0, Tc - 43.0) * th->dt;   /* T:99-100 */
                    else TD_io[i] = TD_io[i] + std::pow(2.0, Tc - 43.0) * th->dt;            /* T:101-102 */
                }
        use_p = !use_p;
        if (snap && isnap < n_snap && snap_steps[isnap] == st + 1) {
            std::memcpy(snap + (size_t)isnap * n, dst.data(), n * sizeof(double));
            ++isnap;
        }
    }
    std::vector<double>& last = use_p ? Ta : Tb;  /* after the final toggle, the latest is T_p if use_p */
    std::memcpy(T_io, last.data(), n * sizeof(double));
    return BD_OK;
}

/* Square spiral of T:141-173 and T:323-410, restated. */
bd_status bdo_spiral_shifts(const bd_trajectory* tr, int32_t* sx, int32_t* sy, int64_t cap,
                            int64_t* n_steps, int64_t* leg_end, int32_t leg_cap) {
    const double dt = tr->dt, dxy = tr->dxy;
    const int Nt_scale = 1 + (int)(tr->scale / (tr->speed * dt));      /* T:167 */
    const int Nt_acc = 1 + (int)(tr->t_acc / dt);                      /* T:170 */
    const double acc = (tr->speed - tr->speed_init) / tr->t_acc;       /* T:146 */
    std::vector<double> speed_acc(Nt_acc);
    for (int i = 0; i < Nt_acc; i++) speed_acc[i] = tr->speed_init + i * dt * acc;   /* T:173 */
    int lines = 0, increase = 1, sign_x = 1, sign_y = -1, shift_x = 0, shift_y = 0;
    bool right_left = true;
    double x_s = 0.0, y_s = 0.0;  /* T:331-332 place the start at the grid node of the axis */
    double x_next = x_s, x_prev = x_s, y_next = y_s, y_prev = y_s;
    double speed_current = tr->speed_init;
    int64_t k = 0;
    while (lines < tr->n_legs) {
        int n = (lines == 0) ? 1 : 0;                                  /* T:347-349 */
        x_next = x_prev + sign_x * dxy;
        y_next = y_prev + sign_y * dxy;
        for (; n < increase * Nt_scale + 2 * Nt_acc; n++) {
            if (n < Nt_acc) speed_current = speed_acc[n];
            if (n >= Nt_acc && n < increase * Nt_scale + Nt_acc) speed_current = tr->speed;
            if (n >= increase * Nt_scale + Nt_acc) speed_current = speed_acc[increase * Nt_scale + 2 * Nt_acc - n - 1];
            if (right_left) {
                x_s = x_s + sign_x * speed_current * dt;
                double dp = std::fabs(x_s - x_prev) / dxy, dn = std::fabs(x_next - x_s) / dxy;
                if (dn < dp) { shift_x += sign_x; x_prev = x_next; x_next = x_next + sign_x * dxy; }
            } else {
                y_s = y_s + sign_y * speed_current * dt;
                double dp = std::fabs(y_s - y_prev) / dxy, dn = std::fabs(y_next - y_s) / dxy;
                if (dn < dp) { shift_y += sign_y; y_prev = y_next; y_next = y_next + sign_y * dxy; }
            }
            if (k < cap) { sx[k] = shift_x; sy[k] = shift_y; }
            ++k;
        }
        right_left = !right_left;                                      /* T:394-406 */
        if (right_left) { increase++; sign_x = -sign_x; x_next = x_prev; }
        else { sign_y = -sign_y; y_next = y_prev; }
        if (leg_end && lines < leg_cap) leg_end[lines] = k;
        lines++;
    }
    *n_steps = k;
    return BD_OK;
}

}  // extern "C"

/* ------------------------------------------------------------------------ */
/* Gilmore-Zener (G:40-429)                                                  */
/* ------------------------------------------------------------------------ */
namespace {

struct GM {
    double rho, P0, S2, mu4, G4_3, C_inf, lambda, n, B, gamma3;
};

struct Drive {
    int nt;
    int mode = 0;        /* 0: sum of tones; 1/2/3: single/dual/triple combo of G:40-78 at amplitude A */
    double A = 0.0;
    double f[BD_MAX_BUBBLE_TONES], a[BD_MAX_BUBBLE_TONES], phi[BD_MAX_BUBBLE_TONES];
    double P(double t) const {
        if (mode == 1) return A * std::sin(2.0 * M_PI * f[0] * t);                                              /* G:47 */
        if (mode == 2) return (A / std::sqrt(2.0)) * (std::sin(2.0 * M_PI * f[0] * t) + std::sin(2.0 * M_PI * f[1] * t));   /* G:52 */
        if (mode == 3)
            return (A / std::sqrt(3.0)) * (std::sin(2.0 * M_PI * f[0] * t) + std::sin(2.0 * M_PI * f[1] * t) +
                                           std::sin(2.0 * M_PI * f[2] * t));                                  /* G:55 */
        double s = 0.0;
        for (int k = 0; k < nt; ++k) s += a[k] * std::sin(2.0 * M_PI * f[k] * t + phi[k]);
        return s;
    }
    double Pdt(double t) const {
        if (mode == 1) return A * 2.0 * M_PI * f[0] * std::cos(2.0 * M_PI * f[0] * t);                          /* G:68 */
        if (mode == 2)
            return A * std::sqrt(2.0) * M_PI * (f[0] * std::cos(2.0 * M_PI * f[0] * t) + f[1] * std::cos(2.0 * M_PI * f[1] * t));   /* G:73 */
        if (mode == 3)
            return A * (2.0 / std::sqrt(3.0)) * M_PI *
                   (f[0] * std::cos(2.0 * M_PI * f[0] * t) + f[1] * std::cos(2.0 * M_PI * f[1] * t) +
                    f[2] * std::cos(2.0 * M_PI * f[2] * t));                                                  /* G:76 */
        double s = 0.0;
        for (int k = 0; k < nt; ++k) s += a[k] * 2.0 * M_PI * f[k] * std::cos(2.0 * M_PI * f[k] * t + phi[k]);
        return s;
    }
};

inline double P_in(const GM& g, double R, double R0) { return (g.P0 + (g.S2 / R0)) * std::pow(R0 / R, g.gamma3); }   /* G:84 */
inline double dP_in_dt(const GM& g, double R0, double R, double R1) {
    return (g.P0 + (g.S2 / R0)) * std::pow(R0, g.gamma3) * (-g.gamma3) * std::pow(R, -g.gamma3 - 1.0) * R1;            /* G:91 */
}
inline double Stress_dt(const GM& g, double R, double R1, double Tau, double R0) {
    double Tau_dt = -g.G4_3 * (1.0 - std::pow(R0 / R, 3)) - (g.mu4 * R1 / R) - Tau;                                    /* G:108 */
    return Tau_dt / g.lambda;
}
inline double Q_dt(const GM& g, double R, double R1, double Tau, double q, double R0) {
    double q_dt = (-g.G4_3 * (1.0 - std::pow(R0 / R, 3)) - (g.mu4 * R1 / R)) / (3.0 * g.lambda);                         /* G:115 */
    return q_dt - (q / g.lambda) - (R1 * Tau / R);
}
inline double F_R(const GM& g, const Drive& d, double t, double R, double R1, double Tau, double q, double R0) {
    double Tau1 = Stress_dt(g, R, R1, Tau, R0);
    double q1 = Q_dt(g, R, R1, Tau, q, R0);
    double p = d.P(t);
    double p_in = P_in(g, R, R0);
    /* Enthalpy G:121-128 */
    double part1 = (g.P0 + p + g.B) * g.n / (g.rho * (g.n - 1.0));
    double part2 = (p_in - (g.S2 / R) + Tau + g.B) / (g.P0 + p + g.B);
    double H = part1 * (std::pow(part2, (g.n - 1.0) / g.n) - 1.0);
    /* Enthalpy_dt G:132-157 */
    double p_dt = d.Pdt(t);
    double part1_dt = p_dt * g.n / (g.rho * (g.n - 1.0));
    double u = p_in - (g.S2 / R) + Tau + g.B;
    double v = g.P0 + p + g.B;
    double I = u / v;
    double part2b = std::pow(I, (g.n - 1.0) / g.n) - 1.0;
    double d_pin = dP_in_dt(g, R0, R, R1);
    double u_dt = d_pin + (g.S2 * R1 / (R * R)) + Tau1;
    double I_dt = (u_dt * v - u * p_dt) / std::pow(v, 2);
    double part2_dt = ((g.n - 1.0) / g.n) * std::pow(I, -1.0 / g.n) * I_dt;
    double H1 = part1_dt * part2b + part1 * part2_dt;
    /* LocalSoundSpeed G:96-103 */
    double Cc = ((p_in - (g.S2 / R) + Tau) + g.B) / (g.P0 + p + g.B);
    double C = g.C_inf * std::pow(Cc, (g.n - 1.0) / (2.0 * g.n));
    /* G:170-178 */
    double a = 1.0 - (R1 / C), b = 1.0 + (R1 / C);
    double pp1 = 1.5 * std::pow(R1, 2) * (1.0 - (R1 / (3.0 * C)));
    double pp2 = b * (H + ((-Tau + 3.0 * q) / g.rho));
    double pp3 = (H1 * a + ((-Tau1 + 3.0 * q1) / g.rho)) * R / C;
    return (-pp1 + pp2 + pp3) / (a * R);
}

const double DP_A[7][7] = {
    {0, 0, 0, 0, 0, 0, 0},
    {0.2, 0, 0, 0, 0, 0, 0},
    {3.0 / 40.0, -9.0 / 40.0, 0, 0, 0, 0, 0},
    {44.0 / 45.0, -56.0 / 15.0, 32.0 / 9.0, 0, 0, 0, 0},
    {19372.0 / 6561.0, -25360.0 / 2187.0, 64448.0 / 6561.0, -212.0 / 729.0, 0, 0, 0},
    {9017.0 / 3168.0, -355.0 / 33.0, 46732.0 / 5247.0, 49.0 / 176.0, -5103.0 / 18656.0, 0, 0},
    {35.0 / 384.0, 0, 500.0 / 1113.0, 125.0 / 192.0, -2187.0 / 6784.0, 11.0 / 84.0, 0}};
const double DP_B[7] = {35.0 / 384.0, 0, 500.0 / 1113.0, 125.0 / 192.0, -2187.0 / 6784.0, 11.0 / 84.0, 0};
const double DP_BB[7] = {5179.0 / 57600.0, 0, 7571.0 / 16695.0, 393.0 / 640.0, -92097.0 / 339200.0, 187.0 / 2100.0, 1.0 / 40.0};
const double DP_C[7] = {0, 0.2, 0.3, 0.8, 8.0 / 9.0, 1.0, 1.0};

/* One accepted Dormand-Prince step, G:212-318 (rejections loop inside). */
void dp_step(const GM& g, const Drive& d, double& t, double& R, double& R1, double& Tau, double& q,
             double& h, bool& thr, double R0, double endT, double atol, double rtol, double fac_max0,
             int64_t& n_rej) {
    double Y[4], err_[4], sc[4], K[7], L[7], TK[7], QK[7];
    double err, max_result = 1.0;
    if (t + h > endT) h = endT - t;                        /* G:240 */
    err = 2.0;
    double fac_max = fac_max0;
    thr = false;
    bool first = true;
    while (err > 1.0) {                                   /* G:246 */
        if (!first) ++n_rej;
        first = false;
        Y[0] = R; Y[1] = R1; Y[2] = Tau; Y[3] = q;
        err_[0] = err_[1] = err_[2] = err_[3] = 0.0;
        for (int i = 0; i < 7; ++i) { K[i] = L[i] = TK[i] = QK[i] = 0.0; }
        for (int i = 0; i < 7; ++i) {
            double kR = 0, kR1 = 0, kT = 0, kq = 0;
            for (int j = 0; j < i; ++j) {
                kR = kR + DP_A[i][j] * K[j] * h;
                kR1 = kR1 + DP_A[i][j] * L[j] * h;
                kT = kT + DP_A[i][j] * TK[j] * h;
                kq = kq + DP_A[i][j] * QK[j] * h;
            }
            K[i] = (R1 + kR1);
            L[i] = F_R(g, d, t + h * DP_C[i], R + kR, R1 + kR1, Tau + kT, q + kq, R0);
            TK[i] = Stress_dt(g, R + kR, R1 + kR1, Tau + kT, R0);
            QK[i] = Q_dt(g, R + kR, R1 + kR1, Tau + kT, q + kq, R0);
            Y[0] = Y[0] + DP_B[i] * K[i] * h;
            Y[1] = Y[1] + DP_B[i] * L[i] * h;
            Y[2] = Y[2] + DP_B[i] * TK[i] * h;
            Y[3] = Y[3] + DP_B[i] * QK[i] * h;
            err_[0] = err_[0] + K[i] * h * (DP_B[i] - DP_BB[i]);
            err_[1] = err_[1] + L[i] * h * (DP_B[i] - DP_BB[i]);
            err_[2] = err_[2] + TK[i] * h * (DP_B[i] - DP_BB[i]);
            err_[3] = err_[3] + QK[i] * h * (DP_B[i] - DP_BB[i]);
        }
        sc[0] = atol + rtol * std::fmax(std::fabs(R), std::fabs(Y[0]));     /* G:289-292 */
        sc[1] = atol + rtol * std::fmax(std::fabs(R1), std::fabs(Y[1]));
        sc[2] = atol + rtol * std::fmax(std::fabs(Tau), std::fabs(Y[2]));
        sc[3] = atol + rtol * std::fmax(std::fabs(q), std::fabs(Y[3]));
        double S = 0.0;
        for (int i = 0; i < 4; ++i) S = S + std::pow(err_[i] / sc[i], 2);   /* G:183-192 */
        err = std::sqrt(S / 4);
        max_result = std::fmax(0.1, 0.9 * std::pow(err, -0.2));            /* G:296 */
        if (err > 1.0) { fac_max = 0.9; h = h * std::fmin(fac_max, max_result); }
    }
    t = t + h;
    R = Y[0]; R1 = Y[1]; Tau = Y[2]; q = Y[3];
    h = h * std::fmin(fac_max, max_result);                 /* G:310 */
    if (Y[1] <= -g.C_inf) thr = true;                       /* G:313 */
}

GM make_gm(const bd_gilmore_medium* m) {
    GM g;
    g.rho = m->rho; g.P0 = m->P0; g.S2 = m->S2; g.mu4 = m->mu4; g.G4_3 = m->G4_3;
    g.C_inf = m->C_inf; g.lambda = m->lambda; g.n = m->n; g.B = m->B; g.gamma3 = 3.0 * m->gamma;
    return g;
}

void combo_drive(double A, double f1, double f2, double f3, Drive& d) {
    /* G:40-57: single if all equal, dual if f1==f2 or f2==f3, else triple */
    for (int k = 0; k < BD_MAX_BUBBLE_TONES; ++k) { d.f[k] = 0; d.a[k] = 0; d.phi[k] = 0; }
    d.A = A;
    if (f1 == f2 && f1 == f3) { d.nt = 1; d.mode = 1; d.f[0] = f1; d.a[0] = A; }
    else if (f1 == f2 || f2 == f3) { d.nt = 2; d.mode = 2; d.f[0] = f1; d.f[1] = f3; d.a[0] = d.a[1] = A / std::sqrt(2.0); }
    else { d.nt = 3; d.mode = 3; d.f[0] = f1; d.f[1] = f2; d.f[2] = f3; d.a[0] = d.a[1] = d.a[2] = A / std::sqrt(3.0); }
}

}  // namespace

extern "C" {

/* Forward run of each bubble with the G:212-318 step (reference arithmetic). */
bd_status bdo_gilmore_run(const bd_gilmore_medium* m, int64_t n, const bd_bubble* b,
                          const bd_ode_params* ode, bd_bubble_result* res) {
    GM g = make_gm(m);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t i = 0; i < n; ++i) {
        Drive d;
        d.nt = b[i].n_tones;
        for (int k = 0; k < BD_MAX_BUBBLE_TONES; ++k) { d.f[k] = b[i].f[k]; d.a[k] = b[i].a[k]; d.phi[k] = b[i].phi[k]; }
        double t = 0, R = b[i].R0, R1 = 0, Tau = 0, q = 0, h = ode->h0;
        bd_bubble_result r;
        std::memset(&r, 0, sizeof r);
        r.R_max = R; r.R_min = R; r.t_threshold = -1.0;
        int64_t nrej = 0, nacc = 0;
        bool thr = false;
        r.status = BD_BUBBLE_DONE;
        while (t < ode->t_end) {
            if (nacc >= ode->max_steps) { r.status = BD_BUBBLE_STEP_CAP; break; }
            dp_step(g, d, t, R, R1, Tau, q, h, thr, b[i].R0, ode->t_end, ode->atol, ode->rtol, ode->fac_max, nrej);
            ++nacc;
            if (!std::isfinite(R) || !std::isfinite(R1)) { r.status = BD_BUBBLE_NONFINITE; break; }
            r.R_max = std::fmax(r.R_max, R); r.R_min = std::fmin(r.R_min, R);
            if (thr && !r.threshold) { r.threshold = 1; r.t_threshold = t; }
            if (thr && ode->stop_at_threshold) { r.status = BD_BUBBLE_THRESHOLD; break; }
        }
        r.R = R; r.Rdot = R1; r.tau = Tau; r.q = q; r.t = t;
        r.n_accept = nacc; r.n_reject = nrej;
        res[i] = r;
    }
    return BD_OK;
}

/* Forward integration with the combo drive of G:40-78 (amplitude A, three
 * frequencies), the inner loop of G:378-379 at a fixed amplitude. */
bd_status bdo_gilmore_forward_combo(const bd_gilmore_medium* m, int64_t n, const double* R0, const double* A,
                                    const double* f3, double endT, double h0, int64_t max_steps,
                                    int32_t stop_at_threshold, double* state, int64_t* counts, double* thr_t) {
    GM g = make_gm(m);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t i = 0; i < n; ++i) {
        Drive d;
        combo_drive(A[i], f3[3 * i], f3[3 * i + 1], f3[3 * i + 2], d);
        double t = 0.0, R = R0[i], R1 = 0.0, Tau = 0.0, q = 0.0, h = h0, tt = -1.0;
        bool th = false;
        int64_t k = 0, nrej = 0;
        while (t < endT && k < max_steps) {
            dp_step(g, d, t, R, R1, Tau, q, h, th, R0[i], endT, 1e-9, 1e-9, 5.0, nrej);
            ++k;
            if (th && tt < 0) tt = t;
            if (th && stop_at_threshold) break;
        }
        state[5 * i] = t; state[5 * i + 1] = R; state[5 * i + 2] = R1; state[5 * i + 3] = Tau; state[5 * i + 4] = q;
        counts[i] = k;
        thr_t[i] = tt;
    }
    return BD_OK;
}

/* Threshold search G:323-429 (printf dropped).  max_steps bounds each
 * integration (0 = unbounded, as in G). */
static bd_status gilmore_threshold_impl(const bd_gilmore_medium* m, const double* fr_combo, int64_t n_combo,
                                       const double* R0s, int64_t n_R0, int64_t max_steps, int bisect, double* out);

bd_status bdo_gilmore_threshold(const bd_gilmore_medium* m, const double* fr_combo, int64_t n_combo,
                                const double* R0s, int64_t n_R0, int64_t max_steps, double* out) {
    return gilmore_threshold_impl(m, fr_combo, n_combo, R0s, n_R0, max_steps, 0, out);
}

/* The same search with stages 2-3 (G:391-426) replaced by bisection on the
 * 1 kPa grid between the last amplitude of stage 1 that stayed below the
 * threshold (A - 0.1 MPa) and the first that reached it (A): under a monotone
 * threshold response it returns the same grid amplitude with about 7
 * integrations instead of up to 20. */
bd_status bdo_gilmore_threshold_bisect(const bd_gilmore_medium* m, const double* fr_combo, int64_t n_combo,
                                       const double* R0s, int64_t n_R0, int64_t max_steps, double* out) {
    return gilmore_threshold_impl(m, fr_combo, n_combo, R0s, n_R0, max_steps, 1, out);
}

static bd_status gilmore_threshold_impl(const bd_gilmore_medium* m, const double* fr_combo, int64_t n_combo,
                                       const double* R0s, int64_t n_R0, int64_t max_steps, int bisect, double* out) {
    GM g = make_gm(m);
    const int64_t N = n_combo * n_R0;
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t idx = 0; idx < N; ++idx) {
        int64_t ic = idx / n_R0, ir = idx % n_R0;                         /* G:327-328 */
        double R0 = R0s[ir];
        double fr1 = fr_combo[3 * ic], fr2 = fr_combo[3 * ic + 1], fr3 = fr_combo[3 * ic + 2];
        double endT = 0.0;                                                 /* G:342-353 */
        if (fr1 <= fr2 && fr1 <= fr3) endT = 5.0 / fr1;
        if (fr2 <= fr1 && fr2 <= fr3) endT = 5.0 / fr2;
        if (fr3 <= fr1 && fr3 <= fr2) endT = 5.0 / fr3;
        double h = std::pow(10.0, -13);
        out[idx] = -1.0;
        double t, R, R1, Tau, q;
        bool th5 = false, th4 = true, th3 = true;
        double A5 = 0.0, A4 = 0.0, A3 = 0.0;
        int64_t nrej = 0;
        auto integrate = [&](double A, bool& thr) {
            Drive d; combo_drive(A, fr1, fr2, fr3, d);
            int64_t k = 0;
            while (t < endT && !thr) {
                dp_step(g, d, t, R, R1, Tau, q, h, thr, R0, endT, 1e-9, 1e-9, 5.0, nrej);
                if (max_steps > 0 && ++k >= max_steps) break;
            }
        };
        while (!th5 && A5 < std::pow(10.0, 7)) {                         /* G:372-380 */
            t = 0.0; R = R0; R1 = 0.0; Tau = 0.0; q = 0.0;
            A5 = A5 + std::pow(10.0, 5);
            th5 = false;
            integrate(A5, th5);
        }
        if (!th5 && A5 == std::pow(10.0, 7)) out[idx] = A5;               /* G:383-387 */
        if (bisect) {
            if (th5) {
                const double lo = A5 - std::pow(10.0, 5);
                int ilo = 0, ihi = 100;                                    /* A = lo + i kPa */
                while (ihi - ilo > 1) {
                    const int imid = (ilo + ihi) / 2;
                    h = std::pow(10.0, -13);
                    t = 0.0; R = R0; R1 = 0.0; Tau = 0.0; q = 0.0;
                    bool hit = false;
                    integrate(lo + imid * std::pow(10.0, 3), hit);
                    if (hit) ihi = imid; else ilo = imid;
                }
                out[idx] = lo + ihi * std::pow(10.0, 3);
            }
            continue;
        }
        A4 = A5;
        while (th5 && th4) {                                              /* G:391-406 */
            h = std::pow(10.0, -13);
            t = 0.0; R = R0; R1 = 0.0; Tau = 0.0; q = 0.0;
            A4 = A4 - std::pow(10.0, 4);
            th4 = false;
            integrate(A4, th4);
            if (!th4) A4 = A4 + std::pow(10.0, 4);
        }
        A3 = A4;
        while (th5 && !th4 && th3) {                                      /* G:411-426 */
            h = std::pow(10.0, -13);
            t = 0.0; R = R0; R1 = 0.0; Tau = 0.0; q = 0.0;
            A3 = A3 - std::pow(10.0, 3);
            th3 = false;
            integrate(A3, th3);
            if (!th3) out[idx] = A3 + std::pow(10.0, 3);
        }
    }
    return BD_OK;
}

/* Frequency combinations G:498-520. */
int64_t bdo_gilmore_combos(int32_t N_fr, double min_fr, double max_fr, double* out, int64_t cap) {
    double step_log = (std::log10(max_fr) - std::log10(min_fr)) / (N_fr - 1.0);   /* G:469 */
    int64_t k = 0;
    for (int i = 0; i < N_fr; i++) {
        bool first_cycle = true;
        for (int ii = i; ii < N_fr; ii++) {
            int iii = first_cycle ? ii : ii + 1;
            for (; iii < N_fr; iii++) {
                if (k < cap) {
                    out[3 * k] = std::pow(10.0, std::log10(min_fr) + i * step_log);
                    out[3 * k + 1] = std::pow(10.0, std::log10(min_fr) + ii * step_log);
                    out[3 * k + 2] = std::pow(10.0, std::log10(min_fr) + iii * step_log);
                }
                k++;
            }
            first_cycle = false;
        }
    }
    return k;
}

}  // extern "C"
