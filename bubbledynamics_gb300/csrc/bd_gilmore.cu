// Gilmore-Zener bubble dynamics: bd_gilmore_run(_device) and
// bd_gilmore_threshold.  Replaces G:40-429 (RHS, Dormand-Prince step,
// threshold-search kernel) and the launch of G:573.
//
// One persistent launch (a few CTAs per SM); every lane pulls the next
// bubble (or threshold work item) from a device counter when its current one
// ends, so bubbles with uneven adaptive step counts keep the lanes busy.  Each
// loop iteration performs exactly one Dormand-Prince attempt for every active
// lane, so lanes of a warp stay converged whatever their bubble's progress.
//
// Arithmetic (FP64 throughout; FP64 units are scarce on this GPU, so the
// fast path trims FP64 work, the ref path mirrors G operation by operation):
//   fast: FSAL (6 RHS per attempt instead of 7); the logarithms and
//         exponentials of (R0/R)^{3 gamma} and I^{(n-1)/n} once per attempt at
//         the step start and, at the stages, short Taylor series in the
//         relative offsets from it; C from the same powers (no sqrt, no
//         division); the drive as a polynomial in the stage offset; error norm
//         and step-size controller in FP32 (they only choose h).
//   ref:  G:84-178 with its pow calls and the 7-stage loop of G:259-286.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "bd_internal.h"

namespace bd {

#define BD_PI_D 3.14159265358979323846

struct GilK {
    double rho, P0, S2, mu4, G4_3, C_inf, lambda, n, B, gamma3;
    double n1n;        // (n-1)/n
    double irho, ilam, i3lam, nrho;   // 1/rho, 1/lambda, 1/(3 lambda), n/(rho (n-1))
    double iCinf;                     // 1/C_inf
};

struct OdeK {
    double t_end, h0, atol, rtol, fac_max;
    long long max_steps;
    int stop_at_threshold;
    int ref_arith;
};

// Dormand-Prince 5(4) tableau (Dormand & Prince 1980)
__constant__ double c_A[7][7] = {
    {0, 0, 0, 0, 0, 0, 0},
    {0.2, 0, 0, 0, 0, 0, 0},
    {3.0 / 40.0, -9.0 / 40.0, 0, 0, 0, 0, 0},
    {44.0 / 45.0, -56.0 / 15.0, 32.0 / 9.0, 0, 0, 0, 0},
    {19372.0 / 6561.0, -25360.0 / 2187.0, 64448.0 / 6561.0, -212.0 / 729.0, 0, 0, 0},
    {9017.0 / 3168.0, -355.0 / 33.0, 46732.0 / 5247.0, 49.0 / 176.0, -5103.0 / 18656.0, 0, 0},
    {35.0 / 384.0, 0, 500.0 / 1113.0, 125.0 / 192.0, -2187.0 / 6784.0, 11.0 / 84.0, 0}};
__constant__ double c_B[7] = {35.0 / 384.0, 0, 500.0 / 1113.0, 125.0 / 192.0, -2187.0 / 6784.0, 11.0 / 84.0, 0};
__constant__ double c_BB[7] = {5179.0 / 57600.0, 0, 7571.0 / 16695.0, 393.0 / 640.0, -92097.0 / 339200.0,
                               187.0 / 2100.0, 1.0 / 40.0};
__constant__ double c_C[7] = {0, 0.2, 0.3, 0.8, 8.0 / 9.0, 1.0, 1.0};

struct Tones {
    int n;
    int mode;          // 0: sum of tones; 1/2/3: single/dual/triple combo of G:40-78 at amplitude A
    double A;
    double f[BD_MAX_BUBBLE_TONES], a[BD_MAX_BUBBLE_TONES], phi[BD_MAX_BUBBLE_TONES];
};

// --------------------------------------------------------------- reference RHS
// G:40-179 in the reference's operation order (pow calls kept).
__device__ double ref_P(const Tones& d, double t) {
    if (d.mode == 1) return d.A * sin(2.0 * BD_PI_D * d.f[0] * t);                                        // G:47
    if (d.mode == 2) return (d.A / sqrt(2.0)) * (sin(2.0 * BD_PI_D * d.f[0] * t) + sin(2.0 * BD_PI_D * d.f[1] * t));   // G:52
    if (d.mode == 3)
        return (d.A / sqrt(3.0)) * (sin(2.0 * BD_PI_D * d.f[0] * t) + sin(2.0 * BD_PI_D * d.f[1] * t) +
                                    sin(2.0 * BD_PI_D * d.f[2] * t));                                          // G:55
    double s = 0.0;
    for (int k = 0; k < d.n; ++k) s += d.a[k] * sin(2.0 * BD_PI_D * d.f[k] * t + d.phi[k]);
    return s;
}
__device__ double ref_Pdt(const Tones& d, double t) {
    if (d.mode == 1) return d.A * 2.0 * BD_PI_D * d.f[0] * cos(2.0 * BD_PI_D * d.f[0] * t);                // G:68
    if (d.mode == 2)
        return d.A * sqrt(2.0) * BD_PI_D * (d.f[0] * cos(2.0 * BD_PI_D * d.f[0] * t) + d.f[1] * cos(2.0 * BD_PI_D * d.f[1] * t));   // G:73
    if (d.mode == 3)
        return d.A * (2.0 / sqrt(3.0)) * BD_PI_D *
               (d.f[0] * cos(2.0 * BD_PI_D * d.f[0] * t) + d.f[1] * cos(2.0 * BD_PI_D * d.f[1] * t) +
                d.f[2] * cos(2.0 * BD_PI_D * d.f[2] * t));                                                      // G:76
    double s = 0.0;
    for (int k = 0; k < d.n; ++k) s += d.a[k] * 2.0 * BD_PI_D * d.f[k] * cos(2.0 * BD_PI_D * d.f[k] * t + d.phi[k]);
    return s;
}
__device__ __forceinline__ double ref_stress_dt(const GilK& g, double R, double R1, double Tau, double R0) {
    double Tau_dt = -g.G4_3 * (1.0 - pow(R0 / R, 3.0)) - (g.mu4 * R1 / R) - Tau;   // G:108
    return Tau_dt / g.lambda;
}
__device__ __forceinline__ double ref_q_dt(const GilK& g, double R, double R1, double Tau, double q, double R0) {
    double q_dt = (-g.G4_3 * (1.0 - pow(R0 / R, 3.0)) - (g.mu4 * R1 / R)) / (3.0 * g.lambda);   // G:115
    return q_dt - (q / g.lambda) - (R1 * Tau / R);
}
__device__ double ref_F_R(const GilK& g, const Tones& d, double t, double R, double R1, double Tau, double q, double R0) {
    const double Tau1 = ref_stress_dt(g, R, R1, Tau, R0);
    const double q1 = ref_q_dt(g, R, R1, Tau, q, R0);
    const double p = ref_P(d, t);
    const double p_in = (g.P0 + (g.S2 / R0)) * pow(R0 / R, g.gamma3);                       // G:84
    const double part1 = (g.P0 + p + g.B) * g.n / (g.rho * (g.n - 1.0));                       // G:125
    const double part2 = (p_in - (g.S2 / R) + Tau + g.B) / (g.P0 + p + g.B);
    const double H = part1 * (pow(part2, (g.n - 1.0) / g.n) - 1.0);                          // G:127
    const double p_dt = ref_Pdt(d, t);
    const double part1_dt = p_dt * g.n / (g.rho * (g.n - 1.0));
    const double u = p_in - (g.S2 / R) + Tau + g.B;
    const double v = g.P0 + p + g.B;
    const double I = u / v;
    const double part2b = pow(I, (g.n - 1.0) / g.n) - 1.0;
    const double d_pin = (g.P0 + (g.S2 / R0)) * pow(R0, g.gamma3) * (-g.gamma3) * pow(R, -g.gamma3 - 1.0) * R1;   // G:91
    const double u_dt = d_pin + (g.S2 * R1 / (R * R)) + Tau1;
    const double I_dt = (u_dt * v - u * p_dt) / pow(v, 2.0);
    const double part2_dt = ((g.n - 1.0) / g.n) * pow(I, -1.0 / g.n) * I_dt;
    const double H1 = part1_dt * part2b + part1 * part2_dt;                                  // G:156
    double C = ((p_in - (g.S2 / R) + Tau) + g.B) / (g.P0 + p + g.B);                        // G:100
    C = g.C_inf * pow(C, (g.n - 1.0) / (2.0 * g.n));
    const double a = 1.0 - (R1 / C), b = 1.0 + (R1 / C);                                    // G:170-176
    const double pp1 = 1.5 * pow(R1, 2.0) * (1.0 - (R1 / (3.0 * C)));
    const double pp2 = b * (H + ((-Tau + 3.0 * q) / g.rho));
    const double pp3 = (H1 * a + ((-Tau1 + 3.0 * q1) / g.rho)) * R / C;
    return (-pp1 + pp2 + pp3) / (a * R);
}

// --------------------------------------------------------------- fast RHS
// Same equations with shared transcendental work.  dP, dPdt come from the caller.
struct Rhs { double dR, dU, dT, dq; };

__device__ __forceinline__ Rhs fast_rhs(const GilK& g, double pin0, double R0, double R, double U, double Tau, double q,
                                        double P, double Pdt) {
    const double iR = 1.0 / R;
    const double x = R0 * iR;
    const double pin = pin0 * exp(g.gamma3 * log(x));            // (P0 + 2S/R0)(R0/R)^{3 gamma}
    const double x3 = x * x * x;
    const double el = -g.G4_3 * (1.0 - x3) - g.mu4 * U * iR;
    const double Tau1 = (el - Tau) * g.ilam;                       // G:108-109
    const double q1 = el * g.i3lam - q * g.ilam - U * Tau * iR;    // G:115-116
    const double u = pin - g.S2 * iR + Tau + g.B;
    const double v = g.P0 + P + g.B;
    const double iv = 1.0 / v;
    const double I = u * iv;
    const double Ip = exp(g.n1n * log(I));                         // I^{(n-1)/n}
    const double Ipm = Ip / I;                                     // I^{-1/n}
    const double C = g.C_inf * sqrt(Ip);                           // G:100-101
    const double part1 = v * g.nrho;
    const double H = part1 * (Ip - 1.0);
    const double dpin = -g.gamma3 * pin * U * iR;                  // G:91
    const double udt = dpin + g.S2 * U * iR * iR + Tau1;
    const double Idt = (udt * v - u * Pdt) * iv * iv;
    const double H1 = Pdt * g.nrho * (Ip - 1.0) + part1 * g.n1n * Ipm * Idt;
    const double iC = 1.0 / C;
    const double a = 1.0 - U * iC, b = 1.0 + U * iC;
    const double pp1 = 1.5 * U * U * (1.0 - U * iC * (1.0 / 3.0));
    const double pp2 = b * (H + (3.0 * q - Tau) * g.irho);
    const double pp3 = (H1 * a + (3.0 * q1 - Tau1) * g.irho) * R * iC;
    Rhs r;
    r.dR = U;
    r.dU = (-pp1 + pp2 + pp3) / (a * R);
    r.dT = Tau1;
    r.dq = q1;
    return r;
}

// sin / cos of a small angle by their Taylor series (|x| <= 0.25: truncation below 1e-20)
__device__ __forceinline__ void small_sincos(double x, double& s, double& c) {
    const double x2 = x * x;
    s = x * (1.0 - x2 / 6.0 * (1.0 - x2 / 20.0 * (1.0 - x2 / 42.0 * (1.0 - x2 / 72.0 * (1.0 - x2 / 110.0 * (1.0 - x2 / 156.0))))));
    c = 1.0 - x2 / 2.0 * (1.0 - x2 / 12.0 * (1.0 - x2 / 30.0 * (1.0 - x2 / 56.0 * (1.0 - x2 / 90.0 * (1.0 - x2 / 132.0 * (1.0 - x2 / 182.0))))));
}

// Drive and its derivative at t0 + dt given sin/cos of the tone phases at t0.
__device__ __forceinline__ void drive_at(const Tones& d, const double* s0, const double* c0, double dt, double& P,
                                         double& Pdt) {
    P = 0.0;
    Pdt = 0.0;
    for (int k = 0; k < d.n; ++k) {
        const double w = 2.0 * BD_PI_D * d.f[k];
        const double th = w * dt;
        double ss, cc;
        if (fabs(th) <= 0.25) small_sincos(th, ss, cc);
        else sincos(th, &ss, &cc);
        const double sk = s0[k] * cc + c0[k] * ss;
        const double ck = c0[k] * cc - s0[k] * ss;
        P += d.a[k] * sk;
        Pdt += d.a[k] * w * ck;
    }
}

// ---------------------------------------------------------------- step-start expansions
// Within one Dormand-Prince attempt the stage states differ from the step start
// by h times a bounded derivative, and on this problem h is tiny next to every
// time scale of R (the 3 ns Zener relaxation keeps h near 1e-11..1e-9 s).  The
// fast path therefore evaluates the transcendentals once per attempt, at the
// step start, and expands around them: with d = R_s/R_b - 1 and e = I_s/I_b - 1
// below 1e-3 the series below are exact to ~1e-21 (first neglected term);
// larger offsets fall back to the direct evaluation.

// log(1 + d), |d| <= 1e-3: Taylor series to d^6
__device__ __forceinline__ double log1p_s(double d) {
    return d * (1.0 - d * (0.5 - d * (1.0 / 3.0 - d * (0.25 - d * (0.2 - d * (1.0 / 6.0))))));
}
// exp(e) - 1, |e| <= 5e-3: Taylor series to e^6
__device__ __forceinline__ double expm1_s(double e) {
    return e * (1.0 + e * (0.5 + e * (1.0 / 6.0 + e * (1.0 / 24.0 + e * (1.0 / 120.0 + e * (1.0 / 720.0))))));
}

// The drive as a polynomial in the offset tau from the step start: with the
// tone phases' sin/cos at the start, d^m/dtau^m sum_k a_k sin(w_k tau + th_k)
// cycles through a_k w_k^m (s, c, -s, -c).  Used when max_k w_k h <= 0.02,
// where the first neglected term (w h)^8 / 8! is below 1e-18.
struct DriveSeries {
    double p[8], q[8];   // P(tau) = sum p[m] tau^m, dP/dt(tau) = sum q[m] tau^m
    __device__ __forceinline__ void eval(double tau, double& P, double& Pdt) const {
        double a = p[7], b = q[7];
#pragma unroll
        for (int m = 6; m >= 0; --m) { a = fma(a, tau, p[m]); b = fma(b, tau, q[m]); }
        P = a;
        Pdt = b;
    }
};

__device__ __forceinline__ bool drive_series(const Tones& d, const double* s0, const double* c0, double h,
                                             DriveSeries& S) {
    double wmax = 0.0;
    for (int k = 0; k < d.n; ++k) wmax = fmax(wmax, 2.0 * BD_PI_D * fabs(d.f[k]));
    if (wmax * fabs(h) > 0.02) return false;
    double D[9];
#pragma unroll
    for (int m = 0; m < 9; ++m) D[m] = 0.0;
    for (int k = 0; k < d.n; ++k) {
        const double w = 2.0 * BD_PI_D * d.f[k];
        double wm = d.a[k];
#pragma unroll
        for (int m = 0; m < 9; ++m) {
            const double v = (m & 1) ? c0[k] : s0[k];
            D[m] = fma(((m & 2) ? -wm : wm), v, D[m]);
            wm *= w;
        }
    }
    double fact = 1.0;
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        if (m > 0) fact *= (double)m;
        const double inv = 1.0 / fact;
        S.p[m] = D[m] * inv;
        S.q[m] = D[m + 1] * inv;
    }
    return true;
}

// Transcendental pieces of the right-hand side at the step start.
struct RhsBase {
    double R, iR, pin, I, iI, Ip, Ipmh, Ipm;
};

__device__ __forceinline__ RhsBase rhs_base(const GilK& g, double pin0, double R0, double R, double Tau, double P) {
    RhsBase b;
    b.R = R;
    b.iR = 1.0 / R;
    const double lx = log(R0 * b.iR);
    b.pin = pin0 * exp(g.gamma3 * lx);
    const double u = b.pin - g.S2 * b.iR + Tau + g.B;
    const double v = g.P0 + P + g.B;
    b.I = u / v;
    b.iI = 1.0 / b.I;
    const double lI = log(b.I);
    b.Ip = exp(g.n1n * lI);                // I^{(n-1)/n}
    b.Ipmh = exp(-0.5 * g.n1n * lI);       // I^{-(n-1)/(2n)}
    b.Ipm = b.Ip * b.iI;                   // I^{-1/n}
    return b;
}

// fast_rhs with every transcendental and the divisions by R and C taken from
// the step-start expansion (falls back to fast_rhs for large offsets).
__device__ __forceinline__ Rhs series_rhs(const GilK& g, const RhsBase& b, double pin0, double R0, double R,
                                          double U, double Tau, double q, double P, double Pdt) {
    const double dr = (R - b.R) * b.iR;
    if (!(fabs(dr) <= 1e-3)) return fast_rhs(g, pin0, R0, R, U, Tau, q, P, Pdt);
    const double iR = b.iR * (1.0 - dr * (1.0 - dr * (1.0 - dr * (1.0 - dr * (1.0 - dr * (1.0 - dr))))));
    const double l1 = log1p_s(dr);
    const double pin = b.pin * (1.0 + expm1_s(-g.gamma3 * l1));
    const double u = pin - g.S2 * iR + Tau + g.B;
    const double v = g.P0 + P + g.B;
    const double iv = 1.0 / v;
    const double I = u * iv;
    const double e = (I - b.I) * b.iI;
    if (!(fabs(e) <= 1e-3)) return fast_rhs(g, pin0, R0, R, U, Tau, q, P, Pdt);
    const double lI = log1p_s(e);
    const double Ip = b.Ip * (1.0 + expm1_s(g.n1n * lI));
    const double Ipmh = b.Ipmh * (1.0 + expm1_s(-0.5 * g.n1n * lI));
    const double Ipm = b.Ipm * (1.0 + expm1_s(-(1.0 - g.n1n) * lI));
    const double x = R0 * iR;
    const double x3 = x * x * x;
    const double el = -g.G4_3 * (1.0 - x3) - g.mu4 * U * iR;
    const double Tau1 = (el - Tau) * g.ilam;                       // G:108-109
    const double q1 = el * g.i3lam - q * g.ilam - U * Tau * iR;    // G:115-116
    const double part1 = v * g.nrho;
    const double H = part1 * (Ip - 1.0);
    const double dpin = -g.gamma3 * pin * U * iR;                  // G:91
    const double udt = dpin + g.S2 * U * iR * iR + Tau1;
    const double Idt = (udt * v - u * Pdt) * iv * iv;
    const double H1 = Pdt * g.nrho * (Ip - 1.0) + part1 * g.n1n * Ipm * Idt;
    const double iC = Ipmh * g.iCinf;                              // 1 / (C_inf sqrt(I^{(n-1)/n}))
    const double a = 1.0 - U * iC, bb = 1.0 + U * iC;
    const double pp1 = 1.5 * U * U * (1.0 - U * iC * (1.0 / 3.0));
    const double pp2 = bb * (H + (3.0 * q - Tau) * g.irho);
    const double pp3 = (H1 * a + (3.0 * q1 - Tau1) * g.irho) * R * iC;
    Rhs r;
    r.dR = U;
    r.dU = (-pp1 + pp2 + pp3) * iR / a;
    r.dT = Tau1;
    r.dq = q1;
    return r;
}

struct Lane {
    double t, h, R, U, T, q;      // time, step, state
    double k1[4];                  // FSAL derivative at (t, y)
    bool have_k1;
    double fac_max;                // 5 at the start of a step, 0.9 after a rejection (G:244, G:299)
    long long nacc, nrej, nrej_step;
    double Rmax, Rmin, t_thr;
    bool thr;
};

// One Dormand-Prince attempt.  Returns true if the step was accepted.
// Follows G:240-317: clamp h to t_end, error norm G:183-192, controller G:296-310.
__device__ bool dp_attempt(const GilK& g, const OdeK& o, const Tones& d, double R0, double pin0, double t_end, Lane& L) {
    if (L.nrej_step == 0) {
        if (L.t + L.h > t_end) L.h = t_end - L.t;                     // G:240
        L.fac_max = o.fac_max;
    }
    const double h = L.h;
    double y[4] = {L.R, L.U, L.T, L.q};
    double K[7][4];
    double Yn[4], E[4];
    if (o.ref_arith) {
        // G:248-286, 7 stages, accumulation order of the reference
        for (int c = 0; c < 4; ++c) { Yn[c] = y[c]; E[c] = 0.0; }
        for (int i = 0; i < 7; ++i) {
            double kR = 0, kR1 = 0, kT = 0, kq = 0;
            for (int j = 0; j < i; ++j) {
                kR = kR + c_A[i][j] * K[j][0] * h;
                kR1 = kR1 + c_A[i][j] * K[j][1] * h;
                kT = kT + c_A[i][j] * K[j][2] * h;
                kq = kq + c_A[i][j] * K[j][3] * h;
            }
            K[i][0] = (y[1] + kR1);
            K[i][1] = ref_F_R(g, d, L.t + h * c_C[i], y[0] + kR, y[1] + kR1, y[2] + kT, y[3] + kq, R0);
            K[i][2] = ref_stress_dt(g, y[0] + kR, y[1] + kR1, y[2] + kT, R0);
            K[i][3] = ref_q_dt(g, y[0] + kR, y[1] + kR1, y[2] + kT, y[3] + kq, R0);
            for (int c = 0; c < 4; ++c) {
                Yn[c] = Yn[c] + c_B[i] * K[i][c] * h;
                E[c] = E[c] + K[i][c] * h * (c_B[i] - c_BB[i]);
            }
        }
    } else {
        // fast path: transcendentals and the drive expanded around the step start
        double s0[BD_MAX_BUBBLE_TONES], c0[BD_MAX_BUBBLE_TONES];
        for (int k = 0; k < d.n; ++k) sincos(2.0 * BD_PI_D * d.f[k] * L.t + d.phi[k], &s0[k], &c0[k]);
        DriveSeries ds;
        const bool dser = drive_series(d, s0, c0, h, ds);
        double Pb, Pdb;
        if (dser) { Pb = ds.p[0]; Pdb = ds.q[0]; }
        else drive_at(d, s0, c0, 0.0, Pb, Pdb);
        const RhsBase B = rhs_base(g, pin0, R0, y[0], y[2], Pb);
        if (!L.have_k1) {
            Rhs r = fast_rhs(g, pin0, R0, y[0], y[1], y[2], y[3], Pb, Pdb);
            L.k1[0] = r.dR; L.k1[1] = r.dU; L.k1[2] = r.dT; L.k1[3] = r.dq;
            L.have_k1 = true;
        }
        for (int c = 0; c < 4; ++c) K[0][c] = L.k1[c];
#pragma unroll
        for (int i = 1; i < 7; ++i) {
            double ys[4];
            for (int c = 0; c < 4; ++c) {
                double acc = 0.0;
#pragma unroll
                for (int j = 0; j < i; ++j) acc += c_A[i][j] * K[j][c];
                ys[c] = y[c] + h * acc;
            }
            double P, Pd;
            if (dser) ds.eval(c_C[i] * h, P, Pd);
            else drive_at(d, s0, c0, c_C[i] * h, P, Pd);
            Rhs r = series_rhs(g, B, pin0, R0, ys[0], ys[1], ys[2], ys[3], P, Pd);
            K[i][0] = r.dR; K[i][1] = r.dU; K[i][2] = r.dT; K[i][3] = r.dq;
            if (i == 6)
                for (int c = 0; c < 4; ++c) Yn[c] = ys[c];   // a[6][:] == b: stage 7 is the solution
        }
        for (int c = 0; c < 4; ++c) {
            double e = 0.0;
#pragma unroll
            for (int j = 0; j < 7; ++j) e += (c_B[j] - c_BB[j]) * K[j][c];
            E[c] = h * e;
        }
    }
    double max_result;
    if (o.ref_arith) {
        double S = 0.0;
        for (int c = 0; c < 4; ++c) {
            const double sc = o.atol + o.rtol * fmax(fabs(y[c]), fabs(Yn[c]));   // G:289-292
            const double r = E[c] / sc;
            S += r * r;
        }
        const double err = sqrt(S / 4.0);                                    // G:183-192
        max_result = fmax(0.1, 0.9 * pow(err, -0.2));                        // G:296
        if (err > 1.0) {                                                     // G:297-301
            L.fac_max = 0.9;
            L.h = h * fmin(L.fac_max, max_result);
            L.nrej++;
            L.nrej_step++;
            return false;
        }
    } else {
        // the same norm and controller in FP32 (they only choose h; the
        // reference-arithmetic path keeps G's FP64 expressions)
        float S = 0.0f;
        for (int c = 0; c < 4; ++c) {
            const double sc = o.atol + o.rtol * fmax(fabs(y[c]), fabs(Yn[c]));
            const float r = (float)E[c] / (float)sc;
            S = fmaf(r, r, S);
        }
        const float err = sqrtf(0.25f * S);
        const float mr = 0.9f * exp2f(-0.2f * log2f(err));
        max_result = err > 0.0f ? fmax(0.1, (double)mr) : 5.0;
        if (!(err <= 1.0f)) {
            L.fac_max = 0.9;
            L.h = h * fmin(L.fac_max, max_result);
            L.nrej++;
            L.nrej_step++;
            return false;
        }
    }
    L.t = L.t + h;                                                       // G:304-310
    L.R = Yn[0]; L.U = Yn[1]; L.T = Yn[2]; L.q = Yn[3];
    L.h = h * fmin(L.fac_max, max_result);
    if (!o.ref_arith) { for (int c = 0; c < 4; ++c) L.k1[c] = K[6][c]; L.have_k1 = true; }
    L.nacc++;
    L.nrej_step = 0;
    L.thr = Yn[1] <= -g.C_inf;                                           // G:313
    return true;
}

__device__ __forceinline__ void load_tones(const bd_bubble& b, Tones& d) {
    d.mode = 0;
    d.A = 0.0;
    d.n = min(max(b.n_tones, 0), BD_MAX_BUBBLE_TONES);
    for (int k = 0; k < d.n; ++k) { d.f[k] = b.f[k]; d.a[k] = b.a[k]; d.phi[k] = b.phi[k]; }
}

__device__ __forceinline__ void lane_reset(Lane& L, double R0, double h0) {
    L.t = 0.0; L.h = h0; L.R = R0; L.U = 0.0; L.T = 0.0; L.q = 0.0;
    L.have_k1 = false; L.fac_max = 5.0;
    L.nacc = 0; L.nrej = 0; L.nrej_step = 0;
    L.Rmax = R0; L.Rmin = R0; L.t_thr = -1.0; L.thr = false;
}

// One integration attempt of a bubble's lane; returns its final status or -1
// while it is still running.
__device__ __forceinline__ int lane_advance(const GilK& g, const OdeK& o, const Tones& d, double R0, double pin0,
                                            Lane& L) {
    const int max_rej_per_step = 200;
    if (L.t >= o.t_end) return BD_BUBBLE_DONE;
    if (L.nacc >= o.max_steps) return BD_BUBBLE_STEP_CAP;
    const bool acc = dp_attempt(g, o, d, R0, pin0, o.t_end, L);
    if (acc) {
        if (!isfinite(L.R) || !isfinite(L.U)) return BD_BUBBLE_NONFINITE;
        L.Rmax = fmax(L.Rmax, L.R);
        L.Rmin = fmin(L.Rmin, L.R);
        if (L.thr && L.t_thr < 0.0) L.t_thr = L.t;
        if (L.thr && o.stop_at_threshold) return BD_BUBBLE_THRESHOLD;
        if (L.t >= o.t_end) return BD_BUBBLE_DONE;
    } else if (L.nrej_step > max_rej_per_step || !(L.h > 0.0) || L.t + L.h == L.t) {
        return BD_BUBBLE_NONFINITE;   // step size collapsed: flagged, never a hang
    }
    return -1;
}

__device__ __forceinline__ void lane_write(const Lane& L, int status, bd_bubble_result* r_out) {
    bd_bubble_result r;
    r.R = L.R; r.Rdot = L.U; r.tau = L.T; r.q = L.q; r.t = L.t;
    r.R_max = L.Rmax; r.R_min = L.Rmin; r.t_threshold = L.t_thr;
    r.n_accept = L.nacc; r.n_reject = L.nrej;
    r.status = status; r.threshold = L.t_thr >= 0.0 ? 1 : 0;
    *r_out = r;
}

// Forward integration of every bubble; a lane whose bubble finishes pulls the
// next work item from *counter, so lanes of one warp never wait for the
// slowest bubble of a static assignment.
__global__ void __launch_bounds__(128) gilmore_persistent_kernel(const bd_bubble* __restrict__ bubbles, long long n,
                                                                 const GilK g, const OdeK o,
                                                                 bd_bubble_result* __restrict__ res,
                                                                 unsigned long long* __restrict__ counter) {
    Lane L;
    Tones d;
    long long item = -1;
    double R0 = 0.0, pin0 = 0.0;
    while (true) {
        if (item < 0) {
            item = (long long)atomicAdd(counter, 1ULL);
            if (item >= n) break;
            const bd_bubble& b = bubbles[item];
            R0 = b.R0;
            load_tones(b, d);
            pin0 = g.P0 + g.S2 / R0;
            lane_reset(L, R0, o.h0);
        }
        const int status = lane_advance(g, o, d, R0, pin0, L);
        if (status >= 0) {
            lane_write(L, status, res + item);
            item = -1;
        }
    }
}

// The same integration with one thread per bubble for its whole run (the
// static schedule that the persistent kernel is measured against).
__global__ void __launch_bounds__(128) gilmore_static_kernel(const bd_bubble* __restrict__ bubbles, long long n,
                                                             const GilK g, const OdeK o,
                                                             bd_bubble_result* __restrict__ res) {
    const long long item = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= n) return;
    Lane L;
    Tones d;
    const bd_bubble& b = bubbles[item];
    const double R0 = b.R0;
    load_tones(b, d);
    const double pin0 = g.P0 + g.S2 / R0;
    lane_reset(L, R0, o.h0);
    int status = -1;
    while (status < 0) status = lane_advance(g, o, d, R0, pin0, L);
    lane_write(L, status, res + item);
}

// Threshold search of G:323-429 as a per-lane state machine around one
// integration attempt per loop iteration.  Stage 1 steps A up by 0.1 MPa
// keeping h between amplitudes (G:372-380), stage 2 down by 10 kPa and stage 3
// down by 1 kPa with h reset to 1e-13 (G:391-426).
__global__ void __launch_bounds__(128) gilmore_threshold_kernel(const double* __restrict__ fr_combo, long long n_combo,
                                                                const double* __restrict__ R0s, long long n_R0,
                                                                const GilK g, const OdeK o, double* __restrict__ out,
                                                                unsigned long long* __restrict__ counter,
                                                                unsigned long long* __restrict__ capped,
                                                                int bisect) {
    const int max_rej_per_step = 200;
    const long long N = n_combo * n_R0;
    int ilo = 0, ihi = 0, imid = 0;   // bisection (stage 2) on A = A5 - 0.1 MPa + i kPa
    Lane L;
    Tones d;
    long long item = -1;
    double R0 = 0, pin0 = 0, endT = 0, f1 = 0, f2 = 0, f3 = 0;
    int stage = 0;           // 5, 4, 3: amplitude step 0.1 MPa, 10 kPa, 1 kPa
    double A5 = 0, A4 = 0, A3 = 0, A = 0, result = -1.0;
    bool th5 = false, th4 = true, th3 = true;
    bool running = false;
    long long steps_this = 0;
    while (true) {
        if (item < 0) {
            item = (long long)atomicAdd(counter, 1ULL);
            if (item >= N) break;
            const long long ic = item / n_R0, ir = item % n_R0;                // G:327-328
            R0 = R0s[ir];
            f1 = fr_combo[3 * ic]; f2 = fr_combo[3 * ic + 1]; f3 = fr_combo[3 * ic + 2];
            endT = 0.0;                                                       // G:342-353
            if (f1 <= f2 && f1 <= f3) endT = 5.0 / f1;
            if (f2 <= f1 && f2 <= f3) endT = 5.0 / f2;
            if (f3 <= f1 && f3 <= f2) endT = 5.0 / f3;
            pin0 = g.P0 + g.S2 / R0;
            result = -1.0;                                                    // G:359
            stage = 5; A5 = 0.0; A4 = 0.0; A3 = 0.0; th5 = false; th4 = true; th3 = true;
            lane_reset(L, R0, 1e-13);                                        // G:355
            running = false;
        }
        if (!running) {
            // next integration of the search, or the end of this work item
            bool start = false, finish = false;
            while (!start && !finish) {
                if (stage == 5) {
                    if (!th5 && A5 < 1e7) { A5 = A5 + 1e5; A = A5; start = true; }          // G:372-376 (h kept)
                    else {
                        if (!th5 && A5 == 1e7) result = A5;                              // G:383-387
                        A4 = A5;
                        if (bisect) { stage = 2; ilo = 0; ihi = 100; }
                        else stage = 4;
                    }
                } else if (stage == 2) {
                    // bisection between A5 - 0.1 MPa (below the threshold) and A5 (reached)
                    if (th5 && ihi - ilo > 1) {
                        imid = (ilo + ihi) / 2;
                        L.h = 1e-13;
                        A = (A5 - 1e5) + imid * 1e3;
                        start = true;
                    } else {
                        if (th5) result = (A5 - 1e5) + ihi * 1e3;
                        finish = true;
                    }
                } else if (stage == 4) {
                    if (th5 && th4) { L.h = 1e-13; A4 = A4 - 1e4; A = A4; start = true; }   // G:391-396
                    else { A3 = A4; stage = 3; }
                } else {
                    if (th5 && !th4 && th3) { L.h = 1e-13; A3 = A3 - 1e3; A = A3; start = true; }   // G:411-416
                    else finish = true;
                }
            }
            if (finish) {
                out[item] = result;
                item = -1;
                continue;
            }
            lane_reset(L, R0, L.h);                                           // G:374 / G:394 / G:414
            // combo drive of G:40-57 at amplitude A
            d.A = A;
            for (int k = 0; k < 3; ++k) d.phi[k] = 0.0;
            if (f1 == f2 && f1 == f3) { d.n = 1; d.mode = 1; d.f[0] = f1; d.a[0] = A; }
            else if (f1 == f2 || f2 == f3) {
                d.n = 2; d.mode = 2; d.f[0] = f1; d.f[1] = f3; d.a[0] = d.a[1] = A / sqrt(2.0);
            } else {
                d.n = 3; d.mode = 3; d.f[0] = f1; d.f[1] = f2; d.f[2] = f3; d.a[0] = d.a[1] = d.a[2] = A / sqrt(3.0);
            }
            running = true;
            steps_this = 0;
        }
        // one attempt of the running integration: while (t < endT && !thr) DPRK_step (G:378)
        bool ended = false, hit = false;
        if (!(L.t < endT)) ended = true;
        else {
            const bool acc = dp_attempt(g, o, d, R0, pin0, endT, L);
            if (acc) {
                ++steps_this;
                if (L.thr) { hit = true; ended = true; }
                else if (!(L.t < endT)) ended = true;
                else if (o.max_steps > 0 && steps_this >= o.max_steps) { ended = true; atomicAdd(capped, 1ULL); }
                else if (!isfinite(L.R)) { ended = true; atomicAdd(capped, 1ULL); }
            } else if (L.nrej_step > max_rej_per_step || !(L.h > 0.0) || L.t + L.h == L.t) {
                ended = true;
                atomicAdd(capped, 1ULL);
            }
        }
        if (ended) {
            running = false;
            if (stage == 5) th5 = hit;
            else if (stage == 2) { if (hit) ihi = imid; else ilo = imid; }
            else if (stage == 4) { th4 = hit; if (!th4) A4 = A4 + 1e4; }                  // G:401-405
            else if (stage == 3) { th3 = hit; if (!th3) result = A3 + 1e3; }               // G:421-424
        }
    }
}

static GilK make_gilk(const bd_gilmore_medium* m) {
    GilK g;
    g.rho = m->rho; g.P0 = m->P0; g.S2 = m->S2; g.mu4 = m->mu4; g.G4_3 = m->G4_3; g.C_inf = m->C_inf;
    g.lambda = m->lambda; g.n = m->n; g.B = m->B; g.gamma3 = 3.0 * m->gamma;
    g.n1n = (m->n - 1.0) / m->n;
    g.irho = 1.0 / m->rho; g.ilam = 1.0 / m->lambda; g.i3lam = 1.0 / (3.0 * m->lambda);
    g.nrho = m->n / (m->rho * (m->n - 1.0));
    g.iCinf = 1.0 / m->C_inf;
    return g;
}

static OdeK make_odek(const bd_ode_params* p) {
    OdeK o;
    o.t_end = p->t_end; o.h0 = p->h0; o.atol = p->atol; o.rtol = p->rtol; o.fac_max = p->fac_max;
    o.max_steps = p->max_steps > 0 ? p->max_steps : (long long)1 << 40;
    o.stop_at_threshold = p->stop_at_threshold; o.ref_arith = p->ref_arith;
    return o;
}

static void check_medium(const bd_gilmore_medium* m) {
    if (!m) fail(BD_ERR_INVALID_ARG, "null medium");
    if (!(m->rho > 0 && m->C_inf > 0 && m->lambda > 0 && m->n > 1 && m->gamma > 0))
        fail(BD_ERR_INVALID_ARG, "bad Gilmore medium constants");
}

static int persistent_grid(bd_context* ctx, const void* kernel) {
    int per_sm = 0;
    BD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 128, 0));
    return ctx->sm_count * std::max(per_sm, 1);
}

static void launch_run(bd_context* ctx, const bd_gilmore_medium* m, long long n, const bd_bubble* d_b,
                       const bd_ode_params* ode, bd_bubble_result* d_r, unsigned long long* d_counter,
                       cudaStream_t st) {
    const GilK g = make_gilk(m);
    const OdeK o = make_odek(ode);
    const int grid = persistent_grid(ctx, (const void*)gilmore_persistent_kernel);
    // with no more bubbles than resident lanes there is nothing to steal: full
    // warps of the static kernel do the same work (and give the same bits)
    if (ode->schedule == BD_SCHEDULE_STATIC || n <= (long long)grid * 128) {
        gilmore_static_kernel<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(d_b, n, g, o, d_r);
        BD_LAUNCHED(ctx);
        return;
    }
    BD_CUDA(cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), st));
    gilmore_persistent_kernel<<<grid, 128, 0, st>>>(d_b, n, g, o, d_r, d_counter);
    BD_LAUNCHED(ctx);
}

static void check_ode(const bd_ode_params* ode) {
    if (!ode) fail(BD_ERR_INVALID_ARG, "null ode params");
    if (!(ode->t_end > 0 && ode->h0 > 0 && ode->atol > 0 && ode->rtol > 0 && ode->fac_max > 0))
        fail(BD_ERR_INVALID_ARG, "bad ODE parameters");
}

}  // namespace bd

using namespace bd;

extern "C" {

bd_status bd_gilmore_run(bd_context* ctx, const bd_gilmore_medium* medium, int64_t n, const bd_bubble* bubbles,
                         const bd_ode_params* ode, bd_bubble_result* results, double* elapsed_ms) {
    return guard([&] {
        ctx_check(ctx);
        check_medium(medium);
        check_ode(ode);
        if (n < 0 || (n > 0 && (!bubbles || !results))) fail(BD_ERR_INVALID_ARG, "bad bubble arrays");
        if (n == 0) { if (elapsed_ms) *elapsed_ms = 0.0; return; }
        for (int64_t i = 0; i < n; ++i)
            if (!(bubbles[i].R0 > 0) || bubbles[i].n_tones < 0 || bubbles[i].n_tones > BD_MAX_BUBBLE_TONES)
                fail(BD_ERR_INVALID_ARG, "bubble %lld: bad R0 or n_tones", (long long)i);
        PoolBuf db, dr, dc;
        db.alloc(ctx, n * sizeof(bd_bubble));
        dr.alloc(ctx, n * sizeof(bd_bubble_result));
        dc.alloc(ctx, 64);
        cudaStream_t st = ctx->stream;
        BD_CUDA(cudaMemcpyAsync(db.p, bubbles, n * sizeof(bd_bubble), cudaMemcpyHostToDevice, st));
        BD_CUDA(cudaEventRecord(ctx->ev0, st));
        launch_run(ctx, medium, n, db.as<bd_bubble>(), ode, dr.as<bd_bubble_result>(), dc.as<unsigned long long>(), st);
        BD_CUDA(cudaEventRecord(ctx->ev1, st));
        BD_CUDA(cudaMemcpyAsync(results, dr.p, n * sizeof(bd_bubble_result), cudaMemcpyDeviceToHost, st));
        BD_CUDA(cudaStreamSynchronize(st));
        float ms = 0;
        BD_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
        if (elapsed_ms) *elapsed_ms = ms;
    });
}

bd_status bd_gilmore_run_device(bd_context* ctx, const bd_gilmore_medium* medium, int64_t n, const bd_bubble* d_bubbles,
                                const bd_ode_params* ode, bd_bubble_result* d_results, void* stream) {
    return guard([&] {
        ctx_check(ctx);
        check_medium(medium);
        check_ode(ode);
        if (n < 0 || (n > 0 && (!d_bubbles || !d_results))) fail(BD_ERR_INVALID_ARG, "bad bubble arrays");
        if (n == 0) return;
        cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
        // the persistent schedule's work counter belongs to the context (one per
        // context: calls on different streams whose work overlaps must be serialised)
        launch_run(ctx, medium, n, d_bubbles, ode, d_results, ctx->gil_counter, st);
    });
}

bd_status bd_gilmore_threshold(bd_context* ctx, const bd_gilmore_medium* medium, const double* fr_combo, int64_t n_combo,
                               const double* R0, int64_t n_R0, int32_t ref_arith, int64_t max_steps, double* results,
                               double* elapsed_ms) {
    return bd_gilmore_threshold_search(ctx, medium, fr_combo, n_combo, R0, n_R0, ref_arith, max_steps, BD_SEARCH_LINEAR,
                                       results, elapsed_ms);
}

bd_status bd_gilmore_threshold_search(bd_context* ctx, const bd_gilmore_medium* medium, const double* fr_combo,
                                      int64_t n_combo, const double* R0, int64_t n_R0, int32_t ref_arith,
                                      int64_t max_steps, int32_t search, double* results, double* elapsed_ms) {
    return guard([&] {
        ctx_check(ctx);
        check_medium(medium);
        if (search != BD_SEARCH_LINEAR && search != BD_SEARCH_BISECT)
            fail(BD_ERR_INVALID_ARG, "search must be BD_SEARCH_LINEAR or BD_SEARCH_BISECT");
        if (n_combo < 0 || n_R0 < 0 || ((n_combo * n_R0) > 0 && (!fr_combo || !R0 || !results)))
            fail(BD_ERR_INVALID_ARG, "bad threshold arrays");
        const long long N = n_combo * n_R0;
        if (N == 0) { if (elapsed_ms) *elapsed_ms = 0; return; }
        for (int64_t i = 0; i < n_R0; ++i) if (!(R0[i] > 0)) fail(BD_ERR_INVALID_ARG, "R0 must be positive");
        for (int64_t i = 0; i < 3 * n_combo; ++i) if (!(fr_combo[i] > 0)) fail(BD_ERR_INVALID_ARG, "frequencies must be positive");
        bd_ode_params op;
        std::memset(&op, 0, sizeof op);
        op.t_end = 1.0; op.h0 = 1e-13; op.atol = 1e-9; op.rtol = 1e-9; op.fac_max = 5.0;   // G:214-215, G:244
        op.max_steps = max_steps; op.stop_at_threshold = 1; op.ref_arith = ref_arith;
        const GilK g = make_gilk(medium);
        OdeK o = make_odek(&op);
        o.max_steps = max_steps > 0 ? max_steps : 0;
        PoolBuf dfr, dR0, dout, dc;
        dfr.alloc(ctx, 3 * n_combo * 8);
        dR0.alloc(ctx, n_R0 * 8);
        dout.alloc(ctx, N * 8);
        dc.alloc(ctx, 64);
        cudaStream_t st = ctx->stream;
        BD_CUDA(cudaMemcpyAsync(dfr.p, fr_combo, 3 * n_combo * 8, cudaMemcpyHostToDevice, st));
        BD_CUDA(cudaMemcpyAsync(dR0.p, R0, n_R0 * 8, cudaMemcpyHostToDevice, st));
        BD_CUDA(cudaMemsetAsync(dc.p, 0, 64, st));
        BD_CUDA(cudaEventRecord(ctx->ev0, st));
        const int grid = persistent_grid(ctx, (const void*)gilmore_threshold_kernel);
        unsigned long long* cnt = dc.as<unsigned long long>();
        gilmore_threshold_kernel<<<grid, 128, 0, st>>>(dfr.as<double>(), n_combo, dR0.as<double>(), n_R0, g, o,
                                                       dout.as<double>(), cnt, cnt + 1, search == BD_SEARCH_BISECT);
        BD_LAUNCHED(ctx);
        BD_CUDA(cudaEventRecord(ctx->ev1, st));
        BD_CUDA(cudaMemcpyAsync(results, dout.p, N * 8, cudaMemcpyDeviceToHost, st));
        unsigned long long capped = 0;
        BD_CUDA(cudaMemcpyAsync(&capped, cnt + 1, 8, cudaMemcpyDeviceToHost, st));
        BD_CUDA(cudaStreamSynchronize(st));
        float ms = 0;
        BD_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
        if (elapsed_ms) *elapsed_ms = ms;
        if (capped) set_error("%llu integrations stopped at the step cap or a collapsed step size", capped);
    });
}

}  // extern "C"
