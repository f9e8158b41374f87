// bd_westervelt — command-line driver that stands in for the reference
// program W (Westervelt_relax_fft_Pressure_Energy.cu, main at W:350-843):
// the reference's parameter block (W:355-416), one bd_westervelt_run in place
// of its three time loops and FFT pass (W:558-757), and its two output files
// (W:767-790) written through the library's writers.
//
//   bd_westervelt [--mini] [--nxy N] [--nz N] [--loop1-periods P] [--periods P]
//                 [--precision f64|f32] [--device D] [--out-dir DIR]
//
// Without options it runs the reference's own problem (426 x 426 x 2003 cells,
// 165 periods, then 4 periods of harmonics).  --mini keeps the reference's
// physics and discretisation on a small box with a scaled bowl (the problem the
// tests run).
#include <cmath>
#include <cstdio>
#include <vector>

#include "cli_common.h"

namespace {

const double kPi = 3.14159265358979323846;

// Host constants of W:355-416.
struct WConst {
    double fr, d, alpha, alpha_hole, p0;
    double rho_w, c_w, abs_w, delta_w, beta_w;
    double rho_t, c_t, beta_t, abs_t, delta_t, c1, c2, tau1, tau2;
    double water_tissue, xy_min, dxy, z_min, dz, dt, t_max;
    int Nxy, Nz, periods, N_harm, iz_tissue;
};

WConst reference_constants() {
    WConst k;
    k.fr = 1.253e6;
    k.d = 0.15;
    const double a = 0.151 / 2.0, a_hole = 0.041 / 2.0;
    const double h = k.d - std::sqrt(k.d * k.d - a * a);
    k.alpha = std::asin(a / k.d);
    k.alpha_hole = std::asin(a_hole / k.d);
    k.rho_w = 1000.0;
    k.c_w = 1500.0;
    k.abs_w = 0.026 * std::pow(k.fr / 1e6, 2);
    k.delta_w = (2.0 * k.abs_w * std::pow(k.c_w, 3)) / std::pow(2.0 * kPi * k.fr, 2);
    k.beta_w = 3.5;
    k.rho_t = 1055.0;
    k.c_t = 1600.0;
    k.beta_t = 4.5;
    k.abs_t = 7.2 * k.fr / 1e6;
    k.delta_t = 4.2318e-5;
    k.c1 = 4.03536;
    k.c2 = 6.14150;
    k.tau1 = 1.6178e-8;
    k.tau2 = 1.1494e-7;
    const double eps = 0.89, E = 100.0;
    const double u0 = std::sqrt(2.0 * E * eps / (k.rho_w * k.c_w * 2.0 * kPi * k.d * h));
    k.p0 = k.rho_w * k.c_w * u0;
    k.water_tissue = 0.12;
    k.xy_min = 0.0;
    k.dxy = 0.0002;
    k.Nxy = 1 + (int)std::lround((0.085 - k.xy_min) / k.dxy);
    k.z_min = -0.0002;
    k.dz = 0.0001;
    k.Nz = 1 + (int)std::lround((0.2 - k.z_min) / k.dz);
    k.dt = 0.01 / k.fr;
    k.t_max = 165.0 / k.fr;
    k.periods = 4;
    k.N_harm = 10;
    k.iz_tissue = 1202;
    return k;
}

// The reference physics on a small box: the same media and discretisation, a
// 5 mm bowl whose ring and focus fall inside the box.
void make_mini(WConst& k, int Nxy, int Nz, int loop1_periods, int periods) {
    k.Nxy = Nxy;
    k.Nz = Nz;
    k.d = 0.005;
    k.alpha = std::asin(0.004 / k.d);
    k.alpha_hole = std::asin(0.0008 / k.d);
    k.p0 = 2.0e5;
    k.water_tissue = 0.003;
    k.t_max = loop1_periods / k.fr;
    k.periods = periods;
    k.iz_tissue = Nz;
    for (int iz = 0; iz < Nz; ++iz)
        if (!(k.z_min + iz * k.dz < k.water_tissue)) { k.iz_tissue = iz; break; }
}

bd_material material(double c0, double rho, double beta, double delta, double absorption) {
    bd_material m;
    std::memset(&m, 0, sizeof m);
    m.c0 = c0;
    m.rho = rho;
    m.beta = beta;
    m.delta = delta;
    m.absorption = absorption;
    return m;
}

}  // namespace

int main(int argc, char** argv) {
    const char* usage =
        "bd_westervelt [--mini] [--nxy N] [--nz N] [--loop1-periods P] [--periods P]\n"
        "              [--precision f64|f32] [--device D] [--out-dir DIR]\n"
        "Westervelt pressure + acoustic power of the reference program W; writes\n"
        "Q_Z_E100_space6_att9_abs7_2_c1600_relax_fft_v3.dat and Q3D_E100_space6_att9_abs7_2_c1600_relax_fft_v3.bin\n";
    cli::Args args(argc, argv, usage);
    WConst k = reference_constants();
    if (args.has("mini"))
        make_mini(k, (int)args.i("nxy", 32), (int)args.i("nz", 64), (int)args.i("loop1-periods", 3),
                  (int)args.i("periods", 4));
    else if (args.has("nxy") || args.has("nz"))
        std::fprintf(stderr, "--nxy / --nz apply with --mini only; running the reference size\n");
    const int precision = args.str("precision", "f64") == "f32" ? BD_F32 : BD_F64;

    // time loops: `while (t < t_max) t += dt` (W:558-564), then 4 periods of
    // 100 steps from the same clock (W:668, W:690-714); the water power runs
    // one period after t_max (W:627)
    std::vector<double> t_src;
    double t = 0.0;
    while (t < k.t_max) { t = t + k.dt; t_src.push_back(t); }
    const long long n1 = (long long)t_src.size();
    const double t165 = t;
    long long n_water = 0;
    for (double tw = t165; tw < k.t_max + 1.0 / k.fr; tw = tw + k.dt) ++n_water;
    const long long n_time = 100LL * k.periods;
    for (long long s = 0; s < n_time; ++s) { t = t + k.dt; t_src.push_back(t); }
    const long long n_steps = n1 + n_time;

    bd_grid g;
    std::memset(&g, 0, sizeof g);
    g.nx = g.ny = k.Nxy;
    g.nz = k.Nz;
    g.x0 = g.y0 = k.xy_min;
    g.z0 = k.z_min;
    g.dx = k.dxy;
    g.dz = k.dz;
    g.dt = k.dt;
    // quarter domain: mirror planes at x = 0 and y = 0 (W:176-200), Mur elsewhere (W:88-135)
    const int faces[6] = {BD_FACE_MIRROR, BD_FACE_MUR, BD_FACE_MIRROR, BD_FACE_MUR, BD_FACE_MUR, BD_FACE_MUR};
    for (int f = 0; f < 6; ++f) g.face[f] = faces[f];
    g.mur_layers = 3;

    bd_medium med;
    std::memset(&med, 0, sizeof med);
    med.n_materials = 2;
    med.mat[0] = material(k.c_w, k.rho_w, k.beta_w, k.delta_w, k.abs_w);
    med.mat[1] = material(k.c_t, k.rho_t, k.beta_t, k.delta_t, k.abs_t);
    med.mat[1].n_relax = 2;
    med.mat[1].relax_c[0] = k.c1;
    med.mat[1].relax_c[1] = k.c2;
    med.mat[1].relax_tau[0] = k.tau1;
    med.mat[1].relax_tau[1] = k.tau2;
    med.mat[1].harm_absorption = 7.2;
    std::vector<int32_t> planes(k.Nz);
    for (int iz = 0; iz < k.Nz; ++iz) planes[iz] = (k.z_min + iz * k.dz) < k.water_tissue ? 0 : 1;   // W:212
    med.plane_material = planes.data();

    bd_source src;
    std::memset(&src, 0, sizeof src);
    src.kind = BD_SRC_BOWL;
    src.plane_iz = 2;                          // W:75
    src.focal_length = k.d;
    src.alpha = k.alpha;
    src.alpha_hole = k.alpha_hole;
    src.p0 = k.p0;
    src.c_delay = k.c_w;
    src.n_tones = 1;
    src.freq[0] = k.fr;
    src.amp[0] = 1.0;

    bd_westervelt_params p;
    std::memset(&p, 0, sizeof p);
    p.precision = precision;
    p.energy_mode = BD_ENERGY_DPDT2;           // W:253-257
    p.n_steps = n_steps;
    p.t_src = t_src.data();
    p.peak_start = 0;
    p.peak_end = n_steps;
    p.energy_start = n1;
    p.energy_end = n1 + n_water;
    p.dft_start = n1;
    p.dft_len = n_time;
    p.n_dft = k.N_harm;
    for (int j = 0; j < k.N_harm; ++j) p.dft_freq[j] = (j + 1) * k.fr;   // bins 4n of the 400-sample window
    p.dft_z_lo = k.iz_tissue;
    p.dft_z_hi = k.Nz;
    p.q_mode = BD_Q_REFERENCE;
    p.q_iz_split = k.iz_tissue;
    p.q_n_harm = k.N_harm;
    p.q_freq = k.fr;
    p.fault_at_step = -1;
    p.tile_variant = -1;
    p.relax_scheme = BD_RELAX_REFERENCE;

    bd_context* ctx = nullptr;
    cli::check(bd_context_create((int)args.i("device", 0), &ctx), "bd_context_create");
    const size_t n = (size_t)k.Nxy * k.Nxy * k.Nz;
    std::vector<double> Q(n);
    bd_westervelt_outputs out;
    std::memset(&out, 0, sizeof out);
    out.Q = Q.data();
    cli::check(bd_westervelt_run(ctx, &g, &med, &src, &p, &out), "bd_westervelt_run");
    std::printf("%lld steps on %d x %d x %d cells in %.3f s of device time\n", (long long)out.steps_done, k.Nxy,
                k.Nxy, k.Nz, out.elapsed_ms * 1e-3);
    const std::string dir = args.str("out-dir", ".");
    cli::check(bd_write_q_axis_dat(cli::join(dir, "Q_Z_E100_space6_att9_abs7_2_c1600_relax_fft_v3.dat").c_str(),
                                   Q.data(), k.Nxy, k.Nxy, k.Nz, k.z_min, k.dz, 2),
               "bd_write_q_axis_dat");
    cli::check(bd_write_q_bin(cli::join(dir, "Q3D_E100_space6_att9_abs7_2_c1600_relax_fft_v3.bin").c_str(), Q.data(),
                              k.Nxy, k.Nxy, k.Nz, 2),
               "bd_write_q_bin");
    cli::check(bd_context_destroy(ctx), "bd_context_destroy");
    return 0;
}
