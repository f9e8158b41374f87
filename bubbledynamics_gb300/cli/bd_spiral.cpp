// bd_spiral — command-line driver that stands in for the reference program T
// (Westervelt_Temperature_SquareSpiral.cu, main at T:109-683): the parameter
// block (T:114-166), W's quarter-domain power volume read and mirrored into
// the full domain (T:269-306), the heat + CEM43 run along the square spiral
// (T:323-566) through bd_spiral_heat_run, and T's slice files (T:411-638).
//
//   bd_spiral [--mini] [--nxy-half H] [--nz N] [--legs L] [--q-bin FILE | --gaussian QMAX]
//             [--precision f64|f32] [--device D] [--out-dir DIR]
//
// Without options it reads Q3D_E100_space6_att9_abs7_2_c1600_relax_fft_v3.bin
// (written by bd_westervelt) and runs the reference's own problem (851 x 851 x
// 2001 cells, 13 legs).  --mini keeps the physics on a small box with a faster,
// tighter spiral; --gaussian replaces the file by a Gaussian focal source.
// Slice positions are the reference's (y = 0, z = 12..17 cm, x = -2..2 cm,
// planes at 15 / 13.5 / 12.5 cm), clipped to the box.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "cli_common.h"

namespace {

struct TConst {
    double dxy, dz, dt, rho_w, ct_w, K_w, rho_t, ct_t, K_t, c_t_sound, water_tissue, T0, T0_w;
    double speed, scale, speed_init, t_acc;
    int Nxy_half, Nz, legs;
};

TConst reference_constants() {
    TConst k;
    k.dxy = 0.0002;
    k.Nxy_half = (1 + (int)std::lround((0.085 - -0.085) / k.dxy)) / 2;
    k.dz = 0.0001;
    k.Nz = 1 + (int)std::lround(0.2 / k.dz);
    k.dt = 0.001;
    k.rho_w = 1000.0; k.ct_w = 4200.0; k.K_w = 0.6;
    k.rho_t = 1055.0; k.ct_t = 3700.0; k.K_t = 0.51;
    k.c_t_sound = 1600.0;
    k.water_tissue = 0.12;
    k.T0 = 23.6 + 273.15;
    k.T0_w = 22.7 + 273.15;
    k.speed = 2.0e-3;
    k.scale = 3.0e-3;
    k.speed_init = 0.05e-3;
    k.t_acc = 0.15;
    k.legs = 13;
    return k;
}

int clampi(int v, int lo, int hi) { return std::max(lo, std::min(hi, v)); }

}  // namespace

int main(int argc, char** argv) {
    const char* usage =
        "bd_spiral [--mini] [--nxy-half H] [--nz N] [--legs L] [--q-bin FILE | --gaussian QMAX]\n"
        "          [--precision f64|f32] [--device D] [--out-dir DIR]\n"
        "Bioheat + CEM43 dose of the reference program T along its square spiral; writes T's\n"
        "T_XZ_* / T_XY_* snapshots after legs 1, 5, 9, 13 and the TD_* dose slices\n";
    cli::Args args(argc, argv, usage);
    TConst k = reference_constants();
    if (args.has("mini")) {
        k.Nxy_half = (int)args.i("nxy-half", 20);
        k.Nz = (int)args.i("nz", 48);
        k.water_tissue = 0.0024;
        k.speed = 0.02;
        k.scale = 0.0006;
        k.t_acc = 0.02;
        k.legs = (int)args.i("legs", 3);
    }
    const int Nxy = 2 * k.Nxy_half + 1, Nz = k.Nz;
    const long long plane = (long long)Nxy * Nxy, n = plane * Nz;
    const std::string dir = args.str("out-dir", ".");

    // heat source: W's quarter domain mirrored into the full one (T:269-306), or a Gaussian
    std::vector<double> Q(n, 0.0);
    if (args.has("gaussian")) {
        const double qmax = args.f("gaussian", 1e7);
        const double cz = 0.6 * Nz, sz = std::max(1.0, Nz / 16.0), sxy = std::max(1.0, Nxy / 20.0);
        for (int iz = 0; iz < Nz; ++iz)
            for (int iy = 0; iy < Nxy; ++iy)
                for (int ix = 0; ix < Nxy; ++ix) {
                    const double a = (iz - cz) / sz, b = (iy - k.Nxy_half) / sxy, c = (ix - k.Nxy_half) / sxy;
                    Q[(iz * (long long)Nxy + iy) * Nxy + ix] = qmax * std::exp(-0.5 * (a * a + b * b + c * c));
                }
    } else {
        const long long ns = (long long)(k.Nxy_half + 1) * (k.Nxy_half + 1) * Nz;
        std::vector<double> small(ns);
        const std::string path = args.str("q-bin", cli::join(dir, "Q3D_E100_space6_att9_abs7_2_c1600_relax_fft_v3.bin"));
        int64_t got = 0;
        cli::check(bd_read_q_bin(path.c_str(), small.data(), ns, &got), "bd_read_q_bin");
        cli::check(bd_unfold_quarter(small.data(), k.Nxy_half, Nz, Q.data()), "bd_unfold_quarter");
    }

    bd_thermal th;
    std::memset(&th, 0, sizeof th);
    th.nx = th.ny = Nxy;
    th.nz = Nz;
    th.precision = args.str("precision", "f64") == "f32" ? BD_F32 : BD_F64;
    th.dx = k.dxy;
    th.dz = k.dz;
    th.dt = k.dt;
    th.T_ref = k.T0;
    th.n_materials = 2;
    th.dose_init = 1;                          // T:246, T:252
    th.mat[0] = bd_thermal_material{k.rho_w, k.ct_w, k.K_w, 0.0, k.T0_w, k.T0_w};
    th.mat[1] = bd_thermal_material{k.rho_t, k.ct_t, k.K_t, 0.0, k.T0, k.T0};
    std::vector<int32_t> planes(Nz);
    for (int iz = 0; iz < Nz; ++iz) planes[iz] = iz * k.dz < k.water_tissue ? 0 : 1;   // T:79, T:84
    th.plane_material = planes.data();

    bd_trajectory tr;
    std::memset(&tr, 0, sizeof tr);
    tr.kind = BD_TRAJ_SQUARE_SPIRAL;
    tr.n_legs = k.legs;
    tr.speed = k.speed;
    tr.scale = k.scale;
    tr.speed_init = k.speed_init;
    tr.t_acc = k.t_acc;
    tr.dxy = k.dxy;
    tr.dt = k.dt;

    // snapshots after legs 1, 5, 9, 13 (T:412-563), those the run has
    std::vector<int32_t> legs;
    for (int l : {1, 5, 9, 13})
        if (l <= k.legs) legs.push_back(l);
    std::vector<double> T(n), TD(n), snaps(legs.size() * (size_t)n);
    bd_heat_outputs out;
    std::memset(&out, 0, sizeof out);
    out.T_final = T.data();
    out.dose = TD.data();
    out.snapshots = snaps.data();
    out.snapshot_legs = legs.data();
    out.n_snap = (int32_t)legs.size();
    bd_context* ctx = nullptr;
    cli::check(bd_context_create((int)args.i("device", 0), &ctx), "bd_context_create");
    cli::check(bd_spiral_heat_run(ctx, &th, Q.data(), &tr, 0, &out), "bd_spiral_heat_run");
    std::printf("%lld heat steps on %d x %d x %d cells in %.3f s of device time\n", (long long)out.steps_done, Nxy,
                Nxy, Nz, out.elapsed_ms * 1e-3);

    // slice positions of T:424-445 and T:578-636 from their coordinates, clipped to the box
    const int h = k.Nxy_half;
    const int x0 = clampi(h - 100, 0, Nxy), x1 = clampi(h + 101, 0, Nxy), x1d = clampi(h + 102, 0, Nxy);
    int zr0 = (int)std::lround(0.12 / k.dz);
    int zr1 = clampi((int)std::lround(0.17 / k.dz) + 1, 0, Nz), zd1 = clampi((int)std::lround(0.16 / k.dz) + 1, 0, Nz);
    if (zr0 >= Nz) { zr0 = 0; zr1 = Nz; zd1 = Nz; }   // a box shorter than 12 cm: every plane
    auto plane_at = [&](double z) { return clampi((int)std::lround(z / k.dz), 0, Nz - 1); };
    char name[256];
    for (size_t s = 0; s < legs.size(); ++s) {
        const double* f = snaps.data() + s * (size_t)n;
        std::snprintf(name, sizeof name, "T_XZ_E100_2mms_3mm_att9_abs7_2_c1600_relax_v2_loop%zu.dat", s);
        cli::check(bd_write_slice_dat(cli::join(dir, name).c_str(), f, Nxy, Nxy, Nz, BD_SLICE_XZ, h, zr0, zr1, x0, x1,
                                      nullptr), "bd_write_slice_dat");
        std::snprintf(name, sizeof name, "T_XY_E100_2mms_3mm_att9_abs7_2_c1600_relax_v2_loop%zu_z15.dat", s);
        cli::check(bd_write_slice_dat(cli::join(dir, name).c_str(), f, Nxy, Nxy, Nz, BD_SLICE_XY, plane_at(0.15), x0,
                                      x1, x0, x1, nullptr), "bd_write_slice_dat");
    }
    char hdr[256];
    const char* tail = "speed=;%g;c_t=;%g;K_t=;%g";
    char params[128];
    std::snprintf(params, sizeof params, tail, k.c_t_sound, k.ct_t, k.K_t);
    std::snprintf(hdr, sizeof hdr, "Z=rows;X=columns;%s", params);
    cli::check(bd_write_slice_dat(cli::join(dir, "TD_XZ_E100_2mms_3mm_att9_abs7_2_c1600_relax_v2.dat").c_str(),
                                  TD.data(), Nxy, Nxy, Nz, BD_SLICE_XZ, h, zr0, zd1, x0, x1d, hdr),
               "bd_write_slice_dat");
    const struct { double z; const char *tag, *label; } xy[] = {
        {0.15, "15", "15"}, {0.135, "13_5", "13.5"}, {0.125, "12_5", "12.5"}};
    for (const auto& p : xy) {
        std::snprintf(hdr, sizeof hdr, "Y=rows;X=columns;z=%scm;%s", p.label, params);
        std::snprintf(name, sizeof name, "TD_XY_E100_2mms_3mm_att9_abs7_2_c1600_relax_v2_z%s.dat", p.tag);
        cli::check(bd_write_slice_dat(cli::join(dir, name).c_str(), TD.data(), Nxy, Nxy, Nz, BD_SLICE_XY,
                                      plane_at(p.z), x0, x1, x0, x1d, hdr),
                   "bd_write_slice_dat");
    }
    cli::check(bd_context_destroy(ctx), "bd_context_destroy");
    return 0;
}
