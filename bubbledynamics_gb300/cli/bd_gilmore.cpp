// bd_gilmore — command-line driver that stands in for the reference program G
// (Gilmore_liver_3fr_combo.cu, main at G:433-631): the medium constants
// (G:440-470), the 27,775 frequency combinations (G:498-520), the R0 ladder
// (G:457-460), the cavitation-threshold search (G:573) through
// bd_gilmore_threshold_search, and G's result table (G:582-613).
//
//   bd_gilmore [--combo-first I] [--combo-count N] [--r0-first J] [--r0-count M]
//              [--max-steps S] [--bisect] [--fast] [--device D] [--out FILE]
//
// Without options it searches every (combination, R0) pair like G; the
// options select a block of the table (the tests run a small one).  --fast
// evaluates the right-hand side with the library's shared-transcendental
// arithmetic instead of G's operation order; --bisect bisects the last 0.1 MPa
// bracket instead of G's 10 kPa / 1 kPa descent.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "cli_common.h"

int main(int argc, char** argv) {
    const char* usage =
        "bd_gilmore [--combo-first I] [--combo-count N] [--r0-first J] [--r0-count M]\n"
        "           [--max-steps S] [--bisect] [--fast] [--device D] [--out FILE]\n"
        "Cavitation thresholds of the reference program G; writes dR_Cinf_liver_fr3_combo_all.dat\n";
    cli::Args args(argc, argv, usage);

    // G:440-450
    bd_gilmore_medium m;
    m.rho = 1100.0;
    m.P0 = 1.013e5;
    m.S2 = 2.0 * 0.056;
    m.mu4 = 4.0 * 0.009;
    m.G4_3 = 0.04e6 * 4.0 / 3.0;
    m.C_inf = 1549.0;
    m.lambda = 3.0e-9;
    m.n = 7.0;
    m.B = (m.C_inf * m.C_inf * m.rho / m.n) - m.P0;
    m.gamma = 1.4;

    // G:498-520: 55 log-spaced frequencies in [0.02, 5] MHz, ordered triples
    int64_t n_all = 0;
    cli::check(bd_gilmore_combos(55, 0.02e6, 5.0e6, nullptr, 0, &n_all), "bd_gilmore_combos");
    std::vector<double> combos(3 * n_all);
    cli::check(bd_gilmore_combos(55, 0.02e6, 5.0e6, combos.data(), n_all, &n_all), "bd_gilmore_combos");
    // G:457-460: R0 = 0.1 .. 10 um in 0.1 um steps
    const double stepR0 = 1e-7, minR0 = 1e-7, maxR0 = 1e-5;
    const int n_R0_all = 1 + (int)((maxR0 - minR0) / stepR0);
    std::vector<double> R0_all(n_R0_all);
    for (int i = 0; i < n_R0_all; ++i) R0_all[i] = minR0 + i * stepR0;

    const long long c0 = std::max(0LL, args.i("combo-first", 0));
    const long long nc = std::min<long long>(args.i("combo-count", n_all), n_all - c0);
    const long long r0 = std::max(0LL, args.i("r0-first", 0));
    const long long nr = std::min<long long>(args.i("r0-count", n_R0_all), n_R0_all - r0);
    if (nc <= 0 || nr <= 0) {
        std::fprintf(stderr, "empty selection\n%s", usage);
        return 2;
    }
    std::vector<double> results((size_t)nc * nr);
    bd_context* ctx = nullptr;
    cli::check(bd_context_create((int)args.i("device", 0), &ctx), "bd_context_create");
    double ms = 0.0;
    const bd_status st = bd_gilmore_threshold_search(ctx, &m, combos.data() + 3 * c0, nc, R0_all.data() + r0, nr,
                                                     args.has("fast") ? 0 : 1, args.i("max-steps", 0),
                                                     args.has("bisect") ? BD_SEARCH_BISECT : BD_SEARCH_LINEAR,
                                                     results.data(), &ms);
    cli::check(st, "bd_gilmore_threshold_search");
    if (bd_last_error_string()[0]) std::fprintf(stderr, "note: %s\n", bd_last_error_string());
    std::printf("%lld combinations x %lld radii in %.3f s of device time\n", nc, nr, ms * 1e-3);
    cli::check(bd_write_threshold_table(args.str("out", "dR_Cinf_liver_fr3_combo_all.dat").c_str(),
                                        combos.data() + 3 * c0, nc, R0_all.data() + r0, nr, results.data(),
                                        ms * 1e-3),
               "bd_write_threshold_table");
    cli::check(bd_context_destroy(ctx), "bd_context_destroy");
    return 0;
}
