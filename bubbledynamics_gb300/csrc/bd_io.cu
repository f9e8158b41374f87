// Readers and writers of the reference programs' files, so results move in
// and out of the reference's workflow unchanged (host code only):
//   - W's absorbed-power volume, Q3D_*.bin (W:778-790): raw doubles, planes
//     iz = iz_first .. nz-1 (W writes from iz = 2, the plane z = 0), rows iy,
//     columns ix; read back by T (T:276-279) as (Nxy_half+1)^2 x Nz doubles;
//   - W's on-axis power, Q_Z_*.dat (W:767-775): "z(m);Q(W/m^3)" then one
//     "z;Q" line per plane from iz_first;
//   - T's temperature / dose slices, T_XZ_* / T_XY_* / TD_* .dat (T:419-448,
//     T:576-640): a header row, then one row per slice row of "value;" cells;
//   - G's threshold table, dR_Cinf_*.dat (G:582-613): "fr1;fr2;fr3 --> R0;R0..."
//     then one row per combination and a final "time (s);t" row.
// Numbers are written like a default C++ stream (6 significant digits).
#include <cstdio>
#include <cstring>
#include <string>

#include "bd_internal.h"

namespace bd {

struct File {
    FILE* f = nullptr;
    File(const char* path, const char* mode) {
        f = std::fopen(path, mode);
        if (!f) fail(BD_ERR_IO, "cannot open %s", path);
    }
    ~File() {
        if (f) std::fclose(f);
    }
    void put(const char* s) {
        if (std::fputs(s, f) < 0) fail(BD_ERR_IO, "write failed");
    }
    void num(double v) {
        char b[64];
        std::snprintf(b, sizeof b, "%g", v);
        put(b);
    }
};

}  // namespace bd

using namespace bd;

extern "C" {

bd_status bd_write_q_bin(const char* path, const double* Q, int32_t nx, int32_t ny, int32_t nz, int32_t iz_first) {
    return guard([&] {
        if (!path || !Q || nx <= 0 || ny <= 0 || nz <= 0 || iz_first < 0 || iz_first > nz)
            fail(BD_ERR_INVALID_ARG, "bad arguments");
        File f(path, "wb");
        const size_t plane = (size_t)nx * ny;
        const size_t n = plane * (size_t)(nz - iz_first);
        if (n && std::fwrite(Q + (size_t)iz_first * plane, sizeof(double), n, f.f) != n)
            fail(BD_ERR_IO, "short write to %s", path);
    });
}

bd_status bd_read_q_bin(const char* path, double* out, int64_t n, int64_t* n_read) {
    return guard([&] {
        if (!path || (!out && n > 0) || n < 0) fail(BD_ERR_INVALID_ARG, "bad arguments");
        File f(path, "rb");
        const size_t got = n > 0 ? std::fread(out, sizeof(double), (size_t)n, f.f) : 0;
        if (n_read) *n_read = (int64_t)got;
        if ((int64_t)got != n) fail(BD_ERR_IO, "%s holds %lld doubles, %lld requested", path, (long long)got, (long long)n);
    });
}

bd_status bd_write_q_axis_dat(const char* path, const double* Q, int32_t nx, int32_t ny, int32_t nz, double z_min,
                              double dz, int32_t iz_first) {
    return guard([&] {
        if (!path || !Q || nx <= 0 || ny <= 0 || nz <= 0 || iz_first < 0) fail(BD_ERR_INVALID_ARG, "bad arguments");
        File f(path, "w");
        f.put("z(m);Q(W/m^3)");
        const size_t plane = (size_t)nx * ny;
        for (int iz = iz_first; iz < nz; ++iz) {
            f.put("\n");
            f.num(z_min + iz * dz);
            f.put(";");
            f.num(Q[(size_t)iz * plane]);        // x = y = 0
        }
    });
}

bd_status bd_write_slice_dat(const char* path, const double* field, int32_t nx, int32_t ny, int32_t nz,
                             int32_t orientation, int32_t fixed, int32_t r0, int32_t r1, int32_t c0, int32_t c1,
                             const char* header) {
    return guard([&] {
        if (!path || !field || nx <= 0 || ny <= 0 || nz <= 0) fail(BD_ERR_INVALID_ARG, "bad arguments");
        const bool xz = orientation == BD_SLICE_XZ;
        if (!xz && orientation != BD_SLICE_XY) fail(BD_ERR_INVALID_ARG, "orientation must be BD_SLICE_XZ or BD_SLICE_XY");
        const int rows = xz ? nz : ny;
        if (r0 < 0 || r1 > rows || r0 > r1 || c0 < 0 || c1 > nx || c0 > c1) fail(BD_ERR_INVALID_ARG, "slice range");
        if (fixed < 0 || fixed >= (xz ? ny : nz)) fail(BD_ERR_INVALID_ARG, "slice index");
        File f(path, "w");
        f.put(header ? header : (xz ? "Z=rows;X=columns" : "Y=rows;X=columns"));
        const size_t plane = (size_t)nx * ny;
        for (int r = r0; r < r1; ++r) {
            f.put("\n");
            for (int c = c0; c < c1; ++c) {
                const size_t i = xz ? (size_t)r * plane + (size_t)fixed * nx + c : (size_t)fixed * plane + (size_t)r * nx + c;
                f.num(field[i]);
                f.put(";");
            }
        }
    });
}

bd_status bd_write_threshold_table(const char* path, const double* fr_combo, int64_t n_combo, const double* R0,
                                   int64_t n_R0, const double* results, double elapsed_s) {
    return guard([&] {
        if (!path || !fr_combo || !R0 || !results || n_combo < 0 || n_R0 < 0) fail(BD_ERR_INVALID_ARG, "bad arguments");
        File f(path, "w");
        f.put("fr1;fr2;fr3 --> R0");
        for (int64_t j = 0; j < n_R0; ++j) {
            f.put(";");
            f.num(R0[j]);
        }
        for (int64_t i = 0; i < n_combo; ++i) {
            f.put("\n");
            for (int k = 0; k < 3; ++k) {
                if (k) f.put(";");
                f.num(fr_combo[3 * i + k]);
            }
            for (int64_t j = 0; j < n_R0; ++j) {
                f.put(";");
                f.num(results[i * n_R0 + j]);
            }
        }
        f.put("\ntime (s);");
        f.num(elapsed_s);
    });
}

}  // extern "C"
