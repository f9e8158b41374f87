// Westervelt solver: host driver behind bd_westervelt_run / _begin / _advance /
// _finish / checkpoints, the z-slab sessions and runs (bd_westervelt_slab_begin,
// bd_westervelt_run_slabs) and the adjoint (bd_westervelt_adjoint, _slabs).
// Replaces the host program W:350-790.
//
// Device layout (cells x-fastest, W:155):
//   P[5]          pressure ring; at step s the buffer (4s + k) mod 5 holds p^{s-k}
//                 and p^{s+1} is written over p^{s-4} (replaces W:575-579)
//   R[v][2]       relaxation ring; R^n is written over R^{n-2} (replaces W:581-584)
//   peak, energy  accumulators on every cell; dre/dim DFT planes [n_dft][planes]
// Steps are issued in chunks of K (a multiple of 10, so that the ring
// arrangement repeats) captured once as a CUDA graph and replayed; every
// step-dependent value is read from device tables indexed by a device step
// counter, so one graph serves every chunk.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include <cudaTypedefs.h>

#include "bd_internal.h"
#include "wv_kernels.cuh"
#include "wv_tma.cuh"
#include "wv_adjoint.cuh"
#include "wv_tma_pair.h"

namespace bd {

// Kernel variants: 0-7 plain (read-only-cache neighbours), 8-23 TMA-pipelined
// (need a row pitch that is a multiple of 16 bytes).  19-23 take two adjacent
// x cells per thread (wv_tma_pair_kernel, pointwise ring of nq slots) and are
// built for FP32 fields with at most two relaxation processes.
struct Variant { int tx, ty, zb, tma, cpt, zu, pair, nq; };
static const Variant kVariants[] = {
    {32, 8, 32, 0, 1, 1, 0, 3}, {32, 4, 32, 0, 1, 1, 0, 3}, {64, 4, 32, 0, 1, 1, 0, 3}, {32, 8, 64, 0, 1, 1, 0, 3},
    {32, 16, 16, 0, 1, 1, 0, 3}, {64, 8, 16, 0, 1, 1, 0, 3}, {128, 2, 32, 0, 1, 1, 0, 3}, {32, 8, 0, 0, 1, 1, 0, 3},
    {32, 4, 32, 1, 1, 1, 0, 3}, {32, 8, 32, 1, 2, 1, 0, 3}, {32, 4, 24, 1, 1, 2, 0, 3}, {32, 4, 16, 1, 1, 1, 0, 3},
    {32, 8, 16, 1, 1, 2, 0, 3}, {32, 4, 20, 1, 1, 2, 0, 3}, {32, 4, 32, 1, 1, 2, 0, 3}, {32, 8, 32, 1, 1, 1, 0, 3},
    // zb = -1: z-chunk fitted so the grid fills a whole number of waves
    {32, 8, -1, 1, 1, 2, 0, 3}, {32, 4, -1, 1, 1, 1, 0, 3}, {32, 4, -1, 1, 1, 2, 0, 3},
    // two x cells per thread, two-slot pointwise ring
    {32, 8, -1, 1, 1, 1, 1, 2}, {32, 8, -1, 1, 1, 2, 1, 2}, {64, 8, -1, 1, 1, 1, 1, 2},
    {64, 8, -1, 1, 1, 2, 1, 2}, {32, 16, -1, 1, 1, 1, 1, 2},
};
static const int kNumVariants = sizeof(kVariants) / sizeof(kVariants[0]);

// tuned variant per problem signature (process-wide)
static std::mutex g_tune_mu;
static std::map<std::string, int> g_tuned;

struct WvSession {
    bd_context* ctx = nullptr;
    bd_grid g{};
    bd_westervelt_params p{};
    bd_source s{};
    int prec = BD_F32;
    size_t esz = 4;
    int nx = 0, ny = 0, nz = 0;
    long long plane = 0, ncell = 0;
    int max_relax = 0;
    int n_dft = 0, dz_lo = 0, dz_hi = 0;
    long long dcells = 0;
    int64_t step = 0;           // steps done
    int variant = 0;
    int chunk = 50;
    bool any_mur = false;
    PoolBuf P[5];
    PoolBuf R[BD_MAX_RELAX][2];
    PoolBuf peak, energy, dre, dim;
    PoolBuf cmap, matmap, planemat, wx, wy, wz;
    PoolBuf sA, sVar, sTau, sAf, sPsi, sTauf, sPhi;
    PoolBuf t_src, theta, tb0, tw;
    PoolBuf step_base, flag, kconst, Qd;
    double tau_max = 0.0;
    double last_ms = 0.0;
    cudaGraphExec_t graph[4] = {nullptr, nullptr, nullptr, nullptr};   // chunk graphs per accumulator mode (ACC_*)
    int graph_variant[4] = {-1, -1, -1, -1};
    // tensor maps of the TMA variant in use (built per tile shape)
    int maps_tx = 0, maps_ty = 0;
    bool adj_fused = false;     // adjoint: one fused pass per backward step (FP32, nx % 4 == 0)
    CUtensorMap mP0[5], mQ[5], mR[BD_MAX_RELAX][2], mC, mPeak, mEnergy, mMat, mDre, mDim;
    bool mat_tile = false;      // the material map travels as a TMA tile (nx % 16 == 0)
    // segment view (TMA variants only): the pressure levels of the next step are
    // read from, and p^{n+1} written to, caller-chosen buffers instead of the ring
    bool pdl = true;            // launch TMA step kernels with programmatic dependent launch
    struct SegView {
        bool on = false;
        CUtensorMap p0, q[4];
        void* out = nullptr;
    } segv;
    std::vector<bd_material> mats;
    int n_materials = 0;
    bool has_cmap = false, has_matmap = false, has_planemat = false;
    // z slab of a larger grid (slab sessions only): local plane 0 is global plane
    // zoff, planes [own0, own1) are owned, the 3 planes beyond an internal face
    // are ghost copies of the neighbour's planes (refreshed by the halo exchange)
    bool slab = false;
    int zoff = 0, nz_glob = 0, own0 = 0, own1 = 0;
    int glob_face_zm = BD_FACE_OPEN, glob_face_zp = BD_FACE_OPEN;
    // DFT output layout: this session's planes sit at cell offset dft_glob_off of
    // frequency blocks of dft_glob_cells cells (a whole grid: dcells and 0)
    long long dft_glob_cells = 0, dft_glob_off = 0;

    ~WvSession() {
        for (auto g : graph)
            if (g) cudaGraphExecDestroy(g);
    }
};

static inline int head_of(int64_t s) { return (int)((4 * (s % 5)) % 5); }

// Internal z face of a slab session (never set by callers): the 3 planes beyond
// it are ghost planes, not updated by the step and not damped or Mur-treated.
static const int kFaceHalo = 3;
static const int kHalo = 3;   // ghost planes: the 6th-order stencil reaches iz +- 3 (W:169-174)

template <class real>
static WvArgs<real> make_args(WvSession& S, int64_t s) {
    WvArgs<real> a;
    std::memset(&a, 0, sizeof a);
    a.nx = S.nx; a.ny = S.ny; a.nz = S.nz;
    a.plane = S.plane;
    const int h = head_of(s);
    a.p0 = S.P[(h + 0) % 5].as<real>();
    a.p1 = S.P[(h + 1) % 5].as<real>();
    a.p2 = S.P[(h + 2) % 5].as<real>();
    a.p3 = S.P[(h + 3) % 5].as<real>();
    a.p4 = S.segv.on ? static_cast<real*>(S.segv.out) : S.P[(h + 4) % 5].as<real>();
    const int rh = (int)(s & 1);
    for (int v = 0; v < S.max_relax; ++v) {
        a.rcur[v] = S.R[v][rh].as<real>();
        a.rold[v] = S.R[v][rh ^ 1].as<real>();
    }
    a.max_relax = S.max_relax;
    a.cmap = S.has_cmap ? S.cmap.as<float>() : nullptr;
    a.matmap = S.has_matmap ? S.matmap.as<uint8_t>() : nullptr;
    a.plane_mat = S.has_planemat ? S.planemat.as<int>() : nullptr;
    const bd_grid& g = S.g;
    a.mir_x = g.face[0] == BD_FACE_MIRROR;
    a.mir_y = g.face[2] == BD_FACE_MIRROR;
    a.mur_xp = g.face[1] == BD_FACE_MUR;
    a.mur_yp = g.face[3] == BD_FACE_MUR;
    a.mur_zm = g.face[4] == BD_FACE_MUR;
    a.mur_zp = g.face[5] == BD_FACE_MUR;
    a.L = g.mur_layers;
    a.src_iz = (S.s.kind != BD_SRC_NONE) ? S.s.plane_iz : -1;
    a.Lzm = a.mur_zm ? (a.src_iz >= 0 ? a.src_iz : a.L) : 0;
    a.xhi = a.mur_xp ? S.nx - 1 - a.L : S.nx - 1;
    a.yhi = a.mur_yp ? S.ny - 1 - a.L : S.ny - 1;
    a.zlo = a.Lzm;
    a.zhi = a.mur_zp ? S.nz - 1 - a.L : S.nz - 1;
    if (g.face[4] == kFaceHalo) a.zlo = std::max(a.zlo, kHalo);
    if (g.face[5] == kFaceHalo) a.zhi = std::min(a.zhi, S.nz - 1 - kHalo);
    if (g.sponge_cells > 0) { a.wx = S.wx.as<real>(); a.wy = S.wy.as<real>(); a.wz = S.wz.as<real>(); }
    a.dt = (real)g.dt;
    a.kxy180 = (real)(g.dt * g.dt / (g.dx * g.dx) / 180.0);
    a.kz180 = (real)(g.dt * g.dt / (g.dz * g.dz) / 180.0);
    a.dt2 = (real)(g.dt * g.dt);
    a.dtdx = (real)(g.dt / g.dx);
    a.dtdz = (real)(g.dt / g.dz);
    a.sA = S.sA.as<double>(); a.sVar = S.sVar.as<double>(); a.sTau = S.sTau.as<double>();
    a.sPhi = S.sPhi.as<double>();
    a.sAf = S.sAf.as<float>(); a.sPsi = S.sPsi.as<float>(); a.sTauf = S.sTauf.as<float>();
    a.n_tones = S.s.n_tones;
    a.burst = S.s.burst_cycles > 0.0;
    for (int k = 0; k < BD_MAX_TONES; ++k) {
        a.freq[k] = S.s.freq[k]; a.tamp[k] = S.s.amp[k]; a.tphase[k] = S.s.phase[k];
        a.tampf[k] = (float)S.s.amp[k];
    }
    a.tau_max = S.tau_max;
    a.burst_len = a.burst ? S.s.burst_cycles / S.s.freq[0] : 0.0;
    a.burst_lenf = (float)a.burst_len;
    a.step_base = S.step_base.as<long long>();
    a.t_src = S.t_src.as<double>();
    a.theta = S.theta.as<float>();
    a.tb0 = S.tb0.as<float>();
    a.peak = S.peak.as<real>();
    a.energy = S.energy.as<real>();
    a.dre = S.dre.as<real>();
    a.dim = S.dim.as<real>();
    a.tw = S.tw.as<real>();
    a.peak_start = S.p.peak_start; a.peak_end = S.p.peak_end;
    a.energy_start = S.p.energy_start; a.energy_end = S.p.energy_end;
    a.dft_start = S.p.dft_start; a.dft_len = S.n_dft > 0 ? S.p.dft_len : 0;
    a.energy_mode = S.p.energy_mode;
    a.n_dft = S.n_dft; a.dz_lo = S.dz_lo; a.dz_hi = S.dz_hi;
    a.relax_scheme = S.p.relax_scheme;
    a.mat_tile = S.mat_tile ? 1 : 0;
    return a;
}

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        BD_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
        if (q != cudaDriverEntryPointSuccess || !p) fail(BD_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
        fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

static CUtensorMap make_map(const WvSession& S, const void* base, bool is_float, int bx, int by,
                            bool is_u8 = false, long long depth = 0) {
    CUtensorMap m;
    const size_t esz = is_u8 ? 1 : is_float ? 4 : 8;
    cuuint64_t dims[3] = {(cuuint64_t)S.nx, (cuuint64_t)S.ny, (cuuint64_t)(depth > 0 ? depth : S.nz)};
    cuuint64_t strides[2] = {(cuuint64_t)S.nx * esz, (cuuint64_t)S.nx * S.ny * esz};
    cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    const CUtensorMapDataType ty = is_u8 ? CU_TENSOR_MAP_DATA_TYPE_UINT8
                                   : is_float ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
    CUresult r = encode_fn()(&m, ty, 3,
                             const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) fail(BD_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return m;
}

static bool tma_eligible(const WvSession& S) {
    return (S.nx * S.esz) % 16 == 0 && S.nx >= 8;
}

// The two-cell variants are compiled for FP32 fields with at most two
// relaxation processes; a 16-byte row pitch makes nx even.
static bool variant_ok(const WvSession& S, int v) {
    if (!kVariants[v].pair) return true;
    return S.prec == BD_F32 && S.max_relax <= 2 && tma_eligible(S);
}

static void build_maps(WvSession& S, int tx, int ty) {
    if (S.maps_tx == tx && S.maps_ty == ty) return;
    const bool f = S.prec == BD_F32;
    for (int k = 0; k < 5; ++k) {
        S.mP0[k] = make_map(S, S.P[k].p, f, tx + 8, ty + 6);
        S.mQ[k] = make_map(S, S.P[k].p, f, tx, ty);
    }
    for (int v = 0; v < S.max_relax; ++v)
        for (int k = 0; k < 2; ++k) S.mR[v][k] = make_map(S, S.R[v][k].p, f, tx, ty);
    S.mPeak = make_map(S, S.peak.p, f, tx, ty);
    S.mEnergy = make_map(S, S.energy.p, f, tx, ty);
    if (S.has_cmap) S.mC = make_map(S, S.cmap.p, true, tx, ty);
    if (S.mat_tile) S.mMat = make_map(S, S.matmap.p, false, tx, ty, true);
    if (f && S.n_dft > 0) {   // the DFT planes of every frequency stacked along z (L2 prefetch only)
        const long long depth = (long long)S.n_dft * (S.dz_hi - S.dz_lo);
        S.mDre = make_map(S, S.dre.p, true, tx, ty, false, depth);
        S.mDim = make_map(S, S.dim.p, true, tx, ty, false, depth);
    }
    S.maps_tx = tx;
    S.maps_ty = ty;
}

template <class real, int TX, int TY, int CPT, int NREL, int ZU, int FL = -1>
static void launch_tma_k(WvSession& S, const WvArgs<real>& a0, const TmaMaps& maps, int koff, cudaStream_t st) {
    using L = TmaLayout<real, TX, TY, (NREL >= 0 ? NREL : BD_MAX_RELAX)>;
    static bool attr_done = false;
    static int per_sm = 0;
    if (!attr_done) {
        BD_CUDA(cudaFuncSetAttribute(wv_tma_kernel<real, TX, TY, CPT, NREL, ZU, FL>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        BD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, wv_tma_kernel<real, TX, TY, CPT, NREL, ZU, FL>,
                                                              TX * TY / CPT, L::SMEM));
        attr_done = true;
    }
    WvArgs<real> a = a0;
    const long long tiles = (long long)((S.nx + TX - 1) / TX) * ((S.ny + TY - 1) / TY);
    if (a.zb <= 0) a.zb = wave_fitted_zb(tiles, S.nz, (long long)S.ctx->sm_count * std::max(per_sm, 1));
    dim3 block(TX, TY / CPT, 1);
    dim3 grid((S.nx + TX - 1) / TX, (S.ny + TY - 1) / TY, (S.nz + a.zb - 1) / a.zb);
    const WvConst<real>* K = S.kconst.as<WvConst<real>>();
    unsigned* errp = S.flag.as<unsigned>() + 1;
    if (S.pdl) {
        // programmatic dependent launch: this grid may start while the previous
        // step's grid finishes (the kernel waits for its data)
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = grid;
        cfg.blockDim = block;
        cfg.dynamicSmemBytes = L::SMEM;
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        const cudaError_t e = cudaLaunchKernelEx(&cfg, wv_tma_kernel<real, TX, TY, CPT, NREL, ZU, FL>, a, K, koff, maps,
                                                 errp);
        if (e == cudaSuccess) {
            BD_LAUNCHED(S.ctx);
            return;
        }
        (void)cudaGetLastError();   // not available here: ordinary launches from now on
        S.pdl = false;
    }
    wv_tma_kernel<real, TX, TY, CPT, NREL, ZU, FL><<<grid, block, L::SMEM, st>>>(a, K, koff, maps, errp);
    BD_LAUNCHED(S.ctx);
}

// Tensor maps of step s: p^n with its halo, p^{n-1..n-4}, R, peak, energy, c.
static void step_maps(WvSession& S, int64_t s, int tx, int ty, TmaMaps& maps) {
    build_maps(S, tx, ty);
    std::memset(&maps, 0, sizeof maps);
    const int h = head_of(s);
    maps.p0 = S.mP0[h];
    for (int k = 0; k < 4; ++k) maps.q[k] = S.mQ[(h + 1 + k) % 5];
    if (S.segv.on) {
        maps.p0 = S.segv.p0;
        for (int k = 0; k < 4; ++k) maps.q[k] = S.segv.q[k];
    }
    const int rh = (int)(s & 1);
    for (int v = 0; v < S.max_relax; ++v) { maps.rc[v] = S.mR[v][rh]; maps.ro[v] = S.mR[v][rh ^ 1]; }
    maps.peak = S.mPeak;
    maps.energy = S.mEnergy;
    if (S.has_cmap) maps.cmap = S.mC;
    if (S.mat_tile) maps.mat = S.mMat;
    if (S.prec == BD_F32 && S.n_dft > 0) { maps.dre = S.mDre; maps.dim = S.mDim; }
}

template <class real, int TX, int TY, int CPT, int ZU>
static void launch_tma_t(WvSession& S, const WvArgs<real>& a, int64_t s, int koff, cudaStream_t st) {
    TmaMaps maps;
    step_maps(S, s, TX, TY, maps);
    // FP32 kernels with 0, 1 or 2 relaxation processes are compiled for their count;
    // FP64 and larger counts use the kernel that reads the count at run time
    if (sizeof(real) == 4 && S.max_relax == 0) launch_tma_k<real, TX, TY, CPT, 0, ZU>(S, a, maps, koff, st);
    else if (sizeof(real) == 4 && S.max_relax == 1 && S.has_cmap && !S.has_matmap && !S.has_planemat)
        launch_tma_k<real, TX, TY, CPT, 1, ZU, 3>(S, a, maps, koff, st);   // one material, c map (cfg1)
    else if (sizeof(real) == 4 && S.max_relax == 1) launch_tma_k<real, TX, TY, CPT, 1, ZU>(S, a, maps, koff, st);
    else if (sizeof(real) == 4 && S.max_relax == 2) launch_tma_k<real, TX, TY, CPT, 2, ZU>(S, a, maps, koff, st);
    else launch_tma_k<real, TX, TY, CPT, -1, ZU>(S, a, maps, koff, st);
}

// Accumulators step s adds to (the ACC_* modes of the paired kernel): all when
// its DFT window is open, peak and energy when the energy window is, the peak
// map only when just the peak window is, none outside every window.
static int step_acc_mode(const WvSession& S, int64_t s) {
    if (S.n_dft > 0 && s >= S.p.dft_start && s < S.p.dft_start + S.p.dft_len) return ACC_ALL;
    if (s >= S.p.energy_start && s < S.p.energy_end) return ACC_PE;
    if (s >= S.p.peak_start && s < S.p.peak_end) return ACC_PEAK;
    return ACC_NONE;
}

// The mode that serves every step of [s0, s0 + n): all > peak and energy > peak > none.
static int range_acc_mode(const WvSession& S, int64_t s0, int64_t n) {
    auto rank = [](int m) { return m == ACC_ALL ? 3 : m == ACC_PE ? 2 : m == ACC_PEAK ? 1 : 0; };
    int m = ACC_NONE;
    for (int64_t s = s0; s < s0 + n; ++s) {
        const int k = step_acc_mode(S, s);
        if (rank(k) > rank(m)) m = k;
        if (m == ACC_ALL) break;
    }
    return m;
}

// Two x cells per thread (FP32; variant_ok has been checked).
template <class real>
static void launch_pair(WvSession& S, const WvArgs<real>& a, int64_t s, int koff, cudaStream_t st, const Variant& v,
                        int acc) {
    if constexpr (sizeof(real) != 4) {
        fail(BD_ERR_INVALID_ARG, "two-cell tile variants take FP32 fields");
    } else {
        TmaMaps maps;
        step_maps(S, s, v.tx, v.ty, maps);
        PairCall c;
        c.ctx = S.ctx;
        c.a = &a;
        c.K = S.kconst.as<WvConst<float>>();
        c.koff = koff;
        c.maps = &maps;
        c.err = S.flag.as<unsigned>() + 1;
        c.pdl = &S.pdl;
        c.st = st;
        c.tx = v.tx;
        c.ty = v.ty;
        c.zu = v.zu;
        c.nq = v.nq;
        c.kind = S.max_relax == 0 ? 0
                 : S.max_relax == 1 ? ((S.has_cmap && !S.has_matmap && !S.has_planemat) ? 1 : 2)
                 : S.max_relax == 2 ? 3 : -1;
        c.acc = acc;
        wv_pair_launch(c);
    }
}

template <class real, int TX, int TY>
static void launch_step_t(WvSession& S, const WvArgs<real>& a, int koff, cudaStream_t st) {
    dim3 block(TX, TY, 1);
    dim3 grid((S.nx + TX - 1) / TX, (S.ny + TY - 1) / TY, (S.nz + a.zb - 1) / a.zb);
    wv_step_kernel<real, TX, TY><<<grid, block, 0, st>>>(a, S.kconst.as<WvConst<real>>(), koff);
    BD_LAUNCHED(S.ctx);
}

template <class real>
static void launch_step(WvSession& S, int variant, int64_t s, int koff, cudaStream_t st, int acc) {
    WvArgs<real> a = make_args<real>(S, s);
    const Variant& v = kVariants[variant];
    a.zb = v.zb > 0 ? v.zb : (v.zb < 0 && v.tma ? -1 : S.nz);
    if (v.tma && !tma_eligible(S)) fail(BD_ERR_INVALID_ARG, "tile variant %d needs a 16-byte row pitch", variant);
    if (!variant_ok(S, variant))
        fail(BD_ERR_INVALID_ARG, "tile variant %d takes FP32 fields with at most two relaxation processes", variant);
    if (v.pair) launch_pair<real>(S, a, s, koff, st, v, acc);
    else switch (variant) {
        case 0: case 3: case 7: launch_step_t<real, 32, 8>(S, a, koff, st); break;
        case 1: launch_step_t<real, 32, 4>(S, a, koff, st); break;
        case 2: launch_step_t<real, 64, 4>(S, a, koff, st); break;
        case 4: launch_step_t<real, 32, 16>(S, a, koff, st); break;
        case 5: launch_step_t<real, 64, 8>(S, a, koff, st); break;
        case 6: launch_step_t<real, 128, 2>(S, a, koff, st); break;
        case 8: case 11: launch_tma_t<real, 32, 4, 1, 1>(S, a, s, koff, st); break;
        case 9: launch_tma_t<real, 32, 8, 2, 1>(S, a, s, koff, st); break;
        case 10: case 13: case 14: launch_tma_t<real, 32, 4, 1, 2>(S, a, s, koff, st); break;
        case 12: case 16: launch_tma_t<real, 32, 8, 1, 2>(S, a, s, koff, st); break;
        case 17: launch_tma_t<real, 32, 4, 1, 1>(S, a, s, koff, st); break;
        case 18: launch_tma_t<real, 32, 4, 1, 2>(S, a, s, koff, st); break;
        case 15: launch_tma_t<real, 32, 8, 1, 1>(S, a, s, koff, st); break;
        default: fail(BD_ERR_INVALID_ARG, "bad tile variant %d", variant);
    }
    if (S.any_mur) {
        const WvConst<real>* K = S.kconst.as<WvConst<real>>();
        if (a.mur_zm || a.mur_zp) {
            dim3 b(32, 8), gr((S.nx + 31) / 32, (S.ny + 7) / 8);
            wv_mur_z_kernel<real><<<gr, b, 0, st>>>(a, K, koff);
            BD_LAUNCHED(S.ctx);
        }
        if (a.mur_xp) {
            dim3 b(128), gr((S.ny + 127) / 128, S.nz);
            wv_mur_x_kernel<real><<<gr, b, 0, st>>>(a, K, koff);
            BD_LAUNCHED(S.ctx);
        }
        if (a.mur_yp) {
            dim3 b(128), gr((S.nx + 127) / 128, S.nz);
            wv_mur_y_kernel<real><<<gr, b, 0, st>>>(a, K, koff);
            BD_LAUNCHED(S.ctx);
        }
    }
}

// Issue steps [s, s+n) on the stream (no graph): kernels read *step_base + koff,
// then one advance kernel moves the counter by n.  acc < 0: each step takes the
// paired kernel that touches only the accumulators it needs (step_acc_mode);
// an ACC_* mode forces that one for every step (a captured chunk).
static void issue_steps(WvSession& S, int variant, int64_t s, int n, cudaStream_t st, int acc = -1) {
    for (int k = 0; k < n; ++k) {
        const int m = acc >= 0 ? acc : step_acc_mode(S, s + k);
        if (S.prec == BD_F32) launch_step<float>(S, variant, s + k, k, st, m);
        else launch_step<double>(S, variant, s + k, k, st, m);
    }
    wv_advance_kernel<<<1, 32, 0, st>>>(S.step_base.as<long long>(), n);
    BD_LAUNCHED(S.ctx);
}

static void build_graph(WvSession& S, int acc) {
    cudaGraphExec_t& G = S.graph[acc];
    if (G) { cudaGraphExecDestroy(G); G = nullptr; }
    cudaStream_t cs;
    BD_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t g = nullptr;
    const int64_t launches_before = S.ctx->launches;
    BD_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    try {
        issue_steps(S, S.variant, 0, S.chunk, cs, acc);   // base arrangement: chunk starts at s = 0 mod 10
    } catch (...) {
        cudaStreamEndCapture(cs, &g);
        if (g) cudaGraphDestroy(g);
        cudaStreamDestroy(cs);
        throw;
    }
    BD_CUDA(cudaStreamEndCapture(cs, &g));
    S.ctx->launches = launches_before;   // captured, not yet launched
    const cudaError_t e = cudaGraphInstantiate(&G, g, 0);
    cudaGraphDestroy(g);
    cudaStreamDestroy(cs);
    BD_CUDA(e);
    S.graph_variant[acc] = S.variant;
}

static int64_t launches_per_step(const WvSession& S) {
    int64_t n = 1;
    if (S.any_mur) {
        if (S.g.face[4] == BD_FACE_MUR || S.g.face[5] == BD_FACE_MUR) n++;
        if (S.g.face[1] == BD_FACE_MUR) n++;
        if (S.g.face[3] == BD_FACE_MUR) n++;
    }
    return n;
}

static void probe(WvSession& S) {
    unsigned* f = S.flag.as<unsigned>();
    BD_CUDA(cudaMemsetAsync(f, 0, sizeof(unsigned), S.ctx->stream));
    const int h = head_of(S.step);
    if (S.prec == BD_F32)
        wv_probe_kernel<float><<<S.ctx->sm_count * 4, 256, 0, S.ctx->stream>>>(S.P[h].as<float>(), S.ncell, S.p.blowup_limit, f);
    else
        wv_probe_kernel<double><<<S.ctx->sm_count * 4, 256, 0, S.ctx->stream>>>(S.P[h].as<double>(), S.ncell, S.p.blowup_limit, f);
    BD_LAUNCHED(S.ctx);
    unsigned hf = 0;
    BD_CUDA(cudaMemcpyAsync(&hf, f, sizeof hf, cudaMemcpyDeviceToHost, S.ctx->stream));
    BD_CUDA(cudaStreamSynchronize(S.ctx->stream));
    if (hf & 1u) fail(BD_ERR_UNSTABLE, "non-finite pressure after step %lld", (long long)S.step);
    if (hf & 2u) fail(BD_ERR_UNSTABLE, "|p| above %g after step %lld", S.p.blowup_limit, (long long)S.step);
}

// Advance n steps from the current step, with graph replays for whole chunks.
static void advance(WvSession& S, int64_t n, bool use_graph) {
    cudaStream_t st = S.ctx->stream;
    int64_t end = S.step + n;
    const int64_t fault = S.p.fault_at_step;
    bool faulted = false;
    if (fault >= 0 && fault >= S.step && fault < end) { end = fault; faulted = true; }
    const int64_t per = launches_per_step(S) + 0;
    int64_t next_probe = S.p.check_every > 0 ? ((S.step / S.p.check_every) + 1) * S.p.check_every : INT64_MAX;
    while (S.step < end) {
        int64_t todo = end - S.step;
        const int64_t to_align = (S.chunk - (S.step % S.chunk)) % S.chunk;
        int64_t take;
        if (use_graph && to_align == 0 && todo >= S.chunk) {
            const int m = range_acc_mode(S, S.step, S.chunk);
            if (!S.graph[m] || S.graph_variant[m] != S.variant) build_graph(S, m);
            BD_CUDA(cudaGraphLaunch(S.graph[m], st));
            S.ctx->launches += per * S.chunk + 1;
            take = S.chunk;
        } else {
            take = std::min<int64_t>(todo, to_align > 0 ? to_align : S.chunk);
            issue_steps(S, S.variant, S.step, (int)take, st);
        }
        S.step += take;
        if (S.step >= next_probe) {
            probe(S);
            next_probe = ((S.step / S.p.check_every) + 1) * S.p.check_every;
        }
    }
    if (faulted) {
        BD_CUDA(cudaStreamSynchronize(st));
        fail(BD_ERR_FAULT_INJECTED, "fault injected before step %lld", (long long)fault);
    }
}

static void zero_state(WvSession& S) {
    cudaStream_t st = S.ctx->stream;
    for (auto& b : S.P) BD_CUDA(cudaMemsetAsync(b.p, 0, b.bytes, st));
    for (int v = 0; v < S.max_relax; ++v)
        for (auto& b : S.R[v]) BD_CUDA(cudaMemsetAsync(b.p, 0, b.bytes, st));
    BD_CUDA(cudaMemsetAsync(S.peak.p, 0, S.peak.bytes, st));
    BD_CUDA(cudaMemsetAsync(S.energy.p, 0, S.energy.bytes, st));
    if (S.dre.p) { BD_CUDA(cudaMemsetAsync(S.dre.p, 0, S.dre.bytes, st)); BD_CUDA(cudaMemsetAsync(S.dim.p, 0, S.dim.bytes, st)); }
    BD_CUDA(cudaMemsetAsync(S.step_base.p, 0, sizeof(long long), st));
    BD_CUDA(cudaMemsetAsync(S.flag.p, 0, 64, st));
    S.step = 0;
}

static std::string tune_key(const WvSession& S) {
    char b[256];
    snprintf(b, sizeof b, "%d:%d:%d:%d:%d:%d:%d:%d:%d:%d", S.nx, S.ny, S.nz, S.prec, S.max_relax, S.has_cmap ? 1 : 0,
             S.has_matmap ? 1 : 0, S.has_planemat ? 1 : 0, S.any_mur ? 1 : 0, S.n_dft);
    return b;
}

// Pick the fastest tile variant: a few steps of each on the (zero) initial
// state, timed with events, then the state is cleared again.  Every trial
// restarts at step 0 (host ring index and device step counter), so the trials
// read only the first kTuneSteps entries of the per-step tables, which hold
// n_steps >= kTuneSteps entries whenever tuning runs.
static const int kTuneWarm = 2, kTuneReps = 8, kTuneSteps = kTuneWarm + kTuneReps;
static void autotune(WvSession& S) {
    const std::string key = tune_key(S);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tuned.find(key);
        if (it != g_tuned.end()) { S.variant = it->second; return; }
    }
    cudaStream_t st = S.ctx->stream;
    if (S.p.n_steps < kTuneSteps) fail(BD_ERR_STATE, "tuning needs at least %d steps", kTuneSteps);
    std::vector<float> best_ms(kNumVariants, 1e30f);
    // two rounds over the variants, best time of each: the rounds are seconds
    // apart, so a clock change during one trial does not decide the choice
    for (int round = 0; round < 2; ++round)
        for (int v = 0; v < kNumVariants; ++v) {
            if (kVariants[v].zb == 0 && S.nz > 512) continue;
            if (kVariants[v].tma && !tma_eligible(S)) continue;
            if (!variant_ok(S, v)) continue;
            BD_CUDA(cudaMemsetAsync(S.step_base.p, 0, sizeof(long long), st));
            S.step = 0;
            issue_steps(S, v, S.step, kTuneWarm, st);  // warm-up
            S.step += kTuneWarm;
            BD_CUDA(cudaEventRecord(S.ctx->ev0, st));
            issue_steps(S, v, S.step, kTuneReps, st);
            S.step += kTuneReps;
            BD_CUDA(cudaEventRecord(S.ctx->ev1, st));
            BD_CUDA(cudaEventSynchronize(S.ctx->ev1));
            float ms = 0;
            BD_CUDA(cudaEventElapsedTime(&ms, S.ctx->ev0, S.ctx->ev1));
            best_ms[v] = std::min(best_ms[v], ms);
        }
    int best_v = 0;
    for (int v = 1; v < kNumVariants; ++v)
        if (best_ms[v] < best_ms[best_v]) best_v = v;
    zero_state(S);
    BD_CUDA(cudaStreamSynchronize(st));
    S.variant = best_v;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tuned[key] = best_v;
}

template <class real>
static void upload_consts(WvSession& S, const bd_medium* m) {
    WvConst<real> K;
    std::memset(&K, 0, sizeof K);
    const double dt = S.g.dt;
    for (int k = 0; k < m->n_materials; ++k) {
        const bd_material& mt = m->mat[k];
        MatConst<real>& M = K.mat[k];
        M.c0 = (real)mt.c0;
        M.delta_2dt = (real)(mt.delta / (2.0 * dt));
        M.beta2_rho = (real)(2.0 * mt.beta / mt.rho);
        M.n_relax = mt.n_relax;
        for (int v = 0; v < mt.n_relax; ++v) {
            const double tau = mt.relax_tau[v], cv = mt.relax_c[v];
            M.ra_num[v] = (real)((2.0 * dt * 2.0 * cv * tau) / (2.0 * dt * dt * dt) / (2.0 * dt + 3.0 * tau));
            M.rb[v] = (real)(tau / (2.0 * dt + 3.0 * tau));
        }
    }
    S.kconst.alloc(S.ctx, sizeof K);
    BD_CUDA(cudaMemcpy(S.kconst.p, &K, sizeof K, cudaMemcpyHostToDevice));
}

template <class T>
static void upload(WvSession& S, PoolBuf& b, const std::vector<T>& v) {
    b.alloc(S.ctx, v.size() * sizeof(T));
    if (!v.empty()) BD_CUDA(cudaMemcpy(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
}

static double frac(double x) { return x - std::floor(x); }

static void setup(WvSession& S, bd_context* ctx, const bd_grid* g, const bd_medium* m, const bd_source* src,
                  const bd_westervelt_params* p) {
    if (!ctx || !g || !m || !p) fail(BD_ERR_INVALID_ARG, "null argument");
    S.ctx = ctx;
    S.g = *g;
    S.p = *p;
    if (src) S.s = *src;
    else { std::memset(&S.s, 0, sizeof S.s); S.s.kind = BD_SRC_NONE; }
    S.prec = p->precision;
    if (S.prec != BD_F32 && S.prec != BD_F64) fail(BD_ERR_INVALID_ARG, "precision must be BD_F32 or BD_F64");
    S.esz = S.prec == BD_F32 ? 4 : 8;
    S.nx = g->nx; S.ny = g->ny; S.nz = g->nz;
    if (S.nx < 8 || S.ny < 8 || S.nz < 8) fail(BD_ERR_INVALID_ARG, "grid must be at least 8 cells per axis");
    if ((long long)S.nx * S.ny >= (1LL << 31)) fail(BD_ERR_INVALID_ARG, "an x-y plane must hold fewer than 2^31 cells");
    if (!(g->dt > 0 && g->dx > 0 && g->dz > 0)) fail(BD_ERR_INVALID_ARG, "dt, dx, dz must be positive");
    if (g->face[0] == BD_FACE_MUR || g->face[2] == BD_FACE_MUR)
        fail(BD_ERR_UNSUPPORTED, "Mur on the x-/y- faces is not supported (the reference mirrors them)");
    if (g->face[1] == BD_FACE_MIRROR || g->face[3] == BD_FACE_MIRROR || g->face[4] == BD_FACE_MIRROR ||
        g->face[5] == BD_FACE_MIRROR)
        fail(BD_ERR_INVALID_ARG, "mirror planes exist only at x = 0 and y = 0");
    for (int f = 0; f < 6; ++f) {
        const bool halo_ok = S.slab && f >= 4 && g->face[f] == kFaceHalo;
        if (!halo_ok && (g->face[f] < BD_FACE_OPEN || g->face[f] > BD_FACE_MIRROR))
            fail(BD_ERR_INVALID_ARG, "face %d: unknown boundary kind %d", f, g->face[f]);
    }
    if (!S.slab) { S.zoff = 0; S.nz_glob = g->nz; S.own0 = 0; S.own1 = g->nz; }
    S.any_mur = false;
    for (int f = 0; f < 6; ++f) if (g->face[f] == BD_FACE_MUR) S.any_mur = true;
    if (S.any_mur && (g->mur_layers < 1 || g->mur_layers > 8)) fail(BD_ERR_INVALID_ARG, "mur_layers must be 1..8");
    if (m->n_materials < 1 || m->n_materials > BD_MAX_MATERIALS) fail(BD_ERR_INVALID_ARG, "n_materials out of range");
    S.plane = (long long)S.nx * S.ny;
    S.ncell = S.plane * S.nz;
    S.max_relax = 0;
    for (int k = 0; k < m->n_materials; ++k) {
        if (m->mat[k].n_relax < 0 || m->mat[k].n_relax > BD_MAX_RELAX) fail(BD_ERR_INVALID_ARG, "n_relax out of range");
        if (!(m->mat[k].c0 > 0 || m->c_map)) fail(BD_ERR_INVALID_ARG, "material %d has no sound speed", k);
        if (!(m->mat[k].rho > 0)) fail(BD_ERR_INVALID_ARG, "material %d density must be positive", k);
        S.max_relax = std::max(S.max_relax, m->mat[k].n_relax);
    }
    if (S.s.kind != BD_SRC_NONE) {
        if (S.s.plane_iz < 0 || S.s.plane_iz >= S.nz) fail(BD_ERR_INVALID_ARG, "source plane outside the grid");
        if (S.s.n_tones < 1 || S.s.n_tones > BD_MAX_TONES) fail(BD_ERR_INVALID_ARG, "n_tones out of range");
        if (S.s.focal_length <= 0 || S.s.c_delay <= 0) fail(BD_ERR_INVALID_ARG, "bad source geometry");
        if (S.s.kind == BD_SRC_ARRAY && (!S.s.element_of_cell || S.s.n_elements <= 0))
            fail(BD_ERR_INVALID_ARG, "array source needs element_of_cell and n_elements");
    }
    if (p->n_steps < 0) fail(BD_ERR_INVALID_ARG, "n_steps < 0");
    if (p->relax_scheme != BD_RELAX_REFERENCE && p->relax_scheme != BD_RELAX_SEMI_IMPLICIT)
        fail(BD_ERR_INVALID_ARG, "unknown relax_scheme");
    S.n_dft = p->n_dft;
    if (S.n_dft < 0 || S.n_dft > BD_MAX_DFT) fail(BD_ERR_INVALID_ARG, "n_dft out of range");
    if (S.n_dft > 0) {
        S.dz_lo = std::max(0, p->dft_z_lo);
        S.dz_hi = std::min(S.nz, p->dft_z_hi);
        if (S.dz_hi <= S.dz_lo || p->dft_len <= 0) S.n_dft = 0;
    }
    S.dcells = S.n_dft > 0 ? (long long)(S.dz_hi - S.dz_lo) * S.plane : 0;
    if (!S.slab) { S.dft_glob_cells = S.dcells; S.dft_glob_off = 0; }
    if (S.slab) S.pdl = false;   // the halo copies between steps are not kernels: plain stream order
    S.chunk = p->graph_chunk > 0 ? ((p->graph_chunk + 9) / 10) * 10 : 50;

    BD_CUDA(cudaSetDevice(ctx->device));
    // state
    for (auto& b : S.P) b.alloc(ctx, S.ncell * S.esz);
    for (int v = 0; v < S.max_relax; ++v)
        for (auto& b : S.R[v]) b.alloc(ctx, S.ncell * S.esz);
    S.peak.alloc(ctx, S.ncell * S.esz);
    S.energy.alloc(ctx, S.ncell * S.esz);
    if (S.n_dft > 0) {
        S.dre.alloc(ctx, (size_t)S.n_dft * S.dcells * S.esz);
        S.dim.alloc(ctx, (size_t)S.n_dft * S.dcells * S.esz);
    }
    S.step_base.alloc(ctx, 64);
    S.flag.alloc(ctx, 64);
    // medium
    S.has_cmap = m->c_map != nullptr;
    S.has_matmap = m->material_map != nullptr;
    S.has_planemat = m->plane_material != nullptr;
    // the paired kernel takes the material map as a uint8 TMA tile when its rows
    // (nx bytes) are a multiple of 16 bytes, else per cell through the cache
    S.mat_tile = S.has_matmap && S.nx % 16 == 0;
    if (S.has_cmap) {
        S.cmap.alloc(ctx, S.ncell * 4);
        BD_CUDA(cudaMemcpy(S.cmap.p, m->c_map, S.ncell * 4, cudaMemcpyHostToDevice));
    }
    if (S.has_matmap) {
        for (long long i = 0; i < S.ncell; ++i)
            if (m->material_map[i] >= m->n_materials) fail(BD_ERR_INVALID_ARG, "material_map entry out of range");
        S.matmap.alloc(ctx, S.ncell);
        BD_CUDA(cudaMemcpy(S.matmap.p, m->material_map, S.ncell, cudaMemcpyHostToDevice));
    }
    if (S.has_planemat) {
        for (int iz = 0; iz < S.nz; ++iz)
            if (m->plane_material[iz] < 0 || m->plane_material[iz] >= m->n_materials)
                fail(BD_ERR_INVALID_ARG, "plane_material entry out of range");
        S.planemat.alloc(ctx, S.nz * 4);
        BD_CUDA(cudaMemcpy(S.planemat.p, m->plane_material, S.nz * 4, cudaMemcpyHostToDevice));
    }
    S.n_materials = m->n_materials;
    S.mats.assign(m->mat, m->mat + m->n_materials);
    if (S.prec == BD_F32) upload_consts<float>(S, m);
    else upload_consts<double>(S, m);
    // sponge profiles w(d) = exp(-strength (d/W)^2) on OPEN faces
    {
        auto prof = [&](int n, int lo, int hi) {
            std::vector<double> w(n, 1.0);
            const int W = g->sponge_cells;
            for (int i = 0; i < n && W > 0; ++i) {
                double f = 1.0;
                if (lo == BD_FACE_OPEN && i < W) { double d = (double)(W - i) / W; f *= std::exp(-g->sponge_strength * d * d); }
                if (hi == BD_FACE_OPEN && i >= n - W) { double d = (double)(i - (n - W) + 1) / W; f *= std::exp(-g->sponge_strength * d * d); }
                w[i] = f;
            }
            return w;
        };
        auto up = [&](PoolBuf& b, const std::vector<double>& w) {
            if (S.prec == BD_F64) upload(S, b, w);
            else upload(S, b, std::vector<float>(w.begin(), w.end()));
        };
        if (g->sponge_cells > 0) {
            up(S.wx, prof(S.nx, g->face[0], g->face[1]));
            up(S.wy, prof(S.ny, g->face[2], g->face[3]));
            if (S.slab) {
                // the whole grid's z profile, restricted to this slab's planes
                const std::vector<double> wz = prof(S.nz_glob, S.glob_face_zm, S.glob_face_zp);
                up(S.wz, std::vector<double>(wz.begin() + S.zoff, wz.begin() + S.zoff + S.nz));
            } else {
                up(S.wz, prof(S.nz, g->face[4], g->face[5]));
            }
        }
    }
    // source plane (W:62-85): amplitude, var, delay per plane cell
    const long long np = S.plane;
    std::vector<double> A(np, 0.0), var(np, 1.0), tau(np, 0.0), phi(np, 0.0);
    S.tau_max = 0.0;
    if (S.s.kind != BD_SRC_NONE) {
        const double d = S.s.focal_length;
        for (int iy = 0; iy < S.ny; ++iy)
            for (int ix = 0; ix < S.nx; ++ix) {
                const long long j = (long long)iy * S.nx + ix;
                const double X = g->x0 + ix * g->dx - S.s.cx;
                const double Y = g->y0 + iy * g->dx - S.s.cy;
                const double r = std::sqrt(X * X + Y * Y);
                if (r <= d * std::tan(S.s.alpha) && r >= d * std::tan(S.s.alpha_hole)) {
                    const double vr = std::sqrt(1.0 + std::pow(r / d, 2));
                    double amp = S.s.p0, ph = 0.0;
                    if (S.s.kind == BD_SRC_ARRAY) {
                        const int e = S.s.element_of_cell[j];
                        if (e < 0 || e >= S.s.n_elements) continue;
                        amp *= S.s.element_amp ? S.s.element_amp[e] : 1.0;
                        ph = S.s.element_phase ? S.s.element_phase[e] : 0.0;
                    }
                    A[j] = amp; var[j] = vr; tau[j] = d * (vr - 1.0) / S.s.c_delay; phi[j] = ph;
                    S.tau_max = std::max(S.tau_max, tau[j]);
                }
            }
    }
    const bool burst = S.s.kind != BD_SRC_NONE && S.s.burst_cycles > 0.0;
    if (S.prec == BD_F64) {
        upload(S, S.sA, A); upload(S, S.sVar, var); upload(S, S.sTau, tau); upload(S, S.sPhi, phi);
    } else {
        std::vector<float> Af(np), psi((size_t)BD_MAX_TONES * np, 0.0f), tauf(np);
        for (long long j = 0; j < np; ++j) {
            Af[j] = (float)(A[j] / var[j]);
            tauf[j] = (float)tau[j];
            for (int k = 0; k < S.s.n_tones && k < BD_MAX_TONES; ++k) {
                // 2 pi frac(f tau) + phase_k + element phase, reduced to [0, 2 pi)
                const double ang = 2.0 * BD_PI * frac(S.s.freq[k] * tau[j]) + S.s.phase[k] + phi[j];
                psi[(size_t)k * np + j] = (float)(ang - 2.0 * BD_PI * std::floor(ang / (2.0 * BD_PI)));
            }
        }
        upload(S, S.sAf, Af); upload(S, S.sPsi, psi); upload(S, S.sTauf, tauf);
    }
    // per-step tables
    const int64_t N = std::max<int64_t>(p->n_steps, 1);
    std::vector<double> ts(N);
    for (int64_t s = 0; s < N; ++s) ts[s] = p->t_src ? p->t_src[s] : p->t0 + (double)(s + 1) * g->dt;
    upload(S, S.t_src, ts);
    if (S.prec == BD_F32) {
        std::vector<float> th((size_t)N * BD_MAX_TONES, 0.0f), tb(N, 0.0f);
        for (int64_t s = 0; s < N; ++s) {
            const double tshift = burst ? ts[s] - S.tau_max : ts[s];
            tb[s] = (float)(ts[s] - S.tau_max);
            for (int k = 0; k < S.s.n_tones && k < BD_MAX_TONES; ++k)
                th[(size_t)s * BD_MAX_TONES + k] = (float)(2.0 * BD_PI * frac(S.s.freq[k] * tshift));
        }
        upload(S, S.theta, th); upload(S, S.tb0, tb);
    }
    if (S.n_dft > 0) {
        const int64_t L = p->dft_len;
        std::vector<double> twd((size_t)L * S.n_dft * 2);
        for (int64_t s = 0; s < L; ++s)
            for (int j = 0; j < S.n_dft; ++j) {
                const double th = 2.0 * BD_PI * p->dft_freq[j] * ((double)s * g->dt);
                twd[((size_t)s * S.n_dft + j) * 2] = std::cos(th);
                twd[((size_t)s * S.n_dft + j) * 2 + 1] = std::sin(th);
            }
        if (S.prec == BD_F64) upload(S, S.tw, twd);
        else {
            std::vector<float> twf(twd.begin(), twd.end());
            upload(S, S.tw, twf);
        }
    }
    zero_state(S);
    BD_CUDA(cudaStreamSynchronize(ctx->stream));
    if (p->tile_variant >= 0) {
        if (p->tile_variant >= kNumVariants) fail(BD_ERR_INVALID_ARG, "tile_variant out of range");
        S.variant = p->tile_variant;
    } else if (S.ncell >= (1LL << 21) && p->n_steps >= 200) {
        autotune(S);
    } else {
        // short or small runs are not worth tuning: the wave-fitted TMA variant
        // where the row pitch allows it, else the plain kernel
        S.variant = tma_eligible(S) ? 17 : 0;
    }
}

// ---------------------------------------------------------------- z slabs
// Global planes of the slab that owns [zb, ze) of grid g: the owned planes plus
// kHalo ghost planes beyond each internal face.
static void slab_extent(const bd_grid* g, int zb, int ze, int& lo, int& hi) {
    lo = zb > 0 ? zb - kHalo : 0;
    hi = ze < g->nz ? ze + kHalo : g->nz;
}

// A session for the planes [zb, ze) of the whole problem (g, m, src, p): the
// grid, medium maps, source plane, sponge profile, DFT planes and power split
// are those of the whole problem restricted to the slab, so that with the ghost
// planes refreshed after every step (halo_exchange) the owned planes evolve
// bit for bit as in a single session over the whole grid.
static void setup_slab(WvSession& S, bd_context* ctx, const bd_grid* g, const bd_medium* m, const bd_source* src,
                       const bd_westervelt_params* p, int zb, int ze) {
    if (!ctx || !g || !m || !p) fail(BD_ERR_INVALID_ARG, "null argument");
    if (!(0 <= zb && zb < ze && ze <= g->nz)) fail(BD_ERR_INVALID_ARG, "slab [%d, %d) outside 0..%d", zb, ze, g->nz);
    if (ze - zb < 8) fail(BD_ERR_INVALID_ARG, "a slab must own at least 8 planes (%d)", ze - zb);
    for (int f = 4; f < 6; ++f)
        if (g->face[f] == kFaceHalo) fail(BD_ERR_INVALID_ARG, "face %d: unknown boundary kind", f);
    // Mur layers at the grid's z faces stay inside the end slabs
    const bool src_on = src && src->kind != BD_SRC_NONE;
    const int Lzm = g->face[4] == BD_FACE_MUR ? (src_on ? src->plane_iz : g->mur_layers) : 0;
    const int Lzp = g->face[5] == BD_FACE_MUR ? g->mur_layers : 0;
    if ((zb > 0 && zb - kHalo < Lzm + 1) || (ze < g->nz && ze + kHalo > g->nz - Lzp - 1))
        fail(BD_ERR_INVALID_ARG, "slab [%d, %d) cuts into the Mur layers of the z faces", zb, ze);
    int lo = 0, hi = 0;
    slab_extent(g, zb, ze, lo, hi);
    const long long plane = (long long)g->nx * g->ny;
    bd_grid gl = *g;
    gl.nz = hi - lo;
    gl.z0 = g->z0 + lo * g->dz;
    if (zb > 0) gl.face[4] = kFaceHalo;
    if (ze < g->nz) gl.face[5] = kFaceHalo;
    bd_medium ml = *m;
    if (m->plane_material) ml.plane_material = m->plane_material + lo;
    if (m->material_map) ml.material_map = m->material_map + (size_t)lo * plane;
    if (m->c_map) ml.c_map = m->c_map + (size_t)lo * plane;
    bd_source sl;
    if (src) {
        sl = *src;
        if (src_on) {
            sl.plane_iz = src->plane_iz - lo;
            if (sl.plane_iz < 0 || sl.plane_iz >= gl.nz) sl.kind = BD_SRC_NONE;
        }
    }
    bd_westervelt_params pl = *p;
    if (p->n_dft > 0) {
        pl.dft_z_lo = std::max(p->dft_z_lo, zb) - lo;
        pl.dft_z_hi = std::min(p->dft_z_hi, ze) - lo;
    }
    pl.q_iz_split = p->q_iz_split - lo;
    S.slab = true;
    S.zoff = lo;
    S.nz_glob = g->nz;
    S.own0 = zb - lo;
    S.own1 = ze - lo;
    S.glob_face_zm = g->face[4];
    S.glob_face_zp = g->face[5];
    setup(S, ctx, &gl, &ml, src ? &sl : nullptr, &pl);
    // DFT planes of this slab inside the whole problem's DFT planes
    if (S.n_dft > 0) {
        const int glo = std::max(0, p->dft_z_lo), ghi = std::min(g->nz, p->dft_z_hi);
        S.dft_glob_cells = (long long)(ghi - glo) * plane;
        S.dft_glob_off = (long long)(S.zoff + S.dz_lo - glo) * plane;
    }
}

// Refresh the ghost planes of two neighbouring slabs on the same device: the
// lower slab's top kHalo owned planes of the newest level p^n go to the upper
// slab's low ghost planes and the upper slab's bottom kHalo owned planes to the
// lower slab's high ghost planes (replaces nothing in W, which runs one grid;
// the exchange a multi-GPU run makes over NCCL or peer copies).
static void halo_exchange(WvSession& lo, WvSession& hi, cudaStream_t st) {
    if (!lo.slab || !hi.slab || lo.zoff + lo.own1 != hi.zoff + hi.own0 || lo.nx != hi.nx || lo.ny != hi.ny ||
        lo.prec != hi.prec || lo.step != hi.step || lo.g.face[5] != kFaceHalo || hi.g.face[4] != kFaceHalo)
        fail(BD_ERR_STATE, "halo exchange between sessions that are not neighbouring slabs at the same step");
    const size_t pb = (size_t)lo.plane * lo.esz;
    char* L = static_cast<char*>(lo.P[head_of(lo.step)].p);
    char* H = static_cast<char*>(hi.P[head_of(hi.step)].p);
    BD_CUDA(cudaMemcpyAsync(H, L + (size_t)(lo.own1 - kHalo) * pb, kHalo * pb, cudaMemcpyDeviceToDevice, st));
    BD_CUDA(cudaMemcpyAsync(L + (size_t)lo.own1 * pb, H + (size_t)hi.own0 * pb, kHalo * pb, cudaMemcpyDeviceToDevice, st));
}

// Copy between the newest level's planes at one internal face and a caller's
// device buffer of kHalo planes: to_ghost = 0 reads the owned planes next to
// the face (what the neighbour needs), 1 writes the ghost planes beyond it.
static void halo_copy(WvSession& S, int side, int to_ghost, void* buf, cudaStream_t st) {
    if (!S.slab || (side != 0 && side != 1)) fail(BD_ERR_INVALID_ARG, "halo copy needs a slab session and side 0 or 1");
    if (S.g.face[4 + side] != kFaceHalo) fail(BD_ERR_INVALID_ARG, "side %d of this slab is a face of the grid", side);
    const size_t pb = (size_t)S.plane * S.esz;
    char* P = static_cast<char*>(S.P[head_of(S.step)].p);
    const int first = side == 0 ? (to_ghost ? S.own0 - kHalo : S.own0) : (to_ghost ? S.own1 : S.own1 - kHalo);
    char* planes = P + (size_t)first * pb;
    if (to_ghost) BD_CUDA(cudaMemcpyAsync(planes, buf, kHalo * pb, cudaMemcpyDeviceToDevice, st));
    else BD_CUDA(cudaMemcpyAsync(buf, planes, kHalo * pb, cudaMemcpyDeviceToDevice, st));
}

// Acoustic power of W:242-265 (water planes) and W:324-345 (harmonics), in double.
template <class real>
__global__ void wv_q_kernel(const real* __restrict__ energy, const real* __restrict__ dre, const real* __restrict__ dim,
                            const float* __restrict__ cmap, const uint8_t* __restrict__ matmap,
                            const int* __restrict__ planemat, const bd_material* __restrict__ mats, int nx, int ny,
                            int nz, int split, int n_harm, int n_dft, int dz_lo, int dz_hi, double f, double dft_len,
                            double* __restrict__ Q) {
    const long long plane = (long long)nx * ny;
    const long long n = plane * nz;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(i / plane);
        const int m = matmap ? matmap[i] : (planemat ? planemat[iz] : 0);
        const bd_material& mt = mats[m];
        const double c = cmap ? (double)cmap[i] : mt.c0;
        double q = 0.0;
        if (iz >= split) {
            if (iz >= dz_lo && iz < dz_hi) {
                const long long pl = (long long)(iz - dz_lo) * plane + (i % plane);
                const long long stride = (long long)(dz_hi - dz_lo) * plane;
                for (int h = 1; h <= n_harm && h <= n_dft; ++h) {
                    const double re = (double)dre[(h - 1) * stride + pl], im = (double)dim[(h - 1) * stride + pl];
                    const double a = sqrt(re * re + im * im) / dft_len;               // W:299
                    const double In = 2.0 * a * a / (mt.rho * c);                     // W:341
                    q = q + (2.0 * (mt.harm_absorption * h * f / 1e6) * In);          // W:342
                }
            }
        } else {
            q = 2.0 * mt.absorption * f * (double)energy[i] / ((2.0 * BD_PI * f) * (2.0 * BD_PI * f) * mt.rho * c);  // W:261
        }
        Q[i] = q;
    }
}

static void finish(WvSession& S, bd_westervelt_outputs* o) {
    cudaStream_t st = S.ctx->stream;
    BD_CUDA(cudaStreamSynchronize(st));
    // owned planes only (a whole grid owns every plane)
    const size_t off = (size_t)S.own0 * S.plane * S.esz;
    const size_t bytes = (size_t)(S.own1 - S.own0) * S.plane * S.esz;
    const int h = head_of(S.step);
    auto at = [&](const PoolBuf& b) { return static_cast<const char*>(b.p) + off; };
    if (o->p_final) BD_CUDA(cudaMemcpy(o->p_final, at(S.P[h]), bytes, cudaMemcpyDeviceToHost));
    if (o->peak) BD_CUDA(cudaMemcpy(o->peak, at(S.peak), bytes, cudaMemcpyDeviceToHost));
    if (o->energy) BD_CUDA(cudaMemcpy(o->energy, at(S.energy), bytes, cudaMemcpyDeviceToHost));
    for (int j = 0; j < S.n_dft; ++j) {
        const size_t src = (size_t)j * S.dcells * S.esz, dst = ((size_t)j * S.dft_glob_cells + S.dft_glob_off) * S.esz;
        const size_t nb = (size_t)S.dcells * S.esz;
        if (o->dft_re) BD_CUDA(cudaMemcpy(static_cast<char*>(o->dft_re) + dst, static_cast<const char*>(S.dre.p) + src, nb,
                                          cudaMemcpyDeviceToHost));
        if (o->dft_im) BD_CUDA(cudaMemcpy(static_cast<char*>(o->dft_im) + dst, static_cast<const char*>(S.dim.p) + src, nb,
                                          cudaMemcpyDeviceToHost));
    }
    if (o->Q && S.p.q_mode == BD_Q_REFERENCE) {
        S.Qd.alloc(S.ctx, S.ncell * 8);
        PoolBuf mats;
        upload(S, mats, S.mats);
        const int blocks = S.ctx->sm_count * 8;
        if (S.prec == BD_F32)
            wv_q_kernel<float><<<blocks, 256, 0, st>>>(S.energy.as<float>(), S.dre.as<float>(), S.dim.as<float>(),
                                                       S.has_cmap ? S.cmap.as<float>() : nullptr,
                                                       S.has_matmap ? S.matmap.as<uint8_t>() : nullptr,
                                                       S.has_planemat ? S.planemat.as<int>() : nullptr,
                                                       mats.as<bd_material>(), S.nx, S.ny, S.nz, S.p.q_iz_split,
                                                       S.p.q_n_harm, S.n_dft, S.dz_lo, S.dz_hi, S.p.q_freq,
                                                       (double)S.p.dft_len, S.Qd.as<double>());
        else
            wv_q_kernel<double><<<blocks, 256, 0, st>>>(S.energy.as<double>(), S.dre.as<double>(), S.dim.as<double>(),
                                                        S.has_cmap ? S.cmap.as<float>() : nullptr,
                                                        S.has_matmap ? S.matmap.as<uint8_t>() : nullptr,
                                                        S.has_planemat ? S.planemat.as<int>() : nullptr,
                                                        mats.as<bd_material>(), S.nx, S.ny, S.nz, S.p.q_iz_split,
                                                        S.p.q_n_harm, S.n_dft, S.dz_lo, S.dz_hi, S.p.q_freq,
                                                        (double)S.p.dft_len, S.Qd.as<double>());
        BD_LAUNCHED(S.ctx);
        BD_CUDA(cudaMemcpyAsync(o->Q, S.Qd.as<double>() + (size_t)S.own0 * S.plane,
                                (size_t)(S.own1 - S.own0) * S.plane * 8, cudaMemcpyDeviceToHost, st));
        BD_CUDA(cudaStreamSynchronize(st));
    }
    o->steps_done = S.step;
    o->tile_variant = S.variant;
}

// ---------------------------------------------------------------- checkpoint
struct CkHeader {
    char magic[8];
    int32_t version, precision, nx, ny, nz, max_relax, n_dft, pad;
    int64_t step, dcells;
};

static size_t ck_size(const WvSession& S) {
    const size_t f = S.ncell * S.esz;
    return sizeof(CkHeader) + f * (5 + 2 * (size_t)S.max_relax + 2) + 2 * (size_t)S.n_dft * S.dcells * S.esz;
}

static void ck_save(WvSession& S, void* blob, size_t bytes) {
    if (bytes < ck_size(S)) fail(BD_ERR_INVALID_ARG, "checkpoint buffer too small (%zu < %zu)", bytes, ck_size(S));
    BD_CUDA(cudaStreamSynchronize(S.ctx->stream));
    CkHeader h;
    std::memset(&h, 0, sizeof h);
    std::memcpy(h.magic, "BDCKPT01", 8);
    h.version = 1; h.precision = S.prec; h.nx = S.nx; h.ny = S.ny; h.nz = S.nz;
    h.max_relax = S.max_relax; h.n_dft = S.n_dft; h.step = S.step; h.dcells = S.dcells;
    char* o = static_cast<char*>(blob);
    std::memcpy(o, &h, sizeof h);
    o += sizeof h;
    const size_t f = S.ncell * S.esz;
    const int hd = head_of(S.step);
    for (int k = 0; k < 5; ++k) { BD_CUDA(cudaMemcpy(o, S.P[(hd + k) % 5].p, f, cudaMemcpyDeviceToHost)); o += f; }
    const int rh = (int)(S.step & 1);
    for (int v = 0; v < S.max_relax; ++v)
        for (int k = 0; k < 2; ++k) { BD_CUDA(cudaMemcpy(o, S.R[v][rh ^ k].p, f, cudaMemcpyDeviceToHost)); o += f; }
    BD_CUDA(cudaMemcpy(o, S.peak.p, f, cudaMemcpyDeviceToHost)); o += f;
    BD_CUDA(cudaMemcpy(o, S.energy.p, f, cudaMemcpyDeviceToHost)); o += f;
    if (S.n_dft > 0) {
        BD_CUDA(cudaMemcpy(o, S.dre.p, S.dre.bytes, cudaMemcpyDeviceToHost)); o += S.dre.bytes;
        BD_CUDA(cudaMemcpy(o, S.dim.p, S.dim.bytes, cudaMemcpyDeviceToHost)); o += S.dim.bytes;
    }
}

static void ck_load(WvSession& S, const void* blob, size_t bytes) {
    if (bytes < sizeof(CkHeader)) fail(BD_ERR_INVALID_ARG, "checkpoint too small");
    CkHeader h;
    std::memcpy(&h, blob, sizeof h);
    if (std::memcmp(h.magic, "BDCKPT01", 8) != 0) fail(BD_ERR_INVALID_ARG, "not a checkpoint blob");
    if (h.precision != S.prec || h.nx != S.nx || h.ny != S.ny || h.nz != S.nz || h.max_relax != S.max_relax ||
        h.n_dft != S.n_dft || h.dcells != S.dcells)
        fail(BD_ERR_STATE, "checkpoint geometry does not match this solve");
    if (bytes < ck_size(S)) fail(BD_ERR_INVALID_ARG, "checkpoint truncated");
    const char* in = static_cast<const char*>(blob) + sizeof h;
    const size_t f = S.ncell * S.esz;
    BD_CUDA(cudaStreamSynchronize(S.ctx->stream));
    const int hd = head_of(h.step);
    for (int k = 0; k < 5; ++k) { BD_CUDA(cudaMemcpy(S.P[(hd + k) % 5].p, in, f, cudaMemcpyHostToDevice)); in += f; }
    const int rh = (int)(h.step & 1);
    for (int v = 0; v < S.max_relax; ++v)
        for (int k = 0; k < 2; ++k) { BD_CUDA(cudaMemcpy(S.R[v][rh ^ k].p, in, f, cudaMemcpyHostToDevice)); in += f; }
    BD_CUDA(cudaMemcpy(S.peak.p, in, f, cudaMemcpyHostToDevice)); in += f;
    BD_CUDA(cudaMemcpy(S.energy.p, in, f, cudaMemcpyHostToDevice)); in += f;
    if (S.n_dft > 0) {
        BD_CUDA(cudaMemcpy(S.dre.p, in, S.dre.bytes, cudaMemcpyHostToDevice)); in += S.dre.bytes;
        BD_CUDA(cudaMemcpy(S.dim.p, in, S.dim.bytes, cudaMemcpyHostToDevice)); in += S.dim.bytes;
    }
    long long st = h.step;
    BD_CUDA(cudaMemcpy(S.step_base.p, &st, sizeof st, cudaMemcpyHostToDevice));
    S.step = h.step;
}


// ---------------------------------------------------------------- adjoint
template <class real, int NR>
static void adj_launch_n(WvSession& S, const AdjArgs<real>& a, cudaStream_t st, int part) {
    const WvConst<real>* K = S.kconst.as<WvConst<real>>();
    constexpr int VEC = 16 / sizeof(real);
    if constexpr (sizeof(real) == 4) {
        if (S.adj_fused) {
            const long long nv = (long long)S.ncell / 4;
            adj_point_kernel<real, NR, 4, true><<<(unsigned)((nv + 255) / 256), 256, 0, st>>>(a, K);
            BD_LAUNCHED(S.ctx);
            return;
        }
    }
    if (part == 2) {                          // the stencil pass alone
        dim3 b(32, 8), g((S.nx + 31) / 32, (S.ny + 7) / 8, (S.nz + a.zb - 1) / a.zb);
        adj_stencil_kernel<real><<<g, b, 0, st>>>(a);
        BD_LAUNCHED(S.ctx);
        return;
    }
    if (S.nx % VEC == 0) {
        const long long nv = (long long)S.ncell / VEC;
        adj_point_kernel<real, NR, VEC><<<(unsigned)((nv + 255) / 256), 256, 0, st>>>(a, K);
    } else {
        adj_point_kernel<real, NR, 1><<<(unsigned)((S.ncell + 255) / 256), 256, 0, st>>>(a, K);
    }
    BD_LAUNCHED(S.ctx);
    if (part == 1) return;                    // the pointwise pass alone
    dim3 b(32, 8), g((S.nx + 31) / 32, (S.ny + 7) / 8, (S.nz + a.zb - 1) / a.zb);
    adj_stencil_kernel<real><<<g, b, 0, st>>>(a);
    BD_LAUNCHED(S.ctx);
}

// One backward step: part 0 = every pass, 1 = the pointwise pass, 2 = the
// stencil pass (the two-pass path; the fused path is one kernel whatever part)
template <class real>
static void adj_launch(WvSession& S, const AdjArgs<real>& a, cudaStream_t st, int part = 0) {
    switch (S.max_relax) {
        case 0: adj_launch_n<real, 0>(S, a, st, part); break;
        case 1: adj_launch_n<real, 1>(S, a, st, part); break;
        case 2: adj_launch_n<real, 2>(S, a, st, part); break;
        default: adj_launch_n<real, BD_MAX_RELAX>(S, a, st, part); break;
    }
}

// loss = sum_x w_L(x) E(x) over the whole grid's energy map, in z-y-x order
template <class real>
static double focal_loss_sum(const std::vector<real>& E, int nx, int ny, int nz, const bd_focal_loss* loss) {
    const int fr2 = loss->focal_radius * loss->focal_radius, sr2 = loss->side_radius * loss->side_radius;
    double L = 0.0;
    for (int iz = 0; iz < nz; ++iz)
        for (int iy = 0; iy < ny; ++iy)
            for (int ix = 0; ix < nx; ++ix) {
                const int dx = ix - loss->focus_ix, dy = iy - loss->focus_iy, dz = iz - loss->focus_iz;
                const int r2 = dx * dx + dy * dy + dz * dz;
                double wl = 0.0;
                if (r2 <= fr2) wl = -1.0;
                else if (iz == loss->focus_iz && r2 >= sr2) wl = loss->side_weight;
                if (wl != 0.0) L += wl * (double)E[((size_t)iz * ny + iy) * nx + ix];
            }
    return L;
}

// Arguments of the backward kernels that come from the session and the loss
// (grid, materials, sponge, source tables, loss region); the buffers of the
// adjoint rings, H and the gradients are the caller's.
template <class real>
static void fill_adj_args(const WvSession& S, const bd_focal_loss* loss, AdjArgs<real>& a) {
    std::memset(&a, 0, sizeof a);
    a.nx = S.nx; a.ny = S.ny; a.nz = S.nz; a.plane = S.plane;
    a.max_relax = S.max_relax;
    a.cmap = S.has_cmap ? S.cmap.as<float>() : nullptr;
    a.matmap = S.has_matmap ? S.matmap.as<uint8_t>() : nullptr;
    a.plane_mat = S.has_planemat ? S.planemat.as<int>() : nullptr;
    if (S.g.sponge_cells > 0) { a.wx = S.wx.as<real>(); a.wy = S.wy.as<real>(); a.wz = S.wz.as<real>(); }
    a.kxy180 = (real)(S.g.dt * S.g.dt / (S.g.dx * S.g.dx) / 180.0);
    a.kz180 = (real)(S.g.dt * S.g.dt / (S.g.dz * S.g.dz) / 180.0);
    a.dt2 = (real)(S.g.dt * S.g.dt);
    a.dt = (real)S.g.dt;
    a.relax_scheme = S.p.relax_scheme;
    a.src_iz = (S.s.kind != BD_SRC_NONE) ? S.s.plane_iz : -1;
    {
        // stencil pass: about four waves of 8 CTAs per SM
        const long long tiles = (long long)((S.nx + 31) / 32) * ((S.ny + 7) / 8);
        const long long target = 32LL * S.ctx->sm_count;
        a.zb = (int)std::min<long long>(64, std::max<long long>(4, (tiles * S.nz + target - 1) / target));
    }
    a.sAf = S.sAf.as<float>(); a.sPsi = S.sPsi.as<float>(); a.sTauf = S.sTauf.as<float>();
    a.theta = S.theta.as<float>(); a.tb0 = S.tb0.as<float>();
    a.sA = S.sA.as<double>(); a.sVar = S.sVar.as<double>(); a.sTau = S.sTau.as<double>(); a.sPhi = S.sPhi.as<double>();
    a.t_src = S.t_src.as<double>();
    a.n_tones = S.s.n_tones;
    a.burst = S.s.burst_cycles > 0.0;
    for (int k = 0; k < BD_MAX_TONES; ++k) {
        a.freq[k] = S.s.freq[k]; a.tamp[k] = S.s.amp[k]; a.tphase[k] = S.s.phase[k]; a.tampf[k] = (float)S.s.amp[k];
    }
    a.tau_max = S.tau_max;
    a.burst_len = a.burst ? S.s.burst_cycles / S.s.freq[0] : 0.0;
    a.burst_lenf = (float)a.burst_len;
    a.fx = loss->focus_ix; a.fy = loss->focus_iy; a.fz = loss->focus_iz - S.zoff;
    a.frad2 = loss->focal_radius * loss->focal_radius;
    a.srad2 = loss->side_radius * loss->side_radius;
    a.side_w = loss->side_weight;
    a.win0 = loss->window_start;
    a.win1 = loss->window_end;
}

template <class real>
static void adjoint_solve(WvSession& S, const bd_focal_loss* loss, double* loss_out, double* grad_phase,
                          double* grad_amp, double* timings) {
    cudaStream_t st = S.ctx->stream;
    const int64_t N = S.p.n_steps;
    const size_t f = S.ncell * S.esz;
    const int64_t sqrtN = std::max<int64_t>(1, (int64_t)std::ceil(std::sqrt((double)N)));
    int64_t Kc = loss->checkpoint_every > 0 ? std::min<int64_t>(loss->checkpoint_every, N) : sqrtN;
    if (loss->checkpoint_every < 0) {
        // the whole history when it fits in half of the free device memory; blocks
        // the context's pool holds from earlier solves count as free (they are reused)
        size_t fr = 0, tot = 0;
        BD_CUDA(cudaMemGetInfo(&fr, &tot));
        if ((double)(N + 5) * (double)f <= 0.5 * ((double)fr + (double)S.ctx->pool_bytes)) Kc = N;
    }
    const int64_t nck = (N + Kc - 1) / Kc;
    const int nlev = 5 + 2 * S.max_relax;
    // checkpoints at steps 0, Kc, ..., (nck - 2) Kc; the last segment is stored level by level
    // during the forward itself and never recomputed
    std::vector<PoolBuf> ck((nck - 1) * nlev);
    for (auto& b : ck) b.alloc(S.ctx, f);
    std::vector<PoolBuf> seg(Kc + 5);   // seg[j] = p^{s0 - 4 + j} of the current segment
    for (auto& b : seg) b.alloc(S.ctx, f);
    // TMA variants step straight through the segment store (each step reads its
    // levels from seg and writes p^{s+1} there: no copy per step); the plain
    // kernel updates p^{n-4} in place, so it steps the ring and copies
    const Variant& var = kVariants[S.variant];
    const bool seg_direct = var.tma != 0;
    std::vector<CUtensorMap> segP0, segQ;
    if (seg_direct) {
        segP0.resize(seg.size());
        segQ.resize(seg.size());
        const bool fl = S.prec == BD_F32;
        for (size_t j = 0; j < seg.size(); ++j) {
            segP0[j] = make_map(S, seg[j].p, fl, var.tx + 8, var.ty + 6);
            segQ[j] = make_map(S, seg[j].p, fl, var.tx, var.ty);
        }
    }
    // Whole segments of Kc steps (the recompute and the backward sweep) replay
    // captured CUDA graphs: a step's buffers depend only on its place in the
    // segment, the parity of its index (relaxation ring) and the number of
    // backward steps done modulo 6 (adjoint rings), and its index comes from a
    // device counter, so one graph per key serves every full segment.
    // (only when several segments share a graph: a graph used once costs its capture)
    const bool use_graphs = S.p.graph_chunk >= 0 && N / Kc >= 3;
    struct GraphCache {
        std::map<int, cudaGraphExec_t> g;
        ~GraphCache() { for (auto& kv : g) cudaGraphExecDestroy(kv.second); }
    } rec_graphs, bwd_graphs;
    auto captured = [&](GraphCache& cache, int key, int64_t launches, auto&& body) {
        auto it = cache.g.find(key);
        if (it == cache.g.end()) {
            cudaStream_t cs;
            BD_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
            cudaGraph_t gr = nullptr;
            const int64_t before = S.ctx->launches;
            BD_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
            try {
                body(cs);
            } catch (...) {
                cudaStreamEndCapture(cs, &gr);
                if (gr) cudaGraphDestroy(gr);
                cudaStreamDestroy(cs);
                throw;
            }
            BD_CUDA(cudaStreamEndCapture(cs, &gr));
            S.ctx->launches = before;      // captured, not launched
            cudaGraphExec_t ex = nullptr;
            const cudaError_t e = cudaGraphInstantiate(&ex, gr, 0);
            cudaGraphDestroy(gr);
            cudaStreamDestroy(cs);
            BD_CUDA(e);
            it = cache.g.emplace(key, ex).first;
        }
        BD_CUDA(cudaGraphLaunch(it->second, st));
        S.ctx->launches += launches;
    };
    auto segment_steps = [&](cudaStream_t cs, int64_t s0, int64_t s1) {
        for (int64_t s = s0; s < s1; ++s) {
            const int64_t j = s - s0;            // seg[j .. j+4] = p^{s-4} .. p^s
            if (seg_direct) {
                S.segv.on = true;
                S.segv.p0 = segP0[j + 4];
                for (int k = 0; k < 4; ++k) S.segv.q[k] = segQ[j + 3 - k];
                S.segv.out = seg[j + 5].p;
                try {
                    issue_steps(S, S.variant, s, 1, cs);
                } catch (...) {
                    S.segv.on = false;
                    throw;
                }
                S.segv.on = false;
            } else {
                issue_steps(S, S.variant, s, 1, cs);
                BD_CUDA(cudaMemcpyAsync(seg[j + 5].p, S.P[head_of(s + 1)].p, f, cudaMemcpyDeviceToDevice, cs));
            }
        }
    };
    auto store_segment = [&](int64_t s0, int64_t s1) {
        for (int k = 0; k < 5; ++k)
            BD_CUDA(cudaMemcpyAsync(seg[4 - k].p, S.P[(head_of(s0) + k) % 5].p, f, cudaMemcpyDeviceToDevice, st));
        if (use_graphs && seg_direct && s1 - s0 == Kc)
            captured(rec_graphs, (int)(s0 & 1), Kc * (launches_per_step(S) + 1),
                     [&](cudaStream_t cs) { segment_steps(cs, s0, s1); });
        else
            segment_steps(st, s0, s1);
        S.step = s1;
    };
    auto level_buf = [&](int64_t s, int k) -> PoolBuf& {   // k < 5: p^{s-k}; 5 + 2v + j: R^{s-1-j} of process v
        if (k < 5) return S.P[(head_of(s) + k) % 5];
        const int v = (k - 5) / 2, j = (k - 5) % 2;
        return S.R[v][(int)(s & 1) ^ j];
    };
    BD_CUDA(cudaEventRecord(S.ctx->ev0, st));
    for (int64_t c = 0; c < nck; ++c) {
        const int64_t s0 = c * Kc, s1 = std::min<int64_t>(N, s0 + Kc);
        if (c + 1 < nck) {
            for (int k = 0; k < nlev; ++k)
                BD_CUDA(cudaMemcpyAsync(ck[c * nlev + k].p, level_buf(s0, k).p, f, cudaMemcpyDeviceToDevice, st));
            advance(S, s1 - s0, S.p.graph_chunk >= 0);
        } else {
            store_segment(s0, s1);
        }
    }
    BD_CUDA(cudaEventRecord(S.ctx->ev1, st));
    BD_CUDA(cudaEventSynchronize(S.ctx->ev1));
    float ms_fwd = 0;
    BD_CUDA(cudaEventElapsedTime(&ms_fwd, S.ctx->ev0, S.ctx->ev1));
    std::vector<real> E(S.ncell);
    BD_CUDA(cudaMemcpy(E.data(), S.energy.p, f, cudaMemcpyDeviceToHost));
    const double L = focal_loss_sum(E, S.nx, S.ny, S.nz, loss);
    if (loss_out) *loss_out = L;
    // backward buffers
    PoolBuf mu[6], muR[BD_MAX_RELAX][3], gphi, gamp, eamp, Hb[2];
    // FP32 grids with nx % 4 == 0 fold the stencil pass into the next step's
    // pointwise pass (H alternates between two buffers by the parity of s);
    // the others run the pointwise and stencil passes
    S.adj_fused = S.prec == BD_F32 && S.nx % 4 == 0;
    for (auto& b : Hb) { b.alloc(S.ctx, f); BD_CUDA(cudaMemsetAsync(b.p, 0, f, st)); }
    struct AdjFusedOff {
        WvSession& s;
        ~AdjFusedOff() { s.adj_fused = false; }
    } adj_fused_off{S};
    const int per_step = S.adj_fused ? 1 : 2;     // kernels per backward step
    for (auto& b : mu) { b.alloc(S.ctx, f); BD_CUDA(cudaMemsetAsync(b.p, 0, f, st)); }
    for (int v = 0; v < S.max_relax; ++v)
        for (auto& b : muR[v]) { b.alloc(S.ctx, f); BD_CUDA(cudaMemsetAsync(b.p, 0, f, st)); }
    gphi.alloc(S.ctx, S.plane * 8); gamp.alloc(S.ctx, S.plane * 8);
    BD_CUDA(cudaMemsetAsync(gphi.p, 0, S.plane * 8, st));
    BD_CUDA(cudaMemsetAsync(gamp.p, 0, S.plane * 8, st));
    std::vector<double> ea(S.plane, 0.0);
    std::vector<int> elem(S.plane, -1);
    for (long long j = 0; j < S.plane; ++j) {
        if (S.s.kind == BD_SRC_ARRAY) {
            const int e = S.s.element_of_cell[j];
            if (e >= 0 && e < S.s.n_elements) { elem[j] = e; ea[j] = S.s.element_amp ? S.s.element_amp[e] : 1.0; }
        } else {
            ea[j] = 1.0;
        }
    }
    upload(S, eamp, ea);
    // recompute without accumulators
    const bd_westervelt_params saved = S.p;
    S.p.peak_end = S.p.peak_start;
    S.p.energy_end = S.p.energy_start;
    S.p.dft_len = 0;
    const int n_dft_saved = S.n_dft;
    S.n_dft = 0;
    AdjArgs<real> a;
    fill_adj_args(S, loss, a);
    a.H = Hb[0].as<real>();
    a.Hin = Hb[1].as<real>();
    a.gphi = gphi.as<double>(); a.gamp = gamp.as<double>(); a.e_amp = eamp.as<double>();
    // backward step counter on the device: forward index of the next backward step
    PoolBuf bstep;
    bstep.alloc(S.ctx, 64);
    {
        const long long last = N - 1;
        BD_CUDA(cudaMemcpyAsync(bstep.p, &last, sizeof last, cudaMemcpyHostToDevice, st));
        BD_CUDA(cudaStreamSynchronize(st));
    }
    a.bstep = bstep.as<long long>();
    // backward steps s1-1 .. s0 of a segment after nb earlier backward steps
    auto backward_steps = [&](cudaStream_t cs, int64_t s0, int64_t s1, int64_t nb) {
        int rot = (int)(nb % 6), rrot = (int)(nb % 3);    // rotation of the adjoint rings
        int koff = 0;
        for (int64_t s = s1 - 1; s >= s0; --s, ++koff) {
            for (int k = 0; k < 5; ++k) a.mu[k] = mu[(rot + k) % 6].as<real>();
            a.mu5 = mu[(rot + 5) % 6].as<real>();
            for (int v = 0; v < S.max_relax; ++v) {
                a.muR1[v] = muR[v][rrot].as<real>();
                a.muR2[v] = muR[v][(rrot + 1) % 3].as<real>();
                a.muR3[v] = muR[v][(rrot + 2) % 3].as<real>();
            }
            for (int k = 0; k < 5; ++k) a.fp[k] = seg[s - s0 + 5 - k].as<real>();
            if (S.adj_fused) {
                a.H = Hb[s & 1].as<real>();            // written by this step
                a.Hin = Hb[(s + 1) & 1].as<real>();    // written by step s + 1 (zero before the first)
            }
            a.koff = koff;
            adj_launch<real>(S, a, cs);
            rot = (rot + 1) % 6;      // lambda_k now sits in the buffer of mu_{k+1}, lambda_4 in the spare
            rrot = (rrot + 1) % 3;
        }
        adj_advance_kernel<<<1, 32, 0, cs>>>(bstep.as<long long>(), (int)(s1 - s0));
        BD_LAUNCHED(S.ctx);
    };
    int64_t nb_done = 0;
    float ms_rec = 0, ms_bwd = 0;
    for (int64_t c = nck - 1; c >= 0; --c) {
        const int64_t s0 = c * Kc, s1 = std::min<int64_t>(N, s0 + Kc);
        BD_CUDA(cudaEventRecord(S.ctx->ev0, st));
        if (c + 1 < nck) {
            for (int k = 0; k < nlev; ++k)
                BD_CUDA(cudaMemcpyAsync(level_buf(s0, k).p, ck[c * nlev + k].p, f, cudaMemcpyDeviceToDevice, st));
            long long sb = s0;
            BD_CUDA(cudaMemcpyAsync(S.step_base.p, &sb, sizeof sb, cudaMemcpyHostToDevice, st));
            BD_CUDA(cudaStreamSynchronize(st));
            S.step = s0;
            store_segment(s0, s1);
        }
        BD_CUDA(cudaEventRecord(S.ctx->ev1, st));
        if (use_graphs && s1 - s0 == Kc) {
            const int64_t nb = nb_done;
            captured(bwd_graphs, (int)(nb % 6), per_step * Kc + 1,
                     [&](cudaStream_t cs) { backward_steps(cs, s0, s1, nb); });
        } else {
            backward_steps(st, s0, s1, nb_done);
        }
        nb_done += s1 - s0;
        cudaEvent_t e2;
        BD_CUDA(cudaEventCreate(&e2));
        BD_CUDA(cudaEventRecord(e2, st));
        BD_CUDA(cudaEventSynchronize(e2));
        float m1 = 0, m2 = 0;
        BD_CUDA(cudaEventElapsedTime(&m1, S.ctx->ev0, S.ctx->ev1));
        BD_CUDA(cudaEventElapsedTime(&m2, S.ctx->ev1, e2));
        cudaEventDestroy(e2);
        ms_rec += m1;
        ms_bwd += m2;
    }
    S.p = saved;
    S.n_dft = n_dft_saved;
    {
        unsigned fl = 0;   // bounded pipeline waits of the forward and stencil kernels
        BD_CUDA(cudaMemcpy(&fl, S.flag.as<unsigned>() + 1, sizeof fl, cudaMemcpyDeviceToHost));
        if (fl & 4u) fail(BD_ERR_TIMEOUT, "a pipeline wait of the adjoint solve timed out");
    }
    // per-element sums of the per-cell gradients
    std::vector<double> gp(S.plane), ga(S.plane);
    BD_CUDA(cudaMemcpy(gp.data(), gphi.p, S.plane * 8, cudaMemcpyDeviceToHost));
    BD_CUDA(cudaMemcpy(ga.data(), gamp.p, S.plane * 8, cudaMemcpyDeviceToHost));
    const int ne = S.s.kind == BD_SRC_ARRAY ? S.s.n_elements : 0;
    if (grad_phase) for (int e = 0; e < ne; ++e) grad_phase[e] = 0.0;
    if (grad_amp) for (int e = 0; e < ne; ++e) grad_amp[e] = 0.0;
    for (long long j = 0; j < S.plane; ++j) {
        const int e = elem[j];
        if (e < 0) continue;
        if (grad_phase) grad_phase[e] += gp[j];
        if (grad_amp) grad_amp[e] += ga[j];
    }
    if (timings) { timings[0] = ms_fwd; timings[1] = ms_rec; timings[2] = ms_bwd; }
}


// Levels of a session at step s: k < 5: p^{s-k}; 5 + 2v + j: R^{s-1-j} of process v.
static PoolBuf& adj_level(WvSession& S, int64_t s, int k) {
    if (k < 5) return S.P[(head_of(s) + k) % 5];
    const int v = (k - 5) / 2, j = (k - 5) % 2;
    return S.R[v][(int)(s & 1) ^ j];
}

// kHalo planes of two buffers of neighbouring slabs: the lower slab's top owned
// planes to the upper slab's low ghost planes, the upper slab's bottom owned
// planes to the lower slab's high ghost planes.
static void exchange_planes(const WvSession& lo, const WvSession& hi, void* lb, void* hb, cudaStream_t st) {
    const size_t pb = (size_t)lo.plane * lo.esz;
    char* L = static_cast<char*>(lb);
    char* H = static_cast<char*>(hb);
    BD_CUDA(cudaMemcpyAsync(H + (size_t)(hi.own0 - kHalo) * pb, L + (size_t)(lo.own1 - kHalo) * pb, kHalo * pb,
                            cudaMemcpyDeviceToDevice, st));
    BD_CUDA(cudaMemcpyAsync(L + (size_t)lo.own1 * pb, H + (size_t)hi.own0 * pb, kHalo * pb, cudaMemcpyDeviceToDevice,
                            st));
}

// The adjoint solve over K z slabs of one device: the z-slab split of a
// multi-GPU gradient (each slab its own fields, checkpoints, adjoint rings and
// H), checked against the one-domain solve.  Forward and recompute steps
// exchange the 3 ghost planes of p^n after every step like the slab forward
// solve; a backward step couples planes only through the transposed stencil of
// H, so after every step the ghost planes of that step's H take the
// neighbours' owned planes (between the pointwise and stencil passes on the
// two-pass path).  Every other backward quantity is pointwise: ghost planes
// compute values nobody reads.  Only the slab that owns the source plane adds
// to the source gradient, and the loss is summed over the whole grid in the
// one-domain order, so loss and gradients are the one-domain bits.  Steps go
// out as plain launches, slab after slab.
template <class real>
static void adjoint_solve_slabs(std::vector<WvSession*>& sl, const bd_focal_loss* loss, double* loss_out,
                                double* grad_phase, double* grad_amp, double* timings) {
    const int K = (int)sl.size();
    WvSession& S0 = *sl[0];
    bd_context* ctx = S0.ctx;
    cudaStream_t st = ctx->stream;
    const int64_t N = S0.p.n_steps;
    const int64_t sqrtN = std::max<int64_t>(1, (int64_t)std::ceil(std::sqrt((double)N)));
    int64_t Kc = loss->checkpoint_every > 0 ? std::min<int64_t>(loss->checkpoint_every, N) : sqrtN;
    if (loss->checkpoint_every < 0) {
        size_t fr = 0, tot = 0, fsum = 0;
        BD_CUDA(cudaMemGetInfo(&fr, &tot));
        for (auto* S : sl) fsum += S->ncell * S->esz;
        if ((double)(N + 5) * (double)fsum <= 0.5 * ((double)fr + (double)ctx->pool_bytes)) Kc = N;
    }
    const int64_t nck = (N + Kc - 1) / Kc;
    const int nlev = 5 + 2 * S0.max_relax;
    // the slab that owns the source plane
    int ko = -1;
    for (int k = 0; k < K; ++k)
        if (sl[k]->s.kind != BD_SRC_NONE && sl[k]->s.plane_iz >= sl[k]->own0 && sl[k]->s.plane_iz < sl[k]->own1) ko = k;
    if (ko < 0) fail(BD_ERR_INVALID_ARG, "no slab owns the source plane");
    struct Per {
        std::vector<PoolBuf> ck, seg;
        PoolBuf mu[6], muR[BD_MAX_RELAX][3], gphi, gamp, eamp, Hb[2];
        AdjArgs<real> a;
        size_t f = 0;
    };
    std::vector<Per> per(K);
    for (int k = 0; k < K; ++k) {
        Per& P = per[k];
        P.f = sl[k]->ncell * sl[k]->esz;
        P.ck.resize((nck - 1) * nlev);
        for (auto& b : P.ck) b.alloc(ctx, P.f);
        P.seg.resize(Kc + 5);
        for (auto& b : P.seg) b.alloc(ctx, P.f);
    }
    auto forward_step = [&]() {
        for (auto* S : sl) {
            issue_steps(*S, S->variant, S->step, 1, st);
            S->step += 1;
        }
        for (int k = 0; k + 1 < K; ++k) halo_exchange(*sl[k], *sl[k + 1], st);
    };
    // levels p^{s0-4} .. p^{s1} of every slab into its segment store
    auto store_segment = [&](int64_t s0, int64_t s1) {
        for (int k = 0; k < K; ++k)
            for (int j = 0; j < 5; ++j)
                BD_CUDA(cudaMemcpyAsync(per[k].seg[4 - j].p, adj_level(*sl[k], s0, j).p, per[k].f,
                                        cudaMemcpyDeviceToDevice, st));
        for (int64_t s = s0; s < s1; ++s) {
            forward_step();
            for (int k = 0; k < K; ++k)
                BD_CUDA(cudaMemcpyAsync(per[k].seg[s - s0 + 5].p, sl[k]->P[head_of(s + 1)].p, per[k].f,
                                        cudaMemcpyDeviceToDevice, st));
        }
    };
    BD_CUDA(cudaEventRecord(ctx->ev0, st));
    for (int64_t c = 0; c < nck; ++c) {
        const int64_t s0 = c * Kc, s1 = std::min<int64_t>(N, s0 + Kc);
        if (c + 1 < nck) {
            for (int k = 0; k < K; ++k)
                for (int j = 0; j < nlev; ++j)
                    BD_CUDA(cudaMemcpyAsync(per[k].ck[c * nlev + j].p, adj_level(*sl[k], s0, j).p, per[k].f,
                                            cudaMemcpyDeviceToDevice, st));
            for (int64_t s = s0; s < s1; ++s) forward_step();
        } else {
            store_segment(s0, s1);
        }
    }
    BD_CUDA(cudaEventRecord(ctx->ev1, st));
    BD_CUDA(cudaEventSynchronize(ctx->ev1));
    float ms_fwd = 0;
    BD_CUDA(cudaEventElapsedTime(&ms_fwd, ctx->ev0, ctx->ev1));
    // the whole grid's energy map from the owned planes, summed in the one-domain order
    const int nz = S0.nz_glob;
    std::vector<real> E((size_t)S0.plane * nz);
    for (auto* S : sl)
        BD_CUDA(cudaMemcpy(E.data() + (size_t)(S->zoff + S->own0) * S->plane,
                           static_cast<const real*>(S->energy.p) + (size_t)S->own0 * S->plane,
                           (size_t)(S->own1 - S->own0) * S->plane * sizeof(real), cudaMemcpyDeviceToHost));
    const double L = focal_loss_sum(E, S0.nx, S0.ny, nz, loss);
    if (loss_out) *loss_out = L;
    // per-element amplitude of every source-plane cell (the owning slab's source)
    const WvSession& So = *sl[ko];
    std::vector<double> ea(So.plane, 0.0);
    std::vector<int> elem(So.plane, -1);
    for (long long j = 0; j < So.plane; ++j) {
        if (So.s.kind == BD_SRC_ARRAY) {
            const int e = So.s.element_of_cell[j];
            if (e >= 0 && e < So.s.n_elements) { elem[j] = e; ea[j] = So.s.element_amp ? So.s.element_amp[e] : 1.0; }
        } else {
            ea[j] = 1.0;
        }
    }
    const bool fused = S0.prec == BD_F32 && S0.nx % 4 == 0;
    PoolBuf bstep;
    bstep.alloc(ctx, 64);
    {
        const long long last = N - 1;
        BD_CUDA(cudaMemcpyAsync(bstep.p, &last, sizeof last, cudaMemcpyHostToDevice, st));
        BD_CUDA(cudaStreamSynchronize(st));
    }
    std::vector<bd_westervelt_params> saved(K);
    std::vector<int> n_dft_saved(K);
    for (int k = 0; k < K; ++k) {
        WvSession& S = *sl[k];
        Per& P = per[k];
        S.adj_fused = fused;
        for (auto& b : P.Hb) { b.alloc(ctx, P.f); BD_CUDA(cudaMemsetAsync(b.p, 0, P.f, st)); }
        for (auto& b : P.mu) { b.alloc(ctx, P.f); BD_CUDA(cudaMemsetAsync(b.p, 0, P.f, st)); }
        for (int v = 0; v < S.max_relax; ++v)
            for (auto& b : P.muR[v]) { b.alloc(ctx, P.f); BD_CUDA(cudaMemsetAsync(b.p, 0, P.f, st)); }
        P.gphi.alloc(ctx, S.plane * 8); P.gamp.alloc(ctx, S.plane * 8);
        BD_CUDA(cudaMemsetAsync(P.gphi.p, 0, S.plane * 8, st));
        BD_CUDA(cudaMemsetAsync(P.gamp.p, 0, S.plane * 8, st));
        upload(S, P.eamp, ea);
        // the recompute runs without accumulators
        saved[k] = S.p;
        n_dft_saved[k] = S.n_dft;
        S.p.peak_end = S.p.peak_start;
        S.p.energy_end = S.p.energy_start;
        S.p.dft_len = 0;
        S.n_dft = 0;
        fill_adj_args(S, loss, P.a);
        if (k != ko) P.a.src_iz = -1;           // a ghost copy of the source plane adds no gradient
        P.a.H = P.Hb[0].as<real>();
        P.a.Hin = P.Hb[1].as<real>();
        P.a.gphi = P.gphi.as<double>(); P.a.gamp = P.gamp.as<double>(); P.a.e_amp = P.eamp.as<double>();
        P.a.bstep = bstep.as<long long>();
    }
    struct Restore {
        std::vector<WvSession*>& sl;
        std::vector<bd_westervelt_params>& p;
        std::vector<int>& nd;
        ~Restore() {
            for (size_t k = 0; k < sl.size(); ++k) { sl[k]->p = p[k]; sl[k]->n_dft = nd[k]; sl[k]->adj_fused = false; }
        }
    } restore{sl, saved, n_dft_saved};
    int64_t nb_done = 0;
    float ms_rec = 0, ms_bwd = 0;
    for (int64_t c = nck - 1; c >= 0; --c) {
        const int64_t s0 = c * Kc, s1 = std::min<int64_t>(N, s0 + Kc);
        BD_CUDA(cudaEventRecord(ctx->ev0, st));
        if (c + 1 < nck) {
            for (int k = 0; k < K; ++k) {
                WvSession& S = *sl[k];
                for (int j = 0; j < nlev; ++j)
                    BD_CUDA(cudaMemcpyAsync(adj_level(S, s0, j).p, per[k].ck[c * nlev + j].p, per[k].f,
                                            cudaMemcpyDeviceToDevice, st));
                long long sb = s0;
                BD_CUDA(cudaMemcpyAsync(S.step_base.p, &sb, sizeof sb, cudaMemcpyHostToDevice, st));
                BD_CUDA(cudaStreamSynchronize(st));
                S.step = s0;
            }
            store_segment(s0, s1);
        }
        BD_CUDA(cudaEventRecord(ctx->ev1, st));
        int rot = (int)(nb_done % 6), rrot = (int)(nb_done % 3);
        int koff = 0;
        for (int64_t s = s1 - 1; s >= s0; --s, ++koff) {
            for (int part = fused ? 0 : 1; part <= (fused ? 0 : 2); ++part) {
                for (int k = 0; k < K; ++k) {
                    WvSession& S = *sl[k];
                    Per& P = per[k];
                    AdjArgs<real> a = P.a;
                    for (int j = 0; j < 5; ++j) a.mu[j] = P.mu[(rot + j) % 6].as<real>();
                    a.mu5 = P.mu[(rot + 5) % 6].as<real>();
                    for (int v = 0; v < S.max_relax; ++v) {
                        a.muR1[v] = P.muR[v][rrot].as<real>();
                        a.muR2[v] = P.muR[v][(rrot + 1) % 3].as<real>();
                        a.muR3[v] = P.muR[v][(rrot + 2) % 3].as<real>();
                    }
                    for (int j = 0; j < 5; ++j) a.fp[j] = P.seg[s - s0 + 5 - j].as<real>();
                    if (fused) {
                        a.H = P.Hb[s & 1].as<real>();            // written by this step
                        a.Hin = P.Hb[(s + 1) & 1].as<real>();    // written by step s + 1
                    }
                    a.koff = koff;
                    adj_launch<real>(S, a, st, part);
                }
                if (part != 2)                  // H of this step: ghost planes from the neighbours
                    for (int k = 0; k + 1 < K; ++k) {
                        const int hb = fused ? (int)(s & 1) : 0;
                        exchange_planes(*sl[k], *sl[k + 1], per[k].Hb[hb].p, per[k + 1].Hb[hb].p, st);
                    }
            }
            rot = (rot + 1) % 6;
            rrot = (rrot + 1) % 3;
        }
        adj_advance_kernel<<<1, 32, 0, st>>>(bstep.as<long long>(), (int)(s1 - s0));
        BD_LAUNCHED(ctx);
        nb_done += s1 - s0;
        cudaEvent_t e2;
        BD_CUDA(cudaEventCreate(&e2));
        BD_CUDA(cudaEventRecord(e2, st));
        BD_CUDA(cudaEventSynchronize(e2));
        float m1 = 0, m2 = 0;
        BD_CUDA(cudaEventElapsedTime(&m1, ctx->ev0, ctx->ev1));
        BD_CUDA(cudaEventElapsedTime(&m2, ctx->ev1, e2));
        cudaEventDestroy(e2);
        ms_rec += m1;
        ms_bwd += m2;
    }
    for (auto* S : sl) {
        unsigned fl = 0;
        BD_CUDA(cudaMemcpy(&fl, S->flag.as<unsigned>() + 1, sizeof fl, cudaMemcpyDeviceToHost));
        if (fl & 4u) fail(BD_ERR_TIMEOUT, "a pipeline wait of the adjoint solve timed out");
    }
    std::vector<double> gp(So.plane), ga(So.plane);
    BD_CUDA(cudaMemcpy(gp.data(), per[ko].gphi.p, So.plane * 8, cudaMemcpyDeviceToHost));
    BD_CUDA(cudaMemcpy(ga.data(), per[ko].gamp.p, So.plane * 8, cudaMemcpyDeviceToHost));
    const int ne = So.s.kind == BD_SRC_ARRAY ? So.s.n_elements : 0;
    if (grad_phase) for (int e = 0; e < ne; ++e) grad_phase[e] = 0.0;
    if (grad_amp) for (int e = 0; e < ne; ++e) grad_amp[e] = 0.0;
    for (long long j = 0; j < So.plane; ++j) {
        const int e = elem[j];
        if (e < 0) continue;
        if (grad_phase) grad_phase[e] += gp[j];
        if (grad_amp) grad_amp[e] += ga[j];
    }
    if (timings) { timings[0] = ms_fwd; timings[1] = ms_rec; timings[2] = ms_bwd; }
}

}  // namespace bd

namespace bd {

// Self-test of the bounded pipeline wait: one warp waits on an mbarrier that
// nothing arrives on; the wait gives up after limit_ns, sets bit 4 of *err
// (as a stalled TMA pipeline would) and the kernel returns.
__global__ void wait_selftest_kernel(unsigned* err, unsigned long long limit_ns) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_fence_init();
    }
    __syncthreads();
    mbar_wait_for(&bar, 0u, err, limit_ns);
}

}  // namespace bd

struct bd_westervelt {
    bd::WvSession S;
};

using namespace bd;

static double timed_advance(WvSession& S, int64_t n) {
    BD_CUDA(cudaEventRecord(S.ctx->ev0, S.ctx->stream));
    bool graph = S.p.graph_chunk >= 0;
    advance(S, n, graph);
    BD_CUDA(cudaEventRecord(S.ctx->ev1, S.ctx->stream));
    BD_CUDA(cudaEventSynchronize(S.ctx->ev1));
    float ms = 0;
    BD_CUDA(cudaEventElapsedTime(&ms, S.ctx->ev0, S.ctx->ev1));
    S.last_ms = ms;
    unsigned f = 0;
    BD_CUDA(cudaMemcpy(&f, S.flag.as<unsigned>() + 1, sizeof f, cudaMemcpyDeviceToHost));
    if (f & 4u) fail(BD_ERR_TIMEOUT, "a pipeline wait in the stencil kernel timed out");
    return ms;
}

extern "C" {

bd_status bd_selftest_bounded_wait(bd_context* ctx, int32_t limit_ms, int32_t* timed_out, double* elapsed_ms) {
    return guard([&] {
        ctx_check(ctx);
        if (limit_ms < 1 || limit_ms > 2000 || !timed_out) fail(BD_ERR_INVALID_ARG, "limit_ms must be 1..2000");
        PoolBuf f;
        f.alloc(ctx, 64);
        cudaStream_t st = ctx->stream;
        BD_CUDA(cudaMemsetAsync(f.p, 0, 64, st));
        BD_CUDA(cudaEventRecord(ctx->ev0, st));
        wait_selftest_kernel<<<1, 32, 0, st>>>(f.as<unsigned>(), (unsigned long long)limit_ms * 1000000ull);
        BD_LAUNCHED(ctx);
        BD_CUDA(cudaEventRecord(ctx->ev1, st));
        unsigned flag = 0;
        BD_CUDA(cudaMemcpyAsync(&flag, f.p, sizeof flag, cudaMemcpyDeviceToHost, st));
        BD_CUDA(cudaStreamSynchronize(st));
        float ms = 0;
        BD_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
        *timed_out = (flag & 4u) ? 1 : 0;
        if (elapsed_ms) *elapsed_ms = ms;
    });
}

bd_status bd_westervelt_begin(bd_context* ctx, const bd_grid* grid, const bd_medium* medium, const bd_source* source,
                              const bd_westervelt_params* params, bd_westervelt** out) {
    return guard([&] {
        if (!out) fail(BD_ERR_INVALID_ARG, "null output");
        *out = nullptr;
        ctx_check(ctx);
        auto* w = new bd_westervelt();
        try {
            setup(w->S, ctx, grid, medium, source, params);
        } catch (...) {
            delete w;
            throw;
        }
        *out = w;
    });
}

bd_status bd_westervelt_advance(bd_westervelt* w, int64_t n_steps) {
    return guard([&] {
        if (!w) fail(BD_ERR_INVALID_ARG, "null session");
        ctx_check(w->S.ctx);
        if (n_steps < 0) fail(BD_ERR_INVALID_ARG, "negative step count");
        if (w->S.step + n_steps > w->S.p.n_steps)
            fail(BD_ERR_INVALID_ARG, "advance past n_steps (%lld + %lld > %lld)", (long long)w->S.step,
                 (long long)n_steps, (long long)w->S.p.n_steps);
        timed_advance(w->S, n_steps);
    });
}

bd_status bd_westervelt_step_index(bd_westervelt* w, int64_t* step) {
    return guard([&] {
        if (!w || !step) fail(BD_ERR_INVALID_ARG, "null argument");
        *step = w->S.step;
    });
}

bd_status bd_westervelt_last_ms(bd_westervelt* w, double* ms) {
    return guard([&] {
        if (!w || !ms) fail(BD_ERR_INVALID_ARG, "null argument");
        *ms = w->S.last_ms;
    });
}

bd_status bd_westervelt_finish(bd_westervelt* w, bd_westervelt_outputs* out) {
    return guard([&] {
        if (!w || !out) fail(BD_ERR_INVALID_ARG, "null argument");
        ctx_check(w->S.ctx);
        finish(w->S, out);
        out->elapsed_ms = w->S.last_ms;
    });
}

bd_status bd_westervelt_end(bd_westervelt* w) {
    return guard([&] {
        if (!w) return;
        cudaSetDevice(w->S.ctx->device);
        cudaStreamSynchronize(w->S.ctx->stream);
        delete w;
    });
}

bd_status bd_checkpoint_size(bd_westervelt* w, size_t* bytes) {
    return guard([&] {
        if (!w || !bytes) fail(BD_ERR_INVALID_ARG, "null argument");
        *bytes = ck_size(w->S);
    });
}

bd_status bd_checkpoint_save(bd_westervelt* w, void* blob, size_t bytes) {
    return guard([&] {
        if (!w || !blob) fail(BD_ERR_INVALID_ARG, "null argument");
        ctx_check(w->S.ctx);
        ck_save(w->S, blob, bytes);
    });
}

bd_status bd_checkpoint_load(bd_westervelt* w, const void* blob, size_t bytes) {
    return guard([&] {
        if (!w || !blob) fail(BD_ERR_INVALID_ARG, "null argument");
        ctx_check(w->S.ctx);
        ck_load(w->S, blob, bytes);
    });
}

// Checks of the adjoint's arguments and the forward parameters it runs with.
static bd_westervelt_params adjoint_params(const bd_grid* grid, const bd_source* source,
                                           const bd_westervelt_params* params, const bd_focal_loss* loss) {
    if (!grid || !loss || !params) fail(BD_ERR_INVALID_ARG, "null argument");
    for (int f = 0; f < 6; ++f)
        if (grid->face[f] != BD_FACE_OPEN) fail(BD_ERR_UNSUPPORTED, "the adjoint supports OPEN faces only");
    if (!source || source->kind == BD_SRC_NONE) fail(BD_ERR_INVALID_ARG, "the adjoint needs a source");
    if (loss->window_start < 0 || loss->window_end > params->n_steps || loss->window_start >= loss->window_end)
        fail(BD_ERR_INVALID_ARG, "bad loss window");
    bd_westervelt_params p = *params;
    p.energy_mode = BD_ENERGY_P2;
    p.energy_start = loss->window_start;
    p.energy_end = loss->window_end;
    p.peak_start = p.peak_end = 0;
    p.n_dft = 0;
    p.q_mode = BD_Q_NONE;
    p.fault_at_step = -1;
    return p;
}

bd_status bd_westervelt_adjoint(bd_context* ctx, const bd_grid* grid, const bd_medium* medium, const bd_source* source,
                                const bd_westervelt_params* params, const bd_focal_loss* loss, double* loss_out,
                                double* grad_phase, double* grad_amp, double* timings_ms) {
    return guard([&] {
        ctx_check(ctx);
        const bd_westervelt_params p = adjoint_params(grid, source, params, loss);
        bd_westervelt w;
        setup(w.S, ctx, grid, medium, source, &p);
        if (w.S.prec == BD_F32) adjoint_solve<float>(w.S, loss, loss_out, grad_phase, grad_amp, timings_ms);
        else adjoint_solve<double>(w.S, loss, loss_out, grad_phase, grad_amp, timings_ms);
    });
}

bd_status bd_westervelt_adjoint_slabs(bd_context* ctx, const bd_grid* grid, const bd_medium* medium,
                                      const bd_source* source, const bd_westervelt_params* params,
                                      const bd_focal_loss* loss, int32_t n_slabs, double* loss_out,
                                      double* grad_phase, double* grad_amp, double* timings_ms) {
    return guard([&] {
        ctx_check(ctx);
        const bd_westervelt_params p = adjoint_params(grid, source, params, loss);
        if (n_slabs < 1 || n_slabs > grid->nz / 8) fail(BD_ERR_INVALID_ARG, "n_slabs must be 1..nz/8");
        if (n_slabs == 1) {
            bd_westervelt w;
            setup(w.S, ctx, grid, medium, source, &p);
            if (w.S.prec == BD_F32) adjoint_solve<float>(w.S, loss, loss_out, grad_phase, grad_amp, timings_ms);
            else adjoint_solve<double>(w.S, loss, loss_out, grad_phase, grad_amp, timings_ms);
            return;
        }
        std::vector<std::unique_ptr<WvSession>> own;
        std::vector<WvSession*> sl;
        for (int k = 0; k < n_slabs; ++k) {
            own.emplace_back(new WvSession());
            setup_slab(*own[k], ctx, grid, medium, source, &p, (int)((long long)grid->nz * k / n_slabs),
                       (int)((long long)grid->nz * (k + 1) / n_slabs));
            sl.push_back(own[k].get());
        }
        if (sl[0]->prec == BD_F32) adjoint_solve_slabs<float>(sl, loss, loss_out, grad_phase, grad_amp, timings_ms);
        else adjoint_solve_slabs<double>(sl, loss, loss_out, grad_phase, grad_amp, timings_ms);
    });
}

bd_status bd_westervelt_slab_begin(bd_context* ctx, const bd_grid* grid, const bd_medium* medium,
                                   const bd_source* source, const bd_westervelt_params* params, int32_t z_begin,
                                   int32_t z_end, bd_westervelt** out) {
    return guard([&] {
        if (!out) fail(BD_ERR_INVALID_ARG, "null output");
        *out = nullptr;
        ctx_check(ctx);
        auto* w = new bd_westervelt();
        try {
            setup_slab(w->S, ctx, grid, medium, source, params, z_begin, z_end);
        } catch (...) {
            delete w;
            throw;
        }
        *out = w;
    });
}

bd_status bd_westervelt_halo_bytes(bd_westervelt* w, size_t* bytes) {
    return guard([&] {
        if (!w || !bytes) fail(BD_ERR_INVALID_ARG, "null argument");
        if (!w->S.slab) fail(BD_ERR_INVALID_ARG, "not a slab session");
        *bytes = (size_t)kHalo * w->S.plane * w->S.esz;
    });
}

bd_status bd_westervelt_halo_copy(bd_westervelt* w, int32_t side, int32_t to_ghost, void* d_buf, void* stream) {
    return guard([&] {
        if (!w || !d_buf) fail(BD_ERR_INVALID_ARG, "null argument");
        ctx_check(w->S.ctx);
        halo_copy(w->S, side, to_ghost ? 1 : 0, d_buf, stream ? static_cast<cudaStream_t>(stream) : w->S.ctx->stream);
    });
}

bd_status bd_halo_exchange(bd_westervelt* lower, bd_westervelt* upper) {
    return guard([&] {
        if (!lower || !upper) fail(BD_ERR_INVALID_ARG, "null session");
        if (lower->S.ctx != upper->S.ctx) fail(BD_ERR_INVALID_ARG, "same-device exchange needs one context");
        ctx_check(lower->S.ctx);
        halo_exchange(lower->S, upper->S, lower->S.ctx->stream);
    });
}

bd_status bd_westervelt_run_slabs(bd_context* ctx, const bd_grid* grid, const bd_medium* medium,
                                  const bd_source* source, const bd_westervelt_params* params, int32_t n_slabs,
                                  bd_westervelt_outputs* out) {
    return guard([&] {
        if (!out || !grid || !params) fail(BD_ERR_INVALID_ARG, "null argument");
        ctx_check(ctx);
        if (n_slabs < 1 || n_slabs > grid->nz / 8) fail(BD_ERR_INVALID_ARG, "n_slabs must be 1..nz/8");
        const long long plane = (long long)grid->nx * grid->ny;
        std::vector<int> zb(n_slabs + 1);
        for (int k = 0; k <= n_slabs; ++k) zb[k] = (int)((long long)grid->nz * k / n_slabs);
        std::vector<std::unique_ptr<WvSession>> sl;
        for (int k = 0; k < n_slabs; ++k) {
            sl.emplace_back(new WvSession());
            if (n_slabs == 1) setup(*sl[k], ctx, grid, medium, source, params);
            else setup_slab(*sl[k], ctx, grid, medium, source, params, zb[k], zb[k + 1]);
        }
        cudaStream_t st = ctx->stream;
        BD_CUDA(cudaEventRecord(ctx->ev0, st));
        for (int64_t s = 0; s < params->n_steps; ++s) {
            for (auto& S : sl) {
                issue_steps(*S, S->variant, S->step, 1, st);
                S->step += 1;
            }
            for (int k = 0; k + 1 < n_slabs; ++k) halo_exchange(*sl[k], *sl[k + 1], st);
        }
        BD_CUDA(cudaEventRecord(ctx->ev1, st));
        BD_CUDA(cudaEventSynchronize(ctx->ev1));
        float ms = 0;
        BD_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
        for (auto& S : sl) {
            unsigned f = 0;
            BD_CUDA(cudaMemcpy(&f, S->flag.as<unsigned>() + 1, sizeof f, cudaMemcpyDeviceToHost));
            if (f & 4u) fail(BD_ERR_TIMEOUT, "a pipeline wait in the stencil kernel timed out");
        }
        // each slab writes its owned planes into the whole grid's outputs
        for (int k = 0; k < n_slabs; ++k) {
            WvSession& S = *sl[k];
            bd_westervelt_outputs o = *out;
            const size_t off = (size_t)zb[k] * plane;
            if (out->p_final) o.p_final = static_cast<char*>(out->p_final) + off * S.esz;
            if (out->peak) o.peak = static_cast<char*>(out->peak) + off * S.esz;
            if (out->energy) o.energy = static_cast<char*>(out->energy) + off * S.esz;
            if (out->Q) o.Q = out->Q + off;
            finish(S, &o);
        }
        out->steps_done = params->n_steps;
        out->tile_variant = sl[0]->variant;
        out->elapsed_ms = ms;
    });
}

bd_status bd_westervelt_run(bd_context* ctx, const bd_grid* grid, const bd_medium* medium, const bd_source* source,
                            const bd_westervelt_params* params, bd_westervelt_outputs* out) {
    return guard([&] {
        if (!out) fail(BD_ERR_INVALID_ARG, "null outputs");
        ctx_check(ctx);
        bd_westervelt w;
        setup(w.S, ctx, grid, medium, source, params);
        timed_advance(w.S, params->n_steps);
        finish(w.S, out);
        out->elapsed_ms = w.S.last_ms;
    });
}

}  // extern "C"
