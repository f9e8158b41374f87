/*
 * bubbledyn.h — C ABI of the GB300 focused-ultrasound engine.
 *
 * The reference (FilkinaGramota/BubbleDynamics) has no library interface: it is
 * three stand-alone programs whose contract is their hard-coded parameter blocks
 * and their output files.  Each entry point below replaces one of those programs
 * (or one stage of it) and cites the reference lines it stands in for:
 *
 *   W = Westervelt_relax_fft_Pressure_Energy.cu   (pressure / acoustic power)
 *   T = Westervelt_Temperature_SquareSpiral.cu    (bioheat + CEM43 along a spiral)
 *   G = Gilmore_liver_3fr_combo.cu                (Gilmore-Zener bubble dynamics)
 *
 * Conventions
 *   - Every call returns a bd_status; no exception crosses the ABI.  The text of
 *     the last error on the calling thread is returned by bd_last_error_string().
 *   - The caller owns every host buffer.  A bd_context owns the device memory it
 *     allocates; one context per host thread.
 *   - Arrays of cells are x-fastest: idx = (iz*ny + iy)*nx + ix, as in W:155.
 *   - Calls are blocking unless their name ends in _device (those take device
 *     pointers and a cudaStream_t passed as void*, and return once enqueued).
 */
#ifndef BUBBLEDYN_H
#define BUBBLEDYN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BD_ABI_VERSION 2   /* 2: bd_thermal.plain_launches; z-slab entry points */

#define BD_MAX_MATERIALS 8
#define BD_MAX_RELAX 4
#define BD_MAX_TONES 4
#define BD_MAX_DFT 16
#define BD_MAX_BUBBLE_TONES 9

typedef enum bd_status {
    BD_OK = 0,
    BD_ERR_INVALID_ARG = 1,
    BD_ERR_OOM = 2,
    BD_ERR_CUDA = 3,
    BD_ERR_UNSTABLE = 4,        /* NaN/Inf or amplitude blow-up detected in a field */
    BD_ERR_TIMEOUT = 5,         /* a bounded device wait ran out */
    BD_ERR_IO = 6,
    BD_ERR_FAULT_INJECTED = 7,  /* host-side fault injection fired (bd_westervelt_params.fault_at_step) */
    BD_ERR_UNSUPPORTED = 8,
    BD_ERR_STATE = 9            /* call out of order (e.g. checkpoint of another geometry) */
} bd_status;

typedef enum bd_precision { BD_F32 = 0, BD_F64 = 1 } bd_precision;

/* Boundary treatment of one face of the box. */
typedef enum bd_face_kind {
    BD_FACE_OPEN = 0,    /* stencil sees p = 0 outside; combine with a sponge */
    BD_FACE_MUR = 1,     /* first-order Mur ABC on mur_layers layers (W:88-135) */
    BD_FACE_MIRROR = 2   /* even symmetry plane at index 0: p[-k] = p[k] (W:176-200); x-/y- only */
} bd_face_kind;

/* ------------------------------------------------------------------------- */
/* Context and errors                                                         */
/* ------------------------------------------------------------------------- */
typedef struct bd_context bd_context;

/* Replaces cudaSetDevice(0) at W:353, T:112, G:436. */
bd_status bd_context_create(int device, bd_context** out);
bd_status bd_context_destroy(bd_context* ctx);
/* Thread-local text of the last error (never NULL). */
const char* bd_last_error_string(void);
int bd_abi_version(void);
/* Number of this library's own kernels launched by the context so far. */
bd_status bd_context_kernel_launches(bd_context* ctx, int64_t* out);
/* Self-test of the bounded waits that guard every TMA pipeline in the step
 * kernels (a stalled pipeline ends the kernel with BD_ERR_TIMEOUT instead of
 * hanging): one warp waits on a barrier that nothing completes.  *timed_out is
 * 1 when the wait gave up after limit_ms (1..2000) as designed; *elapsed_ms
 * gets the kernel's device time.  The context stays usable afterwards. */
bd_status bd_selftest_bounded_wait(bd_context* ctx, int32_t limit_ms, int32_t* timed_out, double* elapsed_ms);

/* ------------------------------------------------------------------------- */
/* Westervelt pressure / energy solver (W)                                    */
/* ------------------------------------------------------------------------- */

/* Mesh.  Mirrors W:406-417 (xy_min, dxy, z_min, dz, dt). */
typedef struct bd_grid {
    int32_t nx, ny, nz;         /* cells; the reference uses nx = ny = Nxy (W:410) */
    int32_t pad0;
    double x0, y0, z0;          /* coordinate of cell (0,0,0) [m] (W:48-50) */
    double dx, dz;              /* dy == dx [m] */
    double dt;                  /* time step [s] (W:416) */
    int32_t face[6];            /* bd_face_kind of x-, x+, y-, y+, z-, z+ */
    int32_t mur_layers;         /* Mur layers on MUR faces; 3 in W:108-133 (z- uses source_iz layers) */
    int32_t sponge_cells;       /* damping layer width on OPEN faces (0 = none) */
    double sponge_strength;     /* w(d) = exp(-strength*(d/W)^2) applied each step */
} bd_grid;

/* One acoustic material.  Mirrors the water/tissue blocks W:16-33, W:365-393. */
typedef struct bd_material {
    double c0;                  /* sound speed [m/s] (used where no c map is given) */
    double rho;                 /* density [kg/m^3] */
    double beta;                /* nonlinearity coefficient */
    double delta;               /* acoustic diffusivity [m^2/s] */
    int32_t n_relax;            /* relaxation processes (W hard-codes 2 in tissue, 0 in water) */
    int32_t pad0;
    double relax_c[BD_MAX_RELAX];   /* small sound speeds c_nu [m/s] (W:390-391) */
    double relax_tau[BD_MAX_RELAX]; /* relaxation times tau_nu [s] (W:392-393) */
    double absorption;          /* alpha [Np/m] at the fundamental, for the water power (W:261) */
    double harm_absorption;     /* alpha_n = harm_absorption * n*f/1e6 [Np/m] (W:342) */
} bd_material;

typedef struct bd_medium {
    int32_t n_materials;
    int32_t pad0;
    bd_material mat[BD_MAX_MATERIALS];
    const int32_t* plane_material;  /* nz entries or NULL: material of each z plane (W:212) */
    const uint8_t* material_map;    /* nx*ny*nz or NULL: per-cell material (overrides planes) */
    const float* c_map;             /* nx*ny*nz or NULL: per-cell sound speed (overrides c0) */
} bd_medium;

typedef enum bd_source_kind {
    BD_SRC_NONE = 0,
    BD_SRC_BOWL = 1,            /* spherical bowl projected onto a plane (W:62-85) */
    BD_SRC_ARRAY = 2            /* same projection, cells grouped into phased-array elements */
} bd_source_kind;

/* Dirichlet source plane.  Mirrors W:36-42 and W:355-400. */
typedef struct bd_source {
    int32_t kind;               /* bd_source_kind */
    int32_t plane_iz;           /* z index of the source plane; W:75 uses 2 */
    double focal_length;        /* d [m] (W:38) */
    double alpha;               /* outer aperture half-angle [rad] (W:39) */
    double alpha_hole;          /* central hole half-angle [rad] (W:40) */
    double p0;                  /* on-source pressure amplitude [Pa] (W:42) */
    double c_delay;             /* sound speed of the geometric delay (W:81 uses c_inf) */
    double cx, cy;              /* bowl axis position in the plane [m] (0,0 in W) */
    int32_t n_tones;            /* drive = sum_k amp_k sin(2 pi f_k t' + phase_k) */
    int32_t pad0;
    double freq[BD_MAX_TONES];
    double amp[BD_MAX_TONES];
    double phase[BD_MAX_TONES];
    double burst_cycles;        /* 0 = continuous wave (W); else rectangular burst of this many cycles of freq[0] */
    int32_t n_elements;         /* BD_SRC_ARRAY: number of elements */
    int32_t pad1;
    const int32_t* element_of_cell; /* nx*ny: element index of each plane cell or -1 */
    const double* element_phase;    /* n_elements [rad] */
    const double* element_amp;      /* n_elements (relative) */
} bd_source;

typedef enum bd_energy_mode {
    BD_ENERGY_P2 = 0,           /* E += p^2 dt            (time-integrated intensity * rho c) */
    BD_ENERGY_DPDT2 = 1         /* E += ((p^{n+1}-p^{n-1})/2dt)^2 dt  (W:253-257) */
} bd_energy_mode;

/* Time discretisation of the relaxation memory variables. */
typedef enum bd_relax_scheme {
    BD_RELAX_REFERENCE = 0,     /* W:226-228: BDF2 memory driven by the backward 5-level d3p/dt3 (W:207);
                                   amplifies grid-scale modes when (c dt/dx)^2 * 18.1 exceeds ~0.5 */
    BD_RELAX_SEMI_IMPLICIT = 1  /* same BDF2 memory driven by the 2nd-order d3p/dt3 at t_n through
                                   p^{n+1}..p^{n-3}, solved per cell; damps every mode up to CFL ~0.39 */
} bd_relax_scheme;

typedef enum bd_q_mode {
    BD_Q_NONE = 0,
    BD_Q_REFERENCE = 1          /* W:261 in water planes, W:341-342 harmonics at iz >= q_iz_split */
} bd_q_mode;

typedef struct bd_westervelt_params {
    int32_t precision;          /* bd_precision of the stored fields */
    int32_t energy_mode;        /* bd_energy_mode */
    int64_t n_steps;            /* time steps to run */
    double t0;                  /* time before step 0 [s]; step s runs at t = t0 + (s+1) dt */
    const double* t_src;        /* optional n_steps source times (W:564 accumulates t += dt) */
    int64_t peak_start, peak_end;       /* step window [start, end) of the peak |p| map */
    int64_t energy_start, energy_end;   /* step window of the energy accumulator (W:627) */
    int64_t dft_start, dft_len;         /* DFT window: samples s = dft_start .. dft_start+dft_len-1 */
    int32_t n_dft;                      /* frequencies accumulated on the fly (W:663-755 replacement) */
    int32_t dft_z_lo, dft_z_hi;         /* planes [lo, hi) where the DFT is kept (W:673: tissue) */
    int32_t q_mode;                     /* bd_q_mode */
    double dft_freq[BD_MAX_DFT];        /* [Hz]; sample phase = 2 pi f (s - dft_start) dt */
    int32_t q_iz_split;                 /* W:673 iz_tissue */
    int32_t q_n_harm;                   /* W:670 N_harm */
    double q_freq;                      /* fundamental of the Q formulas (W:261, W:342) */
    int32_t check_every;                /* NaN / blow-up probe interval in steps (0 = off) */
    int32_t fault_at_step;              /* host-side fault injection: fail at this step (-1 = off) */
    double blowup_limit;                /* |p| above this counts as unstable (0 = only NaN/Inf) */
    int32_t graph_chunk;                /* steps per captured CUDA graph (0 = 50, < 0 = plain launches) */
    int32_t tile_variant;               /* kernel variant (-1 = autotuned / default) */
    int32_t relax_scheme;               /* bd_relax_scheme */
    int32_t pad0;
} bd_westervelt_params;

/* Host output buffers; any may be NULL.  Element type is float for BD_F32 and
 * double for BD_F64 (Q is always double, as written by W:778-790). */
typedef struct bd_westervelt_outputs {
    void* p_final;              /* nx*ny*nz pressure after the last step */
    void* peak;                 /* nx*ny*nz max |p| over the peak window */
    void* energy;               /* nx*ny*nz energy accumulator */
    void* dft_re;               /* n_dft * nx*ny*(dft_z_hi-dft_z_lo) */
    void* dft_im;
    double* Q;                  /* nx*ny*nz acoustic power density [W/m^3] (BD_Q_REFERENCE) */
    double elapsed_ms;          /* device time of the solve (filled by the library) */
    int64_t steps_done;
    int32_t tile_variant;       /* step-kernel variant the solve ran (filled by the library) */
    int32_t pad0;
} bd_westervelt_outputs;

/* Full Westervelt solve.  Replaces W:350-790 (the three time loops, the FFT
 * pass and the result copy) with one fused kernel per step. */
bd_status bd_westervelt_run(bd_context* ctx, const bd_grid* grid, const bd_medium* medium,
                            const bd_source* source, const bd_westervelt_params* params,
                            bd_westervelt_outputs* out);

/* Session form of the same solve: begin, advance in pieces, checkpoint/resume,
 * finish.  The reference's only checkpoint is the host snapshot at W:600-613
 * restored at W:690-703. */
typedef struct bd_westervelt bd_westervelt;
bd_status bd_westervelt_begin(bd_context* ctx, const bd_grid* grid, const bd_medium* medium,
                              const bd_source* source, const bd_westervelt_params* params,
                              bd_westervelt** out);
bd_status bd_westervelt_advance(bd_westervelt* wv, int64_t n_steps);
bd_status bd_westervelt_step_index(bd_westervelt* wv, int64_t* step);
bd_status bd_westervelt_finish(bd_westervelt* wv, bd_westervelt_outputs* out);
bd_status bd_westervelt_end(bd_westervelt* wv);
/* Checkpoint blob: header + time-level ring + relaxation state + accumulators. */
bd_status bd_checkpoint_size(bd_westervelt* wv, size_t* bytes);
bd_status bd_checkpoint_save(bd_westervelt* wv, void* blob, size_t bytes);
bd_status bd_checkpoint_load(bd_westervelt* wv, const void* blob, size_t bytes);
/* Device time of the last advance() in milliseconds. */
bd_status bd_westervelt_last_ms(bd_westervelt* wv, double* ms);

/* ------------------------------------------------------------------------- */
/* z-slab domain decomposition of the Westervelt solve                        */
/* ------------------------------------------------------------------------- */
/* The reference runs one grid on one device (cudaSetDevice(0), W:353); these
 * calls split the grid into slabs of whole z planes, one per device (or
 * several on one device).  The 6th-order stencil reads p^n at iz-3..iz+3
 * (W:169-174), so a slab keeps 3 ghost planes beyond each internal face,
 * copied from the neighbour after every step; everything else a step reads is
 * cell-local.  With the ghosts refreshed after every step, the owned planes
 * evolve bit for bit as in one session over the whole grid.
 *
 * bd_westervelt_slab_begin: a session for the planes [z_begin, z_end) of the
 * whole problem (grid, medium, source, params describe the whole grid; at least
 * 8 owned planes; Mur layers of the z faces must lie inside the end slabs).
 * Advance it ONE step at a time and refresh the ghosts between steps.  finish()
 * writes the owned planes only: p_final / peak / energy / Q hold
 * nx*ny*(z_end - z_begin) values, dft_re / dft_im the owned planes inside
 * [dft_z_lo, dft_z_hi). */
bd_status bd_westervelt_slab_begin(bd_context* ctx, const bd_grid* grid, const bd_medium* medium,
                                   const bd_source* source, const bd_westervelt_params* params, int32_t z_begin,
                                   int32_t z_end, bd_westervelt** out);
/* Bytes of one halo message: 3 planes of nx*ny cells of the field type. */
bd_status bd_westervelt_halo_bytes(bd_westervelt* wv, size_t* bytes);
/* Halo transfer of the newest pressure level through a device buffer of
 * bd_westervelt_halo_bytes: to_ghost = 0 copies the 3 owned planes next to
 * internal face `side` (0 = low z, 1 = high z) into d_buf (the message for that
 * neighbour); to_ghost = 1 copies d_buf into the 3 ghost planes beyond it.
 * Enqueued on stream (NULL = the context's stream); the transport between
 * devices (NCCL send/recv, or a copy into the receiver's own memory) is the
 * caller's. */
bd_status bd_westervelt_halo_copy(bd_westervelt* wv, int32_t side, int32_t to_ghost, void* d_buf, void* stream);
/* Same-device exchange between neighbouring slabs of one context (lower owns
 * the planes just below upper's): both directions, enqueued on the context's
 * stream. */
bd_status bd_halo_exchange(bd_westervelt* lower, bd_westervelt* upper);
/* The whole solve as n_slabs equal slabs on this context's device, with the
 * ghost planes exchanged after every step; outputs as bd_westervelt_run (the
 * whole grid).  Checks the decomposition: its results equal bd_westervelt_run's
 * bit for bit. */
bd_status bd_westervelt_run_slabs(bd_context* ctx, const bd_grid* grid, const bd_medium* medium,
                                  const bd_source* source, const bd_westervelt_params* params, int32_t n_slabs,
                                  bd_westervelt_outputs* out);

/* ------------------------------------------------------------------------- */
/* Adjoint Westervelt (phased-array gradients)                                */
/* ------------------------------------------------------------------------- */

/* loss = -sum_{focal region} E + side_weight * sum_{side-lobe region} E,
 * E(x) = sum over the window of p(x)^2 dt.  The focal region is the ball of
 * radius focal_radius cells around the focus; the side-lobe region is the
 * focal plane outside side_radius cells. */
typedef struct bd_focal_loss {
    int32_t focus_ix, focus_iy, focus_iz;
    int32_t focal_radius;
    int32_t side_radius;
    int32_t checkpoint_every;           /* forward checkpoint interval: 0 = ceil(sqrt(n_steps));
                                           < 0 = keep the whole history in device memory when it
                                           fits in half of the free memory, else ceil(sqrt(n_steps)) */
    double side_weight;
    int64_t window_start, window_end;   /* step window [start, end) */
} bd_focal_loss;

/* Gradient of the loss with respect to element phases and amplitudes of a
 * BD_SRC_ARRAY source (no counterpart in the reference; the forward model is
 * W:139-236 + W:62-85).  Discrete adjoint of the step, sqrt(N) forward
 * checkpoints with recomputation per segment; OPEN faces only.  grad_phase /
 * grad_amp have n_elements entries; timings_ms (may be NULL) receives the
 * forward, recompute and backward device times. */
bd_status bd_westervelt_adjoint(bd_context* ctx, const bd_grid* grid, const bd_medium* medium,
                                const bd_source* source, const bd_westervelt_params* params,
                                const bd_focal_loss* loss, double* loss_out,
                                double* grad_phase, double* grad_amp, double* timings_ms);
/* The same gradient computed on n_slabs z slabs of this context's device (the
 * z-slab split of a multi-GPU adjoint, each slab its own fields, checkpoints
 * and adjoint rings): 3 ghost planes of p^n exchanged after every forward and
 * recompute step, of H (the only field the backward stencil couples) after
 * every backward step; loss and gradients equal bd_westervelt_adjoint's bit
 * for bit.  1 <= n_slabs <= nz / 8; plain launches (no graphs). */
bd_status bd_westervelt_adjoint_slabs(bd_context* ctx, const bd_grid* grid, const bd_medium* medium,
                                      const bd_source* source, const bd_westervelt_params* params,
                                      const bd_focal_loss* loss, int32_t n_slabs, double* loss_out,
                                      double* grad_phase, double* grad_amp, double* timings_ms);

/* ------------------------------------------------------------------------- */
/* Bioheat + CEM43 dose along a scan trajectory (T)                           */
/* ------------------------------------------------------------------------- */

typedef struct bd_thermal_material {
    double rho;                 /* density [kg/m^3] (T:125, T:132) */
    double c_t;                 /* specific heat [J/(kg K)] (T:127, T:134) */
    double k_t;                 /* thermal conductivity [W/(m K)] (T:128, T:135) */
    double perfusion;           /* Pennes perfusion rate w [1/s] (0 in T) */
    double T_art;               /* arterial temperature [K] */
    double T_init;              /* initial temperature [K] (T:149-150) */
} bd_thermal_material;

typedef struct bd_thermal {
    int32_t nx, ny, nz;
    int32_t precision;          /* BD_F64: T in double (T exact); BD_F32: dT from T_ref in float */
    double dx, dz, dt;          /* T:157-166 */
    double T_ref;               /* BD_F32 baseline temperature [K] */
    int32_t n_materials;
    int32_t dose_init;          /* 1: TD starts at R^(43-T0) dt like T:246-252; 0: zero */
    bd_thermal_material mat[BD_MAX_MATERIALS];
    const int32_t* plane_material;  /* nz entries (T:84 split by z) */
    const uint8_t* material_map;    /* optional nx*ny*nz */
    const double* T_start;          /* optional nx*ny*nz initial temperature [K] (NULL: mat[].T_init) */
    const double* dose_start;       /* optional nx*ny*nz initial dose [s] (NULL: dose_init rule);
                                       with both, a run continues where an earlier one ended */
    int32_t plain_launches;         /* 0: the step loop replays one captured CUDA graph per 64 steps
                                       (replaces T's launch + cudaDeviceSynchronize per step, T:345-392);
                                       1: one launch per step */
    int32_t pad1;
} bd_thermal;

typedef enum bd_trajectory_kind {
    BD_TRAJ_SQUARE_SPIRAL = 0,  /* continuous motion of T:141-173, T:323-410 */
    BD_TRAJ_SPOTS = 1           /* discrete focal spots, each held for a number of steps */
} bd_trajectory_kind;

typedef struct bd_trajectory {
    int32_t kind;
    int32_t n_legs;             /* T:328 spiral_lines */
    double speed;               /* [m/s] T:141 */
    double scale;               /* spacing between lines [m] T:142 */
    double speed_init;          /* T:144 */
    double t_acc;               /* T:145 */
    double dxy;                 /* grid step of the shift [m] */
    double dt;                  /* heat time step [s] */
    int32_t n_spots;            /* BD_TRAJ_SPOTS */
    int32_t pad0;
    const int32_t* spot_sx;     /* shift of Q in cells per spot */
    const int32_t* spot_sy;
    const int64_t* spot_steps;  /* heat steps per spot */
} bd_trajectory;

/* Expand a trajectory into per-step integer shifts of the heat source.
 * Replaces the host loop T:345-410.  Writes at most cap entries; *n_steps gets
 * the full count and leg_end[k] (may be NULL, n_legs entries) the step count
 * after leg/spot k. */
bd_status bd_trajectory_shifts(const bd_trajectory* traj, int32_t* sx, int32_t* sy,
                               int64_t cap, int64_t* n_steps, int64_t* leg_end, int32_t leg_cap);

/* Mirror a quarter-domain field (ix,iy >= 0 of W's output .bin, W:778-790)
 * into the full domain: full[iz][iy][ix] = small[iz][|iy-h|][|ix-h|], h = n_half
 * (T:269-306).  small has (n_half+1)^2 cells per plane. */
bd_status bd_unfold_quarter(const double* small, int32_t n_half, int32_t nz, double* full);

typedef struct bd_heat_outputs {
    double* T_final;            /* nx*ny*nz temperature [K] */
    double* dose;               /* nx*ny*nz CEM43 dose [s] */
    double* snapshots;          /* n_snap * nx*ny*nz temperature [K] after the listed legs (T:411-563) */
    const int32_t* snapshot_legs;  /* leg numbers (1-based) after which to copy T */
    int32_t n_snap;
    int32_t pad0;
    double elapsed_ms;
    int64_t steps_done;
} bd_heat_outputs;

/* Heat + dose run over a trajectory with a fixed source Q (full domain, W/m^3)
 * shifted by the trajectory.  Replaces T:345-573. */
bd_status bd_spiral_heat_run(bd_context* ctx, const bd_thermal* thermal, const double* Q,
                             const bd_trajectory* traj, int64_t max_steps,
                             bd_heat_outputs* out);
/* The same run as n_slabs z slabs on this context's device (the z-slab split
 * of a multi-GPU heat solve, each slab its own buffers): slab k owns planes
 * [nz k / n_slabs, nz (k + 1) / n_slabs) and keeps one ghost plane beyond each
 * internal face (the stencil reads iz +- 1, T:72-73), refreshed from the
 * neighbour after every step.  Outputs as bd_spiral_heat_run (the whole grid),
 * equal to its bit for bit; 1 <= n_slabs <= nz / 2. */
bd_status bd_spiral_heat_run_slabs(bd_context* ctx, const bd_thermal* thermal, const double* Q,
                                   const bd_trajectory* traj, int64_t max_steps, int32_t n_slabs,
                                   bd_heat_outputs* out);

/* One rank's z slab of the heat run (the multi-GPU split of T:345-573; the
 * reference runs one grid on one device, T:112): the slab owns planes
 * [z_begin, z_end) (at least 2) of the whole problem and keeps one ghost plane
 * beyond each internal face.  The caller steps it (bd_heat_slab_advance, which
 * returns once the steps are done) and refreshes the ghost planes between
 * steps: bd_heat_slab_halo_copy with to_ghost = 0 copies the newest owned
 * plane next to face `side` (0 = low z, 1 = high z) into d_buf (one plane,
 * bd_heat_slab_halo_bytes), to_ghost = 1 copies d_buf into the ghost plane
 * beyond it; the transport between devices is the caller's.  Enqueued on
 * stream (NULL = the context's stream).  bd_heat_slab_finish writes the owned
 * planes of T and the dose into whole-grid host arrays at their own offsets
 * (T_final / dose of bd_heat_outputs; snapshots are not taken). */
typedef struct bd_heat_slab bd_heat_slab;
bd_status bd_heat_slab_begin(bd_context* ctx, const bd_thermal* thermal, const double* Q,
                             const bd_trajectory* traj, int64_t max_steps, int32_t z_begin, int32_t z_end,
                             bd_heat_slab** out);
bd_status bd_heat_slab_steps(bd_heat_slab* slab, int64_t* total, int64_t* done);
bd_status bd_heat_slab_advance(bd_heat_slab* slab, int64_t n);
bd_status bd_heat_slab_halo_bytes(bd_heat_slab* slab, size_t* bytes);
bd_status bd_heat_slab_halo_copy(bd_heat_slab* slab, int32_t side, int32_t to_ghost, void* d_buf, void* stream);
bd_status bd_heat_slab_finish(bd_heat_slab* slab, bd_heat_outputs* out);
bd_status bd_heat_slab_end(bd_heat_slab* slab);

/* Allocation-free variant of the FP32 heat + dose run, for callers that
 * cannot call cudaMalloc: code running inside another framework's memory
 * arena, which owns the device memory and forbids driver allocations, or a
 * real-time loop where an allocation's implicit device synchronisation would
 * stall other work.  No counterpart in the reference (whose host program
 * allocates every field itself, T:259-306).
 *
 * The caller owns every input and output on the device: d_theta (nx*ny*nz
 * floats, T - thermal->T_ref, updated in place), d_Q (nx*ny*nz floats, W/m^3)
 * and d_dose (2*nx*ny*nz floats: hi, lo pairs whose sum is the CEM43 dose in
 * seconds, updated in place).  shifts is a host array of n_steps (sx, sy)
 * int32 pairs, e.g. from bd_trajectory_shifts.  The library's scratch (the
 * second temperature buffer, the shift table and a step counter) is one
 * static device array of BD_NOALLOC_SCRATCH_BYTES that every GPU which loads
 * the library keeps until the process exits; sizes above BD_NOALLOC_MAX_CELLS
 * cells, BD_NOALLOC_MAX_STEPS steps or BD_NOALLOC_MAX_PLANES planes are
 * rejected with BD_ERR_INVALID_ARG.  thermal->precision must be BD_F32 and
 * thermal->material_map NULL (plane_material is honoured).
 *
 * The first call on a device looks up the address of that array (with the
 * device current); make that first call before any stream capture.  The
 * address stays valid for the life of the device's primary context: do not
 * keep using the library after cudaDeviceReset.  Every call shares the array
 * and leaves its contents behind, so two calls whose work overlaps on the GPU
 * (different streams, or different contexts on the same device) race with
 * each other; serialise them.  The call returns once its work is enqueued on
 * stream (NULL = the context's stream).  shifts and thermal->plane_material
 * are read by host-to-device copies enqueued on that stream: from pageable
 * memory they are staged before the call returns; from page-locked memory the
 * copy reads them when the stream reaches it, so keep them alive and unchanged
 * until the stream has passed this call's work. */
#define BD_NOALLOC_MAX_CELLS (1 << 21)
#define BD_NOALLOC_MAX_STEPS (1 << 16)
#define BD_NOALLOC_MAX_PLANES 4096
#define BD_NOALLOC_SCRATCH_BYTES (256 + 4 * BD_NOALLOC_MAX_PLANES + 8 * BD_NOALLOC_MAX_STEPS + 4 * BD_NOALLOC_MAX_CELLS)
bd_status bd_heat_run_device_noalloc(bd_context* ctx, const bd_thermal* thermal, float* d_theta, const float* d_Q,
                                     float* d_dose, const int32_t* shifts, int64_t n_steps, void* stream);

/* ------------------------------------------------------------------------- */
/* Gilmore-Zener bubble dynamics (G)                                          */
/* ------------------------------------------------------------------------- */

/* Medium constants, G:13-23 / G:440-450. */
typedef struct bd_gilmore_medium {
    double rho, P0, S2, mu4, G4_3, C_inf, lambda, n, B, gamma;
} bd_gilmore_medium;

/* Drive: P(t) = sum_k a[k] sin(2 pi f[k] t + phi[k]).  bd_gilmore_combo_tones()
 * builds the single/dual/triple normalisation of G:40-57. */
typedef struct bd_bubble {
    double R0;
    int32_t n_tones;
    int32_t pad0;
    double f[BD_MAX_BUBBLE_TONES];
    double a[BD_MAX_BUBBLE_TONES];
    double phi[BD_MAX_BUBBLE_TONES];
} bd_bubble;

typedef struct bd_ode_params {
    double t_end;               /* integration end [s] */
    double h0;                  /* first step (G:355: 1e-13) */
    double atol, rtol;          /* G:214-215 use 1e-9 / 1e-9 */
    double fac_max;             /* G:244: 5 */
    int64_t max_steps;          /* per-bubble attempt cap (flagged, never a hang) */
    int32_t stop_at_threshold;  /* 1: stop when R' <= -C_inf (G:313) */
    int32_t ref_arith;          /* 1: evaluate the RHS in the reference's operation order (no FSAL) */
    int32_t schedule;           /* bd_schedule: persistent work-stealing lanes (default) or static */
    int32_t pad0;
} bd_ode_params;

typedef enum bd_schedule {
    BD_SCHEDULE_PERSISTENT = 0, /* lanes pull the next bubble when theirs finishes (batches no larger
                                   than the resident lanes run one bubble per thread) */
    BD_SCHEDULE_STATIC = 1      /* one thread per bubble for its whole run (comparison baseline) */
} bd_schedule;

typedef enum bd_bubble_status {
    BD_BUBBLE_DONE = 0,
    BD_BUBBLE_THRESHOLD = 1,    /* stopped at R' <= -C_inf */
    BD_BUBBLE_STEP_CAP = 2,
    BD_BUBBLE_NONFINITE = 3
} bd_bubble_status;

typedef struct bd_bubble_result {
    double R, Rdot, tau, q, t;
    double R_max, R_min;
    double t_threshold;         /* first time R' <= -C_inf, or -1 */
    int64_t n_accept, n_reject;
    int32_t status;             /* bd_bubble_status */
    int32_t threshold;          /* 1 if R' <= -C_inf was reached */
} bd_bubble_result;

/* The single/dual/triple drive of G:40-57 for amplitude A and frequencies
 * f1 <= f2 <= f3 as tones (phases phi may be NULL = 0). */
bd_status bd_gilmore_combo_tones(double A, const double f[3], const double* phi, bd_bubble* b);

/* Frequency combinations of G:498-520: log-spaced n_fr frequencies in
 * [f_min, f_max], ordered triples i <= ii <= iii excluding i < ii == iii.
 * Writes 3*n entries into out (cap triples); *n_combo gets the count. */
bd_status bd_gilmore_combos(int32_t n_fr, double f_min, double f_max, double* out,
                            int64_t cap, int64_t* n_combo);

/* Forward integration of n bubbles with a persistent work-stealing kernel.
 * The integrator is G:183-318 (Dormand-Prince 5(4)); G itself only runs it
 * inside the threshold search. */
bd_status bd_gilmore_run(bd_context* ctx, const bd_gilmore_medium* medium, int64_t n,
                         const bd_bubble* bubbles, const bd_ode_params* ode,
                         bd_bubble_result* results, double* elapsed_ms);
/* Device-pointer form: d_bubbles / d_results on the device, work enqueued on
 * stream (NULL = the context's stream), returns once enqueued.  The persistent
 * schedule's work counter belongs to the context, so two calls on one context
 * whose work overlaps on the GPU (different streams) race on it: serialise
 * them, or give each stream its own context. */
bd_status bd_gilmore_run_device(bd_context* ctx, const bd_gilmore_medium* medium, int64_t n,
                                const bd_bubble* d_bubbles, const bd_ode_params* ode,
                                bd_bubble_result* d_results, void* stream);

/* Threshold search of G:323-429 for every (combo, R0) pair; results are
 * combo-major (results[i_combo*n_R0 + i_R0]) like G:598.  A = 1e7 means no
 * cavitation up to 10 MPa; -1 is never left behind (G:359 initial value). */
bd_status bd_gilmore_threshold(bd_context* ctx, const bd_gilmore_medium* medium,
                               const double* fr_combo, int64_t n_combo,
                               const double* R0, int64_t n_R0, int32_t ref_arith,
                               int64_t max_steps, double* results, double* elapsed_ms);

typedef enum bd_search {
    BD_SEARCH_LINEAR = 0,       /* G's scan: 0.1 MPa up, then 10 kPa and 1 kPa down (G:367-425) */
    BD_SEARCH_BISECT = 1        /* 0.1 MPa up as G, then bisection in 1 kPa units inside the last
                                   0.1 MPa bracket: 7 integrations instead of up to 20; equal to the
                                   linear scan wherever cavitation is monotonic in the amplitude
                                   inside that bracket */
} bd_search;

/* bd_gilmore_threshold with the search chosen (bd_search); BD_SEARCH_LINEAR is
 * bd_gilmore_threshold itself. */
bd_status bd_gilmore_threshold_search(bd_context* ctx, const bd_gilmore_medium* medium,
                                      const double* fr_combo, int64_t n_combo,
                                      const double* R0, int64_t n_R0, int32_t ref_arith,
                                      int64_t max_steps, int32_t search, double* results,
                                      double* elapsed_ms);

/* ------------------------------------------------------------------------- */
/* The reference programs' files (host only)                                  */
/* ------------------------------------------------------------------------- */

/* W's absorbed-power volume Q3D_*.bin (W:778-790): raw doubles of planes
 * iz_first..nz-1 (W: 2), rows iy, columns ix; T reads it back (T:276-279). */
bd_status bd_write_q_bin(const char* path, const double* Q, int32_t nx, int32_t ny, int32_t nz, int32_t iz_first);
/* Reads exactly n doubles (*n_read gets what the file held, up to n). */
bd_status bd_read_q_bin(const char* path, double* out, int64_t n, int64_t* n_read);
/* W's on-axis power Q_Z_*.dat (W:767-775): "z(m);Q(W/m^3)", then z;Q per plane
 * from iz_first at x = y = 0. */
bd_status bd_write_q_axis_dat(const char* path, const double* Q, int32_t nx, int32_t ny, int32_t nz, double z_min,
                              double dz, int32_t iz_first);

typedef enum bd_slice {
    BD_SLICE_XZ = 0,            /* rows z in [r0, r1), columns x in [c0, c1), at y = fixed (T:424-432) */
    BD_SLICE_XY = 1             /* rows y in [r0, r1), columns x in [c0, c1), at z = fixed (T:437-445) */
} bd_slice;

/* T's temperature / dose slices (T:419-448, T:576-640): the header row
 * (NULL: "Z=rows;X=columns" / "Y=rows;X=columns"), then one row per slice row
 * of "value;" cells. */
bd_status bd_write_slice_dat(const char* path, const double* field, int32_t nx, int32_t ny, int32_t nz,
                             int32_t orientation, int32_t fixed, int32_t r0, int32_t r1, int32_t c0, int32_t c1,
                             const char* header);
/* G's threshold table dR_Cinf_*.dat (G:582-613): "fr1;fr2;fr3 --> R0;R0...",
 * one row per combination (fr1;fr2;fr3;A...) and "time (s);t". */
bd_status bd_write_threshold_table(const char* path, const double* fr_combo, int64_t n_combo, const double* R0,
                                   int64_t n_R0, const double* results, double elapsed_s);

#ifdef __cplusplus
}
#endif
#endif /* BUBBLEDYN_H */
