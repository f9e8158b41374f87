"""ctypes mirror of include/bubbledyn.h.

Field order, types and padding follow the C header exactly; ``check_layout``
compares the struct sizes against the ones the compiled library reports.
"""
import ctypes as C

BD_MAX_MATERIALS = 8
BD_MAX_RELAX = 4
BD_MAX_TONES = 4
BD_MAX_DFT = 16
BD_MAX_BUBBLE_TONES = 9

# bd_status
BD_OK = 0
BD_ERR_INVALID_ARG = 1
BD_ERR_OOM = 2
BD_ERR_CUDA = 3
BD_ERR_UNSTABLE = 4
BD_ERR_TIMEOUT = 5
BD_ERR_IO = 6
BD_ERR_FAULT_INJECTED = 7
BD_ERR_UNSUPPORTED = 8
BD_ERR_STATE = 9
STATUS_NAMES = {
    0: "BD_OK", 1: "BD_ERR_INVALID_ARG", 2: "BD_ERR_OOM", 3: "BD_ERR_CUDA",
    4: "BD_ERR_UNSTABLE", 5: "BD_ERR_TIMEOUT", 6: "BD_ERR_IO",
    7: "BD_ERR_FAULT_INJECTED", 8: "BD_ERR_UNSUPPORTED", 9: "BD_ERR_STATE",
}

BD_F32 = 0
BD_F64 = 1

BD_FACE_OPEN = 0
BD_FACE_MUR = 1
BD_FACE_MIRROR = 2

BD_SRC_NONE = 0
BD_SRC_BOWL = 1
BD_SRC_ARRAY = 2

BD_ENERGY_P2 = 0
BD_ENERGY_DPDT2 = 1

BD_RELAX_REFERENCE = 0
BD_RELAX_SEMI_IMPLICIT = 1

BD_Q_NONE = 0
BD_Q_REFERENCE = 1

BD_TRAJ_SQUARE_SPIRAL = 0
BD_TRAJ_SPOTS = 1

BD_BUBBLE_DONE = 0
BD_BUBBLE_THRESHOLD = 1
BD_BUBBLE_STEP_CAP = 2
BD_BUBBLE_NONFINITE = 3

BD_SCHEDULE_PERSISTENT = 0
BD_SCHEDULE_STATIC = 1
BD_SEARCH_LINEAR = 0
BD_SEARCH_BISECT = 1

BD_SLICE_XZ = 0
BD_SLICE_XY = 1

i32 = C.c_int32
i64 = C.c_int64
f64 = C.c_double
vp = C.c_void_p


class Grid(C.Structure):
    _fields_ = [
        ("nx", i32), ("ny", i32), ("nz", i32), ("pad0", i32),
        ("x0", f64), ("y0", f64), ("z0", f64),
        ("dx", f64), ("dz", f64), ("dt", f64),
        ("face", i32 * 6),
        ("mur_layers", i32), ("sponge_cells", i32),
        ("sponge_strength", f64),
    ]


class Material(C.Structure):
    _fields_ = [
        ("c0", f64), ("rho", f64), ("beta", f64), ("delta", f64),
        ("n_relax", i32), ("pad0", i32),
        ("relax_c", f64 * BD_MAX_RELAX), ("relax_tau", f64 * BD_MAX_RELAX),
        ("absorption", f64), ("harm_absorption", f64),
    ]


class Medium(C.Structure):
    _fields_ = [
        ("n_materials", i32), ("pad0", i32),
        ("mat", Material * BD_MAX_MATERIALS),
        ("plane_material", vp), ("material_map", vp), ("c_map", vp),
    ]


class Source(C.Structure):
    _fields_ = [
        ("kind", i32), ("plane_iz", i32),
        ("focal_length", f64), ("alpha", f64), ("alpha_hole", f64), ("p0", f64),
        ("c_delay", f64), ("cx", f64), ("cy", f64),
        ("n_tones", i32), ("pad0", i32),
        ("freq", f64 * BD_MAX_TONES), ("amp", f64 * BD_MAX_TONES), ("phase", f64 * BD_MAX_TONES),
        ("burst_cycles", f64),
        ("n_elements", i32), ("pad1", i32),
        ("element_of_cell", vp), ("element_phase", vp), ("element_amp", vp),
    ]


class WesterveltParams(C.Structure):
    _fields_ = [
        ("precision", i32), ("energy_mode", i32),
        ("n_steps", i64), ("t0", f64), ("t_src", vp),
        ("peak_start", i64), ("peak_end", i64),
        ("energy_start", i64), ("energy_end", i64),
        ("dft_start", i64), ("dft_len", i64),
        ("n_dft", i32), ("dft_z_lo", i32), ("dft_z_hi", i32), ("q_mode", i32),
        ("dft_freq", f64 * BD_MAX_DFT),
        ("q_iz_split", i32), ("q_n_harm", i32),
        ("q_freq", f64),
        ("check_every", i32), ("fault_at_step", i32),
        ("blowup_limit", f64),
        ("graph_chunk", i32), ("tile_variant", i32),
        ("relax_scheme", i32), ("pad1", i32),
    ]


class WesterveltOutputs(C.Structure):
    _fields_ = [
        ("p_final", vp), ("peak", vp), ("energy", vp),
        ("dft_re", vp), ("dft_im", vp), ("Q", vp),
        ("elapsed_ms", f64), ("steps_done", i64), ("tile_variant", i32), ("pad0", i32),
    ]


class FocalLoss(C.Structure):
    _fields_ = [
        ("focus_ix", i32), ("focus_iy", i32), ("focus_iz", i32),
        ("focal_radius", i32), ("side_radius", i32), ("checkpoint_every", i32),
        ("side_weight", f64),
        ("window_start", i64), ("window_end", i64),
    ]


class ThermalMaterial(C.Structure):
    _fields_ = [
        ("rho", f64), ("c_t", f64), ("k_t", f64), ("perfusion", f64),
        ("T_art", f64), ("T_init", f64),
    ]


class Thermal(C.Structure):
    _fields_ = [
        ("nx", i32), ("ny", i32), ("nz", i32), ("precision", i32),
        ("dx", f64), ("dz", f64), ("dt", f64), ("T_ref", f64),
        ("n_materials", i32), ("dose_init", i32),
        ("mat", ThermalMaterial * BD_MAX_MATERIALS),
        ("plane_material", vp), ("material_map", vp),
        ("T_start", vp), ("dose_start", vp),
        ("plain_launches", i32), ("pad1", i32),
    ]


class Trajectory(C.Structure):
    _fields_ = [
        ("kind", i32), ("n_legs", i32),
        ("speed", f64), ("scale", f64), ("speed_init", f64), ("t_acc", f64),
        ("dxy", f64), ("dt", f64),
        ("n_spots", i32), ("pad0", i32),
        ("spot_sx", vp), ("spot_sy", vp), ("spot_steps", vp),
    ]


class HeatOutputs(C.Structure):
    _fields_ = [
        ("T_final", vp), ("dose", vp), ("snapshots", vp), ("snapshot_legs", vp),
        ("n_snap", i32), ("pad0", i32),
        ("elapsed_ms", f64), ("steps_done", i64),
    ]


class GilmoreMedium(C.Structure):
    _fields_ = [(k, f64) for k in ("rho", "P0", "S2", "mu4", "G4_3", "C_inf", "lambda_", "n", "B", "gamma")]


class Bubble(C.Structure):
    _fields_ = [
        ("R0", f64), ("n_tones", i32), ("pad0", i32),
        ("f", f64 * BD_MAX_BUBBLE_TONES), ("a", f64 * BD_MAX_BUBBLE_TONES),
        ("phi", f64 * BD_MAX_BUBBLE_TONES),
    ]


class OdeParams(C.Structure):
    _fields_ = [
        ("t_end", f64), ("h0", f64), ("atol", f64), ("rtol", f64), ("fac_max", f64),
        ("max_steps", i64), ("stop_at_threshold", i32), ("ref_arith", i32),
        ("schedule", i32), ("pad0", i32),
    ]


class BubbleResult(C.Structure):
    _fields_ = [
        ("R", f64), ("Rdot", f64), ("tau", f64), ("q", f64), ("t", f64),
        ("R_max", f64), ("R_min", f64), ("t_threshold", f64),
        ("n_accept", i64), ("n_reject", i64),
        ("status", i32), ("threshold", i32),
    ]


ALL_STRUCTS = {
    "bd_grid": Grid, "bd_material": Material, "bd_medium": Medium, "bd_source": Source,
    "bd_westervelt_params": WesterveltParams, "bd_westervelt_outputs": WesterveltOutputs,
    "bd_focal_loss": FocalLoss, "bd_thermal_material": ThermalMaterial, "bd_thermal": Thermal,
    "bd_trajectory": Trajectory, "bd_heat_outputs": HeatOutputs,
    "bd_gilmore_medium": GilmoreMedium, "bd_bubble": Bubble, "bd_ode_params": OdeParams,
    "bd_bubble_result": BubbleResult,
}


def ptr(a):
    """Address of a numpy array (or None) as a c_void_p value."""
    if a is None:
        return None
    return a.ctypes.data
