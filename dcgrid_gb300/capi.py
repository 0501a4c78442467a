"""ctypes mirrors of the C ABI structs declared in include/dcg.h.

The layouts here must match include/dcg.h field for field; tests check the
sizes against the library's own sizeof values.
"""
import ctypes as C

DCG_OK = 0
DCG_E_INVALID = 1
DCG_E_BUDGET = 2
DCG_E_HASH_FULL = 3
DCG_E_CUDA = 4
DCG_E_TIMEOUT = 5
DCG_E_NAN = 6
DCG_E_NOT_FOUND = 7
DCG_E_DEVICE = 8

STATUS_NAMES = {
    0: "DCG_OK", 1: "DCG_E_INVALID", 2: "DCG_E_BUDGET", 3: "DCG_E_HASH_FULL",
    4: "DCG_E_CUDA", 5: "DCG_E_TIMEOUT", 6: "DCG_E_NAN", 7: "DCG_E_NOT_FOUND",
    8: "DCG_E_DEVICE",
}

MODE_ADAPTIVE = 0
MODE_UNIFORM = 1

SOLIDS_NONE = 0
SOLIDS_SPHERE = 1
SOLIDS_TERRAIN = 2
SOLIDS_BOTH = 3

REFINE_GEOMETRIC = 0
REFINE_FIELDS = 1

PRECISION_FP32 = 0
PRECISION_MIXED = 1       # BF16 scalars
PRECISION_MIXED_FP16 = 2  # FP16 scalars

FIELD_DENSITY = 0
FIELD_VEL_X = 1
FIELD_VEL_Y = 2
FIELD_VEL_Z = 3
FIELD_FLUIDITY = 4
FIELD_PRESSURE = 5
FIELD_PRESSURE_TMP = 6
FIELD_DIVERGENCE = 7
FIELD_TEMPERATURE = 8
FIELD_VAPOR = 9
FIELD_NAMES = {
    "density": 0, "vel_x": 1, "vel_y": 2, "vel_z": 3, "fluidity": 4,
    "pressure": 5, "pressure_tmp": 6, "divergence": 7, "temperature": 8,
    "vapor": 9,
}

HOST = 0
DEVICE = 1

DEVERR_BUDGET = 1
DEVERR_LOOKUP = 2
DEVERR_NAN = 4
DEVERR_TIMEOUT = 8


class DcgParams(C.Structure):
    _fields_ = [
        ("gx", C.c_int32), ("gy", C.c_int32), ("gz", C.c_int32),
        ("levels", C.c_int32),
        ("max_blocks", C.c_int64),
        ("dt", C.c_float), ("dx", C.c_float),
        ("inlet_enabled", C.c_int32),
        ("velocity_emission_rate", C.c_float),
        ("density_emission_rate", C.c_float),
        ("emission_radius", C.c_float),
        ("solids", C.c_int32),
        ("sphere_radius_world", C.c_float),
        ("jacobi_iters", C.c_int32),
        ("init_adapt_passes", C.c_int32),
        ("refine_criterion", C.c_int32),
        ("refine_threshold", C.c_float),
        ("vort_threshold", C.c_float),
        ("grad_threshold", C.c_float),
        ("ref_compat", C.c_int32),
        ("n_scalars", C.c_int32),
        ("buoy_alpha", C.c_float), ("buoy_beta", C.c_float), ("t_ambient", C.c_float),
        ("src_enabled", C.c_int32),
        ("src_center", C.c_float * 3),
        ("src_radius", C.c_float),
        ("src_density", C.c_float), ("src_temperature", C.c_float), ("src_vapor", C.c_float),
        ("wind_enabled", C.c_int32),
        ("wind", C.c_float * 3),
        ("terrain_amplitude", C.c_float),
        ("terrain_base_height", C.c_float),
        ("terrain_frequency", C.c_float),
        ("terrain_persistence", C.c_float),
        ("terrain_octaves", C.c_int32),
        ("terrain_seed", C.c_uint32),
        ("precision", C.c_int32),
        ("emission_n", C.c_int32),
        ("emission_band", C.c_float),
        ("src_jitter", C.c_float), ("src_jitter_seed", C.c_uint32),
        ("defect_passes", C.c_int32),
        ("reserved", C.c_int32 * 3),
    ]


class DcgInfo(C.Structure):
    _fields_ = [
        ("mode", C.c_int32), ("levels", C.c_int32), ("sparse_levels", C.c_int32),
        ("n_scalars", C.c_int32),
        ("max_blocks", C.c_int64), ("num_cells", C.c_int64),
        ("full_blocks", C.c_int64 * 16), ("budget", C.c_int64 * 16),
        ("offset", C.c_int64 * 16), ("device_bytes", C.c_int64),
    ]


class DcgStats(C.Structure):
    _fields_ = [
        ("load", C.c_int64 * 16), ("leaf_cells", C.c_int64 * 16),
        ("active_cells", C.c_int64), ("moved_blocks", C.c_int64),
        ("refined_subblocks", C.c_int64), ("steps", C.c_int64),
        ("residual", C.c_double), ("mass", C.c_double),
        ("device_error", C.c_uint32), ("pad", C.c_uint32),
        ("defect_rel_residual", C.c_double * 2),
    ]


class DcgTuning(C.Structure):
    _fields_ = [
        ("tile", C.c_int32 * 4), ("solve_cache", C.c_int32),
        ("solve_ctas_per_sm", C.c_int32), ("solve_barrier", C.c_int32), ("persistent", C.c_int32),
        ("round_ctas_per_sm", C.c_int16 * 4), ("round_cache", C.c_int8 * 4), ("round_barrier", C.c_int8 * 4), ("solve_ms", C.c_float), ("cells_ms", C.c_float * 4),
    ]


RENDER_FLUID, RENDER_DENSITY, RENDER_VELOCITY, RENDER_FLUIDITY, RENDER_RESOLUTION = range(5)


class DcgRenderParams(C.Structure):
    _fields_ = [
        ("width", C.c_int32), ("height", C.c_int32), ("eye", C.c_float * 3), ("eye_dir", C.c_float * 3),
        ("fov", C.c_float), ("sun_dir", C.c_float * 3), ("aa_samples", C.c_int32), ("channel", C.c_int32),
        ("shadows", C.c_int32), ("solids", C.c_int32), ("precise", C.c_int32), ("ambient", C.c_float),
        ("smoke_color", C.c_float * 3), ("scene_color", C.c_float * 3), ("floor_color", C.c_float * 3),
        ("reserved", C.c_int32 * 4),
    ]


def tuning_to_dict(t):
    return {"tile": list(t.tile), "solve_cache": t.solve_cache, "solve_ctas_per_sm": t.solve_ctas_per_sm,
            "solve_barrier": t.solve_barrier, "persistent": t.persistent, "solve_ms": t.solve_ms,
            "cells_ms": list(t.cells_ms), "round_ctas_per_sm": list(t.round_ctas_per_sm),
            "round_cache": list(t.round_cache), "round_barrier": list(t.round_barrier)}


def tuning_from_dict(d):
    """Inverse of tuning_to_dict (missing keys stay zero)."""
    t = DcgTuning()
    for k, v in d.items():
        if not hasattr(t, k):
            continue
        if isinstance(v, (list, tuple)):
            arr = getattr(t, k)
            for i, x in enumerate(v):
                arr[i] = x
        else:
            setattr(t, k, v)
    return t


def default_params(gx, gy, gz, max_blocks):
    """The reference's SimParams defaults (src/data/sim_params.cpp:4-34) and its
    hard-wired solver/adaptation constants; mirrors dcg_default_params()."""
    p = DcgParams()
    p.gx, p.gy, p.gz = gx, gy, gz
    p.levels = 0
    p.max_blocks = max_blocks
    p.dt = 3.0
    p.dx = 10000.0 / gx
    p.inlet_enabled = 1
    p.velocity_emission_rate = 150.0
    p.density_emission_rate = 0.002
    p.emission_radius = 750.0
    p.solids = SOLIDS_NONE
    p.sphere_radius_world = 2000.0
    p.jacobi_iters = 10
    p.init_adapt_passes = 5
    p.refine_criterion = REFINE_GEOMETRIC
    p.refine_threshold = 1e-4
    p.vort_threshold = 0.5
    p.grad_threshold = 0.05
    p.ref_compat = 1
    p.n_scalars = 1
    p.buoy_alpha = 0.0
    p.buoy_beta = 0.0
    p.t_ambient = 0.0
    p.src_enabled = 0
    p.src_radius = 0.0
    p.src_density = 0.0
    p.src_temperature = 0.0
    p.src_vapor = 0.0
    p.wind_enabled = 0
    p.terrain_amplitude = 0.0
    p.terrain_base_height = 0.0
    p.terrain_frequency = 1.0 / 64.0
    p.terrain_persistence = 0.5
    p.terrain_octaves = 5
    p.terrain_seed = 0
    p.precision = PRECISION_FP32
    return p


def params_to_dict(p):
    out = {}
    for name, _ in DcgParams._fields_:
        val = getattr(p, name)
        if hasattr(val, "__len__"):
            val = list(val)
        out[name] = val
    return out


def params_from_dict(d):
    """Inverse of params_to_dict. Dicts written before src_jitter,
    src_jitter_seed and defect_passes took three of the six reserved words
    carry more (zero) reserved entries; the extra zeros are dropped."""
    p = DcgParams()
    for k, v in d.items():
        if isinstance(v, (list, tuple)):
            arr = getattr(p, k)
            if k == "reserved" and len(v) > len(arr):
                if any(v[len(arr):]):
                    raise ValueError("reserved parameter words must be zero")
                v = v[:len(arr)]
            for i, x in enumerate(v):
                arr[i] = x
        else:
            setattr(p, k, v)
    return p
