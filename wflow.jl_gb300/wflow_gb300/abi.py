"""ctypes mirror of include/wflow_gb300.h and loading of the in-tree shared libraries.

The product library (`_build/libwflow_gb300.so`, CUDA kernels + C ABI) and the host-only
synthetic-input library (`_build/libwflow_synth.so`) are built in-tree by
`wflow_gb300.build` and loaded from there; nothing is installed into site-packages.
"""

import ctypes as C
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent          # .../wflow.jl_gb300
REPO_ROOT = PKG_ROOT.parent
BUILD_DIR = PKG_ROOT / "_build"
LIB_PATH = BUILD_DIR / "libwflow_gb300.so"
SYNTH_LIB_PATH = BUILD_DIR / "libwflow_synth.so"
HEADER = REPO_ROOT / "include" / "wflow_gb300.h"

WF_MAX_LAYERS = 8

# WfStatus
WF_OK = 0
WF_STATIC_SCRATCH_BYTES = 16 * 1024 * 1024  # static scratch of wf_step_static
WF_ERR_INVALID = -1
WF_ERR_CUDA = -2
WF_ERR_CYCLE = -3
WF_ERR_NAN = -4
WF_ERR_SPIN = -5
WF_ERR_UNSUPPORTED = -6
WF_ERR_NOMEM = -7
WF_ERR_STATE = -8

WF_FORM_FP64 = 0
WF_FORM_SPLIT = 1
WF_KV_EXPONENTIAL = 0
WF_KV_EXPONENTIAL_CONSTANT = 1

_i32, _i64, _dbl = C.c_int32, C.c_int64, C.c_double
_pd, _pi32 = C.POINTER(C.c_double), C.POINTER(C.c_int32)
_pf = C.POINTER(C.c_float)


class WfConfig(C.Structure):
    _fields_ = [
        ("dt", _dbl),
        ("n_soil_layer_thickness", _i32),
        ("snow", _i32),
        ("soil_layer_thickness", _dbl * (WF_MAX_LAYERS - 1)),
        ("soil_infiltration_reduction", _i32),
        ("water_mass_balance", _i32),
        ("adaptive_timestep", _i32),
        ("kv_profile", _i32),
        ("land_dt_fixed", _dbl),
        ("river_dt_fixed", _dbl),
        ("subsurface_dt_fixed", _dbl),
        ("subsurface_alpha", _dbl),
        ("form", _i32),
        ("n_members", _i32),
        ("per_member_soil", _i32),
        ("snow_gravitational_transport", _i32),
        ("glacier", _i32),
        ("reserved", _i32 * 5),
    ]


DOMAIN_LAND_ARRAYS = ["area", "flow_width", "flow_length", "surface_flow_width", "slope",
                      "flow_fraction_to_river", "river_fraction", "water_fraction", "elevation",
                      "land_manning_n"]
DOMAIN_RIVER_ARRAYS = ["river_width", "river_length", "river_slope", "river_manning_n",
                       "river_bankfull_depth", "river_external_inflow"]


class WfDomain(C.Structure):
    _fields_ = ([("n_land", _i64), ("land_downstream", _pi32)]
                + [(k, _pd) for k in DOMAIN_LAND_ARRAYS]
                + [("n_river", _i64), ("river_land_index", _pi32), ("river_downstream", _pi32)]
                + [(k, _pd) for k in DOMAIN_RIVER_ARRAYS])


PARAM_FIELDS = [
    "canopy_gap_fraction", "maximum_canopy_storage", "crop_coefficient", "rooting_depth",
    "evaporation_to_precipitation_ratio",
    "degree_day_factor", "temperature_threshold_snowfall", "temperature_interval_snowfall",
    "temperature_threshold_melt", "water_holding_capacity",
    "theta_s", "theta_r", "kv_0", "f", "soil_thickness", "air_entry_pressure",
    "h1", "h2", "h3_high", "h3_low", "h4", "alpha_h1",
    "infiltration_capacity_compacted_soil", "compacted_soil_area_fraction",
    "wet_root_distribution_parameter", "cap_hmax", "cap_n", "maximum_leakage", "w_soil", "cf_soil",
    "z_exp", "brooks_corey_exponent", "kv_factor", "horizontal_to_vertical_ratio",
    "glacier_fraction", "glacier_temperature_threshold_melt", "glacier_degree_day_factor",
    "glacier_snow_to_ice_fraction", "glacier_initial_store",
]


class WfParams(C.Structure):
    _fields_ = [(k, _pd) for k in PARAM_FIELDS]


class WfMetrics(C.Structure):
    _fields_ = [
        ("steps", _i64), ("cell_steps", _i64), ("substeps_land", _i64), ("substeps_river", _i64),
        ("substeps_subsurface", _i64), ("kernel_launches", _i64), ("step_ms_total", _dbl),
        ("max_abs_balance_error", _dbl), ("device_status", _i32), ("n_chains_land", _i32),
        ("n_chains_river", _i32), ("max_chain_land", _i32), ("max_chain_river", _i32),
        ("padding_slots_land", _i32),
    ]


# WfReservoirOutflow
WF_RES_RATING_CURVE = 1
WF_RES_FREE_WEIR = 2
WF_RES_MODIFIED_PULS = 3
WF_RES_SIMPLE = 4
RESERVOIR_PARAMS = ["area", "waterlevel", "maximum_storage", "threshold", "rating_curve_coefficient",
                    "rating_curve_exponent", "maximum_release", "demand", "target_minimum_fraction",
                    "target_full_fraction"]


class WfReservoirs(C.Structure):
    _fields_ = ([("n", _i64), ("river_index", _pi32), ("outflow_curve_type", _pi32)]
                + [(k, _pd) for k in RESERVOIR_PARAMS])


WF_RES_PROFILE_LINEAR = 1
WF_RES_PROFILE_INTERPOLATION = 2


class WfReservoirTables(C.Structure):
    """The reservoirs' S-H and H-Q tables and links (include/wflow_gb300.h)."""
    _fields_ = [("storage_curve_type", _pi32), ("sh_offset", C.POINTER(_i64)), ("sh_h", _pd), ("sh_s", _pd),
                ("hq_offset", C.POINTER(_i64)), ("hq_h", _pd), ("hq_q", _pd), ("lower_reservoir", _pi32)]


class WfTuning(C.Structure):
    _fields_ = [("vertical_block", _i32), ("routing_warps", _i32), ("routing_blocks_per_sm", _i32),
                ("use_graph", _i32), ("reserved", _i32 * 8)]


# WfField ids (enum WfField in the header)
_LAND_FIELDS = [
    "CANOPY_STORAGE", "SNOW_STORAGE", "SNOW_WATER", "SOIL_SURFACE_TEMPERATURE", "SATURATED_WATER_DEPTH",
    "UNSATURATED_LAYER_DEPTH", "SSF_Q", "LAND_Q", "LAND_H", "WATER_TABLE_DEPTH", "UNSATURATED_STORE_DEPTH",
    "TOTAL_SOIL_WATER_STORAGE", "RECHARGE", "NET_RUNOFF", "RUNOFF", "ACTUAL_EVAPOTRANSPIRATION",
    "ACTUAL_LEAKAGE", "TRANSPIRATION", "SOIL_EVAPORATION", "ACTUAL_INFILTRATION",
    "EXFILTRATION_SATURATED_WATER", "INTERCEPTION_RATE", "SNOW_WATER_EQUIVALENT", "NET_RUNOFF_RIVER",
    "SSF_Q_AVERAGE", "SSF_WATER_TABLE_DEPTH", "SSF_STORAGE", "SSF_TO_RIVER_AVERAGE", "LAND_Q_AVERAGE",
    "LAND_STORAGE", "LAND_TO_RIVER_AVERAGE", "LAND_INWATER", "TOTAL_STORAGE", "BALANCE_LAND_ERROR",
    "BALANCE_LAND_RELATIVE_ERROR", "BALANCE_OVERLAND_ERROR", "BALANCE_OVERLAND_RELATIVE_ERROR",
    "BALANCE_SUBSURFACE_ERROR", "BALANCE_SUBSURFACE_RELATIVE_ERROR", "VOLUMETRIC_WATER_CONTENT",
    "LAND_QIN_AVERAGE", "GLACIER_STORE", "GLACIER_MELT", "SNOW_IN", "SNOW_OUT",
]
_RIVER_FIELDS = ["RIVER_Q", "RIVER_H", "RIVER_STORAGE", "RIVER_Q_AVERAGE", "RIVER_QIN_AVERAGE",
                 "RIVER_INWATER", "BALANCE_RIVER_ERROR", "BALANCE_RIVER_RELATIVE_ERROR"]
_RESERVOIR_FIELDS = ["RESERVOIR_STORAGE", "RESERVOIR_WATERLEVEL", "RESERVOIR_OUTFLOW", "RESERVOIR_OUTFLOW_AVERAGE",
                     "RESERVOIR_INFLOW_AVERAGE", "RESERVOIR_ACTEVAP_AVERAGE", "RESERVOIR_ABSTRACTION_AVERAGE",
                     "RESERVOIR_INFLOW_OVERLAND", "RESERVOIR_INFLOW_SUBSURFACE", "RESERVOIR_PRECIPITATION",
                     "RESERVOIR_EVAPORATION", "RESERVOIR_EXTERNAL_INFLOW", "RESERVOIR_OUTFLOW_OBS",
                     "BALANCE_RESERVOIR_ERROR", "BALANCE_RESERVOIR_RELATIVE_ERROR"]
FIELD = {name: i for i, name in enumerate(_LAND_FIELDS)}
FIELD.update({name: 100 + i for i, name in enumerate(_RIVER_FIELDS)})
FIELD.update({name: 200 + i for i, name in enumerate(_RESERVOIR_FIELDS)})
RESERVOIR_INPUT_FIELDS = ["RESERVOIR_PRECIPITATION", "RESERVOIR_EVAPORATION", "RESERVOIR_EXTERNAL_INFLOW",
                          "RESERVOIR_OUTFLOW_OBS"]
LAYERED_FIELDS = {"UNSATURATED_LAYER_DEPTH", "VOLUMETRIC_WATER_CONTENT"}
STATE_FIELDS = ["CANOPY_STORAGE", "SNOW_STORAGE", "SNOW_WATER", "SOIL_SURFACE_TEMPERATURE",
                "SATURATED_WATER_DEPTH", "UNSATURATED_LAYER_DEPTH", "SSF_Q", "LAND_Q", "LAND_H",
                "RIVER_Q", "RIVER_H"]


def is_river_field(fid):
    return 100 <= fid < 200


def is_reservoir_field(fid):
    return fid >= 200


def as_ptr(arr, ctype=C.c_double):
    """Pointer to a contiguous numpy array (None for None)."""
    if arr is None:
        return None
    return arr.ctypes.data_as(C.POINTER(ctype))


_lib = None
_synth = None


def load_library(required=True):
    """Load the in-tree CUDA library. Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            if required:
                raise RuntimeError(f"CUDA library not built: {LIB_PATH} (run __graft_entry__.build())")
            return None
        lib = C.CDLL(str(LIB_PATH))
        _declare(lib)
        _lib = lib
    return _lib


def load_synth():
    global _synth
    if _synth is None:
        if not SYNTH_LIB_PATH.exists():
            from . import build
            build.build_synth()
        lib = C.CDLL(str(SYNTH_LIB_PATH))
        lib.wf_synth_dem_d8.restype = _i32
        lib.wf_synth_dem_d8.argtypes = [_i32, _i32, C.c_uint64, _dbl, _dbl, _dbl, _dbl, _dbl, _pd,
                                        C.POINTER(C.c_uint8), _pi32, _pd, C.POINTER(C.c_int64), _pd, _pd]
        _synth = lib
    return _synth


def _declare(lib):
    H = C.c_void_p
    sig = {
        "wf_abi_version": (_i32, []),
        "wf_create": (_i32, [C.POINTER(WfConfig), C.POINTER(WfDomain), C.POINTER(WfParams), _i32,
                             C.POINTER(H)]),
        "wf_destroy": (None, [H]),
        "wf_last_error": (C.c_char_p, [H]),
        "wf_set_forcing": (_i32, [H, _pd, _pd, _pd, _i64]),
        "wf_set_forcing_async": (_i32, [H, _pd, _pd, _pd, _i64]),
        "wf_set_forcing_f32": (_i32, [H, _pf, _pf, _pf, _i64]),
        "wf_set_forcing_async_f32": (_i32, [H, _pf, _pf, _pf, _i64]),
        "wf_set_forcing_counts_f32": (_i32, [H, _pf, _i64, _pf, _i64, _pf, _i64]),
        "wf_set_forcing_counts_async_f32": (_i32, [H, _pf, _i64, _pf, _i64, _pf, _i64]),
        "wf_set_forcing_device_slots": (_i32, [H, C.c_void_p, C.c_void_p, C.c_void_p]),
        "wf_step": (_i32, [H]),
        "wf_step_async": (_i32, [H]),
        "wf_step_static": (_i32, [H]),
        "wf_synchronize": (_i32, [H]),
        "wf_get_field": (_i32, [H, _i32, _i32, _pd, _i64, _i64]),
        "wf_set_field": (_i32, [H, _i32, _i32, _pd, _i64, _i64]),
        "wf_get_outlets": (_i32, [H, _i32, _pd, _i64, C.POINTER(_i64)]),
        "wf_get_state": (_i32, [H, C.c_void_p, C.POINTER(C.c_size_t)]),
        "wf_set_state": (_i32, [H, C.c_void_p, C.c_size_t]),
        "wf_get_metrics": (_i32, [H, C.POINTER(WfMetrics)]),
        "wf_reset_metrics": (_i32, [H]),
        "wf_set_tuning": (_i32, [H, C.POINTER(WfTuning)]),
        "wf_get_slot_order": (_i32, [H, C.POINTER(_i64), _i64, C.POINTER(_i64)]),
        "wf_get_sizes": (_i32, [H, C.POINTER(_i64), C.POINTER(_i64), C.POINTER(_i64), _pi32, _pi32]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    extra = {
        "wf_get_stream": (_i32, [H, C.POINTER(C.c_void_p)]),
        "wf_get_kernel_times": (_i32, [H, _pd, C.POINTER(_i64)]),
        "wf_struct_size": (_i32, [_i32]),
        "wf_plan_routing": (_i32, [_i64, _pi32, _i32, C.POINTER(_i64), C.POINTER(_i64), _pi32, _pi32]),
        "wf_plan_routing_hinted": (_i32, [_i64, _pi32, _i32, C.POINTER(_i64), C.POINTER(_i64), C.POINTER(_i64),
                                          _pi32, _pi32]),
        "wf_create_with_reservoirs": (_i32, [C.POINTER(WfConfig), C.POINTER(WfDomain), C.POINTER(WfParams),
                                             C.POINTER(WfReservoirs), _i32, C.POINTER(H)]),
        "wf_create_with_reservoir_tables": (_i32, [C.POINTER(WfConfig), C.POINTER(WfDomain), C.POINTER(WfParams),
                                                   C.POINTER(WfReservoirs), C.POINTER(WfReservoirTables), _i32,
                                                   C.POINTER(H)]),
        "wf_set_rating_curve_day": (_i32, [H, _i32]),
        "wf_get_reservoir_count": (_i32, [H, C.POINTER(_i64)]),
        "wf_get_substep_signature": (_i32, [H, _i32, _pd, _i32]),
    }
    for name, (res, args) in extra.items():
        if hasattr(lib, name):
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args


def header_symbols(header="wflow_gb300.h"):
    """Entry points declared in an include/ header (names of functions starting with wf_)."""
    import re
    names = set()
    for h in [REPO_ROOT / "include" / header]:
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(wf_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def check(status, handle=None, what=""):
    if status != WF_OK:
        lib = load_library()
        msg = lib.wf_last_error(handle)
        raise RuntimeError(f"{what} failed with status {status}: {msg.decode() if msg else ''}")
