/*
 * wflow_gb300.h -- C ABI of the GB300 (sm_103a) SBM + kinematic-wave step library.
 *
 * The library replaces the per-timestep hot path of Wflow.jl's `sbm` model:
 *   update_model!(model)          Wflow/src/sbm_model.jl:60-92
 *   compute_mass_balance!(model)  Wflow/src/mass_balance.jl:541-545
 * which Wflow calls through the `update_func` seam of
 *   run_timestep!(model; update_func = update_model!)  Wflow/src/Wflow.jl:311-322
 * A Julia caller binds these entry points with `ccall`; every argument is a plain pointer,
 * size or POD struct. All device memory, the CUDA stream and the
 * captured CUDA graph of a step belong to the handle. Input arrays are copied at call time
 * and never retained.
 *
 * Units are SI inside the path (m, s, K, m s-1, m3 s-1), as after Wflow's to_SI
 * (Wflow/src/units.jl:271). Cell order in every array argument is the reference's land
 * order (`domain.land.network.indices`), river order is `domain.river.network.indices`.
 *
 * Errors: every entry point returns WfStatus (0 = ok, negative = error class) and
 * wf_last_error() gives a message; device-side problems (a bounded spin-wait that ran out,
 * non-finite results) are raised through a device status word read after each step.
 * Nothing traps or aborts.
 */
#ifndef WFLOW_GB300_H
#define WFLOW_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WF_ABI_VERSION 3
#define WF_MAX_LAYERS 8

typedef enum WfStatus {
    WF_OK = 0,
    WF_ERR_INVALID = -1,     /* bad argument or inconsistent sizes */
    WF_ERR_CUDA = -2,        /* a CUDA runtime call failed */
    WF_ERR_CYCLE = -3,       /* the drainage graph has a cycle (routing/utils.jl:26-31) */
    WF_ERR_NAN = -4,         /* non-finite input where the reference requires a value */
    WF_ERR_SPIN = -5,        /* a routing wavefront wait ran out of its spin budget */
    WF_ERR_UNSUPPORTED = -6, /* option outside the supported path */
    WF_ERR_NOMEM = -7,       /* device allocation failed */
    WF_ERR_STATE = -8        /* state blob of the wrong size or version */
} WfStatus;

/* Arithmetic form of the step. */
typedef enum WfForm {
    WF_FORM_FP64 = 0,  /* plain FP64 drop-in: every operation in FP64 */
    WF_FORM_SPLIT = 1  /* FP32 bulk fluxes; FP64 Newton solves and storage/balance state */
} WfForm;

/* Vertical saturated hydraulic conductivity profile (Wflow/src/soil/soil.jl:213-244). */
typedef enum WfKvProfile { WF_KV_EXPONENTIAL = 0, WF_KV_EXPONENTIAL_CONSTANT = 1 } WfKvProfile;

/* Model settings, mirroring Wflow's [model] and [time] TOML sections
 * (Wflow/src/config_structure.jl:62-100). */
typedef struct WfConfig {
    double dt;                                        /* time.timestepsecs [s] */
    int32_t n_soil_layer_thickness;                   /* length of soil_layer__thickness */
    int32_t snow;                                     /* snow__flag */
    double soil_layer_thickness[WF_MAX_LAYERS - 1];   /* soil_layer__thickness [m] */
    int32_t soil_infiltration_reduction;              /* soil_infiltration_reduction__flag */
    int32_t water_mass_balance;                       /* water_mass_balance__flag */
    int32_t adaptive_timestep;                        /* kinematic_wave__adaptive_time_step_flag */
    int32_t kv_profile;                               /* WfKvProfile */
    double land_dt_fixed;                             /* land_kinematic_wave__time_step [s] */
    double river_dt_fixed;                            /* river_kinematic_wave__time_step [s] */
    double subsurface_dt_fixed;                       /* subsurface_kinematic_wave__time_step [s] */
    double subsurface_alpha;                          /* subsurface_kinematic_wave__alpha_coefficient */
    int32_t form;                                     /* WfForm */
    int32_t n_members;                                /* ensemble members sharing the domain (>= 1) */
    int32_t per_member_soil;                          /* kv_0 and f given per member (n_land*n_members) */
    int32_t snow_gravitational_transport;             /* snow_gravitational_transport__flag (with snow) */
    int32_t glacier;                                  /* glacier__flag (with snow, sbm.jl:36-53) */
    int32_t reserved[5];
} WfConfig;

/* Drainage network and shared geometry (Wflow/src/domain.jl:1-45, network.jl:47-258).
 * The graphs are given by one downstream index per node (Graphs.outneighbors of the D8
 * flow graph, routing/utils.jl:6-33): -1 marks a pit. */
typedef struct WfDomain {
    int64_t n_land;
    const int32_t* land_downstream;         /* [n_land] */
    const double* area;                     /* [m2] */
    const double* flow_width;               /* [m] */
    const double* flow_length;              /* [m] */
    const double* surface_flow_width;       /* [m] */
    const double* slope;                    /* [-] (already clamped >= 1e-5) */
    const double* flow_fraction_to_river;   /* [-] */
    const double* river_fraction;           /* [-] */
    const double* water_fraction;           /* [-] */
    const double* elevation;                /* land_surface__elevation [m] */
    const double* land_manning_n;           /* land_surface_water_flow__manning_n_parameter */
    int64_t n_river;
    const int32_t* river_land_index;        /* [n_river] land index of each river cell */
    const int32_t* river_downstream;        /* [n_river], -1 for a pit */
    const double* river_width;              /* river__width [m] */
    const double* river_length;             /* river__length [m] */
    const double* river_slope;              /* river__slope [-] (already clamped >= 1e-5) */
    const double* river_manning_n;          /* river_water_flow__manning_n_parameter */
    const double* river_bankfull_depth;     /* river_bank_water__depth [m] */
    const double* river_external_inflow;    /* river_water__external_inflow_volume_flow_rate [m3 s-1] */
} WfDomain;

/* Static SBM parameters as Wflow reads them from the static maps, in SI units.
 * Layered arrays are cell-major [i * n_layers + k] like Vector{SVector{N}} in the reference.
 * Derived parameters (layer thickness, theta_fc, root fraction, soil water capacity,
 * infiltration capacity of the soil, kh_0, specific yield, Manning alpha) are computed by
 * the library exactly as the reference's initialisation does. */
typedef struct WfParams {
    /* vegetation (vegetation/parameters.jl:1-91, canopy.jl) */
    const double* canopy_gap_fraction;
    const double* maximum_canopy_storage;              /* [m] */
    const double* crop_coefficient;
    const double* rooting_depth;                       /* [m] */
    const double* evaporation_to_precipitation_ratio;  /* Gash only (dt >= 23 h) */
    /* snow (snow/snow.jl:175-224) */
    const double* degree_day_factor;                   /* [m K-1 s-1] */
    const double* temperature_threshold_snowfall;      /* [K] */
    const double* temperature_interval_snowfall;       /* [K] */
    const double* temperature_threshold_melt;          /* [K] */
    const double* water_holding_capacity;              /* [-] */
    /* soil (soil/soil.jl:319-617) */
    const double* theta_s;
    const double* theta_r;
    const double* kv_0;                                /* [m s-1]; n_land*n_members if per_member_soil */
    const double* f;                                   /* scale parameter [m-1]; idem */
    const double* soil_thickness;                      /* [m] */
    const double* air_entry_pressure;                  /* [m] */
    const double* h1;
    const double* h2;
    const double* h3_high;
    const double* h3_low;
    const double* h4;                                  /* Feddes heads [m] */
    const double* alpha_h1;
    const double* infiltration_capacity_compacted_soil; /* [m s-1] */
    const double* compacted_soil_area_fraction;
    const double* wet_root_distribution_parameter;     /* [m-1] */
    const double* cap_hmax;                            /* [m] */
    const double* cap_n;
    const double* maximum_leakage;                     /* [m s-1] */
    const double* w_soil;
    const double* cf_soil;
    const double* z_exp;                               /* [m], exponential_constant profile only */
    const double* brooks_corey_exponent;               /* [n_land * n_layers] */
    const double* kv_factor;                           /* [n_land * n_layers] */
    /* lateral subsurface (routing/subsurface/lateral_subsurface_flow.jl:87-132) */
    const double* horizontal_to_vertical_ratio;        /* KsatHorFrac [-] */
    /* HBV glacier (glacier/glacier.jl:58-98), read with the glacier flag; NULL takes the
     * reference's default (standard_name/standard_name_sbm.jl:70-108) */
    const double* glacier_fraction;                    /* glacier_surface__area_fraction [-] (0) */
    const double* glacier_temperature_threshold_melt;  /* [K] (273.15) */
    const double* glacier_degree_day_factor;           /* [m K-1 s-1] (3 mm degC-1 d-1) */
    const double* glacier_snow_to_ice_fraction;        /* [s-1] (0.001 d-1) */
    const double* glacier_initial_store;               /* glacier_ice__initial_leq_depth [m] (5.5) */
} WfParams;

/* Per-cell and per-river-cell variables exposed through get/set (BMI get_value/set_value,
 * Wflow/src/bmi.jl:208-248). Layered fields take a layer index. */
typedef enum WfField {
    /* land, states */
    WF_F_CANOPY_STORAGE = 0,
    WF_F_SNOW_STORAGE,
    WF_F_SNOW_WATER,
    WF_F_SOIL_SURFACE_TEMPERATURE,
    WF_F_SATURATED_WATER_DEPTH,
    WF_F_UNSATURATED_LAYER_DEPTH,   /* layered */
    WF_F_SSF_Q,
    WF_F_LAND_Q,
    WF_F_LAND_H,
    /* land, diagnostics of the last step */
    WF_F_WATER_TABLE_DEPTH,
    WF_F_UNSATURATED_STORE_DEPTH,
    WF_F_TOTAL_SOIL_WATER_STORAGE,
    WF_F_RECHARGE,
    WF_F_NET_RUNOFF,
    WF_F_RUNOFF,
    WF_F_ACTUAL_EVAPOTRANSPIRATION,
    WF_F_ACTUAL_LEAKAGE,
    WF_F_TRANSPIRATION,
    WF_F_SOIL_EVAPORATION,
    WF_F_ACTUAL_INFILTRATION,
    WF_F_EXFILTRATION_SATURATED_WATER,
    WF_F_INTERCEPTION_RATE,
    WF_F_SNOW_WATER_EQUIVALENT,
    WF_F_NET_RUNOFF_RIVER,
    WF_F_SSF_Q_AVERAGE,
    WF_F_SSF_WATER_TABLE_DEPTH,
    WF_F_SSF_STORAGE,
    WF_F_SSF_TO_RIVER_AVERAGE,
    WF_F_LAND_Q_AVERAGE,
    WF_F_LAND_STORAGE,
    WF_F_LAND_TO_RIVER_AVERAGE,
    WF_F_LAND_INWATER,
    WF_F_TOTAL_STORAGE,
    WF_F_BALANCE_LAND_ERROR,
    WF_F_BALANCE_LAND_RELATIVE_ERROR,
    WF_F_BALANCE_OVERLAND_ERROR,
    WF_F_BALANCE_OVERLAND_RELATIVE_ERROR,
    WF_F_BALANCE_SUBSURFACE_ERROR,
    WF_F_BALANCE_SUBSURFACE_RELATIVE_ERROR,
    WF_F_VOLUMETRIC_WATER_CONTENT,  /* layered */
    WF_F_LAND_QIN_AVERAGE,          /* overland inflow from upstream cells, step average [m3 s-1] */
    WF_F_GLACIER_STORE,             /* glacier_ice__leq_depth [m] (glacier flag) */
    WF_F_GLACIER_MELT,              /* glacier_ice__melt_volume_flux [m s-1] (glacier flag) */
    WF_F_SNOW_IN,                   /* snow moved in from upstream cells [m s-1] (transport flag) */
    WF_F_SNOW_OUT,                  /* snow moved on to the downstream cell [m s-1] (transport flag) */
    WF_F_LAND_END_,
    /* river */
    WF_F_RIVER_Q = 100,
    WF_F_RIVER_H,
    WF_F_RIVER_STORAGE,
    WF_F_RIVER_Q_AVERAGE,
    WF_F_RIVER_QIN_AVERAGE,
    WF_F_RIVER_INWATER,
    WF_F_BALANCE_RIVER_ERROR,
    WF_F_BALANCE_RIVER_RELATIVE_ERROR,
    WF_F_RIVER_END_,
    /* reservoirs (models created with wf_create_with_reservoirs), member-major over the
     * reservoir order of WfReservoirs; ReservoirVariables / ReservoirBC of reservoir.jl:202-297 */
    WF_F_RESERVOIR_STORAGE = 200,       /* state [m3] */
    WF_F_RESERVOIR_WATERLEVEL,          /* state [m] */
    WF_F_RESERVOIR_OUTFLOW,             /* [m3 s-1], last sub-step */
    WF_F_RESERVOIR_OUTFLOW_AVERAGE,     /* [m3 s-1] */
    WF_F_RESERVOIR_INFLOW_AVERAGE,      /* net inflow [m3 s-1] */
    WF_F_RESERVOIR_ACTEVAP_AVERAGE,     /* [m s-1], set by the water balance (mass_balance.jl:274) */
    WF_F_RESERVOIR_ABSTRACTION_AVERAGE, /* actual external abstraction [m3 s-1] */
    WF_F_RESERVOIR_INFLOW_OVERLAND,     /* [m3 s-1] */
    WF_F_RESERVOIR_INFLOW_SUBSURFACE,   /* [m3 s-1] */
    WF_F_RESERVOIR_PRECIPITATION,       /* input: mean over the reservoir area [m s-1] */
    WF_F_RESERVOIR_EVAPORATION,         /* input: mean potential evaporation [m s-1] */
    WF_F_RESERVOIR_EXTERNAL_INFLOW,     /* input [m3 s-1]; negative = abstraction */
    WF_F_RESERVOIR_OUTFLOW_OBS,         /* input [m3 s-1]; NaN = no observation */
    WF_F_BALANCE_RESERVOIR_ERROR,
    WF_F_BALANCE_RESERVOIR_RELATIVE_ERROR,
    WF_F_RESERVOIR_END_
} WfField;

/* Outflow functions of a reservoir (ReservoirOutflowType, Wflow/src/routing/surface/reservoir.jl). */
typedef enum WfReservoirOutflow {
    WF_RES_RATING_CURVE = 1,  /* Q = f(H) from the H-Q table of the day of year (reservoir.jl:455-479);
                               * needs WfReservoirTables */
    WF_RES_FREE_WEIR = 2,     /* Q = b (H - H0)^e, optionally linked to a lower reservoir (reservoir.jl:482-521) */
    WF_RES_MODIFIED_PULS = 3, /* Q = b (H - H0)^2 by the modified Puls approach (reservoir.jl:424-452) */
    WF_RES_SIMPLE = 4         /* simple reservoir (reservoir.jl:389-418) */
} WfReservoirOutflow;

/* Reservoirs at river cells (reservoir__flag; reservoir.jl:1-300, network.jl:296-357), with the
 * linear storage profile S = A H (storage_curve_type 1) unless WfReservoirTables gives an S-H
 * table (wf_create_with_reservoir_tables). The reservoir's outlet cell becomes a pit
 * of the land and river upstream lists (domain.jl:95-121): the outlet cell's overland and
 * subsurface discharge feed the reservoir (surface_kinwave.jl:771-802), its river discharge
 * enters the reservoir within the river sweep and the reservoir outflow is the inflow of the
 * downstream river cell (surface_kinwave.jl:441-489). Per-step inputs (precipitation and
 * evaporation over the reservoir area, external inflow, observed outflow) are set with
 * wf_set_field; the caller averages the forcing over the reservoir area and zeroes the land
 * forcing there, as Wflow's forcing reader does (io.jl:128-137). */
typedef struct WfReservoirs {
    int64_t n;                              /* number of reservoirs */
    const int32_t* river_index;             /* [n] river cell of each reservoir outlet */
    const int32_t* outflow_curve_type;      /* [n] WfReservoirOutflow */
    const double* area;                     /* reservoir_surface__area [m2] */
    const double* waterlevel;               /* initial reservoir_water_surface__elevation [m] */
    const double* maximum_storage;          /* reservoir_water__max_volume [m3] (NaN where unused) */
    const double* threshold;                /* reservoir_water_flow_threshold_level__elevation [m] */
    const double* rating_curve_coefficient; /* reservoir_water__rating_curve_coefficient */
    const double* rating_curve_exponent;    /* reservoir_water__rating_curve_exponent */
    const double* maximum_release;          /* reservoir_water_release_below_spillway__max_volume_flow_rate */
    const double* demand;                   /* reservoir_water_demand__required_downstream_volume_flow_rate */
    const double* target_minimum_fraction;  /* reservoir_water__target_min_volume_fraction */
    const double* target_full_fraction;     /* reservoir_water__target_full_volume_fraction */
} WfReservoirs;

/* Storage profiles of a reservoir (ReservoirProfileType, reservoir.jl:2). */
typedef enum WfReservoirProfile {
    WF_RES_PROFILE_LINEAR = 1,        /* S = A H */
    WF_RES_PROFILE_INTERPOLATION = 2  /* S = f(H) interpolated in the S-H table (reservoir.jl:306-320) */
} WfReservoirProfile;

/* The table inputs of reservoirs (ReservoirParameters, reservoir.jl:5-44; the CSV files
 * reservoir_sh_<id>.csv and reservoir_hq_<id>.csv read by read_sh_csv / read_hq_csv,
 * io.jl:1129-1147) and the links between reservoirs. Tables are concatenated over the
 * reservoirs in WfReservoirs order; reservoir k owns rows offset[k] .. offset[k + 1] - 1.
 * Any pointer may be NULL: all profiles linear, no H-Q tables, no links. */
typedef struct WfReservoirTables {
    const int32_t* storage_curve_type; /* [n] WfReservoirProfile (reservoir_water__storage_curve_type_count) */
    const int64_t* sh_offset;          /* [n + 1] rows of the S-H tables (empty for a linear profile) */
    const double* sh_h;                /* water level H [m], strictly increasing within a table */
    const double* sh_s;                /* storage S [m3], strictly increasing within a table */
    const int64_t* hq_offset;          /* [n + 1] rows of the H-Q tables (empty unless outflow type 1) */
    const double* hq_h;                /* water level H [m], strictly increasing within a table */
    const double* hq_q;                /* [rows x 365] discharge [m3 s-1] of each day of the year, row-major */
    const int32_t* lower_reservoir;    /* [n] linked lower reservoir (0-based index), -1 none
                                        * (reservoir_lower_location__count) */
} WfReservoirTables;

typedef struct WfHandle WfHandle;

/* Per-handle counters since creation (reset with wf_reset_metrics). */
typedef struct WfMetrics {
    int64_t steps;                /* model steps taken */
    int64_t cell_steps;           /* land cells x members x steps */
    int64_t substeps_land;        /* overland sub-steps taken (sum over steps) */
    int64_t substeps_river;
    int64_t substeps_subsurface;
    int64_t kernel_launches;      /* kernels launched by steps (graph nodes count once each) */
    double step_ms_total;         /* CUDA-event time of all steps */
    double max_abs_balance_error; /* reserved, always 0: the balance errors are fields
                                     (WF_F_BALANCE_*), read them with wf_get_field */
    int32_t device_status;        /* last device status word (0 = ok) */
    int32_t n_chains_land;        /* routing chains of the land graph */
    int32_t n_chains_river;
    int32_t max_chain_land;       /* longest chain (= graph height + 1) */
    int32_t max_chain_river;
    int32_t padding_slots_land;   /* padded slots of the land layout */
} WfMetrics;

/* Tuning knobs (filled by the autotuner; zero = library default). */
typedef struct WfTuning {
    int32_t vertical_block;   /* threads per block of the per-cell kernels */
    int32_t routing_warps;    /* warps per block of the routing wavefront kernels */
    int32_t routing_blocks_per_sm;
    int32_t use_graph;        /* capture the step in a CUDA graph (1 = yes, default) */
    int32_t reserved[8];      /* [0] wait budget (us), [1] test hook (0), [2] per-kernel timing,
                               * [3] cap of the routing sweeps' sub-step lanes (0 = default 8),
                               * [4] bit k set: node-major sweep k (0 subsurface, 1 overland,
                               * 2 river) holds its inputs in registers instead of staging them
                               * in shared memory (0 = all staged); [5] blocks per SM of the
                               * split vertical kernel's grid-stride loop, which sets the elements
                               * each thread walks (0 = 16); [6..7] 0 */
} WfTuning;

/* Library version / ABI check. */
int32_t wf_abi_version(void);

/* Model construction (replaces Model(config) for the hot-path state, Wflow/src/sbm_model.jl:7-57):
 * copies inputs, derives parameters, builds the drainage-graph wavefront schedule, allocates
 * device state in the cold-start values (soil.jl:164-178, utils.jl:916-937). */
int32_t wf_create(const WfConfig* config, const WfDomain* domain, const WfParams* params,
                  int32_t device, WfHandle** out);
/* The same with reservoirs (reservoir__flag = true; ReservoirModel, reservoir.jl:290-300);
 * reservoirs may be NULL or hold n = 0. Rejected: a reservoir at a river pit (the reference
 * raises the same error, surface_kinwave.jl:479-483), two reservoirs draining into one river
 * cell (the reference then keeps the outflow of whichever it updates last), an unknown outflow
 * type, a non-positive area. */
int32_t wf_create_with_reservoirs(const WfConfig* config, const WfDomain* domain, const WfParams* params,
                                  const WfReservoirs* reservoirs, int32_t device, WfHandle** out);
/* The same with the reservoirs' tables and links (tables may be NULL). The initial storage of
 * an interpolated profile and the maximum storage of a rating curve follow initialize_storage
 * and get_maximum_storage (reservoir.jl:322-360). A free weir linked to a lower reservoir reads
 * the lower reservoir's level and, when that is higher, moves water back from it within the
 * same sub-step (reservoir.jl:482-521); the lower reservoir must lie downstream of the upper one
 * on the river, the river paths between linked pairs must not join, and the river then routes
 * one sub-step per sweep launch. Rejected as well: a table that is not strictly increasing in
 * H (or in S), a rating curve without its H-Q table, an interpolated profile without its S-H
 * table, a link to itself or out of range. */
int32_t wf_create_with_reservoir_tables(const WfConfig* config, const WfDomain* domain, const WfParams* params,
                                        const WfReservoirs* reservoirs, const WfReservoirTables* tables,
                                        int32_t device, WfHandle** out);
void wf_destroy(WfHandle* h);

/* Message of the last error on this handle (or of the last failed wf_create when h is NULL). */
const char* wf_last_error(const WfHandle* h);

/* Forcing of the next step (AtmosphericForcing, Wflow/src/forcing.jl:2-10; io.jl:108-160):
 * host arrays of n_land*n_members values, member-major, land order (or n_land values, the
 * same for every member). From pinned host memory the copy is asynchronous: the arrays must
 * stay unchanged until the next wf_step (or wf_synchronize after wf_step_async) returns. */
int32_t wf_set_forcing(WfHandle* h, const double* precipitation, const double* potential_evaporation,
                       const double* temperature, int64_t count);
/* The same with the host-to-device copies on a stream of the handle's own, so that they overlap
 * a step still running (call it after wf_step_async of the previous step); the conversion into
 * the model's layout waits for that step. The arrays must stay unchanged until the step that
 * consumes them has returned from wf_step / wf_synchronize. No counterpart in the reference
 * (Wflow reads the forcing between steps); it is the same boundary as wf_set_forcing,
 * pipelined. */
int32_t wf_set_forcing_async(WfHandle* h, const double* precipitation, const double* potential_evaporation,
                             const double* temperature, int64_t count);
/* The same from FP32 arrays (forcing files usually hold FP32), half the bytes to copy: the split
 * form keeps its forcing in FP32 anyway; the FP64 form widens the values exactly. No counterpart
 * in the reference (Wflow converts forcing to Float64 on reading, io.jl:108-160). */
int32_t wf_set_forcing_f32(WfHandle* h, const float* precipitation, const float* potential_evaporation,
                           const float* temperature, int64_t count);
int32_t wf_set_forcing_async_f32(WfHandle* h, const float* precipitation, const float* potential_evaporation,
                                 const float* temperature, int64_t count);
/* The same with a count per array, each n_land * n_members (one set per member) or n_land (one set
 * for every member): an ensemble that perturbs only the precipitation copies the potential
 * evaporation and the temperature once. */
int32_t wf_set_forcing_counts_f32(WfHandle* h, const float* precipitation, int64_t count_precipitation,
                                  const float* potential_evaporation, int64_t count_potential_evaporation,
                                  const float* temperature, int64_t count_temperature);
int32_t wf_set_forcing_counts_async_f32(WfHandle* h, const float* precipitation, int64_t count_precipitation,
                                        const float* potential_evaporation, int64_t count_potential_evaporation,
                                        const float* temperature, int64_t count_temperature);
/* Same from device pointers already in the library's slot order (see wf_get_slot_order). */
int32_t wf_set_forcing_device_slots(WfHandle* h, const void* precipitation,
                                    const void* potential_evaporation, const void* temperature);

/* One model step: update_model! (sbm_model.jl:60-92) followed by compute_mass_balance!
 * (mass_balance.jl:541-545) when water_mass_balance is set. Synchronous on return. */
int32_t wf_step(WfHandle* h);
/* Asynchronous variant: enqueue the step on the handle's stream without waiting. */
int32_t wf_step_async(WfHandle* h);

/* Size of the static scratch of wf_step_static (bytes). */
#define WF_STATIC_SCRATCH_BYTES (16u * 1024u * 1024u)
/* One model step like wf_step (same kernels, same results), allocating nothing: no cudaMalloc,
 * cudaFree, CUDA graph instantiation or other allocating call. It has no counterpart in the
 * reference (Wflow.jl has no allocation-free step); it is for hosts that cannot allocate
 * device memory once the model exists, such as frameworks that reserve the whole device for
 * their own memory pool after set-up and coupling loops that cannot afford the device-wide
 * synchronisation of an allocation.
 *   - The routing wavefronts take their scratch (work ticket, chain-end flags, published
 *     chain-end discharges) from one file-scope device array of WF_STATIC_SCRATCH_BYTES.
 *     Models whose scratch need exceeds it, (256 + 4 * chains * members rounded up to 256 +
 *     8 * chains * members * sub-steps per launch) bytes for the larger of the land and river
 *     graphs, are rejected with WF_ERR_UNSUPPORTED and a message giving the need.
 *   - The first call on a device looks the array's address up (cudaGetSymbolAddress, with that
 *     device current). Under CUDA's lazy module loading (the default) that lookup can also be
 *     what loads the library's module and with it the array, so make the first call at set-up:
 *     before any stream capture and before the host hands the rest of the device memory to a
 *     pool of its own. Later calls load and allocate nothing.
 *   - Every call on a device shares the array, which keeps the last call's contents; each sweep
 *     clears what must start at zero before it runs. Calls that overlap on the GPU (handles
 *     stepped concurrently from different streams or threads) race on the array and must be
 *     serialised by the caller.
 * Synchronous on return, like wf_step. */
int32_t wf_step_static(WfHandle* h);
int32_t wf_synchronize(WfHandle* h);

/* Copy a field to host (count values from element offset; member-major over land or river
 * order). Layered fields take `layer`. BMI get_value / get_value_at_indices (bmi.jl:208-240). */
int32_t wf_get_field(WfHandle* h, int32_t field, int32_t layer, double* host_dst, int64_t offset,
                     int64_t count);
/* Overwrite a state field (BMI set_value, bmi.jl:246-248). */
int32_t wf_set_field(WfHandle* h, int32_t field, int32_t layer, const double* host_src,
                     int64_t offset, int64_t count);

/* Outlet discharge: river q_average (or q) at each river pit, member-major [n_members * n_pits]. */
int32_t wf_get_outlets(WfHandle* h, int32_t which /*0=q_average,1=q*/, double* host_dst,
                       int64_t capacity, int64_t* n_written);

/* Checkpoint of all step-carried state (states.jl; bmi.jl:357-371): query size with dst=NULL. */
int32_t wf_get_state(WfHandle* h, void* dst, size_t* size);
int32_t wf_set_state(WfHandle* h, const void* src, size_t size);

int32_t wf_get_metrics(WfHandle* h, WfMetrics* out);
int32_t wf_reset_metrics(WfHandle* h);
int32_t wf_set_tuning(WfHandle* h, const WfTuning* t);

/* Slot order of the land layout: ext_of_slot[s] = land index of slot s, -1 for padding. */
int32_t wf_get_slot_order(WfHandle* h, int64_t* ext_of_slot, int64_t capacity, int64_t* n_slots);

/* The handle's CUDA stream (a cudaStream_t), for callers that time or order their own work
 * against the step. */
int32_t wf_get_stream(WfHandle* h, void** stream);

/* Per-kernel device time of the steps run with kernel timing on (WfTuning.reserved[2] = 1):
 * ms[0..4] = vertical, subsurface, overland, river, balance (sums), calls = timed steps. */
int32_t wf_get_kernel_times(WfHandle* h, double* ms5, int64_t* calls);

/* Number of land cells, river cells, river pits and layer count of a handle. */
/* Adaptive sub-steps (a diagnostic with no counterpart in the reference): for every member the
 * sum of the squared sizes of the sub-steps that the last model step took in sweep `kind`
 * (0 subsurface, 1 overland, 2 river) [s2]; members whose sequences of sub-steps differ show
 * different sums. */
int32_t wf_get_substep_signature(WfHandle* h, int32_t kind, double* sig, int32_t n_members);
int32_t wf_get_sizes(WfHandle* h, int64_t* n_land, int64_t* n_river, int64_t* n_outlets,
                     int32_t* n_layers, int32_t* n_members);
/* Number of reservoirs of a handle. */
int32_t wf_get_reservoir_count(WfHandle* h, int64_t* n_reservoirs);
/* Day of the year (1..365, leap days not counted) whose column of the H-Q tables the next steps
 * read: update_index_hq! (reservoir.jl:376-382) sets it to julian_day(time - dt) before each
 * step. Default 1. */
int32_t wf_set_rating_curve_day(WfHandle* h, int32_t day_of_year);

/* ---- diagnostics (no counterpart in the reference) ---------------------------------------
 * Size of the ABI structs for binding checks: 0 WfConfig, 1 WfDomain, 2 WfParams,
 * 3 WfMetrics, 4 WfTuning, 5 WfReservoirs, 6 WfReservoirTables; -1 otherwise. */
int32_t wf_struct_size(int32_t which);
/* Host-only planning of a drainage graph's wavefront schedule (no GPU needed):
 * out_counts = {n_chains, n_chunks, n_slots, max_chain_len}; slot_of_node optional [n];
 * ok = 1 when the schedule invariants hold; g_out = chains per chunk. */
int32_t wf_plan_routing(int64_t n, const int32_t* downstream, int32_t members, int64_t* out_counts,
                        int64_t* slot_of_node, int32_t* ok, int32_t* g_out);
/* The same with heavy-child hints (heavy_hint[v]: a child of v that must continue v's chain, -1
 * none; the hints wf_create_with_reservoir_tables gives for linked reservoirs); chain_of_node
 * optional [n]. */
int32_t wf_plan_routing_hinted(int64_t n, const int32_t* downstream, int32_t members, const int64_t* heavy_hint,
                               int64_t* out_counts, int64_t* chain_of_node, int32_t* ok, int32_t* g_out);

#ifdef __cplusplus
}
#endif

#endif /* WFLOW_GB300_H */
