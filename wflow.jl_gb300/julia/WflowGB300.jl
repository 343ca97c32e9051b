"""
    WflowGB300

Julia side of the GB300 drop-in for Wflow.jl's `sbm` hot path. It binds the C ABI of
`libwflow_gb300.so` (include/wflow_gb300.h) with `ccall` and plugs into the reference's own
seam, `Wflow.run_timestep!(model; update_func = ...)` (Wflow/src/Wflow.jl:311-322):

    using Wflow, WflowGB300
    model = Wflow.Model(Wflow.Config("sbm_config.toml"))
    gpu = WflowGB300.GpuStep(model)                 # uploads domain, parameters, state
    Wflow.load_fixed_forcing!(model)
    for t in 1:nsteps
        Wflow.run_timestep!(model; update_func = m -> WflowGB300.gpu_update_model!(gpu, m))
    end

`gpu_update_model!` replaces `update_model!` (Wflow/src/sbm_model.jl:60-92) and
`compute_mass_balance!` (Wflow/src/mass_balance.jl:541-545): it uploads the step's
`AtmosphericForcing`, runs one step on the GPU and refreshes the host mirrors that BMI
`get_value_ptr` hands out (Wflow/src/bmi.jl:208-228): after every step (`mirrors = :eager`, the
default, for Wflow's output writers), or on demand (`GpuStep(model; mirrors = :lazy)`, then
`refresh_mirrors!` before reading and `set_value!` to write through). Errors come back as a negative status
and are rethrown as Julia exceptions with the library's message, like Wflow's own
throw-and-log path (Wflow/src/Wflow.jl:285-299).
"""
module WflowGB300

using Wflow

const LIB = get(ENV, "WFLOW_GB300_LIB", joinpath(@__DIR__, "..", "_build", "libwflow_gb300.so"))
const WF_MAX_LAYERS = 8

# ---- C structs (layout of include/wflow_gb300.h) --------------------------------------------
struct WfConfig
    dt::Float64
    n_soil_layer_thickness::Int32
    snow::Int32
    soil_layer_thickness::NTuple{7, Float64}
    soil_infiltration_reduction::Int32
    water_mass_balance::Int32
    adaptive_timestep::Int32
    kv_profile::Int32
    land_dt_fixed::Float64
    river_dt_fixed::Float64
    subsurface_dt_fixed::Float64
    subsurface_alpha::Float64
    form::Int32
    n_members::Int32
    per_member_soil::Int32
    snow_gravitational_transport::Int32
    glacier::Int32
    reserved::NTuple{5, Int32}
end

struct WfDomain
    n_land::Int64
    land_downstream::Ptr{Int32}
    area::Ptr{Float64}
    flow_width::Ptr{Float64}
    flow_length::Ptr{Float64}
    surface_flow_width::Ptr{Float64}
    slope::Ptr{Float64}
    flow_fraction_to_river::Ptr{Float64}
    river_fraction::Ptr{Float64}
    water_fraction::Ptr{Float64}
    elevation::Ptr{Float64}
    land_manning_n::Ptr{Float64}
    n_river::Int64
    river_land_index::Ptr{Int32}
    river_downstream::Ptr{Int32}
    river_width::Ptr{Float64}
    river_length::Ptr{Float64}
    river_slope::Ptr{Float64}
    river_manning_n::Ptr{Float64}
    river_bankfull_depth::Ptr{Float64}
    river_external_inflow::Ptr{Float64}
end

const PARAM_NAMES = (:canopy_gap_fraction, :maximum_canopy_storage, :crop_coefficient, :rooting_depth,
    :evaporation_to_precipitation_ratio, :degree_day_factor, :temperature_threshold_snowfall,
    :temperature_interval_snowfall, :temperature_threshold_melt, :water_holding_capacity, :theta_s,
    :theta_r, :kv_0, :f, :soil_thickness, :air_entry_pressure, :h1, :h2, :h3_high, :h3_low, :h4,
    :alpha_h1, :infiltration_capacity_compacted_soil, :compacted_soil_area_fraction,
    :wet_root_distribution_parameter, :cap_hmax, :cap_n, :maximum_leakage, :w_soil, :cf_soil, :z_exp,
    :brooks_corey_exponent, :kv_factor, :horizontal_to_vertical_ratio, :glacier_fraction,
    :glacier_temperature_threshold_melt, :glacier_degree_day_factor, :glacier_snow_to_ice_fraction,
    :glacier_initial_store)

struct WfParams
    ptrs::NTuple{39, Ptr{Float64}}
end

# reservoirs (WfReservoirs; ReservoirModel, Wflow/src/routing/surface/reservoir.jl)
struct WfReservoirs
    n::Int64
    river_index::Ptr{Int32}
    outflow_curve_type::Ptr{Int32}
    area::Ptr{Float64}
    waterlevel::Ptr{Float64}
    maximum_storage::Ptr{Float64}
    threshold::Ptr{Float64}
    rating_curve_coefficient::Ptr{Float64}
    rating_curve_exponent::Ptr{Float64}
    maximum_release::Ptr{Float64}
    demand::Ptr{Float64}
    target_minimum_fraction::Ptr{Float64}
    target_full_fraction::Ptr{Float64}
end

# tables and links of reservoirs (WfReservoirTables): S-H and H-Q tables concatenated over the
# reservoirs (offsets [n + 1]), H-Q discharges row-major with 365 columns, lower reservoir 0-based
struct WfReservoirTables
    storage_curve_type::Ptr{Int32}
    sh_offset::Ptr{Int64}
    sh_h::Ptr{Float64}
    sh_s::Ptr{Float64}
    hq_offset::Ptr{Int64}
    hq_h::Ptr{Float64}
    hq_q::Ptr{Float64}
    lower_reservoir::Ptr{Int32}
end

# WfField ids (enum WfField)
const F_LAND = (:canopy_storage, :snow_storage, :snow_water, :soil_surface_temperature,
    :saturated_water_depth, :unsaturated_layer_depth, :ssf_q, :land_q, :land_h, :water_table_depth)
const F_GLACIER_STORE = Int32(41)
const F_GLACIER_MELT = Int32(42)
const F_SNOW_IN = Int32(43)
const F_SNOW_OUT = Int32(44)
const F_RIVER_Q = Int32(100)
const F_RIVER_H = Int32(101)
const F_RIVER_Q_AVERAGE = Int32(103)
const F_RESERVOIR_STORAGE = Int32(200)
const F_RESERVOIR_WATERLEVEL = Int32(201)
const F_RESERVOIR_OUTFLOW = Int32(202)
const F_RESERVOIR_OUTFLOW_AVERAGE = Int32(203)
const F_RESERVOIR_PRECIPITATION = Int32(209)
const F_RESERVOIR_EVAPORATION = Int32(210)
const F_RESERVOIR_EXTERNAL_INFLOW = Int32(211)
const F_RESERVOIR_OUTFLOW_OBS = Int32(212)

mutable struct GpuStep
    handle::Ptr{Cvoid}
    keep::Vector{Any}              # arrays whose pointers were handed to wf_create
    n_land::Int
    n_river::Int
    forcing::NTuple{3, Vector{Float64}}
    n_reservoirs::Int
    li::Any                        # GpuLocalInertial routing the land and river in the step, or nothing
    mirrors::Symbol                # :eager (refresh the host mirrors after every step) or :lazy
    stale::Bool                    # :lazy: the host mirrors predate the last GPU step
end

check(st, h, what) = st == 0 || error("$what failed ($st): " *
                                      unsafe_string(ccall((:wf_last_error, LIB), Cstring, (Ptr{Cvoid},), h)))

"Downstream index of every node of a Graphs.jl D8 flow graph (-1 for a pit), 0-based."
function downstream_index(graph)
    n = Wflow.Graphs.nv(graph)
    ds = fill(Int32(-1), n)
    for v in 1:n
        out = Wflow.Graphs.outneighbors(graph, v)
        isempty(out) || (ds[v] = Int32(only(out) - 1))
    end
    return ds
end

"""
    check_supported(config)

Throw when the model uses a component outside the GPU step (the caller then keeps the
reference's own `update_model!`): model type other than `sbm`, water demand, floodplains,
drains, staggered Manning routing, local-inertial routing of the river alone or of the land alone,
local-inertial routing with reservoirs or adaptive kinematic-wave steps, Kv profiles other than
exponential / exponential_constant, gravitational snow transport together with reservoirs.
Glaciers, gravitational snow transport, reservoirs of every outflow type and storage profile
(linked reservoirs whose river paths join excepted: `wf_create_with_reservoir_tables` refuses
them) and local-inertial routing of the land with its river run on the GPU.
"""
"Land and river both routed by the local-inertial scheme (surface_routing.jl:62-89)."
local_inertial_both(config) = config.model.land_routing == Wflow.RoutingType.local_inertial &&
                              config.model.river_routing == Wflow.RoutingType.local_inertial

function check_supported(config)
    m = config.model
    bad = String[]
    m.type == Wflow.ModelType.sbm || push!(bad, "model type $(m.type)")
    m.snow_gravitational_transport__flag && m.reservoir__flag &&
        push!(bad, "snow_gravitational_transport__flag with reservoir__flag")
    Wflow.do_water_demand(config) && push!(bad, "water demand")
    m.floodplain_1d__flag && push!(bad, "floodplain_1d__flag")
    m.drain__flag && push!(bad, "drain__flag")
    kin = m.land_routing == Wflow.RoutingType.kinematic_wave && m.river_routing == Wflow.RoutingType.kinematic_wave
    li = local_inertial_both(config)
    (kin || li) || push!(bad, "land_routing $(m.land_routing) with river_routing $(m.river_routing)")
    li && m.reservoir__flag && push!(bad, "local-inertial routing with reservoir__flag")
    li && m.kinematic_wave__adaptive_time_step_flag &&
        push!(bad, "local-inertial routing with kinematic_wave__adaptive_time_step_flag")
    m.saturated_hydraulic_conductivity_profile in (Wflow.VerticalConductivityProfile.exponential,
        Wflow.VerticalConductivityProfile.exponential_constant) ||
        push!(bad, "saturated_hydraulic_conductivity_profile $(m.saturated_hydraulic_conductivity_profile)")
    isempty(bad) || error("not supported by the GPU step: " * join(bad, ", "))
    return nothing
end

"""
    GpuStep(model::Wflow.Model; mirrors = :eager)

Copy the model's domain, parameters (as read from the static maps, in SI) and current state
to a new library handle (`wf_create`, then `wf_set_field` for a warm state). `mirrors`: when
the host copies of the GPU state are refreshed (`gpu_update_model!`, `refresh_mirrors!`).
"""
function GpuStep(model; mirrors::Symbol = :eager)
    mirrors in (:eager, :lazy) || error("mirrors must be :eager or :lazy")
    (; domain, land, routing, config) = model
    check_supported(config)
    lp = domain.land.parameters
    rp = domain.river.parameters
    soil = land.soil.parameters
    veg = soil.vegetation_parameter_set
    keep = Any[]
    k(x) = (push!(keep, x); pointer(x))
    ds_land = downstream_index(domain.land.network.graph)
    ds_river = downstream_index(domain.river.network.graph)
    nl = length(config.model.soil_layer__thickness)
    thick = ntuple(i -> i <= nl ? config.model.soil_layer__thickness[i] / 1000.0 : 0.0, 7)
    cfg = WfConfig(tosecond(model.clock.dt), Int32(nl), Int32(config.model.snow__flag), thick,
        Int32(config.model.soil_infiltration_reduction__flag), Int32(config.model.water_mass_balance__flag),
        Int32(config.model.kinematic_wave__adaptive_time_step_flag), Int32(0),
        config.model.land_kinematic_wave__time_step, config.model.river_kinematic_wave__time_step,
        config.model.subsurface_kinematic_wave__time_step,
        config.model.subsurface_kinematic_wave__alpha_coefficient, Int32(0), Int32(1), Int32(0),
        Int32(config.model.snow__flag && config.model.snow_gravitational_transport__flag),
        Int32(config.model.snow__flag && config.model.glacier__flag), ntuple(_ -> Int32(0), 5))
    # the kinematic-wave land roughness; unused when the local-inertial scheme routes the land
    land_n = local_inertial_both(config) ? fill(0.072, length(ds_land)) : routing.overland_flow.parameters.mannings_n
    dom = WfDomain(length(ds_land), k(ds_land), k(lp.area), k(lp.flow_width), k(lp.flow_length),
        k(lp.surface_flow_width), k(lp.slope), k(lp.flow_fraction_to_river), k(lp.river_fraction),
        k(lp.water_fraction), k(routing.subsurface_flow.parameters.top), k(land_n), length(ds_river),
        k(Int32.(domain.river.network.land_indices .- 1)), k(ds_river), k(rp.flow_width), k(rp.flow_length),
        k(rp.slope), k(routing.river_flow.parameters.mannings_n),
        k(routing.river_flow.parameters.bankfull_depth),
        k(routing.river_flow.boundary_conditions.external_inflow))
    layered(v) = collect(Iterators.flatten(v))
    # static parameters as read (before derivation), see WfParams in the header
    src = Dict{Symbol, Vector{Float64}}(
        :canopy_gap_fraction => veg.canopy_gap_fraction, :maximum_canopy_storage => veg.maximum_canopy_storage,
        :crop_coefficient => veg.crop_coefficient, :rooting_depth => veg.rooting_depth,
        :theta_s => soil.theta_s, :theta_r => soil.theta_r, :kv_0 => soil.kv_profile.kv_0,
        :f => soil.kv_profile.hydraulic_conductivity_scale_parameter, :soil_thickness => soil.soil_thickness,
        :air_entry_pressure => soil.air_entry_pressure, :h1 => soil.h1, :h2 => soil.h2,
        :h3_high => soil.h3_high, :h3_low => soil.h3_low, :h4 => soil.h4, :alpha_h1 => soil.alpha_h1,
        :infiltration_capacity_compacted_soil => soil.infiltration_capacity_compacted_soil,
        :compacted_soil_area_fraction => soil.compacted_soil_area_fraction,
        :wet_root_distribution_parameter => soil.wet_root_distribution_parameter,
        :cap_hmax => soil.cap_hmax, :cap_n => soil.cap_n, :maximum_leakage => soil.maximum_leakage,
        :w_soil => soil.w_soil, :cf_soil => soil.cf_soil,
        :brooks_corey_exponent => layered(soil.brooks_corey_exponent),
        :kv_factor => layered(soil.vertical_hydraulic_conductivity_factor),
        :horizontal_to_vertical_ratio =>
            routing.subsurface_flow.parameters.horizontal_to_vertical_hydraulic_conductivity_ratio)
    if config.model.snow__flag
        sp = land.snow.parameters
        src[:degree_day_factor] = sp.degree_day_factor
        src[:temperature_threshold_snowfall] = sp.temperature_threshold_snowfall
        src[:temperature_interval_snowfall] = sp.temperature_interval_snowfall
        src[:temperature_threshold_melt] = sp.temperature_threshold_melt
        src[:water_holding_capacity] = sp.water_holding_capacity
    end
    if config.model.snow__flag && config.model.glacier__flag
        gp = land.glacier.parameters
        src[:glacier_fraction] = gp.glacier_fraction
        src[:glacier_temperature_threshold_melt] = gp.temperature_threshold_melt
        src[:glacier_degree_day_factor] = gp.degree_day_factor
        src[:glacier_snow_to_ice_fraction] = gp.snow_to_ice_fraction
        src[:glacier_initial_store] = land.glacier.variables.glacier_store
    end
    params = WfParams(ntuple(i -> haskey(src, PARAM_NAMES[i]) ? k(src[PARAM_NAMES[i]]) : Ptr{Float64}(0), 39))
    # reservoirs at their outlet river cells, in the reservoir model's order
    # (NetworkReservoir.river_indices, network.jl:333-350), with their S-H / H-Q tables and links
    nres = 0
    res = WfReservoirs(0, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL,
        C_NULL, C_NULL)
    tables = WfReservoirTables(C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL)
    if config.model.reservoir__flag
        rv = routing.river_flow.boundary_conditions.reservoir
        p = rv.parameters
        nres = length(p.area)
        res = WfReservoirs(nres, k(Int32.(domain.reservoir.network.river_indices .- 1)),
            k(Int32.(Integer.(p.outflow_curve_type))), k(p.area), k(rv.variables.waterlevel),
            k(p.maximum_storage), k(p.threshold), k(p.rating_curve_coefficient), k(p.rating_curve_exponent),
            k(p.maximum_release), k(p.demand), k(p.target_minimum_fraction), k(p.target_full_fraction))
        tables = reservoir_tables(p, k)
    end
    h = Ref{Ptr{Cvoid}}(C_NULL)
    st = ccall((:wf_create_with_reservoir_tables, LIB), Int32,
        (Ref{WfConfig}, Ref{WfDomain}, Ref{WfParams}, Ref{WfReservoirs}, Ref{WfReservoirTables}, Int32,
         Ref{Ptr{Cvoid}}), cfg, dom, params, res, tables, Int32(0), h)
    check(st, C_NULL, "wf_create_with_reservoir_tables")
    n = length(ds_land)
    gpu = GpuStep(h[], keep, n, length(ds_river), (zeros(n), zeros(n), zeros(n)), nres, nothing, mirrors, false)
    finalizer(g -> ccall((:wf_destroy, LIB), Cvoid, (Ptr{Cvoid},), g.handle), gpu)
    if local_inertial_both(config)
        # the land grid with its river routes inside wf_step (wf_attach_local_inertial); the
        # domain handle outlives the step handle through gpu.li
        gpu.li = GpuLocalInertial(model)
        check(ccall((:wf_attach_local_inertial, LIB), Int32, (Ptr{Cvoid}, Ptr{Cvoid}), gpu.handle, gpu.li.handle),
            gpu.handle, "wf_attach_local_inertial")
    end
    return gpu
end

"""
    reservoir_tables(p, k)

The S-H and H-Q tables (`storage_waterlevel_curve`, `waterlevel_discharge_curve`, read from
reservoir_sh_<id>.csv / reservoir_hq_<id>.csv by read_sh_csv / read_hq_csv, io.jl:1129-1147) and
the links (`lower_reservoir_ind`, 1-based, 0 none) of ReservoirParameters `p` as a
WfReservoirTables; `k` keeps the arrays alive.
"""
function reservoir_tables(p, k)
    n = length(p.area)
    sh_off, hq_off = zeros(Int64, n + 1), zeros(Int64, n + 1)
    sh_h, sh_s, hq_h, hq_q = Float64[], Float64[], Float64[], Float64[]
    for i in 1:n
        sh = p.storage_waterlevel_curve[i]
        if p.storage_curve_type[i] == Wflow.ReservoirProfileType.interpolation
            append!(sh_h, sh.H)
            append!(sh_s, sh.S)
        end
        sh_off[i + 1] = length(sh_h)
        hq = p.waterlevel_discharge_curve[i]
        if p.outflow_curve_type[i] == Wflow.ReservoirOutflowType.rating_curve
            append!(hq_h, hq.H)
            append!(hq_q, vec(permutedims(hq.Q)))  # row-major: the 365 days of each level
        end
        hq_off[i + 1] = length(hq_h)
    end
    ptr(v) = isempty(v) ? Ptr{Float64}(0) : k(v)
    return WfReservoirTables(k(Int32.(Integer.(p.storage_curve_type))), k(sh_off), ptr(sh_h), ptr(sh_s),
        k(hq_off), ptr(hq_h), ptr(hq_q), k(Int32.(p.lower_reservoir_ind .- 1)))
end

"""
    gpu_update_model!(gpu::GpuStep, model)

`update_func` for `Wflow.run_timestep!`: one update_model! + compute_mass_balance! on the GPU.
"""
function gpu_update_model!(gpu::GpuStep, model)
    f = model.land.atmospheric_forcing
    st = ccall((:wf_set_forcing, LIB), Int32, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Int64),
        gpu.handle, f.precipitation, f.potential_evaporation, f.temperature, gpu.n_land)
    check(st, gpu.handle, "wf_set_forcing")
    if gpu.n_reservoirs > 0
        # the reservoir inputs Wflow's forcing reader filled (io.jl:128-137) and the boundary
        # conditions of the reservoir model
        rv = model.routing.river_flow.boundary_conditions.reservoir
        set_field!(gpu, F_RESERVOIR_PRECIPITATION, rv.boundary_conditions.precipitation)
        set_field!(gpu, F_RESERVOIR_EVAPORATION, rv.boundary_conditions.evaporation)
        set_field!(gpu, F_RESERVOIR_EXTERNAL_INFLOW, rv.boundary_conditions.external_inflow)
        set_field!(gpu, F_RESERVOIR_OUTFLOW_OBS, rv.variables.outflow_obs)
        # update_index_hq! (reservoir.jl:379-385): the H-Q column of the step's first day
        if Wflow.ReservoirOutflowType.rating_curve in rv.parameters.outflow_curve_type
            day = Wflow.julian_day(model.clock.time - model.clock.dt)
            rv.parameters.col_index_hq[1] = day
            check(ccall((:wf_set_rating_curve_day, LIB), Int32, (Ptr{Cvoid}, Int32), gpu.handle, Int32(day)),
                gpu.handle, "wf_set_rating_curve_day")
        end
    end
    check(ccall((:wf_step, LIB), Int32, (Ptr{Cvoid},), gpu.handle), gpu.handle, "wf_step")
    if gpu.mirrors === :eager
        sync_mirrors!(gpu, model)
    else
        gpu.stale = true
    end
    gpu.li === nothing || li_copy_back!(gpu.li, model, tosecond(model.clock.dt))
    return nothing
end

"Copy a library field into a host vector (BMI get_value semantics)."
function get_field!(dst::Vector{Float64}, gpu::GpuStep, field::Integer; layer::Integer = 0)
    st = ccall((:wf_get_field, LIB), Int32, (Ptr{Cvoid}, Int32, Int32, Ptr{Float64}, Int64, Int64),
        gpu.handle, Int32(field), Int32(layer), dst, 0, length(dst))
    check(st, gpu.handle, "wf_get_field")
    return dst
end

"Write a host vector into a library state field (BMI set_value semantics)."
function set_field!(gpu::GpuStep, field::Integer, src::Vector{Float64}; layer::Integer = 0)
    st = ccall((:wf_set_field, LIB), Int32, (Ptr{Cvoid}, Int32, Int32, Ptr{Float64}, Int64, Int64),
        gpu.handle, Int32(field), Int32(layer), src, 0, length(src))
    check(st, gpu.handle, "wf_set_field")
end

"""
    refresh_mirrors!(gpu::GpuStep, model)

With `mirrors = :lazy`, copy the GPU state into the host vectors if a step ran since the last
refresh (a dirty flag); call it before BMI `get_value` / `get_value_ptr` (Wflow/src/bmi.jl:208-228)
or before writing output. With `:eager` the mirrors are always current.
"""
function refresh_mirrors!(gpu::GpuStep, model)
    if gpu.stale
        sync_mirrors!(gpu, model)
        gpu.stale = false
    end
    return nothing
end

"""
    set_value!(gpu::GpuStep, model, host::Vector{Float64}, field::Integer, values)

BMI `set_value` for a field the GPU step owns (Wflow/src/bmi.jl:241-262): the host vector is
brought up to date first (a lazy mirror), then `values` is written through to both the host
vector and the GPU field `field` (a WfField id), so the next step and the next read see it.
"""
function set_value!(gpu::GpuStep, model, host::Vector{Float64}, field::Integer, values)
    refresh_mirrors!(gpu, model)
    copyto!(host, values)
    set_field!(gpu, field, host)
    return nothing
end

"Refresh the host vectors Wflow's BMI and writers read after a GPU step."
function sync_mirrors!(gpu::GpuStep, model)
    (; routing) = model
    if gpu.li === nothing  # local-inertial routing: li_copy_back! copies the scheme's variables
        get_field!(routing.river_flow.variables.q, gpu, F_RIVER_Q)
        get_field!(routing.river_flow.variables.h, gpu, F_RIVER_H)
        get_field!(routing.river_flow.variables.q_average, gpu, F_RIVER_Q_AVERAGE)
        get_field!(routing.overland_flow.variables.q, gpu, 7)
        get_field!(routing.overland_flow.variables.h, gpu, 8)
    end
    get_field!(routing.subsurface_flow.variables.q, gpu, 6)
    get_field!(model.land.soil.variables.saturated_water_depth, gpu, 4)
    (; config) = model
    if config.model.snow__flag
        sv = model.land.snow.variables
        get_field!(sv.snow_storage, gpu, 1)
        get_field!(sv.snow_water, gpu, 2)
        if config.model.snow_gravitational_transport__flag
            get_field!(sv.snow_in, gpu, F_SNOW_IN)
            get_field!(sv.snow_out, gpu, F_SNOW_OUT)
        end
        if config.model.glacier__flag
            get_field!(model.land.glacier.variables.glacier_store, gpu, F_GLACIER_STORE)
            get_field!(model.land.glacier.variables.glacier_melt, gpu, F_GLACIER_MELT)
        end
    end
    if gpu.n_reservoirs > 0
        rv = routing.river_flow.boundary_conditions.reservoir.variables
        get_field!(rv.storage, gpu, F_RESERVOIR_STORAGE)
        get_field!(rv.waterlevel, gpu, F_RESERVOIR_WATERLEVEL)
        get_field!(rv.outflow, gpu, F_RESERVOIR_OUTFLOW)
        get_field!(rv.outflow_average, gpu, F_RESERVOIR_OUTFLOW_AVERAGE)
    end
    return nothing
end

# ---- local-inertial routing (include/wflow_gb300_li.h) -----------------------------------------

struct WfLiLandGrid
    n::Int64
    ind_x_up::Ptr{Int64}
    ind_x_down::Ptr{Int64}
    ind_y_up::Ptr{Int64}
    ind_y_down::Ptr{Int64}
    river_index::Ptr{Int64}
    x_length::Ptr{Float64}
    y_length::Ptr{Float64}
    elevation::Ptr{Float64}
    mannings_n_sq::Ptr{Float64}
    xwidth_at_edge::Ptr{Float64}
    ywidth_at_edge::Ptr{Float64}
    theta::Float64
    h_thresh::Float64
    alpha::Float64
    froude_limit::Int32
end

struct WfLiRiverNetwork
    n::Int64
    n_active::Int64
    n_edges::Int64
    src::Ptr{Int64}
    dst::Ptr{Int64}
    zb::Ptr{Float64}
    flow_length::Ptr{Float64}
    flow_width::Ptr{Float64}
    bankfull_depth::Ptr{Float64}
    zb_edge::Ptr{Float64}
    width_edge::Ptr{Float64}
    length_edge::Ptr{Float64}
    mannings_n_sq_edge::Ptr{Float64}
    h_thresh::Float64
    alpha::Float64
    froude_limit::Int32
end

# enum WfLiDomainField
const LI_LAND_H, LI_LAND_STORAGE, LI_LAND_ERROR, LI_LAND_QX, LI_LAND_QY, LI_LAND_QX_AVERAGE,
      LI_LAND_QY_AVERAGE, LI_RIVER_H, LI_RIVER_STORAGE, LI_RIVER_Q, LI_RIVER_Q_AVERAGE,
      LI_RIVER_ABSTRACTION_CUMULATIVE = Int32.(0:11)

mutable struct GpuLocalInertial
    handle::Ptr{Cvoid}
    keep::Vector{Any}
    n_land::Int
    n_river::Int       # river cells with the ghost cells after them
    n_edges::Int
end

li_check(st, h, what) = st == 0 || error("$what failed ($st): " *
                                         unsafe_string(ccall((:wf_li_domain_last_error, LIB), Cstring,
                                                             (Ptr{Cvoid},), h)))

# 0-based copy of a 1-based index vector (the value n + 1, outside, becomes n)
zero_based(v) = Int64.(v) .- 1

# a river cell vector padded to the ghost cells (their lengths and widths are not used; their
# inflows are zero)
pad_river(v, n_total) = vcat(Float64.(v), ones(n_total - length(v)))
pad_zero(v, n_total) = vcat(Float64.(v), zeros(n_total - length(v)))

"""
    GpuLocalInertial(model)

The land grid and river of a model with `land_routing = "local_inertial"` and `river_routing =
"local_inertial"` (no reservoirs, no 1D floodplain) as a `wf_li_domain` handle: the land edge
indices, river locations, lengths, elevation, Manning's n squared and effective widths of
`LocalInertialOverlandFlowParameters`, the river network and `RiverFlowStaggeredParameters`,
and the current state (`wf_li_domain_set_state`).
"""
function GpuLocalInertial(model)
    (; domain, routing, config) = model
    m = config.model
    (m.land_routing == Wflow.RoutingType.local_inertial &&
     m.river_routing == Wflow.RoutingType.local_inertial) ||
        error("GpuLocalInertial needs local-inertial land and river routing")
    (m.reservoir__flag || m.floodplain_1d__flag) &&
        error("GpuLocalInertial: reservoirs and the 1D floodplain are not supported")
    land, river = routing.overland_flow, routing.river_flow
    lp, rp = land.parameters, river.parameters
    ei = domain.land.network.edge_indices
    riv_loc = domain.land.parameters.river_location
    riv_idx = domain.land.network.river_indices
    n = lp.n
    n_total = length(river.variables.h)
    keep = Any[
        zero_based(ei.ind_x_up), zero_based(ei.ind_x_down), zero_based(ei.ind_y_up), zero_based(ei.ind_y_down),
        Int64[riv_loc[i] ? riv_idx[i] - 1 : -1 for i in 1:n],
        Float64.(domain.land.parameters.x_length), Float64.(domain.land.parameters.y_length), lp.z,
        lp.mannings_n_sq_at_edge, lp.xwidth_at_edge, lp.ywidth_at_edge,
    ]
    g = WfLiLandGrid(n, pointer(keep[1]), pointer(keep[2]), pointer(keep[3]), pointer(keep[4]),
        pointer(keep[5]), pointer(keep[6]), pointer(keep[7]), pointer(keep[8]), pointer(keep[9]),
        pointer(keep[10]), pointer(keep[11]), lp.theta, lp.h_thresh, land.timestepping.alpha_coefficient,
        Int32(lp.froude_limit))
    nae = domain.river.network.nodes_at_edge
    rk = Any[
        zero_based(nae.src), zero_based(nae.dst), Float64.(rp.zb),
        pad_river(domain.river.parameters.flow_length, n_total),
        pad_river(domain.river.parameters.flow_width, n_total), pad_river(rp.bankfull_depth, n_total),
        rp.zb_at_edge, rp.flow_width_at_edge, rp.flow_length_at_edge, rp.mannings_n_sq_at_edge,
        copy(river.variables.h),
    ]
    length(rk[3]) == n_total || error("river bed levels must cover the ghost cells")
    append!(keep, rk)
    r = WfLiRiverNetwork(n_total, rp.n, rp.n_edges, pointer(rk[1]), pointer(rk[2]), pointer(rk[3]),
        pointer(rk[4]), pointer(rk[5]), pointer(rk[6]), pointer(rk[7]), pointer(rk[8]), pointer(rk[9]),
        pointer(rk[10]), rp.h_thresh, river.timestepping.alpha_coefficient, Int32(rp.froude_limit))
    handle = Ref{Ptr{Cvoid}}(C_NULL)
    st = GC.@preserve keep ccall((:wf_li_domain_create, LIB), Int32,
        (Ref{WfLiLandGrid}, Ref{WfLiRiverNetwork}, Ptr{Float64}, Int32, Ref{Ptr{Cvoid}}),
        g, r, rk[11], Int32(0), handle)
    li_check(st, C_NULL, "wf_li_domain_create")
    gpu = GpuLocalInertial(handle[], keep, n, n_total, rp.n_edges)
    finalizer(x -> ccall((:wf_li_domain_destroy, LIB), Cvoid, (Ptr{Cvoid},), x.handle), gpu)
    lv = land.variables
    st = ccall((:wf_li_domain_set_state, LIB), Int32,
        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
        gpu.handle, lv.h, river.variables.h, lv.qx, lv.qy, river.variables.q)
    li_check(st, gpu.handle, "wf_li_domain_set_state")
    return gpu
end

li_get!(dst, gpu::GpuLocalInertial, field) =
    li_check(ccall((:wf_li_domain_get, LIB), Int32, (Ptr{Cvoid}, Int32, Ptr{Float64}), gpu.handle, field, dst),
        gpu.handle, "wf_li_domain_get")

"""
    gpu_update_local_inertial!(gpu::GpuLocalInertial, model, dt)

In place of `update_overland_flow_model!(overland, river, domain, clock, dt)`
(Wflow/src/routing/surface/surface_staggered_scheme.jl:1153-1193): uploads the runoff, external
inflow and abstraction, runs the model step's sub-steps on the GPU and copies the land and river
variables back into the model.
"""
function gpu_update_local_inertial!(gpu::GpuLocalInertial, model, dt)
    land, river = model.routing.overland_flow, model.routing.river_flow
    rbc = river.boundary_conditions
    ext = pad_zero(rbc.external_inflow, gpu.n_river)
    abst = pad_zero(rbc.abstraction, gpu.n_river)
    st = ccall((:wf_li_domain_set_inputs, LIB), Int32, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
        gpu.handle, land.boundary_conditions.runoff, ext, abst)
    li_check(st, gpu.handle, "wf_li_domain_set_inputs")
    li_check(ccall((:wf_li_domain_step, LIB), Int32, (Ptr{Cvoid}, Float64, Ptr{Int64}), gpu.handle, dt, C_NULL),
        gpu.handle, "wf_li_domain_step")
    li_copy_back!(gpu, model, dt)
    return nothing
end

"The land and river variables of the local-inertial domain into the model (after its step)."
function li_copy_back!(gpu::GpuLocalInertial, model, dt)
    land, river = model.routing.overland_flow, model.routing.river_flow
    rbc = river.boundary_conditions
    lv, rv = land.variables, river.variables
    n = gpu.n_land
    for (field, v) in ((LI_LAND_H, lv.h), (LI_LAND_STORAGE, lv.storage), (LI_LAND_ERROR, lv.error))
        li_get!(v, gpu, field)
    end
    tmp = Vector{Float64}(undef, n)
    for (field, v) in ((LI_LAND_QX, lv.qx), (LI_LAND_QY, lv.qy), (LI_LAND_QX_AVERAGE, lv.qx_average),
                       (LI_LAND_QY_AVERAGE, lv.qy_average))
        li_get!(tmp, gpu, field)
        v[1:n] .= tmp      # the n + 1-th value (outside the grid) stays zero
    end
    li_get!(rv.h, gpu, LI_RIVER_H)
    rs = Vector{Float64}(undef, gpu.n_river)
    li_get!(rs, gpu, LI_RIVER_STORAGE)
    rv.storage .= rs[1:length(rv.storage)]
    li_get!(rv.q, gpu, LI_RIVER_Q)
    li_get!(rv.q_average, gpu, LI_RIVER_Q_AVERAGE)
    li_get!(rs, gpu, LI_RIVER_ABSTRACTION_CUMULATIVE)
    rbc.actual_external_abstraction_cumulative .= rs[1:length(rbc.actual_external_abstraction_cumulative)]
    # average_flow_vars! (surface_kinwave.jl:283-290)
    rbc.actual_external_abstraction_average .= rbc.actual_external_abstraction_cumulative ./ dt
    return nothing
end

"""
    GpuLocalInertialRiver(model)

The river of a model with `river_routing = "local_inertial"` or `"manning_staggered"`
(kinematic-wave land, no reservoirs, no 1D floodplain) as a `wf_li_river` handle, with the stable
time step over the real river cells (the ghost cells follow them) and the current depths and
discharges.
"""
mutable struct GpuLocalInertialRiver
    handle::Ptr{Cvoid}
    keep::Vector{Any}
    n_river::Int
    n_real::Int
end

function GpuLocalInertialRiver(model)
    (; domain, routing, config) = model
    m = config.model
    manning = m.river_routing == Wflow.RoutingType.manning_staggered
    (m.river_routing == Wflow.RoutingType.local_inertial || manning) ||
        error("GpuLocalInertialRiver needs local-inertial or staggered Manning rivers")
    (m.reservoir__flag || m.floodplain_1d__flag) &&
        error("GpuLocalInertialRiver: reservoirs and the 1D floodplain are not supported")
    river = routing.river_flow
    rp = river.parameters
    n_total = length(river.variables.h)
    nae = domain.river.network.nodes_at_edge
    keep = Any[zero_based(nae.src), zero_based(nae.dst), Float64.(rp.zb),
        pad_river(domain.river.parameters.flow_length, n_total), pad_river(domain.river.parameters.flow_width, n_total),
        copy(river.variables.h), rp.zb_at_edge, rp.flow_width_at_edge, rp.flow_length_at_edge,
        manning ? ones(rp.n_edges) : rp.mannings_n_sq_at_edge]  # (unused by the Manning scheme)
    handle = Ref{Ptr{Cvoid}}(C_NULL)
    st = GC.@preserve keep ccall((:wf_li_river_create, LIB), Int32,
        (Int64, Int64, Int64, Ptr{Int64}, Ptr{Int64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
         Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Float64, Int32, Float64, Int32, Ref{Ptr{Cvoid}}),
        n_total, rp.n, rp.n_edges, keep[1], keep[2], keep[3], keep[4], keep[5], keep[6], keep[7], keep[8], keep[9],
        keep[10], rp.h_thresh, Int32(rp.froude_limit), river.timestepping.alpha_coefficient, Int32(0), handle)
    riv_check(st, C_NULL, "wf_li_river_create")
    gpu = GpuLocalInertialRiver(handle[], keep, n_total, rp.n)
    finalizer(x -> ccall((:wf_li_river_destroy, LIB), Cvoid, (Ptr{Cvoid},), x.handle), gpu)
    riv_check(ccall((:wf_li_river_set_timestep_cells, LIB), Int32, (Ptr{Cvoid}, Int64), gpu.handle, rp.n),
        gpu.handle, "wf_li_river_set_timestep_cells")
    if manning  # river_routing = "manning_staggered" (surface_staggered_scheme.jl:386-434)
        push!(gpu.keep, rp.slope_at_edge, rp.mannings_n_at_edge)
        riv_check(ccall((:wf_li_river_set_manning, LIB), Int32, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}),
                gpu.handle, rp.slope_at_edge, rp.mannings_n_at_edge), gpu.handle, "wf_li_river_set_manning")
    end
    riv_check(ccall((:wf_li_river_set_state, LIB), Int32, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}),
            gpu.handle, river.variables.h, river.variables.q), gpu.handle, "wf_li_river_set_state")
    return gpu
end

riv_check(st, h, what) = st == 0 || error("$what failed ($st): " *
                                          unsafe_string(ccall((:wf_li_river_last_error, LIB), Cstring,
                                                              (Ptr{Cvoid},), h)))

"""
    gpu_update_river_flow_model!(gpu::GpuLocalInertialRiver, model, dt)

In place of `update_river_flow_model!` for a local-inertial river
(Wflow/src/routing/surface/surface_staggered_scheme.jl:800-826): uploads `inwater`, the external
inflow and the abstraction, runs the step on the GPU and copies the river variables back.
"""
function gpu_update_river_flow_model!(gpu::GpuLocalInertialRiver, model, dt)
    river = model.routing.river_flow
    bc, v = river.boundary_conditions, river.variables
    n = gpu.n_river
    riv_check(ccall((:wf_li_river_set_inwater, LIB), Int32, (Ptr{Cvoid}, Ptr{Float64}), gpu.handle,
            pad_zero(bc.inwater, n)), gpu.handle, "wf_li_river_set_inwater")
    riv_check(ccall((:wf_li_river_set_boundary, LIB), Int32, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}), gpu.handle,
            pad_zero(bc.external_inflow, n), pad_zero(bc.abstraction, n)), gpu.handle, "wf_li_river_set_boundary")
    riv_check(ccall((:wf_li_river_step, LIB), Int32, (Ptr{Cvoid}, Float64, Ptr{Int64}), gpu.handle, dt, C_NULL),
        gpu.handle, "wf_li_river_step")
    tmp = Vector{Float64}(undef, n)
    fetch_field!(f) = riv_check(ccall((:wf_li_river_get, LIB), Int32, (Ptr{Cvoid}, Int32, Ptr{Float64}), gpu.handle,
                              Int32(f), f in (2, 3, 4) ? qbuf : tmp), gpu.handle, "wf_li_river_get")
    qbuf = similar(v.q)
    fetch_field!(0); v.h .= tmp[1:length(v.h)]
    fetch_field!(1); v.storage .= tmp[1:length(v.storage)]
    fetch_field!(5); v.error .= tmp[1:length(v.error)]
    fetch_field!(6); bc.actual_external_abstraction_cumulative .= tmp[1:length(bc.actual_external_abstraction_cumulative)]
    bc.actual_external_abstraction_average .= bc.actual_external_abstraction_cumulative ./ dt
    fetch_field!(2); v.q .= qbuf
    fetch_field!(3); v.q_cumulative .= qbuf
    fetch_field!(4); v.q_average .= qbuf
    return nothing
end

end # module
