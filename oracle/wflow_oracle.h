/*
 * wflow_oracle.h -- C ABI of the CPU oracle (FP64 restatement of Wflow.jl's SBM +
 * kinematic-wave step).
 *
 * TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / --impl reference leg as the checker. The product library never links it.
 *
 * The oracle consumes the same input description as the product (include/wflow_gb300.h)
 * and follows the reference functions line by line; every function in wflow_oracle.cpp
 * cites the Wflow.jl file:line it restates.
 */
#ifndef WFLOW_ORACLE_H
#define WFLOW_ORACLE_H

#include <stdint.h>

#include "../include/wflow_gb300.h"
#include "../include/wflow_gb300_li.h"

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAXL WF_MAX_LAYERS

/* One SBM soil column: parameters, boundary conditions and variables of SbmSoilModel
 * (soil/soil.jl:3-211) for a single cell. Field names follow the reference. */
typedef struct OrcSoil {
    int32_t maximum_number_of_layers;
    int32_t number_of_layers;
    int32_t n_unsatlayers;
    int32_t kv_profile; /* WfKvProfile */
    /* parameters */
    double theta_s, theta_r, theta_fc, soil_water_capacity;
    double kv_0, f, z_exp, air_entry_pressure;
    double h1, h2, h3_high, h3_low, h4, alpha_h1;
    double soil_thickness;
    double infiltration_capacity_soil, infiltration_capacity_compacted_soil;
    double compacted_soil_area_fraction, wet_root_distribution_parameter;
    double cap_hmax, cap_n, maximum_leakage, w_soil, cf_soil;
    double rooting_depth, soil_fraction;
    double actual_layer_thickness[ORC_MAXL];
    double cumulative_layer_depth[ORC_MAXL + 1];
    double brooks_corey_exponent[ORC_MAXL];
    double kv_factor[ORC_MAXL];
    double rootfraction[ORC_MAXL];
    /* boundary conditions */
    double water_flux_surface, potential_transpiration, potential_soilevaporation;
    /* variables */
    double unsaturated_layer_depth[ORC_MAXL];
    double unsaturated_layer_thickness[ORC_MAXL];
    double volumetric_water_content[ORC_MAXL];
    double relative_volumetric_water_content[ORC_MAXL];
    double h3, unsaturated_store_capacity, saturated_water_depth, drainable_water_depth;
    double water_table_depth, transpiration, actual_evaporation_unsaturated_store;
    double soil_evaporation, soil_evaporation_saturated_zone, actual_capillary_flux;
    double actual_evaporation_saturated_zone, actual_evapotranspiration, actual_infiltration;
    double actual_infiltration_soil, actual_infiltration_compacted_soil, infiltration;
    double infiltration_excess, saturation_excess_water, exfiltration_saturated_water;
    double excess_water_soil, excess_water_compacted_soil, runoff, net_runoff;
    double root_zone_storage, volumetric_water_content_root_zone;
    double relative_volumetric_water_content_root_zone, unsaturated_store_depth, transfer;
    double recharge, actual_leakage, total_soil_water_storage, soil_surface_temperature;
    double f_infiltration_reduction;
} OrcSoil;

/* layout of OrcSoil for the ctypes mirror: "name:offset:kind;..." (kind i=int32, d=double, aN=array) */
const char* orc_soil_layout(void);
int32_t orc_soil_sizeof(void);

/* elementary functions (oracle_math.h) */
double orc_exp(double x);
double orc_log(double x);
double orc_cbrt(double x);
double orc_pow(double x, double y);
double orc_cld(double x, double y);
double orc_round_sigdigits(double x, int32_t d);

/* process functions; out arrays receive the reference's return tuple in order */
void orc_rainfall_interception_gash(double cmax, double e_r, double gap, double p, double cs,
                                    double max_evap, double dt, double* out4);
void orc_rainfall_interception_modrut(double p, double pet, double cs, double gap, double cmax,
                                      double dt, double* out4);
void orc_precipitation_hbv(double p, double t, double tti, double tt, double* out2);
void orc_snowpack_hbv(double ss, double sw, double sp, double lp, double t, double ttm, double cfmax,
                      double whc, double dt, double* out5);
void orc_glacier_hbv(double gfrac, double gstore, double ss, double t, double g_ttm, double g_cfmax,
                     double g_sifrac, double max_snow_to_glacier, double dt, double* out4);
void orc_infiltration(double pot, double cfrac, double cap_soil, double cap_comp, double ucap,
                      double fred, double dt, double* out2);
void orc_unsatzone_flow_layer(double usd, double kv_z, double l_sat, double c, double dt, double* out2);
double orc_head_brooks_corey(double vwc, double ts, double tr, double c, double psi);
double orc_vwc_brooks_corey(double h, double psi, double ts, double tr, double c);
double orc_feddes_h3(double h3h, double h3l, double tpot);
double orc_rwu_reduction_feddes(double h, double h1, double h2, double h3, double h4, double a);
double orc_soil_temperature(double tsoil_prev, double w_soil, double t);
double orc_infiltration_reduction_factor(double tsoil, double cf, int32_t modelsnow, int32_t flag);
double orc_soil_evaporation_unsaturated_store(double pot, double usld, double ulthick, int32_t nunsat,
                                              double zi, double theta_e);
double orc_soil_evaporation_saturated_store(double pot, int32_t nunsat, double lthick, double zi,
                                            double theta_d, double dt);
void orc_actual_infiltration_soil_path(double pot, double act, double cfrac, double cap_soil,
                                       double cap_comp, double fred, double* out2);
double orc_scurve(double x, double a, double b, double c);
void orc_compute_mass_balance_error(double tin, double tout, double rate, double* out2);
void orc_kinematic_wave(double qin, double qprev, double qlat, double alpha, double dt, double dx,
                        double* out2);
double orc_ssf_celerity(double zi, double slope, double sy, double kh0, double f, int32_t profile,
                        double z_exp);
double orc_kw_ssf_newton_raphson(double q, double c, double cel, double dt, double dx);
/* soil-column functions (soil.jl, utils.jl) on one OrcSoil */
void orc_update_bc_soil_model(OrcSoil* s, double canopy_potevap, double interception_rate,
                              double pet, double wfs_runoff, double runoff_river, double runoff_land);
void orc_unsaturated_zone_flow(OrcSoil* s, double dt);
void orc_soil_evaporation(OrcSoil* s, double dt);
void orc_transpiration(OrcSoil* s, double dt);
void orc_capillary_flux(OrcSoil* s, double dt);
void orc_update_soil_water_storage(OrcSoil* s, double exfilt_avg, double runoff_land, double ae_land,
                                   double dt);
void orc_water_table_change(const OrcSoil* s, double net_flux, double sy, double dt, double* out2);
/* kinematic_wave_ssf (subsurface_process.jl:89-172); out4 = q, zi, exfilt, net_flux */
void orc_kinematic_wave_ssf(double q_in, double q_prev, double zi_prev, double q_net, double slope,
                            double sy, double d, double dt, double dx, double dw, double q_max,
                            double kh0, double f, int32_t profile, double z_exp, OrcSoil* s,
                            double* out4);
/* stable_timestep of a kinematic-wave flow model (surface_kinwave.jl:674-704) */
double orc_kinwave_stable_timestep(const double* q, const double* alpha, const double* flow_length,
                                   int64_t n, double p);
double orc_quantile(double* v, int64_t n, double p);

/* capacity-limited transport over a drainage graph (routing/utils.jl:82-110) and the lateral
 * snow transport built on it (routing/surface/surface_process.jl:1-19), which moves the snow
 * storage and snow water in place (accucapacityflux hands its material to accucapacityflux!,
 * routing/utils.jl:144-148) */
void orc_accucapacityflux(const int32_t* ds, const int64_t* order, int64_t n, double dt, const double* capacity,
                          double* material, double* flux);
/* Graphs.jl topological_sort_by_dfs of a graph of out-degree <= 1 (Wflow's network.order):
 * the order in which the model's snow transport hands material on. 0, or -3 on a cycle. */
int32_t orc_topo_order_dfs(int64_t n, const int32_t* ds, int64_t* order);
void orc_lateral_snow_transport(const int32_t* ds, const int32_t* ups_ds, const int64_t* order, int64_t n, double dt,
                                const double* slope, double* snow_storage, double* snow_water, double* snow_out,
                                double* snow_in);

/* local-inertial river flow on a staggered grid (surface_process.jl:88-163,
 * surface_staggered_scheme.jl:326-385, 723-760, 1004-1020) */
double orc_li_flow_area(double q0, double zs0, double zs1, double hf, double A, double R, double length,
                        double mannings_n_sq, int32_t froude_limit, double dt);
double orc_li_flow_rect(double theta, double q0, double qd, double qu, double zs0, double zs1, double hf,
                        double width, double length, double mannings_n_sq, int32_t froude_limit, double dt);
void orc_li_river_step(int64_t n, int64_t n_active, int64_t n_edges, const int64_t* src, const int64_t* dst,
                       const double* zb, const double* flow_length, const double* flow_width, const double* inwater,
                       const double* zb_e, const double* width_e, const double* length_e, const double* nsq_e,
                       double h_thresh, int32_t froude_limit, double dt, double* h, double* storage, double* q,
                       double* q_prev, double* q_cum, const double* abstraction, const double* external_inflow,
                       double* error, double* abstraction_cum);
double orc_li_stable_timestep(int64_t n, const double* flow_length, const double* h, double alpha);
/* Manning's equation on the staggered grid (river_routing = "manning_staggered",
 * surface_staggered_scheme.jl:386-434, 1050-1075): one sub-step (edge discharges from the
 * upstream depth, limited to the upstream storage over dt; hf_e keeps each edge's depth), and
 * the stable sub-step from the edges' last depths. */
void orc_manning_river_step(int64_t n, int64_t n_active, int64_t n_edges, const int64_t* src, const int64_t* dst,
                            const double* flow_length, const double* flow_width, const double* inwater,
                            const double* width_e, const double* slope_e, const double* n_e, double h_thresh,
                            double dt, double* h, double* storage, double* q, double* q_cum, double* hf_e,
                            const double* abstraction, const double* external_inflow, double* error,
                            double* abstraction_cum);
double orc_manning_stable_timestep(int64_t n_edges, const double* width_e, const double* length_e,
                                   const double* slope_e, const double* n_e, const double* hf_e, double alpha);
/* 2D overland local-inertial flow with a subgrid river (surface_staggered_scheme.jl:1022-1040,
 * 1202-1265, 1322-1546); 0-based indices, index n = the ghost cell outside the grid */
double orc_li_land_stable_timestep(int64_t n, const double* x_length, const double* y_length,
                                   const int32_t* river_location, const double* h, double alpha);
void orc_li_directional_flow(int64_t i, int64_t n, const int64_t* up, const int64_t* down, const double* width_e,
                             const double* zmax_e, const double* length, const double* z, const double* h,
                             const double* nsq_e, double theta, double h_thresh, int32_t froude_limit, double dt,
                             double* q, const double* q_prev, double* q_cum);
double orc_li_land_storage_change(int64_t i, const double* qx, const double* qy, const int64_t* ind_x_down,
                                  const int64_t* ind_y_down, const double* runoff, double dt);
double orc_li_river_storage_change(int64_t i, const double* q_river, const int64_t* e_in, int64_t n_in,
                                   const int64_t* e_out, int64_t n_out, const double* qx, const double* qy,
                                   const int64_t* ind_x_down, const int64_t* ind_y_down, const double* runoff,
                                   double abstraction, double dt);
void orc_li_external_inflow(double external_inflow, double land_storage, double bankfull_storage,
                            double river_storage, double dt, double* out2);
void orc_li_water_depths(double total_storage, double bankfull_storage, double bankfull_depth, double x_length,
                         double y_length, double river_length, double river_width, double* out3);
void orc_li_update_land_cell(int64_t i, const double* qx, const double* qy, const int64_t* ind_x_down,
                             const int64_t* ind_y_down, const double* runoff, const double* x_length,
                             const double* y_length, double dt, double* storage, double* error, double* h);
void orc_li_update_river_cell(int64_t i, const double* q_river, const int64_t* e_in, int64_t n_in,
                              const int64_t* e_out, int64_t n_out, const double* qx, const double* qy,
                              const int64_t* ind_x_down, const int64_t* ind_y_down, const double* runoff,
                              double abstraction, double external_inflow, double bankfull_storage,
                              double bankfull_depth, const double* x_length, const double* y_length,
                              double river_length, double river_width, double dt, double* storage, double* error,
                              double* h_land, double* h_river, double* storage_river,
                              double* abstraction_cumulative);
/* The coupled land + river local-inertial scheme over the product's input description
 * (include/wflow_gb300_li.h): the state arrays of one domain; qx, qy, qx0, qy0, qx_cum, qy_cum
 * hold n + 1 values (the last, outside the grid, stays 0). */
typedef struct OrcLiState {
    double *h_land, *storage, *error, *qx, *qy, *qx0, *qy0, *qx_cum, *qy_cum;
    double *h_river, *storage_river, *q, *q_prev, *q_cum, *abstraction_cum;
} OrcLiState;
/* One sub-step (the loop body of update_overland_flow_model!, surface_staggered_scheme.jl:
 * 1170-1183, without reservoirs): land fluxes, river edges, then the depths of every land cell. */
void orc_li_domain_substep(const WfLiLandGrid* land, const WfLiRiverNetwork* river, const double* runoff,
                           const double* external_inflow, const double* abstraction, double dt, OrcLiState* st);
/* min(river, land) stable time step, each 60 s when infinite (:1171-1174); the river's over its
 * active cells (parameters.n, without the ghost cells), the land's over cells without a river */
double orc_li_domain_stable_timestep(const WfLiLandGrid* land, const WfLiRiverNetwork* river, const OrcLiState* st);

/* full model */
typedef struct OrcModel OrcModel;
int32_t orc_model_create(const WfConfig* c, const WfDomain* d, const WfParams* p, OrcModel** out);
/* Per member, the sum of the squared sub-step sizes of the last model step (kind 0 subsurface,
 * 1 land, 2 river). */
int32_t orc_model_substep_signature(OrcModel* m, int32_t kind, double* out);
/* the same with reservoirs (reservoir outlets cut the land and river upstream lists) */
int32_t orc_model_create_with_reservoirs(const WfConfig* c, const WfDomain* d, const WfParams* p,
                                         const WfReservoirs* rs, OrcModel** out);
int64_t orc_model_reservoirs(const OrcModel* m);
/* the same with the reservoirs' S-H and H-Q tables and links (tables may be NULL) */
int32_t orc_model_create_with_reservoir_tables(const WfConfig* c, const WfDomain* d, const WfParams* p,
                                               const WfReservoirs* rs, const WfReservoirTables* tables,
                                               OrcModel** out);
/* the H-Q tables' column (day of year 1..365, col_index_hq) of the next steps */
int32_t orc_model_set_rating_curve_day(OrcModel* m, int32_t day);
/* Route the land grid with its river by the local-inertial scheme inside the step, in place of
 * the kinematic waves (surface_routing.jl:62-89): one member, no reservoirs, fixed sub-steps;
 * the grid's land and active river cells are the model's. Warm state h_land [n], h_river [river n]. */
int32_t orc_model_attach_li(OrcModel* m, const WfLiLandGrid* land, const WfLiRiverNetwork* river,
                            const double* h_land, const double* h_river);
/* A WfLiDomainField of the coupled scheme; field -1: the sub-steps of the last step. */
int32_t orc_model_li_get(OrcModel* m, int32_t field, double* out);
void orc_model_destroy(OrcModel* m);
const char* orc_model_error(const OrcModel* m);
int32_t orc_model_set_forcing(OrcModel* m, const double* P, const double* PET, const double* T);
int32_t orc_model_step(OrcModel* m, int32_t n_threads);
int32_t orc_model_get(OrcModel* m, int32_t field, int32_t layer, double* out);
int32_t orc_model_set(OrcModel* m, int32_t field, int32_t layer, const double* in);
int32_t orc_model_outlets(OrcModel* m, int32_t which, double* out, int64_t* n);
/* sub-step counts of the last step */
int32_t orc_model_substeps(OrcModel* m, int64_t* land, int64_t* river, int64_t* subsurface);

#ifdef __cplusplus
}
#endif

#endif
