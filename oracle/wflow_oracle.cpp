/*
 * wflow_oracle.cpp -- CPU FP64 restatement of Wflow.jl's `sbm` hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker). Follows, line by line:
 *   vegetation/rainfall_interception.jl:9-130, vegetation/canopy.jl:184-300,
 *   snow/snow_process.jl:26-116, snow/snow.jl:238-293, surfacewater/runoff.jl:36-111,
 *   soil/soil.jl:643-1436, soil/soil_process.jl:16-323, utils.jl:27-30,390-409,470-477,
 *   727-761,916-979,1070-1136, routing/subsurface/lateral_subsurface_flow.jl:174-402,
 *   routing/subsurface/subsurface_process.jl:1-172, routing/subsurface/boundary_conditions.jl:
 *   12-21,219-236, routing/subsurface/groundwater.jl:613-695, routing/surface/surface_process.jl:
 *   24-70, routing/surface/surface_kinwave.jl:32-44,67-86,292-385,491-566,613-766,
 *   routing/timestepping.jl:11-16, sbm.jl:82-182, sbm_model.jl:60-92, mass_balance.jl:84-549,
 *   domain.jl:218-347.
 * The drainage graphs are swept in one topological order (the 1-thread semantics of
 * subdomains.jl:248-252); upstream sums run in ascending node order with a left fold from
 * 0.0, as sum_at (utils.jl:472-477) over Graphs.inneighbors does.
 * Compiled with -ffp-contract=off.
 */
#include "wflow_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <string>
#include <vector>

#include "oracle_math.h"

using namespace orc;

namespace {

const double MISSING = NAN;                                  // MISSING_VALUE, Wflow.jl:192
const double KIN_WAVE_MIN_FLOW = 1e-30;                      // routing/utils.jl:1
const double KIN_WAVE_MIN_FLOW_QROOT = 0x1.0c6f7a0b5ed8ap-20; // 1e-30^0.2, routing/utils.jl:2
const double BETA_KINWAVE = 0.6;                             // surface_kinwave.jl:2
// Unit factors of Wflow's unit system (units.jl:55-118): mm/d and percentage.
const double MM_PER_DAY_FACTOR = (1.0 / 86400.0) * 1e-3;
const double PERCENTAGE_FACTOR = 1e-2;
const double ABSOLUTE_ZERO_C = 273.15;  // to_SI(0.0, ABSOLUTE_DEGREES)

inline bool is_approx_zero(double x) { return x == 0.0; }  // isapprox(x, 0.0), default tolerances

// ---------------------------------------------------------------- process functions ----

// vegetation/rainfall_interception.jl:9-70
void rainfall_interception_gash(double cmax, double e_r, double gap, double precipitation,
                                double canopy_storage, double max_evaporation, double dt,
                                double* out) {
    double throughfall, interception, stem_flow;
    if (cmax > 0.0) {
        double fraction_stemflow, fraction_interception, precipitation_saturation;
        if (gap < 1.0 / 1.1) {
            fraction_stemflow = 0.1 * gap;
            fraction_interception = 1.0 - 1.1 * gap;
            if (e_r > fraction_interception) {
                precipitation_saturation = 0.0;
            } else {
                precipitation_saturation =
                    -cmax / (e_r * dt) * wlog(1.0 - e_r / fraction_interception);
            }
        } else {
            fraction_stemflow = 1.0 - gap;
            fraction_interception = 0.0;
            precipitation_saturation = 0.0;
        }
        bool large_storms = precipitation > precipitation_saturation;
        if (large_storms) {
            double iwet = fraction_interception * precipitation_saturation - cmax / dt;
            double isat = e_r * (precipitation - precipitation_saturation);
            double idry = cmax / dt;
            interception = iwet + isat + idry;
        } else {
            double iwet = fraction_interception * precipitation;
            interception = iwet;
        }
        stem_flow = fraction_stemflow * precipitation;
        throughfall = precipitation - interception - stem_flow;
        if (interception > max_evaporation) {
            double canopy_drainage = interception - max_evaporation;
            interception = max_evaporation;
            throughfall += canopy_drainage;
        }
    } else {
        throughfall = precipitation;
        interception = 0.0;
        stem_flow = 0.0;
    }
    out[0] = throughfall;
    out[1] = interception;
    out[2] = stem_flow;
    out[3] = canopy_storage;
}

// vegetation/rainfall_interception.jl:78-130
void rainfall_interception_modrut(double precipitation, double potential_evaporation,
                                  double canopy_storage, double gap, double cmax, double dt,
                                  double* out) {
    double fraction_stemflow, precipitation_canopy;
    if (gap < 1.0 / 1.1) {
        fraction_stemflow = 0.1 * gap;
        precipitation_canopy = (1.0 - gap - fraction_stemflow) * precipitation;
    } else {
        fraction_stemflow = 1.0 - gap;
        precipitation_canopy = 0.0;
    }
    double stemflow = fraction_stemflow * precipitation;
    double throughfall = gap * precipitation;
    if (canopy_storage > cmax) {
        double canopy_drainage = canopy_storage - cmax;
        canopy_storage = cmax;
        throughfall += canopy_drainage / dt;
    }
    canopy_storage += precipitation_canopy * dt;
    double max_evaporation = canopy_storage / dt;
    double canopy_evaporation;
    if (potential_evaporation > max_evaporation) {
        canopy_evaporation = max_evaporation;
        canopy_storage = 0.0;
    } else {
        canopy_evaporation = potential_evaporation;
        canopy_storage -= canopy_evaporation * dt;
    }
    if (canopy_storage > cmax) {
        double canopy_drainage = canopy_storage - cmax;
        canopy_storage = cmax;
        throughfall += canopy_drainage / dt;
    }
    out[0] = throughfall;
    out[1] = canopy_evaporation;
    out[2] = stemflow;
    out[3] = canopy_storage;
}

// snow/snow_process.jl:90-116
void precipitation_hbv(double precipitation, double temperature, double tti, double tt, double* out) {
    double rainfrac;
    if (tti == 0.0) {
        rainfrac = temperature > tt ? 1.0 : 0.0;
    } else {
        double frac = (temperature - (tt - tti / 2.0)) / tti;
        rainfrac = jclamp(frac, 0.0, 1.0);
    }
    double snowfrac = 1.0 - rainfrac;
    out[0] = snowfrac * 1.0 * precipitation;
    out[1] = rainfrac * 1.0 * precipitation;
}

// snow/snow_process.jl:26-70
void snowpack_hbv(double snow_storage, double snow_water, double snow_precip, double liquid_precip,
                  double temperature, double ttm, double cfmax, double whc, double dt, double* out) {
    const double cfr = 0.05;
    double snow_melt;
    if (temperature > ttm) {
        double potential_snow_melt = cfmax * (temperature - ttm);
        snow_melt = jmin(potential_snow_melt, snow_storage / dt);
        snow_storage -= snow_melt * dt;
        snow_water += snow_melt * dt;
    } else {
        snow_melt = 0.0;
        double potential_refreezing = cfmax * cfr * (ttm - temperature);
        double refreezing = jmin(potential_refreezing * dt, snow_water);
        snow_storage += refreezing;
        snow_water -= refreezing;
    }
    snow_storage = jmax(snow_storage, 0.0);
    snow_water = jmax(snow_water, 0.0);
    snow_storage += snow_precip * dt;
    snow_water += liquid_precip * dt;
    double max_snow_water = snow_storage * whc;
    double runoff;
    if (snow_water > max_snow_water) {
        runoff = (snow_water - max_snow_water) / dt;
        snow_water = max_snow_water;
    } else {
        runoff = 0.0;
    }
    double swe = snow_water + snow_storage;
    out[0] = snow_storage;
    out[1] = snow_water;
    out[2] = swe;
    out[3] = snow_melt;
    out[4] = runoff;
}

// glacier/glacier_process.jl:27-62 (glacier is off on the path; kept for the unit KAT)
void glacier_hbv(double gfrac, double gstore, double snow_storage, double temperature, double ttm,
                 double cfmax, double sifrac, double max_rate, double dt, double* out) {
    double snow_to_glacier = gfrac > 0.0 ? sifrac * snow_storage : 0.0;
    snow_to_glacier = jmin(snow_to_glacier, max_rate);
    snow_storage -= snow_to_glacier * gfrac * dt;
    gstore += snow_to_glacier * dt;
    double potential_melt = temperature > ttm ? cfmax * (temperature - ttm) : 0.0;
    double glacier_melt = snow_storage < 1e-2 ? jmin(potential_melt, gstore / dt) : 0.0;
    gstore -= glacier_melt * dt;
    out[0] = snow_storage;
    out[1] = snow_to_glacier;
    out[2] = gstore;
    out[3] = glacier_melt;
}

// soil/soil_process.jl:16-41
void infiltration_fn(double potential_infiltration, double cfrac, double cap_soil, double cap_comp,
                     double ucap, double fred, double dt, double* out) {
    double soilinf = potential_infiltration * (1.0 - cfrac);
    double pathinf = potential_infiltration * cfrac;
    double max_infiltsoil = jmin(cap_soil * fred, soilinf);
    double max_infiltpath = jmin(cap_comp * fred, pathinf);
    double infiltration = jmin(max_infiltpath + max_infiltsoil, jmax(0.0, ucap / dt));
    double infiltration_excess = (soilinf - max_infiltsoil) + (pathinf - max_infiltpath);
    out[0] = infiltration;
    out[1] = infiltration_excess;
}

// utils.jl:1070-1076
inline double bounded_power(double base, double power) { return base > 1.0 ? 1.0 : jpow(base, power); }

// soil/soil_process.jl:51-92
void unsatzone_flow_layer(double usd, double kv_z, double l_sat, double c, double dt, double* out) {
    if (usd <= 0.0) {
        out[0] = 0.0;
        out[1] = 0.0;
        return;
    }
    double st_sat = jmax(0.0, usd - l_sat);
    double st = kv_z * bounded_power(usd / l_sat, c);
    double sum_ast = jmin(st, st_sat / dt);
    usd -= sum_ast * dt;
    double remainder = jmin((st - sum_ast) * dt, usd);
    long its = (long)jcld(remainder, 2e-4);
    for (long i = 0; i < its; ++i) {
        st = (kv_z / (double)its) * bounded_power(usd / l_sat, c);
        double st_max = usd / dt;
        if (st < st_max) {
            usd -= st * dt;
            sum_ast += st;
        } else {
            usd = 0.0;
            sum_ast += st_max;
            break;
        }
    }
    out[0] = usd;
    out[1] = sum_ast;
}

// soil/soil_process.jl:99-106
double vwc_brooks_corey(double h, double psi, double ts, double tr, double c) {
    if (h < psi) {
        double par_lambda = 2.0 / (c - 3.0);
        return (ts - tr) * jpow(psi / h, par_lambda) + tr;
    }
    return ts;
}

// soil/soil_process.jl:113-130
double head_brooks_corey(double vwc, double ts, double tr, double c, double psi) {
    double par_lambda = 2.0 / (c - 3.0);
    if (par_lambda > 0.0) return psi / jpow(vwc / (ts - tr), 1.0 / par_lambda);
    return psi;
}

// soil/soil_process.jl:137-159
double field_capacity(const double* thickness, int n_layers, double ts, double tr, const double* c,
                      double psi) {
    double theta_fc = 0.0, total_depth = 0.0;
    for (int i = 0; i < n_layers; ++i) {
        theta_fc += vwc_brooks_corey(-1.0, psi, ts, tr, c[i]) * thickness[i];
        total_depth += thickness[i];
    }
    return theta_fc / total_depth;
}

// soil/soil_process.jl:166-176
double feddes_h3(double h3_high, double h3_low, double tpot_SI) {
    double tpot_daily = tpot_SI / MM_PER_DAY_FACTOR;
    if (tpot_daily <= 1.0) return h3_low;
    if (tpot_daily < 5.0) return h3_low + (h3_high - h3_low) * (tpot_daily - 1.0) / (5.0 - 1.0);
    return h3_high;
}

// soil/soil_process.jl:183-200
double rwu_reduction_feddes(double h, double h1, double h2, double h3, double h4, double alpha_h1) {
    if (h < h4) return 0.0;
    if (h < h3) return (h - h4) / (h3 - h4);
    if (alpha_h1 == 0.0) {
        if (h < h2) return 1.0;
        if (h < h1) return (h1 - h) / (h1 - h2);
        return 0.0;
    }
    return 1.0;
}

// soil/soil_process.jl:210-213
double soil_temperature(double tsoil_prev, double w_soil, double temperature) {
    return tsoil_prev + w_soil * (temperature - tsoil_prev);
}

// utils.jl:27-30
double scurve(double x, double a, double b, double c) { return 1.0 / (b + wexp(-c * (x - a))); }

// soil/soil_process.jl:229-244
double infiltration_reduction_factor(double tsoil, double cf, bool modelsnow, bool flag) {
    if (modelsnow && flag) {
        double bb = 1.0 / (1.0 - cf);
        return scurve(tsoil, ABSOLUTE_ZERO_C, bb, 8.0) + cf;
    }
    return 1.0;
}

// soil/soil_process.jl:247-271
double soil_evaporation_unsaturated_store(double pot, double usld, double ulthick, int nunsat,
                                          double zi, double theta_e) {
    if (nunsat == 0) return 0.0;
    if (nunsat == 1) return pot * jmin(1.0, usld / (zi * theta_e));
    return pot * jmin(1.0, usld / (ulthick * theta_e));
}

// soil/soil_process.jl:274-294
double soil_evaporation_saturated_store(double pot, int nunsat, double lthick, double zi,
                                        double theta_d, double dt) {
    if (nunsat == 0 || nunsat == 1) {
        double e = pot * jmin(1.0, (lthick - zi) / lthick);
        return jmin(e, (lthick - zi) * theta_d / dt);
    }
    return 0.0;
}

// soil/soil_process.jl:297-323
void actual_infiltration_soil_path(double pot, double act, double cfrac, double cap_soil,
                                   double cap_comp, double fred, double* out) {
    double soilinf = pot * (1.0 - cfrac);
    double pathinf = pot * cfrac;
    if (act > 0.0) {
        double max_infiltsoil = jmin(cap_soil * fred, soilinf);
        double max_infiltpath = jmin(cap_comp * fred, pathinf);
        out[0] = act * max_infiltsoil / (max_infiltpath + max_infiltsoil);
        out[1] = act * max_infiltpath / (max_infiltpath + max_infiltsoil);
    } else {
        out[0] = 0.0;
        out[1] = 0.0;
    }
}

// mass_balance.jl:84-93
void compute_mass_balance_error(double total_in, double total_out, double storage_rate, double* out) {
    double error = total_in - total_out - storage_rate;
    double average_flow_rate = (total_in + total_out) / 2.0;
    out[0] = error;
    out[1] = average_flow_rate == 0.0 ? 0.0 : error / average_flow_rate;
}

// routing/surface/surface_process.jl:24-70
void kinematic_wave(double q_in, double q_prev, double q_lat, double alpha, double dt, double dx,
                    double* out) {
    if (is_approx_zero(q_in + q_prev + q_lat)) {
        out[0] = 0.0;
        out[1] = 0.0;
        return;
    }
    double dt_dx = dt / dx;
    double u_prev = q_prev >= 0.0 ? jpow(q_prev, 0.2) : 0.0;
    double constant_term = dt_dx * q_in + alpha * u_prev * u_prev * u_prev + dt * q_lat;
    double u = u_prev > 0.0 ? u_prev : wcbrt(constant_term / alpha);
    const int max_iters = 3000;
    const double epsilon = 1.0e-12;
    double const_1 = 5.0 * dt_dx;
    double const_2 = 3.0 * alpha;
    for (int it = 0; it < max_iters; ++it) {
        double u2 = u * u;
        double u3 = u2 * u;
        double f_u = u3 * (dt_dx * u2 + alpha) - constant_term;
        if (std::fabs(f_u) <= epsilon) break;
        double df_u = u2 * (const_1 * u2 + const_2);
        u -= f_u / df_u;
        if (std::isnan(u) || u <= 0.0) u = KIN_WAVE_MIN_FLOW_QROOT;
    }
    u = jmax(u, KIN_WAVE_MIN_FLOW_QROOT);
    double u3 = u * u * u;
    double crossarea = alpha * u3;
    double q = u3 * u * u;
    out[0] = q;
    out[1] = crossarea;
}

// routing/subsurface/subsurface_process.jl:6-41 (KhExponential, KhExponentialConstant)
double ssf_celerity(double zi, double slope, double sy, double kh0, double f, int profile, double z_exp) {
    double z = zi;
    if (profile == WF_KV_EXPONENTIAL_CONSTANT) z = zi < z_exp ? zi : z_exp;
    return (kh0 * wexp(-f * z) * slope) / sy;
}

// routing/subsurface/subsurface_process.jl:57-78
double kw_ssf_newton_raphson(double q, double constant_term, double celerity, double dt, double dx) {
    const double epsilon = 1.0e-12;
    const int max_iters = 3000;
    int count = 0;
    double dt_dx = dt / dx;
    double celerity_inv = 1.0 / celerity;
    double df = dt_dx + celerity_inv;
    while (true) {
        double fq = dt_dx * q + celerity_inv * q - constant_term;
        q -= (fq / df);
        if (std::isnan(q)) q = 0.0;
        q = jmax(q, KIN_WAVE_MIN_FLOW);
        if ((std::fabs(fq) <= epsilon) || (count >= max_iters)) break;
        count += 1;
    }
    return q;
}

// --------------------------------------------------------------- soil column --------

// utils.jl:390-404 (cum depth has N+1 entries, thickness N)
void set_layerthickness(double reference_depth, const double* cum_depth, const double* thickness, int N,
                        double* out) {
    for (int i = 0; i < N; ++i) {
        double t = thickness[i] * MISSING;
        if (reference_depth > cum_depth[i + 1]) {
            t = thickness[i];
        } else if (reference_depth - cum_depth[i] > 0.0) {
            t = reference_depth - cum_depth[i];
        }
        out[i] = t;
    }
}

// utils.jl:406-409
int number_of_active_layers(const double* thickness, int N) {
    int n = N;
    for (int i = 0; i < N; ++i)
        if (std::isnan(thickness[i])) n -= 1;
    return n;
}

// utils.jl:1134-1136
inline double lower_bound_drainable_porosity(double ts, double tfc) { return jmax(ts - tfc, 0.02); }

// utils.jl:727-761 (KvExponential, KvExponentialConstant); n is 1-based layer index
double kv_at_depth(const OrcSoil& s, double z, int n) {
    double zz = z;
    if (s.kv_profile == WF_KV_EXPONENTIAL_CONSTANT && !(z < s.z_exp)) zz = s.z_exp;
    return s.kv_factor[n - 1] * s.kv_0 * wexp(-s.f * zz);
}

// soil/soil.jl:1400-1436 (with unsaturated_store_depth!, soil.jl:700-708)
void update_diagnostic_vars(OrcSoil& s) {
    int N = s.maximum_number_of_layers;
    double usd = 0.0;
    for (int k = 0; k < s.number_of_layers; ++k) usd += s.unsaturated_layer_depth[k];
    s.unsaturated_store_depth = usd;
    s.water_table_depth = jmax(0.0, s.soil_thickness - s.saturated_water_depth / (s.theta_s - s.theta_r));
    s.drainable_water_depth =
        (s.soil_thickness - s.water_table_depth) * lower_bound_drainable_porosity(s.theta_s, s.theta_fc);
    s.unsaturated_store_capacity = s.soil_water_capacity - s.saturated_water_depth - s.unsaturated_store_depth;
    set_layerthickness(s.water_table_depth, s.cumulative_layer_depth, s.actual_layer_thickness, N,
                       s.unsaturated_layer_thickness);
    s.n_unsatlayers = number_of_active_layers(s.unsaturated_layer_thickness, N);
    s.total_soil_water_storage = s.saturated_water_depth + s.unsaturated_store_depth;
}

// soil/soil.jl:764-804
void unsaturated_zone_flow(OrcSoil& s, double dt) {
    if (s.n_unsatlayers > 0) {
        double z[ORC_MAXL];
        double acc = 0.0;
        for (int k = 0; k < s.maximum_number_of_layers; ++k) {
            acc += s.unsaturated_layer_thickness[k];
            z[k] = acc;
        }
        double flow_rate = 0.0;
        for (int m = 1; m <= s.n_unsatlayers; ++m) {
            double l_sat = s.unsaturated_layer_thickness[m - 1] * (s.theta_s - s.theta_r);
            double kv_z = kv_at_depth(s, z[m - 1], m);
            double usd = m == 1 ? s.unsaturated_layer_depth[m - 1] + s.infiltration * dt
                                : s.unsaturated_layer_depth[m - 1] + flow_rate * dt;
            double o[2];
            unsatzone_flow_layer(usd, kv_z, l_sat, s.brooks_corey_exponent[m - 1], dt, o);
            flow_rate = o[1];
            s.unsaturated_layer_depth[m - 1] = o[0];
        }
        s.transfer = flow_rate;
    } else {
        s.transfer = 0.0;
    }
}

// soil/soil.jl:814-856
void soil_evaporation(OrcSoil& s, double dt) {
    double potsoilevap = s.potential_soilevaporation;
    double soilevapunsat = soil_evaporation_unsaturated_store(
        potsoilevap, s.unsaturated_layer_depth[0], s.unsaturated_layer_thickness[0], s.n_unsatlayers,
        s.water_table_depth, s.theta_s - s.theta_r);
    soilevapunsat = jmin(soilevapunsat, s.unsaturated_layer_depth[0] / dt);
    potsoilevap -= soilevapunsat;
    s.unsaturated_layer_depth[0] = s.unsaturated_layer_depth[0] - soilevapunsat * dt;
    double theta_drainable = lower_bound_drainable_porosity(s.theta_s, s.theta_fc);
    double esat = soil_evaporation_saturated_store(potsoilevap, s.n_unsatlayers, s.actual_layer_thickness[0],
                                                   s.water_table_depth, theta_drainable, dt);
    s.soil_evaporation_saturated_zone = esat;
    s.soil_evaporation = soilevapunsat + esat;
    s.drainable_water_depth -= esat * dt;
}

// soil/soil.jl:865-975
void transpiration(OrcSoil& s, double dt) {
    double rd = s.rooting_depth;
    s.h3 = feddes_h3(s.h3_high, s.h3_low, s.potential_transpiration);
    int nu = s.n_unsatlayers;
    double sum_rootfraction_unsat = 0.0;
    double rootfraction_unsat_lowest = 0.0;
    for (int k = 1; k <= nu; ++k) {
        double rfu;
        if (k == nu && s.water_table_depth < rd) {
            double rootlength = jmin(s.actual_layer_thickness[k - 1], rd - s.cumulative_layer_depth[k - 1]);
            rfu = s.rootfraction[k - 1] * (s.unsaturated_layer_thickness[k - 1] / rootlength);
        } else {
            rfu = s.rootfraction[k - 1];
        }
        sum_rootfraction_unsat += rfu;
        rootfraction_unsat_lowest = rfu;
    }
    double actevapustore = 0.0;
    for (int k = 1; k <= nu; ++k) {
        double rfu = k < nu ? s.rootfraction[k - 1] : rootfraction_unsat_lowest;
        double rfu_scaled = rd > 0.0 ? jmax(1.0 / sum_rootfraction_unsat, 1.0) * rfu : 0.0;
        double vwc = jmax(s.unsaturated_layer_depth[k - 1] / s.unsaturated_layer_thickness[k - 1], 1e-7);
        double head = head_brooks_corey(vwc, s.theta_s, s.theta_r, s.brooks_corey_exponent[k - 1],
                                        s.air_entry_pressure);
        double alpha = rwu_reduction_feddes(head, s.h1, s.h2, s.h3, s.h4, s.alpha_h1);
        double availcap =
            jmin(1.0, jmax(0.0, (rd - s.cumulative_layer_depth[k - 1]) / s.unsaturated_layer_thickness[k - 1]));
        double maxextr = s.unsaturated_layer_depth[k - 1] * availcap / dt;
        double act = jmin(alpha * rfu_scaled * s.potential_transpiration, maxextr);
        double usld = s.unsaturated_layer_depth[k - 1] - act * dt;
        actevapustore += act;
        s.unsaturated_layer_depth[k - 1] = usld;
    }
    double wetroots = scurve(s.water_table_depth, rd, 1.0, s.wet_root_distribution_parameter);
    double alpha = rwu_reduction_feddes(0.0, s.h1, s.h2, s.h3, s.h4, s.alpha_h1);
    double restpottrans = s.potential_transpiration - actevapustore;
    double act_sat = jmin(restpottrans * wetroots * alpha, s.drainable_water_depth / dt);
    s.actual_evaporation_unsaturated_store = actevapustore;
    s.actual_evaporation_saturated_zone = act_sat;
    s.drainable_water_depth -= act_sat * dt;
    s.transpiration = actevapustore + act_sat;
}

// soil/soil.jl:987-1017
void actual_infiltration(OrcSoil& s, double dt) {
    double excess = 0.0;
    double ts_tr = s.theta_s - s.theta_r;
    for (int k = s.n_unsatlayers; k >= 1; --k) {
        excess = jmax(0.0, s.unsaturated_layer_depth[k - 1] - s.unsaturated_layer_thickness[k - 1] * ts_tr);
        s.unsaturated_layer_depth[k - 1] = s.unsaturated_layer_depth[k - 1] - excess;
        if (k > 1) s.unsaturated_layer_depth[k - 2] = s.unsaturated_layer_depth[k - 2] + excess;
    }
    s.actual_infiltration = s.infiltration - excess / dt;
}

// soil/soil.jl:1050-1111
void capillary_flux(OrcSoil& s, double dt) {
    if (s.n_unsatlayers > 0) {
        double ksat = kv_at_depth(s, s.water_table_depth, s.n_unsatlayers);
        double maxcapflux = jmax(
            0.0, jmin(jmin(jmin(ksat, s.actual_evaporation_unsaturated_store), s.unsaturated_store_capacity / dt),
                      s.drainable_water_depth / dt));
        double capflux;
        if (s.water_table_depth > s.rooting_depth) {
            capflux = maxcapflux * jpow(1.0 - jmin(s.water_table_depth, s.cap_hmax) / s.cap_hmax, s.cap_n);
        } else {
            capflux = 0.0;
        }
        double netcapflux = capflux;
        double actual = 0.0;
        for (int k = s.n_unsatlayers; k >= 1; --k) {
            double toadd = jmin(
                netcapflux,
                jmax((s.unsaturated_layer_thickness[k - 1] * (s.theta_s - s.theta_r) - s.unsaturated_layer_depth[k - 1]) /
                         dt,
                     0.0));
            s.unsaturated_layer_depth[k - 1] = s.unsaturated_layer_depth[k - 1] + toadd * dt;
            netcapflux -= toadd;
            actual += toadd;
        }
        s.actual_capillary_flux = actual;
    } else {
        s.actual_capillary_flux = 0.0;
    }
}

// soil/soil.jl:1118-1136
void leakage(OrcSoil& s, double dt) {
    double deepksat = kv_at_depth(s, s.soil_thickness, s.number_of_layers);
    double deeptransfer = jmin(s.drainable_water_depth / dt, deepksat);
    s.actual_leakage = jmax(0.0, jmin(s.maximum_leakage, deeptransfer));
}

// soil/soil.jl:658-682 (no paddy, no allocation)
void update_bc_soil_model(OrcSoil& s, double canopy_potevap, double interception_rate, double pet,
                          double wfs_runoff, double runoff_river, double runoff_land) {
    s.potential_transpiration = jmax(0.0, canopy_potevap - interception_rate);  // canopy.jl:296-300
    s.potential_soilevaporation = s.soil_fraction * pet;
    s.potential_soilevaporation -= 0.0;
    s.water_flux_surface = jmax(wfs_runoff + 0.0 - runoff_river - runoff_land + 0.0, 0.0);
}

// soil/soil.jl:1150-1211; ae_river/ae_land from the open-water runoff model
void update_soil_water_flow(OrcSoil& s, double temperature, bool snow, bool infilt_reduction,
                            double ae_river, double ae_land, double dt) {
    update_diagnostic_vars(s);
    if (snow) s.soil_surface_temperature = soil_temperature(s.soil_surface_temperature, s.w_soil, temperature);
    s.f_infiltration_reduction = infiltration_reduction_factor(s.soil_surface_temperature, s.cf_soil, snow,
                                                               infilt_reduction);
    double o[2];
    infiltration_fn(s.water_flux_surface, s.compacted_soil_area_fraction, s.infiltration_capacity_soil,
                    s.infiltration_capacity_compacted_soil, s.unsaturated_store_capacity,
                    s.f_infiltration_reduction, dt, o);
    s.infiltration = o[0];
    s.infiltration_excess = o[1];
    unsaturated_zone_flow(s, dt);
    soil_evaporation(s, dt);
    transpiration(s, dt);
    actual_infiltration(s, dt);
    s.saturation_excess_water = (s.water_flux_surface - s.actual_infiltration) - s.infiltration_excess;
    actual_infiltration_soil_path(s.water_flux_surface, s.actual_infiltration, s.compacted_soil_area_fraction,
                                  s.infiltration_capacity_soil, s.infiltration_capacity_compacted_soil,
                                  s.f_infiltration_reduction, o);
    s.actual_infiltration_soil = o[0];
    s.actual_infiltration_compacted_soil = o[1];
    s.excess_water_soil =
        jmax(s.water_flux_surface * (1.0 - s.compacted_soil_area_fraction) - s.actual_infiltration_soil, 0.0);
    s.excess_water_compacted_soil =
        jmax(s.water_flux_surface * s.compacted_soil_area_fraction - s.actual_infiltration_compacted_soil, 0.0);
    double usd = 0.0;
    for (int k = 0; k < s.number_of_layers; ++k) usd += s.unsaturated_layer_depth[k];
    s.unsaturated_store_depth = usd;
    s.unsaturated_store_capacity = s.soil_water_capacity - s.saturated_water_depth - s.unsaturated_store_depth;
    capillary_flux(s, dt);
    leakage(s, dt);
    s.recharge = (s.transfer - s.actual_capillary_flux - s.actual_leakage - s.actual_evaporation_saturated_zone -
                  s.soil_evaporation_saturated_zone);
    s.actual_evapotranspiration = s.soil_evaporation + s.transpiration + ae_river + ae_land + 0.0;
}

// soil/soil.jl:1213-1259
void update_ustorelayerdepth(OrcSoil& s, double zi_prev, double zi) {
    int N = s.maximum_number_of_layers;
    int n_prev = s.n_unsatlayers;
    double thick_prev[ORC_MAXL];
    std::memcpy(thick_prev, s.unsaturated_layer_thickness, sizeof(thick_prev));
    double thick[ORC_MAXL];
    set_layerthickness(zi, s.cumulative_layer_depth, s.actual_layer_thickness, N, thick);
    int n_new = number_of_active_layers(thick, N);
    double* usld = s.unsaturated_layer_depth;
    if (zi < zi_prev) {
        for (int k = n_new; k <= n_prev; ++k) {
            if (k == 0) continue;
            if (std::isnan(thick[k - 1])) {
                usld[k - 1] = 0.0;
            } else {
                double scale = thick[k - 1] / thick_prev[k - 1];
                usld[k - 1] = scale * usld[k - 1];
            }
        }
    } else {
        for (int k = n_prev; k <= n_new; ++k) {
            if (k == 0) continue;
            double tp = std::isnan(thick_prev[k - 1]) ? 0.0 : thick_prev[k - 1];
            double delta = thick[k - 1] - tp;
            usld[k - 1] = usld[k - 1] + delta * (s.theta_fc - s.theta_r);
        }
    }
    s.n_unsatlayers = n_new;
    std::memcpy(s.unsaturated_layer_thickness, thick, sizeof(thick));
    s.water_table_depth = zi;
}

// utils.jl:1090-1131
void water_table_change(const OrcSoil& s, double net_flux, double sy, double dt, double* out) {
    double theta_e = s.theta_s - s.theta_r;
    double dh;
    if (net_flux <= 0.0) {
        dh = net_flux * dt / sy;
    } else {
        dh = 0.0;
        for (int k = s.n_unsatlayers; k >= 1; --k) {
            double capacity =
                jmax(s.unsaturated_layer_thickness[k - 1] * theta_e - s.unsaturated_layer_depth[k - 1], 0.0) / dt;
            double flux_layer = jmin(net_flux, capacity);
            if (capacity <= net_flux) {
                dh += s.unsaturated_layer_thickness[k - 1];
            } else {
                double syk = theta_e - (s.unsaturated_layer_depth[k - 1] / s.unsaturated_layer_thickness[k - 1]);
                dh += flux_layer * dt / syk;
            }
            net_flux -= flux_layer;
            if (net_flux == 0.0) break;
        }
    }
    out[0] = dh;
    out[1] = jmax(net_flux, 0.0);
}

// routing/subsurface/subsurface_process.jl:89-172
void kinematic_wave_ssf(double q_in, double q_prev, double zi_prev, double q_net_bnds, double slope,
                        double sy, double d, double dt, double dx, double dw, double q_max, double kh0,
                        double f, int profile, double z_exp, OrcSoil& soil, double* out) {
    if (is_approx_zero(q_in + q_prev) && q_net_bnds <= 0.0) {
        out[0] = 0.0;
        out[1] = d;
        out[2] = 0.0;
        out[3] = 0.0;
        return;
    }
    double q = (q_prev + q_in) / 2.0;
    double celerity = ssf_celerity(zi_prev, slope, sy, kh0, f, profile, z_exp);
    double constant_term = (dt / dx) * (q_in + q_net_bnds) + q_prev / celerity;
    q = kw_ssf_newton_raphson(q, constant_term, celerity, dt, dx);
    q = jmin(q, (q_max * dw));
    double net_flux = (q_in + q_net_bnds - q) / (dw * dx);
    double wtc[2];
    water_table_change(soil, net_flux, sy, dt, wtc);
    double dh = wtc[0], exfilt = wtc[1];
    double zi = zi_prev - dh;
    if (zi > d) {
        double q_excess = (dw * dx) * sy * (zi - d) / dt;
        q = jmax(q - q_excess, KIN_WAVE_MIN_FLOW);
    }
    zi = jclamp(zi, 0.0, d);
    const double max_delta_zi = 0.1;
    long its = (long)std::ceil(jround_sigdigits(std::fabs(zi - zi_prev) / max_delta_zi, 12));
    if (its > 1) {
        double dt_s = dt / (double)its;
        double q_sum = 0.0, exfilt_sum = 0.0, net_flux_sum = 0.0;
        for (long i = 0; i < its; ++i) {
            celerity = ssf_celerity(zi_prev, slope, sy, kh0, f, profile, z_exp);
            constant_term = (dt_s / dx) * q_in + q_prev / celerity + q_net_bnds * (dt_s / dx);
            q = kw_ssf_newton_raphson(q_prev, constant_term, celerity, dt_s, dx);
            q = jmin(q, (q_max * dw));
            net_flux = (q_in + q_net_bnds - q) / (dw * dx);
            water_table_change(soil, net_flux, sy, dt_s, wtc);
            dh = wtc[0];
            exfilt = wtc[1];
            zi = zi_prev - dh;
            if (zi > d) {
                double q_excess = (dw * dx) * sy * (zi - d) / dt_s;
                q = jmax(q - q_excess, KIN_WAVE_MIN_FLOW);
            }
            zi = jclamp(zi, 0.0, d);
            update_ustorelayerdepth(soil, zi_prev, zi);
            exfilt_sum += exfilt;
            net_flux_sum += net_flux;
            q_sum += q;
            q_prev = q;
            zi_prev = zi;
        }
        q = q_sum / (double)its;
        exfilt = exfilt_sum / (double)its;
        net_flux = net_flux_sum / (double)its;
    } else {
        update_ustorelayerdepth(soil, zi_prev, zi);
    }
    out[0] = q;
    out[1] = zi;
    out[2] = exfilt;
    out[3] = net_flux;
}

// soil/soil.jl:1294-1392 (no paddy)
void update_soil_water_storage(OrcSoil& s, double exfilt_avg, double runoff_land, double ae_land, double dt) {
    (void)dt;
    int nu = s.n_unsatlayers;
    double usd = 0.0;
    for (int k = 0; k < nu; ++k) usd += s.unsaturated_layer_depth[k];
    double sbm_runoff = jmax(0.0, exfilt_avg + s.saturation_excess_water + runoff_land + s.infiltration_excess);
    double ts_tr = s.theta_s - s.theta_r;
    for (int k = 1; k <= s.number_of_layers; ++k) {
        double v;
        if (k <= nu) {
            v = (s.unsaturated_layer_depth[k - 1] +
                 (s.actual_layer_thickness[k - 1] - s.unsaturated_layer_thickness[k - 1]) * ts_tr) /
                    s.actual_layer_thickness[k - 1] +
                s.theta_r;
        } else {
            v = s.theta_s;
        }
        s.volumetric_water_content[k - 1] = v;
        s.relative_volumetric_water_content[k - 1] = (v / s.theta_s) / PERCENTAGE_FACTOR;
    }
    double rootstore_unsat = 0.0;
    for (int k = 1; k <= nu; ++k) {
        rootstore_unsat += jmin(1.0, (jmax(0.0, s.rooting_depth - s.cumulative_layer_depth[k - 1]) /
                                      s.unsaturated_layer_thickness[k - 1])) *
                           s.unsaturated_layer_depth[k - 1];
    }
    double rootstore_sat = jmax(0.0, s.rooting_depth - s.water_table_depth) * ts_tr;
    double root_zone_storage = rootstore_sat + rootstore_unsat;
    double vwc_rz = root_zone_storage / s.rooting_depth + s.theta_r;
    double rel_vwc_rz = (vwc_rz / s.theta_s) / PERCENTAGE_FACTOR;
    double sat = (s.soil_thickness - s.water_table_depth) * ts_tr;
    double drain = (s.soil_thickness - s.water_table_depth) * lower_bound_drainable_porosity(s.theta_s, s.theta_fc);
    double ucap = s.soil_water_capacity - sat - usd;
    s.unsaturated_store_capacity = ucap;
    s.unsaturated_store_depth = usd;
    s.saturated_water_depth = sat;
    s.drainable_water_depth = drain;
    s.exfiltration_saturated_water = exfilt_avg;
    s.runoff = sbm_runoff;
    s.root_zone_storage = root_zone_storage;
    s.volumetric_water_content_root_zone = vwc_rz;
    s.relative_volumetric_water_content_root_zone = rel_vwc_rz;
    s.total_soil_water_storage = sat + usd;
    s.net_runoff = s.runoff - ae_land;
}

// Statistics.jl v1.11.1 _quantile (type 7, alpha = beta = 1) after a full sort.
double quantile_sorted(const double* v, int64_t n, double p) {
    double m = 1.0 + p * (1.0 - 1.0 - 1.0);
    double aleph = std::fma((double)n, p, m);
    int64_t j = (int64_t)std::trunc(aleph);
    if (j < 1) j = 1;
    if (j > n - 1) j = n - 1;
    double gamma = jclamp(aleph - (double)j, 0.0, 1.0);
    double a, b;
    if (n == 1) {
        a = v[0];
        b = v[0];
    } else {
        a = v[j - 1];
        b = v[j];
    }
    bool approx = std::fabs(a - b) <= 1.4901161193847656e-8 * jmax(std::fabs(a), std::fabs(b));
    if (std::isfinite(a) && std::isfinite(b) && approx) return a + gamma * (b - a);
    return (1.0 - gamma) * a + gamma * b;
}

// routing/surface/surface_kinwave.jl:674-704
double kinwave_stable_timestep(const double* q, const double* alpha, const double* flow_length, int64_t n,
                               double p, std::vector<double>& buf) {
    buf.clear();
    for (int64_t i = 0; i < n; ++i) {
        if (q[i] > KIN_WAVE_MIN_FLOW) {
            double c = 1.0 / (alpha[i] * BETA_KINWAVE * jpow(q[i], (BETA_KINWAVE - 1.0)));
            buf.push_back(flow_length[i] / c);
        }
    }
    int64_t k = (int64_t)buf.size();
    if (k == 1) return buf[0];
    if (k > 0) {
        std::sort(buf.begin(), buf.end());
        return quantile_sorted(buf.data(), k, p);
    }
    return 600.0;
}

// routing/timestepping.jl:11-16
inline double check_timestepsize(double ts, double t, double end) { return t + ts > end ? end - t : ts; }

}  // namespace

// ====================================================================== reservoirs ======
//
// Reservoir update at a river node (routing/surface/reservoir.jl:583-628), with the outflow
// functions of types 1 (rating curve from an H-Q table, :455-479), 2 (free weir, with a linked
// lower reservoir, :482-521), 3 (modified Puls, :424-452) and 4 (simple, :389-418), the
// observed-outflow override (:524-545) and the storage profiles S = A H and S = f(H) from an
// S-H table (:306-320, :612-621). The river-side wrapper (surface_kinwave.jl:441-489) limits a
// negative external inflow (abstraction) to 98 % of the storage per step and forms the net
// inflow.
struct OrcReservoir {
    int32_t outflow_type;  // 1 rating curve, 2 free weir, 3 modified Puls, 4 simple
    double area, maximum_storage, threshold, rating_curve_coefficient, rating_curve_exponent;
    double maximum_release, demand, target_minimum_fraction, target_full_fraction;
    // boundary conditions of the step
    double external_inflow, precipitation, evaporation, inflow_overland, inflow_subsurface, outflow_obs;
    // state
    double storage, waterlevel, outflow;
    double inflow_cumulative, outflow_cumulative, actevap_cumulative, abstraction_cumulative;
    // storage_curve_type: 1 (or 0) S = A H, 2 interpolated from the S-H table (sh_n rows of
    // sh_h, sh_s); the H-Q table of outflow type 1 has hq_n rows of hq_h and 365 discharges per
    // row (hq_q row-major), read in column hq_day (col_index_hq, 1..365); lower: the linked lower
    // reservoir as a 1-based index into the member's reservoirs (lower_reservoir_ind), 0 none
    int32_t storage_curve_type, lower;
    int64_t sh_n, hq_n;
    const double *sh_h, *sh_s, *hq_h, *hq_q;
    int32_t hq_day;
};

namespace {

// reservoir.jl:363-375 (the bounds are the minimum and maximum of the table's columns)
double interpolate_linear(double x, const double* xp, const double* fp, int64_t n) {
    double xmin = xp[0], xmax = xp[0], fmin = fp[0], fmax = fp[0];
    for (int64_t i = 1; i < n; ++i) {
        xmin = jmin(xmin, xp[i]);
        xmax = jmax(xmax, xp[i]);
        fmin = jmin(fmin, fp[i]);
        fmax = jmax(fmax, fp[i]);
    }
    if (x <= xmin) return fmin;
    if (x >= xmax) return fmax;
    int64_t i1 = 0;
    for (int64_t i = 0; i < n; ++i)
        if (xp[i] <= x) i1 = i;
    const int64_t i2 = i1 + 1;
    return fp[i1] * (1.0 - (x - xp[i1]) / (xp[i2] - xp[i1])) + fp[i2] * (x - xp[i1]) / (xp[i2] - xp[i1]);
}

// Column `day` (1..365) of an H-Q table: the discharges of every row on that day.
std::vector<double> hq_column(const OrcReservoir& r) {
    std::vector<double> q((size_t)r.hq_n);
    for (int64_t i = 0; i < r.hq_n; ++i) q[(size_t)i] = r.hq_q[i * 365 + (r.hq_day - 1)];
    return q;
}

// initialize_storage (reservoir.jl:343-360)
double initial_storage(const OrcReservoir& r) {
    if (r.storage_curve_type == 2) return interpolate_linear(r.waterlevel, r.sh_h, r.sh_s, r.sh_n);
    return r.area * r.waterlevel;
}

// get_maximum_storage (reservoir.jl:322-340): the storage at the highest level of the H-Q table
double rating_curve_maximum_storage(const OrcReservoir& r) {
    double hmax = r.hq_h[0];
    for (int64_t i = 1; i < r.hq_n; ++i) hmax = jmax(hmax, r.hq_h[i]);
    if (r.storage_curve_type == 2) return interpolate_linear(hmax, r.sh_h, r.sh_s, r.sh_n);
    return r.area * hmax;
}

// reservoir.jl:389-418
void reservoir_simple(const OrcReservoir& r, double precipitation, double evaporation, double inflow, double dt,
                      double& outflow, double& storage) {
    storage = r.storage + (inflow + precipitation - evaporation) * dt;
    storage = jmax(storage, 0.0);
    double fill_fraction = storage / r.maximum_storage;
    double fac = scurve(fill_fraction, r.target_minimum_fraction, 1.0, 30.0);
    double demand_release = jmin(fac * r.demand, storage / dt);
    storage -= demand_release * dt;
    double release_wanted = jmax(0.0, (storage - r.maximum_storage * r.target_full_fraction) / dt);
    double overflow_q = jmax(0.0, (storage - r.maximum_storage) / dt);
    double release_realized = jmin(release_wanted, overflow_q + r.maximum_release - demand_release);
    storage -= release_realized * dt;
    outflow = release_realized + demand_release;
}

// reservoir.jl:424-452
void reservoir_modified_puls(const OrcReservoir& r, double precipitation, double evaporation, double inflow,
                             double dt, double& outflow, double& storage) {
    double res_factor = r.area / (dt * std::sqrt(r.rating_curve_coefficient));
    double si_factor = r.storage / dt + precipitation - evaporation + inflow;
    double si_factor_adj = si_factor - r.area * r.threshold / dt;
    if (si_factor_adj > 0.0) {
        double quadratic_sol_term = -res_factor + std::sqrt((res_factor * res_factor + 4 * si_factor_adj));
        outflow = quadratic_sol_term > 0.0 ? 0.25 * quadratic_sol_term * quadratic_sol_term : 0.0;
    } else {
        outflow = 0.0;
    }
    outflow = jmin(outflow, si_factor);
    storage = (si_factor - outflow) * dt;
}

// reservoir.jl:455-479
void reservoir_hq(const OrcReservoir& r, double precipitation, double evaporation, double inflow, double dt,
                  double& outflow, double& storage) {
    double storage_input = r.storage / dt + precipitation - evaporation + inflow;
    const std::vector<double> q = hq_column(r);
    outflow = interpolate_linear(r.waterlevel, r.hq_h, q.data(), r.hq_n);
    outflow = jmin(outflow, storage_input);
    storage = (storage_input - outflow) * dt;
    double overflow = jmax(0.0, (storage - r.maximum_storage) / dt);
    storage = jmin(storage, r.maximum_storage);
    outflow += overflow;
}

// reservoir.jl:482-521. With a linked lower reservoir `lo` whose level is above this one's, the
// flow runs back from the lower reservoir (a negative outflow), and the lower reservoir's
// storage, level, outflow and cumulative outflow change at once.
void reservoir_free_weir(OrcReservoir* res, int64_t i, double precipitation, double evaporation, double inflow,
                         double dt, double& outflow, double& storage) {
    OrcReservoir& r = res[i];
    const bool has_lower = r.lower != 0;
    OrcReservoir* lo = has_lower ? &res[r.lower - 1] : nullptr;
    double diff_wl = has_lower ? r.waterlevel - lo->waterlevel : 0.0;
    double storage_input = jmax(r.storage / dt + precipitation - evaporation + inflow, 0.0);
    if (diff_wl >= 0.0) {
        if (r.waterlevel > r.threshold) {
            double dh = r.waterlevel - r.threshold;
            outflow = r.rating_curve_coefficient * jpow(dh, r.rating_curve_exponent);
            double maxflow = dh * r.area / dt;
            outflow = jmin(outflow, maxflow);
        } else {
            outflow = 0.0;
        }
    } else {
        if (lo->waterlevel > r.threshold) {
            double dh = lo->waterlevel - r.threshold;
            outflow = -r.rating_curve_coefficient * jpow(dh, r.rating_curve_exponent);
            double maxflow = dh * lo->area / dt;
            outflow = jmax(outflow, -maxflow);
        } else {
            outflow = 0.0;
        }
    }
    storage = (storage_input - outflow) * dt;
    if (diff_wl < 0.0) {
        double lower_res_storage = lo->storage + outflow * dt;
        double lower_res_waterlevel = lo->storage_curve_type == 2
                                          ? interpolate_linear(lower_res_storage, lo->sh_s, lo->sh_h, lo->sh_n)
                                          : lo->waterlevel + (lower_res_storage - lo->storage) / lo->area;
        lo->outflow = -outflow;
        lo->outflow_cumulative -= outflow * dt;
        lo->storage = lower_res_storage;
        lo->waterlevel = lower_res_waterlevel;
    }
}

// reservoir.jl:524-545
void reservoir_outflow_obs(const OrcReservoir& r, double precipitation, double evaporation, double inflow, double dt,
                           double& outflow, double& storage) {
    double storage_input = jmax(r.storage / dt + precipitation - evaporation + inflow, 0.0);
    outflow = jmin(r.outflow_obs, storage_input);
    storage = (storage_input - outflow) * dt;
    if (!std::isnan(r.maximum_storage)) {
        double overflow = jmax(0.0, (storage - r.maximum_storage) / dt);
        storage -= overflow * dt;
        outflow += overflow;
    }
}

// reservoir.jl:583-628, reservoir i of the member's reservoirs `res`
void update_reservoir(OrcReservoir* res, int64_t i, double inflow, double dt) {
    OrcReservoir& r = res[i];
    double precipitation = r.precipitation * r.area;
    double available_storage = r.storage + (inflow + precipitation) * dt;
    double potential_evaporation = r.evaporation * r.area;
    double evaporation = jmin(available_storage / dt, potential_evaporation);
    double outflow = 0.0, storage = r.storage;
    if (!std::isnan(r.outflow_obs)) reservoir_outflow_obs(r, precipitation, evaporation, inflow, dt, outflow, storage);
    else if (r.outflow_type == 1) reservoir_hq(r, precipitation, evaporation, inflow, dt, outflow, storage);
    else if (r.outflow_type == 2) reservoir_free_weir(res, i, precipitation, evaporation, inflow, dt, outflow, storage);
    else if (r.outflow_type == 3) reservoir_modified_puls(r, precipitation, evaporation, inflow, dt, outflow, storage);
    else reservoir_simple(r, precipitation, evaporation, inflow, dt, outflow, storage);
    double waterlevel = r.storage_curve_type == 2 ? interpolate_linear(storage, r.sh_s, r.sh_h, r.sh_n)
                                                  : r.waterlevel + (storage - r.storage) / r.area;
    r.storage = storage;
    r.waterlevel = waterlevel;
    r.outflow = outflow;
    r.inflow_cumulative += inflow * dt;
    r.outflow_cumulative += outflow * dt;
    r.actevap_cumulative += evaporation / r.area * dt;
}

// surface_kinwave.jl:441-489: net inflow of reservoir i at a river node whose discharge is q
void update_reservoir_at_node(OrcReservoir* res, int64_t i, double q, double dt) {
    OrcReservoir& r = res[i];
    double inflow;
    if (r.external_inflow < 0.0) {
        double abstraction = jmin(-r.external_inflow, (r.storage / dt) * 0.98);
        r.abstraction_cumulative += abstraction * dt;
        inflow = -abstraction;
    } else {
        inflow = r.external_inflow;
    }
    double net_inflow = q + r.inflow_overland + r.inflow_subsurface + inflow;
    update_reservoir(res, i, net_inflow, dt);
}

}  // namespace

// ======================================================================= full model =====

// The land grid with its river routed by the local-inertial scheme in place of the kinematic
// waves (surface_routing.jl:62-89): copies of the grid and network arrays, the scheme's state
// (OrcLiState), its inputs and the averages of the last step.
struct OrcLiCoupled {
    std::vector<int64_t> ixu, ixd, iyu, iyd, riv, src, dst;
    std::vector<double> xl, yl, z, nsq, xw, yw, zb, fl, fw, bd, zbe, we, le, nsqe;
    WfLiLandGrid g{};
    WfLiRiverNetwork r{};
    std::vector<double> h_land, storage, error, qx, qy, qx0, qy0, qx_cum, qy_cum;
    std::vector<double> h_river, storage_river, q, q_prev, q_cum, abstraction_cum;
    std::vector<double> runoff, ext, abstraction, qx_avg, qy_avg, q_avg;
    std::vector<int64_t> out_edge;                  // per river cell: its outgoing edge, or -1
    std::vector<std::vector<int64_t>> e_in, e_out;  // edges_at_node.src / .dst (ascending)
    OrcLiState st{};
    int64_t substeps = 0;
};

struct OrcModel {
    WfConfig cfg{};
    int N = 0;  // maximum_number_of_layers
    int64_t n = 0, nr = 0;
    int M = 1;
    std::string err;
    bool gash = false;
    // land geometry
    std::vector<int32_t> ds;
    std::vector<double> area, flow_width, flow_length, sfw, slope, frac_to_river, river_fraction, water_fraction, top;
    std::vector<int32_t> land_river;  // river index of a land cell or -1
    std::vector<int64_t> topo;        // topological order (upstream first)
    std::vector<std::vector<int32_t>> ups;  // upstream nodes per node (ascending)
    // river geometry
    std::vector<int32_t> r_land, r_ds;
    std::vector<double> r_width, r_length, r_slope, r_alpha, r_ext_inflow;
    std::vector<int64_t> r_topo;
    std::vector<std::vector<int32_t>> r_ups;
    std::vector<int32_t> r_pits;
    // per-cell static params (vegetation, snow)
    std::vector<double> gap, cmax, kc, e_r, ddf, tt, tti, ttm, whc;
    std::vector<double> ol_alpha;
    // ssf params (per member for kh0/f)
    std::vector<double> kh0, ssf_f, sy, q_max, z_exp;
    // per member state/variables (size n*M)
    std::vector<OrcSoil> soil;
    std::vector<double> P, PET, T;
    std::vector<double> canopy_storage, canopy_potevap, interception_rate, throughfall, stemflow;
    std::vector<double> snow_storage, snow_water, swe, snow_melt, snow_runoff;
    // lateral snow transport and glacier (snow_gravitational_transport__flag, glacier__flag)
    bool snow_transport = false, glacier = false;
    std::vector<int64_t> dfs_order;                  // topological_sort_by_dfs of the land graph
    std::vector<double> g_frac, g_ttm, g_ddf, g_sifrac;  // per cell
    std::vector<double> glacier_store, glacier_melt, snow_in, snow_out;  // per member and cell
    std::vector<double> wfs, runoff_river, net_runoff_river, runoff_land, ae_land, ae_river;
    std::vector<double> ssf_zi, ssf_head, ssf_exf_cum, ssf_exf_avg, ssf_q, ssf_q_cum, ssf_q_avg, ssf_qin,
        ssf_qin_cum, ssf_qin_avg, ssf_tr_cum, ssf_tr_avg, ssf_qnet, ssf_qnet_cum, ssf_qnet_avg, ssf_storage;
    std::vector<double> rch_rate, rch_flux, rch_flux_cum, rch_flux_avg;
    std::vector<double> ol_q, ol_qlat, ol_qin, ol_qin_cum, ol_qin_avg, ol_q_cum, ol_q_avg, ol_storage, ol_h,
        ol_tr_cum, ol_tr_avg, ol_inwater;
    std::vector<double> rv_q, rv_qlat, rv_qin, rv_qin_cum, rv_qin_avg, rv_q_cum, rv_q_avg, rv_storage, rv_h,
        rv_inwater, rv_abs_cum, rv_abs_avg;
    std::vector<double> total_storage;
    std::vector<double> bl_prev, bl_err, bl_rel, bo_prev, bo_err, bo_rel, bs_err, bs_rel, br_prev, br_err, br_rel;
    // reservoirs (member-major [mbr * nres + k])
    int64_t nres = 0;
    std::vector<OrcReservoir> res;
    std::vector<double> res_tables;          // the reservoirs' S-H and H-Q tables (OrcReservoir points here)
    std::vector<int64_t> res_sh_at, res_hq_at;  // [nres] start of each reservoir's tables
    std::vector<int32_t> res_of_river;  // [nr] reservoir at a river cell, or -1
    std::vector<int32_t> res_land;      // [nres] land cell of the reservoir outlet
    std::vector<double> res_out_avg, res_in_avg, res_evap_avg, res_abs_avg, res_prev, res_err, res_rel;
    int64_t last_sub_land = 0, last_sub_river = 0, last_sub_ssf = 0;
    std::vector<double> sig[3];  // per member: sum of the squared sub-step sizes (subsurface, land, river)
    std::vector<double> buf;
    std::unique_ptr<OrcLiCoupled> li;  // local-inertial land and river routing (one member)
};

namespace {

bool topo_sort(int64_t n, const int32_t* ds, std::vector<int64_t>& order) {
    std::vector<int32_t> indeg(n, 0);
    for (int64_t i = 0; i < n; ++i)
        if (ds[i] >= 0) indeg[ds[i]]++;
    order.clear();
    order.reserve(n);
    for (int64_t i = 0; i < n; ++i)
        if (indeg[i] == 0) order.push_back(i);
    for (size_t h = 0; h < order.size(); ++h) {
        int64_t v = order[h];
        if (ds[v] >= 0 && --indeg[ds[v]] == 0) order.push_back(ds[v]);
    }
    return (int64_t)order.size() == n;
}

void build_ups(int64_t n, const int32_t* ds, std::vector<std::vector<int32_t>>& ups) {
    ups.assign(n, {});
    for (int64_t i = 0; i < n; ++i)
        if (ds[i] >= 0) ups[ds[i]].push_back((int32_t)i);  // ascending i
}

// Graphs.jl v1.14 topological_sort_by_dfs (Wflow's network.order, network.jl:99), restated for a
// graph of out-degree <= 1: vertices are visited in index order; from an unvisited vertex the
// search follows the downstream links while they lead to unvisited vertices and finishes the
// path from its downstream end back; the order is the reverse of the finishing order.
bool topo_sort_dfs(int64_t n, const int32_t* ds, std::vector<int64_t>& order) {
    std::vector<uint8_t> color(n, 0);
    std::vector<int64_t> verts, stack;
    verts.reserve(n);
    for (int64_t v = 0; v < n; ++v) {
        if (color[v]) continue;
        stack.assign(1, v);
        color[v] = 1;
        while (!stack.empty()) {
            const int64_t u = stack.back();
            const int32_t w = ds[u];
            if (w >= 0 && color[w] == 1) return false;  // a cycle
            if (w >= 0 && color[w] == 0) {
                color[w] = 1;
                stack.push_back(w);
            } else {
                color[u] = 2;
                verts.push_back(u);
                stack.pop_back();
            }
        }
    }
    order.assign(verts.rbegin(), verts.rend());
    return true;
}

inline double prm(const double* p, int64_t i, double dflt) { return p ? p[i] : dflt; }

}  // namespace

extern "C" {

const char* orc_model_error(const OrcModel* m) { return m ? m->err.c_str() : "null model"; }

int32_t orc_model_create(const WfConfig* c, const WfDomain* d, const WfParams* p, OrcModel** out) {
    *out = nullptr;
    OrcModel* m = new OrcModel();
    m->cfg = *c;
    m->N = c->n_soil_layer_thickness + 1;
    m->M = c->n_members > 0 ? c->n_members : 1;
    m->n = d->n_land;
    m->nr = d->n_river;
    m->gash = c->dt >= 23.0 * 3600.0;  // sbm.jl:26-33
    const int64_t n = m->n, nr = m->nr;
    const int M = m->M, N = m->N;
    if (N < 2 || N > ORC_MAXL || n <= 0 || nr < 0) {
        m->err = "invalid sizes";
        *out = m;
        return WF_ERR_INVALID;
    }
    m->ds.assign(d->land_downstream, d->land_downstream + n);
    auto cp = [&](std::vector<double>& v, const double* src, int64_t cnt) { v.assign(src, src + cnt); };
    cp(m->area, d->area, n);
    cp(m->flow_width, d->flow_width, n);
    cp(m->flow_length, d->flow_length, n);
    cp(m->sfw, d->surface_flow_width, n);
    cp(m->slope, d->slope, n);
    cp(m->frac_to_river, d->flow_fraction_to_river, n);
    cp(m->river_fraction, d->river_fraction, n);
    cp(m->water_fraction, d->water_fraction, n);
    cp(m->top, d->elevation, n);
    if (!topo_sort(n, m->ds.data(), m->topo)) {
        m->err = "cycle in land drainage graph";
        *out = m;
        return WF_ERR_CYCLE;
    }
    build_ups(n, m->ds.data(), m->ups);
    m->land_river.assign(n, -1);
    m->r_land.assign(d->river_land_index, d->river_land_index + nr);
    m->r_ds.assign(d->river_downstream, d->river_downstream + nr);
    for (int64_t r = 0; r < nr; ++r) m->land_river[m->r_land[r]] = (int32_t)r;
    cp(m->r_width, d->river_width, nr);
    cp(m->r_length, d->river_length, nr);
    cp(m->r_slope, d->river_slope, nr);
    m->r_ext_inflow.assign(nr, 0.0);
    if (d->river_external_inflow) cp(m->r_ext_inflow, d->river_external_inflow, nr);
    if (!topo_sort(nr, m->r_ds.data(), m->r_topo)) {
        m->err = "cycle in river drainage graph";
        *out = m;
        return WF_ERR_CYCLE;
    }
    build_ups(nr, m->r_ds.data(), m->r_ups);
    for (int64_t r = 0; r < nr; ++r)
        if (m->r_ds[r] < 0) m->r_pits.push_back((int32_t)r);
    // river Manning alpha: surface_kinwave.jl:32-44 with wetted perimeter width + bankfull (:80-82)
    m->r_alpha.resize(nr);
    for (int64_t r = 0; r < nr; ++r) {
        double wp = d->river_width[r] + d->river_bankfull_depth[r];
        double alpha_term = jpow(d->river_manning_n[r] / std::sqrt(d->river_slope[r]), BETA_KINWAVE);
        double alpha_pow = (2.0 / 3.0) * BETA_KINWAVE;
        m->r_alpha[r] = alpha_term * jpow(wp, alpha_pow);
    }
    m->ol_alpha.resize(n);
    for (int64_t i = 0; i < n; ++i) {
        double alpha_term = jpow(d->land_manning_n[i] / std::sqrt(m->slope[i]), BETA_KINWAVE);
        m->ol_alpha[i] = alpha_term * jpow(m->sfw[i], (2.0 / 3.0) * BETA_KINWAVE);
    }
    cp(m->gap, p->canopy_gap_fraction, n);
    cp(m->cmax, p->maximum_canopy_storage, n);
    cp(m->kc, p->crop_coefficient, n);
    m->e_r.assign(n, 0.1);
    if (p->evaporation_to_precipitation_ratio) cp(m->e_r, p->evaporation_to_precipitation_ratio, n);
    cp(m->ddf, p->degree_day_factor, n);
    cp(m->tt, p->temperature_threshold_snowfall, n);
    cp(m->tti, p->temperature_interval_snowfall, n);
    cp(m->ttm, p->temperature_threshold_melt, n);
    cp(m->whc, p->water_holding_capacity, n);
    // lateral snow transport and glacier (sbm.jl:36-53: a glacier needs the snow model)
    m->snow_transport = c->snow_gravitational_transport != 0;
    m->glacier = c->glacier != 0;
    if ((m->snow_transport || m->glacier) && !c->snow) {
        m->err = "gravitational snow transport and glaciers need the snow model (snow__flag)";
        *out = m;
        return WF_ERR_INVALID;
    }
    if (m->snow_transport && !topo_sort_dfs(n, m->ds.data(), m->dfs_order)) {
        m->err = "cycle in land drainage graph";
        *out = m;
        return WF_ERR_CYCLE;
    }
    m->g_frac.assign(n, 0.0);
    m->g_ttm.assign(n, 0.0);
    m->g_ddf.assign(n, 0.0);
    m->g_sifrac.assign(n, 0.0);
    for (int64_t i = 0; i < n && m->glacier; ++i) {  // defaults: standard_name_sbm.jl:70-108, to SI
        // without a glacier model the fraction is zero (NoGlacierModel, glacier.jl:160-166)
        m->g_frac[i] = prm(p->glacier_fraction, i, 0.0);
        m->g_ttm[i] = prm(p->glacier_temperature_threshold_melt, i, 0.0 + ABSOLUTE_ZERO_C);
        m->g_ddf[i] = prm(p->glacier_degree_day_factor, i, 3.0 * MM_PER_DAY_FACTOR);
        m->g_sifrac[i] = prm(p->glacier_snow_to_ice_fraction, i, 0.001 * (1.0 / 86400.0));
    }

    // soil parameters (soil.jl:319-617) and cold state (soil.jl:152-200), per member
    const int64_t nm = n * M;
    m->soil.assign(nm, OrcSoil{});
    m->kh0.resize(nm);
    m->ssf_f.resize(nm);
    m->sy.resize(n);
    m->q_max.resize(nm);
    m->z_exp.assign(n, 0.0);
    if (p->z_exp) cp(m->z_exp, p->z_exp, n);
    double cfg_thick[ORC_MAXL];
    for (int k = 0; k < N - 1; ++k) cfg_thick[k] = c->soil_layer_thickness[k];
    cfg_thick[N - 1] = MISSING;
    double cfg_cum[ORC_MAXL + 1];
    cfg_cum[0] = 0.0;
    for (int k = 0; k < N; ++k) cfg_cum[k + 1] = cfg_cum[k] + cfg_thick[k];
    for (int mbr = 0; mbr < M; ++mbr) {
        for (int64_t i = 0; i < n; ++i) {
            OrcSoil& s = m->soil[mbr * n + i];
            int64_t ip = c->per_member_soil ? mbr * n + i : i;
            s.maximum_number_of_layers = N;
            s.kv_profile = c->kv_profile;
            s.theta_s = p->theta_s[i];
            s.theta_r = p->theta_r[i];
            s.kv_0 = p->kv_0[ip];
            s.f = p->f[ip];
            s.z_exp = m->z_exp[i];
            s.air_entry_pressure = p->air_entry_pressure[i];
            s.h1 = p->h1[i];
            s.h2 = p->h2[i];
            s.h3_high = p->h3_high[i];
            s.h3_low = p->h3_low[i];
            s.h4 = p->h4[i];
            s.alpha_h1 = p->alpha_h1[i];
            s.soil_thickness = p->soil_thickness[i];
            s.infiltration_capacity_compacted_soil = p->infiltration_capacity_compacted_soil[i];
            s.compacted_soil_area_fraction = p->compacted_soil_area_fraction[i];
            s.wet_root_distribution_parameter = p->wet_root_distribution_parameter[i];
            s.cap_hmax = p->cap_hmax[i];
            s.cap_n = p->cap_n[i];
            s.maximum_leakage = p->maximum_leakage[i];
            s.w_soil = p->w_soil[i];
            s.cf_soil = p->cf_soil[i];
            for (int k = 0; k < N; ++k) {
                s.brooks_corey_exponent[k] = p->brooks_corey_exponent[i * N + k];
                s.kv_factor[k] = p->kv_factor[i * N + k];
            }
            // soil.jl:513-516
            set_layerthickness(s.soil_thickness, cfg_cum, cfg_thick, N, s.actual_layer_thickness);
            s.cumulative_layer_depth[0] = 0.0;
            for (int k = 0; k < N; ++k)
                s.cumulative_layer_depth[k + 1] = s.cumulative_layer_depth[k] + s.actual_layer_thickness[k];
            s.number_of_layers = number_of_active_layers(s.actual_layer_thickness, N);
            // soil.jl:527-534
            s.theta_fc = field_capacity(s.actual_layer_thickness, s.number_of_layers, s.theta_s, s.theta_r,
                                        s.brooks_corey_exponent, s.air_entry_pressure);
            // soil.jl:480
            s.infiltration_capacity_soil = s.kv_0 * s.kv_factor[0];
            // sbm.jl:57-58
            s.rooting_depth = jmin(s.soil_thickness * 0.99, p->rooting_depth[i]);
            // soil.jl:543-563 (default root fraction; uses the vegetation rooting depth before
            // the clip of sbm.jl:57, which runs after SbmSoilModel is built)
            double rd0 = p->rooting_depth[i];
            for (int k = 0; k < N; ++k) {
                double rf = 0.0;
                if (rd0 > 0.0) {
                    if ((rd0 - s.cumulative_layer_depth[k]) >= s.actual_layer_thickness[k]) {
                        rf = s.actual_layer_thickness[k] / rd0;
                    } else {
                        rf = jmax((rd0 - s.cumulative_layer_depth[k]) / rd0, 0.0);
                    }
                }
                s.rootfraction[k] = rf;
            }
            s.soil_water_capacity = s.soil_thickness * (s.theta_s - s.theta_r);
            // cold state soil.jl:164-178
            s.saturated_water_depth = 0.85 * s.soil_water_capacity;
            for (int k = 0; k < ORC_MAXL; ++k) s.unsaturated_layer_depth[k] = 0.0;
            s.unsaturated_store_depth = 0.0;
            s.water_table_depth =
                jmax(0.0, s.soil_thickness - s.saturated_water_depth / (s.theta_s - s.theta_r));
            s.drainable_water_depth =
                (s.soil_thickness - s.water_table_depth) * lower_bound_drainable_porosity(s.theta_s, s.theta_fc);
            set_layerthickness(s.water_table_depth, s.cumulative_layer_depth, s.actual_layer_thickness, N,
                               s.unsaturated_layer_thickness);
            s.n_unsatlayers = number_of_active_layers(s.unsaturated_layer_thickness, N);
            s.total_soil_water_storage = s.saturated_water_depth + s.unsaturated_store_depth;
            s.unsaturated_store_capacity = s.soil_water_capacity - s.saturated_water_depth;
            s.soil_surface_temperature = 10.0 + 273.15;
            s.f_infiltration_reduction = 1.0;
            // lateral_subsurface_flow.jl:109,122
            double kh0 = p->horizontal_to_vertical_ratio[i] * s.kv_0;
            m->kh0[mbr * n + i] = kh0;
            m->ssf_f[mbr * n + i] = s.f;
            if (mbr == 0) m->sy[i] = lower_bound_drainable_porosity(s.theta_s, s.theta_fc);
        }
    }
    // per-member variables
    auto z = [&](std::vector<double>& v, int64_t cnt, double val) { v.assign(cnt, val); };
    z(m->P, nm, 0.0); z(m->PET, nm, 0.0); z(m->T, nm, 0.0);
    z(m->canopy_storage, nm, 0.0); z(m->canopy_potevap, nm, 0.0); z(m->interception_rate, nm, 0.0);
    z(m->throughfall, nm, 0.0); z(m->stemflow, nm, 0.0);
    z(m->snow_storage, nm, 0.0); z(m->snow_water, nm, 0.0); z(m->swe, nm, 0.0); z(m->snow_melt, nm, 0.0);
    z(m->snow_runoff, nm, 0.0);
    z(m->glacier_store, nm, 0.0); z(m->glacier_melt, nm, 0.0); z(m->snow_in, nm, 0.0); z(m->snow_out, nm, 0.0);
    if (m->glacier)
        for (int mbr = 0; mbr < M; ++mbr)
            for (int64_t i = 0; i < n; ++i) m->glacier_store[mbr * n + i] = prm(p->glacier_initial_store, i, 5.5);
    z(m->wfs, nm, 0.0); z(m->runoff_river, nm, 0.0); z(m->net_runoff_river, nm, 0.0); z(m->runoff_land, nm, 0.0);
    z(m->ae_land, nm, 0.0); z(m->ae_river, nm, 0.0);
    for (auto* v : {&m->ssf_head, &m->ssf_exf_cum, &m->ssf_exf_avg, &m->ssf_q, &m->ssf_q_cum, &m->ssf_q_avg,
                    &m->ssf_qin, &m->ssf_qin_cum, &m->ssf_qin_avg, &m->ssf_tr_cum, &m->ssf_tr_avg, &m->ssf_qnet,
                    &m->ssf_qnet_cum, &m->ssf_qnet_avg, &m->ssf_storage, &m->ssf_zi, &m->rch_rate, &m->rch_flux,
                    &m->rch_flux_cum, &m->rch_flux_avg, &m->ol_q, &m->ol_qlat, &m->ol_qin, &m->ol_qin_cum,
                    &m->ol_qin_avg, &m->ol_q_cum, &m->ol_q_avg, &m->ol_storage, &m->ol_h, &m->ol_tr_cum,
                    &m->ol_tr_avg, &m->ol_inwater, &m->total_storage, &m->bl_prev, &m->bl_err, &m->bl_rel,
                    &m->bo_prev, &m->bo_err, &m->bo_rel, &m->bs_err, &m->bs_rel})
        z(*v, nm, 0.0);
    const int64_t nrm = nr * M;
    for (auto* v : {&m->rv_q, &m->rv_qlat, &m->rv_qin, &m->rv_qin_cum, &m->rv_qin_avg, &m->rv_q_cum, &m->rv_q_avg,
                    &m->rv_storage, &m->rv_h, &m->rv_inwater, &m->rv_abs_cum, &m->rv_abs_avg, &m->br_prev,
                    &m->br_err, &m->br_rel})
        z(*v, nrm, 0.0);
    // lateral subsurface initial state: lateral_subsurface_flow.jl:134-141, utils.jl:916-979
    for (int mbr = 0; mbr < M; ++mbr) {
        for (int64_t i = 0; i < n; ++i) {
            int64_t j = mbr * n + i;
            const OrcSoil& s = m->soil[j];
            double zi = s.water_table_depth;
            double d = s.soil_thickness;
            double kh0 = m->kh0[j], f = m->ssf_f[j];
            m->ssf_zi[j] = zi;
            m->ssf_storage[j] = m->sy[i] * (d - zi) * m->area[i];
            m->ssf_head[j] = m->top[i] - zi;
            if (c->kv_profile == WF_KV_EXPONENTIAL) {
                m->q_max[j] = ((kh0 * m->slope[i]) / f) * (1.0 - wexp(-f * d));
                m->ssf_q[j] = ((kh0 * m->slope[i]) / f) * (wexp(-f * zi) - wexp(-f * d)) * m->flow_width[i];
            } else {
                double zx = m->z_exp[i];
                double q_constant = kh0 * wexp(-f * zx) * m->slope[i] * (d - zx);
                m->q_max[j] = ((kh0 * m->slope[i]) / f) * (1.0 - wexp(-f * zx)) + q_constant;
                if (zi < zx) {
                    m->ssf_q[j] = (((kh0 * m->slope[i]) / f) * (wexp(-f * zi) - wexp(-f * zx)) + q_constant) *
                                  m->flow_width[i];
                } else {
                    m->ssf_q[j] = kh0 * wexp(-f * zi) * m->slope[i] * (d - zi) * m->flow_width[i];
                }
            }
        }
    }
    *out = m;
    return WF_OK;
}

void orc_model_destroy(OrcModel* m) { delete m; }

// Couple the land grid with its river (local-inertial) to the model's step (li_surface_routing):
// one member, no reservoirs, fixed kinematic-wave settings unused; the grid's land cells are the
// model's land cells and its active river cells the model's river cells (river_index of the
// land cell of river cell r is r). Warm state as wf_li_domain_set_state.
int32_t orc_model_attach_li(OrcModel* m, const WfLiLandGrid* land, const WfLiRiverNetwork* river,
                            const double* h_land, const double* h_river) {
    if (!m || !land || !river || !h_land || !h_river) return WF_ERR_INVALID;
    if (m->M != 1 || m->nres > 0 || m->cfg.adaptive_timestep) {
        m->err = "local-inertial routing in the step needs one member, no reservoirs and fixed sub-steps";
        return WF_ERR_UNSUPPORTED;
    }
    if (land->n != m->n || river->n_active != m->nr) {
        m->err = "the grid's land and active river cells must be the model's";
        return WF_ERR_INVALID;
    }
    for (int64_t r = 0; r < m->nr; ++r)
        if (land->river_index[m->r_land[r]] != r) {
            m->err = "river_index must map the land cell of river cell r to r";
            return WF_ERR_INVALID;
        }
    auto c = std::make_unique<OrcLiCoupled>();
    const int64_t n = land->n, nrt = river->n, ne = river->n_edges;
    auto cpi = [](std::vector<int64_t>& v, const int64_t* p, int64_t k) { v.assign(p, p + k); };
    auto cpd = [](std::vector<double>& v, const double* p, int64_t k) { v.assign(p, p + k); };
    cpi(c->ixu, land->ind_x_up, n);
    cpi(c->ixd, land->ind_x_down, n);
    cpi(c->iyu, land->ind_y_up, n);
    cpi(c->iyd, land->ind_y_down, n);
    cpi(c->riv, land->river_index, n);
    cpd(c->xl, land->x_length, n);
    cpd(c->yl, land->y_length, n);
    cpd(c->z, land->elevation, n);
    cpd(c->nsq, land->mannings_n_sq, n);
    cpd(c->xw, land->xwidth_at_edge, n);
    cpd(c->yw, land->ywidth_at_edge, n);
    cpi(c->src, river->src, ne);
    cpi(c->dst, river->dst, ne);
    cpd(c->zb, river->zb, nrt);
    cpd(c->fl, river->flow_length, nrt);
    cpd(c->fw, river->flow_width, nrt);
    cpd(c->bd, river->bankfull_depth, nrt);
    cpd(c->zbe, river->zb_edge, ne);
    cpd(c->we, river->width_edge, ne);
    cpd(c->le, river->length_edge, ne);
    cpd(c->nsqe, river->mannings_n_sq_edge, ne);
    c->g = *land;
    c->g.ind_x_up = c->ixu.data();
    c->g.ind_x_down = c->ixd.data();
    c->g.ind_y_up = c->iyu.data();
    c->g.ind_y_down = c->iyd.data();
    c->g.river_index = c->riv.data();
    c->g.x_length = c->xl.data();
    c->g.y_length = c->yl.data();
    c->g.elevation = c->z.data();
    c->g.mannings_n_sq = c->nsq.data();
    c->g.xwidth_at_edge = c->xw.data();
    c->g.ywidth_at_edge = c->yw.data();
    c->r = *river;
    c->r.src = c->src.data();
    c->r.dst = c->dst.data();
    c->r.zb = c->zb.data();
    c->r.flow_length = c->fl.data();
    c->r.flow_width = c->fw.data();
    c->r.bankfull_depth = c->bd.data();
    c->r.zb_edge = c->zbe.data();
    c->r.width_edge = c->we.data();
    c->r.length_edge = c->le.data();
    c->r.mannings_n_sq_edge = c->nsqe.data();
    for (auto* v : {&c->h_land, &c->storage, &c->error, &c->runoff}) v->assign(n, 0.0);
    for (auto* v : {&c->qx, &c->qy, &c->qx0, &c->qy0, &c->qx_cum, &c->qy_cum, &c->qx_avg, &c->qy_avg})
        v->assign(n + 1, 0.0);
    for (auto* v : {&c->h_river, &c->storage_river, &c->abstraction_cum, &c->ext, &c->abstraction})
        v->assign(nrt, 0.0);
    for (auto* v : {&c->q, &c->q_prev, &c->q_cum, &c->q_avg}) v->assign(ne, 0.0);
    c->out_edge.assign(nrt, -1);
    c->e_in.assign(nrt, {});
    c->e_out.assign(nrt, {});
    for (int64_t e = 0; e < ne; ++e) {
        c->e_in[c->dst[e]].push_back(e);
        c->e_out[c->src[e]].push_back(e);
        if (c->out_edge[c->src[e]] < 0) c->out_edge[c->src[e]] = e;
    }
    // warm state (sbm_model.jl:135-172)
    for (int64_t i = 0; i < n; ++i) {
        c->h_land[i] = h_land[i];
        const int64_t r = c->riv[i];
        if (r >= 0)
            c->storage[i] = h_land[i] > 0.0 ? h_land[i] * c->xl[i] * c->yl[i] + c->bd[r] * c->fw[r] * c->fl[r]
                                            : h_river[r] * c->fw[r] * c->fl[r];
        else
            c->storage[i] = h_land[i] * c->xl[i] * c->yl[i];
    }
    for (int64_t r = 0; r < nrt; ++r) {
        c->h_river[r] = h_river[r];
        if (r < river->n_active) c->storage_river[r] = h_river[r] * c->fw[r] * c->fl[r];
    }
    c->st = OrcLiState{c->h_land.data(), c->storage.data(), c->error.data(), c->qx.data(), c->qy.data(),
                       c->qx0.data(), c->qy0.data(), c->qx_cum.data(), c->qy_cum.data(), c->h_river.data(),
                       c->storage_river.data(), c->q.data(), c->q_prev.data(), c->q_cum.data(),
                       c->abstraction_cum.data()};
    for (int64_t i = 0; i < n; ++i) {
        m->ol_h[i] = c->h_land[i];
        m->ol_storage[i] = c->storage[i];
    }
    for (int64_t r = 0; r < m->nr; ++r) {
        m->rv_h[r] = c->h_river[r];
        m->rv_storage[r] = c->storage_river[r];
    }
    m->li = std::move(c);
    return WF_OK;
}

// A field of the coupled scheme (the WfLiDomainField ids of wf_li_domain_get), and the sub-steps
// of the last step (field -1, one value).
int32_t orc_model_li_get(OrcModel* m, int32_t field, double* out) {
    if (!m || !m->li || !out) return WF_ERR_INVALID;
    const OrcLiCoupled& c = *m->li;
    const int64_t n = m->n;
    const std::vector<double>* v = nullptr;
    int64_t cnt = 0;
    switch (field) {
        case -1: out[0] = (double)c.substeps; return WF_OK;
        case 0: v = &c.h_land; cnt = n; break;
        case 1: v = &c.storage; cnt = n; break;
        case 2: v = &c.error; cnt = n; break;
        case 3: v = &c.qx; cnt = n; break;
        case 4: v = &c.qy; cnt = n; break;
        case 5: v = &c.qx_avg; cnt = n; break;
        case 6: v = &c.qy_avg; cnt = n; break;
        case 7: v = &c.h_river; cnt = c.r.n; break;
        case 8: v = &c.storage_river; cnt = c.r.n; break;
        case 9: v = &c.q; cnt = c.r.n_edges; break;
        case 10: v = &c.q_avg; cnt = c.r.n_edges; break;
        case 11: v = &c.abstraction_cum; cnt = c.r.n; break;
        default: return WF_ERR_INVALID;
    }
    std::copy(v->begin(), v->begin() + cnt, out);
    return WF_OK;
}

// The land graph order of the snow transport (topological_sort_by_dfs); 0, or -3 on a cycle.
int32_t orc_topo_order_dfs(int64_t n, const int32_t* ds, int64_t* order) {
    std::vector<int64_t> v;
    if (!topo_sort_dfs(n, ds, v)) return WF_ERR_CYCLE;
    for (int64_t k = 0; k < n; ++k) order[k] = v[k];
    return WF_OK;
}

// The model with reservoirs (ReservoirModel, routing/surface/reservoir.jl:290-300). Reservoir
// outlet cells are pits of the land and river upstream lists (domain.jl:95-121,
// utils.jl:61-71); the topological orders stay those of the full graphs, which remain valid.
int32_t orc_model_create_with_reservoirs(const WfConfig* c, const WfDomain* d, const WfParams* p,
                                         const WfReservoirs* rs, OrcModel** out) {
    return orc_model_create_with_reservoir_tables(c, d, p, rs, nullptr, out);
}

// The same with the reservoirs' S-H and H-Q tables and links (ReservoirParameters,
// reservoir.jl:5-44, 152-192): the tables are copied into the model; a linked lower reservoir
// is stored 1-based (lower_reservoir_ind).
int32_t orc_model_create_with_reservoir_tables(const WfConfig* c, const WfDomain* d, const WfParams* p,
                                               const WfReservoirs* rs, const WfReservoirTables* tb,
                                               OrcModel** out) {
    int32_t st = orc_model_create(c, d, p, out);
    if (st != WF_OK || !rs || rs->n == 0) return st;
    OrcModel* m = *out;
    const int64_t nres = rs->n, nr = m->nr, n = m->n;
    const int M = m->M;
    auto fail = [&](const std::string& msg) {
        m->err = msg;
        return WF_ERR_INVALID;
    };
    if (nres < 0 || !rs->river_index || !rs->outflow_curve_type || !rs->area || !rs->waterlevel)
        return fail("reservoir arrays missing");
    if (m->snow_transport) return fail("gravitational snow transport with reservoirs is not supported");
    m->nres = nres;
    m->res_of_river.assign(nr, -1);
    m->res_land.assign(nres, -1);
    std::vector<int32_t> fed(nr, -1);
    for (int64_t k = 0; k < nres; ++k) {
        const int32_t v = rs->river_index[k];
        if (v < 0 || v >= nr) return fail("reservoir river index out of range");
        if (m->res_of_river[v] >= 0) return fail("two reservoirs at one river cell");
        if (m->r_ds[v] < 0) return fail("a reservoir without a downstream river node is not supported");
        if (fed[m->r_ds[v]] >= 0) return fail("two reservoirs drain into one river cell");
        const int32_t t = rs->outflow_curve_type[k];
        if (t < 1 || t > 4) return fail("unsupported reservoir outflow type");
        if (!(rs->area[k] > 0.0)) return fail("reservoir area must be positive");
        fed[m->r_ds[v]] = (int32_t)k;
        m->res_of_river[v] = (int32_t)k;
        m->res_land[k] = m->r_land[v];
    }
    // upstream lists without the reservoir outlets
    std::vector<int32_t> ds_cut(m->ds), rds_cut(m->r_ds);
    for (int64_t k = 0; k < nres; ++k) {
        ds_cut[m->res_land[k]] = -1;
        rds_cut[rs->river_index[k]] = -1;
    }
    build_ups(n, ds_cut.data(), m->ups);
    build_ups(nr, rds_cut.data(), m->r_ups);
    const double NaN = std::numeric_limits<double>::quiet_NaN();
    auto par = [&](const double* a, int64_t k) { return a ? a[k] : NaN; };
    // tables: per reservoir the S-H table (H then S) and the H-Q table (H then Q), copied
    m->res_sh_at.assign(nres, 0);
    m->res_hq_at.assign(nres, 0);
    m->res_tables.clear();
    if (tb) {
        auto increasing = [](const double* v, int64_t a, int64_t b) {
            for (int64_t i = a + 1; i < b; ++i)
                if (!(v[i] > v[i - 1])) return false;
            for (int64_t i = a; i < b; ++i)
                if (!std::isfinite(v[i])) return false;
            return true;
        };
        for (int64_t k = 0; k < nres; ++k) {
            const int32_t prof = tb->storage_curve_type ? tb->storage_curve_type[k] : 1;
            if (prof != 1 && prof != 2) return fail("unknown reservoir storage curve type");
            if (prof == 2) {
                if (!tb->sh_offset || !tb->sh_h || !tb->sh_s) return fail("reservoir S-H tables missing");
                const int64_t a = tb->sh_offset[k], b = tb->sh_offset[k + 1];
                if (a < 0 || b <= a) return fail("empty reservoir S-H table");
                if (!increasing(tb->sh_h, a, b) || !increasing(tb->sh_s, a, b))
                    return fail("reservoir S-H table not strictly increasing");
                m->res_sh_at[k] = (int64_t)m->res_tables.size();
                m->res_tables.insert(m->res_tables.end(), tb->sh_h + a, tb->sh_h + b);
                m->res_tables.insert(m->res_tables.end(), tb->sh_s + a, tb->sh_s + b);
            }
            if (rs->outflow_curve_type[k] == 1) {
                if (!tb->hq_offset || !tb->hq_h || !tb->hq_q) return fail("reservoir H-Q tables missing");
                const int64_t a = tb->hq_offset[k], b = tb->hq_offset[k + 1];
                if (a < 0 || b <= a) return fail("empty reservoir H-Q table");
                if (!increasing(tb->hq_h, a, b)) return fail("reservoir H-Q table not strictly increasing");
                m->res_hq_at[k] = (int64_t)m->res_tables.size();
                m->res_tables.insert(m->res_tables.end(), tb->hq_h + a, tb->hq_h + b);
                m->res_tables.insert(m->res_tables.end(), tb->hq_q + a * 365, tb->hq_q + b * 365);
            }
            if (tb->lower_reservoir) {
                const int32_t lo = tb->lower_reservoir[k];
                if (lo < -1 || lo >= nres || lo == k) return fail("linked lower reservoir out of range");
            }
        }
    } else {
        for (int64_t k = 0; k < nres; ++k)
            if (rs->outflow_curve_type[k] == 1) return fail("reservoir H-Q tables missing");
    }
    m->res.resize((size_t)M * nres);
    for (int mbr = 0; mbr < M; ++mbr)
        for (int64_t k = 0; k < nres; ++k) {
            OrcReservoir& r = m->res[(size_t)mbr * nres + k];
            r = OrcReservoir{};
            r.outflow_type = rs->outflow_curve_type[k];
            r.area = rs->area[k];
            r.maximum_storage = par(rs->maximum_storage, k);
            r.threshold = par(rs->threshold, k);
            r.rating_curve_coefficient = par(rs->rating_curve_coefficient, k);
            r.rating_curve_exponent = par(rs->rating_curve_exponent, k);
            r.maximum_release = par(rs->maximum_release, k);
            r.demand = par(rs->demand, k);
            r.target_minimum_fraction = par(rs->target_minimum_fraction, k);
            r.target_full_fraction = par(rs->target_full_fraction, k);
            r.external_inflow = 0.0;
            r.precipitation = 0.0;
            r.evaporation = 0.0;
            r.inflow_overland = 0.0;
            r.inflow_subsurface = 0.0;
            r.outflow_obs = NaN;
            r.waterlevel = rs->waterlevel[k];
            r.storage_curve_type = 1;
            r.hq_day = 1;
            if (tb) {
                if (tb->storage_curve_type) r.storage_curve_type = tb->storage_curve_type[k];
                if (tb->lower_reservoir) r.lower = tb->lower_reservoir[k] + 1;
                if (r.storage_curve_type == 2) {
                    const int64_t a = tb->sh_offset[k], b = tb->sh_offset[k + 1];
                    r.sh_n = b - a;
                    r.sh_h = m->res_tables.data() + m->res_sh_at[k];
                    r.sh_s = r.sh_h + r.sh_n;
                }
                if (r.outflow_type == 1) {
                    r.hq_n = tb->hq_offset[k + 1] - tb->hq_offset[k];
                    r.hq_h = m->res_tables.data() + m->res_hq_at[k];
                    r.hq_q = r.hq_h + r.hq_n;
                    r.maximum_storage = rating_curve_maximum_storage(r);
                }
            }
            r.storage = initial_storage(r);
            r.outflow = NaN;
        }
    for (auto* v : {&m->res_out_avg, &m->res_in_avg, &m->res_evap_avg, &m->res_abs_avg, &m->res_prev, &m->res_err,
                    &m->res_rel})
        v->assign((size_t)M * nres, 0.0);
    return WF_OK;
}

int32_t orc_model_set_forcing(OrcModel* m, const double* P, const double* PET, const double* T) {
    int64_t nm = m->n * m->M;
    std::memcpy(m->P.data(), P, nm * 8);
    std::memcpy(m->PET.data(), PET, nm * 8);
    std::memcpy(m->T.data(), T, nm * 8);
    return WF_OK;
}

}  // extern "C"

namespace {

// One member's step. Follows sbm_model.jl:60-92 then mass_balance.jl:541-545; the storage_prev!
// of run_timestep! (Wflow.jl:315) runs first.
// surface_routing! of the local-inertial land and river (surface_routing.jl:62-89) for member 0:
// update_bc_overland_flow_model! (surface_staggered_scheme.jl:1080-1097) then
// update_overland_flow_model! (:1153-1193) without reservoirs; the model's overland and river
// variables then hold the scheme's depths, storages and the discharge of each river cell's
// outgoing edge.
void li_surface_routing(OrcModel* m, const OrcSoil* soil, double dt) {
    OrcLiCoupled& c = *m->li;
    const int64_t n = m->n, nr = m->nr;
    for (int64_t i = 0; i < n; ++i) c.runoff[i] = (soil[i].net_runoff + m->net_runoff_river[i]) * m->area[i];
    for (int64_t r = 0; r < nr; ++r) {
        const int64_t li = m->r_land[r];
        c.runoff[li] += m->ssf_tr_avg[li];  // get_flux_to_river (lateral_subsurface_flow.jl:346-347)
        c.ext[r] = m->r_ext_inflow[r];
    }
    for (auto* v : {&c.q_cum, &c.abstraction_cum, &c.qx_cum, &c.qy_cum}) std::fill(v->begin(), v->end(), 0.0);
    double t = 0.0;
    int64_t k = 0;
    while (t < dt) {
        double dt_s = orc_li_domain_stable_timestep(&c.g, &c.r, &c.st);
        dt_s = check_timestepsize(dt_s, t, dt);
        orc_li_domain_substep(&c.g, &c.r, c.runoff.data(), c.ext.data(), c.abstraction.data(), dt_s, &c.st);
        t += dt_s;
        ++k;
    }
    c.substeps = k;
    for (int64_t e = 0; e < c.r.n_edges; ++e) c.q_avg[e] = c.q_cum[e] / dt;
    for (int64_t i = 0; i <= n; ++i) {
        c.qx_avg[i] = c.qx_cum[i] / dt;
        c.qy_avg[i] = c.qy_cum[i] / dt;
    }
    for (int64_t i = 0; i < n; ++i) {
        m->ol_h[i] = c.h_land[i];
        m->ol_storage[i] = c.storage[i];
        m->ol_q[i] = 0.0;
        m->ol_q_avg[i] = 0.0;
    }
    for (int64_t r = 0; r < nr; ++r) {
        m->rv_h[r] = c.h_river[r];
        m->rv_storage[r] = c.storage_river[r];
        const int64_t e = c.out_edge[r];
        m->rv_q[r] = e >= 0 ? c.q[e] : 0.0;
        m->rv_q_avg[r] = e >= 0 ? c.q_avg[e] : 0.0;
    }
}

// compute_flow_balance! of the local-inertial land and river (mass_balance.jl:402-461): per land
// cell, the x and y discharges, the runoff and at river cells the river edges, the positive
// external inflow and the actual abstraction; no reservoirs.
void li_overland_balance(OrcModel* m, double dt) {
    OrcLiCoupled& c = *m->li;
    double eo[2];
    for (int64_t i = 0; i < m->n; ++i) {
        double tin = 0.0, tout = 0.0;
        for (double q : {c.qx_avg[c.g.ind_x_down[i]], c.qy_avg[c.g.ind_y_down[i]], c.runoff[i]}) {  // add_inflow
            if (q > 0.0) tin += q;
            else tout -= q;
        }
        for (double q : {c.qx_avg[i], c.qy_avg[i]}) {  // add_outflow
            if (q > 0.0) tout += q;
            else tin -= q;
        }
        const int64_t k = c.g.river_index[i];
        if (k >= 0) {
            double q_src = 0.0, q_dst = 0.0;
            for (int64_t e : c.e_in[k]) q_src += c.q_avg[e];
            if (q_src > 0.0) tin += q_src;
            else tout -= q_src;
            tin += jmax(0.0, c.ext[k]);
            for (int64_t e : c.e_out[k]) q_dst += c.q_avg[e];
            if (q_dst > 0.0) tout += q_dst;
            else tin -= q_dst;
            tout += c.abstraction_cum[k] / dt + c.abstraction[k];
        }
        compute_mass_balance_error(tin, tout, (c.storage[i] - m->bo_prev[i]) / dt, eo);
        m->bo_err[i] = eo[0];
        m->bo_rel[i] = eo[1];
    }
}

void member_step(OrcModel* m, int mbr, int n_threads) {
    const WfConfig& c = m->cfg;
    const double dt = c.dt;
    const int64_t n = m->n, nr = m->nr;
    const int64_t o = (int64_t)mbr * n, orr = (int64_t)mbr * nr;
    OrcSoil* soil = m->soil.data() + o;
    for (auto& v : m->sig) {
        if ((int)v.size() != m->M) v.assign(m->M, 0.0);
        v[mbr] = 0.0;
    }
    // ---- storage_prev! (mass_balance.jl:170-183)
    if (c.water_mass_balance) {
        for (int64_t i = 0; i < n; ++i) {
            m->bl_prev[o + i] = soil[i].total_soil_water_storage + m->canopy_storage[o + i] +
                                (m->snow_storage[o + i] + m->snow_water[o + i]) +
                                m->glacier_store[o + i] * m->g_frac[i] + 0.0;
            m->bo_prev[o + i] = m->ol_storage[o + i];
        }
        for (int64_t r = 0; r < nr; ++r) m->br_prev[orr + r] = m->rv_storage[orr + r];
        for (int64_t k = 0; k < m->nres; ++k) m->res_prev[mbr * m->nres + k] = m->res[mbr * m->nres + k].storage;
    }
    // ---- update_land_hydrology_model! (sbm.jl:82-132), per cell
#pragma omp parallel for num_threads(n_threads) schedule(dynamic, 256)
    for (int64_t i = 0; i < n; ++i) {
        const int64_t j = o + i;
        double P = m->P[j], PET = m->PET[j], T = m->T[j];
        double out[5];
        // interception (canopy.jl:213-226 Gash, :259-271 Rutter)
        m->canopy_potevap[j] = m->kc[i] * PET * (1.0 - m->gap[i]);
        if (m->gash) {
            rainfall_interception_gash(m->cmax[i], m->e_r[i], m->gap[i], P, m->canopy_storage[j],
                                       m->canopy_potevap[j], dt, out);
        } else {
            rainfall_interception_modrut(P, m->canopy_potevap[j], m->canopy_storage[j], m->gap[i], m->cmax[i], dt,
                                         out);
        }
        m->throughfall[j] = out[0];
        m->interception_rate[j] = out[1];
        m->stemflow[j] = out[2];
        m->canopy_storage[j] = out[3];
        // snow (snow.jl:238-293)
        if (c.snow) {
            double effective_precip = m->throughfall[j] + m->stemflow[j];
            double sp[2];
            precipitation_hbv(effective_precip, T, m->tti[i], m->tt[i], sp);
            snowpack_hbv(m->snow_storage[j], m->snow_water[j], sp[0], sp[1], T, m->ttm[i], m->ddf[i], m->whc[i], dt,
                         out);
            m->snow_storage[j] = out[0];
            m->snow_water[j] = out[1];
            m->swe[j] = out[2];
            m->snow_melt[j] = out[3];
            m->snow_runoff[j] = out[4];
        } else {
            m->wfs[j] = m->throughfall[j] + m->stemflow[j];  // runoff.jl:37-46
        }
    }
    // ---- lateral_snow_transport! (surface_process.jl:1-19), in the land graph's topological
    // order (sbm.jl:97-99)
    if (m->snow_transport)
        orc_lateral_snow_transport(m->ds.data(), m->ds.data(), m->dfs_order.data(), n, dt, m->slope.data(),
                                   m->snow_storage.data() + o, m->snow_water.data() + o, m->snow_out.data() + o,
                                   m->snow_in.data() + o);
#pragma omp parallel for num_threads(n_threads) schedule(dynamic, 256)
    for (int64_t i = 0; i < n; ++i) {
        const int64_t j = o + i;
        const double PET = m->PET[j], T = m->T[j];
        double out[5];
        // update_glacier_model! (glacier.jl:122-154, sbm.jl:102)
        if (m->glacier) {
            glacier_hbv(m->g_frac[i], m->glacier_store[j], m->snow_storage[j], T, m->g_ttm[i], m->g_ddf[i],
                        m->g_sifrac[i], 8.0 * MM_PER_DAY_FACTOR, dt, out);
            m->snow_storage[j] = out[0];
            m->glacier_store[j] = out[2];
            m->glacier_melt[j] = out[3];
        }
        // water flux at the surface (runoff.jl:49-58)
        if (c.snow) m->wfs[j] = m->snow_runoff[j] + m->glacier_melt[j] * m->g_frac[i];
        const double wfs_runoff = m->wfs[j];
        // open water runoff (runoff.jl:61-111)
        double wd_land = m->ol_h[j];
        int32_t r = m->land_river[i];
        double wd_river = r >= 0 ? m->rv_h[orr + r] : 0.0;
        m->runoff_river[j] = jmin(1.0, m->river_fraction[i]) * wfs_runoff;
        m->runoff_land[j] = jmin(1.0, m->water_fraction[i]) * wfs_runoff;
        m->ae_river[j] = m->river_fraction[i] * jmin(wd_river / dt, PET);
        m->ae_land[j] = m->water_fraction[i] * jmin(wd_land / dt, PET);
        m->net_runoff_river[j] = m->runoff_river[j] - m->ae_river[j];
        // soil_fraction! (soil.jl:643-655)
        OrcSoil& s = soil[i];
        s.soil_fraction = jmax(m->gap[i] - m->water_fraction[i] - m->river_fraction[i] - m->g_frac[i], 0.0);
        update_bc_soil_model(s, m->canopy_potevap[j], m->interception_rate[j], PET, wfs_runoff, m->runoff_river[j],
                             m->runoff_land[j]);
        update_soil_water_flow(s, T, c.snow != 0, c.soil_infiltration_reduction != 0, m->ae_river[j], m->ae_land[j],
                               dt);
        s.actual_evapotranspiration += m->interception_rate[j];  // sbm.jl:130
        // sbm_model.jl:74-81
        m->rch_rate[j] = s.recharge;
        m->ssf_zi[j] = s.water_table_depth;
    }
    // ---- update_subsurface_flow_model! (lateral_subsurface_flow.jl:279-304)
    for (int64_t i = 0; i < n; ++i) {
        m->ssf_tr_cum[o + i] = 0.0;
        m->rch_flux_cum[o + i] = 0.0;  // set_flux_vars! (groundwater.jl:606-620)
        m->ssf_exf_cum[o + i] = 0.0;
        m->ssf_qin_cum[o + i] = 0.0;
        m->ssf_q_cum[o + i] = 0.0;
        m->ssf_qnet_cum[o + i] = 0.0;
    }
    {
        double t = 0.0;
        int64_t nsub = 0;
        while (t < dt) {
            for (int64_t i = 0; i < n; ++i) m->ssf_qnet[o + i] = 0.0;
            double dt_s;
            if (c.adaptive_timestep) {
                // stable_timestep (lateral_subsurface_flow.jl:314-344)
                double dtmin = INFINITY;
                int64_t k = 0;
                for (int64_t i = 0; i < n; ++i) {
                    double zi = m->ssf_zi[o + i];
                    if (zi > 0.0) {
                        k++;
                        double cel = ssf_celerity(zi, m->slope[i], m->sy[i], m->kh0[o + i], m->ssf_f[o + i],
                                                  c.kv_profile, m->z_exp[i]);
                        double v = m->flow_length[i] / cel;
                        dtmin = (k == 1) ? v : jmin(dtmin, v);
                    }
                }
                dt_s = (k > 0 ? dtmin : 0.5) * c.subsurface_alpha;
            } else {
                dt_s = c.subsurface_dt_fixed;
            }
            dt_s = check_timestepsize(dt_s, t, dt);
            m->sig[0][mbr] += dt_s * dt_s;  // sub-step signature (a diagnostic)
            // update_fluxes! -> recharge flux! (boundary_conditions.jl:219-236, check_flux :12-21)
            for (int64_t i = 0; i < n; ++i) {
                int64_t j = o + i;
                double flux = m->rch_rate[j] * m->area[i];
                if (m->ssf_zi[j] >= soil[i].soil_thickness) flux = jmax(0.0, flux);
                m->rch_flux[j] = flux;
                m->rch_flux_cum[j] += flux * dt_s;
                m->ssf_qnet[j] += flux;
            }
            // kinwave_subsurface_update! (lateral_subsurface_flow.jl:198-273)
            for (int64_t v : m->topo) {
                int64_t j = o + v;
                double qin = 0.0, tr = 0.0;
                for (int32_t u : m->ups[v]) qin = qin + m->ssf_q[o + u] * (1.0 - m->frac_to_river[u]);
                for (int32_t u : m->ups[v]) tr = tr + m->ssf_q[o + u] * m->frac_to_river[u];
                m->ssf_qin[j] = qin;
                m->ssf_tr_cum[j] += tr * dt_s;
                double r4[4];
                kinematic_wave_ssf(m->ssf_qin[j], m->ssf_q[j], m->ssf_zi[j], m->ssf_qnet[j], m->slope[v], m->sy[v],
                                   soil[v].soil_thickness, dt_s, m->flow_length[v], m->flow_width[v], m->q_max[j],
                                   m->kh0[j], m->ssf_f[j], c.kv_profile, m->z_exp[v], soil[v], r4);
                m->ssf_q[j] = r4[0];
                m->ssf_zi[j] = r4[1];
                m->ssf_qin_cum[j] += m->ssf_qin[j] * dt_s;
                m->ssf_q_cum[j] += m->ssf_q[j] * dt_s;
                m->ssf_exf_cum[j] += r4[2] * dt_s;
                m->ssf_qnet_cum[j] += r4[3] * m->area[v] * dt_s;
                m->ssf_head[j] = m->top[v] - m->ssf_zi[j];
                m->ssf_storage[j] = m->sy[v] * (soil[v].soil_thickness - m->ssf_zi[j]) * m->area[v];
            }
            t += dt_s;
            nsub++;
        }
        if (mbr == 0) m->last_sub_ssf = nsub;
    }
    for (int64_t i = 0; i < n; ++i) {  // average_flux_vars! (groundwater.jl:622-638), flux_to_river!
        int64_t j = o + i;
        m->rch_flux_avg[j] = m->rch_flux_cum[j] / dt;
        m->ssf_qin_avg[j] = m->ssf_qin_cum[j] / dt;
        m->ssf_q_avg[j] = m->ssf_q_cum[j] / dt;
        m->ssf_qnet_avg[j] = m->ssf_qnet_cum[j] / dt;
        m->ssf_exf_avg[j] = m->ssf_exf_cum[j] / dt;
        m->ssf_tr_avg[j] = m->ssf_tr_cum[j] / dt;
    }
    // ---- update_soil_water_storage! (soil.jl:1294-1392)
#pragma omp parallel for num_threads(n_threads) schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        int64_t j = o + i;
        update_soil_water_storage(soil[i], m->ssf_exf_avg[j], m->runoff_land[j], m->ae_land[j], dt);
    }
    OrcReservoir* res = m->nres ? m->res.data() + (size_t)mbr * m->nres : nullptr;
    if (m->li) {
        li_surface_routing(m, soil, dt);
    } else {
    // ---- surface_routing! (surface_routing.jl:7-46)
    // overland lateral inflow (surface_kinwave.jl:740-766)
    for (int64_t i = 0; i < n; ++i) {
        int64_t j = o + i;
        m->ol_inwater[j] = (soil[i].net_runoff + 0.0) * m->area[i] + 0.0;
        m->ol_qlat[j] = m->ol_inwater[j] / m->flow_length[i];  // :365
        m->ol_q_cum[j] = 0.0;
        m->ol_qin_cum[j] = 0.0;
        m->ol_tr_cum[j] = 0.0;
    }
    {
        double t = 0.0;
        int64_t nsub = 0;
        while (t < dt) {
            double dt_s = c.adaptive_timestep ? kinwave_stable_timestep(m->ol_q.data() + o, m->ol_alpha.data(),
                                                                        m->flow_length.data(), n, 0.02, m->buf)
                                              : c.land_dt_fixed;
            dt_s = check_timestepsize(dt_s, t, dt);
            m->sig[1][mbr] += dt_s * dt_s;  // sub-step signature (a diagnostic)
            // kinwave_land_update! (surface_kinwave.jl:293-341)
            for (int64_t i = 0; i < n; ++i) m->ol_qin[o + i] = 0.0;
            for (int64_t v : m->topo) {
                int64_t j = o + v;
                double tr = 0.0;
                for (int32_t u : m->ups[v]) tr = tr + m->ol_q[o + u] * m->frac_to_river[u];
                m->ol_tr_cum[j] += tr * dt_s;
                if (m->sfw[v] > 0.0) {
                    double qin = 0.0;
                    for (int32_t u : m->ups[v]) qin = qin + m->ol_q[o + u] * (1.0 - m->frac_to_river[u]);
                    m->ol_qin[j] = qin;
                }
                double kw[2];
                kinematic_wave(m->ol_qin[j], m->ol_q[j], m->ol_qlat[j], m->ol_alpha[v], dt_s, m->flow_length[v], kw);
                m->ol_q[j] = kw[0];
                if (m->sfw[v] > 0.0) m->ol_h[j] = kw[1] / m->sfw[v];
                m->ol_storage[j] = m->flow_length[v] * m->sfw[v] * m->ol_h[j];
                m->ol_q_cum[j] += m->ol_q[j] * dt_s;
                m->ol_qin_cum[j] += m->ol_qin[j] * dt_s;
            }
            t += dt_s;
            nsub++;
        }
        if (mbr == 0) m->last_sub_land = nsub;
    }
    for (int64_t i = 0; i < n; ++i) {
        int64_t j = o + i;
        m->ol_q_avg[j] = m->ol_q_cum[j] / dt;
        m->ol_tr_avg[j] = m->ol_tr_cum[j] / dt;
        m->ol_qin_avg[j] = m->ol_qin_cum[j] / dt;
    }
    // river lateral inflow (surface_kinwave.jl:710-734)
    for (int64_t r = 0; r < nr; ++r) {
        int64_t li = m->r_land[r];
        int64_t j = o + li;
        m->rv_inwater[orr + r] = (m->ssf_tr_avg[j] + m->ol_tr_avg[j] + m->net_runoff_river[j] * m->area[li] + 0.0);
        m->rv_qlat[orr + r] = m->rv_inwater[orr + r] / m->r_length[r];  // :625
        m->rv_q_cum[orr + r] = 0.0;
        m->rv_abs_cum[orr + r] = 0.0;
        m->rv_qin_cum[orr + r] = 0.0;
    }
    // reservoir inflow from the outlet cell's overland and subsurface flow (update_inflow!,
    // surface_kinwave.jl:771-802) and the reset of the step's cumulatives (set_reservoir_vars!,
    // :227-237)
    for (int64_t k = 0; k < m->nres; ++k) {
        OrcReservoir& r = res[k];
        r.inflow_overland = m->ol_q_avg[o + m->res_land[k]];
        r.inflow_subsurface = m->ssf_q_avg[o + m->res_land[k]];
        r.inflow_cumulative = 0.0;
        r.abstraction_cumulative = 0.0;
        r.outflow_cumulative = 0.0;
        r.actevap_cumulative = 0.0;
    }
    {
        double t = 0.0;
        int64_t nsub = 0;
        while (t < dt) {
            double dt_s = c.adaptive_timestep ? kinwave_stable_timestep(m->rv_q.data() + orr, m->r_alpha.data(),
                                                                        m->r_length.data(), nr, 0.05, m->buf)
                                              : c.river_dt_fixed;
            dt_s = check_timestepsize(dt_s, t, dt);
            m->sig[2][mbr] += dt_s * dt_s;  // sub-step signature (a diagnostic)
            // kinwave_river_update! (surface_kinwave.jl:492-566)
            for (int64_t r = 0; r < nr; ++r) m->rv_qin[orr + r] = 0.0;
            for (int64_t v : m->r_topo) {
                int64_t j = orr + v;
                double s = 0.0;
                for (int32_t u : m->r_ups[v]) s = s + m->rv_q[orr + u];
                m->rv_qin[j] += s;
                double inflow;
                double ext = m->r_ext_inflow[v];
                if (ext < 0.0) {
                    double abstraction = jmin(-ext, (m->rv_storage[j] / dt_s) * 0.80);
                    m->rv_abs_cum[j] += abstraction * dt_s;
                    inflow = -abstraction / m->r_length[v];
                } else {
                    inflow = ext / m->r_length[v];
                }
                inflow -= 0.0 / m->r_length[v];
                double kw[2];
                kinematic_wave(m->rv_qin[j], m->rv_q[j], m->rv_qlat[j] + inflow, m->r_alpha[v], dt_s, m->r_length[v],
                               kw);
                m->rv_q[j] = kw[0];
                if (m->nres && m->res_of_river[v] >= 0) {
                    // update_reservoir_model! (surface_kinwave.jl:441-489): the reservoir outflow
                    // is the inflow of the downstream river cell
                    const int32_t k = m->res_of_river[v];
                    update_reservoir_at_node(res, k, m->rv_q[j], dt_s);
                    m->rv_qin[orr + m->r_ds[v]] = res[k].outflow;
                }
                m->rv_h[j] = kw[1] / m->r_width[v];
                m->rv_storage[j] = m->r_length[v] * kw[1];
                m->rv_q_cum[j] += m->rv_q[j] * dt_s;
                m->rv_qin_cum[j] += m->rv_qin[j] * dt_s;
            }
            t += dt_s;
            nsub++;
        }
        if (mbr == 0) m->last_sub_river = nsub;
    }
    for (int64_t r = 0; r < nr; ++r) {
        m->rv_q_avg[orr + r] = m->rv_q_cum[orr + r] / dt;
        m->rv_abs_avg[orr + r] = m->rv_abs_cum[orr + r] / dt;
        m->rv_qin_avg[orr + r] = m->rv_qin_cum[orr + r] / dt;
    }
    for (int64_t k = 0; k < m->nres; ++k) {  // average_reservoir_vars! (surface_kinwave.jl:244-258)
        const int64_t q = (int64_t)mbr * m->nres + k;
        m->res_out_avg[q] = res[k].outflow_cumulative / dt;
        m->res_in_avg[q] = res[k].inflow_cumulative / dt;
        m->res_abs_avg[q] = res[k].abstraction_cumulative / dt;
    }
    }  // kinematic-wave surface routing
    // ---- update_total_water_storage! (sbm.jl:143-182)
    for (int64_t i = 0; i < n; ++i) m->total_storage[o + i] = 0.0;
    for (int64_t r = 0; r < nr; ++r) {
        int64_t li = m->r_land[r];
        m->total_storage[o + li] = ((m->rv_h[orr + r] * m->r_width[r] * m->r_length[r]) / (m->area[li]));
    }
    for (int64_t i = 0; i < n; ++i) {
        int64_t j = o + i;
        m->total_storage[j] += m->snow_storage[j] + m->snow_water[j] + m->glacier_store[j] * m->g_frac[i] +
                               m->canopy_storage[j] + 0.0;
        double sub_surface = soil[i].unsaturated_store_depth + soil[i].saturated_water_depth;
        double lateral = m->ol_h[j] * (1.0 - m->river_fraction[i]);
        m->total_storage[j] += sub_surface + lateral;
    }
    // ---- compute_mass_balance! (mass_balance.jl:541-545)
    if (c.water_mass_balance) {
        double eo[2];
        for (int64_t i = 0; i < n; ++i) {  // compute_land_hydrology_balance! :215-253
            int64_t j = o + i;
            double area_i = m->area[i];
            double subsurface_flux_in = m->ssf_qin_avg[j] / area_i;
            double total_in = subsurface_flux_in + (m->P[j] + 0.0) + m->snow_in[j] + 0.0 / m->area[i];
            double subsurface_flux_out = m->ssf_q_avg[j] / area_i;
            const OrcSoil& s = soil[i];
            double vertical_flux_out =
                s.net_runoff + s.actual_evapotranspiration + m->net_runoff_river[j] + s.actual_leakage + 0.0;
            double total_out = subsurface_flux_out + vertical_flux_out + m->snow_out[j] + 0.0 / m->area[i];
            double storage = s.total_soil_water_storage + m->canopy_storage[j] +
                             (m->snow_storage[j] + m->snow_water[j]) + m->glacier_store[j] * m->g_frac[i] + 0.0;
            double storage_rate = (storage - m->bl_prev[j]) / dt;
            compute_mass_balance_error(total_in, total_out, storage_rate, eo);
            m->bl_err[j] = eo[0];
            m->bl_rel[j] = eo[1];
        }
        for (int64_t r = 0; r < nr && m->li; ++r) {  // local-inertial routing: no river balance (:516-536)
            m->br_err[orr + r] = 0.0;
            m->br_rel[orr + r] = 0.0;
        }
        for (int64_t r = 0; r < nr && !m->li; ++r) {  // river :290-313
            int64_t j = orr + r;
            double total_in = m->rv_inwater[j] + m->rv_qin_avg[j] + jmax(0.0, m->r_ext_inflow[r]);
            double total_out = m->rv_q_avg[j] + m->rv_abs_avg[j] + 0.0;
            double storage_rate = (m->rv_storage[j] - m->br_prev[j]) / dt;
            compute_mass_balance_error(total_in, total_out, storage_rate, eo);
            m->br_err[j] = eo[0];
            m->br_rel[j] = eo[1];
        }
        for (int64_t k = 0; k < m->nres; ++k) {  // reservoir :261-284
            const int64_t q = (int64_t)mbr * m->nres + k;
            const OrcReservoir& r = res[k];
            m->res_in_avg[q] = r.inflow_cumulative / dt;
            m->res_evap_avg[q] = r.actevap_cumulative / dt;
            double total_in = m->res_in_avg[q] + r.precipitation * r.area;
            double total_out = m->res_out_avg[q] + m->res_evap_avg[q] * r.area;
            double storage_rate = (r.storage - m->res_prev[q]) / dt;
            compute_mass_balance_error(total_in, total_out, storage_rate, eo);
            m->res_err[q] = eo[0];
            m->res_rel[q] = eo[1];
        }
        if (m->li) li_overland_balance(m, dt);
        for (int64_t i = 0; i < n && !m->li; ++i) {  // overland :382-399
            int64_t j = o + i;
            double total_in = m->ol_inwater[j] + m->ol_qin_avg[j];
            double total_out = m->ol_q_avg[j];
            double storage_rate = (m->ol_storage[j] - m->bo_prev[j]) / dt;
            compute_mass_balance_error(total_in, total_out, storage_rate, eo);
            m->bo_err[j] = eo[0];
            m->bo_rel[j] = eo[1];
        }
        for (int64_t i = 0; i < n; ++i) {  // subsurface :470-490 with sum_boundary_fluxes (groundwater.jl:671-695)
            int64_t j = o + i;
            double flux = m->rch_flux_avg[j];
            double flux_in = 0.0, flux_out = 0.0;
            if (flux > 0.0) flux_in += flux; else flux_out -= flux;
            double total_in = m->ssf_qin_avg[j] + flux_in;
            double total_out = m->ssf_q_avg[j] + flux_out;
            compute_mass_balance_error(total_in, total_out, m->ssf_qnet_avg[j], eo);
            m->bs_err[j] = eo[0];
            m->bs_rel[j] = eo[1];
        }
    }
}

}  // namespace

// ============================================================ lateral snow transport ======
//
// Transport of material downstream with a capacity-limited flux over the drainage graph in
// topological order (accucapacityflux!, routing/utils.jl:82-110): each node passes
// min(material / dt, capacity) downstream (a pit passes it out of the domain); and the lateral
// snow transport built on it (lateral_snow_transport!, routing/surface/surface_process.jl:1-19):
// a slope- and storage-dependent fraction of the dry snow and of the liquid water in the snow
// moves downhill each step, the inflow of a cell being the sum of its upstream cells' outflow
// (flux_in!, routing/utils.jl:160-166).
namespace {

void accucapacityflux(const int32_t* ds, const int64_t* order, int64_t n, double dt, const double* capacity,
                      double* material, double* flux) {
    for (int64_t k = 0; k < n; ++k) {
        const int64_t v = order[k];
        const double flux_val = jmin(material[v] / dt, capacity[v]);
        const double update = flux_val * dt;
        material[v] -= update;
        flux[v] = flux_val;
        if (ds[v] >= 0) material[ds[v]] += update;
    }
}

}  // namespace

extern "C" {
// accucapacityflux!: material is updated in place, flux overwritten.
void orc_accucapacityflux(const int32_t* ds, const int64_t* order, int64_t n, double dt, const double* capacity,
                          double* material, double* flux) {
    accucapacityflux(ds, order, n, dt, capacity, material, flux);
}

// lateral_snow_transport!: snow_out and snow_in [m s-1] of every cell, and the snow storage and
// snow water moved downhill in place (the non-mutating-named accucapacityflux passes its
// material to accucapacityflux!, routing/utils.jl:144-148, so Wflow's snow states move); the
// fraction and both capacities come from the states before the move. The graph's upstream
// lists for the inflow are `ups_ds` (the reservoir-cut lists of the domain; equal to ds
// without reservoirs).
void orc_lateral_snow_transport(const int32_t* ds, const int32_t* ups_ds, const int64_t* order, int64_t n, double dt,
                                const double* slope, double* snow_storage, double* snow_water, double* snow_out,
                                double* snow_in) {
    const double TAN80 = 5.67;
    const double snow_storage_max = 10.0;
    std::vector<double> frac(n), maxflux(n), f2(n), cap2(n);
    for (int64_t i = 0; i < n; ++i) {
        frac[i] = jmin(0.5, slope[i] / TAN80) * jmin(1.0, snow_storage[i] / snow_storage_max);
        maxflux[i] = frac[i] * snow_storage[i] / dt;
    }
    accucapacityflux(ds, order, n, dt, maxflux.data(), snow_storage, snow_out);
    for (int64_t i = 0; i < n; ++i) cap2[i] = snow_water[i] * frac[i] / dt;
    accucapacityflux(ds, order, n, dt, cap2.data(), snow_water, f2.data());
    for (int64_t i = 0; i < n; ++i) snow_out[i] += f2[i];
    std::vector<std::vector<int64_t>> ups(n);  // upstream lists in ascending node order
    for (int64_t i = 0; i < n; ++i)
        if (ups_ds[i] >= 0) ups[ups_ds[i]].push_back(i);
    for (int64_t v = 0; v < n; ++v) {
        double acc = 0.0;
        for (int64_t u : ups[v]) acc = acc + snow_out[u];
        snow_in[v] = acc;
    }
}
}  // extern "C"

// ============================================================ local-inertial river =======
//
// River flow on a staggered grid by the local-inertial approximation (de Almeida et al. 2012):
// discharge on the edges between river cells from the water-surface slope, friction and the
// previous discharge (local_inertial_flow, routing/surface/surface_process.jl:88-163), water
// depth on the cells from the edge discharges (update_water_depth_and_storage!,
// routing/surface/surface_staggered_scheme.jl:723-760), edges first (update_river_channel_flow!,
// :326-385), and the stable time step min over cells of alpha dx / sqrt(g h) (:1004-1020).
// Channel only (no floodplain, no reservoirs at edges).
namespace {

constexpr double GRAVITY = 9.80665;

// local_inertial_flow, general cross-section (surface_process.jl:88-115)
double li_flow_area(double q0, double zs0, double zs1, double hf, double A, double R, double length,
                    double mannings_n_sq, bool froude_limit, double dt) {
    const double slope = (zs1 - zs0) / length;
    const double pow_R = wcbrt(R * R * R * R);
    double q = (q0 - GRAVITY * A * dt * slope) / (1.0 + GRAVITY * dt * mannings_n_sq * std::fabs(q0) / (pow_R * A));
    const double fr = ((q / A) / std::sqrt(GRAVITY * hf)) * (froude_limit ? 1.0 : 0.0);
    if (std::fabs(fr) > 1.0 && q > 0.0) q = std::sqrt(GRAVITY * hf) * A;
    if (std::fabs(fr) > 1.0 && q < 0.0) q = -std::sqrt(GRAVITY * hf) * A;
    return q;
}

// local_inertial_flow, rectangular cross-section with the theta weighting (:124-163)
double li_flow_rect(double theta, double q0, double qd, double qu, double zs0, double zs1, double hf, double width,
                    double length, double mannings_n_sq, bool froude_limit, double dt) {
    const double slope = (zs1 - zs0) / length;
    const double pow_hf = wcbrt(hf * hf * hf * hf * hf * hf * hf);
    double q = ((theta * q0 + 0.5 * (1.0 - theta) * (qu + qd)) - GRAVITY * hf * width * dt * slope) /
               (1.0 + GRAVITY * dt * mannings_n_sq * std::fabs(q0) / (pow_hf * width));
    if (froude_limit) {
        const double fr = (q / width / hf) / std::sqrt(GRAVITY * hf);
        if (std::fabs(fr) > 1.0 && q > 0.0) q = hf * std::sqrt(GRAVITY * hf) * width;
        else if (std::fabs(fr) > 1.0 && q < 0.0) q = -hf * std::sqrt(GRAVITY * hf) * width;
    }
    return q;
}

}  // namespace

extern "C" {

double orc_li_flow_area(double q0, double zs0, double zs1, double hf, double A, double R, double length,
                        double mannings_n_sq, int32_t froude_limit, double dt) {
    return li_flow_area(q0, zs0, zs1, hf, A, R, length, mannings_n_sq, froude_limit != 0, dt);
}

double orc_li_flow_rect(double theta, double q0, double qd, double qu, double zs0, double zs1, double hf,
                        double width, double length, double mannings_n_sq, int32_t froude_limit, double dt) {
    return li_flow_rect(theta, q0, qd, qu, zs0, zs1, hf, width, length, mannings_n_sq, froude_limit != 0, dt);
}

// One local-inertial river step over n cells and n_edges edges (edge k from src[k] to dst[k],
// in the graph's edge order); the first n_active cells are updated (the others are boundary
// cells of fixed depth). Arrays: zb, flow_length, flow_width, inwater [n]; zb_e, width_e,
// length_e, nsq_e [n_edges]; state h, storage [n], q, q_prev, q_cum [n_edges]; abstraction,
// external_inflow, error and abstraction_cum [n] (update_water_depth_and_storage!, :723-760;
// each may be NULL: zero inflows, nothing recorded).
// update_river_channel_flow! (:326-385): the discharge of every river edge
static void li_river_edges(int64_t n_edges, const int64_t* src, const int64_t* dst, const double* zb,
                           const double* zb_e, const double* width_e, const double* length_e, const double* nsq_e,
                           double h_thresh, int32_t froude_limit, double dt, const double* h, double* q,
                           double* q_prev, double* q_cum) {
    for (int64_t k = 0; k < n_edges; ++k) q_prev[k] = q[k];
    for (int64_t k = 0; k < n_edges; ++k) {
        const int64_t a = src[k], b = dst[k];
        const double zs_src = zb[a] + h[a];
        const double zs_dst = zb[b] + h[b];
        const double zs_e = jmax(zs_src, zs_dst);
        const double hf = zs_e - zb_e[k];
        const double A = width_e[k] * hf;
        const double R = A / (2.0 * hf + width_e[k]);
        double qk = hf > h_thresh ? li_flow_area(q_prev[k], zs_src, zs_dst, hf, A, R, length_e[k], nsq_e[k],
                                                 froude_limit != 0, dt)
                                  : 0.0;
        if (h[a] <= 0.0) qk = jmin(qk, 0.0);
        if (h[b] <= 0.0) qk = jmax(qk, 0.0);
        q[k] = qk;
        q_cum[k] += qk * dt;
    }
}

static void li_river_cells(int64_t n, int64_t n_active, int64_t n_edges, const int64_t* src, const int64_t* dst,
                           const double* flow_length, const double* flow_width, const double* inwater, double dt,
                           double* h, double* storage, const double* q, const double* abstraction,
                           const double* external_inflow, double* error, double* abstraction_cum);

void orc_li_river_step(int64_t n, int64_t n_active, int64_t n_edges, const int64_t* src, const int64_t* dst,
                       const double* zb, const double* flow_length, const double* flow_width, const double* inwater,
                       const double* zb_e, const double* width_e, const double* length_e, const double* nsq_e,
                       double h_thresh, int32_t froude_limit, double dt, double* h, double* storage, double* q,
                       double* q_prev, double* q_cum, const double* abstraction, const double* external_inflow,
                       double* error, double* abstraction_cum) {
    li_river_edges(n_edges, src, dst, zb, zb_e, width_e, length_e, nsq_e, h_thresh, froude_limit, dt, h, q, q_prev,
                   q_cum);
    li_river_cells(n, n_active, n_edges, src, dst, flow_length, flow_width, inwater, dt, h, storage, q, abstraction,
                   external_inflow, error, abstraction_cum);
}

// Manning's equation on the staggered grid (river_routing = "manning_staggered"): the edge update
// of update_river_channel_flow! (surface_staggered_scheme.jl:386-434; upwind depth, the
// discharge limited to the upstream storage over dt; manning_flow, surface_process.jl:166-169),
// then the same cell update as the local-inertial river.
void orc_manning_river_step(int64_t n, int64_t n_active, int64_t n_edges, const int64_t* src, const int64_t* dst,
                            const double* flow_length, const double* flow_width, const double* inwater,
                            const double* width_e, const double* slope_e, const double* n_e, double h_thresh,
                            double dt, double* h, double* storage, double* q, double* q_cum, double* hf_e,
                            const double* abstraction, const double* external_inflow, double* error,
                            double* abstraction_cum) {
    for (int64_t k = 0; k < n_edges; ++k) {
        const int64_t a = src[k];
        const double hf = h[a];
        hf_e[k] = hf;
        const double A = width_e[k] * hf;
        const double R = A / (2.0 * hf + width_e[k]);
        double qk = hf > h_thresh ? ((wcbrt(R * R) * std::sqrt(slope_e[k])) * A) / n_e[k] : 0.0;
        qk = jmin(qk, storage[a] / dt);
        q[k] = qk;
        q_cum[k] += qk * dt;
    }
    li_river_cells(n, n_active, n_edges, src, dst, flow_length, flow_width, inwater, dt, h, storage, q, abstraction,
                   external_inflow, error, abstraction_cum);
}

// stable_timestep of the Manning river (:1050-1075): wave celerity of a wide rectangular channel
// at each edge's last depth, 60 s when every edge is dry
double orc_manning_stable_timestep(int64_t n_edges, const double* width_e, const double* length_e,
                                   const double* slope_e, const double* n_e, const double* hf_e, double alpha) {
    double dt_min = std::numeric_limits<double>::infinity();
    for (int64_t k = 0; k < n_edges; ++k) {
        const double h_r = (width_e[k] * hf_e[k]) / (2.0 * hf_e[k] + width_e[k]);
        const double celerity = ((wcbrt(h_r * h_r) * std::sqrt(slope_e[k])) / n_e[k]) / 0.6;
        const double dt = alpha * length_e[k] / celerity;
        dt_min = jmin(dt, dt_min);
    }
    return std::isinf(dt_min) ? 60.0 : dt_min;
}

// update_water_depth_and_storage! (:723-760), edges into / out of each cell in edge order
static void li_river_cells(int64_t n, int64_t n_active, int64_t n_edges, const int64_t* src, const int64_t* dst,
                           const double* flow_length, const double* flow_width, const double* inwater, double dt,
                           double* h, double* storage, const double* q, const double* abstraction,
                           const double* external_inflow, double* error, double* abstraction_cum) {
    std::vector<double> qin(n, 0.0), qout(n, 0.0);
    for (int64_t k = 0; k < n_edges; ++k) {
        qin[dst[k]] = qin[dst[k]] + q[k];
        qout[src[k]] = qout[src[k]] + q[k];
    }
    for (int64_t i = 0; i < n_active; ++i) {  // NULL boundary arrays: zero
        const double abs_i = abstraction ? abstraction[i] : 0.0;
        const double ext_i = external_inflow ? external_inflow[i] : 0.0;
        storage[i] += (qin[i] - qout[i] + inwater[i] - abs_i) * dt;
        if (storage[i] < 0.0) {
            if (error) error[i] = error[i] + std::fabs(storage[i]);
            storage[i] = 0.0;
        }
        double inflow = ext_i;
        if (ext_i < 0.0) {  // limit negative external inflow
            const double taken = jmin(-ext_i, storage[i] / dt * 0.80);
            if (abstraction_cum) abstraction_cum[i] += taken * dt;
            inflow = -taken;
        }
        storage[i] += inflow * dt;
        h[i] = storage[i] / (flow_length[i] * flow_width[i]);
    }
}

// ---- 2D overland local-inertial flow with a subgrid river (surface_staggered_scheme.jl
// :1022-1040, 1202-1265, 1322-1546). Index arrays are 0-based; index n is the ghost cell
// outside the grid (discharge arrays hold n + 1 values, the ghost's staying 0).

// stable_timestep of the overland flow: cells without a river (:1022-1040)
double orc_li_land_stable_timestep(int64_t n, const double* x_length, const double* y_length,
                                   const int32_t* river_location, const double* h, double alpha) {
    double dt_min = std::numeric_limits<double>::infinity();
    for (int64_t i = 0; i < n; ++i) {
        const double dt = river_location[i] == 0 ? alpha * jmin(x_length[i], y_length[i]) / std::sqrt(GRAVITY * h[i])
                                                 : std::numeric_limits<double>::infinity();
        dt_min = jmin(dt, dt_min);
    }
    return std::isinf(dt_min) ? 60.0 : dt_min;
}

// update_directional_flow! at cell i for one direction (:1202-1265): up / down are the
// direction's upstream and downstream neighbour indices, width_e / zmax_e / nsq_e the edge
// arrays, length the cell lengths along the direction.
void orc_li_directional_flow(int64_t i, int64_t n, const int64_t* up, const int64_t* down, const double* width_e,
                             const double* zmax_e, const double* length, const double* z, const double* h,
                             const double* nsq_e, double theta, double h_thresh, int32_t froude_limit, double dt,
                             double* q, const double* q_prev, double* q_cum) {
    const int64_t u = up[i];
    if (!(u < n && width_e[i] != 0.0)) return;
    const double zs_current = z[i] + h[i];
    const double zs_upstream = z[u] + h[u];
    const double zs_max = jmax(zs_current, zs_upstream);
    const double hf = zs_max - zmax_e[i];
    if (hf > h_thresh) {
        const double length_e = 0.5 * (length[i] + length[u]);
        double qi = li_flow_rect(theta, q_prev[i], q_prev[down[i]], q_prev[u], zs_current, zs_upstream, hf,
                                 width_e[i], length_e, nsq_e[i], froude_limit != 0, dt);
        if (h[i] <= 0.0) qi = jmin(qi, 0.0);
        if (h[u] <= 0.0) qi = jmax(qi, 0.0);
        q[i] = qi;
    } else {
        q[i] = 0.0;
    }
    q_cum[i] += q[i] * dt;
}

// compute_land_storage_change (:1420-1433)
double orc_li_land_storage_change(int64_t i, const double* qx, const double* qy, const int64_t* ind_x_down,
                                  const int64_t* ind_y_down, const double* runoff, double dt) {
    return (qx[ind_x_down[i]] - qx[i] + qy[ind_y_down[i]] - qy[i] + runoff[i]) * dt;
}

// compute_river_storage_change at a cell holding river cell r (:1322-1351): river discharge of
// the edges into and out of r, overland fluxes, runoff and abstraction
double orc_li_river_storage_change(int64_t i, const double* q_river, const int64_t* e_in, int64_t n_in,
                                   const int64_t* e_out, int64_t n_out, const double* qx, const double* qy,
                                   const int64_t* ind_x_down, const int64_t* ind_y_down, const double* runoff,
                                   double abstraction, double dt) {
    double s_in = 0.0, s_out = 0.0;
    for (int64_t k = 0; k < n_in; ++k) s_in = s_in + q_river[e_in[k]];
    for (int64_t k = 0; k < n_out; ++k) s_out = s_out + q_river[e_out[k]];
    const double net_river_flow = s_in - s_out;
    const double net_land_flow = qx[ind_x_down[i]] - qx[i] + qy[ind_y_down[i]] - qy[i];
    const double net_flow = net_river_flow + net_land_flow + runoff[i] - abstraction;
    return net_flow * dt;
}

// compute_external_inflow (:1358-1380): out2 = inflow, abstraction
void orc_li_external_inflow(double external_inflow, double land_storage, double bankfull_storage,
                            double river_storage, double dt, double* out2) {
    if (external_inflow < 0.0) {
        const double available = land_storage >= bankfull_storage ? bankfull_storage : river_storage;
        const double a = jmin(-external_inflow, available / dt * 0.80);
        out2[0] = -a;
        out2[1] = a;
    } else {
        out2[0] = external_inflow;
        out2[1] = 0.0;
    }
}

// compute_water_depths (:1386-1414): out3 = river depth, land depth, river storage
void orc_li_water_depths(double total_storage, double bankfull_storage, double bankfull_depth, double x_length,
                         double y_length, double river_length, double river_width, double* out3) {
    if (total_storage >= bankfull_storage) {
        const double river_h = bankfull_depth + (total_storage - bankfull_storage) / (x_length * y_length);
        out3[0] = river_h;
        out3[1] = river_h - bankfull_depth;
        out3[2] = river_h * river_length * river_width;
    } else {
        out3[0] = total_storage / (river_length * river_width);
        out3[1] = 0.0;
        out3[2] = total_storage;
    }
}

// update_land_storage_and_depth! (:1481-1503)
void orc_li_update_land_cell(int64_t i, const double* qx, const double* qy, const int64_t* ind_x_down,
                             const int64_t* ind_y_down, const double* runoff, const double* x_length,
                             const double* y_length, double dt, double* storage, double* error, double* h) {
    storage[i] += orc_li_land_storage_change(i, qx, qy, ind_x_down, ind_y_down, runoff, dt);
    if (storage[i] < 0.0) {
        error[i] += std::fabs(storage[i]);
        storage[i] = 0.0;
    }
    h[i] = storage[i] / (x_length[i] * y_length[i]);
}

// update_river_and_land_storage_and_depth! (:1440-1476) at cell i holding river cell r
void orc_li_update_river_cell(int64_t i, const double* q_river, const int64_t* e_in, int64_t n_in,
                              const int64_t* e_out, int64_t n_out, const double* qx, const double* qy,
                              const int64_t* ind_x_down, const int64_t* ind_y_down, const double* runoff,
                              double abstraction, double external_inflow, double bankfull_storage,
                              double bankfull_depth, const double* x_length, const double* y_length,
                              double river_length, double river_width, double dt, double* storage, double* error,
                              double* h_land, double* h_river, double* storage_river,
                              double* abstraction_cumulative) {
    storage[i] += orc_li_river_storage_change(i, q_river, e_in, n_in, e_out, n_out, qx, qy, ind_x_down, ind_y_down,
                                              runoff, abstraction, dt);
    if (storage[i] < 0.0) {
        error[i] += std::fabs(storage[i]);
        storage[i] = 0.0;
    }
    double io[2];
    orc_li_external_inflow(external_inflow, storage[i], bankfull_storage, *storage_river, dt, io);
    storage[i] += io[0] * dt;
    *abstraction_cumulative += io[1] * dt;
    double d[3];
    orc_li_water_depths(storage[i], bankfull_storage, bankfull_depth, x_length[i], y_length[i], river_length,
                        river_width, d);
    *h_river = d[0];
    h_land[i] = d[1];
    *storage_river = d[2];
}

// stable_timestep of the local-inertial river (:1004-1020)
double orc_li_stable_timestep(int64_t n, const double* flow_length, const double* h, double alpha) {
    double dt_min = std::numeric_limits<double>::infinity();
    for (int64_t i = 0; i < n; ++i) dt_min = jmin(alpha * flow_length[i] / std::sqrt(GRAVITY * h[i]), dt_min);
    return std::isinf(dt_min) ? 60.0 : dt_min;
}

// The coupled scheme's sub-step in the reference's order (update_overland_flow_model!,
// :1170-1183): local_inertial_update_fluxes! (:1271-1290; x then y at each cell from the
// previous discharges), staggered_scheme_river_update! without the depth update (:763-797),
// local_inertial_update_water_depth! (:1518-1546). Edge parameters of the land grid as its
// constructor derives them (:929-939): zx_max / zy_max the higher elevation of a cell and its
// upstream neighbour; bankfull storage = depth * width * length (:118).
void orc_li_domain_substep(const WfLiLandGrid* L, const WfLiRiverNetwork* R, const double* runoff,
                           const double* external_inflow, const double* abstraction, double dt, OrcLiState* st) {
    const int64_t n = L->n;
    std::vector<double> zx_max(n, 0.0), zy_max(n, 0.0);
    for (int64_t i = 0; i < n; ++i) {
        if (L->ind_x_up[i] < n) zx_max[i] = jmax(L->elevation[i], L->elevation[L->ind_x_up[i]]);
        if (L->ind_y_up[i] < n) zy_max[i] = jmax(L->elevation[i], L->elevation[L->ind_y_up[i]]);
    }
    const double* nsq = L->mannings_n_sq;
    for (int64_t i = 0; i <= n; ++i) {
        st->qx0[i] = st->qx[i];
        st->qy0[i] = st->qy[i];
    }
    for (int64_t i = 0; i < n; ++i) {
        orc_li_directional_flow(i, n, L->ind_x_up, L->ind_x_down, L->ywidth_at_edge, zx_max.data(), L->x_length,
                                L->elevation, st->h_land, nsq, L->theta, L->h_thresh, L->froude_limit, dt,
                                st->qx, st->qx0, st->qx_cum);
        orc_li_directional_flow(i, n, L->ind_y_up, L->ind_y_down, L->xwidth_at_edge, zy_max.data(), L->y_length,
                                L->elevation, st->h_land, nsq, L->theta, L->h_thresh, L->froude_limit, dt,
                                st->qy, st->qy0, st->qy_cum);
    }
    li_river_edges(R->n_edges, R->src, R->dst, R->zb, R->zb_edge, R->width_edge, R->length_edge,
                   R->mannings_n_sq_edge, R->h_thresh, R->froude_limit, dt, st->h_river, st->q, st->q_prev, st->q_cum);
    std::vector<std::vector<int64_t>> e_in(R->n), e_out(R->n);  // ascending edge order (findall)
    for (int64_t k = 0; k < R->n_edges; ++k) {
        e_in[R->dst[k]].push_back(k);
        e_out[R->src[k]].push_back(k);
    }
    std::vector<double> zero(R->n, 0.0);
    const double* ext = external_inflow ? external_inflow : zero.data();
    const double* abs_ = abstraction ? abstraction : zero.data();
    for (int64_t i = 0; i < n; ++i) {
        const int64_t r = L->river_index[i];
        if (r >= 0) {
            const double bankfull_storage = R->bankfull_depth[r] * R->flow_width[r] * R->flow_length[r];
            orc_li_update_river_cell(i, st->q, e_in[r].data(), (int64_t)e_in[r].size(), e_out[r].data(),
                                     (int64_t)e_out[r].size(), st->qx, st->qy, L->ind_x_down, L->ind_y_down, runoff,
                                     abs_[r], ext[r], bankfull_storage, R->bankfull_depth[r], L->x_length,
                                     L->y_length, R->flow_length[r], R->flow_width[r], dt, st->storage, st->error,
                                     st->h_land, &st->h_river[r], &st->storage_river[r], &st->abstraction_cum[r]);
        } else {
            orc_li_update_land_cell(i, st->qx, st->qy, L->ind_x_down, L->ind_y_down, runoff, L->x_length, L->y_length,
                                    dt, st->storage, st->error, st->h_land);
        }
    }
}

double orc_li_domain_stable_timestep(const WfLiLandGrid* L, const WfLiRiverNetwork* R, const OrcLiState* st) {
    std::vector<int32_t> river_location(L->n);
    for (int64_t i = 0; i < L->n; ++i) river_location[i] = L->river_index[i] >= 0 ? 1 : 0;
    // the river's real cells: stable_timestep loops over parameters.n, the ghosts come after
    const double dt_river = orc_li_stable_timestep(R->n_active, R->flow_length, st->h_river, R->alpha);
    const double dt_land =
        orc_li_land_stable_timestep(L->n, L->x_length, L->y_length, river_location.data(), st->h_land, L->alpha);
    return jmin(dt_river, dt_land);
}

}  // extern "C"

extern "C" {
// Reservoir at a river node with discharge q after the node's kinematic-wave update.
void orc_reservoir_update(OrcReservoir* r, double q, double dt) { update_reservoir_at_node(r, 0, q, dt); }
// update_reservoir_model!(reservoir_model, i, inflow, dt) (reservoir.jl:583-628) on reservoir i
// (0-based) of `res`, which holds every reservoir a linked one refers to
void orc_reservoir_update_model(OrcReservoir* res, int64_t i, double inflow, double dt) {
    update_reservoir(res, i, inflow, dt);
}
double orc_interpolate_linear(double x, const double* xp, const double* fp, int64_t n) {
    return interpolate_linear(x, xp, fp, n);
}
int32_t orc_reservoir_size() { return (int32_t)sizeof(OrcReservoir); }
// col_index_hq of every reservoir (update_index_hq!, reservoir.jl:376-382)
int32_t orc_model_set_rating_curve_day(OrcModel* m, int32_t day) {
    if (day < 1 || day > 365) return WF_ERR_INVALID;
    for (OrcReservoir& r : m->res) r.hq_day = day;
    return WF_OK;
}
int64_t orc_model_reservoirs(const OrcModel* m) { return m->nres; }
}  // extern "C"

extern "C" {

int32_t orc_model_step(OrcModel* m, int32_t n_threads) {
    if (n_threads < 1) n_threads = 1;
    for (int mbr = 0; mbr < m->M; ++mbr) member_step(m, mbr, n_threads);
    return WF_OK;
}

// Sum of the squared sub-step sizes of the last model step per member (kind 0 subsurface,
// 1 land, 2 river): the same diagnostic as wf_get_substep_signature.
int32_t orc_model_substep_signature(OrcModel* m, int32_t kind, double* out) {
    if (kind < 0 || kind > 2 || (int)m->sig[kind].size() != m->M) return WF_ERR_INVALID;
    for (int k = 0; k < m->M; ++k) out[k] = m->sig[kind][k];
    return WF_OK;
}

int32_t orc_model_substeps(OrcModel* m, int64_t* land, int64_t* river, int64_t* subsurface) {
    *land = m->last_sub_land;
    *river = m->last_sub_river;
    *subsurface = m->last_sub_ssf;
    return WF_OK;
}

static double* land_field(OrcModel* m, int field, std::vector<double>** vec) {
    *vec = nullptr;
    switch (field) {
        case WF_F_CANOPY_STORAGE: *vec = &m->canopy_storage; break;
        case WF_F_SNOW_STORAGE: *vec = &m->snow_storage; break;
        case WF_F_SNOW_WATER: *vec = &m->snow_water; break;
        case WF_F_SSF_Q: *vec = &m->ssf_q; break;
        case WF_F_LAND_Q: *vec = &m->ol_q; break;
        case WF_F_LAND_H: *vec = &m->ol_h; break;
        case WF_F_INTERCEPTION_RATE: *vec = &m->interception_rate; break;
        case WF_F_SNOW_WATER_EQUIVALENT: *vec = &m->swe; break;
        case WF_F_NET_RUNOFF_RIVER: *vec = &m->net_runoff_river; break;
        case WF_F_SSF_Q_AVERAGE: *vec = &m->ssf_q_avg; break;
        case WF_F_SSF_WATER_TABLE_DEPTH: *vec = &m->ssf_zi; break;
        case WF_F_SSF_STORAGE: *vec = &m->ssf_storage; break;
        case WF_F_SSF_TO_RIVER_AVERAGE: *vec = &m->ssf_tr_avg; break;
        case WF_F_LAND_Q_AVERAGE: *vec = &m->ol_q_avg; break;
        case WF_F_LAND_QIN_AVERAGE: *vec = &m->ol_qin_avg; break;
        case WF_F_LAND_STORAGE: *vec = &m->ol_storage; break;
        case WF_F_LAND_TO_RIVER_AVERAGE: *vec = &m->ol_tr_avg; break;
        case WF_F_LAND_INWATER: *vec = &m->ol_inwater; break;
        case WF_F_TOTAL_STORAGE: *vec = &m->total_storage; break;
        case WF_F_BALANCE_LAND_ERROR: *vec = &m->bl_err; break;
        case WF_F_BALANCE_LAND_RELATIVE_ERROR: *vec = &m->bl_rel; break;
        case WF_F_BALANCE_OVERLAND_ERROR: *vec = &m->bo_err; break;
        case WF_F_BALANCE_OVERLAND_RELATIVE_ERROR: *vec = &m->bo_rel; break;
        case WF_F_BALANCE_SUBSURFACE_ERROR: *vec = &m->bs_err; break;
        case WF_F_BALANCE_SUBSURFACE_RELATIVE_ERROR: *vec = &m->bs_rel; break;
        case WF_F_GLACIER_STORE: *vec = &m->glacier_store; break;
        case WF_F_GLACIER_MELT: *vec = &m->glacier_melt; break;
        case WF_F_SNOW_IN: *vec = &m->snow_in; break;
        case WF_F_SNOW_OUT: *vec = &m->snow_out; break;
        default: break;
    }
    return *vec ? (*vec)->data() : nullptr;
}

static double* soil_member(OrcSoil& s, int field, int layer) {
    switch (field) {
        case WF_F_SOIL_SURFACE_TEMPERATURE: return &s.soil_surface_temperature;
        case WF_F_SATURATED_WATER_DEPTH: return &s.saturated_water_depth;
        case WF_F_UNSATURATED_LAYER_DEPTH: return &s.unsaturated_layer_depth[layer];
        case WF_F_WATER_TABLE_DEPTH: return &s.water_table_depth;
        case WF_F_UNSATURATED_STORE_DEPTH: return &s.unsaturated_store_depth;
        case WF_F_TOTAL_SOIL_WATER_STORAGE: return &s.total_soil_water_storage;
        case WF_F_RECHARGE: return &s.recharge;
        case WF_F_NET_RUNOFF: return &s.net_runoff;
        case WF_F_RUNOFF: return &s.runoff;
        case WF_F_ACTUAL_EVAPOTRANSPIRATION: return &s.actual_evapotranspiration;
        case WF_F_ACTUAL_LEAKAGE: return &s.actual_leakage;
        case WF_F_TRANSPIRATION: return &s.transpiration;
        case WF_F_SOIL_EVAPORATION: return &s.soil_evaporation;
        case WF_F_ACTUAL_INFILTRATION: return &s.actual_infiltration;
        case WF_F_EXFILTRATION_SATURATED_WATER: return &s.exfiltration_saturated_water;
        case WF_F_VOLUMETRIC_WATER_CONTENT: return &s.volumetric_water_content[layer];
        default: return nullptr;
    }
}

static double* river_field(OrcModel* m, int field) {
    switch (field) {
        case WF_F_RIVER_Q: return m->rv_q.data();
        case WF_F_RIVER_H: return m->rv_h.data();
        case WF_F_RIVER_STORAGE: return m->rv_storage.data();
        case WF_F_RIVER_Q_AVERAGE: return m->rv_q_avg.data();
        case WF_F_RIVER_QIN_AVERAGE: return m->rv_qin_avg.data();
        case WF_F_RIVER_INWATER: return m->rv_inwater.data();
        case WF_F_BALANCE_RIVER_ERROR: return m->br_err.data();
        case WF_F_BALANCE_RIVER_RELATIVE_ERROR: return m->br_rel.data();
        default: return nullptr;
    }
}

// Reservoir fields, member-major [mbr * nres + k]: a pointer into the reservoir record or into
// one of the per-step diagnostic arrays.
static double* reservoir_field(OrcModel* m, int field, int64_t q) {
    OrcReservoir& r = m->res[q];
    switch (field) {
        case WF_F_RESERVOIR_STORAGE: return &r.storage;
        case WF_F_RESERVOIR_WATERLEVEL: return &r.waterlevel;
        case WF_F_RESERVOIR_OUTFLOW: return &r.outflow;
        case WF_F_RESERVOIR_OUTFLOW_AVERAGE: return &m->res_out_avg[q];
        case WF_F_RESERVOIR_INFLOW_AVERAGE: return &m->res_in_avg[q];
        case WF_F_RESERVOIR_ACTEVAP_AVERAGE: return &m->res_evap_avg[q];
        case WF_F_RESERVOIR_ABSTRACTION_AVERAGE: return &m->res_abs_avg[q];
        case WF_F_RESERVOIR_INFLOW_OVERLAND: return &r.inflow_overland;
        case WF_F_RESERVOIR_INFLOW_SUBSURFACE: return &r.inflow_subsurface;
        case WF_F_RESERVOIR_PRECIPITATION: return &r.precipitation;
        case WF_F_RESERVOIR_EVAPORATION: return &r.evaporation;
        case WF_F_RESERVOIR_EXTERNAL_INFLOW: return &r.external_inflow;
        case WF_F_RESERVOIR_OUTFLOW_OBS: return &r.outflow_obs;
        case WF_F_BALANCE_RESERVOIR_ERROR: return &m->res_err[q];
        case WF_F_BALANCE_RESERVOIR_RELATIVE_ERROR: return &m->res_rel[q];
        default: return nullptr;
    }
}

int32_t orc_model_get(OrcModel* m, int32_t field, int32_t layer, double* out) {
    int64_t nm = m->n * m->M;
    if (field >= WF_F_RESERVOIR_STORAGE) {
        if (field >= WF_F_RESERVOIR_END_) return WF_ERR_INVALID;
        for (int64_t q = 0; q < m->nres * m->M; ++q) out[q] = *reservoir_field(m, field, q);
        return WF_OK;
    }
    if (field >= WF_F_RIVER_Q) {
        double* src = river_field(m, field);
        if (!src) return WF_ERR_INVALID;
        std::memcpy(out, src, m->nr * m->M * 8);
        return WF_OK;
    }
    std::vector<double>* vec;
    double* src = land_field(m, field, &vec);
    if (src) {
        std::memcpy(out, src, nm * 8);
        return WF_OK;
    }
    if (layer < 0 || layer >= m->N) layer = 0;
    for (int64_t j = 0; j < nm; ++j) {
        double* p = soil_member(m->soil[j], field, layer);
        if (!p) return WF_ERR_INVALID;
        out[j] = *p;
    }
    return WF_OK;
}

int32_t orc_model_set(OrcModel* m, int32_t field, int32_t layer, const double* in) {
    int64_t nm = m->n * m->M;
    if (field >= WF_F_RESERVOIR_STORAGE) {
        if (field >= WF_F_RESERVOIR_END_) return WF_ERR_INVALID;
        for (int64_t q = 0; q < m->nres * m->M; ++q) *reservoir_field(m, field, q) = in[q];
        return WF_OK;
    }
    if (field >= WF_F_RIVER_Q) {
        double* dst = river_field(m, field);
        if (!dst) return WF_ERR_INVALID;
        std::memcpy(dst, in, m->nr * m->M * 8);
        return WF_OK;
    }
    std::vector<double>* vec;
    double* dst = land_field(m, field, &vec);
    if (dst) {
        std::memcpy(dst, in, nm * 8);
        return WF_OK;
    }
    if (layer < 0 || layer >= m->N) layer = 0;
    for (int64_t j = 0; j < nm; ++j) {
        double* p = soil_member(m->soil[j], field, layer);
        if (!p) return WF_ERR_INVALID;
        *p = in[j];
    }
    return WF_OK;
}

int32_t orc_model_outlets(OrcModel* m, int32_t which, double* out, int64_t* n) {
    int64_t k = 0;
    for (int mbr = 0; mbr < m->M; ++mbr)
        for (int32_t r : m->r_pits) out[k++] = which == 0 ? m->rv_q_avg[mbr * m->nr + r] : m->rv_q[mbr * m->nr + r];
    *n = k;
    return WF_OK;
}

// ----------------------------------------------------------------- KAT wrappers ------
double orc_exp(double x) { return wexp(x); }
double orc_log(double x) { return wlog(x); }
double orc_cbrt(double x) { return wcbrt(x); }
double orc_pow(double x, double y) { return jpow(x, y); }
double orc_cld(double x, double y) { return jcld(x, y); }
double orc_round_sigdigits(double x, int32_t d) { return jround_sigdigits(x, d); }

void orc_rainfall_interception_gash(double cmax, double e_r, double gap, double p, double cs, double max_evap,
                                    double dt, double* out4) {
    rainfall_interception_gash(cmax, e_r, gap, p, cs, max_evap, dt, out4);
}
void orc_rainfall_interception_modrut(double p, double pet, double cs, double gap, double cmax, double dt,
                                      double* out4) {
    rainfall_interception_modrut(p, pet, cs, gap, cmax, dt, out4);
}
void orc_precipitation_hbv(double p, double t, double tti, double tt, double* out2) {
    precipitation_hbv(p, t, tti, tt, out2);
}
void orc_snowpack_hbv(double ss, double sw, double sp, double lp, double t, double ttm, double cfmax, double whc,
                      double dt, double* out5) {
    snowpack_hbv(ss, sw, sp, lp, t, ttm, cfmax, whc, dt, out5);
}
void orc_glacier_hbv(double gfrac, double gstore, double ss, double t, double g_ttm, double g_cfmax,
                     double g_sifrac, double max_snow_to_glacier, double dt, double* out4) {
    glacier_hbv(gfrac, gstore, ss, t, g_ttm, g_cfmax, g_sifrac, max_snow_to_glacier, dt, out4);
}
void orc_infiltration(double pot, double cfrac, double cap_soil, double cap_comp, double ucap, double fred,
                      double dt, double* out2) {
    infiltration_fn(pot, cfrac, cap_soil, cap_comp, ucap, fred, dt, out2);
}
void orc_unsatzone_flow_layer(double usd, double kv_z, double l_sat, double c, double dt, double* out2) {
    unsatzone_flow_layer(usd, kv_z, l_sat, c, dt, out2);
}
double orc_head_brooks_corey(double vwc, double ts, double tr, double c, double psi) {
    return head_brooks_corey(vwc, ts, tr, c, psi);
}
double orc_vwc_brooks_corey(double h, double psi, double ts, double tr, double c) {
    return vwc_brooks_corey(h, psi, ts, tr, c);
}
double orc_feddes_h3(double h3h, double h3l, double tpot) { return feddes_h3(h3h, h3l, tpot); }
double orc_rwu_reduction_feddes(double h, double h1, double h2, double h3, double h4, double a) {
    return rwu_reduction_feddes(h, h1, h2, h3, h4, a);
}
double orc_soil_temperature(double tsoil_prev, double w_soil, double t) { return soil_temperature(tsoil_prev, w_soil, t); }
double orc_infiltration_reduction_factor(double tsoil, double cf, int32_t modelsnow, int32_t flag) {
    return infiltration_reduction_factor(tsoil, cf, modelsnow != 0, flag != 0);
}
double orc_soil_evaporation_unsaturated_store(double pot, double usld, double ulthick, int32_t nunsat, double zi,
                                              double theta_e) {
    return soil_evaporation_unsaturated_store(pot, usld, ulthick, nunsat, zi, theta_e);
}
double orc_soil_evaporation_saturated_store(double pot, int32_t nunsat, double lthick, double zi, double theta_d,
                                            double dt) {
    return soil_evaporation_saturated_store(pot, nunsat, lthick, zi, theta_d, dt);
}
void orc_actual_infiltration_soil_path(double pot, double act, double cfrac, double cap_soil, double cap_comp,
                                       double fred, double* out2) {
    actual_infiltration_soil_path(pot, act, cfrac, cap_soil, cap_comp, fred, out2);
}
double orc_scurve(double x, double a, double b, double c) { return scurve(x, a, b, c); }
void orc_compute_mass_balance_error(double tin, double tout, double rate, double* out2) {
    compute_mass_balance_error(tin, tout, rate, out2);
}
void orc_kinematic_wave(double qin, double qprev, double qlat, double alpha, double dt, double dx, double* out2) {
    kinematic_wave(qin, qprev, qlat, alpha, dt, dx, out2);
}
double orc_ssf_celerity(double zi, double slope, double sy, double kh0, double f, int32_t profile, double z_exp) {
    return ssf_celerity(zi, slope, sy, kh0, f, profile, z_exp);
}
double orc_kw_ssf_newton_raphson(double q, double c, double cel, double dt, double dx) {
    return kw_ssf_newton_raphson(q, c, cel, dt, dx);
}
void orc_update_bc_soil_model(OrcSoil* s, double canopy_potevap, double interception_rate, double pet,
                              double wfs_runoff, double runoff_river, double runoff_land) {
    update_bc_soil_model(*s, canopy_potevap, interception_rate, pet, wfs_runoff, runoff_river, runoff_land);
}
void orc_unsaturated_zone_flow(OrcSoil* s, double dt) { unsaturated_zone_flow(*s, dt); }
void orc_soil_evaporation(OrcSoil* s, double dt) { soil_evaporation(*s, dt); }
void orc_transpiration(OrcSoil* s, double dt) { transpiration(*s, dt); }
void orc_capillary_flux(OrcSoil* s, double dt) { capillary_flux(*s, dt); }
void orc_update_soil_water_storage(OrcSoil* s, double exfilt_avg, double runoff_land, double ae_land, double dt) {
    update_soil_water_storage(*s, exfilt_avg, runoff_land, ae_land, dt);
}
void orc_water_table_change(const OrcSoil* s, double net_flux, double sy, double dt, double* out2) {
    water_table_change(*s, net_flux, sy, dt, out2);
}
void orc_kinematic_wave_ssf(double q_in, double q_prev, double zi_prev, double q_net, double slope, double sy,
                            double d, double dt, double dx, double dw, double q_max, double kh0, double f,
                            int32_t profile, double z_exp, OrcSoil* s, double* out4) {
    kinematic_wave_ssf(q_in, q_prev, zi_prev, q_net, slope, sy, d, dt, dx, dw, q_max, kh0, f, profile, z_exp, *s,
                       out4);
}
double orc_kinwave_stable_timestep(const double* q, const double* alpha, const double* flow_length, int64_t n,
                                   double p) {
    std::vector<double> buf;
    return kinwave_stable_timestep(q, alpha, flow_length, n, p, buf);
}
double orc_quantile(double* v, int64_t n, double p) {
    std::sort(v, v + n);
    return quantile_sorted(v, n, p);
}

int32_t orc_soil_sizeof(void) { return (int32_t)sizeof(OrcSoil); }

#define ORC_I(f) #f ":" + std::to_string(offsetof(OrcSoil, f)) + ":i;"
#define ORC_D(f) #f ":" + std::to_string(offsetof(OrcSoil, f)) + ":d;"
#define ORC_A(f, n) #f ":" + std::to_string(offsetof(OrcSoil, f)) + ":a" #n ";"

const char* orc_soil_layout(void) {
    static std::string s;
    if (!s.empty()) return s.c_str();
    s = std::string() + ORC_I(maximum_number_of_layers) + ORC_I(number_of_layers) + ORC_I(n_unsatlayers) +
        ORC_I(kv_profile) + ORC_D(theta_s) + ORC_D(theta_r) + ORC_D(theta_fc) + ORC_D(soil_water_capacity) +
        ORC_D(kv_0) + ORC_D(f) + ORC_D(z_exp) + ORC_D(air_entry_pressure) + ORC_D(h1) + ORC_D(h2) + ORC_D(h3_high) +
        ORC_D(h3_low) + ORC_D(h4) + ORC_D(alpha_h1) + ORC_D(soil_thickness) + ORC_D(infiltration_capacity_soil) +
        ORC_D(infiltration_capacity_compacted_soil) + ORC_D(compacted_soil_area_fraction) +
        ORC_D(wet_root_distribution_parameter) + ORC_D(cap_hmax) + ORC_D(cap_n) + ORC_D(maximum_leakage) +
        ORC_D(w_soil) + ORC_D(cf_soil) + ORC_D(rooting_depth) + ORC_D(soil_fraction) +
        ORC_A(actual_layer_thickness, 8) + ORC_A(cumulative_layer_depth, 9) + ORC_A(brooks_corey_exponent, 8) +
        ORC_A(kv_factor, 8) + ORC_A(rootfraction, 8) + ORC_D(water_flux_surface) + ORC_D(potential_transpiration) +
        ORC_D(potential_soilevaporation) + ORC_A(unsaturated_layer_depth, 8) + ORC_A(unsaturated_layer_thickness, 8) +
        ORC_A(volumetric_water_content, 8) + ORC_A(relative_volumetric_water_content, 8) + ORC_D(h3) +
        ORC_D(unsaturated_store_capacity) + ORC_D(saturated_water_depth) + ORC_D(drainable_water_depth) +
        ORC_D(water_table_depth) + ORC_D(transpiration) + ORC_D(actual_evaporation_unsaturated_store) +
        ORC_D(soil_evaporation) + ORC_D(soil_evaporation_saturated_zone) + ORC_D(actual_capillary_flux) +
        ORC_D(actual_evaporation_saturated_zone) + ORC_D(actual_evapotranspiration) + ORC_D(actual_infiltration) +
        ORC_D(actual_infiltration_soil) + ORC_D(actual_infiltration_compacted_soil) + ORC_D(infiltration) +
        ORC_D(infiltration_excess) + ORC_D(saturation_excess_water) + ORC_D(exfiltration_saturated_water) +
        ORC_D(excess_water_soil) + ORC_D(excess_water_compacted_soil) + ORC_D(runoff) + ORC_D(net_runoff) +
        ORC_D(root_zone_storage) + ORC_D(volumetric_water_content_root_zone) +
        ORC_D(relative_volumetric_water_content_root_zone) + ORC_D(unsaturated_store_depth) + ORC_D(transfer) +
        ORC_D(recharge) + ORC_D(actual_leakage) + ORC_D(total_soil_water_storage) +
        ORC_D(soil_surface_temperature) + ORC_D(f_infiltration_reduction);
    return s.c_str();
}

}  // extern "C"
