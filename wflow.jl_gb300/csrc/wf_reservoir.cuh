// wf_reservoir.cuh -- reservoir update at a river node, inside the river wavefront.
//
// A reservoir sits at a river cell (its outlet). The river sweep computes the cell's discharge
// with the kinematic wave as usual; the reservoir then takes that discharge plus the outlet
// cell's overland and subsurface discharge and the external inflow as its net inflow, updates
// its storage and water level, and its outflow (not the cell's river discharge) is what the
// downstream river cell receives (Wflow/src/routing/surface/surface_kinwave.jl:441-489).
// Reservoirs are few (hundreds in a large model) and their arithmetic is FP64 in both forms.
//
// Outflow functions (routing/surface/reservoir.jl): 1 rating curve from the H-Q table of the day
// (:455-479), 2 free weir, optionally linked to a lower reservoir (:482-521), 3 modified Puls
// (:424-452), 4 simple (:389-418), each replaced by the observed outflow where one is given
// (:524-545); storage profiles S = A H and S = f(H) interpolated in an S-H table (:306-320,
// :612-621).
//
// A free weir linked to a lower reservoir reads the lower reservoir's level and, when that is
// the higher one, takes water back from it within the sub-step: it writes the lower reservoir's
// storage, level, outflow and cumulative outflow. The planner keeps the river path from the
// upper to the lower reservoir on one chain, so the lane that updates the upper reservoir is the
// lane that reaches the lower one later in the same sweep (program order, no other thread reads
// those words), and the river then runs one sub-step per launch, so the upper reservoir's next
// sub-step sees the lower one's state after the lower one's own update.
#pragma once

#include "wf_fields.cuh"
#include "wf_math.cuh"

namespace wfr {

// Wflow.scurve (utils.jl:27-30)
__device__ __forceinline__ double scurve(double x, double a, double b, double c) {
    return 1.0 / (b + wfm::exp(-c * (x - a)));
}

// Tables of reservoir r: meta[4 r .. 4 r + 3] = start of the S-H table in F.res_tab (levels, then
// storages), its rows, start of the H-Q table (levels, then rows x 365 discharges), its rows.
// reservoir.jl:363-375 on n rows at xp[i] and fp[i * fs] (fs: the stride of a table column);
// the levels and storages of a table are strictly increasing (checked at create).
__device__ inline double interpolate_linear(double x, const double* xp, const double* fp, int64_t fs, int64_t n) {
    double fmin = fp[0], fmax = fp[0];
    for (int64_t i = 1; i < n; ++i) {
        fmin = wfm::jmin(fmin, fp[i * fs]);
        fmax = wfm::jmax(fmax, fp[i * fs]);
    }
    if (x <= xp[0]) return fmin;
    if (x >= xp[n - 1]) return fmax;
    int64_t i1 = 0;
    while (i1 + 1 < n && xp[i1 + 1] <= x) ++i1;
    const int64_t i2 = i1 + 1;
    const double f1 = fp[i1 * fs], f2 = fp[i2 * fs];
    return f1 * (1.0 - (x - xp[i1]) / (xp[i2] - xp[i1])) + f2 * (x - xp[i1]) / (xp[i2] - xp[i1]);
}

// Water level of reservoir r at `storage` after a change from (s0, wl0) (reservoir.jl:612-621).
__device__ __forceinline__ double level_after(const WfDevFields& F, int32_t r, double storage, double s0, double wl0,
                                              double area) {
    if (F.res_profile && F.res_profile[r] == 2) {
        const int64_t* mt = F.res_tab_meta + 4 * (int64_t)r;
        const double* h = F.res_tab + mt[0];
        return interpolate_linear(storage, h + mt[1], h, 1, mt[1]);
    }
    return wl0 + (storage - s0) / area;
}

// Net inflow, storage update and outflow of reservoir r for member m over a sub-step dt, with q
// the river discharge of the reservoir's cell after its kinematic-wave update. Accumulates the
// step's inflow, outflow, evaporation and abstraction; returns the outflow.
__device__ inline double reservoir_node(const WfDevFields& F, int32_t r, int m, double q, double dt) {
    using wfm::jmax;
    using wfm::jmin;
    const int64_t e = (int64_t)r * F.M + m;
    double* const* RS = F.RS;
    double* const* RP = F.RP;
    const double area = RP[RP_AREA][r];
    const double s0 = RS[RS_STORAGE][e];
    const double wl0 = RS[RS_WATERLEVEL][e];
    // negative external inflow: abstraction limited to 98 % of the storage (surface_kinwave.jl:461-469)
    const double ext = RS[RS_EXT][e];
    double inflow;
    if (ext < 0.0) {
        const double abstraction = jmin(-ext, (s0 / dt) * 0.98);
        RS[RS_ABS_CUM][e] += abstraction * dt;
        inflow = -abstraction;
    } else {
        inflow = ext;
    }
    const double net = q + RS[RS_IN_OL][e] + RS[RS_IN_SSF][e] + inflow;
    // evaporation limited by the available volume (reservoir.jl:595-599)
    const double precipitation = RS[RS_PRECIP][e] * area;
    const double available = s0 + (net + precipitation) * dt;
    const double potential_evaporation = RS[RS_EVAP][e] * area;
    const double evaporation = jmin(available / dt, potential_evaporation);
    const double obs = RS[RS_OBS][e];
    const double smax = RP[RP_MAXSTOR][r];
    double outflow, storage;
    if (obs == obs) {  // observed outflow (reservoir.jl:554-575)
        const double input = jmax(s0 / dt + precipitation - evaporation + net, 0.0);
        outflow = jmin(obs, input);
        storage = (input - outflow) * dt;
        if (smax == smax) {
            const double overflow = jmax(0.0, (storage - smax) / dt);
            storage -= overflow * dt;
            outflow += overflow;
        }
    } else if (F.res_type[r] == WF_RES_RATING_CURVE) {
        const double input = s0 / dt + precipitation - evaporation + net;
        const int64_t* mt = F.res_tab_meta + 4 * (int64_t)r;
        const double* h = F.res_tab + mt[2];
        outflow = interpolate_linear(wl0, h, h + mt[3] + (*F.res_hq_day - 1), 365, mt[3]);
        outflow = jmin(outflow, input);
        storage = (input - outflow) * dt;
        const double overflow = jmax(0.0, (storage - smax) / dt);
        storage = jmin(storage, smax);
        outflow += overflow;
    } else if (F.res_type[r] == WF_RES_FREE_WEIR) {
        const int32_t lo = F.res_lower ? F.res_lower[r] : -1;
        const int64_t elo = (int64_t)lo * F.M + m;
        const double wl_lo = lo >= 0 ? RS[RS_WATERLEVEL][elo] : 0.0;
        const double diff_wl = lo >= 0 ? wl0 - wl_lo : 0.0;
        const double input = jmax(s0 / dt + precipitation - evaporation + net, 0.0);
        const double thr = RP[RP_THRESHOLD][r];
        outflow = 0.0;
        if (diff_wl >= 0.0) {
            if (wl0 > thr) {
                const double dh = wl0 - thr;
                outflow = RP[RP_RC_COEF][r] * wfm::pow(dh, RP[RP_RC_EXP][r]);
                outflow = jmin(outflow, dh * area / dt);
            }
        } else if (wl_lo > thr) {  // the lower reservoir's level is the higher: flow back
            const double dh = wl_lo - thr;
            outflow = -RP[RP_RC_COEF][r] * wfm::pow(dh, RP[RP_RC_EXP][r]);
            outflow = jmax(outflow, -(dh * RP[RP_AREA][lo] / dt));
        }
        storage = (input - outflow) * dt;
        if (diff_wl < 0.0) {
            const double s_lo = RS[RS_STORAGE][elo];
            const double s_lo_new = s_lo + outflow * dt;
            RS[RS_WATERLEVEL][elo] = level_after(F, lo, s_lo_new, s_lo, wl_lo, RP[RP_AREA][lo]);
            RS[RS_OUTFLOW][elo] = -outflow;
            RS[RS_OUT_CUM][elo] -= outflow * dt;
            RS[RS_STORAGE][elo] = s_lo_new;
        }
    } else if (F.res_type[r] == WF_RES_MODIFIED_PULS) {
        const double res_factor = area / (dt * wfm::sqrt_(RP[RP_RC_COEF][r]));
        const double si = s0 / dt + precipitation - evaporation + net;
        const double si_adj = si - area * RP[RP_THRESHOLD][r] / dt;
        outflow = 0.0;
        if (si_adj > 0.0) {
            const double t = -res_factor + wfm::sqrt_((res_factor * res_factor + 4.0 * si_adj));
            outflow = t > 0.0 ? 0.25 * t * t : 0.0;
        }
        outflow = jmin(outflow, si);
        storage = (si - outflow) * dt;
    } else {  // simple reservoir
        storage = jmax(s0 + (net + precipitation - evaporation) * dt, 0.0);
        const double fac = scurve(storage / smax, RP[RP_TMIN][r], 1.0, 30.0);
        const double demand_release = jmin(fac * RP[RP_DEMAND][r], storage / dt);
        storage -= demand_release * dt;
        const double wanted = jmax(0.0, (storage - smax * RP[RP_TFULL][r]) / dt);
        const double overflow_q = jmax(0.0, (storage - smax) / dt);
        const double realized = jmin(wanted, overflow_q + RP[RP_MAXREL][r] - demand_release);
        storage -= realized * dt;
        outflow = realized + demand_release;
    }
    RS[RS_WATERLEVEL][e] = level_after(F, r, storage, s0, wl0, area);
    RS[RS_STORAGE][e] = storage;
    RS[RS_OUTFLOW][e] = outflow;
    RS[RS_IN_CUM][e] += net * dt;
    RS[RS_OUT_CUM][e] += outflow * dt;
    // what went to the downstream river cell: the reservoir's own outflows only (RS_OUT_CUM of a
    // linked lower reservoir also counts the water its upper reservoir drew back)
    RS[RS_DOWN_CUM][e] += outflow * dt;
    RS[RS_EVAP_CUM][e] += evaporation / area * dt;
    return outflow;
}

}  // namespace wfr
