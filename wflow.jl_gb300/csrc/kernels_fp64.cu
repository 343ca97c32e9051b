// kernels_fp64.cu -- FP64 plain form of Wflow's SBM + kinematic-wave step (the drop-in).
//
// Compiled with --fmad=false: every multiply and add rounds separately, as in the reference's
// scalar Julia Float64 code. All elementary functions come from wf_math.cuh.
//
// Kernels of one model step (update_model!, Wflow/src/sbm_model.jl:60-92):
//   vertical  : storage_prev! of the land balance, interception, snow, open-water runoff,
//               soil fraction, soil boundary conditions, update_soil_water_flow!  (per cell)
//   ssf       : lateral subsurface kinematic wave (wavefront), fused with
//               update_soil_water_storage! and the overland lateral inflow      (per chain)
//   overland  : overland kinematic wave with fixed sub-steps (wavefront)
//   river     : river lateral inflow + river kinematic wave (wavefront)
//   balance   : update_total_water_storage! and compute_mass_balance!           (per cell)
#include <cuda_runtime.h>

#include "wf_fields.cuh"
#include "wf_li_couple.cuh"
#include "wf_kernels.h"
#include "wf_launch.cuh"
#include "wf_math.cuh"
#include "wf_reservoir.cuh"
#include "snow_scheme.cuh"
#include "wf_ff.cuh"
#include "wf_walker.cuh"

using wfm::jclamp;
using wfm::jmax;
using wfm::jmin;

namespace {

constexpr double KIN_WAVE_MIN_FLOW = 1e-30;                       // routing/utils.jl:1
constexpr double KIN_WAVE_MIN_FLOW_QROOT = 0x1.0c6f7a0b5ed8ap-20;  // 1e-30^0.2 (routing/utils.jl:2)
constexpr double BETA = 0.6;                                      // surface_kinwave.jl:2
constexpr double MM_PER_DAY = (1.0 / 86400.0) * 1e-3;             // units.jl MM_PER_DAY factor
constexpr double PERCENT = 1e-2;                                  // units.jl PERCENTAGE factor
constexpr double NANV = __builtin_nan("");

// ------------------------------------------------------------------ process functions ----

// vegetation/rainfall_interception.jl:9-70
__device__ void interception_gash(double cmax, double e_r, double gap, double P, double max_evap, double dt,
                                  double& tf, double& ic, double& sf) {
    if (cmax > 0.0) {
        double fs, fi, psat;
        if (gap < 1.0 / 1.1) {
            fs = 0.1 * gap;
            fi = 1.0 - 1.1 * gap;
            psat = e_r > fi ? 0.0 : -cmax / (e_r * dt) * wfm::log(1.0 - e_r / fi);
        } else {
            fs = 1.0 - gap;
            fi = 0.0;
            psat = 0.0;
        }
        if (P > psat) {
            ic = (fi * psat - cmax / dt) + e_r * (P - psat) + cmax / dt;
        } else {
            ic = fi * P;
        }
        sf = fs * P;
        tf = P - ic - sf;
        if (ic > max_evap) {
            const double drain = ic - max_evap;
            ic = max_evap;
            tf += drain;
        }
    } else {
        tf = P;
        ic = 0.0;
        sf = 0.0;
    }
}

// vegetation/rainfall_interception.jl:78-130
__device__ void interception_modrut(double P, double pet, double& cs, double gap, double cmax, double dt,
                                    double& tf, double& ce, double& sf) {
    double fs, pc;
    if (gap < 1.0 / 1.1) {
        fs = 0.1 * gap;
        pc = (1.0 - gap - fs) * P;
    } else {
        fs = 1.0 - gap;
        pc = 0.0;
    }
    sf = fs * P;
    tf = gap * P;
    if (cs > cmax) {
        const double d = cs - cmax;
        cs = cmax;
        tf += d / dt;
    }
    cs += pc * dt;
    const double max_evap = cs / dt;
    if (pet > max_evap) {
        ce = max_evap;
        cs = 0.0;
    } else {
        ce = pet;
        cs -= ce * dt;
    }
    if (cs > cmax) {
        const double d = cs - cmax;
        cs = cmax;
        tf += d / dt;
    }
}

// utils.jl:27-30
__device__ __forceinline__ double scurve(double x, double a, double b, double c) {
    return 1.0 / (b + wfm::exp(-c * (x - a)));
}

// utils.jl:1070-1076 with Wflow's pow
__device__ __forceinline__ double bounded_power(double base, double p) { return base > 1.0 ? 1.0 : wfm::pow(base, p); }

// soil/soil_process.jl:51-92
__device__ void unsatzone_flow_layer(double usd, double kv_z, double l_sat, double c, double dt, double& usd_out,
                                     double& flow) {
    if (usd <= 0.0) {
        usd_out = 0.0;
        flow = 0.0;
        return;
    }
    const double st_sat = jmax(0.0, usd - l_sat);
    double st = kv_z * bounded_power(usd / l_sat, c);
    double sum_ast = jmin(st, st_sat / dt);
    usd -= sum_ast * dt;
    const double remainder = jmin((st - sum_ast) * dt, usd);
    const long its = (long)wfm::cld(remainder, 2e-4);
    for (long i = 0; i < its; ++i) {
        st = (kv_z / (double)its) * bounded_power(usd / l_sat, c);
        const double st_max = usd / dt;
        if (st < st_max) {
            usd -= st * dt;
            sum_ast += st;
        } else {
            usd = 0.0;
            sum_ast += st_max;
            break;
        }
    }
    usd_out = usd;
    flow = sum_ast;
}

// soil/soil_process.jl:113-130
__device__ __forceinline__ double head_brooks_corey(double vwc, double ts, double tr, double c, double psi) {
    const double lam = 2.0 / (c - 3.0);
    return lam > 0.0 ? psi / wfm::pow(vwc / (ts - tr), 1.0 / lam) : psi;
}

// soil/soil_process.jl:166-176
__device__ __forceinline__ double feddes_h3(double h3h, double h3l, double tpot) {
    const double td = tpot / MM_PER_DAY;
    if (td <= 1.0) return h3l;
    if (td < 5.0) return h3l + (h3h - h3l) * (td - 1.0) / (5.0 - 1.0);
    return h3h;
}

// soil/soil_process.jl:183-200
__device__ __forceinline__ double rwu_feddes(double h, double h1, double h2, double h3, double h4, double a1) {
    if (h < h4) return 0.0;
    if (h < h3) return (h - h4) / (h3 - h4);
    if (a1 == 0.0) {
        if (h < h2) return 1.0;
        if (h < h1) return (h1 - h) / (h1 - h2);
        return 0.0;
    }
    return 1.0;
}

__device__ __forceinline__ double lb_drainable(double ts, double tfc) { return jmax(ts - tfc, 0.02); }

// kinematic wave for surface flow (routing/surface/surface_process.jl:24-70)
__device__ void kinematic_wave(double q_in, double q_prev, double q_lat, double alpha, double dt, double dx,
                               double& q, double& area) {
    if (q_in + q_prev + q_lat == 0.0) {
        q = 0.0;
        area = 0.0;
        return;
    }
    const double dt_dx = dt / dx;
    const double u_prev = q_prev >= 0.0 ? wfm::pow(q_prev, 0.2) : 0.0;
    const double cterm = dt_dx * q_in + alpha * u_prev * u_prev * u_prev + dt * q_lat;
    double u = u_prev > 0.0 ? u_prev : wfm::cbrt(cterm / alpha);
    const double c1 = 5.0 * dt_dx, c2 = 3.0 * alpha;
    for (int it = 0; it < 3000; ++it) {
        const double u2 = u * u;
        const double u3 = u2 * u;
        const double fu = u3 * (dt_dx * u2 + alpha) - cterm;
        if (wfm::fabs_(fu) <= 1.0e-12) break;
        const double df = u2 * (c1 * u2 + c2);
        const double u_old = u;
        u -= fu / df;
        if (wfm::isnan_(u) || u <= 0.0) u = KIN_WAVE_MIN_FLOW_QROOT;
        // an iterate that no longer changes repeats itself until max_iters: stop here with the
        // identical result (e.g. no positive root when the lateral inflow is negative)
        if (u == u_old) break;
    }
    u = jmax(u, KIN_WAVE_MIN_FLOW_QROOT);
    const double u3 = u * u * u;
    area = alpha * u3;
    q = u3 * u * u;
}

// ------------------------------------------------------------------ soil column ---------

template <int MAXN>
struct Column {
    int N, nl, nu;
    double act[MAXN], cum[MAXN + 1], thick[MAXN], usld[MAXN];
    double ts, tr, tfc, d, kv0, f, zexp;
    int profile;

    __device__ void load_static(const WfDevFields& F, int64_t slot) {
        N = F.N;
        nl = F.nlayers[slot];
        ts = F.L[THETA_S][slot];
        tr = F.L[THETA_R][slot];
        tfc = F.L[THETA_FC][slot];
        d = F.L[SOIL_THICKNESS][slot];
        zexp = F.L[Z_EXP][slot];
        profile = F.kv_profile;
        cum[0] = 0.0;
#pragma unroll
        for (int k = 0; k < MAXN; ++k) {
            act[k] = k < N ? F.LY[LY_ACT_THICK][k][slot] : NANV;
            cum[k + 1] = cum[k] + act[k];
        }
    }
    // utils.jl:390-409
    __device__ void set_thickness(double ref) {
        nu = N;
#pragma unroll
        for (int k = 0; k < MAXN; ++k) {
            if (k >= N) break;
            double t = act[k] * NANV;
            if (ref > cum[k + 1]) {
                t = act[k];
            } else if (ref - cum[k] > 0.0) {
                t = ref - cum[k];
            }
            thick[k] = t;
            if (wfm::isnan_(t)) nu -= 1;
        }
    }
    // utils.jl:727-761 (n is 1-based)
    __device__ __forceinline__ double kv_at(const double* kvf, double z, int n) const {
        double zz = z;
        if (profile == WF_KV_EXPONENTIAL_CONSTANT && !(z < zexp)) zz = zexp;
        return kvf[n - 1] * kv0 * wfm::exp(-f * zz);
    }
    // soil.jl:1213-1259
    __device__ void update_ustorelayerdepth(double zi_prev, double zi) {
        const int n_prev = nu;
        double tprev[MAXN];
#pragma unroll
        for (int k = 0; k < MAXN; ++k) tprev[k] = thick[k];
        set_thickness(zi);
        const int n_new = nu;
        if (zi < zi_prev) {
#pragma unroll
            for (int k = 1; k <= MAXN; ++k) {
                if (k < n_new || k > n_prev) continue;
                if (wfm::isnan_(thick[k - 1])) {
                    usld[k - 1] = 0.0;
                } else {
                    const double sc = thick[k - 1] / tprev[k - 1];
                    usld[k - 1] = sc * usld[k - 1];
                }
            }
        } else {
#pragma unroll
            for (int k = 1; k <= MAXN; ++k) {
                if (k < n_prev || k > n_new) continue;
                const double tp = wfm::isnan_(tprev[k - 1]) ? 0.0 : tprev[k - 1];
                const double delta = thick[k - 1] - tp;
                usld[k - 1] = usld[k - 1] + delta * (tfc - tr);
            }
        }
    }
    // utils.jl:1090-1131
    __device__ void water_table_change(double net_flux, double sy, double dt, double& dh, double& exfilt) const {
        const double te = ts - tr;
        if (net_flux <= 0.0) {
            dh = net_flux * dt / sy;
        } else {
            dh = 0.0;
#pragma unroll
            for (int k = MAXN; k >= 1; --k) {
                if (k > nu) continue;
                const double cap = jmax(thick[k - 1] * te - usld[k - 1], 0.0) / dt;
                const double fl = jmin(net_flux, cap);
                if (cap <= net_flux) {
                    dh += thick[k - 1];
                } else {
                    const double syk = te - (usld[k - 1] / thick[k - 1]);
                    dh += fl * dt / syk;
                }
                net_flux -= fl;
                if (net_flux == 0.0) break;
            }
        }
        exfilt = jmax(net_flux, 0.0);
    }
};

// routing/subsurface/subsurface_process.jl:6-41
__device__ __forceinline__ double ssf_celerity(double zi, double slope, double sy, double kh0, double f, int profile,
                                               double zexp) {
    double z = zi;
    if (profile == WF_KV_EXPONENTIAL_CONSTANT) z = zi < zexp ? zi : zexp;
    return (kh0 * wfm::exp(-f * z) * slope) / sy;
}

// routing/subsurface/subsurface_process.jl:57-78
__device__ double kw_ssf_newton(double q, double cterm, double celerity, double dt, double dx) {
    int count = 0;
    const double dt_dx = dt / dx;
    const double cinv = 1.0 / celerity;
    const double df = dt_dx + cinv;
    while (true) {
        const double fq = dt_dx * q + cinv * q - cterm;
        const double q_old = q;
        q -= (fq / df);
        if (wfm::isnan_(q)) q = 0.0;
        q = jmax(q, KIN_WAVE_MIN_FLOW);
        if ((wfm::fabs_(fq) <= 1.0e-12) || (count >= 3000)) break;
        if (q == q_old) break;  // fixed point: the remaining iterations repeat this one
        count += 1;
    }
    return q;
}

// routing/subsurface/subsurface_process.jl:89-172
template <int MAXN>
__device__ void kinematic_wave_ssf(double q_in, double q_prev, double zi_prev, double q_net, double slope, double sy,
                                   double d, double dt, double dx, double dw, double q_max, double kh0,
                                   Column<MAXN>& col, double& q_out, double& zi_out, double& exfilt_out,
                                   double& netflux_out) {
    if (q_in + q_prev == 0.0 && q_net <= 0.0) {
        q_out = 0.0;
        zi_out = d;
        exfilt_out = 0.0;
        netflux_out = 0.0;
        return;
    }
    const double f = col.f;
    double q = (q_prev + q_in) / 2.0;
    double cel = ssf_celerity(zi_prev, slope, sy, kh0, f, col.profile, col.zexp);
    double cterm = (dt / dx) * (q_in + q_net) + q_prev / cel;
    q = kw_ssf_newton(q, cterm, cel, dt, dx);
    q = jmin(q, (q_max * dw));
    double net_flux = (q_in + q_net - q) / (dw * dx);
    double dh, exfilt;
    col.water_table_change(net_flux, sy, dt, dh, exfilt);
    double zi = zi_prev - dh;
    if (zi > d) {
        const double q_excess = (dw * dx) * sy * (zi - d) / dt;
        q = jmax(q - q_excess, KIN_WAVE_MIN_FLOW);
    }
    zi = jclamp(zi, 0.0, d);
    const long its = (long)wfm::ceil_(wfm::round_sigdigits(wfm::fabs_(zi - zi_prev) / 0.1, 12));
    if (its > 1) {
        const double dt_s = dt / (double)its;
        double q_sum = 0.0, exfilt_sum = 0.0, net_flux_sum = 0.0;
        for (long i = 0; i < its; ++i) {
            cel = ssf_celerity(zi_prev, slope, sy, kh0, f, col.profile, col.zexp);
            cterm = (dt_s / dx) * q_in + q_prev / cel + q_net * (dt_s / dx);
            q = kw_ssf_newton(q_prev, cterm, cel, dt_s, dx);
            q = jmin(q, (q_max * dw));
            net_flux = (q_in + q_net - q) / (dw * dx);
            col.water_table_change(net_flux, sy, dt_s, dh, exfilt);
            zi = zi_prev - dh;
            if (zi > d) {
                const double q_excess = (dw * dx) * sy * (zi - d) / dt_s;
                q = jmax(q - q_excess, KIN_WAVE_MIN_FLOW);
            }
            zi = jclamp(zi, 0.0, d);
            col.update_ustorelayerdepth(zi_prev, zi);
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
        col.update_ustorelayerdepth(zi_prev, zi);
    }
    q_out = q;
    zi_out = zi;
    exfilt_out = exfilt;
    netflux_out = net_flux;
}

// ----------------------------------------------------------------- vertical kernel ------

// glacier_store * glacier_fraction of a cell (compute_total_storage, mass_balance.jl:96-113); the
// reference's zero term without a glacier
__device__ __forceinline__ double glacier_storage(const WfDevFields& F, int64_t e, int64_t slot) {
    return F.glacier ? F.GM[GM_STORE][e] * F.G[G_FRAC][slot] : 0.0 * 0.0;
}

// update_glacier_model! (glacier.jl:122-154) of one cell: glacier_hbv (snow_scheme.cuh) on its
// snow storage and glacier store. Returns the melt rate.
__device__ __forceinline__ double glacier_update(const WfDevFields& F, int64_t e, int64_t slot, double T, double dt,
                                                 double& snow) {
    double store, melt;
    wfsn::glacier_hbv(F.G[G_FRAC][slot], F.GM[GM_STORE][e], snow, T, F.G[G_TTM][slot], F.G[G_DDF][slot],
                      F.G[G_SIFRAC][slot], F.g_max_rate, dt, &snow, &store, &melt);
    F.GM[GM_STORE][e] = store;
    F.GM[GM_MELT][e] = melt;
    return melt;
}

// Parts of the per-cell update. VERT_ALL: the whole update_land_hydrology_model! (sbm.jl:82-132).
// With gravitational snow transport the transport sweep runs between VERT_SNOW (interception and
// snow, sbm.jl:92-96, and the transport capacities) and VERT_SOIL (glacier, open-water runoff and
// soil, sbm.jl:102-131).
enum VertPhase { VERT_ALL = 0, VERT_SNOW = 1, VERT_SOIL = 2 };

template <int MAXN, int PHASE>
__global__ void __launch_bounds__(256) vertical_kernel(WfDevFields F) {
    const int M = F.M;
    const int64_t E = F.land_slots * M;
    const double dt = F.dt;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t slot = e / M;
        if (F.land_node_of_slot[slot] < 0) continue;
        const int m = (int)(e - slot * M);
        double* const* Mf = F.Mf;
        double* const* L = F.L;
        const double Pr = Mf[PRECIP][e], PET = Mf[POTEVAP][e], T = Mf[TEMP][e];
        double canopy = Mf[CANOPY][e];
        double snow = Mf[SNOW][e], snow_water = Mf[SNOW_WATER][e];
        const double gap = L[GAP][slot], cmax = L[CMAX][slot];
        const double potevap = L[KC][slot] * PET * (1.0 - gap);
        double tf = 0.0, ic, sf = 0.0, srunoff = 0.0;
        if (PHASE != VERT_SOIL) {
        // storage_prev! of the land balance (mass_balance.jl:95-125, Wflow.jl:315)
        if (F.mass_balance)
            Mf[BL_PREV][e] = Mf[TSWS][e] + canopy + (snow + snow_water) + glacier_storage(F, e, slot) + 0.0;
        // ---- interception (canopy.jl:213-226 Gash, :259-271 Rutter)
        if (F.gash) {
            interception_gash(cmax, L[E_R][slot], gap, Pr, potevap, dt, tf, ic, sf);
        } else {
            interception_modrut(Pr, potevap, canopy, gap, cmax, dt, tf, ic, sf);
        }
        // ---- snow (snow.jl:238-293, snow_process.jl:26-116)
        if (F.snow) {
            const double eff = tf + sf;
            const double tti = L[TTI][slot], tt = L[TT][slot];
            double rainfrac;
            if (tti == 0.0) {
                rainfrac = T > tt ? 1.0 : 0.0;
            } else {
                rainfrac = jclamp((T - (tt - tti / 2.0)) / tti, 0.0, 1.0);
            }
            const double snowfrac = 1.0 - rainfrac;
            const double sp = snowfrac * 1.0 * eff, lp = rainfrac * 1.0 * eff;
            const double ttm = L[TTM][slot], ddf = L[DDF][slot], whc = L[WHC][slot];
            double melt;
            if (T > ttm) {
                melt = jmin(ddf * (T - ttm), snow / dt);
                snow -= melt * dt;
                snow_water += melt * dt;
            } else {
                melt = 0.0;
                const double refr = jmin(ddf * 0.05 * (ttm - T) * dt, snow_water);
                snow += refr;
                snow_water -= refr;
            }
            snow = jmax(snow, 0.0);
            snow_water = jmax(snow_water, 0.0);
            snow += sp * dt;
            snow_water += lp * dt;
            const double maxsw = snow * whc;
            if (snow_water > maxsw) {
                srunoff = (snow_water - maxsw) / dt;
                snow_water = maxsw;
            } else {
                srunoff = 0.0;
            }
            Mf[SWE][e] = snow_water + snow;
        }
        if (PHASE == VERT_SNOW) {
            // lateral_snow_transport! capacities from the updated states (surface_process.jl:9-19)
            Mf[CANOPY][e] = canopy;
            Mf[SNOW][e] = snow;
            Mf[SNOW_WATER][e] = snow_water;
            F.GM[GM_SRUNOFF][e] = srunoff;
            F.GM[GM_IC][e] = ic;
            const double frac = jmin(0.5, L[SLOPE][slot] / 5.67) * jmin(1.0, snow / 10.0);
            F.GM[GM_CAP][e] = frac * snow / dt;
            F.GM[GM_CAPW][e] = snow_water * frac / dt;
            continue;
        }
        } else {
            // after the transport sweep: the moved snow states, the interception and snow runoff
            // of VERT_SNOW
            ic = F.GM[GM_IC][e];
            srunoff = F.GM[GM_SRUNOFF][e];
        }
        // ---- glacier (glacier.jl:122-154) and the water flux at the surface (runoff.jl:37-58)
        double wfs, gfrac = 0.0;
        if (F.snow) {
            if (F.glacier) {
                gfrac = F.G[G_FRAC][slot];
                const double gmelt = glacier_update(F, e, slot, T, dt, snow);
                wfs = srunoff + gmelt * gfrac;
            } else {
                wfs = srunoff + 0.0 * 0.0;
            }
        } else {
            wfs = tf + sf;
        }
        // ---- open water runoff (runoff.jl:61-111)
        const double rfrac = L[RIVER_FRACTION][slot], wfrac = L[WATER_FRACTION][slot];
        const double wd_land = Mf[OL_H][e];
        const int64_t rs = F.land_river_slot[slot];
        const double wd_river = rs >= 0 ? F.RM[RV_H][rs * M + m] : 0.0;
        const double runoff_river = jmin(1.0, rfrac) * wfs;
        const double runoff_land = jmin(1.0, wfrac) * wfs;
        const double ae_river = rfrac * jmin(wd_river / dt, PET);
        const double ae_land = wfrac * jmin(wd_land / dt, PET);
        // ---- soil (soil.jl:643-682, 1150-1211)
        const double soil_fraction = jmax(gap - wfrac - rfrac - gfrac, 0.0);
        const double pot_trans = jmax(0.0, potevap - ic);
        double pot_soilevap = soil_fraction * PET;
        pot_soilevap -= 0.0;
        const double wfs_soil = jmax(wfs + 0.0 - runoff_river - runoff_land + 0.0, 0.0);

        Column<MAXN> col;
        col.load_static(F, slot);
        col.kv0 = Mf[KV0][e];
        col.f = Mf[FSCALE][e];
        const double ts = col.ts, tr = col.tr;
        const double swc = L[SWC][slot];
        double sat = Mf[SAT][e];
#pragma unroll
        for (int k = 0; k < MAXN; ++k) col.usld[k] = k < col.N ? F.LY[LY_USLD][k][e] : 0.0;
        double kvf[MAXN], cexp[MAXN], rfr[MAXN];
#pragma unroll
        for (int k = 0; k < MAXN; ++k) {
            kvf[k] = k < col.N ? F.LY[LY_KVFRAC][k][slot] : 0.0;
            cexp[k] = k < col.N ? F.LY[LY_C][k][slot] : 0.0;
            rfr[k] = k < col.N ? F.LY[LY_ROOTFRAC][k][slot] : 0.0;
        }
        // update_diagnostic_vars! (soil.jl:1400-1436)
        double usd = 0.0;
#pragma unroll
        for (int k = 0; k < MAXN; ++k)
            if (k < col.nl) usd += col.usld[k];
        double zi = jmax(0.0, col.d - sat / (ts - tr));
        double drain = (col.d - zi) * lb_drainable(ts, col.tfc);
        double ucap = swc - sat - usd;
        col.set_thickness(zi);
        // soil temperature and infiltration reduction (soil.jl:684-729)
        double tsoil = Mf[TSOIL][e];
        if (F.snow) tsoil = tsoil + L[W_SOIL][slot] * (T - tsoil);
        double fred = 1.0;
        if (F.snow && F.infilt_reduction) {
            const double cf = L[CF_SOIL][slot];
            fred = scurve(tsoil, 273.15, 1.0 / (1.0 - cf), 8.0) + cf;
        }
        // infiltration (soil_process.jl:16-41)
        const double cfrac = L[COMPACT_FRAC][slot];
        const double cap_soil = col.kv0 * kvf[0];
        const double cap_comp = L[CAP_COMP][slot];
        const double soilinf = wfs_soil * (1.0 - cfrac);
        const double pathinf = wfs_soil * cfrac;
        const double mis = jmin(cap_soil * fred, soilinf);
        const double mip = jmin(cap_comp * fred, pathinf);
        const double infiltration = jmin(mip + mis, jmax(0.0, ucap / dt));
        const double infex = (soilinf - mis) + (pathinf - mip);
        // unsaturated_zone_flow! (soil.jl:764-804)
        double transfer = 0.0;
        if (col.nu > 0) {
            double z = 0.0, flow = 0.0;
#pragma unroll
            for (int k = 0; k < MAXN; ++k) {
                if (k >= col.nu) break;
                z = z + col.thick[k];
                const double l_sat = col.thick[k] * (ts - tr);
                const double kv_z = col.kv_at(kvf, z, k + 1);
                const double u = k == 0 ? col.usld[k] + infiltration * dt : col.usld[k] + flow * dt;
                double uo;
                unsatzone_flow_layer(u, kv_z, l_sat, cexp[k], dt, uo, flow);
                col.usld[k] = uo;
            }
            transfer = flow;
        }
        // soil_evaporation! (soil.jl:814-856)
        double soilevap, esat;
        {
            double pot = pot_soilevap;
            double se;
            if (col.nu == 0) {
                se = 0.0;
            } else if (col.nu == 1) {
                se = pot * jmin(1.0, col.usld[0] / (zi * (ts - tr)));
            } else {
                se = pot * jmin(1.0, col.usld[0] / (col.thick[0] * (ts - tr)));
            }
            se = jmin(se, col.usld[0] / dt);
            pot -= se;
            col.usld[0] = col.usld[0] - se * dt;
            const double thd = lb_drainable(ts, col.tfc);
            if (col.nu == 0 || col.nu == 1) {
                esat = pot * jmin(1.0, (col.act[0] - zi) / col.act[0]);
                esat = jmin(esat, (col.act[0] - zi) * thd / dt);
            } else {
                esat = 0.0;
            }
            soilevap = se + esat;
            drain -= esat * dt;
        }
        // transpiration! (soil.jl:865-975)
        double actevapustore = 0.0, act_sat, transpiration;
        {
            const double rd = L[ROOTING_DEPTH][slot];
            const double h1 = L[H1][slot], h2 = L[H2][slot], h4 = L[H4][slot], a1 = L[ALPHA_H1][slot];
            const double psi = L[PSI_B][slot];
            const double h3 = feddes_h3(L[H3_HIGH][slot], L[H3_LOW][slot], pot_trans);
            double sum_rf = 0.0, rf_low = 0.0;
#pragma unroll
            for (int k = 1; k <= MAXN; ++k) {
                if (k > col.nu) break;
                double r;
                if (k == col.nu && zi < rd) {
                    const double rl = jmin(col.act[k - 1], rd - col.cum[k - 1]);
                    r = rfr[k - 1] * (col.thick[k - 1] / rl);
                } else {
                    r = rfr[k - 1];
                }
                sum_rf += r;
                rf_low = r;
            }
#pragma unroll
            for (int k = 1; k <= MAXN; ++k) {
                if (k > col.nu) break;
                const double r = k < col.nu ? rfr[k - 1] : rf_low;
                const double rs_ = rd > 0.0 ? jmax(1.0 / sum_rf, 1.0) * r : 0.0;
                const double vwc = jmax(col.usld[k - 1] / col.thick[k - 1], 1e-7);
                const double head = head_brooks_corey(vwc, ts, tr, cexp[k - 1], psi);
                const double alpha = rwu_feddes(head, h1, h2, h3, h4, a1);
                const double availcap = jmin(1.0, jmax(0.0, (rd - col.cum[k - 1]) / col.thick[k - 1]));
                const double maxextr = col.usld[k - 1] * availcap / dt;
                const double a = jmin(alpha * rs_ * pot_trans, maxextr);
                col.usld[k - 1] = col.usld[k - 1] - a * dt;
                actevapustore += a;
            }
            const double wetroots = scurve(zi, rd, 1.0, L[ROOTDISTPAR][slot]);
            const double alpha0 = rwu_feddes(0.0, h1, h2, h3, h4, a1);
            const double rest = pot_trans - actevapustore;
            act_sat = jmin(rest * wetroots * alpha0, drain / dt);
            drain -= act_sat * dt;
            transpiration = actevapustore + act_sat;
        }
        // actual_infiltration! (soil.jl:987-1017)
        double excess = 0.0;
#pragma unroll
        for (int k = MAXN; k >= 1; --k) {
            if (k > col.nu) continue;
            excess = jmax(0.0, col.usld[k - 1] - col.thick[k - 1] * (ts - tr));
            col.usld[k - 1] = col.usld[k - 1] - excess;
            if (k > 1) col.usld[k - 2] = col.usld[k - 2] + excess;
        }
        const double act_infilt = infiltration - excess / dt;
        const double satex = (wfs_soil - act_infilt) - infex;
        // unsaturated store and capacity for the capillary flux (soil.jl:1193-1196)
        usd = 0.0;
#pragma unroll
        for (int k = 0; k < MAXN; ++k)
            if (k < col.nl) usd += col.usld[k];
        ucap = swc - sat - usd;
        // capillary_flux! (soil.jl:1050-1111)
        double capflux_act = 0.0;
        if (col.nu > 0) {
            const double ksat = col.kv_at(kvf, zi, col.nu);
            const double maxcap = jmax(0.0, jmin(jmin(jmin(ksat, actevapustore), ucap / dt), drain / dt));
            const double rd = L[ROOTING_DEPTH][slot];
            const double chmax = L[CAP_HMAX][slot];
            double capflux = zi > rd ? maxcap * wfm::pow(1.0 - jmin(zi, chmax) / chmax, L[CAP_N][slot]) : 0.0;
#pragma unroll
            for (int k = MAXN; k >= 1; --k) {
                if (k > col.nu) continue;
                const double toadd =
                    jmin(capflux, jmax((col.thick[k - 1] * (ts - tr) - col.usld[k - 1]) / dt, 0.0));
                col.usld[k - 1] = col.usld[k - 1] + toadd * dt;
                capflux -= toadd;
                capflux_act += toadd;
            }
        }
        // leakage! (soil.jl:1118-1136)
        const double deepksat = col.kv_at(kvf, col.d, col.nl);
        const double leak = jmax(0.0, jmin(L[MAX_LEAKAGE][slot], jmin(drain / dt, deepksat)));
        const double recharge = (transfer - capflux_act - leak - act_sat - esat);
        double aet = soilevap + transpiration + ae_river + ae_land + 0.0;
        aet += ic;  // sbm.jl:130
        // ---- write back
        Mf[CANOPY][e] = canopy;
        Mf[SNOW][e] = snow;
        Mf[SNOW_WATER][e] = snow_water;
        Mf[TSOIL][e] = tsoil;
#pragma unroll
        for (int k = 0; k < MAXN; ++k)
            if (k < col.N) F.LY[LY_USLD][k][e] = col.usld[k];
        Mf[ZI][e] = zi;
        Mf[SSF_ZI][e] = zi;  // sbm_model.jl:80-81
        Mf[RECHARGE][e] = recharge;
        Mf[NET_RUNOFF_RIVER][e] = runoff_river - ae_river;
        Mf[AET][e] = aet;
        Mf[LEAKAGE][e] = leak;
        Mf[SATEX][e] = satex;
        Mf[INFEX][e] = infex;
        Mf[RUNOFF_LAND][e] = runoff_land;
        Mf[AE_LAND][e] = ae_land;
        Mf[INTERCEPTION][e] = ic;
        Mf[TRANSPIRATION][e] = transpiration;
        Mf[SOIL_EVAP][e] = soilevap;
        Mf[ACT_INFILT][e] = act_infilt;
    }
}

// ------------------------------------------------------------------ SSF wavefront -------

template <int MAXN>
struct SsfPhys {
    WfDevFields F;
    WfDevGraph g;
    WfSweep sw;

    __device__ bool node(int64_t slot, int64_t e, int m, int s, uint32_t ep, int64_t chain, bool is_end,
                         double& hq) {
        double* const* Mf = F.Mf;
        double* const* L = F.L;
        double dt_s;
        bool first, last;
        if (!wf_substep(sw, m, s, dt_s, first, last)) return true;
        const double area = L[AREA][slot];
        const double d = L[SOIL_THICKNESS][slot];
        double zi_ssf = Mf[SSF_ZI][e];
        // recharge flux (boundary_conditions.jl:219-236, check_flux :12-21)
        double flux = Mf[RECHARGE][e] * area;
        if (zi_ssf >= d) flux = jmax(0.0, flux);
        const double q_net = 0.0 + flux;
        // upstream inflow (lateral_subsurface_flow.jl:236-242)
        double qin = 0.0, tr = 0.0;
        for (int32_t o = g.up_ptr[slot]; o < g.up_ptr[slot + 1]; ++o) {
            double qu;
            if (!wfw::upstream_q(g, sw, hq, o, m, s, ep, F.status, qu)) return false;
            const double fr = L[FRAC_TO_RIVER][g.up_slot[o]];
            qin = qin + qu * (1.0 - fr);
            tr = tr + qu * fr;
        }
        Column<MAXN> col;
        col.load_static(F, slot);
        col.kv0 = Mf[KV0][e];
        col.f = Mf[FSCALE][e];
#pragma unroll
        for (int k = 0; k < MAXN; ++k) col.usld[k] = k < col.N ? F.LY[LY_USLD][k][e] : 0.0;
        const double zi_soil = Mf[ZI][e];
        col.set_thickness(zi_soil);
        const double q_prev = Mf[SSF_Q][e];
        const double kh0 = L[KH_RATIO][slot] * col.kv0;
        double q, zi_new, exfilt, netflux;
        kinematic_wave_ssf<MAXN>(qin, q_prev, zi_ssf, q_net, L[SLOPE][slot], L[SY][slot], d, dt_s, L[FLOW_LENGTH][slot],
                                 L[FLOW_WIDTH][slot], Mf[Q_MAX][e], kh0, col, q, zi_new, exfilt, netflux);
        const bool early = (qin + q_prev == 0.0 && q_net <= 0.0);
        Mf[SSF_Q][e] = q;
        hq = q;
        Mf[SSF_ZI][e] = zi_new;
        Mf[SSF_STORAGE][e] = L[SY][slot] * (d - zi_new) * area;
        // cumulative fluxes (set_flux_vars! zeroes them at the start of the model step)
        double c_tr = (first ? 0.0 : Mf[SSF_TR_CUM][e]) + tr * dt_s;
        double c_rf = (first ? 0.0 : Mf[RCH_FLUX_CUM][e]) + flux * dt_s;
        double c_qin = (first ? 0.0 : Mf[SSF_QIN_CUM][e]) + qin * dt_s;
        double c_q = (first ? 0.0 : Mf[SSF_Q_CUM][e]) + q * dt_s;
        double c_ex = (first ? 0.0 : Mf[SSF_EXF_CUM][e]) + exfilt * dt_s;
        double c_nf = (first ? 0.0 : Mf[SSF_QNET_CUM][e]) + netflux * area * dt_s;
        if (!early) {
#pragma unroll
            for (int k = 0; k < MAXN; ++k)
                if (k < col.N) F.LY[LY_USLD][k][e] = col.usld[k];
            Mf[ZI][e] = zi_new;
        }
        if (is_end) wfw::publish(g, chain, m, s, ep, q);
        if (!last) {
            Mf[SSF_TR_CUM][e] = c_tr;
            Mf[RCH_FLUX_CUM][e] = c_rf;
            Mf[SSF_QIN_CUM][e] = c_qin;
            Mf[SSF_Q_CUM][e] = c_q;
            Mf[SSF_EXF_CUM][e] = c_ex;
            Mf[SSF_QNET_CUM][e] = c_nf;
            return true;
        }
        // averages (groundwater.jl:622-638, lateral_subsurface_flow.jl:182-196)
        const double dt = sw.dt;
        const double exf_avg = c_ex / dt;
        Mf[RCH_FLUX_AVG][e] = c_rf / dt;
        Mf[SSF_QIN_AVG][e] = c_qin / dt;
        Mf[SSF_Q_AVG][e] = c_q / dt;
        Mf[SSF_QNET_AVG][e] = c_nf / dt;
        Mf[SSF_EXF_AVG][e] = exf_avg;
        Mf[SSF_TR_AVG][e] = c_tr / dt;
        // ---- update_soil_water_storage! (soil.jl:1294-1392), soil state after the sweep
        if (early) {
            // the soil column kept its state: reload it
#pragma unroll
            for (int k = 0; k < MAXN; ++k) col.usld[k] = k < col.N ? F.LY[LY_USLD][k][e] : 0.0;
            col.set_thickness(zi_soil);
        }
        const double zi_s = early ? zi_soil : Mf[ZI][e];
        const double ts = col.ts, tr_ = col.tr;
        double usd = 0.0;
#pragma unroll
        for (int k = 0; k < MAXN; ++k)
            if (k < col.nu) usd += col.usld[k];
        const double runoff =
            jmax(0.0, exf_avg + Mf[SATEX][e] + Mf[RUNOFF_LAND][e] + Mf[INFEX][e]);
        const double sat = (d - zi_s) * (ts - tr_);
        Mf[SAT][e] = sat;
        Mf[USTOREDEPTH][e] = usd;
        Mf[TSWS][e] = sat + usd;
        Mf[EXFILT][e] = exf_avg;
        Mf[RUNOFF][e] = runoff;
        const double net_runoff = runoff - Mf[AE_LAND][e];
        Mf[NET_RUNOFF][e] = net_runoff;
        // overland lateral inflow (surface_kinwave.jl:740-766, :365)
        const double inwater = (net_runoff + 0.0) * area + 0.0;
        Mf[OL_INWATER][e] = inwater;
        Mf[OL_QLAT][e] = inwater / L[FLOW_LENGTH][slot];
        return true;
    }
};

// --------------------------------------------------------------- overland wavefront -----

struct OverlandPhys {
    WfDevFields F;
    WfDevGraph g;
    WfSweep sw;

    __device__ bool node(int64_t slot, int64_t e, int m, int s, uint32_t ep, int64_t chain, bool is_end,
                         double& hq) {
        double* const* Mf = F.Mf;
        double* const* L = F.L;
        double dt_s;
        bool first, last;
        if (!wf_substep(sw, m, s, dt_s, first, last)) return true;
        if (first && F.mass_balance) Mf[BO_PREV][e] = Mf[OL_STORAGE][e];
        const double sfw = L[SFW][slot];
        double tr = 0.0, qin = 0.0;
        for (int32_t o = g.up_ptr[slot]; o < g.up_ptr[slot + 1]; ++o) {
            double qu;
            if (!wfw::upstream_q(g, sw, hq, o, m, s, ep, F.status, qu)) return false;
            const double fr = L[FRAC_TO_RIVER][g.up_slot[o]];
            tr = tr + qu * fr;
            qin = qin + qu * (1.0 - fr);
        }
        if (!(sfw > 0.0)) qin = 0.0;
        const double fl = L[FLOW_LENGTH][slot];
        double q, a;
        kinematic_wave(qin, Mf[OL_Q][e], Mf[OL_QLAT][e], L[OL_ALPHA][slot], dt_s, fl, q, a);
        double h = Mf[OL_H][e];
        if (sfw > 0.0) h = a / sfw;
        Mf[OL_Q][e] = q;
        hq = q;
        Mf[OL_H][e] = h;
        Mf[OL_STORAGE][e] = fl * sfw * h;
        if (is_end) wfw::publish(g, chain, m, s, ep, q);
        const double c_tr = (first ? 0.0 : Mf[OL_TR_CUM][e]) + tr * dt_s;
        const double c_q = (first ? 0.0 : Mf[OL_Q_CUM][e]) + q * dt_s;
        const double c_qin = (first ? 0.0 : Mf[OL_QIN_CUM][e]) + qin * dt_s;
        if (!last) {
            Mf[OL_TR_CUM][e] = c_tr;
            Mf[OL_Q_CUM][e] = c_q;
            Mf[OL_QIN_CUM][e] = c_qin;
            return true;
        }
        const double dt = sw.dt;
        Mf[OL_Q_AVG][e] = c_q / dt;
        Mf[OL_TR_AVG][e] = c_tr / dt;
        Mf[OL_QIN_AVG][e] = c_qin / dt;
        return true;
    }
};

// ------------------------------------------------------------------ river wavefront ------

// RES: the model has reservoirs. A reservoir cell hands its reservoir's outflow, not its river
// discharge, to the downstream cell: published for a light child, in the walker's hand-off
// register for the heavy child.
template <bool RES>
struct RiverPhys {
    WfDevFields F;
    WfDevGraph g;
    WfSweep sw;

    __device__ bool node(int64_t slot, int64_t e, int m, int s, uint32_t ep, int64_t chain, bool is_end,
                         double& hq) {
        double* const* RM = F.RM;
        double* const* R = F.R;
        const int M = F.M;
        double dt_s;
        bool first, last;
        if (!wf_substep(sw, m, s, dt_s, first, last)) return true;
        const double len = R[R_LENGTH][slot];
        double qlat;
        if (first) {
            if (F.mass_balance) RM[BR_PREV][e] = RM[RV_STORAGE][e];
            // update_lateral_inflow! (surface_kinwave.jl:710-734)
            const int64_t le = F.river_land_slot[slot] * M + m;
            const double inw = F.Mf[SSF_TR_AVG][le] + F.Mf[OL_TR_AVG][le] +
                               F.Mf[NET_RUNOFF_RIVER][le] * R[R_AREA][slot] + 0.0;
            RM[RV_INWATER][e] = inw;
            qlat = inw / len;
            RM[RV_QLAT][e] = qlat;
        } else {
            qlat = RM[RV_QLAT][e];
        }
        double qs = 0.0;
        for (int32_t o = g.up_ptr[slot]; o < g.up_ptr[slot + 1]; ++o) {
            double qu;
            if (!wfw::upstream_q(g, sw, hq, o, m, s, ep, F.status, qu)) return false;
            qs = qs + qu;
        }
        const double qin = 0.0 + qs;
        // external inflow / abstraction (surface_kinwave.jl:523-532)
        const double ext = R[R_EXT_INFLOW][slot];
        double inflow, absd = 0.0;
        if (ext < 0.0) {
            absd = jmin(-ext, (RM[RV_STORAGE][e] / dt_s) * 0.80);
            inflow = -absd / len;
        } else {
            inflow = ext / len;
        }
        inflow -= 0.0 / len;
        double q, a;
        kinematic_wave(qin, RM[RV_Q][e], qlat + inflow, R[R_ALPHA][slot], dt_s, len, q, a);
        RM[RV_Q][e] = q;
        double q_down = q;  // what the downstream cell receives
        if (RES) {
            const int32_t r = F.res_of_rslot[slot];
            if (r >= 0) q_down = wfr::reservoir_node(F, r, m, q, dt_s);
        }
        hq = q_down;
        RM[RV_H][e] = a / R[R_WIDTH][slot];
        RM[RV_STORAGE][e] = len * a;
        if (is_end) wfw::publish(g, chain, m, s, ep, q_down);
        const double c_q = (first ? 0.0 : RM[RV_Q_CUM][e]) + q * dt_s;
        const double c_qin = (first ? 0.0 : RM[RV_QIN_CUM][e]) + qin * dt_s;
        const double c_ab = (first ? 0.0 : RM[RV_ABS_CUM][e]) + absd * dt_s;
        if (!last) {
            RM[RV_Q_CUM][e] = c_q;
            RM[RV_QIN_CUM][e] = c_qin;
            RM[RV_ABS_CUM][e] = c_ab;
            return true;
        }
        const double dt = sw.dt;
        RM[RV_Q_AVG][e] = c_q / dt;
        RM[RV_ABS_AVG][e] = c_ab / dt;
        RM[RV_QIN_AVG][e] = c_qin / dt;
        return true;
    }
};

// --------------------------------------------------------- gravitational snow transport ----

// One material of lateral_snow_transport! (surface_process.jl:9-19): accucapacityflux! over the
// land graph (routing/utils.jl:82-104, 144-148). A cell's material is its own plus the hand-offs
// of its upstream cells, added in the order of the graph's topological sort (the order in which
// the reference's sweep hands them on); it passes min(material / dt, capacity) on to its
// downstream cell and keeps the rest. MAT 0: snow storage (snow_out = its flux), MAT 1: snow
// water (snow_out += its flux). FP64 in both forms (the split form's double-FP32 states are
// converted on the way in and out).
template <int MAT>
struct SnowPhys {
    WfDevFields F;
    WfDevGraph g;
    WfSweep sw;

    __device__ bool node(int64_t slot, int64_t e, int m, int s, uint32_t ep, int64_t chain, bool is_end,
                         double& hq) {
        const int f = MAT == 0 ? SNOW : SNOW_WATER;
        double material = F.split ? (double)F.Mh[f][e] + (double)F.Ml[f][e] : F.Mf[f][e];
        const int32_t o0 = g.up_ptr[slot], o1 = g.up_ptr[slot + 1];
        for (int32_t k = o0; k < o1; ++k) {
            double upd;
            if (!wfw::upstream_q(g, sw, hq, g.snow_up[k], m, s, ep, F.status, upd)) return false;
            material += upd;
        }
        const double dt = sw.dt;
        const double flux = jmin(material / dt, F.GM[MAT == 0 ? GM_CAP : GM_CAPW][e]);
        const double update = flux * dt;
        material -= update;
        if (F.split) {
            const wff::ff v = wff::from_d(material);
            F.Mh[f][e] = v.hi;
            F.Ml[f][e] = v.lo;
        } else {
            F.Mf[f][e] = material;
        }
        F.GM[GM_SNOW_OUT][e] = MAT == 0 ? flux : F.GM[GM_SNOW_OUT][e] + flux;
        hq = update;
        if (is_end) wfw::publish(g, chain, m, s, ep, update);
        return true;
    }
};

// flux_in! (routing/utils.jl:160-166): snow_in = the snow_out of the upstream cells, summed in
// the upstream lists' (ascending) order.
__global__ void __launch_bounds__(256) snow_in_kernel(WfDevFields F, WfDevGraph g) {
    const int M = F.M;
    const int64_t E = F.land_slots * M;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t slot = e / M;
        if (F.land_node_of_slot[slot] < 0) continue;
        const int m = (int)(e - slot * M);
        double acc = 0.0;
        for (int32_t o = g.up_ptr[slot]; o < g.up_ptr[slot + 1]; ++o) acc = acc + F.GM[GM_SNOW_OUT][g.up_slot[o] * M + m];
        F.GM[GM_SNOW_IN][e] = acc;
    }
}

template <class Phys>
__global__ void __launch_bounds__(128) walk_kernel(Phys phys) {
    wfw::walk(phys.g, phys.sw, phys, phys.F.status);
}

// ------------------------------------------------------------------ balance ------------

__device__ __forceinline__ void mb_error(double tin, double tout, double rate, double& err, double& rel) {
    err = tin - tout - rate;
    const double avg = (tin + tout) / 2.0;
    rel = avg == 0.0 ? 0.0 : err / avg;
}

__global__ void __launch_bounds__(256) balance_kernel(WfDevFields F) {
    const int M = F.M;
    const int64_t EL = F.land_slots * M, ER = F.river_slots * M;
    const double dt = F.dt;
    double* const* Mf = F.Mf;
    double* const* L = F.L;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < EL + ER; e += (int64_t)gridDim.x * blockDim.x) {
        if (e >= EL) {
            if (!F.mass_balance || F.li_coupled) continue;
            const int64_t re = e - EL;
            const int64_t rs = re / M;
            if (F.river_node_of_slot[rs] < 0) continue;
            double* const* RM = F.RM;
            // river kinematic wave balance (mass_balance.jl:290-313)
            const double tin = RM[RV_INWATER][re] + RM[RV_QIN_AVG][re] + jmax(0.0, F.R[R_EXT_INFLOW][rs]);
            const double tout = RM[RV_Q_AVG][re] + RM[RV_ABS_AVG][re] + 0.0;
            double err, rel;
            mb_error(tin, tout, (RM[RV_STORAGE][re] - RM[BR_PREV][re]) / dt, err, rel);
            RM[BR_ERR][re] = err;
            RM[BR_REL][re] = rel;
            continue;
        }
        const int64_t slot = e / M;
        if (F.land_node_of_slot[slot] < 0) continue;
        const int m = (int)(e - slot * M);
        // update_total_water_storage! (sbm.jl:143-182)
        const int64_t rs = F.land_river_slot[slot];
        const double area = L[AREA][slot];
        double ts = 0.0;
        if (rs >= 0) ts = ((F.RM[RV_H][rs * M + m] * F.R[R_WIDTH][rs] * F.R[R_LENGTH][rs]) / (area));
        const double snow = Mf[SNOW][e], sw = Mf[SNOW_WATER][e], canopy = Mf[CANOPY][e];
        const double glacier = glacier_storage(F, e, slot);
        ts += snow + sw + glacier + canopy + 0.0;
        const double sub_surface = Mf[USTOREDEPTH][e] + Mf[SAT][e];
        const double lateral = Mf[OL_H][e] * (1.0 - L[RIVER_FRACTION][slot]);
        ts += sub_surface + lateral;
        Mf[TOTAL_STORAGE][e] = ts;
        if (!F.mass_balance) continue;
        double err, rel;
        // land hydrology balance (mass_balance.jl:215-253)
        {
            const double Pv = F.split ? (double)F.Mh[PRECIP][e] : Mf[PRECIP][e];
            const double snow_in = F.snow_transport ? F.GM[GM_SNOW_IN][e] : 0.0;
            const double snow_out = F.snow_transport ? F.GM[GM_SNOW_OUT][e] : 0.0;
            const double tin = Mf[SSF_QIN_AVG][e] / area + (Pv + 0.0) + snow_in + 0.0 / area;
            const double vout = Mf[NET_RUNOFF][e] + Mf[AET][e] + Mf[NET_RUNOFF_RIVER][e] + Mf[LEAKAGE][e] + 0.0;
            const double tout = Mf[SSF_Q_AVG][e] / area + vout + snow_out + 0.0 / area;
            const double storage = Mf[TSWS][e] + canopy + (snow + sw) + glacier + 0.0;
            mb_error(tin, tout, (storage - Mf[BL_PREV][e]) / dt, err, rel);
            Mf[BL_ERR][e] = err;
            Mf[BL_REL][e] = rel;
        }
        // overland balance (mass_balance.jl:382-399); the local-inertial one is written by
        // li_couple_out_kernel
        if (!F.li_coupled) {
            mb_error(Mf[OL_INWATER][e] + Mf[OL_QIN_AVG][e], Mf[OL_Q_AVG][e],
                     (Mf[OL_STORAGE][e] - Mf[BO_PREV][e]) / dt, err, rel);
            Mf[BO_ERR][e] = err;
            Mf[BO_REL][e] = rel;
        }
        // subsurface balance (mass_balance.jl:470-490, groundwater.jl:671-695)
        {
            const double flux = Mf[RCH_FLUX_AVG][e];
            double fin = 0.0, fout = 0.0;
            if (flux > 0.0) fin += flux; else fout -= flux;
            mb_error(Mf[SSF_QIN_AVG][e] + fin, Mf[SSF_Q_AVG][e] + fout, Mf[SSF_QNET_AVG][e], err, rel);
            Mf[BS_ERR][e] = err;
            Mf[BS_REL][e] = rel;
        }
    }
}

// ---------------------------------------------------- local-inertial routing in the step ----
// (wf_li_couple.cuh; one member, FP64 form: element = slot)

// update_bc_overland_flow_model! (surface_staggered_scheme.jl:1080-1097): the land runoff of
// the step into the scheme's input, in its node order; the river's external inflow; the overland
// storage before the step for the balance (storage_prev!, mass_balance.jl:170-183).
__global__ void __launch_bounds__(256) li_couple_in_kernel(WfDevFields F, WfLiCoupleView v) {
    double* const* Mf = F.Mf;
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < F.land_slots;
         s += (int64_t)gridDim.x * blockDim.x) {
        const int64_t node = F.land_node_of_slot[s];
        if (node < 0) continue;
        double ro = (Mf[NET_RUNOFF][s] + Mf[NET_RUNOFF_RIVER][s]) * F.L[AREA][s];
        const int64_t rs = F.land_river_slot[s];
        if (rs >= 0) {
            ro += Mf[SSF_TR_AVG][s];  // get_flux_to_river (lateral_subsurface_flow.jl:346-347)
            v.ext[F.river_node_of_slot[rs]] = F.R[R_EXT_INFLOW][rs];
        }
        v.runoff[node] = ro;
        if (F.mass_balance) Mf[BO_PREV][s] = Mf[OL_STORAGE][s];
    }
}

// After the scheme's step: its depths, storages and the discharge of each river cell's outgoing
// edge into the model's overland and river fields, and the overland balance of every land cell
// (compute_flow_balance!, mass_balance.jl:402-461; add_inflow / add_outflow :355-376) with the
// river balance cleared (the reference computes none for this routing).
__global__ void __launch_bounds__(256) li_couple_out_kernel(WfDevFields F, WfLiCoupleView v, int balance) {
    double* const* Mf = F.Mf;
    double* const* RM = F.RM;
    const double dt = F.dt;
    const int64_t EL = F.land_slots, ER = F.river_slots;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < EL + ER;
         i += (int64_t)gridDim.x * blockDim.x) {
        if (i >= EL) {
            const int64_t rs = i - EL;
            const int64_t r = F.river_node_of_slot[rs];
            if (r < 0) continue;
            RM[RV_H][rs] = v.h_river[r];
            RM[RV_STORAGE][rs] = v.storage_river[r];
            const int64_t e = v.out_ptr[r] < v.out_ptr[r + 1] ? v.out_edge[v.out_ptr[r]] : -1;
            RM[RV_Q][rs] = e >= 0 ? v.q[e] : 0.0;
            RM[RV_Q_AVG][rs] = e >= 0 ? v.q_avg[e] : 0.0;
            if (F.mass_balance && balance) {
                RM[BR_ERR][rs] = 0.0;
                RM[BR_REL][rs] = 0.0;
            }
            continue;
        }
        const int64_t s = i;
        const int64_t node = F.land_node_of_slot[s];
        if (node < 0) continue;
        Mf[OL_H][s] = v.h_land[node];
        Mf[OL_STORAGE][s] = v.storage[node];
        Mf[OL_Q][s] = 0.0;
        Mf[OL_Q_AVG][s] = 0.0;
        if (!F.mass_balance || !balance) continue;
        double tin = 0.0, tout = 0.0;
        auto add_in = [&](double q) {
            if (q > 0.0) tin += q;
            else tout -= q;
        };
        auto add_out = [&](double q) {
            if (q > 0.0) tout += q;
            else tin -= q;
        };
        add_in(v.qx_avg[v.ixd[node]]);
        add_in(v.qy_avg[v.iyd[node]]);
        add_in(v.runoff[node]);
        add_out(v.qx_avg[node]);
        add_out(v.qy_avg[node]);
        const int64_t k = v.river_index[node];
        if (k >= 0) {
            double q_src = 0.0, q_dst = 0.0;
            for (int64_t o = v.in_ptr[k]; o < v.in_ptr[k + 1]; ++o) q_src += v.q_avg[v.in_edge[o]];
            add_in(q_src);
            tin += jmax(0.0, v.ext[k]);
            for (int64_t o = v.out_ptr[k]; o < v.out_ptr[k + 1]; ++o) q_dst += v.q_avg[v.out_edge[o]];
            add_out(q_dst);
            tout += v.abstraction_cum[k] / dt + v.abstraction[k];
        }
        double err, rel;
        mb_error(tin, tout, (v.storage[node] - Mf[BO_PREV][s]) / dt, err, rel);
        Mf[BO_ERR][s] = err;
        Mf[BO_REL][s] = rel;
    }
}

// volumetric water content of one layer after a step (soil.jl:1320-1342)
template <int MAXN>
__global__ void vwc_kernel(WfDevFields F, int layer, double* out) {
    const int M = F.M;
    const int64_t E = F.land_slots * M;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t slot = e / M;
        if (F.land_node_of_slot[slot] < 0) continue;
        Column<MAXN> col;
        col.load_static(F, slot);
        col.set_thickness(F.Mf[ZI][e]);
        const int k = layer + 1;
        double v = NANV;
        if (k <= col.nl) {
            if (k <= col.nu) {
                v = (F.LY[LY_USLD][layer][e] + (col.act[layer] - col.thick[layer]) * (col.ts - col.tr)) / col.act[layer] +
                    col.tr;
            } else {
                v = col.ts;
            }
        }
        out[e] = v;
    }
}

int grid_for(int64_t n, int block, int num_sms) {
    int64_t b = (n + block - 1) / block;
    int64_t cap = (int64_t)num_sms * 16;
    if (b > cap) b = cap;
    return (int)(b < 1 ? 1 : b);
}

template <class Phys>
cudaError_t launch_walk(const Phys& phys, const WfLaunchCfg& c) {
    const int threads = 32 * (c.walk_warps > 0 ? c.walk_warps : 4);
    int blocks;
    Phys p = phys;
    p.sw.SL = p.sw.aflag ? 1 : wave_sub_lanes(p.sw.S, c);
    cudaError_t err = wave_grid(walk_kernel<Phys>, threads, 0, c, p.g, blocks, p.sw.prio_items,
                                wf_items_per_chunk(p.g.G, p.g.M, p.sw.SL));
    if (err != cudaSuccess) return err;
    walk_kernel<Phys><<<blocks, threads, 0, c.stream>>>(p);
    return cudaGetLastError();
}

}  // namespace

template <int PHASE>
cudaError_t launch_vertical(const WfDevFields& F, const WfLaunchCfg& c) {
    const int block = c.vertical_block > 0 ? c.vertical_block : 128;
    const int grid = grid_for(F.land_slots * F.M, block, c.num_sms);
    if (F.N <= 4)
        vertical_kernel<4, PHASE><<<grid, block, 0, c.stream>>>(F);
    else
        vertical_kernel<WF_MAX_LAYERS, PHASE><<<grid, block, 0, c.stream>>>(F);
    return cudaGetLastError();
}

cudaError_t wf_fp64_vertical(const WfDevFields& F, const WfLaunchCfg& c) { return launch_vertical<VERT_ALL>(F, c); }
cudaError_t wf_fp64_vertical_snow(const WfDevFields& F, const WfLaunchCfg& c) {
    return launch_vertical<VERT_SNOW>(F, c);
}
cudaError_t wf_fp64_vertical_soil(const WfDevFields& F, const WfLaunchCfg& c) {
    return launch_vertical<VERT_SOIL>(F, c);
}

cudaError_t wf_fp64_ssf(const WfDevFields& F, const WfDevGraph& g, const WfSweep& sw, const WfLaunchCfg& c) {
    if (F.N <= 4) return launch_walk(SsfPhys<4>{F, g, sw}, c);
    return launch_walk(SsfPhys<WF_MAX_LAYERS>{F, g, sw}, c);
}

cudaError_t wf_snow_transport_sweep(const WfDevFields& F, const WfDevGraph& g, const WfSweep& sw, int material,
                                    const WfLaunchCfg& c) {
    if (material == 0) return launch_walk(SnowPhys<0>{F, g, sw}, c);
    return launch_walk(SnowPhys<1>{F, g, sw}, c);
}

cudaError_t wf_snow_in(const WfDevFields& F, const WfDevGraph& g, const WfLaunchCfg& c) {
    snow_in_kernel<<<grid_for(F.land_slots * F.M, 256, c.num_sms), 256, 0, c.stream>>>(F, g);
    return cudaGetLastError();
}

cudaError_t wf_fp64_li_couple_in(const WfDevFields& F, const WfLiCoupleView& v, const WfLaunchCfg& c) {
    li_couple_in_kernel<<<grid_for(F.land_slots, 256, c.num_sms), 256, 0, c.stream>>>(F, v);
    return cudaGetLastError();
}
cudaError_t wf_fp64_li_couple_out(const WfDevFields& F, const WfLiCoupleView& v, int balance, const WfLaunchCfg& c) {
    li_couple_out_kernel<<<grid_for(F.land_slots + F.river_slots, 256, c.num_sms), 256, 0, c.stream>>>(F, v,
                                                                                                     balance);
    return cudaGetLastError();
}

cudaError_t wf_fp64_overland(const WfDevFields& F, const WfDevGraph& g, const WfSweep& sw, const WfLaunchCfg& c) {
    return launch_walk(OverlandPhys{F, g, sw}, c);
}

cudaError_t wf_fp64_river(const WfDevFields& F, const WfDevGraph& g, const WfSweep& sw, const WfLaunchCfg& c) {
    if (F.n_res > 0) return launch_walk(RiverPhys<true>{F, g, sw}, c);
    return launch_walk(RiverPhys<false>{F, g, sw}, c);
}

// ------------------------------------------------------------------ reservoirs -----------
// Kernels of both arithmetic forms (reservoir state is FP64 in both).

// A member field of the land layout as FP64 (double-FP32 pair in the split form).
__device__ __forceinline__ double land_member_d(const WfDevFields& F, int f, int64_t e) {
    return F.split ? (double)F.Mh[f][e] + (double)F.Ml[f][e] : F.Mf[f][e];
}

// Before the river sweep: storage at the start of the step for the water balance
// (mass_balance.jl:156-160), the inflow from the outlet cell's overland and subsurface flow
// (update_inflow!, surface_kinwave.jl:771-802; the overland part excludes what goes to the
// river, which the river's lateral inflow carries) and the reset of the step's cumulatives
// (set_reservoir_vars!, surface_kinwave.jl:227-237).
__global__ void __launch_bounds__(256) reservoir_prep_kernel(WfDevFields F) {
    const int M = F.M;
    const int64_t E = F.n_res * M;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = e / M;
        const int m = (int)(e - r * M);
        const int64_t le = F.res_land_slot[r] * M + m;
        double* const* RS = F.RS;
        if (F.mass_balance) RS[RS_PREV][e] = RS[RS_STORAGE][e];
        RS[RS_IN_OL][e] = land_member_d(F, OL_Q_AVG, le);
        RS[RS_IN_SSF][e] = land_member_d(F, SSF_Q_AVG, le);
        RS[RS_IN_CUM][e] = 0.0;
        RS[RS_OUT_CUM][e] = 0.0;
        RS[RS_DOWN_CUM][e] = 0.0;
        RS[RS_EVAP_CUM][e] = 0.0;
        RS[RS_ABS_CUM][e] = 0.0;
    }
}

// After the river sweep: step averages (average_reservoir_vars!, surface_kinwave.jl:244-258) and
// the reservoir water balance (compute_flow_balance!, mass_balance.jl:261-284).
__global__ void __launch_bounds__(256) reservoir_post_kernel(WfDevFields F) {
    const int M = F.M;
    const int64_t E = F.n_res * M;
    const double dt = F.dt;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = e / M;
        double* const* RS = F.RS;
        RS[RS_OUT_AVG][e] = RS[RS_OUT_CUM][e] / dt;
        RS[RS_IN_AVG][e] = RS[RS_IN_CUM][e] / dt;
        RS[RS_ABS_AVG][e] = RS[RS_ABS_CUM][e] / dt;
        if (!F.mass_balance) continue;
        RS[RS_EVAP_AVG][e] = RS[RS_EVAP_CUM][e] / dt;
        const double area = F.RP[RP_AREA][r];
        const double tin = RS[RS_IN_AVG][e] + RS[RS_PRECIP][e] * area;
        const double tout = RS[RS_OUT_AVG][e] + RS[RS_EVAP_AVG][e] * area;
        double err, rel;
        mb_error(tin, tout, (RS[RS_STORAGE][e] - RS[RS_PREV][e]) / dt, err, rel);
        RS[RS_ERR][e] = err;
        RS[RS_REL][e] = rel;
    }
}

cudaError_t wf_reservoir_prep(const WfDevFields& F, const WfLaunchCfg& c) {
    if (F.n_res <= 0) return cudaSuccess;
    reservoir_prep_kernel<<<grid_for(F.n_res * F.M, 256, c.num_sms), 256, 0, c.stream>>>(F);
    return cudaGetLastError();
}

cudaError_t wf_reservoir_post(const WfDevFields& F, const WfLaunchCfg& c) {
    if (F.n_res <= 0) return cudaSuccess;
    reservoir_post_kernel<<<grid_for(F.n_res * F.M, 256, c.num_sms), 256, 0, c.stream>>>(F);
    return cudaGetLastError();
}

cudaError_t wf_fp64_balance(const WfDevFields& F, const WfLaunchCfg& c) {
    const int block = 256;
    const int grid = grid_for((F.land_slots + F.river_slots) * F.M, block, c.num_sms);
    balance_kernel<<<grid, block, 0, c.stream>>>(F);
    return cudaGetLastError();
}

cudaError_t wf_fp64_vwc(const WfDevFields& F, int layer, double* out, const WfLaunchCfg& c) {
    const int block = 256;
    const int grid = grid_for(F.land_slots * F.M, block, c.num_sms);
    if (F.N <= 4)
        vwc_kernel<4><<<grid, block, 0, c.stream>>>(F, layer, out);
    else
        vwc_kernel<WF_MAX_LAYERS><<<grid, block, 0, c.stream>>>(F, layer, out);
    return cudaGetLastError();
}
