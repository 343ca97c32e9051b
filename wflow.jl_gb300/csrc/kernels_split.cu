// kernels_split.cu -- FP32/FP64 split form of the SBM + kinematic-wave step.
//
// GB300 runs FP32 at about 64 times its FP64 rate, so this form evaluates every rate that
// needs a transcendental (Brooks-Corey powers, exponential Kv profile, Feddes heads, s-curves,
// the Gash log, soil-column drainage iterations) in FP32 with CUDA's accurate expf/logf, reads
// parameters and forcing as FP32, and keeps in FP64 only:
//   * every storage state (canopy, snow, unsaturated layers, saturated store / water table,
//     subsurface, overland and river discharge and storage) and every update applied to it,
//     so the water balance stays closed to FP64 rounding;
//   * the flux partitions and sums that enter the balance (throughfall/stemflow/canopy,
//     rain/snow, infiltration and excess water, actual evapotranspiration, runoff);
//   * the kinematic-wave Newton-Raphson solves for discharge (surface_process.jl:24-70,
//     subsurface_process.jl:57-78), with FP32 only for the initial guess, the q^0.2 seed
//     (refined by one FP64 Newton step) and the reciprocal of the Newton derivative;
//   * the cumulative sub-step fluxes and the balance terms.
// The process structure, limiters and branch order are those of the FP64 form (see
// kernels_fp64.cu for the reference line citations of each function).
#include <cuda_runtime.h>

#include "wf_fields.cuh"
#include "wf_kernels.h"
#include "wf_math.cuh"
#include "wf_walker.cuh"

using wfm::jclamp;
using wfm::jmax;
using wfm::jmin;

namespace {

constexpr double KIN_WAVE_MIN_FLOW = 1e-30;
constexpr double KIN_WAVE_MIN_FLOW_QROOT = 0x1.0c6f7a0b5ed8ap-20;
constexpr float MM_PER_DAY_F = (float)((1.0 / 86400.0) * 1e-3);

__device__ __forceinline__ float fminj(float x, float y) {
    if (x != x || y != y) return x + y;
    return x < y ? x : y;
}
__device__ __forceinline__ float fmaxj(float x, float y) {
    if (x != x || y != y) return x + y;
    return x > y ? x : y;
}
__device__ __forceinline__ float powj(float x, float y) { return expf(y * logf(x)); }  // Wflow's pow in FP32

// ---- FP32 drainage rate of one unsaturated layer (soil_process.jl:51-92); returns the rate and
// whether the iteration emptied the layer.
__device__ float unsat_rate(float usd, float kv_z, float l_sat, float c, float dt, bool& drained) {
    drained = false;
    const float st_sat = fmaxj(0.0f, usd - l_sat);
    const float ratio = usd / l_sat;
    float st = kv_z * (ratio > 1.0f ? 1.0f : powj(ratio, c));
    float sum_ast = fminj(st, st_sat / dt);
    usd -= sum_ast * dt;
    const float remainder = fminj((st - sum_ast) * dt, usd);
    const int its = (int)ceilf(remainder / 2e-4f);
    for (int i = 0; i < its; ++i) {
        const float r2 = usd / l_sat;
        st = (kv_z / (float)its) * (r2 > 1.0f ? 1.0f : powj(r2, c));
        const float st_max = usd / dt;
        if (st < st_max) {
            usd -= st * dt;
            sum_ast += st;
        } else {
            drained = true;
            break;
        }
    }
    return sum_ast;
}

__device__ __forceinline__ float rwu_feddes_f(float h, float h1, float h2, float h3, float h4, float a1) {
    if (h < h4) return 0.0f;
    if (h < h3) return (h - h4) / (h3 - h4);
    if (a1 == 0.0f) {
        if (h < h2) return 1.0f;
        if (h < h1) return (h1 - h) / (h1 - h2);
        return 0.0f;
    }
    return 1.0f;
}

// kinematic wave for surface flow with an FP64 Newton solve
__device__ void kinematic_wave_split(double q_in, double q_prev, double q_lat, double alpha, double dt, double dx,
                                     double& q, double& area) {
    if (q_in + q_prev + q_lat == 0.0) {
        q = 0.0;
        area = 0.0;
        return;
    }
    const double dt_dx = dt / dx;
    double u_prev = 0.0;
    if (q_prev > 0.0) {
        const float u0 = powj((float)q_prev, 0.2f);
        double u = (double)u0;
        if (u0 > 0.0f) {  // one FP64 Newton step on u^5 = q_prev
            const double u2 = u * u;
            const double inv = (double)(1.0f / (5.0f * u0 * u0 * u0 * u0));
            u = u - (u2 * u2 * u - q_prev) * inv;
        }
        u_prev = u;
    }
    const double cterm = dt_dx * q_in + alpha * u_prev * u_prev * u_prev + dt * q_lat;
    double u = u_prev > 0.0 ? u_prev : (double)cbrtf((float)(cterm / alpha));
    const double c1 = 5.0 * dt_dx, c2 = 3.0 * alpha;
    for (int it = 0; it < 3000; ++it) {
        const double u2 = u * u;
        const double u3 = u2 * u;
        const double fu = u3 * (dt_dx * u2 + alpha) - cterm;
        if (wfm::fabs_(fu) <= 1.0e-12) break;
        const double df = u2 * (c1 * u2 + c2);
        const float rdf = 1.0f / (float)df;
        const double u_old = u;
        u -= (rdf == rdf && rdf != 0.0f && wfm::fabs_((double)rdf) < 3.0e38) ? fu * (double)rdf : fu / df;
        if (wfm::isnan_(u) || u <= 0.0) u = KIN_WAVE_MIN_FLOW_QROOT;
        if (u == u_old) break;
    }
    u = jmax(u, KIN_WAVE_MIN_FLOW_QROOT);
    const double u3 = u * u * u;
    area = alpha * u3;
    q = u3 * u * u;
}

// ----------------------------------------------------------------- soil column ----------

template <int MAXN>
struct ColumnS {
    int N, nl, nu;
    double act[MAXN], cum[MAXN + 1], thick[MAXN], usld[MAXN];
    double ts, tr, tfc, d;
    float kv0, f, zexp;
    int profile;

    __device__ void load_static(const WfDevFields& F, int64_t slot) {
        N = F.N;
        nl = F.nlayers[slot];
        ts = F.L[THETA_S][slot];
        tr = F.L[THETA_R][slot];
        tfc = F.L[THETA_FC][slot];
        d = F.L[SOIL_THICKNESS][slot];
        zexp = F.Lf[Z_EXP][slot];
        profile = F.kv_profile;
        cum[0] = 0.0;
#pragma unroll
        for (int k = 0; k < MAXN; ++k) {
            act[k] = k < N ? F.LY[LY_ACT_THICK][k][slot] : __longlong_as_double(0x7ff8000000000000LL);
            cum[k + 1] = cum[k] + act[k];
        }
    }
    __device__ void set_thickness(double ref) {
        nu = N;
#pragma unroll
        for (int k = 0; k < MAXN; ++k) {
            if (k >= N) break;
            double t = __longlong_as_double(0x7ff8000000000000LL);
            if (ref > cum[k + 1]) {
                t = act[k];
            } else if (ref - cum[k] > 0.0) {
                t = ref - cum[k];
            }
            thick[k] = t;
            if (t != t) nu -= 1;
        }
    }
    __device__ __forceinline__ float kv_at(const float* kvf, double z, int n) const {
        float zz = (float)z;
        if (profile == WF_KV_EXPONENTIAL_CONSTANT && !(zz < zexp)) zz = zexp;
        return kvf[n - 1] * kv0 * expf(-f * zz);
    }
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
                if (thick[k - 1] != thick[k - 1]) {
                    usld[k - 1] = 0.0;
                } else {
                    usld[k - 1] = (thick[k - 1] / tprev[k - 1]) * usld[k - 1];
                }
            }
        } else {
#pragma unroll
            for (int k = 1; k <= MAXN; ++k) {
                if (k < n_prev || k > n_new) continue;
                const double tp = tprev[k - 1] != tprev[k - 1] ? 0.0 : tprev[k - 1];
                usld[k - 1] = usld[k - 1] + (thick[k - 1] - tp) * (tfc - tr);
            }
        }
    }
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
                    dh += fl * dt / (te - (usld[k - 1] / thick[k - 1]));
                }
                net_flux -= fl;
                if (net_flux == 0.0) break;
            }
        }
        exfilt = jmax(net_flux, 0.0);
    }
};

// ----------------------------------------------------------------- vertical kernel ------

template <int MAXN>
__global__ void __launch_bounds__(256) vertical_split_kernel(WfDevFields F) {
    const int M = F.M;
    const int64_t E = F.land_slots * M;
    const double dt = F.dt;
    const float dtf = (float)dt;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t slot = e / M;
        if (F.land_node_of_slot[slot] < 0) continue;
        const int m = (int)(e - slot * M);
        double* const* Mf = F.Mf;
        float* const* Mh = F.Mh;
        float* const* Lf = F.Lf;
        const float Pf = Mh[PRECIP][e], PETf = Mh[POTEVAP][e], Tf = Mh[TEMP][e];
        const double Pd = (double)Pf, PET = (double)PETf;
        double canopy = Mf[CANOPY][e];
        double snow = Mf[SNOW][e], snow_water = Mf[SNOW_WATER][e];
        if (F.mass_balance) Mf[BL_PREV][e] = Mf[TSWS][e] + canopy + (snow + snow_water);
        // ---- interception
        const float gapf = Lf[GAP][slot], cmaxf = Lf[CMAX][slot];
        const double gap = gapf, cmax = cmaxf;
        const double potevap = (double)(Lf[KC][slot] * PETf * (1.0f - gapf));
        double tf, ic, sf;
        if (F.gash) {
            const float e_rf = Lf[E_R][slot];
            const double e_r = e_rf;
            if (cmax > 0.0) {
                double fs, fi, psat;
                if (gap < 1.0 / 1.1) {
                    fs = 0.1 * gap;
                    fi = 1.0 - 1.1 * gap;
                    psat = e_r > fi ? 0.0
                                    : (double)(-cmaxf / (e_rf * dtf) * logf(1.0f - e_rf / (float)fi));
                } else {
                    fs = 1.0 - gap;
                    fi = 0.0;
                    psat = 0.0;
                }
                ic = Pd > psat ? (fi * psat - cmax / dt) + e_r * (Pd - psat) + cmax / dt : fi * Pd;
                sf = fs * Pd;
                tf = Pd - ic - sf;
                if (ic > potevap) {
                    tf += ic - potevap;
                    ic = potevap;
                }
            } else {
                tf = Pd;
                ic = 0.0;
                sf = 0.0;
            }
        } else {
            double fs, pc;
            if (gap < 1.0 / 1.1) {
                fs = 0.1 * gap;
                pc = (1.0 - gap - fs) * Pd;
            } else {
                fs = 1.0 - gap;
                pc = 0.0;
            }
            sf = fs * Pd;
            tf = gap * Pd;
            if (canopy > cmax) {
                tf += (canopy - cmax) / dt;
                canopy = cmax;
            }
            canopy += pc * dt;
            const double max_evap = canopy / dt;
            if (potevap > max_evap) {
                ic = max_evap;
                canopy = 0.0;
            } else {
                ic = potevap;
                canopy -= ic * dt;
            }
            if (canopy > cmax) {
                tf += (canopy - cmax) / dt;
                canopy = cmax;
            }
        }
        // ---- snow
        double wfs;
        float swe_out = 0.0f;
        if (F.snow) {
            const double eff = tf + sf;
            const float tti = Lf[TTI][slot], tt = Lf[TT][slot];
            const float rainfrac = tti == 0.0f ? (Tf > tt ? 1.0f : 0.0f)
                                               : fminj(fmaxj((Tf - (tt - tti / 2.0f)) / tti, 0.0f), 1.0f);
            const double lp = (double)rainfrac * eff;
            const double sp = eff - lp;
            const float ttm = Lf[TTM][slot], ddf = Lf[DDF][slot];
            if (Tf > ttm) {
                const double melt = jmin((double)(ddf * (Tf - ttm)), snow / dt);
                snow -= melt * dt;
                snow_water += melt * dt;
            } else {
                const double refr = jmin((double)(ddf * 0.05f * (ttm - Tf) * dtf), snow_water);
                snow += refr;
                snow_water -= refr;
            }
            snow = jmax(snow, 0.0);
            snow_water = jmax(snow_water, 0.0);
            snow += sp * dt;
            snow_water += lp * dt;
            const double maxsw = snow * (double)Lf[WHC][slot];
            double srunoff = 0.0;
            if (snow_water > maxsw) {
                srunoff = (snow_water - maxsw) / dt;
                snow_water = maxsw;
            }
            swe_out = (float)(snow_water + snow);
            wfs = srunoff;
        } else {
            wfs = tf + sf;
        }
        // ---- open water
        const double rfrac = F.L[RIVER_FRACTION][slot], wfrac = F.L[WATER_FRACTION][slot];
        const double wd_land = Mf[OL_H][e];
        const int64_t rs = F.land_river_slot[slot];
        const double wd_river = rs >= 0 ? F.RM[RV_H][rs * M + m] : 0.0;
        const double runoff_river = jmin(1.0, rfrac) * wfs;
        const double runoff_land = jmin(1.0, wfrac) * wfs;
        const double ae_river = rfrac * jmin(wd_river / dt, PET);
        const double ae_land = wfrac * jmin(wd_land / dt, PET);
        // ---- soil
        const double soil_fraction = jmax(gap - wfrac - rfrac, 0.0);
        const double pot_trans = jmax(0.0, potevap - ic);
        const double pot_soilevap = soil_fraction * PET;
        const double wfs_soil = jmax(wfs - runoff_river - runoff_land, 0.0);
        ColumnS<MAXN> col;
        col.load_static(F, slot);
        col.kv0 = Mh[KV0][e];
        col.f = Mh[FSCALE][e];
        const double ts = col.ts, tr = col.tr, te = ts - tr;
        const float tef = (float)te;
        const double swc = F.L[SWC][slot];
        const double sat = Mf[SAT][e];
#pragma unroll
        for (int k = 0; k < MAXN; ++k) col.usld[k] = k < col.N ? F.LY[LY_USLD][k][e] : 0.0;
        float kvf[MAXN], cexp[MAXN], rfr[MAXN];
#pragma unroll
        for (int k = 0; k < MAXN; ++k) {
            kvf[k] = k < col.N ? F.LYf[LY_KVFRAC][k][slot] : 0.0f;
            cexp[k] = k < col.N ? F.LYf[LY_C][k][slot] : 0.0f;
            rfr[k] = k < col.N ? F.LYf[LY_ROOTFRAC][k][slot] : 0.0f;
        }
        double usd = 0.0;
#pragma unroll
        for (int k = 0; k < MAXN; ++k)
            if (k < col.nl) usd += col.usld[k];
        const double zi = jmax(0.0, col.d - sat / te);
        double drain = (col.d - zi) * jmax(ts - col.tfc, 0.02);
        double ucap = swc - sat - usd;
        col.set_thickness(zi);
        float tsoil = Mh[TSOIL][e];
        if (F.snow) tsoil = tsoil + Lf[W_SOIL][slot] * (Tf - tsoil);
        float fred = 1.0f;
        if (F.snow && F.infilt_reduction) {
            const float cf = Lf[CF_SOIL][slot];
            fred = 1.0f / (1.0f / (1.0f - cf) + expf(-8.0f * (tsoil - 273.15f))) + cf;
        }
        // infiltration
        const double cfrac = F.L[COMPACT_FRAC][slot];
        const double cap_soil = (double)(col.kv0 * kvf[0]);
        const double cap_comp = F.L[CAP_COMP][slot];
        const double soilinf = wfs_soil * (1.0 - cfrac);
        const double pathinf = wfs_soil * cfrac;
        const double mis = jmin(cap_soil * fred, soilinf);
        const double mip = jmin(cap_comp * fred, pathinf);
        const double infiltration = jmin(mip + mis, jmax(0.0, ucap / dt));
        const double infex = (soilinf - mis) + (pathinf - mip);
        // unsaturated zone flow: FP32 rates, FP64 layer stores
        double transfer = 0.0;
        if (col.nu > 0) {
            double z = 0.0, flow = 0.0;
#pragma unroll
            for (int k = 0; k < MAXN; ++k) {
                if (k >= col.nu) break;
                z = z + col.thick[k];
                const double l_sat = col.thick[k] * te;
                const float kv_z = col.kv_at(kvf, z, k + 1);
                const double u = col.usld[k] + (k == 0 ? infiltration : flow) * dt;
                if (u <= 0.0) {
                    col.usld[k] = 0.0;
                    flow = 0.0;
                    continue;
                }
                bool drained;
                double rate = (double)unsat_rate((float)u, kv_z, (float)l_sat, cexp[k], dtf, drained);
                double un = u - rate * dt;
                if (drained || un < 0.0) {
                    rate = u / dt;
                    un = 0.0;
                }
                col.usld[k] = un;
                flow = rate;
            }
            transfer = flow;
        }
        // soil evaporation
        double soilevap, esat;
        {
            double pot = pot_soilevap;
            double se;
            if (col.nu == 0) {
                se = 0.0;
            } else if (col.nu == 1) {
                se = pot * jmin(1.0, col.usld[0] / (zi * te));
            } else {
                se = pot * jmin(1.0, col.usld[0] / (col.thick[0] * te));
            }
            se = jmin(se, col.usld[0] / dt);
            pot -= se;
            col.usld[0] -= se * dt;
            if (col.nu == 0 || col.nu == 1) {
                esat = pot * jmin(1.0, (col.act[0] - zi) / col.act[0]);
                esat = jmin(esat, (col.act[0] - zi) * jmax(ts - col.tfc, 0.02) / dt);
            } else {
                esat = 0.0;
            }
            soilevap = se + esat;
            drain -= esat * dt;
        }
        // transpiration: FP32 heads and reduction factors, FP64 extraction
        double actevapustore = 0.0, act_sat;
        {
            const double rd = F.L[ROOTING_DEPTH][slot];
            const float h1 = Lf[H1][slot], h2 = Lf[H2][slot], h4 = Lf[H4][slot], a1 = Lf[ALPHA_H1][slot];
            const float psi = Lf[PSI_B][slot];
            const float tpd = (float)pot_trans / MM_PER_DAY_F;
            const float h3l = Lf[H3_LOW][slot], h3h = Lf[H3_HIGH][slot];
            const float h3 = tpd <= 1.0f ? h3l : (tpd < 5.0f ? h3l + (h3h - h3l) * (tpd - 1.0f) / 4.0f : h3h);
            double sum_rf = 0.0, rf_low = 0.0;
#pragma unroll
            for (int k = 1; k <= MAXN; ++k) {
                if (k > col.nu) break;
                double r = rfr[k - 1];
                if (k == col.nu && zi < rd) r = r * (col.thick[k - 1] / jmin(col.act[k - 1], rd - col.cum[k - 1]));
                sum_rf += r;
                rf_low = r;
            }
#pragma unroll
            for (int k = 1; k <= MAXN; ++k) {
                if (k > col.nu) break;
                const double r = k < col.nu ? (double)rfr[k - 1] : rf_low;
                const double rs_ = rd > 0.0 ? jmax(1.0 / sum_rf, 1.0) * r : 0.0;
                const float vwc = fmaxj((float)(col.usld[k - 1] / col.thick[k - 1]), 1e-7f);
                const float lam = 2.0f / (cexp[k - 1] - 3.0f);
                const float head = lam > 0.0f ? psi / powj(vwc / tef, 1.0f / lam) : psi;
                const float alpha = rwu_feddes_f(head, h1, h2, h3, h4, a1);
                const double availcap = jmin(1.0, jmax(0.0, (rd - col.cum[k - 1]) / col.thick[k - 1]));
                const double a = jmin((double)alpha * rs_ * pot_trans, col.usld[k - 1] * availcap / dt);
                col.usld[k - 1] -= a * dt;
                actevapustore += a;
            }
            const float wetroots = 1.0f / (1.0f + expf(-Lf[ROOTDISTPAR][slot] * (float)(zi - rd)));
            const float alpha0 = rwu_feddes_f(0.0f, h1, h2, h3, h4, a1);
            act_sat = jmin((pot_trans - actevapustore) * (double)(wetroots * alpha0), drain / dt);
            drain -= act_sat * dt;
        }
        const double transpiration = actevapustore + act_sat;
        // actual infiltration
        double excess = 0.0;
#pragma unroll
        for (int k = MAXN; k >= 1; --k) {
            if (k > col.nu) continue;
            excess = jmax(0.0, col.usld[k - 1] - col.thick[k - 1] * te);
            col.usld[k - 1] -= excess;
            if (k > 1) col.usld[k - 2] += excess;
        }
        const double act_infilt = infiltration - excess / dt;
        const double satex = (wfs_soil - act_infilt) - infex;
        usd = 0.0;
#pragma unroll
        for (int k = 0; k < MAXN; ++k)
            if (k < col.nl) usd += col.usld[k];
        ucap = swc - sat - usd;
        // capillary flux
        double capflux_act = 0.0;
        if (col.nu > 0) {
            const double ksat = (double)col.kv_at(kvf, zi, col.nu);
            const double maxcap = jmax(0.0, jmin(jmin(jmin(ksat, actevapustore), ucap / dt), drain / dt));
            const double rd = F.L[ROOTING_DEPTH][slot];
            const float chmax = Lf[CAP_HMAX][slot];
            double capflux =
                zi > rd ? maxcap * (double)powj(1.0f - fminj((float)zi, chmax) / chmax, Lf[CAP_N][slot]) : 0.0;
#pragma unroll
            for (int k = MAXN; k >= 1; --k) {
                if (k > col.nu) continue;
                const double toadd = jmin(capflux, jmax((col.thick[k - 1] * te - col.usld[k - 1]) / dt, 0.0));
                col.usld[k - 1] += toadd * dt;
                capflux -= toadd;
                capflux_act += toadd;
            }
        }
        const double deepksat = (double)col.kv_at(kvf, col.d, col.nl);
        const double leak = jmax(0.0, jmin(F.L[MAX_LEAKAGE][slot], jmin(drain / dt, deepksat)));
        const double recharge = transfer - capflux_act - leak - act_sat - esat;
        const double aet = soilevap + transpiration + ae_river + ae_land + ic;
        // ---- write back
        Mf[CANOPY][e] = canopy;
        Mf[SNOW][e] = snow;
        Mf[SNOW_WATER][e] = snow_water;
        Mh[TSOIL][e] = tsoil;
#pragma unroll
        for (int k = 0; k < MAXN; ++k)
            if (k < col.N) F.LY[LY_USLD][k][e] = col.usld[k];
        Mf[ZI][e] = zi;
        Mf[SSF_ZI][e] = zi;
        Mf[RECHARGE][e] = recharge;
        Mf[NET_RUNOFF_RIVER][e] = runoff_river - ae_river;
        Mf[AET][e] = aet;
        Mf[LEAKAGE][e] = leak;
        Mf[SATEX][e] = satex;
        Mf[INFEX][e] = infex;
        Mf[RUNOFF_LAND][e] = runoff_land;
        Mf[AE_LAND][e] = ae_land;
        Mh[INTERCEPTION][e] = (float)ic;
        Mh[TRANSPIRATION][e] = (float)transpiration;
        Mh[SOIL_EVAP][e] = (float)soilevap;
        Mh[ACT_INFILT][e] = (float)act_infilt;
        if (F.snow) Mh[SWE][e] = swe_out;
    }
}

// ------------------------------------------------------------------ SSF wavefront -------

__device__ __forceinline__ double kw_ssf_newton_s(double q, double cterm, double celerity, double dt, double dx) {
    int count = 0;
    const double dt_dx = dt / dx;
    const double cinv = 1.0 / celerity;
    const double df = dt_dx + cinv;
    const double rdf = 1.0 / df;
    while (true) {
        const double fq = dt_dx * q + cinv * q - cterm;
        const double q_old = q;
        q -= fq * rdf;
        if (q != q) q = 0.0;
        q = jmax(q, KIN_WAVE_MIN_FLOW);
        if ((wfm::fabs_(fq) <= 1.0e-12) || (count >= 3000)) break;
        if (q == q_old) break;
        count += 1;
    }
    return q;
}

template <int MAXN>
struct SsfSplitPhys {
    WfDevFields F;
    WfDevGraph g;
    WfSweep sw;

    __device__ bool node(int64_t slot, int64_t e, int m, int s, uint32_t ep, int64_t chain, bool is_end) {
        double* const* Mf = F.Mf;
        double* const* L = F.L;
        const double dt_s = sw.dts[s];
        const double area = L[AREA][slot];
        const double d = L[SOIL_THICKNESS][slot];
        double zi_ssf = Mf[SSF_ZI][e];
        double flux = Mf[RECHARGE][e] * area;
        if (zi_ssf >= d) flux = jmax(0.0, flux);
        const double q_net = flux;
        double qin = 0.0, tr = 0.0;
        for (int32_t o = g.up_ptr[slot]; o < g.up_ptr[slot + 1]; ++o) {
            double qu;
            if (!wfw::upstream_q(g, sw, Mf[SSF_Q], o, m, s, ep, F.status, qu)) return false;
            const double fr = L[FRAC_TO_RIVER][g.up_slot[o]];
            qin += qu * (1.0 - fr);
            tr += qu * fr;
        }
        ColumnS<MAXN> col;
        col.load_static(F, slot);
        col.kv0 = F.Mh[KV0][e];
        col.f = F.Mh[FSCALE][e];
#pragma unroll
        for (int k = 0; k < MAXN; ++k) col.usld[k] = k < col.N ? F.LY[LY_USLD][k][e] : 0.0;
        const double zi_soil = Mf[ZI][e];
        col.set_thickness(zi_soil);
        const double q_prev = Mf[SSF_Q][e];
        const double sy = L[SY][slot], dx = L[FLOW_LENGTH][slot], dw = L[FLOW_WIDTH][slot];
        const double slope = L[SLOPE][slot];
        const float kh0 = F.Lf[KH_RATIO][slot] * col.kv0;
        const double q_max = (double)F.Mh[Q_MAX][e];
        double q, zi_new, exfilt, netflux;
        const bool early = (qin + q_prev == 0.0 && q_net <= 0.0);
        if (early) {
            q = 0.0;
            zi_new = d;
            exfilt = 0.0;
            netflux = 0.0;
        } else {
            auto celerity = [&](double zi) {
                float z = (float)zi;
                if (col.profile == WF_KV_EXPONENTIAL_CONSTANT && !(z < col.zexp)) z = col.zexp;
                return (double)(kh0 * expf(-col.f * z) * (float)slope) / sy;
            };
            double cel = celerity(zi_ssf);
            double cterm = (dt_s / dx) * (qin + q_net) + q_prev / cel;
            q = kw_ssf_newton_s((q_prev + qin) / 2.0, cterm, cel, dt_s, dx);
            q = jmin(q, q_max * dw);
            netflux = (qin + q_net - q) / (dw * dx);
            double dh;
            col.water_table_change(netflux, sy, dt_s, dh, exfilt);
            double zi = zi_ssf - dh;
            if (zi > d) q = jmax(q - (dw * dx) * sy * (zi - d) / dt_s, KIN_WAVE_MIN_FLOW);
            zi = jclamp(zi, 0.0, d);
            const long its = (long)wfm::ceil_(wfm::round_sigdigits(wfm::fabs_(zi - zi_ssf) / 0.1, 12));
            if (its > 1) {
                const double dts2 = dt_s / (double)its;
                double q_sum = 0.0, ex_sum = 0.0, nf_sum = 0.0, qp = q_prev, zp = zi_ssf;
                for (long i = 0; i < its; ++i) {
                    cel = celerity(zp);
                    cterm = (dts2 / dx) * qin + qp / cel + q_net * (dts2 / dx);
                    q = kw_ssf_newton_s(qp, cterm, cel, dts2, dx);
                    q = jmin(q, q_max * dw);
                    netflux = (qin + q_net - q) / (dw * dx);
                    col.water_table_change(netflux, sy, dts2, dh, exfilt);
                    zi = zp - dh;
                    if (zi > d) q = jmax(q - (dw * dx) * sy * (zi - d) / dts2, KIN_WAVE_MIN_FLOW);
                    zi = jclamp(zi, 0.0, d);
                    col.update_ustorelayerdepth(zp, zi);
                    ex_sum += exfilt;
                    nf_sum += netflux;
                    q_sum += q;
                    qp = q;
                    zp = zi;
                }
                q = q_sum / (double)its;
                exfilt = ex_sum / (double)its;
                netflux = nf_sum / (double)its;
            } else {
                col.update_ustorelayerdepth(zi_ssf, zi);
            }
            zi_new = zi;
        }
        Mf[SSF_Q][e] = q;
        Mf[SSF_ZI][e] = zi_new;
        Mf[SSF_STORAGE][e] = sy * (d - zi_new) * area;
        const bool first = (sw.first + s == 0);
        const bool last = sw.last_of_step && (s == sw.S - 1);
        // cumulative sub-step fluxes: a single sub-step needs no accumulator
        double c_tr = tr * dt_s, c_rf = flux * dt_s, c_qin = qin * dt_s, c_q = q * dt_s, c_ex = exfilt * dt_s,
               c_nf = netflux * area * dt_s;
        if (!first) {
            c_tr += Mf[SSF_TR_CUM][e];
            c_rf += Mf[RCH_FLUX_CUM][e];
            c_qin += Mf[SSF_QIN_CUM][e];
            c_q += Mf[SSF_Q_CUM][e];
            c_ex += Mf[SSF_EXF_CUM][e];
            c_nf += Mf[SSF_QNET_CUM][e];
        }
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
        const double dt = sw.dt;
        const double exf_avg = c_ex / dt;
        Mf[RCH_FLUX_AVG][e] = c_rf / dt;
        Mf[SSF_QIN_AVG][e] = c_qin / dt;
        Mf[SSF_Q_AVG][e] = c_q / dt;
        Mf[SSF_QNET_AVG][e] = c_nf / dt;
        Mf[SSF_EXF_AVG][e] = exf_avg;
        Mf[SSF_TR_AVG][e] = c_tr / dt;
        if (early) {
#pragma unroll
            for (int k = 0; k < MAXN; ++k) col.usld[k] = k < col.N ? F.LY[LY_USLD][k][e] : 0.0;
            col.set_thickness(zi_soil);
        }
        const double zi_s = early ? zi_soil : zi_new;
        double usd = 0.0;
#pragma unroll
        for (int k = 0; k < MAXN; ++k)
            if (k < col.nu) usd += col.usld[k];
        const double runoff = jmax(0.0, exf_avg + Mf[SATEX][e] + Mf[RUNOFF_LAND][e] + Mf[INFEX][e]);
        const double sat = (d - zi_s) * (col.ts - col.tr);
        Mf[SAT][e] = sat;
        Mf[USTOREDEPTH][e] = usd;
        Mf[TSWS][e] = sat + usd;
        Mf[EXFILT][e] = exf_avg;
        Mf[RUNOFF][e] = runoff;
        const double net_runoff = runoff - Mf[AE_LAND][e];
        Mf[NET_RUNOFF][e] = net_runoff;
        const double inwater = net_runoff * area;
        Mf[OL_INWATER][e] = inwater;
        Mf[OL_QLAT][e] = inwater / L[FLOW_LENGTH][slot];
        return true;
    }
};

// --------------------------------------------------------------- overland wavefront -----

struct OverlandSplitPhys {
    WfDevFields F;
    WfDevGraph g;
    WfSweep sw;

    __device__ bool node(int64_t slot, int64_t e, int m, int s, uint32_t ep, int64_t chain, bool is_end) {
        double* const* Mf = F.Mf;
        double* const* L = F.L;
        const double dt_s = sw.dts[s];
        const bool first = (sw.first + s == 0);
        const bool last = sw.last_of_step && (s == sw.S - 1);
        if (first && F.mass_balance) Mf[BO_PREV][e] = Mf[OL_STORAGE][e];
        const double sfw = L[SFW][slot];
        double tr = 0.0, qin = 0.0;
        for (int32_t o = g.up_ptr[slot]; o < g.up_ptr[slot + 1]; ++o) {
            double qu;
            if (!wfw::upstream_q(g, sw, Mf[OL_Q], o, m, s, ep, F.status, qu)) return false;
            const double fr = L[FRAC_TO_RIVER][g.up_slot[o]];
            tr += qu * fr;
            qin += qu * (1.0 - fr);
        }
        if (!(sfw > 0.0)) qin = 0.0;
        const double fl = L[FLOW_LENGTH][slot];
        double q, a;
        kinematic_wave_split(qin, Mf[OL_Q][e], Mf[OL_QLAT][e], L[OL_ALPHA][slot], dt_s, fl, q, a);
        double h = Mf[OL_H][e];
        if (sfw > 0.0) h = a / sfw;
        Mf[OL_Q][e] = q;
        Mf[OL_H][e] = h;
        Mf[OL_STORAGE][e] = fl * sfw * h;
        if (is_end) wfw::publish(g, chain, m, s, ep, q);
        double c_tr = tr * dt_s, c_q = q * dt_s, c_qin = qin * dt_s;
        if (!first) {
            c_tr += Mf[OL_TR_CUM][e];
            c_q += Mf[OL_Q_CUM][e];
            c_qin += Mf[OL_QIN_CUM][e];
        }
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

struct RiverSplitPhys {
    WfDevFields F;
    WfDevGraph g;
    WfSweep sw;

    __device__ bool node(int64_t slot, int64_t e, int m, int s, uint32_t ep, int64_t chain, bool is_end) {
        double* const* RM = F.RM;
        double* const* R = F.R;
        const int M = F.M;
        const double dt_s = sw.dts[s];
        const bool first = (sw.first + s == 0);
        const bool last = sw.last_of_step && (s == sw.S - 1);
        const double len = R[R_LENGTH][slot];
        double qlat;
        if (first) {
            if (F.mass_balance) RM[BR_PREV][e] = RM[RV_STORAGE][e];
            const int64_t le = F.river_land_slot[slot] * M + m;
            const double inw = F.Mf[SSF_TR_AVG][le] + F.Mf[OL_TR_AVG][le] + F.Mf[NET_RUNOFF_RIVER][le] * R[R_AREA][slot];
            RM[RV_INWATER][e] = inw;
            qlat = inw / len;
            RM[RV_QLAT][e] = qlat;
        } else {
            qlat = RM[RV_QLAT][e];
        }
        double qin = 0.0;
        for (int32_t o = g.up_ptr[slot]; o < g.up_ptr[slot + 1]; ++o) {
            double qu;
            if (!wfw::upstream_q(g, sw, RM[RV_Q], o, m, s, ep, F.status, qu)) return false;
            qin += qu;
        }
        const double ext = R[R_EXT_INFLOW][slot];
        double inflow, absd = 0.0;
        if (ext < 0.0) {
            absd = jmin(-ext, (RM[RV_STORAGE][e] / dt_s) * 0.80);
            inflow = -absd / len;
        } else {
            inflow = ext / len;
        }
        double q, a;
        kinematic_wave_split(qin, RM[RV_Q][e], qlat + inflow, R[R_ALPHA][slot], dt_s, len, q, a);
        RM[RV_Q][e] = q;
        RM[RV_H][e] = a / R[R_WIDTH][slot];
        RM[RV_STORAGE][e] = len * a;
        if (is_end) wfw::publish(g, chain, m, s, ep, q);
        double c_q = q * dt_s, c_qin = qin * dt_s, c_ab = absd * dt_s;
        if (!first) {
            c_q += RM[RV_Q_CUM][e];
            c_qin += RM[RV_QIN_CUM][e];
            c_ab += RM[RV_ABS_CUM][e];
        }
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

template <class Phys>
__global__ void __launch_bounds__(128) walk_split_kernel(Phys phys) {
    wfw::walk(phys.g, phys.sw, phys, phys.F.status);
}

template <class Phys>
cudaError_t launch_walk_split(const Phys& phys, const WfLaunchCfg& c) {
    const int threads = 32 * (c.walk_warps > 0 ? c.walk_warps : 4);
    int blocks = c.walk_blocks;
    if (blocks <= 0) {
        int per_sm = 0;
        cudaError_t err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, walk_split_kernel<Phys>, threads, 0);
        if (err != cudaSuccess) return err;
        blocks = c.num_sms * (per_sm > 0 ? per_sm : 1);
    }
    const int64_t items = phys.g.n_chunks * (phys.g.M > 32 ? phys.g.M / 32 : 1);
    const int64_t need = (items + threads / 32 - 1) / (threads / 32);
    if (blocks > need) blocks = (int)(need < 1 ? 1 : need);
    walk_split_kernel<Phys><<<blocks, threads, 0, c.stream>>>(phys);
    return cudaGetLastError();
}

int grid_for(int64_t n, int block, int num_sms) {
    int64_t b = (n + block - 1) / block;
    int64_t cap = (int64_t)num_sms * 16;
    if (b > cap) b = cap;
    return (int)(b < 1 ? 1 : b);
}

}  // namespace

cudaError_t wf_split_vertical(const WfDevFields& F, const WfLaunchCfg& c) {
    const int block = c.vertical_block > 0 ? c.vertical_block : 256;
    const int grid = grid_for(F.land_slots * F.M, block, c.num_sms);
    if (F.N <= 4)
        vertical_split_kernel<4><<<grid, block, 0, c.stream>>>(F);
    else
        vertical_split_kernel<WF_MAX_LAYERS><<<grid, block, 0, c.stream>>>(F);
    return cudaGetLastError();
}

cudaError_t wf_split_ssf(const WfDevFields& F, const WfDevGraph& g, const WfSweep& sw, const WfLaunchCfg& c) {
    if (F.N <= 4) return launch_walk_split(SsfSplitPhys<4>{F, g, sw}, c);
    return launch_walk_split(SsfSplitPhys<WF_MAX_LAYERS>{F, g, sw}, c);
}

cudaError_t wf_split_overland(const WfDevFields& F, const WfDevGraph& g, const WfSweep& sw, const WfLaunchCfg& c) {
    return launch_walk_split(OverlandSplitPhys{F, g, sw}, c);
}

cudaError_t wf_split_river(const WfDevFields& F, const WfDevGraph& g, const WfSweep& sw, const WfLaunchCfg& c) {
    return launch_walk_split(RiverSplitPhys{F, g, sw}, c);
}

cudaError_t wf_split_balance(const WfDevFields& F, const WfLaunchCfg& c) { return wf_fp64_balance(F, c); }
