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
#include "wf_wave.cuh"

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
//
// GB300 issues FP64 instructions (arithmetic, compares and FP32<->FP64 conversions alike) at
// about 1/70 of its FP32 FMA rate, so this kernel keeps FP64 instructions to the few that the
// water balance needs:
//   * every store (canopy, snow, liquid snow water, unsaturated layers) is its FP64 content at
//     the start of the step plus the exact sum of the step's FP32 increments, accumulated with
//     error-free transformations (TwoSum/TwoProd) in an FP32 pair and added once at the end;
//   * every partition of a flux that crosses the cell boundary (throughfall/interception/
//     stemflow, rain/snow, river/land/soil runoff, infiltration/infiltration excess/saturation
//     excess) is an FP64 residual, so the parts always sum to the whole;
//   * the outputs that enter the balance are FP64 sums of the same FP32 values the stores saw.
// Rates, limiters, layer geometry and all transcendental functions are FP32.

// FP64 reciprocal from an FP32 seed and two Newton steps (about 4 FP64 FMAs instead of a
// division); relative error near 1 ulp for normal inputs, inf/0/NaN handled by the seed check.
__device__ __forceinline__ double wfm_rcp(double x) {
    const float xf = (float)x;
    double r = (double)(1.0f / xf);
    if (!(fabsf(xf) < 3.0e38f && xf != 0.0f)) return 1.0 / x;
    r = r * fma(-x, r, 2.0);
    r = r * fma(-x, r, 2.0);
    return r;
}

// FP64 store updated by FP32 increments without rounding loss.
struct Store {
    double base;
    float bf;      // base rounded to FP32 (for FP32 decisions)
    float hi, lo;  // increments of this step: exactly hi + lo
    bool mod;      // content differs from what was loaded
    __device__ __forceinline__ void init(double b) {
        base = b;
        bf = (float)b;
        hi = 0.0f;
        lo = 0.0f;
        mod = false;
    }
    __device__ __forceinline__ float val() const { return bf + hi; }
    __device__ __forceinline__ void add(float x) {  // TwoSum
        const float s = hi + x;
        const float bp = s - hi;
        const float e = (hi - (s - bp)) + (x - bp);
        hi = s;
        lo += e;
        mod = true;
    }
    __device__ __forceinline__ void add_prod(float a, float b) {  // TwoProd
        const float p = a * b;
        const float e = fmaf(a, b, -p);
        add(p);
        lo += e;
    }
    __device__ __forceinline__ void add_d(double x) {
        const float xh = (float)x;
        add(xh);
        lo += (float)(x - (double)xh);
    }
    __device__ __forceinline__ bool changed() const { return mod; }
    __device__ __forceinline__ double value() const { return base + ((double)hi + (double)lo); }
    __device__ __forceinline__ void zero() {
        base = 0.0;
        bf = 0.0f;
        hi = 0.0f;
        lo = 0.0f;
        mod = true;
    }
    __device__ __forceinline__ void set(double v) {
        init(v);
        mod = true;
    }
    __device__ __forceinline__ double take_all() {  // empties the store, returns its content
        const double v = value();
        zero();
        return v;
    }
};

// Layer geometry at water-table depth zi (utils.jl set_layerthickness): which layers are
// unsaturated is decided in FP64 against the static cumulative depths, thicknesses are FP32.
template <int MAXN>
struct ColG {
    int N, nl, nu;
    float act[MAXN], cum[MAXN + 1], thick[MAXN];
    double thick_last;  // FP64 thickness of the deepest unsaturated layer (0 when none)
    __device__ __forceinline__ void set(const WfDevFields& F, int64_t slot, double zi) {
        N = F.N;
        nl = F.nlayers[slot];
        nu = N;
        cum[0] = 0.0f;
        thick_last = 0.0;
        double c0 = 0.0;
#pragma unroll
        for (int k = 0; k < MAXN; ++k) {
            float t = __int_as_float(0x7fc00000);
            if (k < N) {
                act[k] = F.LYf[LY_ACT_THICK][k][slot];
                cum[k + 1] = F.LYf[LY_CUM][k][slot];
                const double c1 = F.LY[LY_CUM][k][slot];
                if (zi > c1) {
                    t = act[k];
                    thick_last = F.LY[LY_ACT_THICK][k][slot];
                } else {
                    const double r = zi - c0;
                    if (r > 0.0) {
                        t = (float)r;
                        thick_last = r;
                    }
                }
                c0 = c1;
            } else {
                act[k] = t;
                cum[k + 1] = t;
            }
            thick[k] = t;
            if (k < N && t != t) nu -= 1;
        }
    }
};

template <int MAXN>
__global__ void __launch_bounds__(256) vertical_split_kernel(WfDevFields F) {
    const int M = F.M;
    const int64_t E = F.land_slots * M;
    const double dt = F.dt, inv_dt = F.inv_dt;
    const float dtf = (float)F.dt, inv_dtf = (float)F.inv_dt;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t slot = e / M;
        if (F.land_node_of_slot[slot] < 0) continue;
        const int m = (int)(e - slot * M);
        double* const* Mf = F.Mf;
        float* const* Mh = F.Mh;
        float* const* Lf = F.Lf;
        const float Pf = Mh[PRECIP][e], PETf = Mh[POTEVAP][e], Tf = Mh[TEMP][e];
        const double Pd = (double)Pf;
        const double canopy0 = Mf[CANOPY][e], snow0 = F.snow ? Mf[SNOW][e] : 0.0,
                     sw0 = F.snow ? Mf[SNOW_WATER][e] : 0.0;
        if (F.mass_balance) Mf[BL_PREV][e] = Mf[TSWS][e] + canopy0 + (snow0 + sw0);
        // ---- interception (canopy.jl:213-226 Gash, :259-271 Rutter)
        const float gapf = Lf[GAP][slot], cmaxf = Lf[CMAX][slot];
        const float potevap_f = Lf[KC][slot] * PETf * (1.0f - gapf);
        double tf_d, ic_d;
        float icf, sff;
        Store canopy;
        canopy.base = canopy0;
        canopy.hi = canopy.lo = 0.0f;
        canopy.mod = false;
        if (F.gash) {
            if (cmaxf > 0.0f) {
                const float e_r = Lf[E_R][slot];
                float fs, fi, psat;
                if (gapf < 1.0f / 1.1f) {
                    fs = 0.1f * gapf;
                    fi = 1.0f - 1.1f * gapf;
                    psat = e_r > fi ? 0.0f : -cmaxf / (e_r * dtf) * logf(1.0f - e_r / fi);
                } else {
                    fs = 1.0f - gapf;
                    fi = 0.0f;
                    psat = 0.0f;
                }
                const float ic = Pf > psat ? (fi * psat - cmaxf * inv_dtf) + e_r * (Pf - psat) + cmaxf * inv_dtf
                                           : fi * Pf;
                sff = fs * Pf;
                icf = fminf(ic, potevap_f);
                ic_d = (double)icf;
                tf_d = Pd - ic_d - (double)sff;
            } else {
                tf_d = Pd;
                icf = 0.0f;
                ic_d = 0.0;
                sff = 0.0f;
            }
        } else {
            float fs, pcf;
            if (gapf < 1.0f / 1.1f) {
                fs = 0.1f * gapf;
                pcf = (1.0f - gapf - fs) * Pf;
            } else {
                fs = 1.0f - gapf;
                pcf = 0.0f;
            }
            sff = fs * Pf;
            tf_d = Pd - (double)sff - (double)pcf;
            const double cmax_d = F.L[CMAX][slot];
            canopy.bf = (float)canopy0;
            if (canopy0 > cmax_d) {
                tf_d += (canopy0 - cmax_d) * inv_dt;
                canopy.set(cmax_d);
            }
            canopy.add_prod(pcf, dtf);
            if (potevap_f * dtf >= canopy.val() && potevap_f > 0.0f) {
                ic_d = canopy.take_all() * inv_dt;
                icf = (float)ic_d;
            } else {
                icf = potevap_f;
                ic_d = (double)icf;
                canopy.add_prod(-icf, dtf);
            }
            if (canopy.val() > cmaxf) {
                const double c = canopy.value();
                if (c > cmax_d) {
                    tf_d += (c - cmax_d) * inv_dt;
                    canopy.set(cmax_d);
                }
            }
        }
        // ---- snow (snow.jl:238-293, snow_process.jl:26-116)
        double wfs_d;
        float swe_out = 0.0f;
        Store snow, sw;
        if (F.snow) {
            snow.init(snow0);
            sw.init(sw0);
            const double eff_d = tf_d + (double)sff;
            const float tti = Lf[TTI][slot], tt = Lf[TT][slot];
            const float rainfrac = tti == 0.0f ? (Tf > tt ? 1.0f : 0.0f)
                                               : fminf(fmaxf((Tf - (tt - tti / 2.0f)) / tti, 0.0f), 1.0f);
            const double lp_d = (double)rainfrac * eff_d;
            const double sp_d = eff_d - lp_d;
            const float ttm = Lf[TTM][slot], ddf = Lf[DDF][slot];
            if (Tf > ttm) {
                const float melt = ddf * (Tf - ttm);
                if (melt * dtf >= snow.val()) {
                    if (snow.val() > 0.0f) sw.add_d(snow.take_all());
                } else {
                    snow.add_prod(-melt, dtf);
                    sw.add_prod(melt, dtf);
                }
            } else {
                const float refr = ddf * 0.05f * (ttm - Tf) * dtf;
                if (refr >= sw.val()) {
                    if (sw.val() > 0.0f) snow.add_d(sw.take_all());
                } else {
                    snow.add(refr);
                    sw.add(-refr);
                }
            }
            snow.add_d(sp_d * dt);
            sw.add_d(lp_d * dt);
            const float whc = Lf[WHC][slot];
            double srunoff_d = 0.0;
            if (sw.val() > snow.val() * whc) {
                const double maxsw = snow.value() * (double)whc;
                const double s = sw.value();
                if (s > maxsw) {
                    srunoff_d = (s - maxsw) * inv_dt;
                    sw.set(maxsw);
                }
            }
            swe_out = sw.val() + snow.val();
            wfs_d = srunoff_d;
        } else {
            wfs_d = tf_d + (double)sff;
        }
        // ---- open water (runoff.jl open-water runoff and evaporation)
        const double rfrac = F.L[RIVER_FRACTION][slot], wfrac = F.L[WATER_FRACTION][slot];
        const float rfrac_f = Lf[RIVER_FRACTION][slot], wfrac_f = Lf[WATER_FRACTION][slot];
        const float wd_land = (float)Mf[OL_H][e];
        const int64_t rs = F.land_river_slot[slot];
        const float wd_river = rs >= 0 ? (float)F.RM[RV_H][rs * M + m] : 0.0f;
        const double runoff_river_d = fmin(1.0, rfrac) * wfs_d;
        const double runoff_land_d = fmin(1.0, wfrac) * wfs_d;
        const float ae_river_f = rfrac_f * fminf(wd_river * inv_dtf, PETf);
        const float ae_land_f = wfrac_f * fminf(wd_land * inv_dtf, PETf);
        const double ae_river_d = (double)ae_river_f, ae_land_d = (double)ae_land_f;
        // ---- soil (soil.jl update! of SbmSoilModel)
        const double wfs_soil_d = fmax(wfs_d - runoff_river_d - runoff_land_d, 0.0);
        const float soil_fraction = fmaxf(gapf - wfrac_f - rfrac_f, 0.0f);
        const float pot_trans = fmaxf(0.0f, potevap_f - icf);
        const float pot_soilevap = soil_fraction * PETf;
        const double d_soil = F.L[SOIL_THICKNESS][slot];
        const double sat = Mf[SAT][e];
        const double zi = fmax(0.0, d_soil - sat * F.L[INV_TE][slot]);
        ColG<MAXN> g;
        g.set(F, slot, zi);
        const float zif = (float)zi, df = Lf[SOIL_THICKNESS][slot];
        const float ts = Lf[THETA_S][slot], tr = Lf[THETA_R][slot], tfc = Lf[THETA_FC][slot];
        const float te = ts - tr;
        const float kv0 = Mh[KV0][e], fsc = Mh[FSCALE][e], zexp = Lf[Z_EXP][slot];
        const bool kv_const = F.kv_profile == WF_KV_EXPONENTIAL_CONSTANT;
        // Kv at depth z of layer n (1-based); the layer's factor is selected without dynamic
        // indexing so that the per-layer arrays stay in registers
#define WF_KV_AT(z_, n_)                                           \
    ([&]() {                                                       \
        float zz_ = (z_);                                          \
        if (kv_const && !(zz_ < zexp)) zz_ = zexp;                 \
        float kf_ = 0.0f;                                          \
        _Pragma("unroll") for (int j_ = 0; j_ < MAXN; ++j_) if (j_ == (n_) - 1) kf_ = kvf[j_]; \
        return kf_ * kv0 * expf(-fsc * zz_);                       \
    }())
        Store us[MAXN];
        float kvf[MAXN], cexp[MAXN], rfr[MAXN];
        float usd = 0.0f;
#pragma unroll
        for (int k = 0; k < MAXN; ++k) {
            if (k < g.N) {
                us[k].init(F.LY[LY_USLD][k][e]);
                kvf[k] = F.LYf[LY_KVFRAC][k][slot];
                cexp[k] = F.LYf[LY_C][k][slot];
                rfr[k] = F.LYf[LY_ROOTFRAC][k][slot];
            } else {
                us[k].zero();
                kvf[k] = cexp[k] = rfr[k] = 0.0f;
            }
            if (k < g.nl) usd += us[k].val();
        }
        float drain = (df - zif) * fmaxf(ts - tfc, 0.02f);
        float ucap = Lf[SWC][slot] - (float)sat - usd;
        float tsoil = Mh[TSOIL][e];
        if (F.snow) tsoil = tsoil + Lf[W_SOIL][slot] * (Tf - tsoil);
        float fred = 1.0f;
        if (F.snow && F.infilt_reduction) {
            const float cf = Lf[CF_SOIL][slot];
            fred = 1.0f / (1.0f / (1.0f - cf) + expf(-8.0f * (tsoil - 273.15f))) + cf;
        }
        // infiltration (soil_process.jl infiltration): FP64 partition of the water reaching the soil
        const double soilinf_d = wfs_soil_d * (1.0 - F.L[COMPACT_FRAC][slot]);
        const double pathinf_d = wfs_soil_d - soilinf_d;
        const float cap_soil = kv0 * kvf[0] * fred, cap_comp = Lf[CAP_COMP][slot] * fred;
        const float soilinf_f = (float)soilinf_d, pathinf_f = (float)pathinf_d;
        const double mis_d = cap_soil < soilinf_f ? (double)cap_soil : soilinf_d;
        const double mip_d = cap_comp < pathinf_f ? (double)cap_comp : pathinf_d;
        const double infex_d = (soilinf_d - mis_d) + (pathinf_d - mip_d);
        const float capmax = fmaxf(0.0f, ucap * inv_dtf);
        const float infil_f = fminf(__double2float_rz(mis_d + mip_d), capmax);
        // unsaturated zone flow (soil_process.jl:51-92): FP32 rates, exact transfers
        double transfer_d = 0.0;
        if (g.nu > 0) {
            float z = 0.0f, flow_f = infil_f;
            double flow_amt = 0.0;
            bool amt = false;
#pragma unroll
            for (int k = 0; k < MAXN; ++k) {
                if (k >= g.nu) continue;
                z += g.thick[k];
                const float l_sat = g.thick[k] * te;
                const float kv_z = WF_KV_AT(z, k + 1);
                if (amt) us[k].add_d(flow_amt);
                else us[k].add_prod(flow_f, dtf);
                const float u = us[k].val();
                if (u <= 0.0f) {
                    us[k].zero();
                    flow_f = 0.0f;
                    amt = false;
                    continue;
                }
                bool drained;
                const float rate = unsat_rate(u, kv_z, l_sat, cexp[k], dtf, drained);
                if (drained || u - rate * dtf < 0.0f) {
                    flow_amt = us[k].take_all();
                    amt = true;
                } else {
                    us[k].add_prod(-rate, dtf);
                    flow_f = rate;
                    amt = false;
                }
            }
            transfer_d = amt ? flow_amt * inv_dt : (double)flow_f;
        }
        // soil evaporation (soil.jl soil_evaporation!)
        double se_d;
        float se_f, esat_f = 0.0f;
        {
            float se = 0.0f;
            const float u0 = us[0].val();
            if (g.nu == 1) se = pot_soilevap * fminf(1.0f, u0 / (zif * te));
            else if (g.nu > 1) se = pot_soilevap * fminf(1.0f, u0 / (g.thick[0] * te));
            if (se > 0.0f && se * dtf >= u0) {
                se_d = us[0].take_all() * inv_dt;
                se_f = (float)se_d;
            } else {
                se_f = se;
                se_d = (double)se;
                us[0].add_prod(-se, dtf);
            }
            const float pot = pot_soilevap - se_f;
            if (g.nu <= 1) {
                const float a0 = g.act[0];
                esat_f = fminf(pot * fminf(1.0f, (a0 - zif) / a0), (a0 - zif) * fmaxf(ts - tfc, 0.02f) * inv_dtf);
            }
            drain -= esat_f * dtf;
        }
        // transpiration (soil.jl transpiration!): FP32 heads, Feddes reduction and root water uptake
        double actevap_d = 0.0;
        float actevap_f = 0.0f, act_sat_f;
        {
            const float rd = Lf[ROOTING_DEPTH][slot];
            const float h1 = Lf[H1][slot], h2 = Lf[H2][slot], h4 = Lf[H4][slot], a1 = Lf[ALPHA_H1][slot];
            const float psi = Lf[PSI_B][slot];
            const float tpd = pot_trans / MM_PER_DAY_F;
            const float h3l = Lf[H3_LOW][slot], h3h = Lf[H3_HIGH][slot];
            const float h3 = tpd <= 1.0f ? h3l : (tpd < 5.0f ? h3l + (h3h - h3l) * (tpd - 1.0f) / 4.0f : h3h);
            float sum_rf = 0.0f, rf_low = 0.0f;
#pragma unroll
            for (int k = 1; k <= MAXN; ++k) {
                if (k <= g.nu) {
                    float r = rfr[k - 1];
                    if (k == g.nu && zif < rd) r = r * (g.thick[k - 1] / fminf(g.act[k - 1], rd - g.cum[k - 1]));
                    sum_rf += r;
                    rf_low = r;
                }
            }
#pragma unroll
            for (int k = 1; k <= MAXN; ++k) {
                if (k > g.nu) continue;
                const float r = k < g.nu ? rfr[k - 1] : rf_low;
                const float rs_ = rd > 0.0f ? fmaxf(1.0f / sum_rf, 1.0f) * r : 0.0f;
                const float uk = us[k - 1].val();
                const float vwc = fmaxf(uk / g.thick[k - 1], 1e-7f);
                const float lam = 2.0f / (cexp[k - 1] - 3.0f);
                const float head = lam > 0.0f ? psi / powj(vwc / te, 1.0f / lam) : psi;
                const float alpha = rwu_feddes_f(head, h1, h2, h3, h4, a1);
                const float availcap = fminf(1.0f, fmaxf(0.0f, (rd - g.cum[k - 1]) / g.thick[k - 1]));
                const float want = alpha * rs_ * pot_trans;
                const float avail = uk * availcap * inv_dtf;
                if (want > 0.0f && want >= avail && availcap >= 1.0f) {
                    const double a = us[k - 1].take_all() * inv_dt;
                    actevap_d += a;
                    actevap_f += (float)a;
                } else {
                    const float a = fminf(want, avail);
                    us[k - 1].add_prod(-a, dtf);
                    actevap_d += (double)a;
                    actevap_f += a;
                }
            }
            const float wetroots = 1.0f / (1.0f + expf(-Lf[ROOTDISTPAR][slot] * (zif - rd)));
            const float alpha0 = rwu_feddes_f(0.0f, h1, h2, h3, h4, a1);
            act_sat_f = fminf((pot_trans - actevap_f) * (wetroots * alpha0), drain * inv_dtf);
            drain -= act_sat_f * dtf;
        }
        // actual infiltration: water above the capacity of a layer moves up, the top layer's
        // excess leaves the soil (soil.jl)
        float excess = 0.0f;
#pragma unroll
        for (int k = MAXN; k >= 1; --k) {
            if (k > g.nu) continue;
            excess = fmaxf(0.0f, us[k - 1].val() - g.thick[k - 1] * te);
            us[k - 1].add(-excess);
            if (k > 1) us[k - 2].add(excess);
        }
        const double act_infilt_d = (double)infil_f - (double)excess * inv_dt;
        const double satex_d = (wfs_soil_d - act_infilt_d) - infex_d;
        usd = 0.0f;
#pragma unroll
        for (int k = 0; k < MAXN; ++k)
            if (k < g.nl) usd += us[k].val();
        ucap = Lf[SWC][slot] - (float)sat - usd;
        // capillary rise (soil.jl capillary_flux!)
        Store capacc;
        capacc.zero();
        if (g.nu > 0) {
            const float ksat = WF_KV_AT(zif, g.nu);
            const float maxcap = fmaxf(0.0f, fminf(fminf(fminf(ksat, actevap_f), ucap * inv_dtf), drain * inv_dtf));
            const float rd = Lf[ROOTING_DEPTH][slot];
            const float chmax = Lf[CAP_HMAX][slot];
            float capflux = zif > rd ? maxcap * powj(1.0f - fminf(zif, chmax) / chmax, Lf[CAP_N][slot]) : 0.0f;
#pragma unroll
            for (int k = MAXN; k >= 1; --k) {
                if (k > g.nu) continue;
                const float toadd =
                    fminf(capflux, fmaxf((g.thick[k - 1] * te - us[k - 1].val()) * inv_dtf, 0.0f));
                us[k - 1].add_prod(toadd, dtf);
                capflux -= toadd;
                capacc.add(toadd);
            }
        }
        const double capflux_d = (double)capacc.hi + (double)capacc.lo;
        const float deepksat = WF_KV_AT(df, g.nl);
        const float leak_f = fmaxf(0.0f, fminf(Lf[MAX_LEAKAGE][slot], fminf(drain * inv_dtf, deepksat)));
        const double leak_d = (double)leak_f;
        const double recharge = transfer_d - capflux_d - leak_d - (double)act_sat_f - (double)esat_f;
        const double soilevap_d = se_d + (double)esat_f;
        const double transpiration_d = actevap_d + (double)act_sat_f;
        const double aet = soilevap_d + transpiration_d + ae_river_d + ae_land_d + ic_d;
        // ---- write back
        if (!F.gash) Mf[CANOPY][e] = canopy.value();
        if (F.snow) {
            Mf[SNOW][e] = snow.value();
            Mf[SNOW_WATER][e] = sw.value();
            Mh[SWE][e] = swe_out;
        }
        Mh[TSOIL][e] = tsoil;
#pragma unroll
        for (int k = 0; k < MAXN; ++k)
            if (k < g.N && us[k].changed()) F.LY[LY_USLD][k][e] = us[k].value();
        Mf[ZI][e] = zi;
        Mf[SSF_ZI][e] = zi;
        Mf[RECHARGE][e] = recharge;
        Mf[NET_RUNOFF_RIVER][e] = runoff_river_d - ae_river_d;
        Mf[AET][e] = aet;
        Mf[LEAKAGE][e] = leak_d;
        Mf[SATEX][e] = satex_d;
        Mf[INFEX][e] = infex_d;
        Mf[RUNOFF_LAND][e] = runoff_land_d;
        Mf[AE_LAND][e] = ae_land_d;
        Mh[INTERCEPTION][e] = icf;
        Mh[TRANSPIRATION][e] = actevap_f + act_sat_f;
        Mh[SOIL_EVAP][e] = se_f + esat_f;
        Mh[ACT_INFILT][e] = infil_f - excess * inv_dtf;
        // storages at the start of the routing (overland and river balances)
        if (F.mass_balance) {
            Mf[BO_PREV][e] = Mf[OL_STORAGE][e];
            if (rs >= 0) F.RM[BR_PREV][rs * M + m] = F.RM[RV_STORAGE][rs * M + m];
        }
        // terms of the subsurface solve that do not depend on the upstream discharge
        if (F.ssf_single) {
            double flux = recharge * F.L[AREA][slot];  // recharge flux of the subsurface model
            if (zi >= d_soil) flux = fmax(0.0, flux);
            Mf[SSF_QNET][e] = flux;
            float z = zif;
            if (kv_const && !(z < zexp)) z = zexp;
            const float cel = Lf[KH_RATIO][slot] * kv0 * expf(-fsc * z) * Lf[SLOPE][slot] / Lf[SY][slot];
            const float cinv = 1.0f / cel;
            Mf[SSF_T2][e] = Mf[SSF_Q][e] * (double)cinv;
            Mf[SSF_RDF][e] = (double)(1.0f / (Lf[SSF_DTDX][slot] + cinv));
            // deepest unsaturated layer: what a rising water table fills first. The rise it
            // allows, dt * rate / (theta_e - usld / thickness), moves water between the layer and
            // the saturated store, so it is FP64 (with the layer's FP64 thickness and content).
            double rth = 0.0, rcap = 0.0, rrho = 0.0;
            if (g.nu > 0) {
                const double dts = F.dt_ssf;
                const double te_d = F.L[THETA_S][slot] - F.L[THETA_R][slot];
                double uk = 0.0;
#pragma unroll
                for (int k = 0; k < MAXN; ++k)
                    if (k + 1 == g.nu) uk = us[k].changed() ? us[k].value() : us[k].base;
                rth = g.thick_last;
                rcap = fmax(rth * te_d - uk, 0.0) * F.inv_dt_ssf;
                rrho = dts * rth * wfm_rcp(te_d * rth - uk);
            }
            Mf[SSF_RTH][e] = rth;
            Mf[SSF_RCAP][e] = rcap;
            Mf[SSF_RRHO][e] = rrho;
        }
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

// ====================================================================== slim wavefronts ====
//
// The sweeps below keep only the discharge solve on the critical path (wf_wave.cuh); the
// per-cell kernels before (vertical epilogue) and after (post kernels) each sweep do the rest.

// Root of dt_dx u^5 + alpha u^3 = cterm for the kinematic wave in u = Q^0.2 (the reference's
// Newton-Raphson on Q, surface_process.jl:24-70, written for u): Newton iterations in FP32
// from the upper bound min((cterm/alpha)^(1/3), (cterm/dt_dx)^(1/5)) (or the previous u when it
// lies below that bound) until |du| <= 1e-6 u, then one FP64 Newton correction of the FP32
// root, which leaves |f(u)| at the FP64 rounding level of cterm. Results below the reference's
// floor (Q = 1e-30, u = QROOT) are raised to it, as the reference does.
__device__ __forceinline__ void kw_solve_u(double qin, double q_prev, double qlat, double dt_s, double alpha,
                                           double dt_dx, double u_prev, double& u_out, double& q_out) {
    if (qin + q_prev + qlat == 0.0) {
        u_out = 0.0;
        q_out = 0.0;
        return;
    }
    const double cterm = dt_dx * qin + (alpha * (u_prev * u_prev * u_prev) + dt_s * qlat);
    const double QR = KIN_WAVE_MIN_FLOW_QROOT;
    const double floor_c = alpha * (QR * QR * QR) + dt_dx * KIN_WAVE_MIN_FLOW;
    double u;
    if (!(cterm > floor_c)) {
        u = QR;
    } else {
        const float a = (float)dt_dx, b = (float)alpha, c = (float)cterm;
        const float ub = fminf(cbrtf(c / b), powf(c / a, 0.2f));
        const float up = (float)u_prev;
        float v = (up > 0.0f && up < ub) ? up : ub;
        const float a5 = 5.0f * a, b3 = 3.0f * b;
        float dg = 1.0f;
#pragma unroll 1
        for (int it = 0; it < 12; ++it) {
            const float v2 = v * v;
            const float g = v2 * v * fmaf(a, v2, b) - c;
            dg = v2 * fmaf(a5, v2, b3);
            const float dv = __fdividef(g, dg);
            v = fminf(v - dv, ub);
            if (!(fabsf(dv) > 1e-6f * v)) break;
        }
        const float v2 = v * v;
        dg = v2 * fmaf(a5, v2, b3);
        u = (double)v;
        const double u2 = u * u;
        const double f = u2 * u * fma(dt_dx, u2, alpha) - cterm;
        u = fma(-f, (double)(1.0f / dg), u);
        if (!(u > QR)) u = QR;
    }
    const double u2 = u * u;
    u_out = u;
    q_out = u2 * u2 * u;
}

// q^0.2 for a discharge set from outside the step (BMI set_value, restart).
__device__ __forceinline__ double u_of_q(double q) {
    if (!(q > 0.0)) return 0.0;
    const float u0 = powf((float)q, 0.2f);
    double u = (double)u0;
    const double u2 = u * u;
    return u - (u2 * u2 * u - q) * (double)(1.0f / (5.0f * u0 * u0 * u0 * u0));
}

// Subsurface node when the fast path cannot decide: the full column computation of the fused
// form (water-table change over every unsaturated layer, the reference's sub-iterations when
// the water table moves by more than 0.1 per step, subsurface_process.jl:100-196), which also
// writes the updated unsaturated layers and water table.
template <int MAXN>
__device__ __noinline__ void ssf_full_split(const WfDevFields& F, int64_t slot, int64_t e, double qin, double q_net, double dt_s,
                               double& q_out, double& zi_out, double& exf_out, double& nf_out) {
    double* const* Mf = F.Mf;
    double* const* L = F.L;
    const double d = L[SOIL_THICKNESS][slot];
    const double zi_ssf = Mf[SSF_ZI][e];
    ColumnS<MAXN> col;
    col.load_static(F, slot);
    col.kv0 = F.Mh[KV0][e];
    col.f = F.Mh[FSCALE][e];
#pragma unroll
    for (int k = 0; k < MAXN; ++k) col.usld[k] = k < col.N ? F.LY[LY_USLD][k][e] : 0.0;
    col.set_thickness(Mf[ZI][e]);
    const double q_prev = Mf[SSF_Q][e];
    const double sy = L[SY][slot], dx = L[FLOW_LENGTH][slot], dw = L[FLOW_WIDTH][slot];
    const double slope = L[SLOPE][slot];
    const float kh0 = F.Lf[KH_RATIO][slot] * col.kv0;
    const double q_max = (double)F.Mh[Q_MAX][e];
    auto celerity = [&](double zi) {
        float z = (float)zi;
        if (col.profile == WF_KV_EXPONENTIAL_CONSTANT && !(z < col.zexp)) z = col.zexp;
        return (double)(kh0 * expf(-col.f * z) * (float)slope) / sy;
    };
    double cel = celerity(zi_ssf);
    double cterm = (dt_s / dx) * (qin + q_net) + q_prev / cel;
    double q = kw_ssf_newton_s((q_prev + qin) / 2.0, cterm, cel, dt_s, dx);
    q = jmin(q, q_max * dw);
    double netflux = (qin + q_net - q) / (dw * dx);
    double dh, exfilt;
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
#pragma unroll
    for (int k = 0; k < MAXN; ++k)
        if (k < col.N) F.LY[LY_USLD][k][e] = col.usld[k];
    Mf[ZI][e] = zi;
    q_out = q;
    zi_out = zi;
    exf_out = exfilt;
    nf_out = netflux;
}

// Lateral subsurface flow, one sub-step per model step (subsurface_process.jl:100-196 per
// node). The solve of the linear kinematic wave is q = cterm / (dt/dx + 1/c); the water-table
// change is decided from the deepest unsaturated layer prepared by the vertical kernel, and
// anything else (several layers filled, a water table moving by more than 0.1, non-finite
// values) goes through ssf_full_split.
template <int MAXN>
struct SsfWave {
    WfDevFields F;
    WfDevGraph g;
    WfSweep sw;
    struct In {
        double q_prev, q_net, t2, rdf, zi, d, dtdx, idwdx, dtsy, k2, qmaxdw, rth, rcap, rrho;
        wfv::UpList up;
    };
    __device__ __forceinline__ void load(int64_t slot, int64_t e, int m, In& x) const {
        double* const* Mf = F.Mf;
        double* const* L = F.L;
        x.q_prev = Mf[SSF_Q][e];
        x.q_net = Mf[SSF_QNET][e];
        x.t2 = Mf[SSF_T2][e];
        x.rdf = Mf[SSF_RDF][e];
        x.zi = Mf[SSF_ZI][e];
        x.rth = Mf[SSF_RTH][e];
        x.rcap = Mf[SSF_RCAP][e];
        x.rrho = Mf[SSF_RRHO][e];
        x.d = L[SOIL_THICKNESS][slot];
        x.dtdx = L[SSF_DTDX][slot];
        x.idwdx = L[SSF_IDWDX][slot];
        x.dtsy = L[SSF_DTSY][slot];
        x.k2 = L[SSF_K2][slot];
        x.qmaxdw = (double)F.Mh[Q_MAX][e] * L[FLOW_WIDTH][slot];
        wfv::load_up(g, slot, m, x.up);
    }
    __device__ __forceinline__ bool node(const In& x, int64_t slot, int64_t e, int m, int64_t chain, bool is_end,
                                         double* qh) {
        double qin;
        if (!wfv::gather<true>(g, sw, x.up, m, 0, qh[0], F.status, qin)) return false;
        double q, zi_new, exf, nf;
        double flag;
        if (qin + x.q_prev == 0.0 && x.q_net <= 0.0) {
            q = 0.0;
            zi_new = x.d;
            exf = 0.0;
            nf = 0.0;
            flag = 1.0;
        } else {
            const double cterm = x.dtdx * (qin + x.q_net) + x.t2;
            q = cterm * x.rdf;
            if (q != q) q = 0.0;
            q = jmax(q, KIN_WAVE_MIN_FLOW);
            q = jmin(q, x.qmaxdw);
            nf = (qin + x.q_net - q) * x.idwdx;
            bool full = false;
            double dh = 0.0;
            exf = 0.0;
            if (nf <= 0.0) {
                dh = nf * x.dtsy;
            } else if (!(nf > 0.0) || (x.rth != 0.0 && x.rcap <= nf)) {
                full = true;
            } else if (x.rth == 0.0) {
                exf = nf;
            } else {
                dh = nf * x.rrho;
            }
            double zi = x.zi - dh;
            if (!full) {
                if (zi > x.d) q = jmax(q - x.k2 * (zi - x.d), KIN_WAVE_MIN_FLOW);
                zi = jclamp(zi, 0.0, x.d);
                if (!(wfm::fabs_(zi - x.zi) * 10.0 <= 1.0)) full = true;
            }
            if (full) {
                ssf_full_split<MAXN>(F, slot, e, qin, x.q_net, sw.dts[0], q, zi, exf, nf);
                flag = 2.0;
            } else {
                flag = 0.0;
            }
            zi_new = zi;
        }
        double* const* Mf = F.Mf;
        qh[0] = q;
        if (is_end) wfv::publish(g, chain, m, 0, q);
        Mf[SSF_Q][e] = q;
        Mf[SSF_ZI][e] = zi_new;
        Mf[SSF_TEXF][e] = exf;
        Mf[SSF_TNF][e] = nf;
        Mf[SSF_TQIN][e] = qin;
        Mf[SSF_FLAG][e] = flag;
        return true;
    }
};

// Overland flow (surface_process.jl:24-70 per node, routing/surface_kinwave.jl sub-steps).
struct OlWave {
    WfDevFields F;
    WfDevGraph g;
    WfSweep sw;
    struct In {
        double u, q, qlat, alpha, inv_dx;
        bool sfw_pos;
        wfv::UpList up;
    };
    __device__ __forceinline__ void load(int64_t slot, int64_t e, int m, In& x) const {
        x.u = F.Mf[OL_U][e];
        x.q = F.Mf[OL_Q][e];
        x.qlat = F.Mf[OL_QLAT][e];
        x.alpha = F.L[OL_ALPHA][slot];
        x.inv_dx = F.L[INV_FLOW_LENGTH][slot];
        x.sfw_pos = F.L[SFW][slot] > 0.0;
        wfv::load_up(g, slot, m, x.up);
    }
    __device__ __forceinline__ bool node(const In& x, int64_t slot, int64_t e, int m, int64_t chain, bool is_end,
                                         double* qh) {
        const int stride = blockDim.x;
        double u = x.u, qp = x.q, qsum = 0.0;
        for (int s = 0; s < sw.S; ++s) {
            const double dt_s = sw.dts[s];
            double qin;
            if (!wfv::gather<true>(g, sw, x.up, m, s, qh[s * stride], F.status, qin)) return false;
            if (!x.sfw_pos) qin = 0.0;
            double un, qn;
            kw_solve_u(qin, qp, x.qlat, dt_s, x.alpha, dt_s * x.inv_dx, u, un, qn);
            u = un;
            qp = qn;
            qh[s * stride] = qn;
            if (is_end) wfv::publish(g, chain, m, s, qn);
            qsum = fma(qn, dt_s, qsum);
        }
        double* const* Mf = F.Mf;
        Mf[OL_U][e] = u;
        Mf[OL_Q][e] = qp;
        Mf[OL_QSUM][e] = sw.first == 0 ? qsum : Mf[OL_QSUM][e] + qsum;
        return true;
    }
};

// River flow (surface_process.jl:24-70 per node, routing/river_kinwave.jl sub-steps), with the
// abstraction of a negative external inflow limited to 80 % of the storage.
struct RvWave {
    WfDevFields F;
    WfDevGraph g;
    WfSweep sw;
    struct In {
        double u, q, qlat, qlatt, alpha, inv_len, len, ext;
        wfv::UpList up;
    };
    __device__ __forceinline__ void load(int64_t slot, int64_t e, int m, In& x) const {
        x.u = F.RM[RV_U][e];
        x.q = F.RM[RV_Q][e];
        x.qlat = F.RM[RV_QLAT][e];
        x.qlatt = F.RM[RV_QLATT][e];
        x.alpha = F.R[R_ALPHA][slot];
        x.inv_len = F.R[R_INV_LENGTH][slot];
        x.len = F.R[R_LENGTH][slot];
        x.ext = F.R[R_EXT_INFLOW][slot];
        wfv::load_up(g, slot, m, x.up);
    }
    __device__ __forceinline__ bool node(const In& x, int64_t slot, int64_t e, int m, int64_t chain, bool is_end,
                                         double* qh) {
        const int stride = blockDim.x;
        double u = x.u, qp = x.q, qsum = 0.0, asum = 0.0;
        for (int s = 0; s < sw.S; ++s) {
            const double dt_s = sw.dts[s];
            double qin;
            if (!wfv::gather<false>(g, sw, x.up, m, s, qh[s * stride], F.status, qin)) return false;
            double ql = x.qlatt, absd = 0.0;
            if (x.ext < 0.0) {
                const double storage = x.len * (x.alpha * (u * u * u));
                absd = jmin(-x.ext, (storage / dt_s) * 0.80);
                ql = x.qlat + (-absd / x.len);
            }
            double un, qn;
            kw_solve_u(qin, qp, ql, dt_s, x.alpha, dt_s * x.inv_len, u, un, qn);
            u = un;
            qp = qn;
            qh[s * stride] = qn;
            if (is_end) wfv::publish(g, chain, m, s, qn);
            qsum = fma(qn, dt_s, qsum);
            asum = fma(absd, dt_s, asum);
        }
        double* const* RM = F.RM;
        RM[RV_U][e] = u;
        RM[RV_Q][e] = qp;
        RM[RV_QSUM][e] = sw.first == 0 ? qsum : RM[RV_QSUM][e] + qsum;
        RM[RV_ABSSUM][e] = sw.first == 0 ? asum : RM[RV_ABSSUM][e] + asum;
        return true;
    }
};

template <class Phys>
__global__ void __launch_bounds__(128) wave_kernel(Phys phys) {
    wfv::walk(phys.g, phys.sw, phys, phys.F.status);
}

template <class Phys>
cudaError_t launch_wave(const Phys& phys, const WfLaunchCfg& c) {
    const int threads = 32 * (c.walk_warps > 0 ? c.walk_warps : 4);
    const size_t smem = (size_t)threads * phys.sw.S * sizeof(double);
    int blocks = c.walk_blocks;
    if (blocks <= 0) {
        int per_sm = 0;
        cudaError_t err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, wave_kernel<Phys>, threads, smem);
        if (err != cudaSuccess) return err;
        blocks = c.num_sms * (per_sm > 0 ? per_sm : 1);
    }
    const int64_t items = phys.g.n_chunks * (phys.g.M > 32 ? phys.g.M / 32 : 1);
    const int64_t need = (items + threads / 32 - 1) / (threads / 32);
    if (blocks > need) blocks = (int)(need < 1 ? 1 : need);
    wave_kernel<Phys><<<blocks, threads, smem, c.stream>>>(phys);
    return cudaGetLastError();
}

// --------------------------------------------------------------- post-sweep kernels ------

// After the subsurface sweep: unsaturated-layer adjustment to the new water table
// (soil.jl update_ustorelayerdepth!), averages of the sweep, subsurface storage, the soil
// water storage update (sbm.jl update_soil_water_storage!) and the overland lateral inflow.
// FP64 for the stores; divisions replaced by static reciprocals.
template <int MAXN>
__global__ void __launch_bounds__(256) ssf_post_kernel(WfDevFields F, WfDevGraph g) {
    const int M = F.M;
    const int N = F.N;
    const int64_t E = F.land_slots * M;
    const double r_s = F.dt_ssf * F.inv_dt;  // sub-step / step (1 when they are equal)
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t slot = e / M;
        if (F.land_node_of_slot[slot] < 0) continue;
        const int m = (int)(e - slot * M);
        double* const* Mf = F.Mf;
        double* const* L = F.L;
        const int flag = (int)Mf[SSF_FLAG][e];
        const double zi_soil = Mf[ZI][e];
        const double zi_new = Mf[SSF_ZI][e];
        double usld[MAXN], act[MAXN], cum[MAXN + 1];  // cum[k]: depth of the top of layer k
        cum[0] = 0.0;
#pragma unroll
        for (int k = 0; k < MAXN; ++k) {
            usld[k] = k < N ? F.LY[LY_USLD][k][e] : 0.0;
            act[k] = k < N ? F.LY[LY_ACT_THICK][k][slot] : 0.0;
            cum[k + 1] = k < N ? F.LY[LY_CUM][k][slot] : __longlong_as_double(0x7ff8000000000000LL);
        }
        // layer k is unsaturated iff the water table lies below its top (utils.jl set_layerthickness)
        auto nu_at = [&](double ref) {
            int c = 0;
#pragma unroll
            for (int k = 0; k < MAXN; ++k)
                if (k < N && ref > cum[k]) ++c;
            return c;
        };
        auto thick_at = [&](double ref, int k) {
            return ref > cum[k + 1] ? act[k] : (ref > cum[k] ? ref - cum[k] : __longlong_as_double(0x7ff8000000000000LL));
        };
        double zi_s = zi_new;
        if (flag == 0) {
            if (zi_new != zi_soil) {
                const int n_prev = nu_at(zi_soil), n_new = nu_at(zi_new);
                if (zi_new < zi_soil) {
#pragma unroll
                    for (int k = 1; k <= MAXN; ++k) {
                        if (k < n_new || k > n_prev) continue;
                        const double t = thick_at(zi_new, k - 1);
                        usld[k - 1] = t != t ? 0.0 : t * wfm_rcp(thick_at(zi_soil, k - 1)) * usld[k - 1];
                        F.LY[LY_USLD][k - 1][e] = usld[k - 1];
                    }
                } else {
                    const double tfc_tr = L[THETA_FC][slot] - L[THETA_R][slot];
#pragma unroll
                    for (int k = 1; k <= MAXN; ++k) {
                        if (k < n_prev || k > n_new) continue;
                        double tp = thick_at(zi_soil, k - 1);
                        tp = tp != tp ? 0.0 : tp;
                        usld[k - 1] = usld[k - 1] + (thick_at(zi_new, k - 1) - tp) * tfc_tr;
                        F.LY[LY_USLD][k - 1][e] = usld[k - 1];
                    }
                }
                Mf[ZI][e] = zi_new;
            }
        } else if (flag == 1) {
            zi_s = zi_soil;
        }
        const int nu = nu_at(zi_s);
        double tr = 0.0;
        for (int32_t o = g.up_ptr[slot]; o < g.up_ptr[slot + 1]; ++o)
            tr += Mf[SSF_Q][g.up_slot[o] * M + m] * g.up_fr[o];
        const double area = L[AREA][slot], d = L[SOIL_THICKNESS][slot];
        const double q = Mf[SSF_Q][e], qin = Mf[SSF_TQIN][e], exf = Mf[SSF_TEXF][e], nf = Mf[SSF_TNF][e];
        const double flux = Mf[SSF_QNET][e];
        Mf[SSF_STORAGE][e] = L[SY][slot] * (d - zi_new) * area;
        const double exf_avg = exf * r_s;
        Mf[RCH_FLUX_AVG][e] = flux * r_s;
        Mf[SSF_QIN_AVG][e] = qin * r_s;
        Mf[SSF_Q_AVG][e] = q * r_s;
        Mf[SSF_QNET_AVG][e] = nf * area * r_s;
        Mf[SSF_EXF_AVG][e] = exf_avg;
        Mf[SSF_TR_AVG][e] = tr * r_s;
        double usd = 0.0;
#pragma unroll
        for (int k = 0; k < MAXN; ++k)
            if (k < nu) usd += usld[k];
        const double runoff = fmax(0.0, exf_avg + Mf[SATEX][e] + Mf[RUNOFF_LAND][e] + Mf[INFEX][e]);
        const double sat = (d - zi_s) * (L[THETA_S][slot] - L[THETA_R][slot]);
        Mf[SAT][e] = sat;
        Mf[USTOREDEPTH][e] = usd;
        Mf[TSWS][e] = sat + usd;
        Mf[EXFILT][e] = exf_avg;
        Mf[RUNOFF][e] = runoff;
        const double net_runoff = runoff - Mf[AE_LAND][e];
        Mf[NET_RUNOFF][e] = net_runoff;
        const double inwater = net_runoff * area;
        Mf[OL_INWATER][e] = inwater;
        Mf[OL_QLAT][e] = inwater * L[INV_FLOW_LENGTH][slot];
    }
}

// After the overland sweep: water depth and storage, averages, and the lateral inflow of the
// river cell of each land cell (routing/river_kinwave.jl update_lateral_inflow!).
__global__ void __launch_bounds__(256) ol_post_kernel(WfDevFields F, WfDevGraph g) {
    const int M = F.M;
    const int64_t E = F.land_slots * M;
    const double inv_dt = F.inv_dt;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t slot = e / M;
        if (F.land_node_of_slot[slot] < 0) continue;
        const int m = (int)(e - slot * M);
        double* const* Mf = F.Mf;
        double* const* L = F.L;
        const double inv_sfw = L[INV_SFW][slot];
        if (inv_sfw > 0.0) {
            const double u = Mf[OL_U][e];
            const double h = L[OL_ALPHA][slot] * (u * u * u) * inv_sfw;
            Mf[OL_H][e] = h;
            Mf[OL_STORAGE][e] = L[FLOW_LENGTH][slot] * L[SFW][slot] * h;
        }
        double qin = 0.0, tr = 0.0;
        for (int32_t o = g.up_ptr[slot]; o < g.up_ptr[slot + 1]; ++o) {
            const double qs = Mf[OL_QSUM][g.up_slot[o] * M + m];
            qin += qs * g.up_w[o];
            tr += qs * g.up_fr[o];
        }
        if (!(inv_sfw > 0.0)) qin = 0.0;
        Mf[OL_Q_AVG][e] = Mf[OL_QSUM][e] * inv_dt;
        const double tr_avg = tr * inv_dt;
        Mf[OL_TR_AVG][e] = tr_avg;
        Mf[OL_QIN_AVG][e] = qin * inv_dt;
        const int64_t rs = F.land_river_slot[slot];
        if (rs >= 0) {
            const int64_t re = rs * M + m;
            const double inv_len = F.R[R_INV_LENGTH][rs];
            const double inw = Mf[SSF_TR_AVG][e] + tr_avg + Mf[NET_RUNOFF_RIVER][e] * F.R[R_AREA][rs];
            F.RM[RV_INWATER][re] = inw;
            const double qlat = inw * inv_len;
            F.RM[RV_QLAT][re] = qlat;
            const double ext = F.R[R_EXT_INFLOW][rs];
            F.RM[RV_QLATT][re] = ext < 0.0 ? qlat : qlat + ext * inv_len;
        }
    }
}

// After the river sweep: water depth, storage and averages.
__global__ void __launch_bounds__(256) rv_post_kernel(WfDevFields F, WfDevGraph g) {
    const int M = F.M;
    const int64_t E = F.river_slots * M;
    const double inv_dt = F.inv_dt;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t slot = e / M;
        if (F.river_node_of_slot[slot] < 0) continue;
        const int m = (int)(e - slot * M);
        double* const* RM = F.RM;
        double* const* R = F.R;
        const double u = RM[RV_U][e];
        const double a = R[R_ALPHA][slot] * (u * u * u);
        RM[RV_H][e] = a * R[R_INV_WIDTH][slot];
        RM[RV_STORAGE][e] = R[R_LENGTH][slot] * a;
        double qin = 0.0;
        for (int32_t o = g.up_ptr[slot]; o < g.up_ptr[slot + 1]; ++o) qin += RM[RV_QSUM][g.up_slot[o] * M + m];
        RM[RV_Q_AVG][e] = RM[RV_QSUM][e] * inv_dt;
        RM[RV_QIN_AVG][e] = qin * inv_dt;
        RM[RV_ABS_AVG][e] = RM[RV_ABSSUM][e] * inv_dt;
    }
}

// Water balance of the split form (mass_balance.jl:215-253 land, :382-399 overland,
// :470-490 subsurface, :290-313 river) and update_total_water_storage! (sbm.jl:143-182):
// the error terms are FP64 differences of the FP64 totals, the relative errors are FP32
// quotients, and every division by dt or area is a multiplication by a static reciprocal.
__device__ __forceinline__ void mb_error_s(double tin, double tout, double rate, double& err, double& rel) {
    err = tin - tout - rate;
    const float avg = (float)((tin + tout) * 0.5);
    rel = avg == 0.0f ? 0.0 : (double)((float)err / avg);
}

__global__ void __launch_bounds__(256) balance_split_kernel(WfDevFields F) {
    const int M = F.M;
    const int64_t EL = F.land_slots * M, ER = F.river_slots * M;
    const double inv_dt = F.inv_dt;
    double* const* Mf = F.Mf;
    double* const* L = F.L;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < EL + ER; e += (int64_t)gridDim.x * blockDim.x) {
        if (e >= EL) {
            if (!F.mass_balance) continue;
            const int64_t re = e - EL;
            const int64_t rs = re / M;
            if (F.river_node_of_slot[rs] < 0) continue;
            double* const* RM = F.RM;
            const double tin = RM[RV_INWATER][re] + RM[RV_QIN_AVG][re] + fmax(0.0, F.R[R_EXT_INFLOW][rs]);
            const double tout = RM[RV_Q_AVG][re] + RM[RV_ABS_AVG][re];
            double err, rel;
            mb_error_s(tin, tout, (RM[RV_STORAGE][re] - RM[BR_PREV][re]) * inv_dt, err, rel);
            RM[BR_ERR][re] = err;
            RM[BR_REL][re] = rel;
            continue;
        }
        const int64_t slot = e / M;
        if (F.land_node_of_slot[slot] < 0) continue;
        const int m = (int)(e - slot * M);
        const int64_t rs = F.land_river_slot[slot];
        const double inv_area = L[INV_AREA][slot];
        double ts = 0.0;
        if (rs >= 0) ts = F.RM[RV_H][rs * M + m] * F.R[R_WIDTH][rs] * F.R[R_LENGTH][rs] * inv_area;
        const double snow = Mf[SNOW][e], sw = Mf[SNOW_WATER][e], canopy = Mf[CANOPY][e];
        const double tsws = Mf[TSWS][e];
        ts += snow + sw + canopy + tsws + Mf[OL_H][e] * (1.0 - L[RIVER_FRACTION][slot]);
        Mf[TOTAL_STORAGE][e] = ts;
        if (!F.mass_balance) continue;
        double err, rel;
        {
            const double tin = Mf[SSF_QIN_AVG][e] * inv_area + (double)F.Mh[PRECIP][e];
            const double vout = Mf[NET_RUNOFF][e] + Mf[AET][e] + Mf[NET_RUNOFF_RIVER][e] + Mf[LEAKAGE][e];
            const double tout = Mf[SSF_Q_AVG][e] * inv_area + vout;
            const double storage = tsws + canopy + (snow + sw);
            mb_error_s(tin, tout, (storage - Mf[BL_PREV][e]) * inv_dt, err, rel);
            Mf[BL_ERR][e] = err;
            Mf[BL_REL][e] = rel;
        }
        mb_error_s(Mf[OL_INWATER][e] + Mf[OL_QIN_AVG][e], Mf[OL_Q_AVG][e], (Mf[OL_STORAGE][e] - Mf[BO_PREV][e]) * inv_dt,
                   err, rel);
        Mf[BO_ERR][e] = err;
        Mf[BO_REL][e] = rel;
        {
            const double flux = Mf[RCH_FLUX_AVG][e];
            const double fin = fmax(flux, 0.0), fout = fmax(-flux, 0.0);
            mb_error_s(Mf[SSF_QIN_AVG][e] + fin, Mf[SSF_Q_AVG][e] + fout, Mf[SSF_QNET_AVG][e], err, rel);
            Mf[BS_ERR][e] = err;
            Mf[BS_REL][e] = rel;
        }
    }
}

// u = Q^0.2 of the overland and river discharges (after a discharge was set from outside).
__global__ void __launch_bounds__(256) sync_u_kernel(WfDevFields F) {
    const int M = F.M;
    const int64_t EL = F.land_slots * M, ER = F.river_slots * M;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < EL + ER; i += (int64_t)gridDim.x * blockDim.x) {
        if (i < EL) {
            F.Mf[OL_U][i] = u_of_q(F.Mf[OL_Q][i]);
        } else {
            const int64_t e = i - EL;
            F.RM[RV_U][e] = u_of_q(F.RM[RV_Q][e]);
        }
    }
}

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

cudaError_t wf_split_balance(const WfDevFields& F, const WfLaunchCfg& c) {
    const int block = 256;
    balance_split_kernel<<<grid_for((F.land_slots + F.river_slots) * F.M, block, c.num_sms), block, 0, c.stream>>>(F);
    return cudaGetLastError();
}

cudaError_t wf_split_ssf_wave(const WfDevFields& F, const WfDevGraph& g, const WfSweep& sw, const WfLaunchCfg& c) {
    if (F.N <= 4) return launch_wave(SsfWave<4>{F, g, sw}, c);
    return launch_wave(SsfWave<WF_MAX_LAYERS>{F, g, sw}, c);
}

cudaError_t wf_split_overland_wave(const WfDevFields& F, const WfDevGraph& g, const WfSweep& sw,
                                   const WfLaunchCfg& c) {
    return launch_wave(OlWave{F, g, sw}, c);
}

cudaError_t wf_split_river_wave(const WfDevFields& F, const WfDevGraph& g, const WfSweep& sw, const WfLaunchCfg& c) {
    return launch_wave(RvWave{F, g, sw}, c);
}

cudaError_t wf_split_ssf_post(const WfDevFields& F, const WfDevGraph& g, const WfLaunchCfg& c) {
    const int block = 256;
    const int grid = grid_for(F.land_slots * F.M, block, c.num_sms);
    if (F.N <= 4)
        ssf_post_kernel<4><<<grid, block, 0, c.stream>>>(F, g);
    else
        ssf_post_kernel<WF_MAX_LAYERS><<<grid, block, 0, c.stream>>>(F, g);
    return cudaGetLastError();
}

cudaError_t wf_split_overland_post(const WfDevFields& F, const WfDevGraph& g, const WfLaunchCfg& c) {
    ol_post_kernel<<<grid_for(F.land_slots * F.M, 256, c.num_sms), 256, 0, c.stream>>>(F, g);
    return cudaGetLastError();
}

cudaError_t wf_split_river_post(const WfDevFields& F, const WfDevGraph& g, const WfLaunchCfg& c) {
    rv_post_kernel<<<grid_for(F.river_slots * F.M, 256, c.num_sms), 256, 0, c.stream>>>(F, g);
    return cudaGetLastError();
}

cudaError_t wf_split_sync_u(const WfDevFields& F, const WfLaunchCfg& c) {
    sync_u_kernel<<<grid_for((F.land_slots + F.river_slots) * F.M, 256, c.num_sms), 256, 0, c.stream>>>(F);
    return cudaGetLastError();
}
