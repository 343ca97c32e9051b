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
#include "wf_launch.cuh"
#include "wf_math.cuh"
#include "wf_walker.cuh"
#include "wf_ff.cuh"
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
    __device__ __forceinline__ void set(const WfDevFields& F, int64_t slot, double zi) {
        N = F.N;
        nl = F.nlayers[slot];
        nu = N;
        cum[0] = 0.0f;
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
                } else {
                    const double r = zi - c0;
                    if (r > 0.0) t = (float)r;
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
        // terms of the subsurface solve that do not depend on the upstream discharge: the FP64
        // recharge flux for the exact bookkeeping, FP32 inputs of the walker
        if (F.ssf_single) {
            double flux = recharge * F.L[AREA][slot];  // recharge flux of the subsurface model
            if (zi >= d_soil) flux = fmax(0.0, flux);
            Mf[SSF_QNET][e] = flux;
            Mh[SSF_QNETF][e] = (float)flux;
            Mh[SSF_ZIF][e] = zif;
            float z = zif;
            if (kv_const && !(z < zexp)) z = zexp;
            const float cel = Lf[KH_RATIO][slot] * kv0 * expf(-fsc * z) * Lf[SLOPE][slot] / Lf[SY][slot];
            const float cinv = 1.0f / cel;
            Mh[SSF_T2][e] = (float)Mf[SSF_Q][e] * cinv;
            Mh[SSF_RDF][e] = 1.0f / (Lf[SSF_DTDX][slot] + cinv);
            // deepest unsaturated layer: what a rising water table fills first
            float rth = 0.0f, rcap = 0.0f, rrho = 0.0f;
            const float dts = (float)F.dt_ssf;
#pragma unroll
            for (int k = 0; k < MAXN; ++k) {
                if (k + 1 != g.nu) continue;
                rth = g.thick[k];
                const float uk = us[k].val();
                rcap = fmaxf(rth * te - uk, 0.0f) / dts;
                rrho = dts / (te - uk / rth);
            }
            Mh[SSF_RTH][e] = rth;
            Mh[SSF_RCAP][e] = rcap;
            Mh[SSF_RRHO][e] = rrho;
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
        const double qlat = inwater / L[FLOW_LENGTH][slot];
        Mf[OL_QLAT][e] = qlat;
        const wff::ff qlf = wff::from_d(qlat);
        F.Mh[OL_QLATH][e] = qlf.hi;
        F.Mh[OL_QLATL][e] = qlf.lo;
        return true;
    }
};

// ====================================================================== slim wavefronts ====
//
// The sweeps below keep only the discharge solve on the critical path (wf_wave.cuh); the
// per-cell kernels before (vertical epilogue) and after (post kernels) each sweep do the rest.

// Root of dt_dx u^5 + alpha u^3 = cterm for the kinematic wave in u = Q^0.2 (the reference's
// Newton-Raphson on Q, surface_process.jl:24-70, written for u), in double-FP32: Newton
// iterations in FP32 from the upper bound min((cterm/alpha)^(1/3), (cterm/dt_dx)^(1/5)) (or
// from the previous u when it lies below that bound) until |du| <= 3e-7 u, then one Newton
// correction with the residual evaluated in double-FP32, which leaves |f(u)| at about 1e-13 of
// cterm. Q = u^5 is formed from the correction du as v^5 - 5 v^4 du (the dropped terms are of
// relative size (du/v)^2). Results below the reference's floor (Q = 1e-30, u = QROOT) are
// raised to it, as the reference does.
__device__ __forceinline__ void kw_solve_ff(wff::ff cterm, wff::ff dt_dx, float alpha, float u_prev, wff::ff& u_out,
                                            wff::ff& q_out) {
    const float QR = (float)KIN_WAVE_MIN_FLOW_QROOT;
    const float floor_c = alpha * (QR * QR * QR);
    if (!(cterm.hi > floor_c)) {
        u_out = {QR, 0.0f};
        q_out = {(float)KIN_WAVE_MIN_FLOW, 0.0f};
        return;
    }
    const float a = dt_dx.hi, b = alpha, c = cterm.hi;
    const float ub = 1.00001f * fminf(__powf(__fdividef(c, b), 1.0f / 3.0f), __powf(__fdividef(c, a), 0.2f));
    float v = (u_prev > 0.0f && u_prev < ub) ? u_prev : ub;
    const float a5 = 5.0f * a, b3 = 3.0f * b;
#pragma unroll 1
    for (int it = 0; it < 12; ++it) {
        const float v2 = v * v;
        const float g = v2 * v * fmaf(a, v2, b) - c;
        const float dg = v2 * fmaf(a5, v2, b3);
        const float dv = __fdividef(g, dg);
        v = fminf(v - dv, ub);
        if (!(fabsf(dv) > 3e-7f * v)) break;
    }
    const wff::ff v2 = wff::two_prod(v, v);
    const wff::ff v3 = wff::mul(v2, v);
    const wff::ff v5 = wff::mul(v3, v2);
    const wff::ff f = wff::add(wff::add(wff::mul(dt_dx, v5), wff::mul(v3, b)), wff::neg(cterm));
    const float dv = __fdividef(f.hi, v2.hi * fmaf(a5, v2.hi, b3));
    wff::ff u = wff::two_sum(v, -dv);
    wff::ff q = wff::add(v5, wff::mul(wff::mul(v2, v2), -5.0f * dv));
    if (!(u.hi > QR)) {
        u = {QR, 0.0f};
        q = {(float)KIN_WAVE_MIN_FLOW, 0.0f};
    }
    u_out = u;
    q_out = q;
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
// node), FP32 on the critical path. The linear kinematic wave gives q = cterm / (dt/dx + 1/c);
// what q depends on beyond that -- the cut of q when the water table would fall below the soil
// (zi > d) and the reference's sub-iterations when the water table moves by more than 0.1 --
// is decided in FP32 with margins, and every case too close to call in FP32 (or a water table
// rising through more than one layer, or non-finite values) goes through the exact FP64
// computation of ssf_full_split. The FP64 bookkeeping of the fast cases (net flux, water-table
// change, exfiltration) is redone exactly by ssf_post_kernel from the same q.
enum SsfFlag { SSF_FAST = 0, SSF_EARLY = 1, SSF_FULL = 2, SSF_CUT = 3 };

template <int MAXN>
struct SsfWave {
    WfDevFields F;
    WfDevGraph g;
    WfSweep sw;
    struct In {
        float qnet, t2, rdf, zi, rth, rcap, rrho, qmaxdw, d, dtdx, idwdx, dtsy, k2;
        bool qprev_zero;
        wfv::UpList up;
    };
    __device__ __forceinline__ void load(int64_t slot, int64_t e, int m, In& x) const {
        float* const* Mh = F.Mh;
        float* const* Lf = F.Lf;
        x.qnet = Mh[SSF_QNETF][e];
        x.t2 = Mh[SSF_T2][e];
        x.rdf = Mh[SSF_RDF][e];
        x.zi = Mh[SSF_ZIF][e];
        x.rth = Mh[SSF_RTH][e];
        x.rcap = Mh[SSF_RCAP][e];
        x.rrho = Mh[SSF_RRHO][e];
        x.qmaxdw = Mh[Q_MAX][e] * Lf[FLOW_WIDTH][slot];
        x.d = Lf[SOIL_THICKNESS][slot];
        x.dtdx = Lf[SSF_DTDX][slot];
        x.idwdx = Lf[SSF_IDWDX][slot];
        x.dtsy = Lf[SSF_DTSY][slot];
        x.k2 = Lf[SSF_K2][slot];
        x.qprev_zero = (__double_as_longlong(F.Mf[SSF_Q][e]) << 1) == 0;
        wfv::load_up(g, sw, slot, m, x.up);
    }
    __device__ __forceinline__ bool node(const In& x, int64_t slot, int64_t e, int m, int64_t chain, bool is_end,
                                         unsigned long long* qh) {
        wff::ff qinff;
        if (!wfv::gather<true>(g, sw, x.up, m, 0, qh[0], F.status, qinff)) return false;
        const float qin = qinff.hi + qinff.lo;
        float q = 0.0f, qu = 0.0f;
        int flag;
        if (qinff.hi == 0.0f && x.qprev_zero && x.qnet <= 0.0f) {
            flag = SSF_EARLY;
        } else {
            const float cterm = x.dtdx * (qin + x.qnet) + x.t2;
            q = cterm * x.rdf;
            if (q != q) q = 0.0f;
            q = fminf(fmaxf(q, 1e-30f), x.qmaxdw);
            qu = q;
            const float nf = (qin + x.qnet - q) * x.idwdx;
            bool full = false;
            float dh = 0.0f;
            if (nf <= 0.0f) {
                dh = nf * x.dtsy;
            } else if (!(nf > 0.0f) || (x.rth != 0.0f && x.rcap <= nf * 1.0001f)) {
                full = true;
            } else if (x.rth != 0.0f) {
                dh = nf * x.rrho;
            }
            flag = SSF_FAST;
            if (!full) {
                float zi = x.zi - dh;
                if (fabsf(zi - x.d) <= 1e-5f * x.d) {
                    full = true;
                } else if (zi > x.d) {
                    q = fmaxf(q - x.k2 * (zi - x.d), 1e-30f);
                    zi = x.d;
                    flag = SSF_CUT;
                }
                zi = fminf(fmaxf(zi, 0.0f), x.d);
                if (!(fabsf(zi - x.zi) * 10.0f <= 0.999f)) full = true;
            }
            if (full) {
                double qd, zid, exfd, nfd;
                const double qind = (double)qin;
                ssf_full_split<MAXN>(F, slot, e, qind, F.Mf[SSF_QNET][e], sw.dts[0], qd, zid, exfd, nfd);
                double* const* Mf = F.Mf;
                Mf[SSF_Q][e] = qd;
                Mf[SSF_ZI][e] = zid;
                Mf[SSF_TEXF][e] = exfd;
                Mf[SSF_TNF][e] = nfd;
                Mf[SSF_TQIN][e] = qind;
                q = (float)qd;
                flag = SSF_FULL;
            }
        }
        float* const* Mh = F.Mh;
        const wff::ff qf = {q, 0.0f};
        qh[0] = wff::pack(qf);
        if (is_end) wfv::publish(g, chain, m, 0, qf);
        Mh[SSF_QF][e] = q;
        Mh[SSF_QUF][e] = qu;
        Mh[SSF_QINF][e] = qin;
        Mh[SSF_FLAG][e] = (float)flag;
        return true;
    }
};

// Overland flow (surface_process.jl:24-70 per node, routing/surface_kinwave.jl sub-steps) in
// double-FP32: discharge, u = Q^0.2 and the lateral inflow are pairs of FP32 arrays.
struct OlWave {
    WfDevFields F;
    WfDevGraph g;
    WfSweep sw;
    struct In {
        wff::ff u, q, qlat, invdx;
        float alpha;
        bool sfw_pos;
        wfv::UpList up;
    };
    __device__ __forceinline__ void load(int64_t slot, int64_t e, int m, In& x) const {
        float* const* Mh = F.Mh;
        x.u = {Mh[OL_UH][e], Mh[OL_UL][e]};
        x.q = {Mh[OL_QH][e], Mh[OL_QL][e]};
        x.qlat = {Mh[OL_QLATH][e], Mh[OL_QLATL][e]};
        x.invdx = {F.Lf[INV_FLOW_LENGTH][slot], F.Lf[INV_DX_LO][slot]};
        x.alpha = F.Lf[OL_ALPHA][slot];
        x.sfw_pos = F.Lf[SFW][slot] > 0.0f;
        wfv::load_up(g, sw, slot, m, x.up);
    }
    __device__ __forceinline__ bool node(const In& x, int64_t slot, int64_t e, int m, int64_t chain, bool is_end,
                                         unsigned long long* qh) {
        const int stride = blockDim.x;
        wff::ff u = x.u, qp = x.q, qsum = {0.0f, 0.0f};
        for (int s = 0; s < sw.S; ++s) {
            const float dt_s = sw.dts_f[s];
            wff::ff qin;
            if (!wfv::gather<true>(g, sw, x.up, m, s, qh[s * stride], F.status, qin)) return false;
            if (!x.sfw_pos) qin = {0.0f, 0.0f};
            wff::ff un, qn;
            if (qin.hi == 0.0f && qp.hi == 0.0f && x.qlat.hi == 0.0f) {
                un = {0.0f, 0.0f};
                qn = {0.0f, 0.0f};
            } else {
                const wff::ff dt_dx = wff::mul(x.invdx, dt_s);
                const wff::ff u3 = wff::mul(wff::mul(u, u), u);
                const wff::ff cterm =
                    wff::add(wff::mul(dt_dx, qin), wff::add(wff::mul(u3, x.alpha), wff::mul(x.qlat, dt_s)));
                kw_solve_ff(cterm, dt_dx, x.alpha, u.hi, un, qn);
            }
            u = un;
            qp = qn;
            qh[s * stride] = wff::pack(qn);
            if (is_end) wfv::publish(g, chain, m, s, qn);
            qsum = wff::add(qsum, wff::mul(qn, dt_s));
        }
        float* const* Mh = F.Mh;
        Mh[OL_UH][e] = u.hi;
        Mh[OL_UL][e] = u.lo;
        Mh[OL_QH][e] = qp.hi;
        Mh[OL_QL][e] = qp.lo;
        if (sw.first != 0) qsum = wff::add(qsum, wff::ff{Mh[OL_QSUMH][e], Mh[OL_QSUML][e]});
        Mh[OL_QSUMH][e] = qsum.hi;
        Mh[OL_QSUML][e] = qsum.lo;
        return true;
    }
};

// River flow (surface_process.jl:24-70 per node, routing/river_kinwave.jl sub-steps) in
// double-FP32, with the abstraction of a negative external inflow limited to 80 % of the
// storage.
struct RvWave {
    WfDevFields F;
    WfDevGraph g;
    WfSweep sw;
    struct In {
        wff::ff u, q, qlatt, invlen;
        float alpha, len, ext;
        wfv::UpList up;
    };
    __device__ __forceinline__ void load(int64_t slot, int64_t e, int m, In& x) const {
        float* const* RMh = F.RMh;
        x.u = {RMh[RV_UH][e], RMh[RV_UL][e]};
        x.q = {RMh[RV_QH][e], RMh[RV_QL][e]};
        x.qlatt = {RMh[RV_QLATTH][e], RMh[RV_QLATTL][e]};
        x.invlen = {F.Rf[R_INV_LENGTH][slot], F.Rf[R_INV_LEN_LO][slot]};
        x.alpha = F.Rf[R_ALPHA][slot];
        x.len = F.Rf[R_LENGTH][slot];
        x.ext = F.Rf[R_EXT_INFLOW][slot];
        wfv::load_up(g, sw, slot, m, x.up);
    }
    __device__ __forceinline__ bool node(const In& x, int64_t slot, int64_t e, int m, int64_t chain, bool is_end,
                                         unsigned long long* qh) {
        const int stride = blockDim.x;
        wff::ff u = x.u, qp = x.q, qsum = {0.0f, 0.0f}, asum = {0.0f, 0.0f};
        for (int s = 0; s < sw.S; ++s) {
            const float dt_s = sw.dts_f[s];
            wff::ff qin;
            if (!wfv::gather<false>(g, sw, x.up, m, s, qh[s * stride], F.status, qin)) return false;
            wff::ff ql = x.qlatt;
            if (x.ext < 0.0f) {  // abstraction: qlatt holds the lateral inflow alone
                const float storage = x.len * (x.alpha * (u.hi * u.hi * u.hi));
                const float absd = fminf(-x.ext, (storage / dt_s) * 0.80f);
                ql = wff::add(ql, wff::mul(x.invlen, -absd));
                asum = wff::add(asum, wff::two_prod(absd, dt_s));
            }
            wff::ff un, qn;
            if (qin.hi == 0.0f && qp.hi == 0.0f && ql.hi == 0.0f) {
                un = {0.0f, 0.0f};
                qn = {0.0f, 0.0f};
            } else {
                const wff::ff dt_dx = wff::mul(x.invlen, dt_s);
                const wff::ff u3 = wff::mul(wff::mul(u, u), u);
                const wff::ff cterm =
                    wff::add(wff::mul(dt_dx, qin), wff::add(wff::mul(u3, x.alpha), wff::mul(ql, dt_s)));
                kw_solve_ff(cterm, dt_dx, x.alpha, u.hi, un, qn);
            }
            u = un;
            qp = qn;
            qh[s * stride] = wff::pack(qn);
            if (is_end) wfv::publish(g, chain, m, s, qn);
            qsum = wff::add(qsum, wff::mul(qn, dt_s));
        }
        float* const* RMh = F.RMh;
        RMh[RV_UH][e] = u.hi;
        RMh[RV_UL][e] = u.lo;
        RMh[RV_QH][e] = qp.hi;
        RMh[RV_QL][e] = qp.lo;
        if (sw.first != 0) {
            qsum = wff::add(qsum, wff::ff{RMh[RV_QSUMH][e], RMh[RV_QSUML][e]});
            asum = wff::add(asum, wff::ff{RMh[RV_ABSH][e], RMh[RV_ABSL][e]});
        }
        RMh[RV_QSUMH][e] = qsum.hi;
        RMh[RV_QSUML][e] = qsum.lo;
        RMh[RV_ABSH][e] = asum.hi;
        RMh[RV_ABSL][e] = asum.lo;
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
    const size_t smem = (size_t)threads * phys.sw.S * sizeof(unsigned long long);
    int blocks;
    Phys p = phys;
    cudaError_t err = wave_grid(wave_kernel<Phys>, threads, smem, c, p.g, blocks, p.sw.prio_items);
    if (err != cudaSuccess) return err;
    wave_kernel<Phys><<<blocks, threads, smem, c.stream>>>(p);
    return cudaGetLastError();
}

// --------------------------------------------------------------- post-sweep kernels ------

// After the subsurface sweep: the exact FP64 bookkeeping of the fast cases (net flux and
// water-table change from the walker's q, exfiltration), the unsaturated-layer adjustment to
// the new water table (soil.jl update_ustorelayerdepth!), averages, subsurface storage, the soil
// water storage update (sbm.jl update_soil_water_storage!) and the overland lateral inflow.
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
        float* const* Mh = F.Mh;
        double* const* L = F.L;
        const int flag = (int)Mh[SSF_FLAG][e];
        const double zi_soil = Mf[ZI][e];
        const double d = L[SOIL_THICKNESS][slot];
        const double te = L[THETA_S][slot] - L[THETA_R][slot];
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
        double q, qin, exf, nf, zi_new, zi_s;
        if (flag == SSF_EARLY) {
            q = qin = exf = nf = 0.0;
            zi_new = d;
            zi_s = zi_soil;
            Mf[SSF_Q][e] = 0.0;
            Mf[SSF_ZI][e] = d;
        } else if (flag == SSF_FULL) {
            q = Mf[SSF_Q][e];
            qin = Mf[SSF_TQIN][e];
            exf = Mf[SSF_TEXF][e];
            nf = Mf[SSF_TNF][e];
            zi_new = zi_s = Mf[SSF_ZI][e];
#pragma unroll
            for (int k = 0; k < MAXN; ++k) usld[k] = k < N ? F.LY[LY_USLD][k][e] : 0.0;
        } else {
            q = (double)Mh[SSF_QF][e];
            qin = (double)Mh[SSF_QINF][e];
            const double qu = (double)Mh[SSF_QUF][e];
            nf = (qin + Mf[SSF_QNET][e] - qu) * L[SSF_IDWDX][slot];
            // water_table_change (subsurface_process.jl): falling by net flux / specific yield,
            // rising through the unsaturated layers from the deepest up
            double dh = 0.0, rem = nf;
            if (nf <= 0.0) {
                dh = nf * L[SSF_DTSY][slot];
            } else {
                const double dts = F.dt_ssf;
                const int nu0 = nu_at(zi_soil);
#pragma unroll
                for (int k = MAXN; k >= 1; --k) {
                    if (k > nu0 || rem == 0.0) continue;
                    const double t = thick_at(zi_soil, k - 1);
                    const double cap = fmax(t * te - usld[k - 1], 0.0) * F.inv_dt_ssf;
                    const double fl = fmin(rem, cap);
                    dh += cap <= rem ? t : fl * dts * wfm_rcp(te - usld[k - 1] * wfm_rcp(t));
                    rem -= fl;
                }
            }
            exf = fmax(rem, 0.0);
            double zi = zi_soil - dh;
            if (flag == SSF_CUT || zi > d) zi = d;
            zi_new = zi_s = fmin(fmax(zi, 0.0), d);
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
            Mf[SSF_Q][e] = q;
            Mf[SSF_ZI][e] = zi_new;
        }
        const int nu = nu_at(zi_s);
        double tr = 0.0;
        for (int32_t o = g.up_ptr[slot]; o < g.up_ptr[slot + 1]; ++o)
            tr += (double)Mh[SSF_QF][g.up_slot[o] * M + m] * g.up_fr[o];
        const double area = L[AREA][slot];
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
        const double sat = (d - zi_s) * te;
        Mf[SAT][e] = sat;
        Mf[USTOREDEPTH][e] = usd;
        Mf[TSWS][e] = sat + usd;
        Mf[EXFILT][e] = exf_avg;
        Mf[RUNOFF][e] = runoff;
        const double net_runoff = runoff - Mf[AE_LAND][e];
        Mf[NET_RUNOFF][e] = net_runoff;
        const double inwater = net_runoff * area;
        Mf[OL_INWATER][e] = inwater;
        const double qlat = inwater * L[INV_FLOW_LENGTH][slot];
        Mf[OL_QLAT][e] = qlat;
        const wff::ff qlf = wff::from_d(qlat);
        Mh[OL_QLATH][e] = qlf.hi;
        Mh[OL_QLATL][e] = qlf.lo;
    }
}

// After the overland sweep: discharge, water depth and storage in FP64 from the double-FP32
// state, averages, and the lateral inflow of the river cell of each land cell
// (routing/river_kinwave.jl update_lateral_inflow!).
__global__ void __launch_bounds__(256) ol_post_kernel(WfDevFields F, WfDevGraph g) {
    const int M = F.M;
    const int64_t E = F.land_slots * M;
    const double inv_dt = F.inv_dt;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t slot = e / M;
        if (F.land_node_of_slot[slot] < 0) continue;
        const int m = (int)(e - slot * M);
        double* const* Mf = F.Mf;
        float* const* Mh = F.Mh;
        double* const* L = F.L;
        Mf[OL_Q][e] = wff::to_d({Mh[OL_QH][e], Mh[OL_QL][e]});
        const double inv_sfw = L[INV_SFW][slot];
        if (inv_sfw > 0.0) {
            const double u = wff::to_d({Mh[OL_UH][e], Mh[OL_UL][e]});
            const double a = (double)F.Lf[OL_ALPHA][slot] * (u * u * u);
            Mf[OL_H][e] = a * inv_sfw;
            Mf[OL_STORAGE][e] = L[FLOW_LENGTH][slot] * a;
        }
        double qin = 0.0, tr = 0.0;
        for (int32_t o = g.up_ptr[slot]; o < g.up_ptr[slot + 1]; ++o) {
            const int64_t ue = g.up_slot[o] * M + m;
            const double qs = wff::to_d({Mh[OL_QSUMH][ue], Mh[OL_QSUML][ue]});
            qin += qs * (double)g.up_wf[o];
            tr += qs * g.up_fr[o];
        }
        if (!(inv_sfw > 0.0)) qin = 0.0;
        Mf[OL_Q_AVG][e] = wff::to_d({Mh[OL_QSUMH][e], Mh[OL_QSUML][e]}) * inv_dt;
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
            const wff::ff qlt = wff::from_d(ext < 0.0 ? qlat : qlat + ext * inv_len);
            F.RMh[RV_QLATTH][re] = qlt.hi;
            F.RMh[RV_QLATTL][re] = qlt.lo;
        }
    }
}

// After the river sweep: discharge, water depth, storage and averages in FP64.
__global__ void __launch_bounds__(256) rv_post_kernel(WfDevFields F, WfDevGraph g) {
    const int M = F.M;
    const int64_t E = F.river_slots * M;
    const double inv_dt = F.inv_dt;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t slot = e / M;
        if (F.river_node_of_slot[slot] < 0) continue;
        const int m = (int)(e - slot * M);
        double* const* RM = F.RM;
        float* const* RMh = F.RMh;
        double* const* R = F.R;
        RM[RV_Q][e] = wff::to_d({RMh[RV_QH][e], RMh[RV_QL][e]});
        const double u = wff::to_d({RMh[RV_UH][e], RMh[RV_UL][e]});
        const double a = (double)F.Rf[R_ALPHA][slot] * (u * u * u);
        RM[RV_H][e] = a * R[R_INV_WIDTH][slot];
        RM[RV_STORAGE][e] = R[R_LENGTH][slot] * a;
        double qin = 0.0;
        for (int32_t o = g.up_ptr[slot]; o < g.up_ptr[slot + 1]; ++o) {
            const int64_t ue = g.up_slot[o] * M + m;
            qin += wff::to_d({RMh[RV_QSUMH][ue], RMh[RV_QSUML][ue]});
        }
        RM[RV_Q_AVG][e] = wff::to_d({RMh[RV_QSUMH][e], RMh[RV_QSUML][e]}) * inv_dt;
        RM[RV_QIN_AVG][e] = qin * inv_dt;
        RM[RV_ABS_AVG][e] = wff::to_d({RMh[RV_ABSH][e], RMh[RV_ABSL][e]}) * inv_dt;
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

// Double-FP32 discharge and u = Q^0.2 of the overland and river state from the FP64 fields
// (after a discharge was set from outside, and at creation).
__global__ void __launch_bounds__(256) sync_u_kernel(WfDevFields F) {
    const int M = F.M;
    const int64_t EL = F.land_slots * M, ER = F.river_slots * M;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < EL + ER; i += (int64_t)gridDim.x * blockDim.x) {
        if (i < EL) {
            const double q = F.Mf[OL_Q][i];
            const wff::ff qf = wff::from_d(q), uf = wff::from_d(u_of_q(q));
            F.Mh[OL_QH][i] = qf.hi;
            F.Mh[OL_QL][i] = qf.lo;
            F.Mh[OL_UH][i] = uf.hi;
            F.Mh[OL_UL][i] = uf.lo;
        } else {
            const int64_t e = i - EL;
            const double q = F.RM[RV_Q][e];
            const wff::ff qf = wff::from_d(q), uf = wff::from_d(u_of_q(q));
            F.RMh[RV_QH][e] = qf.hi;
            F.RMh[RV_QL][e] = qf.lo;
            F.RMh[RV_UH][e] = uf.hi;
            F.RMh[RV_UL][e] = uf.lo;
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
    int blocks;
    Phys p = phys;
    cudaError_t err = wave_grid(walk_split_kernel<Phys>, threads, 0, c, p.g, blocks, p.sw.prio_items);
    if (err != cudaSuccess) return err;
    walk_split_kernel<Phys><<<blocks, threads, 0, c.stream>>>(p);
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
