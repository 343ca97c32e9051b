// kernels_split.cu -- FP32/FP64 split form of the SBM + kinematic-wave step.
//
// GB300 runs FP32 at about 64 times its FP64 rate, so this form evaluates every rate that
// needs a transcendental (Brooks-Corey powers, exponential Kv profile, Feddes heads, s-curves,
// the Gash log, soil-column drainage iterations) in FP32 with CUDA's accurate expf/logf, reads
// parameters and forcing as FP32, and keeps at higher precision:
//   * every storage state (canopy, snow, unsaturated layers, subsurface, overland and river
//     discharge and storage) and every update applied to it as a double-FP32 pair (wf_ff.cuh,
//     a 48-bit significand), and the large stores that a step changes by as little as 1e-15 of
//     their size (saturated depth, water-table depths, total soil water, the land balance's
//     previous storage) in FP64, so the water balance stays closed;
//   * the flux partitions and sums that enter the balance (throughfall/stemflow/canopy,
//     rain/snow, infiltration and excess water, actual evapotranspiration, runoff) as pairs;
//   * the kinematic-wave solves for discharge: overland and river (surface_process.jl:24-70)
//     iterate Newton in FP32 from an FP32 initial guess and finish with one Newton correction
//     evaluated in double-FP32 (kw_node_ff), so the discharge carries the pair's precision
//     although the iterations are FP32; the subsurface solve (subsurface_process.jl:57-78) runs
//     in FP64 (kw_ssf_newton_s);
//   * the cumulative sub-step fluxes and the balance terms as pairs; reservoirs in FP64.
// The process structure, limiters and branch order are those of the FP64 form (see
// kernels_fp64.cu for the reference line citations of each function).
#include <cuda_runtime.h>

#include <type_traits>

#include "wf_fields.cuh"
#include "wf_kernels.h"
#include "wf_launch.cuh"
#include "wf_math.cuh"
#include "wf_reservoir.cuh"
#include "snow_scheme.cuh"
#include "wf_walker.cuh"
#include "wf_ff.cuh"
#include "wf_wave.cuh"

// Compile-time loop: fn(std::integral_constant<int, k>) for k = B, B + S, ... while k != E
// (S = 1 or -1). The layer loops of the vertical kernel use it so that every per-layer array is
// indexed by constants from the start and stays in registers.
namespace wfu {
template <int B, int E, int S, class Fn>
__device__ __forceinline__ void static_for(Fn&& fn) {
    if constexpr (B != E) {
        fn(std::integral_constant<int, B>{});
        static_for<B + S, E, S>(fn);
    }
}
}  // namespace wfu


using wfm::jclamp;
using wfm::jmax;
using wfm::jmin;

namespace {

// FP64 view of the split form's double-FP32 member fields, for the rare paths that keep the
// reference's FP64 arithmetic (the full subsurface column computation, sub-stepped subsurface
// flow): Mf[field][e] reads and writes a (high, low) pair as one double.
struct FFRef {
    float* h;
    float* l;
    double* d;  // the field is FP64 (a large store)
    __device__ __forceinline__ operator double() const { return d ? *d : (double)*h + (double)*l; }
    __device__ __forceinline__ FFRef& operator=(double v) {
        if (d) {
            *d = v;
            return *this;
        }
        const float a = (float)v;
        *h = a;
        *l = (float)(v - (double)a);
        return *this;
    }
};
struct FFRow {
    float* h;
    float* l;
    double* d;
    __device__ __forceinline__ FFRef operator[](int64_t e) const {
        return d ? FFRef{nullptr, nullptr, d + e} : FFRef{h + e, l + e, nullptr};
    }
};
struct FFMem {  // member fields
    const WfDevFields& F;
    __device__ __forceinline__ FFRow operator[](int f) const {
        return wf_split_fp64_member(f) ? FFRow{nullptr, nullptr, F.Mf[f]} : FFRow{F.Mh[f], F.Ml[f], nullptr};
    }
};
struct FFUsld {  // unsaturated layer stores
    const WfDevFields& F;
    __device__ __forceinline__ FFRow operator[](int k) const { return {F.LYf[LY_USLD][k], F.LYl[k], nullptr}; }
};

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


// Store of the split form: its content at the start of the step (a double-FP32 pair) plus
// the exact sum of the step's FP32 increments (TwoSum / TwoProd), added once at the end.
struct Store {
    wff::ff base;
    float hi, lo;  // increments of this step: exactly hi + lo
    bool mod;      // content differs from what was loaded
    __device__ __forceinline__ void init(wff::ff b) {
        base = b;
        hi = 0.0f;
        lo = 0.0f;
        mod = false;
    }
    __device__ __forceinline__ float val() const { return base.hi + hi; }
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
    __device__ __forceinline__ void add(wff::ff x) {
        add(x.hi);
        lo += x.lo;
    }
    __device__ __forceinline__ bool changed() const { return mod; }
    __device__ __forceinline__ wff::ff value() const { return wff::add(base, wff::ff{hi, lo}); }
    __device__ __forceinline__ void zero() {
        base = {0.0f, 0.0f};
        hi = 0.0f;
        lo = 0.0f;
        mod = true;
    }
    __device__ __forceinline__ void set(wff::ff v) {
        init(v);
        mod = true;
    }
    __device__ __forceinline__ wff::ff take_all() {  // empties the store, returns its content
        const wff::ff v = value();
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
    // from the field arrays, or (s32, s64 non-null) from a staged copy: layer thicknesses and
    // bottom depths (FP32) at s32[0..MAXN) and s32[MAXN..2 MAXN), bottom depths (FP64) at s64
    __device__ __forceinline__ void set(const WfDevFields& F, int64_t slot, double zi, const float* s32 = nullptr,
                                        const double* s64 = nullptr) {
        N = F.N;
        nl = F.nlayers[slot];
        nu = N;
        cum[0] = 0.0f;
        double c0 = 0.0;
#pragma unroll
        for (int k = 0; k < MAXN; ++k) {
            float t = __int_as_float(0x7fc00000);
            if (k < N) {
                act[k] = s32 ? s32[k] : F.LYf[LY_ACT_THICK][k][slot];
                const double c1 = s64 ? s64[k] : F.LY[LY_CUM][k][slot];
                cum[k + 1] = s32 ? s32[MAXN + k] : F.LYf[LY_CUM][k][slot];
                if (zi > c1) {
                    t = act[k];
                } else if (zi > c0) {
                    t = (float)(zi - c0);
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

__device__ __forceinline__ wff::ff ldm(const WfDevFields& F, int f, int64_t e) { return {F.Mh[f][e], F.Ml[f][e]}; }
__device__ __forceinline__ void stm(const WfDevFields& F, int f, int64_t e, wff::ff v) {
    F.Mh[f][e] = v.hi;
    F.Ml[f][e] = v.lo;
}
__device__ __forceinline__ wff::ff lds(const WfDevFields& F, int f, int64_t slot) { return {F.Lf[f][slot], F.Ll[f][slot]}; }
__device__ __forceinline__ wff::ff ldr(const WfDevFields& F, int f, int64_t e) { return {F.RMh[f][e], F.RMl[f][e]}; }
__device__ __forceinline__ void str(const WfDevFields& F, int f, int64_t e, wff::ff v) {
    F.RMh[f][e] = v.hi;
    F.RMl[f][e] = v.lo;
}
__device__ __forceinline__ wff::ff ldrs(const WfDevFields& F, int f, int64_t slot) {
    return {F.Rf[f][slot], F.Rl[f][slot]};
}

// ----------------------------------------------------------------- member-field staging --
//
// The vertical kernel reads some 27 member fields per element, each from its own array, and is
// bound by the latency of those loads at the occupancy its registers allow. Each thread
// therefore copies the member fields of the element it will compute next into its own
// shared-memory slots with asynchronous copies (cp.async, 4 and 8 bytes) while it computes the
// current one, and waits for them (cp.async.wait_group) only when it gets there: a per-thread
// double buffer, so no barrier is involved (a thread reads back only what it copied itself).
// The per-cell parameters stay ordinary loads: they are shared by the members of a cell and
// come from L1/L2.
enum VStage32 {
    VS_PRECIP, VS_POTEVAP, VS_TEMP, VS_KV0, VS_FSCALE, VS_TSOIL, VS_OL_H, VS_CANOPY_H, VS_CANOPY_L, VS_SNOW_H,
    VS_SNOW_L, VS_SW_H, VS_SW_L, VS_SSFQ_H, VS_SSFQ_L, VS_OLST_H, VS_OLST_L, VS_USLD_H
};
enum VStage64 { VD_SAT, VD_TSWS, VD_COUNT };
template <int MAXN>
struct VStage {
    static constexpr int N32 = VS_USLD_H + 2 * MAXN;  // USLD high parts, then low parts
    static constexpr size_t bytes_per_thread = N32 * sizeof(float) + VD_COUNT * sizeof(double);
};

__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(a), "l"(gmem));
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(a), "l"(gmem));
}
// No compiler memory clobber on the copies and the commit (it would make the compiler reload every
// shared value it holds after each copy); the wait has one, and the loop of the vertical kernel
// puts a compiler barrier before each refill of a buffer that was read in the previous iteration.
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;"); }
__device__ __forceinline__ void cp_async_wait_prev() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// Stage the member fields of element e into buffer (f32, f64) of this thread (stride = block
// size between fields).
template <int MAXN>
__device__ __forceinline__ void stage_vertical(const WfDevFields& F, int64_t e, float* f32, double* f64, int st) {
    auto c4 = [&](int i, const float* src) { cp_async4(f32 + i * st, src + e); };
    c4(VS_PRECIP, F.Mh[PRECIP]);
    c4(VS_POTEVAP, F.Mh[POTEVAP]);
    c4(VS_TEMP, F.Mh[TEMP]);
    c4(VS_KV0, F.Mh[KV0]);
    c4(VS_FSCALE, F.Mh[FSCALE]);
    c4(VS_TSOIL, F.Mh[TSOIL]);
    c4(VS_OL_H, F.Mh[OL_H]);
    c4(VS_CANOPY_H, F.Mh[CANOPY]);
    c4(VS_CANOPY_L, F.Ml[CANOPY]);
    if (F.snow) {
        c4(VS_SNOW_H, F.Mh[SNOW]);
        c4(VS_SNOW_L, F.Ml[SNOW]);
        c4(VS_SW_H, F.Mh[SNOW_WATER]);
        c4(VS_SW_L, F.Ml[SNOW_WATER]);
    }
    if (F.ssf_single) {
        c4(VS_SSFQ_H, F.Mh[SSF_Q]);
        c4(VS_SSFQ_L, F.Ml[SSF_Q]);
    }
    if (F.mass_balance) {
        c4(VS_OLST_H, F.Mh[OL_STORAGE]);
        c4(VS_OLST_L, F.Ml[OL_STORAGE]);
    }
#pragma unroll
    for (int k = 0; k < MAXN; ++k)
        if (k < F.N) {
            c4(VS_USLD_H + k, F.LYf[LY_USLD][k]);
            c4(VS_USLD_H + MAXN + k, F.LYl[k]);
        }
    cp_async8(f64 + VD_SAT * st, F.Mf[SAT] + e);
    cp_async8(f64 + VD_TSWS * st, F.Mf[TSWS] + e);
}

// Per-cell parameters of the vertical kernel, staged once per warp. With a multiple of 32 members
// the 32 lanes of a warp compute 32 members of one cell (members are innermost), so the cell's
// parameters are the same for the whole warp: its lanes copy them (cp.async) into a per-warp
// shared row for the warp's next element, and every lane reads them back as broadcasts. They
// then occupy no registers while the element computes and cost no global round trip.
#define WF_VW_LFIELDS(X)                                                                            \
    X(ALPHA_H1) X(CAP_COMP) X(CAP_HMAX) X(CAP_N) X(CF_SOIL) X(CMAX) X(COMPACT_FRAC) X(DDF) X(E_R) X(GAP) X(H1) X(H2) \
    X(H3_HIGH) X(H3_LOW) X(H4) X(KC) X(KH_RATIO) X(MAX_LEAKAGE) X(PSI_B) X(RIVER_FRACTION) X(ROOTDISTPAR)          \
    X(ROOTING_DEPTH) X(SLOPE) X(SOIL_THICKNESS) X(SSF_DTDX) X(SWC) X(SY) X(THETA_FC) X(THETA_R) X(THETA_S) X(TT)  \
    X(TTI) X(TTM) X(WATER_FRACTION) X(WHC) X(W_SOIL) X(Z_EXP)
#define WF_VW_ITEM(name) VW_##name,
enum VW32 {
    WF_VW_LFIELDS(WF_VW_ITEM)
    VW_CMAX_LO, VW_AREA_HI, VW_AREA_LO, VW_LY  // then per layer: thickness, bottom depth, Kv factor, c, root fraction
};
#undef WF_VW_ITEM
enum VW64 { VW_D_SOIL_THICKNESS, VW_D_INV_TE, VW_D_SLOPE, VW_D_CUM };  // then one bottom depth per layer
template <int MAXN>
struct VWarp {
    static constexpr int N32 = VW_LY + 5 * MAXN;
    static constexpr int N64 = VW_D_CUM + MAXN + 2;  // + node and river slot (int64)
    static constexpr size_t bytes = ((size_t)N64 * 8 + (size_t)N32 * 4 + 7) / 8 * 8;  // one buffer
};

// Lanes of a warp copy the parameters of cell `slot` into the warp's buffer (w64: doubles and
// the two slot indices, w32: floats).
template <int MAXN>
__device__ __forceinline__ void stage_vertical_warp(const WfDevFields& F, int64_t slot, double* w64, float* w32,
                                                    int lane) {
    constexpr int N32 = VWarp<MAXN>::N32;
    for (int i = lane; i < N32; i += 32) {
        const float* src = nullptr;
        if (i < VW_CMAX_LO) {
#define WF_VW_SRC(name) if (i == VW_##name) src = F.Lf[name];
            WF_VW_LFIELDS(WF_VW_SRC)
#undef WF_VW_SRC
        } else if (i == VW_CMAX_LO) {
            src = F.Ll[CMAX];
        } else if (i == VW_AREA_HI) {
            src = F.Lf[AREA];
        } else if (i == VW_AREA_LO) {
            src = F.Ll[AREA];
        } else {
            const int k = (i - VW_LY) % MAXN, which = (i - VW_LY) / MAXN;
            if (k < F.N) {
#pragma unroll
                for (int kk = 0; kk < MAXN; ++kk) {
                    if (kk != k) continue;
                    src = which == 0   ? F.LYf[LY_ACT_THICK][kk]
                          : which == 1 ? F.LYf[LY_CUM][kk]
                          : which == 2 ? F.LYf[LY_KVFRAC][kk]
                          : which == 3 ? F.LYf[LY_C][kk]
                                       : F.LYf[LY_ROOTFRAC][kk];
                }
            }
        }
        if (src) cp_async4(w32 + i, src + slot);
    }
    if (lane < VW_D_CUM + MAXN) {
        const double* src = nullptr;
        if (lane == VW_D_SOIL_THICKNESS) src = F.L[SOIL_THICKNESS];
        else if (lane == VW_D_INV_TE) src = F.L[INV_TE];
        else if (lane == VW_D_SLOPE) src = F.L[SLOPE];
        else {
#pragma unroll
            for (int kk = 0; kk < MAXN; ++kk)
                if (lane - VW_D_CUM == kk && kk < F.N) src = F.LY[LY_CUM][kk];
        }
        if (src) cp_async8(w64 + lane, src + slot);
    } else if (lane < VW_D_CUM + MAXN + 2) {
        const int64_t* src = lane == VW_D_CUM + MAXN ? F.land_node_of_slot : F.land_river_slot;
        cp_async8(w64 + lane, src + slot);
    }
}

// ----------------------------------------------------------------- vertical kernel ------
//
// GB300 issues FP64 instructions (arithmetic, compares and FP32<->FP64 conversions alike) at
// about 1/70 of its FP32 FMA rate, so the split form executes none here: rates, limiters and
// transcendental functions are FP32; every store (canopy, snow, liquid snow water,
// unsaturated layers) and every flux that enters the water balance is a double-FP32 pair
// (wf_ff.cuh); stores take the step's FP32 increments exactly (TwoSum/TwoProd); partitions of
// a flux are exact residuals, so the parts always sum to the whole.
// Parts of the per-cell update, as in the FP64 form: VERT_ALL the whole update; with gravitational
// snow transport VERT_SNOW (interception, snow, transport capacities) and VERT_SOIL (glacier,
// open water, soil) around the transport sweep.
enum VertPhase { VERT_ALL = 0, VERT_SNOW = 1, VERT_SOIL = 2 };

// WS: the members of a cell fill whole warps (a multiple of 32 members), and the cell's
// parameters are staged once per warp (stage_vertical_warp).
template <int MAXN, int PHASE, bool WS>
__global__ void __launch_bounds__(256, 2) vertical_split_kernel(WfDevFields F) {
    using wff::ff;
    const int M = F.M;
    const int64_t E = F.land_slots * M;
    const float dtf = (float)F.dt;
    const ff inv_dt = {F.inv_dt_hi, F.inv_dt_lo};
    const float inv_dtf = F.inv_dt_hi;
    // per-thread double buffer of staged member fields (layout: field-major, stride blockDim)
    extern __shared__ double vstage_smem[];
    const int bd = blockDim.x;
    constexpr int N32 = VStage<MAXN>::N32;
    double* const my64 = vstage_smem + threadIdx.x;  // buffer b: my64 + b * VD_COUNT * bd
    float* const my32 = reinterpret_cast<float*>(vstage_smem + (size_t)2 * VD_COUNT * bd) + threadIdx.x;
    // per-warp double buffer of the cell's parameters (WS)
    const int lane = (int)(threadIdx.x & 31u);
    unsigned char* const wbase = reinterpret_cast<unsigned char*>(vstage_smem + (size_t)2 * VD_COUNT * bd) +
                                 (size_t)2 * N32 * bd * sizeof(float) +
                                 (size_t)(threadIdx.x >> 5) * 2 * VWarp<MAXN>::bytes;
    auto w64 = [&](int b) { return reinterpret_cast<double*>(wbase + (size_t)b * VWarp<MAXN>::bytes); };
    auto w32 = [&](int b) {
        return reinterpret_cast<float*>(wbase + (size_t)b * VWarp<MAXN>::bytes + (size_t)VWarp<MAXN>::N64 * 8);
    };
    const int64_t stride = (int64_t)gridDim.x * bd;
    int64_t e = blockIdx.x * (int64_t)bd + threadIdx.x;
    if (e < E) {
        stage_vertical<MAXN>(F, e, my32, my64, bd);
        if (WS) stage_vertical_warp<MAXN>(F, e / M, w64(0), w32(0), lane);
    }
    cp_async_commit();
    for (int buf = 0; e < E; e += stride, buf ^= 1) {
        // every lane is done reading the warp buffer about to be refilled (the previous element's),
        // and the compiler keeps this thread's reads of the buffer before its refill
        if (WS) __syncwarp();
        asm volatile("" ::: "memory");
        // stage the next element while this one computes
        if (e + stride < E) {
            stage_vertical<MAXN>(F, e + stride, my32 + (buf ^ 1) * N32 * bd, my64 + (buf ^ 1) * VD_COUNT * bd, bd);
            if (WS) stage_vertical_warp<MAXN>(F, (e + stride) / M, w64(buf ^ 1), w32(buf ^ 1), lane);
        }
        cp_async_commit();
        cp_async_wait_prev();
        if (WS) __syncwarp();  // the warp's parameter row was copied by all of its lanes
        const float* const vs = my32 + buf * N32 * bd;
        const double* const vd = my64 + buf * VD_COUNT * bd;
        const float* const W32 = w32(buf);
        const double* const W64 = w64(buf);
        auto V = [&](int i) { return vs[i * bd]; };
        auto VF = [&](int ih, int il) { return ff{vs[ih * bd], vs[il * bd]}; };
        const int64_t slot = e / M;
        const int64_t node =
            WS ? (int64_t)__double_as_longlong(W64[VW_D_CUM + MAXN]) : F.land_node_of_slot[slot];
        if (node < 0) continue;
        const int m = (int)(e - slot * M);
        float* const* Mh = F.Mh;
        float* const* Lf = F.Lf;
#define VP(name) (WS ? W32[VW_##name] : Lf[name][slot])
        // per-cell parameters, loaded up front so that the loads are in flight together
        const float p_alpha_h1 = VP(ALPHA_H1);
        const float p_cap_comp = VP(CAP_COMP);
        const float p_cap_hmax = VP(CAP_HMAX);
        const float p_cap_n = VP(CAP_N);
        const float p_cf_soil = VP(CF_SOIL);
        const float p_cmax = VP(CMAX);
        const float p_compact_frac = VP(COMPACT_FRAC);
        const float p_ddf = VP(DDF);
        const float p_e_r = VP(E_R);
        const float p_gap = VP(GAP);
        const float p_h1 = VP(H1);
        const float p_h2 = VP(H2);
        const float p_h3_high = VP(H3_HIGH);
        const float p_h3_low = VP(H3_LOW);
        const float p_h4 = VP(H4);
        const float p_kc = VP(KC);
        const float p_kh_ratio = VP(KH_RATIO);
        const float p_max_leakage = VP(MAX_LEAKAGE);
        const float p_psi_b = VP(PSI_B);
        const float p_river_fraction = VP(RIVER_FRACTION);
        const float p_rootdistpar = VP(ROOTDISTPAR);
        const float p_rooting_depth = VP(ROOTING_DEPTH);
        const float p_slope = VP(SLOPE);
        const float p_soil_thickness = VP(SOIL_THICKNESS);
        const float p_ssf_dtdx = VP(SSF_DTDX);
        const float p_swc = VP(SWC);
        const float p_sy = VP(SY);
        const float p_theta_fc = VP(THETA_FC);
        const float p_theta_r = VP(THETA_R);
        const float p_theta_s = VP(THETA_S);
        const float p_tt = VP(TT);
        const float p_tti = VP(TTI);
        const float p_ttm = VP(TTM);
        const float p_water_fraction = VP(WATER_FRACTION);
        const float p_whc = VP(WHC);
        const float p_w_soil = VP(W_SOIL);
        const float p_z_exp = VP(Z_EXP);
        const float Pf = V(VS_PRECIP), PETf = V(VS_POTEVAP), Tf = V(VS_TEMP);
        const ff canopy0 = VF(VS_CANOPY_H, VS_CANOPY_L);
        const ff snow0 = F.snow ? VF(VS_SNOW_H, VS_SNOW_L) : ff{0.0f, 0.0f};
        const ff sw0 = F.snow ? VF(VS_SW_H, VS_SW_L) : ff{0.0f, 0.0f};
        if (F.mass_balance && PHASE != VERT_SOIL)
            F.Mf[BL_PREV][e] = vd[VD_TSWS * bd] + wff::to_d(wff::add(canopy0, wff::add(snow0, sw0))) +
                               (F.glacier ? F.GM[GM_STORE][e] * F.G[G_FRAC][slot] : 0.0);
        // ---- interception (canopy.jl:213-226 Gash, :259-271 Rutter)
        const float gapf = p_gap, cmaxf = p_cmax;
        const float potevap_f = p_kc * PETf * (1.0f - gapf);
        ff tf, ic;
        float icf, sff;
        Store canopy;
        canopy.init(canopy0);
        if (PHASE == VERT_SOIL) {  // after the transport sweep: the interception of VERT_SNOW
            ic = wff::from_d(F.GM[GM_IC][e]);
            icf = wff::to_f(ic);
            tf = {0.0f, 0.0f};
            sff = 0.0f;
        } else if (F.gash) {
            if (cmaxf > 0.0f) {
                const float e_r = p_e_r;
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
                const float icr = Pf > psat ? (fi * psat - cmaxf * inv_dtf) + e_r * (Pf - psat) + cmaxf * inv_dtf
                                            : fi * Pf;
                sff = fs * Pf;
                icf = fminf(icr, potevap_f);
                ic = wff::from_f(icf);
                tf = wff::sub(wff::two_sum(Pf, -icf), sff);
            } else {
                tf = wff::from_f(Pf);
                icf = 0.0f;
                ic = {0.0f, 0.0f};
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
            tf = wff::sub(wff::two_sum(Pf, -sff), pcf);
            const ff cmax = WS ? ff{W32[VW_CMAX], W32[VW_CMAX_LO]} : lds(F, CMAX, slot);
            if (wff::gt(canopy0, cmax)) {
                tf = wff::add(tf, wff::mul(wff::sub(canopy0, cmax), inv_dt));
                canopy.set(cmax);
            }
            canopy.add_prod(pcf, dtf);
            if (potevap_f * dtf >= canopy.val() && potevap_f > 0.0f) {
                ic = wff::mul(canopy.take_all(), inv_dt);
                icf = wff::to_f(ic);
            } else {
                icf = potevap_f;
                ic = wff::from_f(icf);
                canopy.add_prod(-icf, dtf);
            }
            if (canopy.val() > cmaxf) {
                const ff c = canopy.value();
                if (wff::gt(c, cmax)) {
                    tf = wff::add(tf, wff::mul(wff::sub(c, cmax), inv_dt));
                    canopy.set(cmax);
                }
            }
        }
        // ---- snow (snow.jl:238-293, snow_process.jl:26-116)
        ff wfs;
        float swe_out = 0.0f;
        Store snow, sw;
        if (PHASE == VERT_SOIL) {  // the moved snow states and the snow runoff of VERT_SNOW
            snow.init(snow0);
            sw.init(sw0);
            wfs = wff::from_d(F.GM[GM_SRUNOFF][e]);
        } else if (F.snow) {
            snow.init(snow0);
            sw.init(sw0);
            const ff eff = wff::add(tf, sff);
            const float tti = p_tti, tt = p_tt;
            const float rainfrac = tti == 0.0f ? (Tf > tt ? 1.0f : 0.0f)
                                               : fminf(fmaxf((Tf - (tt - tti / 2.0f)) / tti, 0.0f), 1.0f);
            const ff lp = wff::mul(eff, rainfrac);
            const ff sp = wff::sub(eff, lp);
            const float ttm = p_ttm, ddf = p_ddf;
            if (Tf > ttm) {
                const float melt = ddf * (Tf - ttm);
                if (melt * dtf >= snow.val()) {
                    if (snow.val() > 0.0f) sw.add(snow.take_all());
                } else {
                    snow.add_prod(-melt, dtf);
                    sw.add_prod(melt, dtf);
                }
            } else {
                const float refr = ddf * 0.05f * (ttm - Tf) * dtf;
                if (refr >= sw.val()) {
                    if (sw.val() > 0.0f) snow.add(sw.take_all());
                } else {
                    snow.add(refr);
                    sw.add(-refr);
                }
            }
            snow.add(wff::mul(sp, dtf));
            sw.add(wff::mul(lp, dtf));
            const float whc = p_whc;
            wfs = {0.0f, 0.0f};
            if (sw.val() > snow.val() * whc) {
                const ff maxsw = wff::mul(snow.value(), whc);
                const ff s = sw.value();
                if (wff::gt(s, maxsw)) {
                    wfs = wff::mul(wff::sub(s, maxsw), inv_dt);
                    sw.set(maxsw);
                }
            }
            swe_out = sw.val() + snow.val();
        } else {
            wfs = wff::add(tf, sff);
        }
        if (PHASE == VERT_SNOW) {
            // lateral_snow_transport! capacities from the updated states (surface_process.jl:9-19)
            if (!F.gash && canopy.changed()) stm(F, CANOPY, e, canopy.value());
            stm(F, SNOW, e, snow.value());
            stm(F, SNOW_WATER, e, sw.value());
            Mh[SWE][e] = swe_out;
            Mh[INTERCEPTION][e] = icf;
            F.GM[GM_IC][e] = wff::to_d(ic);
            F.GM[GM_SRUNOFF][e] = wff::to_d(wfs);
            const double snow_d = wff::to_d(snow.value()), sw_d = wff::to_d(sw.value());
            const double frac = fmin(0.5, (WS ? W64[VW_D_SLOPE] : F.L[SLOPE][slot]) / wfsn::TAN80) *
                                fmin(1.0, snow_d / wfsn::SNOW_STORAGE_MAX);
            F.GM[GM_CAP][e] = frac * snow_d / F.dt;
            F.GM[GM_CAPW][e] = sw_d * frac / F.dt;
            continue;
        }
        // glacier (glacier.jl:122-154, FP64) and its melt in the water flux at the surface
        // (runoff.jl:49-58)
        float gfrac_f = 0.0f;
        if (F.glacier) {
            const double gfrac = F.G[G_FRAC][slot];
            double snow_d = wff::to_d(snow.value()), store, melt;
            wfsn::glacier_hbv(gfrac, F.GM[GM_STORE][e], snow_d, (double)Tf, F.G[G_TTM][slot], F.G[G_DDF][slot],
                              F.G[G_SIFRAC][slot], F.g_max_rate, F.dt, &snow_d, &store, &melt);
            F.GM[GM_STORE][e] = store;
            F.GM[GM_MELT][e] = melt;
            snow.set(wff::from_d(snow_d));
            wfs = wff::from_d(wff::to_d(wfs) + melt * gfrac);
            gfrac_f = (float)gfrac;
        }
        // ---- open water (runoff.jl open-water runoff and evaporation)
        const float rfrac_f = p_river_fraction, wfrac_f = p_water_fraction;
        const float wd_land = V(VS_OL_H);
        const int64_t rs = WS ? (int64_t)__double_as_longlong(W64[VW_D_CUM + MAXN + 1]) : F.land_river_slot[slot];
        const float wd_river = rs >= 0 ? F.RMh[RV_H][rs * M + m] : 0.0f;
        const ff runoff_river = wff::mul(wfs, fminf(1.0f, rfrac_f));
        const ff runoff_land = wff::mul(wfs, fminf(1.0f, wfrac_f));
        const float ae_river_f = rfrac_f * fminf(wd_river * inv_dtf, PETf);
        const float ae_land_f = wfrac_f * fminf(wd_land * inv_dtf, PETf);
        // ---- soil (soil.jl update! of SbmSoilModel)
        const ff wfs_soil = wff::fmax0(wff::sub(wff::sub(wfs, runoff_river), runoff_land));
        const float soil_fraction = fmaxf(gapf - wfrac_f - rfrac_f - gfrac_f, 0.0f);
        const float pot_trans = fmaxf(0.0f, potevap_f - icf);
        const float pot_soilevap = soil_fraction * PETf;
        const double d_soil = WS ? W64[VW_D_SOIL_THICKNESS] : F.L[SOIL_THICKNESS][slot];
        const double sat = vd[VD_SAT * bd];
        const double zi = fmax(0.0, fma(-sat, WS ? W64[VW_D_INV_TE] : F.L[INV_TE][slot], d_soil));
        ColG<MAXN> g;
        g.set(F, slot, zi, WS ? W32 + VW_LY : nullptr, WS ? W64 + VW_D_CUM : nullptr);
        const float zif = (float)zi, df = p_soil_thickness, satf = (float)sat;
        const float ts = p_theta_s, tr = p_theta_r, tfc = p_theta_fc;
        const float te = ts - tr;
        const float kv0 = V(VS_KV0), fsc = V(VS_FSCALE), zexp = p_z_exp;
        const bool kv_const = F.kv_profile == WF_KV_EXPONENTIAL_CONSTANT;
        Store us[MAXN];
        float kvf[MAXN], cexp[MAXN], rfr[MAXN];
        float usd = 0.0f;
        wfu::static_for<0, MAXN, 1>([&](auto kc) {
            constexpr int k = decltype(kc)::value;
            if (k < g.N) {
                us[k].init(VF(VS_USLD_H + k, VS_USLD_H + MAXN + k));
                kvf[k] = WS ? W32[VW_LY + 2 * MAXN + k] : F.LYf[LY_KVFRAC][k][slot];
                cexp[k] = WS ? W32[VW_LY + 3 * MAXN + k] : F.LYf[LY_C][k][slot];
                rfr[k] = WS ? W32[VW_LY + 4 * MAXN + k] : F.LYf[LY_ROOTFRAC][k][slot];
            } else {
                us[k].init({0.0f, 0.0f});
                kvf[k] = cexp[k] = rfr[k] = 0.0f;
            }
            if (k < g.nl) usd += us[k].val();
        });
        // Kv at depth z of layer n (1-based); the layer's factor is selected without dynamic
        // indexing so that the per-layer arrays stay in registers
#define WF_KV_AT(z_, n_)                                           \
    ([&]() {                                                       \
        float zz_ = (z_);                                          \
        if (kv_const && !(zz_ < zexp)) zz_ = zexp;                 \
        float kf_ = 0.0f;                                          \
        wfu::static_for<0, MAXN, 1>([&](auto jc_) {                \
            if (decltype(jc_)::value == (n_) - 1) kf_ = kvf[decltype(jc_)::value]; \
        });                                                        \
        return kf_ * kv0 * expf(-fsc * zz_);                       \
    }())
        float drain = (df - zif) * fmaxf(ts - tfc, 0.02f);
        float ucap = p_swc - satf - usd;
        float tsoil = V(VS_TSOIL);
        if (F.snow) tsoil = tsoil + p_w_soil * (Tf - tsoil);
        float fred = 1.0f;
        if (F.snow && F.infilt_reduction) {
            const float cf = p_cf_soil;
            fred = 1.0f / (1.0f / (1.0f - cf) + expf(-8.0f * (tsoil - 273.15f))) + cf;
        }
        // infiltration (soil_process.jl infiltration): exact partition of the water reaching the soil
        const ff soilinf = wff::mul(wfs_soil, 1.0f - p_compact_frac);
        const ff pathinf = wff::sub(wfs_soil, soilinf);
        const float cap_soil = kv0 * kvf[0] * fred, cap_comp = p_cap_comp * fred;
        const ff mis = cap_soil < soilinf.hi ? wff::from_f(cap_soil) : soilinf;
        const ff mip = cap_comp < pathinf.hi ? wff::from_f(cap_comp) : pathinf;
        const ff infex = wff::add(wff::sub(soilinf, mis), wff::sub(pathinf, mip));
        const float capmax = fmaxf(0.0f, ucap * inv_dtf);
        const ff infil_sum = wff::add(mis, mip);
        const ff infil = infil_sum.hi > capmax ? wff::from_f(capmax) : infil_sum;
        // unsaturated zone flow (soil_process.jl:51-92): FP32 rates, exact transfers
        ff transfer = {0.0f, 0.0f};
        if (g.nu > 0) {
            float z = 0.0f;
            ff flow = infil;  // inflow of the layer as a rate
            wfu::static_for<0, MAXN, 1>([&](auto kc) {
                constexpr int k = decltype(kc)::value;
                if (k >= g.nu) return;
                z += g.thick[k];
                const float l_sat = g.thick[k] * te;
                const float kv_z = WF_KV_AT(z, k + 1);
                us[k].add(wff::mul(flow, dtf));
                const float u = us[k].val();
                if (u <= 0.0f) {
                    us[k].zero();
                    flow = {0.0f, 0.0f};
                    return;
                }
                bool drained;
                const float rate = unsat_rate(u, kv_z, l_sat, cexp[k], dtf, drained);
                if (drained || u - rate * dtf < 0.0f) {
                    flow = wff::mul(us[k].take_all(), inv_dt);
                } else {
                    us[k].add_prod(-rate, dtf);
                    flow = wff::from_f(rate);
                }
            });
            transfer = flow;
        }
        // soil evaporation (soil.jl soil_evaporation!)
        ff soilevap;
        float se_f, esat_f = 0.0f;
        {
            float se = 0.0f;
            const float u0 = us[0].val();
            if (g.nu == 1) se = pot_soilevap * fminf(1.0f, u0 / (zif * te));
            else if (g.nu > 1) se = pot_soilevap * fminf(1.0f, u0 / (g.thick[0] * te));
            ff se_ff;
            if (se > 0.0f && se * dtf >= u0) {
                se_ff = wff::mul(us[0].take_all(), inv_dt);
                se_f = wff::to_f(se_ff);
            } else {
                se_f = se;
                se_ff = wff::from_f(se);
                us[0].add_prod(-se, dtf);
            }
            const float pot = pot_soilevap - se_f;
            if (g.nu <= 1) {
                const float a0 = g.act[0];
                esat_f = fminf(pot * fminf(1.0f, (a0 - zif) / a0), (a0 - zif) * fmaxf(ts - tfc, 0.02f) * inv_dtf);
            }
            drain -= esat_f * dtf;
            soilevap = wff::add(se_ff, esat_f);
        }
        // transpiration (soil.jl transpiration!): FP32 heads, Feddes reduction and root water uptake
        ff actevap = {0.0f, 0.0f};
        float actevap_f = 0.0f, act_sat_f;
        {
            const float rd = p_rooting_depth;
            const float h1 = p_h1, h2 = p_h2, h4 = p_h4, a1 = p_alpha_h1;
            const float psi = p_psi_b;
            const float tpd = pot_trans / MM_PER_DAY_F;
            const float h3l = p_h3_low, h3h = p_h3_high;
            const float h3 = tpd <= 1.0f ? h3l : (tpd < 5.0f ? h3l + (h3h - h3l) * (tpd - 1.0f) / 4.0f : h3h);
            float sum_rf = 0.0f, rf_low = 0.0f;
            wfu::static_for<1, MAXN + 1, 1>([&](auto kc) {
                constexpr int k = decltype(kc)::value;
                if (k <= g.nu) {
                    float r = rfr[k - 1];
                    if (k == g.nu && zif < rd) r = r * (g.thick[k - 1] / fminf(g.act[k - 1], rd - g.cum[k - 1]));
                    sum_rf += r;
                    rf_low = r;
                }
            });
            wfu::static_for<1, MAXN + 1, 1>([&](auto kc) {
                constexpr int k = decltype(kc)::value;
                if (k > g.nu) return;
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
                    const ff a = wff::mul(us[k - 1].take_all(), inv_dt);
                    actevap = wff::add(actevap, a);
                    actevap_f += wff::to_f(a);
                } else {
                    const float a = fminf(want, avail);
                    us[k - 1].add_prod(-a, dtf);
                    actevap = wff::add(actevap, a);
                    actevap_f += a;
                }
            });
            const float wetroots = 1.0f / (1.0f + expf(-p_rootdistpar * (zif - rd)));
            const float alpha0 = rwu_feddes_f(0.0f, h1, h2, h3, h4, a1);
            act_sat_f = fminf((pot_trans - actevap_f) * (wetroots * alpha0), drain * inv_dtf);
            drain -= act_sat_f * dtf;
        }
        // actual infiltration: water above the capacity of a layer moves up, the top layer's
        // excess leaves the soil (soil.jl). The capacity thick * te is FP32 here, while the
        // subsurface completion decides how far a rising water table saturates a layer from the
        // double-FP32 capacity; a layer left fuller than that by FP32 rounding would lose the
        // surplus when the table saturates it, so the capacities that fill layers (this one and the
        // capillary rise below) are taken a relative 1e-6 short of the FP32 figure (its error is
        // below 2e-7).
        const float cap_short = 1.0f - 1e-6f;
        float excess = 0.0f;
        wfu::static_for<MAXN, 0, -1>([&](auto kc) {
            constexpr int k = decltype(kc)::value;
            if (k > g.nu) return;
            excess = fmaxf(0.0f, us[k - 1].val() - g.thick[k - 1] * te * cap_short);
            us[k - 1].add(-excess);
            if constexpr (k > 1) us[k - 2].add(excess);
        });
        const ff act_infilt = wff::sub(infil, wff::mul(inv_dt, excess));
        const ff satex = wff::sub(wff::sub(wfs_soil, act_infilt), infex);
        usd = 0.0f;
        wfu::static_for<0, MAXN, 1>([&](auto kc) {
            constexpr int k = decltype(kc)::value;
            if (k < g.nl) usd += us[k].val();
        });
        ucap = p_swc - satf - usd;
        // capillary rise (soil.jl capillary_flux!)
        Store capacc;
        capacc.init({0.0f, 0.0f});
        if (g.nu > 0) {
            const float ksat = WF_KV_AT(zif, g.nu);
            const float maxcap = fmaxf(0.0f, fminf(fminf(fminf(ksat, actevap_f), ucap * inv_dtf), drain * inv_dtf));
            const float rd = p_rooting_depth;
            const float chmax = p_cap_hmax;
            float capflux = zif > rd ? maxcap * powj(1.0f - fminf(zif, chmax) / chmax, p_cap_n) : 0.0f;
            wfu::static_for<MAXN, 0, -1>([&](auto kc) {
                constexpr int k = decltype(kc)::value;
                if (k > g.nu) return;
                const float toadd =
                    fminf(capflux, fmaxf((g.thick[k - 1] * te * cap_short - us[k - 1].val()) * inv_dtf, 0.0f));
                us[k - 1].add_prod(toadd, dtf);
                capflux -= toadd;
                capacc.add(toadd);
            });
        }
        const ff capflux = wff::fast_two_sum(capacc.hi, capacc.lo);
        const float deepksat = WF_KV_AT(df, g.nl);
#undef WF_KV_AT
        const float leak_f = fmaxf(0.0f, fminf(p_max_leakage, fminf(drain * inv_dtf, deepksat)));
        const ff recharge = wff::sub(wff::sub(wff::sub(wff::sub(transfer, capflux), leak_f), act_sat_f), esat_f);
        const ff transpiration = wff::add(actevap, act_sat_f);
        const ff aet = wff::add(wff::add(wff::add(wff::add(soilevap, transpiration), ae_river_f), ae_land_f), ic);
        // ---- write back
        if (!F.gash && canopy.changed()) stm(F, CANOPY, e, canopy.value());
        if (F.snow && PHASE == VERT_ALL) {
            stm(F, SNOW, e, snow.value());
            stm(F, SNOW_WATER, e, sw.value());
            Mh[SWE][e] = swe_out;
        } else if (PHASE == VERT_SOIL && F.glacier) {
            stm(F, SNOW, e, snow.value());
        }
        Mh[TSOIL][e] = tsoil;
        wfu::static_for<0, MAXN, 1>([&](auto kc) {
            constexpr int k = decltype(kc)::value;
            if (k < g.N && us[k].changed()) {
                const ff v = us[k].value();
                F.LYf[LY_USLD][k][e] = v.hi;
                F.LYl[k][e] = v.lo;
            }
        });
        F.Mf[ZI][e] = zi;
        F.Mf[SSF_ZI][e] = zi;
        stm(F, RECHARGE, e, recharge);
        stm(F, NET_RUNOFF_RIVER, e, wff::sub(runoff_river, ae_river_f));
        stm(F, AET, e, aet);
        stm(F, LEAKAGE, e, wff::from_f(leak_f));
        stm(F, SATEX, e, satex);
        stm(F, INFEX, e, infex);
        stm(F, RUNOFF_LAND, e, runoff_land);
        stm(F, AE_LAND, e, wff::from_f(ae_land_f));
        if (PHASE == VERT_ALL) Mh[INTERCEPTION][e] = icf;
        Mh[TRANSPIRATION][e] = wff::to_f(transpiration);
        Mh[SOIL_EVAP][e] = wff::to_f(soilevap);
        Mh[ACT_INFILT][e] = wff::to_f(act_infilt);
        // storages at the start of the routing (overland and river balances)
        if (F.mass_balance) {
            stm(F, BO_PREV, e, VF(VS_OLST_H, VS_OLST_L));
            if (rs >= 0) str(F, BR_PREV, rs * M + m, ldr(F, RV_STORAGE, rs * M + m));
        }
        // terms of the subsurface solve that do not depend on the upstream discharge: the
        // double-FP32 recharge flux for the exact bookkeeping, FP32 inputs of the walker
        if (F.ssf_single) {
            ff flux = wff::mul(recharge, WS ? ff{W32[VW_AREA_HI], W32[VW_AREA_LO]} : lds(F, AREA, slot));  // recharge flux of the subsurface model
            if (zi >= d_soil) flux = wff::fmax0(flux);
            stm(F, SSF_QNET, e, flux);
            Mh[SSF_QNETF][e] = wff::to_f(flux);
            Mh[SSF_ZIF][e] = zif;
            float z = zif;
            if (kv_const && !(z < zexp)) z = zexp;
            const float cel = p_kh_ratio * kv0 * expf(-fsc * z) * p_slope / p_sy;
            const float cinv = 1.0f / cel;
            Mh[SSF_T2][e] = wff::to_f(VF(VS_SSFQ_H, VS_SSFQ_L)) * cinv;
            Mh[SSF_RDF][e] = 1.0f / (p_ssf_dtdx + cinv);
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
#undef VP

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

// q of upstream entry o (sub-stepped subsurface flow): the heavy child from the double-FP32
// discharge field, a light child from the published chain ends.
__device__ __forceinline__ bool upstream_q_ff(const WfDevGraph& g, const WfSweep& sw, FFRow q, int32_t o, int m, int s,
                                              uint32_t ep, int32_t* status, double& out) {
    const int32_t uc = g.up_chain[o];
    if (uc < 0) {
        out = (double)q[g.up_slot[o] * g.M + m];
        return true;
    }
    const int64_t fe = (int64_t)uc * g.M + m;
    if (!wfw::wait_epoch(&g.flags[fe], ep + sw.wait_offset, sw, status)) return false;
    out = __ldcg(&g.end_q[fe * g.s_cap + s]);
    return true;
}

template <int MAXN>
struct SsfSplitPhys {
    WfDevFields F;
    WfDevGraph g;
    WfSweep sw;

    // the heavy child's discharge is read from the double-FP32 field (hq is unused): this walker
    // runs one sub-step per launch (adaptive sub-steps), one lane per chain-member pair
    __device__ bool node(int64_t slot, int64_t e, int m, int s, uint32_t ep, int64_t chain, bool is_end,
                         double& /*hq*/) {
        const FFMem Mf{F};
        double* const* L = F.L;
        double dt_s;
        bool first, last;
        if (!wf_substep(sw, m, s, dt_s, first, last)) return true;
        const double area = L[AREA][slot];
        const double d = L[SOIL_THICKNESS][slot];
        double zi_ssf = Mf[SSF_ZI][e];
        double flux = Mf[RECHARGE][e] * area;
        if (zi_ssf >= d) flux = jmax(0.0, flux);
        const double q_net = flux;
        double qin = 0.0, tr = 0.0;
        for (int32_t o = g.up_ptr[slot]; o < g.up_ptr[slot + 1]; ++o) {
            double qu;
            if (!upstream_q_ff(g, sw, Mf[SSF_Q], o, m, s, ep, F.status, qu)) return false;
            const double fr = L[FRAC_TO_RIVER][g.up_slot[o]];
            qin += qu * (1.0 - fr);
            tr += qu * fr;
        }
        ColumnS<MAXN> col;
        col.load_static(F, slot);
        col.kv0 = F.Mh[KV0][e];
        col.f = F.Mh[FSCALE][e];
#pragma unroll
        for (int k = 0; k < MAXN; ++k) col.usld[k] = k < col.N ? FFUsld{F}[k][e] : 0.0;
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
                if (k < col.N) FFUsld{F}[k][e] = col.usld[k];
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
            for (int k = 0; k < MAXN; ++k) col.usld[k] = k < col.N ? FFUsld{F}[k][e] : 0.0;
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
// relative size (du/v)^2). Results below the reference's floor (u = QROOT) are raised to it, as
// the reference does.
//
// The floor discharge QROOT^5 is 9.999999999999968e-31, just below KIN_WAVE_MIN_FLOW, so a cell
// whose solve ended at the floor does not count as flowing in the Courant quantile of adaptive
// sub-stepping; a floored cell whose next solve stops at once (kw_node_ff) keeps
// pow(q, 0.2)^5 = 1.000000000000002e-30, just above it, and counts from then on. Both values
// are held exactly as double-FP32 pairs (the low parts are FP32 subnormals).
__device__ __forceinline__ wff::ff q_floor() { return {__uint_as_float(0x0da24260u), __uint_as_float(0x802287aeu)}; }
__device__ __forceinline__ wff::ff q_rest() { return {__uint_as_float(0x0da24260u), __uint_as_float(0x802287abu)}; }

__device__ __forceinline__ void kw_solve_ff(wff::ff cterm, wff::ff dt_dx, float alpha, float u_prev, wff::ff& u_out,
                                            wff::ff& q_out) {
    const float QR = (float)KIN_WAVE_MIN_FLOW_QROOT;
    const float floor_c = alpha * (QR * QR * QR);
    if (!(cterm.hi > floor_c)) {
        u_out = {QR, 0.0f};
        q_out = q_floor();
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
        q = q_floor();
    }
    u_out = u;
    q_out = q;
}

// One kinematic-wave node update (surface_process.jl:24-70) from the upstream inflow qin, the
// previous discharge qp (u = qp^0.2) and the lateral inflow ql. As in the reference: no flow at
// all gives Q = 0; a cell with flow whose residual at the previous u is already within the
// reference's absolute tolerance (|f| <= 1e-12) keeps its discharge (its Newton loop stops
// before the first update); otherwise the root of the solve. The solve is evaluated in every
// case and the early-stop test beside it, so that the test does not lengthen the chain's
// critical path.
//
// The early stop matters where a cell's discharge sits at or near the 1e-30 floor: it decides
// whether the cell counts in the Courant quantile of adaptive sub-stepping, so the adaptive
// sweeps apply it (ADAPT); with fixed sub-steps it changes discharges of about 1e-13 m3/s and
// below only, and the fixed sweeps skip it (as well as the per-member sub-step sizes) to keep
// their registers, and so their resident warps, at the fixed path's need. `DT` is float (fixed
// sub-step, exact in FP32) or wff::ff (adaptive sub-step).
__device__ __forceinline__ wff::ff mul_dt(wff::ff a, float dt) { return wff::mul(a, dt); }
__device__ __forceinline__ wff::ff mul_dt(wff::ff a, wff::ff dt) { return wff::mul(a, dt); }

template <bool ADAPT, class DT>
__device__ __forceinline__ void kw_node_ff(wff::ff qin, wff::ff qp, wff::ff ql, wff::ff u, wff::ff inv_dx, DT dt_s,
                                           float alpha, wff::ff& un, wff::ff& qn) {
    if (!ADAPT && qin.hi == 0.0f && qp.hi == 0.0f && ql.hi == 0.0f) {
        un = {0.0f, 0.0f};
        qn = {0.0f, 0.0f};
        return;
    }
    const wff::ff dt_dx = mul_dt(inv_dx, dt_s);
    const wff::ff u3 = wff::mul(wff::mul(u, u), u);
    const wff::ff cterm = wff::add(wff::mul(dt_dx, qin), wff::add(wff::mul(u3, alpha), mul_dt(ql, dt_s)));
    kw_solve_ff(cterm, dt_dx, alpha, u.hi, un, qn);
    if (ADAPT) {
        const wff::ff f0 = wff::sub(wff::mul(dt_dx, wff::sub(qp, qin)), mul_dt(ql, dt_s));
        if (qp.hi > 0.0f && fabsf(f0.hi) <= 1.0e-12f) {
            const wff::ff fl = q_floor();
            un = u;
            qn = (qp.hi == fl.hi && qp.lo == fl.lo) ? q_rest() : qp;
        }
        if (qin.hi == 0.0f && qp.hi == 0.0f && ql.hi == 0.0f) {
            un = {0.0f, 0.0f};
            qn = {0.0f, 0.0f};
        }
    }
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
    const FFMem Mf{F};
    double* const* L = F.L;
    const double d = L[SOIL_THICKNESS][slot];
    const double zi_ssf = Mf[SSF_ZI][e];
    ColumnS<MAXN> col;
    col.load_static(F, slot);
    col.kv0 = F.Mh[KV0][e];
    col.f = F.Mh[FSCALE][e];
#pragma unroll
    for (int k = 0; k < MAXN; ++k) col.usld[k] = k < col.N ? FFUsld{F}[k][e] : 0.0;
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
        if (k < col.N) FFUsld{F}[k][e] = col.usld[k];
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
    static constexpr int kDepth = 1;  // the per-node inputs are many: one position ahead
    WfDevFields F;
    WfDevGraph g;
    WfSweep sw;
    struct In {
        float qnet, t2, rdf, zi, rth, rcap, rrho, qmaxdw, d, dtdx, idwdx, dtsy, k2;
        bool qprev_zero;
        wfv::UpRec up;
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
        x.qprev_zero = F.Mh[SSF_Q][e] == 0.0f;
        wfv::load_rec<true>(g, slot, x.up);
    }
    // the same inputs staged in shared memory (wfv::walk_ring)
    static constexpr int kSweep = 0;  // bit of WfLaunchCfg::walk_inputs
    static constexpr int kWords = 15;
    static constexpr bool kWeighted = true;
    __device__ __forceinline__ void sources(int64_t slot, int64_t e, const void** src) const {
        float* const* Mh = F.Mh;
        float* const* Lf = F.Lf;
        src[0] = &Mh[SSF_QNETF][e];
        src[1] = &Mh[SSF_T2][e];
        src[2] = &Mh[SSF_RDF][e];
        src[3] = &Mh[SSF_ZIF][e];
        src[4] = &Mh[SSF_RTH][e];
        src[5] = &Mh[SSF_RCAP][e];
        src[6] = &Mh[SSF_RRHO][e];
        src[7] = &Mh[Q_MAX][e];
        src[8] = &Lf[FLOW_WIDTH][slot];
        src[9] = &Lf[SOIL_THICKNESS][slot];
        src[10] = &Lf[SSF_DTDX][slot];
        src[11] = &Lf[SSF_IDWDX][slot];
        src[12] = &Lf[SSF_DTSY][slot];
        src[13] = &Lf[SSF_K2][slot];
        src[14] = &Mh[SSF_Q][e];
    }
    __device__ __forceinline__ void from_words(const uint32_t* w, int st, In& x) const {
        auto f = [&](int i) { return __uint_as_float(w[i * st]); };
        x.qnet = f(0);
        x.t2 = f(1);
        x.rdf = f(2);
        x.zi = f(3);
        x.rth = f(4);
        x.rcap = f(5);
        x.rrho = f(6);
        x.qmaxdw = f(7) * f(8);
        x.d = f(9);
        x.dtdx = f(10);
        x.idwdx = f(11);
        x.dtsy = f(12);
        x.k2 = f(13);
        x.qprev_zero = f(14) == 0.0f;
    }
    __device__ __forceinline__ bool node(const In& x, const wfv::Ends& ends, int64_t slot, int64_t e, int m,
                                         int64_t chain, bool is_end, bool heavy, unsigned long long* qh) {
        wff::ff qinff;
        if (!wfv::gather<true>(g, sw, x.up, ends, slot, m, 0, heavy, qh[0], F.status, qinff)) return false;
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
                const FFMem Mf{F};
                ssf_full_split<MAXN>(F, slot, e, qind, (double)Mf[SSF_QNET][e], sw.dts[0], qd, zid, exfd, nfd);
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

// The lateral inflow of river cell rs (element re) from the land cell of element le, with trsum
// the step's sum of the overland flow to the river (update_lateral_inflow!,
// surface_kinwave.jl:710-734): stores the river cell's inflow, lateral inflow and the lateral
// inflow with the external inflow, and returns the latter. One function for the overland
// wavefront and the per-cell completion kernel, so both give the same words.
__device__ __forceinline__ wff::ff river_lateral(const WfDevFields& F, int64_t le, int64_t rs, int64_t re,
                                                 wff::ff trsum) {
    using wff::ff;
    const ff tr_avg = wff::mul(trsum, ff{F.inv_dt_hi, F.inv_dt_lo});
    const ff inv_len = ldrs(F, R_INV_LENGTH, rs);
    const ff inw = wff::add(wff::add(ldm(F, SSF_TR_AVG, le), tr_avg),
                            wff::mul(ldm(F, NET_RUNOFF_RIVER, le), ldrs(F, R_AREA, rs)));
    str(F, RV_INWATER, re, inw);
    const ff qlat = wff::mul(inw, inv_len);
    str(F, RV_QLAT, re, qlat);
    const float ext = F.Rf[R_EXT_INFLOW][rs];
    const ff qlt = ext < 0.0f ? qlat : wff::add(qlat, wff::mul(inv_len, ext));
    F.RMh[RV_QLATTH][re] = qlt.hi;
    F.RMh[RV_QLATTL][re] = qlt.lo;
    return qlt;
}

// Overland flow (surface_process.jl:24-70 per node, routing/surface_kinwave.jl sub-steps) in
// double-FP32: discharge, u = Q^0.2 and the lateral inflow are pairs of FP32 arrays. ADAPT: one
// sub-step per launch of each member's own (adaptive) size.
// At the land cell of a river cell the walker also sums the upstream discharge that goes to the
// river (q of each upstream cell times its flow fraction to the river, times the sub-step;
// to_river_cumulative, surface_kinwave.jl:310-318), the only cells where it is not zero
// (get_flow_fraction_to_river, utils.jl:485-505). FUSE: a river wavefront shares the launch;
// after the step's last sub-step the walker publishes the river cell's lateral inflow for it
// (F.rv_lat_pub).
template <bool ADAPT, bool FUSE = false>
struct OlWave {
    static constexpr int kDepth = 2;
    WfDevFields F;
    WfDevGraph g;
    WfSweep sw;
    struct In {
        wff::ff u, q, qlat, invdx;
        float alpha;
        bool sfw_pos;
        int32_t rs;           // river slot of the cell, or -1
        float fr_hv, fr0, fr1;  // fractions to the river of the heavy child and light children 0, 1
        wfv::UpRec up;
    };
    __device__ __forceinline__ void load_river(int64_t slot, In& x) const {
        if (x.rs >= 0) {
            const float4 f = g.up_frec[slot];
            x.fr_hv = f.x;
            x.fr0 = f.y;
            x.fr1 = f.z;
        } else {
            x.fr_hv = x.fr0 = x.fr1 = 0.0f;
        }
    }
    __device__ __forceinline__ void load(int64_t slot, int64_t e, int m, In& x) const {
        float* const* Mh = F.Mh;
        x.u = {Mh[OL_UH][e], Mh[OL_UL][e]};
        x.q = ldm(F, OL_Q, e);
        x.qlat = ldm(F, OL_QLAT, e);
        x.invdx = {F.Lf[INV_FLOW_LENGTH][slot], F.Lf[INV_DX_LO][slot]};
        x.alpha = F.Lf[OL_ALPHA][slot];
        x.sfw_pos = F.Lf[SFW][slot] > 0.0f;
        x.rs = (int32_t)F.land_river_slot[slot];
        load_river(slot, x);
        wfv::load_rec<true>(g, slot, x.up);
    }
    // the same inputs staged in shared memory (wfv::walk_ring)
    static constexpr int kSweep = 1;
    static constexpr int kWords = 14;
    static constexpr bool kWeighted = true;
    __device__ __forceinline__ void sources(int64_t slot, int64_t e, const void** src) const {
        src[0] = &F.Mh[OL_UH][e];
        src[1] = &F.Mh[OL_UL][e];
        src[2] = &F.Mh[OL_Q][e];
        src[3] = &F.Ml[OL_Q][e];
        src[4] = &F.Mh[OL_QLAT][e];
        src[5] = &F.Ml[OL_QLAT][e];
        src[6] = &F.Lf[INV_FLOW_LENGTH][slot];
        src[7] = &F.Lf[INV_DX_LO][slot];
        src[8] = &F.Lf[OL_ALPHA][slot];
        src[9] = &F.Lf[SFW][slot];
        src[10] = &F.land_river_slot[slot];  // the low word (slots < 2^31; -1 stays -1)
        src[11] = &g.up_frec[slot].x;
        src[12] = &g.up_frec[slot].y;
        src[13] = &g.up_frec[slot].z;
    }
    __device__ __forceinline__ void from_words(const uint32_t* w, int st, In& x) const {
        auto f = [&](int i) { return __uint_as_float(w[i * st]); };
        x.u = {f(0), f(1)};
        x.q = {f(2), f(3)};
        x.qlat = {f(4), f(5)};
        x.invdx = {f(6), f(7)};
        x.alpha = f(8);
        x.sfw_pos = f(9) > 0.0f;
        x.rs = (int32_t)w[10 * st];
        x.fr_hv = f(11);
        x.fr0 = f(12);
        x.fr1 = f(13);
    }
    struct St {
        wff::ff u, qp, qsum, trsum;
        int32_t rs;
    };
    __device__ __forceinline__ void start(const In& x, St& st) const {
        st.u = x.u;
        st.qp = x.q;
        st.qsum = {0.0f, 0.0f};
        st.trsum = {0.0f, 0.0f};
        st.rs = x.rs;
    }
    // entry hook of the diagonal schedule (nothing to wait for)
    __device__ __forceinline__ bool enter(St&, int64_t) const { return true; }
    // gather_w<true> with, at the land cell of a river cell, the upstream flow to the river
    __device__ __forceinline__ bool gather_tr(const In& x, unsigned long long w0, unsigned long long w1, int64_t slot,
                                              int m, int s, bool heavy, unsigned long long qh, wff::ff& qin,
                                              wff::ff& tr) const {
        const wfv::UpRec& r = x.up;
        const bool riv = x.rs >= 0;
        wff::ff acc = {0.0f, 0.0f}, t = {0.0f, 0.0f};
        if (heavy) {
            const wff::ff q = wff::unpack(qh);
            acc = wff::mul(q, r.w_hv);
            if (riv) t = wff::mul(q, x.fr_hv);
        }
        if (r.lt0 >= 0) {
            const int64_t idx = wfv::end_index(g, r.lt0, m, s);
            unsigned long long first = w0;
            if (first == wfv::SENTINEL) first = wfv::ld_relaxed(&g.end_q[idx]);
            unsigned long long w;
            if (!wfv::await_end(g, sw, idx, first, F.status, w)) return false;
            const wff::ff q = wff::unpack(w);
            acc = wff::add(acc, wff::mul(q, r.w_lt0));
            if (riv) t = wff::add(t, wff::mul(q, x.fr0));
        }
        if (r.lt1 >= 0) {
            const int64_t idx = wfv::end_index(g, r.lt1, m, s);
            unsigned long long first = w1;
            if (first == wfv::SENTINEL) first = wfv::ld_relaxed(&g.end_q[idx]);
            unsigned long long w;
            if (!wfv::await_end(g, sw, idx, first, F.status, w)) return false;
            const wff::ff q = wff::unpack(w);
            acc = wff::add(acc, wff::mul(q, r.w_lt1));
            if (riv) t = wff::add(t, wff::mul(q, x.fr1));
        }
        if (r.n_lt > 2) {  // further light children, in up-list order after the first two
            int seen = 0;
            for (int32_t o = g.up_ptr[slot]; o < g.up_ptr[slot + 1]; ++o) {
                const int32_t uc = g.up_chain[o];
                if (uc < 0 || ++seen <= 2) continue;
                const int64_t idx = wfv::end_index(g, uc, m, s);
                unsigned long long w;
                if (!wfv::await_end(g, sw, idx, wfv::ld_relaxed(&g.end_q[idx]), F.status, w)) return false;
                const wff::ff q = wff::unpack(w);
                acc = wff::add(acc, wff::mul(q, g.up_wf[o]));
                if (riv) t = wff::add(t, wff::mul(q, g.up_frf[o]));
            }
        }
        qin = acc;
        tr = t;
        return true;
    }
    // sub-step s of the node
    __device__ __forceinline__ bool sub(const In& x, St& st, unsigned long long w0, unsigned long long w1,
                                        int64_t slot, int64_t e, int m, int s, int64_t chain, bool is_end, bool heavy,
                                        unsigned long long qh_in, unsigned long long& qh_out) const {
        using DT = typename std::conditional<ADAPT, wff::ff, float>::type;
        DT dt_s;
        if constexpr (ADAPT) dt_s = wff::ff{sw.adt_hi[m], sw.adt_lo[m]};
        else dt_s = sw.dts_f[s];
        wff::ff qin, tr;
        if (!gather_tr(x, w0, w1, slot, m, s, heavy, qh_in, qin, tr)) return false;
        if (!x.sfw_pos) qin = {0.0f, 0.0f};
        wff::ff un, qn;
        kw_node_ff<ADAPT>(qin, st.qp, x.qlat, st.u, x.invdx, dt_s, x.alpha, un, qn);
        st.u = un;
        st.qp = qn;
        qh_out = wff::pack(qn);
        if (is_end) wfv::publish(g, chain, m, s, qn);
        st.qsum = wff::add(st.qsum, mul_dt(qn, dt_s));
        if (x.rs >= 0) st.trsum = wff::add(st.trsum, mul_dt(tr, dt_s));
        return true;
    }
    // the node's state after the last sub-step of the launch (or of a round of the diagonal
    // schedule); add_stored: the step's cumulative discharge so far is added. At the land cell of
    // a river cell, the flow to the river goes to the river cell's element; with FUSE, after the
    // step's last sub-step, the river cell's lateral inflow is published.
    __device__ __forceinline__ void finish(const St& st, int64_t e, bool add_stored) const {
        float* const* Mh = F.Mh;
        Mh[OL_UH][e] = st.u.hi;
        Mh[OL_UL][e] = st.u.lo;
        stm(F, OL_Q, e, st.qp);
        wff::ff qsum = st.qsum;
        if (add_stored) qsum = wff::add(qsum, wff::ff{Mh[OL_QSUMH][e], Mh[OL_QSUML][e]});
        Mh[OL_QSUMH][e] = qsum.hi;
        Mh[OL_QSUML][e] = qsum.lo;
        if (st.rs >= 0) {
            const int m = (int)(e % F.M);
            const int64_t re = (int64_t)st.rs * F.M + m;
            wff::ff trsum = st.trsum;
            if (add_stored) trsum = wff::add(trsum, wff::ff{F.RMh[RV_TRSUMH][re], F.RMh[RV_TRSUML][re]});
            F.RMh[RV_TRSUMH][re] = trsum.hi;
            F.RMh[RV_TRSUML][re] = trsum.lo;
            if (FUSE && sw.last_of_step)
                wfv::st_relaxed(&F.rv_lat_pub[re], wff::pack(river_lateral(F, e, st.rs, re, trsum)));
        }
    }
    __device__ __forceinline__ bool node(const In& x, const wfv::Ends& ends, int64_t slot, int64_t e, int m,
                                         int64_t chain, bool is_end, bool heavy, unsigned long long* qh) {
        const int stride = blockDim.x;
        bool first = sw.first == 0;
        if (ADAPT) {
            const uint8_t f = sw.aflag[m];
            if (!(f & WF_SUB_ACTIVE)) return true;
            first = (f & WF_SUB_FIRST) != 0;
        }
        St st;
        start(x, st);
        for (int s = 0; s < sw.S; ++s) {
            unsigned long long out;
            if (!sub(x, st, wfv::end_word0(ends, s), s == 0 ? ends.lq1 : wfv::SENTINEL, slot, e, m, s, chain, is_end,
                     heavy, qh[s * stride], out))
                return false;
            qh[s * stride] = out;
        }
        finish(st, e, !first);
        return true;
    }
};

// River flow (surface_process.jl:24-70 per node, routing/river_kinwave.jl sub-steps) in
// double-FP32, with the abstraction of a negative external inflow limited to 80 % of the
// storage. ADAPT as for OlWave.
// RES: the model has reservoirs. At a reservoir cell the reservoir update follows the cell's
// kinematic wave in every sub-step (FP64, wf_reservoir.cuh) and the reservoir's outflow, not the
// cell's discharge, is handed downstream (heavy hand-off row and published chain end alike).
// FUSE: the overland wavefront shares the launch (its tickets first); a node takes its lateral
// inflow from the word the overland walker publishes at the river cell's land cell
// (F.rv_lat_pub), waiting for it like for a light child.
template <bool ADAPT, bool RES, bool FUSE = false>
struct RvWave {
    static constexpr int kDepth = 2;
    WfDevFields F;
    WfDevGraph g;
    WfSweep sw;
    struct In {
        wff::ff u, q, qlatt, invlen;
        float alpha, len, ext;
        int32_t res;  // reservoir at this cell (RES only), or -1
        wfv::UpRec up;
    };
    __device__ __forceinline__ void load(int64_t slot, int64_t e, int m, In& x) const {
        float* const* RMh = F.RMh;
        x.u = {RMh[RV_UH][e], RMh[RV_UL][e]};
        x.q = ldr(F, RV_Q, e);
        x.qlatt = {RMh[RV_QLATTH][e], RMh[RV_QLATTL][e]};
        x.invlen = {F.Rf[R_INV_LENGTH][slot], F.Rf[R_INV_LEN_LO][slot]};
        x.alpha = F.Rf[R_ALPHA][slot];
        x.len = F.Rf[R_LENGTH][slot];
        x.ext = F.Rf[R_EXT_INFLOW][slot];
        x.res = RES ? F.res_of_rslot[slot] : -1;
        wfv::load_rec<false>(g, slot, x.up);
    }
    // the same inputs staged in shared memory (wfv::walk_ring)
    static constexpr int kSweep = 2;
    static constexpr int kWords = 12;
    static constexpr bool kWeighted = false;
    __device__ __forceinline__ void sources(int64_t slot, int64_t e, const void** src) const {
        float* const* RMh = F.RMh;
        src[0] = &RMh[RV_UH][e];
        src[1] = &RMh[RV_UL][e];
        src[2] = &F.RMh[RV_Q][e];
        src[3] = &F.RMl[RV_Q][e];
        src[4] = &RMh[RV_QLATTH][e];
        src[5] = &RMh[RV_QLATTL][e];
        src[6] = &F.Rf[R_INV_LENGTH][slot];
        src[7] = &F.Rf[R_INV_LEN_LO][slot];
        src[8] = &F.Rf[R_ALPHA][slot];
        src[9] = &F.Rf[R_LENGTH][slot];
        src[10] = &F.Rf[R_EXT_INFLOW][slot];
        src[11] = RES ? (const void*)&F.res_of_rslot[slot] : (const void*)&F.Rf[R_ALPHA][slot];
    }
    __device__ __forceinline__ void from_words(const uint32_t* w, int st, In& x) const {
        auto f = [&](int i) { return __uint_as_float(w[i * st]); };
        x.u = {f(0), f(1)};
        x.q = {f(2), f(3)};
        x.qlatt = {f(4), f(5)};
        x.invlen = {f(6), f(7)};
        x.alpha = f(8);
        x.len = f(9);
        x.ext = f(10);
        x.res = RES ? (int32_t)w[11 * st] : -1;
    }
    struct St {
        wff::ff u, qp, qsum, asum, qlatt;
    };
    __device__ __forceinline__ void start(const In& x, St& st) const {
        st.u = x.u;
        st.qp = x.q;
        st.qsum = {0.0f, 0.0f};
        st.asum = {0.0f, 0.0f};
        st.qlatt = x.qlatt;
    }
    // FUSE: the lateral inflow the overland walker publishes for element e (entry hook of both
    // schedules); false when the wait ran out
    __device__ __forceinline__ bool enter(St& st, int64_t e) const {
        if (!FUSE) return true;
        unsigned long long w;
        if (!wfv::await_word(sw, &F.rv_lat_pub[e], F.status, w)) return false;
        st.qlatt = wff::unpack(w);
        return true;
    }
    // sub-step s of the node
    __device__ __forceinline__ bool sub(const In& x, St& st, unsigned long long w0, unsigned long long w1,
                                        int64_t slot, int64_t e, int m, int s, int64_t chain, bool is_end, bool heavy,
                                        unsigned long long qh_in, unsigned long long& qh_out) const {
        using DT = typename std::conditional<ADAPT, wff::ff, float>::type;
        DT dt_s;
        float dt_f;
        if constexpr (ADAPT) {
            dt_s = wff::ff{sw.adt_hi[m], sw.adt_lo[m]};
            dt_f = dt_s.hi;
        } else {
            dt_s = sw.dts_f[s];
            dt_f = dt_s;
        }
        wff::ff qin;
        if (!wfv::gather_w<false>(g, sw, x.up, w0, w1, slot, m, s, heavy, qh_in, F.status, qin)) return false;
        wff::ff ql = st.qlatt;
        if (x.ext < 0.0f) {  // abstraction: qlatt holds the lateral inflow alone
            const float storage = x.len * (x.alpha * (st.u.hi * st.u.hi * st.u.hi));
            const float absd = fminf(-x.ext, (storage / dt_f) * 0.80f);
            ql = wff::add(ql, wff::mul(x.invlen, -absd));
            st.asum = wff::add(st.asum, mul_dt(wff::ff{absd, 0.0f}, dt_s));
        }
        wff::ff un, qn;
        kw_node_ff<ADAPT>(qin, st.qp, ql, st.u, x.invlen, dt_s, x.alpha, un, qn);
        st.u = un;
        st.qp = qn;
        wff::ff q_down = qn;
        if (RES && x.res >= 0) {
            const double dt_d = ADAPT ? sw.adt[m] : sw.dts[s];
            q_down = wff::from_d(wfr::reservoir_node(F, x.res, m, wff::to_d(qn), dt_d));
        }
        qh_out = wff::pack(q_down);
        if (is_end) wfv::publish(g, chain, m, s, q_down);
        st.qsum = wff::add(st.qsum, mul_dt(qn, dt_s));
        return true;
    }
    // the node's state after the last sub-step of the launch (or of a round of the diagonal
    // schedule); add_stored: the step's cumulative discharge and abstraction so far are added
    __device__ __forceinline__ void finish(const St& st, int64_t e, bool add_stored) const {
        float* const* RMh = F.RMh;
        RMh[RV_UH][e] = st.u.hi;
        RMh[RV_UL][e] = st.u.lo;
        str(F, RV_Q, e, st.qp);
        wff::ff qsum = st.qsum, asum = st.asum;
        if (add_stored) {
            qsum = wff::add(qsum, wff::ff{RMh[RV_QSUMH][e], RMh[RV_QSUML][e]});
            asum = wff::add(asum, wff::ff{RMh[RV_ABSH][e], RMh[RV_ABSL][e]});
        }
        RMh[RV_QSUMH][e] = qsum.hi;
        RMh[RV_QSUML][e] = qsum.lo;
        RMh[RV_ABSH][e] = asum.hi;
        RMh[RV_ABSL][e] = asum.lo;
    }
    __device__ __forceinline__ bool node(const In& x, const wfv::Ends& ends, int64_t slot, int64_t e, int m,
                                         int64_t chain, bool is_end, bool heavy, unsigned long long* qh) {
        const int stride = blockDim.x;
        bool first = sw.first == 0;
        if (ADAPT) {
            const uint8_t f = sw.aflag[m];
            if (!(f & WF_SUB_ACTIVE)) return true;
            first = (f & WF_SUB_FIRST) != 0;
        }
        St st;
        start(x, st);
        if (!enter(st, e)) return false;
        for (int s = 0; s < sw.S; ++s) {
            unsigned long long out;
            if (!sub(x, st, wfv::end_word0(ends, s), s == 0 ? ends.lq1 : wfv::SENTINEL, slot, e, m, s, chain, is_end,
                     heavy, qh[s * stride], out))
                return false;
            qh[s * stride] = out;
        }
        finish(st, e, !first);
        return true;
    }
};

template <class Phys>
__global__ void __launch_bounds__(128) wave_kernel(Phys phys) {
    wfv::walk(phys.g, phys.sw, phys, phys.F.status);
}

template <class Phys>
__global__ void __launch_bounds__(128) wave_diag_kernel(Phys phys) {
    wfv::walk_diag(phys.g, phys.sw, phys, phys.F.status);
}

template <class Phys>
__global__ void __launch_bounds__(128) wave_ring_kernel(Phys phys) {
    wfv::walk_ring(phys.g, phys.sw, phys, phys.F.status);
}

// Node-major sweeps: inputs staged in shared memory (walk_ring) unless the tuning asks for the
// register pipeline (walk) for this sweep (bit Phys::kSweep of walk_inputs).
template <class Phys>
cudaError_t launch_wave(const Phys& phys, const WfLaunchCfg& c) {
    const int threads = 32 * (c.walk_warps > 0 ? c.walk_warps : 4);
    int blocks;
    Phys p = phys;
    p.sw.SL = 1;
    if (!((c.walk_inputs >> Phys::kSweep) & 1)) {
        const size_t smem = wfv::ring_smem(threads, phys.sw.S, Phys::kWords);
        cudaError_t err = cudaFuncSetAttribute(wave_ring_kernel<Phys>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)smem);
        if (err != cudaSuccess) return err;
        err = wave_grid(wave_ring_kernel<Phys>, threads, smem, c, p.g, blocks, p.sw.prio_items);
        if (err != cudaSuccess) return err;
        wave_ring_kernel<Phys><<<blocks, threads, smem, c.stream>>>(p);
        return cudaGetLastError();
    }
    const size_t smem = wfv::walk_smem(threads, phys.sw.S);
    cudaError_t err = wave_grid(wave_kernel<Phys>, threads, smem, c, p.g, blocks, p.sw.prio_items);
    if (err != cudaSuccess) return err;
    wave_kernel<Phys><<<blocks, threads, smem, c.stream>>>(p);
    return cudaGetLastError();
}

// Overland and river launches of several fixed sub-steps run on the diagonal schedule
// (wfv::walk_diag); one sub-step per launch (and the subsurface sweep) node-major.
template <class Phys>
cudaError_t launch_wave_sub(const Phys& phys, const WfLaunchCfg& c) {
    const int SL = wave_sub_lanes(phys.sw.S, c);
    if (phys.sw.aflag || SL <= 1) return launch_wave(phys, c);
    const int threads = 32 * (c.walk_warps > 0 ? c.walk_warps : 4);
    const size_t smem = wfv::diag_smem(threads);
    int blocks;
    Phys p = phys;
    p.sw.SL = SL;
    cudaError_t err = wave_grid(wave_diag_kernel<Phys>, threads, smem, c, p.g, blocks, p.sw.prio_items,
                                wf_items_per_chunk(p.g.G, p.g.M, SL));
    if (err != cudaSuccess) return err;
    wave_diag_kernel<Phys><<<blocks, threads, smem, c.stream>>>(p);
    return cudaGetLastError();
}

// --------------------------------------------------------------- post-sweep kernels ------

// After the subsurface sweep: the exact bookkeeping of the fast cases (net flux and
// water-table change from the walker's q, exfiltration), the unsaturated-layer adjustment to
// the new water table (soil.jl update_ustorelayerdepth!), averages, subsurface storage, the soil
// water storage update (sbm.jl update_soil_water_storage!) and the overland lateral inflow.
// Fluxes and the unsaturated stores are double-FP32; the water table and the saturated store
// are FP64 (large stores, see wf_split_fp64_member).
template <int MAXN>
__global__ void __launch_bounds__(256) ssf_post_kernel(WfDevFields F, WfDevGraph g) {
    using wff::ff;
    const int M = F.M;
    const int N = F.N;
    const int64_t E = F.land_slots * M;
    const float r_s = F.r_s;  // sub-step / step (1 when they are equal)
    const ff dts = wff::from_f((float)F.dt_ssf);
    const ff inv_dts = {F.inv_dts_hi, F.inv_dts_lo};
    const ff NANF = {__int_as_float(0x7fc00000), 0.0f};
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t slot = e / M;
        if (F.land_node_of_slot[slot] < 0) continue;
        const int m = (int)(e - slot * M);
        float* const* Mh = F.Mh;
        const int flag = (int)Mh[SSF_FLAG][e];
        const double zi_soil = F.Mf[ZI][e];
        const ff zis = wff::from_d(zi_soil);
        const ff d = lds(F, SOIL_THICKNESS, slot);
        const ff te = wff::sub(lds(F, THETA_S, slot), lds(F, THETA_R, slot));
        ff usld[MAXN], act[MAXN], cum[MAXN + 1];  // cum[k]: depth of the top of layer k
        cum[0] = {0.0f, 0.0f};
#pragma unroll
        for (int k = 0; k < MAXN; ++k) {
            usld[k] = k < N ? ff{F.LYf[LY_USLD][k][e], F.LYl[k][e]} : ff{0.0f, 0.0f};
            act[k] = k < N ? ff{F.LYf[LY_ACT_THICK][k][slot], F.LYsl[LY_ACT_THICK][k][slot]} : NANF;
            cum[k + 1] = k < N ? ff{F.LYf[LY_CUM][k][slot], F.LYsl[LY_CUM][k][slot]} : NANF;
        }
        // layer geometry (utils.jl set_layerthickness) on the double-FP32 pairs of the depths:
        // layer k is unsaturated iff the water table lies below its top
        auto nu_at = [&](ff ref) {
            int c = 0;
#pragma unroll
            for (int k = 0; k < MAXN; ++k)
                if (k < N && wff::gt(ref, cum[k])) ++c;
            return c;
        };
        auto thick_at = [&](ff ref, int k) {
            return wff::gt(ref, cum[k + 1]) ? act[k] : (wff::gt(ref, cum[k]) ? wff::sub(ref, cum[k]) : NANF);
        };
        ff q, qin, exf, nf;
        double zi_new, zi_s;
        ff zin, zss;  // double-FP32 copies of zi_new and zi_s
        if (flag == SSF_EARLY) {
            q = qin = exf = nf = {0.0f, 0.0f};
            zi_new = F.L[SOIL_THICKNESS][slot];
            zin = d;
            zi_s = zi_soil;
            zss = zis;
            stm(F, SSF_Q, e, q);
            F.Mf[SSF_ZI][e] = zi_new;
        } else if (flag == SSF_FULL) {
            q = ldm(F, SSF_Q, e);
            qin = ldm(F, SSF_TQIN, e);
            exf = ldm(F, SSF_TEXF, e);
            nf = ldm(F, SSF_TNF, e);
            zi_new = zi_s = F.Mf[SSF_ZI][e];
            zin = zss = wff::from_d(zi_new);
#pragma unroll
            for (int k = 0; k < MAXN; ++k) usld[k] = k < N ? ff{F.LYf[LY_USLD][k][e], F.LYl[k][e]} : ff{0.0f, 0.0f};
        } else {
            q = wff::from_f(Mh[SSF_QF][e]);
            qin = wff::from_f(Mh[SSF_QINF][e]);
            const float qu = Mh[SSF_QUF][e];
            nf = wff::mul(wff::sub(wff::add(ldm(F, SSF_QNET, e), qin), qu), lds(F, SSF_IDWDX, slot));
            // water_table_change (subsurface_process.jl): falling by net flux / specific yield,
            // rising through the unsaturated layers from the deepest up
            ff dh = {0.0f, 0.0f}, rem = nf;
            if (nf.hi <= 0.0f) {
                dh = wff::mul(nf, lds(F, SSF_DTSY, slot));
            } else {
                const int nu0 = nu_at(zis);
#pragma unroll
                for (int k = MAXN; k >= 1; --k) {
                    if (k > nu0 || rem.hi == 0.0f) continue;
                    const ff t = thick_at(zis, k - 1);
                    const ff cap = wff::mul(wff::fmax0(wff::sub(wff::mul(t, te), usld[k - 1])), inv_dts);
                    const ff fl = wff::fmin(rem, cap);
                    if (wff::le(cap, rem)) dh = wff::add(dh, t);
                    else dh = wff::add(dh, wff::div(wff::mul(fl, dts), wff::sub(te, wff::div(usld[k - 1], t))));
                    rem = wff::sub(rem, fl);
                }
            }
            exf = wff::fmax0(rem);
            // the water table itself is an FP64 store
            const double dmax = F.L[SOIL_THICKNESS][slot];
            double zi = zi_soil - wff::to_d(dh);
            if (flag == SSF_CUT || zi > dmax) zi = dmax;
            zi = fmax(zi, 0.0);
            zi_new = zi_s = zi;
            zin = zss = wff::from_d(zi);
            if (zi_new != zi_soil) {
                const int n_prev = nu_at(zis), n_new = nu_at(zin);
                if (zi_new < zi_soil) {
#pragma unroll
                    for (int k = 1; k <= MAXN; ++k) {
                        if (k < n_new || k > n_prev) continue;
                        const ff t = thick_at(zin, k - 1);
                        usld[k - 1] = t.hi != t.hi ? ff{0.0f, 0.0f} : wff::mul(wff::div(t, thick_at(zis, k - 1)), usld[k - 1]);
                        F.LYf[LY_USLD][k - 1][e] = usld[k - 1].hi;
                        F.LYl[k - 1][e] = usld[k - 1].lo;
                    }
                } else {
                    const ff tfc_tr = wff::sub(lds(F, THETA_FC, slot), lds(F, THETA_R, slot));
#pragma unroll
                    for (int k = 1; k <= MAXN; ++k) {
                        if (k < n_prev || k > n_new) continue;
                        ff tp = thick_at(zis, k - 1);
                        if (tp.hi != tp.hi) tp = {0.0f, 0.0f};
                        usld[k - 1] = wff::add(usld[k - 1], wff::mul(wff::sub(thick_at(zin, k - 1), tp), tfc_tr));
                        F.LYf[LY_USLD][k - 1][e] = usld[k - 1].hi;
                        F.LYl[k - 1][e] = usld[k - 1].lo;
                    }
                }
                F.Mf[ZI][e] = zi_new;
            }
            stm(F, SSF_Q, e, q);
            F.Mf[SSF_ZI][e] = zi_new;
        }
        const int nu = nu_at(zss);
        ff tr = {0.0f, 0.0f};
        for (int32_t o = g.up_ptr[slot]; o < g.up_ptr[slot + 1]; ++o)
            tr = wff::add(tr, wff::two_prod(Mh[SSF_QF][g.up_slot[o] * M + m], g.up_frf[o]));
        const ff area = lds(F, AREA, slot);
        const ff flux = ldm(F, SSF_QNET, e);
        stm(F, SSF_STORAGE, e, wff::mul(wff::mul(wff::sub(d, zin), F.Lf[SY][slot]), area));
        const ff exf_avg = wff::mul(exf, r_s);
        stm(F, RCH_FLUX_AVG, e, wff::mul(flux, r_s));
        stm(F, SSF_QIN_AVG, e, wff::mul(qin, r_s));
        stm(F, SSF_Q_AVG, e, wff::mul(q, r_s));
        stm(F, SSF_QNET_AVG, e, wff::mul(wff::mul(nf, area), r_s));
        stm(F, SSF_EXF_AVG, e, exf_avg);
        stm(F, SSF_TR_AVG, e, wff::mul(tr, r_s));
        ff usd = {0.0f, 0.0f};
#pragma unroll
        for (int k = 0; k < MAXN; ++k)
            if (k < nu) usd = wff::add(usd, usld[k]);
        const ff runoff = wff::fmax0(
            wff::add(wff::add(wff::add(exf_avg, ldm(F, SATEX, e)), ldm(F, RUNOFF_LAND, e)), ldm(F, INFEX, e)));
        // saturated store and total soil water: FP64 stores
        const double sat = (F.L[SOIL_THICKNESS][slot] - zi_s) * (F.L[THETA_S][slot] - F.L[THETA_R][slot]);
        F.Mf[SAT][e] = sat;
        stm(F, USTOREDEPTH, e, usd);
        F.Mf[TSWS][e] = sat + wff::to_d(usd);
        stm(F, EXFILT, e, exf_avg);
        stm(F, RUNOFF, e, runoff);
        const ff net_runoff = wff::sub(runoff, ldm(F, AE_LAND, e));
        stm(F, NET_RUNOFF, e, net_runoff);
        const ff inwater = wff::mul(net_runoff, area);
        stm(F, OL_INWATER, e, inwater);
        stm(F, OL_QLAT, e, wff::mul(inwater, lds(F, INV_FLOW_LENGTH, slot)));
    }
}

// After the overland sweep: water depth and storage from the double-FP32 state, averages, and
// the lateral inflow of the river cell of each land cell (routing/river_kinwave.jl
// update_lateral_inflow!).
__global__ void __launch_bounds__(256) ol_post_kernel(WfDevFields F, WfDevGraph g) {
    using wff::ff;
    const int M = F.M;
    const int64_t E = F.land_slots * M;
    const ff inv_dt = {F.inv_dt_hi, F.inv_dt_lo};
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t slot = e / M;
        if (F.land_node_of_slot[slot] < 0) continue;
        const int m = (int)(e - slot * M);
        float* const* Mh = F.Mh;
        const ff inv_sfw = lds(F, INV_SFW, slot);
        if (inv_sfw.hi > 0.0f) {
            const ff u = {Mh[OL_UH][e], Mh[OL_UL][e]};
            const ff a = wff::mul(wff::mul(wff::mul(u, u), u), F.Lf[OL_ALPHA][slot]);
            stm(F, OL_H, e, wff::mul(a, inv_sfw));
            stm(F, OL_STORAGE, e, wff::mul(a, lds(F, FLOW_LENGTH, slot)));
        }
        ff qin = {0.0f, 0.0f};
        for (int32_t o = g.up_ptr[slot]; o < g.up_ptr[slot + 1]; ++o) {
            const int64_t ue = g.up_slot[o] * M + m;
            const ff qs = {Mh[OL_QSUMH][ue], Mh[OL_QSUML][ue]};
            qin = wff::add(qin, wff::mul(qs, g.up_wf[o]));
        }
        if (!(inv_sfw.hi > 0.0f)) qin = {0.0f, 0.0f};
        stm(F, OL_Q_AVG, e, wff::mul(ff{Mh[OL_QSUMH][e], Mh[OL_QSUML][e]}, inv_dt));
        stm(F, OL_QIN_AVG, e, wff::mul(qin, inv_dt));
        // the flow to the river, summed by the wavefront at the land cells of river cells (zero
        // elsewhere), and the river cell's lateral inflow
        const int64_t rs = F.land_river_slot[slot];
        ff tr_avg = {0.0f, 0.0f};
        if (rs >= 0) {
            const int64_t re = rs * M + m;
            const ff trsum = {F.RMh[RV_TRSUMH][re], F.RMh[RV_TRSUML][re]};
            tr_avg = wff::mul(trsum, inv_dt);
            river_lateral(F, e, rs, re, trsum);
        }
        stm(F, OL_TR_AVG, e, tr_avg);
    }
}

// After the river sweep: water depth, storage and averages.
__global__ void __launch_bounds__(256) rv_post_kernel(WfDevFields F, WfDevGraph g) {
    using wff::ff;
    const int M = F.M;
    const int64_t E = F.river_slots * M;
    const ff inv_dt = {F.inv_dt_hi, F.inv_dt_lo};
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t slot = e / M;
        if (F.river_node_of_slot[slot] < 0) continue;
        const int m = (int)(e - slot * M);
        float* const* RMh = F.RMh;
        const ff u = {RMh[RV_UH][e], RMh[RV_UL][e]};
        const ff a = wff::mul(wff::mul(wff::mul(u, u), u), F.Rf[R_ALPHA][slot]);
        str(F, RV_H, e, wff::mul(a, ldrs(F, R_INV_WIDTH, slot)));
        str(F, RV_STORAGE, e, wff::mul(a, ldrs(F, R_LENGTH, slot)));
        ff qin = {0.0f, 0.0f};
        for (int32_t o = g.up_ptr[slot]; o < g.up_ptr[slot + 1]; ++o) {
            const int64_t us = g.up_slot[o];
            const int64_t ue = us * M + m;
            const int32_t ru = F.n_res > 0 ? F.res_of_rslot[us] : -1;
            // a reservoir cell contributes its reservoir's outflow (sum of outflow x sub-step)
            qin = wff::add(qin, ru >= 0 ? wff::from_d(F.RS[RS_DOWN_CUM][(int64_t)ru * M + m])
                                        : ff{RMh[RV_QSUMH][ue], RMh[RV_QSUML][ue]});
        }
        str(F, RV_Q_AVG, e, wff::mul(ff{RMh[RV_QSUMH][e], RMh[RV_QSUML][e]}, inv_dt));
        str(F, RV_QIN_AVG, e, wff::mul(qin, inv_dt));
        str(F, RV_ABS_AVG, e, wff::mul(ff{RMh[RV_ABSH][e], RMh[RV_ABSL][e]}, inv_dt));
    }
}

// Water balance of the split form (mass_balance.jl:215-253 land, :382-399 overland,
// :470-490 subsurface, :290-313 river) and update_total_water_storage! (sbm.jl:143-182), in
// double-FP32; relative errors are FP32 quotients.
__device__ __forceinline__ void mb_error_ff(wff::ff tin, wff::ff tout, wff::ff rate, wff::ff& err, wff::ff& rel) {
    err = wff::sub(wff::sub(tin, tout), rate);
    const float avg = (wff::to_f(tin) + wff::to_f(tout)) * 0.5f;
    rel = {avg == 0.0f ? 0.0f : __fdividef(wff::to_f(err), avg), 0.0f};
}

__global__ void __launch_bounds__(256, 4) balance_split_kernel(WfDevFields F) {
    using wff::ff;
    const int M = F.M;
    const int64_t EL = F.land_slots * M, ER = F.river_slots * M;
    const ff inv_dt = {F.inv_dt_hi, F.inv_dt_lo};
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < EL + ER; e += (int64_t)gridDim.x * blockDim.x) {
        ff err, rel;
        if (e >= EL) {
            if (!F.mass_balance) continue;
            const int64_t re = e - EL;
            const int64_t rs = re / M;
            if (F.river_node_of_slot[rs] < 0) continue;
            const ff tin = wff::add(wff::add(ldr(F, RV_INWATER, re), ldr(F, RV_QIN_AVG, re)),
                                    wff::fmax0(ldrs(F, R_EXT_INFLOW, rs)));
            const ff tout = wff::add(ldr(F, RV_Q_AVG, re), ldr(F, RV_ABS_AVG, re));
            mb_error_ff(tin, tout, wff::mul(wff::sub(ldr(F, RV_STORAGE, re), ldr(F, BR_PREV, re)), inv_dt), err, rel);
            str(F, BR_ERR, re, err);
            str(F, BR_REL, re, rel);
            continue;
        }
        const int64_t slot = e / M;
        if (F.land_node_of_slot[slot] < 0) continue;
        const int m = (int)(e - slot * M);
        const int64_t rs = F.land_river_slot[slot];
        const ff inv_area = lds(F, INV_AREA, slot);
        const ff snow = ldm(F, SNOW, e), sw = ldm(F, SNOW_WATER, e), canopy = ldm(F, CANOPY, e);
        const double tsws = F.Mf[TSWS][e];
        // glacier store x fraction (FP64, mass_balance.jl:96-113)
        const double glacier = F.glacier ? F.GM[GM_STORE][e] * F.G[G_FRAC][slot] : 0.0;
        ff ts = wff::add(wff::add(wff::add(snow, sw), canopy), wff::from_d(tsws + glacier));
        ts = wff::add(ts, wff::mul(ldm(F, OL_H, e), 1.0f - F.Lf[RIVER_FRACTION][slot]));
        if (rs >= 0)
            ts = wff::add(ts, wff::mul(wff::mul(wff::mul(ldr(F, RV_H, rs * M + m), ldrs(F, R_WIDTH, rs)),
                                                ldrs(F, R_LENGTH, rs)),
                                       inv_area));
        stm(F, TOTAL_STORAGE, e, ts);
        if (!F.mass_balance) continue;
        {
            ff tin = wff::add(wff::mul(ldm(F, SSF_QIN_AVG, e), inv_area), F.Mh[PRECIP][e]);
            const ff vout = wff::add(wff::add(wff::add(ldm(F, NET_RUNOFF, e), ldm(F, AET, e)),
                                              ldm(F, NET_RUNOFF_RIVER, e)),
                                     ldm(F, LEAKAGE, e));
            ff tout = wff::add(wff::mul(ldm(F, SSF_Q_AVG, e), inv_area), vout);
            if (F.snow_transport) {  // snow moved in and out (mass_balance.jl:236-244)
                tin = wff::add(tin, wff::from_d(F.GM[GM_SNOW_IN][e]));
                tout = wff::add(tout, wff::from_d(F.GM[GM_SNOW_OUT][e]));
            }
            const double ds =
                (tsws - F.Mf[BL_PREV][e]) + glacier + wff::to_d(wff::add(canopy, wff::add(snow, sw)));
            mb_error_ff(tin, tout, wff::mul(wff::from_d(ds), inv_dt), err, rel);
            stm(F, BL_ERR, e, err);
            stm(F, BL_REL, e, rel);
        }
        mb_error_ff(wff::add(ldm(F, OL_INWATER, e), ldm(F, OL_QIN_AVG, e)), ldm(F, OL_Q_AVG, e),
                    wff::mul(wff::sub(ldm(F, OL_STORAGE, e), ldm(F, BO_PREV, e)), inv_dt), err, rel);
        stm(F, BO_ERR, e, err);
        stm(F, BO_REL, e, rel);
        {
            const ff flux = ldm(F, RCH_FLUX_AVG, e);
            const ff fin = wff::fmax0(flux), fout = wff::fmax0(wff::neg(flux));
            mb_error_ff(wff::add(ldm(F, SSF_QIN_AVG, e), fin), wff::add(ldm(F, SSF_Q_AVG, e), fout),
                        ldm(F, SSF_QNET_AVG, e), err, rel);
            stm(F, BS_ERR, e, err);
            stm(F, BS_REL, e, rel);
        }
    }
}

// u = Q^0.2 of the overland and river discharges (after a discharge was set from outside,
// and at creation), in double-FP32 from an FP64 root.
__global__ void __launch_bounds__(256) sync_u_kernel(WfDevFields F) {
    const int M = F.M;
    const int64_t EL = F.land_slots * M, ER = F.river_slots * M;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < EL + ER; i += (int64_t)gridDim.x * blockDim.x) {
        if (i < EL) {
            const wff::ff uf = wff::from_d(u_of_q(wff::to_d(ldm(F, OL_Q, i))));
            F.Mh[OL_UH][i] = uf.hi;
            F.Mh[OL_UL][i] = uf.lo;
        } else {
            const int64_t e = i - EL;
            const wff::ff uf = wff::from_d(u_of_q(wff::to_d(ldr(F, RV_Q, e))));
            F.RMh[RV_UH][e] = uf.hi;
            F.RMh[RV_UL][e] = uf.lo;
        }
    }
}

// Volumetric water content of one layer after a step (soil.jl:1320-1342), split form.
__global__ void __launch_bounds__(256) vwc_split_kernel(WfDevFields F, int layer, double* out) {
    const int M = F.M;
    const int64_t E = F.land_slots * M;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t slot = e / M;
        if (F.land_node_of_slot[slot] < 0) continue;
        const double zi = F.Mf[ZI][e];
        const double top = layer == 0 ? 0.0 : F.LY[LY_CUM][layer - 1][slot];
        const double bot = F.LY[LY_CUM][layer][slot];
        const double act = F.LY[LY_ACT_THICK][layer][slot];
        const double ts = F.L[THETA_S][slot], tr = F.L[THETA_R][slot];
        double v = __longlong_as_double(0x7ff8000000000000LL);
        if (layer < F.nlayers[slot]) {
            if (zi > top) {
                const double thick = zi > bot ? act : zi - top;
                const double usld = (double)F.LYf[LY_USLD][layer][e] + (double)F.LYl[layer][e];
                v = (usld + (act - thick) * (ts - tr)) / act + tr;
            } else {
                v = ts;
            }
        }
        out[e] = v;
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
    p.sw.SL = 1;
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

namespace {
template <int MAXN, int PHASE, bool WS>
cudaError_t launch_vertical_split_n(const WfDevFields& F, int grid, int block, cudaStream_t st) {
    size_t smem = 2 * VStage<MAXN>::bytes_per_thread * block;
    if (WS) smem += (size_t)(block / 32) * 2 * VWarp<MAXN>::bytes;
    cudaError_t e = cudaFuncSetAttribute(vertical_split_kernel<MAXN, PHASE, WS>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    vertical_split_kernel<MAXN, PHASE, WS><<<grid, block, smem, st>>>(F);
    return cudaGetLastError();
}

template <int PHASE>
cudaError_t launch_vertical_split(const WfDevFields& F, const WfLaunchCfg& c) {
    const int block = c.vertical_block > 0 ? c.vertical_block : 256;
    // blocks per SM of the grid-stride loop (tuning; each thread walks E / (grid x block) elements)
    int grid = grid_for(F.land_slots * F.M, block, c.num_sms);
    if (c.vertical_blocks_per_sm > 0) grid = std::min(grid, c.num_sms * c.vertical_blocks_per_sm);
    // the cell's parameters once per warp when its members fill whole warps
    const bool ws = F.M % 32 == 0 && block % 32 == 0;
    if (F.N <= 4)
        return ws ? launch_vertical_split_n<4, PHASE, true>(F, grid, block, c.stream)
                  : launch_vertical_split_n<4, PHASE, false>(F, grid, block, c.stream);
    return ws ? launch_vertical_split_n<WF_MAX_LAYERS, PHASE, true>(F, grid, block, c.stream)
              : launch_vertical_split_n<WF_MAX_LAYERS, PHASE, false>(F, grid, block, c.stream);
}
}  // namespace

cudaError_t wf_split_vertical(const WfDevFields& F, const WfLaunchCfg& c) { return launch_vertical_split<VERT_ALL>(F, c); }
cudaError_t wf_split_vertical_snow(const WfDevFields& F, const WfLaunchCfg& c) {
    return launch_vertical_split<VERT_SNOW>(F, c);
}
cudaError_t wf_split_vertical_soil(const WfDevFields& F, const WfLaunchCfg& c) {
    return launch_vertical_split<VERT_SOIL>(F, c);
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
    if (sw.aflag) return launch_wave(OlWave<true>{F, g, sw}, c);
    return launch_wave_sub(OlWave<false>{F, g, sw}, c);
}

cudaError_t wf_split_river_wave(const WfDevFields& F, const WfDevGraph& g, const WfSweep& sw, const WfLaunchCfg& c) {
    if (F.n_res > 0) {
        if (sw.aflag) return launch_wave(RvWave<true, true>{F, g, sw}, c);
        return launch_wave_sub(RvWave<false, true>{F, g, sw}, c);
    }
    if (sw.aflag) return launch_wave(RvWave<true, false>{F, g, sw}, c);
    return launch_wave_sub(RvWave<false, false>{F, g, sw}, c);
}

namespace {
template <class PA, class PB>
__global__ void __launch_bounds__(128) wave_pair_kernel(PA pa, PB pb, int S_alloc) {
    wfv::walk_pair(pa, pb, S_alloc, pa.F.status);
}
template <class PA, class PB>
__global__ void __launch_bounds__(128) wave_pair_diag_kernel(PA pa, PB pb, int S_alloc, int64_t p_chunks, int SL) {
    wfv::walk_pair_diag(pa, pb, S_alloc, p_chunks, SL, pa.F.status);
}
}  // namespace

// The river's first-dispatched chunks run on the diagonal schedule when the river launch has
// several sub-steps and the tuning's sub-step lanes (wave_sub_lanes) give more than one lane per
// chain-member pair; the rest of both sweeps node-major.
cudaError_t wf_split_overland_river_wave(const WfDevFields& F, const WfDevGraph& gl, const WfSweep& swl,
                                         const WfDevGraph& gr, const WfSweep& swr, const WfLaunchCfg& c) {
    using PA = OlWave<false, true>;
    using PB = RvWave<false, false, true>;
    PA pa{F, gl, swl};
    PB pb{F, gr, swr};
    pa.sw.SL = 1;
    pb.sw.SL = 1;
    const int threads = 32 * (c.walk_warps > 0 ? c.walk_warps : 4);
    const int S_alloc = swl.S > swr.S ? swl.S : swr.S;
    const int SL = wave_sub_lanes(swr.S, c);
    int blocks_l, blocks_r;
    // a persistent launch gains nothing from blocks beyond those resident at once (the shared
    // launch holds more registers per thread than the separate sweeps the tuning was made for)
    WfLaunchCfg cp = c;
    cp.walk_blocks = 0;
    if (SL <= 1) {
        const size_t smem = wfv::walk_smem(threads, S_alloc);
        auto kernel = wave_pair_kernel<PA, PB>;
        int per_sm = 0;
        cudaError_t err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
        if (err != cudaSuccess) return err;
        if (c.walk_blocks > 0) cp.walk_blocks = std::min(c.walk_blocks, c.num_sms * std::max(per_sm, 1));
        err = wave_grid(kernel, threads, smem, cp, gl, blocks_l, pa.sw.prio_items);
        if (err != cudaSuccess) return err;
        err = wave_grid(kernel, threads, smem, cp, gr, blocks_r, pb.sw.prio_items);
        if (err != cudaSuccess) return err;
        kernel<<<blocks_l > blocks_r ? blocks_l : blocks_r, threads, smem, c.stream>>>(pa, pb, S_alloc);
        return cudaGetLastError();
    }
    const size_t smem = wfv::pair_diag_smem(threads, S_alloc);
    auto kernel = wave_pair_diag_kernel<PA, PB>;
    int64_t prio_r;
    cudaError_t err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    int per_sm = 0;
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
    if (err != cudaSuccess) return err;
    if (c.walk_blocks > 0) cp.walk_blocks = std::min(c.walk_blocks, c.num_sms * std::max(per_sm, 1));
    err = wave_grid(kernel, threads, smem, cp, gl, blocks_l, pa.sw.prio_items);
    if (err != cudaSuccess) return err;
    err = wave_grid(kernel, threads, smem, cp, gr, blocks_r, prio_r);
    if (err != cudaSuccess) return err;
    const int blocks = blocks_l > blocks_r ? blocks_l : blocks_r;
    // at most half of the resident warps hold first-dispatched river tickets (diagonal items and
    // node-major long chunks together), as in wave_grid
    const int64_t resident = (int64_t)std::min(blocks, c.num_sms * std::max(per_sm, 1)) * (threads / 32);
    const int64_t ipc_d = wf_items_per_chunk(gr.G, gr.M, SL);
    const int64_t gpc = gr.M > 32 ? gr.M / 32 : 1;
    const int64_t p_chunks = std::min<int64_t>(gr.n_long_chunks, (resident / 2) / ipc_d);
    pb.sw.prio_items = std::max<int64_t>(0, std::min<int64_t>((gr.n_long_chunks - p_chunks) * gpc,
                                                              resident / 2 - p_chunks * ipc_d));
    kernel<<<blocks, threads, smem, c.stream>>>(pa, pb, S_alloc, p_chunks, SL);
    return cudaGetLastError();
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

cudaError_t wf_split_vwc(const WfDevFields& F, int layer, double* out, const WfLaunchCfg& c) {
    vwc_split_kernel<<<grid_for(F.land_slots * F.M, 256, c.num_sms), 256, 0, c.stream>>>(F, layer, out);
    return cudaGetLastError();
}

cudaError_t wf_split_sync_u(const WfDevFields& F, const WfLaunchCfg& c) {
    sync_u_kernel<<<grid_for((F.land_slots + F.river_slots) * F.M, 256, c.num_sms), 256, 0, c.stream>>>(F);
    return cudaGetLastError();
}
