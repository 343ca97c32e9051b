// wf_fields.cuh -- device field table of a model handle.
//
// Structure-of-arrays: one device array per field. Land fields are indexed in the wavefront
// slot layout (see wf_plan.h): static per-cell parameters by slot, member-specific
// parameters, forcing, states and outputs by element e = slot * M + m. River fields use the
// river graph's own slot layout. Padding slots exist in both layouts and are skipped by every
// kernel (node_of_slot < 0).
#pragma once

#include <cstdint>

#include <vector_types.h>

#include "wflow_gb300.h"

#define WF_L_FIELDS(X)                                                                             \
    X(AREA) X(FLOW_WIDTH) X(FLOW_LENGTH) X(SFW) X(SLOPE) X(FRAC_TO_RIVER) X(RIVER_FRACTION)          \
    X(WATER_FRACTION) X(TOP) X(OL_ALPHA) X(SY) X(GAP) X(CMAX) X(KC) X(E_R) X(DDF) X(TT) X(TTI) X(TTM) \
    X(WHC) X(THETA_S) X(THETA_R) X(THETA_FC) X(SWC) X(SOIL_THICKNESS) X(PSI_B) X(H1) X(H2) X(H3_HIGH) \
    X(H3_LOW) X(H4) X(ALPHA_H1) X(CAP_COMP) X(COMPACT_FRAC) X(ROOTDISTPAR) X(CAP_HMAX) X(CAP_N)       \
    X(MAX_LEAKAGE) X(W_SOIL) X(CF_SOIL) X(ROOTING_DEPTH) X(Z_EXP) X(KH_RATIO) X(INV_FLOW_LENGTH)  \
    X(SSF_DTDX) X(SSF_IDWDX) X(SSF_DTSY) X(SSF_K2) X(INV_TE) X(INV_AREA) X(INV_SFW) X(INV_DX_LO)

#define WF_M_FIELDS(X)                                                                             \
    X(KV0) X(FSCALE) X(Q_MAX) X(PRECIP) X(POTEVAP) X(TEMP) X(CANOPY) X(SNOW) X(SNOW_WATER) X(TSOIL) X(SAT) X(TSWS)    \
    X(USTOREDEPTH) X(ZI) X(SSF_ZI) X(SSF_Q) X(SSF_Q_AVG) X(SSF_QIN_AVG) X(SSF_TR_AVG) X(SSF_EXF_AVG) \
    X(SSF_QNET_AVG) X(RCH_FLUX_AVG) X(SSF_STORAGE) X(SSF_QIN_CUM) X(SSF_Q_CUM) X(SSF_TR_CUM)         \
    X(SSF_EXF_CUM) X(SSF_QNET_CUM) X(RCH_FLUX_CUM) X(OL_Q) X(OL_H) X(OL_STORAGE) X(OL_Q_AVG)          \
    X(OL_QIN_AVG) X(OL_TR_AVG) X(OL_INWATER) X(OL_QLAT) X(OL_Q_CUM) X(OL_QIN_CUM) X(OL_TR_CUM)       \
    X(RECHARGE) X(NET_RUNOFF_RIVER) X(AET) X(LEAKAGE) X(SATEX) X(INFEX) X(RUNOFF_LAND) X(AE_LAND)     \
    X(INTERCEPTION) X(TRANSPIRATION) X(SOIL_EVAP) X(ACT_INFILT) X(SWE) X(NET_RUNOFF) X(RUNOFF)        \
    X(EXFILT) X(BL_PREV) X(BO_PREV) X(TOTAL_STORAGE) X(BL_ERR) X(BL_REL) X(BO_ERR) X(BO_REL)          \
    X(BS_ERR) X(BS_REL)                                                                            \
    X(SSF_QNET) X(SSF_TQIN) X(SSF_TEXF) X(SSF_TNF)                                                 \
    X(SSF_T2) X(SSF_RDF) X(SSF_RTH) X(SSF_RCAP) X(SSF_RRHO) X(SSF_FLAG) X(SSF_QNETF) X(SSF_ZIF)      \
    X(SSF_QF) X(SSF_QUF) X(SSF_QINF) X(OL_UH) X(OL_UL) X(OL_QSUMH) X(OL_QSUML)

#define WF_R_FIELDS(X) X(R_WIDTH) X(R_LENGTH) X(R_ALPHA) X(R_EXT_INFLOW) X(R_AREA) X(R_INV_LENGTH) X(R_INV_WIDTH) X(R_INV_LEN_LO)

#define WF_RM_FIELDS(X)                                                                            \
    X(RV_Q) X(RV_H) X(RV_STORAGE) X(RV_Q_AVG) X(RV_QIN_AVG) X(RV_INWATER) X(RV_QLAT) X(RV_ABS_AVG)    \
    X(RV_Q_CUM) X(RV_QIN_CUM) X(RV_ABS_CUM) X(BR_PREV) X(BR_ERR) X(BR_REL)                         \
    X(RV_UH) X(RV_UL) X(RV_QSUMH) X(RV_QSUML) X(RV_ABSH) X(RV_ABSL) X(RV_QLATTH) X(RV_QLATTL)      \
    X(RV_TRSUMH) X(RV_TRSUML)

// Reservoirs, per reservoir and member (element r * M + m), FP64 in both forms. The first
// fifteen follow the order of the WF_F_RESERVOIR_* field ids (WF_F_RESERVOIR_STORAGE + i).
#define WF_RS_FIELDS(X)                                                                            \
    X(RS_STORAGE) X(RS_WATERLEVEL) X(RS_OUTFLOW) X(RS_OUT_AVG) X(RS_IN_AVG) X(RS_EVAP_AVG)          \
    X(RS_ABS_AVG) X(RS_IN_OL) X(RS_IN_SSF) X(RS_PRECIP) X(RS_EVAP) X(RS_EXT) X(RS_OBS) X(RS_ERR)     \
    X(RS_REL) X(RS_OUT_CUM) X(RS_IN_CUM) X(RS_EVAP_CUM) X(RS_ABS_CUM) X(RS_PREV) X(RS_DOWN_CUM)

// Reservoir parameters, per reservoir.
#define WF_RP_FIELDS(X)                                                                            \
    X(RP_AREA) X(RP_MAXSTOR) X(RP_THRESHOLD) X(RP_RC_COEF) X(RP_RC_EXP) X(RP_MAXREL) X(RP_DEMAND)   \
    X(RP_TMIN) X(RP_TFULL)

// Gravitational snow transport and the HBV glacier (FP64 in both forms; allocated only when the
// model runs them): per-slot glacier parameters, and per element the glacier store and melt, the
// snow moved in and out, and the terms the vertical kernel hands to the transport sweep and to
// its soil part (the snow runoff, the interception rate, the two transport capacities).
#define WF_G_FIELDS(X) X(G_FRAC) X(G_TTM) X(G_DDF) X(G_SIFRAC)
#define WF_GM_FIELDS(X)                                                                            \
    X(GM_STORE) X(GM_MELT) X(GM_SNOW_IN) X(GM_SNOW_OUT) X(GM_SRUNOFF) X(GM_IC) X(GM_CAP) X(GM_CAPW)

#define WF_ENUM_ITEM(name) name,
enum WfLandStatic { WF_L_FIELDS(WF_ENUM_ITEM) L_COUNT };
enum WfLandMember { WF_M_FIELDS(WF_ENUM_ITEM) M_COUNT };
enum WfRiverStatic { WF_R_FIELDS(WF_ENUM_ITEM) R_COUNT };
enum WfRiverMember { WF_RM_FIELDS(WF_ENUM_ITEM) RM_COUNT };
enum WfReservoirMember { WF_RS_FIELDS(WF_ENUM_ITEM) RS_COUNT };
enum WfReservoirStatic { WF_RP_FIELDS(WF_ENUM_ITEM) RP_COUNT };
enum WfGlacierStatic { WF_G_FIELDS(WF_ENUM_ITEM) G_COUNT };
enum WfSnowGlacierMember { WF_GM_FIELDS(WF_ENUM_ITEM) GM_COUNT };
#undef WF_ENUM_ITEM

// Layered fields: N arrays each.
// LY_CUM: depth of the bottom of each layer (cumulative thickness, static).
enum WfLayered { LY_ACT_THICK = 0, LY_C, LY_KVFRAC, LY_ROOTFRAC, LY_USLD, LY_CUM, LY_COUNT };

// Member fields kept in FP32 by the split form (pure diagnostics, forcing, parameters);
// every other member field (storages, balance terms, routing state) stays FP64.
__host__ __device__ inline bool wf_split_f32_member(int f) {
    return f == KV0 || f == FSCALE || f == Q_MAX || f == PRECIP || f == POTEVAP || f == TEMP || f == TSOIL ||
           f == INTERCEPTION || f == TRANSPIRATION || f == SOIL_EVAP || f == ACT_INFILT || f == SWE;
}

// Member fields only the split form's slim wavefronts use (not allocated by the FP64 form).
__host__ __device__ inline bool wf_split_only_member(int f) { return f >= SSF_QNET; }
__host__ __device__ inline bool wf_split_only_river_member(int f) { return f >= RV_UH; }
// Of those, the ones held only in FP32 (Mh / RMh): walker inputs and the double-FP32 routing
// state (pairs *H + *L).
__host__ __device__ inline bool wf_split_f32_only(int f) { return f >= SSF_T2; }
__host__ __device__ inline bool wf_split_f32_only_river(int f) { return f >= RV_UH; }
// Split form: the large stores stay FP64 (saturated depth, water-table depths, total soil
// water and the land balance's previous storage): a step changes them by as little as
// 1e-15 of their size in dry cells, below the double-FP32 resolution.
__host__ __device__ inline bool wf_split_fp64_member(int f) {
    return f == SAT || f == ZI || f == SSF_ZI || f == TSWS || f == BL_PREV;
}
// Split form: member fields held as double-FP32 pairs (every other field that is FP64 in the
// FP64 form and not one of the FP32 fields above).
__host__ __device__ inline bool wf_split_ff_member(int f) {
    return !wf_split_f32_member(f) && !wf_split_f32_only(f) && !wf_split_fp64_member(f);
}
__host__ __device__ inline bool wf_split_ff_river(int f) { return !wf_split_f32_only_river(f); }

struct WfDevFields {
    double* L[L_COUNT];
    double* Mf[M_COUNT];
    double* R[R_COUNT];
    double* RM[RM_COUNT];
    double* LY[LY_COUNT][WF_MAX_LAYERS];  // ACT_THICK/C/KVFRAC/ROOTFRAC by slot, USLD by element
    // split form only: FP32 copies of the static fields and the FP32 member fields
    float* Lf[L_COUNT];
    float* LYf[LY_COUNT][WF_MAX_LAYERS];
    float* Mh[M_COUNT];
    float* Rf[R_COUNT];
    float* RMh[RM_COUNT];
    // split form: the member fields that are FP64 in the FP64 form are double-FP32 pairs
    // (high part in Mh / RMh / LYf[LY_USLD], low part here); low parts of the static fields
    float* Ml[M_COUNT];
    float* RMl[RM_COUNT];
    float* LYl[WF_MAX_LAYERS];
    float* Ll[L_COUNT];
    float* Rl[R_COUNT];
    float* LYsl[LY_COUNT][WF_MAX_LAYERS];  // low parts of LY_ACT_THICK and LY_CUM
    float inv_dt_hi, inv_dt_lo;            // 1/dt as a double-FP32 pair
    float inv_dts_hi, inv_dts_lo;          // 1/dt_ssf as a double-FP32 pair
    float r_s;                             // dt_ssf / dt
    int32_t split;
    const int8_t* nlayers;                // [land slots]
    const int64_t* land_node_of_slot;     // [land slots], -1 padding
    const int64_t* land_river_slot;       // [land slots], river slot or -1
    const int64_t* river_node_of_slot;    // [river slots], -1 padding
    const int64_t* river_land_slot;       // [river slots], land slot of the river cell
    int64_t land_slots;
    int64_t river_slots;
    int32_t N;      // maximum_number_of_layers
    int32_t M;      // members
    int32_t snow;
    int32_t infilt_reduction;
    int32_t gash;
    int32_t kv_profile;
    int32_t mass_balance;
    int32_t ssf_single;   // split form: one subsurface sub-step per step (slim subsurface wavefront)
    double dt;
    double inv_dt;        // 1 / dt
    double dt_ssf;        // subsurface sub-step when ssf_single
    double inv_dt_ssf;    // 1 / dt_ssf
    int32_t* status;  // device status word (0 = ok)
    // reservoirs (none: n_res = 0 and null pointers)
    int64_t n_res;
    double* RS[RS_COUNT];          // [n_res * M]
    double* RP[RP_COUNT];          // [n_res]
    const int32_t* res_type;       // [n_res] WfReservoirOutflow
    const int64_t* res_land_slot;  // [n_res] land slot of the reservoir outlet cell
    const int32_t* res_of_rslot;   // [river slots] reservoir at a river slot, or -1
    // reservoir tables and links (null without them): storage profile (1 S = A H, 2 S-H table),
    // linked lower reservoir (-1 none), per reservoir {S-H start, rows, H-Q start, rows} into
    // res_tab, and the day of the year (1..365) whose H-Q column the rating curves read
    const int32_t* res_profile;    // [n_res]
    const int32_t* res_lower;      // [n_res]
    const int64_t* res_tab_meta;   // [4 n_res]
    const double* res_tab;
    const int32_t* res_hq_day;     // [1]
    // gravitational snow transport and glacier (off: flags 0 and null pointers)
    int32_t snow_transport;
    int32_t glacier;
    double g_max_rate;             // maximum snow-to-ice rate [m s-1]
    double* G[G_COUNT];            // [land slots]
    double* GM[GM_COUNT];          // [land slots * M]
    // local-inertial land and river routing in place of the kinematic waves (wf_li_couple.cuh):
    // the overland and river balances are the scheme's
    int32_t li_coupled;
    // split form: the lateral inflow of each river cell and member as a packed double-FP32
    // word, published by the overland wavefront for a river wavefront sharing its launch
    // (filled with the sentinel pattern before such a launch)
    unsigned long long* rv_lat_pub;  // [river slots * M]
};

// Routing graph on the device (one per land / river graph).
struct WfDevGraph {
    int64_t n_slots;
    int64_t n_chunks;
    int64_t n_chains;
    int64_t n_long_chunks;  // trailing chunks of the first-dispatched group (one chain each)
    int64_t n_short_chunks; // leading chunks of at most 8 positions (batched per work ticket)
    int32_t G;
    int32_t M;
    const int64_t* chunk_base;
    const int32_t* chunk_len;
    const int32_t* chunk_g;        // chains in each chunk (G, or 1 for a long chain)
    const int64_t* chunk_chain0;   // first chain of each chunk
    const int32_t* chain_len;
    const int32_t* up_ptr;
    const int64_t* up_slot;
    const int32_t* up_chain;
    const uint8_t* is_chain_end;
    const double* up_w;   // [up entries] weight of the upstream discharge (land: 1 - fraction to river)
    const double* up_fr;  // [up entries] fraction of the upstream discharge to the river (land only)
    const float* up_wf;   // FP32 copies of up_w / up_fr (split form)
    const float* up_frf;
    // per-slot upstream records of the split form's slim wavefronts (wf_wave.cuh UpRec):
    // {chain of light child 0, chain of light child 1, their weights as float bits}, the heavy
    // child's weight and the number of light children
    const int4* up_rec;
    const float* up_whv;
    const uint8_t* up_nlt;
    // land graph: per slot, the fractions to the river of the heavy child and of light children
    // 0 and 1 (up_frf of those entries; 0 where absent)
    const float4* up_frec;
    uint32_t* flags;      // [n_chains * M] epoch of the last published sub-step
    double* end_q;        // [n_chains * M * s_cap] q of each chain end per sub-step
    unsigned long long* ticket;  // work counter of the current launch
    int32_t s_cap;        // sub-steps per launch
    // land graph with snow transport: for each slot's upstream entries up_ptr[slot] ..
    // up_ptr[slot + 1], the entry indices in the order of the graph's topological sort (the
    // order in which the transport hands material on)
    const int32_t* snow_up;
};

// Work items per chunk of a wavefront launch with SL sub-step lanes per chain-member pair: a
// chunk holds G chains x M members (M <= 32) or one chain x M members, 32 / SL pairs per item.
__host__ __device__ __forceinline__ int64_t wf_items_per_chunk(int G, int M, int SL) {
    const int64_t pairs = M <= 32 ? (int64_t)G * M : M;
    const int64_t per_item = 32 / (SL > 1 ? SL : 1);
    return (pairs + per_item - 1) / per_item;
}

// Sub-stepping of one routing sweep launch.
struct WfSweep {
    int32_t S;            // sub-steps in this launch
    int32_t SL;           // sub-step lanes of the diagonal schedule (a power of two; 0 or 1: one lane)
    int32_t first;        // index of the first sub-step within the model step
    int32_t last_of_step; // 1 when the launch ends the model step's sub-stepping
    int32_t total;        // total sub-steps of the model step
    uint32_t epoch0;      // epoch of sub-step 0 of this launch
    double dt;            // model step
    const double* dts;    // [S] sub-step sizes (device)
    int64_t prio_items;   // work items dispatched first (the longest chains), set at launch
    float dts_f[16];      // FP32 copy of the first 16 sub-step sizes (split form's slim walkers)
    uint64_t wait_ns;     // spin-wait budget per wait [ns]
    uint32_t wait_offset; // test hook: added to awaited epochs (0 in production)
    // adaptive sub-stepping (one sub-step per launch, sizes per member); null for fixed steps
    const double* adt;    // [M] sub-step of each member
    const float* adt_hi;  // [M] the same as a double-FP32 pair (split form)
    const float* adt_lo;
    const uint8_t* aflag; // [M] WF_SUB_* bits
};

// Per-member flags of an adaptive sub-step
#define WF_SUB_ACTIVE 1  // the member takes this sub-step (it has not reached the end of the step)
#define WF_SUB_FIRST 2   // first sub-step of the model step
#define WF_SUB_LAST 4    // last sub-step of the model step

#ifdef __CUDACC__
// Sub-step s of a sweep launch for member m: its size and whether it is the first or the last of
// the model step. False when the member has already reached the end of the step (adaptive
// sub-steps end at different times for different members).
__device__ __forceinline__ bool wf_substep(const WfSweep& sw, int m, int s, double& dt_s, bool& first, bool& last) {
    if (sw.aflag) {
        const uint8_t f = sw.aflag[m];
        dt_s = sw.adt[m];
        first = (f & WF_SUB_FIRST) != 0;
        last = (f & WF_SUB_LAST) != 0;
        return (f & WF_SUB_ACTIVE) != 0;
    }
    dt_s = sw.dts[s];
    first = (sw.first + s == 0);
    last = sw.last_of_step && (s == sw.S - 1);
    return true;
}
#endif

// Adaptive (Courant) sub-step selection of one sweep kind: the Courant time of every cell, the
// order statistics of the quantile (or the minimum for the subsurface) per member, and each
// member's progress through the model step.
struct WfAdaptive {
    int32_t kind;           // WF_ADAPT_SSF, WF_ADAPT_LAND or WF_ADAPT_RIVER
    int32_t M;
    int32_t fp32_keys;      // keys are FP32 bit patterns (split form), else FP64
    int32_t kv_profile;
    double p;               // quantile probability (land 0.02, river 0.05)
    double dt;              // model step
    double alpha;           // subsurface stability coefficient
    int64_t n_slots;        // slots of the swept graph
    unsigned long long* keys;    // [n_slots * M] Courant time bit patterns, all ones for no value
    uint32_t* hist;         // [2][M][256] digit histogram of the current pass
    unsigned long long* prefix;  // [2][M] digits selected so far (then the two order statistics)
    long long* rank;        // [2][M] rank left to select within the prefix
    long long* count;       // [M] cells with a Courant time
    unsigned long long* minkey;  // [M] minimum (subsurface)
    uint32_t* done;         // blocks finished in the current pass
    double* t;              // [M] time reached within the model step
    double* dt_s;           // [M] current sub-step
    float* dt_hi;           // [M] double-FP32 copy
    float* dt_lo;
    uint8_t* flags;         // [M] WF_SUB_* bits of the current sub-step
    int32_t* nsub;          // [M] sub-steps taken in this model step
    double* sig;            // [M] sum of the squared sub-step sizes of this model step (a diagnostic)
    int32_t* more;          // 1 when some member has not reached the end of the step
};

#define WF_ADAPT_SSF 0
#define WF_ADAPT_LAND 1
#define WF_ADAPT_RIVER 2

// Device status codes (OR-ed bits)
#define WF_DEV_SPIN_TIMEOUT 1
#define WF_DEV_NONFINITE 2
