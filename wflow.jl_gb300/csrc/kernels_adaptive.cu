// kernels_adaptive.cu -- adaptive (Courant) sub-step sizes of the kinematic-wave sweeps.
//
// Overland and river flow (routing/surface/surface_kinwave.jl:674-704, stable_timestep): every
// cell with Q > 1e-30 has the Courant time dx / c with celerity c = 1 / (alpha beta Q^(beta-1));
// the sub-step is the type-7 quantile (Statistics.jl quantile!) of these times, p = 0.02 over
// land cells and 0.05 over river cells, the single time when only one cell has flow, and 600 s
// when no cell has. Lateral subsurface flow (routing/subsurface/lateral_subsurface_flow.jl:
// 314-344): the minimum of dx / celerity over the cells whose water table lies below the
// surface (zi > 0), 0.5 when there is none, times the alpha coefficient. Each sub-step is
// clamped to the end of the model step (check_timestepsize, routing/timestepping.jl:11-16).
// Members advance independently, each as its own model would.
//
// The quantile is an exact selection of two order statistics (ranks j-1 and j of the type-7
// definition) by radix select over the bit patterns of the Courant times, which are positive
// and so order like their values: 8-bit digits from the most significant, one histogram pass
// per digit (8 passes over the FP64 form's double keys, 4 over the split form's float keys).
// A pass histograms the keys that match the digits chosen so far into shared memory (warp-
// aggregated increments, since the keys of one member crowd into few bins), flushes it to a
// global histogram, and the last block to finish (block counter, no block ever waits) picks the
// digit holding each rank. The pass that computes the keys also takes the first histogram.
//
// The FP64 form evaluates the Courant time and the quantile with the same operations as the
// reference (this unit is compiled without floating-point contraction, and pow is the project's
// exp(y log x) used on both sides), so the sub-step sequence is bit-identical; the split form
// evaluates the Courant times in FP32 and the quantile interpolation in FP64.
#include <cstdint>

#include "wf_fields.cuh"
#include "wf_kernels.h"
#include "wf_math.cuh"

namespace {

constexpr double KIN_WAVE_MIN_FLOW = 1e-30;  // routing/utils.jl:1
constexpr double BETA = 0.6;                 // surface_kinwave.jl:2
constexpr unsigned long long NO_KEY = ~0ULL;
constexpr int THREADS = 256;
constexpr int MAX_GROUP_MEMBERS = 32;  // members histogrammed by one block

__device__ __forceinline__ int group_members(int M) { return M < MAX_GROUP_MEMBERS ? M : MAX_GROUP_MEMBERS; }

// Courant time bit pattern of element e (slot, member m) of the land or river graph.
__device__ __forceinline__ unsigned long long courant_key(const WfDevFields& F, const WfAdaptive& A, int64_t slot,
                                                          int64_t e) {
    const bool river = A.kind == WF_ADAPT_RIVER;
    const int64_t node = river ? F.river_node_of_slot[slot] : F.land_node_of_slot[slot];
    if (node < 0) return NO_KEY;
    if (A.fp32_keys) {
        // the flow test on the double-FP32 discharge, which holds the floor values exactly
        const float q = river ? F.RMh[RV_Q][e] : F.Mh[OL_Q][e];
        const float q_lo = river ? F.RMl[RV_Q][e] : F.Ml[OL_Q][e];
        if (!((double)q + (double)q_lo > KIN_WAVE_MIN_FLOW)) return NO_KEY;
        const float alpha = river ? F.Rf[R_ALPHA][slot] : F.Lf[OL_ALPHA][slot];
        const float dx = river ? F.Rf[R_LENGTH][slot] : F.Lf[FLOW_LENGTH][slot];
        const float c = 1.0f / (alpha * (float)BETA * powf(q, (float)BETA - 1.0f));
        return (unsigned long long)__float_as_uint(dx / c);
    }
    const double q = river ? F.RM[RV_Q][e] : F.Mf[OL_Q][e];
    if (!(q > KIN_WAVE_MIN_FLOW)) return NO_KEY;
    const double alpha = river ? F.R[R_ALPHA][slot] : F.L[OL_ALPHA][slot];
    const double dx = river ? F.R[R_LENGTH][slot] : F.L[FLOW_LENGTH][slot];
    const double c = 1.0 / (alpha * BETA * wfm::pow(q, (BETA - 1.0)));
    return wfm::to_bits(dx / c);
}

__device__ __forceinline__ double key_value(unsigned long long k, int fp32) {
    return fp32 ? (double)__uint_as_float((uint32_t)k) : wfm::from_bits(k);
}

// Type-7 quantile position for n values (Statistics.jl v1.11.1 _quantile with alpha = beta = 1):
// the 1-based index j and the weight gamma of the interpolation between v[j] and v[j+1].
__device__ __forceinline__ void quantile_position(int64_t n, double p, int64_t& j, double& gamma) {
    const double m = 1.0 + p * (1.0 - 1.0 - 1.0);
    const double aleph = fma((double)n, p, m);
    j = (int64_t)wfm::trunc_(aleph);
    if (j < 1) j = 1;
    if (j > n - 1) j = n - 1;
    gamma = wfm::jclamp(aleph - (double)j, 0.0, 1.0);
}

__device__ __forceinline__ double quantile_value(double a, double b, double gamma) {
    const bool approx = wfm::fabs_(a - b) <= 1.4901161193847656e-8 * wfm::jmax(wfm::fabs_(a), wfm::fabs_(b));
    if (isfinite(a) && isfinite(b) && approx) return a + gamma * (b - a);
    return (1.0 - gamma) * a + gamma * b;
}

// Digit d of 256 bins holding rank r (0-based), and the rank left within that bin; one warp.
// Returns false when the bins hold no more than r keys.
__device__ __forceinline__ bool warp_pick(const uint32_t* bins, long long r, int& digit, long long& r_left) {
    const int lane = threadIdx.x & 31;
    uint32_t c[8];
    long long local = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        c[i] = __ldcg(&bins[lane * 8 + i]);
        local += c[i];
    }
    long long incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    const unsigned hit = __ballot_sync(0xffffffffu, incl > r);
    if (!hit) return false;
    const int src = __ffs(hit) - 1;
    int d = 0;
    long long left = 0;
    if (lane == src) {
        long long cum = incl - local;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            if (cum + (long long)c[i] > r) {
                d = lane * 8 + i;
                left = r - cum;
                break;
            }
            cum += c[i];
        }
    }
    digit = __shfl_sync(0xffffffffu, d, src);
    r_left = __shfl_sync(0xffffffffu, left, src);
    return true;
}

// One radix-select pass. Pass 0 computes the keys of the current state and histograms their
// top digit; pass k > 0 histograms digit k of the keys matching the digits chosen so far, for
// each of the two order statistics. Grid: x over slots, y over groups of members.
__global__ void __launch_bounds__(THREADS) select_pass_kernel(WfDevFields F, WfAdaptive A, int pass) {
    extern __shared__ uint32_t sh[];  // [2][MG][256]
    const int M = A.M;
    const int MG = group_members(M);
    const int nbins = 2 * MG * 256;
    const int top = A.fp32_keys ? 24 : 56;
    const int shift = top - 8 * pass;
    for (int i = threadIdx.x; i < nbins; i += blockDim.x) sh[i] = 0;
    __syncthreads();
    const int m0 = blockIdx.y * MG;
    const int64_t total = A.n_slots * MG;
    const unsigned lane = threadIdx.x & 31u;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    // warp-uniform loop so that every lane takes part in the aggregation
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < total; base += stride) {
        const int64_t idx = base + lane;
        unsigned long long key = NO_KEY;
        int mm = 0;
        if (idx < total) {
            const int64_t slot = idx / MG;
            mm = (int)(idx - slot * MG);
            const int64_t e = slot * M + m0 + mm;
            if (pass == 0) {
                key = courant_key(F, A, slot, e);
                A.keys[e] = key;
            } else {
                key = __ldcg(&A.keys[e]);
            }
        }
        const int digit = (int)((key >> shift) & 0xFFu);
        for (int sel = 0; sel < (pass == 0 ? 1 : 2); ++sel) {
            bool match = key != NO_KEY;
            if (match && pass > 0) match = (key >> (shift + 8)) == A.prefix[sel * M + m0 + mm];
            const uint32_t bin = match ? (uint32_t)((sel * MG + mm) * 256 + digit) : 0xFFFFFFFFu;
            const unsigned peers = __match_any_sync(0xffffffffu, bin);
            if (match && (int)lane == __ffs(peers) - 1) atomicAdd(&sh[bin], (uint32_t)__popc(peers));
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nbins; i += blockDim.x) {
        const uint32_t v = sh[i];
        if (v) {
            const int sel = i / (MG * 256);
            const int rest = i - sel * MG * 256;
            const int mm = rest >> 8;
            atomicAdd(&A.hist[((int64_t)sel * M + m0 + mm) * 256 + (rest & 255)], v);
        }
    }
    // the last block to finish picks the digits
    __shared__ int last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(A.done, 1u) == gridDim.x * gridDim.y - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    for (int w = warp; w < 2 * M; w += nwarps) {
        const int sel = w / M;
        const int m = w - sel * M;
        const uint32_t* bins = A.hist + ((int64_t)(pass == 0 ? 0 : sel) * M + m) * 256;
        long long r;
        if (pass == 0) {
            // number of keys and the ranks of the two order statistics of the quantile
            long long n = 0;
            for (int i = (int)lane; i < 256; i += 32) n += __ldcg(&bins[i]);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
            r = 0;
            if (n > 1) {
                int64_t j;
                double gamma;
                quantile_position(n, A.p, j, gamma);
                r = sel == 0 ? j - 1 : j;
            }
            if (lane == 0 && sel == 0) A.count[m] = n;
        } else {
            r = A.rank[sel * M + m];
        }
        int d;
        long long left;
        const bool ok = warp_pick(bins, r, d, left);
        if (lane == 0 && ok) {
            const unsigned long long pre = pass == 0 ? 0ULL : A.prefix[sel * M + m];
            A.prefix[sel * M + m] = (pre << 8) | (unsigned long long)d;
            A.rank[sel * M + m] = left;
        }
    }
    __syncthreads();
    // clear the histograms for the next pass
    for (int64_t i = threadIdx.x; i < (int64_t)2 * M * 256; i += blockDim.x) A.hist[i] = 0;
    if (threadIdx.x == 0) *A.done = 0;
}

// Minimum Courant time of the subsurface flow per member (cells with zi > 0) and their number.
__global__ void __launch_bounds__(THREADS) ssf_min_kernel(WfDevFields F, WfAdaptive A) {
    __shared__ unsigned long long smin[MAX_GROUP_MEMBERS];
    __shared__ unsigned long long scnt[MAX_GROUP_MEMBERS];
    const int M = A.M;
    const int MG = group_members(M);
    for (int i = threadIdx.x; i < MG; i += blockDim.x) {
        smin[i] = NO_KEY;
        scnt[i] = 0;
    }
    __syncthreads();
    const int m0 = blockIdx.y * MG;
    const int64_t total = A.n_slots * MG;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t slot = idx / MG;
        const int mm = (int)(idx - slot * MG);
        if (F.land_node_of_slot[slot] < 0) continue;
        const int64_t e = slot * M + m0 + mm;
        const double zi = F.Mf[SSF_ZI][e];
        if (!(zi > 0.0)) continue;
        double cel;
        if (A.fp32_keys) {  // the split form's celerity (FP32 conductivity profile)
            float z = (float)zi;
            const float zexp = F.Lf[Z_EXP][slot];
            if (A.kv_profile == WF_KV_EXPONENTIAL_CONSTANT && !(z < zexp)) z = zexp;
            const float kh0 = F.Lf[KH_RATIO][slot] * F.Mh[KV0][e];
            cel = (double)(kh0 * expf(-F.Mh[FSCALE][e] * z) * (float)F.L[SLOPE][slot]) / F.L[SY][slot];
        } else {  // ssf_celerity (routing/subsurface/subsurface_process.jl:6-41)
            double z = zi;
            const double zexp = F.L[Z_EXP][slot];
            if (A.kv_profile == WF_KV_EXPONENTIAL_CONSTANT) z = zi < zexp ? zi : zexp;
            const double kh0 = F.L[KH_RATIO][slot] * F.Mf[KV0][e];
            cel = (kh0 * wfm::exp(-F.Mf[FSCALE][e] * z) * F.L[SLOPE][slot]) / F.L[SY][slot];
        }
        const double v = F.L[FLOW_LENGTH][slot] / cel;
        atomicMin(&smin[mm], wfm::to_bits(v));
        atomicAdd(&scnt[mm], 1ULL);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < MG; i += blockDim.x) {
        if (scnt[i]) {
            atomicMin(&A.minkey[m0 + i], smin[i]);
            atomicAdd((unsigned long long*)&A.count[m0 + i], scnt[i]);
        }
    }
}

// Size and flags of every member's next sub-step; one block.
__global__ void substep_kernel(WfAdaptive A) {
    __shared__ int more;
    if (threadIdx.x == 0) more = 0;
    __syncthreads();
    for (int m = threadIdx.x; m < A.M; m += blockDim.x) {
        const double t = A.t[m];
        uint8_t fl = 0;
        if (t < A.dt) {
            double ts;
            const long long n = A.count[m];
            if (A.kind == WF_ADAPT_SSF) {
                ts = (n > 0 ? wfm::from_bits(A.minkey[m]) : 0.5) * A.alpha;
            } else if (n == 0) {
                ts = 600.0;
            } else {
                const double a = key_value(A.prefix[m], A.fp32_keys);
                if (n == 1) {
                    ts = a;
                } else {
                    int64_t j;
                    double gamma;
                    quantile_position(n, A.p, j, gamma);
                    ts = quantile_value(a, key_value(A.prefix[A.M + m], A.fp32_keys), gamma);
                }
            }
            if (t + ts > A.dt) ts = A.dt - t;  // check_timestepsize
            const double tn = t + ts;
            fl = WF_SUB_ACTIVE;
            if (A.nsub[m] == 0) fl |= WF_SUB_FIRST;
            if (!(tn < A.dt)) fl |= WF_SUB_LAST;
            else more = 1;
            A.t[m] = tn;
            A.dt_s[m] = ts;
            const float hi = (float)ts;
            A.dt_hi[m] = hi;
            A.dt_lo[m] = (float)(ts - (double)hi);
            A.nsub[m] += 1;
            A.sig[m] += ts * ts;
        }
        A.flags[m] = fl;
        if (A.kind == WF_ADAPT_SSF) {
            A.minkey[m] = NO_KEY;
            A.count[m] = 0;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) *A.more = more;
}

}  // namespace

cudaError_t wf_adaptive_substep(const WfDevFields& F, const WfAdaptive& A, const WfLaunchCfg& c) {
    const int MG = A.M < MAX_GROUP_MEMBERS ? A.M : MAX_GROUP_MEMBERS;
    const int groups = A.M / MG;
    const int64_t per_group = A.n_slots * MG;
    int64_t bx = (per_group + THREADS * 8 - 1) / (THREADS * 8);
    const int64_t cap = (int64_t)4 * c.num_sms / groups > 0 ? (int64_t)4 * c.num_sms / groups : 1;
    if (bx > cap) bx = cap;
    if (bx < 1) bx = 1;
    const dim3 grid((unsigned)bx, (unsigned)groups);
    if (A.kind == WF_ADAPT_SSF) {
        ssf_min_kernel<<<grid, THREADS, 0, c.stream>>>(F, A);
    } else {
        const size_t smem = (size_t)2 * MG * 256 * sizeof(uint32_t);
        cudaError_t e = cudaFuncSetAttribute(select_pass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             2 * MAX_GROUP_MEMBERS * 256 * (int)sizeof(uint32_t));
        if (e != cudaSuccess) return e;
        const int passes = A.fp32_keys ? 4 : 8;
        for (int p = 0; p < passes; ++p) select_pass_kernel<<<grid, THREADS, smem, c.stream>>>(F, A, p);
    }
    const int threads = A.M < 1024 ? ((A.M + 31) / 32) * 32 : 1024;
    substep_kernel<<<1, threads, 0, c.stream>>>(A);
    return cudaGetLastError();
}
