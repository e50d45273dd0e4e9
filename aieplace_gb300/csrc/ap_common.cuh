// Device-side definitions shared by the placement kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ap {

typedef unsigned long long ull;

constexpr float kCoordScale = 65536.0f;                 // 2^16, coordinates
// WA gradient: each pin's contribution is rounded to 2^-20 (|g| is below 2
// for a WA partial) and accumulated per node in int64
constexpr float kGradScale = 1048576.0f;                // 2^20
constexpr float kInvGradScale = 1.0f / 1048576.0f;
constexpr float kGradClamp = 3.99f;                     // |g| 2^20 < 2^22: magic-number rounding is exact
constexpr double kLambdaMax = 1e30;                     // density penalty cap (the oracle's OR_LAMBDA_MAX)

// field source of a loop trial; launches gated on the mode run when
// (1 << mode) & mask
enum { kFieldExact = 0, kFieldSurr = 1, kFieldJudge = 2 };
constexpr int kGateExact = (1 << kFieldExact) | (1 << kFieldJudge);
constexpr int kGateSurr = (1 << kFieldSurr) | (1 << kFieldJudge);
constexpr int kGateJudge = 1 << kFieldJudge;
constexpr int kThreads = 256;

// One trial of the loop, as the trajectory log keeps it: written by the
// gather's last block into a ring in device memory, drained by the host
// whenever it reads the scalars (no synchronisation per iteration).
struct TrajRec {
    int eval;        // trial number (gradient evaluations before it)
    int iteration;   // accepted iterations after it
    int accepted;    // 1 accepted, 0 retried with a shorter step, -1 diverged
    int field_mode;  // kFieldExact / kFieldSurr / kFieldJudge
    double hpwl, overflow, overflow_abs, lambda, alpha, gamma;
    double surr_err;               // last judged surrogate field error
    unsigned long long t_ns;       // device clock (%globaltimer) at the trial's end
};

// FP64 scalars of the optimiser; live in device memory so a whole iteration
// runs without host round trips (and can be captured in a CUDA graph).
// Each launch of the iteration sequence is one trial step from the accepted
// state (buffers [cur]) into buffers [1 - cur]; the gather's last block
// accepts it (flips cur) or, when the re-predicted step is below 0.95 of the
// step tried, keeps the accepted state and retries with the new step.
struct DevScalars {
    double alpha;       // step length of the next trial
    double mom;         // (a_k - 1) / a_{k+1} for the current iteration
    double a_k;
    double a_next;      // a_{k+1} for the current iteration
    double lambda;
    // WA smoothing of the next evaluation.  A loop trial's WA uses gamma(tau)
    // of the previous evaluation (one-evaluation lag), so the WA launches do
    // not wait for the trial's own density: rho writes gamma_next, the
    // gather's last block makes it current.
    double gamma, gamma_next;
    double hpwl, hpwl_prev, wa;      // accepted point
    double tau, tau_abs;             // accepted point
    double t_hpwl, t_wa, t_tau, t_tau_abs, t_du;  // last trial
    double t_dv2;  // last trial: |v_trial - v_accepted|^2 (the position update's sum)
    double du_prev, tau_prev;        // restart tests
    double sum_dv2, sum_dg2, sum_gwl, sum_f;
    double gmax;
    // constants
    double ref_dh, mu_max, mu_min, gamma_base, init_density_weight, bin_avg;
    double mov_area_q;  // movable area in 2^-32 units
    int iteration;      // accepted iterations
    int evals;          // trials (gradient evaluations)
    int backtracks;     // retries of the current iteration
    int max_backtracks;
    int restart_mode;   // 0 none, 1 gradient, 2 always, 3 speed, 4 overflow rise
    int restarts;
    int cur;            // buffer index of the accepted state
    int status;
    // learned-surrogate schedule: the rho kernel's last block picks the field
    // source of each loop trial (kField*); the judge compares the surrogate
    // with the exact field and sets surr_ok
    int field_mode;
    int surr_attached, surr_ok, surr_judge_every;
    int surr_used, surr_judged, surr_fallbacks;
    float surr_tau_min, surr_err_bound;
    double surr_err;    // last judged relative field error
    // FP32 copies of alpha, mom, lambda, gamma for the per-thread kernels
    // (a double -> float conversion in every thread costs FP64-pipe time);
    // refreshed by publish_f32 wherever the doubles change on the device
    float f_alpha, f_mom, f_lambda, f_gamma;
    // trajectory log (null: off): record of trial e at traj[e % traj_cap]
    TrajRec *traj;
    int traj_cap;
};

__device__ __forceinline__ void publish_f32(DevScalars *sc) {
    sc->f_alpha = (float)sc->alpha;
    sc->f_mom = (float)sc->mom;
    sc->f_lambda = (float)sc->lambda;
    sc->f_gamma = (float)sc->gamma;
}

// Bin geometry, identical to or_grid in the oracle.
struct Grid {
    int mx, my;
    float bw, bh;
    float small_threshold;
    float inv_ab;  // 1 / (bw_q * bh_q) in float, for gather weights
    long long bw_q, bh_q;
};

// Integer <-> float conversions execute on the FP64 pipe, which is narrow on
// this part; the helpers below do them with integer and FMA-pipe arithmetic.

// Round-to-nearest-even of s to an integer for |s| < 2^31 (the same integer
// llrintf gives), in FMA-pipe and integer arithmetic without branches:
// adding M = 1.5 2^32 (whose binade has an ulp of 512) rounds s to 512 k,
// read off as the difference of the bit patterns; the remainder
// l = s - 512 k (|l| <= 256) is exact, and RNE(s) = 512 k + RNE(l) because
// 512 k is an even integer; RNE(l) by the 1.5 2^23 magic number.  The sum is
// formed in unsigned arithmetic (512 k can be 2^31 when s rounds to 2^31 - 128).
__device__ __forceinline__ int f2i_rn_bits(float s) {
    const float M = 6442450944.0f;  // 1.5 * 2^32
    const float t = __fadd_rn(s, M);
    const unsigned k = (unsigned)(__float_as_int(t) - __float_as_int(M));
    const float l = __fsub_rn(s, __fsub_rn(t, M));
    const unsigned r = (unsigned)(__float_as_int(__fadd_rn(l, 12582912.0f)) - 0x4B400000);
    return (int)(k * 512u + r);
}

// Truncation toward zero of s to an integer for |s| < 2^31 (= (int)s).
__device__ __forceinline__ int f2i_rz_bits(float s) {
    const unsigned b = __float_as_uint(s);
    const unsigned ex = (b >> 23) & 0xFFu;
    const unsigned m = (b & 0x7FFFFFu) | 0x800000u;
    const int e = (int)ex - 150;
    const unsigned r = e >= 0 ? m << e : (e < -23 ? 0u : m >> (unsigned)(-e));
    return (b >> 31) ? -(int)r : (int)r;
}

// Truncation toward zero for -1 < s < 2^23 (= (int)s there): s clamped at 0
// (truncation maps (-1, 0] to 0), then 2^23 added rounding toward zero, which
// drops the fraction and leaves the integer in the low mantissa bits.
__device__ __forceinline__ int f2i_rz_small(float s) {
    return __float_as_int(__fadd_rz(fmaxf(s, 0.0f), 8388608.0f)) - 0x4B000000;
}

// Round-to-nearest-even int64 -> float from integer arithmetic (= (float)v).
__device__ __forceinline__ float ll2f_rn_bits(long long v) {
    if (v == 0) return 0.0f;
    const unsigned sign = v < 0 ? 0x80000000u : 0u;
    const ull a = v < 0 ? 0ull - (ull)v : (ull)v;
    int msb = 63 - __clzll((long long)a);
    ull q;
    if (msb <= 23) {
        q = a << (23 - msb);
    } else {
        const int sh = msb - 23;
        q = a >> sh;
        const ull rem = a & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
        if (rem > half || (rem == half && (q & 1ull))) {
            q += 1ull;
            if (q == (1ull << 24)) {
                q >>= 1;
                msb += 1;
            }
        }
    }
    return __uint_as_float(sign | ((unsigned)(msb + 127) << 23) | ((unsigned)q & 0x7FFFFFu));
}

// Exact int -> float for |v| < 2^22 (magic-number addition).
__device__ __forceinline__ float i2f_small(int v) { return __int_as_float(v + 0x4B400000) - 12582912.0f; }

// Round-to-nearest of v * 2^16 to an integer, equal to llrintf(v * 65536).
__device__ __forceinline__ long long to_q(float v) {
    const float s = __fmul_rn(v, kCoordScale);
    if (fabsf(s) < 2147483520.0f) return (long long)f2i_rn_bits(s);
    return __float2ll_rn(s);
}

// float of an int64 fixed-point value, rounded to nearest (= (float)q):
// exact below 2^22 by the magic-number addition, in the int32 range by one
// FMA of two exact parts, else by integer arithmetic.  (Splitting q into 32-bit halves and converting each is not: for a small
// negative q the low word is close to 2^32, and its rounding to 24 bits is
// off by up to 256 units -- 2.4e-4 on a WA gradient below -4.)
__device__ __forceinline__ float i64_to_float(long long q) {
    if (q > -4194304ll && q < 4194304ll) return i2f_small((int)q);
    if (q >= -2147483647ll && q <= 2147483647ll) {
        // q = hi 2^12 + lo with |hi| < 2^19 and 0 <= lo < 2^12: both parts
        // are exact by the magic number, and the FMA rounds their exact sum once
        const int v = (int)q, hi = v >> 12, lo = v & 0xFFF;
        return fmaf(i2f_small(hi), 4096.0f, i2f_small(lo));
    }
    return ll2f_rn_bits(q);
}

// per-pin WA contribution in the int64 accumulators' fixed point: g 2^20
// rounded to nearest by the magic-number FMA (|g 2^20| < 2^22)
__device__ __forceinline__ int grad_q32(float g) {
    const float c = fminf(fmaxf(g, -kGradClamp), kGradClamp);
    return __float_as_int(fmaf(c, kGradScale, 12582912.0f)) - 0x4B400000;
}
__device__ __forceinline__ ull grad_q(float g) { return (ull)(long long)grad_q32(g); }

// Both axes of a node's WA gradient in one int64 accumulator, y 2^32 + x: the
// int64 sum is exact and order independent, and its halves decode exactly
// while |sum x| and |sum y| stay below 2^31 -- at most kPackMaxPins pins of
// |q| <= 3.99 2^20.  Nodes with more pins (flagged by the top bit of their
// pin_node entries) use one accumulator per axis.
constexpr int kPackMaxPins = 512;
constexpr int kPinHeavy = (int)0x80000000u;
constexpr int kPinNode = 0x7fffffff;
__device__ __forceinline__ ull pack_q(int qx, int qy) {
    return (ull)((long long)qy * 4294967296ll + (long long)qx);
}
__device__ __forceinline__ void unpack_q(ull p, long long &sx, long long &sy) {
    const int lo = (int)(unsigned)p;
    sx = lo;
    sy = ((long long)p - (long long)lo) >> 32;
}

// The bins a node touches under the reference rules (Grid.cpp:38-110,
// Node.h:100-104); exactly the arithmetic of or_density_q.  Returns false if
// the node adds nothing.
__device__ __forceinline__ bool bin_range(const Grid &g, float x, float y, float w, float h, int &c0,
                                          int &c1, int &r0, int &r1, bool &small) {
    const float area = __fmul_rn(w, h);
    if (!(area > 0.0f)) return false;
    small = !(area > g.small_threshold);
    const float qx = __fdiv_rn(x, g.bw), qy = __fdiv_rn(y, g.bh);
    if (small) {
        if (!(qx > -1.0f) || !(qx < (float)g.mx) || !(qy > -1.0f) || !(qy < (float)g.my)) return false;
        c0 = c1 = f2i_rz_small(qx);  // bin counts <= 4096: in range
        r0 = r1 = f2i_rz_small(qy);
        return true;
    }
    if (!(qx > -1.0f) || !(qy > -1.0f)) return false;
    const float qx1 = __fdiv_rn(__fadd_rn(x, w), g.bw), qy1 = __fdiv_rn(__fadd_rn(y, h), g.bh);
    if (qx1 != qx1 || qy1 != qy1) return false;
    // each conversion is taken only for -1 < q < bins <= 4096 (qx1 >= qx)
    c0 = qx >= (float)g.mx ? g.mx : f2i_rz_small(qx);
    r0 = qy >= (float)g.my ? g.my : f2i_rz_small(qy);
    c1 = qx1 >= (float)g.mx ? g.mx - 1 : f2i_rz_small(qx1);
    r1 = qy1 >= (float)g.my ? g.my - 1 : f2i_rz_small(qy1);
    if (c1 > g.mx - 1) c1 = g.mx - 1;
    if (r1 > g.my - 1) r1 = g.my - 1;
    return c0 <= c1 && r0 <= r1;
}

__device__ __forceinline__ long long overlap_1d(long long lo_bin, long long span, long long lo, long long len) {
    const long long hi_bin = lo_bin + span, hi = lo + len;
    return (hi_bin < hi ? hi_bin : hi) - (lo_bin > lo ? lo_bin : lo);
}

// The same integer in 32-bit arithmetic, for bin records, whose values and
// sums are checked to fit when the record is made
__device__ __forceinline__ int overlap_1d32(int lo_bin, int span, int lo, int len) {
    return min(lo_bin + span, lo + len) - max(lo_bin, lo);
}

// float of a non-negative 32-bit fixed-point value: exact below 2^22, else as
// i64_to_float
__device__ __forceinline__ float i32_to_float(int q) {
    return q < 4194304 ? i2f_small(q) : i64_to_float((long long)q);
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Deterministic block sum (fixed shuffle tree); result valid in thread 0.
template <typename T>
__device__ __forceinline__ T block_sum(T v, T *smem /* >= 32 */) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) smem[wid] = v;
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    v = threadIdx.x < nw ? smem[threadIdx.x] : T(0);
    if (wid == 0) v = warp_sum(v);
    __syncthreads();
    return v;
}

// Deterministic block sum of FP32 per-thread partials: warps reduce in FP32,
// the 32 warp sums in FP64 (only warp 0 touches the FP64 pipe).  Valid in
// thread 0.
__device__ __forceinline__ double block_sum_f(float v, double *smem /* >= 32 */) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) smem[wid] = (double)v;
    __syncthreads();
    double d = 0.0;
    if (wid == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        d = lane < nw ? smem[lane] : 0.0;
        d = warp_sum(d);
    }
    __syncthreads();
    return d;
}

// NV block sums entirely in FP32 with one barrier pair (each value in the
// same shuffle tree as block_sum_ff); valid in thread 0.  smem holds 32 * NV
// floats; the caller passes a barrier before reusing it.
template <int NV>
__device__ __forceinline__ void block_sums_ff(float (&v)[NV], float *smem) {
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = warp_sum(v[k]);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) smem[32 * k + wid] = v[k];
    }
    __syncthreads();
    if (wid == 0) {
        const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
        for (int k = 0; k < NV; ++k) v[k] = warp_sum(lane < nw ? smem[32 * k + lane] : 0.f);
    }
}

// Block sum entirely in FP32 (fixed shuffle tree); valid in thread 0.
__device__ __forceinline__ float block_sum_ff(float v, float *smem /* >= 32 */) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) smem[wid] = v;
    __syncthreads();
    if (wid == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        v = lane < nw ? smem[lane] : 0.f;
        v = warp_sum(v);
    }
    __syncthreads();
    return v;
}

// Compensated (Kahan) FP32 sum of partials[i0], partials[i0 + stride], ...
// over i < n, by one thread in a fixed order.
__device__ __forceinline__ float kahan_strided(const float *partials, int i0, int n, int stride, int step) {
    float s = 0.f, c = 0.f;
    for (int i = i0; i < n; i += stride) {
        const float y = __ldcg(partials + (size_t)i * step) - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    return s;
}

// One block of a launch: its index and the launch's block count.  A kernel
// body written against VBlock instead of blockIdx.x / gridDim.x runs both as
// a launch of its own (grid_block()) and as a work item of a persistent
// launch that executes the blocks of many such launches (the batched form).
struct VBlock {
    int id, n;
};
__device__ __forceinline__ VBlock grid_block() { return VBlock{(int)blockIdx.x, (int)gridDim.x}; }

// Last-block detection for grid-wide reductions without waiting: every block
// publishes its partials, the block that arrives last of `blocks` reduces
// them in block order (so the result does not depend on scheduling) and
// resets the counter.
__device__ __forceinline__ bool arrive_last(unsigned int *counter, int blocks) {
    __shared__ bool last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned int t = atomicAdd(counter, 1u);
        last = (t == (unsigned int)blocks - 1u);
    }
    __syncthreads();
    if (last) __threadfence();
    return last;
}

// Sum of partials[0..n) in a fixed order by one block.
template <typename T>
__device__ __forceinline__ T reduce_partials(const T *partials, int n, T *smem) {
    T acc = T(0);
    for (int i = threadIdx.x; i < n; i += blockDim.x) acc += __ldcg(partials + i);
    return block_sum(acc, smem);
}

}  // namespace ap
