// Device-side definitions shared by the placement kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ap {

typedef unsigned long long ull;

constexpr float kCoordScale = 65536.0f;                 // 2^16, coordinates
// WA gradient: each pin's contribution is rounded to 2^-24 in int32 (|g| is
// below 2 for a WA partial) and accumulated per node in int64
constexpr float kGradScale = 16777216.0f;               // 2^24
constexpr float kInvGradScale = 1.0f / 16777216.0f;
constexpr float kGradClamp = 127.0f;                    // keeps g * 2^24 inside int32
constexpr int kThreads = 256;

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
    double gamma;
    double hpwl, hpwl_prev, wa;      // accepted point
    double tau, tau_abs;             // accepted point
    double t_hpwl, t_wa, t_tau, t_tau_abs, t_du;  // last trial
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
};

// Bin geometry, identical to or_grid in the oracle.
struct Grid {
    int mx, my;
    float bw, bh;
    float small_threshold;
    float inv_ab;  // 1 / (bw_q * bh_q) in float, for gather weights
    long long bw_q, bh_q;
};

// Round-to-nearest conversion of v * 2^16 to an integer.  In int32 range the
// 32-bit conversion gives the same integer as the 64-bit one and stays off the
// FP64 pipe, which executes 64-bit integer conversions.
__device__ __forceinline__ long long to_q(float v) {
    const float s = __fmul_rn(v, kCoordScale);
    if (fabsf(s) < 2147483520.0f) return (long long)__float2int_rn(s);
    return __float2ll_rn(s);
}

// float of an int64 fixed-point value through two 32-bit conversions (within
// one ulp of the correctly rounded conversion)
__device__ __forceinline__ float i64_to_float(long long q) {
    return fmaf(__int2float_rn((int)(q >> 32)), 4294967296.0f, __uint2float_rn((unsigned)q));
}

// per-pin WA contribution in the int64 accumulators' fixed point
__device__ __forceinline__ ull grad_q(float g) {
    return (ull)(long long)__float2int_rn(fminf(fmaxf(g, -kGradClamp), kGradClamp) * kGradScale);
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
        c0 = c1 = __float2int_rz(qx);
        r0 = r1 = __float2int_rz(qy);
        return true;
    }
    if (!(qx > -1.0f) || !(qy > -1.0f)) return false;
    const float qx1 = __fdiv_rn(__fadd_rn(x, w), g.bw), qy1 = __fdiv_rn(__fadd_rn(y, h), g.bh);
    if (qx1 != qx1 || qy1 != qy1) return false;
    c0 = qx >= (float)g.mx ? g.mx : __float2int_rz(qx);
    r0 = qy >= (float)g.my ? g.my : __float2int_rz(qy);
    c1 = qx1 >= (float)g.mx ? g.mx - 1 : __float2int_rz(qx1);
    r1 = qy1 >= (float)g.my ? g.my - 1 : __float2int_rz(qy1);
    if (c1 > g.mx - 1) c1 = g.mx - 1;
    if (r1 > g.my - 1) r1 = g.my - 1;
    return c0 <= c1 && r0 <= r1;
}

__device__ __forceinline__ long long overlap_1d(long long lo_bin, long long span, long long lo, long long len) {
    const long long hi_bin = lo_bin + span, hi = lo + len;
    return (hi_bin < hi ? hi_bin : hi) - (lo_bin > lo ? lo_bin : lo);
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

// Last-block detection for grid-wide reductions without waiting: every block
// publishes its partials, the block that arrives last reduces them in block
// order (so the result does not depend on scheduling) and resets the counter.
__device__ __forceinline__ bool arrive_last(unsigned int *counter) {
    __shared__ bool last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned int t = atomicAdd(counter, 1u);
        last = (t == gridDim.x - 1);
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
