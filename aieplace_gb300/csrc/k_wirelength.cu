// Weighted-average wirelength gradient and HPWL over a net/pin CSR.
//
// Replaces Placer::computeAllPartials_CPU -> computeNetPartials_CPU ->
// compute_bc_terms_CPU -> compute_a_terms_CPU (vck5000/host/src/AIEplace.cpp:
// 574-673) and the AIE graph compute_abc + compute_partials
// (vck5000/aie/src/partials/compute_abc.cpp:23-125, compute_partials.cpp:
// 11-63).  Per net and axis the reference forms
//   a+_i = exp((x_i - x_max)/g), a-_i = exp((x_min - x_i)/g),
//   b+- = sum a+-, c+- = sum a+- x_i,
//   dWA/dx_i = ((1 + x_i/g) b+ - c+/g) a+_i / b+^2 - ((1 - x_i/g) b- + c-/g) a-_i / b-^2.
// The kernels evaluate the same expression in the algebraically equal
// shifted form
//   dWA/dx_i = a+_i/b+ (1 + (x_i - WA+)/g) - a-_i/b- (1 - (x_i - WA-)/g),
//   WA+ = x_max + sum a+ (x - x_max) / b+,  WA- = x_min + sum a- (x - x_min) / b-,
// which keeps FP32 exact where the reference form cancels (x_i/g ~ 1e4).
// Each pin's gradient is rounded to 2^-20 and accumulated per node in int64,
// so the sum over a node's nets is the same whatever order the atomics land in.
#include "ap_common.cuh"
#include "ap_kernels.h"

namespace ap {

namespace {

struct AxisTerms {
    float inv_bp, inv_bm, wp, wm;  // 1/b+, 1/b-, shifted WA+ - x_max, WA- - x_min
};

// Warp sums of 8 values at once (transposed butterfly): halving exchanges at
// offsets 16, 8, 4 leave lane L with a partial of quantity (L >> 2) & 7,
// offsets 2, 1 finish it, and 8 broadcasts hand every lane every total --
// 17 shuffles instead of 40.  Fixed order, so the same on every run.
__device__ __forceinline__ void warp_sum8(float v[8]) {
    const int lane = threadIdx.x & 31;
    const bool a = lane & 16, b = lane & 8, c = lane & 4;
    float u[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float send = a ? v[k] : v[k + 4];
        u[k] = (a ? v[k + 4] : v[k]) + __shfl_xor_sync(0xffffffffu, send, 16);
    }
    float t[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const float send = b ? u[k] : u[k + 2];
        t[k] = (b ? u[k + 2] : u[k]) + __shfl_xor_sync(0xffffffffu, send, 8);
    }
    float s = (c ? t[1] : t[0]) + __shfl_xor_sync(0xffffffffu, c ? t[0] : t[1], 4);
    s += __shfl_xor_sync(0xffffffffu, s, 2);
    s += __shfl_xor_sync(0xffffffffu, s, 1);
    // lane L holds quantity q = 4 a + 2 b + c = (L >> 2) & 7
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = __shfl_sync(0xffffffffu, s, 4 * q);
}

// Warp maxima of 4 values at once, the same scheme: 10 shuffles instead of 20.
__device__ __forceinline__ void warp_max4(float v[4]) {
    const int lane = threadIdx.x & 31;
    const bool a = lane & 16, b = lane & 8;
    float u[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const float send = a ? v[k] : v[k + 2];
        u[k] = fmaxf(a ? v[k + 2] : v[k], __shfl_xor_sync(0xffffffffu, send, 16));
    }
    float s = fmaxf(b ? u[1] : u[0], __shfl_xor_sync(0xffffffffu, b ? u[0] : u[1], 8));
    s = fmaxf(s, __shfl_xor_sync(0xffffffffu, s, 4));
    s = fmaxf(s, __shfl_xor_sync(0xffffffffu, s, 2));
    s = fmaxf(s, __shfl_xor_sync(0xffffffffu, s, 1));
    // lane L holds quantity q = 2 a + b = (L >> 3) & 3
#pragma unroll
    for (int q = 0; q < 4; ++q) v[q] = __shfl_sync(0xffffffffu, s, 8 * q);
}

// One net with d <= D pins held in registers by one thread.
template <int D>
__device__ __forceinline__ void net_thread(const int *__restrict__ pins, int d, const float *__restrict__ px,
                                           const float *__restrict__ py, float inv_g, ull *gqx, ull *gqy,
                                           int n_grad, float &hp_acc, float &wa_acc) {
    int node[D];
    float xs[D], ys[D];
    float xmx = -3.0e38f, xmn = 3.0e38f, ymx = -3.0e38f, ymn = 3.0e38f;
#pragma unroll
    for (int j = 0; j < D; ++j) {
        if (j < d) {
            node[j] = __ldg(pins + j);
            xs[j] = __ldg(px + node[j]);
            ys[j] = __ldg(py + node[j]);
            xmx = fmaxf(xmx, xs[j]);
            xmn = fminf(xmn, xs[j]);
            ymx = fmaxf(ymx, ys[j]);
            ymn = fminf(ymn, ys[j]);
        }
    }
    float gxs[D];
#pragma unroll
    for (int j = 0; j < D; ++j) gxs[j] = 0.f;
    float wa_net = 0.f;
#pragma unroll
    for (int axis = 0; axis < 2; ++axis) {
        const float cmx = axis ? ymx : xmx, cmn = axis ? ymn : xmn;
        float ep[D], em[D];
        float bp = 0.f, bm = 0.f, cp = 0.f, cm = 0.f;
#pragma unroll
        for (int j = 0; j < D; ++j) {
            if (j < d) {
                const float c = axis ? ys[j] : xs[j];
                const float dp = c - cmx, dm = c - cmn;
                ep[j] = __expf(dp * inv_g);
                em[j] = __expf(-dm * inv_g);
                bp += ep[j];
                bm += em[j];
                cp += ep[j] * dp;
                cm += em[j] * dm;
            }
        }
        const float ibp = 1.f / bp, ibm = 1.f / bm, wp = cp * ibp, wm = cm * ibm;
        wa_net += (cmx - cmn) + wp - wm;
#pragma unroll
        for (int j = 0; j < D; ++j) {
            if (j < d) {
                const float c = axis ? ys[j] : xs[j];
                const float g = ep[j] * ibp * (1.f + ((c - cmx) - wp) * inv_g) -
                                em[j] * ibm * (1.f - ((c - cmn) - wm) * inv_g);
                if (axis == 0) {
                    gxs[j] = g;
                } else if (node[j] < n_grad) {
                    atomicAdd(gqx + node[j], grad_q(gxs[j]));
                    atomicAdd(gqy + node[j], grad_q(g));
                }
            }
        }
    }
    hp_acc += (xmx - xmn) + (ymx - ymn);
    wa_acc += wa_net;
}

}  // namespace

// Bucket B (degree <= D) of the thread-per-net nets: registers sized for D.
template <int D, int B>
__global__ void __launch_bounds__(kThreads) wa_small_kernel(WaArgs a) {
    __shared__ double red[32];
    const float gamma = a.gamma > 0.f ? a.gamma : a.sc->f_gamma;
    const float inv_g = 1.f / gamma;
    const float *px = a.px, *py = a.py;
    if (a.mode == WA_LOOP) {
        const int t = 1 - a.sc->cur;
        px = a.pxs[t];
        py = a.pys[t];
    }
    // per-thread partials in FP32 (a thread owns a few nets), FP64 from the
    // block sum on: the FP64 pipe of this part is narrow
    float hpf = 0.f, waf = 0.f;
    const int hi = a.bucket_lo[B + 1];
    for (int e = a.bucket_lo[B] + blockIdx.x * blockDim.x + threadIdx.x; e < hi; e += gridDim.x * blockDim.x) {
        const int s = __ldg(a.net_ptr + e);
        const int d = __ldg(a.net_ptr + e + 1) - s;
        net_thread<D>(a.pin_node + s, d, px, py, inv_g, a.gqx, a.gqy, a.n_grad, hpf, waf);
    }
    // per-block partials in FP32 (folded with compensation by the last block
    // of the warp-per-net launch)
    const float hp = block_sum_ff(hpf, reinterpret_cast<float *>(red));
    const float wa = block_sum_ff(waf, reinterpret_cast<float *>(red));
    int off = 0;
#pragma unroll
    for (int b = 0; b < B; ++b) off += a.bucket_blocks[b];
    if (threadIdx.x == 0) {
        float *pf = reinterpret_cast<float *>(a.partials);
        pf[2 * (off + blockIdx.x)] = hp;
        pf[2 * (off + blockIdx.x) + 1] = wa;
    }
}

// Nets [n_small, n_nets): one warp per net, any degree.
__global__ void __launch_bounds__(kThreads) wa_large_kernel(WaArgs a) {
    __shared__ double red[32];
    const float gamma = a.gamma > 0.f ? a.gamma : a.sc->f_gamma;
    const float inv_g = 1.f / gamma;
    const float *px = a.px, *py = a.py;
    if (a.mode == WA_LOOP) {
        const int t = 1 - a.sc->cur;
        px = a.pxs[t];
        py = a.pys[t];
    }
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    // per-thread partials in FP32 (a thread owns a few nets), FP64 from the
    // block sum on: the FP64 pipe of this part is narrow
    float hpf = 0.f, waf = 0.f;
    for (int e = a.bucket_lo[3] + warp; e < a.bucket_lo[4]; e += nwarps) {
        const int s = __ldg(a.net_ptr + e), d = __ldg(a.net_ptr + e + 1) - s;
        if (d <= 64) {
            // pins lane and lane + 32 held in registers: one load pass, each
            // exponential evaluated once
            const bool v0 = lane < d, v1 = lane + 32 < d;
            const int n0 = v0 ? __ldg(a.pin_node + s + lane) : 0;
            const int n1 = v1 ? __ldg(a.pin_node + s + lane + 32) : 0;
            const float c0[2] = {v0 ? __ldg(px + n0) : 0.f, v0 ? __ldg(py + n0) : 0.f};
            const float c1[2] = {v1 ? __ldg(px + n1) : 0.f, v1 ? __ldg(py + n1) : 0.f};
            float mx[2], mn[2];
            {
                float m4[4];
#pragma unroll
                for (int ax = 0; ax < 2; ++ax) {
                    m4[ax] = fmaxf(v0 ? c0[ax] : -3.0e38f, v1 ? c1[ax] : -3.0e38f);
                    m4[2 + ax] = fmaxf(v0 ? -c0[ax] : -3.0e38f, v1 ? -c1[ax] : -3.0e38f);
                }
                warp_max4(m4);
#pragma unroll
                for (int ax = 0; ax < 2; ++ax) {
                    mx[ax] = m4[ax];
                    mn[ax] = -m4[2 + ax];
                }
            }
            float ep0[2], em0[2], ep1[2], em1[2], dp0[2], dm0[2], dp1[2], dm1[2], s8[8], gsum[2][2];
#pragma unroll
            for (int ax = 0; ax < 2; ++ax) {
                dp0[ax] = c0[ax] - mx[ax];
                dm0[ax] = c0[ax] - mn[ax];
                dp1[ax] = c1[ax] - mx[ax];
                dm1[ax] = c1[ax] - mn[ax];
                ep0[ax] = v0 ? __expf(dp0[ax] * inv_g) : 0.f;
                em0[ax] = v0 ? __expf(-dm0[ax] * inv_g) : 0.f;
                ep1[ax] = v1 ? __expf(dp1[ax] * inv_g) : 0.f;
                em1[ax] = v1 ? __expf(-dm1[ax] * inv_g) : 0.f;
                s8[4 * ax + 0] = ep0[ax] + ep1[ax];
                s8[4 * ax + 1] = em0[ax] + em1[ax];
                s8[4 * ax + 2] = ep0[ax] * dp0[ax] + ep1[ax] * dp1[ax];
                s8[4 * ax + 3] = em0[ax] * dm0[ax] + em1[ax] * dm1[ax];
            }
            warp_sum8(s8);
            float wa_net = 0.f;
#pragma unroll
            for (int ax = 0; ax < 2; ++ax) {
                const float ibp = 1.f / s8[4 * ax + 0], ibm = 1.f / s8[4 * ax + 1];
                const float wp = s8[4 * ax + 2] * ibp, wm = s8[4 * ax + 3] * ibm;
                gsum[ax][0] = ep0[ax] * ibp * (1.f + (dp0[ax] - wp) * inv_g) -
                              em0[ax] * ibm * (1.f - (dm0[ax] - wm) * inv_g);
                gsum[ax][1] = ep1[ax] * ibp * (1.f + (dp1[ax] - wp) * inv_g) -
                              em1[ax] * ibm * (1.f - (dm1[ax] - wm) * inv_g);
                wa_net += (mx[ax] - mn[ax]) + wp - wm;
            }
            if (v0 && n0 < a.n_grad) {
                atomicAdd(a.gqx + n0, grad_q(gsum[0][0]));
                atomicAdd(a.gqy + n0, grad_q(gsum[1][0]));
            }
            if (v1 && n1 < a.n_grad) {
                atomicAdd(a.gqx + n1, grad_q(gsum[0][1]));
                atomicAdd(a.gqy + n1, grad_q(gsum[1][1]));
            }
            if (lane == 0) {
                hpf += (mx[0] - mn[0]) + (mx[1] - mn[1]);
                waf += wa_net;
            }
            continue;
        }
        float xmx = -3.0e38f, xmn = 3.0e38f, ymx = -3.0e38f, ymn = 3.0e38f;
        for (int j = lane; j < d; j += 32) {
            const int n = __ldg(a.pin_node + s + j);
            const float x = __ldg(px + n), y = __ldg(py + n);
            xmx = fmaxf(xmx, x);
            xmn = fminf(xmn, x);
            ymx = fmaxf(ymx, y);
            ymn = fminf(ymn, y);
        }
        {
            float m4[4] = {xmx, ymx, -xmn, -ymn};
            warp_max4(m4);
            xmx = m4[0];
            ymx = m4[1];
            xmn = -m4[2];
            ymn = -m4[3];
        }
        float s8[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // bp bm cp cm for x then y
        for (int j = lane; j < d; j += 32) {
            const int n = __ldg(a.pin_node + s + j);
            const float c2[2] = {__ldg(px + n), __ldg(py + n)};
#pragma unroll
            for (int ax = 0; ax < 2; ++ax) {
                const float dp = c2[ax] - (ax ? ymx : xmx), dm = c2[ax] - (ax ? ymn : xmn);
                const float ep = __expf(dp * inv_g), em = __expf(-dm * inv_g);
                s8[4 * ax + 0] += ep;
                s8[4 * ax + 1] += em;
                s8[4 * ax + 2] += ep * dp;
                s8[4 * ax + 3] += em * dm;
            }
        }
        warp_sum8(s8);
        AxisTerms t[2];
#pragma unroll
        for (int ax = 0; ax < 2; ++ax) {
            t[ax].inv_bp = 1.f / s8[4 * ax + 0];
            t[ax].inv_bm = 1.f / s8[4 * ax + 1];
            t[ax].wp = s8[4 * ax + 2] * t[ax].inv_bp;
            t[ax].wm = s8[4 * ax + 3] * t[ax].inv_bm;
        }
        for (int j = lane; j < d; j += 32) {
            const int n = __ldg(a.pin_node + s + j);
            if (n >= a.n_grad) continue;
            const float c2[2] = {__ldg(px + n), __ldg(py + n)};
            float g[2];
#pragma unroll
            for (int ax = 0; ax < 2; ++ax) {
                const float dp = c2[ax] - (ax ? ymx : xmx), dm = c2[ax] - (ax ? ymn : xmn);
                const float ep = __expf(dp * inv_g), em = __expf(-dm * inv_g);
                g[ax] = ep * t[ax].inv_bp * (1.f + (dp - t[ax].wp) * inv_g) -
                        em * t[ax].inv_bm * (1.f - (dm - t[ax].wm) * inv_g);
            }
            atomicAdd(a.gqx + n, grad_q(g[0]));
            atomicAdd(a.gqy + n, grad_q(g[1]));
        }
        if (lane == 0) {
            hpf += (xmx - xmn) + (ymx - ymn);
            waf += ((xmx - xmn) + t[0].wp - t[0].wm) + ((ymx - ymn) + t[1].wp - t[1].wm);
        }
    }
    const float hp = block_sum_ff(hpf, reinterpret_cast<float *>(red));
    const float wa = block_sum_ff(waf, reinterpret_cast<float *>(red));
    float *pf = reinterpret_cast<float *>(a.partials);
    if (threadIdx.x == 0) {
        pf[2 * (a.small_blocks + blockIdx.x)] = hp;
        pf[2 * (a.small_blocks + blockIdx.x) + 1] = wa;
    }
    // the last block of this launch folds both launches' partials
    if (arrive_last(a.counter)) {
        const int nb = a.small_blocks + gridDim.x;
        const double h = block_sum_f(kahan_strided(pf, threadIdx.x, nb, blockDim.x, 2), red);
        const double w = block_sum_f(kahan_strided(pf + 1, threadIdx.x, nb, blockDim.x, 2), red);
        if (threadIdx.x == 0) {
            if (a.out) {
                a.out[0] = h;
                a.out[1] = w;
            }
            DevScalars *sc = a.sc;
            if (a.mode == WA_INIT) {
                sc->hpwl = h;
                sc->hpwl_prev = h;
                sc->wa = w;
            } else if (a.mode == WA_LOOP) {
                sc->t_hpwl = h;  // becomes the reported HPWL if the trial is accepted
                sc->t_wa = w;
            }
            *a.counter = 0u;
        }
    }
}

void launch_wirelength(const WaArgs &a0, cudaStream_t st) {
    WaArgs a = a0;
    auto grid = [](int items) {
        int b = (items + kThreads - 1) / kThreads;
        return b < 1 ? 1 : (b > kWaMaxBlocks ? kWaMaxBlocks : b);
    };
    for (int b = 0; b < 3; ++b) a.bucket_blocks[b] = grid(a.bucket_lo[b + 1] - a.bucket_lo[b]);
    a.bucket_blocks[3] = grid((a.bucket_lo[4] - a.bucket_lo[3]) * 32);
    a.small_blocks = a.bucket_blocks[0] + a.bucket_blocks[1] + a.bucket_blocks[2];
    wa_small_kernel<2, 0><<<a.bucket_blocks[0], kThreads, 0, st>>>(a);
    wa_small_kernel<4, 1><<<a.bucket_blocks[1], kThreads, 0, st>>>(a);
    wa_small_kernel<8, 2><<<a.bucket_blocks[2], kThreads, 0, st>>>(a);
    wa_large_kernel<<<a.bucket_blocks[3], kThreads, 0, st>>>(a);
}

}  // namespace ap
