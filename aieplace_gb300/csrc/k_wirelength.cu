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
// so the sum over a node's nets is the same whatever order the atomics land in;
// both axes share one 64-bit atomic (pack_q) unless the node has more than
// kPackMaxPins pins.
#include <algorithm>

#include "ap_common.cuh"
#include "ap_kernels.h"

namespace ap {

namespace {

struct AxisTerms {
    float inv_bp, inv_bm, wp, wm;  // 1/b+, 1/b-, shifted WA+ - x_max, WA- - x_min
};

// 1/b for the sums b+- (1 <= b <= net degree: the extreme pin adds exp(0)):
// the 2-ulp reciprocal, well inside its range; IEEE division spent a dozen
// instructions and a branch per call here
__device__ __forceinline__ float rcp(float b) { return __fdividef(1.f, b); }

// one pin's gradient into its node's accumulators; `raw` is the pin_node entry
__device__ __forceinline__ void add_grad(ull *gq, ull *gqx, ull *gqy, int raw, float gx, float gy) {
    const int n = raw & kPinNode;
    if (__builtin_expect(raw >= 0, 1)) {  // nodes of more than kPackMaxPins pins are rare
        atomicAdd(gq + n, pack_q(grad_q32(gx), grad_q32(gy)));
    } else {
        atomicAdd(gqx + n, grad_q(gx));
        atomicAdd(gqy + n, grad_q(gy));
    }
}

// Sums of 8 values at once over an aligned group of G lanes (transposed
// butterfly): halving exchanges at offsets G/2, G/4, G/8 leave lane-in-group
// l with a partial of quantity (l / (G/8)) & 7, the remaining offsets finish
// it, and 8 broadcasts hand every lane of the group every total -- 3 + log2(G/8)
// + 8 shuffles instead of 8 log2(G).  Fixed order, so the same on every run.
// `mask`: the group's lanes; `base`: its first lane.
template <int G>
__device__ __forceinline__ void group_sum8(float v[8], int l, unsigned mask, int base) {
    static_assert(G >= 8 && G <= 32, "group of 8..32 lanes");
    const bool a = l & (G / 2), b = l & (G / 4), c = l & (G / 8);
    float u[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float send = a ? v[k] : v[k + 4];
        u[k] = (a ? v[k + 4] : v[k]) + __shfl_xor_sync(mask, send, G / 2);
    }
    float t[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const float send = b ? u[k] : u[k + 2];
        t[k] = (b ? u[k + 2] : u[k]) + __shfl_xor_sync(mask, send, G / 4);
    }
    float sum = (c ? t[1] : t[0]) + __shfl_xor_sync(mask, c ? t[0] : t[1], G / 8);
#pragma unroll
    for (int o = G / 16; o > 0; o >>= 1) sum += __shfl_xor_sync(mask, sum, o);
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = __shfl_sync(mask, sum, base + q * (G / 8));
}

// Maxima of 4 values at once over an aligned group of G lanes, the same scheme.
template <int G>
__device__ __forceinline__ void group_max4(float v[4], int l, unsigned mask, int base) {
    const bool a = l & (G / 2), b = l & (G / 4);
    float u[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const float send = a ? v[k] : v[k + 2];
        u[k] = fmaxf(a ? v[k + 2] : v[k], __shfl_xor_sync(mask, send, G / 2));
    }
    float m = fmaxf(b ? u[1] : u[0], __shfl_xor_sync(mask, b ? u[0] : u[1], G / 4));
#pragma unroll
    for (int o = G / 8; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(mask, m, o));
#pragma unroll
    for (int q = 0; q < 4; ++q) v[q] = __shfl_sync(mask, m, base + q * (G / 4));
}

// One net of degree d <= G P by an aligned group of G lanes, P pins per lane
// in registers (pin j on lane j mod G): one load pass, each exponential once.
template <int G, int P>
__device__ __forceinline__ void net_group(const WaArgs &a, int s, int d, int l, unsigned mask, int base,
                                          const float2 *xy, float inv_g, float &hpf, float &waf) {
    bool v[P];
    int nd[P];
    float c[P][2];
#pragma unroll
    for (int p = 0; p < P; ++p) {
        const int j = l + p * G;
        v[p] = j < d;
        // a slot past the net's end repeats its last pin: the extrema are
        // unchanged and no load waits on a branch (its terms are zeroed below)
        nd[p] = __ldg(a.pin_node + s + min(j, d - 1));  // raw entry (heavy flag)
        const float2 q = __ldg(xy + (nd[p] & kPinNode));
        c[p][0] = q.x;
        c[p][1] = q.y;
    }
    float m4[4] = {-3.0e38f, -3.0e38f, -3.0e38f, -3.0e38f};  // max x, max y, -min x, -min y
#pragma unroll
    for (int p = 0; p < P; ++p) {
        m4[0] = fmaxf(m4[0], c[p][0]);
        m4[1] = fmaxf(m4[1], c[p][1]);
        m4[2] = fmaxf(m4[2], -c[p][0]);
        m4[3] = fmaxf(m4[3], -c[p][1]);
    }
    group_max4<G>(m4, l, mask, base);
    const float mx[2] = {m4[0], m4[1]}, mn[2] = {-m4[2], -m4[3]};
    float ep[P][2], em[P][2], s8[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) s8[k] = 0.f;
#pragma unroll
    for (int ax = 0; ax < 2; ++ax)
#pragma unroll
        for (int p = 0; p < P; ++p) {
            const float dp = c[p][ax] - mx[ax], dm = c[p][ax] - mn[ax];
            ep[p][ax] = v[p] ? __expf(dp * inv_g) : 0.f;
            em[p][ax] = v[p] ? __expf(-dm * inv_g) : 0.f;
            s8[4 * ax + 0] += ep[p][ax];
            s8[4 * ax + 1] += em[p][ax];
            s8[4 * ax + 2] += ep[p][ax] * dp;
            s8[4 * ax + 3] += em[p][ax] * dm;
        }
    group_sum8<G>(s8, l, mask, base);
    float g[P][2], wa_net = 0.f;
#pragma unroll
    for (int ax = 0; ax < 2; ++ax) {
        const float ibp = rcp(s8[4 * ax + 0]), ibm = rcp(s8[4 * ax + 1]);
        const float wp = s8[4 * ax + 2] * ibp, wm = s8[4 * ax + 3] * ibm;
#pragma unroll
        for (int p = 0; p < P; ++p) {
            const float dp = c[p][ax] - mx[ax], dm = c[p][ax] - mn[ax];
            g[p][ax] = ep[p][ax] * ibp * (1.f + (dp - wp) * inv_g) - em[p][ax] * ibm * (1.f - (dm - wm) * inv_g);
        }
        wa_net += (mx[ax] - mn[ax]) + wp - wm;
    }
#pragma unroll
    for (int p = 0; p < P; ++p)
        if (v[p] && (nd[p] & kPinNode) < a.n_grad) add_grad(a.gq, a.gqx, a.gqy, nd[p], g[p][0], g[p][1]);
    if (l == 0) {
        hpf += (mx[0] - mn[0]) + (mx[1] - mn[1]);
        waf += wa_net;
    }
}

// Nets of sub-bucket [lo, hi) by groups of G lanes; the launch's blocks
// [b0, b0 + nb) serve this sub-bucket, this one is block `bid`.
template <int G, int P>
__device__ __forceinline__ void net_groups(const WaArgs &a, int bid, int lo, int hi, int b0, int nb,
                                           const float2 *xy, float inv_g, float &hpf, float &waf) {
    constexpr int per_block = kThreads / G;
    const int lane = threadIdx.x & 31, l = lane & (G - 1), base = lane - l;
    const unsigned mask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << base);
    const int group = (bid - b0) * per_block + (int)threadIdx.x / G, n_groups = nb * per_block;
    for (int e = lo + group; e < hi; e += n_groups) {
        const int s = __ldg(a.net_ptr + e), d = __ldg(a.net_ptr + e + 1) - s;
        net_group<G, P>(a, s, d, l, mask, base, xy, inv_g, hpf, waf);
    }
}

// One net with d <= D pins held in registers by one thread.
template <int D>
__device__ __forceinline__ void net_thread(const int *__restrict__ pins, int d, const float2 *__restrict__ xy,
                                           float inv_g, ull *gq, ull *gqx, ull *gqy, int n_grad, float &hp_acc,
                                           float &wa_acc) {
    int node[D];
    float xs[D], ys[D];
    float xmx = -3.0e38f, xmn = 3.0e38f, ymx = -3.0e38f, ymn = 3.0e38f;
#pragma unroll
    for (int j = 0; j < D; ++j) {
        if (j < d) {
            node[j] = __ldg(pins + j);  // raw entry (heavy flag)
            const float2 q = __ldg(xy + (node[j] & kPinNode));
            xs[j] = q.x;
            ys[j] = q.y;
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
        const float ibp = rcp(bp), ibm = rcp(bm), wp = cp * ibp, wm = cm * ibm;
        wa_net += (cmx - cmn) + wp - wm;
#pragma unroll
        for (int j = 0; j < D; ++j) {
            if (j < d) {
                const float c = axis ? ys[j] : xs[j];
                const float g = ep[j] * ibp * (1.f + ((c - cmx) - wp) * inv_g) -
                                em[j] * ibm * (1.f - ((c - cmn) - wm) * inv_g);
                if (axis == 0) {
                    gxs[j] = g;
                } else if ((node[j] & kPinNode) < n_grad) {
                    add_grad(gq, gqx, gqy, node[j], gxs[j], g);
                }
            }
        }
    }
    hp_acc += (xmx - xmn) + (ymx - ymn);
    wa_acc += wa_net;
}

// One 2-pin net (pins a, b) in closed form.  With d = |x_a - x_b|, e =
// exp(-d/g) and r = 1/(1 + e), the terms above reduce to b+ = b- = 1 + e and
//   dWA/dx_max = (1 - e) r + 2 d e r^2 / g = -dWA/dx_min,
//   WA = d (1 - e) r,  HPWL = d
// (the same quantities; one exponential per axis instead of four).
__device__ __forceinline__ void net_pair(const WaArgs &a, int s, const float2 *__restrict__ xy, float inv_g,
                                         float &hp_acc, float &wa_acc) {
    const int na = __ldg(a.pin_node + s), nb = __ldg(a.pin_node + s + 1);  // raw entries (heavy flag)
    const float2 pa = __ldg(xy + (na & kPinNode)), pb = __ldg(xy + (nb & kPinNode));
    const float dd[2] = {pa.x - pb.x, pa.y - pb.y};
    float g[2];
#pragma unroll
    for (int ax = 0; ax < 2; ++ax) {
        const float d = fabsf(dd[ax]);
        const float e = __expf(-d * inv_g);
        const float r = rcp(1.f + e);
        const float gmax = r * (1.f - e) + 2.f * d * e * r * r * inv_g;
        g[ax] = dd[ax] >= 0.f ? gmax : -gmax;  // pin a is the larger coordinate, or they coincide (g = 0)
        hp_acc += d;
        wa_acc += d * (1.f - e) * r;
    }
    if ((na & kPinNode) < a.n_grad) add_grad(a.gq, a.gqx, a.gqy, na, g[0], g[1]);
    if ((nb & kPinNode) < a.n_grad) add_grad(a.gq, a.gqx, a.gqy, nb, -g[0], -g[1]);
}

}  // namespace

// Bucket B (degree <= D) of the thread-per-net nets: registers sized for D.
template <int D, int B>
__device__ __forceinline__ void wa_small_body(const WaArgs &a, VBlock vb) {
    __shared__ double red[32];
    const float gamma = a.gamma > 0.f ? a.gamma : a.sc->f_gamma;
    const float inv_g = 1.f / gamma;
    const float2 *xy = a.xy;  // every node's position, interleaved
    // per-thread partials in FP32 (a thread owns a few nets), FP64 from the
    // block sum on: the FP64 pipe of this part is narrow
    float hpf = 0.f, waf = 0.f;
    const int lo = a.bucket_lo[B], hi = a.bucket_lo[B + 1];
    // every net of the 2-pin bucket has degree 2: its pins sit at a computed
    // offset, one dependent load fewer per net
    const int s0 = D == 2 && lo < hi ? __ldg(a.net_ptr + lo) : 0;
    for (int e = lo + vb.id * blockDim.x + threadIdx.x; e < hi; e += vb.n * blockDim.x) {
        if (D == 2) {
            net_pair(a, s0 + 2 * (e - lo), xy, inv_g, hpf, waf);
        } else {
            const int s = __ldg(a.net_ptr + e);
            net_thread<D>(a.pin_node + s, __ldg(a.net_ptr + e + 1) - s, xy, inv_g, a.gq, a.gqx, a.gqy, a.n_grad,
                          hpf, waf);
        }
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
        pf[2 * (off + vb.id)] = hp;
        pf[2 * (off + vb.id) + 1] = wa;
    }
}

template <int D, int B>
__global__ void __launch_bounds__(kThreads) wa_small_kernel(WaArgs a) { wa_small_body<D, B>(a, grid_block()); }

// General path of one net of any degree by a warp: three passes over the pins
// (extrema; sums; gradients), pins lane, lane + 32, ...
__device__ __forceinline__ void net_warp_loop(const WaArgs &a, int s, int d, const float2 *xy, float inv_g,
                                              float &hpf, float &waf) {
    const int lane = threadIdx.x & 31;
    float m4[4] = {-3.0e38f, -3.0e38f, -3.0e38f, -3.0e38f};  // max x, max y, -min x, -min y
    for (int j = lane; j < d; j += 32) {
        const int n = __ldg(a.pin_node + s + j) & kPinNode;
        const float2 q = __ldg(xy + n);
        const float x = q.x, y = q.y;
        m4[0] = fmaxf(m4[0], x);
        m4[1] = fmaxf(m4[1], y);
        m4[2] = fmaxf(m4[2], -x);
        m4[3] = fmaxf(m4[3], -y);
    }
    group_max4<32>(m4, lane, 0xffffffffu, 0);
    const float xmx = m4[0], ymx = m4[1], xmn = -m4[2], ymn = -m4[3];
    float s8[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // bp bm cp cm for x then y
    for (int j = lane; j < d; j += 32) {
        const int n = __ldg(a.pin_node + s + j) & kPinNode;
        const float2 q = __ldg(xy + n);
        const float c2[2] = {q.x, q.y};
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
    group_sum8<32>(s8, lane, 0xffffffffu, 0);
    AxisTerms t[2];
#pragma unroll
    for (int ax = 0; ax < 2; ++ax) {
        t[ax].inv_bp = rcp(s8[4 * ax + 0]);
        t[ax].inv_bm = rcp(s8[4 * ax + 1]);
        t[ax].wp = s8[4 * ax + 2] * t[ax].inv_bp;
        t[ax].wm = s8[4 * ax + 3] * t[ax].inv_bm;
    }
    for (int j = lane; j < d; j += 32) {
        const int raw = __ldg(a.pin_node + s + j), n = raw & kPinNode;
        if (n >= a.n_grad) continue;
        const float2 q = __ldg(xy + n);
        const float c2[2] = {q.x, q.y};
        float g[2];
#pragma unroll
        for (int ax = 0; ax < 2; ++ax) {
            const float dp = c2[ax] - (ax ? ymx : xmx), dm = c2[ax] - (ax ? ymn : xmn);
            const float ep = __expf(dp * inv_g), em = __expf(-dm * inv_g);
            g[ax] = ep * t[ax].inv_bp * (1.f + (dp - t[ax].wp) * inv_g) -
                    em * t[ax].inv_bm * (1.f - (dm - t[ax].wm) * inv_g);
        }
        add_grad(a.gq, a.gqx, a.gqy, raw, g[0], g[1]);
    }
    if (lane == 0) {
        hpf += (xmx - xmn) + (ymx - ymn);
        waf += ((xmx - xmn) + t[0].wp - t[0].wm) + ((ymx - ymn) + t[1].wp - t[1].wm);
    }
}

// Nets of degree > 8 (buckets 3..6): blocks [0, b3) take degrees 9..16 with
// 8 lanes per net (two pins per lane, four nets per warp), then 17..32 with 16
// lanes (two pins per lane), 33..64 with 16 lanes (four pins per lane), and
// above 64 with a warp looping over the pins -- the lane group fits the net,
// so few lanes idle, and each group reduction serves two or four pins per lane
// (one pin per lane on 16 and 32 lanes took 9% longer for the stage).
__device__ __forceinline__ void wa_large_body(const WaArgs &a, VBlock vb) {
    __shared__ double red[32];
    const float gamma = a.gamma > 0.f ? a.gamma : a.sc->f_gamma;
    const float inv_g = 1.f / gamma;
    const float2 *xy = a.xy;  // every node's position, interleaved
    // per-thread partials in FP32 (a thread owns a few nets), FP64 from the
    // block sum on: the FP64 pipe of this part is narrow
    float hpf = 0.f, waf = 0.f;
    int b0 = 0;
    const int bid = vb.id;
    if (bid < b0 + a.bucket_blocks[3]) {
        net_groups<8, 2>(a, bid, a.bucket_lo[3], a.bucket_lo[4], b0, a.bucket_blocks[3], xy, inv_g, hpf, waf);
    } else if (bid < (b0 += a.bucket_blocks[3]) + a.bucket_blocks[4]) {
        net_groups<16, 2>(a, bid, a.bucket_lo[4], a.bucket_lo[5], b0, a.bucket_blocks[4], xy, inv_g, hpf, waf);
    } else if (bid < (b0 += a.bucket_blocks[4]) + a.bucket_blocks[5]) {
        net_groups<16, 4>(a, bid, a.bucket_lo[5], a.bucket_lo[6], b0, a.bucket_blocks[5], xy, inv_g, hpf, waf);
    } else {
        b0 += a.bucket_blocks[5];
        const int warp = ((bid - b0) * kThreads + (int)threadIdx.x) >> 5, nwarps = (a.bucket_blocks[6] * kThreads) >> 5;
        for (int e = a.bucket_lo[6] + warp; e < a.bucket_lo[7]; e += nwarps) {
            const int s = __ldg(a.net_ptr + e), d = __ldg(a.net_ptr + e + 1) - s;
            net_warp_loop(a, s, d, xy, inv_g, hpf, waf);
        }
    }
    const float hp = block_sum_ff(hpf, reinterpret_cast<float *>(red));
    const float wa = block_sum_ff(waf, reinterpret_cast<float *>(red));
    float *pf = reinterpret_cast<float *>(a.partials);
    if (threadIdx.x == 0) {
        pf[2 * (a.small_blocks + vb.id)] = hp;
        pf[2 * (a.small_blocks + vb.id) + 1] = wa;
    }
}

// HPWL and WA of partials [0, nb) of all four bucket launches (one block).
__device__ __forceinline__ void wa_fold(const WaArgs &a, int nb) {
    __shared__ double red[32];
    const float *pf = reinterpret_cast<const float *>(a.partials);
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

// The last of the four launches: it folds the partials of all of them (the
// three before it ran earlier on the same stream).
__global__ void __launch_bounds__(kThreads, 4) wa_large_kernel(WaArgs a) {
    wa_large_body(a, grid_block());
    if (arrive_last(a.counter, gridDim.x)) wa_fold(a, a.small_blocks + (int)gridDim.x);
}

int wa_plan(WaArgs &a) {
    const int per = a.block_nets > kThreads ? a.block_nets : kThreads;
    auto grid = [per](int items) {
        int b = (items + per - 1) / per;
        return b < 1 ? 1 : (b > kWaMaxBlocks ? kWaMaxBlocks : b);
    };
    for (int b = 0; b < 3; ++b) a.bucket_blocks[b] = grid(a.bucket_lo[b + 1] - a.bucket_lo[b]);
    // large-net sub-buckets: lanes per net 16, 32, 16, 32; <= kWaMaxBlocks in all
    const int lanes[4] = {8, 16, 16, 32};
    int large = 0;
    for (int b = 3; b < kWaBuckets; ++b) {
        a.bucket_blocks[b] = std::min(grid((a.bucket_lo[b + 1] - a.bucket_lo[b]) * lanes[b - 3]), kWaMaxBlocks / 4);
        large += a.bucket_blocks[b];
    }
    a.small_blocks = a.bucket_blocks[0] + a.bucket_blocks[1] + a.bucket_blocks[2];
    return a.small_blocks + large;
}

// Positions (px, py) of all nodes -> the interleaved copy the WA kernels read.
__global__ void interleave_kernel(int n, const float *__restrict__ px, const float *__restrict__ py,
                                  float2 *__restrict__ xy) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        xy[i] = make_float2(px[i], py[i]);
}

void launch_interleave(int n, const float *px, const float *py, float2 *xy, cudaStream_t st) {
    if (n <= 0) return;
    int blocks = (n + kThreads - 1) / kThreads;
    if (blocks > 2048) blocks = 2048;
    interleave_kernel<<<blocks, kThreads, 0, st>>>(n, px, py, xy);
}

void launch_wirelength(const WaArgs &a0, cudaStream_t st) {
    WaArgs a = a0;
    if (a.mode != WA_LOOP) launch_interleave(a.n_nodes, a.px, a.py, a.xy, st);
    const int large = wa_plan(a) - a.small_blocks;
    wa_small_kernel<2, 0><<<a.bucket_blocks[0], kThreads, 0, st>>>(a);
    wa_small_kernel<4, 1><<<a.bucket_blocks[1], kThreads, 0, st>>>(a);
    wa_small_kernel<8, 2><<<a.bucket_blocks[2], kThreads, 0, st>>>(a);
    wa_large_kernel<<<large, kThreads, 0, st>>>(a);
}

// The batched form: the four bucket launches of every instance as four
// persistent launches (one record per instance each; registers sized per
// bucket as in the instance's own launches); the last one folds each
// instance's sums in the record's last block, after the other three ended.
template <int D, int B>
__global__ void __launch_bounds__(kThreads, D == 8 ? 3 : 4) persist_wa_small_kernel(PersistQueue q, const WaArgs *recs) {
    persist_loop(q, recs, [](const WaArgs &a, VBlock vb, int) { wa_small_body<D, B>(a, vb); });
}

__global__ void __launch_bounds__(kThreads, 4) persist_wa_large_kernel(PersistQueue q, const WaArgs *recs) {
    persist_loop(q, recs, [](const WaArgs &a, VBlock vb, int) {
        wa_large_body(a, vb);
        if (arrive_last(a.counter, vb.n)) wa_fold(a, a.small_blocks + vb.n);
    });
}

int persist_wa_wave(int bucket) {
    static int waves[4] = {0, 0, 0, 0};
    if (bucket < 0 || bucket > 3) return 0;
    if (!waves[bucket]) {
        const void *k[4] = {(const void *)persist_wa_small_kernel<2, 0>, (const void *)persist_wa_small_kernel<4, 1>,
                            (const void *)persist_wa_small_kernel<8, 2>, (const void *)persist_wa_large_kernel};
        waves[bucket] = wave_of(k[bucket], kThreads, 1216);
    }
    return waves[bucket];
}

void launch_persist_wa(int bucket, const PersistQueue &q, const WaArgs *recs, cudaStream_t st) {
    const int w = persist_wa_wave(bucket);
    switch (bucket) {
    case 0:
        persist_wa_small_kernel<2, 0><<<w, kThreads, 0, st>>>(q, recs);
        break;
    case 1:
        persist_wa_small_kernel<4, 1><<<w, kThreads, 0, st>>>(q, recs);
        break;
    case 2:
        persist_wa_small_kernel<8, 2><<<w, kThreads, 0, st>>>(q, recs);
        break;
    default:
        persist_wa_large_kernel<<<w, kThreads, 0, st>>>(q, recs);
        break;
    }
}

}  // namespace ap
