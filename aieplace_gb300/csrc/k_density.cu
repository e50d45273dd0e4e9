// Density map, overflow, field gather and the Nesterov position update.
//
// scatter_kernel   Placer::computeOverlaps -> Grid::computeBinOverlaps
//                  (vck5000/host/src/AIEplace.cpp:937-967, Grid.cpp:38-110,
//                  Bin.h:78-121) as int64 fixed-point atomics, fused with the
//                  position update that produces the evaluation point.
// rho_kernel       Grid::getRho / computeTotalOverflow (Grid.cpp:112-151):
//                  fixed-point map -> density per bin for the solver, overflow
//                  in exact integer sums; clears the map for the next pass.
// gather_kernel    Placer::nudgeNode (AIEplace.cpp:1004-1046): overlap-weighted
//                  field per node, combined with the wirelength gradient and
//                  preconditioned; FP64 norms re-predict the Lipschitz step and
//                  decide whether the trial is accepted (ePlace) -- the
//                  reference moves by a fixed learning rate instead.
#include <math.h>

#include "ap_common.cuh"
#include "ap_kernels.h"

namespace ap {

namespace {

__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }

// block max in a fixed shuffle tree; valid in thread 0
__device__ __forceinline__ double block_max(double v, double *smem) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) smem[threadIdx.x >> 5] = v;
    __syncthreads();
    v = threadIdx.x < (blockDim.x >> 5) ? smem[threadIdx.x] : 0.0;
    if (threadIdx.x < 32)
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    return v;
}

}  // namespace

// Each block owns a contiguous chunk of kScatterChunk nodes.  Nodes with
// nearby indices share nets and sit close together, so a chunk's bins usually
// span a small rectangle: when that rectangle fits kScatterWindow bins the
// block accumulates in shared memory and adds only its non-zero bins to the
// global map (one global atomic per bin and block instead of one per node
// and bin -- right after initial placement every node sits in a few bins).
// Integer sums make both paths give the same map bit for bit.
constexpr int kScatterPerThread = 8;
constexpr int kScatterChunk = kThreads * kScatterPerThread;
constexpr int kScatterWindow = 4096;

template <typename F>
__device__ __forceinline__ void for_each_overlap(const Grid &g, float x, float y, float w, float h, F &&f) {
    int c0, c1, r0, r1;
    bool small;
    if (!bin_range(g, x, y, w, h, c0, c1, r0, r1, small)) return;
    const long long xq = to_q(x), yq = to_q(y), wq = to_q(w), hq = to_q(h);
    if (small) {
        f(c0, r0, wq * hq);
        return;
    }
    for (int c = c0; c <= c1; ++c) {
        const long long ow = overlap_1d((long long)c * g.bw_q, g.bw_q, xq, wq);
        for (int r = r0; r <= r1; ++r) f(c, r, ow * overlap_1d((long long)r * g.bh_q, g.bh_q, yq, hq));
    }
}

__global__ void __launch_bounds__(kThreads) scatter_kernel(ScatterArgs a) {
    __shared__ double red[32];
    __shared__ int box[4];  // bin bounding box of the chunk: c0, c1, r0, r1
    __shared__ ull win[kScatterWindow];
    const int n = a.update ? a.n_mov : (a.hi - a.lo);
    float alpha = 0.f, mom = 0.f;
    int cur = 0;
    if (a.update) {
        alpha = (float)a.sc->alpha;
        mom = (float)a.sc->mom;
        cur = a.sc->cur;
    }
    const int nxt = 1 - cur;
    const Grid g = a.g;
    if (threadIdx.x == 0) {
        box[0] = box[2] = 0x7fffffff;
        box[1] = box[3] = -1;
    }
    __syncthreads();
    float du = 0.f;  // per-thread partial in FP32; FP64 from the block sum on
    float px[kScatterPerThread], py[kScatterPerThread], pw[kScatterPerThread], ph[kScatterPerThread];
    int bc0 = 0x7fffffff, bc1 = -1, br0 = 0x7fffffff, br1 = -1;
    const int base = blockIdx.x * kScatterChunk;
#pragma unroll
    for (int k = 0; k < kScatterPerThread; ++k) {
        const int i = base + k * kThreads + threadIdx.x;
        pw[k] = 0.f;  // zero area: nothing to scatter
        ph[k] = 0.f;
        px[k] = py[k] = 0.f;
        if (i >= n) continue;
        const int node = a.update ? i : a.lo + i;
        const float w = __ldg(a.w + node), h = __ldg(a.h + node);
        float x, y;
        if (a.update) {
            const float xhi = fmaxf(a.die_w - w, 0.f), yhi = fmaxf(a.die_h - h, 0.f);
            const float ux = a.ux[cur][i], uy = a.uy[cur][i];
            const float nux = clampf(a.vx[cur][i] - alpha * a.gx[cur][i], 0.f, xhi);
            const float nuy = clampf(a.vy[cur][i] - alpha * a.gy[cur][i], 0.f, yhi);
            x = clampf(nux + mom * (nux - ux), 0.f, xhi);
            y = clampf(nuy + mom * (nuy - uy), 0.f, yhi);
            a.ux[nxt][i] = nux;
            a.uy[nxt][i] = nuy;
            a.vx[nxt][i] = x;
            a.vy[nxt][i] = y;
            du += (nux - ux) * (nux - ux) + (nuy - uy) * (nuy - uy);
        } else {
            x = __ldg(a.px + node);
            y = __ldg(a.py + node);
        }
        px[k] = x;
        py[k] = y;
        pw[k] = w;
        ph[k] = h;
        int c0, c1, r0, r1;
        bool small;
        if (bin_range(g, x, y, w, h, c0, c1, r0, r1, small)) {
            bc0 = min(bc0, c0);
            bc1 = max(bc1, c1);
            br0 = min(br0, r0);
            br1 = max(br1, r1);
        }
    }
    if (bc1 >= 0) {
        atomicMin(box + 0, bc0);
        atomicMax(box + 1, bc1);
        atomicMin(box + 2, br0);
        atomicMax(box + 3, br1);
    }
    __syncthreads();
    const int wc0 = box[0], wr0 = box[2];
    const int wc = box[1] - wc0 + 1, wr = box[3] - wr0 + 1;
    const bool use_win = box[1] >= 0 && (long long)wc * wr <= kScatterWindow;
    if (use_win) {
        for (int t = threadIdx.x; t < wc * wr; t += kThreads) win[t] = 0ull;
        __syncthreads();
    }
#pragma unroll
    for (int k = 0; k < kScatterPerThread; ++k) {
        if (use_win) {
            for_each_overlap(g, px[k], py[k], pw[k], ph[k], [&](int c, int r, long long v) {
                atomicAdd(win + (c - wc0) * wr + (r - wr0), (ull)v);
            });
        } else {
            for_each_overlap(g, px[k], py[k], pw[k], ph[k], [&](int c, int r, long long v) {
                atomicAdd(a.rho_q + (long long)c * g.my + r, (ull)v);
            });
        }
    }
    if (use_win) {
        __syncthreads();
        for (int t = threadIdx.x; t < wc * wr; t += kThreads) {
            const ull v = win[t];
            if (v) atomicAdd(a.rho_q + (long long)(wc0 + t / wr) * g.my + (wr0 + t % wr), v);
        }
    }
    if (!a.update) return;
    const double dub = block_sum((double)du, red);
    if (threadIdx.x == 0) a.partials[blockIdx.x] = dub;
    if (arrive_last(a.counter)) {
        const double t = reduce_partials(a.partials, gridDim.x, red);
        if (threadIdx.x == 0) {
            a.sc->t_du = t;
            *a.counter = 0u;
        }
    }
}

void launch_scatter(const ScatterArgs &a, cudaStream_t st) {
    const int n = a.update ? a.n_mov : (a.hi - a.lo);
    if (n <= 0) return;
    const int blocks = (n + kScatterChunk - 1) / kScatterChunk;  // <= 8192 partials for 16M nodes
    scatter_kernel<<<blocks, kThreads, 0, st>>>(a);
}

__device__ __forceinline__ double gamma_of(const DevScalars *sc, double tau) {
    double e = (tau - 0.1) * 20.0 / 9.0 - 1.0;
    e = fmin(fmax(e, -1.0), 1.0);
    return sc->gamma_base * sc->bin_avg * pow(10.0, e);
}

__global__ void __launch_bounds__(kThreads) rho_kernel(RhoArgs a) {
    __shared__ long long red[32];
    long long over = 0, over_abs = 0;
    // two bins per thread and step: 16-byte loads of the int64 maps
    const int npairs = a.nbins >> 1;
    longlong2 *mov2 = reinterpret_cast<longlong2 *>(a.mov_q);
    const longlong2 *fs2 = reinterpret_cast<const longlong2 *>(a.fixs_q);
    const longlong2 *fx2 = reinterpret_cast<const longlong2 *>(a.fix_q);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npairs; p += gridDim.x * blockDim.x) {
        const longlong2 mov = mov2[p];
        mov2[p] = make_longlong2(0, 0);
        const longlong2 fs = fs2[p], fx = fx2[p];
        const long long m[2] = {mov.x, mov.y}, s[2] = {fs.x, fs.y}, f[2] = {fx.x, fx.y};
        float d[2];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const long long tot = m[k] + s[k];
            const long long t = tot - a.cap_q;
            over += t > 0 ? t : 0;
            const long long ab = m[k] + f[k] - a.ab_q;
            over_abs += ab > 0 ? ab : 0;
            d[k] = __ll2float_rn(tot) * a.inv_ab_f;  // same float ops as or_density_float
        }
        if (a.d_f32) reinterpret_cast<float2 *>(a.d_f32)[p] = make_float2(d[0], d[1]);
        if (a.d_hi) {
            const __nv_bfloat16 h0 = __float2bfloat16_rn(d[0]), h1 = __float2bfloat16_rn(d[1]);
            reinterpret_cast<__nv_bfloat162 *>(a.d_hi)[p] = __halves2bfloat162(h0, h1);
            reinterpret_cast<__nv_bfloat162 *>(a.d_lo)[p] = __floats2bfloat162_rn(
                d[0] - __bfloat162float(h0), d[1] - __bfloat162float(h1));
        }
    }
    over = block_sum(over, red);
    over_abs = block_sum(over_abs, red);
    if (threadIdx.x == 0) {
        a.partials[2 * blockIdx.x] = over;
        a.partials[2 * blockIdx.x + 1] = over_abs;
    }
    if (arrive_last(a.counter)) {
        long long o = 0, oa = 0;
        for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) {
            o += __ldcg(a.partials + 2 * i);
            oa += __ldcg(a.partials + 2 * i + 1);
        }
        o = block_sum(o, red);
        oa = block_sum(oa, red);
        if (threadIdx.x == 0) {
            DevScalars *sc = a.sc;
            const double tau = sc->mov_area_q > 0 ? (double)o / sc->mov_area_q : 0.0;
            const double tau_abs = ldexp((double)oa, -32);
            if (a.out) {
                a.out[0] = tau;
                a.out[1] = tau_abs;
            }
            if (a.mode == RHO_INIT) {
                sc->tau = tau;
                sc->tau_abs = tau_abs;
            }
            if (a.mode != RHO_OUT_ONLY) {
                sc->t_tau = tau;
                sc->t_tau_abs = tau_abs;
                sc->gamma = gamma_of(sc, tau);
            }
            *a.counter = 0u;
        }
    }
}

void launch_rho(const RhoArgs &a, cudaStream_t st) {
    int blocks = (a.nbins / 2 + kThreads - 1) / kThreads;
    if (blocks > 608) blocks = 608;  // 4 blocks per SM: each thread walks several bin pairs
    rho_kernel<<<blocks, kThreads, 0, st>>>(a);
}

// Accept / retry decision of one trial (one thread).  Mirrors or_step in the
// oracle: backtracking while the re-predicted step falls below 0.95 of the
// step tried; on acceptance the momentum restart test, the density-penalty
// update (RePlAce: mu = mu_max^(1 - dHPWL/ref) in [mu_min, mu_max]) and the
// momentum coefficients of the next iteration.
__device__ void finish_trial(DevScalars *sc, double dv2, double dg2) {
    sc->sum_dv2 = dv2;
    sc->sum_dg2 = dg2;
    sc->evals += 1;
    const double ahat = dg2 > 0.0 ? sqrt(dv2) / sqrt(dg2) : 0.0;
    if (!isfinite(ahat) || !isfinite(dv2) || !isfinite(dg2)) {
        sc->status = 9;
        return;
    }
    if (ahat <= 0.95 * sc->alpha && sc->backtracks < sc->max_backtracks) {
        sc->alpha = ahat;
        sc->backtracks += 1;
        return;
    }
    bool restart = false;
    if (sc->restart_mode == 2) restart = true;
    if (sc->restart_mode == 3) restart = sc->t_du < sc->du_prev;
    if (sc->restart_mode == 4) restart = sc->t_tau > sc->tau_prev;
    sc->du_prev = sc->t_du;
    sc->tau_prev = sc->t_tau;
    sc->alpha = ahat;
    sc->a_k = restart ? 1.0 : sc->a_next;
    if (restart && sc->restart_mode != 2) sc->restarts += 1;
    sc->a_next = (1.0 + sqrt(4.0 * sc->a_k * sc->a_k + 1.0)) / 2.0;
    sc->mom = (sc->a_k - 1.0) / sc->a_next;
    const double pc = (sc->t_hpwl - sc->hpwl_prev) / sc->ref_dh;
    double mu = pc < 0.0 ? sc->mu_max : pow(sc->mu_max, 1.0 - pc);
    mu = fmin(fmax(mu, sc->mu_min), sc->mu_max);
    sc->lambda *= mu;
    sc->hpwl_prev = sc->t_hpwl;
    sc->hpwl = sc->t_hpwl;
    sc->wa = sc->t_wa;
    sc->tau = sc->t_tau;
    sc->tau_abs = sc->t_tau_abs;
    sc->backtracks = 0;
    sc->cur = 1 - sc->cur;
    sc->iteration += 1;
}

__global__ void __launch_bounds__(kThreads) gather_kernel(GatherArgs a) {
    __shared__ double red[32];
    const Grid g = a.g;
    const float lam = (float)a.sc->lambda;
    const int at = a.mode == GATHER_STEP ? 1 - a.sc->cur : a.at;
    const float *vx = a.vx[at], *vy = a.vy[at], *vpx = a.vx[1 - at], *vpy = a.vy[1 - at];
    float *gx_out = a.gx[at], *gy_out = a.gy[at];
    const float *gpx = a.gx[1 - at], *gpy = a.gy[1 - at];
    // per-thread partials in FP32 (a thread owns a couple of nodes); FP64 from
    // the block sums on -- the FP64 pipe of this part is narrow
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n_mov; i += gridDim.x * blockDim.x) {
        const float x = vx[i], y = vy[i];
        const float w = __ldg(a.w + i), h = __ldg(a.h + i);
        float fx = 0.f, fy = 0.f;
        int c0, c1, r0, r1;
        bool small;
        if (bin_range(g, x, y, w, h, c0, c1, r0, r1, small)) {
            const long long xq = to_q(x), yq = to_q(y), wq = to_q(w), hq = to_q(h);
            if (small) {
                const long long b = (long long)c0 * g.my + r0;
                // both sides exact in float: one rounding, = (float)(wq * hq)
                const float wt = (__int2float_rn((int)wq) * __int2float_rn((int)hq)) * g.inv_ab;
                fx = wt * __ldg(a.ex + b);
                fy = wt * __ldg(a.ey + b);
            } else {
                for (int c = c0; c <= c1; ++c) {
                    const long long ow = overlap_1d((long long)c * g.bw_q, g.bw_q, xq, wq);
                    for (int r = r0; r <= r1; ++r) {
                        const long long oh = overlap_1d((long long)r * g.bh_q, g.bh_q, yq, hq);
                        const long long b = (long long)c * g.my + r;
                        const float wt = (__int2float_rn((int)ow) * __int2float_rn((int)oh)) * g.inv_ab;
                        fx += wt * __ldg(a.ex + b);
                        fy += wt * __ldg(a.ey + b);
                    }
                }
            }
        }
        if (a.mode == GATHER_FORCE_ONLY) {
            a.fx[i] = fx;
            a.fy[i] = fy;
            continue;
        }
        const float wlx = i64_to_float((long long)a.gqx[i]) * kInvGradScale;
        const float wly = i64_to_float((long long)a.gqy[i]) * kInvGradScale;
        if (a.mode == GATHER_INIT_NORMS) {
            s2 += fabsf(wlx) + fabsf(wly);
            s3 += fabsf(fx) + fabsf(fy);
            continue;
        }
        a.gqx[i] = 0ull;
        a.gqy[i] = 0ull;
        const float hd = fmaxf(1.f, a.pins[i] + lam * a.charge[i]);
        const float gx = (wlx - lam * fx) / hd, gy = (wly - lam * fy) / hd;
        gx_out[i] = gx;
        gy_out[i] = gy;
        if (a.mode == GATHER_INIT_GRAD) {
            s2 = fmaxf(s2, fmaxf(fabsf(gx), fabsf(gy)));
        } else {
            const float dx = x - vpx[i], dy = y - vpy[i];
            const float ddx = gx - gpx[i], ddy = gy - gpy[i];
            s0 += dx * dx + dy * dy;
            s1 += ddx * ddx + ddy * ddy;
        }
    }
    if (a.mode == GATHER_FORCE_ONLY) return;
    const bool is_max = a.mode == GATHER_INIT_GRAD;
    const double b0 = block_sum((double)s0, red);
    const double b1 = block_sum((double)s1, red);
    const double b2 = is_max ? block_max((double)s2, red) : block_sum((double)s2, red);
    const double b3 = block_sum((double)s3, red);
    if (threadIdx.x == 0) {
        double *p = a.partials + 4 * blockIdx.x;
        p[0] = b0;
        p[1] = b1;
        p[2] = b2;
        p[3] = b3;
    }
    if (arrive_last(a.counter)) {
        double t0 = 0.0, t1 = 0.0, t2 = 0.0, t3 = 0.0;
        for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) {
            const double *p = a.partials + 4 * k;
            t0 += __ldcg(p);
            t1 += __ldcg(p + 1);
            t2 = is_max ? fmax(t2, __ldcg(p + 2)) : t2 + __ldcg(p + 2);
            t3 += __ldcg(p + 3);
        }
        t0 = block_sum(t0, red);
        t1 = block_sum(t1, red);
        t2 = is_max ? block_max(t2, red) : block_sum(t2, red);
        t3 = block_sum(t3, red);
        if (threadIdx.x == 0) {
            DevScalars *sc = a.sc;
            if (a.mode == GATHER_INIT_NORMS) {
                sc->sum_gwl = t2;
                sc->sum_f = t3;
                sc->lambda = t3 > 0.0 ? sc->init_density_weight * t2 / t3 : sc->init_density_weight;
            } else if (a.mode == GATHER_INIT_GRAD) {
                sc->gmax = t2;
            } else if (a.mode == GATHER_INIT_PREV) {
                // first predicted step from v_0 and the probe point v_{-1}
                sc->sum_dv2 = t0;
                sc->sum_dg2 = t1;
                sc->alpha = t1 > 0.0 ? sqrt(t0) / sqrt(t1) : 0.0;
                sc->a_k = 1.0;
                sc->a_next = (1.0 + sqrt(5.0)) / 2.0;
                sc->mom = 0.0;
                if (!isfinite(sc->alpha)) sc->status = 9;
            } else {
                finish_trial(sc, t0, t1);
            }
            *a.counter = 0u;
        }
    }
}

void launch_gather(const GatherArgs &a, cudaStream_t st) {
    int blocks = (a.n_mov + kThreads - 1) / kThreads;
    if (blocks > 4096) blocks = 4096;
    if (blocks < 1) blocks = 1;
    gather_kernel<<<blocks, kThreads, 0, st>>>(a);
}

__global__ void perturb_kernel(int n, const float *vx, const float *vy, const float *gx, const float *gy,
                               float *ox, float *oy, const double *gmax, float coef_bw, float die_w,
                               float die_h, const float *w, const float *h) {
    const double gm = *gmax;
    const float s = gm > 0.0 ? (float)(coef_bw / gm) : 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        ox[i] = clampf(vx[i] - s * gx[i], 0.f, fmaxf(die_w - w[i], 0.f));
        oy[i] = clampf(vy[i] - s * gy[i], 0.f, fmaxf(die_h - h[i], 0.f));
    }
}

void launch_perturb(int n_mov, const float *vx, const float *vy, const float *gx, const float *gy,
                    float *ox, float *oy, const double *gmax, float coef_bw, float die_w, float die_h,
                    const float *w, const float *h, cudaStream_t st) {
    if (n_mov <= 0) return;
    int blocks = (n_mov + kThreads - 1) / kThreads;
    if (blocks > 4096) blocks = 4096;
    perturb_kernel<<<blocks, kThreads, 0, st>>>(n_mov, vx, vy, gx, gy, ox, oy, gmax, coef_bw, die_w,
                                                 die_h, w, h);
}

}  // namespace ap
