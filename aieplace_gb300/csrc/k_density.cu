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

#include <algorithm>

#include "ap_common.cuh"
#include "ap_kernels.h"
#include "ap_persist.cuh"

namespace ap {

namespace {

__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }

// block max of non-negative FP32 values, FP64 result valid in thread 0
__device__ __forceinline__ double block_max_f(float v, double *smem) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) smem[threadIdx.x >> 5] = (double)v;
    __syncthreads();
    double d = 0.0;
    if (threadIdx.x < 32) {
        d = threadIdx.x < (blockDim.x >> 5) ? smem[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) d = fmax(d, __shfl_xor_sync(0xffffffffu, d, o));
    }
    __syncthreads();
    return d;
}

}  // namespace

// The density scatter.  A node adds ow(c) * oh(r) to every bin (c, r) it
// overlaps, ow and oh its fixed-point overlaps with column c and row r.
// Right after the initial placement -- for hundreds of iterations of the
// 2M-cell workload -- most nodes sit in a dense core a few bins across (up
// to ~450k nodes in one bin), where atomic adds to the map collide; later
// they spread over the die, where plain global reductions run at the L2's
// rate (measured on GB300: 4.5M int64 reductions to spread addresses in
// ~23 us, 428 us when they crowd into a few bins).  Each block therefore
// takes a contiguous range of nodes, finds the mean base bin of a sample of
// the range (its first node per thread) and counts the sample's nodes inside
// a kCoreT x kCoreT tile and a kWinT x kWinT window about it; then,
// uniformly over the block:
//   * 85% or more in the core: the core tile in shared memory, kCoreC copies
//     (lane l adds to copy l % kCoreC, so a warp's lanes hitting the same
//     bin do not collide);
//   * else half or more in the window (ranges of kWinMinNodes or more): the window
//     in shared memory, kWinC copies;
//   * else no tile.
// Nodes inside the tile add to it (red.shared.add.u64), the rest straight to
// the map (red.global.add); at the end each tile bin's copies are summed and
// the non-zero bins added to the map once.  Copy k of bin e sits at
// [k t^2 + e].  All sums are integers, so the map is the same bit for bit
// whatever the path or the order (and equal to or_density_q).
constexpr int kCoreT = 8;
constexpr int kCoreC = 32;
constexpr int kWinT = 32;
constexpr int kWinC = 8;
constexpr int kWinMinNodes = 2048;
// dynamic shared memory of the scatter: the larger of the two tiles
constexpr int kScatterSmem = 8 * (kCoreT * kCoreT * kCoreC > kWinT * kWinT * kWinC ? kCoreT * kCoreT * kCoreC
                                                                                  : kWinT * kWinT * kWinC);
constexpr int kScatterThreads = 256;

// A node's contribution as a record of 5 int32: the base bin (c0, r0), the
// spans nc, nr <= 8 and a small-node flag packed in `bin` (non-negative), the
// node's fixed-point x and y relative to the base bin's corner and its
// fixed-point width and height.  Column c0 + j overlaps the node by
// overlap_1d(j bw, bw, xr, wq) -- the same integer as from absolute
// coordinates, evaluated in 32-bit arithmetic (a record is made only when its
// values and their sums fit int32).  Nodes that span more bins, or whose
// extents do not fit, are re-evaluated in full (kRecFull).  Bin counts are at
// most 4096 per axis.
constexpr int kRecNone = -1, kRecFull = -2;
constexpr int kRecSmall = 1 << 30, kRecMaxSpan = 8;

struct NodeRec {
    int bin;  // c0 | r0 << 12 | (nc - 1) << 24 | (nr - 1) << 27 | small << 30
    int xr, wq, yr, hq;
};

__device__ __forceinline__ int rec_c0(int b) { return b & 0xFFF; }
__device__ __forceinline__ int rec_r0(int b) { return (b >> 12) & 0xFFF; }
__device__ __forceinline__ int rec_nc(int b) { return ((b >> 24) & 7) + 1; }
__device__ __forceinline__ int rec_nr(int b) { return ((b >> 27) & 7) + 1; }

__device__ __forceinline__ bool fits_i32(long long v) { return v >= -2147483647ll && v <= 2147483647ll; }

__device__ __forceinline__ NodeRec make_rec(const Grid &g, float x, float y, float w, float h, int &c0, int &c1,
                                            int &r0, int &r1, int2 whq = make_int2(kSizeQNone, kSizeQNone)) {
    NodeRec r{kRecNone, 0, 0, 0, 0};
    bool small;
    if (!bin_range(g, x, y, w, h, c0, c1, r0, r1, small)) {
        c1 = r1 = -1;
        return r;
    }
    // the sizes' fixed point from launch_size_q where it was made (the same integers)
    const long long wq = whq.x != kSizeQNone ? (long long)whq.x : to_q(w);
    const long long hq = whq.y != kSizeQNone ? (long long)whq.y : to_q(h);
    if (small) {
        if (!fits_i32(wq) || !fits_i32(hq)) {
            r.bin = kRecFull;
            return r;
        }
        r.bin = c0 | (r0 << 12) | kRecSmall;
        r.wq = (int)wq;
        r.hq = (int)hq;
        return r;
    }
    const long long xr = to_q(x) - (long long)c0 * g.bw_q, yr = to_q(y) - (long long)r0 * g.bh_q;
    // every integer of emit_rec / the gather's record path must fit int32:
    // xr + wq, yr + hq and (span + 1) bin widths
    if (c1 - c0 >= kRecMaxSpan || r1 - r0 >= kRecMaxSpan || !fits_i32(xr) || !fits_i32(yr) || !fits_i32(wq) ||
        !fits_i32(hq) || !fits_i32(xr + wq) || !fits_i32(yr + hq) || g.bw_q * (kRecMaxSpan + 1) > 2147483647ll ||
        g.bh_q * (kRecMaxSpan + 1) > 2147483647ll) {
        r.bin = kRecFull;
        return r;
    }
    r.bin = c0 | (r0 << 12) | ((c1 - c0) << 24) | ((r1 - r0) << 27);
    r.xr = (int)xr;
    r.wq = (int)wq;
    r.yr = (int)yr;
    r.hq = (int)hq;
    return r;
}

// Calls add(c, r, value) for each bin of a record with the values
// for_each_overlap produces, in the same order (column-major).
template <typename F>
__device__ __forceinline__ void emit_rec(const Grid &g, int bin, int xr, int wq, int yr, int hq, F &&add) {
    const int c0 = rec_c0(bin), r0 = rec_r0(bin);
    if (bin & kRecSmall) {
        add(c0, r0, (long long)wq * hq);
        return;
    }
    const int nc = rec_nc(bin), nr = rec_nr(bin);
    for (int j = 0; j < nc; ++j) {
        const int bw = (int)g.bw_q, bh = (int)g.bh_q;  // record bins: (span + 1) widths fit int32
        const int ow = overlap_1d32(j * bw, bw, xr, wq);
        for (int k = 0; k < nr; ++k) add(c0 + j, r0 + k, (long long)ow * overlap_1d32(k * bh, bh, yr, hq));
    }
}

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

// Update mode, first of the two launches: the Nesterov step of every movable
// node from the accepted state (buffers [cur]) to the trial point (buffers
// [1 - cur]) and the node's bin record there, one node per thread -- a
// streaming pass; block sums of |u' - u|^2 folded by the last block.  Split
// from the bin adds, which need few threads per SM's worth of registers and
// shared memory, so that this part runs at full occupancy.
template <bool kPair>
__device__ __forceinline__ void update_body(const ScatterArgs &a, VBlock vb) {
    __shared__ double red[32];  // 64 floats: two block sums
    const float alpha = a.sc->f_alpha, mom = a.sc->f_mom;
    const int cur = a.sc->cur, nxt = 1 - cur;
    const Grid g = a.g;
    // per-thread partials in FP32 (|u_new - u|^2 for the speed restart and
    // |v_new - v|^2 for the step-length estimate); FP64 from the block sums on
    float du = 0.f, dv = 0.f;
    // distinct arrays: the loads of a node need not wait for the stores of
    // the thread's previous node (grid-stride over one wave of blocks)
    const float *__restrict__ uxc = a.ux[cur], *__restrict__ uyc = a.uy[cur];
    const float *__restrict__ vxc = a.in_x ? a.in_x : a.vx[cur], *__restrict__ vyc = a.in_y ? a.in_y : a.vy[cur];
    const float *__restrict__ gxc = a.gx[cur], *__restrict__ gyc = a.gy[cur];
    float *__restrict__ uxn = a.ux[nxt], *__restrict__ uyn = a.uy[nxt];
    float *__restrict__ vxn = a.vx[nxt], *__restrict__ vyn = a.vy[nxt];
    int *__restrict__ rbin = a.rec_bin;
    int4 *__restrict__ rov = a.rec_ov;
    const int lo = a.upd_hi > 0 ? a.upd_lo : 0, hi = a.upd_hi > 0 ? a.upd_hi : a.n_mov;
    auto node = [&](int i, float w, float h, int2 whq, float ux, float uy, float vx, float vy, float gx,
                    float gy) {
        const float xhi = fmaxf(a.die_w - w, 0.f), yhi = fmaxf(a.die_h - h, 0.f);
        const float nux = clampf(vx - alpha * gx, 0.f, xhi);
        const float nuy = clampf(vy - alpha * gy, 0.f, yhi);
        const float x = clampf(nux + mom * (nux - ux), 0.f, xhi);
        const float y = clampf(nuy + mom * (nuy - uy), 0.f, yhi);
        uxn[i] = nux;
        uyn[i] = nuy;
        vxn[i] = x;
        vyn[i] = y;
        if (a.trial_x) {
            a.trial_x[i] = x;
            a.trial_y[i] = y;
        }
        if (a.xy_out) a.xy_out[i] = make_float2(x, y);
        du += (nux - ux) * (nux - ux) + (nuy - uy) * (nuy - uy);
        dv += (x - vx) * (x - vx) + (y - vy) * (y - vy);
        int c0, c1, r0, r1;
        const NodeRec r = make_rec(g, x, y, w, h, c0, c1, r0, r1, whq);
        rbin[i] = r.bin;
        rov[i] = make_int4(r.xr, r.wq, r.yr, r.hq);
    };
    const int2 *__restrict__ whqa = a.whq;
    auto size_q = [&](int i) { return whqa ? __ldg(whqa + i) : make_int2(kSizeQNone, kSizeQNone); };
    // two nodes of the thread's grid-stride sequence per trip, every load of
    // both issued before either is used (twice the loads in flight per warp);
    // the nodes are taken in the same order as one per trip, so the FP32
    // partial sums are the same
    // (kPair; the persistent batched form keeps one node per trip, where the
    // pair's registers would cost it a resident block per SM)
    const int S = vb.n * blockDim.x;
    int i = lo + vb.id * blockDim.x + threadIdx.x;
    for (; kPair && i + S < hi; i += 2 * S) {
        const int j = i + S;
        const float w0 = __ldg(a.w + i), h0 = __ldg(a.h + i), w1 = __ldg(a.w + j), h1 = __ldg(a.h + j);
        const float ux0 = uxc[i], uy0 = uyc[i], ux1 = uxc[j], uy1 = uyc[j];
        const float vx0 = vxc[i], vy0 = vyc[i], vx1 = vxc[j], vy1 = vyc[j];
        const float gx0 = gxc[i], gy0 = gyc[i], gx1 = gxc[j], gy1 = gyc[j];
        const int2 q0 = size_q(i), q1 = size_q(j);
        node(i, w0, h0, q0, ux0, uy0, vx0, vy0, gx0, gy0);
        node(j, w1, h1, q1, ux1, uy1, vx1, vy1, gx1, gy1);
    }
    for (; i < hi; i += S)
        node(i, __ldg(a.w + i), __ldg(a.h + i), size_q(i), uxc[i], uyc[i], vxc[i], vyc[i], gxc[i], gyc[i]);
    float *pf = reinterpret_cast<float *>(a.partials);
    float bs[2] = {du, dv};
    block_sums_ff<2>(bs, reinterpret_cast<float *>(red));
    if (threadIdx.x == 0) {
        pf[2 * (a.part_base + vb.id)] = bs[0];
        pf[2 * (a.part_base + vb.id) + 1] = bs[1];
    }
}

// The step sums of partials [0, nb) into the device scalars (one block).
__device__ __forceinline__ void update_fold(const ScatterArgs &a, int nb) {
    __shared__ double red[32];
    const float *pf = reinterpret_cast<const float *>(a.partials);
    const double t = block_sum_f(kahan_strided(pf, threadIdx.x, nb, blockDim.x, 2), red);
    const double t2 = block_sum_f(kahan_strided(pf + 1, threadIdx.x, nb, blockDim.x, 2), red);
    if (threadIdx.x == 0) {
        a.sc->t_du = t;
        a.sc->t_dv2 = t2;
        *a.counter = 0u;
    }
}

__global__ void __launch_bounds__(kThreads) update_kernel(ScatterArgs a) {
    update_body<true>(a, grid_block());
    if (a.no_fold) return;  // uniform: an earlier chunk of a chunked update
    // the partials of this launch and of the chunks before it (launched
    // earlier on the same stream, so complete)
    if (arrive_last(a.counter, gridDim.x)) update_fold(a, a.part_base + (int)gridDim.x);
}

// Per block: the shared tile's shape and place, from where the block's
// nodes lie (uniform over the block).
struct TileShape {
    int t, c;       // t x t bins, c copies; t == 0: no tile (every add to the map)
    int c0, r0;     // the tile's first column and row
    int n, m;       // its bins inside the grid (t, or fewer at a small grid)
};

// The non-zero bins of the shared tile (copy k of bin e at [k t^2 + e])
// into the map, a thread per bin.  With 32-bit slots a slot's low word sums
// the values' bits [0, 16) and its high word their bits [16, 48).
__device__ __forceinline__ void flush_tile(const ull *acc, const TileShape &s, const Grid &g, ull *map, int tile32) {
    const int tt = s.t * s.t;
    for (int e = threadIdx.x; e < tt; e += kScatterThreads) {
        ull v = 0ull;
        for (int k = 0; k < s.c; ++k) {
            const ull w = acc[k * tt + e];
            v += tile32 ? ((w >> 32) << 16) + (w & 0xFFFFFFFFull) : w;
        }
        const int u = e / s.t, w = e - u * s.t;
        if (v && u < s.n && w < s.m) atomicAdd(map + (long long)(s.c0 + u) * g.my + s.r0 + w, v);
    }
}

// The bin adds of nodes [lo, hi) split into vb.n contiguous ranges; this
// block takes range vb.id.  Dynamic shared memory: kScatterSmem bytes.
__device__ __forceinline__ void scatter_body(const ScatterArgs &a, VBlock vb) {
    extern __shared__ __align__(16) ull scatter_acc[];
    __shared__ long long sums[2];
    const int nxt = a.update ? 1 - a.sc->cur : 0;
    const Grid g = a.g;
    const int n = a.hi - a.lo;
    const int per = (n + vb.n - 1) / vb.n;
    const int r_lo = min(n, vb.id * per), r_hi = min(n, r_lo + per);
    const int tid = threadIdx.x, lane = tid & 31;
    // 1. a sample of the range, its first kScatterThreads nodes (one per
    //    thread, kept in registers): their mean base bin places the tiles
    int sb = kRecNone;
    if (r_lo + tid < r_hi) {
        const int node = a.lo + r_lo + tid;
        if (a.update) {
            sb = __ldg(a.rec_bin + node);
        } else {
            int c0, c1, r0, r1;
            sb = make_rec(g, __ldg(a.px + node), __ldg(a.py + node), __ldg(a.w + node), __ldg(a.h + node), c0, c1,
                          r0, r1)
                     .bin;
        }
    }
    const bool valid = sb >= 0;
    const int scol = valid ? rec_c0(sb) : 0, srow = valid ? rec_r0(sb) : 0;
    const int snc = valid && !(sb & kRecSmall) ? rec_nc(sb) : 1, snr = valid && !(sb & kRecSmall) ? rec_nr(sb) : 1;
    const int wsc = __reduce_add_sync(0xffffffffu, scol), wsr = __reduce_add_sync(0xffffffffu, srow);
    if (tid < 2) sums[tid] = 0;
    __syncthreads();
    if (lane == 0) {
        atomicAdd(reinterpret_cast<ull *>(sums + 0), (ull)(long long)wsc);
        atomicAdd(reinterpret_cast<ull *>(sums + 1), (ull)(long long)wsr);
    }
    const int n_valid = __syncthreads_count(valid);  // also orders the adds above before the reads below
    const long long tot = n_valid;
    const int mc = tot ? (int)((2 * sums[0] + tot) / (2 * tot)) : 0;  // rounded means
    const int mr = tot ? (int)((2 * sums[1] + tot) / (2 * tot)) : 0;
    // the core tile and the window about the mean (clamped to the grid)
    auto place = [&](int t, int c) {
        TileShape s;
        s.t = t;
        s.c = c;
        s.n = min(t, g.mx);
        s.m = min(t, g.my);
        s.c0 = min(max(mc - s.n / 2, 0), g.mx - s.n);
        s.r0 = min(max(mr - s.m / 2, 0), g.my - s.m);
        return s;
    };
    const TileShape core = place(kCoreT, kCoreC), win = place(kWinT, kWinC);
    auto inside = [](const TileShape &s, int c0, int r0, int nc, int nr) {
        return c0 >= s.c0 && r0 >= s.r0 && c0 + nc <= s.c0 + s.n && r0 + nr <= s.r0 + s.m;
    };
    // 2. the tile shape, from the sample: the core tile when it holds at
    //    least 85% of the sample (with fewer, the dense ring around it goes
    //    to the map's atomics and the window is faster: measured 37 against
    //    74 us at 60%); else, for ranges of kWinMinNodes or more, the window
    //    when it holds half; else none
    const int in_core = __syncthreads_count(valid && inside(core, scol, srow, snc, snr));
    const int in_win = __syncthreads_count(valid && inside(win, scol, srow, snc, snr));
    TileShape ts = place(0, 0);
    if (n_valid > 0 && 20 * in_core >= 17 * n_valid) ts = core;
    else if (n_valid > 0 && r_hi - r_lo >= kWinMinNodes && 2 * in_win >= n_valid) ts = win;
    // 3. clear the tile (kScatterSmem bytes hold either shape)
    const int nz = ts.t * ts.t * ts.c;
    for (int t = tid; t < nz / 2; t += kScatterThreads)
        reinterpret_cast<ulonglong2 *>(scatter_acc)[t] = make_ulonglong2(0ull, 0ull);
    __syncthreads();
    const unsigned tile_s = (unsigned)__cvta_generic_to_shared(scatter_acc) +
                            8u * (unsigned)(ts.c ? (lane % ts.c) * ts.t * ts.t : 0);
    auto add_glb = [&](int c, int r, long long v) { atomicAdd(a.rho_q + (long long)c * g.my + r, (ull)v); };
    const int tile32 = a.tile32;
    const ull vmax = (ull)(g.bw_q * g.bh_q);  // a bin's area: no add within the die exceeds it
    auto add_tile = [&](int c, int r, long long v) {
        const unsigned addr = tile_s + 8u * (unsigned)((c - ts.c0) * ts.t + (r - ts.r0));
        if (tile32) {
            if ((ull)v <= vmax) {
                // two 32-bit adds (3.6x the rate of one 64-bit add on this
                // part's shared memory); exact, the launcher bounds both words' sums
                asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(addr), "r"((unsigned)v & 0xFFFFu) : "memory");
                asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(addr + 4u), "r"((unsigned)((ull)v >> 16))
                             : "memory");
            } else {
                // outside [0, bin area] (a node partly off the die has negative
                // overlaps under the reference's clamped bin range): the map itself
                atomicAdd(a.rho_q + (long long)c * g.my + r, (ull)v);
            }
        } else {
            asm volatile("red.shared.add.u64 [%0], %1;" ::"r"(addr), "l"(v) : "memory");
        }
    };
    int had = 0;  // this thread added to the tile
    // a node's raw inputs (update mode: its record; plain mode: x, y, w, h as
    // bits), loaded two iterations ahead: the loads of the next two nodes are
    // in flight while this one is added
    auto load_raw = [&](int i, int &rb, int4 &ro) {
        rb = kRecNone;
        ro = make_int4(0, 0, 0, 0);
        if (i >= r_hi) return;
        const int node = a.lo + i;
        if (a.update) {
            rb = __ldg(a.rec_bin + node);
            ro = __ldg(a.rec_ov + node);
        } else {
            rb = 0;
            ro = make_int4(__float_as_int(__ldg(a.px + node)), __float_as_int(__ldg(a.py + node)),
                           __float_as_int(__ldg(a.w + node)), __float_as_int(__ldg(a.h + node)));
        }
    };
    int next_b[2];  // two nodes ahead
    int4 next_o[2];
    load_raw(r_lo + tid, next_b[0], next_o[0]);
    load_raw(r_lo + tid + kScatterThreads, next_b[1], next_o[1]);
    for (int base = r_lo; base < r_hi; base += kScatterThreads) {
        const int i = base + tid;
        const int node = a.lo + i;
        const int rb = next_b[0];
        const int4 ro = next_o[0];
        next_b[0] = next_b[1];
        next_o[0] = next_o[1];
        load_raw(i + 2 * kScatterThreads, next_b[1], next_o[1]);
        if (i >= r_hi) continue;
        NodeRec q;
        if (a.update) {
            q = NodeRec{rb, ro.x, ro.y, ro.z, ro.w};
        } else {
            int c0, c1, r0, r1;
            q = make_rec(g, __int_as_float(ro.x), __int_as_float(ro.y), __int_as_float(ro.z),
                         __int_as_float(ro.w), c0, c1, r0, r1);
        }
        if (q.bin == kRecNone) continue;
        if (q.bin >= 0) {
            const int nc = (q.bin & kRecSmall) ? 1 : rec_nc(q.bin), nr = (q.bin & kRecSmall) ? 1 : rec_nr(q.bin);
            if (inside(ts, rec_c0(q.bin), rec_r0(q.bin), nc, nr)) {
                emit_rec(g, q.bin, q.xr, q.wq, q.yr, q.hq, add_tile);
                had = 1;
            } else {
                emit_rec(g, q.bin, q.xr, q.wq, q.yr, q.hq, add_glb);
            }
        } else {
            // outside the record's range: re-evaluated from the node's position
            const float x = a.update ? a.vx[nxt][node] : __ldg(a.px + node);
            const float y = a.update ? a.vy[nxt][node] : __ldg(a.py + node);
            for_each_overlap(g, x, y, __ldg(a.w + node), __ldg(a.h + node), add_glb);
        }
    }
    // 4. the tile's non-zero bins (the test is a barrier after the last shared add)
    if (__syncthreads_or(had)) flush_tile(scatter_acc, ts, g, a.rho_q, tile32);
}

__global__ void __launch_bounds__(kScatterThreads, 3) scatter_kernel(ScatterArgs a) { scatter_body(a, grid_block()); }

// Resident blocks of `kernel` on the whole GPU (one wave), or `fallback`.
int wave_of(const void *kernel, int threads, int fallback, int dyn_smem) {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, (size_t)dyn_smem) == cudaSuccess &&
        sms * per_sm > 0)
        return sms * per_sm;
    return fallback;
}

__global__ void size_q_kernel(int n, const float *__restrict__ w, const float *__restrict__ h, int2 *out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const long long wq = to_q(w[i]), hq = to_q(h[i]);
        out[i] = make_int2(fits_i32(wq) ? (int)wq : kSizeQNone, fits_i32(hq) ? (int)hq : kSizeQNone);
    }
}

void launch_size_q(int n, const float *w, const float *h, int2 *out, cudaStream_t st) {
    if (n <= 0) return;
    size_q_kernel<<<std::min((n + kThreads - 1) / kThreads, 4096), kThreads, 0, st>>>(n, w, h, out);
}

int update_grid(const ScatterArgs &a) {
    // one wave of resident blocks (at most 8192, the partials buffer),
    // grid-stride beyond: fewer block sums and last-block folds
    static int wave = 0;
    if (wave <= 0) {
        wave = wave_of((const void *)update_kernel, kThreads, 1216);
        if (wave > 8192) wave = 1216;
    }
    const int n = a.upd_hi > 0 ? a.upd_hi - a.upd_lo : a.n_mov;
    const int per = a.block_nodes > kThreads ? a.block_nodes : kThreads;
    int ub = (n + per - 1) / per;
    if (ub > wave) ub = wave;
    if (ub < 1) ub = 1;  // an empty chunk still writes its partials (zero) and may fold
    return ub;
}

int launch_update(const ScatterArgs &a, cudaStream_t st) {
    if (!a.update || a.n_mov <= 0) return 0;
    const int ub = update_grid(a);
    update_kernel<<<ub, kThreads, 0, st>>>(a);
    return ub;
}

int scatter_grid(int n, int block_nodes) {
    // one wave of resident blocks, each a contiguous range of nodes (fewer
    // blocks: fewer tile flushes onto the dense core's bins)
    static int wave = 0;
    if (wave <= 0) {
        cudaFuncSetAttribute(scatter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kScatterSmem);
        wave = wave_of((const void *)scatter_kernel, kScatterThreads, 304, kScatterSmem);
    }
    const int per = block_nodes > kScatterThreads ? block_nodes : kScatterThreads;
    int blocks = (n + per - 1) / per;
    if (blocks > wave) blocks = wave;
    return blocks < 1 ? 1 : blocks;
}

// Whether the bin adds of n nodes over `blocks` blocks may use 32-bit tile
// slots: a slot takes at most one add per node of the threads sharing its
// copy (kScatterThreads / kWinC threads, the fewest copies of a tile), each
// add at most bw_q bh_q; the low word sums at most that many 2^16 - 1, the
// high word that many (bw_q bh_q) >> 16.
bool tile32_exact(const Grid &g, int n, int blocks) {
    const long long range = (n + blocks - 1) / blocks;
    const long long per_slot = (range + kScatterThreads - 1) / kScatterThreads * (kScatterThreads / kWinC);
    const double vmax = (double)g.bw_q * (double)g.bh_q;
    return vmax < 281474976710656.0 && (double)per_slot * 65535.0 < 4294967295.0 &&
           (double)per_slot * floor(vmax / 65536.0) < 4294967295.0;
}

void launch_scatter_bins(const ScatterArgs &a0, cudaStream_t st) {
    const int n = a0.hi - a0.lo;
    if (n <= 0) return;
    ScatterArgs a = a0;
    const int blocks = scatter_grid(n, a.block_nodes);
    a.tile32 = tile32_exact(a.g, n, blocks) ? 1 : 0;
    scatter_kernel<<<blocks, kScatterThreads, kScatterSmem, st>>>(a);
}

void launch_scatter(const ScatterArgs &a, cudaStream_t st) {
    launch_update(a, st);
    launch_scatter_bins(a, st);
}

// gamma(tau) in FP32 (10^e as 2^(e log2 10)): a single-thread FP64 pow at the
// end of the kernel costs microseconds on this part's narrow FP64 pipe
__device__ __forceinline__ double gamma_of(const DevScalars *sc, double tau) {
    float e = ((float)tau - 0.1f) * (20.0f / 9.0f) - 1.0f;
    e = fminf(fmaxf(e, -1.0f), 1.0f);
    return (double)((float)(sc->gamma_base * sc->bin_avg) * exp2f(e * 3.32192809f));
}

constexpr int kRhoBatch = 2;  // 2 pairs a round: 17.4 us at 1024^2 bins (4: 19.4 us, 8: 21.6 us)

__device__ __forceinline__ void rho_body(const RhoArgs &a, VBlock vb) {
    __shared__ long long red[32];
    long long over = 0, over_abs = 0;
    // two bins per 16-byte load of the int64 maps; kRhoBatch such pairs per
    // thread and round, every load of the round issued before any store (the
    // kernel is bound by memory latency, not bandwidth)
    const int npairs = a.nbins >> 1;
    longlong2 *mov2 = reinterpret_cast<longlong2 *>(a.mov_q);
    const longlong2 *__restrict__ fs2 = reinterpret_cast<const longlong2 *>(a.fixs_q);
    const longlong2 *__restrict__ fx2 = reinterpret_cast<const longlong2 *>(a.fix_q);
    longlong2 *fl2 = reinterpret_cast<longlong2 *>(a.fill_q);  // filler cells, or null
    const int stride = vb.n * blockDim.x;
    for (int p0 = vb.id * blockDim.x + threadIdx.x; p0 < npairs; p0 += kRhoBatch * stride) {
        longlong2 mv[kRhoBatch], fs[kRhoBatch], fx[kRhoBatch], fl[kRhoBatch];
#pragma unroll
        for (int j = 0; j < kRhoBatch; ++j) {
            const int p = p0 + j * stride;
            fl[j] = make_longlong2(0, 0);
            if (p < npairs) {
                mv[j] = __ldcg(mov2 + p);
                fs[j] = __ldg(fs2 + p);
                fx[j] = __ldg(fx2 + p);
                if (fl2) fl[j] = __ldcg(fl2 + p);
            }
        }
#pragma unroll
        for (int j = 0; j < kRhoBatch; ++j) {
            const int p = p0 + j * stride;
            if (p >= npairs) break;
            mov2[p] = make_longlong2(0, 0);
            if (fl2) fl2[p] = make_longlong2(0, 0);
            const long long m[2] = {mv[j].x, mv[j].y}, sq[2] = {fs[j].x, fs[j].y}, f[2] = {fx[j].x, fx[j].y};
            const long long fil[2] = {fl[j].x, fl[j].y};
            float d[2];
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const long long tot = m[k] + sq[k];
                const long long t = tot - a.cap_q;
                over += t > 0 ? t : 0;
                const long long ab = m[k] + f[k] - a.ab_q;
                over_abs += ab > 0 ? ab : 0;
                d[k] = ll2f_rn_bits(tot + fil[k]) * a.inv_ab_f - a.d_shift;
            }
            if (a.d_f32) reinterpret_cast<float2 *>(a.d_f32)[p] = make_float2(d[0], d[1]);
            if (a.d_hi) {
                const __nv_bfloat16 h0 = __float2bfloat16_rn(d[0]), h1 = __float2bfloat16_rn(d[1]);
                reinterpret_cast<__nv_bfloat162 *>(a.d_hi)[p] = __halves2bfloat162(h0, h1);
                reinterpret_cast<__nv_bfloat162 *>(a.d_lo)[p] = __floats2bfloat162_rn(
                    d[0] - __bfloat162float(h0), d[1] - __bfloat162float(h1));
            }
        }
    }
    over = block_sum(over, red);
    over_abs = block_sum(over_abs, red);
    if (threadIdx.x == 0) {
        a.partials[2 * vb.id] = over;
        a.partials[2 * vb.id + 1] = over_abs;
    }
}

// The overflow sums of partials [0, nb) into the device scalars, gamma of the
// next evaluation and the trial's field source (one block).
__device__ __forceinline__ void rho_fold(const RhoArgs &a, int nb) {
    __shared__ long long red[32];
    long long o = 0, oa = 0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        o += __ldcg(a.partials + 2 * i);
        oa += __ldcg(a.partials + 2 * i + 1);
    }
    o = block_sum(o, red);
    oa = block_sum(oa, red);
    if (threadIdx.x == 0) {
        DevScalars *sc = a.sc;
        const double tau = sc->mov_area_q > 0 ? (double)o / sc->mov_area_q : 0.0;
        const double tau_abs = (double)oa * 0x1p-32;  // exact power-of-two scaling
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
            sc->gamma_next = gamma_of(sc, tau);
        }
        if (a.mode == RHO_INIT) {
            // the first evaluation's WA uses its own overflow
            sc->gamma = sc->gamma_next;
            sc->f_gamma = (float)sc->gamma;
        }
        // field source of this trial: the surrogate while the overflow is
        // above its threshold and its last judgement passed, the exact
        // solve judging it every surr_judge_every trials
        int fm = kFieldExact;
        if (a.mode == RHO_LOOP && sc->surr_attached && tau > (double)sc->surr_tau_min) {
            if (sc->evals % sc->surr_judge_every == 0)
                fm = kFieldJudge;
            else if (sc->surr_ok)
                fm = kFieldSurr;
        }
        sc->field_mode = fm;
        if (a.field_switch) cudaGraphSetConditional(a.field_switch, (unsigned int)fm);
        if (fm == kFieldSurr) sc->surr_used += 1;
        *a.counter = 0u;
    }
}

__global__ void __launch_bounds__(kThreads) rho_kernel(RhoArgs a) {
    rho_body(a, grid_block());
    if (arrive_last(a.counter, gridDim.x)) rho_fold(a, gridDim.x);
}

int rho_grid(int nbins) {
    // about one round of kRhoBatch pairs per thread, but no more blocks than
    // fit the GPU at once: a partial second wave nearly doubled the time
    // (512 blocks against 456 resident at 1024^2 bins: 19.0 -> 16.9 us)
    static int wave = 0;
    if (wave <= 0) wave = wave_of((const void *)rho_kernel, kThreads, 1216);
    int blocks = (nbins / 2 + kRhoBatch * kThreads - 1) / (kRhoBatch * kThreads);
    if (blocks > wave) blocks = wave;
    return blocks < 1 ? 1 : blocks;
}

void launch_rho(const RhoArgs &a, cudaStream_t st) { rho_kernel<<<rho_grid(a.nbins), kThreads, 0, st>>>(a); }

// The trajectory record of the trial just decided (trial number sc->evals - 1).
__device__ void log_trial(DevScalars *sc, int accepted) {
    if (!sc->traj) return;
    TrajRec r;
    r.eval = sc->evals - 1;
    r.iteration = sc->iteration;
    r.accepted = accepted;
    r.field_mode = sc->field_mode;
    r.hpwl = sc->t_hpwl;
    r.overflow = sc->t_tau;
    r.overflow_abs = sc->t_tau_abs;
    r.lambda = sc->lambda;
    r.alpha = sc->alpha;
    r.gamma = sc->gamma;
    r.surr_err = sc->surr_err;
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    r.t_ns = t;
    sc->traj[(unsigned)r.eval % (unsigned)sc->traj_cap] = r;
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
    // step and momentum arithmetic in FP32 (single thread; FP64 sqrt/pow here
    // cost microseconds per trial on the narrow FP64 pipe)
    const double ahat = dg2 > 0.0 ? (double)(sqrtf((float)dv2) / sqrtf((float)dg2)) : 0.0;
    if (!isfinite(ahat) || !isfinite(dv2) || !isfinite(dg2)) {
        sc->status = 9;
        log_trial(sc, -1);
        return;
    }
    if (ahat <= 0.95 * sc->alpha && sc->backtracks < sc->max_backtracks) {
        sc->alpha = ahat;
        sc->backtracks += 1;
        log_trial(sc, 0);
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
    const float ak = (float)sc->a_k, an = 0.5f * (1.0f + sqrtf(4.0f * ak * ak + 1.0f));
    sc->a_next = (double)an;
    sc->mom = (double)((ak - 1.0f) / an);
    const float pc = (float)(sc->t_hpwl - sc->hpwl_prev) / (float)sc->ref_dh;
    const float mmax = (float)sc->mu_max, mmin = (float)sc->mu_min;
    float mu = pc < 0.0f ? mmax : exp2f(log2f(mmax) * (1.0f - pc));
    mu = fminf(fmaxf(mu, mmin), mmax);
    // capped where the density term dominates completely: keeps the FP32
    // products finite when the target overflow is out of reach (lambda would
    // otherwise grow 5% per iteration until it overflows)
    sc->lambda = fmin(sc->lambda * mu, kLambdaMax);
    sc->hpwl_prev = sc->t_hpwl;
    sc->hpwl = sc->t_hpwl;
    sc->wa = sc->t_wa;
    sc->tau = sc->t_tau;
    sc->tau_abs = sc->t_tau_abs;
    sc->backtracks = 0;
    sc->cur = 1 - sc->cur;
    sc->iteration += 1;
    log_trial(sc, 1);
}

__device__ __forceinline__ void gather_body(const GatherArgs &a, VBlock vb) {
    __shared__ double red[64];  // 128 floats: four block sums
    const Grid g = a.g;
    const float lam = a.mode == GATHER_NODE_OUT ? a.lambda : a.sc->f_lambda;
    const int at = a.mode == GATHER_STEP ? 1 - a.sc->cur : a.at;
    const float *vx = a.vx[at], *vy = a.vy[at], *vpx = a.vx[1 - at], *vpy = a.vy[1 - at];
    float *gx_out = a.gx[at], *gy_out = a.gy[at];
    const float *gpx = a.gx[1 - at], *gpy = a.gy[1 - at];
    // per-thread partials in FP32 (a thread owns a couple of nodes); FP64 from
    // the block sums on -- the FP64 pipe of this part is narrow
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    const bool use_rec = (a.mode == GATHER_STEP || a.mode == GATHER_NODE_OUT) && a.rec_bin != nullptr;
    for (int i = vb.id * blockDim.x + threadIdx.x; i < a.n_mov; i += vb.n * blockDim.x) {
        float fx = 0.f, fy = 0.f;
        int c0, c1, r0, r1;
        bool small;
        // every load that does not depend on the field is issued here, ahead
        // of the field gather: loads after its data-dependent loop would wait
        // for it, and loads under the record's branch for the record
        const int rb = use_rec ? __ldg(a.rec_bin + i) : kRecFull;
        const int4 o = use_rec ? __ldg(a.rec_ov + i) : make_int4(0, 0, 0, 0);  // xr, wq, yr, hq
        ull gqv = 0ull;
        float pc = 0.f, chg = 0.f, gpxv = 0.f, gpyv = 0.f;
        if (a.mode != GATHER_FORCE_ONLY) {
            gqv = a.gq[i];
            pc = __ldg(a.pins + i);
        }
        if (a.mode == GATHER_STEP || a.mode == GATHER_INIT_GRAD || a.mode == GATHER_INIT_PREV ||
            a.mode == GATHER_NODE_OUT) {
            chg = __ldg(a.charge + i);
            if (a.mode != GATHER_INIT_GRAD && a.mode != GATHER_NODE_OUT) {
                gpxv = __ldg(gpx + i);
                gpyv = __ldg(gpy + i);
            }
        }
        if (rb >= 0) {
            // the scatter's record at this point: the weights of the path
            // below, in the same order, without the bin arithmetic
            const int c0r = rec_c0(rb), r0r = rec_r0(rb);
            if (rb & kRecSmall) {
                const int b = c0r * g.my + r0r;
                const float wt = (i64_to_float(o.y) * i64_to_float(o.w)) * g.inv_ab;
                fx = wt * __ldg(a.ex + b);
                fy = wt * __ldg(a.ey + b);
            } else {
                const int nc = rec_nc(rb), nr = rec_nr(rb);
                for (int j = 0; j < nc; ++j) {
                    const float fw = i32_to_float(overlap_1d32(j * (int)g.bw_q, (int)g.bw_q, o.x, o.y));
                    const int bc = (c0r + j) * g.my + r0r;
                    for (int k = 0; k < nr; ++k) {
                        const float fh = i32_to_float(overlap_1d32(k * (int)g.bh_q, (int)g.bh_q, o.z, o.w));
                        const float wt = (fw * fh) * g.inv_ab;
                        fx += wt * __ldg(a.ex + bc + k);
                        fy += wt * __ldg(a.ey + bc + k);
                    }
                }
            }
        } else if (rb == kRecFull && bin_range(g, vx[i], vy[i], __ldg(a.w + i), __ldg(a.h + i), c0, c1, r0, r1,
                                               small)) {
            const float x = vx[i], y = vy[i], w = __ldg(a.w + i), h = __ldg(a.h + i);
            const long long xq = to_q(x), yq = to_q(y), wq = to_q(w), hq = to_q(h);
            if (small) {
                const long long b = (long long)c0 * g.my + r0;
                // both sides exact in float: one rounding, = (float)(wq * hq)
                const float wt = (i64_to_float(wq) * i64_to_float(hq)) * g.inv_ab;
                fx = wt * __ldg(a.ex + b);
                fy = wt * __ldg(a.ey + b);
            } else {
                for (int c = c0; c <= c1; ++c) {
                    const long long ow = overlap_1d((long long)c * g.bw_q, g.bw_q, xq, wq);
                    for (int r = r0; r <= r1; ++r) {
                        const long long oh = overlap_1d((long long)r * g.bh_q, g.bh_q, yq, hq);
                        const long long b = (long long)c * g.my + r;
                        const float wt = (i64_to_float(ow) * i64_to_float(oh)) * g.inv_ab;
                        fx += wt * __ldg(a.ex + b);
                        fy += wt * __ldg(a.ey + b);
                    }
                }
            }
        }
        if (a.mode == GATHER_FORCE_ONLY || a.mode == GATHER_NODE_OUT) {
            a.fx[i] = fx;
            a.fy[i] = fy;
            if (a.mode == GATHER_FORCE_ONLY) continue;
        }
        long long qx, qy;
        unpack_q(gqv, qx, qy);
        const bool heavy = pc > (float)kPackMaxPins;
        if (heavy) {
            qx += (long long)a.gqx[i];
            qy += (long long)a.gqy[i];
        }
        const float wlx = i64_to_float(qx) * kInvGradScale;
        const float wly = i64_to_float(qy) * kInvGradScale;
        if (a.mode == GATHER_INIT_NORMS) {
            s2 += fabsf(wlx) + fabsf(wly);
            s3 += fabsf(fx) + fabsf(fy);
            continue;
        }
        a.gq[i] = 0ull;
        if (heavy) {
            a.gqx[i] = 0ull;
            a.gqy[i] = 0ull;
        }
        const float hd = fmaxf(1.f, pc + lam * chg);
        const float ihd = __frcp_rn(hd);
        const float gx = (wlx - lam * fx) * ihd, gy = (wly - lam * fy) * ihd;
        if (a.mode == GATHER_NODE_OUT) {
            if (a.gxo) {
                a.gxo[i] = gx;
                a.gyo[i] = gy;
            }
            continue;
        }
        gx_out[i] = gx;
        gy_out[i] = gy;
        if (a.mode == GATHER_INIT_GRAD) {
            s2 = fmaxf(s2, fmaxf(fabsf(gx), fabsf(gy)));
        } else {
            // |v - v_prev|^2 of a loop trial comes from the position update
            if (a.mode != GATHER_STEP) {
                const float dx = vx[i] - vpx[i], dy = vy[i] - vpy[i];
                s0 += dx * dx + dy * dy;
            }
            const float ddx = gx - gpxv, ddy = gy - gpyv;
            s1 += ddx * ddx + ddy * ddy;
        }
    }
    if (a.mode == GATHER_FORCE_ONLY || a.mode == GATHER_NODE_OUT) return;
    const bool is_max = a.mode == GATHER_INIT_GRAD;
    // per-block partials in FP32; the last block sums them with compensation
    // and only its warp 0 adds in FP64 (the FP64 pipe of this part is narrow)
    float bs[4] = {s0, s1, s2, s3};
    if (is_max)
        bs[2] = (float)block_max_f(s2, red);  // s0, s1, s3 are zero in this mode
    else
        block_sums_ff<4>(bs, reinterpret_cast<float *>(red));
    float *pf = reinterpret_cast<float *>(a.partials);
    if (threadIdx.x == 0) {
        float *p = pf + 4 * vb.id;
        p[0] = bs[0];
        p[1] = bs[1];
        p[2] = bs[2];
        p[3] = bs[3];
    }
}

// The sums of partials [0, nb) into the device scalars; in a loop trial the
// accept / retry decision (one block).
__device__ __forceinline__ void gather_fold(const GatherArgs &a, int nb) {
    __shared__ double red[64];
    const bool is_max = a.mode == GATHER_INIT_GRAD;
    const float *pf = reinterpret_cast<const float *>(a.partials);
    const double t0 = a.mode == GATHER_STEP
                          ? 0.0
                          : block_sum_f(kahan_strided(pf + 0, threadIdx.x, nb, blockDim.x, 4), red);
    const double t1 = block_sum_f(kahan_strided(pf + 1, threadIdx.x, nb, blockDim.x, 4), red);
    double t2;
    if (is_max) {
        float m = 0.f;
        for (int k = threadIdx.x; k < nb; k += blockDim.x) m = fmaxf(m, __ldcg(pf + 4 * k + 2));
        t2 = block_max_f(m, red);
    } else {
        t2 = block_sum_f(kahan_strided(pf + 2, threadIdx.x, nb, blockDim.x, 4), red);
    }
    const double t3 = block_sum_f(kahan_strided(pf + 3, threadIdx.x, nb, blockDim.x, 4), red);
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
            // the next evaluation's WA smoothing: this trial's gamma(tau),
            // whether the trial is accepted or not
            sc->gamma = sc->gamma_next;
            finish_trial(sc, sc->t_dv2, t1);
        }
        publish_f32(sc);
        *a.counter = 0u;
    }
}

__global__ void __launch_bounds__(kThreads, 4) gather_kernel(GatherArgs a) {
    gather_body(a, grid_block());
    if (a.mode == GATHER_FORCE_ONLY || a.mode == GATHER_NODE_OUT) return;
    if (arrive_last(a.counter, gridDim.x)) gather_fold(a, gridDim.x);
}

int gather_grid(int n_mov, int block_nodes) {
    // one wave of resident blocks, grid-stride beyond: 61 -> 50 us at 2M
    // nodes against 4096 blocks (a partial last wave, 912 blocks, 59 us)
    static int wave = 0;
    if (wave <= 0) {
        wave = wave_of((const void *)gather_kernel, kThreads, 608);
        if (wave > kGatherMaxBlocks) wave = 608;
    }
    const int per = block_nodes > kThreads ? block_nodes : kThreads;
    int blocks = (n_mov + per - 1) / per;
    if (blocks > wave) blocks = wave;
    return blocks < 1 ? 1 : blocks;
}

void launch_gather(const GatherArgs &a, cudaStream_t st) {
    gather_kernel<<<gather_grid(a.n_mov, a.block_nodes), kThreads, 0, st>>>(a);
}

// Bin records of movable nodes at given positions, as update_kernel writes
// them at a trial point (the per-node stage entry point reads them through
// the gather's record path).
__global__ void records_kernel(Grid g, int n_mov, const float *x, const float *y, const float *w, const float *h,
                               int *rec_bin, int4 *rec_ov) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_mov; i += gridDim.x * blockDim.x) {
        int c0, c1, r0, r1;
        const NodeRec r = make_rec(g, x[i], y[i], w[i], h[i], c0, c1, r0, r1);
        rec_bin[i] = r.bin;
        rec_ov[i] = make_int4(r.xr, r.wq, r.yr, r.hq);
    }
}

void launch_records(const Grid &g, int n_mov, const float *x, const float *y, const float *w, const float *h,
                    int *rec_bin, int4 *rec_ov, cudaStream_t st) {
    if (n_mov <= 0) return;
    int blocks = (n_mov + kThreads - 1) / kThreads;
    if (blocks > 4096) blocks = 4096;
    records_kernel<<<blocks, kThreads, 0, st>>>(g, n_mov, x, y, w, h, rec_bin, rec_ov);
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

// Compares the integer-arithmetic conversions of ap_common.cuh with the
// hardware conversion instructions they replace, on hashed samples that
// include rounding ties and the carry of a mantissa that rounds up to 2^24.
__global__ void numerics_selftest_kernel(long long n, ull seed, int *mism) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        ull z = seed + (ull)i * 0x9E3779B97F4A7C15ull;  // splitmix64
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        const unsigned lo = (unsigned)z, hi = (unsigned)(z >> 32);
        // float with |s| < 2^31 (biased exponent <= 157), or a tie k + 1/2
        float s = __uint_as_float((lo & 0x807FFFFFu) | (((hi >> 8) % 158u) << 23));
        if ((hi & 3u) == 0u) s = (float)((int)(lo & 0xFFFFFu) - 0x80000) + 0.5f;
        if (f2i_rn_bits(s) != __float2int_rn(s)) atomicAdd(mism + 0, 1);
        if (f2i_rz_bits(s) != __float2int_rz(s)) atomicAdd(mism + 1, 1);
        // int64 of any magnitude; 1/8 exact ties, some with an all-ones mantissa
        const int sh = (int)(hi & 63u);
        long long v = (long long)(z >> sh);
        if ((hi & 0x380u) == 0u) {
            const ull m = (hi & 0x400u) ? 0xFFFFFFull : (0x800000ull | (lo & 0x7FFFFFu));
            v = (long long)(((m << 1) | 1ull) << (sh % 38));
        }
        if (hi & 0x40u) v = (long long)(0ull - (ull)v);
        if (__float_as_uint(ll2f_rn_bits(v)) != __float_as_uint(__ll2float_rn(v))) atomicAdd(mism + 2, 1);
        const float c = (__uint_as_float(0x3F800000u | (lo >> 9)) - 1.5f) * 7.98f;  // [-3.99, 3.99)
        if ((long long)grad_q(c) != (long long)__float2int_rn(c * kGradScale)) atomicAdd(mism + 3, 1);
        // |q| < 2^22 (the magic-number path) or any int64 of either sign
        const long long q = (hi & 0x1000u) ? v : (long long)(lo % 8388607u) - 4194303ll;
        if (__float_as_uint(i64_to_float(q)) != __float_as_uint(__ll2float_rn(q))) atomicAdd(mism + 4, 1);
        // (-1, 2^23): [1, 2^23) with every exponent, or (-1, 1)
        const float t = __uint_as_float((lo & 0x007FFFFFu) | ((127u + (hi >> 12) % 23u) << 23));
        const float u = (hi & 0x800u) ? t : __fmul_rn(t, 1.0f / 4194304.0f) - 1.0f;
        if (u > -1.0f && f2i_rz_small(u) != __float2int_rz(u)) atomicAdd(mism + 5, 1);
    }
}

// ---- persistent launches of the batched form ------------------------------
// Each record is one instance's launch of the stage (its arguments and its
// grid as the launchers above would size it); the per-instance sums fold in
// the record's last block, as in the instance's own launch.

__global__ void __launch_bounds__(kThreads) persist_update_kernel(PersistQueue q, const ScatterArgs *recs) {
    persist_loop(q, recs, [](const ScatterArgs &a, VBlock vb, int) {
        update_body<false>(a, vb);
        if (arrive_last(a.counter, vb.n)) update_fold(a, vb.n);
    });
}

__global__ void __launch_bounds__(kScatterThreads, 3) persist_scatter_kernel(PersistQueue q, const ScatterArgs *recs) {
    persist_loop(q, recs, [](const ScatterArgs &a, VBlock vb, int) { scatter_body(a, vb); });
}

__global__ void __launch_bounds__(kThreads) persist_rho_kernel(PersistQueue q, const RhoArgs *recs) {
    persist_loop(q, recs, [](const RhoArgs &a, VBlock vb, int) {
        rho_body(a, vb);
        if (arrive_last(a.counter, vb.n)) rho_fold(a, vb.n);
    });
}

__global__ void __launch_bounds__(kThreads, 4) persist_gather_kernel(PersistQueue q, const GatherArgs *recs) {
    persist_loop(q, recs, [](const GatherArgs &a, VBlock vb, int) {
        gather_body(a, vb);
        if (arrive_last(a.counter, vb.n)) gather_fold(a, vb.n);
    });
}

int persist_density_wave(int stage) {
    static int waves[4] = {0, 0, 0, 0};
    switch (stage) {
    case PS_UPDATE:
        if (!waves[0]) waves[0] = wave_of((const void *)persist_update_kernel, kThreads, 1216);
        return waves[0];
    case PS_SCATTER:
        // two blocks per SM, not the three that fit: the WA launches run
        // beside the scatter and need shared memory and warp slots too
        if (!waves[1]) {
            cudaFuncSetAttribute(persist_scatter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kScatterSmem);
            int dev = 0, sms = 0;
            const int full = wave_of((const void *)persist_scatter_kernel, kScatterThreads, 304, kScatterSmem);
            if (cudaGetDevice(&dev) == cudaSuccess &&
                cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && sms > 0)
                waves[1] = std::min(full, 2 * sms);
            else
                waves[1] = full;
        }
        return waves[1];
    case PS_RHO:
        if (!waves[2]) waves[2] = wave_of((const void *)persist_rho_kernel, kThreads, 1216);
        return waves[2];
    case PS_GATHER:
        if (!waves[3]) waves[3] = wave_of((const void *)persist_gather_kernel, kThreads, 608);
        return waves[3];
    default:
        return 0;
    }
}

void launch_persist_density(int stage, const PersistQueue &q, const void *recs, cudaStream_t st) {
    const int w = persist_density_wave(stage);
    switch (stage) {
    case PS_UPDATE:
        persist_update_kernel<<<w, kThreads, 0, st>>>(q, static_cast<const ScatterArgs *>(recs));
        break;
    case PS_SCATTER:
        persist_scatter_kernel<<<w, kScatterThreads, kScatterSmem, st>>>(q, static_cast<const ScatterArgs *>(recs));
        break;
    case PS_RHO:
        persist_rho_kernel<<<w, kThreads, 0, st>>>(q, static_cast<const RhoArgs *>(recs));
        break;
    case PS_GATHER:
        persist_gather_kernel<<<w, kThreads, 0, st>>>(q, static_cast<const GatherArgs *>(recs));
        break;
    default:
        break;
    }
}

}  // namespace ap

/* Self-check of the conversion helpers; no counterpart in the reference.
 * mismatches[0..5]: f2i_rn_bits, f2i_rz_bits, ll2f_rn_bits, grad_q,
 * i64_to_float (small and any int64), f2i_rz_small, each over `samples`
 * hashed inputs. */
extern "C" int ap_selftest_numerics(int32_t *mismatches, int64_t samples) {
    if (!mismatches || samples <= 0 || samples > (1ll << 32)) return 1;  // AP_ERR_INVALID_ARG
    int *d = nullptr;
    if (cudaMalloc(&d, 6 * sizeof(int)) != cudaSuccess) return 4;  // AP_ERR_CUDA
    int rc = 0;
    if (cudaMemset(d, 0, 6 * sizeof(int)) != cudaSuccess) rc = 4;
    if (!rc) {
        ap::numerics_selftest_kernel<<<152 * 8, ap::kThreads>>>(samples, 0x243F6A8885A308D3ull, d);
        if (cudaGetLastError() != cudaSuccess || cudaMemcpy(mismatches, d, 6 * sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = 4;
    }
    cudaFree(d);
    return rc;
}
