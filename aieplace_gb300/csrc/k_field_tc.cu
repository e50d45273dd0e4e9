// Electrostatic field solve on the 5th-generation tensor cores (sm_103a).
//
// Same four contraction stages as the FP32 path (k_field_simt.cu, restating
// replace::FFT::doFFT, python/AIEmath/fft_replace/fft.cpp:204-299), each
//   D[i][j] = sum_k A[i][k] B[j][k]
// with A a constant transform matrix and B the data, both stored as a BF16
// pair (hi = bf16(x), lo = bf16(x - hi)).  Every k-step issues three MMAs into
// one FP32 accumulator in tensor memory: A_hi B_hi + A_hi B_lo + A_lo B_hi
// (the "bf16x3" split; the dropped A_lo B_lo term is 2^-16 relative).
//
// Kernel layout (a 128 x BN output tile per cluster of S CTAs, 4 warps each;
// the S CTAs split K):
//   warp 0 lane 0   TMA producer: 4-stage ring of {A_hi, A_lo, B_hi, B_lo}
//                   128B-swizzled K-major tiles, mbarrier complete_tx
//   warp 1 lane 0   MMA issuer: tcgen05.mma.cta_group::1.kind::f16, M=128,
//                   N=64, K=16; tcgen05.commit frees stages / signals the end
//   warps 0-3       epilogue: tcgen05.ld 32x32b (warp w owns TMEM lanes
//                   32w..32w+31 = output rows); CTA r of the cluster finishes
//                   rows [r 128/S, (r+1) 128/S): once every CTA of the cluster
//                   is past its K loop (cluster barrier), every CTA stores its partial
//                   of those rows into CTA r's shared memory (distributed
//                   shared memory, slot = source rank); cluster barrier; CTA
//                   r sums its S slots in rank order, applies the stage
//                   epilogue and stores a warp per row, coalesced
// Every mbarrier wait is bounded; a wait that gives up sets the solver's
// status word and the CTA drains and exits without further issue.
//
// A second form, persist_solve_kernel, runs the four stages as one launch
// (tiles claimed from a device queue, row-block dependency counters between
// the stages, TMA tile stores); the tile autotuner times it beside the
// four-launch shapes and keeps whichever is fastest.
#include <cuda.h>

#include <algorithm>
#include <cudaTypedefs.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "../../include/aieplace.h"
#include "ap_kernels.h"

namespace ap {
namespace tc {

constexpr int BM = 128, BK = 64, THREADS = 128;
constexpr int A_TILE = BM * BK * 2;                   // 16 KB
constexpr unsigned long long WAIT_NS = 2000000000ull;  // 2 s bound on any single wait

// Output tile 128 x BN; the accumulator takes BN TMEM columns.  Both shapes
// fit one CTA per SM; field_solver_bind_bf16 times them and keeps the faster.
template <int BN_, int STAGES_>
struct TileCfg {
    static constexpr int BN = BN_, STAGES = STAGES_;
    static constexpr int B_TILE = BN * BK * 2;
    static constexpr int STAGE_BYTES = 2 * A_TILE + 2 * B_TILE;
    static constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 256;
    static constexpr uint32_t TMEM_COLS = BN;
};
using Tile64 = TileCfg<64, 4>;    // 48 KB stages
using Tile128 = TileCfg<128, 3>;  // 64 KB stages
using Tile64x2 = TileCfg<64, 2>;  // 2 stages, ~97 KB: two CTAs per SM
// variants 0-2: the four-launch solve with these tiles; 3, 4: the persistent
// solve (one launch) with Tile128 pipelines, stages 1-2 with K split in two (3)
// or not (4)
constexpr int kTcVariants = kTcCandidates;

enum { EPI_SPLIT = 0, EPI_SPECTRAL = 1, EPI_F32 = 2 };

struct Maps {
    CUtensorMap a_hi[2], a_lo[2], b_hi[2], b_lo[2];
};

struct Epi {
    int m;
    int mode;
    int split;  // S: CTAs per cluster splitting K (the cluster's x extent)
    __nv_bfloat16 *o_hi[2], *o_lo[2];  // EPI_SPLIT; EPI_SPECTRAL: [0] = Px, [1] = Py
    float *o_f32[2];                   // EPI_F32
    const float *wx, *wy;
    float scale;
    unsigned int *status;
    const int *gate;  // run only if gate is null or (1 << *gate) & gate_mask
    int gate_mask;
    int pdl;  // launched as a programmatic dependent of the previous stage
    // failure injection (tests of the timeout path): the load issuer issues
    // nothing, so the MMA issuer's wait for data runs out after wait_ns with
    // no copy in flight
    int skip_loads;
    unsigned long long wait_ns;  // bound on any single mbarrier wait
};

// ---- PTX wrappers ----------------------------------------------------------

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: false (and the status flag set) if the phase did not complete
// within wait_ns.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, unsigned int *status,
                                          unsigned long long wait_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (;;) {
        for (int i = 0; i < 64; ++i)
            if (mbar_try_wait(bar, parity)) return true;
        if (global_ns() - t0 > wait_ns) {
            atomicOr(status, 1u);
            return false;
        }
    }
}

__device__ __forceinline__ void tma_load_2d(const CUtensorMap *map, uint64_t *bar, void *dst, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
            smem_u32(dst)),
        "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}

__device__ __forceinline__ void tma_prefetch(const CUtensorMap *map) {
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)map) : "memory");
}

__device__ __forceinline__ void cluster_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// shared::cluster address of the same offset in CTA `rank` of the cluster
__device__ __forceinline__ uint32_t map_rank(uint32_t local, int rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local), "r"(rank));
    return r;
}

__device__ __forceinline__ void st_shared_f4(uint32_t addr, float4 v) {
    asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w)
                 : "memory");
}

__device__ __forceinline__ void st_cluster_f4(uint32_t addr, float4 v) {
    asm volatile("st.shared::cluster.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "f"(v.x), "f"(v.y), "f"(v.z),
                 "f"(v.w)
                 : "memory");
}

// explicit shared-space loads: a generic load could alias the epilogue's
// global stores and would wait for them
__device__ __forceinline__ float2 ld_shared_f2(uint32_t addr) {
    float2 v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr));
    return v;
}

__device__ __forceinline__ void st_shared_f1(uint32_t addr, float v) {
    asm volatile("st.shared.f32 [%0], %1;" ::"r"(addr), "f"(v) : "memory");
}

__device__ __forceinline__ float ld_shared_f1(uint32_t addr) {
    float v;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(addr));
    return v;
}

// explicit global stores: a generic store could alias shared memory, and the
// staging loads that follow it would wait for it
__device__ __forceinline__ float4 ld_shared_f4(uint32_t addr) {
    float4 v;
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(addr));
    return v;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// K-major operand in the 128B-swizzled canonical layout: 8-row x 128-byte
// atoms stacked along M/N every 1024 bytes (stride byte offset), the leading
// byte offset unused for swizzled K-major operands, descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;             // leading byte offset (16 B, ignored here)
    d |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset
    d |= (uint64_t)1 << 46;             // descriptor version
    d |= (uint64_t)2 << 61;             // 128-byte swizzle
    return d;
}

// kind::f16 instruction descriptor: D f32, A and B bf16, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
        "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
          "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
          "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
          "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&v);
}

// VEC FP32 values -> hi/lo BF16 (VEC = 2 or 4 consecutive outputs)
template <int VEC>
__device__ __forceinline__ void store_split_vec(const float (&v)[VEC], __nv_bfloat16 *hi, __nv_bfloat16 *lo) {
    uint32_t h[VEC / 2], l[VEC / 2];
#pragma unroll
    for (int i = 0; i < VEC / 2; ++i) {
        const __nv_bfloat16 a = __float2bfloat16_rn(v[2 * i]), b = __float2bfloat16_rn(v[2 * i + 1]);
        const __nv_bfloat162 hp = __halves2bfloat162(a, b);
        h[i] = *reinterpret_cast<const uint32_t *>(&hp);
        l[i] = pack_bf16(v[2 * i] - __bfloat162float(a), v[2 * i + 1] - __bfloat162float(b));
    }
    if (VEC == 4) {
        *reinterpret_cast<uint2 *>(hi) = make_uint2(h[0], h[VEC / 2 - 1]);
        *reinterpret_cast<uint2 *>(lo) = make_uint2(l[0], l[VEC / 2 - 1]);
    } else {
        *reinterpret_cast<uint32_t *>(hi) = h[0];
        *reinterpret_cast<uint32_t *>(lo) = l[0];
    }
}

// Two adjacent FP32 outputs -> their BF16 hi and lo pairs (4-byte stores)
// Output pointers of one CTA's stage epilogue, resolved before the row loop:
// indexing the parameter block by blockIdx.z inside the loop made the compiler
// copy it to local memory.
struct EpiOut {
    int m, mode;
    float *f32;
    __nv_bfloat16 *hi0, *lo0, *hi1, *lo1;
    float scale;
};

// Stage epilogue of VEC consecutive outputs (row, col..col+VEC-1); a warp
// covers one row's BN columns, so each store instruction writes one
// contiguous 128-512 byte segment.  wx, wy: the row's and the columns'
// spectral frequencies (EPI_SPECTRAL).
template <int VEC>
__device__ __forceinline__ void epi_store(const EpiOut &o, int row, int col, const float (&v)[VEC], float wx,
                                          const float (&wy)[VEC]) {
    const size_t off = (size_t)row * o.m + col;
    if (o.mode == EPI_F32) {
        if (VEC == 4)
            *reinterpret_cast<float4 *>(o.f32 + off) = make_float4(v[0], v[1], v[VEC - 2], v[VEC - 1]);
        else
            *reinterpret_cast<float2 *>(o.f32 + off) = make_float2(v[0], v[1]);
    } else if (o.mode == EPI_SPLIT) {
        store_split_vec<VEC>(v, o.hi0 + off, o.lo0 + off);
    } else {
        // spectral scaling of fft.cpp:217-273: halve row/column 0, 4/(Mx My),
        // phi = a / (wx^2 + wy^2), Px = phi wx, Py = phi wy (straight-line
        // 2-ulp division: the IEEE divide's slow path is a call)
        const float rs = row == 0 ? 0.5f * o.scale : o.scale;
        float px[VEC], py[VEC];
#pragma unroll
        for (int i = 0; i < VEC; ++i) {
            float c = v[i] * rs;
            if (col + i == 0) c *= 0.5f;
            const float den = wx * wx + wy[i] * wy[i];
            c = den > 0.f ? __fdividef(c, den) : 0.f;
            px[i] = c * wx;
            py[i] = c * wy[i];
        }
        store_split_vec<VEC>(px, o.hi0 + off, o.lo0 + off);
        store_split_vec<VEC>(py, o.hi1 + off, o.lo1 + off);
    }
}

template <class T>
__global__ void __launch_bounds__(THREADS, 1) gemm_bf16x3_kernel(const __grid_constant__ Maps maps, Epi e) {
    // uniform for the whole grid, before any barrier or TMEM allocation
    if (e.gate && !((1 << *e.gate) & e.gate_mask)) return;
    constexpr int BN = T::BN, STAGES = T::STAGES, STAGE_BYTES = T::STAGE_BYTES, B_TILE = T::B_TILE;
    constexpr uint32_t TMEM_COLS = T::TMEM_COLS;
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *full = (uint64_t *)(smem + STAGES * STAGE_BYTES);
    uint64_t *empty = full + STAGES;
    uint64_t *done = empty + STAGES;
    uint32_t *tmem_slot = (uint32_t *)(done + 1);
    volatile int *abort_flag = (volatile int *)(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int z = blockIdx.z;
    // cluster of S CTAs along x: rank r accumulates k-blocks [r nk, (r+1) nk)
    const int S = e.split, rank = (int)blockIdx.x % S;
    const int n0 = ((int)blockIdx.x / S) * BN, m0 = blockIdx.y * BM;
    const int nk = e.m / BK / S, kb0 = rank * nk;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(full + s, 1);
            mbar_init(empty + s, 1);
        }
        mbar_init(done, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        tma_prefetch(&maps.a_hi[z]);
        tma_prefetch(&maps.a_lo[z]);
        tma_prefetch(&maps.b_hi[z]);
        tma_prefetch(&maps.b_lo[z]);
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    // A programmatic dependent (stages 2-4) starts as SMs free up while the
    // previous stage finishes, and has its barriers and TMEM set up by then;
    // the previous stage's outputs are this stage's data, so nothing is
    // loaded or stored before that grid has completed.
    if (e.pdl) asm volatile("griddepcontrol.wait;" ::: "memory");

    int issued = 0;  // producer: k-blocks whose loads were issued
    if (warp == 0 && lane == 0) {
        const int nk_issue = e.skip_loads ? 0 : nk;
        for (int kb = 0; kb < nk_issue; ++kb) {
            const int s = kb % STAGES, round = kb / STAGES;
            if (round > 0 && !mbar_wait(empty + s, (round - 1) & 1, e.status, e.wait_ns)) {
                *abort_flag = 1;
                break;
            }
            if (*abort_flag) break;
            uint8_t *st = smem + s * STAGE_BYTES;
            mbar_expect_tx(full + s, STAGE_BYTES);
            const int kx = (kb0 + kb) * BK;
            tma_load_2d(&maps.a_hi[z], full + s, st, kx, m0);
            tma_load_2d(&maps.a_lo[z], full + s, st + A_TILE, kx, m0);
            tma_load_2d(&maps.b_hi[z], full + s, st + 2 * A_TILE, kx, n0);
            tma_load_2d(&maps.b_lo[z], full + s, st + 2 * A_TILE + B_TILE, kx, n0);
            issued = kb + 1;
        }
    } else if (warp == 1 && lane == 0) {
        constexpr uint32_t idesc = idesc_bf16(BM, BN);
        for (int kb = 0; kb < nk; ++kb) {
            const int s = kb % STAGES, round = kb / STAGES;
            if (!mbar_wait(full + s, round & 1, e.status, e.wait_ns)) {
                *abort_flag = 1;
                break;
            }
            tc_fence_after();
            const uint32_t base = smem_u32(smem + s * STAGE_BYTES);
            const uint64_t ahi = smem_desc(base), alo = smem_desc(base + A_TILE);
            const uint64_t bhi = smem_desc(base + 2 * A_TILE), blo = smem_desc(base + 2 * A_TILE + B_TILE);
#pragma unroll
            for (int k = 0; k < BK / 16; ++k) {
                const uint64_t adv = (uint64_t)((k * 32) >> 4);  // 16 bf16 = 32 bytes along K
                mma_bf16(tmem, ahi + adv, bhi + adv, idesc, (kb | k) != 0);
                mma_bf16(tmem, ahi + adv, blo + adv, idesc, 1u);
                mma_bf16(tmem, alo + adv, bhi + adv, idesc, 1u);
            }
            mma_commit(empty + s);  // stage s reusable once these MMAs have read it
        }
        mma_commit(done);  // accumulator complete (or, after an abort, all issued MMAs retired)
    }
    __syncwarp();

    // ---- epilogue ----------------------------------------------------------
    // twice the bound of the K loop's waits: an MMA issuer whose wait for data
    // ran out commits `done` before any wait on `done` can give up, so no
    // thread leaves with that arrival still pending
    const bool ok = mbar_wait(done, 0, e.status, 2 * e.wait_ns) && !*abort_flag;
    // the next stage may be scheduled once every CTA of this one is here
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    tc_fence_after();
    // The pipeline buffers are free once the accumulator is complete (every
    // issued load landed and was read): they hold the FP32 staging slots,
    // slot q (source rank) x 128/S rows, row stride BN + 4 floats (16-byte
    // rows, conflict-free v4 stores).
    constexpr int LD = BN + 4, VEC = BN / 32;
    static_assert(BM * LD * 4 <= STAGES * STAGE_BYTES, "staging tile fits the pipeline buffers");
    const uint32_t stg = smem_u32(smem);
    const int RS = BM / S;  // rows finished per CTA
    // a peer's pipeline buffers are free only once its accumulator is
    // complete too: no partial goes out before every CTA of the cluster is
    // past its K loop
    if (S > 1) cluster_sync();
    if (ok) {
        const int row = warp * 32 + lane, dst = row / RS, lr = row - dst * RS;
        const uint32_t la = stg + (uint32_t)(((rank * RS + lr) * LD) * 4);
        const uint32_t ra = dst == rank ? la : map_rank(la, dst);
#pragma unroll
        for (int c0 = 0; c0 < BN; c0 += 32) {
            uint32_t r[32];
            tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, r);
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const float4 v = make_float4(__uint_as_float(r[4 * i]), __uint_as_float(r[4 * i + 1]),
                                             __uint_as_float(r[4 * i + 2]), __uint_as_float(r[4 * i + 3]));
                const uint32_t off = (uint32_t)((c0 + 4 * i) * 4);
                if (dst == rank)
                    st_shared_f4(la + off, v);
                else
                    st_cluster_f4(ra + off, v);
            }
        }
    }
    // every CTA of the cluster arrives on every path (an aborted CTA too);
    // release/acquire makes the peers' slot stores visible
    if (S > 1)
        cluster_sync();
    else
        __syncthreads();
    if (ok) {
        // this CTA's rows, the S slots summed in rank order; a warp per row,
        // VEC columns per lane.  Pointers and frequencies go to registers
        // first: the loop reads nothing but shared memory.
        EpiOut o;
        o.m = e.m;
        o.mode = e.mode;
        o.scale = e.scale;
        o.f32 = z ? e.o_f32[1] : e.o_f32[0];
        const bool two = e.mode == EPI_SPECTRAL;  // Px and Py
        o.hi0 = (z && !two) ? e.o_hi[1] : e.o_hi[0];
        o.lo0 = (z && !two) ? e.o_lo[1] : e.o_lo[0];
        o.hi1 = e.o_hi[1];
        o.lo1 = e.o_lo[1];
        float wy[VEC], wx_lane = 0.f;
#pragma unroll
        for (int i = 0; i < VEC; ++i) wy[i] = 0.f;
        if (two) {
#pragma unroll
            for (int i = 0; i < VEC; ++i) wy[i] = __ldg(e.wy + n0 + lane * VEC + i);
            // lane k holds the frequency of this warp's k-th row (<= 32 rows)
            const int lr = warp + (THREADS / 32) * lane;
            if (lr < RS) wx_lane = __ldg(e.wx + m0 + rank * RS + lr);
        }
        // rows lr = warp + 4 k; four rows a batch, every slot load of the
        // batch issued before the first add (one load in flight per row
        // measured ~250 cycles a row)
        constexpr int NR = 4, W = THREADS / 32;
        static_assert(BM % (NR * W * 4) == 0, "rows per warp a multiple of the batch for S <= 4");
        for (int k0 = 0; warp + k0 * W < RS; k0 += NR) {
            float p[4][NR][VEC];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (q < S) {
#pragma unroll
                    for (int j = 0; j < NR; ++j) {
                        const int lr = warp + (k0 + j) * W;
                        const uint32_t a = stg + (uint32_t)((((q * RS + lr) * LD) + lane * VEC) * 4);
                        if (VEC == 4) {
                            const float4 t = ld_shared_f4(a);
                            p[q][j][0] = t.x;
                            p[q][j][1] = t.y;
                            p[q][j][VEC - 2] = t.z;
                            p[q][j][VEC - 1] = t.w;
                        } else {
                            const float2 t = ld_shared_f2(a);
                            p[q][j][0] = t.x;
                            p[q][j][VEC - 1] = t.y;
                        }
                    }
                }
            }
#pragma unroll
            for (int j = 0; j < NR; ++j) {
                const int lr = warp + (k0 + j) * W;
                float acc[VEC];
#pragma unroll
                for (int i = 0; i < VEC; ++i) acc[i] = 0.f;
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (q < S) {
#pragma unroll
                        for (int i = 0; i < VEC; ++i) acc[i] += p[q][j][i];
                    }
                const float wx = __shfl_sync(0xffffffffu, wx_lane, (k0 + j) & 31);
                epi_store<VEC>(o, m0 + rank * RS + lr, n0 + lane * VEC, acc, wx, wy);
            }
        }
    }
    // (no second cluster barrier: peers write this CTA's slots only before
    // the one above, whose release orders those stores ahead of its arrival)
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x == 0 && issued > 0) {
        // after an abort, let every issued load land before the CTA exits
        for (int kb = issued - 1; kb >= 0 && kb >= issued - STAGES; --kb)
            mbar_wait(full + (kb % STAGES), (kb / STAGES) & 1, e.status, e.wait_ns);
    }
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

// ---- persistent dataflow solve ------------------------------------------------
//
// All four stages in one launch of at most one CTA per SM, 128 x 128 output
// tiles.  The work items are the stages' output tiles in a fixed order
// (stage; row block; the product z of stages 3-4; column block; for stages
// 1-2 with K split, the half of K), claimed one at a time from a device
// queue.  The data operand of a tile (mb, nb) of stage s > 1 is rows
// [nb BN, nb BN + BN) of stage s-1's output: row block R = nb BN / 128 of
// that stage, complete once the four epilogue warps of each of its m / BN
// tiles have stored their rows and each bumped the row block's counter.  An
// item waits only on items of lower index, and those were claimed earlier by
// CTAs that are running, so the lowest unfinished item always proceeds,
// however many of the CTAs are resident (other kernels, or another
// instance's solve in a batch, may hold SMs).
//
// Stages 1-2 have only (m/128)^2 tiles -- 64 at 1024^2 bins, against 152 SMs
// -- so with ks = 2 each of their tiles is two items, one per half of K.  Both
// halves store their FP32 partial (a per-stage scratch); the epilogue warp
// that arrives second on the tile's counter (one counter per warp, its 32
// rows) adds partial 0 and partial 1 in that order -- the same bits whichever
// half ends first -- and finishes the rows.
//
// Warps 0-3 epilogue (TMEM lanes 32w..32w+31 = rows), warp 4 lane 0 TMA
// producer (it claims the items and hands them to the other roles through a
// ring of kItemRing slots), warp 5 lane 0 MMA issuer.  Two accumulators in
// TMEM: the epilogue of one tile runs while the MMAs of the CTA's next tile
// fill the other, and the producer's ring of pipeline stages runs on across
// tiles.  Every wait is bounded; one that gives up sets the solver's status
// word, and the other CTAs' dependency waits then give up at once.

constexpr int P_THREADS = 192;
constexpr int P_STG_FLOATS = 4 * 32 * 33;  // per epilogue warp: 32 rows x 32 columns, row stride 33
constexpr int kItemRing = 4;

template <class T>
struct PCfg {
    static constexpr int SMEM_BYTES = T::STAGES * T::STAGE_BYTES + P_STG_FLOATS * 4 + 1024 + 512;
};

// outputs of the persistent solve, 32 x 32 boxes (stores): [0, 1] T hi/lo,
// [2, 3] Px hi/lo, [4, 5] Py hi/lo, [6, 7] Ux hi/lo, [8, 9] Uy hi/lo, [10, 11] Ex, Ey
enum { OUT_T = 0, OUT_PX = 2, OUT_PY = 4, OUT_UX = 6, OUT_UY = 8, OUT_EX = 10, kOutMaps = 12 };
constexpr int kBox = 32;

struct PMaps {
    Maps st[4];
    CUtensorMap out[kOutMaps];
};

struct PEpi {
    int m;
    int ks;  // K split of stages 1-2 (1 or 2)
    // the outputs are written through the tile-store maps of PMaps::out
    const float *wx, *wy;
    float scale;
    unsigned int *status;
    // [0] the item queue's head; [1] CTAs finished; [2 + (2 s + z) nM + R]
    // epilogue warps (four a tile) done with stage s, product z, row block R;
    // then, with ks = 2, [2 + 8 nM + 4 (s tiles + tile) + warp] halves of
    // stage s < 2's tile whose partial rows of that warp are stored.  The
    // last CTA to finish zeroes them all.
    unsigned int *sync;
    float *part;  // ks = 2: FP32 partials [stage][half][tile][128 x BN]
    const int *gate;
    int gate_mask;
    int skip_loads;
    unsigned long long wait_ns;
};

struct PItem {
    int s, z, mb, nb, kh;
};

__device__ __forceinline__ PItem p_item(int t, int nM, int nN, int ks) {
    const int one = nM * nN;  // tiles of a product; stages 3 and 4 have two products
    PItem it;
    it.kh = 0;
    it.z = 0;
    if (t < 2 * ks * one) {
        it.s = t / (ks * one);
        const int r = t - it.s * ks * one;
        const int tile = r / ks;
        it.kh = r - tile * ks;
        it.mb = tile / nN;
        it.nb = tile - it.mb * nN;
    } else {
        int r = t - 2 * ks * one;
        it.s = r < 2 * one ? 2 : 3;
        if (it.s == 3) r -= 2 * one;
        it.mb = r / (2 * nN);
        const int q = r - it.mb * 2 * nN;
        it.z = q / nN;
        it.nb = q - it.z * nN;
    }
    return it;
}

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int *p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Bounded wait that also gives up once the CTA is aborting.
__device__ __forceinline__ bool mbar_wait_ab(uint64_t *bar, uint32_t parity, unsigned int *status,
                                             unsigned long long wait_ns, volatile int *abort_flag) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (;;) {
        for (int i = 0; i < 64; ++i)
            if (mbar_try_wait(bar, parity)) return true;
        if (*abort_flag) return false;
        if (global_ns() - t0 > wait_ns) {
            atomicOr(status, 1u);
            *abort_flag = 1;
            return false;
        }
    }
}

// Until the row block's counter reaches `need`; false once the wait ran out,
// this CTA is aborting or another CTA reported a failure.
__device__ __forceinline__ bool dep_wait(const unsigned int *c, unsigned int need, unsigned int *status,
                                         unsigned long long wait_ns, volatile int *abort_flag) {
    if (ld_acquire_u32(c) >= need) return true;
    const unsigned long long t0 = global_ns();
    for (;;) {
        for (int i = 0; i < 16; ++i) {
            if (ld_acquire_u32(c) >= need) return true;
            __nanosleep(100);
        }
        if (*abort_flag || *(volatile unsigned int *)status != 0u) return false;
        if (global_ns() - t0 > wait_ns) {
            atomicOr(status, 1u);
            return false;
        }
    }
}

// tile stores by the tensor memory accelerator: shared -> global, one
// bulk group per issuing thread
__device__ __forceinline__ void tma_store_2d(const CUtensorMap *map, uint32_t src, int x, int y) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];" ::"l"((uint64_t)map),
                 "r"(src), "r"(x), "r"(y)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// the issued stores have read their shared-memory source
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// the issued stores are complete in global memory
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void st_shared_u32(uint32_t addr, uint32_t v) {
    asm volatile("st.shared.b32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
}
__device__ __forceinline__ void st_shared_f2(uint32_t addr, float a, float b) {
    asm volatile("st.shared.v2.f32 [%0], {%1, %2};" ::"r"(addr), "f"(a), "f"(b) : "memory");
}

__device__ __forceinline__ void st_global_f4(float *p, float4 v) {
    asm volatile("st.global.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w)
                 : "memory");
}

template <class T>
__global__ void __launch_bounds__(P_THREADS, 1) persist_solve_kernel(const __grid_constant__ PMaps maps, PEpi e) {
    // uniform for the whole grid, before any barrier or TMEM allocation
    if (e.gate && !((1 << *e.gate) & e.gate_mask)) return;
    constexpr int BN = T::BN, STAGES = T::STAGES, STAGE_BYTES = T::STAGE_BYTES, B_TILE = T::B_TILE;
    constexpr uint32_t TMEM_COLS = 2 * BN;  // two accumulators
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    float *stg = (float *)(smem + STAGES * STAGE_BYTES);
    uint64_t *full = (uint64_t *)(stg + P_STG_FLOATS);
    uint64_t *empty = full + STAGES;
    uint64_t *acc_full = empty + STAGES;  // [2]
    uint64_t *acc_empty = acc_full + 2;   // [2]
    uint64_t *drain = acc_empty + 2;
    uint64_t *item_full = drain + 1;               // [kItemRing], the producer's arrival
    uint64_t *item_empty = item_full + kItemRing;  // [kItemRing], MMA issuer + 4 epilogue warps
    uint32_t *tmem_slot = (uint32_t *)(item_empty + kItemRing);
    volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
    volatile int *issued_kb = abort_flag + 1;    // producer: k-blocks whose loads were issued
    volatile int *consumed_kb = abort_flag + 2;  // MMA issuer: k-blocks whose data it waited for
    volatile int *item_ring = abort_flag + 3;    // [kItemRing] claimed items (>= total: no more)

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m = e.m, nM = m / BM, nN = m / BN, nk = m / BK, ks = e.ks;
    const int one = nM * nN, total = 2 * ks * one + 4 * one, G = (int)gridDim.x;
    unsigned int *queue = e.sync, *finished = e.sync + 1, *rows_done = e.sync + 2;
    unsigned int *halves = rows_done + 8 * nM;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(full + s, 1);
            mbar_init(empty + s, 1);
        }
        mbar_init(acc_full + 0, 1);
        mbar_init(acc_full + 1, 1);
        mbar_init(acc_empty + 0, 128);
        mbar_init(acc_empty + 1, 128);
        mbar_init(drain, 1);
        for (int q = 0; q < kItemRing; ++q) {
            mbar_init(item_full + q, 1);
            mbar_init(item_empty + q, 5);
        }
        *abort_flag = 0;
        *issued_kb = 0;
        *consumed_kb = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 4 && lane == 0) {
        // ---- TMA producer
        int g = 0;
        for (int j = 0; !*abort_flag; ++j) {
            const int q = j % kItemRing;
            if (j >= kItemRing && !mbar_wait_ab(item_empty + q, ((j / kItemRing) - 1) & 1, e.status, e.wait_ns,
                                                abort_flag))
                break;
            // failure injection: no item is taken, so the other roles' waits run out
            int t = e.skip_loads ? -1 : (int)atomicAdd(queue, 1u);
            if (t > total) t = total;
            if (t < 0) break;
            item_ring[q] = t;
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(item_full + q)) : "memory");
            if (t >= total) break;
            {
                const PItem it = p_item(t, nM, nN, ks);
                if (it.s > 0) {
                    // stage 2 and both products of stage 3 read stage 1 / stage 2's
                    // single product; product z of stage 4 reads product z of stage 3
                    const int zd = it.s == 3 ? it.z : 0;
                    const unsigned int *c = rows_done + (2 * (it.s - 1) + zd) * nM + (it.nb * BN) / BM;
                    if (!dep_wait(c, 4u * (unsigned int)nN, e.status, e.wait_ns, abort_flag)) {
                        *abort_flag = 1;
                        break;
                    }
                    // the previous stage's generic-proxy stores, acquired above,
                    // before this thread's tensor (async-proxy) loads of them
                    asm volatile("fence.proxy.async.global;" ::: "memory");
                }
                const Maps &mp = maps.st[it.s];
                const int z = it.z, ay = it.mb * BM, by = it.nb * BN;
                const int nki = it.s < 2 ? nk / ks : nk, kb0 = it.kh * nki;
                bool ok = true;
                for (int kb = 0; kb < nki; ++kb, ++g) {
                    const int s = g % STAGES, round = g / STAGES;
                    if (round > 0 && !mbar_wait_ab(empty + s, (round - 1) & 1, e.status, e.wait_ns, abort_flag)) {
                        ok = false;
                        break;
                    }
                    uint8_t *st = smem + s * STAGE_BYTES;
                    mbar_expect_tx(full + s, STAGE_BYTES);
                    const int kx = (kb0 + kb) * BK;
                    tma_load_2d(&mp.a_hi[z], full + s, st, kx, ay);
                    tma_load_2d(&mp.a_lo[z], full + s, st + A_TILE, kx, ay);
                    tma_load_2d(&mp.b_hi[z], full + s, st + 2 * A_TILE, kx, by);
                    tma_load_2d(&mp.b_lo[z], full + s, st + 2 * A_TILE + B_TILE, kx, by);
                    *issued_kb = g + 1;
                }
                if (!ok) break;
            }
        }
    } else if (warp == 5 && lane == 0) {
        // ---- MMA issuer
        constexpr uint32_t idesc = idesc_bf16(BM, BN);
        int g = 0;
        for (int j = 0; !*abort_flag; ++j) {
            const int q = j % kItemRing;
            if (!mbar_wait_ab(item_full + q, (j / kItemRing) & 1, e.status, e.wait_ns, abort_flag)) break;
            const int t = item_ring[q];
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(item_empty + q)) : "memory");
            if (t >= total) break;
            const int nki = t < 2 * ks * one ? nk / ks : nk;
            const int b = j & 1, u = j >> 1;
            if (u > 0 && !mbar_wait_ab(acc_empty + b, (u - 1) & 1, e.status, e.wait_ns, abort_flag)) break;
            tc_fence_after();
            const uint32_t d = tmem + (uint32_t)(b * BN);
            bool ok = true;
            for (int kb = 0; kb < nki; ++kb, ++g) {
                const int s = g % STAGES, round = g / STAGES;
                if (!mbar_wait_ab(full + s, round & 1, e.status, e.wait_ns, abort_flag)) {
                    ok = false;
                    break;
                }
                *consumed_kb = g + 1;
                tc_fence_after();
                const uint32_t base = smem_u32(smem + s * STAGE_BYTES);
                const uint64_t ahi = smem_desc(base), alo = smem_desc(base + A_TILE);
                const uint64_t bhi = smem_desc(base + 2 * A_TILE), blo = smem_desc(base + 2 * A_TILE + B_TILE);
#pragma unroll
                for (int k = 0; k < BK / 16; ++k) {
                    const uint64_t adv = (uint64_t)((k * 32) >> 4);  // 16 bf16 = 32 bytes along K
                    mma_bf16(d, ahi + adv, bhi + adv, idesc, (kb | k) != 0);
                    mma_bf16(d, ahi + adv, blo + adv, idesc, 1u);
                    mma_bf16(d, alo + adv, bhi + adv, idesc, 1u);
                }
                mma_commit(empty + s);  // stage s reusable once these MMAs have read it
            }
            if (!ok) break;
            mma_commit(acc_full + b);  // accumulator b complete
        }
        mma_commit(drain);  // every MMA this thread issued has retired
    } else if (warp < 4) {
        // ---- epilogue: a warp's 32 rows through its own staging rows (lane =
        // row -> lane = column), then two rows per store instruction, coalesced
        float *wst = stg + warp * 32 * 33;
        const uint32_t wst_s = smem_u32(wst);
        const int rl = warp * 32 + lane;  // this lane's row in the tile
        for (int j = 0;; ++j) {
            // one decision for the warp on every wait (its lanes poll on their
            // own, and the TMEM loads and warp syncs below need all of them)
            const int q = j % kItemRing;
            if (!__all_sync(0xffffffffu, mbar_wait_ab(item_full + q, (j / kItemRing) & 1, e.status, e.wait_ns,
                                                      abort_flag)))
                break;
            const int t = item_ring[q];
            __syncwarp();
            if (lane == 0)
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(item_empty + q)) : "memory");
            if (t >= total) break;
            const int b = j & 1, u = j >> 1;
            if (!__all_sync(0xffffffffu, mbar_wait_ab(acc_full + b, u & 1, e.status, e.wait_ns, abort_flag))) break;
            tc_fence_after();
            const PItem it = p_item(t, nM, nN, ks);
            const int row0 = it.mb * BM + warp * 32;
            const bool split = it.s < 2 && ks > 1;
            const int tile = it.mb * nN + it.nb;
            // spectral stage: this lane's row frequency (rows row0 + lane)
            const float wx_lane = it.s == 1 ? __ldg(e.wx + row0 + lane) : 0.f;
            const float rscale = e.scale;
            const size_t tile_elems = (size_t)BM * BN;
            float *part_mine = split ? e.part + ((size_t)(it.s * 2 + it.kh) * one + tile) * tile_elems : nullptr;

            // the staged 32 x 32 block of columns c0.. of this warp's rows ->
            // the stage's outputs: every staging load first, then the same
            // region holds the output boxes (32 x 32, row-major: two rows per
            // store instruction, two adjacent columns per lane, packed BF16
            // conversions), which lane 0 hands to the TMA as tile stores
            const int box_x0 = it.nb * BN, box_y = row0;
            auto store_chunk = [&](int c0) {
                const int half = lane >> 4, cp = 2 * (lane & 15);
                const int col = box_x0 + c0 + cp;
                float v[32];
#pragma unroll
                for (int k = 0; k < 16; ++k) {
                    const uint32_t sa = wst_s + (uint32_t)(((2 * k + half) * 33 + cp) * 4);
                    v[2 * k] = ld_shared_f1(sa);
                    v[2 * k + 1] = ld_shared_f1(sa + 4);
                }
                __syncwarp();  // the region is free for the boxes
                auto put_split = [&](int map) {
                    // hi box at +0, lo box at +2048 (64-byte rows)
#pragma unroll
                    for (int k = 0; k < 16; ++k) {
                        const float a = v[2 * k], b = v[2 * k + 1];
                        const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
                        const float2 hf = __bfloat1622float2(h);
                        const uint32_t o = (uint32_t)((2 * k + half) * 64 + cp * 2);
                        st_shared_u32(wst_s + o, *reinterpret_cast<const uint32_t *>(&h));
                        st_shared_u32(wst_s + 2048 + o, pack_bf16(a - hf.x, b - hf.y));
                    }
                    fence_async_smem();
                    __syncwarp();
                    if (lane == 0) {
                        tma_store_2d(&maps.out[map], wst_s, box_x0 + c0, box_y);
                        tma_store_2d(&maps.out[map + 1], wst_s + 2048, box_x0 + c0, box_y);
                        bulk_commit();
                        bulk_wait_read();
                    }
                    __syncwarp();
                };
                if (it.s == 3) {
#pragma unroll
                    for (int k = 0; k < 16; ++k)
                        st_shared_f2(wst_s + (uint32_t)((2 * k + half) * 128 + cp * 4), v[2 * k], v[2 * k + 1]);
                    fence_async_smem();
                    __syncwarp();
                    if (lane == 0) {
                        tma_store_2d(&maps.out[OUT_EX + it.z], wst_s, box_x0 + c0, box_y);
                        bulk_commit();
                        bulk_wait_read();
                    }
                    __syncwarp();
                } else if (it.s == 1) {
                    // spectral scaling of fft.cpp:217-273, as epi_store; Px then Py
                    const float wy0 = __ldg(e.wy + col), wy1 = __ldg(e.wy + col + 1);
                    float phi[32], wxr[16];
#pragma unroll
                    for (int k = 0; k < 16; ++k) {
                        const int lr = 2 * k + half, row = row0 + lr;
                        const float wx = __shfl_sync(0xffffffffu, wx_lane, lr);
                        const float rs = row == 0 ? 0.5f * rscale : rscale;
                        float v0 = v[2 * k] * rs, v1 = v[2 * k + 1] * rs;
                        if (col == 0) v0 *= 0.5f;
                        const float d0 = wx * wx + wy0 * wy0, d1 = wx * wx + wy1 * wy1;
                        phi[2 * k] = d0 > 0.f ? __fdividef(v0, d0) : 0.f;
                        phi[2 * k + 1] = d1 > 0.f ? __fdividef(v1, d1) : 0.f;
                        wxr[k] = wx;
                    }
#pragma unroll
                    for (int k = 0; k < 16; ++k) {
                        v[2 * k] = phi[2 * k] * wxr[k];
                        v[2 * k + 1] = phi[2 * k + 1] * wxr[k];
                    }
                    put_split(OUT_PX);
#pragma unroll
                    for (int k = 0; k < 16; ++k) {
                        v[2 * k] = phi[2 * k] * wy0;
                        v[2 * k + 1] = phi[2 * k + 1] * wy1;
                    }
                    put_split(OUT_PY);
                } else {
                    put_split(it.s == 0 ? OUT_T : (it.z ? OUT_UY : OUT_UX));
                }
            };

            bool finish = true;
#pragma unroll 1
            for (int c0 = 0; c0 < BN; c0 += 32) {
                uint32_t r[32];
                tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(b * BN + c0), r);
                if (c0 + 32 == BN) {
                    // accumulator b read out: the MMAs of a later tile may overwrite it
                    tc_fence_before();
                    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(acc_empty + b))
                                 : "memory");
                }
                if (split) {
                    // this half's partial of the lane's row, 128 contiguous bytes
                    float *pr = part_mine + (size_t)rl * BN + c0;
#pragma unroll
                    for (int i = 0; i < 8; ++i)
                        st_global_f4(pr + 4 * i, make_float4(__uint_as_float(r[4 * i]), __uint_as_float(r[4 * i + 1]),
                                                             __uint_as_float(r[4 * i + 2]),
                                                             __uint_as_float(r[4 * i + 3])));
                } else {
#pragma unroll
                    for (int i = 0; i < 32; ++i)
                        st_shared_f1(wst_s + (uint32_t)((lane * 33 + i) * 4), __uint_as_float(r[i]));
                    __syncwarp();
                    store_chunk(c0);
                    __syncwarp();
                }
            }
            if (split) {
                // the second of the two halves (per warp: its 32 rows) adds the
                // partials in a fixed order and finishes the rows
                __threadfence();
                __syncwarp();
                unsigned int prior = 0;
                if (lane == 0) prior = atomicAdd(halves + 4 * (it.s * one + tile) + warp, 1u);
                prior = __shfl_sync(0xffffffffu, prior, 0);
                finish = prior == 1u;
                if (finish) {
                    __threadfence();
                    const float *p0 = e.part + ((size_t)(it.s * 2 + 0) * one + tile) * tile_elems + (size_t)rl * BN;
                    const float *p1 = e.part + ((size_t)(it.s * 2 + 1) * one + tile) * tile_elems + (size_t)rl * BN;
#pragma unroll 1
                    for (int c0 = 0; c0 < BN; c0 += 32) {
                        float4 a[8], c[8];
#pragma unroll
                        for (int i = 0; i < 8; ++i) {
                            a[i] = __ldcg(reinterpret_cast<const float4 *>(p0 + c0) + i);
                            c[i] = __ldcg(reinterpret_cast<const float4 *>(p1 + c0) + i);
                        }
#pragma unroll
                        for (int i = 0; i < 8; ++i) {
                            const uint32_t sa = wst_s + (uint32_t)((lane * 33 + 4 * i) * 4);
                            st_shared_f1(sa, a[i].x + c[i].x);
                            st_shared_f1(sa + 4, a[i].y + c[i].y);
                            st_shared_f1(sa + 8, a[i].z + c[i].z);
                            st_shared_f1(sa + 12, a[i].w + c[i].w);
                        }
                        __syncwarp();
                        store_chunk(c0);
                        __syncwarp();
                    }
                }
            }
            if (finish && lane == 0) {
                // this warp's tile stores complete in global memory before its
                // count moves (their readers load them with the TMA too); each
                // epilogue warp counts for itself (no barrier across warps that
                // an abort could leave one of them waiting at)
                bulk_wait_all();
                asm volatile("fence.proxy.async.global;" ::: "memory");
                __threadfence();
                atomicAdd(rows_done + (2 * it.s + it.z) * nM + it.mb, 1u);
            }
            __syncwarp();
        }
        if (lane == 0) bulk_wait_all();  // no tile store in flight when the CTA leaves
    }
    __syncwarp();

    // ---- teardown: no MMA in flight, no load in flight, then TMEM back
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_wait(drain, 0, e.status, 2 * e.wait_ns);
        // loads issued but never waited for (after an abort): let them land
        for (int kb = *consumed_kb; kb < *issued_kb; ++kb)
            mbar_wait(full + (kb % STAGES), (kb / STAGES) & 1, e.status, e.wait_ns);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
    // the last CTA out leaves the queue and the counters at zero for the next solve
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(finished, 1u) == (unsigned int)G - 1u) {
            *queue = 0u;
            const int n = 8 * nM + (ks > 1 ? 8 * one : 0);
            for (int i = 0; i < n; ++i) rows_done[i] = 0u;
            __threadfence();
            *finished = 0u;
        }
    }
}

// ---- host side ---------------------------------------------------------------

PFN_cuTensorMapEncodeTiled_v12000 encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

// row-major m x m bf16 matrix, K (columns) innermost, box 64 x rows
bool make_map(CUtensorMap *map, const __nv_bfloat16 *base, int m, int box_rows) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = encoder();
    if (!enc || ((uintptr_t)base & 15)) return false;
    cuuint64_t dims[2] = {(cuuint64_t)m, (cuuint64_t)m};
    cuuint64_t strides[1] = {(cuuint64_t)m * 2};
    cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void *)base, dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

struct StageMaps {
    Maps s1, s2, s3, s4;
    CUtensorMap out[kOutMaps];  // the persistent solve's outputs ([10, 11]: set per call)
};

// m x m outputs of 2- or 4-byte elements, 32 x 32 boxes (tile stores)
bool make_out_map(CUtensorMap *map, void *base, bool f32, int m) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = encoder();
    if (!enc || ((uintptr_t)base & 15)) return false;
    const int elem = f32 ? 4 : 2;
    cuuint64_t dims[2] = {(cuuint64_t)m, (cuuint64_t)m};
    cuuint64_t strides[1] = {(cuuint64_t)m * elem};
    cuuint32_t box[2] = {(cuuint32_t)kBox, (cuuint32_t)kBox};
    cuuint32_t estr[2] = {1, 1};
    return enc(map, f32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides,
               box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Tensor maps of the four stages for B tiles of `bn` rows.
bool build_stage_maps(StageMaps &h, const FieldSolver &f, const __nv_bfloat16 *d_hi, const __nv_bfloat16 *d_lo,
                      int bn) {
    const int m = f.m;
    bool ok = true;
    // S1: T = C . d^T          S2: a = C . T^T (spectral epilogue)
    ok &= make_map(&h.s1.a_hi[0], f.C_hi, m, BM) && make_map(&h.s1.a_lo[0], f.C_lo, m, BM);
    ok &= make_map(&h.s1.b_hi[0], d_hi, m, bn) && make_map(&h.s1.b_lo[0], d_lo, m, bn);
    ok &= make_map(&h.s2.a_hi[0], f.C_hi, m, BM) && make_map(&h.s2.a_lo[0], f.C_lo, m, BM);
    ok &= make_map(&h.s2.b_hi[0], f.b_t_hi, m, bn) && make_map(&h.s2.b_lo[0], f.b_t_lo, m, bn);
    // S3: Ux = Ct . Px^T, Uy = St . Py^T      S4: Ex = St . Ux^T, Ey = Ct . Uy^T
    ok &= make_map(&h.s3.a_hi[0], f.Ct_hi, m, BM) && make_map(&h.s3.a_lo[0], f.Ct_lo, m, BM);
    ok &= make_map(&h.s3.b_hi[0], f.b_px_hi, m, bn) && make_map(&h.s3.b_lo[0], f.b_px_lo, m, bn);
    ok &= make_map(&h.s3.a_hi[1], f.St_hi, m, BM) && make_map(&h.s3.a_lo[1], f.St_lo, m, BM);
    ok &= make_map(&h.s3.b_hi[1], f.b_py_hi, m, bn) && make_map(&h.s3.b_lo[1], f.b_py_lo, m, bn);
    ok &= make_map(&h.s4.a_hi[0], f.St_hi, m, BM) && make_map(&h.s4.a_lo[0], f.St_lo, m, BM);
    ok &= make_map(&h.s4.b_hi[0], f.b_ux_hi, m, bn) && make_map(&h.s4.b_lo[0], f.b_ux_lo, m, bn);
    ok &= make_map(&h.s4.a_hi[1], f.Ct_hi, m, BM) && make_map(&h.s4.a_lo[1], f.Ct_lo, m, BM);
    ok &= make_map(&h.s4.b_hi[1], f.b_uy_hi, m, bn) && make_map(&h.s4.b_lo[1], f.b_uy_lo, m, bn);
    __nv_bfloat16 *outs[10] = {f.b_t_hi, f.b_t_lo, f.b_px_hi, f.b_px_lo, f.b_py_hi,
                               f.b_py_lo, f.b_ux_hi, f.b_ux_lo, f.b_uy_hi, f.b_uy_lo};
    for (int i = 0; i < 10; ++i) ok &= make_out_map(&h.out[i], outs[i], false, m);
    // the batch-1 slots of S1/S2 repeat batch 0 (never read: those launches have gridDim.z == 1)
    h.s1.a_hi[1] = h.s1.a_hi[0]; h.s1.a_lo[1] = h.s1.a_lo[0]; h.s1.b_hi[1] = h.s1.b_hi[0]; h.s1.b_lo[1] = h.s1.b_lo[0];
    h.s2.a_hi[1] = h.s2.a_hi[0]; h.s2.a_lo[1] = h.s2.a_lo[0]; h.s2.b_hi[1] = h.s2.b_hi[0]; h.s2.b_lo[1] = h.s2.b_lo[0];
    return ok;
}

struct TcState {
    StageMaps maps[2];  // [0] 128 x 64 tiles, [1] 128 x 128 tiles
};

// CTAs per cluster splitting K: doubled (up to 4) while the k-blocks divide
// and the launch still fits one wave of `per_sm` CTAs per SM -- small grids
// (few output tiles) then use more SMs
int pick_split(int tiles, int nk, int per_sm) {
    static int sms = 0;
    if (sms <= 0) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
            sms = 148;
    }
    int s = 1;
    while (s < 4 && nk % (2 * s) == 0 && tiles * 2 * s <= sms * per_sm) s *= 2;
    return s;
}

template <class T>
void launch_stage(const Maps &maps, Epi e, int m, int batch, int per_sm, cudaStream_t st) {
    const int tiles = (m / T::BN) * (m / BM) * batch;
    e.split = pick_split(tiles, m / BK, per_sm);
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((m / T::BN) * e.split, m / BM, batch);
    cfg.blockDim = dim3(THREADS);
    cfg.dynamicSmemBytes = T::SMEM_BYTES;
    cfg.stream = st;
    cudaLaunchAttribute at[2];
    unsigned int na = 0;
    if (e.split > 1) {
        at[na].id = cudaLaunchAttributeClusterDimension;
        at[na].val.clusterDim.x = e.split;
        at[na].val.clusterDim.y = 1;
        at[na].val.clusterDim.z = 1;
        ++na;
    }
    if (e.pdl) {
        at[na].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[na].val.programmaticStreamSerializationAllowed = 1;
        ++na;
    }
    cfg.attrs = at;
    cfg.numAttrs = na;
    cudaLaunchKernelEx(&cfg, gemm_bf16x3_kernel<T>, maps, e);
}

template <class T>
void run_stages(const StageMaps &h, FieldSolver &f, float *ex, float *ey, cudaStream_t st, const int *gate,
                int gate_mask) {
    const int m = f.m;
    const int per_sm = T::SMEM_BYTES * 2 <= 227 * 1024 ? 2 : 1;
    Epi e{};
    e.gate = gate;
    e.gate_mask = gate_mask;
    e.m = m;
    e.status = f.tc_status;
    e.skip_loads = f.fault_stall;
    e.wait_ns = f.fault_stall ? f.fault_wait_ns : WAIT_NS;
    e.wx = f.wx;
    e.wy = f.wy;
    e.scale = 4.0f / ((float)m * (float)m);
    e.mode = EPI_SPLIT;
    e.o_hi[0] = f.b_t_hi;
    e.o_lo[0] = f.b_t_lo;
    launch_stage<T>(h.s1, e, m, 1, per_sm, st);
    e.pdl = 1;  // stages 2-4 overlap their set-up with the previous stage's end
    e.mode = EPI_SPECTRAL;
    e.o_hi[0] = f.b_px_hi;
    e.o_lo[0] = f.b_px_lo;
    e.o_hi[1] = f.b_py_hi;
    e.o_lo[1] = f.b_py_lo;
    launch_stage<T>(h.s2, e, m, 1, per_sm, st);
    e.mode = EPI_SPLIT;
    e.o_hi[0] = f.b_ux_hi;
    e.o_lo[0] = f.b_ux_lo;
    e.o_hi[1] = f.b_uy_hi;
    e.o_lo[1] = f.b_uy_lo;
    launch_stage<T>(h.s3, e, m, 2, per_sm, st);
    e.mode = EPI_F32;
    e.o_f32[0] = ex;
    e.o_f32[1] = ey;
    launch_stage<T>(h.s4, e, m, 2, per_sm, st);
}

// Resident CTAs of the persistent solve on the whole GPU (0: cannot run).
template <class T>
int persist_capacity() {
    static int cap = -1;
    if (cap < 0) {
        int dev = 0, sms = 0, per_sm = 0;
        cap = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
            cudaFuncSetAttribute(persist_solve_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 PCfg<T>::SMEM_BYTES) == cudaSuccess &&
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, persist_solve_kernel<T>, P_THREADS,
                                                          PCfg<T>::SMEM_BYTES) == cudaSuccess)
            cap = sms * per_sm;
    }
    return cap;
}

// false (nothing launched) if the field outputs cannot take tile stores
template <class T>
bool run_persistent(const StageMaps &h, FieldSolver &f, int ks, float *ex, float *ey, cudaStream_t st,
                    const int *gate, int gate_mask) {
    const int m = f.m, one = (m / BM) * (m / T::BN), total = 2 * ks * one + 4 * one;
    const int grid = std::min(total, persist_capacity<T>());
    PMaps pm;
    pm.st[0] = h.s1;
    pm.st[1] = h.s2;
    pm.st[2] = h.s3;
    pm.st[3] = h.s4;
    for (int i = 0; i < OUT_EX; ++i) pm.out[i] = h.out[i];
    // the field outputs are the caller's buffers: their maps are made per call
    if (!make_out_map(&pm.out[OUT_EX], ex, true, m) || !make_out_map(&pm.out[OUT_EX + 1], ey, true, m)) return false;
    PEpi e{};
    e.m = m;
    e.ks = ks;
    e.part = f.tc_part;
    e.wx = f.wx;
    e.wy = f.wy;
    e.scale = 4.0f / ((float)m * (float)m);
    e.status = f.tc_status;
    e.sync = f.tc_sync;
    e.gate = gate;
    e.gate_mask = gate_mask;
    e.skip_loads = f.fault_stall;
    e.wait_ns = f.fault_stall ? f.fault_wait_ns : WAIT_NS;
    persist_solve_kernel<T><<<grid, P_THREADS, PCfg<T>::SMEM_BYTES, st>>>(pm, e);
    return true;
}

void run_variant(int v, FieldSolver &f, float *ex, float *ey, cudaStream_t st, const int *gate = nullptr,
                 int gate_mask = 0) {
    const TcState &s = *reinterpret_cast<const TcState *>(f.tc_maps);
    if (v >= 3 && run_persistent<Tile128>(s.maps[1], f, v == 3 ? 2 : 1, ex, ey, st, gate, gate_mask)) return;
    if (v == 1 || v >= 3)
        run_stages<Tile128>(s.maps[1], f, ex, ey, st, gate, gate_mask);
    else if (v == 2)
        run_stages<Tile64x2>(s.maps[0], f, ex, ey, st, gate, gate_mask);
    else
        run_stages<Tile64>(s.maps[0], f, ex, ey, st, gate, gate_mask);
}

}  // namespace tc

// Builds the tensor maps of both tile shapes, then times one full solve of
// each variant (128 x 64 tiles with 4 pipeline stages, 128 x 128 with 3,
// 128 x 64 with 2 so that two CTAs share an SM; 3 warm, 5 timed, CUDA
// events) and keeps the fastest: the tile autotuner of the tensor-core path.
// The scratch outputs are overwritten.
int field_solver_bind_bf16(FieldSolver &f, const __nv_bfloat16 *d_hi, const __nv_bfloat16 *d_lo) {
    using namespace tc;
    if (f.m < BM || (f.m % BM) != 0 || !f.C_hi) return AP_ERR_UNSUPPORTED;
    TcState s{};
    if (!build_stage_maps(s.maps[0], f, d_hi, d_lo, Tile64::BN) ||
        !build_stage_maps(s.maps[1], f, d_hi, d_lo, Tile128::BN))
        return AP_ERR_UNSUPPORTED;
    if (!f.tc_maps && !(f.tc_maps = malloc(sizeof(TcState)))) return AP_ERR_CUDA;
    *reinterpret_cast<TcState *>(f.tc_maps) = s;
    if (!f.tc_status && cudaMalloc(&f.tc_status, sizeof(unsigned int)) != cudaSuccess) return AP_ERR_CUDA;
    if (cudaMemset(f.tc_status, 0, sizeof(unsigned int)) != cudaSuccess) return AP_ERR_CUDA;
    // the persistent solve's counters (queue head, CTAs finished, 4 stages x 2
    // products x row blocks, 2 stages x tiles x 4 warps of halves) and its
    // split-K partials (2 stages x 2 halves x tiles of 128 x 128 FP32)
    const size_t nm = (size_t)(f.m / BM), tiles = nm * nm;
    const size_t sync_bytes = sizeof(unsigned int) * (2 + 8 * nm + 8 * tiles);
    if (!f.tc_sync && cudaMalloc(&f.tc_sync, sync_bytes) != cudaSuccess) return AP_ERR_CUDA;
    if (cudaMemset(f.tc_sync, 0, sync_bytes) != cudaSuccess) return AP_ERR_CUDA;
    if (!f.tc_part && cudaMalloc(&f.tc_part, sizeof(float) * 4 * tiles * BM * BM) != cudaSuccess) return AP_ERR_CUDA;
    if (cudaFuncSetAttribute(gemm_bf16x3_kernel<Tile64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             Tile64::SMEM_BYTES) != cudaSuccess ||
        cudaFuncSetAttribute(gemm_bf16x3_kernel<Tile128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             Tile128::SMEM_BYTES) != cudaSuccess ||
        cudaFuncSetAttribute(gemm_bf16x3_kernel<Tile64x2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             Tile64x2::SMEM_BYTES) != cudaSuccess)
        return AP_ERR_CUDA;
    // the input map holds whatever the caller's buffer holds; timing does not depend on values
    if (cudaMemset((void *)d_hi, 0, sizeof(__nv_bfloat16) * (size_t)f.m * f.m) != cudaSuccess ||
        cudaMemset((void *)d_lo, 0, sizeof(__nv_bfloat16) * (size_t)f.m * f.m) != cudaSuccess)
        return AP_ERR_CUDA;
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return AP_ERR_CUDA;
    // two passes over the candidates, each keeping its faster pass: the
    // first candidate timed on a cold GPU (clocks, caches) would otherwise
    // look slower than it is
    for (int v = 0; v < kTcVariants; ++v) f.tc_tune_ms[v] = -1.f;  // not run
    for (int pass = 0; pass < 2; ++pass) {
        for (int v = 0; v < kTcVariants; ++v) {
            if (v >= 3 && persist_capacity<Tile128>() <= 0) continue;
            for (int w = 0; w < 3; ++w) run_variant(v, f, f.ux, f.uy, 0);
            cudaEventRecord(e0, 0);
            for (int t = 0; t < 5; ++t) run_variant(v, f, f.ux, f.uy, 0);
            cudaEventRecord(e1, 0);
            if (cudaEventSynchronize(e1) != cudaSuccess) {
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                return AP_ERR_CUDA;
            }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            ms /= 5;
            if (f.tc_tune_ms[v] < 0.f || ms < f.tc_tune_ms[v]) f.tc_tune_ms[v] = ms;
        }
    }
    f.tc_variant = 0;
    for (int v = 1; v < kTcVariants; ++v)
        if (f.tc_tune_ms[v] >= 0.f && f.tc_tune_ms[v] < f.tc_tune_ms[f.tc_variant]) f.tc_variant = v;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    // AP_TC_VARIANT=0..4 pins a candidate that ran (tests of each variant)
    if (const char *pin = getenv("AP_TC_VARIANT")) {
        const int v = atoi(pin);
        if (v >= 0 && v < kTcVariants && f.tc_tune_ms[v] >= 0.f) f.tc_variant = v;
    }
    unsigned int st = 0;
    if (cudaMemcpy(&st, f.tc_status, sizeof(st), cudaMemcpyDeviceToHost) != cudaSuccess) return AP_ERR_CUDA;
    if (st) return AP_ERR_TIMEOUT;
    f.tc_ready = 1;
    return AP_OK;
}

int field_solve_bf16x3(FieldSolver &f, const __nv_bfloat16 *d_hi, const __nv_bfloat16 *d_lo, float *ex,
                       float *ey, cudaStream_t st, const int *gate, int gate_mask) {
    (void)d_hi;
    (void)d_lo;  // bound into the stage-1 tensor maps by field_solver_bind_bf16
    if (!f.tc_ready) return AP_ERR_UNSUPPORTED;
    tc::run_variant(f.tc_variant, f, ex, ey, st, gate, gate_mask);
    return cudaGetLastError() == cudaSuccess ? AP_OK : AP_ERR_CUDA;
}

int field_solver_clear_status(FieldSolver &f) {
    if (!f.tc_status) return AP_OK;
    return cudaMemset(f.tc_status, 0, sizeof(unsigned int)) == cudaSuccess ? AP_OK : AP_ERR_CUDA;
}

}  // namespace ap
