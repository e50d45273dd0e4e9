// Electrostatic field solve as dense per-axis transform contractions, FP32 SIMT.
//
// Restates replace::FFT::doFFT (python/AIEmath/fft_replace/fft.cpp:204-299)
// and Placer::compute_a_uv_DCT / compute_eField_DCT (vck5000/host/src/
// AIEplace.cpp:752-934): 2-D DCT-II of the density, halved edge rows,
// 4/(Mx My), phi = a/(wx^2+wy^2), Ex = S^T (phi wx) C, Ey = C^T (phi wy) S.
// Every stage is one TN contraction  D[i][j] = sum_k A[i][k] B[j][k]  with A a
// constant transform matrix and B the data, both K-contiguous:
//   S1  T[v][x]  = sum_y C[v][y]  d[x][y]
//   S2  a[u][v]  = sum_x C[u][x]  T[v][x]      epilogue -> Px, Py
//   S3  Ux[y][u] = sum_v Ct[y][v] Px[u][v]     Uy[y][u] = sum_v St[y][v] Py[u][v]
//   S4  Ex[x][y] = sum_u St[x][u] Ux[y][u]     Ey[x][y] = sum_u Ct[x][u] Uy[y][u]
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include <vector>

#include "../../include/aieplace.h"
#include "ap_kernels.h"

namespace ap {

namespace {

constexpr int BK = 16;

struct GemmSet {
    const float *A[2];
    const float *B[2];
    float *C[2];
    const int *gate;  // run only if gate is null or (1 << *gate) & gate_mask
    int gate_mask;
};

struct SpectralEpi {
    float *px, *py;
    const float *wx, *wy;
    float scale;  // 4 / m^2
};

__device__ __forceinline__ void spectral_store(const SpectralEpi &e, int m, int u, int v, float acc) {
    float px = 0.f, py = 0.f;
    if (u != 0 || v != 0) {
        const float wx = e.wx[u], wy = e.wy[v];
        float c = acc * e.scale;
        if (u == 0) c *= 0.5f;
        if (v == 0) c *= 0.5f;
        c = c / (wx * wx + wy * wy);
        px = c * wx;
        py = c * wy;
    }
    e.px[(size_t)u * m + v] = px;
    e.py[(size_t)u * m + v] = py;
}

// One BM x BM output tile (rows i0.., columns j0..) of D = A B^T on an m x m
// problem, 256 threads.  FRESH_B: B was written by other blocks of the same
// launch (a persistent launch's earlier stage), so it is read through L2
// (ld.global.cg) rather than the non-coherent read-only path.
template <int BM, bool SPECTRAL, bool FRESH_B>
__device__ __forceinline__ void gemm_tile(int m, const GemmSet &s, int z, const SpectralEpi &e, int i0, int j0) {
    constexpr int TM = BM / 16;
    const float *__restrict__ A = s.A[z];
    const float *__restrict__ B = s.B[z];
    __shared__ __align__(16) float As[BK][BM + 4];
    __shared__ __align__(16) float Bs[BK][BM + 4];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    float acc[TM][TM];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TM; ++j) acc[i][j] = 0.f;
    for (int k0 = 0; k0 < m; k0 += BK) {
        for (int q = tid; q < BM * BK / 4; q += 256) {
            const int row = q >> 2, kq = (q & 3) * 4;
            const float4 va = *reinterpret_cast<const float4 *>(A + (size_t)(i0 + row) * m + k0 + kq);
            const float4 *pb = reinterpret_cast<const float4 *>(B + (size_t)(j0 + row) * m + k0 + kq);
            const float4 vb = FRESH_B ? __ldcg(pb) : *pb;
            As[kq + 0][row] = va.x;
            As[kq + 1][row] = va.y;
            As[kq + 2][row] = va.z;
            As[kq + 3][row] = va.w;
            Bs[kq + 0][row] = vb.x;
            Bs[kq + 1][row] = vb.y;
            Bs[kq + 2][row] = vb.z;
            Bs[kq + 3][row] = vb.w;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            float a[TM], b[TM];
#pragma unroll
            for (int i = 0; i < TM; ++i) a[i] = As[kk][ty * TM + i];
#pragma unroll
            for (int j = 0; j < TM; ++j) b[j] = Bs[kk][tx * TM + j];
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TM; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < TM; ++i) {
        const int gi = i0 + ty * TM + i;
#pragma unroll
        for (int j = 0; j < TM; ++j) {
            const int gj = j0 + tx * TM + j;
            if (SPECTRAL)
                spectral_store(e, m, gi, gj, acc[i][j]);
            else
                s.C[z][(size_t)gi * m + gj] = acc[i][j];
        }
    }
}

// D = A B^T on an m x m problem; one BM x BM output tile per block.
template <int BM, bool SPECTRAL>
__global__ void __launch_bounds__(256) gemm_tn_simt(int m, GemmSet s, SpectralEpi e) {
    if (s.gate && !((1 << *s.gate) & s.gate_mask)) return;
    const int z = blockIdx.z;
    gemm_tile<BM, SPECTRAL, false>(m, s, z, e, blockIdx.y * BM, blockIdx.x * BM);
}

// bm: output tile side chosen by the autotuner in field_solver_init (0 = size rule)
template <bool SPECTRAL>
void gemm(int m, const GemmSet &s, int batch, const SpectralEpi &e, cudaStream_t st, int bm = 0) {
    if (bm == 0) bm = m >= 512 ? 64 : 32;
    if (bm == 64 && m % 64 == 0) {
        dim3 grid(m / 64, m / 64, batch);
        gemm_tn_simt<64, SPECTRAL><<<grid, 256, 0, st>>>(m, s, e);
    } else {
        dim3 grid(m / 32, m / 32, batch);
        gemm_tn_simt<32, SPECTRAL><<<grid, 256, 0, st>>>(m, s, e);
    }
}

__global__ void split_kernel(int n, const float *src, __nv_bfloat16 *hi, __nv_bfloat16 *lo) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float v = src[i];
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        hi[i] = h;
        lo[i] = __float2bfloat16_rn(v - __bfloat162float(h));
    }
}

template <typename T>
int dmalloc(T **p, size_t n) {
    return cudaMalloc((void **)p, sizeof(T) * (n ? n : 1)) == cudaSuccess ? 0 : -1;
}

}  // namespace

void launch_split_bf16(int n, const float *src, __nv_bfloat16 *hi, __nv_bfloat16 *lo, cudaStream_t st) {
    int blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    split_kernel<<<blocks, 256, 0, st>>>(n, src, hi, lo);
}

static int tune_simt(FieldSolver &f);

int field_solver_init(FieldSolver &f, int m, float bin_ratio, int want_bf16) {
    f = FieldSolver();
    if (m < 32 || (m % 32) != 0) return AP_ERR_UNSUPPORTED;
    f.m = m;
    f.bin_ratio = bin_ratio;
    const size_t nn = (size_t)m * m;
    std::vector<float> C(nn), Ct(nn), St(nn), wx(m), wy(m);
    const double pi = 3.14159265358979323846;
    for (int k = 0; k < m; ++k)
        for (int i = 0; i < m; ++i) {
            const double t = pi * k * (i + 0.5) / m;
            C[(size_t)k * m + i] = (float)cos(t);
            Ct[(size_t)i * m + k] = (float)cos(t);
            St[(size_t)i * m + k] = (float)sin(t);
        }
    for (int u = 0; u < m; ++u) {
        wx[u] = (float)(pi * u / m);
        wy[u] = (float)(pi * u / m * bin_ratio);
    }
    int e = 0;
    e |= dmalloc(&f.C, nn) | dmalloc(&f.Ct, nn) | dmalloc(&f.St, nn) | dmalloc(&f.wx, m) |
         dmalloc(&f.wy, m);
    e |= dmalloc(&f.t0, nn) | dmalloc(&f.px, nn) | dmalloc(&f.py, nn) | dmalloc(&f.ux, nn) |
         dmalloc(&f.uy, nn);
    if (e) return AP_ERR_CUDA;
    cudaMemcpy(f.C, C.data(), nn * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(f.Ct, Ct.data(), nn * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(f.St, St.data(), nn * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(f.wx, wx.data(), m * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(f.wy, wy.data(), m * 4, cudaMemcpyHostToDevice);
    if (want_bf16) {
        e |= dmalloc(&f.C_hi, nn) | dmalloc(&f.C_lo, nn) | dmalloc(&f.Ct_hi, nn) | dmalloc(&f.Ct_lo, nn) |
             dmalloc(&f.St_hi, nn) | dmalloc(&f.St_lo, nn);
        e |= dmalloc(&f.b_t_hi, nn) | dmalloc(&f.b_t_lo, nn) | dmalloc(&f.b_px_hi, nn) |
             dmalloc(&f.b_px_lo, nn) | dmalloc(&f.b_py_hi, nn) | dmalloc(&f.b_py_lo, nn) |
             dmalloc(&f.b_ux_hi, nn) | dmalloc(&f.b_ux_lo, nn) | dmalloc(&f.b_uy_hi, nn) |
             dmalloc(&f.b_uy_lo, nn);
        if (e) return AP_ERR_CUDA;
        launch_split_bf16((int)nn, f.C, f.C_hi, f.C_lo, 0);
        launch_split_bf16((int)nn, f.Ct, f.Ct_hi, f.Ct_lo, 0);
        launch_split_bf16((int)nn, f.St, f.St_hi, f.St_lo, 0);
    }
    if (cudaDeviceSynchronize() != cudaSuccess) return AP_ERR_CUDA;
    return tune_simt(f);
}

void field_solver_free(FieldSolver &f) {
    void *ptrs[] = {f.C,       f.Ct,      f.St,      f.C_hi,    f.C_lo,    f.Ct_hi,   f.Ct_lo,
                    f.St_hi,   f.St_lo,   f.wx,      f.wy,      f.t0,      f.px,      f.py,
                    f.ux,      f.uy,      f.b_t_hi,  f.b_t_lo,  f.b_px_hi, f.b_px_lo, f.b_py_hi,
                    f.b_py_lo, f.b_ux_hi, f.b_ux_lo, f.b_uy_hi, f.b_uy_lo, f.tc_status, f.tc_sync, f.tc_part};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    free(f.tc_maps);  // host-side tensor-map table
    f = FieldSolver();
}

void field_solve_fp32(FieldSolver &f, const float *d, float *ex, float *ey, cudaStream_t st, const int *gate,
                      int gate_mask) {
    const int m = f.m;
    SpectralEpi none{};
    GemmSet s1{{f.C, nullptr}, {d, nullptr}, {f.t0, nullptr}, gate, gate_mask};
    gemm<false>(m, s1, 1, none, st, f.simt_bm);
    SpectralEpi epi{f.px, f.py, f.wx, f.wy, 4.0f / ((float)m * (float)m)};
    GemmSet s2{{f.C, nullptr}, {f.t0, nullptr}, {nullptr, nullptr}, gate, gate_mask};
    gemm<true>(m, s2, 1, epi, st, f.simt_bm);
    GemmSet s3{{f.Ct, f.St}, {f.px, f.py}, {f.ux, f.uy}, gate, gate_mask};
    gemm<false>(m, s3, 2, none, st, f.simt_bm);
    GemmSet s4{{f.St, f.Ct}, {f.ux, f.uy}, {ex, ey}, gate, gate_mask};
    gemm<false>(m, s4, 2, none, st, f.simt_bm);
}

void field_records(const FieldSolver &f, const float *d, float *ex, float *ey, FieldRec rec[4]) {
    const int m = f.m;
    const int bm = (f.simt_bm == 64 && m % 64 == 0) ? 64 : (f.simt_bm == 0 && m >= 512 && m % 64 == 0 ? 64 : 32);
    const float scale = 4.0f / ((float)m * (float)m);
    for (int k = 0; k < 4; ++k) {
        rec[k] = FieldRec{};
        rec[k].m = m;
        rec[k].bm = bm;
        rec[k].batch = k < 2 ? 1 : 2;
    }
    rec[0].A[0] = f.C;
    rec[0].B[0] = d;
    rec[0].C[0] = f.t0;
    rec[1].A[0] = f.C;
    rec[1].B[0] = f.t0;
    rec[1].spectral = 1;
    rec[1].px = f.px;
    rec[1].py = f.py;
    rec[1].wx = f.wx;
    rec[1].wy = f.wy;
    rec[1].scale = scale;
    rec[2].A[0] = f.Ct;
    rec[2].A[1] = f.St;
    rec[2].B[0] = f.px;
    rec[2].B[1] = f.py;
    rec[2].C[0] = f.ux;
    rec[2].C[1] = f.uy;
    rec[3].A[0] = f.St;
    rec[3].A[1] = f.Ct;
    rec[3].B[0] = f.ux;
    rec[3].B[1] = f.uy;
    rec[3].C[0] = ex;
    rec[3].C[1] = ey;
}

// The batched form: the four contractions of every instance in one launch,
// record k + 1 of an instance waiting for its record k (the queue's
// dependencies); tiles as gemm_tn_simt, B read through L2.
__global__ void __launch_bounds__(256) persist_field_kernel(PersistQueue q, const FieldRec *recs) {
    persist_loop(q, recs, [](const FieldRec &r, VBlock vb, int) {
        const int nt = r.m / r.bm, tiles = nt * nt;
        const int z = vb.id / tiles, t = vb.id - z * tiles;
        const int i0 = (t / nt) * r.bm, j0 = (t % nt) * r.bm;
        const GemmSet s{{r.A[0], r.A[1]}, {r.B[0], r.B[1]}, {r.C[0], r.C[1]}, nullptr, 0};
        const SpectralEpi e{r.px, r.py, r.wx, r.wy, r.scale};
        if (r.bm == 64) {
            if (r.spectral)
                gemm_tile<64, true, true>(r.m, s, z, e, i0, j0);
            else
                gemm_tile<64, false, true>(r.m, s, z, e, i0, j0);
        } else {
            if (r.spectral)
                gemm_tile<32, true, true>(r.m, s, z, e, i0, j0);
            else
                gemm_tile<32, false, true>(r.m, s, z, e, i0, j0);
        }
    });
}

int persist_field_wave() {
    static int wave = 0;
    if (!wave) wave = wave_of((const void *)persist_field_kernel, 256, 608);
    return wave;
}

void launch_persist_field(const PersistQueue &q, const FieldRec *recs, cudaStream_t st) {
    persist_field_kernel<<<persist_field_wave(), 256, 0, st>>>(q, recs);
}

// Tile autotuner of the FP32 path: times a full solve with 32 and with 64
// tiles (2 warm, 4 timed) on the solver's own scratch and keeps the faster.
static int tune_simt(FieldSolver &f) {
    if (f.m % 64 != 0) {
        f.simt_bm = 32;
        return AP_OK;
    }
    const size_t nn = (size_t)f.m * f.m;
    float *din = nullptr, *eo = nullptr;
    if (dmalloc(&din, 3 * nn)) return AP_ERR_CUDA;
    eo = din + nn;
    cudaEvent_t e0, e1;
    int r = AP_OK;
    if (cudaMemset(din, 0, sizeof(float) * nn) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess) {
        cudaFree(din);
        return AP_ERR_CUDA;
    }
    const int cand[2] = {32, 64};
    for (int v = 0; v < 2 && r == AP_OK; ++v) {
        f.simt_bm = cand[v];
        for (int w = 0; w < 2; ++w) field_solve_fp32(f, din, eo, eo + nn, 0);
        cudaEventRecord(e0, 0);
        for (int t = 0; t < 4; ++t) field_solve_fp32(f, din, eo, eo + nn, 0);
        cudaEventRecord(e1, 0);
        if (cudaEventSynchronize(e1) != cudaSuccess) r = AP_ERR_CUDA;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        f.simt_tune_ms[v] = ms / 4;
    }
    f.simt_bm = f.simt_tune_ms[0] <= f.simt_tune_ms[1] ? 32 : 64;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(din);
    return r;
}

// ---- field solve without allocation -------------------------------------------
// Some callers cannot allocate device memory at all: code that runs inside a
// host framework which owns every device allocation and hands out only the
// buffers it manages, or code on a path where a cudaMalloc would synchronise
// the device or fail under a fixed memory budget.  For them the FP32 solve
// also runs from one fixed scratch array in the library's static device
// memory.  The array holds the transform tables and the intermediate maps of
// one grid of up to kNoAllocMaxBins x kNoAllocMaxBins bins (8 m^2 + 2 m
// floats, 2.1 MB at the maximum); every GPU that loads the library keeps it
// until the process exits.

namespace {

constexpr int kNoAllocMaxBins = 256;
constexpr size_t kNoAllocFloats = 8ull * kNoAllocMaxBins * kNoAllocMaxBins + 2ull * kNoAllocMaxBins;
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) float g_field_scratch[kNoAllocFloats];

// Per device: which context's copy of g_field_scratch holds the tables of
// which grid.  A context that is destroyed and recreated (cudaDeviceReset)
// gets a fresh, zeroed copy of the array, so the key includes the context's
// unique id; without a way to read that id the tables are refilled on every
// call.
struct NoAllocState {
    unsigned long long ctx_id;  // 0: nothing cached
    float *base;
    int m;
    float ratio;
};
static NoAllocState g_noalloc_state[kNoAllocMaxDevices];

typedef int (*PfnCtxGetCurrent)(void **ctx);
typedef int (*PfnCtxGetId)(void *ctx, unsigned long long *id);

// Unique id of the calling thread's current context (driver entry points
// looked up through the runtime, so the library needs no libcuda link), or
// 0 if it cannot be read.
unsigned long long current_context_id() {
    static PfnCtxGetCurrent get_cur = nullptr;
    static PfnCtxGetId get_id = nullptr;
    static bool looked_up = false;
    if (!looked_up) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_cur = (PfnCtxGetCurrent)p;
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = (PfnCtxGetId)p;
        looked_up = true;
    }
    if (!get_cur || !get_id) return 0ull;
    void *ctx = nullptr;
    unsigned long long id = 0ull;
    if (get_cur(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0ull;
    return id;
}

__global__ void noalloc_tables_kernel(float *C, float *Ct, float *St, float *wx, float *wy, int m, float ratio) {
    const double pi = 3.14159265358979323846;
    const int n = m * m;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
        const int k = idx / m, i = idx % m;
        double s, c;
        sincospi((double)k * (i + 0.5) / m, &s, &c);
        C[(size_t)k * m + i] = (float)c;
        Ct[(size_t)i * m + k] = (float)c;
        St[(size_t)i * m + k] = (float)s;
        if (idx < m) {
            wx[idx] = (float)(pi * idx / m);
            wy[idx] = (float)(pi * idx / m * ratio);
        }
    }
}

}  // namespace

}  // namespace ap

// Same result as ap_field_solve with the FP32 solver, on caller-owned device
// buffers and without allocating.  Every call looks the scratch address up
// with cudaGetSymbolAddress (host code may not use the symbol as an address);
// the first call on a device, the first after the bin count or bin_ratio
// changes and the first in a new context fill the transform tables, so make
// that first call before any stream capture.  All calls share the one
// scratch array: calls whose GPU work overlaps (other streams, other threads)
// race on it.  The density is read in 16-byte vectors, so it must start on a
// 16-byte boundary; ex and ey must be float-aligned.
extern "C" int ap_field_solve_noalloc(const float *density, float *ex, float *ey, int32_t bins, float bin_ratio,
                                      void *stream) {
    using namespace ap;
    if (!density || !ex || !ey) return AP_ERR_INVALID_ARG;
    if (((uintptr_t)density & 15u) != 0 || ((uintptr_t)ex & 3u) != 0 || ((uintptr_t)ey & 3u) != 0)
        return AP_ERR_INVALID_ARG;
    if (bins < 32 || bins > kNoAllocMaxBins || (bins % 32) != 0) return AP_ERR_INVALID_ARG;
    if (!(bin_ratio > 0.f) || !(bin_ratio < 1e30f)) return AP_ERR_INVALID_ARG;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) return AP_ERR_NO_DEVICE;
    cudaStream_t st = (cudaStream_t)stream;
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_field_scratch) != cudaSuccess || !p) return AP_ERR_CUDA;
    const unsigned long long ctx = current_context_id();
    NoAllocState &s = g_noalloc_state[dev];
    const bool fresh = ctx == 0ull || s.ctx_id != ctx || s.base != (float *)p || s.m != bins || s.ratio != bin_ratio;
    const size_t mm = (size_t)bins * bins;
    FieldSolver f{};
    f.m = bins;
    f.bin_ratio = bin_ratio;
    f.C = (float *)p;
    f.Ct = f.C + mm;
    f.St = f.Ct + mm;
    f.t0 = f.St + mm;
    f.px = f.t0 + mm;
    f.py = f.px + mm;
    f.ux = f.py + mm;
    f.uy = f.ux + mm;
    f.wx = f.uy + mm;
    f.wy = f.wx + bins;
    if (fresh) {
        s.ctx_id = 0ull;  // set again only once the fill is enqueued
        noalloc_tables_kernel<<<(int)((mm + 255) / 256), 256, 0, st>>>(f.C, f.Ct, f.St, f.wx, f.wy, bins,
                                                                      bin_ratio);
        if (cudaGetLastError() != cudaSuccess) return AP_ERR_CUDA;
        s.ctx_id = ctx;
        s.base = (float *)p;
        s.m = bins;
        s.ratio = bin_ratio;
    }
    field_solve_fp32(f, density, ex, ey, st);  // writes every scratch element before reading it
    return cudaGetLastError() == cudaSuccess ? AP_OK : AP_ERR_CUDA;
}
