// Kernel argument blocks and launchers of the placement iteration.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "ap_common.cuh"
#include "ap_persist.cuh"

namespace ap {

// ---- wirelength -------------------------------------------------------------
enum { WA_OUT_ONLY = 0, WA_LOOP = 1, WA_INIT = 2 };

// Nets are bucketed by degree: [2], [3,4], [5,8] (one thread per net, pins in
// registers), [9,16] (16 lanes per net), [17,32], [33,64] (a warp, one or two
// pins per lane in registers) and > 64 (a warp looping over the pins); bucket
// b spans nets [bucket_lo[b], bucket_lo[b+1]).
constexpr int kWaBuckets = 7;

struct WaArgs {
    const int *net_ptr;    // [n_nets + 1], nets in bucket order
    const int *pin_node;   // internal node ids (| kPinHeavy: node of more than kPackMaxPins pins)
    int n_small, n_nets;
    int bucket_lo[kWaBuckets + 1];
    int bucket_blocks[kWaBuckets];  // grid of each bucket's launch (filled by the launcher)
    // positions of all nodes, interleaved (one 8-byte load per pin), read by
    // the kernels: in WA_LOOP mode written by the position update (movable
    // nodes) and once at creation (the fixed ones); in the other modes
    // filled by launch_wirelength from (px, py)
    float2 *xy;
    int n_nodes;
    const float *px, *py;  // modes other than WA_LOOP: positions of all nodes
    float gamma;           // > 0 overrides sc->gamma
    DevScalars *sc;
    ull *gq;               // int64 fixed-point gradient accumulators, both axes packed (pack_q)
    ull *gqx, *gqy;        // the same, one per axis, for nodes of more than kPackMaxPins pins
    int n_grad;            // nodes [0, n_grad) receive gradient
    double *partials;      // 2 per block over all bucket launches
    unsigned int *counter;
    int small_blocks;      // blocks of the three thread-per-net launches together
    int block_nets;        // nets (lanes of the larger nets) per block, at least (<= 256: one per thread)
    double *out;           // [2]: HPWL, WA
    int mode;
};
// launches the four bucket kernels (after filling a.xy from a.px, a.py in
// the modes other than WA_LOOP); the last one (warp per net) folds the sums
void launch_wirelength(const WaArgs &a, cudaStream_t st);
// xy[i] = (px[i], py[i]), i < n
void launch_interleave(int n, const float *px, const float *py, float2 *xy, cudaStream_t st);
// Block partials buffer (doubles; the per-block partials are FP32, two per
// double): holds 2 FP32 per block of the four WA launches at kWaMaxBlocks
// each, 4 per gather block at kGatherMaxBlocks, 2 per update block (at most
// 8192 blocks).
constexpr int kPartialDoubles = 4 * 8192 + 64;
// Blocks per bucket launch, grid-stride beyond (at 2M cells: 4096 blocks
// 131 us for the WA stage, 2432 blocks 123 us, 1216 blocks 133 us)
constexpr int kWaMaxBlocks = 2432;

// ---- density scatter (+ Nesterov position update) ---------------------------
struct ScatterArgs {
    Grid g;
    const float *w, *h;
    // the bin adds take nodes [lo, hi): plain mode at (px, py), update mode
    // from the records the position update wrote
    const float *px, *py;
    int lo, hi;
    // update mode: movable nodes [0, n_mov) step from the accepted state
    // (buffers [cur]) to the trial point (buffers [1 - cur]), then scatter
    int update;
    int n_mov;
    float die_w, die_h;
    float *ux[2], *uy[2];
    float *vx[2], *vy[2];
    const float *gx[2], *gy[2];
    DevScalars *sc;
    ull *rho_q;
    double *partials;      // update mode: |u_{k+1} - u_k|^2 per block
    unsigned int *counter;
    // update mode, optional: each movable node's bin record (packed base bin
    // or a sentinel; overlaps ow0, ow1, oh0, oh1) for the gather at the same point
    int *rec_bin;
    int4 *rec_ov;
    // update mode, optional: the trial point also written here (movable
    // nodes), for a copy to the host that overlaps the rest of the trial
    float *trial_x, *trial_y;
    // update mode, optional: the trial point interleaved (movable nodes),
    // for the loop's WA kernels
    float2 *xy_out;
    // update mode, optional: the accepted point read from here instead of
    // buffers [cur] (a host step's input)
    const float *in_x, *in_y;
    // update mode: nodes [upd_lo, upd_hi) when upd_hi > 0 (one chunk of a
    // host step's input); block partials from slot part_base on; no_fold: a
    // later launch folds the sums
    int upd_lo, upd_hi, part_base, no_fold;
    // nodes per block of the position update and the bin adds, at least
    // (<= the block size: one per thread); results depend on it only
    // through the order of the update's FP32 block sums
    int block_nodes;
    // bin adds: the shared tile accumulates each value's bits [0, 16) and
    // [16, 48) in two 32-bit words (set by the launcher where no word can
    // overflow); 0: one 64-bit word
    int tile32;
    // optional: each node's fixed-point width and height (to_q(w), to_q(h);
    // kSizeQNone where they do not fit int32), made once by launch_size_q:
    // the position update reads them instead of converting every iteration
    const int2 *whq;
};
constexpr int kSizeQNone = (int)0x80000000u;
void launch_size_q(int n, const float *w, const float *h, int2 *out, cudaStream_t st);
void launch_scatter(const ScatterArgs &a, cudaStream_t st);
// the two launches of launch_scatter: the position update and records (update
// mode only), then the bin adds
int launch_update(const ScatterArgs &a, cudaStream_t st);  // returns the blocks launched
void launch_scatter_bins(const ScatterArgs &a, cudaStream_t st);

// ---- density map -> solver input + overflow ---------------------------------
enum { RHO_OUT_ONLY = 0, RHO_LOOP = 1, RHO_INIT = 2 };

struct RhoArgs {
    int nbins;
    ull *mov_q;                 // read, then cleared for the next iteration
    ull *fill_q;                // filler cells (null: none): in the solver input, not in the overflow; cleared
    const long long *fix_q;     // fixed nodes at weight 1
    const long long *fixs_q;    // fixed nodes scaled by rho_t
    long long cap_q, ab_q;
    double inv_ab;
    float inv_ab_f;             // (float)(1 / ab_q): density = (float)tot * inv_ab_f - d_shift
    // A constant taken off the solver input: the field ignores the map's mean
    // (the DC coefficient is dropped, phi_00 = 0), and without it the large
    // mean's rounding in the transforms' DC sums swamps the small AC terms
    float d_shift;
    float *d_f32;               // FP32 solver input, or null
    __nv_bfloat16 *d_hi, *d_lo; // BF16x3 solver input, or null
    DevScalars *sc;
    long long *partials;        // 2 * grid
    unsigned int *counter;
    double *out;                // [2]: tau, tau_abs
    int mode;
    // graph switch node selecting the field source of a loop trial (0: none);
    // the last block sets it to the trial's field mode
    unsigned long long field_switch;
};
void launch_rho(const RhoArgs &a, cudaStream_t st);

// ---- field gather + preconditioned gradient + optimiser scalars -------------
enum { GATHER_STEP = 0, GATHER_INIT_NORMS = 1, GATHER_INIT_GRAD = 2, GATHER_INIT_PREV = 3,
       GATHER_FORCE_ONLY = 4, GATHER_NODE_OUT = 5 };

struct GatherArgs {
    Grid g;
    int n_mov;
    int at;                 // evaluation buffer (GATHER_STEP: 1 - sc->cur)
    float *vx[2], *vy[2];   // evaluation point [at], comparison point [1 - at]
    const float *w, *h;
    const float *ex, *ey;   // field per bin
    ull *gq;                // WA gradient accumulators, packed (cleared after reading)
    ull *gqx, *gqy;         // per-axis accumulators of nodes of more than kPackMaxPins pins
    const float *pins;      // pin count per movable node
    const float *charge;    // area / bin area
    float *gx[2], *gy[2];   // preconditioned gradient: output [at], comparison [1 - at]
    float *fx, *fy;         // GATHER_FORCE_ONLY / NODE_OUT output: overlap-weighted field per node
    // GATHER_NODE_OUT (the per-node stage entry point): the preconditioned
    // gradient at the density weight `lambda` into gxo, gyo (if non-null);
    // the bin records of the evaluation point (launch_records) are read as in
    // a loop trial
    float lambda;
    float *gxo, *gyo;
    DevScalars *sc;
    double *partials;       // 4 * grid
    unsigned int *counter;
    int mode;
    // GATHER_STEP / NODE_OUT, optional: the bin records of this point
    const int *rec_bin;
    const int4 *rec_ov;
    int block_nodes;        // nodes per block, at least (<= the block size: one per thread)
};
void launch_gather(const GatherArgs &a, cudaStream_t st);
// bin records (as the position update writes them) of movable nodes at (x, y)
void launch_records(const Grid &g, int n_mov, const float *x, const float *y, const float *w, const float *h,
                    int *rec_bin, int4 *rec_ov, cudaStream_t st);
constexpr int kGatherMaxBlocks = 4096;  // partials capacity; launched as one wave of resident blocks

// v_{-1} = v_0 - s g_0, s = coef * bw / max|g_0| (first Lipschitz estimate)
void launch_perturb(int n_mov, const float *vx, const float *vy, const float *gx, const float *gy,
                    float *ox, float *oy, const double *gmax, float coef_bw, float die_w, float die_h,
                    const float *w, const float *h, cudaStream_t st);

// ---- field solve ------------------------------------------------------------
// Spectral solver state for an m x m grid (square, m a multiple of 32).
constexpr int kTcCandidates = 5;  // tensor-core solve variants the autotuner times

struct FieldSolver {
    int m;
    float bin_ratio;
    // constant transform matrices, row-major m x m:
    //   C[k][i] = cos(pi k (i+1/2)/m), Ct = C^T, St[i][k] = sin(pi k (i+1/2)/m)
    float *C, *Ct, *St;
    __nv_bfloat16 *C_hi, *C_lo, *Ct_hi, *Ct_lo, *St_hi, *St_lo;
    float *wx, *wy;          // spectral frequencies per index
    // scratch (fp32 path)
    float *t0, *px, *py, *ux, *uy;
    // scratch (bf16 path): hi/lo pairs
    __nv_bfloat16 *b_t_hi, *b_t_lo, *b_px_hi, *b_px_lo, *b_py_hi, *b_py_lo, *b_ux_hi, *b_ux_lo,
        *b_uy_hi, *b_uy_lo;
    void *tc_maps;           // tensor maps of the tcgen05 path (host table)
    int tc_ready;
    unsigned int *tc_status; // device error flag of the tcgen05 kernels
    unsigned int *tc_sync;   // row-block counters of the persistent tcgen05 solve
    float *tc_part;          // its split-K partials
    // tile autotuner results
    int tc_variant;          // 0: 128 x 64 tiles, 1: 128 x 128, 2: 128 x 64 with 2 stages (2 CTAs per SM),
                             // 3, 4: one persistent launch of 128 x 128 tiles, K of stages 1-2
                             // split in two (3) or not (4)
    float tc_tune_ms[kTcCandidates];  // measured solve time of each variant (-1: not run)
    int simt_bm;             // FP32 path tile (32 or 64); 0 = size rule
    float simt_tune_ms[2];   // measured solve time with 32 / 64 tiles
    // failure injection (ap_debug_inject): the tcgen05 kernels issue no loads
    // and bound each wait by fault_wait_ns, so their waits run out
    int fault_stall;
    unsigned long long fault_wait_ns;
};

int field_solver_init(FieldSolver &f, int m, float bin_ratio, int want_bf16);
void field_solver_free(FieldSolver &f);
// density d (x-major) -> ex, ey; FP32 SIMT contraction
// gate: the launches run only if gate is null or (1 << *gate) & gate_mask
// (the loop's surrogate schedule lives in device memory)
void field_solve_fp32(FieldSolver &f, const float *d, float *ex, float *ey, cudaStream_t st,
                      const int *gate = nullptr, int gate_mask = 0);
// Builds the TMA tensor maps of the tcgen05 path with (d_hi, d_lo) as the
// density input; needs m a multiple of 128.
int field_solver_bind_bf16(FieldSolver &f, const __nv_bfloat16 *d_hi, const __nv_bfloat16 *d_lo);
// density as bf16 hi/lo split (the bound buffers) -> ex, ey; tcgen05 BF16x3 contraction
int field_solve_bf16x3(FieldSolver &f, const __nv_bfloat16 *d_hi, const __nv_bfloat16 *d_lo,
                       float *ex, float *ey, cudaStream_t st, const int *gate = nullptr, int gate_mask = 0);
// tc_status (nonzero once a bounded wait in a tcgen05 kernel gave up) back to zero
int field_solver_clear_status(FieldSolver &f);
// float -> bf16 hi/lo split (for per-stage API calls)
void launch_split_bf16(int n, const float *src, __nv_bfloat16 *hi, __nv_bfloat16 *lo, cudaStream_t st);

// ---- batched form: persistent launches (ap_persist.cuh) ----------------------
// the persistent launches of one trial step; PS_WA is the WA launch of the
// nets of more than 8 pins (it folds the sums), PS_WA2/4/8 those of the
// thread-per-net buckets (2, 3-4 and 5-8 pins)
enum { PS_UPDATE = 0, PS_SCATTER = 1, PS_RHO = 2, PS_WA = 3, PS_FIELD = 4, PS_GATHER = 5,
       PS_WA2 = 6, PS_WA4 = 7, PS_WA8 = 8, PS_COUNT = 9 };

// resident blocks of `kernel` on the whole GPU (dyn_smem bytes of dynamic
// shared memory per block), or `fallback`
int wave_of(const void *kernel, int threads, int fallback, int dyn_smem = 0);
// the grids the launchers give an instance's own launches (a persistent
// record of the same instance runs the same blocks)
int update_grid(const ScatterArgs &a);
int scatter_grid(int n, int block_nodes);
// whether the bin adds of n nodes over `blocks` blocks may use 32-bit tile slots
bool tile32_exact(const Grid &g, int n, int blocks);
int rho_grid(int nbins);
int gather_grid(int n_mov, int block_nodes);
// fills bucket_blocks and small_blocks as launch_wirelength does; returns
// the blocks of all four bucket launches
int wa_plan(WaArgs &a);

// One contraction stage of an FP32 field solve (S1..S4 of k_field_simt.cu):
// D[z] = A[z] B[z]^T on an m x m grid in bm x bm tiles, `batch` values of z,
// the spectral epilogue (phi -> px, py) when `spectral`.
struct FieldRec {
    const float *A[2];
    const float *B[2];
    float *C[2];
    float *px, *py;
    const float *wx, *wy;
    float scale;
    int m, bm, spectral, batch;
};
// the four stages of field_solve_fp32(f, d, ex, ey) with the solver's tuned tile
void field_records(const FieldSolver &f, const float *d, float *ex, float *ey, FieldRec rec[4]);
inline int field_rec_blocks(const FieldRec &r) { return (r.m / r.bm) * (r.m / r.bm) * r.batch; }

// one persistent launch of a stage over the records `recs` (device memory)
// with the grid persist_*_wave() (one wave of resident blocks)
int persist_density_wave(int stage);
int persist_wa_wave(int bucket);  // 0, 1, 2: the thread-per-net buckets; 3: the larger nets
int persist_field_wave();
void launch_persist_density(int stage, const PersistQueue &q, const void *recs, cudaStream_t st);
void launch_persist_wa(int bucket, const PersistQueue &q, const WaArgs *recs, cudaStream_t st);
void launch_persist_field(const PersistQueue &q, const FieldRec *recs, cudaStream_t st);

}  // namespace ap
