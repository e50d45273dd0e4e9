// C ABI of the placement library: handle life cycle, the iteration sequence
// (captured in CUDA graphs), initialisation, per-stage entry points, readout
// and snapshots.  Host-side equivalent of Placer (vck5000/host/src/
// AIEplace.cpp:9-138, 993-1124) over device-resident SoA state.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "../../include/aieplace.h"
#include "ap_kernels.h"
#include "ap_surrogate.h"

using namespace ap;

namespace {

#define CK(call)                                                               \
    do {                                                                       \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess) {                                               \
            fprintf(stderr, "aieplace: %s failed: %s\n", #call, cudaGetErrorString(e_)); \
            return AP_ERR_CUDA;                                                \
        }                                                                      \
    } while (0)

template <typename T>
cudaError_t dalloc(T **p, size_t n) {
    return cudaMalloc((void **)p, sizeof(T) * (n ? n : 1));
}

}  // namespace

struct ap_handle {
    // sizes
    // internal node order: real movable cells [0, n_real), filler cells
    // [n_real, n_mov), fixed nodes with area [n_mov, n_mov + n_fixa), then
    // zero-area fixed nodes; n_nodes counts all of them, n_ext the netlist's
    int n_nodes = 0, n_mov = 0, n_fixa = 0, n_nets = 0, n_pins = 0, n_small = 0;
    int n_ext = 0, n_real = 0, n_fill = 0;
    float fill_w = 0.f, fill_h = 0.f;
    std::vector<float> fill_x0, fill_y0;  // fillers' starting points (internal die coordinates)
    std::vector<int> ext2int, int2ext;    // int2ext[i] = -1 for fillers
    bool identity = true;
    float die_xl = 0, die_yl = 0, die_w = 0, die_h = 0;
    ap_params p{};
    Grid g{};
    long long cap_q = 0, ab_q = 0;
    double inv_ab = 0, mov_area_q = 0;
    float d_shift = 0.f;  // mean density of the loop's solver input, taken off before the solve
    // device state
    int *d_net_ptr = nullptr, *d_pin_node = nullptr;
    float *d_w = nullptr, *d_h = nullptr;
    int2 *d_whq = nullptr;  // to_q of the sizes, made once (launch_size_q)
    float *d_px[2] = {nullptr, nullptr}, *d_py[2] = {nullptr, nullptr};
    // all nodes' positions interleaved for the WA kernels: the loop's trial
    // point (movable nodes written by each position update, fixed nodes at
    // creation), and a scratch copy for WA evaluations at other points
    float2 *d_xy_loop = nullptr, *d_xy_tmp = nullptr;
    float *d_ux[2] = {nullptr, nullptr}, *d_uy[2] = {nullptr, nullptr};
    float *d_gx[2] = {nullptr, nullptr}, *d_gy[2] = {nullptr, nullptr};
    float *d_pins = nullptr, *d_charge = nullptr;
    int *d_rec_bin = nullptr;  // per movable node: bin record of the trial point
    int4 *d_rec_ov = nullptr;
    ull *d_gq = nullptr;                     // packed WA gradient accumulators (pack_q)
    ull *d_gqx = nullptr, *d_gqy = nullptr;  // per axis, nodes of more than kPackMaxPins pins
    ull *d_mov_q = nullptr;
    ull *d_fill_q = nullptr;  // filler cells' map: in the field, not in the overflow
    long long *d_fix_q = nullptr, *d_fixs_q = nullptr;
    float *d_dens = nullptr, *d_ex = nullptr, *d_ey = nullptr;
    __nv_bfloat16 *d_dens_hi = nullptr, *d_dens_lo = nullptr;
    float *d_sx = nullptr, *d_sy = nullptr;  // staging (external order / scratch positions)
    DevScalars *d_sc = nullptr;
    DevScalars *h_sc = nullptr;  // pinned
    double *d_partials = nullptr;
    long long *d_partials_ll = nullptr;
    unsigned int *d_counters = nullptr;
    double *d_out = nullptr;
    double *h_out = nullptr;  // pinned [4]
    unsigned int *h_status = nullptr;  // pinned: the tensor-core solve's status word, read by sync()
    int bucket_lo[kWaBuckets + 1] = {};
    FieldSolver fs{};
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    bool initialized = false;
    cudaGraphExec_t graph = nullptr;  // one trial step (parity lives in device scalars)
    bool graph_ok = false;
    // attached learned surrogate (not owned) and its per-handle buffers
    ap_surrogate *surr = nullptr;
    SurrState surr_state{};
    cudaStream_t side = nullptr;  // captures the field-switch bodies
    // the WA launches of a trial run beside scatter -> rho -> field
    cudaStream_t wa_stream = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // host step: the trial point's copy to the host runs on copy_stream from
    // the position update on (ev_upd), joined before the call returns (ev_copy)
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_upd = nullptr, ev_copy = nullptr;
    // host step input: copied in chunks on copy_in (ev_in[k] behind chunk k)
    // into d_ix / d_iy, each chunk's position update waiting for its copy
    cudaStream_t copy_in = nullptr;
    cudaEvent_t ev_start = nullptr, ev_in[4] = {nullptr, nullptr, nullptr, nullptr};
    float *d_ix = nullptr, *d_iy = nullptr;
    ap_surrogate_policy policy{0.3f, 8, 0.02f, 1};
    // trajectory log: device ring of per-trial records, drained into `log`
    // (JSON lines) whenever the scalars are read
    TrajRec *d_traj = nullptr;
    int traj_cap = 0;
    FILE *log = nullptr;
    long long log_next = 0;         // first trial not yet written
    unsigned long long log_t0 = 0;  // device clock of the first record written
    std::vector<TrajRec> log_buf;
};

namespace {

int solver_of(const ap_handle *h, int32_t solver) { return solver >= 0 ? solver : h->p.field_solver; }

// density map (bf16 split or fp32 already in place) -> ex, ey
int run_field(ap_handle *h, int solver, cudaStream_t st, const int *gate = nullptr, int gate_mask = 0) {
    if (solver == AP_FIELD_BF16X3) {
        int r = field_solve_bf16x3(h->fs, h->d_dens_hi, h->d_dens_lo, h->d_ex, h->d_ey, st, gate, gate_mask);
        if (r != AP_OK) return r;
    } else {
        field_solve_fp32(h->fs, h->d_dens, h->d_ex, h->d_ey, st, gate, gate_mask);
    }
    return AP_OK;
}

ScatterArgs scatter_args(ap_handle *h) {
    ScatterArgs a{};
    a.g = h->g;
    a.w = h->d_w;
    a.h = h->d_h;
    a.whq = h->d_whq;
    a.die_w = h->die_w;
    a.die_h = h->die_h;
    a.sc = h->d_sc;
    a.rho_q = h->d_mov_q;
    a.n_mov = h->n_mov;
    for (int b = 0; b < 2; ++b) {
        a.ux[b] = h->d_ux[b];
        a.uy[b] = h->d_uy[b];
        a.vx[b] = h->d_px[b];
        a.vy[b] = h->d_py[b];
        a.gx[b] = h->d_gx[b];
        a.gy[b] = h->d_gy[b];
    }
    a.partials = h->d_partials;
    a.counter = h->d_counters + 3;
    a.block_nodes = h->p.block_nodes;
    return a;
}

RhoArgs rho_args(ap_handle *h, int mode, double *out) {
    RhoArgs a{};
    a.nbins = h->p.bins_x * h->p.bins_y;
    a.mov_q = h->d_mov_q;
    a.fill_q = h->d_fill_q;
    a.fix_q = h->d_fix_q;
    a.fixs_q = h->d_fixs_q;
    a.cap_q = h->cap_q;
    a.ab_q = h->ab_q;
    a.inv_ab = h->inv_ab;
    a.inv_ab_f = (float)h->inv_ab;
    a.d_shift = h->d_shift;
    if (h->p.field_solver == AP_FIELD_BF16X3) {
        a.d_hi = h->d_dens_hi;
        a.d_lo = h->d_dens_lo;
    } else {
        a.d_f32 = h->d_dens;
    }
    a.sc = h->d_sc;
    a.partials = h->d_partials_ll;
    a.counter = h->d_counters + 1;
    a.out = out;
    a.mode = mode;
    return a;
}

WaArgs wa_args(ap_handle *h, const float *px, const float *py, float gamma, int n_grad, int mode,
               double *out) {
    WaArgs a{};
    a.net_ptr = h->d_net_ptr;
    a.pin_node = h->d_pin_node;
    a.n_small = h->n_small;
    for (int b = 0; b <= kWaBuckets; ++b) a.bucket_lo[b] = h->bucket_lo[b];
    a.n_nets = h->n_nets;
    a.px = px;
    a.py = py;
    a.xy = mode == WA_LOOP ? h->d_xy_loop : h->d_xy_tmp;
    a.n_nodes = h->n_nodes;
    a.gamma = gamma;
    a.sc = h->d_sc;
    a.gq = h->d_gq;
    a.gqx = h->d_gqx;
    a.gqy = h->d_gqy;
    a.n_grad = n_grad;
    a.partials = h->d_partials;
    a.counter = h->d_counters + 0;
    a.out = out;
    a.mode = mode;
    a.block_nets = h->p.block_nodes;
    return a;
}

GatherArgs gather_args(ap_handle *h, int at, int mode) {
    GatherArgs a{};
    a.g = h->g;
    a.n_mov = h->n_mov;
    a.at = at;
    for (int b = 0; b < 2; ++b) {
        a.vx[b] = h->d_px[b];
        a.vy[b] = h->d_py[b];
        a.gx[b] = h->d_gx[b];
        a.gy[b] = h->d_gy[b];
    }
    a.w = h->d_w;
    a.h = h->d_h;
    a.ex = h->d_ex;
    a.ey = h->d_ey;
    a.gq = h->d_gq;
    a.gqx = h->d_gqx;
    a.gqy = h->d_gqy;
    a.pins = h->d_pins;
    a.charge = h->d_charge;
    a.sc = h->d_sc;
    a.partials = h->d_partials;
    a.counter = h->d_counters + 2;
    a.mode = mode;
    a.block_nodes = h->p.block_nodes;
    return a;
}

// The loop's scatter (update mode, writes the bin records) and gather (reads them).
ScatterArgs loop_scatter_args(ap_handle *h) {
    ScatterArgs s = scatter_args(h);
    s.update = 1;
    s.rec_bin = h->d_rec_bin;
    s.rec_ov = h->d_rec_ov;
    s.xy_out = h->d_xy_loop;
    s.lo = 0;
    s.hi = h->n_mov;
    return s;
}

// Bin adds of the movable nodes (either mode): real cells into the movable
// map, filler cells into their own.
void launch_movable_bins(ap_handle *h, ScatterArgs s, cudaStream_t st) {
    s.lo = 0;
    s.hi = h->n_real;
    s.rho_q = h->d_mov_q;
    launch_scatter_bins(s, st);
    if (h->n_fill) {
        s.lo = h->n_real;
        s.hi = h->n_mov;
        s.rho_q = h->d_fill_q;
        launch_scatter_bins(s, st);
    }
}

GatherArgs loop_gather_args(ap_handle *h) {
    GatherArgs a = gather_args(h, 0, GATHER_STEP);
    a.rec_bin = h->d_rec_bin;
    a.rec_ov = h->d_rec_ov;
    return a;
}

// One trial step from the accepted state (buffers [cur]) to buffers
// [1 - cur]; cur lives in device scalars, so one captured graph serves every
// launch.  The gather's last block accepts the trial or asks for a retry.
// Field stage of a trial with a surrogate attached.  The rho kernel's last
// block picks the source (device scalars): exact, surrogate, or both with the
// surrogate judged.  branch < 0: every launch, each reading the mode from
// device memory and returning early if it is not selected; branch >= 0: the
// launches of that source only (one body of the graph's switch node).
int enqueue_field_surrogate(ap_handle *h, cudaStream_t st, int branch) {
    const int *gate = &h->d_sc->field_mode;
    const bool f32 = h->p.field_solver != AP_FIELD_BF16X3;
    if (branch != kFieldExact)
        surr_enqueue_field(h->surr->net, h->surr_state, f32 ? h->d_dens : nullptr, f32 ? nullptr : h->d_dens_hi,
                           f32 ? nullptr : h->d_dens_lo, h->d_ex, h->d_ey, gate, st);
    if (branch != kFieldSurr) {
        int r = run_field(h, h->p.field_solver, st, gate, kGateExact);
        if (r != AP_OK) return r;
    }
    if (branch < 0 || branch == kFieldJudge) surr_enqueue_judge(h->surr_state, h->d_ex, h->d_ey, h->d_sc, gate, st);
    return AP_OK;
}

// The WA launches of a trial on their own stream, after the position update
// and joined before the gather (fork_wa / join_wa): the WA gradient needs the
// trial point and the previous evaluation's gamma, not this trial's density.
int fork_wa(ap_handle *h, cudaStream_t st) {
    CK(cudaEventRecord(h->ev_fork, st));
    CK(cudaStreamWaitEvent(h->wa_stream, h->ev_fork, 0));
    launch_wirelength(wa_args(h, h->d_px[0], h->d_py[0], 0.f, h->n_mov, WA_LOOP, nullptr), h->wa_stream);
    CK(cudaEventRecord(h->ev_join, h->wa_stream));
    return AP_OK;
}

int join_wa(ap_handle *h, cudaStream_t st) {
    CK(cudaStreamWaitEvent(st, h->ev_join, 0));
    return AP_OK;
}

// The trial after its position update.
int enqueue_after_update(ap_handle *h, cudaStream_t st) {
    int r = fork_wa(h, st);
    if (r != AP_OK) return r;
    launch_movable_bins(h, loop_scatter_args(h), st);
    launch_rho(rho_args(h, RHO_LOOP, nullptr), st);
    if (h->surr) {
        r = enqueue_field_surrogate(h, st, -1);
        if (r != AP_OK) return r;
    } else {
        r = run_field(h, h->p.field_solver, st);
        if (r != AP_OK) return r;
    }
    r = join_wa(h, st);
    if (r != AP_OK) return r;
    launch_gather(loop_gather_args(h), st);
    return cudaGetLastError() == cudaSuccess ? AP_OK : AP_ERR_CUDA;
}

int enqueue_iteration(ap_handle *h, cudaStream_t st) {
    launch_update(loop_scatter_args(h), st);
    return enqueue_after_update(h, st);
}

// Density/overflow + WA + field at buffer `at` (no position update).
int enqueue_eval(ap_handle *h, int at, int rho_mode, int wa_mode, cudaStream_t st) {
    ScatterArgs s = scatter_args(h);
    s.update = 0;
    s.px = h->d_px[at];
    s.py = h->d_py[at];
    launch_movable_bins(h, s, st);
    launch_rho(rho_args(h, rho_mode, h->d_out), st);
    launch_wirelength(wa_args(h, h->d_px[at], h->d_py[at], 0.f, h->n_mov, wa_mode, h->d_out + 2), st);
    return run_field(h, h->p.field_solver, st);
}

// Waits for the handle's stream; a tensor-core solve that gave up reports
// AP_ERR_TIMEOUT.  Its status word is copied behind the stream's work, so
// one wait covers both (a separate read after the wait was a second round
// trip per call).
int sync(ap_handle *h) {
    const bool tc = h->fs.tc_ready && h->fs.tc_status;
    if (tc)
        CK(cudaMemcpyAsync(h->h_status, h->fs.tc_status, sizeof(unsigned int), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (tc && *h->h_status) return AP_ERR_TIMEOUT;
    return AP_OK;
}

void destroy_graphs(ap_handle *h) {
    if (h->graph) {
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
    }
    h->graph_ok = false;
}

// One trial with a surrogate attached, captured with a switch node over the
// field sources: the rho kernel sets the switch (cudaGraphSetConditional), so
// only the selected source's kernels launch.
int capture_trial_switched(ap_handle *h) {
    cudaStream_t st = h->stream;
    if (!h->side) CK(cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking));
    cudaStreamCaptureStatus cs;
    cudaGraph_t cg = nullptr;
    CK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &cg, nullptr, nullptr, nullptr));
    cudaGraphConditionalHandle sw_handle;
    CK(cudaGraphConditionalHandleCreate(&sw_handle, cg, kFieldExact, cudaGraphCondAssignDefault));
    const ScatterArgs sa = loop_scatter_args(h);
    launch_update(sa, st);
    const int fr = fork_wa(h, st);
    if (fr != AP_OK) return fr;
    launch_movable_bins(h, sa, st);
    RhoArgs ra = rho_args(h, RHO_LOOP, nullptr);
    ra.field_switch = sw_handle;
    launch_rho(ra, st);
    const cudaGraphNode_t *dp = nullptr;
    size_t nd = 0;
    CK(cudaStreamGetCaptureInfo(st, &cs, nullptr, nullptr, &dp, nullptr, &nd));
    std::vector<cudaGraphNode_t> deps(dp, dp + nd);
    cudaGraphNodeParams np{};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = sw_handle;
    np.conditional.type = cudaGraphCondTypeSwitch;
    np.conditional.size = 3;  // kFieldExact, kFieldSurr, kFieldJudge
    cudaGraphNode_t sw = nullptr;
    CK(cudaGraphAddNode(&sw, cg, deps.data(), nullptr, deps.size(), &np));
    for (int b = 0; b < 3; ++b) {
        CK(cudaStreamBeginCaptureToGraph(h->side, np.conditional.phGraph_out[b], nullptr, nullptr, 0,
                                         cudaStreamCaptureModeThreadLocal));
        const int r = enqueue_field_surrogate(h, h->side, b);
        cudaGraph_t body = nullptr;
        const cudaError_t e = cudaStreamEndCapture(h->side, &body);
        if (r != AP_OK) return r;
        CK(e);
    }
    CK(cudaStreamUpdateCaptureDependencies(st, &sw, nullptr, 1, cudaStreamSetCaptureDependencies));
    const int jr = join_wa(h, st);
    if (jr != AP_OK) return jr;
    launch_gather(loop_gather_args(h), st);
    return cudaGetLastError() == cudaSuccess ? AP_OK : AP_ERR_CUDA;
}

int build_graphs(ap_handle *h) {
    destroy_graphs(h);
    cudaGraph_t gr = nullptr;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int r = h->surr ? capture_trial_switched(h) : enqueue_iteration(h, h->stream);
    cudaError_t e = cudaStreamEndCapture(h->stream, &gr);
    if (r != AP_OK || e != cudaSuccess) {
        if (gr) cudaGraphDestroy(gr);
        return r != AP_OK ? r : AP_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&h->graph, gr, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(gr);
    if (e != cudaSuccess) return AP_ERR_CUDA;
    h->graph_ok = true;
    return AP_OK;
}

// external-order host arrays -> internal positions of buffer `at` (movable
// nodes only; fixed nodes keep their place)
int upload_positions(ap_handle *h, int at, const float *x, const float *y) {
    std::vector<float> ix((size_t)h->n_mov), iy((size_t)h->n_mov);
    for (int i = 0; i < h->n_mov; ++i) {
        const int e = h->int2ext[(size_t)i];
        if (e < 0) {  // filler cells start where ap_create put them
            ix[(size_t)i] = h->fill_x0[(size_t)(i - h->n_real)];
            iy[(size_t)i] = h->fill_y0[(size_t)(i - h->n_real)];
            continue;
        }
        ix[(size_t)i] = x[e] - h->die_xl;
        iy[(size_t)i] = y[e] - h->die_yl;
        if (!std::isfinite(ix[(size_t)i]) || !std::isfinite(iy[(size_t)i])) return AP_ERR_NONFINITE;
    }
    CK(cudaMemcpyAsync(h->d_px[at], ix.data(), sizeof(float) * h->n_mov, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->d_py[at], iy.data(), sizeof(float) * h->n_mov, cudaMemcpyHostToDevice, h->stream));
    return sync(h);
}

// Writes the trajectory records of the trials run since the last drain (the
// scalars in h_sc are fresh).  A ring that wrapped since then loses its
// oldest records; the log says how many.
int drain_log(ap_handle *h) {
    const long long ev = h->h_sc->evals;
    if (ev < h->log_next) h->log_next = 0;  // the optimiser was reset
    if (ev == h->log_next) return AP_OK;
    if (ev - h->log_next > h->traj_cap) {
        fprintf(h->log, "{\"lost_trials\": %lld}\n", ev - h->traj_cap - h->log_next);
        h->log_next = ev - h->traj_cap;
    }
    const long long n = ev - h->log_next;
    h->log_buf.resize((size_t)n);
    const long long first = h->log_next % h->traj_cap;
    const long long run1 = std::min(n, h->traj_cap - first);
    CK(cudaMemcpyAsync(h->log_buf.data(), h->d_traj + first, sizeof(TrajRec) * run1, cudaMemcpyDeviceToHost,
                       h->stream));
    if (run1 < n)
        CK(cudaMemcpyAsync(h->log_buf.data() + run1, h->d_traj, sizeof(TrajRec) * (n - run1), cudaMemcpyDeviceToHost,
                           h->stream));
    CK(cudaStreamSynchronize(h->stream));
    static const char *fields[] = {"exact", "surrogate", "judged"};
    for (const TrajRec &r : h->log_buf) {
        if (!h->log_t0) h->log_t0 = r.t_ns;
        const char *fm = r.field_mode >= 0 && r.field_mode < 3 ? fields[r.field_mode] : "exact";
        fprintf(h->log,
                "{\"eval\": %d, \"iteration\": %d, \"accepted\": %s, \"hpwl\": %.17g, \"overflow\": %.17g, "
                "\"overflow_abs\": %.17g, \"lambda\": %.17g, \"alpha\": %.17g, \"gamma\": %.17g, \"field\": \"%s\", "
                "\"surrogate_error\": %.9g, \"t_ms\": %.6f}\n",
                r.eval, r.iteration, r.accepted > 0 ? "true" : (r.accepted == 0 ? "false" : "\"diverged\""), r.hpwl,
                r.overflow, r.overflow_abs, r.lambda, r.alpha, r.gamma, fm, r.surr_err,
                (double)(r.t_ns - h->log_t0) * 1e-6);
    }
    fflush(h->log);
    h->log_next = ev;
    return AP_OK;
}

int read_scalars(ap_handle *h) {
    CK(cudaMemcpyAsync(h->h_sc, h->d_sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, h->stream));
    const int r = sync(h);
    if (r != AP_OK || !h->log) return r;
    return drain_log(h);
}

// Positions of the accepted buffer (device scalar `cur`) <-> staging arrays,
// on the device, so the host needs no round trip to learn `cur`:
// to_cur = 1: s -> [cur] for the first n nodes, else [cur] -> s.
__global__ void stage_cur_kernel(int n, int to_cur, const DevScalars *sc, float *x0, float *y0, float *x1, float *y1,
                                 float *sx, float *sy) {
    const int cur = sc->cur;
    float *x = cur ? x1 : x0, *y = cur ? y1 : y0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (to_cur) {
            x[i] = sx[i];
            y[i] = sy[i];
        } else {
            sx[i] = x[i];
            sy[i] = y[i];
        }
    }
}

// Host step: the fixed nodes' positions (nodes [first, first + n)) from
// buffers [cur] into the staging arrays, which hold the whole result once the
// position update has written the trial point of the movable nodes.
__global__ void stage_in_kernel(int n, int first, const DevScalars *sc, const float *x0, const float *y0,
                                const float *x1, const float *y1, float *sx, float *sy) {
    const int cur = sc->cur;
    const float *x = cur ? x1 : x0, *y = cur ? y1 : y0;
    for (int i = first + blockIdx.x * blockDim.x + threadIdx.x; i < first + n; i += gridDim.x * blockDim.x) {
        sx[i] = x[i];
        sy[i] = y[i];
    }
}

void stage_cur(ap_handle *h, int n, int to_cur) {
    if (n <= 0) return;
    const int blocks = std::min((n + kThreads - 1) / kThreads, 4096);
    stage_cur_kernel<<<blocks, kThreads, 0, h->stream>>>(n, to_cur, h->d_sc, h->d_px[0], h->d_py[0], h->d_px[1],
                                                         h->d_py[1], h->d_sx, h->d_sy);
}

void fill_stats(const ap_handle *h, ap_stats *s) {
    const DevScalars &c = *h->h_sc;
    s->iteration = c.iteration;
    s->status = c.status;
    s->hpwl = c.hpwl;
    s->wa_wirelength = c.wa;
    s->overflow = c.tau;
    s->overflow_abs = c.tau_abs;
    s->lambda = c.lambda;
    s->gamma = c.gamma;
    s->alpha = c.alpha;
    s->a_k = c.a_k;
    s->evals = c.evals;
    s->restarts = c.restarts;
}

// Evaluates v_0, lambda_0, g_0, the probe point v_{-1} and g_{-1}, and the
// first step length (ePlace: Lipschitz prediction from two points).  Leaves
// the accepted state in buffers [0].
int init_optimizer(ap_handle *h) {
    cudaStream_t st = h->stream;
    destroy_graphs(h);
    DevScalars sc{};
    sc.a_k = 1.0;
    sc.gamma_base = h->p.gamma_base_bins;
    sc.bin_avg = 0.5 * ((double)h->g.bw + (double)h->g.bh);
    sc.mu_max = h->p.lambda_mu_max;
    sc.mu_min = h->p.lambda_mu_min;
    sc.init_density_weight = h->p.init_density_weight;
    sc.ref_dh = h->p.ref_delta_hpwl > 0 ? h->p.ref_delta_hpwl : 0.1 * h->n_nets * (double)h->g.bw;
    sc.mov_area_q = h->mov_area_q;
    sc.max_backtracks = h->p.max_backtracks;
    sc.restart_mode = h->p.restart_mode;
    sc.cur = 0;
    sc.surr_attached = h->surr != nullptr;
    sc.surr_ok = 1;
    sc.surr_judge_every = h->policy.judge_every;
    sc.surr_tau_min = h->policy.overflow_min;
    sc.surr_err_bound = h->policy.max_error;
    sc.traj = h->d_traj;
    sc.traj_cap = h->traj_cap;
    h->log_next = 0;
    h->log_t0 = 0;
    CK(cudaMemcpyAsync(h->d_sc, &sc, sizeof(sc), cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(h->d_gq, 0, sizeof(ull) * h->n_nodes, st));
    CK(cudaMemsetAsync(h->d_gqx, 0, sizeof(ull) * h->n_nodes, st));
    CK(cudaMemsetAsync(h->d_gqy, 0, sizeof(ull) * h->n_nodes, st));
    CK(cudaMemsetAsync(h->d_mov_q, 0, sizeof(ull) * (size_t)h->p.bins_x * h->p.bins_y, st));
    if (h->d_fill_q) CK(cudaMemsetAsync(h->d_fill_q, 0, sizeof(ull) * (size_t)h->p.bins_x * h->p.bins_y, st));
    CK(cudaMemsetAsync(h->d_counters, 0, sizeof(unsigned int) * 8, st));
    // u_0 = v_0
    CK(cudaMemcpyAsync(h->d_ux[0], h->d_px[0], sizeof(float) * h->n_mov, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(h->d_uy[0], h->d_py[0], sizeof(float) * h->n_mov, cudaMemcpyDeviceToDevice, st));
    int r = enqueue_eval(h, 0, RHO_INIT, WA_INIT, st);
    if (r != AP_OK) return r;
    launch_gather(gather_args(h, 0, GATHER_INIT_NORMS), st);
    launch_gather(gather_args(h, 0, GATHER_INIT_GRAD), st);
    launch_perturb(h->n_mov, h->d_px[0], h->d_py[0], h->d_gx[0], h->d_gy[0], h->d_px[1], h->d_py[1],
                   &h->d_sc->gmax, h->p.init_step_coef * h->g.bw, h->die_w, h->die_h, h->d_w, h->d_h, st);
    r = enqueue_eval(h, 1, RHO_OUT_ONLY, WA_OUT_ONLY, st);
    if (r != AP_OK) return r;
    launch_gather(gather_args(h, 1, GATHER_INIT_PREV), st);
    CK(cudaGetLastError());
    h->initialized = true;
    r = sync(h);
    if (r != AP_OK) return r;
    if (h->p.use_graph) {
        r = build_graphs(h);
        if (r != AP_OK) return r;
    }
    return AP_OK;
}

// n trial launches (no host synchronisation)
int launch_trials(ap_handle *h, int n) {
    for (int i = 0; i < n; ++i) {
        if (h->graph_ok) {
            CK(cudaGraphLaunch(h->graph, h->stream));
        } else {
            int r = enqueue_iteration(h, h->stream);
            if (r != AP_OK) return r;
        }
    }
    CK(cudaGetLastError());
    return AP_OK;
}

// Runs trials until `n` more iterations are accepted.  Launches in batches
// of the remaining count (each accepted iteration needs at least one trial)
// and reads the counters back between batches.
int step_n(ap_handle *h, int n) {
    int r = read_scalars(h);
    if (r != AP_OK) return r;
    const int target = h->h_sc->iteration + n;
    for (int guard = 0; guard < 64; ++guard) {
        const int left = target - h->h_sc->iteration;
        if (left <= 0 || h->h_sc->status) break;
        r = launch_trials(h, left);
        if (r != AP_OK) return r;
        r = read_scalars(h);
        if (r != AP_OK) return r;
    }
    return h->h_sc->status;
}

}  // namespace

extern "C" {

int ap_abi_version(void) { return AP_ABI_VERSION; }

const char *ap_status_string(int s) {
    switch (s) {
        case AP_OK: return "ok";
        case AP_ERR_INVALID_ARG: return "invalid argument";
        case AP_ERR_BAD_NETLIST: return "malformed netlist";
        case AP_ERR_NONFINITE: return "non-finite input";
        case AP_ERR_CUDA: return "CUDA error";
        case AP_ERR_NO_DEVICE: return "no sm_103 device";
        case AP_ERR_UNSUPPORTED: return "unsupported configuration";
        case AP_ERR_TIMEOUT: return "device wait timed out";
        case AP_ERR_STATE: return "call out of order";
        case AP_ERR_DIVERGED: return "optimiser diverged";
        default: return "unknown status";
    }
}

int ap_params_default(ap_params *p) {
    if (!p) return AP_ERR_INVALID_ARG;
    memset(p, 0, sizeof(*p));
    p->bins_x = 512;
    p->bins_y = 512;
    p->target_density = 1.0f;
    p->gamma_base_bins = 4.0f;
    p->field_solver = AP_FIELD_FP32;
    p->init_density_weight = 8e-5f;
    p->ref_delta_hpwl = 0.f;
    p->lambda_mu_max = 1.05f;
    p->lambda_mu_min = 0.95f;
    p->init_step_coef = 0.1f;
    p->target_overflow = 0.10f;
    p->max_iterations = 5000;
    p->check_interval = 16;
    p->use_graph = 1;
    p->max_backtracks = 0;
    p->restart_mode = 4;
    p->filler_cells = 0;
    p->block_nodes = 0;
    return AP_OK;
}

int ap_create(const ap_netlist *nl, const ap_params *params, ap_handle **out) {
    if (!nl || !params || !out) return AP_ERR_INVALID_ARG;
    *out = nullptr;
    const ap_params &p = *params;
    if (nl->num_nodes <= 0 || nl->num_nets < 0 || nl->num_pins < 0 || !nl->net_ptr ||
        (nl->num_pins > 0 && !nl->pin_node) || !nl->node_w || !nl->node_h || !nl->node_x || !nl->node_y)
        return AP_ERR_INVALID_ARG;
    if (p.bins_x != p.bins_y || p.bins_x < 32 || p.bins_x > 4096 || (p.bins_x & (p.bins_x - 1)))
        return AP_ERR_UNSUPPORTED;
    if (!(p.target_density > 0.f) || !(p.gamma_base_bins > 0.f)) return AP_ERR_INVALID_ARG;
    if (p.field_solver != AP_FIELD_FP32 && p.field_solver != AP_FIELD_BF16X3) return AP_ERR_INVALID_ARG;
    const float die_w = nl->die_xh - nl->die_xl, die_h = nl->die_yh - nl->die_yl;
    if (!(die_w > 0.f) || !(die_h > 0.f)) return AP_ERR_INVALID_ARG;
    // CSR checks
    if (nl->net_ptr[0] != 0 || nl->net_ptr[nl->num_nets] != nl->num_pins) return AP_ERR_BAD_NETLIST;
    for (int e = 0; e < nl->num_nets; ++e)
        if (nl->net_ptr[e + 1] < nl->net_ptr[e]) return AP_ERR_BAD_NETLIST;
    for (int q = 0; q < nl->num_pins; ++q)
        if (nl->pin_node[q] < 0 || nl->pin_node[q] >= nl->num_nodes) return AP_ERR_BAD_NETLIST;
    for (int i = 0; i < nl->num_nodes; ++i)
        if (!std::isfinite(nl->node_w[i]) || !std::isfinite(nl->node_h[i]) || !std::isfinite(nl->node_x[i]) ||
            !std::isfinite(nl->node_y[i]) || nl->node_w[i] < 0.f || nl->node_h[i] < 0.f)
            return AP_ERR_NONFINITE;
    int dev = 0;
    cudaDeviceProp prop;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess)
        return AP_ERR_NO_DEVICE;
    if (prop.major != 10 || prop.minor != 3) return AP_ERR_NO_DEVICE;

    ap_handle *h = new ap_handle();
    h->p = p;
    h->die_xl = nl->die_xl;
    h->die_yl = nl->die_yl;
    h->die_w = die_w;
    h->die_h = die_h;
    const int NE = nl->num_nodes;
    h->n_ext = NE;
    // filler cells (ePlace): unconnected movable cells that take the white
    // space the target density leaves, so that the density force spreads
    // the real cells evenly; the overflow counts real cells only
    if (p.filler_cells) {
        double a_mov = 0.0, a_fix = 0.0;
        std::vector<double> areas;
        for (int i = 0; i < NE; ++i) {
            const bool fixed = nl->node_fixed && nl->node_fixed[i];
            const double w = nl->node_w[i], hh = nl->node_h[i];
            if (!fixed) {
                a_mov += w * hh;
                areas.push_back(w * hh);
            } else {  // the part of the fixed node on the die
                const double ox = std::min((double)nl->die_xh, (double)nl->node_x[i] + w) -
                                  std::max((double)nl->die_xl, (double)nl->node_x[i]);
                const double oy = std::min((double)nl->die_yh, (double)nl->node_y[i] + hh) -
                                  std::max((double)nl->die_yl, (double)nl->node_y[i]);
                if (ox > 0 && oy > 0) a_fix += ox * oy;
            }
        }
        const double a_fill = (double)p.target_density * ((double)die_w * die_h - a_fix) - a_mov;
        if (a_fill > 0 && !areas.empty()) {
            // filler size: mean width and height of the cells between the 10th
            // and the 90th area percentile (ePlace)
            std::vector<int> idx;
            for (int i = 0; i < NE; ++i)
                if (!(nl->node_fixed && nl->node_fixed[i])) idx.push_back(i);
            std::sort(idx.begin(), idx.end(), [&](int a, int b) {
                return (double)nl->node_w[a] * nl->node_h[a] < (double)nl->node_w[b] * nl->node_h[b];
            });
            const size_t lo = idx.size() / 10, hi = idx.size() - idx.size() / 10;
            double sw = 0, sh = 0;
            for (size_t k = lo; k < hi; ++k) {
                sw += nl->node_w[idx[k]];
                sh += nl->node_h[idx[k]];
            }
            h->fill_w = (float)(sw / (double)(hi - lo));
            h->fill_h = (float)(sh / (double)(hi - lo));
            if (h->fill_w > 0.f && h->fill_h > 0.f)
                h->n_fill = (int)std::min(a_fill / ((double)h->fill_w * h->fill_h), 2e9 - NE);
        }
    }
    const int N = NE + h->n_fill;
    h->n_nodes = N;
    // internal order: movable, fillers, fixed with area, zero-area fixed
    h->ext2int.assign((size_t)NE, -1);
    for (int pass = 0; pass < 3; ++pass) {
        for (int i = 0; i < NE; ++i) {
            const bool fixed = nl->node_fixed && nl->node_fixed[i];
            const bool area = nl->node_w[i] * nl->node_h[i] > 0.f;
            const int cls = !fixed ? 0 : (area ? 1 : 2);
            if (cls == pass) {
                h->ext2int[(size_t)i] = (int)h->int2ext.size();
                h->int2ext.push_back(i);
                if (cls == 0) h->n_real++;
                if (cls == 1) h->n_fixa++;
            }
        }
        if (pass == 0) h->int2ext.insert(h->int2ext.end(), (size_t)h->n_fill, -1);
    }
    h->n_mov = h->n_real + h->n_fill;
    h->identity = h->n_fill == 0;
    for (int i = 0; i < NE; ++i)
        if (h->ext2int[(size_t)i] != i) h->identity = false;
    if (h->n_fill) {  // seeded, uniform over the die
        uint64_t z = 0x5EED0F111E4ull;
        auto uni = [&]() {
            z += 0x9E3779B97F4A7C15ull;
            uint64_t t = z;
            t = (t ^ (t >> 30)) * 0xBF58476D1CE4E5B9ull;
            t = (t ^ (t >> 27)) * 0x94D049BB133111EBull;
            return (double)((t ^ (t >> 31)) >> 11) * (1.0 / 9007199254740992.0);
        };
        h->fill_x0.resize((size_t)h->n_fill);
        h->fill_y0.resize((size_t)h->n_fill);
        for (int k = 0; k < h->n_fill; ++k) {
            h->fill_x0[(size_t)k] = (float)(uni() * std::max(0.0, (double)die_w - h->fill_w));
            h->fill_y0[(size_t)k] = (float)(uni() * std::max(0.0, (double)die_h - h->fill_h));
        }
    }
    // nets of degree >= 2 in degree buckets [2], [3,4], [5,8], [9,16], [17,32],
    // [33,64], [65,...); within a bucket by their lowest internal node index, so
    // neighbouring threads gather and accumulate neighbouring nodes
    auto bucket_of = [](int d) {
        return d <= 2 ? 0 : d <= 4 ? 1 : d <= 8 ? 2 : d <= 16 ? 3 : d <= 32 ? 4 : d <= 64 ? 5 : 6;
    };
    std::vector<int> order, first((size_t)nl->num_nets, 0);
    for (int e = 0; e < nl->num_nets; ++e) {
        if (nl->net_ptr[e + 1] - nl->net_ptr[e] < 2) continue;
        order.push_back(e);
        int lo = INT32_MAX;
        for (int q = nl->net_ptr[e]; q < nl->net_ptr[e + 1]; ++q) lo = std::min(lo, h->ext2int[(size_t)nl->pin_node[q]]);
        first[(size_t)e] = lo;
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        const int ka = bucket_of(nl->net_ptr[a + 1] - nl->net_ptr[a]), kb = bucket_of(nl->net_ptr[b + 1] - nl->net_ptr[b]);
        return ka != kb ? ka < kb : first[(size_t)a] < first[(size_t)b];
    });
    std::vector<int> net_ptr(1, 0), pin_node;
    std::vector<float> pins((size_t)N, 0.f);
    for (int b = 0; b <= kWaBuckets; ++b) h->bucket_lo[b] = 0;
    for (int e : order) {
        const int d = nl->net_ptr[e + 1] - nl->net_ptr[e];
        if (d <= 8) h->n_small++;
        for (int b = bucket_of(d) + 1; b <= kWaBuckets; ++b) h->bucket_lo[b]++;
        for (int q = nl->net_ptr[e]; q < nl->net_ptr[e + 1]; ++q) {
            const int in = h->ext2int[(size_t)nl->pin_node[q]];
            pin_node.push_back(in);
            pins[(size_t)in] += 1.f;
        }
        net_ptr.push_back((int)pin_node.size());
    }
    h->n_nets = (int)order.size();
    h->n_pins = (int)pin_node.size();
    // pins of nodes past the packed accumulators' range carry the heavy flag
    for (int &q : pin_node)
        if (pins[(size_t)q] > (float)kPackMaxPins) q |= kPinHeavy;
    // node arrays in internal order
    std::vector<float> w((size_t)N), hh((size_t)N), x((size_t)N), y((size_t)N), charge((size_t)N);
    for (int i = 0; i < N; ++i) {
        const int e = h->int2ext[(size_t)i];
        if (e < 0) {
            const size_t k = (size_t)(i - h->n_real);
            w[(size_t)i] = h->fill_w;
            hh[(size_t)i] = h->fill_h;
            x[(size_t)i] = h->fill_x0[k];
            y[(size_t)i] = h->fill_y0[k];
            continue;
        }
        w[(size_t)i] = nl->node_w[e];
        hh[(size_t)i] = nl->node_h[e];
        x[(size_t)i] = nl->node_x[e] - nl->die_xl;
        y[(size_t)i] = nl->node_y[e] - nl->die_yl;
    }
    // grid (Grid::init, Grid.cpp:6-22) and fixed-point constants
    Grid &g = h->g;
    g.mx = p.bins_x;
    g.my = p.bins_y;
    g.bw = die_w / (float)p.bins_x;
    g.bh = die_h / (float)p.bins_y;
    g.small_threshold = g.bw * g.bh / 16;
    g.bw_q = llrintf(g.bw * 65536.0f);
    g.bh_q = llrintf(g.bh * 65536.0f);
    h->ab_q = g.bw_q * g.bh_q;
    h->cap_q = llrint((double)p.target_density * (double)h->ab_q);
    h->inv_ab = 1.0 / (double)h->ab_q;
    g.inv_ab = (float)h->inv_ab;
    double mov_area_q = 0.0, fill_area_q = 0.0;  // the overflow's denominator counts real cells
    for (int i = 0; i < h->n_mov; ++i) {
        const double a = (double)(llrintf(w[(size_t)i] * 65536.0f) * llrintf(hh[(size_t)i] * 65536.0f));
        if (i < h->n_real)
            mov_area_q += a;
        else
            fill_area_q += a;
        charge[(size_t)i] = (w[(size_t)i] * hh[(size_t)i]) / (g.bw * g.bh);
    }
    h->mov_area_q = mov_area_q;

    const size_t nb = (size_t)p.bins_x * p.bins_y;
    bool ok = true;
    auto A = [&](cudaError_t e) { ok = ok && e == cudaSuccess; };
    A(dalloc(&h->d_net_ptr, net_ptr.size()));
    A(dalloc(&h->d_pin_node, pin_node.size()));
    A(dalloc(&h->d_w, N));
    A(dalloc(&h->d_h, N));
    A(dalloc(&h->d_whq, N));
    for (int b = 0; b < 2; ++b) {
        A(dalloc(&h->d_px[b], N));
        A(dalloc(&h->d_py[b], N));
        A(dalloc(b ? &h->d_xy_tmp : &h->d_xy_loop, N));
        A(dalloc(&h->d_gx[b], std::max(1, h->n_mov)));
        A(dalloc(&h->d_gy[b], std::max(1, h->n_mov)));
    }
    for (int b = 0; b < 2; ++b) {
        A(dalloc(&h->d_ux[b], std::max(1, h->n_mov)));
        A(dalloc(&h->d_uy[b], std::max(1, h->n_mov)));
    }
    A(dalloc(&h->d_pins, N));
    A(dalloc(&h->d_charge, N));
    A(dalloc(&h->d_rec_bin, std::max(1, h->n_mov)));
    A(dalloc(&h->d_rec_ov, std::max(1, h->n_mov)));
    A(dalloc(&h->d_gq, N));
    A(dalloc(&h->d_gqx, N));
    A(dalloc(&h->d_gqy, N));
    A(dalloc(&h->d_mov_q, nb));
    if (h->n_fill) A(dalloc(&h->d_fill_q, nb));
    A(dalloc(&h->d_fix_q, nb));
    A(dalloc(&h->d_fixs_q, nb));
    A(dalloc(&h->d_dens, nb));
    A(dalloc(&h->d_dens_hi, nb));
    A(dalloc(&h->d_dens_lo, nb));
    A(dalloc(&h->d_ex, nb));
    A(dalloc(&h->d_ey, nb));
    A(dalloc(&h->d_sx, N));
    A(dalloc(&h->d_sy, N));
    A(dalloc(&h->d_sc, 1));
    A(dalloc(&h->d_partials, kPartialDoubles));
    A(dalloc(&h->d_partials_ll, 2 * 4096 + 64));
    A(dalloc(&h->d_counters, 8));
    A(dalloc(&h->d_out, 8));
    A(cudaMallocHost((void **)&h->h_sc, sizeof(DevScalars)));
    A(cudaMallocHost((void **)&h->h_out, sizeof(double) * 8));
    A(cudaMallocHost((void **)&h->h_status, sizeof(unsigned int)));
    // the WA launches run beside the density chain (scatter -> rho -> field)
    // at the same priority: with the chain's stream at the highest priority a
    // 2M-cell trial took 1.5% longer (its blocks kept the WA blocks waiting
    // where both would have shared the SMs)
    A(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    h->own_stream = true;
    A(cudaStreamCreateWithFlags(&h->wa_stream, cudaStreamNonBlocking));
    A(cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming));
    A(cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming));
    A(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
    A(cudaEventCreateWithFlags(&h->ev_upd, cudaEventDisableTiming));
    A(cudaEventCreateWithFlags(&h->ev_copy, cudaEventDisableTiming));
    A(cudaStreamCreateWithFlags(&h->copy_in, cudaStreamNonBlocking));
    A(cudaEventCreateWithFlags(&h->ev_start, cudaEventDisableTiming));
    for (cudaEvent_t &e : h->ev_in) A(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    A(dalloc(&h->d_ix, std::max(1, h->n_mov)));
    A(dalloc(&h->d_iy, std::max(1, h->n_mov)));
    if (!ok) {
        ap_destroy(h);
        return AP_ERR_CUDA;
    }
    A(cudaMemcpy(h->d_net_ptr, net_ptr.data(), sizeof(int) * net_ptr.size(), cudaMemcpyHostToDevice));
    if (!pin_node.empty())
        A(cudaMemcpy(h->d_pin_node, pin_node.data(), sizeof(int) * pin_node.size(), cudaMemcpyHostToDevice));
    A(cudaMemcpy(h->d_w, w.data(), sizeof(float) * N, cudaMemcpyHostToDevice));
    A(cudaMemcpy(h->d_h, hh.data(), sizeof(float) * N, cudaMemcpyHostToDevice));
    if (ok) {
        launch_size_q(N, h->d_w, h->d_h, h->d_whq, 0);
        A(cudaGetLastError());
        A(cudaStreamSynchronize(0));
    }
    for (int b = 0; b < 2; ++b) {
        A(cudaMemcpy(h->d_px[b], x.data(), sizeof(float) * N, cudaMemcpyHostToDevice));
        A(cudaMemcpy(h->d_py[b], y.data(), sizeof(float) * N, cudaMemcpyHostToDevice));
    }
    launch_interleave(N, h->d_px[0], h->d_py[0], h->d_xy_loop, 0);
    A(cudaGetLastError());
    A(cudaMemcpy(h->d_pins, pins.data(), sizeof(float) * N, cudaMemcpyHostToDevice));
    A(cudaMemcpy(h->d_charge, charge.data(), sizeof(float) * N, cudaMemcpyHostToDevice));
    A(cudaMemset(h->d_mov_q, 0, sizeof(ull) * nb));
    if (h->d_fill_q) A(cudaMemset(h->d_fill_q, 0, sizeof(ull) * nb));
    A(cudaMemset(h->d_counters, 0, sizeof(unsigned int) * 8));
    A(cudaMemset(h->d_gq, 0, sizeof(ull) * N));
    A(cudaMemset(h->d_gqx, 0, sizeof(ull) * N));
    A(cudaMemset(h->d_gqy, 0, sizeof(ull) * N));
    if (!ok) {
        ap_destroy(h);
        return AP_ERR_CUDA;
    }
    // fixed-macro map, once: the scatter kernel over fixed nodes with area
    {
        ScatterArgs s = scatter_args(h);
        s.update = 0;
        s.px = h->d_px[0];
        s.py = h->d_py[0];
        s.lo = h->n_mov;
        s.hi = h->n_mov + h->n_fixa;
        launch_scatter(s, 0);
        std::vector<long long> fq(nb), fs(nb);
        A(cudaMemcpy(fq.data(), h->d_mov_q, sizeof(long long) * nb, cudaMemcpyDeviceToHost));
        double fixed_scaled = 0.0;
        for (size_t b = 0; b < nb; ++b) {
            fs[b] = llrint((double)p.target_density * (double)fq[b]);
            fixed_scaled += (double)fs[b];
        }
        // mean of movable + scaled fixed density over the bins (the movable
        // nodes stay on the die, so their total is constant)
        h->d_shift = (float)((mov_area_q + fill_area_q + fixed_scaled) * h->inv_ab / (double)nb);
        A(cudaMemcpy(h->d_fix_q, fq.data(), sizeof(long long) * nb, cudaMemcpyHostToDevice));
        A(cudaMemcpy(h->d_fixs_q, fs.data(), sizeof(long long) * nb, cudaMemcpyHostToDevice));
        A(cudaMemset(h->d_mov_q, 0, sizeof(ull) * nb));
    }
    int r = ok ? field_solver_init(h->fs, p.bins_x, g.bh / g.bw, 1)
               : AP_ERR_CUDA;
    if (r == AP_OK && p.bins_x % 128 == 0) {
        r = field_solver_bind_bf16(h->fs, h->d_dens_hi, h->d_dens_lo);
        if (r != AP_OK && p.field_solver != AP_FIELD_BF16X3) r = AP_OK;  // tensor path optional here
    } else if (r == AP_OK && p.field_solver == AP_FIELD_BF16X3) {
        r = AP_ERR_UNSUPPORTED;  // the tcgen05 tiles need bins a multiple of 128
    }
    if (r != AP_OK) {
        ap_destroy(h);
        return r;
    }
    if (cudaDeviceSynchronize() != cudaSuccess) {
        ap_destroy(h);
        return AP_ERR_CUDA;
    }
    *out = h;
    return AP_OK;
}

int ap_destroy(ap_handle *h) {
    if (!h) return AP_ERR_INVALID_ARG;
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->log) {
        if (h->initialized) read_scalars(h);  // the trials not yet written
        fclose(h->log);
    }
    if (h->d_traj) cudaFree(h->d_traj);
    destroy_graphs(h);
    surr_state_free(h->surr_state);
    if (h->side) cudaStreamDestroy(h->side);
    if (h->wa_stream) cudaStreamDestroy(h->wa_stream);
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
    if (h->ev_upd) cudaEventDestroy(h->ev_upd);
    if (h->ev_copy) cudaEventDestroy(h->ev_copy);
    if (h->copy_in) cudaStreamDestroy(h->copy_in);
    if (h->ev_start) cudaEventDestroy(h->ev_start);
    for (cudaEvent_t e : h->ev_in)
        if (e) cudaEventDestroy(e);
    field_solver_free(h->fs);
    void *ptrs[] = {h->d_net_ptr, h->d_pin_node, h->d_w,      h->d_h,       h->d_px[0], h->d_px[1],
                    h->d_py[0],   h->d_py[1],    h->d_gx[0],  h->d_gx[1],   h->d_gy[0], h->d_gy[1],
                    h->d_ux[0],   h->d_uy[0],    h->d_ux[1],  h->d_uy[1],
                    h->d_pins,    h->d_charge,   h->d_gqx,    h->d_gqy,
                    h->d_mov_q,   h->d_fill_q,   h->d_fix_q,  h->d_fixs_q,  h->d_dens,  h->d_ex,    h->d_ey,
                    h->d_dens_hi, h->d_dens_lo,  h->d_sx,     h->d_sy,      h->d_sc,    h->d_partials,
                    h->d_partials_ll, h->d_counters, h->d_out, h->d_rec_bin, h->d_rec_ov, h->d_gq,
                    h->d_ix,      h->d_iy,       h->d_xy_loop, h->d_xy_tmp, h->d_whq};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    if (h->h_sc) cudaFreeHost(h->h_sc);
    if (h->h_out) cudaFreeHost(h->h_out);
    if (h->h_status) cudaFreeHost(h->h_status);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return AP_OK;
}

int ap_get_fillers(ap_handle *h, int32_t *count, float *width, float *height) {
    if (!h) return AP_ERR_INVALID_ARG;
    if (count) *count = h->n_fill;
    if (width) *width = h->fill_w;
    if (height) *height = h->fill_h;
    return AP_OK;
}

int ap_set_stream(ap_handle *h, void *stream) {
    if (!h) return AP_ERR_INVALID_ARG;
    CK(cudaStreamSynchronize(h->stream));
    destroy_graphs(h);
    if (h->own_stream) cudaStreamDestroy(h->stream);
    h->stream = (cudaStream_t)stream;
    h->own_stream = false;
    if (h->initialized && h->p.use_graph) return build_graphs(h);
    return AP_OK;
}

int ap_init_positions(ap_handle *h, const float *x, const float *y) {
    if (!h || !x || !y) return AP_ERR_INVALID_ARG;
    int r = upload_positions(h, 0, x, y);
    if (r != AP_OK) return r;
    return init_optimizer(h);
}

int ap_init_seeded(ap_handle *h, uint64_t seed, float sigma) {
    if (!h) return AP_ERR_INVALID_ARG;
    // splitmix64 + Box-Muller, the generator's normal draw
    std::vector<float> x((size_t)h->n_ext, 0.f), y((size_t)h->n_ext, 0.f);
    uint64_t z = seed;
    auto next = [&]() {
        z += 0x9E3779B97F4A7C15ull;
        uint64_t t = z;
        t = (t ^ (t >> 30)) * 0xBF58476D1CE4E5B9ull;
        t = (t ^ (t >> 27)) * 0x94D049BB133111EBull;
        return t ^ (t >> 31);
    };
    auto uni = [&]() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); };
    auto normal = [&]() {
        double u1 = std::max(uni(), 1e-300), u2 = uni();
        return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
    };
    const double cx = h->die_xl + 0.5 * h->die_w, cy = h->die_yl + 0.5 * h->die_h;
    for (int i = 0; i < h->n_real; ++i) {
        const int e = h->int2ext[(size_t)i];
        x[(size_t)e] = (float)(cx + sigma * normal());
        y[(size_t)e] = (float)(cy + sigma * normal());
    }
    return ap_init_positions(h, x.data(), y.data());
}

int ap_step(ap_handle *h, int32_t n_iter) {
    if (!h || n_iter < 0) return AP_ERR_INVALID_ARG;
    if (!h->initialized) return AP_ERR_STATE;
    int r = step_n(h, n_iter);
    if (r != AP_OK) return r;
    return sync(h);
}

int ap_set_log(ap_handle *h, const char *path, int32_t capacity) {
    if (!h || (path && capacity < 1)) return AP_ERR_INVALID_ARG;
    CK(cudaStreamSynchronize(h->stream));
    if (h->log) {
        if (h->initialized) {
            const int r = read_scalars(h);  // what is left of the old log
            if (r != AP_OK) return r;
        }
        fclose(h->log);
        h->log = nullptr;
    }
    if (h->d_traj) {
        CK(cudaFree(h->d_traj));
        h->d_traj = nullptr;
        h->traj_cap = 0;
    }
    if (path) {
        h->log = fopen(path, "w");
        if (!h->log) return AP_ERR_INVALID_ARG;
        if (cudaMalloc((void **)&h->d_traj, sizeof(TrajRec) * (size_t)capacity) != cudaSuccess) {
            fclose(h->log);
            h->log = nullptr;
            return AP_ERR_CUDA;
        }
        h->traj_cap = capacity;
    }
    if (!h->initialized) return AP_OK;  // init_optimizer installs the ring
    CK(cudaMemcpyAsync(h->h_sc, h->d_sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->h_sc->traj = h->d_traj;
    h->h_sc->traj_cap = h->traj_cap;
    h->log_next = h->h_sc->evals;
    h->log_t0 = 0;
    CK(cudaMemcpyAsync(h->d_sc, h->h_sc, sizeof(DevScalars), cudaMemcpyHostToDevice, h->stream));
    return sync(h);
}

int ap_solver_info(ap_handle *h, int32_t *tc_variant, float *tc_ms, int32_t *simt_tile, float *simt_ms) {
    if (!h) return AP_ERR_INVALID_ARG;
    if (tc_variant) *tc_variant = h->fs.tc_ready ? h->fs.tc_variant : -1;
    if (tc_ms)
        for (int v = 0; v < kTcCandidates; ++v) tc_ms[v] = h->fs.tc_tune_ms[v];
    if (simt_tile) *simt_tile = h->fs.simt_bm;
    if (simt_ms) {
        simt_ms[0] = h->fs.simt_tune_ms[0];
        simt_ms[1] = h->fs.simt_tune_ms[1];
    }
    return AP_OK;
}

int ap_step_async(ap_handle *h, int32_t n_trials) {
    if (!h || n_trials < 0) return AP_ERR_INVALID_ARG;
    if (!h->initialized) return AP_ERR_STATE;
    return launch_trials(h, n_trials);
}

int ap_profile_stages(ap_handle *h, int32_t n_trials, float *stage_ms, int32_t *n_stages) {
    if (!h || n_trials <= 0 || !stage_ms || !n_stages) return AP_ERR_INVALID_ARG;
    if (!h->initialized) return AP_ERR_STATE;
    constexpr int S = 5;
    cudaEvent_t ev[S + 1];
    for (int i = 0; i <= S; ++i) CK(cudaEventCreate(&ev[i]));
    double acc[S] = {0, 0, 0, 0, 0};
    cudaStream_t st = h->stream;
    int r = AP_OK;
    for (int t = 0; t < n_trials && r == AP_OK; ++t) {
        CK(cudaEventRecord(ev[0], st));
        launch_update(loop_scatter_args(h), st);
        launch_movable_bins(h, loop_scatter_args(h), st);
        CK(cudaEventRecord(ev[1], st));
        launch_rho(rho_args(h, RHO_LOOP, nullptr), st);
        CK(cudaEventRecord(ev[2], st));
        launch_wirelength(wa_args(h, h->d_px[0], h->d_py[0], 0.f, h->n_mov, WA_LOOP, nullptr), st);
        CK(cudaEventRecord(ev[3], st));
        r = run_field(h, h->p.field_solver, st);
        CK(cudaEventRecord(ev[4], st));
        launch_gather(loop_gather_args(h), st);
        CK(cudaEventRecord(ev[5], st));
        CK(cudaEventSynchronize(ev[5]));
        for (int i = 0; i < S; ++i) {
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, ev[i], ev[i + 1]));
            acc[i] += ms;
        }
    }
    for (int i = 0; i <= S; ++i) cudaEventDestroy(ev[i]);
    if (r != AP_OK) return r;
    CK(cudaGetLastError());
    for (int i = 0; i < S; ++i) stage_ms[i] = (float)(acc[i] / n_trials);
    *n_stages = S;
    return AP_OK;
}

int ap_run(ap_handle *h, int32_t *iterations_done) {
    if (!h) return AP_ERR_INVALID_ARG;
    if (!h->initialized) return AP_ERR_STATE;
    const int chunk = std::max(1, h->p.check_interval);
    int r = read_scalars(h);
    if (r != AP_OK) return r;
    const int start = h->h_sc->iteration;
    int done = 0;
    while (done < h->p.max_iterations) {
        const int n = std::min(chunk, h->p.max_iterations - done);
        r = step_n(h, n);  // leaves fresh scalars in h_sc
        done = h->h_sc->iteration - start;
        if (r != AP_OK) {
            if (iterations_done) *iterations_done = done;
            return r;
        }
        if (h->h_sc->tau < h->p.target_overflow) break;
    }
    if (iterations_done) *iterations_done = done;
    return AP_OK;
}

int ap_get_positions(ap_handle *h, float *x, float *y) {
    if (!h || !x || !y) return AP_ERR_INVALID_ARG;
    int r = read_scalars(h);
    if (r != AP_OK) return r;
    const int cur = h->h_sc->cur;
    std::vector<float> ix((size_t)h->n_nodes), iy((size_t)h->n_nodes);
    CK(cudaMemcpyAsync(ix.data(), h->d_px[cur], sizeof(float) * h->n_nodes, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(iy.data(), h->d_py[cur], sizeof(float) * h->n_nodes, cudaMemcpyDeviceToHost, h->stream));
    r = sync(h);
    if (r != AP_OK) return r;
    for (int i = 0; i < h->n_nodes; ++i) {
        const int e = h->int2ext[(size_t)i];
        if (e < 0) continue;  // filler cells are internal
        x[e] = ix[(size_t)i] + h->die_xl;
        y[e] = iy[(size_t)i] + h->die_yl;
    }
    return AP_OK;
}

int ap_step_host(ap_handle *h, const float *x_in, const float *y_in, float *x_out, float *y_out,
                 ap_stats *stats) {
    if (!h) return AP_ERR_INVALID_ARG;
    if (!h->initialized) return AP_ERR_STATE;
    const bool direct = h->identity && h->die_xl == 0.f && h->die_yl == 0.f;
    if (direct && h->p.max_backtracks == 0) {
        // Without backtracking every trial is accepted: one trial is the
        // iteration, and positions move through the staging arrays by device
        // kernels that read `cur` themselves -- one host round trip per call.
        if (x_out && y_out && !h->surr) {
            // The accepted point is the trial point (no backtracking).  The
            // input arrives in chunks, each chunk's position update starting
            // once its copy has landed; the update writes the trial point to
            // the staging arrays, whose copy back runs beside the rest of the
            // trial.  Launched eagerly: the host pointers change every call.
            cudaStream_t st = h->stream;
            const bool in = x_in && y_in;
            const int nc = in && h->n_mov >= 65536 ? 4 : 1;
            if (in) {
                CK(cudaEventRecord(h->ev_start, st));  // after the stream's earlier work
                CK(cudaStreamWaitEvent(h->copy_in, h->ev_start, 0));
            }
            if (h->n_nodes > h->n_mov) {  // fixed nodes' positions into the staging arrays
                const int nf = h->n_nodes - h->n_mov, blocks = std::min((nf + kThreads - 1) / kThreads, 4096);
                stage_in_kernel<<<blocks, kThreads, 0, st>>>(nf, h->n_mov, h->d_sc, h->d_px[0], h->d_py[0],
                                                             h->d_px[1], h->d_py[1], h->d_sx, h->d_sy);
            }
            ScatterArgs sa = loop_scatter_args(h);
            sa.trial_x = h->d_sx;
            sa.trial_y = h->d_sy;
            if (in) {
                sa.in_x = h->d_ix;
                sa.in_y = h->d_iy;
            }
            // chunk k's update runs while chunk k + 1 is copied; only the last
            // chunk's update runs after the whole input has landed, so the
            // chunks shrink: 40, 30, 20, 10% of the nodes (tenths)
            static const int kCut[5] = {0, 4, 7, 9, 10};
            int base = 0;
            for (int k = 0; k < nc; ++k) {
                const int lo = nc == 4 ? (int)((long long)h->n_mov * kCut[k] / 10) : 0;
                const int hi = nc == 4 ? (int)((long long)h->n_mov * kCut[k + 1] / 10) : h->n_mov;
                if (in) {
                    const size_t b = sizeof(float) * (size_t)(hi - lo);
                    CK(cudaMemcpyAsync(h->d_ix + lo, x_in + lo, b, cudaMemcpyHostToDevice, h->copy_in));
                    CK(cudaMemcpyAsync(h->d_iy + lo, y_in + lo, b, cudaMemcpyHostToDevice, h->copy_in));
                    CK(cudaEventRecord(h->ev_in[k], h->copy_in));
                    CK(cudaStreamWaitEvent(st, h->ev_in[k], 0));
                }
                sa.upd_lo = lo;
                sa.upd_hi = hi;  // chunks are non-empty: nc > 1 only for n_mov >= 65536
                sa.part_base = base;
                sa.no_fold = k < nc - 1;
                base += launch_update(sa, st);
            }
            CK(cudaEventRecord(h->ev_upd, st));
            int r = enqueue_after_update(h, st);
            if (r != AP_OK) return r;
            CK(cudaStreamWaitEvent(h->copy_stream, h->ev_upd, 0));
            CK(cudaMemcpyAsync(x_out, h->d_sx, sizeof(float) * h->n_nodes, cudaMemcpyDeviceToHost, h->copy_stream));
            CK(cudaMemcpyAsync(y_out, h->d_sy, sizeof(float) * h->n_nodes, cudaMemcpyDeviceToHost, h->copy_stream));
            CK(cudaEventRecord(h->ev_copy, h->copy_stream));
            CK(cudaStreamWaitEvent(h->stream, h->ev_copy, 0));
            CK(cudaGetLastError());
            r = read_scalars(h);
            if (r != AP_OK) return r;
            if (stats) fill_stats(h, stats);
            return h->h_sc->status;
        }
        if (x_in && y_in) {
            CK(cudaMemcpyAsync(h->d_sx, x_in, sizeof(float) * h->n_mov, cudaMemcpyHostToDevice, h->stream));
            CK(cudaMemcpyAsync(h->d_sy, y_in, sizeof(float) * h->n_mov, cudaMemcpyHostToDevice, h->stream));
            stage_cur(h, h->n_mov, 1);
        }
        int r = launch_trials(h, 1);
        if (r != AP_OK) return r;
        if (x_out && y_out) {
            stage_cur(h, h->n_nodes, 0);
            CK(cudaMemcpyAsync(x_out, h->d_sx, sizeof(float) * h->n_nodes, cudaMemcpyDeviceToHost, h->stream));
            CK(cudaMemcpyAsync(y_out, h->d_sy, sizeof(float) * h->n_nodes, cudaMemcpyDeviceToHost, h->stream));
        }
        CK(cudaGetLastError());
        r = read_scalars(h);
        if (r != AP_OK) return r;
        if (stats) fill_stats(h, stats);
        return h->h_sc->status;
    }
    int r = read_scalars(h);
    if (r != AP_OK) return r;
    if (x_in && y_in) {
        const int cur = h->h_sc->cur;
        if (direct) {
            CK(cudaMemcpyAsync(h->d_px[cur], x_in, sizeof(float) * h->n_mov, cudaMemcpyHostToDevice, h->stream));
            CK(cudaMemcpyAsync(h->d_py[cur], y_in, sizeof(float) * h->n_mov, cudaMemcpyHostToDevice, h->stream));
        } else {
            r = upload_positions(h, cur, x_in, y_in);
            if (r != AP_OK) return r;
        }
    }
    r = step_n(h, 1);
    if (r != AP_OK) return r;
    if (x_out && y_out) {
        if (direct) {
            const int cur = h->h_sc->cur;
            CK(cudaMemcpyAsync(x_out, h->d_px[cur], sizeof(float) * h->n_nodes, cudaMemcpyDeviceToHost, h->stream));
            CK(cudaMemcpyAsync(y_out, h->d_py[cur], sizeof(float) * h->n_nodes, cudaMemcpyDeviceToHost, h->stream));
            r = sync(h);
        } else {
            r = ap_get_positions(h, x_out, y_out);
        }
        if (r != AP_OK) return r;
    }
    if (stats) fill_stats(h, stats);
    return h->h_sc->status;
}

int ap_get_stats(ap_handle *h, ap_stats *s) {
    if (!h || !s) return AP_ERR_INVALID_ARG;
    int r = read_scalars(h);
    if (r != AP_OK) return r;
    fill_stats(h, s);
    return AP_OK;
}

int ap_hpwl(ap_handle *h, double *hpwl) {
    if (!h || !hpwl) return AP_ERR_INVALID_ARG;
    if (!h->initialized) return AP_ERR_STATE;
    int r = read_scalars(h);
    if (r != AP_OK) return r;
    *hpwl = h->h_sc->hpwl;
    return AP_OK;
}

int ap_overflow(ap_handle *h, double *overflow, double *overflow_abs) {
    if (!h || !overflow) return AP_ERR_INVALID_ARG;
    if (!h->initialized) return AP_ERR_STATE;
    int r = read_scalars(h);
    if (r != AP_OK) return r;
    *overflow = h->h_sc->tau;
    if (overflow_abs) *overflow_abs = h->h_sc->tau_abs;
    return AP_OK;
}

// ---- per-stage entry points ----------------------------------------------

namespace {
// external-order positions of all nodes -> internal scratch (d_sx, d_sy)
int stage_positions(ap_handle *h, const float *x, const float *y) {
    std::vector<float> ix((size_t)h->n_nodes), iy((size_t)h->n_nodes);
    for (int i = 0; i < h->n_nodes; ++i) {
        const int e = h->int2ext[(size_t)i];
        if (e < 0) {  // filler cells: their starting points (no per-stage result depends on them)
            ix[(size_t)i] = h->fill_x0[(size_t)(i - h->n_real)];
            iy[(size_t)i] = h->fill_y0[(size_t)(i - h->n_real)];
            continue;
        }
        ix[(size_t)i] = x[e] - h->die_xl;
        iy[(size_t)i] = y[e] - h->die_yl;
        if (!std::isfinite(ix[(size_t)i]) || !std::isfinite(iy[(size_t)i])) return AP_ERR_NONFINITE;
    }
    CK(cudaMemcpyAsync(h->d_sx, ix.data(), sizeof(float) * h->n_nodes, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->d_sy, iy.data(), sizeof(float) * h->n_nodes, cudaMemcpyHostToDevice, h->stream));
    return sync(h);
}
}  // namespace

int ap_wirelength_grad(ap_handle *h, const float *x, const float *y, float gamma, float *gx, float *gy,
                       double *wa, double *hpwl) {
    if (!h || !x || !y || !gx || !gy || !(gamma > 0.f)) return AP_ERR_INVALID_ARG;
    int r = stage_positions(h, x, y);
    if (r != AP_OK) return r;
    const size_t N = (size_t)h->n_nodes;
    CK(cudaMemsetAsync(h->d_gq, 0, sizeof(ull) * N, h->stream));
    CK(cudaMemsetAsync(h->d_gqx, 0, sizeof(ull) * N, h->stream));
    CK(cudaMemsetAsync(h->d_gqy, 0, sizeof(ull) * N, h->stream));
    launch_wirelength(wa_args(h, h->d_sx, h->d_sy, gamma, h->n_nodes, WA_OUT_ONLY, h->d_out), h->stream);
    CK(cudaGetLastError());
    std::vector<unsigned long long> q(N), qx(N), qy(N);
    CK(cudaMemcpyAsync(q.data(), h->d_gq, sizeof(ull) * N, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(qx.data(), h->d_gqx, sizeof(ull) * N, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(qy.data(), h->d_gqy, sizeof(ull) * N, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(h->h_out, h->d_out, sizeof(double) * 2, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemsetAsync(h->d_gq, 0, sizeof(ull) * N, h->stream));
    CK(cudaMemsetAsync(h->d_gqx, 0, sizeof(ull) * N, h->stream));
    CK(cudaMemsetAsync(h->d_gqy, 0, sizeof(ull) * N, h->stream));
    r = sync(h);
    if (r != AP_OK) return r;
    for (size_t i = 0; i < N; ++i) {
        // packed halves (y 2^32 + x, x the signed low word) plus the per-axis sums
        const long long lo = (long long)(int32_t)(uint32_t)q[i];
        const long long sx = lo + (long long)qx[i];
        const long long sy = (((long long)q[i] - lo) >> 32) + (long long)qy[i];
        const int e = h->int2ext[i];
        if (e < 0) continue;
        gx[e] = (float)ldexp((double)sx, -20);  // kGradScale = 2^20
        gy[e] = (float)ldexp((double)sy, -20);
    }
    if (hpwl) *hpwl = h->h_out[0];
    if (wa) *wa = h->h_out[1];
    return AP_OK;
}

int ap_density_map(ap_handle *h, const float *x, const float *y, int64_t *rho_q) {
    if (!h || !x || !y || !rho_q) return AP_ERR_INVALID_ARG;
    int r = stage_positions(h, x, y);
    if (r != AP_OK) return r;
    const size_t nb = (size_t)h->p.bins_x * h->p.bins_y;
    CK(cudaMemsetAsync(h->d_mov_q, 0, sizeof(ull) * nb, h->stream));
    // the netlist's nodes: real movable cells and fixed nodes with area
    ScatterArgs s = scatter_args(h);
    s.update = 0;
    s.px = h->d_sx;
    s.py = h->d_sy;
    s.lo = 0;
    s.hi = h->n_real;
    launch_scatter(s, h->stream);
    s.lo = h->n_mov;
    s.hi = h->n_mov + h->n_fixa;
    launch_scatter(s, h->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(rho_q, h->d_mov_q, sizeof(long long) * nb, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemsetAsync(h->d_mov_q, 0, sizeof(ull) * nb, h->stream));
    return sync(h);
}

int ap_field_solve(ap_handle *h, const float *density, float *ex, float *ey, int32_t solver) {
    if (!h || !density || !ex || !ey) return AP_ERR_INVALID_ARG;
    const int sv = solver_of(h, solver);
    if (sv != AP_FIELD_FP32 && sv != AP_FIELD_BF16X3) return AP_ERR_INVALID_ARG;
    const int nb = h->p.bins_x * h->p.bins_y;
    if (sv == AP_FIELD_BF16X3 && !h->fs.tc_ready) return AP_ERR_UNSUPPORTED;
    // the field does not depend on the map's mean (phi_00 = 0); taking it off
    // keeps the transforms' DC sums from swamping the AC terms in rounding
    double mean = 0.0;
    for (int b = 0; b < nb; ++b) mean += (double)density[b];
    mean /= (double)nb;
    std::vector<float> shifted((size_t)nb);
    for (int b = 0; b < nb; ++b) shifted[(size_t)b] = density[b] - (float)mean;
    CK(cudaMemcpyAsync(h->d_dens, shifted.data(), sizeof(float) * nb, cudaMemcpyHostToDevice, h->stream));
    if (sv == AP_FIELD_BF16X3) launch_split_bf16(nb, h->d_dens, h->d_dens_hi, h->d_dens_lo, h->stream);
    int r = run_field(h, sv, h->stream);
    if (r != AP_OK) return r;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(ex, h->d_ex, sizeof(float) * nb, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(ey, h->d_ey, sizeof(float) * nb, cudaMemcpyDeviceToHost, h->stream));
    return sync(h);
}

int ap_node_force(ap_handle *h, const float *x, const float *y, const float *ex, const float *ey, float gamma,
                  float lambda, float *fx, float *fy, float *gx, float *gy) {
    if (!h || !x || !y || !ex || !ey || !fx || !fy || (!gx) != (!gy)) return AP_ERR_INVALID_ARG;
    const bool grad = gx != nullptr;
    if (grad && (!(gamma > 0.f) || !(lambda >= 0.f) || !std::isfinite(lambda))) return AP_ERR_INVALID_ARG;
    int r = stage_positions(h, x, y);
    if (r != AP_OK) return r;
    const size_t nb = (size_t)h->p.bins_x * h->p.bins_y, N = (size_t)h->n_nodes, M = (size_t)h->n_mov;
    CK(cudaMemcpyAsync(h->d_ex, ex, sizeof(float) * nb, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->d_ey, ey, sizeof(float) * nb, cudaMemcpyHostToDevice, h->stream));
    // the bin records of this point, as a loop trial's position update makes
    // them, so that the gather below runs the loop's record path
    launch_records(h->g, h->n_mov, h->d_sx, h->d_sy, h->d_w, h->d_h, h->d_rec_bin, h->d_rec_ov, h->stream);
    float *d_g = nullptr;
    if (grad) {
        CK(cudaMallocAsync((void **)&d_g, sizeof(float) * 2 * std::max<size_t>(M, 1), h->stream));
        CK(cudaMemsetAsync(h->d_gq, 0, sizeof(ull) * N, h->stream));
        CK(cudaMemsetAsync(h->d_gqx, 0, sizeof(ull) * N, h->stream));
        CK(cudaMemsetAsync(h->d_gqy, 0, sizeof(ull) * N, h->stream));
        launch_wirelength(wa_args(h, h->d_sx, h->d_sy, gamma, h->n_mov, WA_OUT_ONLY, h->d_out), h->stream);
    }
    GatherArgs a = gather_args(h, 0, GATHER_NODE_OUT);
    a.vx[0] = a.vx[1] = h->d_sx;
    a.vy[0] = a.vy[1] = h->d_sy;
    a.rec_bin = h->d_rec_bin;
    a.rec_ov = h->d_rec_ov;
    a.fx = h->d_ix;  // host-step input staging, n_mov floats each
    a.fy = h->d_iy;
    a.lambda = lambda;
    a.gxo = grad ? d_g : nullptr;
    a.gyo = grad ? d_g + M : nullptr;
    launch_gather(a, h->stream);
    const cudaError_t le = cudaGetLastError();
    std::vector<float> hf(2 * std::max<size_t>(M, 1)), hg(grad ? 2 * std::max<size_t>(M, 1) : 0);
    cudaError_t ce = cudaSuccess;
    if (M) {
        if (ce == cudaSuccess) ce = cudaMemcpyAsync(hf.data(), h->d_ix, sizeof(float) * M, cudaMemcpyDeviceToHost, h->stream);
        if (ce == cudaSuccess) ce = cudaMemcpyAsync(hf.data() + M, h->d_iy, sizeof(float) * M, cudaMemcpyDeviceToHost, h->stream);
        if (grad && ce == cudaSuccess)
            ce = cudaMemcpyAsync(hg.data(), d_g, sizeof(float) * 2 * M, cudaMemcpyDeviceToHost, h->stream);
    }
    if (d_g) cudaFreeAsync(d_g, h->stream);
    CK(le);
    CK(ce);
    r = sync(h);
    if (r != AP_OK) return r;
    for (size_t i = 0; i < N; ++i) {
        const int e = h->int2ext[i];
        if (e < 0) continue;
        const bool mov = i < M;
        fx[e] = mov ? hf[i] : 0.f;
        fy[e] = mov ? hf[M + i] : 0.f;
        if (grad) {
            gx[e] = mov ? hg[i] : 0.f;
            gy[e] = mov ? hg[M + i] : 0.f;
        }
    }
    return AP_OK;
}

int ap_debug_inject(ap_handle *h, int32_t kind, int64_t wait_ns) {
    if (!h) return AP_ERR_INVALID_ARG;
    if (kind != AP_FAULT_NONE && kind != AP_FAULT_TC_STALL) return AP_ERR_INVALID_ARG;
    if (kind == AP_FAULT_TC_STALL && (wait_ns < 1000000 || wait_ns > 2000000000)) return AP_ERR_INVALID_ARG;
    if (kind == AP_FAULT_TC_STALL && !h->fs.tc_ready) return AP_ERR_UNSUPPORTED;
    // nothing of this handle may be in flight while the solver changes
    CK(cudaStreamSynchronize(h->stream));
    if (h->wa_stream) CK(cudaStreamSynchronize(h->wa_stream));
    h->fs.fault_stall = kind == AP_FAULT_TC_STALL;
    h->fs.fault_wait_ns = kind == AP_FAULT_TC_STALL ? (unsigned long long)wait_ns : 0ull;
    if (kind == AP_FAULT_NONE) {
        const int r = field_solver_clear_status(h->fs);
        if (r != AP_OK) return r;
    }
    // the trial graph holds the solver's launch parameters
    const bool rebuild = h->graph_ok;
    destroy_graphs(h);
    if (rebuild && h->initialized && h->p.use_graph) return build_graphs(h);
    return AP_OK;
}

// ---- snapshots ------------------------------------------------------------
// layout: magic, n_nodes, n_mov, 0, DevScalars, px[2][N], py[2][N], ux[2], uy[2], gx[2], gy[2]

static size_t snap_bytes(const ap_handle *h) {
    return 4 * sizeof(int32_t) + sizeof(DevScalars) + sizeof(float) * (4 * (size_t)h->n_nodes + 8 * (size_t)h->n_mov);
}

int ap_snapshot_size(ap_handle *h, size_t *bytes) {
    if (!h || !bytes) return AP_ERR_INVALID_ARG;
    *bytes = snap_bytes(h);
    return AP_OK;
}

int ap_snapshot(ap_handle *h, void *buf, size_t bytes) {
    if (!h || !buf || bytes < snap_bytes(h)) return AP_ERR_INVALID_ARG;
    if (!h->initialized) return AP_ERR_STATE;
    CK(cudaStreamSynchronize(h->stream));
    char *p = (char *)buf;
    int32_t hdr[4] = {0x41505336, h->n_nodes, h->n_mov, 0};
    memcpy(p, hdr, sizeof(hdr));
    p += sizeof(hdr);
    CK(cudaMemcpy(p, h->d_sc, sizeof(DevScalars), cudaMemcpyDeviceToHost));
    p += sizeof(DevScalars);
    const size_t N = (size_t)h->n_nodes, M = (size_t)h->n_mov;
    float *arrs_n[4] = {h->d_px[0], h->d_px[1], h->d_py[0], h->d_py[1]};
    for (float *a : arrs_n) {
        CK(cudaMemcpy(p, a, sizeof(float) * N, cudaMemcpyDeviceToHost));
        p += sizeof(float) * N;
    }
    float *arrs_m[8] = {h->d_ux[0], h->d_ux[1], h->d_uy[0], h->d_uy[1], h->d_gx[0], h->d_gx[1], h->d_gy[0], h->d_gy[1]};
    for (float *a : arrs_m) {
        CK(cudaMemcpy(p, a, sizeof(float) * M, cudaMemcpyDeviceToHost));
        p += sizeof(float) * M;
    }
    return AP_OK;
}

int ap_restore(ap_handle *h, const void *buf, size_t bytes) {
    if (!h || !buf || bytes < snap_bytes(h)) return AP_ERR_INVALID_ARG;
    const char *p = (const char *)buf;
    int32_t hdr[4];
    memcpy(hdr, p, sizeof(hdr));
    if (hdr[0] != 0x41505336 || hdr[1] != h->n_nodes || hdr[2] != h->n_mov) return AP_ERR_INVALID_ARG;
    p += sizeof(hdr);
    CK(cudaStreamSynchronize(h->stream));
    // The optimiser state comes from the snapshot; the handle's configuration
    // (loop constants, surrogate attachment and policy) stays the handle's.
    // A snapshot taken with another surrogate attachment restarts the
    // surrogate schedule and its counters.
    DevScalars sc;
    memcpy(&sc, p, sizeof(DevScalars));
    p += sizeof(DevScalars);
    sc.max_backtracks = h->p.max_backtracks;
    sc.restart_mode = h->p.restart_mode;
    sc.mu_max = h->p.lambda_mu_max;
    sc.mu_min = h->p.lambda_mu_min;
    sc.gamma_base = h->p.gamma_base_bins;
    sc.init_density_weight = h->p.init_density_weight;
    const int attached = h->surr != nullptr;
    if (sc.surr_attached != attached) {
        sc.surr_ok = 1;
        sc.surr_used = sc.surr_judged = sc.surr_fallbacks = 0;
        sc.surr_err = 0.0;
    }
    sc.surr_attached = attached;
    sc.surr_judge_every = h->policy.judge_every;
    sc.surr_tau_min = h->policy.overflow_min;
    sc.surr_err_bound = h->policy.max_error;
    sc.field_mode = kFieldExact;
    sc.traj = h->d_traj;
    sc.traj_cap = h->traj_cap;
    h->log_next = sc.evals;  // the log goes on from the restored trial
    CK(cudaMemcpy(h->d_sc, &sc, sizeof(DevScalars), cudaMemcpyHostToDevice));
    const size_t N = (size_t)h->n_nodes, M = (size_t)h->n_mov;
    float *arrs_n[4] = {h->d_px[0], h->d_px[1], h->d_py[0], h->d_py[1]};
    for (float *a : arrs_n) {
        CK(cudaMemcpy(a, p, sizeof(float) * N, cudaMemcpyHostToDevice));
        p += sizeof(float) * N;
    }
    float *arrs_m[8] = {h->d_ux[0], h->d_ux[1], h->d_uy[0], h->d_uy[1], h->d_gx[0], h->d_gx[1], h->d_gy[0], h->d_gy[1]};
    for (float *a : arrs_m) {
        CK(cudaMemcpy(a, p, sizeof(float) * M, cudaMemcpyHostToDevice));
        p += sizeof(float) * M;
    }
    CK(cudaMemset(h->d_gq, 0, sizeof(ull) * N));
    CK(cudaMemset(h->d_gqx, 0, sizeof(ull) * N));
    CK(cudaMemset(h->d_gqy, 0, sizeof(ull) * N));
    CK(cudaMemset(h->d_mov_q, 0, sizeof(ull) * (size_t)h->p.bins_x * h->p.bins_y));
    if (h->d_fill_q) CK(cudaMemset(h->d_fill_q, 0, sizeof(ull) * (size_t)h->p.bins_x * h->p.bins_y));
    CK(cudaMemset(h->d_counters, 0, sizeof(unsigned int) * 8));
    h->initialized = true;
    if (h->p.use_graph && !h->graph_ok) return build_graphs(h);
    return AP_OK;
}


// ---- learned surrogate: attachment, sample collection, statistics ------------

namespace {
// writes the surrogate schedule fields of the device scalars (read-modify-write)
int upload_schedule(ap_handle *h) {
    int r = read_scalars(h);
    if (r != AP_OK) return r;
    DevScalars &c = *h->h_sc;
    c.surr_attached = h->surr != nullptr;
    c.surr_ok = 1;
    c.surr_judge_every = h->policy.judge_every;
    c.surr_tau_min = h->policy.overflow_min;
    c.surr_err_bound = h->policy.max_error;
    c.field_mode = kFieldExact;
    CK(cudaMemcpyAsync(h->d_sc, h->h_sc, sizeof(DevScalars), cudaMemcpyHostToDevice, h->stream));
    return sync(h);
}
}  // namespace

int ap_attach_surrogate(ap_handle *h, ap_surrogate *s, const ap_surrogate_policy *policy) {
    if (!h) return AP_ERR_INVALID_ARG;
    if (policy && (policy->judge_every < 1 || !(policy->max_error > 0.f))) return AP_ERR_INVALID_ARG;
    int r = sync(h);
    if (r != AP_OK) return r;
    destroy_graphs(h);
    surr_state_free(h->surr_state);
    h->surr = nullptr;
    if (s) {
        if (policy) h->policy = *policy;
        r = surr_state_init(h->surr_state, s->net, h->p.bins_x, h->g.bh / h->g.bw);
        if (r != AP_OK) return r;
        h->surr_state.use_net = h->policy.use_net != 0;
        h->surr = s;
    }
    if (!h->initialized) return AP_OK;
    r = upload_schedule(h);
    if (r != AP_OK) return r;
    return h->p.use_graph ? build_graphs(h) : AP_OK;
}

int ap_surrogate_get_stats(ap_handle *h, ap_surrogate_stats *st) {
    if (!h || !st) return AP_ERR_INVALID_ARG;
    int r = read_scalars(h);
    if (r != AP_OK) return r;
    st->used = h->h_sc->surr_used;
    st->judged = h->h_sc->surr_judged;
    st->fallbacks = h->h_sc->surr_fallbacks;
    st->last_error = h->h_sc->surr_err;
    return AP_OK;
}

int ap_surrogate_collect(ap_handle *h, ap_surrogate *s, int32_t n_trials, int32_t every, int32_t *collected) {
    if (!h || !s || n_trials < 0 || every < 1) return AP_ERR_INVALID_ARG;
    if (!h->initialized) return AP_ERR_STATE;
    const int M = h->p.bins_x;
    if (!s->d_X || M % s->net.f != 0 || M / s->net.f != s->R) return AP_ERR_INVALID_ARG;
    int r = sync(h);
    if (r != AP_OK) return r;
    SurrState tmp{};
    SurrState *ss = &h->surr_state;
    if (h->surr != s) {
        r = surr_state_init(tmp, s->net, M, h->g.bh / h->g.bw);
        if (r != AP_OK) return r;
        ss = &tmp;
    }
    // exact trials while collecting: the schedule is off
    ap_surrogate *attached = h->surr;
    h->surr = nullptr;
    r = upload_schedule(h);
    const bool f32 = h->p.field_solver != AP_FIELD_BF16X3;
    const size_t RR = (size_t)s->R * s->R;
    int got = 0;
    cudaStream_t st = h->stream;
    for (int t = 1; t <= n_trials && r == AP_OK; ++t) {
        launch_update(loop_scatter_args(h), st);
        launch_movable_bins(h, loop_scatter_args(h), st);
        launch_rho(rho_args(h, RHO_LOOP, nullptr), st);
        launch_wirelength(wa_args(h, h->d_px[0], h->d_py[0], 0.f, h->n_mov, WA_LOOP, nullptr), st);
        r = run_field(h, h->p.field_solver, st);
        if (r != AP_OK) break;
        if (t % every == 0 && s->n < s->cap) {
            const int slot = s->n;
            surr_enqueue_input(s->net, *ss, f32 ? h->d_dens : nullptr, f32 ? nullptr : h->d_dens_hi,
                               f32 ? nullptr : h->d_dens_lo, nullptr, 0, st);
            surr_enqueue_sample(s->net, *ss, s->d_X + (size_t)slot * s->net.cin0 * RR,
                                s->d_T + (size_t)slot * s->net.cout * RR, s->d_s + slot, s->d_e2 + slot, h->d_ex,
                                h->d_ey, st);
            s->n += 1;
            ++got;
        }
        launch_gather(loop_gather_args(h), st);
        if (cudaGetLastError() != cudaSuccess) r = AP_ERR_CUDA;
        if (r == AP_OK && t % 64 == 0) r = sync(h);
    }
    if (r == AP_OK) r = sync(h);
    h->surr = attached;
    const int r2 = upload_schedule(h);
    if (ss == &tmp) surr_state_free(tmp);
    if (collected) *collected = got;
    return r != AP_OK ? r : r2;
}

}  // extern "C"

// ---- batched form ---------------------------------------------------------------

// The persistent form's device tables, rebuilt whenever the set of active
// instances changes.  Stage records in item order; the field stage holds
// four records per instance (its contractions S1..S4), all instances' S1
// first, record k + 1 of an instance depending on its record k.
struct PersistPlan {
    int n_rec[PS_COUNT] = {};
    int chunk[PS_COUNT] = {};  // blocks per work item
    int items[PS_COUNT] = {};
    void *d_recs[PS_COUNT] = {};
    int *d_start[PS_COUNT] = {};
    int *d_nblk[PS_COUNT] = {};
    int *d_dep = nullptr;
    // queue heads and the field stage's done counters, laid out so that each
    // launch zeroes the counters of the launch before it on its stream as
    // one range: [0] gather, [1] update, [2] scatter, [3] rho, [4..7] the
    // four WA launches, [8] field, [9 ..) field done counters (the gather
    // follows the field and the WA launches)
    unsigned int *d_cnt = nullptr;
    int field_bm = 0;  // 0: each instance's own tuned tile; else 32 or 64 for all
    int item_blocks = 0;  // blocks per work item of the non-field stages; 0: the size rule
};

// Nodes per block of a batch instance's node- and net-parallel launches
// unless its parameters set them: instances of a few thousand cells would
// otherwise spend more on each block's sums and folds than on its nodes.
constexpr int kBatchBlockNodes = 2048;

struct ap_batch {
    std::vector<ap_handle *> inst;
    std::vector<char> active;
    cudaStream_t main = nullptr;
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> join;
    cudaGraphExec_t graph = nullptr;
    int form = AP_BATCH_GRAPH;
    // persistent form
    PersistPlan plan;
    cudaStream_t wa_stream = nullptr;
    cudaEvent_t wa_fork = nullptr, wa_join = nullptr;
    unsigned int *d_status = nullptr;  // a dependency wait of a persistent launch gave up
    unsigned long long wait_ns = 1000000000ull;
    int never_arrive = 0;
    int tuned_bm = 0;                  // the field tile the batch autotuner chose (0: not tuned)
    int item_blocks = 0;               // blocks per work item (0: the size rule)
    float tune_ms[2] = {0.f, 0.f};     // persistent field launch with 32 / 64 tiles
};

namespace {

void batch_free_graph(ap_batch *b) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
}

void plan_free(PersistPlan &pp) {
    for (int k = 0; k < PS_COUNT; ++k) {
        if (pp.d_recs[k]) cudaFree(pp.d_recs[k]);
        if (pp.d_start[k]) cudaFree(pp.d_start[k]);
        if (pp.d_nblk[k]) cudaFree(pp.d_nblk[k]);
    }
    if (pp.d_dep) cudaFree(pp.d_dep);
    if (pp.d_cnt) cudaFree(pp.d_cnt);
    const int bm = pp.field_bm, ib = pp.item_blocks;
    pp = PersistPlan();
    pp.field_bm = bm;
    pp.item_blocks = ib;
}

// Whether the persistent form serves every instance: the FP32 field solve,
// no surrogate.
bool persist_supported(const ap_batch *b) {
    for (const ap_handle *h : b->inst)
        if (h->p.field_solver == AP_FIELD_BF16X3 || h->surr) return false;
    return true;
}

constexpr int kFieldDone = 9;  // first field done counter in PersistPlan::d_cnt

int stage_wave(int k) {
    switch (k) {
    case PS_WA2:
        return persist_wa_wave(0);
    case PS_WA4:
        return persist_wa_wave(1);
    case PS_WA8:
        return persist_wa_wave(2);
    case PS_WA:
        return persist_wa_wave(3);
    case PS_FIELD:
        return persist_field_wave();
    default:
        return persist_density_wave(k);
    }
}

// Blocks per work item of a stage: every stage but the field (whose items
// are contraction tiles waited on one by one) takes about kItemsPerBlock
// items per resident block, so that the per-item costs (queue fetch,
// argument copy, barriers) stay small against the work.
constexpr int kItemsPerBlock = 4;

int stage_chunk(const PersistPlan &pp, int k, long long blocks) {
    if (k == PS_FIELD) return 1;
    if (pp.item_blocks > 0) return pp.item_blocks;
    const long long per = (long long)kItemsPerBlock * std::max(1, stage_wave(k));
    return (int)std::max(1ll, blocks / per);
}

template <typename T>
int upload_stage(PersistPlan &pp, int k, const std::vector<T> &recs, const std::vector<int> &blocks) {
    long long total = 0;
    for (int b : blocks) total += b;
    const int chunk = stage_chunk(pp, k, total);
    std::vector<int> start(blocks.size() + 1, 0);
    for (size_t r = 0; r < blocks.size(); ++r) start[r + 1] = start[r] + (blocks[r] + chunk - 1) / chunk;
    pp.n_rec[k] = (int)recs.size();
    pp.chunk[k] = chunk;
    pp.items[k] = start.back();
    CK(dalloc(reinterpret_cast<T **>(&pp.d_recs[k]), recs.size()));
    CK(dalloc(&pp.d_start[k], start.size()));
    CK(dalloc(&pp.d_nblk[k], blocks.size()));
    if (!recs.empty()) {
        CK(cudaMemcpy(pp.d_recs[k], recs.data(), sizeof(T) * recs.size(), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(pp.d_nblk[k], blocks.data(), sizeof(int) * blocks.size(), cudaMemcpyHostToDevice));
    }
    CK(cudaMemcpy(pp.d_start[k], start.data(), sizeof(int) * start.size(), cudaMemcpyHostToDevice));
    return AP_OK;
}

// Records of every active instance, each stage as the instance's own
// launches would run it (enqueue_iteration).
int plan_build(ap_batch *b, PersistPlan &pp) {
    plan_free(pp);
    std::vector<ScatterArgs> upd, sct;
    std::vector<RhoArgs> rho;
    std::vector<WaArgs> wa;
    std::vector<GatherArgs> gat;
    std::vector<int> bu, bs, br, bg, bw[4];
    std::vector<FieldRec> fld[4];
    for (size_t i = 0; i < b->inst.size(); ++i) {
        if (!b->active[i]) continue;
        ap_handle *h = b->inst[i];
        if (h->n_mov <= 0) return AP_ERR_UNSUPPORTED;
        const ScatterArgs sa = loop_scatter_args(h);
        upd.push_back(sa);
        bu.push_back(update_grid(sa));
        ScatterArgs s = sa;  // launch_movable_bins: real cells, then fillers
        s.lo = 0;
        s.hi = h->n_real;
        s.rho_q = h->d_mov_q;
        if (s.hi > s.lo) {
            bs.push_back(scatter_grid(s.hi - s.lo, s.block_nodes));
            s.tile32 = tile32_exact(s.g, s.hi - s.lo, bs.back()) ? 1 : 0;
            sct.push_back(s);
        }
        if (h->n_fill) {
            s.lo = h->n_real;
            s.hi = h->n_mov;
            s.rho_q = h->d_fill_q;
            bs.push_back(scatter_grid(s.hi - s.lo, s.block_nodes));
            s.tile32 = tile32_exact(s.g, s.hi - s.lo, bs.back()) ? 1 : 0;
            sct.push_back(s);
        }
        const RhoArgs ra = rho_args(h, RHO_LOOP, nullptr);
        rho.push_back(ra);
        br.push_back(rho_grid(ra.nbins));
        WaArgs wr = wa_args(h, h->d_px[0], h->d_py[0], 0.f, h->n_mov, WA_LOOP, nullptr);
        const int all = wa_plan(wr);
        for (int k = 0; k < 3; ++k) bw[k].push_back(wr.bucket_blocks[k]);
        bw[3].push_back(all - wr.small_blocks);
        wa.push_back(wr);
        FieldRec fr[4];
        field_records(h->fs, h->d_dens, h->d_ex, h->d_ey, fr);
        for (int k = 0; k < 4; ++k) {
            if (pp.field_bm == 64 && fr[k].m % 64 == 0) fr[k].bm = 64;
            if (pp.field_bm == 32) fr[k].bm = 32;
            fld[k].push_back(fr[k]);
        }
        gat.push_back(loop_gather_args(h));
        bg.push_back(gather_grid(h->n_mov, h->p.block_nodes));
    }
    const int ni = (int)upd.size();
    if (4 * ni > kPersistMaxRecords || (int)sct.size() > kPersistMaxRecords) return AP_ERR_UNSUPPORTED;
    std::vector<FieldRec> fall;
    std::vector<int> bf, dep;
    for (int k = 0; k < 4; ++k)
        for (int i = 0; i < ni; ++i) {
            fall.push_back(fld[k][i]);
            bf.push_back(field_rec_blocks(fld[k][i]));
            dep.push_back(k == 0 ? -1 : (k - 1) * ni + i);
        }
    int r = upload_stage(pp, PS_UPDATE, upd, bu);
    if (r == AP_OK) r = upload_stage(pp, PS_SCATTER, sct, bs);
    if (r == AP_OK) r = upload_stage(pp, PS_RHO, rho, br);
    if (r == AP_OK) r = upload_stage(pp, PS_WA2, wa, bw[0]);
    if (r == AP_OK) r = upload_stage(pp, PS_WA4, wa, bw[1]);
    if (r == AP_OK) r = upload_stage(pp, PS_WA8, wa, bw[2]);
    if (r == AP_OK) r = upload_stage(pp, PS_WA, wa, bw[3]);
    if (r == AP_OK) r = upload_stage(pp, PS_FIELD, fall, bf);
    if (r == AP_OK) r = upload_stage(pp, PS_GATHER, gat, bg);
    if (r != AP_OK) return r;
    CK(dalloc(&pp.d_dep, dep.size()));
    CK(cudaMemcpy(pp.d_dep, dep.data(), sizeof(int) * dep.size(), cudaMemcpyHostToDevice));
    CK(dalloc(&pp.d_cnt, kFieldDone + dep.size()));
    CK(cudaMemset(pp.d_cnt, 0, sizeof(unsigned int) * (kFieldDone + dep.size())));
    return AP_OK;
}

PersistQueue plan_queue(const ap_batch *b, int k, int reset_lo, int reset_n) {
    const PersistPlan &pp = b->plan;
    PersistQueue q{};
    q.start = pp.d_start[k];
    q.nblk = pp.d_nblk[k];
    q.n_rec = pp.n_rec[k];
    q.chunk = pp.chunk[k];
    // PS_* -> counter slot (PersistPlan::d_cnt)
    static const int head_slot[PS_COUNT] = {1, 2, 3, 7, 8, 0, 4, 5, 6};
    q.head = pp.d_cnt + head_slot[k];
    q.status = b->d_status;
    q.wait_ns = b->wait_ns;
    q.reset = pp.d_cnt + reset_lo;
    q.n_reset = reset_n;
    if (k == PS_FIELD) {
        q.dep = pp.d_dep;
        q.done = pp.d_cnt + kFieldDone;
        q.never_arrive = b->never_arrive;
    }
    return q;
}

// Synchronises the batch stream; AP_ERR_TIMEOUT once a persistent wait gave up.
int batch_sync(ap_batch *b) {
    CK(cudaStreamSynchronize(b->main));
    if (b->d_status) {
        unsigned int st = 0;
        CK(cudaMemcpy(&st, b->d_status, sizeof(st), cudaMemcpyDeviceToHost));
        if (st) return AP_ERR_TIMEOUT;
    }
    return AP_OK;
}

// The four WA launches of a trial (stream `st`): the thread-per-net buckets,
// then the larger nets, whose records fold the sums.
void enqueue_persist_wa(ap_batch *b, cudaStream_t st) {
    const PersistPlan &pp = b->plan;
    const int stage[4] = {PS_WA2, PS_WA4, PS_WA8, PS_WA};
    for (int k = 0; k < 4; ++k)
        launch_persist_wa(k, plan_queue(b, stage[k], 0, 0), static_cast<const WaArgs *>(pp.d_recs[stage[k]]), st);
}

// The gather zeroes the counters of the field and the WA launches.
int gather_reset_n(const PersistPlan &pp) { return kFieldDone - 4 + pp.n_rec[PS_FIELD]; }

// One trial step of every active instance as nine persistent launches: the
// position update; the four WA launches on a second stream beside scatter ->
// density/overflow -> field; the gather with each instance's accept / retry.
int enqueue_persist(ap_batch *b, cudaStream_t st) {
    const PersistPlan &pp = b->plan;
    launch_persist_density(PS_UPDATE, plan_queue(b, PS_UPDATE, 0, 1), pp.d_recs[PS_UPDATE], st);
    CK(cudaEventRecord(b->wa_fork, st));
    CK(cudaStreamWaitEvent(b->wa_stream, b->wa_fork, 0));
    enqueue_persist_wa(b, b->wa_stream);
    CK(cudaEventRecord(b->wa_join, b->wa_stream));
    launch_persist_density(PS_SCATTER, plan_queue(b, PS_SCATTER, 1, 1), pp.d_recs[PS_SCATTER], st);
    launch_persist_density(PS_RHO, plan_queue(b, PS_RHO, 2, 1), pp.d_recs[PS_RHO], st);
    launch_persist_field(plan_queue(b, PS_FIELD, 3, 1), static_cast<const FieldRec *>(pp.d_recs[PS_FIELD]), st);
    CK(cudaStreamWaitEvent(st, b->wa_join, 0));
    launch_persist_density(PS_GATHER, plan_queue(b, PS_GATHER, 4, gather_reset_n(pp)), pp.d_recs[PS_GATHER], st);
    return cudaGetLastError() == cudaSuccess ? AP_OK : AP_ERR_CUDA;
}

// n_trials trial steps of the persistent form as eager launches, the WA
// launches between the update and the scatter on the same stream, with
// events around each stage: the mean milliseconds of each (update, scatter,
// rho, WA -- its four launches --, field, gather) in ms[6].
int persist_profile(ap_batch *b, int n_trials, float *ms) {
    const PersistPlan &pp = b->plan;
    cudaEvent_t ev[7];
    for (cudaEvent_t &e : ev) CK(cudaEventCreate(&e));
    double acc[6] = {0, 0, 0, 0, 0, 0};
    int r = AP_OK;
    cudaStream_t st = b->main;
    for (int t = 0; t < n_trials && r == AP_OK; ++t) {
        CK(cudaEventRecord(ev[0], st));
        launch_persist_density(PS_UPDATE, plan_queue(b, PS_UPDATE, 0, 1), pp.d_recs[PS_UPDATE], st);
        CK(cudaEventRecord(ev[1], st));
        enqueue_persist_wa(b, st);
        CK(cudaEventRecord(ev[2], st));
        launch_persist_density(PS_SCATTER, plan_queue(b, PS_SCATTER, 1, 1), pp.d_recs[PS_SCATTER], st);
        CK(cudaEventRecord(ev[3], st));
        launch_persist_density(PS_RHO, plan_queue(b, PS_RHO, 2, 1), pp.d_recs[PS_RHO], st);
        CK(cudaEventRecord(ev[4], st));
        launch_persist_field(plan_queue(b, PS_FIELD, 3, 1), static_cast<const FieldRec *>(pp.d_recs[PS_FIELD]), st);
        CK(cudaEventRecord(ev[5], st));
        launch_persist_density(PS_GATHER, plan_queue(b, PS_GATHER, 4, gather_reset_n(pp)), pp.d_recs[PS_GATHER],
                               st);
        CK(cudaEventRecord(ev[6], st));
        r = batch_sync(b);
        // the events around each stage, in the order update, scatter, rho, WA, field, gather
        const int from[6] = {0, 2, 3, 1, 4, 5};
        for (int k = 0; k < 6 && r == AP_OK; ++k) {
            float v = 0.f;
            cudaEventElapsedTime(&v, ev[from[k]], ev[from[k] + 1]);
            acc[k] += v;
        }
    }
    for (cudaEvent_t &e : ev) cudaEventDestroy(e);
    for (int k = 0; k < 6; ++k) ms[k] = n_trials > 0 ? (float)(acc[k] / n_trials) : 0.f;
    return r;
}

// One graph: fork from the main stream to every active instance's stream,
// one trial step per instance, join back (graph form); or the six
// persistent launches over all active instances (persistent form).
int batch_build_graph(ap_batch *b) {
    batch_free_graph(b);
    if (b->form == AP_BATCH_PERSISTENT) {
        const int pr = plan_build(b, b->plan);
        if (pr != AP_OK) return pr;
    }
    cudaGraph_t gr = nullptr;
    CK(cudaStreamBeginCapture(b->main, cudaStreamCaptureModeThreadLocal));
    int r = AP_OK;
    if (b->form == AP_BATCH_PERSISTENT) {
        r = enqueue_persist(b, b->main);
    } else {
        cudaError_t e = cudaEventRecord(b->fork, b->main);
        r = e == cudaSuccess ? AP_OK : AP_ERR_CUDA;
        for (size_t i = 0; i < b->inst.size() && r == AP_OK; ++i) {
            if (!b->active[i]) continue;
            ap_handle *h = b->inst[i];
            if (cudaStreamWaitEvent(h->stream, b->fork, 0) != cudaSuccess) r = AP_ERR_CUDA;
            if (r == AP_OK) r = enqueue_iteration(h, h->stream);
            if (r == AP_OK && cudaEventRecord(b->join[i], h->stream) != cudaSuccess) r = AP_ERR_CUDA;
            if (r == AP_OK && cudaStreamWaitEvent(b->main, b->join[i], 0) != cudaSuccess) r = AP_ERR_CUDA;
        }
    }
    const cudaError_t e = cudaStreamEndCapture(b->main, &gr);
    if (r != AP_OK || e != cudaSuccess) {
        if (gr) cudaGraphDestroy(gr);
        return r != AP_OK ? r : AP_ERR_CUDA;
    }
    const cudaError_t ei = cudaGraphInstantiate(&b->graph, gr, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(gr);
    return ei == cudaSuccess ? AP_OK : AP_ERR_CUDA;
}

// Tile autotuner of the persistent field launch: every active instance's
// four contractions with 32 x 32 and with 64 x 64 tiles (instances whose
// grid is not a multiple of 64 keep 32), 2 warm and 5 timed launches each on
// the instances' own scratch; the faster is kept.  The tile does not change
// the results (each output sums its products in the same order).
int batch_tune_field(ap_batch *b) {
    if (b->form != AP_BATCH_PERSISTENT) return AP_OK;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    int r = AP_OK;
    const int cand[2] = {32, 64};
    for (int v = 0; v < 2 && r == AP_OK; ++v) {
        b->plan.field_bm = cand[v];
        r = plan_build(b, b->plan);
        if (r != AP_OK) break;
        const int nf = b->plan.n_rec[PS_FIELD];
        for (int t = 0; t < 7 && r == AP_OK; ++t) {
            if (t == 2 && cudaEventRecord(e0, b->main) != cudaSuccess) r = AP_ERR_CUDA;
            // zero the field counters the way the launch before it would
            if (cudaMemsetAsync(b->plan.d_cnt + kFieldDone - 1, 0, sizeof(unsigned int) * (1 + nf), b->main) !=
                cudaSuccess)
                r = AP_ERR_CUDA;
            launch_persist_field(plan_queue(b, PS_FIELD, 3, 0),
                                 static_cast<const FieldRec *>(b->plan.d_recs[PS_FIELD]), b->main);
        }
        if (r == AP_OK && (cudaEventRecord(e1, b->main) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess))
            r = AP_ERR_CUDA;
        float ms = 0.f;
        if (r == AP_OK) cudaEventElapsedTime(&ms, e0, e1);
        b->tune_ms[v] = ms / 5.f;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (r == AP_OK) r = batch_sync(b);
    b->tuned_bm = b->tune_ms[0] <= b->tune_ms[1] ? 32 : 64;
    b->plan.field_bm = b->tuned_bm;
    return r;
}

}  // namespace

extern "C" {

int ap_create_batch(int32_t n, const ap_netlist *netlists, const ap_params *params, ap_batch **out) {
    if (n <= 0 || !netlists || !params || !out) return AP_ERR_INVALID_ARG;
    *out = nullptr;
    ap_batch *b = new ap_batch();
    int r = AP_OK;
    for (int i = 0; i < n && r == AP_OK; ++i) {
        ap_params p = params[i];
        p.use_graph = 0;  // the batch graph replaces the per-instance graphs
        if (p.block_nodes <= 0) p.block_nodes = kBatchBlockNodes;
        ap_handle *h = nullptr;
        r = ap_create(&netlists[i], &p, &h);
        if (r == AP_OK) b->inst.push_back(h);
    }
    if (r == AP_OK && (cudaStreamCreateWithFlags(&b->main, cudaStreamNonBlocking) != cudaSuccess ||
                       cudaStreamCreateWithFlags(&b->wa_stream, cudaStreamNonBlocking) != cudaSuccess ||
                       cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
                       cudaEventCreateWithFlags(&b->wa_fork, cudaEventDisableTiming) != cudaSuccess ||
                       cudaEventCreateWithFlags(&b->wa_join, cudaEventDisableTiming) != cudaSuccess ||
                       dalloc(&b->d_status, 1) != cudaSuccess ||
                       cudaMemset(b->d_status, 0, sizeof(unsigned int)) != cudaSuccess))
        r = AP_ERR_CUDA;
    for (int i = 0; i < n && r == AP_OK; ++i) {
        cudaEvent_t ev;
        if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) r = AP_ERR_CUDA;
        else b->join.push_back(ev);
    }
    b->active.assign((size_t)n, 1);
    // the persistent form where it serves every instance, its field tile
    // chosen by the batch autotuner
    if (r == AP_OK && persist_supported(b)) {
        b->form = AP_BATCH_PERSISTENT;
        r = batch_tune_field(b);
    }
    if (r != AP_OK) {
        ap_batch_destroy(b);
        return r;
    }
    *out = b;
    return AP_OK;
}

int ap_batch_destroy(ap_batch *b) {
    if (!b) return AP_ERR_INVALID_ARG;
    if (b->main) cudaStreamSynchronize(b->main);
    if (b->wa_stream) cudaStreamSynchronize(b->wa_stream);
    batch_free_graph(b);
    plan_free(b->plan);
    for (ap_handle *h : b->inst) ap_destroy(h);
    for (cudaEvent_t e : b->join) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->wa_fork) cudaEventDestroy(b->wa_fork);
    if (b->wa_join) cudaEventDestroy(b->wa_join);
    if (b->d_status) cudaFree(b->d_status);
    if (b->wa_stream) cudaStreamDestroy(b->wa_stream);
    if (b->main) cudaStreamDestroy(b->main);
    delete b;
    return AP_OK;
}

int ap_batch_set_form(ap_batch *b, int32_t form) {
    if (!b || (form != AP_BATCH_GRAPH && form != AP_BATCH_PERSISTENT)) return AP_ERR_INVALID_ARG;
    if (form == AP_BATCH_PERSISTENT && !persist_supported(b)) return AP_ERR_UNSUPPORTED;
    CK(cudaStreamSynchronize(b->main));
    const bool rebuild = b->graph != nullptr;
    b->form = form;
    if (form == AP_BATCH_PERSISTENT && !b->tuned_bm) {
        const int r = batch_tune_field(b);
        if (r != AP_OK) return r;
    }
    return rebuild ? batch_build_graph(b) : AP_OK;
}

int ap_batch_get_info(ap_batch *b, ap_batch_info *info) {
    if (!b || !info) return AP_ERR_INVALID_ARG;
    memset(info, 0, sizeof(*info));
    info->form = b->form;
    info->instances = (int32_t)b->inst.size();
    int act = 0;
    for (char a : b->active) act += a ? 1 : 0;
    info->active = act;
    info->field_tile = b->tuned_bm;
    info->field_tune_ms[0] = b->tune_ms[0];
    info->field_tune_ms[1] = b->tune_ms[1];
    for (int k = 0; k < 6; ++k) {  // the WA entry: the launch of the larger nets; its items: all four launches'
        info->records[k] = b->plan.n_rec[k];
        info->item_blocks[k] = b->plan.chunk[k];
        info->items[k] = b->plan.items[k] + (k == PS_WA ? b->plan.items[PS_WA2] + b->plan.items[PS_WA4] +
                                                              b->plan.items[PS_WA8]
                                                        : 0);
    }
    return AP_OK;
}

int ap_batch_set_item_blocks(ap_batch *b, int32_t blocks) {
    if (!b || blocks < 0 || blocks > 4096) return AP_ERR_INVALID_ARG;
    CK(cudaStreamSynchronize(b->main));
    b->item_blocks = blocks;
    b->plan.item_blocks = blocks;
    return b->graph ? batch_build_graph(b) : AP_OK;
}

int ap_batch_profile(ap_batch *b, int32_t n_trials, float *stage_ms) {
    if (!b || n_trials <= 0 || !stage_ms) return AP_ERR_INVALID_ARG;
    if (b->form != AP_BATCH_PERSISTENT) return AP_ERR_UNSUPPORTED;
    if (!b->graph) return AP_ERR_STATE;
    CK(cudaStreamSynchronize(b->main));
    return persist_profile(b, n_trials, stage_ms);
}

int ap_batch_debug_inject(ap_batch *b, int32_t kind, int64_t wait_ns) {
    if (!b) return AP_ERR_INVALID_ARG;
    if (kind != AP_FAULT_NONE && kind != AP_FAULT_NEVER_ARRIVE) return AP_ERR_INVALID_ARG;
    if (kind == AP_FAULT_NEVER_ARRIVE && (wait_ns < 1000000 || wait_ns > 2000000000)) return AP_ERR_INVALID_ARG;
    if (kind == AP_FAULT_NEVER_ARRIVE && b->form != AP_BATCH_PERSISTENT) return AP_ERR_UNSUPPORTED;
    CK(cudaStreamSynchronize(b->main));
    b->never_arrive = kind == AP_FAULT_NEVER_ARRIVE;
    b->wait_ns = kind == AP_FAULT_NEVER_ARRIVE ? (unsigned long long)wait_ns : 1000000000ull;
    if (kind == AP_FAULT_NONE) CK(cudaMemset(b->d_status, 0, sizeof(unsigned int)));
    return b->graph ? batch_build_graph(b) : AP_OK;
}

int ap_batch_init_seeded(ap_batch *b, uint64_t seed, float sigma) {
    if (!b) return AP_ERR_INVALID_ARG;
    CK(cudaStreamSynchronize(b->main));
    for (size_t i = 0; i < b->inst.size(); ++i) {
        int r = ap_init_seeded(b->inst[i], seed + i, sigma);
        if (r != AP_OK) return r;
    }
    CK(cudaDeviceSynchronize());  // the instances' streams before the batch stream's first launch
    CK(cudaMemset(b->d_status, 0, sizeof(unsigned int)));
    b->active.assign(b->inst.size(), 1);
    return batch_build_graph(b);
}

int ap_batch_step(ap_batch *b, int32_t n_trials) {
    if (!b || n_trials < 0) return AP_ERR_INVALID_ARG;
    if (!b->graph) return AP_ERR_STATE;
    for (int t = 0; t < n_trials; ++t) CK(cudaGraphLaunch(b->graph, b->main));
    return batch_sync(b);
}

int ap_batch_run(ap_batch *b, int32_t *iterations) {
    if (!b) return AP_ERR_INVALID_ARG;
    if (!b->graph) return AP_ERR_STATE;
    for (;;) {
        int interval = 1;
        for (size_t i = 0; i < b->inst.size(); ++i)
            if (b->active[i]) interval = std::max(interval, b->inst[i]->p.check_interval);
        for (int t = 0; t < interval; ++t) CK(cudaGraphLaunch(b->graph, b->main));
        const int sr = batch_sync(b);
        if (sr != AP_OK) return sr;
        bool changed = false, any = false;
        for (size_t i = 0; i < b->inst.size(); ++i) {
            if (!b->active[i]) continue;
            ap_handle *h = b->inst[i];
            int r = read_scalars(h);
            if (r != AP_OK) return r;
            // a diverged instance leaves the graph; its stats report the status
            if (h->h_sc->status || h->h_sc->tau < h->p.target_overflow ||
                h->h_sc->iteration >= h->p.max_iterations) {
                b->active[i] = 0;
                changed = true;
            } else {
                any = true;
            }
        }
        if (!any) break;
        if (changed) {
            int r = batch_build_graph(b);
            if (r != AP_OK) return r;
        }
    }
    if (iterations)
        for (size_t i = 0; i < b->inst.size(); ++i) {
            int r = read_scalars(b->inst[i]);
            if (r != AP_OK) return r;
            iterations[i] = b->inst[i]->h_sc->iteration;
        }
    return AP_OK;
}

int ap_batch_get_stats(ap_batch *b, int32_t i, ap_stats *s) {
    if (!b || i < 0 || i >= (int32_t)b->inst.size()) return AP_ERR_INVALID_ARG;
    return ap_get_stats(b->inst[(size_t)i], s);
}

int ap_batch_get_positions(ap_batch *b, int32_t i, float *x, float *y) {
    if (!b || i < 0 || i >= (int32_t)b->inst.size()) return AP_ERR_INVALID_ARG;
    return ap_get_positions(b->inst[(size_t)i], x, y);
}

}  // extern "C"
