/*
 * aieplace.h -- C ABI of the GB300 ePlace global-placement library.
 *
 * One handle holds one placement instance resident on one GPU.  Every call
 * returns an int status (AP_OK == 0).  Arrays passed in are caller-owned host
 * memory and are copied; nothing keeps a pointer past the call.  A handle is
 * not re-entrant: calls on the same handle must not overlap.  Calls are
 * synchronous with respect to the host unless a stream is set with
 * ap_set_stream, in which case host-visible results are still complete when
 * the call returns (results are read back through pinned memory on that
 * stream).
 *
 * Coordinate conventions follow the reference host placer:
 *   - a node's position (x, y) is its lower-left corner and every pin of the
 *     node sits at that corner (Net.cpp:136-155 reads Node::getX/getY);
 *   - bin maps are x-major: element [bx * bins_y + by] is bin column bx, row
 *     by (Grid.h:16 m_bins[col][row], fft.cpp binDensity_[x][y]).
 *
 * Reference citations are paths inside searsm8/AIEplace.
 */
#ifndef AIEPLACE_H
#define AIEPLACE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AP_ABI_VERSION 3

/* ---- status codes ------------------------------------------------------ */
enum {
    AP_OK = 0,
    AP_ERR_INVALID_ARG = 1, /* null pointer, size out of range */
    AP_ERR_BAD_NETLIST = 2, /* malformed CSR: non-monotone net_ptr, pin index out of range */
    AP_ERR_NONFINITE = 3,   /* NaN / Inf in positions or sizes */
    AP_ERR_CUDA = 4,        /* a CUDA runtime call failed */
    AP_ERR_NO_DEVICE = 5,   /* no usable sm_103 device */
    AP_ERR_UNSUPPORTED = 6, /* configuration the selected kernels do not handle */
    AP_ERR_TIMEOUT = 7,     /* a bounded device-side wait gave up */
    AP_ERR_STATE = 8,       /* call out of order (e.g. ap_step before positions exist) */
    AP_ERR_DIVERGED = 9     /* the optimiser produced non-finite state */
};

/* ---- field solvers ----------------------------------------------------- */
enum {
    AP_FIELD_FP32 = 0,   /* dense per-axis transforms, FP32 SIMT contraction */
    AP_FIELD_BF16X3 = 1  /* dense per-axis transforms, tcgen05 BF16 x3 split, FP32 accumulate */
};

/* Netlist in CSR form.  Replaces the object graph the reference builds from
 * LEF/DEF (DataBase.cpp:351-416 add_def_* callbacks, Net.h:10-84, Node.h:31-158).
 * Nets of degree < 2 are accepted and ignored.  Nodes with fixed != 0 never
 * move; their x/y are final.  Zero-area nodes (IO pads) carry pins only. */
typedef struct ap_netlist {
    int32_t num_nodes;
    int32_t num_nets;
    int32_t num_pins;
    const int32_t *net_ptr;     /* [num_nets + 1], net_ptr[0] == 0, non-decreasing */
    const int32_t *pin_node;    /* [num_pins] node index of each pin */
    const float *node_w;        /* [num_nodes] width  (die units) */
    const float *node_h;        /* [num_nodes] height (die units) */
    const float *node_x;        /* [num_nodes] initial lower-left x */
    const float *node_y;        /* [num_nodes] initial lower-left y */
    const uint8_t *node_fixed;  /* [num_nodes] 1 = fixed; may be NULL (all movable) */
    float die_xl, die_yl, die_xh, die_yh;
} ap_netlist;

/* Placer parameters.  Key names follow host/config_aieplace.json where the
 * reference has one (bins_per_row -> bins_x/bins_y, gamma, max_iterations). */
typedef struct ap_params {
    int32_t bins_x;             /* density bins along x (power of two, 16..4096) */
    int32_t bins_y;             /* density bins along y (== bins_x) */
    float target_density;       /* rho_t: bin capacity fraction used by overflow and fixed scaling */
    float gamma_base_bins;      /* WA smoothing base, in bins; gamma = base*bin_w*10^(20/9 (tau-0.1) - 1) */
    int32_t field_solver;       /* AP_FIELD_* */
    float init_density_weight;  /* lambda_0 = this * |grad WL|_1 / |grad D|_1 */
    float ref_delta_hpwl;       /* lambda update reference HPWL change; <= 0 selects 0.1 * nets * bin_w */
    float lambda_mu_max;        /* lambda multiplier bounds: mu in [mu_min, mu_max] */
    float lambda_mu_min;
    float init_step_coef;       /* first step: v_{-1} = v_0 - coef * g_0 (in bins) */
    float target_overflow;      /* ap_run stops once overflow < this */
    int32_t max_iterations;     /* ap_run upper bound */
    int32_t check_interval;     /* ap_run reads the device status every this many iterations */
    int32_t use_graph;          /* capture the iteration in a CUDA graph (1) or launch eagerly (0) */
    int32_t max_backtracks;     /* step re-predictions per iteration (ePlace backtracking), 0 = off */
    int32_t restart_mode;       /* momentum restart: 0 none, 1 gradient, 2 every step, 3 speed, 4 overflow rise */
    int32_t filler_cells;       /* 1: add ePlace filler cells (internal, unconnected, movable) that take the
                                   white space target_density leaves: area rho_t (die - fixed) - movable, size
                                   the mean width x height of the cells between the 10th and 90th area
                                   percentile; they are in the density the field sees, not in the overflow,
                                   and never appear in positions passed in or out */
    int32_t block_nodes;        /* nodes (nets) per block of the node- and net-parallel launches, at least;
                                   0 = one per thread, the GPU filled by one instance (the batched form
                                   uses 2048 when 0).  Results depend on it only through the order of
                                   FP32 block sums */
} ap_params;

/* Per-iteration readout; the fields of printIterationResults (AIEplace.cpp:1048-1070)
 * plus the optimiser scalars the reference lacks. */
typedef struct ap_stats {
    int32_t iteration;
    int32_t status;
    double hpwl;          /* sum over nets of bounding-box half perimeter (Net.cpp:136-155) */
    double wa_wirelength; /* weighted-average wirelength at the same positions */
    double overflow;      /* sum_b max(0, rho_b - rho_t*A_b) / movable area */
    double overflow_abs;  /* reference form: sum_b max(0, overlap_b - A_b) (Grid.cpp:144-151) */
    double lambda;        /* density weight */
    double gamma;         /* WA smoothing, die units */
    double alpha;         /* Nesterov step length predicted for the next step */
    double a_k;           /* Nesterov momentum sequence */
    int32_t evals;        /* gradient evaluations (accepted and backtracked trials) */
    int32_t restarts;     /* momentum restarts */
} ap_stats;

typedef struct ap_handle ap_handle;

int ap_abi_version(void);
const char *ap_status_string(int status);

/* Fills defaults (bins 512, rho_t 1.0, gamma base 4 bins, FP32 solver, lambda_0 8e-5 ...). */
int ap_params_default(ap_params *p);

/* Builds the device-resident instance.  Replaces Placer::Placer
 * (vck5000/host/src/AIEplace.cpp:87-138) and Grid::Grid (Grid.cpp:6-22). */
int ap_create(const ap_netlist *netlist, const ap_params *params, ap_handle **out);
int ap_destroy(ap_handle *h);

/* Filler cells the handle added (ap_params.filler_cells): count and size. */
int ap_get_fillers(ap_handle *h, int32_t *count, float *width, float *height);

/* Runs all following device work of this handle on `stream` (a cudaStream_t). */
int ap_set_stream(ap_handle *h, void *cuda_stream);

/* Sets movable positions from caller arrays indexed like the netlist (fixed
 * entries ignored) and resets the optimiser.  Replaces the placement half of
 * Placer::initializePlacement (AIEplace.cpp:187-243). */
int ap_init_positions(ap_handle *h, const float *x, const float *y);

/* Seeded initial placement: die centre plus N(0, sigma) per movable node
 * (the reference uses unseeded rand() in +-dieW/4, AIEplace.cpp:200-213). */
int ap_init_seeded(ap_handle *h, uint64_t seed, float sigma);

/* n_iter accepted iterations of the preconditioned Nesterov loop; one
 * iteration is the reference's performIteration (AIEplace.cpp:9-39):
 * wirelength gradient, density map, field solve, field gather and position
 * update, HPWL and overflow readout.  A step whose re-predicted length falls
 * below 0.95 of the one tried is redone (ePlace backtracking), so an
 * iteration costs one or more gradient evaluations. */
int ap_step(ap_handle *h, int32_t n_iter);

/* Enqueues n_trials trial steps (each one gradient evaluation; accepted ones
 * advance the iteration count) on the handle's stream and returns without
 * waiting: the building block of device-side timing. */
int ap_step_async(ap_handle *h, int32_t n_trials);

/* Runs n_trials trial steps with one CUDA event between stages and returns
 * the mean milliseconds per stage: [0] density scatter + position update,
 * [1] density -> solver input + overflow, [2] wirelength gradient,
 * [3] field solve, [4] field gather + step control.  *n_stages = 5. */
int ap_profile_stages(ap_handle *h, int32_t n_trials, float *stage_ms, int32_t *n_stages);

/* Per-trial trajectory log, one JSON object a line: eval, iteration,
 * accepted, hpwl, overflow, overflow_abs, lambda, alpha, gamma, field (exact,
 * surrogate or judged), surrogate_error (the last judged surrogate field
 * error), t_ms (device clock since the first record).  The reference prints
 * the same quantities per iteration (printIterationResults,
 * AIEplace.cpp:1048-1070).  The loop writes each trial's record into a
 * device ring of `capacity` records; the host drains it into `path` whenever
 * a call reads the optimiser's state (ap_run every check_interval
 * iterations, ap_step, ap_step_host, ap_get_stats ...), so logging adds no
 * synchronisation to the loop.  Trials overwritten in the ring before a
 * drain are counted in a {"lost_trials": n} line.  path NULL stops logging. */
int ap_set_log(ap_handle *h, const char *path, int32_t capacity);

/* Tile shapes the autotuner picked at ap_create for this bin count, and the
 * solve times it measured: tc_variant is the tensor-core candidate (0: four
 * launches of 128 x 64 tiles, 4 pipeline stages; 1: 128 x 128, 3 stages; 2:
 * 128 x 64, 2 stages, two CTAs per SM; 3: one persistent launch over the four
 * stages' 128 x 128 tiles, K of the first two stages split in two; 4: the
 * same without the split; -1 if the
 * tensor-core path is unavailable), simt_tile the FP32 tile side (32 or 64);
 * tc_ms[5] and simt_ms[2] the candidates' times (-1: not run).  The
 * environment variable AP_TC_VARIANT=0..4, read at ap_create, pins a
 * candidate that ran instead of the fastest (for testing each one). */
int ap_solver_info(ap_handle *h, int32_t *tc_variant, float *tc_ms, int32_t *simt_tile, float *simt_ms);

/* Iterates until overflow < params.target_overflow or max_iterations;
 * replaces Placer::run (AIEplace.cpp:44-76). */
int ap_run(ap_handle *h, int32_t *iterations_done);

/* Host-buffer iteration for callers that own the positions, as the reference
 * host does (Node::m_pos): x_in/y_in replace the current positions (NULL keeps
 * them), one iteration runs, the new positions and readout are copied out.
 * The optimiser state stays on the device. */
int ap_step_host(ap_handle *h, const float *x_in, const float *y_in,
                 float *x_out, float *y_out, ap_stats *stats);

int ap_get_positions(ap_handle *h, float *x, float *y);
int ap_get_stats(ap_handle *h, ap_stats *stats);

/* Readout at the current positions: DataBase::computeTotalWirelength
 * (DataBase.cpp:143-149) and Grid::computeTotalOverflow (Grid.cpp:144-151). */
int ap_hpwl(ap_handle *h, double *hpwl);
int ap_overflow(ap_handle *h, double *overflow, double *overflow_abs);

/* ---- per-stage entry points (one per reference function) --------------- */

/* WA wirelength gradient at the given node positions (all nodes, netlist
 * order).  Replaces Placer::computeAllPartials_CPU / computeNetPartials_CPU
 * (AIEplace.cpp:574-673) and the AIE partials graph (aie/src/partials/
 * compute_abc.cpp:23-125, compute_partials.cpp:11-63).  Unlike the reference
 * it covers every net degree >= 2 (the reference stops at 8, AIEplace.cpp:586).
 * gx/gy receive dWA/dx, dWA/dy per node (fixed nodes included); wa/hpwl may be NULL. */
int ap_wirelength_grad(ap_handle *h, const float *x, const float *y, float gamma,
                       float *gx, float *gy, double *wa, double *hpwl);

/* Density map at the given positions, int64 fixed point (2^32 per unit area),
 * movable and fixed nodes at weight 1.  Replaces Placer::computeOverlaps
 * (AIEplace.cpp:937-967) + Grid::computeBinOverlaps (Grid.cpp:38-110) +
 * Grid::getRho (Grid.cpp:112-127).  rho_q has bins_x*bins_y entries, x-major. */
int ap_density_map(ap_handle *h, const float *x, const float *y, int64_t *rho_q);

/* Electrostatic solve on a caller density map (x-major, bins_x*bins_y) with
 * the RePlAce conventions of python/AIEmath/fft_replace/fft.cpp:204-299
 * (FFT::doFFT): DCT-II, halved edge rows, 4/(Mx My), phi = a/(wx^2+wy^2),
 * Ex by sine-cosine, Ey by cosine-sine inverse transforms.  ex/ey receive the
 * field per bin; the solver is params.field_solver or `solver` if >= 0. */
int ap_field_solve(ap_handle *h, const float *density, float *ex, float *ey, int32_t solver);

/* Per-node field force and preconditioned gradient at given positions, on
 * caller field maps: the stage of a loop trial between the field solve and
 * the position update, evaluated by the loop's own gather kernel (through
 * the bin records a trial's position update makes).  Replaces the
 * per-component force of Placer::nudgeNode (AIEplace.cpp:1004-1046), which
 * the reference turns into a fixed-rate step.  x, y: all nodes, netlist
 * order; ex, ey: field per bin, x-major bins_x*bins_y (as ap_field_solve
 * returns).  fx, fy receive F_i = sum over the bins b the node overlaps of
 * (overlap_ib / bin area) * E_b, for movable nodes (0 for fixed nodes).  gx,
 * gy (both NULL to skip) receive the preconditioned gradient
 * (dWA/dx_i - lambda F_i) / max(1, pins_i + lambda * area_i / bin area),
 * the WA gradient taken at smoothing gamma (die units). */
int ap_node_force(ap_handle *h, const float *x, const float *y, const float *ex, const float *ey, float gamma,
                  float lambda, float *fx, float *fy, float *gx, float *gy);

/* Allocation-free field solve.  No counterpart in the reference.  For callers
 * that cannot allocate device memory -- a host framework that owns every
 * device allocation and hands out only its own buffers, a fixed memory
 * budget, a path where cudaMalloc must not run -- this is the FP32 solve of
 * ap_field_solve on caller-owned DEVICE buffers (density in; ex, ey out;
 * x-major bins*bins floats) that allocates nothing: its scratch is one fixed
 * array in the library's static device memory, sized for bins <= 256 (2.1 MB,
 * held on every GPU that loads the library until the process exits).  bins
 * must be a multiple of 32 in [32, 256]; other sizes return
 * AP_ERR_INVALID_ARG.  bin_ratio is bin height / bin width (ap_create uses
 * (die height / bins_y) / (die width / bins_x)); it scales the y frequencies.
 * density must start on a 16-byte boundary (it is read in 16-byte vectors)
 * and ex, ey on a 4-byte boundary; otherwise AP_ERR_INVALID_ARG and nothing
 * is launched.  The first call on a device, the first after bins or
 * bin_ratio change and the first in a new CUDA context fill the transform
 * tables: make that call before any stream capture.  All calls share the one
 * scratch array, so calls whose GPU work overlaps race on it.  Work is
 * enqueued on `cuda_stream` (a cudaStream_t, NULL = legacy default stream). */
int ap_field_solve_noalloc(const float *density, float *ex, float *ey, int32_t bins, float bin_ratio,
                           void *cuda_stream);

/* Self-check of the library's integer-arithmetic float<->integer conversions
 * (used on the hot path in place of conversion instructions) against the
 * GPU's own conversion instructions.  No counterpart in the reference.
 * mismatches[6] receives the number of differing results of: round-to-nearest
 * float->int32, truncating float->int32, int64->float, the gradient
 * quantiser, fixed-point int64->float (|q| < 2^22 and any int64), truncating
 * float->int32 on (-1, 2^23); each
 * over `samples` (<= 2^32) hashed inputs
 * including rounding ties.  Runs on the current device, synchronously. */
int ap_selftest_numerics(int32_t *mismatches, int64_t samples);

/* Failure injection for tests of the error paths.  No counterpart in the
 * reference.  Nothing is faulted: AP_FAULT_TC_STALL makes the tensor-core
 * solve's load issuer issue no copies and bounds each of its kernels' waits
 * by wait_ns (1 ms .. 2 s), so the MMA issuer's wait for data that never
 * arrives runs out, every CTA leaves through the abort path with no copy in
 * flight (TMEM freed, cluster barriers met), and the next synchronising call
 * of the handle returns AP_ERR_TIMEOUT; the GPU context stays usable.
 * AP_FAULT_NONE removes the injection and clears the handle's timeout status.
 * Needs the tensor-core solver (AP_ERR_UNSUPPORTED otherwise). */
enum { AP_FAULT_NONE = 0, AP_FAULT_TC_STALL = 1, AP_FAULT_NEVER_ARRIVE = 2 };
int ap_debug_inject(ap_handle *h, int32_t kind, int64_t wait_ns);

/* ---- checkpoint / resume ----------------------------------------------- */
int ap_snapshot_size(ap_handle *h, size_t *bytes);
int ap_snapshot(ap_handle *h, void *buf, size_t bytes);
int ap_restore(ap_handle *h, const void *buf, size_t bytes);

/* ---- batched form ---------------------------------------------------------
 * Many independent placements stepped together.  The reference places one
 * design per run (Placer::run, AIEplace.cpp:44-76); small designs cannot fill
 * a GB300 alone, so a batch advances every active instance by one trial step
 * per launch of one CUDA graph, in one of two forms:
 *   AP_BATCH_PERSISTENT  nine persistent kernels per trial step, one per stage
 *                        (position update, four WA launches by net degree, bin
 *                        scatter, density/overflow, field solve, gather), each
 *                        over all instances: its resident blocks pull
 *                        (instance, block)
 *                        work items off a device queue, so instances of uneven
 *                        size share the GPU; the field solve's four
 *                        contractions of an instance wait on one another
 *                        inside the launch (bounded waits, below), with the
 *                        tile chosen by the batch's autotuner.  Needs the FP32
 *                        field solve and no surrogate; the default where it
 *                        serves every instance.
 *   AP_BATCH_GRAPH       every instance's own launches as parallel branches.
 * Instances keep their own parameters (bin counts may differ) and produce,
 * in either form, exactly the results they produce when stepped alone. */
typedef struct ap_batch ap_batch;
enum { AP_BATCH_GRAPH = 0, AP_BATCH_PERSISTENT = 1 };
typedef struct {
    int32_t form;                /* AP_BATCH_* */
    int32_t instances, active;
    int32_t field_tile;          /* persistent form: field tile of the autotuner (32 or 64; 0 = not tuned) */
    float field_tune_ms[2];      /* its measured field launch with 32 and with 64 tiles */
    int32_t records[6];          /* work records per persistent launch: update, scatter, rho, WA, field, gather */
    int32_t item_blocks[6];      /* blocks of a record's own launch per work item */
    int32_t items[6];            /* work items per persistent launch */
} ap_batch_info;

int ap_create_batch(int32_t n, const ap_netlist *netlists, const ap_params *params, ap_batch **out);
int ap_batch_destroy(ap_batch *b);
/* instance i gets ap_init_seeded(seed + i, sigma) */
int ap_batch_init_seeded(ap_batch *b, uint64_t seed, float sigma);
/* n_trials graph launches (each one trial step of every active instance) */
int ap_batch_step(ap_batch *b, int32_t n_trials);
/* steps until every instance has overflow < its target_overflow (or reached
 * its max_iterations); converged instances leave the graph, and so does an
 * instance whose optimiser diverges (its ap_stats.status then reads
 * AP_ERR_DIVERGED; the others go on).  iterations[i] receives instance i's
 * accepted iterations (may be NULL). */
int ap_batch_run(ap_batch *b, int32_t *iterations);
int ap_batch_get_stats(ap_batch *b, int32_t i, ap_stats *stats);
int ap_batch_get_positions(ap_batch *b, int32_t i, float *x, float *y);
/* switches the form (AP_ERR_UNSUPPORTED: the persistent form cannot serve
 * every instance); takes effect at the next step */
int ap_batch_set_form(ap_batch *b, int32_t form);
int ap_batch_get_info(ap_batch *b, ap_batch_info *info);
/* persistent form: blocks of a record's own launch per work item of the
 * non-field stages (1 .. 4096); 0 (the default) sizes them so that each
 * launch has about four items per resident block.  Results do not depend on
 * it. */
int ap_batch_set_item_blocks(ap_batch *b, int32_t blocks);
/* persistent form: n_trials trial steps (they advance the instances) as
 * eager launches with events around each; stage_ms[6] receives the mean
 * milliseconds of the update, scatter, rho, WA, field and gather launches
 * (the WA launch then runs alone, not beside the density chain) */
int ap_batch_profile(ap_batch *b, int32_t n_trials, float *stage_ms);
/* Failure injection (persistent form): AP_FAULT_NEVER_ARRIVE makes every
 * dependency wait of the field launch wait for one work item more than the
 * awaited contraction has, bounded by wait_ns (1 ms .. 2 s): the first wait
 * runs out, the launch's remaining items skip their work, the launch ends,
 * and ap_batch_step / ap_batch_run return AP_ERR_TIMEOUT.  The instances'
 * state is then undefined until ap_batch_init_seeded; AP_FAULT_NONE removes
 * the injection and clears the status.  Without injection each wait is
 * bounded by 1 s. */
int ap_batch_debug_inject(ap_batch *b, int32_t kind, int64_t wait_ns);

/* ---- learned density-to-field surrogate ------------------------------------
 * No counterpart in the reference (its field solves are exact).  A surrogate
 * stands in for the exact solve of an M x M map during the early,
 * high-overflow trials of the loop:
 *   coarse grid R = M / factor: the density is pooled factor x factor, the
 *   field is solved exactly at R (FP32), and a 4-layer conv net (32 hidden
 *   channels, ReLU) maps the factor^2 sub-bin densities of each coarse bin
 *   plus the coarse field (scaled by its RMS) to the fine-resolution residual
 *   field (2 factor^2 output channels, depth-to-space).
 * Training runs on the GPU with the library's own forward/backward kernels
 * (FP32, Adam, deterministic) on (density, field) pairs that the exact solver
 * produces during loop runs (ap_surrogate_collect).  Parameters are one flat
 * FP32 vector: per layer the weights [cout][cin][k][k], then the biases.
 * R must be a multiple of 16.  Tensors are [batch][channel][x][y], y fastest. */
typedef struct ap_surrogate ap_surrogate;

typedef struct ap_surrogate_config {
    int32_t factor;     /* pooling factor f (M = f R); 1..4 */
    int32_t kernel[4];  /* kernel size of each layer, 1 or 3 */
    int32_t width;      /* hidden channels, <= 32 (32 in the shipped form) */
    uint64_t seed;      /* weight initialisation (He normal; last layer zero) */
} ap_surrogate_config;

typedef struct ap_surrogate_policy {
    float overflow_min;  /* surrogate used while the trial's overflow exceeds this (0.3) */
    int32_t judge_every; /* every n-th trial the exact solve runs and judges the surrogate (8) */
    float max_error;     /* relative field error above which the exact solve takes over (0.02) */
    int32_t use_net;     /* 0: coarse spectral layer only (the ablation), 1: with the net */
} ap_surrogate_policy;

typedef struct ap_surrogate_stats {
    int32_t used;        /* trials whose field came from the surrogate */
    int32_t judged;      /* trials that ran both and compared */
    int32_t fallbacks;   /* judgements above max_error */
    double last_error;   /* last judged relative field error */
} ap_surrogate_stats;

int ap_surrogate_config_default(ap_surrogate_config *cfg);
int ap_surrogate_create(const ap_surrogate_config *cfg, ap_surrogate **out);
int ap_surrogate_destroy(ap_surrogate *s);
int ap_surrogate_num_params(ap_surrogate *s, int32_t *n);
int ap_surrogate_get_params(ap_surrogate *s, float *params, int32_t n);
int ap_surrogate_set_params(ap_surrogate *s, const float *params, int32_t n);
/* network forward on host tensors: x [batch][f^2 + 2][res][res] -> y [batch][2 f^2][res][res] */
int ap_surrogate_forward(ap_surrogate *s, const float *x, int32_t batch, int32_t res, float *y);
/* loss = mean over pixels >= margin from the edges of (y - t)^2 and its
 * gradient with respect to every parameter (grad: num_params floats) */
int ap_surrogate_gradient(ap_surrogate *s, const float *x, const float *t, int32_t batch, int32_t res,
                          int32_t margin, float *loss, float *grad);
/* sample store on the device for n samples at coarse resolution res */
int ap_surrogate_reserve(ap_surrogate *s, int32_t n, int32_t res);
int ap_surrogate_num_samples(ap_surrogate *s, int32_t *n);
/* runs n_trials exact loop trials of h, storing every `every`-th trial's
 * (network input, residual target) pair; *collected receives the count */
int ap_surrogate_collect(ap_handle *h, ap_surrogate *s, int32_t n_trials, int32_t every, int32_t *collected);
/* Adam on random crop x crop patches (batch per step) of samples
 * [first, first + count); loss_per_step may be NULL */
int ap_surrogate_train(ap_surrogate *s, int32_t steps, int32_t batch, int32_t crop, float lr, uint64_t seed,
                       int32_t first, int32_t count, float *loss_per_step);
/* per-sample relative field error (over the whole fine map) with the net
 * and with the coarse layer alone */
int ap_surrogate_validate(ap_surrogate *s, int32_t first, int32_t count, double *err_net, double *err_coarse);
/* attaches (s != NULL) or detaches (s == NULL) a surrogate to the loop of h */
int ap_attach_surrogate(ap_handle *h, ap_surrogate *s, const ap_surrogate_policy *policy);
int ap_surrogate_get_stats(ap_handle *h, ap_surrogate_stats *stats);

/* ---- LEF/DEF designs ---------------------------------------------------------
 * Replaces the reference host's DataBase ingest (DataBase.cpp:42-96, readLEF
 * / readDEF through Limbo, and the callbacks that keep data, :340-416) and
 * DataBase::writeDEF (:538-655), for the subset those callbacks consume: LEF
 * MACRO SIZE; DEF DESIGN, UNITS DISTANCE MICRONS, DIEAREA, COMPONENTS, PINS
 * (first LAYER rectangle, placement, direction) and NETS (component and IO
 * pin connections).  Other statements and sections are skipped.
 * Netlist view (ap_design_netlist): nodes are the DEF components in file
 * order, then the DEF IO pins; coordinates are DEF database units.
 * Components placed FIXED or COVER are fixed; IO pins are fixed zero-area
 * nodes carrying pins only (the reference leaves them out of the density
 * map, AIEplace.cpp:937-958).
 * Macro sizes: AP_LEF_SIZE_DBU scales the LEF SIZE (microns) by UNITS
 * DISTANCE MICRONS and swaps width and height of components placed E, W, FE
 * or FW, so sizes and positions share one unit; AP_LEF_SIZE_AS_READ takes the
 * LEF numbers as they are and ignores orientation, as the reference host
 * does (lef_macro_cbk keeps lefiMacro::sizeX/sizeY beside DEF coordinates in
 * database units). */
enum { AP_LEF_SIZE_DBU = 0, AP_LEF_SIZE_AS_READ = 1 };

typedef struct ap_design ap_design;

typedef struct ap_design_info {
    int32_t num_nodes, num_nets, num_pins;  /* sizes of the netlist view */
    int32_t num_components, num_io_pins;
    int32_t units_per_micron;               /* DEF UNITS DISTANCE MICRONS */
    float die_xl, die_yl, die_xh, die_yh;   /* DIEAREA (bounding box), database units */
} ap_design_info;

/* LEF files are read in order (a later MACRO of a name replaces an earlier
 * one), then the DEF.  Syntax errors and references to undefined macros,
 * components or pins return AP_ERR_BAD_NETLIST; ap_last_error() then
 * names the file, line and cause. */
int ap_design_read(const char *const *lef_paths, int32_t n_lef, const char *def_path, int32_t size_mode,
                   ap_design **out);
/* The reference's input convention (DataBase.cpp:42-96): every *.lef file of
 * `dir` (in name order) and dir/floorplan.def. */
int ap_design_read_dir(const char *dir, int32_t size_mode, ap_design **out);
int ap_design_get_info(ap_design *d, ap_design_info *info);
/* Fills *nl with pointers into the design (valid until ap_design_destroy);
 * ready for ap_create. */
int ap_design_netlist(ap_design *d, ap_netlist *nl);
const char *ap_design_name(ap_design *d);
const char *ap_design_node_name(ap_design *d, int32_t node);
/* Writes the design as DEF 5.8 with the node positions x, y (netlist order,
 * database units, lower-left corners, as ap_get_positions returns them)
 * rounded to integers: movable components PLACED at their new position, fixed
 * ones where they were.  The position export a downstream legaliser reads. */
int ap_design_write_def(ap_design *d, const float *x, const float *y, const char *path);
int ap_design_destroy(ap_design *d);

/* ---- run configuration -----------------------------------------------------
 * The placer's configuration file, the counterpart of the reference host's
 * host/config_aieplace.json (read at AIEplace.cpp:87-109).  Keys under
 * "params" (or at the top level).  Reference keys: use_aie (accepted,
 * unused), input_filepath (design directory: *.lef + floorplan.def),
 * output_filepath (directory of the placed <design>.def), wirelength_method
 * ("HPWL" | "WA", the wirelength reported), bins_per_row (bins_x = bins_y),
 * gamma (gamma_base_bins: WA smoothing in bins, scaled with the overflow),
 * max_iterations, init_learning_rate (accepted, unused: the Nesterov loop
 * predicts its steps), init_global_lambda (init_density_weight if > 0).
 * Keys of this placer: every ap_params field by name (field_solver "fp32" |
 * "bf16x3"), log_path, lef_size_mode ("dbu" | "as_read"), seed, init_sigma
 * (die units; 0 = one bin width), filler_cells.  Unknown keys and
 * ill-typed values return AP_ERR_INVALID_ARG, ap_last_error() naming them. */
typedef struct ap_run_config {
    char input_dir[1024];
    char output_dir[1024];
    char log_path[1024];         /* per-trial trajectory (ap_set_log); "" = none */
    int32_t size_mode;           /* AP_LEF_SIZE_* */
    int32_t wirelength_method;   /* 0 HPWL, 1 WA */
    float init_sigma;            /* seeded initial spread, die units; 0 = one bin width */
    uint64_t seed;
    int32_t filler_cells;        /* 1: ap_params.filler_cells */
    int32_t use_aie;             /* as read; unused */
    float ignored_learning_rate; /* init_learning_rate as read; unused */
} ap_run_config;

int ap_run_config_default(ap_params *params, ap_run_config *run);
int ap_run_config_read(const char *path, ap_params *params, ap_run_config *run);

/* the message of the last failed design read/write or config read on this
 * thread ("" if none) */
const char *ap_last_error(void);

/* ---- seeded synthetic netlists ------------------------------------------ */
/* Stands in for the ISPD suites the reference reads through LEF/DEF.  Nodes
 * are ordered: movable cells, fixed macros, IO pads. */
typedef struct ap_synth_config {
    int32_t num_cells;        /* movable cells */
    int32_t num_nets;
    int32_t num_macros;       /* fixed macros */
    int32_t num_pads;         /* zero-area fixed IO pads on the die boundary */
    int32_t unit_cells;       /* 1: every cell 1x1; 0: width ~ LogNormal(ln 2, 0.5), height 1 */
    int32_t degree_mix;       /* 0: 70% 2, 20% 3, 10% 4 pins; 1: 65% 2, 20% 3, 10% U[4,10], 5% U[11,64] */
    float locality;           /* probability a pin is drawn within `window` node indices of the net anchor */
    int32_t window;           /* locality window (node indices) */
    float macro_area_min;     /* macro area U[min, max] (square-ish) */
    float macro_area_max;
    float target_density;     /* sizes the die: area = movable/rho_t + macros */
    float die_side;           /* > 0 forces a square die of this side */
    uint64_t seed;
} ap_synth_config;

int ap_synth_counts(const ap_synth_config *cfg, int32_t *num_nodes, int32_t *num_nets,
                    int32_t *num_pins);
/* Arrays sized by ap_synth_counts; die receives {xl, yl, xh, yh}. */
int ap_synth_generate(const ap_synth_config *cfg, int32_t *net_ptr, int32_t *pin_node,
                      float *node_w, float *node_h, float *node_x, float *node_y,
                      uint8_t *node_fixed, float *die);

#ifdef __cplusplus
}
#endif
#endif /* AIEPLACE_H */
