/*
 * oracle.h -- CPU restatement of the reference ePlace iteration.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load this library, and only
 * as the checker or the timed CPU baseline.  The product path never calls it.
 *
 * Every function cites the reference source it restates (paths inside
 * searsm8/AIEplace).  Values are FP64 unless stated; the density map uses the
 * same int64 fixed-point definition as the GPU kernels so the two are
 * bit-exact.
 */
#ifndef AP_ORACLE_H
#define AP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* fixed point: coordinates carry 16 fractional bits, areas 32 */
#define OR_COORD_SHIFT 16
#define OR_AREA_SHIFT 32

/* python/AIEmath/computeTerm.py:6-13 fast_exp: (1 + a/2^prec)^(2^prec) */
double or_fast_exp(double a, int prec);

/* computeTerm.py:15-56 on one ascending-sorted coordinate list: a+ a- per pin,
 * b+ b- c+ c-, and dWA/dx_i per pin.  use_fast_exp selects fast_exp(prec 16)
 * instead of exp (the AIE kernel uses fast_exp, compute_abc.cpp:12-18). */
void or_wa_terms_sorted(int n, const double *x, double gamma, int use_fast_exp, double *a_plus,
                        double *a_minus, double *bc /* b+ c+ b- c- */, double *partial);

/* AIEplace.cpp:612-673 compute_a_terms_CPU / compute_bc_terms_CPU /
 * computeNetPartials_CPU over a CSR netlist, FP64.  Nets of degree outside
 * [min_deg, max_deg] are skipped (the reference uses 2..8).  gx/gy are
 * overwritten.  wa/hpwl receive the totals (HPWL: Net.cpp:136-155 summed in
 * double as DataBase.cpp:143-149). */
void or_wa_grad(int n_nodes, int n_nets, const int32_t *net_ptr, const int32_t *pin_node,
                const float *x, const float *y, double gamma, int min_deg, int max_deg,
                double *gx, double *gy, double *wa, double *hpwl);

/* Bin geometry of Grid::init (Grid.cpp:6-22): float bin width/height, the
 * small-node threshold bin_area/16 (AIEplace.cpp:200), and the fixed-point
 * bin sides. */
typedef struct or_grid {
    int mx, my;
    float die_w, die_h;
    float bw, bh;
    float small_threshold;
    int64_t bw_q, bh_q;
} or_grid;

void or_grid_init(or_grid *g, float die_w, float die_h, int mx, int my);

/* Grid::computeBinOverlaps (Grid.cpp:38-110) + Bin::computeOverlap
 * (Bin.h:78-121) for every node with include[i] != 0 (NULL = all) and
 * nonzero area: bin indices by float truncation of x/bw exactly as the
 * reference, overlap areas in int64 fixed point.  rho_q is accumulated into
 * (caller zeroes it), x-major [bx*my+by]. */
void or_density_q(const or_grid *g, int n_nodes, const float *x, const float *y, const float *w,
                  const float *h, const uint8_t *include, int64_t *rho_q);

/* Placer::nudgeNode per-component force (AIEplace.cpp:1004-1046): F_i =
 * sum over the bins node i overlaps of (overlap / bin area) * E_b, with the
 * fixed-point overlaps of or_density_q and FP64 sums; fx/fy overwritten
 * (0 for nodes with include[i] == 0 or no overlap). */
void or_node_force(const or_grid *g, int n_nodes, const float *x, const float *y, const float *w,
                   const float *h, const uint8_t *include, const double *ex, const double *ey, double *fx,
                   double *fy);

/* Overflow: tau = sum_b max(0, tot_b - rho_t*A_b) / movable area (ePlace),
 * and the reference absolute form sum_b max(0, overlap_b - A_b)
 * (Grid.cpp:144-151, Bin.h:123-126).  tot = mov + fixed_scaled. */
void or_overflow(const or_grid *g, const int64_t *mov_q, const int64_t *fixed_q,
                 const int64_t *fixed_scaled_q, double rho_t, double movable_area_q,
                 double *tau, double *abs_overflow);

/* fixed_scaled_q[b] = llrint(rho_t * fixed_q[b]) */
void or_scale_fixed(int nbins, const int64_t *fixed_q, double rho_t, int64_t *out);

/* density d_b = (float)tot_q * (float)(1 / A_b_q) (FP32 ops) as the solver input */
void or_density_float(const or_grid *g, const int64_t *mov_q, const int64_t *fixed_scaled_q,
                      float *d);

/* RePlAce electrostatics, fft.cpp:204-299 (FFT::doFFT), restated with direct
 * separable transforms in FP64 (the Ooura ddct2d/ddsct2d/ddcst2d of
 * fftsg2d.cpp:569-760 compute the same sums).  d, phi, ex, ey are x-major
 * mx*my; phi may be NULL.  bin_ratio = bh/bw (fft.cpp:172-175). */
void or_field_solve(int mx, int my, double bin_ratio, const double *d, double *phi, double *ex,
                    double *ey);

/* The same sums as or_field_solve in O(n^2 log n) (fft_solve.c: fast
 * DCT-II / cosine / sine sums through radix-2 complex FFTs, Makhoul 1980).
 * n = mx = my a power of two; returns 0, or -1 for other sizes.  The oracle
 * loop and the timed CPU baseline use this one; the dense solve above is
 * the checker it is pinned against. */
int or_field_solve_fft(int mx, int my, double bin_ratio, const double *d, double *phi, double *ex,
                       double *ey);

/* DCT.cpp:24-82 DCT_naive / IDCT_naive / IDXST_naive in FP64 */
void or_dct_1d(int n, const double *in, double *out);
void or_idct_1d(int n, const double *in, double *out);
void or_idxst_1d(int n, const double *in, double *out);

/* ---- whole-loop FP64 oracle (preconditioned Nesterov, ePlace) ---------- */
typedef struct or_params {
    int mx, my;
    double target_density;
    double gamma_base_bins;
    double init_density_weight;
    double ref_delta_hpwl; /* <= 0: 0.1 * nets * bw */
    double mu_max, mu_min;
    double init_step_coef;
    int restart;        /* momentum restart: 0 none, 1 gradient, 2 every step, 3 speed, 4 overflow rise */
    int max_backtracks; /* step re-predictions per iteration */
} or_params;

typedef struct or_stats {
    int iteration;
    double hpwl, wa, overflow, overflow_abs, lambda, gamma, alpha, a_k;
    int evals; /* gradient evaluations, backtracking included */
    double norm_wl, norm_f; /* L1 norms of grad WL and of the field force, last evaluation */
    int restarts;           /* momentum restarts so far */
} or_stats;

typedef struct or_placer or_placer;

or_placer *or_create(int n_nodes, int n_nets, const int32_t *net_ptr, const int32_t *pin_node,
                     const float *w, const float *h, const float *x, const float *y,
                     const uint8_t *fixed, float die_w, float die_h, const or_params *p);
/* sets movable positions, then evaluates the starting point (gradient, lambda_0, first step) */
void or_init(or_placer *o, const float *x, const float *y);
void or_step(or_placer *o, int n);
void or_get_stats(const or_placer *o, or_stats *s);
void or_get_positions(const or_placer *o, float *x, float *y);
void or_destroy(or_placer *o);

/* multi-threading for the timed CPU baseline (OpenMP); returns threads used */
int or_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
