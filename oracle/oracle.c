/*
 * oracle.c -- CPU restatement of the reference ePlace iteration (FP64).
 *
 * TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and the
 * CPU legs of bench.py as the checker / timed CPU baseline, never by the
 * product path.  Compile with -ffp-contract=off so the operation order below
 * is the one evaluated (golden KATs compare bit for bit).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_PI 3.14159265358979323846
#define OR_LAMBDA_MAX 1e30 /* density penalty cap, the same as the CUDA path */

int or_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

/* ---- WA terms ---------------------------------------------------------- */

/* computeTerm.py:6-13 */
double or_fast_exp(double a, int prec) {
    a = 1.0 + a / ldexp(1.0, prec);
    for (int i = 0; i < prec; ++i) a *= a;
    return a;
}

static double wa_exp(double a, int use_fast) { return use_fast ? or_fast_exp(a, 16) : exp(a); }

/* computeTerm.py:15-56 (a_plus, a_minus, b_term, c_term, WA_partial) */
void or_wa_terms_sorted(int n, const double *x, double gamma, int use_fast_exp, double *a_plus,
                        double *a_minus, double *bc, double *partial) {
    double bp = 0.0, cp = 0.0, bm = 0.0, cm = 0.0;
    for (int i = 0; i < n; ++i) a_plus[i] = wa_exp((x[i] - x[n - 1]) / gamma, use_fast_exp);
    a_minus[0] = 1.0;
    for (int i = 1; i < n; ++i) a_minus[i] = wa_exp((x[0] - x[i]) / gamma, use_fast_exp);
    for (int i = 0; i < n; ++i) bp += a_plus[i];
    for (int i = 0; i < n; ++i) cp += x[i] * a_plus[i];
    for (int i = 0; i < n; ++i) bm += a_minus[i];
    for (int i = 0; i < n; ++i) cm += x[i] * a_minus[i];
    bc[0] = bp;
    bc[1] = cp;
    bc[2] = bm;
    bc[3] = cm;
    for (int i = 0; i < n; ++i) {
        double t1 = ((1 + x[i] / gamma) * bp - cp / gamma) * a_plus[i] / (bp * bp);
        double t2 = ((1 - x[i] / gamma) * bm + cm / gamma) * a_minus[i] / (bm * bm);
        partial[i] = t1 - t2;
    }
}

/* One axis of AIEplace.cpp:612-673 for one net: returns WA, writes partials. */
static double wa_net_axis(int d, const double *c, double gamma, double *part) {
    double cmax = c[0], cmin = c[0];
    for (int j = 1; j < d; ++j) {
        if (c[j] > cmax) cmax = c[j];
        if (c[j] < cmin) cmin = c[j];
    }
    double bp = 0, cp = 0, bm = 0, cm = 0;
    for (int j = 0; j < d; ++j) {
        double ap = exp((c[j] - cmax) / gamma), am = exp((cmin - c[j]) / gamma);
        bp += ap;
        bm += am;
        cp += ap * c[j];
        cm += am * c[j];
    }
    for (int j = 0; j < d; ++j) {
        double ap = exp((c[j] - cmax) / gamma), am = exp((cmin - c[j]) / gamma);
        part[j] = ((1 + c[j] / gamma) * bp - cp / gamma) * (ap / (bp * bp)) -
                  ((1 - c[j] / gamma) * bm + cm / gamma) * (am / (bm * bm));
    }
    return cp / bp - cm / bm;
}

void or_wa_grad(int n_nodes, int n_nets, const int32_t *net_ptr, const int32_t *pin_node,
                const float *x, const float *y, double gamma, int min_deg, int max_deg,
                double *gx, double *gy, double *wa, double *hpwl) {
    int32_t n_pins = net_ptr[n_nets];
    double *px = (double *)malloc(sizeof(double) * (size_t)(n_pins > 0 ? n_pins : 1));
    double *py = (double *)malloc(sizeof(double) * (size_t)(n_pins > 0 ? n_pins : 1));
    double wa_sum = 0.0, hp_sum = 0.0;
#pragma omp parallel
    {
        double cx[64], cy[64];
        double *bx = cx, *by = cy;
        int cap = 64;
#pragma omp for schedule(dynamic, 1024) reduction(+ : wa_sum, hp_sum)
        for (int e = 0; e < n_nets; ++e) {
            int s = net_ptr[e], d = net_ptr[e + 1] - s;
            if (d < 2) {
                for (int j = 0; j < d; ++j) px[s + j] = py[s + j] = 0.0;
                continue;
            }
            if (d > cap) {
                if (bx != cx) { free(bx); free(by); }
                cap = d;
                bx = (double *)malloc(sizeof(double) * (size_t)cap);
                by = (double *)malloc(sizeof(double) * (size_t)cap);
            }
            for (int j = 0; j < d; ++j) {
                bx[j] = (double)x[pin_node[s + j]];
                by[j] = (double)y[pin_node[s + j]];
            }
            double xmx = bx[0], xmn = bx[0], ymx = by[0], ymn = by[0];
            for (int j = 1; j < d; ++j) {
                xmx = bx[j] > xmx ? bx[j] : xmx;
                xmn = bx[j] < xmn ? bx[j] : xmn;
                ymx = by[j] > ymx ? by[j] : ymx;
                ymn = by[j] < ymn ? by[j] : ymn;
            }
            hp_sum += (xmx - xmn) + (ymx - ymn);
            if (d < min_deg || d > max_deg) {
                for (int j = 0; j < d; ++j) px[s + j] = py[s + j] = 0.0;
                continue;
            }
            wa_sum += wa_net_axis(d, bx, gamma, px + s);
            wa_sum += wa_net_axis(d, by, gamma, py + s);
        }
        if (bx != cx) { free(bx); free(by); }
    }
    for (int i = 0; i < n_nodes; ++i) gx[i] = gy[i] = 0.0;
    /* accumulate in pin order: deterministic whatever the thread count */
    for (int32_t p = 0; p < n_pins; ++p) {
        gx[pin_node[p]] += px[p];
        gy[pin_node[p]] += py[p];
    }
    free(px);
    free(py);
    if (wa) *wa = wa_sum;
    if (hpwl) *hpwl = hp_sum;
}

/* ---- density ----------------------------------------------------------- */

void or_grid_init(or_grid *g, float die_w, float die_h, int mx, int my) {
    g->mx = mx;
    g->my = my;
    g->die_w = die_w;
    g->die_h = die_h;
    g->bw = die_w / (float)mx; /* Grid.cpp:8-9 */
    g->bh = die_h / (float)my;
    g->small_threshold = g->bw * g->bh / 16; /* AIEplace.cpp:200 */
    g->bw_q = llrintf(g->bw * 65536.0f);
    g->bh_q = llrintf(g->bh * 65536.0f);
}

/* The bin range of one node under the reference rules; returns 0 if the
 * node adds nothing.  Small nodes get c0 == c1, r0 == r1 and *small = 1. */
static int bin_range(const or_grid *g, float x, float y, float w, float h, int *c0, int *c1,
                     int *r0, int *r1, int *small) {
    const float area = w * h;
    if (!(area > 0.0f)) return 0;
    *small = !(area > g->small_threshold); /* Node.h:100-104 */
    float qx = x / g->bw, qy = y / g->bh;
    if (*small) { /* Grid.cpp:46-57 */
        if (!(qx > -1.0f) || !(qx < (float)g->mx) || !(qy > -1.0f) || !(qy < (float)g->my)) return 0;
        *c0 = *c1 = (int)qx;
        *r0 = *r1 = (int)qy;
        return 1;
    }
    /* Grid.cpp:61-81: start = trunc(x/bw), final = min(M-1, trunc((x+w)/bw)),
     * nothing when start < 0 */
    if (!(qx > -1.0f) || !(qy > -1.0f)) return 0;
    float qx1 = (x + w) / g->bw, qy1 = (y + h) / g->bh;
    if (qx1 != qx1 || qy1 != qy1) return 0;
    *c0 = qx >= (float)g->mx ? g->mx : (int)qx;
    *r0 = qy >= (float)g->my ? g->my : (int)qy;
    *c1 = qx1 >= (float)g->mx ? g->mx - 1 : (int)qx1;
    *r1 = qy1 >= (float)g->my ? g->my - 1 : (int)qy1;
    if (*c1 > g->mx - 1) *c1 = g->mx - 1;
    if (*r1 > g->my - 1) *r1 = g->my - 1;
    return *c0 <= *c1 && *r0 <= *r1;
}

void or_density_q(const or_grid *g, int n_nodes, const float *x, const float *y, const float *w,
                  const float *h, const uint8_t *include, int64_t *rho_q) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n_nodes; ++i) {
        if (include && !include[i]) continue;
        int c0, c1, r0, r1, small;
        if (!bin_range(g, x[i], y[i], w[i], h[i], &c0, &c1, &r0, &r1, &small)) continue;
        const int64_t xq = llrintf(x[i] * 65536.0f), yq = llrintf(y[i] * 65536.0f);
        const int64_t wq = llrintf(w[i] * 65536.0f), hq = llrintf(h[i] * 65536.0f);
        if (small) {
            int64_t a = wq * hq;
#pragma omp atomic
            rho_q[(int64_t)c0 * g->my + r0] += a;
            continue;
        }
        for (int c = c0; c <= c1; ++c) {
            int64_t lo = (int64_t)c * g->bw_q, hi = lo + g->bw_q;
            int64_t ow = (hi < xq + wq ? hi : xq + wq) - (lo > xq ? lo : xq);
            for (int r = r0; r <= r1; ++r) {
                int64_t lo2 = (int64_t)r * g->bh_q, hi2 = lo2 + g->bh_q;
                int64_t oh = (hi2 < yq + hq ? hi2 : yq + hq) - (lo2 > yq ? lo2 : yq);
#pragma omp atomic
                rho_q[(int64_t)c * g->my + r] += ow * oh;
            }
        }
    }
}

/* Placer::nudgeNode's per-component force (AIEplace.cpp:1004-1046): the
 * field of every bin the node overlaps, weighted by overlap / bin area, with
 * the overlaps of or_density_q (fixed point, so the weights are exact) and
 * FP64 sums.  fx, fy are overwritten; nodes with include[i] == 0 get 0. */
void or_node_force(const or_grid *g, int n_nodes, const float *x, const float *y, const float *w,
                   const float *h, const uint8_t *include, const double *ex, const double *ey, double *fx,
                   double *fy) {
    const double inv_ab = 1.0 / (double)(g->bw_q * g->bh_q);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n_nodes; ++i) {
        double sx = 0.0, sy = 0.0;
        int c0, c1, r0, r1, small;
        if ((!include || include[i]) && bin_range(g, x[i], y[i], w[i], h[i], &c0, &c1, &r0, &r1, &small)) {
            const int64_t xq = llrintf(x[i] * 65536.0f), yq = llrintf(y[i] * 65536.0f);
            const int64_t wq = llrintf(w[i] * 65536.0f), hq = llrintf(h[i] * 65536.0f);
            if (small) {
                const int64_t b = (int64_t)c0 * g->my + r0;
                const double wt = (double)(wq * hq) * inv_ab;
                sx = wt * ex[b];
                sy = wt * ey[b];
            } else {
                for (int c = c0; c <= c1; ++c) {
                    int64_t lo = (int64_t)c * g->bw_q, hi = lo + g->bw_q;
                    int64_t ow = (hi < xq + wq ? hi : xq + wq) - (lo > xq ? lo : xq);
                    for (int r = r0; r <= r1; ++r) {
                        int64_t lo2 = (int64_t)r * g->bh_q, hi2 = lo2 + g->bh_q;
                        int64_t oh = (hi2 < yq + hq ? hi2 : yq + hq) - (lo2 > yq ? lo2 : yq);
                        const int64_t b = (int64_t)c * g->my + r;
                        const double wt = (double)(ow * oh) * inv_ab;
                        sx += wt * ex[b];
                        sy += wt * ey[b];
                    }
                }
            }
        }
        fx[i] = sx;
        fy[i] = sy;
    }
}

void or_scale_fixed(int nbins, const int64_t *fixed_q, double rho_t, int64_t *out) {
    for (int b = 0; b < nbins; ++b) out[b] = llrint(rho_t * (double)fixed_q[b]);
}

void or_overflow(const or_grid *g, const int64_t *mov_q, const int64_t *fixed_q,
                 const int64_t *fixed_scaled_q, double rho_t, double movable_area_q, double *tau,
                 double *abs_overflow) {
    const int64_t ab = g->bw_q * g->bh_q;
    const int64_t cap = llrint(rho_t * (double)ab);
    int64_t over = 0, over_abs = 0;
    const int nb = g->mx * g->my;
    for (int b = 0; b < nb; ++b) {
        int64_t t = mov_q[b] + (fixed_scaled_q ? fixed_scaled_q[b] : 0) - cap;
        if (t > 0) over += t;
        int64_t a = mov_q[b] + (fixed_q ? fixed_q[b] : 0) - ab;
        if (a > 0) over_abs += a;
    }
    if (tau) *tau = movable_area_q > 0 ? (double)over / movable_area_q : 0.0;
    if (abs_overflow) *abs_overflow = ldexp((double)over_abs, -OR_AREA_SHIFT);
}

void or_density_float(const or_grid *g, const int64_t *mov_q, const int64_t *fixed_scaled_q,
                      float *d) {
    const float inv_ab = (float)(1.0 / (double)(g->bw_q * g->bh_q));
    const int nb = g->mx * g->my;
    for (int b = 0; b < nb; ++b)
        d[b] = (float)(mov_q[b] + (fixed_scaled_q ? fixed_scaled_q[b] : 0)) * inv_ab;
}

/* ---- spectral solve ---------------------------------------------------- */

/* out[i][j] = sum_k A[i][k] * B[j][k]  (n x n, row-major) */
static void mm_tn(int n, const double *A, const double *B, double *out) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        const double *a = A + (size_t)i * n;
        for (int j = 0; j < n; ++j) {
            const double *b = B + (size_t)j * n;
            double s = 0.0;
            for (int k = 0; k < n; ++k) s += a[k] * b[k];
            out[(size_t)i * n + j] = s;
        }
    }
}

static void transpose(int n, const double *in, double *out) {
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) out[(size_t)j * n + i] = in[(size_t)i * n + j];
}

/* cos_t[u][x] = cos(pi u (x+1/2)/n), sin_t[u][x] = sin(...) */
static void trig_tables(int n, double *cos_t, double *sin_t) {
    for (int u = 0; u < n; ++u)
        for (int x = 0; x < n; ++x) {
            double t = OR_PI * (double)u * ((double)x + 0.5) / (double)n;
            cos_t[(size_t)u * n + x] = cos(t);
            sin_t[(size_t)u * n + x] = sin(t);
        }
}

void or_field_solve(int mx, int my, double bin_ratio, const double *d, double *phi, double *ex,
                    double *ey) {
    /* square grids (mx == my), the GPU path's contract */
    const int n = mx;
    (void)my;
    const size_t nn = (size_t)n * n;
    double *C = (double *)malloc(sizeof(double) * nn), *S = (double *)malloc(sizeof(double) * nn);
    double *Ct = (double *)malloc(sizeof(double) * nn), *St = (double *)malloc(sizeof(double) * nn);
    double *a = (double *)malloc(sizeof(double) * nn), *t = (double *)malloc(sizeof(double) * nn);
    double *tt = (double *)malloc(sizeof(double) * nn);
    double *pc = (double *)malloc(sizeof(double) * nn), *exc = (double *)malloc(sizeof(double) * nn);
    double *eyc = (double *)malloc(sizeof(double) * nn);
    trig_tables(n, C, S); /* C[k][i] = cos(pi k (i+1/2)/n), S likewise */
    transpose(n, C, Ct);
    transpose(n, S, St);
    /* a = C d C^T: 2-D DCT-II, fft.cpp:206 ddct2d(-1) */
    mm_tn(n, d, C, t);   /* t[x][v] = sum_y d[x][y] C[v][y] */
    transpose(n, t, tt); /* tt[v][x] */
    mm_tn(n, C, tt, a);  /* a[u][v] = sum_x C[u][x] t[x][v] */
    /* fft.cpp:217-229: halve row/column 0, scale by 4/(Mx My) */
    for (int u = 0; u < n; ++u)
        for (int v = 0; v < n; ++v) {
            double c = a[(size_t)u * n + v];
            if (u == 0) c *= 0.5;
            if (v == 0) c *= 0.5;
            a[(size_t)u * n + v] = c * (4.0 / n / n);
        }
    /* fft.cpp:165-176, 238-273: phi = a / (wx^2 + wy^2), E = phi * w */
    for (int u = 0; u < n; ++u) {
        double wx = OR_PI * u / n;
        for (int v = 0; v < n; ++v) {
            double wy = OR_PI * v / n * bin_ratio;
            size_t k = (size_t)u * n + v;
            if (u == 0 && v == 0) {
                pc[k] = exc[k] = eyc[k] = 0.0;
            } else {
                double p = a[k] / (wx * wx + wy * wy);
                pc[k] = p;
                exc[k] = p * wx;
                eyc[k] = p * wy;
            }
        }
    }
    /* Ex = S^T exc C   (ddsct2d: sine along x, cosine along y)
     * Ey = C^T eyc S   (ddcst2d: cosine along x, sine along y)
     * phi = C^T pc C   (ddct2d +1) */
    mm_tn(n, exc, Ct, t);  /* t[u][y] = sum_v exc[u][v] C[v][y] */
    transpose(n, t, tt);   /* tt[y][u] */
    mm_tn(n, St, tt, ex);  /* ex[x][y] = sum_u S[u][x] t[u][y] */
    mm_tn(n, eyc, St, t);  /* t[u][y] = sum_v eyc[u][v] S[v][y] */
    transpose(n, t, tt);
    mm_tn(n, Ct, tt, ey);
    if (phi) {
        mm_tn(n, pc, Ct, t);
        transpose(n, t, tt);
        mm_tn(n, Ct, tt, phi);
    }
    free(C); free(S); free(Ct); free(St); free(a); free(t); free(tt); free(pc); free(exc); free(eyc);
}

/* DCT.cpp:24-40 */
void or_dct_1d(int n, const double *in, double *out) {
    for (int k = 0; k < n; ++k) {
        double s = 0.0;
        for (int j = 0; j < n; ++j) s += in[j] * cos(OR_PI / n * (j + .5) * k);
        out[k] = s;
    }
}

/* DCT.cpp:45-59 */
void or_idct_1d(int n, const double *in, double *out) {
    for (int k = 0; k < n; ++k) {
        double s = 0.0;
        for (int j = 1; j < n; ++j) s += in[j] * cos(OR_PI / n * (k + .5) * j);
        out[k] = 0.5 * in[0] + s;
    }
}

/* DCT.cpp:64-82 */
void or_idxst_1d(int n, const double *in, double *out) {
    double *t = (double *)malloc(sizeof(double) * (size_t)n);
    t[0] = in[0];
    for (int j = 1; j < n; ++j) t[j] = in[n - j];
    or_idct_1d(n, t, out);
    for (int k = 1; k < n; k += 2) out[k] = -out[k];
    free(t);
}

/* ---- whole-loop FP64 oracle ------------------------------------------------
 * The reference loop is fixed-step descent (AIEplace.cpp:44-76, 1004-1046;
 * python/AIEplacer.py:523-552).  The loop below is the preconditioned
 * Nesterov method with Lipschitz step prediction of ePlace (Lu et al., TODAES
 * 2015), the schedule the GPU path runs, evaluated entirely in FP64 with
 * exact (double) bin overlaps. */

struct or_placer {
    int n_nodes, n_nets, n_mov;
    int32_t *net_ptr, *pin_node;
    float *w, *h;
    uint8_t *fixed;
    float *xf, *yf;           /* float copy of the evaluation point for or_wa_grad */
    double *x, *y;            /* evaluation point v (fixed nodes at their place) */
    double *ux, *uy, *vpx, *vpy, *gx, *gy, *gpx, *gpy, *wlx, *wly, *fx, *fy;
    double *rho, *fixmap, *d, *ex, *ey;
    int *pins;
    or_params p;
    double bw, bh, die_w, die_h, ab, mov_area, ref_dh;
    double a, alpha, lambda, gamma, hpwl, hpwl_prev, wa, tau, tau_abs;
    double norm_wl, norm_f; /* L1 norms of grad WL and of the field force at the last evaluation */
    double du_prev, tau_prev;
    int iteration, evals, restarts;
};

static double lipschitz_step(const or_placer *o, const double *vx, const double *vy, const double *kx,
                             const double *ky, const double *gx, const double *gy, const double *hx,
                             const double *hy);

static double *dalloc(size_t n) { return (double *)calloc(n ? n : 1, sizeof(double)); }

/* bins overlapped by a node in double, reference rules (Grid.cpp:38-110) */
typedef void (*ov_cb)(void *ctx, int bin, double ov);

static void node_overlaps(const or_placer *o, double x, double y, double w, double h, ov_cb cb,
                          void *ctx) {
    const int mx = o->p.mx, my = o->p.my;
    const double area = w * h;
    if (!(area > 0)) return;
    double qx = x / o->bw, qy = y / o->bh;
    if (!(area > o->bw * o->bh / 16)) {
        if (!(qx > -1) || !(qx < mx) || !(qy > -1) || !(qy < my)) return;
        cb(ctx, (int)qx * my + (int)qy, area);
        return;
    }
    if (!(qx > -1) || !(qy > -1)) return;
    double qx1 = (x + w) / o->bw, qy1 = (y + h) / o->bh;
    int c0 = qx >= mx ? mx : (int)qx, r0 = qy >= my ? my : (int)qy;
    int c1 = qx1 >= mx ? mx - 1 : (int)qx1, r1 = qy1 >= my ? my - 1 : (int)qy1;
    for (int c = c0; c <= c1; ++c) {
        double ow = fmin((c + 1) * o->bw, x + w) - fmax(c * o->bw, x);
        for (int r = r0; r <= r1; ++r) {
            double oh = fmin((r + 1) * o->bh, y + h) - fmax(r * o->bh, y);
            cb(ctx, c * my + r, ow * oh);
        }
    }
}

static void add_cb(void *ctx, int bin, double ov) { ((double *)ctx)[bin] += ov; }

typedef struct { const double *ex, *ey; double fx, fy, inv_ab; } gather_ctx;
static void gather_cb(void *ctx, int bin, double ov) {
    gather_ctx *g = (gather_ctx *)ctx;
    g->fx += ov * g->inv_ab * g->ex[bin];
    g->fy += ov * g->inv_ab * g->ey[bin];
}

static double gamma_of(const or_placer *o, double tau) {
    double e = (tau - 0.1) * 20.0 / 9.0 - 1.0;
    if (e > 1.0) e = 1.0;
    if (e < -1.0) e = -1.0;
    return o->p.gamma_base_bins * 0.5 * (o->bw + o->bh) * pow(10.0, e);
}

/* density, overflow, WA gradient + HPWL, field, gather at (x, y).
 * gamma_mode 0: keep gamma; 1: gamma(tau) of this point before the WA terms
 * (the first evaluation); 2: the WA terms with the current gamma, then
 * gamma(tau) of this point for the next evaluation (loop trials: a
 * one-evaluation lag, so that the GPU's WA launches need not wait for the
 * trial's density). */
static void evaluate(or_placer *o, int gamma_mode) {
    const int nb = o->p.mx * o->p.my, n = o->n_nodes;
    for (int b = 0; b < nb; ++b) o->rho[b] = 0.0;
    for (int i = 0; i < o->n_mov; ++i) node_overlaps(o, o->x[i], o->y[i], o->w[i], o->h[i], add_cb, o->rho);
    const double rt = o->p.target_density;
    double over = 0, over_abs = 0;
    for (int b = 0; b < nb; ++b) {
        double t = o->rho[b] + rt * o->fixmap[b] - rt * o->ab;
        if (t > 0) over += t;
        double a = o->rho[b] + o->fixmap[b] - o->ab;
        if (a > 0) over_abs += a;
        o->d[b] = (o->rho[b] + rt * o->fixmap[b]) / o->ab;
    }
    o->tau = over / o->mov_area;
    o->tau_abs = over_abs;
    if (gamma_mode == 1) o->gamma = gamma_of(o, o->tau);
    for (int i = 0; i < n; ++i) {
        o->xf[i] = (float)o->x[i];
        o->yf[i] = (float)o->y[i];
    }
    /* WA in FP64 on the double positions (or_wa_grad reads float; use a local copy) */
    {
        int32_t np = o->net_ptr[o->n_nets];
        double *px = dalloc((size_t)np), *py = dalloc((size_t)np);
        /* per-net terms summed in net order afterwards: the same sum for any
         * thread count and schedule (HPWL drives the lambda update, so a
         * run-dependent last bit would move the loop's trajectory) */
        double *hpn = dalloc((size_t)o->n_nets + 1), *wan = dalloc((size_t)o->n_nets + 1);
#pragma omp parallel for schedule(dynamic, 512)
        for (int e = 0; e < o->n_nets; ++e) {
            int s = o->net_ptr[e], dg = o->net_ptr[e + 1] - s;
            hpn[e] = wan[e] = 0.0;
            if (dg < 2) continue;
            double bxl[64], byl[64];
            double *bx = dg <= 64 ? bxl : dalloc((size_t)dg), *by = dg <= 64 ? byl : dalloc((size_t)dg);
            double xmx = -1e300, xmn = 1e300, ymx = -1e300, ymn = 1e300;
            for (int j = 0; j < dg; ++j) {
                bx[j] = o->x[o->pin_node[s + j]];
                by[j] = o->y[o->pin_node[s + j]];
                xmx = fmax(xmx, bx[j]); xmn = fmin(xmn, bx[j]);
                ymx = fmax(ymx, by[j]); ymn = fmin(ymn, by[j]);
            }
            hpn[e] = (xmx - xmn) + (ymx - ymn);
            wan[e] = wa_net_axis(dg, bx, o->gamma, px + s);
            wan[e] += wa_net_axis(dg, by, o->gamma, py + s);
            if (dg > 64) { free(bx); free(by); }
        }
        double wa = 0, hp = 0;
        for (int e = 0; e < o->n_nets; ++e) {
            hp += hpn[e];
            wa += wan[e];
        }
        free(hpn);
        free(wan);
        for (int i = 0; i < n; ++i) o->wlx[i] = o->wly[i] = 0;
        for (int32_t q = 0; q < np; ++q) {
            o->wlx[o->pin_node[q]] += px[q];
            o->wly[o->pin_node[q]] += py[q];
        }
        free(px);
        free(py);
        o->wa = wa;
        o->hpwl = hp;
    }
    if (gamma_mode == 2) o->gamma = gamma_of(o, o->tau);
    if (or_field_solve_fft(o->p.mx, o->p.my, o->bh / o->bw, o->d, NULL, o->ex, o->ey) != 0)
        or_field_solve(o->p.mx, o->p.my, o->bh / o->bw, o->d, NULL, o->ex, o->ey);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < o->n_mov; ++i) {
        gather_ctx g = {o->ex, o->ey, 0.0, 0.0, 1.0 / o->ab};
        node_overlaps(o, o->x[i], o->y[i], o->w[i], o->h[i], gather_cb, &g);
        o->fx[i] = g.fx;
        o->fy[i] = g.fy;
    }
    double nw = 0, nf = 0;
    for (int i = 0; i < o->n_mov; ++i) {
        nw += fabs(o->wlx[i]) + fabs(o->wly[i]);
        nf += fabs(o->fx[i]) + fabs(o->fy[i]);
    }
    o->norm_wl = nw;
    o->norm_f = nf;
}

/* preconditioned gradient of f = WL + lambda * D at the evaluated point;
 * dD/dx_i = -F_i; H_i = max(1, pins_i + lambda * area_i / A_b) */
static void precond_grad(or_placer *o, double *gx, double *gy) {
    for (int i = 0; i < o->n_mov; ++i) {
        double hdiag = o->pins[i] + o->lambda * ((double)o->w[i] * o->h[i]) / o->ab;
        if (hdiag < 1.0) hdiag = 1.0;
        gx[i] = (o->wlx[i] - o->lambda * o->fx[i]) / hdiag;
        gy[i] = (o->wly[i] - o->lambda * o->fy[i]) / hdiag;
    }
}

static double clampd(double v, double lo, double hi) { return v < lo ? lo : (v > hi ? hi : v); }

or_placer *or_create(int n_nodes, int n_nets, const int32_t *net_ptr, const int32_t *pin_node,
                     const float *w, const float *h, const float *x, const float *y,
                     const uint8_t *fixed, float die_w, float die_h, const or_params *p) {
    or_placer *o = (or_placer *)calloc(1, sizeof(or_placer));
    o->n_nodes = n_nodes;
    o->n_nets = n_nets;
    o->p = *p;
    int32_t np = net_ptr[n_nets];
    o->net_ptr = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n_nets + 1));
    o->pin_node = (int32_t *)malloc(sizeof(int32_t) * (size_t)(np ? np : 1));
    memcpy(o->net_ptr, net_ptr, sizeof(int32_t) * (size_t)(n_nets + 1));
    memcpy(o->pin_node, pin_node, sizeof(int32_t) * (size_t)np);
    o->w = (float *)malloc(sizeof(float) * (size_t)n_nodes);
    o->h = (float *)malloc(sizeof(float) * (size_t)n_nodes);
    o->fixed = (uint8_t *)calloc((size_t)n_nodes, 1);
    memcpy(o->w, w, sizeof(float) * (size_t)n_nodes);
    memcpy(o->h, h, sizeof(float) * (size_t)n_nodes);
    if (fixed) memcpy(o->fixed, fixed, (size_t)n_nodes);
    /* the loop expects movable nodes first (the synthetic generator's order) */
    o->n_mov = 0;
    while (o->n_mov < n_nodes && !o->fixed[o->n_mov]) o->n_mov++;
    o->xf = (float *)malloc(sizeof(float) * (size_t)n_nodes);
    o->yf = (float *)malloc(sizeof(float) * (size_t)n_nodes);
    o->x = dalloc((size_t)n_nodes);
    o->y = dalloc((size_t)n_nodes);
    for (int i = 0; i < n_nodes; ++i) {
        o->x[i] = x[i];
        o->y[i] = y[i];
    }
    size_t m = (size_t)(o->n_mov ? o->n_mov : 1);
    o->ux = dalloc(m); o->uy = dalloc(m); o->vpx = dalloc(m); o->vpy = dalloc(m);
    o->gx = dalloc(m); o->gy = dalloc(m); o->gpx = dalloc(m); o->gpy = dalloc(m);
    o->wlx = dalloc((size_t)n_nodes); o->wly = dalloc((size_t)n_nodes);
    o->fx = dalloc(m); o->fy = dalloc(m);
    o->pins = (int *)calloc((size_t)n_nodes, sizeof(int));
    for (int e = 0; e < n_nets; ++e)
        if (net_ptr[e + 1] - net_ptr[e] >= 2)
            for (int q = net_ptr[e]; q < net_ptr[e + 1]; ++q) o->pins[pin_node[q]]++;
    const int nb = p->mx * p->my;
    o->rho = dalloc((size_t)nb); o->fixmap = dalloc((size_t)nb); o->d = dalloc((size_t)nb);
    o->ex = dalloc((size_t)nb); o->ey = dalloc((size_t)nb);
    o->die_w = die_w;
    o->die_h = die_h;
    o->bw = (double)die_w / p->mx;
    o->bh = (double)die_h / p->my;
    o->ab = o->bw * o->bh;
    o->mov_area = 0;
    for (int i = 0; i < o->n_mov; ++i) o->mov_area += (double)w[i] * h[i];
    for (int i = o->n_mov; i < n_nodes; ++i)
        node_overlaps(o, x[i], y[i], w[i], h[i], add_cb, o->fixmap);
    o->ref_dh = p->ref_delta_hpwl > 0 ? p->ref_delta_hpwl : 0.1 * n_nets * o->bw;
    return o;
}

void or_init(or_placer *o, const float *x, const float *y) {
    const int m = o->n_mov;
    for (int i = 0; i < m; ++i) {
        o->x[i] = clampd(x[i], 0.0, o->die_w - o->w[i]);
        o->y[i] = clampd(y[i], 0.0, o->die_h - o->h[i]);
    }
    evaluate(o, 1);
    double swl = 0, sf = 0;
    for (int i = 0; i < m; ++i) {
        swl += fabs(o->wlx[i]) + fabs(o->wly[i]);
        sf += fabs(o->fx[i]) + fabs(o->fy[i]);
    }
    o->lambda = sf > 0 ? o->p.init_density_weight * swl / sf : o->p.init_density_weight;
    precond_grad(o, o->gx, o->gy);
    /* v_{-1} = v_0 - s g_0 with the largest move init_step_coef bins */
    double gmax = 0;
    for (int i = 0; i < m; ++i) gmax = fmax(gmax, fmax(fabs(o->gx[i]), fabs(o->gy[i])));
    double s = gmax > 0 ? o->p.init_step_coef * o->bw / gmax : 0.0;
    for (int i = 0; i < m; ++i) {
        o->ux[i] = o->x[i];
        o->uy[i] = o->y[i];
        o->vpx[i] = clampd(o->x[i] - s * o->gx[i], 0.0, o->die_w - o->w[i]);
        o->vpy[i] = clampd(o->y[i] - s * o->gy[i], 0.0, o->die_h - o->h[i]);
    }
    double hp0 = o->hpwl, wa0 = o->wa, tau0 = o->tau, tabs0 = o->tau_abs;
    /* gradient at v_{-1} with lambda_0, gamma_0 */
    for (int i = 0; i < m; ++i) {
        double t = o->x[i]; o->x[i] = o->vpx[i]; o->vpx[i] = t;
        t = o->y[i]; o->y[i] = o->vpy[i]; o->vpy[i] = t;
    }
    evaluate(o, 0);
    precond_grad(o, o->gpx, o->gpy);
    for (int i = 0; i < m; ++i) {
        double t = o->x[i]; o->x[i] = o->vpx[i]; o->vpx[i] = t;
        t = o->y[i]; o->y[i] = o->vpy[i]; o->vpy[i] = t;
    }
    o->hpwl = o->hpwl_prev = hp0;
    o->wa = wa0;
    o->tau = tau0;
    o->tau_abs = tabs0;
    o->a = 1.0;
    o->alpha = lipschitz_step(o, o->x, o->y, o->vpx, o->vpy, o->gx, o->gy, o->gpx, o->gpy);
    o->iteration = 0;
    o->evals = 0;
    o->restarts = 0;
}

/* ||v - vk|| / ||g - gk|| over movable nodes */
static double lipschitz_step(const or_placer *o, const double *vx, const double *vy, const double *kx,
                             const double *ky, const double *gx, const double *gy, const double *hx,
                             const double *hy) {
    double dv = 0, dg = 0;
    for (int i = 0; i < o->n_mov; ++i) {
        double a = vx[i] - kx[i], b = vy[i] - ky[i];
        double c = gx[i] - hx[i], e = gy[i] - hy[i];
        dv += a * a + b * b;
        dg += c * c + e * e;
    }
    return dg > 0 ? sqrt(dv) / sqrt(dg) : 0.0;
}

/* One accepted iteration per count.  Each trial steps from the accepted
 * state (u_k, v_k, g_k) with the predicted alpha, evaluates the gradient at
 * the new reference point and re-predicts alpha from the two points; a
 * prediction below 0.95 of the alpha used redoes the step with it (ePlace
 * steplength prediction with backtracking, at most max_backtracks redos). */
void or_step(or_placer *o, int n) {
    const int m = o->n_mov;
    for (int it = 0; it < n; ++it) {
        const double a_next = (1.0 + sqrt(4.0 * o->a * o->a + 1.0)) / 2.0;
        const double mom = (o->a - 1.0) / a_next;
        /* accepted v_k into vpx; trial gradient into gpx; trial u into fx/fy scratch */
        memcpy(o->vpx, o->x, sizeof(double) * (size_t)m);
        memcpy(o->vpy, o->y, sizeof(double) * (size_t)m);
        double *tux = dalloc((size_t)m), *tuy = dalloc((size_t)m);
        double alpha = o->alpha, ahat = alpha;
        for (int bt = 0; bt <= o->p.max_backtracks; ++bt) {
            for (int i = 0; i < m; ++i) {
                double nux = clampd(o->vpx[i] - alpha * o->gx[i], 0.0, o->die_w - o->w[i]);
                double nuy = clampd(o->vpy[i] - alpha * o->gy[i], 0.0, o->die_h - o->h[i]);
                tux[i] = nux;
                tuy[i] = nuy;
                o->x[i] = clampd(nux + mom * (nux - o->ux[i]), 0.0, o->die_w - o->w[i]);
                o->y[i] = clampd(nuy + mom * (nuy - o->uy[i]), 0.0, o->die_h - o->h[i]);
            }
            evaluate(o, 2);
            precond_grad(o, o->gpx, o->gpy);
            o->evals++;
            ahat = lipschitz_step(o, o->x, o->y, o->vpx, o->vpy, o->gpx, o->gpy, o->gx, o->gy);
            if (ahat > 0.95 * alpha || bt == o->p.max_backtracks) break;
            alpha = ahat;
        }
        /* adaptive restart (O'Donoghue & Candes 2015, gradient scheme): the
         * momentum sequence restarts when the accepted major step points uphill
         * along the gradient it was taken from, <g_k, u_{k+1} - u_k> > 0 */
        double uphill = 0.0, du = 0.0;
        for (int i = 0; i < m; ++i) {
            uphill += o->gx[i] * (tux[i] - o->ux[i]) + o->gy[i] * (tuy[i] - o->uy[i]);
            du += (tux[i] - o->ux[i]) * (tux[i] - o->ux[i]) + (tuy[i] - o->uy[i]) * (tuy[i] - o->uy[i]);
        }
        if (o->p.restart == 3) uphill = du < o->du_prev ? 1.0 : -1.0;       /* speed restart */
        if (o->p.restart == 4) uphill = o->tau > o->tau_prev ? 1.0 : -1.0;  /* overflow rose */
        o->du_prev = du;
        o->tau_prev = o->tau;
        memcpy(o->ux, tux, sizeof(double) * (size_t)m);
        memcpy(o->uy, tuy, sizeof(double) * (size_t)m);
        memcpy(o->gx, o->gpx, sizeof(double) * (size_t)m);
        memcpy(o->gy, o->gpy, sizeof(double) * (size_t)m);
        free(tux);
        free(tuy);
        o->alpha = ahat;
        o->a = (o->p.restart == 2 || (o->p.restart && uphill > 0.0)) ? 1.0 : a_next;
        if (o->p.restart && uphill > 0.0) o->restarts++;
        /* lambda update (RePlAce NesterovPlace): mu = mu_max^(1 - dHPWL/ref), in [mu_min, mu_max] */
        double pc = (o->hpwl - o->hpwl_prev) / o->ref_dh;
        double mu = pc < 0 ? o->p.mu_max : pow(o->p.mu_max, 1.0 - pc);
        if (mu < o->p.mu_min) mu = o->p.mu_min;
        if (mu > o->p.mu_max) mu = o->p.mu_max;
        o->lambda *= mu;
        /* capped where the density term dominates completely: keeps the
         * CUDA path's FP32 products finite when the target overflow is out
         * of reach and lambda would otherwise grow 5% per iteration forever */
        if (o->lambda > OR_LAMBDA_MAX) o->lambda = OR_LAMBDA_MAX;
        o->hpwl_prev = o->hpwl;
        o->iteration++;
    }
}

void or_get_stats(const or_placer *o, or_stats *s) {
    s->iteration = o->iteration;
    s->hpwl = o->hpwl;
    s->wa = o->wa;
    s->overflow = o->tau;
    s->overflow_abs = o->tau_abs;
    s->lambda = o->lambda;
    s->gamma = o->gamma;
    s->alpha = o->alpha;
    s->a_k = o->a;
    s->evals = o->evals;
    s->norm_wl = o->norm_wl;
    s->norm_f = o->norm_f;
    s->restarts = o->restarts;
}

void or_get_positions(const or_placer *o, float *x, float *y) {
    for (int i = 0; i < o->n_nodes; ++i) {
        x[i] = (float)o->x[i];
        y[i] = (float)o->y[i];
    }
}

void or_destroy(or_placer *o) {
    if (!o) return;
    free(o->net_ptr); free(o->pin_node); free(o->w); free(o->h); free(o->fixed);
    free(o->xf); free(o->yf); free(o->x); free(o->y);
    free(o->ux); free(o->uy); free(o->vpx); free(o->vpy); free(o->gx); free(o->gy);
    free(o->gpx); free(o->gpy); free(o->wlx); free(o->wly); free(o->fx); free(o->fy);
    free(o->pins); free(o->rho); free(o->fixmap); free(o->d); free(o->ex); free(o->ey);
    free(o);
}
