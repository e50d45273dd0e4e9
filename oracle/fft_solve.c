/*
 * fft_solve.c -- the oracle's electrostatic solve in O(n^2 log n).
 *
 * TEST INFRASTRUCTURE ONLY (the timed CPU baseline and the oracle loop).
 *
 * or_field_solve_fft evaluates exactly the sums of or_field_solve (the
 * RePlAce doFFT conventions, python/AIEmath/fft_replace/fft.cpp:204-299:
 * DCT-II of the density, halved edge rows, 4/(Mx My), phi = a/(wx^2+wy^2),
 * Ex by sine-cosine and Ey by cosine-sine inverse transforms) with fast 1-D
 * transforms instead of dense n x n products.  It is checked against the
 * dense solve and against the reference's own Ooura solver output
 * (tests/golden/replace_field.npz); the dense solve stays the checker.
 *
 * Method (published, restated here in our own code):
 *   - DCT-II  X[k] = sum_j x[j] cos(pi k (j + 1/2) / n) through one n-point
 *     complex FFT of the even/odd reordered input v[j] = x[2j],
 *     v[n-1-j] = x[2j+1]:  X[k] = Re(exp(-i pi k / 2n) V[k])
 *     (J. Makhoul, "A fast cosine transform in one and two dimensions",
 *     IEEE Trans. ASSP 28(1):27-34, 1980);
 *   - its transpose, y[j] = sum_k c[k] cos(pi k (j + 1/2) / n), by running
 *     that map backwards: V[k] = exp(i pi k / 2n) (X[k] - i X[n-k]) with
 *     X = (2 c[0], c[1], ...), X[n] = 0, then y[2j] = Re v[j] / 2 and
 *     y[2j+1] = Re v[n-1-j] / 2 for v the unnormalised inverse DFT of V;
 *   - the sine sums s[j] = sum_k c[k] sin(pi k (j + 1/2) / n) from
 *     sin(pi k (j+1/2)/n) = (-1)^j cos(pi (n-k) (j+1/2)/n): the cosine sum
 *     of the reversed coefficients (c[n-1], ..., c[1] at 1..n-1, 0 at 0)
 *     with alternating output signs;
 *   - the complex FFT is the iterative radix-2 Cooley-Tukey algorithm with
 *     bit-reversed input order (n a power of two).
 * Rows run in parallel (OpenMP); columns are transposed to rows.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

#define FS_PI 3.14159265358979323846

typedef struct fs_plan {
    int n, log2n;
    int *rev;     /* bit reversal of 0..n-1 */
    double *twr;  /* cos(2 pi k / n), k < n/2 */
    double *twi;  /* -sin(2 pi k / n) (forward) */
    double *hcr;  /* cos(pi k / 2n), k < n */
    double *hci;  /* sin(pi k / 2n) */
} fs_plan;

static int fs_plan_init(fs_plan *p, int n) {
    memset(p, 0, sizeof(*p));
    if (n < 2 || (n & (n - 1))) return -1;
    p->n = n;
    while ((1 << p->log2n) < n) p->log2n++;
    p->rev = (int *)malloc(sizeof(int) * (size_t)n);
    p->twr = (double *)malloc(sizeof(double) * (size_t)(n / 2));
    p->twi = (double *)malloc(sizeof(double) * (size_t)(n / 2));
    p->hcr = (double *)malloc(sizeof(double) * (size_t)n);
    p->hci = (double *)malloc(sizeof(double) * (size_t)n);
    for (int i = 0; i < n; ++i) {
        int r = 0;
        for (int b = 0; b < p->log2n; ++b) r |= ((i >> b) & 1) << (p->log2n - 1 - b);
        p->rev[i] = r;
        p->hcr[i] = cos(FS_PI * i / (2.0 * n));
        p->hci[i] = sin(FS_PI * i / (2.0 * n));
    }
    for (int k = 0; k < n / 2; ++k) {
        p->twr[k] = cos(2.0 * FS_PI * k / n);
        p->twi[k] = -sin(2.0 * FS_PI * k / n);
    }
    return 0;
}

static void fs_plan_free(fs_plan *p) {
    free(p->rev);
    free(p->twr);
    free(p->twi);
    free(p->hcr);
    free(p->hci);
}

/* in-place complex DFT of (re, im), already in bit-reversed order;
 * sign -1: sum x[j] e^{-2 pi i jk/n}, +1: e^{+2 pi i jk/n} (no scaling) */
static void fs_fft_core(const fs_plan *p, double *re, double *im, int sign) {
    const int n = p->n;
    for (int len = 2; len <= n; len <<= 1) {
        const int half = len >> 1, step = n / len;
        for (int s = 0; s < n; s += len) {
            for (int k = 0; k < half; ++k) {
                const double wr = p->twr[k * step], wi = sign < 0 ? p->twi[k * step] : -p->twi[k * step];
                const int a = s + k, b = a + half;
                const double tr = re[b] * wr - im[b] * wi, ti = re[b] * wi + im[b] * wr;
                re[b] = re[a] - tr;
                im[b] = im[a] - ti;
                re[a] += tr;
                im[a] += ti;
            }
        }
    }
}

/* DCT-II of x (length n) into out; re, im scratch of n */
static void fs_dct2(const fs_plan *p, const double *x, double *out, double *re, double *im) {
    const int n = p->n;
    for (int j = 0; j < n / 2; ++j) {
        const int a = p->rev[j], b = p->rev[n - 1 - j];
        re[a] = x[2 * j];
        re[b] = x[2 * j + 1];
        im[a] = 0.0;
        im[b] = 0.0;
    }
    fs_fft_core(p, re, im, -1);
    for (int k = 0; k < n; ++k) out[k] = re[k] * p->hcr[k] + im[k] * p->hci[k];
}

/* y[j] = sum_k c[k] cos(pi k (j + 1/2) / n) */
static void fs_cos_sum(const fs_plan *p, const double *c, double *y, double *re, double *im) {
    const int n = p->n;
    for (int k = 0; k < n; ++k) {
        const double xk = k == 0 ? 2.0 * c[0] : c[k];
        const double xnk = k == 0 ? 0.0 : c[n - k];
        /* exp(i pi k / 2n) (xk - i xnk) */
        const double vr = p->hcr[k] * xk + p->hci[k] * xnk;
        const double vi = p->hci[k] * xk - p->hcr[k] * xnk;
        re[p->rev[k]] = vr;
        im[p->rev[k]] = vi;
    }
    fs_fft_core(p, re, im, +1);
    for (int j = 0; j < n / 2; ++j) {
        y[2 * j] = 0.5 * re[j];
        y[2 * j + 1] = 0.5 * re[n - 1 - j];
    }
}

/* s[j] = sum_k c[k] sin(pi k (j + 1/2) / n); t scratch of n */
static void fs_sin_sum(const fs_plan *p, const double *c, double *s, double *t, double *re, double *im) {
    const int n = p->n;
    t[0] = 0.0;
    for (int k = 1; k < n; ++k) t[k] = c[n - k];
    fs_cos_sum(p, t, s, re, im);
    for (int j = 1; j < n; j += 2) s[j] = -s[j];
}

enum { FS_DCT2 = 0, FS_COS = 1, FS_SIN = 2 };

/* applies a 1-D transform to every row of the n x n matrix a (in place) */
static void fs_rows(const fs_plan *p, double *a, int kind) {
    const int n = p->n;
#pragma omp parallel
    {
        double *re = (double *)malloc(sizeof(double) * (size_t)n * 4);
        double *im = re + n, *t = im + n, *o = t + n;
#pragma omp for schedule(static)
        for (int r = 0; r < n; ++r) {
            double *row = a + (size_t)r * n;
            if (kind == FS_DCT2)
                fs_dct2(p, row, o, re, im);
            else if (kind == FS_COS)
                fs_cos_sum(p, row, o, re, im);
            else
                fs_sin_sum(p, row, o, t, re, im);
            memcpy(row, o, sizeof(double) * (size_t)n);
        }
        free(re);
    }
}

static void fs_transpose(int n, const double *in, double *out) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i += 32)
        for (int j = 0; j < n; j += 32)
            for (int ii = i; ii < i + 32 && ii < n; ++ii)
                for (int jj = j; jj < j + 32 && jj < n; ++jj) out[(size_t)jj * n + ii] = in[(size_t)ii * n + jj];
}

/* out[x][y] = sum_u T_x[u][x] sum_v T_y[v][y] in[u][v], with T the
 * transforms of kind_x (along the first index) and kind_y (second) */
static void fs_separable(const fs_plan *p, const double *in, double *out, double *tmp, int kind_x, int kind_y) {
    const int n = p->n;
    memcpy(tmp, in, sizeof(double) * (size_t)n * n);
    fs_rows(p, tmp, kind_y);   /* along the second index */
    fs_transpose(n, tmp, out); /* out[v'][u] */
    fs_rows(p, out, kind_x);   /* along the first index */
    fs_transpose(n, out, tmp);
    memcpy(out, tmp, sizeof(double) * (size_t)n * n);
}

int or_field_solve_fft(int mx, int my, double bin_ratio, const double *d, double *phi, double *ex, double *ey) {
    const int n = mx;
    if (mx != my) return -1;
    fs_plan p;
    if (fs_plan_init(&p, n) != 0) return -1;
    const size_t nn = (size_t)n * n;
    double *a = (double *)malloc(sizeof(double) * nn), *tmp = (double *)malloc(sizeof(double) * nn);
    double *pc = (double *)malloc(sizeof(double) * nn), *exc = (double *)malloc(sizeof(double) * nn);
    double *eyc = (double *)malloc(sizeof(double) * nn);
    /* a[u][v] = sum_x sum_y cos(pi u (x+1/2)/n) cos(pi v (y+1/2)/n) d[x][y] */
    fs_separable(&p, d, a, tmp, FS_DCT2, FS_DCT2);
    /* scaling, potential and field coefficients: the arithmetic of or_field_solve */
    for (int u = 0; u < n; ++u) {
        const double wx = FS_PI * u / n;
        for (int v = 0; v < n; ++v) {
            const double wy = FS_PI * v / n * bin_ratio;
            const size_t k = (size_t)u * n + v;
            double c = a[k];
            if (u == 0) c *= 0.5;
            if (v == 0) c *= 0.5;
            c = c * (4.0 / n / n);
            if (u == 0 && v == 0) {
                pc[k] = exc[k] = eyc[k] = 0.0;
            } else {
                const double q = c / (wx * wx + wy * wy);
                pc[k] = q;
                exc[k] = q * wx;
                eyc[k] = q * wy;
            }
        }
    }
    fs_separable(&p, exc, ex, tmp, FS_SIN, FS_COS); /* Ex: sine along x, cosine along y */
    fs_separable(&p, eyc, ey, tmp, FS_COS, FS_SIN); /* Ey: cosine along x, sine along y */
    if (phi) fs_separable(&p, pc, phi, tmp, FS_COS, FS_COS);
    free(a);
    free(tmp);
    free(pc);
    free(exc);
    free(eyc);
    fs_plan_free(&p);
    return 0;
}
