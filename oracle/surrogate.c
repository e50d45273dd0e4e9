/*
 * surrogate.c -- FP64 restatement of the learned field surrogate's network
 * and loss (aieplace_gb300/csrc/k_surrogate.cu: conv_fwd_kernel,
 * conv_bwd_data_kernel, conv_bwd_weight_kernel, mse_kernel) and of its data
 * preparation (pool_kernel, prep_kernel, target_kernel, combine_kernel).
 *
 * TEST INFRASTRUCTURE ONLY: the checker of the GPU forward/backward kernels
 * (gradient check) and of the input/target layout.  Plain loops.
 *
 * Network: 4 layers; layer l maps cin_l -> cout_l channels with a k_l x k_l
 * kernel (zero padding, stride 1), ReLU on layers 0..2.  Parameters are one
 * flat vector: per layer W[cout][cin][k][k] then b[cout].  Tensors are
 * [batch][channel][x][y], y fastest.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define NL 4

typedef struct {
    int cin, cout, k, relu;
    long w_off, b_off;
} layer_t;

static long layout(int cin0, int width, int cout, const int *k, layer_t *L) {
    long off = 0;
    for (int l = 0; l < NL; ++l) {
        L[l].cin = l == 0 ? cin0 : width;
        L[l].cout = l == NL - 1 ? cout : width;
        L[l].k = k[l];
        L[l].relu = l < NL - 1;
        L[l].w_off = off;
        off += (long)L[l].cout * L[l].cin * k[l] * k[l];
        L[l].b_off = off;
        off += L[l].cout;
    }
    return off;
}

int or_surr_num_params(int cin0, int width, int cout, const int *k) {
    layer_t L[NL];
    return (int)layout(cin0, width, cout, k, L);
}

static void conv(const layer_t *L, int B, int R, const double *p, const double *in, double *out) {
    const int h = L->k / 2;
    for (int b = 0; b < B; ++b)
        for (int co = 0; co < L->cout; ++co)
            for (int x = 0; x < R; ++x)
                for (int y = 0; y < R; ++y) {
                    double acc = p[L->b_off + co];
                    for (int ci = 0; ci < L->cin; ++ci)
                        for (int kx = 0; kx < L->k; ++kx)
                            for (int ky = 0; ky < L->k; ++ky) {
                                const int xx = x + kx - h, yy = y + ky - h;
                                if (xx < 0 || xx >= R || yy < 0 || yy >= R) continue;
                                acc += p[L->w_off + (((long)co * L->cin + ci) * L->k + kx) * L->k + ky] *
                                       in[(((long)b * L->cin + ci) * R + xx) * R + yy];
                            }
                    if (L->relu && acc < 0.0) acc = 0.0;
                    out[(((long)b * L->cout + co) * R + x) * R + y] = acc;
                }
}

/* y [B][cout][R][R] */
void or_surr_forward(int B, int R, int cin0, int width, int cout, const int *k, const double *p, const double *x,
                     double *y) {
    layer_t L[NL];
    layout(cin0, width, cout, k, L);
    const long RR = (long)R * R;
    double *a = (double *)malloc(sizeof(double) * B * width * RR);
    double *c = (double *)malloc(sizeof(double) * B * width * RR);
    conv(&L[0], B, R, p, x, a);
    conv(&L[1], B, R, p, a, c);
    conv(&L[2], B, R, p, c, a);
    conv(&L[3], B, R, p, a, y);
    free(a);
    free(c);
}

/* loss = mean over pixels >= margin from the edges of (y - t)^2; grad of loss
 * w.r.t. every parameter (backpropagation through the four layers) */
double or_surr_loss_grad(int B, int R, int cin0, int width, int cout, const int *k, const double *p, const double *x,
                         const double *t, int margin, double *grad) {
    layer_t L[NL];
    const long np = layout(cin0, width, cout, k, L);
    const long RR = (long)R * R;
    double *act[NL + 1];
    act[0] = (double *)x;
    for (int l = 0; l < NL; ++l) {
        act[l + 1] = (double *)malloc(sizeof(double) * B * L[l].cout * RR);
        conv(&L[l], B, R, p, act[l], act[l + 1]);
    }
    const int inner = R - 2 * margin;
    const double n = (double)B * cout * inner * inner;
    double loss = 0.0;
    double *g = (double *)malloc(sizeof(double) * B * cout * RR);
    for (int b = 0; b < B; ++b)
        for (int c = 0; c < cout; ++c)
            for (int xx = 0; xx < R; ++xx)
                for (int yy = 0; yy < R; ++yy) {
                    const long i = (((long)b * cout + c) * R + xx) * R + yy;
                    const int in = xx >= margin && xx < R - margin && yy >= margin && yy < R - margin;
                    const double d = in ? act[NL][i] - t[i] : 0.0;
                    loss += d * d;
                    g[i] = 2.0 * d / n;
                }
    loss /= n;
    memset(grad, 0, sizeof(double) * np);
    for (int l = NL - 1; l >= 0; --l) {
        const layer_t *Ly = &L[l];
        const int h = Ly->k / 2;
        /* gradient at the pre-activation */
        if (Ly->relu)
            for (long i = 0; i < (long)B * Ly->cout * RR; ++i)
                if (!(act[l + 1][i] > 0.0)) g[i] = 0.0;
        double *gin = l > 0 ? (double *)calloc((size_t)B * Ly->cin * RR, sizeof(double)) : NULL;
        for (int b = 0; b < B; ++b)
            for (int co = 0; co < Ly->cout; ++co)
                for (int xx = 0; xx < R; ++xx)
                    for (int yy = 0; yy < R; ++yy) {
                        const double go = g[(((long)b * Ly->cout + co) * R + xx) * R + yy];
                        if (go == 0.0) continue;
                        grad[Ly->b_off + co] += go;
                        for (int ci = 0; ci < Ly->cin; ++ci)
                            for (int kx = 0; kx < Ly->k; ++kx)
                                for (int ky = 0; ky < Ly->k; ++ky) {
                                    const int xi = xx + kx - h, yi = yy + ky - h;
                                    if (xi < 0 || xi >= R || yi < 0 || yi >= R) continue;
                                    const long wi = Ly->w_off + (((long)co * Ly->cin + ci) * Ly->k + kx) * Ly->k + ky;
                                    const long ii = (((long)b * Ly->cin + ci) * R + xi) * R + yi;
                                    grad[wi] += go * act[l][ii];
                                    if (gin) gin[ii] += go * p[wi];
                                }
                    }
        free(g);
        g = gin;
    }
    for (int l = 1; l <= NL; ++l) free(act[l]);
    return loss;
}

/* Data preparation for one M x M map with factor f (R = M / f):
 *   x0 [f^2 + 2][R][R]: sub-bin densities, then f ex_c / s, f ey_c / s
 *   given the coarse field (ex_c, ey_c) of the pooled density and s.
 * pooled [R][R] = mean of the f x f bins. */
void or_surr_pool(int M, int f, const double *d, double *pooled) {
    const int R = M / f;
    for (int I = 0; I < R; ++I)
        for (int J = 0; J < R; ++J) {
            double s = 0.0;
            for (int a = 0; a < f; ++a)
                for (int b = 0; b < f; ++b) s += d[(long)(I * f + a) * M + J * f + b];
            pooled[(long)I * R + J] = s / (f * f);
        }
}

static double bilinear(const double *c, int R, int f, int X, int Y) {
    const double u = (X + 0.5) / f - 0.5, v = (Y + 0.5) / f - 0.5;
    int i0 = (int)floor(u), j0 = (int)floor(v);
    double tu = u - floor(u), tv = v - floor(v);
    if (i0 < 0) { i0 = 0; tu = 0.0; }
    if (j0 < 0) { j0 = 0; tv = 0.0; }
    if (i0 >= R - 1) { i0 = R - 1; tu = 0.0; }
    if (j0 >= R - 1) { j0 = R - 1; tv = 0.0; }
    const int i1 = i0 + 1 < R ? i0 + 1 : R - 1, j1 = j0 + 1 < R ? j0 + 1 : R - 1;
    return (1 - tu) * ((1 - tv) * c[(long)i0 * R + j0] + tv * c[(long)i0 * R + j1]) +
           tu * ((1 - tv) * c[(long)i1 * R + j0] + tv * c[(long)i1 * R + j1]);
}

/* fine field of the coarse layer plus (y != NULL) the network residual */
void or_surr_combine(int M, int f, const double *cex, const double *cey, const double *y, double s, double *ex,
                     double *ey) {
    const int R = M / f, f2 = f * f;
    const long RR = (long)R * R;
    for (int X = 0; X < M; ++X)
        for (int Y = 0; Y < M; ++Y) {
            double vx = f * bilinear(cex, R, f, X, Y), vy = f * bilinear(cey, R, f, X, Y);
            if (y) {
                const int I = X / f, a = X % f, J = Y / f, b = Y % f;
                const long q = (long)I * R + J;
                vx += s * y[(long)(a * f + b) * RR + q];
                vy += s * y[(long)(f2 + a * f + b) * RR + q];
            }
            ex[(long)X * M + Y] = vx;
            ey[(long)X * M + Y] = vy;
        }
}
