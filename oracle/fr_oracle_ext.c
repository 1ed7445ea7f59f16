/*
 * fr_oracle_ext.c -- CPU oracle for the components that have no counterpart
 * in the reference: analytic DCF, degridding, Pipe-Menon DCF, sample-density
 * features and the DCF network.
 *
 * TEST INFRASTRUCTURE ONLY (same status as fr_oracle.c): the tests use it as
 * the checker; the product library never links, loads or calls it.
 *
 * Geometry is the reference's gridding geometry (GridLut.cpp:98-136: clamped
 * cell range, LUT index of the float distance), shared with fr_oracle.c, so a
 * degridding is the exact adjoint of orc_grid_channel_f64.  Arithmetic is in
 * double.  The published algorithms restated here:
 *   - Pipe & Menon, "Sampling density compensation in MRI: rationale and an
 *     iterative numerical solution", MRM 41:179-186 (1999): w <- w / (C w)
 *     with C w = degrid(grid(w)) on the same convolution kernel.
 *   - a fully connected network 5 -> 64 -> 64 -> 1 with tanh activations,
 *     mean squared error, reverse-mode gradients.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "fr_oracle.h"

/* float -> int as the x86 conversion the reference runs on: out-of-range and
 * NaN give INT_MIN (same rule as fr_oracle.c). */
static int f2i(float v)
{
    if (!(v >= -2147483648.0f && v < 2147483648.0f)) return (int)0x80000000u;
    return (int)v;
}

/* GridLut.cpp:100-105: start = max(ceil(c - hw), 0), end = min(floor(c + hw), G-1). */
static void cell_range(float c, float kHW, unsigned G, int *s, int *e)
{
    int st = f2i(ceilf(c - kHW));
    int en = f2i(floorf(c + kHW));
    *s = st > 0 ? st : 0;
    *e = en < (int)G - 1 ? en : (int)G - 1;
}

void orc_dcf_analytic(const float *traj, size_t n, int dim, double power, float *out)
{
    for (size_t s = 0; s < n; ++s) {
        double q = 0;
        for (int d = 0; d < dim; ++d) q += (double)traj[4 * s + d] * (double)traj[4 * s + d];
        double k = sqrt(q);
        double w = power == 1.0 ? k : (power == 2.0 ? k * k : pow(k, power));
        out[s] = (float)w;
    }
}

/* Visit the taps of sample s: calls body(cell, weight) for each valid tap. */
#define FOR_TAPS(traj, s, dim, G, kHW, lut, klength, BODY)                                      \
    do {                                                                                        \
        float c_[3] = {0, 0, 0};                                                                \
        int st_[3] = {0, 0, 0}, en_[3] = {0, 0, 0};                                             \
        for (int i_ = 0; i_ < (dim); ++i_) {                                                    \
            c_[i_] = (traj)[4 * (s) + i_];                                                      \
            cell_range(c_[i_], (kHW), (G), &st_[i_], &en_[i_]);                                 \
        }                                                                                       \
        for (int z_ = st_[2]; z_ <= en_[2]; z_++)                                               \
            for (int y_ = st_[1]; y_ <= en_[1]; y_++) {                                         \
                size_t row_ = ((size_t)z_ * (G) + (size_t)y_) * (G);                            \
                for (int x_ = st_[0]; x_ <= en_[0]; x_++) {                                     \
                    int ki_ = orc_tap_lut_index((float)x_ - c_[0], (float)y_ - c_[1],           \
                                                (float)z_ - c_[2], (kHW), (klength));           \
                    if (ki_ >= 0) {                                                             \
                        size_t cell = row_ + (size_t)x_;                                        \
                        double wt = (double)(lut)[ki_];                                         \
                        BODY;                                                                   \
                    }                                                                           \
                }                                                                               \
            }                                                                                   \
    } while (0)

void orc_degrid_f64(const float *traj, size_t n, int dim, unsigned G, float kWidth, const float *lut,
                    int klength, const double *grid, int channels, double *out)
{
    const float kHW = kWidth / 2;
    const size_t cells = dim == 3 ? (size_t)G * G * G : (size_t)G * G;
    for (int c = 0; c < channels; ++c) {
        const double *g = grid + 2 * cells * (size_t)c;
        for (size_t s = 0; s < n; ++s) {
            double re = 0, im = 0;
            FOR_TAPS(traj, s, dim, G, kHW, lut, klength, {
                re += wt * g[2 * cell];
                im += wt * g[2 * cell + 1];
            });
            out[2 * ((size_t)c * n + s)] = re;
            out[2 * ((size_t)c * n + s) + 1] = im;
        }
    }
}

void orc_grid_real_f64(const float *traj, const double *w, size_t n, int dim, unsigned G, float kWidth,
                       const float *lut, int klength, double *grid)
{
    const float kHW = kWidth / 2;
    const size_t cells = dim == 3 ? (size_t)G * G * G : (size_t)G * G;
    memset(grid, 0, cells * sizeof(double));
    for (size_t s = 0; s < n; ++s) {
        const double v = w[s];
        FOR_TAPS(traj, s, dim, G, kHW, lut, klength, { grid[cell] += wt * v; });
    }
}

int orc_dcf_pipe_f64(const float *traj, size_t n, int dim, unsigned G, float kWidth, const float *lut,
                     int klength, int iterations, double *w)
{
    const float kHW = kWidth / 2;
    const size_t cells = dim == 3 ? (size_t)G * G * G : (size_t)G * G;
    double *g = (double *)malloc(cells * sizeof(double));
    if (!g) return -2;
    for (int it = 0; it < iterations; ++it) {
        orc_grid_real_f64(traj, w, n, dim, G, kWidth, lut, klength, g);
        for (size_t s = 0; s < n; ++s) {
            double p = 0;
            FOR_TAPS(traj, s, dim, G, kHW, lut, klength, { p += wt * g[cell]; });
            /* a sample without taps keeps its weight */
            if (p > 0) w[s] = w[s] / p;
        }
    }
    free(g);
    return 0;
}

/* Nearest cell of a normalised coordinate, clamped to [0, G-1]. */
static int nearest_cell(float x, unsigned G)
{
    int c = f2i(floorf(x + 0.5f));
    if (c < 0) c = 0;
    if (c > (int)G - 1) c = (int)G - 1;
    return c;
}

int orc_density_counts(const float *traj, size_t n, int dim, unsigned G, const int *radii, int nradii,
                       int *counts)
{
    const size_t cells = dim == 3 ? (size_t)G * G * G : (size_t)G * G;
    int *hist = (int *)calloc(cells, sizeof(int));
    if (!hist) return -2;
    int *cell_of = (int *)malloc(n * 3 * sizeof(int));
    if (!cell_of) {
        free(hist);
        return -2;
    }
    for (size_t s = 0; s < n; ++s) {
        int c[3] = {0, 0, 0};
        for (int d = 0; d < dim; ++d) c[d] = nearest_cell(traj[4 * s + d], G);
        for (int d = 0; d < 3; ++d) cell_of[3 * s + d] = c[d];
        hist[((size_t)c[2] * G + (size_t)c[1]) * G + (size_t)c[0]]++;
    }
    const int Gz = dim == 3 ? (int)G : 1;
    for (size_t s = 0; s < n; ++s) {
        for (int k = 0; k < nradii; ++k) {
            const int r = radii[k];
            int lo[3], hi[3];
            for (int d = 0; d < 3; ++d) {
                const int lim = d < 2 ? (int)G - 1 : Gz - 1;
                lo[d] = cell_of[3 * s + d] - r;
                hi[d] = cell_of[3 * s + d] + r;
                if (lo[d] < 0) lo[d] = 0;
                if (hi[d] > lim) hi[d] = lim;
            }
            if (dim == 2) lo[2] = hi[2] = 0;
            long long sum = 0;
            for (int z = lo[2]; z <= hi[2]; ++z)
                for (int y = lo[1]; y <= hi[1]; ++y)
                    for (int x = lo[0]; x <= hi[0]; ++x) sum += hist[((size_t)z * G + (size_t)y) * G + (size_t)x];
            counts[s * (size_t)nradii + k] = (int)sum;
        }
    }
    free(cell_of);
    free(hist);
    return 0;
}

void orc_dcf_features(const int *counts, const float *raw_traj, size_t n, int dim, const int *radii, int nradii,
                      float kmax, float *feat)
{
    const int nf = nradii + 1;
    for (size_t s = 0; s < n; ++s) {
        for (int k = 0; k < nradii; ++k) {
            const float side = (float)(2 * radii[k] + 1);
            const float vol = dim == 3 ? side * side * side : side * side;
            feat[s * nf + k] = logf((float)counts[s * (size_t)nradii + k] / vol);
        }
        float q = 0.f;
        for (int d = 0; d < dim; ++d) q += raw_traj[4 * s + d] * raw_traj[4 * s + d];
        feat[s * nf + nradii] = logf(sqrtf(q) / kmax + 0.0009765625f);
    }
}

/* ---- network 5 -> 64 -> 64 -> 1, tanh ---------------------------------- */

/* Parameter layout (ORC_MLP_PARAMS floats):
 * W1[64][5] | b1[64] | W2[64][64] | b2[64] | W3[64] | b3 */
#define NI ORC_MLP_IN
#define NH ORC_MLP_HIDDEN
#define OFF_W1 0
#define OFF_B1 (OFF_W1 + NH * NI)
#define OFF_W2 (OFF_B1 + NH)
#define OFF_B2 (OFF_W2 + NH * NH)
#define OFF_W3 (OFF_B2 + NH)
#define OFF_B3 (OFF_W3 + NH)

static double forward1(const float *p, const float *x, double *h1, double *h2)
{
    for (int j = 0; j < NH; ++j) {
        double a = p[OFF_B1 + j];
        for (int i = 0; i < NI; ++i) a += (double)p[OFF_W1 + j * NI + i] * (double)x[i];
        h1[j] = tanh(a);
    }
    for (int j = 0; j < NH; ++j) {
        double a = p[OFF_B2 + j];
        for (int i = 0; i < NH; ++i) a += (double)p[OFF_W2 + j * NH + i] * h1[i];
        h2[j] = tanh(a);
    }
    double y = p[OFF_B3];
    for (int i = 0; i < NH; ++i) y += (double)p[OFF_W3 + i] * h2[i];
    return y;
}

void orc_mlp_forward(const float *params, const float *x, size_t n, double *y)
{
    double h1[NH], h2[NH];
    for (size_t s = 0; s < n; ++s) y[s] = forward1(params, x + s * NI, h1, h2);
}

void orc_mlp_forward_residual(const float *params, const float *x, size_t n, double *y)
{
    double h1[NH], h2[NH];
    for (size_t s = 0; s < n; ++s) y[s] = forward1(params, x + s * NI, h1, h2) - (double)x[s * NI + 1];
}

double orc_mlp_backward(const float *params, const float *x, const float *target, const float *weight, size_t n,
                        double *grad)
{
    memset(grad, 0, ORC_MLP_PARAMS * sizeof(double));
    double h1[NH], h2[NH], d2[NH], d1[NH];
    double loss = 0;
    const double inv = n ? 1.0 / (double)n : 0.0;
    for (size_t s = 0; s < n; ++s) {
        const float *xs = x + s * NI;
        const double y = forward1(params, xs, h1, h2);
        const double r = y - (double)target[s];
        const double c = weight ? (double)weight[s] : 1.0;
        loss += c * r * r * inv;
        const double dy = 2.0 * c * r * inv;
        grad[OFF_B3] += dy;
        for (int i = 0; i < NH; ++i) {
            grad[OFF_W3 + i] += dy * h2[i];
            d2[i] = dy * (double)params[OFF_W3 + i] * (1.0 - h2[i] * h2[i]);
        }
        for (int j = 0; j < NH; ++j) {
            grad[OFF_B2 + j] += d2[j];
            for (int i = 0; i < NH; ++i) grad[OFF_W2 + j * NH + i] += d2[j] * h1[i];
        }
        for (int i = 0; i < NH; ++i) {
            double a = 0;
            for (int j = 0; j < NH; ++j) a += (double)params[OFF_W2 + j * NH + i] * d2[j];
            d1[i] = a * (1.0 - h1[i] * h1[i]);
        }
        for (int j = 0; j < NH; ++j) {
            grad[OFF_B1 + j] += d1[j];
            for (int i = 0; i < NI; ++i) grad[OFF_W1 + j * NI + i] += d1[j] * (double)xs[i];
        }
    }
    return loss;
}
