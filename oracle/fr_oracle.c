/*
 * fr_oracle.c -- CPU oracle for the fastrecon gridding/recon path.
 *
 * TEST INFRASTRUCTURE ONLY (checker and timed CPU baseline).  Plain-C
 * restatement of the reference CPU code of pengwg/fastrecon; every function
 * cites the reference file:line it follows.  Compile with
 * -ffp-contract=off so no multiply-add is fused, which is what the
 * reference's own x86-64 build does (no FMA without -mfma).
 */
#include "fr_oracle.h"

#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ---------------------------------------------------------------------- */
/* Kaiser-Bessel LUT                                                       */
/* ---------------------------------------------------------------------- */

double orc_bessel_i0(double x)
{
    /* I0(x) = sum_k ((x/2)^2)^k / (k!)^2, all terms positive (A&S 9.6.12). */
    if (isnan(x))
        return x;
    double q = 0.25 * x * x;
    double term = 1.0, sum = 1.0;
    for (int k = 1; k < 1000; ++k) {
        term *= q / ((double)k * (double)k);
        sum += term;
        if (term < sum * 1e-18)
            break;
    }
    return sum;
}

/* ConvKernel::ConvKernel, ConvKernel.cpp:7-30.  The float/double mix of the
 * reference is kept operation by operation. */
int orc_kb_lut(float kWidth, float overGridFactor, int length, float *out)
{
    if (length < 2 || out == NULL)
        return -1;
    float w = kWidth;
    float a = overGridFactor;
    /* ConvKernel.cpp:14: w*w/(a*a) is float, (a - 0.5) is double. */
    float wa = w * w / (a * a);
    float beta = (float)(M_PI * sqrt((double)wa * ((double)a - 0.5) * ((double)a - 0.5) - 0.8));
    /* ConvKernel.cpp:16: w / 2.0 / (length - 1) in double, stored float. */
    float dk = (float)((double)w / 2.0 / (double)(length - 1));
    float kernel0 = 1;
    for (int i = 0; i < length; i++) {
        float k = dk * (float)i;                        /* :20 */
        float r = 2 * k / w;                             /* :21, float */
        double x = (double)beta * sqrt(1 - (double)r * (double)r);
        out[i] = (float)(orc_bessel_i0(x) / (double)w); /* :23 */
        if (i == 0)
            kernel0 = out[0];                            /* :25 */
        out[i] /= kernel0;                               /* :26, float */
    }
    return 0;
}

/* ---------------------------------------------------------------------- */
/* Trajectory bounds and normalisation                                     */
/* ---------------------------------------------------------------------- */

/* ReconData::loadTraj bounds loop, ReconData.cpp:156-175. */
void orc_comp_bounds(const float *traj, size_t n, int dim, float *lo, float *hi)
{
    for (int i = 0; i < dim; ++i) {
        lo[i] = 3.402823466e+38F;
        hi[i] = -3.402823466e+38F;
    }
    for (size_t s = 0; s < n; ++s) {
        for (int i = 0; i < dim; ++i) {
            float v = traj[4 * s + i];
            if (lo[i] > v)
                lo[i] = v;
            if (hi[i] < v)
                hi[i] = v;
        }
    }
}

/* ReconData::normalizeTraj (ReconData.cpp:211-225) and
 * ReconData::transformLocalTraj (ReconData.cpp:201-209). */
void orc_normalize_traj(float *traj, size_t n, int dim, unsigned G, float *lo, float *hi,
                        float *tr_out, float *scale_out)
{
    float tr = -lo[0];
    float scale = (float)(G - 1) / (hi[0] - lo[0]);
    for (int c = 0; c < dim; ++c) {
        lo[c] = (lo[c] + tr) * scale;
        hi[c] = (hi[c] + tr) * scale;
    }
    for (size_t s = 0; s < n; ++s)
        for (int c = 0; c < dim; ++c)
            traj[4 * s + c] = (traj[4 * s + c] + tr) * scale;
    if (tr_out)
        *tr_out = tr;
    if (scale_out)
        *scale_out = scale;
}

/* ---------------------------------------------------------------------- */
/* Gridding                                                                */
/* ---------------------------------------------------------------------- */

/* float -> int the way the reference's x86-64 build converts (cvttss2si):
 * out-of-range and NaN give INT_MIN. */
static int x86_f2i(float v)
{
    if (v >= -2147483648.0f && v < 2147483648.0f)
        return (int)v;
    return INT_MIN;
}

/* GridLut.cpp:98-106 for one component. */
static void comp_range(float c, float kHW, unsigned G, int *s, int *e)
{
    int st = x86_f2i(ceilf(c - kHW));
    int en = x86_f2i(floorf(c + kHW));
    st = (int)fmax((double)st, 0.0);
    en = (int)fmin((double)en, (double)(G - 1));
    *s = st;
    *e = en;
}

void orc_sample_range(const float *traj, size_t n, int dim, unsigned G, float kHW,
                      int *start, int *end)
{
    for (size_t s = 0; s < n; ++s) {
        for (int i = 0; i < 3; ++i) {
            start[3 * s + i] = 0;
            end[3 * s + i] = 0;
        }
        for (int i = 0; i < dim; ++i)
            comp_range(traj[4 * s + i], kHW, G, &start[3 * s + i], &end[3 * s + i]);
    }
}

/* GridLut.cpp:120-136: dk = sqrtf(dz2 + dy2 + dx*dx); if dk < kHW the LUT
 * index is round(dk / kHW * (klength - 1)). */
int orc_tap_lut_index(float dx, float dy, float dz, float kHW, int klength)
{
    float dz2 = dz * dz;
    float dy2 = dy * dy;
    float dk = sqrtf(dz2 + dy2 + dx * dx);
    if (dk < kHW)
        return (int)roundf(dk / kHW * (float)(klength - 1));
    return -1;
}

void orc_lut_index_of_s(const float *s, size_t n, float kHW, int klength, int *out)
{
    for (size_t i = 0; i < n; ++i) {
        float dk = sqrtf(s[i]);
        out[i] = dk < kHW ? (int)roundf(dk / kHW * (float)(klength - 1)) : -1;
    }
}

/* GridLut::griddingChannel, GridLut.cpp:80-147, restricted to the cells of
 * the last axis (z in 3D, y in 2D) in [b0, b1): every sample is visited in
 * sample order and only its taps inside the band are added, so each cell of
 * the band receives exactly the adds of the full loop, in the same order.
 * The band is not cleared here. */
static void grid_channel_band(const float *traj, const float *dcf, const float *kdata, size_t n,
                              int dim, unsigned G, float kWidth, const float *lut, int klength,
                              float *out, int b0, int b1)
{
    float kHW = kWidth / 2;
    const int last = dim - 1;
    for (size_t s = 0; s < n; ++s) {
        float center[3] = {0, 0, 0};
        int start[3] = {0, 0, 0}, end[3] = {0, 0, 0};
        for (int i = 0; i < dim; ++i) {
            center[i] = traj[4 * s + i];
            comp_range(center[i], kHW, G, &start[i], &end[i]);
        }
        if (start[last] < b0)
            start[last] = b0;
        if (end[last] > b1 - 1)
            end[last] = b1 - 1;
        if (start[last] > end[last])
            continue;
        /* GridLut.cpp:109: data = dcf * sample (complex<float> times float). */
        float dre = dcf[s] * kdata[2 * s];
        float dim_ = dcf[s] * kdata[2 * s + 1];

        for (int z = start[2]; z <= end[2]; z++) {
            float dz = (float)z - center[2];
            float dz2 = dz * dz;
            for (int y = start[1]; y <= end[1]; y++) {
                float dy = (float)y - center[1];
                float dy2 = dy * dy;
                size_t row = ((size_t)z * G + (size_t)y) * G;
                for (int x = start[0]; x <= end[0]; x++) {
                    float dx = (float)x - center[0];
                    float dk = sqrtf(dz2 + dy2 + dx * dx);
                    if (dk < kHW) {
                        int ki = (int)roundf(dk / kHW * (float)(klength - 1));
                        float k = lut[ki];
                        float *o = out + 2 * (row + (size_t)x);
                        /* GridLut.cpp:137: *itOut += k * data */
                        o[0] = o[0] + k * dre;
                        o[1] = o[1] + k * dim_;
                    }
                }
            }
        }
    }
}

/* GridLut::griddingChannel, GridLut.cpp:80-147. */
void orc_grid_channel(const float *traj, const float *dcf, const float *kdata, size_t n,
                      int dim, unsigned G, float kWidth, const float *lut, int klength,
                      float *out)
{
    size_t cells = (dim == 3) ? (size_t)G * G * G : (size_t)G * G;
    memset(out, 0, cells * 2 * sizeof(float));
    grid_channel_band(traj, dcf, kdata, n, dim, G, kWidth, lut, klength, out, 0, (int)G);
}

void orc_grid_bands(const float *traj, const float *dcf, const float *kdata, size_t n,
                    int channels, int dim, unsigned G, float kWidth, const float *lut,
                    int klength, float *out, int threads)
{
    size_t cells = (dim == 3) ? (size_t)G * G * G : (size_t)G * G;
    size_t band_cells = cells / G; /* cells per z (3D) or y (2D) index */
    if (threads < 1)
        threads = 1;
    int nb = threads * 4;
    if (nb > (int)G)
        nb = (int)G;
    (void)threads;
    for (int c = 0; c < channels; ++c) {
        float *o = out + 2 * (size_t)c * cells;
        const float *kd = kdata + 2 * (size_t)c * n;
#pragma omp parallel for schedule(dynamic) num_threads(threads)
        for (int b = 0; b < nb; ++b) {
            int b0 = (int)((long long)G * b / nb), b1 = (int)((long long)G * (b + 1) / nb);
            memset(o + 2 * (size_t)b0 * band_cells, 0, (size_t)(b1 - b0) * band_cells * 2 * sizeof(float));
            grid_channel_band(traj, dcf, kd, n, dim, G, kWidth, lut, klength, o, b0, b1);
        }
    }
}

/* GridLut::execute, GridLut.cpp:53-78. */
void orc_grid(const float *traj, const float *dcf, const float *kdata, size_t n,
              int channels, int dim, unsigned G, float kWidth, const float *lut,
              int klength, float *out, int threads)
{
    size_t cells = (dim == 3) ? (size_t)G * G * G : (size_t)G * G;
    if (threads < 1)
        threads = 1;
    (void)threads;
#pragma omp parallel for schedule(dynamic) num_threads(threads)
    for (int c = 0; c < channels; ++c)
        orc_grid_channel(traj, dcf, kdata + 2 * (size_t)c * n, n, dim, G, kWidth, lut, klength,
                         out + 2 * (size_t)c * cells);
}

static void grid_channel_band_f64(const float *traj, const float *dcf, const float *kdata, size_t n,
                                  int dim, unsigned G, float kWidth, const float *lut, int klength,
                                  double *out, int b0, int b1)
{
    float kHW = kWidth / 2;
    const int last = dim - 1;
    for (size_t s = 0; s < n; ++s) {
        float center[3] = {0, 0, 0};
        int start[3] = {0, 0, 0}, end[3] = {0, 0, 0};
        for (int i = 0; i < dim; ++i) {
            center[i] = traj[4 * s + i];
            comp_range(center[i], kHW, G, &start[i], &end[i]);
        }
        if (start[last] < b0)
            start[last] = b0;
        if (end[last] > b1 - 1)
            end[last] = b1 - 1;
        if (start[last] > end[last])
            continue;
        double dre = (double)dcf[s] * (double)kdata[2 * s];
        double dimg = (double)dcf[s] * (double)kdata[2 * s + 1];
        for (int z = start[2]; z <= end[2]; z++) {
            for (int y = start[1]; y <= end[1]; y++) {
                size_t row = ((size_t)z * G + (size_t)y) * G;
                for (int x = start[0]; x <= end[0]; x++) {
                    int ki = orc_tap_lut_index((float)x - center[0], (float)y - center[1],
                                               (float)z - center[2], kHW, klength);
                    if (ki >= 0) {
                        double k = (double)lut[ki];
                        out[2 * (row + x)] += k * dre;
                        out[2 * (row + x) + 1] += k * dimg;
                    }
                }
            }
        }
    }
}

void orc_grid_channel_f64(const float *traj, const float *dcf, const float *kdata, size_t n,
                          int dim, unsigned G, float kWidth, const float *lut, int klength,
                          double *out)
{
    size_t cells = (dim == 3) ? (size_t)G * G * G : (size_t)G * G;
    memset(out, 0, cells * 2 * sizeof(double));
    grid_channel_band_f64(traj, dcf, kdata, n, dim, G, kWidth, lut, klength, out, 0, (int)G);
}

void orc_grid_f64_bands(const float *traj, const float *dcf, const float *kdata, size_t n,
                        int channels, int dim, unsigned G, float kWidth, const float *lut,
                        int klength, double *out, int threads)
{
    size_t cells = (dim == 3) ? (size_t)G * G * G : (size_t)G * G;
    size_t band_cells = cells / G;
    if (threads < 1)
        threads = 1;
    int nb = threads * 4;
    if (nb > (int)G)
        nb = (int)G;
    (void)threads;
    for (int c = 0; c < channels; ++c) {
        double *o = out + 2 * (size_t)c * cells;
        const float *kd = kdata + 2 * (size_t)c * n;
#pragma omp parallel for schedule(dynamic) num_threads(threads)
        for (int b = 0; b < nb; ++b) {
            int b0 = (int)((long long)G * b / nb), b1 = (int)((long long)G * (b + 1) / nb);
            memset(o + 2 * (size_t)b0 * band_cells, 0, (size_t)(b1 - b0) * band_cells * 2 * sizeof(double));
            grid_channel_band_f64(traj, dcf, kd, n, dim, G, kWidth, lut, klength, o, b0, b1);
        }
    }
}

void orc_sample_mass(const float *traj, size_t n, int dim, unsigned G, float kWidth,
                     const float *lut, int klength, double *mass, int threads)
{
    float kHW = kWidth / 2;
    if (threads < 1)
        threads = 1;
    (void)threads;
#pragma omp parallel for schedule(static) num_threads(threads)
    for (long long s = 0; s < (long long)n; ++s) {
        float center[3] = {0, 0, 0};
        int start[3] = {0, 0, 0}, end[3] = {0, 0, 0};
        for (int i = 0; i < dim; ++i) {
            center[i] = traj[4 * s + i];
            comp_range(center[i], kHW, G, &start[i], &end[i]);
        }
        double m = 0;
        for (int z = start[2]; z <= end[2]; z++)
            for (int y = start[1]; y <= end[1]; y++)
                for (int x = start[0]; x <= end[0]; x++) {
                    int ki = orc_tap_lut_index((float)x - center[0], (float)y - center[1],
                                               (float)z - center[2], kHW, klength);
                    if (ki >= 0)
                        m += (double)lut[ki];
                }
        mass[s] = m;
    }
}

void orc_sample_tiles(const int *start, const int *end, size_t n, int dim,
                      const int *tile_shape, int *tlo, int *thi)
{
    for (size_t s = 0; s < n; ++s) {
        int empty = 0;
        for (int i = 0; i < dim; ++i)
            if (start[3 * s + i] > end[3 * s + i])
                empty = 1;
        for (int i = 0; i < 3; ++i) {
            if (i >= dim) {
                tlo[3 * s + i] = 0;
                thi[3 * s + i] = 0;
            } else if (empty) {
                tlo[3 * s + i] = 1;
                thi[3 * s + i] = 0;
            } else {
                tlo[3 * s + i] = start[3 * s + i] / tile_shape[i];
                thi[3 * s + i] = end[3 * s + i] / tile_shape[i];
            }
        }
    }
}

/* ---------------------------------------------------------------------- */
/* FFT (mixed radix, double precision), stand-in for FFTW3f                */
/* ---------------------------------------------------------------------- */

typedef struct {
    double re, im;
} cplx;

static int smallest_factor(int n)
{
    if (n % 4 == 0)
        return 4;
    for (int p = 2; p * p <= n; ++p)
        if (n % p == 0)
            return p;
    return n;
}

/* out[k] = sum_j in[j*stride] * W^{j k}, W = tw[N/n]; tw has N entries
 * tw[j] = exp(sign * 2 pi i j / N).  Recursive decimation in time. */
static void dft_rec(const cplx *in, size_t stride, cplx *out, int n, int N, const cplx *tw,
                    cplx *tmp)
{
    if (n == 1) {
        out[0] = in[0];
        return;
    }
    int p = smallest_factor(n);
    int m = n / p;
    for (int r = 0; r < p; ++r)
        dft_rec(in + (size_t)r * stride, stride * (size_t)p, out + (size_t)r * m, m, N, tw, tmp);
    int step = N / n;  /* W_n = tw[step] */
    for (int k = 0; k < m; ++k) {
        for (int r = 0; r < p; ++r) {
            cplx v = out[(size_t)r * m + k];
            size_t e = ((size_t)r * (size_t)k * (size_t)step) % (size_t)N;
            cplx w = tw[e];
            tmp[r].re = v.re * w.re - v.im * w.im;
            tmp[r].im = v.re * w.im + v.im * w.re;
        }
        for (int q = 0; q < p; ++q) {
            double sr = 0, si = 0;
            for (int r = 0; r < p; ++r) {
                size_t e = ((size_t)r * (size_t)q * (size_t)m * (size_t)step) % (size_t)N;
                cplx w = tw[e];
                sr += tmp[r].re * w.re - tmp[r].im * w.im;
                si += tmp[r].re * w.im + tmp[r].im * w.re;
            }
            out[(size_t)k + (size_t)q * m].re = sr;
            out[(size_t)k + (size_t)q * m].im = si;
        }
    }
}

/* Transform every line along one axis: lines of length n, element stride
 * `stride`, count `lines`, line start offsets from line_offset(). */
static void fft_axis(float *data, size_t total, size_t n, size_t stride, int sign, int threads)
{
    if (n <= 1)
        return;
    cplx *tw = (cplx *)malloc(n * sizeof(cplx));
    for (size_t j = 0; j < n; ++j) {
        double a = (double)sign * 2.0 * M_PI * (double)j / (double)n;
        tw[j].re = cos(a);
        tw[j].im = sin(a);
    }
    size_t lines = total / n;
    if (threads < 1)
        threads = 1;
    (void)threads;
#pragma omp parallel num_threads(threads)
    {
        cplx *buf = (cplx *)malloc(2 * n * sizeof(cplx));
        cplx *tmp = (cplx *)malloc((n + 4) * sizeof(cplx));
#pragma omp for schedule(static)
        for (long long l = 0; l < (long long)lines; ++l) {
            /* line l: block = l / stride, offset within block = l % stride */
            size_t blk = (size_t)l / stride, off = (size_t)l % stride;
            size_t base = blk * stride * n + off;
            for (size_t j = 0; j < n; ++j) {
                buf[j].re = data[2 * (base + j * stride)];
                buf[j].im = data[2 * (base + j * stride) + 1];
            }
            dft_rec(buf, 1, buf + n, (int)n, (int)n, tw, tmp);
            for (size_t j = 0; j < n; ++j) {
                data[2 * (base + j * stride)] = (float)buf[n + j].re;
                data[2 * (base + j * stride) + 1] = (float)buf[n + j].im;
            }
        }
        free(buf);
        free(tmp);
    }
    free(tw);
}

int orc_fft(float *data, int dim, const unsigned *size, int batch, int sign, int threads)
{
    if (dim < 1 || dim > 3)
        return -1;
    size_t sx = size[0], sy = dim > 1 ? size[1] : 1, sz = dim > 2 ? size[2] : 1;
    size_t total = sx * sy * sz;
    for (int b = 0; b < batch; ++b) {
        float *d = data + 2 * total * (size_t)b;
        fft_axis(d, total, sx, 1, sign, threads);
        if (dim > 1)
            fft_axis(d, total, sy, sx, sign, threads);
        if (dim > 2)
            fft_axis(d, total, sz, sx * sy, sign, threads);
    }
    return 0;
}

/* ---------------------------------------------------------------------- */
/* Image filters                                                           */
/* ---------------------------------------------------------------------- */

static void swap_c(float *data, size_t i, size_t j)
{
    float r = data[2 * i], m = data[2 * i + 1];
    data[2 * i] = data[2 * j];
    data[2 * i + 1] = data[2 * j + 1];
    data[2 * j] = r;
    data[2 * j + 1] = m;
}

/* ImageFilter::fftShift2 (ImageFilter.cpp:231-251) and fftShift3
 * (ImageFilter.cpp:253-280). */
void orc_fft_shift(float *data, int dim, const unsigned *size)
{
    size_t sx = size[0], sy = size[1], sz = dim == 3 ? size[2] : 1;
    size_t n0h = sx / 2, n1h = sy / 2, n2h = sz / 2;
    if (dim == 3) {
        for (size_t z = 0; z < n2h; z++) {
            size_t z1 = z + n2h;
            for (size_t y = 0; y < sy; y++) {
                size_t y1 = y < n1h ? y + n1h : y - n1h;
                for (size_t x = 0; x < sx; x++) {
                    size_t x1 = x < n0h ? x + n0h : x - n0h;
                    swap_c(data, z * sx * sy + y * sx + x, z1 * sx * sy + y1 * sx + x1);
                }
            }
        }
    } else {
        for (size_t y = 0; y < n1h; y++) {
            size_t y1 = y + n1h;
            for (size_t x = 0; x < sx; x++) {
                size_t x1 = x < n0h ? x + n0h : x - n0h;
                swap_c(data, y * sx + x, y1 * sx + x1);
            }
        }
    }
}

/* ImageFilter::SOS(reconSize) = SOS(self, reconSize) then sqrt
 * (ImageFilter.cpp:159-209).  The complex product x*conj(x) of the
 * reference evaluates to (re*re + im*im, +0) in float. */
void orc_sos(const float *imgs, int channels, int dim, const unsigned *size,
             const unsigned *recon, float *out)
{
    unsigned isx = size[0], isy = size[1], isz = dim == 3 ? size[2] : 1;
    unsigned rsx = recon[0], rsy = recon[1], rsz = recon[2];
    unsigned x0 = (isx - rsx) / 2, y0 = (isy - rsy) / 2, z0 = (isz - rsz) / 2;
    size_t nout = (size_t)rsx * rsy * rsz;
    size_t cells = (size_t)isx * isy * isz;
    memset(out, 0, nout * 2 * sizeof(float));
    for (int c = 0; c < channels; ++c) {
        const float *img = imgs + 2 * cells * (size_t)c;
        for (unsigned z = 0; z < rsz; z++) {
            size_t in1 = (size_t)(z + z0) * ((size_t)isx * isy) + (size_t)y0 * isx;
            size_t out1 = (size_t)z * ((size_t)rsx * rsy);
            for (unsigned y = 0; y < rsy; y++) {
                size_t in2 = (size_t)y * isx + in1 + x0;
                size_t out2 = (size_t)y * rsx + out1;
                for (unsigned x = 0; x < rsx; x++) {
                    float a = img[2 * (x + in2)], b = img[2 * (x + in2) + 1];
                    float re = a * a - b * (-b);
                    out[2 * (x + out2)] = out[2 * (x + out2)] + re;
                }
            }
        }
    }
    for (size_t i = 0; i < nout; ++i) {
        out[2 * i] = sqrtf(out[2 * i]);
        out[2 * i + 1] = 0.0f;
    }
}

/* ImageFilter::lowFilter, ImageFilter.cpp:55-93. */
void orc_low_filter(float *imgs, int channels, int dim, const unsigned *size, int res)
{
    unsigned sx = size[0], sy = size[1], sz = dim == 3 ? size[2] : 1;
    long long x0 = sx / 2, y0 = sy / 2, z0 = sz / 2;
    float att = (float)(2.0 * res * res / 4.0);
    float coeff[2000];
    for (int r = 0; r < 2000; r++)
        coeff[r] = expf((float)(-r / 100.0));
    size_t cells = (size_t)sx * sy * sz;
    for (int c = 0; c < channels; ++c) {
        float *d = imgs + 2 * cells * (size_t)c;
        size_t o = 0;
        for (long long z = 0; z < sz; z++) {
            int r1 = (int)((z - z0) * (z - z0));
            for (long long y = 0; y < sy; y++) {
                int r2 = (int)((y - y0) * (y - y0) + r1);
                for (long long x = 0; x < sx; x++, o++) {
                    int r = (int)((x - x0) * (x - x0) + r2);
                    int idx = (int)((double)((float)r / att) * 100.0);
                    if (idx >= 2000) {
                        d[2 * o] = 0;
                        d[2 * o + 1] = 0;
                    } else {
                        d[2 * o] = d[2 * o] * coeff[idx];
                        d[2 * o + 1] = d[2 * o + 1] * coeff[idx];
                    }
                }
            }
        }
    }
}

/* ImageFilter::normalize, ImageFilter.cpp:95-118 (std::norm is re*re + im*im). */
void orc_normalize_channels(float *imgs, int channels, int dim, const unsigned *size)
{
    size_t cells = (size_t)size[0] * size[1] * (dim == 3 ? size[2] : 1);
    for (size_t v = 0; v < cells; ++v) {
        float mag = 0;
        for (int c = 0; c < channels; ++c) {
            float a = imgs[2 * (cells * c + v)], b = imgs[2 * (cells * c + v) + 1];
            mag = mag + (a * a + b * b);
        }
        float s = sqrtf(mag);
        for (int c = 0; c < channels; ++c) {
            imgs[2 * (cells * c + v)] = imgs[2 * (cells * c + v)] / s;
            imgs[2 * (cells * c + v) + 1] = imgs[2 * (cells * c + v) + 1] / s;
        }
    }
}

/* ImageFilter::SOS(map, reconSize), ImageFilter.cpp:170-209. */
void orc_sos_map(const float *imgs, const float *maps, int channels, int dim, const unsigned *size,
                 const unsigned *recon, float *out)
{
    unsigned isx = size[0], isy = size[1], isz = dim == 3 ? size[2] : 1;
    unsigned rsx = recon[0], rsy = recon[1], rsz = dim == 3 ? recon[2] : 1;
    unsigned x0 = (isx - rsx) / 2, y0 = (isy - rsy) / 2, z0 = (isz - rsz) / 2;
    size_t nout = (size_t)rsx * rsy * rsz, cells = (size_t)isx * isy * isz;
    memset(out, 0, nout * 2 * sizeof(float));
    for (int c = 0; c < channels; ++c) {
        const float *img = imgs + 2 * cells * (size_t)c, *map = maps + 2 * cells * (size_t)c;
        for (unsigned z = 0; z < rsz; z++)
            for (unsigned y = 0; y < rsy; y++)
                for (unsigned x = 0; x < rsx; x++) {
                    size_t in3 = ((size_t)(z + z0) * isy + (y + y0)) * isx + (x + x0);
                    size_t out3 = ((size_t)z * rsy + y) * rsx + x;
                    float a = img[2 * in3], b = img[2 * in3 + 1];
                    float cr = map[2 * in3], nd = -map[2 * in3 + 1];
                    float re = a * cr - b * nd;
                    float im = a * nd + b * cr;
                    out[2 * out3] = out[2 * out3] + re;
                    out[2 * out3 + 1] = out[2 * out3 + 1] + im;
                }
    }
}

/* Program/Main.cpp:101-181 without file I/O. */
int orc_recon(float *traj, const float *dcf, const float *kdata, size_t n, int channels,
              int dim, unsigned reconSize, float os, float kWidth, int klength,
              const unsigned *recon, float *out_mag, int threads)
{
    unsigned G = (unsigned)((float)reconSize * os); /* GridLut.cpp:45 */
    float lo[3], hi[3];
    float *lut = (float *)malloc(sizeof(float) * (size_t)klength);
    if (!lut || orc_kb_lut(kWidth, os, klength, lut) != 0) {
        free(lut);
        return -1;
    }
    orc_comp_bounds(traj, n, dim, lo, hi);
    orc_normalize_traj(traj, n, dim, G, lo, hi, NULL, NULL);
    size_t cells = (dim == 3) ? (size_t)G * G * G : (size_t)G * G;
    float *grid = (float *)malloc(cells * 2 * sizeof(float) * (size_t)channels);
    if (!grid) {
        free(lut);
        return -2;
    }
    orc_grid(traj, dcf, kdata, n, channels, dim, G, kWidth, lut, klength, grid, threads);
    unsigned sz[3] = {G, G, dim == 3 ? G : 1};
    orc_fft(grid, dim, sz, channels, +1, threads);
    for (int c = 0; c < channels; ++c)
        orc_fft_shift(grid + 2 * cells * (size_t)c, dim, sz);
    size_t nout = (size_t)recon[0] * recon[1] * recon[2];
    float *sos = (float *)malloc(nout * 2 * sizeof(float));
    orc_sos(grid, channels, dim, sz, recon, sos);
    for (size_t i = 0; i < nout; ++i)
        out_mag[i] = fabsf(sos[2 * i]);
    free(sos);
    free(grid);
    free(lut);
    return 0;
}
