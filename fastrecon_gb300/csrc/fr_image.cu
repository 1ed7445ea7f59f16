// fr_image.cu -- image-domain kernels: fftShift, crop, fused crop + SoS.
//
// Replaces the host-side ImageFilter::fftShift / crop / SOS that the
// reference runs even in GPU mode (ImageFilter.cpp:40-53,120-209,231-280;
// cuImageFilter.cpp:40-52).  The SoS kernel reads each coil image once over
// the crop window and reproduces the reference's float arithmetic exactly:
// per channel, in channel order, acc += (re*re - im*(-im)), then sqrt.
#include <cuda_runtime.h>

#include "fr_internal.h"

namespace fr {
namespace {

struct Size3 {
    unsigned x, y, z;
};

// sos_mode bit 1: continue the sum already in `out` (coils in slabs);
// bit 2: apply sqrt (/ deapod), else store the plain sum.
__global__ void sos_kernel(const float2 *__restrict__ imgs, int channels, Size3 in, Size3 rec,
                           Size3 off, const float *__restrict__ deapod, float *__restrict__ out, int sos_mode)
{
    const size_t nout = (size_t)rec.x * rec.y * rec.z;
    const size_t cells = (size_t)in.x * in.y * in.z;
    for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < nout;
         o += (size_t)gridDim.x * blockDim.x) {
        unsigned x = (unsigned)(o % rec.x);
        size_t r = o / rec.x;
        unsigned y = (unsigned)(r % rec.y);
        unsigned z = (unsigned)(r / rec.y);
        size_t in_idx = ((size_t)(z + off.z) * in.y + (y + off.y)) * in.x + (x + off.x);
        float acc = (sos_mode & 1) ? out[o] : 0.f;
        for (int c = 0; c < channels; ++c) {
            float2 v = imgs[(size_t)c * cells + in_idx];
            // std::complex<float>: x * conj(x) real part = a*a - b*(-b)
            float re = __fsub_rn(__fmul_rn(v.x, v.x), __fmul_rn(v.y, -v.y));
            acc = __fadd_rn(acc, re);
        }
        float m = acc;
        if (sos_mode & 2) {
            m = __fsqrt_rn(m);
            if (deapod) m = __fdiv_rn(m, deapod[o]);
        }
        out[o] = m;
    }
}

__global__ void crop_kernel(const float2 *__restrict__ imgs, int channels, Size3 in, Size3 rec, Size3 off,
                            float2 *__restrict__ out)
{
    const size_t nout = (size_t)rec.x * rec.y * rec.z;
    const size_t cells = (size_t)in.x * in.y * in.z;
    const size_t total = nout * (size_t)channels;
    for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < total;
         o += (size_t)gridDim.x * blockDim.x) {
        size_t c = o / nout;
        size_t v = o - c * nout;
        unsigned x = (unsigned)(v % rec.x);
        size_t r = v / rec.x;
        unsigned y = (unsigned)(r % rec.y);
        unsigned z = (unsigned)(r / rec.y);
        out[o] = imgs[c * cells + ((size_t)(z + off.z) * in.y + (y + off.y)) * in.x + (x + off.x)];
    }
}

// Even sizes: the reference's swap loops are a set of disjoint swaps, done
// in parallel.  Each thread handles one element of the lower half (z < n2h
// in 3D, y < n1h in 2D) and swaps it with its partner.
__global__ void shift_even_kernel(float2 *__restrict__ imgs, int channels, int dim, Size3 s)
{
    const size_t cells = (size_t)s.x * s.y * s.z;
    const size_t half = dim == 3 ? cells / 2 : (size_t)s.x * (s.y / 2);
    const size_t total = half * (size_t)channels;
    const unsigned n0h = s.x / 2, n1h = s.y / 2, n2h = s.z / 2;
    for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < total;
         o += (size_t)gridDim.x * blockDim.x) {
        size_t c = o / half;
        size_t i = o - c * half;
        unsigned x = (unsigned)(i % s.x);
        size_t r = i / s.x;
        size_t a, b;
        unsigned x1 = x < n0h ? x + n0h : x - n0h;
        if (dim == 3) {
            unsigned y = (unsigned)(r % s.y);
            unsigned z = (unsigned)(r / s.y);
            unsigned y1 = y < n1h ? y + n1h : y - n1h;
            unsigned z1 = z + n2h;
            a = ((size_t)z * s.y + y) * s.x + x;
            b = ((size_t)z1 * s.y + y1) * s.x + x1;
        } else {
            unsigned y = (unsigned)r;
            a = (size_t)y * s.x + x;
            b = (size_t)(y + n1h) * s.x + x1;
        }
        float2 *img = imgs + c * cells;
        float2 t = img[a];
        img[a] = img[b];
        img[b] = t;
    }
}

// Odd sizes: the swap sequence overlaps, so it is replayed in the
// reference's order, one thread per independent (channel, slab pair).
__global__ void shift_serial_kernel(float2 *__restrict__ imgs, int channels, int dim, Size3 s)
{
    const size_t cells = (size_t)s.x * s.y * s.z;
    const unsigned n0h = s.x / 2, n1h = s.y / 2, n2h = s.z / 2;
    const unsigned pairs = dim == 3 ? n2h : n1h;
    const size_t total = (size_t)pairs * channels;
    for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < total;
         o += (size_t)gridDim.x * blockDim.x) {
        size_t c = o / pairs;
        unsigned k = (unsigned)(o - c * pairs);
        float2 *img = imgs + c * cells;
        if (dim == 3) {
            unsigned z = k, z1 = k + n2h;
            for (unsigned y = 0; y < s.y; y++) {
                unsigned y1 = y < n1h ? y + n1h : y - n1h;
                for (unsigned x = 0; x < s.x; x++) {
                    unsigned x1 = x < n0h ? x + n0h : x - n0h;
                    size_t a = ((size_t)z * s.y + y) * s.x + x;
                    size_t b = ((size_t)z1 * s.y + y1) * s.x + x1;
                    float2 t = img[a];
                    img[a] = img[b];
                    img[b] = t;
                }
            }
        } else {
            unsigned y = k, y1 = k + n1h;
            for (unsigned x = 0; x < s.x; x++) {
                unsigned x1 = x < n0h ? x + n0h : x - n0h;
                size_t a = (size_t)y * s.x + x;
                size_t b = (size_t)y1 * s.x + x1;
                float2 t = img[a];
                img[a] = img[b];
                img[b] = t;
            }
        }
    }
}

int blocks_for(size_t n, int threads)
{
    size_t b = (n + threads - 1) / threads;
    if (b > 152 * 64) b = 152 * 64;
    return (int)(b ? b : 1);
}

Size3 size_of(int dim, const unsigned *s)
{
    return Size3{s[0], s[1], dim == 3 ? s[2] : 1u};
}

int check_crop(int dim, const unsigned *size, const unsigned *rec, Size3 &in, Size3 &r, Size3 &off)
{
    in = size_of(dim, size);
    r = Size3{rec[0], rec[1], dim == 3 ? rec[2] : 1u};
    if (r.x > in.x || r.y > in.y || r.z > in.z)
        return fail(FR_ERR_INVALID_ARGUMENT, "crop size larger than image");  // ImageFilter.cpp:128-131
    off = Size3{(in.x - r.x) / 2, (in.y - r.y) / 2, (in.z - r.z) / 2};
    return FR_OK;
}

}  // namespace

int sos_run(const float *d_imgs, int channels, int dim, const unsigned *size, const unsigned *recon,
            const float *d_deapod, float *d_out, cudaStream_t s, int sos_mode)
{
    Size3 in, r, off;
    int st = check_crop(dim, size, recon, in, r, off);
    if (st) return st;
    size_t nout = (size_t)r.x * r.y * r.z;
    sos_kernel<<<blocks_for(nout, 256), 256, 0, s>>>(reinterpret_cast<const float2 *>(d_imgs), channels, in, r,
                                                     off, d_deapod, d_out, sos_mode);
    FR_CHECK_LAUNCH("sos_kernel");
    return FR_OK;
}

int crop_run(const float *d_imgs, int channels, int dim, const unsigned *size, const unsigned *crop,
             float *d_out, cudaStream_t s)
{
    Size3 in, r, off;
    int st = check_crop(dim, size, crop, in, r, off);
    if (st) return st;
    size_t total = (size_t)r.x * r.y * r.z * channels;
    crop_kernel<<<blocks_for(total, 256), 256, 0, s>>>(reinterpret_cast<const float2 *>(d_imgs), channels, in, r,
                                                       off, reinterpret_cast<float2 *>(d_out));
    FR_CHECK_LAUNCH("crop_kernel");
    return FR_OK;
}

int shift_run(float *d_imgs, int channels, int dim, const unsigned *size, cudaStream_t s)
{
    Size3 sz = size_of(dim, size);
    bool even = (sz.x % 2 == 0) && (sz.y % 2 == 0) && (dim != 3 || sz.z % 2 == 0);
    float2 *p = reinterpret_cast<float2 *>(d_imgs);
    if (even) {
        size_t cells = (size_t)sz.x * sz.y * sz.z;
        size_t half = dim == 3 ? cells / 2 : (size_t)sz.x * (sz.y / 2);
        shift_even_kernel<<<blocks_for(half * channels, 256), 256, 0, s>>>(p, channels, dim, sz);
    } else {
        size_t pairs = (size_t)(dim == 3 ? sz.z / 2 : sz.y / 2) * channels;
        shift_serial_kernel<<<blocks_for(pairs, 64), 64, 0, s>>>(p, channels, dim, sz);
    }
    FR_CHECK_LAUNCH("shift_kernel");
    return FR_OK;
}

}  // namespace fr

// --------------------------------------------------------------------------
// Deapodization (absent in the reference): the image-domain apodization of
// the gridding kernel, obtained by gridding one unit sample at the FFT origin
// of the shifted image (cell G/2 on every axis) with the same LUT and tap
// rule, transforming it with the same backward FFT, and taking |.|
// normalised to the centre.
// --------------------------------------------------------------------------
namespace fr {
namespace {

__global__ void deapod_seed_kernel(float2 *__restrict__ grid, int dim, int G, float hw, const float *__restrict__ lut,
                                   int L, int reach, int checkerboard)
{
    const int w = 2 * reach + 1;
    const int total = dim == 3 ? w * w * w : w * w;
    const int c0 = G / 2;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        int ix = t % w, iy = (t / w) % w, iz = dim == 3 ? t / (w * w) : reach;
        int dx = ix - reach, dy = iy - reach, dz = iz - reach;
        int x = c0 + dx, y = c0 + dy, z = dim == 3 ? c0 + dz : 0;
        if (x < 0 || y < 0 || z < 0 || x >= G || y >= G || z >= G) continue;
        float fdy = (float)dy, fdz = (float)dz;
        float s = __fadd_rn(__fadd_rn(__fmul_rn(fdz, fdz), __fmul_rn(fdy, fdy)), __fmul_rn((float)dx, (float)dx));
        float dk = __fsqrt_rn(s);
        if (!(dk < hw)) continue;
        int ki = (int)roundf(__fmul_rn(__fdiv_rn(dk, hw), (float)(L - 1)));
        if (ki > L - 1) ki = L - 1;
        float v = lut[ki];
        if (checkerboard && ((x + y + z) & 1)) v = -v;
        grid[((size_t)z * G + y) * G + x] = make_float2(v, 0.f);
    }
}

__global__ void deapod_map_kernel(const float2 *__restrict__ img, Size3 in, Size3 rec, Size3 off,
                                  float *__restrict__ out)
{
    const size_t nout = (size_t)rec.x * rec.y * rec.z;
    const size_t ctr = ((size_t)(in.z / 2) * in.y + in.y / 2) * in.x + in.x / 2;
    const float2 c = img[ctr];
    const float norm = sqrtf(c.x * c.x + c.y * c.y);
    for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < nout; o += (size_t)gridDim.x * blockDim.x) {
        unsigned x = (unsigned)(o % rec.x);
        size_t r = o / rec.x;
        unsigned y = (unsigned)(r % rec.y);
        unsigned z = (unsigned)(r / rec.y);
        float2 v = img[((size_t)(z + off.z) * in.y + (y + off.y)) * in.x + (x + off.x)];
        float m = sqrtf(v.x * v.x + v.y * v.y) / norm;
        out[o] = m > 1e-6f ? m : 1e-6f;
    }
}

}  // namespace

int deapod_seed_run(float *d_grid, int dim, int G, float hw, const float *d_lut, int L, int checkerboard,
                    cudaStream_t s)
{
    size_t cells = dim == 3 ? (size_t)G * G * G : (size_t)G * G;
    FR_CUDA(cudaMemsetAsync(d_grid, 0, cells * 8, s));
    int reach = (int)ceilf(hw) + 1;
    deapod_seed_kernel<<<1, 256, 0, s>>>(reinterpret_cast<float2 *>(d_grid), dim, G, hw, d_lut, L, reach,
                                         checkerboard);
    FR_CHECK_LAUNCH("deapod_seed_kernel");
    return FR_OK;
}

int deapod_map_run(const float *d_img, int dim, const unsigned *size, const unsigned *recon, float *d_out,
                   cudaStream_t s)
{
    Size3 in, r, off;
    int st = check_crop(dim, size, recon, in, r, off);
    if (st) return st;
    size_t nout = (size_t)r.x * r.y * r.z;
    deapod_map_kernel<<<blocks_for(nout, 256), 256, 0, s>>>(reinterpret_cast<const float2 *>(d_img), in, r, off,
                                                            d_out);
    FR_CHECK_LAUNCH("deapod_map_kernel");
    return FR_OK;
}

}  // namespace fr

// --------------------------------------------------------------------------
// PILS image operations (ImageFilter.cpp:55-118,170-209) and helpers.
// --------------------------------------------------------------------------
namespace fr {
namespace {

__global__ void real_to_complex_kernel(const float *__restrict__ in, size_t n, float2 *__restrict__ out)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = make_float2(in[i], 0.f);
}

// ImageFilter::lowFilter: r = squared distance to (size/2) in integers,
// idx = (int)((float)r / att * 100.0), coefficient table from the host.
__global__ void low_filter_kernel(float2 *__restrict__ imgs, int channels, Size3 s, float att,
                                  const float *__restrict__ coeff)
{
    const size_t cells = (size_t)s.x * s.y * s.z;
    const size_t total = cells * (size_t)channels;
    const long long x0 = s.x / 2, y0 = s.y / 2, z0 = s.z / 2;
    for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < total; o += (size_t)gridDim.x * blockDim.x) {
        size_t v = o % cells;
        long long x = (long long)(v % s.x);
        size_t r0 = v / s.x;
        long long y = (long long)(r0 % s.y);
        long long z = (long long)(r0 / s.y);
        int r = (int)((x - x0) * (x - x0) + (y - y0) * (y - y0) + (z - z0) * (z - z0));
        int idx = (int)((double)__fdiv_rn((float)r, att) * 100.0);
        float2 a = imgs[o];
        if (idx >= 2000) {
            a = make_float2(0.f, 0.f);
        } else {
            float c = coeff[idx];
            a.x = __fmul_rn(a.x, c);
            a.y = __fmul_rn(a.y, c);
        }
        imgs[o] = a;
    }
}

// ImageFilter::normalize: mag = sum over channels of std::norm, each value
// divided by sqrtf(mag).
__global__ void normalize_channels_kernel(float2 *__restrict__ imgs, int channels, size_t cells)
{
    for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < cells; v += (size_t)gridDim.x * blockDim.x) {
        float mag = 0.f;
        for (int c = 0; c < channels; ++c) {
            float2 a = imgs[(size_t)c * cells + v];
            mag = __fadd_rn(mag, __fadd_rn(__fmul_rn(a.x, a.x), __fmul_rn(a.y, a.y)));
        }
        float d = __fsqrt_rn(mag);
        for (int c = 0; c < channels; ++c) {
            float2 a = imgs[(size_t)c * cells + v];
            imgs[(size_t)c * cells + v] = make_float2(__fdiv_rn(a.x, d), __fdiv_rn(a.y, d));
        }
    }
}

// ImageFilter::SOS(map, reconSize): out += data * conj(map) per channel.
__global__ void sos_map_kernel(const float2 *__restrict__ imgs, const float2 *__restrict__ maps, int channels,
                               Size3 in, Size3 rec, Size3 off, float2 *__restrict__ out)
{
    const size_t nout = (size_t)rec.x * rec.y * rec.z;
    const size_t cells = (size_t)in.x * in.y * in.z;
    for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < nout; o += (size_t)gridDim.x * blockDim.x) {
        unsigned x = (unsigned)(o % rec.x);
        size_t r = o / rec.x;
        unsigned y = (unsigned)(r % rec.y);
        unsigned z = (unsigned)(r / rec.y);
        size_t in_idx = ((size_t)(z + off.z) * in.y + (y + off.y)) * in.x + (x + off.x);
        float2 acc = make_float2(0.f, 0.f);
        for (int c = 0; c < channels; ++c) {
            float2 a = imgs[(size_t)c * cells + in_idx];
            float2 m = maps[(size_t)c * cells + in_idx];
            float nd = -m.y;  // conj
            float re = __fsub_rn(__fmul_rn(a.x, m.x), __fmul_rn(a.y, nd));
            float im = __fadd_rn(__fmul_rn(a.x, nd), __fmul_rn(a.y, m.x));
            acc.x = __fadd_rn(acc.x, re);
            acc.y = __fadd_rn(acc.y, im);
        }
        out[o] = acc;
    }
}

}  // namespace

int real_to_complex_run(const float *d_in, size_t n, float *d_out, cudaStream_t s)
{
    if (n == 0) return FR_OK;
    real_to_complex_kernel<<<blocks_for(n, 256), 256, 0, s>>>(d_in, n, reinterpret_cast<float2 *>(d_out));
    FR_CHECK_LAUNCH("real_to_complex_kernel");
    return FR_OK;
}

int low_filter_run(float *d_imgs, int channels, int dim, const unsigned *size, float att, const float *d_coeff,
                   cudaStream_t s)
{
    Size3 sz = size_of(dim, size);
    size_t total = (size_t)sz.x * sz.y * sz.z * channels;
    low_filter_kernel<<<blocks_for(total, 256), 256, 0, s>>>(reinterpret_cast<float2 *>(d_imgs), channels, sz, att,
                                                            d_coeff);
    FR_CHECK_LAUNCH("low_filter_kernel");
    return FR_OK;
}

int normalize_channels_run(float *d_imgs, int channels, int dim, const unsigned *size, cudaStream_t s)
{
    Size3 sz = size_of(dim, size);
    size_t cells = (size_t)sz.x * sz.y * sz.z;
    normalize_channels_kernel<<<blocks_for(cells, 256), 256, 0, s>>>(reinterpret_cast<float2 *>(d_imgs), channels,
                                                                    cells);
    FR_CHECK_LAUNCH("normalize_channels_kernel");
    return FR_OK;
}

int sos_map_run(const float *d_imgs, const float *d_maps, int channels, int dim, const unsigned *size,
                const unsigned *recon, float *d_out, cudaStream_t s)
{
    Size3 in, r, off;
    int st = check_crop(dim, size, recon, in, r, off);
    if (st) return st;
    size_t nout = (size_t)r.x * r.y * r.z;
    sos_map_kernel<<<blocks_for(nout, 256), 256, 0, s>>>(reinterpret_cast<const float2 *>(d_imgs),
                                                        reinterpret_cast<const float2 *>(d_maps), channels, in, r,
                                                        off, reinterpret_cast<float2 *>(d_out));
    FR_CHECK_LAUNCH("sos_map_kernel");
    return FR_OK;
}

}  // namespace fr
