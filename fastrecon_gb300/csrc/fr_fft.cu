// fr_fft.cu -- pruned backward FFT with fused crop and multi-coil sum of
// squares.
//
// Replaces cuFFT::excute + fftShift + crop + SOS (cuFFT.cpp:24-37,
// ImageFilter.cpp:40-53,159-209) when the grid was flushed with the
// (-1)^(x+y+z) modulation (even G), so the transform output is already
// shifted.  Only the centred out_size crop of the image is kept, so each of
// the d one-dimensional stages keeps only the cropped outputs of its axis:
//   x stage: lines along x of the grid          -> [C][Gz][Gy][Rx]
//   y stage: lines along y                      -> [C][Gz][Ry][Rx]
//   z stage: lines along z, all coils of a column in turn, |X|^2 summed over
//            coils in coil order, sqrt (and / deapod)  -> [Rz][Ry][Rx]
// (in 2D the y stage is the last one).  Each line is transformed in shared
// memory by a self-sorting (Stockham) mixed-radix FFT with radix 2, 3, 4, 5
// and 8 passes and a double-precision twiddle table rounded to float.  In 3D
// at the specialised sizes the x stage is a batched 1D cuFFT into a full-size
// buffer (faster than the shared-memory x stage there: every line is
// transformed either way), and the y and z stages read its cropped columns.
#include <cuda_runtime.h>
#include <cufft.h>

#include <cmath>
#include <cstdlib>
#include <new>
#include <vector>

#include "fr_internal.h"

namespace fr {
namespace {

constexpr int kMaxPasses = 12;
constexpr int kMaxN = 1024;
// SoS modes of the last stage (coils in slabs): continue the sum already in
// the output, and apply sqrt (/ deapod) at the end
constexpr int kSosAccIn = 1, kSosFinal = 2;

struct FftPlan1D {
    int n;
    int npass;
    int radix[kMaxPasses];
};

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// multiply by +i
__device__ __forceinline__ float2 cmuli(float2 a) { return make_float2(-a.y, a.x); }

// In-register DFTs with kernel exp(+2 pi i r k / p) (backward transform).
__device__ __forceinline__ void dft2(float2 *v)
{
    const float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
}
__device__ __forceinline__ void dft4(float2 *v)
{
    const float2 a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
    const float2 a2 = cadd(v[1], v[3]), a3 = cmuli(csub(v[1], v[3]));
    v[0] = cadd(a0, a2);
    v[2] = csub(a0, a2);
    v[1] = cadd(a1, a3);
    v[3] = csub(a1, a3);
}
__device__ __forceinline__ void dft3(float2 *v)
{
    const float c = -0.5f, s = 0.86602540378443864676f;  // cos, sin of 2 pi / 3
    const float2 t1 = cadd(v[1], v[2]);
    const float2 d = csub(v[1], v[2]);
    const float2 m = cadd(v[0], cscale(t1, c));
    const float2 r = cmuli(cscale(d, s));
    v[0] = cadd(v[0], t1);
    v[1] = cadd(m, r);
    v[2] = csub(m, r);
}
__device__ __forceinline__ void dft5(float2 *v)
{
    const float c1 = 0.30901699437494742410f, c2 = -0.80901699437494742410f;  // cos(2pi/5), cos(4pi/5)
    const float s1 = 0.95105651629515357212f, s2 = 0.58778525229247312917f;   // sin(2pi/5), sin(4pi/5)
    const float2 t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
    const float2 t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
    const float2 a = cadd(v[0], cadd(cscale(t1, c1), cscale(t2, c2)));
    const float2 b = cmuli(cadd(cscale(t3, s1), cscale(t4, s2)));
    const float2 c = cadd(v[0], cadd(cscale(t1, c2), cscale(t2, c1)));
    const float2 d = cmuli(csub(cscale(t3, s2), cscale(t4, s1)));
    v[0] = cadd(v[0], cadd(t1, t2));
    v[1] = cadd(a, b);
    v[4] = csub(a, b);
    v[2] = cadd(c, d);
    v[3] = csub(c, d);
}
__device__ __forceinline__ void dft8(float2 *v)
{
    const float h = 0.70710678118654752440f;  // 1/sqrt(2)
    float2 e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
    dft4(e);
    dft4(o);
    // twiddles exp(+2 pi i k / 8), k = 0..3
    const float2 o1 = make_float2(h * (o[1].x - o[1].y), h * (o[1].x + o[1].y));
    const float2 o2 = cmuli(o[2]);
    const float2 o3 = make_float2(-h * (o[3].x + o[3].y), h * (o[3].x - o[3].y));
    v[0] = cadd(e[0], o[0]);
    v[4] = csub(e[0], o[0]);
    v[1] = cadd(e[1], o1);
    v[5] = csub(e[1], o1);
    v[2] = cadd(e[2], o2);
    v[6] = csub(e[2], o2);
    v[3] = cadd(e[3], o3);
    v[7] = csub(e[3], o3);
}

template <int R>
__device__ __forceinline__ void dft(float2 *v)
{
    if constexpr (R == 2) dft2(v);
    if constexpr (R == 3) dft3(v);
    if constexpr (R == 4) dft4(v);
    if constexpr (R == 5) dft5(v);
    if constexpr (R == 8) dft8(v);
}

#include "fr_fft_reg.cuh"

// One Stockham pass of radix R over `lines` lines in shared memory:
// for j < n/R: v[r] = in[j + r n/R] * W^(r (j mod ns) n/(ns R)), DFT_R,
// out[(j/ns) ns R + (j mod ns) + r ns] = v[r].  Element e of line l sits at
// buf + l * lstride + e * estride.
template <int R>
__device__ __forceinline__ void stockham_pass(const float2 *__restrict__ in, float2 *__restrict__ out, int n, int ns,
                                              int lines, int lstride, int estride, const float2 *__restrict__ tw)
{
    const int m = n / R;
    const int tstep = n / (ns * R);
    for (int idx = threadIdx.x; idx < m * lines; idx += blockDim.x) {
        const int l = idx / m, j = idx - l * m;
        const int k = j % ns;
        float2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            float2 a = in[l * lstride + (j + r * m) * estride];
            if (r > 0 && k > 0) a = cmul(a, tw[(r * k * tstep) % n]);
            v[r] = a;
        }
        dft<R>(v);
        const int o = (j / ns) * ns * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) out[l * lstride + (o + r * ns) * estride] = v[r];
    }
}

// Full transform of `lines` lines held in buf0 (result in buf0 or buf1;
// returns the buffer holding it).
__device__ float2 *line_fft(float2 *buf0, float2 *buf1, const FftPlan1D &pl, int lines, int lstride, int estride,
                            const float2 *tw)
{
    float2 *in = buf0, *out = buf1;
    int ns = 1;
    for (int p = 0; p < pl.npass; ++p) {
        const int R = pl.radix[p];
        switch (R) {
        case 2: stockham_pass<2>(in, out, pl.n, ns, lines, lstride, estride, tw); break;
        case 3: stockham_pass<3>(in, out, pl.n, ns, lines, lstride, estride, tw); break;
        case 4: stockham_pass<4>(in, out, pl.n, ns, lines, lstride, estride, tw); break;
        case 5: stockham_pass<5>(in, out, pl.n, ns, lines, lstride, estride, tw); break;
        default: stockham_pass<8>(in, out, pl.n, ns, lines, lstride, estride, tw); break;
        }
        __syncthreads();
        ns *= R;
        float2 *t = in;
        in = out;
        out = t;
    }
    return in;
}

// The same passes with the transform length, radices and buffer geometry
// known at compile time (the index arithmetic becomes multiplies and
// shifts).  The common grid sizes are instantiated; others use line_fft.
// Element e of a line sits at e + e / 32 (one pad slot per 32) when the
// elements are contiguous (ES == 1), which spreads the radix-strided writes
// of a pass over the banks; column buffers (ES == lines) put the lines
// fastest instead.
template <int ES>
__device__ __forceinline__ int pad_e(int e)
{
    if constexpr (ES == 1) {
        return e + (e >> 5);
    } else {
        return e * ES;
    }
}

template <int N, int R, int NS, int LINES, int LS, int ES>
__device__ __forceinline__ void stockham_pass_ct(const float2 *__restrict__ in, float2 *__restrict__ out,
                                                 const float2 *__restrict__ tw)
{
    constexpr int M = N / R;
    constexpr int TSTEP = N / (NS * R);  // r * k * TSTEP < N: no reduction needed
    for (int idx = threadIdx.x; idx < M * LINES; idx += blockDim.x) {
        // contiguous lines: consecutive threads on consecutive butterflies;
        // column buffers: consecutive threads on consecutive lines
        const int l = ES == 1 ? idx / M : idx % LINES;
        const int j = ES == 1 ? idx - l * M : idx / LINES;
        const int k = j % NS;
        float2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            float2 a = in[l * LS + pad_e<ES>(j + r * M)];
            if (r > 0 && k > 0) a = cmul(a, tw[r * k * TSTEP]);
            v[r] = a;
        }
        dft<R>(v);
        const int o = (j / NS) * NS * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) out[l * LS + pad_e<ES>(o + r * NS)] = v[r];
    }
}

template <int N, int NS, int LINES, int LS, int ES, int R, int... Rest>
__device__ __forceinline__ float2 *fft_passes(float2 *in, float2 *out, const float2 *tw)
{
    stockham_pass_ct<N, R, NS, LINES, LS, ES>(in, out, tw);
    __syncthreads();
    if constexpr (sizeof...(Rest) == 0) {
        return out;
    } else {
        return fft_passes<N, NS * R, LINES, LS, ES, Rest...>(out, in, tw);
    }
}

// x stage: LINES consecutive lines of length n (contiguous) per CTA, keep
// outputs [x0, x0 + rx).  in: nlines x n, out: nlines x rx.
__global__ void __launch_bounds__(256) fft_x_kernel(const float2 *__restrict__ in, float2 *__restrict__ out,
                                                    long long nlines, FftPlan1D pl, int x0, int rx,
                                                    const float2 *__restrict__ tw_g, int lines_per_cta)
{
    extern __shared__ float2 sm[];
    const int n = pl.n;
    float2 *tw = sm;
    float2 *b0 = tw + n;
    const int lstride = n + 1;  // pad against bank conflicts
    float2 *b1 = b0 + lines_per_cta * lstride;
    for (int i = threadIdx.x; i < n; i += blockDim.x) tw[i] = tw_g[i];
    const long long l0 = (long long)blockIdx.x * lines_per_cta;
    const int lines = (int)min((long long)lines_per_cta, nlines - l0);
    for (int i = threadIdx.x; i < lines * n; i += blockDim.x) {
        const int l = i / n, e = i - l * n;
        b0[l * lstride + e] = in[(l0 + l) * n + e];
    }
    __syncthreads();
    float2 *res = line_fft(b0, b1, pl, lines, lstride, 1, tw);
    for (int i = threadIdx.x; i < lines * rx; i += blockDim.x) {
        const int l = i / rx, e = i - l * rx;
        out[(l0 + l) * rx + e] = res[l * lstride + x0 + e];
    }
}

// Column stage: for each (outer, column block of COLS) transform the lines
// along an axis of length n with element stride `stride` (in elements of the
// input), keep outputs [y0, y0 + ry).  Input index: base(outer) + e*stride + c.
// If `sos_out` is given this is the last stage: |X|^2 is summed over `coils`
// consecutive inputs (coil stride `cstride`), then sqrt (/ deapod).
// sos_mode (coils in slabs): kSosAccIn starts the sum from the value in
// sos_out, kSosFinal applies sqrt (/ deapod); without kSosFinal the plain
// sum is stored.
constexpr int kCols = 16;

__global__ void __launch_bounds__(256) fft_col_kernel(const float2 *__restrict__ in, float2 *__restrict__ out,
                                                      FftPlan1D pl, int y0, int ry, int ncols, long long stride,
                                                      long long in_outer_stride, long long out_outer_stride,
                                                      long long out_stride, const float2 *__restrict__ tw_g,
                                                      int coils, long long cstride, float *__restrict__ sos_out,
                                                      const float *__restrict__ deapod, int sos_mode)
{
    extern __shared__ float2 sm[];
    const int n = pl.n;
    float2 *tw = sm;
    float2 *b0 = tw + n;
    float2 *b1 = b0 + n * kCols;
    float *acc = reinterpret_cast<float *>(b1 + n * kCols);  // [ry][kCols] for the SoS stage
    for (int i = threadIdx.x; i < n; i += blockDim.x) tw[i] = tw_g[i];
    const int cblocks = (ncols + kCols - 1) / kCols;
    const long long outer = blockIdx.x / cblocks;
    const int c0 = (blockIdx.x % cblocks) * kCols;
    const int cw = min(kCols, ncols - c0);
    if (sos_out)
        for (int i = threadIdx.x; i < ry * kCols; i += blockDim.x) {
            const int e = i / kCols, c = i - e * kCols;
            acc[i] = (sos_mode & kSosAccIn) && c < cw ? sos_out[outer * out_outer_stride + c0 + e * out_stride + c] : 0.f;
        }
    for (int coil = 0; coil < (sos_out ? coils : 1); ++coil) {
        const float2 *src = in + coil * cstride + outer * in_outer_stride + c0;
        __syncthreads();
        for (int i = threadIdx.x; i < n * kCols; i += blockDim.x) {
            const int e = i / kCols, c = i - e * kCols;
            b0[i] = c < cw ? src[e * stride + c] : make_float2(0.f, 0.f);
        }
        __syncthreads();
        // lines are columns: line stride 1, element stride kCols
        float2 *res = line_fft(b0, b1, pl, kCols, 1, kCols, tw);
        if (sos_out) {
            for (int i = threadIdx.x; i < ry * kCols; i += blockDim.x) {
                const int e = i / kCols, c = i - e * kCols;
                const float2 v = res[(y0 + e) * kCols + c];
                // x * conj(x) of the reference's SOS: re*re - im*(-im)
                acc[i] = __fadd_rn(acc[i], __fsub_rn(__fmul_rn(v.x, v.x), __fmul_rn(v.y, -v.y)));
            }
        } else {
            float2 *dst = out + outer * out_outer_stride + c0;
            for (int i = threadIdx.x; i < ry * kCols; i += blockDim.x) {
                const int e = i / kCols, c = i - e * kCols;
                if (c < cw) dst[e * out_stride + c] = res[(y0 + e) * kCols + c];
            }
        }
    }
    if (sos_out) {
        __syncthreads();
        float *dst = sos_out + outer * out_outer_stride + c0;
        const float *dp = deapod ? deapod + outer * out_outer_stride + c0 : nullptr;
        for (int i = threadIdx.x; i < ry * kCols; i += blockDim.x) {
            const int e = i / kCols, c = i - e * kCols;
            if (c < cw) {
                float m = acc[i];
                if (sos_mode & kSosFinal) {
                    m = __fsqrt_rn(m);
                    if (dp) m = __fdiv_rn(m, dp[e * out_stride + c]);
                }
                dst[e * out_stride + c] = m;
            }
        }
    }
}

constexpr int kLinesX = 4;   // lines per CTA of the specialised x stage (128 threads)
constexpr int kThreadsX = 128;
constexpr int kColsCt = 8;   // columns per CTA of the specialised column stages

template <int N, int... Rs>
__global__ void __launch_bounds__(kThreadsX) fft_x_kernel_ct(const float2 *__restrict__ in, float2 *__restrict__ out,
                                                       long long nlines, int x0, int rx,
                                                       const float2 *__restrict__ tw_g)
{
    extern __shared__ float2 sm[];
    constexpr int LS = N + N / 32 + 1;  // padded line (pad_e) + 1 against line-to-line conflicts
    float2 *tw = sm;
    float2 *b0 = tw + N;
    float2 *b1 = b0 + kLinesX * LS;
    for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = tw_g[i];
    const long long l0 = (long long)blockIdx.x * kLinesX;
    const int lines = (int)min((long long)kLinesX, nlines - l0);
    for (int i = threadIdx.x; i < kLinesX * N; i += blockDim.x) {
        const int l = i / N, e = i - l * N;
        b0[l * LS + pad_e<1>(e)] = l < lines ? in[(l0 + l) * N + e] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    float2 *res = fft_passes<N, 1, kLinesX, LS, 1, Rs...>(b0, b1, tw);
    for (int i = threadIdx.x; i < lines * rx; i += blockDim.x) {
        const int l = i / rx, e = i - l * rx;
        out[(l0 + l) * rx + e] = res[l * LS + pad_e<1>(x0 + e)];
    }
}

template <int N, int... Rs>
__global__ void __launch_bounds__(256) fft_col_kernel_ct(const float2 *__restrict__ in, float2 *__restrict__ out,
                                                         int y0, int ry, int ncols, long long stride,
                                                         long long in_outer_stride, long long out_outer_stride,
                                                         long long out_stride, const float2 *__restrict__ tw_g,
                                                         int coils, long long cstride, float *__restrict__ sos_out,
                                                         const float *__restrict__ deapod, int sos_mode)
{
    extern __shared__ float2 sm[];
    constexpr int C = kColsCt;
    float2 *tw = sm;
    float2 *b0 = tw + N;
    float2 *b1 = b0 + N * C;
    float *acc = reinterpret_cast<float *>(b1 + N * C);  // [ry][C] for the SoS stage
    for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = tw_g[i];
    const int cblocks = (ncols + C - 1) / C;
    const long long outer = blockIdx.x / cblocks;
    const int c0 = (blockIdx.x % cblocks) * C;
    const int cw = min(C, ncols - c0);
    if (sos_out)
        for (int i = threadIdx.x; i < ry * C; i += blockDim.x) {
            const int e = i / C, c = i - e * C;
            acc[i] = (sos_mode & kSosAccIn) && c < cw ? sos_out[outer * out_outer_stride + c0 + e * out_stride + c] : 0.f;
        }
    for (int coil = 0; coil < (sos_out ? coils : 1); ++coil) {
        const float2 *src = in + coil * cstride + outer * in_outer_stride + c0;
        __syncthreads();
        for (int i = threadIdx.x; i < N * C; i += blockDim.x) {
            const int e = i / C, c = i - e * C;
            b0[i] = c < cw ? src[e * stride + c] : make_float2(0.f, 0.f);
        }
        __syncthreads();
        float2 *res = fft_passes<N, 1, C, 1, C, Rs...>(b0, b1, tw);
        if (sos_out) {
            for (int i = threadIdx.x; i < ry * C; i += blockDim.x) {
                const int e = i / C, c = i - e * C;
                const float2 v = res[(y0 + e) * C + c];
                // x * conj(x) of the reference's SOS: re*re - im*(-im)
                acc[i] = __fadd_rn(acc[i], __fsub_rn(__fmul_rn(v.x, v.x), __fmul_rn(v.y, -v.y)));
            }
        } else {
            float2 *dst = out + outer * out_outer_stride + c0;
            for (int i = threadIdx.x; i < ry * C; i += blockDim.x) {
                const int e = i / C, c = i - e * C;
                if (c < cw) dst[e * out_stride + c] = res[(y0 + e) * C + c];
            }
        }
    }
    if (sos_out) {
        __syncthreads();
        float *dst = sos_out + outer * out_outer_stride + c0;
        const float *dp = deapod ? deapod + outer * out_outer_stride + c0 : nullptr;
        for (int i = threadIdx.x; i < ry * C; i += blockDim.x) {
            const int e = i / C, c = i - e * C;
            if (c < cw) {
                float m = acc[i];
                if (sos_mode & kSosFinal) {
                    m = __fsqrt_rn(m);
                    if (dp) m = __fdiv_rn(m, dp[e * out_stride + c]);
                }
                dst[e * out_stride + c] = m;
            }
        }
    }
}

using FftXFn = void (*)(const float2 *, float2 *, long long, int, int, const float2 *);
using FftColFn = void (*)(const float2 *, float2 *, int, int, int, long long, long long, long long, long long,
                          const float2 *, int, long long, float *, const float *, int);
struct CtKernels {
    int n;
    FftXFn x;
    FftColFn col;
};

// Specialised sizes, radices in the order factor() chooses them.
#define FR_CT(N, ...) {N, fft_x_kernel_ct<N, __VA_ARGS__>, fft_col_kernel_ct<N, __VA_ARGS__>}
const CtKernels kCtKernels[] = {
    FR_CT(64, 8, 8),          FR_CT(128, 8, 8, 2),      FR_CT(160, 8, 5, 4),     FR_CT(192, 8, 8, 3),
    FR_CT(240, 8, 5, 3, 2),   FR_CT(256, 8, 8, 4),      FR_CT(320, 8, 8, 5),     FR_CT(384, 8, 8, 3, 2),
    FR_CT(480, 8, 5, 4, 3),   FR_CT(512, 8, 8, 8),      FR_CT(640, 8, 8, 5, 2),  FR_CT(768, 8, 8, 4, 3),
    FR_CT(1024, 8, 8, 8, 2),
};
#undef FR_CT

const CtKernels *ct_kernels(int n)
{
    for (const CtKernels &k : kCtKernels)
        if (k.n == n) return &k;
    return nullptr;
}

// Register two-step stages (fr_fft_reg.cuh) for the specialised sizes.
using FftXRegFn = void (*)(const float2 *, float2 *, long long, int, int, const float2 *, XMask);
using FftColRegFn = void (*)(const float2 *, float2 *, int, int, int, long long, long long, long long, long long,
                             const float2 *, int, long long, float *, const float *, int, int, long long);
struct RegKernels {
    int n;
    FftXRegFn x;
    FftColRegFn col, col_sos;
    size_t xsmem, colsmem;
    int xthreads, colthreads;
};
#define FR_REG(N)                                                                                            \
    {N, fft_x_kernel_reg<N>, fft_col_kernel_reg<N, false>, fft_col_kernel_reg<N, true>, reg_x_smem<N>(),      \
     reg_col_smem<N>(), kRegLinesX * RegSplit<N>::TH, kRegCols * RegSplit<N>::TH}
const RegKernels kRegKernels[] = {
    FR_REG(64),  FR_REG(128), FR_REG(160), FR_REG(192), FR_REG(240), FR_REG(256), FR_REG(320),
    FR_REG(384), FR_REG(480), FR_REG(512), FR_REG(640),
};
#undef FR_REG

constexpr int kColPer = 8;  // (coil, z) planes per CTA of the register y stage

const RegKernels *reg_kernels(int n)
{
    for (const RegKernels &k : kRegKernels)
        if (k.n == n) return &k;
    return nullptr;
}

bool factor(int n, FftPlan1D &pl)
{
    pl.n = n;
    pl.npass = 0;
    int m = n;
    const int radices[] = {8, 5, 4, 3, 2};
    while (m > 1) {
        bool ok = false;
        for (int r : radices) {
            if (m % r == 0) {
                if (pl.npass >= kMaxPasses) return false;
                pl.radix[pl.npass++] = r;
                m /= r;
                ok = true;
                break;
            }
        }
        if (!ok) return false;
    }
    return n >= 2 && n <= kMaxN;
}

}  // namespace

bool pruned_fft_specialised(int G) { return ct_kernels(G) != nullptr; }

}  // namespace fr

using namespace fr;

struct fr_fftcs_s {
    int dim = 3;
    unsigned G = 0;
    int channels = 0;
    unsigned out[3] = {0, 0, 0};
    FftPlan1D pl;
    DevBuf tw;    // G float2
    DevBuf b1;    // x-stage output
    DevBuf b2;    // y-stage output (3D)
    int lines_x = 8;
    const RegKernels *reg = nullptr;  // register two-step stages for this G (else Stockham passes)
    cufftHandle xplan = 0;  // 3D, specialised G without register stages: batched 1D x transforms
    DevBuf bx;              // their output: channels x G^3 complex
    ~fr_fftcs_s()
    {
        if (xplan) cufftDestroy(xplan);
    }
};

extern "C" {

int fr_fft_crop_sos_create(int dim, unsigned G, int channels, const unsigned *out_size, fr_fftcs *out)
{
    if (!out || !out_size || (dim != 2 && dim != 3) || channels < 1)
        return fail(FR_ERR_INVALID_ARGUMENT, "bad pruned FFT arguments");
    *out = nullptr;
    auto f = new (std::nothrow) fr_fftcs_s;
    if (!f) return fail(FR_ERR_OUT_OF_MEMORY, "pruned FFT");
    f->dim = dim;
    f->G = G;
    f->channels = channels;
    for (int i = 0; i < 3; ++i) f->out[i] = (i < dim) ? out_size[i] : 1u;
    if (!factor((int)G, f->pl) || f->out[0] > G || f->out[1] > G || (dim == 3 && f->out[2] > G)) {
        delete f;
        return fail(FR_ERR_UNSUPPORTED, "pruned FFT needs G = 2^a 3^b 5^c <= 1024 and out_size <= G");
    }
    // exp(+2 pi i t / G) in double, rounded to float
    std::vector<float2> tw(G);
    for (unsigned t = 0; t < G; ++t) {
        const double a = 2.0 * M_PI * (double)t / (double)G;
        tw[t] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    const size_t Gz = dim == 3 ? G : 1;
    {
        const char *st = std::getenv("FR_FFT_STOCKHAM");
        if (!(st && std::atoi(st) != 0)) f->reg = reg_kernels((int)G);
    }
    const bool cufft_x = dim == 3 && ct_kernels((int)G) != nullptr && !f->reg;
    if (f->tw.reserve(G * sizeof(float2)) ||
        (!cufft_x && f->b1.reserve((size_t)channels * Gz * G * f->out[0] * sizeof(float2))) ||
        (cufft_x && f->bx.reserve((size_t)channels * G * G * G * sizeof(float2))) ||
        (dim == 3 && f->b2.reserve((size_t)channels * G * f->out[1] * f->out[0] * sizeof(float2)))) {
        delete f;
        return FR_ERR_OUT_OF_MEMORY;
    }
    if (cufft_x) {
        int nn[1] = {(int)G};
        const long long lines = (long long)channels * G * G;
        if (lines > 0x7FFFFFFFll ||
            cufftPlanMany(&f->xplan, 1, nn, nullptr, 1, (int)G, nullptr, 1, (int)G, CUFFT_C2C, (int)lines) !=
                CUFFT_SUCCESS) {
            f->xplan = 0;
            delete f;
            return fail(FR_ERR_CUFFT, "cufftPlanMany (pruned FFT x stage)");
        }
    }
    cudaError_t e = cudaMemcpy(f->tw.ptr, tw.data(), G * sizeof(float2), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        delete f;
        return cuda_fail(e, "twiddle upload");
    }
    f->lines_x = 8;
    *out = f;
    return FR_OK;
}

int fr_fft_crop_sos_destroy(fr_fftcs f)
{
    delete f;
    return FR_OK;
}

}  // extern "C"

namespace fr {
// The pruned transform of `channels` <= the object's coils; sos_mode as in
// the column kernels (kSosFinal alone: the whole SoS of these coils).
bool fftcs_masks_tiles(fr_fftcs f) { return f && f->reg != nullptr; }

int fftcs_execute(fr_fftcs f, const float *d_grid, int channels, const float *d_deapod, float *d_out, int sos_mode,
                  cudaStream_t s, const TileMask *tiles)
{
    const int G = (int)f->G;
    const int C = channels;
    const int rx = f->out[0], ry = f->out[1], rz = f->out[2];
    const int x0 = (G - rx) / 2, y0 = (G - ry) / 2, z0 = (G - rz) / 2;
    const float2 *tw = f->tw.as<float2>();
    const float2 *grid = reinterpret_cast<const float2 *>(d_grid);
    float2 *b1 = f->b1.as<float2>();

    const long long Gz = f->dim == 3 ? G : 1;
    const long long nl = (long long)C * Gz * G;
    if (const RegKernels *rk = f->reg) {
        // register two-step stages: x (cropped), y (cropped), z or y with SoS
        if (rk->xsmem > 48 * 1024)
            FR_CUDA(cudaFuncSetAttribute(rk->x, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rk->xsmem));
        if (rk->colsmem > 48 * 1024) {
            FR_CUDA(cudaFuncSetAttribute(rk->col, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rk->colsmem));
            FR_CUDA(cudaFuncSetAttribute(rk->col_sos, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rk->colsmem));
        }
        XMask xm{};
        if (tiles && tiles->bits) {
            auto lg = [](int v) { return (v & (v - 1)) == 0 ? __builtin_ctz((unsigned)v) : -1; };
            xm = XMask{tiles->bits, lg(tiles->tile[0]), lg(tiles->tile[1]), lg(tiles->tile[2]), tiles->ntile[0],
                       tiles->ntile[1], G, (int)Gz, FastDiv((unsigned)G), FastDiv((unsigned)Gz)};
            if (xm.sx < 0 || xm.sy < 0 || xm.sz < 0)
                return fail(FR_ERR_UNSUPPORTED, "tile masks need power-of-two tile edges");
            if (nl >= (1ll << 31)) return fail(FR_ERR_UNSUPPORTED, "more than 2^31 lines in a tile-masked transform");
        }
        rk->x<<<(unsigned)((nl + kRegLinesX - 1) / kRegLinesX), rk->xthreads, rk->xsmem, s>>>(grid, b1, nl, x0, rx, tw,
                                                                                          xm);
        FR_CHECK_LAUNCH("fft_x_kernel_reg");
        const int cb = (rx + kRegCols - 1) / kRegCols;
        if (f->dim == 2) {
            rk->col_sos<<<cb, rk->colthreads, rk->colsmem, s>>>(b1, nullptr, y0, ry, rx, rx, 0, 0, rx, tw, C,
                                                            (long long)G * rx, d_out, d_deapod, sos_mode, 1, 1);
            FR_CHECK_LAUNCH("fft_col_kernel_reg(y, sos)");
            return FR_OK;
        }
        float2 *b2 = f->b2.as<float2>();
        // y stage: kColPer consecutive (coil, z) planes per CTA
        const long long nouter = (long long)C * G;
        rk->col<<<(unsigned)((nouter + kColPer - 1) / kColPer * cb), rk->colthreads, rk->colsmem, s>>>(
            b1, b2, y0, ry, rx, rx, (long long)G * rx, (long long)ry * rx, rx, tw, 1, 0, nullptr, nullptr, 0, kColPer,
            nouter);
        FR_CHECK_LAUNCH("fft_col_kernel_reg(y)");
        rk->col_sos<<<(unsigned)((long long)ry * cb), rk->colthreads, rk->colsmem, s>>>(
            b2, nullptr, z0, rz, rx, (long long)ry * rx, rx, rx, (long long)ry * rx, tw, C, (long long)G * ry * rx, d_out,
            d_deapod, sos_mode, 1, ry);
        FR_CHECK_LAUNCH("fft_col_kernel_reg(z, sos)");
        return FR_OK;
    }
    if (const CtKernels *ck = ct_kernels(G); ck && f->xplan) {
        // 3D, specialised size: x by cuFFT (out of place; C2C leaves its input
        // intact), then the y and z stages on the cropped x columns
        if (cufftSetStream(f->xplan, s) != CUFFT_SUCCESS ||
            cufftExecC2C(f->xplan, (cufftComplex *)const_cast<float2 *>(grid), f->bx.as<cufftComplex>(),
                         CUFFT_INVERSE) != CUFFT_SUCCESS)
            return fail(FR_ERR_CUFFT, "cufftExecC2C (pruned FFT x stage)");
        const size_t smc = (size_t)(G + 2 * G * kColsCt) * sizeof(float2) + (size_t)G * kColsCt * sizeof(float);
        if (smc > 48 * 1024)
            FR_CUDA(cudaFuncSetAttribute(ck->col, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smc));
        const int cb = (rx + kColsCt - 1) / kColsCt;
        float2 *b2 = f->b2.as<float2>();
        // y stage: input bx[c][z][y][x], columns x0..x0+rx, element (y) stride G
        ck->col<<<(unsigned)((long long)C * G * cb), 256, smc, s>>>(f->bx.as<float2>() + x0, b2, y0, ry, rx, G,
                                                                   (long long)G * G, (long long)ry * rx, rx, tw, 1, 0,
                                                                   nullptr, nullptr, 0);
        FR_CHECK_LAUNCH("fft_col_kernel_ct(y)");
        ck->col<<<(unsigned)((long long)ry * cb), 256, smc, s>>>(b2, nullptr, z0, rz, rx, (long long)ry * rx, rx, rx,
                                                                (long long)ry * rx, tw, C, (long long)G * ry * rx,
                                                                d_out, d_deapod, sos_mode);
        FR_CHECK_LAUNCH("fft_col_kernel_ct(z, sos)");
        return FR_OK;
    }
    if (const CtKernels *ck = ct_kernels(G)) {
        // specialised sizes
        const size_t smx = (size_t)(G + 2 * kLinesX * (G + G / 32 + 1)) * sizeof(float2);
        if (smx > 48 * 1024) FR_CUDA(cudaFuncSetAttribute(ck->x, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smx));
        ck->x<<<(unsigned)((nl + kLinesX - 1) / kLinesX), kThreadsX, smx, s>>>(grid, b1, nl, x0, rx, tw);
        FR_CHECK_LAUNCH("fft_x_kernel_ct");
        const size_t smc = (size_t)(G + 2 * G * kColsCt) * sizeof(float2) + (size_t)G * kColsCt * sizeof(float);
        if (smc > 48 * 1024)
            FR_CUDA(cudaFuncSetAttribute(ck->col, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smc));
        const int cb = (rx + kColsCt - 1) / kColsCt;
        if (f->dim == 2) {
            ck->col<<<cb, 256, smc, s>>>(b1, nullptr, y0, ry, rx, rx, 0, 0, rx, tw, C, (long long)G * rx, d_out,
                                         d_deapod, sos_mode);
            FR_CHECK_LAUNCH("fft_col_kernel_ct(y, sos)");
            return FR_OK;
        }
        float2 *b2 = f->b2.as<float2>();
        ck->col<<<(unsigned)((long long)C * G * cb), 256, smc, s>>>(b1, b2, y0, ry, rx, rx, (long long)G * rx,
                                                                   (long long)ry * rx, rx, tw, 1, 0, nullptr, nullptr, 0);
        FR_CHECK_LAUNCH("fft_col_kernel_ct(y)");
        ck->col<<<(unsigned)((long long)ry * cb), 256, smc, s>>>(b2, nullptr, z0, rz, rx, (long long)ry * rx, rx, rx,
                                                                (long long)ry * rx, tw, C, (long long)G * ry * rx,
                                                                d_out, d_deapod, sos_mode);
        FR_CHECK_LAUNCH("fft_col_kernel_ct(z, sos)");
        return FR_OK;
    }
    // x stage over all lines of all coils
    const int L = f->lines_x;
    size_t smx = (size_t)(G + 2 * L * (G + 1)) * sizeof(float2);
    if (smx > 48 * 1024) FR_CUDA(cudaFuncSetAttribute(fft_x_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smx));
    fft_x_kernel<<<(unsigned)((nl + L - 1) / L), 256, smx, s>>>(grid, b1, nl, f->pl, x0, rx, tw, L);
    FR_CHECK_LAUNCH("fft_x_kernel");

    size_t smc = (size_t)(G + 2 * G * kCols) * sizeof(float2) + (size_t)G * kCols * sizeof(float);
    if (smc > 48 * 1024)
        FR_CUDA(cudaFuncSetAttribute(fft_col_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smc));
    const int cblocks = (rx + kCols - 1) / kCols;
    if (f->dim == 2) {
        // y stage + SoS: outer = nothing (one plane), columns = x'
        // input b1[c][y][x'] : element stride rx, coil stride G*rx
        fft_col_kernel<<<cblocks, 256, smc, s>>>(b1, nullptr, f->pl, y0, ry, rx, rx, 0, 0, rx, tw, C,
                                                 (long long)G * rx, d_out, d_deapod, sos_mode);
        FR_CHECK_LAUNCH("fft_col_kernel(y, sos)");
        return FR_OK;
    }
    // y stage: outer = (c, z), columns = x', input b1[c][z][y][x']
    float2 *b2 = f->b2.as<float2>();
    fft_col_kernel<<<(unsigned)((long long)C * G * cblocks), 256, smc, s>>>(
        b1, b2, f->pl, y0, ry, rx, rx, (long long)G * rx, (long long)ry * rx, rx, tw, 1, 0, nullptr, nullptr, 0);
    FR_CHECK_LAUNCH("fft_col_kernel(y)");
    // z stage + SoS: outer = y', columns = x', input b2[c][z][y'][x'] with
    // element (z) stride ry*rx, coil stride G*ry*rx; output out[z'][y'][x']
    fft_col_kernel<<<(unsigned)((long long)ry * cblocks), 256, smc, s>>>(
        b2, nullptr, f->pl, z0, rz, rx, (long long)ry * rx, rx, rx, (long long)ry * rx, tw, C,
        (long long)G * ry * rx, d_out, d_deapod, sos_mode);
    FR_CHECK_LAUNCH("fft_col_kernel(z, sos)");
    return FR_OK;
}
}  // namespace fr

extern "C" {

int fr_fft_crop_sos_execute(fr_fftcs f, const float *d_grid, const float *d_deapod, float *d_out, void *stream)
{
    if (!f || !d_grid || !d_out) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    return fftcs_execute(f, d_grid, f->channels, d_deapod, d_out, kSosFinal, (cudaStream_t)stream);
}

}  // extern "C"
