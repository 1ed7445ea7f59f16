// fr_fft_reg.cuh -- two-step register FFT stages of the pruned transform.
//
// A line of length N = T * M is transformed by two sets of in-register DFTs
// with one exchange through shared memory (n = t + T m, k = k1 + M k2):
//   step A: T threads per line; thread t loads x[t + T m] (m < M), computes
//           a DFT of length M over m, multiplies output k1 by W_N^(t k1) and
//           stores it at [k1][t];
//   step B: M threads per line; thread k1 loads [k1][t] (t < T), computes a
//           DFT of length T over t and holds X[k1 + M k2] (k2 < T).
// W = exp(+2 pi i / N) (backward transform).  Every element crosses shared
// memory once instead of once per radix pass, and the global loads of step A
// are issued M at a time per thread.  Included by fr_fft.cu inside its
// anonymous namespace (uses cadd/csub/cmul/cmuli and dft2..dft8).
#pragma once

#include <type_traits>

// ---------------------------------------------------------------- constants

constexpr double kPiD = 3.141592653589793238462643383279502884;

// Taylor series on |x| <= pi/4 (12 terms: truncation far below double
// rounding there).
__host__ __device__ constexpr double cx_sin_r(double x)
{
    double x2 = x * x, term = x, sum = x;
    for (int i = 1; i < 12; ++i) {
        term *= -x2 / (double)((2 * i) * (2 * i + 1));
        sum += term;
    }
    return sum;
}
__host__ __device__ constexpr double cx_cos_r(double x)
{
    double x2 = x * x, term = 1.0, sum = 1.0;
    for (int i = 1; i < 12; ++i) {
        term *= -x2 / (double)((2 * i - 1) * (2 * i));
        sum += term;
    }
    return sum;
}
struct CxD {
    double re, im;
};
// exp(+2 pi i k / n) at compile time: the angle is q * pi/2 + x with q the
// nearest quadrant and |x| <= pi/4.
__host__ __device__ constexpr CxD cx_twiddle(long long k, long long n)
{
    k %= n;
    if (k < 0) k += n;
    const long long q = (8 * k + n) / (2 * n);  // round(4 k / n)
    const double x = (double)(4 * k - q * n) / (double)n * (kPiD / 2);
    const double c = cx_cos_r(x), s = cx_sin_r(x);
    switch (q & 3) {
    case 0: return CxD{c, s};
    case 1: return CxD{-s, c};
    case 2: return CxD{-c, -s};
    default: return CxD{s, -c};
    }
}

// a * exp(+2 pi i K / N) with the twiddle folded at compile time.
template <int K, int N>
__device__ __forceinline__ float2 twmul(float2 a)
{
    constexpr int k = ((K % N) + N) % N;
    if constexpr (k == 0) {
        return a;
    } else if constexpr (4 * k == N) {
        return cmuli(a);
    } else if constexpr (2 * k == N) {
        return make_float2(-a.x, -a.y);
    } else if constexpr (4 * k == 3 * N) {
        return make_float2(a.y, -a.x);
    } else {
        constexpr CxD w = cx_twiddle(k, N);
        constexpr float wr = (float)w.re, wi = (float)w.im;
        return make_float2(a.x * wr - a.y * wi, a.x * wi + a.y * wr);
    }
}

template <int I, int N, typename F>
__device__ __forceinline__ void static_for(F &&f)
{
    if constexpr (I < N) {
        f(std::integral_constant<int, I>{});
        static_for<I + 1, N>(f);
    }
}

// Radix taken first by the recursive register DFT.
__host__ __device__ constexpr int reg_radix(int n)
{
    return n % 8 == 0 ? 8 : n % 4 == 0 ? 4 : n % 2 == 0 ? 2 : n % 3 == 0 ? 3 : 5;
}

// In-register DFT of length N (natural order in and out), exp(+2 pi i / N):
// n = Q p + q, k = k1 + P k2 with P = reg_radix(N), Q = N / P.
template <int N>
__device__ __forceinline__ void rdft(float2 *v)
{
    if constexpr (N == 1) {
        return;
    } else if constexpr (N == 2 || N == 3 || N == 4 || N == 5 || N == 8) {
        dft<N>(v);
    } else {
        constexpr int P = reg_radix(N), Q = N / P;
        float2 a[N];  // a[Q k1 + q] = W_N^(q k1) * DFT_P over p of v[Q p + q]
        static_for<0, Q>([&](auto qc) {
            constexpr int q = decltype(qc)::value;
            float2 t[P];
            static_for<0, P>([&](auto pc) { t[decltype(pc)::value] = v[Q * decltype(pc)::value + q]; });
            dft<P>(t);
            static_for<0, P>([&](auto kc) {
                constexpr int k1 = decltype(kc)::value;
                a[Q * k1 + q] = twmul<q * k1, N>(t[k1]);
            });
        });
        static_for<0, P>([&](auto kc) {
            constexpr int k1 = decltype(kc)::value;
            rdft<Q>(a + Q * k1);
            static_for<0, Q>([&](auto k2c) { v[k1 + P * decltype(k2c)::value] = a[Q * k1 + decltype(k2c)::value]; });
        });
    }
}

// ------------------------------------------------------------------ kernels

template <int N>
struct RegSplit {
    static constexpr int T = N > 768 ? 32 : 16;  // step A threads per line
    static constexpr int M = N / T;              // step B threads per line
    static constexpr int TH = T > M ? T : M;     // threads per line
};

constexpr int kRegLinesX = 8;  // lines per CTA of the register x stage
constexpr int kRegCols = 16;   // columns per CTA of the register column stages (128-byte rows)

// Cells the gridding left unwritten (tiles without samples) read as zero:
// bit ((z >> sz) * nty + (y >> sy)) * ntx + (x >> sx) of `bits` is set for
// written tiles (power-of-two tile edges; bits == nullptr: every cell).
// n / d for n < 2^31 by a multiply and a shift: m = ceil(2^s / d) with
// s = 31 + ceil(log2 d) leaves an error below 2^-ceil(log2 d) <= 1/d in
// n * m / 2^s, too small to reach the next integer.
struct FastDiv {
    unsigned d = 1, m = 0x80000000u;
    int s = 31;
    FastDiv() = default;
    explicit FastDiv(unsigned dd) : d(dd)
    {
        int l = 0;
        while ((1ull << l) < dd) ++l;
        s = 31 + l;
        m = (unsigned)(((1ull << s) + dd - 1) / dd);
    }
    __device__ __forceinline__ unsigned div(unsigned n) const
    {
        return (unsigned)(((unsigned long long)n * m) >> s);
    }
};

struct XMask {
    const unsigned *bits;
    int sx, sy, sz, ntx, nty, G, Gz;
    FastDiv by_g, by_gz;  // line -> (y, z) without divisions
};

// x stage: kRegLinesX contiguous lines of length N per CTA, outputs
// [x0, x0 + rx) of each line.  in: nlines x N, out: nlines x rx.
template <int N>
__global__ void __launch_bounds__(kRegLinesX * RegSplit<N>::TH) fft_x_kernel_reg(
    const float2 *__restrict__ in, float2 *__restrict__ out, long long nlines, int x0, int rx,
    const float2 *__restrict__ tw_g, XMask xm)
{
    constexpr int T = RegSplit<N>::T, M = RegSplit<N>::M;
    constexpr int LS = M * (T + 1);  // [k1][t] with one pad slot per row
    extern __shared__ float2 sm[];
    // twiddles of step A by (k1, t): tw[k1 T + t] = W^(t k1) (t k1 < T M = N),
    // so the 16 lanes of a line read 16 consecutive entries
    float2 *tw = sm;
    float2 *ex = tw + N;
    for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = tw_g[(i % T) * (i / T)];
    const long long l0 = (long long)blockIdx.x * kRegLinesX;
    __syncthreads();
    if (threadIdx.x < kRegLinesX * T) {
        const int l = threadIdx.x / T, t = threadIdx.x % T;
        const long long line = l0 + l;
        float2 v[M];
        if (line < nlines && xm.bits) {
            // nlines = coils * Gz * G < 2^31 (checked by the caller)
            const unsigned yz = xm.by_g.div((unsigned)line), cz = xm.by_gz.div(yz);
            const int y = (int)((unsigned)line - yz * (unsigned)xm.G), z = (int)(yz - cz * (unsigned)xm.Gz);
            const int tb = ((z >> xm.sz) * xm.nty + (y >> xm.sy)) * xm.ntx;
            const float2 *src = in + line * N + t;
#pragma unroll
            for (int m = 0; m < M; ++m) {
                const int tile = tb + ((t + T * m) >> xm.sx);
                v[m] = (xm.bits[tile >> 5] >> (tile & 31)) & 1u ? src[T * m] : make_float2(0.f, 0.f);
            }
        } else if (line < nlines) {
            const float2 *src = in + line * N + t;
#pragma unroll
            for (int m = 0; m < M; ++m) v[m] = src[T * m];
        } else {
#pragma unroll
            for (int m = 0; m < M; ++m) v[m] = make_float2(0.f, 0.f);
        }
        rdft<M>(v);
        float2 *dst = ex + l * LS + t;
        dst[0] = v[0];
#pragma unroll
        for (int k1 = 1; k1 < M; ++k1) dst[k1 * (T + 1)] = cmul(v[k1], tw[k1 * T + t]);
    }
    __syncthreads();
    if (threadIdx.x < kRegLinesX * M) {
        const int l = threadIdx.x / M, k1 = threadIdx.x % M;
        const long long line = l0 + l;
        float2 b[T];
        const float2 *src = ex + l * LS + k1 * (T + 1);
#pragma unroll
        for (int t = 0; t < T; ++t) b[t] = src[t];
        rdft<T>(b);
        if (line < nlines) {
            float2 *o = out + line * rx - x0;
#pragma unroll
            for (int k2 = 0; k2 < T; ++k2) {
                const int k = k1 + M * k2;
                if (k >= x0 && k < x0 + rx) o[k] = b[k2];
            }
        }
    }
}

// Column stage: for each (outer, block of kRegCols columns) transform the
// lines along an axis of length N with element stride `stride`, keep outputs
// [y0, y0 + ry).  Input index: coil * cstride + outer * in_outer_stride +
// e * stride + column.  Without `sos_out` one coil is transformed and written
// to out[outer * out_outer_stride + (k - y0) * out_stride + column]; with it
// |X|^2 is summed over `coils` in coil order, then sqrt (and / deapod) goes
// to sos_out at the same offsets.
template <int N, bool SOS>
__global__ void __launch_bounds__(kRegCols * RegSplit<N>::TH, N <= 384 ? 2 : 1) fft_col_kernel_reg(
    const float2 *__restrict__ in, float2 *__restrict__ out, int y0, int ry, int ncols, long long stride,
    long long in_outer_stride, long long out_outer_stride, long long out_stride, const float2 *__restrict__ tw_g,
    int coils, long long cstride, float *__restrict__ sos_out, const float *__restrict__ deapod, int sos_mode,
    int per, long long nouter)
{
    constexpr int T = RegSplit<N>::T, M = RegSplit<N>::M;
    constexpr int CB = kRegCols;
    extern __shared__ float2 sm[];
    float2 *tw = sm;
    float2 *ex = tw + N;  // [k1][t][column]
    // The CTA's units, one after the other: with SOS the coils of one outer,
    // else `per` consecutive outers of one coil.  The next unit's input block
    // [e][column] is filled by cp.async while the current unit's second step
    // runs (whole 16-byte column pairs only).
    float2 *stage = ex + N * CB;
    for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = tw_g[i];
    const int cblocks = (ncols + CB - 1) / CB;
    const long long outer0 = SOS ? blockIdx.x / cblocks : (long long)(blockIdx.x / cblocks) * per;
    const long long outer = outer0;  // the SoS outer
    const int c0 = (blockIdx.x % cblocks) * CB;
    const int col = threadIdx.x % CB;
    const bool col_ok = c0 + col < ncols;
    const bool pipe = ncols % CB == 0 && ((stride | in_outer_stride | cstride) & 1) == 0 &&
                      (reinterpret_cast<uintptr_t>(in) & 15) == 0;
    auto issue = [&](int unit) {
        const float2 *src = in + (SOS ? unit * cstride + outer0 * in_outer_stride : (outer0 + unit) * in_outer_stride) + c0;
        for (int i = threadIdx.x; i < N * CB / 2; i += blockDim.x) {
            const int e = i / (CB / 2), cc = 2 * (i % (CB / 2));
            const unsigned dst = (unsigned)__cvta_generic_to_shared(stage + e * CB + cc);
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src + (long long)e * stride + cc)
                         : "memory");
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    float acc[SOS ? T : 1];
#pragma unroll
    for (int k2 = 0; k2 < (SOS ? T : 1); ++k2) acc[k2] = 0.f;
    if (SOS && (sos_mode & kSosAccIn) && threadIdx.x < CB * M && col_ok) {
        // coils in slabs: continue the previous slabs' sum
        const int k1 = threadIdx.x / CB;
        const float *o = sos_out + outer * out_outer_stride + c0 + col;
#pragma unroll
        for (int k2 = 0; k2 < T; ++k2) {
            const int k = k1 + M * k2;
            if (k >= y0 && k < y0 + ry) acc[k2] = o[(long long)(k - y0) * out_stride];
        }
    }
    const int nunit = SOS ? coils : (int)min((long long)per, nouter - outer0);
    if (pipe) issue(0);
    for (int u = 0; u < nunit; ++u) {
        const int coil = SOS ? u : 0;
        const long long ou = SOS ? outer0 : outer0 + u;
        if (pipe) asm volatile("cp.async.wait_group 0;" ::: "memory");
        __syncthreads();  // twiddles staged; the previous unit's exchange is read; this unit's block landed
        if (threadIdx.x < CB * T) {
            const int t = threadIdx.x / CB;
            float2 v[M];
            if (pipe) {
#pragma unroll
                for (int m = 0; m < M; ++m) v[m] = stage[(t + T * m) * CB + col];
            } else {
                const float2 *src = in + coil * cstride + ou * in_outer_stride + (long long)t * stride + c0 + col;
#pragma unroll
                for (int m = 0; m < M; ++m) v[m] = col_ok ? src[(long long)(T * m) * stride] : make_float2(0.f, 0.f);
            }
            rdft<M>(v);
            float2 *dst = ex + t * CB + col;
            dst[0] = v[0];
#pragma unroll
            for (int k1 = 1; k1 < M; ++k1) dst[k1 * T * CB] = cmul(v[k1], tw[t * k1]);
        }
        __syncthreads();
        if (pipe && u + 1 < nunit) issue(u + 1);  // the block is free: every thread passed step A
        if (threadIdx.x < CB * M) {
            const int k1 = threadIdx.x / CB;
            float2 b[T];
            const float2 *src = ex + k1 * T * CB + col;
#pragma unroll
            for (int t = 0; t < T; ++t) b[t] = src[t * CB];
            rdft<T>(b);
            if constexpr (SOS) {
#pragma unroll
                for (int k2 = 0; k2 < T; ++k2)
                    // x * conj(x) of the reference's SOS: re*re - im*(-im)
                    acc[k2] = __fadd_rn(acc[k2], __fsub_rn(__fmul_rn(b[k2].x, b[k2].x), __fmul_rn(b[k2].y, -b[k2].y)));
            } else if (col_ok) {
                float2 *o = out + ou * out_outer_stride + c0 + col;
#pragma unroll
                for (int k2 = 0; k2 < T; ++k2) {
                    const int k = k1 + M * k2;
                    if (k >= y0 && k < y0 + ry) o[(long long)(k - y0) * out_stride] = b[k2];
                }
            }
        }
    }
    if (SOS && threadIdx.x < CB * M && col_ok) {
        const int k1 = threadIdx.x / CB;
        float *o = sos_out + outer * out_outer_stride + c0 + col;
        const float *dp = deapod ? deapod + outer * out_outer_stride + c0 + col : nullptr;
#pragma unroll
        for (int k2 = 0; k2 < T; ++k2) {
            const int k = k1 + M * k2;
            if (k >= y0 && k < y0 + ry) {
                float m = acc[k2];
                if (sos_mode & kSosFinal) {
                    m = __fsqrt_rn(m);
                    if (dp) m = __fdiv_rn(m, dp[(long long)(k - y0) * out_stride]);
                }
                o[(long long)(k - y0) * out_stride] = m;
            }
        }
    }
}

template <int N>
constexpr size_t reg_x_smem()
{
    return (size_t)(N + kRegLinesX * RegSplit<N>::M * (RegSplit<N>::T + 1)) * sizeof(float2);
}
// twiddles, exchange buffer and the next unit's input block
template <int N>
constexpr size_t reg_col_smem()
{
    return (size_t)(N + 2 * N * kRegCols) * sizeof(float2);
}
