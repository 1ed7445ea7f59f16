// fr_mlp.cu -- the learned-DCF network: 5 -> 64 -> 64 -> 1, tanh, predicting
// log-DCF from sample-density features.  No counterpart in the reference.
//
// Parameters are kept as an FP32 master copy (optimiser state) and a BF16
// copy that the forward and backward kernels read; all arithmetic is FP32.
// Layout (FR_MLP_PARAMS values): W1[64][5] | b1[64] | W2[64][64] | b2[64] |
// W3[64] | b3.
//
//  * mlp_forward_mma_kernel (inference): the hidden layer on the tensor
//    cores (mma.sync, BF16 operands in three terms, FP32 accumulation).
//  * mlp_forward_kernel (FR_MLP_SIMT=1): one thread per sample, the BF16
//    parameters widened into shared memory once per CTA; first-layer units
//    are produced one at a time and scattered into the 64 second-layer
//    accumulators held in registers.
//  * backward: mlp_train_kernel does the forward pass and the per-sample
//    reverse pass (dL/dy, the two hidden-layer deltas) and writes the
//    per-sample activations and deltas; mlp_grad_kernel reduces the
//    outer products over a block of samples into one partial gradient per
//    CTA; mlp_reduce_kernel sums the partials in a fixed order (the
//    gradient is deterministic).
//  * mlp_adam_kernel: Adam on the master copy, then the BF16 copy.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>

#include "fr_internal.h"

namespace fr {
namespace {

constexpr int NI = FR_MLP_IN;
constexpr int NH = FR_MLP_HIDDEN;
constexpr int OFF_W1 = 0;
constexpr int OFF_B1 = OFF_W1 + NH * NI;
constexpr int OFF_W2 = OFF_B1 + NH;
constexpr int OFF_B2 = OFF_W2 + NH * NH;
constexpr int OFF_W3 = OFF_B2 + NH;
constexpr int OFF_B3 = OFF_W3 + NH;
constexpr int NP = OFF_B3 + 1;
static_assert(NP == FR_MLP_PARAMS, "parameter layout");

constexpr int kGradSamples = 256;  // samples reduced by one mlp_grad_kernel CTA
constexpr int kFwdThreads = 128;

// Widen the BF16 parameters into shared memory, W2 transposed (row i of the
// shared copy holds W2[.][i]) so that both passes read it along rows.
__device__ __forceinline__ void load_params(const __nv_bfloat16 *__restrict__ pb, float *ps)
{
    for (int p = threadIdx.x; p < NP; p += blockDim.x) {
        int q = p;
        if (p >= OFF_W2 && p < OFF_B2) {
            const int j = (p - OFF_W2) / NH, i = (p - OFF_W2) % NH;
            q = OFF_W2 + i * NH + j;
        }
        ps[q] = __bfloat162float(pb[p]);
    }
    __syncthreads();
}

// Hidden unit i of the first layer.
__device__ __forceinline__ float unit1(const float *ps, const float *x, int i)
{
    float a = ps[OFF_B1 + i];
#pragma unroll
    for (int k = 0; k < NI; ++k) a = fmaf(ps[OFF_W1 + i * NI + k], x[k], a);
    return tanhf(a);
}

// acc[j] += W2[j][i] * v for all j (row i of the transposed copy).
__device__ __forceinline__ void axpy_row(const float *ps, int i, float v, float *acc)
{
    const float4 *w = reinterpret_cast<const float4 *>(ps + OFF_W2 + i * NH);
#pragma unroll
    for (int q = 0; q < NH / 4; ++q) {
        const float4 c = w[q];
        acc[4 * q] = fmaf(c.x, v, acc[4 * q]);
        acc[4 * q + 1] = fmaf(c.y, v, acc[4 * q + 1]);
        acc[4 * q + 2] = fmaf(c.z, v, acc[4 * q + 2]);
        acc[4 * q + 3] = fmaf(c.w, v, acc[4 * q + 3]);
    }
}

// sum_j W2[j][i] * d[j] (row i of the transposed copy).
__device__ __forceinline__ float dot_row(const float *ps, int i, const float *d)
{
    const float4 *w = reinterpret_cast<const float4 *>(ps + OFF_W2 + i * NH);
    float a = 0.f;
#pragma unroll
    for (int q = 0; q < NH / 4; ++q) {
        const float4 c = w[q];
        a = fmaf(c.x, d[4 * q], a);
        a = fmaf(c.y, d[4 * q + 1], a);
        a = fmaf(c.z, d[4 * q + 2], a);
        a = fmaf(c.w, d[4 * q + 3], a);
    }
    return a;
}

// Second-layer activations h2 (in place of the pre-activations) and the output.
__device__ __forceinline__ float forward_sample(const float *ps, const float *xs, float *h2)
{
#pragma unroll
    for (int j = 0; j < NH; ++j) h2[j] = ps[OFF_B2 + j];
#pragma unroll 1
    for (int i = 0; i < NH; ++i) axpy_row(ps, i, unit1(ps, xs, i), h2);
    float out = ps[OFF_B3];
#pragma unroll
    for (int j = 0; j < NH; ++j) {
        h2[j] = tanhf(h2[j]);
        out = fmaf(ps[OFF_W3 + j], h2[j], out);
    }
    return out;
}

__global__ void __launch_bounds__(kFwdThreads) mlp_forward_kernel(const __nv_bfloat16 *__restrict__ pb,
                                                                  const float *__restrict__ x, long long n, int exp_out,
                                                                  int residual, float scale, float *__restrict__ y)
{
    __shared__ __align__(16) float ps[NP + 3];
    load_params(pb, ps);
    for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < n; s += (long long)gridDim.x * blockDim.x) {
        float xs[NI], h2[NH];
#pragma unroll
        for (int k = 0; k < NI; ++k) xs[k] = x[s * NI + k];
        float out = forward_sample(ps, xs, h2);
        if (residual) out = __fsub_rn(out, xs[1]);  // the network predicts log-DCF + log density (radius 2)
        y[s] = exp_out ? __fmul_rn(scale, expf(out)) : out;
    }
}

// The forward pass with the hidden layer (64 x 64) on the tensor cores:
// mma.sync m16n8k16, BF16 operands, FP32 accumulation.  One warp holds a
// tile of 16 samples: each lane evaluates, in FP32 as forward_sample does,
// exactly the first-layer activations its A fragments hold (2 samples x 16
// units), splits each into three BF16 terms hi + mid + lo (the residual of
// a BF16 rounding, twice: together within ~2^-24 of the FP32 value), and the
// warp accumulates W2 h1 = W2 hi + W2 mid + W2 lo into FP32 fragments that
// start from b2; the weights are BF16 already, so every product is exact
// and the sums carry FP32 rounding only.  The output layer reduces each
// lane's 16 units and the 4 lanes of a row with shuffles.
__device__ __forceinline__ unsigned pack_bf16(float lo_half, float hi_half)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo_half, hi_half);
    return *reinterpret_cast<const unsigned *>(&v);
}

__device__ __forceinline__ void mma_bf16_16816(float *d, const unsigned *a, unsigned b0, unsigned b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

constexpr int kMmaThreads = 128;  // 4 warps, 16 samples each per step

__global__ void __launch_bounds__(kMmaThreads) mlp_forward_mma_kernel(const __nv_bfloat16 *__restrict__ pb,
                                                                      const float *__restrict__ x, long long n,
                                                                      int exp_out, int residual, float scale,
                                                                      float *__restrict__ y)
{
    __shared__ __align__(16) __nv_bfloat16 pw[NP + 7];
    for (int p = threadIdx.x; p < NP; p += blockDim.x) pw[p] = pb[p];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int g = lane >> 2, tig = lane & 3;
    const unsigned *w2 = reinterpret_cast<const unsigned *>(pw + OFF_W2);  // bf16 pairs of W2[j][i], i fastest
    const long long ntile = (n + 15) / 16;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long tile = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5); tile < ntile;
         tile += warps) {
        const long long s0 = tile * 16 + g, s1 = s0 + 8;
        float x0[NI], x1[NI];
#pragma unroll
        for (int k = 0; k < NI; ++k) {
            x0[k] = s0 < n ? x[s0 * NI + k] : 0.f;
            x1[k] = s1 < n ? x[s1 * NI + k] : 0.f;
        }
        float acc[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int j = 8 * nt + 2 * tig;
            acc[nt][0] = acc[nt][2] = __bfloat162float(pw[OFF_B2 + j]);
            acc[nt][1] = acc[nt][3] = __bfloat162float(pw[OFF_B2 + j + 1]);
        }
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
            // this lane's first-layer units: i0 + {0, 1} and i0 + 8 + {0, 1}
            const int i0 = 16 * ks + 2 * tig;
            float h[2][4];  // [sample row g / g + 8][unit i0, i0 + 1, i0 + 8, i0 + 9]
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int i = i0 + (u & 1) + (u >> 1) * 8;
                float a0 = __bfloat162float(pw[OFF_B1 + i]), a1 = a0;
#pragma unroll
                for (int k = 0; k < NI; ++k) {
                    const float wk = __bfloat162float(pw[OFF_W1 + i * NI + k]);
                    a0 = fmaf(wk, x0[k], a0);
                    a1 = fmaf(wk, x1[k], a1);
                }
                h[0][u] = tanhf(a0);
                h[1][u] = tanhf(a1);
            }
            // three BF16 terms per activation; A registers: a0a1 row g k lo,
            // a2a3 row g+8 k lo, a4a5 row g k hi, a6a7 row g+8 k hi
            unsigned A[3][4];
#pragma unroll
            for (int r = 0; r < 2; ++r)
#pragma unroll
                for (int qq = 0; qq < 2; ++qq) {
                    const float v0 = h[r][2 * qq], v1 = h[r][2 * qq + 1];
                    const float hi0 = __bfloat162float(__float2bfloat16_rn(v0));
                    const float hi1 = __bfloat162float(__float2bfloat16_rn(v1));
                    const float r0 = __fsub_rn(v0, hi0), r1 = __fsub_rn(v1, hi1);
                    const float md0 = __bfloat162float(__float2bfloat16_rn(r0));
                    const float md1 = __bfloat162float(__float2bfloat16_rn(r1));
                    const int reg = r + 2 * qq;
                    A[0][reg] = pack_bf16(hi0, hi1);
                    A[1][reg] = pack_bf16(md0, md1);
                    A[2][reg] = pack_bf16(__fsub_rn(r0, md0), __fsub_rn(r1, md1));
                }
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                const int j = 8 * nt + g;  // B column = output unit
                const unsigned b0 = w2[(j * NH + i0) >> 1], b1 = w2[(j * NH + i0 + 8) >> 1];
                mma_bf16_16816(acc[nt], A[2], b0, b1);
                mma_bf16_16816(acc[nt], A[1], b0, b1);
                mma_bf16_16816(acc[nt], A[0], b0, b1);
            }
        }
        float o0 = 0.f, o1 = 0.f;
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int j = 8 * nt + 2 * tig;
            const float w3a = __bfloat162float(pw[OFF_W3 + j]), w3b = __bfloat162float(pw[OFF_W3 + j + 1]);
            o0 = fmaf(w3a, tanhf(acc[nt][0]), o0);
            o0 = fmaf(w3b, tanhf(acc[nt][1]), o0);
            o1 = fmaf(w3a, tanhf(acc[nt][2]), o1);
            o1 = fmaf(w3b, tanhf(acc[nt][3]), o1);
        }
        o0 += __shfl_xor_sync(0xffffffffu, o0, 1);
        o0 += __shfl_xor_sync(0xffffffffu, o0, 2);
        o1 += __shfl_xor_sync(0xffffffffu, o1, 1);
        o1 += __shfl_xor_sync(0xffffffffu, o1, 2);
        if (tig == 0) {
            const float b3 = __bfloat162float(pw[OFF_B3]);
            float out0 = __fadd_rn(o0, b3), out1 = __fadd_rn(o1, b3);
            if (residual) {  // the network predicts log-DCF + log density (radius 2)
                out0 = __fsub_rn(out0, x0[1]);
                out1 = __fsub_rn(out1, x1[1]);
            }
            if (s0 < n) y[s0] = exp_out ? __fmul_rn(scale, expf(out0)) : out0;
            if (s1 < n) y[s1] = exp_out ? __fmul_rn(scale, expf(out1)) : out1;
        }
    }
}

// Forward + per-sample reverse pass of the (optionally weighted) mean squared
// error (1/n) sum_s c_s (y_s - t_s)^2.  Writes H1, H2, D1, D2 (64 x n each,
// unit-major so that a warp's stores are coalesced), DY (n) and one partial
// sum of squared residuals per CTA.  First-layer units are recomputed where
// needed, so only one 64-wide register array is live.
__global__ void __launch_bounds__(kFwdThreads) mlp_train_kernel(const __nv_bfloat16 *__restrict__ pb,
                                                                const float *__restrict__ x,
                                                                const float *__restrict__ t,
                                                                const float *__restrict__ cw, long long n,
                                                                float *H1, float *H2, float *D1, float *D2, float *DY,
                                                                float *loss_part)
{
    __shared__ __align__(16) float ps[NP + 3];
    __shared__ float red[kFwdThreads / 32];
    load_params(pb, ps);
    const float inv_n = 1.f / (float)n;
    float lsum = 0.f;
    for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < n; s += (long long)gridDim.x * blockDim.x) {
        float xs[NI], a[NH];
#pragma unroll
        for (int k = 0; k < NI; ++k) xs[k] = x[s * NI + k];
        const float out = forward_sample(ps, xs, a);
        const float r = out - t[s];
        const float c = cw ? cw[s] : 1.f;
        lsum = fmaf(c * r, r, lsum);
        const float dy = 2.f * c * r * inv_n;
        DY[s] = dy;
#pragma unroll
        for (int j = 0; j < NH; ++j) {
            H2[(size_t)j * n + s] = a[j];
            a[j] = dy * ps[OFF_W3 + j] * (1.f - a[j] * a[j]);  // delta of layer 2
            D2[(size_t)j * n + s] = a[j];
        }
#pragma unroll 1
        for (int i = 0; i < NH; ++i) {
            const float h = unit1(ps, xs, i);
            H1[(size_t)i * n + s] = h;
            D1[(size_t)i * n + s] = dot_row(ps, i, a) * (1.f - h * h);
        }
    }
    for (int d = 16; d; d >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, d);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = lsum;
    __syncthreads();
    if (threadIdx.x == 0) {
        float v = 0.f;
        for (int w = 0; w < kFwdThreads / 32; ++w) v += red[w];
        loss_part[blockIdx.x] = v;
    }
}

// Partial gradient of samples [b*256, b*256+256): 256 threads, each owning
// 16 entries of gW2 and at most 3 of the other parameters.
__global__ void __launch_bounds__(256) mlp_grad_kernel(const float *__restrict__ x, long long n,
                                                       const float *__restrict__ H1, const float *__restrict__ H2,
                                                       const float *__restrict__ D1, const float *__restrict__ D2,
                                                       const float *__restrict__ DY, float *partials)
{
    constexpr int CH = 32;  // samples staged per step
    __shared__ __align__(16) float sh1[CH][NH], sh2[CH][NH], sd1[CH][NH], sd2[CH][NH];
    __shared__ float sx[CH][NI], sdy[CH];
    const int tid = threadIdx.x;
    const int j2 = tid >> 2, i2 = (tid & 3) * 16;  // gW2 rows j2, columns i2..i2+15
    float g2[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) g2[k] = 0.f;
    float g1[NI];  // gW1 row tid (tid < 64)
#pragma unroll
    for (int k = 0; k < NI; ++k) g1[k] = 0.f;
    float gb = 0.f;  // b1 (tid < 64), b2 (64..127), W3 (128..191), b3 (192)
    const long long s0 = (long long)blockIdx.x * kGradSamples;
    const long long s1 = min(s0 + kGradSamples, n);
    for (long long c = s0; c < s1; c += CH) {
        const int m = (int)(s1 - c < CH ? s1 - c : CH);
        __syncthreads();
        for (int e = tid; e < CH * NH; e += 256) {
            const int q = e / CH, r = e % CH;
            const bool ok = r < m;
            const size_t g = (size_t)q * n + (size_t)(c + r);
            sh1[r][q] = ok ? H1[g] : 0.f;
            sh2[r][q] = ok ? H2[g] : 0.f;
            sd1[r][q] = ok ? D1[g] : 0.f;
            sd2[r][q] = ok ? D2[g] : 0.f;
        }
        for (int e = tid; e < CH * NI; e += 256) {
            const int r = e / NI, q = e % NI;
            sx[r][q] = r < m ? x[(size_t)(c + r) * NI + q] : 0.f;
        }
        if (tid < CH) sdy[tid] = tid < m ? DY[c + tid] : 0.f;
        __syncthreads();
        for (int r = 0; r < CH; ++r) {
            const float d = sd2[r][j2];
            const float4 *h = reinterpret_cast<const float4 *>(&sh1[r][i2]);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float4 v = h[k];
                g2[4 * k] = fmaf(d, v.x, g2[4 * k]);
                g2[4 * k + 1] = fmaf(d, v.y, g2[4 * k + 1]);
                g2[4 * k + 2] = fmaf(d, v.z, g2[4 * k + 2]);
                g2[4 * k + 3] = fmaf(d, v.w, g2[4 * k + 3]);
            }
            if (tid < NH) {
                const float d1 = sd1[r][tid];
#pragma unroll
                for (int k = 0; k < NI; ++k) g1[k] = fmaf(d1, sx[r][k], g1[k]);
                gb += d1;
            } else if (tid < 2 * NH) {
                gb += sd2[r][tid - NH];
            } else if (tid < 3 * NH) {
                gb = fmaf(sdy[r], sh2[r][tid - 2 * NH], gb);
            } else if (tid == 3 * NH) {
                gb += sdy[r];
            }
        }
    }
    float *out = partials + (size_t)blockIdx.x * NP;
#pragma unroll
    for (int k = 0; k < 16; ++k) out[OFF_W2 + j2 * NH + i2 + k] = g2[k];
    if (tid < NH) {
#pragma unroll
        for (int k = 0; k < NI; ++k) out[OFF_W1 + tid * NI + k] = g1[k];
        out[OFF_B1 + tid] = gb;
    } else if (tid < 2 * NH) {
        out[OFF_B2 + tid - NH] = gb;
    } else if (tid < 3 * NH) {
        out[OFF_W3 + tid - 2 * NH] = gb;
    } else if (tid == 3 * NH) {
        out[OFF_B3] = gb;
    }
}

__global__ void mlp_reduce_kernel(const float *__restrict__ partials, int nblocks, const float *__restrict__ loss_part,
                                  int nloss, float inv_n, float *grad, float *loss)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < NP) {
        float a = 0.f;
        for (int b = 0; b < nblocks; ++b) a += partials[(size_t)b * NP + p];
        grad[p] = a;
    }
    if (p == 0 && loss) {
        float a = 0.f;
        for (int b = 0; b < nloss; ++b) a += loss_part[b];
        *loss = a * inv_n;
    }
}

__global__ void mlp_adam_kernel(float *master, __nv_bfloat16 *pb, const float *__restrict__ g, float *m, float *v,
                                int count, float lr, float b1, float b2, float eps, float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float w = master[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    master[i] = w;
    pb[i] = __float2bfloat16_rn(w);
}

__global__ void to_bf16_kernel(const float *__restrict__ a, __nv_bfloat16 *b, int count)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) b[i] = __float2bfloat16_rn(a[i]);
}

int sm_count_mlp()
{
    int dev = 0, n = 132;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n;
}

// FR_MLP_SIMT=1: the forward pass on the FP32 CUDA cores (A/B measurements).
bool mlp_use_simt()
{
    const char *e = std::getenv("FR_MLP_SIMT");
    return e && std::atoi(e) != 0;
}

int train_blocks(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + kFwdThreads - 1) / kFwdThreads, (long long)sm_count_mlp() * 8)); }

}  // namespace

size_t mlp_workspace_bytes(size_t n)
{
    const size_t gblocks = (n + kGradSamples - 1) / kGradSamples;
    const size_t a = (4 * (size_t)NH + 1) * n * 4;
    return a + std::max<size_t>(gblocks, 1) * NP * 4 + (size_t)train_blocks((long long)std::max<size_t>(n, 1)) * 4 + 256;
}

int mlp_forward_run(const void *d_params, const float *d_x, size_t n, int exp_out, int residual, float scale,
                    float *d_y, cudaStream_t s)
{
    if (n == 0) return FR_OK;
    const int blocks = (int)std::max<long long>(1, std::min<long long>(((long long)n + kFwdThreads - 1) / kFwdThreads,
                                                                       (long long)sm_count_mlp() * 16));
    if (mlp_use_simt()) {
        mlp_forward_kernel<<<blocks, kFwdThreads, 0, s>>>(static_cast<const __nv_bfloat16 *>(d_params), d_x,
                                                          (long long)n, exp_out, residual, scale, d_y);
        FR_CHECK_LAUNCH("mlp_forward_kernel");
        return FR_OK;
    }
    const long long tiles = ((long long)n + 15) / 16;
    const int mblocks = (int)std::max<long long>(
        1, std::min<long long>((tiles + kMmaThreads / 32 - 1) / (kMmaThreads / 32), (long long)sm_count_mlp() * 16));
    mlp_forward_mma_kernel<<<mblocks, kMmaThreads, 0, s>>>(static_cast<const __nv_bfloat16 *>(d_params), d_x,
                                                          (long long)n, exp_out, residual, scale, d_y);
    FR_CHECK_LAUNCH("mlp_forward_mma_kernel");
    return FR_OK;
}

int mlp_backward_run(const void *d_params, const float *d_x, const float *d_t, const float *d_w, size_t n, void *ws,
                     float *d_grad, float *d_loss, cudaStream_t s)
{
    if (n == 0) return fail(FR_ERR_INVALID_ARGUMENT, "empty batch");
    float *H1 = static_cast<float *>(ws);
    float *H2 = H1 + (size_t)NH * n;
    float *D1 = H2 + (size_t)NH * n;
    float *D2 = D1 + (size_t)NH * n;
    float *DY = D2 + (size_t)NH * n;
    float *partials = DY + n;
    const int gblocks = (int)((n + kGradSamples - 1) / kGradSamples);
    float *loss_part = partials + (size_t)gblocks * NP;
    const int tb = train_blocks((long long)n);
    mlp_train_kernel<<<tb, kFwdThreads, 0, s>>>(static_cast<const __nv_bfloat16 *>(d_params), d_x, d_t, d_w, (long long)n,
                                                H1, H2, D1, D2, DY, loss_part);
    FR_CHECK_LAUNCH("mlp_train_kernel");
    mlp_grad_kernel<<<gblocks, 256, 0, s>>>(d_x, (long long)n, H1, H2, D1, D2, DY, partials);
    FR_CHECK_LAUNCH("mlp_grad_kernel");
    mlp_reduce_kernel<<<(NP + 255) / 256, 256, 0, s>>>(partials, gblocks, loss_part, tb, 1.f / (float)n, d_grad,
                                                      d_loss);
    FR_CHECK_LAUNCH("mlp_reduce_kernel");
    return FR_OK;
}

int mlp_adam_run(float *d_master, void *d_params, const float *d_grad, float *d_m, float *d_v, int count, float lr,
                 float beta1, float beta2, float eps, int step, cudaStream_t s)
{
    if (count <= 0 || step < 1) return fail(FR_ERR_INVALID_ARGUMENT, "count > 0 and step >= 1");
    const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
    mlp_adam_kernel<<<(count + 255) / 256, 256, 0, s>>>(d_master, static_cast<__nv_bfloat16 *>(d_params), d_grad, d_m,
                                                        d_v, count, lr, beta1, beta2, eps, c1, c2);
    FR_CHECK_LAUNCH("mlp_adam_kernel");
    return FR_OK;
}

int to_bf16_run(const float *d_a, void *d_b, int count, cudaStream_t s)
{
    if (count <= 0) return FR_OK;
    to_bf16_kernel<<<(count + 255) / 256, 256, 0, s>>>(d_a, static_cast<__nv_bfloat16 *>(d_b), count);
    FR_CHECK_LAUNCH("to_bf16_kernel");
    return FR_OK;
}

}  // namespace fr
