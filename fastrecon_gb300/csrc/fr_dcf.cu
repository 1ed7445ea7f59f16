// fr_dcf.cu -- density compensation and degridding.  No counterpart in the
// reference, which reads its DCF from a file (ReconData.cpp:108-121) and has
// no interpolation from the grid back to the samples.
//
//  * fr_dcf_analytic: |k|^p of the raw coordinates (|k| for 2D radial, |k|^2
//    for 3D radial), computed in double like the CPU restatement.
//  * fr_degrid: interpolation of a multi-coil grid at the samples, the adjoint
//    of gridding (same clamped cell range and exact LUT index as the scatter,
//    GridLut.cpp:98-136).  One thread per sample and block of coils; the grid
//    is read through L1/L2 (consecutive samples of a readout share cells).
//  * Pipe-Menon DCF (Pipe & Menon, MRM 41:179-186, 1999):
//        w <- w / (C w),  C w = degrid(grid(w)),
//    with grid(w) a real-valued tile scatter over the plan's bins (shared-
//    memory accumulation, one flush per tile, no global atomics) and the
//    degridding fused with the division.
#include <cuda_runtime.h>

#include <algorithm>

#include "fr_device.cuh"
#include "fr_internal.h"

namespace fr {
namespace {

// Weight of a tap at squared distance s2 from the exact LUT-index table
// {thr[k+1], lut[k], lut[k+1], 0}: returns false outside the kernel radius.
__device__ __forceinline__ bool lut_weight(float s2, const float4 *lutS, float smax, float kc, int L, float &w)
{
    if (!(s2 < smax)) return false;
    float a;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(a) : "f"(s2));
    const int k0 = min((int)fmaf(a, kc, 0.25f), L - 1);
    const float4 en = lutS[k0];
    w = s2 >= en.x ? en.z : en.y;
    return true;
}

// -- analytic DCF -----------------------------------------------------------
__global__ void dcf_analytic_kernel(const float4 *__restrict__ traj, long long n, int dim, double power, int mode,
                                    float *__restrict__ out)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float4 p = traj[i];
        double q = __dmul_rn((double)p.x, (double)p.x);
        if (dim >= 2) q = __dadd_rn(q, __dmul_rn((double)p.y, (double)p.y));
        if (dim >= 3) q = __dadd_rn(q, __dmul_rn((double)p.z, (double)p.z));
        const double k = __dsqrt_rn(q);
        const double w = mode == 1 ? k : (mode == 2 ? __dmul_rn(k, k) : pow(k, power));
        out[i] = __double2float_rn(w);
    }
}

// -- degridding ---------------------------------------------------------------
struct DegridParams {
    const float4 *traj;  // normalised
    long long n;
    int dim, G;
    float hw;
    int L;
    float smax, kc;
    const float4 *lut_e;
    const float2 *grid;  // channels x cells
    int channels;
    long long cells;
    int checkerboard;
    float2 *out;         // channels x n
};

template <int CB>
__global__ void __launch_bounds__(256) degrid_kernel(DegridParams P)
{
    extern __shared__ float4 lutS[];
    for (int i = threadIdx.x; i < P.L; i += blockDim.x) lutS[i] = P.lut_e[i];
    __syncthreads();
    const int c0 = blockIdx.y * CB;
    const size_t G = (size_t)P.G;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < P.n;
         i += (long long)gridDim.x * blockDim.x) {
        const float4 p = P.traj[i];
        int xs, xe, ys, ye, zs = 0, ze = 0;
        comp_range(p.x, P.hw, P.G, xs, xe);
        comp_range(p.y, P.hw, P.G, ys, ye);
        if (P.dim == 3) comp_range(p.z, P.hw, P.G, zs, ze);
        float2 acc[CB];
#pragma unroll
        for (int c = 0; c < CB; ++c) acc[c] = make_float2(0.f, 0.f);
        for (int z = zs; z <= ze; ++z) {
            const float dz = P.dim == 3 ? __fsub_rn((float)z, p.z) : 0.f;
            const float dz2 = __fmul_rn(dz, dz);
            for (int y = ys; y <= ye; ++y) {
                const float dy = __fsub_rn((float)y, p.y);
                const float dzy = __fadd_rn(dz2, __fmul_rn(dy, dy));
                const size_t row = ((size_t)z * G + (size_t)y) * G;
                for (int x = xs; x <= xe; ++x) {
                    const float dx = __fsub_rn((float)x, p.x);
                    float w;
                    if (!lut_weight(__fadd_rn(dzy, __fmul_rn(dx, dx)), lutS, P.smax, P.kc, P.L, w)) continue;
                    if (P.checkerboard && ((x + y + z) & 1)) w = -w;
#pragma unroll
                    for (int c = 0; c < CB; ++c) {
                        if (c0 + c < P.channels) {
                            const float2 g = P.grid[(size_t)(c0 + c) * P.cells + row + x];
                            acc[c].x = fmaf(w, g.x, acc[c].x);
                            acc[c].y = fmaf(w, g.y, acc[c].y);
                        }
                    }
                }
            }
        }
#pragma unroll
        for (int c = 0; c < CB; ++c)
            if (c0 + c < P.channels) P.out[(size_t)(c0 + c) * P.n + i] = acc[c];
    }
}

// -- streaming acquisition: incremental regridding -----------------------------
// The gridded change dcf * (new - old) of the samples [begin, begin + count)
// added into the grid with global atomic adds: thread per (sample, block of
// CB coils), the same cell range, LUT index and checkerboard signs as the
// scatter and the degridding.
struct UpdateParams {
    DegridParams g;          // geometry, LUT, grid size, checkerboard flag
    const float2 *old_k;     // channels x n: the k-space the grid was made from
    const float2 *new_k;     // channels x count: the new values
    const float *dcf;        // n
    float2 *grid;            // channels x cells
    long long begin, count;
};

template <int CB>
__global__ void __launch_bounds__(256) grid_update_kernel(UpdateParams U)
{
    extern __shared__ float4 lutS[];
    const DegridParams &P = U.g;
    for (int i = threadIdx.x; i < P.L; i += blockDim.x) lutS[i] = P.lut_e[i];
    __syncthreads();
    const int c0 = blockIdx.y * CB;
    const size_t G = (size_t)P.G;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < U.count;
         i += (long long)gridDim.x * blockDim.x) {
        const long long sidx = U.begin + i;
        const float4 p = P.traj[sidx];
        const float d = U.dcf[sidx];
        float2 v[CB];
#pragma unroll
        for (int c = 0; c < CB; ++c) {
            v[c] = make_float2(0.f, 0.f);
            if (c0 + c < P.channels) {
                const float2 a = U.new_k[(size_t)(c0 + c) * U.count + i];
                const float2 b = U.old_k[(size_t)(c0 + c) * P.n + sidx];
                v[c] = make_float2(__fmul_rn(d, __fsub_rn(a.x, b.x)), __fmul_rn(d, __fsub_rn(a.y, b.y)));
            }
        }
        int xs, xe, ys, ye, zs = 0, ze = 0;
        comp_range(p.x, P.hw, P.G, xs, xe);
        comp_range(p.y, P.hw, P.G, ys, ye);
        if (P.dim == 3) comp_range(p.z, P.hw, P.G, zs, ze);
        for (int z = zs; z <= ze; ++z) {
            const float dz = P.dim == 3 ? __fsub_rn((float)z, p.z) : 0.f;
            const float dz2 = __fmul_rn(dz, dz);
            for (int y = ys; y <= ye; ++y) {
                const float dy = __fsub_rn((float)y, p.y);
                const float dzy = __fadd_rn(dz2, __fmul_rn(dy, dy));
                const size_t row = ((size_t)z * G + (size_t)y) * G;
                for (int x = xs; x <= xe; ++x) {
                    const float dx = __fsub_rn((float)x, p.x);
                    float w;
                    if (!lut_weight(__fadd_rn(dzy, __fmul_rn(dx, dx)), lutS, P.smax, P.kc, P.L, w)) continue;
                    if (P.checkerboard && ((x + y + z) & 1)) w = -w;
#pragma unroll
                    for (int c = 0; c < CB; ++c) {
                        if (c0 + c < P.channels) {
                            float *g = reinterpret_cast<float *>(U.grid + (size_t)(c0 + c) * P.cells + row + x);
                            atomicAdd(g, __fmul_rn(w, v[c].x));
                            atomicAdd(g + 1, __fmul_rn(w, v[c].y));
                        }
                    }
                }
            }
        }
    }
}

// -- real-valued tile scatter of per-sample weights ---------------------------
struct RealGridParams {
    const float4 *traj;
    const unsigned long long *recs;
    const WorkItem *items;
    const SplitTile *splits;
    const float *w;
    const float4 *lut_e;
    float *grid;      // G^d floats
    float *partials;  // nslots x K floats
    int dim, G, L;
    int tile[3], ntile[3], K;
    float smax, kc;
};

constexpr int kRealWarps = 8;

__global__ void __launch_bounds__(kRealWarps * 32) grid_real_kernel(RealGridParams P)
{
    extern __shared__ float4 smr[];
    float4 *lutS = smr;
    float *acc = reinterpret_cast<float *>(smr + P.L);
    const WorkItem it = P.items[blockIdx.x];
    const int t = it.tile;
    const int ox = (t % P.ntile[0]) * P.tile[0];
    const int oy = ((t / P.ntile[0]) % P.ntile[1]) * P.tile[1];
    const int oz = (t / (P.ntile[0] * P.ntile[1])) * P.tile[2];
    const int Tx = P.tile[0], Ty = P.tile[1], Tz = P.tile[2];
    for (int i = threadIdx.x; i < P.L; i += blockDim.x) lutS[i] = P.lut_e[i];
    for (int i = threadIdx.x; i < P.K; i += blockDim.x) acc[i] = 0.f;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned long long *recs = P.recs + it.begin;
    for (int j = warp; j < it.count; j += kRealWarps) {
        const unsigned long long rec = recs[j];
        const unsigned s = (unsigned)rec;
        const unsigned box = (unsigned)(rec >> 32);
        const int lx0 = box & 63, ly0 = (box >> 6) & 63, lz0 = (box >> 12) & 63;
        const int nx = (box >> 18) & 15, ny = (box >> 22) & 15, nz = (box >> 26) & 15;
        const int ntap = nx * ny * nz;
        if (ntap == 0) continue;
        const float4 p = P.traj[s];
        const float v = P.w[s];
        for (int tt = lane; tt < ntap; tt += 32) {
            const int ix = tt % nx, r = tt / nx, iy = r % ny, iz = r / ny;
            const int lx = lx0 + ix, ly = ly0 + iy, lz = lz0 + iz;
            const float dx = __fsub_rn((float)(ox + lx), p.x);
            const float dy = __fsub_rn((float)(oy + ly), p.y);
            const float dz = P.dim == 3 ? __fsub_rn((float)(oz + lz), p.z) : 0.f;
            const float s2 = __fadd_rn(__fadd_rn(__fmul_rn(dz, dz), __fmul_rn(dy, dy)), __fmul_rn(dx, dx));
            float w;
            if (lut_weight(s2, lutS, P.smax, P.kc, P.L, w)) atomicAdd(&acc[(lz * Ty + ly) * Tx + lx], w * v);
        }
    }
    __syncthreads();
    if (it.slot >= 0) {
        float *dst = P.partials + (size_t)it.slot * P.K;
        for (int i = threadIdx.x; i < P.K; i += blockDim.x) dst[i] = acc[i];
        return;
    }
    const size_t G = (size_t)P.G;
    const int Gz = P.dim == 3 ? P.G : 1;
    for (int i = threadIdx.x; i < P.K; i += blockDim.x) {
        const int lx = i % Tx, r = i / Tx, ly = r % Ty, lz = r / Ty;
        const int gx = ox + lx, gy = oy + ly, gz = oz + lz;
        if (gx < P.G && gy < P.G && gz < Gz && lz < Tz) P.grid[((size_t)gz * G + gy) * G + gx] = acc[i];
    }
}

__global__ void reduce_real_splits_kernel(RealGridParams P)
{
    const SplitTile st = P.splits[blockIdx.x];
    const int t = st.tile;
    const int ox = (t % P.ntile[0]) * P.tile[0];
    const int oy = ((t / P.ntile[0]) % P.ntile[1]) * P.tile[1];
    const int oz = (t / (P.ntile[0] * P.ntile[1])) * P.tile[2];
    const size_t G = (size_t)P.G;
    const int Gz = P.dim == 3 ? P.G : 1;
    const float *base = P.partials + (size_t)st.first_slot * P.K;
    for (int i = threadIdx.x; i < P.K; i += blockDim.x) {
        const int lx = i % P.tile[0], r = i / P.tile[0], ly = r % P.tile[1], lz = r / P.tile[1];
        const int gx = ox + lx, gy = oy + ly, gz = oz + lz;
        if (gx >= P.G || gy >= P.G || gz >= Gz) continue;
        float v = 0.f;
        for (int k = 0; k < st.nslots; ++k) v = __fadd_rn(v, base[(size_t)k * P.K + i]);
        P.grid[((size_t)gz * G + gy) * G + gx] = v;
    }
}

// Degrid a real grid at each sample and divide the sample's weight by it.
__global__ void __launch_bounds__(256) pipe_update_kernel(DegridParams P, const float *__restrict__ g, float *w)
{
    extern __shared__ float4 lutS[];
    for (int i = threadIdx.x; i < P.L; i += blockDim.x) lutS[i] = P.lut_e[i];
    __syncthreads();
    const size_t G = (size_t)P.G;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < P.n;
         i += (long long)gridDim.x * blockDim.x) {
        const float4 p = P.traj[i];
        int xs, xe, ys, ye, zs = 0, ze = 0;
        comp_range(p.x, P.hw, P.G, xs, xe);
        comp_range(p.y, P.hw, P.G, ys, ye);
        if (P.dim == 3) comp_range(p.z, P.hw, P.G, zs, ze);
        float acc = 0.f;
        for (int z = zs; z <= ze; ++z) {
            const float dz = P.dim == 3 ? __fsub_rn((float)z, p.z) : 0.f;
            const float dz2 = __fmul_rn(dz, dz);
            for (int y = ys; y <= ye; ++y) {
                const float dy = __fsub_rn((float)y, p.y);
                const float dzy = __fadd_rn(dz2, __fmul_rn(dy, dy));
                const float *grow = g + ((size_t)z * G + (size_t)y) * G;
                for (int x = xs; x <= xe; ++x) {
                    const float dx = __fsub_rn((float)x, p.x);
                    float wt;
                    if (lut_weight(__fadd_rn(dzy, __fmul_rn(dx, dx)), lutS, P.smax, P.kc, P.L, wt))
                        acc = fmaf(wt, grow[x], acc);
                }
            }
        }
        if (acc > 0.f) w[i] = w[i] / acc;
    }
}

int sm_count()
{
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 132;
    }
    return n;
}

DegridParams degrid_params(fr_plan p)
{
    DegridParams P;
    P.traj = p->traj.as<float4>();
    P.n = (long long)p->n;
    P.dim = p->dim;
    P.G = (int)p->G;
    P.hw = p->hw;
    P.L = p->L;
    P.smax = p->lut_smax;
    P.kc = p->lut_kc;
    P.lut_e = p->lut_e.as<float4>();
    P.cells = p->dim == 3 ? (long long)p->G * p->G * p->G : (long long)p->G * p->G;
    P.checkerboard = (p->flags & FR_PLAN_CHECKERBOARD) ? 1 : 0;
    P.grid = nullptr;
    P.channels = 0;
    P.out = nullptr;
    return P;
}

}  // namespace

int dcf_analytic_run(const float *d_traj, size_t n, int dim, float power, float *d_out, cudaStream_t s)
{
    if (n == 0) return FR_OK;
    const int mode = power == 1.f ? 1 : (power == 2.f ? 2 : 0);
    const int blocks = (int)std::min<long long>(((long long)n + 255) / 256, (long long)sm_count() * 8);
    dcf_analytic_kernel<<<blocks, 256, 0, s>>>(reinterpret_cast<const float4 *>(d_traj), (long long)n, dim,
                                               (double)power, mode, d_out);
    FR_CHECK_LAUNCH("dcf_analytic_kernel");
    return FR_OK;
}

int degrid_run(fr_plan p, const float *d_grid, int channels, float *d_out, cudaStream_t s)
{
    if (!p->planned) return fail(FR_ERR_NOT_PLANNED, "fr_degrid called before fr_plan_set_trajectory");
    if (channels <= 0) return fail(FR_ERR_INVALID_ARGUMENT, "channels must be positive");
    if (p->n == 0) return FR_OK;
    DegridParams P = degrid_params(p);
    P.grid = reinterpret_cast<const float2 *>(d_grid);
    P.channels = channels;
    P.out = reinterpret_cast<float2 *>(d_out);
    constexpr int CB = 4;
    const size_t smem = (size_t)P.L * 16;
    if (smem > 48 * 1024)
        FR_CUDA(cudaFuncSetAttribute(degrid_kernel<CB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int bx = (int)std::min<long long>((P.n + 255) / 256, (long long)sm_count() * 8);
    dim3 grid(bx, (channels + CB - 1) / CB);
    degrid_kernel<CB><<<grid, 256, smem, s>>>(P);
    FR_CHECK_LAUNCH("degrid_kernel");
    return FR_OK;
}

int grid_update_run(fr_plan p, float *d_kdata, const float *d_new, size_t begin, size_t count, const float *d_dcf,
                    int channels, float *d_grid, cudaStream_t s)
{
    if (!p->planned) return fail(FR_ERR_NOT_PLANNED, "fr_grid_update called before fr_plan_set_trajectory");
    if (channels <= 0) return fail(FR_ERR_INVALID_ARGUMENT, "channels must be positive");
    if (begin > p->n || count > p->n - begin) return fail(FR_ERR_SIZE_MISMATCH, "sample range exceeds the plan's samples");
    if (count == 0) return FR_OK;
    UpdateParams U;
    U.g = degrid_params(p);
    U.g.channels = channels;
    U.old_k = reinterpret_cast<const float2 *>(d_kdata);
    U.new_k = reinterpret_cast<const float2 *>(d_new);
    U.dcf = d_dcf;
    U.grid = reinterpret_cast<float2 *>(d_grid);
    U.begin = (long long)begin;
    U.count = (long long)count;
    constexpr int CB = 4;
    const size_t smem = (size_t)U.g.L * 16;
    if (smem > 48 * 1024)
        FR_CUDA(cudaFuncSetAttribute(grid_update_kernel<CB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int bx = (int)std::min<long long>(((long long)count + 255) / 256, (long long)sm_count() * 8);
    dim3 grid(bx, (channels + CB - 1) / CB);
    grid_update_kernel<CB><<<grid, 256, smem, s>>>(U);
    FR_CHECK_LAUNCH("grid_update_kernel");
    // then the k-space itself: row c of the new values into coil c at `begin`
    FR_CUDA(cudaMemcpy2DAsync(d_kdata + 2 * begin, p->n * 8, d_new, count * 8, count * 8, (size_t)channels,
                              cudaMemcpyDeviceToDevice, s));
    return FR_OK;
}

int grid_real_run(fr_plan p, const float *d_w, float *d_grid, cudaStream_t s)
{
    if (!p->planned) return fail(FR_ERR_NOT_PLANNED, "plan has no trajectory");
    RealGridParams P;
    P.traj = p->traj.as<float4>();
    P.recs = p->pairs.as<unsigned long long>();
    P.items = p->items.as<WorkItem>();
    P.splits = p->splits.as<SplitTile>();
    P.w = d_w;
    P.lut_e = p->lut_e.as<float4>();
    P.grid = d_grid;
    P.dim = p->dim;
    P.G = (int)p->G;
    P.L = p->L;
    P.K = 1;
    for (int d = 0; d < 3; ++d) {
        P.tile[d] = p->tile[d];
        P.ntile[d] = p->ntile[d];
        P.K *= p->tile[d];
    }
    P.smax = p->lut_smax;
    P.kc = p->lut_kc;
    if (p->nslots > 0 && p->real_partials.reserve((size_t)p->nslots * P.K * 4)) return FR_ERR_CUDA;
    P.partials = p->real_partials.as<float>();
    if (p->nitems == 0) return FR_OK;
    const size_t smem = (size_t)P.L * 16 + (size_t)P.K * 4;
    if (smem > 227 * 1024) return fail(FR_ERR_UNSUPPORTED, "tile too large for the real-valued scatter");
    if (smem > 48 * 1024)
        FR_CUDA(cudaFuncSetAttribute(grid_real_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    grid_real_kernel<<<(unsigned)p->nitems, kRealWarps * 32, smem, s>>>(P);
    FR_CHECK_LAUNCH("grid_real_kernel");
    if (p->nsplits > 0) {
        reduce_real_splits_kernel<<<(unsigned)p->nsplits, 256, 0, s>>>(P);
        FR_CHECK_LAUNCH("reduce_real_splits_kernel");
    }
    return FR_OK;
}

int dcf_pipe_run(fr_plan p, int iterations, float *d_w, cudaStream_t s)
{
    if (!p->planned) return fail(FR_ERR_NOT_PLANNED, "fr_dcf_pipe called before fr_plan_set_trajectory");
    if (iterations < 0) return fail(FR_ERR_INVALID_ARGUMENT, "iterations must be >= 0");
    if (p->n == 0 || iterations == 0) return FR_OK;
    const size_t cells = p->dim == 3 ? (size_t)p->G * p->G * p->G : (size_t)p->G * p->G;
    if (p->real_grid.reserve(cells * 4)) return FR_ERR_CUDA;
    DegridParams P = degrid_params(p);
    const size_t smem = (size_t)P.L * 16;
    if (smem > 48 * 1024)
        FR_CUDA(cudaFuncSetAttribute(pipe_update_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int bx = (int)std::min<long long>((P.n + 255) / 256, (long long)sm_count() * 8);
    for (int it = 0; it < iterations; ++it) {
        int st = grid_real_run(p, d_w, p->real_grid.as<float>(), s);
        if (st) return st;
        pipe_update_kernel<<<bx, 256, smem, s>>>(P, p->real_grid.as<float>(), d_w);
        FR_CHECK_LAUNCH("pipe_update_kernel");
    }
    return FR_OK;
}

}  // namespace fr
