// fr_density.cu -- sample-density features for the learned DCF.  No
// counterpart in the reference.
//
// Every sample is binned to its nearest grid cell (floor(x + 0.5) of the
// plan's normalised coordinate, clamped to the grid), the per-cell counts are
// turned into a summed-area table (inclusive prefix sums along x, y, z), and
// the number of samples in the (2r+1)^d box around each sample's cell is read
// from the table with 2^d corner lookups.  Counts are exact integers.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "fr_device.cuh"
#include "fr_internal.h"

namespace fr {
namespace {

constexpr int kMaxRadii = 8;

struct Radii {
    int r[kMaxRadii];
    int n;
};

__device__ __forceinline__ int nearest_cell(float x, int G)
{
    const int c = f2i_ref(floorf(__fadd_rn(x, 0.5f)));
    return min(max(c, 0), G - 1);
}

__global__ void cell_hist_kernel(const float4 *__restrict__ traj, long long n, int dim, int G, int *hist)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float4 p = traj[i];
        const int x = nearest_cell(p.x, G), y = nearest_cell(p.y, G), z = dim == 3 ? nearest_cell(p.z, G) : 0;
        atomicAdd(&hist[((size_t)z * G + y) * G + x], 1);
    }
}

// Inclusive scan along x: one warp per row.
__global__ void scan_x_kernel(int *a, long long rows, int G)
{
    const int lane = threadIdx.x & 31;
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long r = warp; r < rows; r += nwarps) {
        int *row = a + r * G;
        int carry = 0;
        for (int b = 0; b < G; b += 32) {
            int v = b + lane < G ? row[b + lane] : 0;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int u = __shfl_up_sync(0xffffffffu, v, d);
                if (lane >= d) v += u;
            }
            v += carry;
            if (b + lane < G) row[b + lane] = v;
            carry = __shfl_sync(0xffffffffu, v, 31);
        }
    }
}

// Inclusive scan along an outer axis: thread per column, sequential along
// the axis (stride `step` elements), consecutive threads on consecutive x.
__global__ void scan_outer_kernel(int *a, long long columns, int len, long long step, long long plane)
{
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < columns;
         c += (long long)gridDim.x * blockDim.x) {
        // column c: x = c % step within a plane block, block = c / step
        int *p = a + (c / step) * plane + (c % step);
        int acc = 0;
        for (int k = 0; k < len; ++k) {
            acc += p[(size_t)k * step];
            p[(size_t)k * step] = acc;
        }
    }
}

__device__ __forceinline__ long long sat_at(const int *sat, int G, int x, int y, int z)
{
    if (x < 0 || y < 0 || z < 0) return 0;
    return sat[((size_t)z * G + y) * G + x];
}

__global__ void box_count_kernel(const float4 *__restrict__ traj, long long n, int dim, int G, const int *sat,
                                 Radii R, int *counts)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float4 p = traj[i];
        const int cx = nearest_cell(p.x, G), cy = nearest_cell(p.y, G), cz = dim == 3 ? nearest_cell(p.z, G) : 0;
        for (int k = 0; k < R.n; ++k) {
            const int r = R.r[k];
            const int x0 = max(cx - r, 0) - 1, x1 = min(cx + r, G - 1);
            const int y0 = max(cy - r, 0) - 1, y1 = min(cy + r, G - 1);
            long long s;
            if (dim == 3) {
                const int z0 = max(cz - r, 0) - 1, z1 = min(cz + r, G - 1);
                s = sat_at(sat, G, x1, y1, z1) - sat_at(sat, G, x0, y1, z1) - sat_at(sat, G, x1, y0, z1) -
                    sat_at(sat, G, x1, y1, z0) + sat_at(sat, G, x0, y0, z1) + sat_at(sat, G, x0, y1, z0) +
                    sat_at(sat, G, x1, y0, z0) - sat_at(sat, G, x0, y0, z0);
            } else {
                s = sat_at(sat, G, x1, y1, 0) - sat_at(sat, G, x0, y1, 0) - sat_at(sat, G, x1, y0, 0) +
                    sat_at(sat, G, x0, y0, 0);
            }
            counts[i * R.n + k] = (int)s;
        }
    }
}

// max |k| of the raw coordinates (non-negative floats order like their bits)
__global__ void kmax_kernel(const float4 *__restrict__ traj, long long n, int dim, unsigned *out)
{
    float m = 0.f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float4 p = traj[i];
        float q = __fmul_rn(p.x, p.x);
        if (dim >= 2) q = __fadd_rn(q, __fmul_rn(p.y, p.y));
        if (dim >= 3) q = __fadd_rn(q, __fmul_rn(p.z, p.z));
        m = fmaxf(m, __fsqrt_rn(q));
    }
    for (int d = 16; d; d >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, d));
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

__global__ void features_kernel(const int *__restrict__ counts, const float4 *__restrict__ traj, long long n, int dim,
                                Radii R, const unsigned *kmax_bits, float kmax_given, float *feat)
{
    const float kmax = kmax_bits ? __uint_as_float(*kmax_bits) : kmax_given;
    const int nf = R.n + 1;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        for (int k = 0; k < R.n; ++k) {
            const float side = (float)(2 * R.r[k] + 1);
            const float vol = dim == 3 ? __fmul_rn(__fmul_rn(side, side), side) : __fmul_rn(side, side);
            feat[i * nf + k] = logf(__fdiv_rn((float)counts[i * R.n + k], vol));
        }
        const float4 p = traj[i];
        float q = __fmul_rn(p.x, p.x);
        if (dim >= 2) q = __fadd_rn(q, __fmul_rn(p.y, p.y));
        if (dim >= 3) q = __fadd_rn(q, __fmul_rn(p.z, p.z));
        feat[i * nf + R.n] = logf(__fadd_rn(__fdiv_rn(__fsqrt_rn(q), kmax), 0.0009765625f));
    }
}

int blocks_for(long long n, int threads)
{
    int dev = 0, sms = 132;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return (int)std::max<long long>(1, std::min<long long>((n + threads - 1) / threads, (long long)sms * 16));
}

int make_radii(const int *radii, int nradii, Radii *R)
{
    if (nradii < 1 || nradii > kMaxRadii || !radii) return fail(FR_ERR_INVALID_ARGUMENT, "1 to 8 radii");
    R->n = nradii;
    for (int k = 0; k < nradii; ++k) {
        if (radii[k] < 0 || radii[k] > 4096) return fail(FR_ERR_INVALID_ARGUMENT, "radius out of range");
        R->r[k] = radii[k];
    }
    return FR_OK;
}

}  // namespace

int density_counts_run(fr_plan p, const int *radii, int nradii, int *d_counts, cudaStream_t s)
{
    if (!p->planned) return fail(FR_ERR_NOT_PLANNED, "fr_density_counts called before fr_plan_set_trajectory");
    Radii R;
    int st = make_radii(radii, nradii, &R);
    if (st) return st;
    if (p->n == 0) return FR_OK;
    const int G = (int)p->G;
    const size_t cells = p->dim == 3 ? (size_t)G * G * G : (size_t)G * G;
    if (cells > 0x7FFFFFFFull) return fail(FR_ERR_UNSUPPORTED, "grid too large for the density table");
    if (p->density_sat.reserve(cells * 4)) return FR_ERR_CUDA;
    int *sat = p->density_sat.as<int>();
    FR_CUDA(cudaMemsetAsync(sat, 0, cells * 4, s));
    const long long n = (long long)p->n;
    const float4 *traj = p->traj.as<float4>();
    cell_hist_kernel<<<blocks_for(n, 256), 256, 0, s>>>(traj, n, p->dim, G, sat);
    FR_CHECK_LAUNCH("cell_hist_kernel");
    const long long rows = (long long)(cells / G);
    scan_x_kernel<<<blocks_for(rows * 32, 256), 256, 0, s>>>(sat, rows, G);
    FR_CHECK_LAUNCH("scan_x_kernel");
    // y: columns (z, x), stride G, planes of G*G
    const long long gz = p->dim == 3 ? G : 1;
    scan_outer_kernel<<<blocks_for(gz * G, 256), 256, 0, s>>>(sat, gz * G, G, G, (long long)G * G);
    FR_CHECK_LAUNCH("scan_outer_kernel");
    if (p->dim == 3) {  // z: columns (y, x), stride G*G
        scan_outer_kernel<<<blocks_for((long long)G * G, 256), 256, 0, s>>>(sat, (long long)G * G, G,
                                                                            (long long)G * G, 0);
        FR_CHECK_LAUNCH("scan_outer_kernel");
    }
    box_count_kernel<<<blocks_for(n, 256), 256, 0, s>>>(traj, n, p->dim, G, sat, R, d_counts);
    FR_CHECK_LAUNCH("box_count_kernel");
    return FR_OK;
}

int dcf_features_run(const int *d_counts, const float *d_raw, size_t n, int dim, const int *radii, int nradii,
                     float kmax, float *d_feat, unsigned *d_scratch, cudaStream_t s)
{
    Radii R;
    int st = make_radii(radii, nradii, &R);
    if (st) return st;
    if (n == 0) return FR_OK;
    const float4 *traj = reinterpret_cast<const float4 *>(d_raw);
    const unsigned *kb = nullptr;
    if (!(kmax > 0.f)) {
        FR_CUDA(cudaMemsetAsync(d_scratch, 0, 4, s));
        kmax_kernel<<<blocks_for((long long)n, 256), 256, 0, s>>>(traj, (long long)n, dim, d_scratch);
        FR_CHECK_LAUNCH("kmax_kernel");
        kb = d_scratch;
    }
    features_kernel<<<blocks_for((long long)n, 256), 256, 0, s>>>(d_counts, traj, (long long)n, dim, R, kb, kmax,
                                                                  d_feat);
    FR_CHECK_LAUNCH("features_kernel");
    return FR_OK;
}

}  // namespace fr
