// fr_grid.cu -- tiled Kaiser-Bessel scatter (gridding).
//
// Replaces cuGridLut::griddingChannel / gridding_kernel (cuGridLut.cu:231-309)
// and the CPU loop GridLut::griddingChannel (GridLut.cpp:80-147).
//
// One CTA per (work item, coil group).  A work item is one grid tile plus a
// chunk of the samples binned to it.  The CTA accumulates the tile for a
// group of coils in shared memory, laid out [cell][coil float] with an XOR
// swizzle, and flushes it to HBM once, coalesced along x, each grid cell
// written exactly once (zeros for empty tiles).  Tiles whose bin was split
// into several items write their partial tiles to a scratch area and a
// second kernel sums the partials in item order.  No global atomics.
//
// Per sample, lanes evaluate the kernel taps (geometry bit-exact with
// GridLut.cpp:98-136), the valid taps are compacted with a ballot and
// broadcast with shuffles, and lanes mapped to (tap slot, coil float) add
// weight * dcf * sample into the shared tile.  The weight is computed once
// per sample and reused for every coil of the group.
#include <cuda_runtime.h>

#include <algorithm>

#include "fr_device.cuh"
#include "fr_internal.h"

namespace fr {
namespace {

struct GridParams {
    const float4 *traj;
    const unsigned *pairs;
    const WorkItem *items;
    const SplitTile *splits;
    const float *kdata;  // channels x n complex64, as floats
    const float *dcf;
    const float *lut;    // global copy, staged into shared memory
    float *grid;         // channels x G^d complex64, as floats
    float *partials;     // nslots x ngroups x K x R floats
    long long n;
    int channels, coil_group, ngroups;
    int dim, G;
    int tile[3], ntile[3], K;
    int L;
    float hw, inv_hw, lm1;
    int hw_pow2, prefilter, checkerboard;
};

// Column swizzle of cell i in a row of R floats: keeps (re, im) pairs
// adjacent and spreads the flush (lanes along cells) over all banks.
template <int R>
__device__ __forceinline__ int swz(int i)
{
    if constexpr (R >= 32) {
        return (i & 15) << 1;
    } else {
        constexpr int per = 32 / R;  // cells per 32-bank row
        return ((i / per) & (R / 2 - 1)) << 1;
    }
}

template <int R>
__device__ __forceinline__ void write_cell_group(const GridParams &P, const float *acc, int cg, int ox,
                                                 int oy, int oz, bool zero)
{
    const int CG = P.coil_group;
    const int K = P.K;
    const int Tx = P.tile[0], Ty = P.tile[1];
    const size_t G = (size_t)P.G;
    const size_t cells = P.dim == 3 ? G * G * G : G * G;
    float2 *grid = reinterpret_cast<float2 *>(P.grid);
    const int total = CG * K;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        int cl = idx / K;
        int i = idx - cl * K;
        int c = cg * CG + cl;
        if (c >= P.channels) break;
        int lx = i % Tx;
        int r = i / Tx;
        int ly = r % Ty;
        int lz = r / Ty;
        int gx = ox + lx, gy = oy + ly, gz = oz + lz;
        if (gx >= P.G || gy >= P.G || gz >= (P.dim == 3 ? P.G : 1)) continue;
        float2 v = make_float2(0.f, 0.f);
        if (!zero) {
            int col = (2 * cl) ^ swz<R>(i);
            v = *reinterpret_cast<const float2 *>(acc + (size_t)i * R + col);
            if (P.checkerboard && ((gx + gy + gz) & 1)) {
                v.x = -v.x;
                v.y = -v.y;
            }
        }
        grid[(size_t)c * cells + ((size_t)gz * G + (size_t)gy) * G + (size_t)gx] = v;
    }
}

template <int DIM, int R>
__global__ void __launch_bounds__(512) grid_tiles_kernel(GridParams P)
{
    extern __shared__ float4 smem4[];
    float *acc = reinterpret_cast<float *>(smem4);
    const int K = P.K;
    float *lut = acc + (size_t)K * R;

    const WorkItem it = P.items[blockIdx.x];
    const int cg = blockIdx.y;
    const int t = it.tile;
    const int tx = t % P.ntile[0];
    const int ty = (t / P.ntile[0]) % P.ntile[1];
    const int tz = t / (P.ntile[0] * P.ntile[1]);
    const int ox = tx * P.tile[0], oy = ty * P.tile[1], oz = tz * P.tile[2];

    if (it.count == 0) {  // empty tile: stream zeros
        write_cell_group<R>(P, acc, cg, ox, oy, oz, true);
        return;
    }

    for (int i = threadIdx.x; i < K * R / 4; i += blockDim.x) smem4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int i = threadIdx.x; i < P.L; i += blockDim.x) lut[i] = P.lut[i];
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    constexpr int NG = R >= 32 ? 1 : 32 / R;  // taps per accumulate step
    constexpr int NF = R > 32 ? R / 32 : 1;   // floats per lane per tap
    const int q = R >= 32 ? 0 : lane / R;     // tap slot of this lane
    const int f0 = R >= 32 ? lane : lane % R; // first coil float of this lane
    const int CG = P.coil_group;
    const int hx = ox + P.tile[0] - 1, hy = oy + P.tile[1] - 1, hz = oz + P.tile[2] - 1;

    int coil[NF];
    bool coil_ok[NF];
#pragma unroll
    for (int k = 0; k < NF; ++k) {
        int f = f0 + 32 * k;
        coil[k] = cg * CG + (f >> 1);
        coil_ok[k] = (f >> 1) < CG && coil[k] < P.channels;
    }
    const float2 *kd = reinterpret_cast<const float2 *>(P.kdata);

    for (int j = warp; j < it.count; j += nwarps) {
        const unsigned s = P.pairs[it.begin + j];
        const float4 p = P.traj[s];
        const float d = P.dcf[s];
        float val[NF];
#pragma unroll
        for (int k = 0; k < NF; ++k) {
            val[k] = 0.f;
            if (coil_ok[k]) {
                float2 z = kd[(size_t)coil[k] * (size_t)P.n + s];
                // GridLut.cpp:109: data = dcf * sample
                val[k] = __fmul_rn(d, ((f0 + 32 * k) & 1) ? z.y : z.x);
            }
        }
        // Clamped cell range (GridLut.cpp:98-106), clipped to this tile.
        int sx, ex, sy, ey, sz = 0, ez = 0;
        comp_range(p.x, P.hw, (unsigned)P.G, sx, ex);
        comp_range(p.y, P.hw, (unsigned)P.G, sy, ey);
        if (DIM == 3) comp_range(p.z, P.hw, (unsigned)P.G, sz, ez);
        sx = max(sx, ox); ex = min(ex, hx);
        sy = max(sy, oy); ey = min(ey, hy);
        if (DIM == 3) { sz = max(sz, oz); ez = min(ez, hz); }
        if (P.prefilter) {
            // Drop end taps with |d| >= kHW: with kHW^2 exact such taps
            // have dk >= kHW, so the valid set is unchanged.
            if (sx <= ex && !(fabsf(__fsub_rn((float)sx, p.x)) < P.hw)) ++sx;
            if (sx <= ex && !(fabsf(__fsub_rn((float)ex, p.x)) < P.hw)) --ex;
            if (sy <= ey && !(fabsf(__fsub_rn((float)sy, p.y)) < P.hw)) ++sy;
            if (sy <= ey && !(fabsf(__fsub_rn((float)ey, p.y)) < P.hw)) --ey;
            if (DIM == 3) {
                if (sz <= ez && !(fabsf(__fsub_rn((float)sz, p.z)) < P.hw)) ++sz;
                if (sz <= ez && !(fabsf(__fsub_rn((float)ez, p.z)) < P.hw)) --ez;
            }
        }
        const int nx = ex - sx + 1, ny = ey - sy + 1, nz = ez - sz + 1;
        if (nx <= 0 || ny <= 0 || nz <= 0) continue;
        const int ntap = nx * ny * nz;
        const bool small = nx <= 4 && ny <= 4 && nz <= 4;
        // Small footprints use a fixed 4x4(x4) lane layout: one round in 2D,
        // one or two (z pairs) in 3D.
        const int nround = small ? (DIM == 3 && nz > 2 ? 2 : 1) : (ntap + 31) / 32;
        for (int rnd = 0; rnd < nround; ++rnd) {
            int ix, iy, iz;
            bool ok;
            if (small) {
                int tt = rnd * 32 + lane;
                ix = tt & 3;
                iy = (tt >> 2) & 3;
                iz = tt >> 4;
                ok = ix < nx && iy < ny && iz < nz;
            } else {
                int tt = rnd * 32 + lane;
                ok = tt < ntap;
                ix = tt % nx;
                int r = tt / nx;
                iy = r % ny;
                iz = r / ny;
            }
            int cell = 0;
            float w = 0.f;
            if (ok) {
                int x = sx + ix, y = sy + iy, z = sz + iz;
                float dx = __fsub_rn((float)x, p.x);
                float dy = __fsub_rn((float)y, p.y);
                float dz = DIM == 3 ? __fsub_rn((float)z, p.z) : 0.f;
                int ki = tap_index(dx, __fmul_rn(dy, dy), __fmul_rn(dz, dz), P.hw, P.inv_hw, P.hw_pow2,
                                   P.lm1, P.L);
                ok = ki >= 0;
                if (ok) {
                    w = lut[ki];
                    cell = ((z - oz) * P.tile[1] + (y - oy)) * P.tile[0] + (x - ox);
                }
            }
            unsigned m = __ballot_sync(0xffffffffu, ok);
            while (m) {
                int src[NG];
#pragma unroll
                for (int g = 0; g < NG; ++g) {
                    src[g] = m ? __ffs(m) - 1 : -1;
                    m &= m - 1;
                }
                int mysrc = src[0];
#pragma unroll
                for (int g = 1; g < NG; ++g)
                    if (q == g) mysrc = src[g];
                int cq = __shfl_sync(0xffffffffu, cell, mysrc & 31);
                float wq = __shfl_sync(0xffffffffu, w, mysrc & 31);
                if (mysrc >= 0) {
                    float *row = acc + (size_t)cq * R;
                    const int sw = swz<R>(cq);
#pragma unroll
                    for (int k = 0; k < NF; ++k)
                        if (coil_ok[k]) atomicAdd(row + ((f0 + 32 * k) ^ sw), __fmul_rn(wq, val[k]));
                }
            }
        }
    }
    __syncthreads();

    if (it.slot < 0) {
        write_cell_group<R>(P, acc, cg, ox, oy, oz, false);
    } else {
        float4 *dst = reinterpret_cast<float4 *>(
            P.partials + ((size_t)it.slot * P.ngroups + cg) * (size_t)K * R);
        for (int i = threadIdx.x; i < K * R / 4; i += blockDim.x) dst[i] = smem4[i];
    }
}

// Sum the partial tiles of each split tile in item order and write the grid.
template <int R>
__global__ void reduce_splits_kernel(GridParams P)
{
    const SplitTile st = P.splits[blockIdx.x];
    const int cg = blockIdx.y;
    const int t = st.tile;
    const int ox = (t % P.ntile[0]) * P.tile[0];
    const int oy = ((t / P.ntile[0]) % P.ntile[1]) * P.tile[1];
    const int oz = (t / (P.ntile[0] * P.ntile[1])) * P.tile[2];
    const int K = P.K, CG = P.coil_group;
    const size_t G = (size_t)P.G;
    const size_t cells = P.dim == 3 ? G * G * G : G * G;
    float2 *grid = reinterpret_cast<float2 *>(P.grid);
    const size_t slot_stride = (size_t)P.ngroups * K * R;
    const float *base = P.partials + ((size_t)st.first_slot * P.ngroups + cg) * (size_t)K * R;
    const int total = CG * K;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        int cl = idx / K;
        int i = idx - cl * K;
        int c = cg * CG + cl;
        if (c >= P.channels) break;
        int lx = i % P.tile[0];
        int r = i / P.tile[0];
        int ly = r % P.tile[1];
        int lz = r / P.tile[1];
        int gx = ox + lx, gy = oy + ly, gz = oz + lz;
        if (gx >= P.G || gy >= P.G || gz >= (P.dim == 3 ? P.G : 1)) continue;
        int col = (2 * cl) ^ swz<R>(i);
        float2 v = make_float2(0.f, 0.f);
        for (int k = 0; k < st.nslots; ++k) {
            float2 a = *reinterpret_cast<const float2 *>(base + k * slot_stride + (size_t)i * R + col);
            v.x = __fadd_rn(v.x, a.x);
            v.y = __fadd_rn(v.y, a.y);
        }
        if (P.checkerboard && ((gx + gy + gz) & 1)) {
            v.x = -v.x;
            v.y = -v.y;
        }
        grid[(size_t)c * cells + ((size_t)gz * G + (size_t)gy) * G + (size_t)gx] = v;
    }
}

template <int DIM, int R>
int launch(fr_plan p, const GridParams &P, long long nitems, long long nsplits, cudaStream_t s)
{
    size_t smem = (size_t)P.K * R * 4 + (size_t)P.L * 4;
    static_assert(R % 4 == 0, "rows of whole float4");
    auto kern = grid_tiles_kernel<DIM, R>;
    if (smem > 48 * 1024) FR_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int threads = 512;
    dim3 grid((unsigned)nitems, (unsigned)P.ngroups);
    cudaEvent_t *ev = nullptr;
    if (p->profile) {
        if (p->prof_used * 2 + 2 > (int)p->prof_ev.size()) {
            cudaEvent_t a, b;
            FR_CUDA(cudaEventCreate(&a));
            FR_CUDA(cudaEventCreate(&b));
            p->prof_ev.push_back(a);
            p->prof_ev.push_back(b);
        }
        ev = &p->prof_ev[p->prof_used * 2];
        p->prof_used++;
        FR_CUDA(cudaEventRecord(ev[0], s));
    }
    kern<<<grid, threads, smem, s>>>(P);
    FR_CHECK_LAUNCH("grid_tiles_kernel");
    if (ev) FR_CUDA(cudaEventRecord(ev[1], s));
    if (nsplits > 0) {
        dim3 g2((unsigned)nsplits, (unsigned)P.ngroups);
        reduce_splits_kernel<R><<<g2, 256, 0, s>>>(P);
        FR_CHECK_LAUNCH("reduce_splits_kernel");
    }
    return FR_OK;
}

}  // namespace

int floats_per_cell(int coil_group)
{
    int r = 8;
    while (r < 2 * coil_group) r <<= 1;
    return r;
}

void default_tiling(int dim, int *tile, int *coil_group, int channels)
{
    if (dim == 3) {
        tile[0] = 8; tile[1] = 8; tile[2] = 8;
    } else {
        tile[0] = 32; tile[1] = 32; tile[2] = 1;
    }
    if (*coil_group <= 0) {
        int cg = 4;
        while (cg < channels && cg < 16) cg <<= 1;
        *coil_group = cg;
    }
}

int grid_run(fr_plan p, const float *d_kdata, const float *d_dcf, int channels, float *d_grid,
             cudaStream_t s)
{
    if (!p->planned) return fail(FR_ERR_NOT_PLANNED, "fr_grid called before fr_plan_set_trajectory");
    if (channels <= 0) return fail(FR_ERR_INVALID_ARGUMENT, "channels must be positive");
    const int R = floats_per_cell(p->coil_group);
    GridParams P;
    P.traj = p->traj.as<float4>();
    P.pairs = p->pairs.as<unsigned>();
    P.items = p->items.as<WorkItem>();
    P.splits = p->splits.as<SplitTile>();
    P.kdata = d_kdata;
    P.dcf = d_dcf;
    P.lut = p->lut_d.as<float>();
    P.grid = d_grid;
    P.n = (long long)p->n;
    P.channels = channels;
    P.coil_group = p->coil_group;
    P.ngroups = (channels + p->coil_group - 1) / p->coil_group;
    P.dim = p->dim;
    P.G = (int)p->G;
    P.K = 1;
    for (int d = 0; d < 3; ++d) {
        P.tile[d] = p->tile[d];
        P.ntile[d] = p->ntile[d];
        P.K *= p->tile[d];
    }
    P.L = p->L;
    P.hw = p->hw;
    int e;
    float m = frexpf(p->hw, &e);
    P.hw_pow2 = (m == 0.5f);
    P.inv_hw = P.hw_pow2 ? ldexpf(1.0f, 1 - e) : 0.f;
    P.lm1 = (float)(p->L - 1);
    {
        // Prefilter is exact when sqrt(fl(hw*hw)) rounds back to hw.
        float h2 = p->hw * p->hw;
        P.prefilter = (sqrtf(h2) == p->hw) && (h2 == (double)p->hw * (double)p->hw);
    }
    P.checkerboard = (p->flags & FR_PLAN_CHECKERBOARD) ? 1 : 0;
    if (p->nslots > 0) {
        size_t bytes = (size_t)p->nslots * P.ngroups * (size_t)P.K * R * 4;
        if (p->partials.reserve(bytes)) return FR_ERR_OUT_OF_MEMORY;
    }
    P.partials = p->partials.as<float>();
    if (p->nitems == 0) return FR_OK;
    if (p->dim == 3) {
        switch (R) {
        case 8: return launch<3, 8>(p, P, p->nitems, p->nsplits, s);
        case 16: return launch<3, 16>(p, P, p->nitems, p->nsplits, s);
        case 32: return launch<3, 32>(p, P, p->nitems, p->nsplits, s);
        case 64: return launch<3, 64>(p, P, p->nitems, p->nsplits, s);
        }
    } else {
        switch (R) {
        case 8: return launch<2, 8>(p, P, p->nitems, p->nsplits, s);
        case 16: return launch<2, 16>(p, P, p->nitems, p->nsplits, s);
        case 32: return launch<2, 32>(p, P, p->nitems, p->nsplits, s);
        case 64: return launch<2, 64>(p, P, p->nitems, p->nsplits, s);
        }
    }
    return fail(FR_ERR_UNSUPPORTED, "coil group must be 4, 8, 16 or 32");
}

}  // namespace fr
