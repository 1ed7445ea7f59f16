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
    const unsigned long long *recs;  // sample index | tap box << 32, sorted by tile
    const WorkItem *items;
    const SplitTile *splits;
    const float *kdata;  // channels x n complex64, as floats
    const float *dcf;
    const float4 *lut_e; // {thr[k+1], lut[k], lut[k+1], 0}, staged into shared memory
    float *grid;         // channels x G^d complex64, as floats
    float *partials;     // nslots x ngroups x K x R floats
    long long n;
    int channels, coil_group, ngroups;
    int dim, G;
    int tile[3], ntile[3], K;
    int L;
    float smax, kc, khalf;  // exact LUT index from s = dk^2 (LutIndexTable)
    int checkerboard;
    // batches of frames (nullptr / 0 for one trajectory): frame f owns
    // samples [frame_off[f], frame_off[f+1]), its k-space block starts at
    // channels * frame_off[f] complex values, its grid at f * grid_frame_floats;
    // work items and split tiles carry their frame in `pad`.
    const long long *frame_off;
    long long grid_frame_floats;
    int *work_counter;  // persistent kernel: next work index
    long long nwork;    // persistent kernel: nitems * ngroups
    float lut_absmax;   // max |lut[k]|: bounds every tap weight
    // k-space sample-major ([n][channels] complex, from transpose_kspace):
    // a record's coil values are one contiguous run instead of one value per
    // coil plane
    int sample_major;
    // k-space values already multiplied by the DCF (the sample-major copy),
    // with mag[s] = max over the sample's coil floats of |dcf * k|: the
    // per-item scale then needs one float per record
    const float *mag;
    int skip_empty;     // tiles without samples are left unwritten
    // tap lists (grid_taps_kernel): per record sample | first word << 32 |
    // taps << 40, per sample a slot of tap_words tap words
    const unsigned long long *trecs = nullptr;
    const unsigned *taps = nullptr;
    const float *lutw = nullptr;        // L weights
    const float *item_inv = nullptr;    // per work item: inverse fixed-point scale
    int tap_words = 0;
    long long kstride = 0;    // complex values per sample row of the sample-major k-space
    int *err = nullptr;       // mapped error word
    int accumulate = 0;       // add the tiles to the grid instead of overwriting it (sample partitions)
    long long kin_stride = 0; // complex values between coils of the caller's coil-major k-space (0: n)
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

// Explicit shared-memory accesses on 32-bit shared addresses (generic
// pointers would make every float atomic a run-time address-space dispatch).
__device__ __forceinline__ unsigned smem_addr(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}
// Fixed-point accumulation: a float shared-memory add is a compare-and-swap
// loop on this GPU, an integer add is one native instruction.  Each tap adds
// round(w * v * S) (S a power of two chosen per work item and coil float so
// that no partial sum can leave the int32 range, see grid_item); the float
// value is acc / S at the flush.
__device__ __forceinline__ void red_add_fx(unsigned a, float w, float vs)
{
    // w * vs rounded to the nearest integer: |w * vs| < 2^22, so adding
    // 1.5 * 2^23 in the same fused operation lands in [2^23, 2^24), where the
    // float spacing is 1, and the low mantissa bits are the integer.
    const int i = __float_as_int(fmaf(w, vs, 12582912.f)) - 0x4B400000;
    asm volatile("red.shared.add.s32 [%0], %1;" ::"r"(a), "r"(i));
}
__device__ __forceinline__ int2 lds_i32x2(unsigned a)
{
    int2 r;
    asm volatile("ld.shared.v2.s32 {%0, %1}, [%2];" : "=r"(r.x), "=r"(r.y) : "r"(a) : "memory");
    return r;
}
__device__ __forceinline__ int4 lds_s32x4(unsigned a)
{
    int4 r;
    asm volatile("ld.shared.v4.s32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
                 : "r"(a)
                 : "memory");
    return r;
}
__device__ __forceinline__ int2 lds_s32x2(unsigned a)
{
    int2 r;
    asm volatile("ld.shared.v2.s32 {%0, %1}, [%2];" : "=r"(r.x), "=r"(r.y) : "r"(a) : "memory");
    return r;
}
__device__ __forceinline__ float lds_f32(unsigned a)
{
    float r;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(r) : "r"(a) : "memory");
    return r;
}
__device__ __forceinline__ float4 lds_f32x4(unsigned a)
{
    float4 r;
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w)
                 : "r"(a)
                 : "memory");
    return r;
}
__device__ __forceinline__ void sts_s32x2(unsigned a, int2 v)
{
    asm volatile("st.shared.v2.s32 [%0], {%1, %2};" ::"r"(a), "r"(v.x), "r"(v.y) : "memory");
}

// A cell pair / cell of the grid: stored, or added to what is there when the
// plan accumulates sample partitions into one grid.
__device__ __forceinline__ void put_cells(float4 *dst, float4 v, int add)
{
    if (add) {
        const float4 o = *dst;
        v = make_float4(__fadd_rn(o.x, v.x), __fadd_rn(o.y, v.y), __fadd_rn(o.z, v.z), __fadd_rn(o.w, v.w));
    }
    *dst = v;
}
__device__ __forceinline__ void put_cells(float2 *dst, float2 v, int add)
{
    if (add) {
        const float2 o = *dst;
        v = make_float2(__fadd_rn(o.x, v.x), __fadd_rn(o.y, v.y));
    }
    *dst = v;
}

// Flush (or zero-fill) the tile's cells for one coil group.  Threads map to
// (x pair, row): each writes two consecutive x cells as one 16-byte store
// (even tile x extent and grid size), rows advance without divisions.
template <int R>
__device__ __forceinline__ void write_cell_group(const GridParams &P, float *gridf, unsigned acc, int cg, int ox, int oy,
                                                 int oz, bool zero, const float *inv_scale)
{
    const int CG = P.coil_group;
    const int Tx = P.tile[0], Ty = P.tile[1], Tz = P.tile[2];
    const int ncl = min(CG, P.channels - cg * CG);
    const size_t G = (size_t)P.G;
    const int Gz = P.dim == 3 ? P.G : 1;
    const size_t cells = P.dim == 3 ? G * G * G : G * G;
    const int rows = Ty * Tz;
    const bool pairs = (Tx % 2 == 0) && (P.G % 2 == 0) && ((int)blockDim.x % (Tx / 2) == 0) &&
                       ((reinterpret_cast<uintptr_t>(gridf) & 15) == 0);
    const int npair = (Tx / 2) * rows;  // x pairs of the tile
    if (pairs && (int)blockDim.x % npair == 0) {
        // Each thread keeps one x pair for every coil it writes (coils
        // tid / npair, + blockDim / npair, ...): the pair's grid offset, its
        // swizzled columns and checkerboard signs are computed once.
        const int slot = threadIdx.x % npair, cstep = blockDim.x / npair;
        const int lx = 2 * (slot % (Tx / 2)), r = slot / (Tx / 2);
        const int gx = ox + lx, gy = oy + r % Ty, gz = oz + r / Ty;
        if (gx >= P.G || gy >= P.G || gz >= Gz) return;  // gx even, G even: gx + 1 < G as well
        float4 *gridc = reinterpret_cast<float4 *>(gridf) + ((((size_t)gz * G + (size_t)gy) * G + (size_t)gx) >> 1);
        const size_t cstride4 = cells >> 1;  // float4 per coil plane (G even)
        const int i = r * Tx + lx;
        const unsigned ra = acc + 4u * (unsigned)(i * R), rb = ra + 4u * (unsigned)R;
        const int swa = swz<R>(i), swb = swz<R>(i + 1);
        // (-1)^(x+y+z): opposite signs for x and x+1
        const float sa = P.checkerboard && ((gx + gy + gz) & 1) ? -1.f : 1.f;
        const float sb = P.checkerboard ? -sa : 1.f;
        for (int cl = threadIdx.x / npair; cl < ncl; cl += cstep) {
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (!zero) {
                const int2 a = lds_i32x2(ra + 4u * (unsigned)((2 * cl) ^ swa));
                const int2 b = lds_i32x2(rb + 4u * (unsigned)((2 * cl) ^ swb));
                const float ir = inv_scale[2 * cl], ii = inv_scale[2 * cl + 1];
                v = make_float4((float)a.x * ir * sa, (float)a.y * ii * sa, (float)b.x * ir * sb, (float)b.y * ii * sb);
            }
            put_cells(&gridc[(size_t)(cg * CG + cl) * cstride4], v, P.accumulate);
        }
        return;
    }
    if (pairs) {
        const int hx = Tx / 2;
        const int lx = 2 * (threadIdx.x % hx), rr0 = threadIdx.x / hx, rstep = blockDim.x / hx;
        const int dy = rstep % Ty, dz = rstep / Ty;
        const int gx = ox + lx;
        const bool xin = gx < P.G;  // gx even, G even: gx + 1 < G as well
        for (int cl = 0; cl < ncl; ++cl) {
            float4 *gridc = reinterpret_cast<float4 *>(gridf + 2 * (size_t)(cg * CG + cl) * cells);
            const float ir = zero ? 0.f : inv_scale[2 * cl], ii = zero ? 0.f : inv_scale[2 * cl + 1];
            int ly = rr0 % Ty, lz = rr0 / Ty;
            for (int r = rr0; r < rows; r += rstep) {
                const int gy = oy + ly, gz = oz + lz;
                if (xin && gy < P.G && gz < Gz) {
                    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (!zero) {
                        const int i = r * Tx + lx;
                        const int2 a = lds_i32x2(acc + 4u * (unsigned)(i * R + ((2 * cl) ^ swz<R>(i))));
                        const int2 b = lds_i32x2(acc + 4u * (unsigned)((i + 1) * R + ((2 * cl) ^ swz<R>(i + 1))));
                        v = make_float4((float)a.x * ir, (float)a.y * ii, (float)b.x * ir, (float)b.y * ii);
                        if (P.checkerboard) {  // (-1)^(x+y+z): opposite signs for x and x+1
                            if ((gx + gy + gz) & 1) {
                                v.x = -v.x;
                                v.y = -v.y;
                            } else {
                                v.z = -v.z;
                                v.w = -v.w;
                            }
                        }
                    }
                    put_cells(&gridc[(((size_t)gz * G + (size_t)gy) * G + (size_t)gx) >> 1], v, P.accumulate);
                }
                ly += dy;
                lz += dz;
                if (ly >= Ty) {
                    ly -= Ty;
                    ++lz;
                }
            }
        }
        return;
    }
    const int K = P.K;
    float2 *grid = reinterpret_cast<float2 *>(gridf);
    for (int idx = threadIdx.x; idx < ncl * K; idx += blockDim.x) {
        int cl = idx / K;
        int i = idx - cl * K;
        int lx = i % Tx;
        int r = i / Tx;
        int ly = r % Ty;
        int lz = r / Ty;
        int gx = ox + lx, gy = oy + ly, gz = oz + lz;
        if (gx >= P.G || gy >= P.G || gz >= Gz) continue;
        float2 v = make_float2(0.f, 0.f);
        if (!zero) {
            const int2 a = lds_i32x2(acc + 4u * (unsigned)(i * R + ((2 * cl) ^ swz<R>(i))));
            v = make_float2((float)a.x * inv_scale[2 * cl], (float)a.y * inv_scale[2 * cl + 1]);
            if (P.checkerboard && ((gx + gy + gz) & 1)) {
                v.x = -v.x;
                v.y = -v.y;
            }
        }
        put_cells(&grid[(size_t)(cg * CG + cl) * cells + ((size_t)gz * G + (size_t)gy) * G + (size_t)gx], v,
                  P.accumulate);
    }
}

constexpr int kWarps = 16;         // 512 threads per CTA
constexpr int kListEntries = 32;   // per warp and buffer
constexpr int kScaleBatch = 4;     // records per warp step of the scale pass
constexpr int kDecBytes = 16 * 64 * 16;  // tap decode table: 16 box classes x 64 taps x float4

// Shared-memory layout of the scatter: accumulator tile [K][R] int32 | LUT
// entries [L] float4 | per warp two tap-list buffers [32] {shared address of
// the tap's cell row (swizzled), weight} | tap decode table [16][64] float4 |
// per coil float: bound sum, bound max, inverse scale [3][64] floats.
//
// Decode table: for a tap box of nx x ny x nz cells (nx, ny <= 4; class
// (nx-1)*4 + (ny-1)), tap tt = ix + nx (iy + ny iz) is the float4 {ix, iy,
// iz, cell offset (iz Ty + iy) Tx + ix as int bits}: one 16-byte load per
// lane, no unpacking or conversions.  Built without divisions: t / n for
// n <= 4 and t < 64 is (t * {128, 64, 43, 32}[n-1]) >> 7.
template <int R>
__device__ __forceinline__ void stage_tables(const GridParams &P, float4 *smem4)
{
    float4 *lutE_g = reinterpret_cast<float4 *>(reinterpret_cast<float *>(smem4) + (size_t)P.K * R);
    float4 *dec_g = reinterpret_cast<float4 *>(reinterpret_cast<unsigned char *>(lutE_g + P.L) +
                                               kWarps * 2 * kListEntries * 8);
    for (int i = threadIdx.x; i < P.L; i += blockDim.x) lutE_g[i] = P.lut_e[i];
    const int Tx = P.tile[0], Ty = P.tile[1];
    for (int i = threadIdx.x; i < 16 * 64; i += blockDim.x) {
        const int c = i >> 6, tt = i & 63;
        const int nx = (c >> 2) + 1, ny = (c & 3) + 1;
        const int mx = nx == 1 ? 128 : nx == 2 ? 64 : nx == 3 ? 43 : 32;
        const int my = ny == 1 ? 128 : ny == 2 ? 64 : ny == 3 ? 43 : 32;
        const int q1 = (tt * mx) >> 7, ix = tt - q1 * nx;
        const int iz = (q1 * my) >> 7, iy = q1 - iz * ny;
        dec_g[i] = make_float4((float)ix, (float)iy, (float)iz, __int_as_float((iz * Ty + iy) * Tx + ix));
    }
}

// Scale of the fixed-point tile, per coil float f: with B_f = sum and
// M_f = max over the item's samples of |dcf * k_f|, and |w| <= lut_absmax,
// every partial sum is below B_f * lut_absmax and every add below
// M_f * lut_absmax, so S_f = the largest power of two with
// S_f * B_f * lut_absmax <= 2^30 and S_f * M_f * lut_absmax <= 2^21 keeps
// the tile in int32 and each add exact to +-1/2.  The rounding error of an
// add is then at most B_f / 2^31 (dense items) or 2^-23 M_f.
//
// This warp's part of B_f and M_f over records warp, warp + NW, ... in steps
// of kScaleBatch records with every load of a step issued before the first
// is used (the pass is bound by the latency of these gathers).  PF: lane b of
// a step also pulls record b's position into L1 for the accumulation pass.
template <int NF, int NW, bool PF>
__device__ __forceinline__ void scale_bounds(const unsigned long long *recs, int count, int warp, int lane,
                                             const float4 *traj, const float *dcf, const float *const *kdf,
                                             size_t ks, const bool *coil_ok, float *bs, float *bm)
{
#pragma unroll
    for (int k = 0; k < NF; ++k) bs[k] = bm[k] = 0.f;
    for (int j0 = warp * kScaleBatch; j0 < count; j0 += NW * kScaleBatch) {
        unsigned sl = 0u;
        bool vl = false;
        if (lane < kScaleBatch && j0 + lane < count) {
            const unsigned long long rec = recs[j0 + lane];
            const unsigned box = (unsigned)(rec >> 32);
            sl = (unsigned)rec;
            vl = ((box >> 18) & 15) * ((box >> 22) & 15) * ((box >> 26) & 15) != 0;
            if (PF && vl) asm volatile("prefetch.global.L1 [%0];" ::"l"(traj + sl));
        }
        const unsigned vm = __ballot_sync(0xffffffffu, vl);
        float db[kScaleBatch], kb[kScaleBatch][NF];
#pragma unroll
        for (int b = 0; b < kScaleBatch; ++b) {
            const unsigned sv = __shfl_sync(0xffffffffu, sl, b);
            const bool v = (vm >> b) & 1u;
            db[b] = v ? dcf[sv] : 0.f;
#pragma unroll
            for (int k = 0; k < NF; ++k) kb[b][k] = v && coil_ok[k] ? kdf[k][ks * sv] : 0.f;
        }
#pragma unroll
        for (int b = 0; b < kScaleBatch; ++b) {
#pragma unroll
            for (int k = 0; k < NF; ++k) {
                const float a = fabsf(__fmul_rn(db[b], kb[b][k]));
                bs[k] += a;
                bm[k] = fmaxf(bm[k], a);
            }
        }
    }
}

// The bound of scale_bounds from the per-sample magnitudes mag[s] >= every
// |dcf * k_f| of sample s, one record per lane: one B and M for all coil
// floats of the item.  Also pulls each record's position into L1.
template <int NW>
__device__ __forceinline__ void scale_bounds_mag(const unsigned long long *recs, int count, int warp, int lane,
                                                 const float4 *traj, const float *mag, float &bs, float &bm)
{
    bs = bm = 0.f;
    for (int j = warp * 32 + lane; j < count; j += NW * 32) {
        const unsigned long long rec = recs[j];
        const unsigned box = (unsigned)(rec >> 32);
        const unsigned sl = (unsigned)rec;
        if (((box >> 18) & 15) * ((box >> 22) & 15) * ((box >> 26) & 15) != 0) {
            asm volatile("prefetch.global.L1 [%0];" ::"l"(traj + sl));
            const float a = mag[sl];
            bs += a;
            bm = fmaxf(bm, a);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        bs += __shfl_xor_sync(0xffffffffu, bs, o);
        bm = fmaxf(bm, __shfl_xor_sync(0xffffffffu, bm, o));
    }
}

// 1 / S_f from the item's B_f and M_f (exact: a power of two).
__device__ __forceinline__ float inv_scale_of(float bsum, unsigned bmax_bits, float lut_absmax)
{
    const float B = __fmul_rn(bsum, lut_absmax);
    const float M = __fmul_rn(__uint_as_float(bmax_bits), lut_absmax);
    int e = 0;
    if (B > 0.f && M > 0.f) {
        // largest power of two 2^e <= min(2^30 / B, 2^21 / M)
        const float t = fminf(__fdiv_rn(1073741824.f, B), __fdiv_rn(2097152.f, M));
        frexpf(t, &e);
        e = max(min(e - 1, 100), -100);
    }
    return ldexpf(1.f, -e);
}

// The k-space pointers of a lane: kdf[k][ks s] is coil float f0 + 32 k of
// sample s (coil_ok false past the group's or the data's last coil), ks = 2
// for coil-major k-space, 2 * channels for sample-major.
template <int NF>
__device__ __forceinline__ void lane_kspace(const GridParams &P, int cg, int f0, long long s_off, long long n_f,
                                            const float **kdf, bool *coil_ok)
{
    const int CG = P.coil_group;
#pragma unroll
    for (int k = 0; k < NF; ++k) {
        const int fl = f0 + 32 * k;
        const int coil = cg * CG + (fl >> 1);
        coil_ok[k] = (fl >> 1) < CG && coil < P.channels;
        const size_t cstride = P.sample_major ? (size_t)1 : P.frame_off ? (size_t)n_f : (size_t)P.kin_stride;
        kdf[k] = P.kdata + 2 * (size_t)P.channels * (size_t)s_off + 2 * (size_t)(coil_ok[k] ? coil : 0) * cstride +
                 (fl & 1);
    }
}

// One work item for one coil group: zero the tile, accumulate the item's
// samples, flush (or write the partial tile).  The LUT and decode tables must
// be staged; the caller synchronises the CTA before the next item.
template <int DIM, int R>
__device__ __forceinline__ void grid_item(const GridParams &P, const WorkItem &it, int cg, float4 *smem4)
{
    const int K = P.K;
    const unsigned acc = smem_addr(smem4);
    const unsigned lutE = acc + (unsigned)K * R * 4u;
    const unsigned lists = lutE + (unsigned)P.L * 16u;
    const unsigned dec = lists + (unsigned)(kWarps * 2 * kListEntries * 8);

    const int t = it.tile;
    const int tx = t % P.ntile[0];
    const int ty = (t / P.ntile[0]) % P.ntile[1];
    const int tz = t / (P.ntile[0] * P.ntile[1]);
    const int ox = tx * P.tile[0], oy = ty * P.tile[1], oz = tz * P.tile[2];

    // frame of this item (a single trajectory is frame 0 of one)
    const int f = P.frame_off ? it.pad : 0;
    const long long s_off = P.frame_off ? P.frame_off[f] : 0;
    const long long n_f = P.frame_off ? P.frame_off[f + 1] - s_off : P.n;
    float *gridf = P.grid + (size_t)f * (size_t)P.grid_frame_floats;
    const float4 *traj = P.traj + s_off;
    const float *dcf = P.dcf + s_off;

    float *bsum_s = reinterpret_cast<float *>(reinterpret_cast<unsigned char *>(smem4) + (size_t)K * R * 4 +
                                              (size_t)P.L * 16 + kWarps * 2 * kListEntries * 8 + kDecBytes);
    unsigned *bmax_s = reinterpret_cast<unsigned *>(bsum_s + 64);
    float *inv_s = bsum_s + 128;

    if (it.count == 0) {  // empty tile: stream zeros, unless the reader masks it
        if (!P.skip_empty) write_cell_group<R>(P, gridf, acc, cg, ox, oy, oz, true, inv_s);
        return;
    }

    for (int i = threadIdx.x; i < K * R / 4; i += blockDim.x) smem4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int i = threadIdx.x; i < 128; i += blockDim.x) bsum_s[i] = 0.f;  // bsum_s and bmax_s
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    constexpr int NG = R >= 32 ? 1 : 32 / R;  // taps per accumulate step
    constexpr int NF = R > 32 ? R / 32 : 1;   // floats per lane per tap
    const int q = R >= 32 ? 0 : lane / R;     // tap slot of this lane
    const int f0 = R >= 32 ? lane : lane % R; // first coil float of this lane
    const unsigned f0b = (unsigned)f0 << 2;   // its byte offset in a cell row
    const int Tx = P.tile[0], Ty = P.tile[1];
    const unsigned mylist = lists + (unsigned)(warp * 2 * kListEntries * 8);
    unsigned buf = 0;

    const float *kdf[NF];
    bool coil_ok[NF];
    lane_kspace<NF>(P, cg, f0, s_off, n_f, kdf, coil_ok);
    const size_t ks = P.sample_major ? 2 * (size_t)P.kstride : 2;
    const unsigned long long *recs = P.recs + it.begin;

    if (P.mag) {
        float bs, bm;
        scale_bounds_mag<kWarps>(recs, it.count, warp, lane, traj, P.mag + s_off, bs, bm);
        if (lane == 0) {
            atomicAdd(&bsum_s[0], bs);
            atomicMax(&bmax_s[0], __float_as_uint(bm));
        }
        __syncthreads();
        if (threadIdx.x < R) inv_s[threadIdx.x] = inv_scale_of(bsum_s[0], bmax_s[0], P.lut_absmax);
        __syncthreads();
    } else {
        float bs[NF], bm[NF];
        scale_bounds<NF, kWarps, true>(recs, it.count, warp, lane, traj, dcf, kdf, ks, coil_ok, bs, bm);
        if (q == 0) {
#pragma unroll
            for (int k = 0; k < NF; ++k) {
                if (coil_ok[k]) {
                    atomicAdd(&bsum_s[f0 + 32 * k], bs[k]);
                    atomicMax(&bmax_s[f0 + 32 * k], __float_as_uint(bm[k]));
                }
            }
        }
        __syncthreads();
        if (threadIdx.x < R) inv_s[threadIdx.x] = inv_scale_of(bsum_s[threadIdx.x], bmax_s[threadIdx.x], P.lut_absmax);
        __syncthreads();
    }
    const bool premul = P.mag != nullptr;
    float sc[NF];
#pragma unroll
    for (int k = 0; k < NF; ++k) sc[k] = __fdiv_rn(1.f, inv_s[f0 + 32 * k]);  // exact

    for (int j = warp; j < it.count; j += kWarps) {
        const unsigned long long rec = recs[j];
        const unsigned s = (unsigned)rec;
        const unsigned box = (unsigned)(rec >> 32);
        // tap box inside this tile, precomputed by the plan from the
        // reference cell range (GridLut.cpp:98-106)
        const int lx0 = box & 63, ly0 = (box >> 6) & 63, lz0 = (box >> 12) & 63;
        const int nx = (box >> 18) & 15, ny = (box >> 22) & 15, nz = (box >> 26) & 15;
        const int ntap = nx * ny * nz;
        if (ntap == 0) continue;
        const float4 p = traj[s];
        // GridLut.cpp:109 dcf * k (made by the k-space copy when premultiplied: the same product), scaled
        const float d = premul ? 1.f : dcf[s];
        float val[NF];
#pragma unroll
        for (int k = 0; k < NF; ++k) {
            const float dk = premul ? kdf[k][ks * s] : __fmul_rn(d, kdf[k][ks * s]);
            val[k] = coil_ok[k] ? __fmul_rn(dk, sc[k]) : 0.f;
        }
        const bool small = nx <= 4 && ny <= 4 && nz <= 4;
        const unsigned dtab = dec + (unsigned)((((nx - 1) & 3) * 4 + ((ny - 1) & 3)) * 64 * 16);
        // box origin as floats (integers below 2^24: exact), its first cell
        const float fgx = (float)(ox + lx0), fgy = (float)(oy + ly0), fgz = (float)(oz + lz0);
        const int cell0 = (lz0 * Ty + ly0) * Tx + lx0;
        const int nround = (ntap + 31) >> 5;
        for (int rnd = 0; rnd < nround; ++rnd) {
            // Every lane evaluates its tap (lanes past the box too, on table
            // entries that exist) and the ballot keeps the valid ones.
            const int tt = rnd * 32 + lane;
            float4 d4;
            if (small) {  // warp-uniform; nround <= 2, so tt < 64
                d4 = lds_f32x4(dtab + 16u * (unsigned)tt);
            } else {
                const int ix = tt % nx, r = tt / nx, iy = r % ny, iz = r / ny;
                d4 = make_float4((float)ix, (float)iy, (float)iz, __int_as_float((iz * Ty + iy) * Tx + ix));
            }
            const float dx = __fsub_rn(__fadd_rn(fgx, d4.x), p.x);
            const float dy = __fsub_rn(__fadd_rn(fgy, d4.y), p.y);
            const float dz = DIM == 3 ? __fsub_rn(__fadd_rn(fgz, d4.z), p.z) : 0.f;
            // GridLut.cpp:131: dk^2 = (dz^2 + dy^2) + dx^2, unfused
            const float s2 = __fadd_rn(__fadd_rn(__fmul_rn(dz, dz), __fmul_rn(dy, dy)), __fmul_rn(dx, dx));
            const bool ok = tt < ntap && s2 < P.smax;  // sqrtf(s2) < kHW
            // first guess k0 in {ki-1, ki}, then one exact threshold test
            float a;
            asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(a) : "f"(s2));
            const int k0 = (int)fminf(fmaf(a, P.kc, P.khalf), (float)(P.L - 1));
            const float4 en = lds_f32x4(lutE + 16u * (unsigned)k0);
            const float w = s2 >= en.x ? en.z : en.y;
            const int cell = cell0 + __float_as_int(d4.w);
            const int ex = (int)(acc + ((unsigned)(cell * R + swz<R>(cell)) << 2));
            const unsigned m = __ballot_sync(0xffffffffu, ok);
            if (m == 0) continue;
            // the list, padded to a multiple of four with weight-0 entries on
            // the tile's first cell row (they add exactly 0)
            const int n = __popc(m), n4 = (n + 3) & ~3;
            const unsigned lst = mylist + buf * (kListEntries * 8);
            buf ^= 1;
            const int pos = ok ? __popc(m & lt) : n + __popc(~m & lt);
            if (pos < n4) sts_s32x2(lst + 8u * (unsigned)pos, ok ? make_int2(ex, __float_as_int(w)) : make_int2((int)acc, 0));
            __syncwarp();
            // Entries hold the shared address of the tap's cell row; the tile
            // is 128-byte aligned, so the lane's swizzled float is address ^
            // f0b.  Lanes of coils beyond the last carry value 0 and add 0.
            if (NG == 1) {
                for (int k = 0; k < n4; k += 4) {
                    const int4 e2 = lds_s32x4(lst + 8u * k);
                    const int4 e3 = lds_s32x4(lst + 8u * k + 16u);
                    const unsigned a0 = (unsigned)e2.x ^ f0b, a1 = (unsigned)e2.z ^ f0b;
                    const unsigned a2 = (unsigned)e3.x ^ f0b, a3 = (unsigned)e3.z ^ f0b;
#pragma unroll
                    for (int kk = 0; kk < NF; ++kk) {
                        red_add_fx(a0 + 128u * kk, __int_as_float(e2.y), val[kk]);
                        red_add_fx(a1 + 128u * kk, __int_as_float(e2.w), val[kk]);
                        red_add_fx(a2 + 128u * kk, __int_as_float(e3.y), val[kk]);
                        red_add_fx(a3 + 128u * kk, __int_as_float(e3.w), val[kk]);
                    }
                }
            } else {
                for (int k = q; k < n4; k += NG) {
                    const int2 e1 = lds_s32x2(lst + 8u * k);
                    red_add_fx((unsigned)e1.x ^ f0b, __int_as_float(e1.y), val[0]);
                }
            }
        }
    }
    __syncthreads();

    if (it.slot < 0) {
        write_cell_group<R>(P, gridf, acc, cg, ox, oy, oz, false, inv_s);
    } else {
        // partial tile as floats, same swizzled [cell][coil float] layout
        float4 *dst = reinterpret_cast<float4 *>(
            P.partials + ((size_t)it.slot * P.ngroups + cg) * (size_t)K * R);
        const int4 *src = reinterpret_cast<const int4 *>(smem4);
        for (int i = threadIdx.x; i < K * R / 4; i += blockDim.x) {
            const int cell = (4 * i) / R, p0 = (4 * i) % R, sw = swz<R>(cell);
            const int4 a = src[i];
            dst[i] = make_float4((float)a.x * inv_s[p0 ^ sw], (float)a.y * inv_s[(p0 + 1) ^ sw],
                                 (float)a.z * inv_s[(p0 + 2) ^ sw], (float)a.w * inv_s[(p0 + 3) ^ sw]);
        }
    }
}

// One CTA per (work item, coil group).
// The dynamic shared memory from its first 128-byte boundary (every launch
// adds 128 bytes): tap-list entries carry absolute tile-row addresses that a
// lane XORs with its float offset.
__device__ __forceinline__ float4 *aligned_smem(float4 *raw)
{
    const unsigned a = smem_addr(raw);
    return raw + (((128u - (a & 127u)) & 127u) >> 4);
}

template <int DIM, int R>
__global__ void __launch_bounds__(512) grid_tiles_kernel(GridParams P)
{
    extern __shared__ float4 smem_raw[];
    float4 *smem4 = aligned_smem(smem_raw);
    const WorkItem it = P.items[blockIdx.x];
    if (it.count > 0) {
        stage_tables<R>(P, smem4);
        // grid_item's first barrier (after zeroing the tile) orders the staging
    }
    grid_item<DIM, R>(P, it, blockIdx.y, smem4);
}

// Persistent: as many CTAs as fit on the GPU, each taking work indices
// (coil group major, then item) from a counter until none are left.  Used
// for batches of frames with uneven sample counts; the counter is zeroed
// before each launch.
template <int DIM, int R>
__global__ void __launch_bounds__(512) grid_persistent_kernel(GridParams P)
{
    extern __shared__ float4 smem_raw[];
    float4 *smem4 = aligned_smem(smem_raw);
    __shared__ long long next;
    stage_tables<R>(P, smem4);
    const long long nitems = P.nwork / P.ngroups;
    for (;;) {
        __syncthreads();  // the previous item's flush is done with the tile
        if (threadIdx.x == 0) next = atomicAdd(P.work_counter, 1);
        __syncthreads();
        const long long w = next;
        if (w >= P.nwork) break;
        const int cg = (int)(w / nitems);
        const WorkItem it = P.items[w - (long long)cg * nitems];
        grid_item<DIM, R>(P, it, cg, smem4);
    }
}

// ---------------------------------------------------------------------------
// Scatter from the plan's tap lists.
//
// The geometry of every tap was evaluated once per trajectory by the plan,
// so per bin record the CTA only moves data and accumulates.  Each warp
// walks its share of the work item's records with the loads of kTapDepth
// records in flight: for record k + kTapDepth, lane t loads the record's tap
// word t (t + 32) and lane f its coil float f of the record's dcf * k values
// into registers while record k is accumulated.  Lanes decode the taps
// into the warp's list {shared address of the tap's cell row, weight}, and
// lanes mapped to coil floats add round(w * v * S) into the fixed-point
// tile as grid_item does.
// ---------------------------------------------------------------------------
constexpr int kTapDepth = 4;   // records in flight per warp
constexpr int kTapList = 64;   // list entries per warp (records hold <= kTapRecMax taps, padded)

// Shared-memory layout of grid_taps_kernel, from its 128-byte aligned base:
// tile [K][R] int32 | inverse scales [R] (256 B) | weights [L] | per warp two
// lists [kTapList] {address, weight} (consecutive records alternate).
struct TapSmem {
    unsigned inv, lutw, lists, end;
};
__host__ __device__ __forceinline__ TapSmem tap_smem_layout(long long K, int R, int L)
{
    TapSmem m;
    m.inv = (unsigned)(K * R * 4);
    m.lutw = m.inv + 256u;
    m.lists = m.lutw + (unsigned)((L * 4 + 15) & ~15);
    m.end = m.lists + (unsigned)(kWarps * 2 * kTapList * 8);
    return m;
}

// One record's data in flight: its tap count, the lane's tap words and the
// lane's coil float.
struct TapStage {
    int nt;
    unsigned t0, t1;
    float v;
};

// IT: index type of the tap words and values (32-bit when every index fits).
template <int R, typename IT>
__global__ void __launch_bounds__(512, 2) grid_taps_kernel(GridParams P)
{
    extern __shared__ float4 smem_raw[];
    float4 *smem4 = aligned_smem(smem_raw);
    const WorkItem it = P.items[blockIdx.x];
    const int cg = blockIdx.y;
    const int K = P.K;
    const int CG = P.coil_group;
    const TapSmem L_ = tap_smem_layout(K, R, P.L);
    const unsigned acc = smem_addr(smem4);
    float *inv_s = reinterpret_cast<float *>(reinterpret_cast<unsigned char *>(smem4) + L_.inv);
    float *lutw_s = reinterpret_cast<float *>(reinterpret_cast<unsigned char *>(smem4) + L_.lutw);

    const int t = it.tile;
    const int ox = (t % P.ntile[0]) * P.tile[0];
    const int oy = ((t / P.ntile[0]) % P.ntile[1]) * P.tile[1];
    const int oz = (t / (P.ntile[0] * P.ntile[1])) * P.tile[2];

    if (it.count == 0) {
        if (!P.skip_empty) write_cell_group<R>(P, P.grid, acc, cg, ox, oy, oz, true, inv_s);
        return;
    }
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const unsigned lists = acc + L_.lists + (unsigned)(warp * 2 * kTapList * 8);

    for (int i = threadIdx.x; i < K * R / 4; i += blockDim.x) smem4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int i = threadIdx.x; i < P.L; i += blockDim.x) lutw_s[i] = P.lutw[i];
    const float inv = P.item_inv[blockIdx.x];
    if (threadIdx.x < R) inv_s[threadIdx.x] = inv;
    __syncthreads();

    constexpr int NG = R >= 32 ? 1 : 32 / R;  // taps per accumulate step
    constexpr int PAD = NG > 2 ? NG : 2;      // list length granularity
    const int q = R >= 32 ? 0 : lane / R;     // tap slot of this lane
    const int f0 = R >= 32 ? lane : lane % R; // coil float of this lane
    const unsigned f0b = (unsigned)f0 << 2;
    const float sc = __fdiv_rn(1.f, inv);     // exact: a power of two
    const int ncl = min(CG, P.channels - cg * CG);
    const bool vlane = (f0 >> 1) < ncl;
    const float *kt = P.kdata + 2 * (size_t)cg * CG + f0;
    const unsigned *taps = P.taps;
    const size_t tw = (size_t)P.tap_words;

    // the warp's records: record k of warp w is record w + kWarps k of the
    // item (every warp within one record of the others); their words are
    // read 32 at a time, record k from lane k % 32 of batch k / 32.  Words
    // past the item read as 0 (no taps).
    const int nrec = warp < it.count ? (it.count - warp + kWarps - 1) / kWarps : 0;
    const unsigned long long *trecs = P.trecs + it.begin;
    // a batch of 32 records, one per lane, as index of the lane's record's
    // first tap word, index of its coil group's values, tap count
    struct Batch {
        IT tb, vo;
        int nt;
    };
    auto load_batch = [&](int i) -> Batch {
        const int k = 32 * i + lane;
        const unsigned long long rw = k < nrec ? __ldg(trecs + warp + kWarps * k) : 0ull;
        Batch b;
        b.nt = (int)((rw >> 40) & 0xFF);
        b.tb = (IT)(unsigned)rw * (IT)tw + (IT)((rw >> 32) & 0xFF);
        b.vo = (IT)(unsigned)rw * (IT)(2 * P.kstride);
        return b;
    };
    auto fetch = [&](const Batch &b, int src_lane, TapStage &st) {
        st.nt = __shfl_sync(0xffffffffu, b.nt, src_lane);
        const IT tb = __shfl_sync(0xffffffffu, b.tb, src_lane);
        const IT vo = __shfl_sync(0xffffffffu, b.vo, src_lane);
        st.t0 = lane < st.nt ? __ldg(taps + tb + (IT)lane) : 0u;
        st.t1 = lane + 32 < st.nt ? __ldg(taps + tb + (IT)(lane + 32)) : 0u;
        st.v = vlane && st.nt ? __ldg(kt + vo) : 0.f;
    };

    Batch cur = load_batch(0), nxt = load_batch(1);
    TapStage st[kTapDepth];
#pragma unroll
    for (int d = 0; d < kTapDepth; ++d) fetch(cur, d, st[d]);

    static_assert(kTapDepth % 2 == 0 && 32 % kTapDepth == 0, "records alternate lists; batches hold whole groups");
    for (int k0 = 0; k0 < nrec; k0 += kTapDepth) {
        if (k0 > 0 && (k0 & 31) == 0) {
            cur = nxt;
            nxt = load_batch((k0 >> 5) + 1);
        }
        // the refills of this group come from the next batch only in the
        // batch's last group
        const Batch &src = (k0 & 31) == 32 - kTapDepth ? nxt : cur;
#pragma unroll
        for (int d = 0; d < kTapDepth; ++d) {
            const int k = k0 + d;
            // consecutive records alternate lists: record k + 1's decode
            // never overwrites the list record k is still adding from, so
            // one warp barrier per record (after the decode) orders both
            const unsigned list = lists + (unsigned)((d & 1) * kTapList * 8);
            const int ntap = st[d].nt;
            const int np = (ntap + PAD - 1) / PAD * PAD;
            const float vs = __fmul_rn(st[d].v, sc);
            if (ntap > 0) {
                // decode: list entry i = {address of tap i's cell row, weight};
                // pad entries add 0 to the first cell row
                int2 e = make_int2((int)acc, 0);
                if (lane < ntap) {
                    const int cell = (int)(st[d].t0 & ((1u << kTapCellBits) - 1u));
                    e.x = (int)(acc + ((unsigned)(cell * R + swz<R>(cell)) << 2));
                    e.y = __float_as_int(lds_f32(acc + L_.lutw + 4u * (st[d].t0 >> kTapCellBits)));
                }
                if (lane < np) sts_s32x2(list + 8u * (unsigned)lane, e);
                if (np > 32) {
                    int2 e1 = make_int2((int)acc, 0);
                    if (lane + 32 < ntap) {
                        const int cell = (int)(st[d].t1 & ((1u << kTapCellBits) - 1u));
                        e1.x = (int)(acc + ((unsigned)(cell * R + swz<R>(cell)) << 2));
                        e1.y = __float_as_int(lds_f32(acc + L_.lutw + 4u * (st[d].t1 >> kTapCellBits)));
                    }
                    if (lane + 32 < np) sts_s32x2(list + 8u * (unsigned)(lane + 32), e1);
                }
            }
            __syncwarp();
            // refill this stage with record k + kTapDepth
            const int k2 = k + kTapDepth;
            if (k2 < nrec) {
                fetch(src, k2 & 31, st[d]);
            } else {
                st[d].nt = 0;
            }
            if (ntap > 0) {
                if (NG == 1) {
#pragma unroll 2
                    for (int m = 0; m < np; m += 2) {
                        const int4 e = lds_s32x4(list + 8u * (unsigned)m);
                        red_add_fx((unsigned)e.x ^ f0b, __int_as_float(e.y), vs);
                        red_add_fx((unsigned)e.z ^ f0b, __int_as_float(e.w), vs);
                    }
                } else {
                    for (int m = q; m < np; m += NG) {
                        const int2 e = lds_s32x2(list + 8u * (unsigned)m);
                        red_add_fx((unsigned)e.x ^ f0b, __int_as_float(e.y), vs);
                    }
                }
            }
        }
    }
    __syncthreads();
    if (it.slot < 0) {
        write_cell_group<R>(P, P.grid, acc, cg, ox, oy, oz, false, inv_s);
    } else {
        float4 *dst = reinterpret_cast<float4 *>(P.partials + ((size_t)it.slot * P.ngroups + cg) * (size_t)K * R);
        const int4 *src = reinterpret_cast<const int4 *>(smem4);
        for (int i = threadIdx.x; i < K * R / 4; i += blockDim.x) {
            const int4 a = src[i];
            dst[i] = make_float4((float)a.x * inv, (float)a.y * inv, (float)a.z * inv, (float)a.w * inv);
        }
    }
}

// ---------------------------------------------------------------------------
// Tap-lane scatter (rows of 32 coil floats, the tap lists of the plan): each
// lane owns a group of kLaneTaps taps of one bin record and adds them for all
// 32 coil floats of its coil group, so the taps' cell rows and weights stay
// in the lane's registers and no per-record tap list goes through shared
// memory.
//
// A warp holds 32 of its records at a time (a window): their tap groups are
// numbered by a warp scan and dealt to the lanes 32 per pass, so a pass packs
// the groups of several records (a record's groups are consecutive).  Each
// record's 32 coil values (dcf * k) are first copied into a 128-byte slot of
// the warp's staging area by a bulk (TMA) copy, issued by the lane holding
// the record and completing on the warp's mbarrier; the item's fixed-point
// scale goes on the weights.
//
// Bank-conflict-free adds: at step t lane j adds coil float t ^ j of each of
// its taps.  The tile is [cell][32] int32 with 128-byte rows, so the 32
// lanes of one red.shared hit the 32 banks once each, whatever their cells;
// the lane reads the same float t ^ j of its record's slot (again one bank
// per lane).  The adds are those of grid_taps_kernel (same fixed-point
// values), so a tile held by one work item grids to the same bits.
// ---------------------------------------------------------------------------
constexpr int kLaneWarps = 8;   // 256 threads per CTA
constexpr int kLaneBatch = 32;  // records per warp window (one per lane)
constexpr int kLaneTaps = 4;    // taps of one record per lane (one read of its values serves them all)
static_assert(kLaneTaps == 4, "a lane's taps are loaded as one 16-byte word from aligned runs");

// Shared-memory layout of grid_lanes_kernel from its 128-byte aligned base:
// tile [K][32] int32 | weights [L] | per warp: value slots [32][32] floats,
// record table [32] int4 {sample, first word | taps << 8, first group, 0} |
// per warp one mbarrier (8 bytes).
struct LaneSmem {
    unsigned lutw, stage, table, mbar, end;
};
__host__ __device__ __forceinline__ LaneSmem lane_smem_layout(long long K, int L)
{
    LaneSmem m;
    m.lutw = (unsigned)(K * 32 * 4);
    m.stage = m.lutw + (unsigned)((L * 4 + 127) & ~127);
    m.table = m.stage + (unsigned)(kLaneWarps * kLaneBatch * 128);
    m.mbar = m.table + (unsigned)(kLaneWarps * kLaneBatch * 16);
    m.end = m.mbar + (unsigned)(kLaneWarps * 8);
    return m;
}

__device__ __forceinline__ float lds_f32_v(unsigned a)
{
    float r;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(r) : "r"(a));
    return r;
}

// Bulk copies of the records' coil values into the warp's slots, completing
// on the warp's mbarrier (the copies are issued by the lanes holding the
// records, one 16..128-byte copy each; global source and shared slot 16-byte
// aligned, sizes a multiple of 16).
__device__ __forceinline__ void mbar_init(unsigned mbar)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned mbar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_copy_g2s(unsigned dst, const void *src, unsigned bytes, unsigned mbar)
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the slot was last read by plain loads
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(mbar)
                 : "memory");
}
// Waits (non-blocking polls, bounded: about 2^20 polls with short sleeps,
// tens of milliseconds) for the phase of the given parity; false on timeout.
__device__ __forceinline__ bool mbar_wait(unsigned mbar, unsigned parity)
{
    for (int i = 0; i < (1 << 20); ++i) {
        unsigned done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
        if (i >= 32) __nanosleep(32);
    }
    return false;
}

// Flush of a [cell][32] tile (rows not swizzled): lane = (coil cl = lane & 15,
// pair px = lane >> 4), so that one 8-byte shared load per lane covers the 32
// banks and lanes cl, cl + 16 write the two halves of one 32-byte sector of
// coil plane cl.  Units (tile row, two x pairs) are dealt to the warps.
__device__ __forceinline__ void lanes_flush(const GridParams &P, unsigned acc, int cg, int ox, int oy, int oz, float inv)
{
    const int Tx = P.tile[0], Ty = P.tile[1], Tz = P.tile[2];
    const int CG = P.coil_group;
    const int ncl = min(CG, P.channels - cg * CG);
    const size_t G = (size_t)P.G;
    const int Gz = P.dim == 3 ? P.G : 1;
    const size_t cells = P.dim == 3 ? G * G * G : G * G;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    float *gridf = P.grid;
    if ((Tx % 4) == 0 && (P.G % 2) == 0 && ((reinterpret_cast<uintptr_t>(gridf) & 15) == 0)) {
        const int cl = lane & 15, px = lane >> 4;
        const int ppr = Tx / 4;  // x pair-pairs per row
        const int units = Ty * Tz * ppr;
        const size_t cstride4 = cells >> 1;
        float4 *grid4 = reinterpret_cast<float4 *>(gridf) + (size_t)(cg * CG + cl) * cstride4;
        for (int u = warp; u < units; u += nwarps) {
            const int r = u / ppr, pp = u - r * ppr;
            const int lx = 4 * pp + 2 * px;
            const int gx = ox + lx, gy = oy + r % Ty, gz = oz + r / Ty;
            if (cl >= ncl || gx >= P.G || gy >= P.G || gz >= Gz) continue;
            const int i = r * Tx + lx;
            const int2 a = lds_i32x2(acc + ((unsigned)i << 7) + ((unsigned)cl << 3));
            const int2 b = lds_i32x2(acc + ((unsigned)(i + 1) << 7) + ((unsigned)cl << 3));
            const float sa = P.checkerboard && ((gx + gy + gz) & 1) ? -inv : inv;
            const float sb = P.checkerboard ? -sa : inv;
            const float4 v = make_float4((float)a.x * sa, (float)a.y * sa, (float)b.x * sb, (float)b.y * sb);
            put_cells(&grid4[(((size_t)gz * G + (size_t)gy) * G + (size_t)gx) >> 1], v, P.accumulate);
        }
        return;
    }
    const int K = P.K;
    float2 *grid = reinterpret_cast<float2 *>(gridf);
    for (int idx = threadIdx.x; idx < ncl * K; idx += blockDim.x) {
        const int i = idx / ncl, cl = idx - i * ncl;
        const int lx = i % Tx, r = i / Tx;
        const int gx = ox + lx, gy = oy + r % Ty, gz = oz + r / Ty;
        if (gx >= P.G || gy >= P.G || gz >= Gz) continue;
        const int2 a = lds_i32x2(acc + ((unsigned)i << 7) + ((unsigned)cl << 3));
        const float sg = P.checkerboard && ((gx + gy + gz) & 1) ? -inv : inv;
        put_cells(&grid[(size_t)(cg * CG + cl) * cells + ((size_t)gz * G + (size_t)gy) * G + (size_t)gx],
                  make_float2((float)a.x * sg, (float)a.y * sg), P.accumulate);
    }
}

template <typename IT>
__global__ void __launch_bounds__(kLaneWarps * 32, 2) grid_lanes_kernel(GridParams P)
{
    extern __shared__ float4 smem_raw[];
    float4 *smem4 = aligned_smem(smem_raw);
    const WorkItem it = P.items[blockIdx.x];
    const int cg = blockIdx.y;
    const int K = P.K;
    const int CG = P.coil_group;
    const LaneSmem L_ = lane_smem_layout(K, P.L);
    const unsigned acc = smem_addr(smem4);

    const int t = it.tile;
    const int ox = (t % P.ntile[0]) * P.tile[0];
    const int oy = ((t / P.ntile[0]) % P.ntile[1]) * P.tile[1];
    const int oz = (t / (P.ntile[0] * P.ntile[1])) * P.tile[2];
    if (it.count == 0) {
        if (!P.skip_empty) write_cell_group<32>(P, P.grid, acc, cg, ox, oy, oz, true, nullptr);
        return;
    }
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    float *lutw_s = reinterpret_cast<float *>(reinterpret_cast<unsigned char *>(smem4) + L_.lutw);
    // the tile starts at zero, and so do the value slots of a partial coil
    // group (a slot's coils past the group's last are never copied)
    for (int i = threadIdx.x; i < K * 8; i += blockDim.x) smem4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (min(CG, P.channels - cg * CG) < 16) {  // copies of fewer than 128 bytes (a partial group)
        float4 *stage_all = reinterpret_cast<float4 *>(reinterpret_cast<unsigned char *>(smem4) + L_.stage);
        for (int i = threadIdx.x; i < kLaneWarps * kLaneBatch * 8; i += blockDim.x)
            stage_all[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    for (int i = threadIdx.x; i < P.L; i += blockDim.x) lutw_s[i] = P.lutw[i];
    const float inv = P.item_inv[blockIdx.x];
    const float sc = __fdiv_rn(1.f, inv);  // exact: a power of two
    const unsigned mbar = acc + L_.mbar + 8u * (unsigned)warp;
    if (lane == 0) mbar_init(mbar);
    __syncthreads();

    const unsigned stage = acc + L_.stage + (unsigned)(warp * kLaneBatch * 128);
    int4 *table4 = reinterpret_cast<int4 *>(reinterpret_cast<unsigned char *>(smem4) + L_.table) + warp * kLaneBatch;
    const int ncl = min(CG, P.channels - cg * CG);
    // bytes of a record's coil values: whole coil pairs (an odd count's pad
    // coil is zero in the sample-major copy)
    const unsigned vbytes = 16u * (unsigned)((ncl + 1) >> 1);
    unsigned parity = 0u;
    const float *kt = P.kdata + 2 * (size_t)cg * CG;
    const unsigned *taps = P.taps;
    const IT tw = (IT)P.tap_words;
    const IT vstride = (IT)(2 * P.kstride);
    const unsigned cmask = (1u << kTapCellBits) - 1u;
    const unsigned lane4 = (unsigned)lane << 2;

    const int nrec = warp < it.count ? (it.count - warp + kLaneWarps - 1) / kLaneWarps : 0;
    const unsigned long long *trecs = P.trecs + it.begin + warp;
    // global loads run one step ahead of their use: the record words after
    // the window while it runs, the tap words of the next pass during the
    // current pass's adds, the first pass's tap words while the window's
    // bulk copies are in flight
    auto load_rw = [&](int k0) -> unsigned long long {
        const int k = k0 + lane;
        return k < nrec ? __ldg(trecs + (size_t)kLaneWarps * k) : 0ull;
    };
    // Records go through a window of 32, one per lane.  A window processes
    // only whole passes of 32 tap groups (the warp's last window: all its
    // groups); the records it finished leave, the rest (the first possibly
    // part-done: its first tap word and tap count advanced past the done
    // groups) move to the front and the window fills up from the next records.
    unsigned long long rw = load_rw(0), rw_next = load_rw(kLaneBatch);
    for (int wbase = 0; wbase < nrec;) {
        // this lane's record of the window: its tap groups (kLaneTaps taps
        // each, the last possibly short), their first number
        const int nt = (int)((rw >> 40) & 0xFF);
        const int np = (nt + kLaneTaps - 1) / kLaneTaps;
        const unsigned nz = __ballot_sync(0xffffffffu, np > 0);
        int incl = np;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        const int excl = incl - np;
        const int all = __shfl_sync(0xffffffffu, incl, 31);
        // groups this window processes, records it finishes (a prefix: incl
        // grows with the lane) and records it stages (those with groups below
        // `total`, also a prefix of the records with taps)
        const int total = wbase + kLaneBatch >= nrec ? all : min(all, 32 * max(all >> 5, 1));
        const int consumed = __popc(__ballot_sync(0xffffffffu, incl <= total));
        const unsigned staged = __ballot_sync(0xffffffffu, np > 0 && excl < total);
        const int nnz = __popc(staged);
        {
            // the next window: records consumed + lane of (this window, the next 32)
            const int src = consumed + lane;
            const unsigned long long a = __shfl_sync(0xffffffffu, rw, src & 31);
            const unsigned long long b = __shfl_sync(0xffffffffu, rw_next, src & 31);
            const int done = total - __shfl_sync(0xffffffffu, excl, consumed & 31);
            unsigned long long nrw = src < kLaneBatch ? a : b;
            if (lane == 0 && consumed < kLaneBatch && done > 0) {  // kLaneTaps done taps per done group
                const unsigned long long dt = (unsigned long long)(kLaneTaps * done);
                nrw = nrw + (dt << 32) - (dt << 40);
            }
            const unsigned long long nnext = load_rw(wbase + consumed + kLaneBatch);
            // the staged records' coil values (dcf * k) into the slots by bulk
            // copies, slot c for the c-th: lane 0 arms the mbarrier with the
            // window's bytes before any copy is issued
            if (nnz > 0) {
                if (lane == 0) mbar_expect_tx(mbar, (unsigned)nnz * vbytes);
                __syncwarp();
                if ((staged >> lane) & 1u) {
                    const int c = __popc(staged & ((1u << lane) - 1u));
                    table4[c] =
                        make_int4((int)(unsigned)rw, (int)(((rw >> 32) & 0xFF) | ((unsigned)nt << 8)), excl, 0);
                    bulk_copy_g2s(stage + ((unsigned)c << 7), kt + (IT)(unsigned)rw * vstride, vbytes, mbar);
                }
            }
            rw = nrw;
            rw_next = nnext;
        }
        wbase += consumed;
        __syncwarp();
        // pass setup: the lane's group number p0 + lane, its record (compact
        // index cr), the taps left in the group (nl) and their tap words
        int recbase = 0;
        auto pass_setup = [&](int p0, int &cr, int &nl, unsigned *tg) {
            // bit i of starts: a record's first group is group p0 + i
            const bool in_pass = np > 0 && excl >= p0 && excl < p0 + 32;
            const unsigned starts = __reduce_or_sync(0xffffffffu, in_pass ? 1u << (excl - p0) : 0u);
            cr = recbase + __popc(starts & (0xffffffffu >> (31 - lane))) - 1;
            recbase += __popc(starts);
            nl = 0;
#pragma unroll
            for (int k = 0; k < kLaneTaps; ++k) tg[k] = 0u;
            if (p0 + lane < total) {
                const int4 e = table4[cr];
                const int gi = kLaneTaps * (p0 + lane - e.z);
                nl = min((e.y >> 8) - gi, kLaneTaps);
                const IT tb = (IT)(unsigned)e.x * tw + (IT)(e.y & 0xFF) + (IT)gi;
                if ((tb & (IT)3) == 0) {
                    // a run the plan placed on a 4-word boundary (slots are
                    // multiples of 4 words, so the group stays in the slot)
                    const uint4 q = __ldg(reinterpret_cast<const uint4 *>(taps + tb));
                    tg[0] = q.x;
                    tg[1] = q.y;
                    tg[2] = q.z;
                    tg[3] = q.w;
                } else {
#pragma unroll
                    for (int k = 0; k < kLaneTaps; ++k)
                        if (k < nl) tg[k] = __ldg(taps + tb + k);
                }
            }
        };
        int cr_n, nl_n;
        unsigned t_n[kLaneTaps];
        pass_setup(0, cr_n, nl_n, t_n);  // the first pass's tap words load during the copies
        if (nnz > 0) {
            if (!mbar_wait(mbar, parity)) {
                // a copy that never lands: report it and wait once more for
                // the copies in flight before the slots are read
                if (lane == 0 && P.err) atomicExch(P.err, FR_ERR_DEVICE_TIMEOUT);
                mbar_wait(mbar, parity);
            }
            parity ^= 1u;
        }
        for (int p0 = 0; p0 < total; p0 += 32) {
            const int cr = cr_n, nl = nl_n;
            unsigned t[kLaneTaps];
#pragma unroll
            for (int k = 0; k < kLaneTaps; ++k) t[k] = t_n[k];
            if (p0 + 32 < total) pass_setup(p0 + 32, cr_n, nl_n, t_n);
            if (p0 + lane < total) {
                // each tap's cell row (this lane's float offset folded in)
                // and weight, the item's power-of-two scale on the weight
                // (exact: the same products w * v * S as scaling the values)
                unsigned a[kLaneTaps];
                float w[kLaneTaps];
#pragma unroll
                for (int k = 0; k < kLaneTaps; ++k) {
                    a[k] = (acc + (min(t[k] & cmask, (unsigned)(K - 1)) << 7)) | lane4;
                    w[k] = k < nl ? __fmul_rn(lutw_s[min(t[k] >> kTapCellBits, (unsigned)(P.L - 1))], sc) : 0.f;
                }
                const unsigned va = (stage + ((unsigned)cr << 7)) | lane4;
                float v[32];
#pragma unroll
                for (int f = 0; f < 32; ++f) v[f] = lds_f32_v(va ^ ((unsigned)f << 2));
#pragma unroll
                for (int k = 0; k < kLaneTaps; ++k) {
                    if (k < nl) {
#pragma unroll
                        for (int f = 0; f < 32; ++f) red_add_fx(a[k] ^ ((unsigned)f << 2), w[k], v[f]);
                    }
                }
            }
        }
        __syncwarp();  // the next window rewrites the table and the slots
    }
    __syncthreads();
    if (it.slot < 0) {
        lanes_flush(P, acc, cg, ox, oy, oz, inv);
    } else {
        // partial tile in the [cell][32] layout the reduction reads (float g
        // of cell c at g ^ ((c & 15) << 1)): float4 q of a row is plain quad
        // q ^ ((c & 15) >> 1), pairs swapped for odd cells
        float4 *dst = reinterpret_cast<float4 *>(P.partials + ((size_t)it.slot * P.ngroups + cg) * (size_t)K * 32);
        for (int i4 = threadIdx.x; i4 < K * 8; i4 += blockDim.x) {
            const int c = i4 >> 3, q = i4 & 7;
            int4 a = lds_s32x4(acc + ((unsigned)c << 7) + ((unsigned)(q ^ ((c & 15) >> 1)) << 4));
            if (c & 1) a = make_int4(a.z, a.w, a.x, a.y);
            dst[i4] = make_float4((float)a.x * inv, (float)a.y * inv, (float)a.z * inv, (float)a.w * inv);
        }
    }
}

// Per work item, from the per-sample bounds (mag[s] >= every |dcf * k| of
// sample s), one warp per item: the sum and the maximum over the item's
// records with taps.  The sum is exact and independent of the records'
// order: each bound is rounded up to a multiple of 2^-e (2^e bmax = 2^40..41)
// and the multiples are added as 64-bit integers; the float result is
// rounded up.
__global__ void item_bound_kernel(const WorkItem *__restrict__ items, long long nitems,
                                  const unsigned long long *__restrict__ trecs, const float *__restrict__ mag,
                                  float2 *__restrict__ bound)
{
    const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= nitems) return;
    const WorkItem it = items[w];
    float bm = 0.f;
    for (int j = lane; j < it.count; j += 32) {
        const unsigned long long rw = trecs[it.begin + j];
        if ((rw >> 40) & 0xFF) bm = fmaxf(bm, mag[(unsigned)rw]);
    }
    bm = __uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(bm)));  // bounds are >= 0
    float bs = 0.f;
    if (bm > 0.f) {
        const int e = 40 - ilogbf(bm);
        unsigned long long q = 0;
        for (int j = lane; j < it.count; j += 32) {
            const unsigned long long rw = trecs[it.begin + j];
            if ((rw >> 40) & 0xFF) q += __float2ull_ru(ldexpf(mag[(unsigned)rw], e));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) q += __shfl_xor_sync(0xffffffffu, q, o);
        bs = ldexpf(__ull2float_ru(q), -e);
    }
    if (lane == 0) bound[w] = make_float2(bs, bm);
}

// Inverse fixed-point scale of every work item from its own bound (see
// inv_scale_of).
__global__ void item_inv_kernel(const float2 *__restrict__ bound, long long nitems, float lut_absmax,
                                float *__restrict__ inv)
{
    for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < nitems;
         w += (long long)gridDim.x * blockDim.x) {
        const float2 b = bound[w];
        inv[w] = inv_scale_of(b.x, __float_as_uint(b.y), lut_absmax);
    }
}

// Sum the partial tiles of each split tile in item order and write the grid.
// CTA (split tile, coil group, part): part z of kReduceParts holds a run of
// the tile's rows.  The partial rows are read as contiguous float4 ([cell][R]
// swizzled, as the scatter wrote them), summed slot after slot (the float
// order of a plain loop over the items), staged in shared memory, and written
// as x pairs of one coil per thread, each pair's offset computed once.
constexpr int kReduceParts = 4, kReduceThreads = 256;

template <int R>
__global__ void __launch_bounds__(kReduceThreads) reduce_splits_kernel(GridParams P)
{
    extern __shared__ float4 red_raw[];
    float *sum = reinterpret_cast<float *>(red_raw);
    const SplitTile st = P.splits[blockIdx.x];
    const int cg = blockIdx.y;
    const int t = st.tile;
    const int Tx = P.tile[0], Ty = P.tile[1];
    const int rows = Ty * P.tile[2];
    const int nparts = gridDim.z;
    const int r0 = rows * (int)blockIdx.z / nparts, r1 = rows * ((int)blockIdx.z + 1) / nparts;
    const int c0 = r0 * Tx, ncell = (r1 - r0) * Tx;
    const int K = P.K, CG = P.coil_group;
    const int ox = (t % P.ntile[0]) * Tx;
    const int oy = ((t / P.ntile[0]) % P.ntile[1]) * Ty;
    const int oz = (t / (P.ntile[0] * P.ntile[1])) * P.tile[2];
    const size_t stride4 = (size_t)P.ngroups * K * R / 4;
    const float4 *src = reinterpret_cast<const float4 *>(P.partials) +
                        ((size_t)st.first_slot * P.ngroups + cg) * (size_t)K * R / 4 + (size_t)c0 * R / 4;
    const int n4 = ncell * R / 4;
    for (int i = threadIdx.x; i < n4; i += kReduceThreads) {
        float4 v = src[i];
        int k = 1;
        for (; k + 4 <= st.nslots; k += 4) {
            const float4 a0 = src[(size_t)k * stride4 + i], a1 = src[(size_t)(k + 1) * stride4 + i];
            const float4 a2 = src[(size_t)(k + 2) * stride4 + i], a3 = src[(size_t)(k + 3) * stride4 + i];
            v = make_float4(__fadd_rn(v.x, a0.x), __fadd_rn(v.y, a0.y), __fadd_rn(v.z, a0.z), __fadd_rn(v.w, a0.w));
            v = make_float4(__fadd_rn(v.x, a1.x), __fadd_rn(v.y, a1.y), __fadd_rn(v.z, a1.z), __fadd_rn(v.w, a1.w));
            v = make_float4(__fadd_rn(v.x, a2.x), __fadd_rn(v.y, a2.y), __fadd_rn(v.z, a2.z), __fadd_rn(v.w, a2.w));
            v = make_float4(__fadd_rn(v.x, a3.x), __fadd_rn(v.y, a3.y), __fadd_rn(v.z, a3.z), __fadd_rn(v.w, a3.w));
        }
        for (; k < st.nslots; ++k) {
            const float4 a = src[(size_t)k * stride4 + i];
            v = make_float4(__fadd_rn(v.x, a.x), __fadd_rn(v.y, a.y), __fadd_rn(v.z, a.z), __fadd_rn(v.w, a.w));
        }
        red_raw[i] = v;
    }
    __syncthreads();
    const size_t G = (size_t)P.G;
    const int Gz = P.dim == 3 ? P.G : 1;
    const size_t cells = P.dim == 3 ? G * G * G : G * G;
    const int ncl = min(CG, P.channels - cg * CG);
    float *gridf = P.grid + (P.frame_off ? (size_t)st.pad * (size_t)P.grid_frame_floats : 0);
    const int npair = ncell / 2;
    if ((Tx % 2) == 0 && (P.G % 2) == 0 && kReduceThreads % npair == 0 &&
        (reinterpret_cast<uintptr_t>(gridf) & 15) == 0) {
        const int slot = threadIdx.x % npair, cstep = kReduceThreads / npair;
        const int lx = 2 * (slot % (Tx / 2)), r = r0 + slot / (Tx / 2);
        const int gx = ox + lx, gy = oy + r % Ty, gz = oz + r / Ty;
        if (gx >= P.G || gy >= P.G || gz >= Gz) return;  // gx even, G even: gx + 1 < G as well
        float4 *gridc = reinterpret_cast<float4 *>(gridf) + ((((size_t)gz * G + (size_t)gy) * G + (size_t)gx) >> 1);
        const int i = r * Tx + lx, il = i - c0;
        const int swa = swz<R>(i), swb = swz<R>(i + 1);
        const float sa = P.checkerboard && ((gx + gy + gz) & 1) ? -1.f : 1.f;
        const float sb = P.checkerboard ? -sa : 1.f;
        for (int cl = threadIdx.x / npair; cl < ncl; cl += cstep) {
            const float2 a = *reinterpret_cast<const float2 *>(sum + il * R + ((2 * cl) ^ swa));
            const float2 b = *reinterpret_cast<const float2 *>(sum + (il + 1) * R + ((2 * cl) ^ swb));
            put_cells(&gridc[(size_t)(cg * CG + cl) * (cells >> 1)], make_float4(a.x * sa, a.y * sa, b.x * sb, b.y * sb),
                      P.accumulate);
        }
        return;
    }
    float2 *grid = reinterpret_cast<float2 *>(gridf);
    for (int idx = threadIdx.x; idx < ncl * ncell; idx += kReduceThreads) {
        const int cl = idx / ncell, il = idx - cl * ncell, i = c0 + il;
        const int lx = i % Tx, r = i / Tx;
        const int gx = ox + lx, gy = oy + r % Ty, gz = oz + r / Ty;
        if (gx >= P.G || gy >= P.G || gz >= Gz) continue;
        float2 v = *reinterpret_cast<const float2 *>(sum + il * R + ((2 * cl) ^ swz<R>(i)));
        if (P.checkerboard && ((gx + gy + gz) & 1)) {
            v.x = -v.x;
            v.y = -v.y;
        }
        put_cells(&grid[(size_t)(cg * CG + cl) * cells + ((size_t)gz * G + (size_t)gy) * G + (size_t)gx], v,
                  P.accumulate);
    }
}

// The reduction of the split tiles (none: nothing to launch).
template <int R>
int launch_reduce(const GridParams &P, long long nsplits, cudaStream_t s)
{
    if (nsplits <= 0) return FR_OK;
    const int rows = P.tile[1] * P.tile[2];
    const int parts = rows % kReduceParts == 0 ? kReduceParts : 1;
    const size_t smem = (size_t)(rows / parts) * P.tile[0] * R * sizeof(float);
    if (smem > 48 * 1024)
        FR_CUDA(cudaFuncSetAttribute(reduce_splits_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 g2((unsigned)nsplits, (unsigned)P.ngroups, (unsigned)parts);
    reduce_splits_kernel<R><<<g2, kReduceThreads, smem, s>>>(P);
    FR_CHECK_LAUNCH("reduce_splits_kernel");
    return FR_OK;
}

// [channels][n] complex -> [n][channels] complex, kTrSamples samples per CTA
// through shared memory (coalesced reads along n, writes along channels).
// Each thread issues kTrPer loads before it stores any of them (the copy is
// bound by the latency of these reads).
constexpr int kTrSamples = 128;
constexpr int kTrThreads = 256, kTrPer = 8;
// The copy holds dcf * k (the product GridLut.cpp:109 forms, same rounding)
// and mag[s] = the largest |re| or |im| of sample s's products.
__global__ void __launch_bounds__(kTrThreads) transpose_kspace_kernel(const float2 *__restrict__ in,
                                                                      const float *__restrict__ dcf,
                                                                      float2 *__restrict__ out,
                                                                      float *__restrict__ mag, long long n,
                                                                      int channels, int cstride, long long in_stride)
{
    extern __shared__ float2 tr[];  // [channels][kTrSamples + 1]
    __shared__ float dsh[kTrSamples];
    const long long s0 = (long long)blockIdx.x * kTrSamples;
    const int ns = (int)min((long long)kTrSamples, n - s0);
    for (int j = threadIdx.x; j < ns; j += kTrThreads) dsh[j] = dcf[s0 + j];
    const int total = channels * kTrSamples;
    for (int i0 = 0; i0 < total; i0 += kTrThreads * kTrPer) {
        float2 v[kTrPer];
#pragma unroll
        for (int k = 0; k < kTrPer; ++k) {
            const int i = i0 + k * kTrThreads + threadIdx.x;
            const int c = i / kTrSamples, j = i % kTrSamples;
            v[k] = i < total && j < ns ? in[(size_t)c * in_stride + s0 + j] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int k = 0; k < kTrPer; ++k) {
            const int i = i0 + k * kTrThreads + threadIdx.x;
            if (i < total) tr[(i / kTrSamples) * (kTrSamples + 1) + i % kTrSamples] = v[k];
        }
    }
    __syncthreads();
    // rows of cstride >= channels complex values (the pad, if any, is zero)
    for (int i = threadIdx.x; i < cstride * ns; i += kTrThreads) {
        const int j = i / cstride, c = i - j * cstride;
        float2 o = make_float2(0.f, 0.f);
        if (c < channels) {
            const float2 v = tr[c * (kTrSamples + 1) + j];
            const float d = dsh[j];
            o = make_float2(__fmul_rn(d, v.x), __fmul_rn(d, v.y));
        }
        out[(size_t)(s0 + j) * cstride + c] = o;
    }
    for (int j = threadIdx.x; j < ns; j += kTrThreads) {
        const float d = dsh[j];
        float m = 0.f;
        for (int c = 0; c < channels; ++c) {
            const float2 v = tr[c * (kTrSamples + 1) + j];
            m = fmaxf(m, fmaxf(fabsf(__fmul_rn(d, v.x)), fabsf(__fmul_rn(d, v.y))));
        }
        mag[s0 + j] = m;
    }
}

template <int DIM, int R>
int launch(fr_plan p, const GridParams &P, long long nitems, long long nsplits, cudaStream_t s)
{
    size_t smem = grid_smem_bytes(P.K, R, P.L);
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
    return launch_reduce<R>(P, nsplits, s);
}

template <int R>
int launch_taps(fr_plan p, const GridParams &P, long long nitems, long long nsplits, cudaStream_t s)
{
    // per-item scales first (every launched item, so the indices match
    // blockIdx.x); the bounds go to the scratch past the scales
    {
        const int threads = 256;
        const long long blocks = (nitems * 32 + threads - 1) / threads;
        const long long boff = (nitems + 1) & ~1ll;  // 8-byte aligned float2
        float2 *bound = reinterpret_cast<float2 *>(const_cast<float *>(P.item_inv) + boff);
        item_bound_kernel<<<(unsigned)blocks, threads, 0, s>>>(P.items, nitems, P.trecs, P.mag, bound);
        FR_CHECK_LAUNCH("item_bound_kernel");
        item_inv_kernel<<<(unsigned)std::min<long long>((nitems + threads - 1) / threads, 152 * 8), threads, 0, s>>>(
            bound, nitems, P.lut_absmax, const_cast<float *>(P.item_inv));
        FR_CHECK_LAUNCH("item_inv_kernel");
    }
    // 32-bit indices when the tap words and sample-major values allow them
    const bool idx32 = (double)P.n * (double)P.tap_words < 2147483647.0 &&
                       (double)P.n * (double)(2 * P.kstride) < 2147483647.0;
    // rows of 32 coil floats: the tap-lane scatter, unless a plan asks for
    // the per-warp tap lists
    const LaneSmem lm = lane_smem_layout(P.K, P.L);
    const bool lanes = R == 32 && !p->scatter_warp_lists && lm.end + 128 <= 227 * 1024 && (P.kstride % 2) == 0;
    const TapSmem m = tap_smem_layout(P.K, R, P.L);
    const size_t smem = lanes ? lm.end + 128 : m.end + 128;
    if (smem > 227 * 1024) return fail(FR_ERR_UNSUPPORTED, "tap-list scatter does not fit in shared memory");
    auto kern = lanes ? (idx32 ? grid_lanes_kernel<unsigned> : grid_lanes_kernel<unsigned long long>)
                      : (idx32 ? grid_taps_kernel<R, unsigned> : grid_taps_kernel<R, unsigned long long>);
    const int threads = lanes ? kLaneWarps * 32 : kWarps * 32;
    if (smem > 48 * 1024) FR_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
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
    FR_CHECK_LAUNCH(lanes ? "grid_lanes_kernel" : "grid_taps_kernel");
    if (ev) FR_CUDA(cudaEventRecord(ev[1], s));
    return launch_reduce<R>(P, nsplits, s);
}

}  // namespace

size_t grid_smem_bytes(long long K, int R, int L)
{
    // accumulator tile + LUT + double-buffered per-warp tap lists + tap decode
    // table + scale words + alignment of the tile to 128 bytes
    return (size_t)K * R * 4 + (size_t)L * 16 + (size_t)kWarps * 2 * kListEntries * 8 + kDecBytes + 3 * 64 * 4 + 128;
}

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

int kspace_prepare(fr_plan p, const float *d_kdata, const float *d_dcf, int channels, cudaStream_t s,
                   size_t kin_stride)
{
    p->kt_prepared = nullptr;
    if (p->n == 0) return FR_OK;
    const size_t trsmem = (size_t)channels * (kTrSamples + 1) * sizeof(float2);
    if (trsmem > 96 * 1024) return fail(FR_ERR_UNSUPPORTED, "too many channels for the sample-major copy");
    const int cstride = channels + (channels & 1);  // even: rows start on 16-byte boundaries
    if (p->kt.reserve(p->n * (size_t)cstride * sizeof(float2)) || p->kmag.reserve(p->n * sizeof(float)))
        return FR_ERR_OUT_OF_MEMORY;
    if (trsmem > 48 * 1024)
        FR_CUDA(cudaFuncSetAttribute(transpose_kspace_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)trsmem));
    transpose_kspace_kernel<<<(unsigned)((p->n + kTrSamples - 1) / kTrSamples), kTrThreads, trsmem, s>>>(
        reinterpret_cast<const float2 *>(d_kdata), d_dcf, p->kt.as<float2>(), p->kmag.as<float>(), (long long)p->n,
        channels, cstride, (long long)(kin_stride ? kin_stride : p->n));
    FR_CHECK_LAUNCH("transpose_kspace_kernel");
    p->kt_prepared = d_kdata;
    p->kt_prepared_channels = channels;
    return FR_OK;
}

int grid_run(fr_plan p, const float *d_kdata, const float *d_dcf, int channels, float *d_grid,
             cudaStream_t s, bool skip_empty, size_t kin_stride)
{
    if (kin_stride && kin_stride < p->n) return fail(FR_ERR_INVALID_ARGUMENT, "coil stride below the samples");
    const bool accumulate = (p->flags & FR_PLAN_ACCUMULATE) != 0;
    skip_empty = skip_empty || accumulate;  // adding zeros is a no-op
    if (!p->planned) return fail(FR_ERR_NOT_PLANNED, "fr_grid called before fr_plan_set_trajectory");
    if (channels <= 0) return fail(FR_ERR_INVALID_ARGUMENT, "channels must be positive");
    const int R = floats_per_cell(p->coil_group);
    GridParams P;
    P.traj = p->traj.as<float4>();
    P.recs = p->pairs.as<unsigned long long>();
    P.items = p->items.as<WorkItem>();
    P.splits = p->splits.as<SplitTile>();
    P.kdata = d_kdata;
    P.dcf = d_dcf;
    P.lut_e = p->lut_e.as<float4>();
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
    P.smax = p->lut_smax;
    P.kc = p->lut_kc;
    P.lut_absmax = p->lut_absmax;
    P.khalf = 0.25f;  // 0.5 - slack 0.25: the guess is the exact index or one below
    P.checkerboard = (p->flags & FR_PLAN_CHECKERBOARD) ? 1 : 0;
    P.frame_off = nullptr;
    P.grid_frame_floats = 0;
    P.work_counter = nullptr;
    P.nwork = 0;
    P.sample_major = 0;
    P.skip_empty = skip_empty ? 1 : 0;
    P.accumulate = accumulate ? 1 : 0;
    P.kin_stride = (long long)(kin_stride ? kin_stride : p->n);
    const size_t trsmem = (size_t)channels * (kTrSamples + 1) * sizeof(float2);
    P.mag = nullptr;
    P.kstride = channels;
    if (p->err_host && *p->err_host) {  // a kernel of an earlier call found an internal error
        const int e = *p->err_host;
        *p->err_host = 0;
        return fail(e, e == FR_ERR_DEVICE_TIMEOUT ? "a bulk copy of the scatter never completed (an earlier call)"
                                                  : "the plan's tap lists overflowed a sample slot (internal error)");
    }
    P.err = p->err_dev;
    // the tap-list scatter reads each record's coil values from the
    // sample-major copy; the geometry scatter uses the copy from 4 coils on
    const bool taps = p->tap_words > 0 && R <= 32;
    if (p->kspace_sample_major && (channels >= 4 || taps) && p->n > 0 && trsmem <= 96 * 1024) {
        const int cstride = channels + (channels & 1);  // even: rows start on 16-byte boundaries
        const bool ready = p->kt_prepared == d_kdata && p->kt_prepared_channels == channels;
        p->kt_prepared = nullptr;
        if (!ready) {
            const int st = kspace_prepare(p, d_kdata, d_dcf, channels, s, kin_stride);
            p->kt_prepared = nullptr;
            if (st) return st;
        }
        P.kdata = p->kt.as<float>();
        P.sample_major = 1;
        P.mag = p->kmag.as<float>();
        P.kstride = cstride;
    }
    if (p->nslots > 0) {
        size_t bytes = (size_t)p->nslots * P.ngroups * (size_t)P.K * R * 4;
        if (p->partials.reserve(bytes)) return FR_ERR_OUT_OF_MEMORY;
    }
    P.partials = p->partials.as<float>();
    // with skip_empty only the occupied tiles' items (the empty tiles'
    // zero-fill items are last in the list)
    const long long nlaunch = skip_empty ? p->nitems_occupied : p->nitems;
    if (nlaunch == 0) return FR_OK;
    if (taps && P.sample_major) {
        P.trecs = p->trecs.as<unsigned long long>();
        P.taps = p->taps.as<unsigned>();
        P.lutw = p->lut_d.as<float>();
        P.tap_words = p->tap_words;
        // nlaunch item scales, then (from an even word) nlaunch float2 bounds
        const size_t words = (((size_t)nlaunch + 1) & ~(size_t)1) + 2 * (size_t)nlaunch;
        if (p->item_inv.reserve(words * 4)) return FR_ERR_OUT_OF_MEMORY;
        P.item_inv = p->item_inv.as<float>();
        switch (R) {
        case 8: return launch_taps<8>(p, P, nlaunch, p->nsplits, s);
        case 16: return launch_taps<16>(p, P, nlaunch, p->nsplits, s);
        case 32: return launch_taps<32>(p, P, nlaunch, p->nsplits, s);
        }
    }
    if (p->dim == 3) {
        switch (R) {
        case 8: return launch<3, 8>(p, P, nlaunch, p->nsplits, s);
        case 16: return launch<3, 16>(p, P, nlaunch, p->nsplits, s);
        case 32: return launch<3, 32>(p, P, nlaunch, p->nsplits, s);
        case 64: return launch<3, 64>(p, P, nlaunch, p->nsplits, s);
        }
    } else {
        switch (R) {
        case 8: return launch<2, 8>(p, P, nlaunch, p->nsplits, s);
        case 16: return launch<2, 16>(p, P, nlaunch, p->nsplits, s);
        case 32: return launch<2, 32>(p, P, nlaunch, p->nsplits, s);
        case 64: return launch<2, 64>(p, P, nlaunch, p->nsplits, s);
        }
    }
    return fail(FR_ERR_UNSUPPORTED, "coil group must be 4, 8, 16 or 32");
}

// --------------------------------------------------------------------------
// The same scatter from a plan held in caller-provided memory
// (fr_grid_noalloc): identical kernels and launch shapes, no allocation.
// --------------------------------------------------------------------------
namespace {
template <int DIM, int R>
int launch_into(const GridParams &P, long long nitems, long long nsplits, cudaStream_t s)
{
    size_t smem = grid_smem_bytes(P.K, R, P.L);
    auto kern = grid_tiles_kernel<DIM, R>;
    if (smem > 48 * 1024) FR_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid((unsigned)nitems, (unsigned)P.ngroups);
    kern<<<grid, kWarps * 32, smem, s>>>(P);
    FR_CHECK_LAUNCH("grid_tiles_kernel");
    return launch_reduce<R>(P, nsplits, s);
}
}  // namespace

size_t grid_partials_bytes(long long nslots, int channels, int coil_group, long long K)
{
    const long long ngroups = (channels + coil_group - 1) / coil_group;
    return (size_t)nslots * ngroups * K * floats_per_cell(coil_group) * 4;
}

int grid_into(const GridInto &gi, const float *d_kdata, const float *d_dcf, int channels, float *d_grid,
              cudaStream_t s)
{
    const int R = floats_per_cell(gi.coil_group);
    GridParams P;
    P.traj = gi.traj;
    P.recs = gi.recs;
    P.items = gi.items;
    P.splits = gi.splits;
    P.kdata = d_kdata;
    P.dcf = d_dcf;
    P.lut_e = gi.lut_e;
    P.grid = d_grid;
    P.partials = gi.partials;
    P.n = (long long)gi.n;
    P.channels = channels;
    P.coil_group = gi.coil_group;
    P.ngroups = (channels + gi.coil_group - 1) / gi.coil_group;
    P.dim = gi.dim;
    P.G = (int)gi.G;
    P.K = 1;
    for (int d = 0; d < 3; ++d) {
        P.tile[d] = gi.tile[d];
        P.ntile[d] = gi.ntile[d];
        P.K *= gi.tile[d];
    }
    P.L = gi.L;
    P.smax = gi.smax;
    P.kc = gi.kc;
    P.lut_absmax = gi.lut_absmax;
    P.khalf = 0.25f;
    P.checkerboard = 0;
    P.frame_off = nullptr;
    P.grid_frame_floats = 0;
    P.work_counter = nullptr;
    P.nwork = 0;
    P.sample_major = 0;
    P.mag = nullptr;
    P.skip_empty = 0;
    P.kin_stride = (long long)gi.n;
    if (gi.nitems == 0) return FR_OK;
    if (gi.dim == 3) {
        switch (R) {
        case 8: return launch_into<3, 8>(P, gi.nitems, gi.nsplits, s);
        case 16: return launch_into<3, 16>(P, gi.nitems, gi.nsplits, s);
        case 32: return launch_into<3, 32>(P, gi.nitems, gi.nsplits, s);
        case 64: return launch_into<3, 64>(P, gi.nitems, gi.nsplits, s);
        }
    } else {
        switch (R) {
        case 8: return launch_into<2, 8>(P, gi.nitems, gi.nsplits, s);
        case 16: return launch_into<2, 16>(P, gi.nitems, gi.nsplits, s);
        case 32: return launch_into<2, 32>(P, gi.nitems, gi.nsplits, s);
        case 64: return launch_into<2, 64>(P, gi.nitems, gi.nsplits, s);
        }
    }
    return fail(FR_ERR_UNSUPPORTED, "coil group must be 4, 8, 16 or 32");
}

// --------------------------------------------------------------------------
// Batches of frames: one persistent launch over every frame's work items.
// --------------------------------------------------------------------------
namespace {
template <int DIM, int R>
int batch_setup_t(long long K, int L, int *blocks)
{
    const size_t smem = grid_smem_bytes(K, R, L);
    auto kern = grid_persistent_kernel<DIM, R>;
    if (smem > 48 * 1024) FR_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0, dev = 0, sms = 0;
    FR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kWarps * 32, smem));
    FR_CUDA(cudaGetDevice(&dev));
    FR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (per_sm < 1) return fail(FR_ERR_UNSUPPORTED, "persistent scatter does not fit on an SM");
    *blocks = per_sm * sms;
    return FR_OK;
}

template <int DIM, int R>
int batch_launch_t(const GridParams &P, int blocks, long long nsplits, cudaStream_t s)
{
    const size_t smem = grid_smem_bytes(P.K, R, P.L);
    FR_CUDA(cudaMemsetAsync(P.work_counter, 0, sizeof(int), s));
    const long long nb = std::min<long long>(blocks, P.nwork);
    grid_persistent_kernel<DIM, R><<<(unsigned)nb, kWarps * 32, smem, s>>>(P);
    FR_CHECK_LAUNCH("grid_persistent_kernel");
    return launch_reduce<R>(P, nsplits, s);
}
}  // namespace

int batch_grid_setup(int dim, long long K, int coil_group, int L, int *blocks)
{
    const int R = floats_per_cell(coil_group);
    if (grid_smem_bytes(K, R, L) > 227 * 1024) return fail(FR_ERR_UNSUPPORTED, "tile does not fit in shared memory");
#define FR_BATCH_SETUP(D)                                                   \
    switch (R) {                                                            \
    case 8: return batch_setup_t<D, 8>(K, L, blocks);                       \
    case 16: return batch_setup_t<D, 16>(K, L, blocks);                     \
    case 32: return batch_setup_t<D, 32>(K, L, blocks);                     \
    case 64: return batch_setup_t<D, 64>(K, L, blocks);                     \
    }
    if (dim == 3) {
        FR_BATCH_SETUP(3)
    } else {
        FR_BATCH_SETUP(2)
    }
#undef FR_BATCH_SETUP
    return fail(FR_ERR_UNSUPPORTED, "coil group must be 4, 8, 16 or 32");
}

int batch_grid_run(const BatchGrid &b, const float *d_kdata, const float *d_dcf, int channels, float *d_grid,
                   cudaStream_t s)
{
    const int R = floats_per_cell(b.coil_group);
    GridParams P;
    P.traj = b.traj;
    P.recs = b.recs;
    P.items = b.items;
    P.splits = b.splits;
    P.kdata = d_kdata;
    P.dcf = d_dcf;
    P.lut_e = b.lut_e;
    P.grid = d_grid;
    P.partials = b.partials;
    P.n = b.n_total;
    P.channels = channels;
    P.coil_group = b.coil_group;
    P.ngroups = (channels + b.coil_group - 1) / b.coil_group;
    P.dim = b.dim;
    P.G = (int)b.G;
    P.K = 1;
    for (int d = 0; d < 3; ++d) {
        P.tile[d] = b.tile[d];
        P.ntile[d] = b.ntile[d];
        P.K *= b.tile[d];
    }
    P.L = b.L;
    P.smax = b.smax;
    P.kc = b.kc;
    P.lut_absmax = b.lut_absmax;
    P.khalf = 0.25f;
    P.checkerboard = b.checkerboard;
    P.frame_off = b.frame_off;
    const size_t cells = b.dim == 3 ? (size_t)b.G * b.G * b.G : (size_t)b.G * b.G;
    P.grid_frame_floats = (long long)(2 * (size_t)channels * cells);
    P.work_counter = b.work_counter;
    P.nwork = b.nitems * P.ngroups;
    P.sample_major = 0;
    P.mag = nullptr;
    P.skip_empty = 0;
    if (P.nwork == 0) return FR_OK;
    if (P.nwork > 0x7FFFFFFFll) return fail(FR_ERR_UNSUPPORTED, "too many work items");
    if (b.dim == 3) {
        switch (R) {
        case 8: return batch_launch_t<3, 8>(P, b.blocks, b.nsplits, s);
        case 16: return batch_launch_t<3, 16>(P, b.blocks, b.nsplits, s);
        case 32: return batch_launch_t<3, 32>(P, b.blocks, b.nsplits, s);
        case 64: return batch_launch_t<3, 64>(P, b.blocks, b.nsplits, s);
        }
    } else {
        switch (R) {
        case 8: return batch_launch_t<2, 8>(P, b.blocks, b.nsplits, s);
        case 16: return batch_launch_t<2, 16>(P, b.blocks, b.nsplits, s);
        case 32: return batch_launch_t<2, 32>(P, b.blocks, b.nsplits, s);
        case 64: return batch_launch_t<2, 64>(P, b.blocks, b.nsplits, s);
        }
    }
    return fail(FR_ERR_UNSUPPORTED, "coil group must be 4, 8, 16 or 32");
}

}  // namespace fr
