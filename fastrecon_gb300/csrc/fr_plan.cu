// fr_plan.cu -- trajectory normalisation and tile binning (the plan).
//
// Replaces ReconData::normalizeTraj (ReconData.cpp:211-225) and
// cuGridLut::plan (cuGridLut.cu:151-226).  Instead of materialising one
// (cell, sample) pair per kernel tap and sorting them, each sample is binned
// into the grid tiles its clamped cell range touches (at most 2^d tiles when
// the tile edge is at least the kernel footprint), with an integer counting
// sort: count per tile, exclusive scan, fill.  The per-sample cell range is
// the reference's (GridLut.cpp:98-106), computed with the same float
// operations, so the set of touched tiles is bit-exact.
#include <cuda_runtime.h>
#include <float.h>
#include <limits.h>

#include <algorithm>
#include <cmath>

#include "fr_device.cuh"
#include "fr_internal.h"

namespace fr {
namespace {

constexpr int kBoundsSlots = 32;
// bounds buffer layout (32-bit words)
constexpr int kRawLoEnc = 0;   // 3 ordered-int encodings
constexpr int kRawHiEnc = 3;   // 3
constexpr int kTr = 6;         // float
constexpr int kScale = 7;      // float
constexpr int kNormLo = 8;     // 3 floats
constexpr int kNormHi = 11;    // 3 floats
constexpr int kRawLo = 14;     // 3 floats (decoded)
constexpr int kRawHi = 17;     // 3 floats

__device__ __forceinline__ int float_order(float f)
{
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float order_float(int i)
{
    return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF);
}

__global__ void bounds_init_kernel(int *b)
{
    int t = threadIdx.x;
    if (t < 3) {
        // ReconData.cpp:158-161: first = max(), second = lowest()
        b[kRawLoEnc + t] = float_order(FLT_MAX);
        b[kRawHiEnc + t] = float_order(-FLT_MAX);
    }
}

// Component bounds as ReconData::loadTraj accumulates them
// (ReconData.cpp:167-174): NaN never replaces a bound.
__global__ void bounds_kernel(const float4 *__restrict__ traj, size_t n, int dim, int *b)
{
    int lo[3] = {INT_MAX, INT_MAX, INT_MAX}, hi[3] = {INT_MIN, INT_MIN, INT_MIN};
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        float4 p = traj[i];
        float c[3] = {p.x, p.y, p.z};
        for (int d = 0; d < 3; ++d) {
            if (d < dim && !isnan(c[d])) {
                int o = float_order(c[d]);
                lo[d] = min(lo[d], o);
                hi[d] = max(hi[d], o);
            }
        }
    }
    for (int d = 0; d < 3; ++d) {
        for (int off = 16; off > 0; off >>= 1) {
            lo[d] = min(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], off));
            hi[d] = max(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], off));
        }
    }
    // one set of global atomics per block (few blocks: contention on the six
    // words stays low)
    __shared__ int wlo[32][3], whi[32][3];
    const int warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int d = 0; d < 3; ++d) {
            wlo[warp][d] = lo[d];
            whi[warp][d] = hi[d];
        }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < nw; ++w)
            for (int d = 0; d < 3; ++d) {
                lo[d] = min(lo[d], wlo[w][d]);
                hi[d] = max(hi[d], whi[w][d]);
            }
        for (int d = 0; d < dim; ++d) {
            if (lo[d] != INT_MAX) atomicMin(&b[kRawLoEnc + d], lo[d]);
            if (hi[d] != INT_MIN) atomicMax(&b[kRawHiEnc + d], hi[d]);
        }
    }
}

// ReconData::normalizeTraj (ReconData.cpp:211-225), one thread.
__global__ void scale_kernel(int *b, int dim, unsigned G)
{
    float *f = reinterpret_cast<float *>(b);
    float lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
        lo[d] = d < dim ? order_float(b[kRawLoEnc + d]) : 0.f;
        hi[d] = d < dim ? order_float(b[kRawHiEnc + d]) : 0.f;
        f[kRawLo + d] = lo[d];
        f[kRawHi + d] = hi[d];
    }
    float tr = -lo[0];
    float scale = __fdiv_rn((float)(G - 1u), __fsub_rn(hi[0], lo[0]));
    f[kTr] = tr;
    f[kScale] = scale;
    for (int d = 0; d < 3; ++d) {
        f[kNormLo + d] = d < dim ? __fmul_rn(__fadd_rn(lo[d], tr), scale) : 0.f;
        f[kNormHi + d] = d < dim ? __fmul_rn(__fadd_rn(hi[d], tr), scale) : 0.f;
    }
}

struct BinGeom {
    int dim;
    unsigned G;
    float hw;
    int prefilter;
    int tile[3];
    int ntile[3];
    int tshift[3];  // log2(tile[d]) for power-of-two tiles, else -1
};

// Cell index -> tile index along axis d (x >= 0).
__device__ __forceinline__ int tile_div(const BinGeom &g, int x, int d)
{
    return g.tshift[d] >= 0 ? x >> g.tshift[d] : x / g.tile[d];
}

// The tiles of one sample's cell range, visited in x, y, z order by an
// odometer (no divisions per step).
struct TileWalk {
    int lo[3], n[3];
    int jx = 0, jy = 0, jz = 0;
    __device__ __forceinline__ void next()
    {
        if (++jx == n[0]) {
            jx = 0;
            if (++jy == n[1]) {
                jy = 0;
                ++jz;
            }
        }
    }
    __device__ __forceinline__ int tile(const BinGeom &g) const
    {
        return ((lo[2] + jz) * g.ntile[1] + lo[1] + jy) * g.ntile[0] + lo[0] + jx;
    }
};

// Find the tiles a sample's clamped cell range touches (s/e: the range,
// GridLut.cpp:98-106).  Returns the number of tiles and sets up the walk.
__device__ __forceinline__ int sample_tiles(const BinGeom &g, const float4 &p, TileWalk &w, int *s, int *e)
{
    const float c[3] = {p.x, p.y, p.z};
    int cnt = 1;
    for (int d = 0; d < 3; ++d) {
        if (d < g.dim) {
            comp_range(c[d], g.hw, g.G, s[d], e[d]);
            if (s[d] > e[d]) cnt = 0;
        } else {
            s[d] = e[d] = 0;
        }
    }
    for (int d = 0; d < 3; ++d) {
        w.lo[d] = cnt ? tile_div(g, s[d], d) : 0;
        w.n[d] = cnt ? tile_div(g, e[d], d) - w.lo[d] + 1 : 1;
    }
    return cnt ? w.n[0] * w.n[1] * w.n[2] : 0;
}

// Runs of consecutive lanes with the same tile (consecutive samples of a
// readout usually share tiles): one counter update per run instead of one
// per sample.  run: the run's length (valid in its first lane); head_lane:
// the first lane of this lane's run.
__device__ __forceinline__ void lane_runs(int t, int lane, int &run, int &head_lane)
{
    const int tp = __shfl_up_sync(0xffffffffu, t, 1);
    const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || tp != t);
    const unsigned upto = lane == 31 ? 0xffffffffu : (2u << lane) - 1u;  // lanes 0..lane
    head_lane = 31 - __clz(heads & upto);
    const unsigned after = heads & ~upto;
    run = (after ? __ffs(after) - 1 : 32) - lane;
}

// Bin counters are striped: the samples of 32-sample group g count into
// stripe g mod kStripes of a tile, so the many warps whose spokes all cross
// the dense centre tiles spread their atomics over kStripes counters.  A
// tile's records stay contiguous (stripe-major within the tile).
constexpr int kStripes = 8;
__device__ __forceinline__ int stripe_of(size_t first_sample_of_warp)
{
    return (int)((first_sample_of_warp >> 5) & (kStripes - 1));
}

// Tile totals from the stripe counters.
__global__ void stripe_total_kernel(const int *__restrict__ stripe_count, long long ntiles, int *__restrict__ tile_count)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ntiles;
         t += (long long)gridDim.x * blockDim.x) {
        int c = 0;
#pragma unroll
        for (int k = 0; k < kStripes; ++k) c += stripe_count[t * kStripes + k];
        tile_count[t] = c;
    }
}

// First record of every (tile, stripe) from the scanned tile offsets.
__global__ void stripe_base_kernel(const int *__restrict__ stripe_count, const TileScan *__restrict__ scan,
                                   long long ntiles, long long *__restrict__ stripe_base)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ntiles;
         t += (long long)gridDim.x * blockDim.x) {
        long long o = scan[t].pairs;
#pragma unroll
        for (int k = 0; k < kStripes; ++k) {
            stripe_base[t * kStripes + k] = o;
            o += stripe_count[t * kStripes + k];
        }
    }
}

// Pass 1: normalise, store the normalised trajectory, count samples per
// tile.  Counts are aggregated per warp over lanes that hit the same tile
// (consecutive samples of a readout usually do), so a dense tile sees one
// atomic per warp instead of one per sample.
__device__ __forceinline__ float4 normalize_point(float4 p, int dim, float tr, float scale, int prenorm)
{
    float4 q;
    if (prenorm) {
        q.x = p.x;
        q.y = dim > 1 ? p.y : 0.f;
        q.z = dim > 2 ? p.z : 0.f;
    } else {
        q.x = __fmul_rn(__fadd_rn(p.x, tr), scale);
        q.y = dim > 1 ? __fmul_rn(__fadd_rn(p.y, tr), scale) : 0.f;
        q.z = dim > 2 ? __fmul_rn(__fadd_rn(p.z, tr), scale) : 0.f;
    }
    q.w = 0.f;
    return q;
}

__global__ void normalize_kernel(const float4 *__restrict__ raw, size_t n, int dim, const int *__restrict__ b,
                                 float4 *__restrict__ out)
{
    const float *bf = reinterpret_cast<const float *>(b);
    const float tr = bf[kTr], scale = bf[kScale];
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = normalize_point(raw[i], dim, tr, scale, 0);
}

__global__ void normalize_count_kernel(const float4 *__restrict__ raw, size_t n, BinGeom g, int *b, int prenorm,
                                       float4 *__restrict__ out, int *__restrict__ stripe_count)
{
    const float *bf = reinterpret_cast<const float *>(b);
    const float tr = bf[kTr], scale = bf[kScale];
    const int lane = threadIdx.x & 31;
    for (size_t base = blockIdx.x * (size_t)blockDim.x; base < n;
         base += (size_t)gridDim.x * blockDim.x) {
        size_t i = base + threadIdx.x;
        TileWalk w;
        int s[3], e[3];
        int cnt = 0;
        if (i < n) {
            float4 q = normalize_point(raw[i], g.dim, tr, scale, prenorm);
            out[i] = q;
            cnt = sample_tiles(g, q, w, s, e);
        } else {
            w.lo[0] = w.lo[1] = w.lo[2] = 0;
            w.n[0] = w.n[1] = w.n[2] = 1;
        }
        const int stripe = stripe_of(base + threadIdx.x - lane);
        int maxcnt = __reduce_max_sync(0xffffffffu, cnt);
        for (int j = 0; j < maxcnt; ++j, w.next()) {
            bool valid = j < cnt;
            int t = valid ? w.tile(g) : -1 - lane;
            int run, head_lane;
            lane_runs(t, lane, run, head_lane);
            if (valid && lane == head_lane) atomicAdd(&stripe_count[t * kStripes + stripe], run);
        }
    }
}

// Tap box of a sample inside one tile: the sample's clamped cell range
// (GridLut.cpp:98-106) with end taps |x - c| >= kHW removed when that test
// is exact (they can never pass dk < kHW), clipped to the tile, in tile-local
// coordinates.  Packed as lx0 | ly0<<6 | lz0<<12 | nx<<18 | ny<<22 | nz<<26.
__device__ __forceinline__ unsigned tile_box(const BinGeom &g, const float *c, const int *s, const int *e,
                                             int tx, int ty, int tz)
{
    const int t3[3] = {tx, ty, tz};
    unsigned box = 0;
    for (int d = 0; d < 3; ++d) {
        int lo = 0, num = 1;
        if (d < g.dim) {
            int o = t3[d] * g.tile[d];
            int a = max(s[d], o), b = min(e[d], o + g.tile[d] - 1);
            if (g.prefilter && a <= b) {
                if (!(fabsf(__fsub_rn((float)a, c[d])) < g.hw)) ++a;
                if (a <= b && !(fabsf(__fsub_rn((float)b, c[d])) < g.hw)) --b;
            }
            lo = a - o;
            num = a <= b ? b - a + 1 : 0;
            if (num == 0) lo = 0;
        }
        box |= (unsigned)lo << (6 * d);
        box |= (unsigned)num << (18 + 4 * d);
    }
    return box;
}

// Pass 3: fill the sorted bin lists with (sample index, tap box) records.
__global__ void fill_kernel(const float4 *__restrict__ traj, size_t n, BinGeom g,
                            const long long *__restrict__ stripe_base, int *__restrict__ tile_fill,
                            unsigned long long *__restrict__ recs)
{
    const int lane = threadIdx.x & 31;
    for (size_t base = blockIdx.x * (size_t)blockDim.x; base < n;
         base += (size_t)gridDim.x * blockDim.x) {
        size_t i = base + threadIdx.x;
        TileWalk w;
        int s[3] = {0, 0, 0}, e[3] = {0, 0, 0};
        float c[3] = {0.f, 0.f, 0.f};
        int cnt = 0;
        if (i < n) {
            float4 q = traj[i];
            cnt = sample_tiles(g, q, w, s, e);
            c[0] = q.x;
            c[1] = q.y;
            c[2] = q.z;
        } else {
            w.lo[0] = w.lo[1] = w.lo[2] = 0;
            w.n[0] = w.n[1] = w.n[2] = 1;
        }
        const int stripe = stripe_of(base + threadIdx.x - lane);
        int maxcnt = __reduce_max_sync(0xffffffffu, cnt);
        for (int j = 0; j < maxcnt; ++j, w.next()) {
            bool valid = j < cnt;
            int t = valid ? w.tile(g) : -1 - lane;
            int run, head_lane;
            lane_runs(t, lane, run, head_lane);
            int basepos = 0;
            const int ts = t * kStripes + stripe;
            if (valid && lane == head_lane) basepos = atomicAdd(&tile_fill[ts], run);
            basepos = __shfl_sync(0xffffffffu, basepos, head_lane);
            if (valid) {
                long long pos = stripe_base[ts] + basepos + (lane - head_lane);
                unsigned box = tile_box(g, c, s, e, w.lo[0] + w.jx, w.lo[1] + w.jy, w.lo[2] + w.jz);
                recs[pos] = ((unsigned long long)box << 32) | (unsigned long long)i;
            }
        }
    }
}

// Tap lists (the scatter's taps, evaluated once per trajectory).
struct TapGeom {
    unsigned *taps;                  // n x words
    unsigned long long *trecs;       // in bin order, beside the (sample | box) records
    const float4 *lut_e;             // {thr[k+1], lut[k], lut[k+1], 0}
    float smax, kc;
    int L, words;                    // tap words per sample slot
    int recmax;                      // records (tiles) one sample's range can touch
    int *err;                        // set when a slot would overflow (never, by the slot bound)
};

// Exact LUT index of s2 = dk^2 < smax, as the scatter's weight lookup: a
// first guess from an approximate square root (the exact index or one below)
// and one exact threshold test (thr[k] = smallest s with index >= k).
__device__ __forceinline__ int tap_lut_index(float s2, const float4 *__restrict__ lut_e, float kc, int L)
{
    float a;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(a) : "f"(s2));
    const int k0 = (int)fminf(fmaf(a, kc, 0.25f), (float)(L - 1));
    return k0 + (s2 >= __ldg(&lut_e[k0].x) ? 1 : 0);
}
// The same with the thresholds thr[k] = lut_e[k].x staged in shared memory.
__device__ __forceinline__ int tap_lut_index_s(float s2, const float *thr, float kc, int L)
{
    float a;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(a) : "f"(s2));
    const int k0 = (int)fminf(fmaf(a, kc, 0.25f), (float)(L - 1));
    return k0 + (s2 >= thr[k0] ? 1 : 0);
}

// Pass 3 with tap lists: the records of fill_kernel, and for each record the
// taps of the sample inside the record's tile, evaluated with the
// reference's geometry (GridLut.cpp:98-136: the clamped cell range, dk^2 =
// (dz^2 + dy^2) + dx^2 unfused, valid iff dk < kHW), as tap words in the
// sample's slot: one run per record, in the order of the sample's tile
// walk; trecs[pos] gives the run (first word, count).  Each thread walks its
// sample's whole cell range twice (the same box shape for neighbouring
// samples, so the lanes of a warp stay together): once to count the taps
// per record, once to place them, into a shared-memory copy of the slot;
// the block's slots, consecutive in memory, are then written out with
// coalesced 16-byte stores.
constexpr int kFillThreads = 256;
constexpr int kFillRecMax = 32;  // records per sample (tiles a sample's range touches) the fill supports

// cnt[j * kFillThreads], off[j * kFillThreads]: this thread's tap count and
// first slot word of record j (record-major, so a warp's lanes touch
// consecutive bytes).  XR >= the cells of the range along x: the x loop is
// unrolled over XR candidates whose dx^2 (or +inf past the range), tile-
// relative index and tile-local x are computed once per sample.
template <int XR>
__device__ __forceinline__ void sample_taps(const BinGeom &g, const TapGeom &tg, const float *c, const int *s,
                                            const int *e, const TileWalk &w, bool place, unsigned char *cnt,
                                            const unsigned char *off, unsigned *slot)
{
    float dx2[XR];
    int jx[XR], lx[XR];
#pragma unroll
    for (int i = 0; i < XR; ++i) {
        const int x = s[0] + i;
        const float dx = __fsub_rn((float)x, c[0]);
        dx2[i] = x <= e[0] ? __fmul_rn(dx, dx) : __int_as_float(0x7f800000);
        jx[i] = tile_div(g, x, 0) - w.lo[0];
        lx[i] = x - (w.lo[0] + jx[i]) * g.tile[0];
    }
    float fz = (float)s[2];
    for (int z = s[2]; z <= e[2]; ++z, fz = __fadd_rn(fz, 1.f)) {
        const float dz = g.dim == 3 ? __fsub_rn(fz, c[2]) : 0.f;
        const float dz2 = __fmul_rn(dz, dz);
        const int jz = tile_div(g, z, 2) - w.lo[2];
        const int lz = z - (w.lo[2] + jz) * g.tile[2];
        float fy = (float)s[1];
        for (int y = s[1]; y <= e[1]; ++y, fy = __fadd_rn(fy, 1.f)) {
            const float dy = __fsub_rn(fy, c[1]);
            const float dzy = __fadd_rn(dz2, __fmul_rn(dy, dy));
            const int jy = tile_div(g, y, 1) - w.lo[1];
            const int ly = y - (w.lo[1] + jy) * g.tile[1];
            const int jzy = (jz * w.n[1] + jy) * w.n[0];
            const int rowzy = (lz * g.tile[1] + ly) * g.tile[0];
#pragma unroll
            for (int i = 0; i < XR; ++i) {
                const float s2 = __fadd_rn(dzy, dx2[i]);
                if (s2 < tg.smax) {
                    const int j = (jzy + jx[i]) * kFillThreads;
                    const int k = cnt[j]++;
                    if (place) {
                        const int wi = off[j] + k;
                        if (wi < tg.words)
                            slot[wi] = (unsigned)(rowzy + lx[i]) |
                                       ((unsigned)tap_lut_index(s2, tg.lut_e, tg.kc, tg.L) << kTapCellBits);
                    }
                }
            }
        }
    }
}

// The same walk for samples whose range touches at most 8 tiles (at most 2
// along x), with the per-record tap counts and first words packed as bytes
// in two 64-bit registers (byte j: record j) instead of shared-memory
// counters: no load-add-store chain through shared memory per candidate
// cell, the counting walk one bitmask of valid x candidates per row (a popc
// per x tile), and the LUT thresholds read from shared memory.  The words and
// their order are those of sample_taps.
template <int XR>
__device__ __forceinline__ void sample_taps_pk(const BinGeom &g, const TapGeom &tg, const float *thr, const float *c,
                                               const int *s, const int *e, const TileWalk &w, bool place,
                                               unsigned long long &cnt, unsigned long long off, unsigned *slot)
{
    float dx2[XR];
    int jx[XR], lx[XR];
    unsigned pm1 = 0u;  // candidates in the second x tile (at most 2 x tiles)
#pragma unroll
    for (int i = 0; i < XR; ++i) {
        const int x = s[0] + i;
        const float dx = __fsub_rn((float)x, c[0]);
        dx2[i] = x <= e[0] ? __fmul_rn(dx, dx) : __int_as_float(0x7f800000);
        jx[i] = tile_div(g, x, 0) - w.lo[0];
        lx[i] = x - (w.lo[0] + jx[i]) * g.tile[0];
        if (jx[i] != 0) pm1 |= 1u << i;
    }
    float fz = (float)s[2];
    for (int z = s[2]; z <= e[2]; ++z, fz = __fadd_rn(fz, 1.f)) {
        const float dz = g.dim == 3 ? __fsub_rn(fz, c[2]) : 0.f;
        const float dz2 = __fmul_rn(dz, dz);
        const int jz = tile_div(g, z, 2) - w.lo[2];
        const int lz = z - (w.lo[2] + jz) * g.tile[2];
        float fy = (float)s[1];
        for (int y = s[1]; y <= e[1]; ++y, fy = __fadd_rn(fy, 1.f)) {
            const float dy = __fsub_rn(fy, c[1]);
            const float dzy = __fadd_rn(dz2, __fmul_rn(dy, dy));
            const int jy = tile_div(g, y, 1) - w.lo[1];
            const int ly = y - (w.lo[1] + jy) * g.tile[1];
            const int jzy = (jz * w.n[1] + jy) * w.n[0];
            const int rowzy = (lz * g.tile[1] + ly) * g.tile[0];
            if (!place) {
                // counting: the row's valid candidates as a bitmask, one
                // count per x tile (records (jz, jy, 0) and (jz, jy, 1))
                unsigned m = 0u;
#pragma unroll
                for (int i = 0; i < XR; ++i)
                    if (__fadd_rn(dzy, dx2[i]) < tg.smax) m |= 1u << i;
                cnt += (unsigned long long)((unsigned)__popc(m & ~pm1) | ((unsigned)__popc(m & pm1) << 8))
                       << (8u * (unsigned)jzy);
                continue;
            }
#pragma unroll
            for (int i = 0; i < XR; ++i) {
                const float s2 = __fadd_rn(dzy, dx2[i]);
                if (s2 < tg.smax) {
                    const unsigned sh = 8u * (unsigned)(jzy + jx[i]);
                    if (place) {
                        const int wi = (int)(((off >> sh) & 255ull) + ((cnt >> sh) & 255ull));
                        if (wi < tg.words)
                            slot[wi] = (unsigned)(rowzy + lx[i]) |
                                       ((unsigned)tap_lut_index_s(s2, thr, tg.kc, tg.L) << kTapCellBits);
                    }
                    cnt += 1ull << sh;
                }
            }
        }
    }
}

template <int XR>
__global__ void __launch_bounds__(kFillThreads) fill_taps_kernel(const float4 *__restrict__ traj, size_t n,
                                                                 BinGeom g, TapGeom tg,
                                                                 const long long *__restrict__ stripe_base,
                                                                 int *__restrict__ tile_fill,
                                                                 unsigned long long *__restrict__ recs)
{
    // [kFillThreads][S] slot words (S = words | 1: odd, no bank conflicts),
    // then the tap counts and the run offsets, recmax x kFillThreads each
    extern __shared__ unsigned stage[];
    const int S = tg.words | 1;
    const int lane = threadIdx.x & 31;
    unsigned *mine = stage + threadIdx.x * S;
    unsigned char *cnt = reinterpret_cast<unsigned char *>(stage + kFillThreads * S) + threadIdx.x;
    unsigned char *off = cnt + tg.recmax * kFillThreads;
    for (size_t base = blockIdx.x * (size_t)kFillThreads; base < n; base += (size_t)gridDim.x * kFillThreads) {
        size_t i = base + threadIdx.x;
        TileWalk w;
        int s[3] = {0, 0, 0}, e[3] = {0, 0, 0};
        float c[3] = {0.f, 0.f, 0.f};
        int cnt_t = 0;
        if (i < n) {
            float4 q = traj[i];
            cnt_t = sample_tiles(g, q, w, s, e);
            c[0] = q.x;
            c[1] = q.y;
            c[2] = q.z;
        } else {
            w.lo[0] = w.lo[1] = w.lo[2] = 0;
            w.n[0] = w.n[1] = w.n[2] = 1;
        }
        // taps per record, then each record's first word, then the taps
        int tot = 0;
        for (int j = 0; j < cnt_t; ++j) cnt[j * kFillThreads] = 0;
        // ranges of XR - 1 cells along x (all but samples on a cell
        // boundary: hw = 2 gives 4 cells unless c - 2 is an integer) walk
        // one candidate fewer per row
        const bool narrow = e[0] - s[0] + 1 < XR;
        if (cnt_t > 0) {
            if (narrow)
                sample_taps<XR - 1>(g, tg, c, s, e, w, false, cnt, off, mine);
            else
                sample_taps<XR>(g, tg, c, s, e, w, false, cnt, off, mine);
        }
        for (int j = 0; j < cnt_t; ++j) {
            off[j * kFillThreads] = (unsigned char)min(tot, 255);
            tot += cnt[j * kFillThreads];
            cnt[j * kFillThreads] = 0;
        }
        if (tot <= tg.words && cnt_t > 0) {
            if (narrow)
                sample_taps<XR - 1>(g, tg, c, s, e, w, true, cnt, off, mine);
            else
                sample_taps<XR>(g, tg, c, s, e, w, true, cnt, off, mine);
        }
        if (tot > tg.words) *tg.err = FR_ERR_CAPACITY;  // never: the slot bounds every sample's taps

        const int stripe = stripe_of(base + threadIdx.x - lane);
        int maxcnt = __reduce_max_sync(0xffffffffu, cnt_t);
        for (int j = 0; j < maxcnt; ++j, w.next()) {
            bool valid = j < cnt_t;
            int t = valid ? w.tile(g) : -1 - lane;
            int run, head_lane;
            lane_runs(t, lane, run, head_lane);
            int basepos = 0;
            const int ts = t * kStripes + stripe;
            if (valid && lane == head_lane) basepos = atomicAdd(&tile_fill[ts], run);
            basepos = __shfl_sync(0xffffffffu, basepos, head_lane);
            if (valid) {
                long long pos = stripe_base[ts] + basepos + (lane - head_lane);
                unsigned box = tile_box(g, c, s, e, w.lo[0] + w.jx, w.lo[1] + w.jy, w.lo[2] + w.jz);
                recs[pos] = ((unsigned long long)box << 32) | (unsigned long long)i;
                const int ntap = tot > tg.words ? 0 : cnt[j * kFillThreads];  // a dropped run (never) has no taps
                tg.trecs[pos] = (unsigned long long)i | ((unsigned long long)off[j * kFillThreads] << 32) |
                                ((unsigned long long)ntap << 40);
            }
        }
        __syncthreads();
        // the block's slots are words [base * words, (base + nv) * words):
        // 16-byte aligned (base is a multiple of kFillThreads), copied as uint4
        const int nv = (int)min((size_t)kFillThreads, n - base);
        const int W = tg.words, total = nv * W;
        uint4 *dst = reinterpret_cast<uint4 *>(tg.taps + base * (size_t)W);
        {
            // word wi = 4 qd + k of the block's slots is word (wi mod W) of
            // sample wi / W: kept as a (sample, word) pair advanced without
            // divisions (one division to start, then steps of 4 kFillThreads)
            const int step = 4 * kFillThreads, sq = step / W, sr = step - sq * W;
            int smp = (4 * threadIdx.x) / W, wd = 4 * threadIdx.x - smp * W;
            for (int qd = threadIdx.x; qd < total / 4; qd += kFillThreads) {
                unsigned v[4];
                int sm = smp, wk = wd;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    v[k] = stage[sm * S + wk];
                    if (++wk == W) {
                        wk = 0;
                        ++sm;
                    }
                }
                dst[qd] = make_uint4(v[0], v[1], v[2], v[3]);
                smp += sq;
                wd += sr;
                if (wd >= W) {
                    wd -= W;
                    ++smp;
                }
            }
        }
        for (int wi = (total & ~3) + threadIdx.x; wi < total; wi += kFillThreads) {
            const int smp = wi / W;
            tg.taps[base * (size_t)W + wi] = stage[smp * S + (wi - smp * W)];
        }
        __syncthreads();
    }
}

// fill_taps_kernel for samples touching at most 8 tiles (the 3D 4-wide
// kernel on 8^3 tiles, 2D on 32^2): counts and first words in registers
// (sample_taps_pk), LUT thresholds staged in shared memory after the slots.
template <int XR>
__global__ void __launch_bounds__(kFillThreads) fill_taps_pk_kernel(const float4 *__restrict__ traj, size_t n,
                                                                    BinGeom g, TapGeom tg,
                                                                    const long long *__restrict__ stripe_base,
                                                                    int *__restrict__ tile_fill,
                                                                    unsigned long long *__restrict__ recs)
{
    extern __shared__ unsigned stage[];
    const int S = tg.words | 1;
    const int lane = threadIdx.x & 31;
    unsigned *mine = stage + threadIdx.x * S;
    float *thr = reinterpret_cast<float *>(stage + kFillThreads * S);
    for (int k = threadIdx.x; k < tg.L; k += kFillThreads) thr[k] = __ldg(&tg.lut_e[k].x);
    __syncthreads();
    for (size_t base = blockIdx.x * (size_t)kFillThreads; base < n; base += (size_t)gridDim.x * kFillThreads) {
        size_t i = base + threadIdx.x;
        TileWalk w;
        int s[3] = {0, 0, 0}, e[3] = {0, 0, 0};
        float c[3] = {0.f, 0.f, 0.f};
        int cnt_t = 0;
        if (i < n) {
            float4 q = traj[i];
            cnt_t = sample_tiles(g, q, w, s, e);
            c[0] = q.x;
            c[1] = q.y;
            c[2] = q.z;
        } else {
            w.lo[0] = w.lo[1] = w.lo[2] = 0;
            w.n[0] = w.n[1] = w.n[2] = 1;
        }
        // taps per record (byte j of cnt), each record's first word (byte j
        // of off), then the taps
        unsigned long long cnt = 0ull, off = 0ull;
        const bool narrow = e[0] - s[0] + 1 < XR;
        if (cnt_t > 0) {
            if (narrow)
                sample_taps_pk<XR - 1>(g, tg, thr, c, s, e, w, false, cnt, 0ull, mine);
            else
                sample_taps_pk<XR>(g, tg, thr, c, s, e, w, false, cnt, 0ull, mine);
        }
        // runs at multiples of 4 words when the sample's padded runs fit in
        // its slot (the scatter then loads a lane's 4 taps as one 16-byte
        // word), else packed
        int tot = 0, totp = 0;
        unsigned long long offp = 0ull;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int cj = (int)((cnt >> (8 * j)) & 255ull);
            off |= (unsigned long long)min(tot, 255) << (8 * j);
            offp |= (unsigned long long)min(totp, 255) << (8 * j);
            tot += cj;
            totp += (cj + 3) & ~3;
        }
        if (totp <= tg.words) off = offp;
        if (tot <= tg.words && cnt_t > 0) {
            unsigned long long k = 0ull;  // taps placed per record
            if (narrow)
                sample_taps_pk<XR - 1>(g, tg, thr, c, s, e, w, true, k, off, mine);
            else
                sample_taps_pk<XR>(g, tg, thr, c, s, e, w, true, k, off, mine);
        }
        if (tot > tg.words) *tg.err = FR_ERR_CAPACITY;  // never: the slot bounds every sample's taps

        const int stripe = stripe_of(base + threadIdx.x - lane);
        int maxcnt = __reduce_max_sync(0xffffffffu, cnt_t);
        for (int j = 0; j < maxcnt; ++j, w.next()) {
            bool valid = j < cnt_t;
            int t = valid ? w.tile(g) : -1 - lane;
            int run, head_lane;
            lane_runs(t, lane, run, head_lane);
            int basepos = 0;
            const int ts = t * kStripes + stripe;
            if (valid && lane == head_lane) basepos = atomicAdd(&tile_fill[ts], run);
            basepos = __shfl_sync(0xffffffffu, basepos, head_lane);
            if (valid) {
                long long pos = stripe_base[ts] + basepos + (lane - head_lane);
                unsigned box = tile_box(g, c, s, e, w.lo[0] + w.jx, w.lo[1] + w.jy, w.lo[2] + w.jz);
                recs[pos] = ((unsigned long long)box << 32) | (unsigned long long)i;
                const unsigned sh = 8u * (unsigned)j;
                const unsigned long long ntap = tot > tg.words ? 0ull : (cnt >> sh) & 255ull;  // a dropped run (never) has no taps
                tg.trecs[pos] = (unsigned long long)i | (((off >> sh) & 255ull) << 32) | (ntap << 40);
            }
        }
        __syncthreads();
        // the block's slots are words [base * words, (base + nv) * words):
        // 16-byte aligned (base is a multiple of kFillThreads), copied as uint4
        const int nv = (int)min((size_t)kFillThreads, n - base);
        const int W = tg.words, total = nv * W;
        uint4 *dst = reinterpret_cast<uint4 *>(tg.taps + base * (size_t)W);
        {
            const int step = 4 * kFillThreads, sq = step / W, sr = step - sq * W;
            int smp = (4 * threadIdx.x) / W, wd = 4 * threadIdx.x - smp * W;
            for (int qd = threadIdx.x; qd < total / 4; qd += kFillThreads) {
                unsigned v[4];
                int sm = smp, wk = wd;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    v[k] = stage[sm * S + wk];
                    if (++wk == W) {
                        wk = 0;
                        ++sm;
                    }
                }
                dst[qd] = make_uint4(v[0], v[1], v[2], v[3]);
                smp += sq;
                wd += sr;
                if (wd >= W) {
                    wd -= W;
                    ++smp;
                }
            }
        }
        for (int wi = (total & ~3) + threadIdx.x; wi < total; wi += kFillThreads) {
            const int smp = wi / W;
            tg.taps[base * (size_t)W + wi] = stage[smp * S + (wi - smp * W)];
        }
        __syncthreads();
    }
}

__device__ __forceinline__ TileScan tile_value(int cnt, int chunk)
{
    TileScan v;
    long long items = (cnt + chunk - 1) / chunk;
    v.pairs = cnt;
    v.items = items;
    v.slots = items > 1 ? items : 0;
    v.splits = items > 1 ? 1 : 0;
    v.empties = cnt == 0 ? 1 : 0;
    return v;
}

__device__ __forceinline__ TileScan add(const TileScan &a, const TileScan &b)
{
    return TileScan{a.pairs + b.pairs, a.items + b.items, a.slots + b.slots, a.splits + b.splits,
                    a.empties + b.empties};
}

__device__ __forceinline__ TileScan shfl_up(const TileScan &v, int d)
{
    TileScan r;
    r.pairs = __shfl_up_sync(0xffffffffu, v.pairs, d);
    r.items = __shfl_up_sync(0xffffffffu, v.items, d);
    r.slots = __shfl_up_sync(0xffffffffu, v.slots, d);
    r.splits = __shfl_up_sync(0xffffffffu, v.splits, d);
    r.empties = __shfl_up_sync(0xffffffffu, v.empties, d);
    return r;
}

constexpr int kScanThreads = 256;
constexpr int kScanPerThread = 8;
constexpr int kScanSeg = kScanThreads * kScanPerThread;

// Block-wide exclusive scan of one value per thread; returns the exclusive
// prefix and writes the block total to *total.
__device__ TileScan block_exclusive(TileScan v, TileScan *total)
{
    __shared__ TileScan warp_tot[kScanThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    TileScan inc = v;
    for (int d = 1; d < 32; d <<= 1) {
        TileScan o = shfl_up(inc, d);
        if (lane >= d) inc = add(inc, o);
    }
    if (lane == 31) warp_tot[warp] = inc;
    __syncthreads();
    TileScan wpre{0, 0, 0, 0, 0}, all{0, 0, 0, 0, 0};
    for (int w = 0; w < kScanThreads / 32; ++w) {
        if (w < warp) wpre = add(wpre, warp_tot[w]);
        all = add(all, warp_tot[w]);
    }
    __syncthreads();
    *total = all;
    TileScan exc = add(wpre, inc);
    exc.pairs -= v.pairs;
    exc.items -= v.items;
    exc.slots -= v.slots;
    exc.splits -= v.splits;
    exc.empties -= v.empties;
    return exc;
}

__global__ void scan_reduce_kernel(const int *__restrict__ cnt, long long ntiles, int chunk,
                                   TileScan *__restrict__ block_sums)
{
    long long seg0 = (long long)blockIdx.x * kScanSeg;
    TileScan v{0, 0, 0, 0};
    for (int k = 0; k < kScanPerThread; ++k) {
        long long t = seg0 + (long long)k * kScanThreads + threadIdx.x;
        if (t < ntiles) v = add(v, tile_value(cnt[t], chunk));
    }
    TileScan tot;
    block_exclusive(v, &tot);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = tot;
}

// Exclusive scan of the block sums in place (single block, looping).
__global__ void scan_blocks_kernel(TileScan *sums, int nblocks)
{
    __shared__ TileScan carry;
    if (threadIdx.x == 0) carry = TileScan{0, 0, 0, 0, 0};
    __syncthreads();
    for (int base = 0; base < nblocks; base += kScanThreads) {
        int i = base + threadIdx.x;
        TileScan v = i < nblocks ? sums[i] : TileScan{0, 0, 0, 0, 0};
        TileScan tot;
        TileScan exc = block_exclusive(v, &tot);
        TileScan c = carry;
        if (i < nblocks) sums[i] = add(exc, c);
        __syncthreads();
        if (threadIdx.x == 0) carry = add(c, tot);
        __syncthreads();
    }
}

__global__ void scan_write_kernel(const int *__restrict__ cnt, long long ntiles, int chunk,
                                  const TileScan *__restrict__ block_sums, TileScan *__restrict__ out)
{
    // Each thread owns kScanPerThread consecutive tiles of the segment.
    long long seg0 = (long long)blockIdx.x * kScanSeg;
    long long t0 = seg0 + (long long)threadIdx.x * kScanPerThread;
    TileScan local[kScanPerThread];
    TileScan v{0, 0, 0, 0};
    for (int k = 0; k < kScanPerThread; ++k) {
        long long t = t0 + k;
        local[k] = t < ntiles ? tile_value(cnt[t], chunk) : TileScan{0, 0, 0, 0, 0};
        v = add(v, local[k]);
    }
    TileScan tot;
    TileScan exc = add(block_exclusive(v, &tot), block_sums[blockIdx.x]);
    for (int k = 0; k < kScanPerThread; ++k) {
        long long t = t0 + k;
        if (t < ntiles) out[t] = exc;
        exc = add(exc, local[k]);
        if (t == ntiles - 1) out[ntiles] = exc;
    }
}

__global__ void items_kernel(const int *__restrict__ cnt, const TileScan *__restrict__ scan,
                             long long ntiles, int chunk, WorkItem *__restrict__ items,
                             SplitTile *__restrict__ splits)
{
    const long long occupied = scan[ntiles].items;  // the zero-fill items of empty tiles follow
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ntiles;
         t += (long long)gridDim.x * blockDim.x) {
        int c = cnt[t];
        TileScan v = tile_value(c, chunk);
        TileScan o = scan[t];
        if (c == 0) {
            WorkItem w;
            w.begin = o.pairs;
            w.count = 0;
            w.tile = (int)t;
            w.slot = -1;
            w.pad = 0;
            items[occupied + o.empties] = w;
        }
        for (long long k = 0; k < v.items; ++k) {
            WorkItem w;
            w.begin = o.pairs + k * chunk;
            w.count = c == 0 ? 0 : (int)min((long long)chunk, (long long)c - k * chunk);
            w.tile = (int)t;
            w.slot = v.items > 1 ? (int)(o.slots + k) : -1;
            w.pad = 0;
            items[o.items + k] = w;
        }
        if (v.items > 1) {
            SplitTile s;
            s.tile = (int)t;
            s.first_slot = (int)o.slots;
            s.nslots = (int)v.items;
            s.pad = 0;
            splits[o.splits] = s;
        }
    }
}

// Deterministic plans (FR_PLAN_DETERMINISTIC).  The bin fill places a
// tile's records with atomics, so which records each work item of a split
// tile holds -- and with them each item's fixed-point scale and rounding --
// varies from run to run.  These two kernels put the records of every split
// tile in sample order (sample indices are unique within a tile), moving the
// tap records beside them: the records are bucketed by sample index (one
// CTA per split tile, buckets of ~kSortBucket records over the tile's
// index range), then each bucket is rank-sorted by one warp.
constexpr int kSortBucket = 256;
constexpr int kSortMaxBuckets = 8192;
constexpr int kSortThreads = 1024;

__global__ void __launch_bounds__(kSortThreads) split_bucket_kernel(
    const SplitTile *__restrict__ splits, const TileScan *__restrict__ scan, const int *__restrict__ tile_count,
    const unsigned long long *__restrict__ recs, const unsigned long long *__restrict__ trecs,
    unsigned long long *__restrict__ recs_tmp, unsigned long long *__restrict__ trecs_tmp,
    SortBucket *__restrict__ buckets, int *__restrict__ nbuckets)
{
    __shared__ unsigned hist[kSortMaxBuckets];
    __shared__ unsigned part[kSortThreads / 32];
    __shared__ unsigned mnmx[2];
    __shared__ int base;
    const int t = splits[blockIdx.x].tile;
    const long long b = scan[t].pairs;
    const int c = tile_count[t];
    const int B = min((c + kSortBucket - 1) / kSortBucket, kSortMaxBuckets);
    if (threadIdx.x == 0) {
        mnmx[0] = 0xffffffffu;
        mnmx[1] = 0u;
        base = atomicAdd(nbuckets, B);
    }
    for (int i = threadIdx.x; i < kSortMaxBuckets; i += kSortThreads) hist[i] = 0u;
    __syncthreads();
    unsigned lmn = 0xffffffffu, lmx = 0u;
    for (int i = threadIdx.x; i < c; i += kSortThreads) {
        const unsigned k = (unsigned)recs[b + i];
        lmn = min(lmn, k);
        lmx = max(lmx, k);
    }
    lmn = __reduce_min_sync(0xffffffffu, lmn);
    lmx = __reduce_max_sync(0xffffffffu, lmx);
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&mnmx[0], lmn);
        atomicMax(&mnmx[1], lmx);
    }
    __syncthreads();
    const unsigned mn = mnmx[0];
    const unsigned long long span = (unsigned long long)(mnmx[1] - mn) + 1ull;
    auto bucket_of = [&](unsigned k) { return (int)(((unsigned long long)(k - mn) * (unsigned)B) / span); };
    for (int i = threadIdx.x; i < c; i += kSortThreads) atomicAdd(&hist[bucket_of((unsigned)recs[b + i])], 1u);
    __syncthreads();
    // exclusive scan of hist[0, kSortMaxBuckets): 8 consecutive entries per thread
    constexpr int PER = kSortMaxBuckets / kSortThreads;
    unsigned v[PER], sum = 0;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        v[k] = hist[threadIdx.x * PER + k];
        sum += v[k];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned inc = sum;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned o = __shfl_up_sync(0xffffffffu, inc, d);
        if (lane >= d) inc += o;
    }
    if (lane == 31) part[warp] = inc;
    __syncthreads();
    unsigned wpre = 0;
    for (int w = 0; w < warp; ++w) wpre += part[w];
    unsigned off = wpre + inc - sum;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int i = threadIdx.x * PER + k;
        if (i < B) buckets[base + i] = SortBucket{b + off, (int)v[k], 0};
        hist[i] = off;  // cursor
        off += v[k];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < c; i += kSortThreads) {
        const unsigned long long r = recs[b + i];
        const unsigned pos = atomicAdd(&hist[bucket_of((unsigned)r)], 1u);
        recs_tmp[b + pos] = r;
        if (trecs) trecs_tmp[b + pos] = trecs[b + i];
    }
}

__global__ void split_sort_kernel(const SortBucket *__restrict__ buckets, const int *__restrict__ nbuckets,
                                  const unsigned long long *__restrict__ recs_tmp,
                                  const unsigned long long *__restrict__ trecs_tmp,
                                  unsigned long long *__restrict__ recs, unsigned long long *__restrict__ trecs)
{
    const int lane = threadIdx.x & 31;
    const int nb = *nbuckets;
    for (long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; w < nb;
         w += ((long long)gridDim.x * blockDim.x) >> 5) {
        const SortBucket bk = buckets[w];
        const unsigned long long *src = recs_tmp + bk.start;
        for (int i = lane; i < bk.count; i += 32) {
            const unsigned long long r = src[i];
            const unsigned key = (unsigned)r;
            int rank = 0;
            for (int j = 0; j < bk.count; ++j) rank += (unsigned)__ldg(src + j) < key ? 1 : 0;
            recs[bk.start + rank] = r;
            if (trecs) trecs[bk.start + rank] = trecs_tmp[bk.start + i];
        }
    }
}

// Bit t of the occupancy bitmap: tile t holds at least one bin record.
__global__ void tile_mask_kernel(const int *__restrict__ cnt, long long ntiles, unsigned *__restrict__ mask)
{
    const long long nw = (ntiles + 31) / 32;
    for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < nw; w += (long long)gridDim.x * blockDim.x) {
        unsigned m = 0;
        for (int b = 0; b < 32; ++b) {
            const long long t = w * 32 + b;
            if (t < ntiles && cnt[t] > 0) m |= 1u << b;
        }
        mask[w] = m;
    }
}

__global__ void ranges_kernel(const float4 *__restrict__ traj, size_t n, int dim, unsigned G, float hw,
                              int *__restrict__ start, int *__restrict__ end)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        float4 p = traj[i];
        float c[3] = {p.x, p.y, p.z};
        for (int d = 0; d < 3; ++d) {
            int s = 0, e = 0;
            if (d < dim) comp_range(c[d], hw, G, s, e);
            start[3 * i + d] = s;
            end[3 * i + d] = e;
        }
    }
}

int grid_blocks(size_t n, int threads)
{
    size_t b = (n + threads - 1) / threads;
    return (int)std::max<size_t>(1, std::min<size_t>(b, 152 * 32));
}

}  // namespace

int plan_run(fr_plan p, const float *d_traj, size_t n, cudaStream_t s)
{
    if ((reinterpret_cast<uintptr_t>(d_traj) & 15) != 0)
        return fail(FR_ERR_INVALID_ARGUMENT, "trajectory pointer must be 16-byte aligned");
    if (n > 0xFFFFFFFFull) return fail(FR_ERR_UNSUPPORTED, "more than 2^32-1 samples");
    p->planned = false;
    p->n = n;
    p->chunk = p->chunk_req > 0 ? p->chunk_req : plan_chunk(n, p->dim);
    if (p->bounds.reserve(kBoundsSlots * 4)) return FR_ERR_OUT_OF_MEMORY;
    if (p->traj.reserve(std::max<size_t>(n, 1) * 16)) return FR_ERR_OUT_OF_MEMORY;
    if (p->tile_count.reserve(p->ntiles * 4) || p->tile_fill.reserve(p->ntiles * kStripes * 4) ||
        p->stripe_count.reserve(p->ntiles * kStripes * 4) || p->stripe_base.reserve(p->ntiles * kStripes * 8) ||
        p->tile_scan.reserve((p->ntiles + 1) * sizeof(TileScan)))
        return FR_ERR_OUT_OF_MEMORY;
    long long nblocks = (p->ntiles + kScanSeg - 1) / kScanSeg;
    if (p->scan_blocks.reserve(std::max<long long>(nblocks, 1) * sizeof(TileScan))) return FR_ERR_OUT_OF_MEMORY;

    int *b = p->bounds.as<int>();
    FR_CUDA(cudaMemsetAsync(p->stripe_count.ptr, 0, p->ntiles * kStripes * 4, s));
    FR_CUDA(cudaMemsetAsync(p->tile_fill.ptr, 0, p->ntiles * kStripes * 4, s));
    bounds_init_kernel<<<1, 32, 0, s>>>(b);
    FR_CHECK_LAUNCH("bounds_init_kernel");
    const float4 *raw = reinterpret_cast<const float4 *>(d_traj);
    if (n > 0) {
        bounds_kernel<<<std::min(grid_blocks(n, 256), 152 * 4), 256, 0, s>>>(raw, n, p->dim, b);
        FR_CHECK_LAUNCH("bounds_kernel");
    }
    scale_kernel<<<1, 1, 0, s>>>(b, p->dim, p->G);
    FR_CHECK_LAUNCH("scale_kernel");

    BinGeom g;
    g.dim = p->dim;
    g.G = p->G;
    g.hw = p->hw;
    g.prefilter = p->prefilter;
    for (int d = 0; d < 3; ++d) {
        g.tile[d] = p->tile[d];
        g.ntile[d] = p->ntile[d];
        g.tshift[d] = (g.tile[d] & (g.tile[d] - 1)) == 0 ? __builtin_ctz((unsigned)g.tile[d]) : -1;
    }
    float4 *traj = p->traj.as<float4>();
    if (n > 0) {
        normalize_count_kernel<<<grid_blocks(n, 256), 256, 0, s>>>(
            raw, n, g, b, (p->flags & FR_PLAN_PRENORMALIZED) ? 1 : 0, traj, p->stripe_count.as<int>());
        FR_CHECK_LAUNCH("normalize_count_kernel");
    }
    stripe_total_kernel<<<grid_blocks(p->ntiles, 256), 256, 0, s>>>(p->stripe_count.as<int>(), p->ntiles,
                                                                    p->tile_count.as<int>());
    FR_CHECK_LAUNCH("stripe_total_kernel");
    TileScan *bs = p->scan_blocks.as<TileScan>();
    TileScan *scan = p->tile_scan.as<TileScan>();
    scan_reduce_kernel<<<(int)nblocks, kScanThreads, 0, s>>>(p->tile_count.as<int>(), p->ntiles, p->chunk, bs);
    FR_CHECK_LAUNCH("scan_reduce_kernel");
    scan_blocks_kernel<<<1, kScanThreads, 0, s>>>(bs, (int)nblocks);
    FR_CHECK_LAUNCH("scan_blocks_kernel");
    scan_write_kernel<<<(int)nblocks, kScanThreads, 0, s>>>(p->tile_count.as<int>(), p->ntiles, p->chunk, bs,
                                                            scan);
    FR_CHECK_LAUNCH("scan_write_kernel");
    stripe_base_kernel<<<grid_blocks(p->ntiles, 256), 256, 0, s>>>(p->stripe_count.as<int>(), scan, p->ntiles,
                                                                   p->stripe_base.as<long long>());
    FR_CHECK_LAUNCH("stripe_base_kernel");

    TileScan tot;
    FR_CUDA(cudaMemcpyAsync(&tot, scan + p->ntiles, sizeof(TileScan), cudaMemcpyDeviceToHost, s));
    FR_CUDA(cudaMemcpyAsync(p->bounds_host, reinterpret_cast<float *>(b) + kNormLo, 6 * 4,
                            cudaMemcpyDeviceToHost, s));
    float raw_b[6];
    FR_CUDA(cudaMemcpyAsync(raw_b, reinterpret_cast<float *>(b) + kRawLo, 6 * 4, cudaMemcpyDeviceToHost, s));
    FR_CUDA(cudaStreamSynchronize(s));
    // bounds_host: raw lo[3], raw hi[3], norm lo[3], norm hi[3]
    float norm_b[6];
    for (int i = 0; i < 6; ++i) norm_b[i] = p->bounds_host[i];
    const bool prenorm = (p->flags & FR_PLAN_PRENORMALIZED) != 0;
    for (int i = 0; i < 6; ++i) p->bounds_host[i] = raw_b[i];
    for (int i = 0; i < 6; ++i) p->bounds_host[6 + i] = prenorm ? raw_b[i] : norm_b[i];

    if (tot.pairs > 0xFFFFFFFFll || tot.items + tot.empties > INT_MAX || tot.slots > INT_MAX)
        return fail(FR_ERR_UNSUPPORTED, "bin lists exceed 32-bit indexing");
    p->npairs = tot.pairs;
    p->nitems = tot.items + tot.empties;
    p->nitems_occupied = tot.items;
    p->nslots = tot.slots;
    p->nsplits = tot.splits;
    if (p->pairs.reserve(std::max<long long>(tot.pairs, 1) * 8) ||
        p->items.reserve(std::max<long long>(p->nitems, 1) * sizeof(WorkItem)) ||
        p->splits.reserve(std::max<long long>(tot.splits, 1) * sizeof(SplitTile)))
        return FR_ERR_OUT_OF_MEMORY;
    // tap lists, when the tile and kernel allow them and the memory is there
    p->tap_words = 0;
    int recmax = 1;
    if (p->taps_enabled && n > 0 && p->err_dev && p->L < (1 << (32 - kTapCellBits)) &&
        (long long)p->tile[0] * p->tile[1] * p->tile[2] <= (1 << kTapCellBits)) {
        if (p->tap_layout_words == 0) tap_slot_layout(p->dim, p->hw, &p->tap_layout_words);
        const int words = p->tap_layout_words;
        // tiles one sample's cell range (at most floor(2 hw) + 1 cells per axis) can touch
        const int F = (int)std::floor(2.0 * p->hw) + 1;
        recmax = 1;
        for (int d = 0; d < p->dim; ++d) recmax *= (F - 1 + p->tile[d] - 1) / p->tile[d] + 1;
        if (words <= kTapRecMax && recmax <= kFillRecMax && F <= 9 && !p->taps.reserve(n * (size_t)words * 4) &&
            !p->trecs.reserve(std::max<long long>(tot.pairs, 1) * 8))
            p->tap_words = words;
    }
    if (n > 0 && p->tap_words > 0) {
        TapGeom tg;
        tg.taps = p->taps.as<unsigned>();
        tg.trecs = p->trecs.as<unsigned long long>();
        tg.lut_e = p->lut_e.as<float4>();
        tg.smax = p->lut_smax;
        tg.kc = p->lut_kc;
        tg.L = p->L;
        tg.words = p->tap_words;
        tg.err = p->err_dev;
        tg.recmax = recmax;
        // slot staging plus 2 bytes per possible record: 4 CTAs of 256 per SM
        // for the 3D 4-wide kernel (42 words, 8 records)
        // (packed-counter form when a sample touches at most 8 tiles and at
        // most 2 along x: slot staging plus the L thresholds)
        const bool pk = recmax <= 8 && ((int)std::floor(2.0 * p->hw) + p->tile[0] - 1) / p->tile[0] + 1 <= 2;
        const size_t smem = pk ? (size_t)kFillThreads * (size_t)(p->tap_words | 1) * 4 + (size_t)p->L * 4
                               : (size_t)kFillThreads * ((size_t)(p->tap_words | 1) * 4 + 2 * recmax);
        // cells of a sample's range along x: at most floor(2 hw) + 1
        const int Fx = (int)std::floor(2.0 * p->hw) + 1;
        auto kern = pk ? (Fx <= 5 ? fill_taps_pk_kernel<5> : fill_taps_pk_kernel<9>)
                       : (Fx <= 5 ? fill_taps_kernel<5> : fill_taps_kernel<9>);
        if ((int)std::floor(2.0 * p->hw) + 1 > 9) return fail(FR_ERR_UNSUPPORTED, "tap lists: kernel too wide");
        if (smem > 48 * 1024)
            FR_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<grid_blocks(n, kFillThreads), kFillThreads, smem, s>>>(
            traj, n, g, tg, p->stripe_base.as<long long>(), p->tile_fill.as<int>(), p->pairs.as<unsigned long long>());
        FR_CHECK_LAUNCH(pk ? "fill_taps_pk_kernel" : "fill_taps_kernel");
    } else if (n > 0) {
        fill_kernel<<<grid_blocks(n, 256), 256, 0, s>>>(traj, n, g, p->stripe_base.as<long long>(), p->tile_fill.as<int>(),
                                                        p->pairs.as<unsigned long long>());
        FR_CHECK_LAUNCH("fill_kernel");
    }
    items_kernel<<<grid_blocks(p->ntiles, 256), 256, 0, s>>>(p->tile_count.as<int>(), scan, p->ntiles,
                                                             p->chunk, p->items.as<WorkItem>(),
                                                             p->splits.as<SplitTile>());
    FR_CHECK_LAUNCH("items_kernel");
    if ((p->flags & FR_PLAN_DETERMINISTIC) && p->nsplits > 0) {
        // split tiles' records in sample order (see split_bucket_kernel)
        const bool taps = p->tap_words > 0;
        const long long nb_max = p->npairs / kSortBucket + p->nsplits + 1;
        if (p->nsplits > INT_MAX || p->sort_tmp.reserve((size_t)p->npairs * 8 * (taps ? 2 : 1)) ||
            p->sort_buckets.reserve((size_t)nb_max * sizeof(SortBucket) + 16))
            return FR_ERR_OUT_OF_MEMORY;
        unsigned long long *rt = p->sort_tmp.as<unsigned long long>();
        unsigned long long *tt = taps ? rt + p->npairs : nullptr;
        SortBucket *bk = p->sort_buckets.as<SortBucket>();
        int *nbk = reinterpret_cast<int *>(bk + nb_max);
        FR_CUDA(cudaMemsetAsync(nbk, 0, sizeof(int), s));
        split_bucket_kernel<<<(unsigned)p->nsplits, kSortThreads, 0, s>>>(
            p->splits.as<SplitTile>(), scan, p->tile_count.as<int>(), p->pairs.as<unsigned long long>(),
            taps ? p->trecs.as<unsigned long long>() : nullptr, rt, tt, bk, nbk);
        FR_CHECK_LAUNCH("split_bucket_kernel");
        split_sort_kernel<<<152 * 8, 256, 0, s>>>(bk, nbk, rt, tt, p->pairs.as<unsigned long long>(),
                                                 taps ? p->trecs.as<unsigned long long>() : nullptr);
        FR_CHECK_LAUNCH("split_sort_kernel");
    }
    if (p->tile_mask.reserve((size_t)((p->ntiles + 31) / 32) * 4)) return FR_ERR_OUT_OF_MEMORY;
    tile_mask_kernel<<<grid_blocks((p->ntiles + 31) / 32, 256), 256, 0, s>>>(p->tile_count.as<int>(), p->ntiles,
                                                                              p->tile_mask.as<unsigned>());
    FR_CHECK_LAUNCH("tile_mask_kernel");
    p->planned = true;
    return FR_OK;
}

namespace {
__global__ void transform_kernel(float4 *__restrict__ traj, size_t n, int dim, float tr, float scale)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float4 p = traj[i];
        p.x = __fmul_rn(__fadd_rn(p.x, tr), scale);
        if (dim > 1) p.y = __fmul_rn(__fadd_rn(p.y, tr), scale);
        if (dim > 2) p.z = __fmul_rn(__fadd_rn(p.z, tr), scale);
        traj[i] = p;
    }
}
}  // namespace

int transform_run(float *d_traj, size_t n, int dim, float tr, float scale, cudaStream_t s)
{
    if (reinterpret_cast<uintptr_t>(d_traj) & 15)
        return fail(FR_ERR_INVALID_ARGUMENT, "trajectory pointer must be 16-byte aligned");
    if (n == 0) return FR_OK;
    transform_kernel<<<grid_blocks(n, 256), 256, 0, s>>>(reinterpret_cast<float4 *>(d_traj), n, dim, tr, scale);
    FR_CHECK_LAUNCH("transform_kernel");
    return FR_OK;
}

int normalize_run(const float *d_traj, size_t n, int dim, unsigned G, float *d_out, float *bounds12,
                  cudaStream_t s)
{
    if ((reinterpret_cast<uintptr_t>(d_traj) & 15) || (reinterpret_cast<uintptr_t>(d_out) & 15))
        return fail(FR_ERR_INVALID_ARGUMENT, "trajectory pointers must be 16-byte aligned");
    int *b = nullptr;
    FR_CUDA(cudaMallocAsync(reinterpret_cast<void **>(&b), kBoundsSlots * 4, s));
    bounds_init_kernel<<<1, 32, 0, s>>>(b);
    FR_CHECK_LAUNCH("bounds_init_kernel");
    const float4 *raw = reinterpret_cast<const float4 *>(d_traj);
    if (n > 0) {
        bounds_kernel<<<std::min(grid_blocks(n, 256), 152 * 4), 256, 0, s>>>(raw, n, dim, b);
        FR_CHECK_LAUNCH("bounds_kernel");
    }
    scale_kernel<<<1, 1, 0, s>>>(b, dim, G);
    FR_CHECK_LAUNCH("scale_kernel");
    if (n > 0) {
        normalize_kernel<<<grid_blocks(n, 256), 256, 0, s>>>(raw, n, dim, b, reinterpret_cast<float4 *>(d_out));
        FR_CHECK_LAUNCH("normalize_kernel");
    }
    float hb[12];
    FR_CUDA(cudaMemcpyAsync(hb, reinterpret_cast<float *>(b) + kRawLo, 6 * 4, cudaMemcpyDeviceToHost, s));
    FR_CUDA(cudaMemcpyAsync(hb + 6, reinterpret_cast<float *>(b) + kNormLo, 6 * 4, cudaMemcpyDeviceToHost, s));
    FR_CUDA(cudaFreeAsync(b, s));
    FR_CUDA(cudaStreamSynchronize(s));
    if (bounds12)
        for (int i = 0; i < 12; ++i) bounds12[i] = hb[i];
    return FR_OK;
}

int plan_stripes() { return kStripes; }

void tap_slot_layout(int dim, float hw, int *words)
{
    // Most lattice points strictly inside a ball of radius hw, over all
    // centres: centres on a grid of step h over the unit cell, counted with
    // radius hw + h sqrt(d) / 2 (every centre lies that close to a grid
    // centre), so the count bounds every sample's taps from above.
    const double h = 1.0 / 16, r = (double)hw + h * std::sqrt((double)dim) / 2, r2 = r * r;
    const int R = (int)std::ceil(r) + 1;
    int nmax = 0;
    const int nc = 16, ncz = dim == 3 ? 16 : 1;
    for (int cz = 0; cz < ncz; ++cz)
        for (int cy = 0; cy < nc; ++cy)
            for (int cx = 0; cx < nc; ++cx) {
                const double c[3] = {cx * h, cy * h, cz * h};
                int cnt = 0;
                for (int z = (dim == 3 ? -R : 0); z <= (dim == 3 ? R + 1 : 0); ++z)
                    for (int y = -R; y <= R + 1; ++y)
                        for (int x = -R; x <= R + 1; ++x) {
                            const double dx = x - c[0], dy = y - c[1], dz = dim == 3 ? z - c[2] : 0.0;
                            if (dx * dx + dy * dy + dz * dz < r2) ++cnt;
                        }
                nmax = std::max(nmax, cnt);
            }
    // a multiple of 4 words: slots start on 16-byte boundaries, so runs placed
    // at multiples of 4 words in a slot are 16-byte aligned
    *words = (nmax + 3) & ~3;
}

int plan_chunk(size_t n, int dim)
{
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        sms = 152;
    // ~2.7 records per sample with 8^3 tiles in 3D, ~1.2 with 32^2 tiles in 2D;
    // 2 CTAs per SM, at least 8 items each
    const double records = (double)n * (dim == 3 ? 2.7 : 1.2);
    const double per = records / ((double)sms * 2 * 8);
    int c = 512;
    while (c < 4096 && 2.0 * c <= per) c <<= 1;
    return c;
}

long long plan_scan_blocks(long long ntiles)
{
    return std::max<long long>((ntiles + kScanSeg - 1) / kScanSeg, 1);
}

// The plan of plan_run, into caller-provided buffers (fr_grid_noalloc).
int plan_into(const PlanInto &pi, const float *d_traj, size_t n, cudaStream_t s, PlanIntoOut *out)
{
    const long long nblocks = (pi.ntiles + kScanSeg - 1) / kScanSeg;
    int *b = pi.bounds;
    FR_CUDA(cudaMemsetAsync(pi.stripe_count, 0, pi.ntiles * kStripes * 4, s));
    FR_CUDA(cudaMemsetAsync(pi.tile_fill, 0, pi.ntiles * kStripes * 4, s));
    bounds_init_kernel<<<1, 32, 0, s>>>(b);
    FR_CHECK_LAUNCH("bounds_init_kernel");
    const float4 *raw = reinterpret_cast<const float4 *>(d_traj);
    if (n > 0) {
        bounds_kernel<<<std::min(grid_blocks(n, 256), 152 * 4), 256, 0, s>>>(raw, n, pi.dim, b);
        FR_CHECK_LAUNCH("bounds_kernel");
    }
    scale_kernel<<<1, 1, 0, s>>>(b, pi.dim, pi.G);
    FR_CHECK_LAUNCH("scale_kernel");
    BinGeom g;
    g.dim = pi.dim;
    g.G = pi.G;
    g.hw = pi.hw;
    g.prefilter = pi.prefilter;
    for (int d = 0; d < 3; ++d) {
        g.tile[d] = pi.tile[d];
        g.ntile[d] = pi.ntile[d];
        g.tshift[d] = (g.tile[d] & (g.tile[d] - 1)) == 0 ? __builtin_ctz((unsigned)g.tile[d]) : -1;
    }
    if (n > 0) {
        normalize_count_kernel<<<grid_blocks(n, 256), 256, 0, s>>>(raw, n, g, b, 0, pi.traj, pi.stripe_count);
        FR_CHECK_LAUNCH("normalize_count_kernel");
    }
    stripe_total_kernel<<<grid_blocks(pi.ntiles, 256), 256, 0, s>>>(pi.stripe_count, pi.ntiles, pi.tile_count);
    FR_CHECK_LAUNCH("stripe_total_kernel");
    scan_reduce_kernel<<<(int)nblocks, kScanThreads, 0, s>>>(pi.tile_count, pi.ntiles, pi.chunk, pi.scan_blocks);
    FR_CHECK_LAUNCH("scan_reduce_kernel");
    scan_blocks_kernel<<<1, kScanThreads, 0, s>>>(pi.scan_blocks, (int)nblocks);
    FR_CHECK_LAUNCH("scan_blocks_kernel");
    scan_write_kernel<<<(int)nblocks, kScanThreads, 0, s>>>(pi.tile_count, pi.ntiles, pi.chunk, pi.scan_blocks,
                                                            pi.scan);
    FR_CHECK_LAUNCH("scan_write_kernel");
    stripe_base_kernel<<<grid_blocks(pi.ntiles, 256), 256, 0, s>>>(pi.stripe_count, pi.scan, pi.ntiles,
                                                                   pi.stripe_base);
    FR_CHECK_LAUNCH("stripe_base_kernel");
    TileScan tot;
    FR_CUDA(cudaMemcpyAsync(&tot, pi.scan + pi.ntiles, sizeof(TileScan), cudaMemcpyDeviceToHost, s));
    FR_CUDA(cudaStreamSynchronize(s));
    if (tot.pairs > 0xFFFFFFFFll || tot.items + tot.empties > INT_MAX || tot.slots > INT_MAX)
        return fail(FR_ERR_UNSUPPORTED, "bin lists exceed 32-bit indexing");
    tot.items += tot.empties;  // every tile's items, the empty tiles' zero-fill items last
    // carve records, items and split tiles (256-byte aligned) from `rest`
    auto align = [](size_t v) { return (v + 255) & ~(size_t)255; };
    const size_t recs_b = align(std::max<long long>(tot.pairs, 1) * 8);
    const size_t items_b = align(std::max<long long>(tot.items, 1) * sizeof(WorkItem));
    const size_t splits_b = align(std::max<long long>(tot.splits, 1) * sizeof(SplitTile));
    if (recs_b + items_b + splits_b > pi.rest_bytes)
        return fail(FR_ERR_CAPACITY, "bin lists of this trajectory do not fit the no-allocation scratch");
    out->npairs = tot.pairs;
    out->nitems = tot.items;
    out->nslots = tot.slots;
    out->nsplits = tot.splits;
    out->recs = reinterpret_cast<unsigned long long *>(pi.rest);
    out->items = reinterpret_cast<WorkItem *>(pi.rest + recs_b);
    out->splits = reinterpret_cast<SplitTile *>(pi.rest + recs_b + items_b);
    out->rest_used = recs_b + items_b + splits_b;
    if (n > 0) {
        fill_kernel<<<grid_blocks(n, 256), 256, 0, s>>>(pi.traj, n, g, pi.stripe_base, pi.tile_fill, out->recs);
        FR_CHECK_LAUNCH("fill_kernel");
    }
    items_kernel<<<grid_blocks(pi.ntiles, 256), 256, 0, s>>>(pi.tile_count, pi.scan, pi.ntiles, pi.chunk, out->items,
                                                             out->splits);
    FR_CHECK_LAUNCH("items_kernel");
    return FR_OK;
}

int sample_ranges_run(fr_plan p, int *d_start, int *d_end, cudaStream_t s)
{
    if (p->n == 0) return FR_OK;
    ranges_kernel<<<grid_blocks(p->n, 256), 256, 0, s>>>(p->traj.as<float4>(), p->n, p->dim, p->G, p->hw,
                                                          d_start, d_end);
    FR_CHECK_LAUNCH("ranges");
    return FR_OK;
}

}  // namespace fr
