// fr_noalloc.cu -- gridding that allocates no device memory (fr_grid_noalloc).
//
// For callers that own the device-memory budget and cannot let a library call
// cudaMalloc in the middle of their work: a scanner's real-time reconstruction
// loop that reserves its memory at start-up, or a host framework whose caching
// allocator already holds the device memory.  The call does the work of
// fr_plan_create + fr_plan_set_trajectory + fr_grid (default tiling, no
// checkerboard) with every plan and scatter buffer carved from one fixed
// scratch array in device memory, declared below.
//
// The scratch is a file-scope __device__ array of FR_NOALLOC_SCRATCH_BYTES
// (32 MiB): every GPU that loads this library holds it until the process
// exits.  Its device address is looked up with cudaGetSymbolAddress on every
// call, on the caller's current device (a host-side query; nothing is cached,
// so a device reset or a reloaded module never leaves a stale address); the
// address of the array's name in host code is only a host-side stand-in and
// is never passed to a kernel.  All calls share the array and it keeps the
// last call's contents: the counters that must start at zero are cleared by
// each call, and calls that overlap on the GPU (other streams, other host
// threads) race on it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "fr_internal.h"

namespace fr {
namespace {

__device__ __align__(256) unsigned char g_noalloc_scratch[FR_NOALLOC_SCRATCH_BYTES];

// Device address of the scratch on the current device.
int scratch_on_current_device(unsigned char **out)
{
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-allocation scratch)");
    *out = static_cast<unsigned char *>(p);
    return FR_OK;
}

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

}  // namespace
}  // namespace fr

using namespace fr;

extern "C" int fr_grid_noalloc(const float *d_traj, size_t n, int dim, unsigned grid_size, float kernel_width,
                               const float *lut_host, int lut_length, const float *d_kdata, const float *d_dcf,
                               int channels, float *d_grid, void *stream)
{
    // ---- arguments (host only, before touching the GPU) ----
    if (dim != 2 && dim != 3) return fail(FR_ERR_INVALID_ARGUMENT, "dim must be 2 or 3");
    if (grid_size < 1 || grid_size > 4096) return fail(FR_ERR_UNSUPPORTED, "grid size must be in [1, 4096]");
    if (!(kernel_width > 0.f) || kernel_width > 13.f) return fail(FR_ERR_UNSUPPORTED, "kernel width must be in (0, 13]");
    if (!lut_host || lut_length < 2) return fail(FR_ERR_INVALID_ARGUMENT, "lut must have at least 2 entries");
    if (lut_length > FR_NOALLOC_MAX_LUT)
        return fail(FR_ERR_CAPACITY, "fr_grid_noalloc: lut_length above FR_NOALLOC_MAX_LUT (1024)");
    if (channels < 1) return fail(FR_ERR_INVALID_ARGUMENT, "channels must be positive");
    if (!d_grid || (n && (!d_traj || !d_kdata || !d_dcf))) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    if ((reinterpret_cast<uintptr_t>(d_traj) & 15) || (reinterpret_cast<uintptr_t>(d_kdata) & 7) ||
        (reinterpret_cast<uintptr_t>(d_grid) & 7))
        return fail(FR_ERR_INVALID_ARGUMENT, "trajectory must be 16-byte and complex buffers 8-byte aligned");
    if (n > 0xFFFFFFFFull) return fail(FR_ERR_UNSUPPORTED, "more than 2^32-1 samples");

    int tile[3], cg = 4;
    while (cg < channels && cg < 16) cg <<= 1;
    default_tiling(dim, tile, &cg, channels);
    const unsigned G = grid_size;
    int ntile[3];
    long long ntiles = 1, K = 1;
    for (int d = 0; d < 3; ++d) {
        const unsigned gd = d < dim ? G : 1u;
        ntile[d] = (int)((gd + tile[d] - 1) / tile[d]);
        ntiles *= ntile[d];
        K *= tile[d];
    }
    const int L = lut_length;
    const int R = floats_per_cell(cg);
    if (grid_smem_bytes(K, R, L) > 227 * 1024) return fail(FR_ERR_UNSUPPORTED, "tile does not fit in shared memory");
    const long long nblocks = plan_scan_blocks(ntiles);

    // fixed part of the scratch layout
    const size_t off_lut = 0;
    const size_t off_bounds = align256(off_lut + (size_t)L * 16);
    const size_t off_traj = align256(off_bounds + 32 * 4);
    const size_t off_count = align256(off_traj + std::max<size_t>(n, 1) * 16);
    const long long nstripes = ntiles * plan_stripes();
    const size_t off_fill = align256(off_count + (size_t)ntiles * 4);
    const size_t off_scount = align256(off_fill + (size_t)nstripes * 4);
    const size_t off_sbase = align256(off_scount + (size_t)nstripes * 4);
    const size_t off_scan = align256(off_sbase + (size_t)nstripes * 8);
    const size_t off_sblk = align256(off_scan + (size_t)(ntiles + 1) * sizeof(TileScan));
    const size_t off_rest = align256(off_sblk + (size_t)nblocks * sizeof(TileScan));
    if (off_rest > FR_NOALLOC_SCRATCH_BYTES)
        return fail(FR_ERR_CAPACITY, "fr_grid_noalloc: trajectory and tile tables exceed the 32 MiB "
                                     "FR_NOALLOC_SCRATCH_BYTES scratch; use fr_plan_create/fr_grid");

    unsigned char *scratch = nullptr;
    int st = scratch_on_current_device(&scratch);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;

    // exact LUT index entries {thr[k+1], lut[k], lut[k+1], 0}, built on the stack
    const float hw = kernel_width / 2;
    float thr[FR_NOALLOC_MAX_LUT + 1];
    float4 ent[FR_NOALLOC_MAX_LUT];
    float smax = 0.f, kc = 0.f;
    lut_index_table_into(hw, L, thr, &smax, &kc);
    for (int k = 0; k < L; ++k)
        ent[k] = make_float4(thr[k + 1], lut_host[k], k + 1 < L ? lut_host[k + 1] : 0.f, 0.f);
    FR_CUDA(cudaMemcpyAsync(scratch + off_lut, ent, (size_t)L * 16, cudaMemcpyHostToDevice, s));

    PlanInto pi;
    pi.dim = dim;
    pi.G = G;
    pi.hw = hw;
    {
        const float h2 = hw * hw;  // |x - c| >= kHW excludes a tap exactly when kHW^2 and its sqrt are exact
        pi.prefilter = (std::sqrt(h2) == hw) && ((double)h2 == (double)hw * (double)hw);
    }
    for (int d = 0; d < 3; ++d) {
        pi.tile[d] = tile[d];
        pi.ntile[d] = ntile[d];
    }
    pi.ntiles = ntiles;
    pi.chunk = plan_chunk(n, dim);
    pi.bounds = reinterpret_cast<int *>(scratch + off_bounds);
    pi.traj = reinterpret_cast<float4 *>(scratch + off_traj);
    pi.tile_count = reinterpret_cast<int *>(scratch + off_count);
    pi.tile_fill = reinterpret_cast<int *>(scratch + off_fill);
    pi.stripe_count = reinterpret_cast<int *>(scratch + off_scount);
    pi.stripe_base = reinterpret_cast<long long *>(scratch + off_sbase);
    pi.scan = reinterpret_cast<TileScan *>(scratch + off_scan);
    pi.scan_blocks = reinterpret_cast<TileScan *>(scratch + off_sblk);
    pi.rest = scratch + off_rest;
    pi.rest_bytes = FR_NOALLOC_SCRATCH_BYTES - off_rest;
    PlanIntoOut po;
    st = plan_into(pi, d_traj, n, s, &po);
    if (st) return st;

    const size_t off_part = align256(po.rest_used);
    const size_t part_b = po.nslots > 0 ? grid_partials_bytes(po.nslots, channels, cg, K) : 0;
    if (off_part + part_b > pi.rest_bytes)
        return fail(FR_ERR_CAPACITY, "fr_grid_noalloc: partial tiles of this trajectory exceed the 32 MiB "
                                     "FR_NOALLOC_SCRATCH_BYTES scratch; use fr_plan_create/fr_grid");
    GridInto gi;
    gi.dim = dim;
    gi.G = G;
    for (int d = 0; d < 3; ++d) {
        gi.tile[d] = tile[d];
        gi.ntile[d] = ntile[d];
    }
    gi.coil_group = cg;
    gi.L = L;
    gi.smax = smax;
    gi.kc = kc;
    gi.lut_absmax = 0.f;
    for (int k = 0; k < L; ++k) gi.lut_absmax = std::max(gi.lut_absmax, std::fabs(lut_host[k]));
    if (!(gi.lut_absmax > 0.f) || !std::isfinite(gi.lut_absmax)) gi.lut_absmax = 1.f;
    gi.traj = pi.traj;
    gi.recs = po.recs;
    gi.items = po.items;
    gi.splits = po.splits;
    gi.lut_e = reinterpret_cast<const float4 *>(scratch + off_lut);
    gi.nitems = po.nitems;
    gi.nsplits = po.nsplits;
    gi.n = n;
    gi.partials = reinterpret_cast<float *>(pi.rest + off_part);
    return grid_into(gi, d_kdata, d_dcf, channels, d_grid, s);
}
