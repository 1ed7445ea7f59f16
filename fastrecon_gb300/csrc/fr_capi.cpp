// fr_capi.cpp -- the C ABI of libfastrecon_gb300.so (include/fastrecon_gb300.h).
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>

#include "fr_internal.h"

namespace fr {

static thread_local std::string g_last_error;
static std::atomic<long long> g_launches{0};

void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int fail(int status, const std::string &msg)
{
    g_last_error = msg;
    return status;
}

int cuda_fail(cudaError_t e, const char *what)
{
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return FR_ERR_OUT_OF_MEMORY;
    return FR_ERR_CUDA;
}

DevBuf::~DevBuf() { release(); }

void DevBuf::release()
{
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}

// Host-side fault injection for the out-of-memory paths: with
// FR_FAIL_ALLOC_BYTES=B in the environment, every device reservation of B
// bytes or more fails as cudaMalloc would (nothing is allocated).
static bool injected_alloc_failure(size_t want)
{
    const char *v = std::getenv("FR_FAIL_ALLOC_BYTES");
    if (!v || !*v) return false;
    const unsigned long long b = std::strtoull(v, nullptr, 10);
    return b > 0 && want >= b;
}

int DevBuf::reserve(size_t n)
{
    if (n <= bytes && ptr) return 0;
    release();
    size_t want = std::max<size_t>(n, 256);
    if (injected_alloc_failure(want)) {
        fail(FR_ERR_OUT_OF_MEMORY, "device allocation refused (FR_FAIL_ALLOC_BYTES)");
        return 1;
    }
    cudaError_t e = cudaMalloc(&ptr, want);
    if (e != cudaSuccess) {
        ptr = nullptr;
        cuda_fail(e, "cudaMalloc");
        return 1;
    }
    bytes = want;
    return 0;
}

// Modified Bessel I0 by its power series (Abramowitz & Stegun 9.6.12);
// the reference calls GSL's gsl_sf_bessel_I0 (ConvKernel.cpp:23).
static double bessel_i0(double x)
{
    if (std::isnan(x)) return x;
    double q = 0.25 * x * x, term = 1.0, sum = 1.0;
    for (int k = 1; k < 1000; ++k) {
        term *= q / ((double)k * (double)k);
        sum += term;
        if (term < sum * 1e-18) break;
    }
    return sum;
}

// GridLut.cpp:131-136 on the host: dk = sqrtf(s), valid iff dk < kHW,
// index roundf(dk / kHW * (L-1)).  volatile keeps each float rounding.
int lut_reference_index(float s, float hw, int L)
{
    volatile float dk = std::sqrt(s);
    if (!(dk < hw)) return -1;
    volatile float q = dk / hw;
    volatile float t = q * (float)(L - 1);
    return (int)std::round((float)t);
}

static inline unsigned fbits(float f)
{
    unsigned u;
    std::memcpy(&u, &f, 4);
    return u;
}
static inline float bitsf(unsigned u)
{
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

LutIndexTable lut_index_table(float hw, int L)
{
    LutIndexTable t;
    // non-negative floats are ordered like their bit patterns
    unsigned lo = 0, hi = fbits(std::max(4.f * hw * hw, 1.f));
    while (lo < hi) {  // smallest s with !(sqrtf(s) < hw)
        unsigned mid = lo + (hi - lo) / 2;
        if (lut_reference_index(bitsf(mid), hw, L) < 0)
            hi = mid;
        else
            lo = mid + 1;
    }
    t.smax = bitsf(lo);
    const unsigned top = lo;  // all valid s are below bitsf(top)
    t.thr.assign(L + 1, INFINITY);
    t.thr[0] = 0.f;
    for (int k = 1; k < L; ++k) {
        unsigned a = 0, b = top;  // smallest s < smax with ki(s) >= k, else +inf
        while (a < b) {
            unsigned mid = a + (b - a) / 2;
            if (lut_reference_index(bitsf(mid), hw, L) >= k)
                b = mid;
            else
                a = mid + 1;
        }
        t.thr[k] = a < top ? bitsf(a) : INFINITY;
    }
    t.kc = (float)(L - 1) / hw;
    return t;
}

void lut_index_table_into(float hw, int L, float *thr, float *smax, float *kc)
{
    unsigned lo = 0, hi = fbits(std::max(4.f * hw * hw, 1.f));
    while (lo < hi) {
        unsigned mid = lo + (hi - lo) / 2;
        if (lut_reference_index(bitsf(mid), hw, L) < 0)
            hi = mid;
        else
            lo = mid + 1;
    }
    const unsigned top = lo;
    thr[0] = 0.f;
    for (int k = 1; k <= L; ++k) thr[k] = INFINITY;
    for (int k = 1; k < L; ++k) {
        unsigned a = 0, b = top;
        while (a < b) {
            unsigned mid = a + (b - a) / 2;
            if (lut_reference_index(bitsf(mid), hw, L) >= k)
                b = mid;
            else
                a = mid + 1;
        }
        thr[k] = a < top ? bitsf(a) : INFINITY;
    }
    *smax = bitsf(top);
    *kc = (float)(L - 1) / hw;
}

}  // namespace fr

fr_plan_s::~fr_plan_s()
{
    for (auto e : prof_ev) cudaEventDestroy(e);
    if (err_host) cudaFreeHost(err_host);
}

using namespace fr;

extern "C" {

const char *fr_status_string(int status)
{
    switch (status) {
    case FR_OK: return "ok";
    case FR_ERR_INVALID_ARGUMENT: return "invalid argument";
    case FR_ERR_SIZE_MISMATCH: return "size mismatch";
    case FR_ERR_OUT_OF_MEMORY: return "out of memory";
    case FR_ERR_CUDA: return "CUDA error";
    case FR_ERR_CUFFT: return "cuFFT error";
    case FR_ERR_NOT_PLANNED: return "not planned";
    case FR_ERR_UNSUPPORTED: return "unsupported";
    case FR_ERR_DEVICE_TIMEOUT: return "device wait timed out";
    case FR_ERR_CAPACITY: return "capacity exceeded";
    }
    return "unknown status";
}

const char *fr_last_error(void) { return g_last_error.c_str(); }

const char *fr_version(void) { return "fastrecon_gb300 0.1 (sm_103a)"; }

// ConvKernel::ConvKernel (ConvKernel.cpp:7-30): the same float/double mix.
int fr_kb_lut(float kWidth, float overGridFactor, int length, float *out)
{
    if (length < 2 || !out) return fail(FR_ERR_INVALID_ARGUMENT, "lut length must be >= 2");
    float w = kWidth, a = overGridFactor;
    float wa = w * w / (a * a);
    float beta = (float)(M_PI * std::sqrt((double)wa * ((double)a - 0.5) * ((double)a - 0.5) - 0.8));
    float dk = (float)((double)w / 2.0 / (double)(length - 1));
    volatile float kernel0 = 1;  // volatile: keep the float rounding of each step
    for (int i = 0; i < length; i++) {
        volatile float k = dk * (float)i;
        volatile float r = 2 * k / w;
        double x = (double)beta * std::sqrt(1 - (double)r * (double)r);
        out[i] = (float)(bessel_i0(x) / (double)w);
        if (i == 0) kernel0 = out[0];
        out[i] = out[i] / kernel0;
    }
    return FR_OK;
}

int fr_lut_index_table(float kernel_width, int length, float *thresholds, float *smax, float *kc)
{
    if (!(kernel_width > 0.f) || length < 2 || !thresholds)
        return fail(FR_ERR_INVALID_ARGUMENT, "bad lut index table arguments");
    LutIndexTable t = lut_index_table(kernel_width / 2, length);
    std::memcpy(thresholds, t.thr.data(), sizeof(float) * (length + 1));
    if (smax) *smax = t.smax;
    if (kc) *kc = t.kc;
    return FR_OK;
}

int fr_plan_create(const fr_plan_desc *d, fr_plan *out)
{
    if (!d || !out) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    if (d->dim != 2 && d->dim != 3) return fail(FR_ERR_INVALID_ARGUMENT, "dim must be 2 or 3");
    if (d->grid_size < 1 || d->grid_size > 4096) return fail(FR_ERR_UNSUPPORTED, "grid size must be in [1, 4096]");
    if (!(d->kernel_width > 0.f) || d->kernel_width > 13.f)
        return fail(FR_ERR_UNSUPPORTED, "kernel width must be in (0, 13]");
    if (d->lut_length < 2 || d->lut_length > 16384 || !d->lut)
        return fail(FR_ERR_INVALID_ARGUMENT, "lut must have 2..16384 entries");
    auto p = new (std::nothrow) fr_plan_s;
    if (!p) return fail(FR_ERR_OUT_OF_MEMORY, "plan");
    cudaGetDevice(&p->device);
    p->dim = d->dim;
    p->G = d->grid_size;
    p->W = d->kernel_width;
    p->hw = d->kernel_width / 2;  // GridLut.cpp:86: float kHW = width / 2
    p->L = d->lut_length;
    p->lut.assign(d->lut, d->lut + d->lut_length);
    p->flags = d->flags;
    int tile[3] = {d->tile[0], d->tile[1], d->tile[2]};
    int cg = d->coil_group;
    int deft[3];
    default_tiling(p->dim, deft, &cg, 16);
    for (int i = 0; i < 3; ++i)
        if (tile[i] <= 0) tile[i] = deft[i];
    if (p->dim == 2) tile[2] = 1;
    if (cg != 4 && cg != 8 && cg != 16 && cg != 32) {
        delete p;
        return fail(FR_ERR_UNSUPPORTED, "coil group must be 4, 8, 16 or 32");
    }
    long long K = (long long)tile[0] * tile[1] * tile[2];
    int R = floats_per_cell(cg);
    size_t smem = grid_smem_bytes(K, R, p->L);
    if (smem > 227 * 1024) {
        delete p;
        return fail(FR_ERR_UNSUPPORTED, "tile x coil group does not fit in shared memory");
    }
    if (tile[0] < 1 || tile[1] < 1 || tile[2] < 1 || tile[0] > 64 || tile[1] > 64 || tile[2] > 64 ||
        tile[0] % (32 / std::min(R, 32)) != 0) {
        delete p;
        return fail(FR_ERR_UNSUPPORTED,
                    "tile extents must be 1..64 and x a multiple of 32 / floats per cell");
    }
    p->coil_group = cg;
    p->ntiles = 1;
    for (int i = 0; i < 3; ++i) {
        p->tile[i] = tile[i];
        unsigned gi = (i < p->dim) ? p->G : 1u;
        p->ntile[i] = (int)((gi + tile[i] - 1) / tile[i]);
        p->ntiles *= p->ntile[i];
    }
    if (p->ntiles > (1ll << 30)) {
        delete p;
        return fail(FR_ERR_UNSUPPORTED, "too many tiles");
    }
    p->chunk_req = d->chunk > 0 ? d->chunk : 0;
    p->chunk = p->chunk_req > 0 ? p->chunk_req : 4096;
    {
        const char *cm = std::getenv("FR_KSPACE_COIL_MAJOR");
        p->kspace_sample_major = !(cm && std::atoi(cm) != 0);
        p->taps_enabled = !(d->flags & FR_PLAN_NO_TAP_LISTS);
        const char *wl = std::getenv("FR_SCATTER_WARP_LISTS");
        p->scatter_warp_lists = wl && std::atoi(wl) != 0;
    }
    {
        // exact when hw^2 is representable and sqrt rounds back to hw
        float h2 = p->hw * p->hw;
        p->prefilter = (std::sqrt(h2) == p->hw) && ((double)h2 == (double)p->hw * (double)p->hw);
    }
    // Device LUT entries {thr[k+1], lut[k], lut[k+1], 0}: the exact LUT
    // index and weight from s = dk^2 without a square root (LutIndexTable).
    {
        LutIndexTable lt = lut_index_table(p->hw, p->L);
        p->lut_smax = lt.smax;
        p->lut_kc = lt.kc;
        p->lut_absmax = 0.f;
        for (float v : p->lut) p->lut_absmax = std::max(p->lut_absmax, std::fabs(v));
        if (!(p->lut_absmax > 0.f) || !std::isfinite(p->lut_absmax)) p->lut_absmax = 1.f;
        p->lut_entries.resize(4 * (size_t)p->L);
        for (int k = 0; k < p->L; ++k) {
            p->lut_entries[4 * k + 0] = lt.thr[k + 1];
            p->lut_entries[4 * k + 1] = p->lut[k];
            p->lut_entries[4 * k + 2] = k + 1 < p->L ? p->lut[k + 1] : 0.f;
            p->lut_entries[4 * k + 3] = 0.f;
        }
    }
    if (p->lut_d.reserve((size_t)p->L * 4) || p->lut_e.reserve((size_t)p->L * 16)) {
        delete p;
        return FR_ERR_OUT_OF_MEMORY;
    }
    cudaError_t e = cudaMemcpy(p->lut_e.ptr, p->lut_entries.data(), (size_t)p->L * 16, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(p->lut_d.ptr, p->lut.data(), (size_t)p->L * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        delete p;
        return cuda_fail(e, "lut upload");
    }
    // a word the kernels set on an internal error, read by the host without a copy
    e = cudaHostAlloc(reinterpret_cast<void **>(&p->err_host), sizeof(int), cudaHostAllocMapped);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer(reinterpret_cast<void **>(&p->err_dev), p->err_host, 0);
    if (e != cudaSuccess) {
        delete p;
        return cuda_fail(e, "error word");
    }
    *p->err_host = 0;
    *out = p;
    return FR_OK;
}

int fr_plan_destroy(fr_plan p)
{
    delete p;
    return FR_OK;
}

int fr_plan_set_trajectory(fr_plan p, const float *d_traj, size_t n, void *stream)
{
    if (!p || (!d_traj && n)) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    return plan_run(p, d_traj, n, (cudaStream_t)stream);
}

int fr_plan_normalized_trajectory(fr_plan p, float *d_out, void *stream)
{
    if (!p || !d_out) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    if (!p->planned) return fail(FR_ERR_NOT_PLANNED, "no trajectory");
    if (p->n == 0) return FR_OK;
    FR_CUDA(cudaMemcpyAsync(d_out, p->traj.ptr, p->n * 16, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
    return FR_OK;
}

int fr_plan_bounds(fr_plan p, float *raw_lo, float *raw_hi, float *norm_lo, float *norm_hi)
{
    if (!p) return fail(FR_ERR_INVALID_ARGUMENT, "null plan");
    if (!p->planned) return fail(FR_ERR_NOT_PLANNED, "no trajectory");
    for (int i = 0; i < 3; ++i) {
        if (raw_lo) raw_lo[i] = p->bounds_host[i];
        if (raw_hi) raw_hi[i] = p->bounds_host[3 + i];
        if (norm_lo) norm_lo[i] = p->bounds_host[6 + i];
        if (norm_hi) norm_hi[i] = p->bounds_host[9 + i];
    }
    return FR_OK;
}

int fr_plan_sample_ranges(fr_plan p, int *d_start, int *d_end, void *stream)
{
    if (!p || !d_start || !d_end) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    if (!p->planned) return fail(FR_ERR_NOT_PLANNED, "no trajectory");
    return sample_ranges_run(p, d_start, d_end, (cudaStream_t)stream);
}

int fr_plan_stats(fr_plan p, long long *tiles, long long *pairs, long long *items, long long *slots)
{
    if (!p) return fail(FR_ERR_INVALID_ARGUMENT, "null plan");
    if (tiles) *tiles = p->ntiles;
    if (pairs) *pairs = p->npairs;
    if (items) *items = p->nitems;
    if (slots) *slots = p->nslots;
    return FR_OK;
}

int fr_plan_tap_words(fr_plan p, int *words)
{
    if (!p || !words) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    *words = p->planned ? p->tap_words : 0;
    return FR_OK;
}

int fr_plan_bins(fr_plan p, long long *d_tile_offset, unsigned *d_pairs, void *stream)
{
    if (!p || !d_tile_offset || !d_pairs) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    if (!p->planned) return fail(FR_ERR_NOT_PLANNED, "no trajectory");
    cudaStream_t s = (cudaStream_t)stream;
    // tile offsets are the .pairs field of the exclusive TileScan
    FR_CUDA(cudaMemcpy2DAsync(d_tile_offset, sizeof(long long), p->tile_scan.ptr, sizeof(TileScan),
                              sizeof(long long), (size_t)p->ntiles + 1, cudaMemcpyDeviceToDevice, s));
    if (p->npairs)  // the sample index is the low word of each 8-byte record
        FR_CUDA(cudaMemcpy2DAsync(d_pairs, 4, p->pairs.ptr, 8, 4, (size_t)p->npairs, cudaMemcpyDeviceToDevice, s));
    return FR_OK;
}

int fr_plan_profile(fr_plan p, int enable)
{
    if (!p) return fail(FR_ERR_INVALID_ARGUMENT, "null plan");
    p->profile = enable != 0;
    p->prof_used = 0;
    return FR_OK;
}

int fr_plan_profile_read(fr_plan p, double *ms, int *launches)
{
    if (!p) return fail(FR_ERR_INVALID_ARGUMENT, "null plan");
    double total = 0;
    if (p->prof_used > 0) FR_CUDA(cudaEventSynchronize(p->prof_ev[p->prof_used * 2 - 1]));
    for (int i = 0; i < p->prof_used; ++i) {
        float t = 0;
        FR_CUDA(cudaEventElapsedTime(&t, p->prof_ev[2 * i], p->prof_ev[2 * i + 1]));
        total += t;
    }
    if (ms) *ms = total;
    if (launches) *launches = p->prof_used;
    p->prof_used = 0;
    return FR_OK;
}

long long fr_kernel_launches(void) { return g_launches.load(); }

int fr_grid(fr_plan p, const float *d_kdata, const float *d_dcf, int channels, float *d_grid, void *stream)
{
    if (!p || !d_grid || (p->n && (!d_kdata || !d_dcf))) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    if ((reinterpret_cast<uintptr_t>(d_kdata) & 7) || (reinterpret_cast<uintptr_t>(d_grid) & 7))
        return fail(FR_ERR_INVALID_ARGUMENT, "complex buffers must be 8-byte aligned");
    return grid_run(p, d_kdata, d_dcf, channels, d_grid, (cudaStream_t)stream);
}

int fr_grid_partitioned(const fr_plan_desc *desc, const float *d_traj, size_t n, const float *d_kdata,
                        const float *d_dcf, int channels, float *d_grid, size_t partition, void *stream)
{
    if (!desc || !d_grid || (n && (!d_traj || !d_kdata || !d_dcf)) || channels < 1)
        return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    if (desc->dim != 2 && desc->dim != 3) return fail(FR_ERR_INVALID_ARGUMENT, "dim must be 2 or 3");
    if ((reinterpret_cast<uintptr_t>(d_kdata) & 7) || (reinterpret_cast<uintptr_t>(d_grid) & 7))
        return fail(FR_ERR_INVALID_ARGUMENT, "complex buffers must be 8-byte aligned");
    if (reinterpret_cast<uintptr_t>(d_traj) & 15) return fail(FR_ERR_INVALID_ARGUMENT, "trajectory must be 16-byte aligned");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t G = desc->grid_size;
    const size_t cells = desc->dim == 3 ? G * G * G : G * G;
    if (partition == 0 || partition > n) partition = n;

    const bool prenormalized = (desc->flags & FR_PLAN_PRENORMALIZED) != 0;
    fr_plan_desc d = *desc;
    d.flags |= FR_PLAN_PRENORMALIZED | FR_PLAN_ACCUMULATE;
    fr_plan plan = nullptr;
    int st = fr_plan_create(&d, &plan);
    if (st) return st;
    float *tn = nullptr;
    if (n && !prenormalized) {
        if (cudaMallocAsync(reinterpret_cast<void **>(&tn), n * 4 * sizeof(float), s) != cudaSuccess) {
            cudaGetLastError();
            fr_plan_destroy(plan);
            return fail(FR_ERR_OUT_OF_MEMORY, "normalised trajectory");
        }
        // the whole trajectory's bounds, as one plan would take them
        st = fr_normalize_trajectory(d_traj, n, desc->dim, desc->grid_size, tn, nullptr, stream);
    }
    const float *traj = prenormalized ? d_traj : tn;
    if (!st && cudaMemsetAsync(d_grid, 0, (size_t)channels * cells * 2 * sizeof(float), s) != cudaSuccess)
        st = fail(FR_ERR_CUDA, "grid memset");
    for (size_t b = 0; !st && b < n; b += partition) {
        const size_t m = std::min(partition, n - b);
        st = fr_plan_set_trajectory(plan, traj + 4 * b, m, stream);
        if (!st) st = grid_run(plan, d_kdata + 2 * b, d_dcf + b, channels, d_grid, s, false, n);
    }
    if (tn) cudaFreeAsync(tn, s);
    fr_plan_destroy(plan);
    return st;
}

// --------------------------------------------------------------------------
// Density compensation and degridding
// --------------------------------------------------------------------------

int fr_dcf_analytic(const float *d_traj, size_t n, int dim, float power, float *d_dcf, void *stream)
{
    if (dim < 1 || dim > 3) return fail(FR_ERR_INVALID_ARGUMENT, "dim must be 1, 2 or 3");
    if (n && (!d_traj || !d_dcf)) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    if (reinterpret_cast<uintptr_t>(d_traj) & 15) return fail(FR_ERR_INVALID_ARGUMENT, "trajectory must be 16-byte aligned");
    if (!(power >= 0.f)) return fail(FR_ERR_INVALID_ARGUMENT, "power must be >= 0");
    return dcf_analytic_run(d_traj, n, dim, power, d_dcf, (cudaStream_t)stream);
}

int fr_degrid(fr_plan p, const float *d_grid, int channels, float *d_kdata, void *stream)
{
    if (!p || (p->n && (!d_grid || !d_kdata))) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    if ((reinterpret_cast<uintptr_t>(d_grid) & 7) || (reinterpret_cast<uintptr_t>(d_kdata) & 7))
        return fail(FR_ERR_INVALID_ARGUMENT, "complex buffers must be 8-byte aligned");
    return degrid_run(p, d_grid, channels, d_kdata, (cudaStream_t)stream);
}

int fr_grid_update(fr_plan p, float *d_kdata, const float *d_new, size_t sample_begin, size_t count,
                   const float *d_dcf, int channels, float *d_grid, void *stream)
{
    if (!p || (count && (!d_kdata || !d_new || !d_dcf || !d_grid))) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    if ((reinterpret_cast<uintptr_t>(d_kdata) & 7) || (reinterpret_cast<uintptr_t>(d_new) & 7) ||
        (reinterpret_cast<uintptr_t>(d_grid) & 7))
        return fail(FR_ERR_INVALID_ARGUMENT, "complex buffers must be 8-byte aligned");
    return grid_update_run(p, d_kdata, d_new, sample_begin, count, d_dcf, channels, d_grid, (cudaStream_t)stream);
}

int fr_grid_real(fr_plan p, const float *d_w, float *d_grid, void *stream)
{
    if (!p || !d_grid || (p->n && !d_w)) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    return grid_real_run(p, d_w, d_grid, (cudaStream_t)stream);
}

int fr_dcf_pipe(fr_plan p, int iterations, float *d_dcf, void *stream)
{
    if (!p || (p->n && !d_dcf)) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    return dcf_pipe_run(p, iterations, d_dcf, (cudaStream_t)stream);
}

// --------------------------------------------------------------------------
// Learned DCF: density features and the network
// --------------------------------------------------------------------------

int fr_density_counts(fr_plan p, const int *radii, int nradii, int *d_counts, void *stream)
{
    if (!p || (p->n && !d_counts)) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    return density_counts_run(p, radii, nradii, d_counts, (cudaStream_t)stream);
}

int fr_dcf_features(fr_plan p, const int *d_counts, const float *d_raw_traj, const int *radii, int nradii, float kmax,
                    float *d_features, void *stream)
{
    if (!p || (p->n && (!d_counts || !d_raw_traj || !d_features))) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    if (reinterpret_cast<uintptr_t>(d_raw_traj) & 15) return fail(FR_ERR_INVALID_ARGUMENT, "trajectory must be 16-byte aligned");
    if (p->small.reserve(256)) return FR_ERR_CUDA;
    return dcf_features_run(d_counts, d_raw_traj, p->n, p->dim, radii, nradii, kmax, d_features,
                            p->small.as<unsigned>(), (cudaStream_t)stream);
}

int fr_mlp_forward(const void *d_params, const float *d_features, size_t n, unsigned flags, float scale, float *d_out,
                   void *stream)
{
    if (n && (!d_params || !d_features || !d_out)) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    if (reinterpret_cast<uintptr_t>(d_params) & 1) return fail(FR_ERR_INVALID_ARGUMENT, "parameters must be 2-byte aligned");
    return mlp_forward_run(d_params, d_features, n, (flags & FR_MLP_EXP) ? 1 : 0, (flags & FR_MLP_RESIDUAL) ? 1 : 0,
                           scale, d_out, (cudaStream_t)stream);
}

size_t fr_mlp_workspace_bytes(size_t n) { return mlp_workspace_bytes(n); }

int fr_mlp_backward(const void *d_params, const float *d_features, const float *d_target, const float *d_weight,
                    size_t n, void *d_workspace, float *d_grad, float *d_loss, void *stream)
{
    if (!d_params || !d_features || !d_target || !d_workspace || !d_grad)
        return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    if (reinterpret_cast<uintptr_t>(d_workspace) & 15) return fail(FR_ERR_INVALID_ARGUMENT, "workspace must be 16-byte aligned");
    return mlp_backward_run(d_params, d_features, d_target, d_weight, n, d_workspace, d_grad, d_loss,
                            (cudaStream_t)stream);
}

int fr_mlp_adam(float *d_master, void *d_params, const float *d_grad, float *d_m, float *d_v, int count, float lr,
                float beta1, float beta2, float eps, int step, void *stream)
{
    if (!d_master || !d_params || !d_grad || !d_m || !d_v) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    return mlp_adam_run(d_master, d_params, d_grad, d_m, d_v, count, lr, beta1, beta2, eps, step, (cudaStream_t)stream);
}

int fr_mlp_to_bf16(const float *d_master, void *d_params, int count, void *stream)
{
    if (count > 0 && (!d_master || !d_params)) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    return to_bf16_run(d_master, d_params, count, (cudaStream_t)stream);
}

// --------------------------------------------------------------------------
// cuFFT stage
// --------------------------------------------------------------------------

struct fr_fft_s {
    cufftHandle h = 0;
    int sign = CUFFT_INVERSE;
    size_t elems = 0;
};

int fr_fft_create(int dim, const unsigned *size, int batch, int sign, fr_fft *out)
{
    if (!out || !size || (dim != 2 && dim != 3) || batch < 1)
        return fail(FR_ERR_INVALID_ARGUMENT, "bad fft arguments");
    *out = nullptr;
    auto f = new (std::nothrow) fr_fft_s;
    if (!f) return fail(FR_ERR_OUT_OF_MEMORY, "fft");
    // Layout x fastest: cuFFT wants the slowest dimension first.
    long long n[3];
    if (dim == 3) {
        n[0] = size[2];
        n[1] = size[1];
        n[2] = size[0];
    } else {
        n[0] = size[1];
        n[1] = size[0];
    }
    long long dist = (long long)size[0] * size[1] * (dim == 3 ? size[2] : 1);
    cufftResult r = cufftCreate(&f->h);
    size_t work = 0;
    if (r == CUFFT_SUCCESS)
        r = cufftMakePlanMany64(f->h, dim, n, nullptr, 1, dist, nullptr, 1, dist, CUFFT_C2C, batch, &work);
    if (r != CUFFT_SUCCESS) {
        if (f->h) cufftDestroy(f->h);
        delete f;
        return fail(FR_ERR_CUFFT, "cufftMakePlanMany64 failed (" + std::to_string((int)r) + ")");
    }
    // FFTW_BACKWARD (+1) == CUFFT_INVERSE (cuImageFilter.cpp:27-31)
    f->sign = sign > 0 ? CUFFT_INVERSE : CUFFT_FORWARD;
    f->elems = (size_t)dist * batch;
    *out = f;
    return FR_OK;
}

int fr_fft_execute(fr_fft f, float *d_data, void *stream)
{
    if (!f || !d_data) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    cufftResult r = cufftSetStream(f->h, (cudaStream_t)stream);
    if (r == CUFFT_SUCCESS)
        r = cufftExecC2C(f->h, reinterpret_cast<cufftComplex *>(d_data), reinterpret_cast<cufftComplex *>(d_data),
                         f->sign);
    if (r != CUFFT_SUCCESS) return fail(FR_ERR_CUFFT, "cufftExecC2C failed (" + std::to_string((int)r) + ")");
    return FR_OK;
}

int fr_fft_destroy(fr_fft f)
{
    if (f) {
        cufftDestroy(f->h);
        delete f;
    }
    return FR_OK;
}

int fr_fft_shift(float *d_imgs, int channels, int dim, const unsigned *size, void *stream)
{
    if (!d_imgs || !size || channels < 1 || (dim != 2 && dim != 3))
        return fail(FR_ERR_INVALID_ARGUMENT, "bad shift arguments");
    return shift_run(d_imgs, channels, dim, size, (cudaStream_t)stream);
}

int fr_crop(const float *d_imgs, int channels, int dim, const unsigned *size, const unsigned *crop, float *d_out,
            void *stream)
{
    if (!d_imgs || !d_out || !size || !crop || channels < 1 || (dim != 2 && dim != 3))
        return fail(FR_ERR_INVALID_ARGUMENT, "bad crop arguments");
    return crop_run(d_imgs, channels, dim, size, crop, d_out, (cudaStream_t)stream);
}

int fr_sos(const float *d_imgs, int channels, int dim, const unsigned *size, const unsigned *recon,
           const float *d_deapod, float *d_out, void *stream)
{
    if (!d_imgs || !d_out || !size || !recon || channels < 1 || (dim != 2 && dim != 3))
        return fail(FR_ERR_INVALID_ARGUMENT, "bad sos arguments");
    return sos_run(d_imgs, channels, dim, size, recon, d_deapod, d_out, (cudaStream_t)stream);
}

int fr_normalize_trajectory(const float *d_traj, size_t n, int dim, unsigned grid_size, float *d_out,
                            float *bounds12, void *stream)
{
    if ((n && (!d_traj || !d_out)) || (dim != 2 && dim != 3) || grid_size < 1)
        return fail(FR_ERR_INVALID_ARGUMENT, "bad normalize arguments");
    return normalize_run(d_traj, n, dim, grid_size, d_out, bounds12, (cudaStream_t)stream);
}

int fr_transform_trajectory(float *d_traj, size_t n, int dim, float translation, float scale, void *stream)
{
    if ((n && !d_traj) || dim < 1 || dim > 3) return fail(FR_ERR_INVALID_ARGUMENT, "bad transform arguments");
    return transform_run(d_traj, n, dim, translation, scale, (cudaStream_t)stream);
}

int fr_real_to_complex(const float *d_in, size_t n, float *d_out, void *stream)
{
    if (n && (!d_in || !d_out)) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    return real_to_complex_run(d_in, n, d_out, (cudaStream_t)stream);
}

int fr_low_filter(float *d_imgs, int channels, int dim, const unsigned *size, int res, void *stream)
{
    if (!d_imgs || !size || channels < 1 || (dim != 2 && dim != 3))
        return fail(FR_ERR_INVALID_ARGUMENT, "bad low filter arguments");
    // ImageFilter.cpp:62-68: att = 2 res^2 / 4 (double, stored float) and
    // coeff[r] = expf(-r / 100.0) for r < 2000, evaluated on the host.
    float att = (float)(2.0 * res * res / 4.0);
    float coeff[2000];
    for (int r = 0; r < 2000; r++) coeff[r] = expf((float)(-r / 100.0));
    cudaStream_t s = (cudaStream_t)stream;
    float *d_coeff = nullptr;
    FR_CUDA(cudaMallocAsync(reinterpret_cast<void **>(&d_coeff), sizeof(coeff), s));
    FR_CUDA(cudaMemcpyAsync(d_coeff, coeff, sizeof(coeff), cudaMemcpyHostToDevice, s));
    int st = low_filter_run(d_imgs, channels, dim, size, att, d_coeff, s);
    cudaFreeAsync(d_coeff, s);
    // the host table must outlive the async copy
    FR_CUDA(cudaStreamSynchronize(s));
    return st;
}

int fr_normalize_channels(float *d_imgs, int channels, int dim, const unsigned *size, void *stream)
{
    if (!d_imgs || !size || channels < 1 || (dim != 2 && dim != 3))
        return fail(FR_ERR_INVALID_ARGUMENT, "bad normalize arguments");
    return normalize_channels_run(d_imgs, channels, dim, size, (cudaStream_t)stream);
}

int fr_sos_map(const float *d_imgs, const float *d_maps, int channels, int dim, const unsigned *size,
               const unsigned *recon, float *d_out, void *stream)
{
    if (!d_imgs || !d_maps || !d_out || !size || !recon || channels < 1 || (dim != 2 && dim != 3))
        return fail(FR_ERR_INVALID_ARGUMENT, "bad sos arguments");
    return sos_map_run(d_imgs, d_maps, channels, dim, size, recon, d_out, (cudaStream_t)stream);
}

}  // extern "C"
