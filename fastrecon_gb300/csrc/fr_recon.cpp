// fr_recon.cpp -- the whole reconstruction behind one object
// (Program/Main.cpp:101-181 without file I/O): normalise + bin the
// trajectory, grid every coil, backward FFT of all coils in one batched
// cuFFT call, crop + sum of squares (+ optional deapodization).
//
// With an even grid the fftShift of the reference (ImageFilter.cpp:40-53)
// is folded into the gridding flush as a (-1)^(x+y+z) modulation, so the
// FFT output is already shifted and no extra pass over the grid is needed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <new>

#include "fr_internal.h"

using namespace fr;

struct fr_recon_s {
    fr_recon_desc d;
    unsigned G = 0;
    size_t cells = 0;
    int slab = 0;            // coils gridded and transformed together (grid_budget)
    bool checkerboard = false;
    std::vector<float> lut;
    fr_plan plan = nullptr;
    fr_fft fft = nullptr;
    fr_fft fft1 = nullptr;  // single-image plan for the deapodization map
    fr_fftcs pruned = nullptr;  // pruned FFT + crop + SoS (even G)
    DevBuf grid;            // channels x G^d complex
    DevBuf deapod;          // out_size floats
    DevBuf h_traj, h_dcf, h_kdata, h_img;  // device staging for host-buffer runs
    bool deapod_ready = false;
    bool timing = false;
    cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    float stage_ms[4] = {-1, -1, -1, -1};
    // host-buffer runs: the k-space upload runs on its own stream while the
    // trajectory is planned
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t copy_start = nullptr, copy_done = nullptr;
    // the scatter's sample-major k-space copy is made on its own stream while
    // the plan's tap fill runs (one reads and writes HBM, the other computes)
    cudaStream_t prep_stream = nullptr;
    cudaEvent_t prep_start = nullptr, prep_done = nullptr;
    // submitted host-buffer volumes (fr_recon_submit_host): two staging
    // slots, so volume i + 1 uploads while volume i is reconstructed and
    // volume i - 1's image downloads
    struct Slot {
        DevBuf traj, dcf, kdata, img;
        cudaEvent_t uploaded = nullptr;    // inputs on the device
        cudaEvent_t consumed = nullptr;    // recon done with the inputs and wrote img
        cudaEvent_t downloaded = nullptr;  // img copied to the host
    } slot[2];
    int next_slot = 0;
    cudaStream_t up_stream = nullptr, down_stream = nullptr;
    ~fr_recon_s()
    {
        if (up_stream) cudaStreamSynchronize(up_stream);
        if (down_stream) cudaStreamSynchronize(down_stream);
        for (auto &sl : slot) {
            if (sl.consumed) cudaEventSynchronize(sl.consumed);
            for (cudaEvent_t e : {sl.uploaded, sl.consumed, sl.downloaded})
                if (e) cudaEventDestroy(e);
        }
        if (up_stream) cudaStreamDestroy(up_stream);
        if (down_stream) cudaStreamDestroy(down_stream);
        if (copy_start) cudaEventDestroy(copy_start);
        if (copy_done) cudaEventDestroy(copy_done);
        if (copy_stream) cudaStreamDestroy(copy_stream);
        if (prep_stream) cudaStreamSynchronize(prep_stream);
        if (prep_stream) cudaStreamDestroy(prep_stream);
        if (prep_start) cudaEventDestroy(prep_start);
        if (prep_done) cudaEventDestroy(prep_done);
        if (plan) fr_plan_destroy(plan);
        if (fft) fr_fft_destroy(fft);
        if (fft1) fr_fft_destroy(fft1);
        if (pruned) fr_fft_crop_sos_destroy(pruned);
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
    }
};

extern "C" {

int fr_recon_create(const fr_recon_desc *d, fr_recon *out)
{
    if (!d || !out) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    if (d->dim != 2 && d->dim != 3) return fail(FR_ERR_INVALID_ARGUMENT, "dim must be 2 or 3");
    if (d->channels < 1) return fail(FR_ERR_INVALID_ARGUMENT, "channels must be positive");
    auto r = new (std::nothrow) fr_recon_s;
    if (!r) return fail(FR_ERR_OUT_OF_MEMORY, "recon");
    r->d = *d;
    if (d->dim == 2) r->d.out_size[2] = 1;
    // GridLut.cpp:45: m_gridSize = unsigned(reconSize * overGridFactor)
    r->G = (unsigned)((float)d->recon_size * d->overgrid_factor);
    r->cells = d->dim == 3 ? (size_t)r->G * r->G * r->G : (size_t)r->G * r->G;
    r->checkerboard = (r->G % 2) == 0;
    r->slab = d->channels;
    if (d->grid_budget > 0) {
        const size_t per = r->cells * 8;
        r->slab = (int)std::max<size_t>(1, std::min<size_t>((size_t)d->channels, d->grid_budget / per));
    }
    r->lut.resize(d->lut_length > 1 ? d->lut_length : 2);
    int st = fr_kb_lut(d->kernel_width, d->overgrid_factor, d->lut_length, r->lut.data());
    if (st) {
        delete r;
        return st;
    }
    fr_plan_desc pd = {};
    pd.dim = d->dim;
    pd.grid_size = r->G;
    pd.kernel_width = d->kernel_width;
    pd.lut_length = d->lut_length;
    pd.lut = r->lut.data();
    for (int i = 0; i < 3; ++i) pd.tile[i] = d->tile[i];
    pd.coil_group = d->coil_group > 0 ? d->coil_group : 0;
    if (pd.coil_group == 0) {
        int cg = 4;
        while (cg < d->channels && cg < 16) cg <<= 1;
        pd.coil_group = cg;
    }
    pd.flags = (r->checkerboard ? FR_PLAN_CHECKERBOARD : 0) |
               ((d->flags & FR_RECON_DETERMINISTIC) ? FR_PLAN_DETERMINISTIC : 0);
    st = fr_plan_create(&pd, &r->plan);
    // the pruned transform with fused crop + SoS where it is specialised for
    // G (faster than cuFFT + SoS there), or when asked for
    const bool want_pruned = (d->flags & FR_RECON_PRUNED_FFT) || pruned_fft_specialised((int)r->G);
    if (!st && r->checkerboard && want_pruned && !(d->flags & FR_RECON_CUFFT)) {
        // the pruned transform where the grid size factors into 2, 3, 5
        if (fr_fft_crop_sos_create(d->dim, r->G, r->slab, r->d.out_size, &r->pruned) != FR_OK)
            r->pruned = nullptr;
    }
    if (!st && !r->pruned) {
        unsigned sz[3] = {r->G, r->G, d->dim == 3 ? r->G : 1u};
        st = fr_fft_create(d->dim, sz, r->slab, +1, &r->fft);
    }
    if (!st && r->grid.reserve(r->cells * 8 * (size_t)r->slab)) st = FR_ERR_OUT_OF_MEMORY;
    if (st) {
        delete r;
        return st;
    }
    const char *tm = std::getenv("FR_TIMING");
    r->timing = tm && tm[0] == '1';
    if (r->timing)
        for (auto &e : r->ev) cudaEventCreate(&e);
    *out = r;
    return FR_OK;
}

int fr_recon_destroy(fr_recon r)
{
    delete r;
    return FR_OK;
}

static int ensure_deapod(fr_recon r, cudaStream_t s)
{
    if (r->deapod_ready) return FR_OK;
    size_t nout = (size_t)r->d.out_size[0] * r->d.out_size[1] * r->d.out_size[2];
    if (r->deapod.reserve(nout * 4)) return FR_ERR_OUT_OF_MEMORY;
    if (!r->fft1) {
        unsigned sz[3] = {r->G, r->G, r->d.dim == 3 ? r->G : 1u};
        int st = fr_fft_create(r->d.dim, sz, 1, +1, &r->fft1);
        if (st) return st;
    }
    float *g = r->grid.as<float>();
    int st = deapod_seed_run(g, r->d.dim, (int)r->G, r->d.kernel_width / 2, r->plan->lut_d.as<float>(),
                             r->d.lut_length, r->checkerboard ? 1 : 0, s);
    if (!st) st = fr_fft_execute(r->fft1, g, s);
    unsigned sz[3] = {r->G, r->G, r->d.dim == 3 ? r->G : 1u};
    if (!st && !r->checkerboard) st = shift_run(g, 1, r->d.dim, sz, s);
    if (!st) st = deapod_map_run(g, r->d.dim, sz, r->d.out_size, r->deapod.as<float>(), s);
    if (!st) r->deapod_ready = true;
    return st;
}

}  // extern "C"

namespace {
// The recon of fr_recon_run; `kdata_ready` (if given) is waited for on the
// stream between planning and gridding.
int recon_run(fr_recon r, const float *d_traj, const float *d_dcf, const float *d_kdata, size_t n, float *d_image,
              cudaStream_t s, cudaEvent_t kdata_ready)
{
    void *stream = (void *)s;
    int st = FR_OK;
    if (r->d.flags & FR_RECON_DEAPODIZE) {
        st = ensure_deapod(r, s);
        if (st) return st;
    }
    unsigned sz[3] = {r->G, r->G, r->d.dim == 3 ? r->G : 1u};
    float *g = r->grid.as<float>();
    if (r->timing) cudaEventRecord(r->ev[0], s);
    st = fr_plan_set_trajectory(r->plan, d_traj, n, stream);
    // the first slab's sample-major k-space copy, on the side stream while
    // the plan's last kernels run on `s` (after everything before them)
    const int slab0 = std::min(r->slab, r->d.channels);
    if (!st && n > 0 && r->plan->tap_words > 0 && !r->timing) {
        if (!r->prep_stream) {
            FR_CUDA(cudaStreamCreateWithFlags(&r->prep_stream, cudaStreamNonBlocking));
            FR_CUDA(cudaEventCreateWithFlags(&r->prep_start, cudaEventDisableTiming));
            FR_CUDA(cudaEventCreateWithFlags(&r->prep_done, cudaEventDisableTiming));
        }
        FR_CUDA(cudaEventRecord(r->prep_start, s));
        FR_CUDA(cudaStreamWaitEvent(r->prep_stream, r->prep_start, 0));
        if (kdata_ready) FR_CUDA(cudaStreamWaitEvent(r->prep_stream, kdata_ready, 0));
        st = kspace_prepare(r->plan, d_kdata, d_dcf, slab0, r->prep_stream);
        if (!st) FR_CUDA(cudaEventRecord(r->prep_done, r->prep_stream));
        if (!st) FR_CUDA(cudaStreamWaitEvent(s, r->prep_done, 0));
    }
    if (r->timing) cudaEventRecord(r->ev[1], s);
    if (!st && kdata_ready) {
        cudaError_t e = cudaStreamWaitEvent(s, kdata_ready, 0);
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamWaitEvent");
    }
    const float *deapod = (r->d.flags & FR_RECON_DEAPODIZE) ? r->deapod.as<float>() : nullptr;
    // coils in slabs of r->slab (all at once unless grid_budget asks for
    // less): the first slab stores its sum of |x|^2, later slabs add to it in
    // coil order, the last applies sqrt (/ deapod).  With several slabs the
    // stage times are those of the first slab's gridding and of everything
    // after it.
    // The register FFT stages read the grid through the plan's tile bitmap,
    // so the scatter leaves tiles without samples unwritten (for the
    // kooshball about half the 384^3 grid: its corners).
    TileMask tm;
    const fr_plan p = r->plan;
    const bool pow2 = ((p->tile[0] | p->tile[1] | p->tile[2]) > 0) && !(p->tile[0] & (p->tile[0] - 1)) &&
                      !(p->tile[1] & (p->tile[1] - 1)) && !(p->tile[2] & (p->tile[2] - 1));
    const bool skip = r->pruned && fftcs_masks_tiles(r->pruned) && pow2;
    if (skip) {
        tm.bits = p->tile_mask.as<unsigned>();
        for (int i = 0; i < 3; ++i) {
            tm.tile[i] = p->tile[i];
            tm.ntile[i] = p->ntile[i];
        }
    }
    const int C = r->d.channels;
    for (int c0 = 0; !st && c0 < C; c0 += r->slab) {
        const int cs = std::min(r->slab, C - c0);
        const int mode = (c0 > 0 ? 1 : 0) | (c0 + cs == C ? 2 : 0);
        st = grid_run(r->plan, d_kdata + 2 * (size_t)c0 * n, d_dcf, cs, g, s, skip);
        if (r->timing && c0 == 0) cudaEventRecord(r->ev[2], s);
        if (r->pruned) {
            // transform, crop and SoS in one pruned pass (the stage times are
            // reported as fft, with sos 0)
            if (!st) st = fftcs_execute(r->pruned, g, cs, deapod, d_image, mode, s, skip ? &tm : nullptr);
            if (r->timing && c0 + cs == C) cudaEventRecord(r->ev[3], s);
        } else {
            if (!st) st = fr_fft_execute(r->fft, g, stream);
            if (!st && !r->checkerboard) st = shift_run(g, cs, r->d.dim, sz, s);
            if (r->timing && c0 + cs == C) cudaEventRecord(r->ev[3], s);
            if (!st) st = sos_run(g, cs, r->d.dim, sz, r->d.out_size, deapod, d_image, s, mode);
        }
    }
    if (r->timing) {
        cudaEventRecord(r->ev[4], s);
        cudaEventSynchronize(r->ev[4]);
        for (int i = 0; i < 4; ++i) cudaEventElapsedTime(&r->stage_ms[i], r->ev[i], r->ev[i + 1]);
    }
    return st;
}

}  // namespace

extern "C" {

int fr_recon_run(fr_recon r, const float *d_traj, const float *d_dcf, const float *d_kdata, size_t n,
                 float *d_image, void *stream)
{
    if (!r || !d_image || (n && (!d_traj || !d_dcf || !d_kdata)))
        return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    return recon_run(r, d_traj, d_dcf, d_kdata, n, d_image, (cudaStream_t)stream, nullptr);
}

int fr_recon_run_host(fr_recon r, const float *h_traj, const float *h_dcf, const float *h_kdata, size_t n,
                      float *h_image, void *stream)
{
    if (!r || !h_image || (n && (!h_traj || !h_dcf || !h_kdata)))
        return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    if (n > r->d.max_samples) return fail(FR_ERR_CAPACITY, "n exceeds max_samples");
    cudaStream_t s = (cudaStream_t)stream;
    size_t nout = (size_t)r->d.out_size[0] * r->d.out_size[1] * r->d.out_size[2];
    size_t cap = r->d.max_samples > 0 ? r->d.max_samples : 1;
    if (r->h_traj.reserve(cap * 16) || r->h_dcf.reserve(cap * 4) ||
        r->h_kdata.reserve(cap * 8 * (size_t)r->d.channels) || r->h_img.reserve(nout * 4))
        return FR_ERR_OUT_OF_MEMORY;
    if (!r->copy_stream) {
        FR_CUDA(cudaStreamCreateWithFlags(&r->copy_stream, cudaStreamNonBlocking));
        FR_CUDA(cudaEventCreateWithFlags(&r->copy_start, cudaEventDisableTiming));
        FR_CUDA(cudaEventCreateWithFlags(&r->copy_done, cudaEventDisableTiming));
    }
    cudaEvent_t ready = nullptr;
    if (n) {
        // k-space on the copy stream (after whatever `s` has queued), the
        // trajectory and DCF on `s`, which plans while the k-space arrives
        FR_CUDA(cudaEventRecord(r->copy_start, s));
        FR_CUDA(cudaStreamWaitEvent(r->copy_stream, r->copy_start, 0));
        FR_CUDA(cudaMemcpyAsync(r->h_kdata.ptr, h_kdata, n * 8 * (size_t)r->d.channels, cudaMemcpyHostToDevice,
                                r->copy_stream));
        FR_CUDA(cudaEventRecord(r->copy_done, r->copy_stream));
        ready = r->copy_done;
        FR_CUDA(cudaMemcpyAsync(r->h_traj.ptr, h_traj, n * 16, cudaMemcpyHostToDevice, s));
        FR_CUDA(cudaMemcpyAsync(r->h_dcf.ptr, h_dcf, n * 4, cudaMemcpyHostToDevice, s));
    }
    int st = recon_run(r, r->h_traj.as<float>(), r->h_dcf.as<float>(), r->h_kdata.as<float>(), n,
                       r->h_img.as<float>(), s, ready);
    if (st && ready) cudaStreamSynchronize(r->copy_stream);  // leave no copy in flight on an error
    if (st) return st;
    FR_CUDA(cudaMemcpyAsync(h_image, r->h_img.ptr, nout * 4, cudaMemcpyDeviceToHost, s));
    FR_CUDA(cudaStreamSynchronize(s));
    return FR_OK;
}

int fr_recon_submit_host(fr_recon r, const float *h_traj, const float *h_dcf, const float *h_kdata, size_t n,
                         float *h_image, void *stream)
{
    if (!r || !h_image || (n && (!h_traj || !h_dcf || !h_kdata)))
        return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    if (n > r->d.max_samples) return fail(FR_ERR_CAPACITY, "n exceeds max_samples");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t nout = (size_t)r->d.out_size[0] * r->d.out_size[1] * r->d.out_size[2];
    const size_t cap = r->d.max_samples > 0 ? r->d.max_samples : 1;
    if (!r->up_stream) {
        FR_CUDA(cudaStreamCreateWithFlags(&r->up_stream, cudaStreamNonBlocking));
        FR_CUDA(cudaStreamCreateWithFlags(&r->down_stream, cudaStreamNonBlocking));
        for (auto &sl : r->slot)
            for (cudaEvent_t *e : {&sl.uploaded, &sl.consumed, &sl.downloaded})
                FR_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    }
    auto &sl = r->slot[r->next_slot];
    if (sl.traj.reserve(cap * 16) || sl.dcf.reserve(cap * 4) || sl.kdata.reserve(cap * 8 * (size_t)r->d.channels) ||
        sl.img.reserve(nout * 4))
        return FR_ERR_OUT_OF_MEMORY;
    r->next_slot ^= 1;
    // upload once this slot's previous volume has been reconstructed (an
    // event never recorded is complete)
    FR_CUDA(cudaStreamWaitEvent(r->up_stream, sl.consumed, 0));
    if (n) {
        FR_CUDA(cudaMemcpyAsync(sl.traj.ptr, h_traj, n * 16, cudaMemcpyHostToDevice, r->up_stream));
        FR_CUDA(cudaMemcpyAsync(sl.dcf.ptr, h_dcf, n * 4, cudaMemcpyHostToDevice, r->up_stream));
        FR_CUDA(cudaMemcpyAsync(sl.kdata.ptr, h_kdata, n * 8 * (size_t)r->d.channels, cudaMemcpyHostToDevice,
                                r->up_stream));
    }
    FR_CUDA(cudaEventRecord(sl.uploaded, r->up_stream));
    // reconstruct once the inputs are there and the slot's previous image
    // has left for the host
    FR_CUDA(cudaStreamWaitEvent(s, sl.uploaded, 0));
    FR_CUDA(cudaStreamWaitEvent(s, sl.downloaded, 0));
    int st = recon_run(r, sl.traj.as<float>(), sl.dcf.as<float>(), sl.kdata.as<float>(), n, sl.img.as<float>(), s,
                       nullptr);
    if (st) {
        fr_recon_sync(r, stream);  // leave nothing in flight on an error
        return st;
    }
    FR_CUDA(cudaEventRecord(sl.consumed, s));
    FR_CUDA(cudaStreamWaitEvent(r->down_stream, sl.consumed, 0));
    FR_CUDA(cudaMemcpyAsync(h_image, sl.img.ptr, nout * 4, cudaMemcpyDeviceToHost, r->down_stream));
    FR_CUDA(cudaEventRecord(sl.downloaded, r->down_stream));
    return FR_OK;
}

int fr_recon_sync(fr_recon r, void *stream)
{
    if (!r) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    FR_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    if (r->up_stream) FR_CUDA(cudaStreamSynchronize(r->up_stream));
    if (r->down_stream) FR_CUDA(cudaStreamSynchronize(r->down_stream));
    return FR_OK;
}

int fr_recon_plan(fr_recon r, fr_plan *out)
{
    if (!r || !out) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    *out = r->plan;
    return FR_OK;
}

int fr_recon_stage_ms(fr_recon r, float *plan_ms, float *grid_ms, float *fft_ms, float *sos_ms)
{
    if (!r) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    if (plan_ms) *plan_ms = r->stage_ms[0];
    if (grid_ms) *grid_ms = r->stage_ms[1];
    if (fft_ms) *fft_ms = r->stage_ms[2];
    if (sos_ms) *sos_ms = r->stage_ms[3];
    return FR_OK;
}

}  // extern "C"
