// fr_batch.cu -- gridding of many frames (coils x frames of a dynamic
// acquisition, or several volumes) with uneven sample counts in ONE
// persistent launch, replayable as a captured CUDA graph, and an autotuner
// for the tile shape, bin chunk and coil group.  No counterpart in the
// reference, which grids one dataset per GridLut::execute call
// (GridLut.cpp:53-78).
//
// Planning: every frame is normalised with its own bounds
// (ReconData::normalizeTraj, ReconData.cpp:201-225) and binned by the
// single-trajectory planner; its normalised samples, bin records, work items
// and split tiles are appended to batch-wide arrays, and the items and split
// tiles are relabelled with their frame and global offsets.  Gridding: the
// persistent scatter kernel takes (coil group, item) work indices from a
// counter until the batch is done; frame f's k-space is the block
// channels x n_f at complex offset channels * offset[f] and its grid the
// block channels x G^d at f * channels * G^d.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "fr_internal.h"

using namespace fr;

struct fr_batch_s {
    fr_plan plan = nullptr;  // per-frame planner (tiling, LUT)
    int frames = 0;
    std::vector<long long> off;
    DevBuf frame_off, traj, recs, items, splits, partials, counter;
    long long n_total = 0, npairs = 0, nitems = 0, nslots = 0, nsplits = 0;
    int blocks = 0;
    bool ready = false;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    ~fr_batch_s()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (plan) fr_plan_destroy(plan);
    }
};

namespace {

__global__ void fixup_items_kernel(WorkItem *it, long long n, long long rec_off, int slot_off, int frame)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        WorkItem w = it[i];
        w.begin += rec_off;
        if (w.slot >= 0) w.slot += slot_off;
        w.pad = frame;
        it[i] = w;
    }
}

__global__ void fixup_splits_kernel(SplitTile *st, long long n, int slot_off, int frame)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        st[i].first_slot += slot_off;
        st[i].pad = frame;
    }
}

// Grow `b` to hold `need` bytes, keeping its first `used` bytes.
int grow_keep(DevBuf &b, size_t used, size_t need, cudaStream_t s)
{
    if (need <= b.bytes && b.ptr) return FR_OK;
    size_t want = std::max<size_t>(need, b.bytes + b.bytes / 2);
    void *p = nullptr;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(want, 256));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    if (used) {
        e = cudaMemcpyAsync(p, b.ptr, used, cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) {
            cudaFree(p);
            return cuda_fail(e, "cudaMemcpyAsync");
        }
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            cudaFree(p);
            return cuda_fail(e, "cudaStreamSynchronize");
        }
    }
    b.release();
    b.ptr = p;
    b.bytes = std::max<size_t>(want, 256);
    return FR_OK;
}

int fill_batch_grid(fr_batch b, BatchGrid *g)
{
    fr_plan p = b->plan;
    g->dim = p->dim;
    g->G = p->G;
    for (int d = 0; d < 3; ++d) {
        g->tile[d] = p->tile[d];
        g->ntile[d] = p->ntile[d];
    }
    g->coil_group = p->coil_group;
    g->L = p->L;
    g->smax = p->lut_smax;
    g->kc = p->lut_kc;
    g->lut_absmax = p->lut_absmax;
    g->checkerboard = (p->flags & FR_PLAN_CHECKERBOARD) ? 1 : 0;
    g->traj = b->traj.as<float4>();
    g->recs = b->recs.as<unsigned long long>();
    g->items = b->items.as<WorkItem>();
    g->splits = b->splits.as<SplitTile>();
    g->lut_e = p->lut_e.as<float4>();
    g->frame_off = b->frame_off.as<long long>();
    g->nitems = b->nitems;
    g->nsplits = b->nsplits;
    g->n_total = b->n_total;
    g->partials = b->partials.as<float>();
    g->work_counter = b->counter.as<int>();
    g->blocks = b->blocks;
    return FR_OK;
}

int ensure_partials(fr_batch b, int channels)
{
    fr_plan p = b->plan;
    if (b->nslots == 0) return FR_OK;
    const long long K = (long long)p->tile[0] * p->tile[1] * p->tile[2];
    if (b->partials.reserve(grid_partials_bytes(b->nslots, channels, p->coil_group, K))) return FR_ERR_OUT_OF_MEMORY;
    return FR_OK;
}

int check_grid_args(fr_batch b, const float *d_kdata, const float *d_dcf, int channels, const float *d_grid)
{
    if (!b || !d_grid) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    if (!b->ready) return fail(FR_ERR_NOT_PLANNED, "fr_batch_set_trajectories has not run");
    if (channels <= 0) return fail(FR_ERR_INVALID_ARGUMENT, "channels must be positive");
    if (b->n_total && (!d_kdata || !d_dcf)) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    if ((reinterpret_cast<uintptr_t>(d_kdata) & 7) || (reinterpret_cast<uintptr_t>(d_grid) & 7))
        return fail(FR_ERR_INVALID_ARGUMENT, "complex buffers must be 8-byte aligned");
    return FR_OK;
}

}  // namespace

extern "C" {

int fr_batch_create(const fr_plan_desc *desc, fr_batch *out)
{
    if (!out) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    auto b = new (std::nothrow) fr_batch_s;
    if (!b) return fail(FR_ERR_OUT_OF_MEMORY, "batch");
    int st = fr_plan_create(desc, &b->plan);
    if (st) {
        delete b;
        return st;
    }
    *out = b;
    return FR_OK;
}

int fr_batch_destroy(fr_batch b)
{
    delete b;
    return FR_OK;
}

int fr_batch_set_trajectories(fr_batch b, const float *d_traj, const size_t *offsets, int frames, void *stream)
{
    if (!b || !offsets || frames < 1) return fail(FR_ERR_INVALID_ARGUMENT, "null argument or no frames");
    if (offsets[0] != 0) return fail(FR_ERR_INVALID_ARGUMENT, "offsets[0] must be 0");
    for (int f = 0; f < frames; ++f)
        if (offsets[f + 1] < offsets[f]) return fail(FR_ERR_INVALID_ARGUMENT, "offsets must be non-decreasing");
    if (offsets[frames] && !d_traj) return fail(FR_ERR_INVALID_ARGUMENT, "null trajectory");
    if (reinterpret_cast<uintptr_t>(d_traj) & 15) return fail(FR_ERR_INVALID_ARGUMENT, "trajectory must be 16-byte aligned");
    cudaStream_t s = (cudaStream_t)stream;
    fr_plan p = b->plan;
    b->ready = false;
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    if (b->graph) {
        cudaGraphDestroy(b->graph);
        b->graph = nullptr;
    }
    b->frames = frames;
    b->off.assign(offsets, offsets + frames + 1);
    b->n_total = (long long)offsets[frames];
    if (b->traj.reserve(std::max<long long>(b->n_total, 1) * 16) ||
        b->frame_off.reserve((size_t)(frames + 1) * 8) || b->counter.reserve(256))
        return FR_ERR_OUT_OF_MEMORY;
    FR_CUDA(cudaMemcpyAsync(b->frame_off.ptr, b->off.data(), (size_t)(frames + 1) * 8, cudaMemcpyHostToDevice, s));
    long long npairs = 0, nitems = 0, nslots = 0, nsplits = 0;
    for (int f = 0; f < frames; ++f) {
        const size_t nf = offsets[f + 1] - offsets[f];
        int st = plan_run(p, d_traj + 4 * offsets[f], nf, s);  // synchronises s
        if (st) return st;
        if (nslots + p->nslots > 0x7FFFFFFFll || nitems + p->nitems > 0x7FFFFFFFll)
            return fail(FR_ERR_UNSUPPORTED, "batch too large for 32-bit item indices");
        if ((st = grow_keep(b->recs, (size_t)npairs * 8, (size_t)(npairs + p->npairs) * 8, s)) ||
            (st = grow_keep(b->items, (size_t)nitems * sizeof(WorkItem), (size_t)(nitems + p->nitems) * sizeof(WorkItem), s)) ||
            (st = grow_keep(b->splits, (size_t)nsplits * sizeof(SplitTile),
                            (size_t)(nsplits + std::max<long long>(p->nsplits, 0)) * sizeof(SplitTile), s)))
            return st;
        if (nf) FR_CUDA(cudaMemcpyAsync(b->traj.as<float4>() + offsets[f], p->traj.ptr, nf * 16, cudaMemcpyDeviceToDevice, s));
        if (p->npairs)
            FR_CUDA(cudaMemcpyAsync(b->recs.as<unsigned long long>() + npairs, p->pairs.ptr, (size_t)p->npairs * 8,
                                    cudaMemcpyDeviceToDevice, s));
        if (p->nitems) {
            WorkItem *dst = b->items.as<WorkItem>() + nitems;
            FR_CUDA(cudaMemcpyAsync(dst, p->items.ptr, (size_t)p->nitems * sizeof(WorkItem), cudaMemcpyDeviceToDevice, s));
            fixup_items_kernel<<<(int)std::min<long long>((p->nitems + 255) / 256, 1024), 256, 0, s>>>(
                dst, p->nitems, npairs, (int)nslots, f);
            FR_CHECK_LAUNCH("fixup_items_kernel");
        }
        if (p->nsplits) {
            SplitTile *dst = b->splits.as<SplitTile>() + nsplits;
            FR_CUDA(cudaMemcpyAsync(dst, p->splits.ptr, (size_t)p->nsplits * sizeof(SplitTile), cudaMemcpyDeviceToDevice, s));
            fixup_splits_kernel<<<(int)std::min<long long>((p->nsplits + 255) / 256, 1024), 256, 0, s>>>(
                dst, p->nsplits, (int)nslots, f);
            FR_CHECK_LAUNCH("fixup_splits_kernel");
        }
        npairs += p->npairs;
        nitems += p->nitems;
        nslots += p->nslots;
        nsplits += p->nsplits;
    }
    FR_CUDA(cudaStreamSynchronize(s));  // the planner's buffers are reused by the next call
    b->npairs = npairs;
    b->nitems = nitems;
    b->nslots = nslots;
    b->nsplits = nsplits;
    const long long K = (long long)p->tile[0] * p->tile[1] * p->tile[2];
    int st = batch_grid_setup(p->dim, K, p->coil_group, p->L, &b->blocks);
    if (st) return st;
    b->ready = true;
    return FR_OK;
}

int fr_batch_stats(fr_batch b, long long *frames, long long *samples, long long *items, long long *slots,
                   int *persistent_ctas)
{
    if (!b) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    if (frames) *frames = b->frames;
    if (samples) *samples = b->n_total;
    if (items) *items = b->nitems;
    if (slots) *slots = b->nslots;
    if (persistent_ctas) *persistent_ctas = b->blocks;
    return FR_OK;
}

int fr_batch_grid(fr_batch b, const float *d_kdata, const float *d_dcf, int channels, float *d_grid, void *stream)
{
    int st = check_grid_args(b, d_kdata, d_dcf, channels, d_grid);
    if (st) return st;
    if ((st = ensure_partials(b, channels))) return st;
    BatchGrid g;
    fill_batch_grid(b, &g);
    return batch_grid_run(g, d_kdata, d_dcf, channels, d_grid, (cudaStream_t)stream);
}

int fr_batch_capture(fr_batch b, const float *d_kdata, const float *d_dcf, int channels, float *d_grid, void *stream)
{
    int st = check_grid_args(b, d_kdata, d_dcf, channels, d_grid);
    if (st) return st;
    if (!stream) return fail(FR_ERR_INVALID_ARGUMENT, "capture needs a created stream, not the legacy default stream");
    if ((st = ensure_partials(b, channels))) return st;
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    if (b->graph) {
        cudaGraphDestroy(b->graph);
        b->graph = nullptr;
    }
    cudaStream_t s = (cudaStream_t)stream;
    BatchGrid g;
    fill_batch_grid(b, &g);
    FR_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    st = batch_grid_run(g, d_kdata, d_dcf, channels, d_grid, s);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(s, &graph);
    if (st) {
        if (graph) cudaGraphDestroy(graph);
        return st;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&b->exec, graph, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(graph);
        b->exec = nullptr;
        return cuda_fail(e, "cudaGraphInstantiate");
    }
    b->graph = graph;
    return FR_OK;
}

int fr_batch_replay(fr_batch b, void *stream)
{
    if (!b) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    if (!b->exec) return fail(FR_ERR_NOT_PLANNED, "no captured graph: call fr_batch_capture first");
    FR_CUDA(cudaGraphLaunch(b->exec, (cudaStream_t)stream));
    note_launch();
    return FR_OK;
}

int fr_batch_autotune(const fr_plan_desc *base, const float *d_traj, const size_t *offsets, int frames,
                      const float *d_kdata, const float *d_dcf, int channels, float *d_grid, int repeats,
                      fr_plan_desc *best, float *best_ms, void *stream)
{
    if (!base || !best) return fail(FR_ERR_INVALID_ARGUMENT, "null argument");
    if (repeats < 1) repeats = 3;
    cudaStream_t s = (cudaStream_t)stream;
    struct Cand {
        int t[3];
        int chunk;
        int cg;
    };
    std::vector<Cand> cands;
    const int cgs[3] = {8, 16, 32};
    if (base->dim == 3) {
        const int shapes[][3] = {{8, 8, 8}, {16, 8, 8}, {8, 8, 4}, {16, 8, 4}, {16, 16, 4}};
        for (auto &sh : shapes)
            for (int chunk : {2048, 4096, 8192})
                for (int cg : cgs) cands.push_back({{sh[0], sh[1], sh[2]}, chunk, cg});
    } else {
        const int shapes[][2] = {{16, 16}, {32, 16}, {32, 32}, {64, 32}, {64, 64}};
        for (auto &sh : shapes)
            for (int chunk : {1024, 2048, 4096, 8192})
                for (int cg : cgs) cands.push_back({{sh[0], sh[1], 1}, chunk, cg});
    }
    cudaEvent_t e0, e1;
    FR_CUDA(cudaEventCreate(&e0));
    FR_CUDA(cudaEventCreate(&e1));
    float bestv = 1e30f;
    int found = 0;
    for (const Cand &c : cands) {
        if (c.cg > 8 && c.cg >= 2 * channels) continue;  // a coil group at least twice the coils
        fr_plan_desc d = *base;
        for (int i = 0; i < 3; ++i) d.tile[i] = c.t[i];
        d.chunk = c.chunk;
        d.coil_group = c.cg;
        fr_batch b = nullptr;
        if (fr_batch_create(&d, &b) != FR_OK) continue;  // shape does not fit: skip
        float ms = 1e30f;
        int st = fr_batch_set_trajectories(b, d_traj, offsets, frames, stream);
        if (!st) st = fr_batch_grid(b, d_kdata, d_dcf, channels, d_grid, stream);  // warm-up
        for (int r = 0; !st && r < repeats; ++r) {
            cudaEventRecord(e0, s);
            st = fr_batch_grid(b, d_kdata, d_dcf, channels, d_grid, stream);
            cudaEventRecord(e1, s);
            if (!st && cudaEventSynchronize(e1) == cudaSuccess) {
                float t = 0.f;
                cudaEventElapsedTime(&t, e0, e1);
                ms = std::min(ms, t);
            }
        }
        fr_batch_destroy(b);
        if (st == FR_ERR_CUDA || st == FR_ERR_OUT_OF_MEMORY) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return st;
        }
        if (!st && ms < bestv) {
            bestv = ms;
            *best = d;
            found = 1;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!found) return fail(FR_ERR_UNSUPPORTED, "no tiling candidate ran");
    if (best_ms) *best_ms = bestv;
    return FR_OK;
}

}  // extern "C"
