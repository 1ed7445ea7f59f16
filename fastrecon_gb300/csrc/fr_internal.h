// fr_internal.h -- internal declarations of libfastrecon_gb300.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/fastrecon_gb300.h"

namespace fr {

// Thread-local error detail; returns `status` for use in `return fail(...)`.
int fail(int status, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);
void note_launch();

#define FR_CUDA(call)                                   \
    do {                                                \
        cudaError_t e_ = (call);                        \
        if (e_ != cudaSuccess) return ::fr::cuda_fail(e_, #call); \
    } while (0)

// Call once after every kernel launch: counts it and checks the launch.
#define FR_CHECK_LAUNCH(name)                           \
    do {                                                \
        ::fr::note_launch();                            \
        cudaError_t e_ = cudaGetLastError();            \
        if (e_ != cudaSuccess) return ::fr::cuda_fail(e_, name); \
    } while (0)

// Device buffer with capacity reuse (cudaMalloc / cudaFree).
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    ~DevBuf();
    int reserve(size_t n);  // grows only; contents are not preserved
    void release();
    template <typename T> T *as() const { return static_cast<T *>(ptr); }
};

// One work item of the scatter: a tile and a chunk of its sorted bin.
struct WorkItem {
    long long begin;  // first index into pairs[]
    int count;        // samples in this chunk
    int tile;         // tile index (row-major over the tile grid)
    int slot;         // partial slot for split tiles, -1 otherwise
    int pad;
};

// A tile whose bin was split into several work items.
struct SplitTile {
    int tile;
    int first_slot;
    int nslots;
    int pad;
};

// One bucket of a split tile's records being put in sample order
// (deterministic plans).
struct SortBucket {
    long long start;  // first record
    int count;
    int pad;
};

// Scan tuple over tiles: pairs, work items of occupied tiles, partial
// slots, split tiles, empty tiles (whose zero-fill items follow every
// occupied tile's items in the item list).
struct TileScan {
    long long pairs, items, slots, splits, empties;
};

}  // namespace fr

struct fr_plan_s {
    int device = 0;
    int dim = 2;
    unsigned G = 0;
    float W = 4.f, hw = 2.f;
    int L = 0;
    std::vector<float> lut;
    int tile[3] = {1, 1, 1};
    int ntile[3] = {1, 1, 1};
    long long ntiles = 0;
    int coil_group = 8;
    int chunk = 4096;       // records per work item of the current trajectory
    int chunk_req = 0;      // the descriptor's chunk (0: chosen per trajectory, plan_chunk)
    int prefilter = 0;  // |x - c| >= kHW implies dk >= kHW (kHW^2 and sqrt exact)
    unsigned flags = 0;

    size_t n = 0;
    bool planned = false;
    long long npairs = 0, nitems = 0, nslots = 0, nsplits = 0;
    long long nitems_occupied = 0;  // items[0, nitems_occupied): tiles with samples; the rest zero-fill
    float bounds_host[12] = {0};  // raw lo[3], raw hi[3], norm lo[3], norm hi[3]

    fr::DevBuf lut_d;         // L floats
    fr::DevBuf lut_e;         // L float4 {thr[k+1], lut[k], lut[k+1], 0}
    std::vector<float> lut_entries;
    float lut_smax = 0.f, lut_kc = 0.f;
    float lut_absmax = 1.f;   // max |lut[k]| (bounds every tap weight)
    fr::DevBuf traj;          // n float4, normalised
    fr::DevBuf bounds;        // 16 floats: raw lo/hi as ordered ints, tr, scale, norm lo/hi
    fr::DevBuf tile_count;    // ntiles int
    fr::DevBuf tile_fill;     // ntiles x stripes int (fill cursors)
    fr::DevBuf stripe_count;  // ntiles x stripes int (bin counts per stripe)
    fr::DevBuf stripe_base;   // ntiles x stripes long long (first record of each stripe)
    fr::DevBuf tile_scan;     // (ntiles + 1) TileScan, exclusive
    fr::DevBuf scan_blocks;   // scan scratch
    fr::DevBuf pairs;         // npairs records: sample index | tap box << 32
    fr::DevBuf items;         // nitems WorkItem
    fr::DevBuf splits;        // nsplits SplitTile
    fr::DevBuf partials;      // nslots * ngroups * K * R floats
    fr::DevBuf ranges;        // scratch for fr_plan_sample_ranges (unused otherwise)
    fr::DevBuf real_grid;     // G^d floats: Pipe-Menon weight grid
    fr::DevBuf real_partials; // nslots * K floats: split tiles of the real-valued scatter
    fr::DevBuf density_sat;   // G^d ints: per-cell counts -> summed-area table
    fr::DevBuf small;         // 256 bytes of scratch (feature max |k|)
    fr::DevBuf kt;            // n x channels complex: sample-major copy of dcf * k-space (fr_grid)
    fr::DevBuf kmag;          // n floats: per sample max |re|, |im| of dcf * k over the coils
    const float *kt_prepared = nullptr;  // k-space whose copy kspace_prepare made for the next grid_run
    int kt_prepared_channels = 0;
    fr::DevBuf tile_mask;     // ntiles bits: tile holds bin records (recon path skips the others)
    bool kspace_sample_major = true;  // cleared by FR_KSPACE_COIL_MAJOR=1

    // Tap lists: every sample's kernel taps evaluated once per trajectory by
    // the plan (GridLut.cpp:98-136 geometry), so the scatter reads them
    // instead of evaluating the geometry of each of the sample's bin records.
    // Slot of sample s: tap_words words holding the runs of its records (one
    // per tile it touches, in the plan's tile-walk order).  Tap word:
    // tile-local cell | LUT index << 13.
    bool taps_enabled = true;  // cleared by FR_PLAN_NO_TAP_LISTS
    bool scatter_warp_lists = false;  // FR_SCATTER_WARP_LISTS=1: per-warp tap lists instead of tap lanes
    int tap_words = 0;         // 0: this plan has no tap lists
    int tap_layout_words = 0;  // tap_slot_layout of this plan (computed once)
    fr::DevBuf taps;           // n x tap_words words
    fr::DevBuf trecs;          // npairs words, in bin order: sample | first word << 32 | taps << 40
    fr::DevBuf item_inv;       // per work item: inverse fixed-point scale, then the items' bounds
    fr::DevBuf sort_tmp;       // deterministic plans: split tiles' records (and tap records) being sorted
    fr::DevBuf sort_buckets;   // deterministic plans: SortBucket table + its count
    int *err_host = nullptr;   // mapped pinned word the kernels set on an internal error
    int *err_dev = nullptr;

    // scatter-kernel timing (fr_plan_profile)
    bool profile = false;
    std::vector<cudaEvent_t> prof_ev;  // pairs (start, stop)
    int prof_used = 0;
    ~fr_plan_s();
};

namespace fr {
// Kernel-side entry points implemented in the .cu files.
int plan_run(fr_plan p, const float *d_traj, size_t n, cudaStream_t s);
// skip_empty: leave the cells of tiles without samples unwritten (the
// caller's next reader masks them with the plan's tile bitmap).
// kin_stride: complex values between coils of d_kdata (0: the plan's n),
// for a sample range of a larger coil-major k-space.
int grid_run(fr_plan p, const float *d_kdata, const float *d_dcf, int channels, float *d_grid,
             cudaStream_t s, bool skip_empty = false, size_t kin_stride = 0);
// The scatter's sample-major dcf * k-space copy, made ahead of grid_run
// (e.g. on another stream while the plan's kernels run); the next grid_run
// with the same k-space pointer and channel count uses it instead of making
// its own.  The caller orders that grid_run after this copy.
int kspace_prepare(fr_plan p, const float *d_kdata, const float *d_dcf, int channels, cudaStream_t s,
                   size_t kin_stride = 0);
int sample_ranges_run(fr_plan p, int *d_start, int *d_end, cudaStream_t s);
// sos_mode: 2 = the whole SoS (sqrt, / deapod); for coils in slabs 0 = store
// the plain sum of |x|^2, | 1 = add to the sum already in d_out.
int sos_run(const float *d_imgs, int channels, int dim, const unsigned *size, const unsigned *recon,
            const float *d_deapod, float *d_out, cudaStream_t s, int sos_mode = 2);
int shift_run(float *d_imgs, int channels, int dim, const unsigned *size, cudaStream_t s);
int crop_run(const float *d_imgs, int channels, int dim, const unsigned *size, const unsigned *crop,
             float *d_out, cudaStream_t s);
// Default tile shape / coil group for a configuration.
void default_tiling(int dim, int *tile, int *coil_group, int channels);
// Floats per tile cell in shared memory for a coil group.
int floats_per_cell(int coil_group);
// Dynamic shared memory of the scatter kernel for K cells of R floats and an
// L-entry LUT.
size_t grid_smem_bytes(long long K, int R, int L);

// Exact LUT index without a square root.  The reference index
//   ki(s) = roundf(fl(fl(sqrtf(s)) / kHW) * (L-1)),  valid iff sqrtf(s) < kHW,
// of s = dz^2 + dy^2 + dx^2 is a non-decreasing step function of s.
// thr[k] (k = 1..L-1) is the smallest float s with ki(s) >= k, thr[L] = +inf,
// and smax the smallest s with sqrtf(s) >= kHW.  Host computation, exact.
struct LutIndexTable {
    std::vector<float> thr;  // L + 1 entries, thr[0] = 0
    float smax = 0.f;
    float kc = 0.f;          // (L-1) / kHW for the approximate first guess
};
int lut_reference_index(float s, float hw, int L);  // the reference formula on the host (-1 if invalid)
LutIndexTable lut_index_table(float hw, int L);
// The same table into caller storage: thr has L + 1 entries.
void lut_index_table_into(float hw, int L, float *thr, float *smax, float *kc);

// Plan into caller-provided device memory (no allocation).  The fixed-size
// buffers are given; records, work items and split tiles are carved from
// [rest, rest + rest_bytes) once their counts are known.
struct PlanInto {
    int dim;
    unsigned G;
    float hw;
    int prefilter;
    int tile[3], ntile[3];
    long long ntiles;
    int chunk;
    int *bounds;  // 32 words
    float4 *traj;
    int *tile_count;          // ntiles
    int *tile_fill;           // ntiles x plan_stripes()
    int *stripe_count;        // ntiles x plan_stripes()
    long long *stripe_base;   // ntiles x plan_stripes()
    TileScan *scan;         // ntiles + 1
    TileScan *scan_blocks;  // plan_scan_blocks(ntiles)
    unsigned char *rest;
    size_t rest_bytes;
};
struct PlanIntoOut {
    long long npairs, nitems, nslots, nsplits;
    unsigned long long *recs;
    WorkItem *items;
    SplitTile *splits;
    size_t rest_used;
};
long long plan_scan_blocks(long long ntiles);
// Records per work item for n samples: enough items for every SM to take
// several (a small trajectory's dense centre tile would otherwise be one
// long item that the whole launch waits for), at most 4096.
int plan_chunk(size_t n, int dim);
int plan_stripes();  // bin-counter stripes per tile
// Tap-list slot of a sample for a kernel half-width: words per sample, an
// upper bound on the lattice points strictly inside a ball of radius hw.
void tap_slot_layout(int dim, float hw, int *words);
constexpr int kTapCellBits = 13;            // tile-local cell index bits of a tap word
constexpr int kTapRecMax = 60;              // samples with more taps use the geometry scatter
int plan_into(const PlanInto &pi, const float *d_traj, size_t n, cudaStream_t s, PlanIntoOut *out);

// Grid from a plan held in caller-provided memory (no allocation).
struct GridInto {
    int dim;
    unsigned G;
    int tile[3], ntile[3];
    int coil_group;
    int L;
    float smax, kc;
    float lut_absmax;
    const float4 *traj;
    const unsigned long long *recs;
    const WorkItem *items;
    const SplitTile *splits;
    const float4 *lut_e;
    long long nitems, nsplits;
    size_t n;
    float *partials;
};
size_t grid_partials_bytes(long long nslots, int channels, int coil_group, long long K);

// Gridding of a batch of frames in one persistent launch (fr_batch_*).
struct BatchGrid {
    int dim;
    unsigned G;
    int tile[3], ntile[3];
    int coil_group;
    int L;
    float smax, kc;
    float lut_absmax;
    int checkerboard;
    const float4 *traj;               // all frames, normalised, concatenated
    const unsigned long long *recs;   // all frames' bin records (frame-local sample index)
    const WorkItem *items;            // pad = frame
    const SplitTile *splits;          // pad = frame
    const float4 *lut_e;
    const long long *frame_off;       // frames + 1 sample offsets (device)
    long long nitems, nsplits, n_total;
    float *partials;
    int *work_counter;
    int blocks;                       // persistent CTAs (batch_grid_setup)
};
// Sets the kernel attributes for a configuration and returns how many
// persistent CTAs fill the GPU.  Call outside stream capture.
int batch_grid_setup(int dim, long long K, int coil_group, int L, int *blocks);
int batch_grid_run(const BatchGrid &b, const float *d_kdata, const float *d_dcf, int channels, float *d_grid,
                   cudaStream_t s);
int grid_into(const GridInto &gi, const float *d_kdata, const float *d_dcf, int channels, float *d_grid,
              cudaStream_t s);
}  // namespace fr

namespace fr {
// Density compensation and degridding (fr_dcf.cu).
int dcf_analytic_run(const float *d_traj, size_t n, int dim, float power, float *d_out, cudaStream_t s);
int degrid_run(fr_plan p, const float *d_grid, int channels, float *d_out, cudaStream_t s);
int grid_update_run(fr_plan p, float *d_kdata, const float *d_new, size_t begin, size_t count, const float *d_dcf,
                    int channels, float *d_grid, cudaStream_t s);
int grid_real_run(fr_plan p, const float *d_w, float *d_grid, cudaStream_t s);
int dcf_pipe_run(fr_plan p, int iterations, float *d_w, cudaStream_t s);
// Density features (fr_density.cu) and the DCF network (fr_mlp.cu).
int density_counts_run(fr_plan p, const int *radii, int nradii, int *d_counts, cudaStream_t s);
int dcf_features_run(const int *d_counts, const float *d_raw, size_t n, int dim, const int *radii, int nradii,
                     float kmax, float *d_feat, unsigned *d_scratch, cudaStream_t s);
size_t mlp_workspace_bytes(size_t n);
int mlp_forward_run(const void *d_params, const float *d_x, size_t n, int exp_out, int residual, float scale,
                    float *d_y, cudaStream_t s);
int mlp_backward_run(const void *d_params, const float *d_x, const float *d_t, const float *d_w, size_t n, void *ws,
                     float *d_grad, float *d_loss, cudaStream_t s);
int mlp_adam_run(float *d_master, void *d_params, const float *d_grad, float *d_m, float *d_v, int count, float lr,
                 float beta1, float beta2, float eps, int step, cudaStream_t s);
int to_bf16_run(const float *d_a, void *d_b, int count, cudaStream_t s);
}  // namespace fr

namespace fr {
// True when the pruned FFT has compile-time specialised passes for G.
bool pruned_fft_specialised(int G);
// The pruned transform + crop + SoS of `channels` (<= the object's) coils;
// sos_mode as sos_run's.
// tiles (optional): the grid's unwritten tiles, as the plan's occupancy
// bitmap over tiles of edge tile[0..2]; cells of empty tiles read as zero.
struct TileMask {
    const unsigned *bits = nullptr;
    int tile[3] = {1, 1, 1};
    int ntile[3] = {1, 1, 1};
};
int fftcs_execute(fr_fftcs f, const float *d_grid, int channels, const float *d_deapod, float *d_out, int sos_mode,
                  cudaStream_t s, const TileMask *tiles = nullptr);
bool fftcs_masks_tiles(fr_fftcs f);  // the x stage takes a TileMask (register stages)
}  // namespace fr

namespace fr {
int deapod_seed_run(float *d_grid, int dim, int G, float hw, const float *d_lut, int L, int checkerboard,
                    cudaStream_t s);
int deapod_map_run(const float *d_img, int dim, const unsigned *size, const unsigned *recon, float *d_out,
                   cudaStream_t s);
}  // namespace fr

namespace fr {
int normalize_run(const float *d_traj, size_t n, int dim, unsigned G, float *d_out, float *bounds12,
                  cudaStream_t s);
int transform_run(float *d_traj, size_t n, int dim, float tr, float scale, cudaStream_t s);
int real_to_complex_run(const float *d_in, size_t n, float *d_out, cudaStream_t s);
int low_filter_run(float *d_imgs, int channels, int dim, const unsigned *size, float att, const float *d_coeff,
                   cudaStream_t s);
int normalize_channels_run(float *d_imgs, int channels, int dim, const unsigned *size, cudaStream_t s);
int sos_map_run(const float *d_imgs, const float *d_maps, int channels, int dim, const unsigned *size,
                const unsigned *recon, float *d_out, cudaStream_t s);
}  // namespace fr
