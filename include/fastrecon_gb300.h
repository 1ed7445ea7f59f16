/*
 * fastrecon_gb300.h -- C ABI of libfastrecon_gb300.so, the GB300 (sm_103a)
 * gridding / reconstruction path behind fastrecon's C++ API.
 *
 * Every entry point takes plain pointers, sizes and an optional CUDA stream
 * (passed as `void *`, a cudaStream_t; NULL = the legacy default stream) and
 * returns an fr_status.  Device pointers are caller-owned; the library only
 * allocates the internal buffers of the opaque plan objects.  Each entry
 * point cites the reference (pengwg/fastrecon) interface it replaces.
 *
 * Layouts are the reference's in-memory layouts:
 *   trajectory : Point<float>{x[4]} per sample (16 B, sample-major),
 *                ReconData/ReconData.h:12-15
 *   dcf        : float per sample (ReconData.h:59)
 *   k-space    : channel-major, N complex64 per channel (ReconData.h:58)
 *   grid/image : channel-major, G^d complex64 per channel, x fastest
 *                (ImageData/ImageData.h, GridLut.cpp:94,111)
 * Sizes are (x, y, z) like ImageSize (ImageData/common.h:7-12); z = 1 in 2D.
 */
#ifndef FASTRECON_GB300_H
#define FASTRECON_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    FR_OK = 0,
    FR_ERR_INVALID_ARGUMENT = 1, /* bad pointer, dimension or size */
    FR_ERR_SIZE_MISMATCH = 2,    /* sizes that must agree do not */
    FR_ERR_OUT_OF_MEMORY = 3,    /* device or host allocation failed */
    FR_ERR_CUDA = 4,             /* a CUDA runtime call failed */
    FR_ERR_CUFFT = 5,            /* a cuFFT call failed */
    FR_ERR_NOT_PLANNED = 6,      /* execute before plan (cuGridLut.cu:31-34) */
    FR_ERR_UNSUPPORTED = 7,      /* parameter outside the supported range */
    FR_ERR_DEVICE_TIMEOUT = 8,   /* a bounded device-side wait expired */
    FR_ERR_CAPACITY = 9          /* a fixed-capacity buffer is too small */
} fr_status;

/* Text for a status code; never NULL. */
const char *fr_status_string(int status);
/* Detail of the last error raised on the calling thread (may be ""). */
const char *fr_last_error(void);
/* Library version string. */
const char *fr_version(void);

/* ------------------------------------------------------------------------
 * ConvKernel (ReconData/ConvKernel.h:10-14, ConvKernel.cpp:7-30)
 * Radial Kaiser-Bessel LUT of `length` entries on radius [0, W/2],
 * Beatty beta, normalised so lut[0] = 1.  Host computation.
 * ---------------------------------------------------------------------- */
int fr_kb_lut(float kernel_width, float overgrid_factor, int length, float *lut_host);

/* Exact LUT index from s = dk^2 without a square root (host computation).
 * The reference index roundf(fl(fl(sqrtf(s)) / kHW) * (L-1)) (GridLut.cpp:
 * 131-136) is a non-decreasing step function of s; thresholds[k] (k < L) is
 * the smallest float s whose index is >= k (thresholds[0] = 0, +inf if never
 * reached), thresholds[L] = +inf, *smax the smallest s with sqrtf(s) >= kHW
 * (taps with s >= smax are outside the kernel), *kc = (L-1)/kHW.  The
 * scatter kernel guesses k0 from an approximate square root, which lands on
 * the exact index or one below, and corrects it with one comparison against
 * thresholds[k0+1]. */
int fr_lut_index_table(float kernel_width, int length, float *thresholds, float *smax, float *kc);

/* ------------------------------------------------------------------------
 * Gridding plan: GridLut::plan + cuGridLut::plan
 * (ReconData/GridLut.h:20, GridLut.cpp:41-51, cuGridLut.cu:151-226)
 *
 * The plan normalises the trajectory exactly like ReconData::normalizeTraj
 * (ReconData.cpp:211-225: translation -min, scale (G-1)/(max-min) of
 * component 0, applied to every component), computes each sample's clamped
 * cell range exactly like GridLut.cpp:98-106, and bins samples into grid
 * tiles with an integer counting sort.  The input trajectory is not
 * modified; fr_plan_normalized_trajectory returns the normalised copy.
 * ---------------------------------------------------------------------- */
typedef struct fr_plan_s *fr_plan;

enum {
    FR_PLAN_CHECKERBOARD = 1u << 0, /* multiply grid cell (x,y,z) by (-1)^(x+y+z)
                                       on output, which makes the backward FFT
                                       produce the fftShift-ed image (even G) */
    FR_PLAN_PRENORMALIZED = 1u << 1, /* the trajectory given to
                                       fr_plan_set_trajectory is already in
                                       grid units (ReconData::normalizeTraj was
                                       applied, e.g. by fr_normalize_trajectory):
                                       bin it as is */
    FR_PLAN_NO_TAP_LISTS = 1u << 2, /* keep no per-sample tap lists: the
                                       scatter evaluates each bin record's
                                       kernel taps itself (saves ~170 bytes
                                       per 3D sample of device memory, slower) */
    FR_PLAN_ACCUMULATE = 1u << 3,   /* fr_grid adds the plan's samples to
                                       d_grid instead of overwriting it (cells
                                       of tiles without samples are left as
                                       they are): one grid from several plans
                                       over sample ranges of one trajectory */
    FR_PLAN_DETERMINISTIC = 1u << 4 /* bit-reproducible grids: the records of
                                       tiles split into several work items are
                                       put in sample order after the bin fill
                                       (the fill places them with atomics), so
                                       each item holds the same records on
                                       every run.  Applies to the tap-list
                                       scatter; costs two short kernels and
                                       16 bytes per bin record of scratch */
};

/* ReconData::normalizeTraj (ReconData.cpp:211-225) on the device: component
 * bounds of d_traj (n Point<float>), translation -min and scale
 * (G-1)/(max-min) of component 0, x <- (x + tr) * scale for components < dim
 * into d_out (may equal d_traj).  bounds12 (host, nullable) receives raw
 * lo[3], raw hi[3], normalised lo[3], normalised hi[3].  Synchronises
 * `stream`. */
int fr_normalize_trajectory(const float *d_traj, size_t n, int dim, unsigned grid_size, float *d_out,
                            float *bounds12, void *stream);

/* cuReconData::transformLocalTraj (cuReconData.cu:88-99, scale_functor
 * cuReconData.h:23-37): x <- (x + translation) * scale for components < dim
 * of n Point<float> samples, in place on the device. */
int fr_transform_trajectory(float *d_traj, size_t n, int dim, float translation, float scale, void *stream);

typedef struct {
    int dim;               /* 2 or 3 (ReconData::rcDim) */
    unsigned grid_size;    /* G = unsigned(reconSize * overGridFactor), GridLut.cpp:45 */
    float kernel_width;    /* W (full width), ConvKernel kWidth */
    int lut_length;        /* L, ConvKernel length (512 in Program/Main.cpp:127) */
    const float *lut;      /* host pointer to the L-entry LUT (fr_kb_lut) */
    int tile[3];           /* tile shape in cells (x,y,z); 0 = default */
    int coil_group;        /* coils per scatter pass (4, 8, 16, 32); 0 = default */
    int chunk;             /* max samples per work item before a tile is split; 0 = default */
    unsigned flags;        /* FR_PLAN_* */
} fr_plan_desc;

int fr_plan_create(const fr_plan_desc *desc, fr_plan *out_plan);
int fr_plan_destroy(fr_plan plan);

/* Bin a trajectory (device pointer, n Point<float> samples, raw k-space
 * coordinates).  Replaces ReconData::normalizeTraj + cuGridLut::plan.
 * Synchronises `stream` once (to size the bin lists). */
int fr_plan_set_trajectory(fr_plan plan, const float *d_traj, size_t n, void *stream);

/* Normalised trajectory (device, n x 4 floats) as ReconData::getTraj would
 * hold it after plan; component bounds before/after normalisation
 * (ReconData::getCompBounds, ReconData.h:31-33) as host floats lo[3],hi[3]. */
int fr_plan_normalized_trajectory(fr_plan plan, float *d_traj_out, void *stream);
int fr_plan_bounds(fr_plan plan, float *raw_lo, float *raw_hi, float *norm_lo, float *norm_hi);

/* Per-sample clamped cell ranges (device, n x 3 ints each), exactly the
 * start/end of GridLut.cpp:98-106; components >= dim are 0. */
int fr_plan_sample_ranges(fr_plan plan, int *d_start, int *d_end, void *stream);

/* Plan statistics: number of tiles, (sample, tile) pairs, work items and
 * split-tile partial slots.  Host ints. */
int fr_plan_stats(fr_plan plan, long long *tiles, long long *pairs, long long *items,
                  long long *partial_slots);

/* Tap lists of the current trajectory: 4-byte words per sample of the
 * plan's per-sample tap slots, or 0 when the plan keeps none (the scatter
 * then evaluates the taps of each bin record itself).  The plan evaluates
 * every sample's kernel taps once per trajectory (GridLut.cpp:120-136
 * geometry) -- the counterpart of cuGridLut::plan materialising (cell,
 * sample) pairs (cuGridLut.cu:50-113) -- in one word per tap. */
int fr_plan_tap_words(fr_plan plan, int *words_per_sample);

/* Sorted bin lists (device): tile_offset[tiles+1] (int64) and
 * pairs[pairs] (uint32 sample index), for bit-exact binning checks. */
int fr_plan_bins(fr_plan plan, long long *d_tile_offset, unsigned *d_pairs, void *stream);

/* Kernel timing (the reference prints per-stage wall times,
 * cuGridLut.cu:36-45; this is its device-side counterpart).  While enabled,
 * every fr_grid call records CUDA events on its stream around the tile
 * scatter kernel alone; fr_plan_profile_read waits for the last one and
 * returns the summed duration (ms) and launch count, then resets. */
int fr_plan_profile(fr_plan plan, int enable);
int fr_plan_profile_read(fr_plan plan, double *scatter_ms, int *launches);

/* Number of kernels this library has launched in the process (its own
 * kernels; cuFFT's are not counted). */
long long fr_kernel_launches(void);

/* ------------------------------------------------------------------------
 * Gridding: cuGridLut::execute / griddingChannel
 * (cuGridLut.cu:28-48,231-309; CPU oracle GridLut.cpp:80-147)
 * d_kdata: channels x n complex64; d_dcf: n floats; d_grid: channels x G^d
 * complex64, fully overwritten (cells no sample touches are written 0).
 * The scatter's waits on its bulk copies are bounded: one that expires sets
 * the plan's error word, and the plan's next fr_grid returns
 * FR_ERR_DEVICE_TIMEOUT (the grid of the call that expired is not valid).
 * ---------------------------------------------------------------------- */
int fr_grid(fr_plan plan, const float *d_kdata, const float *d_dcf, int channels,
            float *d_grid, void *stream);

/* ------------------------------------------------------------------------
 * Gridding in sample partitions: cuGridLut's partitioned plan
 * (cuGridLut::setNumOfPartitions, cuGridLut.h:40-42; cuGridLut.cu:128-149,
 * 182-220), for trajectories whose plan would not fit in device memory.
 *
 * Normalises the whole trajectory once (ReconData::normalizeTraj bounds,
 * ReconData.cpp:211-225, as fr_plan_set_trajectory would; skipped when
 * desc->flags holds FR_PLAN_PRENORMALIZED), zeroes d_grid,
 * then plans and grids consecutive ranges of `partition` samples with one
 * FR_PLAN_PRENORMALIZED | FR_PLAN_ACCUMULATE plan, each range's tiles added
 * to the grid.  Device memory beyond the caller's buffers: the normalised
 * trajectory (16 bytes per sample) plus a plan for `partition` samples.
 * d_kdata: channels x n complex64 (coil-major, as fr_grid); d_grid: channels
 * x G^d complex64, fully overwritten.  `partition` = 0 or >= n grids in one
 * plan.  The result equals fr_grid's to float rounding (each range's tile
 * sums are rounded to float before they are added).  Synchronises `stream`
 * once per range.
 * ---------------------------------------------------------------------- */
int fr_grid_partitioned(const fr_plan_desc *desc, const float *d_traj, size_t n, const float *d_kdata,
                        const float *d_dcf, int channels, float *d_grid, size_t partition, void *stream);

/* ------------------------------------------------------------------------
 * Gridding without device allocation.  No counterpart in the reference.
 *
 * For callers that cannot let a library allocate device memory during their
 * work -- a scanner's real-time reconstruction loop that reserves its memory
 * at start-up, or a host framework whose caching allocator already holds the
 * device memory.  Does what fr_plan_create (default tiling) +
 * fr_plan_set_trajectory + fr_grid do, with every plan and scatter buffer
 * taken from one fixed scratch array of FR_NOALLOC_SCRATCH_BYTES (32 MiB)
 * in device memory that each GPU loading the library holds until exit; it
 * calls no cudaMalloc or cudaFree.  Enough for a 2D radial trajectory of
 * 512 x 1024 samples (0.5 M) on a 512^2 grid; 1024 x 1024 is already too
 * large.  Larger trajectories, tile tables or split-tile partials are
 * rejected with FR_ERR_CAPACITY before any GPU work on them.
 * lut_length <= FR_NOALLOC_MAX_LUT.  The first call on a device looks the
 * scratch up (make it before any stream capture).  All calls share the
 * scratch: calls that overlap on the GPU (other streams or host threads) race.
 * Synchronises `stream` once.  Same arguments and output as fr_grid.
 * ---------------------------------------------------------------------- */
#define FR_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
#define FR_NOALLOC_MAX_LUT 1024
int fr_grid_noalloc(const float *d_traj, size_t n, int dim, unsigned grid_size, float kernel_width,
                    const float *lut_host, int lut_length, const float *d_kdata, const float *d_dcf, int channels,
                    float *d_grid, void *stream);

/* ------------------------------------------------------------------------
 * Batches: many frames (time frames of a dynamic scan, or volumes) with
 * uneven sample counts gridded in ONE persistent launch, replayable as a
 * captured CUDA graph.  No counterpart in the reference, which grids one
 * dataset per GridLut::execute (GridLut.cpp:53-78).
 *
 * Frame f owns samples [offsets[f], offsets[f+1]) of the concatenated raw
 * trajectory and is normalised with its own bounds (ReconData.cpp:201-225).
 * k-space: frame-major, frame f is a channels x n_f complex64 block at
 * complex offset channels * offsets[f]; DCF concatenated like the samples;
 * grid: frames x channels x G^d complex64.
 * ---------------------------------------------------------------------- */
typedef struct fr_batch_s *fr_batch;
int fr_batch_create(const fr_plan_desc *desc, fr_batch *out);
int fr_batch_destroy(fr_batch batch);
/* Plans every frame (synchronises `stream`); offsets has frames + 1 entries. */
int fr_batch_set_trajectories(fr_batch batch, const float *d_traj, const size_t *offsets, int frames, void *stream);
int fr_batch_stats(fr_batch batch, long long *frames, long long *samples, long long *items, long long *slots,
                   int *persistent_ctas);
int fr_batch_grid(fr_batch batch, const float *d_kdata, const float *d_dcf, int channels, float *d_grid,
                  void *stream);
/* Capture fr_batch_grid on `stream` (a created stream, not the legacy
 * default stream) into a CUDA graph bound to these buffers; fr_batch_replay
 * launches it (the buffers' contents are read at replay time). */
int fr_batch_capture(fr_batch batch, const float *d_kdata, const float *d_dcf, int channels, float *d_grid,
                     void *stream);
int fr_batch_replay(fr_batch batch, void *stream);
/* Times fr_batch_grid over tile shapes, bin chunks and coil groups on the
 * given data and returns the fastest descriptor (base supplies the rest). */
int fr_batch_autotune(const fr_plan_desc *base, const float *d_traj, const size_t *offsets, int frames,
                      const float *d_kdata, const float *d_dcf, int channels, float *d_grid, int repeats,
                      fr_plan_desc *best, float *best_ms, void *stream);

/* ------------------------------------------------------------------------
 * Density compensation and degridding.  No counterpart in the reference,
 * which reads its DCF from a file (ReconData.cpp:108-121).
 * ---------------------------------------------------------------------- */
/* |k|^power of the RAW coordinates (Point<float> per sample, before
 * normalisation): |k| = sqrt(x^2 + y^2 [+ z^2]) in double; power 1 -> |k|
 * (2D radial ramp), power 2 -> |k|*|k| (3D radial), else pow(|k|, power). */
int fr_dcf_analytic(const float *d_traj, size_t n, int dim, float power, float *d_dcf, void *stream);
/* Interpolate a channels x G^d complex grid at the plan's samples into
 * channels x n complex64 (the adjoint of fr_grid without DCF: same cell
 * range and LUT index; a checkerboard plan reads the grid with the same
 * (-1)^(x+y+z) signs). */
int fr_degrid(fr_plan plan, const float *d_grid, int channels, float *d_kdata, void *stream);
/* Streaming acquisition: ReconData::updateSingleAcquisition on the device
 * (ReconData.cpp:179-189, cuReconData.cu:52-62: copy one readout into each
 * channel at offset samples * acquisition and patch the device copy) plus
 * incremental regridding, so a grid made by fr_grid follows the data as
 * readouts arrive or are replaced without regridding every sample.
 * d_kdata: the channels x n complex64 k-space d_grid was made from (device,
 * coil-major, n = the plan's samples); d_new: channels x count complex64 new
 * values of samples [sample_begin, sample_begin + count) (one readout:
 * sample_begin = samples * acquisition, count = samples); d_dcf: the n DCF
 * values.  Adds dcf * (new - old) gridded with the plan's kernel (and its
 * checkerboard signs) into d_grid with global atomic adds, then copies
 * d_new into d_kdata.  d_grid then equals fr_grid of the updated k-space up
 * to float rounding (the adds' order is not fixed).  FR_ERR_SIZE_MISMATCH
 * when the range exceeds the plan's samples. */
int fr_grid_update(fr_plan plan, float *d_kdata, const float *d_new, size_t sample_begin, size_t count,
                   const float *d_dcf, int channels, float *d_grid, void *stream);
/* Real-valued gridding of per-sample weights into G^d floats (no DCF). */
int fr_grid_real(fr_plan plan, const float *d_w, float *d_grid, void *stream);
/* Pipe-Menon iterative DCF (MRM 41:179, 1999): `iterations` times
 * w <- w / degrid(grid(w)) on the plan's kernel; d_dcf holds the initial
 * weights (e.g. all 1) and receives the result.  Samples whose degridded
 * value is not positive keep their weight.  Stream-ordered, no host sync. */
int fr_dcf_pipe(fr_plan plan, int iterations, float *d_dcf, void *stream);

/* ------------------------------------------------------------------------
 * Learned DCF.  No counterpart in the reference.  A small network maps
 * sample-density features to log-DCF; it is trained on Pipe-Menon weights
 * (fr_dcf_pipe), which remain its fallback and its reference.
 * ---------------------------------------------------------------------- */
/* Density counts: each sample binned to its nearest cell (floor(x + 0.5) of
 * the plan's normalised coordinate, clamped); d_counts[s][k] (n x nradii
 * ints) = samples whose cell lies in the (2 r_k + 1)^d box around the cell
 * of s, clipped to the grid.  1 <= nradii <= 8.  Exact integers. */
int fr_density_counts(fr_plan plan, const int *radii, int nradii, int *d_counts, void *stream);
/* Network inputs, n x (nradii + 1) floats: log(count_k / (2 r_k + 1)^d) per
 * radius, then log(|k| / kmax + 1/1024) of the RAW coordinates (kmax <= 0:
 * the largest |k| of the trajectory, found on the device). */
int fr_dcf_features(fr_plan plan, const int *d_counts, const float *d_raw_traj, const int *radii, int nradii,
                    float kmax, float *d_features, void *stream);

/* The network: 5 -> 64 -> 64 -> 1, tanh hidden layers, BF16 parameters,
 * FP32 arithmetic.  Parameter layout (FR_MLP_PARAMS values):
 * W1[64][5] | b1[64] | W2[64][64] | b2[64] | W3[64] | b3. */
#define FR_MLP_IN 5
#define FR_MLP_HIDDEN 64
#define FR_MLP_PARAMS (64 * 5 + 64 + 64 * 64 + 64 + 64 + 1)
#define FR_MLP_EXP 1u      /* write scale * exp(output): the DCF instead of its log */
#define FR_MLP_RESIDUAL 2u /* the network predicts log-DCF + feature 1 (log density at radius 2):
                              subtract that feature from its output */
int fr_mlp_forward(const void *d_params_bf16, const float *d_features, size_t n, unsigned flags, float scale,
                   float *d_out, void *stream);
/* Workspace (16-byte aligned) for fr_mlp_backward on a batch of n samples. */
size_t fr_mlp_workspace_bytes(size_t n);
/* Weighted mean squared error (1/n) sum_s c_s (y_s - t_s)^2 of the output
 * against d_target over the batch (d_weight = NULL: all c_s = 1), and its
 * gradient with respect to the parameters (FR_MLP_PARAMS floats; the
 * reduction order is fixed, so the result is deterministic). */
int fr_mlp_backward(const void *d_params_bf16, const float *d_features, const float *d_target,
                    const float *d_weight, size_t n, void *d_workspace, float *d_grad, float *d_loss, void *stream);
/* One Adam step (step >= 1) on the FP32 master parameters; refreshes the
 * BF16 copy. */
int fr_mlp_adam(float *d_master, void *d_params_bf16, const float *d_grad, float *d_m, float *d_v, int count,
                float lr, float beta1, float beta2, float eps, int step, void *stream);
/* The BF16 copy of FP32 master parameters (round to nearest even). */
int fr_mlp_to_bf16(const float *d_master, void *d_params_bf16, int count, void *stream);

/* ------------------------------------------------------------------------
 * FFT stage: cuFFT::plan / cuFFT::excute (ImageFilter/cuFFT.cpp:15-37),
 * ImageFilter::fftPlan / fftExecute (ImageFilter.cpp:211-229).
 * In-place unnormalised C2C transform of `batch` contiguous images;
 * sign +1 = CUFFT_INVERSE / FFTW_BACKWARD (the reference default).
 * ---------------------------------------------------------------------- */
typedef struct fr_fft_s *fr_fft;
int fr_fft_create(int dim, const unsigned *size, int batch, int sign, fr_fft *out_fft);
int fr_fft_execute(fr_fft fft, float *d_data, void *stream);
int fr_fft_destroy(fr_fft fft);

/* Backward FFT + fftShift + crop + SOS in one pruned pass
 * (cuFFT.cpp:24-37, ImageFilter.cpp:40-53,159-209), for a grid flushed with
 * FR_PLAN_CHECKERBOARD (even G, G = 2^a 3^b 5^c <= 1024): only the centred
 * out_size crop is transformed through, and the last axis sums |x|^2 over the
 * channels in channel order, takes the square root and divides by d_deapod
 * (nullable, out_size floats).  d_out: out_size floats. */
typedef struct fr_fftcs_s *fr_fftcs;
int fr_fft_crop_sos_create(int dim, unsigned grid_size, int channels, const unsigned *out_size, fr_fftcs *out);
int fr_fft_crop_sos_execute(fr_fftcs f, const float *d_grid, const float *d_deapod, float *d_out, void *stream);
int fr_fft_crop_sos_destroy(fr_fftcs f);

/* ImageFilter::fftShift (ImageFilter.cpp:40-53,231-280) on `channels`
 * images of `size`, in place, with the reference's swap semantics (also for
 * odd sizes). */
int fr_fft_shift(float *d_imgs, int channels, int dim, const unsigned *size, void *stream);

/* ImageFilter::crop (ImageFilter.cpp:120-157): centred crop, offset
 * (size - crop)/2, of each channel into d_out (channels x crop complex). */
int fr_crop(const float *d_imgs, int channels, int dim, const unsigned *size,
            const unsigned *crop, float *d_out, void *stream);

/* ImageFilter::SOS(reconSize) + the |.| of Program/Main.cpp:177-180
 * (ImageFilter.cpp:159-209): centred crop, sum over channels of re^2+im^2
 * in channel order, sqrt.  d_out: recon-size floats.  d_deapod (nullable):
 * recon-size floats the magnitude is divided by (deapodization, absent in
 * the reference; NULL reproduces the reference). */
int fr_sos(const float *d_imgs, int channels, int dim, const unsigned *size,
           const unsigned *recon, const float *d_deapod, float *d_out, void *stream);

/* (m, 0) complex from n real values, device to device: the complex image the
 * reference's SOS leaves in channel 0 (ImageFilter.cpp:163-166). */
int fr_real_to_complex(const float *d_in, size_t n, float *d_out, void *stream);

/* PILS image operations (Program/Main.cpp:131-164), on channel images in
 * place, with the reference's float arithmetic:
 *   fr_low_filter  : ImageFilter::lowFilter(res)  (ImageFilter.cpp:55-93)
 *   fr_normalize_channels : ImageFilter::normalize (ImageFilter.cpp:95-118)
 *   fr_sos_map     : ImageFilter::SOS(map, reconSize) (ImageFilter.cpp:170-209),
 *                    sum over channels of x * conj(map) over the centred crop,
 *                    complex output (recon size), no square root. */
int fr_low_filter(float *d_imgs, int channels, int dim, const unsigned *size, int res, void *stream);
int fr_normalize_channels(float *d_imgs, int channels, int dim, const unsigned *size, void *stream);
int fr_sos_map(const float *d_imgs, const float *d_maps, int channels, int dim, const unsigned *size,
               const unsigned *recon, float *d_out, void *stream);

/* ------------------------------------------------------------------------
 * Whole reconstruction (Program/Main.cpp:101-181 without file I/O):
 * normalise + bin, grid, backward FFT, shift, crop + SoS (+ optional
 * deapodization), magnitude.
 * ---------------------------------------------------------------------- */
typedef struct fr_recon_s *fr_recon;

enum {
    FR_RECON_DEAPODIZE = 1u << 0, /* divide by the kernel's image-domain apodization */
    FR_RECON_CUFFT = 1u << 1,     /* always the full cuFFT transform + crop/SoS kernel */
    FR_RECON_PRUNED_FFT = 1u << 2, /* the pruned transform with fused crop + SoS (fr_fft_crop_sos)
                                     wherever it applies (even G = 2^a 3^b 5^c <= 1024); by default
                                     it is used for the grid sizes it has specialised passes for
                                     (64, 128, 160, 192, 240, 256, 320, 384, 480, 512, 640, 768, 1024) */
    FR_RECON_DETERMINISTIC = 1u << 3 /* plan with FR_PLAN_DETERMINISTIC: bit-reproducible images */
};

typedef struct {
    int dim;                 /* 2 or 3 */
    unsigned recon_size;     /* rcxres: G = unsigned(recon_size * overgrid_factor) */
    float overgrid_factor;   /* os */
    float kernel_width;      /* W */
    int lut_length;          /* L (512 in Program/Main.cpp:127) */
    unsigned out_size[3];    /* rcxres, rcyres, rczres (z = 1 in 2D) */
    int channels;            /* coils */
    size_t max_samples;      /* capacity for n */
    int tile[3];             /* 0 = default */
    int coil_group;          /* 0 = default */
    unsigned flags;          /* FR_RECON_* */
    size_t grid_budget;      /* out-of-core coils (cuGridLut's partitions, cuGridLut.cu:128-149,182-220,
                                bound the memory of its pair map; here the grid is the large buffer):
                                0 = grid all coils at once; else coils are gridded and transformed in
                                slabs whose complex grid fits grid_budget bytes (at least one coil per
                                slab), the |x|^2 of each slab added to the image in coil order, so the
                                image equals the single-slab one while the grid workspace shrinks from
                                channels x G^d x 8 to slab x G^d x 8 bytes */
} fr_recon_desc;

/* One fr_recon object holds one plan and one grid workspace: give all its
 * calls the same stream (calls on other streams or host threads race), or
 * use one object per stream.  fr_recon_destroy waits for its submitted
 * volumes. */
int fr_recon_create(const fr_recon_desc *desc, fr_recon *out);
int fr_recon_destroy(fr_recon r);
/* Device buffers: d_traj n x 4 raw coordinates, d_dcf n, d_kdata channels x n
 * complex64, d_image out_size floats (|SoS|).  Re-bins the trajectory. */
int fr_recon_run(fr_recon r, const float *d_traj, const float *d_dcf, const float *d_kdata,
                 size_t n, float *d_image, void *stream);
/* Same with HOST buffers (pinned for full speed): the host->device copies of
 * the inputs and the device->host copy of the image are part of the call,
 * which returns once the image is in h_image. */
int fr_recon_run_host(fr_recon r, const float *h_traj, const float *h_dcf, const float *h_kdata,
                      size_t n, float *h_image, void *stream);
/* Pipelined form of fr_recon_run_host for a sequence of volumes (no
 * counterpart in the reference, whose program reconstructs one data set per
 * run): queues the upload of the inputs, the recon on `stream` and the
 * download of the image, and returns without waiting.  Two device staging
 * slots alternate, so the upload of one volume and the download of the
 * previous image overlap the recon of the one in between.  The copies may
 * still be reading h_traj, h_dcf and h_kdata, and writing h_image, after this
 * call returns: every one of these host buffers (pinned for overlap) must
 * stay valid, the inputs unmodified, and h_image unread, until fr_recon_sync
 * returns; the images are fr_recon_run_host's. */
int fr_recon_submit_host(fr_recon r, const float *h_traj, const float *h_dcf, const float *h_kdata,
                         size_t n, float *h_image, void *stream);
/* Waits until every submitted volume's image is in its host buffer. */
int fr_recon_sync(fr_recon r, void *stream);
/* Plan object and grid workspace used by the recon (for stage timing). */
int fr_recon_plan(fr_recon r, fr_plan *out_plan);
/* Stage timings of the last fr_recon_run* call in ms (plan, grid, fft, sos),
 * measured with CUDA events when FR_TIMING=1 in the environment, else -1.
 * No counterpart in the reference, which prints its stages' wall times. */
int fr_recon_stage_ms(fr_recon r, float *plan_ms, float *grid_ms, float *fft_ms, float *sos_ms);

#ifdef __cplusplus
}
#endif
#endif /* FASTRECON_GB300_H */
