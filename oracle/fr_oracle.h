/*
 * fr_oracle.h -- CPU oracle for the fastrecon gridding/recon path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * CPU algorithm (pengwg/fastrecon, ReconData/GridLut.cpp, ReconData/ConvKernel.cpp,
 * ReconData/ReconData.cpp, ImageFilter/ImageFilter.cpp).  It is used by the
 * tests as the checker, by __graft_entry__.smoke() as the checker and by
 * bench.py as the timed CPU baseline.  The product library never links,
 * loads or calls it.
 *
 * Parity pin: the restatement is checked bit-for-bit against the reference's
 * own CPU sources compiled in oracle/ref_shim (oracle/_ref/libfastrecon_ref.so)
 * and against fixtures generated from that build (tests/golden/).
 *
 * Data layouts (all identical to the reference's in-memory layouts):
 *   traj   : Point<float>{x[4]} per sample, 16 bytes, sample-major (ReconData.h:12-15)
 *   dcf    : float per sample
 *   kdata  : channel-major, each channel N complex64 (re, im interleaved)
 *   grid   : channel-major, each channel G^d complex64, x fastest (GridLut.cpp:224)
 */
#ifndef FR_ORACLE_H
#define FR_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Modified Bessel function I0 in double precision (power series,
 * Abramowitz & Stegun 9.6.12).  Stand-in for GSL gsl_sf_bessel_I0, which the
 * reference calls at ConvKernel.cpp:23.  NaN in -> NaN out. */
double orc_bessel_i0(double x);

/* Kaiser-Bessel radial LUT, ConvKernel::ConvKernel (ConvKernel.cpp:7-30),
 * same float/double mix as the reference.  Returns 0 on success. */
int orc_kb_lut(float kWidth, float overGridFactor, int length, float *out);

/* Per-component bounds as ReconData::loadTraj accumulates them
 * (ReconData.cpp:159-167).  lo/hi have dim entries. */
void orc_comp_bounds(const float *traj, size_t n, int dim, float *lo, float *hi);

/* ReconData::normalizeTraj + transformLocalTraj (ReconData.cpp:201-225):
 * tr = -lo[0], s = (G-1)/(hi[0]-lo[0]) in float; x <- (x + tr) * s for every
 * component < dim.  lo/hi are updated in place like m_bounds. */
void orc_normalize_traj(float *traj, size_t n, int dim, unsigned G, float *lo, float *hi,
                        float *tr_out, float *scale_out);

/* Per-sample clamped cell range, GridLut::griddingChannel (GridLut.cpp:98-106).
 * start/end are n*3 ints; components >= dim are 0/0 like the reference's
 * zero-initialised arrays.  Non-finite centres yield an empty range
 * (start > end), which is what the reference's x86 build produces. */
void orc_sample_range(const float *traj, size_t n, int dim, unsigned G, float kHW,
                      int *start, int *end);

/* LUT index the reference uses for one tap (GridLut.cpp:131-136), or -1 if
 * the tap is outside the kernel radius. */
int orc_tap_lut_index(float dx, float dy, float dz, float kHW, int klength);

/* The same LUT index from s = dz^2 + dy^2 + dx^2 directly, for n values:
 * out[i] = roundf(sqrtf(s[i]) / kHW * (klength - 1)) or -1 when
 * sqrtf(s[i]) >= kHW (GridLut.cpp:131-136). */
void orc_lut_index_of_s(const float *s, size_t n, float kHW, int klength, int *out);

/* One channel of GridLut::griddingChannel (GridLut.cpp:80-147), FP32,
 * sequential in sample order.  out is G^d complex, overwritten. */
void orc_grid_channel(const float *traj, const float *dcf, const float *kdata, size_t n,
                      int dim, unsigned G, float kWidth, const float *lut, int klength,
                      float *out);

/* GridLut::execute (GridLut.cpp:53-78): all channels, OpenMP over channels
 * with `threads` threads.  out is channels*G^d complex. */
void orc_grid(const float *traj, const float *dcf, const float *kdata, size_t n,
              int channels, int dim, unsigned G, float kWidth, const float *lut,
              int klength, float *out, int threads);

/* FP64 gridding oracle: same geometry and LUT index as the reference, weights
 * and accumulation in double.  out is G^d complex double. */
void orc_grid_channel_f64(const float *traj, const float *dcf, const float *kdata, size_t n,
                          int dim, unsigned G, float kWidth, const float *lut, int klength,
                          double *out);

/* orc_grid with each channel split over `threads` threads by bands of the
 * last grid axis (z in 3D, y in 2D) instead of one thread per channel: every
 * thread walks all samples in sample order and adds only the taps inside its
 * band, so every cell gets the reference's adds in the reference's order and
 * the result is bit-for-bit that of orc_grid.  For full-size checks. */
void orc_grid_bands(const float *traj, const float *dcf, const float *kdata, size_t n,
                    int channels, int dim, unsigned G, float kWidth, const float *lut,
                    int klength, float *out, int threads);

/* The FP64 gridding oracle for all channels, split into bands the same way
 * (bit-for-bit orc_grid_channel_f64 per channel).  out: channels*G^d complex
 * double. */
void orc_grid_f64_bands(const float *traj, const float *dcf, const float *kdata, size_t n,
                        int channels, int dim, unsigned G, float kWidth, const float *lut,
                        int klength, double *out, int threads);

/* Per-sample kernel mass: sum over the sample's valid taps of lut[ki], with
 * the reference geometry (GridLut.cpp:98-136), in double.  Gridding is
 * linear, so sum_cells grid[c] = sum_s dcf[s]*kdata[c][s]*mass[s]: a
 * size-independent checksum for full-size runs.  OpenMP over samples. */
void orc_sample_mass(const float *traj, size_t n, int dim, unsigned G, float kWidth,
                     const float *lut, int klength, double *mass, int threads);

/* Tiles touched by each sample for a tile shape (tx,ty,tz): fills, per
 * sample, lo/hi tile coordinates (n*3 each).  Empty samples get lo > hi on
 * axis 0.  Used to check the device bin lists bit-for-bit. */
void orc_sample_tiles(const int *start, const int *end, size_t n, int dim,
                      const int *tile_shape, int *tlo, int *thi);

/* In-place d-dimensional complex FFT of `batch` contiguous arrays, x fastest,
 * unnormalised, e^{sign*2*pi*i*k*n/N} (sign=+1 is FFTW_BACKWARD /
 * CUFFT_INVERSE as used at FFT.cpp:45-47 and cuFFT.cpp:33).  Mixed radix,
 * computed in double.  Stand-in for FFTW3f, absent on this system. */
int orc_fft(float *data, int dim, const unsigned *size, int batch, int sign, int threads);

/* ImageFilter::fftShift2 / fftShift3 (ImageFilter.cpp:231-280): the
 * reference's swap sequence, exactly (also for odd sizes). */
void orc_fft_shift(float *data, int dim, const unsigned *size);

/* ImageFilter::SOS(reconSize) (ImageFilter.cpp:159-209): centred crop with
 * offset (size-recon)/2, sum over channels of x*conj(x) in complex float in
 * channel order, then complex sqrt.  out is recon-size complex. */
void orc_sos(const float *imgs, int channels, int dim, const unsigned *size,
             const unsigned *recon, float *out);

/* PILS operations, in place on `channels` images of `size`:
 * ImageFilter::lowFilter(res) (ImageFilter.cpp:55-93), ImageFilter::normalize
 * (ImageFilter.cpp:95-118).  orc_sos_map is ImageFilter::SOS(map, reconSize)
 * (ImageFilter.cpp:170-209): centred crop, sum over channels of x*conj(map),
 * complex output, no square root. */
void orc_low_filter(float *imgs, int channels, int dim, const unsigned *size, int res);
void orc_normalize_channels(float *imgs, int channels, int dim, const unsigned *size);
void orc_sos_map(const float *imgs, const float *maps, int channels, int dim, const unsigned *size,
                 const unsigned *recon, float *out);

/* The whole reference pipeline (Program/Main.cpp:101-181) without I/O:
 * normalizeTraj, grid, backward FFT, fftShift, SOS, |.| -> float image.
 * traj is modified in place (as the reference does).  Returns 0 on success. */
int orc_recon(float *traj, const float *dcf, const float *kdata, size_t n, int channels,
              int dim, unsigned reconSize, float os, float kWidth, int klength,
              const unsigned *recon, float *out_mag, int threads);

/* ---- fr_oracle_ext.c: components with no counterpart in the reference ---- */

/* |k|^power of the raw coordinates: |k| = sqrt(sum x_d^2) in double; power 1
 * gives |k|, power 2 gives |k|*|k|, otherwise pow(|k|, power); rounded to float. */
void orc_dcf_analytic(const float *traj, size_t n, int dim, double power, float *out);

/* Degridding (interpolation), the adjoint of gridding without DCF:
 * out[c][s] = sum over the sample's valid taps of lut[ki] * grid[c][cell].
 * grid: channels x G^d complex (double pairs); out: channels x n complex. */
void orc_degrid_f64(const float *traj, size_t n, int dim, unsigned G, float kWidth, const float *lut,
                    int klength, const double *grid, int channels, double *out);

/* Real-valued gridding of weights w (no DCF) into grid (G^d doubles). */
void orc_grid_real_f64(const float *traj, const double *w, size_t n, int dim, unsigned G, float kWidth,
                       const float *lut, int klength, double *grid);

/* Pipe-Menon iteration, `iterations` times: w <- w / degrid(grid(w)); samples
 * whose degridded value is not positive keep their weight.  w in/out. */
int orc_dcf_pipe_f64(const float *traj, size_t n, int dim, unsigned G, float kWidth, const float *lut,
                     int klength, int iterations, double *w);

/* Sample-density counts: every sample is binned to its nearest cell
 * (floor(x + 0.5), clamped to the grid); counts[s][k] = samples whose cell
 * lies in the (2 r_k + 1)^d box around the cell of s, clipped to the grid. */
int orc_density_counts(const float *traj, size_t n, int dim, unsigned G, const int *radii, int nradii,
                       int *counts);

/* Network inputs: log(count_k / (2 r_k + 1)^d) for each radius, then
 * log(|k| / kmax + 1/1024) of the raw coordinates.  feat: n x (nradii + 1). */
void orc_dcf_features(const int *counts, const float *raw_traj, size_t n, int dim, const int *radii, int nradii,
                      float kmax, float *feat);

/* DCF network: 5 -> 64 -> 64 -> 1, tanh, predicting log-DCF.
 * Parameters (float): W1[64][5] | b1[64] | W2[64][64] | b2[64] | W3[64] | b3. */
#define ORC_MLP_IN 5
#define ORC_MLP_HIDDEN 64
#define ORC_MLP_PARAMS (64 * 5 + 64 + 64 * 64 + 64 + 64 + 1)
void orc_mlp_forward(const float *params, const float *x, size_t n, double *y);
/* The same minus feature 1 (a network trained on log-DCF + log density). */
void orc_mlp_forward_residual(const float *params, const float *x, size_t n, double *y);
/* Weighted mean squared error (1/n) sum c_s (y_s - t_s)^2 (weight NULL: c = 1)
 * and its gradient (ORC_MLP_PARAMS doubles). */
double orc_mlp_backward(const float *params, const float *x, const float *target, const float *weight, size_t n,
                        double *grad);

#ifdef __cplusplus
}
#endif
#endif /* FR_ORACLE_H */
