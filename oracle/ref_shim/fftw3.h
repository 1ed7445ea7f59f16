/* Stand-in for the part of FFTW3 single precision that FFT.cpp uses
 * (FFT.cpp:30-52,83), backed by the oracle's double-precision FFT.
 * Test infrastructure. */
#ifndef FR_SHIM_FFTW3_H
#define FR_SHIM_FFTW3_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_DESTROY_INPUT (1U << 0)
typedef float fftwf_complex[2];
typedef struct fr_fftwf_plan_s *fftwf_plan;
void *fftwf_malloc(size_t n);
void fftwf_free(void *p);
fftwf_plan fftwf_plan_dft_2d(int n0, int n1, fftwf_complex *in, fftwf_complex *out, int sign,
                             unsigned flags);
fftwf_plan fftwf_plan_dft_3d(int n0, int n1, int n2, fftwf_complex *in, fftwf_complex *out,
                             int sign, unsigned flags);
void fftwf_execute(const fftwf_plan p);
void fftwf_destroy_plan(fftwf_plan p);
#ifdef __cplusplus
}
#endif
#endif
