// Library stand-ins the reference's CPU sources link against (GSL I0 and
// the FFTW3f calls of FFT.cpp), implemented by the oracle.  Test
// infrastructure: linked only into oracle/_ref/libfastrecon_ref.so.
#include <cstdlib>
#include <cstring>
#include "fftw3.h"
#include "gsl/gsl_sf_bessel.h"
#include "../fr_oracle.h"

extern "C" double gsl_sf_bessel_I0(double x) { return orc_bessel_i0(x); }

struct fr_fftwf_plan_s {
    int dim;
    unsigned size[3];  // x fastest
    fftwf_complex *in, *out;
    int sign;
};

extern "C" void *fftwf_malloc(size_t n) { return std::malloc(n); }
extern "C" void fftwf_free(void *p) { std::free(p); }

extern "C" fftwf_plan fftwf_plan_dft_2d(int n0, int n1, fftwf_complex *in, fftwf_complex *out,
                                        int sign, unsigned)
{
    auto p = new fr_fftwf_plan_s;
    p->dim = 2;
    p->size[0] = (unsigned)n1;  // row-major: last dimension fastest
    p->size[1] = (unsigned)n0;
    p->size[2] = 1;
    p->in = in;
    p->out = out;
    p->sign = sign;
    return p;
}

extern "C" fftwf_plan fftwf_plan_dft_3d(int n0, int n1, int n2, fftwf_complex *in,
                                        fftwf_complex *out, int sign, unsigned)
{
    auto p = new fr_fftwf_plan_s;
    p->dim = 3;
    p->size[0] = (unsigned)n2;
    p->size[1] = (unsigned)n1;
    p->size[2] = (unsigned)n0;
    p->in = in;
    p->out = out;
    p->sign = sign;
    return p;
}

extern "C" void fftwf_execute(const fftwf_plan p)
{
    size_t total = (size_t)p->size[0] * p->size[1] * p->size[2];
    if (p->out != p->in)
        std::memcpy(p->out, p->in, total * sizeof(fftwf_complex));
    // One thread per plan: FFT.cpp already runs one plan per OpenMP thread.
    orc_fft(reinterpret_cast<float *>(p->out), p->dim, p->size, 1, p->sign, 1);
}

extern "C" void fftwf_destroy_plan(fftwf_plan p) { delete p; }
