/* Stand-in for GSL's gsl_sf_bessel_I0 (the only GSL call on the path,
 * ConvKernel.cpp:23).  Implemented by the oracle's power series.  Test
 * infrastructure. */
#ifndef FR_SHIM_GSL_SF_BESSEL_H
#define FR_SHIM_GSL_SF_BESSEL_H
#ifdef __cplusplus
extern "C" {
#endif
double gsl_sf_bessel_I0(double x);
#ifdef __cplusplus
}
#endif
#endif
