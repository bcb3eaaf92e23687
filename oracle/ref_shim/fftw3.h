/* Stand-in for <fftw3.h> (FFTW 3, single precision; not installed here and
 * not vendored by the reference, which pins no version).  header.h names the
 * types in prototypes; xcorr_msf.c also calls the functions below, which
 * oracle/ref_fftw_shim.c implements from the published definition of FFTW's
 * unnormalised real DFTs (r2c: X[k] = sum_j x[j] e^{-2 pi i jk/n},
 * k = 0..n/2; c2r: the inverse sum over the Hermitian extension, without
 * the 1/n factor). */
#ifndef ORC_FFTW3_SHIM_H
#define ORC_FFTW3_SHIM_H
#include <stddef.h>
typedef float fftwf_complex[2];
typedef struct orc_fftwf_plan_s *fftwf_plan;
#define FFTW_ESTIMATE (1U << 6)
void *fftwf_malloc(size_t n);
void fftwf_free(void *p);
fftwf_plan fftwf_plan_dft_r2c_1d(int n, float *in, fftwf_complex *out, unsigned flags);
fftwf_plan fftwf_plan_dft_c2r_1d(int n, fftwf_complex *in, float *out, unsigned flags);
void fftwf_execute_dft_r2c(const fftwf_plan p, float *in, fftwf_complex *out);
void fftwf_execute_dft_c2r(const fftwf_plan p, fftwf_complex *in, float *out);
void fftwf_destroy_plan(fftwf_plan p);
/* CBLAS single-precision dot product (xcorr_msf.c:127-128) */
float cblas_sdot(const int n, const float *x, const int incx, const float *y, const int incy);
#endif
