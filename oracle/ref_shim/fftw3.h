/* Minimal stand-in for <fftw3.h>: header.h (reference) only names these two
 * types in prototypes of misfit routines that the oracle does not compile. */
#ifndef ORC_FFTW3_SHIM_H
#define ORC_FFTW3_SHIM_H
typedef float fftwf_complex[2];
typedef void *fftwf_plan;
#endif
