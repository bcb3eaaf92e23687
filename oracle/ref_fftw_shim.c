/*
 * ref_fftw_shim.c -- the FFTW 3 (single precision) and CBLAS entry points that
 * the reference's xcorr_msf.c calls, restated from their published
 * definitions so that the reference's XCORR1D compiles and runs here
 * (TEST INFRASTRUCTURE ONLY; built into oracle/_ref by `make ref`).
 *
 * The DFTs are evaluated directly in double precision (O(n^2)), i.e. the
 * exact transforms that FFTW approximates; cblas_sdot accumulates in single
 * precision from the first element on.
 */
#include <math.h>
#include <stdlib.h>
#include "fftw3.h"

struct orc_fftwf_plan_s { int n; };

void *fftwf_malloc(size_t n) { return malloc(n); }
void fftwf_free(void *p) { free(p); }

static fftwf_plan make_plan(int n)
{
    fftwf_plan p = malloc(sizeof(*p));
    if (p) p->n = n;
    return p;
}
fftwf_plan fftwf_plan_dft_r2c_1d(int n, float *in, fftwf_complex *out, unsigned flags)
{
    (void)in; (void)out; (void)flags;
    return make_plan(n);
}
fftwf_plan fftwf_plan_dft_c2r_1d(int n, fftwf_complex *in, float *out, unsigned flags)
{
    (void)in; (void)out; (void)flags;
    return make_plan(n);
}
void fftwf_destroy_plan(fftwf_plan p) { free(p); }

/* X[k] = sum_j x[j] exp(-2 pi i j k / n), k = 0 .. n/2 */
void fftwf_execute_dft_r2c(const fftwf_plan p, float *in, fftwf_complex *out)
{
    const int n = p->n;
    const double w = -2.0 * M_PI / n;
    for (int k = 0; k <= n / 2; k++) {
        double re = 0, im = 0;
        for (int j = 0; j < n; j++) {
            const long long jk = ((long long)j * k) % n;
            re += in[j] * cos(w * jk);
            im += in[j] * sin(w * jk);
        }
        out[k][0] = (float)re;
        out[k][1] = (float)im;
    }
}

/* x[j] = sum_{k=0}^{n-1} X[k] exp(+2 pi i j k / n) with X[n-k] = conj(X[k]) */
void fftwf_execute_dft_c2r(const fftwf_plan p, fftwf_complex *in, float *out)
{
    const int n = p->n;
    const double w = 2.0 * M_PI / n;
    for (int j = 0; j < n; j++) {
        double acc = in[0][0];
        for (int k = 1; k < (n + 1) / 2; k++) {
            const long long jk = ((long long)j * k) % n;
            acc += 2.0 * (in[k][0] * cos(w * jk) - in[k][1] * sin(w * jk));
        }
        if (n % 2 == 0) acc += in[n / 2][0] * ((j % 2) ? -1.0 : 1.0);
        out[j] = (float)acc;
    }
}

float cblas_sdot(const int n, const float *x, const int incx, const float *y, const int incy)
{
    float s = 0.0f;
    for (int i = 0; i < n; i++) s += x[(size_t)i * incx] * y[(size_t)i * incy];
    return s;
}
