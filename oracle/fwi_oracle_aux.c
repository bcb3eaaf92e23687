/*
 * fwi_oracle_aux.c -- CPU oracle for the routines around the gradient:
 * gradient preconditioning (grad_precond_new5 + triangle2), the Butterworth
 * band-pass (sfbandpass) and the cross-correlation misfit (XCORR1D).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the device versions.  Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU baseline may load it.
 *
 * Each function restates the reference's FP32 arithmetic operation by
 * operation (same loop order, same float/double promotions; compiled with
 * -ffp-contract=off), so that
 *   - orc_triangle2 / orc_grad_precond equal triangle_smooth.c:5-110 and
 *     grad_prec.c:5-52 bit for bit;
 *   - orc_butter_init / orc_bandpass equal butterworth_filter.c:32-200 bit
 *     for bit;
 *   - orc_xcorr1d follows xcorr_msf.c:4-181, except that the two
 *     correlations the reference evaluates with single-precision FFTs are
 *     evaluated here as direct sums in double precision (the exact values the
 *     FFTs approximate), so it agrees with the reference to FFT rounding.
 * tests/test_oracle_aux.py checks all of this against the reference sources
 * compiled by `make ref` and against the fixtures in tests/golden/.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* PI as butterworth_filter.c sees it: Mpar.h defines it first, fwi_sys.h
 * (included second) redefines it to this value, which wins. */
#define ORC_PI 3.141592654

/* ---- triangle smoothing (triangle_smooth.c:5-110) ----------------------- */

/* Box convolution: prefix sums, then differences at distance nb
 * (triangle_smooth.c:5-34); yy has nx+nb-1 entries. */
static void box_conv(int nb, int nx, const float *xx, float *yy, float *bb)
{
    const int ny = nx + nb - 1;
    bb[0] = xx[0];
    for (int i = 1; i < nx; i++) bb[i] = bb[i - 1] + xx[i];
    for (int i = nx; i < ny; i++) bb[i] = bb[i - 1];
    for (int i = 0; i < nb; i++) yy[i] = bb[i];
    for (int i = nb; i < ny; i++) yy[i] = bb[i] - bb[i - nb];
}

/* Triangle filter of half-width nr on one line of n12 samples, edges folded
 * back (triangle_smooth.c:36-68). */
static void triangle_line(int nr, int n12, const float *uu, float *vv, float *work)
{
    const int np = nr + n12 - 1, nq = nr + np - 1;
    float *pp = work, *qq = pp + np, *tt = qq + nq, *bb = tt + n12;
    memset(qq, 0, sizeof(float) * nq);
    for (int i = 0; i < n12; i++) qq[i] = uu[i];
    box_conv(nr, n12, qq, pp, bb);
    box_conv(nr, np, pp, qq, bb);
    for (int i = 0; i < n12; i++) tt[i] = qq[i + nr - 1];
    for (int i = 0; i < nr - 1; i++) tt[i] = tt[i] + qq[nr - (i + 2)];
    for (int i = 0; i < nr - 1; i++) tt[n12 - (i + 2) + 1] = tt[n12 - (i + 2) + 1] + qq[np + i];
    const int nr2 = nr * nr;
    for (int i = 0; i < n12; i++) vv[i] = tt[i] / nr2;
}

/* Scratch floats triangle_line needs for a line of n samples. */
static size_t triangle_work(int nr, int n) { return (size_t)4 * (n + 2 * nr) + 8; }

/* triangle2 (triangle_smooth.c:70-110): rect1 along the fast axis n1, nt
 * times, then rect2 along n2, nt times. */
int orc_triangle2(int rect1, int rect2, int nt, int n1, int n2, const float *uu, float *vv)
{
    const int nmax = n1 > n2 ? n1 : n2, rmax = rect1 > rect2 ? rect1 : rect2;
    float *line = malloc(sizeof(float) * 2 * nmax);
    float *work = malloc(sizeof(float) * triangle_work(rmax, nmax));
    if (!line || !work) { free(line); free(work); return -3; }
    float *rr = line, *tmp = line + nmax;
    memcpy(vv, uu, sizeof(float) * (size_t)n1 * n2);
    for (int it = 0; it < nt; it++)
        for (int i2 = 0; i2 < n2; i2++) {
            for (int i1 = 0; i1 < n1; i1++) rr[i1] = vv[i2 * n1 + i1];
            triangle_line(rect1, n1, rr, tmp, work);
            for (int i1 = 0; i1 < n1; i1++) vv[i2 * n1 + i1] = tmp[i1];
        }
    for (int it = 0; it < nt; it++)
        for (int i1 = 0; i1 < n1; i1++) {
            for (int i2 = 0; i2 < n2; i2++) rr[i2] = vv[i2 * n1 + i1];
            triangle_line(rect2, n2, rr, tmp, work);
            for (int i2 = 0; i2 < n2; i2++) vv[i2 * n1 + i1] = tmp[i2];
        }
    free(line);
    free(work);
    return 0;
}

/* grad_precond_new5 (grad_prec.c:5-52) on body[mnz][mnx] in place:
 * clip to perc * (min, max) when perc != 0, triangle2(rectx1, rectx1,
 * repeat1), zero above bottom[ix], triangle2(rectx2, rectx2, repeat2),
 * scale by alpha_grad. */
int orc_grad_precond(float *body, int mnx, int mnz, float perc, int rectx1, int repeat1,
                     int rectx2, int repeat2, float alpha_grad, const int *bottom)
{
    const size_t n = (size_t)mnx * mnz;
    float *tmp = malloc(sizeof(float) * n), *sm = malloc(sizeof(float) * n);
    if (!tmp || !sm) { free(tmp); free(sm); return -3; }
    memcpy(tmp, body, sizeof(float) * n);
    /* argmin / argmax with flt_cmp (min_max.c): the first extreme value */
    float vmin = tmp[0], vmax = tmp[0];
    for (size_t i = 1; i < n; i++) {
        if (vmin > tmp[i]) vmin = tmp[i];
        if (tmp[i] > vmax) vmax = tmp[i];
    }
    if (perc != 0) {
        for (size_t i = 0; i < n; i++) {
            if (tmp[i] > vmax * perc) tmp[i] = vmax * perc;
            if (tmp[i] < vmin * perc) tmp[i] = vmin * perc;
        }
    }
    int s = orc_triangle2(rectx1, rectx1, repeat1, mnx, mnz, tmp, sm);
    if (!s) {
        for (int iz = 0; iz < mnz; iz++)
            for (int ix = 0; ix < mnx; ix++)
                if (iz < bottom[ix]) sm[(size_t)iz * mnx + ix] = 0;
        s = orc_triangle2(rectx2, rectx2, repeat2, mnx, mnz, sm, tmp);
    }
    if (!s)
        for (size_t i = 0; i < n; i++) body[i] = tmp[i] * alpha_grad;
    free(tmp);
    free(sm);
    return s;
}

/* ---- Butterworth band-pass (butterworth_filter.c:32-200) ---------------- */

/* sf_butter_init (butterworth_filter.c:32-70): den[(nn+1)/2][2] and mid. */
void orc_butter_init(int low, float cutoff, int nn, float *den, float *mid)
{
    float arg, ss, sinw, cosw, fact;
    arg = 2. * ORC_PI * cutoff;
    sinw = sin(arg);
    cosw = cos(arg);
    if (nn % 2) {
        if (low) {
            fact = (1. + cosw) / sinw;
            den[2 * (nn / 2)] = 1. / (1. + fact);
            den[2 * (nn / 2) + 1] = 1. - fact;
        } else {
            fact = sinw / (1. + cosw);
            den[2 * (nn / 2)] = 1. / (fact + 1.);
            den[2 * (nn / 2) + 1] = fact - 1.;
        }
    }
    fact = low ? sin(0.5 * arg) : cos(0.5 * arg);
    fact *= fact;
    for (int j = 0; j < nn / 2; j++) {
        ss = sin(ORC_PI * (2 * j + 1) / (2 * nn)) * sinw;
        den[2 * j] = fact / (1. + ss);
        den[2 * j + 1] = (1. - ss) / fact;
    }
    *mid = -2. * cosw / fact;
}

/* sf_butter_apply (butterworth_filter.c:84-117) on one trace in place. */
static void butter_apply(int low, int nn, const float *den, float mid, int nx, float *x)
{
    float d0, d1, d2, x0, x1, x2, y0, y1, y2;
    d1 = mid;
    if (nn % 2) {
        d0 = den[2 * (nn / 2)];
        d2 = den[2 * (nn / 2) + 1];
        x0 = y1 = 0.;
        for (int ix = 0; ix < nx; ix++) {
            x1 = x0; x0 = x[ix];
            y0 = low ? (x0 + x1 - d2 * y1) * d0 : (x0 - x1 - d2 * y1) * d0;
            x[ix] = y1 = y0;
        }
    }
    for (int j = 0; j < nn / 2; j++) {
        d0 = den[2 * j];
        d2 = den[2 * j + 1];
        x1 = x0 = y1 = y2 = 0.;
        for (int ix = 0; ix < nx; ix++) {
            x2 = x1; x1 = x0; x0 = x[ix];
            y0 = low ? (x0 + 2 * x1 + x2 - d1 * y1 - d2 * y2) * d0 : (x0 - 2 * x1 + x2 - d1 * y1 - d2 * y2) * d0;
            y2 = y1; x[ix] = y1 = y0;
        }
    }
}

static void reverse_trace(int n, float *t)
{
    for (int i = 0; i < n / 2; i++) { float v = t[i]; t[i] = t[n - 1 - i]; t[n - 1 - i] = v; }
}

/* sfbandpass (butterworth_filter.c:127-200) of nr traces of nt samples.
 * Returns -1 for flo < 0 (where the reference exits). */
int orc_bandpass(const float *indat, int nt, int nr, float dt, int phase, int nphi, int nplo,
                 float fhi, float flo, float *outdat)
{
    const float eps = 0.0001;
    if (0. > flo) return -1;
    flo *= dt;
    fhi *= dt;
    if (nplo < 1) nplo = 1;
    if (nplo > 1 && !phase) nplo /= 2;
    if (nphi < 1) nphi = 1;
    if (nphi > 1 && !phase) nphi /= 2;
    float *dlo = calloc((size_t)(nplo + 1), sizeof(float)), *dhi = calloc((size_t)(nphi + 1), sizeof(float));
    float *trace = calloc((size_t)nt, sizeof(float));
    if (!dlo || !dhi || !trace) { free(dlo); free(dhi); free(trace); return -3; }
    float mlo = 0, mhi = 0;
    const int use_lo = flo > eps, use_hi = fhi < 0.5 - eps;
    if (use_lo) orc_butter_init(0, flo, nplo, dlo, &mlo);
    if (use_hi) orc_butter_init(1, fhi, nphi, dhi, &mhi);
    for (int j1 = 0; j1 < nr; j1++) {
        for (int i1 = 0; i1 < nt; i1++) trace[i1] = indat[i1 + j1 * nt];
        if (use_lo) {
            butter_apply(0, nplo, dlo, mlo, nt, trace);
            if (!phase) {
                reverse_trace(nt, trace);
                butter_apply(0, nplo, dlo, mlo, nt, trace);
                reverse_trace(nt, trace);
            }
        }
        if (use_hi) {
            butter_apply(1, nphi, dhi, mhi, nt, trace);
            if (!phase) {
                reverse_trace(nt, trace);
                butter_apply(1, nphi, dhi, mhi, nt, trace);
                reverse_trace(nt, trace);
            }
        }
        for (int i1 = 0; i1 < nt; i1++) outdat[i1 + j1 * nt] = trace[i1];
    }
    free(dlo);
    free(dhi);
    free(trace);
    return 0;
}

/* ---- cross-correlation misfit (xcorr_msf.c:4-181) ---------------------- */

/* XCORR1D of nr traces of nt samples ([nr][nt]).  sr_xyz = source x, z then
 * receiver x, z pairs; mode 0 slices the correlations "middle", 1
 * "leading".  misfit[0] accumulates |obs reversed - syn|, misfit[1] the
 * normalised weighted lag energy alpha; res receives d(alpha)/d(syn).
 * Traces whose absolute sums differ by more than 10x or whose offset lies
 * outside [omin, omax] contribute nothing and get res = 0. */
int orc_xcorr1d(const float *obs, const float *syn, int nr, int nt, const float *sr_xyz, float omin, float omax,
                int mode, float *misfit, float *res)
{
    float *T = malloc(sizeof(float) * nt), *x = malloc(sizeof(float) * nt), *b = malloc(sizeof(float) * nt);
    if (!T || !x || !b) { free(T); free(x); free(b); return -3; }
    for (int i = 0; i < nt; i++) {
        if (mode == 0) T[i] = (i > nt / 2) ? i - nt / 2 : nt / 2 - i;
        else T[i] = i;
    }
    const int off = mode == 0 ? nt / 2 : 0;      /* first correlation sample kept */
    misfit[0] = 0.0;
    misfit[1] = 0.0;
    for (int ir = 0; ir < nr; ir++) {
        const float *o = obs + (size_t)ir * nt, *sy = syn + (size_t)ir * nt;
        float *rs = res + (size_t)ir * nt;
        float e1 = 0, e2 = 0, ds, dr;
        for (int it = 0; it < nt; it++) {
            rs[it] = 0.0f;
            e1 += fabs(o[it]);
            e2 += fabs(sy[it]);
        }
        ds = sr_xyz[2 + 2 * ir] - sr_xyz[0];
        ds *= ds;
        dr = sr_xyz[2 + 2 * ir + 1] - sr_xyz[1];
        dr *= dr;
        dr = sqrt(ds + dr);
        if (e2 / (e1 + 1e-12) > 10 || e1 / (e2 + 1e-12) > 10 || dr < omin || dr > omax) continue;
        for (int it = 0; it < nt; it++) misfit[0] += fabs(o[nt - 1 - it] - sy[it]);
        /* x[i] = (reversed obs * syn)[i + off] = sum_j obs[j] syn[j + i + off - nt + 1] */
        for (int i = 0; i < nt; i++) {
            const int lag = i + off - nt + 1;
            double acc = 0;
            for (int j = 0; j < nt; j++) {
                const int k = j + lag;
                if (k >= 0 && k < nt) acc += (double)o[j] * sy[k];
            }
            x[i] = (float)acc;
        }
        for (int i = 0; i < nt; i++) b[i] = T[i] * x[i];
        float tt1 = 0, tt2 = 0;                     /* cblas_sdot, single precision */
        for (int i = 0; i < nt; i++) tt1 += b[i] * b[i];
        for (int i = 0; i < nt; i++) tt2 += x[i] * x[i];
        const float alpha = tt1 / tt2;
        misfit[1] += alpha;
        for (int i = 0; i < nt; i++) x[i] = (T[i] * b[i] - x[i] * alpha) / tt2 * 2.0;
        /* res[n] = (obs * x)[n + off] = sum_i obs[n + off - i] x[i] */
        for (int n = 0; n < nt; n++) {
            double acc = 0;
            for (int i = 0; i < nt; i++) {
                const int k = n + off - i;
                if (k >= 0 && k < nt) acc += (double)o[k] * x[i];
            }
            rs[n] = (float)acc;
        }
    }
    free(T);
    free(x);
    free(b);
    return 0;
}
