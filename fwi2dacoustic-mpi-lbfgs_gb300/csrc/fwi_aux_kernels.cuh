// fwi_aux_kernels.cuh -- kernels of the routines around the gradient:
// gradient preconditioning, Butterworth band-pass, XCORR misfit.  Included
// by fwi_aux.cu only; fwi_aux.cuh declares the launchers other files use.
#pragma once
#include "fwi_aux.cuh"
#include <cmath>

namespace fwi {

// ---------------------------------------------------------------------------
// Gradient preconditioning (grad_prec.c:5-52, triangle_smooth.c:5-110)
// ---------------------------------------------------------------------------

// Minimum and maximum of a[0..n) into mm[0], mm[1] (one block; exact).
__global__ void k_minmax(const float* __restrict__ a, long long n, float* __restrict__ mm)
{
    __shared__ float smin[32], smax[32];
    float lo = a[0], hi = a[0];
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        lo = fminf(lo, a[i]);
        hi = fmaxf(hi, a[i]);
    }
    for (int o = 16; o; o >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) { smin[threadIdx.x >> 5] = lo; smax[threadIdx.x >> 5] = hi; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (unsigned w = 1; w < blockDim.x / 32; ++w) { lo = fminf(lo, smin[w]); hi = fmaxf(hi, smax[w]); }
        mm[0] = lo;
        mm[1] = hi;
    }
}

// Clip to [vmin * perc, vmax * perc] as grad_prec.c:24-35 (upper bound first).
__global__ void k_clip(float* __restrict__ a, long long n, const float* __restrict__ mm, float perc)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float hi = __fmul_rn(mm[1], perc), lo = __fmul_rn(mm[0], perc);
    float v = a[i];
    if (v > hi) v = hi;
    if (v < lo) v = lo;
    a[i] = v;
}

// Zero the cells above bottom[ix] (grad_prec.c:39-42).
__global__ void k_mask_bottom(float* __restrict__ a, int mnx, int mnz, const int* __restrict__ bottom)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)mnx * mnz) return;
    const int iz = (int)(i / mnx), ix = (int)(i - (long long)iz * mnx);
    if (iz < bottom[ix]) a[i] = 0.f;
}

__global__ void k_scale(float* __restrict__ a, long long n, float s)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = __fmul_rn(a[i], s);
}

// Scratch floats per line of triangle smoothing: box 1 output (nr+n-1) and
// box 2's running sums and output (2 * (2nr+n-2) each).
__host__ __device__ inline size_t tri_work_floats(int nr, int n) { return (size_t)3 * n + 5 * nr; }

// Triangle filter of half-width nr along nlines lines of n samples each
// (sample i of line L at v[L * sl + i * ss]), one thread per line, with the
// reference's sequence of float operations (triangle_smooth.c:5-68): two
// box convolutions as prefix-sum differences, the edges folded back, then a
// division by nr^2.  Scratch is sample-major (entry i of line L at
// i * nlines + L) so that the lines of a warp access consecutive words.
__global__ void k_tri_lines(float* __restrict__ v, int nlines, int n, long long sl, long long ss, int nr,
                            float* __restrict__ work)
{
    const int L = blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= nlines) return;
    float* x = v + (long long)L * sl;
    const int np = nr + n - 1, nq = nr + np - 1;
    float* pp = work;                                  // np per line; later tt
    float* bb = pp + (size_t)np * nlines;              // nq per line: running sums
    float* qq = bb + (size_t)nq * nlines;              // nq per line
    #define W(a, i) a[(size_t)(i) * nlines + L]
    // box 1 (boxconv(nr, n, u, pp))
    W(bb, 0) = x[0];
    for (int i = 1; i < n; i++) W(bb, i) = __fadd_rn(W(bb, i - 1), x[(long long)i * ss]);
    for (int i = n; i < np; i++) W(bb, i) = W(bb, i - 1);
    for (int i = 0; i < nr && i < np; i++) W(pp, i) = W(bb, i);
    for (int i = nr; i < np; i++) W(pp, i) = __fsub_rn(W(bb, i), W(bb, i - nr));
    // box 2 (boxconv(nr, np, pp, qq))
    W(bb, 0) = W(pp, 0);
    for (int i = 1; i < np; i++) W(bb, i) = __fadd_rn(W(bb, i - 1), W(pp, i));
    for (int i = np; i < nq; i++) W(bb, i) = W(bb, i - 1);
    for (int i = 0; i < nr && i < nq; i++) W(qq, i) = W(bb, i);
    for (int i = nr; i < nq; i++) W(qq, i) = __fsub_rn(W(bb, i), W(bb, i - nr));
    // fold the edges back (tt reuses pp), divide by nr^2
    float* tt = pp;
    for (int i = 0; i < n; i++) W(tt, i) = W(qq, i + nr - 1);
    for (int i = 0; i < nr - 1; i++) W(tt, i) = __fadd_rn(W(tt, i), W(qq, nr - (i + 2)));
    for (int i = 0; i < nr - 1; i++) W(tt, n - (i + 2) + 1) = __fadd_rn(W(tt, n - (i + 2) + 1), W(qq, np + i));
    const float nr2 = (float)(nr * nr);
    for (int i = 0; i < n; i++) x[(long long)i * ss] = __fdiv_rn(W(tt, i), nr2);
    #undef W
}

// triangle2 (triangle_smooth.c:70-110) of v[n2][n1] in place: rect1 along
// n1, nt times, then rect2 along n2, nt times.  work holds
// max(n1, n2) * tri_work_floats(max rect, max(n1, n2)) floats.
inline void launch_triangle2(float* v, int n1, int n2, int rect1, int rect2, int nt, float* work, cudaStream_t st)
{
    for (int it = 0; it < nt; it++)
        FWI_LAUNCH(k_tri_lines, (unsigned)((n2 + 127) / 128), 128, 0, st, v, n2, n1, (long long)n1, 1LL, rect1, work);
    for (int it = 0; it < nt; it++)
        FWI_LAUNCH(k_tri_lines, (unsigned)((n1 + 127) / 128), 128, 0, st, v, n1, n2, 1LL, (long long)n1, rect2, work);
}

// ---------------------------------------------------------------------------
// Butterworth band-pass (butterworth_filter.c:32-200)
// ---------------------------------------------------------------------------
constexpr int BUTTER_MAX_ORDER = 32;
constexpr double BUTTER_PI = 3.141592654;     // PI as butterworth_filter.c sees it (fwi_sys.h:1)

struct ButterSec {
    int nn;                                   // order (0: not applied)
    float mid;
    float den[BUTTER_MAX_ORDER + 2];          // [(nn+1)/2][2]
};
struct ButterPair {
    ButterSec lo, hi;                         // low-cut (high-pass) and high-cut (low-pass)
    int phase;                                // 0: zero-phase (forward and backward passes)
};

// Coefficients of one Butterworth filter (the steps of sf_butter_init,
// butterworth_filter.c:32-70, with its float/double promotions).
inline void butter_init(int low, float cutoff, int nn, ButterSec* b)
{
    float arg, ss, sinw, cosw, fact;
    b->nn = nn;
    arg = 2. * BUTTER_PI * cutoff;
    sinw = std::sin(arg);
    cosw = std::cos(arg);
    if (nn % 2) {
        if (low) {
            fact = (1. + cosw) / sinw;
            b->den[2 * (nn / 2)] = 1. / (1. + fact);
            b->den[2 * (nn / 2) + 1] = 1. - fact;
        } else {
            fact = sinw / (1. + cosw);
            b->den[2 * (nn / 2)] = 1. / (fact + 1.);
            b->den[2 * (nn / 2) + 1] = fact - 1.;
        }
    }
    fact = low ? std::sin(0.5 * arg) : std::cos(0.5 * arg);
    fact *= fact;
    for (int j = 0; j < nn / 2; j++) {
        ss = std::sin(BUTTER_PI * (2 * j + 1) / (2 * nn)) * sinw;
        b->den[2 * j] = fact / (1. + ss);
        b->den[2 * j + 1] = (1. - ss) / fact;
    }
    b->mid = -2. * cosw / fact;
}

// Parameter handling of sfbandpass (butterworth_filter.c:127-164): corner
// frequencies in cycles per sample, orders halved for zero-phase filtering,
// filters only where the corner is inside (eps, 0.5 - eps).
inline void butter_pair(float dt, int phase, int nphi, int nplo, float fhi, float flo, ButterPair* bp)
{
    const float eps = 0.0001;
    flo *= dt;
    fhi *= dt;
    if (nplo < 1) nplo = 1;
    if (nplo > 1 && !phase) nplo /= 2;
    if (nphi < 1) nphi = 1;
    if (nphi > 1 && !phase) nphi /= 2;
    *bp = ButterPair{};
    bp->phase = phase;
    if (flo > eps) butter_init(0, flo, nplo, &bp->lo);
    if (fhi < 0.5 - eps) butter_init(1, fhi, nphi, &bp->hi);
}

// sf_butter_apply (butterworth_filter.c:84-117) along x[0..n) (dir = +1) or
// x[n-1..0] (dir = -1, the reference's reverse / apply / reverse).
__device__ inline void butter_apply(const ButterSec& b, int low, float* x, int n, int dir)
{
    const int nn = b.nn;
    const float d1 = b.mid;
    const int i0 = dir > 0 ? 0 : n - 1;
    float x0 = 0.f, x1, x2, y0, y1, y2;
    if (nn % 2) {
        const float d0 = b.den[2 * (nn / 2)], d2 = b.den[2 * (nn / 2) + 1];
        x0 = y1 = 0.f;
        for (int k = 0, ix = i0; k < n; k++, ix += dir) {
            x1 = x0; x0 = x[ix];
            const float s = low ? __fadd_rn(x0, x1) : __fsub_rn(x0, x1);
            y0 = __fmul_rn(__fsub_rn(s, __fmul_rn(d2, y1)), d0);
            x[ix] = y1 = y0;
        }
    }
    for (int j = 0; j < nn / 2; j++) {
        const float d0 = b.den[2 * j], d2 = b.den[2 * j + 1];
        x1 = x0 = y1 = y2 = 0.f;
        for (int k = 0, ix = i0; k < n; k++, ix += dir) {
            x2 = x1; x1 = x0; x0 = x[ix];
            const float t2 = __fmul_rn(2.f, x1);
            float s = low ? __fadd_rn(x0, t2) : __fsub_rn(x0, t2);
            s = __fadd_rn(s, x2);
            s = __fsub_rn(s, __fmul_rn(d1, y1));
            s = __fsub_rn(s, __fmul_rn(d2, y2));
            y0 = __fmul_rn(s, d0);
            y2 = y1; x[ix] = y1 = y0;
        }
    }
}

// sfbandpass's per-trace loop (butterworth_filter.c:166-193), one thread per
// trace of data[nr][nt], in place.
__global__ void k_bandpass(float* __restrict__ data, int nt, int nr, const ButterPair bp)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nr) return;
    float* x = data + (long long)j * nt;
    if (bp.lo.nn) {
        butter_apply(bp.lo, 0, x, nt, +1);
        if (!bp.phase) butter_apply(bp.lo, 0, x, nt, -1);
    }
    if (bp.hi.nn) {
        butter_apply(bp.hi, 1, x, nt, +1);
        if (!bp.phase) butter_apply(bp.hi, 1, x, nt, -1);
    }
}

// ---------------------------------------------------------------------------
// XCORR1D misfit (xcorr_msf.c:4-181)
// ---------------------------------------------------------------------------
__device__ inline double block_sum(double v, double* red)
{
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0;
    for (int w = 0; w < XT / 32; ++w) t += red[w];
    return t;
}

// Lag weight T[i] (xcorr_msf.c:39-54).
__device__ inline float xcorr_T(int i, int nt, int mode)
{
    if (mode == 0) return (float)(i > nt / 2 ? i - nt / 2 : nt / 2 - i);
    return (float)i;
}

// out[i0 + b] = sum_k bc[k] * op[m0 + k - b]  (dir = +1) or op[m0 - k + b] (dir = -1),
// b < XB, k < nt: a sliding window over op, bc broadcast.
__device__ inline void corr_window(const float* bc, const float* op, int nt, int m0, int dir, float* acc)
{
    float w[XB];
    #pragma unroll
    for (int b = 0; b < XB; ++b) { w[b] = op[m0 - dir * b]; acc[b] = 0.f; }
    for (int k = 0; k < nt; ++k) {
        const float c = bc[k];
        #pragma unroll
        for (int b = 0; b < XB; ++b) acc[b] = fmaf(c, w[b], acc[b]);
        #pragma unroll
        for (int b = XB - 1; b > 0; --b) w[b] = w[b - 1];
        w[0] = op[m0 + dir * (k + 1)];
    }
}

// One block per trace: skip test, misfit[0] term, x = (reversed obs * syn)
// sliced, alpha, gradient g, res = (obs * g) sliced.  part[tr] =
// {misfit[0] term, alpha}; a skipped trace gets res = 0 and {0, 0}.
__global__ void __launch_bounds__(XT) k_xcorr(const float* __restrict__ obs, const float* __restrict__ syn,
                                              float* __restrict__ res, const float4* __restrict__ geo,
                                              float2* __restrict__ part, int nt, float omin, float omax, int mode)
{
    FWI_DYN_SMEM(smraw);
    double* red = reinterpret_cast<double*>(smraw);
    const int P = nt + XB + 1;                                   // zero pad on each side of obs
    float* op = reinterpret_cast<float*>(smraw + 64 * sizeof(double));
    float* sy = op + 2 * P + nt;
    float* gx = sy + nt;
    const int tr = blockIdx.x, tid = threadIdx.x;
    const float* o = obs + (long long)tr * nt;
    const float* s = syn + (long long)tr * nt;
    float* r = res + (long long)tr * nt;
    for (int i = tid; i < 2 * P + nt; i += XT) op[i] = (i >= P && i < P + nt) ? o[i - P] : 0.f;
    double e1 = 0, e2 = 0, m0 = 0;
    for (int i = tid; i < nt; i += XT) {
        sy[i] = s[i];
        e1 += fabs((double)o[i]);
        e2 += fabs((double)s[i]);
        m0 += fabs((double)(o[nt - 1 - i] - s[i]));
    }
    e1 = block_sum(e1, red);
    e2 = block_sum(e2, red);
    m0 = block_sum(m0, red);
    // skip test (xcorr_msf.c:61-78) with the reference's float offsets
    const float4 gg = geo[tr];
    float ds = gg.z - gg.x, dr = gg.w - gg.y;
    ds *= ds;
    dr *= dr;
    dr = (float)sqrt((double)(ds + dr));
    const float fe1 = (float)e1, fe2 = (float)e2;
    if (fe2 / (fe1 + 1e-12) > 10 || fe1 / (fe2 + 1e-12) > 10 || dr < omin || dr > omax) {
        for (int i = tid; i < nt; i += XT) r[i] = 0.f;
        if (tid == 0) part[tr] = make_float2(0.f, 0.f);
        return;
    }
    const int off = mode == 0 ? nt / 2 : 0;
    // x[i] = sum_k syn[k] obs[k - i - off + nt - 1]
    for (int i0 = tid * XB; i0 < nt; i0 += XT * XB) {
        float acc[XB];
        corr_window(sy, op, nt, P + nt - 1 - off - i0, +1, acc);
        #pragma unroll
        for (int b = 0; b < XB; ++b) if (i0 + b < nt) gx[i0 + b] = acc[b];
    }
    __syncthreads();
    double t1 = 0, t2 = 0;
    for (int i = tid; i < nt; i += XT) {
        const float bx = __fmul_rn(xcorr_T(i, nt, mode), gx[i]);
        t1 += (double)bx * bx;
        t2 += (double)gx[i] * gx[i];
    }
    const float tt1 = (float)block_sum(t1, red), tt2 = (float)block_sum(t2, red);
    const float alpha = __fdiv_rn(tt1, tt2);
    // gradient of alpha with respect to x (xcorr_msf.c:133-134)
    for (int i = tid; i < nt; i += XT) {
        const float T = xcorr_T(i, nt, mode), xv = gx[i];
        const float q = __fdiv_rn(__fsub_rn(__fmul_rn(T, __fmul_rn(T, xv)), __fmul_rn(xv, alpha)), tt2);
        gx[i] = (float)((double)q * 2.0);
    }
    __syncthreads();
    // res[n] = sum_i g[i] obs[n + off - i]
    for (int n0 = tid * XB; n0 < nt; n0 += XT * XB) {
        float acc[XB];
        corr_window(gx, op, nt, P + n0 + off, -1, acc);
        // acc[b] belongs to output n0 + b with window op[P + n0 + b + off - i]
        #pragma unroll
        for (int b = 0; b < XB; ++b) if (n0 + b < nt) r[n0 + b] = acc[b];
    }
    if (tid == 0) part[tr] = make_float2((float)m0, alpha);
}

// misfit[0] = sum of the misfit[0] terms, misfit[1] = sum of alpha (FP64).
__global__ void k_xcorr_sum(const float2* __restrict__ part, int n, double* __restrict__ out)
{
    __shared__ double s0[32], s1[32];
    double a = 0, b = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) { a += part[i].x; b += part[i].y; }
    for (int o = 16; o; o >>= 1) { a += __shfl_xor_sync(0xffffffffu, a, o); b += __shfl_xor_sync(0xffffffffu, b, o); }
    if ((threadIdx.x & 31) == 0) { s0[threadIdx.x >> 5] = a; s1[threadIdx.x >> 5] = b; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (unsigned w = 1; w < blockDim.x / 32; ++w) { a += s0[w]; b += s1[w]; }
        out[0] = a;
        out[1] = b;
    }
}

}  // namespace fwi
