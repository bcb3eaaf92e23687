/*
 * fwi_oracle_lbfgs.c -- CPU oracle of the L-BFGS driver of MBotOpt.c
 * (TEST INFRASTRUCTURE ONLY: the checker of the device optimizer).
 *
 * orc_lbfgs_run restates MBotOpt.c:55-214 for one rank: the initial
 * gradient, d = -g, step 0.8; per iteration a line search from xp along d
 * with the Armijo test (fx > finit + step * ftol * dginit -> step *= 0.5),
 * the curvature test (dg < wolfe * dginit -> step *= 2.1) and the strong
 * curvature test (dg > -wolfe * dginit -> step *= 0.5), at most
 * max_linesearch trials; then the convergence test |g| / |x| <= epsilon,
 * the iteration limit, the memory update (s = x - xp, y = g - gp) and the
 * two-loop recursion over the last min(m, k) pairs scaled by ys / yy; the
 * next first step is 0.2 for k < 4, else the mean of the last two accepted
 * steps.  The vector helpers follow lbfgs.h:7-62 (sequential sums).
 *
 * Compiled twice: REAL = float reproduces the reference's single-precision
 * arithmetic operation for operation (checked against the reference's own
 * MBotOpt.c run on the same objective, tests/test_oracle_lbfgs.py); REAL =
 * double is the FP64 oracle of the device optimizer.  The objective is
 * lbfgs_objective.h.
 */
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "lbfgs_objective.h"

#ifndef REAL_T
#define REAL_T float
#endif
typedef REAL_T real;

OBJ_DEFINE(real, objective)

static void vecncpy(real *y, const real *x, long n) { for (long i = 0; i < n; ++i) y[i] = -x[i]; }
static void vecadd(real *y, const real *x, const real c, long n) { for (long i = 0; i < n; ++i) y[i] += c * x[i]; }
static void vecdot(real *s, const real *x, const real *y, long n)
{
    *s = 0.;
    for (long i = 0; i < n; ++i) *s += x[i] * y[i];
}
static void vec2norm(real *s, const real *x, long n) { vecdot(s, x, x, n); *s = (real)sqrt(*s); }
static void veccpy(real *y, const real *x, long n) { memcpy(y, x, sizeof(real) * n); }
static void vecdiff(real *z, const real *x, const real *y, long n) { for (long i = 0; i < n; ++i) z[i] = x[i] - y[i]; }
static void vecscale(real *y, const real c, long n) { for (long i = 0; i < n; ++i) y[i] *= c; }

/* Runs the optimizer from obj_x0 on n unknowns.  ftrace[k] receives the
 * objective of evaluation k (at most max_evals), x_out the final x.  Returns
 * the reference's ret code (0 success, 1 line-search limit, 2 iteration
 * limit); *nevals the evaluations made. */
int orc_lbfgs_run(long n, int m, double epsilon, int max_iterations, int max_linesearch, double ftol,
                  double wolfe, int max_evals, double *ftrace, double *x_out, int *nevals)
{
    const real dec = 0.5, inc = 2.1;
    /* the parameters as the reference holds them (lbfgs_parameter_t, lbfgs.h:63-70) */
    const real eps_r = (real)epsilon, ftol_r = (real)ftol, wolfe_r = (real)wolfe;
    real *x = malloc(sizeof(real) * n), *xp = malloc(sizeof(real) * n), *g = malloc(sizeof(real) * n),
         *gp = malloc(sizeof(real) * n), *d = malloc(sizeof(real) * n);
    real *S = malloc(sizeof(real) * n * m), *Y = malloc(sizeof(real) * n * m);
    real *alpha = calloc(m, sizeof(real)), *ysv = calloc(m, sizeof(real));
    real *step_arr = calloc(max_iterations + 2, sizeof(real));
    int ret = -1, ne = 0, k = 1, end = 0;
    if (!x || !xp || !g || !gp || !d || !S || !Y || !alpha || !ysv || !step_arr) {
        free(x); free(xp); free(g); free(gp); free(d); free(S); free(Y); free(alpha); free(ysv); free(step_arr);
        *nevals = 0;
        return -3;
    }
    real fx, step, width = 0, dg, finit, dginit, dgtest, ys, yy, xnorm, gnorm, beta;
    for (long i = 0; i < n; ++i) x[i] = (real)obj_x0(i);
    memset(S, 0, sizeof(real) * n * m);
    memset(Y, 0, sizeof(real) * n * m);
#define EVAL(F) do { F = objective(n, x, g); if (ne < max_evals) ftrace[ne] = F; ++ne; } while (0)
    EVAL(fx);
    vecncpy(d, g, n);
    vec2norm(&xnorm, x, n);
    vec2norm(&gnorm, g, n);
    step = 0.8;
    for (;;) {
        veccpy(xp, x, n);
        veccpy(gp, g, n);
        int count = 0;
        vecdot(&dginit, g, d, n);
        finit = fx;
        dgtest = ftol_r * dginit;
        for (;;) {
            veccpy(x, xp, n);
            vecadd(x, d, step, n);
            EVAL(fx);
            ++count;
            if (fx > finit + step * dgtest) {
                width = dec;
            } else {
                vecdot(&dg, g, d, n);
                if (dg < wolfe_r * dginit) width = inc;
                else if (dg > -wolfe_r * dginit) width = dec;
                else break;
            }
            if (max_linesearch <= count) { ret = 1; goto done; }
            step *= width;
        }
        vec2norm(&xnorm, x, n);
        vec2norm(&gnorm, g, n);
        step_arr[k] = step;
        if (gnorm / xnorm <= eps_r) { ret = 0; goto done; }
        if (max_iterations != 0 && max_iterations < k + 1) { ret = 2; goto done; }
        real *s = S + (size_t)end * n, *y = Y + (size_t)end * n;
        vecdiff(s, x, xp, n);
        vecdiff(y, g, gp, n);
        vecdot(&ys, y, s, n);
        vecdot(&yy, y, y, n);
        ysv[end] = ys;
        const int bound = (m <= k) ? m : k;
        ++k;
        end = (end + 1) % m;
        vecncpy(d, g, n);
        int j = end;
        for (int i = 0; i < bound; ++i) {
            j = (j + m - 1) % m;
            vecdot(&alpha[j], S + (size_t)j * n, d, n);
            alpha[j] /= ysv[j];
            vecadd(d, Y + (size_t)j * n, -alpha[j], n);
        }
        vecscale(d, ys / yy, n);
        for (int i = 0; i < bound; ++i) {
            vecdot(&beta, Y + (size_t)j * n, d, n);
            beta /= ysv[j];
            vecadd(d, S + (size_t)j * n, alpha[j] - beta, n);
            j = (j + 1) % m;
        }
        if (k < 4) step = 0.2; else step = 0.5 * (step_arr[k - 1] + step_arr[k - 2]);
    }
done:
    for (long i = 0; i < n; ++i) x_out[i] = x[i];
    *nevals = ne;
    free(x); free(xp); free(g); free(gp); free(d); free(S); free(Y); free(alpha); free(ysv); free(step_arr);
    return ret;
}

/* The objective of lbfgs_objective.h at x (gradient into g), for driving the
 * device optimizer with the same evaluations as orc_lbfgs_run. */
double orc_lbfgs_objective(long n, const real *x, real *g) { return (double)objective(n, x, g); }

/* Start point of lbfgs_objective.h. */
void orc_lbfgs_x0(long n, double *x0) { for (long i = 0; i < n; i++) x0[i] = (real)obj_x0(i); }
