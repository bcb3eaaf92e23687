/* lbfgs_objective.h -- the test objective of the L-BFGS pin (TEST
 * INFRASTRUCTURE ONLY), shared by the oracle (fwi_oracle_lbfgs.c) and the
 * stand-in gradient of the reference's own MBotOpt.c (ref_mbotopt_driver.c):
 *
 *   f(x) = 1/2 sum_i w_i (x_i - c_i)^2 + 1/4 sum_i q (x_i - c_i)^4
 *
 * with w_i in [1, 10] (ill-conditioned) and a small quartic term so that the
 * line search has to adapt its step.  OBJ_REAL is the arithmetic type; the
 * sums run from i = 0 upwards.  x0 is the start point. */
#ifndef LBFGS_OBJECTIVE_H
#define LBFGS_OBJECTIVE_H
#include <math.h>

#define OBJ_Q 0.05

static inline double obj_w(long i) { return 1.0 + 9.0 * (double)(i % 7) / 6.0; }
static inline double obj_c(long i) { return 2000.0 + 300.0 * sin(0.001 * (double)i); }
static inline double obj_x0(long i) { return obj_c(i) + 1.0 + 0.5 * cos(0.01 * (double)i); }

#define OBJ_DEFINE(OBJ_REAL, NAME)                                                            \
    static OBJ_REAL NAME(long n, const OBJ_REAL *x, OBJ_REAL *g)                              \
    {                                                                                         \
        OBJ_REAL f = 0;                                                                       \
        for (long i = 0; i < n; i++) {                                                        \
            const OBJ_REAL r = x[i] - (OBJ_REAL)obj_c(i);                                     \
            const OBJ_REAL w = (OBJ_REAL)obj_w(i);                                            \
            f += (OBJ_REAL)0.5 * w * r * r + (OBJ_REAL)(0.25 * OBJ_Q) * r * r * r * r;         \
            g[i] = w * r + (OBJ_REAL)OBJ_Q * r * r * r;                                       \
        }                                                                                     \
        return f;                                                                             \
    }
#endif
