/*
 * grad4_1shot_gpu.c -- drop-in definition of the reference's missing per-shot
 * gradient driver on top of the GB300 engine.
 *
 *     void grad4_1shot(fwi_plan *plan, int iter);            header.h:283
 *
 * MBotOpt.c calls it once per MPI rank and L-BFGS trial (MBotOpt.c:55,99)
 * after fwi_init(plan, rank) (MBotOpt.c:51) and MPI_Bcast of the model
 * (MBotOpt.c:98); rank 0 then reads the total misfit plan->msf->val[1]
 * (MBotOpt.c:88,102) and the total gradient plan->grad->body (MBotOpt.c:53).
 * This file is compiled together with the reference's own sources (it
 * includes the reference's header.h) and links libfwigpu.so:
 *
 *   mpicc -O2 -fopenmp -DFWI_SHIM_MPI -I<reference> -I<this repo>/include \
 *         MBotOpt.c fwi_2d.c grad_prec.c triangle_smooth.c min_max.c alloc.c \
 *         read_write.c ... grad4_1shot_gpu.c -L<dir> -lfwigpu -o MBotOpt
 *
 * Per call it uploads the model, runs forward + L2 misfit + exact adjoint +
 * imaging for this rank's shot on the GPU, applies the reference's own
 * preconditioning grad_precond_new5 (grad_prec.c:5-52) unchanged, and with
 * FWI_SHIM_MPI sums gradient and misfit over the ranks in FP64 (the
 * reduction the reference performed inside grad4_1shot).
 *
 * Single-process batching: fwi_plans_gradient() takes the plans of all shots
 * (one fwi_init per shot) and runs them as one batch on one GPU.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "header.h"
#include "fwi_gb300.h"
#ifdef FWI_SHIM_MPI
#include <mpi.h>
#endif

/* CPML constants of fwi_sys.h:2-4 unless the build overrides them */
#ifndef MAX_F
#define MAX_F 15
#endif
#ifndef MAX_V
#define MAX_V 6000.0
#endif
#ifndef COEF_R
#define COEF_R 0.001
#endif

static fwi_ctx *g_ctx = NULL;
static int g_nshots = 0;

static fwi_config config_of(const fwi_plan *plan)
{
    const fwi_base *b = plan->grid->base;
    fwi_config c = {0};
    c.nx = (int)b->nx;
    c.nz = (int)b->nz;
    c.dx = b->dx;
    c.dz = b->dz;
    c.dt = b->dt;
    c.nt_max = (int)b->nt;
    c.npml = (int)b->npml;
    c.free_surface = b->free_surface ? 1 : 0;
    c.jump = (int)plan->msf->jump;
    c.pml_max_f = MAX_F;
    c.pml_max_v = MAX_V;
    c.pml_coef_r = COEF_R;
    c.use_graph = 1;
    return c;
}

static fwi_shot shot_of(const fwi_plan *plan)
{
    fwi_shot s;
    s.nt = (int)plan->grid->base->nt;
    s.nr = (int)plan->msf->nr;
    s.src_x = plan->sou->xyz_sr[0];          /* fwi_2d.c:343, (1+nr) (x,z) pairs */
    s.src_z = plan->sou->xyz_sr[1];
    s.rec_xz = plan->sou->xyz_sr + 2;
    s.wavelet = plan->sou->wav0;             /* fwi_2d.c:352-353 */
    return s;
}

static int report(int st, const char *what)
{
    if (st != FWI_OK)
        fprintf(stderr, "grad4_1shot: %s failed: %s (%s)\n", what, fwi_status_string(st),
                g_ctx ? fwi_last_error(g_ctx) : "");
    return st;
}

/* Sets up the engine for the given plans (all shots of one process). */
static int setup(fwi_plan **plans, int n)
{
    int st = FWI_OK;
    if (g_ctx && g_nshots == n) return FWI_OK;
    if (g_ctx) { fwi_destroy(g_ctx); g_ctx = NULL; }
    fwi_config cfg = config_of(plans[0]);
    g_ctx = fwi_create(&cfg, &st);
    if (!g_ctx) return report(st, "fwi_create");
    fwi_shot *shots = (fwi_shot *)malloc(sizeof(fwi_shot) * (size_t)n);
    size_t nobs = 0;
    for (int i = 0; i < n; i++) {
        shots[i] = shot_of(plans[i]);
        nobs += plans[i]->msf->nr * plans[i]->msf->nt;
    }
    st = report(fwi_set_shots(g_ctx, n, shots), "fwi_set_shots");
    free(shots);
    if (st) return st;
    float *obs = (float *)malloc(sizeof(float) * nobs);
    size_t off = 0;
    for (int i = 0; i < n; i++) {                       /* obs0 is [nr][nt0] (fwi_2d.c:196) */
        size_t m = plans[i]->msf->nr * plans[i]->msf->nt;
        for (size_t k = 0; k < m; k++) obs[off + k] = plans[i]->msf->obs0[0][k];
        off += m;
    }
    st = report(fwi_set_observed(g_ctx, obs), "fwi_set_observed");
    free(obs);
    if (!st) g_nshots = n;
    return st;
}

int fwi_plans_gradient(fwi_plan **plans, int n, int iter)
{
    (void)iter;
    if (n < 1) return FWI_ERR_ARG;
    int st = setup(plans, n);
    if (st) return st;
    fwi_plan *p0 = plans[0];
    st = report(fwi_set_model(g_ctx, p0->model->md[0]), "fwi_set_model");
    if (st) return st;
    double mis[2] = {0, 0};
    st = report(fwi_gradient_f32(g_ctx, mis, p0->grad->body), "fwi_gradient");
    if (st) return st;
#ifdef FWI_SHIM_MPI
    {
        const size_t ng = p0->grid->b->mnx * p0->grid->b->mnz;
        double *buf = (double *)malloc(sizeof(double) * (ng + 2));
        for (size_t i = 0; i < ng; i++) buf[i] = p0->grad->body[i];
        buf[ng] = mis[0];
        buf[ng + 1] = mis[1];
        MPI_Allreduce(MPI_IN_PLACE, buf, (int)(ng + 2), MPI_DOUBLE, MPI_SUM, MPI_COMM_WORLD);
        for (size_t i = 0; i < ng; i++) p0->grad->body[i] = (float)buf[i];
        mis[0] = buf[ng];
        mis[1] = buf[ng + 1];
        free(buf);
    }
#endif
    p0->msf->val[0] = (float)mis[0];
    p0->msf->val[1] = (float)mis[1];
    /* the reference's preconditioning, unchanged */
    grad_precond_new5(p0->grad, p0->grid->b, p0->model->ibtry);
    for (int i = 1; i < n; i++) {
        const size_t ng = p0->grid->b->mnx * p0->grid->b->mnz;
        for (size_t k = 0; k < ng; k++) plans[i]->grad->body[k] = p0->grad->body[k];
        plans[i]->msf->val[0] = p0->msf->val[0];
        plans[i]->msf->val[1] = p0->msf->val[1];
    }
    return FWI_OK;
}

void grad4_1shot(fwi_plan *plan, int iter)
{
    if (fwi_plans_gradient(&plan, 1, iter) != FWI_OK) {
        plan->msf->val[0] = NAN;                         /* the caller sees a failed trial */
        plan->msf->val[1] = NAN;
    }
}
