/*
 * ref_mbotopt_driver.c -- stand-ins for fwi_init and grad4_1shot so that the
 * reference's own MBotOpt.c (its L-BFGS driver, MBotOpt.c:7-242) runs on the
 * objective of lbfgs_objective.h (TEST INFRASTRUCTURE ONLY; linked into
 * oracle/_ref/mbotopt by `make ref`).
 *
 * fwi_init allocates the plan members MBotOpt.c reads (model->md [NZ][NX],
 * grad->body, msf->val) and sets the start point; grad4_1shot evaluates the
 * objective in single precision into msf->val[1] and grad->body and appends
 * the value to the file named by $ORC_LBFGS_TRACE (one "%.9e" line per
 * evaluation).  At exit the final model is written to $ORC_LBFGS_TRACE.x
 * (raw float32).
 */
#include "header.h"
#include "Mpar.h"
#include "lbfgs_objective.h"

OBJ_DEFINE(float, objective)

static FILE *trace_file(void)
{
    static FILE *f = NULL;
    if (!f) {
        const char *p = getenv("ORC_LBFGS_TRACE");
        f = fopen(p ? p : "lbfgs_trace.txt", "w");
    }
    return f;
}

static float *model_block;

static void write_final_model(void)
{
    const char *p = getenv("ORC_LBFGS_TRACE");
    char name[600];
    snprintf(name, sizeof name, "%s.x", p ? p : "lbfgs_trace.txt");
    FILE *f = fopen(name, "wb");
    if (f) { fwrite(model_block, sizeof(float), (size_t)NX * NZ, f); fclose(f); }
    fclose(trace_file());
}

void fwi_init(fwi_plan *plan, int id)
{
    (void)id;
    const long n = (long)NX * NZ;
    plan->model = calloc(1, sizeof(fwi_model));
    plan->model->md = malloc(sizeof(float *) * NZ);
    plan->model->md[0] = malloc(sizeof(float) * n);
    for (int i = 1; i < NZ; i++) plan->model->md[i] = plan->model->md[0] + (size_t)i * NX;
    model_block = malloc(sizeof(float) * n);
    for (long i = 0; i < n; i++) plan->model->md[0][i] = (float)obj_x0(i);
    fwi_grad g0 = {0, 0.f, 0.f, 1.f, 0.f, 1, 1, 1, 1, 1, 1, 1, NULL};
    plan->grad = malloc(sizeof(fwi_grad));
    memcpy(plan->grad, &g0, sizeof g0);
    plan->grad->body = malloc(sizeof(float) * n);
    fwi_msf m0 = {0};
    plan->msf = malloc(sizeof(fwi_msf));
    memcpy(plan->msf, &m0, sizeof m0);
    plan->msf->val = calloc(2, sizeof(float));
    atexit(write_final_model);
}

void grad4_1shot(fwi_plan *plan, int iter)
{
    (void)iter;
    const long n = (long)NX * NZ;
    const float f = objective(n, plan->model->md[0], plan->grad->body);
    plan->msf->val[0] = plan->msf->val[1] = f;
    memcpy(model_block, plan->model->md[0], sizeof(float) * n);
    fprintf(trace_file(), "%.9e\n", (double)f);
}
