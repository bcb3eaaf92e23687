/* Runs the grad4_1shot drop-in (fwi_plans_gradient) on real plans.
 *
 *     shim_gpu_main <dir>
 *
 * Builds one fwi_plan per shot the way fwi_init fills the fields the shim
 * reads (fwi_2d.c:148-224, 376-381; header.h:21-185), from raw files written
 * by the test:
 *   params.txt   nx nz nt jump npml dx dt nshots perc rectx1 repeat1 rectx2 repeat2 alpha_grad
 *   model.bin    [nz][nx] float velocity (model->md)
 *   ibtry.bin    [nx] int sea-floor rows (model->ibtry)
 *   xyz_<s>.bin  (1 + nr) (x, z) pairs in metres (sou->xyz_sr, fwi_2d.c:343)
 *   wav_<s>.bin  [nt] wavelet (sou->wav0)
 *   obs_<s>.bin  [nr][nt0] observed traces (msf->obs0)
 * then calls fwi_plans_gradient once for all shots and writes
 *   grad.bin     [nz][nx] float plan->grad->body (preconditioned by the
 *                reference's own grad_precond_new5)
 *   val.txt      msf->val[0] msf->val[1]
 * Exit status 0 when the call succeeded. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "header.h"
#include "alloc.h"

int fwi_plans_gradient(fwi_plan **plans, int n, int iter);

static void *load(const char *dir, const char *name, size_t bytes)
{
    char path[1024];
    snprintf(path, sizeof path, "%s/%s", dir, name);
    FILE *f = fopen(path, "rb");
    if (!f) { fprintf(stderr, "cannot open %s\n", path); exit(2); }
    void *p = malloc(bytes ? bytes : 1);
    if (fread(p, 1, bytes, f) != bytes) { fprintf(stderr, "short read %s\n", path); exit(2); }
    fclose(f);
    return p;
}

int main(int argc, char **argv)
{
    if (argc != 2) return 2;
    const char *dir = argv[1];
    char path[1024];
    snprintf(path, sizeof path, "%s/params.txt", dir);
    FILE *f = fopen(path, "r");
    if (!f) return 2;
    int nx, nz, nt, jump, npml, nshots, rectx1, repeat1, rectx2, repeat2;
    float dx, dt, perc, alpha;
    if (fscanf(f, "%d %d %d %d %d %f %f %d %f %d %d %d %d %f", &nx, &nz, &nt, &jump, &npml, &dx, &dt, &nshots, &perc,
               &rectx1, &repeat1, &rectx2, &repeat2, &alpha) != 14)
        return 2;
    fclose(f);
    const int nt0 = (nt - 1) / jump + 1;

    fwi_base base_v = {.dim = 2, .mm = 2, .npml = (size_t)npml, .nx = (size_t)nx, .nz = (size_t)nz, .nt = (size_t)nt,
                       .nt_mem = (size_t)nt, .free_surface = 1, .dx = dx, .dz = dx, .dt = dt};
    fwi_base *base = malloc(sizeof *base);
    memcpy(base, &base_v, sizeof base_v);
    fwi_shape gb = {.mnx = (size_t)nx, .mnz = (size_t)nz, .pnx = (size_t)nx, .pnz = (size_t)nz,
                    .unx = (size_t)nx + 1, .unz = (size_t)nz, .vnx = (size_t)nx, .vnz = (size_t)nz + 1};
    fwi_specs grid = {.base = base, .b = &gb, .f = &gb};

    fwi_model model;
    memset(&model, 0, sizeof model);
    model.md = allocate2d(nx, nz);
    float *md = load(dir, "model.bin", sizeof(float) * (size_t)nx * nz);
    memcpy(model.md[0], md, sizeof(float) * (size_t)nx * nz);
    free(md);
    model.ibtry = load(dir, "ibtry.bin", sizeof(int) * (size_t)nx);

    fwi_plan **plans = calloc((size_t)nshots, sizeof *plans);
    for (int s = 0; s < nshots; s++) {
        char name[64];
        snprintf(name, sizeof name, "xyz_%d.bin", s);
        snprintf(path, sizeof path, "%s/%s", dir, name);
        FILE *g = fopen(path, "rb");
        if (!g) return 2;
        fseek(g, 0, SEEK_END);
        const long bytes = ftell(g);
        fclose(g);
        const int nr = (int)(bytes / (long)(2 * sizeof(float))) - 1;
        fwi_msf msf_v = {.nt = (size_t)nt0, .nr = (size_t)nr, .jump = (size_t)jump};
        fwi_msf *msf = malloc(sizeof *msf);
        memcpy(msf, &msf_v, sizeof msf_v);
        msf->obs0 = allocate2d(nt0, nr);
        snprintf(name, sizeof name, "obs_%d.bin", s);
        float *obs = load(dir, name, sizeof(float) * (size_t)nr * nt0);
        memcpy(msf->obs0[0], obs, sizeof(float) * (size_t)nr * nt0);
        free(obs);
        msf->val = calloc(2, sizeof(float));
        fwi_sou *sou = calloc(1, sizeof *sou);
        snprintf(name, sizeof name, "xyz_%d.bin", s);
        sou->xyz_sr = load(dir, name, (size_t)bytes);
        snprintf(name, sizeof name, "wav_%d.bin", s);
        sou->wav0 = load(dir, name, sizeof(float) * (size_t)nt);
        fwi_grad grad_v = {.alpha_grad = alpha, .perc = perc, .jump = 1, .rectx1 = (size_t)rectx1,
                           .rectz1 = (size_t)rectx1, .repeat1 = (size_t)repeat1, .rectx2 = (size_t)rectx2,
                           .rectz2 = (size_t)rectx2, .repeat2 = (size_t)repeat2};
        fwi_grad *grad = malloc(sizeof *grad);
        memcpy(grad, &grad_v, sizeof grad_v);
        grad->body = calloc((size_t)nx * nz, sizeof(float));
        fwi_plan *p = calloc(1, sizeof *p);
        p->grid = &grid;
        p->model = &model;
        p->msf = msf;
        p->sou = sou;
        p->grad = grad;
        plans[s] = p;
    }
    const int st = fwi_plans_gradient(plans, nshots, 0);
    if (st != 0) {
        fprintf(stderr, "fwi_plans_gradient returned %d\n", st);
        return 1;
    }
    snprintf(path, sizeof path, "%s/grad.bin", dir);
    f = fopen(path, "wb");
    fwrite(plans[0]->grad->body, sizeof(float), (size_t)nx * nz, f);
    fclose(f);
    snprintf(path, sizeof path, "%s/val.txt", dir);
    f = fopen(path, "w");
    fprintf(f, "%.9e %.9e\n", plans[0]->msf->val[0], plans[0]->msf->val[1]);
    fclose(f);
    return 0;
}
