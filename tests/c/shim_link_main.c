/* Links the grad4_1shot shim with the reference's own sources and calls it on a
 * hand-built plan.  Without a GPU the engine reports FWI_ERR_NODEVICE and the
 * shim must mark the trial as failed (NaN misfit) instead of exiting. */
#include <math.h>
#include <stdio.h>
#include "header.h"
#include "alloc.h"

int main(void)
{
    static fwi_base base = {.dim = 2, .mm = 2, .npml = 8, .nx = 32, .nz = 24, .nt = 11, .nt_mem = 11,
                            .free_surface = 1, .dx = 10.f, .dz = 10.f, .dt = 0.001f};
    static fwi_shape gb = {.mnx = 32, .mnz = 24, .pnx = 32, .pnz = 24, .unx = 33, .unz = 24, .vnx = 32, .vnz = 25};
    static fwi_specs grid = {.base = &base, .b = &gb, .f = &gb};
    static fwi_msf msf = {.nt = 11, .nr = 2, .jump = 1};
    static fwi_grad grad = {.perc = 0.f, .alpha_grad = 1.f, .rectx1 = 1, .repeat1 = 1, .rectx2 = 1, .repeat2 = 1};
    fwi_model model;
    fwi_sou sou;
    fwi_plan plan;
    float xyz[6] = {100.f, 10.f, 50.f, 2.f, 150.f, 2.f}, wav[11] = {0};
    int ibtry[32] = {0};
    model.md = allocate2d(32, 24);
    model.ibtry = ibtry;
    for (int i = 0; i < 32 * 24; i++) model.md[0][i] = 2000.f;
    msf.obs0 = allocate2d(11, 2);
    msf.val = (float[2]){0, 0};
    sou.xyz_sr = xyz;
    sou.wav0 = wav;
    grad.body = (float *)calloc(32 * 24, sizeof(float));
    plan.grid = &grid; plan.model = &model; plan.msf = &msf; plan.sou = &sou; plan.grad = &grad;
    grad4_1shot(&plan, 0);
    printf("val %f %f\n", msf.val[0], msf.val[1]);
    return isnan(msf.val[1]) ? 0 : 1;
}
