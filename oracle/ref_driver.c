/*
 * ref_driver.c -- flat C entry points over the reference's OWN propagator
 * kernels, for pinning the oracle restatement (TEST INFRASTRUCTURE ONLY).
 *
 * Built by oracle/Makefile (target ref) together with the unmodified
 * reference files fwi_2d.c, alloc.c and read_write.c, compiled where they lie
 * in the reference checkout, into oracle/_ref/libfwiref.so.  Nothing here is
 * copied from the reference: this file builds the reference's plan structures
 * (header.h:21-185) the way fwi_init does (fwi_2d.c:148-316) and then calls
 * the reference kernels:
 *   cpml_coe            fwi_2d.c:110-137
 *   model_ext(_fs_no)   fwi_2d.c:29-107
 *   a_lap_opt_2d_pml    fwi_2d.c:761-864   (free surface only: the all-sides
 *                                          variant is declared, never defined)
 *   a_lap_opt_2d        fwi_2d.c:722-759
 *   time_integral       fwi_2d.c:866-880
 *   write_bdr(_fs_no)   fwi_2d.c:882-917, 962-997  (chunked to a temp file)
 *   read_bdr            fwi_2d.c:919-960           (chunks read back in reverse)
 * Source injection and receiver sampling follow the oracle's definition of
 * the missing driver grad4_1shot (header.h:283).
 */
#include "header.h"
#include "alloc.h"
#include "fwi_oracle.h"

static float **rows_of(float *base, int n1, int n2)
{
    float **r = (float **)malloc(sizeof(float *)*(size_t)n2);
    for (int i = 0; i < n2; i++) r[i] = base + (size_t)i*n1;
    return r;
}

int ref_cpml_coe(float *a0, float *b0, int npml, float d, float dt, float maxF, float maxV, float coefR)
{
    pml_base meta = {2, maxF, maxV, coefR};   /* as fwi_2d.c:257 */
    cpml_coe(a0, b0, &meta, npml, d, dt);
    return 0;
}

int ref_model_ext(const float *model, int n1, int n2, float *emodel, int en1, int en2, int fs)
{
    float **m = rows_of((float *)model, n1, n2), **e = rows_of(emodel, en1, en2);
    if (fs) model_ext(m, n1, n2, e, en1, en2); else model_ext_fs_no(m, n1, n2, e, en1, en2);
    free(m); free(e);
    return 0;
}

typedef struct {
    fwi_base *base;
    fwi_shape gf, gb;
    fwi_fdcoe coe;
    pml_profile pml;
} ref_plan;

/* Shapes, coefficients and CPML profile as fwi_init builds them. */
static ref_plan *plan_new(const orc_config *cfg, int nt_mem)
{
    ref_plan *p = (ref_plan *)calloc(1, sizeof(ref_plan));
    fwi_base b = {.dim=2, .mm=2, .npml=(size_t)cfg->npml, .nx=(size_t)cfg->nx, .nz=(size_t)cfg->nz,
                  .nt=(size_t)cfg->nt, .nt_mem=(size_t)nt_mem, .free_surface=(size_t)cfg->free_surface,
                  .dx=cfg->dx, .dz=cfg->dz, .dt=cfg->dt};
    p->base = (fwi_base *)malloc(sizeof(fwi_base));
    memcpy(p->base, &b, sizeof(b));
    fwi_shape *gb = &p->gb, *gf = &p->gf;
    gb->mnx = cfg->nx; gb->mnz = cfg->nz;
    gb->pnx = gb->mnx; gb->pnz = gb->mnz;
    gb->unx = gb->pnx + 1; gb->unz = gb->pnz;
    gb->vnx = gb->pnx; gb->vnz = gb->pnz + 1;
    int np = cfg->npml;
    gf->mnx = gb->mnx + 2*np; gf->mnz = gb->mnz + np;
    gf->pnx = gb->pnx + 2*np; gf->pnz = gb->pnz + np;
    gf->unx = gb->unx + 2*np; gf->unz = gb->unz + np;
    gf->vnx = gb->vnx + 2*np; gf->vnz = gb->vnz + np;
    if (!cfg->free_surface) {
        gf->mnz = gb->mnz + 2*np; gf->pnz = gb->pnz + 2*np;
        gf->unz = gb->unz + 2*np; gf->vnz = gb->vnz + 2*np;
    }
    /* FD coefficients as fwi_init sets them (fwi_2d.c:304-314) */
    p->coe.ix = 1.0/p->base->dx;
    p->coe.iz = 1.0/p->base->dz;
    p->coe.c0x =  0.1129042e1 *p->coe.ix;
    p->coe.c1x = -0.4301412e-1*p->coe.ix;
    p->coe.c0z =  0.1129042e1 *p->coe.iz;
    p->coe.c1z = -0.4301412e-1*p->coe.iz;
    p->coe.iz840 = p->coe.iz/840.0;
    p->coe.iz24  = p->coe.iz/ 24.0;
    pml_base meta = {2, cfg->pml_max_f, cfg->pml_max_v, cfg->pml_coef_r};
    pml_profile *pm = &p->pml;
    pm->npml = np;
    for (int i = 0; i < 2; i++) {
        pm->a0[i] = (float *)malloc((2*np+1)*sizeof(float));
        pm->a1[i] = (float *)malloc((2*np+1)*sizeof(float));
        pm->b0[i] = (float *)malloc((2*np+1)*sizeof(float));
        pm->b1[i] = (float *)malloc((2*np+1)*sizeof(float));
    }
    cpml_coe(pm->a0[0], pm->b0[0], &meta, np, cfg->dx, cfg->dt);
    cpml_coe(pm->a0[1], pm->b0[1], &meta, np, cfg->dz, cfg->dt);
    for (int i = 0; i < 2*np+1; i++) {
        pm->a1[0][i] = pm->a0[0][2*np-i]; pm->b1[0][i] = pm->b0[0][2*np-i];
        pm->a1[1][i] = pm->a0[1][2*np-i]; pm->b1[1][i] = pm->b0[1][2*np-i];
    }
    pm->u0 = allocate2d(np+1, gf->unz); pm->u1 = allocate2d(np+1, gf->unz);
    pm->v0 = allocate2d(gf->vnx, np+1); pm->v1 = allocate2d(gf->vnx, np+1);
    pm->ux0 = allocate2d(np, gf->pnz);  pm->ux1 = allocate2d(np, gf->pnz);
    pm->vz0 = allocate2d(gf->pnx, np);  pm->vz1 = allocate2d(gf->pnx, np);
    return p;
}

static void plan_free(ref_plan *p)
{
    pml_profile *pm = &p->pml;
    for (int i = 0; i < 2; i++) { free(pm->a0[i]); free(pm->a1[i]); free(pm->b0[i]); free(pm->b1[i]); }
    free2d(pm->u0); free2d(pm->u1); free2d(pm->v0); free2d(pm->v1);
    free2d(pm->ux0); free2d(pm->ux1); free2d(pm->vz0); free2d(pm->vz1);
    free(p->base); free(p);
}

static void state_alloc(fwi_state *s, const fwi_shape *g)
{
    s->pold = allocate2d(g->pnx, g->pnz); s->pnow = allocate2d(g->pnx, g->pnz);
    s->pnew = allocate2d(g->pnx, g->pnz);
    s->u = allocate2d(g->unx, g->unz); s->v = allocate2d(g->vnx, g->vnz);
    s->ux = allocate2d(g->pnx, g->pnz); s->vz = allocate2d(g->pnx, g->pnz);
}
static void state_free(fwi_state *s)
{
    free2d(s->pold); free2d(s->pnow); free2d(s->pnew); free2d(s->u); free2d(s->v);
    free2d(s->ux); free2d(s->vz);
}

/* psi arrays in the oracle's concatenated order u0,u1,v0,v1,ux0,ux1,vz0,vz1 */
static void psi_copy(ref_plan *p, float *flat, int to_flat)
{
    const fwi_shape *g = &p->gf; int np = p->pml.npml;
    float *arr[8] = {p->pml.u0[0], p->pml.u1[0], p->pml.v0[0], p->pml.v1[0],
                     p->pml.ux0[0], p->pml.ux1[0], p->pml.vz0[0], p->pml.vz1[0]};
    size_t len[8] = {(size_t)g->unz*(np+1), (size_t)g->unz*(np+1), (size_t)(np+1)*g->vnx, (size_t)(np+1)*g->vnx,
                     (size_t)g->pnz*np, (size_t)g->pnz*np, (size_t)np*g->pnx, (size_t)np*g->pnx};
    for (int i = 0; i < 8; i++) {
        if (to_flat) memcpy(flat, arr[i], len[i]*sizeof(float)); else memcpy(arr[i], flat, len[i]*sizeof(float));
        flat += len[i];
    }
}

/* One a_lap_opt_2d_pml step (free surface); w = ux + vz. */
int ref_apply_op(const orc_config *cfg, const float *p_in, float *psi, float *w)
{
    if (!cfg->free_surface) return -1;
    ref_plan *p = plan_new(cfg, 1);
    fwi_state s; state_alloc(&s, &p->gf);
    memcpy(s.pnow[0], p_in, sizeof(float)*p->gf.pnx*p->gf.pnz);
    psi_copy(p, psi, 0);
    a_lap_opt_2d_pml(s.pnow, s.u, s.v, s.ux, s.vz, &p->coe, &p->gf, &p->pml);
    psi_copy(p, psi, 1);
    for (size_t i = 0; i < p->gf.pnx*p->gf.pnz; i++) w[i] = s.ux[0][i] + s.vz[0][i];
    state_free(&s); plan_free(p);
    return 0;
}

/* One a_lap_opt_2d step on the interior grid. */
int ref_apply_int(const orc_config *cfg, const float *p_in, float *ux, float *vz)
{
    ref_plan *p = plan_new(cfg, 1);
    fwi_state s; state_alloc(&s, &p->gb);
    memcpy(s.pnow[0], p_in, sizeof(float)*p->gb.pnx*p->gb.pnz);
    a_lap_opt_2d(s.pnow, s.u, s.v, s.ux, s.vz, &p->coe, &p->gb);
    memcpy(ux, s.ux[0], sizeof(float)*p->gb.pnx*p->gb.pnz);
    memcpy(vz, s.vz[0], sizeof(float)*p->gb.pnx*p->gb.pnz);
    state_free(&s); plan_free(p);
    return 0;
}

/* Strips of one padded field via write_bdr(_fs_no) (no file flush: nt_mem > 1). */
int ref_strips_write(const orc_config *cfg, const float *p_pad, float *ud, float *lr)
{
    ref_plan *p = plan_new(cfg, 2);
    float ***bud = allocate3d(p->gb.pnx, 6, 2), ***blr = allocate3d(6, p->gb.pnz, 2);
    float **pp = rows_of((float *)p_pad, p->gf.pnx, p->gf.pnz);
    if (cfg->free_surface) write_bdr(bud, blr, pp, &p->gb, p->base, NULL, 0);
    else write_bdr_fs_no(bud, blr, pp, &p->gb, p->base, NULL, 0);
    memcpy(ud, bud[0][0], sizeof(float)*6*p->gb.pnx);
    memcpy(lr, blr[0][0], sizeof(float)*6*p->gb.pnz);
    free(pp); free3d(bud); free3d(blr); plan_free(p);
    return 0;
}

/* Forward loop + strip-based rebuild with the reference kernels (free
 * surface).  Snapshots p^{steps[i]}: fwd_snaps padded, reb_snaps interior. */
int ref_forward(const orc_config *cfg, const float *vel, const orc_shot *sh, int nt_mem,
                float *syn, float *pfin, float *pprev,
                int nsnap, const int *steps, float *fwd_snaps, float *reb_snaps)
{
    if (!cfg->free_surface || nt_mem < 1 || cfg->nt % nt_mem) return -1;
    ref_plan *p = plan_new(cfg, nt_mem);
    const fwi_shape *gf = &p->gf, *gb = &p->gb;
    const int np = cfg->npml, nt = cfg->nt, jump = cfg->jump, nt0 = (nt-1)/jump + 1;
    const size_t npad = (size_t)gf->pnx*gf->pnz, nint = (size_t)gb->pnx*gb->pnz;
    fwi_state fw; state_alloc(&fw, gf);
    float **vm = rows_of((float *)vel, cfg->nx, cfg->nz);
    float **ekp = allocate2d(gf->pnx, gf->pnz);
    model_ext(vm, cfg->nx, cfg->nz, ekp, gf->pnx, gf->pnz);
    for (size_t i = 0; i < npad; i++) { float v = ekp[0][i]; ekp[0][i] = v*v*cfg->dt*cfg->dt; }
    const float iarea = 1.0/(cfg->dx*cfg->dz);   /* fwi_2d.c:216 */
    float ***bc_ud = allocate3d(gb->pnx, 6, nt_mem), ***bc_lr = allocate3d(6, gb->pnz, nt_mem);
    int offset = gb->pnx*6*nt_mem*sizeof(float) + gb->pnz*6*nt_mem*sizeof(float);   /* fwi_2d.c:391-392 */
    FILE *fp = tmpfile();
    if (!fp) return -2;
    const int sx = sh->isx + np, sz = sh->isz;
    for (int it = 0; it < nt; it++) {
        a_lap_opt_2d_pml(fw.pnow, fw.u, fw.v, fw.ux, fw.vz, &p->coe, gf, &p->pml);
        time_integral(fw.pnew, fw.pnow, fw.pold, fw.ux, fw.vz, ekp, gf->pnz, gf->pnx);
        float amp = sh->wav[it]*iarea;
        fw.pnew[sz][sx] += amp*ekp[sz][sx];
        if (syn && it % jump == 0)
            for (int r = 0; r < sh->nr; r++)
                syn[(size_t)r*nt0 + it/jump] = fw.pnew[sh->irz[r]][sh->irx[r]+np];
        write_bdr(bc_ud, bc_lr, fw.pnew, gb, p->base, fp, it);
        for (int i = 0; i < nsnap; i++)
            if (fwd_snaps && steps[i] == it+1) memcpy(fwd_snaps + (size_t)i*npad, fw.pnew[0], npad*sizeof(float));
        float **t = fw.pold; fw.pold = fw.pnow; fw.pnow = fw.pnew; fw.pnew = t;
    }
    if (pfin) memcpy(pfin, fw.pnow[0], npad*sizeof(float));
    if (pprev) memcpy(pprev, fw.pold[0], npad*sizeof(float));
    if (reb_snaps) {
        fwi_state bw; state_alloc(&bw, gb);
        float **ekpi = (float **)malloc(sizeof(float *)*gb->pnz);
        for (int i = 0; i < (int)gb->pnz; i++) ekpi[i] = ekp[i] + np;
        for (int iz = 0; iz < cfg->nz; iz++)
            for (int ix = 0; ix < cfg->nx; ix++) {
                bw.pold[iz][ix] = fw.pnow[iz][ix+np];   /* p^{nt}   */
                bw.pnow[iz][ix] = fw.pold[iz][ix+np];   /* p^{nt-1} */
            }
        float **scratch = allocate2d(gb->pnx, gb->pnz);
        read_bdr(bc_ud, bc_lr, scratch, gb, p->base, fp, offset, nt-1);
        if (nt >= 2) read_bdr(bc_ud, bc_lr, scratch, gb, p->base, fp, offset, nt-2);
        for (int m = nt; m >= 1; m--) {
            a_lap_opt_2d(bw.pnow, bw.u, bw.v, bw.ux, bw.vz, &p->coe, gb);
            time_integral(bw.pnew, bw.pnow, bw.pold, bw.ux, bw.vz, ekpi, gb->pnz, gb->pnx);
            float f = sh->wav[m-1]*iarea;
            bw.pnew[sh->isz][sh->isx] += f*ekpi[sh->isz][sh->isx];
            if (m-3 >= 0) {
                read_bdr(bc_ud, bc_lr, bw.pnew, gb, p->base, fp, offset, m-3);
            } else {
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < cfg->nx; j++) { bw.pnew[i][j] = 0; bw.pnew[cfg->nz-1-i][j] = 0; }
                for (int i = 0; i < cfg->nz; i++)
                    for (int j = 0; j < 3; j++) { bw.pnew[i][j] = 0; bw.pnew[i][cfg->nx-1-j] = 0; }
            }
            for (int i = 0; i < nsnap; i++)
                if (steps[i] == m-2) memcpy(reb_snaps + (size_t)i*nint, bw.pnew[0], nint*sizeof(float));
            float **t = bw.pold; bw.pold = bw.pnow; bw.pnow = bw.pnew; bw.pnew = t;
        }
        free2d(scratch); free(ekpi); state_free(&bw);
    }
    fclose(fp);
    free3d(bc_ud); free3d(bc_lr);
    free2d(ekp); free(vm); state_free(&fw); plan_free(p);
    return 0;
}

/* Whole L2 gradient of nshots shots on the reference's own kernels (free
 * surface), the CPU path the reference would run: per shot (one MPI rank
 * each, MBotOpt.c:51,99, here one after another on all OpenMP threads)
 *   forward   a_lap_opt_2d_pml + time_integral (fwi_2d.c:761-880), source
 *             injection, receiver sampling, write_bdr chunked to a temp file
 *             every nt_mem steps (fwi_2d.c:882-917);
 *   misfit    J = 1/2 sum (syn - obs)^2, res = syn - obs;
 *   backward  pml_var_init (fwi_2d.c:16-27), then per step the rebuild
 *             a_lap_opt_2d + time_integral + read_bdr (fwi_2d.c:722-759,
 *             866-880, 919-960) and the adjoint field with the reference's
 *             forward operator a_lap_opt_2d_pml + time_integral (the
 *             reference has no transposed operator), residuals injected at
 *             the receivers, and the imaging g += b (ux + vz) of the rebuilt
 *             field on the physical grid ((p^m - 2 p^{m-1} + p^{m-2}) / K on
 *             the three outer rows and columns, which a_lap_opt_2d leaves);
 *   gradient  (2 / v) sum over shots, FP64.
 * It is the timing path of the reference arm: its gradient agrees with the
 * exact-adjoint gradient of the oracle only approximately: the CPML
 * operator is not self-adjoint. */
int ref_gradient(const orc_config *cfg, const float *vel, int nshots, const orc_shot *shots,
                 const float *obs, int nt_mem, double *misfit, double *grad)
{
    if (!cfg->free_surface || nt_mem < 1 || cfg->nt % nt_mem) return -1;
    ref_plan *p = plan_new(cfg, nt_mem);
    const fwi_shape *gf = &p->gf, *gb = &p->gb;
    const int np = cfg->npml, nt = cfg->nt, jump = cfg->jump, nt0 = (nt-1)/jump + 1;
    const int nx = cfg->nx, nz = cfg->nz;
    const size_t npad = (size_t)gf->pnx*gf->pnz, nint = (size_t)gb->pnx*gb->pnz;
    fwi_state fw, aw, bw;
    state_alloc(&fw, gf); state_alloc(&aw, gf); state_alloc(&bw, gb);
    float **vm = rows_of((float *)vel, nx, nz);
    float **ekp = allocate2d(gf->pnx, gf->pnz);
    model_ext(vm, nx, nz, ekp, gf->pnx, gf->pnz);
    for (size_t i = 0; i < npad; i++) { float v = ekp[0][i]; ekp[0][i] = v*v*cfg->dt*cfg->dt; }
    float **ekpi = (float **)malloc(sizeof(float *)*gb->pnz);
    for (int i = 0; i < (int)gb->pnz; i++) ekpi[i] = ekp[i] + np;
    const float iarea = 1.0/(cfg->dx*cfg->dz);   /* fwi_2d.c:216 */
    float ***bc_ud = allocate3d(gb->pnx, 6, nt_mem), ***bc_lr = allocate3d(6, gb->pnz, nt_mem);
    int offset = gb->pnx*6*nt_mem*sizeof(float) + gb->pnz*6*nt_mem*sizeof(float);   /* fwi_2d.c:391-392 */
    double *gsum = (double *)calloc(nint, sizeof(double));
    double J = 0;
    size_t off = 0;
    int st = 0;
    for (int s = 0; s < nshots && !st; s++) {
        const orc_shot *sh = &shots[s];
        const int nr = sh->nr;
        float *syn = (float *)calloc((size_t)nr*nt0 + 1, sizeof(float));
        float *res = (float *)calloc((size_t)nr*nt0 + 1, sizeof(float));
        FILE *fp = tmpfile();
        if (!syn || !res || !fp) { st = -2; free(syn); free(res); if (fp) fclose(fp); break; }
        state_var_init(&fw, (fwi_shape *)gf);
        pml_var_init(&p->pml, (fwi_shape *)gf);
        const int sx = sh->isx + np, sz = sh->isz;
        for (int it = 0; it < nt; it++) {
            a_lap_opt_2d_pml(fw.pnow, fw.u, fw.v, fw.ux, fw.vz, &p->coe, gf, &p->pml);
            time_integral(fw.pnew, fw.pnow, fw.pold, fw.ux, fw.vz, ekp, gf->pnz, gf->pnx);
            fw.pnew[sz][sx] += sh->wav[it]*iarea*ekp[sz][sx];
            if (it % jump == 0)
                for (int r = 0; r < nr; r++) syn[(size_t)r*nt0 + it/jump] = fw.pnew[sh->irz[r]][sh->irx[r]+np];
            write_bdr(bc_ud, bc_lr, fw.pnew, gb, p->base, fp, it);
            float **t = fw.pold; fw.pold = fw.pnow; fw.pnow = fw.pnew; fw.pnew = t;
        }
        for (size_t i = 0; i < (size_t)nr*nt0; i++) {
            res[i] = syn[i] - obs[off + i];
            J += 0.5*(double)res[i]*(double)res[i];
        }
        state_var_init(&aw, (fwi_shape *)gf);
        state_var_init(&bw, (fwi_shape *)gb);
        pml_var_init(&p->pml, (fwi_shape *)gf);
        for (int iz = 0; iz < nz; iz++)
            for (int ix = 0; ix < nx; ix++) {
                bw.pold[iz][ix] = fw.pnow[iz][ix+np];   /* p^{nt}   */
                bw.pnow[iz][ix] = fw.pold[iz][ix+np];   /* p^{nt-1} */
            }
        float **scratch = allocate2d(gb->pnx, gb->pnz);
        read_bdr(bc_ud, bc_lr, scratch, gb, p->base, fp, offset, nt-1);
        if (nt >= 2) read_bdr(bc_ud, bc_lr, scratch, gb, p->base, fp, offset, nt-2);
        free2d(scratch);
        for (int m = nt; m >= 1; m--) {
            a_lap_opt_2d_pml(aw.pnow, aw.u, aw.v, aw.ux, aw.vz, &p->coe, gf, &p->pml);
            time_integral(aw.pnew, aw.pnow, aw.pold, aw.ux, aw.vz, ekp, gf->pnz, gf->pnx);
            if ((m-1) % jump == 0)
                for (int r = 0; r < nr; r++)
                    aw.pnew[sh->irz[r]][sh->irx[r]+np] += res[(size_t)r*nt0 + (m-1)/jump]*ekp[sh->irz[r]][sh->irx[r]+np];
            a_lap_opt_2d(bw.pnow, bw.u, bw.v, bw.ux, bw.vz, &p->coe, gb);
            time_integral(bw.pnew, bw.pnow, bw.pold, bw.ux, bw.vz, ekpi, gb->pnz, gb->pnx);
            bw.pnew[sh->isz][sh->isx] += sh->wav[m-1]*iarea*ekpi[sh->isz][sh->isx];
            if (m-3 >= 0) read_bdr(bc_ud, bc_lr, bw.pnew, gb, p->base, fp, offset, m-3);
            #pragma omp parallel for
            for (int iz = 0; iz < nz; iz++)
                for (int ix = 0; ix < nx; ix++) {
                    const int strip = iz < 3 || iz >= nz-3 || ix < 3 || ix >= nx-3;
                    const float lp = strip ? ((bw.pold[iz][ix] - 2.0f*bw.pnow[iz][ix]) + bw.pnew[iz][ix])/ekpi[iz][ix]
                                           : bw.ux[iz][ix] + bw.vz[iz][ix];
                    gsum[(size_t)iz*nx + ix] += (double)(aw.pnew[iz][ix+np]*lp);
                }
            float **t = aw.pold; aw.pold = aw.pnow; aw.pnow = aw.pnew; aw.pnew = t;
            t = bw.pold; bw.pold = bw.pnow; bw.pnow = bw.pnew; bw.pnew = t;
        }
        fclose(fp);
        free(syn); free(res);
        off += (size_t)nr*nt0;
    }
    for (size_t i = 0; i < nint; i++) grad[i] = gsum[i]*2.0/(double)vel[i];
    if (misfit) misfit[0] = J;
    free(gsum); free(ekpi);
    free3d(bc_ud); free3d(bc_lr);
    free2d(ekp); free(vm); state_free(&fw); state_free(&aw); state_free(&bw); plan_free(p);
    return st;
}

/* ---- routines around the gradient ---------------------------------------
 * grad_precond_new5  grad_prec.c:5-52 (with triangle2, triangle_smooth.c:70-110,
 *                    and argmin/argmax, min_max.c)
 * sfbandpass         butterworth_filter.c:127-200 (exported as is)
 * XCORR1D            xcorr_msf.c:4-181 (FFTW/CBLAS from ref_fftw_shim.c)
 */
int ref_grad_precond(float *body, int mnx, int mnz, float perc, int rectx1, int repeat1,
                     int rectx2, int repeat2, float alpha_grad, int *bottom)
{
    fwi_grad g = {0, 0.f, 0.f, alpha_grad, perc, 1, (size_t)rectx1, (size_t)rectx1, (size_t)repeat1,
                  (size_t)rectx2, (size_t)rectx2, (size_t)repeat2, body};
    fwi_shape bw = {(size_t)mnx, (size_t)mnz, 0, 0, 0, 0, 0, 0};
    grad_precond_new5(&g, &bw, bottom);
    return 0;
}

int ref_triangle2(int rect1, int rect2, int nt, int n1, int n2, float *uu, float *vv)
{
    triangle2(rect1, rect2, nt, n1, n2, uu, vv);
    return 0;
}

int ref_xcorr1d(const float *obs, const float *syn, int nr, int nt, float *sr_xyz, float omin, float omax,
                int npad, int mode, float *misfit, float *res)
{
    float **o = rows_of((float *)obs, nt, nr), **s = rows_of((float *)syn, nt, nr), **r = rows_of(res, nt, nr);
    char slice_middle[] = "middle", slice_leading[] = "leading";
    par_xcorr1d par = {nr, nt, npad, mode == 0 ? slice_middle : slice_leading};
    XCORR1D(o, s, sr_xyz, omin, omax, &par, misfit, r);
    free(o); free(s); free(r);
    return 0;
}
