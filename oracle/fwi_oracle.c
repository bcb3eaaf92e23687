/*
 * fwi_oracle.c -- CPU oracle for the FWI gradient hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  Loaded by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg; never by the
 * product path.  See fwi_oracle.h for the contract.
 *
 * Part 1 restates the reference's FP32 kernels operation for operation
 * (same loop ranges, same expression trees, same float/double promotions),
 * each citing the reference lines it follows.  Compiled with
 * -ffp-contract=off it reproduces the reference bit for bit.
 *
 * Part 2 restates the per-shot gradient driver that the reference declares
 * (header.h:283) and calls (MBotOpt.c:55,99) but never defines.  Its
 * definition here (source scaling, receiver timing, exact discrete adjoint,
 * imaging condition) is this project's, and the GPU engine implements the
 * same definition:
 *   forward   p^{it+1} = 2 p^it - p^{it-1} + K (L p^it) + s^it,
 *             K = v^2 dt^2 on the padded grid (model_ext), s^it = K_s iarea wav[it]
 *             at the source cell (iarea fwi_2d.c:216); syn[r][k] = p^{k*jump+1}(rec_r).
 *   misfit    J = 1/2 sum (syn - obs)^2, res = syn - obs.
 *   adjoint   b^m = 2 b^{m+1} - b^{m+2} + K (L^T b^{m+1} + r^m), m = nt..1,
 *             b^{nt+1} = b^{nt+2} = 0; L^T is the exact transpose of the
 *             CPML operator including its psi memory; r^m injects res[:, k]
 *             at the receivers when m-1 = k*jump.
 *   source    p^{m-2} = 2 p^{m-1} - p^m + K (L p^{m-1}) + s^{m-1} on the
 *   rebuild   physical interior (a_lap_opt_2d, fwi_2d.c:722-759), with the
 *             2M-1 = 3 outer rows/columns restored from the boundary strips
 *             saved by write_bdr (fwi_2d.c:882-917) / read_bdr (919-960).
 *   imaging   g += b^m (L p^{m-1} + f^{m-1}) on the physical grid, where the
 *             stencil value is used in the interior and
 *             (p^m - 2 p^{m-1} + p^{m-2}) / K on the strips;
 *             grad_v = (2 / v) sum_shots g.
 * The gradient is exact for velocity perturbations that vanish on the
 * outermost physical cells adjacent to a CPML (those cells are replicated
 * into the CPML by model_ext, and the CPML contribution is not imaged).
 */
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "fwi_oracle.h"
#ifdef _OPENMP
#include <omp.h>
#endif

typedef REAL_T real;

/* fwi_sys.h:1 and Mpar.h:10 both define PI; fwi_2d.c includes Mpar.h before
 * fwi_sys.h, so cpml_coe sees the fwi_sys.h value. */
#define ORC_PI 3.141592654

typedef struct {
    int nx, nz, npml, fs;
    int pnx, pnz, unx, unz, vnx, vnz;
    int x0, z0;            /* physical origin inside the padded grid */
    int M;                 /* half the FD order: 2 (the reference's 4th order) or 4 (8th order) */
    int S;                 /* strip width 2M-1 (fwi_sys.h:7 for M = 2) */
} grid_t;

typedef struct {
    float c0x, c1x, ix, c0z, c1z, iz, iz840, iz24;
    float c8x[4], c8z[4];  /* 8th-order staggered weights / h (fd_order 8) */
} coe_t;

typedef struct {
    int npml;
    float *a0[2], *b0[2], *a1[2], *b1[2];   /* [0] = x, [1] = z; 2*npml+1 each */
} pmlc_t;

typedef struct { real *u0, *u1, *v0, *v1, *ux0, *ux1, *vz0, *vz1, *base; size_t len; } psi_t;

int orc_real_bytes(void) { return (int)sizeof(real); }

/* ------------------------------------------------------------------------ */
/* Part 1: restated reference kernels                                        */
/* ------------------------------------------------------------------------ */

/* cpml_coe, fwi_2d.c:110-137, with pml_base {dim=2, maxF, maxV, coefR}
 * (fwi_2d.c:257).  Types follow the reference: float locals, double libm. */
void orc_cpml_coe(float *a0, float *b0, int npml, float dx, float dt,
                  float maxF, float maxV, float coefR)
{
    const float ndx = dx*0.5;
    int npower = 2;
    float thickness_pml, PIf0, slope, d0, d, alpha;
    thickness_pml = npml*dx; PIf0 = ORC_PI*maxF; slope = PIf0/thickness_pml;
    d0 = -(npower + 1)*maxV*log(coefR)/(2.0*thickness_pml);
    for (int i = 0; i < 2*npml+1; i++) {
        d = (1.0-i*ndx/thickness_pml); d *= d; d *= d0;
        alpha = slope*(i*ndx);
        b0[i] = exp(-(d+alpha)*dt);
        a0[i] = d/(d+alpha)*(b0[i]-1.0);
    }
}

/* model_ext (fwi_2d.c:67-107): pad x on both sides and z at the bottom;
 * model_ext_fs_no (fwi_2d.c:29-65): pad both axes on both sides. */
void orc_model_ext(const float *model, int n1, int n2, float *emodel, int en1, int en2, int fs)
{
#define MD(i2,i1) model[(size_t)(i2)*n1+(i1)]
#define EM(i2,i1) emodel[(size_t)(i2)*en1+(i1)]
    if (fs) {
        int gap1 = (en1-n1)/2, gap2 = (en2-n2);
        for (int i2 = 0; i2 < en2-gap2; i2++) {
            for (int i1 = gap1; i1 < en1-gap1; i1++) EM(i2,i1) = MD(i2,i1-gap1);
            for (int i1 = 0; i1 < gap1; i1++) EM(i2,i1) = MD(i2,0);
            for (int i1 = en1-gap1; i1 < en1; i1++) EM(i2,i1) = MD(i2,n1-1);
        }
        for (int i2 = en2-gap2; i2 < en2; i2++)
            for (int i1 = gap1; i1 < en1-gap1; i1++) EM(i2,i1) = MD(n2-1,i1-gap1);
        for (int i2 = en2-gap2; i2 < en2; i2++)
            for (int i1 = en1-gap1; i1 < en1; i1++) EM(i2,i1) = MD(n2-1,n1-1);
        for (int i2 = en2-gap2; i2 < en2; i2++)
            for (int i1 = 0; i1 < gap1; i1++) EM(i2,i1) = MD(n2-1,0);
    } else {
        int gap1 = (en1-n1)/2, gap2 = (en2-n2)/2;
        for (int i2 = gap2; i2 < en2-gap2; i2++) {
            for (int i1 = gap1; i1 < en1-gap1; i1++) EM(i2,i1) = MD(i2-gap2,i1-gap1);
            for (int i1 = 0; i1 < gap1; i1++) EM(i2,i1) = MD(i2-gap2,0);
            for (int i1 = en1-gap1; i1 < en1; i1++) EM(i2,i1) = MD(i2-gap2,n1-1);
        }
        for (int i2 = 0; i2 < gap2; i2++)
            for (int i1 = gap1; i1 < en1-gap1; i1++) {
                EM(i2,i1) = MD(0,i1-gap1);
                EM(i2+en2-gap2,i1) = MD(n2-1,i1-gap1);
            }
        for (int i2 = 0; i2 < gap2; i2++)
            for (int i1 = 0; i1 < gap1; i1++) {
                EM(i2,i1) = MD(0,0);
                EM(i2,i1+en1-gap1) = MD(0,n1-1);
                EM(i2+en2-gap2,i1) = MD(n2-1,0);
                EM(i2+en2-gap2,i1+en1-gap1) = MD(n2-1,n1-1);
            }
    }
#undef MD
#undef EM
}

/* FD coefficients, fwi_2d.c:304-314 (optimized 4th-order staggered pair). */
/* Cell of a position in metres, fwi_2d.c:363-364: the float quotient, then
 * C's round (half away from zero) in double, truncated to int. */
void orc_cell_of(float x, float z, float dx, float dz, int *ix, int *iz)
{
    *ix = (int)round(x/dx);
    *iz = (int)round(z/dz - 0.5);
}

void orc_fd_coeffs(float dx, float dz, float out[8])
{
    coe_t c;
    c.ix = 1.0/dx;
    c.iz = 1.0/dz;
    c.c0x =  0.1129042e1 *c.ix;
    c.c1x = -0.4301412e-1*c.ix;
    c.c0z =  0.1129042e1 *c.iz;
    c.c1z = -0.4301412e-1*c.iz;
    c.iz840 = c.iz/840.0;
    c.iz24  = c.iz/ 24.0;
    out[0] = c.c0x; out[1] = c.c1x; out[2] = c.ix;
    out[3] = c.c0z; out[4] = c.c1z; out[5] = c.iz; out[6] = c.iz840; out[7] = c.iz24;
}

/* Grid shapes, fwi_2d.c:148-165. */
static void make_grid(const orc_config *cfg, grid_t *g)
{
    g->nx = cfg->nx; g->nz = cfg->nz; g->npml = cfg->npml; g->fs = cfg->free_surface ? 1 : 0;
    g->pnx = cfg->nx + 2*cfg->npml;
    g->pnz = cfg->nz + (g->fs ? 1 : 2)*cfg->npml;
    g->unx = g->pnx + 1; g->unz = g->pnz;
    g->vnx = g->pnx;     g->vnz = g->pnz + 1;
    g->x0 = cfg->npml;   g->z0 = g->fs ? 0 : cfg->npml;
    g->M = cfg->fd_order == 8 ? 4 : 2;
    g->S = 2*g->M - 1;
}

void orc_grid(const orc_config *cfg, int out[4])
{
    grid_t g; make_grid(cfg, &g);
    out[0] = g.pnx; out[1] = g.pnz; out[2] = g.x0; out[3] = g.z0;
}

/* The 8th-order staggered first-derivative weights (Taylor, M = 4):
 * f'(x) h = sum_k w_k (f(x + (k - 1/2) h) - f(x - (k - 1/2) h)),
 * w = 1225/1024, -245/3072, 49/5120, -5/7168, rounded to float after the
 * division by h (the reference has no 8th-order operator; fwi_sys.h:7). */
void orc_fd8_coeffs(float dx, float dz, float out[8])
{
    static const double w[4] = {1225.0/1024.0, -245.0/3072.0, 49.0/5120.0, -5.0/7168.0};
    for (int k = 0; k < 4; k++) {
        out[k]   = (float)(w[k]/(double)dx);
        out[4+k] = (float)(w[k]/(double)dz);
    }
}

static void make_coe(const orc_config *cfg, coe_t *c)
{
    float o[8]; orc_fd_coeffs(cfg->dx, cfg->dz, o);
    c->c0x = o[0]; c->c1x = o[1]; c->ix = o[2];
    c->c0z = o[3]; c->c1z = o[4]; c->iz = o[5]; c->iz840 = o[6]; c->iz24 = o[7];
    float w[8]; orc_fd8_coeffs(cfg->dx, cfg->dz, w);
    for (int k = 0; k < 4; k++) { c->c8x[k] = w[k]; c->c8z[k] = w[4+k]; }
}

/* CPML profiles, fwi_2d.c:263-283: a0/b0 from cpml_coe, a1/b1 mirrored. */
static int make_pmlc(const orc_config *cfg, pmlc_t *pm)
{
    int n = 2*cfg->npml+1;
    float *blk = (float *)calloc((size_t)8*n, sizeof(float));
    if (!blk) return ORC_ERR_NOMEM;
    pm->npml = cfg->npml;
    for (int i = 0; i < 2; i++) {
        pm->a0[i] = blk + (4*i+0)*n; pm->b0[i] = blk + (4*i+1)*n;
        pm->a1[i] = blk + (4*i+2)*n; pm->b1[i] = blk + (4*i+3)*n;
    }
    orc_cpml_coe(pm->a0[0], pm->b0[0], cfg->npml, cfg->dx, cfg->dt, cfg->pml_max_f, cfg->pml_max_v, cfg->pml_coef_r);
    orc_cpml_coe(pm->a0[1], pm->b0[1], cfg->npml, cfg->dz, cfg->dt, cfg->pml_max_f, cfg->pml_max_v, cfg->pml_coef_r);
    for (int i = 0; i < n; i++) {
        pm->a1[0][i] = pm->a0[0][2*cfg->npml-i];
        pm->b1[0][i] = pm->b0[0][2*cfg->npml-i];
        pm->a1[1][i] = pm->a0[1][2*cfg->npml-i];
        pm->b1[1][i] = pm->b0[1][2*cfg->npml-i];
    }
    return ORC_OK;
}
static void free_pmlc(pmlc_t *pm) { free(pm->a0[0]); }

/* psi arrays, fwi_2d.c:288-296 (zeroed as pml_var_init, fwi_2d.c:16-27). */
static size_t psi_len_g(const grid_t *g)
{
    size_t np = (size_t)g->npml;
    return 2*(size_t)g->unz*(np+1) + 2*(np+1)*(size_t)g->vnx + 2*(size_t)g->pnz*np + 2*np*(size_t)g->pnx;
}
static void psi_bind(const grid_t *g, real *base, psi_t *s)
{
    size_t np = (size_t)g->npml;
    s->base = base; s->len = psi_len_g(g);
    s->u0 = base;                        s->u1 = s->u0 + (size_t)g->unz*(np+1);
    s->v0 = s->u1 + (size_t)g->unz*(np+1); s->v1 = s->v0 + (np+1)*(size_t)g->vnx;
    s->ux0 = s->v1 + (np+1)*(size_t)g->vnx; s->ux1 = s->ux0 + (size_t)g->pnz*np;
    s->vz0 = s->ux1 + (size_t)g->pnz*np;   s->vz1 = s->vz0 + np*(size_t)g->pnx;
}
int orc_psi_len(const orc_config *cfg) { grid_t g; make_grid(cfg, &g); return (int)psi_len_g(&g); }

/* a_lap_opt_2d_pml, fwi_2d.c:761-864 (fs = 1).  For fs = 0 (the all-sides
 * variant declared at header.h:318-328 but not defined) the top edge mirrors
 * the x edges: v[0] = 0, v[1] = iz (p1 - p0), vz[0] = iz (v1 - v0), and the
 * top psi layers v0/vz0 use the a0/b0 profile like u0/ux0 do. */
static void lap_pml(const grid_t *g, const coe_t *c, const pmlc_t *pm, psi_t *s,
                    const real *p, real *u, real *v, real *ux, real *vz)
{
    const int pnx = g->pnx, pnz = g->pnz, unx = g->unx, unz = g->unz;
    const int vnx = g->vnx, vnz = g->vnz, np = g->npml, un1 = np+1;
#define P(z,x)  p [(size_t)(z)*pnx+(x)]
#define U(z,x)  u [(size_t)(z)*unx+(x)]
#define V(z,x)  v [(size_t)(z)*vnx+(x)]
#define UX(z,x) ux[(size_t)(z)*pnx+(x)]
#define VZ(z,x) vz[(size_t)(z)*pnx+(x)]
    /* fwi_2d.c:775-778 */
    #pragma omp parallel for
    for (int iz = 0; iz < unz; iz++)
        for (int ix = 2; ix < unx-2; ix++)
            U(iz,ix) = c->c0x*(P(iz,ix) - P(iz,ix-1)) + c->c1x*(P(iz,ix+1) - P(iz,ix-2));
    /* fwi_2d.c:780-784; u[.][0] and u[.][unx-1] are never assigned by the
     * reference and hold 0 (calloc, alloc.c:9) */
    #pragma omp parallel for
    for (int iz = 0; iz < unz; iz++) {
        U(iz,1)     = c->ix*(P(iz,1)     - P(iz,0));
        U(iz,unx-2) = c->ix*(P(iz,pnx-1) - P(iz,pnx-2));
        U(iz,0) = 0; U(iz,unx-1) = 0;
    }
    /* fwi_2d.c:786-795 */
    #pragma omp parallel for
    for (int iz = 0; iz < unz; iz++)
        for (int ix = 0; ix < np+1; ix++) {
            real *q0 = &s->u0[(size_t)iz*un1+ix], *q1 = &s->u1[(size_t)iz*un1+ix];
            *q0 = pm->b0[0][2*ix]*(*q0) + pm->a0[0][2*ix]*U(iz,ix);
            U(iz,ix) += *q0;
            *q1 = pm->b1[0][2*ix]*(*q1) + pm->a1[0][2*ix]*U(iz,ix+unx-np-1);
            U(iz,ix+unx-np-1) += *q1;
        }
    /* fwi_2d.c:797-800 */
    #pragma omp parallel for
    for (int iz = 2; iz < vnz-2; iz++)
        for (int ix = 0; ix < vnx; ix++)
            V(iz,ix) = c->c0z*(P(iz,ix) - P(iz-1,ix)) + c->c1z*(P(iz+1,ix) - P(iz-2,ix));
    /* fwi_2d.c:802-810 */
    #pragma omp parallel for
    for (int ix = 0; ix < vnx; ix++) {
        if (g->fs) {
            V(0,ix) = ( 3675.0*P(0,ix)-1225.0*P(1,ix)+441.0*P(2,ix)-75.0*P(3,ix))*c->iz840;
            V(1,ix) = (-1085.0*P(0,ix)+1015.0*P(1,ix)- 63.0*P(2,ix) +5.0*P(3,ix))*c->iz840;
        } else {
            V(0,ix) = 0;
            V(1,ix) = c->iz*(P(1,ix) - P(0,ix));
        }
        V(vnz-2,ix) = (P(pnz-1,ix)-P(pnz-2,ix))*c->iz;
        V(vnz-1,ix) = 0;
    }
    /* fwi_2d.c:812-819 (bottom); fs = 0 adds the top layer */
    #pragma omp parallel for
    for (int iz = 0; iz < np+1; iz++)
        for (int ix = 0; ix < vnx; ix++) {
            if (!g->fs) {
                real *q0 = &s->v0[(size_t)iz*vnx+ix];
                *q0 = pm->b0[1][2*iz]*(*q0) + pm->a0[1][2*iz]*V(iz,ix);
                V(iz,ix) += *q0;
            }
            real *q1 = &s->v1[(size_t)iz*vnx+ix];
            *q1 = pm->b1[1][2*iz]*(*q1) + pm->a1[1][2*iz]*V(iz+vnz-np-1,ix);
            V(iz+vnz-np-1,ix) += *q1;
        }
    /* fwi_2d.c:821-824 */
    #pragma omp parallel for
    for (int iz = 0; iz < pnz; iz++)
        for (int ix = 1; ix < pnx-1; ix++)
            UX(iz,ix) = c->c0x*(U(iz,ix+1) - U(iz,ix)) + c->c1x*(U(iz,ix+2) - U(iz,ix-1));
    /* fwi_2d.c:827-832 */
    #pragma omp parallel for
    for (int iz = 0; iz < pnz; iz++) {
        UX(iz,0)     = (U(iz,1)-U(iz,0))*c->ix;
        UX(iz,pnx-1) = (U(iz,unx-1)-U(iz,unx-2))*c->ix;
    }
    /* fwi_2d.c:834-843 */
    #pragma omp parallel for
    for (int iz = 0; iz < pnz; iz++)
        for (int ix = 0; ix < np; ix++) {
            real *q0 = &s->ux0[(size_t)iz*np+ix], *q1 = &s->ux1[(size_t)iz*np+ix];
            *q0 = pm->b0[0][2*ix+1]*(*q0) + pm->a0[0][2*ix+1]*UX(iz,ix);
            UX(iz,ix) += *q0;
            *q1 = pm->b1[0][2*ix+1]*(*q1) + pm->a1[0][2*ix+1]*UX(iz,ix+pnx-np);
            UX(iz,ix+pnx-np) += *q1;
        }
    /* fwi_2d.c:846-850 */
    #pragma omp parallel for
    for (int ix = 0; ix < pnx; ix++) {
        if (g->fs)
            VZ(0,ix) = (-22.*V(0,ix)+17.*V(1,ix)+9.*V(2,ix)-5.*V(3,ix)+V(4,ix))*c->iz24;
        else
            VZ(0,ix) = (V(1,ix)-V(0,ix))*c->iz;
        VZ(pnz-1,ix) = (V(vnz-1,ix)-V(vnz-2,ix))*c->iz;
    }
    /* fwi_2d.c:852-855 */
    #pragma omp parallel for
    for (int iz = 1; iz < pnz-1; iz++)
        for (int ix = 0; ix < pnx; ix++)
            VZ(iz,ix) = c->c0z*(V(iz+1,ix) - V(iz,ix)) + c->c1z*(V(iz+2,ix) - V(iz-1,ix));
    /* fwi_2d.c:857-862 (bottom); fs = 0 adds the top layer */
    #pragma omp parallel for
    for (int iz = 0; iz < np; iz++)
        for (int ix = 0; ix < pnx; ix++) {
            if (!g->fs) {
                real *q0 = &s->vz0[(size_t)iz*pnx+ix];
                *q0 = pm->b0[1][2*iz+1]*(*q0) + pm->a0[1][2*iz+1]*VZ(iz,ix);
                VZ(iz,ix) += *q0;
            }
            real *q1 = &s->vz1[(size_t)iz*pnx+ix];
            *q1 = pm->b1[1][2*iz+1]*(*q1) + pm->a1[1][2*iz+1]*VZ(iz+pnz-np,ix);
            VZ(iz+pnz-np,ix) += *q1;
        }
#undef P
#undef U
#undef V
#undef UX
#undef VZ
}

/* a_lap_opt_2d, fwi_2d.c:722-759, on the interior grid [nz][nx]. */
static void lap_int(int nx, int nz, const coe_t *c, const real *p, real *u, real *v, real *ux, real *vz)
{
    const int pnx = nx, pnz = nz, unx = nx+1, unz = nz, vnx = nx, vnz = nz+1;
#define P(z,x)  p [(size_t)(z)*pnx+(x)]
#define U(z,x)  u [(size_t)(z)*unx+(x)]
#define V(z,x)  v [(size_t)(z)*vnx+(x)]
#define UX(z,x) ux[(size_t)(z)*pnx+(x)]
#define VZ(z,x) vz[(size_t)(z)*pnx+(x)]
    #pragma omp parallel for
    for (int iz = 2; iz < unz-2; iz++)
        for (int ix = 2; ix < unx-2; ix++)
            U(iz,ix) = c->c0x*(P(iz,ix) - P(iz,ix-1)) + c->c1x*(P(iz,ix+1) - P(iz,ix-2));
    #pragma omp parallel for
    for (int iz = 2; iz < vnz-2; iz++)
        for (int ix = 2; ix < vnx-2; ix++)
            V(iz,ix) = c->c0z*(P(iz,ix) - P(iz-1,ix))+c->c1z*(P(iz+1,ix) - P(iz-2,ix));
    #pragma omp parallel for
    for (int iz = 3; iz < pnz-3; iz++)
        for (int ix = 3; ix < pnx-3; ix++)
            UX(iz,ix) = c->c0x*(U(iz,ix+1) - U(iz,ix))+c->c1x*(U(iz,ix+2) - U(iz,ix-1));
    #pragma omp parallel for
    for (int iz = 3; iz < pnz-3; iz++)
        for (int ix = 3; ix < pnx-3; ix++)
            VZ(iz,ix) = c->c0z*(V(iz+1,ix) - V(iz,ix))+c->c1z*(V(iz+2,ix) - V(iz-1,ix));
#undef P
#undef U
#undef V
#undef UX
#undef VZ
}

/* time_integral, fwi_2d.c:866-880 (2.0 is a double constant there). */
static void time_integral(real *pnew, const real *pnow, const real *pold,
                          const real *pxx, const real *pzz, const float *ekp,
                          int m, int n, int ld_ekp)
{
    #pragma omp parallel for
    for (int i = 0; i < m; i++)
        for (int j = 0; j < n; j++) {
            size_t k = (size_t)i*n + j;
            pnew[k] = 2.0*pnow[k] - pold[k] + ekp[(size_t)i*ld_ekp+j]*(pxx[k] + pzz[k]);
        }
}

/* Adjoint leapfrog: b^m = 2 b^{m+1} - b^{m+2} + K pbar, written in the
 * style of time_integral (double constant 2.0). */
static void adjoint_update(real *bnew, const real *bcur, const real *bprev,
                           const real *pbar, const float *ekp, size_t n)
{
    #pragma omp parallel for
    for (size_t k = 0; k < n; k++)
        bnew[k] = 2.0*bcur[k] - bprev[k] + ekp[k]*pbar[k];
}

/* write_bdr (fwi_2d.c:882-917) / write_bdr_fs_no (962-997) into an in-memory
 * ring: ud [6][nx], lr [nz][6] per step (bc_ud, bc_lr of fwi_2d.c:385-386). */
static void write_strips(const grid_t *g, const real *p, real *ud, real *lr)
{
    const int nx = g->nx, nz = g->nz, pnx = g->pnx, np = g->npml, zo = g->z0;
    const int S = g->S;   /* 2*mm-1, mm = 2 in the reference (fwi_sys.h:7) */
    for (int i = 0; i < S; i++)
        for (int j = 0; j < nx; j++) {
            ud[(size_t)i*nx+j]     = p[(size_t)(i+zo)*pnx + j+np];
            ud[(size_t)(i+S)*nx+j] = p[(size_t)(nz-i-1+zo)*pnx + j+np];
        }
    for (int i = 0; i < nz; i++)
        for (int j = 0; j < S; j++) {
            lr[(size_t)i*2*S+j]   = p[(size_t)(i+zo)*pnx + j+np];
            lr[(size_t)i*2*S+j+S] = p[(size_t)(i+zo)*pnx + nx+np-j-1];
        }
}

/* read_bdr, fwi_2d.c:940-957, into the interior-grid field [nz][nx]; S is
 * the strip width 2M-1. */
static void read_strips(int nx, int nz, int S, const real *ud, const real *lr, real *p)
{
    for (int i = 0; i < S; i++)
        for (int j = 0; j < nx; j++) {
            p[(size_t)i*nx+j]          = ud[(size_t)i*nx+j];
            p[(size_t)(nz-i-1)*nx+j]   = ud[(size_t)(i+S)*nx+j];
        }
    for (int i = 0; i < nz; i++)
        for (int j = 0; j < S; j++) {
            p[(size_t)i*nx+j]          = lr[(size_t)i*2*S+j];
            p[(size_t)i*nx+nx-j-1]     = lr[(size_t)i*2*S+j+S];
        }
}

/* ------------------------------------------------------------------------ */
/* Part 2: the gradient driver (definition in the file header)               */
/* ------------------------------------------------------------------------ */

/* Exact transpose of lap_pml for one step.  Input q is the cotangent of
 * w = ux + vz; output pbar = d<q, w>/dp.  psib carries the cotangents of the
 * psi states from the later step (zero at m = nt).  The x chain is written
 * in scatter form (transposed statements in reverse order), the z chain in
 * gather form; the dot-product test checks both against lap_pml. */
static void lap_pml_t(const grid_t *g, const coe_t *c, const pmlc_t *pm, psi_t *s,
                      const real *q, real *pbar, real *rx, real *ub, real *rz, real *vb)
{
    const int pnx = g->pnx, pnz = g->pnz, unx = g->unx, vnx = g->vnx, vnz = g->vnz;
    const int np = g->npml, un1 = np+1;
    /* x chain, one row at a time */
    #pragma omp parallel for
    for (int iz = 0; iz < pnz; iz++) {
        real *r = rx + (size_t)iz*pnx, *b = ub + (size_t)iz*unx, *pb = pbar + (size_t)iz*pnx;
        const real *qr = q + (size_t)iz*pnx;
        for (int i = 0; i < pnx; i++) r[i] = qr[i];
        /* transpose of fwi_2d.c:834-843 */
        for (int ix = 0; ix < np; ix++) {
            real *c0 = &s->ux0[(size_t)iz*np+ix], *c1 = &s->ux1[(size_t)iz*np+ix];
            int i1 = ix+pnx-np;
            real t = r[i1] + *c1; r[i1] = r[i1] + pm->a1[0][2*ix+1]*t; *c1 = pm->b1[0][2*ix+1]*t;
            t = r[ix] + *c0; r[ix] = r[ix] + pm->a0[0][2*ix+1]*t; *c0 = pm->b0[0][2*ix+1]*t;
        }
        for (int j = 0; j < unx; j++) b[j] = 0;
        /* transpose of fwi_2d.c:827-832 */
        b[1] += c->ix*r[0];         b[0] -= c->ix*r[0];
        b[unx-1] += c->ix*r[pnx-1]; b[unx-2] -= c->ix*r[pnx-1];
        /* transpose of fwi_2d.c:821-824 */
        for (int i = 1; i < pnx-1; i++) {
            b[i+1] += c->c0x*r[i]; b[i]   -= c->c0x*r[i];
            b[i+2] += c->c1x*r[i]; b[i-1] -= c->c1x*r[i];
        }
        /* transpose of fwi_2d.c:786-795 */
        for (int ix = 0; ix < np+1; ix++) {
            real *c0 = &s->u0[(size_t)iz*un1+ix], *c1 = &s->u1[(size_t)iz*un1+ix];
            int j1 = ix+unx-np-1;
            real t = b[j1] + *c1; b[j1] = b[j1] + pm->a1[0][2*ix]*t; *c1 = pm->b1[0][2*ix]*t;
            t = b[ix] + *c0; b[ix] = b[ix] + pm->a0[0][2*ix]*t; *c0 = pm->b0[0][2*ix]*t;
        }
        for (int i = 0; i < pnx; i++) pb[i] = 0;
        /* transpose of fwi_2d.c:780-784 (u[0], u[unx-1] are constants) */
        pb[1] += c->ix*b[1];           pb[0] -= c->ix*b[1];
        pb[pnx-1] += c->ix*b[unx-2];   pb[pnx-2] -= c->ix*b[unx-2];
        /* transpose of fwi_2d.c:775-778 */
        for (int j = 2; j < unx-2; j++) {
            pb[j]   += c->c0x*b[j]; pb[j-1] -= c->c0x*b[j];
            pb[j+1] += c->c1x*b[j]; pb[j-2] -= c->c1x*b[j];
        }
    }
    /* z chain: psi transpose on vz rows (fwi_2d.c:857-862) */
    #pragma omp parallel for
    for (int k = 0; k < pnz; k++)
        for (int ix = 0; ix < pnx; ix++) {
            size_t o = (size_t)k*pnx+ix;
            real val = q[o];
            if (k >= pnz-np) {
                int kk = k-(pnz-np);
                real *cc = &s->vz1[(size_t)kk*pnx+ix];
                real t = val + *cc; val = val + pm->a1[1][2*kk+1]*t; *cc = pm->b1[1][2*kk+1]*t;
            }
            if (!g->fs && k < np) {
                real *cc = &s->vz0[(size_t)k*pnx+ix];
                real t = val + *cc; val = val + pm->a0[1][2*k+1]*t; *cc = pm->b0[1][2*k+1]*t;
            }
            rz[o] = val;
        }
    /* vbar = Hz^T rz: transpose of fwi_2d.c:846-855, gathered per v row */
    #pragma omp parallel for
    for (int kv = 0; kv < vnz; kv++)
        for (int ix = 0; ix < vnx; ix++) {
#define RZM(k) (((k) >= 1 && (k) <= pnz-2) ? rz[(size_t)(k)*pnx+ix] : (real)0)
            real acc = c->c0z*(RZM(kv-1) - RZM(kv)) + c->c1z*(RZM(kv-2) - RZM(kv+1));
#undef RZM
            real r0 = rz[ix];
            if (g->fs) {
                static const double h[5] = {-22., 17., 9., -5., 1.};
                if (kv <= 4) acc += (real)(h[kv]*r0*c->iz24);
            } else {
                if (kv == 1) acc += c->iz*r0;
                if (kv == 0) acc -= c->iz*r0;
            }
            real rb = rz[(size_t)(pnz-1)*pnx+ix];
            if (kv == pnz)   acc += c->iz*rb;
            if (kv == pnz-1) acc -= c->iz*rb;
            vb[(size_t)kv*vnx+ix] = acc;
        }
    /* psi transpose on v rows (fwi_2d.c:812-819) */
    #pragma omp parallel for
    for (int kv = 0; kv < vnz; kv++)
        for (int ix = 0; ix < vnx; ix++) {
            size_t o = (size_t)kv*vnx+ix;
            real val = vb[o];
            if (kv >= vnz-np-1) {
                int kk = kv-(vnz-np-1);
                real *cc = &s->v1[(size_t)kk*vnx+ix];
                real t = val + *cc; val = val + pm->a1[1][2*kk]*t; *cc = pm->b1[1][2*kk]*t;
            }
            if (!g->fs && kv <= np) {
                real *cc = &s->v0[(size_t)kv*vnx+ix];
                real t = val + *cc; val = val + pm->a0[1][2*kv]*t; *cc = pm->b0[1][2*kv]*t;
            }
            vb[o] = val;
        }
    /* pbar += Gz^T vbar: transpose of fwi_2d.c:797-810, gathered per p row */
    #pragma omp parallel for
    for (int k = 0; k < pnz; k++)
        for (int ix = 0; ix < pnx; ix++) {
#define VBM(kv) (((kv) >= 2 && (kv) <= pnz-2) ? vb[(size_t)(kv)*vnx+ix] : (real)0)
            real acc = c->c0z*(VBM(k) - VBM(k+1)) + c->c1z*(VBM(k-1) - VBM(k+2));
#undef VBM
            real v0b = vb[ix], v1b = vb[(size_t)vnx+ix];
            if (g->fs) {
                static const double g0[4] = {3675., -1225., 441., -75.};
                static const double g1[4] = {-1085., 1015., -63., 5.};
                if (k <= 3) acc += (real)((g0[k]*v0b + g1[k]*v1b)*c->iz840);
            } else {
                if (k == 1) acc += c->iz*v1b;
                if (k == 0) acc -= c->iz*v1b;
            }
            real vbb = vb[(size_t)(pnz-1)*vnx+ix];
            if (k == pnz-1) acc += c->iz*vbb;
            if (k == pnz-2) acc -= c->iz*vbb;
            pbar[(size_t)k*pnx+ix] += acc;
        }
}

/* ------------------------------------------------------------------------ */
/* Part 3: the 8th-order extension (fd_order 8, M = 4)                       */
/* ------------------------------------------------------------------------ */
/* The reference is 4th order only (MM 2, fwi_sys.h:7).  The 8th-order
 * operator is defined here, and the GPU engine implements the same
 * definition: every staggered first difference uses the 8th-order stencil
 * where its 8 points lie inside the grid, and the reference's own formulas
 * of a_lap_opt_2d_pml everywhere else (the 4th-order pair, the 2nd-order
 * edge differences and, with a free surface, the one-sided top rows
 * fwi_2d.c:805-807 and 848).  The CPML psi recursions are the reference's,
 * applied to these differences.  Along a line of n cells:
 *   D+ at position j = 0..n (between cells j-1 and j):
 *       4 <= j <= n-4: sum_k w_k (a[j+k-1] - a[j-k])
 *       else the M = 2 rules (fwi_2d.c:775-784, 798-810)
 *   D- at cell i = 0..n-1 from positions b[0..n]:
 *       3 <= i <= n-4: sum_k w_k (b[i+k] - b[i-k+1])
 *       else the M = 2 rules (fwi_2d.c:821-832, 846-855)
 * The interior operator of the rebuild applies the 8th-order stencil only
 * (u positions [4, n-4], cells [7, n-7)); the 2M-1 = 7 outer rows and
 * columns come from the strips.  At those cells the padded operator is the
 * same stencil, so the rebuild reverses the forward exactly (up to
 * rounding).  Its exact transpose is written below in scatter form; the
 * adjoint and finite-difference tests check it. */

#define A8(k) a[(size_t)(k)*st]
/* D+ at position j of n cells (stride st); top_fs: the free-surface top rows */
static real dp8(const real *a, size_t st, int n, int j, const float *w, float c0, float c1, float ih, float ih840,
                int top_fs)
{
    if (j >= 4 && j <= n-4)
        return w[0]*(A8(j) - A8(j-1)) + w[1]*(A8(j+1) - A8(j-2)) + w[2]*(A8(j+2) - A8(j-3)) + w[3]*(A8(j+3) - A8(j-4));
    if (top_fs && j == 0) return ( 3675.0*A8(0)-1225.0*A8(1)+441.0*A8(2)-75.0*A8(3))*ih840;
    if (top_fs && j == 1) return (-1085.0*A8(0)+1015.0*A8(1)- 63.0*A8(2) +5.0*A8(3))*ih840;
    if (j >= 2 && j <= n-2) return c0*(A8(j) - A8(j-1)) + c1*(A8(j+1) - A8(j-2));
    if (j == 1) return ih*(A8(1) - A8(0));
    if (j == n-1) return ih*(A8(n-1) - A8(n-2));
    return 0;
}
/* transpose: abar += d(D+ a at j)/da * ybar */
static void dp8_t(real *a, size_t st, int n, int j, real y, const float *w, float c0, float c1, float ih, float ih840,
                  int top_fs)
{
    if (j >= 4 && j <= n-4) {
        for (int k = 0; k < 4; k++) { A8(j+k) += w[k]*y; A8(j-1-k) -= w[k]*y; }
        return;
    }
    if (top_fs && j <= 1) {
        static const double h0[4] = {3675., -1225., 441., -75.}, h1[4] = {-1085., 1015., -63., 5.};
        for (int k = 0; k < 4; k++) A8(k) += (real)((j == 0 ? h0[k] : h1[k])*y*ih840);
        return;
    }
    if (j >= 2 && j <= n-2) { A8(j) += c0*y; A8(j-1) -= c0*y; A8(j+1) += c1*y; A8(j-2) -= c1*y; return; }
    if (j == 1) { A8(1) += ih*y; A8(0) -= ih*y; return; }
    if (j == n-1) { A8(n-1) += ih*y; A8(n-2) -= ih*y; }
}
/* D- at cell i from positions b[0..n] */
static real dm8(const real *a, size_t st, int n, int i, const float *w, float c0, float c1, float ih, float ih24,
                int top_fs)
{
    if (i >= 3 && i <= n-4)
        return w[0]*(A8(i+1) - A8(i)) + w[1]*(A8(i+2) - A8(i-1)) + w[2]*(A8(i+3) - A8(i-2)) + w[3]*(A8(i+4) - A8(i-3));
    if (top_fs && i == 0) return (-22.*A8(0)+17.*A8(1)+9.*A8(2)-5.*A8(3)+A8(4))*ih24;
    if (i >= 1 && i <= n-2) return c0*(A8(i+1) - A8(i)) + c1*(A8(i+2) - A8(i-1));
    if (i == 0) return (A8(1) - A8(0))*ih;
    return (A8(n) - A8(n-1))*ih;
}
static void dm8_t(real *a, size_t st, int n, int i, real y, const float *w, float c0, float c1, float ih, float ih24,
                  int top_fs)
{
    if (i >= 3 && i <= n-4) {
        for (int k = 0; k < 4; k++) { A8(i+1+k) += w[k]*y; A8(i-k) -= w[k]*y; }
        return;
    }
    if (top_fs && i == 0) {
        static const double h[5] = {-22., 17., 9., -5., 1.};
        for (int k = 0; k < 5; k++) A8(k) += (real)(h[k]*y*ih24);
        return;
    }
    if (i >= 1 && i <= n-2) { A8(i+1) += c0*y; A8(i) -= c0*y; A8(i+2) += c1*y; A8(i-1) -= c1*y; return; }
    if (i == 0) { A8(1) += ih*y; A8(0) -= ih*y; return; }
    A8(n) += ih*y; A8(n-1) -= ih*y;
}
#undef A8

/* The 8th-order CPML operator, the counterpart of lap_pml. */
static void lap_pml8(const grid_t *g, const coe_t *c, const pmlc_t *pm, psi_t *s,
                     const real *p, real *u, real *v, real *ux, real *vz)
{
    const int pnx = g->pnx, pnz = g->pnz, unx = g->unx, unz = g->unz;
    const int vnx = g->vnx, vnz = g->vnz, np = g->npml, un1 = np+1, fs = g->fs;
    #pragma omp parallel for
    for (int iz = 0; iz < unz; iz++)
        for (int j = 0; j < unx; j++)
            u[(size_t)iz*unx+j] = dp8(p + (size_t)iz*pnx, 1, pnx, j, c->c8x, c->c0x, c->c1x, c->ix, 0.f, 0);
    #pragma omp parallel for
    for (int iz = 0; iz < unz; iz++)
        for (int ix = 0; ix < np+1; ix++) {
            real *q0 = &s->u0[(size_t)iz*un1+ix], *q1 = &s->u1[(size_t)iz*un1+ix];
            real *a0 = &u[(size_t)iz*unx+ix], *a1 = &u[(size_t)iz*unx+ix+unx-np-1];
            *q0 = pm->b0[0][2*ix]*(*q0) + pm->a0[0][2*ix]*(*a0);
            *a0 += *q0;
            *q1 = pm->b1[0][2*ix]*(*q1) + pm->a1[0][2*ix]*(*a1);
            *a1 += *q1;
        }
    #pragma omp parallel for
    for (int kv = 0; kv < vnz; kv++)
        for (int ix = 0; ix < vnx; ix++)
            v[(size_t)kv*vnx+ix] = dp8(p + ix, pnx, pnz, kv, c->c8z, c->c0z, c->c1z, c->iz, c->iz840, fs);
    #pragma omp parallel for
    for (int iz = 0; iz < np+1; iz++)
        for (int ix = 0; ix < vnx; ix++) {
            if (!fs) {
                real *q0 = &s->v0[(size_t)iz*vnx+ix], *a0 = &v[(size_t)iz*vnx+ix];
                *q0 = pm->b0[1][2*iz]*(*q0) + pm->a0[1][2*iz]*(*a0);
                *a0 += *q0;
            }
            real *q1 = &s->v1[(size_t)iz*vnx+ix], *a1 = &v[(size_t)(iz+vnz-np-1)*vnx+ix];
            *q1 = pm->b1[1][2*iz]*(*q1) + pm->a1[1][2*iz]*(*a1);
            *a1 += *q1;
        }
    #pragma omp parallel for
    for (int iz = 0; iz < pnz; iz++)
        for (int i = 0; i < pnx; i++)
            ux[(size_t)iz*pnx+i] = dm8(u + (size_t)iz*unx, 1, pnx, i, c->c8x, c->c0x, c->c1x, c->ix, 0.f, 0);
    #pragma omp parallel for
    for (int iz = 0; iz < pnz; iz++)
        for (int ix = 0; ix < np; ix++) {
            real *q0 = &s->ux0[(size_t)iz*np+ix], *q1 = &s->ux1[(size_t)iz*np+ix];
            real *a0 = &ux[(size_t)iz*pnx+ix], *a1 = &ux[(size_t)iz*pnx+ix+pnx-np];
            *q0 = pm->b0[0][2*ix+1]*(*q0) + pm->a0[0][2*ix+1]*(*a0);
            *a0 += *q0;
            *q1 = pm->b1[0][2*ix+1]*(*q1) + pm->a1[0][2*ix+1]*(*a1);
            *a1 += *q1;
        }
    #pragma omp parallel for
    for (int k = 0; k < pnz; k++)
        for (int ix = 0; ix < pnx; ix++)
            vz[(size_t)k*pnx+ix] = dm8(v + ix, vnx, pnz, k, c->c8z, c->c0z, c->c1z, c->iz, c->iz24, fs);
    #pragma omp parallel for
    for (int iz = 0; iz < np; iz++)
        for (int ix = 0; ix < pnx; ix++) {
            if (!fs) {
                real *q0 = &s->vz0[(size_t)iz*pnx+ix], *a0 = &vz[(size_t)iz*pnx+ix];
                *q0 = pm->b0[1][2*iz+1]*(*q0) + pm->a0[1][2*iz+1]*(*a0);
                *a0 += *q0;
            }
            real *q1 = &s->vz1[(size_t)iz*pnx+ix], *a1 = &vz[(size_t)(iz+pnz-np)*pnx+ix];
            *q1 = pm->b1[1][2*iz+1]*(*q1) + pm->a1[1][2*iz+1]*(*a1);
            *a1 += *q1;
        }
}

/* psi transpose of one site: y = x + psi', psi' = b psi + a x, carried
 * cotangent cc: t = ybar + cc; xbar = ybar + a t; cc = b t. */
static inline real psi_t1(real y, real *cc, float a, float b)
{
    real t = y + *cc;
    *cc = b*t;
    return y + a*t;
}

/* Exact transpose of lap_pml8 (scatter form, one row or column per thread). */
static void lap_pml8_t(const grid_t *g, const coe_t *c, const pmlc_t *pm, psi_t *s,
                       const real *q, real *pbar, real *rx, real *ub, real *rz, real *vb)
{
    const int pnx = g->pnx, pnz = g->pnz, unx = g->unx, vnx = g->vnx, vnz = g->vnz;
    const int np = g->npml, un1 = np+1, fs = g->fs;
    #pragma omp parallel for
    for (int iz = 0; iz < pnz; iz++) {
        real *r = rx + (size_t)iz*pnx, *b = ub + (size_t)iz*unx, *pb = pbar + (size_t)iz*pnx;
        for (int i = 0; i < pnx; i++) r[i] = q[(size_t)iz*pnx+i];
        for (int ix = 0; ix < np; ix++) {
            r[ix+pnx-np] = psi_t1(r[ix+pnx-np], &s->ux1[(size_t)iz*np+ix], pm->a1[0][2*ix+1], pm->b1[0][2*ix+1]);
            r[ix] = psi_t1(r[ix], &s->ux0[(size_t)iz*np+ix], pm->a0[0][2*ix+1], pm->b0[0][2*ix+1]);
        }
        for (int j = 0; j < unx; j++) b[j] = 0;
        for (int i = 0; i < pnx; i++) dm8_t(b, 1, pnx, i, r[i], c->c8x, c->c0x, c->c1x, c->ix, 0.f, 0);
        for (int ix = 0; ix < np+1; ix++) {
            b[ix+unx-np-1] = psi_t1(b[ix+unx-np-1], &s->u1[(size_t)iz*un1+ix], pm->a1[0][2*ix], pm->b1[0][2*ix]);
            b[ix] = psi_t1(b[ix], &s->u0[(size_t)iz*un1+ix], pm->a0[0][2*ix], pm->b0[0][2*ix]);
        }
        for (int i = 0; i < pnx; i++) pb[i] = 0;
        for (int j = 0; j < unx; j++) dp8_t(pb, 1, pnx, j, b[j], c->c8x, c->c0x, c->c1x, c->ix, 0.f, 0);
    }
    #pragma omp parallel for
    for (int ix = 0; ix < pnx; ix++) {
        for (int k = 0; k < pnz; k++) {
            real val = q[(size_t)k*pnx+ix];
            if (k >= pnz-np) { int kk = k-(pnz-np); val = psi_t1(val, &s->vz1[(size_t)kk*pnx+ix], pm->a1[1][2*kk+1], pm->b1[1][2*kk+1]); }
            if (!fs && k < np) val = psi_t1(val, &s->vz0[(size_t)k*pnx+ix], pm->a0[1][2*k+1], pm->b0[1][2*k+1]);
            rz[(size_t)k*pnx+ix] = val;
        }
        for (int kv = 0; kv < vnz; kv++) vb[(size_t)kv*vnx+ix] = 0;
        for (int k = 0; k < pnz; k++)
            dm8_t(vb + ix, vnx, pnz, k, rz[(size_t)k*pnx+ix], c->c8z, c->c0z, c->c1z, c->iz, c->iz24, fs);
        for (int kv = 0; kv < vnz; kv++) {
            real *o = &vb[(size_t)kv*vnx+ix];
            if (kv >= vnz-np-1) { int kk = kv-(vnz-np-1); *o = psi_t1(*o, &s->v1[(size_t)kk*vnx+ix], pm->a1[1][2*kk], pm->b1[1][2*kk]); }
            if (!fs && kv <= np) *o = psi_t1(*o, &s->v0[(size_t)kv*vnx+ix], pm->a0[1][2*kv], pm->b0[1][2*kv]);
        }
        for (int kv = 0; kv < vnz; kv++)
            dp8_t(pbar + ix, pnx, pnz, kv, vb[(size_t)kv*vnx+ix], c->c8z, c->c0z, c->c1z, c->iz, c->iz840, fs);
    }
}

/* The 8th-order interior operator of the rebuild on [nz][nx]: u positions
 * [4, nx-4], v positions [4, nz-4], ux/vz cells [7, n-7). */
static void lap_int8(int nx, int nz, const coe_t *c, const real *p, real *u, real *v, real *ux, real *vz)
{
    const int unx = nx+1;
    const float *wx = c->c8x, *wz = c->c8z;
    #pragma omp parallel for
    for (int iz = 0; iz < nz; iz++)
        for (int j = 4; j <= nx-4; j++) {
            const real *a = p + (size_t)iz*nx;
            u[(size_t)iz*unx+j] = wx[0]*(a[j]-a[j-1]) + wx[1]*(a[j+1]-a[j-2]) + wx[2]*(a[j+2]-a[j-3]) + wx[3]*(a[j+3]-a[j-4]);
        }
    #pragma omp parallel for
    for (int kv = 4; kv <= nz-4; kv++)
        for (int ix = 0; ix < nx; ix++) {
#define PA(k) p[(size_t)(k)*nx+ix]
            v[(size_t)kv*nx+ix] = wz[0]*(PA(kv)-PA(kv-1)) + wz[1]*(PA(kv+1)-PA(kv-2)) + wz[2]*(PA(kv+2)-PA(kv-3)) +
                                  wz[3]*(PA(kv+3)-PA(kv-4));
#undef PA
        }
    #pragma omp parallel for
    for (int iz = 7; iz < nz-7; iz++)
        for (int i = 7; i < nx-7; i++) {
            const real *b = u + (size_t)iz*unx;
            ux[(size_t)iz*nx+i] = wx[0]*(b[i+1]-b[i]) + wx[1]*(b[i+2]-b[i-1]) + wx[2]*(b[i+3]-b[i-2]) + wx[3]*(b[i+4]-b[i-3]);
        }
    #pragma omp parallel for
    for (int k = 7; k < nz-7; k++)
        for (int ix = 0; ix < nx; ix++) {
#define VA(kk) v[(size_t)(kk)*nx+ix]
            vz[(size_t)k*nx+ix] = wz[0]*(VA(k+1)-VA(k)) + wz[1]*(VA(k+2)-VA(k-1)) + wz[2]*(VA(k+3)-VA(k-2)) +
                                  wz[3]*(VA(k+4)-VA(k-3));
#undef VA
        }
}

/* Operator selection by the FD order. */
static void lap_op(const grid_t *g, const coe_t *c, const pmlc_t *pm, psi_t *s,
                   const real *p, real *u, real *v, real *ux, real *vz)
{
    if (g->M == 4) lap_pml8(g, c, pm, s, p, u, v, ux, vz); else lap_pml(g, c, pm, s, p, u, v, ux, vz);
}
static void lap_op_t(const grid_t *g, const coe_t *c, const pmlc_t *pm, psi_t *s,
                     const real *q, real *pbar, real *rx, real *ub, real *rz, real *vb)
{
    if (g->M == 4) lap_pml8_t(g, c, pm, s, q, pbar, rx, ub, rz, vb); else lap_pml_t(g, c, pm, s, q, pbar, rx, ub, rz, vb);
}
static void lap_int_op(const grid_t *g, const coe_t *c, const real *p, real *u, real *v, real *ux, real *vz)
{
    if (g->M == 4) lap_int8(g->nx, g->nz, c, p, u, v, ux, vz); else lap_int(g->nx, g->nz, c, p, u, v, ux, vz);
}

typedef struct {
    orc_config cfg;
    grid_t g;
    coe_t c;
    pmlc_t pm;
    float *ekp;          /* [pnz][pnx] */
    float iarea;         /* fwi_2d.c:216 */
    int nt0;
} orc_ctx;

static int ctx_init(orc_ctx *x, const orc_config *cfg, const float *vel)
{
    if (!cfg || !vel || cfg->nx < 8 || cfg->nz < 8 || cfg->npml < 1 || cfg->nt < 1 || cfg->jump < 1)
        return ORC_ERR_ARG;
    if ((cfg->nt - 1) % cfg->jump != 0) return ORC_ERR_ARG;   /* fwi_2d.c:195 */
#ifdef _OPENMP
    if (cfg->nthreads > 0) omp_set_num_threads(cfg->nthreads);
#endif
    memset(x, 0, sizeof(*x));
    x->cfg = *cfg;
    make_grid(cfg, &x->g);
    make_coe(cfg, &x->c);
    if (make_pmlc(cfg, &x->pm)) return ORC_ERR_NOMEM;
    x->ekp = (float *)malloc(sizeof(float)*(size_t)x->g.pnx*x->g.pnz);
    if (!x->ekp) { free_pmlc(&x->pm); return ORC_ERR_NOMEM; }
    orc_ekp(cfg, vel, x->ekp);
    x->iarea = 1.0/(cfg->dx*cfg->dz);
    x->nt0 = (cfg->nt-1)/cfg->jump + 1;
    return ORC_OK;
}
static void ctx_free(orc_ctx *x) { free(x->ekp); free_pmlc(&x->pm); }

int orc_ekp(const orc_config *cfg, const float *vel, float *ekp)
{
    grid_t g; make_grid(cfg, &g);
    orc_model_ext(vel, g.nx, g.nz, ekp, g.pnx, g.pnz, g.fs);
    const float dt = cfg->dt;
    for (size_t i = 0; i < (size_t)g.pnx*g.pnz; i++) {
        float v = ekp[i];
        ekp[i] = v*v*dt*dt;
    }
    return ORC_OK;
}

static int check_shot(const orc_ctx *x, const orc_shot *s)
{
    if (!s || !s->wav || s->nr < 0 || (s->nr > 0 && (!s->irx || !s->irz))) return ORC_ERR_ARG;
    if (s->isx < 0 || s->isx >= x->g.nx || s->isz < 0 || s->isz >= x->g.nz) return ORC_ERR_GEOMETRY;
    for (int r = 0; r < s->nr; r++)
        if (s->irx[r] < 0 || s->irx[r] >= x->g.nx || s->irz[r] < 0 || s->irz[r] >= x->g.nz)
            return ORC_ERR_GEOMETRY;
    return ORC_OK;
}

/* Forward loop of one shot (first half of grad4_1shot, header.h:283):
 * lap_pml + time_integral per step as fwi_2d.c:761-880, then source
 * injection, receiver sampling and strip saving. */
static int run_forward(const orc_ctx *x, const orc_shot *sh, real *syn,
                       real *ring_ud, real *ring_lr, real *pfin, real *pprev,
                       int nsnap, const int *steps, real *snaps)
{
    const grid_t *g = &x->g;
    const size_t np2 = (size_t)g->pnx*g->pnz;
    const size_t nu = (size_t)g->unx*g->unz, nv = (size_t)g->vnx*g->vnz;
    const size_t npsi = psi_len_g(g);
    real *blk = (real *)calloc(5*np2 + nu + nv + npsi, sizeof(real));
    if (!blk) return ORC_ERR_NOMEM;
    real *pold = blk, *pnow = blk+np2, *pnew = blk+2*np2, *ux = blk+3*np2, *vz = blk+4*np2;
    real *u = blk+5*np2, *v = u+nu;
    psi_t s; psi_bind(g, v+nv, &s);
    const size_t isrc = (size_t)(sh->isz+g->z0)*g->pnx + sh->isx+g->x0;
    const size_t udn = (size_t)2*g->S*g->nx, lrn = (size_t)2*g->S*g->nz;
    for (int it = 0; it < x->cfg.nt; it++) {
        lap_op(g, &x->c, &x->pm, &s, pnow, u, v, ux, vz);
        time_integral(pnew, pnow, pold, ux, vz, x->ekp, g->pnz, g->pnx, g->pnx);
        real amp = (real)sh->wav[it]*(real)x->iarea;
        pnew[isrc] += amp*(real)x->ekp[isrc];
        if (syn && it % x->cfg.jump == 0) {
            int k = it/x->cfg.jump;
            for (int r = 0; r < sh->nr; r++)
                syn[(size_t)r*x->nt0+k] =
                    pnew[(size_t)(sh->irz[r]+g->z0)*g->pnx + sh->irx[r]+g->x0];
        }
        if (ring_ud) write_strips(g, pnew, ring_ud + (size_t)it*udn, ring_lr + (size_t)it*lrn);
        for (int i = 0; i < nsnap; i++)
            if (steps[i] == it+1) memcpy(snaps + (size_t)i*np2, pnew, np2*sizeof(real));
        real *t = pold; pold = pnow; pnow = pnew; pnew = t;
    }
    if (pfin)  memcpy(pfin,  pnow, np2*sizeof(real));
    if (pprev) memcpy(pprev, pold, np2*sizeof(real));
    free(blk);
    return ORC_OK;
}

/* Backward loop of one shot (second half of grad4_1shot): exact adjoint on
 * the padded grid, source-field rebuild on the interior grid, imaging.
 * g accumulates sum_m b^m (L p^{m-1} + f^{m-1}) (without the 2/v factor).
 * wbar (optional, [nt]) receives iarea * b^{it+1}(src). */
static int run_backward(const orc_ctx *x, const orc_shot *sh, const real *res,
                        const real *ring_ud, const real *ring_lr,
                        const real *pfin, const real *pprev, real *gacc, real *wbar,
                        int nsnap, const int *steps, real *snaps)
{
    const grid_t *g = &x->g;
    const int nx = g->nx, nz = g->nz, pnx = g->pnx, pnz = g->pnz;
    const size_t np2 = (size_t)pnx*pnz, ni = (size_t)nx*nz;
    const size_t nu = (size_t)g->unx*g->unz, nv = (size_t)g->vnx*g->vnz;
    const size_t nui = (size_t)(nx+1)*nz, nvi = (size_t)nx*(nz+1);
    const size_t npsi = psi_len_g(g);
    real *blk = (real *)calloc(6*np2 + nu + nv + npsi + 5*ni + nui + nvi, sizeof(real));
    if (!blk) return ORC_ERR_NOMEM;
    real *bprev = blk, *bcur = blk+np2, *bnew = blk+2*np2, *pbar = blk+3*np2, *rx = blk+4*np2, *rz = blk+5*np2;
    real *ub = blk+6*np2, *vb = ub+nu;
    psi_t s; psi_bind(g, vb+nv, &s);
    real *rp_prev = s.base + npsi, *rp_cur = rp_prev+ni, *rp_new = rp_cur+ni, *rux = rp_new+ni, *rvz = rux+ni;
    real *ru = rvz+ni, *rv = ru+nui;
    float *ekpi = (float *)malloc(ni*sizeof(float));
    if (!ekpi) { free(blk); return ORC_ERR_NOMEM; }
    for (int iz = 0; iz < nz; iz++)
        for (int ix = 0; ix < nx; ix++) {
            size_t o = (size_t)(iz+g->z0)*pnx + ix+g->x0;
            ekpi[(size_t)iz*nx+ix] = x->ekp[o];
            rp_prev[(size_t)iz*nx+ix] = pfin[o];    /* p^{nt}   */
            rp_cur [(size_t)iz*nx+ix] = pprev[o];   /* p^{nt-1} */
        }
    const size_t isrc = (size_t)(sh->isz+g->z0)*pnx + sh->isx+g->x0;
    const size_t isrc_i = (size_t)sh->isz*nx + sh->isx;
    const int S = g->S;
    const int src_interior = sh->isz >= S && sh->isz < nz-S && sh->isx >= S && sh->isx < nx-S;
    const size_t udn = (size_t)2*S*nx, lrn = (size_t)2*S*nz;
    const int jump = x->cfg.jump;
    for (int m = x->cfg.nt; m >= 1; m--) {
        /* adjoint step: b^m = 2 b^{m+1} - b^{m+2} + K (L^T b^{m+1} + r^m) */
        lap_op_t(g, &x->c, &x->pm, &s, bcur, pbar, rx, ub, rz, vb);
        if ((m-1) % jump == 0) {
            int k = (m-1)/jump;
            for (int r = 0; r < sh->nr; r++)
                pbar[(size_t)(sh->irz[r]+g->z0)*pnx + sh->irx[r]+g->x0] += res[(size_t)r*x->nt0+k];
        }
        adjoint_update(bnew, bcur, bprev, pbar, x->ekp, np2);
        if (wbar) wbar[m-1] = (real)x->iarea*bnew[isrc];
        /* source-field rebuild: p^{m-2} */
        lap_int_op(g, &x->c, rp_cur, ru, rv, rux, rvz);
        time_integral(rp_new, rp_cur, rp_prev, rux, rvz, ekpi, nz, nx, nx);
        real fsrc = (real)sh->wav[m-1]*(real)x->iarea;
        rp_new[isrc_i] += fsrc*(real)ekpi[isrc_i];
        if (m-2 >= 1) {
            read_strips(nx, nz, S, ring_ud + (size_t)(m-3)*udn, ring_lr + (size_t)(m-3)*lrn, rp_new);
        } else {
            for (int i = 0; i < S; i++)
                for (int j = 0; j < nx; j++) { rp_new[(size_t)i*nx+j] = 0; rp_new[(size_t)(nz-1-i)*nx+j] = 0; }
            for (int i = 0; i < nz; i++)
                for (int j = 0; j < S; j++) { rp_new[(size_t)i*nx+j] = 0; rp_new[(size_t)i*nx+nx-1-j] = 0; }
        }
        for (int i = 0; i < nsnap; i++)
            if (steps[i] == m-2) memcpy(snaps + (size_t)i*ni, rp_new, ni*sizeof(real));
        /* imaging on the physical grid */
        #pragma omp parallel for
        for (int iz = 0; iz < nz; iz++)
            for (int ix = 0; ix < nx; ix++) {
                size_t o = (size_t)iz*nx+ix;
                real lp;
                if (iz >= S && iz < nz-S && ix >= S && ix < nx-S) {
                    lp = rux[o] + rvz[o];
                    if (src_interior && o == isrc_i) lp += fsrc;
                } else {
                    lp = ((rp_prev[o] - (real)2*rp_cur[o]) + rp_new[o]) / (real)ekpi[o];
                }
                gacc[o] += bnew[(size_t)(iz+g->z0)*pnx + ix+g->x0]*lp;
            }
        real *t = bprev; bprev = bcur; bcur = bnew; bnew = t;
        t = rp_prev; rp_prev = rp_cur; rp_cur = rp_new; rp_new = t;
    }
    free(ekpi);
    free(blk);
    return ORC_OK;
}

int orc_apply_op(const orc_config *cfg, const REAL_T *p, REAL_T *psi, REAL_T *w)
{
    if (!cfg || !p || !psi || !w) return ORC_ERR_ARG;
    grid_t g; make_grid(cfg, &g);
    coe_t c; make_coe(cfg, &c);
    pmlc_t pm; if (make_pmlc(cfg, &pm)) return ORC_ERR_NOMEM;
    const size_t np2 = (size_t)g.pnx*g.pnz, nu = (size_t)g.unx*g.unz, nv = (size_t)g.vnx*g.vnz;
    real *blk = (real *)calloc(2*np2 + nu + nv, sizeof(real));
    if (!blk) { free_pmlc(&pm); return ORC_ERR_NOMEM; }
    psi_t s; psi_bind(&g, psi, &s);
    lap_op(&g, &c, &pm, &s, p, blk+2*np2, blk+2*np2+nu, blk, blk+np2);
    for (size_t i = 0; i < np2; i++) w[i] = blk[i] + blk[np2+i];
    free(blk); free_pmlc(&pm);
    return ORC_OK;
}

int orc_apply_op_t(const orc_config *cfg, const REAL_T *q, REAL_T *psib, REAL_T *pbar)
{
    if (!cfg || !q || !psib || !pbar) return ORC_ERR_ARG;
    grid_t g; make_grid(cfg, &g);
    coe_t c; make_coe(cfg, &c);
    pmlc_t pm; if (make_pmlc(cfg, &pm)) return ORC_ERR_NOMEM;
    const size_t np2 = (size_t)g.pnx*g.pnz, nu = (size_t)g.unx*g.unz, nv = (size_t)g.vnx*g.vnz;
    real *blk = (real *)calloc(2*np2 + nu + nv, sizeof(real));
    if (!blk) { free_pmlc(&pm); return ORC_ERR_NOMEM; }
    psi_t s; psi_bind(&g, psib, &s);
    lap_op_t(&g, &c, &pm, &s, q, pbar, blk, blk+2*np2, blk+np2, blk+2*np2+nu);
    free(blk); free_pmlc(&pm);
    return ORC_OK;
}

int orc_forward(const orc_config *cfg, const float *vel, const orc_shot *shot,
                REAL_T *syn, REAL_T *pfin, REAL_T *pprev)
{
    orc_ctx x; int st = ctx_init(&x, cfg, vel); if (st) return st;
    st = check_shot(&x, shot);
    if (!st) st = run_forward(&x, shot, syn, NULL, NULL, pfin, pprev, 0, NULL, NULL);
    ctx_free(&x);
    return st;
}

/* forward (with strips) + backward for one shot; res computed by the caller
 * (mode 0: res given) or from obs (mode 1: res = syn - obs, J accumulated). */
static int shot_gradient(const orc_ctx *x, const orc_shot *sh, const float *obs, const real *res_in,
                         double *J, real *syn_out, real *gacc, real *wbar)
{
    const grid_t *g = &x->g;
    const size_t np2 = (size_t)g->pnx*g->pnz;
    const size_t nrt = (size_t)sh->nr*x->nt0;
    const size_t nt = (size_t)x->cfg.nt;
    real *ud = (real *)malloc(nt*2*g->S*(size_t)g->nx*sizeof(real));
    real *lr = (real *)malloc(nt*2*g->S*(size_t)g->nz*sizeof(real));
    real *pf = (real *)malloc(2*np2*sizeof(real));
    real *syn = (real *)calloc(nrt ? nrt : 1, sizeof(real));
    real *res = (real *)calloc(nrt ? nrt : 1, sizeof(real));
    int st = ORC_ERR_NOMEM;
    if (!ud || !lr || !pf || !syn || !res) goto done;
    st = run_forward(x, sh, syn, ud, lr, pf, pf+np2, 0, NULL, NULL);
    if (st) goto done;
    if (syn_out) memcpy(syn_out, syn, nrt*sizeof(real));
    if (res_in) {
        memcpy(res, res_in, nrt*sizeof(real));
    } else {
        double acc = 0;
        for (size_t i = 0; i < nrt; i++) {
            res[i] = syn[i] - (real)obs[i];
            acc += (double)res[i]*(double)res[i];
        }
        if (J) *J += 0.5*acc;
    }
    st = run_backward(x, sh, res, ud, lr, pf, pf+np2, gacc, wbar, 0, NULL, NULL);
done:
    free(ud); free(lr); free(pf); free(syn); free(res);
    return st;
}

int orc_gradient(const orc_config *cfg, const float *vel, int nshots, const orc_shot *shots,
                 const float *obs, double *misfit, double *grad, REAL_T *syn_out)
{
    if (nshots < 0 || !shots || !obs || !grad) return ORC_ERR_ARG;
    orc_ctx x; int st = ctx_init(&x, cfg, vel); if (st) return st;
    const size_t ni = (size_t)cfg->nx*cfg->nz;
    real *gacc = (real *)malloc(ni*sizeof(real));
    if (!gacc) { ctx_free(&x); return ORC_ERR_NOMEM; }
    for (size_t i = 0; i < ni; i++) grad[i] = 0;
    double J = 0;
    size_t off = 0;
    for (int s = 0; s < nshots && !st; s++) {
        st = check_shot(&x, &shots[s]);
        if (st) break;
        for (size_t i = 0; i < ni; i++) gacc[i] = 0;
        st = shot_gradient(&x, &shots[s], obs + off, NULL, &J,
                           syn_out ? syn_out + off : NULL, gacc, NULL);
        for (size_t i = 0; i < ni; i++) grad[i] += (double)gacc[i];   /* FP64 shot reduction */
        off += (size_t)shots[s].nr*x.nt0;
    }
    for (size_t i = 0; i < ni; i++) grad[i] *= 2.0/(double)vel[i];
    if (misfit) misfit[0] = J;
    free(gacc); ctx_free(&x);
    return st;
}

int orc_backward(const orc_config *cfg, const float *vel, const orc_shot *shot,
                 const REAL_T *res, double *grad)
{
    if (!res || !grad) return ORC_ERR_ARG;
    orc_ctx x; int st = ctx_init(&x, cfg, vel); if (st) return st;
    st = check_shot(&x, shot);
    const size_t ni = (size_t)cfg->nx*cfg->nz;
    real *gacc = (real *)calloc(ni, sizeof(real));
    if (!st && !gacc) st = ORC_ERR_NOMEM;
    if (!st) st = shot_gradient(&x, shot, NULL, res, NULL, NULL, gacc, NULL);
    if (!st) for (size_t i = 0; i < ni; i++) grad[i] = 2.0/(double)vel[i]*(double)gacc[i];
    free(gacc); ctx_free(&x);
    return st;
}

int orc_adjoint_wavelet(const orc_config *cfg, const float *vel, const orc_shot *shot,
                        const REAL_T *res, REAL_T *wbar)
{
    if (!res || !wbar) return ORC_ERR_ARG;
    orc_ctx x; int st = ctx_init(&x, cfg, vel); if (st) return st;
    st = check_shot(&x, shot);
    const size_t ni = (size_t)cfg->nx*cfg->nz;
    real *gacc = (real *)calloc(ni, sizeof(real));
    if (!st && !gacc) st = ORC_ERR_NOMEM;
    if (!st) st = shot_gradient(&x, shot, NULL, res, NULL, NULL, gacc, wbar);
    free(gacc); ctx_free(&x);
    return st;
}

int orc_probe(const orc_config *cfg, const float *vel, const orc_shot *shot,
              int nsnap, const int *steps, REAL_T *fwd_snaps, REAL_T *reb_snaps)
{
    orc_ctx x; int st = ctx_init(&x, cfg, vel); if (st) return st;
    st = check_shot(&x, shot);
    if (st) { ctx_free(&x); return st; }
    const grid_t *g = &x.g;
    const size_t np2 = (size_t)g->pnx*g->pnz, ni = (size_t)g->nx*g->nz;
    const size_t nt = (size_t)cfg->nt, nrt = (size_t)shot->nr*x.nt0;
    real *ud = (real *)malloc(nt*2*g->S*(size_t)g->nx*sizeof(real));
    real *lr = (real *)malloc(nt*2*g->S*(size_t)g->nz*sizeof(real));
    real *pf = (real *)malloc(2*np2*sizeof(real));
    real *res = (real *)calloc(nrt ? nrt : 1, sizeof(real));
    real *gacc = (real *)calloc(ni, sizeof(real));
    st = ORC_ERR_NOMEM;
    if (ud && lr && pf && res && gacc) {
        st = run_forward(&x, shot, NULL, ud, lr, pf, pf+np2, fwd_snaps ? nsnap : 0, steps, fwd_snaps);
        if (!st && reb_snaps)
            st = run_backward(&x, shot, res, ud, lr, pf, pf+np2, gacc, NULL, nsnap, steps, reb_snaps);
    }
    free(ud); free(lr); free(pf); free(res); free(gacc); ctx_free(&x);
    return st;
}

int orc_strips_write(const orc_config *cfg, const REAL_T *p, REAL_T *ud, REAL_T *lr)
{
    grid_t g; make_grid(cfg, &g);
    write_strips(&g, p, ud, lr);
    return ORC_OK;
}

int orc_strips_read(const orc_config *cfg, const REAL_T *ud, const REAL_T *lr, REAL_T *p)
{
    grid_t g; make_grid(cfg, &g);
    read_strips(cfg->nx, cfg->nz, g.S, ud, lr, p);
    return ORC_OK;
}

int orc_apply_int(const orc_config *cfg, const REAL_T *p, REAL_T *ux, REAL_T *vz)
{
    coe_t c; make_coe(cfg, &c);
    grid_t g; make_grid(cfg, &g);
    const size_t nu = (size_t)(cfg->nx+1)*cfg->nz, nv = (size_t)cfg->nx*(cfg->nz+1);
    real *blk = (real *)calloc(nu+nv, sizeof(real));
    if (!blk) return ORC_ERR_NOMEM;
    lap_int_op(&g, &c, p, blk, blk+nu, ux, vz);
    free(blk);
    return ORC_OK;
}
