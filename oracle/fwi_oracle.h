/*
 * fwi_oracle.h -- CPU oracle for the FWI gradient hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker: a plain-C restatement of the
 * reference's propagator kernels (fwi_2d.c) plus a restatement of the per-shot
 * gradient driver that the reference declares (header.h:283, grad4_1shot) but
 * never defines.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline may load it.  The product path never calls it.
 *
 * The same source is compiled twice: with REAL=float (the FP32 twin, which
 * reproduces the reference's FP32 arithmetic operation for operation) and
 * with REAL=double (the FP64 twin, the precision oracle).  Both twins use the
 * same FP32-rounded coefficients (FD, CPML, ekp), so the FP64 twin solves the
 * identical discrete problem with less rounding.
 *
 * Pinning: the FP32 twin's operators are checked bit for bit against the
 * reference's own a_lap_opt_2d_pml / a_lap_opt_2d / time_integral /
 * write_bdr / read_bdr / cpml_coe / model_ext compiled from the reference
 * sources (oracle/Makefile, target ref).  The gradient driver has no reference
 * definition; it is pinned by the adjoint dot-product test and by central
 * finite differences of the misfit (tests/).
 */
#ifndef FWI_ORACLE_H
#define FWI_ORACLE_H

#ifndef REAL_T
#define REAL_T float   /* -DREAL_T=double builds the FP64 twin */
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int nx, nz;          /* physical grid, x fastest ([nz][nx]) */
    int npml;            /* CPML thickness in cells */
    int free_surface;    /* 1: CPML left/right/bottom (fwi_2d.c:154-157); 0: all four sides (fwi_2d.c:159-165) */
    int nt;              /* time steps per shot */
    int jump;            /* receiver sampling interval in steps ((nt0-1)*jump == nt-1, fwi_2d.c:195) */
    float dx, dz, dt;
    float pml_max_f;     /* MAX_F  (fwi_sys.h:2) */
    float pml_max_v;     /* MAX_V  (fwi_sys.h:3) */
    float pml_coef_r;    /* COEF_R (fwi_sys.h:4) */
    int nthreads;        /* OpenMP threads; <= 0 keeps the runtime default */
    int fd_order;        /* 4 (or 0): the reference's staggered 4th order (M = 2);
                            8: the 8th-order extension (M = 4, strips of 2M-1 = 7) */
} orc_config;

typedef struct {
    int isx, isz;        /* source cell, physical indices */
    int nr;              /* receivers */
    const int *irx;      /* [nr] receiver x indices (physical) */
    const int *irz;      /* [nr] receiver z indices (physical) */
    const float *wav;    /* [nt] source wavelet */
} orc_shot;

/* Status codes (0 = ok). */
#define ORC_OK           0
#define ORC_ERR_ARG     -1
#define ORC_ERR_GEOMETRY -2
#define ORC_ERR_NOMEM   -3

int  orc_real_bytes(void);   /* 4 for the FP32 twin, 8 for the FP64 twin */

/* Restatement of cpml_coe (fwi_2d.c:110-137) with pml_base {2, maxF, maxV, coefR}. */
void orc_cpml_coe(float *a0, float *b0, int npml, float d, float dt,
                  float maxF, float maxV, float coefR);

/* Restatement of model_ext (fwi_2d.c:67-107) for fs=1 and model_ext_fs_no (fwi_2d.c:29-65) for fs=0. */
void orc_model_ext(const float *model, int n1, int n2, float *emodel, int en1, int en2, int fs);

/* FD coefficients as fwi_2d.c:304-314 computes them:
 * out = {c0x, c1x, ix, c0z, c1z, iz, iz840, iz24}. */
void orc_fd_coeffs(float dx, float dz, float out[8]);

/* 8th-order staggered weights / h: out = {w1..w4 / dx, w1..w4 / dz}. */
void orc_fd8_coeffs(float dx, float dz, float out[8]);

/* Cell (ix, iz) of a position (x, z) in metres, as fwi_2d.c:363-364. */
void orc_cell_of(float x, float z, float dx, float dz, int *ix, int *iz);

/* Padded-grid ekp = vext*vext*dt*dt (edge-replicated velocity). [pnz][pnx] */
int  orc_ekp(const orc_config *cfg, const float *vel, float *ekp);

/* Padded grid sizes: out = {pnx, pnz, x0 (physical x offset), z0 (physical z offset)}. */
void orc_grid(const orc_config *cfg, int out[4]);

/* One application of the padded CPML operator (a_lap_opt_2d_pml and its
 * all-sides variant) to p [pnz][pnx], updating the ten psi arrays in place
 * (psi layout: u0,u1 [pnz][npml+1]; v0,v1 [npml+1][pnx]; ux0,ux1 [pnz][npml];
 * vz0,vz1 [npml][pnx], concatenated in that order).  w = ux + vz. */
int  orc_apply_op(const orc_config *cfg, const REAL_T *p, REAL_T *psi, REAL_T *w);
/* Exact transpose of one orc_apply_op step: pbar = L^T q, with adjoint psi
 * states (same layout) carried in psib. */
int  orc_apply_op_t(const orc_config *cfg, const REAL_T *q, REAL_T *psib, REAL_T *pbar);
int  orc_psi_len(const orc_config *cfg);

/* Forward modelling of one shot.  syn [nr][nt0] (nt0 = (nt-1)/jump + 1)
 * records p^{it+1} at the receivers for it % jump == 0.  Optional outputs
 * (NULL to skip): pfin/pprev = p^{nt}, p^{nt-1} on the padded grid. */
int  orc_forward(const orc_config *cfg, const float *vel, const orc_shot *shot,
                 REAL_T *syn, REAL_T *pfin, REAL_T *pprev);

/* Gradient of J = 1/2 sum (syn-obs)^2 over all shots with respect to the
 * physical velocity.  obs is [nshots][nr_s][nt0] concatenated; misfit[0] = J.
 * grad [nz][nx] (double).  syn_out (optional) receives the modelled data in
 * the layout of obs. */
int  orc_gradient(const orc_config *cfg, const float *vel, int nshots, const orc_shot *shots,
                  const float *obs, double *misfit, double *grad, REAL_T *syn_out);

/* Backward half only: gradient for a given residual res [nr][nt0] of one shot
 * (the forward pass is re-run internally to obtain the boundary strips). */
int  orc_backward(const orc_config *cfg, const float *vel, const orc_shot *shot,
                  const REAL_T *res, double *grad);

/* Adjoint of the linear map wavelet -> seismogram for one shot:
 * wbar[it] = d <syn, res> / d wav[it].  Used by the dot-product test. */
int  orc_adjoint_wavelet(const orc_config *cfg, const float *vel, const orc_shot *shot,
                         const REAL_T *res, REAL_T *wbar);

/* Snapshots for pinning: p^{steps[i]} from the forward loop (padded grid,
 * [nsnap][pnz][pnx]) and from the boundary-strip rebuild of the backward
 * loop (interior grid, [nsnap][nz][nx]); steps[i] in [1, nt]. */
int  orc_probe(const orc_config *cfg, const float *vel, const orc_shot *shot,
               int nsnap, const int *steps, REAL_T *fwd_snaps, REAL_T *reb_snaps);

/* Single pieces for pinning against the reference kernels. */
int  orc_strips_write(const orc_config *cfg, const REAL_T *p_padded, REAL_T *ud, REAL_T *lr);
int  orc_strips_read(const orc_config *cfg, const REAL_T *ud, const REAL_T *lr, REAL_T *p_interior);
int  orc_apply_int(const orc_config *cfg, const REAL_T *p, REAL_T *ux, REAL_T *vz);

#ifdef __cplusplus
}
#endif
#endif
