/*
 * oracle.h - CPU restatement of the reference libwave/libinv hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (seismic_gb300/) links,
 * loads or calls this code; only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py use it, as the result
 * the GPU path is compared against and as the timed CPU baseline.
 *
 * Parity status: UNPINNED.  The reference is Fortran (ifort + SEPlib) and
 * cannot be compiled in this environment, and its tree holds no golden
 * vectors or known-answer tests for this path.  The restatement is pinned
 * instead by analytic checks (tests/test_oracle_analytic.py): stencil
 * exactness on polynomials, the time scheme's characteristic roots, Higdon
 * coefficient identities, sinc normalisation, and dot-product / adjoint
 * identities; plus committed fixtures that freeze its outputs.
 *
 * Arithmetic follows the Fortran evaluation order term by term (left to
 * right, explicit parentheses), compiled with -ffp-contract=off, so the
 * FP32 build is a well-defined IEEE-754 sequence.  The FP64 twin (_f64
 * entry points) runs the identical algorithm in double precision and is the
 * accuracy yardstick.
 */
#ifndef SWAVE_ORACLE_H
#define SWAVE_ORACLE_H

#include "../include/swave.h"

#ifdef __cplusplus
extern "C" {
#endif

/* FP64 twin of sw_prop_io: every float array becomes double. */
typedef struct or_prop_io64 {
  const double *vel;
  int nsou;
  const double *sou_coord;
  const double *sou_trace;
  int nrec;
  const double *rec_coord;
  double *rec_trace;
  double *wave;
  double *image;
  double *illum;
  const double *ref;
  double *final_u2;
  const double *rho;
  double *image2;
} or_prop_io64;

/* propagator_acoustic (libs/libwave/Propagator.f90:27-270). */
int oracle_propagate_f32(const sw_prop_desc *d, const sw_prop_io *io);
int oracle_propagate_f64(const sw_prop_desc *d, const or_prop_io64 *io);

/* Drivers, same meaning as the sw_* entry points of the same name. */
int oracle_modeling_f32(const sw_genpar *g, const float *vel,
                        const float *sou_coord, const float *wavelet,
                        int nrec, const float *rec_coord, float *data,
                        float *final_u2);
int oracle_modeling_f64(const sw_genpar *g, const double *vel,
                        const double *sou_coord, const double *wavelet,
                        int nrec, const double *rec_coord, double *data,
                        double *final_u2);
int oracle_rtm_f32(const sw_genpar *g, const float *vel,
                   const float *sou_coord, const float *wavelet, int nrec,
                   const float *rec_coord, const float *data, float *image,
                   float *illum);
int oracle_rtm_f64(const sw_genpar *g, const double *vel, const double *sou_coord,
                   const double *wavelet, int nrec, const double *rec_coord,
                   const double *data, double *image, double *illum);
int oracle_born_f32(const sw_genpar *g, const float *vel, const float *ref,
                    const float *sou_coord, const float *wavelet, int nrec,
                    const float *rec_coord, float *data);
int oracle_born_f64(const sw_genpar *g, const double *vel, const double *ref,
                    const double *sou_coord, const double *wavelet, int nrec,
                    const double *rec_coord, double *data);
int oracle_lsrtm_f32(const sw_genpar *g, const float *vel,
                     const float *sou_coord, const float *wavelet, int nrec,
                     const float *rec_coord, const float *data, float *image,
                     float *illum);
int oracle_lsrtm_f64(const sw_genpar *g, const double *vel,
                     const double *sou_coord, const double *wavelet, int nrec,
                     const double *rec_coord, const double *data,
                     double *image, double *illum);
/* bandpass (Bandpass.f90:89-149, bandpass.c), in place over trace-major data. */
int oracle_bandpass(float *traces, int ntr, int nt, float dt, float flo, float fhi, int nplo,
                    int nphi, int phase);
int oracle_mute_mask(int nrec, int nt, float dt, float ot, const float *sou,
                     const float *rec, float v0, float v1, float t0, float t1, float tramp,
                     float *mask);
int oracle_rho_wavelet(float *w, int nt, int lsinc);
int oracle_born_wavelet(float *wavelet, int nt, float dt);
int oracle_vel_check(const sw_genpar *g, const float *vel, float *courant,
                     float *samplerate);

/* compute_fct_gdt (progs/afwi/compute_function_gradient.f90:208-350). */
int oracle_fwi_fct_gdt(const sw_fwi_desc *d, const float *vel,
                       const float *wavelet, int nshot,
                       const sw_fwi_shot *shots, const float *vpmask,
                       double *f, float *grad, float *illum);

/* Compute_OF_RES_ADJ of one gather (Objective_Function_Residual_Adjsource.f90:
 * 17-40 with libs/libinv/Norm.f90): dmod holds the nrec*nt modelled traces
 * and receives the adjoint source; resid (optional) the muted residual;
 * *f the gather's misfit.  ntype is SW_NRM_* (0 = L2). */
int oracle_data_norm(int ntype, float thresh, int nrec, int nt, const float *dobs,
                     const float *mute, float *dmod, float *resid, double *f);

/* compute_fct_gdt_reg's regularisation terms, same meaning as
 * sw_fwi_regularize. */
int oracle_fwi_regularize(const sw_reg_desc *d, sw_reg_state *state, int eval, const float *vel,
                          const float *vpmask, double *f, float *grad);

/* Multi-shot RTM stacking, same meaning as sw_rtm_job_* run over all shots. */
int oracle_rtm_job(const sw_genpar *model, float apx, float apy, const float *vel,
                   const float *wavelet, int nshot, const sw_shot *shots, float *image,
                   float *illum, float *image_norm);

/* LBFGS (libs/libinv/lbfgs.f:49-558) with its SAVE state in a handle. */
typedef struct or_lbfgs or_lbfgs;
or_lbfgs *oracle_lbfgs_create(int n, int m, double xmin, double xmax,
                              const float *mask, int bound_type,
                              int freeze_soft, const double *xinit);
void oracle_lbfgs_destroy(or_lbfgs *s);
int oracle_lbfgs_step(or_lbfgs *s, double *x, double f, const double *g,
                      double eps, double xtol, int *iflag, int *myinfo);
void oracle_lbfgs_diag(const or_lbfgs *s, double *out8);
int oracle_lbfgs_oc_step(const sw_lbfgs_oc_desc *d, double *x, double f, const double *g,
                         double *w, double *diag, sw_lbfgs_oc_state *st, int *iflag,
                         int *myinfo);

/* triangle2 smoothing (libs/libwave/Smoothing.f90:87-138), in place. */
int oracle_triangle2(float *uu, int n1, int n2, int n3, int rect1, int rect2,
                     int rect3, int doz, int dox, int doy);

/* One stencil application on a padded FP64 field (analytic tests). */
/* 1: skip the Higdon boundary in every propagation (rigid halo). */
void oracle_set_rigid(int on);
int oracle_stencil_f64(const sw_genpar *g, int adjoint, const double *vel,
                       const double *u2, double *u3);
/* One application of the variable-density operator v^2*rho*div(grad(u2)/rho2)
 * (FDderivatives.f90:263-382,588-657) to a padded field, FP64. */
int oracle_stencil_rho_f64(const sw_genpar *g, const double *vel, const double *rho,
                           const double *u2, double *u3);

/* mksinc (libs/libwave/Interpolate.f90:15-42). */
void oracle_mksinc(float *sinc, int lsinc, float shift);

#ifdef __cplusplus
}
#endif
#endif
