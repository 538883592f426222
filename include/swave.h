/*
 * swave.h - C-ABI of the GB300 acoustic wave-equation engine (libswave.so).
 *
 * The engine replaces the hot path of the seismic suite's libwave:
 * the 8th-order / 5-level finite-difference propagator with Higdon absorbing
 * boundaries, sinc / nearest-node source injection and receiver extraction,
 * snapshot saving, the RTM / LSRTM / AFWI imaging conditions, the Born
 * secondary source, and the FWI objective/gradient plus its FP64 L-BFGS
 * update.  Every compute step runs in hand-written sm_103a CUDA kernels;
 * there is no CPU fallback.
 *
 * Conventions
 *  - All arrays are host arrays owned by the caller, read or written only
 *    during the call.  Device memory is owned by the context.
 *  - Model / image arrays are Fortran order, z fastest: a(nz, nx, ny).
 *  - Traces are trace-major, time fastest: trace r, sample it (1-based in
 *    the reference) lives at tr[r*nt + it-1].
 *  - Snapshots: wave(nz, nx, ny, ntsnap) with ntsnap = nt/snapi.
 *  - Coordinates are physical (z, x, y) triples in the same units as the
 *    grid origin and spacing.
 *  - Every entry point returns an sw_status; sw_last_error() gives text.
 *  - One context per host thread; calls on one context are serialised.
 */
#ifndef SWAVE_H
#define SWAVE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The reference aborts through erexit() instead
 * (e.g. libs/libwave/ReadSouVelRho.f90:650-756); these codes carry the
 * same conditions back to the caller. */
typedef enum sw_status {
  SW_OK = 0,
  SW_BAD_PARAM = 1,      /* invalid sizes, vel_check failure, bad coords    */
  SW_OOM_ADMISSION = 2,  /* the work does not fit the device memory budget  */
  SW_TIMEOUT = 3,        /* a bounded device-side wait ran out              */
  SW_NUMERIC = 4,        /* NaN / Inf in the FWI misfit or gradient; eps of
                            the regularisation not computable               */
  SW_CUDA_ERR = 5,       /* a CUDA runtime call failed                      */
  SW_UNSUPPORTED = 6     /* option not built (an adjoint grid with rho, ...) */
} sw_status;

/* Subset of GeneralParam (libs/libwave/GeneralParamTypes.f90:9-48) that the
 * propagation path reads.  nz/nx/ny are the (windowed) model sizes, i.e.
 * model%nz, model%nxw, model%nyw; oz/ox/oy the window origin
 * (genpar%omodel).  ny = 1 and twoD = 1 for 2D. */
typedef struct sw_genpar {
  int twoD;
  int nz, nx, ny;
  float dz, dx, dy;
  float oz, ox, oy;
  float dt;
  int nt;
  int ntaper;      /* padding cells per side (ReadParam.f90:19, default 20) */
  int lsinc;       /* sinc length (ReadParam.f90:24, default 7)             */
  int snapi;       /* snapshot decimation (ReadParam.f90:20, default 4)     */
  int surf_type, shot_type, rec_type;   /* 0: none; surf_type 1 / 2: sinc free
                      surface on a row / between rows (Boundary.f90:1609-1658);
                      shot_type, rec_type 1: mirror sources / receivers
                      (Injection.f90:274-338, Extraction.f90:276-337); all
                      entry points but sw_modeling_noalloc (0 only)          */
  float fmax;      /* used by vel_check only                                */
} sw_genpar;

/* The procedure arguments of propagator_acoustic
 * (libs/libwave/Propagator.f90:27-120) become enum selectors. */
typedef enum sw_fd_scheme {
  SW_FD_FORWARD = 0,  /* FD_2nd_{2D,3D}_derivatives_scalar_forward_grid   */
  SW_FD_ADJOINT = 1   /* FD_2nd_{2D,3D}_derivatives_scalar_adjoint_grid   */
} sw_fd_scheme;

typedef enum sw_injection {
  SW_INJ_NONE = 0,
  SW_INJ_SINC = 1,        /* Injection_sinc          (Injection.f90:151)    */
  SW_INJ_SIMPLE = 2,      /* Injection_simple_noomp  (Injection.f90:63)     */
  SW_INJ_LSRTM_SINC = 3   /* Injection_LSRTM_sinc    (Injection.f90:239)    */
} sw_injection;

typedef enum sw_extraction {
  SW_EXT_NONE = 0,
  SW_EXT_SINC = 1,         /* Extraction_array_sinc        (Extraction.f90:109) */
  SW_EXT_SIMPLE_AFWI = 2,  /* Extraction_array_simple_afwi (Extraction.f90:71)  */
  SW_EXT_LSRTM_SINC = 3,   /* Extraction_array_LSRTM_sinc  (Extraction.f90:217) */
  SW_EXT_SINC_AFWI = 4     /* Extraction_array_sinc_afwi   (Extraction.f90:137) */
} sw_extraction;

typedef enum sw_imaging {
  SW_IMG_NONE = 0,
  SW_IMG_RTM = 1,    /* Imaging_condition_sourceonly_from_memory (Imaging.f90:228) */
  SW_IMG_LSRTM = 2,  /* Imaging_condition_LSRTM_sourceonly_...   (Imaging.f90:698) */
  SW_IMG_AFWI = 3,   /* Imaging_condition_AFWI_from_memory       (Imaging.f90:371) */
  SW_IMG_BORN = 4,   /* Injection_Born                           (Imaging.f90:747) */
  SW_IMG_AFWI_RHO = 5 /* Imaging_condition_AFWI_RHOVP_from_memory (Imaging.f90:424):
                         the velocity gradient into image, the density
                         gradient into image2; needs rho (withRho)    */
} sw_imaging;

/* One propagation = one call of propagator_acoustic. */
typedef struct sw_prop_desc {
  sw_genpar g;
  int tmin, tmax, tstep;   /* genpar%tmin/tmax/tstep (tstep = +1 or -1) */
  int fd_scheme;           /* sw_fd_scheme  */
  int injection;           /* sw_injection  */
  int extraction;          /* sw_extraction */
  int extract_wave;        /* 1: Extraction_wavefield into io.wave       */
  int imaging;             /* sw_imaging    */
} sw_prop_desc;

/* Arrays of one propagation.  vel is the unpadded window velocity; the
 * engine pads it by edge replication exactly like model_pad
 * (ReadSouVelRho.f90:545-596).  NULL is allowed for every array the
 * selected options do not use. */
typedef struct sw_prop_io {
  const float *vel;         /* nz*nx*ny                                    */
  int nsou;
  const float *sou_coord;   /* 3*nsou  (z,x,y)                             */
  const float *sou_trace;   /* nsou*nt                                     */
  int nrec;
  const float *rec_coord;   /* 3*nrec                                      */
  float *rec_trace;         /* nrec*nt, accumulated (+=) like trace(it,1)  */
  float *wave;              /* nz*nx*ny*ntsnap: written by extract_wave,
                               read by the imaging conditions              */
  float *image;             /* nz*nx*ny accumulator (imagesmall)           */
  float *illum;             /* nz*nx*ny accumulator (illumsmall)           */
  const float *ref;         /* nz*nx*ny reflectivity for SW_IMG_BORN       */
  float *final_u2;          /* optional: padded u2 after the last step,
                               (nz+2nt+8)*(nx+2nt+8)*(ny>1?ny+2nt+8:1)    */
  const float *rho;         /* nz*nx*ny density (withRho), or NULL: the
                               variable-density operator
                               FD_{2D,3D}_derivatives_acoustic_forward_grid
                               (FDderivatives.f90:263-382,588-657) with
                               sinc- and nearest-node injection scaled by
                               v^2*rho (Injection.f90:170-190); requires
                               fd_scheme = SW_FD_FORWARD                   */
  float *image2;            /* nz*nx*ny second accumulator of
                               SW_IMG_AFWI_RHO (imagesmall_nparam(:,:,:,2)) */
} sw_prop_io;

typedef struct sw_ctx sw_ctx;

/* Context: one CUDA stream, a device-buffer arena, graph cache, counters. */
int sw_ctx_create(int device, sw_ctx **out);
int sw_ctx_destroy(sw_ctx *ctx);
const char *sw_last_error(const sw_ctx *ctx);

/* Library version string and the CUDA arch it was built for. */
const char *sw_version(void);

/* vel_check (ReadSouVelRho.f90:603-756): Courant <= 0.45 (2D) / 0.35 (3D)
 * and >= 2 samples per minimum wavelength.  Returns SW_OK or SW_BAD_PARAM;
 * *courant and *samplerate receive the computed numbers.  Host only. */
int sw_vel_check(const sw_genpar *g, const float *vel, float *courant,
                 float *samplerate);

/* propagator_acoustic (Propagator.f90:27-270) for one shot.  Step order per
 * time sample (Propagator.f90:168-234): extract(u2) -> snapshot(u2) ->
 * [imaging(u2) if tstep=-1] -> stencil(u2->u3) -> inject(u3) ->
 * [Born source(u3) if tstep=+1] -> 5-level time update -> Higdon -> rotate. */
int sw_propagate(sw_ctx *ctx, const sw_prop_desc *d, const sw_prop_io *io);

/* ---- Operator drivers (progs/{modeling,rtm,afwi}: to_disk_to_memory_*.f90) -
 * Snapshots stay in device memory between the two propagations. */

/* Acoustic modelling: forward, Injection_sinc, Extraction_array_sinc
 * (progs/modeling/Acoustic_modeling.f90:115-123). */
int sw_modeling(sw_ctx *ctx, const sw_genpar *g, const float *vel,
                const float *sou_coord, const float *wavelet,
                int nrec, const float *rec_coord, float *data,
                float *final_u2);

/* RTM_to_memory (progs/rtm/to_disk_to_memory_RTM.f90:358-492): forward with
 * snapshots, backward with the 2D adjoint (3D forward) stencil injecting the
 * data, zero-lag imaging.  image/illum are nz*nx*ny, overwritten. */
int sw_rtm(sw_ctx *ctx, const sw_genpar *g, const float *vel,
           const float *sou_coord, const float *wavelet,
           int nrec, const float *rec_coord, const float *data,
           float *image, float *illum);

/* BORN_to_memory (progs/modeling/to_disk_to_memory_BORN.f90:123-220).
 * wavelet must already be the 2nd time derivative (readsou with Born=T,
 * ReadSouVelRho.f90:318-326; see sw_born_wavelet).  data is overwritten. */
int sw_born(sw_ctx *ctx, const sw_genpar *g, const float *vel,
            const float *ref, const float *sou_coord, const float *wavelet,
            int nrec, const float *rec_coord, float *data);

/* LSRTM_to_memory (progs/rtm/to_disk_to_memory_RTM.f90:494-580): the Born
 * adjoint.  image/illum overwritten. */
int sw_lsrtm(sw_ctx *ctx, const sw_genpar *g, const float *vel,
             const float *sou_coord, const float *wavelet,
             int nrec, const float *rec_coord, const float *data,
             float *image, float *illum);

/* readsou's Born/LSRTM preprocessing (ReadSouVelRho.f90:318-326): in place
 * centred 2nd difference / dt^2. */
int sw_born_wavelet(float *wavelet, int nt, float dt);

/* bandpass (libs/libwave/Bandpass.f90:89-149, filters of bandpass.c): ntr
 * traces of nt samples (trace-major, in place) padded by 10 samples of
 * cosine-squared ramps at each end, then a Butterworth low-cut (flo Hz,
 * nplo poles) and high-cut (fhi Hz, nphi poles); phase 0 = zero phase
 * (each filter with half the poles, run forward and backward), 1 = minimum
 * phase.  The low-cut is skipped for flo*dt <= 1e-6; flo*dt < 1e-4 together
 * with fhi*dt > 0.4999 is refused.  Runs on the GPU, one thread per trace. */
int sw_bandpass(sw_ctx *ctx, int ntr, int nt, float dt, float flo, float fhi, int nplo,
                int nphi, int phase, float *traces);

/* MuteParam_compute_mask (libs/libwave/Mute.f90:50-95, 172-219): the mute
 * mask of nrec traces of nt samples (first sample at time ot), top mute at
 * sqrt(t0^2 + ((hx+hy)/v0)^2) with a sin^2 ramp of tramp seconds before it,
 * bottom mute at sqrt(t1^2 + ((hx+hy)/v1)^2) with a cos^2 ramp after it
 * (hx, hy: receiver minus source x and y).  mask is nrec*nt.  Host only;
 * defaults of the reference: v0 1500, v1 10000, t0 0, t1 40, tramp 0.5. */
int sw_mute_mask(int nrec, int nt, float dt, float ot, const float *sou_coord,
                 const float *rec_coord, float v0, float v1, float t0, float t1, float tramp,
                 float *mask);

/* readsou's withRho preprocessing (ReadSouVelRho.f90:328-343): in place,
 * w'(t) = w(t + dt/2) by an lsinc-point sinc (staggered grid), edge taps
 * dropped and the weights renormalised.  Host only. */
int sw_rho_wavelet(float *wavelet, int nt, int lsinc);

/* ---- Multi-shot RTM job (3DRTM.f90 per shot + compute_mig's stacking) ---
 * Shots of uneven aperture and record length are windowed out of one model
 * (extract_coord_source_receiver_patch + copy_window_vel_gath,
 * ExtractPadModel.f90:19-85,395-507), migrated with RTM_to_memory
 * (to_disk_to_memory_RTM.f90:358-492) and stacked into the full grid with
 * mod_copy_image (ExtractPadModel.f90:662-697).  Many shots advance in the
 * same kernel launches; the number per batch is set by their HBM footprint
 * (snapshots dominate).  All inputs are copied to device memory at
 * creation. */
typedef struct sw_shot {
  float sou_coord[3];
  int nrec;
  const float *rec_coord;   /* 3*nrec                                    */
  const float *data;        /* nrec*nt observed traces                   */
  int nt;                   /* record length of this shot, <= model g.nt */
} sw_shot;

typedef struct sw_rtm_job sw_rtm_job;
/* model: full-grid geometry (nz, nx, ny, spacing, origins, dt, nt = the
 * longest record, ntaper, lsinc, snapi); vel: nz*nx*ny; wavelet: g.nt. */
int sw_rtm_job_create(sw_ctx *ctx, const sw_genpar *model, float aperture_x,
                      float aperture_y, const float *vel, const float *wavelet,
                      int nshot, const sw_shot *shots, sw_rtm_job **out);
/* Admission: at most max_shots per batch and at most mem_fraction of the
 * free device memory (defaults 64 and 0.85). */
int sw_rtm_job_set_batch(sw_rtm_job *job, int max_shots, double mem_fraction);
/* Migrates shots [first, first+count) and adds them to the job's image.
 * Every migrated shot needs observed data. */
int sw_rtm_job_run(sw_rtm_job *job, int first, int count);
/* Forward modelling of shots [first, first+count), batched like the RTM:
 * Injection_sinc of the wavelet and Extraction_array_sinc at the receivers
 * (progs/modeling/Acoustic_modeling.f90:115-123) on each shot's window.
 * data[q] receives the nrec*nt traces of shot first+q.  Shots may have been
 * created without observed data (sw_shot.data = NULL). */
int sw_rtm_job_model(sw_rtm_job *job, int first, int count, float *const *data);
/* How many shots from shot `first` the admission above puts in one batch
 * now (the job's max_shots and mem_fraction, the device memory free at the
 * call, the job's arena counted as free), for an RTM run (modeling = 0:
 * snapshots of every shot) or a modelling run (modeling = 1: traces).
 * Host only.  SW_OOM_ADMISSION, with *count = 0, when shot `first` alone
 * does not fit.  No counterpart in the reference (its shot loop holds one
 * shot per thread). */
int sw_rtm_job_admit(sw_rtm_job *job, int first, int modeling, int *count);
/* Shots per batch used by the last run, and compute-domain point updates. */
int sw_rtm_job_info(const sw_rtm_job *job, int *last_batch, uint64_t *points);
/* image, illum: stacked nz*nx*ny sums; image_norm: image divided by the
 * normalised illumination (compute_function_gradient.f90:452-453).  Any
 * pointer may be NULL. */
int sw_rtm_job_result(sw_rtm_job *job, float *image, float *illum, float *image_norm);
int sw_rtm_job_reset(sw_rtm_job *job);
int sw_rtm_job_destroy(sw_rtm_job *job);

/* ---- Shot windows (host only; no context) --------------------------------
 * The source/receiver patch widened by the aperture
 * (extract_coord_source_receiver_patch, ExtractPadModel.f90:19-85) and its
 * grid size (read_window_vel, ExtractPadModel.f90:176-182): nxw =
 * nint((endx - oxw)/dx) + 1, and likewise in y (nyw = 1, oyw = oy in 2D).
 * The window's genpar is the model's with nx = nxw, ny = nyw, ox = oxw,
 * oy = oyw. */
typedef struct sw_window {
  float oxw, oyw, endx, endy;
  int nxw, nyw;
} sw_window;
int sw_shot_window(const sw_genpar *model, float aperture_x, float aperture_y,
                   const float *sou_coord, int nrec, const float *rec_coord, sw_window *out);
/* small (nz*nxw*nyw) = the model columns nearest each window column, clamped
 * to the model (mod_window_pad adj=.true., ExtractPadModel.f90:517-531). */
int sw_window_extract(const sw_genpar *model, const sw_window *w, const float *big, float *small);
/* big (nz*nx*ny) += the window columns that fall inside the model
 * (mod_window_pad adj=.false. and mod_copy_image_to_disk,
 * ExtractPadModel.f90:532-546,551-590). */
int sw_window_scatter_add(const sw_genpar *model, const sw_window *w, const float *small,
                          float *big);

/* ---- FWI objective / gradient (progs/afwi/compute_function_gradient.f90) */

typedef struct sw_fwi_shot {
  float sou_coord[3];
  int nrec;
  const float *rec_coord;   /* 3*nrec                                    */
  const float *dobs;        /* nrec*nt observed data                     */
  const float *mute;        /* nrec*nt mute mask (NULL = all ones)       */
  float *resid;             /* optional out: nrec*nt residual            */
} sw_fwi_shot;

typedef struct sw_fwi_desc {
  sw_genpar g;              /* full-model geometry: nz, nx, ny, origins    */
  float aperture_x, aperture_y;
  float illu_pow;           /* invparam%illupow (default 1)               */
  int smooth_rect1, smooth_rect2, smooth_rect3;  /* triangle2 half-widths  */
  int smooth_doz, smooth_dox, smooth_doy;
  /* Snapshot memory (no counterpart in the reference, which keeps every
   * snapshot in RAM or on disk, 3DRTM.f90:77-109):
   *   0      store all ntsnap snapshots of a shot in HBM;
   *   K > 0  keep the forward state (4 padded fields) every K snapshots and
   *          recompute K + 2 snapshots at a time during the backward pass:
   *          memory (ntsnap/K) x 4 padded fields + (K + 2) snapshots, one
   *          extra forward propagation; results identical to store-all. */
  int checkpoint_snaps;
  /* Data norm of the misfit and its adjoint source (invparam%dat_nrm_type,
   * Inversion_types.f90:61-68; fct_compute / gdt_compute,
   * libs/libinv/Norm.f90:12-141): SW_NRM_L2 (also 0), SW_NRM_L1,
   * SW_NRM_HUBER, SW_NRM_CAUCHY, SW_NRM_HYPERBOLIC.  dat_thresh is
   * data_threshold; when it is 0 the threshold of a shot is max|r| of the
   * first of its traces whose muted residual r is not all zero
   * (Norm.f90:37-40 resets the caller's threshold, which the following
   * traces of the gather then use). */
  int dat_nrm_type;
  float dat_thresh;
  /* Binomial checkpointing (revolve; no counterpart in the reference): with
   * checkpoint_snaps = K > 0 and revolve_slots = s > 0 the forward states
   * at segment boundaries are kept in s slots (+ one work slot) chosen by
   * the binomial schedule over the ntsnap/K segments instead of all of
   * them: memory (s + 1) x 4 padded fields + (K + 2) snapshots, segment
   * advances = the minimum for s + 1 checkpoints (the zero initial state
   * is the first); results identical to store-all.  0 = every boundary. */
  int revolve_slots;
} sw_fwi_desc;

enum { SW_NRM_L1 = 1, SW_NRM_L2 = 2, SW_NRM_CAUCHY = 3, SW_NRM_HYPERBOLIC = 4,
       SW_NRM_HUBER = 12 };

/* compute_fct_gdt (compute_function_gradient.f90:208-350): for every shot
 * window + pad the model, AMOD (forward, nearest-node extraction,
 * snapshots), residual/misfit (FP64), AGRAD (backward with the AFWI imaging
 * condition), scatter-add into the full grid; then scaling, illumination
 * normalisation, mask, triangle smoothing, mask.  vel/grad/illum/mask are
 * nz*nx*ny.  *f receives the FP64 misfit.  A misfit or gradient that is not
 * finite returns SW_NUMERIC (the outputs then hold what was computed). */
int sw_fwi_fct_gdt(sw_ctx *ctx, const sw_fwi_desc *d, const float *vel,
                   const float *wavelet, int nshot, const sw_fwi_shot *shots,
                   const float *vpmask, double *f, float *grad, float *illum);

/* ---- Model regularisation of 2DAFWI (compute_fct_gdt_reg,
 * progs/afwi/compute_function_gradient.f90:98-206) ----------------------
 * wantreg: SparseRegularization_apply (libs/libwave/Sparse_regularization.
 * f90:238-327): the model, padded by edge replication (sparse_taperz/x/y),
 * is differenced by the helix filters 1 - Z^lag (lag 1 along z, nz+2*taperz
 * along x; derivdy applies the x filter a second time, as the reference's
 * helicon2_mod_lop does), weighted by Z_weights, and its norm
 * (model_nrm_type, reg_threshold) and gradient are formed; log_z_plus keeps
 * only the positive z differences.  wantlog: LogisticRegularization_apply
 * (:329-397): the z difference where it is <= 0 under hinge_nrm_type and
 * hin_threshold.  Both terms are divided by nz*nx*ny, weighted by eps and
 * eps_log (computed at evaluation 0 from ratio / ratio_log when
 * compute_eps / compute_eps_log) and added to f and subtracted from grad;
 * grad is then multiplied by vpmask (always, also without
 * regularisation).  Norms are taken, as in the reference, over the first
 * nz*nx samples of the model and the first (nz+2*taperz)*(nx+2*taperx) of
 * the padded differences. */
typedef struct sw_reg_desc {
  int nz, nx, ny;
  int wantreg, wantlog;
  int derivdx, derivdy, derivdz, log_z_plus;
  int ntaperz, ntaperx, ntapery;  /* sparse_taperz/x/y (10, 10, 0); y is 0 in 2D */
  int mod_nrm_type, hin_nrm_type; /* SW_NRM_*; model_nrm_type, hinge_nrm_type */
  int compute_eps, compute_eps_log;
  float ratio, ratio_log;         /* ratio (10), ratio_logistic (10)           */
  const float *zweight;           /* Z_weights (nz*nx*ny) or NULL              */
} sw_reg_desc;

/* What compute_fct_gdt_reg keeps between evaluations: eps and eps_log
 * (parameters eps / eps_log, default 1, or the computed values), and the
 * norm thresholds, which fct_compute sets to max|.| when they are 0 and
 * which then stay set. */
typedef struct sw_reg_state {
  float eps, eps_log;
  float mod_thresh, hin_thresh;
} sw_reg_state;

/* f and grad hold compute_fct_gdt's misfit and gradient (nz*nx*ny) on entry
 * and compute_fct_gdt_reg's on return; eval is invparam%eval (0 on the first
 * evaluation).  vel is the current model, vpmask the inversion mask (NULL =
 * ones). */
int sw_fwi_regularize(sw_ctx *ctx, const sw_reg_desc *d, sw_reg_state *state, int eval,
                      const float *vel, const float *vpmask, double *f, float *grad);

/* ---- L-BFGS (libs/libinv/lbfgs.f:49-558, FP64 on the device) ----------
 * Reverse communication exactly like LBFGS(): the caller evaluates f and g
 * at x whenever *iflag returns 1, and calls again. */
typedef struct sw_lbfgs sw_lbfgs;
int sw_lbfgs_create(sw_ctx *ctx, int n, int m, double xmin, double xmax,
                    const float *mask, int bound_type, int freeze_soft,
                    const double *xinit, sw_lbfgs **out);
int sw_lbfgs_destroy(sw_lbfgs *s);
/* x: n doubles (in/out), f, g: n doubles.  iflag (in/out) and info (out)
 * follow LBFGS: iflag=0 on the first call; 1 = evaluate and call again;
 * 0 = converged; <0 = error.  *myinfo = 1 when an iteration completed. */
int sw_lbfgs_step(sw_lbfgs *s, double *x, double f, const double *g,
                  double eps, double xtol, int *iflag, int *myinfo);
/* Scalars of the last step: [iter, nfun, stp, gnorm, ys, yy, dginit, dg]. */
int sw_lbfgs_diag(const sw_lbfgs *s, double *out8);

/* ---- Out-of-core L-BFGS (libs/libnlinv/nlinv_lbfgs.f) ----------------------
 * LBFGSOC / MCSRCHOC (lbfgs_type 1: per-parameter bounds, nlinv_lbfgs.f:
 * 1-22,31-967) and LBFGSOLD / MCSRCHOLD (lbfgs_type 0: no bounds,
 * :1066-1990), the solver of progs/inversion/L_BFGS.f90.  One call is one
 * reverse-communication call of the reference: the caller keeps everything
 * the solver saves between calls (the reference keeps it in files between
 * program invocations: WorkArray.dat, Diag.dat, LbfgsDat.dat,
 * McsrchDat.dat, Iflag.dat, Info.dat) and hands it back on the next call.
 * The vectors run on the device in FP64 during the call. */
typedef struct sw_lbfgs_oc_state {
  /* LBFGSOC's SAVE scalars, in the order of LbfgsDat.dat
   * (nlinv_lbfgs.f:277-281) */
  double gtol, one, zero, gnorm, stp1, ftol, stpmin;
  double stpmax, stp, ys, yy, sq, yr, beta, xnorm;
  int mp, lp, iter, nfun, point, ispt, iypt, maxfev, info;
  int bound, npt, cp, i, nfev, inmc, iycn, iscn;
  int finish;
  /* MCSRCHOC's SAVE scalars, in the order of McsrchDat.dat (:725-730) */
  int infoc, j;
  int brackt, stage1;
  double dg, dgm, dginit, dgtest, dgx, dgxm, dgy, dgym;
  double finit, ftest1, fm, fx, fxm, fy, fym, stx, sty;
  double stmin, stmax, width, width1;
} sw_lbfgs_oc_state;

typedef struct sw_lbfgs_oc_desc {
  int n;                  /* model size (all parameters)                    */
  int m;                  /* corrections kept (MSAVE, 5 in L_BFGS.f90)       */
  int nparam;             /* parameter blocks of n / nparam values           */
  const double *xmin;     /* nparam lower bounds (lbfgs_type 1)              */
  const double *xmax;     /* nparam upper bounds                             */
  int lbfgs_type;         /* 0: LBFGSOLD, no clipping; 1: LBFGSOC            */
  int bound_type;         /* 1: clip every trial model, 2: every new iterate */
  int stp1_opt;           /* first trial step: 1: |x| / |g| / 100, else 1 / |g| */
  double step_init;       /* 999999: none; else the first trial step          */
  double eps, xtol;       /* 1e-20 and machine epsilon in L_BFGS.f90          */
} sw_lbfgs_oc_desc;

/* One LBFGSOC call.  x (n, in/out): the model; f and g (n): the objective
 * and gradient at x; w (n(2m+1) + 2m) and diag (n): the working array and
 * DIAG in the reference's layout; state, *iflag and *myinfo in and out.
 * *iflag = 0 starts a new solve (w, diag and state are then written, not
 * read).  Returns with *iflag = 1 (evaluate f, g at x and call again),
 * 0 (converged) or < 0 (the reference's error codes); *myinfo = 1 when the
 * call completed an iteration. */
int sw_lbfgs_oc_step(sw_ctx *ctx, const sw_lbfgs_oc_desc *d, double *x, double f,
                     const double *g, double *w, double *diag, sw_lbfgs_oc_state *state,
                     int *iflag, int *myinfo);

/* ---- Tuning (no counterpart in the reference: launch shape knobs) -------- */
typedef struct sw_tuning {
  int step_kernel;   /* fused step: 0 = 32x8 point tiles, 1 = streaming, 2 = TMA-staged
                        tiles, 2 CTAs per SM (default), 3 = TMA-staged tiles,
                        warp-specialised, 4 = two time steps per launch on 64x64 TMA tiles
                        for 2D batches of up to 32 shots without AFWI / Born
                        imaging (others run 2); 3D uses streaming for 1 and the
                        TMA plane pipeline for 2-4 */
  int tile_z;        /* 2D streaming kernel: rows per CTA (32, 64 or 128)     */
  int tile_x;        /* 2D streaming kernel: columns walked per CTA (>= 1)    */
  int tile_y;        /* 3D streaming kernel: y planes marched per CTA (>= 1)  */
  int graph_chunk;   /* time steps per captured CUDA graph (>= 1)             */
  int use_graph;     /* 0: launch every step directly                         */
} sw_tuning;
int sw_ctx_set_tuning(sw_ctx *ctx, const sw_tuning *t);
int sw_ctx_get_tuning(const sw_ctx *ctx, sw_tuning *t);

/* ---- Convolutional gradient preconditioner (N4) --------------------------- */
/* No counterpart in the reference.  A stack of nlayers 3x3 convolutions
 * (zero padding, ReLU between layers, channels[0..nlayers], each 1..32,
 * the last 1) mapping planar FP32 input channels of an nz x nx image
 * (z fastest) to one output channel.  BF16 weights, activations and
 * back-propagated gradients on the tcgen05 tensor cores (convolutions,
 * input gradients and weight gradients) with FP32 accumulation; FP32
 * master weights and Adam state.  Weights are packed per layer as
 * w[co][tap][ci] (tap = 3 * (dx + 1) + (dz + 1)) followed by b[co]. */
typedef struct sw_cnn sw_cnn;
int sw_cnn_create(sw_ctx *ctx, int nlayers, const int *channels, uint64_t seed, sw_cnn **out);
int sw_cnn_destroy(sw_cnn *net);
int sw_cnn_num_weights(const sw_cnn *net);
int sw_cnn_get_weights(const sw_cnn *net, float *w);
int sw_cnn_set_weights(sw_cnn *net, const float *w);
/* in: channels[0] x nz x nx (planar), out: nz x nx. */
int sw_cnn_forward(sw_cnn *net, int nz, int nx, const float *in, float *out);
/* grad (sw_cnn_num_weights values, packed like the weights) receives the
 * gradient of the mean over nbatch images of 0.5 * mean((out - target)^2)
 * and *loss that mean loss; the weights do not change.  in: nbatch x
 * channels[0] x nz x nx, target: nbatch x nz x nx. */
int sw_cnn_gradient(sw_cnn *net, int nbatch, int nz, int nx, const float *in,
                    const float *target, float *grad, double *loss);
/* One Adam step (lr; beta 0.9 / 0.999) on the mean over nbatch images of
 * 0.5 * mean((out - target)^2); *loss receives that mean loss. */
int sw_cnn_train_step(sw_cnn *net, int nbatch, int nz, int nx, const float *in,
                      const float *target, float lr, double *loss);
/* The same network with 3 x 3 x 3 kernels on nz x nx x ny volumes (z
 * fastest, then x): weights packed per layer as w[co][tap][ci] with tap =
 * 9 * (dy + 1) + 3 * (dx + 1) + (dz + 1), then b[co].  The image entry
 * points above take 3 x 3 networks only and these 3 x 3 x 3 networks only
 * (SW_BAD_PARAM otherwise). */
int sw_cnn_create3d(sw_ctx *ctx, int nlayers, const int *channels, uint64_t seed, sw_cnn **out);
int sw_cnn_forward3d(sw_cnn *net, int nz, int nx, int ny, const float *in, float *out);
int sw_cnn_gradient3d(sw_cnn *net, int nbatch, int nz, int nx, int ny, const float *in,
                      const float *target, float *grad, double *loss);
int sw_cnn_train_step3d(sw_cnn *net, int nbatch, int nz, int nx, int ny, const float *in,
                        const float *target, float lr, double *loss);

/* ---- Modelling without device allocation --------------------------------- */
/* No counterpart in the reference (its modelling allocates the wavefields of
 * every shot it runs).  Same arguments, run and results as sw_modeling for
 * a 2D model (host arrays in and out), for callers that cannot allocate
 * device memory during the call: a process whose device memory is committed
 * to its own pool (e.g. an RTM job's snapshot arena) or one that must not
 * let cudaMalloc / cudaFree synchronise the device mid-run.  It allocates
 * nothing: every device array lives in one file-scope scratch array of
 * 32 MiB that each GPU loading the library holds until the process exits,
 * which limits the padded grid to about 1.3 million points (6 float arrays
 * of ld1 x (nx + 2*ntaper + 8) plus plans and traces).  Larger runs return
 * SW_OOM_ADMISSION before any device work.  Runs on the current device's
 * legacy default stream and returns when the traces are on the host.  The
 * first call on a device looks the scratch array's device address up there
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * All calls share the array: calls that overlap on the GPU (from several
 * host threads at once) race on it.  Do not cudaDeviceReset a device this
 * entry point has run on (the cached address would go stale).  3D models
 * and surf_type / shot_type / rec_type other than 0 return SW_UNSUPPORTED;
 * a bounded device wait that gave up returns SW_TIMEOUT. */
int sw_modeling_noalloc(const sw_genpar *g, const float *vel, const float *sou_coord,
                        const float *wavelet, int nrec, const float *rec_coord, float *data);

/* ---- Instrumentation ----------------------------------------------------- */
typedef struct sw_stats {
  uint64_t launches_total;      /* kernels launched by this context          */
  uint64_t launches_step;       /* fused stencil/time-update launches        */
  uint64_t points_updated;      /* compute-domain point updates              */
  double   step_kernel_ms;      /* event-timed total of the fused kernel
                                   (only while profiling is on)              */
  uint64_t step_kernel_timed;   /* number of timed fused-kernel launches     */
  uint64_t step_bytes;          /* algorithmic bytes of those launches       */
  uint64_t steps_forward;       /* time steps of forward (tstep = +1) runs    */
  uint64_t steps_backward;      /* time steps of backward (tstep = -1) runs   */
  uint64_t ckpt_advances;       /* checkpoint-segment advances of FWI runs    */
  double   cnn_conv_ms;         /* event-timed total of the preconditioner's
                                   tensor-core convolution and weight-gradient
                                   kernels (only while profiling is on)      */
  uint64_t cnn_conv_timed;      /* number of those timed launches            */
  uint64_t cnn_conv_bytes;      /* their algorithmic HBM bytes (activations
                                   and gradients read once, outputs written)  */
  uint64_t cnn_conv_flops;      /* their tensor-core FLOPs (2 x M x N x K of
                                   the real channels)                        */
} sw_stats;
int sw_ctx_get_stats(const sw_ctx *ctx, sw_stats *out);
int sw_ctx_reset_stats(sw_ctx *ctx);
/* Boundary of every propagation on this context: 0 = the reference's
 * Higdon absorbing boundary (default), 1 = rigid (no Higdon recurrence,
 * zero halo; no counterpart in the reference).  With 1 the Born
 * (sw_born) and LSRTM (sw_lsrtm) operators are an exact adjoint pair: the
 * Higdon boundary is what makes the reference's pair approximate. */
int sw_ctx_set_boundary(sw_ctx *ctx, int mode);
/* on=1: bracket fused-kernel launches with CUDA events: every launch when
   the time loop runs without a CUDA graph, otherwise the launches of every
   8th graph chunk (the event records cost a few microseconds each). */
int sw_ctx_set_profiling(sw_ctx *ctx, int on);

#ifdef __cplusplus
}
#endif
#endif /* SWAVE_H */
