/* 2DAFWI.x - multi-shot acoustic modelling and migration over a survey
 * (progs/afwi/2DAFWI.f90).  The wavelet comes from stdin= (or standard
 * input), the model from vel=, and the survey from coordfile= (n1 keys by
 * n2 traces); consecutive traces with the same (sx, sy) form one shot
 * gather (readgathercoords, ReadSouVelRho.f90:139-212,828-890).  Every
 * gather is propagated on its own window of the model (aperture_x,
 * aperture_y).
 *
 *   Task=MOD: compute_mod (compute_function_gradient.f90:472-588): AMOD
 *     forward modelling (sinc injection, nearest-node AFWI extraction) of
 *     every gather; data= receives all traces in coordfile order.
 *   Task=MIG: compute_mig (compute_function_gradient.f90:352-470): AMOD
 *     with snapshots, then the AGRAD back-propagation of the recorded traces
 *     of traces= (nearest-node injection, AFWI imaging condition); the
 *     gathers' images and illuminations are stacked on the full grid and
 *     image= receives image / ((illum + max/10000) / rms(illum)).
 *   Task=INV: the inversion of 2DAFWI.f90:73-100.  The wavelet and the
 *     traces are band-passed (sw_bandpass; fhi, flo, nphi, nplo, phase),
 *     the residuals muted (sw_mute_mask; v0, v1, t0, t1, tramp), the
 *     gradient smoothed over percx/percz of the reference wavelength; then
 *     the l_bfgs loop of Inversion.f90:29-189 over sw_fwi_fct_gdt and the
 *     device L-BFGS (niter, neval, vpmin, vpmax, bound, freeze_soft,
 *     illu_pow, vpmask=).  inv= receives the final model after Freeze and
 *     ApplyMask; model=, gradient=, function= and residual= (when given)
 *     receive every iteration's model, gradient, scaled misfit and residual
 *     traces.  data_nrm_type (L2norm, L1norm, Huber, Cauchy) and
 *     data_threshold select the data norm; wantreg / wantlog add the sparse
 *     and logistic model regularisation of compute_fct_gdt_reg
 *     (sw_fwi_regularize: derivdx/dy/dz, log_z_plus, model_nrm_type,
 *     hinge_nrm_type, eps/ratio, eps_log/ratio_logistic, reg_threshold,
 *     hin_threshold, sparse_taperx/y/z, Z_weights=).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "swcli.h"

typedef struct gather {
  int begi, ntr;   /* first trace (0-based) and trace count */
  float sou[3];
} gather;

static float *read_all_keys(int *nkeys_out, int *ntot_out) {
  if (!sep_exist("coordfile")) cli_fail("need coordfile");
  sep_file *f = sep_open_in("coordfile");
  if (!f) cli_fail("%s", sep_error());
  int nkeys = 0, ntot = 0;
  if (sep_hdr_int(f, "n1", &nkeys) != 1 || nkeys < 1) cli_fail("coordfile header needs n1");
  if (sep_hdr_int(f, "n2", &ntot) != 1 || ntot < 1) cli_fail("coordfile header needs n2");
  float *keys = (float *)malloc((size_t)nkeys * ntot * 4);
  if (!keys) cli_fail("out of host memory");
  if (sep_read(f, keys, (size_t)nkeys * ntot)) cli_fail("%s", sep_error());
  sep_close(f);
  *nkeys_out = nkeys;
  *ntot_out = ntot;
  return keys;
}

static float maxabs(const float *a, size_t n) {
  float m = 0.f;
  for (size_t i = 0; i < n; ++i) m = fabsf(a[i]) > m ? fabsf(a[i]) : m;
  return m;
}

/* Freeze (2DAFWI.f90:224-244) and ApplyMask (2DAFWI.f90:214-222). */
static void freeze_and_mask(float *x, size_t n, float xmin, float xmax, const float *mask,
                            int soft, const double *xinit) {
  for (size_t i = 0; i < n; ++i) {
    if (soft) {
      x[i] = xmin > x[i] ? xmin : x[i];
      x[i] = xmax < x[i] ? xmax : x[i];
    } else if (mask[i] != 0.f && mask[i] != 2.f) {
      x[i] = xmin > x[i] ? xmin : x[i];
      x[i] = xmax < x[i] ? xmax : x[i];
    }
  }
  if (!soft)
    for (size_t i = 0; i < n; ++i)
      if (mask[i] == 0.f || mask[i] == 2.f) x[i] = (float)xinit[i];
  for (size_t i = 0; i < n; ++i) x[i] = mask[i] * x[i] + (1.f - mask[i]) * (float)xinit[i];
}

/* FREEZE_X (libs/libinv/lbfgs.f) on the saved model. */
static void freeze_x(double *x, size_t n, double xmin, double xmax, const float *mask, int soft,
                     const double *xinit) {
  for (size_t i = 0; i < n; ++i)
    if (soft || (mask[i] != 0.f && mask[i] != 2.f)) {
      x[i] = xmin > x[i] ? xmin : x[i];
      x[i] = xmax < x[i] ? xmax : x[i];
    }
  if (!soft)
    for (size_t i = 0; i < n; ++i)
      if (mask[i] == 0.f || mask[i] == 2.f) x[i] = xinit[i];
}

static sep_file *open_optional(const char *tag) {
  if (!sep_exist(tag)) return NULL;
  sep_file *f = sep_open_out(tag);
  if (!f) cli_fail("%s", sep_error());
  return f;
}

static void put_model_axes(sep_file *f, const sw_genpar *g) {
  sep_put_int(f, "n1", g->nz);
  sep_put_int(f, "n2", g->nx);
  sep_put_int(f, "n3", g->ny);
  sep_put_float(f, "d1", g->dz);
  sep_put_float(f, "d2", g->dx);
  sep_put_float(f, "d3", g->dy);
  sep_put_float(f, "o1", g->oz);
  sep_put_float(f, "o2", g->ox);
  sep_put_float(f, "o3", g->oy);
}

/* Task=INV (2DAFWI.f90:73-100, Inversion.f90:29-189). */
static int run_inversion(sw_ctx *ctx, cli_par *p, float *wavelet, float *vel, float *traces,
                         float ot, const float *rec, int ntot, const gather *gs, int ng) {
  const sw_genpar *g = &p->g;
  const int nt = g->nt;
  const size_t n = (size_t)g->nz * g->nx * g->ny;
  /* read_inv_params (Inversion_types.f90:46-104). */
  int niter = 10, neval, freeze_soft = 1, bound = 2, wantreg = 0, wantlog = 0;
  float vpmin = 1500.f, vpmax = 4500.f, illu_pow = 1.f;
  char nrm[32] = "L2norm";
  sep_par_int("niter", &niter);
  neval = 3 * niter;
  sep_par_int("neval", &neval);
  sep_par_float("vpmin", &vpmin);
  sep_par_float("vpmax", &vpmax);
  sep_par_bool("freeze_soft", &freeze_soft);
  sep_par_int("bound", &bound);
  sep_par_bool("wantreg", &wantreg);
  sep_par_bool("wantlog", &wantlog);
  sep_par_float("illu_pow", &illu_pow);
  sep_par_str("data_nrm_type", nrm, sizeof(nrm));
  float dat_thresh = 0.f;
  sep_par_float("data_threshold", &dat_thresh);
  int nrm_type = 0;
  if (strncmp(nrm, "Cauch", 5) == 0) nrm_type = SW_NRM_CAUCHY;
  if (strncmp(nrm, "Huber", 5) == 0) nrm_type = SW_NRM_HUBER;
  if (strncmp(nrm, "L1nor", 5) == 0) nrm_type = SW_NRM_L1;
  if (strncmp(nrm, "L2nor", 5) == 0) nrm_type = SW_NRM_L2;
  if (!nrm_type) cli_fail("data_nrm_type=%s is not L2norm, L1norm, Huber or Cauchy", nrm);
  /* Init_SparseRegularization (Sparse_regularization.f90:51-143), read only
   * with wantreg or wantlog as in 2DAFWI.f90:80-84. */
  sw_reg_desc rd;
  sw_reg_state rs;
  memset(&rd, 0, sizeof(rd));
  memset(&rs, 0, sizeof(rs));
  rd.nz = g->nz;
  rd.nx = g->nx;
  rd.ny = g->ny;
  rd.wantreg = wantreg;
  rd.wantlog = wantlog;
  float *zweight = NULL;
  if (wantreg || wantlog) {
    char mn[32] = "Cauchy", hn[32] = "L2norm";
    sep_par_bool("compute_eps", &rd.compute_eps);
    sep_par_bool("compute_eps_log", &rd.compute_eps_log);
    sep_par_bool("derivdx", &rd.derivdx);
    sep_par_bool("derivdy", &rd.derivdy);
    sep_par_bool("derivdz", &rd.derivdz);
    sep_par_bool("log_z_plus", &rd.log_z_plus);
    sep_par_str("model_nrm_type", mn, sizeof(mn));
    sep_par_str("hinge_nrm_type", hn, sizeof(hn));
    rd.ratio = 10.f;
    rd.ratio_log = 10.f;
    rs.eps = 1.f;
    rs.eps_log = 1.f;
    if (rd.compute_eps) sep_par_float("ratio", &rd.ratio);
    else sep_par_float("eps", &rs.eps);
    if (rd.compute_eps_log) sep_par_float("ratio_logistic", &rd.ratio_log);
    else sep_par_float("eps_log", &rs.eps_log);
    sep_par_float("reg_threshold", &rs.mod_thresh);
    sep_par_float("hin_threshold", &rs.hin_thresh);
    rd.ntaperx = 10;
    rd.ntapery = 0;
    rd.ntaperz = 10;
    sep_par_int("sparse_taperx", &rd.ntaperx);
    sep_par_int("sparse_tapery", &rd.ntapery);
    sep_par_int("sparse_taperz", &rd.ntaperz);
    const char *names[2] = {mn, hn};
    int *types[2] = {&rd.mod_nrm_type, &rd.hin_nrm_type};
    for (int k = 0; k < 2; ++k) {
      if (strncmp(names[k], "Cauch", 5) == 0) *types[k] = SW_NRM_CAUCHY;
      if (strncmp(names[k], "Huber", 5) == 0) *types[k] = SW_NRM_HUBER;
      if (strncmp(names[k], "L1nor", 5) == 0) *types[k] = SW_NRM_L1;
      if (strncmp(names[k], "L2nor", 5) == 0) *types[k] = SW_NRM_L2;
      if (!*types[k]) cli_fail("%s is not L2norm, L1norm, Huber or Cauchy", names[k]);
    }
    /* Init_SparseRegularization_Array (:145-164). */
    if (sep_exist("Z_weights")) {
      sep_file *f = sep_open_in("Z_weights");
      if (!f) cli_fail("%s", sep_error());
      int n1 = 0, n2 = 0;
      sep_hdr_int(f, "n1", &n1);
      sep_hdr_int(f, "n2", &n2);
      if (n1 != g->nz) cli_fail("Error: n1 and nz mask/vel different, exit now");
      if (n2 != g->nx) cli_fail("Error: n2 and nx mask/vel different, exit now");
      zweight = (float *)malloc(n * 4);
      if (!zweight || sep_read(f, zweight, n)) cli_fail("Z_weights: %s", sep_error());
      sep_close(f);
      rd.zweight = zweight;
    }
  }
  /* Init_BandPassParam + BandpassSouTraces (Bandpass.f90:26-87). */
  float fhi = 20.f, flo = 0.f;
  int nphi = 14, nplo = 14, phase = 0;
  sep_par_float("fhi", &fhi);
  sep_par_float("flo", &flo);
  sep_par_int("nphi", &nphi);
  sep_par_int("nplo", &nplo);
  sep_par_int("phase", &phase);
  cli_check(ctx, sw_bandpass(ctx, 1, nt, g->dt, flo, fhi, nplo, nphi, phase, wavelet),
            "band-pass of the wavelet");
  cli_check(ctx, sw_bandpass(ctx, ntot, nt, g->dt, flo, fhi, nplo, nphi, phase, traces),
            "band-pass of the traces");
  /* Init_SmoothingParam (Smoothing.f90:36-68). */
  float percx = 0.5f, percz = 0.5f, percy = 0.f;
  sep_par_float("percx", &percx);
  sep_par_float("percz", &percz);
  sep_par_float("percy", &percy);
  float vmin = vel[0], vmax = vel[0];
  for (size_t i = 1; i < n; ++i) {
    vmin = vel[i] < vmin ? vel[i] : vmin;
    vmax = vel[i] > vmax ? vel[i] : vmax;
  }
  const float velref = (vmax - vmin) / 2.f + vmin;
  const float freqref = flo + (fhi - flo) / 2.f;
  const float wavex = percx * velref / freqref, wavey = percy * velref / freqref,
              wavez = percz * velref / freqref;
  sw_fwi_desc desc;
  memset(&desc, 0, sizeof(desc));
  desc.g = *g;
  desc.aperture_x = p->aperture_x;
  desc.aperture_y = p->aperture_y;
  desc.illu_pow = illu_pow;
  desc.smooth_rect1 = (int)((wavez / g->dz + 1.5f) / 2.f);
  desc.smooth_rect2 = (int)((wavex / g->dx + 1.5f) / 2.f);
  desc.smooth_rect3 = (int)((wavey / g->dy + 1.5f) / 2.f);
  desc.smooth_doz = !(wavez <= g->dz || wavez == 0.f);
  desc.smooth_dox = !(wavex <= g->dx || wavex == 0.f);
  desc.smooth_doy = !(wavey <= g->dy || wavey == 0.f);
  desc.checkpoint_snaps = 0;
  sep_par_int("checkpoint_snaps", &desc.checkpoint_snaps);
  desc.dat_nrm_type = nrm_type;
  desc.dat_thresh = dat_thresh;
  /* Init_Inversion_Array (Inversion_types.f90:106-134). */
  double *vpinit = (double *)malloc(n * sizeof(double));
  float *vpmask = (float *)malloc(n * 4);
  if (!vpinit || !vpmask) cli_fail("out of host memory");
  for (size_t i = 0; i < n; ++i) vpinit[i] = vel[i];
  if (sep_exist("vpmask")) {
    sep_file *f = sep_open_in("vpmask");
    if (!f) cli_fail("%s", sep_error());
    int m1 = 0, m2 = 0;
    sep_hdr_int(f, "n1", &m1);
    sep_hdr_int(f, "n2", &m2);
    if (m1 != g->nz) cli_fail("n1 and nz mask/vel different, exit now");
    if (m2 != g->nx) cli_fail("n2 and nx mask/vel different, exit now");
    if (sep_read(f, vpmask, n)) cli_fail("%s", sep_error());
    sep_close(f);
  } else {
    for (size_t i = 0; i < n; ++i) vpmask[i] = 1.f;
  }
  /* Init_MuteParam + MuteParam_compute_mask (Mute.f90:27-95). */
  float v0 = 1500.f, v1 = 10000.f, t0 = 0.f, t1 = 40.f, tramp = 0.5f;
  sep_par_float("v0", &v0);
  sep_par_float("v1", &v1);
  sep_par_float("t0", &t0);
  sep_par_float("t1", &t1);
  sep_par_float("tramp", &tramp);
  float *mute = (float *)malloc((size_t)ntot * nt * 4);
  float *resid = (float *)calloc((size_t)ntot * nt, 4);
  sw_fwi_shot *shots = (sw_fwi_shot *)calloc((size_t)ng, sizeof(sw_fwi_shot));
  if (!mute || !resid || !shots) cli_fail("out of host memory");
  for (int ig = 0; ig < ng; ++ig) {
    const gather *G = &gs[ig];
    sw_mute_mask(G->ntr, nt, g->dt, ot, G->sou, rec + 3 * (size_t)G->begi, v0, v1, t0, t1,
                 tramp, mute + (size_t)G->begi * nt);
    sw_fwi_shot *S = &shots[ig];
    memcpy(S->sou_coord, G->sou, sizeof(S->sou_coord));
    S->nrec = G->ntr;
    S->rec_coord = rec + 3 * (size_t)G->begi;
    S->dobs = traces + (size_t)G->begi * nt;
    S->mute = mute + (size_t)G->begi * nt;
    S->resid = resid + (size_t)G->begi * nt;
  }
  sep_file *fmodel = open_optional("model"), *fgrad = open_optional("gradient"),
           *ffunc = open_optional("function"), *fres = open_optional("residual");
  /* l_bfgs (Inversion.f90:29-189). */
  const double xmin = vpmin, xmax = vpmax;
  sw_lbfgs *lb = NULL;
  cli_check(ctx, sw_lbfgs_create(ctx, (int)n, 5, xmin, xmax, vpmask, bound, freeze_soft, vpinit,
                                 &lb), "sw_lbfgs_create");
  float *x = vel;    /* the model, updated in place */
  float *grad = (float *)malloc(n * 4), *illum = (float *)malloc(n * 4);
  double *xd = (double *)malloc(n * sizeof(double)), *gd = (double *)malloc(n * sizeof(double));
  double *xsave = (double *)malloc(n * sizeof(double));
  double *xdsave = (double *)malloc(n * sizeof(double));
  if (!grad || !illum || !xd || !gd || !xsave || !xdsave) cli_fail("out of host memory");
  for (size_t i = 0; i < n; ++i) xsave[i] = xdsave[i] = x[i];
  int eval = 0, iter = 0, count = 0, cont = 1, found = 0, iflag = 0, info = 0;
  float g0 = 0.f;
  double f0 = 0.0;
  while (cont && !found) {
    double fd = 0.0;
    cli_check(ctx, sw_fwi_fct_gdt(ctx, &desc, x, wavelet, ng, shots, vpmask, &fd, grad, illum),
              "sw_fwi_fct_gdt");
    cli_check(ctx, sw_fwi_regularize(ctx, &rd, &rs, eval, x, vpmask, &fd, grad),
              "sw_fwi_regularize");
    if (eval == 0) {
      float mx = x[0];
      for (size_t i = 1; i < n; ++i) mx = x[i] > mx ? x[i] : mx;
      g0 = mx / (100.f * maxabs(grad, n));
      f0 = (double)(mx * mx) / fabs(fd);
      if (ffunc) {
        const float v = (float)(f0 * fd);
        sep_write(ffunc, &v, 1);
      }
    }
    for (size_t i = 0; i < n; ++i) grad[i] = g0 * grad[i];
    fd = f0 * fd;
    for (size_t i = 0; i < n; ++i) {
      xd[i] = x[i];
      gd[i] = -(double)grad[i];
      xdsave[i] = xd[i];
    }
    int myinfo = 0;
    cli_check(ctx, sw_lbfgs_step(lb, xd, fd, gd, 1.0e-20, 2.220446049250313e-16, &iflag, &myinfo),
              "sw_lbfgs_step");
    for (size_t i = 0; i < n; ++i) x[i] = (float)xd[i];
    info = myinfo;
    if (myinfo == 1) {
      if (bound == 2) freeze_x(xdsave, n, xmin, xmax, vpmask, freeze_soft, vpinit);
      memcpy(xsave, xdsave, n * sizeof(double));
      ++iter;
      ++count;
      if (count >= niter) found = 1;
      if (fmodel)
        for (size_t i = 0; i < n; ++i) {
          const float v = (float)xdsave[i];
          sep_write(fmodel, &v, 1);
        }
      if (ffunc) {
        const float v = (float)fd;
        sep_write(ffunc, &v, 1);
      }
      if (fgrad)
        for (size_t i = 0; i < n; ++i) {
          const float v = -grad[i];
          sep_write(fgrad, &v, 1);
        }
      if (fres) sep_write(fres, resid, (size_t)ntot * nt);
      fprintf(stderr, "INFO: iteration %d, scaled misfit %g\n", iter, fd);
    }
    if (iflag <= 0) {
      cont = 0;
      if (iflag == -1) fprintf(stderr, "INFO: LBFGS stopped, info=%d\n", info);
    }
    ++eval;
    if (eval >= neval) cont = 0;
  }
  if (!cont)
    for (size_t i = 0; i < n; ++i) x[i] = (float)xsave[i];
  sw_lbfgs_destroy(lb);
  freeze_and_mask(x, n, vpmin, vpmax, vpmask, freeze_soft, vpinit);
  sep_file *fo = sep_open_out("inv");
  if (!fo) cli_fail("%s", sep_error());
  if (sep_write(fo, x, n)) cli_fail("%s", sep_error());
  put_model_axes(fo, g);
  if (sep_close(fo)) cli_fail("%s", sep_error());
  /* create_header (2DAFWI.f90:126-197). */
  if (fgrad) {
    put_model_axes(fgrad, g);
    sep_put_int(fgrad, "n4", iter);
    sep_close(fgrad);
  }
  if (fmodel) {
    put_model_axes(fmodel, g);
    sep_put_int(fmodel, "n4", iter);
    sep_close(fmodel);
  }
  if (ffunc) {
    sep_put_int(ffunc, "n1", iter + 1);
    sep_close(ffunc);
  }
  if (fres) {
    sep_put_int(fres, "n1", nt);
    sep_put_int(fres, "n2", ntot);
    sep_put_int(fres, "n3", iter);
    sep_put_float(fres, "d1", g->dt);
    sep_put_float(fres, "d2", 1.f);
    sep_put_float(fres, "o1", ot);
    sep_put_float(fres, "o2", 0.f);
    sep_close(fres);
  }
  fprintf(stderr, "INFO: %d iterations, %d evaluations\n", iter, eval);
  free(grad);
  free(illum);
  free(xd);
  free(gd);
  free(xsave);
  free(xdsave);
  free(vpinit);
  free(vpmask);
  free(zweight);
  free(mute);
  free(resid);
  free(shots);
  return 0;
}

int main(int argc, char **argv) {
  if (sep_init(argc, argv)) cli_fail("%s", sep_error());
  if (!sep_exist("vel")) cli_fail("need velocity file");
  cli_par p;
  cli_read_params(&p);
  if (p.withRho) cli_fail("Rho not implemented in this version");
  const int mod = !strcmp(p.task, "MOD") || !strcmp(p.task, "mod");
  const int mig = !strcmp(p.task, "MIG") || !strcmp(p.task, "mig");
  const int inv = !strcmp(p.task, "INV") || !strcmp(p.task, "inv");
  if (!mod && !mig && !inv) cli_fail("Task=%s: expected MOD, MIG or INV", p.task);
  float *wavelet = cli_read_source(&p);
  const int nt = p.g.nt;

  const char *names[6] = {"keygx", "keysx", "keygy", "keysy", "keyselev", "keygelev"};
  int idx[6];
  for (int k = 0; k < 6; ++k)
    if (sep_par_int(names[k], &idx[k]) != 1) cli_fail("need %s", names[k]);
  int nkeys = 0, ntot = 0;
  float *keys = read_all_keys(&nkeys, &ntot);
  for (int k = 0; k < 6; ++k)
    if (idx[k] < 1 || idx[k] > nkeys) cli_fail("%s=%d is outside 1..%d", names[k], idx[k], nkeys);
  float *rec = (float *)malloc((size_t)ntot * 3 * 4);
  gather *gs = (gather *)malloc((size_t)ntot * sizeof(gather));
  if (!rec || !gs) cli_fail("out of host memory");
  int ng = 0;
  for (int i = 0; i < ntot; ++i) {
    const float *k = keys + (size_t)i * nkeys;
    rec[3 * i + 0] = k[idx[5] - 1];
    rec[3 * i + 1] = k[idx[0] - 1];
    rec[3 * i + 2] = k[idx[2] - 1];
    const float sx = k[idx[1] - 1], sy = k[idx[3] - 1];
    if (ng == 0 || sx != gs[ng - 1].sou[1] || sy != gs[ng - 1].sou[2]) {
      gs[ng].begi = i;
      gs[ng].ntr = 0;
      ++ng;
    }
    gather *g = &gs[ng - 1];
    g->ntr++;
    g->sou[0] = k[idx[4] - 1];  /* the gather's last trace gives the source */
    g->sou[1] = sx;
    g->sou[2] = sy;
  }
  fprintf(stderr, "INFO: ngathers %d nkeys %d ntraces %d\n", ng, nkeys, ntot);

  float *traces = NULL;
  float ot = 0.f;
  if (mig || inv) {
    int ntr = 0;
    traces = cli_read_traces(nt, &ntr, &ot);
    if (ntr != ntot) cli_fail("number of read traces is different from n2 in traces");
  }
  float *vel = cli_read_model(&p, "vel");
  float cour = 0.f, sr = 0.f;
  if (sw_vel_check(&p.g, vel, &cour, &sr) != SW_OK)
    cli_fail("vel_check: Courant number %g or %g samples per minimum wavelength out of range",
             (double)cour, (double)sr);
  const char *out_tag = mod ? "data" : mig ? "image" : "inv";
  if (!sep_exist(out_tag)) cli_fail("need %s file for output", out_tag);

  sw_ctx *ctx = cli_context();
  if (inv) {
    const int rc = run_inversion(ctx, &p, wavelet, vel, traces, ot, rec, ntot, gs, ng);
    sw_ctx_destroy(ctx);
    free(vel);
    free(traces);
    free(rec);
    free(gs);
    free(keys);
    free(wavelet);
    sep_finish();
    return rc;
  }
  const size_t nm = (size_t)p.g.nz * p.g.nx * p.g.ny;
  float *out = (float *)calloc(mod ? (size_t)ntot * nt : nm, 4);
  float *illu = mig ? (float *)calloc(nm, 4) : NULL;
  if (!out || (mig && !illu)) cli_fail("out of host memory");
  for (int ig = 0; ig < ng; ++ig) {
    const gather *G = &gs[ig];
    const float *grec = rec + 3 * (size_t)G->begi;
    sw_window w;
    sw_genpar gw;
    cli_shot_window(&p, G->sou, G->ntr, grec, &w, &gw);
    const size_t nw = (size_t)gw.nz * gw.nx * gw.ny;
    float *vs = (float *)malloc(nw * 4);
    if (!vs) cli_fail("out of host memory");
    sw_window_extract(&p.g, &w, vel, vs);
    sw_prop_desc fd;
    memset(&fd, 0, sizeof(fd));
    fd.g = gw;
    fd.tmin = 1;
    fd.tmax = nt;
    fd.tstep = 1;
    fd.fd_scheme = SW_FD_FORWARD;
    fd.injection = SW_INJ_SINC;
    sw_prop_io a;
    memset(&a, 0, sizeof(a));
    a.vel = vs;
    a.nsou = 1;
    a.sou_coord = G->sou;
    a.sou_trace = wavelet;
    if (mod) {
      /* AMOD_to_memory (to_disk_to_memory_AMOD.f90:27-82). */
      fd.extraction = SW_EXT_SIMPLE_AFWI;
      a.nrec = G->ntr;
      a.rec_coord = grec;
      a.rec_trace = out + (size_t)G->begi * nt;
      cli_check(ctx, sw_propagate(ctx, &fd, &a), "AMOD propagation");
    } else {
      const int ntsnap = nt / gw.snapi;
      float *wave = (float *)malloc(nw * (size_t)(ntsnap > 0 ? ntsnap : 1) * 4);
      float *ims = (float *)calloc(nw, 4), *ils = (float *)calloc(nw, 4);
      if (!wave || !ims || !ils) cli_fail("out of host memory");
      fd.extract_wave = 1;
      a.wave = wave;
      cli_check(ctx, sw_propagate(ctx, &fd, &a), "AMOD propagation");
      /* AGRAD_to_memory (to_disk_to_memory_AGRAD.f90:27-79). */
      sw_prop_desc bd;
      memset(&bd, 0, sizeof(bd));
      bd.g = gw;
      bd.tmin = nt;
      bd.tmax = 1;
      bd.tstep = -1;
      bd.fd_scheme = SW_FD_FORWARD;
      bd.injection = SW_INJ_SIMPLE;
      bd.imaging = SW_IMG_AFWI;
      sw_prop_io b;
      memset(&b, 0, sizeof(b));
      b.vel = vs;
      b.nsou = G->ntr;
      b.sou_coord = grec;
      b.sou_trace = traces + (size_t)G->begi * nt;
      b.wave = wave;
      b.image = ims;
      b.illum = ils;
      cli_check(ctx, sw_propagate(ctx, &bd, &b), "AGRAD propagation");
      sw_window_scatter_add(&p.g, &w, ims, out);
      sw_window_scatter_add(&p.g, &w, ils, illu);
      free(wave);
      free(ims);
      free(ils);
    }
    free(vs);
    if ((ig + 1) % 10 == 0) fprintf(stderr, "INFO: %d of %d gathers done\n", ig + 1, ng);
  }

  sep_file *f = sep_open_out(out_tag);
  if (!f) cli_fail("%s", sep_error());
  if (mod) {
    if (sep_write(f, out, (size_t)ntot * nt)) cli_fail("%s", sep_error());
    sep_put_int(f, "n1", nt);
    sep_put_int(f, "n2", ntot);
    sep_put_float(f, "d1", p.g.dt);
    sep_put_float(f, "d2", 1.f);
    sep_put_float(f, "o1", 0.f);
    sep_put_float(f, "o2", 0.f);
  } else {
    /* illu = (illu + maxval(illu)/10000) / sqrt(sum(dprod(illu,illu))/size(illu));
     * imag = imag/illu (compute_function_gradient.f90:452-453). */
    float mx = illu[0];
    double ss = 0.0;
    for (size_t q = 0; q < nm; ++q) {
      mx = illu[q] > mx ? illu[q] : mx;
      ss += (double)illu[q] * (double)illu[q];
    }
    const double r = sqrt(ss / (double)nm);
    for (size_t q = 0; q < nm; ++q) {
      const float v = (float)((double)(illu[q] + mx / 10000.f) / r);
      out[q] = out[q] / v;
    }
    if (sep_write(f, out, nm)) cli_fail("%s", sep_error());
    sep_put_int(f, "n1", p.g.nz);
    sep_put_int(f, "n2", p.g.nx);
    sep_put_int(f, "n3", p.g.ny);
  }
  if (sep_close(f)) cli_fail("%s", sep_error());
  sw_ctx_destroy(ctx);
  free(out);
  free(illu);
  free(vel);
  free(traces);
  free(rec);
  free(gs);
  free(keys);
  free(wavelet);
  sep_finish();
  return 0;
}
